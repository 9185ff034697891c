// fse_server.cu -- continuous batching of world-tick requests under an HBM budget.
//
// Worlds are registered once and keep their state in HBM. A request asks for n
// ticks of one world. Each scheduling step admits queued requests (arrival order,
// one request per world at a time, at most max_active), then enqueues one batched
// tick of every active world -- the same launches as a batch step, over a device
// table of the active worlds -- and returns without waiting: up to `depth` steps
// are in flight on the server's stream while the host schedules the next ones.
// Each step ends in a CUDA event; a request is complete when the event of the step
// that ran its last tick has fired, and its completion time is that event's device
// timestamp on the server clock.
//
// Admission is by HBM footprint per request. The budget covers the resident
// worlds; a world that does not fit is parked in host memory as an exact
// checkpoint (every plane, particles, tick counter, seed, ledger). A request for a
// parked world is admitted when its footprint fits: the server first parks idle
// resident worlds, least recently ticked first, and then restores the requested
// world from its checkpoint. A restored world continues bit for bit, so a
// request's result is the same however often its world was parked.
#include <math.h>
#include <string.h>

#include <algorithm>
#include <chrono>
#include <deque>
#include <vector>

#include "fse_host.cuh"

using namespace fse;

namespace {
constexpr int STAGES = 4;             // pinned buffers for table uploads
constexpr double REBASE_US = 1.0e6;   // an idle server re-anchors a device clock older than this
constexpr size_t TICK_LOG = 1 << 20;  // step durations kept until fse_server_tick_times reads them
}  // namespace

struct fse_server {
    int64_t budget = 0, in_use = 0;
    int max_active = 1;
    int depth = 3;  // steps in flight before a step waits for the oldest
    int C = 128;
    cudaStream_t stream = nullptr;
    struct Slot {
        bool used = false;
        fse_world *w = nullptr;       // resident state; nullptr while parked
        std::vector<uint8_t> parked;  // exact checkpoint while parked
        int W = 0, H = 0;
        fse_config cfg{};
        int64_t bytes = 0;   // device bytes of the world when resident
        uint64_t last = 0;   // sequence number of its last step (LRU order)
        int queued = 0;      // its requests waiting in the queue
        bool active = false; // a request of it is active
    };
    std::vector<Slot> slots;
    struct Req {
        int64_t id;
        int slot, left;
        double arrival;
    };
    std::deque<Req> queue;
    std::vector<Req> active;
    std::vector<std::pair<int64_t, double>> done;
    std::vector<float> tick_ms;  // device time of each retired step
    int64_t next_id = 0;
    struct Flight {
        cudaEvent_t start, end;
        std::vector<int64_t> finishing;  // requests whose last tick this step runs
    };
    std::deque<Flight> flights;
    std::vector<cudaEvent_t> spare;
    cudaEvent_t base = nullptr;  // device-clock anchor: its host time is base_us
    double base_us = 0.0;
    uint64_t seq = 0;
    int64_t page_ins = 0, page_outs = 0, max_flight = 0;
    // device table of the active worlds and their chunk items, one upload per change
    uint8_t *arena = nullptr;
    size_t arena_cap = 0;
    WorldDev *d_table = nullptr;
    uint32_t *items[4] = {nullptr, nullptr, nullptr, nullptr};
    int n_items[4] = {0, 0, 0, 0};
    std::vector<int> table_slots;
    struct Stage {
        uint8_t *host = nullptr;
        size_t cap = 0;
        cudaEvent_t copied = nullptr;
    };
    Stage stage[STAGES];
    int stage_next = 0;
    std::chrono::steady_clock::time_point t0;

    double now_us() const {
        return std::chrono::duration<double, std::micro>(std::chrono::steady_clock::now() - t0).count();
    }
};

namespace {

// device bytes a world of this size and configuration allocates (an upper bound)
int64_t world_footprint(int w, int h, const fse_config *cfg) {
    long long cells = (long long)w * h;
    long long pc = (cfg && cfg->particle_capacity > 0) ? cfg->particle_capacity : std::max<long long>(65536, cells / 4);
    long long sc = (cfg && cfg->spawn_capacity > 0) ? cfg->spawn_capacity : pc;
    // planes; two particle SoAs, the outcome byte, four outcome words and two merge-list words
    return cells * 15 + pc * (2 * 56 + 1 + 4 * 6) + sc * (long long)sizeof(SpawnRec) + (1 << 20);
}

size_t round_up(size_t n, size_t a) { return (n + a - 1) / a * a; }

cudaEvent_t take_event(fse_server *s) {
    if (!s->spare.empty()) {
        cudaEvent_t e = s->spare.back();
        s->spare.pop_back();
        return e;
    }
    cudaEvent_t e = nullptr;
    if (cudaEventCreate(&e) != cudaSuccess) return nullptr;
    return e;
}

// anchor the device clock: an event on the idle stream and the host time it completed
int rebase(fse_server *s) {
    if (!s->base && cudaEventCreate(&s->base) != cudaSuccess) return FSE_E_CUDA;
    FSE_CUDA_TRY(cudaEventRecord(s->base, s->stream));
    FSE_CUDA_TRY(cudaEventSynchronize(s->base));
    s->base_us = s->now_us();
    return FSE_OK;
}

// retire finished steps in order; block = wait for the oldest one at least
int retire(fse_server *s, bool block) {
    while (!s->flights.empty()) {
        fse_server::Flight &f = s->flights.front();
        cudaError_t e = block ? cudaEventSynchronize(f.end) : cudaEventQuery(f.end);
        if (e == cudaErrorNotReady) break;
        if (e != cudaSuccess) return FSE_E_CUDA;
        float at = 0.f, dur = 0.f;
        FSE_CUDA_TRY(cudaEventElapsedTime(&at, s->base, f.end));
        FSE_CUDA_TRY(cudaEventElapsedTime(&dur, f.start, f.end));
        const double t = s->base_us + 1e3 * (double)at;
        for (int64_t id : f.finishing) s->done.push_back({id, t});
        if (s->tick_ms.size() >= TICK_LOG) s->tick_ms.erase(s->tick_ms.begin(), s->tick_ms.begin() + TICK_LOG / 2);
        s->tick_ms.push_back(dur);
        s->spare.push_back(f.start);
        s->spare.push_back(f.end);
        s->flights.pop_front();
        block = false;
    }
    return FSE_OK;
}

int drain(fse_server *s) {
    while (!s->flights.empty()) {
        int rc = retire(s, true);
        if (rc) return rc;
    }
    return FSE_OK;
}

// park a resident world: exact checkpoint to host memory, device memory freed
int park(fse_server *s, int slot) {
    fse_server::Slot &sl = s->slots[slot];
    int rc = drain(s);
    if (rc) return rc;
    int64_t bound = 0, size = 0;
    if ((rc = fse_world_checkpoint_bound(sl.w, &bound))) return rc;
    sl.parked.resize((size_t)bound);
    if ((rc = fse_world_checkpoint(sl.w, sl.parked.data(), bound, &size))) return rc;
    sl.parked.resize((size_t)size);
    sl.parked.shrink_to_fit();
    fse_world_destroy(sl.w);
    sl.w = nullptr;
    s->in_use -= sl.bytes;
    s->page_outs++;
    s->table_slots.clear();  // descriptors of the active set may have moved
    return FSE_OK;
}

// make room for `need` more bytes by parking idle resident worlds, least recently
// ticked first; worlds with queued requests only when take_queued. Parks nothing
// unless the room can be made.
int make_room(fse_server *s, int64_t need, bool take_queued, int except) {
    int64_t free_b = s->budget - s->in_use;
    if (need <= free_b) return FSE_OK;
    std::vector<int> cand;
    for (int i = 0; i < (int)s->slots.size(); i++) {
        const fse_server::Slot &sl = s->slots[i];
        if (i == except || !sl.used || !sl.w || sl.active) continue;
        if (sl.queued && !take_queued) continue;
        cand.push_back(i);
    }
    std::sort(cand.begin(), cand.end(), [&](int a, int b) {
        const fse_server::Slot &x = s->slots[a], &y = s->slots[b];
        if ((x.queued > 0) != (y.queued > 0)) return x.queued == 0;
        return x.last != y.last ? x.last < y.last : a < b;
    });
    int64_t avail = free_b;
    size_t k = 0;
    while (k < cand.size() && avail < need) avail += s->slots[cand[k++]].bytes;
    if (avail < need) return FSE_E_BUDGET;
    for (size_t i = 0; i < k; i++) {
        int rc = park(s, cand[i]);
        if (rc) return rc;
    }
    return FSE_OK;
}

// bring a parked world back into HBM
int page_in(fse_server *s, int slot, bool take_queued) {
    fse_server::Slot &sl = s->slots[slot];
    if (sl.w) return FSE_OK;
    int rc = make_room(s, sl.bytes, take_queued, slot);
    if (rc) return rc;
    fse_config c = sl.cfg;
    c.stream = (void *)s->stream;
    fse_world *w = nullptr;
    if ((rc = fse_world_create(sl.W, sl.H, &c, &w))) return rc;
    if ((rc = fse_world_restore(w, sl.parked.data(), (int64_t)sl.parked.size())) || (rc = fse_world_trim(w))) {
        fse_world_destroy(w);
        return rc;
    }
    sl.w = w;
    sl.bytes = (int64_t)w->bytes;
    s->in_use += sl.bytes;
    std::vector<uint8_t>().swap(sl.parked);
    s->page_ins++;
    s->table_slots.clear();
    return FSE_OK;
}

// admit queued requests in arrival order while active slots are free; a request
// whose world is busy waits for it, one whose world is parked waits for room. The
// oldest request of a parked world may park worlds that have queued requests.
int admit(fse_server *s) {
    bool oldest_parked = true;
    for (auto it = s->queue.begin(); it != s->queue.end() && (int)s->active.size() < s->max_active;) {
        fse_server::Slot &sl = s->slots[it->slot];
        if (sl.active) {
            ++it;
            continue;
        }
        if (!sl.w) {
            int rc = page_in(s, it->slot, oldest_parked);
            oldest_parked = false;
            if (rc == FSE_E_BUDGET) {
                ++it;
                continue;
            }
            if (rc) return rc;
        }
        sl.active = true;
        sl.queued--;
        s->active.push_back(*it);
        it = s->queue.erase(it);
    }
    return FSE_OK;
}

// upload the table of the active worlds through a pinned staging buffer (stream order)
int upload_tables(fse_server *s, const std::vector<int> &want) {
    const size_t A = 256;
    std::vector<uint32_t> it[4];
    for (size_t i = 0; i < want.size(); i++) {
        const WorldDev &h = s->slots[want[i]].w->h;
        for (int tk = 0; tk < 4; tk++) {
            int ox = tk % 2, oy = 1 - tk / 2;
            int na = (h.nCx - ox + 1) / 2, nb = (h.nCy - oy + 1) / 2;
            int ns = std::max(0, na) * std::max(0, nb);
            for (int c = 0; c < ns; c++) it[tk].push_back(((uint32_t)i << 20) | (uint32_t)c);
        }
    }
    size_t off[5];
    off[0] = round_up(std::max<size_t>(want.size(), 1) * sizeof(WorldDev), A);
    for (int tk = 0; tk < 4; tk++) off[tk + 1] = off[tk] + round_up(std::max<size_t>(it[tk].size(), 1) * 4, A);
    const size_t total = off[4];
    if (total > s->arena_cap) {
        int rc = drain(s);  // in-flight steps read the old arena
        if (rc) return rc;
        const size_t cap = std::max(total, 2 * s->arena_cap);
        if (s->arena) cudaFree(s->arena);
        s->arena = nullptr;
        s->arena_cap = 0;
        if (cudaMalloc(&s->arena, cap) != cudaSuccess) {
            cudaGetLastError();
            return FSE_E_NOMEM;
        }
        s->arena_cap = cap;
    }
    fse_server::Stage &st = s->stage[s->stage_next];
    s->stage_next = (s->stage_next + 1) % STAGES;
    if (st.copied) FSE_CUDA_TRY(cudaEventSynchronize(st.copied));  // its last copy has read it
    else if (cudaEventCreateWithFlags(&st.copied, cudaEventDisableTiming) != cudaSuccess) return FSE_E_CUDA;
    if (total > st.cap) {
        const size_t cap = std::max(total, 2 * st.cap);
        if (st.host) cudaFreeHost(st.host);
        st.host = nullptr;
        st.cap = 0;
        if (cudaMallocHost(&st.host, cap) != cudaSuccess) {
            cudaGetLastError();
            return FSE_E_NOMEM;
        }
        st.cap = cap;
    }
    WorldDev *tab = reinterpret_cast<WorldDev *>(st.host);
    for (size_t i = 0; i < want.size(); i++) tab[i] = s->slots[want[i]].w->h;
    for (int tk = 0; tk < 4; tk++)
        if (!it[tk].empty()) memcpy(st.host + off[tk], it[tk].data(), it[tk].size() * 4);
    FSE_CUDA_TRY(cudaMemcpyAsync(s->arena, st.host, total, cudaMemcpyHostToDevice, s->stream));
    FSE_CUDA_TRY(cudaEventRecord(st.copied, s->stream));
    s->d_table = reinterpret_cast<WorldDev *>(s->arena);
    for (int tk = 0; tk < 4; tk++) {
        s->items[tk] = reinterpret_cast<uint32_t *>(s->arena + off[tk]);
        s->n_items[tk] = (int)it[tk].size();
    }
    s->table_slots = want;
    return FSE_OK;
}

}  // namespace

extern "C" {

int fse_server_create(int64_t budget, int max_active, fse_server **out) {
    if (!out || budget <= 0 || max_active <= 0 || max_active > 4095) return FSE_E_INVAL;
    fse_server *s = new fse_server();
    s->budget = budget;
    s->max_active = max_active;
    s->t0 = std::chrono::steady_clock::now();
    if (cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking) != cudaSuccess || rebase(s) != FSE_OK) {
        if (s->stream) cudaStreamDestroy(s->stream);
        if (s->base) cudaEventDestroy(s->base);
        delete s;
        return FSE_E_CUDA;
    }
    *out = s;
    return FSE_OK;
}

int fse_server_destroy(fse_server *s) {
    if (!s) return FSE_E_INVAL;
    drain(s);
    cudaStreamSynchronize(s->stream);
    for (auto &sl : s->slots)
        if (sl.w) fse_world_destroy(sl.w);
    if (s->arena) cudaFree(s->arena);
    for (auto &st : s->stage) {
        if (st.host) cudaFreeHost(st.host);
        if (st.copied) cudaEventDestroy(st.copied);
    }
    for (cudaEvent_t e : s->spare) cudaEventDestroy(e);
    if (s->base) cudaEventDestroy(s->base);
    cudaStreamDestroy(s->stream);
    delete s;
    return FSE_OK;
}

int fse_server_add_world(fse_server *s, int w, int h, const fse_config *cfg, int gen_kind, uint32_t gen_seed,
                         int *out_slot) {
    if (!s || !out_slot) return FSE_E_INVAL;
    const int64_t need = world_footprint(w, h, cfg);
    if (need > s->budget) return FSE_E_BUDGET;  // could never be resident
    fse_config c{};
    if (cfg) c = *cfg;
    if (c.chunk_size == 0) c.chunk_size = 128;
    // servers batch their worlds in the partitioned order with Q16.16 amounts
    if (c.flags & (FSE_CFG_REFERENCE_ORDER | FSE_CFG_F32_FLUID)) return FSE_E_INVAL;
    for (auto &sl : s->slots)
        if (sl.used && sl.cfg.chunk_size != c.chunk_size) return FSE_E_INVAL;
    int rc = make_room(s, need, false, -1);
    if (rc) return rc;
    fse_config cw = c;
    cw.stream = (void *)s->stream;
    fse_world *wd = nullptr;
    if ((rc = fse_world_create(w, h, &cw, &wd))) return rc;
    if ((rc = fse_world_generate(wd, gen_kind, gen_seed))) {
        fse_world_destroy(wd);
        return rc;
    }
    s->C = c.chunk_size;
    int slot = -1;
    for (size_t i = 0; i < s->slots.size(); i++)
        if (!s->slots[i].used) {
            slot = (int)i;
            break;
        }
    if (slot < 0) {
        slot = (int)s->slots.size();
        s->slots.emplace_back();
    }
    fse_server::Slot &sl = s->slots[slot];
    sl = fse_server::Slot();
    sl.used = true;
    sl.w = wd;
    sl.W = w;
    sl.H = h;
    sl.cfg = c;
    sl.cfg.stream = nullptr;
    sl.bytes = (int64_t)wd->bytes;
    sl.last = s->seq;
    s->in_use += sl.bytes;
    if (s->in_use > s->budget && make_room(s, 0, false, slot) != FSE_OK) {
        // the world came out larger than its footprint and no idle world can make up for it
        fse_world_destroy(wd);
        s->in_use -= sl.bytes;
        sl = fse_server::Slot();
        return FSE_E_BUDGET;
    }
    *out_slot = slot;
    return FSE_OK;
}

int fse_server_remove_world(fse_server *s, int slot) {
    if (!s || slot < 0 || slot >= (int)s->slots.size() || !s->slots[slot].used) return FSE_E_INVAL;
    fse_server::Slot &sl = s->slots[slot];
    if (sl.active || sl.queued) return FSE_E_STATE;
    int rc = drain(s);  // its last step may still be in flight
    if (rc) return rc;
    if (sl.w) {
        fse_world_destroy(sl.w);
        s->in_use -= sl.bytes;
    }
    sl = fse_server::Slot();
    s->table_slots.clear();
    return FSE_OK;
}

int64_t fse_server_bytes_in_use(const fse_server *s) { return s ? s->in_use : -1; }

double fse_server_now_us(const fse_server *s) { return s ? s->now_us() : 0.0; }

fse_world *fse_server_world(fse_server *s, int slot) {
    if (!s || slot < 0 || slot >= (int)s->slots.size() || !s->slots[slot].used) return nullptr;
    if (!s->slots[slot].w && page_in(s, slot, false) != FSE_OK) return nullptr;
    return s->slots[slot].w;
}

int fse_server_submit(fse_server *s, int slot, int n_ticks, double arrival_us, int64_t *out_request) {
    if (!s || slot < 0 || slot >= (int)s->slots.size() || !s->slots[slot].used || n_ticks <= 0) return FSE_E_INVAL;
    fse_server::Req r{s->next_id++, slot, n_ticks, arrival_us};
    s->queue.push_back(r);
    s->slots[slot].queued++;
    if (out_request) *out_request = r.id;
    return FSE_OK;
}

int fse_server_step(fse_server *s, int *out_active) {
    if (!s) return FSE_E_INVAL;
    int rc = retire(s, false);
    if (rc) return rc;
    if ((rc = admit(s))) return rc;
    if (out_active) *out_active = (int)s->active.size();
    if (s->active.empty()) {
        // nothing to enqueue: wait for the steps in flight; re-anchor an old device clock
        if ((rc = drain(s))) return rc;
        if (s->now_us() - s->base_us > REBASE_US) return rebase(s);
        return FSE_OK;
    }
    std::vector<int> want;
    for (auto &a : s->active) want.push_back(a.slot);
    std::sort(want.begin(), want.end());
    if (want != s->table_slots && (rc = upload_tables(s, want))) return rc;
    int max_iter = 0, mb = 1, sb = 1;
    std::vector<fse_world *> act;
    for (int sl : want) {
        fse_world *w = s->slots[sl].w;
        act.push_back(w);
        max_iter = std::max(max_iter, w->cell_iter);
        mb = std::max(mb, std::min(sm_count() * 2, ceil_div(w->part_cap, 256)));
        sb = std::max(sb, std::min(sm_count(), ceil_div(w->stage_cap, 256)));
    }
    if ((rc = ensure_materials_pushed())) return rc;
    fse_server::Flight f;
    f.start = take_event(s);
    f.end = take_event(s);
    if (!f.start || !f.end) return FSE_E_CUDA;
    FSE_CUDA_TRY(cudaEventRecord(f.start, s->stream));
    rc = enqueue_step(s->d_table, (int)want.size(), s->items, s->n_items, max_iter, s->C, CP_THREADS, FUSED_GRID, true,
                      mb, sb, s->stream, nullptr, temp_tiles_of(act), temp_track_of(act));
    if (rc) return rc;
    FSE_CUDA_TRY(cudaEventRecord(f.end, s->stream));
    s->seq++;
    std::vector<fse_server::Req> keep;
    for (auto &a : s->active) {
        fse_server::Slot &sl = s->slots[a.slot];
        sl.last = s->seq;
        if (--a.left <= 0) {
            f.finishing.push_back(a.id);
            sl.active = false;  // its world may take its next request in the next step
        } else {
            keep.push_back(a);
        }
    }
    s->active.swap(keep);
    s->flights.push_back(std::move(f));
    s->max_flight = std::max<int64_t>(s->max_flight, (int64_t)s->flights.size());
    if ((int)s->flights.size() > s->depth) return retire(s, true);
    return FSE_OK;
}

int fse_server_poll(fse_server *s, double now_us, int64_t *ids, double *done_us, int cap, int *out_n) {
    (void)now_us;
    if (!s || cap < 0) return FSE_E_INVAL;
    int rc = retire(s, false);
    if (rc) return rc;
    int m = std::min<int>(cap, (int)s->done.size());
    for (int i = 0; i < m; i++) {
        if (ids) ids[i] = s->done[i].first;
        if (done_us) done_us[i] = s->done[i].second;
    }
    s->done.erase(s->done.begin(), s->done.begin() + m);
    if (out_n) *out_n = m;
    return FSE_OK;
}

int fse_server_set_depth(fse_server *s, int depth) {
    if (!s || depth < 1 || depth > 64) return FSE_E_INVAL;
    s->depth = depth;
    return retire(s, false);
}

int fse_server_drain(fse_server *s) { return s ? drain(s) : FSE_E_INVAL; }

int fse_server_stats(fse_server *s, int64_t *out, int n) {
    if (!s || !out || n < 0) return FSE_E_INVAL;
    int64_t resident = 0, parked = 0;
    for (auto &sl : s->slots) {
        if (!sl.used) continue;
        if (sl.w) resident++;
        else parked++;
    }
    const int64_t v[8] = {(int64_t)s->seq, s->page_ins, s->page_outs, resident, parked, s->max_flight,
                          (int64_t)s->queue.size(), (int64_t)s->active.size()};
    for (int i = 0; i < n && i < 8; i++) out[i] = v[i];
    return FSE_OK;
}

int fse_server_tick_times(fse_server *s, float *ms, int cap, int *out_n) {
    if (!s || cap < 0) return FSE_E_INVAL;
    int rc = retire(s, false);
    if (rc) return rc;
    int m = std::min<int>(cap, (int)s->tick_ms.size());
    if (ms)
        for (int i = 0; i < m; i++) ms[i] = s->tick_ms[i];
    s->tick_ms.erase(s->tick_ms.begin(), s->tick_ms.begin() + m);
    if (out_n) *out_n = m;
    return FSE_OK;
}

}  // extern "C"
