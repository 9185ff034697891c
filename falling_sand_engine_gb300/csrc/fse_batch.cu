// fse_batch.cu -- many worlds per launch, multi-tick CUDA graphs, the launch-shape
// autotuner, and the continuously batched serving loop.
//
// A batch owns a device table of the member worlds' descriptors (descriptors are
// immutable; all mutable per-world state lives behind their pointers), so one
// colour-pass launch walks the chunks of every world and one particle launch
// handles every world in blockIdx.y. Results are the same as ticking each world
// on its own: worlds never read each other's memory and every random draw is
// keyed on the world's own seed and tick.
#include <math.h>
#include <string.h>

#include <algorithm>
#include <chrono>
#include <deque>
#include <map>
#include <vector>

#include "fse_host.cuh"

using namespace fse;

struct fse_batch {
    std::vector<fse_world *> worlds;
    WorldDev *d_table = nullptr;
    uint32_t *items[4] = {nullptr, nullptr, nullptr, nullptr};
    int n_items[4] = {0, 0, 0, 0};
    int C = 128, max_iter = 0, move_blocks = 1, stage_blocks = 1;
    int max_move_blocks = 1;       // particle blocks per world that cover the largest list
    int threads = 1024, grid = 0;  // grid 0 = one CTA per chunk, else persistent CTAs
    cudaStream_t stream = nullptr;
    std::map<int, cudaGraphExec_t> graphs;
    std::map<int, long long> graph_kernels;  // kernels one replay launches
    // event timing (fse_batch_timing): colour-pass launches and tick boundaries;
    // graphs captured while it is on carry the events as nodes and are kept apart
    PassTimer *timer = nullptr;
    struct GraphEvents {
        std::vector<std::pair<cudaEvent_t, cudaEvent_t>> pairs;
        std::vector<cudaEvent_t> ticks;
    };
    std::map<int, cudaGraphExec_t> tgraphs;
    std::map<int, GraphEvents> tgraph_events;
    std::map<int, long long> tgraph_kernels;
};

namespace {

int build_tables(const std::vector<fse_world *> &ws, WorldDev **d_table, uint32_t *items[4], int n_items[4],
                 cudaStream_t s) {
    std::vector<WorldDev> tab(ws.size());
    std::vector<uint32_t> it[4];
    for (size_t i = 0; i < ws.size(); i++) {
        tab[i] = ws[i]->h;
        const WorldDev &h = ws[i]->h;
        for (int tk = 0; tk < 4; tk++) {
            int ox = tk % 2, oy = 1 - tk / 2;
            int na = (h.nCx - ox + 1) / 2, nb = (h.nCy - oy + 1) / 2;
            int ns = std::max(0, na) * std::max(0, nb);
            for (int sl = 0; sl < ns; sl++) it[tk].push_back(((uint32_t)i << 20) | (uint32_t)sl);
        }
    }
    if (*d_table) cudaFree(*d_table);
    if (cudaMalloc(d_table, std::max<size_t>(tab.size(), 1) * sizeof(WorldDev)) != cudaSuccess) return FSE_E_NOMEM;
    cudaMemcpyAsync(*d_table, tab.data(), tab.size() * sizeof(WorldDev), cudaMemcpyHostToDevice, s);
    for (int tk = 0; tk < 4; tk++) {
        if (items[tk]) cudaFree(items[tk]);
        items[tk] = nullptr;
        n_items[tk] = (int)it[tk].size();
        if (cudaMalloc(&items[tk], std::max<size_t>(it[tk].size(), 1) * 4) != cudaSuccess) return FSE_E_NOMEM;
        if (!it[tk].empty()) cudaMemcpyAsync(items[tk], it[tk].data(), it[tk].size() * 4, cudaMemcpyHostToDevice, s);
    }
    if (cudaStreamSynchronize(s) != cudaSuccess) return FSE_E_CUDA;
    return FSE_OK;
}

// the most temperature tiles of the worlds that run the temperature step (0: none)
int temp_tiles_of(const std::vector<fse_world *> &ws) {
    int t = 0;
    for (const fse_world *w : ws)
        if (w->h.temp_on) t = std::max(t, temperature_tiles(w->W, w->H));
    return t;
}
// some world keeps liquid temperatures: the colour pass that copies them runs
bool temp_track_of(const std::vector<fse_world *> &ws) {
    for (const fse_world *w : ws)
        if (w->h.tp) return true;
    return false;
}

int batch_enqueue(fse_batch *b, int n) {
    int rc = ensure_materials_pushed();
    if (rc) return rc;
    const int tt = temp_tiles_of(b->worlds);
    const bool tr = temp_track_of(b->worlds);
    PassTimer *tm = b->timer;
    std::vector<cudaEvent_t> ticks;  // tick boundaries: n + 1 events
    auto boundary = [&]() -> int {
        if (!tm) return FSE_OK;
        cudaEvent_t e = tm->get();
        ticks.push_back(e);
        return tm->record(e, b->stream) == cudaSuccess ? FSE_OK : FSE_E_CUDA;
    };
    for (int i = 0; i < n; i++) {
        if ((rc = boundary())) return rc;
        rc = enqueue_step(b->d_table, (int)b->worlds.size(), b->items, b->n_items, b->max_iter, b->C, b->threads,
                          b->grid, true, b->move_blocks, b->stage_blocks, b->stream, tm, tt, tr, false,
                          b->worlds[0]->h.f32 != 0);
        if (rc) return rc;
    }
    if (n > 0 && (rc = boundary())) return rc;
    if (tm && !ticks.empty()) tm->tick_groups.push_back(ticks);
    return FSE_OK;
}

void drop_timed_graphs(fse_batch *b) {
    for (auto &g : b->tgraphs) cudaGraphExecDestroy(g.second);
    for (auto &g : b->tgraph_events) {
        for (auto &pr : g.second.pairs) {
            cudaEventDestroy(pr.first);
            cudaEventDestroy(pr.second);
        }
        for (cudaEvent_t e : g.second.ticks) cudaEventDestroy(e);
    }
    b->tgraphs.clear();
    b->tgraph_events.clear();
    b->tgraph_kernels.clear();
}

int batch_sync(fse_batch *b) {
    if (cudaStreamSynchronize(b->stream) != cudaSuccess) return FSE_E_CUDA;
    int worst = FSE_OK;
    for (fse_world *w : b->worlds) {
        int rc = fse_world_sync(w);
        if (rc && !worst) worst = rc;
    }
    return worst;
}

// ---- snapshots: device-side copies of everything a step mutates
struct Snapshot {
    std::vector<void *> bufs;
    std::vector<std::pair<void *, size_t>> src;
};

bool snap_take(fse_world *w, Snapshot &s, cudaStream_t st) {
    size_t n = (size_t)w->W * w->H;
    const WorldDev &h = w->h;
    std::vector<std::pair<void *, size_t>> list = {
        {h.id, n * 2}, {h.col, n * 4}, {h.sc, n * 4}, {h.fl, n}, {h.df, n * 4}, {h.tp, n * 2}, {w->ctr, 64},
        {h.ledger, LED_ROWS * MAXMAT * 8}};
    const PartSoA &p = h.p;
    size_t pc = (size_t)w->part_cap;
    void *pa[] = {p.x, p.y, p.vx, p.vy, p.ax, p.ay, p.tx, p.ty, p.tf, p.life, p.fade, p.col, p.sc};
    for (void *q : pa) list.push_back({q, pc * 4});
    list.push_back({p.id, pc * 2});
    list.push_back({p.tp, pc * 2});
    list.push_back({p.fl, pc});
    list.push_back({p.bits, pc});
    for (auto &e : list) {
        if (!e.first) continue;  // planes the world does not keep
        void *d = nullptr;
        if (cudaMalloc(&d, e.second) != cudaSuccess) return false;
        cudaMemcpyAsync(d, e.first, e.second, cudaMemcpyDeviceToDevice, st);
        s.bufs.push_back(d);
        s.src.push_back(e);
    }
    return true;
}
void snap_restore(Snapshot &s, cudaStream_t st) {
    for (size_t i = 0; i < s.bufs.size(); i++)
        cudaMemcpyAsync(s.src[i].first, s.bufs[i], s.src[i].second, cudaMemcpyDeviceToDevice, st);
}
void snap_free(Snapshot &s) {
    for (void *d : s.bufs) cudaFree(d);
    s.bufs.clear();
    s.src.clear();
}

}  // namespace

extern "C" {

int fse_batch_create(fse_world **worlds, int n, fse_batch **out) {
    if (!worlds || n <= 0 || !out || n > 4095) return FSE_E_INVAL;
    fse_batch *b = new fse_batch();
    for (int i = 0; i < n; i++) {
        if (!worlds[i]) {
            delete b;
            return FSE_E_INVAL;
        }
        if ((i > 0 && (worlds[i]->C != worlds[0]->C || worlds[i]->h.f32 != worlds[0]->h.f32)) || worlds[i]->seq) {
            delete b;
            // one shared-memory tile shape and one kind of liquid amounts per launch;
            // partitioned order only
            return FSE_E_INVAL;
        }
        b->worlds.push_back(worlds[i]);
        b->max_iter = std::max(b->max_iter, worlds[i]->cell_iter);
        b->max_move_blocks = std::max(b->max_move_blocks, std::min(sm_count() * 2, ceil_div(worlds[i]->part_cap, 256)));
        b->move_blocks = b->max_move_blocks;
        b->stage_blocks = std::max(b->stage_blocks, std::min(sm_count(), ceil_div(worlds[i]->stage_cap, 256)));
    }
    b->C = worlds[0]->C;
    if (cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess) {
        delete b;
        return FSE_E_CUDA;
    }
    for (fse_world *w : b->worlds) cudaStreamSynchronize(w->stream);
    int rc = build_tables(b->worlds, &b->d_table, b->items, b->n_items, b->stream);
    if (rc) {
        fse_batch_destroy(b);
        return rc;
    }
    *out = b;
    return FSE_OK;
}

int fse_batch_destroy(fse_batch *b) {
    if (!b) return FSE_E_INVAL;
    if (b->stream) cudaStreamSynchronize(b->stream);
    for (auto &g : b->graphs) cudaGraphExecDestroy(g.second);
    drop_timed_graphs(b);
    if (b->timer) {
        b->timer->drain();
        for (cudaEvent_t e : b->timer->pool) cudaEventDestroy(e);
        delete b->timer;
    }
    if (b->d_table) cudaFree(b->d_table);
    for (int k = 0; k < 4; k++)
        if (b->items[k]) cudaFree(b->items[k]);
    if (b->stream) cudaStreamDestroy(b->stream);
    delete b;
    return FSE_OK;
}

int fse_batch_step(fse_batch *b, int n) {
    if (!b || n < 0) return FSE_E_INVAL;
    int rc = batch_enqueue(b, n);
    if (rc) return rc;
    return batch_sync(b);
}

}  // extern "C"

// The graph of k steps for the batch's current timing mode, captured on first use.
// With timing on, graphs carry event nodes and are kept apart from the plain ones.
static int batch_graph(fse_batch *b, int k, cudaGraphExec_t *out) {
    const bool timed = b->timer != nullptr;
    auto &graphs = timed ? b->tgraphs : b->graphs;
    auto &kernels = timed ? b->tgraph_kernels : b->graph_kernels;
    auto it = graphs.find(k);
    if (it != graphs.end()) {
        *out = it->second;
        return FSE_OK;
    }
    cudaGraph_t g;
    cudaGraphExec_t ex;
    // kernels are counted when a replay launches them, not at capture
    const long long c0 = fse_launch_counter();
    FSE_CUDA_TRY(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
    if (timed) b->timer->capture = true;
    int erc = batch_enqueue(b, k);
    cudaError_t e = cudaStreamEndCapture(b->stream, &g);
    const long long kn = fse_launch_counter() - c0;
    count_launches(-kn);
    if (timed) {
        // the events recorded during capture belong to this graph from now on
        fse_batch::GraphEvents ge;
        ge.pairs.swap(b->timer->pending);
        if (!b->timer->tick_groups.empty()) {
            ge.ticks.swap(b->timer->tick_groups.back());
            b->timer->tick_groups.pop_back();
        }
        b->timer->capture = false;
        b->tgraph_events[k] = std::move(ge);
    }
    if (erc || e != cudaSuccess) return FSE_E_CUDA;
    FSE_CUDA_TRY(cudaGraphInstantiate(&ex, g, 0));
    cudaGraphDestroy(g);
    graphs[k] = ex;
    kernels[k] = kn;
    *out = ex;
    return FSE_OK;
}

extern "C" {

int fse_batch_step_graph(fse_batch *b, int n, int graph_ticks) {
    if (!b || n < 0) return FSE_E_INVAL;
    if (graph_ticks <= 0) graph_ticks = 32;
    int rc = ensure_materials_pushed();
    if (rc) return rc;
    const bool timed = b->timer != nullptr;
    int done = 0;
    while (done < n) {
        const int k = std::min(graph_ticks, n - done);
        cudaGraphExec_t ex;
        if ((rc = batch_graph(b, k, &ex))) return rc;
        FSE_CUDA_TRY(cudaGraphLaunch(ex, b->stream));
        count_launches(timed ? b->tgraph_kernels[k] : b->graph_kernels[k]);
        if (timed) {
            // each replay is read back before the next one reuses its events
            const fse_batch::GraphEvents &ge = b->tgraph_events[k];
            if (!ge.ticks.empty()) FSE_CUDA_TRY(cudaEventSynchronize(ge.ticks.back()));
            b->timer->accumulate(ge.pairs, ge.ticks);
        }
        done += k;
    }
    return batch_sync(b);
}

int fse_batch_prepare_graphs(fse_batch *b, int n, int graph_ticks) {
    if (!b || n < 0) return FSE_E_INVAL;
    if (graph_ticks <= 0) graph_ticks = 32;
    int rc = ensure_materials_pushed();
    if (rc) return rc;
    for (int done = 0; done < n;) {
        const int k = std::min(graph_ticks, n - done);
        cudaGraphExec_t ex;
        if ((rc = batch_graph(b, k, &ex))) return rc;
        done += k;
    }
    return FSE_OK;
}

int fse_batch_timing(fse_batch *b, int enable, double *out_pass_ms, int64_t *out_pass_launches, float *tick_ms,
                     int cap, int *out_ticks) {
    if (!b || cap < 0 || (cap > 0 && !tick_ms)) return FSE_E_INVAL;
    FSE_CUDA_TRY(cudaStreamSynchronize(b->stream));
    PassTimer *tm = b->timer;
    if (tm) tm->drain();
    if (out_pass_ms) *out_pass_ms = tm ? tm->ms : 0.0;
    if (out_pass_launches) *out_pass_launches = tm ? tm->launches : 0;
    const int nt = tm ? (int)tm->tick_ms.size() : 0;
    if (out_ticks) *out_ticks = nt;
    for (int i = 0; i < std::min(cap, nt); i++) tick_ms[i] = tm->tick_ms[i];
    if (enable) {
        if (!b->timer) b->timer = new PassTimer();
        b->timer->ms = 0.0;
        b->timer->launches = 0;
        b->timer->tick_ms.clear();
    } else if (tm) {
        drop_timed_graphs(b);
        for (cudaEvent_t e : tm->pool) cudaEventDestroy(e);
        delete tm;
        b->timer = nullptr;
    }
    return FSE_OK;
}

int fse_batch_set_launch(fse_batch *b, int colour_ctas_per_sm, int particle_blocks) {
    if (!b || colour_ctas_per_sm < 0 || colour_ctas_per_sm > 3 || particle_blocks < 0) return FSE_E_INVAL;
    colour_shape(colour_ctas_per_sm, &b->threads, &b->grid);
    b->move_blocks = particle_blocks == 0 ? b->max_move_blocks : std::min(particle_blocks, b->max_move_blocks);
    for (auto &g : b->graphs) cudaGraphExecDestroy(g.second);
    b->graphs.clear();
    drop_timed_graphs(b);
    return FSE_OK;
}

// Time each launch shape on the batch itself and put every world back as it
// was. The shape never changes results: a chunk's pass does not depend on which
// CTA runs it or when, and particle kernels stride over their lists whatever the
// grid. Knobs: the colour-pass grid (one CTA per chunk, scheduled by the hardware,
// or one persistent CTA per SM walking the chunk list) and the number of blocks
// each world's particle kernels get (batches of small worlds waste launches on
// empty blocks).
int fse_batch_autotune(fse_batch *b, int32_t out_choice[4]) {
    if (!b) return FSE_E_INVAL;
    int rc = batch_sync(b);
    if (rc) return rc;
    std::vector<Snapshot> snaps(b->worlds.size());
    for (size_t i = 0; i < b->worlds.size(); i++)
        if (!snap_take(b->worlds[i], snaps[i], b->stream)) {
            for (auto &s : snaps) snap_free(s);
            return FSE_E_NOMEM;
        }
    // the candidates' steps are not part of any timing the caller asked for
    PassTimer *keep_timer = b->timer;
    b->timer = nullptr;
    const int cand[][2] = {{0, 0}, {1, 0}, {0, 4}, {0, 16}, {1, 16}, {2, 4}, {3, 4}, {2, 16}};
    const int n_cand = (int)(sizeof(cand) / sizeof(cand[0]));
    float best = 1e30f;
    int bi = 0;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    for (int c = 0; c < n_cand; c++) {
        fse_batch_set_launch(b, cand[c][0], cand[c][1]);
        batch_enqueue(b, 1);  // warm-up
        cudaEventRecord(e0, b->stream);
        batch_enqueue(b, 2);
        cudaEventRecord(e1, b->stream);
        cudaEventSynchronize(e1);
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        for (auto &s : snaps) snap_restore(s, b->stream);
        if (ms < best) {
            best = ms;
            bi = c;
        }
    }
    cudaStreamSynchronize(b->stream);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    for (auto &s : snaps) snap_free(s);
    b->timer = keep_timer;
    fse_batch_set_launch(b, cand[bi][0], cand[bi][1]);
    if (out_choice) {
        out_choice[0] = cand[bi][0];
        out_choice[1] = cand[bi][1];
        out_choice[2] = (int32_t)(best * 1000.f);
        out_choice[3] = bi;
    }
    return batch_sync(b);
}

int fse_batch_sync(fse_batch *b) {
    if (!b) return FSE_E_INVAL;
    return batch_sync(b);
}

void *fse_batch_stream(fse_batch *b) { return b ? (void *)b->stream : nullptr; }

}  // extern "C"

// ================================================================ serving
struct fse_server {
    int64_t budget, in_use = 0;
    int max_active;
    std::vector<fse_world *> slots;
    std::vector<int64_t> slot_bytes;
    struct Req {
        int64_t id;
        int slot, left;
        double arrival;
    };
    std::deque<Req> queue;
    std::vector<Req> active;
    std::vector<std::pair<int64_t, double>> done;
    int64_t next_id = 0;
    // batch tables for the current active set
    WorldDev *d_table = nullptr;
    uint32_t *items[4] = {nullptr, nullptr, nullptr, nullptr};
    int n_items[4] = {0, 0, 0, 0};
    std::vector<int> table_slots;
    cudaStream_t stream = nullptr;
    int C = 128;
    std::chrono::steady_clock::time_point t0;
};

static int64_t world_footprint(int w, int h, const fse_config *cfg) {
    long long cells = (long long)w * h;
    long long pc = (cfg && cfg->particle_capacity > 0) ? cfg->particle_capacity : std::max<long long>(65536, cells / 4);
    long long sc = (cfg && cfg->spawn_capacity > 0) ? cfg->spawn_capacity : pc;
    // planes; two particle SoAs, the outcome byte, four outcome words and two merge-list words
    return cells * 15 + pc * (2 * 56 + 1 + 4 * 6) + sc * (long long)sizeof(SpawnRec) + (1 << 20);
}

extern "C" {

int fse_server_create(int64_t budget, int max_active, fse_server **out) {
    if (!out || budget <= 0 || max_active <= 0) return FSE_E_INVAL;
    fse_server *s = new fse_server();
    s->budget = budget;
    s->max_active = max_active;
    if (cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking) != cudaSuccess) {
        delete s;
        return FSE_E_CUDA;
    }
    s->t0 = std::chrono::steady_clock::now();
    *out = s;
    return FSE_OK;
}

int fse_server_destroy(fse_server *s) {
    if (!s) return FSE_E_INVAL;
    cudaStreamSynchronize(s->stream);
    for (fse_world *w : s->slots)
        if (w) fse_world_destroy(w);
    if (s->d_table) cudaFree(s->d_table);
    for (int k = 0; k < 4; k++)
        if (s->items[k]) cudaFree(s->items[k]);
    cudaStreamDestroy(s->stream);
    delete s;
    return FSE_OK;
}

int fse_server_add_world(fse_server *s, int w, int h, const fse_config *cfg, int gen_kind, uint32_t gen_seed,
                         int *out_slot) {
    if (!s || !out_slot) return FSE_E_INVAL;
    int64_t need = world_footprint(w, h, cfg);
    if (s->in_use + need > s->budget) return FSE_E_BUDGET;
    fse_config c{};
    if (cfg) c = *cfg;
    if (c.chunk_size == 0) c.chunk_size = 128;
    // servers batch their worlds in the partitioned order with Q16.16 amounts
    if (c.flags & (FSE_CFG_REFERENCE_ORDER | FSE_CFG_F32_FLUID)) return FSE_E_INVAL;
    if (!s->slots.empty()) {
        for (fse_world *x : s->slots)
            if (x && x->C != c.chunk_size) return FSE_E_INVAL;
    }
    c.stream = (void *)s->stream;
    fse_world *wd = nullptr;
    int rc = fse_world_create(w, h, &c, &wd);
    if (rc) return rc;
    rc = fse_world_generate(wd, gen_kind, gen_seed);
    if (rc) {
        fse_world_destroy(wd);
        return rc;
    }
    s->C = c.chunk_size;
    int slot = -1;
    for (size_t i = 0; i < s->slots.size(); i++)
        if (!s->slots[i]) slot = (int)i;
    if (slot < 0) {
        slot = (int)s->slots.size();
        s->slots.push_back(nullptr);
        s->slot_bytes.push_back(0);
    }
    s->slots[slot] = wd;
    s->slot_bytes[slot] = (int64_t)wd->bytes;
    s->in_use += (int64_t)wd->bytes;
    *out_slot = slot;
    return FSE_OK;
}

int fse_server_remove_world(fse_server *s, int slot) {
    if (!s || slot < 0 || slot >= (int)s->slots.size() || !s->slots[slot]) return FSE_E_INVAL;
    for (auto &r : s->active)
        if (r.slot == slot) return FSE_E_STATE;
    for (auto &r : s->queue)
        if (r.slot == slot) return FSE_E_STATE;
    fse_world_destroy(s->slots[slot]);
    s->slots[slot] = nullptr;
    s->in_use -= s->slot_bytes[slot];
    s->slot_bytes[slot] = 0;
    return FSE_OK;
}

int64_t fse_server_bytes_in_use(const fse_server *s) { return s ? s->in_use : -1; }

double fse_server_now_us(const fse_server *s) {
    if (!s) return 0.0;
    return std::chrono::duration<double, std::micro>(std::chrono::steady_clock::now() - s->t0).count();
}

fse_world *fse_server_world(fse_server *s, int slot) {
    if (!s || slot < 0 || slot >= (int)s->slots.size()) return nullptr;
    return s->slots[slot];
}

int fse_server_submit(fse_server *s, int slot, int n_ticks, double arrival_us, int64_t *out_request) {
    if (!s || slot < 0 || slot >= (int)s->slots.size() || !s->slots[slot] || n_ticks <= 0) return FSE_E_INVAL;
    fse_server::Req r{s->next_id++, slot, n_ticks, arrival_us};
    s->queue.push_back(r);
    if (out_request) *out_request = r.id;
    return FSE_OK;
}

// one scheduling step: admit queued requests while slots are free (one request
// per world at a time, arrival order), tick every active world once in one
// batched launch sequence, retire finished requests
int fse_server_step(fse_server *s, int *out_active) {
    if (!s) return FSE_E_INVAL;
    bool changed = false;
    for (auto it = s->queue.begin(); it != s->queue.end() && (int)s->active.size() < s->max_active;) {
        bool busy = false;
        for (auto &a : s->active)
            if (a.slot == it->slot) busy = true;
        if (busy) {
            ++it;
            continue;
        }
        s->active.push_back(*it);
        it = s->queue.erase(it);
        changed = true;
    }
    if (out_active) *out_active = (int)s->active.size();
    if (s->active.empty()) return FSE_OK;
    std::vector<int> want;
    for (auto &a : s->active) want.push_back(a.slot);
    std::sort(want.begin(), want.end());
    if (changed || want != s->table_slots) {
        std::vector<fse_world *> ws;
        for (int sl : want) ws.push_back(s->slots[sl]);
        int rc = build_tables(ws, &s->d_table, s->items, s->n_items, s->stream);
        if (rc) return rc;
        s->table_slots = want;
    }
    int max_iter = 0, mb = 1, sb = 1;
    for (int sl : want) {
        fse_world *w = s->slots[sl];
        max_iter = std::max(max_iter, w->cell_iter);
        mb = std::max(mb, std::min(sm_count() * 2, ceil_div(w->part_cap, 256)));
        sb = std::max(sb, std::min(sm_count(), ceil_div(w->stage_cap, 256)));
    }
    int rc = ensure_materials_pushed();
    if (rc) return rc;
    std::vector<fse_world *> act;
    for (int sl : want) act.push_back(s->slots[sl]);
    rc = enqueue_step(s->d_table, (int)want.size(), s->items, s->n_items, max_iter, s->C, 1024, 0, true, mb, sb,
                      s->stream, nullptr, temp_tiles_of(act), temp_track_of(act));
    if (rc) return rc;
    if (cudaStreamSynchronize(s->stream) != cudaSuccess) return FSE_E_CUDA;
    double now = std::chrono::duration<double, std::micro>(std::chrono::steady_clock::now() - s->t0).count();
    std::vector<fse_server::Req> keep;
    for (auto &a : s->active) {
        a.left--;
        if (a.left <= 0)
            s->done.push_back({a.id, now});
        else
            keep.push_back(a);
    }
    s->active.swap(keep);
    return FSE_OK;
}

int fse_server_poll(fse_server *s, double now_us, int64_t *ids, double *done_us, int cap, int *out_n) {
    (void)now_us;
    if (!s || cap < 0) return FSE_E_INVAL;
    int m = std::min<int>(cap, (int)s->done.size());
    for (int i = 0; i < m; i++) {
        if (ids) ids[i] = s->done[i].first;
        if (done_us) done_us[i] = s->done[i].second;
    }
    s->done.erase(s->done.begin(), s->done.begin() + m);
    if (out_n) *out_n = m;
    return FSE_OK;
}

}  // extern "C"
