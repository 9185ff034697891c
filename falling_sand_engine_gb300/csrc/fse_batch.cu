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
    // the colour pass's launch shape (colour_shape): the fused tick until the autotuner
    // or fse_batch_set_launch chooses
    int threads = CP_THREADS, grid = FUSED_GRID;
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
    // whole-batch plane I/O (fse_batch_upload_all / download_all): every member's
    // planes in one device buffer laid out as the host buffer, and the segment table
    // that scatters it into the members' planes (allocated on first use)
    uint8_t *io_stage = nullptr;
    void *io_segs = nullptr;
    int io_nseg = 0;
    int64_t io_bytes = 0;
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

}  // namespace

// the most temperature tiles of the worlds that run the temperature step (0: none)
int fse::temp_tiles_of(const std::vector<fse_world *> &ws) {
    int t = 0;
    for (const fse_world *w : ws)
        if (w->h.temp_on) t = std::max(t, temperature_tiles(w->W, w->H));
    return t;
}
// some world keeps liquid temperatures: the colour pass that copies them runs
bool fse::temp_track_of(const std::vector<fse_world *> &ws) {
    for (const fse_world *w : ws)
        if (w->h.tp) return true;
    return false;
}

namespace {

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

// ---- whole-batch plane I/O: planes id, colour, scalar, flags, diff of every member,
// each starting on a 16-byte boundary of one buffer
constexpr int IO_PLANES = 5;
inline int64_t io_plane_size(int p) { return p == 0 ? 2 : (p == 3 ? 1 : 4); }

struct IoSeg {
    uint8_t *dev;    // the member's plane
    int64_t off;     // its place in the buffer
    int64_t bytes;
    int kind;        // 0 copy, 1 material ids (checked on upload), 2 flags (visited bit cleared on upload)
    int *bad;        // the member's flag for replaced ids
};

// one segment per blockIdx.y; 16-byte words by the grid-stride loop, the tail by bytes
__global__ void k_io_segments(const IoSeg *__restrict__ segs, uint8_t *stage, int up, int nmat, int air) {
    const IoSeg sg = segs[blockIdx.y];
    uint8_t *buf = stage + sg.off;
    const int64_t nv = sg.bytes >> 4;
    const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x, stride = (int64_t)gridDim.x * blockDim.x;
    bool bad = false;
    for (int64_t v = tid; v < nv; v += stride) {
        if (!up) {
            reinterpret_cast<uint4 *>(buf)[v] = reinterpret_cast<const uint4 *>(sg.dev)[v];
            continue;
        }
        uint4 q = reinterpret_cast<const uint4 *>(buf)[v];
        if (sg.kind == 2) {
            q.x &= ~0x40404040u;  // bit 6 of a flags byte is the kernel's visited mark
            q.y &= ~0x40404040u;
            q.z &= ~0x40404040u;
            q.w &= ~0x40404040u;
        } else if (sg.kind == 1) {
            uint32_t *u = &q.x;
            for (int k = 0; k < 4; k++) {
                uint32_t lo = u[k] & 0xFFFFu, hi = u[k] >> 16;
                if ((int)lo >= nmat) lo = (uint32_t)air, bad = true;
                if ((int)hi >= nmat) hi = (uint32_t)air, bad = true;
                u[k] = lo | (hi << 16);
            }
        }
        reinterpret_cast<uint4 *>(sg.dev)[v] = q;
    }
    // the last bytes (fewer than 16): whole cells, by thread 0 of block 0
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        for (int64_t i = nv << 4; i < sg.bytes; i++) {
            if (!up) {
                buf[i] = sg.dev[i];
            } else if (sg.kind == 1) {
                if ((i & 1) == 0) {
                    uint16_t idv = (uint16_t)(buf[i] | (buf[i + 1] << 8));
                    if ((int)idv >= nmat) idv = (uint16_t)air, bad = true;
                    sg.dev[i] = (uint8_t)idv;
                    sg.dev[i + 1] = (uint8_t)(idv >> 8);
                }
            } else {
                sg.dev[i] = sg.kind == 2 ? (uint8_t)(buf[i] & ~0x40u) : buf[i];
            }
        }
    }
    if (bad) atomicOr(sg.bad, 1);
}

int batch_io_prepare(fse_batch *b) {
    int64_t total = 0;
    fse_batch_io_layout(b, nullptr, &total);
    if (b->io_stage && b->io_bytes == total) return FSE_OK;
    if (b->io_stage) cudaFree(b->io_stage);
    if (b->io_segs) cudaFree(b->io_segs);
    b->io_stage = nullptr;
    b->io_segs = nullptr;
    std::vector<IoSeg> segs;
    int64_t at = 0;
    for (fse_world *w : b->worlds) {
        const int64_t n = (int64_t)w->W * w->H;
        uint8_t *planes[IO_PLANES] = {(uint8_t *)w->h.id, (uint8_t *)w->h.col, (uint8_t *)w->h.sc, w->h.fl,
                                      (uint8_t *)w->h.df};
        for (int p = 0; p < IO_PLANES; p++) {
            const int64_t nb = n * io_plane_size(p);
            segs.push_back({planes[p], at, nb, p == 0 ? 1 : (p == 3 ? 2 : 0), w->ctr + 15});
            at += (nb + 15) & ~(int64_t)15;
        }
    }
    if (cudaMalloc(&b->io_stage, (size_t)std::max<int64_t>(total, 16)) != cudaSuccess ||
        cudaMalloc(&b->io_segs, segs.size() * sizeof(IoSeg)) != cudaSuccess) {
        cudaGetLastError();
        return FSE_E_NOMEM;
    }
    if (cudaMemcpy(b->io_segs, segs.data(), segs.size() * sizeof(IoSeg), cudaMemcpyHostToDevice) != cudaSuccess)
        return FSE_E_CUDA;
    b->io_nseg = (int)segs.size();
    b->io_bytes = total;
    return FSE_OK;
}

int launch_io_segments(fse_batch *b, bool up) {
    if (b->io_nseg == 0) return FSE_OK;
    int rc = ensure_materials_pushed();
    if (rc) return rc;
    const MatTable &t = host_table();
    // enough blocks per segment for the largest member's planes
    int64_t most = 0;
    for (fse_world *w : b->worlds) most = std::max<int64_t>(most, (int64_t)w->W * w->H * 4);
    const int per_seg = (int)std::min<int64_t>(256, std::max<int64_t>(1, (most / 16 + 255) / 256 / 8));
    for (int s0 = 0; s0 < b->io_nseg; s0 += 65535) {
        dim3 g(per_seg, std::min(65535, b->io_nseg - s0));
        k_io_segments<<<g, 256, 0, b->stream>>>(reinterpret_cast<const IoSeg *>(b->io_segs) + s0, b->io_stage,
                                                up ? 1 : 0, t.n, t.id_air);
    }
    count_launches(1);
    return cudaGetLastError() == cudaSuccess ? FSE_OK : FSE_E_CUDA;
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
    if (b->io_stage) cudaFree(b->io_stage);
    if (b->io_segs) cudaFree(b->io_segs);
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

int fse_batch_enqueue(fse_batch *b, int n) {
    if (!b || n < 0) return FSE_E_INVAL;
    return batch_enqueue(b, n);
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
    if (!b || colour_ctas_per_sm < 0 || colour_ctas_per_sm >= COLOUR_SHAPES || particle_blocks < 0)
        return FSE_E_INVAL;
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
// grid. Knobs: the colour-pass shape (one CTA per chunk scheduled by the hardware,
// one persistent CTA per SM walking the chunk list, a CTA pair per chunk, or the
// fused tick with every pass in one launch) and the number of blocks each world's
// particle kernels get (batches of small worlds waste launches on empty blocks).
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
    const int cand[][2] = {{0, 0}, {1, 0}, {4, 0}, {0, 4}, {0, 16}, {4, 16}, {1, 16}, {2, 4}};
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

int fse_batch_io_layout(fse_batch *b, int64_t *offsets, int64_t *out_bytes) {
    if (!b) return FSE_E_INVAL;
    int64_t at = 0;
    for (size_t k = 0; k < b->worlds.size(); k++) {
        const int64_t n = (int64_t)b->worlds[k]->W * b->worlds[k]->H;
        for (int p = 0; p < IO_PLANES; p++) {
            if (offsets) offsets[IO_PLANES * k + p] = at;
            at += (n * io_plane_size(p) + 15) & ~(int64_t)15;
        }
    }
    if (out_bytes) *out_bytes = at;
    return FSE_OK;
}

int fse_batch_upload_all(fse_batch *b, const void *host, int64_t bytes) {
    if (!b || !host) return FSE_E_INVAL;
    int rc = batch_io_prepare(b);
    if (rc) return rc;
    if (bytes != b->io_bytes) return FSE_E_INVAL;
    FSE_CUDA_TRY(cudaMemcpyAsync(b->io_stage, host, (size_t)bytes, cudaMemcpyHostToDevice, b->stream));
    rc = launch_io_segments(b, true);
    if (rc) return rc;
    for (fse_world *w : b->worlds)  // repaint everything
        if (w->h.dirty) FSE_CUDA_TRY(cudaMemsetAsync(w->h.dirty, 1, (size_t)w->W * w->H, b->stream));
    return FSE_OK;
}

int fse_batch_download_all(fse_batch *b, void *host, int64_t bytes) {
    if (!b || !host) return FSE_E_INVAL;
    int rc = batch_io_prepare(b);
    if (rc) return rc;
    if (bytes != b->io_bytes) return FSE_E_INVAL;
    rc = launch_io_segments(b, false);
    if (rc) return rc;
    FSE_CUDA_TRY(cudaMemcpyAsync(host, b->io_stage, (size_t)bytes, cudaMemcpyDeviceToHost, b->stream));
    return FSE_OK;
}

int fse_batch_upload(fse_batch *b, int index, const uint16_t *id, const uint32_t *col, const int32_t *sc,
                     const uint8_t *fl, const int32_t *df) {
    if (!b || index < 0 || index >= (int)b->worlds.size()) return FSE_E_INVAL;
    fse_world *w = b->worlds[index];
    return world_upload_async(w, id, col, sc, fl, df, b->stream, w->ctr + 15);
}

int fse_batch_download(fse_batch *b, int index, uint16_t *id, uint32_t *col, int32_t *sc, uint8_t *fl, int32_t *df) {
    if (!b || index < 0 || index >= (int)b->worlds.size()) return FSE_E_INVAL;
    return world_download_async(b->worlds[index], id, col, sc, fl, df, b->stream);
}

}  // extern "C"
