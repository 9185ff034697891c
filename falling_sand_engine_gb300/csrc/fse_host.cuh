// fse_host.cuh -- host-side structures shared by the C ABI translation units.
#pragma once

#include <cuda_runtime.h>

#include <map>
#include <string>
#include <vector>

#include "fse_internal.cuh"

namespace fse {
// CUDA events around each colour-pass launch, on the launching stream; read back
// lazily so timing adds no host synchronisation to the tick
struct PassTimer {
    std::vector<cudaEvent_t> pool;
    std::vector<std::pair<cudaEvent_t, cudaEvent_t>> pending;
    double ms = 0.0;
    long long launches = 0;
    // recording into a stream capture: the records become event nodes of the graph
    bool capture = false;
    // tick boundaries (batches): one group per enqueue call, n + 1 events for n ticks
    std::vector<std::vector<cudaEvent_t>> tick_groups;
    std::vector<float> tick_ms;  // duration of each tick read back so far
    cudaEvent_t get();
    cudaError_t record(cudaEvent_t e, cudaStream_t s) {
        return capture ? cudaEventRecordWithFlags(e, s, cudaEventRecordExternal) : cudaEventRecord(e, s);
    }
    void record_pair(cudaEvent_t a, cudaEvent_t b) { pending.push_back({a, b}); }
    void drain();  // after a synchronize: accumulate and recycle events
    // accumulate pairs and tick groups recorded by a graph replay (the events stay
    // with the graph)
    void accumulate(const std::vector<std::pair<cudaEvent_t, cudaEvent_t>> &pairs,
                    const std::vector<cudaEvent_t> &ticks);
};
}  // namespace fse

struct fse_world {
    int W, H, C, cell_iter;
    uint32_t seed;
    int part_cap, stage_cap;
    cudaStream_t stream;
    bool own_stream;
    bool seq;  // FSE_CFG_REFERENCE_ORDER: chunks updated in the reference's order
    fse::WorldDev h;      // host mirror of the device descriptor (pointers, sizes)
    fse::WorldDev *d;     // device descriptor
    uint32_t *items[4];   // chunk slots per colour
    int n_items[4];
    int32_t *ctr;         // small device counters
    uint32_t *claim;      // object stamp / readback claims (allocated on first use)
    uint8_t *mask_bits;   // object mask scratch (allocated on first use)
    uint32_t *obj_list;   // object list scratch
    size_t obj_list_cap;
    int64_t *obj_n;       // object list count
    std::map<int, cudaGraphExec_t> graphs;  // n_ticks -> step graph
    std::map<int, long long> graph_kernels;  // n_ticks -> kernels one replay launches
    size_t bytes;         // device bytes owned
    int threads, grid;    // colour-pass launch shape
    fse::PassTimer *timer;  // colour-pass event timer (enabled on request)
    // render state (FSE_CFG_RENDER): textures, smoothed flows, particle-layer owners,
    // per-material dirty counts
    uint32_t *tex[5];
    float *pflow;
    int32_t *owner;
    long long *moving;
    // solid-island scratch (allocated on first use): flood marks and their epoch,
    // labels and sizes, the flood's cell list, region image, results, island table
    uint32_t *isl_mark;
    uint32_t isl_epoch;
    int32_t *isl_lab, *isl_aux, *isl_list, *isl_out, *isl_seg;
    uint32_t *isl_pix;
    fse_island *isl_tab;
    int isl_tab_cap;
    // temperature read/write staging (allocated on first use)
    int16_t *temp_io;
    // the colour pass's tensor maps (h.tmap points here; NULL without TMA staging)
    void *tmaps;
    // array-of-structs tile staging (allocated on first use)
    uint8_t *tile_stage;
    size_t tile_stage_bytes;
    // pack / unpack scratch, grown on first use and kept until fse_world_trim
    void *pk_scr[16];
    size_t pk_scr_bytes[16];
};

namespace fse {

extern MatTable *g_dev_mt;
int ensure_materials_pushed();
const MatTable &host_table();

size_t colour_pass_smem(int C, int halo);
// temp: some world of the table keeps liquid temperatures (tp != NULL)
cudaError_t launch_colour_pass(const WorldDev *worlds, const uint32_t *items, int n_items, int iter, int tk,
                               const MatTable *mt, int halo, int C, int threads, int grid, cudaStream_t s,
                               bool temp = false, bool seq = false, bool f32 = false);
// every colour pass of a tick in one launch of `grid` CTAs (the fused tick)
cudaError_t launch_colour_fused(const WorldDev *worlds, const FusedTick &ft, const MatTable *mt, int halo, int C,
                                int grid, cudaStream_t s, bool temp);
cudaError_t launch_colour_fused_f32(const WorldDev *worlds, const FusedTick &ft, const MatTable *mt, int halo, int C,
                                    int grid, cudaStream_t s, bool temp);
cudaError_t launch_spawn_append(WorldDev *d_worlds, int n_worlds, int stage_blocks, cudaStream_t s);
cudaError_t launch_particle_tick(WorldDev *d_worlds, int n_worlds, const MatTable *mt, int move_blocks,
                                 cudaStream_t s);
constexpr int PARTICLE_TICK_LAUNCHES = 8;  // kernels launch_particle_tick issues
// world::tickTemperature over a set of worlds (max_tiles: the most 128 x 32 tiles of
// any of them); gated: only worlds with temp_on, after ticks whose index is 2 mod 4
cudaError_t launch_temperature(const WorldDev *d_worlds, int n_worlds, int max_tiles, const MatTable *mt, bool gated,
                               cudaStream_t s);
constexpr int TEMPERATURE_LAUNCHES = 2;
size_t temperature_scratch_cells(int W, int H);
int temperature_tiles(int W, int H);
void particle_prepare();
int particle_scan_blocks();
int sm_count();
int status_from_err(int err);
int tick_halo();

// one world::tick() + optionally world::tickCells() for a set of worlds that
// share a device descriptor table
int enqueue_step(WorldDev *d_worlds, int n_worlds, uint32_t *const items[4], const int n_items[4], int max_iter,
                 int C, int threads, int grid, bool particles, int move_blocks, int stage_blocks, cudaStream_t s,
                 PassTimer *timer = nullptr, int temp_tiles = 0, bool temp_track = false, bool seq = false,
                 bool f32 = false);
void count_launches(long long n);
// a world's plane upload (copies, flag masking, id check into *bad, repaint) and
// download, enqueued on stream s without waiting
int world_upload_async(fse_world *w, const uint16_t *id, const uint32_t *col, const int32_t *sc, const uint8_t *fl,
                       const int32_t *df, cudaStream_t s, int *bad);
int world_download_async(fse_world *w, uint16_t *id, uint32_t *col, int32_t *sc, uint8_t *fl, int32_t *df,
                         cudaStream_t s);
// the most temperature tiles of the worlds that run the temperature step (0: none)
int temp_tiles_of(const std::vector<fse_world *> &ws);
// some world keeps liquid temperatures: the colour pass that copies them runs
bool temp_track_of(const std::vector<fse_world *> &ws);

// Launch shapes of the colour pass (threads per CTA, chunk workers; 0 = one per chunk):
// 0 one 1024-thread CTA per chunk; 1 one persistent CTA per SM walking the chunks;
// 2 each chunk split over a CTA pair (a cluster of two 512-thread CTAs); 3 persistent
// pairs, two CTAs per SM; 4 the fused tick (every pass in one launch, one CTA per SM,
// chunk-passes started as their neighbourhoods finish), FUSED_GRID
constexpr int COLOUR_SHAPES = 5;
constexpr int FUSED_GRID = -1;
inline void colour_shape(int shape, int *threads, int *grid) {
    *threads = (shape == 2 || shape == 3) ? 512 : 1024;
    *grid = (shape == 1 || shape == 3) ? sm_count() : (shape == 4 ? FUSED_GRID : 0);
}

}  // namespace fse

#define FSE_CUDA_TRY(expr)                     \
    do {                                       \
        cudaError_t e_ = (expr);               \
        if (e_ != cudaSuccess) return FSE_E_CUDA; \
    } while (0)
