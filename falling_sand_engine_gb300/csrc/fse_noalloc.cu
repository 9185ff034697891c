// fse_noalloc.cu -- one world::tick() on caller-owned device memory that allocates
// nothing.
//
// Some hosts cannot let a library call cudaMalloc: engines that hand out every
// byte of device memory from their own arena and enforce their own budget, and
// real-time loops that forbid allocation after start-up because cudaMalloc and
// cudaFree can block the device for milliseconds and can fail under memory
// pressure in the middle of a frame. fse_tick_noalloc serves them: the caller
// owns the cell planes and the output particle buffer, and the scratch the tick
// needs (chunk lists, per-chunk-pass spawn counters, spawn staging records, the
// world descriptor, the material table) lives in one file-scope __device__ array
// of fixed size, loaded with the library and held until the process exits.
//
// It runs the same colour-pass kernel and spawn scan as fse_world_tick, so its
// results are the same bit for bit.
#include <string.h>

#include <algorithm>

#include "fse_host.cuh"

namespace fse {
cudaError_t launch_spawn_scan(WorldDev *d_worlds, int n_worlds, cudaStream_t s);
}

using namespace fse;

namespace {

// limits of the allocation-free tick
constexpr int NA_MAX_SLOTS = 4096;      // chunks per colour (16384 x 16384 cells at chunk 128, 8192 x 8192 at 64)
constexpr int NA_MAX_ITER = 8;          // cell_iter
constexpr int NA_MAX_SPAWNS = 65536;    // particles spawned by one tick
constexpr int NA_CP = NA_MAX_ITER * 4 * NA_MAX_SLOTS + 1;

// byte layout of the scratch array
constexpr size_t OFF_DESC = 0;                                                        // WorldDev
constexpr size_t OFF_CTR = 1024;                                                      // 16 int counters
constexpr size_t OFF_MT = 2048;                                                       // MatTable
constexpr size_t OFF_LED = (OFF_MT + sizeof(MatTable) + 255) & ~(size_t)255;          // ledger
constexpr size_t OFF_ITEMS = (OFF_LED + LED_ROWS * MAXMAT * 8 + 255) & ~(size_t)255;  // 4 x slots
constexpr size_t OFF_CPC = (OFF_ITEMS + 4 * NA_MAX_SLOTS * 4 + 255) & ~(size_t)255;   // cp_count
constexpr size_t OFF_CPB = (OFF_CPC + NA_CP * 4 + 255) & ~(size_t)255;                // cp_base
constexpr size_t OFF_STAGE = (OFF_CPB + NA_CP * 4 + 255) & ~(size_t)255;              // SpawnRec
constexpr size_t NA_BYTES = OFF_STAGE + (size_t)NA_MAX_SPAWNS * sizeof(SpawnRec);
static_assert(sizeof(WorldDev) <= OFF_CTR - OFF_DESC, "the world descriptor overlaps the counters");
static_assert(16 * sizeof(int32_t) <= OFF_MT - OFF_CTR, "the counters overlap the material table");

}  // namespace

// The scratch of fse_tick_noalloc, about 4 MB. Every GPU that loads the library
// holds it until the process exits. Every call uses the same array, so calls whose
// work overlaps on the GPU (for example on two streams) race and must not be made.
static __device__ __align__(256) unsigned char g_noalloc_scratch[NA_BYTES];

namespace {

// host addresses of the array per device; looked up once per device, on the
// first call made while that device is current
constexpr int NA_MAX_DEVICES = 64;
unsigned char *g_scratch_ptr[NA_MAX_DEVICES] = {nullptr};

int scratch_for_current_device(unsigned char **out) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= NA_MAX_DEVICES) return FSE_E_CUDA;
    if (!g_scratch_ptr[dev]) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || p == nullptr) return FSE_E_CUDA;
        g_scratch_ptr[dev] = (unsigned char *)p;
    }
    *out = g_scratch_ptr[dev];
    return FSE_OK;
}

// spawn staging records -> the caller's fse_particle array, in the final order
__global__ void k_na_spawn_out(const WorldDev *__restrict__ wd, fse_particle *out) {
    const WorldDev &w = *wd;
    const int n = min(*w.stage_count, w.stage_cap);
    const int first = w.cp_base[w.cell_iter * 4 * w.max_slots];
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) {
        const SpawnRec s = w.stage[r];
        long long pos = (long long)first + w.cp_base[s.cp] + s.rank;
        if (pos >= w.part_cap) continue;
        fse_particle p;
        p.x = s.x;
        p.y = s.y;
        p.vx = s.vx;
        p.vy = s.vy;
        p.ax = 0.f;
        p.ay = s.ay;
        p.target_x = 0.f;
        p.target_y = 0.f;
        p.target_force = 0.f;
        p.lifetime = s.lifetime;
        p.fade_time = s.fade;
        p.colour = s.colour;
        p.scalar = s.scalar;
        p.id = s.id;
        p.flags = s.flags;
        p.bits = s.bits;
        p.temperature = s.temp;
        p.reserved = 0;
        out[pos] = p;
    }
}

}  // namespace

extern "C" int fse_tick_noalloc(uint16_t *id, uint32_t *colour, int32_t *scalar, uint8_t *flags, int32_t *diff,
                                int width, int height, int chunk_size, int cell_iter, uint32_t seed, uint32_t tick,
                                fse_particle *out_spawned, int spawn_cap, int *out_n_spawned, void *stream) {
    if (!id || !colour || !scalar || !flags || !diff || width <= 0 || height <= 0 || !out_n_spawned ||
        (spawn_cap > 0 && !out_spawned) || spawn_cap < 0)
        return FSE_E_INVAL;
    if (chunk_size == 0) chunk_size = 128;
    if (cell_iter == 0) cell_iter = 3;
    if (chunk_size < 16 || chunk_size > 128 || cell_iter < 1 || cell_iter > NA_MAX_ITER) return FSE_E_INVAL;
    const int nCx = ceil_div(width, chunk_size), nCy = ceil_div(height, chunk_size);
    const int max_slots = ceil_div(nCx, 2) * ceil_div(nCy, 2);
    if (max_slots > NA_MAX_SLOTS) return FSE_E_INVAL;  // world too large for the fixed scratch
    if ((long long)width * height > (1LL << 31) - 1) return FSE_E_INVAL;

    unsigned char *base = nullptr;
    int rc = scratch_for_current_device(&base);
    if (rc) return rc;
    cudaStream_t s = (cudaStream_t)stream;

    // descriptor: the caller's planes, scratch for everything else
    WorldDev h;
    memset(&h, 0, sizeof(h));
    int32_t *ctr = (int32_t *)(base + OFF_CTR);
    h.id = id;
    h.col = colour;
    h.sc = scalar;
    h.fl = flags;
    h.df = diff;
    h.W = width;
    h.H = height;
    h.C = chunk_size;
    h.cell_iter = cell_iter;
    h.seed = seed;
    h.nCx = nCx;
    h.nCy = nCy;
    h.zw = width;  // the tick zone is the whole world
    h.zh = height;
    h.max_slots = max_slots;
    h.cp_rows = 1;
    h.stage = (SpawnRec *)(base + OFF_STAGE);
    h.stage_cap = NA_MAX_SPAWNS;
    h.cp_count = (int32_t *)(base + OFF_CPC);
    h.cp_base = (int32_t *)(base + OFF_CPB);
    h.stage_count = ctr + 0;
    h.part_count = ctr + 1;  // spawns placed so far in the output
    h.part_cap = spawn_cap;
    h.req_count = ctr + 2;
    h.err = ctr + 5;
    h.tick = (uint32_t *)(ctr + 6);
    h.bar = (unsigned *)(ctr + 8);
    h.ledger = (long long *)(base + OFF_LED);

    // per-colour chunk slots of this world (a fixed host table: no heap either)
    static uint32_t items[4 * NA_MAX_SLOTS];
    int n_items[4];
    uint32_t *d_items[4];
    for (int tk = 0; tk < 4; tk++) {
        int ox = tk % 2, oy = 1 - tk / 2;
        int na = (nCx - ox + 1) / 2, nb = (nCy - oy + 1) / 2;
        n_items[tk] = std::max(0, na) * std::max(0, nb);
        for (int k = 0; k < n_items[tk]; k++) items[(size_t)tk * NA_MAX_SLOTS + k] = (uint32_t)k;
        d_items[tk] = (uint32_t *)(base + OFF_ITEMS) + (size_t)tk * NA_MAX_SLOTS;
    }

    // everything that must start at zero is cleared on every call: the counters
    // (spawn count, output count, error bits; the tick is the caller's), the ledger
    // and the per-chunk-pass spawn counts. The colour pass writes a count only for
    // the chunk slots a colour has, while the spawn scan sums max_slots of them per
    // colour, so counts left by an earlier call on a world of another shape would
    // otherwise shift this call's spawn order.
    int32_t c16[16] = {0};
    c16[6] = (int32_t)tick;
    const MatTable &mt = host_table();
    if (cudaMemcpyAsync(base + OFF_DESC, &h, sizeof(h), cudaMemcpyHostToDevice, s) != cudaSuccess ||
        cudaMemcpyAsync(base + OFF_CTR, c16, sizeof(c16), cudaMemcpyHostToDevice, s) != cudaSuccess ||
        cudaMemcpyAsync(base + OFF_MT, &mt, sizeof(MatTable), cudaMemcpyHostToDevice, s) != cudaSuccess ||
        cudaMemsetAsync(base + OFF_LED, 0, LED_ROWS * MAXMAT * 8, s) != cudaSuccess ||
        cudaMemsetAsync(base + OFF_CPC, 0, ((size_t)cell_iter * 4 * max_slots + 1) * sizeof(int32_t), s) !=
            cudaSuccess ||
        cudaMemcpyAsync(base + OFF_ITEMS, items, sizeof(items), cudaMemcpyHostToDevice, s) != cudaSuccess)
        return FSE_E_CUDA;

    WorldDev *d_desc = (WorldDev *)(base + OFF_DESC);
    const MatTable *d_mt = (const MatTable *)(base + OFF_MT);
    const int halo = mt.has_inter ? 5 : 2;
    for (int iter = 0; iter < cell_iter; iter++)
        for (int tk = 0; tk < 4; tk++)
            if (launch_colour_pass(d_desc, d_items[tk], n_items[tk], iter, tk, d_mt, halo, chunk_size, 1024, 0, s) !=
                cudaSuccess)
                return FSE_E_CUDA;
    if (launch_spawn_scan(d_desc, 1, s) != cudaSuccess) return FSE_E_CUDA;
    k_na_spawn_out<<<std::max(1, std::min(sm_count() * 2, ceil_div(NA_MAX_SPAWNS, 256))), 256, 0, s>>>(d_desc,
                                                                                                    out_spawned);
    if (cudaGetLastError() != cudaSuccess) return FSE_E_CUDA;
    int32_t back[16];
    if (cudaMemcpyAsync(back, base + OFF_CTR, sizeof(back), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
        return FSE_E_CUDA;
    *out_n_spawned = back[1];
    return status_from_err(back[5]);
}
