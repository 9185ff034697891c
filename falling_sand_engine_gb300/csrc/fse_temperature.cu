// fse_temperature.cu -- world::tickTemperature (source/engine/world.cpp:1950-2004):
// heat conduction between neighbouring cells, a Jacobi step of a 3x3 stencil.
//
// Per cell (x, y), over the nine cells (x + xa, y + ya) in the order of the
// reference's FN(...) list (xa = -1, 0, 1 outer; ya = -1, 0, 1 inner), each
// neighbour with temperature t != 0 adds
//     factor = (float)(abs(t) / 64) * conductionOther      (integer division first)
//     v += (float)t * factor;   n += factor;               (n starts at (float)0.01)
// and the cell's new temperature is
//     v != 0: (i32)(addTemp + v / n * conductionSelf + t0 * (1 - conductionSelf))
//     v == 0: addTemp + t0 (u32 arithmetic)
// stored into the i16 MaterialInstance::temperature. Every operation is one
// IEEE float operation rounded to nearest (no contraction into fused
// multiply-adds, as on the reference's x86-64 targets); the float -> i32
// conversion is x86's cvttss2si (truncation; NaN or out of range -> INT32_MIN).
//
// Data: SOUP cells keep their temperature in the tp plane (the scalar is their
// amount), all other cells in the scalar. A neighbour outside the world reads
// Tiles_TEST_SOLID, temperature 0, so it adds nothing.
//
// Kernels. The world is cut into 128 x 32 tiles; persistent 256-thread CTAs take
// them in turn. A CTA stages its tile plus a one-cell ring in shared memory as
// per-cell (v term, n term) pairs -- each thread loads one column, 17 rows, with
// 32-bit cell offsets, and keeps its own 16 cells in registers -- then computes
// its 16 results with a 3 x 3 register window sliding down the column and writes
// changed temperatures in place, except on the tile's own edge ring: those cells
// are what the neighbouring tiles read as their halo, so their results go to a
// side array and k_temp_commit stores them after every tile has read its halo.
// HBM traffic: id 2 B + scalar 4 B + tp 2 B read per cell, plus 4 B (scalar) or
// 2 B (tp) per changed cell written. Worlds have fewer than 2^31 cells
// (fse_world_create), so 32-bit offsets address every cell.
#include <cuda_runtime.h>

#include <algorithm>

#include "fse_host.cuh"
#include "fse_internal.cuh"

namespace fse {
namespace {

constexpr int TT_X = 128, TT_Y = 32, TT_THREADS = 256;
constexpr int TT_RX = TT_X + 2, TT_RY = TT_Y + 2;          // staged region with the halo ring
constexpr int TT_RING = 2 * TT_X + 2 * (TT_Y - 2);         // edge cells of a tile
constexpr int TT_ROWS_PER_THREAD = TT_X * TT_Y / TT_THREADS;  // 16 consecutive rows of one column
constexpr uint32_t TC_CHANGED = 0x10000u, TC_SOUP = 0x20000u;

struct TempSmem {
    // per staged cell: x = (float)t * factor (the v term), y = factor (the n term);
    // both 0 where t == 0
    float2 pvn[TT_RY * TT_RX];
    float cs[MAXMAT], co[MAXMAT];
    uint32_t add[MAXMAT];
    uint8_t soup[MAXMAT];
};

__host__ __device__ __forceinline__ int tiles_x(int W) { return (W + TT_X - 1) / TT_X; }
__host__ __device__ __forceinline__ int tiles_y(int H) { return (H + TT_Y - 1) / TT_Y; }

// the step runs after ticks whose index is 2 modulo GameTick (4) when enabled
// (game.cpp:2157); the tick counter already counts the finished tick
__device__ __forceinline__ bool temp_due(const WorldDev &w, int gated) {
    return !gated || (w.temp_on && ((*w.tick - 1u) & 3u) == 2u);
}

// position of ring entry e within its tile
__device__ __forceinline__ void ring_pos(int e, int &lx, int &ly) {
    if (e < TT_X) {
        lx = e;
        ly = 0;
    } else if (e < 2 * TT_X) {
        lx = e - TT_X;
        ly = TT_Y - 1;
    } else if (e < 2 * TT_X + TT_Y - 2) {
        lx = 0;
        ly = e - 2 * TT_X + 1;
    } else {
        lx = TT_X - 1;
        ly = e - (2 * TT_X + TT_Y - 2) + 1;
    }
}
// (v, n) + (p, f) as one paired instruction: add.rn.f32x2 rounds each lane to
// nearest like add.rn.f32, so the two sums are exactly the two scalar chains
__device__ __forceinline__ float2 add2(float2 a, float2 b) {
    float2 d;
    asm("{\n\t.reg .b64 ra, rb, rd;\n\tmov.b64 ra, {%2, %3};\n\tmov.b64 rb, {%4, %5};\n\t"
        "add.rn.f32x2 rd, ra, rb;\n\tmov.b64 {%0, %1}, rd;\n\t}"
        : "=f"(d.x), "=f"(d.y)
        : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
    return d;
}

// x86-64 cvttss2si: truncation toward zero; NaN and values outside the int32
// range give INT32_MIN (the reference's `newTemps[...] = <f32>` on its targets)
__device__ __forceinline__ int32_t f2i_x86(float r) {
    return (r >= -2147483648.0f && r < 2147483648.0f) ? __float2int_rz(r) : (int32_t)0x80000000;
}

// (v term, n term) of one staged cell: world.cpp:1970-1974 for a neighbour with
// temperature t (0 where t == 0, which adds nothing)
__device__ __forceinline__ void temp_terms(int t, float co, float &pv, float &pn) {
    pv = 0.0f;
    pn = 0.0f;
    if (t != 0) {
        const int at = t < 0 ? -t : t;  // |t| <= 32768: abs(t) / 64 is a shift
        pn = __fmul_rn((float)(at >> 6), co);
        pv = __fmul_rn((float)t, pn);
    }
}

// Thread (lx = tid % 128, g = tid / 128) stages column lx + 1 of staged rows
// 17g .. 17g + 16 (the region is 34 rows x 130 columns: the tile and its ring),
// keeping its own cells (staged rows 1 .. 16 for g = 0, 17 .. 32 for g = 1) in
// registers, then computes output rows 16g .. 16g + 15 of column lx.
__global__ void __launch_bounds__(TT_THREADS, 4) k_temp_tiles(const WorldDev *__restrict__ worlds,
                                                             const MatTable *__restrict__ mt, int gated) {
    extern __shared__ __align__(16) unsigned char tsm_raw[];
    TempSmem &S = *reinterpret_cast<TempSmem *>(tsm_raw);
    const WorldDev &w = worlds[blockIdx.y];
    if (!temp_due(w, gated)) return;
    const int W = w.W, H = w.H, tid = threadIdx.x;
    for (int k = tid; k < MAXMAT; k += TT_THREADS) {
        const bool live = k < mt->n;
        S.cs[k] = live ? mt->cond_self[k] : 1.0f;
        S.co[k] = live ? mt->cond_other[k] : 1.0f;
        S.add[k] = live ? mt->add_temp[k] : 0u;
        S.soup[k] = live && mt_type(mt->a[k]) == T_SOUP;
    }
    const int ntx = tiles_x(W), ntiles = ntx * tiles_y(H);
    const uint16_t *__restrict__ gid = w.id;
    const int32_t *__restrict__ gsc = w.sc;
    const int16_t *__restrict__ gtp = w.tp;
    const int lx = tid % TT_X, g = tid / TT_X;
    const bool col_ring = lx == 0 || lx == TT_X - 1;
    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int x0 = (tile % ntx) * TT_X, y0 = (tile / ntx) * TT_Y;
        const int gx = x0 + lx;
        const bool xin = gx < W;
        __syncthreads();  // the previous tile's readers are done; material params are in place
        // own cells: t (low 16 bits) | material << 16 | 1 << 31 where the scalar is wider than int16
        uint32_t own[TT_ROWS_PER_THREAD];
        // ---- stage column lx + 1, rows 17g .. 17g + 16
        {
            const int ry0 = 17 * g;
            int gy = y0 - 1 + ry0;
            uint32_t o = (uint32_t)gy * (uint32_t)W + (uint32_t)gx;  // wraps for gy = -1: used only in the world
#pragma unroll
            for (int i = 0; i < 17; i++, gy++, o += (uint32_t)W) {
                int t = 0, id = 0;
                uint32_t wide = 0;
                if (xin && (unsigned)gy < (unsigned)H) {
                    id = gid[o] & (MAXMAT - 1);  // ids are checked on upload; the mask keeps tables in bounds
                    const int32_t sc = gsc[o];
                    const int16_t tp = gtp ? gtp[o] : (int16_t)0;
                    const bool soup = S.soup[id] != 0;
                    t = soup ? (int)tp : (int)(int16_t)sc;
                    wide = (!soup && sc != (int32_t)(int16_t)sc) ? 0x80000000u : 0u;
                }
                float pv, pn;
                temp_terms(t, S.co[id], pv, pn);
                S.pvn[(ry0 + i) * TT_RX + lx + 1] = make_float2(pv, pn);
                // own rows: staged 1 .. 16 (g = 0: i = 1 .. 16; g = 1: i = 0 .. 15); g is
                // warp-uniform and both branches index `own` with constants
                const uint32_t packed = (uint32_t)(uint16_t)t | ((uint32_t)id << 16) | wide;
                if (g == 0) {
                    if (i >= 1) own[i - 1] = packed;
                } else {
                    if (i < TT_ROWS_PER_THREAD) own[i] = packed;
                }
            }
        }
        // ---- the ring columns 0 and 129 of the region (34 rows each)
        if (tid < 2 * TT_RY) {
            const int side = tid / TT_RY, ry = tid % TT_RY;
            const int hx = side ? x0 + TT_X : x0 - 1, hy = y0 - 1 + ry;
            int t = 0, id = 0;
            if ((unsigned)hx < (unsigned)W && (unsigned)hy < (unsigned)H) {
                const uint32_t o = (uint32_t)hy * (uint32_t)W + (uint32_t)hx;
                id = gid[o] & (MAXMAT - 1);
                t = S.soup[id] ? (int)(gtp ? gtp[o] : (int16_t)0) : (int)(int16_t)gsc[o];
            }
            float pv, pn;
            temp_terms(t, S.co[id], pv, pn);
            S.pvn[ry * TT_RX + (side ? TT_RX - 1 : 0)] = make_float2(pv, pn);
        }
        __syncthreads();
        // ---- outputs: column lx, rows ly0 .. ly0 + 15, window = staged columns lx .. lx + 2
        const int ly0 = g * TT_ROWS_PER_THREAD;
        float2 q0[3], q1[3], q2[3];
#pragma unroll
        for (int c = 0; c < 3; c++) {
            q0[c] = S.pvn[ly0 * TT_RX + lx + c];
            q1[c] = S.pvn[(ly0 + 1) * TT_RX + lx + c];
        }
        uint32_t o = (uint32_t)(y0 + ly0) * (uint32_t)W + (uint32_t)gx;
#pragma unroll
        for (int k = 0; k < TT_ROWS_PER_THREAD; k++, o += (uint32_t)W) {
            const int ly = ly0 + k;
#pragma unroll
            for (int c = 0; c < 3; c++) q2[c] = S.pvn[(ly + 2) * TT_RX + lx + c];
            if (xin && y0 + ly < H) {
                float2 vn = make_float2(0.0f, 0.01f);  // f32 v = 0; f32 n = 0.01;
#pragma unroll
                for (int c = 0; c < 3; c++) {  // FN(xa, -1), FN(xa, 0), FN(xa, 1)
                    vn = add2(vn, q0[c]);
                    vn = add2(vn, q1[c]);
                    vn = add2(vn, q2[c]);
                }
                const float v = vn.x, n = vn.y;
                const uint32_t me = own[k];
                const int t0 = (int)(int16_t)(me & 0xFFFFu);
                const int id = (int)((me >> 16) & (MAXMAT - 1));
                const uint32_t add = S.add[id];
                int32_t r;
                if (v != 0.0f) {  // world.cpp:1988-1990
                    const float cs = S.cs[id];
                    const float a = __fadd_rn(__uint2float_rn(add), __fmul_rn(__fdiv_rn(v, n), cs));
                    r = f2i_x86(__fadd_rn(a, __fmul_rn((float)t0, __fsub_rn(1.0f, cs))));
                } else {  // world.cpp:1992
                    r = (int32_t)(add + (uint32_t)t0);
                }
                const int16_t nt = (int16_t)(uint16_t)(uint32_t)r;
                const bool soup = S.soup[id] != 0;
                // world.cpp:1952-1953, 1996-2001: only the tick zone's cells change
                const int gy = y0 + ly;
                const bool inzone = gx >= w.zx && gy >= w.zy && gx < w.zx + w.zw && gy < w.zy + w.zh;
                const bool changed = inzone && (nt != t0 || (me >> 31));
                // tile-edge cells are read by the neighbouring tiles: deferred
                const bool row_ring = (g == 0 && k == 0) || (g == 1 && k == TT_ROWS_PER_THREAD - 1);
                if (row_ring || col_ring) {
                    const int e = row_ring ? (ly == 0 ? lx : TT_X + lx)
                                           : (lx == 0 ? 2 * TT_X + ly - 1 : 2 * TT_X + (TT_Y - 2) + ly - 1);
                    w.tnew[(size_t)tile * TT_RING + e] =
                        (int32_t)((changed ? TC_CHANGED : 0u) | (soup ? TC_SOUP : 0u) | (uint32_t)(uint16_t)nt);
                } else if (changed) {
                    if (soup) {
                        if (gtp) w.tp[o] = nt;
                    } else {
                        w.sc[o] = nt;
                    }
                }
            }
#pragma unroll
            for (int c = 0; c < 3; c++) {
                q0[c] = q1[c];
                q1[c] = q2[c];
            }
        }
    }
}

// store the deferred results of the tiles' edge rings
__global__ void k_temp_commit(const WorldDev *__restrict__ worlds, int gated) {
    const WorldDev &w = worlds[blockIdx.y];
    if (!temp_due(w, gated)) return;
    const int W = w.W, H = w.H, ntx = tiles_x(W);
    const long long total = (long long)ntx * tiles_y(H) * TT_RING;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
         e += (long long)gridDim.x * blockDim.x) {
        const int tile = (int)(e / TT_RING), r = (int)(e - (long long)tile * TT_RING);
        int lx, ly;
        ring_pos(r, lx, ly);
        const int gx = (tile % ntx) * TT_X + lx, gy = (tile / ntx) * TT_Y + ly;
        if (gx >= W || gy >= H) continue;
        const uint32_t v = (uint32_t)w.tnew[e];
        if (!(v & TC_CHANGED)) continue;
        const int16_t nt = (int16_t)(uint16_t)(v & 0xFFFFu);
        const size_t g = (size_t)gy * W + gx;
        if (v & TC_SOUP) {
            if (w.tp) w.tp[g] = nt;
        } else {
            w.sc[g] = nt;
        }
    }
}

// per-cell temperature view <-> int16 buffer
__global__ void k_temp_read(const WorldDev *__restrict__ wd, const MatTable *__restrict__ mt, int16_t *out) {
    const WorldDev &w = *wd;
    const size_t n = (size_t)w.W * w.H;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        out[i] = mt_type(mt->a[w.id[i]]) == T_SOUP ? (w.tp ? w.tp[i] : (int16_t)0) : (int16_t)w.sc[i];
}
__global__ void k_temp_write(const WorldDev *__restrict__ wd, const MatTable *__restrict__ mt, const int16_t *in) {
    const WorldDev &w = *wd;
    const size_t n = (size_t)w.W * w.H;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        if (mt_type(mt->a[w.id[i]]) == T_SOUP) {
            if (w.tp) w.tp[i] = in[i];
        } else {
            w.sc[i] = in[i];
        }
    }
}

}  // namespace

size_t temperature_scratch_cells(int W, int H) { return (size_t)tiles_x(W) * tiles_y(H) * TT_RING; }
int temperature_tiles(int W, int H) { return tiles_x(W) * tiles_y(H); }

cudaError_t launch_temperature(const WorldDev *d_worlds, int n_worlds, int max_tiles, const MatTable *mt, bool gated,
                               cudaStream_t s) {
    if (n_worlds <= 0 || max_tiles <= 0) return cudaSuccess;
    static bool attr = false;
    if (!attr) {
        cudaError_t e =
            cudaFuncSetAttribute(k_temp_tiles, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(TempSmem));
        if (e != cudaSuccess) return e;
        attr = true;
    }
    // 4 CTAs of 256 threads fit an SM (about 56 KB of shared memory each)
    const int gx = std::max(1, std::min(max_tiles, sm_count() * 4));
    k_temp_tiles<<<dim3(gx, n_worlds), TT_THREADS, sizeof(TempSmem), s>>>(d_worlds, mt, gated ? 1 : 0);
    const long long ring = (long long)max_tiles * TT_RING;
    const int cx = (int)std::max(1LL, std::min<long long>((ring + 255) / 256, sm_count() * 8));
    k_temp_commit<<<dim3(cx, n_worlds), 256, 0, s>>>(d_worlds, gated ? 1 : 0);
    return cudaGetLastError();
}

}  // namespace fse

using namespace fse;

namespace {
int ensure_temperature_scratch(fse_world *w) {
    if (w->h.tnew) return FSE_OK;
    int32_t *p = nullptr;
    const size_t n = temperature_scratch_cells(w->W, w->H);
    if (cudaMalloc(&p, n * sizeof(int32_t)) != cudaSuccess) return FSE_E_NOMEM;
    w->h.tnew = p;
    w->bytes += n * sizeof(int32_t);
    if (cudaMemcpyAsync(w->d, &w->h, sizeof(WorldDev), cudaMemcpyHostToDevice, w->stream) != cudaSuccess)
        return FSE_E_CUDA;
    return FSE_OK;
}
int ensure_temperature_io(fse_world *w) {
    if (w->temp_io) return FSE_OK;
    if (cudaMalloc(&w->temp_io, (size_t)w->W * w->H * sizeof(int16_t)) != cudaSuccess) {
        w->temp_io = nullptr;
        return FSE_E_NOMEM;
    }
    return FSE_OK;
}
int io_blocks(const fse_world *w) {
    return (int)std::max<long long>(1, std::min<long long>(((long long)w->W * w->H + 255) / 256, sm_count() * 16));
}
}  // namespace

extern "C" {

int fse_world_tick_temperature(fse_world *w) {
    if (!w) return FSE_E_INVAL;
    if (!w->h.tp) return FSE_E_STATE;  // the world keeps no liquid temperatures
    int rc = ensure_materials_pushed();
    if (rc) return rc;
    rc = ensure_temperature_scratch(w);
    if (rc) return rc;
    if (launch_temperature(w->d, 1, temperature_tiles(w->W, w->H), g_dev_mt, false, w->stream) != cudaSuccess)
        return FSE_E_CUDA;
    count_launches(2);
    return FSE_OK;
}

int fse_world_temperature_read(fse_world *w, int16_t *out) {
    if (!w || !out) return FSE_E_INVAL;
    if (!w->h.tp) return FSE_E_STATE;
    int rc = ensure_materials_pushed();
    if (rc) return rc;
    rc = ensure_temperature_io(w);
    if (rc) return rc;
    k_temp_read<<<io_blocks(w), 256, 0, w->stream>>>(w->d, g_dev_mt, w->temp_io);
    FSE_CUDA_TRY(cudaGetLastError());
    FSE_CUDA_TRY(cudaMemcpyAsync(out, w->temp_io, (size_t)w->W * w->H * 2, cudaMemcpyDeviceToHost, w->stream));
    FSE_CUDA_TRY(cudaStreamSynchronize(w->stream));
    return FSE_OK;
}

int fse_world_temperature_write(fse_world *w, const int16_t *in) {
    if (!w || !in) return FSE_E_INVAL;
    if (!w->h.tp) return FSE_E_STATE;
    int rc = ensure_materials_pushed();
    if (rc) return rc;
    rc = ensure_temperature_io(w);
    if (rc) return rc;
    FSE_CUDA_TRY(cudaMemcpyAsync(w->temp_io, in, (size_t)w->W * w->H * 2, cudaMemcpyHostToDevice, w->stream));
    k_temp_write<<<io_blocks(w), 256, 0, w->stream>>>(w->d, g_dev_mt, w->temp_io);
    FSE_CUDA_TRY(cudaGetLastError());
    FSE_CUDA_TRY(cudaStreamSynchronize(w->stream));
    return FSE_OK;
}

}  // extern "C"
