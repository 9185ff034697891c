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
// Kernels. The world is cut into 128 x 32 tiles, one 256-thread CTA each. A CTA
// stages its tile plus a one-cell ring in shared memory as per-cell (v term,
// n term) pairs, computes its 4096 results with a 3 x 3 register window that
// slides down each column, and writes changed temperatures in place, except on
// the tile's own edge ring: those cells are what the neighbouring tiles read as
// their halo, so their results go to a side array and k_temp_commit stores them
// after every tile has read its halo. HBM traffic: id 2 B + scalar 4 B + tp 2 B
// read per cell, plus 4 B (scalar) or 2 B (tp) per changed cell written.
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
    float pv[TT_RY * TT_RX];  // (float)t * factor of each staged cell (0 where t == 0)
    float pn[TT_RY * TT_RX];  // factor (0 where t == 0)
    int16_t t[TT_Y * TT_X];   // the tile's own temperatures
    uint16_t id[TT_Y * TT_X];  // material | 0x8000 where a scalar holds a value outside int16 (always stored)
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
__device__ __forceinline__ int ring_index(int lx, int ly) {
    if (ly == 0) return lx;
    if (ly == TT_Y - 1) return TT_X + lx;
    if (lx == 0) return 2 * TT_X + ly - 1;
    if (lx == TT_X - 1) return 2 * TT_X + (TT_Y - 2) + ly - 1;
    return -1;
}

// x86-64 cvttss2si: truncation toward zero; NaN and values outside the int32
// range give INT32_MIN (the reference's `newTemps[...] = <f32>` on its targets)
__device__ __forceinline__ int32_t f2i_x86(float r) {
    return (r >= -2147483648.0f && r < 2147483648.0f) ? __float2int_rz(r) : (int32_t)0x80000000;
}

__global__ void __launch_bounds__(TT_THREADS) k_temp_tiles(const WorldDev *__restrict__ worlds,
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
    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int x0 = (tile % ntx) * TT_X, y0 = (tile / ntx) * TT_Y;
        __syncthreads();  // the previous tile's readers are done; material params are in place
        // stage the region [x0 - 1, x0 + TT_X] x [y0 - 1, y0 + TT_Y]
#pragma unroll 6
        for (int r = tid; r < TT_RY * TT_RX; r += TT_THREADS) {
            const int ry = r / TT_RX, rx = r - ry * TT_RX;
            const int gx = x0 - 1 + rx, gy = y0 - 1 + ry;
            int t = 0, id = 0, wide = 0;
            if ((unsigned)gx < (unsigned)W && (unsigned)gy < (unsigned)H) {
                const size_t g = (size_t)gy * W + gx;
                id = gid[g] & (MAXMAT - 1);  // ids are checked on upload; the mask keeps tables in bounds
                const int32_t sc = gsc[g];
                const int16_t tp = gtp ? gtp[g] : (int16_t)0;
                const bool soup = S.soup[id] != 0;
                t = soup ? (int)tp : (int)(int16_t)sc;
                wide = !soup && sc != (int32_t)(int16_t)sc;
            }
            float pv = 0.0f, pn = 0.0f;
            if (t != 0) {  // world.cpp:1970-1974
                const int at = t < 0 ? -t : t;
                pn = __fmul_rn((float)(at / 64), S.co[id]);
                pv = __fmul_rn((float)t, pn);
            }
            S.pv[r] = pv;
            S.pn[r] = pn;
            if (ry >= 1 && ry <= TT_Y && rx >= 1 && rx <= TT_X) {
                const int o = (ry - 1) * TT_X + (rx - 1);
                S.t[o] = (int16_t)t;
                S.id[o] = (uint16_t)(id | (wide << 15));
            }
        }
        __syncthreads();
        // each thread: column lx, TT_ROWS_PER_THREAD consecutive rows from ly0
        const int lx = tid % TT_X, ly0 = (tid / TT_X) * TT_ROWS_PER_THREAD;
        const int gx = x0 + lx;
        // window columns lx .. lx + 2 of the staged region (xa = -1, 0, 1), rows k .. k + 2
        float v0[3], v1[3], v2[3], n0[3], n1[3], n2[3];
#pragma unroll
        for (int c = 0; c < 3; c++) {
            v0[c] = S.pv[ly0 * TT_RX + lx + c];
            n0[c] = S.pn[ly0 * TT_RX + lx + c];
            v1[c] = S.pv[(ly0 + 1) * TT_RX + lx + c];
            n1[c] = S.pn[(ly0 + 1) * TT_RX + lx + c];
        }
#pragma unroll 4
        for (int k = 0; k < TT_ROWS_PER_THREAD; k++) {
            const int ly = ly0 + k;
#pragma unroll
            for (int c = 0; c < 3; c++) {
                v2[c] = S.pv[(ly + 2) * TT_RX + lx + c];
                n2[c] = S.pn[(ly + 2) * TT_RX + lx + c];
            }
            const int gy = y0 + ly;
            if (gx < W && gy < H) {
                float v = 0.0f, n = 0.01f;  // f32 v = 0; f32 n = 0.01;
#pragma unroll
                for (int c = 0; c < 3; c++) {  // FN(xa, -1), FN(xa, 0), FN(xa, 1)
                    v = __fadd_rn(v, v0[c]);
                    n = __fadd_rn(n, n0[c]);
                    v = __fadd_rn(v, v1[c]);
                    n = __fadd_rn(n, n1[c]);
                    v = __fadd_rn(v, v2[c]);
                    n = __fadd_rn(n, n2[c]);
                }
                const int o = ly * TT_X + lx;
                const int t0 = S.t[o];
                const int idw = S.id[o], id = idw & 0x7FFF;
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
                const bool changed = nt != t0 || (idw >> 15);
                const int e = ring_index(lx, ly);
                const size_t g = (size_t)gy * W + gx;
                if (e >= 0) {
                    w.tnew[(size_t)tile * TT_RING + e] =
                        (int32_t)((changed ? TC_CHANGED : 0u) | (soup ? TC_SOUP : 0u) | (uint32_t)(uint16_t)nt);
                } else if (changed) {
                    if (soup) {
                        if (w.tp) w.tp[g] = nt;
                    } else {
                        w.sc[g] = nt;
                    }
                }
            }
#pragma unroll
            for (int c = 0; c < 3; c++) {
                v0[c] = v1[c];
                n0[c] = n1[c];
                v1[c] = v2[c];
                n1[c] = n2[c];
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
