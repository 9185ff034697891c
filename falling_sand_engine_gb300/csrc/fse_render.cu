// fse_render.cu -- headless versions of the game's per-tick texture updates: the
// dirty-cell pass (source/engine/game.cpp:1994-2067) and the free-particle layer
// (world::renderCells, source/engine/world.cpp:2006-2028, after the clear of
// game.cpp:1881). Textures are device planes of 4 bytes per cell (r, g, b, a).
//
// The dirty pass reads one byte per cell (the dirty mark) and touches the rest only
// for dirty cells. The flow channel gives the results of the reference's mixed
// float/double arithmetic bit for bit: the final scaling stays in double, and the
// smoothing, whose double evaluation provably equals the float one for normal
// operands, runs in float except for subnormal operands (FP64 is slow here and
// was the pass's bound when every step ran in double).
#include <algorithm>

#include "fse_host.cuh"

namespace fse {

struct RenderTex {
    uint32_t *tex[5];
    float *pflow;
    int32_t *owner;
    long long *moving;
};

__device__ __forceinline__ uint32_t rgba(uint32_t r, uint32_t g, uint32_t b, uint32_t a) {
    return (r & 0xff) | ((g & 0xff) << 8) | ((b & 0xff) << 16) | ((a & 0xff) << 24);
}

// game.cpp:2048-2053: a = flow * (3.0 / iterations + 0.5) / 4.0 + 0.5 in double,
// clamped to [0, 1], times 255, truncated to a byte. k = 3.0 / iterations + 0.5
// comes from the material table; / 4.0 is the exact * 0.25. (A NaN, from a
// material with zero iterations, gives 0.)
__device__ __forceinline__ uint32_t flow_byte(float f, double k) {
    const double a = __dadd_rn(__dmul_rn(__dmul_rn((double)f, k), 0.25), 0.5);
    if (!(a > 0.0)) return 0u;
    return a >= 1.0 ? 255u : (uint32_t)__dmul_rn(a, 255.0);
}

// the same byte from the material's thresholds (the largest j with thr[j] <= f):
// a float estimate, then exact steps along the table; float compares only
__device__ __forceinline__ uint32_t flow_byte_thr(float f, const float *__restrict__ thr, float kf) {
    if (!(f == f)) return 0u;  // NaN: 0, as in the double evaluation
    const float est = __fmul_rn(__fadd_rn(__fmul_rn(__fmul_rn(f, kf), 0.25f), 0.5f), 255.0f);
    int j = est >= 255.0f ? 255 : (est > 0.0f ? (int)est : 0);
    while (j < 255 && f >= thr[j + 1]) j++;
    while (j > 0 && f < thr[j]) j--;
    return (uint32_t)j;
}

// prev + (cur - prev) * 0.25 with the product and the sum in double, rounded to
// float (game.cpp:2041-2042). For normal operands this equals the float
// evaluation: * 0.25 is exact, and the double sum of two floats is exact unless
// their exponents differ by more than 28, when the smaller one is below half a
// float ulp of the larger either way. Subnormal operands (flows decaying towards
// zero) take the double path.
__device__ __forceinline__ float smooth(float prev, float cur) {
    const float d = __fsub_rn(cur, prev);
    const float m = 0x1p-120f;
    if ((fabsf(prev) >= m || prev == 0.0f) && (fabsf(d) >= m || d == 0.0f))
        return __fadd_rn(prev, __fmul_rn(d, 0.25f));
    return __double2float_rn(__dadd_rn((double)prev, __dmul_rn((double)d, 0.25)));
}

// v * 0.5 in double, rounded to float (game.cpp:2043): exact halving for normal v
__device__ __forceinline__ float half_of(float v) {
    if (fabsf(v) >= 0x1p-120f) return __fmul_rn(v, 0.5f);
    return __double2float_rn(__dmul_rn((double)v, 0.5));
}

// one dirty cell of game.cpp:1997-2063
__device__ __forceinline__ void paint(const WorldDev &w, const MatTable *__restrict__ mt, const RenderTex &rt,
                                      size_t i, const uint8_t *s_type, const uint32_t *s_alpha, const uint32_t *s_emit,
                                      const double *s_k, int id_fire, unsigned *s_mov) {
    w.dirty[i] = 0;
    const int id = w.id[i];
    {
        // movingTiles: lanes with the same material add once
        const unsigned grp = __match_any_sync(__activemask(), id);
        if ((threadIdx.x & 31) == __ffs(grp) - 1) atomicAdd(&s_mov[id], (unsigned)__popc(grp));
    }
    int32_t *fl = w.flow + 2 * i;
    const int type = s_type[id];
    if (type == T_AIR) {
        rt.tex[0][i] = 0u;  // ME_ALPHA_TRANSPARENT
        rt.tex[2][i] = 0u;
        rt.tex[1][i] = 0u;
        fl[0] = 0;
        fl[1] = 0;
        return;
    }
    const uint32_t col = w.col[i], e = s_emit[id];
    const uint32_t px = rgba(col >> 16, col >> 8, col, s_alpha[id]);
    rt.tex[0][i] = px;
    rt.tex[1][i] = rgba(e >> 16, e >> 8, e, e >> 24);
    if (id == id_fire) rt.tex[2][i] = px;  // other cells keep their fire texel
    if (type == T_SOUP) {
        float *pf = rt.pflow + 2 * i;
        // the tick's flow sums: f32 in worlds with f32 amounts, else Q16.16
        const float fx = w.f32 ? __int_as_float(fl[0]) : __fmul_rn(__int2float_rn(fl[0]), 1.0f / 65536.0f);
        const float fy = w.f32 ? __int_as_float(fl[1]) : __fmul_rn(__int2float_rn(fl[1]), 1.0f / 65536.0f);
        const float nfx = smooth(pf[0], fx);
        float nfy = smooth(pf[1], fy);
        if (nfy < 0.0f) nfy = half_of(nfy);
        uint32_t bx, by;
        if (mt->flow_thr_ok[id]) {
            const float kf = (float)s_k[id];
            bx = flow_byte_thr(nfx, mt->flow_thr[id], kf);
            by = flow_byte_thr(nfy, mt->flow_thr[id], kf);
        } else {
            bx = flow_byte(nfx, s_k[id]);
            by = flow_byte(nfy, s_k[id]);
        }
        rt.tex[3][i] = rgba(bx, by, 0u, 0xffu);
        pf[0] = nfx;
        pf[1] = nfy;
    }
    fl[0] = 0;
    fl[1] = 0;
}

// the dirty pass over one world, one cell per thread (consecutive cells on
// consecutive lanes, so every plane is read and written coalesced)
__global__ void k_render_dirty(const WorldDev *__restrict__ wd, const MatTable *__restrict__ mt, RenderTex rt) {
    __shared__ uint8_t s_type[MAXMAT];
    __shared__ uint32_t s_alpha[MAXMAT], s_emit[MAXMAT];
    __shared__ double s_k[MAXMAT];
    __shared__ unsigned s_mov[MAXMAT];
    for (int k = threadIdx.x; k < MAXMAT; k += blockDim.x) {
        const bool ok = k < mt->n;
        s_type[k] = (uint8_t)(ok ? mt_type(mt->a[k]) : 0);
        s_alpha[k] = ok ? mt->alpha[k] : 0u;
        s_emit[k] = ok ? mt->emit_col[k] : 0u;
        s_k[k] = ok ? mt->flow_k[k] : 0.0;
        s_mov[k] = 0u;
    }
    __syncthreads();
    const WorldDev &w = *wd;
    const int id_fire = mt->id_fire;
    const size_t n = (size_t)w.W * w.H;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        if (w.dirty[i]) paint(w, mt, rt, i, s_type, s_alpha, s_emit, s_k, id_fire, s_mov);
    __syncthreads();
    for (int k = threadIdx.x; k < MAXMAT; k += blockDim.x)
        if (s_mov[k]) atomicAdd((unsigned long long *)&rt.moving[k], (unsigned long long)s_mov[k]);
}

__device__ __forceinline__ bool in_world(float x, float y, int W, int H) {
    // `x < 0 || x >= width || y < 0 || y >= height` skips (world.cpp:2009); NaN skips too
    return x >= 0.0f && x < (float)W && y >= 0.0f && y < (float)H;
}

// particle layer, step 1: the last particle (in list order) on each texel
__global__ void k_cells_claim(const WorldDev *__restrict__ wd, int32_t *owner) {
    const WorldDev &w = *wd;
    const int n = *w.part_count;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float x = w.p.x[i], y = w.p.y[i];
        if (!in_world(x, y, w.W, w.H)) continue;
        atomicMax(&owner[(size_t)(int)y * w.W + (int)x], i);
    }
}

// step 2: that particle paints its texel (world.cpp:2011-2026)
__global__ void k_cells_draw(const WorldDev *__restrict__ wd, const MatTable *__restrict__ mt, const int32_t *owner,
                             uint32_t *tex) {
    const WorldDev &w = *wd;
    const int n = *w.part_count;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float x = w.p.x[i], y = w.p.y[i];
        if (!in_world(x, y, w.W, w.H)) continue;
        const size_t t = (size_t)(int)y * w.W + (int)x;
        if (owner[t] != i) continue;
        float amod = 1.0f;
        const int32_t life = w.p.life[i], fade = w.p.fade[i];
        if ((w.p.bits[i] & 2) && life < fade) amod = __fdiv_rn((float)life, (float)fade);
        const float a = __fmul_rn((float)mt->alpha[w.p.id[i]], amod);
        const uint32_t ab = a > 0.0f ? (uint32_t)a : 0u;  // a negative lifetime draws transparent
        const uint32_t col = w.p.col[i];
        tex[t] = rgba(col >> 16, col >> 8, col, ab);
    }
}

}  // namespace fse

using namespace fse;

static RenderTex render_tex(fse_world *w) {
    RenderTex rt;
    for (int k = 0; k < 5; k++) rt.tex[k] = w->tex[k];
    rt.pflow = w->pflow;
    rt.owner = w->owner;
    rt.moving = w->moving;
    return rt;
}

extern "C" {

int fse_world_render_dirty(fse_world *w, int64_t *moving) {
    if (!w) return FSE_E_INVAL;
    if (!w->h.dirty) return FSE_E_STATE;
    int rc = ensure_materials_pushed();
    if (rc) return rc;
    const size_t n = (size_t)w->W * w->H;
    FSE_CUDA_TRY(cudaMemsetAsync(w->moving, 0, MAXMAT * sizeof(long long), w->stream));
    const int blocks = (int)std::max<size_t>(1, std::min<size_t>((n + 255) / 256, (size_t)sm_count() * 16));
    k_render_dirty<<<blocks, 256, 0, w->stream>>>(w->d, g_dev_mt, render_tex(w));
    FSE_CUDA_TRY(cudaGetLastError());
    count_launches(1);
    if (moving) {
        const int nm = fse_material_count();
        FSE_CUDA_TRY(cudaMemcpyAsync(moving, w->moving, (size_t)nm * sizeof(int64_t), cudaMemcpyDeviceToHost,
                                     w->stream));
        FSE_CUDA_TRY(cudaStreamSynchronize(w->stream));
    }
    return FSE_OK;
}

int fse_world_render_cells(fse_world *w) {
    if (!w) return FSE_E_INVAL;
    if (!w->h.dirty) return FSE_E_STATE;
    int rc = ensure_materials_pushed();
    if (rc) return rc;
    const size_t n = (size_t)w->W * w->H;
    FSE_CUDA_TRY(cudaMemsetAsync(w->tex[FSE_TEX_CELLS], 0, n * 4, w->stream));
    FSE_CUDA_TRY(cudaMemsetAsync(w->owner, 0xff, n * 4, w->stream));  // -1: no particle
    const int blocks = std::max(1, std::min(sm_count() * 4, ceil_div(w->part_cap, 256)));
    k_cells_claim<<<blocks, 256, 0, w->stream>>>(w->d, w->owner);
    k_cells_draw<<<blocks, 256, 0, w->stream>>>(w->d, g_dev_mt, w->owner, w->tex[FSE_TEX_CELLS]);
    FSE_CUDA_TRY(cudaGetLastError());
    count_launches(2);
    return FSE_OK;
}

int fse_world_render_read(fse_world *w, int which, uint8_t *out) {
    if (!w || !out || which < 0 || which > 4) return FSE_E_INVAL;
    if (!w->h.dirty) return FSE_E_STATE;
    const size_t n = (size_t)w->W * w->H;
    FSE_CUDA_TRY(cudaMemcpyAsync(out, w->tex[which], n * 4, cudaMemcpyDeviceToHost, w->stream));
    FSE_CUDA_TRY(cudaStreamSynchronize(w->stream));
    return FSE_OK;
}

void *fse_world_render_texture(fse_world *w, int which) {
    if (!w || which < 0 || which > 4 || !w->h.dirty) return nullptr;
    return w->tex[which];
}

}  // extern "C"
