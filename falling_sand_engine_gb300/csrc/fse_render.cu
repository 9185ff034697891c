// fse_render.cu -- headless versions of the game's per-tick texture updates: the
// dirty-cell pass (source/engine/game.cpp:1994-2067) and the free-particle layer
// (world::renderCells, source/engine/world.cpp:2006-2028, after the clear of
// game.cpp:1881). Textures are device planes of 4 bytes per cell (r, g, b, a).
//
// The dirty pass reads one byte per cell (the dirty mark) and touches the rest only
// for dirty cells, so it is bound by HBM. The flow channel repeats the reference's
// mixed float/double arithmetic operation by operation with explicitly rounded
// intrinsics, so it agrees bit for bit with a strict IEEE CPU evaluation.
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
// clamped to [0, 1], times 255, truncated to a byte
__device__ __forceinline__ uint32_t flow_byte(float f, int iterations) {
    const double k = __dadd_rn(__ddiv_rn(3.0, (double)iterations), 0.5);
    const double a = __dadd_rn(__ddiv_rn(__dmul_rn((double)f, k), 4.0), 0.5);
    double c = a < 0.0 ? 0.0 : a;
    c = c > 1.0 ? 1.0 : c;
    return (uint32_t)__dmul_rn(c, 255.0);
}

// one dirty cell of game.cpp:1997-2063
__device__ __forceinline__ void paint(const WorldDev &w, const RenderTex &rt, size_t i, const uint8_t *s_type,
                                      const uint32_t *s_alpha, const uint32_t *s_emit, const int *s_iter, int id_fire,
                                      unsigned *s_mov) {
    w.dirty[i] = 0;
    const int id = w.id[i];
    atomicAdd(&s_mov[id], 1u);  // movingTiles
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
        const float fx = __fmul_rn(__int2float_rn(fl[0]), 1.0f / 65536.0f);
        const float fy = __fmul_rn(__int2float_rn(fl[1]), 1.0f / 65536.0f);
        // f32 + (f32 - f32) * 0.25: the product and the sum in double, stored as f32
        const float nfx = __double2float_rn(__dadd_rn((double)pf[0], __dmul_rn((double)__fsub_rn(fx, pf[0]), 0.25)));
        float nfy = __double2float_rn(__dadd_rn((double)pf[1], __dmul_rn((double)__fsub_rn(fy, pf[1]), 0.25)));
        if (nfy < 0.0f) nfy = __double2float_rn(__dmul_rn((double)nfy, 0.5));
        rt.tex[3][i] = rgba(flow_byte(nfx, s_iter[id]), flow_byte(nfy, s_iter[id]), 0u, 0xffu);
        pf[0] = nfx;
        pf[1] = nfy;
    }
    fl[0] = 0;
    fl[1] = 0;
}

// the dirty pass over one world; four cells per thread, their marks read as one word
__global__ void k_render_dirty(const WorldDev *__restrict__ wd, const MatTable *__restrict__ mt, RenderTex rt) {
    __shared__ uint8_t s_type[MAXMAT];
    __shared__ uint32_t s_alpha[MAXMAT], s_emit[MAXMAT];
    __shared__ int s_iter[MAXMAT];
    __shared__ unsigned s_mov[MAXMAT];
    for (int k = threadIdx.x; k < MAXMAT; k += blockDim.x) {
        const bool ok = k < mt->n;
        s_type[k] = (uint8_t)(ok ? mt_type(mt->a[k]) : 0);
        s_alpha[k] = ok ? mt->alpha[k] : 0u;
        s_emit[k] = ok ? mt->emit_col[k] : 0u;
        s_iter[k] = ok ? mt->iterations[k] : 1;
        s_mov[k] = 0u;
    }
    __syncthreads();
    const WorldDev &w = *wd;
    const int id_fire = mt->id_fire;
    const size_t n = (size_t)w.W * w.H, n4 = n / 4;
    const uint32_t *d4 = reinterpret_cast<const uint32_t *>(w.dirty);  // cudaMalloc alignment
    for (size_t g = blockIdx.x * (size_t)blockDim.x + threadIdx.x; g < n4; g += (size_t)gridDim.x * blockDim.x) {
        const uint32_t m = d4[g];
        if (m == 0u) continue;
#pragma unroll
        for (int k = 0; k < 4; k++)
            if ((m >> (8 * k)) & 0xffu) paint(w, rt, 4 * g + k, s_type, s_alpha, s_emit, s_iter, id_fire, s_mov);
    }
    for (size_t i = 4 * n4 + blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        if (w.dirty[i]) paint(w, rt, i, s_type, s_alpha, s_emit, s_iter, id_fire, s_mov);
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
    const int blocks = (int)std::max<size_t>(1, std::min<size_t>((n / 4 + 255) / 256, (size_t)sm_count() * 8));
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
