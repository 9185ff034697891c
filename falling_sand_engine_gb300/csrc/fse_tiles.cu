// fse_tiles.cu -- the grid to and from an array of tile structs, such as the
// reference's real_tiles of MaterialInstance (source/engine/game_datastruct.hpp:
// 205-222): one thread per cell converts between the caller's struct fields
// (at the byte offsets of an fse_tile_layout) and the world's planes, on the device.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>

#include "fse_host.cuh"
#include "fse_internal.cuh"

namespace fse {
namespace {

struct Layout {
    int stride, id, mat, colour, temperature, moved, fluid, fluid_diff, settle;
};

__device__ __forceinline__ int32_t to_q16(float f) {
    // the nearest multiple of 1/65536; out of range saturates, NaN gives 0
    const float q = f * 65536.0f;
    if (!(q == q)) return 0;
    return __float2int_rn(q);
}

__global__ void k_tiles_in(const WorldDev *__restrict__ wd, const MatTable *__restrict__ mt, const uint8_t *tiles,
                           Layout L, int *bad) {
    const WorldDev &w = *wd;
    const size_t n = (size_t)w.W * w.H;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const uint8_t *t = tiles + i * (size_t)L.stride;
        uint32_t id = *reinterpret_cast<const uint32_t *>(t + L.id);
        if (id >= (uint32_t)mt->n) {
            atomicOr(bad, 1);
            id = (uint32_t)mt->id_air;
        }
        const uint32_t col = L.colour >= 0 ? *reinterpret_cast<const uint32_t *>(t + L.colour) : 0u;
        const int16_t temp = L.temperature >= 0 ? *reinterpret_cast<const int16_t *>(t + L.temperature) : (int16_t)0;
        const bool moved = L.moved >= 0 && t[L.moved] != 0;
        const int settle = L.settle >= 0 ? min((int)t[L.settle], (int)SETTLE_MASK) : 0;
        w.id[i] = (uint16_t)id;
        w.col[i] = col;
        w.fl[i] = (uint8_t)((moved ? MOVED : 0) | settle);
        if (mt_type(mt->a[id]) == T_SOUP) {
            if (w.f32) {  // f32 amounts: the caller's floats as they are
                w.sc[i] = L.fluid >= 0 ? *reinterpret_cast<const int32_t *>(t + L.fluid) : F_DEFAULT_BITS;
                w.df[i] = L.fluid_diff >= 0 ? *reinterpret_cast<const int32_t *>(t + L.fluid_diff) : 0;
            } else {
                w.sc[i] = L.fluid >= 0 ? to_q16(*reinterpret_cast<const float *>(t + L.fluid)) : Q_DEFAULT;
                w.df[i] = L.fluid_diff >= 0 ? to_q16(*reinterpret_cast<const float *>(t + L.fluid_diff)) : 0;
            }
            if (w.tp) w.tp[i] = temp;
        } else {
            w.sc[i] = temp;
            w.df[i] = 0;
        }
        if (w.dirty) w.dirty[i] = 1;
    }
}

__global__ void k_tiles_out(const WorldDev *__restrict__ wd, const MatTable *__restrict__ mt, uint8_t *tiles,
                            Layout L, const uint64_t *__restrict__ mat_table, int n_table) {
    const WorldDev &w = *wd;
    const size_t n = (size_t)w.W * w.H;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        uint8_t *t = tiles + i * (size_t)L.stride;
        const uint32_t id = w.id[i];
        const bool soup = mt_type(mt->a[id]) == T_SOUP;
        *reinterpret_cast<uint32_t *>(t + L.id) = id;
        if (L.mat >= 0 && mat_table && (int)id < n_table) *reinterpret_cast<uint64_t *>(t + L.mat) = mat_table[id];
        if (L.colour >= 0) *reinterpret_cast<uint32_t *>(t + L.colour) = w.col[i];
        if (L.temperature >= 0)
            *reinterpret_cast<int16_t *>(t + L.temperature) =
                soup ? (w.tp ? w.tp[i] : (int16_t)0) : (int16_t)w.sc[i];
        const uint8_t f = w.fl[i];
        if (L.moved >= 0) t[L.moved] = (f & MOVED) ? 1 : 0;
        if (L.settle >= 0) t[L.settle] = (uint8_t)(f & SETTLE_MASK);
        if (soup && w.f32) {
            if (L.fluid >= 0) *reinterpret_cast<int32_t *>(t + L.fluid) = w.sc[i];
            if (L.fluid_diff >= 0) *reinterpret_cast<int32_t *>(t + L.fluid_diff) = w.df[i];
        } else if (soup) {
            if (L.fluid >= 0) *reinterpret_cast<float *>(t + L.fluid) = (float)w.sc[i] * (1.0f / 65536.0f);
            if (L.fluid_diff >= 0) *reinterpret_cast<float *>(t + L.fluid_diff) = (float)w.df[i] * (1.0f / 65536.0f);
        }
    }
}

// offsets inside the stride and naturally aligned; the stride keeps them aligned
bool layout_ok(const fse_tile_layout *l, Layout &L) {
    if (!l || l->stride <= 0 || l->id < 0) return false;
    L = Layout{l->stride, l->id, l->mat, l->colour, l->temperature, l->moved, l->fluid_amount, l->fluid_amount_diff,
               l->settle_count};
    auto fits = [&](int off, int size) { return off < 0 || (off + size <= l->stride && off % size == 0); };
    const int align = l->mat >= 0 ? 8 : 4;
    return l->stride % align == 0 && fits(l->id, 4) && fits(l->mat, 8) && fits(l->colour, 4) &&
           fits(l->temperature, 2) && fits(l->moved, 1) && fits(l->fluid_amount, 4) &&
           fits(l->fluid_amount_diff, 4) && fits(l->settle_count, 1);
}

int ensure_tile_stage(fse_world *w, size_t bytes) {
    if (w->tile_stage && w->tile_stage_bytes >= bytes) return FSE_OK;
    if (w->tile_stage) cudaFree(w->tile_stage);
    w->tile_stage = nullptr;
    w->tile_stage_bytes = 0;
    if (cudaMalloc(&w->tile_stage, bytes) != cudaSuccess) {
        w->tile_stage = nullptr;
        return FSE_E_NOMEM;
    }
    w->tile_stage_bytes = bytes;
    return FSE_OK;
}

int grid_of(const fse_world *w) {
    return (int)std::max<long long>(1, std::min<long long>(((long long)w->W * w->H + 255) / 256, sm_count() * 16));
}

}  // namespace
}  // namespace fse

using namespace fse;

extern "C" {

int fse_world_upload_tiles(fse_world *w, const void *tiles, const fse_tile_layout *layout) {
    Layout L;
    if (!w || !tiles || !layout_ok(layout, L)) return FSE_E_INVAL;
    int rc = ensure_materials_pushed();
    if (rc) return rc;
    const size_t bytes = (size_t)w->W * w->H * (size_t)L.stride;
    rc = ensure_tile_stage(w, bytes);
    if (rc) return rc;
    FSE_CUDA_TRY(cudaMemcpyAsync(w->tile_stage, tiles, bytes, cudaMemcpyHostToDevice, w->stream));
    FSE_CUDA_TRY(cudaMemsetAsync(w->ctr + 7, 0, 4, w->stream));
    k_tiles_in<<<grid_of(w), 256, 0, w->stream>>>(w->d, g_dev_mt, w->tile_stage, L, w->ctr + 7);
    FSE_CUDA_TRY(cudaGetLastError());
    count_launches(1);
    int bad = 0;
    FSE_CUDA_TRY(cudaMemcpyAsync(&bad, w->ctr + 7, 4, cudaMemcpyDeviceToHost, w->stream));
    FSE_CUDA_TRY(cudaStreamSynchronize(w->stream));
    return bad ? FSE_E_INVAL : FSE_OK;
}

int fse_world_download_tiles(fse_world *w, void *tiles, const fse_tile_layout *layout, const uint64_t *mat_table,
                             int n_mat) {
    Layout L;
    if (!w || !tiles || !layout_ok(layout, L) || n_mat < 0 || (n_mat > 0 && !mat_table)) return FSE_E_INVAL;
    int rc = ensure_materials_pushed();
    if (rc) return rc;
    const size_t bytes = (size_t)w->W * w->H * (size_t)L.stride;
    rc = ensure_tile_stage(w, bytes + (size_t)std::max(n_mat, 1) * 8);
    if (rc) return rc;
    uint64_t *d_table = nullptr;
    if (n_mat > 0) {
        d_table = reinterpret_cast<uint64_t *>(w->tile_stage + ((bytes + 7) & ~(size_t)7));
        FSE_CUDA_TRY(cudaMemcpyAsync(d_table, mat_table, (size_t)n_mat * 8, cudaMemcpyHostToDevice, w->stream));
    }
    // the caller's bytes first, so that the fields not written survive
    FSE_CUDA_TRY(cudaMemcpyAsync(w->tile_stage, tiles, bytes, cudaMemcpyHostToDevice, w->stream));
    k_tiles_out<<<grid_of(w), 256, 0, w->stream>>>(w->d, g_dev_mt, w->tile_stage, L, d_table, n_mat);
    FSE_CUDA_TRY(cudaGetLastError());
    count_launches(1);
    FSE_CUDA_TRY(cudaMemcpyAsync(tiles, w->tile_stage, bytes, cudaMemcpyDeviceToHost, w->stream));
    FSE_CUDA_TRY(cudaStreamSynchronize(w->stream));
    return FSE_OK;
}

}  // extern "C"
