// fse_islands.cu -- solid islands: world::physicsCheck (source/engine/world.cpp:
// 3330-3445), the 4-connected flood fill from one cell that cuts a small floating
// SOLID region (at most 1000 cells) out of the grid so the host can make a rigid
// body of it, and the same test for every region at once by connected-component
// labelling.
//
// physicsCheck's result does not depend on the flood's order: the reference stops
// counting past 1000 cells and cuts only a region of at most 1000, so the outcome
// is the whole region or nothing. Here one CTA floods level by level (a breadth-
// first frontier in a shared list, visits marked with a per-call epoch so nothing
// needs clearing) and stops as soon as the count passes 1000.
//
// The all-regions pass is union-find labelling: every SOLID cell starts as its own
// root, each SOLID right/down pair is united by linking the larger root under the
// smaller with an atomic compare-and-swap, so a region's final label is its
// smallest cell index whatever the thread timing.
#include <algorithm>
#include <vector>

#include "fse_host.cuh"

namespace fse {

constexpr int FLOOD_MAX = 1000;  // world.cpp:3348: count <= 1000
constexpr int FLOOD_THREADS = 1024;

__device__ __forceinline__ bool solid_at(const WorldDev &w, const uint8_t *s_type, int c) {
    return s_type[w.id[c]] == T_SOLID;
}

// remove one cell as physicsCheck does (Tiles_NOTHING, dirty), counted as destroyed
__device__ __forceinline__ void cut_cell(const WorldDev &w, const MatTable *mt, size_t c) {
    atomicAdd((unsigned long long *)&w.ledger[LED_DN * MAXMAT + w.id[c]], 1ull);
    w.id[c] = (uint16_t)mt->id_air;
    w.col[c] = 0u;
    w.sc[c] = 0;
    w.fl[c] = 0;
    w.df[c] = 0;
    if (w.dirty) w.dirty[c] = 1;
}

// out: [0] cells cut, [1..4] bbox (min x, min y, max x, max y)
__global__ void __launch_bounds__(FLOOD_THREADS) k_flood(const WorldDev *__restrict__ wd, const MatTable *__restrict__ mt,
                                                         int x0, int y0, uint32_t epoch, uint32_t *mark, int32_t *list,
                                                         int32_t *out, uint32_t *pix, int want_pix) {
    __shared__ uint8_t s_type[MAXMAT];
    __shared__ int s_tail, s_over, s_minx, s_miny, s_maxx, s_maxy;
    for (int k = threadIdx.x; k < MAXMAT; k += blockDim.x) s_type[k] = (uint8_t)(k < mt->n ? mt_type(mt->a[k]) : 0);
    const WorldDev &w = *wd;
    const int W = w.W, H = w.H;
    if (threadIdx.x == 0) {
        s_tail = 0;
        s_over = 0;
        s_minx = W;
        s_miny = H;
        s_maxx = -1;
        s_maxy = -1;
    }
    __syncthreads();
    const int seed = y0 * W + x0;
    if (!solid_at(w, s_type, seed)) {  // world.cpp:3332
        if (threadIdx.x == 0) out[0] = 0;
        return;
    }
    if (threadIdx.x == 0) {
        atomicExch(&mark[seed], epoch);
        list[0] = seed;
        s_tail = 1;
    }
    __syncthreads();
    int head = 0;
    // a region of n cells has at most n levels; past FLOOD_MAX + 1 cells the flood stops
    for (int level = 0; level <= FLOOD_MAX + 1; level++) {
        const int tail = s_tail;
        const bool stop = head >= tail || s_over != 0;
        __syncthreads();
        if (stop) break;
        for (int k = head + (int)threadIdx.x; k < tail; k += blockDim.x) {
            const int c = list[k], cx = c % W, cy = c / W;
            const int nb[4] = {cx + 1 < W ? c + 1 : -1, cy + 1 < H ? c + W : -1, cx > 0 ? c - 1 : -1,
                               cy > 0 ? c - W : -1};
#pragma unroll
            for (int j = 0; j < 4; j++) {
                const int n = nb[j];
                if (n < 0 || !solid_at(w, s_type, n)) continue;
                if (atomicExch(&mark[n], epoch) == epoch) continue;  // visited in this call
                const int slot = atomicAdd(&s_tail, 1);
                if (slot <= FLOOD_MAX)
                    list[slot] = n;
                else
                    s_over = 1;  // more than FLOOD_MAX cells: nothing is cut
            }
        }
        head = tail;
        __syncthreads();
    }
    const int count = s_tail;
    if (s_over || count > FLOOD_MAX) {
        if (threadIdx.x == 0) out[0] = 0;
        return;
    }
    for (int k = threadIdx.x; k < count; k += blockDim.x) {
        const int c = list[k];
        atomicMin(&s_minx, c % W);
        atomicMax(&s_maxx, c % W);
        atomicMin(&s_miny, c / W);
        atomicMax(&s_maxy, c / W);
    }
    __syncthreads();
    const int bw = s_maxx - s_minx + 1, bh = s_maxy - s_miny + 1;
    if (want_pix && count > 10) {  // world.cpp:3350-3366: the region's colours
        for (int k = threadIdx.x; k < bw * bh; k += blockDim.x) pix[k] = 0u;
        __syncthreads();
        for (int k = threadIdx.x; k < count; k += blockDim.x) {
            const int c = list[k];
            pix[(c / W - s_miny) * bw + (c % W - s_minx)] = w.col[c];
        }
        __syncthreads();
    }
    for (int k = threadIdx.x; k < count; k += blockDim.x) cut_cell(w, mt, (size_t)list[k]);
    if (threadIdx.x == 0) {
        out[0] = count;
        out[1] = s_minx;
        out[2] = s_miny;
        out[3] = s_maxx;
        out[4] = s_maxy;
    }
}

// ---------------------------------------------------------- labelling
// lab[x] <= x holds throughout; a root has lab[r] == r
__device__ __forceinline__ int root_of(int32_t *lab, int x) {
    int cur = lab[x];
    if (cur != x) {
        int next, prev = x;
        while (cur > (next = lab[cur])) {  // path halving on the way up
            lab[prev] = next;
            prev = cur;
            cur = next;
        }
    }
    return cur;
}

__device__ __forceinline__ void unite(int32_t *lab, int a, int b, int32_t *err) {
    int ra = root_of(lab, a), rb = root_of(lab, b);
    for (int guard = 0; ra != rb; guard++) {
        if (guard > (1 << 20)) {  // cannot happen: every retry moves to a smaller root
            atomicOr(err, ERR_TIMEOUT);
            return;
        }
        if (ra < rb) {
            const int ret = atomicCAS(&lab[rb], rb, ra);
            if (ret == rb) return;
            rb = root_of(lab, ret);
        } else {
            const int ret = atomicCAS(&lab[ra], ra, rb);
            if (ret == ra) return;
            ra = root_of(lab, ret);
        }
    }
}

__global__ void k_ccl_init(const WorldDev *__restrict__ wd, const MatTable *__restrict__ mt, int32_t *lab) {
    __shared__ uint8_t s_type[MAXMAT];
    for (int k = threadIdx.x; k < MAXMAT; k += blockDim.x) s_type[k] = (uint8_t)(k < mt->n ? mt_type(mt->a[k]) : 0);
    __syncthreads();
    const WorldDev &w = *wd;
    const int n = w.W * w.H;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        lab[i] = solid_at(w, s_type, i) ? i : -1;
}

__global__ void k_ccl_unite(const WorldDev *__restrict__ wd, int32_t *lab) {
    const WorldDev &w = *wd;
    const int W = w.W, n = w.W * w.H;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        if (lab[i] < 0) continue;
        if ((i % W) + 1 < W && lab[i + 1] >= 0) unite(lab, i, i + 1, w.err);
        if (i + W < n && lab[i + W] >= 0) unite(lab, i, i + W, w.err);
    }
}

// labels to roots, and region sizes into aux (zeroed before). The walk to the root
// only reads: the one write per cell is its own root, so a walk passing through a
// cell sees its old parent or its root, both on the way up. (Path-halving writes
// here could overwrite a cell's freshly written root with an older ancestor.)
__global__ void k_ccl_size(const WorldDev *__restrict__ wd, int32_t *lab, int32_t *aux) {
    const WorldDev &w = *wd;
    const int n = w.W * w.H;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        if (lab[i] < 0) continue;
        int r = i, p;
        while ((p = lab[r]) != r) r = p;
        lab[i] = r;
        atomicAdd(&aux[r], 1);
    }
}

// The regions to report are numbered in root order by a scan over contiguous
// segments of the cell range (one segment per block), so the table comes out
// sorted by root. Step 1: per segment, the roots of regions of at most max_cells.
constexpr int SEG_BLOCKS = 1024;
constexpr int SEG_THREADS = 256;

__device__ __forceinline__ bool picked(const int32_t *lab, const int32_t *aux, int r, int max_cells) {
    return lab[r] == r && aux[r] <= max_cells;
}

__device__ __forceinline__ int block_sum(int v, int *s_warp) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) s_warp[threadIdx.x >> 5] = v;
    __syncthreads();
    int t = 0;
    if (threadIdx.x == 0)
        for (int k = 0; k < (int)(blockDim.x >> 5); k++) t += s_warp[k];
    __syncthreads();
    return t;  // valid in thread 0
}

__global__ void k_ccl_count(const WorldDev *__restrict__ wd, const int32_t *lab, const int32_t *aux, int max_cells,
                            int32_t *seg_sum) {
    __shared__ int s_warp[32];
    const WorldDev &w = *wd;
    const int n = w.W * w.H, seg = (n + gridDim.x - 1) / gridDim.x;
    const int b0 = blockIdx.x * seg, b1 = min(n, b0 + seg);
    int c = 0;
    for (int r = b0 + threadIdx.x; r < b1; r += blockDim.x) c += picked(lab, aux, r, max_cells) ? 1 : 0;
    const int t = block_sum(c, s_warp);
    if (threadIdx.x == 0) seg_sum[blockIdx.x] = t;
}

// step 2: exclusive scan of the segment counts (one block of SEG_BLOCKS threads);
// seg_sum[SEG_BLOCKS] = the total
__global__ void k_ccl_scan(int32_t *seg_sum) {
    __shared__ int s[32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int v = seg_sum[threadIdx.x];
    int inc = v;
    for (int o = 1; o < 32; o <<= 1) {
        const int u = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += u;
    }
    if (lane == 31) s[wid] = inc;
    __syncthreads();
    if (wid == 0) {
        int a = s[lane];
        for (int o = 1; o < 32; o <<= 1) {
            const int u = __shfl_up_sync(0xffffffffu, a, o);
            if (lane >= o) a += u;
        }
        s[lane] = a;
    }
    __syncthreads();
    const int excl = (wid > 0 ? s[wid - 1] : 0) + inc - v;
    seg_sum[threadIdx.x] = excl;
    if (threadIdx.x == SEG_BLOCKS - 1) seg_sum[SEG_BLOCKS] = excl + v;
}

// step 3: each segment numbers its roots in order; aux[r] becomes -(entry + 1)
__global__ void k_ccl_pick(const WorldDev *__restrict__ wd, const int32_t *lab, int32_t *aux, int max_cells,
                           const int32_t *seg_base, fse_island *tab) {
    __shared__ int s_warp[SEG_THREADS / 32];
    __shared__ int s_carry;
    const WorldDev &w = *wd;
    const int n = w.W * w.H, seg = (n + gridDim.x - 1) / gridDim.x;
    const int b0 = blockIdx.x * seg, b1 = min(n, b0 + seg);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (threadIdx.x == 0) s_carry = seg_base[blockIdx.x];
    __syncthreads();
    for (int base = b0; base < b1; base += blockDim.x) {
        const int r = base + threadIdx.x;
        const bool p = r < b1 && picked(lab, aux, r, max_cells);
        const unsigned m = __ballot_sync(0xffffffffu, p);
        if (lane == 0) s_warp[wid] = __popc(m);
        __syncthreads();
        int before = s_carry;
        for (int k = 0; k < wid; k++) before += s_warp[k];
        if (p) {
            const int idx = before + __popc(m & ((1u << lane) - 1u));
            fse_island t;
            t.root = r;
            t.cells = aux[r];
            t.min_x = w.W;
            t.min_y = w.H;
            t.max_x = -1;
            t.max_y = -1;
            tab[idx] = t;
            aux[r] = -(idx + 1);
        }
        __syncthreads();
        if (threadIdx.x == 0)
            for (int k = 0; k < SEG_THREADS / 32; k++) s_carry += s_warp[k];
        __syncthreads();
    }
}

__global__ void k_ccl_bbox(const WorldDev *__restrict__ wd, const MatTable *__restrict__ mt, const int32_t *lab,
                           const int32_t *aux, fse_island *tab, int remove) {
    const WorldDev &w = *wd;
    const int W = w.W, n = w.W * w.H;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        if (lab[i] < 0) continue;
        const int a = aux[lab[i]];
        if (a >= 0) continue;
        fse_island &t = tab[-a - 1];
        atomicMin(&t.min_x, i % W);
        atomicMax(&t.max_x, i % W);
        atomicMin(&t.min_y, i / W);
        atomicMax(&t.max_y, i / W);
        if (remove) cut_cell(w, mt, (size_t)i);
    }
}

}  // namespace fse

using namespace fse;

template <typename T>
static bool grow(fse_world *w, T **p, size_t n) {
    if (*p) return true;
    if (cudaMalloc((void **)p, std::max<size_t>(n, 1) * sizeof(T)) != cudaSuccess) {
        *p = nullptr;
        cudaGetLastError();
        return false;
    }
    w->bytes += n * sizeof(T);
    return true;
}

extern "C" {

int fse_world_physics_check(fse_world *w, int x, int y, int *out_cells, int32_t out_bbox[4], uint32_t *pixels,
                            int64_t pixels_cap) {
    if (!w || !out_cells) return FSE_E_INVAL;
    *out_cells = 0;
    if (x < 0 || y < 0 || x >= w->W || y >= w->H) return FSE_OK;
    int rc = ensure_materials_pushed();
    if (rc) return rc;
    const size_t n = (size_t)w->W * w->H;
    if (!w->isl_mark) {
        if (!grow(w, &w->isl_mark, n)) return FSE_E_NOMEM;
        FSE_CUDA_TRY(cudaMemsetAsync(w->isl_mark, 0, n * 4, w->stream));
        w->isl_epoch = 0;
    }
    // a region of at most 1000 cells fits a 1000 x 1000 image
    if (!grow(w, &w->isl_list, FLOOD_MAX + 8) || !grow(w, &w->isl_out, 8) ||
        !grow(w, &w->isl_pix, (size_t)FLOOD_MAX * FLOOD_MAX))
        return FSE_E_NOMEM;
    if (++w->isl_epoch == 0) {  // epochs wrapped: clear the marks once
        FSE_CUDA_TRY(cudaMemsetAsync(w->isl_mark, 0, n * 4, w->stream));
        w->isl_epoch = 1;
    }
    k_flood<<<1, FLOOD_THREADS, 0, w->stream>>>(w->d, g_dev_mt, x, y, w->isl_epoch, w->isl_mark, w->isl_list,
                                                  w->isl_out, w->isl_pix, pixels ? 1 : 0);
    FSE_CUDA_TRY(cudaGetLastError());
    count_launches(1);
    int32_t res[5];
    FSE_CUDA_TRY(cudaMemcpyAsync(res, w->isl_out, sizeof(res), cudaMemcpyDeviceToHost, w->stream));
    FSE_CUDA_TRY(cudaStreamSynchronize(w->stream));
    *out_cells = res[0];
    if (res[0] > 0) {
        if (out_bbox)
            for (int k = 0; k < 4; k++) out_bbox[k] = res[1 + k];
        const int64_t bw = res[3] - res[1] + 1, bh = res[4] - res[2] + 1;
        if (pixels && res[0] > 10 && bw * bh <= pixels_cap) {
            FSE_CUDA_TRY(cudaMemcpy(pixels, w->isl_pix, (size_t)(bw * bh) * 4, cudaMemcpyDeviceToHost));
        }
    }
    return status_from_err(0);
}

int fse_world_islands(fse_world *w, int max_cells, int remove, fse_island *out, int cap, int *out_n) {
    if (!w || max_cells < 0 || cap < 0 || (cap > 0 && !out)) return FSE_E_INVAL;
    int rc = ensure_materials_pushed();
    if (rc) return rc;
    const size_t n = (size_t)w->W * w->H;
    if (!grow(w, &w->isl_lab, n) || !grow(w, &w->isl_aux, n) || !grow(w, &w->isl_seg, SEG_BLOCKS + 1))
        return FSE_E_NOMEM;
    const int blocks = (int)std::max<size_t>(1, std::min<size_t>((n + 255) / 256, (size_t)sm_count() * 16));
    cudaStream_t s = w->stream;
    k_ccl_init<<<blocks, 256, 0, s>>>(w->d, g_dev_mt, w->isl_lab);
    k_ccl_unite<<<blocks, 256, 0, s>>>(w->d, w->isl_lab);
    FSE_CUDA_TRY(cudaMemsetAsync(w->isl_aux, 0, n * 4, s));
    k_ccl_size<<<blocks, 256, 0, s>>>(w->d, w->isl_lab, w->isl_aux);
    k_ccl_count<<<SEG_BLOCKS, SEG_THREADS, 0, s>>>(w->d, w->isl_lab, w->isl_aux, max_cells, w->isl_seg);
    k_ccl_scan<<<1, SEG_BLOCKS, 0, s>>>(w->isl_seg);
    int32_t found = 0;
    FSE_CUDA_TRY(cudaMemcpyAsync(&found, w->isl_seg + SEG_BLOCKS, 4, cudaMemcpyDeviceToHost, s));
    FSE_CUDA_TRY(cudaStreamSynchronize(s));
    count_launches(5);
    if (found > w->isl_tab_cap) {
        if (w->isl_tab) cudaFree(w->isl_tab);
        w->isl_tab = nullptr;
        w->isl_tab_cap = 0;
        if (!grow(w, &w->isl_tab, (size_t)found)) return FSE_E_NOMEM;
        w->isl_tab_cap = found;
    }
    if (found > 0) {
        k_ccl_pick<<<SEG_BLOCKS, SEG_THREADS, 0, s>>>(w->d, w->isl_lab, w->isl_aux, max_cells, w->isl_seg, w->isl_tab);
        k_ccl_bbox<<<blocks, 256, 0, s>>>(w->d, g_dev_mt, w->isl_lab, w->isl_aux, w->isl_tab, remove);
        FSE_CUDA_TRY(cudaGetLastError());
        count_launches(2);
    }
    if (out_n) *out_n = found;
    if (cap > 0 && found > 0)  // the table is in root order already
        FSE_CUDA_TRY(cudaMemcpyAsync(out, w->isl_tab, (size_t)std::min(found, cap) * sizeof(fse_island),
                                     cudaMemcpyDeviceToHost, s));
    FSE_CUDA_TRY(cudaStreamSynchronize(s));
    int32_t err = 0;
    FSE_CUDA_TRY(cudaMemcpy(&err, w->h.err, 4, cudaMemcpyDeviceToHost));
    return status_from_err(err);
}

}  // extern "C"
