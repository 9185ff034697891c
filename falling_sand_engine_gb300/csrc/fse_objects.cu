// fse_objects.cu -- rigid-body OBJECT tiles: stamping before the tick
// (source/engine/game.cpp:1768-1814), readback after it (game.cpp:1896-1983) and
// the per-tick OBJECT-cell export to the host-side rigid-body solver.
//
// Stamp and readback resolve body tiles inside one CTA per world by deferred
// acceptance (see k_obj_rounds): the result is the reference's tile-by-tile one,
// and displaced particles are appended in (body, tile) order.
#include <algorithm>
#include <vector>

#include "fse_host.cuh"

namespace fse {

__constant__ int c_dirs[5][2] = {{0, 0}, {1, 0}, {-1, 0}, {0, 1}, {0, -1}};

__device__ __forceinline__ void body_pos(const fse_body &b, int tx, int ty, int &wx, int &wy) {
    // int wx = (int)(tx * c - (ty + 1) * s + x); int wy = (int)(tx * s + (ty + 1) * c + y);
    float fx = __fadd_rn(__fsub_rn(__fmul_rn((float)tx, b.cos_a), __fmul_rn((float)(ty + 1), b.sin_a)), b.x);
    float fy = __fadd_rn(__fadd_rn(__fmul_rn((float)tx, b.sin_a), __fmul_rn((float)(ty + 1), b.cos_a)), b.y);
    wx = (int)fx;
    wy = (int)fy;
}

__device__ __forceinline__ int block_scan_excl(int v, int *s, int *total) {
    int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    int inc = v;
    for (int o = 1; o < 32; o <<= 1) {
        int t = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += t;
    }
    if (lane == 31) s[wid] = inc;
    __syncthreads();
    if (wid == 0) {
        int a = lane < nw ? s[lane] : 0;
        for (int o = 1; o < 32; o <<= 1) {
            int t = __shfl_up_sync(0xffffffffu, a, o);
            if (lane >= o) a += t;
        }
        if (lane < nw) s[lane] = a;
    }
    __syncthreads();
    int before = wid > 0 ? s[wid - 1] : 0;
    *total = s[nw - 1];
    __syncthreads();
    return before + inc - v;
}

__device__ __forceinline__ int body_of(const uint32_t *__restrict__ prefix, int nb, uint32_t g) {
    int lo = 0, hi = nb - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (prefix[mid] <= g) lo = mid; else hi = mid - 1;
    }
    return lo;
}

// mode 0 = stamp, 1 = readback; prefix[b] = first global tile index of body b.
// ptr (per tile: the next offset to try, 5 = none left) and held (per tile: the
// cell it holds, -1 = none) are scratch of prefix[nb] entries.
//
// The reference walks the tiles one after another (bodies in order, tx-major,
// ty-minor): each takes the first of its five cells that is usable at that moment
// (stamp: AIR, SAND or SOUP; readback: the body's material), and a taken cell is
// not usable by the tiles after it. Here the tiles propose in parallel, each cell
// keeping its lowest proposer (claim = atomicMin of the tile index) and displacing
// higher ones, a rejected or displaced tile proposing its next cell: deferred
// acceptance with the same priority order at every cell, whose outcome is the
// sequential one. Usability is read from the grid before any write, since only the
// taking itself makes a cell unusable. Displaced particles are then appended in
// tile order.
__device__ __forceinline__ bool tile_usable(const WorldDev &w, const MatTable *__restrict__ mt, int mode, int c,
                                            int body_id) {
    const int cid = w.id[c];
    if (mode == 0) {
        const int ty = mt_type(mt->a[cid]);
        return ty == T_AIR || ty == T_SAND || ty == T_SOUP;
    }
    return cid == body_id;
}

// tile g proposes its next usable cell from ptr[g] on (a cell claimed by an
// earlier tile is skipped for good); returns the proposer displaced from that cell
// (or 0xffffffff), and records the cell in held[g] (-1 when none is left)
__device__ __forceinline__ uint32_t tile_propose(const WorldDev &w, const MatTable *__restrict__ mt,
                                                 const fse_body *__restrict__ bodies,
                                                 const uint32_t *__restrict__ prefix, int nb, int mode, uint32_t g,
                                                 uint32_t *ptr, int32_t *held, uint32_t *claim) {
    const int bi = body_of(prefix, nb, g);
    const fse_body b = bodies[bi];
    const int t = (int)(g - prefix[bi]);
    int wx, wy;
    body_pos(b, t / b.h, t % b.h, wx, wy);
    int d = (int)ptr[g];
    for (; d < 5; d++) {
        const int xd = wx + c_dirs[d][0], yd = wy + c_dirs[d][1];
        if (xd < 0 || yd < 0 || xd >= w.W || yd >= w.H) continue;
        const int c = yd * w.W + xd;
        if (!tile_usable(w, mt, mode, c, (int)b.id) || claim[c] < g) continue;
        const uint32_t old = atomicMin(&claim[c], g);
        ptr[g] = (uint32_t)d;
        held[g] = c;
        return old;
    }
    ptr[g] = 5;
    held[g] = -1;
    return 0xffffffffu;
}

// mode 0 = stamp, 1 = readback; prefix[b] = first global tile index of body b.
// Scratch of prefix[nb] entries: ptr (the next offset to try, 5 = none left), held
// (the cell a tile holds, -1 = none), two work lists and a queued mark.
//
// The reference walks the tiles one after another (bodies in order, tx-major,
// ty-minor): each takes the first of its five cells that is usable at that moment
// (stamp: AIR, SAND or SOUP; readback: the body's material), and a taken cell is
// not usable by the tiles after it. Here the tiles propose in parallel, each cell
// keeping its lowest proposer (claim = atomicMin of the tile index) and displacing
// higher ones, a rejected or displaced tile proposing its next cell: deferred
// acceptance with the same priority order at every cell, whose outcome is the
// sequential one. Usability is read from the grid before any write, since only the
// taking itself makes a cell unusable. After one round over all tiles, only the
// tiles that lost a cell and the holders their proposals displace are looked at.
// Displaced particles are then appended in tile order.
__global__ void __launch_bounds__(1024) k_obj_rounds(WorldDev *wd, const MatTable *__restrict__ mt, fse_body *bodies,
                                                     const uint32_t *__restrict__ prefix, int nb, uint32_t *ptr,
                                                     int32_t *held, uint32_t *list_a, uint32_t *list_b,
                                                     uint32_t *queued, uint32_t *claim, int mode,
                                                     long long *removed) {
    WorldDev &w = *wd;
    const int W = w.W;
    __shared__ int s_scan[40];
    __shared__ int s_na, s_nb, s_spawn_base;
    const uint32_t total = prefix[nb];
    if (threadIdx.x == 0) {
        s_spawn_base = *w.part_count;
        s_na = 0;
    }
    for (uint32_t g = threadIdx.x; g < total; g += blockDim.x) {
        ptr[g] = 0;
        queued[g] = 0;
    }
    __syncthreads();
    // ---- first round: every tile proposes
    for (uint32_t g = threadIdx.x; g < total; g += blockDim.x)
        tile_propose(w, mt, bodies, prefix, nb, mode, g, ptr, held, claim);
    __syncthreads();
    for (uint32_t g = threadIdx.x; g < total; g += blockDim.x) {
        const int c = held[g];
        if (c >= 0 && claim[c] != g) {  // lost its cell to an earlier tile
            held[g] = -1;
            ptr[g] += 1;
            if (ptr[g] < 5) list_a[atomicAdd(&s_na, 1)] = g;
        }
    }
    __syncthreads();
    // ---- later rounds over the open tiles (list_a) and the holders they displace
    for (long long round = 0; s_na > 0; round++) {
        if (round > 8LL * total + 8) {  // cannot happen: every round moves a pointer forward
            if (threadIdx.x == 0) atomicOr(w.err, ERR_TIMEOUT);
            break;
        }
        const int na = s_na;
        if (threadIdx.x == 0) s_nb = 0;
        __syncthreads();
        // propose; the proposer and the holder it may displace are checked next
        for (int j = threadIdx.x; j < na; j += blockDim.x) {
            const uint32_t g = list_a[j];
            const uint32_t old = tile_propose(w, mt, bodies, prefix, nb, mode, g, ptr, held, claim);
            if (held[g] >= 0 && atomicExch(&queued[g], 1u) == 0u) list_b[atomicAdd(&s_nb, 1)] = g;
            if (old != 0xffffffffu && old > g && atomicExch(&queued[old], 1u) == 0u) list_b[atomicAdd(&s_nb, 1)] = old;
        }
        __syncthreads();
        if (threadIdx.x == 0) s_na = 0;
        __syncthreads();
        const int nbv = s_nb;
        for (int j = threadIdx.x; j < nbv; j += blockDim.x) {
            const uint32_t g = list_b[j];
            queued[g] = 0;
            const int c = held[g];
            if (c >= 0 && claim[c] != g) {
                held[g] = -1;
                ptr[g] += 1;
                if (ptr[g] < 5) list_a[atomicAdd(&s_na, 1)] = g;
            }
        }
        __syncthreads();
    }
    // ---- apply, tiles in order; reads of the cells first (the displaced
    // particles), then the writes
    const uint32_t pk = pass_key(w.seed, *w.tick, PH_STAMP);
    if (mode == 0) {
        for (uint32_t base = 0; base < total; base += blockDim.x) {
            const uint32_t g = base + threadIdx.x;
            const int tg = g < total ? held[g] : -1;
            int ty = -1;
            if (tg >= 0) ty = mt_type(mt->a[w.id[tg]]);
            const bool spawn = ty == T_SAND || ty == T_SOUP;
            int tot_s;
            const int ex_s = block_scan_excl(spawn ? 1 : 0, s_scan, &tot_s);
            if (spawn) {
                const int bi = body_of(prefix, nb, g);
                fse_body &b = bodies[bi];
                const int pos = s_spawn_base + ex_s;
                if (pos < w.part_cap) {
                    const uint32_t ck = cell_key(pk, (uint32_t)bi, g - prefix[bi]);
                    // CellData(tile, wxd, wyd - 3, (rand()%10-5)/10.0f, -(rand()%5+5)/10.0f, 0, 0.1)
                    w.p.x[pos] = (float)(tg % W);
                    w.p.y[pos] = (float)(tg / W - 3);
                    w.p.vx[pos] = (float)((int)(draw_k(ck, 0) % 10) - 5) / 10.0f;
                    w.p.vy[pos] = (float)(-((int)(draw_k(ck, 1) % 5) + 5)) / 10.0f;
                    w.p.ax[pos] = 0.f;
                    w.p.ay[pos] = 0.1f;
                    w.p.tx[pos] = 0.f;
                    w.p.ty[pos] = 0.f;
                    w.p.tf[pos] = 0.f;
                    w.p.life[pos] = 0;
                    w.p.fade[pos] = 60;
                    w.p.col[pos] = w.col[tg];
                    w.p.sc[pos] = w.sc[tg];
                    if (w.tp) w.p.tp[pos] = ty == T_SOUP ? w.tp[tg] : (int16_t)0;
                    w.p.id[pos] = w.id[tg];
                    w.p.fl[pos] = w.fl[tg];
                    w.p.bits[pos] = 0;
                } else {
                    atomicOr(w.err, ERR_PART_CAP);
                }
                if (ty == T_SOUP) {
                    if (!w.f32)  // f32 amounts: no fluid rows
                        atomicAdd((unsigned long long *)&w.ledger[LED_DF * MAXMAT + w.id[tg]],
                                  (unsigned long long)(long long)w.df[tg]);
                    atomicAdd(&b.n_soup, 1);
                } else {
                    atomicAdd(&b.n_sand, 1);
                }
            }
            __syncthreads();
            if (threadIdx.x == 0) s_spawn_base += tot_s;
            __syncthreads();
        }
    }
    long long rem_local = 0;
    for (uint32_t g = threadIdx.x; g < total; g += blockDim.x) {
        const int tg = held[g];
        if (tg < 0) continue;
        fse_body &b = bodies[body_of(prefix, nb, g)];
        if (mode == 0) {
            w.id[tg] = b.id;
            w.col[tg] = b.colour;
            w.sc[tg] = 0;
            w.fl[tg] = 0;
            w.df[tg] = 0;
            atomicAdd(&b.n_placed, 1);
            atomicAdd((unsigned long long *)&w.ledger[LED_CN * MAXMAT + b.id], 1ull);
        } else {
            atomicAdd((unsigned long long *)&w.ledger[LED_DN * MAXMAT + w.id[tg]], 1ull);
            w.id[tg] = (uint16_t)mt->id_air;
            w.col[tg] = 0;
            w.sc[tg] = 0;
            w.fl[tg] = 0;
            w.df[tg] = 0;
            atomicAdd(&b.n_recovered, 1);
            rem_local++;
        }
        if (w.dirty) w.dirty[tg] = 1;
        claim[tg] = 0xffffffffu;  // every claimed cell has its lowest proposer as holder
    }
    if (rem_local) atomicAdd((unsigned long long *)removed, (unsigned long long)rem_local);
    __syncthreads();
    if (threadIdx.x == 0 && mode == 0) *w.part_count = min(s_spawn_base, w.part_cap);
}

// 1 bit per cell, LSB first: one warp vote per 32 cells
__global__ void k_obj_mask(const WorldDev *__restrict__ wd, const MatTable *__restrict__ mt, uint32_t *bits) {
    const WorldDev &w = *wd;
    const size_t n = (size_t)w.W * w.H;
    const size_t nwords = (n + 31) / 32;
    const int lane = threadIdx.x & 31;
    const size_t warp = (blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5;
    const size_t nwarps = ((size_t)gridDim.x * blockDim.x) >> 5;
    for (size_t wd_i = warp; wd_i < nwords; wd_i += nwarps) {
        size_t c = wd_i * 32 + lane;
        bool obj = c < n && mt_type(mt->a[w.id[c]]) == T_OBJECT;
        unsigned m = __ballot_sync(0xffffffffu, obj);
        if (lane == 0) bits[wd_i] = m;
    }
}

// ascending list of OBJECT cells from the mask: per-block word ranges, scanned
__global__ void k_obj_list_count(const uint32_t *bits, size_t nwords, int32_t *blk) {
    size_t seg = (nwords + gridDim.x - 1) / gridDim.x;
    size_t b0 = blockIdx.x * seg, b1 = min(nwords, b0 + seg);
    int c = 0;
    for (size_t i = b0 + threadIdx.x; i < b1; i += blockDim.x) c += __popc(bits[i]);
    for (int o = 16; o > 0; o >>= 1) c += __shfl_down_sync(0xffffffffu, c, o);
    __shared__ int s[32];
    if ((threadIdx.x & 31) == 0) s[threadIdx.x >> 5] = c;
    __syncthreads();
    if (threadIdx.x == 0) {
        int t = 0;
        for (int k = 0; k < (int)(blockDim.x >> 5); k++) t += s[k];
        blk[blockIdx.x] = t;
    }
}
__global__ void k_obj_list_scan(int32_t *blk, int nb, long long *total) {
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        long long run = 0;
        for (int b = 0; b < nb; b++) {
            long long v = blk[b];
            blk[b] = (int32_t)run;
            run += v;
        }
        *total = run;
    }
}
__global__ void k_obj_list_scatter(const uint32_t *bits, size_t nwords, const int32_t *blk, uint32_t *out, long long cap) {
    size_t seg = (nwords + gridDim.x - 1) / gridDim.x;
    size_t b0 = blockIdx.x * seg, b1 = min(nwords, b0 + seg);
    __shared__ int s[32];
    __shared__ long long s_carry;
    if (threadIdx.x == 0) s_carry = blk[blockIdx.x];
    __syncthreads();
    for (size_t base = b0; base < b1; base += blockDim.x) {
        size_t i = base + threadIdx.x;
        uint32_t m = i < b1 ? bits[i] : 0u;
        int v = __popc(m);
        int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
        int inc = v;
        for (int o = 1; o < 32; o <<= 1) {
            int t = __shfl_up_sync(0xffffffffu, inc, o);
            if (lane >= o) inc += t;
        }
        if (lane == 31) s[wid] = inc;
        __syncthreads();
        long long pos = s_carry + inc - v;
        for (int k = 0; k < wid; k++) pos += s[k];
        while (m) {
            int b = __ffs(m) - 1;
            m &= m - 1;
            if (pos < cap) out[pos] = (uint32_t)(i * 32 + b);
            pos++;
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            long long t = 0;
            for (int k = 0; k < nw; k++) t += s[k];
            s_carry += t;
        }
        __syncthreads();
    }
}

}  // namespace fse

using namespace fse;

static int obj_prepare(fse_world *w) {
    size_t n = (size_t)w->W * w->H;
    if (!w->claim) {
        if (cudaMalloc(&w->claim, n * 4) != cudaSuccess) {
            w->claim = nullptr;
            return FSE_E_NOMEM;
        }
        w->bytes += n * 4;
        cudaMemset(w->claim, 0xff, n * 4);
    }
    return FSE_OK;
}

static int obj_run(fse_world *w, fse_body *bodies, int n, int mode, int64_t *out_removed) {
    if (!w || n < 0 || (n > 0 && !bodies)) return FSE_E_INVAL;
    int rc = ensure_materials_pushed();
    if (rc) return rc;
    rc = obj_prepare(w);
    if (rc) return rc;
    if (n == 0) {
        if (out_removed) *out_removed = 0;
        return FSE_OK;
    }
    std::vector<uint32_t> prefix(n + 1, 0);
    const MatTable &t = host_table();
    for (int b = 0; b < n; b++) {
        if (bodies[b].w < 0 || bodies[b].h <= 0 || bodies[b].id >= t.n) return FSE_E_INVAL;
        if (mode == 0) bodies[b].n_sand = bodies[b].n_soup = bodies[b].n_placed = 0;
        else bodies[b].n_recovered = 0;
        prefix[b + 1] = prefix[b] + (uint32_t)(bodies[b].w * bodies[b].h);
    }
    size_t total = prefix[n];
    fse_body *d_b = nullptr;
    uint32_t *d_pref = nullptr, *d_open = nullptr, *d_next = nullptr, *d_la = nullptr, *d_lb = nullptr,
             *d_q = nullptr;
    int32_t *d_tgt = nullptr;
    long long *d_rem = nullptr;
    bool ok = cudaMalloc(&d_b, n * sizeof(fse_body)) == cudaSuccess &&
              cudaMalloc(&d_pref, (n + 1) * 4) == cudaSuccess &&
              cudaMalloc(&d_open, std::max<size_t>(total, 1) * 4) == cudaSuccess &&
              cudaMalloc(&d_next, std::max<size_t>(total, 1) * 4) == cudaSuccess &&
              cudaMalloc(&d_tgt, std::max<size_t>(total, 1) * 4) == cudaSuccess &&
              cudaMalloc(&d_la, std::max<size_t>(total, 1) * 4) == cudaSuccess &&
              cudaMalloc(&d_lb, std::max<size_t>(2 * total, 1) * 4) == cudaSuccess &&
              cudaMalloc(&d_q, std::max<size_t>(total, 1) * 4) == cudaSuccess &&
              cudaMalloc(&d_rem, 8) == cudaSuccess;
    int result = FSE_OK;
    if (!ok) {
        result = FSE_E_NOMEM;
    } else {
        cudaMemcpyAsync(d_b, bodies, n * sizeof(fse_body), cudaMemcpyHostToDevice, w->stream);
        cudaMemcpyAsync(d_pref, prefix.data(), (n + 1) * 4, cudaMemcpyHostToDevice, w->stream);
        cudaMemsetAsync(d_rem, 0, 8, w->stream);
        k_obj_rounds<<<1, 1024, 0, w->stream>>>(w->d, g_dev_mt, d_b, d_pref, n, d_open, d_tgt, d_la, d_lb, d_q,
                                                w->claim, mode, d_rem);
        long long rem = 0;
        cudaMemcpyAsync(bodies, d_b, n * sizeof(fse_body), cudaMemcpyDeviceToHost, w->stream);
        cudaMemcpyAsync(&rem, d_rem, 8, cudaMemcpyDeviceToHost, w->stream);
        if (cudaStreamSynchronize(w->stream) != cudaSuccess) result = FSE_E_CUDA;
        if (out_removed) *out_removed = rem;
    }
    cudaFree(d_b);
    cudaFree(d_pref);
    cudaFree(d_open);
    cudaFree(d_next);
    cudaFree(d_la);
    cudaFree(d_lb);
    cudaFree(d_q);
    cudaFree(d_tgt);
    cudaFree(d_rem);
    if (result) return result;
    return fse_world_sync(w);
}

extern "C" {

int fse_object_stamp(fse_world *w, fse_body *bodies, int n) { return obj_run(w, bodies, n, 0, nullptr); }

int fse_object_readback(fse_world *w, fse_body *bodies, int n, int64_t *out_removed) {
    return obj_run(w, bodies, n, 1, out_removed);
}

static int obj_mask_dev(fse_world *w) {
    size_t n = (size_t)w->W * w->H;
    size_t nwords = (n + 31) / 32;
    if (!w->mask_bits) {
        if (cudaMalloc(&w->mask_bits, nwords * 4) != cudaSuccess) {
            w->mask_bits = nullptr;
            return FSE_E_NOMEM;
        }
        w->bytes += nwords * 4;
    }
    int rc = ensure_materials_pushed();
    if (rc) return rc;
    int blocks = (int)std::min<size_t>((nwords * 32 + 255) / 256, (size_t)sm_count() * 8);
    k_obj_mask<<<std::max(blocks, 1), 256, 0, w->stream>>>(w->d, g_dev_mt, (uint32_t *)w->mask_bits);
    return cudaGetLastError() == cudaSuccess ? FSE_OK : FSE_E_CUDA;
}

int fse_object_mask_export(fse_world *w, uint8_t *host_bits) {
    if (!w || !host_bits) return FSE_E_INVAL;
    int rc = obj_mask_dev(w);
    if (rc) return rc;
    size_t n = (size_t)w->W * w->H;
    FSE_CUDA_TRY(cudaMemcpyAsync(host_bits, w->mask_bits, (n + 7) / 8, cudaMemcpyDeviceToHost, w->stream));
    FSE_CUDA_TRY(cudaStreamSynchronize(w->stream));
    return FSE_OK;
}

int fse_object_list_export(fse_world *w, uint32_t *host_idx, int64_t cap, int64_t *out_n) {
    if (!w || cap < 0 || (cap > 0 && !host_idx)) return FSE_E_INVAL;
    int rc = obj_mask_dev(w);
    if (rc) return rc;
    size_t n = (size_t)w->W * w->H, nwords = (n + 31) / 32;
    const int NB = 256;
    if (!w->obj_n) {
        if (cudaMalloc(&w->obj_n, 8 + (NB + 1) * 4) != cudaSuccess) return FSE_E_NOMEM;
    }
    int32_t *blk = (int32_t *)((char *)w->obj_n + 8);
    long long cap_dev = std::max<long long>(cap, 1);
    if (!w->obj_list || w->obj_list_cap < (size_t)cap_dev) {
        if (w->obj_list) cudaFree(w->obj_list);
        if (cudaMalloc(&w->obj_list, (size_t)cap_dev * 4) != cudaSuccess) {
            w->obj_list = nullptr;
            w->obj_list_cap = 0;
            return FSE_E_NOMEM;
        }
        w->obj_list_cap = (size_t)cap_dev;
    }
    k_obj_list_count<<<NB, 256, 0, w->stream>>>((uint32_t *)w->mask_bits, nwords, blk);
    k_obj_list_scan<<<1, 32, 0, w->stream>>>(blk, NB, (long long *)w->obj_n);
    k_obj_list_scatter<<<NB, 256, 0, w->stream>>>((uint32_t *)w->mask_bits, nwords, blk, w->obj_list, cap);
    long long total = 0;
    FSE_CUDA_TRY(cudaMemcpyAsync(&total, w->obj_n, 8, cudaMemcpyDeviceToHost, w->stream));
    FSE_CUDA_TRY(cudaStreamSynchronize(w->stream));
    long long m = std::min<long long>(total, cap);
    if (m > 0) {
        FSE_CUDA_TRY(cudaMemcpyAsync(host_idx, w->obj_list, (size_t)m * 4, cudaMemcpyDeviceToHost, w->stream));
        FSE_CUDA_TRY(cudaStreamSynchronize(w->stream));
    }
    if (out_n) *out_n = total;
    return FSE_OK;
}

}  // extern "C"
