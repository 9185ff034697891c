// fse_particles.cu -- free particles: the ordered append of particles spawned by
// the cell tick (world.cpp:1078,1110-1119,1222,1298,1901-1913) and the particle
// update world::tickCells() (world.cpp:2030-2195).
//
// Every kernel takes the world table, so one launch serves a single world or a
// whole batch: the per-world kernels handle world blockIdx.y (or blockIdx.x), the
// cooperative update and the compaction run over one index space holding every
// world's particles. Arithmetic on particle state uses the
// explicitly rounded intrinsics (__fadd_rn, __fmul_rn, __fdiv_rn, __fsqrt_rn) so
// that no multiply-add is contracted: the FP32 results equal a strict IEEE CPU
// evaluation of the same expressions bit for bit.
#include <algorithm>

#include "fse_internal.cuh"

namespace fse {

constexpr int PART_BLOCKS = 512;  // scan_tmp holds PART_BLOCKS + 1 entries per world
// per-world words of scan_tmp used by the compaction; world 0's entries
// 0 .. CMP_BLOCKS - 1 hold the compaction blocks' kept counts, then their prefix
constexpr int ST_KEPT_BEFORE = PART_BLOCKS - 2;  // kept particles of the worlds before
constexpr int ST_KEPT = PART_BLOCKS - 1;         // this world's kept particles (atomics)
constexpr int ST_COUNT = PART_BLOCKS;            // the world's new particle count

// p_state values
enum : uint8_t { PS_ALIVE = 0, PS_DEAD = 1 };

__constant__ int8_t c_spiral[1024][2];
__constant__ int c_spiral_n;

// -------------------------------------------------------------- spawn append
// Exclusive scan of the per-chunk-pass spawn counts of one world (one CTA per
// world); reserves the tail of the particle list for this tick's spawns.
__global__ void k_spawn_scan(const WorldDev *__restrict__ worlds) {
    const WorldDev &w = worlds[blockIdx.x];
    __shared__ int s_sum[32];
    __shared__ int s_carry;
    const int n = w.cell_iter * 4 * w.max_slots * w.cp_rows;
    if (threadIdx.x == 0) s_carry = 0;
    __syncthreads();
    for (int base = 0; base < n; base += blockDim.x) {
        int i = base + threadIdx.x;
        int v = (i < n) ? w.cp_count[i] : 0;
        int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
        int inc = v;
        for (int o = 1; o < 32; o <<= 1) {
            int t = __shfl_up_sync(0xffffffffu, inc, o);
            if (lane >= o) inc += t;
        }
        if (lane == 31) s_sum[wid] = inc;
        __syncthreads();
        if (wid == 0) {
            int s = lane < nw ? s_sum[lane] : 0;
            for (int o = 1; o < 32; o <<= 1) {
                int t = __shfl_up_sync(0xffffffffu, s, o);
                if (lane >= o) s += t;
            }
            if (lane < nw) s_sum[lane] = s;
        }
        __syncthreads();
        int before = (wid > 0 ? s_sum[wid - 1] : 0) + s_carry;
        if (i < n) w.cp_base[i] = before + inc - v;
        __syncthreads();
        if (threadIdx.x == 0) s_carry += s_sum[nw - 1];
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        int old = *w.part_count;
        long long nn = (long long)old + s_carry;
        if (nn > w.part_cap) {
            atomicOr(w.err, ERR_PART_CAP);
            nn = w.part_cap;
        }
        w.cp_base[n] = old;  // list position of the first spawned particle
        *w.part_count = (int)nn;
    }
}

__global__ void k_spawn_scatter(const WorldDev *__restrict__ worlds) {
    const WorldDev &w = worlds[blockIdx.y];
    const int n = min(*w.stage_count, w.stage_cap);
    const int first = w.cp_base[w.cell_iter * 4 * w.max_slots * w.cp_rows];
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) {
        const SpawnRec s = w.stage[r];
        long long pos = (long long)first + w.cp_base[s.cp] + s.rank;
        if (pos >= w.part_cap) continue;  // ERR_PART_CAP already recorded
        int i = (int)pos;
        w.p.x[i] = s.x;
        w.p.y[i] = s.y;
        w.p.vx[i] = s.vx;
        w.p.vy[i] = s.vy;
        w.p.ax[i] = 0.f;
        w.p.ay[i] = s.ay;
        w.p.tx[i] = 0.f;
        w.p.ty[i] = 0.f;
        w.p.tf[i] = 0.f;
        w.p.life[i] = s.lifetime;
        w.p.fade[i] = s.fade;
        w.p.col[i] = s.colour;
        w.p.sc[i] = s.scalar;
        if (w.tp) w.p.tp[i] = s.temp;  // particle temperatures exist with the grid's
        w.p.id[i] = s.id;
        w.p.fl[i] = s.flags;
        w.p.bits[i] = s.bits;
    }
}

// reset the per-tick spawn bookkeeping and advance the tick counter
__global__ void k_tick_end(const WorldDev *worlds) {
    const WorldDev &w = worlds[blockIdx.x];
    if (threadIdx.x == 0) {
        *w.stage_count = 0;
        *w.tick += 1;  // world.cpp:1925
    }
}

// ----------------------------------------------------------------- motion
__device__ __forceinline__ bool out_of_world(float x, float y, int W, int H) {
    // `x < 0 || (int)x >= width || y < 0 || (int)y >= height` (world.cpp:2056);
    // written so that NaN and huge values also count as outside
    return !(x >= 0.0f && x < (float)W && y >= 0.0f && y < (float)H);
}

__device__ __forceinline__ void led_part(const WorldDev &w, const MatTable *mt, int row_n, int row_f, int id,
                                         int32_t sc) {
    int ty = mt_type(mt->a[id]);
    if (ty == T_AIR) return;
    atomicAdd((unsigned long long *)&w.ledger[row_n * MAXMAT + id], 1ull);
    if (ty == T_SOUP && sc != 0 && !w.f32)  // f32 amounts: no fluid rows
        atomicAdd((unsigned long long *)&w.ledger[row_f * MAXMAT + id], (unsigned long long)(long long)sc);
}

// ------------------------------------------------------ the particle update
// world::tickCells (world.cpp:2030-2195) runs the particles one after another in
// list order, and each one moves, collides and deposits against the grid as the
// particles before it left it: a deposit can stop a later particle's flight, turn
// its previous cell from AIR into a tile (so it searches the spiral instead) and
// take a cell its spiral would have taken. Here every particle is computed at once
// and the sequential result is reached by iterating to a fixed point:
//
//   iteration k computes every particle's outcome (state, and the cell it fills or
//   merges into) against the grid of this tick's start plus the fills that
//   particles of lower index made in iteration k - 1;
//
// particle 0's outcome is final after iteration 0, particle 1's after iteration 1 at
// the latest, and so on, so the iteration ends (usually after a few rounds, as long
// as the chains of particles landing on each other's deposits) when the set of
// filled cells no longer changes, and its outcome is then exactly the sequential
// one. Fills are recorded in the diff word of the AIR cell they fill (the diff means
// nothing in an AIR cell; k_air_map zeroes it): 0x7fffffff - index, the largest
// value (lowest index) kept by atomicMax. A particle is computed again only if a
// fill changed near what it read (its bounding box of path and spiral cells against
// per-8x8-block change marks). The grid itself is written once, after convergence.

// outcome of a particle during the update (p_state); after the commit only
// PS_ALIVE and PS_DEAD remain
enum : uint8_t { PS_EXIT = 2, PS_DESTROY = 3, PS_FILL = 4, PS_MERGE = 5, PS_FAIL = 6 };

__device__ __forceinline__ void load_types(uint8_t *s_type, const MatTable *mt) {
    for (int k = threadIdx.x; k < MAXMAT; k += blockDim.x) s_type[k] = (uint8_t)(k < mt->n ? mt_type(mt->a[k]) : 0);
    __syncthreads();
}

__device__ __forceinline__ int32_t fill_code(int i) { return 0x7fffffff - i; }

// the material particle i sees at cell c: the grid's, or the tile a particle of
// lower index deposits there (fills are rewritten between iterations by other
// blocks, so they are read past L1)
__device__ __forceinline__ int view_id(const WorldDev &w, const uint8_t *s_type, int c, int i) {
    int id = w.id[c];
    if (s_type[id] == T_AIR) {
        const int32_t v = __ldcg(&w.df[c]);
        if (v != 0) {
            const int j = 0x7fffffff - v;
            if (j < i) id = w.p.id[j];
        }
    }
    return id;
}

// which 8x8 blocks hold AIR, from the grid the cell tick left (one thread per block);
// the diff word of every AIR cell is cleared for the fill records
__global__ void k_air_map(const WorldDev *__restrict__ worlds, const MatTable *__restrict__ mt) {
    __shared__ uint8_t s_type[MAXMAT];
    load_types(s_type, mt);
    const WorldDev &w = worlds[blockIdx.y];
    const int nb = w.amw * w.amh;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        w.scan_tmp[ST_KEPT] = 0;  // for the compaction's counts
        w.chg_n[2] = 0x7FFFFFFF;  // the particle update's lowest changing index, per parity
        w.chg_n[3] = 0x7FFFFFFF;
    }
    for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < nb; b += gridDim.x * blockDim.x) {
        const int bx = b % w.amw, by = b / w.amw;
        const int x0 = bx * 8, y0 = by * 8, x1 = min(x0 + 8, w.W), y1 = min(y0 + 8, w.H);
        uint8_t any = 0;
        for (int y = y0; y < y1; y++)
            for (int x = x0; x < x1; x++) {
                const size_t c = (size_t)y * w.W + x;
                if (s_type[w.id[c]] == T_AIR) {
                    any = 1;
                    w.df[c] = 0;
                }
            }
        w.airmap[b] = any;
        w.chg[b] = 0xFFFFFFFFu;
        w.chg[nb + b] = 0xFFFFFFFFu;
    }
}

// bounding box of the cells a particle read, packed as (x0 | y0 << 16, x1 | y1 << 16)
struct Box {
    int x0, y0, x1, y1;
    __device__ __forceinline__ void add(int x, int y) {
        x0 = min(x0, x);
        y0 = min(y0, y);
        x1 = max(x1, x);
        y1 = max(y1, y);
    }
};

// One particle's flight of world.cpp:2032-2188 against the view of particle i: writes
// its state into w.q, its kind into p_state, its target cell into p_cell and the box
// of the cells it read into p_box0 / p_box1. A particle that must search the spiral
// (world.cpp:2093-2147) returns true with its kind and cell not yet written; the
// caller's warp walks the spiral with it (warp_spiral) and finishes it.
__device__ bool part_flight(const WorldDev &w, const uint8_t *s_type, int i) {
    uint8_t bits = w.p.bits[i];
    int32_t life = w.p.life[i];
    float x = w.p.x[i], y = w.p.y[i], vx = w.p.vx[i], vy = w.p.vy[i];
    const int W = w.W, H = w.H;
    uint8_t kind = PS_ALIVE;
    int cell = -1;
    bool spiral = false;
    Box bx = {W, H, -1, -1};
    if ((bits & 2) && life <= 0) {  // :2033-2037
        kind = PS_DESTROY;
    } else {
        const float tf = w.p.tf[i];
        if (tf != 0.f) {  // :2039-2051
            const float tdx = __fsub_rn(w.p.tx[i], x), tdy = __fsub_rn(w.p.ty[i], y);
            const float nf = __fsqrt_rn(__fadd_rn(__fmul_rn(tdx, tdx), __fmul_rn(tdy, tdy)));
            vx = __fadd_rn(vx, __fmul_rn(__fdiv_rn(tdx, nf), tf));
            vy = __fadd_rn(vy, __fmul_rn(__fdiv_rn(tdy, nf), tf));
            if (nf < 100.f) {
                vx = __fmul_rn(vx, 0.95f);
                vy = __fmul_rn(vy, 0.95f);
            }
        }
        const int lx = (int)x, ly = (int)y;
        if (out_of_world(x, y, W, H)) {  // :2056-2059
            kind = PS_EXIT;
        } else if (lx < w.zx || ly < w.zy || lx >= w.zx + w.zw || ly >= w.zy + w.zh) {
            // :2061, outside the tick zone: kept as it is (steered velocity included),
            // having read no cell
        } else {
            bx.add(lx, ly);
            vx = __fadd_rn(vx, w.p.ax[i]);  // :2063-2064
            vy = __fadd_rn(vy, w.p.ay[i]);
            const int div = (int)__fadd_rn(__fadd_rn(fabsf(vx), fabsf(vy)), 1.0f);
            const float dvx = __fdiv_rn(vx, (float)div), dvy = __fdiv_rn(vy, (float)div);
            int hit = 0;  // 1: deposit at the previous cell, 2: spiral search
            for (int s = 0; s < div; s++) {  // :2071-2184
                x = __fadd_rn(x, dvx);
                y = __fadd_rn(y, dvy);
                if (out_of_world(x, y, W, H)) {
                    kind = PS_EXIT;
                    break;
                }
                bx.add((int)x, (int)y);
                const int ct = s_type[view_id(w, s_type, (int)y * W + (int)x, i)];
                if (!(bits & 1) && ct != T_AIR) {
                    const bool isObject = ct == T_OBJECT;
                    int ps = (bits >> 2) & 3;
                    if (ps == 0)
                        ps = isObject ? 1 : 2;
                    else if (ps == 1 && !isObject)
                        ps = 2;
                    bits = (uint8_t)((bits & ~0x0Cu) | ((unsigned)ps << 2));
                    if (!isObject || ps == 2) {
                        if (bits & 2)
                            kind = PS_DESTROY;
                        else
                            hit = (s_type[view_id(w, s_type, ly * W + lx, i)] != T_AIR) ? 2 : 1;
                        break;
                    }
                }
            }
            if (kind == PS_ALIVE && hit == 0 && life > 0) life--;  // :2186-2188
            if (hit == 1) {  // :2148-2152
                kind = PS_FILL;
                cell = ly * W + lx;
            } else if (hit == 2) {
                spiral = true;
            }
        }
    }
    w.q.x[i] = x;
    w.q.y[i] = y;
    w.q.vx[i] = vx;
    w.q.vy[i] = vy;
    w.q.bits[i] = bits;
    w.q.life[i] = life;
    if (!spiral) {
        w.p_state[i] = kind;
        w.p_cell[i] = cell;
    }
    const int x0 = min(max(bx.x0, 0), W - 1), y0 = min(max(bx.y0, 0), H - 1);
    const int x1 = min(max(bx.x1, 0), W - 1), y1 = min(max(bx.y1, 0), H - 1);
    w.p_box0[i] = bx.x1 < 0 ? -1 : (int32_t)((uint32_t)x0 | ((uint32_t)y0 << 16));
    w.p_box1[i] = (int32_t)((uint32_t)x1 | ((uint32_t)y1 << 16));
    return spiral;
}

// :2093-2147, the 32x32 spiral from the collision point (x, y) of particle i of world
// w, walked by the whole warp, 32 cells a step: the first cell that is AIR or holds
// the same liquid, in the particle's view. A window (the 33x33 cells the walk reaches)
// whose 8x8 blocks held no AIR when the update began holds none now (deposits only
// take AIR), so unless the particle is a liquid that may merge the walk can only fail
// and is skipped. Every lane returns the result: kind PS_FILL / PS_MERGE with *cell,
// or PS_FAIL; *ring = the ring of the last cell looked at (-1: no walk).
__device__ uint8_t warp_spiral(const WorldDev &w, const uint8_t *s_type, int i, float x, float y, int *cell,
                               int *ring) {
    const int lane = threadIdx.x & 31;
    const int W = w.W, H = w.H;
    const int pid = w.p.id[i];
    const bool psoup = s_type[pid] == T_SOUP;
    bool walk = true;
    if (!psoup && x > -32.0f && x < (float)W + 32.0f && y > -32.0f && y < (float)H + 32.0f) {
        const int ix = (int)floorf(x), iy = (int)floorf(y);
        const int bx0 = max(0, (ix - 17) >> 3), bx1 = min(w.amw - 1, (ix + 17) >> 3);
        const int by0 = max(0, (iy - 17) >> 3), by1 = min(w.amh - 1, (iy + 17) >> 3);
        const int nbx = bx1 - bx0 + 1, nblk = nbx * (by1 - by0 + 1);
        bool any = false;
        for (int k = lane; k < nblk; k += 32) any |= w.airmap[(by0 + k / nbx) * w.amw + bx0 + k % nbx] != 0;
        walk = __any_sync(0xffffffffu, any);
    }
    *ring = -1;
    *cell = -1;
    if (!walk) return PS_FAIL;
    const int n = c_spiral_n;
    for (int base = 0; base < n; base += 32) {
        const int j = base + lane;
        int hit = 0, c = -1;
        if (j < n) {
            const int cx = (int)__fadd_rn(x, (float)c_spiral[j][0]);
            const int cy = (int)__fadd_rn(y, (float)c_spiral[j][1]);
            if (cx >= 0 && cy >= 0 && cx < W && cy < H) {
                c = cy * W + cx;
                const int cid = view_id(w, s_type, c, i);
                hit = s_type[cid] == T_AIR ? 1 : ((psoup && cid == pid) ? 2 : 0);
            }
        }
        const unsigned m = __ballot_sync(0xffffffffu, hit != 0);
        if (m) {
            const int src = __ffs(m) - 1;
            *cell = __shfl_sync(0xffffffffu, c, src);
            const int h = __shfl_sync(0xffffffffu, hit, src);
            const int jl = base + src;
            *ring = max(abs((int)c_spiral[jl][0]), abs((int)c_spiral[jl][1]));
            return h == 1 ? PS_FILL : PS_MERGE;
        }
    }
    *ring = max(abs((int)c_spiral[n - 1][0]), abs((int)c_spiral[n - 1][1]));
    return PS_FAIL;
}

// the fill a particle's outcome makes (-1: none)
__device__ __forceinline__ int fill_of(const WorldDev &w, int i) {
    return w.p_state[i] == PS_FILL ? w.p_cell[i] : -1;
}

// Grid-wide barrier of the cooperative update. The spin is bounded: if it ever
// gives up it records ERR_TIMEOUT and lets the block continue, so a wait can never
// hang the device.
struct GridBar {
    unsigned count;
    unsigned gen;
};

__device__ __forceinline__ void grid_sync(GridBar *gb, unsigned nblocks, int32_t *err) {
    __syncthreads();
    if (threadIdx.x == 0) {
        volatile unsigned *vgen = &gb->gen;
        const unsigned g = *vgen;
        __threadfence();
        if (atomicAdd(&gb->count, 1u) + 1u == nblocks) {
            gb->count = 0u;
            __threadfence();
            atomicAdd(&gb->gen, 1u);
        } else {
            long long spins = 0;
            while (*vgen == g) {
                if (++spins > (1LL << 25)) {
                    atomicOr(err, ERR_TIMEOUT);
                    break;
                }
                __nanosleep(100);
            }
        }
        __threadfence();
    }
    __syncthreads();
}

constexpr int SERIAL_MAX_ITER = 1 << 16;
constexpr int SERIAL_MAX_WORLDS = 4096;  // worlds of one launch (a batch holds at most 4095)
constexpr int SERIAL_THREADS = 1024;  // one block per SM: 152 arrivals at each grid barrier

// index g of a flattened index space: its entry in s_pref (prefix sums over the
// entries, in shared memory)
__device__ __forceinline__ int entry_of(const int *s_pref, int n, int g) {
    int lo = 0, hi = n - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (s_pref[mid] <= g)
            lo = mid;
        else
            hi = mid - 1;
    }
    return lo;
}

// exclusive scan of one value per thread over the block (SERIAL_THREADS threads)
__device__ __forceinline__ int block_excl_sum(int v, int *s_warp, int *total) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    int inc = v;
    for (int o = 1; o < 32; o <<= 1) {
        const int t = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += t;
    }
    if (lane == 31) s_warp[wid] = inc;
    __syncthreads();
    if (wid == 0) {
        int x = lane < SERIAL_THREADS / 32 ? s_warp[lane] : 0;
        for (int o = 1; o < 32; o <<= 1) {
            const int t = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += t;
        }
        if (lane < SERIAL_THREADS / 32) s_warp[lane] = x;
    }
    __syncthreads();
    const int ex = (wid > 0 ? s_warp[wid - 1] : 0) + inc - v;
    *total = s_warp[SERIAL_THREADS / 32 - 1];
    __syncthreads();
    return ex;
}

// The worlds with a non-zero count(k), as a flattened index space in shared memory:
// s_ids[j] the j-th such world, s_apref[j] the index its entries start at,
// s_apref[n_act] the total. Every thread of the block calls it; returns n_act.
template <class F>
__device__ int active_worlds(int n_worlds, F count, int *s_ids, int *s_apref, int *s_warp) {
    const int seg = (n_worlds + SERIAL_THREADS - 1) / SERIAL_THREADS;
    const int k0 = min((int)threadIdx.x * seg, n_worlds), k1 = min(k0 + seg, n_worlds);
    int sum = 0, nact = 0;
    for (int k = k0; k < k1; k++) {
        const int c = count(k);
        sum += c;
        nact += c > 0;
    }
    int tot_sum, tot_act;
    int at = block_excl_sum(sum, s_warp, &tot_sum);
    int j = block_excl_sum(nact, s_warp, &tot_act);
    for (int k = k0; k < k1; k++) {
        const int c = count(k);
        if (c > 0) {
            s_ids[j] = k;
            s_apref[j] = at;
            j++;
            at += c;
        }
    }
    if (threadIdx.x == 0) s_apref[tot_act] = tot_sum;
    __syncthreads();
    return tot_act;
}

// The fixed-point iteration and the commit for every world of the table, in one
// cooperative launch (every block resident, so the grid barrier is safe). Change
// marks are per 8x8 block the lowest index whose fill moved into or out of the
// block: a particle is computed again only if a lower index changed a fill near
// what it read. Iteration work is restricted to the worlds that need it: a world
// whose fills did not change in an iteration has converged (its particles read
// only its own cells), so later iterations skip its particles, and the fills that
// changed are listed per world (chg_n[parity] of them, their indices in the first
// part_cap entries of merge_list, free until the commit) so that clearing their
// records does not scan the particles. req_count[0..1] of world 0 count every
// world's fill changes of even and odd iterations; stats[0] of world 0 receives
// the number of iterations. Dynamic shared memory: 3 * n_worlds + 2 ints.
__global__ void __launch_bounds__(SERIAL_THREADS) k_part_serial(const WorldDev *__restrict__ worlds, int n_worlds,
                                                                 const MatTable *__restrict__ mt) {
    __shared__ uint8_t s_type[MAXMAT];
    __shared__ int s_warp[SERIAL_THREADS / 32];
    extern __shared__ int s_dyn[];
    int *s_pref = s_dyn;                       // [n_worlds + 1] particles before world k
    int *s_apref = s_dyn + n_worlds + 1;       // [n_worlds + 1] the active index space
    int *s_ids = s_dyn + 2 * (n_worlds + 1);   // [n_worlds]
    load_types(s_type, mt);
    for (int k = threadIdx.x; k < n_worlds; k += blockDim.x) s_pref[k + 1] = *worlds[k].part_count;
    __syncthreads();
    if (threadIdx.x == 0) {
        s_pref[0] = 0;
        for (int k = 0; k < n_worlds; k++) s_pref[k + 1] += s_pref[k];
    }
    __syncthreads();
    const int total = s_pref[n_worlds];
    auto parts = [&](int k) { return s_pref[k + 1] - s_pref[k]; };
    GridBar *gb = (GridBar *)worlds[0].bar;
    const unsigned nb = gridDim.x;
    int32_t *err = worlds[0].err;
    int32_t *cnt = worlds[0].req_count;
    const int gtid = (int)(blockIdx.x * blockDim.x + threadIdx.x), gstride = (int)(gridDim.x * blockDim.x);
    const int lane = threadIdx.x & 31;
    int it = 0;
    for (;; it++) {
        if (it >= SERIAL_MAX_ITER) {
            if (gtid == 0) atomicOr(err, ERR_TIMEOUT);
            break;
        }
        const int par = it & 1;
        // A: outcomes of the particles whose box saw a fill change by a lower index (all
        // at first; later only in worlds whose fills changed in the last iteration);
        // changed fills are counted, listed and their blocks marked for the next
        // iteration with the changing index. A thread takes particle g, its warp walks
        // the spirals of the warp's particles together.
        // After the first iteration only particles above the lowest index whose fill
        // changed in the last iteration can see a change (a particle is computed again
        // only for a change by a lower index), so each world's space starts there.
        const int n_act = it == 0 ? active_worlds(n_worlds, parts, s_ids, s_apref, s_warp)
                                  : active_worlds(
                                        n_worlds,
                                        [&](int k) {
                                            const int32_t *cn = worlds[k].chg_n;
                                            return __ldcg(&cn[1 - par]) > 0
                                                       ? max(0, parts(k) - 1 - __ldcg(&cn[2 + par]))
                                                       : 0;
                                        },
                                        s_ids, s_apref, s_warp);
        const int total_a = s_apref[n_act];
        for (int gb0 = gtid - lane; gb0 < total_a; gb0 += gstride) {
            const int g = gb0 + lane;
            bool work = g < total_a, spiral = false;
            int wi = 0, i = 0, before = -1;
            if (work) {
                const int j = entry_of(s_apref, n_act, g);
                wi = s_ids[j];
                i = g - s_apref[j];
                const WorldDev &w = worlds[wi];
                if (it > 0) {
                    i += __ldcg(&w.chg_n[2 + par]) + 1;
                    const int32_t b0 = w.p_box0[i];
                    if (b0 < 0) {
                        work = false;  // read no cell: nothing can change it
                    } else {
                        const int nblk = w.amw * w.amh;
                        const uint32_t *seen = w.chg + (size_t)par * nblk;
                        const int32_t b1 = w.p_box1[i];
                        const int x0 = (b0 & 0xFFFF) >> 3, y0 = ((uint32_t)b0 >> 16) >> 3;
                        const int x1 = (b1 & 0xFFFF) >> 3, y1 = ((uint32_t)b1 >> 16) >> 3;
                        // the lowest changing index over the box's blocks (the loads do not
                        // wait on each other)
                        uint32_t lo = 0xFFFFFFFFu;
                        for (int by = y0; by <= y1; by++)
                            for (int bxx = x0; bxx <= x1; bxx++) lo = min(lo, __ldcg(&seen[by * w.amw + bxx]));
                        if (lo >= (uint32_t)i)
                            work = false;
                        else
                            before = fill_of(w, i);
                    }
                }
                if (work) spiral = part_flight(w, s_type, i);
            }
            // the spirals of this warp's particles, one after another, 32 cells a step
            unsigned pend = __ballot_sync(0xffffffffu, spiral);
            while (pend) {
                const int src = __ffs(pend) - 1;
                pend &= pend - 1;
                const int swi = __shfl_sync(0xffffffffu, wi, src), si = __shfl_sync(0xffffffffu, i, src);
                const WorldDev &sw = worlds[swi];
                float sx = 0.f, sy = 0.f;
                if (lane == src) {
                    sx = sw.q.x[si];
                    sy = sw.q.y[si];
                }
                sx = __shfl_sync(0xffffffffu, sx, src);
                sy = __shfl_sync(0xffffffffu, sy, src);
                int cell, ring;
                const uint8_t k = warp_spiral(sw, s_type, si, sx, sy, &cell, &ring);
                if (lane == src) {
                    sw.p_state[si] = k;
                    sw.p_cell[si] = cell;
                    if (k == PS_FAIL) {  // :2141-2144
                        sw.q.vy[si] = -4.0f;
                        sw.q.y[si] = __fsub_rn(sy, 16.0f);
                    }
                    if (ring >= 0) {
                        // the cells looked at lie in the square of the last one's ring
                        const int r = ring + 1;
                        const int32_t b0 = sw.p_box0[si], b1 = sw.p_box1[si];
                        const int ix = (int)floorf(sx), iy = (int)floorf(sy);
                        const int x0 = min(max(min((int)(b0 & 0xFFFF), ix - r), 0), sw.W - 1);
                        const int y0 = min(max(min((int)((uint32_t)b0 >> 16), iy - r), 0), sw.H - 1);
                        const int x1 = min(max(max((int)(b1 & 0xFFFF), ix + r), 0), sw.W - 1);
                        const int y1 = min(max(max((int)((uint32_t)b1 >> 16), iy + r), 0), sw.H - 1);
                        sw.p_box0[si] = (int32_t)((uint32_t)x0 | ((uint32_t)y0 << 16));
                        sw.p_box1[si] = (int32_t)((uint32_t)x1 | ((uint32_t)y1 << 16));
                    }
                }
            }
            if (work) {
                const WorldDev &w = worlds[wi];
                const int after = fill_of(w, i);
                if (after != before) {
                    const int nblk = w.amw * w.amh;
                    uint32_t *mark = w.chg + (size_t)(1 - par) * nblk;
                    atomicAdd(&cnt[par], 1);
                    w.merge_list[atomicAdd(&w.chg_n[par], 1)] = i;  // at most once per particle
                    atomicMin(&w.chg_n[3 - par], i);
                    if (before >= 0)
                        atomicMin(&mark[(before / w.W >> 3) * w.amw + ((before % w.W) >> 3)], (uint32_t)i);
                    if (after >= 0) atomicMin(&mark[(after / w.W >> 3) * w.amw + ((after % w.W) >> 3)], (uint32_t)i);
                    w.p_prev[i] = before;  // the cell whose record B1 clears
                }
            }
        }
        grid_sync(gb, nb, err);
        const int changed = __ldcg(&cnt[par]);
        if (changed == 0) break;
        // B1: clear the records of the fills that moved away (the listed particles of
        // this iteration), and the marks A read (set by the last iteration's changes)
        {
            const int na = active_worlds(
                n_worlds, [&](int k) { return __ldcg(&worlds[k].chg_n[par]); }, s_ids, s_apref, s_warp);
            for (int g = gtid; g < s_apref[na]; g += gstride) {
                const int j = entry_of(s_apref, na, g);
                const WorldDev &w = worlds[s_ids[j]];
                const int i = w.merge_list[g - s_apref[j]];
                const int c = w.p_prev[i];
                if (c >= 0) w.df[c] = 0;
            }
        }
        if (it > 0) {
            const int nm = active_worlds(
                n_worlds,
                [&](int k) {
                    const WorldDev &w = worlds[k];
                    return __ldcg(&w.chg_n[1 - par]) > 0 ? w.amw * w.amh : 0;
                },
                s_ids, s_apref, s_warp);
            for (int g = gtid; g < s_apref[nm]; g += gstride) {
                const int j = entry_of(s_apref, nm, g);
                const WorldDev &w = worlds[s_ids[j]];
                w.chg[(size_t)par * w.amw * w.amh + (g - s_apref[j])] = 0xFFFFFFFFu;
            }
        }
        if (gtid == 0) cnt[1 - par] = 0;
        grid_sync(gb, nb, err);
        // B2: every current fill of the worlds that changed records itself; the lowest
        // index stays. The last iteration's counts have been used: cleared for the next.
        {
            const int na = active_worlds(
                n_worlds, [&](int k) { return __ldcg(&worlds[k].chg_n[par]) > 0 ? parts(k) : 0; }, s_ids,
                s_apref, s_warp);
            for (int g = gtid; g < s_apref[na]; g += gstride) {
                const int j = entry_of(s_apref, na, g);
                const WorldDev &w = worlds[s_ids[j]];
                const int i = g - s_apref[j];
                const int c = fill_of(w, i);
                // records only grow, so one already at or above this fill's code stays
                // there: only the cells cleared in B1 take atomics
                if (c >= 0 && __ldcg(&w.df[c]) < fill_code(i)) atomicMax(&w.df[c], fill_code(i));
            }
            for (int k = gtid; k < n_worlds; k += gstride) {
                worlds[k].chg_n[1 - par] = 0;
                worlds[k].chg_n[2 + par] = 0x7FFFFFFF;  // read by this iteration's A
            }
        }
        grid_sync(gb, nb, err);
    }
    // the sequential outcome: commit it
    for (int g = gtid; g < total; g += gstride) {
        const int wi = entry_of(s_pref, n_worlds, g);
        const WorldDev &w = worlds[wi];
        const int i = g - s_pref[wi];
        const uint8_t k = w.p_state[i];
        const int c = w.p_cell[i];
        if (k == PS_EXIT || k == PS_DESTROY) {
            led_part(w, mt, k == PS_EXIT ? LED_XN : LED_DN, k == PS_EXIT ? LED_XF : LED_DF, w.p.id[i], w.p.sc[i]);
            w.p_state[i] = PS_DEAD;
        } else if (k == PS_FILL) {  // :2115-2118, :2148-2152
            w.id[c] = w.p.id[i];
            w.col[c] = w.p.col[i];
            w.sc[c] = w.p.sc[i];
            w.fl[c] = w.p.fl[i];
            w.df[c] = 0;
            // the target was AIR, whose temperature word means nothing: the particle's
            // (a SOUP tile's temperature; 0 for the others) is stored without a type test
            if (w.tp) w.tp[c] = w.p.tp[i];
            if (w.dirty) w.dirty[c] = 1;
            w.p_state[i] = PS_DEAD;
        } else if (k == PS_MERGE) {  // :2119-2125, added by k_merge in particle order
            w.p_box0[i] = c;
            w.merge_list[atomicAdd(w.merge_count, 1)] = i;
            if (w.dirty) w.dirty[c] = 1;
            atomicAdd((unsigned long long *)&w.ledger[LED_DN * MAXMAT + w.p.id[i]], 1ull);
            w.p_state[i] = PS_DEAD;
        } else {  // PS_ALIVE, PS_FAIL: the particle lives on
            w.p.x[i] = w.q.x[i];
            w.p.y[i] = w.q.y[i];
            w.p.vx[i] = w.q.vx[i];
            w.p.vy[i] = w.q.vy[i];
            w.p.bits[i] = w.q.bits[i];
            w.p.life[i] = w.q.life[i];
            w.p_state[i] = PS_ALIVE;
        }
    }
    // the marks A of the last iteration read (set by the changes of the one before)
    // are cleared for the next update; the last iteration changed nothing, so it
    // set none. The per-world counts are cleared by k_part_end.
    if (it > 0 && it < SERIAL_MAX_ITER) {
        const int par = it & 1;
        const int nm = active_worlds(
            n_worlds,
            [&](int k) {
                const WorldDev &w = worlds[k];
                return __ldcg(&w.chg_n[1 - par]) > 0 ? w.amw * w.amh : 0;
            },
            s_ids, s_apref, s_warp);
        for (int g = gtid; g < s_apref[nm]; g += gstride) {
            const int j = entry_of(s_apref, nm, g);
            const WorldDev &w = worlds[s_ids[j]];
            w.chg[(size_t)par * w.amw * w.amh + (g - s_apref[j])] = 0xFFFFFFFFu;
        }
    }
    if (gtid == 0) {
        cnt[0] = 0;
        cnt[1] = 0;
        worlds[0].stats[0] = it + 1;
    }
}

// The deposits into liquid of this particle update: Q16.16 amounts are added at once;
// f32 amounts (tile.fluidAmount += particle amount, world.cpp:2123, the reference's
// float add) cell by cell in particle-index order, after any fill of the cell (a
// fill comes from a lower index). One block per world: each round every cell takes
// its lowest-index pending deposit, so a cell with k deposits is done after k rounds.
__global__ void k_merge(const WorldDev *__restrict__ worlds) {
    const WorldDev &w = worlds[blockIdx.x];
    __shared__ int s_open, s_next;
    const int n0 = *w.merge_count;
    if (n0 == 0) return;
    if (!w.f32) {
        for (int j = threadIdx.x; j < n0; j += blockDim.x) {
            const int i = w.merge_list[j];
            atomicAdd(&w.sc[w.p_box0[i]], w.p.sc[i]);
        }
        __syncthreads();
        if (threadIdx.x == 0) *w.merge_count = 0;
        return;
    }
    // two lists of part_cap entries: the open deposits of this round, the next's
    int32_t *cur = w.merge_list, *nxt = w.merge_list + w.part_cap;
    if (threadIdx.x == 0) s_open = n0;
    __syncthreads();
    for (int round = 0; round < (1 << 24); round++) {
        const int n = s_open;
        if (n == 0) break;
        for (int j = threadIdx.x; j < n; j += blockDim.x) {
            const int i = cur[j];
            atomicMin(&w.merge_claim[w.p_box0[i]], (uint32_t)i);
        }
        if (threadIdx.x == 0) s_next = 0;
        __syncthreads();
        // the winners add (one thread per cell); the others go to the next round
        for (int j = threadIdx.x; j < n; j += blockDim.x) {
            const int i = cur[j];
            const int c = w.p_box0[i];
            if (w.merge_claim[c] == (uint32_t)i)
                w.sc[c] = __float_as_int(__fadd_rn(__int_as_float(w.sc[c]), __int_as_float(w.p.sc[i])));
            else
                nxt[atomicAdd(&s_next, 1)] = i;
        }
        __syncthreads();
        for (int j = threadIdx.x; j < n; j += blockDim.x) w.merge_claim[w.p_box0[cur[j]]] = 0xFFFFFFFFu;
        __syncthreads();
        if (threadIdx.x == 0) s_open = s_next;
        int32_t *t = cur;
        cur = nxt;
        nxt = t;
        __syncthreads();
    }
    if (threadIdx.x == 0) *w.merge_count = 0;
}

// ------------------------------------------------------------- compaction
// stable removal of dead particles (std::erase_if, world.cpp:2190) and of
// particles below the world (world.cpp:2203)
__device__ __forceinline__ bool keep(const WorldDev &w, int i) {
    return w.p_state[i] == PS_ALIVE && !(w.p.y[i] > (float)w.H);
}

// The compaction runs over one index space holding every world's particles in
// world order (world k's at s_pref[k] .. s_pref[k + 1]), cut into CMP_BLOCKS
// contiguous ranges: a batch of many small worlds costs the blocks of one world of
// the same total. g kept particles before index g of that space, G(g), give
// particle g its place in its world's list: G(g) - G(start of its world), the
// second term being the kept particles of the worlds before it.
constexpr int CMP_THREADS = SERIAL_THREADS;  // block_excl_sum's block size
constexpr int CMP_BLOCKS = 304;
static_assert(CMP_BLOCKS < ST_KEPT_BEFORE && CMP_BLOCKS <= CMP_THREADS, "compaction scratch layout");

// s_pref[k] = val(0) + ... + val(k - 1) for k = 0 .. n, in shared memory; every
// thread of the block calls it
template <class F>
__device__ __forceinline__ void block_prefix(int n, F val, int *s_pref, int *s_warp) {
    const int seg = (n + CMP_THREADS - 1) / CMP_THREADS;
    const int k0 = min((int)threadIdx.x * seg, n), k1 = min(k0 + seg, n);
    int sum = 0;
    for (int k = k0; k < k1; k++) sum += val(k);
    int tot;
    int at = block_excl_sum(sum, s_warp, &tot);
    for (int k = k0; k < k1; k++) {
        s_pref[k] = at;
        at += val(k);
    }
    if (threadIdx.x == 0) s_pref[n] = tot;
    __syncthreads();
}

// this block's range of the particle index space
__device__ __forceinline__ void cmp_range(int total, int *b0, int *b1) {
    const int seg = (total + (int)gridDim.x - 1) / (int)gridDim.x;
    *b0 = min(total, (int)blockIdx.x * seg);
    *b1 = min(total, *b0 + seg);
}

// kept particles per block (world 0's scan_tmp) and per world (ST_KEPT, cleared
// by k_air_map). Dynamic shared memory: n_worlds + 1 ints.
__global__ void __launch_bounds__(CMP_THREADS) k_cmp_count(const WorldDev *__restrict__ worlds, int n_worlds) {
    extern __shared__ int s_pref[];
    __shared__ int s_warp[CMP_THREADS / 32];
    block_prefix(n_worlds, [&](int k) { return *worlds[k].part_count; }, s_pref, s_warp);
    int b0, b1;
    cmp_range(s_pref[n_worlds], &b0, &b1);
    const int lane = threadIdx.x & 31;
    int cnt = 0;
    for (int base = b0; base < b1; base += CMP_THREADS) {
        const int g = base + (int)threadIdx.x;
        int wi = -1;
        bool v = false;
        if (g < b1) {
            wi = entry_of(s_pref, n_worlds, g);
            v = keep(worlds[wi], g - s_pref[wi]);
        }
        cnt += v ? 1 : 0;
        // one atomic per world among the warp's kept particles
        const unsigned kept = __ballot_sync(0xffffffffu, v);
        const unsigned same = __match_any_sync(0xffffffffu, wi) & kept;
        if (v && lane == __ffs(same) - 1) atomicAdd(&worlds[wi].scan_tmp[ST_KEPT], __popc(same));
    }
    int tot;
    block_excl_sum(cnt, s_warp, &tot);
    if (threadIdx.x == 0) worlds[0].scan_tmp[blockIdx.x] = tot;
}

// one block: the blocks' exclusive prefix, each world's kept particles before it
// and its new count
__global__ void __launch_bounds__(CMP_THREADS) k_cmp_scan(const WorldDev *__restrict__ worlds, int n_worlds,
                                                          int nblocks) {
    __shared__ int s_warp[CMP_THREADS / 32];
    int32_t *blk = worlds[0].scan_tmp;
    const int v = (int)threadIdx.x < nblocks ? blk[threadIdx.x] : 0;
    int tot;
    const int ex = block_excl_sum(v, s_warp, &tot);
    if ((int)threadIdx.x < nblocks) blk[threadIdx.x] = ex;
    const int seg = (n_worlds + CMP_THREADS - 1) / CMP_THREADS;
    const int k0 = min((int)threadIdx.x * seg, n_worlds), k1 = min(k0 + seg, n_worlds);
    int sum = 0;
    for (int k = k0; k < k1; k++) sum += worlds[k].scan_tmp[ST_KEPT];
    int at = block_excl_sum(sum, s_warp, &tot);
    for (int k = k0; k < k1; k++) {
        int32_t *st = worlds[k].scan_tmp;
        const int c = st[ST_KEPT];
        st[ST_KEPT_BEFORE] = at;
        st[ST_COUNT] = c;
        at += c;
    }
}

// the kept particles to their places in each world's second list (q), in order.
// Dynamic shared memory: n_worlds + 1 ints.
__global__ void __launch_bounds__(CMP_THREADS) k_cmp_scatter(const WorldDev *__restrict__ worlds, int n_worlds) {
    extern __shared__ int s_pref[];
    __shared__ int s_warp[CMP_THREADS / 32];
    block_prefix(n_worlds, [&](int k) { return *worlds[k].part_count; }, s_pref, s_warp);
    int b0, b1;
    cmp_range(s_pref[n_worlds], &b0, &b1);
    int run = worlds[0].scan_tmp[blockIdx.x];  // kept particles before the range
    for (int base = b0; base < b1; base += CMP_THREADS) {
        const int g = base + (int)threadIdx.x;
        int wi = 0, i = 0;
        bool v = false;
        if (g < b1) {
            wi = entry_of(s_pref, n_worlds, g);
            i = g - s_pref[wi];
            v = keep(worlds[wi], i);
        }
        int tot;
        const int ex = block_excl_sum(v ? 1 : 0, s_warp, &tot);
        if (v) {
            const WorldDev &w = worlds[wi];
            const int o = run + ex - w.scan_tmp[ST_KEPT_BEFORE];
            w.q.x[o] = w.p.x[i];
            w.q.y[o] = w.p.y[i];
            w.q.vx[o] = w.p.vx[i];
            w.q.vy[o] = w.p.vy[i];
            w.q.ax[o] = w.p.ax[i];
            w.q.ay[o] = w.p.ay[i];
            w.q.tx[o] = w.p.tx[i];
            w.q.ty[o] = w.p.ty[i];
            w.q.tf[o] = w.p.tf[i];
            w.q.life[o] = w.p.life[i];
            w.q.fade[o] = w.p.fade[i];
            w.q.col[o] = w.p.col[i];
            w.q.sc[o] = w.p.sc[i];
            if (w.tp) w.q.tp[o] = w.p.tp[i];
            w.q.id[o] = w.p.id[i];
            w.q.fl[o] = w.p.fl[i];
            w.q.bits[o] = w.p.bits[i];
        }
        run += tot;
    }
}

// the compacted lists back to the first list (p), over the index space of the kept
// particles. Dynamic shared memory: n_worlds + 1 ints.
__global__ void __launch_bounds__(CMP_THREADS) k_cmp_copy(const WorldDev *__restrict__ worlds, int n_worlds) {
    extern __shared__ int s_pref[];
    __shared__ int s_warp[CMP_THREADS / 32];
    block_prefix(n_worlds, [&](int k) { return worlds[k].scan_tmp[ST_COUNT]; }, s_pref, s_warp);
    const int total = s_pref[n_worlds];
    for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < total; g += gridDim.x * blockDim.x) {
        const int wi = entry_of(s_pref, n_worlds, g);
        const WorldDev &w = worlds[wi];
        const int o = g - s_pref[wi];
        w.p.x[o] = w.q.x[o];
        w.p.y[o] = w.q.y[o];
        w.p.vx[o] = w.q.vx[o];
        w.p.vy[o] = w.q.vy[o];
        w.p.ax[o] = w.q.ax[o];
        w.p.ay[o] = w.q.ay[o];
        w.p.tx[o] = w.q.tx[o];
        w.p.ty[o] = w.q.ty[o];
        w.p.tf[o] = w.q.tf[o];
        w.p.life[o] = w.q.life[o];
        w.p.fade[o] = w.q.fade[o];
        w.p.col[o] = w.q.col[o];
        w.p.sc[o] = w.q.sc[o];
        if (w.tp) w.p.tp[o] = w.q.tp[o];
        w.p.id[o] = w.q.id[o];
        w.p.fl[o] = w.q.fl[o];
        w.p.bits[o] = w.q.bits[o];
    }
}

__global__ void k_part_end(const WorldDev *worlds, int nblocks) {
    const WorldDev &w = worlds[blockIdx.x];
    if (threadIdx.x == 0) {
        *w.part_count = w.scan_tmp[nblocks];
        w.req_count[0] = 0;
        w.req_count[1] = 0;
        w.req_count[2] = 0;
        w.chg_n[0] = 0;
        w.chg_n[1] = 0;
    }
}

// ---------------------------------------------------------------- launchers
static bool g_spiral_ready = false;

static void spiral_upload() {
    if (g_spiral_ready) return;
    // the spiral walk of world.cpp:2105-2133 (X = Y = 32, maxI = 1024)
    int8_t tab[1024][2];
    int X = 32, Y = 32, x = 0, y = 0, dx = 0, dy = -1;
    int t = X > Y ? X : Y;
    int maxI = t * t, n = 0;
    for (int j = 0; j < maxI; j++) {
        if ((-X / 2 <= x) && (x <= X / 2) && (-Y / 2 <= y) && (y <= Y / 2)) {
            tab[n][0] = (int8_t)x;
            tab[n][1] = (int8_t)y;
            n++;
        }
        if ((x == y) || ((x < 0) && (x == -y)) || ((x > 0) && (x == 1 - y))) {
            t = dx;
            dx = -dy;
            dy = t;
        }
        x += dx;
        y += dy;
    }
    cudaMemcpyToSymbol(c_spiral, tab, sizeof(tab));
    cudaMemcpyToSymbol(c_spiral_n, &n, sizeof(int));
    g_spiral_ready = true;
}

void particle_prepare() { spiral_upload(); }

// the per-chunk-pass spawn offsets alone (the allocation-free tick writes its own output)
cudaError_t launch_spawn_scan(WorldDev *d_worlds, int n_worlds, cudaStream_t s) {
    k_spawn_scan<<<n_worlds, 1024, 0, s>>>(d_worlds);
    return cudaGetLastError();
}

// this tick's spawns -> end of the particle list, then the tick counter
cudaError_t launch_spawn_append(WorldDev *d_worlds, int n_worlds, int stage_blocks, cudaStream_t s) {
    k_spawn_scan<<<n_worlds, 1024, 0, s>>>(d_worlds);
    dim3 g(stage_blocks, n_worlds);
    k_spawn_scatter<<<g, 256, 0, s>>>(d_worlds);
    k_tick_end<<<n_worlds, 32, 0, s>>>(d_worlds);
    return cudaGetLastError();
}

cudaError_t launch_particle_tick(WorldDev *d_worlds, int n_worlds, const MatTable *mt, int move_blocks,
                                 cudaStream_t s) {
    spiral_upload();
    dim3 gm(move_blocks, n_worlds);
    k_air_map<<<gm, 256, 0, s>>>(d_worlds, mt);
    {
        // every block of a cooperative launch is resident, so the grid barrier is safe;
        // the blocks per SM depend on the shared memory the table's size asks for
        if (n_worlds > SERIAL_MAX_WORLDS) return cudaErrorInvalidValue;
        const size_t dyn = (size_t)(3 * n_worlds + 2) * sizeof(int);
        static size_t dyn_set = 0;
        if (dyn > 48 * 1024 && dyn > dyn_set) {
            cudaFuncSetAttribute(k_part_serial, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn);
            dyn_set = dyn;
        }
        static int nsm = 0;
        if (!nsm) {
            int dev = 0;
            cudaGetDevice(&dev);
            cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
        }
        int per_sm = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_part_serial, SERIAL_THREADS, dyn);
        const int coop_blocks = std::max(1, std::min(per_sm, 4) * nsm);
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(coop_blocks);
        cfg.blockDim = dim3(SERIAL_THREADS);
        cfg.dynamicSmemBytes = dyn;
        cfg.stream = s;
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeCooperative;
        attr[0].val.cooperative = 1;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
        cudaLaunchKernelEx(&cfg, k_part_serial, (const WorldDev *)d_worlds, n_worlds, mt);
    }
    k_merge<<<n_worlds, 1024, 0, s>>>(d_worlds);
    const size_t pref = (size_t)(n_worlds + 1) * sizeof(int);
    k_cmp_count<<<CMP_BLOCKS, CMP_THREADS, pref, s>>>(d_worlds, n_worlds);
    k_cmp_scan<<<1, CMP_THREADS, 0, s>>>(d_worlds, n_worlds, CMP_BLOCKS);
    k_cmp_scatter<<<CMP_BLOCKS, CMP_THREADS, pref, s>>>(d_worlds, n_worlds);
    k_cmp_copy<<<CMP_BLOCKS, CMP_THREADS, pref, s>>>(d_worlds, n_worlds);
    k_part_end<<<n_worlds, 32, 0, s>>>(d_worlds, PART_BLOCKS);
    return cudaGetLastError();
}

int particle_scan_blocks() { return PART_BLOCKS; }

}  // namespace fse
