// fse_particles.cu -- free particles: the ordered append of particles spawned by
// the cell tick (world.cpp:1078,1110-1119,1222,1298,1901-1913) and the particle
// update world::tickCells() (world.cpp:2030-2195).
//
// Every kernel takes the world table and handles world blockIdx.y, so one launch
// serves a single world or a whole batch. Arithmetic on particle state uses the
// explicitly rounded intrinsics (__fadd_rn, __fmul_rn, __fdiv_rn, __fsqrt_rn) so
// that no multiply-add is contracted: the FP32 results equal a strict IEEE CPU
// evaluation of the same expressions bit for bit.
#include <algorithm>

#include "fse_internal.cuh"

namespace fse {

constexpr int PART_BLOCKS = 512;  // blocks per world for the particle list kernels (<= k_cmp_scan threads)
constexpr int PART_THREADS = 256;

// p_state values
enum : uint8_t { PS_ALIVE = 0, PS_DEAD = 1, PS_DIRECT = 2, PS_SPIRAL = 3 };

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

// world.cpp:2032-2188 for every particle against the grid left by the cell tick;
// collisions become deposit requests resolved by the kernels below.
__device__ __forceinline__ void load_types(uint8_t *s_type, const MatTable *mt);

__global__ void k_part_move(const WorldDev *__restrict__ worlds, const MatTable *__restrict__ mt) {
    __shared__ uint8_t s_type[MAXMAT];
    load_types(s_type, mt);
    const WorldDev &w = worlds[blockIdx.y];
    const int n = *w.part_count;
    const int W = w.W, H = w.H;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        uint8_t bits = w.p.bits[i];
        int32_t life = w.p.life[i];
        if ((bits & 2) && life <= 0) {  // :2033-2037
            w.p_state[i] = PS_DEAD;
            led_part(w, mt, LED_DN, LED_DF, w.p.id[i], w.p.sc[i]);
            continue;
        }
        float x = w.p.x[i], y = w.p.y[i], vx = w.p.vx[i], vy = w.p.vy[i];
        float tf = w.p.tf[i];
        if (tf != 0.f) {  // :2039-2051
            float tdx = __fsub_rn(w.p.tx[i], x), tdy = __fsub_rn(w.p.ty[i], y);
            float nf = __fsqrt_rn(__fadd_rn(__fmul_rn(tdx, tdx), __fmul_rn(tdy, tdy)));
            vx = __fadd_rn(vx, __fmul_rn(__fdiv_rn(tdx, nf), tf));
            vy = __fadd_rn(vy, __fmul_rn(__fdiv_rn(tdy, nf), tf));
            if (nf < 100.f) {
                vx = __fmul_rn(vx, 0.95f);
                vy = __fmul_rn(vy, 0.95f);
            }
        }
        uint8_t st = PS_ALIVE;
        if (out_of_world(x, y, W, H)) {  // :2056-2059
            w.p_state[i] = PS_DEAD;
            w.p.vx[i] = vx;
            w.p.vy[i] = vy;
            led_part(w, mt, LED_XN, LED_XF, w.p.id[i], w.p.sc[i]);
            continue;
        }
        const int lx = (int)x, ly = (int)y;
        vx = __fadd_rn(vx, w.p.ax[i]);  // :2063-2064
        vy = __fadd_rn(vy, w.p.ay[i]);
        const int div = (int)__fadd_rn(__fadd_rn(fabsf(vx), fabsf(vy)), 1.0f);
        const float dvx = __fdiv_rn(vx, (float)div), dvy = __fdiv_rn(vy, (float)div);
        bool done = false;
        for (int s = 0; s < div && !done; s++) {  // :2071-2184
            x = __fadd_rn(x, dvx);
            y = __fadd_rn(y, dvy);
            if (out_of_world(x, y, W, H)) {
                st = PS_DEAD;
                led_part(w, mt, LED_XN, LED_XF, w.p.id[i], w.p.sc[i]);
                done = true;
                break;
            }
            int ct = s_type[w.id[(size_t)(int)y * W + (int)x]];
            if (!(bits & 1) && ct != T_AIR) {
                bool isObject = ct == T_OBJECT;
                int ps = (bits >> 2) & 3;
                if (ps == 0)
                    ps = isObject ? 1 : 2;
                else if (ps == 1 && !isObject)
                    ps = 2;
                bits = (uint8_t)((bits & ~0x0Cu) | ((unsigned)ps << 2));
                if (!isObject || ps == 2) {
                    if (bits & 2) {
                        st = PS_DEAD;
                        led_part(w, mt, LED_DN, LED_DF, w.p.id[i], w.p.sc[i]);
                    } else {
                        st = (s_type[w.id[(size_t)ly * W + lx]] != T_AIR) ? PS_SPIRAL : PS_DIRECT;
                    }
                    done = true;
                }
            }
        }
        if (!done && life > 0) life--;  // :2186-2188
        w.p.x[i] = x;
        w.p.y[i] = y;
        w.p.vx[i] = vx;
        w.p.vy[i] = vy;
        w.p.bits[i] = bits;
        w.p.life[i] = life;
        w.p_state[i] = st;
        if (st == PS_DIRECT || st == PS_SPIRAL) {
            w.p_lxly[i] = ly * W + lx;
            int j = atomicAdd(&w.req_count[0], 1);
            w.req_list[j] = i;
        }
    }
}

// ------------------------------------------------------------- deposits
// Target of a deposit against the current grid (world.cpp:2093-2147): the cell
// index, with bit 31 set for a merge into the same liquid; -1 if none.
// s_type: physics type per material (shared memory).
//
// A particle whose search window (the 33x33 cells the spiral walk can reach) holds
// no AIR can only fail, unless it is a liquid that may merge. The airmap records,
// per 8x8 block, whether the block held AIR when this particle tick began; deposits
// only remove AIR, so a window whose blocks are all AIR-free now is AIR-free too and
// the walk is skipped. The result is the walk's result either way.
__device__ __forceinline__ int dep_target(const WorldDev &w, const uint8_t *s_type, int i, uint8_t st) {
    const int W = w.W, H = w.H;
    if (st == PS_DIRECT) {
        int c = w.p_lxly[i];
        if (s_type[w.id[c]] == T_AIR) return c;
    }
    const float x = w.p.x[i], y = w.p.y[i];
    const int pid = w.p.id[i];
    const bool psoup = s_type[pid] == T_SOUP;
    if (!psoup && x > -32.0f && x < (float)W + 32.0f && y > -32.0f && y < (float)H + 32.0f) {
        // window [x-17, x+17] x [y-17, y+17] covers every (int)(x + ofs), |ofs| <= 16;
        // positions far outside the world (or NaN) take the walk unfiltered
        const int ix = (int)floorf(x), iy = (int)floorf(y);
        const int bx0 = max(0, (ix - 17) >> 3), bx1 = min(w.amw - 1, (ix + 17) >> 3);
        const int by0 = max(0, (iy - 17) >> 3), by1 = min(w.amh - 1, (iy + 17) >> 3);
        bool any = false;
        for (int by = by0; by <= by1 && !any; by++)
            for (int bx = bx0; bx <= bx1; bx++)
                if (w.airmap[by * w.amw + bx]) {
                    any = true;
                    break;
                }
        if (!any) return -1;
    }
    const int n = c_spiral_n;
    for (int j = 0; j < n; j++) {
        int cx = (int)__fadd_rn(x, (float)c_spiral[j][0]);
        int cy = (int)__fadd_rn(y, (float)c_spiral[j][1]);
        if (cx < 0 || cy < 0 || cx >= W || cy >= H) continue;
        int c = cy * W + cx;
        int cid = w.id[c];
        if (s_type[cid] == T_AIR) return c;
        if (psoup && cid == pid) return c | (int)0x80000000u;
    }
    return -1;
}

// which 8x8 blocks hold AIR, from the grid the cell tick left (one thread per block)
__global__ void k_air_map(const WorldDev *__restrict__ worlds, const MatTable *__restrict__ mt) {
    __shared__ uint8_t s_type[MAXMAT];
    load_types(s_type, mt);
    const WorldDev &w = worlds[blockIdx.y];
    const int nb = w.amw * w.amh;
    for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < nb; b += gridDim.x * blockDim.x) {
        const int bx = b % w.amw, by = b / w.amw;
        const int x0 = bx * 8, y0 = by * 8, x1 = min(x0 + 8, w.W), y1 = min(y0 + 8, w.H);
        uint8_t any = 0;
        for (int y = y0; y < y1 && !any; y++)
            for (int x = x0; x < x1; x++)
                if (s_type[w.id[(size_t)y * w.W + x]] == T_AIR) {
                    any = 1;
                    break;
                }
        w.airmap[b] = any;
    }
}

__device__ __forceinline__ void load_types(uint8_t *s_type, const MatTable *mt) {
    for (int k = threadIdx.x; k < MAXMAT; k += blockDim.x) s_type[k] = (uint8_t)(k < mt->n ? mt_type(mt->a[k]) : 0);
    __syncthreads();
}

__device__ __forceinline__ void dep_fail(const WorldDev &w, int i) {
    // :2141-2144
    w.p.vy[i] = -4.0f;
    w.p.y[i] = __fsub_rn(w.p.y[i], 16.0f);
    w.p_state[i] = PS_ALIVE;
}
__device__ __forceinline__ void dep_merge(const WorldDev &w, const MatTable *mt, int i, int c) {
    // :2119-2125
    if (w.f32) {
        // f32 amounts: added after the rounds, cell by cell in particle-index order
        // (k_merge_f32), as the reference's list order adds them
        w.p_lxly[i] = c;
        w.merge_list[atomicAdd(w.merge_count, 1)] = i;
    } else {
        atomicAdd(&w.sc[c], w.p.sc[i]);
    }
    if (w.dirty) w.dirty[c] = 1;
    w.p_state[i] = PS_DEAD;
    atomicAdd((unsigned long long *)&w.ledger[LED_DN * MAXMAT + w.p.id[i]], 1ull);
}
__device__ __forceinline__ void dep_fill(const WorldDev &w, int i, int c) {
    // :2115-2118, :2148-2152; the cell's diff word still holds the claim and is
    // cleared by k_dep_clear
    w.id[c] = w.p.id[i];
    w.col[c] = w.p.col[i];
    w.sc[c] = w.p.sc[i];
    w.fl[c] = w.p.fl[i];
    // the target was AIR, whose temperature word means nothing: the particle's
    // (a SOUP tile's temperature; 0 for the others) is stored without a type test
    if (w.tp) w.tp[c] = w.p.tp[i];
    if (w.dirty) w.dirty[c] = 1;
    w.p_state[i] = PS_DEAD;
}

// round 1 over all requests, phase 1: pick targets; AIR targets get the claim sentinel
__global__ void k_dep_target(const WorldDev *__restrict__ worlds, const MatTable *__restrict__ mt) {
    __shared__ uint8_t s_type[MAXMAT];
    load_types(s_type, mt);
    const WorldDev &w = worlds[blockIdx.y];
    const int n = w.req_count[0];
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
        int i = w.req_list[j];
        int t = dep_target(w, s_type, i, w.p_state[i]);
        w.req_target[j] = t;
        if (t >= 0) w.df[t] = 0x7fffffff;
    }
}
// phase 2: claims (lowest particle index wins an AIR cell), merges, failures
__global__ void k_dep_claim(const WorldDev *__restrict__ worlds, const MatTable *__restrict__ mt) {
    const WorldDev &w = worlds[blockIdx.y];
    const int n = w.req_count[0];
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
        int i = w.req_list[j], t = w.req_target[j];
        if (t == -1)
            dep_fail(w, i);
        else if (t < 0)
            dep_merge(w, mt, i, t & 0x7fffffff);
        else
            atomicMin(&w.df[t], i);
    }
}
// phase 3: winners write their tile; losers search again from where they stopped
__global__ void k_dep_decide(const WorldDev *__restrict__ worlds) {
    const WorldDev &w = worlds[blockIdx.y];
    const int n = w.req_count[0];
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
        int i = w.req_list[j], t = w.req_target[j];
        if (t < 0) continue;
        if (w.df[t] == i) {
            dep_fill(w, i, t);
            int k = atomicAdd(&w.req_count[2], 1);  // filled cells, for k_dep_clear
            w.req_list2[w.part_cap + k] = t;
        } else {
            w.p_state[i] = PS_SPIRAL;
            int k = atomicAdd(&w.req_count[1], 1);
            w.req_list2[k] = i;
        }
    }
}

// Grid-wide barrier for the cooperative deposit kernel. The spin is bounded: if
// it ever gives up it records ERR_TIMEOUT and lets the block continue, so a wait
// can never hang the device.
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

// Rounds 2.. of the deposit resolution for every world, in one cooperative launch.
// Open requests of round r live in list (r even: req_list2, odd: req_list) with
// their count in req_count[1] (r even) / req_count[0] (r odd).
//
// The last rounds have few open requests (tens, then one or two on a 4096x2048
// world), and a grid-wide barrier costs far more than their work. So once a round
// starts with at most DEP_SOLO_MAX open requests (at most one per thread of a
// block: each request's walk is a chain of global loads and must not queue behind
// others), block 0 finishes the rounds alone with block barriers and the other
// blocks leave. Every block reads the same counts (written before the last grid
// barrier or before the launch), so they all take the same decision.
constexpr int DEP_SOLO_MAX = 256;

__global__ void k_dep_rounds(const WorldDev *__restrict__ worlds, int n_worlds, const MatTable *__restrict__ mt) {
    __shared__ uint8_t s_type[MAXMAT];
    load_types(s_type, mt);
    GridBar *gb = (GridBar *)worlds[0].bar;
    const unsigned nb = gridDim.x;
    int32_t *err = worlds[0].err;
    bool solo = false;
    for (int r = 0;; r++) {
        if (r > (1 << 22)) {
            if (threadIdx.x == 0 && blockIdx.x == 0) atomicOr(err, ERR_TIMEOUT);
            break;
        }
        const int ci = (r & 1) ? 0 : 1, ni = (r & 1) ? 1 : 0;
        if (!solo) {
            int open = 0;
            for (int wi = 0; wi < n_worlds; wi++) open += ((volatile int32_t *)worlds[wi].req_count)[ci];
            if (open <= DEP_SOLO_MAX) {
                if (blockIdx.x != 0) return;
                solo = true;
            }
        }
        const int gtid = solo ? (int)threadIdx.x : (int)(blockIdx.x * blockDim.x + threadIdx.x);
        const int gstride = solo ? (int)blockDim.x : (int)(gridDim.x * blockDim.x);
        auto sync = [&]() {
            if (solo)
                __syncthreads();
            else
                grid_sync(gb, nb, err);
        };
        // phase 1: targets against the grid at the start of the round
        for (int wi = 0; wi < n_worlds; wi++) {
            const WorldDev &w = worlds[wi];
            const int n = w.req_count[ci];
            const int32_t *cur = (r & 1) ? w.req_list : w.req_list2;
            if (gtid == 0) w.req_count[ni] = 0;
            for (int j = gtid; j < n; j += gstride) {
                int i = cur[j];
                int t = dep_target(w, s_type, i, w.p_state[i]);
                w.req_target[j] = t;
                if (t >= 0) w.df[t] = 0x7fffffff;
            }
        }
        sync();
        // phase 2: claims, merges, failures
        for (int wi = 0; wi < n_worlds; wi++) {
            const WorldDev &w = worlds[wi];
            const int n = w.req_count[ci];
            const int32_t *cur = (r & 1) ? w.req_list : w.req_list2;
            for (int j = gtid; j < n; j += gstride) {
                int i = cur[j], t = w.req_target[j];
                if (t == -1)
                    dep_fail(w, i);
                else if (t < 0)
                    dep_merge(w, mt, i, t & 0x7fffffff);
                else
                    atomicMin(&w.df[t], i);
            }
        }
        sync();
        // phase 3: winners fill, losers go to the next round's list
        for (int wi = 0; wi < n_worlds; wi++) {
            const WorldDev &w = worlds[wi];
            const int n = w.req_count[ci];
            const int32_t *cur = (r & 1) ? w.req_list : w.req_list2;
            int32_t *nxt = (r & 1) ? w.req_list2 : w.req_list;
            for (int j = gtid; j < n; j += gstride) {
                int i = cur[j], t = w.req_target[j];
                if (t < 0) continue;
                if (w.df[t] == i) {
                    dep_fill(w, i, t);
                    int k = atomicAdd(&w.req_count[2], 1);
                    w.req_list2[w.part_cap + k] = t;
                } else {
                    int k = atomicAdd(&w.req_count[ni], 1);
                    nxt[k] = i;
                }
            }
        }
        sync();
        int open = 0;
        for (int wi = 0; wi < n_worlds; wi++) open += ((volatile int32_t *)worlds[wi].req_count)[ni];
        if (open == 0) break;
    }
}

// filled cells no longer hold a claim: their diff word becomes 0
__global__ void k_dep_clear(const WorldDev *__restrict__ worlds) {
    const WorldDev &w = worlds[blockIdx.y];
    const int n = w.req_count[2];
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x)
        w.df[w.req_list2[w.part_cap + j]] = 0;
}

// f32 worlds: the deposits into liquid of this particle tick, applied to each cell in
// particle-index order (tile.fluidAmount += particle amount, world.cpp:2123, in the
// reference's float add). One block per world: each round every cell takes its
// lowest-index pending deposit, so a cell with k deposits is done after k rounds.
__global__ void k_merge_f32(const WorldDev *__restrict__ worlds) {
    const WorldDev &w = worlds[blockIdx.x];
    if (!w.f32) return;
    __shared__ int s_open, s_next;
    const int n0 = *w.merge_count;
    if (n0 == 0) return;
    // two lists of part_cap entries: the open deposits of this round, the next's
    int32_t *cur = w.merge_list, *nxt = w.merge_list + w.part_cap;
    if (threadIdx.x == 0) s_open = n0;
    __syncthreads();
    for (int round = 0; round < (1 << 24); round++) {
        const int n = s_open;
        if (n == 0) break;
        for (int j = threadIdx.x; j < n; j += blockDim.x) {
            const int i = cur[j];
            atomicMin(&w.merge_claim[w.p_lxly[i]], (uint32_t)i);
        }
        if (threadIdx.x == 0) s_next = 0;
        __syncthreads();
        // the winners add (one thread per cell); the others go to the next round
        for (int j = threadIdx.x; j < n; j += blockDim.x) {
            const int i = cur[j];
            const int c = w.p_lxly[i];
            if (w.merge_claim[c] == (uint32_t)i)
                w.sc[c] = __float_as_int(__fadd_rn(__int_as_float(w.sc[c]), __int_as_float(w.p.sc[i])));
            else
                nxt[atomicAdd(&s_next, 1)] = i;
        }
        __syncthreads();
        for (int j = threadIdx.x; j < n; j += blockDim.x) w.merge_claim[w.p_lxly[cur[j]]] = 0xFFFFFFFFu;
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

__global__ void k_cmp_count(const WorldDev *__restrict__ worlds) {
    const WorldDev &w = worlds[blockIdx.y];
    const int n = *w.part_count;
    const int seg = (n + gridDim.x - 1) / gridDim.x;
    const int b0 = blockIdx.x * seg, b1 = min(n, b0 + seg);
    int cnt = 0;
    for (int i = b0 + threadIdx.x; i < b1; i += blockDim.x) cnt += keep(w, i) ? 1 : 0;
    __shared__ int s[32];
    for (int o = 16; o > 0; o >>= 1) cnt += __shfl_down_sync(0xffffffffu, cnt, o);
    if ((threadIdx.x & 31) == 0) s[threadIdx.x >> 5] = cnt;
    __syncthreads();
    if (threadIdx.x == 0) {
        int t = 0;
        for (int k = 0; k < (int)(blockDim.x >> 5); k++) t += s[k];
        w.scan_tmp[blockIdx.x] = t;
    }
}

// exclusive scan of the per-block counts (nblocks <= blockDim.x), one block per world
__global__ void k_cmp_scan(const WorldDev *__restrict__ worlds, int nblocks) {
    const WorldDev &w = worlds[blockIdx.x];
    __shared__ int s[32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int v = (int)threadIdx.x < nblocks ? w.scan_tmp[threadIdx.x] : 0;
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
    const int excl = (wid > 0 ? s[wid - 1] : 0) + inc - v;
    if ((int)threadIdx.x < nblocks) w.scan_tmp[threadIdx.x] = excl;
    if ((int)threadIdx.x == nblocks - 1) w.scan_tmp[nblocks] = excl + v;
}

__global__ void k_cmp_scatter(const WorldDev *__restrict__ worlds) {
    const WorldDev &w = worlds[blockIdx.y];
    const int n = *w.part_count;
    const int seg = (n + gridDim.x - 1) / gridDim.x;
    const int b0 = blockIdx.x * seg, b1 = min(n, b0 + seg);
    __shared__ int s[32];
    __shared__ int s_carry;
    if (threadIdx.x == 0) s_carry = w.scan_tmp[blockIdx.x];
    __syncthreads();
    for (int base = b0; base < b1; base += blockDim.x) {
        int i = base + threadIdx.x;
        int v = (i < b1 && keep(w, i)) ? 1 : 0;
        int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
        unsigned m = __ballot_sync(0xffffffffu, v);
        int inwarp = __popc(m & ((1u << lane) - 1u));
        if (lane == 0) s[wid] = __popc(m);
        __syncthreads();
        int before = s_carry;
        for (int k = 0; k < wid; k++) before += s[k];
        if (v) {
            int o = before + inwarp;
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
        __syncthreads();
        if (threadIdx.x == 0) {
            int t = 0;
            for (int k = 0; k < nw; k++) t += s[k];
            s_carry += t;
        }
        __syncthreads();
    }
}

__global__ void k_cmp_copy(const WorldDev *__restrict__ worlds, int nblocks) {
    const WorldDev &w = worlds[blockIdx.y];
    const int m = w.scan_tmp[nblocks];
    for (int o = blockIdx.x * blockDim.x + threadIdx.x; o < m; o += gridDim.x * blockDim.x) {
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
    k_part_move<<<gm, 256, 0, s>>>(d_worlds, mt);
    k_dep_target<<<gm, 256, 0, s>>>(d_worlds, mt);
    k_dep_claim<<<gm, 256, 0, s>>>(d_worlds, mt);
    k_dep_decide<<<gm, 256, 0, s>>>(d_worlds);
    {
        // every block of a cooperative launch is resident, so the grid barrier is safe
        static int coop_blocks = 0;
        if (!coop_blocks) {
            int per_sm = 0;
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_dep_rounds, 256, 0);
            int dev = 0, nsm = 1;
            cudaGetDevice(&dev);
            cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
            coop_blocks = std::max(1, std::min(per_sm, 4) * nsm);
        }
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(coop_blocks);
        cfg.blockDim = dim3(256);
        cfg.dynamicSmemBytes = 0;
        cfg.stream = s;
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeCooperative;
        attr[0].val.cooperative = 1;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
        cudaLaunchKernelEx(&cfg, k_dep_rounds, (const WorldDev *)d_worlds, n_worlds, mt);
    }
    k_dep_clear<<<gm, 256, 0, s>>>(d_worlds);
    k_merge_f32<<<n_worlds, 1024, 0, s>>>(d_worlds);
    dim3 gc(PART_BLOCKS, n_worlds);
    k_cmp_count<<<gc, PART_THREADS, 0, s>>>(d_worlds);
    k_cmp_scan<<<n_worlds, PART_BLOCKS, 0, s>>>(d_worlds, PART_BLOCKS);
    k_cmp_scatter<<<gc, PART_THREADS, 0, s>>>(d_worlds);
    k_cmp_copy<<<gm, 256, 0, s>>>(d_worlds, PART_BLOCKS);
    k_part_end<<<n_worlds, 32, 0, s>>>(d_worlds, PART_BLOCKS);
    return cudaGetLastError();
}

int particle_scan_blocks() { return PART_BLOCKS; }

}  // namespace fse
