// fse_tick.cu -- the cell update of world::tick() (source/engine/world.cpp:1036-1948)
// as one colour-pass kernel.
//
// A launch handles one chunk colour of one iteration (world.cpp:1050-1077) for a
// list of chunks, possibly of many worlds. Each CTA stages its chunk plus a halo in
// shared memory (id, flags, scalar, colour; the pending fluid diff stays in HBM and
// is touched only by SOUP cells), runs sweeps A, B and C as sequences of lattice
// sub-phases separated by __syncthreads(), and writes back only the cells it
// changed. Inside a sub-phase every cell is processed by its own thread; the
// lattice spacing makes every write set disjoint from every other cell's read and
// write sets, so the result does not depend on thread timing.
//
// A sub-phase costs about one rule's dependent chain of shared-memory accesses
// plus one barrier, whatever the mix of materials in a warp (sorting cells by type
// first was measured and did not pay), so every thread simply runs the rule of its
// own cells; spawned particles are ranked in the lattice enumeration order.
//
// The reference copies neighbour cells into locals and writes those copies back
// later; no rule modifies such a neighbour between the copy and the write-back, so
// here the write-back is a move inside shared memory at write time (move()), which
// keeps only the active cell in registers.
//
// The kernel is built twice (template TEMP): worlds that keep liquid temperatures
// (FSE_CFG_TEMPERATURE) copy them with every liquid move; the others run code with
// no trace of that plane. fse_tick_temp.cu compiles the TEMP instantiation as a
// translation unit of its own (including this file with FSE_TICK_TEMP_TU), so the
// two build in parallel.
#include "fse_internal.cuh"

// Optional per-phase cycle counters of the colour pass (build with
// -DFSE_PHASE_CLOCKS): thread 0 of each CTA accumulates clock64() deltas between
// barriers; fse_debug_phase_clocks() reads the totals. Off by default: no cost.
#ifdef FSE_PHASE_CLOCKS
static __device__ unsigned long long g_phase_clk[16];  // per translation unit
static __device__ unsigned long long g_phase_max[16];  // per phase: the largest CTA total; [15]: largest CTA
#define FSE_PT_DECL                       \
    __shared__ long long pt_acc[16];      \
    long long pt_last = clock64();        \
    const long long pt_first = pt_last;   \
    if (threadIdx.x < 16) pt_acc[threadIdx.x] = 0;
#define FSE_PT(k)                           \
    if (threadIdx.x == 0) {                 \
        long long t_ = clock64();           \
        pt_acc[(k)] += t_ - pt_last;        \
        pt_last = t_;                       \
    }
#define FSE_PT_FLUSH                                                                                   \
    __syncthreads();                                                                                   \
    if (threadIdx.x < 15) {                                                                            \
        atomicAdd(&g_phase_clk[threadIdx.x], (unsigned long long)pt_acc[threadIdx.x]);                 \
        atomicMax(&g_phase_max[threadIdx.x], (unsigned long long)pt_acc[threadIdx.x]);                 \
    }                                                                                                  \
    if (threadIdx.x == 15) atomicMax(&g_phase_max[15], (unsigned long long)(clock64() - pt_first));
#else
#define FSE_PT_DECL
#define FSE_PT(k)
#define FSE_PT_FLUSH
#endif

namespace fse {

constexpr int MAXRW = 160;        // tile row width bound (chunk <= 128, halo <= 5), a multiple of 32

// 4-byte global -> shared copy that does not pass through registers (sm_80+ cp.async)
__device__ __forceinline__ void cp_async4(void *smem, const void *gmem) {
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

// q = e / n and r = e % n for 0 <= e < 2^16, 1 <= n <= 256, from a float reciprocal
// of n: (e + 0.5) / n sits at least 0.5 / n from an integer, far more than the
// float error, so the truncation is exact.
__device__ __forceinline__ void divmod_small(int e, int n, float rn, int &q, int &r) {
    q = (int)(((float)e + 0.5f) * rn);
    r = e - q * n;
}

struct Cell {
    uint16_t id;
    uint8_t fl;
    int32_t sc;
    uint32_t col;
    int32_t df;
};

struct SpawnEv {
    int n;     // particles to emit (0 = none)
    int kind;  // 1 sand, 2 soup, 3 fire
    int x, y;
    uint16_t id;
    uint8_t fl;
    uint32_t col;
    int32_t sc;
    float vx, vy;
    uint32_t ck, k0;
    int16_t tp;  // temperature of a SOUP tile (kind 2; set only where temperatures are kept)
};

// ------------------------------------------------------- shared-memory tile
// Region: x in [cx - HALO, cx + C + HALO), full state for y in
// [cy - HALO, cy + C + HALO), material ids only down to y < cy + C + 10 (the
// deepest read, the friction pillar of world.cpp:1619-1627).
//
// Every access of the rules stays inside the tile: relative to the active cell
// they reach x +- 2 (fire), y - 2 .. y + 2 in the full planes, ids down to y + 4
// (sand and liquid free fall), and the interaction boxes, whose |offset| + radius
// <= 5 is enforced at registration and which run with HALO = 5; the sweep-B pillar
// reads ids down to cy + C + 9. So the tile needs no bounds checks. EDGE selects
// the world bounds policy of world.cpp:999-1008 (outside reads GENERIC_SOLID,
// outside writes dropped); it is needed only when the tile crosses the world edge.
struct TileData {
    uint16_t *s_id;
    uint8_t *s_fl;
    int32_t *s_sc;
    uint32_t *s_col;
    const uint32_t *ma;  // material word A in shared memory
    const float *md;     // density in shared memory
    int32_t *df;         // HBM diff plane
    int16_t *tp;         // HBM temperature plane of SOUP cells (NULL: not kept)
    int x0, y0, RW, RHF, RHI;
    int W, H;
    int id_solid, id_air;
    // sweep-B pillar snapshot: AIR bits of columns ax0.., rows ay0.., 5 words per column
    const uint32_t *s_air;
    int ax0, ay0, aw;
    // a chunk split over a CTA pair: the partner's copy of the planes (shared::cluster
    // addresses) and the world row of its first tile row; both copies have RW, RHF
    // and RHI of this one
    uint32_t p_id, p_fl, p_sc, p_col;
    int py0;
};

// --------------------------------------------------- CTA-pair (cluster) helpers
__device__ __forceinline__ uint32_t smem_addr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }
// the address of this CTA's shared location `a` in the shared memory of cluster rank r
__device__ __forceinline__ uint32_t mapa_rank(uint32_t a, uint32_t r) {
    uint32_t o;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(o) : "r"(a), "r"(r));
    return o;
}
__device__ __forceinline__ void st_cluster_u8(uint32_t a, uint8_t v) {
    asm volatile("st.shared::cluster.u8 [%0], %1;" ::"r"(a), "h"((unsigned short)v) : "memory");
}
__device__ __forceinline__ void st_cluster_u16(uint32_t a, uint16_t v) {
    asm volatile("st.shared::cluster.u16 [%0], %1;" ::"r"(a), "h"(v) : "memory");
}
__device__ __forceinline__ void st_cluster_u32(uint32_t a, uint32_t v) {
    asm volatile("st.shared::cluster.u32 [%0], %1;" ::"r"(a), "r"(v) : "memory");
}
__device__ __forceinline__ uint32_t cluster_rank() {
    uint32_t r;
    asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
    return r;
}
// every thread of both CTAs of the pair; the partner's shared-memory stores made
// before it are visible after it
__device__ __forceinline__ void cluster_sync() {
    asm volatile("barrier.cluster.arrive.release;\n\tbarrier.cluster.wait.acquire;" ::: "memory");
}

// ------------------------------------------------------ TMA staging helpers
// The 4-byte planes of a tile come in as two 2D tensor copies (cp.async.bulk.tensor)
// completing on one mbarrier; thread 0 issues them, every thread waits.
__device__ __forceinline__ void mbar_init(uint64_t *bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
// orders this thread's generic shared-memory accesses before later async-proxy ones
__device__ __forceinline__ void fence_proxy_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, unsigned parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
// box of the tensor map at (x, y) (x a multiple of 4 cells: a 16-byte boundary) into
// dst (128-byte aligned); complete_tx on bar
__device__ __forceinline__ void tma_load_2d(void *dst, const void *tmap, int x, int y, uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], "
        "[%4];" ::"r"(smem_addr(dst)),
        "l"(tmap), "r"(x), "r"(y), "r"(smem_addr(bar))
        : "memory");
}

// ------------------------------------------------- fused-tick flag helpers
__device__ __forceinline__ uint32_t ld_acquire_gpu(const uint32_t *p) {
    uint32_t v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_release_gpu(uint32_t *p, uint32_t v) {
    asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
constexpr unsigned long long FUSED_WAIT_NS = 2000000000ull;  // a dependency wait gives up after 2 s

// LIVE: the pillar reads the tile as it stands (the reference's own order, where
// one thread updates the chunk's cells in turn) instead of the sweep-B snapshot.
// F32: liquid amounts and diffs are f32 bit patterns (FSE_CFG_F32_FLUID).
// PAIR: the chunk is split over a CTA pair; every write to a row the partner's tile
// holds is made in both copies (reads are always local), so both copies of the
// shared rows stay equal; at the end of a sub-phase the cluster barrier makes them
// visible.
template <bool EDGE, bool TEMP, bool LIVE = false, bool F32 = false, bool PAIR = false>
struct Tile : TileData {
    static constexpr bool kTemp = TEMP;
    static constexpr bool kF32 = F32;
    __device__ __forceinline__ explicit Tile(const TileData &d) : TileData(d) {}

    // the partner's index of cell (x, y): -1 outside its tile; *full: a full-state row
    __device__ __forceinline__ int pli(int x, int y, bool *full) const {
        const int r = y - py0;
        if (r < 0 || r >= RHI) return -1;
        *full = r < RHF;
        return r * RW + (x - x0);
    }
    // the same bytes as the local copy of cell i, in the partner's copy of (x, y)
    __device__ __forceinline__ void mirror(int x, int y, int i) const {
        if constexpr (PAIR) {
            bool full;
            const int j = pli(x, y, &full);
            if (j < 0) return;
            st_cluster_u16(p_id + 2u * (uint32_t)j, s_id[i]);
            if (full) {
                st_cluster_u8(p_fl + (uint32_t)j, s_fl[i]);
                st_cluster_u32(p_sc + 4u * (uint32_t)j, (uint32_t)s_sc[i]);
                st_cluster_u32(p_col + 4u * (uint32_t)j, s_col[i]);
            }
        }
    }
    __device__ __forceinline__ void mirror_idfl(int x, int y, int i) const {
        if constexpr (PAIR) {
            bool full;
            const int j = pli(x, y, &full);
            if (j < 0) return;
            st_cluster_u16(p_id + 2u * (uint32_t)j, s_id[i]);
            if (full) st_cluster_u8(p_fl + (uint32_t)j, s_fl[i]);
        }
    }

    // 10 AIR bits of column x starting at row y: from the snapshot (0 outside it), or
    // live
    __device__ __forceinline__ uint32_t air10(int x, int y) const {
        if constexpr (LIVE) {
            uint32_t bits = 0;
            for (int k = 0; k < 10; k++)
                if (type(x, y + k) == T_AIR) bits |= 1u << k;
            return bits;
        }
        int sx = x - ax0, sy = y - ay0;
        if ((unsigned)sx >= (unsigned)aw || sy < 0) return 0u;
        const uint32_t *col = s_air + sx * 5;
        int wi = sy >> 5, b = sy & 31;
        if (wi >= 5) return 0u;
        unsigned long long v = col[wi] | ((unsigned long long)(wi + 1 < 5 ? col[wi + 1] : 0u) << 32);
        return (uint32_t)(v >> b) & 0x3FFu;
    }

    // inside the world (always true away from the world edge)
    __device__ __forceinline__ bool inw(int x, int y) const {
        return !EDGE || ((unsigned)x < (unsigned)W && (unsigned)y < (unsigned)H);
    }
    // inside the world whatever EDGE: the writes of fire and interactions can reach
    // cells outside the world, where world.cpp:1003-1008 drops them
    __device__ __forceinline__ bool in_world(int x, int y) const {
        return (unsigned)x < (unsigned)W && (unsigned)y < (unsigned)H;
    }
    __device__ __forceinline__ int li(int x, int y) const { return (y - y0) * RW + (x - x0); }

    // world.cpp:999-1002: outside the world reads Tiles_TEST_SOLID
    __device__ __forceinline__ int id(int x, int y) const {
        if (!inw(x, y)) return id_solid;
        return s_id[li(x, y)] & 0x7FFF;
    }
    __device__ __forceinline__ int type(int x, int y) const { return mt_type(ma[id(x, y)]); }
    __device__ __forceinline__ int32_t sc(int x, int y) const {
        if (!inw(x, y)) return 0;
        return s_sc[li(x, y)];
    }
    __device__ __forceinline__ int32_t df_of(int x, int y) const {
        if (!inw(x, y) || mt_type(ma[id(x, y)]) != T_SOUP) return 0;
        return df[y * W + x];
    }
    // The active cell. Its df field starts at 0 and collects the change of its
    // pending diff (put_delta applies it with a reduction); the stored diff is
    // loaded only where a rule needs the value itself (df_load).
    __device__ __forceinline__ Cell get_active(int x, int y) const {
        Cell c;
        int i = li(x, y);
        c.id = s_id[i] & 0x7FFF;
        c.fl = s_fl[i] & (uint8_t)~VISITED;
        c.sc = s_sc[i];
        c.col = s_col[i];
        c.df = 0;
        return c;
    }
    __device__ __forceinline__ int32_t df_load(int x, int y) const { return df[y * W + x]; }
    // write the active cell back at its own position, adding its diff change
    __device__ __forceinline__ void put_delta(int x, int y, const Cell &c) const {
        int i = li(x, y);
        s_id[i] = c.id | DIRTY;
        s_fl[i] = (uint8_t)((c.fl & (uint8_t)~VISITED) | (s_fl[i] & VISITED));
        s_sc[i] = c.sc;
        s_col[i] = c.col;
        mirror(x, y, i);
        if (c.df != 0) atomicAdd(&df[y * W + x], c.df);  // no return value: a fire-and-forget reduction
    }
    // world.cpp:1004-1008: outside the world writes are dropped
    __device__ __forceinline__ void put(int x, int y, const Cell &c) const {
        if (!inw(x, y)) return;
        int i = li(x, y);
        s_id[i] = c.id | DIRTY;
        s_fl[i] = (uint8_t)((c.fl & (uint8_t)~VISITED) | (s_fl[i] & VISITED));
        s_sc[i] = c.sc;
        s_col[i] = c.col;
        mirror(x, y, i);
        if (mt_type(ma[c.id]) == T_SOUP) df[y * W + x] = c.df;
    }
    __device__ __forceinline__ void set_nothing(int x, int y) const {
        Cell c;
        c.id = (uint16_t)id_air;
        c.fl = 0;
        c.sc = 0;
        c.col = 0;
        c.df = 0;
        put(x, y, c);
    }
    // write the cell at (sx, sy) over (dx, dy); the visited mark stays with the position
    __device__ __forceinline__ void move(int dx, int dy, int sx, int sy) const {
        if (!inw(dx, dy)) return;
        int d = li(dx, dy);
        if (!inw(sx, sy)) {
            s_id[d] = (uint16_t)id_solid | DIRTY;
            s_fl[d] = (uint8_t)(s_fl[d] & VISITED);
            s_sc[d] = 0;
            s_col[d] = 0xff0000u;
            mirror(dx, dy, d);
            return;
        }
        int s = li(sx, sy);
        uint16_t v = s_id[s] & 0x7FFF;
        s_id[d] = v | DIRTY;
        s_fl[d] = (uint8_t)((s_fl[s] & (uint8_t)~VISITED) | (s_fl[d] & VISITED));
        s_sc[d] = s_sc[s];
        s_col[d] = s_col[s];
        mirror(dx, dy, d);
        if (mt_type(ma[v]) == T_SOUP) {
            df[dy * W + dx] = df[sy * W + sx];
            if (TEMP && tp) tp[dy * W + dx] = tp[sy * W + sx];
        }
    }
    // Temperatures of SOUP cells live in HBM beside the diff; the tile's scalar is
    // their amount. They move only where a SOUP cell moves or is made, so the
    // rules touch them at those few places and nowhere else.
    __device__ __forceinline__ int16_t tp_load(int x, int y) const {
        return (TEMP && tp) ? tp[y * W + x] : (int16_t)0;
    }
    __device__ __forceinline__ void tp_store(int x, int y, int16_t v) const {
        if (TEMP && tp && inw(x, y)) tp[y * W + x] = v;
    }
    // put a tile just made by a factory (TilesCreate): a SOUP tile takes the
    // factory temperature, or `keep` (a reaction keeps the old temperature)
    __device__ __forceinline__ void put_new(int x, int y, const Cell &c, const MatTable *mt, bool keep = false,
                                            int32_t keep_t = 0) const {
        put(x, y, c);
        if (TEMP && tp && mt_type(ma[c.id]) == T_SOUP)
            tp_store(x, y, keep ? (int16_t)keep_t : (int16_t)__ldg(&mt->f_temp[c.id]));
    }
    // only a change marks the cell for write-back (settled sand clears an already
    // clear flag every pass)
    __device__ __forceinline__ void set_moved(int x, int y, bool on) const {
        if (!inw(x, y)) return;
        int i = li(x, y);
        const uint8_t f = s_fl[i];
        const uint8_t nf = on ? (uint8_t)(f | MOVED) : (uint8_t)(f & (uint8_t)~MOVED);
        if (nf != f) {
            s_fl[i] = nf;
            s_id[i] |= DIRTY;
            mirror_idfl(x, y, i);
        }
    }
    __device__ __forceinline__ void add_diff(int x, int y, int32_t v) const {
        if (!inw(x, y)) return;
        atomicAdd(&df[y * W + x], v);  // fire-and-forget reduction: the thread does not wait
    }
    // f32 worlds: fluidAmountDiff += v as the reference's float add. No other cell of
    // the sub-phase (or wavefront step) touches this diff, and the ones that touched
    // it before did so in the reference's order, so a plain read-modify-write adds in
    // that order.
    __device__ __forceinline__ void add_diff_f(int x, int y, float v) const {
        if (!inw(x, y)) return;
        int32_t *p = &df[y * W + x];
        *p = __float_as_int(__fadd_rn(__int_as_float(*p), v));
    }
    // write the active cell back at its own position with its diff (f32 worlds)
    __device__ __forceinline__ void put_df(int x, int y, const Cell &c, float dfv) const {
        int i = li(x, y);
        s_id[i] = c.id | DIRTY;
        s_fl[i] = (uint8_t)((c.fl & (uint8_t)~VISITED) | (s_fl[i] & VISITED));
        s_sc[i] = c.sc;
        s_col[i] = c.col;
        mirror(x, y, i);
        df[y * W + x] = __float_as_int(dfv);
    }
    __device__ __forceinline__ bool vis(int x, int y) const { return (s_fl[li(x, y)] & VISITED) != 0; }
    __device__ __forceinline__ void setvis(int x, int y) const {
        if (!inw(x, y)) return;
        const int i = li(x, y);
        s_fl[i] |= VISITED;
        mirror_idfl(x, y, i);
    }
};

// ------------------------------------------------------------- rule context
struct Ctx {
    uint32_t pk, ck, k;
    int kx, ky;   // the active cell, whose key ck is derived on the first draw
    bool have_ck;
    int iter;
    int id_fire, id_water, id_lava, id_steam, id_obsidian, has_inter;
    bool f32;  // f32 liquid amounts: the ledger keeps no fluid rows (a compile-time constant)
    const MatTable *mt;
    long long *led_s;      // shared ledger [LED_ROWS][64]
    long long *led_g;      // global ledger [LED_ROWS][MAXMAT]
    const uint32_t *ma;
    const uint8_t *mreact;  // reactions per material (shared)
    // the cell's spawn event, a local of its own: emit_spawns takes its address, and a
    // member whose address escapes keeps the whole context in local memory
    SpawnEv *ev;
    // start the draws of the cell at (x, y); most cells never draw, so the key
    // (two hash rounds) is computed only when the first draw needs it
    __device__ __forceinline__ void at(int x, int y) {
        kx = x;
        ky = y;
        have_ck = false;
        k = 0;
    }
    __device__ __forceinline__ uint32_t key() {
        if (!have_ck) {
            ck = cell_key(pk, (uint32_t)kx, (uint32_t)ky);
            have_ck = true;
        }
        return ck;
    }
    __device__ __forceinline__ uint32_t D() { return draw_k(key(), k++); }
};

__device__ __forceinline__ void led_add(Ctx &c, int row, int mat, long long v) {
    if (v == 0 || mt_type(c.ma[mat]) == T_AIR) return;
    if (mat < 64 && v > -(1LL << 24) && v < (1LL << 24)) {
        // lanes of a warp mostly hit the same counter: sum them first, one atomic per group
        const unsigned act = __activemask();
        const unsigned grp = __match_any_sync(act, row * 64 + mat);
        const int sum = __reduce_add_sync(grp, (int)v);
        if ((threadIdx.x & 31) == __ffs(grp) - 1)
            atomicAdd((unsigned long long *)&c.led_s[row * 64 + mat], (unsigned long long)(long long)sum);
    } else if (mat < 64) {
        atomicAdd((unsigned long long *)&c.led_s[row * 64 + mat], (unsigned long long)v);
    } else {
        atomicAdd((unsigned long long *)&c.led_g[row * MAXMAT + mat], (unsigned long long)v);
    }
}
// a conversion (not a move) of the content old -> nw
__device__ __forceinline__ void led_swap(Ctx &c, int old_id, long long old_fluid, int new_id, long long new_fluid) {
    led_add(c, LED_DN, old_id, 1);
    if (!c.f32 && mt_type(c.ma[old_id]) == T_SOUP) led_add(c, LED_DF, old_id, old_fluid);
    led_add(c, LED_CN, new_id, 1);
    if (!c.f32 && mt_type(c.ma[new_id]) == T_SOUP) led_add(c, LED_CF, new_id, new_fluid);
}
// conversion of whatever is at (x, y) into nw
template <class TL>
__device__ __forceinline__ void led_replace_at(const TL &T, Ctx &c, int x, int y, const Cell &nw) {
    if (!T.inw(x, y)) return;
    int oid = T.id(x, y);
    long long of = (!c.f32 && mt_type(c.ma[oid]) == T_SOUP) ? (long long)T.sc(x, y) + T.df_of(x, y) : 0;
    led_swap(c, oid, of, nw.id, (long long)nw.sc + nw.df);
}

// TilesCreate(id, x, y), game_datastruct.cpp:494-574
__device__ __forceinline__ Cell create_tile(Ctx &c, int mid) {
    Cell t;
    t.id = (uint16_t)mid;
    t.fl = 0;
    t.df = 0;
    t.sc = soup_scalar(c.mt, mid, c.f32);  // a temperature, or a SOUP tile's amount
    t.col = __ldg(&c.mt->f_base[mid]);
    uint32_t fp = __ldg(&c.mt->f_pack[mid]);
    int mod = (int)(fp >> 20);
    if (mod > 0) {
        int shift = (int)(fp & 0xFF), lo = (int)((fp >> 8) & 0xFFF);
        t.col = t.col + ((uint32_t)(lo + (int)(c.D() % (uint32_t)mod)) << shift);
    }
    return t;
}

// CalculateVerticalFlowValue, world.cpp:1021-1034, Q16.16
__device__ __forceinline__ int32_t vflow(int32_t rem, int32_t dst) {
    long long sum = (long long)rem + dst;
    if (sum <= Q_MAXV) return Q_MAXV;
    if (sum < 2 * Q_MAXV + Q_MAXCOMP)  // here MAXV^2 + sum * MAXCOMP < 2^31: 32-bit unsigned is exact
        return (int32_t)(((uint32_t)Q_MAXV * Q_MAXV + (uint32_t)sum * Q_MAXCOMP) / (uint32_t)(Q_MAXV + Q_MAXCOMP));
    return (int32_t)((sum + Q_MAXCOMP) / 2);
}
__device__ __forceinline__ int32_t clampflow(int32_t flow, int32_t rem) {
    if (flow < 0) flow = 0;
    int32_t lim = rem < Q_MAXFLOW ? rem : Q_MAXFLOW;
    return flow > lim ? lim : flow;
}

// CalculateVerticalFlowValue, world.cpp:1021-1034, in the reference's f32: every
// operation separately rounded as the reference's x86-64 build does (no contraction)
__device__ __forceinline__ float vflow_f(float rem, float dst) {
    const float sum = __fadd_rn(rem, dst);
    if (sum <= F_MAXV) return F_MAXV;
    if (sum < __fadd_rn(2.0f * F_MAXV, F_MAXCOMP))
        return __fdiv_rn(__fadd_rn(F_MAXV * F_MAXV, __fmul_rn(sum, F_MAXCOMP)), __fadd_rn(F_MAXV, F_MAXCOMP));
    return __fdiv_rn(__fadd_rn(sum, F_MAXCOMP), 2.0f);
}
// flow = std::max(flow, 0.0f); if (flow > std::min(FLUID_MaxFlow, rem)) flow = ...
// (world.cpp:1320-1321 and its three copies), with std::max/min's own comparisons;
// the FLUID_FlowSpeed factor of 1.0f before it changes no float and is left out
__device__ __forceinline__ float clampflow_f(float flow, float rem) {
    if (flow < 0.0f) flow = 0.0f;
    const float lim = (rem < F_MAXFLOW) ? rem : F_MAXFLOW;
    return (flow > lim) ? lim : flow;
}

__device__ __forceinline__ bool can_sink(const uint32_t *ma, const float *md, int other, int self) {
    int t = mt_type(ma[other]);
    return t == T_AIR || (t != T_SOLID && md[other] < md[self]);
}

// the world of the CTA's current chunk (copied per chunk by thread 0)
__shared__ WorldDev s_w;

// one SOUP flow from (x, y) towards (x + dx, y + dy), shared by the four directions
// of world.cpp:1309-1460; a rendering world also adds it to the flow of (x, y)
// (flowX -= / += flow for left / right, flowY += / -= for down / up,
// world.cpp:1334,1374,1402,1432), a reduction no other cell of the sub-phase makes
template <class TL>
__device__ __forceinline__ void soup_flow(const TL &T, Ctx &c, Cell &t, int32_t &rem, int32_t flow, int nT, int x,
                                          int y, int dx, int dy) {
    if (flow == 0) return;
    const int nx = x + dx, ny = y + dy;
    int32_t *fw = s_w.flow;
    if (fw) atomicAdd(&fw[2 * ((size_t)y * T.W + x) + (dx != 0 ? 0 : 1)], (dx + dy) * flow);
    rem -= flow;
    t.df -= flow;
    if (nT == T_AIR) {
        Cell nt;
        nt.id = t.id;
        nt.fl = 0;
        nt.sc = 0;
        nt.col = t.col;
        nt.df = flow;
        T.put(nx, ny, nt);
        T.tp_store(nx, ny, T.tp_load(x, y));  // MaterialInstance(tile.mat, tile.color, tile.temperature)
        led_add(c, LED_CN, t.id, 1);
    } else {
        T.add_diff(nx, ny, flow);
    }
}

// f32 worlds: one flow of world.cpp:1309-1460 from (x, y) towards (x + dx, y + dy);
// dfv is the active cell's fluidAmountDiff, updated in the reference's order
template <class TL>
__device__ __forceinline__ void soup_flow_f(const TL &T, Ctx &c, const Cell &t, float &rem, float &dfv, float flow,
                                            int nT, int x, int y, int dx, int dy) {
    if (flow == 0.0f) return;
    const int nx = x + dx, ny = y + dy;
    float *fw = reinterpret_cast<float *>(s_w.flow);
    if (fw) {
        // flowX / flowY of (x, y) (world.cpp:1334,1374,1402,1432): only this cell adds to them
        float *q = &fw[2 * ((size_t)y * T.W + x) + (dx != 0 ? 0 : 1)];
        *q = (dx + dy) > 0 ? __fadd_rn(*q, flow) : __fsub_rn(*q, flow);
    }
    rem = __fsub_rn(rem, flow);
    dfv = __fsub_rn(dfv, flow);
    if (nT == T_AIR) {
        // MaterialInstance(tile.mat, tile.color, tile.temperature), fluidAmount 0,
        // then fluidAmountDiff (0) += flow
        Cell nt;
        nt.id = t.id;
        nt.fl = 0;
        nt.sc = __float_as_int(0.0f);
        nt.col = t.col;
        nt.df = __float_as_int(__fadd_rn(0.0f, flow));
        T.put(nx, ny, nt);
        T.tp_store(nx, ny, T.tp_load(x, y));
        led_add(c, LED_CN, t.id, 1);
    } else {
        T.add_diff_f(nx, ny, flow);
    }
}

__device__ __forceinline__ void spawn_one(Ctx &c, int kind, int x, int y, const Cell &t, float vx, float vy) {
    c.ev->n = 1;
    c.ev->kind = kind;
    c.ev->x = x;
    c.ev->y = y;
    c.ev->id = t.id;
    c.ev->fl = t.fl;
    c.ev->col = t.col;
    c.ev->sc = t.sc;
    c.ev->vx = vx;
    c.ev->vy = vy;
}

// ------------------------------------------------- sweep A, f32 liquids
// world.cpp:1269-1567 with the reference's own float amounts (FSE_CFG_F32_FLUID):
// the same branches as the Q16.16 rule, in f32 with every operation rounded on its
// own; the cell's fluidAmountDiff is read when its turn begins (it already holds the
// flows of the cells updated before it) and written back with its own flows
// subtracted in order, as the reference's copy of the tile does.
template <class TL>
__device__ __forceinline__ void rule_a_soup_f32(const TL &T, Ctx &c, Cell &t, int x, int y) {
    const uint32_t *ma = T.ma;
    const float amount = __int_as_float(t.sc);
    if (amount == 0.0f) return;
    if (amount < F_MINV) {
        t.sc = __float_as_int(0.0f);
        T.put_delta(x, y, t);  // t.df is 0: the diff stays as it is
        return;
    }
    // tile.fluidAmount > 0.005 compares in double (0.005 is a double literal)
    if ((double)amount > 0.005 && T.type(x, y + 1) == T_AIR && T.type(x, y + 2) == T_AIR &&
        T.type(x, y + 3) == T_AIR && T.type(x, y + 4) == T_AIR) {  // world.cpp:1283-1305
        T.set_nothing(x, y);
        int n = (int)__fdiv_rn(amount, 4.0f);  // int n = tile.fluidAmount / 4
        if (n < 1) n = 1;
        led_add(c, LED_CN, t.id, n - 1);
        c.ev->n = n;
        c.ev->kind = 2;
        c.ev->x = x;
        c.ev->y = y + 1;
        c.ev->id = t.id;
        c.ev->fl = 0;
        c.ev->col = t.col;
        c.ev->sc = t.sc;
        if (TL::kTemp) c.ev->tp = T.tp_load(x, y);
        c.ev->ck = c.key();
        c.ev->k0 = c.k;
        c.k += 2 * n;
        return;
    }
    if (t.fl & MOVED) return;
    const float start = amount;
    float rem = amount;
    float dfv = __int_as_float(T.df_load(x, y));
    const int bid = T.id(x, y + 1);
    const int bT = mt_type(ma[bid]);
    const bool airBelow = bT == T_AIR;
    if ((airBelow && c.iter <= 2) || bid == (int)t.id) {
        const float dst = (bT == T_SOUP) ? __int_as_float(T.sc(x, y + 1)) : 0.0f;
        soup_flow_f(T, c, t, rem, dfv, clampflow_f(__fsub_rn(vflow_f(start, dst), dst), start), bT, x, y, 0, 1);
    } else if (c.iter == 0 && bT == T_SOUP && bid != (int)t.id) {
        if (c.D() % 10 == 0) {
            t.df = __float_as_int(dfv);  // the cell leaves its position with its diff
            const int16_t tv = T.tp_load(x, y);
            T.move(x, y, x, y + 1);
            T.put(x, y + 1, t);
            T.tp_store(x, y + 1, tv);
            return;
        }
    }
    if (rem < F_MINV) {
        T.put_df(x, y, t, __fsub_rn(dfv, rem));
        return;
    }
    const int lid = T.id(x - 1, y);
    const int lT = mt_type(ma[lid]);
    const bool canL = (lT == T_AIR || lid == (int)t.id) && !airBelow;
    const int rid = T.id(x + 1, y);
    const int rT = mt_type(ma[rid]);
    const bool canR = (rT == T_AIR || rid == (int)t.id) && !airBelow;
    if (canL) {
        const float dst = (lT == T_SOUP) ? __int_as_float(T.sc(x - 1, y)) : 0.0f;
        soup_flow_f(T, c, t, rem, dfv, clampflow_f(__fdiv_rn(__fsub_rn(rem, dst), canR ? 3.0f : 2.0f), rem), lT, x,
                    y, -1, 0);
    }
    if (rem < F_MINV) {
        T.put_df(x, y, t, __fsub_rn(dfv, rem));
        return;
    }
    if (canR) {
        const float dst = (rT == T_SOUP) ? __int_as_float(T.sc(x + 1, y)) : 0.0f;
        soup_flow_f(T, c, t, rem, dfv, clampflow_f(__fdiv_rn(__fsub_rn(rem, dst), 2.0f), rem), rT, x, y, 1, 0);
    }
    if (rem < F_MINV) {
        T.put_df(x, y, t, __fsub_rn(dfv, rem));
        return;
    }
    const int tid = T.id(x, y - 1);
    const int tT = mt_type(ma[tid]);
    if (tT == T_AIR || tid == (int)t.id) {
        const float dst = (tT == T_SOUP) ? __int_as_float(T.sc(x, y - 1)) : 0.0f;
        soup_flow_f(T, c, t, rem, dfv, clampflow_f(__fsub_rn(rem, vflow_f(rem, dst)), rem), tT, x, y, 0, -1);
    } else if (c.iter == 0 && tT == T_SOUP && tid != (int)t.id) {
        if (c.D() % 10 == 0) {
            t.df = __float_as_int(dfv);
            const int16_t tv = T.tp_load(x, y);
            T.move(x, y, x, y - 1);
            T.put(x, y - 1, t);
            T.tp_store(x, y - 1, tv);
            return;
        }
    }
    if (rem < F_MINV) {
        T.put_df(x, y, t, __fsub_rn(dfv, rem));
        return;
    }
    if (start == rem) {  // world.cpp:1472-1483
        uint8_t s = t.fl & SETTLE_MASK;
        if (s < SETTLE_MASK) s++;
        t.fl = (uint8_t)((t.fl & ~SETTLE_MASK) | s);
        if (s >= 10) t.fl |= MOVED;
    } else {
        if (tT == T_SOUP) T.set_moved(x, y - 1, false);
        if (bT == T_SOUP) T.set_moved(x, y + 1, false);
        if (lT == T_SOUP) T.set_moved(x - 1, y, false);
        if (rT == T_SOUP) T.set_moved(x + 1, y, false);
    }
    T.put_df(x, y, t, dfv);
    // WATER on LAVA, world.cpp:1519-1537
    if ((int)t.id == c.id_water && T.id(x, y + 1) == c.id_lava) {
        const MatTable *mt = c.mt;
        Cell st = create_tile(c, c.id_steam);
        led_swap(c, t.id, 0, st.id, 0);
        T.put_new(x, y, st, mt);
        Cell ob = create_tile(c, c.id_obsidian);
        led_replace_at(T, c, x, y + 1, ob);
        T.put_new(x, y + 1, ob, mt);
        T.setvis(x, y + 1);
        for (int xx = -1; xx <= 1; xx++)
            for (int yy = 0; yy <= 2; yy++) {
                if (T.id(x + xx, y + yy) == c.id_lava) {
                    Cell o2 = create_tile(c, c.id_obsidian);
                    led_replace_at(T, c, x + xx, y + yy, o2);
                    T.put_new(x + xx, y + yy, o2, mt);
                    T.setvis(x + xx, y + yy);
                }
            }
    }
}

// ----------------------------------------------------------------- sweep A
template <class TL>
__device__ __forceinline__ void rule_a(const TL &T, Ctx &c, int x, int y) {
    if (T.vis(x, y)) return;  // world.cpp:1091
    const uint32_t *ma = T.ma;
    const float *md = T.md;
    const int sid = T.id(x, y);
    const uint32_t a = ma[sid];
    if (c.iter >= mt_iter(a)) {  // world.cpp:1093-1096
        T.setvis(x, y);
        return;
    }
    const int type = mt_type(a);
    if (type != T_SAND && type != T_SOUP && type != T_GAS && sid != c.id_fire) return;
    if (sid != c.id_fire) {
        // the common no-op cases, decided before the cell is loaded: sand that
        // cannot sink (world.cpp:1206, without interactions or reactions) and gas
        // with no AIR above (world.cpp:1573)
        if (type == T_SAND && !c.has_inter && c.mreact[sid] == 0 && !can_sink(ma, md, T.id(x, y + 1), sid)) return;
        if (type == T_GAS && T.type(x, y - 1) != T_AIR) return;
    }
    Cell t = T.get_active(x, y);
    c.at(x, y);
    const MatTable *mt = c.mt;

    if (sid == c.id_fire) {  // world.cpp:1101-1146
        if (c.D() % 10 == 0) t.col = (255u << 16) | ((uint32_t)(100 + (int)(c.D() % 50)) << 8) | 50u;
        if (c.D() % 10 == 0) {
            float vx = (float)((int)(c.D() % 10) - 5) / 20.0f;
            float vy = -((float)(int)(c.D() % 10) / 10.0f) / 3.0f + -0.5f;
            spawn_one(c, 3, x, y - 1, t, vx, vy);
            led_add(c, LED_CN, t.id, 1);
        }
        if (c.D() % 150 == 0) {
            led_swap(c, t.id, (long long)t.sc + t.df, T.id_air, 0);
            T.set_nothing(x, y);
            T.setvis(x, y);
        } else {
            bool found = false;
            for (int xx = -2; xx <= 2; xx++)
                for (int yy = -2; yy <= 2; yy++) {
                    if (T.type(x + xx, y + yy) == T_SOLID) {
                        found = true;
                        if (c.D() % 500 == 0) {
                            Cell f = create_tile(c, c.id_fire);
                            if (T.in_world(x + xx, y + yy)) {
                                led_replace_at(T, c, x + xx, y + yy, f);
                                T.put_new(x + xx, y + yy, f, mt);
                                T.setvis(x + xx, y + yy);
                            }
                        }
                    }
                }
            if (!found && c.D() % 120 == 0) {
                led_swap(c, t.id, (long long)t.sc + t.df, T.id_air, 0);
                T.set_nothing(x, y);
                T.setvis(x, y);
            }
        }
    }

    if (type == T_SAND) {
        const int bid = T.id(x, y + 1);  // world.cpp:1150
        const int bt = mt_type(ma[bid]);
        if (c.has_inter) {  // world.cpp:1153-1179
            int hit = -1;
            for (int i = 0; i < mt->n_inter; i++)
                if (mt->inter[i][0] == (int)t.id && mt->inter[i][1] == bid) hit = i;
            if (hit >= 0) {
                for (int i = 0; i < mt->n_inter; i++) {
                    if (mt->inter[i][0] != (int)t.id || mt->inter[i][1] != bid) continue;
                    int kind = mt->inter[i][2], d1 = mt->inter[i][3], d2 = mt->inter[i][4];
                    int ox = mt->inter[i][5], oy = mt->inter[i][6];
                    // the radius is a u32 in the reference, so its loops compare
                    // unsigned: a box whose low corner is negative is not visited
                    if (ox - d2 < 0 || oy - d2 < 0) continue;
                    for (int xx = ox - d2; xx <= ox + d2; xx++)
                        for (int yy = oy - d2; yy <= oy + d2; yy++) {
                            bool doit = (kind == INTER_TRANSFORM)
                                            ? (T.id(x + xx, y + yy) == bid)
                                            : ((xx == 0 && yy == 0) || T.id(x + xx, y + yy) == T.id_air);
                            if (doit) {
                                Cell nt = create_tile(c, d1);
                                if (T.in_world(x + xx, y + yy)) {
                                    led_replace_at(T, c, x + xx, y + yy, nt);
                                    T.put_new(x + xx, y + yy, nt, mt);
                                    T.setvis(x + xx, y + yy);
                                }
                            }
                        }
                }
                return;
            }
        }
        const int nr = c.mreact[t.id];
        if (nr > 0) {  // world.cpp:1181-1204
            bool react = false;
            for (int i = 0; i < nr; i++) {
                int kind = mt->react[t.id][i][0], temp = mt->react[t.id][i][1], res = mt->react[t.id][i][2];
                bool hit = (kind == REACT_BELOW) ? (t.sc < temp) : (t.sc > temp);
                if (hit) {
                    Cell nt = create_tile(c, res);
                    // the temperature is kept (world.cpp:1188,1196): in the scalar,
                    // or beside the amount of a SOUP result
                    if (mt_type(ma[nt.id]) != T_SOUP) nt.sc = t.sc;
                    led_replace_at(T, c, x, y, nt);
                    T.put_new(x, y, nt, mt, true, t.sc);
                    T.setvis(x, y);
                    react = true;
                }
            }
            if (react) return;
        }
        // world.cpp:1206-1267
        if (!can_sink(ma, md, bid, t.id)) return;
        const bool canL = can_sink(ma, md, T.id(x - 1, y + 1), t.id);
        const bool canR = can_sink(ma, md, T.id(x + 1, y + 1), t.id);
        if (!((canL || canR) && c.D() % 20 == 0)) {
            if (bt == T_AIR && T.type(x, y + 2) == T_AIR && T.type(x, y + 3) == T_AIR && T.type(x, y + 4) == T_AIR) {
                T.move(x, y, x, y + 1);
                float vx = (float)((int)(c.D() % 10) - 5) / 20.0f;
                float vy = (float)(-((int)(c.D() % 2) + 3)) / 10.0f + 1.5f;
                spawn_one(c, 1, x, y + 1, t, vx, vy);
            } else {
                T.move(x, y, x, y + 1);
                if (c.D() % 2 == 0) t.fl |= MOVED;
                T.put(x, y + 1, t);
                T.setvis(x, y + 1);
            }
            if (c.D() % 2 == 0) {
                if (x > 0 && T.type(x - 1, y + 1) == T_SAND) {
                    if (c.D() % 2 == 0) T.set_moved(x - 1, y + 1, true);
                }
                if (x < T.W - 1 && T.type(x + 1, y + 1) == T_SAND) {
                    if (c.D() % 2 == 0) T.set_moved(x + 1, y + 1, true);
                }
            }
        }
    } else if (TL::kF32 && type == T_SOUP) {
        rule_a_soup_f32(T, c, t, x, y);
    } else if (type == T_SOUP) {  // world.cpp:1269-1567
        if (t.sc == 0) return;
        if (t.sc < Q_MINV) {
            led_add(c, LED_DF, t.id, t.sc);
            t.sc = 0;
            T.put_delta(x, y, t);
            return;
        }
        if (t.sc > Q_FREEFALL && T.type(x, y + 1) == T_AIR && T.type(x, y + 2) == T_AIR &&
            T.type(x, y + 3) == T_AIR && T.type(x, y + 4) == T_AIR) {  // world.cpp:1283-1305
            led_add(c, LED_DF, t.id, T.df_load(x, y));
            T.set_nothing(x, y);
            int n = t.sc >> 18;
            if (n < 1) n = 1;
            led_add(c, LED_CN, t.id, n - 1);
            c.ev->n = n;
            c.ev->kind = 2;
            c.ev->x = x;
            c.ev->y = y + 1;
            c.ev->id = t.id;
            c.ev->fl = 0;
            c.ev->col = t.col;
            c.ev->sc = t.sc;
            if (TL::kTemp) c.ev->tp = T.tp_load(x, y);
            c.ev->ck = c.key();
            c.ev->k0 = c.k;
            c.k += 2 * n;
            return;
        }
        if (t.fl & MOVED) return;
        const int32_t start = t.sc;
        int32_t rem = t.sc;
        const int bid = T.id(x, y + 1);
        const int bT = mt_type(ma[bid]);
        const bool airBelow = bT == T_AIR;
        if ((airBelow && c.iter <= 2) || bid == (int)t.id) {
            int32_t dst = (bT == T_SOUP) ? T.sc(x, y + 1) : 0;
            soup_flow(T, c, t, rem, clampflow(vflow(start, dst) - dst, start), bT, x, y, 0, 1);
        } else if (c.iter == 0 && bT == T_SOUP && bid != (int)t.id) {
            if (c.D() % 10 == 0) {
                t.df += T.df_load(x, y);  // the cell leaves its position: carry the whole diff
                const int16_t tv = T.tp_load(x, y);
                T.move(x, y, x, y + 1);
                T.put(x, y + 1, t);
                T.tp_store(x, y + 1, tv);
                return;
            }
        }
        if (rem < Q_MINV) {
            t.df -= rem;
            led_add(c, LED_DF, t.id, rem);
            T.put_delta(x, y, t);
            return;
        }
        const int lid = T.id(x - 1, y);
        const int lT = mt_type(ma[lid]);
        const bool canL = (lT == T_AIR || lid == (int)t.id) && !airBelow;
        const int rid = T.id(x + 1, y);
        const int rT = mt_type(ma[rid]);
        const bool canR = (rT == T_AIR || rid == (int)t.id) && !airBelow;
        if (canL) {
            int32_t dst = (lT == T_SOUP) ? T.sc(x - 1, y) : 0;
            soup_flow(T, c, t, rem, clampflow(canR ? (rem - dst) / 3 : (rem - dst) / 2, rem), lT, x, y, -1, 0);
        }
        if (rem < Q_MINV) {
            t.df -= rem;
            led_add(c, LED_DF, t.id, rem);
            T.put_delta(x, y, t);
            return;
        }
        if (canR) {
            int32_t dst = (rT == T_SOUP) ? T.sc(x + 1, y) : 0;
            soup_flow(T, c, t, rem, clampflow((rem - dst) / 2, rem), rT, x, y, 1, 0);
        }
        if (rem < Q_MINV) {
            t.df -= rem;
            led_add(c, LED_DF, t.id, rem);
            T.put_delta(x, y, t);
            return;
        }
        const int tid = T.id(x, y - 1);
        const int tT = mt_type(ma[tid]);
        if (tT == T_AIR || tid == (int)t.id) {
            int32_t dst = (tT == T_SOUP) ? T.sc(x, y - 1) : 0;
            soup_flow(T, c, t, rem, clampflow(rem - vflow(rem, dst), rem), tT, x, y, 0, -1);
        } else if (c.iter == 0 && tT == T_SOUP && tid != (int)t.id) {
            if (c.D() % 10 == 0) {
                t.df += T.df_load(x, y);
                const int16_t tv = T.tp_load(x, y);
                T.move(x, y, x, y - 1);
                T.put(x, y - 1, t);
                T.tp_store(x, y - 1, tv);
                return;
            }
        }
        if (rem < Q_MINV) {
            t.df -= rem;
            led_add(c, LED_DF, t.id, rem);
            T.put_delta(x, y, t);
            return;
        }
        if (start == rem) {  // world.cpp:1472-1483
            uint8_t s = t.fl & SETTLE_MASK;
            if (s < SETTLE_MASK) s++;
            t.fl = (uint8_t)((t.fl & ~SETTLE_MASK) | s);
            if (s >= 10) t.fl |= MOVED;
        } else {
            if (tT == T_SOUP) T.set_moved(x, y - 1, false);
            if (bT == T_SOUP) T.set_moved(x, y + 1, false);
            if (lT == T_SOUP) T.set_moved(x - 1, y, false);
            if (rT == T_SOUP) T.set_moved(x + 1, y, false);
        }
        T.put_delta(x, y, t);
        // WATER on LAVA, world.cpp:1519-1537
        if ((int)t.id == c.id_water && T.id(x, y + 1) == c.id_lava) {
            Cell st = create_tile(c, c.id_steam);
            led_swap(c, t.id, (long long)t.sc + T.df_load(x, y), st.id, (long long)st.sc);
            T.put_new(x, y, st, mt);
            Cell ob = create_tile(c, c.id_obsidian);
            led_replace_at(T, c, x, y + 1, ob);
            T.put_new(x, y + 1, ob, mt);
            T.setvis(x, y + 1);
            for (int xx = -1; xx <= 1; xx++)
                for (int yy = 0; yy <= 2; yy++) {
                    if (T.id(x + xx, y + yy) == c.id_lava) {
                        Cell o2 = create_tile(c, c.id_obsidian);
                        led_replace_at(T, c, x + xx, y + yy, o2);
                        T.put_new(x + xx, y + yy, o2, mt);
                        T.setvis(x + xx, y + yy);
                    }
                }
            return;
        }
    } else if (type == T_GAS) {  // world.cpp:1569-1585
        const int above = T.type(x, y - 1);
        const int aboveL = T.type(x - 1, y - 1);
        const int aboveR = T.type(x + 1, y - 1);
        if (above == T_AIR && !((aboveL == T_AIR || aboveR == T_AIR) && c.D() % 2 == 0)) {
            T.move(x, y, x, y - 1);
            T.put(x, y - 1, t);
            T.setvis(x, y - 1);
        }
    }
}

// ----------------------------------------------------------------- sweep B
// dfv: the cell's pending fluid diff, read when the sub-phase began (no other cell
// of the sub-phase writes it)
template <class TL>
__device__ __forceinline__ void rule_b(const TL &T, Ctx &c, int x, int y, int32_t dfv) {
    if (T.vis(x, y)) return;  // world.cpp:1597
    const uint32_t *ma = T.ma;
    const float *md = T.md;
    const int sid = T.id(x, y);
    const uint32_t a = ma[sid];
    const int type = mt_type(a);
    if (type != T_SAND && type != T_SOUP && type != T_GAS) return;
    c.at(x, y);
    if (type == T_SAND) {  // world.cpp:1602-1727
        const int i = T.li(x, y);
        const uint8_t fl0 = T.s_fl[i] & (uint8_t)~VISITED;
        const bool canL = can_sink(ma, md, T.id(x - 1, y + 1), sid);
        const bool canR = can_sink(ma, md, T.id(x + 1, y + 1), sid);
        bool stopped = !(fl0 & MOVED);
        const int slip = mt_slip(a);
        if (stopped) {
            // world.cpp:1619-1627 over the AIR snapshot taken when sweep B began
            const int drop = __popc(T.air10(x - 1, y + 1) | T.air10(x + 1, y + 1));
            int d = drop + 1 - mt_stab(a);
            if (d > 0) {
                int chance = 1000 / d;
                if (chance < 1000) {
                    if (c.D() % (uint32_t)chance == 0) {
                        stopped = false;
                        T.set_moved(x, y, true);
                    }
                }
            }
        }
        if (stopped || !(canL || canR)) {
            T.set_moved(x, y, false);
            return;
        }
        // the moving cell as it was when its turn began
        Cell t;
        t.id = (uint16_t)sid;
        t.fl = fl0;
        t.sc = T.s_sc[i];
        t.col = T.s_col[i];
        t.df = 0;
        const bool shouldMove = (slip > 0) ? (c.D() % (uint32_t)(2 * slip) != 0) : true;
        if (shouldMove && (canL || canR)) {
            if (c.D() % 2 == 0) {
                if (T.type(x, y + 1) == T_SAND) {
                    if (c.D() % 2 == 0) T.set_moved(x, y + 1, true);
                }
            }
        }
        if (shouldMove && canL && (!canR || c.D() % 2 == 0)) {
            if (T.type(x - 1, y) == T_AIR) {
                T.move(x - 1, y, x - 1, y + 1);
                T.setvis(x - 1, y);
                T.set_nothing(x, y);
            } else {
                T.move(x, y, x - 1, y + 1);
                T.setvis(x, y);
            }
            if (slip > 0 && c.D() % (uint32_t)(20 * slip) == 0) t.fl &= (uint8_t)~MOVED;
            T.put(x - 1, y + 1, t);
            T.setvis(x - 1, y + 1);
        } else if (shouldMove && canR) {
            if (T.type(x + 1, y) == T_AIR) {
                T.move(x + 1, y, x + 1, y + 1);
                T.set_nothing(x, y);
            } else {
                T.move(x, y, x + 1, y + 1);
                T.setvis(x, y);
            }
            if (slip > 0 && c.D() % (uint32_t)(20 * slip) == 0) t.fl &= (uint8_t)~MOVED;
            T.put(x + 1, y + 1, t);
            T.setvis(x + 1, y + 1);
        } else {
            T.set_moved(x, y, false);
        }
    } else if (TL::kF32 && type == T_SOUP) {  // world.cpp:1728-1745 in f32
        Cell t = T.get_active(x, y);
        const float a = __fadd_rn(__int_as_float(t.sc), __int_as_float(dfv));
        t.sc = __float_as_int(a);
        t.df = __float_as_int(0.0f);
        if (a < F_MINV) {
            led_add(c, LED_DN, t.id, 1);
            T.set_nothing(x, y);
            T.setvis(x, y);
        } else {
            T.put(x, y, t);
            T.setvis(x, y);
        }
    } else if (type == T_SOUP) {  // world.cpp:1728-1745
        Cell t = T.get_active(x, y);
        t.sc += dfv;
        t.df = 0;
        if (t.sc < Q_MINV) {
            led_add(c, LED_DN, t.id, 1);
            led_add(c, LED_DF, t.id, t.sc);
            T.set_nothing(x, y);
            T.setvis(x, y);
        } else {
            T.put(x, y, t);
            T.setvis(x, y);
        }
    } else {  // GAS, world.cpp:1799-1818
        const int aboveL = T.type(x - 1, y - 1);
        const int aboveR = T.type(x + 1, y - 1);
        if (aboveL != T_AIR && aboveR != T_AIR) return;
        const Cell t = T.get_active(x, y);
        if (aboveL == T_AIR && !(aboveR == T_AIR && c.D() % 2 == 0)) {
            T.move(x, y, x - 1, y - 1);
            T.put(x - 1, y - 1, t);
            T.setvis(x - 1, y - 1);
        } else if (aboveR == T_AIR) {
            T.move(x, y, x + 1, y - 1);
            T.put(x + 1, y - 1, t);
            T.setvis(x + 1, y - 1);
        }
    }
}

// ----------------------------------------------------------------- sweep C
template <class TL>
__device__ __forceinline__ void rule_c(const TL &T, Ctx &c, int x, int y) {
    if (T.vis(x, y)) return;  // world.cpp:1831
    const int sid = T.id(x, y);
    if (mt_type(T.ma[sid]) != T_GAS) return;
    c.at(x, y);
    // world.cpp:1862-1889
    const int l = T.type(x - 1, y);
    const int r = T.type(x + 1, y);
    if (l != T_AIR && r != T_AIR && sid != c.id_steam) return;
    const Cell t = T.get_active(x, y);
    if (l == T_AIR && !(r == T_AIR && c.D() % 2 == 0)) {
        T.move(x, y, x - 1, y);
        T.put(x - 1, y, t);
        T.setvis(x - 1, y);
    } else if (r == T_AIR) {
        T.move(x, y, x + 1, y);
        T.put(x + 1, y, t);
        T.setvis(x + 1, y);
    } else if (sid == c.id_steam) {
        if (c.D() % 10 == 0) {
            Cell wt = create_tile(c, c.id_water);
            led_swap(c, t.id, 0, wt.id, (long long)wt.sc);
            T.put_new(x, y, wt, c.mt);
        }
    }
}

// --------------------------------------------------------------- lattices
// (Px, Py) per sweep and chunk mode; see the oracle's lattice() for the derivation.
__device__ __forceinline__ void lattice(int sweep, int mode, int &px, int &py) {
    if (sweep == 0) {
        if (mode == 2) {
            px = 11;
            py = 11;
        } else if (mode == 1) {
            px = 5;
            py = 7;
        } else {
            px = 3;
            py = 6;
        }
    } else if (sweep == 1) {
        // the friction pillar reads the sweep-B snapshot, so only rows y-1..y+1 are live
        px = 3;
        py = 3;
    } else {
        px = 3;
        py = 1;
    }
}

// block-wide exclusive scan of one int per thread; returns the exclusive prefix,
// *total = block sum. scratch: >= 33 ints of shared memory.
__device__ __forceinline__ int block_excl_scan(int v, int *scratch, int *total) {
    int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
    int inc = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int n = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += n;
    }
    if (lane == 31) scratch[wid] = inc;
    __syncthreads();
    if (wid == 0) {
        int s = (lane < nw) ? scratch[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            int n = __shfl_up_sync(0xffffffffu, s, o);
            if (lane >= o) s += n;
        }
        if (lane < nw) scratch[lane] = s;  // inclusive warp totals
    }
    __syncthreads();
    int before = (wid > 0) ? scratch[wid - 1] : 0;
    *total = scratch[nw - 1];
    __syncthreads();
    return before + inc - v;
}

// write the particles of one spawn event (world.cpp:1110-1119,1222,1298)
template <bool TEMP, bool F32>
static __device__ __noinline__ void emit_spawns(const WorldDev &w, const SpawnEv &ev, uint32_t cp, uint32_t rank0,
                                                int base) {
    int32_t base_amt = 0, extra = 0;
    if (ev.kind == 2) {
        if (F32) {
            // f32 amt = tile.fluidAmount / n for every particle (world.cpp:1292)
            base_amt = __float_as_int(__fdiv_rn(__int_as_float(ev.sc), (float)ev.n));
        } else {
            base_amt = ev.sc / ev.n;
            extra = ev.sc % ev.n;
        }
    }
    for (int i = 0; i < ev.n; i++) {
        int slot = base + i;
        if (slot >= w.stage_cap) {
            atomicOr(w.err, ERR_SPAWN_CAP);
            return;
        }
        SpawnRec r;
        r.cp = cp;
        r.rank = rank0 + (uint32_t)i;
        r.x = (float)ev.x;
        r.y = (float)ev.y;
        r.id = ev.id;
        r.colour = ev.col;
        r.temp = (TEMP && ev.kind == 2) ? ev.tp : (int16_t)0;
        r.pad = 0;
        if (ev.kind == 1) {
            r.vx = ev.vx;
            r.vy = ev.vy;
            r.ay = 0.1f;
            r.scalar = ev.sc;
            r.flags = ev.fl;
            r.bits = 0;
            r.lifetime = 0;
            r.fade = 60;
        } else if (ev.kind == 3) {
            r.vx = ev.vx;
            r.vy = ev.vy;
            r.ay = 0.01f;
            r.scalar = ev.sc;
            r.flags = ev.fl;
            r.bits = 2;
            r.lifetime = 30;
            r.fade = 10;
        } else {
            uint32_t d0 = draw_k(ev.ck, ev.k0 + 2u * (uint32_t)i), d1 = draw_k(ev.ck, ev.k0 + 2u * (uint32_t)i + 1u);
            r.vx = (float)((int)(d0 % 10) - 5) / 30.0f;
            r.vy = (float)(-((int)(d1 % 2) + 3)) / 10.0f + 1.0f;
            r.ay = 0.1f;
            r.scalar = base_amt + (i < extra ? 1 : 0);
            r.flags = 0;
            r.bits = 0;
            r.lifetime = 0;
            r.fade = 60;
        }
        w.stage[slot] = r;
    }
}

// -------------------------------------------------------------- the kernel
// shared memory besides the tile planes
template <int NT>
struct SmemHeadT {
    uint32_t ma[MAXMAT];
    float md[MAXMAT];
    long long led[LED_ROWS * 64];
    int scan[40];
    uint8_t mreact[MAXMAT];
    int cnt[NT];  // sweep-A spawns per enumeration index, then their ranks
    uint32_t air[(128 + 2) * 5];  // sweep-B pillar snapshot (chunk edge <= 128)
    // CTA pair: what the partner wrote here: [0..1] its chunk flags, [2..3] its spawn
    // count of a sweep-A sub-phase (alternate slots)
    uint32_t xch[4];
    uint32_t vote[32];  // each warp's activity (bit 0) and fire (bit 1) votes of the chunk-pass
};
using SmemHead = SmemHeadT<CP_THREADS>;

// items: (world << 20) | chunk slot within the colour; iter, tk select the pass.
// FUSED: every pass of the tick in one launch (iter, tk, items and n_items unused;
// ft holds the work). CTAs take chunk-passes in pass order from a ticket counter; a
// chunk-pass starts when the last earlier pass of each chunk of its 3 x 3
// neighbourhood is done (a chunk-pass reads and writes its chunk plus a halo of at
// most 5 cells, and each pass's chunks tile the zone, so these are all the
// chunk-passes it can conflict with, directly or through a chain), and publishes
// its own completion with a release store. A CTA only waits for tickets taken
// before its own by CTAs that are running, so the launch cannot deadlock whatever
// its grid; each wait is also bounded (ERR_TIMEOUT). The last CTA to finish clears
// the flags and the counters for the next launch.
// SEQ: the reference's own order inside each chunk (bottom row first, left to right,
// sweep by sweep; world.cpp:1084-1087, 1589, 1823), with the same rules, run as a
// wavefront of one thread per chunk row (see sweeps_seq)
// PAIR: each chunk is split over the two CTAs of a cluster, 512 threads each: rank 0
// updates the top half of its rows, rank 1 the bottom half, each staging its half
// plus the rows its rules reach (the shared rows are kept equal by mirrored writes)
// and writing back its own rows; sub-phases end with a cluster barrier. A chunk's
// sub-phases then run on two SMs, and an SM holds halves of two chunks whose
// barriers interleave.
template <int HALO, bool TEMP, bool SEQ, bool F32, bool PAIR = false, bool FUSED = false>
__global__ void __launch_bounds__(PAIR ? CP_THREADS / 2 : CP_THREADS, PAIR ? 2 : 1)
    k_colour_pass(const WorldDev *__restrict__ worlds, const uint32_t *__restrict__ items, int n_items, int iter_arg,
                  int tk_arg, const MatTable *__restrict__ mt, const FusedTick ft) {
    static_assert(!(PAIR && SEQ), "the reference order runs a chunk in one CTA");
    static_assert(!(FUSED && (PAIR || SEQ)), "the fused tick runs partitioned chunk-passes in one CTA each");
    constexpr int T = PAIR ? CP_THREADS / 2 : CP_THREADS;
    using Head = SmemHeadT<T>;
    extern __shared__ __align__(16) unsigned char smem[];
    Head &S = *reinterpret_cast<Head *>(smem);
    // the planes start on a 128-byte boundary of the shared window (TMA destinations)
    const uint32_t sbase = smem_addr(smem);
    unsigned char *planes = smem + (((sbase + (uint32_t)sizeof(Head) + 127u) & ~127u) - sbase);
    // TMA staging of the 4-byte planes: the partitioned order with a 2-cell halo, in
    // worlds with tensor maps (one phase of s_tma_bar per staged chunk-pass)
    constexpr bool kTma = HALO == 2 && !PAIR && !SEQ;
    __shared__ __align__(8) uint64_t s_tma_bar;
    uint32_t tma_phase = 0;

    const int tid = threadIdx.x;
    const int rank = PAIR ? (int)cluster_rank() : 0;
    int npass = 0;  // chunks taken so far (the same count in both CTAs of a pair)
    for (int i = tid; i < MAXMAT; i += T) {
        S.ma[i] = (i < mt->n) ? mt->a[i] : 0u;
        S.md[i] = (i < mt->n) ? mt->density[i] : 0.f;
        S.mreact[i] = (uint8_t)((i < mt->n) ? mt->n_react[i] : 0);
    }
    for (int i = tid; i < LED_ROWS * 64; i += T) S.led[i] = 0;
    Ctx c;
    SpawnEv ev_store;  // outside the context (see Ctx::ev)
    c.ev = &ev_store;
    c.iter = iter_arg;
    c.mt = mt;
    c.led_s = S.led;
    c.ma = S.ma;
    c.mreact = S.mreact;
    c.id_fire = mt->id_fire;
    c.id_water = mt->id_water;
    c.id_lava = mt->id_lava;
    c.id_steam = mt->id_steam;
    c.id_obsidian = mt->id_obsidian;
    // interactions exist exactly when the launch runs the 5-cell halo (tick_halo)
    c.has_inter = HALO == 5;
    c.f32 = F32;
    const int id_solid = mt->id_solid, id_air = mt->id_air;
    if (kTma && tid == 0) mbar_init(&s_tma_bar, 1);
    FSE_PT_DECL
    __syncthreads();

    int iter = iter_arg, tk = tk_arg;
    long long *led_g_last = nullptr;

    const int wstart = PAIR ? (int)(blockIdx.x >> 1) : (int)blockIdx.x;
    const int wstride = PAIR ? (int)(gridDim.x >> 1) : (int)gridDim.x;
    // FUSED: the ticket taken, and the completion flag this CTA publishes before it
    // takes the next one (kept in shared memory: the tile code needs the registers)
    __shared__ int s_ticket;
    __shared__ uint32_t *s_done_flag;
    __shared__ uint32_t s_done_value;
    if (FUSED && tid == 0) s_done_flag = nullptr;
    for (int it = wstart;; it += wstride) {
        uint32_t item;
        if constexpr (FUSED) {
            if (tid == 0) {
                if (s_done_flag) {
                    __threadfence();
                    st_release_gpu(s_done_flag, s_done_value);
                    s_done_flag = nullptr;
                }
                s_ticket = (int)atomicAdd(&worlds[0].sched[0], 1u);
            }
            __syncthreads();
            int t = s_ticket;
            const int per_iter = ft.n[0] + ft.n[1] + ft.n[2] + ft.n[3];
            if (t >= per_iter * (ft.passes / 4)) break;
            iter = t / per_iter;
            t -= iter * per_iter;
            // the colour and the index within it (no dynamic indexing of the parameters)
            const uint32_t *li = ft.items[0];
            tk = 0;
            if (t >= ft.n[0]) {
                t -= ft.n[0];
                tk = 1;
                li = ft.items[1];
                if (t >= ft.n[1]) {
                    t -= ft.n[1];
                    tk = 2;
                    li = ft.items[2];
                    if (t >= ft.n[2]) {
                        t -= ft.n[2];
                        tk = 3;
                        li = ft.items[3];
                    }
                }
            }
            item = __ldg(&li[t]);
        } else {
            if (it >= n_items) break;
            item = __ldg(&items[it]);
        }
        const int ox = tk % 2, oy = 1 - tk / 2;
        c.iter = iter;
        // the last chunk-pass's generic accesses to the planes come before this one's
        // tensor copies into them
        if constexpr (kTma) fence_proxy_async_smem();
        {
            // the world's descriptor into shared memory, 8 bytes a thread (one thread
            // copying it load by load took ~5% of a chunk-pass)
            static_assert(sizeof(WorldDev) % 8 == 0, "the descriptor is copied in 8-byte words");
            constexpr int NW8 = (int)(sizeof(WorldDev) / 8);
            static_assert(NW8 <= T, "one word per thread");
            if (tid < NW8)
                reinterpret_cast<uint2 *>(&s_w)[tid] =
                    __ldg(reinterpret_cast<const uint2 *>(&worlds[item >> 20]) + tid);
        }
        __syncthreads();
        FSE_PT(0)
        const WorldDev &w = s_w;
        const int slot = (int)(item & 0xFFFFF);
        if constexpr (FUSED) {
            // wait until the chunk-passes this one depends on are done: for each chunk
            // of the 3 x 3 neighbourhood, its last pass before this one
            const int nbq = (w.nCy - oy + 1) / 2;
            const int a = ox + 2 * (slot / nbq), b = oy + 2 * (slot % nbq);
            const int q = iter * 4 + tk;
            if (tid < 9) {
                const int a2 = a + tid % 3 - 1, b2 = b + tid / 3 - 1;
                if (a2 >= 0 && a2 < w.nCx && b2 >= 0 && b2 < w.nCy) {
                    const int tn = (a2 & 1) + 2 * (1 - (b2 & 1));
                    const int p = tn < tk ? iter * 4 + tn : (iter - 1) * 4 + tn;
                    if (p >= 0) {
                        const uint32_t *f = &w.cdone[(size_t)b2 * w.nCx + a2];
                        // sched[2]: a wait of this launch gave up; the others do not wait
                        volatile uint32_t *abort = &worlds[0].sched[2];
                        if (ld_acquire_gpu(f) <= (uint32_t)p && !*abort) {
                            const unsigned long long t0 = global_ns();
                            while (ld_acquire_gpu(f) <= (uint32_t)p && !*abort) {
                                if (global_ns() - t0 > FUSED_WAIT_NS) {
                                    atomicOr(w.err, ERR_TIMEOUT);
                                    *abort = 1u;
                                    break;
                                }
                                __nanosleep(64);
                            }
                        }
                    }
                }
            }
            if (tid == 0) {
                s_done_flag = &w.cdone[(size_t)b * w.nCx + a];
                s_done_value = (uint32_t)q + 1u;
            }
            __syncthreads();
        }
        if (led_g_last != w.ledger && led_g_last != nullptr) {
            // flush the shared ledger before switching worlds
            for (int i = tid; i < LED_ROWS * 64; i += T) {
                long long v = S.led[i];
                if (v) atomicAdd((unsigned long long *)&led_g_last[(i / 64) * MAXMAT + (i % 64)], (unsigned long long)v);
                S.led[i] = 0;
            }
            __syncthreads();
        }
        led_g_last = w.ledger;
        if (iter >= w.cell_iter) {
            __syncthreads();
            continue;
        }
        const int C = w.C, W = w.W, H = w.H;
        const int nb = (w.nCy - oy + 1) / 2;
        const int cx = w.zx + (ox + 2 * (slot / nb)) * C, cy = w.zy + (oy + 2 * (slot % nb)) * C;
        const uint32_t cp = (uint32_t)((iter * 4 + tk) * w.max_slots + slot);

        // the chunk rows this CTA updates, [o0, o1)
        const int half = C / 2;
        const int o0 = PAIR ? rank * half : 0, o1 = PAIR ? (rank ? C : half) : C;
        const int own = o1 - o0;
        TileData Tl;
        const bool tma = kTma && w.tmap != nullptr;
        // with TMA the rows start on a 16-byte boundary and are tma_tile_width wide
        Tl.RW = tma ? tma_tile_width(C) : C + 2 * HALO;
        Tl.RHF = own + 2 * HALO;
        Tl.RHI = own + HALO + 10;
        Tl.x0 = tma ? ((cx - HALO) & ~3) : cx - HALO;
        Tl.y0 = cy + o0 - HALO;
        Tl.W = W;
        Tl.H = H;
        Tl.ma = S.ma;
        Tl.md = S.md;
        Tl.df = w.df;
        Tl.tp = w.tp;
        Tl.id_solid = id_solid;
        Tl.id_air = id_air;
        Tl.s_air = S.air;
        Tl.ax0 = cx - 1;
        Tl.ay0 = cy + o0 + 1;
        Tl.aw = C + 2;
        const int nid = Tl.RW * Tl.RHI, nfull = Tl.RW * Tl.RHF;
        Tl.s_sc = (int32_t *)planes;
        Tl.s_col = (uint32_t *)(Tl.s_sc + ((nfull + 31) & ~31));  // 128-byte aligned
        Tl.s_id = (uint16_t *)(Tl.s_col + nfull);
        Tl.s_fl = (uint8_t *)(Tl.s_id + ((nid + 1) & ~1));
        if constexpr (PAIR) {
            // the partner's planes lie at the same offsets of its shared memory
            const uint32_t pr = (uint32_t)(rank ^ 1);
            Tl.p_id = mapa_rank(smem_addr(Tl.s_id), pr);
            Tl.p_fl = mapa_rank(smem_addr(Tl.s_fl), pr);
            Tl.p_sc = mapa_rank(smem_addr(Tl.s_sc), pr);
            Tl.p_col = mapa_rank(smem_addr(Tl.s_col), pr);
            Tl.py0 = cy + (rank ? 0 : half) - HALO;
        }

        // ---- stage the tile, one warp per row. The 4-byte planes go straight to
        // shared memory, as two tensor copies (TMA) or with cp.async; ids and flags
        // are loaded a row at a time, all loads of a row in flight together. The
        // chunk's ids decide the skip and the lattice mode.
        if (tma && tid == 0) {
            const char *tm = static_cast<const char *>(w.tmap);
            mbar_expect_tx(&s_tma_bar, 2u * (uint32_t)nfull * 4u);
            tma_load_2d(Tl.s_sc, tm, Tl.x0, Tl.y0, &s_tma_bar);
            tma_load_2d(Tl.s_col, tm + 128, Tl.x0, Tl.y0, &s_tma_bar);
        }
        int active = 0, fire = 0;
        {
            const int lane = tid & 31, wid = tid >> 5;
            constexpr int NW = T / 32;
            for (int r = wid; r < Tl.RHI; r += NW) {
                const int gy = Tl.y0 + r;
                const bool rin = (unsigned)gy < (unsigned)H;
                const size_t gb = (size_t)gy * W;
                const bool full = r < Tl.RHF;
                uint16_t v[MAXRW / 32];
                uint8_t f[MAXRW / 32];
#pragma unroll
                for (int k = 0; k < MAXRW / 32; k++) {
                    const int lx = lane + 32 * k, gx = Tl.x0 + lx;
                    v[k] = (uint16_t)id_solid;
                    f[k] = 0;
                    if (lx < Tl.RW && rin && (unsigned)gx < (unsigned)W) {
                        v[k] = w.id[gb + gx];
                        if (full) f[k] = w.fl[gb + gx];
                    }
                }
                if (full && !tma) {
#pragma unroll
                    for (int k = 0; k < MAXRW / 32; k++) {
                        const int lx = lane + 32 * k, gx = Tl.x0 + lx;
                        if (lx >= Tl.RW) continue;
                        const int i = r * Tl.RW + lx;
                        if (rin && (unsigned)gx < (unsigned)W) {
                            cp_async4(&Tl.s_sc[i], &w.sc[gb + gx]);
                            cp_async4(&Tl.s_col[i], &w.col[gb + gx]);
                        } else {
                            Tl.s_sc[i] = 0;
                            Tl.s_col[i] = 0xff0000u;
                        }
                    }
                }
#pragma unroll
                for (int k = 0; k < MAXRW / 32; k++) {
                    const int lx = lane + 32 * k, gx = Tl.x0 + lx;
                    if (lx >= Tl.RW) continue;
                    const int i = r * Tl.RW + lx;
                    Tl.s_id[i] = v[k];
                    if (full) Tl.s_fl[i] = f[k];
                    if (gx >= cx && gx < cx + C && gy >= cy + o0 && gy < cy + o1 && rin && gx < W) {
                        if (mt_iter(S.ma[v[k]]) > c.iter) active = 1;
                        if ((int)v[k] == c.id_fire) fire = 1;
                    }
                }
            }
        }
        if (tma) {
            // the tensor copies have landed (a bounded wait); cells outside the world
            // read as zero there and take the outside colour
            long long spins = 0;
            while (!mbar_try_wait(&s_tma_bar, tma_phase)) {
                if (++spins > (1LL << 26)) {
                    atomicOr(w.err, ERR_TIMEOUT);
                    break;
                }
            }
            tma_phase ^= 1u;
            if (Tl.x0 < 0 || Tl.y0 < 0 || Tl.x0 + Tl.RW > W || Tl.y0 + Tl.RHF > H) {
                for (int i = tid; i < nfull; i += T) {
                    const int r = i / Tl.RW, gx = Tl.x0 + (i - r * Tl.RW), gy = Tl.y0 + r;
                    if ((unsigned)gx >= (unsigned)W || (unsigned)gy >= (unsigned)H) Tl.s_col[i] = 0xff0000u;
                }
            }
        }
        if constexpr (PAIR) {
            active = __syncthreads_or(active);
            fire = __syncthreads_or(fire);
            cp_async_wait_all();
            // the pair decides together whether the chunk runs and with which lattice
            const int slot_x = npass & 1;
            if (tid == 0) st_cluster_u32(mapa_rank(smem_addr(&S.xch[slot_x]), (uint32_t)(rank ^ 1)),
                                         (uint32_t)(active | (fire << 1)));
            cluster_sync();
            const uint32_t o = S.xch[slot_x];
            active |= (int)(o & 1u);
            fire |= (int)((o >> 1) & 1u);
        } else {
            // the copies are in and the chunk's votes are taken with one barrier: each
            // warp's leader writes its warp's votes, every warp ORs the 32 words after
            cp_async_wait_all();
            const unsigned bits = (__any_sync(0xffffffffu, active) ? 1u : 0u) | (__any_sync(0xffffffffu, fire) ? 2u : 0u);
            if ((tid & 31) == 0) S.vote[tid >> 5] = bits;
            __syncthreads();
            const unsigned vv = __reduce_or_sync(0xffffffffu, (tid & 31) < T / 32 ? S.vote[tid & 31] : 0u);
            active = (int)(vv & 1u);
            fire = (int)((vv >> 1) & 1u);
        }
        npass++;
        FSE_PT(1)
        if (!active) {
            // every chunk cell has iterations <= iter: the pass only marks cells visited
            if constexpr (SEQ) {
                if (tid < w.cp_rows) w.cp_count[cp * w.cp_rows + tid] = 0;
            } else if (tid == 0 && rank == 0) {
                w.cp_count[cp] = 0;
            }
            __syncthreads();
            continue;
        }
        FSE_PT(2)

        const int mode = c.has_inter ? 2 : (fire ? 1 : 0);
        const int cw = min(C, W - cx), chh = min(C, H - cy);
        int running = 0;  // spawns emitted so far by this chunk-pass
        int nsub = 0;     // sweep-A sub-phases so far (CTA pair: alternate exchange slots)
        c.led_g = w.ledger;
        // The reference's order as a wavefront: thread k updates chunk row k counted
        // from the bottom (the row world.cpp's loop takes k-th), cell dx at step
        // dx + s*k. A cell reads and writes at most RX columns to either side
        // (RX = 1; 2 with fire; 5 with interactions, whose boxes lie right of the
        // cell), so two cells whose accesses meet are at least 2*RX+1 = s steps apart
        // in the reference's order's direction: every cell still sees exactly the
        // cells the sequential loop would have updated before it, and no two cells
        // of one step touch the same cell. Each row ranks its own spawns.
        auto sweeps_seq = [&](const auto &Tl) {
            const int s = mode == 2 ? 11 : (mode == 1 ? 5 : 3);
            const int k = tid, dy = chh - 1 - tid;
            const bool row = k < chh;
            int spawned = 0;
            for (int sweep = 0; sweep < 3; sweep++) {
                c.pk = pass_key(w.seed, *w.tick, (uint32_t)(c.iter * 3 + sweep));
                const int steps = cw + s * (chh - 1);
                for (int t = 0; t < steps; t++) {
                    const int dx = t - s * k;
                    if (row && dx >= 0 && dx < cw) {
                        const int x = cx + dx, y = cy + dy;
                        if (sweep == 0) {
                            c.ev->n = 0;
                            rule_a(Tl, c, x, y);
                            if (c.ev->n > 0) {
                                const int base = atomicAdd(w.stage_count, c.ev->n);
                                emit_spawns<TEMP, F32>(w, *c.ev, cp * (uint32_t)w.cp_rows + (uint32_t)k, (uint32_t)spawned,
                                                  base);
                                spawned += c.ev->n;
                            }
                        } else if (sweep == 1) {
                            rule_b(Tl, c, x, y, w.df[(size_t)y * W + x]);
                        } else {
                            rule_c(Tl, c, x, y);
                        }
                    }
                    __syncthreads();
                }
            }
            if (tid < w.cp_rows) w.cp_count[cp * w.cp_rows + tid] = spawned;
        };
        auto sweeps = [&](const auto &Tl) {
        for (int sweep = 0; sweep < 3; sweep++) {
            c.pk = pass_key(w.seed, *w.tick, (uint32_t)(c.iter * 3 + sweep));
            if (sweep == 1) {
                // AIR snapshot for the friction pillar: columns cx-1..cx+C, rows cy+1..cy+C+9
                for (int task = tid; task < (C + 2) * 5; task += T) {
                    const int sx = task / 5, wi = task - sx * 5;
                    uint32_t bits = 0;
                    for (int b = 0; b < 32; b++) {
                        const int sy = wi * 32 + b;
                        if (sy < own + 9) {
                            const int gx = cx - 1 + sx, gy = Tl.ay0 + sy;
                            if (Tl.inw(gx, gy) && Tl.type(gx, gy) == T_AIR) bits |= 1u << b;
                        }
                    }
                    S.air[task] = bits;
                }
                __syncthreads();
            }
            int px, py;
            lattice(sweep, mode, px, py);
            for (int ry = py - 1; ry >= 0; ry--) {
                // this CTA's rows of the sub-phase: dyb, dyb + py, ... below o1
                const int dyb = ry + (o0 > ry ? (o0 - ry + py - 1) / py * py : 0);
                const int ny = dyb < o1 ? (o1 - dyb + py - 1) / py : 0;
                for (int rx = 0; rx < px; rx++) {
                    const int nx = (C - rx + px - 1) / px;
                    const int total = nx * ny;
                    const float rnx = __frcp_rn((float)nx);
                    if (sweep == 0) {
                        // sweep A sub-phases have at most 43 x 22 <= T cells: one per thread,
                        // so every spawn event stays in its thread until it is ranked
                        const int e = tid;
                        c.ev->n = 0;
                        S.cnt[tid] = 0;
                        if (e < total) {
                            int q, r;
                            divmod_small(e, nx, rnx, q, r);
                            const int dy = dyb + q * py, dx = rx + r * px;
                            if (dx < cw && dy < chh) rule_a(Tl, c, cx + dx, cy + dy);
                        }
                        FSE_PT(3)
                        // rank spawned particles in enumeration order. S.cnt[e] and the scan
                        // scratch are next written after the next sub-phase's barrier, so no
                        // barrier is needed after this block.
                        if (c.ev->n > 0) S.cnt[e] = c.ev->n;
                        if constexpr (PAIR) {
                            // the sub-phase's enumeration runs through rank 0's rows first:
                            // each CTA ranks its own spawns, the partner's count of the
                            // sub-phase comes through the cluster barrier that ends it
                            int tot = 0, ex = 0;
                            if (__syncthreads_or(c.ev->n > 0)) ex = block_excl_scan(S.cnt[tid], S.scan, &tot);
                            const int slot_t = 2 + (nsub & 1);
                            if (tid == 0)
                                st_cluster_u32(mapa_rank(smem_addr(&S.xch[slot_t]), (uint32_t)(rank ^ 1)),
                                               (uint32_t)tot);
                            cluster_sync();
                            const int tot_p = (int)S.xch[slot_t];
                            nsub++;
                            if (c.ev->n > 0) {
                                const int base = atomicAdd(w.stage_count, c.ev->n);
                                emit_spawns<TEMP, F32>(w, *c.ev, cp, (uint32_t)(running + (rank ? tot_p : 0) + ex),
                                                       base);
                            }
                            running += tot + tot_p;
                        } else if (__syncthreads_or(c.ev->n > 0)) {
                            // ranks with one more barrier: each warp's total in shared
                            // memory, a thread's rank the totals of the warps before it plus
                            // its lanes' prefix (the scratch is next written after the next
                            // sub-phase's barrier)
                            const int lane = tid & 31, wid = tid >> 5;
                            int inc = c.ev->n;
#pragma unroll
                            for (int o = 1; o < 32; o <<= 1) {
                                const int t = __shfl_up_sync(0xffffffffu, inc, o);
                                if (lane >= o) inc += t;
                            }
                            if (lane == 31) S.scan[wid] = inc;
                            __syncthreads();
                            const int ws = lane < T / 32 ? S.scan[lane] : 0;
                            const int tot = (int)__reduce_add_sync(0xffffffffu, (unsigned)ws);
                            const int ex = (int)__reduce_add_sync(0xffffffffu, lane < wid ? (unsigned)ws : 0u) + inc -
                                           c.ev->n;
                            if (c.ev->n > 0) {
                                // staging slots are taken in any order; the (chunk-pass, rank)
                                // key orders the particles later
                                const int base = atomicAdd(w.stage_count, c.ev->n);
                                emit_spawns<TEMP, F32>(w, *c.ev, cp, (uint32_t)(running + ex), base);
                            }
                            running += tot;
                        }
                        FSE_PT(4)
                    } else {
                        // cells of one sub-phase never conflict: each thread takes all of its
                        // cells in turn, one barrier per sub-phase
                        int q, r;
                        divmod_small(tid, nx, rnx, q, r);
                        int dq, dr;
                        divmod_small(T, nx, rnx, dq, dr);
                        if (sweep == 1) {
                            // at most 43 x 43 < 2 T cells: two per thread, their pending
                            // diffs requested together before either is processed
                            const int q1 = q + dq + (r + dr >= nx ? 1 : 0);
                            const int r1 = r + dr - (r + dr >= nx ? nx : 0);
                            const int dy0 = dyb + q * py, dx0 = rx + r * px;
                            const int dy1 = dyb + q1 * py, dx1 = rx + r1 * px;
                            const bool v0 = tid < total && dx0 < cw && dy0 < chh;
                            const bool v1 = tid + T < total && dx1 < cw && dy1 < chh;
                            const int32_t df0 = v0 ? w.df[(size_t)(cy + dy0) * W + cx + dx0] : 0;
                            const int32_t df1 = v1 ? w.df[(size_t)(cy + dy1) * W + cx + dx1] : 0;
                            if (v0) rule_b(Tl, c, cx + dx0, cy + dy0, df0);
                            if (v1) rule_b(Tl, c, cx + dx1, cy + dy1, df1);
                        } else {
                            for (int e = tid; e < total; e += T) {
                                const int dy = dyb + q * py, dx = rx + r * px;
                                if (dx < cw && dy < chh) rule_c(Tl, c, cx + dx, cy + dy);
                                q += dq;
                                r += dr;
                                if (r >= nx) {
                                    r -= nx;
                                    q++;
                                }
                            }
                        }
                        FSE_PT(3 + 2 * sweep)
                        if constexpr (PAIR)
                            cluster_sync();
                        else
                            __syncthreads();
                        FSE_PT(4 + 2 * sweep)
                    }
                }
            }
        }
        };
        // One instantiation of the sweeps for every chunk (a second one for the chunks
        // at the world edge doubles the register pressure of the kernel, whose spills
        // cost more than the checks they would save): the tile holds GENERIC_SOLID
        // outside the world, which is what world.cpp:999-1002 reads there, and the only
        // writes that can reach such cells (fire and interactions) check the world
        // bounds themselves.
        if constexpr (SEQ)
            sweeps_seq(Tile<false, TEMP, true, F32>(Tl));
        else
            sweeps(Tile<false, TEMP, false, F32, PAIR>(Tl));

        // ---- write back the cells this CTA changed (full-state rows inside the world),
        // one warp per row
        {
            const int lane = tid & 31, wid = tid >> 5;
            for (int r = wid; r < Tl.RHF; r += T / 32) {
                const int gy = Tl.y0 + r;
                if ((unsigned)gy >= (unsigned)H) continue;
                // a CTA pair: rank 0 writes rows above the chunk's middle, rank 1 the
                // others (each row is written by the CTA that owns it)
                if (PAIR && (rank == 0 ? gy >= cy + half : gy < cy + half)) continue;
                const size_t gb = (size_t)gy * W;
#pragma unroll
                for (int k = 0; k < MAXRW / 32; k++) {
                    const int lx = lane + 32 * k, gx = Tl.x0 + lx;
                    if (lx >= Tl.RW || (unsigned)gx >= (unsigned)W) continue;
                    const int i = r * Tl.RW + lx;
                    const uint16_t v = Tl.s_id[i];
                    if (!(v & DIRTY)) continue;
                    w.id[gb + gx] = (uint16_t)(v & 0x7FFF);
                    w.fl[gb + gx] = (uint8_t)(Tl.s_fl[i] & (uint8_t)~VISITED);
                    w.sc[gb + gx] = Tl.s_sc[i];
                    w.col[gb + gx] = Tl.s_col[i];
                    if (w.dirty) w.dirty[gb + gx] = 1;
                }
            }
        }
        if (!SEQ && tid == 0 && rank == 0) w.cp_count[cp] = running;
        __syncthreads();
        FSE_PT(9)
    }
    if (led_g_last) {
        __syncthreads();
        for (int i = tid; i < LED_ROWS * 64; i += T) {
            long long v = S.led[i];
            if (v) atomicAdd((unsigned long long *)&led_g_last[(i / 64) * MAXMAT + (i % 64)], (unsigned long long)v);
        }
    }
    // a CTA of a pair leaves only when its partner no longer writes to it
    if constexpr (PAIR) cluster_sync();
    if constexpr (FUSED) {
        // the last CTA out clears the completion flags and the counters
        __syncthreads();
        if (tid == 0) {
            __threadfence();
            s_ticket = (atomicAdd(&worlds[0].sched[1], 1u) == gridDim.x - 1) ? 1 : 0;
        }
        __syncthreads();
        if (s_ticket) {
            __threadfence();
            for (int wi = 0; wi < ft.n_worlds; wi++) {
                uint32_t *f = worlds[wi].cdone;
                const int nc = worlds[wi].nCx * worlds[wi].nCy;
                for (int i = tid; i < nc; i += T) f[i] = 0u;
            }
            if (tid == 0) {
                worlds[0].sched[0] = 0u;
                worlds[0].sched[1] = 0u;
                worlds[0].sched[2] = 0u;
            }
        }
    }
    FSE_PT_FLUSH
}

#if !defined(FSE_TICK_TEMP_TU) && !defined(FSE_TICK_SEQ_TU) && !defined(FSE_TICK_F32_TU) && \
    !defined(FSE_TICK_PAIR_TU) && !defined(FSE_TICK_FUSED_TU)
size_t colour_pass_smem(int C, int halo) {
    // a 2-cell halo leaves room for the TMA-staged tile's wider rows
    size_t RW = (size_t)C + 2 * halo;
    if (halo == 2) RW = std::max(RW, (size_t)tma_tile_width(C));
    size_t RHF = (size_t)C + 2 * halo, RHI = (size_t)C + halo + 10;
    size_t nid = RW * RHI, nfull = RW * RHF;
    // the planes start on a 128-byte boundary of the window: up to 128 bytes of padding
    size_t head = (sizeof(SmemHead) + 127) & ~(size_t)127;
    return 128 + head + ((nfull + 31) & ~(size_t)31) * 4 + nfull * 4 + ((nid + 1) & ~(size_t)1) * 2 + nfull;
}

#endif

template <int HALO, bool TEMP, bool SEQ = false, bool F32 = false>
static cudaError_t launch_t(const WorldDev *worlds, const uint32_t *items, int n_items, int iter, int tk,
                            const MatTable *mt, size_t sm, int grid, cudaStream_t s) {
    // opt in to the full shared-memory carve-out once per instantiation
    static size_t set = 0;
    if (set < sm) {
        cudaFuncSetAttribute(k_colour_pass<HALO, TEMP, SEQ, F32>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)sm);
        set = sm;
    }
    k_colour_pass<HALO, TEMP, SEQ, F32><<<grid, CP_THREADS, sm, s>>>(worlds, items, n_items, iter, tk, mt,
                                                                     FusedTick{});
    return cudaGetLastError();
}

// the fused tick: one CTA per SM (the tile takes most of an SM's shared memory)
template <int HALO, bool TEMP, bool F32>
static cudaError_t launch_fused_t(const WorldDev *worlds, const FusedTick &ft, const MatTable *mt, size_t sm,
                                  int grid, cudaStream_t s) {
    static size_t set = 0;
    if (set < sm) {
        cudaFuncSetAttribute(k_colour_pass<HALO, TEMP, false, F32, false, true>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        set = sm;
    }
    k_colour_pass<HALO, TEMP, false, F32, false, true><<<grid, CP_THREADS, sm, s>>>(worlds, nullptr, 0, 0, 0, mt, ft);
    return cudaGetLastError();
}

// shared memory of one CTA of a pair: half the chunk's rows plus the reach of its rules
static size_t colour_pass_smem_pair(int C, int halo) {
    const size_t own = (size_t)C / 2;
    size_t RW = (size_t)C + 2 * halo, RHF = own + 2 * halo, RHI = own + halo + 10;
    size_t nid = RW * RHI, nfull = RW * RHF;
    size_t head = (sizeof(SmemHeadT<CP_THREADS / 2>) + 127) & ~(size_t)127;
    return 128 + head + ((nfull + 31) & ~(size_t)31) * 4 + nfull * 4 + ((nid + 1) & ~(size_t)1) * 2 + nfull;
}

// the chunks split over CTA pairs (thread-block clusters of two): `clusters` pairs
template <int HALO, bool TEMP, bool F32>
static cudaError_t launch_pair_t(const WorldDev *worlds, const uint32_t *items, int n_items, int iter, int tk,
                                 const MatTable *mt, size_t sm, int clusters, cudaStream_t s) {
    static size_t set = 0;
    if (set < sm) {
        cudaFuncSetAttribute(k_colour_pass<HALO, TEMP, false, F32, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)sm);
        // all of the unified L1/shared storage as shared memory, so that two CTAs fit an SM
        cudaFuncSetAttribute(k_colour_pass<HALO, TEMP, false, F32, true>,
                             cudaFuncAttributePreferredSharedMemoryCarveout, 100);
        set = sm;
    }
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(2 * clusters);
    cfg.blockDim = dim3(CP_THREADS / 2);
    cfg.dynamicSmemBytes = sm;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = 2;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, k_colour_pass<HALO, TEMP, false, F32, true>, worlds, items, n_items, iter, tk, mt,
                              FusedTick{});
}

// Each translation unit that includes this file with one of the defines below
// compiles one family of instantiations, so that they build in parallel.
#if defined(FSE_TICK_FUSED_TU)
// the fused tick, Q16.16 amounts (FSE_TICK_FUSED_TU = 1) or f32 (2)
#define FSE_FUSED_F32 (FSE_TICK_FUSED_TU == 2)
size_t colour_pass_smem(int C, int halo);
#if FSE_TICK_FUSED_TU == 2
cudaError_t launch_colour_fused_f32(const WorldDev *worlds, const FusedTick &ft, const MatTable *mt, int halo, int C,
                                    int grid, cudaStream_t s, bool temp) {
#else
cudaError_t launch_colour_fused(const WorldDev *worlds, const FusedTick &ft, const MatTable *mt, int halo, int C,
                                int grid, cudaStream_t s, bool temp) {
#endif
    const size_t sm = colour_pass_smem(C, halo);
    if (temp) {
        if (halo == 5) return launch_fused_t<5, true, FSE_FUSED_F32>(worlds, ft, mt, sm, grid, s);
        return launch_fused_t<2, true, FSE_FUSED_F32>(worlds, ft, mt, sm, grid, s);
    }
    if (halo == 5) return launch_fused_t<5, false, FSE_FUSED_F32>(worlds, ft, mt, sm, grid, s);
    return launch_fused_t<2, false, FSE_FUSED_F32>(worlds, ft, mt, sm, grid, s);
}
#elif defined(FSE_TICK_PAIR_TU)
// chunks split over CTA pairs, Q16.16 amounts (FSE_TICK_PAIR_TU = 1) or f32 (2)
#define FSE_PAIR_F32 (FSE_TICK_PAIR_TU == 2)
#if FSE_TICK_PAIR_TU == 2
cudaError_t launch_colour_pass_pair_f32(const WorldDev *worlds, const uint32_t *items, int n_items, int iter, int tk,
                                        const MatTable *mt, int halo, int C, int clusters, cudaStream_t s, bool temp) {
#else
cudaError_t launch_colour_pass_pair(const WorldDev *worlds, const uint32_t *items, int n_items, int iter, int tk,
                                    const MatTable *mt, int halo, int C, int clusters, cudaStream_t s, bool temp) {
#endif
    const size_t sm = colour_pass_smem_pair(C, halo);
    if (temp) {
        if (halo == 5)
            return launch_pair_t<5, true, FSE_PAIR_F32>(worlds, items, n_items, iter, tk, mt, sm, clusters, s);
        return launch_pair_t<2, true, FSE_PAIR_F32>(worlds, items, n_items, iter, tk, mt, sm, clusters, s);
    }
    if (halo == 5) return launch_pair_t<5, false, FSE_PAIR_F32>(worlds, items, n_items, iter, tk, mt, sm, clusters, s);
    return launch_pair_t<2, false, FSE_PAIR_F32>(worlds, items, n_items, iter, tk, mt, sm, clusters, s);
}
#elif defined(FSE_TICK_F32_TU)
// f32 liquid amounts (FSE_CFG_F32_FLUID), in the partitioned order (FSE_TICK_F32_TU
// = 1) or in the reference's order (2)
#define FSE_F32_SEQ (FSE_TICK_F32_TU == 2)
#if FSE_TICK_F32_TU == 2
cudaError_t launch_colour_pass_f32_seq(const WorldDev *worlds, const uint32_t *items, int n_items, int iter, int tk,
                                       const MatTable *mt, int halo, size_t sm, int grid, cudaStream_t s, bool temp) {
#else
cudaError_t launch_colour_pass_f32(const WorldDev *worlds, const uint32_t *items, int n_items, int iter, int tk,
                                   const MatTable *mt, int halo, size_t sm, int grid, cudaStream_t s, bool temp) {
#endif
    if (temp) {
        if (halo == 5) return launch_t<5, true, FSE_F32_SEQ, true>(worlds, items, n_items, iter, tk, mt, sm, grid, s);
        return launch_t<2, true, FSE_F32_SEQ, true>(worlds, items, n_items, iter, tk, mt, sm, grid, s);
    }
    if (halo == 5) return launch_t<5, false, FSE_F32_SEQ, true>(worlds, items, n_items, iter, tk, mt, sm, grid, s);
    return launch_t<2, false, FSE_F32_SEQ, true>(worlds, items, n_items, iter, tk, mt, sm, grid, s);
}
#elif defined(FSE_TICK_SEQ_TU)
cudaError_t launch_colour_pass_seq(const WorldDev *worlds, const uint32_t *items, int n_items, int iter, int tk,
                                   const MatTable *mt, int halo, size_t sm, int grid, cudaStream_t s, bool temp) {
    if (temp) {
        if (halo == 5) return launch_t<5, true, true>(worlds, items, n_items, iter, tk, mt, sm, grid, s);
        return launch_t<2, true, true>(worlds, items, n_items, iter, tk, mt, sm, grid, s);
    }
    if (halo == 5) return launch_t<5, false, true>(worlds, items, n_items, iter, tk, mt, sm, grid, s);
    return launch_t<2, false, true>(worlds, items, n_items, iter, tk, mt, sm, grid, s);
}
#elif defined(FSE_TICK_TEMP_TU)
cudaError_t launch_colour_pass_temp(const WorldDev *worlds, const uint32_t *items, int n_items, int iter, int tk,
                                    const MatTable *mt, int halo, size_t sm, int grid, cudaStream_t s) {
    if (halo == 5) return launch_t<5, true>(worlds, items, n_items, iter, tk, mt, sm, grid, s);
    return launch_t<2, true>(worlds, items, n_items, iter, tk, mt, sm, grid, s);
}
#else
cudaError_t launch_colour_pass_temp(const WorldDev *worlds, const uint32_t *items, int n_items, int iter, int tk,
                                    const MatTable *mt, int halo, size_t sm, int grid, cudaStream_t s);
cudaError_t launch_colour_pass_seq(const WorldDev *worlds, const uint32_t *items, int n_items, int iter, int tk,
                                   const MatTable *mt, int halo, size_t sm, int grid, cudaStream_t s, bool temp);
cudaError_t launch_colour_pass_f32(const WorldDev *worlds, const uint32_t *items, int n_items, int iter, int tk,
                                   const MatTable *mt, int halo, size_t sm, int grid, cudaStream_t s, bool temp);
cudaError_t launch_colour_pass_f32_seq(const WorldDev *worlds, const uint32_t *items, int n_items, int iter, int tk,
                                       const MatTable *mt, int halo, size_t sm, int grid, cudaStream_t s, bool temp);

cudaError_t launch_colour_pass_pair(const WorldDev *worlds, const uint32_t *items, int n_items, int iter, int tk,
                                    const MatTable *mt, int halo, int C, int clusters, cudaStream_t s, bool temp);
cudaError_t launch_colour_pass_pair_f32(const WorldDev *worlds, const uint32_t *items, int n_items, int iter, int tk,
                                        const MatTable *mt, int halo, int C, int clusters, cudaStream_t s, bool temp);

// threads: CP_THREADS (one CTA per chunk) or CP_THREADS / 2 (each chunk split over a
// CTA pair; the partitioned order and an even chunk edge only); grid: chunk workers
// (CTAs, or pairs), 0 = one per chunk
cudaError_t launch_colour_pass(const WorldDev *worlds, const uint32_t *items, int n_items, int iter, int tk,
                               const MatTable *mt, int halo, int C, int threads, int grid, cudaStream_t s,
                               bool temp, bool seq, bool f32) {
    size_t sm = colour_pass_smem(C, halo);
    if (n_items <= 0) return cudaSuccess;
    if (grid <= 0 || grid > n_items) grid = n_items;
    if (threads == CP_THREADS / 2 && !seq && C % 2 == 0) {
        if (f32) return launch_colour_pass_pair_f32(worlds, items, n_items, iter, tk, mt, halo, C, grid, s, temp);
        return launch_colour_pass_pair(worlds, items, n_items, iter, tk, mt, halo, C, grid, s, temp);
    }
    if (f32 && seq) return launch_colour_pass_f32_seq(worlds, items, n_items, iter, tk, mt, halo, sm, grid, s, temp);
    if (f32) return launch_colour_pass_f32(worlds, items, n_items, iter, tk, mt, halo, sm, grid, s, temp);
    if (seq) return launch_colour_pass_seq(worlds, items, n_items, iter, tk, mt, halo, sm, grid, s, temp);
    if (temp) return launch_colour_pass_temp(worlds, items, n_items, iter, tk, mt, halo, sm, grid, s);
    if (halo == 5) return launch_t<5, false>(worlds, items, n_items, iter, tk, mt, sm, grid, s);
    return launch_t<2, false>(worlds, items, n_items, iter, tk, mt, sm, grid, s);
}
#endif

}  // namespace fse

#if defined(FSE_PHASE_CLOCKS) && !defined(FSE_TICK_TEMP_TU) && !defined(FSE_TICK_SEQ_TU) && !defined(FSE_TICK_F32_TU) && \
    !defined(FSE_TICK_PAIR_TU) && !defined(FSE_TICK_FUSED_TU)
extern "C" int fse_debug_phase_clocks(unsigned long long out[16], int reset) {
    cudaDeviceSynchronize();
    cudaMemcpyFromSymbol(out, g_phase_clk, 16 * sizeof(unsigned long long));
    if (reset) {
        unsigned long long z[16] = {0};
        cudaMemcpyToSymbol(g_phase_clk, z, sizeof(z));
    }
    return 0;
}
// the per-phase maxima over CTAs (out[15]: the longest CTA, start to end)
extern "C" int fse_debug_phase_max(unsigned long long out[16], int reset) {
    cudaDeviceSynchronize();
    cudaMemcpyFromSymbol(out, g_phase_max, 16 * sizeof(unsigned long long));
    if (reset) {
        unsigned long long z[16] = {0};
        cudaMemcpyToSymbol(g_phase_max, z, sizeof(z));
    }
    return 0;
}
#endif
