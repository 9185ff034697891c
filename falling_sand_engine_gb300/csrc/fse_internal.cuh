// fse_internal.cuh -- device-side definitions shared by the tick, particle and
// object kernels and by the host orchestration.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/fse.h"

namespace fse {

// PhysicsType, source/engine/game_datastruct.hpp:87-95
enum : int { T_AIR = 0, T_SOLID = 1, T_SAND = 2, T_SOUP = 3, T_GAS = 4, T_OBJECT = 5 };
enum : int { INTER_TRANSFORM = 1, INTER_SPAWN = 2, REACT_BELOW = 4, REACT_ABOVE = 5 };

constexpr int MAXMAT = 256;
constexpr int CP_THREADS = 1024;  // colour-pass CTA: >= the largest sweep-A sub-phase (43 x 22 cells, 128-cell chunks)
constexpr uint8_t MOVED = 0x80;
constexpr uint8_t VISITED = 0x40;  // shared-memory copy only; never stored to HBM
constexpr uint8_t SETTLE_MASK = 0x3F;
constexpr uint16_t DIRTY = 0x8000;  // shared-memory copy only: cell must be written back

// FLUID_* (source/engine/core/const.h:23-34) in Q16.16
constexpr int32_t Q_MAXV = 32768;
constexpr int32_t Q_MINV = 33;
constexpr int32_t Q_MAXCOMP = 6554;
constexpr int32_t Q_MAXFLOW = 524288;
constexpr int32_t Q_FREEFALL = 327;
constexpr int32_t Q_DEFAULT = 131072;
// the same constants as the reference's own floats, for worlds created with
// FSE_CFG_F32_FLUID (amounts and diffs are then f32 bit patterns in the 32-bit planes)
constexpr float F_MAXV = 0.5f;
constexpr float F_MINV = 0.0005f;
constexpr float F_MAXCOMP = 0.1f;
constexpr float F_MAXFLOW = 8.0f;
constexpr int32_t F_DEFAULT_BITS = 0x40000000;  // 2.0f, MaterialInstance::fluidAmount's default

constexpr uint32_t PH_GEN = 0x47454E00u;
constexpr uint32_t PH_STAMP = 0x5354414Du;

// ledger rows
enum : int { LED_CN = 0, LED_DN = 1, LED_XN = 2, LED_CF = 3, LED_DF = 4, LED_XF = 5, LED_ROWS = 6 };

// error bits recorded by kernels (world->err)
enum : int { ERR_SPAWN_CAP = 1, ERR_PART_CAP = 2, ERR_BOUNDS = 4, ERR_TIMEOUT = 8 };

// ------------------------------------------------------------------ RNG
// lowbias32 integer finaliser (C. Wellons, public domain); keys follow
// (seed, tick, phase) -> (x, y) -> draw index.
__host__ __device__ __forceinline__ uint32_t hash32(uint32_t h) {
    h ^= h >> 16;
    h *= 0x7feb352dU;
    h ^= h >> 15;
    h *= 0x846ca68bU;
    h ^= h >> 16;
    return h;
}
__host__ __device__ __forceinline__ uint32_t pass_key(uint32_t seed, uint32_t tick, uint32_t phase) {
    uint32_t h = hash32(seed ^ 0x5bd1e995U);
    h = hash32(h ^ tick);
    return hash32(h ^ (phase * 0x9E3779B9U + 0x7F4A7C15U));
}
__host__ __device__ __forceinline__ uint32_t cell_key(uint32_t pk, uint32_t x, uint32_t y) {
    return hash32(hash32(pk ^ x) ^ (y * 0x85EBCA6BU));
}
__host__ __device__ __forceinline__ uint32_t draw_k(uint32_t ck, uint32_t k) {
    return hash32(ck + k * 0x9E3779B9U + 0x632BE5ABU);
}

// --------------------------------------------------------- material table
// Packed per-material word A: type | iterations << 8 | slip << 16 | max_stab << 24,
// word B: density bits. Factory: base colour, (shift | lo << 8 | mod << 20), scalar.
struct MatTable {
    int n;
    int id_air, id_solid, id_fire, id_water, id_lava, id_steam, id_obsidian;
    int has_inter;
    uint32_t a[MAXMAT];
    float density[MAXMAT];
    uint32_t f_base[MAXMAT];
    uint32_t f_pack[MAXMAT];
    int32_t f_scalar[MAXMAT];
    // reactions: up to 4 per material, (kind, temperature, result)
    int32_t n_react[MAXMAT];
    int32_t react[MAXMAT][4][3];
    // interactions: flat list of (mat, other, kind, data1, data2, ofsx, ofsy), n_inter entries
    int32_t n_inter;
    int32_t inter[512][7];
    // rendering: Material::alpha (u8), emitColor, and 3.0 / iterations + 0.5 of the
    // flow texture (game.cpp:2048), evaluated once in double
    uint32_t alpha[MAXMAT];
    uint32_t emit_col[MAXMAT];
    double flow_k[MAXMAT];
    // The flow texel byte is a non-decreasing step function of the float flow for
    // k > 0: flow_thr[m][j] is the smallest float whose byte is >= j (j = 1..255),
    // found on the host by bisection with the double arithmetic above, so the
    // byte of f is the largest j with flow_thr[m][j] <= f. flow_thr_ok[m] = 0:
    // no table (k <= 0 or not finite), evaluate in double.
    float flow_thr[MAXMAT][256];
    uint8_t flow_thr_ok[MAXMAT];
    // temperature: the factory temperature of SOUP tiles (whose scalar is the
    // amount), and Material::addTemp / conductionSelf / conductionOther
    int32_t f_temp[MAXMAT];
    uint32_t add_temp[MAXMAT];
    float cond_self[MAXMAT];
    float cond_other[MAXMAT];
};

__host__ __device__ __forceinline__ int mt_type(uint32_t a) { return (int)(a & 0xFF); }
__host__ __device__ __forceinline__ int mt_iter(uint32_t a) { return (int)((a >> 8) & 0xFF); }
__host__ __device__ __forceinline__ int mt_slip(uint32_t a) { return (int)((a >> 16) & 0xFF); }
__host__ __device__ __forceinline__ int mt_stab(uint32_t a) { return (int)((a >> 24) & 0xFF); }

// ------------------------------------------------------------------ world
struct SpawnRec {  // one spawned particle awaiting its place in the list (48 B)
    uint32_t cp;    // chunk-pass index within the tick
    uint32_t rank;  // position within that chunk-pass
    float x, y, vx, vy, ay;
    uint32_t colour;
    int32_t scalar;
    uint16_t id;
    uint8_t flags;
    uint8_t bits;
    int16_t lifetime;
    int16_t fade;
    int16_t temp;  // temperature of a SOUP tile
    uint16_t pad;
};

struct PartSoA {  // particle list, structure of arrays
    float *x, *y, *vx, *vy, *ax, *ay, *tx, *ty, *tf;
    int32_t *life, *fade;
    uint32_t *col;
    int32_t *sc;
    int16_t *tp;  // temperature of SOUP tiles
    uint16_t *id;
    uint8_t *fl, *bits;
};

struct WorldDev {
    uint16_t *id;
    uint32_t *col;
    int32_t *sc;
    uint8_t *fl;
    int32_t *df;  // pending fluid diff; meaningful only where the cell is SOUP
    // temperature of SOUP cells (MaterialInstance::temperature; every other cell
    // keeps it in sc). Kept only by worlds created with FSE_CFG_TEMPERATURE (NULL
    // otherwise, and then the particle lists have no temperatures either): liquid
    // temperatures change no other result of a tick, and copying them with every
    // liquid move costs the colour pass global-memory round trips.
    int16_t *tp;
    int W, H, C, cell_iter;
    uint32_t seed;
    uint32_t *tick;  // device counter, advanced on the device so multi-tick graphs replay correctly
    // world::tickZone (world.hpp:138), inside the world: chunks start at its corner
    // (nCx x nCy of them, C cells each way whatever the zone's end), particles outside
    // it stay as they are, the temperature step changes its cells only; max_slots is
    // the most chunks of one colour any zone of the world has (the whole world's)
    int zx, zy, zw, zh;
    int nCx, nCy, max_slots;
    // spawned-particle staging for the current tick
    SpawnRec *stage;
    int32_t *stage_count;
    int32_t stage_cap;
    // spawn counts per chunk-pass (cell_iter * 4 * max_slots of them), each split in
    // cp_rows rows: 1, or the chunk edge in the reference's order, where every chunk
    // row ranks its own spawns (rows bottom first, the order of world.cpp's loop)
    int cp_rows;
    int32_t *cp_count;  // [cell_iter * 4 * max_slots * cp_rows]
    int32_t *cp_base;
    // particles
    PartSoA p, q;           // p = live list, q = compaction scratch
    int32_t *part_count;    // device-resident live count
    int32_t part_cap;
    uint8_t *p_state;       // per particle: 0 alive, 1 dead; during the update its outcome
    // per particle during the update: the cells it read as a box (x0 | y0 << 16 and
    // x1 | y1 << 16; box0 -1: none), the cell it fills or merges into (-1: none), the
    // fill cell an iteration moved it away from; box0 holds the merge cell afterwards
    int32_t *p_box0, *p_box1, *p_cell, *p_prev;
    int32_t *req_count;     // [3] counters of the update (fill changes of even / odd iterations)
    uint32_t *chg;          // 2 x airmap blocks: lowest index whose fill changed there (read / written by an iteration)
    int32_t *stats;         // [0]: iterations of the last particle update (of the launch's first world)
    // [0..1] fills of this world changed by the update's even / odd iterations,
    // [2..3] the lowest index among those changes
    int32_t *chg_n;
    int32_t *scan_tmp;      // block sums for compaction
    long long *ledger;      // [LED_ROWS][MAXMAT]
    int32_t *err;
    unsigned *bar;          // grid barrier {count, generation} of the cooperative deposit kernel
    uint8_t *airmap;        // per 8x8 block of cells: 1 if it held AIR when the particle tick began
    int amw, amh;           // airmap size in blocks
    // render state, NULL unless the world renders: cells written since the last
    // dirty pass, and the tick's flows per cell (Q16.16, x then y, wrapping sums)
    uint8_t *dirty;
    int32_t *flow;
    // temperature step (FSE_CFG_TEMPERATURE): run after ticks whose index is 2 mod 4;
    // tnew holds the deferred results of tile-edge cells
    int temp_on;
    int32_t *tnew;
    // FSE_CFG_F32_FLUID: liquid amounts and pending diffs are f32 (the reference's
    // own arithmetic) rather than Q16.16; the ledger then keeps no fluid rows
    int f32;
    // deposits of liquid particles into liquid cells, applied after the update
    // (particle indices, 2 x part_cap for the ordered rounds; the target cell is in
    // p_box0), and in f32 worlds the per-cell claims of those rounds (all ones
    // between ticks)
    int32_t *merge_list;
    int32_t *merge_count;
    uint32_t *merge_claim;
    // the fused tick (all colour passes of a tick in one launch, each chunk-pass
    // started when the chunk-passes it depends on are done): per chunk of the zone,
    // the index + 1 of the last pass done on it in the running launch (all zero
    // between launches); sched = {next ticket, CTAs finished, a wait gave up} of a
    // launch whose table starts with this world
    uint32_t *cdone;
    uint32_t *sched;
    // two CUtensorMaps (128 B each, scalar then colour) over the world's planes for
    // the colour pass's TMA staging with a 2-cell halo; NULL when the world's row
    // pitch is not a multiple of 16 bytes (then the tile is staged with cp.async)
    const void *tmap;
};

// the TMA-staged tile's width for chunk edge C and a 2-cell halo: the row starts at
// (cx - 2) rounded down to a multiple of 4 cells (a 16-byte boundary) and covers
// cx + C + 1, in a whole number of 16-byte groups
__host__ __device__ constexpr int tma_tile_width(int C) { return (C + 2 * 2 + 3 + 3) & ~3; }

// The fused tick's work list: the chunk slots of each colour ((world << 20) | slot,
// the per-pass launches' items), passes = cell_iter * 4 of the longest world, and
// the worlds of the table (their completion flags are cleared at the end)
struct FusedTick {
    const uint32_t *items[4];
    int n[4];
    int passes;
    int n_worlds;
};

// the amount of a new SOUP tile of material mid (TilesCreate, and the
// MaterialInstance default 2.0): the factory's Q16.16 scalar, or its f32 value in
// worlds with f32 amounts; other materials' scalar (a temperature) as it is
__host__ __device__ __forceinline__ int32_t soup_scalar(const MatTable *mt, int mid, int f32) {
    const int32_t q = mt->f_scalar[mid];
    if (!f32 || mt_type(mt->a[mid]) != T_SOUP) return q;
    const float f = (float)q * (1.0f / 65536.0f);  // exact: q is a multiple of 2^-16 well below 2^24
    union {
        float f;
        int32_t i;
    } u;
    u.f = f;
    return u.i;
}

__host__ __device__ __forceinline__ int ceil_div(int a, int b) { return (a + b - 1) / b; }

}  // namespace fse
