// ref_tick.cpp -- TEST INFRASTRUCTURE ONLY (never linked into the product).
//
// Compiles the reference's own world::tick (source/engine/world.cpp:1036-1948) so
// that the oracle's restatement of the cell rules (reference chunk order) can be
// checked against it. oracle/Makefile (target `ref`) extracts, unchanged, into _ref/:
// world::tick, world::getTile / setTile (world.cpp:999-1008),
// CalculateVerticalFlowValue (world.cpp:1021-1034), the FLUID_* constants
// (core/const.h:23-34), the interaction kinds, MaterialInteraction and Material
// (game_datastruct.hpp:96-168), MaterialInstance (game_datastruct.hpp:206-224) with
// its constructors and Tiles_NOTHING / Tiles_TEST_SOLID (game_datastruct.cpp:40-52,
// 304-314), and CellData (game_utils/cells.h:15-36). This file supplies the rest:
//  - the GAME() registry (materials_container, materials_list, materials_count),
//    filled from a table passed in (ids, types, densities, iterations,
//    slipperiness, reactions, interactions);
//  - the tile factories TilesCreate*: their colours come from textures in the
//    reference; here they follow the oracle's factory parameters (base colour, one
//    draw when a channel jitters, the factory temperature);
//  - the thread pools: by default each pushed task runs at once and hands back a
//    ready future, so the chunk tasks of a colour run in push order (they touch
//    disjoint cells; the spawned particles are merged in push order as in the
//    reference); for timing, a pool of worker threads as the reference's
//    (world.cpp:59), with the draw state kept per thread;
//  - rand(): a macro expanded inside the cell loops, where `x`, `y` and `iter` are
//    the cell being updated; it returns the oracle's counter draw for that cell
//    update -- keyed on (seed, tick, iter * 3 + sweep, x, y), counted from 0 per
//    update -- as a value whose `%` is the oracle's unsigned modulo. The factories
//    called from the loops draw from the same counter. The sweep is counted at
//    `CHUNK_H - 1`, which starts each of the three sweeps of a chunk task;
//  - physicsCheck: nothing (it is a separate call of its own);
//  - argument order: the reference's Linux build uses clang (xmake.lua:107), which
//    evaluates a call's arguments left to right, so the two draws of a spawned
//    particle's velocity are taken vx first. g++ evaluates them right to left, so a
//    macro makes each `CellData(...)` construction a brace initialisation, whose
//    elements are evaluated in order (the int positions narrow to f32 as in the call).
#include <algorithm>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <deque>
#include <mutex>
#include <thread>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <future>
#include <string>
#include <type_traits>
#include <vector>
// the reference's mathlib_base.hpp:8-9 includes these, so abs(float) is the float one
#include <math.h>
#include <stdlib.h>

typedef float f32;
typedef uint32_t u32;
typedef int32_t i32;
typedef int16_t i16;
typedef uint8_t u8;

enum PhysicsType { AIR = 0, SOLID = 1, SAND = 2, SOUP = 3, GAS = 4, PASSABLE = 5, OBJECT = 5 };

#include "tick_interact_defs.inc"

using mat_id = u32;
using mat_instance_id = mat_id;
using mat_temperature = i16;

#include "tick_material_interaction.inc"
#include "tick_material_struct.inc"
#include "tick_material_ctor.inc"

struct MaterialsList {
    Material GENERIC_AIR, GENERIC_SOLID, FIRE, WATER, LAVA, STEAM, OBSIDIAN;
};
struct GameReg {
    MaterialsList materials_list;
    std::vector<Material *> materials_container;
    int materials_count = 0;
};
static GameReg g_reg;
static GameReg *GAME() { return &g_reg; }

#include "tick_material_instance.inc"
#include "tick_material_instance_ctor.inc"
#include "tick_tiles_globals.inc"
#include "tick_cell_data.inc"
#include "tick_fluid_consts.inc"
#include "tick_vertical_flow.inc"

// ---------------------------------------------------------------- the draws
// the oracle's counter RNG (fse_oracle.c: hash32, pass_key, cell_key, draw_k)
static inline uint32_t h32(uint32_t h) {
    h ^= h >> 16;
    h *= 0x7feb352dU;
    h ^= h >> 15;
    h *= 0x846ca68bU;
    h ^= h >> 16;
    return h;
}
static inline uint32_t pass_key(uint32_t seed, uint32_t tick, uint32_t phase) {
    uint32_t h = h32(seed ^ 0x5bd1e995U);
    h = h32(h ^ tick);
    return h32(h ^ (phase * 0x9E3779B9U + 0x7F4A7C15U));
}
static inline uint32_t cell_key(uint32_t pk, uint32_t x, uint32_t y) { return h32(h32(pk ^ x) ^ (y * 0x85EBCA6BU)); }
static inline uint32_t draw_k(uint32_t ck, uint32_t k) { return h32(ck + k * 0x9E3779B9U + 0x632BE5ABU); }

static uint32_t g_seed = 0, g_tick = 0;
static thread_local int g_sweep = 2;       // the first `CHUNK_H - 1` makes it 0
static thread_local long long g_cur = -1;  // the cell update the counter belongs to
static thread_local uint32_t g_ck = 0, g_k = 0;
static thread_local long long g_draws = 0;

struct Draw {
    uint32_t v;
};
static inline int operator%(Draw d, int m) { return (int)(d.v % (uint32_t)m); }

static inline void sync_cell(int x, int y, int iter) {
    const long long key = ((((long long)iter * 3 + g_sweep) << 24 | (long long)y) << 24) | (long long)x;
    if (key != g_cur) {
        g_cur = key;
        g_ck = cell_key(pass_key(g_seed, g_tick, (uint32_t)(iter * 3 + g_sweep)), (uint32_t)x, (uint32_t)y);
        g_k = 0;
    }
}
static inline Draw fse_ref_draw(int x, int y, int iter) {
    sync_cell(x, y, iter);
    g_draws++;
    return Draw{draw_k(g_ck, g_k++)};
}

// the tile factories: the oracle's parameters for material id
struct Factory {
    u32 base = 0;
    int shift = 0, lo = 0, mod = 0;
    int temperature = 0;
};
static std::vector<Factory> g_fac;
static MaterialInstance fse_ref_create(int x, int y, int iter, int id) {
    const Factory &f = g_fac[id];
    u32 col = f.base;
    if (f.mod > 0) col = f.base + ((u32)(f.lo + (fse_ref_draw(x, y, iter) % f.mod)) << f.shift);
    return MaterialInstance(GAME()->materials_container[id], col, (mat_temperature)f.temperature);
}

// ---------------------------------------------------------------- the world
struct ChunkH {
    operator int() const { return 128; }
    int operator-(int k) const {
        g_sweep = (g_sweep + 1) % 3;
        return 128 - k;
    }
};
static constexpr int CHUNK_W = 128;
static constexpr ChunkH CHUNK_H{};

struct GlobalDef {
    int cell_iter = 3;
};
struct IsoState {
    GlobalDef globaldef;
};
struct GameState {
    IsoState Iso;
};
struct Globals {
    GameState *game;
};
static GameState g_game_state;
static Globals global{&g_game_state};

struct Pool {
    // workers == 0: run each task at once in the caller
    std::vector<std::thread> workers;
    std::deque<std::function<void()>> q;
    std::mutex mu;
    std::condition_variable cv;
    bool stop = false;
    void start(int n) {
        for (int i = 0; i < n; i++)
            workers.emplace_back([this] {
                for (;;) {
                    std::function<void()> job;
                    {
                        std::unique_lock<std::mutex> lk(mu);
                        cv.wait(lk, [this] { return stop || !q.empty(); });
                        if (stop && q.empty()) return;
                        job = std::move(q.front());
                        q.pop_front();
                    }
                    job();
                }
            });
    }
    void halt() {
        {
            std::lock_guard<std::mutex> lk(mu);
            stop = true;
        }
        cv.notify_all();
        for (auto &t : workers) t.join();
        workers.clear();
        stop = false;
    }
    template <class F>
    auto push(F &&f) -> std::future<decltype(f(0))> {
        using R = decltype(f(0));
        if (workers.empty()) {
            std::promise<R> p;
            if constexpr (std::is_void_v<R>) {
                f(0);
                p.set_value();
            } else {
                p.set_value(f(0));
            }
            return p.get_future();
        }
        auto task = std::make_shared<std::packaged_task<R(int)>>(std::forward<F>(f));
        std::future<R> fut = task->get_future();
        {
            std::lock_guard<std::mutex> lk(mu);
            q.emplace_back([task] { (*task)(0); });
        }
        cv.notify_one();
        return fut;
    }
};
struct WorldSys {
    Pool *tickPool, *tickVisitedPool;
};
static Pool g_pool, g_vpool;
static WorldSys world_sys{&g_pool, &g_vpool};

struct TickZone {
    int x, y, w, h;
};
struct world {
    int width = 0, height = 0;
    MaterialInstance *real_tiles = nullptr;
    bool *dirty = nullptr;
    bool *tickVisited1 = nullptr, *tickVisited2 = nullptr;
    f32 *flowX = nullptr, *flowY = nullptr;
    TickZone tickZone{};
    std::vector<CellData *> cells;
    int tickCt = 0;
    MaterialInstance getTile(int x, int y);
    void setTile(int x, int y, MaterialInstance type);
    void physicsCheck(int, int) {}
    void tick();
    void tickCells();
};

#include "tick_world_gettile.inc"
#include "tick_world_settile.inc"
#include "tick_cells.inc"

// the loops' draws and factories take the cell being updated from their scope;
// the rand() after the loops (physicsCheck's position) reads these
static int x = 0, y = 0, iter = 0;
#define rand() fse_ref_draw(x, y, iter)
#define TilesCreate(id, a, b) fse_ref_create(x, y, iter, (int)(id))
#define TilesCreateFire() fse_ref_create(x, y, iter, (int)GAME()->materials_list.FIRE.id)
#define TilesCreateSteam() fse_ref_create(x, y, iter, (int)GAME()->materials_list.STEAM.id)
#define TilesCreateWater() fse_ref_create(x, y, iter, (int)GAME()->materials_list.WATER.id)
#define TilesCreateObsidian(a, b) fse_ref_create(x, y, iter, (int)GAME()->materials_list.OBSIDIAN.id)
#define CellData(...) CellData{__VA_ARGS__}
#include "tick_world_tick.inc"
#undef rand
#undef TilesCreate
#undef TilesCreateFire
#undef TilesCreateSteam
#undef TilesCreateWater
#undef TilesCreateObsidian
#undef CellData

// ---------------------------------------------------------------- entry
// Materials: n rows of 10 ints -- physicsType, density bits, iterations,
// slipperyness, factory base, shift, lo, mod, temperature, 0; special ids: air,
// solid, fire, water, lava, steam, obsidian. Reactions: n x 4 rows (kind,
// temperature, result; kind 0 = none). Interactions: ni rows (material, other, kind,
// data1, data2, ofsX, ofsY) in registration order.
// Grid (in/out, W * H): ids, colours, temperatures, moved. Runs n_ticks ticks from
// `tick` with cell_iter iterations; writes the spawned particles (16 values each:
// id, colour, temperature, x, y, vx, vy, ax, ay, targetX, targetY, targetForce,
// phase, temporary, lifetime, fadeTime; floats as bits) up to cap and returns their
// count (or -1 when a cell outside the grid would be read: the grid needs its
// border).
struct Registry {
    std::vector<Material> store;
    std::vector<int *> n_arrays;
    std::vector<std::vector<MaterialInteraction> *> i_arrays;
    ~Registry() {
        for (int *p : n_arrays) delete[] p;
        for (auto *p : i_arrays) delete[] p;
    }
};

// fills the GAME() registry and the factories from the table (see below)
static void setup_registry(Registry &reg, int n, const int32_t *mats, const int32_t *special,
                           const int32_t *reactions, int ni, const int32_t *inter) {
    g_reg = GameReg();
    reg.store.assign((size_t)n, Material());
    std::vector<Material> &store = reg.store;
    g_reg.materials_container.assign((size_t)n, nullptr);
    g_reg.materials_count = n;
    Material *named[7] = {&g_reg.materials_list.GENERIC_AIR, &g_reg.materials_list.GENERIC_SOLID,
                          &g_reg.materials_list.FIRE,        &g_reg.materials_list.WATER,
                          &g_reg.materials_list.LAVA,        &g_reg.materials_list.STEAM,
                          &g_reg.materials_list.OBSIDIAN};
    for (int k = 0; k < 7; k++)
        if (special[k] >= 0 && special[k] < n) g_reg.materials_container[special[k]] = named[k];
    for (int i = 0; i < n; i++)
        if (!g_reg.materials_container[i]) g_reg.materials_container[i] = &store[i];
    g_fac.assign((size_t)n, Factory());
    std::vector<std::vector<int>> n_int((size_t)n, std::vector<int>((size_t)n, 0));
    std::vector<std::vector<std::vector<MaterialInteraction>>> ints(
        (size_t)n, std::vector<std::vector<MaterialInteraction>>((size_t)n));
    for (int j = 0; j < ni; j++) {
        const int32_t *r = inter + 7 * j;
        MaterialInteraction e;
        e.type = r[2];
        e.data1 = (mat_temperature)r[3];
        e.data2 = (mat_id)r[4];
        e.ofsX = r[5];
        e.ofsY = r[6];
        ints[r[0]][r[1]].push_back(e);
    }
    for (int i = 0; i < n; i++) {
        Material &m = *g_reg.materials_container[i];
        const int32_t *r = mats + 10 * i;
        m.id = (mat_id)i;
        m.physicsType = r[0];
        memcpy(&m.density, &r[1], 4);
        m.iterations = r[2];
        m.slipperyness = r[3];
        g_fac[i] = Factory{(u32)r[4], r[5], r[6], r[7], r[8]};
        m.reactions.clear();
        for (int q = 0; q < 4; q++) {
            const int32_t *e = reactions + 12 * i + 3 * q;
            if (!e[0]) continue;
            MaterialInteraction in;
            in.type = e[0];
            in.data1 = (mat_temperature)e[1];
            in.data2 = (mat_id)e[2];
            m.reactions.push_back(in);
        }
        m.nReactions = (int)m.reactions.size();
        m.react = m.nReactions > 0;
        int *cnt = new int[(size_t)n];
        auto *lists = new std::vector<MaterialInteraction>[(size_t)n];
        bool any = false;
        for (int o = 0; o < n; o++) {
            lists[o] = ints[i][o];
            cnt[o] = (int)lists[o].size();
            any = any || cnt[o] > 0;
        }
        m.nInteractions = cnt;
        m.interactions = lists;
        m.interact = any;
        reg.n_arrays.push_back(cnt);
        reg.i_arrays.push_back(lists);
    }

}

// n_ticks world::tick() calls on a grid given as planes. amounts / diffs / settle
// (NULL: the MaterialInstance defaults 2.0, 0, 0) are each cell's fluidAmount,
// fluidAmountDiff and settleCount, read and written back as they are; particle rows
// hold `row` ints (16, or 17 with the carried tile's fluidAmount bits last).
static int tick_planes(int W, int H, int cell_iter, uint32_t seed, uint32_t tick, int n_ticks, int n,
                       const int32_t *mats, const int32_t *special, const int32_t *reactions, int ni,
                       const int32_t *inter, uint16_t *ids, uint32_t *cols, int32_t *temps, uint8_t *moved,
                       float *amounts, float *diffs, uint8_t *settle, int32_t *parts, int row, int cap,
                       long long *draws, const int32_t *zone) {
    Registry reg;
    setup_registry(reg, n, mats, special, reactions, ni, inter);

    // the grid with 16 solid rows above and below, so that no read leaves the array
    const size_t N = (size_t)W * H, pad = (size_t)16 * W;
    std::vector<MaterialInstance> tiles(N + 2 * pad, Tiles_TEST_SOLID);
    std::vector<char> dirty(N), tv1(N), tv2(N);
    std::vector<f32> fx(N), fy(N);
    for (size_t i = 0; i < N; i++) {
        MaterialInstance t(g_reg.materials_container[ids[i]], cols[i], (mat_temperature)temps[i]);
        t.moved = moved[i] != 0;
        if (amounts) t.fluidAmount = amounts[i];
        if (diffs) t.fluidAmountDiff = diffs[i];
        if (settle) t.settleCount = settle[i];
        tiles[pad + i] = t;
    }
    world wd;
    wd.width = W;
    wd.height = H;
    wd.real_tiles = tiles.data() + pad;
    wd.dirty = reinterpret_cast<bool *>(dirty.data());
    wd.tickVisited1 = reinterpret_cast<bool *>(tv1.data());
    wd.tickVisited2 = reinterpret_cast<bool *>(tv2.data());
    wd.flowX = fx.data();
    wd.flowY = fy.data();
    wd.tickZone = zone ? TickZone{zone[0], zone[1], zone[2], zone[3]} : TickZone{0, 0, W, H};
    global.game->Iso.globaldef.cell_iter = cell_iter;
    g_seed = seed;
    g_draws = 0;
    for (int t = 0; t < n_ticks; t++) {
        g_tick = tick + (uint32_t)t;
        g_sweep = 2;
        g_cur = -1;
        wd.tick();
    }
    int ok = 1;
    for (size_t i = 0; i < pad; i++)
        if (tiles[i].mat->id != Tiles_TEST_SOLID.mat->id || tiles[pad + N + i].mat->id != Tiles_TEST_SOLID.mat->id)
            ok = 0;
    for (size_t i = 0; i < N; i++) {
        const MaterialInstance &t = tiles[pad + i];
        ids[i] = (uint16_t)t.mat->id;
        cols[i] = t.color;
        temps[i] = t.temperature;
        moved[i] = t.moved ? 1 : 0;
        if (amounts) amounts[i] = t.fluidAmount;
        if (diffs) diffs[i] = t.fluidAmountDiff;
        if (settle) settle[i] = t.settleCount;
    }
    int np = 0;
    for (CellData *c : wd.cells) {
        if (np < cap) {
            int32_t *o = parts + (size_t)row * np;
            const f32 fv[9] = {c->x, c->y, c->vx, c->vy, c->ax, c->ay, c->targetX, c->targetY, c->targetForce};
            o[0] = (int32_t)c->tile.mat->id;
            o[1] = (int32_t)c->tile.color;
            o[2] = c->tile.temperature;
            memcpy(o + 3, fv, sizeof(fv));
            o[12] = c->phase;
            o[13] = c->temporary;
            o[14] = c->lifetime;
            o[15] = c->fadeTime;
            if (row > 16) memcpy(o + 16, &c->tile.fluidAmount, 4);
        }
        np++;
        delete c;
    }
    if (draws) *draws = g_draws;
    return ok ? np : -1;
}

extern "C" int ref_world_tick(int W, int H, int cell_iter, uint32_t seed, uint32_t tick, int n_ticks, int n,
                              const int32_t *mats, const int32_t *special, const int32_t *reactions, int ni,
                              const int32_t *inter, uint16_t *ids, uint32_t *cols, int32_t *temps, uint8_t *moved,
                              int32_t *parts, int cap, long long *draws) {
    return tick_planes(W, H, cell_iter, seed, tick, n_ticks, n, mats, special, reactions, ni, inter, ids, cols, temps,
                       moved, nullptr, nullptr, nullptr, parts, 16, cap, draws, nullptr);
}

// the same with every cell's fluidAmount, fluidAmountDiff and settleCount in and out,
// particle rows of 17 ints (the carried tile's fluidAmount bits last) and the tick
// zone (x, y, w, h; NULL: the whole world)
extern "C" int ref_world_tick_fluid(int W, int H, int cell_iter, uint32_t seed, uint32_t tick, int n_ticks, int n,
                                    const int32_t *mats, const int32_t *special, const int32_t *reactions, int ni,
                                    const int32_t *inter, uint16_t *ids, uint32_t *cols, int32_t *temps,
                                    uint8_t *moved, float *amounts, float *diffs, uint8_t *settle, int32_t *parts,
                                    int cap, long long *draws, const int32_t *zone) {
    return tick_planes(W, H, cell_iter, seed, tick, n_ticks, n, mats, special, reactions, ni, inter, ids, cols, temps,
                       moved, amounts, diffs, settle, parts, 17, cap, draws, zone);
}

// Timing: the reference's own world::tick() + world::tickCells() on a grid (ids,
// colours, temperatures; liquids at the MaterialInstance default amount) and
// particles (rows of x, y, vx, vy, ax, ay as floats, then id, colour), `warm`
// untimed steps then `steps` timed ones, the chunk tasks on a pool of `threads`
// workers, stopping early once the timed steps pass budget_s seconds (*done = the
// steps timed). Returns their seconds (negative when the grid's padding was
// written: the scene needs its border).
extern "C" double ref_world_bench(int W, int H, int cell_iter, uint32_t seed, int n, const int32_t *mats,
                                  const int32_t *special, const int32_t *reactions, int ni, const int32_t *inter,
                                  const uint16_t *ids, const uint32_t *cols, const int32_t *temps, int n_parts,
                                  const float *pf, const uint32_t *pi, int threads, int warm, int steps,
                                  double budget_s, int *done) {
    Registry reg;
    setup_registry(reg, n, mats, special, reactions, ni, inter);
    const size_t N = (size_t)W * H, pad = (size_t)16 * W;
    std::vector<MaterialInstance> tiles(N + 2 * pad, Tiles_TEST_SOLID);
    std::vector<char> dirty(N), tv1(N), tv2(N);
    std::vector<f32> fx(N), fy(N);
    for (size_t i = 0; i < N; i++) tiles[pad + i] = MaterialInstance(g_reg.materials_container[ids[i]], cols[i],
                                                                      (mat_temperature)temps[i]);
    world wd;
    wd.width = W;
    wd.height = H;
    wd.real_tiles = tiles.data() + pad;
    wd.dirty = reinterpret_cast<bool *>(dirty.data());
    wd.tickVisited1 = reinterpret_cast<bool *>(tv1.data());
    wd.tickVisited2 = reinterpret_cast<bool *>(tv2.data());
    wd.flowX = fx.data();
    wd.flowY = fy.data();
    wd.tickZone = TickZone{0, 0, W, H};
    for (int i = 0; i < n_parts; i++) {
        const float *f = pf + 6 * i;
        const uint32_t *u = pi + 2 * i;
        MaterialInstance t(g_reg.materials_container[u[0]], u[1], 0);
        wd.cells.push_back(new CellData(t, f[0], f[1], f[2], f[3], f[4], f[5]));
    }
    global.game->Iso.globaldef.cell_iter = cell_iter;
    g_seed = seed;
    if (threads > 1) {
        g_pool.start(threads);
        g_vpool.start(1);
    }
    double secs = 0;
    int timed = 0;
    for (int s = 0; s < warm + steps; s++) {
        const auto t0 = std::chrono::steady_clock::now();
        g_tick = (uint32_t)s;
        wd.tick();
        wd.tickCells();
        const auto t1 = std::chrono::steady_clock::now();
        if (s >= warm) {
            secs += std::chrono::duration<double>(t1 - t0).count();
            timed++;
            if (secs > budget_s) break;
        }
    }
    if (done) *done = timed;
    if (threads > 1) {
        g_pool.halt();
        g_vpool.halt();
    }
    int ok = 1;
    for (size_t i = 0; i < pad; i++)
        if (tiles[i].mat->id != Tiles_TEST_SOLID.mat->id || tiles[pad + N + i].mat->id != Tiles_TEST_SOLID.mat->id)
            ok = 0;
    for (CellData *c : wd.cells) delete c;
    return ok ? secs : -secs - 1.0;
}
