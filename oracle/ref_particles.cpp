// ref_particles.cpp -- TEST INFRASTRUCTURE ONLY (never linked into the product).
//
// Compiles the reference's own world::tickCells (source/engine/world.cpp:
// 2030-2195) so that the oracle's free-particle update can be pinned against it.
// oracle/Makefile (target `ref`) extracts that one function, unchanged, from the
// reference tree into _ref/tick_cells.inc; this file supplies stand-ins for the
// names it touches -- CellData (source/engine/game_utils/cells.h:15-36), the
// MaterialInstance fields it reads and copies (game_datastruct.hpp:205-222),
// PhysicsType (game_datastruct.hpp:87-95), and the world's width, height,
// tickZone, real_tiles, dirty and cells -- and a C entry point.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <functional>
#include <vector>
// as the reference's engine/core/mathlib_base.hpp:8-9 does: these make the
// unqualified abs() of tickCells the float overload
#include <math.h>
#include <stdlib.h>

typedef float f32;
typedef int32_t i32;
typedef uint32_t u32;
typedef int16_t i16;
typedef uint8_t u8;

enum PhysicsType { AIR = 0, SOLID = 1, SAND = 2, SOUP = 3, GAS = 4, PASSABLE = 5, OBJECT = 5 };

struct Material {
    int id = 0;
    int physicsType = 0;
};
struct MaterialInstance {
    u32 id = 0;
    Material *mat = nullptr;
    u32 color = 0;
    i16 temperature = 0;
    bool moved = false;
    f32 fluidAmount = 2.0f;
    f32 fluidAmountDiff = 0.0f;
    u8 settleCount = 0;
};
struct CellData {
    MaterialInstance tile{};
    f32 x = 0, y = 0, vx = 0, vy = 0, ax = 0, ay = 0;
    f32 targetX = 0, targetY = 0, targetForce = 0;
    bool phase = false;
    bool temporary = false;
    int lifetime = 0;
    int fadeTime = 60;
    u8 inObjectState = 0;
    std::function<void()> killCallback = []() {};
};
struct TickZone {
    int x, y, w, h;
};
struct world {
    int width = 0, height = 0;
    TickZone tickZone{};
    MaterialInstance *real_tiles = nullptr;
    bool *dirty = nullptr;
    std::vector<CellData *> cells;
    void tickCells();
};

#include "tick_cells.inc"

// The particle record of the oracle / C ABI (60 bytes).
struct Part {
    float x, y, vx, vy, ax, ay, tx, ty, tf;
    int32_t lifetime, fade;
    uint32_t colour;
    int32_t scalar;
    uint16_t id;
    uint8_t flags, bits;
    int16_t temperature;
    uint16_t reserved;
};
static_assert(sizeof(Part) == 60, "particle record");

// One world::tickCells on a w x h grid. Cells: material index, colour, fluid amount
// (Q16.16, exact in float for the amounts used) and the material types; particles
// in list order; the tick zone (x, y, w, h; NULL: the whole world). Outputs the grid
// (same arrays, updated), the dirty marks, and the surviving particles in order
// (*n_out).
static int tick_cells(int w, int h, uint16_t *id, uint32_t *colour, int32_t *amount, uint8_t *dirty,
                      const int32_t *mat_type, int n_mat, const Part *in, int n_in, Part *out, int *n_out,
                      const int32_t *zone) {
    std::vector<Material> mats((size_t)n_mat);
    for (int k = 0; k < n_mat; k++) {
        mats[k].id = k;
        mats[k].physicsType = mat_type[k];
    }
    const size_t n = (size_t)w * h;
    std::vector<MaterialInstance> tiles(n);
    std::vector<uint8_t> dflag(n, 0);
    for (size_t i = 0; i < n; i++) {
        if (id[i] >= n_mat) return -1;
        tiles[i].id = id[i];
        tiles[i].mat = &mats[id[i]];
        tiles[i].color = colour[i];
        tiles[i].fluidAmount = (float)amount[i] / 65536.0f;
    }
    world wd;
    wd.width = w;
    wd.height = h;
    wd.tickZone = zone ? TickZone{zone[0], zone[1], zone[2], zone[3]} : TickZone{0, 0, w, h};
    wd.real_tiles = tiles.data();
    static_assert(sizeof(bool) == 1, "bool");
    wd.dirty = reinterpret_cast<bool *>(dflag.data());
    std::vector<CellData *> keep;
    for (int i = 0; i < n_in; i++) {
        const Part &p = in[i];
        if (p.id >= n_mat) return -1;
        CellData *c = new CellData();
        c->tile.id = p.id;
        c->tile.mat = &mats[p.id];
        c->tile.color = p.colour;
        c->tile.fluidAmount = (float)p.scalar / 65536.0f;
        c->x = p.x;
        c->y = p.y;
        c->vx = p.vx;
        c->vy = p.vy;
        c->ax = p.ax;
        c->ay = p.ay;
        c->targetX = p.tx;
        c->targetY = p.ty;
        c->targetForce = p.tf;
        c->lifetime = p.lifetime;
        c->fadeTime = p.fade;
        c->phase = (p.bits & 1) != 0;
        c->temporary = (p.bits & 2) != 0;
        c->inObjectState = (uint8_t)((p.bits >> 2) & 3);
        wd.cells.push_back(c);
    }
    std::vector<const Part *> src;  // to carry the fields the function does not touch
    for (int i = 0; i < n_in; i++) src.push_back(&in[i]);
    std::vector<CellData *> order = wd.cells;
    wd.tickCells();
    int m = 0;
    for (CellData *c : wd.cells) {
        // the survivor's original record (pointers are unique until deleted)
        int k = (int)(std::find(order.begin(), order.end(), c) - order.begin());
        Part p = *src[k];
        p.x = c->x;
        p.y = c->y;
        p.vx = c->vx;
        p.vy = c->vy;
        p.lifetime = c->lifetime;
        p.bits = (uint8_t)((c->phase ? 1 : 0) | (c->temporary ? 2 : 0) | ((c->inObjectState & 3) << 2));
        out[m++] = p;
    }
    *n_out = m;
    for (size_t i = 0; i < n; i++) {
        id[i] = (uint16_t)tiles[i].mat->id;
        colour[i] = tiles[i].color;
        amount[i] = (int32_t)std::lround((double)tiles[i].fluidAmount * 65536.0);
        dirty[i] = dflag[i];
    }
    for (CellData *c : wd.cells) delete c;
    return 0;
}

extern "C" int ref_tick_cells(int w, int h, uint16_t *id, uint32_t *colour, int32_t *amount, uint8_t *dirty,
                              const int32_t *mat_type, int n_mat, const Part *in, int n_in, Part *out, int *n_out) {
    return tick_cells(w, h, id, colour, amount, dirty, mat_type, n_mat, in, n_in, out, n_out, nullptr);
}

extern "C" int ref_tick_cells_zone(int w, int h, uint16_t *id, uint32_t *colour, int32_t *amount, uint8_t *dirty,
                                   const int32_t *mat_type, int n_mat, const Part *in, int n_in, Part *out,
                                   int *n_out, const int32_t *zone) {
    return tick_cells(w, h, id, colour, amount, dirty, mat_type, n_mat, in, n_in, out, n_out, zone);
}
