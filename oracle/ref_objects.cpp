// ref_objects.cpp -- TEST INFRASTRUCTURE ONLY (never linked into the product).
//
// Compiles the reference's own rigid-body tile loops of game::tick -- the stamp
// (source/engine/game.cpp:1766-1813, before the tick) and the readback (1907-1967,
// after it) -- so that the oracle's restatement of OBJECT stamping can be pinned
// against them. oracle/Makefile (target `ref`) extracts each loop, unchanged, into
// _ref/stamp_loop.inc and _ref/readback_loop.inc; this file supplies stand-ins for
// the names they touch (the body's tiles, size, position, sin/cos and velocity
// calls, Iso.world's grid, dirty marks and particle list, the texture array the
// readback paints, GAME()->materials_list.GENERIC_AIR, Tiles_NOTHING) and C entry
// points. The stamp draws particle velocities from libc rand(); those are the only
// outputs the pin does not compare.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <format>
#include <stdexcept>
#include <vector>
#include <math.h>
#include <stdlib.h>

typedef float f32;
typedef uint32_t u32;
typedef int16_t i16;
typedef uint8_t u8;

enum PhysicsType { AIR = 0, SOLID = 1, SAND = 2, SOUP = 3, GAS = 4, PASSABLE = 5, OBJECT = 5 };

struct Material {
    int id = 0;
    int physicsType = 0;
    u8 alpha = 255;
};
struct MaterialInstance {
    u32 id = 0;
    Material *mat = nullptr;
    u32 color = 0;
    i16 temperature = 0;
    f32 fluidAmount = 2.0f;
};
static Material g_air;  // GENERIC_AIR, set per call
static MaterialInstance Tiles_NOTHING;
struct CellData {
    MaterialInstance tile;
    f32 x, y, vx, vy, ax, ay;
    CellData(MaterialInstance t, f32 x_, f32 y_, f32 vx_, f32 vy_, f32 ax_, f32 ay_)
        : tile(t), x(x_), y(y_), vx(vx_), vy(vy_), ax(ax_), ay(ay_) {}
};
struct Vec2 {
    f32 x, y;
};
struct Body {
    int n_sand = 0, n_soup = 0;  // velocity damping calls, by kind
    Vec2 GetLinearVelocity() const { return {1.0f, 1.0f}; }
    void SetLinearVelocity(Vec2) {}
    f32 GetAngularVelocity() const { return 1.0f; }
    void SetAngularVelocity(f32 v) {
        if (v == (f32)0.98) n_sand++;
        if (v == (f32)0.99) n_soup++;
    }
};
struct RigidBodyS {
    int matWidth = 0, matHeight = 0;
    MaterialInstance *tiles = nullptr;
    Body *body = nullptr;
};
struct WorldS {
    int width = 0, height = 0;
    std::vector<MaterialInstance> real_tiles;
    bool *dirty = nullptr;
    std::vector<CellData *> cells;
    void addCell(CellData *c) { cells.push_back(c); }
};
struct GlobalDef {
    bool draw_load_zones = false;
};
struct IsoS {
    WorldS *world = nullptr;
    GlobalDef globaldef;
};
struct MatList {
    Material GENERIC_AIR;
};
struct GameS {
    MatList materials_list;
};
static GameS g_game;
static GameS *GAME() { return &g_game; }
#define ME_ASSERT(x) (void)(x)
#define METADOT_ERROR(x) (void)(x)

struct Grid {
    std::vector<Material> mats;
    WorldS world;
    IsoS Iso;
};

// the grid as arrays <-> the stand-in world
static int grid_in(Grid &g, int w, int h, const uint16_t *id, const uint32_t *colour, const int32_t *type,
                   const uint8_t *alpha, int n_mat, int air_id, uint8_t *dirty) {
    g.mats.resize((size_t)n_mat);
    for (int k = 0; k < n_mat; k++) {
        g.mats[k].id = k;
        g.mats[k].physicsType = type[k];
        g.mats[k].alpha = alpha[k];
    }
    g_game.materials_list.GENERIC_AIR = g.mats[air_id];
    Tiles_NOTHING = MaterialInstance{(u32)air_id, &g.mats[air_id], 0, 0, 2.0f};
    g.world.width = w;
    g.world.height = h;
    g.world.real_tiles.resize((size_t)w * h);
    for (size_t i = 0; i < (size_t)w * h; i++) {
        if (id[i] >= n_mat) return -1;
        g.world.real_tiles[i] = MaterialInstance{id[i], &g.mats[id[i]], colour[i], 0, 2.0f};
    }
    static_assert(sizeof(bool) == 1, "bool");
    g.world.dirty = reinterpret_cast<bool *>(dirty);
    g.Iso.world = &g.world;
    return 0;
}
static void grid_out(const Grid &g, uint16_t *id, uint32_t *colour) {
    for (size_t i = 0; i < g.world.real_tiles.size(); i++) {
        id[i] = (uint16_t)g.world.real_tiles[i].mat->id;
        colour[i] = g.world.real_tiles[i].color;
    }
}

// Stamp bodies (x, y, sin, cos, w, h, tile material, colour: 8 floats/ints each) in
// order. Ejected particles: out_parts (tile id, colour, x, y as 4 x 4 bytes each),
// per body the sand and liquid displacements.
extern "C" int ref_object_stamp(int w, int h, uint16_t *id, uint32_t *colour, uint8_t *dirty, const int32_t *type,
                                const uint8_t *alpha, int n_mat, int air_id, const float *bodyf, const int32_t *bodyi,
                                int n_bodies, int32_t *counts, float *out_parts, int cap, int *n_parts) {
    Grid g;
    if (grid_in(g, w, h, id, colour, type, alpha, n_mat, air_id, dirty)) return -1;
    IsoS &Iso = g.Iso;
    srand(1);
    for (int b = 0; b < n_bodies; b++) {
        const f32 x = bodyf[4 * b + 0], y = bodyf[4 * b + 1], s = bodyf[4 * b + 2], c = bodyf[4 * b + 3];
        const int bw = bodyi[4 * b + 0], bh = bodyi[4 * b + 1], mid = bodyi[4 * b + 2];
        std::vector<MaterialInstance> tiles((size_t)bw * bh,
                                            MaterialInstance{(u32)mid, &g.mats[mid], (u32)bodyi[4 * b + 3], 0, 2.0f});
        Body body;
        RigidBodyS rb;
        rb.matWidth = bw;
        rb.matHeight = bh;
        rb.tiles = tiles.data();
        rb.body = &body;
        RigidBodyS *cur = &rb;
#include "stamp_dirs.inc"
#include "stamp_loop.inc"
        counts[2 * b] = body.n_sand;
        counts[2 * b + 1] = body.n_soup;
    }
    int m = 0;
    for (CellData *cd : g.world.cells) {
        if (m < cap) {
            uint32_t rec[2] = {(uint32_t)cd->tile.mat->id, cd->tile.color};
            memcpy(out_parts + 4 * m, rec, 8);
            out_parts[4 * m + 2] = cd->x;
            out_parts[4 * m + 3] = cd->y;
        }
        m++;
        delete cd;
    }
    *n_parts = m;
    grid_out(g, id, colour);
    return 0;
}

// Read the bodies back in order; per body the tiles found (recovered) and the tiles
// the body loses (not found, its own cell AIR). The readback also paints the pixel
// texture (4 bytes per cell), as the reference does.
extern "C" int ref_object_readback(int w, int h, uint16_t *id, uint32_t *colour, uint8_t *dirty,
                                   const int32_t *type, const uint8_t *alpha, int n_mat, int air_id,
                                   const float *bodyf, const int32_t *bodyi, int n_bodies, int32_t *counts,
                                   uint8_t *pixels) {
    Grid g;
    if (grid_in(g, w, h, id, colour, type, alpha, n_mat, air_id, dirty)) return -1;
    IsoS &Iso = g.Iso;
    u8 *dpixels_ar = pixels;
    for (int b = 0; b < n_bodies; b++) {
        const f32 x = bodyf[4 * b + 0], y = bodyf[4 * b + 1], s = bodyf[4 * b + 2], c = bodyf[4 * b + 3];
        const int bw = bodyi[4 * b + 0], bh = bodyi[4 * b + 1], mid = bodyi[4 * b + 2];
        std::vector<MaterialInstance> tiles((size_t)bw * bh,
                                            MaterialInstance{(u32)mid, &g.mats[mid], (u32)bodyi[4 * b + 3], 0, 2.0f});
        Body body;
        RigidBodyS rb;
        rb.matWidth = bw;
        rb.matHeight = bh;
        rb.tiles = tiles.data();
        rb.body = &body;
        RigidBodyS *cur = &rb;
        // every tile found erases one non-AIR cell
        auto air_cells = [&]() {
            long k = 0;
            for (const MaterialInstance &t : g.world.real_tiles) k += t.mat->physicsType == AIR;
            return k;
        };
        const long air0 = air_cells();
#include "readback_dirs.inc"
#include "readback_loop.inc"
        int lost = 0;
        for (const MaterialInstance &t : tiles) lost += t.mat->id == air_id;
        counts[2 * b] = (int)(air_cells() - air0);  // recovered
        counts[2 * b + 1] = lost;
    }
    grid_out(g, id, colour);
    return 0;
}
