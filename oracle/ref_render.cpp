// ref_render.cpp -- TEST INFRASTRUCTURE ONLY (never linked into the product).
//
// Compiles the reference's own dirty-pixel texture loop of game::tick (the task
// body of source/engine/game.cpp:1995-2061) so that the oracle's restatement of the
// render pass can be pinned against it. oracle/Makefile (target `ref`) extracts
// that loop, unchanged, into _ref/dirty_loop.inc; this file supplies stand-ins for
// the names it touches (Iso.world's width, height, dirty, real_tiles, flowX/Y and
// prevFlowX/Y, the material fields id, physicsType, alpha, emitColor and
// iterations, GAME()->materials_list.FIRE, the four texture arrays, movingTiles and
// the had* flags) and a C entry point.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <vector>
#include <math.h>
#include <stdlib.h>

typedef float f32;
typedef double f64;
typedef uint32_t u32;
typedef uint16_t u16;
typedef uint8_t u8;

#define ME_ALPHA_TRANSPARENT 0  // source/engine/renderer/renderer_gpu.h:27

enum PhysicsType { AIR = 0, SOLID = 1, SAND = 2, SOUP = 3, GAS = 4, PASSABLE = 5, OBJECT = 5 };

struct Material {
    int id = 0;
    int physicsType = 0;
    u8 alpha = 255;
    u32 emitColor = 0;
    int iterations = 1;
};
struct MaterialInstance {
    Material *mat = nullptr;
    u32 color = 0;
};
struct WorldS {
    int width = 0, height = 0;
    bool *dirty = nullptr;
    MaterialInstance *real_tiles = nullptr;
    f32 *flowX = nullptr, *flowY = nullptr, *prevFlowX = nullptr, *prevFlowY = nullptr;
};
struct IsoS {
    WorldS *world = nullptr;
};
struct MatList {
    Material FIRE;
};
struct GameS {
    MatList materials_list;
};
static GameS g_game;
static GameS *GAME() { return &g_game; }

// One pass of the loop over a w x h world; textures are 4 bytes per cell in the
// loop's own byte order; moving (u16 per material) is accumulated as the loop does.
extern "C" int ref_render_dirty(int w, int h, const uint16_t *id, const uint32_t *colour, uint8_t *dirty,
                                float *flow_x, float *flow_y, float *prev_x, float *prev_y, int n_mat,
                                const int32_t *type, const uint8_t *alpha, const uint32_t *emit, const int32_t *iters,
                                int fire_id, uint8_t *tex_pixels, uint8_t *tex_fire, uint8_t *tex_emission,
                                uint8_t *tex_flow, uint16_t *moving) {
    std::vector<Material> mats((size_t)n_mat);
    for (int k = 0; k < n_mat; k++) {
        mats[k].id = k;
        mats[k].physicsType = type[k];
        mats[k].alpha = alpha[k];
        mats[k].emitColor = emit[k];
        mats[k].iterations = iters[k];
    }
    g_game.materials_list.FIRE.id = fire_id;
    const size_t n = (size_t)w * h;
    std::vector<MaterialInstance> tiles(n);
    for (size_t i = 0; i < n; i++) {
        if (id[i] >= n_mat) return -1;
        tiles[i].mat = &mats[id[i]];
        tiles[i].color = colour[i];
    }
    WorldS world;
    world.width = w;
    world.height = h;
    static_assert(sizeof(bool) == 1, "bool");
    world.dirty = reinterpret_cast<bool *>(dirty);
    world.real_tiles = tiles.data();
    world.flowX = flow_x;
    world.flowY = flow_y;
    world.prevFlowX = prev_x;
    world.prevFlowY = prev_y;
    IsoS Iso;
    Iso.world = &world;
    u8 *dpixels_ar = tex_pixels, *dpixelsFire_ar = tex_fire, *dpixelsEmission_ar = tex_emission,
       *dpixelsFlow_ar = tex_flow;
    u16 *movingTiles = moving;
    bool hadDirty = false, hadFire = false, hadFlow = false;
#include "dirty_loop.inc"
    (void)hadDirty;
    (void)hadFire;
    (void)hadFlow;
    return 0;
}
