// ref_materials.cpp -- TEST INFRASTRUCTURE ONLY (never linked into the product).
//
// Compiles the reference's own built-in material list -- test() of
// source/engine/game_datastruct.cpp:70-111 with the Material constructor it calls
// (game_datastruct.cpp:40-52) and the delegating constructors of
// game_datastruct.hpp:160-167 -- so that the material table restated here can be
// checked against it; and the tile struct MaterialInstance (game_datastruct.hpp:
// 206-224, with its size assertion), whose field offsets the library's default
// array-of-structs tile layout must match. oracle/Makefile (target `ref`) extracts the three pieces,
// unchanged, into _ref/; this file supplies a stand-in Material with the fields they
// set, the GAME() registry they fill, and a C entry point.
#include <cstddef>
#include <cstdint>
#include <cstring>
#include <string>

typedef uint32_t mat_id;
typedef uint32_t u32;
typedef uint8_t u8;
typedef float f32;
typedef int16_t i16;
typedef mat_id mat_instance_id;
typedef i16 mat_temperature;

enum PhysicsType { AIR = 0, SOLID = 1, SAND = 2, SOUP = 3, GAS = 4, PASSABLE = 5, OBJECT = 5 };

struct Material {
    std::string name, index_name;
    mat_id id = 0;
    PhysicsType physicsType = AIR;
    int slipperyness = 0;
    u8 alpha = 0;
    f32 density = 0;
    int iterations = 0;
    int emit = 0;
    u32 emitColor = 0;
    u32 color = 0;
#include "material_ctors.inc"
};
#include "material_ctor_def.inc"

#include "material_instance.inc"

// sizeof and the offsets of id, mat, color, temperature, moved, fluidAmount,
// fluidAmountDiff, settleCount
extern "C" void ref_tile_layout(int32_t *out) {
    const int32_t v[9] = {(int32_t)sizeof(MaterialInstance),
                          (int32_t)offsetof(MaterialInstance, id),
                          (int32_t)offsetof(MaterialInstance, mat),
                          (int32_t)offsetof(MaterialInstance, color),
                          (int32_t)offsetof(MaterialInstance, temperature),
                          (int32_t)offsetof(MaterialInstance, moved),
                          (int32_t)offsetof(MaterialInstance, fluidAmount),
                          (int32_t)offsetof(MaterialInstance, fluidAmountDiff),
                          (int32_t)offsetof(MaterialInstance, settleCount)};
    memcpy(out, v, sizeof(v));
}

struct MaterialsList {
    Material GENERIC_AIR, GENERIC_SOLID, GENERIC_SAND, GENERIC_LIQUID, GENERIC_GAS, GENERIC_PASSABLE, GENERIC_OBJECT,
        STONE, GRASS, DIRT, SMOOTH_STONE, COBBLE_STONE, SMOOTH_DIRT, COBBLE_DIRT, SOFT_DIRT, WATER, LAVA, CLOUD,
        GOLD_ORE, GOLD_MOLTEN, GOLD_SOLID, IRON_ORE, OBSIDIAN, STEAM, SOFT_DIRT_SAND, FIRE, FLAT_COBBLE_STONE,
        FLAT_COBBLE_DIRT;
};
struct GameS {
    MaterialsList materials_list;
    int materials_count = 0;
};
static GameS g_game;
static GameS *GAME() { return &g_game; }

#include "materials_test.inc"

// After test(): per material (in id order) 10 ints -- id, physicsType, slipperyness,
// alpha, density bits, iterations, emit, emitColor, color, 0 -- and the index names
// (48 bytes each, NUL-terminated). Returns the number of materials.
extern "C" int ref_materials(int32_t *out, char *names, int cap) {
    g_game = GameS();
    test();
    MaterialsList &L = g_game.materials_list;
    Material *all[] = {&L.GENERIC_AIR, &L.GENERIC_SOLID, &L.GENERIC_SAND, &L.GENERIC_LIQUID, &L.GENERIC_GAS,
                       &L.GENERIC_PASSABLE, &L.GENERIC_OBJECT, &L.STONE, &L.GRASS, &L.DIRT, &L.SMOOTH_STONE,
                       &L.COBBLE_STONE, &L.SMOOTH_DIRT, &L.COBBLE_DIRT, &L.SOFT_DIRT, &L.WATER, &L.LAVA, &L.CLOUD,
                       &L.GOLD_ORE, &L.GOLD_MOLTEN, &L.GOLD_SOLID, &L.IRON_ORE, &L.OBSIDIAN, &L.STEAM,
                       &L.SOFT_DIRT_SAND, &L.FIRE, &L.FLAT_COBBLE_STONE, &L.FLAT_COBBLE_DIRT};
    const int n = (int)(sizeof(all) / sizeof(all[0]));
    for (int k = 0; k < n && k < cap; k++) {
        const Material &m = *all[k];
        int32_t db;
        memcpy(&db, &m.density, 4);
        const int32_t v[10] = {(int32_t)m.id, (int32_t)m.physicsType, m.slipperyness, m.alpha, db, m.iterations,
                               m.emit, (int32_t)m.emitColor, (int32_t)m.color, 0};
        memcpy(out + 10 * k, v, sizeof(v));
        strncpy(names + 48 * k, m.index_name.c_str(), 47);
        names[48 * k + 47] = 0;
    }
    return n;
}
