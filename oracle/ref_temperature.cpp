// ref_temperature.cpp -- TEST INFRASTRUCTURE ONLY (never linked into the product).
//
// Compiles the reference's own world::tickTemperature (source/engine/world.cpp:
// 1950-2004) so that the oracle's restatement (om_tick_temperature) can be pinned
// against it. oracle/Makefile (target `ref`) extracts that one function, unchanged,
// from the reference tree into _ref/tick_temperature.inc at build time; this file
// supplies minimal stand-ins for the names the function touches (the world's
// width, tickZone, real_tiles and newTemps, MaterialInstance::temperature/mat and
// Material::addTemp/conductionSelf/conductionOther, game_datastruct.hpp:109,
// 142-144,213) and a C entry point. The rest of world.cpp needs SDL and the
// engine, so it is not built.
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <vector>

typedef float f32;
typedef int32_t i32;
typedef uint32_t u32;
typedef int16_t i16;

struct Material {
    u32 addTemp = 0;
    f32 conductionSelf = 1.0;
    f32 conductionOther = 1.0;
};
struct MaterialInstance {
    Material *mat;
    i16 temperature;
};
struct TickZone {
    int x, y, w, h;
};
struct world {
    int width = 0, height = 0;
    TickZone tickZone{};
    MaterialInstance *real_tiles = nullptr;
    i32 *newTemps = nullptr;
    void tickTemperature();
};

#include "tick_temperature.inc"

// One call of world::tickTemperature on a w x h world of material indices `mat`
// and temperatures `temp` (updated in place), with the tick zone (zx, zy, zw, zh)
// and per-material addTemp / conductionSelf / conductionOther.
extern "C" int ref_tick_temperature(int w, int h, const uint16_t *mat, int16_t *temp, int n_mat,
                                    const uint32_t *add_temp, const float *cond_self, const float *cond_other,
                                    int zx, int zy, int zw, int zh) {
    if (w <= 0 || h <= 0 || n_mat <= 0) return -1;
    std::vector<Material> mats((size_t)n_mat);
    for (int k = 0; k < n_mat; k++) {
        mats[k].addTemp = add_temp[k];
        mats[k].conductionSelf = cond_self[k];
        mats[k].conductionOther = cond_other[k];
    }
    const size_t n = (size_t)w * h;
    std::vector<MaterialInstance> tiles(n);
    std::vector<i32> nt(n, 0);
    for (size_t i = 0; i < n; i++) {
        if (mat[i] >= n_mat) return -1;
        tiles[i].mat = &mats[mat[i]];
        tiles[i].temperature = temp[i];
    }
    world wd;
    wd.width = w;
    wd.height = h;
    wd.tickZone = TickZone{zx, zy, zw, zh};
    wd.real_tiles = tiles.data();
    wd.newTemps = nt.data();
    wd.tickTemperature();
    for (size_t i = 0; i < n; i++) temp[i] = tiles[i].temperature;
    return 0;
}
