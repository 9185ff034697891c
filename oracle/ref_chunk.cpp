// ref_chunk.cpp -- TEST INFRASTRUCTURE ONLY (never linked into the product).
//
// Compiles the reference's own Chunk::ChunkWrite and Chunk::ChunkRead
// (source/engine/chunk.cpp:68-330) with MaterialInstanceData (chunk.hpp:26-30),
// extracted unchanged by oracle/Makefile (target `ref`), against the reference's
// vendored LZ4, so that the .pack files of the oracle and of the device codec can be
// checked against the files the reference writes and against what it reads back.
// This file supplies the chunk's few members, a MaterialInstance with the fields the
// two functions touch, the GAME() material array and an error macro that drops the
// message.
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <format>
#include <fstream>
#include <stdexcept>
#include <string>
#include <vector>

#include "lz4.h"

typedef uint32_t u32;
typedef uint16_t u16;
typedef int16_t i16;
typedef int8_t i8;
using mat_id = u32;
using mat_instance_id = mat_id;
using mat_temperature = i16;

#include "chunk_data.inc"

struct Material {
    u32 id = 0;
};
struct MaterialInstance {
    u32 id = 0;
    Material *mat = nullptr;
    u32 color = 0;
    i16 temperature = 0;
};
struct GameReg {
    std::vector<Material *> materials_array;
};
static GameReg g_reg;
static GameReg *GAME() { return &g_reg; }

static const int CHUNK_W = 128, CHUNK_H = 128;
#define METADOT_ERROR(msg) ((void)(msg))

struct Chunk {
    int x = 0, y = 0;
    MaterialInstance *tiles = nullptr, *layer2 = nullptr;
    u32 *background = nullptr;
    bool hasTileCache = false, hasMeta = false;
    int8_t generationPhase = 0;
    std::string pack_filename;
    void ChunkWrite(MaterialInstance *tiles, MaterialInstance *layer2, u32 *background);
    void ChunkRead();
};

#include "chunk_write.inc"
#include "chunk_read.inc"

static std::vector<Material> g_mats;
static void materials() {
    g_mats.assign(1024, Material());
    g_reg.materials_array.assign(1024, nullptr);
    for (int i = 0; i < 1024; i++) {
        g_mats[i].id = (u32)i;
        g_reg.materials_array[i] = &g_mats[i];
    }
}

// ChunkWrite of one 128 x 128 chunk (ids, colours, temperatures; no second layer and
// no background, as zeros) to `path` with the generation phase
extern "C" int ref_chunk_write(const char *path, int phase, const uint16_t *ids, const uint32_t *cols,
                               const int16_t *temps) {
    materials();
    const int n = CHUNK_W * CHUNK_H;
    std::vector<MaterialInstance> tiles(n), layer2(n);
    std::vector<u32> bg(n, 0u);
    for (int i = 0; i < n; i++) {
        tiles[i].mat = g_reg.materials_array[ids[i]];
        tiles[i].id = ids[i];
        tiles[i].color = cols[i];
        tiles[i].temperature = temps[i];
        layer2[i].mat = g_reg.materials_array[0];
    }
    Chunk c;
    c.pack_filename = path;
    c.generationPhase = (int8_t)phase;
    c.ChunkWrite(tiles.data(), layer2.data(), bg.data());
    return 0;
}

// ChunkRead of `path`: the tiles' material ids, colours and temperatures and the phase
extern "C" int ref_chunk_read(const char *path, uint16_t *ids, uint32_t *cols, int16_t *temps, int *phase) {
    materials();
    Chunk c;
    c.pack_filename = path;
    try {
        c.ChunkRead();
    } catch (const std::exception &) {
        return -1;
    }
    for (int i = 0; i < CHUNK_W * CHUNK_H; i++) {
        ids[i] = (uint16_t)c.tiles[i].mat->id;
        cols[i] = c.tiles[i].color;
        temps[i] = c.tiles[i].temperature;
    }
    *phase = c.generationPhase;
    delete[] c.tiles;
    delete[] c.layer2;
    delete[] c.background;
    return 0;
}
