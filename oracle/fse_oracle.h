/*
 * fse_oracle.h -- CPU oracle for the falling-sand world tick.
 *
 * TEST INFRASTRUCTURE ONLY. This library is the checker that the CUDA path is
 * compared against; it is loaded by tests/, by __graft_entry__.smoke() and by
 * bench.py's CPU-baseline leg, and never by the product library.
 *
 * It restates, in plain C, the reference's cell update `world::tick()`
 * (source/engine/world.cpp:1036-1948), its vertical-flow helper
 * (world.cpp:1021-1034), the bounds policy of getTile/setTile
 * (world.cpp:999-1008), the free-particle update `world::tickCells()`
 * (world.cpp:2030-2195), the built-in material table
 * (source/engine/game_datastruct.cpp:69-111,117-300) and the tile factories
 * (game_datastruct.cpp:320-574), under two update orders:
 *
 *   OM_ORDER_SEQ   the reference order: 4 chunk colours x in-chunk sweeps A/B/C,
 *                  each sweep bottom-to-top, left-to-right, in place;
 *   OM_ORDER_PART  the partitioned (lattice) order executed by the GPU, in which
 *                  every cell move of a sub-phase is race-free.
 *
 * Both orders use the same rules, the same counter-based RNG and the same
 * Q16.16 fixed-point fluid arithmetic, so the conservation ledger holds for both
 * and OM_ORDER_PART is bit-exact with the CUDA kernels.
 *
 * Parity pinning: the reference ships no test, fixture or golden vector for this
 * path (its tests cover only FFI/reflection/promises), and its world.cpp as a whole
 * cannot be compiled without SDL2/xmake. Self-contained pieces of the reference's
 * own code are compiled in place by oracle/Makefile (target `ref`) and pin this
 * restatement bit for bit: world::tickCells (the particle update),
 * world::tickTemperature, the dirty-pixel loop of game::tick and the vendored LZ4.
 * The cell update itself (libc rand(), float fluid) is anchored on this
 * restatement, which cites the reference line by line, plus the committed fixtures
 * under tests/golden/ generated from it.
 */
#ifndef FSE_ORACLE_H
#define FSE_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define OM_ORDER_SEQ 0
#define OM_ORDER_PART 1

/* Same byte layout as fse_particle in include/fse.h (60 bytes). */
typedef struct om_particle {
    float x, y, vx, vy, ax, ay;
    float target_x, target_y, target_force;
    int32_t lifetime, fade_time;
    uint32_t colour;
    int32_t scalar;
    uint16_t id;
    uint8_t flags;
    uint8_t bits; /* bit0 phase, bit1 temporary, bits2-3 inObjectState */
    int16_t temperature; /* temperature of a SOUP tile (its scalar holds the amount) */
    uint16_t reserved;
} om_particle;

typedef struct om_world om_world;

/* material table (process-global, like GAME()->materials_array) */
void om_materials_reset_builtin(void);
int om_material_register(int s_id, const char *name, const char *index_name, int physics_type, int slipperyness,
                         int alpha, float density, int iterations, int emit, uint32_t emit_colour, uint32_t colour);
int om_material_set_factory(int mat, uint32_t base, int shift, int lo, int mod, int32_t scalar);
int om_material_set_reaction(int mat, int kind, int temperature, int result);
/* Material::addTemp / conductionSelf / conductionOther */
int om_material_set_conduction(int mat, uint32_t add_temp, float cond_self, float cond_other);
/* addTemp, conductionSelf bits, conductionOther bits */
void om_material_conduction(int mat, uint32_t out[3]);
/* temperature of a new SOUP tile of this material (TilesCreate) */
int om_material_set_factory_temperature(int mat, int32_t temperature);
int om_material_set_interaction(int mat, int other, int kind, int data1, int data2, int ofs_x, int ofs_y);
int om_material_count(void);
int om_material_tile_temperature(int mat);
int om_material_rules(int32_t *react, int32_t *inter, int cap);
int om_material_find(const char *index_name);
/* 16 ints: type, density bits, iterations, slip, max_stab, alpha, colour, emit, emit_colour,
 * f_base, f_shift, f_lo, f_mod, f_scalar, n_react, interact */
void om_material_get(int id, int32_t out[16]);

/* worlds */
om_world *om_world_new(int w, int h, int chunk, int cell_iter, uint32_t seed);
void om_world_free(om_world *wd);
void om_world_set(om_world *wd, const uint16_t *id, const uint32_t *col, const int32_t *sc, const uint8_t *fl,
                  const int32_t *df);
void om_world_get(const om_world *wd, uint16_t *id, uint32_t *col, int32_t *sc, uint8_t *fl, int32_t *df);
void om_world_generate(om_world *wd, int kind, uint32_t seed);
void om_world_set_tick(om_world *wd, uint32_t tick);
uint32_t om_world_get_tick(const om_world *wd);

/* one world::tick() under the given order; returns the number of race violations
 * found by the instrumented checker when check_races != 0, else 0 */
long om_world_tick(om_world *wd, int order, int check_races);
/* one world::tickCells(); returns the number of particles after the tick */
int om_particles_tick(om_world *wd);
/* world::tick() followed by world::tickCells(), n times */
void om_world_step(om_world *wd, int order, int n);
/* world::tickTemperature (world.cpp:1950-2004), one Jacobi step over every cell */
void om_tick_temperature(om_world *wd);
/* om_world_step also runs om_tick_temperature after ticks whose index is 2 mod 4 */
void om_world_set_temperature(om_world *wd, int on);
/* f32 liquid amounts and diffs: the reference's own float arithmetic (the GPU's
 * FSE_CFG_F32_FLUID); set before the world is generated or loaded */
void om_world_set_f32(om_world *wd, int on);
/* world::tickZone: the rectangle inside the world whose chunks tick (from its
 * corner), whose particles move and whose temperatures conduct; -1 if it is not
 * inside the world */
int om_world_set_tick_zone(om_world *wd, int x, int y, int w, int h);
/* chunk .pack codec (chunk.cpp:219-330): LZ4 block format helpers and whole-world
 * pack/unpack, chunks row-major; see fse_oracle.c for the layout */
int om_lz4_bound(int n);
int om_lz4_encode(const uint8_t *buf, int n, uint8_t *dst, int cap);
int om_lz4_decode(const uint8_t *src, int n, uint8_t *dst, int cap);
int om_world_pack(const om_world *wd, int phase, uint8_t *out, int64_t cap, int64_t *offsets);
int om_world_unpack(om_world *wd, const uint8_t *in, const int64_t *offsets, int n_chunks, int8_t *phases);
/* per-cell temperature (i16): SOUP cells' own plane, the scalar of the others */
void om_temperature_get(const om_world *wd, int16_t *out);
void om_temperature_set(om_world *wd, const int16_t *in);

int om_particles_count(const om_world *wd);
void om_particles_get(const om_world *wd, om_particle *out);
void om_particles_set(om_world *wd, const om_particle *in, int n);

/* ledger: 6 rows of om_material_count() int64: created_n, destroyed_n, exited_n,
 * created_f, destroyed_f, exited_f (fluid in Q16.16 units) */
void om_ledger_get(const om_world *wd, int64_t *out);
void om_ledger_reset(om_world *wd);
/* census: 4 rows: grid_count, grid_fluid (amount + pending diff), part_count, part_fluid */
void om_census(const om_world *wd, int64_t *out);

/* FP64 kinematics oracle of one particle step against the current grid, without
 * deposits: out4 = final (x, y, vx, vy) in double, ev = outcome code
 * (0 flying, 1 exit, 2 killed, 3 collide-direct, 4 collide-spiral), sub = sub-step
 * of the event (-1 if none). The same routine in FP32 is om_particles_kinematics_f32. */
void om_particles_kinematics_f64(const om_world *wd, const om_particle *in, int n, double *out4, int32_t *ev,
                                 int32_t *sub);
void om_particles_kinematics_f32(const om_world *wd, const om_particle *in, int n, float *out4, int32_t *ev,
                                 int32_t *sub);

/* rigid OBJECT bodies (axis-aligned or rotated tile boxes) */
typedef struct om_body {
    float x, y, sin_a, cos_a; /* position and sin/cos of the body angle (computed once on the host) */
    int32_t w, h;             /* tile box of the body */
    uint16_t id;              /* material of every tile of the body */
    uint16_t pad;
    uint32_t colour;
    int32_t n_sand, n_soup;   /* displacements seen by the last stamp (body damping) */
    int32_t n_placed, n_recovered;
} om_body; /* 48 bytes, same layout as fse_body */
void om_object_stamp(om_world *wd, om_body *bodies, int n);
/* erase the stamped tiles again; returns the number of OBJECT cells removed */
long om_object_readback(om_world *wd, const om_body *bodies, int n);
/* 1 bit per cell: cell physics type == OBJECT; bits LSB-first, row-major */
void om_object_mask(const om_world *wd, uint8_t *bits);

void om_set_threads(int n);
/* test hook: override the sub-phase lattice of one sweep (px = 0 restores it) */
void om_debug_set_lattice(int sweep, int px, int py);

/* headless render textures (game.cpp:1994-2067, world.cpp:2006-2028), 4 bytes
 * r, g, b, a per cell; which: 0 pixels, 1 emission, 2 fire, 3 flow, 4 particles */
void om_render_enable(om_world *w);
void om_render_dirty(om_world *w, int64_t *moving);
void om_render_cells(om_world *w);
void om_render_get(const om_world *w, int which, uint32_t *out);
void om_render_dirty_get(const om_world *w, uint8_t *out);
void om_render_set(om_world *wd, const uint8_t *dirty, const int32_t *flow, const float *pflow);
void om_render_pflow_get(const om_world *wd, float *out);

/* solid islands: world::physicsCheck (world.cpp:3330-3445) and every region at once */
typedef struct om_island {
    int32_t root, cells, min_x, min_y, max_x, max_y;
} om_island;
int om_physics_check(om_world *w, int x, int y, int32_t bbox[4], uint32_t *pixels, int pixels_cap);
int om_islands(om_world *w, int max_cells, int remove, om_island *out, int cap);

#ifdef __cplusplus
}
#endif
#endif
