/*
 * fse.h -- C ABI of the GB300 falling-sand world tick.
 *
 * Drop-in boundary for the reference engine's world update. Every function is
 * extern "C", takes plain pointers and sizes, returns an int status (0 = FSE_OK,
 * negative = error) and never throws. Worlds are opaque handles used by one host
 * thread at a time; each world is bound to one CUDA stream. Device memory is owned
 * by the library and released by fse_world_destroy().
 *
 * Reference interfaces replaced (paths relative to the reference project root):
 *   fse_materials_begin       InitMaterials()            source/engine/game_datastruct.cpp:117-280
 *   fse_material_register     RegisterMaterial(...)      source/engine/game_datastruct.cpp:282-289
 *   fse_materials_push        PushMaterials()            source/engine/game_datastruct.cpp:291-300
 *   fse_materials_load_lua    Lua materials_register()   source/engine/game_basic.cpp:79-81
 *   fse_world_create          world::init (grids)        source/engine/world.cpp:43-145
 *   fse_world_tick            world::tick()              source/engine/world.cpp:1036-1948
 *   fse_particles_tick        world::tickCells()         source/engine/world.cpp:2030-2195
 *   fse_particles_add         world::addCell(CellData*)  source/engine/world.cpp:2292
 *   fse_world_get_tile/set    world::getTile/setTile     source/engine/world.cpp:999-1008
 *   fse_world_upload/download_tiles  real_tiles (MaterialInstance[]) source/engine/game_datastruct.hpp:205-222
 *   fse_object_stamp          rigid-body tile stamping   source/engine/game.cpp:1768-1814
 *   fse_object_readback       rigid-body tile readback   source/engine/game.cpp:1896-1983
 *   fse_world_tick_temperature world::tickTemperature()  source/engine/world.cpp:1950-2004
 *   fse_world_pack/unpack     Chunk::ChunkWrite/ChunkRead source/engine/chunk.cpp:68-330
 */
#ifndef FSE_H
#define FSE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------ status codes */
#define FSE_OK 0
#define FSE_E_INVAL (-1)    /* bad argument or handle */
#define FSE_E_NOMEM (-2)    /* device or host allocation failed */
#define FSE_E_BUDGET (-3)   /* admission refused by the HBM budget */
#define FSE_E_CUDA (-4)     /* CUDA runtime error */
#define FSE_E_TIMEOUT (-5)  /* a bounded device wait gave up */
#define FSE_E_CAPACITY (-6) /* particle / spawn capacity exceeded (excess dropped) */
#define FSE_E_STATE (-7)    /* call not valid in the current state */
#define FSE_E_BOUNDS (-8)   /* a kernel's own bounds check fired (access skipped) */

/* PhysicsType, source/engine/game_datastruct.hpp:87-95 */
#define FSE_AIR 0
#define FSE_SOLID 1
#define FSE_SAND 2
#define FSE_SOUP 3
#define FSE_GAS 4
#define FSE_PASSABLE 5
#define FSE_OBJECT 5

/* reaction / interaction kinds, source/engine/game_datastruct.hpp:97-103 */
#define FSE_INTERACT_TRANSFORM_MATERIAL 1
#define FSE_INTERACT_SPAWN_MATERIAL 2
#define FSE_REACT_TEMPERATURE_BELOW 4
#define FSE_REACT_TEMPERATURE_ABOVE 5

/* fluid amounts are Q16.16 fixed point: 1.0 == FSE_FLUID_ONE */
#define FSE_FLUID_ONE 65536

/* synthetic world generators */
#define FSE_GEN_EMPTY 0  /* all GENERIC_AIR */
#define FSE_GEN_MIX 1    /* bottom 8 rows STONE; top 60%: 30% sand, 20% water, 10% gas, 15% stone, 25% air */
#define FSE_GEN_ZIPF8 2  /* 8 materials, Zipf(s=1) frequencies, whole world */

/* Per-world configuration. Zero-initialise and set what you need. */
typedef struct fse_config {
    int32_t chunk_size;   /* colour-partition chunk edge (CHUNK_W/H, const.h:19-20); 0 -> 128 */
    int32_t cell_iter;    /* iterations per tick (global_def.cell_iter); 0 -> 3 */
    uint32_t seed;        /* counter-RNG seed (replaces srand/rand) */
    int32_t particle_capacity; /* max live particles; 0 -> max(65536, cells / 4) */
    int32_t spawn_capacity;    /* max particles spawned per tick; 0 -> particle_capacity */
    void *stream;         /* cudaStream_t to bind; NULL -> a library-owned stream */
    int32_t flags;        /* FSE_CFG_* */
} fse_config;

/* the world keeps the render state of fse_world_render_*: a per-cell dirty plane
 * and the tick's per-cell flow sums (13 more bytes per cell, 20 with textures) */
#define FSE_CFG_RENDER 1
/* the world keeps MaterialInstance::temperature for liquids too (2 more bytes per
 * cell, carried by every liquid move, flow, free fall and deposit, and by
 * particles): needed by the fse_world_temperature_* calls and by
 * fse_world_tick_temperature. Without it a world keeps only the temperatures its
 * scalars hold (every non-liquid cell): liquid temperatures change no other
 * result of a tick, the temperature calls return FSE_E_STATE and particles read
 * temperature 0. */
#define FSE_CFG_TEMPERATURE 2
/* FSE_CFG_TEMPERATURE, and fse_world_tick/step (and batches and servers) run
 * world::tickTemperature() after every tick whose index is 2 modulo GameTick (4),
 * as game::tick does (game.cpp:2157-2159, const.h:38); the test runs on the
 * device, so step graphs replay it correctly */
#define FSE_CFG_TEMPERATURE_STEP 4
/* the reference's own update order inside each chunk: the chunk's cells in turn,
 * bottom row first and left to right, sweep by sweep (world.cpp:1084-1087, 1589,
 * 1823), with the same rules and draws, run as a wavefront of one thread per chunk
 * row; the default partitioned order updates a chunk's cells in 30 lattice
 * sub-phases with a thread per cell. Results then equal the reference's
 * world::tick for every rule (liquid amounts in Q16.16 rather than f32); a tick
 * takes about 13 times longer. Worlds with it cannot join batches or servers. */
#define FSE_CFG_REFERENCE_ORDER 8
/* liquid amounts (MaterialInstance::fluidAmount) and pending diffs (fluidAmountDiff)
 * are kept as the reference's own f32, computed with its float arithmetic (every
 * operation separately rounded, no contraction), instead of Q16.16 fixed point: the
 * scalar plane of a SOUP cell, the diff plane, particle scalars of SOUP tiles and the
 * tile structs then hold f32 bit patterns. Deposits of liquid particles into liquid
 * add their amounts cell by cell in particle-index order. With
 * FSE_CFG_REFERENCE_ORDER the tick then equals the reference's world::tick bit for
 * bit, liquids included. The ledger and census keep no fluid rows (f32 sums are not
 * conserved); cell counts are kept as ever. Worlds with it cannot join servers, and
 * a batch takes worlds of one kind only. */
#define FSE_CFG_F32_FLUID 16

/* One free particle (CellData, source/engine/game_utils/cells.h:15-36). 60 bytes. */
typedef struct fse_particle {
    float x, y, vx, vy, ax, ay;
    float target_x, target_y, target_force;
    int32_t lifetime, fade_time;
    uint32_t colour;
    int32_t scalar; /* fluid amount (Q16.16, or f32 bits in FSE_CFG_F32_FLUID worlds) for SOUP tiles,
                       temperature otherwise */
    uint16_t id;    /* material of the carried tile */
    uint8_t flags;  /* tile flags: bit7 moved, bits0-5 settle count */
    uint8_t bits;   /* bit0 phase, bit1 temporary, bits2-3 inObjectState */
    int16_t temperature; /* temperature of a SOUP tile (its scalar holds the amount) in worlds created
                          with FSE_CFG_TEMPERATURE; 0 otherwise */
    uint16_t reserved;
} fse_particle;

/* A rigid body stamped into the grid as OBJECT tiles. 48 bytes. */
typedef struct fse_body {
    float x, y, sin_a, cos_a; /* body position and sin/cos of its angle */
    int32_t w, h;             /* tile box (matWidth x matHeight) */
    uint16_t id;              /* tile material (e.g. GENERIC_OBJECT) */
    uint16_t pad;
    uint32_t colour;
    int32_t n_sand, n_soup;   /* out: SAND / SOUP cells displaced by the last stamp (damping) */
    int32_t n_placed, n_recovered; /* out: tiles placed by stamp / taken back by readback */
} fse_body;

typedef struct fse_world fse_world;
typedef struct fse_batch fse_batch;
typedef struct fse_server fse_server;

/* ---------------------------------------------------------------- version */
const char *fse_version(void);
const char *fse_status_string(int status);

/* -------------------------------------------------------------- materials */
/* Reset the table to the built-in materials in InitMaterials order (ids 0-27,
 * then TEST_SAND, TEST_TEXTURED_SAND, TEST_LIQUID as 28-30). */
int fse_materials_begin(void);
/* RegisterMaterial(s_id, name, index_name, physicsType, slipperyness, alpha,
 * density, iterations, emit, emitColor, color); *out_id = the new material id. */
int fse_material_register(int s_id, const char *name, const char *index_name, int physics_type, int slipperyness,
                          int alpha, float density, int iterations, int emit, uint32_t emit_colour, uint32_t colour,
                          int *out_id);
int fse_material_set_reaction(int mat, int kind, int temperature, int result_mat);
int fse_material_set_interaction(int mat, int other, int kind, int data1_mat, int data2_radius, int ofs_x, int ofs_y);
/* tile factory of a material: colour = base + ((lo + rand % mod) << shift) when mod > 0 */
int fse_material_set_factory(int mat, uint32_t base, int shift, int lo, int mod, int32_t scalar);
/* temperature of the tiles the factory makes of a SOUP material (whose scalar is
 * the amount): WATER -1023, LAVA 1024 (game_datastruct.cpp:427-437); the scalar
 * is the temperature of every other material */
int fse_material_set_factory_temperature(int mat, int32_t temperature);
/* Material::addTemp, conductionSelf, conductionOther (game_datastruct.hpp:142-144,
 * set in InitMaterials, game_datastruct.cpp:124-141) */
int fse_material_set_conduction(int mat, uint32_t add_temp, float conduction_self, float conduction_other);
/* out: addTemp, conductionSelf bits, conductionOther bits, factory temperature */
int fse_material_get_conduction(int mat, uint32_t out[4]);
/* Execute the materials_register(...) calls of a Lua script text (the subset of
 * Lua used by data/scripts: literal arguments and integer/float expressions).
 * *out_count = number of materials registered. */
int fse_materials_load_lua(const char *script, int *out_count);
/* Freeze the table and upload it to the device (PushMaterials). */
int fse_materials_push(void);
int fse_material_count(void);
int fse_material_find(const char *index_name);
/* 16 ints: type, density bits, iterations, slip, max_stab, alpha, colour, emit,
 * emit_colour, f_base, f_shift, f_lo, f_mod, f_scalar, n_react, interact */
int fse_material_get(int id, int32_t out[16]);

/* ----------------------------------------------------------------- worlds */
int fse_world_create(int width, int height, const fse_config *cfg, fse_world **out);
int fse_world_destroy(fse_world *world);
int fse_world_info(const fse_world *world, int32_t out[8]); /* w, h, chunk, cell_iter, seed, tick, particles, err */
/* host SoA <-> device SoA (cells row-major, width * height each); NULL planes are skipped */
int fse_world_upload(fse_world *world, const uint16_t *id, const uint32_t *colour, const int32_t *scalar,
                     const uint8_t *flags, const int32_t *diff);
int fse_world_download(fse_world *world, uint16_t *id, uint32_t *colour, int32_t *scalar, uint8_t *flags,
                       int32_t *diff);
int fse_world_generate(fse_world *world, int kind, uint32_t seed);
int fse_world_set_tick(fse_world *world, uint32_t tick);
/* world::tickZone (world.hpp:138; the game sets it every frame to the world less a
 * chunk on each side, game.cpp:1629-1636): the rectangle x, y, width, height inside
 * the world that the tick works on. Chunks start at its corner every chunk_size
 * cells while the start lies in it, and reach chunk_size cells whatever the zone's
 * end (world.cpp:1078-1087); particles whose cell is outside it neither move nor
 * age (their velocity is still steered, world.cpp:2039-2061); the temperature step
 * changes only its cells (world.cpp:1952-2001). The whole world by default. Batches
 * and servers use the zone their worlds had when they were made. */
int fse_world_set_tick_zone(fse_world *world, int x, int y, int width, int height);
/* The launch shape of the world's colour pass (results never depend on it; a new
 * world, batch or server uses 4, the fastest measured on the bench workloads):
 * 0 one 1024-thread CTA per chunk, 1 one persistent CTA per SM walking the chunks,
 * 2 each chunk split over a pair of 512-thread CTAs (a thread-block cluster; the
 * partitioned order only), 3 persistent pairs, 4 the fused tick: every pass of a
 * tick in one launch of one CTA per SM, each chunk-pass started as soon as the
 * chunk-passes of its 3 x 3 chunk neighbourhood it depends on are done (the
 * partitioned order only; worlds in the reference's order run shape 0). */
int fse_world_set_launch(fse_world *world, int colour_shape);
int fse_world_get_tile(fse_world *world, int x, int y, uint16_t *id, uint32_t *colour, int32_t *scalar,
                       uint8_t *flags);
int fse_world_set_tile(fse_world *world, int x, int y, uint16_t id, uint32_t colour, int32_t scalar, uint8_t flags);

/* Array-of-structs grids such as the reference's real_tiles: where the fields of
 * the caller's tile struct lie (byte offsets, -1 = absent; 4-byte fields 4-aligned,
 * the temperature 2-aligned, the pointer slot 8-aligned, stride a multiple of 8). */
typedef struct fse_tile_layout {
    int32_t stride;            /* bytes per tile */
    int32_t id;                /* u32 material index (MaterialInstance::id == mat->id) */
    int32_t mat;               /* pointer slot written on download from mat_table[id] */
    int32_t colour;            /* u32 */
    int32_t temperature;       /* i16 */
    int32_t moved;             /* bool / u8 */
    int32_t fluid_amount;      /* f32 */
    int32_t fluid_amount_diff; /* f32 */
    int32_t settle_count;      /* u8 */
} fse_tile_layout;
/* MaterialInstance (game_datastruct.hpp:205-222) on LP64 targets, 40 bytes */
#define FSE_TILE_LAYOUT_MATERIAL_INSTANCE {40, 0, 8, 16, 20, 22, 24, 28, 32}
/* Load the whole grid from / store it into such an array (width * height tiles,
 * row-major): liquid amounts and diffs are rounded to the nearest 1/65536 (copied
 * bit for bit in worlds created with FSE_CFG_F32_FLUID), the
 * settle count saturates at 63, a liquid's temperature is kept only by worlds with
 * FSE_CFG_TEMPERATURE. Download writes id, colour, temperature, moved and settle
 * count of every tile, the amounts of liquid tiles only, and (with a mat_table of
 * n_mat pointers, and layout->mat >= 0) the Material pointer; other bytes are kept.
 * The conversion runs on the device: the array travels once per upload, twice per
 * download (read, then written back). */
int fse_world_upload_tiles(fse_world *world, const void *tiles, const fse_tile_layout *layout);
int fse_world_download_tiles(fse_world *world, void *tiles, const fse_tile_layout *layout, const uint64_t *mat_table,
                             int n_mat);

/* Temperatures of all cells (int16, MaterialInstance::temperature) of a world
 * created with FSE_CFG_TEMPERATURE (else FSE_E_STATE): SOUP cells keep theirs
 * beside the amount, every other cell in its scalar. Upload and set_tile leave
 * SOUP temperatures as they were; the generators give new SOUP tiles their
 * factory temperature. */
int fse_world_temperature_read(fse_world *world, int16_t *out);
int fse_world_temperature_write(fse_world *world, const int16_t *temps);
/* world::tickTemperature() (world.cpp:1950-2004): one Jacobi step of the 3x3
 * conduction stencil over every cell; a neighbour outside the world counts as
 * temperature 0. Enqueued on the world's stream. */
int fse_world_tick_temperature(fse_world *world);

/* ------------------------------------------------------- chunk .pack codec */
/* Chunk::ChunkWrite for every 128 x 128 chunk, row-major (chunk k covers cells
 * x = (k % ceil(w/128)) * 128 + [0, 128), y = (k / ceil(w/128)) * 128 + [0, 128);
 * cells outside the world are GENERIC_AIR records): each .pack is the i8
 * generation phase, src_size, the tile block's size, src_size2, the background
 * block's size (ints) and two LZ4 blocks (chunk.cpp:219-330). The records are
 * MaterialInstanceData {u32 index, u32 colour, i16 temperature} (chunk.hpp:26-30);
 * the second layer and the background, which this world does not have, are
 * zeros. Liquid temperatures are written as 0 unless the world keeps them
 * (FSE_CFG_TEMPERATURE). out: host buffer of cap bytes; offsets[k] = start of
 * chunk k's .pack in out, offsets[n] = total; *out_n_chunks = n. */
int fse_world_pack_bound(int width, int height, int64_t *out_bytes, int *out_chunks);
int fse_world_pack(fse_world *world, int generation_phase, uint8_t *out, int64_t cap, int64_t *offsets,
                   int *out_n_chunks);
/* Chunk::ChunkRead for every chunk: in + offsets as fse_world_pack writes them (any
 * LZ4 encoder's blocks are read). Tiles take the records' material, colour and
 * temperature; a SOUP tile's amount is the MaterialInstance default 2.0, flags
 * and pending diffs are cleared. out_phases[k] (optional) = chunk k's generation
 * phase. A malformed chunk (header, sizes, LZ4 block or a material index out of
 * range) ends the load: FSE_E_INVAL with *out_bad_chunk = its index, the chunks
 * before it written, none after. */
int fse_world_unpack(fse_world *world, const uint8_t *in, const int64_t *offsets, int n_chunks, int8_t *out_phases,
                     int *out_bad_chunk);
/* Pack, unpack and the tile-struct calls keep their device scratch (about 1 MB per
 * chunk for pack and unpack) between calls; this frees it. */
int fse_world_trim(fse_world *world);

/* Exact checkpoint of a world (the .pack files keep only material, colour and
 * temperature): every plane, the particle list, the tick counter, seed and ledger,
 * as LZ4 blocks written by the .pack encoder. A world restored from it (same
 * size, chunk size and cell_iter; particle capacity at least the checkpoint's
 * particles) continues bit for bit as the original would. Liquid temperatures are
 * saved when the world keeps them; restoring them needs FSE_CFG_TEMPERATURE
 * (FSE_E_STATE otherwise). Malformed input (sizes, block lengths, LZ4 tokens)
 * returns FSE_E_INVAL; like the .pack files the format has no checksum. */
int fse_world_checkpoint_bound(fse_world *world, int64_t *out_bytes);
int fse_world_checkpoint(fse_world *world, uint8_t *out, int64_t cap, int64_t *out_size);
int fse_world_restore(fse_world *world, const uint8_t *in, int64_t size);

/* world::tick(), n times (no particle step in between) */
int fse_world_tick(fse_world *world, int n_ticks);
/* world::tickCells() */
int fse_particles_tick(fse_world *world);
/* the game-loop order: n x (world::tick(); world::tickCells()) */
int fse_world_step(fse_world *world, int n_ticks);
/* enqueue n_ticks steps (with_particles != 0) or ticks on the world's stream and
 * return without waiting; fse_world_sync() waits and reports kernel errors */
int fse_world_enqueue(fse_world *world, int n_ticks, int with_particles);
/* record n_ticks steps into a CUDA graph once and replay it: same results as
 * fse_world_step, fewer launches */
int fse_world_step_graph(fse_world *world, int n_ticks);
/* wait for the world's stream; returns the first error the kernels recorded */
int fse_world_sync(fse_world *world);
int fse_world_set_stream(fse_world *world, void *stream);
void *fse_world_stream(fse_world *world);

/* ------------------------------------------------------------- particles */
int fse_particles_add(fse_world *world, const fse_particle *parts, int n);
int fse_particles_count(fse_world *world, int *out_n);
int fse_particles_read(fse_world *world, fse_particle *out, int cap, int *out_n);

/* ---------------------------------------------------------------- objects */
int fse_object_stamp(fse_world *world, fse_body *bodies, int n);
int fse_object_readback(fse_world *world, fse_body *bodies, int n, int64_t *out_removed);
/* 1 bit per cell (row-major, LSB first): physics type == OBJECT; host buffer of
 * ceil(w*h/8) bytes */
int fse_object_mask_export(fse_world *world, uint8_t *host_bits);
/* compact list of OBJECT cell indices (y*w+x, ascending); *out_n = count (may exceed cap) */
int fse_object_list_export(fse_world *world, uint32_t *host_idx, int64_t cap, int64_t *out_n);

/* ------------------------------------------------------------ diagnostics */
/* Time every colour-pass launch of this world with CUDA events on its stream.
 * enable = 1 starts (and zeroes) the timer, 0 stops it; both first report the
 * accumulated kernel milliseconds and launch count since the last start. */
int fse_world_pass_timing(fse_world *world, int enable, double *out_ms, int64_t *out_launches);
/* iterations the last particle update of this world needed to reach the list-order
 * result (for a batch: recorded on its first world); diagnostics */
int fse_world_particle_iterations(fse_world *world, int *out);
/* kernels this library has launched so far (all worlds, batches and servers) */
int64_t fse_launch_counter(void);

/* ----------------------------------------------------------------- ledger */
/* 6 rows x fse_material_count(): created_n, destroyed_n, exited_n, created_f,
 * destroyed_f, exited_f (f in Q16.16) accumulated since creation or reset */
int fse_world_ledger(fse_world *world, int64_t *out);
int fse_world_ledger_reset(fse_world *world);
/* 4 rows: grid_count, grid_fluid (amount + pending diff), part_count, part_fluid */
int fse_world_census(fse_world *world, int64_t *out);

/* -------------------------------------------------------------- rendering */
/* Headless device textures of the game's per-tick texture updates, 4 bytes per
 * cell (r, g, b, a), row-major. Worlds created with FSE_CFG_RENDER only
 * (FSE_E_STATE otherwise). Every cell starts dirty; the tick, deposits, bodies
 * and uploads mark the cells they write. */
#define FSE_TEX_PIXELS 0   /* pixels_ar: colour and material alpha; AIR transparent */
#define FSE_TEX_EMISSION 1 /* pixelsEmission_ar: the material's emitColor */
#define FSE_TEX_FIRE 2     /* pixelsFire_ar: FIRE cells, kept until the cell turns AIR */
#define FSE_TEX_FLOW 3     /* pixelsFlow_ar: smoothed liquid flow */
#define FSE_TEX_CELLS 4    /* pixelsCells_ar: the free-particle layer */
/* the dirty-cell pass (game.cpp:1994-2067): repaints the dirty cells and clears
 * their marks; moving (fse_material_count() entries, may be NULL) receives the
 * dirty cells per material (movingTiles) */
int fse_world_render_dirty(fse_world *world, int64_t *moving);
/* the particle layer (world::renderCells, world.cpp:2006-2028, after the clear of
 * game.cpp:1881): later particles in list order cover earlier ones */
int fse_world_render_cells(fse_world *world);
/* copy a texture (W * H * 4 bytes) to host memory */
int fse_world_render_read(fse_world *world, int which, uint8_t *out);
/* the texture's device pointer (valid until the world is destroyed), NULL on error */
void *fse_world_render_texture(fse_world *world, int which);

/* ---------------------------------------------------------- solid islands */
typedef struct fse_island {
    int32_t root;  /* the region's smallest cell index (y * W + x) */
    int32_t cells;
    int32_t min_x, min_y, max_x, max_y;
} fse_island;
/* world::physicsCheck(x, y) (world.cpp:3330-3445): if (x, y) is SOLID and its
 * 4-connected SOLID region has at most 1000 cells, the region is cut out of the grid
 * (its cells become GENERIC_AIR, counted as destroyed in the ledger). *out_cells =
 * cells cut (0: nothing), out_bbox = min x, min y, max x, max y; for more than 10
 * cells and a non-NULL `pixels` of at least bbox-width * bbox-height entries, the
 * region's colours as that image, 0 elsewhere (the surface the host makes the rigid
 * body from). */
int fse_world_physics_check(fse_world *world, int x, int y, int *out_cells, int32_t out_bbox[4], uint32_t *pixels,
                            int64_t pixels_cap);
/* every 4-connected SOLID region at once (connected-component labelling on the
 * device): the regions of at most max_cells cells, by increasing root; the first
 * `cap` are written to `out`, *out_n = how many there are; with `remove` they are
 * all cut out of the grid as physicsCheck does. */
int fse_world_islands(fse_world *world, int max_cells, int remove, fse_island *out, int cap, int *out_n);

/* ------------------------------------------------- allocation-free tick */
/* One world::tick() (no particle step) on cell planes the caller owns in device
 * memory, for hosts that cannot let a library allocate device memory: engines
 * that serve every byte from their own arena under their own budget, and
 * real-time loops that forbid cudaMalloc/cudaFree after start-up because those
 * calls can stall the device and can fail under memory pressure mid-frame.
 * No counterpart in the reference (its tick allocates per-task particle lists).
 *
 * id/colour/scalar/flags/diff: device planes of width*height cells, updated in
 * place. out_spawned: device array of spawn_cap particles that receives the
 * particles this tick spawns, in the order fse_world_tick would append them;
 * *out_n_spawned = their number (FSE_E_CAPACITY when more than spawn_cap).
 * tick: the world's tick count (keys the counter RNG; the caller advances it).
 * Results equal fse_world_tick's bit for bit, except that no temperature plane is
 * passed: liquid temperatures are not carried, and SOUP particles are spawned
 * with temperature 0.
 *
 * Scratch: one fixed device array of about 4 MB inside the library, held by every
 * GPU that loads it until the process exits. Limits: at most 4096 chunks per
 * colour (16384 x 16384 cells at chunk 128, 8192 x 8192 at chunk 64), cell_iter <= 8, at most 65536
 * particles spawned per tick; larger requests return FSE_E_INVAL. The first call
 * on a device looks the array up (cudaGetSymbolAddress) and should be made before
 * any stream capture. Every call shares the array: calls that overlap on the GPU
 * (other streams, other host threads) race and must not be made. The call calls
 * no cudaMalloc/cudaFree and returns after its work is done. */
int fse_tick_noalloc(uint16_t *id, uint32_t *colour, int32_t *scalar, uint8_t *flags, int32_t *diff, int width,
                     int height, int chunk_size, int cell_iter, uint32_t seed, uint32_t tick, fse_particle *out_spawned,
                     int spawn_cap, int *out_n_spawned, void *stream);

/* --------------------------------------------------------------- batches */
/* Many worlds ticked by one launch per colour pass over the chunks of all worlds. */
int fse_batch_create(fse_world **worlds, int n, fse_batch **out);
int fse_batch_destroy(fse_batch *batch);
int fse_batch_step(fse_batch *batch, int n_ticks);
/* enqueue n_ticks steps on the batch's stream and return without waiting (errors
 * of those steps come from the next fse_batch_sync); batches of disjoint worlds
 * step concurrently, each on its own stream */
int fse_batch_enqueue(fse_batch *batch, int n_ticks);
/* capture graph_ticks steps into one CUDA graph (default 32) and replay */
int fse_batch_step_graph(fse_batch *batch, int n_ticks, int graph_ticks);
/* capture (without running) the graphs a later fse_batch_step_graph(n_ticks,
 * graph_ticks) replays, so that the capture cost stays out of a timed region */
int fse_batch_prepare_graphs(fse_batch *batch, int n_ticks, int graph_ticks);
/* choose the launch shape by timing candidates on the batch itself, then restore
 * every world; results never change. out_choice: colour_ctas_per_sm,
 * particle_blocks, microseconds of two timed steps, candidate index */
int fse_batch_autotune(fse_batch *batch, int32_t out_choice[4]);
/* colour_ctas_per_sm: the colour pass's launch shape as in fse_world_set_launch
 * (0 one CTA per chunk, 1 one persistent CTA per SM, 2 a CTA pair per chunk,
 * 3 persistent pairs, 4 the fused tick); particle_blocks: blocks per world of the
 * particle kernels (0 = enough for the largest particle list) */
int fse_batch_set_launch(fse_batch *batch, int colour_ctas_per_sm, int particle_blocks);
int fse_batch_sync(fse_batch *batch);
/* Time the batch's steps with CUDA events on its stream: every colour-pass launch
 * and every tick, for plain and graph steps (graphs captured while timing is on
 * carry the events as nodes, and each replay is read back before the next one is
 * launched). enable = 1 starts (and zeroes) the timers, 0 stops them; both first
 * report what was accumulated since the last start: colour-pass milliseconds and
 * launches, and each tick's duration in ms into tick_ms[0 .. min(cap, n) - 1] with
 * *out_ticks = n. */
int fse_batch_timing(fse_batch *batch, int enable, double *out_pass_ms, int64_t *out_pass_launches, float *tick_ms,
                     int cap, int *out_ticks);
/* the CUDA stream (cudaStream_t) the batch enqueues its work on */
void *fse_batch_stream(fse_batch *batch);
/* Plane I/O of member `index` enqueued on the batch's stream, in order with its
 * steps, without waiting (host buffers should be pinned for the copies to run
 * asynchronously; the member's own stream must be idle). Upload: the planes given
 * (NULL keeps a plane), as fse_world_upload; an out-of-range id becomes GENERIC_AIR
 * and the next fse_batch_sync returns FSE_E_INVAL. Download: as fse_world_download;
 * the host buffers hold the planes after the next fse_batch_sync. */
int fse_batch_upload(fse_batch *batch, int index, const uint16_t *id, const uint32_t *colour, const int32_t *scalar,
                     const uint8_t *flags, const int32_t *diff);
int fse_batch_download(fse_batch *batch, int index, uint16_t *id, uint32_t *colour, int32_t *scalar, uint8_t *flags,
                       int32_t *diff);
/* Every member's planes in one host buffer, moved by one large copy each way (host
 * buffer pinned for the copy to run asynchronously): member k's planes id, colour,
 * scalar, flags, diff start at offsets[5k .. 5k + 4] (bytes, multiples of 16) of a
 * buffer of *out_bytes bytes; offsets may be NULL. */
int fse_batch_io_layout(fse_batch *batch, int64_t *offsets, int64_t *out_bytes);
/* enqueue on the batch's stream the copy of the whole buffer and its scatter into
 * the members' planes (ids checked and flags masked as fse_batch_upload does) */
int fse_batch_upload_all(fse_batch *batch, const void *host, int64_t bytes);
/* enqueue the gather of every member's planes and one copy into the buffer; the
 * buffer holds them after the next fse_batch_sync */
int fse_batch_download_all(fse_batch *batch, void *host, int64_t bytes);

/* ---------------------------------------------------------------- serving */
/* Continuous batching of world-tick requests (no analogue in the reference, which
 * ticks one world per frame). Worlds are registered with the server and keep their
 * state in HBM; the budget caps the device bytes of the resident worlds. A world
 * that does not fit is parked in host memory as an exact checkpoint and restored
 * when a request for it is admitted; restored worlds continue bit for bit. At most
 * max_active requests (up to 4095) run at once. */
int fse_server_create(int64_t hbm_budget_bytes, int max_active, fse_server **out);
int fse_server_destroy(fse_server *srv);
/* register a world, generated by fse_world_generate(gen_kind, gen_seed); *out_slot
 * = its slot. It is resident when it fits the budget after parking idle worlds
 * without queued requests (least recently ticked first). FSE_E_BUDGET when it
 * could never be resident (its footprint exceeds the budget) or no idle world can
 * make room; FSE_E_INVAL for FSE_CFG_REFERENCE_ORDER, FSE_CFG_F32_FLUID or a chunk
 * size other than the server's first world's. */
int fse_server_add_world(fse_server *srv, int width, int height, const fse_config *cfg, int gen_kind,
                         uint32_t gen_seed, int *out_slot);
/* unregister a world with no queued or active request (FSE_E_STATE otherwise) */
int fse_server_remove_world(fse_server *srv, int slot);
/* device bytes of the resident worlds */
int64_t fse_server_bytes_in_use(const fse_server *srv);
/* the world of a slot, restored into HBM first when parked (NULL when no idle world
 * can make room). The pointer stays valid until a later server call parks the world:
 * only worlds without queued or active requests are parked. */
fse_world *fse_server_world(fse_server *srv, int slot);
/* queue a request of n_ticks steps (world::tick + world::tickCells each) for a
 * world; arrival_us is the caller's clock */
int fse_server_submit(fse_server *srv, int slot, int n_ticks, double arrival_us, int64_t *out_request);
/* One scheduling step: retire finished steps; admit queued requests in arrival
 * order (one request per world at a time; a parked world is restored when its
 * footprint fits, parking idle worlds first); enqueue one batched tick of every
 * active world on the server's stream and return without waiting, unless more
 * than `depth` steps are then in flight (it waits for the oldest). With no active
 * request it waits for every step in flight. *out_active = requests this step ticks. */
int fse_server_step(fse_server *srv, int *out_active);
/* microseconds since the server was created: the clock of arrivals and completions */
double fse_server_now_us(const fse_server *srv);
/* completed requests: ids and completion times, the device timestamp of the end of
 * the step that ran their last tick, on the fse_server_now_us clock */
int fse_server_poll(fse_server *srv, double now_us, int64_t *ids, double *done_us, int cap, int *out_n);
/* steps in flight before fse_server_step waits (1..64, default 3) */
int fse_server_set_depth(fse_server *srv, int depth);
/* wait for every step in flight */
int fse_server_drain(fse_server *srv);
/* out[0..n-1] of: steps enqueued, worlds restored, worlds parked, resident worlds,
 * parked worlds, most steps in flight, queued requests, active requests */
int fse_server_stats(fse_server *srv, int64_t *out, int n);
/* device milliseconds of each retired step (start to end event), oldest first;
 * the values returned are consumed */
int fse_server_tick_times(fse_server *srv, float *ms, int cap, int *out_n);

#ifdef __cplusplus
}
#endif
#endif /* FSE_H */
