/*
 * fse_oracle.c -- CPU oracle for the falling-sand world tick (TEST INFRASTRUCTURE).
 *
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load this
 * library; the product library never links or calls it.
 *
 * Each rule below cites the reference line it restates (paths relative to the
 * reference project root). Deviations from the reference that the GPU design needs
 * are stated where they occur; they are the same in both update orders:
 *   - fluid amounts are Q16.16 fixed point (int32) instead of f32, so that flows,
 *     commits and the mass ledger are exact and order-independent;
 *   - rand() is replaced by a counter RNG keyed on (seed, tick, iter, sweep, x, y, k);
 *   - out-of-world reads return the GENERIC_SOLID instance and out-of-world writes
 *     are dropped, for every access (the reference does this only in getTile/setTile
 *     and relies on a one-chunk margin elsewhere);
 *   - the settle counter is 6 bits, saturating at 63 (u8, wrapping, in the reference);
 *   - soup free-fall splits the amount exactly (remainder to the first particles).
 */
#include "fse_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ------------------------------------------------------------------ constants */
/* PhysicsType, source/engine/game_datastruct.hpp:87-95 */
enum { T_AIR = 0, T_SOLID = 1, T_SAND = 2, T_SOUP = 3, T_GAS = 4, T_OBJECT = 5 };
/* interaction/reaction kinds, game_datastruct.hpp:97-103 */
enum { INTER_TRANSFORM = 1, INTER_SPAWN = 2, REACT_BELOW = 4, REACT_ABOVE = 5 };

#define MAXMAT 256
#define MOVED 0x80u
#define SETTLE_MASK 0x3Fu

/* FLUID_* constants, source/engine/core/const.h:23-34, in Q16.16 */
#define Q_ONE 65536
#define Q_MAXV 32768     /* FLUID_MaxValue 0.5 */
#define Q_MINV 33        /* amount < FLUID_MinValue (0.0005 = 32.77) <=> q < 33 */
#define Q_MAXCOMP 6554   /* FLUID_MaxCompression 0.1 */
#define Q_MAXFLOW 524288 /* FLUID_MaxFlow 8.0 */
#define Q_FREEFALL 327   /* amount > 0.005 (327.68) <=> q > 327, world.cpp:1283 */
#define Q_DEFAULT 131072 /* MaterialInstance::fluidAmount default 2.0f, game_datastruct.hpp:221 */

/* RNG phases */
#define PH_GEN 0x47454E00u
#define PH_STAMP 0x5354414Du

/* ---------------------------------------------------------------------- RNG */
/* lowbias32 integer finaliser (C. Wellons, public domain) */
static inline uint32_t hash32(uint32_t h) {
    h ^= h >> 16;
    h *= 0x7feb352dU;
    h ^= h >> 15;
    h *= 0x846ca68bU;
    h ^= h >> 16;
    return h;
}
static inline uint32_t pass_key(uint32_t seed, uint32_t tick, uint32_t phase) {
    uint32_t h = hash32(seed ^ 0x5bd1e995U);
    h = hash32(h ^ tick);
    return hash32(h ^ (phase * 0x9E3779B9U + 0x7F4A7C15U));
}
static inline uint32_t cell_key(uint32_t pk, uint32_t x, uint32_t y) {
    return hash32(hash32(pk ^ x) ^ (y * 0x85EBCA6BU));
}
static inline uint32_t draw_k(uint32_t ck, uint32_t k) { return hash32(ck + k * 0x9E3779B9U + 0x632BE5ABU); }

/* ---------------------------------------------------------------- materials */
typedef struct {
    int kind, data1, data2, ofsx, ofsy;
} inter_t;

typedef struct {
    int type;
    float density;
    int iterations, slip, max_stab, alpha;
    uint32_t colour;
    int emit;
    uint32_t emit_colour;
    /* tile factory: colour = base + ((lo + draw % mod) << shift) if mod > 0 */
    uint32_t f_base;
    int f_shift, f_lo, f_mod;
    int32_t f_scalar;
    /* temperature of a new SOUP tile (the scalar holds its amount); the
     * MaterialInstance temperature of TilesCreate, game_datastruct.cpp:427-437 */
    int32_t f_temp;
    /* Material::addTemp, conductionSelf, conductionOther (game_datastruct.hpp:142-144) */
    uint32_t add_temp;
    float cond_self, cond_other;
    int n_react;
    inter_t react[4];
    int interact;
    char index_name[48];
} mat_t;

static mat_t M[MAXMAT];
static int NMAT = 0;
static int HAS_INTER = 0;
/* interactions: (mat, other) -> up to 4 entries */
typedef struct {
    int mat, other, n;
    inter_t e[4];
} inter_list_t;
static inter_list_t INTER[512];
static int NINTER = 0;
static int ID_AIR = 0, ID_SOLID = 1, ID_FIRE = -1, ID_WATER = -1, ID_LAVA = -1, ID_STEAM = -1, ID_OBSIDIAN = -1;

static int max_stability(int slip) {
    /* world.cpp:1623 `int maxStability = 8 / sqrt(slipperyness) + 1;` (double math) */
    if (slip <= 0) return 1 << 20;
    return (int)(8.0 / sqrt((double)slip) + 1.0);
}

static int reg(const char *index_name, int type, int slip, int alpha, float density, int iterations, int emit,
               uint32_t emit_colour, uint32_t colour) {
    if (NMAT >= MAXMAT) return -1;
    mat_t *m = &M[NMAT];
    memset(m, 0, sizeof(*m));
    m->type = type;
    m->density = density;
    m->iterations = iterations;
    m->slip = slip;
    m->max_stab = max_stability(slip);
    m->alpha = alpha;
    m->colour = colour;
    m->emit = emit;
    m->emit_colour = emit_colour;
    m->f_base = colour;
    m->f_scalar = (type == T_SOUP) ? Q_DEFAULT : 0;
    m->cond_self = 1.0f;
    m->cond_other = 1.0f;
    strncpy(m->index_name, index_name, sizeof(m->index_name) - 1);
    return NMAT++;
}

int om_material_find(const char *index_name) {
    for (int i = 0; i < NMAT; i++)
        if (strcmp(M[i].index_name, index_name) == 0) return i;
    return -1;
}

static void refresh_ids(void) {
    ID_AIR = om_material_find("GENERIC_AIR");
    ID_SOLID = om_material_find("GENERIC_SOLID");
    ID_FIRE = om_material_find("FIRE");
    ID_WATER = om_material_find("WATER");
    ID_LAVA = om_material_find("LAVA");
    ID_STEAM = om_material_find("STEAM");
    ID_OBSIDIAN = om_material_find("OBSIDIAN");
    if (ID_AIR < 0) ID_AIR = 0;
    if (ID_SOLID < 0) ID_SOLID = 1;
}

int om_material_set_factory(int mat, uint32_t base, int shift, int lo, int mod, int32_t scalar) {
    if (mat < 0 || mat >= NMAT) return -1;
    M[mat].f_base = base;
    M[mat].f_shift = shift;
    M[mat].f_lo = lo;
    M[mat].f_mod = mod;
    M[mat].f_scalar = scalar;
    return 0;
}

int om_material_set_conduction(int mat, uint32_t add_temp, float cond_self, float cond_other) {
    if (mat < 0 || mat >= NMAT) return -1;
    M[mat].add_temp = add_temp;
    M[mat].cond_self = cond_self;
    M[mat].cond_other = cond_other;
    return 0;
}

/* addTemp, conductionSelf and conductionOther (as bits) of a material */
void om_material_conduction(int mat, uint32_t out[3]) {
    if (mat < 0 || mat >= NMAT) return;
    out[0] = M[mat].add_temp;
    memcpy(&out[1], &M[mat].cond_self, 4);
    memcpy(&out[2], &M[mat].cond_other, 4);
}

int om_material_set_factory_temperature(int mat, int32_t temperature) {
    if (mat < 0 || mat >= NMAT) return -1;
    M[mat].f_temp = temperature;
    return 0;
}

/* InitMaterials, game_datastruct.cpp:69-111 (the constructor calls) and :117-280
 * (registration order, conduction, reactions, scriptable test materials). The ten
 * random `Mat_i` materials (:171-239) are drawn with rand() at start-up and are
 * never made interactive (:196,206); they are left out so that ids are
 * reproducible: TEST_SAND/TEST_TEXTURED_SAND/TEST_LIQUID get ids 28-30. Texture
 * colours (data/assets is absent from the reference tree) are replaced by the
 * constant colours below. */
void om_materials_reset_builtin(void) {
    NMAT = 0;
    NINTER = 0;
    HAS_INTER = 0;
    const uint32_t W = 0xffffffffu; /* Material default colour (game_datastruct.hpp:172-176) */
    reg("GENERIC_AIR", T_AIR, 0, 255, 0, 0, 16, 0, W);
    reg("GENERIC_SOLID", T_SOLID, 0, 255, 1, 0, 0, 0, W);
    reg("GENERIC_SAND", T_SAND, 20, 255, 10, 2, 0, 0, W);
    reg("GENERIC_LIQUID", T_SOUP, 0, 255, 1.5f, 3, 0, 0, W);
    reg("GENERIC_GAS", T_GAS, 0, 255, -1, 1, 0, 0, W);
    reg("GENERIC_PASSABLE", T_OBJECT, 0, 255, 0, 0, 0, 0, W);
    reg("GENERIC_OBJECT", T_OBJECT, 0, 255, 1000.0f, 0, 0, 0, W);
    reg("STONE", T_SOLID, 0, 255, 1, 0, 0, 0, W);
    reg("GRASS", T_SAND, 20, 255, 12, 1, 0, 0, W);
    reg("DIRT", T_SAND, 8, 255, 15, 1, 0, 0, W);
    reg("SMOOTH_STONE", T_SOLID, 0, 255, 1, 0, 0, 0, W);
    reg("COBBLE_STONE", T_SOLID, 0, 255, 1, 0, 0, 0, W);
    reg("SMOOTH_DIRT", T_SOLID, 0, 255, 1, 0, 0, 0, W);
    reg("COBBLE_DIRT", T_SOLID, 0, 255, 1, 0, 0, 0, W);
    reg("SOFT_DIRT", T_SOLID, 0, 255, 15, 2, 0, 0, W);
    reg("WATER", T_SOUP, 0, 0x80, 1.5f, 6, 40, 0x3000AFB5u, W);
    reg("LAVA", T_SOUP, 0, 0xC0, 2, 1, 40, 0xFFFF6900u, W);
    reg("CLOUD", T_SOLID, 0, 127, 1, 0, 0, 0, W);
    reg("GOLD_ORE", T_SAND, 20, 255, 20, 2, 8, 0x804000u, W);
    reg("GOLD_MOLTEN", T_SOUP, 0, 255, 20, 2, 8, 0x6FFF9B40u, W);
    reg("GOLD_SOLID", T_SOLID, 0, 255, 20, 2, 8, 0, W);
    reg("IRON_ORE", T_SAND, 20, 255, 20, 2, 8, 0x7F442Fu, W);
    reg("OBSIDIAN", T_SOLID, 0, 255, 1, 0, 0, 0, W);
    reg("STEAM", T_GAS, 0, 255, -1, 1, 0, 0, W);
    reg("SOFT_DIRT_SAND", T_SAND, 8, 255, 15, 2, 0, 0, W);
    reg("FIRE", T_OBJECT, 0, 255, 20, 1, 0, 0, W);
    reg("FLAT_COBBLE_STONE", T_SOLID, 0, 255, 1, 0, 0, 0, W);
    reg("FLAT_COBBLE_DIRT", T_SOLID, 0, 255, 1, 0, 0, 0, W);
    reg("TEST_SAND", T_SAND, 20, 255, 10, 2, 0, 0, W);
    reg("TEST_TEXTURED_SAND", T_SAND, 20, 255, 10, 2, 0, 0, W);
    reg("TEST_LIQUID", T_SOUP, 0, 255, 1.5f, 4, 0, 0, W);
    refresh_ids();

    /* tile factories, game_datastruct.cpp:320-574 */
    om_material_set_factory(om_material_find("TEST_SAND"), (220u << 16) | 100u, 8, 155, 30, 0); /* :320-325 */
    om_material_set_factory(om_material_find("TEST_TEXTURED_SAND"), 0xDC9B64u, 0, 0, 0, 0);     /* texture */
    om_material_set_factory(om_material_find("TEST_LIQUID"), 0x0000FFu, 0, 0, 0, Q_DEFAULT);     /* :337-342 */
    om_material_set_factory(om_material_find("STONE"), 0x808080u, 0, 0, 0, 0);                  /* texture */
    om_material_set_factory(om_material_find("GRASS"), (40u << 16) | 20u, 8, 120, 20, 0);        /* :358-363 */
    om_material_set_factory(om_material_find("DIRT"), (40u << 8) | 20u, 16, 60, 10, 0);          /* :365-370 */
    om_material_set_factory(om_material_find("SMOOTH_STONE"), 0x9A9A9Au, 0, 0, 0, 0);
    om_material_set_factory(om_material_find("COBBLE_STONE"), 0x707070u, 0, 0, 0, 0);
    om_material_set_factory(om_material_find("SMOOTH_DIRT"), 0x6B4A2Fu, 0, 0, 0, 0);
    om_material_set_factory(om_material_find("COBBLE_DIRT"), 0x5A3D25u, 0, 0, 0, 0);
    om_material_set_factory(om_material_find("SOFT_DIRT"), 0x7A5533u, 0, 0, 0, 0);
    om_material_set_factory(om_material_find("WATER"), 0x00B69Fu, 0, 0, 0, Q_DEFAULT); /* :427-431 temp -1023 */
    om_material_set_factory(om_material_find("LAVA"), 0xFF7C00u, 0, 0, 0, Q_DEFAULT);  /* :433-437 temp 1024 */
    om_material_set_factory(om_material_find("CLOUD"), 0xE6E6F0u, 0, 0, 0, 0);
    om_material_set_factory(om_material_find("GOLD_ORE"), 0xC8A032u, 0, 0, 0, 0);
    om_material_set_factory(om_material_find("GOLD_MOLTEN"), 0xFFB43Cu, 0, 0, 0, Q_DEFAULT);
    om_material_set_factory(om_material_find("GOLD_SOLID"), 0xE6C34Bu, 0, 0, 0, 0);
    om_material_set_factory(om_material_find("IRON_ORE"), 0x8C6E5Au, 0, 0, 0, 0);
    om_material_set_factory(om_material_find("OBSIDIAN"), 0x1E1428u, 0, 0, 0, 0);
    om_material_set_factory(om_material_find("STEAM"), 0x666666u, 0, 0, 0, 0);                  /* :483 */
    om_material_set_factory(om_material_find("FIRE"), (255u << 16) | 50u, 8, 100, 50, 0);       /* :485-492 */
    om_material_set_factory(om_material_find("FLAT_COBBLE_STONE"), 0x787878u, 0, 0, 0, 0);
    om_material_set_factory(om_material_find("FLAT_COBBLE_DIRT"), 0x624530u, 0, 0, 0, 0);
    om_material_set_factory(ID_AIR, 0x000000u, 0, 0, 0, 0);   /* Tiles_NOTHING, :311 */
    om_material_set_factory(ID_SOLID, 0xff0000u, 0, 0, 0, 0); /* Tiles_TEST_SOLID, :312 */
    om_material_set_factory_temperature(ID_WATER, -1023); /* :427-431 */
    om_material_set_factory_temperature(ID_LAVA, 1024);   /* :433-437 */

    /* conduction, game_datastruct.cpp:124-141 (double literals rounded to float) */
    om_material_set_conduction(ID_AIR, 0, (float)0.8, (float)0.8);
    om_material_set_conduction(ID_LAVA, 2, (float)0.5, (float)0.7);
    om_material_set_conduction(om_material_find("COBBLE_STONE"), 0, (float)0.01, (float)0.4);
    om_material_set_conduction(om_material_find("COBBLE_DIRT"), 0, 1.0f, 1.0f);
    om_material_set_conduction(om_material_find("GOLD_ORE"), 0, 1.0f, 1.0f);
    om_material_set_conduction(om_material_find("GOLD_MOLTEN"), 0, 1.0f, 1.0f);

    /* reactions, game_datastruct.cpp:246-260 */
    om_material_set_reaction(ID_LAVA, REACT_BELOW, 512, ID_OBSIDIAN);
    om_material_set_reaction(ID_WATER, REACT_ABOVE, 128, ID_STEAM);
    om_material_set_reaction(om_material_find("GOLD_ORE"), REACT_ABOVE, 512, om_material_find("GOLD_MOLTEN"));
    om_material_set_reaction(om_material_find("GOLD_MOLTEN"), REACT_BELOW, 128, om_material_find("GOLD_SOLID"));
}

/* RegisterMaterial, game_datastruct.cpp:282-289 */
int om_material_register(int s_id, const char *name, const char *index_name, int physics_type, int slipperyness,
                         int alpha, float density, int iterations, int emit, uint32_t emit_colour, uint32_t colour) {
    (void)s_id;
    (void)name;
    if (physics_type < 0 || physics_type > 5) return -1;
    int id = reg(index_name, physics_type, slipperyness, alpha, density, iterations, emit, emit_colour, colour);
    refresh_ids();
    return id;
}

int om_material_set_reaction(int mat, int kind, int temperature, int result) {
    if (mat < 0 || mat >= NMAT || result < 0 || result >= NMAT) return -1;
    if (kind != REACT_BELOW && kind != REACT_ABOVE) return -1;
    mat_t *m = &M[mat];
    if (m->n_react >= 4) return -1;
    m->react[m->n_react].kind = kind;
    /* MaterialInteraction::data1 is a mat_temperature (i16), game_datastruct.hpp:114 */
    m->react[m->n_react].data1 = (int16_t)temperature;
    m->react[m->n_react].data2 = result;
    m->n_react++;
    return 0;
}

int om_material_set_interaction(int mat, int other, int kind, int data1, int data2, int ofs_x, int ofs_y) {
    if (mat < 0 || mat >= NMAT || other < 0 || other >= NMAT || data1 < 0 || data1 >= NMAT) return -1;
    if (kind != INTER_TRANSFORM && kind != INTER_SPAWN) return -1;
    if (data2 < 0 || abs(ofs_x) + data2 > 5 || abs(ofs_y) + data2 > 5) return -1;
    int li = -1;
    for (int i = 0; i < NINTER; i++)
        if (INTER[i].mat == mat && INTER[i].other == other) li = i;
    if (li < 0) {
        if (NINTER >= 512) return -1;
        li = NINTER++;
        INTER[li].mat = mat;
        INTER[li].other = other;
        INTER[li].n = 0;
    }
    if (INTER[li].n >= 4) return -1;
    inter_t *e = &INTER[li].e[INTER[li].n++];
    e->kind = kind;
    e->data1 = data1;
    e->data2 = data2;
    e->ofsx = ofs_x;
    e->ofsy = ofs_y;
    M[mat].interact = 1;
    HAS_INTER = 1;
    return 0;
}

static const inter_list_t *find_inter(int mat, int other) {
    for (int i = 0; i < NINTER; i++)
        if (INTER[i].mat == mat && INTER[i].other == other) return &INTER[i];
    return NULL;
}

int om_material_count(void) { return NMAT; }

/* MaterialInstance::temperature of a new tile of the material (TilesCreate) */
int om_material_tile_temperature(int mat) {
    if (mat < 0 || mat >= NMAT) return 0;
    return M[mat].type == T_SOUP ? M[mat].f_temp : M[mat].f_scalar;
}

/* every material's reactions (4 rows of kind, temperature, result; kind 0 = none)
 * and the interactions in registration order (material, other, kind, data1, data2,
 * ofs_x, ofs_y); returns the number of interaction rows (up to cap written) */
int om_material_rules(int32_t *react, int32_t *inter, int cap) {
    memset(react, 0, sizeof(int32_t) * 12 * (size_t)NMAT);
    for (int m = 0; m < NMAT; m++)
        for (int q = 0; q < M[m].n_react; q++) {
            react[12 * m + 3 * q] = M[m].react[q].kind;
            react[12 * m + 3 * q + 1] = M[m].react[q].data1;
            react[12 * m + 3 * q + 2] = M[m].react[q].data2;
        }
    int n = 0;
    for (int i = 0; i < NINTER; i++)
        for (int q = 0; q < INTER[i].n; q++, n++) {
            if (n >= cap) continue;
            const inter_t *e = &INTER[i].e[q];
            int32_t *r = inter + 7 * n;
            r[0] = INTER[i].mat;
            r[1] = INTER[i].other;
            r[2] = e->kind;
            r[3] = e->data1;
            r[4] = e->data2;
            r[5] = e->ofsx;
            r[6] = e->ofsy;
        }
    return n;
}

void om_material_get(int id, int32_t out[16]) {
    const mat_t *m = &M[id];
    int32_t dbits;
    memcpy(&dbits, &m->density, 4);
    out[0] = m->type;
    out[1] = dbits;
    out[2] = m->iterations;
    out[3] = m->slip;
    out[4] = m->max_stab;
    out[5] = m->alpha;
    out[6] = (int32_t)m->colour;
    out[7] = m->emit;
    out[8] = (int32_t)m->emit_colour;
    out[9] = (int32_t)m->f_base;
    out[10] = m->f_shift;
    out[11] = m->f_lo;
    out[12] = m->f_mod;
    out[13] = m->f_scalar;
    out[14] = m->n_react;
    out[15] = m->interact;
}

/* --------------------------------------------------------------------- world */
typedef struct {
    uint16_t id;
    uint8_t fl;
    int32_t sc;
    uint32_t col;
    int32_t df;
    int16_t tp; /* temperature of a SOUP tile (its scalar holds the amount); 0 otherwise */
} cell_t;

typedef struct {
    om_particle *p;
    int n, cap;
} pvec;

static void pv_push(pvec *v, const om_particle *p) {
    if (v->n == v->cap) {
        v->cap = v->cap ? v->cap * 2 : 64;
        v->p = (om_particle *)realloc(v->p, (size_t)v->cap * sizeof(om_particle));
    }
    v->p[v->n++] = *p;
}

#define LED_CN 0
#define LED_DN 1
#define LED_XN 2
#define LED_CF 3
#define LED_DF 4
#define LED_XF 5

struct om_world {
    int W, H, C, cell_iter;
    uint32_t seed, tick;
    int temp_on; /* om_world_step runs om_tick_temperature every 4th tick */
    uint16_t *id;
    uint32_t *col;
    int32_t *sc;
    uint8_t *fl;
    int32_t *df;
    int16_t *tp; /* SOUP cells: MaterialInstance::temperature (other cells keep it in sc) */
    uint8_t *vis;
    pvec parts;
    int64_t led[6][MAXMAT];
    /* race checker */
    int check;
    long viol;
    int32_t stamp;
    int32_t *wst, *wown, *rst, *rown;
    /* render state (om_render_enable): cells written since the last dirty pass, the
     * tick's per-cell flows (Q16.16, x then y, wrapping int32 sums), the textures
     * (4 bytes r, g, b, a per cell) and the smoothed flows */
    uint8_t *dirty;
    int32_t *flow;
    uint32_t *tex[5];
    float *pflow;
    /* f32 liquid amounts and diffs (om_world_set_f32): the reference's own float
     * arithmetic; the ledger and census keep no fluid rows */
    int f32;
    /* world::tickZone (world.hpp:138): chunk origins of the tick, the particles that
     * move and the cells the temperature step updates; the whole world by default */
    int zx, zy, zw, zh;
};

static inline void mark_dirty(om_world *w, size_t i) {
    if (w->dirty) w->dirty[i] = 1;
}
static inline void add_flow(om_world *w, int x, int y, int axis, int32_t v) {
    if (!w->flow || x < 0 || y < 0 || x >= w->W || y >= w->H) return;
    int32_t *f = &w->flow[2 * ((size_t)y * w->W + x) + axis];
    *f = (int32_t)((uint32_t)*f + (uint32_t)v);
}

static inline int inw(const om_world *w, int x, int y) { return x >= 0 && y >= 0 && x < w->W && y < w->H; }

/* f32 bit patterns of the 32-bit planes (f32 worlds) */
static inline float i2f(int32_t v) {
    float f;
    memcpy(&f, &v, 4);
    return f;
}
static inline int32_t f2i(float f) {
    int32_t v;
    memcpy(&v, &f, 4);
    return v;
}
/* the amount of a new SOUP tile: the factory's Q16.16 scalar, or its f32 value in f32
 * worlds (a temperature for other materials) */
static inline int32_t soup_scalar(const om_world *w, int mid) {
    if (!w->f32 || M[mid].type != T_SOUP) return M[mid].f_scalar;
    return f2i((float)M[mid].f_scalar * (1.0f / 65536.0f));
}
/* f32 worlds: flowX / flowY of a cell as float bits, added in the reference's order */
static inline void add_flow_f(om_world *w, int x, int y, int axis, float v, int sub) {
    if (!w->flow || x < 0 || y < 0 || x >= w->W || y >= w->H) return;
    int32_t *f = &w->flow[2 * ((size_t)y * w->W + x) + axis];
    *f = f2i(sub ? i2f(*f) - v : i2f(*f) + v);
}

void om_world_set_f32(om_world *w, int on) { w->f32 = on ? 1 : 0; }

om_world *om_world_new(int w, int h, int chunk, int cell_iter, uint32_t seed) {
    if (w <= 0 || h <= 0 || chunk < 16 || cell_iter < 0) return NULL;
    om_world *wd = (om_world *)calloc(1, sizeof(om_world));
    size_t n = (size_t)w * h;
    wd->W = w;
    wd->H = h;
    wd->C = chunk;
    wd->cell_iter = cell_iter;
    wd->seed = seed;
    wd->id = (uint16_t *)calloc(n, 2);
    wd->col = (uint32_t *)calloc(n, 4);
    wd->sc = (int32_t *)calloc(n, 4);
    wd->fl = (uint8_t *)calloc(n, 1);
    wd->df = (int32_t *)calloc(n, 4);
    wd->tp = (int16_t *)calloc(n, 2);
    wd->vis = (uint8_t *)calloc(n, 1);
    for (size_t i = 0; i < n; i++) wd->id[i] = (uint16_t)ID_AIR;
    wd->zx = 0;
    wd->zy = 0;
    wd->zw = w;
    wd->zh = h;
    return wd;
}

int om_world_set_tick_zone(om_world *wd, int x, int y, int w, int h) {
    if (x < 0 || y < 0 || w < 0 || h < 0 || x + w > wd->W || y + h > wd->H) return -1;
    wd->zx = x;
    wd->zy = y;
    wd->zw = w;
    wd->zh = h;
    return 0;
}
static inline int in_zone(const om_world *w, int x, int y) {
    return x >= w->zx && y >= w->zy && x < w->zx + w->zw && y < w->zy + w->zh;
}

void om_world_free(om_world *wd) {
    if (!wd) return;
    free(wd->id);
    free(wd->col);
    free(wd->sc);
    free(wd->fl);
    free(wd->df);
    free(wd->tp);
    free(wd->vis);
    free(wd->parts.p);
    free(wd->wst);
    free(wd->wown);
    free(wd->rst);
    free(wd->rown);
    free(wd->dirty);
    free(wd->flow);
    for (int k = 0; k < 5; k++) free(wd->tex[k]);
    free(wd->pflow);
    free(wd);
}

void om_world_set(om_world *wd, const uint16_t *id, const uint32_t *col, const int32_t *sc, const uint8_t *fl,
                  const int32_t *df) {
    size_t n = (size_t)wd->W * wd->H;
    memcpy(wd->id, id, n * 2);
    memcpy(wd->col, col, n * 4);
    memcpy(wd->sc, sc, n * 4);
    memcpy(wd->fl, fl, n);
    memcpy(wd->df, df, n * 4);
    if (wd->dirty) memset(wd->dirty, 1, n);
}

void om_world_get(const om_world *wd, uint16_t *id, uint32_t *col, int32_t *sc, uint8_t *fl, int32_t *df) {
    size_t n = (size_t)wd->W * wd->H;
    memcpy(id, wd->id, n * 2);
    memcpy(col, wd->col, n * 4);
    memcpy(sc, wd->sc, n * 4);
    memcpy(fl, wd->fl, n);
    memcpy(df, wd->df, n * 4);
}

void om_world_set_tick(om_world *wd, uint32_t t) { wd->tick = t; }
uint32_t om_world_get_tick(const om_world *wd) { return wd->tick; }

/* ----------------------------------------------------------- race checker */
static void chk_init(om_world *w) {
    size_t n = (size_t)w->W * w->H;
    if (!w->wst) {
        w->wst = (int32_t *)calloc(n, 4);
        w->wown = (int32_t *)calloc(n, 4);
        w->rst = (int32_t *)calloc(n, 4);
        w->rown = (int32_t *)calloc(n, 4);
    }
}
static int32_t g_owner; /* linear index of the active cell (checker runs single-threaded) */
static inline void chk(om_world *w, int x, int y, int write) {
    if (!w->check || !inw(w, x, y)) return;
    size_t i = (size_t)y * w->W + x;
    int32_t s = w->stamp, o = g_owner;
    if (w->wst[i] == s && w->wown[i] != o) w->viol++;
    if (write) {
        if (w->rst[i] == s && w->rown[i] != o) w->viol++;
        w->wst[i] = s;
        w->wown[i] = o;
    } else {
        if (w->rst[i] == s) {
            if (w->rown[i] != o) w->rown[i] = -2;
        } else {
            w->rst[i] = s;
            w->rown[i] = o;
        }
    }
}

/* ------------------------------------------------------- cell accessors */
/* getTile/setTile bounds policy, world.cpp:999-1008, applied to every access */
static inline int gid(om_world *w, int x, int y) {
    chk(w, x, y, 0);
    return inw(w, x, y) ? w->id[(size_t)y * w->W + x] : ID_SOLID;
}
static inline int gtype(om_world *w, int x, int y) { return M[gid(w, x, y)].type; }
static inline cell_t gcell(om_world *w, int x, int y) {
    cell_t c;
    chk(w, x, y, 0);
    if (!inw(w, x, y)) {
        c.id = (uint16_t)ID_SOLID;
        c.fl = 0;
        c.sc = 0;
        c.col = 0xff0000u;
        c.df = 0;
        c.tp = 0;
        return c;
    }
    size_t i = (size_t)y * w->W + x;
    c.id = w->id[i];
    c.fl = w->fl[i];
    c.sc = w->sc[i];
    c.col = w->col[i];
    c.df = (M[c.id].type == T_SOUP) ? w->df[i] : 0;
    c.tp = (M[c.id].type == T_SOUP) ? w->tp[i] : 0;
    return c;
}
static inline void pcell(om_world *w, int x, int y, cell_t c) {
    chk(w, x, y, 1);
    if (!inw(w, x, y)) return;
    size_t i = (size_t)y * w->W + x;
    w->id[i] = c.id;
    w->fl[i] = c.fl;
    w->sc[i] = c.sc;
    w->col[i] = c.col;
    w->df[i] = (M[c.id].type == T_SOUP) ? c.df : 0;
    if (M[c.id].type == T_SOUP) w->tp[i] = c.tp;
    mark_dirty(w, i);
}
static inline void set_moved(om_world *w, int x, int y, int on) {
    chk(w, x, y, 1);
    if (!inw(w, x, y)) return;
    size_t i = (size_t)y * w->W + x;
    uint8_t f = on ? (uint8_t)(w->fl[i] | MOVED) : (uint8_t)(w->fl[i] & (uint8_t)~MOVED);
    if (f != w->fl[i]) {
        w->fl[i] = f;
        mark_dirty(w, i); /* a write that changes nothing marks nothing */
    }
}
static inline void add_diff(om_world *w, int x, int y, int32_t v) {
    chk(w, x, y, 1);
    if (!inw(w, x, y)) return;
    w->df[(size_t)y * w->W + x] += v;
}
static inline int getvis(om_world *w, int x, int y) {
    chk(w, x, y, 0);
    return inw(w, x, y) ? w->vis[(size_t)y * w->W + x] : 0;
}
static inline void setvis(om_world *w, int x, int y) {
    chk(w, x, y, 1);
    if (inw(w, x, y)) w->vis[(size_t)y * w->W + x] = 1;
}

static inline cell_t nothing(void) {
    cell_t c = {(uint16_t)ID_AIR, 0, 0, 0u, 0, 0};
    return c;
}

/* ------------------------------------------------------------ rule context */
typedef struct {
    om_world *w;
    uint32_t pk; /* pass key for (tick, iter, sweep) */
    uint32_t ck; /* cell key */
    uint32_t k;  /* draw counter */
    int iter;
    pvec *spawn; /* particles spawned by this chunk-pass, in order */
    int64_t (*led)[MAXMAT];
    /* partitioned order only: AIR-ness of the cells below the chunk as they stood
     * when sweep B began, for the friction pillar (NULL: read the live grid) */
    const uint8_t *snap;
    int snap_x0, snap_y0, snap_w, snap_h;
} rctx;

/* the pillar cell (x, y) is AIR: in the snapshot when there is one, else live */
static inline int pillar_air(rctx *c, int x, int y) {
    if (!c->snap) return gtype(c->w, x, y) == T_AIR;
    int sx = x - c->snap_x0, sy = y - c->snap_y0;
    if (sx < 0 || sy < 0 || sx >= c->snap_w || sy >= c->snap_h) return 0;
    return c->snap[sy * c->snap_w + sx];
}

static inline uint32_t D(rctx *c) { return draw_k(c->ck, c->k++); }

static inline void led_add(rctx *c, int row, int mat, int64_t v) {
    if (mat < 0 || M[mat].type == T_AIR || v == 0) return;
    if (c->w->f32 && row >= LED_CF) return; /* f32 amounts: no fluid rows */
#pragma omp atomic
    c->led[row][mat] += v;
}

/* account a cell replaced by a conversion (not a move) */
static void led_replace(rctx *c, cell_t old, cell_t nw) {
    led_add(c, LED_DN, old.id, 1);
    if (M[old.id].type == T_SOUP) led_add(c, LED_DF, old.id, (int64_t)old.sc + old.df);
    led_add(c, LED_CN, nw.id, 1);
    if (M[nw.id].type == T_SOUP) led_add(c, LED_CF, nw.id, (int64_t)nw.sc + nw.df);
}

/* TilesCreate(id, x, y), game_datastruct.cpp:494-574: colour from the factory
 * (one draw when the factory jitters a channel), scalar = temperature or, for
 * SOUP materials, the default amount */
static cell_t create_tile(rctx *c, int mid) {
    const mat_t *m = &M[mid];
    cell_t t;
    t.id = (uint16_t)mid;
    t.fl = 0;
    t.df = 0;
    t.sc = soup_scalar(c->w, mid);
    t.tp = (m->type == T_SOUP) ? (int16_t)m->f_temp : 0;
    t.col = m->f_base;
    if (m->f_mod > 0) t.col = m->f_base + ((uint32_t)(m->f_lo + (int)(D(c) % (uint32_t)m->f_mod)) << m->f_shift);
    return t;
}

static void spawn(rctx *c, cell_t tile, int x, int y, float vx, float vy, float ax, float ay, int temporary,
                  int lifetime, int fade) {
    /* CellData(tile, x, y, vx, vy, ax, ay), source/engine/game_utils/cells.h:15-35 */
    om_particle p;
    memset(&p, 0, sizeof(p));
    p.x = (float)x;
    p.y = (float)y;
    p.vx = vx;
    p.vy = vy;
    p.ax = ax;
    p.ay = ay;
    p.lifetime = lifetime;
    p.fade_time = fade;
    p.colour = tile.col;
    p.scalar = tile.sc;
    p.temperature = (M[tile.id].type == T_SOUP) ? tile.tp : 0;
    p.id = tile.id;
    p.flags = tile.fl;
    p.bits = (uint8_t)(temporary ? 2 : 0);
    pv_push(c->spawn, &p);
}

/* CalculateVerticalFlowValue, world.cpp:1021-1034, in Q16.16 */
static inline int32_t vflow(int32_t rem, int32_t dst) {
    int64_t sum = (int64_t)rem + dst;
    if (sum <= Q_MAXV) return Q_MAXV;
    if (sum < 2 * Q_MAXV + Q_MAXCOMP)
        return (int32_t)(((int64_t)Q_MAXV * Q_MAXV + sum * Q_MAXCOMP) / (Q_MAXV + Q_MAXCOMP));
    return (int32_t)((sum + Q_MAXCOMP) / 2);
}
static inline int32_t clampflow(int32_t flow, int32_t rem) {
    /* world.cpp:1320-1321 and the three copies below it */
    if (flow < 0) flow = 0;
    int32_t lim = rem < Q_MAXFLOW ? rem : Q_MAXFLOW;
    if (flow > lim) flow = lim;
    return flow;
}

/* CalculateVerticalFlowValue, world.cpp:1021-1034, in the reference's f32 (every
 * operation rounded on its own: the oracle is built with -ffp-contract=off) */
static inline float vflow_f(float rem, float dst) {
    float sum = rem + dst;
    if (sum <= 0.5f) return 0.5f;
    if (sum < 2 * 0.5f + 0.1f) return (0.5f * 0.5f + sum * 0.1f) / (0.5f + 0.1f);
    return (sum + 0.1f) / 2.0f;
}
/* std::max(flow, 0.0f) and the std::min(FLUID_MaxFlow, rem) cap, world.cpp:1320-1321;
 * the FLUID_FlowSpeed factor (1.0f) changes no float */
static inline float clampflow_f(float flow, float rem) {
    if (flow < 0.0f) flow = 0.0f;
    float lim = rem < 8.0f ? rem : 8.0f;
    return flow > lim ? lim : flow;
}
/* one f32 flow from (x, y) towards (x + dx, y + dy), world.cpp:1309-1460 */
static void soup_flow_f(rctx *c, const cell_t *t, float *rem, float *dfv, float flow, int nT, int x, int y, int dx,
                        int dy) {
    om_world *w = c->w;
    if (flow == 0.0f) return;
    *rem -= flow;
    *dfv -= flow;
    if (nT == T_AIR) {
        cell_t nt = {t->id, 0, f2i(0.0f), t->col, f2i(0.0f + flow), t->tp};
        pcell(w, x + dx, y + dy, nt);
        led_add(c, LED_CN, t->id, 1);
    } else if (inw(w, x + dx, y + dy)) {
        chk(w, x + dx, y + dy, 1);
        int32_t *d = &w->df[(size_t)(y + dy) * w->W + x + dx];
        *d = f2i(i2f(*d) + flow);
    }
    add_flow_f(w, x, y, dx != 0 ? 0 : 1, flow, (dx + dy) < 0);
}
/* world.cpp:1269-1567 with f32 amounts; the cell's diff (t->df) already holds the
 * flows of the cells updated before it, and its own flows are subtracted in order */
static void rule_a_soup_f32(rctx *c, cell_t t, int x, int y) {
    om_world *w = c->w;
    float amount = i2f(t.sc);
    if (amount == 0.0f) return;
    if (amount < 0.0005f) {
        t.sc = f2i(0.0f);
        pcell(w, x, y, t);
        return;
    }
    if ((double)amount > 0.005 && gtype(w, x, y + 1) == T_AIR && gtype(w, x, y + 2) == T_AIR &&
        gtype(w, x, y + 3) == T_AIR && gtype(w, x, y + 4) == T_AIR) { /* world.cpp:1283-1305 */
        pcell(w, x, y, nothing());
        int n = (int)(amount / 4);
        if (n < 1) n = 1;
        led_add(c, LED_CN, t.id, n - 1);
        for (int i = 0; i < n; i++) {
            cell_t nt = t;
            nt.sc = f2i(amount / (float)n);
            nt.df = 0;
            nt.fl = 0;
            float vx = (float)((int)(D(c) % 10) - 5) / 30.0f;
            float vy = (float)(-((int)(D(c) % 2) + 3)) / 10.0f + 1.0f;
            spawn(c, nt, x, y + 1, vx, vy, 0.0f, 0.1f, 0, 0, 60);
        }
        return;
    }
    if (t.fl & MOVED) return;
    float start = amount, rem = amount, dfv = i2f(t.df);
    cell_t bottom = gcell(w, x, y + 1);
    int bT = M[bottom.id].type;
    int airBelow = bT == T_AIR;
    if ((airBelow && c->iter <= 2) || bottom.id == t.id) {
        float dst = (bT == T_SOUP) ? i2f(bottom.sc) : 0.0f;
        soup_flow_f(c, &t, &rem, &dfv, clampflow_f(vflow_f(start, dst) - dst, start), bT, x, y, 0, 1);
    } else if (c->iter == 0 && bT == T_SOUP && bottom.id != t.id) {
        if (D(c) % 10 == 0) {
            t.df = f2i(dfv);
            pcell(w, x, y, bottom);
            pcell(w, x, y + 1, t);
            return;
        }
    }
    if (rem < 0.0005f) {
        t.df = f2i(dfv - rem);
        pcell(w, x, y, t);
        return;
    }
    cell_t left = gcell(w, x - 1, y);
    int lT = M[left.id].type;
    int canL = (lT == T_AIR || left.id == t.id) && !airBelow;
    cell_t right = gcell(w, x + 1, y);
    int rT = M[right.id].type;
    int canR = (rT == T_AIR || right.id == t.id) && !airBelow;
    if (canL) {
        float dst = (lT == T_SOUP) ? i2f(left.sc) : 0.0f;
        soup_flow_f(c, &t, &rem, &dfv, clampflow_f((rem - dst) / (canR ? 3.0f : 2.0f), rem), lT, x, y, -1, 0);
    }
    if (rem < 0.0005f) {
        t.df = f2i(dfv - rem);
        pcell(w, x, y, t);
        return;
    }
    if (canR) {
        float dst = (rT == T_SOUP) ? i2f(right.sc) : 0.0f;
        soup_flow_f(c, &t, &rem, &dfv, clampflow_f((rem - dst) / 2.0f, rem), rT, x, y, 1, 0);
    }
    if (rem < 0.0005f) {
        t.df = f2i(dfv - rem);
        pcell(w, x, y, t);
        return;
    }
    cell_t top = gcell(w, x, y - 1);
    int tT = M[top.id].type;
    if (tT == T_AIR || top.id == t.id) {
        float dst = (tT == T_SOUP) ? i2f(top.sc) : 0.0f;
        soup_flow_f(c, &t, &rem, &dfv, clampflow_f(rem - vflow_f(rem, dst), rem), tT, x, y, 0, -1);
    } else if (c->iter == 0 && tT == T_SOUP && top.id != t.id) {
        if (D(c) % 10 == 0) {
            t.df = f2i(dfv);
            pcell(w, x, y, top);
            pcell(w, x, y - 1, t);
            return;
        }
    }
    if (rem < 0.0005f) {
        t.df = f2i(dfv - rem);
        pcell(w, x, y, t);
        return;
    }
    if (start == rem) { /* world.cpp:1472-1483 */
        uint8_t s = t.fl & SETTLE_MASK;
        if (s < SETTLE_MASK) s++;
        t.fl = (uint8_t)((t.fl & ~SETTLE_MASK) | s);
        if (s >= 10) t.fl |= MOVED;
    } else {
        if (tT == T_SOUP) set_moved(w, x, y - 1, 0);
        if (bT == T_SOUP) set_moved(w, x, y + 1, 0);
        if (lT == T_SOUP) set_moved(w, x - 1, y, 0);
        if (rT == T_SOUP) set_moved(w, x + 1, y, 0);
    }
    t.df = f2i(dfv);
    pcell(w, x, y, t);
    /* WATER on LAVA, world.cpp:1519-1537 */
    if ((int)t.id == ID_WATER && gid(w, x, y + 1) == ID_LAVA) {
        cell_t st = create_tile(c, ID_STEAM);
        led_replace(c, t, st);
        pcell(w, x, y, st);
        cell_t ob = create_tile(c, ID_OBSIDIAN);
        led_replace(c, gcell(w, x, y + 1), ob);
        pcell(w, x, y + 1, ob);
        setvis(w, x, y + 1);
        for (int xx = -1; xx <= 1; xx++)
            for (int yy = 0; yy <= 2; yy++) {
                if (gid(w, x + xx, y + yy) == ID_LAVA) {
                    cell_t o2 = create_tile(c, ID_OBSIDIAN);
                    led_replace(c, gcell(w, x + xx, y + yy), o2);
                    pcell(w, x + xx, y + yy, o2);
                    setvis(w, x + xx, y + yy);
                }
            }
    }
}

/* ---------------------------------------------------------------- sweep A */
static void rule_a(rctx *c, int x, int y) {
    om_world *w = c->w;
    if (getvis(w, x, y)) return; /* world.cpp:1091 */
    cell_t t = gcell(w, x, y);
    const mat_t *m = &M[t.id];
    if (c->iter >= m->iterations) { /* world.cpp:1093-1096 */
        setvis(w, x, y);
        return;
    }
    int type = m->type;
    c->ck = cell_key(c->pk, (uint32_t)x, (uint32_t)y);
    c->k = 0;

    if ((int)t.id == ID_FIRE) { /* world.cpp:1101-1146 */
        if (D(c) % 10 == 0) t.col = (255u << 16) | ((uint32_t)(100 + (int)(D(c) % 50)) << 8) | 50u;
        if (D(c) % 10 == 0) {
            float vx = (float)((int)(D(c) % 10) - 5) / 20.0f;
            float vy = -((float)(int)(D(c) % 10) / 10.0f) / 3.0f + -0.5f;
            spawn(c, t, x, y - 1, vx, vy, 0.0f, 0.01f, 1, 30, 10);
            led_add(c, LED_CN, t.id, 1);
        }
        if (D(c) % 150 == 0) {
            led_replace(c, t, nothing());
            pcell(w, x, y, nothing());
            setvis(w, x, y);
        } else {
            int found = 0;
            for (int xx = -2; xx <= 2; xx++)
                for (int yy = -2; yy <= 2; yy++) {
                    if (gtype(w, x + xx, y + yy) == T_SOLID) {
                        found = 1;
                        if (D(c) % 500 == 0) {
                            cell_t f = create_tile(c, ID_FIRE);
                            if (inw(w, x + xx, y + yy)) led_replace(c, gcell(w, x + xx, y + yy), f);
                            pcell(w, x + xx, y + yy, f);
                            setvis(w, x + xx, y + yy);
                        }
                    }
                }
            if (!found && D(c) % 120 == 0) {
                led_replace(c, gcell(w, x, y), nothing());
                pcell(w, x, y, nothing());
                setvis(w, x, y);
            }
        }
    }

    if (type == T_SAND) {
        cell_t below = gcell(w, x, y + 1); /* world.cpp:1150 */
        int bt = M[below.id].type;
        const inter_list_t *il = m->interact ? find_inter(t.id, below.id) : NULL;
        if (il && il->n > 0) { /* world.cpp:1153-1179 */
            for (int i = 0; i < il->n; i++) {
                const inter_t *in = &il->e[i];
                /* the radius (MaterialInteraction::data2) is a u32, so the loops'
                 * `xx <= ofsX + data2` compares unsigned: a box whose low corner
                 * ofs - radius is negative is not visited at all (when ofs + radius
                 * is negative too the reference never leaves the loop; empty here) */
                if (in->ofsx - in->data2 < 0 || in->ofsy - in->data2 < 0) continue;
                for (int xx = in->ofsx - in->data2; xx <= in->ofsx + in->data2; xx++)
                    for (int yy = in->ofsy - in->data2; yy <= in->ofsy + in->data2; yy++) {
                        if (in->kind == INTER_TRANSFORM) {
                            if (gid(w, x + xx, y + yy) == below.id) {
                                cell_t nt = create_tile(c, in->data1);
                                if (inw(w, x + xx, y + yy)) led_replace(c, gcell(w, x + xx, y + yy), nt);
                                pcell(w, x + xx, y + yy, nt);
                                setvis(w, x + xx, y + yy);
                            }
                        } else {
                            if ((xx == 0 && yy == 0) || gid(w, x + xx, y + yy) == ID_AIR) {
                                cell_t nt = create_tile(c, in->data1);
                                if (inw(w, x + xx, y + yy)) led_replace(c, gcell(w, x + xx, y + yy), nt);
                                pcell(w, x + xx, y + yy, nt);
                                setvis(w, x + xx, y + yy);
                            }
                        }
                    }
            }
            return;
        }
        if (m->n_react > 0) { /* world.cpp:1181-1204 */
            int react = 0;
            for (int i = 0; i < m->n_react; i++) {
                const inter_t *r = &m->react[i];
                int hit = (r->kind == REACT_BELOW) ? (t.sc < r->data1) : (t.sc > r->data1);
                if (hit) {
                    cell_t nt = create_tile(c, r->data2);
                    /* keeps the temperature (:1188,1196): in the scalar, or beside the
                     * amount of a SOUP result */
                    if (M[nt.id].type != T_SOUP)
                        nt.sc = t.sc;
                    else
                        nt.tp = (int16_t)t.sc;
                    led_replace(c, gcell(w, x, y), nt);
                    pcell(w, x, y, nt);
                    setvis(w, x, y);
                    react = 1;
                }
            }
            if (react) return;
        }
        /* world.cpp:1206-1267 */
        int canB = (bt == T_AIR || (bt != T_SOLID && M[below.id].density < m->density));
        if (!canB) return;
        cell_t bl = gcell(w, x - 1, y + 1), br = gcell(w, x + 1, y + 1);
        int blt = M[bl.id].type, brt = M[br.id].type;
        int canL = (blt == T_AIR || (blt != T_SOLID && M[bl.id].density < m->density));
        int canR = (brt == T_AIR || (brt != T_SOLID && M[br.id].density < m->density));
        if (!((canL || canR) && D(c) % 20 == 0)) {
            if (bt == T_AIR && gtype(w, x, y + 2) == T_AIR && gtype(w, x, y + 3) == T_AIR &&
                gtype(w, x, y + 4) == T_AIR) {
                pcell(w, x, y, below);
                float vx = (float)((int)(D(c) % 10) - 5) / 20.0f;
                float vy = (float)(-((int)(D(c) % 2) + 3)) / 10.0f + 1.5f;
                spawn(c, t, x, y + 1, vx, vy, 0.0f, 0.1f, 0, 0, 60);
            } else {
                pcell(w, x, y, below);
                if (D(c) % 2 == 0) t.fl |= MOVED;
                pcell(w, x, y + 1, t);
                setvis(w, x, y + 1);
            }
            if (D(c) % 2 == 0) {
                if (x > 0 && gtype(w, x - 1, y + 1) == T_SAND) {
                    if (D(c) % 2 == 0) set_moved(w, x - 1, y + 1, 1);
                }
                if (x < w->W - 1 && gtype(w, x + 1, y + 1) == T_SAND) {
                    if (D(c) % 2 == 0) set_moved(w, x + 1, y + 1, 1);
                }
            }
        }
    } else if (type == T_SOUP && w->f32) {
        rule_a_soup_f32(c, t, x, y);
    } else if (type == T_SOUP) { /* world.cpp:1269-1567 */
        if (t.sc == 0) return;
        if (t.sc < Q_MINV) {
            led_add(c, LED_DF, t.id, t.sc);
            t.sc = 0;
            pcell(w, x, y, t);
            return;
        }
        if (t.sc > Q_FREEFALL && gtype(w, x, y + 1) == T_AIR && gtype(w, x, y + 2) == T_AIR &&
            gtype(w, x, y + 3) == T_AIR && gtype(w, x, y + 4) == T_AIR) { /* world.cpp:1283-1305 */
            pcell(w, x, y, nothing());
            int n = t.sc >> 18; /* int(amount / 4) */
            if (n < 1) n = 1;
            int32_t base = t.sc / n, extra = t.sc % n;
            led_add(c, LED_DF, t.id, t.df); /* the pending diff of the cell is dropped */
            led_add(c, LED_CN, t.id, n - 1);
            for (int i = 0; i < n; i++) {
                cell_t nt = t;
                nt.sc = base + (i < extra ? 1 : 0);
                nt.df = 0;
                nt.fl = 0;
                float vx = (float)((int)(D(c) % 10) - 5) / 30.0f;
                float vy = (float)(-((int)(D(c) % 2) + 3)) / 10.0f + 1.0f;
                spawn(c, nt, x, y + 1, vx, vy, 0.0f, 0.1f, 0, 0, 60);
            }
            return;
        }
        if (t.fl & MOVED) return;
        int32_t start = t.sc, rem = t.sc;
        cell_t bottom = gcell(w, x, y + 1);
        int bT = M[bottom.id].type;
        int airBelow = bT == T_AIR;
        if ((airBelow && c->iter <= 2) || bottom.id == t.id) {
            int32_t dst = (bT == T_SOUP) ? bottom.sc : 0;
            int32_t flow = clampflow(vflow(start, dst) - dst, start);
            if (flow != 0) {
                rem -= flow;
                t.df -= flow;
                if (bT == T_AIR) {
                    cell_t nt = {t.id, 0, 0, t.col, flow, t.tp};
                    pcell(w, x, y + 1, nt);
                    led_add(c, LED_CN, t.id, 1);
                } else
                    add_diff(w, x, y + 1, flow);
                add_flow(w, x, y, 1, flow); /* :1334 flowY += flow */
            }
        } else if (c->iter == 0 && bT == T_SOUP && bottom.id != t.id) {
            if (D(c) % 10 == 0) {
                pcell(w, x, y, bottom);
                pcell(w, x, y + 1, t);
                return;
            }
        }
        if (rem < Q_MINV) {
            t.df -= rem;
            led_add(c, LED_DF, t.id, rem);
            pcell(w, x, y, t);
            return;
        }
        cell_t left = gcell(w, x - 1, y);
        int lT = M[left.id].type;
        int canL = (lT == T_AIR || left.id == t.id) && !airBelow;
        cell_t right = gcell(w, x + 1, y);
        int rT = M[right.id].type;
        int canR = (rT == T_AIR || right.id == t.id) && !airBelow;
        if (canL) {
            int32_t dst = (lT == T_SOUP) ? left.sc : 0;
            int32_t flow = clampflow((rem - dst) / (canR ? 3 : 2), rem);
            if (flow != 0) {
                rem -= flow;
                t.df -= flow;
                if (lT == T_AIR) {
                    cell_t nt = {t.id, 0, 0, t.col, flow, t.tp};
                    pcell(w, x - 1, y, nt);
                    led_add(c, LED_CN, t.id, 1);
                } else
                    add_diff(w, x - 1, y, flow);
                add_flow(w, x, y, 0, -flow); /* :1374 flowX -= flow */
            }
        }
        if (rem < Q_MINV) {
            t.df -= rem;
            led_add(c, LED_DF, t.id, rem);
            pcell(w, x, y, t);
            return;
        }
        if (canR) {
            int32_t dst = (rT == T_SOUP) ? right.sc : 0;
            int32_t flow = clampflow((rem - dst) / 2, rem);
            if (flow != 0) {
                rem -= flow;
                t.df -= flow;
                if (rT == T_AIR) {
                    cell_t nt = {t.id, 0, 0, t.col, flow, t.tp};
                    pcell(w, x + 1, y, nt);
                    led_add(c, LED_CN, t.id, 1);
                } else
                    add_diff(w, x + 1, y, flow);
                add_flow(w, x, y, 0, flow); /* :1402 flowX += flow */
            }
        }
        if (rem < Q_MINV) {
            t.df -= rem;
            led_add(c, LED_DF, t.id, rem);
            pcell(w, x, y, t);
            return;
        }
        cell_t top = gcell(w, x, y - 1);
        int tT = M[top.id].type;
        if (tT == T_AIR || top.id == t.id) {
            int32_t dst = (tT == T_SOUP) ? top.sc : 0;
            int32_t flow = clampflow(rem - vflow(rem, dst), rem);
            if (flow != 0) {
                rem -= flow;
                t.df -= flow;
                if (tT == T_AIR) {
                    cell_t nt = {t.id, 0, 0, t.col, flow, t.tp};
                    pcell(w, x, y - 1, nt);
                    led_add(c, LED_CN, t.id, 1);
                } else
                    add_diff(w, x, y - 1, flow);
                add_flow(w, x, y, 1, -flow); /* :1432 flowY -= flow */
            }
        } else if (c->iter == 0 && tT == T_SOUP && top.id != t.id) {
            if (D(c) % 10 == 0) {
                pcell(w, x, y, top);
                pcell(w, x, y - 1, t);
                return;
            }
        }
        if (rem < Q_MINV) {
            t.df -= rem;
            led_add(c, LED_DF, t.id, rem);
            pcell(w, x, y, t);
            return;
        }
        if (start == rem) { /* world.cpp:1472-1483 */
            uint8_t s = t.fl & SETTLE_MASK;
            if (s < SETTLE_MASK) s++;
            t.fl = (uint8_t)((t.fl & ~SETTLE_MASK) | s);
            if (s >= 10) t.fl |= MOVED;
        } else {
            if (tT == T_SOUP) set_moved(w, x, y - 1, 0);
            if (bT == T_SOUP) set_moved(w, x, y + 1, 0);
            if (lT == T_SOUP) set_moved(w, x - 1, y, 0);
            if (rT == T_SOUP) set_moved(w, x + 1, y, 0);
        }
        pcell(w, x, y, t);
        /* WATER on LAVA, world.cpp:1519-1537 */
        if ((int)t.id == ID_WATER && gid(w, x, y + 1) == ID_LAVA) {
            cell_t st = create_tile(c, ID_STEAM);
            led_replace(c, t, st);
            pcell(w, x, y, st);
            cell_t ob = create_tile(c, ID_OBSIDIAN);
            led_replace(c, gcell(w, x, y + 1), ob);
            pcell(w, x, y + 1, ob);
            setvis(w, x, y + 1);
            for (int xx = -1; xx <= 1; xx++)
                for (int yy = 0; yy <= 2; yy++) {
                    if (gid(w, x + xx, y + yy) == ID_LAVA) {
                        cell_t o2 = create_tile(c, ID_OBSIDIAN);
                        led_replace(c, gcell(w, x + xx, y + yy), o2);
                        pcell(w, x + xx, y + yy, o2);
                        setvis(w, x + xx, y + yy);
                    }
                }
            return;
        }
    } else if (type == T_GAS) { /* world.cpp:1569-1585 */
        int above = gtype(w, x, y - 1);
        int aboveL = gtype(w, x - 1, y - 1);
        int aboveR = gtype(w, x + 1, y - 1);
        if (above == T_AIR && !((aboveL == T_AIR || aboveR == T_AIR) && D(c) % 2 == 0)) {
            pcell(w, x, y, gcell(w, x, y - 1));
            pcell(w, x, y - 1, t);
            setvis(w, x, y - 1);
        }
    }
}

/* ---------------------------------------------------------------- sweep B */
static void rule_b(rctx *c, int x, int y) {
    om_world *w = c->w;
    if (getvis(w, x, y)) return; /* world.cpp:1597 */
    cell_t t = gcell(w, x, y);
    const mat_t *m = &M[t.id];
    int type = m->type;
    if (type != T_SAND && type != T_SOUP && type != T_GAS) return;
    c->ck = cell_key(c->pk, (uint32_t)x, (uint32_t)y);
    c->k = 0;
    if (type == T_SAND) { /* world.cpp:1602-1727 */
        cell_t bl = gcell(w, x - 1, y + 1), br = gcell(w, x + 1, y + 1);
        int blt = M[bl.id].type, brt = M[br.id].type;
        int canL = (blt == T_AIR || (blt != T_SOLID && M[bl.id].density < m->density));
        int canR = (brt == T_AIR || (brt != T_SOLID && M[br.id].density < m->density));
        int stopped = !(t.fl & MOVED);
        int slip = m->slip;
        if (stopped) {
            int drop = 0;
            for (int pil = 0; pil < 10; pil++) {
                if (pillar_air(c, x - 1, y + 1 + pil) || pillar_air(c, x + 1, y + 1 + pil)) drop++;
            }
            int d = drop + 1 - m->max_stab;
            if (d > 0) {
                int chance = 1000 / d;
                if (chance < 1000) {
                    if (D(c) % (uint32_t)chance == 0) {
                        stopped = 0;
                        set_moved(w, x, y, 1);
                    }
                }
            }
        }
        if (stopped || !(canL || canR)) {
            set_moved(w, x, y, 0);
            return;
        }
        int shouldMove = (slip > 0) ? (D(c) % (uint32_t)(2 * slip) != 0) : 1;
        if (shouldMove && (canL || canR)) {
            if (D(c) % 2 == 0) {
                if (gtype(w, x, y + 1) == T_SAND) {
                    if (D(c) % 2 == 0) set_moved(w, x, y + 1, 1);
                }
            }
        }
        if (shouldMove && canL && (!canR || D(c) % 2 == 0)) {
            if (gtype(w, x - 1, y) == T_AIR) {
                pcell(w, x - 1, y, bl);
                setvis(w, x - 1, y);
                pcell(w, x, y, nothing());
            } else {
                pcell(w, x, y, bl);
                setvis(w, x, y);
            }
            if (slip > 0 && D(c) % (uint32_t)(20 * slip) == 0) t.fl &= (uint8_t)~MOVED;
            pcell(w, x - 1, y + 1, t);
            setvis(w, x - 1, y + 1);
        } else if (shouldMove && canR) {
            if (gtype(w, x + 1, y) == T_AIR) {
                pcell(w, x + 1, y, br);
                pcell(w, x, y, nothing());
            } else {
                pcell(w, x, y, br);
                setvis(w, x, y);
            }
            if (slip > 0 && D(c) % (uint32_t)(20 * slip) == 0) t.fl &= (uint8_t)~MOVED;
            pcell(w, x + 1, y + 1, t);
            setvis(w, x + 1, y + 1);
        } else {
            set_moved(w, x, y, 0);
        }
    } else if (type == T_SOUP && w->f32) { /* world.cpp:1728-1745 in f32 */
        float a = i2f(t.sc) + i2f(t.df);
        t.sc = f2i(a);
        t.df = f2i(0.0f);
        if (a < 0.0005f) {
            led_add(c, LED_DN, t.id, 1);
            pcell(w, x, y, nothing());
            setvis(w, x, y);
        } else {
            pcell(w, x, y, t);
            setvis(w, x, y);
        }
    } else if (type == T_SOUP) { /* world.cpp:1728-1745 */
        t.sc += t.df;
        t.df = 0;
        if (t.sc < Q_MINV) {
            led_add(c, LED_DN, t.id, 1);
            led_add(c, LED_DF, t.id, t.sc);
            pcell(w, x, y, nothing());
            setvis(w, x, y);
        } else {
            pcell(w, x, y, t);
            setvis(w, x, y);
        }
    } else { /* GAS, world.cpp:1799-1818 */
        int aboveL = gtype(w, x - 1, y - 1);
        int aboveR = gtype(w, x + 1, y - 1);
        if (aboveL == T_AIR && !(aboveR == T_AIR && D(c) % 2 == 0)) {
            pcell(w, x, y, gcell(w, x - 1, y - 1));
            pcell(w, x - 1, y - 1, t);
            setvis(w, x - 1, y - 1);
        } else if (aboveR == T_AIR) {
            pcell(w, x, y, gcell(w, x + 1, y - 1));
            pcell(w, x + 1, y - 1, t);
            setvis(w, x + 1, y - 1);
        }
    }
}

/* ---------------------------------------------------------------- sweep C */
static void rule_c(rctx *c, int x, int y) {
    om_world *w = c->w;
    if (getvis(w, x, y)) return; /* world.cpp:1831 */
    cell_t t = gcell(w, x, y);
    if (M[t.id].type != T_GAS) return;
    c->ck = cell_key(c->pk, (uint32_t)x, (uint32_t)y);
    c->k = 0;
    /* world.cpp:1862-1889 */
    int l = gtype(w, x - 1, y);
    int r = gtype(w, x + 1, y);
    if (l == T_AIR && !(r == T_AIR && D(c) % 2 == 0)) {
        pcell(w, x, y, gcell(w, x - 1, y));
        pcell(w, x - 1, y, t);
        setvis(w, x - 1, y);
    } else if (r == T_AIR) {
        pcell(w, x, y, gcell(w, x + 1, y));
        pcell(w, x + 1, y, t);
        setvis(w, x + 1, y);
    } else if ((int)t.id == ID_STEAM) {
        if (D(c) % 10 == 0) {
            cell_t wt = create_tile(c, ID_WATER);
            led_replace(c, t, wt);
            pcell(w, x, y, wt);
        }
    }
}

/* ------------------------------------------------------------ lattices */
/* Sub-phase lattice (Px, Py) per sweep and chunk mode: two cells of one sub-phase
 * differ by a multiple of Px in x or (same column) of Py in y, which keeps every
 * cell's write set disjoint from every other cell's read and write sets. */
enum { MODE_NARROW = 0, MODE_FIRE = 1, MODE_INTER = 2 };
static int DBG_PX[3] = {0, 0, 0}, DBG_PY[3] = {0, 0, 0};
/* test hook: force a lattice for one sweep (0 restores the derived one), so a test
 * can plant a too-small spacing and see the race checker fire */
void om_debug_set_lattice(int sweep, int px, int py) {
    if (sweep < 0 || sweep > 2) return;
    DBG_PX[sweep] = px;
    DBG_PY[sweep] = py;
}
static void lattice(int sweep, int mode, int *px, int *py) {
    if (DBG_PX[sweep] > 0) {
        *px = DBG_PX[sweep];
        *py = DBG_PY[sweep];
        return;
    }
    if (sweep == 0) {
        if (mode == MODE_INTER) {
            *px = 11;
            *py = 11;
        } else if (mode == MODE_FIRE) {
            *px = 5;
            *py = 7;
        } else {
            *px = 3;
            *py = 6;
        }
    } else if (sweep == 1) {
        /* the friction pillar reads a snapshot, so only rows y-1..y+1 are live */
        *px = 3;
        *py = 3;
    } else {
        *px = 3;
        *py = 1;
    }
}

static int chunk_mode(const om_world *w, int cx, int cy) {
    if (HAS_INTER) return MODE_INTER;
    if (ID_FIRE < 0) return MODE_NARROW;
    int x1 = cx + w->C < w->W ? cx + w->C : w->W, y1 = cy + w->C < w->H ? cy + w->C : w->H;
    for (int y = cy; y < y1; y++)
        for (int x = cx; x < x1; x++)
            if (w->id[(size_t)y * w->W + x] == (uint16_t)ID_FIRE) return MODE_FIRE;
    return MODE_NARROW;
}

typedef void (*rule_fn)(rctx *, int, int);

static void process_chunk(om_world *w, int order, int iter, int cx, int cy, pvec *spawn) {
    rctx c;
    memset(&c, 0, sizeof(c));
    c.w = w;
    c.iter = iter;
    c.spawn = spawn;
    c.led = w->led;
    int x1 = cx + w->C < w->W ? cx + w->C : w->W, y1 = cy + w->C < w->H ? cy + w->C : w->H;
    rule_fn rules[3] = {rule_a, rule_b, rule_c};
    int mode = (order == OM_ORDER_PART) ? chunk_mode(w, cx, cy) : MODE_NARROW;
    /* pillar snapshot region: columns cx-1 .. cx+C, rows cy+1 .. cy+C+9 */
    uint8_t *snap = NULL;
    c.snap_x0 = cx - 1;
    c.snap_y0 = cy + 1;
    c.snap_w = w->C + 2;
    c.snap_h = w->C + 9;
    for (int sweep = 0; sweep < 3; sweep++) {
        c.pk = pass_key(w->seed, w->tick, (uint32_t)(iter * 3 + sweep));
        if (sweep == 1 && order == OM_ORDER_PART) {
            /* partitioned order: the friction pillar of world.cpp:1619-1627 reads the
             * AIR cells as they stood when sweep B began */
            snap = (uint8_t *)malloc((size_t)c.snap_w * c.snap_h);
            for (int sy = 0; sy < c.snap_h; sy++)
                for (int sx = 0; sx < c.snap_w; sx++) {
                    int gx = c.snap_x0 + sx, gy = c.snap_y0 + sy;
                    snap[sy * c.snap_w + sx] =
                        (uint8_t)(inw(w, gx, gy) && M[w->id[(size_t)gy * w->W + gx]].type == T_AIR);
                }
            c.snap = snap;
        } else {
            c.snap = NULL;
        }
        if (order == OM_ORDER_SEQ) {
            /* world.cpp:1084-1087 (and 1589, 1823): bottom-to-top, left-to-right */
            for (int y = y1 - 1; y >= cy; y--)
                for (int x = cx; x < x1; x++) rules[sweep](&c, x, y);
        } else {
            int px, py;
            lattice(sweep, mode, &px, &py);
            for (int ry = py - 1; ry >= 0; ry--)
                for (int rx = 0; rx < px; rx++) {
                    w->stamp++;
                    for (int y = cy + ry; y < y1; y += py)
                        for (int x = cx + rx; x < x1; x += px) {
                            g_owner = y * w->W + x;
                            rules[sweep](&c, x, y);
                        }
                }
        }
    }
    free(snap);
}

long om_world_tick(om_world *w, int order, int check_races) {
    w->check = check_races ? 1 : 0;
    w->viol = 0;
    if (w->check) chk_init(w);
    /* chunks start at the tick zone's corner, every C cells while the start is in the
     * zone (world.cpp:1078-1079); a chunk reaches C cells whatever the zone's end */
    int nCx = (w->zw + w->C - 1) / w->C, nCy = (w->zh + w->C - 1) / w->C;
    size_t ncell = (size_t)w->W * w->H;
    for (int iter = 0; iter < w->cell_iter; iter++) { /* world.cpp:1050 */
        for (int tk = 0; tk < 4; tk++) {              /* world.cpp:1057-1060 */
            int ox = tk % 2, oy = 1 - tk / 2;
            memset(w->vis, 0, ncell); /* world.cpp:1046,1066-1067 */
            int na = (nCx - ox + 1) / 2, nb = (nCy - oy + 1) / 2;
            int nslot = na * nb;
            if (nslot <= 0) continue;
            pvec *sp = (pvec *)calloc((size_t)nslot, sizeof(pvec));
            /* chunks of one colour are independent (2-chunk spacing); slot order is
             * cx-major like the task push order of world.cpp:1073-1077 */
#pragma omp parallel for schedule(dynamic, 1) if (!w->check)
            for (int s = 0; s < nslot; s++) {
                int a = s / nb, b = s % nb;
                int cx = w->zx + (ox + 2 * a) * w->C, cy = w->zy + (oy + 2 * b) * w->C;
                process_chunk(w, order, iter, cx, cy, &sp[s]);
            }
            /* world.cpp:1901-1913: append spawned particles in task order */
            for (int s = 0; s < nslot; s++) {
                for (int i = 0; i < sp[s].n; i++) pv_push(&w->parts, &sp[s].p[i]);
                free(sp[s].p);
            }
            free(sp);
        }
    }
    w->tick++; /* world.cpp:1925 */
    w->check = 0;
    return w->viol;
}

/* --------------------------------------------------------------- particles */
#define P_PHASE 1u
#define P_TEMP 2u
#define P_STATE_SHIFT 2

static int SPIRAL_N = 0;
static int8_t SPIRAL[1024][2];
static void spiral_init(void) {
    /* the spiral walk of world.cpp:2105-2133 (X = Y = 32, maxI = 1024) */
    if (SPIRAL_N) return;
    int X = 32, Y = 32, x = 0, y = 0, dx = 0, dy = -1;
    int t = X > Y ? X : Y;
    int maxI = t * t;
    int n = 0;
    for (int j = 0; j < maxI; j++) {
        if ((-X / 2 <= x) && (x <= X / 2) && (-Y / 2 <= y) && (y <= Y / 2)) {
            SPIRAL[n][0] = (int8_t)x;
            SPIRAL[n][1] = (int8_t)y;
            n++;
        }
        if ((x == y) || ((x < 0) && (x == -y)) || ((x > 0) && (x == 1 - y))) {
            t = dx;
            dx = -dy;
            dy = t;
        }
        x += dx;
        y += dy;
    }
    SPIRAL_N = n;
}

enum { REQ_NONE = 0, REQ_DIRECT = 1, REQ_SPIRAL = 2 };
enum { OUT_ALIVE = 0, OUT_DEAD = 1 };

/* One particle's motion for world::tickCells (world.cpp:2032-2188) against the
 * grid as it stands before any deposit of this particle tick. Returns the request
 * kind; *out is OUT_DEAD when the particle is removed without a deposit. */
static int particle_move(om_world *w, om_particle *p, int *out, int *lx_o, int *ly_o) {
    *out = OUT_ALIVE;
    if ((p->bits & P_TEMP) && p->lifetime <= 0) { /* :2033-2037 */
        *out = OUT_DEAD;
        return -1; /* destroyed */
    }
    if (p->target_force != 0) { /* :2039-2051 */
        float tdx = p->target_x - p->x;
        float tdy = p->target_y - p->y;
        float nf = sqrtf(tdx * tdx + tdy * tdy);
        p->vx += tdx / nf * p->target_force;
        p->vy += tdy / nf * p->target_force;
        if (nf < 100) {
            p->vx *= 0.95f;
            p->vy *= 0.95f;
        }
    }
    int lx = (int)p->x, ly = (int)p->y;
    *lx_o = lx;
    *ly_o = ly;
    if (p->x < 0 || (int)p->x >= w->W || p->y < 0 || (int)p->y >= w->H) { /* :2056-2059 */
        *out = OUT_DEAD;
        return -2; /* exited */
    }
    if (!in_zone(w, lx, ly)) return REQ_NONE; /* :2061, outside the tick zone: kept as it is */
    p->vx += p->ax; /* :2063-2064 */
    p->vy += p->ay;
    int div = (int)((fabsf(p->vx) + fabsf(p->vy)) + 1);
    float dvx = p->vx / div;
    float dvy = p->vy / div;
    for (int i = 0; i < div; i++) { /* :2071-2184 */
        p->x += dvx;
        p->y += dvy;
        if (p->x < 0 || (int)p->x >= w->W || p->y < 0 || (int)p->y >= w->H) {
            *out = OUT_DEAD;
            return -2;
        }
        int ct = M[w->id[(size_t)(int)p->y * w->W + (int)p->x]].type;
        if (!(p->bits & P_PHASE) && ct != T_AIR) {
            int isObject = ct == T_OBJECT;
            int st = (p->bits >> P_STATE_SHIFT) & 3;
            if (st == 0)
                st = isObject ? 1 : 2;
            else if (st == 1 && !isObject)
                st = 2;
            p->bits = (uint8_t)((p->bits & ~(3u << P_STATE_SHIFT)) | ((unsigned)st << P_STATE_SHIFT));
            if (!isObject || st == 2) {
                if (p->bits & P_TEMP) {
                    *out = OUT_DEAD;
                    return -1;
                }
                if (M[w->id[(size_t)ly * w->W + lx]].type != T_AIR) return REQ_SPIRAL;
                return REQ_DIRECT;
            }
        }
    }
    if (p->lifetime > 0) p->lifetime--; /* :2186-2188 */
    return REQ_NONE;
}

/* target of a deposit against the current grid: 1 = fill an AIR cell, 2 = merge
 * into a cell of the same liquid, 0 = no target (world.cpp:2093-2147) */
static int find_target(om_world *w, const om_particle *p, int kind, int lx, int ly, int *tx, int *ty) {
    if (kind == REQ_DIRECT) {
        if (M[w->id[(size_t)ly * w->W + lx]].type == T_AIR) {
            *tx = lx;
            *ty = ly;
            return 1;
        }
    }
    int psoup = M[p->id].type == T_SOUP;
    for (int j = 0; j < SPIRAL_N; j++) {
        int cx = (int)(p->x + (float)SPIRAL[j][0]);
        int cy = (int)(p->y + (float)SPIRAL[j][1]);
        if (cx < 0 || cy < 0 || cx >= w->W || cy >= w->H) continue;
        int cid = w->id[(size_t)cy * w->W + cx];
        if (M[cid].type == T_AIR) {
            *tx = cx;
            *ty = cy;
            return 1;
        }
        if (psoup && cid == p->id) {
            *tx = cx;
            *ty = cy;
            return 2;
        }
    }
    return 0;
}

/* world::tickCells (world.cpp:2030-2195) as the reference runs it: particles one
 * after another in list order, each moving, colliding and depositing against the
 * grid as the particles before it left it (a deposit is visible to every later
 * particle's flight, its previous-cell test and its spiral search), then the stable
 * erase of the removed ones. */
int om_particles_tick(om_world *w) {
    spiral_init();
    int n = w->parts.n;
    om_particle *P = w->parts.p;
    uint8_t *dead = (uint8_t *)calloc((size_t)n + 1, 1);
    for (int i = 0; i < n; i++) {
        om_particle *p = &P[i];
        int lx = 0, ly = 0, out;
        int r = particle_move(w, p, &out, &lx, &ly);
        if (out == OUT_DEAD) {
            dead[i] = 1;
            int64_t f = (M[p->id].type == T_SOUP && !w->f32) ? p->scalar : 0; /* f32: no fluid rows */
            if (r == -2) {
                if (M[p->id].type != T_AIR) w->led[LED_XN][p->id] += 1;
                w->led[LED_XF][p->id] += f;
            } else {
                if (M[p->id].type != T_AIR) w->led[LED_DN][p->id] += 1;
                w->led[LED_DF][p->id] += f;
            }
            continue;
        }
        if (r != REQ_DIRECT && r != REQ_SPIRAL) continue;
        int tx = 0, ty = 0;
        int k = find_target(w, p, r, lx, ly, &tx, &ty);
        if (k == 0) { /* :2141-2144: no room found */
            p->vy = -4;
            p->y -= 16;
            continue;
        }
        size_t ci = (size_t)ty * w->W + tx;
        if (k == 2) { /* :2119-2125 */
            if (w->f32)
                w->sc[ci] = f2i(i2f(w->sc[ci]) + i2f(p->scalar));
            else
                w->sc[ci] += p->scalar;
            mark_dirty(w, ci);
            dead[i] = 1;
            w->led[LED_DN][p->id] += 1;
            continue;
        }
        /* :2115-2118 and :2148-2152 */
        w->id[ci] = p->id;
        w->col[ci] = p->colour;
        w->sc[ci] = p->scalar;
        if (M[p->id].type == T_SOUP) w->tp[ci] = p->temperature;
        mark_dirty(w, ci);
        w->fl[ci] = p->flags;
        w->df[ci] = 0;
        dead[i] = 1;
    }
    /* the stable erase (std::erase_if, :2179) and the y > height erase (:2190) */
    int m = 0;
    for (int i = 0; i < n; i++) {
        if (dead[i]) continue;
        if (P[i].y > (float)w->H) continue;
        P[m++] = P[i];
    }
    w->parts.n = m;
    free(dead);
    return m;
}

void om_tick_temperature(om_world *w);
/* game::tick's order (game.cpp:1839,1878-1889,2157-2159): world::tick(),
 * world::tickCells(), then world::tickTemperature() when enabled and the tick
 * index is 2 modulo GameTick (4, core/const.h:38) */
void om_world_step(om_world *wd, int order, int n) {
    for (int i = 0; i < n; i++) {
        uint32_t t = wd->tick;
        om_world_tick(wd, order, 0);
        om_particles_tick(wd);
        if (wd->temp_on && (t & 3u) == 2u) om_tick_temperature(wd);
    }
}
void om_world_set_temperature(om_world *wd, int on) { wd->temp_on = on ? 1 : 0; }

int om_particles_count(const om_world *wd) { return wd->parts.n; }
void om_particles_get(const om_world *wd, om_particle *out) {
    memcpy(out, wd->parts.p, (size_t)wd->parts.n * sizeof(om_particle));
}
void om_particles_set(om_world *wd, const om_particle *in, int n) {
    wd->parts.n = 0;
    for (int i = 0; i < n; i++) pv_push(&wd->parts, &in[i]);
}

/* FP64 / FP32 kinematics of one particle step (no deposits), for the precision
 * check of the FP32 particle kernel. Same control flow as particle_move(). */
#define KIN_BODY(T, FABS)                                                                                    \
    for (int i = 0; i < n; i++) {                                                                            \
        const om_particle *p = &in[i];                                                                       \
        T x = p->x, y = p->y, vx = p->vx, vy = p->vy;                                                        \
        ev[i] = 0;                                                                                           \
        sub[i] = -1;                                                                                         \
        if ((p->bits & P_TEMP) && p->lifetime <= 0) {                                                        \
            ev[i] = 2;                                                                                       \
            goto done_##T;                                                                                   \
        }                                                                                                    \
        if (x < 0 || (int)x >= w->W || y < 0 || (int)y >= w->H) {                                            \
            ev[i] = 1;                                                                                       \
            goto done_##T;                                                                                   \
        }                                                                                                    \
        {                                                                                                    \
            int lx = (int)x, ly = (int)y;                                                                    \
            vx += (T)p->ax;                                                                                  \
            vy += (T)p->ay;                                                                                  \
            int div = (int)((FABS(vx) + FABS(vy)) + 1);                                                      \
            T dvx = vx / div, dvy = vy / div;                                                                \
            for (int s = 0; s < div; s++) {                                                                  \
                x += dvx;                                                                                    \
                y += dvy;                                                                                    \
                if (x < 0 || (int)x >= w->W || y < 0 || (int)y >= w->H) {                                    \
                    ev[i] = 1;                                                                               \
                    sub[i] = s;                                                                              \
                    goto done_##T;                                                                           \
                }                                                                                            \
                int ct = M[w->id[(size_t)(int)y * w->W + (int)x]].type;                                      \
                if (!(p->bits & P_PHASE) && ct != T_AIR && ct != T_OBJECT) {                                 \
                    sub[i] = s;                                                                              \
                    if (p->bits & P_TEMP)                                                                    \
                        ev[i] = 2;                                                                           \
                    else                                                                                     \
                        ev[i] = (M[w->id[(size_t)ly * w->W + lx]].type != T_AIR) ? 4 : 3;                    \
                    goto done_##T;                                                                           \
                }                                                                                            \
            }                                                                                                \
        }                                                                                                    \
    done_##T:                                                                                                \
        out4[4 * i + 0] = x;                                                                                 \
        out4[4 * i + 1] = y;                                                                                 \
        out4[4 * i + 2] = vx;                                                                                \
        out4[4 * i + 3] = vy;                                                                                \
    }

void om_particles_kinematics_f64(const om_world *w, const om_particle *in, int n, double *out4, int32_t *ev,
                                 int32_t *sub) {
    KIN_BODY(double, fabs)
}
void om_particles_kinematics_f32(const om_world *w, const om_particle *in, int n, float *out4, int32_t *ev,
                                 int32_t *sub) {
    KIN_BODY(float, fabsf)
}

/* ------------------------------------------------------------- generators */
void om_world_generate(om_world *w, int kind, uint32_t seed) {
    int mats_mix[5] = {om_material_find("GENERIC_SAND"), om_material_find("WATER"), om_material_find("GENERIC_GAS"),
                       om_material_find("STONE"), ID_AIR};
    int mats_z[8] = {ID_AIR,
                     om_material_find("STONE"),
                     om_material_find("GENERIC_SAND"),
                     om_material_find("WATER"),
                     om_material_find("GENERIC_GAS"),
                     om_material_find("DIRT"),
                     om_material_find("GENERIC_LIQUID"),
                     om_material_find("SOFT_DIRT_SAND")};
    /* Zipf(s=1) weights 1/k over 8 ranks, scaled by 840 */
    const int zw[8] = {840, 420, 280, 210, 168, 140, 120, 105};
    uint32_t pk = pass_key(seed, 0, PH_GEN + (uint32_t)kind);
    int top = (w->H * 3) / 5;
    for (int y = 0; y < w->H; y++)
        for (int x = 0; x < w->W; x++) {
            uint32_t ck = cell_key(pk, (uint32_t)x, (uint32_t)y);
            uint32_t r = draw_k(ck, 0);
            int mid = ID_AIR;
            if (kind == 0) {
                if (y >= w->H - 8)
                    mid = mats_mix[3];
                else if (y < top) {
                    uint32_t u = r % 100u;
                    mid = u < 30 ? mats_mix[0] : u < 50 ? mats_mix[1] : u < 60 ? mats_mix[2] : u < 75 ? mats_mix[3] : ID_AIR;
                }
            } else if (kind == 1) {
                uint32_t u = r % 2283u, acc = 0;
                for (int k = 0; k < 8; k++) {
                    acc += (uint32_t)zw[k];
                    if (u < acc) {
                        mid = mats_z[k];
                        break;
                    }
                }
            }
            const mat_t *m = &M[mid];
            size_t i = (size_t)y * w->W + x;
            w->id[i] = (uint16_t)mid;
            w->fl[i] = 0;
            w->df[i] = 0;
            w->sc[i] = soup_scalar(w, w->id[i]);
            w->tp[i] = (m->type == T_SOUP) ? (int16_t)m->f_temp : 0;
            w->col[i] = m->f_base;
            if (m->f_mod > 0)
                w->col[i] = m->f_base + ((uint32_t)(m->f_lo + (int)(draw_k(ck, 1) % (uint32_t)m->f_mod)) << m->f_shift);
        }
    if (w->dirty) memset(w->dirty, 1, (size_t)w->W * w->H);
}

/* ------------------------------------------------------------- temperature */
/* The temperature of every cell as the reference keeps it in
 * MaterialInstance::temperature (i16, game_datastruct.hpp:109,213): SOUP cells
 * hold it beside their amount, every other cell in its scalar. */
static inline int16_t temp_at(const om_world *w, size_t i) {
    return M[w->id[i]].type == T_SOUP ? w->tp[i] : (int16_t)w->sc[i];
}
static inline void temp_put(om_world *w, size_t i, int16_t t) {
    if (M[w->id[i]].type == T_SOUP)
        w->tp[i] = t;
    else
        w->sc[i] = t;
}
void om_temperature_get(const om_world *w, int16_t *out) {
    size_t n = (size_t)w->W * w->H;
    for (size_t i = 0; i < n; i++) out[i] = temp_at(w, i);
}
void om_temperature_set(om_world *w, const int16_t *in) {
    size_t n = (size_t)w->W * w->H;
    for (size_t i = 0; i < n; i++) temp_put(w, i, in[i]);
}

/* float -> int32 the way x86-64's cvttss2si converts it (truncation toward zero;
 * NaN and values outside the int32 range give INT32_MIN): the conversion of
 * `newTemps[...] = <f32 expression>` (world.cpp:1989) on the reference's
 * targets. Written out because a plain C cast of an out-of-range float is
 * undefined and saturates on other CPUs. */
static inline int32_t f2i_x86(float r) {
    if (r >= -2147483648.0f && r < 2147483648.0f) return (int32_t)r;
    return INT32_MIN;
}

/* world::tickTemperature, world.cpp:1950-2004: a Jacobi step of the 3x3
 * conduction stencil over all cells (the reference's tickZone is the world
 * minus a 128-cell margin, so its stencil never leaves the world; here every
 * cell is updated and a neighbour outside the world reads Tiles_TEST_SOLID,
 * whose temperature 0 skips it, world.cpp:1970). Terms are taken in the order
 * of the FN(...) list, column by column, each operation rounded in float. */
void om_tick_temperature(om_world *w) {
    const int W = w->W, H = w->H;
    size_t n = (size_t)W * H;
    int16_t *old = (int16_t *)malloc(n * 2);
    for (size_t i = 0; i < n; i++) old[i] = temp_at(w, i);
    for (int y = 0; y < H; y++)
        for (int x = 0; x < W; x++) {
            float nn = (float)0.01; /* f32 n = 0.01; */
            float v = 0.0f;
            for (int xa = -1; xa <= 1; xa++)
                for (int ya = -1; ya <= 1; ya++) {
                    int xx = x + xa, yy = y + ya;
                    if (xx < 0 || yy < 0 || xx >= W || yy >= H) continue;
                    size_t j = (size_t)yy * W + xx;
                    int t = old[j];
                    if (t == 0) continue;
                    /* abs(temperature) / 64 is integer division, then * conductionOther */
                    float factor = (float)(abs(t) / 64) * M[w->id[j]].cond_other;
                    v += (float)t * factor;
                    nn += factor;
                }
            size_t i = (size_t)y * W + x;
            const mat_t *m = &M[w->id[i]];
            int t0 = old[i];
            int32_t r;
            if (v != 0.0f)
                r = f2i_x86((float)m->add_temp + v / nn * m->cond_self + (float)t0 * (1.0f - m->cond_self));
            else
                r = (int32_t)(m->add_temp + (uint32_t)t0); /* u32 + int, stored into i32 */
            /* world.cpp:1952-1953, 1996-2001: only the tick zone's cells change */
            if (in_zone(w, x, y)) temp_put(w, i, (int16_t)(uint16_t)(uint32_t)r);
        }
    free(old);
}

/* ------------------------------------------------------------ chunk .pack */
/* Chunk::ChunkWrite / ChunkRead (source/engine/chunk.cpp:219-330, 68-200) with the
 * record MaterialInstanceData {u32 index; u32 color; i16 temperature} (12 bytes
 * with 2 of padding, chunk.hpp:26-30): per 128 x 128 chunk, the i8 generation
 * phase, then src_size (int, 128*128*2*12), the LZ4 block size of the tile and
 * layer2 records, src_size2 (int, 128*128*4) and the LZ4 block size of the
 * background, then the two LZ4 blocks. This world has no second layer and no
 * background: layer2 records and background words are written as zeros
 * (GENERIC_AIR, colour 0, temperature 0) and skipped on reading.
 *
 * LZ4 block format (the vendored LZ4 1.9.4, source/libs/lz4, as its documented
 * block format): sequences of token (literal length << 4 | match length - 4),
 * optional 255-run length bytes, literals, a 16-bit little-endian offset,
 * optional match length bytes; the last sequence holds literals only, and the
 * last match starts at least 12 bytes before the end of the block.
 *
 * The encoder here is this project's own (the GPU kernels compute the same parse
 * with a warp per chunk): instead of a hash table of earlier positions it tries
 * 16 fixed distances matched to the 12-byte record and the 128-cell chunk row,
 * which on generated worlds gives smaller blocks than LZ4_compress_fast with the
 * acceleration 10 Chunk::ChunkWrite uses. Any LZ4 block decoder reads them. */
#define PK_EDGE 128
#define PK_CELLS (PK_EDGE * PK_EDGE)
#define PK_SRC1 (PK_CELLS * 2 * 12)
#define PK_SRC2 (PK_CELLS * 4)
#define PK_HEADER 17

int om_lz4_bound(int n) { return n + n / 255 + 16; }

static int pk_put_len(uint8_t *dst, int op, int cap, int v) { /* v >= 15 already taken out of the nibble */
    while (v >= 255) {
        if (op >= cap) return -1;
        dst[op++] = 255;
        v -= 255;
    }
    if (op >= cap) return -1;
    dst[op++] = (uint8_t)v;
    return op;
}

/* one sequence: literal records [ls, ls + nl) and, when ml > 0, a match of ml
 * bytes at distance off bytes */
static int pk_emit(uint8_t *dst, int op, int cap, const uint8_t *rec, int R, int ls, int nl, int off, int ml) {
    const int lb = nl * R;
    const int mcode = ml > 0 ? ml - 4 : 0;
    if (op >= cap) return -1;
    dst[op++] = (uint8_t)(((lb < 15 ? lb : 15) << 4) | (ml > 0 ? (mcode < 15 ? mcode : 15) : 0));
    if (lb >= 15 && (op = pk_put_len(dst, op, cap, lb - 15)) < 0) return -1;
    if (lb > cap - op) return -1;
    memcpy(dst + op, rec + (size_t)ls * R, (size_t)lb);
    op += lb;
    if (ml > 0) {
        if (cap - op < 2) return -1;
        dst[op++] = (uint8_t)(off & 255);
        dst[op++] = (uint8_t)(off >> 8);
        if (mcode >= 15 && (op = pk_put_len(dst, op, cap, mcode - 15)) < 0) return -1;
    }
    return op;
}

/* The candidate distances of the encoder, ascending (a tie goes to the nearer):
 * small multiples of 4 and of the 12-byte record, and the cells one chunk row
 * (128 records = 1536 bytes) and two rows above, with their diagonal neighbours. */
static const int PK_DIST[16] = {4, 8, 12, 16, 20, 24, 36, 48, 60, 72, 84, 96, 1524, 1536, 1548, 3072};

/* LZ4 block of buf[0, n): greedy from the first byte -- at position p, the
 * longest run buf[p + i] == buf[p + i - d] over the candidate distances d <= p
 * (ties to the smaller d) is taken as a match when it is at least 4 bytes long,
 * else p is a literal. A match starts at most n - 12 and ends at most n - 5 (the
 * block format's end conditions), and ends at the latest at the end of the
 * 24576-byte segment it starts in (segments are parsed in parallel on the GPU;
 * a match still refers to any earlier byte). Returns the block size, or -1 when
 * cap is too small. */
#define PK_SEG 24576
int om_lz4_encode(const uint8_t *buf, int n, uint8_t *dst, int cap) {
    const int mflimit = n - 12, mend = n - 5;
    int p = 0, anchor = 0, op = 0;
    while (p <= mflimit) {
        int best = 0, bd = 0;
        const int seg_end = (p / PK_SEG + 1) * PK_SEG;
        const int lim = mend < seg_end ? mend : seg_end;
        for (int k = 0; k < 16 && PK_DIST[k] <= p; k++) {
            const int d = PK_DIST[k];
            if (p + 4 > lim || memcmp(buf + p, buf + p - d, 4) != 0) continue;
            int L = 4;
            while (p + L + 8 <= lim) { /* 8 bytes at a time: the first differing byte */
                uint64_t x, y;
                memcpy(&x, buf + p + L, 8);
                memcpy(&y, buf + p + L - d, 8);
                if (x != y) break;
                L += 8;
            }
            while (p + L < lim && buf[p + L] == buf[p + L - d]) L++;
            if (L > best) {
                best = L;
                bd = d;
            }
        }
        if (best >= 4) {
            op = pk_emit(dst, op, cap, buf, 1, anchor, p - anchor, bd, best);
            if (op < 0) return -1;
            p += best;
            anchor = p;
        } else {
            p++;
        }
    }
    return pk_emit(dst, op, cap, buf, 1, anchor, n - anchor, 0, 0);
}

/* LZ4 block decoder; returns the decoded size, or a negative value for a block
 * that reads or writes out of bounds or refers before the start */
int om_lz4_decode(const uint8_t *src, int n, uint8_t *dst, int cap) {
    int ip = 0, op = 0;
    for (;;) {
        if (ip >= n) return -1;
        const int token = src[ip++];
        int ll = token >> 4;
        if (ll == 15) {
            int b;
            do {
                if (ip >= n) return -2;
                b = src[ip++];
                ll += b;
                if (ll > cap) return -3;
            } while (b == 255);
        }
        if (ll > n - ip || ll > cap - op) return -3;
        memcpy(dst + op, src + ip, (size_t)ll);
        ip += ll;
        op += ll;
        if (ip == n) return op; /* the last sequence: literals only */
        if (n - ip < 2) return -4;
        const int off = src[ip] | (src[ip + 1] << 8);
        ip += 2;
        if (off == 0 || off > op) return -5;
        int ml = token & 15;
        if (ml == 15) {
            int b;
            do {
                if (ip >= n) return -6;
                b = src[ip++];
                ml += b;
                if (ml > cap) return -7;
            } while (b == 255);
        }
        ml += 4;
        if (ml > cap - op) return -7;
        for (int k = 0; k < ml; k++) dst[op + k] = dst[op - off + k]; /* overlapping copies repeat the pattern */
        op += ml;
    }
}

/* the MaterialInstanceData buffer of chunk (cx, cy): tile records, then the
 * (zero) second layer; cells outside the world are GENERIC_AIR records */
static void pk_records(const om_world *w, int cx, int cy, uint8_t *rec) {
    memset(rec, 0, PK_SRC1);
    for (int j = 0; j < PK_CELLS; j++) {
        int x = cx * PK_EDGE + (j % PK_EDGE), y = cy * PK_EDGE + (j / PK_EDGE);
        if (x >= w->W || y >= w->H) continue;
        size_t i = (size_t)y * w->W + x;
        uint32_t id = w->id[i], col = w->col[i];
        int16_t t = temp_at(w, i);
        uint8_t *r = rec + (size_t)j * 12;
        memcpy(r, &id, 4);
        memcpy(r + 4, &col, 4);
        memcpy(r + 8, &t, 2);
    }
}

/* every chunk of the world, row-major, into out (offsets[k] = start of chunk k,
 * offsets[n] = total); returns the chunk count or -1 when cap is too small */
int om_world_pack(const om_world *w, int phase, uint8_t *out, int64_t cap, int64_t *offsets) {
    const int ncx = (w->W + PK_EDGE - 1) / PK_EDGE, ncy = (w->H + PK_EDGE - 1) / PK_EDGE;
    uint8_t *rec = (uint8_t *)malloc(PK_SRC1);
    uint8_t *bg = (uint8_t *)calloc(PK_SRC2, 1);
    uint8_t *c1 = (uint8_t *)malloc((size_t)om_lz4_bound(PK_SRC1));
    uint8_t *c2 = (uint8_t *)malloc((size_t)om_lz4_bound(PK_SRC2));
    int64_t op = 0;
    int rc = ncx * ncy;
    const int n2 = om_lz4_encode(bg, PK_SRC2, c2, om_lz4_bound(PK_SRC2));
    for (int k = 0; k < ncx * ncy && rc >= 0; k++) {
        pk_records(w, k % ncx, k / ncx, rec);
        const int n1 = om_lz4_encode(rec, PK_SRC1, c1, om_lz4_bound(PK_SRC1));
        offsets[k] = op;
        if (n1 < 0 || n2 < 0 || op + PK_HEADER + n1 + n2 > cap) {
            rc = -1;
            break;
        }
        const int8_t ph = (int8_t)phase;
        const int32_t hd[4] = {PK_SRC1, n1, PK_SRC2, n2};
        memcpy(out + op, &ph, 1);
        memcpy(out + op + 1, hd, 16);
        memcpy(out + op + PK_HEADER, c1, (size_t)n1);
        memcpy(out + op + PK_HEADER + n1, c2, (size_t)n2);
        op += PK_HEADER + n1 + n2;
    }
    if (rc >= 0) offsets[ncx * ncy] = op;
    free(rec);
    free(bg);
    free(c1);
    free(c2);
    return rc;
}

/* ChunkRead for every chunk: tiles take the records' material, colour and
 * temperature (a SOUP tile's amount is the MaterialInstance default 2.0,
 * game_datastruct.hpp:216); flags and pending diffs are cleared. phases[k] gets
 * each chunk's generation phase. Returns 0, or -1 - k for the first chunk k that
 * is malformed (bad header, sizes or block, or a material index out of range),
 * in which case no chunk from k on has been written. */
int om_world_unpack(om_world *w, const uint8_t *in, const int64_t *offsets, int n_chunks, int8_t *phases) {
    const int ncx = (w->W + PK_EDGE - 1) / PK_EDGE, ncy = (w->H + PK_EDGE - 1) / PK_EDGE;
    if (n_chunks != ncx * ncy) return -1;
    uint8_t *rec = (uint8_t *)malloc(PK_SRC1);
    uint8_t *bg = (uint8_t *)malloc(PK_SRC2);
    int rc = 0;
    for (int k = 0; k < n_chunks && rc == 0; k++) {
        const int64_t len = offsets[k + 1] - offsets[k];
        const uint8_t *p = in + offsets[k];
        int32_t hd[4];
        if (len < PK_HEADER) {
            rc = -1 - k;
            break;
        }
        memcpy(hd, p + 1, 16);
        if (hd[0] != PK_SRC1 || hd[2] != PK_SRC2 || hd[1] < 0 || hd[3] < 0 ||
            (int64_t)PK_HEADER + hd[1] + hd[3] > len ||
            om_lz4_decode(p + PK_HEADER, hd[1], rec, PK_SRC1) != PK_SRC1 ||
            om_lz4_decode(p + PK_HEADER + hd[1], hd[3], bg, PK_SRC2) != PK_SRC2) {
            rc = -1 - k;
            break;
        }
        for (int j = 0; j < PK_CELLS; j++) {
            uint32_t id;
            memcpy(&id, rec + (size_t)j * 12, 4);
            if (id >= (uint32_t)NMAT) rc = -1 - k;
        }
        if (rc) break;
        if (phases) phases[k] = (int8_t)p[0];
        const int cx = k % ncx, cy = k / ncx;
        for (int j = 0; j < PK_CELLS; j++) {
            int x = cx * PK_EDGE + (j % PK_EDGE), y = cy * PK_EDGE + (j / PK_EDGE);
            if (x >= w->W || y >= w->H) continue;
            size_t i = (size_t)y * w->W + x;
            const uint8_t *r = rec + (size_t)j * 12;
            uint32_t id, col;
            int16_t t;
            memcpy(&id, r, 4);
            memcpy(&col, r + 4, 4);
            memcpy(&t, r + 8, 2);
            w->id[i] = (uint16_t)id;
            w->col[i] = col;
            w->fl[i] = 0;
            w->df[i] = 0;
            if (M[id].type == T_SOUP) {
                w->sc[i] = w->f32 ? f2i(2.0f) : Q_DEFAULT;
                w->tp[i] = t;
            } else {
                w->sc[i] = t;
                w->tp[i] = 0;
            }
            mark_dirty(w, i);
        }
    }
    free(rec);
    free(bg);
    return rc;
}

/* --------------------------------------------------------------- rendering */
/* Headless textures of the game's per-tick update, 4 bytes (r, g, b, a) per cell.
 * om_render_enable allocates them with every cell dirty; from then on the tick,
 * particle deposits and bodies mark the cells they write, and soup flows add to
 * the per-cell flow sums (world.cpp:1334,1374,1402,1432). */
void om_render_enable(om_world *w) {
    size_t n = (size_t)w->W * w->H;
    if (w->dirty) return;
    w->dirty = (uint8_t *)malloc(n);
    memset(w->dirty, 1, n);
    w->flow = (int32_t *)calloc(2 * n, 4);
    for (int k = 0; k < 5; k++) w->tex[k] = (uint32_t *)calloc(n, 4);
    w->pflow = (float *)calloc(2 * n, 4);
}

static inline uint32_t rgba(uint32_t r, uint32_t g, uint32_t b, uint32_t a) {
    return (r & 0xff) | ((g & 0xff) << 8) | ((b & 0xff) << 16) | ((a & 0xff) << 24);
}

/* flow texture channel, game.cpp:2048-2053 (double arithmetic, truncation to u8) */
static inline uint32_t flow_byte(float f, int iterations) {
    double a = (double)f * (3.0 / iterations + 0.5) / 4.0 + 0.5;
    if (!(a > 0.0)) return 0u; /* also a NaN (zero iterations), which the reference leaves undefined */
    double c = a > 1.0 ? 1.0 : a;
    return (uint32_t)(c * 255);
}

/* the dirty-cell pass, game.cpp:1994-2067: moving[mat] counts the dirty cells */
void om_render_dirty(om_world *w, int64_t *moving) {
    if (!w->dirty) return;
    size_t n = (size_t)w->W * w->H;
    if (moving) memset(moving, 0, sizeof(int64_t) * NMAT);
    for (size_t i = 0; i < n; i++) {
        if (!w->dirty[i]) continue;
        w->dirty[i] = 0;
        const mat_t *m = &M[w->id[i]];
        if (moving) moving[w->id[i]]++;
        int32_t *fl = &w->flow[2 * i];
        if (m->type == T_AIR) {
            w->tex[0][i] = 0;
            w->tex[2][i] = 0;
            w->tex[1][i] = 0;
            fl[0] = fl[1] = 0;
            continue;
        }
        uint32_t col = w->col[i], emit = m->emit_colour;
        w->tex[0][i] = rgba(col >> 16, col >> 8, col, (uint32_t)m->alpha);
        w->tex[1][i] = rgba(emit >> 16, emit >> 8, emit, emit >> 24);
        if ((int)w->id[i] == ID_FIRE) w->tex[2][i] = rgba(col >> 16, col >> 8, col, (uint32_t)m->alpha);
        if (m->type == T_SOUP) {
            float *pf = &w->pflow[2 * i];
            /* the tick's flow sums: f32 in f32 worlds, else Q16.16 */
            float fx = w->f32 ? i2f(fl[0]) : (float)fl[0] * (1.0f / 65536.0f);
            float fy = w->f32 ? i2f(fl[1]) : (float)fl[1] * (1.0f / 65536.0f);
            /* f32 + (f32 - f32) * 0.25 evaluated in double, stored as f32 */
            float nfx = (float)((double)pf[0] + (double)(fx - pf[0]) * 0.25);
            float nfy = (float)((double)pf[1] + (double)(fy - pf[1]) * 0.25);
            if (nfy < 0) nfy = (float)((double)nfy * 0.5);
            w->tex[3][i] = rgba(flow_byte(nfx, m->iterations), flow_byte(nfy, m->iterations), 0, 0xff);
            pf[0] = nfx;
            pf[1] = nfy;
        }
        fl[0] = fl[1] = 0;
    }
}

/* the particle layer, world::renderCells (world.cpp:2006-2028) after the clear of
 * game.cpp:1881: particles in list order, a later one over an earlier one */
void om_render_cells(om_world *w) {
    if (!w->tex[4]) return;
    size_t n = (size_t)w->W * w->H;
    memset(w->tex[4], 0, n * 4);
    for (int k = 0; k < w->parts.n; k++) {
        const om_particle *p = &w->parts.p[k];
        if (!(p->x >= 0 && p->x < (float)w->W && p->y >= 0 && p->y < (float)w->H)) continue;
        float amod = 1.0f;
        if ((p->bits & 2) && p->lifetime < p->fade_time) amod = (float)p->lifetime / (float)p->fade_time;
        float a = (float)(uint8_t)M[p->id].alpha * amod; /* Material::alpha is a u8 */
        uint32_t ab = a > 0.0f ? (uint32_t)a : 0u; /* negative lifetimes draw transparent */
        size_t i = (size_t)(int)p->y * w->W + (int)p->x;
        w->tex[4][i] = rgba(p->colour >> 16, p->colour >> 8, p->colour, ab);
    }
}

/* which: 0 pixels, 1 emission, 2 fire, 3 flow, 4 particle layer */
void om_render_get(const om_world *w, int which, uint32_t *out) {
    if (which < 0 || which > 4 || !w->tex[which]) return;
    memcpy(out, w->tex[which], (size_t)w->W * w->H * 4);
}

/* set the dirty marks, the tick's flow sums (Q16.16 pairs) and the smoothed flows */
void om_render_set(om_world *w, const uint8_t *dirty, const int32_t *flow, const float *pflow) {
    if (!w->dirty) return;
    size_t n = (size_t)w->W * w->H;
    if (dirty) memcpy(w->dirty, dirty, n);
    if (flow) memcpy(w->flow, flow, 2 * n * sizeof(int32_t));
    if (pflow) memcpy(w->pflow, pflow, 2 * n * sizeof(float));
}
void om_render_pflow_get(const om_world *w, float *out) {
    if (w->pflow) memcpy(out, w->pflow, 2 * (size_t)w->W * w->H * sizeof(float));
}
void om_render_dirty_get(const om_world *w, uint8_t *out) {
    if (w->dirty) memcpy(out, w->dirty, (size_t)w->W * w->H);
}

/* ------------------------------------------------------------------ ledger */
void om_ledger_get(const om_world *w, int64_t *out) {
    for (int r = 0; r < 6; r++)
        for (int m = 0; m < NMAT; m++) out[r * NMAT + m] = w->led[r][m];
}
void om_ledger_reset(om_world *w) { memset(w->led, 0, sizeof(w->led)); }

void om_census(const om_world *w, int64_t *out) {
    memset(out, 0, sizeof(int64_t) * 4 * (size_t)NMAT);
    size_t n = (size_t)w->W * w->H;
    for (size_t i = 0; i < n; i++) {
        int id = w->id[i];
        out[id] += 1;
        if (M[id].type == T_SOUP && !w->f32) out[NMAT + id] += (int64_t)w->sc[i] + w->df[i];
    }
    for (int i = 0; i < w->parts.n; i++) {
        int id = w->parts.p[i].id;
        out[2 * NMAT + id] += 1;
        if (M[id].type == T_SOUP && !w->f32) out[3 * NMAT + id] += w->parts.p[i].scalar;
    }
}

/* ------------------------------------------------------------------ objects */
/* Rigid-body stamping before the tick, source/engine/game.cpp:1768-1814: every
 * body tile is rotated into the grid, trying offsets (0,0),(1,0),(-1,0),(0,1),
 * (0,-1); an AIR cell takes the tile; a SAND or SOUP cell is ejected as a particle
 * and damps the body. Tiles are resolved in rounds: each open tile picks its first
 * usable offset against the grid at the start of the round and the lowest
 * (body, tile) index wins a contested cell; the others look again. */
static const int DIRS[5][2] = {{0, 0}, {1, 0}, {-1, 0}, {0, 1}, {0, -1}};

static void body_tile_pos(const om_body *b, int tx, int ty, int *wx, int *wy) {
    float fx = (float)tx * b->cos_a - (float)(ty + 1) * b->sin_a + b->x;
    float fy = (float)tx * b->sin_a + (float)(ty + 1) * b->cos_a + b->y;
    *wx = (int)fx;
    *wy = (int)fy;
}

/* The stamp, game.cpp:1766-1813: bodies in order, tiles tx-major then ty-minor;
 * each tile takes the first of its five cells that is AIR, SAND or SOUP at that
 * moment (a cell it takes becomes the body's tile), displacing SAND and SOUP into a
 * particle (CellData(tile, wxd, wyd - 3, ...), velocities from the counter RNG
 * instead of rand()) and counting the displacement for the body's damping. */
void om_object_stamp(om_world *w, om_body *bodies, int n) {
    uint32_t pk = pass_key(w->seed, w->tick, PH_STAMP);
    for (int b = 0; b < n; b++) {
        om_body *bd = &bodies[b];
        bd->n_sand = bd->n_soup = bd->n_placed = 0;
        for (int t = 0; t < bd->w * bd->h; t++) {
            int wx, wy;
            body_tile_pos(bd, t / bd->h, t % bd->h, &wx, &wy);
            for (int d = 0; d < 5; d++) {
                int xd = wx + DIRS[d][0], yd = wy + DIRS[d][1];
                if (xd < 0 || yd < 0 || xd >= w->W || yd >= w->H) continue;
                size_t ci = (size_t)yd * w->W + xd;
                int ty = M[w->id[ci]].type;
                if (ty != T_AIR && ty != T_SAND && ty != T_SOUP) continue;
                if (ty == T_SAND || ty == T_SOUP) {
                    om_particle p;
                    memset(&p, 0, sizeof(p));
                    uint32_t ck = cell_key(pk, (uint32_t)b, (uint32_t)t);
                    p.x = (float)xd;
                    p.y = (float)(yd - 3);
                    p.vx = (float)((int)(draw_k(ck, 0) % 10) - 5) / 10.0f;
                    p.vy = (float)(-((int)(draw_k(ck, 1) % 5) + 5)) / 10.0f;
                    p.ay = 0.1f;
                    p.fade_time = 60;
                    p.id = w->id[ci];
                    p.colour = w->col[ci];
                    p.scalar = w->sc[ci];
                    if (ty == T_SOUP) p.temperature = w->tp[ci];
                    p.flags = w->fl[ci];
                    pv_push(&w->parts, &p);
                    if (ty == T_SOUP) {
                        /* the cell's pending diff leaves with it */
                        if (!w->f32) w->led[LED_DF][p.id] += w->df[ci];
                        bd->n_soup++;
                    } else
                        bd->n_sand++;
                }
                w->id[ci] = bd->id;
                w->col[ci] = bd->colour;
                w->sc[ci] = 0;
                w->fl[ci] = 0;
                w->df[ci] = 0;
                mark_dirty(w, ci);
                bd->n_placed++;
                w->led[LED_CN][bd->id] += 1;
                break;
            }
        }
    }
}

/* The readback after the tick, game.cpp:1907-1967: bodies and tiles in the same
 * order; each tile takes back the first of its five cells that holds the body's
 * material at that moment and erases it (Tiles_NOTHING). Returns the cells erased.
 * (The reference also drops a tile from the body when none is found and its own
 * cell is AIR; the body images stay with the caller here.) */
long om_object_readback(om_world *w, const om_body *bodies_c, int n) {
    om_body *bodies = (om_body *)bodies_c;
    long removed = 0;
    for (int b = 0; b < n; b++) {
        om_body *bd = &bodies[b];
        bd->n_recovered = 0;
        for (int t = 0; t < bd->w * bd->h; t++) {
            int wx, wy;
            body_tile_pos(bd, t / bd->h, t % bd->h, &wx, &wy);
            for (int d = 0; d < 5; d++) {
                int xd = wx + DIRS[d][0], yd = wy + DIRS[d][1];
                if (xd < 0 || yd < 0 || xd >= w->W || yd >= w->H) continue;
                size_t ci = (size_t)yd * w->W + xd;
                if (w->id[ci] != bd->id) continue;
                w->led[LED_DN][w->id[ci]] += 1;
                w->id[ci] = (uint16_t)ID_AIR;
                w->col[ci] = 0;
                w->sc[ci] = 0;
                w->fl[ci] = 0;
                w->df[ci] = 0;
                mark_dirty(w, ci);
                bd->n_recovered++;
                removed++;
                break;
            }
        }
    }
    return removed;
}

void om_object_mask(const om_world *w, uint8_t *bits) {
    size_t n = (size_t)w->W * w->H;
    memset(bits, 0, (n + 7) / 8);
    for (size_t i = 0; i < n; i++)
        if (M[w->id[i]].type == T_OBJECT) bits[i >> 3] |= (uint8_t)(1u << (i & 7));
}

/* ------------------------------------------------------------ solid islands */
static inline int is_solid(const om_world *w, size_t i) { return M[w->id[i]].type == T_SOLID; }

/* cut one cell out of the grid (Tiles_NOTHING, dirty), counted as destroyed */
static void cut_cell(om_world *w, size_t i) {
    w->led[LED_DN][w->id[i]] += 1;
    w->id[i] = (uint16_t)ID_AIR;
    w->col[i] = 0;
    w->sc[i] = 0;
    w->fl[i] = 0;
    w->df[i] = 0;
    mark_dirty(w, i);
}

/* world::physicsCheck(x, y), world.cpp:3330-3424, with the recursive 4-way flood
 * of :3427-3445 as an explicit stack in the same visiting order (+x, +y, -x, -y).
 * The flood stops counting past 1000 cells, and only a region of at most 1000
 * cells is cut out, so the result is the whole region or nothing. Returns the
 * number of cells cut; bbox = min x, min y, max x, max y; for more than 10 cells
 * `pixels` (if not NULL and big enough) gets the region's colours as a bbox-sized
 * image, 0 elsewhere (the rigid body's surface, :3357-3365). */
int om_physics_check(om_world *w, int x, int y, int32_t bbox[4], uint32_t *pixels, int pixels_cap) {
    if (x < 0 || y < 0 || x >= w->W || y >= w->H) return 0;
    if (!is_solid(w, (size_t)y * w->W + x)) return 0;
    size_t n = (size_t)w->W * w->H;
    uint8_t *vis = (uint8_t *)calloc(n, 1);
    int32_t *cells = (int32_t *)malloc(1001 * sizeof(int32_t));
    int32_t *stack = (int32_t *)malloc(4 * 1100 * sizeof(int32_t));
    int count = 0, sp = 0, minx = w->W, maxx = 0, miny = w->H, maxy = 0;
    stack[sp++] = y * w->W + x;
    while (sp > 0) {
        int c = stack[--sp];
        if (count > 1000) break; /* :3428 every further call returns */
        int cx = c % w->W, cy = c / w->W;
        if (vis[c] || !is_solid(w, (size_t)c)) continue;
        vis[c] = 1;
        if (count < 1001) cells[count] = c;
        count++;
        if (cx < minx) minx = cx;
        if (cx > maxx) maxx = cx;
        if (cy < miny) miny = cy;
        if (cy > maxy) maxy = cy;
        /* pushed in reverse so that +x is explored first */
        if (cy > 0 && sp < 4 * 1100) stack[sp++] = c - w->W;
        if (cx > 0 && sp < 4 * 1100) stack[sp++] = c - 1;
        if (cy + 1 < w->H && sp < 4 * 1100) stack[sp++] = c + w->W;
        if (cx + 1 < w->W && sp < 4 * 1100) stack[sp++] = c + 1;
    }
    int cut = 0;
    if (count > 0 && count <= 1000) {
        int bw = maxx - minx + 1, bh = maxy - miny + 1;
        if (count > 10 && pixels && bw * bh <= pixels_cap) {
            memset(pixels, 0, (size_t)bw * bh * 4);
            for (int k = 0; k < count; k++) {
                int c = cells[k];
                pixels[(c / w->W - miny) * bw + (c % w->W - minx)] = w->col[c];
            }
        }
        for (int k = 0; k < count; k++) cut_cell(w, (size_t)cells[k]);
        cut = count;
        bbox[0] = minx;
        bbox[1] = miny;
        bbox[2] = maxx;
        bbox[3] = maxy;
    }
    free(vis);
    free(cells);
    free(stack);
    return cut;
}

/* every 4-connected SOLID region: those of at most max_cells cells are listed in
 * `out` by increasing root (the region's smallest cell index) and, with `remove`,
 * cut out of the grid. Returns the number of such regions (entries beyond cap are
 * not written). */
int om_islands(om_world *w, int max_cells, int remove, om_island *out, int cap) {
    size_t n = (size_t)w->W * w->H;
    uint8_t *vis = (uint8_t *)calloc(n, 1);
    int32_t *q = (int32_t *)malloc(n * sizeof(int32_t));
    int found = 0;
    for (size_t r = 0; r < n; r++) {
        if (vis[r] || !is_solid(w, r)) continue;
        size_t head = 0, tail = 0;
        q[tail++] = (int32_t)r;
        vis[r] = 1;
        int minx = w->W, maxx = 0, miny = w->H, maxy = 0;
        while (head < tail) {
            int c = q[head++];
            int cx = c % w->W, cy = c / w->W;
            if (cx < minx) minx = cx;
            if (cx > maxx) maxx = cx;
            if (cy < miny) miny = cy;
            if (cy > maxy) maxy = cy;
            int nb[4] = {cx + 1 < w->W ? c + 1 : -1, cx > 0 ? c - 1 : -1, cy + 1 < w->H ? c + w->W : -1,
                         cy > 0 ? c - w->W : -1};
            for (int k = 0; k < 4; k++)
                if (nb[k] >= 0 && !vis[nb[k]] && is_solid(w, (size_t)nb[k])) {
                    vis[nb[k]] = 1;
                    q[tail++] = nb[k];
                }
        }
        if ((long)tail <= max_cells) {
            if (found < cap) {
                om_island *is = &out[found];
                is->root = (int32_t)r;
                is->cells = (int32_t)tail;
                is->min_x = minx;
                is->min_y = miny;
                is->max_x = maxx;
                is->max_y = maxy;
            }
            found++;
            if (remove)
                for (size_t k = 0; k < tail; k++) cut_cell(w, (size_t)q[k]);
        }
    }
    free(vis);
    free(q);
    return found;
}

void om_set_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

__attribute__((constructor)) static void om_init(void) {
    om_materials_reset_builtin();
    spiral_init();
}
