// fse_api.cu -- C ABI: material table, world lifecycle, the world::tick() /
// world::tickCells() launch sequences, CUDA-graph replay, particles, ledger.
#include <math.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <array>
#include <cstddef>
#include <cctype>
#include <atomic>
#include <mutex>
#include <string>
#include <vector>

#include <cuda.h>  // CUtensorMap and its encoder's types (the encoder comes from the driver at run time)

#include "fse_host.cuh"

using namespace fse;

// ================================================================ materials
namespace {

struct HostMat {
    std::string name, index_name;
    int type;
    float density;
    int iterations, slip, alpha;
    uint32_t colour;
    int emit;
    uint32_t emit_colour;
    uint32_t f_base;
    int f_shift, f_lo, f_mod;
    int32_t f_scalar;
    int32_t f_temp;  // factory temperature of SOUP tiles
    uint32_t add_temp;
    float cond_self, cond_other;
    int n_react;
    int react[4][3];
    int interact;
};

std::mutex g_mu;
std::vector<HostMat> g_mats;
std::vector<std::array<int, 7>> g_inter;
bool g_dirty = true;
MatTable g_host_mt;

int max_stability(int slip) {
    // world.cpp:1623 `int maxStability = 8 / sqrt(slipperyness) + 1;`
    if (slip <= 0) return 255;
    int v = (int)(8.0 / sqrt((double)slip) + 1.0);
    return v > 255 ? 255 : v;
}

int add_mat(const char *name, const char *index_name, int type, int slip, int alpha, float density, int iterations,
            int emit, uint32_t emit_colour, uint32_t colour) {
    if ((int)g_mats.size() >= MAXMAT) return -1;
    HostMat m{};
    m.name = name ? name : "";
    m.index_name = index_name ? index_name : "";
    m.type = type;
    m.density = density;
    m.iterations = iterations;
    m.slip = slip;
    m.alpha = alpha;
    m.colour = colour;
    m.emit = emit;
    m.emit_colour = emit_colour;
    m.f_base = colour;
    m.f_scalar = (type == T_SOUP) ? Q_DEFAULT : 0;
    m.cond_self = 1.0f;  // Material defaults, game_datastruct.hpp:142-144
    m.cond_other = 1.0f;
    g_mats.push_back(m);
    g_dirty = true;
    return (int)g_mats.size() - 1;
}

int find_mat(const char *index_name) {
    for (size_t i = 0; i < g_mats.size(); i++)
        if (g_mats[i].index_name == index_name) return (int)i;
    return -1;
}

void set_factory(int mid, uint32_t base, int shift, int lo, int mod, int32_t scalar) {
    if (mid < 0) return;
    HostMat &m = g_mats[mid];
    m.f_base = base;
    m.f_shift = shift;
    m.f_lo = lo;
    m.f_mod = mod;
    m.f_scalar = scalar;
    g_dirty = true;
}

int add_reaction(int mid, int kind, int temp, int res) {
    if (mid < 0 || mid >= (int)g_mats.size() || res < 0 || res >= (int)g_mats.size()) return FSE_E_INVAL;
    if (kind != REACT_BELOW && kind != REACT_ABOVE) return FSE_E_INVAL;
    HostMat &m = g_mats[mid];
    if (m.n_react >= 4) return FSE_E_INVAL;
    m.react[m.n_react][0] = kind;
    // MaterialInteraction::data1 is a mat_temperature (i16), game_datastruct.hpp:114
    m.react[m.n_react][1] = (int16_t)temp;
    m.react[m.n_react][2] = res;
    m.n_react++;
    g_dirty = true;
    return FSE_OK;
}

// InitMaterials, source/engine/game_datastruct.cpp:69-111 and :117-280, without
// the ten rand()-drawn Mat_i materials (never interactive, :196,206); texture
// colours are replaced by constants (data/assets is absent from the reference).
void builtin_materials() {
    g_mats.clear();
    g_inter.clear();
    const uint32_t W = 0xffffffffu;
    add_mat("_AIR", "GENERIC_AIR", T_AIR, 0, 255, 0, 0, 16, 0, W);
    add_mat("_SOLID", "GENERIC_SOLID", T_SOLID, 0, 255, 1, 0, 0, 0, W);
    add_mat("_SAND", "GENERIC_SAND", T_SAND, 20, 255, 10, 2, 0, 0, W);
    add_mat("_LIQUID", "GENERIC_LIQUID", T_SOUP, 0, 255, 1.5f, 3, 0, 0, W);
    add_mat("_GAS", "GENERIC_GAS", T_GAS, 0, 255, -1, 1, 0, 0, W);
    add_mat("_PASSABLE", "GENERIC_PASSABLE", T_OBJECT, 0, 255, 0, 0, 0, 0, W);
    add_mat("_OBJECT", "GENERIC_OBJECT", T_OBJECT, 0, 255, 1000.0f, 0, 0, 0, W);
    add_mat("Stone", "STONE", T_SOLID, 0, 255, 1, 0, 0, 0, W);
    add_mat("Grass", "GRASS", T_SAND, 20, 255, 12, 1, 0, 0, W);
    add_mat("Dirt", "DIRT", T_SAND, 8, 255, 15, 1, 0, 0, W);
    add_mat("Stone", "SMOOTH_STONE", T_SOLID, 0, 255, 1, 0, 0, 0, W);
    add_mat("Cobblestone", "COBBLE_STONE", T_SOLID, 0, 255, 1, 0, 0, 0, W);
    add_mat("Ground", "SMOOTH_DIRT", T_SOLID, 0, 255, 1, 0, 0, 0, W);
    add_mat("Hard Ground", "COBBLE_DIRT", T_SOLID, 0, 255, 1, 0, 0, 0, W);
    add_mat("Dirt", "SOFT_DIRT", T_SOLID, 0, 255, 15, 2, 0, 0, W);
    add_mat("Water", "WATER", T_SOUP, 0, 0x80, 1.5f, 6, 40, 0x3000AFB5u, W);
    add_mat("Lava", "LAVA", T_SOUP, 0, 0xC0, 2, 1, 40, 0xFFFF6900u, W);
    add_mat("Cloud", "CLOUD", T_SOLID, 0, 127, 1, 0, 0, 0, W);
    add_mat("Gold Ore", "GOLD_ORE", T_SAND, 20, 255, 20, 2, 8, 0x804000u, W);
    add_mat("Molten Gold", "GOLD_MOLTEN", T_SOUP, 0, 255, 20, 2, 8, 0x6FFF9B40u, W);
    add_mat("Solid Gold", "GOLD_SOLID", T_SOLID, 0, 255, 20, 2, 8, 0, W);
    add_mat("Iron Ore", "IRON_ORE", T_SAND, 20, 255, 20, 2, 8, 0x7F442Fu, W);
    add_mat("Obsidian", "OBSIDIAN", T_SOLID, 0, 255, 1, 0, 0, 0, W);
    add_mat("Steam", "STEAM", T_GAS, 0, 255, -1, 1, 0, 0, W);
    add_mat("Soft Dirt Sand", "SOFT_DIRT_SAND", T_SAND, 8, 255, 15, 2, 0, 0, W);
    add_mat("Fire", "FIRE", T_OBJECT, 0, 255, 20, 1, 0, 0, W);
    add_mat("Flat Cobblestone", "FLAT_COBBLE_STONE", T_SOLID, 0, 255, 1, 0, 0, 0, W);
    add_mat("Flat Hard Ground", "FLAT_COBBLE_DIRT", T_SOLID, 0, 255, 1, 0, 0, 0, W);
    add_mat("Test Sand", "TEST_SAND", T_SAND, 20, 255, 10, 2, 0, 0, W);
    add_mat("Test Textured Sand", "TEST_TEXTURED_SAND", T_SAND, 20, 255, 10, 2, 0, 0, W);
    add_mat("Test Liquid", "TEST_LIQUID", T_SOUP, 0, 255, 1.5f, 4, 0, 0, W);

    // tile factories, game_datastruct.cpp:320-574
    set_factory(find_mat("TEST_SAND"), (220u << 16) | 100u, 8, 155, 30, 0);
    set_factory(find_mat("TEST_TEXTURED_SAND"), 0xDC9B64u, 0, 0, 0, 0);
    set_factory(find_mat("TEST_LIQUID"), 0x0000FFu, 0, 0, 0, Q_DEFAULT);
    set_factory(find_mat("STONE"), 0x808080u, 0, 0, 0, 0);
    set_factory(find_mat("GRASS"), (40u << 16) | 20u, 8, 120, 20, 0);
    set_factory(find_mat("DIRT"), (40u << 8) | 20u, 16, 60, 10, 0);
    set_factory(find_mat("SMOOTH_STONE"), 0x9A9A9Au, 0, 0, 0, 0);
    set_factory(find_mat("COBBLE_STONE"), 0x707070u, 0, 0, 0, 0);
    set_factory(find_mat("SMOOTH_DIRT"), 0x6B4A2Fu, 0, 0, 0, 0);
    set_factory(find_mat("COBBLE_DIRT"), 0x5A3D25u, 0, 0, 0, 0);
    set_factory(find_mat("SOFT_DIRT"), 0x7A5533u, 0, 0, 0, 0);
    set_factory(find_mat("WATER"), 0x00B69Fu, 0, 0, 0, Q_DEFAULT);
    set_factory(find_mat("LAVA"), 0xFF7C00u, 0, 0, 0, Q_DEFAULT);
    set_factory(find_mat("CLOUD"), 0xE6E6F0u, 0, 0, 0, 0);
    set_factory(find_mat("GOLD_ORE"), 0xC8A032u, 0, 0, 0, 0);
    set_factory(find_mat("GOLD_MOLTEN"), 0xFFB43Cu, 0, 0, 0, Q_DEFAULT);
    set_factory(find_mat("GOLD_SOLID"), 0xE6C34Bu, 0, 0, 0, 0);
    set_factory(find_mat("IRON_ORE"), 0x8C6E5Au, 0, 0, 0, 0);
    set_factory(find_mat("OBSIDIAN"), 0x1E1428u, 0, 0, 0, 0);
    set_factory(find_mat("STEAM"), 0x666666u, 0, 0, 0, 0);
    set_factory(find_mat("FIRE"), (255u << 16) | 50u, 8, 100, 50, 0);
    set_factory(find_mat("FLAT_COBBLE_STONE"), 0x787878u, 0, 0, 0, 0);
    set_factory(find_mat("FLAT_COBBLE_DIRT"), 0x624530u, 0, 0, 0, 0);
    set_factory(find_mat("GENERIC_AIR"), 0x000000u, 0, 0, 0, 0);
    set_factory(find_mat("GENERIC_SOLID"), 0xff0000u, 0, 0, 0, 0);
    // SOUP factory temperatures, game_datastruct.cpp:427-437
    g_mats[find_mat("WATER")].f_temp = -1023;
    g_mats[find_mat("LAVA")].f_temp = 1024;
    // conduction, game_datastruct.cpp:124-141 (double literals rounded to float)
    auto cond = [](const char *nm, uint32_t add, double cs, double co) {
        HostMat &m = g_mats[find_mat(nm)];
        m.add_temp = add;
        m.cond_self = (float)cs;
        m.cond_other = (float)co;
    };
    cond("GENERIC_AIR", 0, 0.8, 0.8);
    cond("LAVA", 2, 0.5, 0.7);
    cond("COBBLE_STONE", 0, 0.01, 0.4);
    cond("COBBLE_DIRT", 0, 1.0, 1.0);
    cond("GOLD_ORE", 0, 1.0, 1.0);
    cond("GOLD_MOLTEN", 0, 1.0, 1.0);

    // reactions, game_datastruct.cpp:246-260
    add_reaction(find_mat("LAVA"), REACT_BELOW, 512, find_mat("OBSIDIAN"));
    add_reaction(find_mat("WATER"), REACT_ABOVE, 128, find_mat("STEAM"));
    add_reaction(find_mat("GOLD_ORE"), REACT_ABOVE, 512, find_mat("GOLD_MOLTEN"));
    add_reaction(find_mat("GOLD_MOLTEN"), REACT_BELOW, 128, find_mat("GOLD_SOLID"));
    g_dirty = true;
}

// The flow texel byte of game.cpp:2048-2053 for a float flow f and k = 3.0 /
// iterations + 0.5, in double; volatile temporaries keep each operation separately
// rounded (no contraction into a fused multiply-add).
static uint32_t flow_byte_host(float f, double k) {
    volatile double p = (double)f * k;
    volatile double q = p * 0.25;
    volatile double a = q + 0.5;
    if (!(a > 0.0)) return 0u;
    if (a >= 1.0) return 255u;
    volatile double b = a * 255.0;
    return (uint32_t)b;
}
// float <-> unsigned key with the same order (non-NaN values)
static uint32_t float_key(float f) {
    uint32_t u;
    memcpy(&u, &f, 4);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
static float key_float(uint32_t k) {
    uint32_t u = (k & 0x80000000u) ? (k & 0x7FFFFFFFu) : ~k;
    float f;
    memcpy(&f, &u, 4);
    return f;
}
// thr[j] = the smallest float with flow_byte_host >= j, j = 1..255 (thr[0] = -inf);
// the byte is non-decreasing in f when k > 0
static bool flow_thresholds(double k, float thr[256]) {
    if (!(k > 0.0) || !std::isfinite(k)) return false;
    const uint32_t lo0 = float_key(-INFINITY), hi0 = float_key(INFINITY);
    thr[0] = -INFINITY;
    for (int j = 1; j < 256; j++) {
        uint32_t lo = lo0, hi = hi0;  // invariant: byte(hi) >= j
        if (flow_byte_host(key_float(hi), k) < (uint32_t)j) {
            thr[j] = INFINITY;  // not reached by any finite float
            continue;
        }
        while (lo < hi) {
            const uint32_t mid = lo + (hi - lo) / 2;
            if (flow_byte_host(key_float(mid), k) >= (uint32_t)j)
                hi = mid;
            else
                lo = mid + 1;
        }
        thr[j] = key_float(lo);
    }
    return true;
}

void build_table(MatTable &t) {
    memset(&t, 0, sizeof(t));
    t.n = (int)g_mats.size();
    auto idx = [](const char *s, int def) {
        int v = find_mat(s);
        return v < 0 ? def : v;
    };
    t.id_air = idx("GENERIC_AIR", 0);
    t.id_solid = idx("GENERIC_SOLID", 1);
    t.id_fire = idx("FIRE", -1);
    t.id_water = idx("WATER", -1);
    t.id_lava = idx("LAVA", -1);
    t.id_steam = idx("STEAM", -1);
    t.id_obsidian = idx("OBSIDIAN", -1);
    for (int i = 0; i < t.n; i++) {
        const HostMat &m = g_mats[i];
        int iters = std::min(std::max(m.iterations, 0), 255);
        int slip = std::min(std::max(m.slip, 0), 255);
        t.a[i] = (uint32_t)m.type | ((uint32_t)iters << 8) | ((uint32_t)slip << 16) |
                 ((uint32_t)max_stability(m.slip) << 24);
        t.density[i] = m.density;
        t.f_base[i] = m.f_base;
        t.f_pack[i] = (uint32_t)(m.f_shift & 0xFF) | ((uint32_t)(m.f_lo & 0xFFF) << 8) | ((uint32_t)(m.f_mod & 0xFFF) << 20);
        t.f_scalar[i] = m.f_scalar;
        t.f_temp[i] = m.f_temp;
        t.add_temp[i] = m.add_temp;
        t.cond_self[i] = m.cond_self;
        t.cond_other[i] = m.cond_other;
        t.n_react[i] = m.n_react;
        for (int r = 0; r < m.n_react; r++)
            for (int k = 0; k < 3; k++) t.react[i][r][k] = m.react[r][k];
        t.alpha[i] = (uint32_t)(uint8_t)m.alpha;
        t.emit_col[i] = m.emit_colour;
        t.flow_k[i] = 3.0 / m.iterations + 0.5;  // IEEE double, as the reference evaluates it
        t.flow_thr_ok[i] = (m.type == T_SOUP && flow_thresholds(t.flow_k[i], t.flow_thr[i])) ? 1 : 0;
    }
    t.n_inter = (int)g_inter.size();
    for (size_t i = 0; i < g_inter.size(); i++)
        for (int k = 0; k < 7; k++) t.inter[i][k] = g_inter[i][k];
    t.has_inter = t.n_inter > 0 ? 1 : 0;
}

struct MatInit {
    MatInit() { builtin_materials(); }
} g_mat_init;

}  // namespace

namespace fse {
MatTable *g_dev_mt = nullptr;

int ensure_materials_pushed() {
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_dirty && g_dev_mt) return FSE_OK;
    build_table(g_host_mt);
    if (!g_dev_mt) {
        if (cudaMalloc(&g_dev_mt, sizeof(MatTable)) != cudaSuccess) {
            g_dev_mt = nullptr;
            return FSE_E_NOMEM;
        }
    } else {
        // the table may be read by work in flight
        cudaDeviceSynchronize();
    }
    if (cudaMemcpy(g_dev_mt, &g_host_mt, sizeof(MatTable), cudaMemcpyHostToDevice) != cudaSuccess) return FSE_E_CUDA;
    g_dirty = false;
    return FSE_OK;
}
const MatTable &host_table() {
    std::lock_guard<std::mutex> lk(g_mu);
    if (g_dirty) build_table(g_host_mt);
    return g_host_mt;
}

int sm_count() {
    static int n = 0;
    if (!n) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        if (n <= 0) n = 1;
    }
    return n;
}

int status_from_err(int err) {
    if (err & ERR_BOUNDS) return FSE_E_BOUNDS;
    if (err & ERR_TIMEOUT) return FSE_E_TIMEOUT;
    if (err & (ERR_SPAWN_CAP | ERR_PART_CAP)) return FSE_E_CAPACITY;
    return FSE_OK;
}

int tick_halo() {
    const MatTable &t = host_table();
    return t.has_inter ? 5 : 2;
}

static std::atomic<long long> g_launches{0};
void count_launches(long long n) { g_launches += n; }

cudaEvent_t PassTimer::get() {
    if (!pool.empty()) {
        cudaEvent_t e = pool.back();
        pool.pop_back();
        return e;
    }
    cudaEvent_t e;
    cudaEventCreate(&e);
    return e;
}
void PassTimer::drain() {
    for (auto &pr : pending) {
        float t = 0.f;
        if (cudaEventElapsedTime(&t, pr.first, pr.second) == cudaSuccess) {
            ms += t;
            launches++;
        }
        pool.push_back(pr.first);
        pool.push_back(pr.second);
    }
    pending.clear();
    for (auto &g : tick_groups) {
        for (size_t i = 0; i + 1 < g.size(); i++) {
            float t = 0.f;
            if (cudaEventElapsedTime(&t, g[i], g[i + 1]) == cudaSuccess) tick_ms.push_back(t);
        }
        for (cudaEvent_t e : g) pool.push_back(e);
    }
    tick_groups.clear();
}
void PassTimer::accumulate(const std::vector<std::pair<cudaEvent_t, cudaEvent_t>> &pairs,
                           const std::vector<cudaEvent_t> &ticks) {
    for (auto &pr : pairs) {
        float t = 0.f;
        if (cudaEventElapsedTime(&t, pr.first, pr.second) == cudaSuccess) {
            ms += t;
            launches++;
        }
    }
    for (size_t i = 0; i + 1 < ticks.size(); i++) {
        float t = 0.f;
        if (cudaEventElapsedTime(&t, ticks[i], ticks[i + 1]) == cudaSuccess) tick_ms.push_back(t);
    }
}

int enqueue_step(WorldDev *d_worlds, int n_worlds, uint32_t *const items[4], const int n_items[4], int max_iter, int C,
                 int threads, int grid, bool particles, int move_blocks, int stage_blocks, cudaStream_t s,
                 PassTimer *timer, int temp_tiles, bool temp_track, bool seq, bool f32) {
    int halo = tick_halo();
    const bool fused = grid == FUSED_GRID && !seq && threads == CP_THREADS;
    if (grid == FUSED_GRID && !fused) grid = 0;  // the reference's order runs pass by pass
    if (fused && max_iter > 0) {
        // the fused tick: one launch for every pass (world.cpp:1050-1060)
        cudaEvent_t a = nullptr, b = nullptr;
        if (timer) {
            a = timer->get();
            b = timer->get();
            if (timer->record(a, s) != cudaSuccess) return FSE_E_CUDA;
        }
        FusedTick ft;
        for (int tk = 0; tk < 4; tk++) {
            ft.items[tk] = items[tk];
            ft.n[tk] = n_items[tk];
        }
        ft.passes = 4 * max_iter;
        ft.n_worlds = n_worlds;
        // one CTA per SM, but no more than the chunks of an iteration: a CTA beyond them
        // would only set up its shared memory and find no chunk-pass it may start
        const int per_iter = n_items[0] + n_items[1] + n_items[2] + n_items[3];
        const int grid_f = std::max(1, std::min(sm_count(), per_iter));
        cudaError_t e = f32 ? launch_colour_fused_f32(d_worlds, ft, g_dev_mt, halo, C, grid_f, s, temp_track)
                            : launch_colour_fused(d_worlds, ft, g_dev_mt, halo, C, grid_f, s, temp_track);
        if (e != cudaSuccess) return FSE_E_CUDA;
        if (timer) {
            if (timer->record(b, s) != cudaSuccess) return FSE_E_CUDA;
            timer->record_pair(a, b);
        }
        count_launches(1);
    }
    for (int iter = 0; iter < max_iter && !fused; iter++)  // world.cpp:1050
        for (int tk = 0; tk < 4; tk++) {         // world.cpp:1057-1060
            cudaEvent_t a = nullptr, b = nullptr;
            if (timer) {
                a = timer->get();
                b = timer->get();
                if (timer->record(a, s) != cudaSuccess) return FSE_E_CUDA;
            }
            cudaError_t e = launch_colour_pass(d_worlds, items[tk], n_items[tk], iter, tk, g_dev_mt, halo, C, threads,
                                               grid, s, temp_track, seq, f32);
            if (e != cudaSuccess) return FSE_E_CUDA;
            if (timer) {
                if (timer->record(b, s) != cudaSuccess) return FSE_E_CUDA;
                timer->record_pair(a, b);
            }
            if (n_items[tk] > 0) count_launches(1);
        }
    if (launch_spawn_append(d_worlds, n_worlds, stage_blocks, s) != cudaSuccess) return FSE_E_CUDA;
    count_launches(3);
    if (particles) {
        if (launch_particle_tick(d_worlds, n_worlds, g_dev_mt, move_blocks, s) != cudaSuccess) return FSE_E_CUDA;
        count_launches(PARTICLE_TICK_LAUNCHES);
    }
    if (temp_tiles > 0) {  // game.cpp:2157-2159, decided per world on the device
        if (launch_temperature(d_worlds, n_worlds, temp_tiles, g_dev_mt, true, s) != cudaSuccess) return FSE_E_CUDA;
        count_launches(TEMPERATURE_LAUNCHES);
    }
    return FSE_OK;
}
}  // namespace fse

extern "C" {

const char *fse_version(void) { return "fse-gb300 0.1 (sm_103a)"; }

const char *fse_status_string(int s) {
    switch (s) {
        case FSE_OK: return "ok";
        case FSE_E_INVAL: return "invalid argument";
        case FSE_E_NOMEM: return "out of memory";
        case FSE_E_BUDGET: return "HBM budget exceeded";
        case FSE_E_CUDA: return "CUDA error";
        case FSE_E_TIMEOUT: return "device wait timed out";
        case FSE_E_CAPACITY: return "particle capacity exceeded";
        case FSE_E_STATE: return "invalid state";
        case FSE_E_BOUNDS: return "kernel bounds check fired";
        default: return "unknown status";
    }
}

int fse_materials_begin(void) {
    std::lock_guard<std::mutex> lk(g_mu);
    builtin_materials();
    return FSE_OK;
}

int fse_material_register(int s_id, const char *name, const char *index_name, int physics_type, int slipperyness,
                          int alpha, float density, int iterations, int emit, uint32_t emit_colour, uint32_t colour,
                          int *out_id) {
    (void)s_id;
    if (physics_type < 0 || physics_type > 5 || !index_name) return FSE_E_INVAL;
    if (slipperyness < 0 || slipperyness > 255 || iterations < 0 || iterations > 255) return FSE_E_INVAL;
    std::lock_guard<std::mutex> lk(g_mu);
    int id = add_mat(name, index_name, physics_type, slipperyness, alpha, density, iterations, emit, emit_colour, colour);
    if (id < 0) return FSE_E_INVAL;
    if (out_id) *out_id = id;
    return FSE_OK;
}

int fse_material_set_reaction(int mat, int kind, int temperature, int result_mat) {
    std::lock_guard<std::mutex> lk(g_mu);
    return add_reaction(mat, kind, temperature, result_mat);
}

int fse_material_set_interaction(int mat, int other, int kind, int data1_mat, int data2_radius, int ofs_x, int ofs_y) {
    std::lock_guard<std::mutex> lk(g_mu);
    int n = (int)g_mats.size();
    if (mat < 0 || mat >= n || other < 0 || other >= n || data1_mat < 0 || data1_mat >= n) return FSE_E_INVAL;
    if (kind != INTER_TRANSFORM && kind != INTER_SPAWN) return FSE_E_INVAL;
    // the shared-memory halo covers offsets with |ofs| + radius <= 5
    if (data2_radius < 0 || abs(ofs_x) + data2_radius > 5 || abs(ofs_y) + data2_radius > 5) return FSE_E_INVAL;
    int cnt = 0;
    for (auto &e : g_inter)
        if (e[0] == mat && e[1] == other) cnt++;
    if (cnt >= 4 || g_inter.size() >= 512) return FSE_E_INVAL;
    g_inter.push_back({mat, other, kind, data1_mat, data2_radius, ofs_x, ofs_y});
    g_mats[mat].interact = 1;
    g_dirty = true;
    return FSE_OK;
}

int fse_material_set_factory(int mat, uint32_t base, int shift, int lo, int mod, int32_t scalar) {
    std::lock_guard<std::mutex> lk(g_mu);
    if (mat < 0 || mat >= (int)g_mats.size() || shift < 0 || shift > 24 || lo < 0 || lo > 4095 || mod < 0 || mod > 4095)
        return FSE_E_INVAL;
    set_factory(mat, base, shift, lo, mod, scalar);
    return FSE_OK;
}

int fse_materials_push(void) { return ensure_materials_pushed(); }

int fse_material_count(void) {
    std::lock_guard<std::mutex> lk(g_mu);
    return (int)g_mats.size();
}

int fse_material_find(const char *index_name) {
    if (!index_name) return -1;
    std::lock_guard<std::mutex> lk(g_mu);
    return find_mat(index_name);
}

int fse_material_set_factory_temperature(int mat, int32_t temperature) {
    std::lock_guard<std::mutex> lk(g_mu);
    if (mat < 0 || mat >= (int)g_mats.size()) return FSE_E_INVAL;
    g_mats[mat].f_temp = temperature;
    g_dirty = true;
    return FSE_OK;
}

int fse_material_set_conduction(int mat, uint32_t add_temp, float conduction_self, float conduction_other) {
    std::lock_guard<std::mutex> lk(g_mu);
    if (mat < 0 || mat >= (int)g_mats.size()) return FSE_E_INVAL;
    HostMat &m = g_mats[mat];
    m.add_temp = add_temp;
    m.cond_self = conduction_self;
    m.cond_other = conduction_other;
    g_dirty = true;
    return FSE_OK;
}

int fse_material_get_conduction(int mat, uint32_t out[4]) {
    std::lock_guard<std::mutex> lk(g_mu);
    if (mat < 0 || mat >= (int)g_mats.size() || !out) return FSE_E_INVAL;
    const HostMat &m = g_mats[mat];
    out[0] = m.add_temp;
    memcpy(&out[1], &m.cond_self, 4);
    memcpy(&out[2], &m.cond_other, 4);
    out[3] = (uint32_t)m.f_temp;
    return FSE_OK;
}

int fse_material_get(int id, int32_t out[16]) {
    std::lock_guard<std::mutex> lk(g_mu);
    if (id < 0 || id >= (int)g_mats.size() || !out) return FSE_E_INVAL;
    const HostMat &m = g_mats[id];
    int32_t dbits;
    memcpy(&dbits, &m.density, 4);
    out[0] = m.type;
    out[1] = dbits;
    out[2] = m.iterations;
    out[3] = m.slip;
    out[4] = m.slip <= 0 ? (1 << 20) : (int)(8.0 / sqrt((double)m.slip) + 1.0);
    out[5] = m.alpha;
    out[6] = (int32_t)m.colour;
    out[7] = m.emit;
    out[8] = (int32_t)m.emit_colour;
    out[9] = (int32_t)m.f_base;
    out[10] = m.f_shift;
    out[11] = m.f_lo;
    out[12] = m.f_mod;
    out[13] = m.f_scalar;
    out[14] = m.n_react;
    out[15] = m.interact;
    return FSE_OK;
}

// ---- Lua subset: materials_init(), materials_register(...), materials_push()
// (the functions game_basic.cpp:79-81 exposes to data/scripts)
namespace {
struct LuaTok {
    const char *p;
    void ws() {
        for (;;) {
            while (*p && isspace((unsigned char)*p)) p++;
            if (p[0] == '-' && p[1] == '-') {
                if (p[2] == '[' && p[3] == '[') {
                    const char *e = strstr(p + 4, "]]");
                    p = e ? e + 2 : p + strlen(p);
                } else {
                    while (*p && *p != '\n') p++;
                }
                continue;
            }
            break;
        }
    }
    bool str(std::string &out) {
        ws();
        if (*p != '"' && *p != '\'') return false;
        char q = *p++;
        out.clear();
        while (*p && *p != q) {
            if (*p == '\\' && p[1]) p++;
            out.push_back(*p++);
        }
        if (*p != q) return false;
        p++;
        return true;
    }
    // number with optional unary minus and + - * / between terms
    bool num(double &v) {
        ws();
        if (!term(v)) return false;
        for (;;) {
            ws();
            char op = *p;
            if (op != '+' && op != '-' && op != '*' && op != '/') return true;
            p++;
            double r;
            if (!term(r)) return false;
            if (op == '+') v += r;
            else if (op == '-') v -= r;
            else if (op == '*') v *= r;
            else v /= r;
        }
    }
    bool term(double &v) {
        ws();
        bool neg = false;
        while (*p == '-') {
            neg = !neg;
            p++;
            ws();
        }
        char *e = nullptr;
        if (p[0] == '0' && (p[1] == 'x' || p[1] == 'X'))
            v = (double)strtoull(p, &e, 16);
        else
            v = strtod(p, &e);
        if (e == p) return false;
        p = e;
        if (neg) v = -v;
        return true;
    }
    bool ch(char c) {
        ws();
        if (*p != c) return false;
        p++;
        return true;
    }
};
}  // namespace

// the script without Lua comments (-- line, --[[ block ]]), string literals kept
static std::string strip_lua_comments(const char *s) {
    std::string out;
    for (const char *p = s; *p;) {
        if (*p == '"' || *p == '\'') {
            char q = *p;
            out.push_back(*p++);
            while (*p && *p != q) {
                if (*p == '\\' && p[1]) out.push_back(*p++);
                out.push_back(*p++);
            }
            if (*p) out.push_back(*p++);
        } else if (p[0] == '-' && p[1] == '-') {
            if (p[2] == '[' && p[3] == '[') {
                const char *e = strstr(p + 4, "]]");
                p = e ? e + 2 : p + strlen(p);
            } else {
                while (*p && *p != '\n') p++;
            }
            out.push_back(' ');
        } else {
            out.push_back(*p++);
        }
    }
    return out;
}

int fse_materials_load_lua(const char *script_in, int *out_count) {
    if (!script_in) return FSE_E_INVAL;
    const std::string stripped = strip_lua_comments(script_in);
    const char *script = stripped.c_str();
    int count = 0;
    const char *p = script;
    for (;;) {
        const char *reg = strstr(p, "materials_register");
        const char *ini = strstr(p, "materials_init");
        const char *next = reg;
        if (!next || (ini && ini < next)) next = ini;
        if (!next) break;
        if (next == ini) {
            fse_materials_begin();
            p = ini + 14;
            continue;
        }
        LuaTok t{reg + 18};
        if (!t.ch('(')) return FSE_E_INVAL;
        double sid, ptype, slip, alpha, dens, iters, emit, ecol, col;
        std::string name, iname;
        if (!t.num(sid) || !t.ch(',') || !t.str(name) || !t.ch(',') || !t.str(iname) || !t.ch(',') || !t.num(ptype) ||
            !t.ch(',') || !t.num(slip) || !t.ch(',') || !t.num(alpha) || !t.ch(',') || !t.num(dens) || !t.ch(',') ||
            !t.num(iters) || !t.ch(',') || !t.num(emit) || !t.ch(',') || !t.num(ecol) || !t.ch(',') || !t.num(col) ||
            !t.ch(')'))
            return FSE_E_INVAL;
        int id;
        int rc = fse_material_register((int)sid, name.c_str(), iname.c_str(), (int)ptype, (int)slip, (int)alpha,
                                       (float)dens, (int)iters, (int)emit, (uint32_t)(uint64_t)ecol,
                                       (uint32_t)(uint64_t)col, &id);
        if (rc != FSE_OK) return rc;
        count++;
        p = t.p;
    }
    if (out_count) *out_count = count;
    return FSE_OK;
}

}  // extern "C"

// ================================================================== worlds
static void free_world(fse_world *w) {
    for (auto &g : w->graphs) cudaGraphExecDestroy(g.second);
    w->graphs.clear();
    WorldDev &h = w->h;
    void *ptrs[] = {h.id, h.col, h.sc, h.fl, h.df, h.tp, h.tnew, h.stage, h.cp_count, h.cp_base, h.p_state, h.p_box0,
                    h.p_box1, h.p_cell, h.p_prev, h.chg, h.scan_tmp, h.ledger, h.airmap, w->ctr, w->d, w->claim,
                    w->mask_bits, w->obj_list, w->obj_n, h.merge_list, h.merge_count, h.merge_claim, h.cdone};
    for (void *q : ptrs)
        if (q) cudaFree(q);
    PartSoA *ps[2] = {&h.p, &h.q};
    for (PartSoA *p : ps) {
        void *a[] = {p->x, p->y, p->vx, p->vy, p->ax, p->ay, p->tx, p->ty, p->tf, p->life, p->fade, p->col, p->sc,
                     p->tp, p->id, p->fl, p->bits};
        for (void *q : a)
            if (q) cudaFree(q);
    }
    for (int k = 0; k < 4; k++)
        if (w->items[k]) cudaFree(w->items[k]);
    void *rs[] = {h.dirty,      h.flow,      w->pflow,    w->owner,    w->moving,   w->tex[0],   w->tex[1],
                  w->tex[2],    w->tex[3],   w->tex[4],   w->isl_mark, w->isl_lab,  w->isl_aux,  w->isl_list,
                  w->isl_out,   w->isl_pix,  w->isl_tab,  w->isl_seg,  w->temp_io, w->tile_stage,
                  w->tmaps};
    for (void *q : rs)
        if (q) cudaFree(q);
    for (void *q : w->pk_scr)
        if (q) cudaFree(q);
    if (w->own_stream && w->stream) cudaStreamDestroy(w->stream);
    if (w->timer) {
        w->timer->drain();
        for (cudaEvent_t e : w->timer->pool) cudaEventDestroy(e);
        delete w->timer;
    }
    delete w;
}

// cuTensorMapEncodeTiled, taken from the driver through the runtime (no link
// against the driver library); NULL when the driver does not offer it
typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                  const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
static EncodeTiledFn tensor_map_encoder() {
    static EncodeTiledFn fn = nullptr;
    static bool tried = false;
    if (!tried) {
        tried = true;
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<EncodeTiledFn>(p);
        cudaGetLastError();
    }
    return fn;
}

// The tensor maps of the colour pass's TMA staging (2-cell halo): the scalar and
// colour planes as W x H grids of 4-byte cells, boxes of tma_tile_width(C) x (C + 4)
// cells. A row pitch that is not a multiple of 16 bytes (W % 4 != 0), or no encoder,
// leaves h.tmap NULL and the tile is staged with cp.async.
static bool world_tensor_maps(fse_world *w) {
    WorldDev &h = w->h;
    h.tmap = nullptr;
    const int C = h.C, bw = tma_tile_width(C), bh = C + 4;
    EncodeTiledFn enc = tensor_map_encoder();
    if (!enc || h.W % 4 != 0 || bw > 256 || bh > 256) return true;
    CUtensorMap maps[2];
    const cuuint64_t dims[2] = {(cuuint64_t)h.W, (cuuint64_t)h.H};
    const cuuint64_t strides[1] = {(cuuint64_t)h.W * 4};
    const cuuint32_t box[2] = {(cuuint32_t)bw, (cuuint32_t)bh};
    const cuuint32_t es[2] = {1, 1};
    void *planes[2] = {h.sc, h.col};
    for (int k = 0; k < 2; k++)
        if (enc(&maps[k], k == 0 ? CU_TENSOR_MAP_DATA_TYPE_INT32 : CU_TENSOR_MAP_DATA_TYPE_UINT32, 2, planes[k], dims,
                strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
            return true;  // not encodable: cp.async staging
    if (cudaMalloc(&w->tmaps, sizeof(maps)) != cudaSuccess) {
        cudaGetLastError();
        w->tmaps = nullptr;
        return false;
    }
    w->bytes += sizeof(maps);
    if (cudaMemcpy(w->tmaps, maps, sizeof(maps), cudaMemcpyHostToDevice) != cudaSuccess) return false;
    h.tmap = w->tmaps;
    return true;
}

// the chunk slots of each colour for the current tick zone
static int world_items(fse_world *w) {
    const WorldDev &h = w->h;
    for (int tk = 0; tk < 4; tk++) {
        int ox = tk % 2, oy = 1 - tk / 2;
        int na = (h.nCx - ox + 1) / 2, nb = (h.nCy - oy + 1) / 2;
        int ns = std::max(0, na) * std::max(0, nb);
        w->n_items[tk] = ns;
        std::vector<uint32_t> v(ns);
        for (int s = 0; s < ns; s++) v[s] = (uint32_t)s;
        if (ns && cudaMemcpy(w->items[tk], v.data(), ns * 4, cudaMemcpyHostToDevice) != cudaSuccess)
            return FSE_E_CUDA;
    }
    return FSE_OK;
}

template <class T>
static bool dalloc(fse_world *w, T **p, size_t n) {
    size_t b = n * sizeof(T);
    if (b == 0) b = sizeof(T);
    if (cudaMalloc((void **)p, b) != cudaSuccess) {
        *p = nullptr;
        cudaGetLastError();
        return false;
    }
    w->bytes += b;
    return true;
}

extern "C" {

int fse_world_create(int width, int height, const fse_config *cfg, fse_world **out) {
    if (!out || width <= 0 || height <= 0 || (long long)width * height > (1LL << 31) - 1) return FSE_E_INVAL;
    fse_config c{};
    if (cfg) c = *cfg;
    if (c.chunk_size == 0) c.chunk_size = 128;
    if (c.cell_iter == 0) c.cell_iter = 3;
    if (c.chunk_size < 16 || c.chunk_size > 128 || c.cell_iter < 0 || c.cell_iter > 64) return FSE_E_INVAL;
    long long ncell = (long long)width * height;
    if (c.particle_capacity <= 0) c.particle_capacity = (int)std::max<long long>(65536, ncell / 4);
    if (c.spawn_capacity <= 0) c.spawn_capacity = c.particle_capacity;
    int rc = ensure_materials_pushed();
    if (rc != FSE_OK) return rc;
    particle_prepare();

    fse_world *w = new fse_world();
    memset(&w->h, 0, sizeof(w->h));
    w->W = width;
    w->H = height;
    w->C = c.chunk_size;
    w->cell_iter = c.cell_iter;
    w->seq = (c.flags & FSE_CFG_REFERENCE_ORDER) != 0;
    w->seed = c.seed;
    w->part_cap = c.particle_capacity;
    w->stage_cap = c.spawn_capacity;
    // the fused tick (launch shape 4) by default; worlds in the reference's order
    // run their passes one launch each whatever the shape
    colour_shape(4, &w->threads, &w->grid);
    w->timer = nullptr;
    if (c.stream) {
        w->stream = (cudaStream_t)c.stream;
        w->own_stream = false;
    } else {
        if (cudaStreamCreateWithFlags(&w->stream, cudaStreamNonBlocking) != cudaSuccess) {
            delete w;
            return FSE_E_CUDA;
        }
        w->own_stream = true;
    }
    WorldDev &h = w->h;
    h.W = width;
    h.H = height;
    h.C = c.chunk_size;
    h.cell_iter = c.cell_iter;
    h.seed = c.seed;
    h.nCx = ceil_div(width, h.C);
    h.nCy = ceil_div(height, h.C);
    h.max_slots = ceil_div(h.nCx, 2) * ceil_div(h.nCy, 2);
    h.zx = 0;  // the tick zone: the whole world until fse_world_set_tick_zone
    h.zy = 0;
    h.zw = width;
    h.zh = height;
    h.stage_cap = c.spawn_capacity;
    h.part_cap = c.particle_capacity;
    h.amw = ceil_div(width, 8);
    h.amh = ceil_div(height, 8);
    size_t n = (size_t)ncell;
    h.cp_rows = (c.flags & FSE_CFG_REFERENCE_ORDER) ? h.C : 1;
    int ncp = h.cell_iter * 4 * h.max_slots * h.cp_rows + 1;
    bool ok = dalloc(w, &h.id, n) && dalloc(w, &h.col, n) && dalloc(w, &h.sc, n) && dalloc(w, &h.fl, n) &&
              dalloc(w, &h.df, n) && dalloc(w, &h.stage, (size_t)h.stage_cap) && dalloc(w, &h.cp_count, ncp) &&
              dalloc(w, &h.cp_base, ncp) && dalloc(w, &w->ctr, 24) && dalloc(w, &h.ledger, LED_ROWS * MAXMAT) &&
              dalloc(w, &h.p_state, (size_t)h.part_cap) && dalloc(w, &h.p_box0, (size_t)h.part_cap) &&
              dalloc(w, &h.p_box1, (size_t)h.part_cap) && dalloc(w, &h.p_cell, (size_t)h.part_cap) &&
              dalloc(w, &h.p_prev, (size_t)h.part_cap) && dalloc(w, &h.scan_tmp, particle_scan_blocks() + 1) &&
              dalloc(w, &h.airmap, (size_t)h.amw * h.amh) && dalloc(w, &h.chg, 2 * (size_t)h.amw * h.amh) &&
              dalloc(w, &h.merge_list, 2 * (size_t)h.part_cap) && dalloc(w, &h.merge_count, 1) &&
              dalloc(w, &h.cdone, (size_t)h.nCx * h.nCy) && dalloc(w, &w->d, 1);
    PartSoA *ps[2] = {&h.p, &h.q};
    size_t pc = (size_t)h.part_cap;
    for (int k = 0; k < 2 && ok; k++) {
        PartSoA *p = ps[k];
        ok = dalloc(w, &p->x, pc) && dalloc(w, &p->y, pc) && dalloc(w, &p->vx, pc) && dalloc(w, &p->vy, pc) &&
             dalloc(w, &p->ax, pc) && dalloc(w, &p->ay, pc) && dalloc(w, &p->tx, pc) && dalloc(w, &p->ty, pc) &&
             dalloc(w, &p->tf, pc) && dalloc(w, &p->life, pc) && dalloc(w, &p->fade, pc) && dalloc(w, &p->col, pc) &&
             dalloc(w, &p->sc, pc) && dalloc(w, &p->id, pc) && dalloc(w, &p->fl, pc) && dalloc(w, &p->bits, pc);
    }
    if (ok && (c.flags & (FSE_CFG_TEMPERATURE | FSE_CFG_TEMPERATURE_STEP))) {  // liquid temperatures
        ok = dalloc(w, &h.tp, n) && dalloc(w, &h.p.tp, pc) && dalloc(w, &h.q.tp, pc);
        if (ok) cudaMemset(h.tp, 0, n * 2);
    }
    if (ok && (c.flags & FSE_CFG_TEMPERATURE_STEP)) {  // and the conduction step inside every step
        h.temp_on = 1;
        ok = dalloc(w, &h.tnew, temperature_scratch_cells(width, height));
    }
    if (ok && (c.flags & FSE_CFG_F32_FLUID)) {  // f32 amounts, deposits into liquid merged in index order
        h.f32 = 1;
        ok = dalloc(w, &h.merge_claim, n);
        if (ok) cudaMemset(h.merge_claim, 0xFF, n * sizeof(uint32_t));
    }
    if (ok && (c.flags & FSE_CFG_RENDER)) {
        ok = dalloc(w, &h.dirty, n) && dalloc(w, &h.flow, 2 * n) && dalloc(w, &w->pflow, 2 * n) &&
             dalloc(w, &w->owner, n) && dalloc(w, &w->moving, (size_t)MAXMAT);
        for (int k = 0; k < 5 && ok; k++) ok = dalloc(w, &w->tex[k], n);
        if (ok) {
            cudaMemset(h.dirty, 1, n);  // the first dirty pass paints every cell
            cudaMemset(h.flow, 0, 2 * n * sizeof(int32_t));
            cudaMemset(w->pflow, 0, 2 * n * sizeof(float));
            for (int k = 0; k < 5; k++) cudaMemset(w->tex[k], 0, n * sizeof(uint32_t));
        }
    }
    // chunk slots per colour: (world 0 << 20) | slot; room for the whole world's
    for (int tk = 0; tk < 4 && ok; tk++) ok = dalloc(w, &w->items[tk], (size_t)std::max(h.max_slots, 1));
    if (ok) ok = world_items(w) == FSE_OK;
    if (ok) ok = world_tensor_maps(w);
    if (!ok) {
        free_world(w);
        return FSE_E_NOMEM;
    }
    h.stage_count = w->ctr + 0;
    h.part_count = w->ctr + 1;
    h.req_count = w->ctr + 2;  // [3]
    h.err = w->ctr + 5;
    h.tick = (uint32_t *)(w->ctr + 6);
    h.bar = (unsigned *)(w->ctr + 8);  // [8] arrivals, [9] generation
    h.stats = w->ctr + 10;             // [10] iterations of the last particle update
    h.sched = (uint32_t *)(w->ctr + 12);  // [12] next ticket, [13] CTAs finished, [14] a wait gave up (fused tick)
    h.chg_n = w->ctr + 16;  // [16..17] fill changes per iteration parity, [18..19] their lowest index (particle update)
    cudaMemset(w->ctr, 0, 24 * sizeof(int32_t));
    cudaMemset(h.cdone, 0, (size_t)h.nCx * h.nCy * sizeof(uint32_t));
    cudaMemset(h.ledger, 0, LED_ROWS * MAXMAT * sizeof(long long));
    cudaMemset(h.cp_count, 0, ncp * sizeof(int32_t));
    cudaMemset(h.merge_count, 0, sizeof(int32_t));
    // an empty world: GENERIC_AIR everywhere (world.cpp:133-145)
    cudaMemset(h.id, 0, n * 2);
    cudaMemset(h.col, 0, n * 4);
    cudaMemset(h.sc, 0, n * 4);
    cudaMemset(h.fl, 0, n);
    cudaMemset(h.df, 0, n * 4);
    if (cudaMemcpy(w->d, &h, sizeof(WorldDev), cudaMemcpyHostToDevice) != cudaSuccess) {
        free_world(w);
        return FSE_E_CUDA;
    }
    if (cudaDeviceSynchronize() != cudaSuccess) {
        free_world(w);
        return FSE_E_CUDA;
    }
    *out = w;
    return FSE_OK;
}

int fse_world_destroy(fse_world *w) {
    if (!w) return FSE_E_INVAL;
    cudaStreamSynchronize(w->stream);
    free_world(w);
    return FSE_OK;
}

static int read_ctr(fse_world *w, int32_t *out16) {
    FSE_CUDA_TRY(cudaMemcpyAsync(out16, w->ctr, 16 * sizeof(int32_t), cudaMemcpyDeviceToHost, w->stream));
    FSE_CUDA_TRY(cudaStreamSynchronize(w->stream));
    return FSE_OK;
}

static uint32_t read_tick(fse_world *w) {
    uint32_t t = 0;
    cudaMemcpyAsync(&t, w->h.tick, 4, cudaMemcpyDeviceToHost, w->stream);
    cudaStreamSynchronize(w->stream);
    return t;
}

int fse_world_particle_iterations(fse_world *w, int *out) {
    if (!w || !out) return FSE_E_INVAL;
    int32_t c[16];
    int rc = read_ctr(w, c);
    if (rc) return rc;
    *out = c[10];
    return FSE_OK;
}

int fse_world_info(const fse_world *wc, int32_t out[8]) {
    fse_world *w = (fse_world *)wc;
    if (!w || !out) return FSE_E_INVAL;
    int32_t c[16];
    int rc = read_ctr(w, c);
    if (rc) return rc;
    out[0] = w->W;
    out[1] = w->H;
    out[2] = w->C;
    out[3] = w->cell_iter;
    out[4] = (int32_t)w->seed;
    out[5] = (int32_t)read_tick(w);
    out[6] = c[1];
    out[7] = c[5];
    return FSE_OK;
}

int fse_world_set_tick(fse_world *w, uint32_t tick) {
    if (!w) return FSE_E_INVAL;
    FSE_CUDA_TRY(cudaMemcpyAsync(w->h.tick, &tick, 4, cudaMemcpyHostToDevice, w->stream));
    FSE_CUDA_TRY(cudaStreamSynchronize(w->stream));
    return FSE_OK;
}

int fse_world_set_launch(fse_world *w, int colour_shape_id) {
    if (!w || colour_shape_id < 0 || colour_shape_id >= COLOUR_SHAPES) return FSE_E_INVAL;
    FSE_CUDA_TRY(cudaStreamSynchronize(w->stream));
    colour_shape(colour_shape_id, &w->threads, &w->grid);
    for (auto &g : w->graphs) cudaGraphExecDestroy(g.second);
    w->graphs.clear();
    w->graph_kernels.clear();
    return FSE_OK;
}

int fse_world_set_tick_zone(fse_world *w, int x, int y, int width, int height) {
    if (!w || x < 0 || y < 0 || width < 0 || height < 0 || (long long)x + width > w->W ||
        (long long)y + height > w->H)
        return FSE_E_INVAL;
    FSE_CUDA_TRY(cudaStreamSynchronize(w->stream));
    WorldDev &h = w->h;
    h.zx = x;
    h.zy = y;
    h.zw = width;
    h.zh = height;
    h.nCx = ceil_div(width, h.C);
    h.nCy = ceil_div(height, h.C);
    int rc = world_items(w);
    if (rc) return rc;
    // the colour passes write the spawn counts of the zone's chunk slots only, and the
    // spawn scan sums every slot: counts left by a larger zone must go
    const size_t ncp = (size_t)h.cell_iter * 4 * h.max_slots * h.cp_rows + 1;
    FSE_CUDA_TRY(cudaMemset(h.cp_count, 0, ncp * sizeof(int32_t)));
    FSE_CUDA_TRY(cudaMemcpy(w->d, &h, sizeof(WorldDev), cudaMemcpyHostToDevice));
    // captured step graphs hold the old chunk counts
    for (auto &g : w->graphs) cudaGraphExecDestroy(g.second);
    w->graphs.clear();
    w->graph_kernels.clear();
    return FSE_OK;
}

__global__ void k_mask_flags(uint8_t *fl, size_t n) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        fl[i] &= (uint8_t)~VISITED;
}

// uploaded material ids must index the table: out-of-range ids become GENERIC_AIR
// and the upload reports FSE_E_INVAL (*bad |= 1)
__global__ void k_check_ids(uint16_t *id, size_t n, int nmat, int air, int *bad) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        if (id[i] >= nmat) {
            id[i] = (uint16_t)air;
            atomicOr(bad, 1);
        }
}

}  // extern "C"

namespace fse {

// the copies and checks of an upload, enqueued on s; out-of-range ids set *bad
int world_upload_async(fse_world *w, const uint16_t *id, const uint32_t *col, const int32_t *sc, const uint8_t *fl,
                       const int32_t *df, cudaStream_t s, int *bad) {
    size_t n = (size_t)w->W * w->H;
    const MatTable &t = host_table();
    if (id) FSE_CUDA_TRY(cudaMemcpyAsync(w->h.id, id, n * 2, cudaMemcpyHostToDevice, s));
    if (col) FSE_CUDA_TRY(cudaMemcpyAsync(w->h.col, col, n * 4, cudaMemcpyHostToDevice, s));
    if (sc) FSE_CUDA_TRY(cudaMemcpyAsync(w->h.sc, sc, n * 4, cudaMemcpyHostToDevice, s));
    if (fl) {
        FSE_CUDA_TRY(cudaMemcpyAsync(w->h.fl, fl, n, cudaMemcpyHostToDevice, s));
        // bit 6 of the flags is reserved for the kernel's visited mark
        k_mask_flags<<<std::max(1, std::min<int>((int)(n / 1024) + 1, 4096)), 256, 0, s>>>(w->h.fl, n);
    }
    if (df) FSE_CUDA_TRY(cudaMemcpyAsync(w->h.df, df, n * 4, cudaMemcpyHostToDevice, s));
    if (id) {
        int blocks = (int)std::min<size_t>((n + 255) / 256, (size_t)sm_count() * 8);
        k_check_ids<<<std::max(blocks, 1), 256, 0, s>>>(w->h.id, n, t.n, t.id_air, bad);
    }
    if (w->h.dirty) FSE_CUDA_TRY(cudaMemsetAsync(w->h.dirty, 1, n, s));  // repaint everything
    return cudaGetLastError() == cudaSuccess ? FSE_OK : FSE_E_CUDA;
}

int world_download_async(fse_world *w, uint16_t *id, uint32_t *col, int32_t *sc, uint8_t *fl, int32_t *df,
                         cudaStream_t s) {
    size_t n = (size_t)w->W * w->H;
    if (id) FSE_CUDA_TRY(cudaMemcpyAsync(id, w->h.id, n * 2, cudaMemcpyDeviceToHost, s));
    if (col) FSE_CUDA_TRY(cudaMemcpyAsync(col, w->h.col, n * 4, cudaMemcpyDeviceToHost, s));
    if (sc) FSE_CUDA_TRY(cudaMemcpyAsync(sc, w->h.sc, n * 4, cudaMemcpyDeviceToHost, s));
    if (fl) FSE_CUDA_TRY(cudaMemcpyAsync(fl, w->h.fl, n, cudaMemcpyDeviceToHost, s));
    if (df) FSE_CUDA_TRY(cudaMemcpyAsync(df, w->h.df, n * 4, cudaMemcpyDeviceToHost, s));
    return FSE_OK;
}

}  // namespace fse

extern "C" {

int fse_world_upload(fse_world *w, const uint16_t *id, const uint32_t *col, const int32_t *sc, const uint8_t *fl,
                     const int32_t *df) {
    if (!w) return FSE_E_INVAL;
    int bad = 0;
    FSE_CUDA_TRY(cudaMemsetAsync(w->ctr + 7, 0, 4, w->stream));
    int rc = world_upload_async(w, id, col, sc, fl, df, w->stream, w->ctr + 7);
    if (rc) return rc;
    if (id) FSE_CUDA_TRY(cudaMemcpyAsync(&bad, w->ctr + 7, 4, cudaMemcpyDeviceToHost, w->stream));
    FSE_CUDA_TRY(cudaStreamSynchronize(w->stream));
    return bad ? FSE_E_INVAL : FSE_OK;
}

int fse_world_download(fse_world *w, uint16_t *id, uint32_t *col, int32_t *sc, uint8_t *fl, int32_t *df) {
    if (!w) return FSE_E_INVAL;
    int rc = world_download_async(w, id, col, sc, fl, df, w->stream);
    if (rc) return rc;
    FSE_CUDA_TRY(cudaStreamSynchronize(w->stream));
    return FSE_OK;
}

// synthetic worlds; the same draw as the oracle's om_world_generate
__global__ void k_generate(WorldDev *wd, int kind, uint32_t seed, const MatTable *__restrict__ mt, int m_sand,
                           int m_water, int m_gas, int m_stone, int z0, int z1, int z2, int z3, int z4, int z5, int z6,
                           int z7) {
    const WorldDev &w = *wd;
    const size_t n = (size_t)w.W * w.H;
    const uint32_t pk = pass_key(seed, 0, PH_GEN + (uint32_t)(kind == FSE_GEN_ZIPF8 ? 1 : (kind == FSE_GEN_MIX ? 0 : 2)));
    const int top = (w.H * 3) / 5;
    const int zm[8] = {z0, z1, z2, z3, z4, z5, z6, z7};
    const int zw[8] = {840, 420, 280, 210, 168, 140, 120, 105};
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        int y = (int)(i / w.W), x = (int)(i % w.W);
        uint32_t ck = cell_key(pk, (uint32_t)x, (uint32_t)y);
        uint32_t r = draw_k(ck, 0);
        int mid = mt->id_air;
        if (kind == FSE_GEN_MIX) {
            if (y >= w.H - 8)
                mid = m_stone;
            else if (y < top) {
                uint32_t u = r % 100u;
                mid = u < 30 ? m_sand : u < 50 ? m_water : u < 60 ? m_gas : u < 75 ? m_stone : mt->id_air;
            }
        } else if (kind == FSE_GEN_ZIPF8) {
            uint32_t u = r % 2283u, acc = 0;
            for (int k = 0; k < 8; k++) {
                acc += (uint32_t)zw[k];
                if (u < acc) {
                    mid = zm[k];
                    break;
                }
            }
        }
        w.id[i] = (uint16_t)mid;
        w.fl[i] = 0;
        w.df[i] = 0;
        w.sc[i] = soup_scalar(mt, mid, w.f32);
        if (w.tp) w.tp[i] = mt_type(mt->a[mid]) == T_SOUP ? (int16_t)mt->f_temp[mid] : (int16_t)0;
        uint32_t colour = mt->f_base[mid];
        uint32_t fp = mt->f_pack[mid];
        int mod = (int)(fp >> 20);
        if (mod > 0) colour += (uint32_t)((int)((fp >> 8) & 0xFFF) + (int)(draw_k(ck, 1) % (uint32_t)mod)) << (fp & 0xFF);
        w.col[i] = colour;
    }
}

int fse_world_generate(fse_world *w, int kind, uint32_t seed) {
    if (!w || kind < 0 || kind > 2) return FSE_E_INVAL;
    int rc = ensure_materials_pushed();
    if (rc) return rc;
    auto f = [](const char *s) {
        int v = fse_material_find(s);
        return v < 0 ? 0 : v;
    };
    size_t n = (size_t)w->W * w->H;
    int blocks = (int)std::min<size_t>((n + 255) / 256, (size_t)sm_count() * 16);
    k_generate<<<blocks, 256, 0, w->stream>>>(w->d, kind, seed, g_dev_mt, f("GENERIC_SAND"), f("WATER"), f("GENERIC_GAS"),
                                              f("STONE"), f("GENERIC_AIR"), f("STONE"), f("GENERIC_SAND"), f("WATER"),
                                              f("GENERIC_GAS"), f("DIRT"), f("GENERIC_LIQUID"), f("SOFT_DIRT_SAND"));
    FSE_CUDA_TRY(cudaGetLastError());
    if (w->h.dirty) FSE_CUDA_TRY(cudaMemsetAsync(w->h.dirty, 1, (size_t)w->W * w->H, w->stream));
    FSE_CUDA_TRY(cudaStreamSynchronize(w->stream));
    return FSE_OK;
}

int fse_world_get_tile(fse_world *w, int x, int y, uint16_t *id, uint32_t *col, int32_t *sc, uint8_t *fl) {
    if (!w) return FSE_E_INVAL;
    if (x < 0 || y < 0 || x >= w->W || y >= w->H) {
        // world.cpp:1000: out of range reads Tiles_TEST_SOLID
        if (id) *id = (uint16_t)host_table().id_solid;
        if (col) *col = 0xff0000u;
        if (sc) *sc = 0;
        if (fl) *fl = 0;
        return FSE_OK;
    }
    size_t i = (size_t)y * w->W + x;
    if (id) FSE_CUDA_TRY(cudaMemcpyAsync(id, w->h.id + i, 2, cudaMemcpyDeviceToHost, w->stream));
    if (col) FSE_CUDA_TRY(cudaMemcpyAsync(col, w->h.col + i, 4, cudaMemcpyDeviceToHost, w->stream));
    if (sc) FSE_CUDA_TRY(cudaMemcpyAsync(sc, w->h.sc + i, 4, cudaMemcpyDeviceToHost, w->stream));
    if (fl) FSE_CUDA_TRY(cudaMemcpyAsync(fl, w->h.fl + i, 1, cudaMemcpyDeviceToHost, w->stream));
    FSE_CUDA_TRY(cudaStreamSynchronize(w->stream));
    return FSE_OK;
}

int fse_world_set_tile(fse_world *w, int x, int y, uint16_t id, uint32_t col, int32_t sc, uint8_t fl) {
    if (!w) return FSE_E_INVAL;
    if (x < 0 || y < 0 || x >= w->W || y >= w->H) return FSE_OK;  // world.cpp:1005: dropped
    if (id >= host_table().n) return FSE_E_INVAL;
    size_t i = (size_t)y * w->W + x;
    fl &= (uint8_t)~VISITED;
    int32_t zero = 0;
    FSE_CUDA_TRY(cudaMemcpyAsync(w->h.id + i, &id, 2, cudaMemcpyHostToDevice, w->stream));
    FSE_CUDA_TRY(cudaMemcpyAsync(w->h.col + i, &col, 4, cudaMemcpyHostToDevice, w->stream));
    FSE_CUDA_TRY(cudaMemcpyAsync(w->h.sc + i, &sc, 4, cudaMemcpyHostToDevice, w->stream));
    FSE_CUDA_TRY(cudaMemcpyAsync(w->h.fl + i, &fl, 1, cudaMemcpyHostToDevice, w->stream));
    FSE_CUDA_TRY(cudaMemcpyAsync(w->h.df + i, &zero, 4, cudaMemcpyHostToDevice, w->stream));
    if (w->h.dirty) FSE_CUDA_TRY(cudaMemsetAsync(w->h.dirty + i, 1, 1, w->stream));
    FSE_CUDA_TRY(cudaStreamSynchronize(w->stream));
    return FSE_OK;
}

static int world_move_blocks(const fse_world *w) { return std::max(1, std::min(sm_count() * 4, ceil_div(w->part_cap, 256))); }
static int world_stage_blocks(const fse_world *w) { return std::max(1, std::min(sm_count() * 2, ceil_div(w->stage_cap, 256))); }

// 128 x 32 tiles of the temperature step when the world runs it inside its steps
static int world_temp_tiles(const fse_world *w) { return w->h.temp_on ? temperature_tiles(w->W, w->H) : 0; }

static int world_enqueue(fse_world *w, bool particles_after_tick, bool tick, bool particles) {
    int rc = ensure_materials_pushed();
    if (rc) return rc;
    if (tick) {
        rc = enqueue_step(w->d, 1, w->items, w->n_items, w->cell_iter, w->C, w->threads, w->grid, particles_after_tick,
                          world_move_blocks(w), world_stage_blocks(w), w->stream, w->timer, world_temp_tiles(w),
                          w->h.tp != nullptr, w->seq, w->h.f32 != 0);
        if (rc) return rc;
    } else if (particles) {
        if (launch_particle_tick(w->d, 1, g_dev_mt, world_move_blocks(w), w->stream) != cudaSuccess) return FSE_E_CUDA;
        count_launches(PARTICLE_TICK_LAUNCHES);
    }
    return FSE_OK;
}

int fse_world_sync(fse_world *w) {
    if (!w) return FSE_E_INVAL;
    int32_t c[16];
    int rc = read_ctr(w, c);
    if (rc) return rc;
    if (cudaGetLastError() != cudaSuccess) return FSE_E_CUDA;
    rc = status_from_err(c[5]);
    if (c[15]) {  // an asynchronous upload (fse_batch_upload) replaced out-of-range ids
        FSE_CUDA_TRY(cudaMemset(w->ctr + 15, 0, 4));
        if (!rc) rc = FSE_E_INVAL;
    }
    return rc;
}

int fse_world_tick(fse_world *w, int n) {
    if (!w || n < 0) return FSE_E_INVAL;
    for (int i = 0; i < n; i++) {
        int rc = world_enqueue(w, false, true, false);
        if (rc) return rc;
    }
    return fse_world_sync(w);
}

int fse_particles_tick(fse_world *w) {
    if (!w) return FSE_E_INVAL;
    int rc = world_enqueue(w, false, false, true);
    if (rc) return rc;
    return fse_world_sync(w);
}

int fse_world_step(fse_world *w, int n) {
    if (!w || n < 0) return FSE_E_INVAL;
    for (int i = 0; i < n; i++) {
        int rc = world_enqueue(w, true, true, true);
        if (rc) return rc;
    }
    return fse_world_sync(w);
}

int fse_world_enqueue(fse_world *w, int n, int with_particles) {
    if (!w || n < 0) return FSE_E_INVAL;
    for (int i = 0; i < n; i++) {
        int rc = world_enqueue(w, with_particles != 0, true, with_particles != 0);
        if (rc) return rc;
    }
    return cudaGetLastError() == cudaSuccess ? FSE_OK : FSE_E_CUDA;
}

// capture `ticks` steps once, replay to cover n
int fse_world_step_graph(fse_world *w, int n) {
    if (!w || n < 0) return FSE_E_INVAL;
    int rc = ensure_materials_pushed();
    if (rc) return rc;
    const int G = 32;
    int done = 0;
    while (done < n) {
        int k = std::min(G, n - done);
        auto it = w->graphs.find(k);
        cudaGraphExec_t ex;
        if (it == w->graphs.end()) {
            cudaGraph_t g;
            // kernels are counted when a replay launches them, not at capture
            const long long c0 = fse_launch_counter();
            FSE_CUDA_TRY(cudaStreamBeginCapture(w->stream, cudaStreamCaptureModeThreadLocal));
            int erc = FSE_OK;
            for (int i = 0; i < k && erc == FSE_OK; i++)
                erc = enqueue_step(w->d, 1, w->items, w->n_items, w->cell_iter, w->C, w->threads, w->grid, true,
                                   world_move_blocks(w), world_stage_blocks(w), w->stream, nullptr,
                                   world_temp_tiles(w), w->h.tp != nullptr, w->seq, w->h.f32 != 0);
            cudaError_t e = cudaStreamEndCapture(w->stream, &g);
            const long long kn = fse_launch_counter() - c0;
            count_launches(-kn);
            if (erc != FSE_OK || e != cudaSuccess) return FSE_E_CUDA;
            FSE_CUDA_TRY(cudaGraphInstantiate(&ex, g, 0));
            cudaGraphDestroy(g);
            w->graphs[k] = ex;
            w->graph_kernels[k] = kn;
        } else {
            ex = it->second;
        }
        FSE_CUDA_TRY(cudaGraphLaunch(ex, w->stream));
        count_launches(w->graph_kernels[k]);
        done += k;
    }
    return fse_world_sync(w);
}

int fse_world_set_stream(fse_world *w, void *stream) {
    if (!w) return FSE_E_INVAL;
    cudaStreamSynchronize(w->stream);
    for (auto &g : w->graphs) cudaGraphExecDestroy(g.second);
    w->graphs.clear();
    if (w->own_stream) cudaStreamDestroy(w->stream);
    if (stream) {
        w->stream = (cudaStream_t)stream;
        w->own_stream = false;
    } else {
        FSE_CUDA_TRY(cudaStreamCreateWithFlags(&w->stream, cudaStreamNonBlocking));
        w->own_stream = true;
    }
    return FSE_OK;
}

void *fse_world_stream(fse_world *w) { return w ? (void *)w->stream : nullptr; }

// =============================================================== particles
int fse_particles_count(fse_world *w, int *out_n) {
    if (!w || !out_n) return FSE_E_INVAL;
    int32_t c[16];
    int rc = read_ctr(w, c);
    if (rc) return rc;
    *out_n = c[1];
    return FSE_OK;
}

int fse_particles_add(fse_world *w, const fse_particle *parts, int n) {
    if (!w || (n > 0 && !parts) || n < 0) return FSE_E_INVAL;
    if (n == 0) return FSE_OK;
    int cur;
    int rc = fse_particles_count(w, &cur);
    if (rc) return rc;
    if ((long long)cur + n > w->part_cap) return FSE_E_CAPACITY;
    std::vector<float> f[9];
    std::vector<int32_t> life(n), fade(n), sc(n);
    std::vector<int16_t> tp(n);
    std::vector<uint32_t> col(n);
    std::vector<uint16_t> id(n);
    std::vector<uint8_t> fl(n), bits(n);
    for (int k = 0; k < 9; k++) f[k].resize(n);
    const MatTable &t = host_table();
    for (int i = 0; i < n; i++) {
        const fse_particle &p = parts[i];
        if (p.id >= t.n) return FSE_E_INVAL;
        const float v[9] = {p.x, p.y, p.vx, p.vy, p.ax, p.ay, p.target_x, p.target_y, p.target_force};
        for (int k = 0; k < 9; k++) f[k][i] = v[k];
        life[i] = p.lifetime;
        fade[i] = p.fade_time;
        sc[i] = p.scalar;
        tp[i] = p.temperature;
        col[i] = p.colour;
        id[i] = p.id;
        fl[i] = p.flags & (uint8_t)~VISITED;
        bits[i] = p.bits;
    }
    PartSoA &P = w->h.p;
    float *dst[9] = {P.x, P.y, P.vx, P.vy, P.ax, P.ay, P.tx, P.ty, P.tf};
    for (int k = 0; k < 9; k++)
        FSE_CUDA_TRY(cudaMemcpyAsync(dst[k] + cur, f[k].data(), n * 4, cudaMemcpyHostToDevice, w->stream));
    FSE_CUDA_TRY(cudaMemcpyAsync(P.life + cur, life.data(), n * 4, cudaMemcpyHostToDevice, w->stream));
    FSE_CUDA_TRY(cudaMemcpyAsync(P.fade + cur, fade.data(), n * 4, cudaMemcpyHostToDevice, w->stream));
    FSE_CUDA_TRY(cudaMemcpyAsync(P.sc + cur, sc.data(), n * 4, cudaMemcpyHostToDevice, w->stream));
    if (P.tp) FSE_CUDA_TRY(cudaMemcpyAsync(P.tp + cur, tp.data(), n * 2, cudaMemcpyHostToDevice, w->stream));
    FSE_CUDA_TRY(cudaMemcpyAsync(P.col + cur, col.data(), n * 4, cudaMemcpyHostToDevice, w->stream));
    FSE_CUDA_TRY(cudaMemcpyAsync(P.id + cur, id.data(), n * 2, cudaMemcpyHostToDevice, w->stream));
    FSE_CUDA_TRY(cudaMemcpyAsync(P.fl + cur, fl.data(), n, cudaMemcpyHostToDevice, w->stream));
    FSE_CUDA_TRY(cudaMemcpyAsync(P.bits + cur, bits.data(), n, cudaMemcpyHostToDevice, w->stream));
    int32_t nn = cur + n;
    FSE_CUDA_TRY(cudaMemcpyAsync(w->h.part_count, &nn, 4, cudaMemcpyHostToDevice, w->stream));
    FSE_CUDA_TRY(cudaStreamSynchronize(w->stream));
    return FSE_OK;
}

int fse_particles_read(fse_world *w, fse_particle *out, int cap, int *out_n) {
    if (!w || cap < 0 || (cap > 0 && !out)) return FSE_E_INVAL;
    int n;
    int rc = fse_particles_count(w, &n);
    if (rc) return rc;
    if (out_n) *out_n = n;
    int m = std::min(n, cap);
    if (m == 0) return FSE_OK;
    std::vector<float> f[9];
    std::vector<int32_t> life(m), fade(m), sc(m);
    std::vector<int16_t> tp(m);
    std::vector<uint32_t> col(m);
    std::vector<uint16_t> id(m);
    std::vector<uint8_t> fl(m), bits(m);
    PartSoA &P = w->h.p;
    float *src[9] = {P.x, P.y, P.vx, P.vy, P.ax, P.ay, P.tx, P.ty, P.tf};
    for (int k = 0; k < 9; k++) {
        f[k].resize(m);
        FSE_CUDA_TRY(cudaMemcpyAsync(f[k].data(), src[k], m * 4, cudaMemcpyDeviceToHost, w->stream));
    }
    FSE_CUDA_TRY(cudaMemcpyAsync(life.data(), P.life, m * 4, cudaMemcpyDeviceToHost, w->stream));
    FSE_CUDA_TRY(cudaMemcpyAsync(fade.data(), P.fade, m * 4, cudaMemcpyDeviceToHost, w->stream));
    FSE_CUDA_TRY(cudaMemcpyAsync(sc.data(), P.sc, m * 4, cudaMemcpyDeviceToHost, w->stream));
    if (P.tp) FSE_CUDA_TRY(cudaMemcpyAsync(tp.data(), P.tp, m * 2, cudaMemcpyDeviceToHost, w->stream));
    FSE_CUDA_TRY(cudaMemcpyAsync(col.data(), P.col, m * 4, cudaMemcpyDeviceToHost, w->stream));
    FSE_CUDA_TRY(cudaMemcpyAsync(id.data(), P.id, m * 2, cudaMemcpyDeviceToHost, w->stream));
    FSE_CUDA_TRY(cudaMemcpyAsync(fl.data(), P.fl, m, cudaMemcpyDeviceToHost, w->stream));
    FSE_CUDA_TRY(cudaMemcpyAsync(bits.data(), P.bits, m, cudaMemcpyDeviceToHost, w->stream));
    FSE_CUDA_TRY(cudaStreamSynchronize(w->stream));
    for (int i = 0; i < m; i++) {
        fse_particle &p = out[i];
        p.x = f[0][i];
        p.y = f[1][i];
        p.vx = f[2][i];
        p.vy = f[3][i];
        p.ax = f[4][i];
        p.ay = f[5][i];
        p.target_x = f[6][i];
        p.target_y = f[7][i];
        p.target_force = f[8][i];
        p.lifetime = life[i];
        p.fade_time = fade[i];
        p.colour = col[i];
        p.scalar = sc[i];
        p.id = id[i];
        p.flags = fl[i];
        p.bits = bits[i];
        p.temperature = tp[i];
        p.reserved = 0;
    }
    return FSE_OK;
}

// ============================================================ diagnostics
int fse_world_pass_timing(fse_world *w, int enable, double *out_ms, int64_t *out_launches) {
    if (!w) return FSE_E_INVAL;
    FSE_CUDA_TRY(cudaStreamSynchronize(w->stream));
    if (w->timer) w->timer->drain();
    if (out_ms) *out_ms = w->timer ? w->timer->ms : 0.0;
    if (out_launches) *out_launches = w->timer ? w->timer->launches : 0;
    if (enable) {
        if (!w->timer) w->timer = new PassTimer();
        w->timer->ms = 0.0;
        w->timer->launches = 0;
    } else if (w->timer) {
        for (cudaEvent_t e : w->timer->pool) cudaEventDestroy(e);
        delete w->timer;
        w->timer = nullptr;
    }
    return FSE_OK;
}

int64_t fse_launch_counter(void) { return (int64_t)g_launches.load(); }

// ================================================================= ledger
int fse_world_ledger(fse_world *w, int64_t *out) {
    if (!w || !out) return FSE_E_INVAL;
    std::vector<long long> buf(LED_ROWS * MAXMAT);
    FSE_CUDA_TRY(cudaMemcpyAsync(buf.data(), w->h.ledger, buf.size() * 8, cudaMemcpyDeviceToHost, w->stream));
    FSE_CUDA_TRY(cudaStreamSynchronize(w->stream));
    int n = fse_material_count();
    for (int r = 0; r < LED_ROWS; r++)
        for (int m = 0; m < n; m++) out[r * n + m] = buf[r * MAXMAT + m];
    return FSE_OK;
}

int fse_world_ledger_reset(fse_world *w) {
    if (!w) return FSE_E_INVAL;
    FSE_CUDA_TRY(cudaMemsetAsync(w->h.ledger, 0, LED_ROWS * MAXMAT * 8, w->stream));
    FSE_CUDA_TRY(cudaStreamSynchronize(w->stream));
    return FSE_OK;
}

__global__ void k_census(const WorldDev *__restrict__ wd, const MatTable *__restrict__ mt, long long *out) {
    __shared__ unsigned long long s[4 * MAXMAT];
    for (int i = threadIdx.x; i < 4 * MAXMAT; i += blockDim.x) s[i] = 0;
    __syncthreads();
    const WorldDev &w = *wd;
    const size_t n = (size_t)w.W * w.H;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        int id = w.id[i];
        atomicAdd(&s[id], 1ull);
        if (!w.f32 && mt_type(mt->a[id]) == T_SOUP)  // no fluid rows for f32 amounts
            atomicAdd(&s[MAXMAT + id], (unsigned long long)((long long)w.sc[i] + w.df[i]));
    }
    const int np = *w.part_count;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < np; i += gridDim.x * blockDim.x) {
        int id = w.p.id[i];
        atomicAdd(&s[2 * MAXMAT + id], 1ull);
        if (!w.f32 && mt_type(mt->a[id]) == T_SOUP)
            atomicAdd(&s[3 * MAXMAT + id], (unsigned long long)(long long)w.p.sc[i]);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < 4 * MAXMAT; i += blockDim.x)
        if (s[i]) atomicAdd((unsigned long long *)&out[i], s[i]);
}

int fse_world_census(fse_world *w, int64_t *out) {
    if (!w || !out) return FSE_E_INVAL;
    int rc = ensure_materials_pushed();
    if (rc) return rc;
    long long *d = nullptr;
    FSE_CUDA_TRY(cudaMalloc(&d, 4 * MAXMAT * 8));
    cudaMemsetAsync(d, 0, 4 * MAXMAT * 8, w->stream);
    k_census<<<sm_count() * 2, 512, 0, w->stream>>>(w->d, g_dev_mt, d);
    std::vector<long long> buf(4 * MAXMAT);
    cudaMemcpyAsync(buf.data(), d, buf.size() * 8, cudaMemcpyDeviceToHost, w->stream);
    cudaError_t e = cudaStreamSynchronize(w->stream);
    cudaFree(d);
    if (e != cudaSuccess) return FSE_E_CUDA;
    int n = fse_material_count();
    for (int r = 0; r < 4; r++)
        for (int m = 0; m < n; m++) out[r * n + m] = buf[r * MAXMAT + m];
    return FSE_OK;
}

}  // extern "C"
