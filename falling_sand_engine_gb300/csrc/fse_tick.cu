// fse_tick.cu -- the cell update of world::tick() (source/engine/world.cpp:1036-1948)
// as one colour-pass kernel.
//
// A launch handles one chunk colour of one iteration (world.cpp:1050-1077) for a
// list of chunks, possibly of many worlds. Each CTA stages its chunk plus a halo in
// shared memory (id, flags, scalar, colour; the pending fluid diff stays in HBM and
// is touched only by SOUP cells), runs sweeps A, B and C as sequences of lattice
// sub-phases separated by __syncthreads(), and writes back only the cells it
// changed. Inside a sub-phase every cell is processed by its own thread; the
// lattice spacing makes every write set disjoint from every other cell's read and
// write sets, so the result does not depend on thread timing.
#include "fse_internal.cuh"

namespace fse {

struct Cell {
    uint16_t id;
    uint8_t fl;
    int32_t sc;
    uint32_t col;
    int32_t df;   // valid when src < 0
    int32_t src;  // >= 0: the diff still lives in HBM at this cell index
};

struct SpawnEv {
    int n;     // particles to emit (0 = none)
    int kind;  // 1 sand, 2 soup, 3 fire
    int x, y;
    uint16_t id;
    uint8_t fl;
    uint32_t col;
    int32_t sc;
    float vx, vy;
    uint32_t ck, k0;
};

// ------------------------------------------------------- shared-memory tile
// Region: x in [cx - HALO, cx + C + HALO), full state for y in
// [cy - HALO, cy + C + HALO), material ids only down to y < cy + C + 10 (the
// deepest read, the friction pillar of world.cpp:1619-1627).
struct Tile {
    uint16_t *s_id;
    uint8_t *s_fl;
    int32_t *s_sc;
    uint32_t *s_col;
    const uint32_t *ma;  // material word A in shared memory
    const float *md;     // density in shared memory
    int32_t *df;         // HBM diff plane
    int x0, y0, RW, RHF, RHI;
    int W, H;
    int id_solid, id_air;
    int *err;

    __device__ __forceinline__ bool inw(int x, int y) const {
        return (unsigned)x < (unsigned)W && (unsigned)y < (unsigned)H;
    }
    __device__ __forceinline__ int li(int x, int y) const { return (y - y0) * RW + (x - x0); }
    __device__ __forceinline__ bool in_ids(int x, int y) const {
        return (unsigned)(x - x0) < (unsigned)RW && (unsigned)(y - y0) < (unsigned)RHI;
    }
    __device__ __forceinline__ bool in_full(int x, int y) const {
        return (unsigned)(x - x0) < (unsigned)RW && (unsigned)(y - y0) < (unsigned)RHF;
    }
    __device__ __forceinline__ void oob() const { atomicOr(err, ERR_BOUNDS); }

    __device__ __forceinline__ int id(int x, int y) const {
        if (!inw(x, y)) return id_solid;
        if (!in_ids(x, y)) {
            oob();
            return id_solid;
        }
        return s_id[li(x, y)] & 0x7FFF;
    }
    __device__ __forceinline__ int type(int x, int y) const { return mt_type(ma[id(x, y)]); }

    __device__ __forceinline__ Cell get(int x, int y) const {
        Cell c;
        c.df = 0;
        c.src = -1;
        if (!inw(x, y) || !in_full(x, y)) {
            if (inw(x, y)) oob();
            c.id = (uint16_t)id_solid;
            c.fl = 0;
            c.sc = 0;
            c.col = 0xff0000u;  // Tiles_TEST_SOLID, game_datastruct.cpp:312
            return c;
        }
        int i = li(x, y);
        c.id = s_id[i] & 0x7FFF;
        c.fl = s_fl[i] & (uint8_t)~VISITED;
        c.sc = s_sc[i];
        c.col = s_col[i];
        if (mt_type(ma[c.id]) == T_SOUP) c.src = y * W + x;
        return c;
    }
    // the active cell: its diff is needed at once
    __device__ __forceinline__ Cell get_active(int x, int y) const {
        Cell c = get(x, y);
        if (c.src >= 0) {
            c.df = df[c.src];
            c.src = -1;
        }
        return c;
    }
    __device__ __forceinline__ void put(int x, int y, const Cell &c) const {
        if (!inw(x, y)) return;
        if (!in_full(x, y)) {
            oob();
            return;
        }
        int i = li(x, y);
        s_id[i] = c.id | DIRTY;
        s_fl[i] = (uint8_t)((c.fl & (uint8_t)~VISITED) | (s_fl[i] & VISITED));
        s_sc[i] = c.sc;
        s_col[i] = c.col;
        if (mt_type(ma[c.id]) == T_SOUP) {
            int g = y * W + x;
            int32_t v = (c.src >= 0) ? df[c.src] : c.df;
            df[g] = v;
        }
    }
    __device__ __forceinline__ void set_moved(int x, int y, bool on) const {
        if (!inw(x, y)) return;
        if (!in_full(x, y)) {
            oob();
            return;
        }
        int i = li(x, y);
        s_fl[i] = on ? (uint8_t)(s_fl[i] | MOVED) : (uint8_t)(s_fl[i] & (uint8_t)~MOVED);
        s_id[i] |= DIRTY;
    }
    __device__ __forceinline__ void add_diff(int x, int y, int32_t v) const {
        if (!inw(x, y)) return;
        df[y * W + x] += v;
    }
    __device__ __forceinline__ bool vis(int x, int y) const {
        if (!inw(x, y) || !in_full(x, y)) return false;
        return (s_fl[li(x, y)] & VISITED) != 0;
    }
    __device__ __forceinline__ void setvis(int x, int y) const {
        if (!inw(x, y)) return;
        if (!in_full(x, y)) {
            oob();
            return;
        }
        s_fl[li(x, y)] |= VISITED;
    }
};

// ------------------------------------------------------------- rule context
struct Ctx {
    uint32_t pk, ck, k;
    int iter;
    const MatTable *mt;
    long long *led_s;  // shared ledger [LED_ROWS][64]
    long long *led_g;  // global ledger [LED_ROWS][MAXMAT]
    const uint32_t *ma;
    SpawnEv ev;
    __device__ __forceinline__ uint32_t D() { return draw_k(ck, k++); }
};

__device__ __forceinline__ void led_add(Ctx &c, int row, int mat, long long v) {
    if (v == 0 || mt_type(c.ma[mat]) == T_AIR) return;
    if (mat < 64)
        atomicAdd((unsigned long long *)&c.led_s[row * 64 + mat], (unsigned long long)v);
    else
        atomicAdd((unsigned long long *)&c.led_g[row * MAXMAT + mat], (unsigned long long)v);
}
__device__ __forceinline__ void led_replace(Ctx &c, const Cell &old, int32_t old_df, const Cell &nw) {
    led_add(c, LED_DN, old.id, 1);
    if (mt_type(c.ma[old.id]) == T_SOUP) led_add(c, LED_DF, old.id, (long long)old.sc + old_df);
    led_add(c, LED_CN, nw.id, 1);
    if (mt_type(c.ma[nw.id]) == T_SOUP) led_add(c, LED_CF, nw.id, (long long)nw.sc + nw.df);
}
__device__ __forceinline__ int32_t cell_df(const Tile &t, const Cell &c) { return c.src >= 0 ? t.df[c.src] : c.df; }

__device__ __forceinline__ Cell nothing(int id_air) {
    Cell c;
    c.id = (uint16_t)id_air;
    c.fl = 0;
    c.sc = 0;
    c.col = 0;
    c.df = 0;
    c.src = -1;
    return c;
}

// TilesCreate(id, x, y), game_datastruct.cpp:494-574
__device__ __forceinline__ Cell create_tile(Ctx &c, int mid) {
    Cell t;
    t.id = (uint16_t)mid;
    t.fl = 0;
    t.df = 0;
    t.src = -1;
    t.sc = __ldg(&c.mt->f_scalar[mid]);
    t.col = __ldg(&c.mt->f_base[mid]);
    uint32_t fp = __ldg(&c.mt->f_pack[mid]);
    int mod = (int)(fp >> 20);
    if (mod > 0) {
        int shift = (int)(fp & 0xFF), lo = (int)((fp >> 8) & 0xFFF);
        t.col = t.col + ((uint32_t)(lo + (int)(c.D() % (uint32_t)mod)) << shift);
    }
    return t;
}

// CalculateVerticalFlowValue, world.cpp:1021-1034, Q16.16
__device__ __forceinline__ int32_t vflow(int32_t rem, int32_t dst) {
    long long sum = (long long)rem + dst;
    if (sum <= Q_MAXV) return Q_MAXV;
    if (sum < 2 * Q_MAXV + Q_MAXCOMP)
        return (int32_t)(((long long)Q_MAXV * Q_MAXV + sum * Q_MAXCOMP) / (Q_MAXV + Q_MAXCOMP));
    return (int32_t)((sum + Q_MAXCOMP) / 2);
}
__device__ __forceinline__ int32_t clampflow(int32_t flow, int32_t rem) {
    if (flow < 0) flow = 0;
    int32_t lim = rem < Q_MAXFLOW ? rem : Q_MAXFLOW;
    return flow > lim ? lim : flow;
}

__device__ __forceinline__ bool can_sink(const uint32_t *ma, const float *md, int other, int self) {
    int t = mt_type(ma[other]);
    return t == T_AIR || (t != T_SOLID && md[other] < md[self]);
}

// one SOUP flow towards (nx, ny), shared by the four directions of world.cpp:1309-1460
__device__ __forceinline__ void soup_flow(const Tile &T, Ctx &c, Cell &t, int32_t &rem, int32_t flow, int nT, int nx,
                                          int ny) {
    if (flow == 0) return;
    rem -= flow;
    t.df -= flow;
    if (nT == T_AIR) {
        Cell nt;
        nt.id = t.id;
        nt.fl = 0;
        nt.sc = 0;
        nt.col = t.col;
        nt.df = flow;
        nt.src = -1;
        T.put(nx, ny, nt);
        led_add(c, LED_CN, t.id, 1);
    } else {
        T.add_diff(nx, ny, flow);
    }
}

// ----------------------------------------------------------------- sweep A
__device__ void rule_a(const Tile &T, Ctx &c, int x, int y) {
    if (T.vis(x, y)) return;  // world.cpp:1091
    const uint32_t *ma = T.ma;
    const float *md = T.md;
    Cell t = T.get_active(x, y);
    uint32_t a = ma[t.id];
    if (c.iter >= mt_iter(a)) {  // world.cpp:1093-1096
        T.setvis(x, y);
        return;
    }
    int type = mt_type(a);
    c.ck = cell_key(c.pk, (uint32_t)x, (uint32_t)y);
    c.k = 0;
    const MatTable *mt = c.mt;

    if ((int)t.id == mt->id_fire) {  // world.cpp:1101-1146
        if (c.D() % 10 == 0) t.col = (255u << 16) | ((uint32_t)(100 + (int)(c.D() % 50)) << 8) | 50u;
        if (c.D() % 10 == 0) {
            float vx = (float)((int)(c.D() % 10) - 5) / 20.0f;
            float vy = -((float)(int)(c.D() % 10) / 10.0f) / 3.0f + -0.5f;
            c.ev.n = 1;
            c.ev.kind = 3;
            c.ev.x = x;
            c.ev.y = y - 1;
            c.ev.id = t.id;
            c.ev.fl = t.fl;
            c.ev.col = t.col;
            c.ev.sc = t.sc;
            c.ev.vx = vx;
            c.ev.vy = vy;
            led_add(c, LED_CN, t.id, 1);
        }
        if (c.D() % 150 == 0) {
            led_replace(c, t, t.df, nothing(T.id_air));
            T.put(x, y, nothing(T.id_air));
            T.setvis(x, y);
        } else {
            bool found = false;
            for (int xx = -2; xx <= 2; xx++)
                for (int yy = -2; yy <= 2; yy++) {
                    if (T.type(x + xx, y + yy) == T_SOLID) {
                        found = true;
                        if (c.D() % 500 == 0) {
                            Cell f = create_tile(c, mt->id_fire);
                            if (T.inw(x + xx, y + yy)) {
                                Cell o = T.get(x + xx, y + yy);
                                led_replace(c, o, cell_df(T, o), f);
                            }
                            T.put(x + xx, y + yy, f);
                            T.setvis(x + xx, y + yy);
                        }
                    }
                }
            if (!found && c.D() % 120 == 0) {
                Cell o = T.get(x, y);
                led_replace(c, o, cell_df(T, o), nothing(T.id_air));
                T.put(x, y, nothing(T.id_air));
                T.setvis(x, y);
            }
        }
    }

    if (type == T_SAND) {
        Cell below = T.get(x, y + 1);  // world.cpp:1150
        int bt = mt_type(ma[below.id]);
        if (mt->has_inter) {  // world.cpp:1153-1179
            int hit = -1;
            for (int i = 0; i < mt->n_inter; i++)
                if (mt->inter[i][0] == (int)t.id && mt->inter[i][1] == (int)below.id) hit = i;
            if (hit >= 0) {
                for (int i = 0; i < mt->n_inter; i++) {
                    if (mt->inter[i][0] != (int)t.id || mt->inter[i][1] != (int)below.id) continue;
                    int kind = mt->inter[i][2], d1 = mt->inter[i][3], d2 = mt->inter[i][4];
                    int ox = mt->inter[i][5], oy = mt->inter[i][6];
                    for (int xx = ox - d2; xx <= ox + d2; xx++)
                        for (int yy = oy - d2; yy <= oy + d2; yy++) {
                            bool doit = (kind == INTER_TRANSFORM) ? (T.id(x + xx, y + yy) == (int)below.id)
                                                                  : ((xx == 0 && yy == 0) ||
                                                                     T.id(x + xx, y + yy) == T.id_air);
                            if (doit) {
                                Cell nt = create_tile(c, d1);
                                if (T.inw(x + xx, y + yy)) {
                                    Cell o = T.get(x + xx, y + yy);
                                    led_replace(c, o, cell_df(T, o), nt);
                                }
                                T.put(x + xx, y + yy, nt);
                                T.setvis(x + xx, y + yy);
                            }
                        }
                }
                return;
            }
        }
        int nr = mt->n_react[t.id];
        if (nr > 0) {  // world.cpp:1181-1204
            bool react = false;
            for (int i = 0; i < nr; i++) {
                int kind = mt->react[t.id][i][0], temp = mt->react[t.id][i][1], res = mt->react[t.id][i][2];
                bool hit = (kind == REACT_BELOW) ? (t.sc < temp) : (t.sc > temp);
                if (hit) {
                    Cell nt = create_tile(c, res);
                    if (mt_type(ma[nt.id]) != T_SOUP) nt.sc = t.sc;
                    Cell o = T.get(x, y);
                    led_replace(c, o, cell_df(T, o), nt);
                    T.put(x, y, nt);
                    T.setvis(x, y);
                    react = true;
                }
            }
            if (react) return;
        }
        // world.cpp:1206-1267
        if (!can_sink(ma, md, below.id, t.id)) return;
        Cell bl = T.get(x - 1, y + 1), br = T.get(x + 1, y + 1);
        bool canL = can_sink(ma, md, bl.id, t.id);
        bool canR = can_sink(ma, md, br.id, t.id);
        if (!((canL || canR) && c.D() % 20 == 0)) {
            if (bt == T_AIR && T.type(x, y + 2) == T_AIR && T.type(x, y + 3) == T_AIR && T.type(x, y + 4) == T_AIR) {
                T.put(x, y, below);
                float vx = (float)((int)(c.D() % 10) - 5) / 20.0f;
                float vy = (float)(-((int)(c.D() % 2) + 3)) / 10.0f + 1.5f;
                c.ev.n = 1;
                c.ev.kind = 1;
                c.ev.x = x;
                c.ev.y = y + 1;
                c.ev.id = t.id;
                c.ev.fl = t.fl;
                c.ev.col = t.col;
                c.ev.sc = t.sc;
                c.ev.vx = vx;
                c.ev.vy = vy;
            } else {
                T.put(x, y, below);
                if (c.D() % 2 == 0) t.fl |= MOVED;
                T.put(x, y + 1, t);
                T.setvis(x, y + 1);
            }
            if (c.D() % 2 == 0) {
                if (x > 0 && T.type(x - 1, y + 1) == T_SAND) {
                    if (c.D() % 2 == 0) T.set_moved(x - 1, y + 1, true);
                }
                if (x < T.W - 1 && T.type(x + 1, y + 1) == T_SAND) {
                    if (c.D() % 2 == 0) T.set_moved(x + 1, y + 1, true);
                }
            }
        }
    } else if (type == T_SOUP) {  // world.cpp:1269-1567
        if (t.sc == 0) return;
        if (t.sc < Q_MINV) {
            led_add(c, LED_DF, t.id, t.sc);
            t.sc = 0;
            T.put(x, y, t);
            return;
        }
        if (t.sc > Q_FREEFALL && T.type(x, y + 1) == T_AIR && T.type(x, y + 2) == T_AIR &&
            T.type(x, y + 3) == T_AIR && T.type(x, y + 4) == T_AIR) {  // world.cpp:1283-1305
            T.put(x, y, nothing(T.id_air));
            int n = t.sc >> 18;
            if (n < 1) n = 1;
            led_add(c, LED_DF, t.id, t.df);
            led_add(c, LED_CN, t.id, n - 1);
            c.ev.n = n;
            c.ev.kind = 2;
            c.ev.x = x;
            c.ev.y = y + 1;
            c.ev.id = t.id;
            c.ev.fl = 0;
            c.ev.col = t.col;
            c.ev.sc = t.sc;
            c.ev.ck = c.ck;
            c.ev.k0 = c.k;
            c.k += 2 * n;
            return;
        }
        if (t.fl & MOVED) return;
        int32_t start = t.sc, rem = t.sc;
        Cell bottom = T.get(x, y + 1);
        int bT = mt_type(ma[bottom.id]);
        bool airBelow = bT == T_AIR;
        if ((airBelow && c.iter <= 2) || bottom.id == t.id) {
            int32_t dst = (bT == T_SOUP) ? bottom.sc : 0;
            soup_flow(T, c, t, rem, clampflow(vflow(start, dst) - dst, start), bT, x, y + 1);
        } else if (c.iter == 0 && bT == T_SOUP && bottom.id != t.id) {
            if (c.D() % 10 == 0) {
                T.put(x, y, bottom);
                T.put(x, y + 1, t);
                return;
            }
        }
        if (rem < Q_MINV) {
            t.df -= rem;
            led_add(c, LED_DF, t.id, rem);
            T.put(x, y, t);
            return;
        }
        Cell left = T.get(x - 1, y);
        int lT = mt_type(ma[left.id]);
        bool canL = (lT == T_AIR || left.id == t.id) && !airBelow;
        Cell right = T.get(x + 1, y);
        int rT = mt_type(ma[right.id]);
        bool canR = (rT == T_AIR || right.id == t.id) && !airBelow;
        if (canL) {
            int32_t dst = (lT == T_SOUP) ? left.sc : 0;
            soup_flow(T, c, t, rem, clampflow((rem - dst) / (canR ? 3 : 2), rem), lT, x - 1, y);
        }
        if (rem < Q_MINV) {
            t.df -= rem;
            led_add(c, LED_DF, t.id, rem);
            T.put(x, y, t);
            return;
        }
        if (canR) {
            int32_t dst = (rT == T_SOUP) ? right.sc : 0;
            soup_flow(T, c, t, rem, clampflow((rem - dst) / 2, rem), rT, x + 1, y);
        }
        if (rem < Q_MINV) {
            t.df -= rem;
            led_add(c, LED_DF, t.id, rem);
            T.put(x, y, t);
            return;
        }
        Cell top = T.get(x, y - 1);
        int tT = mt_type(ma[top.id]);
        if (tT == T_AIR || top.id == t.id) {
            int32_t dst = (tT == T_SOUP) ? top.sc : 0;
            soup_flow(T, c, t, rem, clampflow(rem - vflow(rem, dst), rem), tT, x, y - 1);
        } else if (c.iter == 0 && tT == T_SOUP && top.id != t.id) {
            if (c.D() % 10 == 0) {
                T.put(x, y, top);
                T.put(x, y - 1, t);
                return;
            }
        }
        if (rem < Q_MINV) {
            t.df -= rem;
            led_add(c, LED_DF, t.id, rem);
            T.put(x, y, t);
            return;
        }
        if (start == rem) {  // world.cpp:1472-1483
            uint8_t s = t.fl & SETTLE_MASK;
            if (s < SETTLE_MASK) s++;
            t.fl = (uint8_t)((t.fl & ~SETTLE_MASK) | s);
            if (s >= 10) t.fl |= MOVED;
        } else {
            if (tT == T_SOUP) T.set_moved(x, y - 1, false);
            if (bT == T_SOUP) T.set_moved(x, y + 1, false);
            if (lT == T_SOUP) T.set_moved(x - 1, y, false);
            if (rT == T_SOUP) T.set_moved(x + 1, y, false);
        }
        T.put(x, y, t);
        // WATER on LAVA, world.cpp:1519-1537
        if ((int)t.id == mt->id_water && T.id(x, y + 1) == mt->id_lava) {
            Cell st = create_tile(c, mt->id_steam);
            led_replace(c, t, t.df, st);
            T.put(x, y, st);
            Cell ob = create_tile(c, mt->id_obsidian);
            Cell o = T.get(x, y + 1);
            led_replace(c, o, cell_df(T, o), ob);
            T.put(x, y + 1, ob);
            T.setvis(x, y + 1);
            for (int xx = -1; xx <= 1; xx++)
                for (int yy = 0; yy <= 2; yy++) {
                    if (T.id(x + xx, y + yy) == mt->id_lava) {
                        Cell o2 = create_tile(c, mt->id_obsidian);
                        Cell oo = T.get(x + xx, y + yy);
                        led_replace(c, oo, cell_df(T, oo), o2);
                        T.put(x + xx, y + yy, o2);
                        T.setvis(x + xx, y + yy);
                    }
                }
            return;
        }
    } else if (type == T_GAS) {  // world.cpp:1569-1585
        int above = T.type(x, y - 1);
        int aboveL = T.type(x - 1, y - 1);
        int aboveR = T.type(x + 1, y - 1);
        if (above == T_AIR && !((aboveL == T_AIR || aboveR == T_AIR) && c.D() % 2 == 0)) {
            T.put(x, y, T.get(x, y - 1));
            T.put(x, y - 1, t);
            T.setvis(x, y - 1);
        }
    }
}

// ----------------------------------------------------------------- sweep B
__device__ void rule_b(const Tile &T, Ctx &c, int x, int y) {
    if (T.vis(x, y)) return;  // world.cpp:1597
    const uint32_t *ma = T.ma;
    const float *md = T.md;
    int sid = T.id(x, y);
    uint32_t a = ma[sid];
    int type = mt_type(a);
    if (type != T_SAND && type != T_SOUP && type != T_GAS) return;
    Cell t = T.get_active(x, y);
    c.ck = cell_key(c.pk, (uint32_t)x, (uint32_t)y);
    c.k = 0;
    if (type == T_SAND) {  // world.cpp:1602-1727
        Cell bl = T.get(x - 1, y + 1), br = T.get(x + 1, y + 1);
        bool canL = can_sink(ma, md, bl.id, t.id);
        bool canR = can_sink(ma, md, br.id, t.id);
        bool stopped = !(t.fl & MOVED);
        int slip = mt_slip(a);
        if (stopped) {
            int drop = 0;
            for (int pil = 0; pil < 10; pil++) {
                int l = T.type(x - 1, y + 1 + pil);
                int r = T.type(x + 1, y + 1 + pil);
                if (l == T_AIR || r == T_AIR) drop++;
            }
            int d = drop + 1 - mt_stab(a);
            if (d > 0) {
                int chance = 1000 / d;
                if (chance < 1000) {
                    if (c.D() % (uint32_t)chance == 0) {
                        stopped = false;
                        T.set_moved(x, y, true);
                    }
                }
            }
        }
        if (stopped || !(canL || canR)) {
            T.set_moved(x, y, false);
            return;
        }
        bool shouldMove = (slip > 0) ? (c.D() % (uint32_t)(2 * slip) != 0) : true;
        if (shouldMove && (canL || canR)) {
            if (c.D() % 2 == 0) {
                if (T.type(x, y + 1) == T_SAND) {
                    if (c.D() % 2 == 0) T.set_moved(x, y + 1, true);
                }
            }
        }
        if (shouldMove && canL && (!canR || c.D() % 2 == 0)) {
            if (T.type(x - 1, y) == T_AIR) {
                T.put(x - 1, y, bl);
                T.setvis(x - 1, y);
                T.put(x, y, nothing(T.id_air));
            } else {
                T.put(x, y, bl);
                T.setvis(x, y);
            }
            if (slip > 0 && c.D() % (uint32_t)(20 * slip) == 0) t.fl &= (uint8_t)~MOVED;
            T.put(x - 1, y + 1, t);
            T.setvis(x - 1, y + 1);
        } else if (shouldMove && canR) {
            if (T.type(x + 1, y) == T_AIR) {
                T.put(x + 1, y, br);
                T.put(x, y, nothing(T.id_air));
            } else {
                T.put(x, y, br);
                T.setvis(x, y);
            }
            if (slip > 0 && c.D() % (uint32_t)(20 * slip) == 0) t.fl &= (uint8_t)~MOVED;
            T.put(x + 1, y + 1, t);
            T.setvis(x + 1, y + 1);
        } else {
            T.set_moved(x, y, false);
        }
    } else if (type == T_SOUP) {  // world.cpp:1728-1745
        t.sc += t.df;
        t.df = 0;
        if (t.sc < Q_MINV) {
            led_add(c, LED_DN, t.id, 1);
            led_add(c, LED_DF, t.id, t.sc);
            T.put(x, y, nothing(T.id_air));
            T.setvis(x, y);
        } else {
            T.put(x, y, t);
            T.setvis(x, y);
        }
    } else {  // GAS, world.cpp:1799-1818
        int aboveL = T.type(x - 1, y - 1);
        int aboveR = T.type(x + 1, y - 1);
        if (aboveL == T_AIR && !(aboveR == T_AIR && c.D() % 2 == 0)) {
            T.put(x, y, T.get(x - 1, y - 1));
            T.put(x - 1, y - 1, t);
            T.setvis(x - 1, y - 1);
        } else if (aboveR == T_AIR) {
            T.put(x, y, T.get(x + 1, y - 1));
            T.put(x + 1, y - 1, t);
            T.setvis(x + 1, y - 1);
        }
    }
}

// ----------------------------------------------------------------- sweep C
__device__ void rule_c(const Tile &T, Ctx &c, int x, int y) {
    if (T.vis(x, y)) return;  // world.cpp:1831
    int sid = T.id(x, y);
    if (mt_type(T.ma[sid]) != T_GAS) return;
    Cell t = T.get_active(x, y);
    c.ck = cell_key(c.pk, (uint32_t)x, (uint32_t)y);
    c.k = 0;
    // world.cpp:1862-1889
    int l = T.type(x - 1, y);
    int r = T.type(x + 1, y);
    if (l == T_AIR && !(r == T_AIR && c.D() % 2 == 0)) {
        T.put(x, y, T.get(x - 1, y));
        T.put(x - 1, y, t);
        T.setvis(x - 1, y);
    } else if (r == T_AIR) {
        T.put(x, y, T.get(x + 1, y));
        T.put(x + 1, y, t);
        T.setvis(x + 1, y);
    } else if ((int)t.id == c.mt->id_steam) {
        if (c.D() % 10 == 0) {
            Cell wt = create_tile(c, c.mt->id_water);
            led_replace(c, t, 0, wt);
            T.put(x, y, wt);
        }
    }
}

// --------------------------------------------------------------- lattices
// (Px, Py) per sweep and chunk mode; see the oracle's lattice() for the derivation.
__device__ __forceinline__ void lattice(int sweep, int mode, int &px, int &py) {
    if (sweep == 0) {
        if (mode == 2) {
            px = 11;
            py = 11;
        } else if (mode == 1) {
            px = 5;
            py = 7;
        } else {
            px = 3;
            py = 6;
        }
    } else if (sweep == 1) {
        px = 3;
        py = 12;
    } else {
        px = 3;
        py = 1;
    }
}

// block-wide exclusive scan of one int per thread; returns the exclusive prefix,
// *total = block sum. scratch: >= 33 ints of shared memory.
__device__ __forceinline__ int block_excl_scan(int v, int *scratch, int *total) {
    int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
    int inc = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int n = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += n;
    }
    if (lane == 31) scratch[wid] = inc;
    __syncthreads();
    if (wid == 0) {
        int s = (lane < nw) ? scratch[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            int n = __shfl_up_sync(0xffffffffu, s, o);
            if (lane >= o) s += n;
        }
        if (lane < nw) scratch[lane] = s;  // inclusive warp totals
    }
    __syncthreads();
    int before = (wid > 0) ? scratch[wid - 1] : 0;
    *total = scratch[nw - 1];
    __syncthreads();
    return before + inc - v;
}

// write the particles of one spawn event (world.cpp:1110-1119,1222,1298)
__device__ void emit_spawns(const WorldDev &w, const SpawnEv &ev, uint32_t cp, uint32_t rank0, int base) {
    int32_t base_amt = 0, extra = 0;
    if (ev.kind == 2) {
        base_amt = ev.sc / ev.n;
        extra = ev.sc % ev.n;
    }
    for (int i = 0; i < ev.n; i++) {
        int slot = base + i;
        if (slot >= w.stage_cap) {
            atomicOr(w.err, ERR_SPAWN_CAP);
            return;
        }
        SpawnRec r;
        r.cp = cp;
        r.rank = rank0 + (uint32_t)i;
        r.x = (float)ev.x;
        r.y = (float)ev.y;
        r.id = ev.id;
        r.colour = ev.col;
        r.pad = 0;
        if (ev.kind == 1) {
            r.vx = ev.vx;
            r.vy = ev.vy;
            r.ay = 0.1f;
            r.scalar = ev.sc;
            r.flags = ev.fl;
            r.bits = 0;
            r.lifetime = 0;
            r.fade = 60;
        } else if (ev.kind == 3) {
            r.vx = ev.vx;
            r.vy = ev.vy;
            r.ay = 0.01f;
            r.scalar = ev.sc;
            r.flags = ev.fl;
            r.bits = 2;
            r.lifetime = 30;
            r.fade = 10;
        } else {
            uint32_t d0 = draw_k(ev.ck, ev.k0 + 2u * (uint32_t)i), d1 = draw_k(ev.ck, ev.k0 + 2u * (uint32_t)i + 1u);
            r.vx = (float)((int)(d0 % 10) - 5) / 30.0f;
            r.vy = (float)(-((int)(d1 % 2) + 3)) / 10.0f + 1.0f;
            r.ay = 0.1f;
            r.scalar = base_amt + (i < extra ? 1 : 0);
            r.flags = 0;
            r.bits = 0;
            r.lifetime = 0;
            r.fade = 60;
        }
        w.stage[slot] = r;
    }
}

// -------------------------------------------------------------- the kernel
// items: (world << 20) | chunk slot within the colour; iter, tk select the pass.
template <int HALO>
__global__ void __launch_bounds__(1024, 1)
    k_colour_pass(const WorldDev *__restrict__ worlds, const uint32_t *__restrict__ items, int n_items, int iter, int tk,
                  const MatTable *__restrict__ mt) {
    extern __shared__ __align__(16) unsigned char smem[];
    uint32_t *s_ma = (uint32_t *)smem;                 // [MAXMAT]
    float *s_md = (float *)(s_ma + MAXMAT);            // [MAXMAT]
    long long *s_led = (long long *)(s_md + MAXMAT);   // [LED_ROWS * 64]
    int *s_scan = (int *)(s_led + LED_ROWS * 64);      // [40]
    unsigned char *planes = (unsigned char *)(s_scan + 40);

    const int tid = threadIdx.x, T = blockDim.x;
    for (int i = tid; i < MAXMAT; i += T) {
        s_ma[i] = (i < mt->n) ? mt->a[i] : 0u;
        s_md[i] = (i < mt->n) ? mt->density[i] : 0.f;
    }
    for (int i = tid; i < LED_ROWS * 64; i += T) s_led[i] = 0;
    __syncthreads();

    const int ox = tk % 2, oy = 1 - tk / 2;
    long long *led_g_last = nullptr;
    int32_t *err_last = nullptr;

    for (int it = blockIdx.x; it < n_items; it += gridDim.x) {
        const uint32_t item = __ldg(&items[it]);
        const WorldDev &w = worlds[item >> 20];
        const int slot = (int)(item & 0xFFFFF);
        if (led_g_last != w.ledger && led_g_last != nullptr) {
            // flush the shared ledger before switching worlds
            __syncthreads();
            for (int i = tid; i < LED_ROWS * 64; i += T) {
                long long v = s_led[i];
                if (v) atomicAdd((unsigned long long *)&led_g_last[(i / 64) * MAXMAT + (i % 64)], (unsigned long long)v);
                s_led[i] = 0;
            }
            __syncthreads();
        }
        led_g_last = w.ledger;
        err_last = w.err;
        if (iter >= w.cell_iter) continue;
        const int C = w.C, W = w.W, H = w.H;
        const int nb = (w.nCy - oy + 1) / 2;
        const int cx = (ox + 2 * (slot / nb)) * C, cy = (oy + 2 * (slot % nb)) * C;
        const uint32_t cp = (uint32_t)((iter * 4 + tk) * w.max_slots + slot);

        Tile Tl;
        Tl.RW = C + 2 * HALO;
        Tl.RHF = C + 2 * HALO;
        Tl.RHI = C + HALO + 10;
        Tl.x0 = cx - HALO;
        Tl.y0 = cy - HALO;
        Tl.W = W;
        Tl.H = H;
        Tl.ma = s_ma;
        Tl.md = s_md;
        Tl.df = w.df;
        Tl.id_solid = mt->id_solid;
        Tl.id_air = mt->id_air;
        Tl.err = w.err;
        const int nid = Tl.RW * Tl.RHI, nfull = Tl.RW * Tl.RHF;
        Tl.s_sc = (int32_t *)planes;
        Tl.s_col = (uint32_t *)(Tl.s_sc + nfull);
        Tl.s_id = (uint16_t *)(Tl.s_col + nfull);
        Tl.s_fl = (uint8_t *)(Tl.s_id + ((nid + 1) & ~1));

        // ---- stage material ids; decide skip and lattice mode from the chunk
        int active = 0, fire = 0;
        for (int i = tid; i < nid; i += T) {
            int ly = i / Tl.RW, lx = i - ly * Tl.RW;
            int gx = Tl.x0 + lx, gy = Tl.y0 + ly;
            uint16_t v = (uint16_t)mt->id_solid;
            if ((unsigned)gx < (unsigned)W && (unsigned)gy < (unsigned)H) {
                v = w.id[(size_t)gy * W + gx];
                if (gx >= cx && gx < cx + C && gy >= cy && gy < cy + C) {
                    if (mt_iter(s_ma[v]) > iter) active = 1;
                    if ((int)v == mt->id_fire) fire = 1;
                }
            }
            Tl.s_id[i] = v;
        }
        active = __syncthreads_or(active);
        fire = __syncthreads_or(fire);
        if (!active) {
            // every chunk cell has iterations <= iter: the pass only marks cells visited
            if (tid == 0) w.cp_count[cp] = 0;
            __syncthreads();
            continue;
        }
        for (int i = tid; i < nfull; i += T) {
            int ly = i / Tl.RW, lx = i - ly * Tl.RW;
            int gx = Tl.x0 + lx, gy = Tl.y0 + ly;
            if ((unsigned)gx < (unsigned)W && (unsigned)gy < (unsigned)H) {
                size_t g = (size_t)gy * W + gx;
                Tl.s_fl[i] = w.fl[g];
                Tl.s_sc[i] = w.sc[g];
                Tl.s_col[i] = w.col[g];
            } else {
                Tl.s_fl[i] = 0;
                Tl.s_sc[i] = 0;
                Tl.s_col[i] = 0xff0000u;
            }
        }
        __syncthreads();

        const int mode = mt->has_inter ? 2 : (fire ? 1 : 0);
        const int cw = min(C, W - cx), chh = min(C, H - cy);
        int running = 0;  // spawns emitted so far by this chunk-pass (thread 0's view is authoritative)
        Ctx c;
        c.iter = iter;
        c.mt = mt;
        c.led_s = s_led;
        c.led_g = w.ledger;
        c.ma = s_ma;
        for (int sweep = 0; sweep < 3; sweep++) {
            c.pk = pass_key(w.seed, *w.tick, (uint32_t)(iter * 3 + sweep));
            int px, py;
            lattice(sweep, mode, px, py);
            for (int ry = py - 1; ry >= 0; ry--) {
                for (int rx = 0; rx < px; rx++) {
                    const int nx = (C - rx + px - 1) / px, ny = (C - ry + py - 1) / py;
                    const int total = nx * ny;
                    for (int base = 0; base < total; base += T) {
                        const int i = base + tid;
                        c.ev.n = 0;
                        if (i < total) {
                            const int dy = ry + (i / nx) * py, dx = rx + (i % nx) * px;
                            if (dx < cw && dy < chh) {
                                if (sweep == 0)
                                    rule_a(Tl, c, cx + dx, cy + dy);
                                else if (sweep == 1)
                                    rule_b(Tl, c, cx + dx, cy + dy);
                                else
                                    rule_c(Tl, c, cx + dx, cy + dy);
                            }
                        }
                        if (sweep == 0) {
                            if (__syncthreads_or(c.ev.n > 0)) {
                                int tot;
                                int ex = block_excl_scan(c.ev.n, s_scan, &tot);
                                if (tid == 0) s_scan[36] = atomicAdd(w.stage_count, tot);
                                __syncthreads();
                                int gbase = s_scan[36];
                                if (c.ev.n > 0) emit_spawns(w, c.ev, cp, (uint32_t)(running + ex), gbase + ex);
                                running += tot;
                            }
                        }
                    }
                    __syncthreads();
                }
            }
        }

        // ---- write back the cells this CTA changed (full-state rows inside the world)
        for (int i = tid; i < nfull; i += T) {
            uint16_t v = Tl.s_id[i];
            if (!(v & DIRTY)) continue;
            int ly = i / Tl.RW, lx = i - ly * Tl.RW;
            int gx = Tl.x0 + lx, gy = Tl.y0 + ly;
            if ((unsigned)gx < (unsigned)W && (unsigned)gy < (unsigned)H) {
                size_t g = (size_t)gy * W + gx;
                w.id[g] = (uint16_t)(v & 0x7FFF);
                w.fl[g] = (uint8_t)(Tl.s_fl[i] & (uint8_t)~VISITED);
                w.sc[g] = Tl.s_sc[i];
                w.col[g] = Tl.s_col[i];
            }
        }
        if (tid == 0) w.cp_count[cp] = running;
        __syncthreads();
    }
    (void)err_last;
    if (led_g_last) {
        __syncthreads();
        for (int i = tid; i < LED_ROWS * 64; i += T) {
            long long v = s_led[i];
            if (v) atomicAdd((unsigned long long *)&led_g_last[(i / 64) * MAXMAT + (i % 64)], (unsigned long long)v);
        }
    }
}

size_t colour_pass_smem(int C, int halo) {
    size_t RW = (size_t)C + 2 * halo, RHF = (size_t)C + 2 * halo, RHI = (size_t)C + halo + 10;
    size_t nid = RW * RHI, nfull = RW * RHF;
    size_t head = MAXMAT * 4 + MAXMAT * 4 + LED_ROWS * 64 * 8 + 40 * 4;
    return head + nfull * 4 + nfull * 4 + ((nid + 1) & ~(size_t)1) * 2 + nfull;
}

cudaError_t launch_colour_pass(const WorldDev *worlds, const uint32_t *items, int n_items, int iter, int tk,
                               const MatTable *mt, int halo, int C, int threads, int grid, cudaStream_t s) {
    size_t sm = colour_pass_smem(C, halo);
    if (n_items <= 0) return cudaSuccess;
    if (grid <= 0 || grid > n_items) grid = n_items;
    // opt in to the full shared-memory carve-out once per process
    static size_t set5 = 0, set2 = 0;
    if (halo == 5) {
        if (set5 < sm) {
            cudaFuncSetAttribute(k_colour_pass<5>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
            set5 = sm;
        }
        k_colour_pass<5><<<grid, threads, sm, s>>>(worlds, items, n_items, iter, tk, mt);
    } else {
        if (set2 < sm) {
            cudaFuncSetAttribute(k_colour_pass<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
            set2 = sm;
        }
        k_colour_pass<2><<<grid, threads, sm, s>>>(worlds, items, n_items, iter, tk, mt);
    }
    return cudaGetLastError();
}

}  // namespace fse
