// fse_pack.cu -- the chunk .pack codec: Chunk::ChunkWrite / Chunk::ChunkRead
// (source/engine/chunk.cpp:219-330 and 68-200) for every 128 x 128 chunk of a
// device world.
//
// A .pack file is the chunk's i8 generation phase, four ints -- src_size
// (128*128*2 MaterialInstanceData records of 12 bytes: {u32 index, u32 color,
// i16 temperature, 2 bytes of padding}, chunk.hpp:26-30, tiles then layer2),
// the size of its LZ4 block, src_size2 (the 128*128 u32 background) and the size
// of that block -- then the two LZ4 blocks (the block format of the vendored
// LZ4 1.9.4, source/libs/lz4). This world has no second layer and no background:
// they are written as zeros and skipped on reading.
//
// Writing. k_pack_stage lays the tile records of a group of chunks out in HBM;
// k_lz4_parse / k_lz4_plan / k_lz4_emit compress each block, one warp per
// 24 KB segment (see seg_run). The encoder is this
// project's own: at each byte p it takes the longest run buf[p + i] ==
// buf[p + i - d] over 16 fixed distances d (ties to the nearer) when it is at
// least 4 bytes, else p is a literal -- the distances are multiples of 4 and of
// the 12-byte record, and one or two chunk rows (1536 bytes) back with the
// diagonal neighbours. The warp tests 32 positions at once for a 4-byte match
// and extends all candidate runs 128 bytes at a time, reading the block through
// an 8 KB shared-memory window that slides along (3 KB behind the position, for
// the farthest distance); runs whose remaining bytes lie in the zero second
// layer on both sides are extended to the end at once.
// On generated worlds the blocks come out smaller than those of the reference's
// LZ4_compress_fast(..., 10). k_pack_assemble writes headers and blocks.
//
// Reading. k_lz4_decode gives each block a CTA of two warps: the block is loaded
// whole into shared memory, warp 0 parses its sequences (tokens, lengths, offsets)
// into one half of a queue while warp 1 copies the sequences of the other half, and
// matches whose offset fits a shared-memory ring of the latest output are copied
// from it (others from HBM). Blocks longer than the shared-memory cap are decoded
// by one warp through a window of the input. Every length and offset is checked
// against both buffers: a malformed block yields a negative status and no access
// out of bounds. k_unpack_check
// rejects material indices outside the table; k_unpack_scatter writes id, colour
// and temperature into the planes (a SOUP tile's amount is the MaterialInstance
// default 2.0, game_datastruct.hpp:216).
#include <cuda_runtime.h>

#include <algorithm>
#include <vector>

#include "fse_host.cuh"
#include "fse_internal.cuh"

namespace fse {
namespace {

constexpr int PK_EDGE = 128;
constexpr int PK_CELLS = PK_EDGE * PK_EDGE;
constexpr int PK_TILES = PK_CELLS * 12;     // tile records of one chunk
constexpr int PK_SRC1 = PK_CELLS * 2 * 12;  // tiles + layer2
constexpr int PK_SRC2 = PK_CELLS * 4;       // background
constexpr int PK_HEADER = 17;
constexpr int PK_GROUP = 1024;  // chunks per device pass (bounds the scratch)
__host__ __device__ constexpr int lz4_bound(int n) { return n + n / 255 + 16; }
constexpr int PK_SLOT1 = (lz4_bound(PK_SRC1) + 15) & ~15;
constexpr int PK_SLOT2 = (lz4_bound(PK_SRC2) + 15) & ~15;

__constant__ int c_dist[16] = {4, 8, 12, 16, 20, 24, 36, 48, 60, 72, 84, 96, 1524, 1536, 1548, 3072};

constexpr unsigned FULL = 0xffffffffu;

// ------------------------------------------------------------------ stage
__global__ void k_pack_stage(const WorldDev *__restrict__ wd, const MatTable *__restrict__ mt, uint32_t *stage,
                             int chunk0, int n_chunks) {
    const WorldDev &w = *wd;
    const int ncx = (w.W + PK_EDGE - 1) / PK_EDGE;
    const long long total = (long long)n_chunks * PK_CELLS;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
         e += (long long)gridDim.x * blockDim.x) {
        const int c = (int)(e / PK_CELLS), j = (int)(e - (long long)c * PK_CELLS);
        const int k = chunk0 + c;
        const int x = (k % ncx) * PK_EDGE + (j % PK_EDGE), y = (k / ncx) * PK_EDGE + (j / PK_EDGE);
        uint32_t id = 0, col = 0, tw = 0;
        if (x < w.W && y < w.H) {
            const size_t i = (size_t)y * w.W + x;
            id = w.id[i];
            col = w.col[i];
            const int16_t t = mt_type(mt->a[id]) == T_SOUP ? (w.tp ? w.tp[i] : (int16_t)0) : (int16_t)w.sc[i];
            tw = (uint32_t)(uint16_t)t;  // i16 temperature, then 2 bytes of padding (0)
        }
        uint32_t *r = stage + (size_t)c * (PK_TILES / 4) + (size_t)j * 3;
        r[0] = id;
        r[1] = col;
        r[2] = tw;
    }
}

// ----------------------------------------------------------------- encode
constexpr int ENC_WIN = 8192;  // bytes of the block a warp keeps in shared memory
constexpr int ENC_WARPS = 4;
constexpr int ENC_BACK = 3072 + 32;  // the farthest distance and a word of slack

// The block's bytes: buf[0, T) from HBM (4-byte aligned), zeros from T to n. The
// warp reads them through a window of shared memory, [wb, wb + ENC_WIN), which
// need() moves (all lanes agree on wb) so that it covers the bytes a step reads.
struct Src {
    const uint32_t *w;  // T / 4 words
    int T;
    uint32_t *sw;  // the window, ENC_WIN / 4 words
    int wb;        // a multiple of 4
    __device__ __forceinline__ uint32_t gword(int i) const { return (4 * i < T) ? __ldg(w + i) : 0u; }
    __device__ __forceinline__ void fill(int at) {
        __syncwarp();
        wb = at;
        const int i0 = at >> 2;
        for (int i = threadIdx.x & 31; i < ENC_WIN / 4; i += 32) sw[i] = gword(i0 + i);
        __syncwarp();
    }
    // the window covers [lo, hi) afterwards (hi - lo <= ENC_WIN - 4)
    __device__ __forceinline__ void need(int lo, int hi) {
        if (lo < wb || hi > wb + ENC_WIN) fill(max(lo, 0) & ~3);
    }
    __device__ __forceinline__ uint32_t word(int i) const { return sw[i - (wb >> 2)]; }
    __device__ __forceinline__ uint32_t load4(int p) const {
        const int i = p >> 2, s = (p & 3) * 8;
        return __funnelshift_r(word(i), word(i + 1), s);
    }
    __device__ __forceinline__ uint32_t byte(int p) const { return (word(p >> 2) >> ((p & 3) * 8)) & 0xFFu; }
    __device__ __forceinline__ uint32_t gbyte(int p) const { return (gword(p >> 2) >> ((p & 3) * 8)) & 0xFFu; }
};

// one sequence: literals [ls, ls + nl), then (when ml > 0) a match of ml bytes at
// distance off; returns the new output position, or -1 when it would not fit
__device__ int emit_seq(Src &s, uint8_t *dst, int op, int cap, int ls, int nl, int off, int ml) {
    const int lane = threadIdx.x & 31;
    const int mcode = ml > 0 ? ml - 4 : 0;
    const int lext = nl >= 15 ? (nl - 15) / 255 + 1 : 0;
    const int mext = (ml > 0 && mcode >= 15) ? (mcode - 15) / 255 + 1 : 0;
    const int need = 1 + lext + nl + (ml > 0 ? 2 + mext : 0);
    if (need > cap - op) return -1;
    if (lane == 0) {
        dst[op] = (uint8_t)(((nl < 15 ? nl : 15) << 4) | (ml > 0 ? (mcode < 15 ? mcode : 15) : 0));
        int o = op + 1;
        if (nl >= 15) {
            int v = nl - 15;
            for (; v >= 255; v -= 255) dst[o++] = 255;
            dst[o++] = (uint8_t)v;
        }
        o += nl;
        if (ml > 0) {
            dst[o++] = (uint8_t)(off & 255);
            dst[o++] = (uint8_t)(off >> 8);
            if (mcode >= 15) {
                int v = mcode - 15;
                for (; v >= 255; v -= 255) dst[o++] = 255;
                dst[o++] = (uint8_t)v;
            }
        }
    }
    const int lo = op + 1 + lext;
    if (nl + 8 <= ENC_WIN - 8) {  // through the window
        s.need(ls, ls + nl + 8);
        for (int i = lane; i < nl; i += 32) dst[lo + i] = (uint8_t)s.byte(ls + i);
    } else {
        for (int i = lane; i < nl; i += 32) dst[lo + i] = (uint8_t)s.gbyte(ls + i);
    }
    return op + need;
}

// Segments: the parse is the sequential greedy parse with every match ending at
// the latest at the end of the ENC_SEG-byte segment it starts in, so each segment
// can be parsed by its own warp (a match still refers to any earlier byte of the
// block). A segment's first sequence takes over the literals left at the end of
// the segments before it, so writing needs each segment's start of literals
// (its `anchor`): k_lz4_parse records per segment what writing it costs apart
// from that first literal run, and its matches (position, distance, length; up to
// ENC_REC of them), k_lz4_plan carries the anchors and places the segments, and
// k_lz4_emit writes the recorded matches (a segment with more parses again).
constexpr int ENC_SEG = 24576;
constexpr int ENC_REC = 1024;  // matches recorded per segment
struct SegInfo {
    int m;       // sequences with a match that start in the segment
    int first;   // the position of its first match (when m > 0)
    int last;    // the position after its last match (when m > 0)
    int fixed;   // bytes of its sequences apart from the first one's token, length bytes and literals
};
__host__ __device__ __forceinline__ int len_bytes(int v) { return v >= 15 ? (v - 15) / 255 + 1 : 0; }

// parse (EMIT = false: fill *info) or parse and write (EMIT = true: from dst[op],
// literals starting at `anchor`) the segment [a, b) of an n-byte block; returns
// the output position after the segment's sequences (EMIT) or -1 when they would
// not fit in cap, and leaves in `anchor` the start of the literals after them
template <bool EMIT>
__device__ int seg_run(Src &s, int n, int a, int b, int &anchor, uint8_t *dst, int op, int cap, SegInfo *info,
                       uint2 *rec) {
    const int lane = threadIdx.x & 31;
    const int mflimit = n - 12, mend = n - 5;
    const int lim = min(mend, b);       // a match ends at the latest here
    const int stop = min(b, mflimit + 1);  // matches start before here
    int p = a, m = 0, first = -1, fixed = 0;
    if (!EMIT) anchor = a;
    while (p < stop && op >= 0) {
        // candidates at p itself: lane k < 16 tests distance k
        s.need(p - ENC_BACK, p + 136);
        int q0 = p;
        unsigned cm = __ballot_sync(FULL, lane < 16 && c_dist[lane & 15] <= p && p + 4 <= lim &&
                                              s.load4(p) == s.load4(p - c_dist[lane & 15]));
        if (!cm) {
            // none: the first position of [p + 1, p + 33) with a 4-byte match at some distance
            const int q = p + 1 + lane;
            unsigned m = 0;
            if (q < stop && q + 4 <= lim) {
                const uint32_t v = s.load4(q);
#pragma unroll
                for (int k = 0; k < 16; k++) {
                    const int d = c_dist[k];
                    if (d <= q && s.load4(q - d) == v) m |= 1u << k;
                }
            }
            const unsigned any = __ballot_sync(FULL, m != 0);
            if (!any) {
                p += 33;
                continue;
            }
            const int f = __ffs(any) - 1;
            q0 = p + 1 + f;
            cm = __shfl_sync(FULL, m, f);
            s.need(q0 - ENC_BACK, q0 + 136);
        }
        // run lengths: lane k extends candidate k by itself up to 128 bytes, 4 at a time
        int L = 0;
        bool open = false;
        if (lane < 16 && ((cm >> lane) & 1u)) {
            const int d = c_dist[lane];
            const int top = min(lim - q0, 128);
            L = 4;
            while (L < top) {
                const int take = min(4, top - L);
                uint32_t diff = s.load4(q0 + L) ^ s.load4(q0 + L - d);
                if (take < 4) diff |= 0xffffffffu << (8 * take);
                if (diff) {
                    L += (__ffs(diff) - 1) >> 3;
                    break;
                }
                L += 4;
            }
            open = L == 128 && q0 + 128 < lim;
        }
        unsigned alive = __ballot_sync(FULL, open);
        if (alive) {
            // runs of 128 bytes and more: the whole warp extends them, 128 bytes per step
            int len[16];
#pragma unroll
            for (int k = 0; k < 16; k++) len[k] = 0;
            for (int base = 128; alive; base += 128) {
                s.need(q0 + base - ENC_BACK, q0 + base + 136);
                const int x = q0 + base + 4 * lane;
                const int vb = min(max(lim - x, 0), 4);  // bytes of this lane before lim
                const uint32_t over = vb == 4 ? 0u : (vb == 0 ? 0xffffffffu : (0xffffffffu << (8 * vb)));
                const uint32_t av = s.load4(x);
#pragma unroll
                for (int k = 0; k < 16; k++) {
                    if (!(alive & (1u << k))) continue;
                    const int d = c_dist[k];
                    if (q0 + base - d >= s.T) {  // both sides in the zero tail from here on: equal up to lim
                        len[k] = lim - q0;
                        alive &= ~(1u << k);
                        continue;
                    }
                    const uint32_t diff = (av ^ s.load4(x - d)) | over;
                    const unsigned miss = __ballot_sync(FULL, diff != 0);
                    if (miss) {
                        const int fl = __ffs(miss) - 1;
                        const uint32_t df = __shfl_sync(FULL, diff, fl);
                        len[k] = base + 4 * fl + ((__ffs(df) - 1) >> 3);
                        alive &= ~(1u << k);
                    }
                }
            }
#pragma unroll
            for (int k = 0; k < 16; k++)
                if (open && lane == k) L = len[k];
        }
        // the longest run, ties to the nearer distance (smaller k)
        const unsigned key = (lane < 16 && ((cm >> lane) & 1u)) ? ((unsigned)L << 4) | (unsigned)(15 - lane) : 0u;
        const unsigned top_key = __reduce_max_sync(FULL, key);
        const int best = (int)(top_key >> 4);
        const int bk = 15 - (int)(top_key & 15u);
        const int bd = c_dist[bk];
        if (EMIT) {
            op = emit_seq(s, dst, op, cap, anchor, q0 - anchor, bd, best);
        } else {
            if (lane == 0 && m < ENC_REC) rec[m] = make_uint2(((unsigned)q0 << 4) | (unsigned)bk, (unsigned)best);
            const int mpart = 2 + len_bytes(best - 4);
            if (m == 0) {
                first = q0;
                fixed += mpart;
            } else {
                const int nl = q0 - anchor;
                fixed += 1 + len_bytes(nl) + nl + mpart;
            }
        }
        m++;
        p = q0 + best;
        anchor = p;
    }
    if (!EMIT && lane == 0) *info = SegInfo{m, first, anchor, fixed};
    return op;
}

// phase 1: one warp per (block, segment)
__global__ void __launch_bounds__(ENC_WARPS * 32) k_lz4_parse(const uint32_t *__restrict__ stage, int T, int n,
                                                             int n_blocks, SegInfo *info, uint2 *rec) {
    __shared__ uint32_t s_win[ENC_WARPS][ENC_WIN / 4];
    const int nseg = (n + ENC_SEG - 1) / ENC_SEG;
    const int u = blockIdx.x * ENC_WARPS + threadIdx.x / 32;
    if (u >= n_blocks * nseg) return;
    const int b = u / nseg, k = u - b * nseg;
    Src s{stage + (size_t)b * (T / 4), T, s_win[threadIdx.x / 32], 0};
    s.fill(max(k * ENC_SEG - ENC_BACK, 0) & ~3);
    int anchor = 0;
    seg_run<false>(s, n, k * ENC_SEG, min(n, (k + 1) * ENC_SEG), anchor, nullptr, 0, 0, info + u,
                   rec + (size_t)u * ENC_REC);
}

// phase 2: one thread per block: each segment's first literal start and output
// position, and the block size (-1 when it would exceed cap)
__global__ void k_lz4_plan(const SegInfo *__restrict__ info, int n, int n_blocks, int cap, int *seg_anchor,
                           int *seg_out, int *sizes) {
    const int nseg = (n + ENC_SEG - 1) / ENC_SEG;
    for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < n_blocks; b += gridDim.x * blockDim.x) {
        long long op = 0;
        int anchor = 0;
        for (int k = 0; k < nseg; k++) {
            const SegInfo &g = info[b * nseg + k];
            seg_anchor[b * nseg + k] = anchor;
            seg_out[b * nseg + k] = (int)min(op, (long long)cap);
            if (g.m > 0) {
                const int nl = g.first - anchor;
                op += 1 + len_bytes(nl) + nl + g.fixed;
                anchor = g.last;
            }
        }
        const int nl = n - anchor;  // the last sequence: literals only
        op += 1 + len_bytes(nl) + nl;
        sizes[b] = op <= cap ? (int)op : -1;
    }
}

// phase 3: one warp per (block, segment); the last segment also writes the final
// literals
__global__ void __launch_bounds__(ENC_WARPS * 32) k_lz4_emit(const uint32_t *__restrict__ stage, int T, int n,
                                                            int n_blocks, const int *__restrict__ seg_anchor,
                                                            const int *__restrict__ seg_out,
                                                            const int *__restrict__ sizes, uint8_t *out, int slot,
                                                            const SegInfo *__restrict__ info,
                                                            const uint2 *__restrict__ rec) {
    __shared__ uint32_t s_win[ENC_WARPS][ENC_WIN / 4];
    const int nseg = (n + ENC_SEG - 1) / ENC_SEG;
    const int u = blockIdx.x * ENC_WARPS + threadIdx.x / 32;
    if (u >= n_blocks * nseg) return;
    const int b = u / nseg, k = u - b * nseg;
    if (sizes[b] < 0) return;  // does not fit: nothing is written (cannot happen within the bound)
    Src s{stage + (size_t)b * (T / 4), T, s_win[threadIdx.x / 32], 0};
    s.fill(max(k * ENC_SEG - ENC_BACK, 0) & ~3);
    uint8_t *dst = out + (size_t)b * slot;
    const int a = k * ENC_SEG, e = min(n, (k + 1) * ENC_SEG);
    // the segment writes [seg_out[u], its end); it ends where the next one starts
    const int end = (k + 1 < nseg) ? seg_out[u + 1] : sizes[b];
    int anchor = seg_anchor[u];
    int op = seg_out[u];
    const int m = info[u].m;
    if (m <= ENC_REC) {
        // the recorded matches, with their literals
        const uint2 *r = rec + (size_t)u * ENC_REC;
        for (int i = 0; i < m && op >= 0; i++) {
            const uint2 v = r[i];
            const int q0 = (int)(v.x >> 4), L = (int)v.y;
            op = emit_seq(s, dst, op, end, anchor, q0 - anchor, c_dist[v.x & 15u], L);
            anchor = q0 + L;
        }
    } else {
        op = seg_run<true>(s, n, a, e, anchor, dst, op, end, nullptr, nullptr);
    }
    if (k + 1 == nseg && op >= 0) op = emit_seq(s, dst, op, end, anchor, n - anchor, 0, 0);  // the last sequence
}

// ---------------------------------------------------------------- assemble
// chunk c of the group: phase, sizes, block 1 (slot c), block 2 (shared)
__global__ void k_pack_assemble(const uint8_t *__restrict__ enc1, int slot1, const int *__restrict__ size1,
                                const uint8_t *__restrict__ enc2, int size2, const long long *__restrict__ offs,
                                int n_chunks, int8_t phase, uint8_t *out) {
    for (int c = blockIdx.x; c < n_chunks; c += gridDim.x) {
        uint8_t *o = out + offs[c];
        const int n1 = size1[c];
        if (threadIdx.x == 0) {
            const int32_t hd[4] = {PK_SRC1, n1, PK_SRC2, size2};
            o[0] = (uint8_t)phase;
            const uint8_t *hb = reinterpret_cast<const uint8_t *>(hd);
            for (int i = 0; i < 16; i++) o[1 + i] = hb[i];
        }
        const uint8_t *e1 = enc1 + (size_t)c * slot1;
        for (int i = threadIdx.x; i < n1; i += blockDim.x) o[PK_HEADER + i] = e1[i];
        for (int i = threadIdx.x; i < size2; i += blockDim.x) o[PK_HEADER + n1 + i] = enc2[i];
    }
}

// ------------------------------------------------------------------ decode
constexpr int DEC_WIN = 2048;   // input window per warp
constexpr int DEC_RING = 8192;  // latest output per warp

// the input window holds src[wb, wb + DEC_WIN) (clipped to n); reads outside it
// refill it at the requested position
struct DecIn {
    const uint8_t *src;
    int n, wb;
    uint8_t *win;
    __device__ __forceinline__ void fill(int at) {
        __syncwarp();
        wb = at;
        const int lane = threadIdx.x & 31;
        for (int i = lane; i < DEC_WIN && at + i < n; i += 32) win[i] = src[at + i];
        __syncwarp();
    }
    __device__ __forceinline__ int get(int ip) {  // 0 <= ip < n
        if (ip < wb || ip >= wb + DEC_WIN) fill(ip);
        return win[ip - wb];
    }
};

__device__ int warp_lz4_decode(const uint8_t *src, int n, uint8_t *dst, int cap, uint8_t *win, uint8_t *ring) {
    const int lane = threadIdx.x & 31;
    DecIn in{src, n, 0, win};
    in.fill(0);
    int ip = 0, op = 0;
    for (;;) {
        if (ip >= n) return -1;
        const int token = in.get(ip++);
        int ll = token >> 4;
        if (ll == 15) {
            int b;
            do {
                if (ip >= n) return -2;
                b = in.get(ip++);
                ll += b;
                if (ll > cap) return -3;
            } while (b == 255);
        }
        if (ll > n - ip || ll > cap - op) return -3;
        // literals: from the window when they lie in it, else from HBM
        const bool inwin = ip >= in.wb && ip + ll <= in.wb + DEC_WIN && ip + ll <= n;
        for (int i = lane; i < ll; i += 32) {
            const uint8_t v = inwin ? in.win[ip - in.wb + i] : src[ip + i];
            dst[op + i] = v;
            ring[(op + i) & (DEC_RING - 1)] = v;
        }
        ip += ll;
        op += ll;
        if (ip == n) return op;  // the last sequence: literals only
        if (n - ip < 2) return -4;
        const int off = in.get(ip) | (in.get(ip + 1) << 8);
        ip += 2;
        if (off == 0 || off > op) return -5;
        int ml = token & 15;
        if (ml == 15) {
            int b;
            do {
                if (ip >= n) return -6;
                b = in.get(ip++);
                ml += b;
                if (ml > cap) return -7;
            } while (b == 255);
        }
        ml += 4;
        if (ml > cap - op) return -7;
        __syncwarp();  // the bytes the match reads are written
        // byte j of the match repeats byte (j mod off) of the `off` bytes before it, so
        // no byte of a round depends on another one of the same round. From the ring,
        // a round copies at most DEC_RING - off bytes, so that it overwrites no ring
        // slot it reads; the next round reads the `off` bytes before it again.
        const bool from_ring = off <= DEC_RING - 32;
        for (int done = 0; done < ml;) {
            const int m = from_ring ? min(ml - done, DEC_RING - off) : ml - done;
            const int base = op + done;
            // sidx = j mod off, kept without a division in the loop: j grows by 32,
            // which is step = 32 mod off
            int sidx = off >= 32 ? lane : lane % off;
            const int step = off >= 32 ? 32 : 32 % off;
            for (int j = lane; j < m; j += 32) {
                const int from = base - off + sidx;
                const uint8_t v = from_ring ? ring[from & (DEC_RING - 1)] : dst[from];
                dst[base + j] = v;
                ring[(base + j) & (DEC_RING - 1)] = v;
                sidx += step;
                if (sidx >= off) sidx -= off;
            }
            __syncwarp();
            done += m;
        }
        op += ml;
    }
}

// ---- the pipelined decoder: a whole block in shared memory, one warp parsing
// sequences into a double-buffered queue while the other copies them
constexpr int DEC_BATCH = 128;                // sequences per queue half
constexpr int DEC_CAP_MAX = 64 * 1024;        // largest block held whole in shared memory
constexpr int DEC_FIXED = 2 * DEC_BATCH * 16 + DEC_RING + 32;

// an extended length (LZ4's 255-continued bytes) read by the whole warp, 32 bytes
// per step: adds the bytes to len and moves ip past them; false when the input ends
// first or len passes cap
__device__ __forceinline__ bool ext_len(const uint8_t *c, int n, int &ip, int &len, int cap) {
    const int lane = threadIdx.x & 31;
    for (;;) {
        const int p = ip + lane;
        const int b = p < n ? (int)c[p] : -1;
        const unsigned stop = __ballot_sync(0xffffffffu, b != 255);
        if (!stop) {
            len += 255 * 32;
            ip += 32;
            if (len > cap) return false;
            continue;
        }
        const int k = __ffs(stop) - 1;
        const int bk = __shfl_sync(0xffffffffu, b, k);
        if (bk < 0) return false;
        len += 255 * k + bk;
        ip += k + 1;
        return len <= cap;
    }
}

// one sequence at ip (all lanes, same values): {literal start, literal length,
// offset, match length} in d; 1 = the last sequence (literals only), 0 = more,
// negative = malformed (the same conditions as warp_lz4_decode)
__device__ __forceinline__ int parse_seq(const uint8_t *c, const uint32_t *area32, int pad, int n, int cap, int &ip,
                                         int &op, int4 &d) {
    if (ip + 8 <= n) {
        // the common sequence from eight bytes at ip (three aligned words): at most
        // four literals, the offset and at most one extra match-length byte inside
        const int pos = pad + ip, w = pos >> 2, sh = (pos & 3) * 8;
        const uint32_t a = area32[w], b = area32[w + 1], e = area32[w + 2];
        const uint64_t v = ((uint64_t)__funnelshift_r(b, e, sh) << 32) | __funnelshift_r(a, b, sh);
        const int token = (int)(v & 255), ll = token >> 4, m4 = token & 15;
        const int x = m4 == 15 ? (int)((v >> (8 * (3 + ll))) & 255) : 0;
        if (ll <= 4 && x < 255) {
            if (ll > cap - op) return -3;
            d.x = ip + 1;
            d.y = ll;
            op += ll;
            const int off = (int)((v >> (8 * (1 + ll))) & 0xffff);
            if (off == 0 || off > op) return -5;
            const int ml = m4 + x + 4;
            ip += 3 + ll + (m4 == 15);
            if (ml > cap - op) return -7;
            d.z = off;
            d.w = ml;
            op += ml;
            return 0;
        }
    }
    if (ip >= n) return -1;
    const int token = c[ip++];
    int ll = token >> 4;
    if (ll == 15) {
        const int b = ip < n ? (int)c[ip] : -1;
        if (b >= 0 && b < 255) {
            ll += b;
            ip++;
        } else if (!ext_len(c, n, ip, ll, cap)) {
            return -3;
        }
    }
    if (ll > n - ip || ll > cap - op) return -3;
    d.x = ip;
    d.y = ll;
    ip += ll;
    op += ll;
    if (ip == n) {
        d.z = d.w = 0;
        return 1;
    }
    if (n - ip < 2) return -4;
    const int off = c[ip] | (c[ip + 1] << 8);
    ip += 2;
    if (off == 0 || off > op) return -5;
    int ml = token & 15;
    if (ml == 15) {
        const int b = ip < n ? (int)c[ip] : -1;
        if (b >= 0 && b < 255) {
            ml += b;
            ip++;
        } else if (!ext_len(c, n, ip, ml, cap)) {
            return -7;
        }
    }
    ml += 4;
    if (ml > cap - op) return -7;
    d.z = off;
    d.w = ml;
    op += ml;
    return 0;
}

// out[k0 + j] = src[spos + j] for j < len, by the warp, into the block's output
// and the ring. Source bytes are src8[pos & smask] (the ring: smask = DEC_RING - 1;
// linear buffers: -1); none of them is written by the copy. Runs of 128 bytes and
// more move as aligned 4-byte words of the output, each built from two aligned
// source words with a funnel shift; the rest bytewise.
__device__ __forceinline__ void copy_run(uint8_t *dst, uint8_t *ring, const uint8_t *src8, int smask, int k0, int spos,
                                         int len, int lane) {
    if (len < 128 || ((uintptr_t)dst & 3)) {
        for (int i = lane; i < len; i += 32) {
            const uint8_t v = src8[(spos + i) & smask];
            dst[k0 + i] = v;
            ring[(k0 + i) & (DEC_RING - 1)] = v;
        }
        return;
    }
    const int head = (4 - (k0 & 3)) & 3;
    const int nw = (len - head) >> 2;
    const int t0 = head + 4 * nw;  // first tail byte, relative to k0
    if (lane < head) {
        const uint8_t v = src8[(spos + lane) & smask];
        dst[k0 + lane] = v;
        ring[(k0 + lane) & (DEC_RING - 1)] = v;
    } else if (lane >= 4 && lane - 4 < len - t0) {
        const int j = t0 + lane - 4;
        const uint8_t v = src8[(spos + j) & smask];
        dst[k0 + j] = v;
        ring[(k0 + j) & (DEC_RING - 1)] = v;
    }
    const uint32_t *src32 = reinterpret_cast<const uint32_t *>(src8);
    uint32_t *dst32 = reinterpret_cast<uint32_t *>(dst);
    uint32_t *ring32 = reinterpret_cast<uint32_t *>(ring);
    const int s0 = spos + head, sh = (s0 & 3) * 8, sw = s0 >> 2, a0 = (k0 + head) >> 2;
    const int wmask = smask >> 2;  // -1 stays -1
    for (int i = lane; i < nw; i += 32) {
        const uint32_t w0 = src32[(sw + i) & wmask];
        const uint32_t v = sh ? __funnelshift_r(w0, src32[(sw + i + 1) & wmask], sh) : w0;
        dst32[a0 + i] = v;
        ring32[(a0 + i) & (DEC_RING / 4 - 1)] = v;
    }
}

// a match of ml bytes at op, offset off: out[op + j] = out[op + j - off]. Rounds
// copy from distance D, a multiple of off (every such distance repeats the
// pattern once op + j - D >= op - off), so no round reads what it writes: D starts
// at off and doubles while the source stays readable (from the ring: D <= half of
// it, so a round of at most D bytes overwrites no slot it reads).
__device__ __forceinline__ void copy_match(uint8_t *dst, uint8_t *ring, int op, int off, int ml, int lane) {
    const bool from_ring = off <= DEC_RING / 2;
    const uint8_t *s8 = from_ring ? ring : dst;
    const int smask = from_ring ? DEC_RING - 1 : -1;
    int D = off;
    for (int done = 0; done < ml;) {
        const int len = min(ml - done, D);
        copy_run(dst, ring, s8, smask, op + done, op + done - D, len, lane);
        __syncwarp();
        done += len;
        if (!from_ring || 2 * D <= DEC_RING / 2) D *= 2;
    }
}

// the parser warp: up to DEC_BATCH sequences into queue half `buf`; the count, whether
// more follow, and the result so far (decoded size or error) go to shared memory
__device__ __forceinline__ void parse_batch(const uint8_t *c, const uint32_t *area32, int pad, int n, int cap, int &ip,
                                            int &pop, int &state, int4 *desc, int *s_cnt, int *s_more, int *s_res,
                                            int buf, int lane) {
    int k = 0;
    while (k < DEC_BATCH && state == 0) {
        int4 d;
        const int r = parse_seq(c, area32, pad, n, cap, ip, pop, d);
        if (r < 0) {
            state = r;
            break;
        }
        if (lane == 0) desc[buf * DEC_BATCH + k] = d;
        k++;
        if (r == 1) state = 1;
    }
    if (lane == 0) {
        s_cnt[buf] = k;
        s_more[buf] = state == 0;
        *s_res = state < 0 ? state : pop;
    }
}

// block b: src + offs[b], lens[b] bytes -> out + b * slot; status[b] = decoded
// size or a negative error. 64 threads per block; blocks longer than cap_in bytes
// are decoded by warp_lz4_decode through a window.
__global__ void __launch_bounds__(64, 1) k_lz4_decode(const uint8_t *__restrict__ src, const long long *__restrict__ offs,
                                                   const int *__restrict__ lens, int n_blocks, int expect,
                                                   uint8_t *out, int slot, int *status, int cap_in) {
    extern __shared__ __align__(16) uint8_t dsm[];
    int4 *desc = reinterpret_cast<int4 *>(dsm);  // [2][DEC_BATCH]
    uint8_t *ring = dsm + 2 * DEC_BATCH * 16;
    uint8_t *area = ring + DEC_RING;             // cap_in + 32 bytes
    __shared__ int s_cnt[2], s_more[2], s_res;
    const int b = blockIdx.x;
    if (b >= n_blocks) return;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int n = lens[b];
    const uint8_t *in = src + offs[b];
    uint8_t *dst = out + (size_t)b * slot;
    if (n <= 0) {
        if (threadIdx.x == 0) status[b] = -8;
        return;
    }
    if (n > cap_in) {
        if (warp == 0) {
            const int r = warp_lz4_decode(in, n, dst, expect, area, ring);
            if (lane == 0) status[b] = r;
        }
        return;
    }
    // the block into shared memory: unaligned head and tail bytewise, the rest as
    // aligned 16-byte words (c[i] == in[i])
    const int head = min(n, (int)((16 - ((uintptr_t)in & 15)) & 15));
    const int nvec = (n - head) >> 4;
    uint8_t *c = area + ((16 - head) & 15);
    if (threadIdx.x < head) c[threadIdx.x] = in[threadIdx.x];
    for (int i = head + nvec * 16 + threadIdx.x; i < n; i += 64) c[i] = in[i];
    {
        const uint4 *vs = reinterpret_cast<const uint4 *>(in + head);
        uint4 *vd = reinterpret_cast<uint4 *>(c + head);
        int i = threadIdx.x;
        for (; i + 192 < nvec; i += 256) {
            const uint4 a0 = vs[i], a1 = vs[i + 64], a2 = vs[i + 128], a3 = vs[i + 192];
            vd[i] = a0;
            vd[i + 64] = a1;
            vd[i + 128] = a2;
            vd[i + 192] = a3;
        }
        for (; i < nvec; i += 64) vd[i] = vs[i];
    }
    __syncthreads();
    int ip = 0, pop = 0, state = 0;  // parser: input and output positions, 0 / 1 done / error
    const uint32_t *area32 = reinterpret_cast<const uint32_t *>(area);
    const int pad = (int)(c - area);  // c[i] == area[pad + i]
    if (warp == 0) parse_batch(c, area32, pad, n, expect, ip, pop, state, desc, s_cnt, s_more, &s_res, 0, lane);
    __syncthreads();
    int op = 0, buf = 0;  // copier: output position
    for (;;) {
        const int cnt = s_cnt[buf];
        const bool more = s_more[buf] != 0;
        if (warp == 0) {
            if (more)
                parse_batch(c, area32, pad, n, expect, ip, pop, state, desc, s_cnt, s_more, &s_res, buf ^ 1, lane);
        } else {
            for (int k = 0; k < cnt; k++) {
                const int4 d = desc[buf * DEC_BATCH + k];
                const int ll = d.y, off = d.z, ml = d.w, tot = ll + ml;
                if (tot <= 32 && off >= ml && off <= DEC_RING - 32) {
                    // one step: byte j is literal j, or the match's byte from j - off,
                    // which lies in this literal (>= 0) or before op (in the ring)
                    if (lane < tot) {
                        const int sidx = lane < ll ? lane : lane - off;
                        const uint8_t v = sidx >= 0 ? c[d.x + sidx] : ring[(op + sidx) & (DEC_RING - 1)];
                        dst[op + lane] = v;
                        ring[(op + lane) & (DEC_RING - 1)] = v;
                    }
                    __syncwarp();
                } else {
                    copy_run(dst, ring, area, -1, op, pad + d.x, ll, lane);
                    __syncwarp();  // the bytes the match reads are written
                    if (ml) copy_match(dst, ring, op + ll, off, ml, lane);
                }
                op += tot;
            }
        }
        if (!more) break;
        __syncthreads();
        buf ^= 1;
    }
    if (threadIdx.x == 0) status[b] = s_res;
}

// decode n_blocks blocks whose longest is max_len bytes
void launch_decode(const uint8_t *src, const long long *offs, const int *lens, int n_blocks, int max_len, int expect,
                   uint8_t *out, int slot, int *status, cudaStream_t s) {
    static bool attr = false;
    if (!attr) {
        cudaFuncSetAttribute(k_lz4_decode, cudaFuncAttributeMaxDynamicSharedMemorySize, DEC_FIXED + DEC_CAP_MAX);
        attr = true;
    }
    const int cap_in = std::max(DEC_WIN, std::min(DEC_CAP_MAX, (max_len + 15) & ~15));
    k_lz4_decode<<<n_blocks, 64, DEC_FIXED + cap_in, s>>>(src, offs, lens, n_blocks, expect, out, slot, status, cap_in);
}

// chunks whose records name a material outside the table: the lowest such chunk
__global__ void k_unpack_check(const uint8_t *__restrict__ rec, int slot, int n_chunks, int n_mat, int *first_bad) {
    const long long total = (long long)n_chunks * PK_CELLS;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
         e += (long long)gridDim.x * blockDim.x) {
        const int c = (int)(e / PK_CELLS), j = (int)(e - (long long)c * PK_CELLS);
        const uint8_t *r = rec + (size_t)c * slot + (size_t)j * 12;
        const uint32_t id = (uint32_t)r[0] | ((uint32_t)r[1] << 8) | ((uint32_t)r[2] << 16) | ((uint32_t)r[3] << 24);
        if (id >= (uint32_t)n_mat) atomicMin(first_bad, c);
    }
}

__global__ void k_unpack_scatter(const WorldDev *__restrict__ wd, const MatTable *__restrict__ mt,
                                 const uint8_t *__restrict__ rec, int slot, int chunk0, int n_chunks) {
    const WorldDev &w = *wd;
    const int ncx = (w.W + PK_EDGE - 1) / PK_EDGE;
    const long long total = (long long)n_chunks * PK_CELLS;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
         e += (long long)gridDim.x * blockDim.x) {
        const int c = (int)(e / PK_CELLS), j = (int)(e - (long long)c * PK_CELLS);
        const int k = chunk0 + c;
        const int x = (k % ncx) * PK_EDGE + (j % PK_EDGE), y = (k / ncx) * PK_EDGE + (j / PK_EDGE);
        if (x >= w.W || y >= w.H) continue;
        const uint8_t *r = rec + (size_t)c * slot + (size_t)j * 12;
        const uint32_t id = (uint32_t)r[0] | ((uint32_t)r[1] << 8) | ((uint32_t)r[2] << 16) | ((uint32_t)r[3] << 24);
        const uint32_t col = (uint32_t)r[4] | ((uint32_t)r[5] << 8) | ((uint32_t)r[6] << 16) | ((uint32_t)r[7] << 24);
        const int16_t t = (int16_t)(uint16_t)((uint32_t)r[8] | ((uint32_t)r[9] << 8));
        const size_t i = (size_t)y * w.W + x;
        w.id[i] = (uint16_t)id;
        w.col[i] = col;
        w.fl[i] = 0;
        w.df[i] = 0;
        if (mt_type(mt->a[id]) == T_SOUP) {
            w.sc[i] = w.f32 ? F_DEFAULT_BITS : Q_DEFAULT;  // MaterialInstance::fluidAmount = 2.0
            if (w.tp) w.tp[i] = t;
        } else {
            w.sc[i] = t;
        }
        if (w.dirty) w.dirty[i] = 1;
    }
}

// the three encoder phases for n_blocks blocks of n bytes (T of them staged)
void encode_blocks(const uint32_t *stage, int T, int n, int n_blocks, uint8_t *out, int slot, int *sizes,
                   SegInfo *info, int *anc, int *sout, uint2 *rec, cudaStream_t s) {
    const int units = n_blocks * ((n + ENC_SEG - 1) / ENC_SEG);
    const int grid = (units + ENC_WARPS - 1) / ENC_WARPS;
    k_lz4_parse<<<grid, ENC_WARPS * 32, 0, s>>>(stage, T, n, n_blocks, info, rec);
    k_lz4_plan<<<(n_blocks + 127) / 128, 128, 0, s>>>(info, n, n_blocks, slot, anc, sout, sizes);
    k_lz4_emit<<<grid, ENC_WARPS * 32, 0, s>>>(stage, T, n, n_blocks, anc, sout, sizes, out, slot, info, rec);
}
constexpr int ENC_MAXSEG = (PK_SRC1 + ENC_SEG - 1) / ENC_SEG;

int grid_for(long long work, int per) {
    return (int)std::max(1LL, std::min<long long>((work + per - 1) / per, sm_count() * 16LL));
}

}  // namespace
}  // namespace fse

using namespace fse;

extern "C" {

int fse_world_pack_bound(int width, int height, int64_t *out_bytes, int *out_chunks) {
    if (width <= 0 || height <= 0) return FSE_E_INVAL;
    const long long n = (long long)((width + PK_EDGE - 1) / PK_EDGE) * ((height + PK_EDGE - 1) / PK_EDGE);
    if (out_bytes) *out_bytes = n * (PK_HEADER + lz4_bound(PK_SRC1) + lz4_bound(PK_SRC2));
    if (out_chunks) *out_chunks = (int)n;
    return FSE_OK;
}

}  // extern "C"

namespace fse {
namespace {
// the world's pack scratch buffer k, at least `bytes` long (contents not kept)
template <typename T>
bool scratch(fse_world *w, int k, T **p, size_t bytes) {
    bytes = std::max<size_t>(bytes, 16);
    if (!w->pk_scr[k] || w->pk_scr_bytes[k] < bytes) {
        if (w->pk_scr[k]) cudaFree(w->pk_scr[k]);
        w->pk_scr[k] = nullptr;
        w->pk_scr_bytes[k] = 0;
        if (cudaMalloc(&w->pk_scr[k], bytes) != cudaSuccess) {
            w->pk_scr[k] = nullptr;
            *p = nullptr;
            return false;
        }
        w->pk_scr_bytes[k] = bytes;
    }
    *p = static_cast<T *>(w->pk_scr[k]);
    return true;
}
}  // namespace
}  // namespace fse

extern "C" {

int fse_world_trim(fse_world *w) {
    if (!w) return FSE_E_INVAL;
    FSE_CUDA_TRY(cudaStreamSynchronize(w->stream));
    for (int k = 0; k < 16; k++) {
        if (w->pk_scr[k]) cudaFree(w->pk_scr[k]);
        w->pk_scr[k] = nullptr;
        w->pk_scr_bytes[k] = 0;
    }
    if (w->tile_stage) cudaFree(w->tile_stage);
    w->tile_stage = nullptr;
    w->tile_stage_bytes = 0;
    return FSE_OK;
}

int fse_world_pack(fse_world *w, int generation_phase, uint8_t *out, int64_t cap, int64_t *offsets, int *out_n_chunks) {
    if (!w || !out || !offsets) return FSE_E_INVAL;
    int rc = ensure_materials_pushed();
    if (rc) return rc;
    int nch = 0;
    fse_world_pack_bound(w->W, w->H, nullptr, &nch);
    if (out_n_chunks) *out_n_chunks = nch;
    const int G = std::min(PK_GROUP, nch);
    uint32_t *stage = nullptr;
    uint8_t *enc1 = nullptr, *enc2 = nullptr, *dout = nullptr;
    int *sizes = nullptr, *anc = nullptr, *sout = nullptr;
    SegInfo *info = nullptr;
    uint2 *rec = nullptr;
    long long *doffs = nullptr;
    cudaStream_t s = w->stream;
    if (!scratch(w, 0, &stage, (size_t)G * PK_TILES) || !scratch(w, 1, &enc1, (size_t)G * PK_SLOT1) ||
        !scratch(w, 2, &enc2, PK_SLOT2) || !scratch(w, 3, &sizes, (size_t)(G + 1) * sizeof(int)) ||
        !scratch(w, 4, &doffs, (size_t)G * sizeof(long long)) ||
        !scratch(w, 5, &info, (size_t)G * ENC_MAXSEG * sizeof(SegInfo)) ||
        !scratch(w, 6, &anc, (size_t)G * ENC_MAXSEG * sizeof(int)) ||
        !scratch(w, 7, &sout, (size_t)G * ENC_MAXSEG * sizeof(int)) ||
        !scratch(w, 15, &rec, (size_t)G * ENC_MAXSEG * ENC_REC * sizeof(uint2)))
        return FSE_E_NOMEM;
    // the background block: 64 KB of zeros, the same for every chunk
    encode_blocks(stage, 0, PK_SRC2, 1, enc2, PK_SLOT2, sizes + G, info, anc, sout, rec, s);
    int size2 = 0;
    std::vector<int> sz(G);
    std::vector<long long> offs(G);
    int64_t pos = 0;
    for (int c0 = 0; c0 < nch && rc == FSE_OK; c0 += G) {
        const int g = std::min(G, nch - c0);
        k_pack_stage<<<grid_for((long long)g * PK_CELLS, 256), 256, 0, s>>>(w->d, g_dev_mt, stage, c0, g);
        encode_blocks(stage, PK_TILES, PK_SRC1, g, enc1, PK_SLOT1, sizes, info, anc, sout, rec, s);
        if (cudaMemcpyAsync(sz.data(), sizes, g * sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
            (c0 == 0 && cudaMemcpyAsync(&size2, sizes + G, sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess) ||
            cudaStreamSynchronize(s) != cudaSuccess) {
            rc = FSE_E_CUDA;
            break;
        }
        long long rel = 0;
        for (int c = 0; c < g; c++) {
            if (sz[c] < 0 || size2 < 0) rc = FSE_E_CUDA;
            offs[c] = rel;
            offsets[c0 + c] = pos + rel;
            rel += PK_HEADER + sz[c] + size2;
        }
        if (rc) break;
        if (pos + rel > cap) {
            rc = FSE_E_CAPACITY;
            break;
        }
        if (!scratch(w, 8, &dout, (size_t)rel)) {
            rc = FSE_E_NOMEM;
            break;
        }
        if (cudaMemcpyAsync(doffs, offs.data(), g * sizeof(long long), cudaMemcpyHostToDevice, s) != cudaSuccess) {
            rc = FSE_E_CUDA;
            break;
        }
        k_pack_assemble<<<std::min(g, sm_count() * 8), 256, 0, s>>>(enc1, PK_SLOT1, sizes, enc2, size2, doffs, g,
                                                                   (int8_t)generation_phase, dout);
        if (cudaMemcpyAsync(out + pos, dout, (size_t)rel, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
            cudaStreamSynchronize(s) != cudaSuccess) {
            rc = FSE_E_CUDA;
            break;
        }
        pos += rel;
    }
    if (rc == FSE_OK) offsets[nch] = pos;
    count_launches(3 + 5LL * ((nch + G - 1) / G));
    return rc;
}

int fse_world_unpack(fse_world *w, const uint8_t *in, const int64_t *offsets, int n_chunks, int8_t *out_phases,
                     int *out_bad_chunk) {
    if (!w || !in || !offsets) return FSE_E_INVAL;
    if (out_bad_chunk) *out_bad_chunk = -1;
    int nch = 0;
    fse_world_pack_bound(w->W, w->H, nullptr, &nch);
    if (n_chunks != nch) return FSE_E_INVAL;
    int rc = ensure_materials_pushed();
    if (rc) return rc;
    const int nmat = host_table().n;
    // headers on the host: the first malformed chunk ends the load (chunks before it are written)
    int bad = nch;
    std::vector<long long> o1(nch), o2(nch);
    std::vector<int> l1(nch), l2(nch);
    for (int k = 0; k < nch; k++) {
        const long long len = offsets[k + 1] - offsets[k];
        int32_t hd[4] = {0, 0, 0, 0};
        if (offsets[k] < 0 || len < PK_HEADER) {
            bad = k;
            break;
        }
        memcpy(hd, in + offsets[k] + 1, 16);
        if (hd[0] != PK_SRC1 || hd[2] != PK_SRC2 || hd[1] <= 0 || hd[3] <= 0 ||
            (long long)PK_HEADER + hd[1] + hd[3] > len) {
            bad = k;
            break;
        }
        if (out_phases) out_phases[k] = (int8_t)in[offsets[k]];
        o1[k] = offsets[k] + PK_HEADER;
        l1[k] = hd[1];
        o2[k] = offsets[k] + PK_HEADER + hd[1];
        l2[k] = hd[3];
    }
    const int G = std::max(1, std::min(PK_GROUP, nch));
    uint8_t *din = nullptr, *rec = nullptr, *bgo = nullptr;
    long long *doff = nullptr;
    int *dlen = nullptr, *dst = nullptr;
    cudaStream_t s = w->stream;
    if (!scratch(w, 9, &rec, (size_t)G * PK_SRC1) || !scratch(w, 10, &bgo, (size_t)G * PK_SRC2) ||
        !scratch(w, 11, &doff, (size_t)2 * G * sizeof(long long)) || !scratch(w, 12, &dlen, (size_t)2 * G * sizeof(int)) ||
        !scratch(w, 13, &dst, (size_t)(2 * G + 1) * sizeof(int)))
        return FSE_E_NOMEM;
    std::vector<int> st(2 * G);
    for (int c0 = 0; c0 < bad && rc == FSE_OK; c0 += G) {
        const int g = std::min(G, bad - c0);
        // the group's input, one copy
        const long long lo = offsets[c0], hi = offsets[c0 + g];
        if (!scratch(w, 14, &din, (size_t)(hi - lo))) {
            rc = FSE_E_NOMEM;
            break;
        }
        std::vector<long long> ho(2 * g);
        std::vector<int> hl(2 * g);
        for (int c = 0; c < g; c++) {
            ho[c] = o1[c0 + c] - lo;
            hl[c] = l1[c0 + c];
            ho[g + c] = o2[c0 + c] - lo;
            hl[g + c] = l2[c0 + c];
        }
        const int big = 0x7fffffff;
        if (cudaMemcpyAsync(din, in + lo, (size_t)(hi - lo), cudaMemcpyHostToDevice, s) != cudaSuccess ||
            cudaMemcpyAsync(doff, ho.data(), 2 * g * sizeof(long long), cudaMemcpyHostToDevice, s) != cudaSuccess ||
            cudaMemcpyAsync(dlen, hl.data(), 2 * g * sizeof(int), cudaMemcpyHostToDevice, s) != cudaSuccess ||
            cudaMemcpyAsync(dst + 2 * G, &big, sizeof(int), cudaMemcpyHostToDevice, s) != cudaSuccess) {
            rc = FSE_E_CUDA;
            break;
        }
        launch_decode(din, doff, dlen, g, *std::max_element(hl.begin(), hl.begin() + g), PK_SRC1, rec, PK_SRC1, dst, s);
        launch_decode(din, doff + g, dlen + g, g, *std::max_element(hl.begin() + g, hl.end()), PK_SRC2, bgo, PK_SRC2,
                      dst + g, s);
        k_unpack_check<<<grid_for((long long)g * PK_CELLS, 256), 256, 0, s>>>(rec, PK_SRC1, g, nmat, dst + 2 * G);
        int first_bad_id = big;
        if (cudaMemcpyAsync(st.data(), dst, 2 * g * sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
            cudaMemcpyAsync(&first_bad_id, dst + 2 * G, sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
            cudaStreamSynchronize(s) != cudaSuccess) {
            rc = FSE_E_CUDA;
            break;
        }
        int gbad = std::min(g, first_bad_id);
        for (int c = 0; c < g; c++)
            if (st[c] != PK_SRC1 || st[g + c] != PK_SRC2) gbad = std::min(gbad, c);
        if (gbad > 0)
            k_unpack_scatter<<<grid_for((long long)gbad * PK_CELLS, 256), 256, 0, s>>>(w->d, g_dev_mt, rec, PK_SRC1,
                                                                                        c0, gbad);
        count_launches(3 + (gbad > 0 ? 1 : 0));
        if (gbad < g) bad = c0 + gbad;
    }
    if (rc == FSE_OK && cudaStreamSynchronize(s) != cudaSuccess) rc = FSE_E_CUDA;
    if (rc) return rc;
    if (bad < nch) {
        if (out_bad_chunk) *out_bad_chunk = bad;
        return FSE_E_INVAL;
    }
    return FSE_OK;
}

}  // extern "C"

// ============================================================ checkpoints
// An exact checkpoint of a world: header, then sections (every plane, the particle
// arrays, the ledger), each as LZ4 blocks of at most CK_BLOCK bytes written by the
// encoder above. Layout (little-endian):
//   "FSECKPT1", i32 W, H, chunk, cell_iter, u32 seed, tick, i32 flags (bit 0:
//   liquid temperatures), i32 particles, i32 sections;
//   per section: u32 tag, i64 bytes, i32 blocks; per block: i32 raw, i32 packed, bytes.
namespace fse {
namespace {

constexpr int CK_BLOCK = 4 << 20;
constexpr int CK_GROUP = 16;  // blocks encoded or decoded per pass
constexpr int CK_SLOT = (lz4_bound(CK_BLOCK) + 15) & ~15;
constexpr int CK_SEGS = (CK_BLOCK + ENC_SEG - 1) / ENC_SEG;
constexpr char CK_MAGIC[8] = {'F', 'S', 'E', 'C', 'K', 'P', 'T', '1'};

struct CkSection {
    uint32_t tag;
    void *dev;
    int64_t bytes;
};

// the sections of a world holding np particles, in file order
std::vector<CkSection> ck_sections(fse_world *w, int np) {
    const WorldDev &h = w->h;
    const int64_t n = (int64_t)w->W * w->H, p = np;
    std::vector<CkSection> v = {{1, h.id, 2 * n}, {2, h.col, 4 * n}, {3, h.sc, 4 * n}, {4, h.fl, n}, {5, h.df, 4 * n}};
    if (h.tp) v.push_back({6, h.tp, 2 * n});
    const PartSoA &q = h.p;
    void *f4[] = {q.x, q.y, q.vx, q.vy, q.ax, q.ay, q.tx, q.ty, q.tf, q.life, q.fade, q.col, q.sc};
    for (int k = 0; k < 13; k++) v.push_back({(uint32_t)(16 + k), f4[k], 4 * p});
    v.push_back({29, q.id, 2 * p});
    v.push_back({30, q.fl, p});
    v.push_back({31, q.bits, p});
    if (h.tp) v.push_back({32, q.tp, 2 * p});
    v.push_back({40, h.ledger, (int64_t)LED_ROWS * MAXMAT * 8});
    return v;
}

struct CkScratch {
    uint32_t *stage = nullptr;
    uint8_t *enc = nullptr;
    int *sizes = nullptr, *anc = nullptr, *sout = nullptr, *status = nullptr;
    SegInfo *info = nullptr;
    uint2 *rec = nullptr;
    uint8_t *din = nullptr;
    long long *doff = nullptr;
    int *dlen = nullptr;
    bool ok() const { return stage && enc && sizes && anc && sout && status && info && rec && din && doff && dlen; }
    void alloc() {
        cudaMalloc(&stage, (size_t)CK_GROUP * CK_BLOCK + 16);  // + a zeroed word after the data
        cudaMalloc(&enc, (size_t)CK_GROUP * CK_SLOT);
        cudaMalloc(&sizes, (CK_GROUP + 1) * sizeof(int));
        cudaMalloc(&anc, (size_t)CK_GROUP * CK_SEGS * sizeof(int));
        cudaMalloc(&sout, (size_t)CK_GROUP * CK_SEGS * sizeof(int));
        cudaMalloc(&status, (CK_GROUP + 1) * sizeof(int));
        cudaMalloc(&info, (size_t)CK_GROUP * CK_SEGS * sizeof(SegInfo));
        cudaMalloc(&rec, (size_t)CK_GROUP * CK_SEGS * ENC_REC * sizeof(uint2));
        cudaMalloc(&din, (size_t)CK_GROUP * CK_SLOT);
        cudaMalloc(&doff, (CK_GROUP + 1) * sizeof(long long));
        cudaMalloc(&dlen, (CK_GROUP + 1) * sizeof(int));
    }
    void release() {
        void *ps[] = {stage, enc, sizes, anc, sout, status, info, rec, din, doff, dlen};
        for (void *q : ps)
            if (q) cudaFree(q);
    }
};

// host writer with a capacity check
struct Out {
    uint8_t *p;
    int64_t cap, n = 0;
    bool room(int64_t k) const { return n + k <= cap; }
    template <class T>
    bool put(const T &v) {
        if (!room(sizeof(T))) return false;
        memcpy(p + n, &v, sizeof(T));
        n += sizeof(T);
        return true;
    }
};

int ck_write_section(const CkSection &sec, Out &o, CkScratch &sc, cudaStream_t s) {
    const int nblk = (int)((sec.bytes + CK_BLOCK - 1) / CK_BLOCK);
    if (!o.put(sec.tag) || !o.put((int64_t)sec.bytes) || !o.put((int32_t)nblk)) return FSE_E_CAPACITY;
    std::vector<int> sz(CK_GROUP);
    for (int g0 = 0; g0 < nblk; g0 += CK_GROUP) {
        const int g = std::min(CK_GROUP, nblk - g0);
        const int64_t lo = (int64_t)g0 * CK_BLOCK, hi = std::min(sec.bytes, (int64_t)(g0 + g) * CK_BLOCK);
        const int64_t span = hi - lo;
        if (cudaMemcpyAsync(sc.stage, (const uint8_t *)sec.dev + lo, (size_t)span, cudaMemcpyDeviceToDevice, s) !=
                cudaSuccess ||
            cudaMemsetAsync((uint8_t *)sc.stage + span, 0, 4, s) != cudaSuccess)  // word-aligned tail
            return FSE_E_CUDA;
        const int full = (int)(span / CK_BLOCK), tail = (int)(span - (int64_t)full * CK_BLOCK);
        if (full)
            encode_blocks(sc.stage, CK_BLOCK, CK_BLOCK, full, sc.enc, CK_SLOT, sc.sizes, sc.info, sc.anc, sc.sout, sc.rec,
                          s);
        if (tail)
            encode_blocks(sc.stage + (size_t)full * (CK_BLOCK / 4), (tail + 3) & ~3, tail, 1,
                          sc.enc + (size_t)full * CK_SLOT, CK_SLOT, sc.sizes + full, sc.info, sc.anc, sc.sout,
                          sc.rec, s);
        count_launches(3LL * ((full ? 1 : 0) + (tail ? 1 : 0)));
        if (cudaMemcpyAsync(sz.data(), sc.sizes, g * sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
            cudaStreamSynchronize(s) != cudaSuccess)
            return FSE_E_CUDA;
        for (int b = 0; b < g; b++) {
            const int raw = b < full ? CK_BLOCK : tail;
            if (sz[b] < 0) return FSE_E_CUDA;
            if (!o.put((int32_t)raw) || !o.put((int32_t)sz[b]) || !o.room(sz[b])) return FSE_E_CAPACITY;
            if (cudaMemcpyAsync(o.p + o.n, sc.enc + (size_t)b * CK_SLOT, (size_t)sz[b], cudaMemcpyDeviceToHost, s) !=
                cudaSuccess)
                return FSE_E_CUDA;
            o.n += sz[b];
        }
        if (cudaStreamSynchronize(s) != cudaSuccess) return FSE_E_CUDA;
    }
    return FSE_OK;
}

// host reader with bounds checks
struct In {
    const uint8_t *p;
    int64_t size, n = 0;
    template <class T>
    bool get(T &v) {
        if (n + (int64_t)sizeof(T) > size) return false;
        memcpy(&v, p + n, sizeof(T));
        n += sizeof(T);
        return true;
    }
};

int ck_read_section(const CkSection &sec, In &in, CkScratch &sc, cudaStream_t s) {
    uint32_t tag;
    int64_t bytes;
    int32_t nblk;
    if (!in.get(tag) || !in.get(bytes) || !in.get(nblk) || tag != sec.tag || bytes != sec.bytes ||
        nblk != (int32_t)((bytes + CK_BLOCK - 1) / CK_BLOCK))
        return FSE_E_INVAL;
    std::vector<long long> off(CK_GROUP);
    std::vector<int> len(CK_GROUP), st(CK_GROUP);
    for (int g0 = 0; g0 < nblk; g0 += CK_GROUP) {
        const int g = std::min((int)CK_GROUP, nblk - g0);
        long long pos = 0;
        int full = 0, tail = 0;
        for (int b = 0; b < g; b++) {
            int32_t raw, packed;
            if (!in.get(raw) || !in.get(packed)) return FSE_E_INVAL;
            const int64_t want = std::min((int64_t)CK_BLOCK, bytes - (int64_t)(g0 + b) * CK_BLOCK);
            if (raw != want || packed <= 0 || packed > CK_SLOT || in.n + packed > in.size) return FSE_E_INVAL;
            if (cudaMemcpyAsync(sc.din + pos, in.p + in.n, (size_t)packed, cudaMemcpyHostToDevice, s) != cudaSuccess)
                return FSE_E_CUDA;
            in.n += packed;
            off[b] = pos;
            len[b] = packed;
            pos += packed;
            if (raw == CK_BLOCK)
                full++;
            else
                tail = raw;
        }
        if (cudaMemcpyAsync(sc.doff, off.data(), g * sizeof(long long), cudaMemcpyHostToDevice, s) != cudaSuccess ||
            cudaMemcpyAsync(sc.dlen, len.data(), g * sizeof(int), cudaMemcpyHostToDevice, s) != cudaSuccess)
            return FSE_E_CUDA;
        uint8_t *dst = (uint8_t *)sec.dev + (int64_t)g0 * CK_BLOCK;
        if (full)
            launch_decode(sc.din, sc.doff, sc.dlen, full, *std::max_element(len.begin(), len.begin() + full), CK_BLOCK,
                          dst, CK_BLOCK, sc.status, s);
        if (tail)
            launch_decode(sc.din, sc.doff + full, sc.dlen + full, 1, len[full], tail, dst + (size_t)full * CK_BLOCK,
                          CK_BLOCK, sc.status + full, s);
        count_launches((full ? 1 : 0) + (tail ? 1 : 0));
        if (cudaMemcpyAsync(st.data(), sc.status, g * sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
            cudaStreamSynchronize(s) != cudaSuccess)
            return FSE_E_CUDA;
        for (int b = 0; b < g; b++)
            if (st[b] != (b < full ? CK_BLOCK : tail)) return FSE_E_INVAL;
    }
    return FSE_OK;
}

}  // namespace
}  // namespace fse

extern "C" {

int fse_world_checkpoint_bound(fse_world *w, int64_t *out_bytes) {
    if (!w || !out_bytes) return FSE_E_INVAL;
    int32_t info[8];
    int rc = fse_world_info(w, info);
    if (rc) return rc;
    int64_t total = 64;
    for (const CkSection &sec : ck_sections(w, info[6])) {  // a block never grows past lz4_bound(raw)
        const int64_t nblk = (sec.bytes + CK_BLOCK - 1) / CK_BLOCK;
        total += 16 + nblk * 24 + sec.bytes + sec.bytes / 255;
    }
    *out_bytes = total;
    return FSE_OK;
}

int fse_world_checkpoint(fse_world *w, uint8_t *out, int64_t cap, int64_t *out_size) {
    if (!w || !out || !out_size) return FSE_E_INVAL;
    int32_t info[8];
    int rc = fse_world_info(w, info);  // also waits for the world's work
    if (rc) return rc;
    const std::vector<CkSection> secs = ck_sections(w, info[6]);
    Out o{out, cap};
    if (!o.room(8)) return FSE_E_CAPACITY;
    memcpy(out, CK_MAGIC, 8);
    o.n = 8;
    // bit 0: liquid temperatures follow; bit 1: liquid amounts are f32
    const int32_t flags = (w->h.tp ? 1 : 0) | (w->h.f32 ? 2 : 0);
    if (!o.put((int32_t)w->W) || !o.put((int32_t)w->H) || !o.put((int32_t)w->C) || !o.put((int32_t)w->cell_iter) ||
        !o.put((uint32_t)w->h.seed) || !o.put((uint32_t)info[5]) || !o.put(flags) || !o.put((int32_t)info[6]) ||
        !o.put((int32_t)secs.size()))
        return FSE_E_CAPACITY;
    CkScratch sc;
    sc.alloc();
    if (!sc.ok()) {
        sc.release();
        return FSE_E_NOMEM;
    }
    for (const CkSection &sec : secs) {
        rc = ck_write_section(sec, o, sc, w->stream);
        if (rc) break;
    }
    sc.release();
    if (rc) return rc;
    *out_size = o.n;
    return FSE_OK;
}

int fse_world_restore(fse_world *w, const uint8_t *in, int64_t size) {
    if (!w || !in || size < 0) return FSE_E_INVAL;
    FSE_CUDA_TRY(cudaStreamSynchronize(w->stream));
    int rc = FSE_OK;
    In r{in, size};
    char magic[8];
    int32_t W, H, C, it, flags, np, nsec;
    uint32_t seed, tick;
    if (size < 8) return FSE_E_INVAL;
    memcpy(magic, in, 8);
    r.n = 8;
    if (memcmp(magic, CK_MAGIC, 8) != 0 || !r.get(W) || !r.get(H) || !r.get(C) || !r.get(it) || !r.get(seed) ||
        !r.get(tick) || !r.get(flags) || !r.get(np) || !r.get(nsec))
        return FSE_E_INVAL;
    if (W != w->W || H != w->H || C != w->C || it != w->cell_iter || np < 0) return FSE_E_INVAL;
    if ((flags & 1) && !w->h.tp) return FSE_E_STATE;  // liquid temperatures need FSE_CFG_TEMPERATURE
    if (((flags & 2) != 0) != (w->h.f32 != 0)) return FSE_E_STATE;  // f32 and Q16.16 amounts do not mix
    if (np > w->part_cap) return FSE_E_CAPACITY;
    // sections in file order; a world that keeps liquid temperatures restores a file
    // without them as 0
    std::vector<CkSection> secs = ck_sections(w, np);
    if (!(flags & 1)) {
        std::vector<CkSection> keep;
        for (const CkSection &sc : secs)
            if (sc.tag != 6 && sc.tag != 32) keep.push_back(sc);
        secs.swap(keep);
        if (w->h.tp && cudaMemsetAsync(w->h.tp, 0, (size_t)w->W * w->H * 2, w->stream) != cudaSuccess)
            return FSE_E_CUDA;
    }
    if (nsec != (int32_t)secs.size()) return FSE_E_INVAL;
    CkScratch sc;
    sc.alloc();
    if (!sc.ok()) {
        sc.release();
        return FSE_E_NOMEM;
    }
    for (const CkSection &sec : secs) {
        rc = ck_read_section(sec, r, sc, w->stream);
        if (rc) break;
    }
    sc.release();
    if (rc) return rc;
    // counters: live particles and the tick; nothing in flight, no error
    int32_t ctr[16] = {0};
    ctr[1] = np;
    ctr[6] = (int32_t)tick;
    w->seed = seed;
    w->h.seed = seed;
    FSE_CUDA_TRY(cudaMemcpyAsync(w->ctr, ctr, sizeof(ctr), cudaMemcpyHostToDevice, w->stream));
    FSE_CUDA_TRY(cudaMemcpyAsync(w->d, &w->h, sizeof(WorldDev), cudaMemcpyHostToDevice, w->stream));
    if (w->h.dirty) FSE_CUDA_TRY(cudaMemsetAsync(w->h.dirty, 1, (size_t)w->W * w->H, w->stream));
    FSE_CUDA_TRY(cudaStreamSynchronize(w->stream));
    return FSE_OK;
}

}  // extern "C"
