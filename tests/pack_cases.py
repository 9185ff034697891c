"""Helpers for the chunk .pack tests (Chunk::ChunkWrite layout, chunk.cpp:219-330)."""
import numpy as np

EDGE = 128
CELLS = EDGE * EDGE
SRC1 = CELLS * 2 * 12  # tiles + layer2 MaterialInstanceData {u32 index, u32 color, i16 temperature}
SRC2 = CELLS * 4       # background
HEADER = 17


def chunk_records(ids, colours, temps, cx, cy):
    """The 393216-byte MaterialInstanceData buffer of chunk (cx, cy); cells outside the
    world and the whole second layer are zero records."""
    h, w = ids.shape
    rec = np.zeros((2 * CELLS, 12), np.uint8)
    y0, x0 = cy * EDGE, cx * EDGE
    sub_i = ids[y0:y0 + EDGE, x0:x0 + EDGE]
    sh, sw = sub_i.shape
    r = rec[:CELLS].reshape(EDGE, EDGE, 12)
    r[:sh, :sw, 0:4] = sub_i.astype("<u4").view(np.uint8).reshape(sh, sw, 4)
    r[:sh, :sw, 4:8] = colours[y0:y0 + EDGE, x0:x0 + EDGE].astype("<u4").view(np.uint8).reshape(sh, sw, 4)
    r[:sh, :sw, 8:10] = temps[y0:y0 + EDGE, x0:x0 + EDGE].astype("<i2").view(np.uint8).reshape(sh, sw, 2)
    return rec.reshape(-1)


def chunk_count(w, h):
    return ((w + EDGE - 1) // EDGE) * ((h + EDGE - 1) // EDGE)


def pack_with(compress, ids, colours, temps, phase=0):
    """A whole world packed chunk by chunk (row-major) with a given LZ4 compressor."""
    h, w = ids.shape
    ncx = (w + EDGE - 1) // EDGE
    parts, offs = [], [0]
    bg = compress(np.zeros(SRC2, np.uint8))
    for k in range(chunk_count(w, h)):
        c1 = compress(chunk_records(ids, colours, temps, k % ncx, k // ncx))
        head = np.zeros(HEADER, np.uint8)
        head[0] = np.uint8(np.int8(phase).view(np.uint8))
        head[1:17] = np.array([SRC1, len(c1), SRC2, len(bg)], "<i4").view(np.uint8)
        parts += [head, c1, bg]
        offs.append(offs[-1] + HEADER + len(c1) + len(bg))
    return np.concatenate(parts), np.array(offs, np.int64)


def split_blocks(data, offsets, k):
    """(header ints, tile block, background block) of chunk k."""
    p = data[offsets[k]:offsets[k + 1]]
    hd = p[1:17].view("<i4")
    c1 = p[HEADER:HEADER + hd[1]]
    c2 = p[HEADER + hd[1]:HEADER + hd[1] + hd[3]]
    return hd, c1, c2


def sample_world(oracle_mod, w, h, seed, steps=4):
    """An oracle world with a generated mix, a few steps, and hot and cold spots."""
    ow = oracle_mod.OracleWorld(w, h, 128, 3, seed)
    ow.generate(0, seed)
    ow.step(steps)
    t = ow.temperature()
    rng = np.random.default_rng(seed)
    spots = rng.random((h, w)) < 0.05
    t = np.where(spots, rng.integers(-32768, 32768, size=(h, w)), t).astype(np.int16)
    ow.set_temperature(t)
    return ow
