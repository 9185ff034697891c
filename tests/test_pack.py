"""Chunk .pack codec (Chunk::ChunkWrite / ChunkRead, chunk.cpp:68-330) on the CPU.

The oracle's LZ4 block encoder and decoder are pinned against the reference's own
vendored LZ4 1.9.4 (source/libs/lz4/lz4.c, compiled in place by oracle/Makefile
`ref`) when the reference tree is present: the reference's LZ4_decompress_safe
reads every block the oracle writes, and the oracle reads blocks written by the
reference's LZ4_compress_fast. tests/golden/pack.npz holds .pack files that the
reference's LZ4 produced, for machines without the reference tree.
"""
import hashlib
import os

import numpy as np
import pytest

from pack_cases import CELLS, SRC1, SRC2, chunk_records, pack_with, sample_world, split_blocks

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "pack.npz")


def _ref_lz4():
    from oracle.binding import ReferenceLZ4, build_reference_lz4

    lib = build_reference_lz4()
    if lib is None:
        pytest.skip("reference tree absent")
    return ReferenceLZ4(lib)


def _buffers(oracle_mod):
    bufs = []
    ow = sample_world(oracle_mod, 256, 192, 5)
    st, t = ow.state(), ow.temperature()
    for k in range(4):
        bufs.append(chunk_records(st["id"], st["colour"], t, k % 2, k // 2))
    rng = np.random.default_rng(1)
    bufs.append(rng.integers(0, 256, size=SRC1, dtype=np.uint8))  # incompressible
    bufs.append(np.zeros(SRC2, np.uint8))                           # the background
    z = np.zeros(4096, np.uint8)
    z[::7] = 9
    bufs.append(z)                                                  # a short periodic block
    bufs.append(np.arange(40, dtype=np.uint8))                      # shortest sizes
    bufs.append(np.zeros(13, np.uint8))
    return bufs


def test_reference_lz4_reads_oracle_blocks(oracle_mod):
    from oracle.binding import lz4_encode

    lz4 = _ref_lz4()
    oracle_mod.Oracle().reset_materials()
    for b in _buffers(oracle_mod):
        c = lz4_encode(b)
        out, m = lz4.decompress(c, len(b))
        assert m == len(b) and np.array_equal(out, b), (len(b), m)


def test_oracle_reads_reference_blocks(oracle_mod):
    from oracle.binding import lz4_decode

    lz4 = _ref_lz4()
    oracle_mod.Oracle().reset_materials()
    for b in _buffers(oracle_mod):
        for acc in (1, 10):
            c = lz4.compress(b, acc)
            out, m = lz4_decode(c, len(b))
            assert m == len(b) and np.array_equal(out, b), (len(b), acc, m)


def test_oracle_packs_smaller_than_reference(oracle_mod):
    """On generated worlds the 16-distance encoder writes smaller blocks than the
    LZ4_compress_fast(..., 10) of Chunk::ChunkWrite."""
    from oracle.binding import lz4_encode

    lz4 = _ref_lz4()
    oracle_mod.Oracle().reset_materials()
    mine = ref = 0
    for b in _buffers(oracle_mod)[:4]:
        mine += len(lz4_encode(b))
        ref += len(lz4.compress(b, 10))
    assert mine < ref, (mine, ref)


def test_oracle_reads_reference_pack_files(oracle_mod):
    g = np.load(GOLDEN)
    w, h, seed, phase = [int(v) for v in g["params"]]
    oracle_mod.Oracle().reset_materials()
    ow = oracle_mod.OracleWorld(w, h, 128, 3, 1)
    rc, phases = ow.unpack(g["ref_data"], g["ref_offsets"])
    assert rc == 0 and np.all(phases == phase)
    st = ow.state()
    assert np.array_equal(st["id"], g["id"]) and np.array_equal(st["colour"], g["colour"])
    assert np.array_equal(ow.temperature(), g["temperature"])
    types = np.array([oracle_mod.Oracle().material(i)[0] for i in range(oracle_mod.Oracle().material_count())])
    soup = types[st["id"]] == 3
    assert np.all(st["scalar"][soup] == 2 * 65536)  # MaterialInstance::fluidAmount default
    assert not st["flags"].any() and not st["diff"].any()


def test_oracle_pack_digest_and_roundtrip(oracle_mod):
    g = np.load(GOLDEN)
    w, h, seed, phase = [int(v) for v in g["params"]]
    oracle_mod.Oracle().reset_materials()
    ow = sample_world(oracle_mod, w, h, seed)
    data, offs = ow.pack(phase)
    assert hashlib.sha256(data.tobytes() + offs.tobytes()).hexdigest() == str(g["oracle_digest"])
    # the same bytes chunk by chunk from the layout helper and the oracle's encoder
    from oracle.binding import lz4_encode

    st, t = ow.state(), ow.temperature()
    d2, o2 = pack_with(lz4_encode, st["id"], st["colour"], t, phase)
    assert np.array_equal(d2, data) and np.array_equal(o2, offs)
    back = oracle_mod.OracleWorld(w, h, 128, 3, 2)
    rc, phases = back.unpack(data, offs)
    assert rc == 0 and np.all(phases == phase)
    assert np.array_equal(back.state()["id"], st["id"]) and np.array_equal(back.temperature(), t)


def test_oracle_rejects_malformed_packs(oracle_mod):
    """Truncated, corrupted or inconsistent files are refused chunk by chunk,
    never read or written out of bounds."""
    oracle_mod.Oracle().reset_materials()
    ow = sample_world(oracle_mod, 128, 128, 3)
    data, offs = ow.pack(0)
    rng = np.random.default_rng(0)
    from oracle.binding import lz4_decode

    hd, c1, c2 = split_blocks(data, offs, 0)
    bad = 0
    for _ in range(300):
        c = c1.copy()
        k = int(rng.integers(0, len(c)))
        c[k] = rng.integers(0, 256)
        if rng.random() < 0.3:
            c = c[: int(rng.integers(1, len(c)))]
        out, m = lz4_decode(c, SRC1)
        bad += m != SRC1 or not np.array_equal(out, lz4_decode(c1, SRC1)[0])
    assert bad > 0
    for mutate in ("short", "size", "block"):
        d, o = data.copy(), offs.copy()
        if mutate == "short":
            o[-1] = 10
        elif mutate == "size":
            d[1:5] = np.array([SRC1 + 12], "<i4").view(np.uint8)
        else:
            d[17:17 + 8] = 255
        back = oracle_mod.OracleWorld(128, 128, 128, 3, 2)
        rc, _ = back.unpack(d, o)
        assert rc == -1, mutate
