"""Chunk .pack codec on the GPU (Chunk::ChunkWrite / ChunkRead, chunk.cpp:68-330).

The device encoder writes exactly the oracle's bytes; the device decoder reads the
.pack files the reference's own LZ4 made (tests/golden/pack.npz) and the oracle's,
and refuses malformed chunks at the same chunk as the oracle.
"""
import os

import numpy as np
import pytest

from pack_cases import HEADER, SRC1, sample_world, split_blocks

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "pack.npz")


def _device_copy(fse, ow, w, h):
    """A device world (keeping liquid temperatures) holding the oracle world's state."""
    world = fse.World(w, h, seed=1, temperature=True)
    st = ow.state()
    world.upload(st)
    world.set_temperature(ow.temperature())
    return world


@pytest.mark.parametrize("w,h,seed", [(256, 192, 77), (200, 136, 5), (384, 256, 9), (128, 128, 3)])
def test_pack_matches_oracle(fse, oracle_mod, w, h, seed):
    oracle_mod.Oracle().reset_materials()
    ow = sample_world(oracle_mod, w, h, seed)
    world = _device_copy(fse, ow, w, h)
    for phase in (0, -3):
        data, offs = world.pack(phase)
        odata, ooffs = ow.pack(phase)
        assert np.array_equal(offs, ooffs) and np.array_equal(data, odata), (w, h, phase)


def test_unpack_reference_files(fse, oracle_mod):
    g = np.load(GOLDEN)
    w, h, seed, phase = [int(v) for v in g["params"]]
    world = fse.World(w, h, seed=1, temperature=True)
    phases = world.unpack(g["ref_data"], g["ref_offsets"])
    assert np.all(phases == phase)
    st = world.state()
    assert np.array_equal(st["id"], g["id"]) and np.array_equal(st["colour"], g["colour"])
    assert np.array_equal(world.temperature(), g["temperature"])
    types = np.array([fse.material_get(i)[0] for i in range(fse.material_count())])
    soup = types[st["id"]] == fse.SOUP
    assert np.all(st["scalar"][soup] == 2 * fse.FLUID_ONE)
    assert not st["flags"].any()
    # the oracle reads the same files to the same state
    ow = oracle_mod.OracleWorld(w, h, 128, 3, 1)
    rc, _ = ow.unpack(g["ref_data"], g["ref_offsets"])
    assert rc == 0
    o = ow.state()
    for k in ("id", "colour", "scalar", "flags"):
        assert np.array_equal(st[k], o[k]), k


@pytest.mark.parametrize("w,h", [(384, 256), (200, 136)])
def test_pack_unpack_roundtrip_and_resume(fse, oracle_mod, w, h):
    """pack -> unpack into a fresh world restores ids, colours and temperatures; both
    worlds then tick identically (liquid amounts read back as 2.0 on both sides)."""
    world = fse.World(w, h, seed=11, temperature=True)
    world.generate(fse.GEN_MIX, 11)
    world.step(5)
    data, offs = world.pack(1)
    a = fse.World(w, h, seed=11, temperature=True)
    assert np.all(a.unpack(data, offs) == 1)
    sa, s0 = a.state(), world.state()
    assert np.array_equal(sa["id"], s0["id"]) and np.array_equal(sa["colour"], s0["colour"])
    assert np.array_equal(a.temperature(), world.temperature())
    b = fse.World(w, h, seed=11, temperature=True)
    b.unpack(data, offs)
    a.step(4)
    b.step(4)
    for k, v in a.state().items():
        assert np.array_equal(v, b.state()[k]), k


def test_unpack_rejects_malformed(fse, oracle_mod):
    """A chunk with a bad header, size or block ends the load at that chunk, as in the
    oracle; the chunks before it are written."""
    oracle_mod.Oracle().reset_materials()
    ow = sample_world(oracle_mod, 384, 256, 4)
    data, offs = ow.pack(0)
    cases = []
    d = data.copy()
    d[offs[2] + 1: offs[2] + 5] = np.array([SRC1 + 12], "<i4").view(np.uint8)  # src_size of chunk 2
    cases.append((d, offs.copy(), 2))
    d = data.copy()
    hd, c1, _ = split_blocks(data, offs, 4)
    d[offs[4] + HEADER: offs[4] + HEADER + 6] = 255  # runaway literal length in chunk 4
    cases.append((d, offs.copy(), 4))
    d = data.copy()
    o = offs.copy()
    o[3] = o[2] + 10  # chunk 2 shorter than a header
    cases.append((d, o, 2))
    d = data.copy()
    d[offs[1] + HEADER + hd[1] - 3: offs[1] + HEADER + hd[1]] = 0  # chunk 1: block cut short of its size
    hd1 = split_blocks(data, offs, 1)[0]
    d[offs[1] + 5: offs[1] + 9] = np.array([hd1[1] - 40], "<i4").view(np.uint8)
    cases.append((d, offs.copy(), 1))
    for d, o, k in cases:
        world = fse.World(384, 256, seed=1, temperature=True)
        with pytest.raises(fse.FseError):
            world.unpack(d, o)
        ob = oracle_mod.OracleWorld(384, 256, 128, 3, 1)
        rc, _ = ob.unpack(d, o)
        assert rc == -1 - k, (rc, k)
        gs, os_ = world.state(), ob.state()
        for key in ("id", "colour", "scalar"):
            assert np.array_equal(gs[key], os_[key]), (key, k)


def test_large_blocks_odd_offsets_and_trim(fse, oracle_mod):
    """Chunks whose colours are noise give tile blocks over 64 KB (decoded through the
    input window) beside ordinary ones (decoded whole from shared memory), in one
    launch; the files start at every offset mod 16; scratch freed by trim is made
    again."""
    oracle_mod.Oracle().reset_materials()
    w, h = 384, 256
    ow = sample_world(oracle_mod, w, h, 21)
    st = ow.state()
    rng = np.random.default_rng(21)
    noisy = np.zeros((h, w), bool)
    noisy[:128, 128:256] = True
    noisy[128:, :128] = True
    st["colour"] = np.where(noisy, rng.integers(0, 2 ** 32, (h, w), dtype=np.uint64).astype(np.uint32), st["colour"])
    ow.set_state(st)
    world = _device_copy(fse, ow, w, h)
    data, offs = world.pack(2)
    odata, ooffs = ow.pack(2)
    assert np.array_equal(offs, ooffs) and np.array_equal(data, odata)
    sizes = [split_blocks(data, offs, k)[0][1] for k in range(len(offs) - 1)]
    assert max(sizes) > 64 * 1024 and min(sizes) < 32 * 1024, sizes
    for shift in range(16):
        buf = np.concatenate([np.full(shift, 0xA5, np.uint8), data])
        b = fse.World(w, h, seed=1, temperature=True)
        assert np.all(b.unpack(buf, offs + shift) == 2)
        sb = b.state()
        assert np.array_equal(sb["id"], st["id"]) and np.array_equal(sb["colour"], st["colour"]), shift
        assert np.array_equal(b.temperature(), ow.temperature()), shift
        if shift == 15:
            b.trim()
            b.trim()
            assert np.all(b.unpack(buf, offs + shift) == 2)
            d2, o2 = b.pack(2)
            assert np.array_equal(o2, offs) and np.array_equal(d2, data)
        b.close()
    world.close()


def _same_world(fse, a, b, temperature):
    for k, v in a.state().items():
        assert np.array_equal(v, b.state()[k]), k
    pa, pb = a.particles(), b.particles()
    assert pa.tobytes() == pb.tobytes()
    assert np.array_equal(a.ledger(), b.ledger())
    assert a.tick_count == b.tick_count
    if temperature:
        assert np.array_equal(a.temperature(), b.temperature())


@pytest.mark.parametrize("temperature", [False, True])
def test_checkpoint_restore_is_exact(fse, temperature):
    """A world restored from a checkpoint (into a world made with another seed)
    continues bit for bit as the original: planes, particles, ledger, tick."""
    kw = dict(temperature=True, temperature_step=True) if temperature else {}
    a = fse.World(320, 256, seed=21, **kw)
    a.generate(fse.GEN_MIX, 21)
    rng = np.random.default_rng(0)
    p = np.zeros(2000, fse.PARTICLE_DTYPE)
    p["x"] = rng.uniform(0, 320, 2000)
    p["y"] = rng.uniform(0, 200, 2000)
    p["vx"] = rng.normal(0, 2, 2000)
    p["vy"] = rng.normal(0, 2, 2000)
    p["ay"] = 0.1
    p["id"] = 2
    p["colour"] = 0xFFFF00
    a.addCell(p)
    a.step(7)
    data = a.checkpoint()
    b = fse.World(320, 256, seed=999, **kw)
    b.restore(data)
    _same_world(fse, a, b, temperature)
    a.step(9)
    b.step(9)
    _same_world(fse, a, b, temperature)
    # a checkpoint of a 5 Mcell world spans several 4 MB blocks per plane
    big = fse.World(2560, 2048, seed=3, **kw)
    big.generate(fse.GEN_MIX, 3)
    big.step(2)
    c = fse.World(2560, 2048, seed=4, **kw)
    c.restore(big.checkpoint())
    big.step(2)
    c.step(2)
    _same_world(fse, big, c, temperature)


def test_restore_rejects_mismatch_and_corruption(fse):
    a = fse.World(256, 192, seed=1, temperature=True)
    a.generate(fse.GEN_MIX, 1)
    a.step(3)
    data = a.checkpoint()
    with pytest.raises(fse.FseError):
        fse.World(256, 256, seed=1, temperature=True).restore(data)  # another size
    with pytest.raises(fse.FseError):
        fse.World(256, 192, seed=1).restore(data)  # liquid temperatures need FSE_CFG_TEMPERATURE
    for cut in (10, 60, len(data) // 2, len(data) - 1):
        with pytest.raises(fse.FseError):
            fse.World(256, 192, seed=1, temperature=True).restore(data[:cut])
    # header 44 bytes; first section: tag @44, bytes @48, blocks @56; first block: raw @60, packed @64, data @68
    # (the format has no checksum, like .pack files: a changed literal byte inside a block
    # decodes; lengths, sizes and tokens are checked)
    for at, val in ((0, 0), (48, 1), (60, 7), (64, 0x7FFFFFF0), (68, 0xFF)):
        bad = data.copy()
        bad[at] = val if val <= 0xFF else 0
        if val > 0xFF:
            bad[at:at + 4] = np.array([val], "<i4").view(np.uint8)
        with pytest.raises(fse.FseError):
            fse.World(256, 192, seed=1, temperature=True).restore(bad)
    # a checkpoint without liquid temperatures restores into a world that keeps them as 0
    d = fse.World(256, 192, seed=1)
    d.generate(fse.GEN_MIX, 1)
    e = fse.World(256, 192, seed=1, temperature=True)
    e.restore(d.checkpoint())
    types = np.array([fse.material_get(i)[0] for i in range(fse.material_count())])
    assert not e.temperature()[types[e.state()["id"]] == fse.SOUP].any()
