"""The grid as an array of tile structs (the reference's real_tiles of
MaterialInstance, game_datastruct.hpp:205-222) through fse_world_upload_tiles /
fse_world_download_tiles.

The conversion is restated here with numpy from the planes: id and colour as they
are; a SOUP cell's Q16.16 amount and pending diff as floats (amount / 65536), its
temperature from the liquid-temperature plane; any other cell's temperature from
the scalar plane; moved = flags bit 7, settleCount = flags bits 0-5. A world loaded
from tiles must tick exactly as the world the tiles came from.
"""
import numpy as np
import pytest

from helpers import compare_particles, compare_states, material_types

pytestmark = pytest.mark.gpu

SOUP = 3


def _expected_tiles(fse, planes, temps, types, base=None):
    t = np.zeros(planes["id"].shape, fse.TILE_DTYPE) if base is None else base.copy()
    soup = types[planes["id"]] == SOUP
    t["id"] = planes["id"]
    t["color"] = planes["colour"]
    t["temperature"] = np.where(soup, temps, planes["scalar"].astype(np.int16))
    t["moved"] = (planes["flags"] >> 7) & 1
    t["settleCount"] = planes["flags"] & 0x3F
    t["fluidAmount"] = np.where(soup, planes["scalar"].astype(np.float32) / np.float32(65536), t["fluidAmount"])
    t["fluidAmountDiff"] = np.where(soup, planes["diff"].astype(np.float32) / np.float32(65536), t["fluidAmountDiff"])
    return t


def _ticked_world(fse, w=300, h=200, seed=77, ticks=4):
    world = fse.World(w, h, seed=seed, temperature=True)
    world.generate(fse.GEN_MIX, seed)
    world.step(ticks)
    return world


def test_download_tiles_matches_planes(fse):
    types = material_types(fse)
    world = _ticked_world(fse)
    planes, temps = world.state(), world.temperature()
    table = (np.arange(fse.material_count(), dtype=np.uint64) * 0x40) + np.uint64(0x7F0000001000)
    base = np.zeros(planes["id"].shape, fse.TILE_DTYPE)
    base["fluidAmount"] = 2.0  # the reference's default for non-liquid tiles
    out = np.zeros(planes["id"].shape, fse.TILE_DTYPE)  # a copy of `base` may leave its padding unset
    out["fluidAmount"] = 2.0
    got = world.download_tiles(out, mat_table=table)
    exp = _expected_tiles(fse, planes, temps, types, base)
    exp["mat"] = table[planes["id"]]
    for k in fse.TILE_DTYPE.names:
        assert np.array_equal(got[k], exp[k]), k
    # the padding bytes of the struct are left as they were
    raw = got.view(np.uint8).reshape(-1, 40)
    assert not raw[:, [4, 5, 6, 7, 23, 33, 34, 35, 36, 37, 38, 39]].any()
    world.close()


def test_tiles_round_trip_and_tick(fse):
    """Tiles of a world loaded into another: the same planes, then the same ticks."""
    types = material_types(fse)
    a = fse.World(257, 190, seed=5, temperature=True)
    a.generate(fse.GEN_MIX, 5)
    a.step(3)
    tiles = a.download_tiles()
    b = fse.World(257, 190, seed=5, temperature=True)
    b.upload_tiles(tiles)
    b.tick_count = a.tick_count
    sa, sb = a.state(), b.state()
    sa["flags"] &= 0xBF
    compare_states(sb, sa, types, "tiles round trip")
    assert np.array_equal(a.temperature(), b.temperature())
    # a world that holds no free particles continues identically from its tiles
    c = fse.World(257, 190, seed=9, temperature=True)
    c.generate(fse.GEN_MIX, 9)
    d = fse.World(257, 190, seed=9, temperature=True)
    d.upload_tiles(c.download_tiles())
    for _ in range(6):
        c.step(1)
        d.step(1)
    compare_states(d.state(), c.state(), types, "ticks after tiles")
    compare_particles(d.particles(), c.particles(), "particles after tiles")
    for x in (a, b, c, d):
        x.close()


def test_custom_layout_and_absent_fields(fse):
    """A packed 16-byte struct without pointer or diff: absent fields load as defaults."""
    types = material_types(fse)
    src = _ticked_world(fse, 160, 96, seed=3, ticks=2)
    planes, temps = src.state(), src.temperature()
    dt = np.dtype({"names": ["id", "color", "temperature", "moved", "settleCount", "fluidAmount"],
                   "formats": ["<u4", "<u4", "<i2", "u1", "u1", "<f4"], "offsets": [0, 4, 8, 10, 11, 12],
                   "itemsize": 16})
    t = np.zeros(planes["id"].shape, dt)
    t = src.download_tiles(t)
    full = _expected_tiles(fse, planes, temps, types)
    for k in dt.names:
        assert np.array_equal(t[k], full[k]), k
    dst = fse.World(160, 96, seed=3, temperature=True)
    dst.upload_tiles(t)
    got = dst.state()
    soup = types[planes["id"]] == SOUP
    for k in ("id", "colour", "scalar"):
        assert np.array_equal(got[k], planes[k]), k
    assert np.array_equal(got["flags"], planes["flags"] & 0xBF)
    assert not got["diff"].any()  # no diff field: liquids load without a pending flow
    assert np.array_equal(dst.temperature()[soup], temps[soup])
    src.close()
    dst.close()


def test_upload_tiles_rounding_and_saturation(fse):
    types = material_types(fse)
    water = fse.material_find("WATER")
    stone = fse.material_find("STONE")
    t = np.zeros((4, 8), fse.TILE_DTYPE)
    t["id"] = water
    t["id"][1] = stone
    amounts = np.array([2.0, 0.5, 1.0 / 3.0, 1e-6, 2.00000763, -0.25, 1234.5, 0.0], np.float32)
    t["fluidAmount"][0] = amounts
    t["fluidAmountDiff"][0] = -amounts
    t["settleCount"][2] = [0, 1, 62, 63, 64, 100, 200, 255]
    t["moved"][3] = [0, 1, 2, 255, 0, 1, 0, 1]
    t["temperature"][1] = [-32768, -1, 0, 1, 300, 1000, 20000, 32767]
    t["temperature"][0] = [5, 6, 7, 8, 9, 10, 11, 12]
    w = fse.World(8, 4, seed=1, temperature=True)
    w.upload_tiles(t)
    s = w.state()
    q = np.rint(amounts.astype(np.float64) * 65536).astype(np.int32)
    assert np.array_equal(s["scalar"][0], q)
    assert np.array_equal(s["diff"][0], -q)
    assert np.array_equal(s["scalar"][1], t["temperature"][1].astype(np.int32))
    assert np.array_equal(s["flags"][2] & 0x3F, np.minimum(t["settleCount"][2], 63))
    assert np.array_equal(s["flags"][3] >> 7, (t["moved"][3] != 0).astype(np.uint8))
    assert np.array_equal(w.temperature()[0], t["temperature"][0])
    assert (types[s["id"]] == SOUP).sum() == 24
    w.close()


def test_upload_tiles_rejects_bad_input(fse):
    t = np.zeros((4, 4), fse.TILE_DTYPE)
    t["id"] = fse.material_find("STONE")
    t["id"][2, 3] = 60000
    w = fse.World(4, 4, seed=1)
    with pytest.raises(fse.FseError):
        w.upload_tiles(t)
    s = w.state()
    assert s["id"][2, 3] == fse.material_find("GENERIC_AIR")
    assert s["id"][0, 0] == fse.material_find("STONE")
    # misaligned fields are refused before any copy
    bad = np.dtype({"names": ["id", "color"], "formats": ["<u4", "<u4"], "offsets": [0, 6], "itemsize": 12})
    with pytest.raises(fse.FseError):
        w.upload_tiles(np.zeros((4, 4), bad))
    with pytest.raises(fse.FseError):
        w.download_tiles(np.zeros((4, 4), bad))
    w.close()
