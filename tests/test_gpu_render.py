"""Headless render textures (the dirty-cell pass of game.cpp:1994-2067 and the
particle layer of world::renderCells, world.cpp:2006-2028) against the oracle,
byte for byte, on a world with liquids, fire, lava, steam and free particles."""
import numpy as np
import pytest

from helpers import compare_particles, compare_states, material_types

pytestmark = pytest.mark.gpu

PART = 1
TEXTURES = ("pixels", "emission", "fire", "flow", "cells")


def _render_pair(fse, oracle_mod, w, h, seed):
    world = fse.World(w, h, chunk_size=128, cell_iter=3, seed=seed, render=True)
    world.generate(fse.GEN_MIX, seed)
    ow = oracle_mod.OracleWorld(w, h, 128, 3, seed)
    ow.generate(0, seed)
    ow.render_enable()
    s = world.state()
    rng = np.random.default_rng(seed)
    for name, frac, scalar in (("FIRE", 0.02, 0), ("LAVA", 0.02, 2 * 65536), ("STEAM", 0.02, 0)):
        pick = rng.random(s["id"].shape) < frac
        s["id"][pick] = fse.material_find(name)
        s["scalar"][pick] = scalar
        s["colour"][pick] = 0x00FF7F3F
        s["flags"][pick] = 0
        s["diff"][pick] = 0
    world.upload(s)
    ow.set_state(s)
    n = 6000
    p = np.zeros(n, fse.PARTICLE_DTYPE)
    p["x"] = rng.uniform(-4, w + 4, n).astype(np.float32)  # some outside the world
    p["y"] = rng.uniform(0, h, n).astype(np.float32)
    p["vx"] = rng.normal(0, 1, n).astype(np.float32)
    p["vy"] = rng.normal(0, 1, n).astype(np.float32)
    p["ay"] = np.float32(0.1)
    p["fade_time"] = 60
    p["id"] = fse.material_find("GENERIC_SAND")
    p["colour"] = rng.integers(0, 1 << 32, n, dtype=np.uint64).astype(np.uint32)
    p["bits"][::3] = 2  # temporary: alpha fades with lifetime / fade_time
    p["lifetime"][::3] = rng.integers(1, 90, len(p["lifetime"][::3]))
    world.addCell(p)
    ow.set_particles(p)
    return world, ow


def _compare_textures(world, ow, which, what):
    for k in which:
        g, o = world.render_texture(k), ow.render_texture(k)
        bad = np.argwhere(np.any(g != o, axis=2))
        assert len(bad) == 0, "%s: texture %s differs at %d texels, first (y, x) %s: gpu %s oracle %s" % (
            what, TEXTURES[k], len(bad), tuple(bad[0]), g[tuple(bad[0])], o[tuple(bad[0])])


def test_render_textures_match_the_oracle(fse, oracle_mod):
    types = material_types(fse)
    world, ow = _render_pair(fse, oracle_mod, 320, 256, 91)
    # the first pass paints every cell
    np.testing.assert_array_equal(world.render_dirty(), ow.render_dirty())
    _compare_textures(world, ow, range(4), "initial")
    for t in range(6):
        world.render_cells()
        ow.render_cells()
        _compare_textures(world, ow, [4], "particles %d" % t)
        world.step(1)
        ow.step(1, PART)
        compare_states(world.state(), ow.state(), types, "step %d" % t)
        compare_particles(world.particles(), ow.particles(), "step %d" % t)
        mg, mo = world.render_dirty(), ow.render_dirty()
        np.testing.assert_array_equal(mg, mo, err_msg="moving tiles, step %d" % t)
        assert mg.sum() > 0
        _compare_textures(world, ow, range(4), "step %d" % t)
    # liquids flowed, so the flow texture has been painted somewhere
    assert (world.render_texture(3)[..., 3] == 255).any()
    # fire cells painted the fire texture
    assert (world.render_texture(2)[..., 3] > 0).any() or not (ow.state()["id"] == fse.material_find("FIRE")).any()


def test_render_needs_a_render_world(fse):
    w = fse.World(128, 128, seed=1)
    with pytest.raises(fse.FseError):
        w.render_dirty()
    w.close()


def test_png_of_a_texture(fse, tmp_path):
    w = fse.World(160, 128, seed=5, render=True)
    w.generate(fse.GEN_MIX, 5)
    w.step(2)
    w.render_dirty()
    px = w.render_texture(fse.TEX_PIXELS)
    path = tmp_path / "pixels.png"
    fse.write_png(str(path), px)
    data = path.read_bytes()
    assert data[:8] == b"\x89PNG\r\n\x1a\n" and len(data) > 100
    w.close()
