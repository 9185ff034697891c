"""Render textures (the dirty-pixel task of game::tick, game.cpp:1995-2061) against
the reference's own loop, compiled from the reference tree with stand-in types
(oracle/ref_render.cpp, oracle/Makefile `ref`): the oracle's restatement must give
the same four textures, smoothed flows and moving counts, bit for bit."""
import numpy as np
import pytest


def _scene(o, seed, w=256, h=192):
    rng = np.random.default_rng(seed)
    n_mat = o.material_count()
    ids = rng.integers(0, n_mat, size=(h, w)).astype(np.uint16)
    ids[rng.random((h, w)) < 0.3] = o.find("GENERIC_AIR")
    colours = rng.integers(0, 1 << 32, size=(h, w), dtype=np.uint64).astype(np.uint32)
    dirty = (rng.random((h, w)) < 0.6).astype(np.uint8)
    flow = rng.integers(-8 << 16, 8 << 16, size=(h, w, 2)).astype(np.int32)
    flow[rng.random((h, w)) < 0.2] = 0
    flow[rng.random((h, w)) < 0.02] = rng.integers(-(1 << 31), (1 << 31) - 1, size=2)  # wrapped sums
    prev = rng.normal(0, 4, size=(h, w, 2)).astype(np.float32)
    tiny = rng.random((h, w, 2)) < 0.05
    prev[tiny] = rng.choice(np.array([1e-40, -1e-39, 1e-38, -3e-37, 0.0, -0.0], np.float32), size=int(tiny.sum()))
    return ids, colours, dirty, flow, prev


def test_oracle_render_matches_reference_loop(oracle_mod):
    from oracle.binding import build_reference_render, reference_render_dirty

    lib = build_reference_render()
    if lib is None:
        pytest.skip("reference tree absent")
    o = oracle_mod.Oracle()
    o.reset_materials()
    try:
        # a liquid with iterations 0: 3.0 / iterations is infinite
        o.register(0, "inf", "TEST_INF_LIQUID", 3, 0, 200, 1.0, 0, 0, 0x11223344, 0x00FF00)
        mats = np.array([o.material(i) for i in range(o.material_count())])
        types, iters, alpha, emit = mats[:, 0], mats[:, 2], mats[:, 5], mats[:, 8].astype(np.uint32)
        fire = o.find("FIRE")
        for seed in range(4):
            ids, colours, dirty, flow, prev = _scene(o, seed)
            h, w = ids.shape
            ow = oracle_mod.OracleWorld(w, h, 128, 3, 1)
            z = np.zeros((h, w), np.int32)
            ow.set_state({"id": ids, "colour": colours, "scalar": z, "flags": np.zeros((h, w), np.uint8),
                          "diff": z})
            ow.render_enable()
            ow.render_set(dirty, flow, prev)
            moving = ow.render_dirty()
            fx = flow[..., 0].astype(np.float32) * np.float32(1.0 / 65536.0)
            fy = flow[..., 1].astype(np.float32) * np.float32(1.0 / 65536.0)
            tex, rfx, rfy, rpx, rpy, rmov = reference_render_dirty(
                lib, ids, colours, dirty, fx, fy, prev[..., 0], prev[..., 1], (types, alpha, emit, iters), fire)
            for k, t in ((0, tex[0]), (1, tex[2]), (2, tex[1]), (3, tex[3])):  # pixels, emission, fire, flow
                got = ow.render_texture(k)
                assert np.array_equal(got, t), (seed, k, int((got != t).any(axis=2).sum()))
            pf = ow.render_pflow()
            soup = (types[ids] == 3) & (dirty == 1)
            assert np.array_equal(pf[..., 0][soup].view(np.uint32), rpx[soup].view(np.uint32)), seed
            assert np.array_equal(pf[..., 1][soup].view(np.uint32), rpy[soup].view(np.uint32)), seed
            assert np.array_equal(moving.astype(np.uint16), rmov[: len(moving)]), seed
            d = dirty == 1
            assert not rfx[d].any() and not rfy[d].any()  # the loop clears the flows it read
    finally:
        o.reset_materials()
