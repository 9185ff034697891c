"""Solid islands against the oracle: world::physicsCheck (world.cpp:3330-3445) from
single seeds, and every SOLID region at once by connected-component labelling."""
import numpy as np
import pytest

from helpers import compare_states, material_types

pytestmark = pytest.mark.gpu


def _speckled(fse, oracle_mod, w, h, seed, frac):
    """A world of AIR with STONE speckles (regions of every size) and some SAND."""
    world = fse.World(w, h, seed=seed, render=True)
    ow = oracle_mod.OracleWorld(w, h, 128, 3, seed)
    ow.render_enable()
    rng = np.random.default_rng(seed)
    s = world.state()
    s["id"][:] = 0
    s["colour"][:] = 0
    stone = fse.material_find("STONE")
    sand = fse.material_find("GENERIC_SAND")
    pick = rng.random((h, w)) < frac
    s["id"][pick] = stone
    s["colour"][pick] = rng.integers(0, 1 << 24, int(pick.sum()), dtype=np.uint64).astype(np.uint32)
    s["id"][rng.random((h, w)) < 0.05] = sand
    s["scalar"][:] = 0
    s["flags"][:] = 0
    s["diff"][:] = 0
    world.upload(s)
    ow.set_state(s)
    return world, ow


def test_physics_check_matches_the_oracle(fse, oracle_mod):
    types = material_types(fse)
    world, ow = _speckled(fse, oracle_mod, 300, 200, 5, 0.5)
    rng = np.random.default_rng(2)
    cut = 0
    for k in range(60):
        x, y = int(rng.integers(0, 300)), int(rng.integers(0, 200))
        g = world.physicsCheck(x, y)
        o = ow.physics_check(x, y)
        assert g[0] == o[0], "seed %d (%d, %d): gpu cut %d, oracle %d" % (k, x, y, g[0], o[0])
        if g[0]:
            cut += 1
            np.testing.assert_array_equal(g[1], o[1])
            if g[0] > 10:
                np.testing.assert_array_equal(g[2], o[2])
    assert cut > 0
    compare_states(world.state(), ow.state(), types, "after physicsCheck")
    np.testing.assert_array_equal(world.ledger(), ow.ledger())
    # a region of more than 1000 cells is left alone
    big, obig = _speckled(fse, oracle_mod, 128, 128, 9, 1.0)
    assert big.physicsCheck(64, 64)[0] == 0 and obig.physics_check(64, 64)[0] == 0


def test_islands_match_the_oracle(fse, oracle_mod):
    types = material_types(fse)
    for seed, frac, max_cells in ((11, 0.45, 1000), (12, 0.58, 1000), (13, 0.3, 10)):
        world, ow = _speckled(fse, oracle_mod, 333, 257, seed, frac)
        gt, gn = world.islands(max_cells, remove=False)
        ot, on = ow.islands(max_cells, remove=False)
        assert gn == on and gn > 0
        for f in ("root", "cells", "min_x", "min_y", "max_x", "max_y"):
            np.testing.assert_array_equal(gt[f], ot[f], err_msg=f)
        gt, gn = world.islands(max_cells, remove=True)
        ow.islands(max_cells, remove=True)
        compare_states(world.state(), ow.state(), types, "islands removed, seed %d" % seed)
        np.testing.assert_array_equal(world.ledger(), ow.ledger())
        # nothing small is left
        assert world.islands(max_cells)[1] == 0
        # the cut cells are dirty: the render pass repaints them as AIR
        world.render_dirty()
        ow.render_dirty()
        np.testing.assert_array_equal(world.render_texture(0), ow.render_texture(0))


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_device_physics_check_matches_reference_digests(fse, oracle_mod, seed):
    """The device physicsCheck, one check after another from the same seed cells,
    against the digests of the reference's own function (tests/golden/islands_ref.json)."""
    import json

    from test_islands_ref import GOLDEN, _scene, result_digest, seed_cells

    o = oracle_mod.Oracle()
    o.reset_materials()
    types_of = np.array([fse.material_get(i)[0] for i in range(fse.material_count())], np.uint8)
    ids, colours, starts = _scene(o, seed)
    h, w = ids.shape
    z = np.zeros((h, w), np.int32)
    world = fse.World(w, h, seed=1)
    world.upload({"id": ids, "colour": colours, "scalar": z, "flags": np.zeros((h, w), np.uint8), "diff": z})
    got = []
    for (y, x) in seed_cells(types_of, ids, starts, seed):
        n, bbox, img = world.physicsCheck(int(x), int(y))
        org = (int(bbox[0]), int(bbox[1])) if img is not None else None
        got.append(result_digest(types_of[world.state()["id"]], img, org))
    world.close()
    assert got == json.load(open(GOLDEN))[str(seed)]
