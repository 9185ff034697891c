"""Rigid-body OBJECT stamping and readback (game.cpp:1766-1813, 1907-1967) against
the reference's own loops, compiled from the reference tree with stand-in types
(oracle/ref_objects.cpp, oracle/Makefile `ref`), and against fixtures they made
(tests/golden/objects.npz): the grid, the displaced particles (tile, position,
order; their velocities come from rand() there), the per-body damping counts and the
cells taken back must match exactly."""
import os

import numpy as np
import pytest

from object_cases import H, W, bodies, particle_rows

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "objects.npz")


def _oracle_run(oracle_mod, seed, b):
    ow = oracle_mod.OracleWorld(W, H, 128, 3, seed)
    ow.generate(0, seed)
    st0 = ow.state()
    n0 = len(ow.particles())
    bs = b.copy()
    ow.object_stamp(bs)
    st1 = ow.state()
    parts = ow.particles()[n0:]
    bb = b.copy()
    ow.object_readback(bb)
    return st0, st1, ow.state(), parts, bs, bb


def test_oracle_matches_reference_fixtures(oracle_mod):
    g = np.load(GOLDEN)
    o = oracle_mod.Oracle()
    o.reset_materials()
    for s in g["seeds"]:
        b = g["%d_bodies" % s]
        st0, st1, st2, parts, bs, bb = _oracle_run(oracle_mod, int(s), b)
        ids = st0["id"].ravel().copy()
        col = st0["colour"].ravel().copy()
        cells = g["%d_stamp_cells" % s]
        ids[cells], col[cells] = g["%d_stamp_ids" % s], g["%d_stamp_col" % s]
        assert np.array_equal(st1["id"].ravel(), ids) and np.array_equal(st1["colour"].ravel(), col), s
        assert np.array_equal(particle_rows(parts), g["%d_parts" % s]), s
        assert np.array_equal(np.stack([bs["n_sand"], bs["n_soup"]], 1), g["%d_counts" % s]), s
        cells = g["%d_back_cells" % s]
        ids[cells] = g["%d_back_ids" % s]
        assert np.array_equal(st2["id"].ravel(), ids), s
        assert np.array_equal(bb["n_recovered"], g["%d_back" % s][:, 0]), s


def test_oracle_matches_reference_loops(oracle_mod):
    from oracle.binding import (BODY_DTYPE, build_reference_objects, reference_object_readback,
                                reference_object_stamp)

    lib = build_reference_objects()
    if lib is None:
        pytest.skip("reference tree absent")
    o = oracle_mod.Oracle()
    o.reset_materials()
    mats = np.array([o.material(i) for i in range(o.material_count())])
    types, alpha = mats[:, 0], mats[:, 5]
    air, obj = o.find("GENERIC_AIR"), o.find("GENERIC_OBJECT")
    displaced = 0
    for s in range(20, 28):
        b = bodies(s, BODY_DTYPE, obj, nb=16)
        st0, st1, st2, parts, bs, bb = _oracle_run(oracle_mod, s, b)
        i1, c1, rparts, counts = reference_object_stamp(lib, st0["id"], st0["colour"], types, alpha, air, b)
        assert np.array_equal(st1["id"], i1) and np.array_equal(st1["colour"], c1), s
        assert np.array_equal(particle_rows(parts), rparts.view(np.uint32)), s
        assert np.array_equal(np.stack([bs["n_sand"], bs["n_soup"]], 1), counts), s
        i2, c2, back = reference_object_readback(lib, i1, c1, types, alpha, air, b)
        assert np.array_equal(st2["id"], i2), s
        assert np.array_equal(bb["n_recovered"], back[:, 0]), s
        displaced += len(parts)
    assert displaced > 100
