"""Device OBJECT stamping and readback against the reference's own loops
(tests/golden/objects.npz, made by tests/golden/make_objects_golden.py): the
deferred-acceptance kernel must give the tile-by-tile result exactly."""
import os

import numpy as np
import pytest

from object_cases import H, W, particle_rows

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "objects.npz")


def test_device_objects_match_reference(fse):
    g = np.load(GOLDEN)
    for s in g["seeds"]:
        world = fse.World(W, H, seed=int(s))
        world.generate(fse.GEN_MIX, int(s))
        st0 = world.state()
        b = np.ascontiguousarray(g["%d_bodies" % s]).copy()
        world.object_stamp(b)
        st1 = world.state()
        ids, col = st0["id"].ravel().copy(), st0["colour"].ravel().copy()
        cells = g["%d_stamp_cells" % s]
        ids[cells], col[cells] = g["%d_stamp_ids" % s], g["%d_stamp_col" % s]
        assert np.array_equal(st1["id"].ravel(), ids) and np.array_equal(st1["colour"].ravel(), col), s
        assert np.array_equal(particle_rows(world.particles()), g["%d_parts" % s]), s
        assert np.array_equal(np.stack([b["n_sand"], b["n_soup"]], 1), g["%d_counts" % s]), s
        bb = np.ascontiguousarray(g["%d_bodies" % s]).copy()
        world.object_readback(bb)
        cells = g["%d_back_cells" % s]
        ids[cells] = g["%d_back_ids" % s]
        assert np.array_equal(world.state()["id"].ravel(), ids), s
        assert np.array_equal(bb["n_recovered"], g["%d_back" % s][:, 0]), s
        world.close()
