"""The device particle update (world::tickCells) against the reference's own results.

tests/golden/particles.npz holds scenes ticked three times by the reference's
world::tickCells compiled from the reference tree (tests/golden/make_particles_golden.py):
the CUDA kernels must reproduce the grid writes and every surviving particle bit for
bit.
"""
import os

import numpy as np
import pytest

from particle_cases import H, W

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "particles.npz")


def test_device_particles_match_reference(fse):
    g = np.load(GOLDEN)
    types = np.array([fse.material_get(i)[0] for i in range(fse.material_count())], np.int32)
    assert np.array_equal(types, g["types"])
    for s in g["seeds"]:
        ids, col, amt = g["%d_ids" % s], g["%d_col" % s], g["%d_amt" % s]
        world = fse.World(W, H, seed=1)
        z = np.zeros((H, W), np.int32)
        world.upload({"id": ids, "colour": col, "scalar": np.where(types[ids] == 3, amt, 0).astype(np.int32),
                      "flags": np.zeros((H, W), np.uint8), "diff": z})
        world.addCell(g["%d_parts" % s])
        for t in range(int(g["ticks"])):
            world.tickCells()
            st = world.state()
            cells = g["%d_t%d_cells" % (s, t)]
            ids, col, amt = ids.copy().ravel(), col.copy().ravel(), amt.copy().ravel()
            ids[cells], col[cells], amt[cells] = g["%d_t%d_ids" % (s, t)], g["%d_t%d_col" % (s, t)], \
                g["%d_t%d_amt" % (s, t)]
            ids, col, amt = ids.reshape(H, W), col.reshape(H, W), amt.reshape(H, W)
            assert np.array_equal(st["id"], ids) and np.array_equal(st["colour"], col), (s, t)
            soup = types[ids] == 3
            assert np.array_equal(st["scalar"][soup], amt[soup]), (s, t)
            assert world.particles().tobytes() == g["%d_t%d_parts" % (s, t)].tobytes(), (s, t)
        world.close()


def test_device_particles_match_reference_on_contested_scenes(fse):
    """Particles as dense as on the 4096 x 2048 bench world, landing on each other's
    deposits (tests/golden/particles_contested.npz, made by the reference's own
    tickCells): the device's fixed-point update reproduces the reference's
    sequential result, grid and every surviving particle, bit for bit."""
    from particle_cases import CH, CW

    g = np.load(os.path.join(os.path.dirname(GOLDEN), "particles_contested.npz"))
    types = np.array([fse.material_get(i)[0] for i in range(fse.material_count())], np.int32)
    assert np.array_equal(types, g["types"])
    for s in g["seeds"]:
        ids, col, amt = g["%d_ids" % s], g["%d_col" % s], g["%d_amt" % s]
        world = fse.World(CW, CH, seed=1)
        z = np.zeros((CH, CW), np.int32)
        world.upload({"id": ids, "colour": col, "scalar": np.where(types[ids] == 3, amt, 0).astype(np.int32),
                      "flags": np.zeros((CH, CW), np.uint8), "diff": z})
        world.addCell(g["%d_parts" % s])
        for t in range(int(g["ticks"])):
            world.tickCells()
            st = world.state()
            cells = g["%d_t%d_cells" % (s, t)]
            ids, col, amt = ids.copy().ravel(), col.copy().ravel(), amt.copy().ravel()
            ids[cells], col[cells], amt[cells] = g["%d_t%d_ids" % (s, t)], g["%d_t%d_col" % (s, t)], \
                g["%d_t%d_amt" % (s, t)]
            ids, col, amt = ids.reshape(CH, CW), col.reshape(CH, CW), amt.reshape(CH, CW)
            assert np.array_equal(st["id"], ids) and np.array_equal(st["colour"], col), (s, t)
            soup = types[ids] == 3
            assert np.array_equal(st["scalar"][soup], amt[soup]), (s, t)
            assert world.particles().tobytes() == g["%d_t%d_parts" % (s, t)].tobytes(), (s, t)
        world.close()
