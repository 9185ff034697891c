"""Free particles (world::tickCells, world.cpp:2030-2195) against the reference's own code.

oracle/Makefile `ref` compiles the reference's world::tickCells with stand-in types
(oracle/ref_particles.cpp) when the reference tree is present; the oracle's
particle update must match it bit for bit (grid writes and every surviving
particle) on scenes where no two particles meet within a tick
(tests/particle_cases.py). tests/golden/particles.npz holds the reference's
results for machines without the tree.
"""
import os

import numpy as np
import pytest

from particle_cases import H, W, scene

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "particles.npz")


def _oracle_world(oracle_mod, ids, col, amt, types, parts):
    ow = oracle_mod.OracleWorld(W, H, 128, 3, 1)
    z = np.zeros((H, W), np.int32)
    ow.set_state({"id": ids, "colour": col, "scalar": np.where(types[ids] == 3, amt, 0).astype(np.int32),
                  "flags": np.zeros((H, W), np.uint8), "diff": z})
    ow.set_particles(parts)
    return ow


def test_oracle_matches_reference_fixtures(oracle_mod):
    g = np.load(GOLDEN)
    o = oracle_mod.Oracle()
    o.reset_materials()
    types = np.array([o.material(i)[0] for i in range(o.material_count())], np.int32)
    assert np.array_equal(types, g["types"])
    for s in g["seeds"]:
        ids, col, amt = g["%d_ids" % s], g["%d_col" % s], g["%d_amt" % s]
        ow = _oracle_world(oracle_mod, ids, col, amt, types, g["%d_parts" % s])
        for t in range(int(g["ticks"])):
            ow.particles_tick()
            st = ow.state()
            cells = g["%d_t%d_cells" % (s, t)]
            ids = ids.copy().ravel()
            col = col.copy().ravel()
            amt = amt.copy().ravel()
            ids[cells], col[cells], amt[cells] = g["%d_t%d_ids" % (s, t)], g["%d_t%d_col" % (s, t)], \
                g["%d_t%d_amt" % (s, t)]
            ids, col, amt = ids.reshape(H, W), col.reshape(H, W), amt.reshape(H, W)
            assert np.array_equal(st["id"], ids) and np.array_equal(st["colour"], col), (s, t)
            soup = types[ids] == 3
            assert np.array_equal(st["scalar"][soup], amt[soup]), (s, t)
            assert ow.particles().tobytes() == g["%d_t%d_parts" % (s, t)].tobytes(), (s, t)


def test_oracle_matches_reference_function(oracle_mod):
    from oracle.binding import build_reference_cells, reference_tick_cells

    lib = build_reference_cells()
    if lib is None:
        pytest.skip("reference tree absent")
    o = oracle_mod.Oracle()
    o.reset_materials()
    types = np.array([o.material(i)[0] for i in range(o.material_count())], np.int32)
    moved = removed = 0
    for seed in range(8):
        ids, col, amt, p = scene(o, seed)
        ow = _oracle_world(oracle_mod, ids, col, amt, types, p)
        for t in range(3):
            ids2, col2, amt2, _, p2 = reference_tick_cells(lib, ids, col, amt, types, p)
            ow.particles_tick()
            st = ow.state()
            assert np.array_equal(st["id"], ids2) and np.array_equal(st["colour"], col2), (seed, t)
            soup = types[ids2] == 3
            assert np.array_equal(st["scalar"][soup], amt2[soup]), (seed, t)
            assert ow.particles().tobytes() == p2.tobytes(), (seed, t)
            moved += int((ids2 != ids).sum())
            removed += len(p) - len(p2)
            ids, col, amt, p = ids2, col2, amt2, p2
    assert moved > 20 and removed > 20  # deposits and removals were exercised


def _contested(oracle_mod, g, s, types):
    from particle_cases import CH, CW

    ids, col, amt = g["%d_ids" % s], g["%d_col" % s], g["%d_amt" % s]
    ow = oracle_mod.OracleWorld(CW, CH, 128, 3, 1)
    z = np.zeros((CH, CW), np.int32)
    ow.set_state({"id": ids, "colour": col, "scalar": np.where(types[ids] == 3, amt, 0).astype(np.int32),
                  "flags": np.zeros((CH, CW), np.uint8), "diff": z})
    ow.set_particles(g["%d_parts" % s])
    return ow, ids, col, amt


def test_oracle_matches_reference_on_contested_scenes(oracle_mod):
    """Particles as dense as on the bench world: flights stop at cells deposited
    earlier in the same tick, previous cells fill up and spiral searches compete.
    The oracle runs the particles in list order, as the reference does, and matches
    its results (tests/golden/particles_contested.npz, made by the reference's own
    tickCells) bit for bit."""
    from particle_cases import CH, CW

    g = np.load(os.path.join(os.path.dirname(GOLDEN), "particles_contested.npz"))
    o = oracle_mod.Oracle()
    o.reset_materials()
    types = np.array([o.material(i)[0] for i in range(o.material_count())], np.int32)
    assert np.array_equal(types, g["types"])
    deposits = 0
    for s in g["seeds"]:
        ow, ids, col, amt = _contested(oracle_mod, g, s, types)
        for t in range(int(g["ticks"])):
            ow.particles_tick()
            st = ow.state()
            cells = g["%d_t%d_cells" % (s, t)]
            ids, col, amt = ids.copy().ravel(), col.copy().ravel(), amt.copy().ravel()
            ids[cells], col[cells], amt[cells] = g["%d_t%d_ids" % (s, t)], g["%d_t%d_col" % (s, t)], \
                g["%d_t%d_amt" % (s, t)]
            ids, col, amt = ids.reshape(CH, CW), col.reshape(CH, CW), amt.reshape(CH, CW)
            assert np.array_equal(st["id"], ids) and np.array_equal(st["colour"], col), (s, t)
            soup = types[ids] == 3
            assert np.array_equal(st["scalar"][soup], amt[soup]), (s, t)
            assert ow.particles().tobytes() == g["%d_t%d_parts" % (s, t)].tobytes(), (s, t)
            deposits += len(cells)
    assert deposits > 1000
