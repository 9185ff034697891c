"""Generates tests/golden/particles_contested.npz: contested scenes ticked by the
reference's own world::tickCells.

oracle/Makefile (target `ref`) compiles world::tickCells (source/engine/world.cpp:
2030-2195) from the reference tree with stand-in types (oracle/ref_particles.cpp);
this script runs two consecutive ticks of it on the seeded contested scenes of
tests/particle_cases.py, where particles are as dense as on the 4096 x 2048 bench
world and land on each other's deposits, and freezes inputs and outputs, so that
the oracle and the device can be checked against the reference's sequential result
on machines without the reference tree. Run from the repository root:
python tests/golden/make_particles_contested.py
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))

import oracle  # noqa: E402
from oracle.binding import build_reference_cells, reference_tick_cells  # noqa: E402
from particle_cases import contested_scene  # noqa: E402

SEEDS = [201, 202]
TICKS = 2


def main():
    lib = build_reference_cells()
    if lib is None:
        raise SystemExit("the reference tree is needed to generate these fixtures")
    o = oracle.Oracle()
    o.reset_materials()
    types = np.array([o.material(i)[0] for i in range(o.material_count())], np.int32)
    out = {"seeds": np.array(SEEDS), "ticks": np.array(TICKS), "types": types}
    for s in SEEDS:
        ids, col, amt, p = contested_scene(o, s)
        out["%d_ids" % s], out["%d_col" % s], out["%d_amt" % s], out["%d_parts" % s] = ids, col, amt, p
        for t in range(TICKS):
            ids2, col2, amt2, _, p = reference_tick_cells(lib, ids, col, amt, types, p)
            ch = np.flatnonzero((ids2 != ids) | (col2 != col) | (amt2 != amt))
            out["%d_t%d_cells" % (s, t)] = ch
            out["%d_t%d_ids" % (s, t)] = ids2.ravel()[ch]
            out["%d_t%d_col" % (s, t)] = col2.ravel()[ch]
            out["%d_t%d_amt" % (s, t)] = amt2.ravel()[ch]
            out["%d_t%d_parts" % (s, t)] = p
            ids, col, amt = ids2, col2, amt2
    np.savez_compressed(os.path.join(os.path.dirname(os.path.abspath(__file__)), "particles_contested.npz"), **out)
    print("wrote", len(SEEDS), "scenes x", TICKS, "ticks")


if __name__ == "__main__":
    main()
