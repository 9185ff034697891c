"""Generates tests/golden/objects.npz: rigid-body stamps and readbacks made by the
reference's own loops of game::tick (game.cpp:1766-1813, 1907-1967), compiled from
the reference tree with stand-in types by oracle/Makefile `ref` (see
oracle/ref_objects.cpp). Scenes: the oracle's generated mix world (seeded, plain C)
and the boxes of tests/object_cases.py; the boxes are frozen in the fixture.
Run from the repository root: python tests/golden/make_objects_golden.py
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))

import oracle  # noqa: E402
from oracle.binding import (BODY_DTYPE, build_reference_objects, reference_object_readback,  # noqa: E402
                            reference_object_stamp)
from object_cases import H, W, bodies  # noqa: E402

SEEDS = [11, 12, 13]


def main():
    lib = build_reference_objects()
    if lib is None:
        raise SystemExit("the reference tree is needed to generate these fixtures")
    o = oracle.Oracle()
    o.reset_materials()
    mats = np.array([o.material(i) for i in range(o.material_count())])
    types, alpha = mats[:, 0], mats[:, 5]
    air, obj = o.find("GENERIC_AIR"), o.find("GENERIC_OBJECT")
    out = {"seeds": np.array(SEEDS), "types": types}
    for s in SEEDS:
        ow = oracle.OracleWorld(W, H, 128, 3, s)
        ow.generate(0, s)
        st = ow.state()
        b = bodies(s, BODY_DTYPE, obj)
        i1, c1, parts, counts = reference_object_stamp(lib, st["id"], st["colour"], types, alpha, air, b)
        i2, c2, back = reference_object_readback(lib, i1, c1, types, alpha, air, b)
        ch1 = np.flatnonzero((i1 != st["id"]) | (c1 != st["colour"]))
        ch2 = np.flatnonzero((i2 != i1) | (c2 != c1))
        out.update({"%d_bodies" % s: b, "%d_stamp_cells" % s: ch1, "%d_stamp_ids" % s: i1.ravel()[ch1],
                    "%d_stamp_col" % s: c1.ravel()[ch1], "%d_parts" % s: parts.view(np.uint32),
                    "%d_counts" % s: counts, "%d_back_cells" % s: ch2, "%d_back_ids" % s: i2.ravel()[ch2],
                    "%d_back" % s: back})
    np.savez_compressed(os.path.join(os.path.dirname(os.path.abspath(__file__)), "objects.npz"), **out)
    print("wrote", len(SEEDS), "scenes")


if __name__ == "__main__":
    main()
