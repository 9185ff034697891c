"""Generates tests/golden/islands_ref.json: digests of the reference's own physicsCheck results.

oracle/Makefile (target `ref`) compiles world::physicsCheck and its flood fill
(source/engine/world.cpp:3330-3430) unchanged (oracle/ref_physics.cpp); this script
runs them on the seeded scenes of tests/test_islands_ref.py, one check after another
from the same seed cells, and records a SHA-256 of each result (the grid's physics
types after the check, and the rigid body's image and origin when one is made).
Run from the repository root: python tests/golden/make_islands_ref.py
"""
import json
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))

import numpy as np  # noqa: E402

import oracle  # noqa: E402
from oracle.binding import build_reference_physics, reference_physics_check  # noqa: E402
from test_islands_ref import SEEDS, _scene, result_digest, seed_cells  # noqa: E402


def main():
    lib = build_reference_physics()
    if lib is None:
        raise SystemExit("the reference tree is needed")
    oracle.build_oracle()
    o = oracle.Oracle()
    o.reset_materials()
    types_of = np.array([o.material(i)[0] for i in range(o.material_count())], np.uint8)
    out = {}
    for seed in SEEDS:
        ids, colours, starts = _scene(o, seed)
        types = types_of[ids]
        res = []
        for (y, x) in seed_cells(types_of, ids, starts, seed):
            types, img, org = reference_physics_check(lib, types, colours, int(x), int(y))
            res.append(result_digest(types, img, org))
        out[str(seed)] = res
    path = os.path.join(ROOT, "tests", "golden", "islands_ref.json")
    with open(path, "w") as f:
        json.dump(out, f, indent=1)
    print(path)


if __name__ == "__main__":
    main()
