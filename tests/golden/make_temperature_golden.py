"""Generates tests/golden/temperature.npz from the reference's own world::tickTemperature.

oracle/Makefile (target `ref`) compiles that one function (source/engine/world.cpp:
1950-2004) from the reference tree; this script runs it on seeded cases and freezes
inputs and outputs, so that the oracle's restatement is checked against the
reference's arithmetic on machines without the reference tree. The world is padded
with one ring of cells at temperature 0 and the tick zone is its interior, which is
how the restatement treats the world's edge (neighbours outside read temperature 0).
Run from the repository root: python tests/golden/make_temperature_golden.py
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))

from oracle.binding import Oracle, build_reference_temperature, reference_tick_temperature  # noqa: E402
from temperature_cases import CASES, case_inputs, material_params  # noqa: E402


def main():
    lib = build_reference_temperature()
    if lib is None:
        raise SystemExit("the reference tree is needed to generate these fixtures")
    o = Oracle()
    out = {"names": np.array([c[0] for c in CASES])}
    for case in CASES:
        name = case[0]
        o.reset_materials()
        mat, temp = case_inputs(o, case)
        add, cs, co = material_params(o)
        h, w = mat.shape
        pm = np.zeros((h + 2, w + 2), np.uint16)
        pt = np.zeros((h + 2, w + 2), np.int16)
        pm[1:-1, 1:-1] = mat
        pt[1:-1, 1:-1] = temp
        res = reference_tick_temperature(lib, pm, pt, add, cs, co, (1, 1, w, h))
        out[name + "_mat"] = mat
        out[name + "_temp"] = temp
        out[name + "_add"] = add
        out[name + "_cs"] = cs
        out[name + "_co"] = co
        out[name + "_out"] = res[1:-1, 1:-1].copy()
    o.reset_materials()
    np.savez_compressed(os.path.join(os.path.dirname(os.path.abspath(__file__)), "temperature.npz"), **out)
    print("wrote", len(CASES), "cases")


if __name__ == "__main__":
    main()
