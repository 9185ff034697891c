"""Generates tests/golden/tick_ref_f32.json: digests of liquid scenes ticked by the
reference's own world::tick with their f32 liquid state.

oracle/Makefile (target `ref`) compiles world::tick (source/engine/world.cpp:
1036-1948) unchanged with the pieces of the reference it calls
(oracle/ref_tick.cpp); this script runs it on the seeded f32 liquid scenes of
tests/tick_cases.py (every cell's fluidAmount, fluidAmountDiff and settleCount
given), with the oracle's material table and draws, and records a SHA-256 of every
result (materials, colours, temperatures, moved flags, liquid amounts, diffs and
settle counts, spawned particles with their amounts), so that the oracle and the
device can be checked against the reference's results on machines without the
reference tree. Run from the repository root:
python tests/golden/make_tick_ref_f32.py
"""
import json
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))

import oracle  # noqa: E402
from oracle.binding import build_reference_tick  # noqa: E402
from test_tick_ref_f32 import case_key, digest, run_reference  # noqa: E402
from tick_cases import F32_CASES, setup_materials  # noqa: E402


def main():
    lib = build_reference_tick()
    if lib is None:
        raise SystemExit("the reference tree is needed")
    oracle.build_oracle()
    o = oracle.Oracle()
    ids = setup_materials(o)
    out = {}
    for case in F32_CASES:
        res = run_reference(oracle, lib, ids, case)
        out[case_key(case)] = {"digest": digest(res), "particles": int(len(res[7]))}
    o.reset_materials()
    path = os.path.join(ROOT, "tests", "golden", "tick_ref_f32.json")
    with open(path, "w") as f:
        json.dump(out, f, indent=1, sort_keys=True)
    print(path)


if __name__ == "__main__":
    main()
