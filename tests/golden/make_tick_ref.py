"""Generates tests/golden/tick_ref.json: digests of scenes ticked by the reference's own world::tick.

oracle/Makefile (target `ref`) compiles world::tick (source/engine/world.cpp:
1036-1948) unchanged with the pieces of the reference it calls
(oracle/ref_tick.cpp); this script runs it on the seeded scenes of
tests/tick_cases.py, with the oracle's material table and draws, and records a
SHA-256 of every result (materials, colours, temperatures, moved flags, spawned
particles), so that the oracle can be checked against the reference's results on
machines without the reference tree. Run from the repository root:
python tests/golden/make_tick_ref.py
"""
import json
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))

import oracle  # noqa: E402
from oracle.binding import build_reference_tick  # noqa: E402
from test_tick_ref import digest, run_reference  # noqa: E402
from tick_cases import CASES, setup_materials  # noqa: E402


def main():
    lib = build_reference_tick()
    if lib is None:
        raise SystemExit("the reference tree is needed")
    oracle.build_oracle()
    o = oracle.Oracle()
    ids = setup_materials(o)
    out = {}
    for case in CASES:
        ri, rc, rt, rm, rp = run_reference(oracle, lib, ids, case)
        out["%d_%d_%d_%s_%d_%d" % case] = {"digest": digest(ri, rc, rt, rm, rp), "particles": int(len(rp))}
    o.reset_materials()
    path = os.path.join(ROOT, "tests", "golden", "tick_ref.json")
    with open(path, "w") as f:
        json.dump(out, f, indent=1, sort_keys=True)
    print(path)


if __name__ == "__main__":
    main()
