"""Generates tests/golden/tick_zone_ref.json: digests of f32 liquid scenes ticked by
the reference's own world::tick with a tick zone.

oracle/Makefile (target `ref`) compiles world::tick (source/engine/world.cpp:
1036-1948) unchanged with the pieces of the reference it calls
(oracle/ref_tick.cpp); this script runs it with world::tickZone set as in
tests/test_tick_zone_ref.py (the game's zone, a chunk off every side, and one that
is not chunk-aligned) and records a SHA-256 of every result, for the device test on
machines without the reference tree. Run from the repository root:
python tests/golden/make_tick_zone_ref.py
"""
import json
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))

import oracle  # noqa: E402
from oracle.binding import build_reference_tick  # noqa: E402
from test_tick_ref_f32 import digest  # noqa: E402
from test_tick_zone_ref import ZONE_CASES, run_reference, zone_key  # noqa: E402
from tick_cases import setup_materials  # noqa: E402


def main():
    lib = build_reference_tick()
    if lib is None:
        raise SystemExit("the reference tree is needed")
    oracle.build_oracle()
    o = oracle.Oracle()
    ids = setup_materials(o)
    out = {}
    for case in ZONE_CASES:
        res = run_reference(oracle, lib, ids, case)
        out[zone_key(case)] = {"digest": digest(res), "particles": int(len(res[7]))}
    o.reset_materials()
    path = os.path.join(ROOT, "tests", "golden", "tick_zone_ref.json")
    with open(path, "w") as f:
        json.dump(out, f, indent=1, sort_keys=True)
    print(path)


if __name__ == "__main__":
    main()
