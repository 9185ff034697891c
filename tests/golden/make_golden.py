"""Generates tests/golden/golden.npz from the CPU oracle.

The reference ships no test vectors for the world tick (its tests cover FFI,
reflection and promises only), so these fixtures freeze the oracle's output on small
seeded worlds: a regression in the oracle or in its material table shows up as a
digest mismatch. Run from the repository root: python tests/golden/make_golden.py
"""
import hashlib
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import OracleWorld, Oracle  # noqa: E402

CASES = [
    # name, w, h, seed, generator kind (0 mix, 1 zipf8), steps, order (0 seq, 1 part)
    ("mix_part", 256, 192, 1234, 0, 10, 1),
    ("mix_seq", 256, 192, 1234, 0, 10, 0),
    ("zipf_part", 192, 192, 42, 1, 6, 1),
    ("ragged_part", 200, 136, 7, 0, 12, 1),
]


def digest(state, parts):
    h = hashlib.sha256()
    for k in ("id", "colour", "scalar", "flags"):
        h.update(np.ascontiguousarray(state[k]).tobytes())
    soup = np.isin(state["id"], [3, 15, 16, 19, 30])
    h.update(np.ascontiguousarray(np.where(soup, state["diff"], 0)).tobytes())
    # the first 56 bytes of each record: the fields the fixtures were made with (the
    # temperature a SOUP particle carries is checked by tests/test_temperature.py)
    h.update(np.ascontiguousarray(parts).view(np.uint8).reshape(len(parts), parts.dtype.itemsize)[:, :56].tobytes())
    return h.hexdigest()


def main():
    Oracle().reset_materials()
    out = {"names": np.array([c[0] for c in CASES])}
    for name, w, h, seed, kind, steps, order in CASES:
        ow = OracleWorld(w, h, 128, 3, seed)
        ow.generate(kind, seed)
        ow.step(steps, order)
        s = ow.state()
        out[name + "_params"] = np.array([w, h, seed, kind, steps, order], np.int64)
        out[name + "_digest"] = np.array(digest(s, ow.particles()))
        out[name + "_id"] = s["id"]
    np.savez_compressed(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden.npz"), **out)
    print("wrote", len(CASES), "cases")


if __name__ == "__main__":
    main()
