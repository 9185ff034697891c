"""Generates tests/golden/pack.npz: chunk .pack files made by the reference's own LZ4.

The reference's vendored LZ4 1.9.4 (source/libs/lz4/lz4.c, compiled in place by
oracle/Makefile `ref`) compresses each chunk's MaterialInstanceData buffer with
LZ4_compress_fast(..., 10) exactly as Chunk::ChunkWrite does (chunk.cpp:219-330),
so machines without the reference tree can check that the device decoder reads
the reference's files. The fixture also freezes a digest of the oracle's own
.pack output for the same world. Run from the repository root:
python tests/golden/make_pack_golden.py
"""
import hashlib
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))

import oracle  # noqa: E402
from oracle.binding import ReferenceLZ4, build_reference_lz4  # noqa: E402
from pack_cases import pack_with, sample_world  # noqa: E402

W, H, SEED, PHASE = 256, 192, 77, 3


def main():
    lib = build_reference_lz4()
    if lib is None:
        raise SystemExit("the reference tree is needed to generate these fixtures")
    lz4 = ReferenceLZ4(lib)
    oracle.Oracle().reset_materials()
    ow = sample_world(oracle, W, H, SEED)
    st = ow.state()
    t = ow.temperature()
    data, offs = pack_with(lambda b: lz4.compress(b, 10), st["id"], st["colour"], t, PHASE)
    mine, moffs = ow.pack(PHASE)
    out = {"params": np.array([W, H, SEED, PHASE], np.int64), "ref_data": data, "ref_offsets": offs,
           "id": st["id"], "colour": st["colour"], "temperature": t,
           "oracle_digest": np.array(hashlib.sha256(mine.tobytes() + moffs.tobytes()).hexdigest())}
    np.savez_compressed(os.path.join(os.path.dirname(os.path.abspath(__file__)), "pack.npz"), **out)
    print("wrote", len(offs) - 1, "chunks,", len(data), "bytes (oracle:", len(mine), ")")


if __name__ == "__main__":
    main()
