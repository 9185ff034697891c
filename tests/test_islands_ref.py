"""physicsCheck against the reference's own code.

oracle/Makefile `ref` compiles world::physicsCheck and its flood fill
(source/engine/world.cpp:3330-3430) unchanged, with stand-ins that record the rigid
body's image and position (oracle/ref_physics.cpp). From seed cells on solid blobs of
every size around the 10- and 1000-cell limits, the oracle must cut exactly the same
cells and hand back the same bounding-box image at the same origin. The device
island kernels are checked against the oracle by tests/test_gpu_islands.py.
"""
import hashlib
import json
import os

import numpy as np
import pytest

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "islands_ref.json")
SEEDS = [1, 2, 3]


def seed_cells(types_of, ids, starts, seed):
    h, w = ids.shape
    rng = np.random.default_rng(100 + seed)
    solid_cells = np.argwhere(types_of[ids] == 1)
    cells = starts + [tuple(solid_cells[i]) for i in rng.choice(len(solid_cells), 30, replace=False)]
    return cells + [(0, 0), (h - 1, w - 1)] + [tuple(rng.integers(0, (h, w))) for _ in range(10)]


def result_digest(types_after, img, origin):
    hs = hashlib.sha256(np.ascontiguousarray(types_after, np.uint8).tobytes())
    if img is not None:
        hs.update(np.ascontiguousarray(img, "<u4").tobytes())
        hs.update(np.array(origin, "<i4").tobytes())
    return hs.hexdigest()


def oracle_run(oracle_mod, seed):
    """(seed cells, digests of the oracle's results) of one scene, checks in order."""
    o = oracle_mod.Oracle()
    o.reset_materials()
    types_of = np.array([o.material(i)[0] for i in range(o.material_count())], np.uint8)
    ids, colours, starts = _scene(o, seed)
    h, w = ids.shape
    z = np.zeros((h, w), np.int32)
    ow = oracle_mod.OracleWorld(w, h, 128, 3, 1)
    ow.set_state({"id": ids, "colour": colours, "scalar": z, "flags": np.zeros((h, w), np.uint8), "diff": z})
    out = []
    for (y, x) in seed_cells(types_of, ids, starts, seed):
        n, bbox, img = ow.physics_check(int(x), int(y))
        org = (int(bbox[0]), int(bbox[1])) if img is not None else None
        out.append(result_digest(types_of[ow.state()["id"]], img, org))
    return out


def _scene(o, seed, w=320, h=256):
    rng = np.random.default_rng(seed)
    solid, stone, sand, water, air = (o.find(n) for n in ("GENERIC_SOLID", "STONE", "GENERIC_SAND", "WATER",
                                                          "GENERIC_AIR"))
    ids = np.full((h, w), air, np.uint16)
    u = rng.random((h, w))
    ids[u < 0.10] = sand
    ids[(u >= 0.10) & (u < 0.15)] = water
    # solid blobs, one per 80 x 64 region (so they never touch): random walks of
    # sizes around the 10- and 1000-cell limits, in two solid materials
    starts = []
    for k, size in enumerate([1, 5, 10, 11, 40, 300, 999, 1000, 1001, 1500, 2500, 12]):
        rx, ry = (k % 4) * 80, (k // 4) * 64
        x, y = rx + 40, ry + 32
        starts.append((y, x))
        cells = set()
        while len(cells) < size:
            cells.add((x, y))
            d = int(rng.integers(0, 4))
            x = min(max(x + (1, 0, -1, 0)[d], rx + 1), rx + 78)
            y = min(max(y + (0, 1, 0, -1)[d], ry + 1), ry + 62)
        for (cx, cy) in cells:
            ids[cy, cx] = solid if k % 2 else stone
    colours = rng.integers(0, 2 ** 32, (h, w), dtype=np.uint64).astype(np.uint32)
    return ids, colours, starts


@pytest.mark.parametrize("seed", SEEDS)
def test_oracle_physics_check_matches_reference(oracle_mod, seed):
    from oracle.binding import build_reference_physics, reference_physics_check

    lib = build_reference_physics()
    if lib is None:
        pytest.skip("reference tree absent")
    o = oracle_mod.Oracle()
    o.reset_materials()
    types_of = np.array([o.material(i)[0] for i in range(o.material_count())], np.uint8)
    ids, colours, starts = _scene(o, seed)
    h, w = ids.shape
    seeds = seed_cells(types_of, ids, starts, seed)
    z = np.zeros((h, w), np.int32)
    ow = oracle_mod.OracleWorld(w, h, 128, 3, 1)
    ow.set_state({"id": ids, "colour": colours, "scalar": z, "flags": np.zeros((h, w), np.uint8), "diff": z})
    cut = 0
    for (y, x) in seeds:
        st = ow.state()
        ref_types, ref_img, ref_org = reference_physics_check(lib, types_of[st["id"]], st["colour"], int(x), int(y))
        n, bbox, img = ow.physics_check(int(x), int(y))
        got_types = types_of[ow.state()["id"]]
        assert np.array_equal(got_types, ref_types), (seed, x, y)
        if ref_img is None:
            assert img is None or n <= 10, (seed, x, y, n)
        else:
            cut += 1
            assert n > 10 and np.array_equal(img, ref_img), (seed, x, y)
            assert (int(bbox[0]), int(bbox[1])) == ref_org, (seed, x, y)
    assert cut > 0


@pytest.mark.parametrize("seed", SEEDS)
def test_oracle_physics_check_matches_reference_digests(oracle_mod, seed):
    """The reference's results frozen by tests/golden/make_islands_ref.py."""
    golden = json.load(open(GOLDEN))
    assert oracle_run(oracle_mod, seed) == golden[str(seed)]
