"""The tick zone (world::tickZone, world.hpp:138) against the reference's own code.

The game ticks the world less a chunk on each side (game.cpp:1629-1636); the tick's
chunks then start at the zone's corner (world.cpp:1078-1079), particles outside the
zone stay as they are (world.cpp:2061) and the temperature step changes the zone's
cells only (world.cpp:1952-2001). The reference's world::tick, world::tickCells and
world::tickTemperature, compiled unchanged (oracle/Makefile `ref`), are run with a
zone and the oracle with the same zone must agree bit for bit: the game's zone and
one that is not chunk-aligned, on the f32 liquid scene (every rule of the tick),
the contested particle scene and a temperature scene.
tests/golden/tick_zone_ref.json keeps digests of the reference's ticks for the
device test on machines without the reference tree.
"""
import json
import os

import numpy as np
import pytest

from oracle.binding import ORDER_SEQ
from test_tick_ref_f32 import NAMES, START_TICK, digest, result_of_planes
from tick_cases import scene_f32, setup_materials

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "tick_zone_ref.json")

# (w, h, seed, cell_iter, ticks, zone)
ZONE_CASES = [
    (512, 384, 31, 3, 2, (128, 128, 256, 128)),  # the game's zone: a chunk off every side
    (512, 384, 32, 3, 2, (37, 21, 300, 200)),    # not chunk-aligned; its chunks stay inside the world
]


def zone_key(case):
    w, h, seed, ci, nt, z = case
    return "%d_%d_%d_%d_%d_%d_%d_%d_%d" % (w, h, seed, ci, nt, *z)


def run_oracle(oracle_mod, ids_d, case):
    w, h, seed, ci, nt, zone = case
    st = scene_f32(ids_d, w, h, seed)
    ow = oracle_mod.OracleWorld(w, h, 128, ci, seed)
    ow.set_f32(True)
    ow.set_state(st)
    ow.set_temperature(st["temperature"])
    ow.set_tick_zone(*zone)
    ow.tick_count = START_TICK
    for _ in range(nt):
        ow.tick(order=ORDER_SEQ)
    return result_of_planes(ids_d, ow.state(), ow.temperature(), ow.particles())


def run_reference(oracle_mod, lib, ids_d, case):
    from test_tick_ref_f32 import SETTLE_MAX
    from oracle.binding import reference_world_tick_fluid

    w, h, seed, ci, nt, zone = case
    st = scene_f32(ids_d, w, h, seed)
    ri, rc, rt, rm, ra, rd, rs, rp, _ = reference_world_tick_fluid(
        lib, oracle_mod.Oracle(), st["id"], st["colour"], st["temperature"].astype(np.int32), st["flags"] >> 7,
        st["amount"], st["fluid_diff"], st["settle"], ci, seed, START_TICK, nt, zone=zone)
    soup = np.isin(ri, [ids_d["WATER"], ids_d["LAVA"]])
    psoup = np.isin(rp[:, 0], [ids_d["WATER"], ids_d["LAVA"]])
    rp = rp.copy()
    rp[~psoup, 16] = 0
    return (ri, rc, rt, rm, np.where(soup, ra.view(np.int32), 0).astype(np.int32),
            np.where(soup, rd.view(np.int32), 0).astype(np.int32),
            np.where(soup, np.minimum(rs, SETTLE_MAX), 0).astype(np.uint8), rp)


@pytest.fixture()
def ids(oracle_mod):
    o = oracle_mod.Oracle()
    yield setup_materials(o)
    o.reset_materials()


@pytest.mark.parametrize("case", ZONE_CASES, ids=[zone_key(c) for c in ZONE_CASES])
def test_zone_tick_matches_reference(oracle_mod, ids, case):
    from oracle.binding import build_reference_tick

    lib = build_reference_tick()
    if lib is None:
        pytest.skip("reference tree absent")
    ref = run_reference(oracle_mod, lib, ids, case)
    got = run_oracle(oracle_mod, ids, case)
    for name, a, b in zip(NAMES, ref, got):
        assert a.shape == b.shape, name
        bad = np.argwhere(a != b)
        assert len(bad) == 0, "%s differs at %d places, first %s" % (name, len(bad), bad[0].tolist())
    # cells farther than a rule's reach (5 cells) from the zone's chunks never change
    w, h, seed, ci, nt, (zx, zy, zw, zh) = case
    st = scene_f32(ids, w, h, seed)
    outside = np.ones((h, w), bool)
    outside[max(0, zy - 5):zy + -(-zh // 128) * 128 + 5, max(0, zx - 5):zx + -(-zw // 128) * 128 + 5] = False
    assert np.array_equal(got[0][outside], st["id"][outside])
    assert not np.array_equal(got[0][~outside], st["id"][~outside])


@pytest.mark.parametrize("case", ZONE_CASES, ids=[zone_key(c) for c in ZONE_CASES])
def test_zone_tick_matches_reference_digests(oracle_mod, ids, case):
    golden = json.load(open(GOLDEN))
    got = run_oracle(oracle_mod, ids, case)
    assert digest(got) == golden[zone_key(case)]["digest"]


def test_zone_particles_match_reference(oracle_mod):
    from oracle.binding import build_reference_cells, reference_tick_cells
    from particle_cases import CH, CW, contested_scene

    lib = build_reference_cells()
    if lib is None:
        pytest.skip("reference tree absent")
    o = oracle_mod.Oracle()
    o.reset_materials()
    types = np.array([o.material(i)[0] for i in range(o.material_count())], np.int32)
    zone = (64, 48, 200, 120)
    ids_, col, amt, p = contested_scene(o, 301)
    ow = oracle_mod.OracleWorld(CW, CH, 128, 3, 1)
    z = np.zeros((CH, CW), np.int32)
    ow.set_state({"id": ids_, "colour": col, "scalar": np.where(types[ids_] == 3, amt, 0).astype(np.int32),
                  "flags": np.zeros((CH, CW), np.uint8), "diff": z})
    ow.set_particles(p)
    ow.set_tick_zone(*zone)
    kept = 0
    for _ in range(2):
        ids2, col2, amt2, _, p2 = reference_tick_cells(lib, ids_, col, amt, types, p, zone=zone)
        ow.particles_tick()
        st = ow.state()
        assert np.array_equal(st["id"], ids2) and np.array_equal(st["colour"], col2)
        soup = types[ids2] == 3
        assert np.array_equal(st["scalar"][soup], amt2[soup])
        assert ow.particles().tobytes() == p2.tobytes()
        inside = (p2["x"] >= zone[0]) & (p2["x"] < zone[0] + zone[2]) & (p2["y"] >= zone[1]) & \
                 (p2["y"] < zone[1] + zone[3])
        kept += int((~inside).sum())
        ids_, col, amt, p = ids2, col2, amt2, p2
    assert kept > 1000  # particles outside the zone stayed


def test_zone_temperature_matches_reference(oracle_mod):
    from oracle.binding import build_reference_temperature, reference_tick_temperature
    from temperature_cases import CASES, case_inputs, material_params

    lib = build_reference_temperature()
    if lib is None:
        pytest.skip("reference tree absent")
    o = oracle_mod.Oracle()
    o.reset_materials()
    mat, temp = case_inputs(o, CASES[0])
    add, cs, co = material_params(o)
    h, w = mat.shape
    pm = np.zeros((h + 2, w + 2), np.uint16)
    pt = np.zeros((h + 2, w + 2), np.int16)
    pm[1:-1, 1:-1] = mat
    pt[1:-1, 1:-1] = temp
    zone = (9, 5, w - 20, h - 12)
    ref = reference_tick_temperature(lib, pm, pt, add, cs, co, zone)
    ow = oracle_mod.OracleWorld(w + 2, h + 2, 128, 3, 1)
    z32 = np.zeros((h + 2, w + 2), np.int32)
    ow.set_state({"id": pm, "colour": z32.view(np.uint32), "scalar": z32, "flags": np.zeros((h + 2, w + 2), np.uint8),
                  "diff": z32})
    ow.set_temperature(pt)
    ow.set_tick_zone(*zone)
    ow.tick_temperature()
    got = ow.temperature()
    assert np.array_equal(got, ref)
    assert not np.array_equal(got, pt)
