"""Liquids bit for bit against the reference's own world::tick, with f32 amounts.

With f32 liquid amounts (the oracle's set_f32, the library's FSE_CFG_F32_FLUID) the
oracle's reference-order tick keeps fluidAmount and fluidAmountDiff in the
reference's own float arithmetic (world.cpp:1021-1034, 1269-1567, 1728-1745). The
reference's world::tick is compiled unchanged (oracle/Makefile `ref`) and given the
same grid, every cell's amount, diff and settle count included, and the same
draws: after 1, 3 and 6 ticks of water, lava, sand, gas and stone (flows into air
and into liquid, compression, free fall into particles, the water-on-lava reaction,
evaporation below FLUID_MinValue, liquid swaps) every cell's material, colour,
temperature, moved flag, and every liquid cell's amount, diff and settle count, and
every spawned particle with its amount agree bit for bit.
tests/golden/tick_ref_f32.json keeps digests of the reference's results
(tests/golden/make_tick_ref_f32.py) for the device test on machines without the
reference tree.
"""
import hashlib
import json
import os

import numpy as np
import pytest

from oracle.binding import ORDER_SEQ
from tick_cases import F32_CASES, setup_materials, scene_f32

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "tick_ref_f32.json")
START_TICK = 7
SETTLE_MAX = 63  # this path saturates the settle count at 63 (the reference's u8 wraps at 256)


def case_key(case):
    return "%d_%d_%d_%d_%d" % case


def rows17(ids_d, parts):
    """Particles (the library's or the oracle's records) as the reference harness's
    17-int rows; the liquid amount (last) only for liquid tiles."""
    soup = np.isin(parts["id"], [ids_d["WATER"], ids_d["LAVA"]])
    rows = np.zeros((len(parts), 17), np.int32)
    rows[:, 0] = parts["id"]
    rows[:, 1] = parts["colour"].view(np.int32)
    rows[:, 2] = np.where(soup, parts["temperature"], parts["scalar"])
    for j, k in enumerate(("x", "y", "vx", "vy", "ax", "ay", "target_x", "target_y", "target_force")):
        rows[:, 3 + j] = np.ascontiguousarray(parts[k]).view(np.int32)
    rows[:, 12] = parts["bits"] & 1
    rows[:, 13] = (parts["bits"] >> 1) & 1
    rows[:, 14] = parts["lifetime"]
    rows[:, 15] = parts["fade_time"]
    rows[:, 16] = np.where(soup, parts["scalar"], 0)
    return rows


def result_of_planes(ids_d, st, temps, parts):
    """(id, colour, temperature, moved, amount, diff, settle, rows) of a state whose
    liquid scalars and diffs are f32 bits; non-liquid cells' amount/diff/settle 0."""
    soup = np.isin(st["id"], [ids_d["WATER"], ids_d["LAVA"]])
    return (st["id"], st["colour"], temps.astype(np.int32), (st["flags"] >> 7).astype(np.uint8),
            np.where(soup, st["scalar"], 0).astype(np.int32), np.where(soup, st["diff"], 0).astype(np.int32),
            np.where(soup, st["flags"] & 0x3F, 0).astype(np.uint8), rows17(ids_d, parts))


def run_oracle(oracle_mod, ids_d, case):
    w, h, seed, ci, nt = case
    st = scene_f32(ids_d, w, h, seed)
    ow = oracle_mod.OracleWorld(w, h, 128, ci, seed)
    ow.set_f32(True)
    ow.set_state(st)
    ow.set_temperature(st["temperature"])
    ow.tick_count = START_TICK
    for _ in range(nt):
        ow.tick(order=ORDER_SEQ)
    return result_of_planes(ids_d, ow.state(), ow.temperature(), ow.particles())


def run_reference(oracle_mod, lib, ids_d, case):
    from oracle.binding import reference_world_tick_fluid

    w, h, seed, ci, nt = case
    st = scene_f32(ids_d, w, h, seed)
    ri, rc, rt, rm, ra, rd, rs, rp, _ = reference_world_tick_fluid(
        lib, oracle_mod.Oracle(), st["id"], st["colour"], st["temperature"].astype(np.int32), st["flags"] >> 7,
        st["amount"], st["fluid_diff"], st["settle"], ci, seed, START_TICK, nt)
    soup = np.isin(ri, [ids_d["WATER"], ids_d["LAVA"]])
    psoup = np.isin(rp[:, 0], [ids_d["WATER"], ids_d["LAVA"]])
    rp = rp.copy()
    rp[~psoup, 16] = 0
    return (ri, rc, rt, rm, np.where(soup, ra.view(np.int32), 0).astype(np.int32),
            np.where(soup, rd.view(np.int32), 0).astype(np.int32),
            np.where(soup, np.minimum(rs, SETTLE_MAX), 0).astype(np.uint8), rp)


def digest(res):
    h = hashlib.sha256()
    for a, dt in zip(res, ("<u2", "<u4", "<i4", "u1", "<i4", "<i4", "u1", "<i4")):
        h.update(np.ascontiguousarray(a, dt).tobytes())
    return h.hexdigest()


NAMES = ("id", "colour", "temperature", "moved", "amount", "diff", "settle", "particles")


@pytest.fixture()
def ids(oracle_mod):
    o = oracle_mod.Oracle()
    yield setup_materials(o)
    o.reset_materials()


@pytest.mark.parametrize("case", F32_CASES, ids=[case_key(c) for c in F32_CASES])
def test_f32_liquids_match_reference_tick(oracle_mod, ids, case):
    from oracle.binding import build_reference_tick

    lib = build_reference_tick()
    if lib is None:
        pytest.skip("reference tree absent")
    ref = run_reference(oracle_mod, lib, ids, case)
    got = run_oracle(oracle_mod, ids, case)
    for name, a, b in zip(NAMES, ref, got):
        assert a.shape == b.shape, (name, a.shape, b.shape)
        bad = np.argwhere(a != b)
        assert len(bad) == 0, "%s differs at %d places, first %s: reference %s, oracle %s" % (
            name, len(bad), bad[0].tolist(), a[tuple(bad[0])], b[tuple(bad[0])])


@pytest.mark.parametrize("case", F32_CASES, ids=[case_key(c) for c in F32_CASES])
def test_f32_liquids_match_reference_digests(oracle_mod, ids, case):
    golden = json.load(open(GOLDEN))
    got = run_oracle(oracle_mod, ids, case)
    assert digest(got) == golden[case_key(case)]["digest"]
    assert len(got[7]) == golden[case_key(case)]["particles"]


def test_f32_scenes_exercise_the_liquid_rules(oracle_mod, ids):
    """The scenes flow, evaporate, free-fall into particles and react."""
    seen = {"amount changed": 0, "liquid particles": 0, "steam or obsidian": 0, "liquid cells made": 0}
    for case in F32_CASES:
        w, h, seed, ci, nt = case
        st = scene_f32(ids, w, h, seed)
        res = run_oracle(oracle_mod, ids, case)
        soup0 = np.isin(st["id"], [ids["WATER"], ids["LAVA"]])
        soup1 = np.isin(res[0], [ids["WATER"], ids["LAVA"]])
        seen["amount changed"] += int((soup0 & soup1 & (res[4] != st["scalar"])).sum())
        seen["liquid cells made"] += int((soup1 & ~soup0).sum())
        seen["liquid particles"] += int(np.isin(res[7][:, 0], [ids["WATER"], ids["LAVA"]]).sum())
        seen["steam or obsidian"] += int(np.isin(res[0], [oracle_mod.Oracle().find("STEAM"),
                                                           oracle_mod.Oracle().find("OBSIDIAN")]).sum())
    assert all(v > 0 for v in seen.values()), seen
