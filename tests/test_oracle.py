"""CPU checks of the oracle itself: race-freedom of the partitioned order, the
conservation ledger in both orders, FP32-vs-FP64 particle kinematics, and the
committed golden fixtures."""
import hashlib
import os

import numpy as np
import pytest

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
SEQ, PART = 0, 1


def _world(oracle_mod, w=256, h=256, seed=1234, kind=0):
    ow = oracle_mod.OracleWorld(w, h, 128, 3, seed)
    ow.generate(kind, seed)
    return ow


def _special_world(oracle_mod, seed=7):
    """A world with fire, lava, water, steam, gold ore and a custom liquid."""
    o = oracle_mod.Oracle()
    ow = _world(oracle_mod, 256, 192, seed)
    s = ow.state()
    rng = np.random.default_rng(seed)
    ids = s["id"]
    for name, frac in (("FIRE", 0.01), ("LAVA", 0.03), ("STEAM", 0.02), ("GOLD_ORE", 0.02), ("DIRT", 0.02)):
        m = o.find(name)
        pick = rng.random(ids.shape) < frac
        ids[pick] = m
        s["scalar"][pick] = 65536 * 2 if name == "LAVA" else (1000 if name == "GOLD_ORE" else 0)
        s["colour"][pick] = 0x123456
        s["flags"][pick] = 0
        s["diff"][pick] = 0
    ow.set_state(s)
    return ow


@pytest.mark.parametrize("kind", [0, 1])
def test_partitioned_order_is_race_free(oracle_mod, kind):
    ow = _world(oracle_mod, 320, 256, 11, kind)
    for _ in range(3):
        assert ow.tick(PART, check_races=True) == 0
        ow.particles_tick()


def test_race_free_with_fire_and_reactions(oracle_mod):
    ow = _special_world(oracle_mod)
    for _ in range(4):
        assert ow.tick(PART, check_races=True) == 0
        ow.particles_tick()


def test_race_free_with_interactions(oracle_mod):
    o = oracle_mod.Oracle()
    o.reset_materials()
    try:
        sand, dirt, water = o.find("GENERIC_SAND"), o.find("DIRT"), o.find("WATER")
        assert o.set_interaction(sand, water, 1, dirt, 2, 3, 2) == 0
        assert o.set_interaction(sand, o.find("STONE"), 2, water, 1, 1, 4) == 0
        ow = _world(oracle_mod, 256, 256, 5)
        for _ in range(3):
            assert ow.tick(PART, check_races=True) == 0
            ow.particles_tick()
    finally:
        o.reset_materials()


def test_race_checker_catches_a_planted_small_lattice(oracle_mod):
    """The checker must see conflicts when sweep A runs on a lattice that is too
    dense (the mistake is planted in the oracle, on the CPU)."""
    o = oracle_mod.Oracle()
    try:
        o.debug_set_lattice(0, 1, 1)
        ow = _world(oracle_mod, 256, 256, 3)
        assert ow.tick(PART, check_races=True) > 0
        o.debug_set_lattice(0, 2, 6)
        ow = _world(oracle_mod, 256, 256, 3)
        assert ow.tick(PART, check_races=True) > 0
        o.debug_set_lattice(1, 3, 2)  # sweep B needs 3 rows between cells of a column
        o.debug_set_lattice(0, 0, 0)
        ow = _world(oracle_mod, 256, 256, 3)
        assert ow.tick(PART, check_races=True) > 0
    finally:
        for s in range(3):
            o.debug_set_lattice(s, 0, 0)


def _ledger_residual(o, c0, c1, led):
    m = o.material_count()
    types = np.array([o.material(i)[0] for i in range(m)])
    nz = types != 0
    count = (c1[0] + c1[2]) - (c0[0] + c0[2]) - (led[0] - led[1] - led[2])
    fluid = (c1[1] + c1[3]) - (c0[1] + c0[3]) - (led[3] - led[4] - led[5])
    return count[nz], fluid[nz]


@pytest.mark.parametrize("order", [SEQ, PART])
@pytest.mark.parametrize("special", [False, True])
def test_conservation_ledger(oracle_mod, order, special):
    """grid + particles - created + destroyed + exited is invariant per material,
    exactly, every tick, in the reference order and in the partitioned order."""
    o = oracle_mod.Oracle()
    ow = _special_world(oracle_mod) if special else _world(oracle_mod, 256, 256, 3)
    for t in range(6):
        c0 = ow.census()
        ow.reset_ledger()
        ow.tick(order)
        ow.particles_tick()
        cnt, fl = _ledger_residual(o, c0, ow.census(), ow.ledger())
        assert not cnt.any(), "tick %d count residual %s" % (t, cnt)
        assert not fl.any(), "tick %d fluid residual %s" % (t, fl)


def test_orders_differ_but_conserve_the_same_totals(oracle_mod):
    a, b = _world(oracle_mod, 256, 256, 9), _world(oracle_mod, 256, 256, 9)
    c0 = a.census()
    a.step(5, SEQ)
    b.step(5, PART)
    sa, sb = a.state(), b.state()
    assert not np.array_equal(sa["id"], sb["id"])  # the update order matters ...
    o = oracle_mod.Oracle()
    for ow in (a, b):  # ... but the ledger closes for both
        cnt, fl = _ledger_residual(o, c0, ow.census(), ow.ledger())
        assert not cnt.any() and not fl.any()


def test_particle_kinematics_fp32_vs_fp64(oracle_mod):
    """The FP32 particle restatement agrees with an FP64 evaluation to 1e-5 relative
    error on (x, y, vx, vy) for particles whose discrete events match."""
    ow = _world(oracle_mod, 512, 512, 21)
    rng = np.random.default_rng(0)
    n = 20000
    p = np.zeros(n, oracle_mod.PARTICLE_DTYPE)
    p["x"] = rng.uniform(0, 512, n).astype(np.float32)
    p["y"] = rng.uniform(0, 512, n).astype(np.float32)
    p["vx"] = rng.normal(0, 2, n).astype(np.float32)
    p["vy"] = rng.normal(0, 2, n).astype(np.float32)
    p["ay"] = np.float32(0.1)
    p["id"] = 2
    o64, e64, s64 = ow.kinematics(p, f64=True)
    o32, e32, s32 = ow.kinematics(p, f64=False)
    match = (e64 == e32) & (s64 == s32)
    assert match.mean() > 0.99
    rel = np.abs(o32[match].astype(np.float64) - o64[match]) / np.maximum(np.abs(o64[match]), 1.0)
    assert rel.max() <= 1e-5, rel.max()


def _digest(state, parts):
    h = hashlib.sha256()
    for k in ("id", "colour", "scalar", "flags"):
        h.update(np.ascontiguousarray(state[k]).tobytes())
    soup = np.isin(state["id"], [3, 15, 16, 19, 30])
    h.update(np.ascontiguousarray(np.where(soup, state["diff"], 0)).tobytes())
    # the first 56 bytes of each record: the fields the fixtures were made with
    h.update(np.ascontiguousarray(parts).view(np.uint8).reshape(len(parts), parts.dtype.itemsize)[:, :56].tobytes())
    return h.hexdigest()


def test_golden_fixtures(oracle_mod):
    """The oracle reproduces the committed fixtures (tests/golden/make_golden.py)."""
    path = os.path.join(GOLDEN, "golden.npz")
    g = np.load(path)
    for name in g["names"]:
        name = str(name)
        w, h, seed, kind, steps, order = [int(v) for v in g[name + "_params"]]
        ow = _world(oracle_mod, w, h, seed, kind)
        ow.step(steps, order)
        s = ow.state()
        assert _digest(s, ow.particles()) == str(g[name + "_digest"]), name
        np.testing.assert_array_equal(s["id"], g[name + "_id"])
