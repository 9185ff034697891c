"""Temperature conduction (world::tickTemperature, world.cpp:1950-2004) on the GPU.

The CUDA stencil is compared bit for bit with the oracle (itself pinned to the
reference's own function, tests/test_temperature.py) on the seeded cases and on
worlds that span many 128 x 32 tiles; liquid temperatures are followed through
full steps (moves, flows into air, free fall into particles, deposits, reactions)
with the temperature step every fourth tick.
"""
import os

import numpy as np
import pytest

from helpers import compare_particles, compare_states, material_types
from temperature_cases import CASES, apply_edits, case_inputs

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "temperature.npz")


def _planes(mat, scalar=None):
    h, w = mat.shape
    z = np.zeros((h, w), np.int32)
    return {"id": mat.astype(np.uint16), "colour": z.view(np.uint32).copy(),
            "scalar": z.copy() if scalar is None else scalar.astype(np.int32),
            "flags": np.zeros((h, w), np.uint8), "diff": z.copy()}


def _gpu_step(fse, mat, temp, scalar=None):
    h, w = mat.shape
    world = fse.World(w, h, seed=1, temperature=True)
    world.upload(_planes(mat, scalar))
    world.set_temperature(temp)
    assert np.array_equal(world.temperature(), temp)
    world.tickTemperature()
    out = world.temperature(), world.state()
    world.close()
    return out


def _oracle_step(oracle_mod, mat, temp, scalar=None):
    h, w = mat.shape
    ow = oracle_mod.OracleWorld(w, h, 128, 3, 1)
    ow.set_state(_planes(mat, scalar))
    ow.set_temperature(temp)
    ow.tick_temperature()
    return ow.temperature(), ow.state()


def _with_edits(fse, oracle_mod, edits, fn):
    o = oracle_mod.Oracle()
    o.reset_materials()
    fse.InitMaterials()
    apply_edits(fse.set_conduction, fse.material_find, edits)
    apply_edits(o.set_conduction, o.find, edits)
    fse.PushMaterials()
    try:
        return fn(o)
    finally:
        o.reset_materials()
        fse.InitMaterials()
        fse.PushMaterials()


def test_material_conduction_table(fse, oracle_mod):
    o = oracle_mod.Oracle()
    o.reset_materials()
    from temperature_cases import material_params

    add, cs, co = material_params(o)
    for k in range(fse.material_count()):
        a, s, c, _ = fse.get_conduction(k)
        assert a == add[k] and np.float32(s) == cs[k] and np.float32(c) == co[k], k
    assert fse.get_conduction(fse.material_find("WATER"))[3] == -1023
    assert fse.get_conduction(fse.material_find("LAVA"))[3] == 1024


def test_stencil_golden_cases(fse, oracle_mod):
    g = np.load(GOLDEN)
    for case in CASES:
        name = case[0]

        def run(o):
            mat, temp = g[name + "_mat"], g[name + "_temp"]
            got, _ = _gpu_step(fse, mat, temp)
            assert np.array_equal(got, g[name + "_out"]), (name, int((got != g[name + "_out"]).sum()))

        _with_edits(fse, oracle_mod, case[5], run)


@pytest.mark.parametrize("w,h,regime,edits", [
    (300, 70, "mixed", "builtin"),      # partial tiles on both axes
    (1000, 300, "wide", "edge"),        # 8 x 10 tiles: ring commits between neighbours
    (129, 33, "sparse", "builtin"),     # one cell past a tile on each axis
    (2048, 512, "mixed", "builtin"),    # 256 tiles, several per CTA
])
def test_stencil_matches_oracle(fse, oracle_mod, w, h, regime, edits):
    def run(o):
        case = ("t", w, h, w * 7 + h, regime, edits)
        mat, temp = case_inputs(o, case)
        # scalars outside int16 on some non-SOUP cells: their temperature is the low
        # 16 bits and the step stores the int16 result
        rng = np.random.default_rng(w + h)
        sc = np.where(rng.random((h, w)) < 0.05, rng.integers(-(1 << 30), 1 << 30, size=(h, w)), 0)
        types = material_types(fse)
        sc = np.where(types[mat] == 3, 0, sc).astype(np.int32)
        temp = np.where(sc != 0, sc.astype(np.int16), temp).astype(np.int16)
        gt, gs = _gpu_step(fse, mat, temp, sc)
        ot, os_ = _oracle_step(oracle_mod, mat, temp, sc)
        assert np.array_equal(gt, ot), int((gt != ot).sum())
        compare_states(gs, os_, types, "temperature step")

    _with_edits(fse, oracle_mod, edits, run)


def _hot_world(fse, oracle_mod, w, h, seed, temperature=True):
    """A mix world with LAVA pools and hot GOLD_ORE (its reaction makes a SOUP tile
    that keeps the ore's temperature), device and oracle side by side; the
    conduction step runs every fourth tick when `temperature`."""
    world = fse.World(w, h, seed=seed, temperature=True, temperature_step=temperature)
    world.generate(fse.GEN_MIX, seed)
    ow = oracle_mod.OracleWorld(w, h, 128, 3, seed)
    ow.generate(0, seed)
    if temperature:
        ow.enable_temperature(True)
    st = world.state()
    rng = np.random.default_rng(seed)
    lava, gold = fse.material_find("LAVA"), fse.material_find("GOLD_ORE")
    pick = rng.random((h, w))
    ids = st["id"].copy()
    ids[(pick < 0.03) & (np.arange(h)[:, None] < h // 2)] = lava
    ids[(pick > 0.985)] = gold
    sc = st["scalar"].copy()
    sc[ids == lava] = 2 * fse.FLUID_ONE
    sc[ids == gold] = 0
    st["id"], st["scalar"] = ids, sc
    st["diff"][:] = 0
    world.upload(st)
    ow.set_state(st)
    t = world.temperature()
    t[ids == lava] = 1024
    t[ids == gold] = rng.integers(400, 700, size=int((ids == gold).sum()))
    world.set_temperature(t)
    ow.set_temperature(t)
    return world, ow


@pytest.mark.parametrize("graph", [False, True])
def test_steps_with_temperature(fse, oracle_mod, graph):
    types = material_types(fse)
    world, ow = _hot_world(fse, oracle_mod, 384, 256, 21)
    steps = 12
    if graph:
        world.step(steps, graph=True)
        ow.step(steps)
    else:
        for s in range(steps):
            world.step(1)
            ow.step(1)
            if s % 4 == 2:
                assert np.array_equal(world.temperature(), ow.temperature()), "step %d" % s
    compare_states(world.state(), ow.state(), types, "steps")
    assert np.array_equal(world.temperature(), ow.temperature())
    compare_particles(world.particles(), ow.particles(), "steps", temperature=True)
    assert (world.temperature() != 0).sum() > 1000  # the step did spread heat


def test_liquid_temperature_travels_without_conduction(fse, oracle_mod):
    """With the temperature step off, SOUP temperatures still move with every
    liquid move, flow, free fall and deposit, as MaterialInstance copies do."""
    types = material_types(fse)
    world, ow = _hot_world(fse, oracle_mod, 320, 192, 5, temperature=False)
    for s in range(10):
        world.step(1)
        ow.step(1)
    compare_states(world.state(), ow.state(), types, "steps")
    assert np.array_equal(world.temperature(), ow.temperature())
    compare_particles(world.particles(), ow.particles(), "steps", temperature=True)


def test_world_without_temperature(fse, oracle_mod):
    """A default world keeps no liquid temperatures: the temperature calls are
    refused and its particles read temperature 0; everything else matches."""
    types = material_types(fse)
    world = fse.World(256, 192, seed=3)
    world.generate(fse.GEN_MIX, 3)
    ow = oracle_mod.OracleWorld(256, 192, 128, 3, 3)
    ow.generate(0, 3)
    for call in (lambda: world.temperature(), lambda: world.tickTemperature(),
                 lambda: world.set_temperature(np.zeros((192, 256), np.int16))):
        with pytest.raises(fse.FseError):
            call()
    world.step(6)
    ow.step(6)
    compare_states(world.state(), ow.state(), types, "steps")
    gp = world.particles()
    assert not gp["temperature"].any()
    compare_particles(gp, ow.particles(), "steps")


def test_batch_with_temperature(fse, oracle_mod):
    """A batch of worlds with and without the temperature step, graph-replayed."""
    types = material_types(fse)
    pairs = [_hot_world(fse, oracle_mod, w, h, 30 + i, temperature=(i % 2 == 0))
             for i, (w, h) in enumerate([(256, 192), (384, 128), (192, 320)])]
    b = fse.Batch([p[0] for p in pairs])
    b.step(8, graph_ticks=4)
    b.sync()
    for k, (world, ow) in enumerate(pairs):
        ow.step(8)
        compare_states(world.state(), ow.state(), types, "batch world %d" % k)
        assert np.array_equal(world.temperature(), ow.temperature()), k
    b.close()
