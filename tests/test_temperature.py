"""Temperature conduction (world::tickTemperature, world.cpp:1950-2004) on the CPU.

The oracle's restatement is pinned against the reference's own function, compiled
from the reference tree (oracle/Makefile `ref`) when that tree is present, and
against fixtures that function produced (tests/golden/temperature.npz).
"""
import os

import numpy as np
import pytest

from temperature_cases import CASES, apply_edits, case_inputs, material_params

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "temperature.npz")


def _oracle_step(oracle_mod, mat, temp):
    h, w = mat.shape
    ow = oracle_mod.OracleWorld(w, h, 128, 3, 1)
    z32 = np.zeros((h, w), np.int32)
    ow.set_state({"id": mat, "colour": z32.view(np.uint32), "scalar": z32, "flags": np.zeros((h, w), np.uint8),
                  "diff": z32})
    ow.set_temperature(temp)
    assert np.array_equal(ow.temperature(), temp)
    ow.tick_temperature()
    return ow.temperature()


def test_oracle_matches_golden(oracle_mod):
    g = np.load(GOLDEN)
    o = oracle_mod.Oracle()
    try:
        for case in CASES:
            name = case[0]
            o.reset_materials()
            apply_edits(o.set_conduction, o.find, case[5])
            add, cs, co = material_params(o)
            assert np.array_equal(add, g[name + "_add"]) and np.array_equal(cs.view(np.uint32), g[name + "_cs"].view(np.uint32))
            assert np.array_equal(co.view(np.uint32), g[name + "_co"].view(np.uint32))
            got = _oracle_step(oracle_mod, g[name + "_mat"], g[name + "_temp"])
            assert np.array_equal(got, g[name + "_out"]), name
    finally:
        o.reset_materials()


def test_oracle_matches_reference_function(oracle_mod):
    from oracle.binding import build_reference_temperature, reference_tick_temperature

    lib = build_reference_temperature()
    if lib is None:
        pytest.skip("reference tree absent")
    o = oracle_mod.Oracle()
    try:
        for k, case in enumerate(CASES):
            # fresh seeds: cases beyond the frozen fixtures
            case = (case[0], case[1] + 7, case[2] + 5, case[3] + 100) + case[4:]
            o.reset_materials()
            mat, temp = case_inputs(o, case)
            add, cs, co = material_params(o)
            h, w = mat.shape
            pm = np.zeros((h + 2, w + 2), np.uint16)
            pt = np.zeros((h + 2, w + 2), np.int16)
            pm[1:-1, 1:-1] = mat
            pt[1:-1, 1:-1] = temp
            ref = reference_tick_temperature(lib, pm, pt, add, cs, co, (1, 1, w, h))[1:-1, 1:-1]
            got = _oracle_step(oracle_mod, mat, temp)
            assert np.array_equal(got, ref), case[0]
    finally:
        o.reset_materials()


def test_oracle_temperature_travels_with_liquid(oracle_mod):
    """A liquid's temperature moves with it: after ticks, every WATER cell (created by
    flow or deposit from water of one temperature) still carries that temperature."""
    o = oracle_mod.Oracle()
    o.reset_materials()
    ow = oracle_mod.OracleWorld(128, 128, 128, 3, 9)
    ow.generate(0, 9)
    st = ow.state()
    water = o.find("WATER")
    t = ow.temperature()
    assert np.all(t[st["id"] == water] == -1023)
    ow.step(12)
    st = ow.state()
    t = ow.temperature()
    assert np.count_nonzero(st["id"] == water) > 0
    assert np.all(t[st["id"] == water] == -1023)
    p = ow.particles()
    assert np.all(p["temperature"][p["id"] == water] == -1023)
