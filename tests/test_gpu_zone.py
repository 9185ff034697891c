"""The tick zone (world::tickZone) on the device.

* In the reference's order with f32 liquid amounts, a world ticked with the game's
  zone and with one that is not chunk-aligned reproduces the digests of the
  reference's own world::tick run with the same zone
  (tests/golden/tick_zone_ref.json).
* In the partitioned order, steps (tick, particles, temperature) with a zone equal
  the oracle's bit for bit; particles outside the zone stay where they are.
* Step graphs captured before the zone changed are not replayed after it.
"""
import json

import numpy as np
import pytest

from helpers import compare_particles, compare_states, material_types
from oracle.binding import ORDER_PART
from test_gpu_reference_order import scene_ids  # noqa: F401 - fixture
from test_tick_ref_f32 import START_TICK, digest, result_of_planes
from test_tick_zone_ref import GOLDEN, ZONE_CASES, zone_key
from tick_cases import scene_f32

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("case", ZONE_CASES, ids=[zone_key(c) for c in ZONE_CASES])
def test_device_zone_matches_reference_digests(fse, scene_ids, case):  # noqa: F811
    w, h, seed, ci, nt, zone = case
    st = scene_f32(scene_ids, w, h, seed)
    world = fse.World(w, h, cell_iter=ci, seed=seed, reference_order=True, temperature=True, f32_fluid=True)
    world.upload({k: st[k] for k in ("id", "colour", "scalar", "flags", "diff")})
    world.set_temperature(st["temperature"])
    world.set_tick_zone(*zone)
    world.tick_count = START_TICK
    world.tick(nt)
    res = result_of_planes(scene_ids, world.state(), world.temperature(), world.particles())
    golden = json.load(open(GOLDEN))
    assert digest(res) == golden[zone_key(case)]["digest"]
    world.close()


@pytest.mark.parametrize("zone", [(128, 128, 256, 128), (37, 21, 300, 200), (0, 0, 0, 0)])
def test_device_zone_steps_match_oracle(fse, oracle_mod, zone):
    import bench

    types = material_types(fse)
    w, h, seed = 512, 384, 51
    world = fse.World(w, h, seed=seed, temperature=True, temperature_step=True)
    world.generate(fse.GEN_MIX, seed)
    parts = bench.config1_particles(20000, w, h, seed)
    world.addCell(parts)
    world.set_tick_zone(*zone)
    ow = oracle_mod.OracleWorld(w, h, 128, 3, seed)
    ow.generate(0, seed)
    ow.enable_temperature(True)
    ow.set_particles(parts)
    ow.set_tick_zone(*zone)
    for t in range(6):
        world.step(1)
        ow.step(1, ORDER_PART)
        what = "zone %s step %d" % (zone, t)
        compare_states(world.state(), ow.state(), types, what)
        compare_particles(world.particles(), ow.particles(), what, temperature=True)
        assert np.array_equal(world.temperature(), ow.temperature()), what
    world.close()


def test_zone_change_invalidates_step_graphs(fse, oracle_mod):
    """A zone set after ticks: the step graphs are captured again and the spawn
    counts of chunk slots the smaller zone no longer has are cleared."""
    types = material_types(fse)
    w, h, seed = 384, 256, 52
    world = fse.World(w, h, seed=seed)
    world.generate(fse.GEN_MIX, seed)
    ow = oracle_mod.OracleWorld(w, h, 128, 3, seed)
    ow.generate(0, seed)
    world.step(4, graph=True)
    ow.step(4, ORDER_PART)
    compare_states(world.state(), ow.state(), types, "before the zone change")
    compare_particles(world.particles(), ow.particles(), "before the zone change")
    world.set_tick_zone(128, 0, 256, 256)
    ow.set_tick_zone(128, 0, 256, 256)
    world.step(4, graph=True)
    ow.step(4, ORDER_PART)
    compare_states(world.state(), ow.state(), types, "after the zone change")
    compare_particles(world.particles(), ow.particles(), "after the zone change")
    with pytest.raises(fse.FseError):
        world.set_tick_zone(200, 0, 256, 256)  # reaches past the world
    world.close()
