"""The device tick with f32 liquid amounts (FSE_CFG_F32_FLUID).

* In the reference's own update order the device reproduces the digests of the
  reference's world::tick on the f32 liquid scenes (tests/golden/tick_ref_f32.json,
  made by compiling world.cpp's function unchanged): every cell's material, colour,
  temperature and moved flag, every liquid cell's amount, diff and settle count,
  and every spawned particle with its amount, bit for bit.
* In the partitioned order the device equals the oracle's f32 tick bit for bit on
  generated worlds, with particle steps (liquid deposits merged in particle order)
  and with liquid temperatures.
* Batches of f32 worlds equal the worlds ticked alone; f32 and Q16.16 worlds do not
  share a batch; the tile-struct calls move f32 amounts bit for bit.
"""
import json

import numpy as np
import pytest

from helpers import compare_particles, compare_states, material_types
from oracle.binding import ORDER_PART
from test_gpu_reference_order import scene_ids  # noqa: F401 - fixture
from test_tick_ref_f32 import GOLDEN, START_TICK, case_key, digest, result_of_planes
from tick_cases import F32_CASES, scene_f32

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("case", F32_CASES, ids=[case_key(c) for c in F32_CASES])
def test_device_f32_matches_reference_digests(fse, scene_ids, case):  # noqa: F811
    w, h, seed, ci, nt = case
    st = scene_f32(scene_ids, w, h, seed)
    world = fse.World(w, h, cell_iter=ci, seed=seed, reference_order=True, temperature=True, f32_fluid=True)
    world.upload({k: st[k] for k in ("id", "colour", "scalar", "flags", "diff")})
    world.set_temperature(st["temperature"])
    world.tick_count = START_TICK
    world.tick(nt)
    res = result_of_planes(scene_ids, world.state(), world.temperature(), world.particles())
    golden = json.load(open(GOLDEN))
    key = case_key(case)
    assert len(res[7]) == golden[key]["particles"], key
    assert digest(res) == golden[key]["digest"], key
    world.close()


@pytest.mark.parametrize("w,h,seed,ci,temperature", [(384, 256, 31, 3, False), (300, 232, 32, 2, True),
                                                      (512, 512, 33, 3, False)])
def test_device_f32_partitioned_matches_oracle(fse, oracle_mod, w, h, seed, ci, temperature):
    types = material_types(fse)
    world = fse.World(w, h, cell_iter=ci, seed=seed, temperature=temperature, f32_fluid=True)
    world.generate(fse.GEN_MIX, seed)
    ow = oracle_mod.OracleWorld(w, h, 128, ci, seed)
    ow.set_f32(True)
    ow.generate(0, seed)
    compare_states(world.state(), ow.state(), types, "f32 generate")
    for t in range(6):
        world.step(1)
        ow.step(1, ORDER_PART)
        what = "f32 step %d" % t
        compare_states(world.state(), ow.state(), types, what)
        compare_particles(world.particles(), ow.particles(), what, temperature=temperature)
        np.testing.assert_array_equal(world.ledger(), ow.ledger(), err_msg=what + " ledger")
    # the mix spawns free-falling water, whose particles merge back into water
    assert (world.particles()["id"] == fse.material_find("WATER")).any()
    world.close()


def test_f32_batch_equals_individual_worlds(fse):
    sizes = [(256, 192), (128, 320), (384, 256)]
    alone, grouped = [], []
    for i, (w, h) in enumerate(sizes):
        for lst in (alone, grouped):
            wd = fse.World(w, h, seed=40 + i, f32_fluid=True)
            wd.generate(fse.GEN_MIX, 40 + i)
            lst.append(wd)
    for wd in alone:
        wd.step(5)
    batch = fse.Batch(grouped)
    batch.step(5, graph_ticks=4)
    for a, b in zip(alone, grouped):
        sa, sb = a.state(), b.state()
        for k in sa:
            np.testing.assert_array_equal(sa[k], sb[k])
        assert a.particles().tobytes() == b.particles().tobytes()
    batch.close()
    q = fse.World(128, 128, seed=1)
    with pytest.raises(fse.FseError):
        fse.Batch([alone[0], q])
    for wd in alone + grouped + [q]:
        wd.close()


def test_f32_tiles_move_amounts_bit_for_bit(fse):
    world = fse.World(192, 160, seed=5, f32_fluid=True)
    world.generate(fse.GEN_MIX, 5)
    world.step(3)
    tiles = world.download_tiles()
    st = world.state()
    soup = material_types(fse)[st["id"]] == 3
    assert soup.any()
    np.testing.assert_array_equal(tiles["fluidAmount"][soup].view(np.int32), st["scalar"][soup])
    np.testing.assert_array_equal(tiles["fluidAmountDiff"][soup].view(np.int32), st["diff"][soup])
    other = fse.World(192, 160, seed=5, f32_fluid=True)
    other.upload_tiles(tiles)
    st2 = other.state()
    np.testing.assert_array_equal(st2["scalar"][soup], st["scalar"][soup])
    np.testing.assert_array_equal(st2["diff"][soup], st["diff"][soup])
    world.close()
    other.close()
