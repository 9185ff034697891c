"""The CUDA tick in the reference's own update order (FSE_CFG_REFERENCE_ORDER).

On the scenes of tests/tick_cases.py the device world, ticked in reference order,
must reproduce the digests of the reference's own world::tick
(tests/golden/tick_ref.json, made by compiling world.cpp's function unchanged):
every cell's material, colour, temperature and moved flag and every spawned
particle. On generated worlds with liquids, temperatures and particle steps (where
the reference's f32 amounts rule out a bit comparison with it) the device must
equal the oracle's reference-order tick.
"""
import json
import os

import numpy as np
import pytest

from helpers import compare_particles, compare_states, material_types
from oracle.binding import ORDER_SEQ
from test_tick_ref import GOLDEN, START_TICK, digest, oracle_rows
from tick_cases import CASES, scene, setup_materials

pytestmark = pytest.mark.gpu


class _Product:
    """The product's material calls under the oracle binding's names."""

    def __init__(self, fse):
        self.fse = fse

    def reset_materials(self):
        self.fse.InitMaterials()

    def register(self, *a):
        return self.fse.RegisterMaterial(*a)

    def set_factory(self, mat, base, shift, lo, mod, scalar):
        return self.fse.lib().fse_material_set_factory(mat, base & 0xFFFFFFFF, shift, lo, mod, scalar)

    def set_reaction(self, *a):
        self.fse.set_reaction(*a)
        return 0

    def set_interaction(self, *a):
        self.fse.set_interaction(*a)
        return 0

    def find(self, name):
        return self.fse.material_find(name)


@pytest.fixture()
def scene_ids(fse, oracle_mod):
    ids = setup_materials(_Product(fse))
    fse.PushMaterials()
    oids = setup_materials(oracle_mod.Oracle())
    assert ids == oids
    yield ids
    fse.InitMaterials()
    fse.PushMaterials()
    oracle_mod.Oracle().reset_materials()


@pytest.mark.parametrize("case", CASES, ids=["%s-%dx%d-i%d-t%d" % (c[3], c[0], c[1], c[4], c[5]) for c in CASES])
def test_device_matches_reference_digests(fse, scene_ids, case):
    w, h, seed, kind, ci, nt = case
    st = scene(scene_ids, w, h, seed, kind)
    world = fse.World(w, h, cell_iter=ci, seed=seed, reference_order=True)
    world.upload(st)
    world.tick_count = START_TICK
    world.tick(nt)
    g = world.state()
    rows = oracle_rows(world.particles())
    golden = json.load(open(GOLDEN))
    key = "%d_%d_%d_%s_%d_%d" % case
    assert len(rows) == golden[key]["particles"], key
    assert digest(g["id"], g["colour"], g["scalar"], (g["flags"] >> 7).astype(np.uint8), rows) == golden[key]["digest"]
    world.close()


@pytest.mark.parametrize("w,h,seed,ci,fire", [(384, 256, 21, 3, False), (300, 200, 22, 2, False),
                                               (512, 384, 23, 3, False), (384, 320, 24, 3, True)])
def test_device_reference_order_matches_oracle(fse, oracle_mod, w, h, seed, ci, fire):
    """Generated worlds (liquids, gas, sand, solids; with fire in one) with liquid
    temperatures and the conduction step every fourth tick, stepped in reference
    order on both sides."""
    types = material_types(fse)
    world = fse.World(w, h, cell_iter=ci, seed=seed, temperature=True, temperature_step=True, reference_order=True)
    world.generate(fse.GEN_MIX, seed)
    if fire:
        st = world.state()
        rng = np.random.default_rng(seed)
        f = rng.random((h, w)) < 0.03
        st["id"][f] = fse.material_find("FIRE")
        st["colour"][f] = 0xFF6432
        st["scalar"][f] = 0
        world.upload(st)
    ow = oracle_mod.OracleWorld(w, h, 128, ci, seed)
    ow.set_state(world.state())
    ow.enable_temperature(True)
    ow.set_temperature(world.temperature())
    for t in range(4):
        world.step(1)
        ow.step(1, order=ORDER_SEQ)
        compare_states(world.state(), ow.state(), types, "reference order step %d" % t)
        compare_particles(world.particles(), ow.particles(), "reference order step %d" % t, temperature=True)
        assert np.array_equal(world.temperature(), ow.temperature())
        assert np.array_equal(world.ledger(), ow.ledger())
    world.close()


def test_reference_order_worlds_stay_out_of_batches(fse):
    a = fse.World(128, 128, seed=1, reference_order=True)
    b = fse.World(128, 128, seed=1)
    with pytest.raises(fse.FseError):
        fse.Batch([a, b])
    a.close()
    b.close()
