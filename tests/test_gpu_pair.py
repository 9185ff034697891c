"""The colour pass with each chunk split over a CTA pair (a thread-block cluster).

Launch shapes 2 and 3 run every chunk on two 512-thread CTAs of a cluster, each
updating half the chunk's rows and keeping the rows both reach equal by mirrored
writes into the partner's shared memory. Results must not depend on the shape: the
device must equal the oracle bit for bit on generated worlds (ragged sizes, both
halos, fire, liquids with temperatures, f32 amounts, other chunk edges and
iteration counts), in steps with particles, in graphs, in batches and with a tick
zone.
"""
import numpy as np
import pytest

from helpers import compare_particles, compare_states, material_types
from oracle.binding import ORDER_PART

pytestmark = pytest.mark.gpu


def _pair(fse, oracle_mod, w, h, seed, chunk=128, cell_iter=3, kind=1, **kw):
    world = fse.World(w, h, chunk_size=chunk, cell_iter=cell_iter, seed=seed, **kw)
    world.generate(kind, seed)
    ow = oracle_mod.OracleWorld(w, h, chunk, cell_iter, seed)
    if kw.get("f32_fluid"):
        ow.set_f32(True)
    ow.generate({1: 0, 2: 1}[kind], seed)
    return world, ow


@pytest.mark.parametrize("shape", [2, 3])
@pytest.mark.parametrize("w,h,kind", [(512, 512, 1), (300, 232, 1), (384, 384, 2), (130, 700, 1)])
def test_pair_steps_match_oracle(fse, oracle_mod, shape, w, h, kind):
    types = material_types(fse)
    world, ow = _pair(fse, oracle_mod, w, h, 300 + w + h, kind=kind)
    world.set_launch(shape)
    for t in range(5):
        world.step(1)
        ow.step(1, ORDER_PART)
        what = "shape %d %dx%d step %d" % (shape, w, h, t)
        compare_states(world.state(), ow.state(), types, what)
        compare_particles(world.particles(), ow.particles(), what)
    np.testing.assert_array_equal(world.ledger(), ow.ledger())
    world.close()


@pytest.mark.parametrize("chunk,cell_iter", [(64, 2), (96, 4), (32, 1)])
def test_pair_chunk_variants(fse, oracle_mod, chunk, cell_iter):
    types = material_types(fse)
    world, ow = _pair(fse, oracle_mod, 288, 200, 77 + chunk, chunk=chunk, cell_iter=cell_iter)
    world.set_launch(2)
    for t in range(4):
        world.step(1)
        ow.step(1, ORDER_PART)
        compare_states(world.state(), ow.state(), types, "chunk %d step %d" % (chunk, t))
        compare_particles(world.particles(), ow.particles(), "chunk %d step %d" % (chunk, t))
    world.close()


def test_pair_fire_temperature_f32(fse, oracle_mod):
    """Fire (the 5 x 7 lattice), liquid temperatures with the conduction step, f32
    amounts, graphs."""
    types = material_types(fse)
    w, h, seed = 384, 320, 91
    world, ow = _pair(fse, oracle_mod, w, h, seed, temperature=True, temperature_step=True, f32_fluid=True)
    st = world.state()
    rng = np.random.default_rng(seed)
    f = rng.random((h, w)) < 0.03
    st["id"][f] = fse.material_find("FIRE")
    st["colour"][f] = 0xFF6432
    st["scalar"][f] = 0
    world.upload(st)
    ow.set_state(world.state())
    ow.enable_temperature(True)
    ow.set_temperature(world.temperature())
    world.set_launch(3)
    world.step(4, graph=True)
    ow.step(4, ORDER_PART)
    compare_states(world.state(), ow.state(), types, "fire f32 pair")
    compare_particles(world.particles(), ow.particles(), "fire f32 pair", temperature=True)
    assert np.array_equal(world.temperature(), ow.temperature())
    world.close()


def test_pair_interactions_wide_halo(fse, oracle_mod):
    """Materials with interactions switch every chunk to the 11 x 11 lattice and the
    5-cell halo; the boxes reach 5 cells to the side and below, across the middle of
    a chunk."""
    o = oracle_mod.Oracle()
    sand, dirt, water, stone, cobble = (fse.material_find(n) for n in ("GENERIC_SAND", "DIRT", "WATER", "STONE",
                                                                       "COBBLE_STONE"))
    rules = [(sand, water, 1, dirt, 2, 3, 2), (sand, stone, 2, water, 1, 1, 4), (sand, cobble, 2, water, 1, -2, 0)]
    try:
        for r in rules:
            fse.set_interaction(*r)
            assert o.set_interaction(*r) == 0
        fse.PushMaterials()
        types = material_types(fse)
        world, ow = _pair(fse, oracle_mod, 320, 256, 13)
        world.set_launch(2)
        for t in range(4):
            world.step(1)
            ow.step(1, ORDER_PART)
            compare_states(world.state(), ow.state(), types, "interactions step %d" % t)
            compare_particles(world.particles(), ow.particles(), "interactions step %d" % t)
        world.close()
    finally:
        fse.InitMaterials()
        fse.PushMaterials()
        o.reset_materials()


def test_pair_batch_and_zone(fse, oracle_mod):
    types = material_types(fse)
    sizes = [(256, 192), (384, 256), (128, 320)]
    worlds, oracles = [], []
    for i, (w, h) in enumerate(sizes):
        world, ow = _pair(fse, oracle_mod, w, h, 500 + i)
        if i == 1:
            world.set_tick_zone(64, 0, 256, 256)
            ow.set_tick_zone(64, 0, 256, 256)
        worlds.append(world)
        oracles.append(ow)
    b = fse.Batch(worlds)
    b.set_launch(3, 0)
    b.step(6, graph_ticks=4)
    for world, ow in zip(worlds, oracles):
        ow.step(6, ORDER_PART)
        compare_states(world.state(), ow.state(), types, "batch pair")
        compare_particles(world.particles(), ow.particles(), "batch pair")
    b.close()
    for world in worlds:
        world.close()
