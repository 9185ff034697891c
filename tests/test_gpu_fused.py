"""The fused tick: every colour pass of a tick in one launch (launch shape 4).

CTAs take chunk-passes in pass order from a ticket counter and start each one when
the last earlier pass of every chunk of its 3 x 3 neighbourhood is done, so passes
overlap across the world instead of meeting at a launch boundary. Results must not
depend on the shape: the device must equal the oracle bit for bit on generated
worlds (ragged sizes, both halos, fire, liquids with temperatures, f32 amounts,
other chunk edges and iteration counts), in steps with particles, in multi-tick
graphs (the completion flags are cleared by each launch for the next), in batches
of worlds with different iteration counts and with tick zones that change.
"""
import numpy as np
import pytest

from helpers import compare_particles, compare_states, material_types
from oracle.binding import ORDER_PART

pytestmark = pytest.mark.gpu

FUSED = 4


def _pair(fse, oracle_mod, w, h, seed, chunk=128, cell_iter=3, kind=1, **kw):
    world = fse.World(w, h, chunk_size=chunk, cell_iter=cell_iter, seed=seed, **kw)
    world.generate(kind, seed)
    ow = oracle_mod.OracleWorld(w, h, chunk, cell_iter, seed)
    if kw.get("f32_fluid"):
        ow.set_f32(True)
    ow.generate({1: 0, 2: 1}[kind], seed)
    return world, ow


@pytest.mark.parametrize("w,h,kind", [(512, 512, 1), (300, 232, 1), (384, 384, 2), (130, 700, 1), (1000, 136, 1)])
def test_fused_steps_match_oracle(fse, oracle_mod, w, h, kind):
    types = material_types(fse)
    world, ow = _pair(fse, oracle_mod, w, h, 700 + w + h, kind=kind)
    world.set_launch(FUSED)
    for t in range(5):
        world.step(1)
        ow.step(1, ORDER_PART)
        what = "fused %dx%d step %d" % (w, h, t)
        compare_states(world.state(), ow.state(), types, what)
        compare_particles(world.particles(), ow.particles(), what)
    np.testing.assert_array_equal(world.ledger(), ow.ledger())
    world.close()


@pytest.mark.parametrize("chunk,cell_iter", [(64, 2), (96, 4), (32, 1), (48, 6)])
def test_fused_chunk_variants(fse, oracle_mod, chunk, cell_iter):
    types = material_types(fse)
    world, ow = _pair(fse, oracle_mod, 288, 200, 177 + chunk, chunk=chunk, cell_iter=cell_iter)
    world.set_launch(FUSED)
    for t in range(4):
        world.step(1)
        ow.step(1, ORDER_PART)
        compare_states(world.state(), ow.state(), types, "chunk %d step %d" % (chunk, t))
        compare_particles(world.particles(), ow.particles(), "chunk %d step %d" % (chunk, t))
    world.close()


def test_fused_fire_temperature_f32_graphs(fse, oracle_mod):
    """Fire (the 5 x 7 lattice), liquid temperatures with the conduction step, f32
    amounts, 16 ticks replayed from a CUDA graph."""
    types = material_types(fse)
    w, h, seed = 384, 320, 191
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
    world.set_launch(FUSED)
    world.step(16, graph=True)
    ow.step(16, ORDER_PART)
    compare_states(world.state(), ow.state(), types, "fire f32 fused")
    compare_particles(world.particles(), ow.particles(), "fire f32 fused", temperature=True)
    assert np.array_equal(world.temperature(), ow.temperature())
    world.close()


def test_fused_interactions_wide_halo(fse, oracle_mod):
    """Interactions: the 11 x 11 lattice and the 5-cell halo."""
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
        world, ow = _pair(fse, oracle_mod, 320, 256, 113)
        world.set_launch(FUSED)
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


def test_fused_batch_mixed_iterations_and_zone(fse, oracle_mod):
    """A batch whose worlds run 3, 1 and 5 iterations (passes past a world's count
    only publish their flags) and one of which ticks a zone; 12-tick graphs."""
    types = material_types(fse)
    spec = [(256, 192, 3), (384, 256, 1), (128, 320, 5), (200, 200, 3)]
    worlds, oracles = [], []
    for i, (w, h, it) in enumerate(spec):
        world, ow = _pair(fse, oracle_mod, w, h, 900 + i, cell_iter=it)
        if i == 1:
            world.set_tick_zone(64, 0, 256, 256)
            ow.set_tick_zone(64, 0, 256, 256)
        worlds.append(world)
        oracles.append(ow)
    b = fse.Batch(worlds)
    b.set_launch(FUSED, 0)
    b.step(12, graph_ticks=12)
    b.step(3)
    for world, ow in zip(worlds, oracles):
        ow.step(15, ORDER_PART)
        compare_states(world.state(), ow.state(), types, "batch fused")
        compare_particles(world.particles(), ow.particles(), "batch fused")
    b.close()
    for world in worlds:
        world.close()


def test_fused_zone_change_and_shape_switch(fse, oracle_mod):
    """The zone shrinks between fused ticks (fewer chunks than the flags last held),
    and the shape switches between per-pass launches and the fused tick."""
    types = material_types(fse)
    world, ow = _pair(fse, oracle_mod, 640, 384, 31)
    world.set_launch(FUSED)
    world.step(2)
    ow.step(2, ORDER_PART)
    for zone in [(128, 0, 256, 256), (0, 128, 640, 256), (0, 0, 640, 384)]:
        world.set_tick_zone(*zone)
        ow.set_tick_zone(*zone)
        world.step(2)
        ow.step(2, ORDER_PART)
        compare_states(world.state(), ow.state(), types, "zone %s" % (zone,))
        compare_particles(world.particles(), ow.particles(), "zone %s" % (zone,))
    for shape in (0, FUSED, 1, FUSED):
        world.set_launch(shape)
        world.step(1)
        ow.step(1, ORDER_PART)
    compare_states(world.state(), ow.state(), types, "shape switches")
    compare_particles(world.particles(), ow.particles(), "shape switches")
    np.testing.assert_array_equal(world.ledger(), ow.ledger())
    world.close()


def test_fused_equals_per_pass_on_a_large_world(fse):
    """Bit-identical planes and particle lists after ticks of a 2048 x 1024 world
    with particles (32 chunk-passes a pass: CTAs run chunk-passes of several passes
    at once)."""
    import bench

    out = []
    for shape in (0, FUSED):
        w = fse.World(2048, 1024, seed=4321, particle_capacity=1 << 20)
        w.generate(fse.GEN_MIX, 4321)
        w.addCell(bench.config1_particles(200_000, 2048, 1024, 4321))
        w.set_launch(shape)
        w.step(6)
        out.append((w.state(), w.particles().tobytes(), w.tick_count))
        w.close()
    (sa, pa, ta), (sb, pb, tb) = out
    for k in sa:
        np.testing.assert_array_equal(sa[k], sb[k], err_msg=k)
    assert pa == pb and ta == tb
