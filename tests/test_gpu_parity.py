"""Bit-exact parity of the CUDA world tick with the partitioned CPU oracle."""
import numpy as np
import pytest

from helpers import compare_particles, compare_states, material_types

pytestmark = pytest.mark.gpu

ORDER_PART = 1


def _pair(fse, oracle_mod, w, h, seed, kind=1, chunk=128, cell_iter=3):
    world = fse.World(w, h, chunk_size=chunk, cell_iter=cell_iter, seed=seed)
    world.generate(kind, seed)
    ow = oracle_mod.OracleWorld(w, h, chunk, cell_iter, seed)
    ow.generate({1: 0, 2: 1}[kind], seed)
    return world, ow


@pytest.mark.parametrize("w,h", [(128, 128), (192, 160), (384, 256)])
def test_generator_matches(fse, oracle_mod, w, h):
    world, ow = _pair(fse, oracle_mod, w, h, 1234)
    compare_states(world.state(), ow.state(), material_types(fse), "generate")


@pytest.mark.parametrize("w,h,ticks", [(192, 160, 1), (256, 256, 6), (320, 192, 12)])
def test_tick_only_parity(fse, oracle_mod, w, h, ticks):
    types = material_types(fse)
    world, ow = _pair(fse, oracle_mod, w, h, 77)
    for t in range(ticks):
        world.tick(1)
        ow.tick(ORDER_PART)
        compare_states(world.state(), ow.state(), types, "tick %d" % t)
    compare_particles(world.particles(), ow.particles(), "spawned")


@pytest.mark.parametrize("w,h,steps", [(256, 192, 8), (512, 512, 4)])
def test_step_parity(fse, oracle_mod, w, h, steps):
    types = material_types(fse)
    world, ow = _pair(fse, oracle_mod, w, h, 1234)
    for t in range(steps):
        world.step(1)
        ow.step(1, ORDER_PART)
        compare_states(world.state(), ow.state(), types, "step %d" % t)
        compare_particles(world.particles(), ow.particles(), "step %d" % t)


def test_zipf_world_parity(fse, oracle_mod):
    types = material_types(fse)
    world, ow = _pair(fse, oracle_mod, 384, 384, 99, kind=2)
    world.step(3)
    ow.step(3, ORDER_PART)
    compare_states(world.state(), ow.state(), types, "zipf")
    compare_particles(world.particles(), ow.particles(), "zipf")


def test_ledger_matches_oracle(fse, oracle_mod):
    world, ow = _pair(fse, oracle_mod, 256, 256, 5)
    world.step(5)
    ow.step(5, ORDER_PART)
    np.testing.assert_array_equal(world.ledger(), ow.ledger())
    np.testing.assert_array_equal(world.census(), ow.census())


@pytest.mark.parametrize("chunk,cell_iter,w,h", [(16, 3, 96, 80), (32, 1, 200, 136), (64, 2, 200, 136),
                                                  (96, 5, 288, 200), (128, 8, 256, 192), (48, 4, 150, 170)])
def test_chunk_and_iteration_variants(fse, oracle_mod, chunk, cell_iter, w, h):
    """Other chunk edges and iteration counts than the reference's 128 / 3, on
    worlds that are not multiples of the chunk: planes and particles after steps."""
    types = material_types(fse)
    world, ow = _pair(fse, oracle_mod, w, h, 4321 + chunk, chunk=chunk, cell_iter=cell_iter)
    for t in range(4):
        world.step(1)
        ow.step(1, ORDER_PART)
        compare_states(world.state(), ow.state(), types, "chunk %d iter %d step %d" % (chunk, cell_iter, t))
        compare_particles(world.particles(), ow.particles(), "chunk %d iter %d step %d" % (chunk, cell_iter, t))
