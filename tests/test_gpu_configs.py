"""Parity on the benchmark configurations themselves, at their stated sizes.

The smaller parity tests exercise the rules on worlds of a few hundred cells a
side; these run the workloads the bench measures and compare the device with the
partitioned CPU oracle bit for bit:

* the 512 x 512 world (seed 1234), all 1000 steps (tick + tickCells): planes,
  particle list and ledger every 50 steps and at the end;
* the 4096 x 2048 world with the bench's own 1M free particles, 10 steps: every
  plane and the particle list after each step;
* 16 of the 256 uneven worlds of the batch workload, ticked inside the whole
  256-world batch by 32-tick CUDA graphs with the autotuned launch shape, each
  against its own oracle world.
"""
import numpy as np
import pytest

from helpers import compare_particles, compare_states, material_types

pytestmark = pytest.mark.gpu

ORDER_PART = 1


def _threads(oracle_mod):
    import os

    oracle_mod.Oracle().set_threads(os.cpu_count() or 1)


def test_config0_512_full_1000_steps(fse, oracle_mod):
    _threads(oracle_mod)
    types = material_types(fse)
    w = h = 512
    world = fse.World(w, h, chunk_size=128, cell_iter=3, seed=1234)
    world.generate(fse.GEN_MIX, 1234)
    ow = oracle_mod.OracleWorld(w, h, 128, 3, 1234)
    ow.generate(0, 1234)
    compare_states(world.state(), ow.state(), types, "config0 generate")
    done = 0
    while done < 1000:
        world.step(50)
        ow.step(50, ORDER_PART)
        done += 50
        what = "config0 step %d" % done
        compare_states(world.state(), ow.state(), types, what)
        compare_particles(world.particles(), ow.particles(), what)
        np.testing.assert_array_equal(world.ledger(), ow.ledger(), err_msg=what + " ledger")
    np.testing.assert_array_equal(world.census(), ow.census())


def test_config1_4096x2048_with_1m_particles(fse, oracle_mod):
    import bench

    _threads(oracle_mod)
    types = material_types(fse)
    W, H, seed = 4096, 2048, 1234
    world = fse.World(W, H, chunk_size=128, cell_iter=3, seed=seed, particle_capacity=4_000_000,
                      spawn_capacity=2_000_000)
    world.generate(fse.GEN_MIX, seed)
    parts = bench.config1_particles(1_000_000, W, H, seed)
    world.addCell(parts)
    ow = oracle_mod.OracleWorld(W, H, 128, 3, seed)
    ow.generate(0, seed)
    ow.set_particles(parts)
    for t in range(10):
        world.step(1)
        ow.step(1, ORDER_PART)
        what = "config1 step %d" % t
        compare_states(world.state(), ow.state(), types, what)
        compare_particles(world.particles(), ow.particles(), what)
    np.testing.assert_array_equal(world.ledger(), ow.ledger())
    world.close()


def test_config2_batched_graph_worlds(fse, oracle_mod):
    import bench

    _threads(oracle_mod)
    types = material_types(fse)
    sizes = bench.config2_sizes(256, 1234)
    worlds = []
    for i, (w, h) in enumerate(sizes):
        wd = fse.World(w, h, chunk_size=128, cell_iter=3, seed=1234 + i)
        wd.generate(fse.GEN_MIX, 1234 + i)
        worlds.append(wd)
    batch = fse.Batch(worlds)
    batch.autotune()  # restores every world: the tuned shape then runs the steps
    batch.step(32, graph_ticks=32)
    for i in range(0, 256, 16):
        w, h = sizes[i]
        ow = oracle_mod.OracleWorld(w, h, 128, 3, 1234 + i)
        ow.generate(0, 1234 + i)
        ow.step(32, ORDER_PART)
        what = "config2 world %d (%dx%d) after 32 graph steps" % (i, w, h)
        compare_states(worlds[i].state(), ow.state(), types, what)
        compare_particles(worlds[i].particles(), ow.particles(), what)
    batch.close()
    for wd in worlds:
        wd.close()
