"""Seeded scenes for pinning the free-particle update against the reference's own
world::tickCells (world.cpp:2030-2195).

Particles sit on a lattice 48 cells apart and move less than 8 cells per tick, so
no particle's path, deposit or 32x32 spiral search meets another's within a tick:
in that case every order of deposits gives the reference's sequential result.
Liquid amounts are multiples of 1/256, exact both in float and in Q16.16.
"""
import numpy as np

W, H = 384, 288
SPACING = 48


def scene(o, seed):
    """(ids, colours, amounts Q16.16, particles) over the oracle's material table."""
    rng = np.random.default_rng(seed)
    f = o.find
    air, stone, sand, water, obj, gas = f("GENERIC_AIR"), f("STONE"), f("GENERIC_SAND"), f("WATER"), \
        f("GENERIC_OBJECT"), f("GENERIC_GAS")
    ids = np.full((H, W), air, np.uint16)
    # blocks of solid, sand, liquid and object, and scattered obstacles
    for _ in range(40):
        x0, y0 = rng.integers(0, W - 20), rng.integers(0, H - 20)
        ww, hh = rng.integers(3, 20), rng.integers(3, 20)
        ids[y0:y0 + hh, x0:x0 + ww] = rng.choice([stone, sand, water, obj])
    ids[rng.random((H, W)) < 0.04] = stone
    colours = rng.choice(np.array([0x202020, 0x808080, 0xC2B280, 0x00B69F, 0x00FF00, 0x8C6E5A, 0xFFFFFF, 0x123456],
                                  np.uint32), size=(H, W))
    amounts = np.where(ids == water, rng.integers(1, 1024, size=(H, W)) * 256, 0).astype(np.int32)
    ys, xs = np.mgrid[24:H - 24:SPACING, 24:W - 24:SPACING]
    n = ys.size
    from oracle.binding import PARTICLE_DTYPE

    p = np.zeros(n, PARTICLE_DTYPE)
    p["x"] = xs.ravel() + rng.uniform(0, 1, n).astype(np.float32)
    p["y"] = ys.ravel() + rng.uniform(0, 1, n).astype(np.float32)
    p["vx"] = rng.uniform(-3, 3, n).astype(np.float32)
    p["vy"] = rng.uniform(-3, 3, n).astype(np.float32)
    p["ax"] = rng.choice([0.0, 0.05, -0.05], n).astype(np.float32)
    p["ay"] = rng.choice([0.0, 0.1, 0.01], n).astype(np.float32)
    steer = rng.random(n) < 0.2
    p["target_x"] = np.where(steer, p["x"] + rng.uniform(-200, 200, n), 0).astype(np.float32)
    p["target_y"] = np.where(steer, p["y"] + rng.uniform(-200, 200, n), 0).astype(np.float32)
    p["target_force"] = np.where(steer, rng.uniform(0.05, 0.5, n), 0).astype(np.float32)
    p["lifetime"] = rng.integers(0, 40, n)
    p["fade_time"] = 60
    tile = rng.choice([sand, water, gas, stone], n)
    p["id"] = tile
    p["colour"] = rng.integers(0, 1 << 24, size=n)
    p["scalar"] = np.where(tile == water, rng.integers(1, 1024, size=n) * 256, 0)
    phase = rng.random(n) < 0.1
    temporary = rng.random(n) < 0.15
    state = rng.integers(0, 3, n)
    p["bits"] = (phase.astype(np.uint8) | (temporary.astype(np.uint8) << 1) | (state.astype(np.uint8) << 2))
    return ids, colours, amounts, p


# Contested scenes: particles as dense as on the 4096 x 2048 bench world (1M particles
# on 8.4M cells), so that flights run into cells deposited earlier in the same tick,
# previous cells fill up and spiral searches compete for the same AIR cells; a
# margin of rock keeps every spiral search inside the grid (the reference's search
# reads neighbours without bounds checks).
CW, CH, CMARGIN = 384, 256, 32


def contested_scene(o, seed):
    """(ids, colours, amounts Q16.16, particles) of a contested scene: the bench mix
    (30% sand, 20% water, 10% gas, 15% stone, 25% air in the top 60%, rock below),
    a rock margin, and sand and water particles at the bench's density with
    velocities N(0, 2) (clipped to 8 cells/tick) and gravity 0.1."""
    rng = np.random.default_rng(seed)
    f = o.find
    air, stone, sand, water, gas = f("GENERIC_AIR"), f("STONE"), f("GENERIC_SAND"), f("WATER"), f("GENERIC_GAS")
    ids = np.full((CH, CW), air, np.uint16)
    u = rng.random((CH, CW))
    top = (np.arange(CH) < int(CH * 0.6))[:, None]
    pal = np.select([u < 0.3, u < 0.5, u < 0.6, u < 0.75], [sand, water, gas, stone], air)
    ids[:] = np.where(top, pal, air)
    ids[CH - 8:, :] = stone
    ids[:CMARGIN // 2, :] = stone
    ids[:, :CMARGIN // 2] = stone
    ids[:, CW - CMARGIN // 2:] = stone
    colours = rng.choice(np.array([0x808080, 0xC2B280, 0x00B69F, 0x8C6E5A], np.uint32), size=(CH, CW))
    amounts = np.where(ids == water, rng.integers(1, 64, size=(CH, CW)) * 4096, 0).astype(np.int32)
    inner = (CW - 2 * CMARGIN) * (CH - 2 * CMARGIN)
    n = int(round(1_000_000 * inner / (4096 * 2048)))
    from oracle.binding import PARTICLE_DTYPE

    p = np.zeros(n, PARTICLE_DTYPE)
    p["x"] = rng.uniform(CMARGIN, CW - CMARGIN, n).astype(np.float32)
    p["y"] = rng.uniform(CMARGIN, CH - CMARGIN, n).astype(np.float32)
    p["vx"] = np.clip(rng.normal(0.0, 2.0, n), -8, 8).astype(np.float32)
    p["vy"] = np.clip(rng.normal(0.0, 2.0, n), -8, 8).astype(np.float32)
    p["ay"] = np.float32(0.1)
    p["fade_time"] = 60
    liquid = rng.random(n) < 0.3
    p["id"] = np.where(liquid, water, sand)
    p["colour"] = np.where(liquid, 0x00B69F, 0xC2B280)
    p["scalar"] = np.where(liquid, rng.integers(1, 64, size=n) * 4096, 0)
    return ids, colours, amounts, p
