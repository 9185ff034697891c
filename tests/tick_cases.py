"""Seeded scenes for pinning the oracle's cell rules against the reference's own
world::tick (source/engine/world.cpp:1036-1948), compiled by oracle/Makefile.

The scenes of CASES hold no liquids: the reference keeps fluid amounts in f32 and
this path in Q16.16 by design, so a flow at the FLUID_MinValue threshold can land on
either side and liquid cells cannot agree bit for bit; the "liquid" scene is compared
with a tolerance instead. Every other rule of the tick runs: falling and sliding sand with friction pillars, slipperiness and
density, gas rising and spreading, fire (particles, recolouring, spreading to solids,
burning out), temperature reactions and both kinds of interaction. A solid border
keeps every read inside the grid (the reference reads raw neighbours there); worlds
are whole chunks (the reference ticks whole chunks).
"""
import numpy as np

BORDER_X, BORDER_TOP, BORDER_BOTTOM = 6, 6, 12
REACT_BELOW, REACT_ABOVE = 4, 5
INTER_TRANSFORM, INTER_SPAWN = 1, 2

# (name, physics type, slipperyness, density, iterations, factory: base, shift, lo, mod, temperature)
CUSTOM = [
    ("PIN_SAND_A", 2, 1, 12.0, 3, 0xFFC8A000, 8, 10, 40, 20),
    ("PIN_SAND_B", 2, 3, 9.0, 2, 0xFF907050, 0, 0, 30, -5),
    ("PIN_SAND_C", 2, 7, 20.0, 1, 0xFF404040, 16, 5, 60, 300),
    ("PIN_GAS", 4, 1, 0.5, 3, 0xFF9090FF, 0, 0, 0, 0),
    ("PIN_ROCK", 1, 1, 50.0, 0, 0xFF303030, 0, 0, 0, 0),
]
SOUP, Q_DEFAULT = 3, 131072


def setup_materials(o):
    """Resets the oracle's table to the built-ins and registers the scene materials,
    their reactions and interactions; returns {name: id}."""
    o.reset_materials()
    ids = {}
    for k, (name, typ, slip, dens, iters, base, sh, lo, mod, temp) in enumerate(CUSTOM):
        mid = o.register(4001 + k, name.title(), name, typ, slip, 255, dens, iters, 0, 0, base)
        assert mid >= 0
        assert o.set_factory(mid, base, sh, lo, mod, temp) == 0
        ids[name] = mid
    for name in ("GENERIC_AIR", "GENERIC_SOLID", "GENERIC_SAND", "GENERIC_GAS", "FIRE", "STONE", "WATER", "LAVA"):
        ids[name] = o.find(name)
    a, b, c = ids["PIN_SAND_A"], ids["PIN_SAND_B"], ids["PIN_SAND_C"]
    assert o.set_reaction(a, REACT_ABOVE, 200, b) == 0
    assert o.set_reaction(b, REACT_BELOW, -100, c) == 0
    # a threshold outside i16: the reference keeps it as an i16 (-65000 -> 536)
    assert o.set_reaction(c, REACT_ABOVE, -65000, ids["GENERIC_SAND"]) == 0
    # sand C on rock turns the rock of a box below it into sand B; sand A on generic
    # sand spawns gas into the air of a box (and into its own cell); sand B on stone
    # has a box with a negative corner, which the reference's loops never visit
    assert o.set_interaction(c, ids["PIN_ROCK"], INTER_TRANSFORM, b, 1, 1, 2) == 0
    assert o.set_interaction(a, ids["GENERIC_SAND"], INTER_SPAWN, ids["PIN_GAS"], 1, 1, 1) == 0
    assert o.set_interaction(b, ids["STONE"], INTER_SPAWN, ids["PIN_GAS"], 1, 0, 1) == 0
    return ids


def scene(ids, w, h, seed, kind):
    """Planes (id, colour, scalar = temperature, flags, diff) of a seeded scene."""
    rng = np.random.default_rng(seed)
    air, solid = ids["GENERIC_AIR"], ids["GENERIC_SOLID"]
    mid = np.full((h, w), air, np.int64)
    u = rng.random((h, w))
    if kind == "sand":
        pal = [ids["PIN_SAND_A"], ids["PIN_SAND_B"], ids["PIN_SAND_C"], ids["GENERIC_SAND"], ids["STONE"],
               ids["PIN_ROCK"]]
        p = np.array([0.16, 0.12, 0.08, 0.16, 0.04, 0.04])
    elif kind == "liquid":
        pal = [ids["WATER"], ids["LAVA"], ids["GENERIC_SAND"], ids["GENERIC_GAS"], ids["STONE"]]
        p = np.array([0.25, 0.05, 0.2, 0.1, 0.1])
    elif kind == "gas":
        pal = [ids["GENERIC_GAS"], ids["PIN_GAS"], ids["GENERIC_SAND"], ids["PIN_ROCK"]]
        p = np.array([0.25, 0.2, 0.1, 0.05])
    else:  # fire among sand, gas and solids
        pal = [ids["FIRE"], ids["STONE"], ids["PIN_ROCK"], ids["GENERIC_SAND"], ids["PIN_SAND_A"], ids["GENERIC_GAS"]]
        p = np.array([0.12, 0.1, 0.06, 0.12, 0.08, 0.08])
    edges = np.cumsum(p)
    for k, m in enumerate(pal):
        lo = 0.0 if k == 0 else edges[k - 1]
        mid[(u >= lo) & (u < edges[k])] = m
    # piles and holes: a few empty rows and a solid shelf
    mid[h // 3: h // 3 + 4, :] = air
    mid[h // 2, w // 4: w // 2] = ids["PIN_ROCK"]
    mid[:BORDER_TOP, :] = solid
    mid[h - BORDER_BOTTOM:, :] = solid
    mid[:, :BORDER_X] = solid
    mid[:, w - BORDER_X:] = solid
    colour = rng.integers(0, 2 ** 32, (h, w), dtype=np.uint64).astype(np.uint32)
    temp = rng.integers(-400, 1400, (h, w)).astype(np.int32)
    temp[mid == air] = 0
    flags = np.where(rng.random((h, w)) < 0.3, 0x80, 0).astype(np.uint8)
    soup = np.isin(mid, [ids["WATER"], ids["LAVA"]])
    # liquids at the MaterialInstance default amount, their temperature beside it
    return {"id": mid.astype(np.uint16), "colour": colour, "scalar": np.where(soup, Q_DEFAULT, temp).astype(np.int32),
            "flags": flags, "diff": np.zeros((h, w), np.int32), "temperature": temp.astype(np.int16)}


# (w, h, seed, kind, cell_iter, ticks)
CASES = [
    (256, 256, 11, "sand", 3, 1),
    (256, 256, 12, "sand", 3, 3),
    (384, 256, 13, "gas", 2, 2),
    (256, 384, 14, "fire", 3, 2),
    (256, 256, 15, "sand", 1, 4),
]


def scene_f32(ids, w, h, seed):
    """The liquid scene with the reference's own f32 liquid state: amounts spread over
    (0, 4) with exact zeros, values below FLUID_MinValue and near the free-fall and
    vertical-flow thresholds; small pending diffs on some cells; settle counts 0-15.
    Returns the planes of scene() (scalar and diff of liquid cells as f32 bit
    patterns) plus the float planes "amount" and "fluid_diff" and "settle"."""
    st = scene(ids, w, h, seed, "liquid")
    rng = np.random.default_rng(seed + 1000)
    amount = rng.uniform(0.0, 4.0, (h, w)).astype(np.float32)
    pick = rng.random((h, w))
    amount[pick < 0.03] = 0.0
    amount[(pick >= 0.03) & (pick < 0.06)] = rng.uniform(0.0, 0.001, (h, w)).astype(np.float32)[
        (pick >= 0.03) & (pick < 0.06)]
    amount[(pick >= 0.06) & (pick < 0.09)] = np.float32(0.5)
    amount[(pick >= 0.09) & (pick < 0.12)] = np.float32(2.0)
    diff = np.where(rng.random((h, w)) < 0.2, rng.uniform(-0.3, 0.3, (h, w)), 0.0).astype(np.float32)
    settle = rng.integers(0, 16, (h, w)).astype(np.uint8)
    soup = np.isin(st["id"], [ids["WATER"], ids["LAVA"]])
    amount = np.where(soup, amount, np.float32(2.0)).astype(np.float32)
    diff = np.where(soup, diff, np.float32(0.0)).astype(np.float32)
    settle = np.where(soup, settle, 0).astype(np.uint8)
    st["scalar"] = np.where(soup, amount.view(np.int32), st["scalar"]).astype(np.int32)
    st["diff"] = np.where(soup, diff.view(np.int32), 0).astype(np.int32)
    st["flags"] = (st["flags"] & 0x80) | np.where(soup, settle, 0).astype(np.uint8)
    st["amount"], st["fluid_diff"], st["settle"] = amount, diff, settle
    return st


# f32 liquid scenes: (w, h, seed, cell_iter, ticks)
F32_CASES = [
    (256, 256, 21, 3, 1),
    (384, 256, 22, 3, 3),
    (256, 384, 23, 2, 6),
]
