"""Seeded inputs for the temperature-conduction parity tests (world.cpp:1950-2004).

Shared by the golden-fixture generator, the CPU tests (oracle against the
reference's own function) and the GPU tests (CUDA against the oracle).
"""
import numpy as np

# name, w, h, seed, temperature regime, material edits
CASES = [
    ("builtin_mixed", 96, 64, 1, "mixed", "builtin"),
    ("builtin_wide", 80, 48, 2, "wide", "builtin"),
    ("builtin_sparse", 128, 40, 3, "sparse", "builtin"),
    ("edge_params", 72, 56, 4, "wide", "edge"),
    ("edge_cancel", 64, 64, 5, "cancel", "edge"),
]

# (index name, addTemp, conductionSelf, conductionOther): values that reach the
# corners of the arithmetic -- u32 wrap of addTemp, negative and zero weights,
# overflow to inf and NaN (0 * inf), the INT32_MIN of an out-of-range conversion
EDGE = [
    ("STONE", 70000, 0.0, 0.25),
    ("GENERIC_SAND", 4294967000, 2.5, -0.5),
    ("WATER", 3, -1.0, 3.0),
    ("DIRT", 0, 1.0, 1e30),
    ("GRASS", 7, 0.3, float("inf")),
    ("OBSIDIAN", 1, 1e-30, 1e-30),
    ("GOLD_ORE", 123456789, 0.75, 0.0),
]


def apply_edits(set_conduction, find, edits):
    """Apply the material edits of a case through a set_conduction(id, add, cs, co) call."""
    if edits != "edge":
        return
    for name, add, cs, co in EDGE:
        mid = find(name)
        assert mid >= 0, name
        set_conduction(mid, add, cs, co)


def case_inputs(o, case):
    """(material ids, temperatures) of a case; applies its material edits to the oracle."""
    name, w, h, seed, regime, edits = case
    rng = np.random.default_rng(seed)
    n_mat = o.material_count()
    mat = rng.integers(0, n_mat, size=(h, w)).astype(np.uint16)
    if regime == "mixed":
        t = np.where(rng.random((h, w)) < 0.5, 0, rng.integers(-200, 201, size=(h, w)))
        wide = rng.random((h, w)) < 0.25
        t = np.where(wide, rng.integers(-32768, 32768, size=(h, w)), t)
    elif regime == "wide":
        t = rng.integers(-32768, 32768, size=(h, w))
    elif regime == "sparse":
        t = np.where(rng.random((h, w)) < 0.9, 0, rng.choice([-1023, 1024, 64, -64, 63, 128], size=(h, w)))
    else:  # "cancel": +-t pairs so that the weighted sum is often exactly zero
        base = rng.choice([64, 128, 640, 1023], size=(h, w))
        sign = np.where((np.add.outer(np.arange(h), np.arange(w)) % 2) == 0, 1, -1)
        t = base * sign
    apply_edits(o.set_conduction, o.find, edits)
    return mat, t.astype(np.int16)


def material_params(o):
    """(addTemp u32, conductionSelf f32, conductionOther f32) per oracle material."""
    import ctypes as C

    n = o.material_count()
    lib = o.lib
    f = lib.om_material_conduction
    f.restype = None
    f.argtypes = [C.c_int, C.c_void_p]
    add = np.zeros(n, np.uint32)
    cs = np.zeros(n, np.float32)
    co = np.zeros(n, np.float32)
    buf = np.zeros(3, np.uint32)
    for k in range(n):
        f(k, buf.ctypes.data_as(C.c_void_p))
        add[k] = buf[0]
        cs[k] = buf[1:2].view(np.float32)[0]
        co[k] = buf[2:3].view(np.float32)[0]
    return add, cs, co
