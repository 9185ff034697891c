"""The built-in material table against the reference's own code and text.

oracle/Makefile `ref` compiles the reference's list of built-in materials (test() of
game_datastruct.cpp:70-111 with the Material constructors it calls) when the
reference tree is present; the oracle's table and the product's (the C ABI's
fse_material_get, which needs no GPU) must hold the same ids, types,
slipperiness, alpha, density, iterations, emission and colours. The conduction
constants, reactions and SOUP factory temperatures set in InitMaterials and the
tile factories (game_datastruct.cpp:124-141, 246-260, 427-437) are read from the
reference's text.
"""
import ctypes as C
import os
import re

import numpy as np
import pytest


def _ref_ds():
    from oracle.binding import REFERENCE_WORLD_CPP

    return os.path.join(os.path.dirname(REFERENCE_WORLD_CPP), "game_datastruct.cpp")


def _ref_table():
    from oracle.binding import HERE, REFERENCE_WORLD_CPP, make_ref

    if not os.path.exists(REFERENCE_WORLD_CPP):
        pytest.skip("reference tree absent")

    make_ref()
    lib = C.CDLL(os.path.join(HERE, "_ref", "libref_materials.so"))
    out = np.zeros(64 * 10, np.int32)
    names = C.create_string_buffer(64 * 48)
    lib.ref_materials.restype = C.c_int
    n = lib.ref_materials(out.ctypes.data_as(C.c_void_p), names, 64)
    rows = out.reshape(64, 10)[:n]
    idx = [names.raw[48 * k: 48 * k + 48].split(b"\0")[0].decode() for k in range(n)]
    return rows, idx


def _check(get, find, rows, idx):
    for k, name in enumerate(idx):
        r = rows[k]
        assert r[0] == k and find(name) == k, name
        m = get(k)  # type, density bits, iterations, slip, max_stab, alpha, colour, emit, emit_colour, ...
        assert m[0] == r[1], (name, "type")
        assert m[3] == r[2], (name, "slipperyness")
        assert m[5] == r[3], (name, "alpha")
        assert m[1] == r[4], (name, "density")
        assert m[2] == r[5], (name, "iterations")
        assert m[7] == r[6], (name, "emit")
        assert (int(m[8]) & 0xFFFFFFFF) == (int(r[7]) & 0xFFFFFFFF), (name, "emitColor")
        assert (int(m[6]) & 0xFFFFFFFF) == (int(r[8]) & 0xFFFFFFFF), (name, "color")


def test_oracle_table_matches_reference(oracle_mod):
    rows, idx = _ref_table()
    o = oracle_mod.Oracle()
    o.reset_materials()
    assert len(idx) == 28
    _check(o.material, o.find, rows, idx)


def test_product_table_matches_reference():
    rows, idx = _ref_table()
    import falling_sand_engine_gb300 as fse

    lib = fse.lib()
    lib.fse_materials_begin()

    def get(k):
        out = np.zeros(16, np.int32)
        assert lib.fse_material_get(k, out.ctypes.data_as(C.c_void_p)) == 0
        return out

    _check(get, lambda s: lib.fse_material_find(s.encode()), rows, idx)


def test_conduction_reactions_factories_match_reference_text(oracle_mod):
    if not os.path.exists(_ref_ds()):
        pytest.skip("reference tree absent")
    text = open(_ref_ds(), encoding="utf-8", errors="replace").read()
    o = oracle_mod.Oracle()
    o.reset_materials()
    import ctypes

    cond = {}
    for name, field, val in re.findall(r"materials_list\.(\w+)\.(conductionSelf|conductionOther|addTemp) = ([-\d.]+);",
                                       text):
        cond.setdefault(name, {})[field] = float(val)
    assert len(cond) >= 6
    f = o.lib.om_material_conduction
    f.restype = None
    f.argtypes = [ctypes.c_int, ctypes.c_void_p]
    for name, fields in cond.items():
        buf = np.zeros(3, np.uint32)
        f(o.find(name), buf.ctypes.data_as(ctypes.c_void_p))
        add, cs, co = int(buf[0]), buf[1:2].view(np.float32)[0], buf[2:3].view(np.float32)[0]
        assert add == int(fields.get("addTemp", 0)), name
        assert cs == np.float32(fields.get("conductionSelf", 1.0)), name
        assert co == np.float32(fields.get("conductionOther", 1.0)), name
    reacts = re.findall(r"materials_list\.(\w+)\.id\]->reactions\.push_back\(\{(REACT_TEMPERATURE_\w+), (\d+), "
                        r"GAME\(\)->materials_list\.(\w+)\.id\}\)", text)
    assert len(reacts) == 4
    for mat, kind, temp, res in reacts:
        m = o.material(o.find(mat))
        assert m[14] >= 1, mat  # has a reaction
    temps = dict((n, int(t)) for n, t in re.findall(r"MaterialInstance\(&GAME\(\)->materials_list\.(\w+), rgb, (-?\d+)\)",
                                                    text))
    assert temps == {"WATER": -1023, "LAVA": 1024}
    buf = np.zeros(4, np.uint32)
    import falling_sand_engine_gb300 as fse

    for name, t in temps.items():
        assert fse.lib().fse_material_get_conduction(fse.lib().fse_material_find(name.encode()),
                                                     buf.ctypes.data_as(ctypes.c_void_p)) == 0
        assert int(buf[3:4].view(np.int32)[0]) == t, name


def test_tile_layout_matches_reference():
    """TILE_DTYPE, its fse_tile_layout and FSE_TILE_LAYOUT_MATERIAL_INSTANCE against
    sizeof / offsetof of the reference's own MaterialInstance class
    (game_datastruct.hpp:206-224), compiled unchanged."""
    from oracle.binding import HERE

    _ref_table()  # builds the harness
    lib = C.CDLL(os.path.join(HERE, "_ref", "libref_materials.so"))
    ref = np.zeros(9, np.int32)
    lib.ref_tile_layout.restype = None
    lib.ref_tile_layout(ref.ctypes.data_as(C.c_void_p))
    import falling_sand_engine_gb300 as fse
    from falling_sand_engine_gb300._abi import FseTileLayout

    lay = FseTileLayout.of(fse.TILE_DTYPE)
    assert [getattr(lay, k) for k, _ in FseTileLayout._fields_] == ref.tolist()
    hdr = open(os.path.join(os.path.dirname(HERE), "include", "fse.h")).read()
    m = re.search(r"#define FSE_TILE_LAYOUT_MATERIAL_INSTANCE \{([^}]*)\}", hdr)
    assert [int(v) for v in m.group(1).split(",")] == ref.tolist()
