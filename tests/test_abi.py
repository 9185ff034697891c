"""CPU checks of the C-ABI library: it loads without a GPU, exports every symbol
declared in include/fse.h, and its host-side logic (material table, Lua loader,
argument validation) matches the oracle and the reference interface."""
import os
import re
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def lib():
    from falling_sand_engine_gb300 import build

    build.build()
    import falling_sand_engine_gb300 as fse

    fse.lib()
    fse.InitMaterials()
    return fse


def _declared():
    text = open(os.path.join(ROOT, "include", "fse.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(fse_[a-z0-9_]+)\s*\(", text)))


def test_every_declared_symbol_is_exported(lib):
    out = subprocess.run(["nm", "-D", "--defined-only", lib._abi.LIB_PATH], capture_output=True, text=True).stdout
    exported = set(re.findall(r" T (fse_[a-z0-9_]+)", out))
    missing = [s for s in _declared() if s not in exported]
    assert not missing, missing
    bound = set(lib._abi.SIGNATURES)
    assert set(_declared()) == bound, set(_declared()) ^ bound


def test_material_table_matches_the_oracle(lib, oracle_mod):
    o = oracle_mod.Oracle()
    assert lib.material_count() == o.material_count() == 31
    for i in range(lib.material_count()):
        np.testing.assert_array_equal(lib.material_get(i), o.material(i), err_msg=str(i))
    # ids follow InitMaterials' registration order (game_datastruct.cpp:143-170)
    for name, mid in (("GENERIC_AIR", 0), ("GENERIC_SAND", 2), ("GENERIC_GAS", 4), ("GENERIC_OBJECT", 6),
                      ("STONE", 7), ("WATER", 15), ("LAVA", 16), ("STEAM", 23), ("FIRE", 25), ("TEST_LIQUID", 30)):
        assert lib.material_find(name) == mid


def test_lua_loader_parses_the_register_call(lib):
    try:
        n = lib.load_lua_materials("""
            materials_register(3001, "A", "MAT_A", 2, 20, 255, 10, 2, 0, 0, 0xFF00FF00) -- sand-like
            --[[ materials_register(0, "commented", "NO", 0, 0, 0, 0, 0, 0, 0, 0) ]]
            materials_register(3002, 'B', 'MAT_B', 3, 0, 128, 1.5 * 2, 3, 40, 0x3000AFB5, 255)
        """)
        assert n == 2
        a, b = lib.material_get(lib.material_find("MAT_A")), lib.material_get(lib.material_find("MAT_B"))
        assert (a[0], a[2], a[3]) == (2, 2, 20)
        assert b[0] == 3 and np.int32(b[1]).view(np.float32) == np.float32(3.0) and b[7] == 40
        assert lib.material_find("NO") == -1
    finally:
        lib.InitMaterials()


def test_bad_arguments_are_status_codes(lib):
    import ctypes as C

    L = lib.lib()
    h = C.c_void_p()
    assert L.fse_world_create(0, 10, None, C.byref(h)) == -1
    cfg = lib._abi.FseConfig(8, 3, 0, 0, 0, None)  # chunk below the lattice reach
    assert L.fse_world_create(64, 64, C.byref(cfg), C.byref(h)) == -1
    out = C.c_int()
    assert L.fse_material_register(0, b"x", b"X", 9, 0, 255, 1.0, 1, 0, 0, 0, C.byref(out)) == -1
    assert L.fse_material_set_interaction(2, 15, 1, 9, 4, 2, 0) == -1  # reach 6 > halo
    assert L.fse_world_tick(None, 1) == -1
    lay = lib._abi.FseTileLayout.of(lib.TILE_DTYPE)
    assert L.fse_world_upload_tiles(None, None, C.byref(lay)) == -1
    assert L.fse_world_download_tiles(None, None, C.byref(lay), None, 0) == -1
    assert L.fse_status_string(-3) == b"HBM budget exceeded"
    with pytest.raises(lib.FseError):
        lib.RegisterMaterial(0, "bad", "BAD", 7, 0, 255, 1.0, 1)
