"""ctypes binding of the C ABI in include/fse.h (libfse.so, built in-tree)."""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libfse.so")

PARTICLE_DTYPE = np.dtype(
    [
        ("x", "<f4"), ("y", "<f4"), ("vx", "<f4"), ("vy", "<f4"), ("ax", "<f4"), ("ay", "<f4"),
        ("target_x", "<f4"), ("target_y", "<f4"), ("target_force", "<f4"),
        ("lifetime", "<i4"), ("fade_time", "<i4"), ("colour", "<u4"), ("scalar", "<i4"),
        ("id", "<u2"), ("flags", "u1"), ("bits", "u1"), ("temperature", "<i2"), ("reserved", "<u2"),
    ]
)
assert PARTICLE_DTYPE.itemsize == 60
BODY_DTYPE = np.dtype(
    [
        ("x", "<f4"), ("y", "<f4"), ("sin_a", "<f4"), ("cos_a", "<f4"),
        ("w", "<i4"), ("h", "<i4"), ("id", "<u2"), ("pad", "<u2"), ("colour", "<u4"),
        ("n_sand", "<i4"), ("n_soup", "<i4"), ("n_placed", "<i4"), ("n_recovered", "<i4"),
    ]
)
# fse_island
ISLAND_DTYPE = np.dtype([("root", "<i4"), ("cells", "<i4"), ("min_x", "<i4"), ("min_y", "<i4"), ("max_x", "<i4"),
                         ("max_y", "<i4")])


# MaterialInstance (source/engine/game_datastruct.hpp:205-222) on LP64 targets
TILE_DTYPE = np.dtype(
    {
        "names": ["id", "mat", "color", "temperature", "moved", "fluidAmount", "fluidAmountDiff", "settleCount"],
        "formats": ["<u4", "<u8", "<u4", "<i2", "u1", "<f4", "<f4", "u1"],
        "offsets": [0, 8, 16, 20, 22, 24, 28, 32],
        "itemsize": 40,
    }
)


class FseTileLayout(C.Structure):
    _fields_ = [(k, C.c_int32) for k in ("stride", "id", "mat", "colour", "temperature", "moved", "fluid_amount",
                                         "fluid_amount_diff", "settle_count")]

    @classmethod
    def of(cls, dtype):
        """The layout of a numpy structured dtype with MaterialInstance's field names."""
        f = dtype.fields
        off = lambda k: f[k][1] if k in f else -1
        return cls(dtype.itemsize, off("id"), off("mat"), off("color"), off("temperature"), off("moved"),
                   off("fluidAmount"), off("fluidAmountDiff"), off("settleCount"))


class FseConfig(C.Structure):
    _fields_ = [
        ("chunk_size", C.c_int32), ("cell_iter", C.c_int32), ("seed", C.c_uint32),
        ("particle_capacity", C.c_int32), ("spawn_capacity", C.c_int32), ("stream", C.c_void_p),
        ("flags", C.c_int32),
    ]


# name -> (restype, argtypes); every symbol declared in include/fse.h
_vp, _i, _u32, _i64, _f, _d = C.c_void_p, C.c_int, C.c_uint32, C.c_int64, C.c_float, C.c_double
_pp = C.POINTER(C.c_void_p)
SIGNATURES = {
    "fse_version": (C.c_char_p, []),
    "fse_status_string": (C.c_char_p, [_i]),
    "fse_materials_begin": (_i, []),
    "fse_material_register": (_i, [_i, C.c_char_p, C.c_char_p, _i, _i, _i, _f, _i, _i, _u32, _u32, C.POINTER(_i)]),
    "fse_material_set_reaction": (_i, [_i, _i, _i, _i]),
    "fse_material_set_interaction": (_i, [_i, _i, _i, _i, _i, _i, _i]),
    "fse_material_set_factory": (_i, [_i, _u32, _i, _i, _i, C.c_int32]),
    "fse_material_set_factory_temperature": (_i, [_i, C.c_int32]),
    "fse_material_set_conduction": (_i, [_i, _u32, _f, _f]),
    "fse_material_get_conduction": (_i, [_i, _vp]),
    "fse_world_temperature_read": (_i, [_vp, _vp]),
    "fse_world_temperature_write": (_i, [_vp, _vp]),
    "fse_world_tick_temperature": (_i, [_vp]),
    "fse_world_pack_bound": (_i, [_i, _i, _vp, _vp]),
    "fse_world_pack": (_i, [_vp, _i, _vp, _i64, _vp, _vp]),
    "fse_world_unpack": (_i, [_vp, _vp, _vp, _i, _vp, _vp]),
    "fse_world_checkpoint_bound": (_i, [_vp, _vp]),
    "fse_world_upload_tiles": (_i, [_vp, _vp, _vp]),
    "fse_world_trim": (_i, [_vp]),
    "fse_world_download_tiles": (_i, [_vp, _vp, _vp, _vp, _i]),
    "fse_world_checkpoint": (_i, [_vp, _vp, _i64, _vp]),
    "fse_world_restore": (_i, [_vp, _vp, _i64]),
    "fse_materials_load_lua": (_i, [C.c_char_p, C.POINTER(_i)]),
    "fse_materials_push": (_i, []),
    "fse_material_count": (_i, []),
    "fse_material_find": (_i, [C.c_char_p]),
    "fse_material_get": (_i, [_i, _vp]),
    "fse_world_create": (_i, [_i, _i, C.POINTER(FseConfig), _pp]),
    "fse_world_destroy": (_i, [_vp]),
    "fse_world_info": (_i, [_vp, _vp]),
    "fse_world_upload": (_i, [_vp, _vp, _vp, _vp, _vp, _vp]),
    "fse_world_download": (_i, [_vp, _vp, _vp, _vp, _vp, _vp]),
    "fse_world_generate": (_i, [_vp, _i, _u32]),
    "fse_world_set_tick": (_i, [_vp, _u32]),
    "fse_world_set_tick_zone": (_i, [_vp, _i, _i, _i, _i]),
    "fse_world_set_launch": (_i, [_vp, _i]),
    "fse_world_particle_iterations": (_i, [_vp, C.POINTER(_i)]),
    "fse_world_get_tile": (_i, [_vp, _i, _i, _vp, _vp, _vp, _vp]),
    "fse_world_set_tile": (_i, [_vp, _i, _i, C.c_uint16, _u32, C.c_int32, C.c_uint8]),
    "fse_world_tick": (_i, [_vp, _i]),
    "fse_particles_tick": (_i, [_vp]),
    "fse_world_step": (_i, [_vp, _i]),
    "fse_world_step_graph": (_i, [_vp, _i]),
    "fse_world_enqueue": (_i, [_vp, _i, _i]),
    "fse_world_sync": (_i, [_vp]),
    "fse_world_set_stream": (_i, [_vp, _vp]),
    "fse_world_stream": (_vp, [_vp]),
    "fse_particles_add": (_i, [_vp, _vp, _i]),
    "fse_particles_count": (_i, [_vp, C.POINTER(_i)]),
    "fse_particles_read": (_i, [_vp, _vp, _i, C.POINTER(_i)]),
    "fse_object_stamp": (_i, [_vp, _vp, _i]),
    "fse_object_readback": (_i, [_vp, _vp, _i, C.POINTER(_i64)]),
    "fse_object_mask_export": (_i, [_vp, _vp]),
    "fse_object_list_export": (_i, [_vp, _vp, _i64, C.POINTER(_i64)]),
    "fse_world_pass_timing": (_i, [_vp, _i, C.POINTER(_d), C.POINTER(_i64)]),
    "fse_launch_counter": (_i64, []),
    "fse_world_ledger": (_i, [_vp, _vp]),
    "fse_world_ledger_reset": (_i, [_vp]),
    "fse_world_census": (_i, [_vp, _vp]),
    "fse_world_render_dirty": (_i, [_vp, _vp]),
    "fse_world_render_cells": (_i, [_vp]),
    "fse_world_render_read": (_i, [_vp, _i, _vp]),
    "fse_world_render_texture": (_vp, [_vp, _i]),
    "fse_world_physics_check": (_i, [_vp, _i, _i, _vp, _vp, _vp, C.c_int64]),
    "fse_world_islands": (_i, [_vp, _i, _i, _vp, _i, _vp]),
    "fse_tick_noalloc": (_i, [_vp, _vp, _vp, _vp, _vp, _i, _i, _i, _i, _u32, _u32, _vp, _i, C.POINTER(_i), _vp]),
    "fse_batch_create": (_i, [_vp, _i, _pp]),
    "fse_batch_destroy": (_i, [_vp]),
    "fse_batch_step": (_i, [_vp, _i]),
    "fse_batch_enqueue": (_i, [_vp, _i]),
    "fse_batch_step_graph": (_i, [_vp, _i, _i]),
    "fse_batch_autotune": (_i, [_vp, _vp]),
    "fse_batch_set_launch": (_i, [_vp, _i, _i]),
    "fse_batch_sync": (_i, [_vp]),
    "fse_batch_stream": (_vp, [_vp]),
    "fse_batch_upload": (_i, [_vp, _i, _vp, _vp, _vp, _vp, _vp]),
    "fse_batch_download": (_i, [_vp, _i, _vp, _vp, _vp, _vp, _vp]),
    "fse_batch_io_layout": (_i, [_vp, _vp, C.POINTER(_i64)]),
    "fse_batch_upload_all": (_i, [_vp, _vp, _i64]),
    "fse_batch_download_all": (_i, [_vp, _vp, _i64]),
    "fse_batch_prepare_graphs": (_i, [_vp, _i, _i]),
    "fse_batch_timing": (_i, [_vp, _i, C.POINTER(_d), C.POINTER(_i64), _vp, _i, C.POINTER(_i)]),
    "fse_server_create": (_i, [_i64, _i, _pp]),
    "fse_server_destroy": (_i, [_vp]),
    "fse_server_add_world": (_i, [_vp, _i, _i, C.POINTER(FseConfig), _i, _u32, C.POINTER(_i)]),
    "fse_server_remove_world": (_i, [_vp, _i]),
    "fse_server_bytes_in_use": (_i64, [_vp]),
    "fse_server_world": (_vp, [_vp, _i]),
    "fse_server_submit": (_i, [_vp, _i, _i, _d, C.POINTER(_i64)]),
    "fse_server_step": (_i, [_vp, C.POINTER(_i)]),
    "fse_server_now_us": (_d, [_vp]),
    "fse_server_poll": (_i, [_vp, _d, _vp, _vp, _i, C.POINTER(_i)]),
    "fse_server_set_depth": (_i, [_vp, _i]),
    "fse_server_drain": (_i, [_vp]),
    "fse_server_stats": (_i, [_vp, _vp, _i]),
    "fse_server_tick_times": (_i, [_vp, _vp, _i, C.POINTER(_i)]),
}

_lib = None


class FseError(RuntimeError):
    def __init__(self, status, what=""):
        self.status = status
        msg = "status %d" % status
        if _lib is not None:
            msg = _lib.fse_status_string(status).decode()
        super().__init__("%s: %s" % (what, msg) if what else msg)


def load(path=None):
    """Load libfse.so; raises if the CUDA library has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or LIB_PATH
    if not os.path.exists(path):
        raise ImportError("libfse.so not built: run `python -c \"import __graft_entry__ as g; g.build()\"`")
    lib = C.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def check(status, what=""):
    if status != 0:
        raise FseError(status, what)
    return status


def ptr(a):
    return a.ctypes.data_as(C.c_void_p)
