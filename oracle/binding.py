"""ctypes binding of the C oracle (oracle/fse_oracle.c).

Test infrastructure: the checker the CUDA path is compared against.
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libfse_oracle.so")
REF_TEMPERATURE_PATH = os.path.join(HERE, "_ref", "libref_temperature.so")
REF_LZ4_PATH = os.path.join(HERE, "_ref", "liblz4ref.so")
REF_CELLS_PATH = os.path.join(HERE, "_ref", "libref_cells.so")
REF_RENDER_PATH = os.path.join(HERE, "_ref", "libref_render.so")
REF_OBJECTS_PATH = os.path.join(HERE, "_ref", "libref_objects.so")
REF_TICK_PATH = os.path.join(HERE, "_ref", "libref_tick.so")
# The reference tree that oracle/Makefile's `ref` recipes extract from: the
# FSE_REFERENCE_ROOT environment variable, else the tree's mount point in the build
# container. Where it is absent, the pieces extracted before (oracle/_ref/*.inc)
# are compiled instead, or the reference-made fixtures under tests/golden are used.
REFERENCE_ROOT = os.environ.get("FSE_REFERENCE_ROOT") or "/root/reference"
REFERENCE_WORLD_CPP = os.path.join(REFERENCE_ROOT, "source", "engine", "world.cpp")

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
assert BODY_DTYPE.itemsize == 48

ISLAND_DTYPE = np.dtype([("root", "<i4"), ("cells", "<i4"), ("min_x", "<i4"), ("min_y", "<i4"), ("max_x", "<i4"),
                         ("max_y", "<i4")])

ORDER_SEQ = 0
ORDER_PART = 1


def make_ref():
    """Run oracle/Makefile's `ref` target on REFERENCE_ROOT."""
    subprocess.run(["make", "-s", "-C", HERE, "ref", "REF=" + REFERENCE_ROOT], check=True)


def build_oracle(force=False):
    """Compile the oracle with its Makefile (gcc, no reference sources)."""
    if force or not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < max(
        os.path.getmtime(os.path.join(HERE, f)) for f in ("fse_oracle.c", "fse_oracle.h", "Makefile")
    ):
        subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB_PATH


def _ptr(a):
    return a.ctypes.data_as(C.c_void_p)


class Oracle:
    """Process-wide handle on the oracle library (its material table is global)."""

    _lib = None

    def __init__(self):
        if Oracle._lib is None:
            build_oracle()
            lib = C.CDLL(LIB_PATH)
            vp, i32, u32 = C.c_void_p, C.c_int, C.c_uint32
            sig = {
                "om_materials_reset_builtin": (None, []),
                "om_material_register": (i32, [i32, C.c_char_p, C.c_char_p, i32, i32, i32, C.c_float, i32, i32, u32, u32]),
                "om_material_set_factory": (i32, [i32, u32, i32, i32, i32, C.c_int32]),
                "om_material_set_reaction": (i32, [i32, i32, i32, i32]),
                "om_material_set_interaction": (i32, [i32, i32, i32, i32, i32, i32, i32]),
                "om_material_count": (i32, []),
                "om_material_rules": (i32, [vp, vp, i32]),
                "om_material_tile_temperature": (i32, [i32]),
                "om_material_find": (i32, [C.c_char_p]),
                "om_material_get": (None, [i32, vp]),
                "om_world_new": (vp, [i32, i32, i32, i32, u32]),
                "om_world_free": (None, [vp]),
                "om_world_set": (None, [vp, vp, vp, vp, vp, vp]),
                "om_world_get": (None, [vp, vp, vp, vp, vp, vp]),
                "om_world_generate": (None, [vp, i32, u32]),
                "om_world_set_tick": (None, [vp, u32]),
                "om_world_get_tick": (u32, [vp]),
                "om_world_tick": (C.c_long, [vp, i32, i32]),
                "om_particles_tick": (i32, [vp]),
                "om_world_step": (None, [vp, i32, i32]),
                "om_particles_count": (i32, [vp]),
                "om_particles_get": (None, [vp, vp]),
                "om_particles_set": (None, [vp, vp, i32]),
                "om_ledger_get": (None, [vp, vp]),
                "om_ledger_reset": (None, [vp]),
                "om_census": (None, [vp, vp]),
                "om_particles_kinematics_f64": (None, [vp, vp, i32, vp, vp, vp]),
                "om_particles_kinematics_f32": (None, [vp, vp, i32, vp, vp, vp]),
                "om_object_stamp": (None, [vp, vp, i32]),
                "om_object_readback": (C.c_long, [vp, vp, i32]),
                "om_object_mask": (None, [vp, vp]),
                "om_set_threads": (None, [i32]),
                "om_debug_set_lattice": (None, [i32, i32, i32]),
                "om_render_enable": (None, [vp]),
                "om_render_dirty": (None, [vp, vp]),
                "om_render_cells": (None, [vp]),
                "om_render_get": (None, [vp, i32, vp]),
                "om_render_dirty_get": (None, [vp, vp]),
                "om_render_set": (None, [vp, vp, vp, vp]),
                "om_render_pflow_get": (None, [vp, vp]),
                "om_physics_check": (i32, [vp, i32, i32, vp, vp, i32]),
                "om_islands": (i32, [vp, i32, i32, vp, i32]),
                "om_material_set_conduction": (i32, [i32, u32, C.c_float, C.c_float]),
                "om_material_set_factory_temperature": (i32, [i32, C.c_int32]),
                "om_tick_temperature": (None, [vp]),
                "om_world_set_temperature": (None, [vp, i32]),
                "om_world_set_f32": (None, [vp, i32]),
                "om_world_set_tick_zone": (i32, [vp, i32, i32, i32, i32]),
                "om_temperature_get": (None, [vp, vp]),
                "om_temperature_set": (None, [vp, vp]),
                "om_lz4_bound": (i32, [i32]),
                "om_lz4_encode": (i32, [vp, i32, vp, i32]),
                "om_lz4_decode": (i32, [vp, i32, vp, i32]),
                "om_world_pack": (i32, [vp, i32, vp, C.c_int64, vp]),
                "om_world_unpack": (i32, [vp, vp, vp, i32, vp]),
            }
            for name, (res, args) in sig.items():
                f = getattr(lib, name)
                f.restype = res
                f.argtypes = args
            Oracle._lib = lib
        self.lib = Oracle._lib

    def reset_materials(self):
        self.lib.om_materials_reset_builtin()

    def material_count(self):
        return self.lib.om_material_count()

    def find(self, index_name):
        return self.lib.om_material_find(index_name.encode())

    def rules(self):
        """(reactions (n, 4, 3), interactions (m, 7)) of the material table."""
        n = self.material_count()
        react = np.zeros((n, 4, 3), np.int32)
        inter = np.zeros((4096, 7), np.int32)
        m = self.lib.om_material_rules(_ptr(react), _ptr(inter), 4096)
        return react, inter[:m].copy()

    def material(self, mid):
        out = np.zeros(16, np.int32)
        self.lib.om_material_get(mid, _ptr(out))
        return out

    def register(self, s_id, name, index_name, physics_type, slipperyness, alpha, density, iterations, emit=0,
                 emit_colour=0, colour=0xFFFFFFFF):
        return self.lib.om_material_register(s_id, name.encode(), index_name.encode(), physics_type, slipperyness,
                                             alpha, density, iterations, emit, emit_colour, colour)

    def set_reaction(self, mat, kind, temperature, result):
        return self.lib.om_material_set_reaction(mat, kind, temperature, result)

    def set_interaction(self, mat, other, kind, data1, data2, ofs_x, ofs_y):
        return self.lib.om_material_set_interaction(mat, other, kind, data1, data2, ofs_x, ofs_y)

    def set_factory(self, mat, base, shift, lo, mod, scalar):
        return self.lib.om_material_set_factory(mat, base, shift, lo, mod, scalar)

    def set_conduction(self, mat, add_temp, cond_self, cond_other):
        return self.lib.om_material_set_conduction(mat, add_temp, cond_self, cond_other)

    def set_factory_temperature(self, mat, temperature):
        return self.lib.om_material_set_factory_temperature(mat, temperature)

    def set_threads(self, n):
        self.lib.om_set_threads(n)

    def debug_set_lattice(self, sweep, px, py):
        self.lib.om_debug_set_lattice(sweep, px, py)


class OracleWorld:
    """One oracle world (SoA planes + particle list)."""

    def __init__(self, w, h, chunk=128, cell_iter=3, seed=1234):
        self.o = Oracle()
        self.lib = self.o.lib
        self.w, self.h = w, h
        self.h_ = self.lib.om_world_new(w, h, chunk, cell_iter, seed)
        if not self.h_:
            raise ValueError("bad world parameters")

    def __del__(self):
        try:
            if self.h_:
                self.lib.om_world_free(self.h_)
                self.h_ = None
        except Exception:
            pass

    def generate(self, kind, seed):
        self.lib.om_world_generate(self.h_, kind, seed)

    def set_state(self, planes):
        n = self.w * self.h
        arrs = [np.ascontiguousarray(planes[k], dt).reshape(n) for k, dt in
                (("id", np.uint16), ("colour", np.uint32), ("scalar", np.int32), ("flags", np.uint8),
                 ("diff", np.int32))]
        self.lib.om_world_set(self.h_, *[_ptr(a) for a in arrs])

    def state(self):
        n = self.w * self.h
        out = {"id": np.empty(n, np.uint16), "colour": np.empty(n, np.uint32), "scalar": np.empty(n, np.int32),
               "flags": np.empty(n, np.uint8), "diff": np.empty(n, np.int32)}
        self.lib.om_world_get(self.h_, *[_ptr(out[k]) for k in ("id", "colour", "scalar", "flags", "diff")])
        return {k: v.reshape(self.h, self.w) for k, v in out.items()}

    @property
    def tick_count(self):
        return self.lib.om_world_get_tick(self.h_)

    @tick_count.setter
    def tick_count(self, t):
        self.lib.om_world_set_tick(self.h_, t)

    def tick(self, order=ORDER_PART, check_races=False):
        return self.lib.om_world_tick(self.h_, order, 1 if check_races else 0)

    def particles_tick(self):
        return self.lib.om_particles_tick(self.h_)

    def step(self, n=1, order=ORDER_PART):
        self.lib.om_world_step(self.h_, order, n)

    def particles(self):
        n = self.lib.om_particles_count(self.h_)
        out = np.zeros(n, PARTICLE_DTYPE)
        if n:
            self.lib.om_particles_get(self.h_, _ptr(out))
        return out

    def set_particles(self, parts):
        parts = np.ascontiguousarray(parts, PARTICLE_DTYPE)
        self.lib.om_particles_set(self.h_, _ptr(parts), len(parts))

    def ledger(self):
        m = self.o.material_count()
        out = np.zeros(6 * m, np.int64)
        self.lib.om_ledger_get(self.h_, _ptr(out))
        return out.reshape(6, m)

    def reset_ledger(self):
        self.lib.om_ledger_reset(self.h_)

    def census(self):
        m = self.o.material_count()
        out = np.zeros(4 * m, np.int64)
        self.lib.om_census(self.h_, _ptr(out))
        return out.reshape(4, m)

    def kinematics(self, parts, f64=True):
        parts = np.ascontiguousarray(parts, PARTICLE_DTYPE)
        n = len(parts)
        out = np.zeros(4 * n, np.float64 if f64 else np.float32)
        ev = np.zeros(n, np.int32)
        sub = np.zeros(n, np.int32)
        fn = self.lib.om_particles_kinematics_f64 if f64 else self.lib.om_particles_kinematics_f32
        fn(self.h_, _ptr(parts), n, _ptr(out), _ptr(ev), _ptr(sub))
        return out.reshape(n, 4), ev, sub

    def object_stamp(self, bodies):
        self.lib.om_object_stamp(self.h_, _ptr(bodies), len(bodies))

    def object_readback(self, bodies):
        return self.lib.om_object_readback(self.h_, _ptr(bodies), len(bodies))

    def object_mask(self):
        n = self.w * self.h
        out = np.zeros((n + 7) // 8, np.uint8)
        self.lib.om_object_mask(self.h_, _ptr(out))
        return out

    # -- chunk .pack codec
    def pack(self, phase=0):
        """All chunks row-major in the reference's .pack layout: (bytes, offsets)."""
        n = ((self.w + 127) // 128) * ((self.h + 127) // 128)
        cap = n * (17 + 2 * (393216 + 393216 // 255 + 16)) + 16
        out = np.zeros(cap, np.uint8)
        offs = np.zeros(n + 1, np.int64)
        rc = self.lib.om_world_pack(self.h_, phase, _ptr(out), cap, _ptr(offs))
        if rc < 0:
            raise ValueError("pack failed")
        return out[: offs[-1]].copy(), offs

    def unpack(self, data, offsets):
        data = np.ascontiguousarray(data, np.uint8)
        offsets = np.ascontiguousarray(offsets, np.int64)
        phases = np.zeros(len(offsets) - 1, np.int8)
        rc = self.lib.om_world_unpack(self.h_, _ptr(data), _ptr(offsets), len(offsets) - 1, _ptr(phases))
        return rc, phases

    # -- temperature
    def temperature(self):
        out = np.zeros(self.w * self.h, np.int16)
        self.lib.om_temperature_get(self.h_, _ptr(out))
        return out.reshape(self.h, self.w)

    def set_temperature(self, temps):
        a = np.ascontiguousarray(temps, np.int16).reshape(self.w * self.h)
        self.lib.om_temperature_set(self.h_, _ptr(a))

    def tick_temperature(self):
        self.lib.om_tick_temperature(self.h_)

    def enable_temperature(self, on=True):
        self.lib.om_world_set_temperature(self.h_, 1 if on else 0)

    def set_tick_zone(self, x, y, w, h):
        """world::tickZone (the whole world by default)."""
        assert self.lib.om_world_set_tick_zone(self.h_, x, y, w, h) == 0

    def set_f32(self, on=True):
        """f32 liquid amounts (the library's FSE_CFG_F32_FLUID); before generate / set_state."""
        self.lib.om_world_set_f32(self.h_, 1 if on else 0)

    # -- render textures
    def render_enable(self):
        self.lib.om_render_enable(self.h_)

    def render_dirty(self):
        moving = np.zeros(256, np.int64)
        self.lib.om_render_dirty(self.h_, _ptr(moving))
        return moving[: self.o.material_count()]

    def render_cells(self):
        self.lib.om_render_cells(self.h_)

    def render_texture(self, which):
        out = np.zeros((self.h, self.w, 4), np.uint8)
        self.lib.om_render_get(self.h_, which, _ptr(out))
        return out

    def render_set(self, dirty, flow, pflow):
        d = np.ascontiguousarray(dirty, np.uint8)
        f = np.ascontiguousarray(flow, np.int32)
        p = np.ascontiguousarray(pflow, np.float32)
        self.lib.om_render_set(self.h_, _ptr(d), _ptr(f), _ptr(p))

    def render_pflow(self):
        out = np.zeros((self.h, self.w, 2), np.float32)
        self.lib.om_render_pflow_get(self.h_, _ptr(out))
        return out

    def render_dirty_plane(self):
        out = np.zeros((self.h, self.w), np.uint8)
        self.lib.om_render_dirty_get(self.h_, _ptr(out))
        return out

    # -- solid islands
    def physics_check(self, x, y, pixels_cap=1 << 20):
        bbox = np.zeros(4, np.int32)
        pix = np.zeros(pixels_cap, np.uint32)
        n = self.lib.om_physics_check(self.h_, x, y, _ptr(bbox), _ptr(pix), pixels_cap)
        if n == 0:
            return 0, None, None
        bw, bh = bbox[2] - bbox[0] + 1, bbox[3] - bbox[1] + 1
        img = pix[: bw * bh].reshape(bh, bw).copy() if n > 10 else None
        return n, bbox, img

    def islands(self, max_cells=1000, remove=False, cap=1 << 16):
        out = np.zeros(cap, ISLAND_DTYPE)
        n = self.lib.om_islands(self.h_, max_cells, 1 if remove else 0, _ptr(out), cap)
        return out[: min(n, cap)], n


def _build_from_inc(so_path, cpp, incs, std):
    """Without the reference tree: compile a harness from the pieces oracle/Makefile
    extracted before into oracle/_ref (they travel with the repository); None when
    they are absent."""
    paths = [os.path.join(HERE, "_ref", i) for i in incs]
    if not all(os.path.exists(p) and os.path.getsize(p) > 0 for p in paths):
        return None
    if not os.path.exists(so_path) or os.path.getmtime(so_path) < os.path.getmtime(os.path.join(HERE, cpp)):
        subprocess.run([os.environ.get("CXX", "g++"), "-O2", "-std=" + std, "-fPIC", "-ffp-contract=off", "-shared",
                        "-I" + os.path.join(HERE, "_ref"), "-o", so_path, os.path.join(HERE, cpp)], check=True)
    return so_path


def build_reference_temperature(force=False):
    """Compile the reference's own world::tickTemperature (oracle/Makefile `ref`), or
    from its extracted pieces without the tree; None when neither is present."""
    if not os.path.exists(REFERENCE_WORLD_CPP):
        return _build_from_inc(REF_TEMPERATURE_PATH, "ref_temperature.cpp", ["tick_temperature.inc"], "c++17")
    if force or not os.path.exists(REF_TEMPERATURE_PATH) or os.path.getmtime(REF_TEMPERATURE_PATH) < max(
        os.path.getmtime(os.path.join(HERE, f)) for f in ("ref_temperature.cpp", "Makefile")
    ):
        make_ref()
    return REF_TEMPERATURE_PATH


def reference_tick_temperature(lib_path, mat, temp, add_temp, cond_self, cond_other, zone):
    """One world::tickTemperature of the compiled reference over (mat, temp) arrays."""
    lib = C.CDLL(lib_path)
    f = lib.ref_tick_temperature
    f.restype = C.c_int
    f.argtypes = [C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p,
                  C.c_int, C.c_int, C.c_int, C.c_int]
    h, w = mat.shape
    m = np.ascontiguousarray(mat, np.uint16)
    t = np.ascontiguousarray(temp, np.int16).copy()
    a = np.ascontiguousarray(add_temp, np.uint32)
    cs = np.ascontiguousarray(cond_self, np.float32)
    co = np.ascontiguousarray(cond_other, np.float32)
    rc = f(w, h, _ptr(m), _ptr(t), len(a), _ptr(a), _ptr(cs), _ptr(co), *zone)
    if rc != 0:
        raise ValueError("ref_tick_temperature failed")
    return t


def lz4_encode(buf):
    """The oracle's LZ4 block encoder (16 fixed match distances, greedy)."""
    o = Oracle()
    buf = np.ascontiguousarray(buf, np.uint8)
    cap = o.lib.om_lz4_bound(len(buf))
    dst = np.zeros(cap, np.uint8)
    m = o.lib.om_lz4_encode(_ptr(buf), len(buf), _ptr(dst), cap)
    if m < 0:
        raise ValueError("encode failed")
    return dst[:m].copy()


def lz4_decode(src, cap):
    """The oracle's LZ4 block decoder: (decoded bytes, status = size or negative)."""
    o = Oracle()
    src = np.ascontiguousarray(src, np.uint8)
    dst = np.zeros(max(cap, 1), np.uint8)
    m = o.lib.om_lz4_decode(_ptr(src), len(src), _ptr(dst), cap)
    return dst[: max(m, 0)].copy(), m


def build_reference_lz4(force=False):
    """Compile the reference's vendored LZ4 (oracle/Makefile `ref`), or its copy in
    oracle/_ref without the tree; None when neither is present."""
    if not os.path.exists(REFERENCE_WORLD_CPP):
        src = os.path.join(HERE, "_ref", "lz4.c")
        if not os.path.exists(src):
            return None
        if not os.path.exists(REF_LZ4_PATH):
            subprocess.run([os.environ.get("CC", "gcc"), "-O2", "-fPIC", "-shared", "-I" + os.path.join(HERE, "_ref"),
                            "-o", REF_LZ4_PATH, src], check=True)
        return REF_LZ4_PATH
    if force or not os.path.exists(REF_LZ4_PATH):
        make_ref()
    return REF_LZ4_PATH


class ReferenceLZ4:
    """LZ4_compress_fast / LZ4_decompress_safe of the reference's vendored LZ4 1.9.4."""

    def __init__(self, path):
        lib = C.CDLL(path)
        lib.LZ4_compress_fast.restype = C.c_int
        lib.LZ4_compress_fast.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int]
        lib.LZ4_decompress_safe.restype = C.c_int
        lib.LZ4_decompress_safe.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int]
        lib.LZ4_compressBound.restype = C.c_int
        lib.LZ4_compressBound.argtypes = [C.c_int]
        self.lib = lib

    def compress(self, data, acceleration=10):
        data = np.ascontiguousarray(data, np.uint8)
        cap = self.lib.LZ4_compressBound(len(data))
        dst = np.zeros(cap, np.uint8)
        m = self.lib.LZ4_compress_fast(_ptr(data), _ptr(dst), len(data), cap, acceleration)
        if m <= 0:
            raise ValueError("LZ4_compress_fast failed")
        return dst[:m].copy()

    def decompress(self, src, size):
        src = np.ascontiguousarray(src, np.uint8)
        dst = np.zeros(max(size, 1), np.uint8)
        m = self.lib.LZ4_decompress_safe(_ptr(src), _ptr(dst), len(src), size)
        return dst[: max(m, 0)].copy(), m


def build_reference_cells(force=False):
    """Compile the reference's own world::tickCells (oracle/Makefile `ref`); None without the tree."""
    if not os.path.exists(REFERENCE_WORLD_CPP):
        return None
    if force or not os.path.exists(REF_CELLS_PATH) or os.path.getmtime(REF_CELLS_PATH) < os.path.getmtime(
            os.path.join(HERE, "ref_particles.cpp")):
        make_ref()
    return REF_CELLS_PATH


def reference_tick_cells(lib_path, ids, colours, amounts, mat_types, parts, zone=None):
    """One world::tickCells of the compiled reference: (ids, colours, amounts, dirty,
    survivors); zone: world::tickZone (x, y, w, h), None for the whole world."""
    lib = C.CDLL(lib_path)
    f = lib.ref_tick_cells_zone
    f.restype = C.c_int
    f.argtypes = [C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int,
                  C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]
    z = None if zone is None else np.ascontiguousarray(zone, np.int32)
    h, w = ids.shape
    i2 = np.ascontiguousarray(ids, np.uint16).copy()
    c2 = np.ascontiguousarray(colours, np.uint32).copy()
    a2 = np.ascontiguousarray(amounts, np.int32).copy()
    d2 = np.zeros((h, w), np.uint8)
    mt = np.ascontiguousarray(mat_types, np.int32)
    pin = np.ascontiguousarray(parts, PARTICLE_DTYPE)
    pout = np.zeros(max(len(pin), 1), PARTICLE_DTYPE)
    nout = C.c_int(0)
    rc = f(w, h, _ptr(i2), _ptr(c2), _ptr(a2), _ptr(d2), _ptr(mt), len(mt), _ptr(pin), len(pin), _ptr(pout),
           C.byref(nout), None if z is None else _ptr(z))
    if rc != 0:
        raise ValueError("ref_tick_cells failed")
    return i2, c2, a2, d2, pout[: nout.value].copy()


TICK_INC = ("world_tick", "world_gettile", "world_settile", "vertical_flow", "fluid_consts", "interact_defs",
            "material_interaction", "material_struct", "material_ctor", "material_instance", "material_instance_ctor",
            "tiles_globals", "cell_data", "cells")


def build_reference_tick(force=False):
    """Compile the reference's own world::tick and world::tickCells (oracle/Makefile
    `ref`). Without the reference tree, the pieces oracle/Makefile extracted before
    (oracle/_ref/*.inc) are compiled where they are present; else None."""
    fresh = (not force and os.path.exists(REF_TICK_PATH) and
             os.path.getmtime(REF_TICK_PATH) >= os.path.getmtime(os.path.join(HERE, "ref_tick.cpp")))
    if fresh:
        return REF_TICK_PATH
    if os.path.exists(REFERENCE_WORLD_CPP):
        make_ref()
        return REF_TICK_PATH
    incs = [os.path.join(HERE, "_ref", "tick_%s.inc" % k) for k in TICK_INC]
    if not all(os.path.exists(p) and os.path.getsize(p) > 0 for p in incs):
        return None
    subprocess.run([os.environ.get("CXX", "g++"), "-O2", "-std=c++20", "-fPIC", "-ffp-contract=off", "-Wno-narrowing",
                    "-pthread", "-shared", "-I" + os.path.join(HERE, "_ref"), "-o", REF_TICK_PATH,
                    os.path.join(HERE, "ref_tick.cpp")], check=True)
    return REF_TICK_PATH


def _reference_tables(oracle):
    """The oracle's material table in the reference harness's layout."""
    n = oracle.material_count()
    mats = np.zeros((n, 10), np.int32)
    for i in range(n):
        m = oracle.material(i)
        mats[i, :9] = [m[0], m[1], m[2], m[3], m[9], m[10], m[11], m[12], oracle.lib.om_material_tile_temperature(i)]
    special = np.array([oracle.find(s) for s in SPECIAL_MATERIALS], np.int32)
    react, inter = oracle.rules()
    return n, mats, special, np.ascontiguousarray(react), np.ascontiguousarray(inter)


def reference_world_bench(lib_path, oracle, ids, colours, temps, parts, cell_iter, seed, threads, warm, steps,
                          budget_s):
    """Times the reference's own world::tick() + world::tickCells() on the grid and
    particles (PARTICLE_DTYPE) with `threads` pool workers: (seconds, steps timed)."""
    lib = C.CDLL(lib_path)
    f = lib.ref_world_bench
    f.restype = C.c_double
    f.argtypes = [C.c_int, C.c_int, C.c_int, C.c_uint32, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int,
                  C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_int, C.c_int,
                  C.c_int, C.c_double, C.c_void_p]
    n, mats, special, react, inter = _reference_tables(oracle)
    h, w = ids.shape
    pf = np.ascontiguousarray(np.stack([parts[k] for k in ("x", "y", "vx", "vy", "ax", "ay")], 1), np.float32)
    pi = np.ascontiguousarray(np.stack([parts["id"].astype(np.uint32), parts["colour"]], 1), np.uint32)
    done = C.c_int(0)
    secs = f(w, h, cell_iter, seed & 0xFFFFFFFF, n, _ptr(mats), _ptr(special), _ptr(react), len(inter), _ptr(inter),
             _ptr(np.ascontiguousarray(ids, np.uint16)), _ptr(np.ascontiguousarray(colours, np.uint32)),
             _ptr(np.ascontiguousarray(temps, np.int32)), len(parts), _ptr(pf), _ptr(pi), threads, warm, steps,
             float(budget_s), C.byref(done))
    if secs < 0:
        raise ValueError("the reference tick wrote outside the grid")
    return secs, done.value


SPECIAL_MATERIALS = ("GENERIC_AIR", "GENERIC_SOLID", "FIRE", "WATER", "LAVA", "STEAM", "OBSIDIAN")


def reference_world_tick(lib_path, oracle, ids, colours, temps, moved, cell_iter, seed, tick, n_ticks=1):
    """n_ticks world::tick() calls of the compiled reference on a grid of non-liquid
    tiles (ids, colours, temperatures, moved flags), with the oracle's material table
    and the oracle's draws. Returns (ids, colours, temperatures, moved, particles as
    (n, 16) int32 rows: id, colour, temperature, x, y, vx, vy, ax, ay, target x, y,
    force (float bits), phase, temporary, lifetime, fade time; draws made)."""
    lib = C.CDLL(lib_path)
    f = lib.ref_world_tick
    f.restype = C.c_int
    f.argtypes = [C.c_int, C.c_int, C.c_int, C.c_uint32, C.c_uint32, C.c_int, C.c_int, C.c_void_p, C.c_void_p,
                  C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                  C.c_int, C.c_void_p]
    n, mats, special, react, inter = _reference_tables(oracle)
    h, w = ids.shape
    i2 = np.ascontiguousarray(ids, np.uint16).copy()
    c2 = np.ascontiguousarray(colours, np.uint32).copy()
    t2 = np.ascontiguousarray(temps, np.int32).copy()
    m2 = np.ascontiguousarray(moved, np.uint8).copy()
    cap = 1 << 16
    parts = np.zeros((cap, 16), np.int32)
    draws = C.c_longlong(0)
    np_ = f(w, h, cell_iter, seed & 0xFFFFFFFF, tick & 0xFFFFFFFF, n_ticks, n, _ptr(mats), _ptr(special),
            _ptr(np.ascontiguousarray(react)), len(inter), _ptr(np.ascontiguousarray(inter)), _ptr(i2), _ptr(c2),
            _ptr(t2), _ptr(m2), _ptr(parts), cap, C.byref(draws))
    if np_ < 0:
        raise ValueError("the reference tick wrote outside the grid: the scene needs its solid border")
    return i2, c2, t2, m2, parts[: min(np_, cap)].copy(), draws.value


def reference_world_tick_fluid(lib_path, oracle, ids, colours, temps, moved, amounts, diffs, settle, cell_iter, seed,
                               tick, n_ticks=1, zone=None):
    """reference_world_tick with every cell's fluidAmount, fluidAmountDiff (f32) and
    settleCount given and returned; particle rows have 17 ints, the last the carried
    tile's fluidAmount bits; zone: world::tickZone (x, y, w, h), None for the whole
    world."""
    lib = C.CDLL(lib_path)
    f = lib.ref_world_tick_fluid
    f.restype = C.c_int
    f.argtypes = [C.c_int, C.c_int, C.c_int, C.c_uint32, C.c_uint32, C.c_int, C.c_int, C.c_void_p, C.c_void_p,
                  C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                  C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p]
    n, mats, special, react, inter = _reference_tables(oracle)
    h, w = ids.shape
    z = None if zone is None else np.ascontiguousarray(zone, np.int32)
    i2 = np.ascontiguousarray(ids, np.uint16).copy()
    c2 = np.ascontiguousarray(colours, np.uint32).copy()
    t2 = np.ascontiguousarray(temps, np.int32).copy()
    m2 = np.ascontiguousarray(moved, np.uint8).copy()
    a2 = np.ascontiguousarray(amounts, np.float32).copy()
    d2 = np.ascontiguousarray(diffs, np.float32).copy()
    s2 = np.ascontiguousarray(settle, np.uint8).copy()
    cap = 1 << 16
    parts = np.zeros((cap, 17), np.int32)
    draws = C.c_longlong(0)
    np_ = f(w, h, cell_iter, seed & 0xFFFFFFFF, tick & 0xFFFFFFFF, n_ticks, n, _ptr(mats), _ptr(special),
            _ptr(np.ascontiguousarray(react)), len(inter), _ptr(np.ascontiguousarray(inter)), _ptr(i2), _ptr(c2),
            _ptr(t2), _ptr(m2), _ptr(a2), _ptr(d2), _ptr(s2), _ptr(parts), cap, C.byref(draws),
            None if z is None else _ptr(z))
    if np_ < 0:
        raise ValueError("the reference tick wrote outside the grid: the scene needs its solid border")
    return i2, c2, t2, m2, a2, d2, s2, parts[: min(np_, cap)].copy(), draws.value


def build_reference_render(force=False):
    """Compile the reference's own dirty-pixel loop of game::tick (oracle/Makefile `ref`),
    or from its extracted piece without the tree; None when neither is present."""
    if not os.path.exists(REFERENCE_WORLD_CPP):
        return _build_from_inc(REF_RENDER_PATH, "ref_render.cpp", ["dirty_loop.inc"], "c++20")
    if force or not os.path.exists(REF_RENDER_PATH) or os.path.getmtime(REF_RENDER_PATH) < os.path.getmtime(
            os.path.join(HERE, "ref_render.cpp")):
        make_ref()
    return REF_RENDER_PATH


def reference_render_dirty(lib_path, ids, colours, dirty, flow_x, flow_y, prev_x, prev_y, mats, fire_id):
    """One pass of the reference's dirty-pixel loop: textures (pixels, fire, emission, flow
    as (H, W, 4) bytes), the updated flows and smoothed flows, the u16 moving counts."""
    lib = C.CDLL(lib_path)
    f = lib.ref_render_dirty
    f.restype = C.c_int
    f.argtypes = [C.c_int] * 2 + [C.c_void_p] * 7 + [C.c_int] + [C.c_void_p] * 4 + [C.c_int] + [C.c_void_p] * 5
    h, w = ids.shape
    arrs = [np.ascontiguousarray(a, dt).copy() for a, dt in
            ((ids, np.uint16), (colours, np.uint32), (dirty, np.uint8), (flow_x, np.float32), (flow_y, np.float32),
             (prev_x, np.float32), (prev_y, np.float32))]
    types, alpha, emit, iters = [np.ascontiguousarray(a, dt) for a, dt in
                                 zip(mats, (np.int32, np.uint8, np.uint32, np.int32))]
    tex = [np.zeros((h, w, 4), np.uint8) for _ in range(4)]
    moving = np.zeros(len(types), np.uint16)
    rc = f(w, h, *[_ptr(a) for a in arrs], len(types), _ptr(types), _ptr(alpha), _ptr(emit), _ptr(iters), fire_id,
           *[_ptr(t) for t in tex], _ptr(moving))
    if rc != 0:
        raise ValueError("ref_render_dirty failed")
    return tex, arrs[3], arrs[4], arrs[5], arrs[6], moving


REF_PHYSICS_PATH = os.path.join(HERE, "_ref", "libref_physics.so")


def build_reference_physics(force=False):
    """Compile the reference's own world::physicsCheck (oracle/Makefile `ref`), or from
    its extracted pieces without the tree; None when neither is present."""
    if not os.path.exists(REFERENCE_WORLD_CPP):
        return _build_from_inc(REF_PHYSICS_PATH, "ref_physics.cpp",
                               ["physics_check.inc", "physics_flood.inc", "physics_gettile.inc"], "c++20")
    if force or not os.path.exists(REF_PHYSICS_PATH) or os.path.getmtime(REF_PHYSICS_PATH) < os.path.getmtime(
            os.path.join(HERE, "ref_physics.cpp")):
        make_ref()
    return REF_PHYSICS_PATH


def reference_physics_check(lib_path, types, colours, x, y):
    """One physicsCheck(x, y) of the compiled reference on a grid of physics types and
    colours: (types after, image or None, (origin x, origin y) or None)."""
    lib = C.CDLL(lib_path)
    f = lib.ref_physics_check
    f.restype = C.c_long
    f.argtypes = [C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_long] + [C.c_void_p] * 4
    h, w = types.shape
    t = np.ascontiguousarray(types, np.uint8).copy()
    c = np.ascontiguousarray(colours, np.uint32)
    img = np.zeros(1 << 20, np.uint32)
    o = [C.c_int(0) for _ in range(4)]
    n = f(w, h, _ptr(t), _ptr(c), x, y, _ptr(img), img.size, *[C.byref(v) for v in o])
    if n == 0:
        return t, None, None
    return t, img[:n].reshape(o[3].value, o[2].value).copy(), (o[0].value, o[1].value)


def build_reference_objects(force=False):
    """Compile the reference's own rigid-body stamp/readback loops (oracle/Makefile `ref`)."""
    if not os.path.exists(REFERENCE_WORLD_CPP):
        return None
    if force or not os.path.exists(REF_OBJECTS_PATH) or os.path.getmtime(REF_OBJECTS_PATH) < os.path.getmtime(
            os.path.join(HERE, "ref_objects.cpp")):
        make_ref()
    return REF_OBJECTS_PATH


def _ref_bodies(bodies):
    bf = np.ascontiguousarray(np.stack([bodies["x"], bodies["y"], bodies["sin_a"], bodies["cos_a"]], 1), np.float32)
    bi = np.ascontiguousarray(np.stack([bodies["w"], bodies["h"], bodies["id"].astype(np.int32),
                                        bodies["colour"].view(np.int32)], 1), np.int32)
    return bf, bi


def reference_object_stamp(lib_path, ids, colours, types, alpha, air_id, bodies):
    """The reference's stamp loop over bodies in order: (ids, colours, particles as
    (id, colour, x, y) rows, per-body [sand, liquid] displacements)."""
    lib = C.CDLL(lib_path)
    f = lib.ref_object_stamp
    f.restype = C.c_int
    f.argtypes = [C.c_int] * 2 + [C.c_void_p] * 5 + [C.c_int] * 2 + [C.c_void_p] * 2 + [C.c_int] + \
        [C.c_void_p] * 2 + [C.c_int, C.c_void_p]
    h, w = ids.shape
    i2 = np.ascontiguousarray(ids, np.uint16).copy()
    c2 = np.ascontiguousarray(colours, np.uint32).copy()
    d2 = np.zeros((h, w), np.uint8)
    t = np.ascontiguousarray(types, np.int32)
    a = np.ascontiguousarray(alpha, np.uint8)
    bf, bi = _ref_bodies(bodies)
    counts = np.zeros((len(bodies), 2), np.int32)
    cap = int(bodies["w"].astype(np.int64) @ bodies["h"].astype(np.int64)) + 1
    parts = np.zeros((cap, 4), np.float32)
    n = C.c_int(0)
    rc = f(w, h, _ptr(i2), _ptr(c2), _ptr(d2), _ptr(t), _ptr(a), len(t), air_id, _ptr(bf), _ptr(bi), len(bodies),
           _ptr(counts), _ptr(parts), cap, C.byref(n))
    if rc != 0:
        raise ValueError("ref_object_stamp failed")
    return i2, c2, parts[: n.value].copy(), counts


def reference_object_readback(lib_path, ids, colours, types, alpha, air_id, bodies):
    """The reference's readback loop: (ids, colours, per-body [recovered, lost])."""
    lib = C.CDLL(lib_path)
    f = lib.ref_object_readback
    f.restype = C.c_int
    f.argtypes = [C.c_int] * 2 + [C.c_void_p] * 5 + [C.c_int] * 2 + [C.c_void_p] * 2 + [C.c_int] + [C.c_void_p] * 2
    h, w = ids.shape
    i2 = np.ascontiguousarray(ids, np.uint16).copy()
    c2 = np.ascontiguousarray(colours, np.uint32).copy()
    d2 = np.zeros((h, w), np.uint8)
    t = np.ascontiguousarray(types, np.int32)
    a = np.ascontiguousarray(alpha, np.uint8)
    bf, bi = _ref_bodies(bodies)
    counts = np.zeros((len(bodies), 2), np.int32)
    pix = np.zeros((h, w, 4), np.uint8)
    rc = f(w, h, _ptr(i2), _ptr(c2), _ptr(d2), _ptr(t), _ptr(a), len(t), air_id, _ptr(bf), _ptr(bi), len(bodies),
           _ptr(counts), _ptr(pix))
    if rc != 0:
        raise ValueError("ref_object_readback failed")
    return i2, c2, counts
