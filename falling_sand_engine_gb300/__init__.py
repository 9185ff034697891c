"""GB300-native falling-sand world tick.

Python host mirror of the reference engine's world-update interface, over the C ABI
of libfse.so (include/fse.h): ``World.tick()`` is ``world::tick()``
(source/engine/world.cpp:1036), ``World.tickCells()`` is ``world::tickCells()``
(world.cpp:2030), ``getTile``/``setTile`` follow world.cpp:999-1008, and the material
functions follow InitMaterials/RegisterMaterial/PushMaterials
(source/engine/game_datastruct.cpp:117-300). All compute runs in the CUDA library;
there is no CPU fallback: without the library or a GPU the calls raise.
"""
import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _abi
from ._abi import BODY_DTYPE, PARTICLE_DTYPE, TILE_DTYPE, FseConfig, FseError, FseTileLayout, check, ptr

__all__ = [
    "World", "Batch", "Server", "MaterialInstance", "FseError", "PARTICLE_DTYPE", "BODY_DTYPE", "TILE_DTYPE",
    "InitMaterials", "RegisterMaterial", "PushMaterials", "load_lua_materials", "material_find",
    "material_count", "material_get", "set_reaction", "set_interaction", "lib",
    "AIR", "SOLID", "SAND", "SOUP", "GAS", "PASSABLE", "OBJECT", "GEN_EMPTY", "GEN_MIX", "GEN_ZIPF8",
    "FLUID_ONE", "CFG_RENDER", "CFG_TEMPERATURE", "CFG_TEMPERATURE_STEP", "CFG_REFERENCE_ORDER", "set_conduction", "set_factory_temperature", "get_conduction",
    "TEX_PIXELS", "TEX_EMISSION", "TEX_FIRE", "TEX_FLOW", "TEX_CELLS", "write_png",
]

AIR, SOLID, SAND, SOUP, GAS, PASSABLE, OBJECT = 0, 1, 2, 3, 4, 5, 5
GEN_EMPTY, GEN_MIX, GEN_ZIPF8 = 0, 1, 2
FLUID_ONE = 65536
INTERACT_TRANSFORM_MATERIAL, INTERACT_SPAWN_MATERIAL = 1, 2
REACT_TEMPERATURE_BELOW, REACT_TEMPERATURE_ABOVE = 4, 5


def lib():
    return _abi.load()


@dataclass
class MaterialInstance:
    """One cell (MaterialInstance, source/engine/game_datastruct.hpp:207-225) in the
    SoA layout: scalar = fluid amount (Q16.16) for SOUP materials, temperature otherwise;
    flags bit 7 = moved, bits 0-5 = settle count."""

    id: int
    colour: int = 0
    scalar: int = 0
    flags: int = 0


# ------------------------------------------------------------------ materials
def InitMaterials():
    check(lib().fse_materials_begin(), "materials_begin")


def RegisterMaterial(s_id, name, index_name, physicsType, slipperyness, alpha, density, iterations, emit=0,
                     emitColor=0, color=0xFFFFFFFF):
    out = C.c_int(-1)
    check(lib().fse_material_register(s_id, name.encode(), index_name.encode(), physicsType, slipperyness, alpha,
                                      float(density), iterations, emit, emitColor & 0xFFFFFFFF,
                                      color & 0xFFFFFFFF, C.byref(out)), "RegisterMaterial")
    return out.value


def PushMaterials():
    check(lib().fse_materials_push(), "PushMaterials")


def load_lua_materials(script):
    n = C.c_int(0)
    check(lib().fse_materials_load_lua(script.encode(), C.byref(n)), "materials_load_lua")
    return n.value


def launch_counter():
    """Number of CUDA kernels the library has launched in this process."""
    return lib().fse_launch_counter()


def material_find(index_name):
    return lib().fse_material_find(index_name.encode())


def material_count():
    return lib().fse_material_count()


def material_get(mid):
    out = np.zeros(16, np.int32)
    check(lib().fse_material_get(mid, ptr(out)), "material_get")
    return out


def set_reaction(mat, kind, temperature, result):
    check(lib().fse_material_set_reaction(mat, kind, temperature, result), "set_reaction")


def set_interaction(mat, other, kind, data1, data2, ofs_x, ofs_y):
    check(lib().fse_material_set_interaction(mat, other, kind, data1, data2, ofs_x, ofs_y), "set_interaction")


def set_conduction(mat, add_temp, conduction_self, conduction_other):
    """Material::addTemp / conductionSelf / conductionOther (game_datastruct.hpp:142-144)."""
    check(lib().fse_material_set_conduction(mat, add_temp & 0xFFFFFFFF, conduction_self, conduction_other),
          "set_conduction")


def set_factory_temperature(mat, temperature):
    """Temperature of new SOUP tiles of a material (TilesCreate, game_datastruct.cpp:427-437)."""
    check(lib().fse_material_set_factory_temperature(mat, temperature), "set_factory_temperature")


def get_conduction(mat):
    """(addTemp, conductionSelf, conductionOther, factory temperature) of a material."""
    out = np.zeros(4, np.uint32)
    check(lib().fse_material_get_conduction(mat, ptr(out)), "get_conduction")
    return int(out[0]), float(out[1:2].view(np.float32)[0]), float(out[2:3].view(np.float32)[0]), \
        int(out[3:4].view(np.int32)[0])


CFG_RENDER = 1
CFG_TEMPERATURE = 2
CFG_TEMPERATURE_STEP = 4
CFG_REFERENCE_ORDER = 8
CFG_F32_FLUID = 16
TEX_PIXELS, TEX_EMISSION, TEX_FIRE, TEX_FLOW, TEX_CELLS = 0, 1, 2, 3, 4


def _config(chunk_size=128, cell_iter=3, seed=0, particle_capacity=0, spawn_capacity=0, stream=None, render=False,
            temperature=False, temperature_step=False, reference_order=False, f32_fluid=False):
    """temperature: keep liquid temperatures (FSE_CFG_TEMPERATURE); temperature_step:
    also run the conduction step every fourth tick inside steps (FSE_CFG_TEMPERATURE_STEP);
    reference_order: update each chunk's cells in the reference's own order
    (FSE_CFG_REFERENCE_ORDER); f32_fluid: liquid amounts and diffs in the reference's
    own f32 arithmetic (FSE_CFG_F32_FLUID)."""
    return FseConfig(chunk_size, cell_iter, seed & 0xFFFFFFFF, particle_capacity, spawn_capacity,
                     C.c_void_p(stream) if stream else None,
                     (CFG_RENDER if render else 0) | (CFG_TEMPERATURE if temperature else 0) |
                     (CFG_TEMPERATURE_STEP if temperature_step else 0) |
                     (CFG_REFERENCE_ORDER if reference_order else 0) | (CFG_F32_FLUID if f32_fluid else 0))


# ---------------------------------------------------------------------- world
class World:
    """One device-resident world (world::init grids, world.cpp:43-145)."""

    PLANES = (("id", np.uint16), ("colour", np.uint32), ("scalar", np.int32), ("flags", np.uint8),
              ("diff", np.int32))

    def __init__(self, width, height, chunk_size=128, cell_iter=3, seed=0, particle_capacity=0, spawn_capacity=0,
                 stream=None, render=False, temperature=False, temperature_step=False, reference_order=False,
                 f32_fluid=False, _handle=None):
        self.lib = lib()
        self.width, self.height = int(width), int(height)
        self._owned = _handle is None
        if _handle is None:
            h = C.c_void_p()
            cfg = _config(chunk_size, cell_iter, seed, particle_capacity, spawn_capacity, stream, render, temperature,
                          temperature_step, reference_order, f32_fluid)
            check(self.lib.fse_world_create(self.width, self.height, C.byref(cfg), C.byref(h)), "world_create")
            self.h = h
        else:
            self.h = C.c_void_p(_handle)
            inf = self.info()
            self.width, self.height = inf["w"], inf["h"]

    def close(self):
        if getattr(self, "h", None) and self._owned:
            self.lib.fse_world_destroy(self.h)
        self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # -- state
    def info(self):
        out = np.zeros(8, np.int32)
        check(self.lib.fse_world_info(self.h, ptr(out)), "world_info")
        return dict(zip(("w", "h", "chunk", "cell_iter", "seed", "tick", "particles", "err"), out.tolist()))

    @property
    def tick_count(self):
        return self.info()["tick"]

    @tick_count.setter
    def tick_count(self, t):
        check(self.lib.fse_world_set_tick(self.h, int(t) & 0xFFFFFFFF), "set_tick")

    def upload(self, planes):
        n = self.width * self.height
        arrs = []
        for k, dt in self.PLANES:
            a = planes.get(k)
            arrs.append(None if a is None else np.ascontiguousarray(a, dt).reshape(n))
        check(self.lib.fse_world_upload(self.h, *[ptr(a) if a is not None else None for a in arrs]), "upload")

    def state(self, out=None):
        """Download the SoA planes (into `out`, e.g. pinned host arrays, when given)."""
        n = self.width * self.height
        if out is None:
            out = {k: np.empty((self.height, self.width), dt) for k, dt in self.PLANES}
        for k, dt in self.PLANES:
            a = out[k]
            if a.dtype != dt or a.size != n or not a.flags["C_CONTIGUOUS"]:
                raise ValueError("plane %s must be a C-contiguous %s array of %d cells" % (k, np.dtype(dt), n))
        check(self.lib.fse_world_download(self.h, *[ptr(out[k]) for k, _ in self.PLANES]), "download")
        return out

    def upload_tiles(self, tiles):
        """Load the grid from an (H, W) array of tile structs (TILE_DTYPE, the reference's
        real_tiles, or any structured dtype with a subset of its field names)."""
        a = np.ascontiguousarray(tiles)
        if a.size != self.width * self.height or a.dtype.fields is None:
            raise ValueError("need a structured array of %d tiles" % (self.width * self.height))
        lay = FseTileLayout.of(a.dtype)
        check(self.lib.fse_world_upload_tiles(self.h, ptr(a), C.byref(lay)), "upload_tiles")

    def download_tiles(self, out=None, mat_table=None):
        """Store the grid into an (H, W) array of tile structs; `mat_table[id]` fills the
        `mat` pointer field when given."""
        if out is None:
            out = np.zeros((self.height, self.width), TILE_DTYPE)
        if out.size != self.width * self.height or out.dtype.fields is None or not out.flags["C_CONTIGUOUS"]:
            raise ValueError("need a C-contiguous structured array of %d tiles" % (self.width * self.height))
        lay = FseTileLayout.of(out.dtype)
        tab = None if mat_table is None else np.ascontiguousarray(mat_table, np.uint64)
        check(self.lib.fse_world_download_tiles(self.h, ptr(out), C.byref(lay), None if tab is None else ptr(tab),
                                                0 if tab is None else tab.size), "download_tiles")
        return out

    def particle_iterations(self):
        """Iterations the last particle update needed (diagnostics)."""
        n = C.c_int()
        check(self.lib.fse_world_particle_iterations(self.h, C.byref(n)), "world_particle_iterations")
        return n.value

    def set_launch(self, colour_shape):
        """Launch shape of the colour pass: 0 CTA per chunk, 1 persistent CTAs, 2 CTA pair
        per chunk, 3 persistent pairs, 4 the fused tick (every pass in one launch,
        chunk-passes started as their neighbourhoods finish). Results never depend on it."""
        check(self.lib.fse_world_set_launch(self.h, colour_shape), "world_set_launch")

    def set_tick_zone(self, x, y, w, h):
        """world::tickZone: the rectangle the tick works on (the whole world by default)."""
        check(self.lib.fse_world_set_tick_zone(self.h, x, y, w, h), "world_set_tick_zone")

    def generate(self, kind, seed):
        check(self.lib.fse_world_generate(self.h, kind, seed & 0xFFFFFFFF), "generate")

    def getTile(self, x, y):
        i, c, s, f = C.c_uint16(), C.c_uint32(), C.c_int32(), C.c_uint8()
        check(self.lib.fse_world_get_tile(self.h, x, y, C.byref(i), C.byref(c), C.byref(s), C.byref(f)), "getTile")
        return MaterialInstance(i.value, c.value, s.value, f.value)

    def setTile(self, x, y, tile):
        check(self.lib.fse_world_set_tile(self.h, x, y, tile.id, tile.colour & 0xFFFFFFFF, tile.scalar,
                                          tile.flags & 0xFF), "setTile")

    # -- the hot path
    def tick(self, n=1):
        """world::tick(), n times."""
        check(self.lib.fse_world_tick(self.h, n), "tick")

    def tickCells(self):
        """world::tickCells()."""
        check(self.lib.fse_particles_tick(self.h), "tickCells")

    def step(self, n=1, graph=False):
        """n x (world::tick(); world::tickCells()), optionally replayed from a CUDA graph."""
        fn = self.lib.fse_world_step_graph if graph else self.lib.fse_world_step
        check(fn(self.h, n), "step")

    def enqueue(self, n=1, particles=True):
        """Queue n steps (or ticks) on the world's stream without waiting."""
        check(self.lib.fse_world_enqueue(self.h, n, 1 if particles else 0), "enqueue")

    def pass_timing(self, enable):
        """Start (True) or stop (False) CUDA-event timing of the colour-pass kernel;
        returns (milliseconds, launches) accumulated since the last start."""
        ms, n = C.c_double(0.0), C.c_int64(0)
        check(self.lib.fse_world_pass_timing(self.h, 1 if enable else 0, C.byref(ms), C.byref(n)), "pass_timing")
        return ms.value, n.value

    def sync(self):
        check(self.lib.fse_world_sync(self.h), "sync")

    def set_stream(self, stream_ptr):
        check(self.lib.fse_world_set_stream(self.h, C.c_void_p(stream_ptr) if stream_ptr else None), "set_stream")

    @property
    def stream(self):
        return self.lib.fse_world_stream(self.h)

    # -- particles
    def addCell(self, parts):
        """world::addCell for an array of PARTICLE_DTYPE records (world.cpp:2292)."""
        parts = np.ascontiguousarray(parts, PARTICLE_DTYPE)
        check(self.lib.fse_particles_add(self.h, ptr(parts), len(parts)), "addCell")

    add_particles = addCell

    def particle_count(self):
        n = C.c_int(0)
        check(self.lib.fse_particles_count(self.h, C.byref(n)), "particles_count")
        return n.value

    def particles(self):
        n = self.particle_count()
        out = np.zeros(n, PARTICLE_DTYPE)
        got = C.c_int(0)
        check(self.lib.fse_particles_read(self.h, ptr(out), n, C.byref(got)), "particles_read")
        return out[: min(n, got.value)]

    # -- objects
    def object_stamp(self, bodies):
        check(self.lib.fse_object_stamp(self.h, ptr(bodies), len(bodies)), "object_stamp")

    def object_readback(self, bodies):
        rem = C.c_int64(0)
        check(self.lib.fse_object_readback(self.h, ptr(bodies), len(bodies), C.byref(rem)), "object_readback")
        return rem.value

    def object_mask(self, out=None):
        n = self.width * self.height
        if out is None:
            out = np.zeros((n + 7) // 8, np.uint8)
        check(self.lib.fse_object_mask_export(self.h, ptr(out)), "object_mask")
        return out

    def object_list(self, cap=None):
        cap = cap if cap is not None else self.width * self.height
        out = np.zeros(max(cap, 1), np.uint32)
        n = C.c_int64(0)
        check(self.lib.fse_object_list_export(self.h, ptr(out), cap, C.byref(n)), "object_list")
        return out[: min(cap, n.value)], n.value

    # -- ledger
    def ledger(self):
        m = material_count()
        out = np.zeros(6 * m, np.int64)
        check(self.lib.fse_world_ledger(self.h, ptr(out)), "ledger")
        return out.reshape(6, m)

    def reset_ledger(self):
        check(self.lib.fse_world_ledger_reset(self.h), "ledger_reset")

    def census(self):
        m = material_count()
        out = np.zeros(4 * m, np.int64)
        check(self.lib.fse_world_census(self.h, ptr(out)), "census")
        return out.reshape(4, m)

    # -- headless render textures (worlds created with render=True)
    def render_dirty(self, moving=True):
        """The dirty-cell texture pass (game.cpp:1994-2067); returns movingTiles."""
        out = np.zeros(material_count(), np.int64) if moving else None
        check(self.lib.fse_world_render_dirty(self.h, ptr(out) if moving else None), "render_dirty")
        return out

    def render_cells(self):
        """The particle layer (world::renderCells, world.cpp:2006-2028)."""
        check(self.lib.fse_world_render_cells(self.h), "render_cells")

    def render_texture(self, which):
        """A texture as an (H, W, 4) uint8 array of r, g, b, a."""
        out = np.zeros((self.height, self.width, 4), np.uint8)
        check(self.lib.fse_world_render_read(self.h, int(which), ptr(out)), "render_read")
        return out

    # -- chunk .pack codec
    def pack(self, phase=0):
        """Chunk::ChunkWrite for every chunk (chunk.cpp:219-330): (bytes, offsets)."""
        nb, nc = C.c_int64(0), C.c_int(0)
        check(self.lib.fse_world_pack_bound(self.width, self.height, C.byref(nb), C.byref(nc)), "pack_bound")
        out = np.empty(nb.value, np.uint8)
        offs = np.zeros(nc.value + 1, np.int64)
        check(self.lib.fse_world_pack(self.h, int(phase), ptr(out), nb.value, ptr(offs), C.byref(nc)), "pack")
        return out[: offs[-1]], offs

    def unpack(self, data, offsets):
        """Chunk::ChunkRead for every chunk: the chunks' generation phases."""
        data = np.ascontiguousarray(data, np.uint8)
        offsets = np.ascontiguousarray(offsets, np.int64)
        phases = np.zeros(len(offsets) - 1, np.int8)
        bad = C.c_int(-1)
        st = self.lib.fse_world_unpack(self.h, ptr(data), ptr(offsets), len(offsets) - 1, ptr(phases), C.byref(bad))
        if st != 0:
            raise FseError(st, "unpack (chunk %d)" % bad.value)
        return phases

    # -- exact checkpoints
    def trim(self):
        """Free the device scratch kept by pack / unpack / the tile-struct calls."""
        check(self.lib.fse_world_trim(self.h), "trim")

    def checkpoint(self):
        """Every plane, particle, the tick, seed and ledger, LZ4-compressed: bytes."""
        nb, size = C.c_int64(0), C.c_int64(0)
        check(self.lib.fse_world_checkpoint_bound(self.h, C.byref(nb)), "checkpoint_bound")
        out = np.empty(nb.value, np.uint8)
        check(self.lib.fse_world_checkpoint(self.h, ptr(out), nb.value, C.byref(size)), "checkpoint")
        return out[: size.value].copy()

    def restore(self, data):
        data = np.ascontiguousarray(data, np.uint8)
        check(self.lib.fse_world_restore(self.h, ptr(data), data.size), "restore")

    # -- temperature
    def temperature(self, out=None):
        """MaterialInstance::temperature of every cell as an (H, W) int16 array."""
        if out is None:
            out = np.empty((self.height, self.width), np.int16)
        check(self.lib.fse_world_temperature_read(self.h, ptr(out)), "temperature_read")
        return out

    def set_temperature(self, temps):
        a = np.ascontiguousarray(temps, np.int16)
        assert a.size == self.width * self.height
        check(self.lib.fse_world_temperature_write(self.h, ptr(a)), "temperature_write")

    def tickTemperature(self):
        """world::tickTemperature (world.cpp:1950-2004), enqueued on the world's stream."""
        check(self.lib.fse_world_tick_temperature(self.h), "tick_temperature")

    # -- solid islands
    def physicsCheck(self, x, y, pixels=True):
        """world::physicsCheck (world.cpp:3330-3445): (cells cut, bbox, colour image or None)."""
        n = C.c_int(0)
        bbox = np.zeros(4, np.int32)
        pix = np.zeros(1000 * 1000, np.uint32) if pixels else None
        check(self.lib.fse_world_physics_check(self.h, int(x), int(y), C.byref(n), ptr(bbox),
                                               ptr(pix) if pixels else None, pix.size if pixels else 0),
              "physics_check")
        if n.value == 0:
            return 0, None, None
        bw, bh = int(bbox[2] - bbox[0] + 1), int(bbox[3] - bbox[1] + 1)
        img = pix[: bw * bh].reshape(bh, bw).copy() if (pixels and n.value > 10) else None
        return n.value, bbox, img

    def islands(self, max_cells=1000, remove=False, cap=1 << 16):
        """Every 4-connected SOLID region of at most max_cells cells: (table, count)."""
        out = np.zeros(max(cap, 1), _abi.ISLAND_DTYPE)
        n = C.c_int(0)
        check(self.lib.fse_world_islands(self.h, int(max_cells), 1 if remove else 0, ptr(out), int(cap),
                                         C.byref(n)), "islands")
        return out[: min(cap, n.value)], n.value


class Batch:
    """Many worlds ticked by one launch per colour pass (configs with uneven sizes)."""

    def __init__(self, worlds):
        self.lib = lib()
        self.worlds = list(worlds)
        arr = (C.c_void_p * len(self.worlds))(*[w.h.value for w in self.worlds])
        h = C.c_void_p()
        check(self.lib.fse_batch_create(arr, len(self.worlds), C.byref(h)), "batch_create")
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            self.lib.fse_batch_destroy(self.h)
        self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def step(self, n=1, graph_ticks=0):
        if graph_ticks:
            check(self.lib.fse_batch_step_graph(self.h, n, graph_ticks), "batch_step_graph")
        else:
            check(self.lib.fse_batch_step(self.h, n), "batch_step")

    def enqueue(self, n=1):
        """Enqueue n ticks on the batch's stream without waiting; sync() waits and
        reports their errors. Batches of disjoint worlds run concurrently."""
        check(self.lib.fse_batch_enqueue(self.h, n), "batch_enqueue")

    def prepare_graphs(self, n, graph_ticks=32):
        """Capture the graphs step(n, graph_ticks) will replay, without running them."""
        check(self.lib.fse_batch_prepare_graphs(self.h, n, graph_ticks), "batch_prepare_graphs")

    def autotune(self):
        out = np.zeros(4, np.int32)
        check(self.lib.fse_batch_autotune(self.h, ptr(out)), "batch_autotune")
        return {"colour_ctas_per_sm": int(out[0]), "particle_blocks": int(out[1]), "us": int(out[2]),
                "index": int(out[3])}

    def set_launch(self, colour_ctas_per_sm, particle_blocks):
        check(self.lib.fse_batch_set_launch(self.h, colour_ctas_per_sm, particle_blocks), "batch_set_launch")

    def upload(self, index, planes):
        """Enqueue an upload of member `index`'s planes (host arrays, pinned for the copy
        to run asynchronously; keep them alive until sync()) on the batch's stream."""
        w = self.worlds[index]
        n = w.width * w.height
        arrs = []
        for k, dt in World.PLANES:
            a = planes.get(k)
            if a is not None and (a.dtype != dt or a.size != n or not a.flags["C_CONTIGUOUS"]):
                raise ValueError("plane %s must be a C-contiguous %s array of %d cells" % (k, np.dtype(dt), n))
            arrs.append(a)
        check(self.lib.fse_batch_upload(self.h, index, *[ptr(a) if a is not None else None for a in arrs]),
              "batch_upload")

    def io_layout(self):
        """(offsets, bytes): member k's planes id, colour, scalar, flags, diff start at
        offsets[k, 0..4] of a buffer of `bytes` bytes (upload_all / download_all)."""
        offs = np.zeros((len(self.worlds), 5), np.int64)
        total = C.c_int64(0)
        check(self.lib.fse_batch_io_layout(self.h, ptr(offs), C.byref(total)), "batch_io_layout")
        return offs, total.value

    def io_views(self, buf):
        """Per member, the plane arrays (World.state() keys) that live in `buf`, a
        uint8 array of io_layout()'s size."""
        offs, total = self.io_layout()
        if buf.dtype != np.uint8 or buf.size != total or not buf.flags["C_CONTIGUOUS"]:
            raise ValueError("need a C-contiguous uint8 buffer of %d bytes" % total)
        out = []
        for k, w in enumerate(self.worlds):
            n = w.width * w.height
            v = {}
            for p, (key, dt) in enumerate(World.PLANES):
                nb = n * np.dtype(dt).itemsize
                v[key] = buf[offs[k, p]:offs[k, p] + nb].view(dt).reshape(w.height, w.width)
            out.append(v)
        return out

    def upload_all(self, buf):
        """Enqueue one copy of every member's planes from `buf` (io_layout; pinned for
        an asynchronous copy; keep it alive until sync())."""
        check(self.lib.fse_batch_upload_all(self.h, ptr(buf), buf.nbytes), "batch_upload_all")

    def download_all(self, buf):
        """Enqueue the gather of every member's planes into `buf` (filled after sync())."""
        check(self.lib.fse_batch_download_all(self.h, ptr(buf), buf.nbytes), "batch_download_all")

    def download(self, index, out):
        """Enqueue a download of member `index`'s planes into the host arrays of `out`
        (filled after sync())."""
        w = self.worlds[index]
        n = w.width * w.height
        for k, dt in World.PLANES:
            a = out[k]
            if a.dtype != dt or a.size != n or not a.flags["C_CONTIGUOUS"]:
                raise ValueError("plane %s must be a C-contiguous %s array of %d cells" % (k, np.dtype(dt), n))
        check(self.lib.fse_batch_download(self.h, index, *[ptr(out[k]) for k, _ in World.PLANES]),
              "batch_download")

    def sync(self):
        check(self.lib.fse_batch_sync(self.h), "batch_sync")

    def timing(self, enable, cap=1 << 16):
        """Start (True) or stop (False) CUDA-event timing of the batch's colour-pass
        launches and ticks; returns what was accumulated since the last start:
        (colour-pass ms, colour-pass launches, per-tick ms array)."""
        ms, n, nt = C.c_double(), C.c_int64(), C.c_int()
        out = np.zeros(cap, np.float32)
        check(self.lib.fse_batch_timing(self.h, 1 if enable else 0, C.byref(ms), C.byref(n), ptr(out), cap,
                                        C.byref(nt)), "batch_timing")
        return ms.value, n.value, out[: min(cap, nt.value)].copy()

    @property
    def stream(self):
        return self.lib.fse_batch_stream(self.h)


class Server:
    """World-tick requests served by continuous batching under an HBM budget.

    Worlds keep their state in HBM while they fit the budget; the rest are parked
    in host memory as exact checkpoints and restored when a request for them is
    admitted. step() enqueues one batched tick of the active requests and returns
    while it runs (up to `depth` steps in flight); poll() reports finished requests
    with their device completion times."""

    def __init__(self, hbm_budget_bytes, max_active):
        self.lib = lib()
        h = C.c_void_p()
        check(self.lib.fse_server_create(int(hbm_budget_bytes), int(max_active), C.byref(h)), "server_create")
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            self.lib.fse_server_destroy(self.h)
        self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def add_world(self, width, height, gen_kind=GEN_MIX, gen_seed=1234, **cfg):
        slot = C.c_int(-1)
        c = _config(**cfg)
        st = self.lib.fse_server_add_world(self.h, width, height, C.byref(c), gen_kind, gen_seed & 0xFFFFFFFF,
                                           C.byref(slot))
        check(st, "server_add_world")
        return slot.value

    def try_add_world(self, width, height, gen_kind=GEN_MIX, gen_seed=1234, **cfg):
        try:
            return self.add_world(width, height, gen_kind, gen_seed, **cfg)
        except FseError as e:
            if e.status == -3:
                return None
            raise

    def remove_world(self, slot):
        check(self.lib.fse_server_remove_world(self.h, slot), "server_remove_world")

    def world(self, slot):
        p = self.lib.fse_server_world(self.h, slot)
        return World(0, 0, _handle=p) if p else None

    def bytes_in_use(self):
        return self.lib.fse_server_bytes_in_use(self.h)

    def now_us(self):
        return self.lib.fse_server_now_us(self.h)

    def submit(self, slot, n_ticks, arrival_us=None):
        rid = C.c_int64(-1)
        t = self.now_us() if arrival_us is None else arrival_us
        check(self.lib.fse_server_submit(self.h, slot, n_ticks, float(t), C.byref(rid)), "server_submit")
        return rid.value

    def step(self):
        act = C.c_int(0)
        check(self.lib.fse_server_step(self.h, C.byref(act)), "server_step")
        return act.value

    def poll(self, cap=4096):
        ids = np.zeros(cap, np.int64)
        done = np.zeros(cap, np.float64)
        n = C.c_int(0)
        check(self.lib.fse_server_poll(self.h, 0.0, ptr(ids), ptr(done), cap, C.byref(n)), "server_poll")
        return ids[: n.value], done[: n.value]

    def set_depth(self, depth):
        """Steps in flight before step() waits for the oldest (1..64)."""
        check(self.lib.fse_server_set_depth(self.h, int(depth)), "server_set_depth")

    def drain(self):
        check(self.lib.fse_server_drain(self.h), "server_drain")

    STAT_KEYS = ("steps", "restored", "parked_out", "resident", "parked", "max_in_flight", "queued", "active")

    def stats(self):
        out = np.zeros(len(self.STAT_KEYS), np.int64)
        check(self.lib.fse_server_stats(self.h, ptr(out), len(out)), "server_stats")
        return dict(zip(self.STAT_KEYS, (int(v) for v in out)))

    def tick_times(self, cap=1 << 20):
        """Device milliseconds of the steps retired since the last call."""
        ms = np.zeros(cap, np.float32)
        n = C.c_int(0)
        check(self.lib.fse_server_tick_times(self.h, ptr(ms), cap, C.byref(n)), "server_tick_times")
        return ms[: n.value].copy()


def write_png(path, rgba):
    """Write an (H, W, 4) uint8 r, g, b, a array as a PNG file (zlib only)."""
    import struct
    import zlib

    a = np.ascontiguousarray(rgba, np.uint8)
    h, w = a.shape[0], a.shape[1]
    raw = b"".join(b"\x00" + a[y].tobytes() for y in range(h))

    def chunk(tag, data):
        return struct.pack(">I", len(data)) + tag + data + struct.pack(">I", zlib.crc32(tag + data) & 0xFFFFFFFF)

    png = b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, 8, 6, 0, 0, 0))
    png += chunk(b"IDAT", zlib.compress(raw, 6)) + chunk(b"IEND", b"")
    with open(path, "wb") as f:
        f.write(png)
