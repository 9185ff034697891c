"""Benchmark of the GB300 falling-sand world tick.

Default workload (the headline metric: Gcell-updates/s and HBM roofline fraction,
batched vs per-world launch, tick latency percentiles): 256 worlds of uneven sizes
(sides uniform in {128, ..., 2048}), the standard material mix, batched launches
replayed from 32-tick CUDA graphs with the autotuned launch shape, against the same
worlds stepped through 256 plain per-world launches; a step is world::tick() +
world::tickCells() of every world. The single 4096x2048 world with 1M free
particles (plain per-world launch) is reported beside it under "config1". Prints
one JSON line.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl fse|reference]
                  [--workload 2|0|1|3|4]

--impl reference times the reference's own world::tick + world::tickCells
(compiled from its extracted sources, all host threads) on a bounded sample of the
same workload. Workloads 0, 1, 3, 4 alone: the 512^2 world; the 4096x2048 world
with particles; the 16384^2 world with OBJECT boxes; the continuous-batching server.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

BYTES_PER_CELL_UPDATE = 22  # 11-byte SoA cell state read once and written once per tick
METRIC = "Gcell-updates/s"
L2_FLUSH_BYTES = 512 << 20
REF_BUDGET_S = 90.0  # cap on the timed region of the CPU reference arm
# ticks per workload: 512^2 world 1000, 4096x2048 world 500, 256 worlds 200,
# 16384^2 world 100; the server workload is timed by its arrival window instead
WORKLOAD_TICKS = {0: 1000, 1: 500, 2: 200, 3: 100, 4: 0}


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def dist_info():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("LOCAL_RANK", 0)), int(os.environ.get("WORLD_SIZE", 1))


class Clocks:
    """nvidia-smi clock/throttle samples taken during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.p = None
        # the raw samples go to FSE_CLOCKS_DIR (a folder to keep them in) or the temp dir
        folder = os.environ.get("FSE_CLOCKS_DIR") or tempfile.gettempdir()
        self.path = os.path.join(folder, "clocks_%d.csv" % os.getpid())

    def start(self):
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.f = open(self.path, "w")
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                                       "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                                      stderr=subprocess.DEVNULL)
        except Exception:
            self.p = None

    def stop(self):
        if self.p is None:
            return None
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except Exception:
            self.p.kill()
        self.f.close()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        with open(self.path) as f:
            for line in f:
                parts = [x.strip() for x in line.split(",")]
                if len(parts) < 9:
                    continue
                try:
                    sm.append(float(parts[1]))
                    mx.append(float(parts[2]))
                except ValueError:
                    continue
                for n, v in zip(names, parts[5:9]):
                    if v.lower() == "active":
                        reasons.add(n)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


# ------------------------------------------------------------------ workloads
def config1_particles(n, w, h, seed):
    """1M free particles: position uniform over the world, velocity N(0, 2)
    cells/tick (FP64 draws rounded to f32), gravity 0.1 cells/tick^2, sand tiles."""
    from falling_sand_engine_gb300 import PARTICLE_DTYPE, material_find

    rng = np.random.default_rng(seed)
    p = np.zeros(n, PARTICLE_DTYPE)
    p["x"] = rng.uniform(0, w, n).astype(np.float32)
    p["y"] = rng.uniform(0, h, n).astype(np.float32)
    p["vx"] = rng.normal(0.0, 2.0, n).astype(np.float32)
    p["vy"] = rng.normal(0.0, 2.0, n).astype(np.float32)
    p["ay"] = np.float32(0.1)
    p["fade_time"] = 60
    p["id"] = material_find("GENERIC_SAND")
    p["colour"] = 0xFFFFFFFF
    return p


def _flush(buf, i):
    buf.fill_(i & 0x7F)


def bench_config1(args, rank, local_rank, world_size):
    import torch

    import falling_sand_engine_gb300 as fse

    W, H, NP = 4096, 2048, 1_000_000
    seed = 1234 + rank
    fse.InitMaterials()
    fse.PushMaterials()
    stream = torch.cuda.Stream()
    world = fse.World(W, H, chunk_size=128, cell_iter=3, seed=seed, particle_capacity=4_000_000,
                      spawn_capacity=2_000_000, stream=stream.cuda_stream)
    world.generate(fse.GEN_MIX, seed)
    world.addCell(config1_particles(NP, W, H, seed))
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.int32, device="cuda")
    for _ in range(args.warmup):
        world.step(1)
    cells = W * H

    # timed region: per-step CUDA events on the world's stream, L2 flushed between
    # steps outside the events
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    clocks = Clocks(local_rank)
    barrier(world_size)
    torch.cuda.synchronize()
    world.pass_timing(True)
    l0 = fse.launch_counter()
    clocks.start()
    t0 = time.perf_counter()
    with torch.cuda.stream(stream):
        for i in range(args.steps):
            _flush(flush, i)
            ev[i][0].record(stream)
            world.enqueue(1, particles=True)
            ev[i][1].record(stream)
    world.sync()
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    clk = clocks.stop()
    launches = fse.launch_counter() - l0
    pass_ms, pass_n = world.pass_timing(False)
    live_particles = world.particle_count()
    step_ms = np.array([a.elapsed_time(b) for a, b in ev])
    gpu_ms = float(step_ms.sum())
    gpu_ms = max_over_ranks(gpu_ms, world_size)
    tick_latency = {"p50": round(float(np.percentile(step_ms, 50)), 4), "p99": round(float(np.percentile(step_ms, 99)), 4),
                    "max": round(float(step_ms.max()), 4), "unit": "ms per step (tick + tickCells), CUDA events"}
    barrier(world_size)

    value = world_size * cells * args.steps / (gpu_ms / 1e3) / 1e9
    peak, peak_kind = peaks()
    roof = colour_roofline(cells, args.steps, pass_ms, pass_n, peak, peak_kind, "colour_pass_config1",
                           "the 4096x2048 world")
    roof["tick_frac"] = round(value * 1e9 * BYTES_PER_CELL_UPDATE / world_size / (peak * 1e9), 4)

    # end to end through the C ABI with host buffers: every step uploads the grid
    # from pinned host memory, ticks, and reads the grid back
    e2e = e2e_config1(world, args, torch, cells, world_size)
    render = render_config1(fse, torch, W, H, seed, NP) if rank == 0 else None
    temperature = temperature_config1(fse, torch, W, H, seed, NP) if rank == 0 else None
    pack = pack_config1(fse, torch, W, H, seed, NP) if rank == 0 else None
    reforder = reference_order_config1(fse, torch, W, H, seed, NP) if rank == 0 else None
    cpu = None
    if rank == 0 and world_size == 1 and not args.no_cpu:
        cpu = cpu_baseline_config1(seed)
    world.close()
    return {
        "metric": METRIC, "value": round(value, 4), "unit": "Gcell/s", "n_gpus": world_size, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(gpu_ms / args.steps, 4), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "int32+f32", "data": "synthetic",
        "config": {"workload": "config1: one 4096x2048 world (mix: 30% sand, 20% water, 10% gas, 15% rock, 25% air in "
                               "the top 60%, 8 rock rows) + 1M free particles, plain per-world launch",
                   "world": [W, H], "particles": NP, "particles_live_after": live_particles, "chunk": 128,
                   "cell_iter": 3, "seed": seed,
                   "l2": "flushed between timed steps (512 MiB write outside the events)",
                   "parallelism": "one independent world per GPU" if world_size > 1 else "single GPU"},
        "roofline": roof, "e2e": e2e, "cpu_baseline": cpu, "clocks": clk, "gpu_launches": int(launches),
        "wall_s": round(wall, 3), "render": render, "temperature": temperature, "pack": pack,
        "reference_order": reforder, "tick_latency": tick_latency,
    }


def render_config1(fse, torch, W, H, seed, NP, ticks=20):
    """The render passes on the same workload (a world created with render state):
    after each tick, the dirty-cell texture pass and the particle layer, timed with
    CUDA events on the world's stream. Algorithmic bytes of the dirty pass: the
    1-byte mark of every cell, plus for a dirty cell its id, colour, flow sums and
    mark (read/cleared) and three texels (27 B), plus 20 B more for a liquid
    (smoothed flows read and written, flow texel)."""
    stream = torch.cuda.Stream()
    world = fse.World(W, H, chunk_size=128, cell_iter=3, seed=seed, particle_capacity=4_000_000,
                      spawn_capacity=2_000_000, stream=stream.cuda_stream, render=True)
    world.generate(fse.GEN_MIX, seed)
    world.addCell(config1_particles(NP, W, H, seed))
    soup = np.array([fse.material_get(i)[0] == fse.SOUP for i in range(fse.material_count())])
    world.render_dirty(moving=False)
    for _ in range(3):
        world.step(1)
        world.render_dirty(moving=False)
    d_ms = c_ms = 0.0
    nbytes = ndirty = 0
    e = [_ev(torch) for _ in range(4)]
    for _ in range(ticks):
        world.step(1)
        with torch.cuda.stream(stream):
            e[0].record(stream)
            world.render_cells()
            e[1].record(stream)
            e[2].record(stream)
        mv = world.render_dirty(moving=True)
        with torch.cuda.stream(stream):
            e[3].record(stream)
        torch.cuda.synchronize()
        c_ms += e[0].elapsed_time(e[1])
        d_ms += e[2].elapsed_time(e[3])
        nbytes += W * H + 27 * int(mv.sum()) + 20 * int(mv[soup].sum())
        ndirty += int(mv.sum())
    peak, peak_kind = peaks()
    gbs = nbytes / (d_ms / 1e3) / 1e9
    # solid islands on the same world: physicsCheck from random seeds (the drop-in,
    # one per tick in the reference) and the all-regions labelling pass (each call
    # is synchronous: host clock around it)
    rng = np.random.default_rng(seed)
    t0 = time.perf_counter()
    cut = 0
    for _ in range(50):
        cut += world.physicsCheck(int(rng.integers(0, W)), int(rng.integers(0, H)))[0] > 0
    pc_ms = (time.perf_counter() - t0) * 1e3 / 50
    world.islands(1000)
    t0 = time.perf_counter()
    for _ in range(5):
        _, n_isl = world.islands(1000)
    isl_ms = (time.perf_counter() - t0) * 1e3 / 5
    ref_cpu = render_reference_cpu(fse, world, stream, torch)
    world.close()
    islands = {"physics_check_ms": round(pc_ms, 3), "physics_check_cut": int(cut), "label_all_ms": round(isl_ms, 3),
               "label_all_gcells": round(W * H / (isl_ms / 1e3) / 1e9, 3), "islands_le_1000": int(n_isl)}
    return {"islands": islands,
            "dirty_pass_ms": round(d_ms / ticks, 4), "dirty_pass_gcells": round(W * H * ticks / (d_ms / 1e3) / 1e9, 3),
            "dirty_cells_per_tick": ndirty // ticks, "dirty_pass_gbs": round(gbs, 1),
            "dirty_pass_frac": round(gbs / peak, 4), "peak": peak, "peak_kind": peak_kind,
            "particle_layer_ms": round(c_ms / ticks, 4), "ticks": ticks, "cpu_reference": ref_cpu}


def render_reference_cpu(fse, world, stream, torch):
    """The reference's own dirty-pixel loop (game.cpp:1995-2061, compiled unchanged;
    one host thread, as one task of its pool) on the world after one more step, with
    the cells that step changed marked dirty: host clock around one pass."""
    from oracle.binding import build_reference_render, reference_render_dirty

    try:
        lib = build_reference_render()
    except Exception:  # noqa: BLE001 - no compiler or sources here
        lib = None
    if lib is None:
        return None
    before = world.state()
    with torch.cuda.stream(stream):
        world.step(1)
    torch.cuda.synchronize()
    st = world.state()
    dirty = ((st["id"] != before["id"]) | (st["colour"] != before["colour"])).astype(np.uint8)
    mats = np.array([fse.material_get(i) for i in range(fse.material_count())])
    types, iters, alpha, emit = mats[:, 0], mats[:, 2], mats[:, 5], mats[:, 8].astype(np.uint32)
    z = np.zeros(st["id"].shape, np.float32)
    t0 = time.perf_counter()
    reference_render_dirty(lib, st["id"], st["colour"], dirty, z, z, z, z, (types, alpha, emit, iters),
                           fse.material_find("FIRE"))
    ms = (time.perf_counter() - t0) * 1e3
    return {"dirty_pass_ms": round(ms, 2), "cores": 1, "kind": "reference", "dirty_cells": int(dirty.sum()),
            "sample": "one pass over the whole world, host clock (includes the harness's copies of the planes)"}


def temperature_config1(fse, torch, W, H, seed, NP, calls=10):
    """world::tickTemperature on the same workload (a world created with the
    temperature step, so every fourth step of the warm-up already conducted heat
    from the -1023 water): standalone conduction steps, each timed with CUDA events
    on the world's stream with the L2 flushed before it. Algorithmic bytes of one
    step: id 2 B + scalar 4 B + SOUP temperature 2 B read per cell, plus 4 B
    (scalar) or 2 B (SOUP temperature) for each cell whose temperature changed,
    counted from the temperature planes before and after each step."""
    stream = torch.cuda.Stream()
    world = fse.World(W, H, chunk_size=128, cell_iter=3, seed=seed, particle_capacity=4_000_000,
                      spawn_capacity=2_000_000, stream=stream.cuda_stream, temperature_step=True)
    world.generate(fse.GEN_MIX, seed)
    world.addCell(config1_particles(NP, W, H, seed))
    world.step(16)
    soup = np.array([fse.material_get(i)[0] == fse.SOUP for i in range(fse.material_count())])
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device="cuda")
    e = [_ev(torch) for _ in range(2)]
    ms = 0.0
    nbytes = nchanged = 0
    cells = W * H
    with torch.cuda.stream(stream):
        world.tickTemperature()  # warm-up (scratch allocation, attribute setup)
    torch.cuda.synchronize()
    for i in range(calls):
        before = world.temperature()
        ids = world.state()["id"]
        with torch.cuda.stream(stream):
            _flush(flush, i)
            e[0].record(stream)
            world.tickTemperature()
            e[1].record(stream)
        torch.cuda.synchronize()
        ms += e[0].elapsed_time(e[1])
        ch = world.temperature() != before
        sp = soup[ids]
        nch_soup = int((ch & sp).sum())
        nch = int(ch.sum())
        nbytes += 8 * cells + 4 * (nch - nch_soup) + 2 * nch_soup
        nchanged += nch
    cpu = temperature_reference_cpu(fse, world)
    world.close()
    peak, peak_kind = peaks()
    gbs = nbytes / (ms / 1e3) / 1e9
    return {"cpu_reference": cpu, "step_ms": round(ms / calls, 4),
            "gcells": round(cells * calls / (ms / 1e3) / 1e9, 3),
            "changed_cells_per_step": nchanged // calls, "achieved_gbs": round(gbs, 1),
            "frac": round(gbs / peak, 4), "peak": peak, "peak_kind": peak_kind, "calls": calls,
            "kernels": "k_temp_tiles + k_temp_commit",
            "l2": "flushed before each step (512 MiB write outside the events)"}


def reference_order_config1(fse, torch, W, H, seed, NP, steps=3):
    """The same workload stepped in the reference's own update order inside each chunk
    (FSE_CFG_REFERENCE_ORDER: the cells of each chunk in world.cpp's loop order, run
    as a wavefront of one thread per chunk row; the semantics of the CPU baseline's
    reference chunk order): steps timed with CUDA
    events on the world's stream after two warm-up steps, L2 flushed between them."""
    stream = torch.cuda.Stream()
    world = fse.World(W, H, chunk_size=128, cell_iter=3, seed=seed, particle_capacity=4_000_000,
                      spawn_capacity=2_000_000, stream=stream.cuda_stream, reference_order=True)
    world.generate(fse.GEN_MIX, seed)
    world.addCell(config1_particles(NP, W, H, seed))
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device="cuda")
    e = [_ev(torch) for _ in range(2)]
    with torch.cuda.stream(stream):
        world.step(2)
    torch.cuda.synchronize()
    ms = 0.0
    for i in range(steps):
        with torch.cuda.stream(stream):
            _flush(flush, i)
            e[0].record(stream)
            world.step(1)
            e[1].record(stream)
        torch.cuda.synchronize()
        ms += e[0].elapsed_time(e[1])
    world.close()
    return {"ms_per_step": round(ms / steps, 3), "gcells": round(W * H * steps / (ms / 1e3) / 1e9, 4),
            "steps": steps, "order": "reference: cells in world.cpp's loop order, one thread per chunk row (wavefront)"}


def pack_reference_cpu(om, data, offs):
    """The reference's own codec core on the same chunks: its vendored LZ4 1.9.4
    (LZ4_compress_fast with acceleration 10, as Chunk::ChunkWrite calls it,
    chunk.cpp:219-330, and LZ4_decompress_safe) on each chunk's two raw blocks, one
    thread, host clock."""
    from oracle.binding import ReferenceLZ4, build_reference_lz4, lz4_decode

    try:
        path = build_reference_lz4()
    except Exception:  # noqa: BLE001 - no compiler or sources here
        path = None
    if path is None:
        return None
    ref = ReferenceLZ4(path)
    blocks = []
    for k in range(len(offs) - 1):
        p = data[offs[k]:offs[k + 1]]
        hd = np.frombuffer(p[1:17].tobytes(), "<i4")
        b1 = p[17:17 + hd[1]]
        b2 = p[17 + hd[1]:17 + hd[1] + hd[3]]
        blocks.append((lz4_decode(b1, int(hd[0]))[0], lz4_decode(b2, int(hd[2]))[0]))
    t0 = time.perf_counter()
    packed = [(ref.compress(r1, 10), ref.compress(r2, 10)) for r1, r2 in blocks]
    pack_s = time.perf_counter() - t0
    t0 = time.perf_counter()
    for (c1, c2), (r1, r2) in zip(packed, blocks):
        ref.decompress(c1, len(r1))
        ref.decompress(c2, len(r2))
    unpack_s = time.perf_counter() - t0
    n = len(blocks)
    return {"chunks": n, "threads": 1, "kind": "reference", "pack_ms_per_chunk": round(pack_s * 1e3 / n, 3),
            "unpack_ms_per_chunk": round(unpack_s * 1e3 / n, 3),
            "packed_bytes_per_chunk": int(sum(len(a) + len(b) for a, b in packed) // n)}


def temperature_reference_cpu(fse, world):
    """The reference's own world::tickTemperature (world.cpp:1950-2004, compiled
    unchanged; single-threaded as in the reference) on the same world, the tick zone
    one cell inside the world edge: host clock around one step."""
    from oracle.binding import build_reference_temperature, reference_tick_temperature

    try:
        lib = build_reference_temperature()
    except Exception:  # noqa: BLE001 - no compiler or sources here
        lib = None
    if lib is None:
        return None
    ids = world.state()["id"]
    temps = world.temperature()
    cond = np.array([fse.get_conduction(i) for i in range(fse.material_count())], np.float64)
    h, w = ids.shape
    t0 = time.perf_counter()
    reference_tick_temperature(lib, ids, temps, cond[:, 0].astype(np.uint32), cond[:, 1].astype(np.float32),
                               cond[:, 2].astype(np.float32), (1, 1, w - 2, h - 2))
    ms = (time.perf_counter() - t0) * 1e3
    return {"step_ms": round(ms, 2), "gcells": round((w - 2) * (h - 2) / (ms / 1e3) / 1e9, 4), "cores": 1,
            "kind": "reference", "sample": "one step over the world less its edge cells, host clock"}


def pack_config1(fse, torch, W, H, seed, NP, calls=5):
    """The chunk .pack codec (Chunk::ChunkWrite / ChunkRead) on the same workload
    after 16 steps: every 128x128 chunk packed into host memory and read back,
    host clock around each call (the calls are synchronous and include the
    host<->device copies). Throughput counts the uncompressed .pack payload, 393216
    + 65536 bytes per chunk. CPU leg: the oracle's C restatement of the same
    codec, one thread, on 16 chunks of the same world."""
    import oracle as om

    om.build_oracle()
    om.Oracle().reset_materials()
    world = fse.World(W, H, chunk_size=128, cell_iter=3, seed=seed, particle_capacity=4_000_000,
                      spawn_capacity=2_000_000, temperature=True)
    world.generate(fse.GEN_MIX, seed)
    world.addCell(config1_particles(NP, W, H, seed))
    world.step(16)
    world.sync()
    data, offs = world.pack(0)  # warm-up
    world.unpack(data, offs)
    t0 = time.perf_counter()
    for _ in range(calls):
        data, offs = world.pack(0)
    pack_s = (time.perf_counter() - t0) / calls
    back = fse.World(W, H, seed=seed, temperature=True)
    t0 = time.perf_counter()
    for _ in range(calls):
        back.unpack(data, offs)
    unpack_s = (time.perf_counter() - t0) / calls
    same = bool(np.array_equal(back.state()["id"], world.state()["id"]))
    n = len(offs) - 1
    raw = n * (393216 + 65536)
    # CPU: the oracle on a 512 x 512 corner (16 chunks) of the same state
    st = world.state()
    temps = world.temperature()
    ow = om.OracleWorld(512, 512, 128, 3, seed)
    sub = {k: np.ascontiguousarray(v[:512, :512]) for k, v in st.items()}
    ow.set_state(sub)
    ow.set_temperature(np.ascontiguousarray(temps[:512, :512]))
    t0 = time.perf_counter()
    od, oo = ow.pack(0)
    cpu_pack_s = time.perf_counter() - t0
    ob = om.OracleWorld(512, 512, 128, 3, seed)
    t0 = time.perf_counter()
    ob.unpack(od, oo)
    cpu_unpack_s = time.perf_counter() - t0
    lz4 = pack_reference_cpu(om, od, oo)
    world.close()
    back.close()
    return {"cpu_reference": lz4, "chunks": n, "packed_bytes": int(offs[-1]), "ratio": round(offs[-1] / raw, 4),
            "pack_ms": round(pack_s * 1e3, 3), "unpack_ms": round(unpack_s * 1e3, 3),
            "pack_gbs": round(raw / pack_s / 1e9, 2), "unpack_gbs": round(raw / unpack_s / 1e9, 2),
            "roundtrip_ids_equal": same,
            "cpu_oracle": {"chunks": len(oo) - 1, "threads": 1, "pack_ms_per_chunk": round(cpu_pack_s * 1e3 / (len(oo) - 1), 3),
                           "unpack_ms_per_chunk": round(cpu_unpack_s * 1e3 / (len(oo) - 1), 3)},
            "timing": "host clock around the synchronous host-buffer calls (copies included)"}


def e2e_config1(world, args, torch, cells, world_size):
    import falling_sand_engine_gb300 as fse

    st = world.state()
    pinned = {}
    for k, v in st.items():
        t = torch.empty(v.size, dtype={np.uint16: torch.int16, np.uint32: torch.int32, np.int32: torch.int32,
                                       np.uint8: torch.uint8}[v.dtype.type], pin_memory=True)
        a = t.numpy().view(v.dtype).reshape(v.shape)
        a[...] = v
        pinned[k] = (t, a)
    host = {k: a for k, (t, a) in pinned.items()}
    bi = sum(a.nbytes for a in host.values())
    steps = max(1, min(args.steps, 5))
    world.sync()
    t0 = time.perf_counter()
    for _ in range(steps):
        world.upload(host)
        world.step(1)
        world.state(out=host)
    dt = max_over_ranks(time.perf_counter() - t0, world_size)
    return {"value": round(world_size * cells * steps / dt / 1e9, 4), "unit": "Gcell/s",
            "h2d_bytes_per_step": int(bi), "d2h_bytes_per_step": int(bi), "steps": steps,
            "path": "fse_world_upload + fse_world_step + fse_world_download (host-resident grid)"}


def cpu_baseline_config1(seed, budget_s=12.0):
    """The reference's own tick + tickCells on the host cores (when they compile
    here), and the oracle's reference-order tick beside it, on bounded samples of the
    same workload (full 4096x2048 world + 1M particles, as many steps as fit the time
    budget, at least one)."""
    ref = reference_timing(4096, 2048, seed, 20, 1, budget_s)
    port = cpu_port_config1(seed, budget_s)
    if ref is None:
        return port
    value, n, cores = ref
    return {"value": round(value, 6), "unit": "Gcell/s", "cores": cores, "kind": "reference",
            "sample": "%d steps (tick + tickCells) of the 4096x2048 world with 1M particles after 1 warm-up step; "
                      % n + REF_NOTE % cores,
            "port": port}


def cpu_port_config1(seed, budget_s=12.0):
    """The oracle's reference-order tick on the host cores (the port), with one
    thread and in the partitioned order beside it."""
    from oracle import Oracle, OracleWorld

    o = Oracle()
    o.reset_materials()
    cores = os.cpu_count() or 1
    o.set_threads(cores)
    W, H = 4096, 2048
    ow = OracleWorld(W, H, 128, 3, seed)
    ow.generate(0, seed)
    ow.set_particles(config1_particles(1_000_000, W, H, seed))
    ow.step(1, 0)  # warm-up
    n, t0 = 0, time.perf_counter()
    while True:
        ow.step(1, 0)
        n += 1
        if time.perf_counter() - t0 > budget_s or n >= 20:
            break
    dt = time.perf_counter() - t0
    # beside it: one host thread in the same order, and all threads in the partitioned order
    o.set_threads(1)
    t1 = time.perf_counter()
    ow.step(1, 0)
    dt1 = time.perf_counter() - t1
    o.set_threads(cores)
    ow.step(1, 1)  # warm-up
    n2, t2 = 0, time.perf_counter()
    while True:
        ow.step(1, 1)
        n2 += 1
        if time.perf_counter() - t2 > budget_s / 2 or n2 >= 20:
            break
    dt2 = time.perf_counter() - t2
    return {"value": round(W * H * n / dt / 1e9, 6), "unit": "Gcell/s", "cores": cores, "kind": "port",
            "sample": "%d steps (tick + tickCells) of the 4096x2048 world with 1M particles, reference chunk order, "
                      "after 1 warm-up step" % n,
            "single_thread": {"value": round(W * H / dt1 / 1e9, 6), "sample": "1 step, reference chunk order"},
            "partitioned_order": {"value": round(W * H * n2 / dt2 / 1e9, 6), "cores": cores,
                                  "sample": "%d steps, the GPU's partitioned order" % n2}}


# ------------------------------------------------------- other workloads
def _common(args, world_size, value, unit, ms_per_step, workload, extra_cfg, launches, clk, e2e=None, cpu=None,
            higher=True, scaling="weak"):
    cfg = {"workload": workload}
    cfg.update(extra_cfg)
    return {"metric": METRIC, "value": round(value, 4), "unit": unit, "n_gpus": world_size, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(ms_per_step, 4), "higher_is_better": higher,
            "scaling": scaling, "vs_baseline": None, "dtype": "int32+f32", "data": "synthetic", "config": cfg,
            "e2e": e2e, "cpu_baseline": cpu, "clocks": clk, "gpu_launches": int(launches)}


def _ev(torch):
    return torch.cuda.Event(enable_timing=True)


def bench_config0(args, rank, local_rank, world_size):
    """512x512 world, reference chunk size, step = tick + tickCells, per-step CUDA
    events with the L2 flushed between steps; also the 32-tick graph replay."""
    import torch

    import falling_sand_engine_gb300 as fse

    W = H = 512
    seed = 1234 + rank
    fse.InitMaterials()
    fse.PushMaterials()
    stream = torch.cuda.Stream()
    world = fse.World(W, H, chunk_size=128, cell_iter=3, seed=seed, stream=stream.cuda_stream)
    world.generate(fse.GEN_MIX, seed)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.int32, device="cuda")
    for _ in range(args.warmup):
        world.step(1)
    ev = [(_ev(torch), _ev(torch)) for _ in range(args.steps)]
    clocks = Clocks(local_rank)
    barrier(world_size)
    torch.cuda.synchronize()
    l0 = fse.launch_counter()
    clocks.start()
    with torch.cuda.stream(stream):
        for i in range(args.steps):
            _flush(flush, i)
            ev[i][0].record(stream)
            world.enqueue(1, particles=True)
            ev[i][1].record(stream)
    world.sync()
    torch.cuda.synchronize()
    clk = clocks.stop()
    launches = fse.launch_counter() - l0
    gpu_ms = max_over_ranks(sum(a.elapsed_time(b) for a, b in ev), world_size)
    value = world_size * W * H * args.steps / (gpu_ms / 1e3) / 1e9
    # the same ticks replayed from 32-tick CUDA graphs (no flush inside a graph)
    g0, g1 = _ev(torch), _ev(torch)
    world.step(32, graph=True)
    torch.cuda.synchronize()
    n_graph = max(32, (args.steps // 32) * 32)
    g0.record(stream)
    world.step(n_graph, graph=True)
    g1.record(stream)
    world.sync()
    torch.cuda.synchronize()
    graph_ms = g0.elapsed_time(g1)
    cpu = None
    if rank == 0 and world_size == 1 and not args.no_cpu:
        cpu = cpu_baseline_world(W, H, seed, 0, 10.0)
    world.close()
    return _common(args, world_size, value, "Gcell/s", gpu_ms / args.steps,
                   "config0: one 512x512 world (mix in the top 60%, 8 rock rows), reference chunk size 128, "
                   "1000 ticks, plain per-world launch",
                   {"world": [W, H], "chunk": 128, "cell_iter": 3, "seed": seed,
                    "l2": "flushed between timed steps (512 MiB write outside the events)",
                    "graph32": {"ticks": n_graph, "ms_per_tick": round(graph_ms / n_graph, 4),
                                "value": round(W * H * n_graph / (graph_ms / 1e3) / 1e9, 4),
                                "note": "32-tick CUDA graph replay; no L2 flush inside a graph"}},
                   launches, clk, cpu=cpu)


def cpu_baseline_world(W, H, seed, gen_kind, budget_s):
    """The oracle's reference-order tick on all host cores on a bounded sample of a
    W x H world of the given generator (as many steps as fit the budget)."""
    from oracle import Oracle, OracleWorld

    o = Oracle()
    o.reset_materials()
    cores = os.cpu_count() or 1
    o.set_threads(cores)
    ow = OracleWorld(W, H, 128, 3, seed)
    ow.generate(gen_kind, seed)
    ow.step(1, 0)
    n, t0 = 0, time.perf_counter()
    while True:
        ow.step(1, 0)
        n += 1
        if time.perf_counter() - t0 > budget_s or n >= 1000:
            break
    dt = time.perf_counter() - t0
    return {"value": round(W * H * n / dt / 1e9, 6), "unit": "Gcell/s", "cores": cores, "kind": "port",
            "sample": "%d steps (tick + tickCells) of the %dx%d world, reference chunk order, after 1 warm-up step"
                      % (n, W, H)}


def config2_sizes(n, seed):
    rng = np.random.default_rng(seed)
    sides = np.arange(128, 2049, 64)
    return [(int(rng.choice(sides)), int(rng.choice(sides))) for _ in range(n)]


CONFIG2_WORLDS = 256
CONFIG2_SEED = 1234
CONFIG2_WORKLOAD = ("config2: 256 worlds, sides uniform in {128, 192, ..., 2048}, per-world seeds 1234+i, mix (30% "
                    "sand, 20% water, 10% gas, 15% rock, 25% air in the top 60%, 8 rock rows); batched launches "
                    "replayed from 32-tick CUDA graphs with the autotuned launch shape, against 256 plain per-world "
                    "launches")
# the worlds of config 2 the CPU legs time (every 32nd: 8 worlds, sizes spread over the range)
CONFIG2_CPU_SAMPLE = tuple(range(0, CONFIG2_WORLDS, 32))


def worlds_digest(worlds, fse):
    """blake2b over every world's planes (the pending diff only where the cell is a
    liquid, the only place it means anything) and particle list, in world order."""
    import hashlib

    soup = np.array([fse.material_get(i)[0] == fse.SOUP for i in range(fse.material_count())])
    h = hashlib.blake2b(digest_size=16)
    for w in worlds:
        st = w.state()
        for k in ("id", "colour", "scalar", "flags"):
            h.update(np.ascontiguousarray(st[k]).tobytes())
        h.update(np.where(soup[st["id"]], st["diff"], 0).astype(np.int32).tobytes())
        h.update(w.particles().tobytes())
    return h.hexdigest()


def bench_config2(args, rank, local_rank, world_size):
    """256 worlds of uneven sizes: batched launches replayed from 32-tick CUDA graphs
    with the autotuned launch shape, against the same worlds stepped one by one
    through their plain per-world launches (each world on its own stream). Both arms
    run the same warm-up and timed steps from the same generated worlds and must end
    in the same state (a digest of every plane and particle of every world). The
    colour-pass launches and the ticks inside the graphs are timed with CUDA events
    recorded by the graphs themselves (the roofline's launch time, the tick latency
    percentiles)."""
    import torch

    import falling_sand_engine_gb300 as fse

    from falling_sand_engine_gb300.sharding import shard_worlds

    fse.InitMaterials()
    fse.PushMaterials()
    # the 256 worlds are split across ranks by cell count (no data exchange); one
    # rank ticks them all
    all_sizes = config2_sizes(CONFIG2_WORLDS, CONFIG2_SEED)
    mine = shard_worlds([w * h for w, h in all_sizes], world_size)[rank]
    sizes = [all_sizes[i] for i in mine]
    cells = sum(w * h for w, h in sizes)
    total_cells = sum(w * h for w, h in all_sizes)

    def make():
        ws = []
        for i, (w, h) in zip(mine, sizes):
            wd = fse.World(w, h, chunk_size=128, cell_iter=3, seed=CONFIG2_SEED + i)
            wd.generate(fse.GEN_MIX, CONFIG2_SEED + i)
            ws.append(wd)
        for wd in ws:
            wd.sync()
        return ws

    worlds = make()
    batch = fse.Batch(worlds)
    if args.launch_shape is not None:
        # a fixed launch shape instead of the autotuner (profiling: under a profiler the
        # candidates' timings are not those of the plain run)
        batch.set_launch(args.launch_shape[0], args.launch_shape[1])
        choice = {"colour_ctas_per_sm": args.launch_shape[0], "particle_blocks": args.launch_shape[1],
                  "fixed": True}
    else:
        choice = batch.autotune()
    bstream = torch.cuda.ExternalStream(batch.stream)
    batch.step(args.warmup)
    batch.timing(True)
    batch.prepare_graphs(args.steps, 32)
    batch.sync()
    clocks = Clocks(local_rank)
    barrier(world_size)
    torch.cuda.synchronize()
    l0 = fse.launch_counter()
    e0, e1 = _ev(torch), _ev(torch)
    clocks.start()
    t0 = time.perf_counter()
    e0.record(bstream)
    batch.step(args.steps, graph_ticks=32)
    e1.record(bstream)
    batch.sync()
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    clk = clocks.stop()
    launches = fse.launch_counter() - l0
    pass_ms, pass_n, tick_ms = batch.timing(False)
    b_ms = max_over_ranks(e0.elapsed_time(e1), world_size)
    value = total_cells * args.steps / (b_ms / 1e3) / 1e9
    if args.batch_only:
        # the batched timed region alone (the launch list of the profiles is taken this way)
        return {"metric": METRIC, "value": round(value, 4), "unit": "Gcell/s", "steps": args.steps,
                "ms_per_step": round(b_ms / args.steps, 4), "gpu_launches": int(launches), "autotune": choice,
                "colour_pass_ms": round(pass_ms / max(pass_n, 1), 4), "note": "--batch-only: no other arm"}
    digest_b = worlds_digest(worlds, fse)

    # end to end through the C ABI with host buffers: every step uploads each
    # world's planes from pinned host memory, runs one step and reads the planes back
    batch.close()
    e2e = e2e_batch(worlds, fse, torch, cells, world_size, choice)
    for w in worlds:
        w.close()
    del worlds

    # the same worlds, plain per-world launches: start and end events join all streams.
    # Both colour shapes are timed (the default fused tick, and one CTA per chunk-pass
    # scheduled by the hardware, which packs 256 worlds launched side by side better)
    # and the faster is the comparison.
    def per_world_arm(shape):
        worlds = make()
        for w in worlds:
            w.set_launch(shape)
        streams = [torch.cuda.ExternalStream(w.stream) for w in worlds]
        for w in worlds:
            w.enqueue(args.warmup, particles=True)
        for w in worlds:
            w.sync()
        torch.cuda.synchronize()
        main = torch.cuda.current_stream()
        p0, p1 = _ev(torch), _ev(torch)
        p0.record(main)
        for s in streams:
            s.wait_event(p0)
        for _ in range(args.steps):
            for w in worlds:
                w.enqueue(1, particles=True)
        for s in streams:
            e = _ev(torch)
            e.record(s)
            main.wait_event(e)
        p1.record(main)
        torch.cuda.synchronize()
        for w in worlds:
            w.sync()
        ms = max_over_ranks(p0.elapsed_time(p1), world_size)
        digest = worlds_digest(worlds, fse)
        for w in worlds:
            w.close()
        return ms, digest

    arms = {shape: per_world_arm(shape) for shape in (0, 4)}
    best_shape = min(arms, key=lambda k: arms[k][0])
    p_ms, digest_p = arms[best_shape]
    per_world = total_cells * args.steps / (p_ms / 1e3) / 1e9

    peak, peak_kind = peaks()
    roof = colour_roofline(cells, args.steps, pass_ms, pass_n, peak, peak_kind, "colour_pass_config2",
                           "all %d worlds" % len(mine))
    roof["tick_frac"] = round(value * 1e9 * BYTES_PER_CELL_UPDATE / world_size / (peak * 1e9), 5)
    lat = {"p50": round(float(np.percentile(tick_ms, 50)), 3), "p99": round(float(np.percentile(tick_ms, 99)), 3),
           "max": round(float(tick_ms.max()), 3), "ticks": int(len(tick_ms)),
           "unit": "ms per batched tick (all worlds: tick + tickCells), CUDA events recorded inside the graphs"} \
        if len(tick_ms) else None
    cpu = None
    if rank == 0 and world_size == 1 and not args.no_cpu:
        cpu = cpu_baseline_config2(all_sizes, budget_s=20.0)
    sub1 = None
    if not args.no_config1:
        sub1 = bench_config1(args, rank, local_rank, world_size)
    out = _common(args, world_size, value, "Gcell/s", b_ms / args.steps, CONFIG2_WORKLOAD,
                  {"worlds": CONFIG2_WORLDS, "cells": total_cells, "worlds_this_rank": len(mine), "chunk": 128,
                   "cell_iter": 3, "autotune": choice, "graph_ticks": 32,
                   "l2": "inputs larger than L2 (%.2f GB of grid state)" % (cells * 15 / 1e9),
                   "parallelism": "worlds sharded across %d GPUs by cell count, no collective" % world_size
                   if world_size > 1 else "single GPU"},
                  launches, clk, e2e=e2e, cpu=cpu, scaling="strong")
    out.update({
        "roofline": roof, "tick_latency": lat, "wall_s": round(wall, 3),
        "per_world_launch": {"value": round(per_world, 4), "unit": "Gcell/s",
                             "ms_per_step": round(p_ms / args.steps, 4), "colour_shape": best_shape,
                             "ms_per_step_by_shape": {str(k): round(v[0] / args.steps, 4) for k, v in arms.items()},
                             "how": "each world's plain fse_world_enqueue on its own stream, same steps; the faster "
                                    "of colour shapes 0 (one CTA per chunk-pass) and 4 (fused tick)"},
        "batched_over_per_world": round(value / per_world, 3),
        "same_result": {"equal": digest_b == digest_p and arms[0][1] == arms[4][1], "digest": digest_b,
                        "what": "blake2b of every world's planes and particle list after warm-up + timed steps"},
        "config1": sub1,
    })
    return out


def e2e_worlds(worlds, step, torch, cells, world_size, path, steps=3):
    """The metric end to end through the C ABI: every step uploads each world's
    planes from pinned host memory, runs `step`, and reads every plane back."""
    pinned = []
    for w in worlds:
        st = w.state()
        host = {}
        for k, v in st.items():
            t = torch.empty(v.size, dtype={np.uint16: torch.int16, np.uint32: torch.int32, np.int32: torch.int32,
                                           np.uint8: torch.uint8}[v.dtype.type], pin_memory=True)
            a = t.numpy().view(v.dtype).reshape(v.shape)
            a[...] = v
            host[k] = (t, a)
        pinned.append(host)
    bi = sum(a.nbytes for host in pinned for (t, a) in host.values())
    for w in worlds:
        w.sync()
    t0 = time.perf_counter()
    for _ in range(steps):
        for w, host in zip(worlds, pinned):
            w.upload({k: a for k, (t, a) in host.items()})
        step()
        for w, host in zip(worlds, pinned):
            w.state(out={k: a for k, (t, a) in host.items()})
    dt = max_over_ranks(time.perf_counter() - t0, world_size)
    return {"value": round(world_size * cells * steps / dt / 1e9, 4), "unit": "Gcell/s",
            "h2d_bytes_per_step": int(bi), "d2h_bytes_per_step": int(bi), "steps": steps, "path": path}


def e2e_batch(worlds, fse, torch, cells, world_size, launch, steps=5, groups=4):
    """The batched metric end to end through the C ABI, the host copies overlapping
    the ticks: the worlds are split into `groups` batches of about equal cells, each
    on its own stream, and every step each batch copies its worlds' planes from its
    pinned host buffer (fse_batch_upload_all: one copy and a scatter kernel),
    enqueues one step (fse_batch_enqueue) and gathers the planes back into the buffer
    (fse_batch_download_all: a gather kernel and one copy); the step ends when every
    batch has synchronised (fse_batch_sync). While one batch ticks, the others'
    copies run."""
    bins = [[] for _ in range(groups)]
    load = [0] * groups
    for k in sorted(range(len(worlds)), key=lambda k: -worlds[k].width * worlds[k].height):
        g = load.index(min(load))
        bins[g].append(k)
        load[g] += worlds[k].width * worlds[k].height
    subs, bufs = [], []
    for ks in bins:
        if not ks:
            continue
        sb = fse.Batch([worlds[k] for k in sorted(ks)])
        sb.set_launch(launch["colour_ctas_per_sm"], launch["particle_blocks"])
        offs, total = sb.io_layout()
        t = torch.empty(total, dtype=torch.uint8, pin_memory=True)
        buf = t.numpy()
        for v, w in zip(sb.io_views(buf), sb.worlds):
            st = w.state()
            for key in v:
                v[key][...] = st[key]
        subs.append(sb)
        bufs.append((t, buf))
    total = sum(int(buf.nbytes) for _, buf in bufs)

    def one_step():
        for sb, (_, buf) in zip(subs, bufs):
            sb.upload_all(buf)
            sb.enqueue(1)
            sb.download_all(buf)
        for sb in subs:
            sb.sync()

    # one untimed round trip: the device staging buffers are allocated on first use
    one_step()
    t0 = time.perf_counter()
    for _ in range(steps):
        one_step()
    dt = max_over_ranks(time.perf_counter() - t0, world_size)
    for sb in subs:
        sb.close()
    return {"value": round(world_size * cells * steps / dt / 1e9, 4), "unit": "Gcell/s",
            "h2d_bytes_per_step": total, "d2h_bytes_per_step": total, "steps": steps,
            "path": "the worlds in %d batches of about equal cells, each on its own stream: fse_batch_upload_all "
                    "(its worlds' planes, one pinned host buffer) + fse_batch_enqueue + fse_batch_download_all, "
                    "then fse_batch_sync of every batch; one batch's copies overlap the others' ticks" % len(subs)}


def reference_timing_worlds(sizes, sample, steps, warm, budget_s):
    """The reference's own tick + tickCells, one world after another (each world
    ticked by its own pool of one worker per host core, as the reference ticks its
    one world), on the sampled worlds of a batch workload: (Gcell/s, steps per world,
    threads, cells sampled), or None when it cannot be compiled here."""
    from oracle import Oracle, OracleWorld
    from oracle.binding import build_reference_tick, reference_world_bench

    try:
        lib = build_reference_tick()
    except Exception:  # noqa: BLE001 - no compiler or sources: the port is timed instead
        lib = None
    if lib is None:
        return None
    o = Oracle()
    o.reset_materials()
    stone = o.find("STONE")
    cores = os.cpu_count() or 1
    secs, work, n_min, sampled = 0.0, 0, None, 0
    for i in sample:
        W, H = sizes[i]
        ow = OracleWorld(W, H, 128, 3, CONFIG2_SEED + i)
        ow.generate(0, CONFIG2_SEED + i)
        st = ow.state()
        # The reference's tick walks whole 128 x 128 chunks (world.cpp:1078-1087) and
        # its worlds are whole chunks; a world whose side is not a multiple of 128 is
        # given to it padded with rock to the next chunk edge (cells that never move,
        # as the library's out-of-world cells are solid), and the padded cells count
        # as cell-updates of the reference.
        W2, H2 = -(-W // 128) * 128, -(-H // 128) * 128
        ids = np.full((H2, W2), stone, np.uint16)
        cols = np.full((H2, W2), 0x808080, np.uint32)
        temps = np.zeros((H2, W2), np.int32)
        ids[:H, :W] = st["id"]
        cols[:H, :W] = st["colour"]
        temps[:H, :W] = ow.temperature()
        s, n = reference_world_bench(lib, o, ids, cols, temps, _np_particles(0, W2, H2, CONFIG2_SEED + i), 3,
                                     CONFIG2_SEED + i, cores, warm, steps, budget_s / len(sample))
        secs += s
        work += W2 * H2 * n
        sampled += W2 * H2
        n_min = n if n_min is None else min(n_min, n)
    return work / secs / 1e9, n_min, cores, sampled


def cpu_baseline_config2(sizes, budget_s=20.0):
    """The reference's own tick + tickCells on the host cores, on a bounded sample of
    the batch: every 32nd world, one step each after one warm-up step."""
    ref = reference_timing_worlds(sizes, CONFIG2_CPU_SAMPLE, 1, 1, budget_s)
    if ref is None:
        return None
    value, n, cores, sampled = ref
    return {"value": round(value, 6), "unit": "Gcell/s", "cores": cores, "kind": "reference",
            "sample": "worlds %s of the 256 (%d cells, padded with rock to whole 128-cell chunks), %d step(s) "
                      "each after 1 warm-up step, one world after another; " % (list(CONFIG2_CPU_SAMPLE), sampled, n)
                      + REF_NOTE % cores}


def bench_config3(args, rank, local_rank, world_size):
    """16384x16384 world, 8 materials with Zipf frequencies, 200 axis-aligned OBJECT
    boxes stamped before every tick, taken back after it, and the OBJECT mask
    (1 bit per cell) exported to the host every tick."""
    import torch

    import falling_sand_engine_gb300 as fse

    W = H = 16384
    seed = 1234 + rank
    fse.InitMaterials()
    fse.PushMaterials()
    stream = torch.cuda.Stream()
    world = fse.World(W, H, chunk_size=128, cell_iter=3, seed=seed, particle_capacity=24 << 20,
                      spawn_capacity=16 << 20, stream=stream.cuda_stream)
    world.generate(fse.GEN_ZIPF8, seed)
    rng = np.random.default_rng(seed)
    bodies = np.zeros(200, fse.BODY_DTYPE)
    bodies["w"] = rng.integers(8, 65, 200)
    bodies["h"] = rng.integers(8, 65, 200)
    bodies["x"] = rng.uniform(0, W - 64, 200).astype(np.float32)
    bodies["y"] = rng.uniform(0, H - 64, 200).astype(np.float32)
    bodies["cos_a"] = 1.0
    bodies["id"] = fse.material_find("GENERIC_OBJECT")
    bodies["colour"] = 0xFF808080
    mask = torch.empty((W * H + 7) // 8, dtype=torch.uint8, pin_memory=True).numpy()

    def one(timed=None):
        world.object_stamp(bodies)
        if timed is not None:
            timed[0].record(stream)
        world.enqueue(1, particles=True)
        if timed is not None:
            timed[1].record(stream)
        world.object_mask(out=mask)
        world.object_readback(bodies)

    for _ in range(args.warmup):
        one()
    ev = [(_ev(torch), _ev(torch)) for _ in range(args.steps)]
    clocks = Clocks(local_rank)
    barrier(world_size)
    torch.cuda.synchronize()
    l0 = fse.launch_counter()
    clocks.start()
    t0 = time.perf_counter()
    with torch.cuda.stream(stream):
        for i in range(args.steps):
            one(ev[i])
    world.sync()
    wall = max_over_ranks(time.perf_counter() - t0, world_size)
    clk = clocks.stop()
    launches = fse.launch_counter() - l0
    tick_ms = max_over_ranks(sum(a.elapsed_time(b) for a, b in ev), world_size)
    cells = W * H
    value = world_size * cells * args.steps / (tick_ms / 1e3) / 1e9
    n_obj = int(np.unpackbits(mask).sum())
    world.close()
    e2e = {"value": round(world_size * cells * args.steps / wall / 1e9, 4), "unit": "Gcell/s",
           "h2d_bytes_per_step": int(2 * bodies.nbytes), "d2h_bytes_per_step": int(mask.nbytes + 2 * bodies.nbytes),
           "path": "fse_object_stamp + fse_world_enqueue + fse_object_mask_export + fse_object_readback per tick"}
    return _common(args, world_size, value, "Gcell/s", tick_ms / args.steps,
                   "config3: one 16384x16384 world (Zipf-8 materials) with 200 OBJECT boxes stamped, ticked, "
                   "exported as a 1-bit mask and taken back every tick",
                   {"world": [W, H], "bodies": 200, "chunk": 128, "cell_iter": 3, "seed": seed,
                    "l2": "inputs larger than L2 (4 GB of grid state)",
                    "object_cells_last_mask": n_obj,
                    "objects_and_export_ms_per_tick": round(wall * 1e3 / args.steps - tick_ms / args.steps, 3)},
                   launches, clk, e2e=e2e)


def serve_window(fse, srv, slot_of, cells, rate, window_s, rng):
    """Offer Poisson arrivals at `rate` req/s for window_s seconds (requests of 1-16
    ticks on uniformly drawn worlds) and serve them until all are done. Returns the
    request latencies (ms, arrival to device completion), the served cell-updates,
    the wall time (s), the scheduler steps and the device time of each step (ms)."""
    n = rng.poisson(rate * window_s)
    arr = np.sort(rng.uniform(0.0, window_s * 1e6, n))
    keys = sorted(slot_of)
    req_slot = np.array([slot_of[keys[int(k)]] for k in rng.integers(0, len(keys), n)], np.int64)
    req_ticks = rng.integers(1, 17, n)
    srv.tick_times()
    base = srv.now_us()
    nxt, lat, ids, steps = 0, [], {}, 0
    while len(lat) < n:
        now = srv.now_us() - base
        while nxt < n and arr[nxt] <= now:
            rid = srv.submit(int(req_slot[nxt]), int(req_ticks[nxt]), arrival_us=base + arr[nxt])
            ids[rid] = nxt
            nxt += 1
        if srv.step() == 0 and nxt < n:
            time.sleep(max(0.0, (arr[nxt] - (srv.now_us() - base)) / 1e6))
        steps += 1
        got, t_done = srv.poll()
        for rid, td in zip(got, t_done):
            k = ids.pop(int(rid))
            lat.append((td - base - arr[k]) / 1e3)
    wall = (srv.now_us() - base) / 1e6
    work = float(sum(cells[int(sl)] * int(t) for sl, t in zip(req_slot, req_ticks)))
    return np.asarray(lat, float), work, wall, steps, srv.tick_times()


def _pct(x):
    x = np.asarray(x, float)
    if len(x) == 0:
        return None
    return {"p50": round(float(np.percentile(x, 50)), 3), "p99": round(float(np.percentile(x, 99)), 3),
            "max": round(float(x.max()), 3), "n": int(len(x))}


def bench_config4(args, rank, local_rank, world_size, window_s=1.0):
    """Serving: 1000 worlds (sides uniform in {256, 320, ..., 4096}) registered with
    a server under a 120 GB HBM budget (worlds beyond it would be parked in host
    memory and restored on admission); requests of 1-16 ticks arrive as a Poisson
    process at 2000 req/s for window_s seconds and are served by continuous batching
    (steps pipelined on the device) until all are done. A second window offers
    about half the measured capacity, so the latency below capacity is seen too.
    Reports throughput and p50/p99 of request latency and of the batched tick."""
    import torch

    import falling_sand_engine_gb300 as fse

    from falling_sand_engine_gb300.sharding import shard_worlds

    fse.InitMaterials()
    fse.PushMaterials()
    # the same 1000 worlds on every rank; each rank serves the worlds of its shard
    # (split by cell count) and draws its requests among them
    rng = np.random.default_rng(1234)
    sides = np.arange(256, 4097, 64)
    dims = [(int(rng.choice(sides)), int(rng.choice(sides))) for _ in range(1000)]
    mine = shard_worlds([w * h for w, h in dims], world_size)[rank]
    srv = fse.Server(120 << 30, 1000)
    srv.set_depth(3)
    slot_of, cells = {}, {}
    t_add = time.perf_counter()
    for i in mine:
        w, h = dims[i]
        s = srv.add_world(w, h, fse.GEN_MIX, 1234 + i, seed=1234 + i,
                          particle_capacity=max(65536, w * h // 32), spawn_capacity=max(65536, w * h // 64))
        slot_of[i] = s
        cells[s] = w * h
    t_add = time.perf_counter() - t_add
    setup = srv.stats()
    # warm-up: one tick of a few worlds
    for s in list(slot_of.values())[:4]:
        srv.submit(s, 1)
    while srv.step() > 0:
        pass
    srv.poll()
    rq = np.random.default_rng(4321 + rank)
    clocks = Clocks(local_rank)
    torch.cuda.synchronize()
    l0 = fse.launch_counter()
    clocks.start()
    lat, work, wall, steps, tick = serve_window(fse, srv, slot_of, cells, 2000.0 / world_size, window_s, rq)
    clk = clocks.stop()
    launches = fse.launch_counter() - l0
    wall = max_over_ranks(wall, world_size)
    work_all = sum(gather_objects(work, world_size))
    lat = np.concatenate([np.asarray(x, float) for x in gather_objects(lat.tolist(), world_size)])
    value = work_all / wall / 1e9
    # below capacity: offer about half of what was just served per second
    mean_work = work_all / max(len(lat), 1)
    rate_lo = max(1.0, 0.5 * value * 1e9 / max(mean_work, 1.0))
    lat_lo, work_lo, wall_lo, steps_lo, tick_lo = serve_window(fse, srv, slot_of, cells, rate_lo / world_size,
                                                               max(window_s, 2.0), rq)
    lat_lo = np.concatenate([np.asarray(x, float) for x in gather_objects(lat_lo.tolist(), world_size)])
    st = srv.stats()
    bytes_used = srv.bytes_in_use()
    srv.close()
    return _common(args, world_size, value, "Gcell/s", wall * 1e3 / max(steps, 1),
                   "config4: serving 1000 worlds (sides uniform in {256, ..., 4096}), Poisson arrivals at "
                   "2000 req/s of 1-16 ticks for %.1f s, continuous batching with pipelined steps, "
                   "120 GB HBM admission budget" % window_s,
                   {"worlds": 1000, "worlds_this_rank": len(slot_of), "requests": int(len(lat)),
                    "worlds_parked_at_setup": setup["parked"], "worlds_restored": st["restored"],
                    "hbm_bytes_resident": int(bytes_used), "world_setup_s": round(t_add, 2),
                    "latency_ms": _pct(lat), "tick_ms": _pct(tick),
                    "offered_gcell_s": round(float(mean_work * 2000.0 / 1e9), 2),
                    "below_capacity": {"rate_req_s": round(rate_lo, 1), "requests": int(len(lat_lo)),
                                       "offered_gcell_s": round(float(mean_work * rate_lo / 1e9), 2),
                                       "served_gcell_s": round(work_lo / wall_lo / 1e9, 3),
                                       "latency_ms": _pct(lat_lo), "tick_ms": _pct(tick_lo)},
                    "steps_in_flight_max": st["max_in_flight"],
                    "served_cell_updates": work_all, "wall_s": round(wall, 2), "scheduler_steps": steps,
                    "timing": "host clock from the first arrival to the last device completion (the arrival "
                              "window plus the drain), max over ranks; latencies end at the device timestamp "
                              "of the step that ran the request's last tick",
                    "parallelism": "worlds sharded across %d GPUs by cell count, no collective" % world_size},
                   launches, clk, scaling="strong")


def colour_roofline(cells, ticks, pass_ms, pass_n, peak, peak_kind, traffic_key, what):
    """The colour pass against the HBM roofline: 22 B per cell-update, a tick being
    12 launches (one colour of one iteration each) or one fused launch of all 12."""
    per_tick = max(1, int(round(pass_n / max(ticks, 1))))
    avg_s = (pass_ms / max(pass_n, 1)) / 1e3
    units = cells / per_tick
    achieved = BYTES_PER_CELL_UPDATE * units / avg_s / 1e9
    fused = per_tick == 1
    return {"bound": "hbm", "achieved": round(achieved, 2), "peak": peak, "unit": "GB/s",
            "frac": round(achieved / peak, 4), "traffic": profile_traffic(traffic_key + ("_fused" if fused else "")),
            "kernel": "k_colour_pass<2, fused>" if fused else "k_colour_pass<2>", "peak_kind": peak_kind,
            "launch_ms_avg": round(pass_ms / max(pass_n, 1), 4), "launches_timed": int(pass_n),
            "units": "22 B per cell-update; one launch = %s over %s (%d cells%s)"
                     % ("every pass of the tick" if fused else "one colour of one iteration", what, cells,
                        "" if fused else " / 12")}


def gather_objects(obj, world_size):
    """Every rank's obj, in rank order (a host-side exchange of results, not data)."""
    if world_size == 1:
        return [obj]
    import torch.distributed as dist

    out = [None] * world_size
    dist.all_gather_object(out, obj)
    return out


def profile_traffic(name):
    try:
        with open(os.path.join(ROOT, "profiles", "traffic.json")) as f:
            return json.load(f).get(name)
    except Exception:
        return None


def barrier(world_size):
    if world_size > 1:
        import torch.distributed as dist

        dist.barrier()


def max_over_ranks(v, world_size):
    if world_size == 1:
        return v
    import torch
    import torch.distributed as dist

    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(v)], device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# ------------------------------------------------------------ reference arm
REF_NOTE = ("the reference's own world::tick and world::tickCells (source/engine/world.cpp:1036-1948, 2030-2195), "
            "compiled unchanged from the extracted sources (oracle/ref_tick.cpp) with its chunk tasks on a pool of "
            "%d worker threads; rand() draws the counter RNG, texture tile factories are constants")


def reference_timing(W, H, seed, steps, warm, budget_s):
    """The reference's own tick + tickCells on the workload, on all host cores:
    (Gcell/s, steps timed, threads), or None when it cannot be compiled here."""
    from oracle import Oracle, OracleWorld
    from oracle.binding import build_reference_tick, reference_world_bench

    try:
        lib = build_reference_tick()
    except Exception:  # noqa: BLE001 - no compiler or sources: the port is timed instead
        lib = None
    if lib is None:
        return None
    o = Oracle()
    o.reset_materials()
    cores = os.cpu_count() or 1
    ow = OracleWorld(W, H, 128, 3, seed)
    ow.generate(0, seed)
    st = ow.state()
    secs, n = reference_world_bench(lib, o, st["id"], st["colour"], ow.temperature(),
                                    _np_particles(1_000_000, W, H, seed), 3, seed, cores, warm, steps, budget_s)
    return W * H * n / secs / 1e9, n, cores


def reference_arm(args, rank, world_size):
    if rank != 0:
        return None
    if args.workload == 2:
        return reference_arm_config2(args, world_size)
    from oracle import Oracle, OracleWorld

    W, H = 4096, 2048
    warm = min(args.warmup, 3)
    ref = reference_timing(W, H, 1234, args.steps, warm, REF_BUDGET_S)
    if ref is not None:
        value, n, cores = ref
        sample = ("%d timed steps (tick + tickCells) of the 4096x2048 world with 1M particles after %d warm-up "
                  "(%d requested; the timed region is capped at %.0f s)" % (n, warm, args.steps, REF_BUDGET_S))
        return {
            "impl": "reference", "metric": METRIC, "value": round(value, 6), "unit": "Gcell/s", "n_gpus": world_size,
            "steps": n, "warmup": warm, "ms_per_step": round(W * H / (value * 1e9) * 1e3, 3),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int32+f32",
            "data": "synthetic",
            "config": {"workload": "config1: one 4096x2048 world + 1M free particles", "world": [W, H],
                       "particles": 1_000_000, "chunk": 128, "cell_iter": 3, "impl_note": REF_NOTE % cores},
            "cpu_baseline": {"value": round(value, 6), "unit": "Gcell/s", "cores": cores, "kind": "reference",
                             "sample": sample},
            "e2e": {"value": round(value, 6), "unit": "Gcell/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        }
    o = Oracle()
    o.reset_materials()
    cores = os.cpu_count() or 1
    o.set_threads(cores)
    ow = OracleWorld(W, H, 128, 3, 1234)
    ow.generate(0, 1234)
    ow.set_particles(_np_particles(1_000_000, W, H, 1234))
    # a step of the CPU tick takes about a second: warm up with at most 3 steps and
    # time at most REF_BUDGET_S seconds of the K requested steps
    warm = min(args.warmup, 3)
    for _ in range(warm):
        ow.step(1, 0)
    n, t0 = 0, time.perf_counter()
    while n < args.steps:
        ow.step(1, 0)
        n += 1
        if time.perf_counter() - t0 > REF_BUDGET_S:
            break
    dt = time.perf_counter() - t0
    value = W * H * n / dt / 1e9
    sample = ("%d timed steps (tick + tickCells) of the 4096x2048 world with 1M particles after %d warm-up "
              "(%d requested; the timed region is capped at %.0f s)" % (n, warm, args.steps, REF_BUDGET_S))
    return {
        "impl": "reference", "metric": METRIC, "value": round(value, 6), "unit": "Gcell/s", "n_gpus": world_size,
        "steps": n, "warmup": warm, "ms_per_step": round(dt * 1e3 / n, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int32+f32", "data": "synthetic",
        "config": {"workload": "config1: one 4096x2048 world + 1M free particles", "world": [W, H],
                   "particles": 1_000_000, "chunk": 128, "cell_iter": 3,
                   "impl_note": "CPU restatement of world::tick/tickCells in the reference chunk order "
                                "(the reference's own functions could not be compiled on this machine)"},
        "cpu_baseline": {"value": round(value, 6), "unit": "Gcell/s", "cores": cores, "kind": "port",
                         "sample": sample},
        "e2e": {"value": round(value, 6), "unit": "Gcell/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


# the worlds the reference arm times on the batch workload (every 16th: 16 worlds)
CONFIG2_REF_SAMPLE = tuple(range(0, CONFIG2_WORLDS, 16))


def reference_arm_config2(args, world_size):
    """The reference's own world::tick + world::tickCells on the batch workload: the
    same world sizes, seeds and generator (the oracle's generator, equal to the
    library's cell for cell), every 16th world, each world ticked by its own pool of
    one worker per host core, one world after another (the reference engine ticks
    its one world this way). At most 3 warm-up steps and REF_BUDGET_S seconds of
    timed steps are spread over the sampled worlds."""
    sizes = config2_sizes(CONFIG2_WORLDS, CONFIG2_SEED)
    warm = min(args.warmup, 3)
    ref = reference_timing_worlds(sizes, CONFIG2_REF_SAMPLE, args.steps, warm, REF_BUDGET_S)
    if ref is None:
        return {"impl": "reference", "unavailable": "the reference's tick sources are not present to compile"}
    value, n, cores, sampled = ref
    sample = ("worlds %s of the 256 (%d cells, padded with rock to whole 128-cell chunks), at least %d timed step(s) each (tick + tickCells) after %d "
              "warm-up (%d requested; the timed region is capped at %.0f s over all sampled worlds)"
              % (list(CONFIG2_REF_SAMPLE), sampled, n, warm, args.steps, REF_BUDGET_S))
    return {
        "impl": "reference", "metric": METRIC, "value": round(value, 6), "unit": "Gcell/s", "n_gpus": world_size,
        "steps": n, "warmup": warm, "ms_per_step": round(sampled / (value * 1e9) * 1e3, 3),
        "higher_is_better": True, "scaling": "strong", "vs_baseline": None, "dtype": "int32+f32",
        "data": "synthetic",
        "config": {"workload": CONFIG2_WORKLOAD, "worlds": CONFIG2_WORLDS, "chunk": 128, "cell_iter": 3,
                   "same_config": True,
                   "same_inputs": "world sizes and seeds of config2_sizes(256, 1234); cells from the oracle's "
                                  "generator, which equals the library's GEN_MIX bit for bit (tests/test_gpu_parity.py "
                                  "and smoke())",
                   "impl_note": REF_NOTE % cores},
        "cpu_baseline": {"value": round(value, 6), "unit": "Gcell/s", "cores": cores, "kind": "reference",
                         "sample": sample},
        "e2e": {"value": round(value, 6), "unit": "Gcell/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def _np_particles(n, w, h, seed):
    from oracle import PARTICLE_DTYPE

    rng = np.random.default_rng(seed)
    p = np.zeros(n, PARTICLE_DTYPE)
    p["x"] = rng.uniform(0, w, n).astype(np.float32)
    p["y"] = rng.uniform(0, h, n).astype(np.float32)
    p["vx"] = rng.normal(0.0, 2.0, n).astype(np.float32)
    p["vy"] = rng.normal(0.0, 2.0, n).astype(np.float32)
    p["ay"] = np.float32(0.1)
    p["fade_time"] = 60
    p["id"] = 2
    p["colour"] = 0xFFFFFFFF
    return p


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=None,
                    help="timed steps (default: the workload's tick count, 200 for the default batch workload)")
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="fse", choices=["fse", "reference"])
    ap.add_argument("--workload", type=int, default=2, choices=[0, 1, 2, 3, 4])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--batch-only", action="store_true",
                    help="batch workload: time the batched steps only (no per-world arm, digests, e2e or CPU legs)")
    ap.add_argument("--no-config1", action="store_true",
                    help="batch workload: skip the 4096x2048 single-world line reported beside it")
    ap.add_argument("--launch-shape", type=int, nargs=2, default=None, metavar=("COLOUR", "PARTICLE_BLOCKS"),
                    help="config 2: this batch launch shape instead of the autotuner's choice (for profiling)")
    ap.add_argument("--only", default=None, choices=["render", "temperature", "pack", "reference_order"],
                    help="run only one side measurement of the 4096x2048 workload (for profiling), print its dict")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.steps is None:
        args.steps = WORKLOAD_TICKS[args.workload]
    rank, local_rank, world_size = dist_info()

    if args.impl == "reference":
        out = reference_arm(args, rank, world_size)
        if out is not None:
            print(json.dumps(out))
        return

    import torch

    torch.cuda.set_device(local_rank)
    if world_size > 1:
        import torch.distributed as dist

        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group("nccl", device_id=torch.device("cuda", local_rank))
    if args.only:
        import falling_sand_engine_gb300 as fse

        fse.InitMaterials()
        fse.PushMaterials()
        fn = {"render": render_config1, "temperature": temperature_config1, "pack": pack_config1,
              "reference_order": reference_order_config1}[args.only]
        print(json.dumps(fn(fse, torch, 4096, 2048, 1234, 1_000_000)))
        return
    run = {0: bench_config0, 1: bench_config1, 2: bench_config2, 3: bench_config3, 4: bench_config4}[args.workload]
    out = run(args, rank, local_rank, world_size)
    if rank == 0 and out is not None:
        print(json.dumps(out))
    if world_size > 1:
        import torch.distributed as dist

        dist.destroy_process_group()


if __name__ == "__main__":
    main()
