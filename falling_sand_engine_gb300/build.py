"""Builds the in-tree CUDA library libfse.so for sm_103a with nvcc."""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libfse.so")
SOURCES = ["fse_tick.cu", "fse_particles.cu", "fse_objects.cu", "fse_api.cu", "fse_batch.cu", "fse_server.cu", "fse_noalloc.cu",
           "fse_render.cu", "fse_islands.cu", "fse_temperature.cu", "fse_tick_temp.cu",
           "fse_pack.cu", "fse_tiles.cu", "fse_tick_seq.cu", "fse_tick_f32.cu", "fse_tick_f32_seq.cu",
           "fse_tick_pair.cu", "fse_tick_pair_f32.cu", "fse_tick_fused.cu", "fse_tick_fused_f32.cu"]
# sources that include another source
SOURCE_DEPS = {"fse_tick_temp.cu": ["fse_tick.cu"], "fse_tick_seq.cu": ["fse_tick.cu"],
               "fse_tick_f32.cu": ["fse_tick.cu"], "fse_tick_f32_seq.cu": ["fse_tick.cu"],
               "fse_tick_pair.cu": ["fse_tick.cu"], "fse_tick_pair_f32.cu": ["fse_tick.cu"],
               "fse_tick_fused.cu": ["fse_tick.cu"], "fse_tick_fused_f32.cu": ["fse_tick.cu"]}
HEADERS = ["fse_internal.cuh", "fse_host.cuh"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr"]


def _nvcc():
    cand = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    return cand if os.path.exists(cand) else "nvcc"


def _stale(out, deps):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose=False, force=False, extra=()):
    os.makedirs(OUT_DIR, exist_ok=True)
    nvcc = _nvcc()
    headers = [os.path.join(CSRC, h) for h in HEADERS] + [os.path.join(HERE, "..", "include", "fse.h")]
    objs, jobs = [], []
    for src in SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OUT_DIR, src.replace(".cu", ".o"))
        objs.append(o)
        deps = [os.path.join(CSRC, d) for d in SOURCE_DEPS.get(src, [])]
        if force or _stale(o, [s] + deps + headers):
            cmd = [nvcc, *ARCH, *FLAGS, *extra, "-c", s, "-o", o]
            if verbose:
                cmd.insert(1, "-Xptxas=-v")
            jobs.append(cmd)

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        return cmd, r

    with ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        for cmd, r in ex.map(run, jobs):
            if verbose or r.returncode:
                sys.stderr.write(r.stdout + r.stderr)
            if r.returncode:
                raise RuntimeError("nvcc failed: " + " ".join(cmd))
    if force or jobs or _stale(LIB, objs):
        cmd = [nvcc, *ARCH, "-shared", "-o", LIB, *objs, "-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode:
            sys.stderr.write(r.stdout + r.stderr)
            raise RuntimeError("link failed")
    return LIB


if __name__ == "__main__":
    build(verbose="-v" in sys.argv, force="-f" in sys.argv)
    print(LIB)
