"""Builds the CUDA product library csrc/_build/libcanvaz_film.so (sm_103a).

Each translation unit is compiled by nvcc in parallel
(-gencode arch=compute_103a,code=sm_103a, -O3, -lineinfo), then linked into a
shared library with the C ABI of include/canvaz_film.h.  No cmake, no torch.
Usage: python build.py [--force] [--verbose]
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
CSRC = HERE / "csrc"
OUT = CSRC / "_build"
LIB = OUT / "libcanvaz_film.so"
SOURCES = ["capi.cu", "capi_batch.cu", "film_kernels.cu", "film_noalloc.cu", "resolve.cu", "snapshot.cu", "deposit.cu", "cg.cu",
           "relief.cu", "render.cu"]
HEADERS = ["film_device.cuh", "strata_device.cuh", "strata_lane.cuh", "film_kernels.h", "film_handle.h", "tma.cuh"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
         "--expt-relaxed-constexpr"]
# Per-file device flags.  The deposit pass decides sample by sample whether a
# lattice point is inside a ribbon (cut planes, x < 1): it keeps one rounding
# per operation, as the reference's f32 host code and the oracle do, so no
# fused multiply-add moves a sample across those edges.
# The renderer's fragment (render.cu) follows the shader's f32 arithmetic the
# same way, so that its image is the shader's up to the last bits of the
# transcendental functions.
FILE_FLAGS = {"deposit.cu": ["--fmad=false"], "render.cu": ["--fmad=false"]}


def nvcc():
    p = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(p).exists():
        raise FileNotFoundError("nvcc not found")
    return p


def _stale(target, deps):
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build(force=False, verbose=False, extra=()):
    OUT.mkdir(exist_ok=True)
    hdrs = [CSRC / h for h in HEADERS] + [HERE.parent / "include" / "canvaz_film.h"]
    objs, jobs = [], []
    for s in SOURCES:
        src = CSRC / s
        obj = OUT / (Path(s).stem + ".o")
        objs.append(obj)
        if force or _stale(obj, [src] + hdrs):
            cmd = [nvcc(), *ARCH, *FLAGS, *FILE_FLAGS.get(s, []), *extra, "-c", str(src), "-o", str(obj)]
            if verbose:
                cmd.insert(1, "-Xptxas=-v")
            jobs.append(cmd)
    with cf.ThreadPoolExecutor(max_workers=max(len(jobs), 1)) as ex:
        for r in ex.map(lambda c: subprocess.run(c, capture_output=True, text=True), jobs):
            if r.returncode != 0 or verbose:
                sys.stderr.write(r.stdout + r.stderr)
            if r.returncode != 0:
                raise RuntimeError("nvcc failed: %s" % " ".join(r.args))
    if force or jobs or not LIB.exists():
        tmp = str(LIB) + ".tmp"
        cmd = [nvcc(), *ARCH, "-shared", "-o", tmp, *map(str, objs), "-lcudart"]
        subprocess.run(cmd, check=True)
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="--verbose" in sys.argv))
