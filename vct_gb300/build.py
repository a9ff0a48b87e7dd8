"""Build recipe of the CUDA library `vct_gb300/libvct.so` (sm_103a).

Every translation unit is compiled in parallel straight with nvcc / g++
(no cmake, no torch extension machinery) and linked into one shared library
that exports the C ABI of include/vct.h.

Every kernel translation unit is compiled with --fmad=false so that no
multiply-add is contracted behind the source's back: the rasterising,
voxelising, normalising, injecting and mip filtering kernels are bit-exact
against the CPU oracle, and the cone tracer writes each of its fused
multiply-adds explicitly, so that every instantiation of it (one scene, a
batch of scenes) rounds the same way.
"""

from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libvct.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
               "-I", os.path.join(ROOT, "include")] + ARCH

# (source, extra nvcc flags)
CUDA_SOURCES = [
    ("voxelize.cu", ["--fmad=false"]),
    ("volume.cu", ["--fmad=false"]),
    ("raster.cu", ["--fmad=false"]),
    ("trace.cu", ["--fmad=false"]),
    ("static_scratch.cu", []),
    ("learned.cu", ["--fmad=false"]),
    ("shade.cu", ["--fmad=false"]),
]
CXX_SOURCES = ["capi.cpp", "batch.cpp", "learned_capi.cpp"]


def nvcc_path() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libvct.so")


def cuda_home(nvcc: str) -> str:
    return os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))


def _run(cmd: list[str]) -> tuple[list[str], int, str]:
    p = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    return cmd, p.returncode, p.stdout


def _stale(out: str, deps: list[str]) -> bool:
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False, ptxas_info: bool = False, force: bool = False) -> str:
    """Compile every TU (in parallel) and link libvct.so. Returns its path."""
    nvcc = nvcc_path()
    home = cuda_home(nvcc)
    os.makedirs(BUILD, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    headers.append(os.path.join(ROOT, "include", "vct.h"))
    jobs, objs = [], []
    for src, extra in CUDA_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src + ".o")
        objs.append(o)
        flags = list(extra)
        if ptxas_info:
            flags += ["-Xptxas", "-v"]
        if force or ptxas_info or _stale(o, [s] + headers):
            jobs.append([nvcc, "-c", s, "-o", o] + NVCC_COMMON + flags)
    for src in CXX_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src + ".o")
        objs.append(o)
        if force or _stale(o, [s] + headers):
            jobs.append([os.environ.get("CXX", "g++"), "-c", s, "-o", o, "-O2", "-std=c++17", "-fPIC",
                         "-ffp-contract=off", "-Wall", "-I", os.path.join(home, "include"),
                         "-I", os.path.join(ROOT, "include")])
    with ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        results = list(ex.map(_run, jobs))
    failed = [r for r in results if r[1] != 0]
    for cmd, rc, out in results:
        if verbose or rc != 0 or ptxas_info:
            sys.stderr.write(" ".join(cmd) + "\n" + out)
    if failed:
        raise RuntimeError(f"libvct build failed ({len(failed)} translation unit(s)); see output above")
    if force or jobs or _stale(LIB, objs):
        cmd = [nvcc, "-shared", "-o", LIB] + objs + ARCH + ["-Xcompiler", "-fPIC"]
        _, rc, out = _run(cmd)
        if rc != 0:
            sys.stderr.write(" ".join(cmd) + "\n" + out)
            raise RuntimeError("libvct link failed")
    return LIB


if __name__ == "__main__":
    build(verbose="-v" in sys.argv, ptxas_info="--ptxas" in sys.argv, force="--force" in sys.argv)
    print(LIB)
