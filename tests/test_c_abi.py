"""include/vct.h from plain C: a C99 program compiled with -pedantic -Werror
and linked against libvct.so runs the calls that need no GPU (ABI version,
status strings, struct layouts, reference defaults, validation before
device work)."""

from __future__ import annotations

import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIBDIR = os.path.join(ROOT, "vct_gb300")


@pytest.mark.skipif(shutil.which("gcc") is None, reason="no C compiler")
def test_header_is_c99_and_the_library_links(tmp_path):
    lib = os.path.join(LIBDIR, "libvct.so")
    if not os.path.exists(lib):
        pytest.skip("libvct.so not built")
    exe = str(tmp_path / "abi_check")
    cmd = ["gcc", "-std=c99", "-pedantic", "-Wall", "-Wextra", "-Werror", "-I", os.path.join(ROOT, "include"),
           os.path.join(ROOT, "tests", "c", "abi_check.c"), "-L", LIBDIR, "-lvct", "-Wl,-rpath," + LIBDIR, "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "abi_check ok" in r.stdout


def _cuda_include() -> str | None:
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    inc = os.path.join(os.path.dirname(os.path.dirname(os.path.realpath(nvcc))), "include")
    return inc if os.path.exists(os.path.join(inc, "cuda_runtime.h")) else None


@pytest.mark.skipif(shutil.which("g++") is None or _cuda_include() is None, reason="no C++ compiler or CUDA headers")
def test_record_slots_match_the_kernels_layout(tmp_path):
    """The accumulator-record slot that the kernels use (record_slot) equals
    the exported vct_record_slot and api.record_slots, which
    read_accumulators inverts; the map is a permutation whose 128-byte lines
    (4 records) are 2 x 2 blocks in x, y."""
    import numpy as np

    from vct_gb300.api import record_slots

    src = tmp_path / "slots.cpp"
    src.write_text('#include "vct_internal.h"\n#include <cstdio>\n#include <cstdlib>\n'
                   "int main(int argc, char** argv) {\n"
                   "    const int n = atoi(argv[1]);\n"
                   "    for (long long v = 0; v < (long long)n * n * n; ++v) {\n"
                   "        if (vct::record_slot(v, n) != vct_record_slot(v, n)) return 1;\n"
                   "        printf(\"%lld\\n\", vct::record_slot(v, n));\n"
                   "    }\n"
                   "}\n")
    exe = str(tmp_path / "slots")
    lib = os.path.join(LIBDIR, "libvct.so")
    if not os.path.exists(lib):
        pytest.skip("libvct.so not built")
    cmd = ["g++", "-std=c++17", "-I", os.path.join(ROOT, "vct_gb300", "csrc"), "-I", _cuda_include(), str(src),
           "-L", LIBDIR, "-lvct", "-Wl,-rpath," + LIBDIR, "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    for n in (16, 32):
        out = subprocess.run([exe, str(n)], capture_output=True, text=True, timeout=60)
        assert out.returncode == 0
        c = np.array(out.stdout.split(), dtype=np.int64)
        py = record_slots(n)
        np.testing.assert_array_equal(c, py)
        assert np.array_equal(np.sort(py), np.arange(n ** 3))
        v = np.arange(n ** 3)
        x, y, z = v % n, (v // n) % n, v // (n * n)
        block = (z * n + y // 2) * n + x // 2  # the 2 x 2 (x, y) block of each voxel
        line_of_block = np.full(block.max() + 1, -1)
        line_of_block[block] = py // 4
        np.testing.assert_array_equal(line_of_block[block], py // 4)
        assert np.array_equal(np.bincount(py // 4), np.full(n ** 3 // 4, 4))
