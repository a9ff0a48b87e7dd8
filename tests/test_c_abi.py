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
