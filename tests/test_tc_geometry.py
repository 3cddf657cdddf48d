"""CPU check of the tensor-core block kernel's index tables.

Compiles ``tests/native/tc_geometry_check.cu`` (which includes
``qgb_tc.cu``) with nvcc and runs it on the host: it replays the kernel's
loads, operand layout, permuted block product, staging and stores with the
tables ``make_geom`` builds and compares against the block applied
directly, and bounds the shared-memory wavefronts of every access pattern.
No kernel is launched; nvcc cross-compiles here.
"""

import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_tc_geometry_tables(tmp_path):
    from qibo_gb300 import _build

    try:
        nvcc = _build.nvcc_path()
    except RuntimeError:
        pytest.skip("nvcc not available")
    if not os.path.exists(_build.LIB):
        _build.build()
    exe = str(tmp_path / "tc_geometry_check")
    libdir = os.path.dirname(_build.LIB)
    libname = os.path.basename(_build.LIB)[3:-3]  # libqgb300.so -> qgb300
    cmd = [nvcc, *_build.ARCH, "-O2", "-std=c++17",
           "-I", os.path.join(ROOT, "qibo_gb300", "csrc"), "-I", os.path.join(ROOT, "include"),
           os.path.join(ROOT, "tests", "native", "tc_geometry_check.cu"), "-o", exe,
           "-L", libdir, f"-l{libname}", "-Xlinker", f"-rpath,{libdir}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-4000:]
    r = subprocess.run([exe], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout[-4000:] + r.stderr[-2000:]
    assert "index failures 0 bank-pattern failures 0" in r.stdout
