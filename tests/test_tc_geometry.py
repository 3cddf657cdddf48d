"""CPU checks of the tensor-core block kernels' host logic and of the
engine's gate fusion (``tests/native/fuse_check.cu``, includes
``qgb_fuse.cu``).

Compiles ``tests/native/tc_geometry_check.cu`` (complex64, includes
``qgb_tc.cu``) and ``tests/native/oz_check.cu`` (complex128 Ozaki scheme,
includes ``qgb_tc128.cu``) with nvcc and runs them on the host: they replay
each kernel's loads, operand layouts, products, staging and stores with the
tables the launchers build (and, for complex128, the same digit / combine
functions the kernel calls), compare against the block applied directly in
FP64, and bound the shared-memory wavefronts of every access pattern.  No
kernel is launched; nvcc cross-compiles here.
"""

import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _build_and_run(tmp_path, name):
    from qibo_gb300 import _build

    try:
        nvcc = _build.nvcc_path()
    except RuntimeError:
        pytest.skip("nvcc not available")
    if not os.path.exists(_build.LIB):
        _build.build()
    exe = str(tmp_path / name)
    libdir = os.path.dirname(_build.LIB)
    libname = os.path.basename(_build.LIB)[3:-3]  # libqgb300.so -> qgb300
    cmd = [nvcc, *_build.ARCH, "-O2", "-std=c++17",
           "-I", os.path.join(ROOT, "qibo_gb300", "csrc"), "-I", os.path.join(ROOT, "include"),
           os.path.join(ROOT, "tests", "native", name + ".cu"), "-o", exe,
           "-L", libdir, f"-l{libname}", "-Xlinker", f"-rpath,{libdir}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-4000:]
    r = subprocess.run([exe], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout[-4000:] + r.stderr[-2000:]
    return r.stdout


def test_tc_geometry_tables(tmp_path):
    out = _build_and_run(tmp_path, "tc_geometry_check")
    assert "index failures 0 bank-pattern failures 0" in out


def test_bench_labels_follow_the_launcher_plan(tmp_path):
    """bench.py names the complex64 block kernel a placement runs on with a
    copy of the launcher's tcm_plan; both agree on every 5-qubit block of a
    16-qubit state."""
    import importlib.util

    _build_and_run(tmp_path, "tc_geometry_check")
    r = subprocess.run([str(tmp_path / "tc_geometry_check"), "plans"], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0
    spec = importlib.util.spec_from_file_location("bench_mod", os.path.join(ROOT, "bench.py"))
    bench = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(bench)
    names = {0: "k_fused5_tc", 1: "k_fused5_tcm (strided lanes)", 2: "k_fused5_tcm (coalesced lanes)"}
    lines = r.stdout.split("\n")
    checked = 0
    for line in lines:
        if not line.strip():
            continue
        bits, plan = line.split()
        bits = [int(x) for x in bits.split(",")]
        assert bench.tc64_kernel(16, [15 - b for b in bits]) == names[int(plan)], bits
        checked += 1
    assert checked == 4368


def test_oz_complex128_blocks(tmp_path):
    out = _build_and_run(tmp_path, "oz_check")
    assert "index failures 0 exactness failures 0 bank-pattern failures 0" in out


def test_engine_fusion(tmp_path):
    """qgb_fuse5: random gate lists (dense, controlled, diagonal, wider than
    5 qubits) fused vs gate by gate on CPU states, 1e-12."""
    out = _build_and_run(tmp_path, "fuse_check")
    assert "failures 0" in out
