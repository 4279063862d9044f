"""Host logic of the library that runs without a GPU, built from small C++
programs against the in-tree library (tests/host/)."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB_DIR = os.path.join(ROOT, "cassia_gb300", "_build")


def _build(src, tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not found")
    if not os.path.exists(os.path.join(LIB_DIR, "libcassia_gb300.so")):
        pytest.skip("library not built")
    exe = str(tmp_path / "prog")
    cmd = [nvcc, "-O2", "-std=c++17", "--expt-relaxed-constexpr", "-I", os.path.join(ROOT, "cassia_gb300", "csrc"),
           "-I", os.path.join(ROOT, "include"), os.path.join(ROOT, "tests", "host", src), "-o", exe,
           "-L", LIB_DIR, "-l:libcassia_gb300.so", "-Xlinker", "-rpath=" + LIB_DIR]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    return exe


def test_set_transforms_parallel_equals_sequential(tmp_path):
    exe = _build("set_transforms_equiv.cu", tmp_path)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("case")]
    assert len(lines) == 6 and all(ln.endswith("same") for ln in lines), r.stdout
