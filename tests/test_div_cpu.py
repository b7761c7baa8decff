"""CPU checks of index arithmetic in tmc_gb300/csrc/common.cuh, built as host code by nvcc:

* the invariant-divisor division (Div32) that every cell kernel uses to split cell indices into
  (i, j, k) must equal n / d for every divisor up to 70000 and random 32-bit divisors
  (tests/cpp/div_check.cpp);
* the chunk mapping of the listed-cell walks (slot_chunk) must hand out every (tile, part) once, in
  windows taken in order, for tile counts 1..1100 and large grids (tests/cpp/chunk_check.cpp)."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_div32_exact(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not available")
    exe = tmp_path / "div_check"
    subprocess.run([nvcc, "-std=c++17", "-O2", "-x", "cu", "-o", str(exe),
                    os.path.join(ROOT, "tests", "cpp", "div_check.cpp")], check=True, capture_output=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0 and out.stdout.strip() == "ok", out.stdout + out.stderr


def test_slot_chunk_covers_every_chunk_once(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not available")
    exe = tmp_path / "chunk_check"
    subprocess.run([nvcc, "-std=c++17", "-O2", "-x", "cu", "-o", str(exe),
                    os.path.join(ROOT, "tests", "cpp", "chunk_check.cpp")], check=True, capture_output=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0 and out.stdout.strip() == "ok", out.stdout + out.stderr
