"""The float arc cosine the GPU triangle split uses (tmc_gb300/csrc/libm_acosf.h) against the
platform C library's acosf, which the reference's minAngle calls through std::acos: one of the two
restated fdlibm kinds (separate roundings on x86-64, fused multiply-adds on aarch64) is bit-equal to
it on every float of [-1, 1] (tests/cpp/acos_check.cpp, built as host code with contraction off)."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def run_acos_check(tmp_path, stride=1):
    cxx = shutil.which("g++")
    if not cxx:
        pytest.skip("g++ not available")
    exe = tmp_path / "acos_check"
    subprocess.run([cxx, "-std=c++17", "-O2", "-ffp-contract=off", "-pthread", "-o", str(exe),
                    os.path.join(ROOT, "tests", "cpp", "acos_check.cpp")], check=True, capture_output=True)
    threads = max(1, min(32, os.cpu_count() or 1))
    out = subprocess.run([str(exe), str(stride), str(threads)], capture_output=True, text=True, timeout=600)
    return out


def test_acosf_restatement_equals_host_library(tmp_path):
    out = run_acos_check(tmp_path)
    assert out.returncode == 0 and out.stdout.startswith("ok ") and out.stdout.split()[2] == "2130706434", \
        out.stdout + out.stderr
