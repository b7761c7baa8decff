"""The C++ adapters (include/tmc_gb300_adapters.hpp) with the reference's call signatures:
dmc::DualMarchingCubes::dualMC on a UniformGrid, and p_mc::MarchingCubes::mc_sharedvertex on a
ushort volume file in the reference's format.  Compiled with g++ against libtmc_gb300.so and run
as a separate program; results compared with the CPU oracle."""
import os
import struct
import subprocess

import numpy as np
import pytest

from tmc_gb300 import volumes as V

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_cpp_adapters(tmp_path, oracle):
    from tmc_gb300 import build
    lib = build.build()
    exe = tmp_path / "adapter_check"
    subprocess.run(["g++", "-std=c++17", "-O1", "-o", str(exe), os.path.join(ROOT, "tests", "cpp", "adapter_check.cpp"),
                    "-L" + os.path.dirname(lib), "-ltmc_gb300", "-Wl,-rpath," + os.path.dirname(lib)], check=True)
    vol = V.small_noise_volume(28, seed=21, coarse=5)
    nx, ny, nz = vol.dims
    field = tmp_path / "field.raw"
    vol.data.astype(np.float32).tofile(field)
    # ushort volume file: dims, spacing, samples (mc/MarchingCubes.cpp:22-66)
    blobs = V.blobs_volume(20, seed=4)
    us = np.clip(blobs.data * 1500.0, 0, 65535).astype(np.uint16)
    vf = tmp_path / "vol.ushort"
    with open(vf, "wb") as f:
        f.write(struct.pack("<3H", 20, 20, 20))
        f.write(struct.pack("<3f", 0.5, 0.5, 0.5))
        f.write(us.tobytes())
    out = tmp_path / "out.bin"
    subprocess.run([str(exe), str(field), str(nx), str(ny), str(nz), str(vol.iso), str(out), str(vf)], check=True)
    raw = out.read_bytes()
    nv, nq, tv, tt = struct.unpack("<4q", raw[:32])
    off = 32
    v = np.frombuffer(raw, np.float64, 3 * nv, off); off += 24 * nv
    q = np.frombuffer(raw, np.int32, 4 * nq, off); off += 16 * nq
    t = np.frombuffer(raw, np.int32, 6 * nq, off); off += 24 * nq
    tri = np.frombuffer(raw, np.int32, 3 * tt, off); off += 12 * tt
    want = oracle.dmc(vol, 1)
    np.testing.assert_array_equal(q, want["q"])
    np.testing.assert_array_equal(v, want["v"])
    assert np.mean(np.all(t.reshape(-1, 6) == want["t"].reshape(-1, 6), axis=1)) > 0.999
    fvol = V.Volume(us.astype(np.float32), origin=(0.0, 0.0, 0.0), spacing=(0.5, 0.5, 0.5), iso=1000.0)
    wt = oracle.tmc(fvol)
    assert tv == wt["v"].size // 3
    np.testing.assert_array_equal(tri, wt["t"])
