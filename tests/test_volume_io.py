"""Volume files and mesh files on the CPU (no GPU needed).

tmc_volume_file_info parses the reference's four volume layouts and rejects bad files; the OBJ
and OFF writers reproduce the reference's text layouts.  Where the reference is compiled here
(oracle/_ref), its own MarchingCubes::operator() reads a ushort volume file and writes its OBJ and
OFF files, and the writers must produce the same files from the same mesh.
"""
import os

import numpy as np
import pytest

from tmc_gb300 import native
from tmc_gb300 import volumes as V

import cpu_libs


def _write_volume(path, fmt, data, spacing):
    nz, ny, nx = data.shape
    with open(path, "wb") as f:
        if fmt == native.FILE_U16:
            f.write(np.array([nx, ny, nz], np.uint16).tobytes())
            f.write(np.array(spacing, np.float32).tobytes())
            f.write(np.ascontiguousarray(data, np.uint16).tobytes())
            return
        f.write(np.array([nx, ny, nz], np.int32).tobytes())
        if fmt == native.FILE_DMC:
            f.write(np.array(spacing, np.float64).tobytes())
        else:
            f.write(np.array(spacing, np.float32).tobytes())
        dtype = np.uint16 if fmt == native.FILE_INT_U16 else np.float32
        f.write(np.ascontiguousarray(data, dtype).tobytes())


@pytest.fixture(scope="module")
def lib():
    try:
        return native.load()
    except RuntimeError:
        from tmc_gb300 import build
        build.build()
        return native.load()


@pytest.mark.parametrize("fmt,offset", [(native.FILE_DMC, 36), (native.FILE_INT_F32, 24), (native.FILE_INT_U16, 24),
                                        (native.FILE_U16, 18)])
def test_file_info(lib, tmp_path, fmt, offset):
    data = np.arange(5 * 6 * 7, dtype=np.float32).reshape(7, 6, 5)
    p = str(tmp_path / "v.raw")
    _write_volume(p, fmt, data, (0.5, 0.25, 0.125))
    dims, sp, off = native.volume_file_info(p, fmt)
    assert dims == (5, 6, 7)
    assert sp == (0.5, 0.25, 0.125)
    assert off == offset


def test_file_info_rejects_bad_files(lib, tmp_path):
    data = np.zeros((4, 4, 4), np.float32)
    p = str(tmp_path / "v.raw")
    _write_volume(p, native.FILE_INT_F32, data, (1, 1, 1))
    with open(p, "r+b") as f:  # truncate the data
        f.truncate(24 + 4 * 63)
    with pytest.raises(native.TmcError):
        native.volume_file_info(p, native.FILE_INT_F32)
    _write_volume(p, native.FILE_INT_F32, np.zeros((4, 4, 1), np.float32), (1, 1, 1))  # nx = 1
    with pytest.raises(native.TmcError):
        native.volume_file_info(p, native.FILE_INT_F32)
    _write_volume(p, native.FILE_INT_F32, data, (1, 0, 1))  # zero spacing
    with pytest.raises(native.TmcError):
        native.volume_file_info(p, native.FILE_INT_F32)
    with pytest.raises(native.TmcError):
        native.volume_file_info(p, 7)
    with pytest.raises(native.TmcError):
        native.volume_file_info(str(tmp_path / "missing.raw"), native.FILE_U16)


def _mesh():
    rng = np.random.Generator(np.random.PCG64(3))
    v = rng.uniform(-2, 2, 3 * 5).astype(np.float32)
    n = rng.uniform(-1, 1, 3 * 5).astype(np.float32)
    q = np.array([0, 1, 2, 3, 1, 2, 3, 4], np.int32)
    t = np.array([0, 1, 2, 2, 3, 4], np.int32)
    return v, n, q, t


def test_obj_and_off_layouts(lib, tmp_path):
    v, n, q, t = _mesh()
    m = native.host_mesh(v, n, quads=q, tris=t)
    p = str(tmp_path / "m")
    native.write_obj(m, p + "_t.obj", native.OBJ_DMC_TRIS)
    native.write_obj(m, p + "_q.obj", native.OBJ_DMC_QUADS)
    native.write_obj(m, p + "_m.obj", native.OBJ_TMC)
    native.write_off(m, p + ".off")
    vd, nd = v.astype(np.float64), n.astype(np.float64)
    vl = ["v %g %g %g" % tuple(vd[3 * i:3 * i + 3]) for i in range(5)]
    nl = ["vn %g %g %g" % tuple(nd[3 * i:3 * i + 3]) for i in range(5)]
    tl = ["f %d//%d %d//%d %d//%d" % (a + 1, a + 1, b + 1, b + 1, c + 1, c + 1) for a, b, c in t.reshape(-1, 3)]
    ql = ["f %d//%d %d//%d %d//%d %d//%d" % (a + 1, a + 1, b + 1, b + 1, c + 1, c + 1, d + 1, d + 1)
          for a, b, c, d in q.reshape(-1, 4)]
    assert open(p + "_t.obj").read().splitlines() == ["#Dual Marching Cubes, triangle mesh"] + vl + nl + tl
    assert open(p + "_q.obj").read().splitlines() == ["#Dual Marching Cubes, quad only mesh"] + vl + nl + ql
    vm = ["v %.7f %.7f %.7f" % tuple(vd[3 * i:3 * i + 3]) for i in range(5)]
    nm = ["vn %.7f %.7f %.7f" % tuple(nd[3 * i:3 * i + 3]) for i in range(5)]
    # the reference writes the second vertex's index as the third normal index
    fm = ["f %d//%d %d//%d %d//%d" % (a + 1, a + 1, b + 1, b + 1, c + 1, b + 1) for a, b, c in t.reshape(-1, 3)]
    assert open(p + "_m.obj").read().splitlines() == ["# Topologically correct and manifold isosurface"] + vm + nm + fm
    off = ["OFF", "5 2 0"] + ["%g %g %g" % tuple(vd[3 * i:3 * i + 3]) for i in range(5)] + \
          ["3 %d %d %d" % tuple(x) for x in t.reshape(-1, 3)]
    assert open(p + ".off").read().splitlines() == off
    # a quad-only mesh writes 4-vertex OFF faces
    mq = native.host_mesh(v, n, quads=q)
    native.write_off(mq, p + "_q.off")
    assert open(p + "_q.off").read().splitlines()[1:2] == ["5 2 0"]
    assert open(p + "_q.off").read().splitlines()[-1] == "4 1 2 3 4"
    with pytest.raises(native.TmcError):
        native.write_obj(mq, p + "_x.obj", native.OBJ_DMC_TRIS)  # no triangles


@pytest.mark.skipif(not cpu_libs.ref_available(), reason="the reference is not compiled here (oracle/_ref)")
def test_writers_match_the_reference_files(lib, tmp_path):
    """The reference reads a ushort volume file and writes OBJ / OFF; the same mesh through the
    writers gives the same files (normals: the mesh holds float32 normals, the reference prints its
    float64 ones, so vn lines agree to the float32 rounding)."""
    rng = np.random.Generator(np.random.PCG64(12))
    d = V.gaussian_blobs(22, 20, 18, rng)
    data = np.round(d * 1000).astype(np.uint16)
    spacing = (0.5, 0.75, 1.25)
    vol_path = str(tmp_path / "ct.raw")
    _write_volume(vol_path, native.FILE_U16, data, spacing)
    iso = 400.5
    ref_obj, ref_off = str(tmp_path / "ref.obj"), str(tmp_path / "ref.off")
    ref = cpu_libs.RefLib()
    ref.tmc_files(iso, vol_path, ref_obj, ref_off)
    # the same mesh: the reference's t_mc on the file's values
    dims, sp, _ = native.volume_file_info(vol_path, native.FILE_U16)
    vol = V.Volume(data.astype(np.float32), spacing=sp, origin=(0.0, 0.0, 0.0), iso=iso)
    mesh = ref.tmc(vol)
    assert mesh["t"].size > 0
    m = native.host_mesh(mesh["v"].astype(np.float32), mesh["n"].astype(np.float32), tris=mesh["t"], v64=mesh["v"])
    our_obj, our_off = str(tmp_path / "our.obj"), str(tmp_path / "our.off")
    native.write_obj(m, our_obj, native.OBJ_TMC)
    native.write_off(m, our_off)
    assert open(our_off).read() == open(ref_off).read()
    a, b = open(our_obj).read().splitlines(), open(ref_obj).read().splitlines()
    assert len(a) == len(b)
    for x, y in zip(a, b):
        if x.startswith("vn "):
            np.testing.assert_allclose([float(s) for s in x.split()[1:]], [float(s) for s in y.split()[1:]],
                                       atol=2e-7)
        else:
            assert x == y
