"""tmc_field_generate: the reference's implicit surfaces (dmc/UniformGrid.cu:21-175) sampled on the
GPU, against a numpy float64 evaluation of the same formulas at the same float32 grid points; and
an extraction from a generated field equals the extraction from the same values passed as a host
field."""
import ctypes

import numpy as np
import pytest

from tmc_gb300 import native
from tmc_gb300 import volumes as V

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    c = native.Context(0)
    yield c
    c.close()


def _device_to_host(ptr, n):
    cudart = ctypes.CDLL("libcudart.so.13")
    out = np.zeros(n, np.float32)
    assert cudart.cudaMemcpy(ctypes.c_void_p(out.ctypes.data), ctypes.c_void_p(ptr), ctypes.c_size_t(4 * n), 2) == 0
    return out


def _surface(name, x, y, z):
    pi = np.pi
    torus = lambda cx, cy, cz, vert: ((x - cx) ** 2 + (y - cy) ** 2 + (z - cz) ** 2 + 0.09 - 0.0225) ** 2 - \
        4 * 0.09 * ((x - cx) ** 2 + ((z - cz) ** 2 if vert else (y - cy) ** 2))
    if name == "sphere":
        return x * x + y * y + z * z - 0.16
    if name == "torus":
        return torus(0, 0, 0, False)
    if name == "two_holed_torus":
        return np.minimum(torus(-0.38, 0, 0, False), torus(0.2, 0.38, 0, False))
    if name == "four_holed_torus":
        return np.minimum(np.minimum(torus(-0.38, 0, 0, False), torus(0.38, 0, 0, False)),
                          np.minimum(torus(0, 0, -0.38, True), torus(0, 0, 0.38, True)))
    if name == "genus_two":
        X, Y, Z = 4 * ((x + 1) / 2) - 2, 4 * ((y + 1) / 2) - 2, 4 * ((z + 1) / 2) - 2
        return 2 * Y * (Y * Y - 3 * X * X) * (1 - Z * Z) + (X * X + Y * Y) ** 2 - (9 * Z * Z - 1) * (1 - Z * Z)
    if name in ("iwp", "pw_hybrid", "neovius"):
        s = {"iwp": 5.01, "pw_hybrid": 1.01, "neovius": 1.0}[name] * pi
        cx, cy, cz = np.cos(s * (x + 1)), np.cos(s * (y + 1)), np.cos(s * (z + 1))
        if name == "iwp":
            return cx * cy + cy * cz + cz * cx - cx * cy * cz
        if name == "pw_hybrid":
            return 4 * (cx * cy + cy * cz + cz * cx) - 3 * cx * cy * cz + 0.8
        return 3 * (cx + cy + cz) + 4 * cx * cy * cz
    if name == "goursat":
        return x ** 4 + y ** 4 + z ** 4 - (x * x + y * y + z * z) + 0.5
    X, Y, Z = 1.5 * x, 1.5 * y, 1.5 * z
    return (X * X + Y * Y + Z * Z - 1) ** 2 - ((Z - 1) ** 2 - 2 * X * X) * ((Z + 1) ** 2 - 2 * Y * Y)


@pytest.mark.parametrize("sc", range(len(native.SURFACES)))
def test_generated_surface(ctx, sc):
    name = native.SURFACES[sc]
    nx, ny, nz = 33, 29, 31
    f = ctx.field_generate(sc, nx, ny, nz)
    try:
        assert (f.vol.nx, f.vol.ny, f.vol.nz) == (nx, ny, nz)
        assert tuple(f.vol.origin) == (-1.0, -1.0, -1.0)
        d = [np.float32(2.0) / np.float32(n - 1.0) for n in (nx, ny, nz)]
        assert tuple(f.vol.spacing) == tuple(float(a) for a in d)
        got = _device_to_host(f.vol.data, nx * ny * nz).reshape(nz, ny, nx)
        ax = [(np.float32(-1.0) + np.arange(n, dtype=np.float32) * a).astype(np.float64) for n, a in zip((nx, ny, nz), d)]
        z, y, x = np.meshgrid(ax[2], ax[1], ax[0], indexing="ij")
        want = _surface(name, x, y, z)
        scale = np.abs(want).max()
        np.testing.assert_allclose(got, want, rtol=2e-5, atol=2e-5 * scale, err_msg=name)
        # the generated field extracts like the same values given as a host field
        host = V.Volume(got, spacing=tuple(f.vol.spacing), origin=(-1.0, -1.0, -1.0), iso=0.0)
        a = ctx.fetch(ctx.dmc_raw(f.vol, 0.0, native.OUT_HOST | native.OUT_POS_F64))
        b = ctx.dmc(host, native.OUT_POS_F64)
        for k in ("v64", "q", "n"):
            np.testing.assert_array_equal(a[k], b[k], err_msg=f"{name}: {k}")
    finally:
        ctx.field_free(f)


def test_generate_rejects(ctx):
    with pytest.raises(native.TmcError):
        ctx.field_generate(10, 8, 8, 8)
    with pytest.raises(native.TmcError):
        ctx.field_generate(0, 1, 8, 8)
