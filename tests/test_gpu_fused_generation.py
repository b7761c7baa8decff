"""Field generation fused into the extraction (tmc_dmc_extract_generated, tmc_tmc_extract_generated):
the classification evaluates the field instead of reading it, so no generation pass and no field
read happen.  Each mesh must equal, bit for bit, the mesh extracted from the same generator's stored
field (tmc_field_generate_ex, then tmc_dmc_extract / tmc_tmc_sharedvertex / tmc_tmc_halfedge), for
every surface kind of the reference's generator and for the batched workload's periodic and blob
fields, on grids of uneven sizes (rows shorter and longer than the 256 cells one classification step
covers, so both coordinate paths of the classification run).  The stored path itself is checked
against a float64 evaluation in test_gpu_field_generate.py."""
import math

import numpy as np
import pytest

from tmc_gb300 import native

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    c = native.Context(0)
    yield c
    c.close()


def _generators():
    rng = np.random.Generator(np.random.PCG64(21))
    blobs = []
    for _ in range(8):
        blobs += list(rng.uniform(-0.6, 0.6, size=3)) + [float(rng.uniform(0.15, 0.35))]
    gens = {}
    dims = [(57, 43, 38), (300, 21, 17), (64, 64, 64), (129, 97, 33), (3, 200, 41)]
    for s, name in enumerate(native.SURFACES):
        gens[name] = (native.make_generator(s, dims[s % len(dims)]), 0.0)
    gens["periodic"] = (native.make_generator(native.SURF_PERIODIC, (150, 90, 70), (6 * math.pi,)), 0.1)
    gens["periodic_long"] = (native.make_generator(native.SURF_PERIODIC, (700, 12, 9), (4.5 * math.pi,)), -0.2)
    gens["blobs"] = (native.make_generator(native.SURF_BLOBS, (80, 72, 66), blobs, count=8), 0.5)
    return gens


GENS = _generators()


def _stored(ctx, gen):
    f = ctx.field_generate_ex(gen)
    return f


def _fetch_raw(ctx, m):
    return ctx.fetch(m)


@pytest.mark.parametrize("name", sorted(GENS))
def test_fused_dmc_equals_stored(ctx, name):
    gen, iso = GENS[name]
    flags = native.OUT_POS_F64 | native.OUT_HOST
    f = _stored(ctx, gen)
    try:
        want = ctx.fetch(ctx.dmc_raw(f.vol, iso, flags))
        want_s = ctx.fetch(ctx.dmc_raw(f.vol, iso, flags | native.DMC_SIMPLIFY | native.OUT_TRIANGLES |
                                       native.OUT_HALFEDGES))
    finally:
        ctx.field_free(f)
    got = ctx.fetch(ctx.dmc_generated_raw(gen, iso, flags))
    got_s = ctx.fetch(ctx.dmc_generated_raw(gen, iso, flags | native.DMC_SIMPLIFY | native.OUT_TRIANGLES |
                                            native.OUT_HALFEDGES))
    assert want["q"].size > 0
    for k in ("q", "v", "n", "v64"):
        np.testing.assert_array_equal(got[k], want[k])
    for k in ("q", "v", "n", "v64", "t", "he", "hv", "hf"):
        np.testing.assert_array_equal(got_s[k], want_s[k])
    np.testing.assert_array_equal(got["stats"][:4], want["stats"][:4])


@pytest.mark.parametrize("name", sorted(GENS))
@pytest.mark.parametrize("halfedge", [False, True])
def test_fused_tmc_equals_stored(ctx, name, halfedge):
    gen, iso = GENS[name]
    flags = native.OUT_POS_F64 | native.OUT_HOST
    f = _stored(ctx, gen)
    try:
        want = ctx.fetch(ctx.tmc_raw(f.vol, iso, flags, halfedge=halfedge))
    finally:
        ctx.field_free(f)
    got = ctx.fetch(ctx.tmc_generated_raw(gen, iso, flags, halfedge=halfedge))
    assert want["t"].size > 0
    for k in ("t", "v", "n", "v64", "he", "hv", "hf"):
        np.testing.assert_array_equal(got[k], want[k])


def test_stored_generated_field_matches_float32_formula(ctx):
    """The parameterised fields themselves: the periodic and blob fields against a float64 evaluation
    at the same float32 grid points (relative 2e-5: float32 arithmetic and sin/cos/exp)."""
    import ctypes
    cudart = ctypes.CDLL("libcudart.so.13")
    for name in ("periodic", "blobs"):
        gen, _ = GENS[name]
        f = ctx.field_generate_ex(gen)
        n = gen.nx * gen.ny * gen.nz
        out = np.zeros(n, np.float32)
        assert cudart.cudaMemcpy(ctypes.c_void_p(out.ctypes.data), ctypes.c_void_p(f.vol.data),
                                 ctypes.c_size_t(4 * n), 2) == 0
        ctx.field_free(f)
        ax = [(-1.0 + np.arange(m, dtype=np.float32) * np.float32(2.0 / np.float32(m - 1))).astype(np.float64)
              for m in (gen.nx, gen.ny, gen.nz)]
        z, y, x = np.meshgrid(ax[2], ax[1], ax[0], indexing="ij")
        if name == "periodic":
            k = np.float32(gen.params[0]).astype(np.float64)
            want = np.sin(k * x) * np.cos(k * y) + np.sin(k * y) * np.cos(k * z) + np.sin(k * z) * np.cos(k * x)
            scale = 3.0
        else:
            want = np.zeros_like(x)
            for b in range(gen.count):
                c = [np.float32(gen.params[4 * b + a]).astype(np.float64) for a in range(3)]
                s = gen.params[4 * b + 3]
                want += np.exp(-((x - c[0]) ** 2 + (y - c[1]) ** 2 + (z - c[2]) ** 2) / (2 * s * s))
            scale = max(1.0, float(np.abs(want).max()))
        assert np.max(np.abs(out.reshape(want.shape) - want)) <= 2e-5 * scale * 8


def test_generator_rejected(ctx):
    bad = native.make_generator(native.SURF_BLOBS, (10, 10, 10), [0, 0, 0, -1.0], count=1)
    with pytest.raises(native.TmcError) as e:
        ctx.dmc_generated_raw(bad, 0.5, 0)
    assert e.value.status == native.TMC_ERR_INVALID_ARG
    bad = native.make_generator(99, (10, 10, 10))
    with pytest.raises(native.TmcError):
        ctx.tmc_generated_raw(bad, 0.0, 0)
    bad = native.make_generator(0, (1, 10, 10))
    with pytest.raises(native.TmcError):
        ctx.field_generate_ex(bad)
