"""TMC on the GPU (through the C ABI) against the CPU oracle.

Topology (triangles, vertex order) bit-exact; float64 vertex positions (OUT_POS_F64) bit-exact;
float32 positions and normals within 2 float32 ulps of the oracle's float64 values."""
import hashlib
import json
import math
import os

import numpy as np
import pytest

from tmc_gb300 import volumes as V

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.fixture(scope="module")
def ctx():
    from tmc_gb300 import native
    c = native.Context(0)
    yield c
    c.close()


def _load_golden_module():
    import importlib.util
    spec = importlib.util.spec_from_file_location("make_golden", os.path.join(GOLDEN, "make_golden.py"))
    mg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mg)
    return mg


def _cases():
    mg = _load_golden_module()
    rng = np.random.Generator(np.random.PCG64(5))
    sad = V.periodic(33, 33, 33, 6 * math.pi)
    V.seed_saddles(sad, rng, frac=0.5)
    cases = {
        "blobs48": V.blobs_volume(48, seed=0),
        "noise32": V.small_noise_volume(32, seed=11),
        "noise64": V.small_noise_volume(64, seed=13, coarse=9),
        "saddle33": V.Volume(sad, spacing=(2 / 32,) * 3, iso=0.0),
        "singular12": mg.singular_volume(),
        "singular32": mg.singular_volume(32, 4),
        # edge cases: corners exactly at the isovalue (integer field, integer isovalue), a slab one cell
        # thick with uneven spacing, and values near 1000 (float32 steps of 6e-5 around the isovalue)
        "iso_on_grid": V.Volume(np.round(V.gaussian_blobs(20, 18, 22, np.random.Generator(np.random.PCG64(8))) * 8)
                                .astype(np.float32), spacing=(0.5, 0.25, 0.75), iso=3.0),
        "slab2": V.Volume(V.gaussian_blobs(40, 33, 2, np.random.Generator(np.random.PCG64(9))), spacing=(0.1, 0.3, 2.0),
                          iso=0.3),
        # a far origin (positions rounded from float64 once) and micro spacing (gradients scaled by ~5e5)
        "origin_far": V.Volume(V.blobs_volume(24, seed=6).data, spacing=(0.25, 0.5, 0.125),
                               origin=(12345.5, -6789.25, 3.0), iso=0.5),
        "tiny_spacing": V.Volume(V.small_noise_volume(20, seed=9).data, spacing=(1e-6, 1.5e-6, 2e-6), iso=0.0),
        # long thin grids: cell indices split by large and small divisors
        "long_x": V.Volume(V.periodic(20000, 3, 4, 900.0), spacing=(1e-3, 0.5, 0.5), iso=0.05),
        "long_y": V.Volume(V.periodic(3, 9000, 5, 400.0), spacing=(0.5, 1e-3, 0.5), iso=-0.1),
        "offset1000": V.Volume(V.small_noise_volume(24, seed=4).data + np.float32(1000.0), spacing=(1.0, 1.0, 1.0),
                               iso=1000.0),
        "batch5": V.batch_volumes(6, seed=2)[5],
    }
    for name, vals, iso in mg.MATLAB_CELLS:
        cases["cell_" + name] = mg.cell_volume(vals, iso)
    return cases


CASES = _cases()


def _close32(a32, b64, ulps=2):
    b32 = b64.astype(np.float32)
    tol = ulps * np.spacing(np.abs(b32).astype(np.float32) + np.float32(1e-30))
    return np.all(np.abs(a32.astype(np.float64) - b64) <= tol.astype(np.float64) + 1e-300)


@pytest.mark.parametrize("name", sorted(CASES))
def test_tmc_matches_oracle(ctx, oracle, name):
    from tmc_gb300 import native
    vol = CASES[name]
    want = oracle.tmc(vol)
    got = ctx.tmc(vol, native.OUT_POS_F64)
    np.testing.assert_array_equal(got["t"], want["t"])
    np.testing.assert_array_equal(got["v64"], want["v"])
    assert _close32(got["v"], want["v"])
    assert _close32(got["n"], want["n"])
    assert got["stats"][5] == want["cases"][10]  # singular faces without a triangulation


@pytest.mark.parametrize("name", ["noise64_tmc", "saddle48_tmc", "singular32_tmc", "batch5_tmc"])
def test_tmc_golden_digests(ctx, name):
    from tmc_gb300 import native
    mg = _load_golden_module()
    case = json.load(open(os.path.join(GOLDEN, "digests.json")))[name]
    vol = mg.make_volume(case["recipe"])
    got = ctx.tmc(vol, native.OUT_POS_F64)
    assert hashlib.sha256(got["t"].tobytes()).hexdigest() == case["digests"]["t"]
    assert hashlib.sha256(got["v64"].tobytes()).hexdigest() == case["digests"]["v"]


@pytest.mark.parametrize("name", ["noise32", "saddle33", "singular12", "blobs48"])
def test_tmc_halfedges_match_oracle(ctx, oracle, name):
    vol = CASES[name]
    got = ctx.tmc(vol, 0, halfedge=True)
    nv = got["v"].size // 3
    want = oracle.halfedges(got["t"], 3, nv)
    he5 = want["he"].reshape(-1, 5)
    np.testing.assert_array_equal(got["he"].reshape(-1, 4), he5[:, :4])
    np.testing.assert_array_equal(got["hv"], want["hv"])
    np.testing.assert_array_equal(got["hf"], want["hf"])
