"""TMC with float32 outputs only (no TMC_OUT_POS_F64), against the CPU oracle.

Without float64 outputs the edge vertices are interpolated in float32 and float pairs, and the
ambiguous cells' inner-vertex normals in float-float (float64 where the corner gradients cancel).
Topology is the same bit for bit.  Positions: the edge parameter is a float32 quotient (relative
error 2^-24), so a coordinate is within 2 float32 ulps of the oracle's float64 value plus 2^-22 of a
cell (absolute: coordinates near zero have tiny ulps).  Unit normals within 1e-5 per component
(absolute)."""
import numpy as np
import pytest

from tmc_gb300 import volumes as V

pytestmark = pytest.mark.gpu

NORMAL_TOL = 1e-5


@pytest.fixture(scope="module")
def ctx():
    from tmc_gb300 import native
    c = native.Context(0)
    yield c
    c.close()


def _cases():
    return {
        "noise48": V.small_noise_volume(48, seed=5, coarse=7),
        "blobs64": V.blobs_volume(64, seed=0),
        "noise512_slab": V.z_slab(V.noise_volume(512, seed=1), 244, 12),
        "saddle1024_slab": V.saddle_slab(1024, 300, 8, seed=3),
    }


@pytest.mark.parametrize("name", ["noise48", "blobs64", "noise512_slab", "saddle1024_slab"])
def test_tmc_float32_outputs(ctx, oracle, name):
    vol = _cases()[name]
    want = oracle.tmc(vol)
    got = ctx.tmc(vol, 0)
    np.testing.assert_array_equal(got["t"], want["t"])
    w = want["v"].astype(np.float64).reshape(-1, 3)
    b32 = w.astype(np.float32)
    cell = np.asarray(vol.spacing, np.float64)
    tol = 2 * np.spacing(np.abs(b32).astype(np.float32) + np.float32(1e-30)).astype(np.float64) + cell * 2.0 ** -22
    perr = np.abs(got["v"].astype(np.float64).reshape(-1, 3) - w)
    err = np.abs(got["n"].astype(np.float64) - want["n"].astype(np.float64))
    print(f"{name}: {w.shape[0]} vertices, ambiguous cells {got['stats'][1]}, position error max "
          f"{(perr / cell).max():.3g} cells, normal error max {err.max():.3g} rms {np.sqrt(np.mean(err ** 2)):.3g}")
    assert np.all(perr <= tol)
    assert err.max() <= NORMAL_TOL
