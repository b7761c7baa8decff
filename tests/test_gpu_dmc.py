"""DMC on the GPU (through the C ABI) against the CPU oracle, bit-exact where the oracle is.

Tolerances: vertex positions as float64 (OUT_POS_F64) and the local cell coordinates are compared
exactly; float32 positions and normals within 2 float32 ulps of the oracle's float64 values
(the kernels compute them in float64 and round once)."""
import math

import numpy as np
import pytest

from tmc_gb300 import volumes as V

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    from tmc_gb300 import native
    c = native.Context(0)
    yield c
    c.close()


def _cases():
    rng = np.random.Generator(np.random.PCG64(5))
    sad = V.periodic(33, 33, 33, 6 * math.pi)
    V.seed_saddles(sad, rng, frac=0.5)
    return {
        "blobs64": V.blobs_volume(64, seed=0),
        "noise32": V.small_noise_volume(32, seed=11),
        "noise48": V.small_noise_volume(48, seed=5, coarse=7),
        "saddle33": V.Volume(sad, spacing=(2 / 32,) * 3, iso=0.0),
        "batch3": V.batch_volumes(4, seed=2)[3],
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
        "tiny2": V.Volume(np.array([[[0.0, 1.0], [1.0, 0.0]], [[1.0, 0.0], [0.0, 1.0]]], np.float32),
                          spacing=(1.0, 1.0, 1.0), origin=(0.0, 0.0, 0.0), iso=0.5),
    }


CASES = _cases()


def _close32(a32, b64, ulps=2, abs_tol=1e-300):
    """|a - b| <= ulps float32 ulps of b, or <= abs_tol."""
    b32 = b64.astype(np.float32)
    tol = ulps * np.spacing(np.abs(b32).astype(np.float32) + np.float32(1e-30))
    return np.all(np.abs(a32.astype(np.float64) - b64) <= np.maximum(tol.astype(np.float64), abs_tol))


# Unit normals: 2 float32 ulps, or 2^-40 absolute for components that are zero up to the
# reference's float64 rounding noise (symmetric saddles give components of ~1e-17 either sign).
NORMAL_ABS_TOL = 2.0 ** -40


def split_differences(got_t, want_t):
    """Number of quads whose two triangles differ from the oracle's (the split decision)."""
    gt, wt = got_t.reshape(-1, 6), want_t.reshape(-1, 6)
    assert gt.shape == wt.shape
    return int(np.count_nonzero(np.any(gt != wt, axis=1)))


@pytest.mark.parametrize("name", sorted(CASES))
@pytest.mark.parametrize("flip", [0, 1])
def test_dmc_front_matches_oracle(ctx, oracle, name, flip):
    from tmc_gb300 import native
    vol = CASES[name]
    want = oracle.dmc_front(vol, flip)
    got = ctx.dmc(vol, native.OUT_POS_F64 | native.OUT_LOCAL | (native.GRAD_FLIP if flip else 0))
    np.testing.assert_array_equal(got["q"], want["q"])
    np.testing.assert_array_equal(got["vcell"], want["vcell"])
    np.testing.assert_array_equal(got["vuvw"], want["vuvw"])
    np.testing.assert_array_equal(got["v64"], want["v"])
    assert _close32(got["v"], want["v"])
    # float32 normals are computed in float32 when nothing needs them in float64
    assert np.max(np.abs(got["n"].astype(np.float64) - want["n"]), initial=0) < 1e-5
    assert got["stats"][2] == want["proj_fail"][0] and got["stats"][3] == want["proj_fail"][1]


def test_dmc_c0_blobs_against_golden_digest(ctx):
    """The 64^3 Gaussian-blob workload (isovalue 0.5, no simplification): quads and float64
    vertices hash-equal to the reference's own output (tests/golden/digests.json)."""
    import hashlib
    import json
    import os
    from tmc_gb300 import native
    d = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "digests.json")))["blobs64_dmc"]
    vol = V.blobs_volume(64, seed=0)
    got = ctx.dmc(vol, native.OUT_POS_F64)
    assert hashlib.sha256(got["q"].tobytes()).hexdigest() == d["digests"]["q"]
    assert hashlib.sha256(got["v64"].tobytes()).hexdigest() == d["digests"]["v"]


def test_dmc_empty_and_host_device_inputs(ctx):
    import torch
    from tmc_gb300 import native
    vol = V.Volume(np.ones((6, 7, 8), np.float32), spacing=(1, 1, 1), iso=0.0)
    got = ctx.dmc(vol)
    assert got["v"].size == 0 and got["q"].size == 0
    vol = V.blobs_volume(24, seed=3)
    host = ctx.dmc(vol, native.OUT_POS_F64)
    dev = torch.from_numpy(vol.data).cuda()
    m = ctx.dmc_raw(native.make_volume(vol, dev.data_ptr(), on_device=True), vol.iso,
                    native.OUT_POS_F64 | native.OUT_HOST)
    got = ctx.fetch(m)
    np.testing.assert_array_equal(got["q"], host["q"])
    np.testing.assert_array_equal(got["v64"], host["v64"])


def test_dmc_invalid_arguments(ctx):
    from tmc_gb300 import native
    vol = V.blobs_volume(8)
    v = native.make_volume(vol)
    v.nx = 1
    with pytest.raises(native.TmcError) as e:
        ctx.dmc_raw(v, 0.5, 0)
    assert e.value.status == 1


FULL_CASES = ["noise32", "noise48", "saddle33", "blobs64", "batch3"]


@pytest.mark.parametrize("name", FULL_CASES)
@pytest.mark.parametrize("simplify", [0, 1])
def test_dmc_full_pipeline_matches_oracle(ctx, oracle, name, simplify):
    """dualMC end to end: front end, P3X3Y colour + isolated passes and P3333 (when simplifying),
    final halfedges and the quad -> triangle split."""
    from tmc_gb300 import native
    vol = CASES[name]
    want = oracle.dmc(vol, simplify)
    flags = native.OUT_POS_F64 | native.OUT_TRIANGLES | native.OUT_HALFEDGES
    if simplify:
        flags |= native.DMC_SIMPLIFY
    got = ctx.dmc(vol, flags)
    np.testing.assert_array_equal(got["q"], want["q"])
    np.testing.assert_array_equal(got["v64"], want["v"])
    assert _close32(got["v"], want["v"])
    if simplify:  # float64 normals are kept through the merges
        assert _close32(got["n"], want["n"], ulps=2, abs_tol=NORMAL_ABS_TOL)
    else:
        assert np.max(np.abs(got["n"].astype(np.float64) - want["n"]), initial=0) < 1e-5
    he5 = want["he"].reshape(-1, 5)
    np.testing.assert_array_equal(got["he"].reshape(-1, 4), he5[:, :4])
    np.testing.assert_array_equal(got["hv"], want["hv"])
    np.testing.assert_array_equal(got["hf"], want["hf"])
    # quad -> triangle split: bit-exact (the host library's float acos restated on the GPU)
    assert split_differences(got["t"], want["t"]) == 0


def test_dmc_saddle_crops_float64_mean_point(ctx):
    """Crops of the 1024^3 precision-stress field around contours with no valid projection sample
    even at 26x26: float64 positions bit-equal to the reference's (its unrounded mean point)."""
    from tmc_gb300 import native
    import os
    z = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "saddle_crops.npz"))
    sp = tuple(z["spacing"].tolist())
    for q in range(11):
        vol = V.Volume(z[f"f{q}"], origin=tuple(z[f"o{q}"].tolist()), spacing=sp, iso=0.0)
        got = ctx.dmc(vol, native.OUT_POS_F64)
        np.testing.assert_array_equal(got["q"], z[f"q{q}"])
        np.testing.assert_array_equal(got["v64"], z[f"v{q}"])
        assert got["stats"][3] >= 1  # the reference's 26x26 failure counter


def test_host_acosf_is_the_restated_one(tmp_path):
    """The split parity above rests on the GPU's float acos being this host C library's acosf
    (what the reference's std::acos calls here).  On the host: one restated kind is bit-equal to it
    on every float of [-1, 1].  On the GPU: the kind the library selects at run time, evaluated by the
    device for every float of [-1, 1], is bit-equal to it (tests/cpp/acos_device_check.cu, built with
    the library's floating-point flags)."""
    import os
    import shutil
    import subprocess
    from test_acos_cpu import ROOT, run_acos_check
    out = run_acos_check(tmp_path)
    assert out.returncode == 0 and out.stdout.startswith("ok "), out.stdout + out.stderr
    host_kind = out.stdout.split()[1]
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    exe = tmp_path / "acos_device_check"
    subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-fmad=false", "-Xcompiler",
                    "-ffp-contract=off", "-o", str(exe), os.path.join(ROOT, "tests", "cpp", "acos_device_check.cu")],
                   check=True, capture_output=True)
    dev = subprocess.run([str(exe)], capture_output=True, text=True, timeout=600)
    assert dev.returncode == 0 and dev.stdout.startswith("ok " + host_kind + " 2130706434"), dev.stdout + dev.stderr
