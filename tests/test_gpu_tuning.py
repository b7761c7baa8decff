"""Launch-shape settings (tmc_ctx_set_tuning) and the autotuner (tmc_ctx_autotune).

The settings choose between kernels that compute the same values: one thread per vertex or a group
of lanes per vertex for the DMC projection, one thread or one warp per float64-fallback vertex, and
the grid sizes of the per-vertex and TMC emission passes.  Every setting must give bit-identical
meshes and the same counters; the oracle parity of the default settings is checked in
test_gpu_dmc.py and test_gpu_tmc.py.
"""
import math
import os

import numpy as np
import pytest

from tmc_gb300 import native
from tmc_gb300 import volumes as V

pytestmark = pytest.mark.gpu

KEYS = ("v", "n", "v64", "q", "t", "he", "hv", "hf", "vcell", "vuvw")
TUNE_KEYS = (native.TUNE_GROUP_LANES, native.TUNE_WARP_LIST_MAX, native.TUNE_VERTEX_BLOCKS_PER_SM,
             native.TUNE_EMIT_BLOCKS_PER_SM)

# (group lanes, warp list max, vertex blocks per SM, emit blocks per SM)
SETTINGS = {
    "threads": (0, 0, 32, 8),              # one thread per vertex everywhere, 26x26 retries by warp
    "lanes": (1 << 40, 1 << 30, 32, 8),    # lane groups and whole lists by warp wherever possible
    "small_grids": (0, 1 << 30, 1, 1),     # minimal grids: every grid-stride loop takes many turns
}


@pytest.fixture(scope="module")
def ctx():
    c = native.Context(0)
    yield c
    c.close()


def _apply(ctx, setting):
    for k, v in zip(TUNE_KEYS, setting):
        ctx.set_tuning(k, v)


def _cases():
    rng = np.random.Generator(np.random.PCG64(8))
    sad = V.periodic(41, 41, 41, 6 * math.pi)
    V.seed_saddles(sad, rng, frac=0.5)
    return {
        "saddle41": V.Volume(sad, spacing=(2 / 40,) * 3, iso=0.0),
        "noise48": V.small_noise_volume(48, seed=5, coarse=7),
        "blobs64": V.blobs_volume(64, seed=0),
    }


CASES = _cases()


def _same(a, b, what):
    for k in KEYS:
        np.testing.assert_array_equal(a[k], b[k], err_msg=f"{what}: {k}")
    # counters 0-6 (cells, projection failures, non-manifold edges ...); 7 counts float64
    # evaluations, which depend on how many samples a path evaluates exactly
    np.testing.assert_array_equal(a["stats"][:7], b["stats"][:7], err_msg=f"{what}: stats")


@pytest.mark.parametrize("name", sorted(CASES))
def test_dmc_identical_under_every_setting(ctx, name):
    vol = CASES[name]
    flag_sets = [native.OUT_POS_F64 | native.OUT_LOCAL,
                 native.DMC_SIMPLIFY | native.DMC_P3333 | native.OUT_TRIANGLES | native.OUT_HALFEDGES]
    default = tuple(ctx.get_tuning(k) for k in TUNE_KEYS)
    try:
        for flags in flag_sets:
            want = ctx.dmc(vol, flags)
            for sname, setting in SETTINGS.items():
                _apply(ctx, setting)
                _same(ctx.dmc(vol, flags), want, f"{name} flags {flags:#x} setting {sname}")
            _apply(ctx, default)
    finally:
        _apply(ctx, default)


def test_saddle_case_reaches_the_retry(ctx):
    """The saddle field has a contour without a valid 7x7 sample, so the test above covers the
    26x26 retry from both the thread and the warp list paths."""
    assert ctx.dmc(CASES["saddle41"], 0)["stats"][2] > 0


def test_saddle_crops_under_every_setting(ctx):
    """Crops around contours without any valid sample even at 26x26 (fixtures made from the
    reference): the float64 mean point comes out of the thread and the warp paths alike."""
    z = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "saddle_crops.npz"))
    sp = tuple(z["spacing"].tolist())
    default = tuple(ctx.get_tuning(k) for k in TUNE_KEYS)
    try:
        for sname, setting in SETTINGS.items():
            _apply(ctx, setting)
            for q in range(11):
                vol = V.Volume(z[f"f{q}"], origin=tuple(z[f"o{q}"].tolist()), spacing=sp, iso=0.0)
                got = ctx.dmc(vol, native.OUT_POS_F64)
                np.testing.assert_array_equal(got["q"], z[f"q{q}"], err_msg=f"crop {q} setting {sname}")
                np.testing.assert_array_equal(got["v64"], z[f"v{q}"], err_msg=f"crop {q} setting {sname}")
                assert got["stats"][3] >= 1
    finally:
        _apply(ctx, default)


@pytest.mark.parametrize("name", ["saddle41", "noise48"])
def test_tmc_identical_under_every_setting(ctx, name):
    vol = CASES[name]
    default = ctx.get_tuning(native.TUNE_EMIT_BLOCKS_PER_SM)
    try:
        want = ctx.tmc(vol, native.OUT_POS_F64, halfedge=True)
        for eb in (1, 3, 64):
            ctx.set_tuning(native.TUNE_EMIT_BLOCKS_PER_SM, eb)
            _same(ctx.tmc(vol, native.OUT_POS_F64, halfedge=True), want, f"{name} emit blocks {eb}")
    finally:
        ctx.set_tuning(native.TUNE_EMIT_BLOCKS_PER_SM, default)


def test_tuning_keys_are_checked(ctx):
    with pytest.raises(native.TmcError):
        ctx.set_tuning(99, 1)
    with pytest.raises(native.TmcError):
        ctx.set_tuning(native.TUNE_VERTEX_BLOCKS_PER_SM, 0)
    with pytest.raises(native.TmcError):
        ctx.set_tuning(native.TUNE_GROUP_LANES, -1)
    old = ctx.get_tuning(native.TUNE_WARP_LIST_MAX)
    ctx.set_tuning(native.TUNE_WARP_LIST_MAX, 123)
    assert ctx.get_tuning(native.TUNE_WARP_LIST_MAX) == 123
    ctx.set_tuning(native.TUNE_WARP_LIST_MAX, old)


def test_autotune_keeps_meshes():
    c = native.Context(0)
    try:
        vols = V.batch_volumes(6, seed=3, hi=80)
        tv = [native.make_volume(v) for v in vols]
        algos = [native.ALGO_DMC if q % 2 == 0 else native.ALGO_TMC for q in range(len(vols))]
        before = c.batch(vols, algos, [0] * len(vols))
        ms = c.autotune(tv, [v.iso for v in vols], algos, [0] * len(vols), rounds=2)
        assert ms > 0
        assert 1 <= c.get_tuning(native.TUNE_VERTEX_BLOCKS_PER_SM) <= 64
        after = c.batch(vols, algos, [0] * len(vols))
        for q in range(len(vols)):
            for k in KEYS:
                np.testing.assert_array_equal(before[q][k], after[q][k], err_msg=f"volume {q}: {k}")
    finally:
        c.close()
