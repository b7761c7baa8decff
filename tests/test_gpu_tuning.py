"""Launch-shape settings (tmc_ctx_set_tuning) and the autotuner (tmc_ctx_autotune).

The settings choose between kernels that compute the same values: one thread per vertex or a group
of lanes per vertex for the DMC projection, one thread or one warp per float64-fallback vertex, and
the grid sizes of the per-vertex, quad and TMC emission passes, and the slab depth and count of a
host field's copy/classification pipeline.  Every setting must give bit-identical
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
             native.TUNE_EMIT_BLOCKS_PER_SM, native.TUNE_QUAD_BLOCKS_PER_SM, native.TUNE_SLAB_MIB,
             native.TUNE_MAX_SLABS)

# (group lanes, warp list max, vertex blocks per SM, emit blocks per SM, quad blocks per SM,
#  slab MiB, max slabs)
SETTINGS = {
    "threads": (0, 0, 32, 8, 1, 32, 16),              # one thread per vertex, 26x26 retries by warp
    "lanes": (1 << 40, 1 << 30, 32, 8, 4, 128, 4),    # lane groups and whole lists by warp wherever possible
    "small_grids": (0, 1 << 30, 1, 1, 1, 4, 64),      # minimal grids, thin slabs: every loop takes many turns
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


def test_host_field_slab_shapes(ctx):
    """A host field copied in slabs of every tuned depth and count (4 MiB to one slab per field, 2 to
    64 slabs) extracts the same meshes as the same field on the device."""
    vol = V.small_noise_volume(160, seed=4, coarse=9)  # 16 MiB
    default = tuple(ctx.get_tuning(k) for k in (native.TUNE_SLAB_MIB, native.TUNE_MAX_SLABS))
    want_d = ctx.dmc(vol, native.OUT_POS_F64 | native.OUT_TRIANGLES | native.OUT_HALFEDGES | native.DMC_SIMPLIFY)
    want_t = ctx.tmc(vol, native.OUT_POS_F64)
    try:
        for mib, slabs in ((4, 2), (4, 64), (8, 3), (16, 16), (1024, 64)):
            ctx.set_tuning(native.TUNE_SLAB_MIB, mib)
            ctx.set_tuning(native.TUNE_MAX_SLABS, slabs)
            got = ctx.dmc(vol, native.OUT_POS_F64 | native.OUT_TRIANGLES | native.OUT_HALFEDGES | native.DMC_SIMPLIFY)
            _same(got, want_d, f"slabs {mib} MiB x {slabs}")
            _same(ctx.tmc(vol, native.OUT_POS_F64), want_t, f"TMC slabs {mib} MiB x {slabs}")
    finally:
        ctx.set_tuning(native.TUNE_SLAB_MIB, default[0])
        ctx.set_tuning(native.TUNE_MAX_SLABS, default[1])


def test_autotune_single_host_volume_tunes_slabs():
    """One request with a host field: the autotuner times the single-volume path and reports the
    slab depth and count it chose; the meshes stay the same."""
    import torch
    c = native.Context(0)
    try:
        vol = V.small_noise_volume(192, seed=6, coarse=9)  # 27 MiB
        pin = torch.from_numpy(vol.data).pin_memory()
        tv = native.make_volume(vol, pin.data_ptr(), on_device=False)
        before = c.dmc(vol, 0)
        ms = c.autotune([tv], [vol.iso], [native.ALGO_DMC], [0], rounds=2)
        assert ms > 0
        assert 4 <= c.get_tuning(native.TUNE_SLAB_MIB) <= 1024
        assert 2 <= c.get_tuning(native.TUNE_MAX_SLABS) <= 64
        after = c.dmc(vol, 0)
        for k in KEYS:
            np.testing.assert_array_equal(before[k], after[k], err_msg=k)
    finally:
        c.close()


def test_tuning_keys_are_checked(ctx):
    with pytest.raises(native.TmcError):
        ctx.set_tuning(99, 1)
    with pytest.raises(native.TmcError):
        ctx.set_tuning(native.TUNE_VERTEX_BLOCKS_PER_SM, 0)
    with pytest.raises(native.TmcError):
        ctx.set_tuning(native.TUNE_GROUP_LANES, -1)
    with pytest.raises(native.TmcError):
        ctx.set_tuning(native.TUNE_SLAB_MIB, 3)
    with pytest.raises(native.TmcError):
        ctx.set_tuning(native.TUNE_MAX_SLABS, 1)
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
