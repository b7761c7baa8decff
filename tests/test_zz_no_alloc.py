"""tmc_dmc_count_static: DMC mesh sizes from a static device scratch array, without allocating.

Called through the C ABI (ctypes) and compared with the existing entry point tmc_dmc_extract
(nr_v, nr_q, stats[0], stats[1] without simplification).  The counts are integers, so the
tolerance is zero.  Every comparison runs two calls in a row: the scratch is shared by all calls,
and the second call must not see what the first left there.  This file is collected last so that
it also runs after the other GPU tests; it passes alone in a fresh process too.
"""
import ctypes

import numpy as np
import pytest

from tmc_gb300 import native
from tmc_gb300 import volumes as V

pytestmark = pytest.mark.gpu

TOL = 0  # integer counts: exact


def _cases():
    return {
        "noise48": V.small_noise_volume(48, seed=5, coarse=7),
        "blobs64": V.blobs_volume(64, seed=0),
        "batch3": V.batch_volumes(4, seed=2)[3],
        "ragged": V.Volume(V.small_noise_volume(40, seed=9).data[:17, :29, :], spacing=(0.05, 0.04, 0.03),
                           iso=0.02),
        "tiny2": V.Volume(np.array([[[0.0, 1.0], [1.0, 0.0]], [[1.0, 0.0], [0.0, 1.0]]], np.float32),
                          spacing=(1.0, 1.0, 1.0), origin=(0.0, 0.0, 0.0), iso=0.5),
    }


@pytest.fixture(scope="module")
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


@pytest.mark.parametrize("name", sorted(_cases()))
def test_count_static_matches_extract_twice(torch_cuda, name):
    vol = _cases()[name]
    ctx = native.Context(0)
    dev = torch_cuda.from_numpy(np.ascontiguousarray(vol.data, np.float32)).cuda()
    v = native.make_volume(vol, dev.data_ptr(), on_device=True)
    m = ctx.dmc_raw(v, vol.iso, 0)
    want = np.array([m.nr_v, m.nr_q, m.stats[0], m.stats[1]], np.int64)
    ctx.free(m)
    for _ in range(2):
        got = np.array(ctx.dmc_count_static(v, vol.iso), np.int64)
        assert np.all(np.abs(got - want) <= TOL), (got, want)
    ctx.close()


def test_count_static_alternating_volumes(torch_cuda):
    """Two volumes in turn: each call's counts depend only on its own field."""
    cases = _cases()
    ctx = native.Context(0)
    vols = [cases["noise48"], cases["blobs64"]]
    devs = [torch_cuda.from_numpy(np.ascontiguousarray(x.data, np.float32)).cuda() for x in vols]
    tv = [native.make_volume(x, d.data_ptr(), on_device=True) for x, d in zip(vols, devs)]
    want = []
    for x, t in zip(vols, tv):
        m = ctx.dmc_raw(t, x.iso, 0)
        want.append((m.nr_v, m.nr_q, m.stats[0], m.stats[1]))
        ctx.free(m)
    for r in range(4):
        k = r % 2
        assert ctx.dmc_count_static(tv[k], vols[k].iso) == want[k]
    ctx.close()


def test_count_static_allocates_nothing_after_setup(torch_cuda):
    """After the first call (the one-time set-up), further calls leave free device memory unchanged."""
    vol = _cases()["noise48"]
    ctx = native.Context(0)
    dev = torch_cuda.from_numpy(np.ascontiguousarray(vol.data, np.float32)).cuda()
    v = native.make_volume(vol, dev.data_ptr(), on_device=True)
    first = ctx.dmc_count_static(v, vol.iso)
    torch_cuda.cuda.synchronize()
    free0 = torch_cuda.cuda.mem_get_info()[0]
    for _ in range(3):
        assert ctx.dmc_count_static(v, vol.iso) == first
    torch_cuda.cuda.synchronize()
    assert torch_cuda.cuda.mem_get_info()[0] == free0
    ctx.close()


def test_count_static_rejects_oversized_and_host_fields(torch_cuda):
    """Checked on the host before any launch: nothing reads the (small) buffer behind these volumes."""
    ctx = native.Context(0)
    small = torch_cuda.zeros(8, dtype=torch_cuda.float32, device="cuda")
    big = native.Volume()
    big.nx = big.ny = big.nz = 514  # 513^3 cells > 134,217,728
    big.origin = (ctypes.c_double * 3)(0, 0, 0)
    big.spacing = (ctypes.c_double * 3)(1, 1, 1)
    big.data = small.data_ptr()
    big.on_device = 1
    with pytest.raises(native.TmcError) as e:
        ctx.dmc_count_static(big, 0.0)
    assert e.value.status == native.TMC_ERR_CAPACITY
    assert "static scratch limit" in str(e.value)
    host = native.make_volume(_cases()["tiny2"])  # host memory
    with pytest.raises(native.TmcError) as e:
        ctx.dmc_count_static(host, 0.5)
    assert e.value.status == native.TMC_ERR_INVALID_ARG
    # spacing and origin are checked as tmc_dmc_extract checks them
    for spacing, origin in (((0.0, 1.0, 1.0), (0, 0, 0)), ((1.0, -1.0, 1.0), (0, 0, 0)),
                            ((1.0, 1.0, float("nan")), (0, 0, 0)), ((1.0, 1.0, 1.0), (0, float("inf"), 0))):
        bad = native.Volume()
        bad.nx = bad.ny = bad.nz = 2
        bad.origin = (ctypes.c_double * 3)(*origin)
        bad.spacing = (ctypes.c_double * 3)(*spacing)
        bad.data = small.data_ptr()
        bad.on_device = 1
        with pytest.raises(native.TmcError) as e:
            ctx.dmc_count_static(bad, 0.5)
        assert e.value.status == native.TMC_ERR_INVALID_ARG
        with pytest.raises(native.TmcError) as e:
            ctx.dmc_raw(bad, 0.5, 0)
        assert e.value.status == native.TMC_ERR_INVALID_ARG
    # the largest accepted grid: 513^3 points
    ok = native.Volume()
    ok.nx = ok.ny = ok.nz = 513
    ok.origin = (ctypes.c_double * 3)(0, 0, 0)
    ok.spacing = (ctypes.c_double * 3)(1, 1, 1)
    field = torch_cuda.zeros(513 ** 3, dtype=torch_cuda.float32, device="cuda")
    ok.data = field.data_ptr()
    ok.on_device = 1
    assert ctx.dmc_count_static(ok, 0.5) == (0, 0, 0, 0)
    ctx.close()
