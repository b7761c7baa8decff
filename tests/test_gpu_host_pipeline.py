"""Host fields and host results at sizes where the runtime overlaps copies with kernels.

A host field of 64 MiB or more is copied in z slabs on the context's copy stream, and the
classification of each range of scan tiles starts once the planes it reads have arrived.  With
TMC_OUT_HOST, result arrays that no later kernel writes are copied out on the copy stream while
the call's remaining kernels run.  Both must give the same meshes, bit for bit, as a device
field with device-resident results.  The context option check_numeric rejects a field that holds
NaN or Inf (TMC_ERR_NUMERIC), for host and device fields alike.
"""
import numpy as np
import pytest
import torch

from tmc_gb300 import native
from tmc_gb300 import volumes as V

pytestmark = pytest.mark.gpu

DMC_FLAGS = native.DMC_SIMPLIFY | native.OUT_HALFEDGES | native.OUT_TRIANGLES
KEYS = ("v", "n", "v64", "q", "t", "he", "hv", "hf")


@pytest.fixture(scope="module")
def ctx():
    c = native.Context(0)
    yield c
    c.close()


class _DevArray:
    """A device array of a mesh, seen by torch through __cuda_array_interface__."""

    def __init__(self, ptr, count, dtype):
        self.__cuda_array_interface__ = {"shape": (count,), "typestr": np.dtype(dtype).str, "data": (ptr, False),
                                         "version": 3}


def _device_mesh(ctx, m):
    """Arrays of a device-resident mesh, copied by torch (independent of the runtime's copies)."""
    assert m.on_device == 1

    def arr(ptr, count, dtype):
        if not ptr or count == 0:
            return np.zeros(0, dtype)
        return torch.as_tensor(_DevArray(ptr, count, dtype), device="cuda").cpu().numpy().copy()

    nv, nq, nt, nh = m.nr_v, m.nr_q, m.nr_t, m.nr_he
    out = dict(v=arr(m.v, 3 * nv, np.float32), n=arr(m.n, 3 * nv, np.float32), v64=arr(m.v64, 3 * nv, np.float64),
               q=arr(m.quads, 4 * nq, np.int32), t=arr(m.tris, 3 * nt, np.int32), he=arr(m.he, 4 * nh, np.int32),
               hv=arr(m.he_v, nv if m.he_v else 0, np.int32),
               hf=arr(m.he_f, (nq if nq else nt) if m.he_f else 0, np.int32))
    ctx.free(m)
    return out


def _volume(name):
    if name == "periodic":  # 310 x 290 x 330 floats = 119 MB: three slabs of uneven plane counts
        return V.Volume(V.periodic(310, 290, 330, k=9.0), spacing=(0.5, 0.25, 0.75), iso=0.1)
    return V.noise_volume(400, seed=17)  # 400^3 = 256 MB: eight slabs, dense ambiguous cells


@pytest.mark.parametrize("name", ["periodic", "noise"])
def test_host_field_and_results_match_device(ctx, name):
    vol = _volume(name)
    dev = torch.from_numpy(vol.data).cuda()
    vdev = native.make_volume(vol, dev.data_ptr(), on_device=True)
    host = torch.from_numpy(vol.data).pin_memory()
    vhost = native.make_volume(vol, host.data_ptr(), on_device=False)
    for algo in ("dmc", "tmc"):
        for f64 in (0, native.OUT_POS_F64):
            if algo == "dmc":
                want = _device_mesh(ctx, ctx.dmc_raw(vdev, vol.iso, DMC_FLAGS | f64))
                got = ctx.fetch(ctx.dmc_raw(vhost, vol.iso, DMC_FLAGS | f64 | native.OUT_HOST))
            else:
                want = _device_mesh(ctx, ctx.tmc_raw(vdev, vol.iso, f64, True))
                got = ctx.fetch(ctx.tmc_raw(vhost, vol.iso, f64 | native.OUT_HOST, True))
            assert want["v"].size > 0 and want["he"].size > 0
            for k in KEYS:
                np.testing.assert_array_equal(got[k], want[k], err_msg=f"{name} {algo} f64={bool(f64)}: {k}")
    # pageable host memory takes the same slab path
    got = ctx.fetch(ctx.dmc_raw(native.make_volume(vol), vol.iso, DMC_FLAGS | native.OUT_HOST))
    want = _device_mesh(ctx, ctx.dmc_raw(vdev, vol.iso, DMC_FLAGS))
    for k in KEYS:
        np.testing.assert_array_equal(got[k], want[k], err_msg=f"{name} pageable: {k}")


@pytest.mark.parametrize("bad", [np.nan, np.inf, -np.inf])
def test_check_numeric(bad):
    vol = V.blobs_volume(40, seed=3)
    data = vol.data.copy()
    data[17, 5, 33] = bad
    badvol = V.Volume(data, spacing=vol.spacing, iso=vol.iso)
    strict = native.Context(0, check_numeric=True)
    try:
        # a clean field passes
        assert strict.dmc(vol)["q"].size > 0
        for on_device in (False, True):
            if on_device:
                dev = torch.from_numpy(data).cuda()
                tv = native.make_volume(badvol, dev.data_ptr(), on_device=True)
            else:
                tv = native.make_volume(badvol)
            for call in (lambda: strict.dmc_raw(tv, vol.iso, native.OUT_HOST),
                         lambda: strict.tmc_raw(tv, vol.iso, native.OUT_HOST)):
                with pytest.raises(native.TmcError) as e:
                    call()
                assert e.value.status == native.TMC_ERR_NUMERIC
        # the context stays usable after the error
        assert strict.tmc(vol)["t"].size > 0
    finally:
        strict.close()


def test_check_numeric_in_a_batch():
    """A batch that holds one field with NaN fails as a whole with TMC_ERR_NUMERIC on a context that
    checks fields; the same context then runs a clean batch."""
    good = V.blobs_volume(24, seed=1)
    data = good.data.copy()
    data[3, 4, 5] = np.nan
    bad = V.Volume(data, spacing=good.spacing, iso=good.iso)
    strict = native.Context(0, check_numeric=True)
    try:
        with pytest.raises(native.TmcError) as e:
            strict.batch([good, bad], [native.ALGO_DMC, native.ALGO_TMC], [0, 0])
        assert e.value.status == native.TMC_ERR_NUMERIC
        out = strict.batch([good, good], [native.ALGO_DMC, native.ALGO_TMC], [0, 0])
        assert out[0]["q"].size > 0 and out[1]["t"].size > 0
    finally:
        strict.close()
