"""tmc_batch_extract: many volumes of uneven sizes in one batched pipeline.

Every mesh of a batch must equal the mesh of the same request extracted alone (bit-exact arrays:
positions, normals, quads/triangles, halfedges, local coordinates), whatever else is in the batch.
The single-volume path is itself checked against the oracle (test_gpu_dmc.py, test_gpu_tmc.py).
"""
import numpy as np
import pytest

from tmc_gb300 import native
from tmc_gb300 import volumes as V

pytestmark = pytest.mark.gpu

KEYS = ("v", "n", "v64", "q", "t", "he", "hv", "hf", "vcell", "vuvw")


@pytest.fixture(scope="module")
def ctx():
    c = native.Context(0)
    yield c
    c.close()


def _vols():
    vols = V.batch_volumes(9, seed=4)
    # small and ragged cases: a single cell, a flat slab, an empty field
    vols.append(V.Volume(np.array([[[0.0, 1.0], [1.0, 0.0]], [[1.0, 0.0], [0.0, 1.0]]], np.float32),
                         spacing=(1.0, 1.0, 1.0), origin=(0.0, 0.0, 0.0), iso=0.5))
    vols.append(V.Volume(V.small_noise_volume(40, seed=9).data[:2, :31, :], spacing=(0.05, 0.04, 0.03), iso=0.02))
    vols.append(V.Volume(np.zeros((9, 10, 11), np.float32), spacing=(0.1, 0.1, 0.1), iso=0.5))
    return vols


def _single(ctx, vol, algo, flags):
    if algo == native.ALGO_DMC:
        return ctx.dmc(vol, flags)
    return ctx.tmc(vol, flags & ~native.OUT_HALFEDGES, halfedge=bool(flags & native.OUT_HALFEDGES))


def _same(a, b, what):
    for k in KEYS:
        np.testing.assert_array_equal(a[k], b[k], err_msg=f"{what}: {k}")
    assert a["stats"][6] == b["stats"][6], what


DMC_FLAG_SETS = [0, native.OUT_POS_F64 | native.OUT_LOCAL, native.DMC_SIMPLIFY | native.OUT_TRIANGLES | native.OUT_HALFEDGES,
                 native.GRAD_FLIP | native.OUT_TRIANGLES]
TMC_FLAG_SETS = [0, native.OUT_POS_F64, native.OUT_HALFEDGES]


@pytest.mark.parametrize("fs", range(len(DMC_FLAG_SETS)))
def test_dmc_batch_equals_single_calls(ctx, fs):
    vols = _vols()
    flags = [DMC_FLAG_SETS[(fs + q) % len(DMC_FLAG_SETS)] for q in range(len(vols))]
    got = ctx.batch(vols, [native.ALGO_DMC] * len(vols), flags)
    for q, (vol, f) in enumerate(zip(vols, flags)):
        _same(got[q], _single(ctx, vol, native.ALGO_DMC, f), f"volume {q} flags {f:#x}")


@pytest.mark.parametrize("fs", range(len(TMC_FLAG_SETS)))
def test_tmc_batch_equals_single_calls(ctx, fs):
    vols = _vols()
    flags = [TMC_FLAG_SETS[(fs + q) % len(TMC_FLAG_SETS)] for q in range(len(vols))]
    got = ctx.batch(vols, [native.ALGO_TMC] * len(vols), flags)
    for q, (vol, f) in enumerate(zip(vols, flags)):
        _same(got[q], _single(ctx, vol, native.ALGO_TMC, f), f"volume {q} flags {f:#x}")


def test_mixed_batch_and_order_independence(ctx):
    """DMC and TMC requests in one call; the same requests in reverse order give the same meshes."""
    vols = _vols()
    algos = [native.ALGO_DMC if q % 2 == 0 else native.ALGO_TMC for q in range(len(vols))]
    flags = [0] * len(vols)
    fwd = ctx.batch(vols, algos, flags)
    rev = ctx.batch(vols[::-1], algos[::-1], flags)[::-1]
    for q in range(len(vols)):
        _same(fwd[q], rev[q], f"volume {q}")
        _same(fwd[q], _single(ctx, vols[q], algos[q], 0), f"volume {q} alone")


def test_device_resident_batch(ctx):
    """Fields already on the device; meshes left on the device and freed one by one."""
    torch = pytest.importorskip("torch")
    vols = _vols()[:6]
    devs = [torch.from_numpy(np.ascontiguousarray(v.data, np.float32)).cuda() for v in vols]
    tv = [native.make_volume(v, d.data_ptr(), on_device=True) for v, d in zip(vols, devs)]
    ms = ctx.batch_raw(tv, [v.iso for v in vols], [native.ALGO_DMC] * len(vols), [0] * len(vols))
    want = [ctx.dmc(v, 0) for v in vols]
    for q, m in enumerate(ms):
        assert m.on_device == 1
        assert (m.nr_v, m.nr_q) == (want[q]["v"].size // 3, want[q]["q"].size // 4)
    # free out of order: the shared arrays stay valid until the last mesh goes
    for q in (3, 0, 5, 1, 4, 2):
        ctx.free(ms[q])


def test_batch_rejects_bad_requests(ctx):
    vols = _vols()[:2]
    with pytest.raises(native.TmcError):
        ctx.batch(vols, [native.ALGO_DMC, 7], [0, 0])
    with pytest.raises(native.TmcError):
        ctx.batch(vols, [native.ALGO_TMC, native.ALGO_TMC], [native.DMC_SIMPLIFY, 0])


def _edge_vols():
    rng = np.random.Generator(np.random.PCG64(8))
    return [
        V.Volume(np.round(V.gaussian_blobs(20, 18, 22, rng) * 8).astype(np.float32), spacing=(0.5, 0.25, 0.75),
                 iso=3.0),  # corners exactly at the isovalue
        V.Volume(V.periodic(20000, 3, 4, 900.0), spacing=(1e-3, 0.5, 0.5), iso=0.05),  # long in x
        V.Volume(V.periodic(3, 9000, 5, 400.0), spacing=(0.5, 1e-3, 0.5), iso=-0.1),  # long in y
        V.Volume(V.blobs_volume(24, seed=6).data, spacing=(0.25, 0.5, 0.125), origin=(12345.5, -6789.25, 3.0),
                 iso=0.5),  # far origin
        V.Volume(V.small_noise_volume(24, seed=4).data + np.float32(1000.0), spacing=(1.0, 1.0, 1.0), iso=1000.0),
    ]


@pytest.mark.parametrize("algo,flags", [(native.ALGO_DMC, native.DMC_SIMPLIFY | native.OUT_TRIANGLES | native.OUT_HALFEDGES),
                                        (native.ALGO_DMC, native.OUT_POS_F64 | native.OUT_LOCAL),
                                        (native.ALGO_TMC, native.OUT_POS_F64 | native.OUT_HALFEDGES)])
def test_batch_of_edge_cases_equals_single_calls(ctx, algo, flags):
    """Grids of very different shapes in one cell space (long thin axes, a far origin, corners at
    the isovalue, values near 1000) give each volume the mesh it gets alone."""
    vols = _edge_vols()
    got = ctx.batch(vols, [algo] * len(vols), [flags] * len(vols))
    for q, vol in enumerate(vols):
        _same(got[q], _single(ctx, vol, algo, flags), f"edge volume {q} algo {algo} flags {flags:#x}")
