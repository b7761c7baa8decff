"""Mesh validation metrics on the GPU (tmc_mesh_quality, tmc_mesh_valence) against a numpy
restatement of the reference's definitions (dmc/ElementQuality.h:69-93, dmc/VertexValence.cu):
the valence histogram exactly, the float32 qualities within float32 rounding of the float64 values."""
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


def _quality_ref(v, faces, P):
    p = v.reshape(-1, 3).astype(np.float64)[faces.reshape(-1, P)]

    def corner(a, b, c):
        e1, e2 = b - a, c - a
        cr = np.stack([e1[:, 2] * e2[:, 1] - e1[:, 1] * e2[:, 2], e1[:, 2] * e2[:, 0] - e1[:, 0] * e2[:, 2],
                       e1[:, 0] * e2[:, 1] - e1[:, 1] * e2[:, 0]], 1)
        return np.sqrt((cr ** 2).sum(1)), (e1 ** 2).sum(1), (e2 ** 2).sum(1)

    if P == 4:
        qs = []
        for k in range(4):
            a, n1, n2 = corner(p[:, k], p[:, (k + 1) % 4], p[:, (k + 3) % 4])
            qs.append(2 * a / (n1 + n2))
        return np.min(np.stack(qs, 1), 1)
    a, _, _ = corner(p[:, 0], p[:, 1], p[:, 2])
    l0 = ((p[:, 1] - p[:, 0]) ** 2).sum(1)
    l1 = ((p[:, 2] - p[:, 1]) ** 2).sum(1)
    l2 = ((p[:, 0] - p[:, 2]) ** 2).sum(1)
    ok = (l0 != 0) & (l1 != 0) & (l2 != 0)
    return np.where(ok, 2 * np.sqrt(3.0) * a / np.where(ok, l0 + l1 + l2, 1), 0.0)


def _valence_ref(nv, faces, P):
    f = faces.reshape(-1, P)
    nb = [set() for _ in range(nv)]
    for r in range(P):
        a, b = f[:, r], f[:, (r + 1) % P]
        for x, y in zip(a.tolist(), b.tolist()):
            if x != y:
                nb[x].add(y)
                nb[y].add(x)
    val = np.minimum(np.array([len(s) for s in nb], np.int64), 99)
    h = np.bincount(val, minlength=100)
    last = np.nonzero(h)[0].max() if nv else -1
    return h[:last + 1]


CASES = {"noise40": V.small_noise_volume(40, seed=5, coarse=7), "blobs48": V.blobs_volume(48, seed=2)}


@pytest.mark.parametrize("name", sorted(CASES))
def test_quality_and_valence(ctx, name):
    vol = CASES[name]
    tv = native.make_volume(vol)
    for algo in ("dmc", "dmc_simplified", "tmc"):
        if algo == "tmc":
            m = ctx.tmc_raw(tv, vol.iso, native.OUT_HOST)
            kinds = [(native.FACES_TRIS, 3)]
        else:
            flags = native.OUT_TRIANGLES | native.OUT_HOST | (native.DMC_SIMPLIFY if algo != "dmc" else 0)
            m = ctx.dmc_raw(tv, vol.iso, flags)
            kinds = [(native.FACES_QUADS, 4), (native.FACES_TRIS, 3)]
        try:
            arr = native._host_array
            v = arr(m.v, 3 * m.nr_v, np.float32)
            for faces, P in kinds:
                f = arr(m.quads if P == 4 else m.tris, P * (m.nr_q if P == 4 else m.nr_t), np.int32)
                q, (mn, mx, mean) = ctx.quality(m, faces)
                want = _quality_ref(v, f, P)
                assert q.size == want.size > 0
                np.testing.assert_allclose(q, want, rtol=1e-5, atol=1e-6, err_msg=f"{name} {algo} P={P}")
                assert mn == pytest.approx(float(want.min()), rel=1e-5, abs=1e-6)
                assert mx == pytest.approx(float(want.max()), rel=1e-5, abs=1e-6)
                assert mean == pytest.approx(float(want.mean()), rel=1e-5)
                np.testing.assert_array_equal(ctx.valence(m, faces), _valence_ref(m.nr_v, f, P),
                                              err_msg=f"{name} {algo} P={P}")
        finally:
            ctx.free(m)


def test_metrics_of_device_mesh_equal_host_mesh(ctx):
    vol = CASES["noise40"]
    tv = native.make_volume(vol)
    md = ctx.dmc_raw(tv, vol.iso, 0)
    mh = ctx.dmc_raw(tv, vol.iso, native.OUT_HOST)
    try:
        qd, sd = ctx.quality(md, native.FACES_QUADS)
        qh, sh = ctx.quality(mh, native.FACES_QUADS)
        np.testing.assert_array_equal(qd, qh)
        assert sd == sh
        np.testing.assert_array_equal(ctx.valence(md, native.FACES_QUADS), ctx.valence(mh, native.FACES_QUADS))
        with pytest.raises(native.TmcError):
            ctx.quality(md, native.FACES_TRIS)  # no triangles requested
    finally:
        ctx.free(md)
        ctx.free(mh)


def _check_cases():
    import math
    rng = np.random.Generator(np.random.PCG64(31))
    sad = V.periodic(21, 21, 21, 6 * math.pi)
    V.seed_saddles(sad, rng, frac=0.5)
    return {"noise40": CASES["noise40"], "blobs48": CASES["blobs48"],
            "saddle21": V.Volume(sad, spacing=(0.1, 0.1, 0.1), iso=0.0)}


@pytest.mark.parametrize("name", ["blobs48", "noise40", "saddle21"])
def test_mesh_check_against_numpy(ctx, name):
    """tmc_mesh_check equals the numpy check (pinned to the reference's connectivity() in
    test_mesh_check_cpu.py) on TMC triangle meshes and DMC quad and triangle meshes.  On edges with
    three or more faces the twins follow the halfedge rules, so components are compared only where
    every edge has at most two faces."""
    from mesh_check_np import mesh_check_np
    vol = _check_cases()[name]
    tv = native.make_volume(vol)
    for algo in ("tmc", "dmc"):
        if algo == "tmc":
            m = ctx.tmc_raw(tv, vol.iso, native.OUT_HOST)
            kinds = [(native.FACES_TRIS, 3)]
        else:
            m = ctx.dmc_raw(tv, vol.iso, native.OUT_HOST | native.OUT_TRIANGLES)
            kinds = [(native.FACES_QUADS, 4), (native.FACES_TRIS, 3)]
        try:
            for faces, P in kinds:
                f = native._host_array(m.quads if P == 4 else m.tris, P * (m.nr_q if P == 4 else m.nr_t), np.int32)
                got = ctx.check(m, faces)
                want = mesh_check_np(m.nr_v, f, P)
                keys = list(want)
                if want["nonmanifold_halfedges"]:
                    keys = [k for k in keys if k not in ("components", "boundary_edges", "boundary_vertices")]
                for k in keys:
                    assert got[k] == want[k], (name, algo, P, k, got, want)
                if name != "saddle21":
                    assert got["orientation_defects"] == 0
        finally:
            ctx.free(m)


def test_mesh_check_unaligned_device_faces(ctx):
    """A caller's device mesh whose quads start 4 bytes into a buffer (not 16-byte aligned) gets
    the counts of the same mesh from host arrays: the per-face twin pass then reads and writes
    without 16-byte vectors."""
    torch = pytest.importorskip("torch")
    vol = V.blobs_volume(40, seed=9)
    d = ctx.dmc(vol, native.OUT_TRIANGLES)
    q, v, n = d["q"], d["v"], d["n"]
    assert q.size > 0
    want = ctx.check(native.host_mesh(v, n, quads=q), native.FACES_QUADS)
    buf = torch.zeros(q.size + 1, dtype=torch.int32, device="cuda")
    buf[1:] = torch.from_numpy(q).cuda()
    vd, nd = torch.from_numpy(v).cuda(), torch.from_numpy(n).cuda()
    m = native.Mesh()
    m.nr_v, m.nr_q, m.on_device = v.size // 3, q.size // 4, 1
    m.v, m.n, m.quads = vd.data_ptr(), nd.data_ptr(), buf.data_ptr() + 4
    assert m.quads % 16 != 0
    assert ctx.check(m, native.FACES_QUADS) == want
