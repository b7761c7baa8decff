"""tmc_server_*: continuous batching of requests.

Requests of different sizes, algorithms and outputs are submitted from several threads while
batches run; every result must equal the same request extracted alone by the single-volume entry
points (bit-exact arrays), whatever batch it landed in.
"""
import threading

import numpy as np
import pytest

from tmc_gb300 import native
from tmc_gb300 import volumes as V

pytestmark = pytest.mark.gpu

KEYS = ("v", "n", "v64", "q", "t", "he", "hv", "hf")


@pytest.fixture(scope="module")
def ctx():
    c = native.Context(0)
    yield c
    c.close()


def _requests():
    vols = V.batch_volumes(10, seed=7, hi=96)
    vols.append(V.small_noise_volume(40, seed=3))
    vols.append(V.Volume(np.zeros((5, 6, 7), np.float32), spacing=(0.1, 0.1, 0.1), iso=0.5))  # empty
    kinds = [(native.ALGO_DMC, 0), (native.ALGO_DMC, native.OUT_HALFEDGES), (native.ALGO_TMC, 0),
             (native.ALGO_TMC, native.OUT_HALFEDGES), (native.ALGO_DMC, native.DMC_SIMPLIFY | native.OUT_TRIANGLES),
             (native.ALGO_TMC, native.OUT_POS_F64)]
    return [(v, kinds[q % len(kinds)][0], kinds[q % len(kinds)][1]) for q, v in enumerate(vols)]


def _alone(ctx, vol, algo, flags):
    if algo == native.ALGO_DMC:
        return ctx.dmc(vol, flags)
    return ctx.tmc(vol, flags & ~native.OUT_HALFEDGES, halfedge=bool(flags & native.OUT_HALFEDGES))


def _same(a, b, what):
    for k in KEYS:
        np.testing.assert_array_equal(a[k], b[k], err_msg=f"{what}: {k}")


def _serve(srv, reqs, threads=3):
    """Submit from several threads, collect every result; returns results in request order."""
    tv = [native.make_volume(v) for v, _, _ in reqs]
    tickets = [None] * len(reqs)
    results = [None] * len(reqs)

    def submitter(part):
        for q in part:
            tickets[q] = srv.submit(tv[q], reqs[q][0].iso, reqs[q][1], reqs[q][2] | native.OUT_HOST)

    parts = [list(range(t, len(reqs), threads)) for t in range(threads)]
    ths = [threading.Thread(target=submitter, args=(p,)) for p in parts]
    for t in ths:
        t.start()
    for t in ths:
        t.join()
    for q in range(len(reqs)):
        results[q] = srv.wait(tickets[q])
    return results


def test_server_results_equal_alone(ctx):
    reqs = _requests()
    srv = native.Server(0)
    try:
        got = _serve(srv, reqs)
        st = srv.stats()
    finally:
        srv.close()
    assert st[0] == st[1] == len(reqs)
    for q, (vol, algo, flags) in enumerate(reqs):
        _same(got[q], _alone(ctx, vol, algo, flags), f"request {q} algo {algo} flags {flags:#x}")


def test_server_admission_by_budget(ctx):
    """A budget below any request's footprint admits one request at a time; results unchanged."""
    reqs = _requests()[:6]
    srv = native.Server(0, hbm_budget=1, workers=2)
    try:
        got = _serve(srv, reqs, threads=2)
        st = srv.stats()
    finally:
        srv.close()
    assert st[5] == 1  # largest batch
    assert st[4] > 1   # peak admitted bytes: one request's estimate
    for q, (vol, algo, flags) in enumerate(reqs):
        _same(got[q], _alone(ctx, vol, algo, flags), f"request {q}")


def test_server_batch_cell_cap(ctx):
    """A cell cap below every request's size puts each request in a batch of its own; results unchanged."""
    reqs = _requests()[:5]
    srv = native.Server(0, workers=2, max_batch_cells=1)
    try:
        got = _serve(srv, reqs, threads=2)
        st = srv.stats()
    finally:
        srv.close()
    assert st[5] == 1  # largest batch
    for q, (vol, algo, flags) in enumerate(reqs):
        _same(got[q], _alone(ctx, vol, algo, flags), f"request {q}")


def test_server_poll_wait_and_errors():
    vol = V.small_noise_volume(24, seed=5)
    tv = native.make_volume(vol)
    srv = native.Server(0, workers=1)
    try:
        t = srv.submit(tv, vol.iso, native.ALGO_DMC, native.OUT_HOST)
        m = srv.wait_raw(t, timeout=60.0)
        assert m.nr_v > 0 and m.on_device == 0
        srv.release(m)
        with pytest.raises(native.TmcError):
            srv.wait_raw(t)  # already collected
        with pytest.raises(native.TmcError):
            srv.submit(tv, vol.iso, 9, 0)  # unknown algorithm
        # malformed requests are refused at submission, so they cannot fail a batch
        bad = native.make_volume(vol)
        bad.spacing = (type(bad.spacing))(0.0, 1.0, 1.0)
        with pytest.raises(native.TmcError) as e:
            srv.submit(bad, vol.iso, native.ALGO_DMC, native.OUT_HOST)
        assert e.value.status == native.TMC_ERR_INVALID_ARG
        with pytest.raises(native.TmcError):
            srv.submit(tv, vol.iso, native.ALGO_TMC, native.DMC_SIMPLIFY)
    finally:
        srv.close()
