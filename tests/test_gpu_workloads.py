"""Parity on the benchmark workloads themselves, not only on small fields.

* The 512^3 dense-ambiguity field of the default benchmark (33^3 U[-1,1] upsampled + 0.02 N(0,1),
  seed 1, isovalue 0): three z-slabs of 24 planes (the bottom boundary, the interior, the top
  boundary), each extracted as a volume of its own with DMC (P3X3Y colour + isolated + P3333,
  halfedges, triangles) and with TMC.
* The 1024^3 precision-stress field (periodic, k = 6 pi, 20 % of a disjoint face family seeded with
  bilinear saddles whose decider lies within 1e-6 of the isovalue 0): two slabs of 16 planes of
  1024^2, generated plane for plane as in the full grid without building it.
* The 256-volume batch of uneven sizes: every mesh of one batched call equal to the same volume
  extracted alone, and every 16th volume equal to the oracle.
* The face colouring and vertex valence stage on its own (tmc_dmc_color_valence) against the
  oracle's colorFaces + vertexValence, on the front-end meshes of these workloads.

Tolerances: topology (quads, triangles including the quad split, halfedges, TMC triangles), the
float64 positions and the colours and valences bit-exact; float32 positions within 2 float32 ulps
of the oracle's float64 values (their max and RMS error in cell units is printed), normals as in
test_gpu_dmc.py."""
import numpy as np
import pytest

from tmc_gb300 import volumes as V

from test_gpu_dmc import NORMAL_ABS_TOL, _close32, split_differences

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    from tmc_gb300 import native
    c = native.Context(0)
    yield c
    c.close()


@pytest.fixture(scope="module")
def noise512():
    return V.noise_volume(512, seed=1)


def _position_error(v32, v64, spacing):
    """max and RMS |float32 - float64| per coordinate, in cells"""
    if v64.size == 0:
        return 0.0, 0.0
    err = np.abs(v32.reshape(-1, 3).astype(np.float64) - v64.reshape(-1, 3)) / np.asarray(spacing)
    return float(err.max()), float(np.sqrt(np.mean(err ** 2)))


def _check_dmc(ctx, oracle, vol, label):
    from tmc_gb300 import native
    want = oracle.dmc(vol, 1)
    got = ctx.dmc(vol, native.OUT_POS_F64 | native.OUT_TRIANGLES | native.OUT_HALFEDGES | native.DMC_SIMPLIFY)
    assert got["q"].size > 0
    np.testing.assert_array_equal(got["q"], want["q"])
    np.testing.assert_array_equal(got["v64"], want["v"])
    assert _close32(got["v"], want["v"])
    assert _close32(got["n"], want["n"], ulps=2, abs_tol=NORMAL_ABS_TOL)
    np.testing.assert_array_equal(got["he"].reshape(-1, 4), want["he"].reshape(-1, 5)[:, :4])
    np.testing.assert_array_equal(got["hv"], want["hv"])
    np.testing.assert_array_equal(got["hf"], want["hf"])
    nsplit = split_differences(got["t"], want["t"])
    emax, erms = _position_error(got["v"], want["v"], vol.spacing)
    print(f"{label} DMC: {got['v'].size // 3} vertices, {got['q'].size // 4} quads, ambiguous cells "
          f"{got['stats'][1]}, split differences {nsplit}, float32 position error max {emax:.3g} rms {erms:.3g} cells")
    assert nsplit == 0
    return got


def _check_tmc(ctx, oracle, vol, label):
    from tmc_gb300 import native
    want = oracle.tmc(vol)
    got = ctx.tmc(vol, native.OUT_POS_F64)
    assert got["t"].size > 0
    np.testing.assert_array_equal(got["t"], want["t"])
    np.testing.assert_array_equal(got["v64"], want["v"])
    assert _close32(got["v"], want["v"])
    assert _close32(got["n"], want["n"])
    emax, erms = _position_error(got["v"], want["v"], vol.spacing)
    print(f"{label} TMC: {got['v'].size // 3} vertices, {got['t'].size // 3} triangles, ambiguous cells "
          f"{got['stats'][1]}, float32 position error max {emax:.3g} rms {erms:.3g} cells")
    return got


SLABS_512 = [(0, 24), (244, 24), (488, 24)]


@pytest.mark.parametrize("z0,planes", SLABS_512)
def test_noise512_slab_dmc(ctx, oracle, noise512, z0, planes):
    got = _check_dmc(ctx, oracle, V.z_slab(noise512, z0, planes), f"512^3 slab z{z0}+{planes}")
    assert got["stats"][1] > 0  # the slab has ambiguous cells


@pytest.mark.parametrize("z0,planes", SLABS_512)
def test_noise512_slab_tmc(ctx, oracle, noise512, z0, planes):
    got = _check_tmc(ctx, oracle, V.z_slab(noise512, z0, planes), f"512^3 slab z{z0}+{planes}")
    assert got["stats"][1] > 0


SLABS_1024 = [(0, 16), (600, 16)]


@pytest.fixture(scope="module", params=SLABS_1024, ids=lambda p: f"z{p[0]}")
def saddle_slab(request):
    z0, planes = request.param
    return V.saddle_slab(1024, z0, planes, seed=3)


def test_saddle1024_slab_dmc(ctx, oracle, saddle_slab):
    got = _check_dmc(ctx, oracle, saddle_slab, f"1024^3 saddle slab z{saddle_slab.meta['z0']}")
    assert saddle_slab.meta["saddle_faces"] > 100000
    assert got["stats"][1] > 100000


def test_saddle1024_slab_tmc(ctx, oracle, saddle_slab):
    got = _check_tmc(ctx, oracle, saddle_slab, f"1024^3 saddle slab z{saddle_slab.meta['z0']}")
    assert got["stats"][1] > 100000


def test_batch256_equals_solo_and_oracle(ctx, oracle):
    """The batched workload as the benchmark runs it (256 volumes, seed 2), DMC shared-vertex quads
    with float64 positions."""
    from tmc_gb300 import native
    vols = V.batch_volumes(256, seed=2)
    outs = ctx.batch(vols, [native.ALGO_DMC] * len(vols), [native.OUT_POS_F64] * len(vols))
    assert len(outs) == len(vols)
    for i, (vol, got) in enumerate(zip(vols, outs)):
        solo = ctx.dmc(vol, native.OUT_POS_F64)
        np.testing.assert_array_equal(got["q"], solo["q"])
        np.testing.assert_array_equal(got["v64"], solo["v64"])
        if i % 16 == 0:
            want = oracle.dmc(vol, 0)
            np.testing.assert_array_equal(got["q"], want["q"])
            np.testing.assert_array_equal(got["v64"], want["v"])


def _color_case(name):
    if name == "noise512_slab":
        return V.z_slab(V.noise_volume(512, seed=1), 244, 24)
    if name == "saddle1024_slab":
        return V.saddle_slab(1024, 300, 12, seed=3)
    if name == "blobs64":
        return V.blobs_volume(64, seed=0)
    return V.small_noise_volume(48, seed=5, coarse=7)


@pytest.mark.parametrize("name", ["noise48", "blobs64", "noise512_slab", "saddle1024_slab"])
def test_color_valence_stage(ctx, oracle, name):
    """colorFaces + vertexValence (cpp_dmc/DualMarchingCubes.cpp:714-871) on the front-end mesh, given
    the same quads and inherited colours: colours and valences bit-equal."""
    vol = _color_case(name)
    front = oracle.dmc_front(vol)
    nv, q, inherited = front["v"].size // 3, front["q"], front["colors"]
    assert q.size > 0
    want_col, want_val = oracle.color_valence(nv, q, inherited)
    got_col, got_val = ctx.dmc_color_valence(nv, q, inherited)
    np.testing.assert_array_equal(got_val, want_val)
    np.testing.assert_array_equal(got_col, want_col)
    assert set(np.unique(got_col).tolist()) <= {0, 1, 2, 3, 4}
