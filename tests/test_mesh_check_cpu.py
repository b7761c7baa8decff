"""The numpy mesh check (tests/mesh_check_np.py) pinned against the reference's own connectivity()
(mc/MarchingCubes.cpp:1769-2226) on the reference's t_mc meshes: the same number of components, and
no orientation to change.  test_gpu_mesh_stats.py then holds tmc_mesh_check to the numpy check."""
import numpy as np
import pytest

from tmc_gb300 import volumes as V

import cpu_libs
from mesh_check_np import mesh_check_np

pytestmark = pytest.mark.skipif(not cpu_libs.ref_available(), reason="the reference is not compiled here (oracle/_ref)")


def _cases():
    # fields whose meshes have at most two faces per edge: on edges with three or more (the seeded
    # saddles of the precision workload make some) the reference links a face to the first other
    # face it finds and its walk then depends on the visiting order
    return {"noise24": V.small_noise_volume(24, seed=4), "noise32": V.small_noise_volume(32, seed=9, coarse=6),
            "blobs30": V.blobs_volume(30, seed=6)}


@pytest.mark.parametrize("name", sorted(_cases()))
def test_numpy_check_matches_reference_connectivity(name):
    vol = _cases()[name]
    ref = cpu_libs.RefLib()
    mesh = ref.tmc(vol)
    comps, changed = ref.tmc_connectivity(vol)
    got = mesh_check_np(mesh["v"].size // 3, mesh["t"], 3)
    assert got["nonmanifold_halfedges"] == 0  # TMC meshes have at most two faces per edge
    assert got["components"] == comps > 0
    assert changed == 0 and got["orientation_defects"] == 0
    assert got["degenerate_faces"] == 0
