"""The slab generators used by the workload parity tests reproduce the same planes of the full-size
workloads element for element (checked here on grids small enough to build whole)."""
import numpy as np

from tmc_gb300 import volumes as V


def test_saddle_slab_equals_planes_of_the_whole_grid():
    full = V.saddle_volume(200, seed=3)
    for z0, planes in ((0, 10), (60, 16), (120, 80), (190, 10)):
        s = V.saddle_slab(200, z0, planes, seed=3)
        np.testing.assert_array_equal(s.data, full.data[z0:z0 + planes])
        assert s.spacing == full.spacing
        assert s.origin[2] == -1.0 + z0 * full.spacing[2]


def test_z_slab_moves_the_origin():
    vol = V.small_noise_volume(24, seed=3)
    s = V.z_slab(vol, 5, 7)
    np.testing.assert_array_equal(s.data, vol.data[5:12])
    assert s.origin[:2] == vol.origin[:2] and s.origin[2] == vol.origin[2] + 5 * vol.spacing[2]
