"""Generate tests/golden/saddle_crops.npz: small crops of the 1024^3 precision-stress field (the
periodic field with k = 6 pi and seeded near-singular saddles, tmc_gb300.volumes.saddle_volume,
seed 3) around cells whose DMC representative finds no valid projection sample even at 26x26, so
that the reference keeps its float64 mean point (cpp_dmc/DualMarchingCubes.cpp:251-283).

Each crop is the 4x4x4 grid points around one such cell (the cell in the middle, so all its edges
are interior and its vertex is emitted).  The reference outputs of every crop are stored beside it
(float64 vertices and quads of dualMC without simplification, from oracle/_ref/libref.so, built
from the reference sources by `make -C oracle ref`).

The cells were located with the reference's own projection-failure counter on the 10-plane z-slab
starting at z = 341 (the slab the precision workload of bench.py checks).
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))

from tmc_gb300 import volumes as V  # noqa: E402
from cpu_libs import RefLib  # noqa: E402

Z0 = 341
# (i, j, k - Z0) of the cells, from the slab's failure counter
CELLS = [(385, 63, 0), (41, 404, 0), (475, 191, 1), (817, 617, 1), (729, 575, 3), (461, 22, 5), (973, 22, 5),
         (751, 501, 5), (769, 9, 6), (637, 363, 7), (47, 831, 7)]


def main():
    vol = V.saddle_volume(1024, seed=3)
    ref = RefLib()
    out = {}
    for q, (i, j, kl) in enumerate(CELLS):
        k = Z0 + kl
        crop = np.ascontiguousarray(vol.data[k - 1:k + 3, j - 1:j + 3, i - 1:i + 3])
        origin = (vol.origin[0] + (i - 1) * vol.spacing[0], vol.origin[1] + (j - 1) * vol.spacing[1],
                  vol.origin[2] + (k - 1) * vol.spacing[2])
        cv = V.Volume(crop, origin=origin, spacing=vol.spacing, iso=0.0)
        r = ref.dmc(cv, 0)
        out[f"f{q}"] = crop
        out[f"o{q}"] = np.array(origin)
        out[f"v{q}"] = r["v"]
        out[f"q{q}"] = r["q"]
    out["spacing"] = np.array(vol.spacing)
    np.savez_compressed(os.path.join(HERE, "saddle_crops.npz"), **out)


if __name__ == "__main__":
    main()
