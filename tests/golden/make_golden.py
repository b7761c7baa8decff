"""Generate the golden fixtures from the reference's own CPU code.

Needs oracle/_ref/libref.so, built from the reference sources by `make -C oracle ref` (only
possible where the reference checkout exists).  Writes:

  tests/golden/golden.npz    full outputs of small cases (fields included)
  tests/golden/digests.json  sha256 digests of the outputs of larger cases (fields are
                             regenerated from their seeds; the field digest is stored too)

Every array is hashed as little-endian raw bytes: float64 for vertices/normals, int32 for
indices.  The reference path: dmc::DualMarchingCubes::dualMC (cpp_dmc/DualMarchingCubes.cpp:5)
and tmc::MarchingCubes::t_mc (mc/MarchingCubes.cpp:151), driven by oracle/ref_*_harness.cpp.
"""
import hashlib
import json
import math
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))

from tmc_gb300 import volumes as V  # noqa: E402
from cpu_libs import RefLib  # noqa: E402

# MC cell configurations from the reference's single-cell study (matlab/t_mc.m:53-94,
# matlab/t_singular.m:59-66): value lists f(1..8) for vertices 0..7, with the isovalue noted
# in the script where it has one, else 0.
MATLAB_CELLS = [
    ("mc3_contour6", [-0.960492426392903, 0.793207329559554, 0.916735525189067, -0.422761282626275,
                      -0.934993247757551, -0.850129305868777, -0.0367116785741896, -0.656740699156587], 0.0),
    ("mc12_contour8", [0.454797708726920, 0.801330575352402, 0.649991492712356, -0.973974554763863,
                       -0.134171007607162, -0.0844698148589140, -0.826313795402046, 0.433391503783462], 0.0),
    ("mc7_contour9", [-15.6504952739285, 2.90290077342601, 24.5454566157887, -24.5274127623786,
                      21.6741877710053, -4.49696327433901, -19.7891575872492, -15.5588482753161], 0.0),
    ("mc7_contour9_b", [1763.0, 1052.0, 1815.0, 1050.0, 960.0, 1325.0, 1150.0, 1260.0], 1233.6),
    ("mc4_tunnel", [-7.70146936482581, -3.21868369245987, -5.44023748418735, 15.6051950593180,
                    12.7611835388515, -4.46952393442309, -11.7240576326183, -9.23038948829007], 0.0),
    ("mc7_tunnel", [-3.42744283804455, 0.621278122151001, 4.48110777981235, -1.95551129669134,
                    2.30448107596369, -1.04182240925489, -3.51087814405650, -6.44976786808517], 0.0),
    ("mc10_tunnel", [-0.1, -6.11, 2, 10.2, 10.8, 1.8, -8.2, -0.18], 0.0),
    ("mc12_tunnel", [-3.37811990337124, 0.473258332744286, 2.54344310345736, 7.87658724379480,
                     4.38700713005133, -1.49950251870885, -4.21025867362045, -1.00233824192217], 0.0),
    ("mc13_tunnel", [2.74742516087490, -3.39187542578189, -12.5297639669456, 0.431517989649243,
                     -6.92460546400188, 2.52228314017858, 14.6950568276448, -10.0732624062474], 0.0),
    ("mc13_contour12", [0.546912886195662, -0.421103532406922, -0.643375084081520, 0.855507421818445,
                        -0.260686312588506, 0.206413666735986, 0.237274227130530, -0.183297728364877], 0.0),
    ("mc13_contour12_b", [1069, 843, 950, 1133, 958, 1029, 1198, 946], 1007.4),
    ("mc13_case16", [0.520482995461163, -0.839814387388296, -0.467491517013617, 0.937814095887345,
                     -0.825777099007084, 0.506695544835103, 0.345318915961394, -0.861107217966913], 0.0293),
    ("singular_a", [2.74742516087490, -3.39187542578189, -12.5297639669456, 0.431517989649243,
                    -6.92460546400188, 2.52228314017858, 14.6950568276448, -10.0732624062474], -1.3064),
    ("singular_b", [-15.6504952739285, 2.90290077342601, 24.5454566157887, -24.5274127623786,
                    21.6741877710053, -4.49696327433901, -19.7891575872492, -15.5588482753161], -1.8061),
]


def digest(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def cell_volume(values, iso):
    d = np.array(values, dtype=np.float32).reshape(2, 2, 2)  # (z, y, x) with v = x + 2y + 4z
    return V.Volume(d, origin=(0.0, 0.0, 0.0), spacing=(1.0, 1.0, 1.0), iso=float(iso), kind="cell")


def singular_volume(n=12, seed=21):
    """Periodic field with xy-faces overwritten by saddles whose decider is exactly 0."""
    rng = np.random.Generator(np.random.PCG64(seed))
    d = V.periodic(n, n, n, 4 * math.pi)
    for k in range(0, n, 3):
        for j in range(0, n - 1, 4):
            for i in range(0, n - 1, 4):
                a, b, c = (float(x) for x in rng.choice([0.25, 0.5, 1.0, 2.0], size=3))
                dd = a * b / c  # exact in binary for these values
                s = 1.0 if rng.random() < 0.5 else -1.0
                d[k, j, i] = s * a
                d[k, j + 1, i + 1] = s * b
                d[k, j, i + 1] = -s * c
                d[k, j + 1, i] = -s * dd
    return V.Volume(d, spacing=(2 / (n - 1),) * 3, iso=0.0, kind="singular")


def small_cases():
    """(name, volume, algorithm, simplify, flip) with full arrays stored."""
    cases = [
        ("blobs16_dmc", V.blobs_volume(16, seed=5), "dmc", 0, 0),
        ("noise16_dmc_simplify", V.small_noise_volume(16, seed=12, coarse=4), "dmc", 1, 0),
        ("noise16_tmc", V.small_noise_volume(16, seed=12, coarse=4), "tmc", 0, 0),
        ("singular12_tmc", singular_volume(), "tmc", 0, 0),
        ("singular12_dmc_simplify", singular_volume(), "dmc", 1, 0),
    ]
    for name, vals, iso in MATLAB_CELLS:
        cases.append((f"cell_{name}_tmc", cell_volume(vals, iso), "tmc", 0, 0))
    return cases


def digest_cases():
    """(name, recipe, algorithm, simplify, flip); recipes are regenerated by the tests."""
    return [
        ("blobs64_dmc", {"fn": "blobs_volume", "kw": {"n": 64, "seed": 0}}, "dmc", 0, 0),
        ("noise64_dmc_simplify", {"fn": "small_noise_volume", "kw": {"n": 64, "seed": 13, "coarse": 9}}, "dmc", 1, 0),
        ("noise64_tmc", {"fn": "small_noise_volume", "kw": {"n": 64, "seed": 13, "coarse": 9}}, "tmc", 0, 0),
        ("saddle48_dmc_simplify", {"fn": "saddle_volume", "kw": {"n": 48, "seed": 3, "frac": 0.5}}, "dmc", 1, 0),
        ("saddle48_tmc", {"fn": "saddle_volume", "kw": {"n": 48, "seed": 3, "frac": 0.5}}, "tmc", 0, 0),
        ("noise32_dmc_simplify_flip", {"fn": "small_noise_volume", "kw": {"n": 32, "seed": 12, "coarse": 5}}, "dmc", 1, 1),
        ("singular32_tmc", {"fn": "singular_volume", "kw": {"n": 32, "seed": 4}}, "tmc", 0, 0),
        ("singular32_dmc_simplify", {"fn": "singular_volume", "kw": {"n": 32, "seed": 4}}, "dmc", 1, 0),
        ("batch3_dmc", {"fn": "batch_volume", "kw": {"index": 3}}, "dmc", 0, 0),
        ("batch6_dmc_simplify", {"fn": "batch_volume", "kw": {"index": 6}}, "dmc", 1, 0),
        ("batch5_tmc", {"fn": "batch_volume", "kw": {"index": 5}}, "tmc", 0, 0),
    ]


def batch_volume(index):
    return V.batch_volumes(count=index + 1, seed=2)[index]


def make_volume(recipe):
    if recipe["fn"] == "singular_volume":
        return singular_volume(**recipe["kw"])
    if recipe["fn"] == "batch_volume":
        return batch_volume(**recipe["kw"])
    return getattr(V, recipe["fn"])(**recipe["kw"])


def main():
    ref = RefLib()
    store = {}
    for name, vol, algo, simp, flip in small_cases():
        store[f"{name}__field"] = vol.data
        store[f"{name}__meta"] = np.array([vol.iso, *vol.origin, *vol.spacing, simp, flip], dtype=np.float64)
        out = ref.dmc(vol, simp, flip) if algo == "dmc" else ref.tmc(vol)
        for k, a in out.items():
            store[f"{name}__{k}"] = a
    np.savez_compressed(os.path.join(HERE, "golden.npz"), **store)
    dig = {}
    for name, recipe, algo, simp, flip in digest_cases():
        vol = make_volume(recipe)
        out = ref.dmc(vol, simp, flip) if algo == "dmc" else ref.tmc(vol)
        dig[name] = {"recipe": recipe, "algo": algo, "simplify": simp, "flip": flip,
                     "field": digest(vol.data),
                     "sizes": {k: int(a.size) for k, a in out.items()},
                     "digests": {k: digest(a) for k, a in out.items()}}
    with open(os.path.join(HERE, "digests.json"), "w") as f:
        json.dump(dig, f, indent=1, sort_keys=True)
    print("wrote", len(store), "arrays and", len(dig), "digests")


if __name__ == "__main__":
    main()
