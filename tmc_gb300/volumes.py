"""Seeded synthetic scalar fields on uniform grids (float32, x fastest, z slowest).

These play the part of the reference's volume sources (cpp_dmc/Volumes.h:107-140 implicit
surfaces sampled on [-1,1]^3, dmc/UniformGrid.cu:21-223 the `volume` kernel).  The reference
ships no datasets, so every workload here is generated from a seed with numpy's PCG64.

Grids span [-1,1] on every axis: origin -1, spacing 2/(n-1) per axis, the same layout as
UniformGrid::init over a [-1,1]^3 bounding box (cpp_dmc/UniformGrid.cpp:86-119).
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np


@dataclass
class Volume:
    """A uniform grid with its scalar field.  `data` has shape (nz, ny, nx)."""

    data: np.ndarray
    origin: tuple = (-1.0, -1.0, -1.0)
    spacing: tuple = (0.0, 0.0, 0.0)
    iso: float = 0.0
    kind: str = ""
    meta: dict = field(default_factory=dict)

    @property
    def dims(self):
        nz, ny, nx = self.data.shape
        return nx, ny, nz

    @property
    def cells(self) -> int:
        nx, ny, nz = self.dims
        return (nx - 1) * (ny - 1) * (nz - 1)


def _axis(n: int) -> np.ndarray:
    return -1.0 + np.arange(n, dtype=np.float64) * (2.0 / (n - 1))


def _spacing(nx, ny, nz):
    return (2.0 / (nx - 1), 2.0 / (ny - 1), 2.0 / (nz - 1))


def gaussian_blobs(nx: int, ny: int, nz: int, rng: np.random.Generator, nblobs: int = 8) -> np.ndarray:
    """f(x) = sum_i exp(-|x-c_i|^2 / (2 s_i^2)), c_i ~ U[-0.6,0.6]^3, s_i ~ U[0.15,0.35]."""
    c = rng.uniform(-0.6, 0.6, size=(nblobs, 3))
    s = rng.uniform(0.15, 0.35, size=nblobs)
    x, y, z = _axis(nx), _axis(ny), _axis(nz)
    out = np.zeros((nz, ny, nx), dtype=np.float64)
    for i in range(nblobs):
        inv = 1.0 / (2.0 * s[i] * s[i])
        ex = np.exp(-((x - c[i, 0]) ** 2) * inv)
        ey = np.exp(-((y - c[i, 1]) ** 2) * inv)
        ez = np.exp(-((z - c[i, 2]) ** 2) * inv)
        out += ez[:, None, None] * ey[None, :, None] * ex[None, None, :]
    return out.astype(np.float32)


def periodic(nx: int, ny: int, nz: int, k: float, zslab: int = 64, planes: tuple | None = None) -> np.ndarray:
    """sin(kx)cos(ky) + sin(ky)cos(kz) + sin(kz)cos(kx), evaluated slab by slab.  `planes` = (z0, z1)
    returns only those z-planes of the nz-plane grid (the same values, element for element)."""
    x, y, z = _axis(nx), _axis(ny), _axis(nz)
    p0, p1 = planes if planes is not None else (0, nz)
    z = z[p0:p1]
    sx, cx = np.sin(k * x), np.cos(k * x)
    sy, cy = np.sin(k * y), np.cos(k * y)
    sz, cz = np.sin(k * z), np.cos(k * z)
    out = np.empty((p1 - p0, ny, nx), dtype=np.float32)
    for z0 in range(0, p1 - p0, zslab):
        z1 = min(p1 - p0, z0 + zslab)
        a = sx[None, None, :] * cy[None, :, None]
        b = sy[None, :, None] * cz[z0:z1, None, None]
        c = sz[z0:z1, None, None] * cx[None, None, :]
        out[z0:z1] = (a + b + c).astype(np.float32)
    return out


def upsampled_noise(n: int, rng: np.random.Generator, coarse: int = 33, noise: float = 0.02,
                    zslab: int = 32) -> np.ndarray:
    """A coarse^3 grid of U[-1,1] values trilinearly upsampled to n^3 (fine index i maps to coarse
    coordinate i*(coarse-1)/(n-1)), plus noise*N(0,1) per voxel."""
    g = rng.uniform(-1.0, 1.0, size=(coarse, coarse, coarse))
    t = np.arange(n, dtype=np.float64) * ((coarse - 1) / (n - 1))
    i0 = np.minimum(np.floor(t).astype(np.int64), coarse - 2)
    w = t - i0
    # separable trilinear interpolation: x, then y, then z (slab by slab)
    gx = g[:, :, i0] * (1 - w)[None, None, :] + g[:, :, i0 + 1] * w[None, None, :]        # (c, c, n)
    gxy = gx[:, i0, :] * (1 - w)[None, :, None] + gx[:, i0 + 1, :] * w[None, :, None]     # (c, n, n)
    out = np.empty((n, n, n), dtype=np.float32)
    for z0 in range(0, n, zslab):
        z1 = min(n, z0 + zslab)
        zz = slice(z0, z1)
        base = gxy[i0[zz]] * (1 - w[zz])[:, None, None] + gxy[i0[zz] + 1] * w[zz][:, None, None]
        base += noise * rng.standard_normal(size=base.shape)
        out[z0:z1] = base.astype(np.float32)
    return out


def seed_saddles(data: np.ndarray, rng: np.random.Generator, frac: float = 0.2, iso: float = 0.0,
                 zslab: int = 64, first_plane: int = 0, total_planes: int | None = None) -> int:
    """Overwrite the four corners of a random subset of a disjoint family of cell faces with a
    bilinear saddle whose asymptotic-decider value (f0 f3 - f1 f2)/(f0 + f3 - f1 - f2) lies within
    1e-6 of `iso` (in practice within a few 1e-8).

    The family is every xy-face whose lower corner has even i and even j: no two of them share a
    grid point, so every overwrite is independent.  Each face of the family is taken with
    probability `frac`.  Returns the number of faces written.

    `data` may hold only the planes first_plane .. first_plane + data.shape[0] of a grid of
    `total_planes` planes: the random draws of the whole grid are replayed and the faces in those
    planes written, so the slab equals the same planes of the whole seeded grid."""
    nz, ny, nx = data.shape
    if total_planes is None:
        total_planes = first_plane + nz
    fi = np.arange(0, nx - 1, 2)
    fj = np.arange(0, ny - 1, 2)
    total = 0
    for z0 in range(0, total_planes, zslab):
        z1 = min(total_planes, z0 + zslab)
        m = rng.random(size=(z1 - z0, fj.size, fi.size)) < frac
        kk, jj, ii = np.nonzero(m)
        if kk.size == 0:
            continue
        a = rng.uniform(0.2, 1.0, size=kk.size)
        b = rng.uniform(0.2, 1.0, size=kk.size)
        c = rng.uniform(0.2, 1.0, size=kk.size)
        a32, b32, c32 = (a.astype(np.float32), b.astype(np.float32), c.astype(np.float32))
        d32 = (a32.astype(np.float64) * b32 / c32).astype(np.float32)
        flip = rng.random(size=kk.size) < 0.5
        s = np.where(flip, -1.0, 1.0).astype(np.float32)
        k = kk + z0 - first_plane
        inside = (k >= 0) & (k < nz)
        if not inside.all():
            k, jj, ii, a32, b32, c32, d32, s = (x[inside] for x in (k, jj, ii, a32, b32, c32, d32, s))
        j = fj[jj]
        i = fi[ii]
        # diagonal sign pattern: corners 0 and 3 on one side, 1 and 2 on the other
        data[k, j, i] = iso + s * a32
        data[k, j + 1, i + 1] = iso + s * b32
        data[k, j, i + 1] = iso - s * c32
        data[k, j + 1, i] = iso - s * d32
        total += k.size
    return total


# ------------------------------------------------------------------------------------------
# The five workloads.  Each returns Volume(s) with their isovalue.
# ------------------------------------------------------------------------------------------

def blobs_volume(n: int = 64, seed: int = 0) -> Volume:
    """64^3 Gaussian-blob field, isovalue 0.5 (plain DMC, no simplification)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    d = gaussian_blobs(n, n, n, rng)
    return Volume(d, spacing=_spacing(n, n, n), iso=0.5, kind="blobs", meta={"seed": seed})


def noise_volume(n: int = 512, seed: int = 1) -> Volume:
    """33^3 uniform noise upsampled to n^3 plus 0.02 N(0,1); isovalue 0 (dense ambiguity)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    d = upsampled_noise(n, rng)
    return Volume(d, spacing=_spacing(n, n, n), iso=0.0, kind="noise", meta={"seed": seed})


def batch_volumes(count: int = 256, seed: int = 2, lo: int = 32, hi: int = 192) -> list:
    """`count` volumes, each axis log-uniform in [lo, hi]; fields alternate between the blob type
    and the periodic type with k ~ U[2pi, 8pi]; isovalue ~ U[-0.3, 0.3]."""
    rng = np.random.Generator(np.random.PCG64(seed))
    out = []
    for v in range(count):
        dims = np.exp(rng.uniform(math.log(lo), math.log(hi), size=3)).astype(np.int64)
        nx, ny, nz = (int(max(lo, min(hi, d))) for d in dims)
        iso = float(rng.uniform(-0.3, 0.3))
        if v % 2 == 0:
            d = gaussian_blobs(nx, ny, nz, rng)
            kind = "blobs"
            k = None
        else:
            k = float(rng.uniform(2 * math.pi, 8 * math.pi))
            d = periodic(nx, ny, nz, k)
            kind = "periodic"
        out.append(Volume(d, spacing=_spacing(nx, ny, nz), iso=iso, kind=kind,
                          meta={"seed": seed, "index": v, "k": k}))
    return out


def saddle_volume(n: int = 1024, seed: int = 3, frac: float = 0.2) -> Volume:
    """Periodic field (k = 6 pi) with seeded near-singular saddle faces; isovalue 0."""
    rng = np.random.Generator(np.random.PCG64(seed))
    d = periodic(n, n, n, 6 * math.pi)
    faces = seed_saddles(d, rng, frac=frac)
    return Volume(d, spacing=_spacing(n, n, n), iso=0.0, kind="saddle",
                  meta={"seed": seed, "saddle_faces": faces})


def saddle_slab(n: int = 1024, z0: int = 0, planes: int = 16, seed: int = 3, frac: float = 0.2) -> Volume:
    """The z-planes z0 .. z0 + planes of saddle_volume(n, seed, frac), bit for bit, without building
    the whole grid: a volume of its own whose origin is the first plane's position."""
    rng = np.random.Generator(np.random.PCG64(seed))
    d = periodic(n, n, n, 6 * math.pi, planes=(z0, z0 + planes))
    faces = seed_saddles(d, rng, frac=frac, first_plane=z0, total_planes=n)
    sp = _spacing(n, n, n)
    return Volume(d, origin=(-1.0, -1.0, -1.0 + z0 * sp[2]), spacing=sp, iso=0.0, kind="saddle",
                  meta={"seed": seed, "saddle_faces": faces, "z0": z0, "n": n})


def z_slab(vol: Volume, z0: int, planes: int) -> Volume:
    """Planes z0 .. z0 + planes of a volume, as a volume of its own (origin moved to the first plane)."""
    d = np.ascontiguousarray(vol.data[z0:z0 + planes])
    return Volume(d, origin=(vol.origin[0], vol.origin[1], vol.origin[2] + z0 * vol.spacing[2]),
                  spacing=vol.spacing, iso=vol.iso, kind=vol.kind, meta=dict(vol.meta, z0=z0))


def serve_request(rng: np.random.Generator, median: int = 128, sigma: float = 0.5,
                  lo: int = 48, hi: int = 512) -> Volume:
    """One serving request: per-axis size lognormal (median 128, sigma 0.5) clipped to [48, 512];
    field type and isovalue as in the batched workload."""
    dims = np.clip(np.round(np.exp(math.log(median) + sigma * rng.standard_normal(3))), lo, hi).astype(int)
    nx, ny, nz = (int(d) for d in dims)
    iso = float(rng.uniform(-0.3, 0.3))
    if rng.random() < 0.5:
        d = gaussian_blobs(nx, ny, nz, rng)
        kind = "blobs"
    else:
        d = periodic(nx, ny, nz, float(rng.uniform(2 * math.pi, 8 * math.pi)))
        kind = "periodic"
    return Volume(d, spacing=_spacing(nx, ny, nz), iso=iso, kind=kind)


def small_noise_volume(n: int = 32, seed: int = 11, coarse: int = 5) -> Volume:
    """A small dense-ambiguity field in the style of the 512^3 workload (for parity tests)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    d = upsampled_noise(n, rng, coarse=coarse)
    return Volume(d, spacing=_spacing(n, n, n), iso=0.0, kind="noise", meta={"seed": seed})
