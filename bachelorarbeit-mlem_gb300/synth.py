"""Seeded synthetic phantoms and Poisson sinograms for the benchmark scanners.

Stands in for the reference's measured data (the MADPET-II matrix and a GATE
Derenzo sinogram, not distributed): emission images are sums of seeded
ellipses (2-D) or ellipsoids (3-D) with intensities U[0.2, 1]; a sinogram is
Poisson(λ) with λ = A·x scaled to a requested total count, drawn with numpy's
PCG64 so the same seed gives the same counts on every machine.
"""
from __future__ import annotations

import numpy as np


def voxel_centres(geo):
    xs = -0.5 * geo.nx * geo.vx + (np.arange(geo.nx) + 0.5) * geo.vx
    ys = -0.5 * geo.ny * geo.vy + (np.arange(geo.ny) + 0.5) * geo.vy
    zs = -0.5 * geo.nz * geo.vz + (np.arange(geo.nz) + 0.5) * geo.vz
    return xs, ys, zs


def phantom(geo, n_shapes: int, seed: int) -> np.ndarray:
    """Image f32[nz*ny*nx] (column order x + nx*(y + ny*z)) of seeded ellipsoids."""
    rng = np.random.Generator(np.random.PCG64(seed))
    xs, ys, zs = voxel_centres(geo)
    Z, Y, X = np.meshgrid(zs, ys, xs, indexing="ij")
    hx, hy, hz = 0.5 * geo.nx * geo.vx, 0.5 * geo.ny * geo.vy, 0.5 * geo.nz * geo.vz
    img = np.zeros(Z.shape, np.float64)
    for _ in range(n_shapes):
        cx, cy = rng.uniform(-0.4, 0.4, 2) * (hx, hy)
        cz = rng.uniform(-0.4, 0.4) * hz if geo.nz > 1 else 0.0
        ax, ay = rng.uniform(0.08, 0.35, 2) * (hx, hy)
        az = rng.uniform(0.2, 0.6) * hz if geo.nz > 1 else 1e9
        th = rng.uniform(0.0, np.pi)
        inten = rng.uniform(0.2, 1.0)
        c, s = np.cos(th), np.sin(th)
        u = (X - cx) * c + (Y - cy) * s
        v = -(X - cx) * s + (Y - cy) * c
        inside = (u / ax) ** 2 + (v / ay) ** 2 + ((Z - cz) / az) ** 2 <= 1.0
        img[inside] += inten
    return img.astype(np.float32).ravel()


def poisson_sinogram(expected: np.ndarray, total: float, seed: int) -> np.ndarray:
    """int32 counts ~ Poisson(expected * total / Σ expected)."""
    e = np.asarray(expected, np.float64)
    s = e.sum()
    lam = e * (total / s) if s > 0 else e
    rng = np.random.Generator(np.random.PCG64(seed))
    return rng.poisson(lam).astype(np.int32)


def project_host(rowptr, col, val, x) -> np.ndarray:
    """A·x in float64 on the host (small matrices only)."""
    rowptr = np.asarray(rowptr, np.int64)
    prod = np.asarray(val, np.float64) * np.asarray(x, np.float64)[np.asarray(col, np.int64)]
    cs = np.concatenate([[0.0], np.cumsum(prod)])
    return cs[rowptr[1:]] - cs[rowptr[:-1]]
