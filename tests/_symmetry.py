"""Python restatement of the 16 scanner symmetries used by the symmetry-compressed
operands (mirror y -> -y, rotation by q * 90 degrees, axial flip z -> -z, applied
in that order; s = q + 4 m + 8 f), on voxels, detectors and LOR rows, and the
symmetric matrix A^ they define from a generated matrix (canonical rows
averaged over their stabilizer, every other row its canonical row mapped).
Test infrastructure only."""
from __future__ import annotations

import numpy as np


def vox_perm(s: int, n: int, nz: int) -> np.ndarray:
    """perm[c] = image of voxel c under symmetry s (c = x + n (y + n z))."""
    c = np.arange(n * n * nz, dtype=np.int64)
    x, y, z = c % n, (c // n) % n, c // (n * n)
    if (s >> 2) & 1:
        y = n - 1 - y
    for _ in range(s & 3):
        x, y = n - 1 - y, x
    if s >> 3:
        z = nz - 1 - z
    return x + n * (y + n * z)


def det_perm(s: int, dpr: int, rings: int) -> np.ndarray:
    d = np.arange(dpr * rings, dtype=np.int64)
    ring, k = d // dpr, d % dpr
    if (s >> 2) & 1:
        k = (dpr - k) % dpr
    k = (k + (s & 3) * (dpr // 4)) % dpr
    if s >> 3:
        ring = rings - 1 - ring
    return ring * dpr + k


def lor_index(a, b, D):
    a, b = np.minimum(a, b), np.maximum(a, b)
    return a * D - a * (a + 1) // 2 + (b - a - 1)


def lor_perm(s: int, dpr: int, rings: int) -> np.ndarray:
    """perm[r] = image of LOR row r (natural lexicographic (a < b) order)."""
    D = dpr * rings
    a, b = np.triu_indices(D, 1)
    dp = det_perm(s, dpr, rings)
    return lor_index(dp[a], dp[b], D)


def symmetric_matrix(geo, A: np.ndarray) -> np.ndarray:
    """A^ (dense) from a dense generated matrix A (rows in natural LOR order)."""
    n, nz, dpr, rings = geo.nx, geo.nz, geo.det_per_ring, geo.n_rings
    L = [lor_perm(s, dpr, rings) for s in range(16)]
    V = [vox_perm(s, n, nz) for s in range(16)]
    inv = [np.argsort(v) for v in V]
    imgs = np.stack(L)                      # [16, rows]
    canon = imgs.min(axis=0) == np.arange(A.shape[0])
    out = np.zeros_like(A, dtype=np.float64)
    for r in np.nonzero(canon)[0]:
        H = [s for s in range(16) if L[s][r] == r]
        row = np.mean([A[r][inv[h]] for h in H], axis=0)   # row'[c] = mean_h A[r, h^-1(c)]
        for s in range(16):
            out[L[s][r], V[s]] = row
    return out
