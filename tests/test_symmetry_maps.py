"""The 16 scanner symmetries (CPU): they form a group acting the same way on
voxels and on LOR rows, the host generator's matrix of the small presets is
invariant under them (so the canonical rows describe it), and the symmetric
matrix A^ restated in Python is exactly invariant on a scanner whose plain
matrix is not (rays along voxel planes)."""
import numpy as np
import pytest

import _symmetry as S


def dense(rp, col, val, cols):
    A = np.zeros((len(rp) - 1, cols), np.float64)
    for r in range(len(rp) - 1):
        A[r, col[rp[r]:rp[r + 1]]] = val[rp[r]:rp[r + 1]]
    return A


def test_group_closure_and_shared_action():
    n, nz, dpr, rings = 7, 5, 12, 3
    V = [S.vox_perm(s, n, nz) for s in range(16)]
    L = [S.lor_perm(s, dpr, rings) for s in range(16)]
    assert len({v.tobytes() for v in V}) == 16 and len({x.tobytes() for x in L}) == 16
    for s in range(16):
        for t in range(16):
            vt = V[s][V[t]]
            u = [k for k in range(16) if np.array_equal(V[k], vt)]
            assert len(u) == 1
            assert np.array_equal(L[u[0]], L[s][L[t]])   # same composition on LORs
    for v in V + L:
        assert np.array_equal(np.sort(v), np.arange(len(v)))


@pytest.mark.parametrize("name", ["ring2d_tiny", "cyl3d_tiny"])
def test_generated_matrix_is_invariant(pkg, name):
    geo = pkg.preset(name)
    A = dense(*pkg.siddon_host(geo))
    for s in range(16):
        L, V = S.lor_perm(s, geo.det_per_ring, geo.n_rings), S.vox_perm(s, geo.nx, geo.nz)
        assert np.array_equal(A[np.ix_(L, V)], A), s
    assert np.array_equal(S.symmetric_matrix(geo, A), A)


def test_symmetric_matrix_on_plane_rays(pkg):
    # 3 sub-rays: the middle sub-rays of LORs (0, 64) and (32, 96) run along the planes y = 0 and x = 0
    geo = pkg.preset("ring2d")
    A = dense(*pkg.siddon_host(geo))
    Ah = S.symmetric_matrix(geo, A)
    for s in range(16):
        L, V = S.lor_perm(s, geo.det_per_ring, geo.n_rings), S.vox_perm(s, geo.nx, geo.nz)
        assert np.array_equal(Ah[np.ix_(L, V)], Ah), s
    differ = np.abs(Ah - A).max(axis=1) > 0
    assert 0 < differ.sum() <= 4                   # only the rows of rays along a voxel plane change
    np.testing.assert_allclose(Ah.sum(axis=1), A.sum(axis=1), rtol=1e-6)
