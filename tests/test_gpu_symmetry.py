"""Symmetry-compressed operands (matrix generated with symmetry = 1) on the GPU.

The handle's matrix becomes A^: the canonical LOR rows of the host generator,
averaged over the symmetries that fix their LOR, mapped onto every other row.
Checks: A^ equals the Python restatement built from the host generator's
matrix, A^ is exactly invariant under the 16 maps, the compact kernels (SYM)
reproduce the FP64 oracle on A^ for MLEM and single projections (FP32 1e-5,
FP16 values 1e-3), the autotuner may pick them, every other mode still runs
on A^, the orbit-order hand-over inside an MLEM loop is bit-exact, and
unsupported geometries and options fail with an error."""
import numpy as np
import pytest

import _symmetry as S
from conftest import problem

pytestmark = pytest.mark.gpu

TOL_F32 = 1e-5
NAMES = ["ring2d_tiny", "cyl3d_tiny", "ring2d", "cyl3d_rows32"]


def dense(rp, col, val, cols):
    rows = len(rp) - 1
    A = np.zeros((rows, cols), np.float64)
    for r in range(rows):
        A[r, col[rp[r]:rp[r + 1]]] = val[rp[r]:rp[r + 1]]
    return A


def dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


@pytest.mark.parametrize("name", NAMES)
def test_symmetric_matrix(pkg, O, cuda, name):
    p = problem(pkg, O, name)
    geo = p["geo"]
    m = pkg.Matrix.generate(geo, symmetry=True)
    rp, col, val = m.csr()
    assert m.rows == len(p["rp"]) - 1 and m.cols == p["cols"]
    Ah = dense(rp, col, val, m.cols)
    want = S.symmetric_matrix(geo, dense(p["rp"], p["col"], p["val"], p["cols"]))
    np.testing.assert_allclose(Ah, want, rtol=1e-6, atol=1e-7)
    # exactly invariant: A^[s(r), s(c)] == A^[r, c] for all 16 maps
    for s in range(16):
        L, V = S.lor_perm(s, geo.det_per_ring, geo.n_rings), S.vox_perm(s, geo.nx, geo.nz)
        assert np.array_equal(Ah[np.ix_(L, V)], Ah), s
    # the transpose and the sensitivity image are those of A^
    cp, ri, tv = m.transpose()
    assert np.array_equal(dense(cp, ri, tv, m.rows), Ah.T)
    np.testing.assert_allclose(m.norm(), Ah.sum(axis=0), rtol=2e-6, atol=1e-6)
    m.close()


@pytest.mark.parametrize("name", NAMES)
def test_symmetric_mlem_and_projections(pkg, O, cuda, name):
    p = problem(pkg, O, name)
    m = pkg.Matrix.generate(p["geo"], symmetry=True)
    A = m.csr()
    norm = m.norm().astype(np.float64)
    g = p["g"]
    f0 = np.full(m.cols, m.initial_value(g), np.float32)
    ref, llref = O.mlem_f64(A, g, norm, f0, 12, loglik=True)
    got, ll = m.run(g, 12, f0=f0, kernel=pkg.KERNEL_SYM, loglik=True)
    assert O.rel_l2(got, ref) < TOL_F32
    np.testing.assert_allclose(ll, llref, rtol=1e-6)
    assert O.rel_l2(m.run(g, 12, f0=f0), ref) < TOL_F32          # autotuned
    assert O.rel_l2(m.run(g, 12, f0=f0, use_graph=False, kernel=pkg.KERNEL_SYM), ref) < TOL_F32
    for spmv, bp in [(0, 0), (1, 0), (0, 1), (1, 1), (0, 2)]:    # every other mode runs on A^
        assert O.rel_l2(m.run(g, 12, f0=f0, spmv=spmv, bp_mode=bp), ref) < TOL_F32, (spmv, bp)
    # single projections through the compact kernels
    x = np.random.default_rng(3).uniform(0.1, 1.0, m.cols).astype(np.float32)
    dx, dg = dev(cuda, x), dev(cuda, g.astype(np.int32))
    ratio = cuda.zeros(m.rows, dtype=cuda.float32, device="cuda")
    fwp = cuda.zeros(m.rows, dtype=cuda.float32, device="cuda")
    m.forward_project(dx.data_ptr(), dg.data_ptr(), ratio.data_ptr(), fwp.data_ptr(), kernel=pkg.KERNEL_SYM)
    cuda.cuda.synchronize()
    want_fp = O.spmv_csrvec(*A, x)
    np.testing.assert_allclose(fwp.cpu().numpy(), want_fp, rtol=2e-5, atol=1e-6)
    want_ratio = np.where(want_fp != 0, g / np.where(want_fp != 0, want_fp, 1), 0)
    np.testing.assert_allclose(ratio.cpu().numpy(), want_ratio, rtol=2e-5, atol=1e-6)
    r = np.random.default_rng(4).uniform(0.0, 2.0, m.rows).astype(np.float32)
    dr = dev(cuda, r)
    bp = cuda.zeros(m.cols, dtype=cuda.float32, device="cuda")
    m.back_project(dr.data_ptr(), bp.data_ptr(), kernel=pkg.KERNEL_SYM)
    cuda.cuda.synchronize()
    np.testing.assert_allclose(bp.cpu().numpy(), O.scatter(*A, r, m.cols), rtol=2e-5, atol=1e-6)
    # device-pointer reconstruction
    fd = dev(cuda, f0)
    m.run_device(dg.data_ptr(), fd.data_ptr(), 12, kernel=pkg.KERNEL_SYM)
    cuda.cuda.synchronize()
    assert O.rel_l2(fd.cpu().numpy(), ref) < TOL_F32
    m.close()


@pytest.mark.parametrize("vt", ["VAL_F16", "VAL_BF16"])
def test_symmetric_low_precision_values(pkg, O, cuda, vt):
    p = problem(pkg, O, "cyl3d_rows32")
    m32 = pkg.Matrix.generate(p["geo"], symmetry=True)
    A = m32.csr()
    norm = m32.norm().astype(np.float64)
    f0 = np.full(m32.cols, m32.initial_value(p["g"]), np.float32)
    ref = O.mlem_f64(A, p["g"], norm, f0, 12)
    m32.close()
    m = pkg.Matrix.generate(p["geo"], symmetry=True, value_type=getattr(pkg, vt))
    tol = 1e-3 if vt == "VAL_F16" else 1e-2
    assert O.rel_l2(m.run(p["g"], 12, f0=f0, kernel=pkg.KERNEL_SYM), ref) < tol
    # the compact kernels agree with the csr-vector kernels on the same stored values
    assert O.rel_l2(m.run(p["g"], 12, f0=f0, kernel=pkg.KERNEL_SYM),
                    m.run(p["g"], 12, f0=f0, kernel=pkg.KERNEL_DIRECT)) < 1e-5
    m.close()


def test_symmetry_errors(pkg, cuda):
    geo = pkg.preset("cyl3d_tiny")
    with pytest.raises(pkg.MlemError):
        pkg.Matrix.generate(geo, symmetry=True, layout=pkg.LAYOUT_LOCALITY)
    with pytest.raises(pkg.MlemError):
        pkg.Matrix.generate(pkg.preset("cyl3d_tiny", det_per_ring=26), symmetry=True)
    with pytest.raises(pkg.MlemError):
        pkg.Matrix.generate(pkg.preset("cyl3d_tiny", ny=10), symmetry=True)
    with pytest.raises(pkg.MlemError):
        pkg.Matrix.generate(pkg.preset("cyl3d_tiny", row_stride=3), symmetry=True)
    m = pkg.Matrix.generate(geo)
    g = np.ones(m.rows, np.int32)
    with pytest.raises(pkg.MlemError):
        m.run(g, 2, kernel=pkg.KERNEL_SYM)
    m.close()


@pytest.mark.parametrize("name", ["cyl3d_tiny", "ring2d"])
def test_symmetric_orbit_exchange_is_exact(pkg, O, cuda, name):
    """In an MLEM loop the two compact kernels hand each other their outputs
    in orbit order; the result equals, bit for bit, the same iterations made
    of single projections (each gathering its input) and the update f*bp/norm."""
    p = problem(pkg, O, name)
    m = pkg.Matrix.generate(p["geo"], symmetry=True)
    g = p["g"].astype(np.int32)
    f0 = np.full(m.cols, m.initial_value(g), np.float32)
    norm = m.norm()
    for graph in (True, False):
        got = m.run(g, 5, f0=f0, kernel=pkg.KERNEL_SYM, use_graph=graph)
        f = f0.copy()
        dg = dev(cuda, g)
        ratio = cuda.zeros(m.rows, dtype=cuda.float32, device="cuda")
        bp = cuda.zeros(m.cols, dtype=cuda.float32, device="cuda")
        for _ in range(5):
            df = dev(cuda, f)
            m.forward_project(df.data_ptr(), dg.data_ptr(), ratio.data_ptr(), kernel=pkg.KERNEL_SYM)
            m.back_project(ratio.data_ptr(), bp.data_ptr(), kernel=pkg.KERNEL_SYM)
            cuda.cuda.synchronize()
            b = bp.cpu().numpy()
            t = (f * b).astype(np.float32)
            f = np.where(norm == 0, t, (t / np.where(norm == 0, 1, norm)).astype(np.float32)).astype(np.float32)
        assert np.array_equal(got, f), graph
    m.close()
