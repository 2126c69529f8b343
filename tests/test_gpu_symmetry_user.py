"""Symmetry-compressed operands on a caller's own matrix (GPU, C ABI).

mlem_matrix_create with symmetry = 1 keeps the caller's matrix unchanged and
builds the compact operands beside it, after checking on the GPU that the
matrix equals, bit for bit, the symmetric matrix rebuilt from its canonical
rows (so it is exactly invariant under the scanner's 16 symmetries).  On the
same inputs the image must then agree with the plain path within the FP32
tolerance (1e-5 relative L2): on the small test scanners whose generated
matrix is exactly symmetric, and at full size on the 3-D mid scanner's
symmetric matrix handed over as host CSR.  Matrices that are not invariant,
or whose rows are not the scanner's detector pairs, are refused."""
import numpy as np
import pytest

from conftest import problem

pytestmark = pytest.mark.gpu

TOL_F32 = 1e-5


def _sym_args(geo):
    return dict(grid=(geo.nx, geo.ny, geo.nz), symmetry=(geo.det_per_ring, geo.n_rings))


@pytest.mark.parametrize("name", ["ring2d_tiny", "cyl3d_tiny"])
def test_callers_symmetric_matrix_matches_plain_path(pkg, O, name):
    p = problem(pkg, O, name)
    A = (p["rp"], p["col"], p["val"])
    iters = 20
    plain = pkg.Matrix.from_csr(*A, p["cols"])
    want = plain.run(p["g"], iters, f0=p["f0"])
    plain.close()
    m = pkg.Matrix.from_csr(*A, p["cols"], **_sym_args(p["geo"]))
    assert m.symmetry["lor_rows"] > 0
    # the caller's matrix is kept as given
    rp, col, val = m.csr()
    assert np.array_equal(rp, p["rp"]) and np.array_equal(col, p["col"]) and np.array_equal(val, p["val"])
    for kern in (pkg.KERNEL_SYM, pkg.KERNEL_AUTO):
        got = m.run(p["g"], iters, f0=p["f0"], kernel=kern)
        assert O.rel_l2(got, want) < TOL_F32, kern
    ref64 = O.mlem_f64(A, p["g"], p["norm"], p["f0"], iters)
    assert O.rel_l2(m.run(p["g"], iters, f0=p["f0"], kernel=pkg.KERNEL_SYM), ref64) < TOL_F32
    m.close()
    # FP16 values: the compact operands hold the same rounded values as the matrix
    h = pkg.Matrix.from_csr(*A, p["cols"], value_type=pkg.VAL_F16, **_sym_args(p["geo"]))
    plain16 = pkg.Matrix.from_csr(*A, p["cols"], value_type=pkg.VAL_F16)
    want16 = plain16.run(p["g"], iters, f0=p["f0"])
    plain16.close()
    got16 = h.run(p["g"], iters, f0=p["f0"], kernel=pkg.KERNEL_SYM)
    h.close()
    assert O.rel_l2(got16, want16) < TOL_F32
    assert O.rel_l2(got16, ref64) < 1e-3


def test_callers_matrix_at_full_size(pkg, O, cuda):
    """The 3-D mid scanner (662,976 x 784,000): its symmetric matrix, read back
    to the host and created again with symmetry, against the plain path on the
    same host CSR, 100 iterations."""
    from test_gpu_full_size import WORKLOADS, _sinogram
    geo = pkg.preset("cyl3d_mid")
    gen = pkg.Matrix.generate(geo, symmetry=True)
    g = _sinogram(pkg, gen, geo, WORKLOADS["cyl3d_mid"], cuda)
    A = gen.csr()
    cols = gen.cols
    gen.close()
    iters = 100
    plain = pkg.Matrix.from_csr(*A, cols)
    f0 = np.full(plain.cols, plain.initial_value(g), np.float32)
    want = plain.run(g, iters, f0=f0)
    plain.close()
    m = pkg.Matrix.from_csr(*A, cols, **_sym_args(geo))
    got = m.run(g, iters, f0=f0, kernel=pkg.KERNEL_SYM)
    auto = m.run(g, iters, f0=f0)
    kinds = (m.tuning(False)["kernel"], m.tuning(True)["kernel"])
    m.close()
    err, err_auto = O.rel_l2(got, want), O.rel_l2(auto, want)
    print(f"\ncyl3d_mid caller's symmetric matrix, {iters} iterations: compact kernels vs plain path {err:.2e}, "
          f"autotuned ({kinds[0]}/{kinds[1]}) {err_auto:.2e}")
    assert err < TOL_F32 and err_auto < TOL_F32


def test_matrix_that_is_not_invariant_is_refused(pkg, O):
    p = problem(pkg, O, "cyl3d_tiny")
    val = p["val"].copy()
    val[123] *= 1.0001
    with pytest.raises(pkg.MlemError) as e:
        pkg.Matrix.from_csr(p["rp"], p["col"], val, p["cols"], **_sym_args(p["geo"]))
    assert e.value.status == "EINVAL" and "not invariant" in str(e.value)
    # the 2-D ring's generated matrix has rays along voxel planes: not exactly symmetric
    q = problem(pkg, O, "ring2d")
    with pytest.raises(pkg.MlemError) as e:
        pkg.Matrix.from_csr(q["rp"], q["col"], q["val"], q["cols"], **_sym_args(q["geo"]))
    assert e.value.status == "EINVAL" and "not invariant" in str(e.value)


def test_rows_must_be_the_scanners_detector_pairs(pkg, O):
    p = problem(pkg, O, "cyl3d_tiny")
    geo = p["geo"]
    with pytest.raises(pkg.MlemError) as e:
        pkg.Matrix.from_csr(p["rp"], p["col"], p["val"], p["cols"], grid=(geo.nx, geo.ny, geo.nz),
                            symmetry=(geo.det_per_ring, geo.n_rings + 1))
    assert e.value.status == "EINVAL" and "detector pairs" in str(e.value)
    with pytest.raises(pkg.MlemError) as e:
        pkg.Matrix.from_csr(p["rp"], p["col"], p["val"], p["cols"], grid=(geo.nx, geo.ny, geo.nz),
                            symmetry=(geo.det_per_ring + 2, geo.n_rings))
    assert e.value.status == "EUNSUPPORTED"
