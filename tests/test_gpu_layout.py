"""Locality layout (rows in LOR tubes, columns in voxel bricks) on the GPU.

Every entry point keeps natural order: the matrix read back, the sensitivity
image, the MLEM images of every mode, single projections, device-pointer runs
and batch slots must equal the natural-layout results (bit for bit for the
matrix, to FP32 rounding for sums whose order changes)."""
import numpy as np
import pytest

from conftest import problem

pytestmark = pytest.mark.gpu

TOL_F32 = 1e-5
MODES = [(s, b) for s in (0, 1) for b in (0, 1, 2)]


def dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


@pytest.mark.parametrize("name", ["ring2d", "cyl3d_tiny", "cyl3d_rows32"])
def test_generated_locality_layout(pkg, O, cuda, name):
    p = problem(pkg, O, name)
    A = (p["rp"], p["col"], p["val"])
    nat = pkg.Matrix.generate(p["geo"])
    loc = pkg.Matrix.generate(p["geo"], layout=pkg.LAYOUT_LOCALITY)
    # the matrix, its transpose and the sensitivity image come back in natural order
    for a, b in zip(loc.csr(), nat.csr()):
        assert np.array_equal(a.view(np.uint32) if a.dtype == np.float32 else a,
                              b.view(np.uint32) if b.dtype == np.float32 else b)
    for a, b in zip(loc.transpose(), nat.transpose()):
        assert np.array_equal(a, b)
    np.testing.assert_allclose(loc.norm(), nat.norm(), rtol=1e-6, atol=0)
    norm = nat.norm().astype(np.float64)
    f0 = np.full(nat.cols, nat.initial_value(p["g"]), np.float32)
    assert loc.initial_value(p["g"]) == nat.initial_value(p["g"])
    ref64 = O.mlem_f64(A, p["g"], norm, f0, 12)
    for spmv, bp in MODES:
        got = loc.run(p["g"], 12, f0=f0, spmv=spmv, bp_mode=bp)
        want = nat.run(p["g"], 12, f0=f0, spmv=spmv, bp_mode=bp)
        assert O.rel_l2(got, want) < TOL_F32, (spmv, bp)
        assert O.rel_l2(got, ref64) < TOL_F32, (spmv, bp)
    # stage timing (eager launches) changes nothing in the result
    img_t, st = loc.run(p["g"], 5, f0=f0, stats=True, kernel_timing=True)
    assert np.array_equal(img_t, loc.run(p["g"], 5, f0=f0))
    assert st["fp_ms"] > 0 and st["bp_ms"] > 0
    _, st = loc.run(p["g"], 5, f0=f0, stats=True)
    assert np.isnan(st["fp_ms"]) and np.isnan(st["bp_ms"])
    # default initial image and the log-likelihood
    img, ll = loc.run(p["g"], 8, loglik=True)
    img2, ll2 = nat.run(p["g"], 8, loglik=True)
    assert O.rel_l2(img, img2) < TOL_F32
    np.testing.assert_allclose(ll, ll2, rtol=1e-7)
    # single projections on device pointers, natural order in and out
    x = np.random.default_rng(3).uniform(0.1, 1.0, nat.cols).astype(np.float32)
    dx, dg = dev(cuda, x), dev(cuda, p["g"].astype(np.int32))
    ratio = cuda.zeros(nat.rows, dtype=cuda.float32, device="cuda")
    fwp = cuda.zeros(nat.rows, dtype=cuda.float32, device="cuda")
    loc.forward_project(dx.data_ptr(), dg.data_ptr(), ratio.data_ptr(), fwp.data_ptr())
    cuda.cuda.synchronize()
    want_fp = O.spmv_csrvec(*A, x)
    np.testing.assert_allclose(fwp.cpu().numpy(), want_fp, rtol=2e-5, atol=1e-6)
    want_ratio = np.where(want_fp != 0, p["g"] / np.where(want_fp != 0, want_fp, 1), 0)
    np.testing.assert_allclose(ratio.cpu().numpy(), want_ratio, rtol=2e-5, atol=1e-6)
    r = np.random.default_rng(4).uniform(0.0, 2.0, nat.rows).astype(np.float32)
    dr = dev(cuda, r)
    for bp_mode in (0, 1):
        bp = cuda.zeros(nat.cols, dtype=cuda.float32, device="cuda")
        loc.back_project(dr.data_ptr(), bp.data_ptr(), bp_mode=bp_mode)
        cuda.cuda.synchronize()
        np.testing.assert_allclose(bp.cpu().numpy(), O.scatter(*A, r, nat.cols), rtol=2e-5, atol=1e-6)
    # device-pointer reconstruction
    fd = dev(cuda, f0)
    loc.run_device(dg.data_ptr(), fd.data_ptr(), 12)
    cuda.cuda.synchronize()
    assert O.rel_l2(fd.cpu().numpy(), loc.run(p["g"], 12, f0=f0)) < 1e-6
    # batch slots
    G = np.stack([p["g"], np.roll(p["g"], 7)]).astype(np.int32)
    its = np.array([12, 5], np.uint32)
    out = loc.batch_run(G, its, tile=8)
    for k in range(2):
        single = loc.run(G[k], int(its[k]))
        assert O.rel_l2(out[k], single) < TOL_F32
    nat.close()
    loc.close()


def test_locality_layout_from_csr_and_csr4(pkg, O, tmp_path):
    p = problem(pkg, O, "cyl3d_rows32")
    geo = p["geo"]
    A = (p["rp"], p["col"], p["val"])
    grid = (geo.nx, geo.ny, geo.nz)
    m = pkg.Matrix.from_csr(*A, p["cols"], layout=pkg.LAYOUT_LOCALITY, grid=grid)
    rp, c, v = m.csr()
    assert np.array_equal(rp, p["rp"]) and np.array_equal(c, p["col"]) and np.array_equal(v, p["val"])
    ref64 = O.mlem_f64(A, p["g"], p["norm"], p["f0"], 10)
    assert O.rel_l2(m.run(p["g"], 10, f0=p["f0"]), ref64) < TOL_F32
    m.close()
    path = tmp_path / "m.csr4"
    pkg.csr4_write(path, *A, p["cols"], geo=geo)
    m = pkg.Matrix.from_csr4(path, layout=pkg.LAYOUT_LOCALITY, value_type=pkg.VAL_F16)
    assert O.rel_l2(m.run(p["g"], 10, f0=p["f0"]), ref64) < 1e-3
    m.close()
    with pytest.raises(pkg.MlemError):  # no voxel grid
        pkg.Matrix.from_csr(*A, p["cols"], layout=pkg.LAYOUT_LOCALITY)
    with pytest.raises(pkg.MlemError):  # grid that does not match the columns
        pkg.Matrix.from_csr(*A, p["cols"], layout=pkg.LAYOUT_LOCALITY, grid=(geo.nx, geo.ny, geo.nz + 1))
    with pytest.raises(pkg.MlemError):
        pkg.Matrix.from_csr(*A, p["cols"], layout=7, grid=grid)


def test_derived_row_order(pkg, O, cuda):
    """A matrix with no detector numbering (rows shuffled, empty rows added)
    gets its row order from its own columns; every entry point stays natural."""
    p = problem(pkg, O, "cyl3d_tiny")
    geo = p["geo"]
    rng = np.random.default_rng(11)
    lens = np.diff(p["rp"])
    rows = [(p["col"][p["rp"][i]:p["rp"][i + 1]], p["val"][p["rp"][i]:p["rp"][i + 1]]) for i in range(len(lens))]
    empty = (np.zeros(0, np.uint32), np.zeros(0, np.float32))
    rows = [rows[i] for i in rng.permutation(len(rows))] + [empty] * 5
    perm = rng.permutation(len(rows))
    rows = [rows[i] for i in perm]
    rp = np.concatenate([[0], np.cumsum([len(c) for c, _ in rows])]).astype(np.uint64)
    col = np.concatenate([c for c, _ in rows]).astype(np.uint32)
    val = np.concatenate([v for _, v in rows]).astype(np.float32)
    A = (rp, col, val)
    cols = p["cols"]
    g = rng.poisson(20.0, len(rows)).astype(np.int32)
    m = pkg.Matrix.from_csr(*A, cols, layout=pkg.LAYOUT_LOCALITY, grid=(geo.nx, geo.ny, geo.nz))
    got = m.csr()
    assert np.array_equal(got[0], rp) and np.array_equal(got[1], col)
    assert np.array_equal(got[2].view(np.uint32), val.view(np.uint32))
    for a, b in zip(m.transpose(), O.transpose(rp, col, val, cols)):
        assert np.array_equal(a, b)
    norm = O.colsum(*A, cols)
    np.testing.assert_allclose(m.norm(), norm, rtol=1e-6, atol=0)
    f0 = np.full(cols, m.initial_value(g), np.float32)
    ref64 = O.mlem_f64(A, g, norm.astype(np.float64), f0, 10)
    for spmv, bp in MODES:
        assert O.rel_l2(m.run(g, 10, f0=f0, spmv=spmv, bp_mode=bp), ref64) < TOL_F32, (spmv, bp)
    x = rng.uniform(0.1, 1.0, cols).astype(np.float32)
    dx, dg = dev(cuda, x), dev(cuda, g)
    ratio = cuda.zeros(len(rows), dtype=cuda.float32, device="cuda")
    fwp = cuda.zeros(len(rows), dtype=cuda.float32, device="cuda")
    m.forward_project(dx.data_ptr(), dg.data_ptr(), ratio.data_ptr(), fwp.data_ptr())
    cuda.cuda.synchronize()
    np.testing.assert_allclose(fwp.cpu().numpy(), O.spmv_csrvec(*A, x), rtol=2e-5, atol=1e-6)
    r = rng.uniform(0.0, 2.0, len(rows)).astype(np.float32)
    bp = cuda.zeros(cols, dtype=cuda.float32, device="cuda")
    m.back_project(dev(cuda, r).data_ptr(), bp.data_ptr())
    cuda.cuda.synchronize()
    np.testing.assert_allclose(bp.cpu().numpy(), O.scatter(*A, r, cols), rtol=2e-5, atol=1e-6)
    G = np.stack([g, rng.poisson(5.0, len(rows)).astype(np.int32)])
    out = m.batch_run(G, np.array([10, 4], np.uint32), tile=8)
    for k, it in enumerate((10, 4)):
        assert O.rel_l2(out[k], m.run(G[k], it)) < TOL_F32
    m.close()


def test_locality_layout_server(pkg, O):
    p = problem(pkg, O, "ring2d")
    loc = pkg.Matrix.generate(p["geo"], layout=pkg.LAYOUT_LOCALITY)
    with pkg.Server() as srv:
        mid = srv.add_matrix(loc)
        rid = srv.submit(mid, p["g"], 9)
        img, _ = srv.wait(rid)
    assert O.rel_l2(img, loc.run(p["g"], 9)) < TOL_F32
    loc.close()
