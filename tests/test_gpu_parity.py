"""CUDA path against the oracle and the reference fixtures (GPU, via the C ABI).

Tolerances (the contract of the FP32 path): image after N iterations within
1e-5 relative L2 of the reference's update (fixtures and FP32 oracle); FP16 /
BF16 value storage within 1e-3 relative L2 of the FP64 oracle; transpose and
merge-path partition indices bit-exact.
"""
from __future__ import annotations

import numpy as np
import pytest

from conftest import golden_cases, golden_csr, problem

pytestmark = pytest.mark.gpu

TOL_F32 = 1e-5
TOL_LOWP = 1e-3


def dev(torch, a):
    a = np.ascontiguousarray(a)
    if a.dtype == np.uint64:
        a = a.view(np.int64)
    elif a.dtype == np.uint32:
        a = a.view(np.int32)
    return torch.from_numpy(a.copy()).cuda()


# ------------------------------------------------------------------ transpose
def test_transpose_matches_reference_fixtures(pkg, golden):
    for name in golden_cases(golden):
        rp, c, v, cols = golden_csr(golden, name)
        cp, rt, vt = pkg.transpose(rp, c, v, cols)
        assert np.array_equal(cp, golden[f"{name}/T_colptr"]), name
        assert np.array_equal(rt, golden[f"{name}/T_row"]), name
        assert np.array_equal(vt.view(np.uint32), golden[f"{name}/T_val"].view(np.uint32)), name


@pytest.mark.parametrize("cols", [7, 300, 70000, 5_000_000])
def test_transpose_bitexact_random(pkg, O, cols):
    rng = np.random.Generator(np.random.PCG64(cols))
    rows = 20000
    lens = rng.integers(0, 120, rows)
    lens[rng.random(rows) < 0.1] = 0
    rp = np.zeros(rows + 1, np.uint64)
    rp[1:] = np.cumsum(lens)
    col = rng.integers(0, cols, int(rp[-1])).astype(np.uint32)  # unsorted, duplicates allowed
    val = rng.uniform(0, 1, int(rp[-1])).astype(np.float32)
    got = pkg.transpose(rp, col, val, cols)
    want = O.transpose(rp, col, val, cols)
    for a, b in zip(got, want):
        assert np.array_equal(a, b)


def test_transpose_round_trip_and_column_sums(pkg, O):
    p = problem(pkg, O, "ring2d")
    m = pkg.Matrix.from_csr(p["rp"], p["col"], p["val"], p["cols"])
    cp, rt, vt = m.transpose()
    back = pkg.transpose(cp, rt, vt, len(p["rp"]) - 1)
    assert np.array_equal(back[0], p["rp"]) and np.array_equal(back[1], p["col"])
    assert np.array_equal(back[2], p["val"])
    np.testing.assert_allclose(m.norm(), O.colsum(p["rp"], p["col"], p["val"], p["cols"]), rtol=1e-7, atol=0)
    m.close()


# ------------------------------------------------------------ merge partition
def _search_case(pkg, O, cuda, rp, nnz, ss):
    rows = len(rp) - 1
    nthreads = -(-(rows + nnz) // (1024 * ss)) * 1024  # the reference grid (main.cu:306)
    drp = dev(cuda, rp)
    di = cuda.zeros(nthreads, dtype=cuda.int64, device="cuda")
    dj = cuda.zeros(nthreads, dtype=cuda.int64, device="cuda")
    pkg.merge_path_search(drp.data_ptr(), rows, nnz, ss, nthreads, di.data_ptr(), dj.data_ptr())
    cuda.cuda.synchronize()
    wi, wj = O.merge_search(rp, rows, ss, nthreads)
    assert np.array_equal(di.cpu().numpy(), wi)
    assert np.array_equal(dj.cpu().numpy(), wj)


def test_merge_search_bitexact(pkg, O, golden, cuda):
    for name in golden_cases(golden):
        rp, c, v, cols = golden_csr(golden, name)
        for ss in (1, 2, 5, 9, 33):
            _search_case(pkg, O, cuda, rp, len(c), ss)
    p = problem(pkg, O, "ring2d")
    for ss in (1, 5, 6):
        _search_case(pkg, O, cuda, p["rp"], len(p["col"]), ss)


# ------------------------------------------------------------ projections
@pytest.mark.parametrize("spmv", [0, 1])
def test_forward_projection(pkg, O, cuda, spmv):
    p = problem(pkg, O, "ring2d")
    m = pkg.Matrix.from_csr(p["rp"], p["col"], p["val"], p["cols"])
    x = np.random.Generator(np.random.PCG64(3)).uniform(0.1, 2, p["cols"]).astype(np.float32)
    dx, dg = dev(cuda, x), dev(cuda, p["g"])
    ratio = cuda.zeros(m.rows, dtype=cuda.float32, device="cuda")
    fp = cuda.zeros(m.rows, dtype=cuda.float32, device="cuda")
    m.forward_project(dx.data_ptr(), dg.data_ptr(), ratio.data_ptr(), fp.data_ptr(), spmv=spmv, secsize_fp=5)
    cuda.cuda.synchronize()
    want = O.spmv_csrvec(p["rp"], p["col"], p["val"], x)
    got = fp.cpu().numpy()
    assert O.rel_l2(got, want) < 1e-6
    np.testing.assert_allclose(got, want, rtol=1e-5, atol=1e-6)
    want_r = np.where(want != 0, p["g"].astype(np.float32) / np.where(want != 0, want, 1), 0)
    np.testing.assert_allclose(ratio.cpu().numpy(), want_r, rtol=1e-5, atol=1e-6)
    m.close()


@pytest.mark.parametrize("bp_mode", [0, 1])
def test_back_projection(pkg, O, cuda, bp_mode):
    p = problem(pkg, O, "cyl3d_tiny")
    m = pkg.Matrix.from_csr(p["rp"], p["col"], p["val"], p["cols"])
    r = np.random.Generator(np.random.PCG64(4)).uniform(0, 2, m.rows).astype(np.float32)
    dr = dev(cuda, r)
    bp = cuda.zeros(m.cols, dtype=cuda.float32, device="cuda")
    m.back_project(dr.data_ptr(), bp.data_ptr(), bp_mode=bp_mode)
    cuda.cuda.synchronize()
    want = O.scatter(p["rp"], p["col"], p["val"], r, p["cols"])
    np.testing.assert_allclose(bp.cpu().numpy(), want, rtol=1e-5, atol=1e-6)
    m.close()


# ------------------------------------------------------------------- MLEM
MODES = [(s, b) for s in (0, 1) for b in (0, 1, 2)]


@pytest.mark.parametrize("spmv,bp_mode", MODES)
def test_mlem_against_reference_fixtures(pkg, golden, spmv, bp_mode):
    for name in ("ring2d_tiny", "cyl3d_tiny"):
        rp, c, v, cols = golden_csr(golden, name)
        g, norm, f0 = golden[f"{name}/g"], golden[f"{name}/norm"], golden[f"{name}/f0"]
        m = pkg.Matrix.from_csr(rp, c, v, cols, norm=norm)
        for iters in (1, 4, 12):
            ut = 1 if bp_mode else 0
            ref = golden[f"{name}/mlem_s{spmv}_t{ut}_ss5x5_it{iters}"]
            for graph in (True, False):
                for kern in ((0, 1, 2, 3) if spmv == 1 else (3,)):
                    got = m.run(g, iters, f0=f0, spmv=spmv, bp_mode=bp_mode, use_graph=graph, kernel=kern)
                    err = float(np.linalg.norm(got.astype(np.float64) - ref) / np.linalg.norm(ref))
                    assert err < TOL_F32, (name, iters, graph, kern, err)
        m.close()


@pytest.mark.parametrize("spmv,bp_mode,kern", [m + (3,) for m in MODES] + [(1, 0, 0), (1, 1, 0), (1, 0, 1), (1, 2, 1),
                                                                          (1, 0, 2)])
@pytest.mark.parametrize("name", ["ring2d", "cyl3d_tiny", "cyl3d_tiny_dense"])
def test_mlem_against_oracle(pkg, O, spmv, bp_mode, kern, name):
    p = problem(pkg, O, name)
    A = (p["rp"], p["col"], p["val"])
    AT = O.transpose(*A, p["cols"])
    m = pkg.Matrix.from_csr(*A, p["cols"], norm=p["norm"])
    iters = 20
    got = m.run(p["g"], iters, f0=p["f0"], spmv=spmv, bp_mode=bp_mode, secsize_fp=5, secsize_bp=5, kernel=kern)
    ref32 = O.mlem_f32(A, AT if bp_mode == 0 else None, p["g"], p["norm"], p["f0"], iters, spmv=spmv,
                       using_trans=1 if bp_mode else 0)
    assert O.rel_l2(got, ref32) < TOL_F32
    ref64 = O.mlem_f64(A, p["g"], p["norm"], p["f0"], iters)
    assert O.rel_l2(got, ref64) < TOL_F32
    assert np.all(got >= 0)
    m.close()


def test_mlem_initial_value_and_dropin(pkg, O, golden):
    name = "ring2d_tiny"
    rp, c, v, cols = golden_csr(golden, name)
    g, norm, f0 = golden[f"{name}/g"], golden[f"{name}/norm"], golden[f"{name}/f0"]
    m = pkg.Matrix.from_csr(rp, c, v, cols, norm=norm)
    assert m.initial_value(g) == f0[0]  # main.cu:83-97, bit-exact
    got_default = m.run(g, 4)           # f0 = NULL -> reference initial value
    ref = golden[f"{name}/mlem_s1_t0_ss5x5_it4"]
    assert O.rel_l2(got_default, ref) < TOL_F32
    m.close()
    for ut in (0, 1):
        for spmv in (0, 1):
            out = np.zeros(cols, np.float32)
            AT = (golden[f"{name}/T_colptr"], golden[f"{name}/T_row"], golden[f"{name}/T_val"])
            t = AT if ut == 0 else (None, None, None)
            pkg.mlem(rp, c, v, *t, g, norm, f0, out, len(rp) - 1, cols, len(c), 12, 1, spmv, 5, 5, ut)
            ref = golden[f"{name}/mlem_s{spmv}_t{ut}_ss5x5_it12"]
            assert O.rel_l2(out, ref) < TOL_F32
    with pytest.raises(pkg.MlemError) as e:
        pkg.mlem(rp, c, v, None, None, None, g, norm, f0, np.zeros(cols, np.float32), len(rp) - 1, cols, len(c),
                 1, 2, 1, 5, 5, 1)
    assert e.value.status == "EUNSUPPORTED"


def test_section_sizes(pkg, O):
    p = problem(pkg, O, "ring2d")
    A = (p["rp"], p["col"], p["val"])
    m = pkg.Matrix.from_csr(*A, p["cols"], norm=p["norm"])
    ref64 = O.mlem_f64(A, p["g"], p["norm"], p["f0"], 8)
    for ss in (1, 2, 3, 7, 16, 64, 512):
        got = m.run(p["g"], 8, f0=p["f0"], spmv=0, secsize_fp=ss, secsize_bp=max(1, 513 - ss))
        assert O.rel_l2(got, ref64) < TOL_F32, ss
    with pytest.raises(pkg.MlemError):
        m.run(p["g"], 1, spmv=0, secsize_fp=513)
    m.close()


def test_deterministic_paths_are_bitwise_repeatable(pkg, O):
    p = problem(pkg, O, "ring2d")
    m = pkg.Matrix.from_csr(p["rp"], p["col"], p["val"], p["cols"])
    runs = {}
    for spmv, kern in ((0, 3), (1, 0), (1, 1), (1, 2), (1, 3)):
        a = m.run(p["g"], 10, spmv=spmv, bp_mode=0, kernel=kern)
        b = m.run(p["g"], 10, spmv=spmv, bp_mode=0, use_graph=False, kernel=kern)
        assert np.array_equal(a, b)
        runs[(spmv, kern)] = a
    m.close()


@pytest.mark.parametrize("vt,kern", [(0, 0), (0, 1), (0, 2), (0, 3), (1, 1), (1, 2), (1, 3)])
def test_kernel_variants_long_and_empty_rows(pkg, O, golden, cuda, vt, kern):
    # rows longer than a pipeline chunk (512), empty rows, one-row matrices
    for name in ("one_row", "rand_long", "empty_rows", "tall", "rand_dup"):
        rp, c, v, cols = golden_csr(golden, name)
        m = pkg.Matrix.from_csr(rp, c, v, cols, value_type=vt)
        x = golden[f"{name}/x"]
        dx, dg = dev(cuda, x), dev(cuda, np.zeros(m.rows, np.int32))
        ratio = cuda.zeros(m.rows, dtype=cuda.float32, device="cuda")
        fp = cuda.full((m.rows,), -1.0, dtype=cuda.float32, device="cuda")
        m.forward_project(dx.data_ptr(), dg.data_ptr(), ratio.data_ptr(), fp.data_ptr(), kernel=kern)
        cuda.cuda.synchronize()
        vq = v if vt == 0 else v.astype(np.float16).astype(np.float32)
        want = O.spmv_csrvec(rp, c, vq, x)
        np.testing.assert_allclose(fp.cpu().numpy(), want, rtol=2e-5, atol=1e-5, err_msg=name)
        m.close()


@pytest.mark.parametrize("vt", [1, 2])
def test_low_precision_values(pkg, O, vt):
    p = problem(pkg, O, "cyl3d_tiny")
    A = (p["rp"], p["col"], p["val"])
    m = pkg.Matrix.from_csr(*A, p["cols"], value_type=vt)
    ref64 = O.mlem_f64(A, p["g"], O.colsum(*A, p["cols"]), p["f0"], 20)
    for bp_mode in (0, 1, 2):
        got = m.run(p["g"], 20, f0=p["f0"], bp_mode=bp_mode)
        tol = TOL_LOWP if vt == 1 else 1e-2
        assert O.rel_l2(got, ref64) < tol, (vt, bp_mode, O.rel_l2(got, ref64))
    m.close()


def test_loglik(pkg, O):
    p = problem(pkg, O, "ring2d")
    A = (p["rp"], p["col"], p["val"])
    m = pkg.Matrix.from_csr(*A, p["cols"], norm=p["norm"])
    img, ll = m.run(p["g"], 15, f0=p["f0"], loglik=True)
    _, ll64 = O.mlem_f64(A, p["g"], p["norm"], p["f0"], 15, loglik=True)
    np.testing.assert_allclose(ll, ll64, rtol=1e-6)
    assert np.all(np.diff(ll) > -1e-9 * abs(ll[0]))  # MLEM never decreases the likelihood
    m.close()


# ------------------------------------------------------------- generator
@pytest.mark.parametrize("name,stride", [("ring2d_tiny", 1), ("cyl3d_tiny", 1), ("ring2d", 1),
                                         ("cyl3d_mid", 97), ("cyl3d_12gb", 1031)])
def test_device_generator_matches_host(pkg, name, stride):
    geo = pkg.preset(name, row_stride=stride)
    rp, c, v, cols = pkg.siddon_host(geo)
    m = pkg.Matrix.generate(geo, build_transpose=False)
    grp, gc, gv = m.csr()
    assert np.array_equal(grp, rp)
    assert np.array_equal(gc, c)
    assert np.array_equal(gv.view(np.uint32), v.view(np.uint32))
    m.close()


# ------------------------------------------------------- compressed indices
@pytest.mark.parametrize("vt", [0, 1, 2])
def test_d16_projection_matches_oracle(pkg, O, golden, cuda, vt):
    # rows out of order (rand_dup, with repeated columns) are sorted in the D16 copy; gaps of
    # 65,536 or more columns (rand_long, one_row) are bridged by dummy entries
    for name in ("rand_small", "rand_long", "rand_dup", "one_row", "empty_rows", "tall", "cyl3d_tiny"):
        rp, c, v, cols = golden_csr(golden, name)
        m = pkg.Matrix.from_csr(rp, c, v, cols, value_type=vt, compress=True)
        x = golden[f"{name}/x"]
        dx, dg = dev(cuda, x), dev(cuda, np.zeros(m.rows, np.int32))
        ratio = cuda.zeros(m.rows, dtype=cuda.float32, device="cuda")
        fp = cuda.full((m.rows,), -1.0, dtype=cuda.float32, device="cuda")
        m.forward_project(dx.data_ptr(), dg.data_ptr(), ratio.data_ptr(), fp.data_ptr(), kernel=pkg.KERNEL_D16)
        cuda.cuda.synchronize()
        vq = {0: v, 1: v.astype(np.float16).astype(np.float32)}.get(vt)
        if vq is None:  # bf16: round to nearest even on the top 16 bits
            u = v.view(np.uint32).astype(np.uint64)
            u = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
            vq = u.astype(np.uint32).view(np.float32)
        want = O.spmv_csrvec(rp, c, vq, x)
        np.testing.assert_allclose(fp.cpu().numpy(), want, rtol=2e-5, atol=1e-5, err_msg=name)
        m.close()


@pytest.mark.parametrize("kern", [3, 4])
def test_d16_mlem(pkg, O, kern):
    p = problem(pkg, O, "cyl3d_tiny_dense")
    A = (p["rp"], p["col"], p["val"])
    ref64 = O.mlem_f64(A, p["g"], p["norm"], p["f0"], 20)
    m = pkg.Matrix.from_csr(*A, p["cols"], norm=p["norm"], compress=True)
    got = m.run(p["g"], 20, f0=p["f0"], kernel=kern)
    assert O.rel_l2(got, ref64) < TOL_F32
    m.close()
    mh = pkg.Matrix.from_csr(*A, p["cols"], value_type=pkg.VAL_F16, compress=True)
    ref64h = O.mlem_f64(A, p["g"], O.colsum(*A, p["cols"]), p["f0"], 20)
    got = mh.run(p["g"], 20, f0=p["f0"], kernel=kern)
    assert O.rel_l2(got, ref64h) < TOL_LOWP
    assert mh.device_bytes > 0
    mh.close()


@pytest.mark.parametrize("vt", [0, 1, 2])
def test_interleaved_projection_matches_oracle(pkg, O, golden, cuda, vt):
    for name in ("rand_small", "rand_long", "rand_dup", "one_row", "empty_rows", "tall", "cyl3d_tiny"):
        rp, c, v, cols = golden_csr(golden, name)
        m = pkg.Matrix.from_csr(rp, c, v, cols, value_type=vt, interleave=True)
        x = golden[f"{name}/x"]
        dx, dg = dev(cuda, x), dev(cuda, np.zeros(m.rows, np.int32))
        ratio = cuda.zeros(m.rows, dtype=cuda.float32, device="cuda")
        fp = cuda.full((m.rows,), -1.0, dtype=cuda.float32, device="cuda")
        m.forward_project(dx.data_ptr(), dg.data_ptr(), ratio.data_ptr(), fp.data_ptr(), kernel=pkg.KERNEL_ILV)
        cuda.cuda.synchronize()
        got = fp.cpu().numpy()
        if vt == 0:
            # the lane-strided order of mat_vec_mul_csr_vector: within FMA rounding of the oracle
            want = O.spmv_csrvec(rp, c, v, x)
            np.testing.assert_allclose(got, want, rtol=2e-6, atol=1e-6, err_msg=name)
        else:
            want = O.spmv_csrvec(rp, c, v, x)
            np.testing.assert_allclose(got, want, rtol=1e-2, atol=1e-3, err_msg=name)
        m.close()


def test_interleaved_and_compressed_mlem(pkg, O):
    p = problem(pkg, O, "cyl3d_tiny_dense")
    A = (p["rp"], p["col"], p["val"])
    ref64 = O.mlem_f64(A, p["g"], p["norm"], p["f0"], 20)
    m = pkg.Matrix.from_csr(*A, p["cols"], norm=p["norm"], interleave=True, compress=True)
    for kern in (3, 4, 5):
        got = m.run(p["g"], 20, f0=p["f0"], kernel=kern)
        assert O.rel_l2(got, ref64) < TOL_F32, kern
    fp_cfg, bp_cfg = m.tuning(False), m.tuning(True)
    assert fp_cfg["ms"] > 0 and bp_cfg["ms"] > 0
    m.close()


@pytest.mark.parametrize("name", ["ring2d", "cyl3d_tiny"])
def test_generated_matrix_locality_order(pkg, O, name):
    """Rows processed in LOR-tube / voxel-brick order give the same image."""
    geo = pkg.preset(name, sub_t=4, sub_z=2, width_t=6.0, width_z=2.0) if name == "cyl3d_tiny" else pkg.preset(name)
    rp, c, v, cols = pkg.siddon_host(geo)
    from mlem_gb300 import synth
    g = synth.poisson_sinogram(synth.project_host(rp, c, v, synth.phantom(geo, 4, seed=9)), 1e6, seed=10)
    m = pkg.Matrix.generate(geo)
    norm = m.norm()
    f0 = np.full(cols, m.initial_value(g), np.float32)
    ref64 = O.mlem_f64((rp, c, v), g, norm, f0, 15)
    for kern in (pkg.KERNEL_ORDERED, pkg.KERNEL_AUTO):
        got = m.run(g, 15, f0=f0, kernel=kern)
        assert O.rel_l2(got, ref64) < TOL_F32, kern
    t = m.tuning(False)
    assert set(t) >= {"kernel", "lanes_per_row", "vectors_in_flight", "locality_order", "pipelined", "ms"}
    m.close()


@pytest.mark.parametrize("name", ["ring2d", "cyl3d_tiny_dense"])
def test_pipelined_and_ordered_kernels_bit_identical_to_direct(pkg, O, name):
    """The persistent software-pipelined kernel (1 or 2 vectors per step) and
    the locality row order change neither a row's summation order nor the
    result: images are bitwise equal to the direct kernel with the same lanes."""
    p = problem(pkg, O, name)
    m = pkg.Matrix.generate(p["geo"])
    f0 = np.full(m.cols, m.initial_value(p["g"]), np.float32)
    ref64 = O.mlem_f64((p["rp"], p["col"], p["val"]), p["g"], m.norm().astype(np.float64), f0, 8)
    for lanes in (16, 32):
        want = m.run(p["g"], 8, f0=f0, kernel=pkg.KERNEL_DIRECT, lanes=lanes, unroll=2)
        assert O.rel_l2(want, ref64) < TOL_F32
        for kern in (pkg.KERNEL_DIRECT, pkg.KERNEL_PERSISTENT):
            for unroll in (1, 2):
                for order in (False, True):
                    for pipe in ((False, True) if kern == pkg.KERNEL_DIRECT else (False,)):
                        for graph in (True, False):
                            got = m.run(p["g"], 8, f0=f0, kernel=kern, lanes=lanes, unroll=unroll, row_order=order,
                                        pipeline=pipe, use_graph=graph)
                            assert np.array_equal(got, want), (lanes, kern, unroll, order, pipe, graph)
        got = m.run(p["g"], 8, f0=f0, kernel=pkg.KERNEL_ORDERED, lanes=lanes)
        assert np.array_equal(got, want)
        got = m.run(p["g"], 8, f0=f0, kernel=pkg.KERNEL_ORDERED, lanes=lanes, pipeline=True)
        assert np.array_equal(got, want)
    with pytest.raises(pkg.MlemError):
        m.run(p["g"], 1, kernel=pkg.KERNEL_PERSISTENT, lanes=8)
    with pytest.raises(pkg.MlemError):
        m.run(p["g"], 1, kernel=pkg.KERNEL_DIRECT, lanes=8, row_order=True)
    m.close()
    h = pkg.Matrix.from_csr(p["rp"], p["col"], p["val"], p["cols"])
    with pytest.raises(pkg.MlemError):
        h.run(p["g"], 1, kernel=pkg.KERNEL_DIRECT, row_order=True)
    h.close()
