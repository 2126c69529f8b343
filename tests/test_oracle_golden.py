"""The oracle against the reference's own outputs (CPU, bit-exact).

The fixtures in tests/golden/reference_outputs.npz were produced by the
reference's sources compiled here (tests/golden/make_golden.py).  The oracle
restates kernel.cu in C; with FMA contraction off (the reference compiled for
the host has separate multiply and add) every result must match bit for bit.
"""
from __future__ import annotations

import numpy as np
import pytest

from conftest import golden_cases, golden_csr


def bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


def test_transpose_bitexact(O, golden):
    for name in golden_cases(golden):
        rp, c, v, cols = golden_csr(golden, name)
        cp, rt, vt = O.transpose(rp, c, v, cols)
        assert np.array_equal(cp, golden[f"{name}/T_colptr"]), name
        assert np.array_equal(rt, golden[f"{name}/T_row"]), name
        assert np.array_equal(bits(vt), bits(golden[f"{name}/T_val"])), name


def test_kernels_bitexact(O, golden):
    for name in golden_cases(golden):
        rp, c, v, cols = golden_csr(golden, name)
        x, r = golden[f"{name}/x"], golden[f"{name}/r"]
        assert np.array_equal(bits(O.spmv_csrvec(rp, c, v, x, use_fma=0)), bits(golden[f"{name}/y_csrvec"])), name
        for ss in (1, 2, 5, 9):
            got = O.spmv_merge(rp, c, v, x, ss, use_fma=0)
            assert np.array_equal(bits(got), bits(golden[f"{name}/y_merge{ss}"])), (name, ss)
        assert np.array_equal(bits(O.scatter(rp, c, v, r, cols)), bits(golden[f"{name}/y_scatter"])), name


def test_mlem_loop_bitexact(O, golden):
    n = 0
    for name in ("ring2d_tiny", "cyl3d_tiny"):
        rp, c, v, cols = golden_csr(golden, name)
        AT = (golden[f"{name}/T_colptr"], golden[f"{name}/T_row"], golden[f"{name}/T_val"])
        g, norm, f0 = golden[f"{name}/g"], golden[f"{name}/norm"], golden[f"{name}/f0"]
        assert O.initial_value(g, norm) == f0[0]
        for k in golden.files:
            if not k.startswith(f"{name}/mlem_"):
                continue
            p = k.split("/")[1].split("_")
            spmv, ut, it = int(p[1][1:]), int(p[2][1:]), int(p[4][2:])
            ss = [int(q) for q in p[3][2:].split("x")]
            f = O.mlem_f32((rp, c, v), AT if ut == 0 else None, g, norm, f0, it, spmv, ss[0], ss[1], ut, use_fma=0)
            assert np.array_equal(bits(f), bits(golden[k])), k
            n += 1
    assert n == 2 * 18


def test_fma_and_f64_oracles_agree_within_tolerance(O, golden):
    name = "cyl3d_tiny"
    rp, c, v, cols = golden_csr(golden, name)
    g, norm, f0 = golden[f"{name}/g"], golden[f"{name}/norm"], golden[f"{name}/f0"]
    AT = (golden[f"{name}/T_colptr"], golden[f"{name}/T_row"], golden[f"{name}/T_val"])
    ref = golden[f"{name}/mlem_s1_t0_ss5x5_it12"]
    f_fma = O.mlem_f32((rp, c, v), AT, g, norm, f0, 12, 1, use_fma=1)
    f64 = O.mlem_f64((rp, c, v), g, norm, f0, 12)
    assert O.rel_l2(f_fma, ref) < 1e-6
    assert O.rel_l2(f64, ref) < 1e-5
    omp = O.mlem_omp((rp, c, v), AT, g, norm, f0, 12, 2)
    assert O.rel_l2(omp, f64) < 1e-6


def test_reference_recompiled_matches_oracle_on_new_inputs(O):
    """Where the reference checkout exists, compare live on fresh random inputs."""
    ref = O.ref()
    if ref is None:
        pytest.skip("reference sources not present on this machine")
    rng = np.random.Generator(np.random.PCG64(99))
    rows, cols = 500, 300
    lens = rng.integers(0, 40, rows)
    rp = np.zeros(rows + 1, np.uint64)
    rp[1:] = np.cumsum(lens)
    col = np.concatenate([np.sort(rng.choice(cols, n, replace=False)) for n in lens]).astype(np.uint32)
    val = rng.uniform(0.01, 1.5, len(col)).astype(np.float32)
    for threads in (1, 5):
        cp = np.zeros(cols + 1, np.uint64)
        rt = np.zeros(len(col), np.uint32)
        vt = np.zeros(len(col), np.float32)
        ref.ref_sptrans(threads, rows, cols, len(col), O.P(rp), O.P(col), O.P(val), O.P(rt), O.P(cp), O.P(vt))
        mine = O.transpose(rp, col, val, cols)
        assert np.array_equal(mine[0], cp) and np.array_equal(mine[1], rt) and np.array_equal(bits(mine[2]), bits(vt))
    x = rng.uniform(0.1, 2, cols).astype(np.float32)
    for ss in (1, 3, 7):
        y = np.zeros(rows, np.float32)
        ref.ref_spmv(0, 0, ss, O.P(rp), O.P(col), O.P(val), O.P(x), rows, len(col), O.P(y))
        assert np.array_equal(bits(y), bits(O.spmv_merge(rp, col, val, x, ss, use_fma=0)))


# --------------------------------------------------------- merge-path search
def _random_rowptr(rng, rows, mean):
    lens = rng.poisson(mean, rows)
    lens[rng.random(rows) < 0.3] = 0
    rp = np.zeros(rows + 1, np.uint64)
    rp[1:] = np.cumsum(lens)
    return rp


@pytest.mark.parametrize("rows,mean", [(1, 50), (2, 3), (3, 0), (17, 4), (1000, 7), (5000, 0.2), (300, 300)])
def test_merge_search_equals_merrill_garland(O, rows, mean):
    rng = np.random.Generator(np.random.PCG64(rows))
    rp = _random_rowptr(rng, rows, mean)
    nnz = int(rp[-1])
    for ss in (1, 2, 5, 13):
        nthreads = (rows + nnz) // ss + 1      # every thread start up to the terminal diagonal
        i, j = O.merge_search(rp, rows, ss, nthreads)
        mi, mj = O.merge_search(rp, rows, ss, nthreads, mg=True, nnz=nnz)
        d = np.arange(nthreads, dtype=np.int64) * ss
        inside = d < rows + nnz
        if rows == 1:
            # the reference loop never runs for rows == 1: (0, d) on every diagonal
            assert np.all(i == 0) and np.array_equal(j, d)
            ok = d <= nnz
            assert np.array_equal(i[ok], mi[ok]) and np.array_equal(j[ok], mj[ok])
        else:
            assert np.array_equal(i[inside], mi[inside]) and np.array_equal(j[inside], mj[inside])
        assert np.array_equal(i + j, d)  # every coordinate lies on its diagonal


def test_f64_oracle_transposed_form_agrees(pkg, O):
    """The FP64 oracle with its back projection over Aᵀ (used at full size)
    equals the row-scatter form to FP64 rounding."""
    from conftest import problem
    p = problem(pkg, O, "cyl3d_tiny")
    A = (p["rp"], p["col"], p["val"])
    AT = O.transpose(*A, p["cols"])
    a, lla = O.mlem_f64(A, p["g"], p["norm"], p["f0"], 12, loglik=True)
    b, llb = O.mlem_f64_t(A, AT, p["g"], p["norm"], p["f0"], 12, loglik=True)
    assert O.rel_l2(b, a) < 1e-13
    np.testing.assert_allclose(llb, lla, rtol=1e-13)
