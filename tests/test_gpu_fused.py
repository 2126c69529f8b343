"""The fused single pass (bp_mode 2: forward projection, correlation and the
scatter back projection of argv[7]=1, the matrix read once per iteration) in each
of its forms, and the scatter back projection streamed through shared-memory
rings (bp_mode 1, kernel TMA), against the oracle (GPU, via the C ABI).

The staged form cuts the rows into chunks of at most 4,096 staged entries and 128
rows and reads a row longer than a stage from global memory.  The ragged matrix
below puts rows on both sides of those limits, runs of empty rows longer than a
chunk's row limit, rows without counts and a wide last row through it.

Tolerances: the image after N iterations within 1e-5 relative L2 of the FP32
oracle's non-transposed MLEM (kernel.cu:118-130, 11-19, 165-177, 28-39) and of the
FP64 oracle (the back-projection sums are atomic in the reference and here, so
only their order differs); FP16 values within 1e-3 of the FP64 oracle; the FP64
log-likelihood within 1e-6 relative.
"""
from __future__ import annotations

import numpy as np
import pytest

from conftest import problem

pytestmark = pytest.mark.gpu

TOL_F32 = 1e-5
TOL_LOWP = 1e-3
FORMS = {"rescan": 0, "staged": 1, "register": 2, "auto": 3}  # the run option `kernel` of the fused pass


def ragged(seed=11, rows=3000, cols=60000):
    rng = np.random.Generator(np.random.PCG64(seed))
    lens = rng.integers(1, 600, rows)
    lens[rng.random(rows) < 0.15] = 0
    lens[200:560] = 0  # 360 empty rows in a row: more than one chunk's 128
    # rows at and around a stage's 4,096 entries (8-aligned spans) and longer
    for i, n in zip(range(1000, 1012), [4080, 4088, 4089, 4090, 4093, 4095, 4096, 4097, 4100, 8192, 9001, 20000]):
        lens[i] = n
    lens[rows - 1] = 5000  # the last row is wide
    rp = np.zeros(rows + 1, np.uint64)
    rp[1:] = np.cumsum(lens)
    col = np.concatenate([np.sort(rng.choice(cols, n, replace=False)) for n in lens if n]).astype(np.uint32)
    val = rng.uniform(0.05, 1.0, len(col)).astype(np.float32)
    xt = rng.uniform(0.0, 1.0, cols)
    A = (rp, col, val)
    return A, cols, rng, xt


def sinogram(O, A, xt, rng):
    g = rng.poisson(O.project_f64(*A, xt) * 50.0).astype(np.int32)
    g[rng.random(len(g)) < 0.2] = 0  # rows without counts scatter nothing
    return g


@pytest.mark.parametrize("form", list(FORMS))
def test_ragged_rows_against_oracle(pkg, O, form):
    A, cols, rng, xt = ragged()
    g = sinogram(O, A, xt, rng)
    norm = O.colsum(*A, cols, f64=True)
    f0 = np.full(cols, O.initial_value(g, norm), np.float32)
    m = pkg.Matrix.from_csr(*A, cols, norm=norm, build_transpose=False)
    iters = 12
    got = m.run(g, iters, f0=f0, bp_mode=pkg.BP_FUSED, kernel=FORMS[form])
    ref32 = O.mlem_f32(A, None, g, norm, f0, iters, spmv=1, using_trans=1)
    ref64 = O.mlem_f64(A, g, norm, f0, iters)
    assert O.rel_l2(got, ref32) < TOL_F32, O.rel_l2(got, ref32)
    assert O.rel_l2(got, ref64) < TOL_F32, O.rel_l2(got, ref64)
    assert np.all(got >= 0)
    # eager launches and graph replay give the same image up to the atomic order
    eager = m.run(g, iters, f0=f0, bp_mode=pkg.BP_FUSED, kernel=FORMS[form], use_graph=False)
    assert O.rel_l2(eager, got) < TOL_F32
    m.close()


@pytest.mark.parametrize("name", ["ring2d", "cyl3d_tiny", "cyl3d_tiny_dense"])
@pytest.mark.parametrize("form", ["staged", "rescan"])
def test_forms_on_scanners(pkg, O, name, form):
    p = problem(pkg, O, name)
    A = (p["rp"], p["col"], p["val"])
    m = pkg.Matrix.from_csr(*A, p["cols"], norm=p["norm"], build_transpose=False)
    ref64 = O.mlem_f64(A, p["g"], p["norm"], p["f0"], 20)
    for lanes, unroll in ((0, 0), (8, 1), (32, 2)):
        got = m.run(p["g"], 20, f0=p["f0"], bp_mode=pkg.BP_FUSED, kernel=FORMS[form], lanes=lanes, unroll=unroll)
        assert O.rel_l2(got, ref64) < TOL_F32, (lanes, unroll, O.rel_l2(got, ref64))
    m.close()


@pytest.mark.parametrize("layout,kern", [(0, 6), (0, 3), (1, 3), (1, 1)])
def test_generated_matrix_orders(pkg, O, layout, kern):
    """A generated matrix: rows visited in LOR-tube order (natural layout,
    kernel ORDERED or the tuner's pick) or stored in that order (locality
    layout, the tuner's pick and the staged form)."""
    geo = pkg.preset("cyl3d_tiny")
    m = pkg.Matrix.generate(geo, build_transpose=False, layout=layout)
    p = problem(pkg, O, "cyl3d_tiny")
    A = (p["rp"], p["col"], p["val"])
    ref64 = O.mlem_f64(A, p["g"], p["norm"], p["f0"], 20)
    got = m.run(p["g"], 20, f0=p["f0"], bp_mode=pkg.BP_FUSED, kernel=kern)
    assert O.rel_l2(got, ref64) < TOL_F32, O.rel_l2(got, ref64)
    m.close()


def test_staged_loglik(pkg, O):
    """The staged pass writes the projection of every row (empty rows: 0) for the
    FP64 log-likelihood."""
    A, cols, rng, xt = ragged(seed=12, rows=1500)
    g = sinogram(O, A, xt, rng)
    norm = O.colsum(*A, cols, f64=True)
    f0 = np.full(cols, O.initial_value(g, norm), np.float32)
    m = pkg.Matrix.from_csr(*A, cols, norm=norm, build_transpose=False)
    img, ll = m.run(g, 10, f0=f0, loglik=True, bp_mode=pkg.BP_FUSED, kernel=FORMS["staged"])
    _, ll64 = O.mlem_f64(A, g, norm, f0, 10, loglik=True)
    np.testing.assert_allclose(ll, ll64, rtol=1e-6)
    m.close()


@pytest.mark.parametrize("vt", [1, 2])
def test_staged_low_precision_values(pkg, O, vt):
    """FP16 / BF16 values staged as 8-entry (16-byte) units."""
    p = problem(pkg, O, "cyl3d_tiny")
    A = (p["rp"], p["col"], p["val"])
    m = pkg.Matrix.from_csr(*A, p["cols"], value_type=vt, build_transpose=False)
    ref64 = O.mlem_f64(A, p["g"], O.colsum(*A, p["cols"]), p["f0"], 20)
    got = m.run(p["g"], 20, f0=p["f0"], bp_mode=pkg.BP_FUSED, kernel=FORMS["staged"])
    tol = TOL_LOWP if vt == 1 else 1e-2
    assert O.rel_l2(got, ref64) < tol, O.rel_l2(got, ref64)
    m.close()


@pytest.mark.parametrize("kern", [1, 0, 3])
def test_scatter_forms_on_ragged_rows(pkg, O, kern):
    """bp_mode 1 (argv[7]=1): TMA rings (rows with ratio 0 and empty rows are not
    staged, long rows go in pieces of 512), the direct kernel and the tuner's pick."""
    A, cols, rng, xt = ragged(seed=13)
    g = sinogram(O, A, xt, rng)
    norm = O.colsum(*A, cols, f64=True)
    f0 = np.full(cols, O.initial_value(g, norm), np.float32)
    m = pkg.Matrix.from_csr(*A, cols, norm=norm, build_transpose=False)
    iters = 12
    got = m.run(g, iters, f0=f0, bp_mode=pkg.BP_SCATTER, kernel=kern)
    ref32 = O.mlem_f32(A, None, g, norm, f0, iters, spmv=1, using_trans=1)
    assert O.rel_l2(got, ref32) < TOL_F32, O.rel_l2(got, ref32)
    eager = m.run(g, iters, f0=f0, bp_mode=pkg.BP_SCATTER, kernel=kern, use_graph=False)
    assert O.rel_l2(eager, got) < TOL_F32
    m.close()


@pytest.mark.parametrize("vt", [1, 2])
def test_scatter_tma_low_precision_values(pkg, O, vt):
    p = problem(pkg, O, "cyl3d_tiny_dense")
    A = (p["rp"], p["col"], p["val"])
    m = pkg.Matrix.from_csr(*A, p["cols"], value_type=vt, build_transpose=False)
    ref64 = O.mlem_f64(A, p["g"], O.colsum(*A, p["cols"]), p["f0"], 20)
    got = m.run(p["g"], 20, f0=p["f0"], bp_mode=pkg.BP_SCATTER, kernel=1)
    tol = TOL_LOWP if vt == 1 else 1e-2
    assert O.rel_l2(got, ref64) < tol, O.rel_l2(got, ref64)
    m.close()
