"""The allocation-free merge-path forward projection (GPU, through the C ABI).

Callers that cannot allocate device memory use
mlem_forward_project_merge_noalloc, whose scratch is a fixed array inside
the library.  Its ratio must agree with the allocating entry point
(mlem_forward_project, merge-based) and with the oracle (the reference's
merge-based product and calcCorrel) on two calls in a row, since the second
call finds the first call's leftovers in the shared array.  Besides the 2-D
ring, a synthetic matrix exercises every branch of the per-thread tiles:
rows far longer than a tile (tiles inside one row, carries chained over
tiles), runs of empty rows and rows that end exactly on a tile boundary, at
section sizes 1, 33 and 125 (three tile shapes).  This file is collected last
so a failure here leaves every other test already run.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from conftest import problem

pytestmark = pytest.mark.gpu


def _dev(torch, a):
    a = np.ascontiguousarray(a)
    view = {np.dtype(np.uint64): np.int64, np.dtype(np.uint32): np.int32}.get(a.dtype)
    return torch.from_numpy((a.view(view) if view else a).copy()).cuda()


def test_noalloc_forward_projection_matches_allocating_entry_point(pkg, O, cuda):
    torch = cuda
    lib = pkg.load_library()
    p = problem(pkg, O, "ring2d")
    rows, cols, nnz = len(p["rp"]) - 1, p["cols"], len(p["col"])
    m = pkg.Matrix.from_csr(p["rp"], p["col"], p["val"], cols)
    rp_d, col_d, val_d, g_d = _dev(torch, p["rp"]), _dev(torch, p["col"]), _dev(torch, p["val"]), _dev(torch, p["g"])
    stream = torch.cuda.current_stream().cuda_stream
    rng = np.random.Generator(np.random.PCG64(11))
    for call, secsize in enumerate((5, 9)):
        x = _dev(torch, rng.uniform(0.1, 2.0, cols).astype(np.float32))
        want = torch.zeros(rows, dtype=torch.float32, device="cuda")
        got = torch.full((rows,), -1.0, dtype=torch.float32, device="cuda")
        m.forward_project(x.data_ptr(), g_d.data_ptr(), want.data_ptr(), spmv=pkg.SPMV_MERGE, secsize_fp=secsize,
                          stream=stream)
        st = lib.mlem_forward_project_merge_noalloc(
            C.c_void_p(rp_d.data_ptr()), C.c_void_p(col_d.data_ptr()), C.c_void_p(val_d.data_ptr()), rows, cols,
            nnz, C.c_void_p(x.data_ptr()), C.c_void_p(g_d.data_ptr()), C.c_void_p(got.data_ptr()), secsize,
            C.c_void_p(stream))
        assert st == 0, lib.mlem_last_error().decode()
        torch.cuda.synchronize()
        a, b = got.cpu().numpy(), want.cpu().numpy()
        np.testing.assert_allclose(a, b, rtol=1e-5, atol=1e-7, err_msg=f"call {call}")
        assert O.rel_l2(a, b) < 1e-6
    m.close()


def _tile_items(secsize):
    """Items (row ends + nonzeros) per tile of the allocation-free kernel."""
    T = max(32, min(256, (4000 // secsize) & ~31))
    return T * secsize


def _synthetic_csr(secsize, seed):
    """Rows of 10k-40k nonzeros, runs of empty rows, short rows, and every
    7th row sized so that its end marker is the last item of a tile."""
    TS = _tile_items(secsize)
    rng = np.random.Generator(np.random.PCG64(seed))
    lengths, nnz = [], 0
    for r in range(2400):
        if r in (5, 700, 1600):
            n = int(rng.integers(10_000, 40_000))
        elif 100 <= r % 600 < 160:
            n = 0
        elif r % 7 == 3:
            n = (-(nnz + r + 1)) % TS
        else:
            n = int(rng.integers(0, 40))
        lengths.append(n)
        nnz += n
    rp = np.concatenate([[0], np.cumsum(lengths)]).astype(np.uint64)
    cols = 5000
    col = np.concatenate([np.sort(rng.choice(cols, n, replace=n > cols)) for n in lengths]).astype(np.uint32)
    val = rng.uniform(0.05, 1.5, nnz).astype(np.float32)
    ends = (rp[1:] + np.arange(1, len(lengths) + 1, dtype=np.uint64)) % TS
    assert (ends == 0).sum() >= 300  # rows ending on a tile boundary
    return rp, col, val, cols


@pytest.mark.parametrize("secsize", [1, 33, 125])
def test_noalloc_synthetic_rows_match_oracle(pkg, O, cuda, secsize):
    torch = cuda
    lib = pkg.load_library()
    rp, col, val, cols = _synthetic_csr(secsize, seed=secsize)
    rows, nnz = len(rp) - 1, len(col)
    g = (np.arange(rows) % 13).astype(np.int32)
    m = pkg.Matrix.from_csr(rp, col, val, cols)
    rp_d, col_d, val_d, g_d = _dev(torch, rp), _dev(torch, col), _dev(torch, val), _dev(torch, g)
    stream = torch.cuda.current_stream().cuda_stream
    rng = np.random.Generator(np.random.PCG64(100 + secsize))
    for call in range(2):
        xh = rng.uniform(0.1, 2.0, cols).astype(np.float32)
        x = _dev(torch, xh)
        got = torch.full((rows,), -1.0, dtype=torch.float32, device="cuda")
        want = torch.zeros(rows, dtype=torch.float32, device="cuda")
        st = lib.mlem_forward_project_merge_noalloc(
            C.c_void_p(rp_d.data_ptr()), C.c_void_p(col_d.data_ptr()), C.c_void_p(val_d.data_ptr()), rows, cols,
            nnz, C.c_void_p(x.data_ptr()), C.c_void_p(g_d.data_ptr()), C.c_void_p(got.data_ptr()), secsize,
            C.c_void_p(stream))
        assert st == 0, lib.mlem_last_error().decode()
        m.forward_project(x.data_ptr(), g_d.data_ptr(), want.data_ptr(), spmv=pkg.SPMV_MERGE, secsize_fp=secsize,
                          stream=stream)
        torch.cuda.synchronize()
        a = got.cpu().numpy()
        # oracle: the reference's merge-based product (kernel.cu:190-286) and calcCorrel (kernel.cu:11-19)
        fp = O.spmv_merge(rp, col, val, xh, secsize)
        ref = fp.copy()
        O.lib().oracle_correl(O.P(g), O.P(ref), rows)
        empty = np.diff(rp.astype(np.int64)) == 0
        assert np.all(a[empty] == 0.0)  # zero guard of calcCorrel
        np.testing.assert_allclose(a, ref, rtol=1e-5, atol=0, err_msg=f"secsize {secsize} call {call} vs oracle")
        np.testing.assert_allclose(a, want.cpu().numpy(), rtol=1e-5, atol=0,
                                   err_msg=f"secsize {secsize} call {call} vs allocating path")
        assert O.rel_l2(a, ref) < 1e-6
    m.close()


def test_noalloc_rejects_inputs_beyond_its_scratch(pkg, cuda):
    torch = cuda
    lib = pkg.load_library()
    dummy = torch.zeros(16, dtype=torch.int64, device="cuda")
    ptr = C.c_void_p(dummy.data_ptr())
    # 2^31 rows + nnz needs far more than the fixed scratch: refused before any launch
    st = lib.mlem_forward_project_merge_noalloc(ptr, ptr, ptr, 1 << 30, 16, 1 << 31, ptr, ptr, ptr, 5, None)
    assert pkg.STATUS[st] == "EINVAL"
    assert "scratch" in lib.mlem_last_error().decode()
    st = lib.mlem_forward_project_merge_noalloc(ptr, ptr, ptr, 4, 4, 4, ptr, ptr, ptr, 200, None)
    assert pkg.STATUS[st] == "EINVAL"
    # rows + nnz beyond 64 bits: refused, not wrapped to a small size
    st = lib.mlem_forward_project_merge_noalloc(ptr, ptr, ptr, 16, 4, (1 << 64) - 8, ptr, ptr, ptr, 5, None)
    assert pkg.STATUS[st] == "EINVAL" and "overflow" in lib.mlem_last_error().decode()
