"""The allocation-free merge-path forward projection (GPU, through the C ABI).

Callers that cannot allocate device memory use
mlem_forward_project_merge_noalloc, whose scratch is a fixed array inside
the library.  Its ratio must agree with the allocating entry point
(mlem_forward_project, merge-based) on two calls in a row, since the second
call finds the first call's leftovers in the shared array.  This file is
collected last so a failure here leaves every other test already run.
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
