"""ctypes view of the oracle (test infrastructure only).

Only tests/, __graft_entry__.smoke() and bench.py's CPU legs use this module,
as the checker.  liboracle.so is the C restatement in mlem_oracle.c;
libmlemref.so (optional, only where the reference checkout exists) is the
reference's own code compiled by ref_build.py.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
_P = C.c_void_p
_SIGS = {
    "oracle_transpose": (None, [C.c_uint32, C.c_uint32, C.c_uint64, _P, _P, _P, _P, _P, _P]),
    "oracle_merge_search": (None, [_P, C.c_uint32, C.c_uint32, C.c_uint64, _P, _P]),
    "oracle_merge_search_mg": (None, [_P, C.c_uint32, C.c_uint64, C.c_uint32, C.c_uint64, _P, _P]),
    "oracle_spmv_csrvec": (None, [_P, _P, _P, _P, C.c_uint32, _P, C.c_int]),
    "oracle_spmv_merge": (None, [_P, _P, _P, _P, C.c_uint32, C.c_uint64, C.c_uint32, C.c_uint64, _P, C.c_int]),
    "oracle_scatter": (None, [_P, _P, _P, _P, C.c_uint32, _P]),
    "oracle_correl": (None, [_P, _P, C.c_uint32]),
    "oracle_update": (None, [_P, _P, _P, C.c_uint32]),
    "oracle_colsum_f32": (None, [_P, _P, _P, C.c_uint32, C.c_uint32, _P]),
    "oracle_colsum_f64": (None, [_P, _P, _P, C.c_uint32, C.c_uint32, _P]),
    "oracle_initial_value": (C.c_float, [_P, C.c_uint32, _P, C.c_uint32]),
    "oracle_mlem_f32": (None, [_P, _P, _P, _P, _P, _P, _P, _P, _P, C.c_uint32, C.c_uint32, C.c_uint64,
                               C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32, C.c_int]),
    "oracle_mlem_f64": (None, [_P, _P, _P, _P, _P, _P, C.c_uint32, C.c_uint32, C.c_uint32, _P, _P]),
    "oracle_mlem_f64_t": (None, [_P, _P, _P, _P, _P, _P, _P, _P, _P, C.c_uint32, C.c_uint32, C.c_uint32, _P, _P]),
    "oracle_mlem_omp": (None, [_P, _P, _P, _P, _P, _P, _P, _P, _P, C.c_uint32, C.c_uint32, C.c_uint32, C.c_int]),
    "oracle_max_threads": (C.c_int, []),
    "oracle_colsum_f64_t": (None, [_P, _P, C.c_uint32, _P]),
    "oracle_project_f64": (None, [_P, _P, _P, _P, C.c_uint32, _P]),
    "oracle_siddon_rows": (C.c_uint64, [_P]),
    "oracle_siddon_count": (C.c_int, [_P, _P]),
    "oracle_siddon_fill": (C.c_int, [_P, _P, _P, _P]),
}
_REF_SIGS = {
    "ref_sptrans": (None, [C.c_int, C.c_uint32, C.c_uint32, C.c_uint64, _P, _P, _P, _P, _P, _P]),
    "ref_csr4_header": (C.c_int, [C.c_char_p, _P, _P, _P]),
    "ref_csr4_read": (C.c_int, [C.c_char_p, _P, _P, _P]),
    "ref_spmv": (None, [C.c_int, C.c_int, C.c_uint32, _P, _P, _P, _P, C.c_uint32, C.c_uint64, _P]),
    "ref_mlem": (None, [_P, _P, _P, _P, _P, _P, _P, _P, _P, C.c_uint32, C.c_uint32, C.c_uint64, C.c_uint32,
                        C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32]),
}
_lib = None
_ref = None


def _bind(lib, sigs):
    for n, (r, a) in sigs.items():
        f = getattr(lib, n)
        f.restype = r
        f.argtypes = a
    return lib


def lib():
    global _lib
    if _lib is None:
        from oracle.build import build
        _lib = _bind(C.CDLL(str(build())), _SIGS)
    return _lib


def ref():
    """The reference compiled here, or None where its sources are absent."""
    global _ref
    if _ref is None:
        from oracle import ref_build
        p = ref_build.build() if ref_build.available() else (ref_build.OUT if ref_build.OUT.exists() else None)
        if p is None:
            return None
        _ref = _bind(C.CDLL(str(p)), _REF_SIGS)
    return _ref


def P(a):
    return None if a is None else a.ctypes.data


def c64(a):
    return np.ascontiguousarray(a, np.uint64)


def c32(a):
    return np.ascontiguousarray(a, np.uint32)


def f32(a):
    return np.ascontiguousarray(a, np.float32)


def i32(a):
    return np.ascontiguousarray(a, np.int32)


def transpose(rowptr, col, val, cols):
    rowptr, col, val = c64(rowptr), c32(col), f32(val)
    nnz = len(col)
    cp = np.zeros(cols + 1, np.uint64)
    rt = np.zeros(max(nnz, 1), np.uint32)
    vt = np.zeros(max(nnz, 1), np.float32)
    lib().oracle_transpose(len(rowptr) - 1, cols, nnz, P(rowptr), P(col), P(val), P(cp), P(rt), P(vt))
    return cp, rt[:nnz], vt[:nnz]


def merge_search(rowptr, rows, secsize, nthreads, mg=False, nnz=None):
    rowptr = c64(rowptr)
    i = np.zeros(max(nthreads, 1), np.int64)
    j = np.zeros(max(nthreads, 1), np.int64)
    if mg:
        lib().oracle_merge_search_mg(P(rowptr), rows, nnz, secsize, nthreads, P(i), P(j))
    else:
        lib().oracle_merge_search(P(rowptr), rows, secsize, nthreads, P(i), P(j))
    return i[:nthreads], j[:nthreads]


def spmv_csrvec(rowptr, col, val, x, use_fma=1):
    rowptr, col, val, x = c64(rowptr), c32(col), f32(val), f32(x)
    y = np.zeros(len(rowptr) - 1, np.float32)
    lib().oracle_spmv_csrvec(P(rowptr), P(col), P(val), P(x), len(rowptr) - 1, P(y), use_fma)
    return y


def spmv_merge(rowptr, col, val, x, secsize, use_fma=1):
    rowptr, col, val, x = c64(rowptr), c32(col), f32(val), f32(x)
    rows = len(rowptr) - 1
    nnz = len(col)
    nthreads = -(-(rows + nnz) // (1024 * secsize)) * 1024
    y = np.zeros(rows, np.float32)
    lib().oracle_spmv_merge(P(rowptr), P(col), P(val), P(x), rows, nnz, secsize, nthreads, P(y), use_fma)
    return y


def scatter(rowptr, col, val, x, cols):
    rowptr, col, val, x = c64(rowptr), c32(col), f32(val), f32(x)
    y = np.zeros(cols, np.float32)
    lib().oracle_scatter(P(rowptr), P(col), P(val), P(x), len(rowptr) - 1, P(y))
    return y


def colsum(rowptr, col, val, cols, f64=True):
    rowptr, col, val = c64(rowptr), c32(col), f32(val)
    out = np.zeros(cols, np.float32)
    fn = lib().oracle_colsum_f64 if f64 else lib().oracle_colsum_f32
    fn(P(rowptr), P(col), P(val), len(rowptr) - 1, cols, P(out))
    return out


def colsum_t(AT, cols):
    """FP64 column sums from the rows of Aᵀ (parallel; the same bits as colsum)."""
    rpt, vt = c64(AT[0]), f32(AT[2])
    out = np.zeros(cols, np.float32)
    lib().oracle_colsum_f64_t(P(rpt), P(vt), cols, P(out))
    return out


def initial_value(g, norm):
    g, norm = i32(g), f32(norm)
    return lib().oracle_initial_value(P(g), len(g), P(norm), len(norm))


def mlem_f32(A, AT, g, norm, f0, iterations, spmv=1, secsize_fp=5, secsize_bp=5, using_trans=0, use_fma=1):
    rp, c, v = c64(A[0]), c32(A[1]), f32(A[2])
    if AT is None:
        rpt = ct = vt = None
    else:
        rpt, ct, vt = c64(AT[0]), c32(AT[1]), f32(AT[2])
    g, norm = i32(g), f32(norm)
    f = f32(f0).copy()
    lib().oracle_mlem_f32(P(rp), P(c), P(v), P(rpt), P(ct), P(vt), P(g), P(norm), P(f), len(rp) - 1, len(norm),
                          len(c), iterations, spmv, secsize_fp, secsize_bp, using_trans, use_fma)
    return f


def mlem_f64(A, g, norm, f0, iterations, loglik=False):
    rp, c, v = c64(A[0]), c32(A[1]), f32(A[2])
    g = i32(g)
    norm = np.ascontiguousarray(norm, np.float64)
    f0 = np.ascontiguousarray(f0, np.float64)
    out = np.zeros(len(norm), np.float64)
    ll = np.zeros(iterations, np.float64)
    lib().oracle_mlem_f64(P(rp), P(c), P(v), P(g), P(norm), P(f0), len(rp) - 1, len(norm), iterations, P(out), P(ll))
    return (out, ll) if loglik else out


def mlem_f64_t(A, AT, g, norm, f0, iterations, loglik=False):
    """mlem_f64 with the back projection over rows of AT (OpenMP), for full-size matrices."""
    rp, c, v = c64(A[0]), c32(A[1]), f32(A[2])
    rpt, ct, vt = c64(AT[0]), c32(AT[1]), f32(AT[2])
    g = i32(g)
    norm = np.ascontiguousarray(norm, np.float64)
    f0 = np.ascontiguousarray(f0, np.float64)
    out = np.zeros(len(norm), np.float64)
    ll = np.zeros(iterations, np.float64)
    lib().oracle_mlem_f64_t(P(rp), P(c), P(v), P(rpt), P(ct), P(vt), P(g), P(norm), P(f0), len(rp) - 1, len(norm),
                            iterations, P(out), P(ll))
    return (out, ll) if loglik else out


def mlem_omp(A, AT, g, norm, f0, iterations, nthreads=0):
    rp, c, v = c64(A[0]), c32(A[1]), f32(A[2])
    rpt, ct, vt = c64(AT[0]), c32(AT[1]), f32(AT[2])
    g, norm = i32(g), f32(norm)
    f = f32(f0).copy()
    lib().oracle_mlem_omp(P(rp), P(c), P(v), P(rpt), P(ct), P(vt), P(g), P(norm), P(f), len(rp) - 1, len(norm),
                          iterations, nthreads)
    return f


class Geometry(C.Structure):
    """Scanner description of the synthetic matrices (the field layout of the
    library's mlem_geometry)."""
    _fields_ = [("det_per_ring", C.c_uint32), ("n_rings", C.c_uint32), ("radius", C.c_float),
                ("ring_pitch", C.c_float), ("nx", C.c_uint32), ("ny", C.c_uint32), ("nz", C.c_uint32),
                ("vx", C.c_float), ("vy", C.c_float), ("vz", C.c_float), ("row_stride", C.c_uint32),
                ("row_phase", C.c_uint32), ("sub_t", C.c_uint32), ("sub_z", C.c_uint32),
                ("width_t", C.c_float), ("width_z", C.c_float)]


def geometry_of(geo) -> Geometry:
    """An oracle Geometry from any object with the same attribute names."""
    return Geometry(*[getattr(geo, n) for n, _ in Geometry._fields_])


def siddon(geo):
    """The synthetic system matrix of a scanner, generated on the host CPU
    (OpenMP).  Returns (rowptr u64[rows+1], col u32[nnz], val f32[nnz], cols)."""
    G = geometry_of(geo)
    rows = int(lib().oracle_siddon_rows(C.byref(G)))
    if rows == 0 and not (G.det_per_ring and G.n_rings):
        raise ValueError("invalid geometry")
    rp = np.zeros(rows + 1, np.uint64)
    if lib().oracle_siddon_count(C.byref(G), P(rp)) != 0:
        raise ValueError("invalid geometry")
    nnz = int(rp[-1])
    col = np.empty(max(nnz, 1), np.uint32)
    val = np.empty(max(nnz, 1), np.float32)
    lib().oracle_siddon_fill(C.byref(G), P(rp), P(col), P(val))
    return rp, col[:nnz], val[:nnz], int(G.nx * G.ny * G.nz)


def project_f64(rowptr, col, val, x):
    """A·x in FP64 (OpenMP over rows)."""
    rowptr, col, val, x = c64(rowptr), c32(col), f32(val), f32(x)
    y = np.zeros(len(rowptr) - 1, np.float64)
    lib().oracle_project_f64(P(rowptr), P(col), P(val), P(x), len(rowptr) - 1, P(y))
    return y


def max_threads() -> int:
    return int(lib().oracle_max_threads())


def rel_l2(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    d = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / (d if d > 0 else 1.0))
