"""GB300-native MLEM reconstructor — Python binding of the C ABI (include/mlem.h).

Host-side mirror of the reference interface (wmd0701/Bachelorarbeit-MLEM):

* :func:`mlem` has the argument list of ``mlem()`` (main.cu:19) and the same
  meaning of every switch; it runs the whole reconstruction on the GPU.
* :class:`Matrix` is the resident form: upload (or generate) once, then run
  many reconstructions, single operators, batches or a request server.

The compute path is the CUDA library ``lib/libmlem_gb300.so`` built for sm_103a
by ``build.py``; there is no CPU fallback.  Importing this module does not
need a GPU; every call that computes raises :class:`MlemError` when the
library is missing or a CUDA call fails.
"""
from __future__ import annotations

import ctypes as C
import math
from pathlib import Path

import numpy as np

PKG = Path(__file__).resolve().parent
LIB_PATH = PKG / "lib" / "libmlem_gb300.so"
CLI_PATH = PKG / "bin" / "mlem_gb300"

SPMV_MERGE, SPMV_CSR_VECTOR = 0, 1
KERNEL_DIRECT, KERNEL_TMA, KERNEL_PERSISTENT, KERNEL_AUTO, KERNEL_D16, KERNEL_ILV, KERNEL_ORDERED, KERNEL_SYM = range(8)
LAYOUT_NATURAL, LAYOUT_LOCALITY = 0, 1
VAL_F32, VAL_F16, VAL_BF16 = 0, 1, 2
BP_TRANS, BP_SCATTER, BP_FUSED = 0, 1, 2

STATUS = {0: "OK", 1: "EINVAL", 2: "EIO", 3: "ENOMEM", 4: "ECUDA", 5: "ETIMEOUT",
          6: "EUNSUPPORTED", 7: "EBUSY"}


class MlemError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{STATUS.get(code, code)}: {msg}")
        self.code = code
        self.status = STATUS.get(code, str(code))


# ------------------------------------------------------------------ C structs
class CsrHost(C.Structure):
    _fields_ = [("rows", C.c_uint32), ("cols", C.c_uint32), ("nnz", C.c_uint64),
                ("rowptr", C.c_void_p), ("col", C.c_void_p), ("val", C.c_void_p)]


class MatrixOpts(C.Structure):
    _fields_ = [("value_type", C.c_int), ("build_transpose", C.c_uint32), ("norm", C.c_void_p),
                ("device", C.c_int), ("compress_indices", C.c_uint32), ("interleave", C.c_uint32),
                ("layout", C.c_uint32), ("grid_nx", C.c_uint32), ("grid_ny", C.c_uint32), ("grid_nz", C.c_uint32),
                ("symmetry", C.c_uint32), ("sym_det_per_ring", C.c_uint32), ("sym_rings", C.c_uint32)]


class MatrixInfo(C.Structure):
    _fields_ = [("rows", C.c_uint32), ("cols", C.c_uint32), ("nnz", C.c_uint64),
                ("value_type", C.c_int), ("has_transpose", C.c_uint32), ("device_bytes", C.c_uint64),
                ("max_row_nnz", C.c_uint32), ("max_col_nnz", C.c_uint32),
                ("sym_lor_rows", C.c_uint32), ("sym_voxel_rows", C.c_uint32),
                ("sym_fp_nnz", C.c_uint64), ("sym_bp_nnz", C.c_uint64),
                ("d16_slots", C.c_uint64), ("d16_slots_t", C.c_uint64),
                ("d16_lanes", C.c_uint32), ("d16_lanes_t", C.c_uint32)]


class RunOpts(C.Structure):
    _fields_ = [("spmv", C.c_int), ("bp_mode", C.c_int), ("secsize_fp", C.c_uint32),
                ("secsize_bp", C.c_uint32), ("use_graph", C.c_uint32), ("loglik_every", C.c_uint32),
                ("l2_window", C.c_uint32), ("kernel", C.c_uint32), ("lanes", C.c_uint32), ("unroll", C.c_uint32),
                ("row_order", C.c_uint32), ("pipeline", C.c_uint32), ("kernel_timing", C.c_uint32),
                ("loglik_rel_tol", C.c_double)]


class Stats(C.Structure):
    _fields_ = [("seconds_total", C.c_double), ("seconds_iterations", C.c_double),
                ("iterations", C.c_uint32), ("kernel_launches", C.c_uint32),
                ("bytes_h2d", C.c_uint64), ("bytes_d2h", C.c_uint64), ("loglik_last", C.c_double),
                ("fp_ms", C.c_double), ("bp_ms", C.c_double)]


class Csr4Header(C.Structure):
    _fields_ = [("rows", C.c_uint32), ("cols", C.c_uint32), ("nnz", C.c_uint64),
                ("sym_flags", C.c_uint8), ("nx", C.c_uint32), ("ny", C.c_uint32), ("nz", C.c_uint32)]


class Csr4Scanner(C.Structure):
    _fields_ = [("n_layers", C.c_uint32), ("crystal_w", C.c_float), ("crystal_h", C.c_float),
                ("crystal_d", C.c_float), ("radius", C.c_float), ("mu", C.c_float),
                ("n_blocks", C.c_uint32), ("block_size", C.c_uint32), ("n_rings", C.c_uint32),
                ("block_gap", C.c_float), ("ring_gap", C.c_float), ("voxel_w", C.c_float),
                ("voxel_h", C.c_float), ("voxel_d", C.c_float), ("nx", C.c_uint32), ("ny", C.c_uint32),
                ("nz", C.c_uint32), ("sym_flags", C.c_uint8)]


class Geometry(C.Structure):
    _fields_ = [("det_per_ring", C.c_uint32), ("n_rings", C.c_uint32), ("radius", C.c_float),
                ("ring_pitch", C.c_float), ("nx", C.c_uint32), ("ny", C.c_uint32), ("nz", C.c_uint32),
                ("vx", C.c_float), ("vy", C.c_float), ("vz", C.c_float), ("row_stride", C.c_uint32),
                ("row_phase", C.c_uint32), ("sub_t", C.c_uint32), ("sub_z", C.c_uint32),
                ("width_t", C.c_float), ("width_z", C.c_float)]


class BatchOpts(C.Structure):
    _fields_ = [("tile", C.c_uint32), ("use_graph", C.c_uint32), ("order_by_iterations", C.c_uint32),
                ("form", C.c_uint32)]


class ServerOpts(C.Structure):
    _fields_ = [("slots_per_matrix", C.c_uint32), ("hbm_budget_bytes", C.c_uint64),
                ("hbm_reserve_bytes", C.c_uint64), ("queue_capacity", C.c_uint32),
                ("stream_priority", C.c_uint32)]


class ServerStats(C.Structure):
    _fields_ = [("submitted", C.c_uint64), ("completed", C.c_uint64), ("cancelled", C.c_uint64),
                ("rejected", C.c_uint64), ("active", C.c_uint64), ("queued", C.c_uint64),
                ("hbm_in_use", C.c_uint64), ("iterations_done", C.c_uint64)]


# Every symbol of include/mlem.h with its signature (restype, argtypes).
_P = C.c_void_p
_SIGS = {
    "mlem_last_error": (C.c_char_p, []),
    "mlem_version": (C.c_char_p, []),
    "mlem_kernel_launch_count": (C.c_uint64, []),
    "mlem_matrix_opts_default": (None, [_P]),
    "mlem_matrix_create": (C.c_int, [_P, _P, _P]),
    "mlem_matrix_load_csr4": (C.c_int, [C.c_char_p, _P, _P]),
    "mlem_matrix_destroy": (C.c_int, [_P]),
    "mlem_matrix_get_info": (C.c_int, [_P, _P]),
    "mlem_matrix_get_norm": (C.c_int, [_P, _P]),
    "mlem_matrix_get_tuning": (C.c_int, [_P, C.c_uint32, _P, _P, _P, _P, _P, _P]),
    "mlem_matrix_get_transpose": (C.c_int, [_P, _P, _P, _P]),
    "mlem_matrix_get_csr": (C.c_int, [_P, _P, _P, _P]),
    "mlem_matrix_generate": (C.c_int, [_P, _P, _P]),
    "mlem_run_opts_default": (None, [_P]),
    "mlem_run": (C.c_int, [_P, _P, _P, C.c_uint32, _P, _P, _P, _P]),
    "mlem_run_device": (C.c_int, [_P, _P, _P, C.c_uint32, _P, _P]),
    "mlem_initial_value": (C.c_int, [_P, _P, _P]),
    "mlem_reconstruct": (C.c_int, [_P, _P, _P, _P, _P, _P, _P, _P, _P, _P, C.c_uint32, C.c_uint32,
                                   C.c_uint64, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32,
                                   C.c_uint32, C.c_uint32]),
    "mlem_forward_project": (C.c_int, [_P, _P, _P, _P, _P, _P, _P]),
    "mlem_back_project": (C.c_int, [_P, _P, _P, _P, _P]),
    "mlem_merge_path_search": (C.c_int, [_P, C.c_uint32, C.c_uint64, C.c_uint32, C.c_uint64, _P, _P, _P]),
    "mlem_forward_project_merge_noalloc": (C.c_int, [_P, _P, _P, C.c_uint32, C.c_uint32, C.c_uint64, _P, _P, _P,
                                                     C.c_uint32, _P]),
    "mlem_transpose_host": (C.c_int, [_P, _P, _P, _P]),
    "mlem_column_sums_host": (C.c_int, [_P, _P]),
    "mlem_partition_rows": (C.c_int, [_P, C.c_uint64, C.c_uint32, C.c_uint32, _P, _P, _P, _P]),
    "mlem_csr4_read_header": (C.c_int, [C.c_char_p, _P]),
    "mlem_csr4_read": (C.c_int, [C.c_char_p, _P, _P, _P]),
    "mlem_csr4_write": (C.c_int, [C.c_char_p, _P, _P]),
    "mlem_read_sinogram": (C.c_int, [C.c_char_p, _P, C.c_uint64, _P]),
    "mlem_write_image": (C.c_int, [C.c_char_p, _P, C.c_uint64]),
    "mlem_siddon_rows": (C.c_uint64, [_P]),
    "mlem_siddon_count_host": (C.c_int, [_P, _P]),
    "mlem_siddon_fill_host": (C.c_int, [_P, _P, _P, _P]),
    "mlem_batch_opts_default": (None, [_P]),
    "mlem_batch_run": (C.c_int, [_P, C.c_uint32, _P, _P, _P, _P, _P, _P]),
    "mlem_server_opts_default": (None, [_P]),
    "mlem_server_create": (C.c_int, [_P, _P]),
    "mlem_server_add_matrix": (C.c_int, [_P, _P, _P]),
    "mlem_server_submit": (C.c_int, [_P, C.c_uint32, _P, C.c_uint32, _P]),
    "mlem_server_wait": (C.c_int, [_P, C.c_uint64, _P, C.c_uint32, _P]),
    "mlem_server_cancel": (C.c_int, [_P, C.c_uint64]),
    "mlem_server_get_stats": (C.c_int, [_P, _P]),
    "mlem_server_destroy": (C.c_int, [_P]),
}

_lib = None


def load_library(path: str | Path | None = None) -> C.CDLL:
    """Loads the CUDA library (raises MlemError if it was not built)."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise MlemError(4, f"CUDA library not built: {p} (run build.py)")
    lib = C.CDLL(str(p))
    for name, (res, args) in _SIGS.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib


def _check(st: int) -> None:
    if st != 0:
        raise MlemError(st, load_library().mlem_last_error().decode())


def _ptr(a: np.ndarray | None):
    if a is None:
        return None
    assert a.flags["C_CONTIGUOUS"], "arrays must be C-contiguous"
    return a.ctypes.data


def _arr(a, dtype) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=dtype)


def version() -> str:
    return load_library().mlem_version().decode()


def kernel_launch_count() -> int:
    return int(load_library().mlem_kernel_launch_count())


# ------------------------------------------------------------------ geometry
def geometry(det_per_ring: int, n_rings: int, radius: float, ring_pitch: float, nx: int, ny: int,
             nz: int, vx: float, vy: float, vz: float, row_stride: int = 1, row_phase: int = 0,
             sub_t: int = 1, sub_z: int = 1, width_t: float = 0.0, width_z: float = 0.0) -> Geometry:
    return Geometry(det_per_ring, n_rings, radius, ring_pitch, nx, ny, nz, vx, vy, vz, row_stride, row_phase,
                    sub_t, sub_z, width_t, width_z)


# The synthetic scanners of the benchmark configurations.
PRESETS = {
    # 128 detectors on r = 40 mm, 64x64 voxels of 1 mm: 8,128 rows, 4,096 cols, ~0.5 M nnz
    "ring2d": dict(det_per_ring=128, n_rings=1, radius=40.0, ring_pitch=1.0, nx=64, ny=64, nz=1,
                   vx=1.0, vy=1.0, vz=1.0, sub_t=3, sub_z=1, width_t=0.6, width_z=0.0),
    # 8 rings x 144 detectors on r = 50 mm, 140x140x40 voxels of 0.5 mm:
    # 662,976 rows, 784,000 cols, ~208 M nnz (~313 per row)
    "cyl3d_mid": dict(det_per_ring=144, n_rings=8, radius=50.0, ring_pitch=2.5, nx=140, ny=140, nz=40,
                      vx=0.5, vy=0.5, vz=0.5, sub_t=2, sub_z=2, width_t=1.0, width_z=1.0),
    # 16 rings x 144 detectors on r = 60 mm, 200x200x64 voxels of 0.4 mm:
    # 2,653,056 rows, 2,560,000 cols, ~1.43 B nnz (~540 per row; 11.5 GB in FP32)
    "cyl3d_12gb": dict(det_per_ring=144, n_rings=16, radius=60.0, ring_pitch=1.6, nx=200, ny=200, nz=64,
                       vx=0.4, vy=0.4, vz=0.4, sub_t=3, sub_z=2, width_t=1.0, width_z=0.8),
    # small 2-D ring for unit tests: 32 detectors, 16x16 voxels of 2 mm (496 rows)
    "ring2d_tiny": dict(det_per_ring=32, n_rings=1, radius=24.0, ring_pitch=1.0, nx=16, ny=16, nz=1,
                        vx=2.0, vy=2.0, vz=2.0, sub_t=2, sub_z=1, width_t=1.0, width_z=0.0),
    # small 3-D cylinder for unit tests: 2 rings x 24 detectors, 12x12x4 voxels (1,128 rows)
    "cyl3d_tiny": dict(det_per_ring=24, n_rings=2, radius=20.0, ring_pitch=3.0, nx=12, ny=12, nz=4,
                       vx=2.0, vy=2.0, vz=1.5, sub_t=2, sub_z=2, width_t=1.0, width_z=0.8),
}


def preset(name: str, row_stride: int = 1, row_phase: int = 0, **over) -> Geometry:
    kw = dict(PRESETS[name])
    kw.update(over)
    return geometry(**kw, row_stride=row_stride, row_phase=row_phase)


def siddon_rows(geo: Geometry) -> int:
    """Number of LOR rows the geometry's matrix has (after its row stride)."""
    return int(load_library().mlem_siddon_rows(C.byref(geo)))


def siddon_host(geo: Geometry):
    """Generates the geometry's system matrix on the host (OpenMP).

    Returns (rowptr u64[rows+1], col u32[nnz], val f32[nnz], cols)."""
    lib = load_library()
    rows = int(lib.mlem_siddon_rows(C.byref(geo)))
    if rows == 0:
        _check(1)
    rowptr = np.zeros(rows + 1, np.uint64)
    _check(lib.mlem_siddon_count_host(C.byref(geo), _ptr(rowptr)))
    nnz = int(rowptr[-1])
    col = np.zeros(max(nnz, 1), np.uint32)[:nnz]
    val = np.zeros(max(nnz, 1), np.float32)[:nnz]
    _check(lib.mlem_siddon_fill_host(C.byref(geo), _ptr(rowptr), _ptr(col), _ptr(val)))
    return rowptr, col, val, geo.nx * geo.ny * geo.nz


# -------------------------------------------------------------------- matrix
class Matrix:
    """A system matrix resident on the GPU (A, optionally Aᵀ, sensitivity image)."""

    def __init__(self, handle: int, keep=None):
        self._h = C.c_void_p(handle)
        self._keep = keep
        info = MatrixInfo()
        _check(load_library().mlem_matrix_get_info(self._h, C.byref(info)))
        self.rows, self.cols, self.nnz = info.rows, info.cols, info.nnz
        self.value_type = info.value_type
        self.has_transpose = bool(info.has_transpose)
        self.device_bytes = info.device_bytes
        self.max_row_nnz, self.max_col_nnz = info.max_row_nnz, info.max_col_nnz
        self.symmetry = {"lor_rows": info.sym_lor_rows, "voxel_rows": info.sym_voxel_rows,
                         "fp_nnz": info.sym_fp_nnz, "bp_nnz": info.sym_bp_nnz} if info.sym_lor_rows else None
        self.d16 = {"slots": info.d16_slots, "slots_t": info.d16_slots_t, "lanes": info.d16_lanes,
                    "lanes_t": info.d16_lanes_t} if info.d16_slots else None

    # construction ---------------------------------------------------------
    @staticmethod
    def _opts(value_type=VAL_F32, build_transpose=True, norm=None, device=0, compress=False, interleave=False,
              layout=0, grid=None, symmetry=False):
        o = MatrixOpts()
        load_library().mlem_matrix_opts_default(C.byref(o))
        o.value_type = value_type
        o.build_transpose = 1 if build_transpose else 0
        o.compress_indices = 1 if compress else 0
        o.interleave = 1 if interleave else 0
        o.layout = int(layout)
        o.symmetry = 1 if symmetry else 0
        if grid is not None:
            o.grid_nx, o.grid_ny, o.grid_nz = (int(v) for v in grid)
        keep = None
        if norm is not None:
            keep = _arr(norm, np.float32)
            o.norm = keep.ctypes.data
        o.device = device
        return o, keep

    @classmethod
    def from_csr(cls, rowptr, col, val, cols: int, value_type=VAL_F32, build_transpose=True, norm=None,
                 device=0, compress=False, interleave=False, layout=LAYOUT_NATURAL, grid=None,
                 symmetry=None) -> "Matrix":
        """grid = (nx, ny, nz) of the voxel columns, needed by the locality layout
        and by symmetry.  symmetry = (det_per_ring, rings): the rows are the
        detector pairs of that ring scanner and the matrix is exactly invariant
        under its 16 symmetries (checked; MlemError EINVAL otherwise); the
        compact symmetric operands are built beside the unchanged matrix."""
        rowptr = _arr(rowptr, np.uint64)
        col = _arr(col, np.uint32)
        val = _arr(val, np.float32)
        csr = CsrHost(len(rowptr) - 1, cols, len(col), _ptr(rowptr), _ptr(col), _ptr(val))
        o, keep = cls._opts(value_type, build_transpose, norm, device, compress, interleave, layout, grid,
                            symmetry=symmetry is not None)
        if symmetry is not None:
            o.sym_det_per_ring, o.sym_rings = (int(v) for v in symmetry)
        h = C.c_void_p()
        _check(load_library().mlem_matrix_create(C.byref(csr), C.byref(o), C.byref(h)))
        return cls(h.value)

    @classmethod
    def from_csr4(cls, path, value_type=VAL_F32, build_transpose=True, norm=None, device=0,
                  layout=LAYOUT_NATURAL) -> "Matrix":
        o, keep = cls._opts(value_type, build_transpose, norm, device, layout=layout)
        h = C.c_void_p()
        _check(load_library().mlem_matrix_load_csr4(str(path).encode(), C.byref(o), C.byref(h)))
        return cls(h.value)

    @classmethod
    def generate(cls, geo: Geometry, value_type=VAL_F32, build_transpose=True, device=0,
                 compress=False, interleave=False, layout=LAYOUT_NATURAL, symmetry=False) -> "Matrix":
        o, _ = cls._opts(value_type, build_transpose, None, device, compress, interleave, layout, symmetry=symmetry)
        h = C.c_void_p()
        _check(load_library().mlem_matrix_generate(C.byref(geo), C.byref(o), C.byref(h)))
        return cls(h.value)

    def close(self) -> None:
        if self._h and self._h.value:
            _check(load_library().mlem_matrix_destroy(self._h))
            self._h = C.c_void_p(None)

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    @property
    def handle(self):
        return self._h

    # accessors ------------------------------------------------------------
    def norm(self) -> np.ndarray:
        out = np.zeros(self.cols, np.float32)
        _check(load_library().mlem_matrix_get_norm(self._h, _ptr(out)))
        return out

    def tuning(self, transposed=False) -> dict:
        """The csr-vector configuration the autotuner chose for A or Aᵀ
        (transposed = 2: the form of the fused single pass)."""
        k, ln, u, od, pp, ms = C.c_int(), C.c_int(), C.c_int(), C.c_int(), C.c_int(), C.c_float()
        _check(load_library().mlem_matrix_get_tuning(self._h, int(transposed), C.byref(k), C.byref(ln),
                                                     C.byref(u), C.byref(od), C.byref(pp), C.byref(ms)))
        names = {0: "direct", 1: "tma", 2: "persistent", 4: "d16", 5: "ilv", 7: "sym"}
        if transposed == 2:
            names = {0: "rescan", 1: "staged", 2: "register"}
        return {"kernel": names.get(k.value, k.value), "lanes_per_row": ln.value, "vectors_in_flight": u.value,
                "locality_order": bool(od.value), "pipelined": bool(pp.value), "ms": ms.value}

    def transpose(self):
        cp = np.zeros(self.cols + 1, np.uint64)
        ri = np.zeros(max(self.nnz, 1), np.uint32)
        v = np.zeros(max(self.nnz, 1), np.float32)
        _check(load_library().mlem_matrix_get_transpose(self._h, _ptr(cp), _ptr(ri), _ptr(v)))
        return cp, ri[: self.nnz], v[: self.nnz]

    def csr(self):
        rp = np.zeros(self.rows + 1, np.uint64)
        c = np.zeros(max(self.nnz, 1), np.uint32)
        v = np.zeros(max(self.nnz, 1), np.float32)
        _check(load_library().mlem_matrix_get_csr(self._h, _ptr(rp), _ptr(c), _ptr(v)))
        return rp, c[: self.nnz], v[: self.nnz]

    def initial_value(self, g) -> float:
        g = _arr(g, np.int32)
        out = C.c_float()
        _check(load_library().mlem_initial_value(self._h, _ptr(g), C.byref(out)))
        return out.value

    # runs -------------------------------------------------------------------
    @staticmethod
    def run_opts(spmv=SPMV_CSR_VECTOR, bp_mode=BP_TRANS, secsize_fp=5, secsize_bp=5, use_graph=True,
                 loglik_every=0, l2_window=True, kernel=KERNEL_AUTO, lanes=0, unroll=0,
                 row_order=False, pipeline=False, kernel_timing=False, loglik_rel_tol=0.0) -> RunOpts:
        o = RunOpts()
        load_library().mlem_run_opts_default(C.byref(o))
        o.spmv, o.bp_mode, o.secsize_fp, o.secsize_bp = spmv, bp_mode, secsize_fp, secsize_bp
        o.use_graph, o.loglik_every, o.l2_window = int(use_graph), loglik_every, int(l2_window)
        o.kernel, o.lanes, o.unroll, o.row_order = int(kernel), int(lanes), int(unroll), int(row_order)
        o.pipeline = int(pipeline)
        o.kernel_timing = int(kernel_timing)
        o.loglik_rel_tol = float(loglik_rel_tol)
        return o

    def run(self, g, iterations: int, f0=None, loglik=False, stats=False, **opts):
        """MLEM on host buffers; returns the image (and log-likelihood / stats)."""
        g = _arr(g, np.int32)
        assert g.size >= self.rows
        f0a = None if f0 is None else _arr(f0, np.float32)
        out = np.zeros(self.cols, np.float32)
        if loglik:
            opts.setdefault("loglik_every", 1)
        ro = self.run_opts(**opts)
        ll = np.zeros(iterations, np.float64) if ro.loglik_every else None
        st = Stats()
        _check(load_library().mlem_run(self._h, _ptr(g), _ptr(f0a), iterations, C.byref(ro), _ptr(out),
                                       _ptr(ll), C.byref(st)))
        res = [out]
        if loglik:
            res.append(ll)
        if stats:
            res.append({k: getattr(st, k) for k, _ in Stats._fields_})
        return res[0] if len(res) == 1 else tuple(res)

    def run_device(self, g_dev: int, f_dev: int, iterations: int, stream: int = 0, **opts) -> None:
        """MLEM on device pointers (e.g. torch tensor .data_ptr()); f_dev is updated in place."""
        ro = self.run_opts(**opts)
        _check(load_library().mlem_run_device(self._h, C.c_void_p(g_dev), C.c_void_p(f_dev), iterations,
                                              C.byref(ro), C.c_void_p(stream or None)))

    def forward_project(self, f_dev: int, g_dev: int, ratio_dev: int, fwproj_dev: int = 0, stream: int = 0,
                        **opts) -> None:
        ro = self.run_opts(**opts)
        _check(load_library().mlem_forward_project(self._h, C.c_void_p(f_dev), C.c_void_p(g_dev),
                                                   C.c_void_p(ratio_dev), C.c_void_p(fwproj_dev or None),
                                                   C.byref(ro), C.c_void_p(stream or None)))

    def back_project(self, ratio_dev: int, bp_dev: int, stream: int = 0, **opts) -> None:
        ro = self.run_opts(**opts)
        _check(load_library().mlem_back_project(self._h, C.c_void_p(ratio_dev), C.c_void_p(bp_dev),
                                                C.byref(ro), C.c_void_p(stream or None)))

    def batch_run(self, g, iterations, f0=None, tile=0, use_graph=True, order_by_iterations=True,
                  stats=False, form=0):
        """Reconstructs g[count][rows] with per-instance iteration counts (mlem_batch_run).

        The tile's slots (8/16/32; 0 = autotuned) form a pool that the instances
        enter longest first (order_by_iterations); an image is bit-identical in
        every tile and slot, and to the same sinogram run alone.  form: 0 =
        autotuned, 1 = one CUDA graph per iteration, 2 = persistent (the
        iterations between two refills in one cooperative launch)."""
        g = _arr(g, np.int32)
        count = g.shape[0]
        its = _arr(iterations, np.uint32)
        assert its.size == count
        f0a = None if f0 is None else _arr(f0, np.float32)
        out = np.zeros((count, self.cols), np.float32)
        o = BatchOpts(tile, int(use_graph), int(order_by_iterations), int(form))
        st = Stats()
        _check(load_library().mlem_batch_run(self._h, count, _ptr(g), _ptr(its), _ptr(f0a), C.byref(o),
                                             _ptr(out), C.byref(st)))
        if stats:
            return out, {k: getattr(st, k) for k, _ in Stats._fields_}
        return out


# ----------------------------------------------------- reference-shaped calls
def mlem(csr_rows, csr_cols, csr_vals, csr_rows_trans, csr_cols_trans, csr_vals_trans, g, norm, f,
         result_f, rows, cols, nnzs, iterations, device_numbers, matrix_vector_mul, secsize_fp, secsize_bp,
         using_trans) -> None:
    """The reference mlem() (main.cu:19, 167-514) on the GPU.

    Same arguments: host CSR of A (u64 row pointers), host CSR of Aᵀ (used when
    using_trans == 0; None = built on the GPU), sinogram g, sensitivity norm,
    initial image f; the image is written into result_f.  The caller's arrays
    are not modified."""
    lib = load_library()
    a = [_arr(csr_rows, np.uint64), _arr(csr_cols, np.uint32), _arr(csr_vals, np.float32)]
    t = [None, None, None]
    if csr_rows_trans is not None:
        t = [_arr(csr_rows_trans, np.uint64), _arr(csr_cols_trans, np.uint32), _arr(csr_vals_trans, np.float32)]
    g = _arr(g, np.int32)
    norm = _arr(norm, np.float32)
    f = _arr(f, np.float32)
    assert isinstance(result_f, np.ndarray) and result_f.dtype == np.float32 and result_f.flags["C_CONTIGUOUS"]
    _check(lib.mlem_reconstruct(_ptr(a[0]), _ptr(a[1]), _ptr(a[2]), _ptr(t[0]), _ptr(t[1]), _ptr(t[2]),
                                _ptr(g), _ptr(norm), _ptr(f), _ptr(result_f), rows, cols, nnzs, iterations,
                                device_numbers, matrix_vector_mul, secsize_fp, secsize_bp, using_trans))


def merge_path_search(rowptr_dev: int, rows: int, nnz: int, secsize: int, nthreads: int, i_dev: int,
                      j_dev: int, stream: int = 0) -> None:
    _check(load_library().mlem_merge_path_search(C.c_void_p(rowptr_dev), rows, nnz, secsize, nthreads,
                                                 C.c_void_p(i_dev), C.c_void_p(j_dev), C.c_void_p(stream or None)))


def transpose(rowptr, col, val, cols: int):
    """GPU stable counting-sort transpose (host in/out)."""
    rowptr, col, val = _arr(rowptr, np.uint64), _arr(col, np.uint32), _arr(val, np.float32)
    nnz = len(col)
    csr = CsrHost(len(rowptr) - 1, cols, nnz, _ptr(rowptr), _ptr(col), _ptr(val))
    cp = np.zeros(cols + 1, np.uint64)
    ri = np.zeros(max(nnz, 1), np.uint32)
    v = np.zeros(max(nnz, 1), np.float32)
    _check(load_library().mlem_transpose_host(C.byref(csr), _ptr(cp), _ptr(ri), _ptr(v)))
    return cp, ri[:nnz], v[:nnz]


def column_sums(rowptr, col, val, cols: int) -> np.ndarray:
    rowptr, col, val = _arr(rowptr, np.uint64), _arr(col, np.uint32), _arr(val, np.float32)
    csr = CsrHost(len(rowptr) - 1, cols, len(col), _ptr(rowptr), _ptr(col), _ptr(val))
    out = np.zeros(cols, np.float32)
    _check(load_library().mlem_column_sums_host(C.byref(csr), _ptr(out)))
    return out


def partition_rows(rowptr, nnz: int, rows: int, nseg: int):
    """partitionMatrix (main.cu:593-611)."""
    rowptr = _arr(rowptr, np.uint64)
    seg = np.zeros(nseg + 1, np.uint32)
    sr = np.zeros(nseg, np.uint32)
    sn = np.zeros(nseg, np.uint32)
    off = np.zeros(nseg, np.uint64)
    _check(load_library().mlem_partition_rows(_ptr(rowptr), nnz, rows, nseg, _ptr(seg), _ptr(sr), _ptr(sn),
                                              _ptr(off)))
    return seg, sr, sn, off


# --------------------------------------------------------------------- files
def csr4_write(path, rowptr, col, val, cols: int, geo: Geometry | None = None, n_rings: int = 1,
               sym_flags: int = 0) -> None:
    rowptr, col, val = _arr(rowptr, np.uint64), _arr(col, np.uint32), _arr(val, np.float32)
    sc = Csr4Scanner()
    sc.n_layers, sc.n_blocks, sc.block_size = 1, 1, 1
    sc.crystal_w = sc.crystal_h = sc.crystal_d = 1.0
    sc.n_rings = geo.n_rings if geo else n_rings
    if geo:
        sc.radius, sc.ring_gap = geo.radius, geo.ring_pitch
        sc.voxel_w, sc.voxel_h, sc.voxel_d = geo.vx, geo.vy, geo.vz
        sc.nx, sc.ny, sc.nz = geo.nx, geo.ny, geo.nz
    else:
        sc.nx, sc.ny, sc.nz = cols, 1, 1
        sc.voxel_w = sc.voxel_h = sc.voxel_d = 1.0
    sc.sym_flags = sym_flags
    csr = CsrHost(len(rowptr) - 1, cols, len(col), _ptr(rowptr), _ptr(col), _ptr(val))
    _check(load_library().mlem_csr4_write(str(path).encode(), C.byref(sc), C.byref(csr)))


def csr4_read(path):
    lib = load_library()
    h = Csr4Header()
    _check(lib.mlem_csr4_read_header(str(path).encode(), C.byref(h)))
    rp = np.zeros(h.rows + 1, np.uint64)
    c = np.zeros(max(h.nnz, 1), np.uint32)
    v = np.zeros(max(h.nnz, 1), np.float32)
    _check(lib.mlem_csr4_read(str(path).encode(), _ptr(rp), _ptr(c), _ptr(v)))
    return rp, c[: h.nnz], v[: h.nnz], h


def read_sinogram(path) -> np.ndarray:
    lib = load_library()
    n = C.c_uint64()
    _check(lib.mlem_read_sinogram(str(path).encode(), None, 0, C.byref(n)))
    g = np.zeros(max(n.value, 1), np.int32)
    _check(lib.mlem_read_sinogram(str(path).encode(), _ptr(g), n.value, C.byref(n)))
    return g[: n.value]


def write_image(path, f) -> None:
    f = _arr(f, np.float32)
    _check(load_library().mlem_write_image(str(path).encode(), _ptr(f), f.size))


# -------------------------------------------------------------------- server
class Server:
    """Continuous-batching reconstruction server over resident matrices (mlem_server_*).

    stream_priority: 0 = three levels by matrix size, 1 (default) = small
    matrices (< 16 M nonzeros) first and the others equal, 2 = all equal."""

    def __init__(self, slots_per_matrix=0, hbm_budget_bytes=0, hbm_reserve_bytes=2 << 30,
                 queue_capacity=4096, stream_priority=1):
        lib = load_library()
        o = ServerOpts(slots_per_matrix, hbm_budget_bytes, hbm_reserve_bytes, queue_capacity, stream_priority)
        h = C.c_void_p()
        _check(lib.mlem_server_create(C.byref(o), C.byref(h)))
        self._h = h
        self._mats = []
        self._req_cols = {}

    def add_matrix(self, m: Matrix) -> int:
        mid = C.c_uint32()
        _check(load_library().mlem_server_add_matrix(self._h, m.handle, C.byref(mid)))
        self._mats.append(m)
        return mid.value

    def submit(self, matrix_id: int, g, iterations: int) -> int:
        g = _arr(g, np.int32)
        rid = C.c_uint64()
        _check(load_library().mlem_server_submit(self._h, matrix_id, _ptr(g), iterations, C.byref(rid)))
        self._req_cols[rid.value] = self._mats[matrix_id].cols
        return rid.value

    def wait(self, request_id: int, timeout_ms: int = 600000):
        """Blocks until the request finishes; returns (image, latency seconds)."""
        lat = C.c_double()
        out = np.zeros(self._req_cols[request_id], np.float32)
        _check(load_library().mlem_server_wait(self._h, request_id, _ptr(out), timeout_ms, C.byref(lat)))
        del self._req_cols[request_id]
        return out, lat.value

    def cancel(self, request_id: int) -> None:
        _check(load_library().mlem_server_cancel(self._h, request_id))

    def stats(self) -> dict:
        st = ServerStats()
        _check(load_library().mlem_server_get_stats(self._h, C.byref(st)))
        return {k: getattr(st, k) for k, _ in ServerStats._fields_}

    def close(self) -> None:
        if self._h and self._h.value:
            _check(load_library().mlem_server_destroy(self._h))
            self._h = C.c_void_p(None)

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
