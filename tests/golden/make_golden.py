"""Generates tests/golden/*.npz from the reference's own code run here.

The reference (wmd0701/Bachelorarbeit-MLEM) has no tests or fixtures, so the
pins are made by compiling its sources in this container (oracle/ref_build.py)
and recording what they compute on small inputs:

* sptrans_scanTrans_specialized (sptrans.h:397-545) transposes, run with 1, 3
  and 8 OpenMP threads (all must agree);
* the kernels of kernel.cu (csr-vector, merge-based for several section sizes,
  the atomic scatter), run on the CPU through the CUDA emulation shim;
* the single-device mlem() loop (main.cu:329-449) around those kernels for
  every combination of the two switches and two section-size pairs;
* the csr4 reader (csr4matrix.cpp) on a file written by this library.

Inputs are seeded (numpy PCG64) or produced by the library's host Siddon
generator; every input array is stored with its outputs, so the tests never
need the reference.  Run:  python tests/golden/make_golden.py
"""
from __future__ import annotations

import ctypes as C
import importlib.util
import sys
import tempfile
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from oracle import oracle as O  # noqa: E402


def load_pkg():
    spec = importlib.util.spec_from_file_location(
        "mlem_gb300", ROOT / "bachelorarbeit-mlem_gb300" / "__init__.py",
        submodule_search_locations=[str(ROOT / "bachelorarbeit-mlem_gb300")])
    m = importlib.util.module_from_spec(spec)
    sys.modules["mlem_gb300"] = m
    spec.loader.exec_module(m)
    return m


def random_csr(rng, rows, cols, mean_len, empty_frac=0.2, dup=False, long_rows=0):
    lens = rng.poisson(mean_len, rows).astype(np.int64)
    lens[rng.random(rows) < empty_frac] = 0
    for r in rng.choice(rows, size=min(long_rows, rows), replace=False):
        lens[r] = rng.integers(cols // 2, cols) if not dup else rng.integers(cols, 2 * cols)
    rowptr = np.zeros(rows + 1, np.uint64)
    rowptr[1:] = np.cumsum(lens)
    cl, vl = [], []
    for r in range(rows):
        n = int(lens[r])
        if dup:
            c = np.sort(rng.integers(0, cols, n))
        else:
            n = min(n, cols)
            c = np.sort(rng.choice(cols, size=n, replace=False))
            lens[r] = n
        cl.append(c)
        vl.append(rng.uniform(0.01, 2.0, len(c)))
    rowptr[1:] = np.cumsum(lens)
    col = np.concatenate(cl).astype(np.uint32) if cl else np.zeros(0, np.uint32)
    val = np.concatenate(vl).astype(np.float32) if vl else np.zeros(0, np.float32)
    return rowptr, col, val


def ref_transpose(ref, rowptr, col, val, cols, threads):
    rows = len(rowptr) - 1
    nnz = len(col)
    cp = np.zeros(cols + 1, np.uint64)
    rt = np.zeros(max(nnz, 1), np.uint32)
    vt = np.zeros(max(nnz, 1), np.float32)
    ref.ref_sptrans(threads, rows, cols, nnz, O.P(rowptr), O.P(col), O.P(val), O.P(rt), O.P(cp), O.P(vt))
    return cp, rt[:nnz], vt[:nnz]


def ref_spmv(ref, spmv, scatter, secsize, rowptr, col, val, x, out_len):
    y = np.zeros(out_len, np.float32)
    ref.ref_spmv(spmv, scatter, secsize, O.P(rowptr), O.P(col), O.P(val), O.P(O.f32(x)), len(rowptr) - 1,
                 len(col), O.P(y))
    return y


def ref_mlem(ref, A, AT, g, norm, f0, iters, spmv, ss_fp, ss_bp, using_trans):
    f = O.f32(f0).copy()
    rpt, ct, vt = (None, None, None) if AT is None else AT
    ref.ref_mlem(O.P(A[0]), O.P(A[1]), O.P(A[2]), O.P(rpt), O.P(ct), O.P(vt), O.P(O.i32(g)), O.P(O.f32(norm)),
                 O.P(f), len(A[0]) - 1, len(norm), len(A[1]), iters, spmv, ss_fp, ss_bp, using_trans)
    return f


def main():
    ref = O.ref()
    if ref is None:
        raise SystemExit("reference checkout not found; fixtures can only be made where it exists")
    pkg = load_pkg()
    rng = np.random.Generator(np.random.PCG64(20241203))
    out = {}
    cases = {}
    # Siddon matrices from the library's host generator
    for name, n_shapes, total in (("ring2d_tiny", 3, 2e4), ("cyl3d_tiny", 4, 5e4)):
        geo = pkg.preset(name)
        rp, c, v, cols = pkg.siddon_host(geo)
        cases[name] = (rp, c, v, cols)
    # seeded random CSRs with the edge cases the reference code meets
    cases["rand_small"] = (*random_csr(rng, 37, 23, 5.0), 23)
    cases["rand_long"] = (*random_csr(rng, 60, 3000, 30.0, long_rows=3), 3000)
    cases["rand_dup"] = (*random_csr(rng, 25, 11, 6.0, dup=True), 11)
    cases["one_row"] = (*random_csr(rng, 1, 5000, 4000.0, empty_frac=0.0), 5000)
    cases["empty_rows"] = (*random_csr(rng, 300, 50, 2.0, empty_frac=0.9), 50)
    cases["tall"] = (*random_csr(rng, 4000, 7, 1.0, empty_frac=0.3), 7)

    for name, (rp, c, v, cols) in cases.items():
        rp, c, v = O.c64(rp), O.c32(c), O.f32(v)
        out[f"{name}/rowptr"] = rp
        out[f"{name}/col"] = c
        out[f"{name}/val"] = v
        out[f"{name}/cols"] = np.array(cols, np.int64)
        ts = [ref_transpose(ref, rp, c, v, cols, t) for t in (1, 3, 8)]
        for t in ts[1:]:
            assert all(np.array_equal(a, b) for a, b in zip(ts[0], t)), f"{name}: sptrans thread dependence"
        out[f"{name}/T_colptr"], out[f"{name}/T_row"], out[f"{name}/T_val"] = ts[0]
        x = rng.uniform(0.1, 3.0, cols).astype(np.float32)
        r = rng.uniform(0.0, 2.0, len(rp) - 1).astype(np.float32)
        out[f"{name}/x"] = x
        out[f"{name}/r"] = r
        out[f"{name}/y_csrvec"] = ref_spmv(ref, 1, 0, 1, rp, c, v, x, len(rp) - 1)
        for ss in (1, 2, 5, 9):
            out[f"{name}/y_merge{ss}"] = ref_spmv(ref, 0, 0, ss, rp, c, v, x, len(rp) - 1)
        out[f"{name}/y_scatter"] = ref_spmv(ref, 0, 1, 1, rp, c, v, r, cols)

    # MLEM loops on the Siddon matrices with a Poisson sinogram
    import importlib
    synth = importlib.import_module("mlem_gb300.synth")
    for name, n_shapes, total in (("ring2d_tiny", 3, 2e4), ("cyl3d_tiny", 4, 5e4)):
        rp, c, v, cols = cases[name]
        geo = pkg.preset(name)
        xt = synth.phantom(geo, n_shapes, seed=1)
        g = synth.poisson_sinogram(synth.project_host(rp, c, v, xt), total, seed=2)
        norm = O.colsum(rp, c, v, cols, f64=False)
        f0 = np.full(cols, O.initial_value(g, norm), np.float32)
        out[f"{name}/g"] = g
        out[f"{name}/norm"] = norm
        out[f"{name}/f0"] = f0
        AT = (out[f"{name}/T_colptr"], out[f"{name}/T_row"], out[f"{name}/T_val"])
        A = (O.c64(rp), O.c32(c), O.f32(v))
        for spmv in (0, 1):
            for ut in (0, 1):
                for ss in ((5, 5), (3, 9)):
                    if spmv == 1 and ss != (5, 5):
                        continue
                    for iters in (1, 4, 12):
                        key = f"{name}/mlem_s{spmv}_t{ut}_ss{ss[0]}x{ss[1]}_it{iters}"
                        out[key] = ref_mlem(ref, A, AT if ut == 0 else None, g, norm, f0, iters, spmv, ss[0],
                                            ss[1], ut)

    # csr4: file written by this library, parsed by the reference reader
    with tempfile.TemporaryDirectory() as td:
        rp, c, v, cols = cases["cyl3d_tiny"]
        path = Path(td) / "m.csr4"
        pkg.csr4_write(path, rp, c, v, cols, geo=pkg.preset("cyl3d_tiny"))
        rows_ = C.c_uint32()
        cols_ = C.c_uint32()
        nnz_ = C.c_uint64()
        assert ref.ref_csr4_header(str(path).encode(), C.byref(rows_), C.byref(cols_), C.byref(nnz_)) == 0
        rrp = np.zeros(rows_.value + 1, np.uint64)
        rc = np.zeros(nnz_.value, np.uint32)
        rv = np.zeros(nnz_.value, np.float32)
        assert ref.ref_csr4_read(str(path).encode(), O.P(rrp), O.P(rc), O.P(rv)) == 0
        out["csr4/file"] = np.frombuffer(path.read_bytes(), np.uint8)
        out["csr4/ref_rowptr"], out["csr4/ref_col"], out["csr4/ref_val"] = rrp, rc, rv
        out["csr4/ref_dims"] = np.array([rows_.value, cols_.value, nnz_.value], np.int64)

    dst = Path(__file__).resolve().parent / "reference_outputs.npz"
    np.savez_compressed(dst, **out)
    print(dst, dst.stat().st_size, "bytes,", len(out), "arrays")


if __name__ == "__main__":
    main()
