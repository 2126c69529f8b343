"""Host-side logic of the library (CPU only; no CUDA call is made)."""
from __future__ import annotations

import ctypes as C
import re
import subprocess
from pathlib import Path

import numpy as np
import pytest

from conftest import ROOT, golden_csr


def header_functions():
    txt = (ROOT / "include" / "mlem.h").read_text()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(mlem_[a-z0-9_]+)\s*\(", txt)))


def test_library_exports_every_declared_symbol(pkg):
    lib = pkg.load_library()
    names = header_functions()
    assert len(names) >= 40
    nm = subprocess.run(["nm", "-D", "--defined-only", str(pkg.LIB_PATH)], capture_output=True, text=True).stdout
    exported = set(re.findall(r" T (mlem_\w+)", nm))
    missing = [n for n in names if n not in exported]
    assert not missing, missing
    for n in names:
        assert hasattr(lib, n)
    assert set(pkg._SIGS) == set(names)  # the Python binding covers the whole ABI


def test_version_and_error_text(pkg):
    assert "sm_103a" in pkg.version()
    with pytest.raises(pkg.MlemError) as e:
        pkg.siddon_host(pkg.geometry(0, 1, 1, 1, 1, 1, 1, 1, 1, 1))
    assert e.value.status == "EINVAL"
    assert "detector" in str(e.value)


# ----------------------------------------------------------------- csr4 files
def test_csr4_writer_is_byte_identical_to_fixture(pkg, golden, tmp_path):
    rp, c, v, cols = golden_csr(golden, "cyl3d_tiny")
    p = tmp_path / "m.csr4"
    pkg.csr4_write(p, rp, c, v, cols, geo=pkg.preset("cyl3d_tiny"))
    assert np.array_equal(np.frombuffer(p.read_bytes(), np.uint8), golden["csr4/file"])


def test_csr4_reader_matches_reference_reader(pkg, golden, tmp_path):
    p = tmp_path / "m.csr4"
    p.write_bytes(golden["csr4/file"].tobytes())
    rp, c, v, h = pkg.csr4_read(p)
    rows, cols, nnz = golden["csr4/ref_dims"]
    assert (h.rows, h.cols, h.nnz) == (rows, cols, nnz)
    assert np.array_equal(rp, golden["csr4/ref_rowptr"])
    assert np.array_equal(c, golden["csr4/ref_col"])
    assert np.array_equal(v.view(np.uint32), golden["csr4/ref_val"].view(np.uint32))
    assert (h.nx, h.ny, h.nz) == (12, 12, 4)


def _corrupt(data: bytes, off: int, payload: bytes) -> bytes:
    b = bytearray(data)
    b[off:off + len(payload)] = payload
    return bytes(b)


@pytest.mark.parametrize("case", ["magic", "version", "short", "scanbytes", "rowidx", "column", "tiny"])
def test_csr4_rejects_malformed_files(pkg, golden, tmp_path, case):
    data = golden["csr4/file"].tobytes()
    scan = int(np.frombuffer(data[24:28], np.uint32)[0])
    rows = int(np.frombuffer(data[8:12], np.uint32)[0])
    if case == "magic":
        data = _corrupt(data, 0, b"XCSR")
    elif case == "version":
        data = _corrupt(data, 4, bytes([3]))
    elif case == "short":
        data = data[:-9]
    elif case == "scanbytes":
        data = _corrupt(data, 24, np.uint32(scan + 4).tobytes())
    elif case == "rowidx":
        off = 28 + scan + 8 * (rows // 2)
        data = _corrupt(data, off, np.uint64(1).tobytes())
    elif case == "column":
        off = 28 + scan + 8 * rows
        data = _corrupt(data, off, np.uint32(10 ** 6).tobytes())
    elif case == "tiny":
        data = data[:20]
    p = tmp_path / "bad.csr4"
    p.write_bytes(data)
    with pytest.raises(pkg.MlemError) as e:
        pkg.csr4_read(p)
    assert e.value.status == "EIO"


def test_raw_vectors(pkg, tmp_path):
    g = np.arange(-5, 100, dtype=np.int32)
    p = tmp_path / "g.raw"
    g.tofile(p)
    assert np.array_equal(pkg.read_sinogram(p), g)
    (tmp_path / "odd.raw").write_bytes(b"\x01\x02\x03")
    with pytest.raises(pkg.MlemError) as e:
        pkg.read_sinogram(tmp_path / "odd.raw")
    assert e.value.status == "EIO"
    with pytest.raises(pkg.MlemError):
        pkg.read_sinogram(tmp_path / "missing.raw")
    f = np.linspace(0, 1, 33, dtype=np.float32)
    pkg.write_image(tmp_path / "f.raw", f)
    assert np.array_equal(np.fromfile(tmp_path / "f.raw", np.float32), f)


# ------------------------------------------------------------------ generator
@pytest.mark.parametrize("name", ["ring2d_tiny", "cyl3d_tiny", "ring2d"])
def test_generator_structure(pkg, name):
    geo = pkg.preset(name)
    rp, c, v, cols = pkg.siddon_host(geo)
    D = geo.det_per_ring * geo.n_rings
    assert len(rp) - 1 == D * (D - 1) // 2 == pkg.load_library().mlem_siddon_rows(C.byref(geo))
    lens = np.diff(rp.astype(np.int64))
    rid = np.repeat(np.arange(len(lens)), lens)
    same = rid[1:] == rid[:-1]
    assert np.all(np.diff(c.astype(np.int64))[same] > 0)  # strictly ascending within a row
    assert np.all(c < cols) and np.all(v > 0)
    diag = np.sqrt((geo.nx * geo.vx) ** 2 + (geo.ny * geo.vy) ** 2 + (geo.nz * geo.vz) ** 2)
    assert np.all(v <= np.sqrt(geo.vx ** 2 + geo.vy ** 2 + geo.vz ** 2) + 1e-5)
    # a row's total length is the mean chord of its sub-rays through the grid
    assert np.all(np.add.reduceat(v.astype(np.float64), rp[:-1][lens > 0].astype(np.int64)) <= diag + 1e-3)


def test_generator_row_sampling(pkg):
    full = pkg.siddon_host(pkg.preset("cyl3d_tiny"))
    for stride, phase in ((3, 0), (7, 5)):
        part = pkg.siddon_host(pkg.preset("cyl3d_tiny", row_stride=stride, row_phase=phase))
        rows = np.arange(phase, len(full[0]) - 1, stride)
        assert len(part[0]) - 1 == len(rows)
        for q, r in enumerate(rows[::17]):
            q *= 17
            a0, a1 = int(full[0][r]), int(full[0][r + 1])
            b0, b1 = int(part[0][q]), int(part[0][q + 1])
            assert np.array_equal(full[1][a0:a1], part[1][b0:b1])
            assert np.array_equal(full[2][a0:a1], part[2][b0:b1])


def test_generator_is_deterministic(pkg):
    a = pkg.siddon_host(pkg.preset("ring2d"))
    b = pkg.siddon_host(pkg.preset("ring2d"))
    for x, y in zip(a[:3], b[:3]):
        assert np.array_equal(x, y)


# ------------------------------------------------------------------ partition
def _partition_restated(rowptr, nnz, rows, nseg):
    seg = [0] * (nseg + 1)
    seg[nseg] = rows
    i = 0
    per = nnz / nseg
    for s in range(nseg):
        while i <= rows and not (float(rowptr[i]) >= per * s):
            i += 1
        seg[s] = i
    return seg


@pytest.mark.parametrize("nseg", [1, 2, 3, 8])
def test_partition_rows(pkg, golden, nseg):
    rp, c, v, cols = golden_csr(golden, "ring2d_tiny")
    rows, nnz = len(rp) - 1, len(c)
    seg, sr, sn, off = pkg.partition_rows(rp, nnz, rows, nseg)
    assert list(seg) == _partition_restated(rp, nnz, rows, nseg)
    assert seg[0] == 0 and seg[-1] == rows
    assert int(sn.sum()) == nnz and int(sr.sum()) == rows
    assert np.array_equal(off, rp[seg[:-1]])


# ------------------------------------------------------------------------ CLI
@pytest.mark.parametrize("argv", [[], ["a", "b", "1", "1", "5", "5", "0"], ["a", "b", "0", "1", "5", "5", "0", "1"],
                                  ["a", "b", "3", "1", "5", "5", "2", "1"], ["a", "b", "3", "1", "0", "5", "0", "1"],
                                  ["a", "b", "3", "1", "5", "5", "0", "7"]])
def test_cli_rejects_bad_arguments(pkg, argv):
    r = subprocess.run([str(pkg.CLI_PATH)] + argv, capture_output=True, text=True, timeout=60)
    assert r.returncode == 1
    assert "Wrong parameters!" in r.stdout and "argv[8]" in r.stdout


def test_cli_reports_missing_files(pkg, tmp_path):
    r = subprocess.run([str(pkg.CLI_PATH), str(tmp_path / "nope.csr4"), str(tmp_path / "g"), "3", "1", "5", "5",
                        "0", "1"], capture_output=True, text=True, timeout=60)
    assert r.returncode == 1 and "Cannot open file" in r.stderr
