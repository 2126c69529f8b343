"""Batched form, serving loop, CLI drop-in (GPU, through the C ABI)."""
from __future__ import annotations

import os
import subprocess
import time

import numpy as np
import pytest

from conftest import problem

pytestmark = pytest.mark.gpu


def sinograms(pkg, p, count, seed=10):
    from mlem_gb300 import synth
    rng = np.random.Generator(np.random.PCG64(seed))
    out = []
    for k in range(count):
        xt = synth.phantom(p["geo"], 4, seed=seed + 100 + k)
        total = float(np.exp(rng.uniform(np.log(1e4), np.log(1e7))))
        out.append(synth.poisson_sinogram(synth.project_host(p["rp"], p["col"], p["val"], xt), total, seed + 200 + k))
    return np.stack(out)


@pytest.mark.parametrize("tile", [8, 16, 32, 0])
def test_batch_matches_single_runs(pkg, O, tile):
    p = problem(pkg, O, "ring2d")
    m = pkg.Matrix.from_csr(p["rp"], p["col"], p["val"], p["cols"])
    G = sinograms(pkg, p, 11)
    its = np.random.Generator(np.random.PCG64(5)).integers(1, 25, len(G)).astype(np.uint32)
    out = m.batch_run(G, its, tile=tile)
    for k in range(len(G)):
        single = m.run(G[k], int(its[k]))
        assert O.rel_l2(out[k], single) < 1e-5, k
        ref64 = O.mlem_f64((p["rp"], p["col"], p["val"]), G[k], m.norm(), np.full(p["cols"], m.initial_value(G[k])),
                           int(its[k]))
        assert O.rel_l2(out[k], ref64) < 1e-5, k
    m.close()


def test_batch_without_transpose_and_fp16(pkg, O):
    p = problem(pkg, O, "cyl3d_tiny")
    G = sinograms(pkg, p, 5)
    its = np.array([3, 9, 1, 20, 7], np.uint32)
    A = (p["rp"], p["col"], p["val"])
    m_scatter = pkg.Matrix.from_csr(*A, p["cols"], build_transpose=False)
    m_half = pkg.Matrix.from_csr(*A, p["cols"], value_type=pkg.VAL_F16)
    o1 = m_scatter.batch_run(G, its, tile=8)
    o2 = m_half.batch_run(G, its, tile=16)
    for k in range(len(G)):
        ref64 = O.mlem_f64(A, G[k], O.colsum(*A, p["cols"]), np.full(p["cols"], m_scatter.initial_value(G[k])),
                           int(its[k]))
        assert O.rel_l2(o1[k], ref64) < 1e-5
        assert O.rel_l2(o2[k], ref64) < 1e-3
    m_scatter.close()
    m_half.close()


def test_batch_bits_independent_of_tile_and_width(pkg, O):
    """Each instance sums its rows in the same order in every tile (8/16/32)
    and at every projection width, so the images agree bit for bit, also
    while a tile empties (uneven iteration counts)."""
    p = problem(pkg, O, "cyl3d_tiny")
    m = pkg.Matrix.from_csr(p["rp"], p["col"], p["val"], p["cols"], value_type=pkg.VAL_F16)
    G = sinograms(pkg, p, 11)
    its = np.random.Generator(np.random.PCG64(9)).integers(1, 30, len(G)).astype(np.uint32)
    its[2] = 0  # a zero-iteration instance returns its initial image
    outs = [m.batch_run(G, its, tile=t) for t in (8, 16, 32)]
    assert np.array_equal(outs[0], outs[1]) and np.array_equal(outs[0], outs[2])
    assert np.array_equal(outs[0][2], np.full(m.cols, m.initial_value(G[2]), np.float32))
    unordered = m.batch_run(G, its, tile=16, order_by_iterations=False)
    assert np.array_equal(unordered, outs[0])
    for k in (0, 5, 10):
        assert np.array_equal(m.batch_run(G[k:k + 1], its[k:k + 1], tile=32)[0], outs[0][k])
    m.close()


@pytest.mark.parametrize("vt", ["f32", "f16"])
def test_batch_persistent_form_is_bit_identical(pkg, O, vt):
    """The persistent form (the iterations between two refills in one
    cooperative launch, grid barriers between the projections) gives the
    bits of the per-iteration graphs, in every tile and with uneven counts
    (widths shrink as the pool empties); the autotuned form is one of them."""
    p = problem(pkg, O, "cyl3d_tiny")
    m = pkg.Matrix.from_csr(p["rp"], p["col"], p["val"], p["cols"],
                            value_type=pkg.VAL_F32 if vt == "f32" else pkg.VAL_F16)
    G = sinograms(pkg, p, 21)
    its = np.random.Generator(np.random.PCG64(4)).integers(1, 40, len(G)).astype(np.uint32)
    its[3] = 0
    for tile in (8, 16, 32):
        graphs = m.batch_run(G, its, tile=tile, form=1)
        loop = m.batch_run(G, its, tile=tile, form=2)
        assert np.array_equal(graphs, loop), tile
    auto = m.batch_run(G, its, tile=16)
    assert np.array_equal(auto, graphs)
    for k in (0, 7):
        single = m.run(G[k], int(its[k]))
        assert O.rel_l2(loop[k], single) < 1e-5
    m.close()


def test_batch_persistent_form_needs_the_transpose(pkg, O):
    p = problem(pkg, O, "ring2d_tiny")
    m = pkg.Matrix.from_csr(p["rp"], p["col"], p["val"], p["cols"], build_transpose=False)
    with pytest.raises(pkg.MlemError) as e:
        m.batch_run(p["g"][None, :], np.array([3], np.uint32), form=2)
    assert e.value.status == "EINVAL"
    out = m.batch_run(p["g"][None, :], np.array([3], np.uint32))  # autotuned: the graph form
    assert O.rel_l2(out[0], m.run(p["g"], 3, bp_mode=pkg.BP_SCATTER)) < 1e-5
    m.close()


def test_batch_instance_independent_of_company(pkg, O):
    p = problem(pkg, O, "ring2d")
    m = pkg.Matrix.from_csr(p["rp"], p["col"], p["val"], p["cols"])
    G = sinograms(pkg, p, 9)
    its = np.full(len(G), 12, np.uint32)
    full = m.batch_run(G, its, tile=16)
    for k in (0, 4, 8):
        alone = m.batch_run(G[k:k + 1], its[k:k + 1], tile=16)
        assert np.array_equal(alone[0], full[k])
    m.close()


@pytest.mark.parametrize("slots,priority", [(8, 0), (32, 2)])
def test_server_same_alone_and_in_mix(pkg, O, slots, priority):
    pa = problem(pkg, O, "ring2d")
    pb = problem(pkg, O, "cyl3d_tiny")
    ma = pkg.Matrix.from_csr(pa["rp"], pa["col"], pa["val"], pa["cols"])
    mb = pkg.Matrix.from_csr(pb["rp"], pb["col"], pb["val"], pb["cols"], value_type=pkg.VAL_F16)
    Ga, Gb = sinograms(pkg, pa, 20, seed=1), sinograms(pkg, pb, 12, seed=2)
    with pytest.raises(pkg.MlemError):
        pkg.Server(stream_priority=3)
    with pkg.Server(slots_per_matrix=slots, stream_priority=priority) as srv:
        ia, ib = srv.add_matrix(ma), srv.add_matrix(mb)
        alone_a, _ = srv.wait(srv.submit(ia, Ga[0], 15))
        alone_b, _ = srv.wait(srv.submit(ib, Gb[0], 9))
        ids = []
        rng = np.random.Generator(np.random.PCG64(3))
        for k in range(20):
            ids.append(("a", k, srv.submit(ia, Ga[k], 15 if k == 0 else int(rng.integers(5, 30)))))
            if k < 12:
                ids.append(("b", k, srv.submit(ib, Gb[k], 9 if k == 0 else int(rng.integers(3, 20)))))
        res = {}
        lat = []
        for which, k, rid in ids:
            img, l = srv.wait(rid)
            res[(which, k)] = img
            lat.append(l)
        st = srv.stats()
        assert st["completed"] == 2 + len(ids)
        assert st["active"] == 0 and st["queued"] == 0
    assert np.array_equal(res[("a", 0)], alone_a)
    assert np.array_equal(res[("b", 0)], alone_b)
    # the batched arithmetic does not depend on the tile: the same bits as batch_run
    assert np.array_equal(alone_a, ma.batch_run(Ga[:1], np.array([15], np.uint32), tile=16)[0])
    single = ma.run(Ga[0], 15)
    assert O.rel_l2(alone_a, single) < 1e-5
    ma.close()
    mb.close()


def test_server_cancel_and_admission(pkg, O):
    p = problem(pkg, O, "ring2d")
    m = pkg.Matrix.from_csr(p["rp"], p["col"], p["val"], p["cols"])
    G = sinograms(pkg, p, 3)
    # a budget too small for any slot state: requests stay queued, cancel works
    with pkg.Server(slots_per_matrix=8, hbm_budget_bytes=1024) as srv:
        mid = srv.add_matrix(m)
        rid = srv.submit(mid, G[0], 5)
        time.sleep(0.2)
        st = srv.stats()
        assert st["queued"] == 1 and st["active"] == 0
        srv.cancel(rid)
        assert srv.stats()["cancelled"] == 1
        with pytest.raises(pkg.MlemError) as e:
            srv.wait(rid, timeout_ms=10)
        assert e.value.status == "EINVAL"
    with pkg.Server(slots_per_matrix=8) as srv:
        mid = srv.add_matrix(m)
        rid = srv.submit(mid, G[1], 3)
        img, lat = srv.wait(rid)
        assert lat > 0 and np.all(img >= 0)
        with pytest.raises(pkg.MlemError):
            srv.submit(7, G[1], 3)
    m.close()


def test_cli_dropin(pkg, O, tmp_path):
    p = problem(pkg, O, "ring2d")
    path = tmp_path / "m.csr4"
    pkg.csr4_write(path, p["rp"], p["col"], p["val"], p["cols"], geo=p["geo"])
    sino = tmp_path / "g.raw"
    p["g"].astype(np.int32).tofile(sino)
    img = tmp_path / "f.raw"
    env = dict(os.environ, MLEM_WRITE_IMAGE=str(img))
    for ut in (0, 1):
        for spmv in (0, 1):
            r = subprocess.run([str(pkg.CLI_PATH), str(path), str(sino), "10", "1", "5", "5", str(ut), str(spmv)],
                               capture_output=True, text=True, env=env, timeout=300)
            assert r.returncode == 0, r.stderr
            assert "\nSum f: " in r.stdout
            f = np.fromfile(img, np.float32)
            norm = O.colsum(p["rp"], p["col"], p["val"], p["cols"])
            ref = O.mlem_f64((p["rp"], p["col"], p["val"]), p["g"], norm,
                             np.full(p["cols"], O.initial_value(p["g"], norm)), 10)
            assert O.rel_l2(f, ref) < 1e-5
            s = float(r.stdout.split("Sum f:")[1])
            assert abs(s - float(np.sum(f, dtype=np.float32))) <= 1e-3 * abs(s)


def test_csr4_device_ingest(pkg, O, tmp_path):
    """mlem_matrix_load_csr4 streams the pairs through pinned staging and splits
    them on the GPU: the device matrix equals the file, across chunk borders
    (a 9 M-nonzero matrix spans two 8 M-pair chunks), and malformed files fail
    with EIO like the host reader."""
    rng = np.random.default_rng(5)
    rows, cols = 30000, 5000
    lens = rng.integers(0, 600, rows)
    lens[rng.integers(0, rows, 50)] = 0
    rp = np.zeros(rows + 1, np.uint64)
    rp[1:] = np.cumsum(lens)
    nnz = int(rp[-1])
    assert nnz > (1 << 23)
    col = np.empty(nnz, np.uint32)
    for r in range(0, rows, 1):
        s, t = int(rp[r]), int(rp[r + 1])
        if t > s:
            col[s:t] = np.sort(rng.choice(cols, t - s, replace=False))
    val = rng.uniform(0.01, 2.0, nnz).astype(np.float32)
    geo = pkg.preset("cyl3d_tiny")
    path = tmp_path / "big.csr4"
    pkg.csr4_write(path, rp, col, val, cols, geo=geo)
    m = pkg.Matrix.from_csr4(path)
    rp2, c2, v2 = m.csr()
    assert np.array_equal(rp2, rp) and np.array_equal(c2, col) and np.array_equal(v2.view(np.uint32), val.view(np.uint32))
    cp, ri, vt = m.transpose()
    cp0, ri0, vt0 = O.transpose(rp, col, val, cols)
    assert np.array_equal(cp, cp0) and np.array_equal(ri, ri0) and np.array_equal(vt, vt0)
    m.close()
    data = bytearray(path.read_bytes())
    scan = int(np.frombuffer(bytes(data[24:28]), np.uint32)[0])
    off = 28 + scan + 8 * rows + 8 * (nnz - 3)  # a column in the second chunk
    data[off:off + 4] = np.uint32(cols).tobytes()
    bad = tmp_path / "bad.csr4"
    bad.write_bytes(bytes(data))
    with pytest.raises(pkg.MlemError) as e:
        pkg.Matrix.from_csr4(bad)
    assert e.value.status == "EIO"
    short = tmp_path / "short.csr4"
    short.write_bytes(bytes(data[:-9]))
    with pytest.raises(pkg.MlemError) as e:
        pkg.Matrix.from_csr4(short)
    assert e.value.status == "EIO"
