"""The oracle's CPU generator of the synthetic matrices (the one the CPU
baseline builds its inputs with) against the library's host generator: the
same matrix bit for bit.  Also the parallel column sums over Aᵀ against the
serial ones over A."""
import numpy as np
import pytest


@pytest.mark.parametrize("name,stride,phase", [("ring2d", 1, 0), ("ring2d_tiny", 1, 0), ("cyl3d_tiny", 1, 0),
                                               ("cyl3d_mid", 97, 5), ("cyl3d_12gb", 997, 3)])
def test_oracle_generator_matches_library(pkg, O, name, stride, phase):
    geo = pkg.preset(name, row_stride=stride, row_phase=phase)
    rp, col, val, cols = pkg.siddon_host(geo)
    orp, ocol, oval, ocols = O.siddon(geo)
    assert ocols == cols
    assert np.array_equal(orp, rp) and np.array_equal(ocol, col)
    assert np.array_equal(oval.view(np.uint32), val.view(np.uint32))


def test_oracle_generator_rejects_bad_geometry(pkg, O):
    with pytest.raises(ValueError):
        O.siddon(pkg.geometry(0, 1, 1, 1, 1, 1, 1, 1, 1, 1))


def test_colsum_over_transpose_matches_serial(pkg, O):
    rp, col, val, cols = O.siddon(pkg.preset("cyl3d_tiny"))
    AT = O.transpose(rp, col, val, cols)
    a = O.colsum(rp, col, val, cols)
    b = O.colsum_t(AT, cols)
    assert np.array_equal(a.view(np.uint32), b.view(np.uint32))


def test_cpu_mlem_thread_count_is_per_call(pkg, O):
    rp, col, val, cols = O.siddon(pkg.preset("ring2d_tiny"))
    AT = O.transpose(rp, col, val, cols)
    norm = O.colsum(rp, col, val, cols)
    g = np.arange(len(rp) - 1, dtype=np.int32) % 7
    f0 = np.ones(cols, np.float32)
    before = O.max_threads()
    one = O.mlem_omp((rp, col, val), AT, g, norm, f0, 3, 1)
    assert O.max_threads() == before
    many = O.mlem_omp((rp, col, val), AT, g, norm, f0, 3, 0)
    # one row / one column per thread step: the same sums whatever the thread count
    assert np.array_equal(one, many)
