"""Whole reconstructions in one persistent launch (kernel LOOP, GPU, C ABI).

The persistent loop runs every iteration of a reconstruction in one
cooperative launch, with grid-wide barriers between the projections.  Its
rows are summed exactly as the per-iteration csr-vector kernel sums them, so
for the same lanes per row and vectors in flight the image must be bit-identical
to the per-iteration path; the autotuned default (which may pick the loop for
small matrices) must agree bit for bit with the eager autotuned run, and all of
them must match the FP64 oracle (1e-5)."""
import numpy as np
import pytest

from conftest import problem

pytestmark = pytest.mark.gpu

TOL_F32 = 1e-5


@pytest.mark.parametrize("name", ["ring2d", "cyl3d_tiny", "cyl3d_rows32"])
@pytest.mark.parametrize("lanes,unroll", [(8, 1), (16, 2), (32, 2), (32, 4)])
def test_loop_bit_identical_to_per_iteration_kernels(pkg, O, name, lanes, unroll):
    p = problem(pkg, O, name)
    m = pkg.Matrix.from_csr(p["rp"], p["col"], p["val"], p["cols"])
    its = 13
    eager = m.run(p["g"], its, f0=p["f0"], kernel=pkg.KERNEL_DIRECT, lanes=lanes, unroll=unroll, use_graph=False)
    graph = m.run(p["g"], its, f0=p["f0"], kernel=pkg.KERNEL_DIRECT, lanes=lanes, unroll=unroll)
    loop = m.run(p["g"], its, f0=p["f0"], kernel=pkg.KERNEL_LOOP, lanes=lanes, unroll=unroll)
    assert np.array_equal(eager, graph)
    assert np.array_equal(loop, eager)
    ref = O.mlem_f64((p["rp"], p["col"], p["val"]), p["g"], p["norm"], p["f0"], its)
    assert O.rel_l2(loop, ref) < TOL_F32
    m.close()


@pytest.mark.parametrize("vt", ["f32", "f16"])
def test_autotuned_default_equals_eager_autotuned(pkg, O, vt):
    p = problem(pkg, O, "ring2d")
    m = pkg.Matrix.from_csr(p["rp"], p["col"], p["val"], p["cols"],
                            value_type=pkg.VAL_F32 if vt == "f32" else pkg.VAL_F16)
    default = m.run(p["g"], 20, f0=p["f0"])       # the loop or per-iteration graphs, as timed
    eager = m.run(p["g"], 20, f0=p["f0"], use_graph=False)
    assert np.array_equal(default, eager)
    again = m.run(p["g"], 20, f0=p["f0"])          # the choice is kept; same bits
    assert np.array_equal(again, default)
    ref = O.mlem_f64((p["rp"], p["col"], p["val"]), p["g"], p["norm"], p["f0"], 20)
    assert O.rel_l2(default, ref) < (TOL_F32 if vt == "f32" else 1e-3)
    m.close()


def test_loop_refuses_what_it_cannot_run(pkg, O):
    p = problem(pkg, O, "ring2d_tiny")
    m = pkg.Matrix.from_csr(p["rp"], p["col"], p["val"], p["cols"])
    for opts in (dict(spmv=pkg.SPMV_MERGE), dict(bp_mode=pkg.BP_SCATTER), dict(loglik_every=1)):
        with pytest.raises(pkg.MlemError) as e:
            m.run(p["g"], 3, kernel=pkg.KERNEL_LOOP, lanes=16, **opts)
        assert e.value.status == "EINVAL"
    m.close()
