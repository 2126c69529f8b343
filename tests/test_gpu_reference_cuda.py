"""The library against the reference's own CUDA kernels on the GPU.

kernel.cu of the reference, compiled unmodified for sm_103a
(oracle/_ref/mlemref_kernels.cubin), is launched by oracle/ref_cuda.py with
the grids and the step order of its MLEM loop (main.cu:302-321, 329-449).
On the same inputs the library's image must agree with the reference's
within the FP32 tolerance (1e-5 relative L2); the reference's own
run-to-run spread (its FP32 atomics) is printed as the noise floor.  Skipped
where the cubin was not built (it needs the reference sources)."""
import sys
from pathlib import Path

import numpy as np
import pytest

sys.path.insert(0, str(Path(__file__).resolve().parent))
from conftest import golden_csr, problem  # noqa: E402

pytestmark = pytest.mark.gpu

TOL_F32 = 1e-5
MODES = [(1, 0), (0, 0), (1, 1), (0, 1)]  # (argv[8] spmv, argv[7] using_trans)


@pytest.fixture(scope="module")
def refcuda(cuda):
    from oracle import ref_cuda
    if not ref_cuda.available():
        pytest.skip("reference cubin not built (built where the reference sources are present)")
    return ref_cuda


@pytest.mark.parametrize("spmv,using_trans", MODES)
@pytest.mark.parametrize("name", ["ring2d", "cyl3d_rows32"])
def test_library_matches_reference_cuda_kernels(pkg, O, refcuda, name, spmv, using_trans):
    p = problem(pkg, O, name)
    A = (p["rp"], p["col"], p["val"])
    AT = O.transpose(*A, p["cols"])
    norm = p["norm"].astype(np.float32)
    iters = 20
    with refcuda.ReferenceCudaMLEM(A, p["cols"], AT) as R:
        assert R.csr_vector_ok(using_trans)
        ref = R.run(p["g"], norm, p["f0"], iters, spmv=spmv, using_trans=using_trans)
        ref_again = R.run(p["g"], norm, p["f0"], iters, spmv=spmv, using_trans=using_trans)
    noise = O.rel_l2(ref_again, ref)
    m = pkg.Matrix.from_csr(*A, p["cols"], norm=norm)
    got = m.run(p["g"], iters, f0=p["f0"], spmv=spmv, bp_mode=using_trans)
    m.close()
    err = O.rel_l2(got, ref)
    print(f"{name} spmv={spmv} trans={using_trans}: library vs reference CUDA {err:.2e}, "
          f"reference run-to-run {noise:.2e}")
    assert err < TOL_F32
    ref64 = O.mlem_f64(A, p["g"], norm, p["f0"], iters)
    assert O.rel_l2(ref, ref64) < TOL_F32  # the reference kernels themselves agree with the FP64 oracle


@pytest.mark.parametrize("spmv,using_trans", [(0, 0), (0, 1)])
def test_reference_cuda_kernels_match_golden_fixtures(pkg, golden, refcuda, O, spmv, using_trans):
    """The golden fixtures came from the reference compiled for the CPU; its
    CUDA kernels give the same images (merge modes: any row count)."""
    for name in ("ring2d_tiny", "cyl3d_tiny"):
        rp, c, v, cols = golden_csr(golden, name)
        g, norm, f0 = golden[f"{name}/g"], golden[f"{name}/norm"], golden[f"{name}/f0"]
        AT = O.transpose(rp, c, v, cols)
        with refcuda.ReferenceCudaMLEM((rp, c, v), cols, AT) as R:
            for iters in (1, 4, 12):
                want = golden[f"{name}/mlem_s{spmv}_t{using_trans}_ss5x5_it{iters}"]
                got = R.run(g, norm, f0, iters, spmv=spmv, using_trans=using_trans)
                assert O.rel_l2(got, want) < TOL_F32, (name, iters)


@pytest.mark.parametrize("name", ["cyl3d_mid", "cyl3d_12gb"])
def test_library_matches_reference_cuda_kernels_full_size(pkg, O, cuda, refcuda, name):
    """The configured matrices at full size (3-D mid: 662,976 x 784,000,
    208 M nonzeros; 12 GB class: 2,653,056 x 2,560,000, 1.43 B nonzeros; both
    dimensions multiples of 32, so every mode of the reference may run), 100
    iterations in all four argv[7]/argv[8] modes: the library in its
    benchmark layout (locality) against the reference's kernels on the natural
    matrix, same sinogram, sensitivity and initial image."""
    from test_gpu_full_size import WORKLOADS, _sinogram
    geo = pkg.preset(name)
    iters = 100
    m = pkg.Matrix.generate(geo, layout=pkg.LAYOUT_LOCALITY)
    g = _sinogram(pkg, m, geo, WORKLOADS[name], cuda)
    f0 = np.full(m.cols, m.initial_value(g), np.float32)
    norm = m.norm().astype(np.float32)
    got = {mode: m.run(g, iters, f0=f0, spmv=mode[0], bp_mode=mode[1]) for mode in MODES}
    A, AT = m.csr(), m.transpose()
    m.close()
    with refcuda.ReferenceCudaMLEM(A, len(norm), AT) as R:
        del A, AT
        for spmv, using_trans in MODES:
            assert R.csr_vector_ok(using_trans)
            ref = R.run(g, norm, f0, iters, spmv=spmv, using_trans=using_trans)
            ref_again = R.run(g, norm, f0, iters, spmv=spmv, using_trans=using_trans)
            err = O.rel_l2(got[(spmv, using_trans)], ref)
            print(f"\n{name} spmv={spmv} trans={using_trans}, {iters} iterations: library vs reference CUDA "
                  f"{err:.2e}, reference run-to-run {O.rel_l2(ref_again, ref):.2e}")
            assert err < TOL_F32


def test_reference_cuda_timing_runs(pkg, O, refcuda):
    p = problem(pkg, O, "ring2d")
    A = (p["rp"], p["col"], p["val"])
    with refcuda.ReferenceCudaMLEM(A, p["cols"], O.transpose(*A, p["cols"])) as R:
        t = R.time(p["g"], p["norm"].astype(np.float32), p["f0"], 5, spmv=1, using_trans=0)
    assert t["iterations_per_s"] > 0 and t["fp_ms"] > 0 and t["bp_ms"] > 0
