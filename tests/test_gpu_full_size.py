"""Full-size accuracy: the 3-D mid matrix (208 M nonzeros) and the 12 GB-class
matrix (1.43 B nonzeros), 100 MLEM iterations, FP32 values (transposed back
projection, and the fused single pass) and FP16 values with 16-bit
delta-coded indices (FP32 accumulation), against the FP64 oracle (back projection over Aᵀ, OpenMP)
on the FP32 matrix.  Bars: image relative L2 1e-5 (FP32) and 1e-3 (FP16);
log-likelihood relative error 1e-6 (FP32) and 1e-4 (FP16).  The measured
errors are printed (run with -s to see them)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

WORKLOADS = {"cyl3d_mid": dict(shapes=20, total=1e8), "cyl3d_12gb": dict(shapes=20, total=1e8)}


def _sinogram(pkg, m, geo, cfg, torch):
    from mlem_gb300 import synth
    xt = torch.from_numpy(synth.phantom(geo, cfg["shapes"], seed=1).astype(np.float32)).cuda()
    dz = torch.zeros(m.rows, dtype=torch.int32, device="cuda")
    ratio = torch.zeros(m.rows, dtype=torch.float32, device="cuda")
    fp = torch.zeros(m.rows, dtype=torch.float32, device="cuda")
    m.forward_project(xt.data_ptr(), dz.data_ptr(), ratio.data_ptr(), fp.data_ptr())
    torch.cuda.synchronize()
    return synth.poisson_sinogram(fp.cpu().numpy().astype(np.float64), cfg["total"], seed=2)


@pytest.mark.parametrize("name", ["cyl3d_mid", "cyl3d_12gb"])
def test_full_size_fp32_and_fp16_against_fp64_oracle(pkg, O, cuda, name):
    cfg = WORKLOADS[name]
    geo = pkg.preset(name)
    iters = 100
    m = pkg.Matrix.generate(geo)
    g = _sinogram(pkg, m, geo, cfg, cuda)
    f0 = np.full(m.cols, m.initial_value(g), np.float32)
    img32, ll32 = m.run(g, iters, f0=f0, loglik=True)
    # the fused single pass (argv[7]=1 arithmetic, A read once per iteration;
    # the form the autotuner picks)
    imgF, llF = m.run(g, iters, f0=f0, loglik=True, bp_mode=pkg.BP_FUSED)
    formF = m.tuning(2)["kernel"]
    A, AT, norm = m.csr(), m.transpose(), m.norm()
    m.close()
    ref, llref = O.mlem_f64_t(A, AT, g, norm, f0, iters, loglik=True)
    del A, AT
    eF = O.rel_l2(imgF, ref)
    lF = float(np.max(np.abs(llF - llref) / np.abs(llref)))
    print(f"\n{name}: fused pass ({formF}) vs FP64 oracle: image rel L2 {eF:.3e}, log-likelihood {lF:.3e}")
    assert eF < 1e-5 and lF < 1e-6
    # FP16 values with 16-bit delta-coded indices (the compact precision form;
    # the autotuner picks among the csr-vector, interleaved and D16 kernels)
    m16 = pkg.Matrix.generate(geo, value_type=pkg.VAL_F16, compress=True)
    img16, ll16 = m16.run(g, iters, f0=f0, loglik=True)
    print(f"\n{name}: FP16 kernels {m16.tuning(False)['kernel']} / {m16.tuning(True)['kernel']}")
    m16.close()
    e32, e16 = O.rel_l2(img32, ref), O.rel_l2(img16, ref)
    l32 = float(np.max(np.abs(ll32 - llref) / np.abs(llref)))
    l16 = float(np.max(np.abs(ll16 - llref) / np.abs(llref)))
    print(f"\n{name}: {iters} iterations vs FP64 oracle: image rel L2 FP32 {e32:.3e}, FP16 {e16:.3e}; "
          f"log-likelihood max rel error FP32 {l32:.3e}, FP16 {l16:.3e}")
    assert e32 < 1e-5 and l32 < 1e-6
    assert e16 < 1e-3 and l16 < 1e-4
    assert np.all(np.diff(llref) > -1e-12 * np.abs(llref[0]))


@pytest.mark.parametrize("name", ["cyl3d_mid", "cyl3d_12gb"])
def test_full_size_symmetric_against_fp64_oracle(pkg, O, cuda, name):
    """The symmetry-compressed form at full size: the matrix is the symmetric Â
    (generate(symmetry=True)); 100 iterations with the autotuned kernels (the
    compact ones, checked) against the FP64 oracle on Â itself."""
    cfg = WORKLOADS[name]
    geo = pkg.preset(name)
    iters = 100
    m = pkg.Matrix.generate(geo, symmetry=True)
    g = _sinogram(pkg, m, geo, cfg, cuda)
    f0 = np.full(m.cols, m.initial_value(g), np.float32)
    img32, ll32 = m.run(g, iters, f0=f0, loglik=True)
    assert m.tuning(False)["kernel"] == "sym" and m.tuning(True)["kernel"] == "sym"
    sym = m.symmetry
    A, AT, norm = m.csr(), m.transpose(), m.norm()
    m.close()
    ref, llref = O.mlem_f64_t(A, AT, g, norm, f0, iters, loglik=True)
    del A, AT
    m16 = pkg.Matrix.generate(geo, value_type=pkg.VAL_F16, symmetry=True)
    img16 = m16.run(g, iters, f0=f0)
    m16.close()
    e32, e16 = O.rel_l2(img32, ref), O.rel_l2(img16, ref)
    l32 = float(np.max(np.abs(ll32 - llref) / np.abs(llref)))
    print(f"\n{name} symmetric ({sym}): {iters} iterations vs FP64 oracle on the symmetric matrix: "
          f"image rel L2 FP32 {e32:.3e}, FP16 {e16:.3e}; log-likelihood max rel error FP32 {l32:.3e}")
    assert e32 < 1e-5 and l32 < 1e-6
    assert e16 < 1e-3


def test_batched_fp16_at_its_configured_scale_against_fp64_oracle(pkg, O, cuda):
    """The batched form where FP16 error would grow: the 3-D mid matrix with
    FP16 values (locality layout), sinograms of the batched workload (phantom
    seeds 1000 + k, totals log-uniform in [1e5, 1e9] drawn with seed 7), 200
    iterations.  The instances with the smallest, the median and the largest
    total run in one batch with five more of the workload, and each image is
    compared with the FP64 oracle on the FP32 matrix.  Bar: 1e-3 relative L2."""
    from mlem_gb300 import synth
    torch = cuda
    geo = pkg.preset("cyl3d_mid")
    iters = 200
    totals = np.exp(np.random.Generator(np.random.PCG64(7)).uniform(np.log(1e5), np.log(1e9), 64))
    order = np.argsort(totals)
    picks = [int(order[0]), int(order[32]), int(order[-1])] + [int(k) for k in order[1:64:13][:5]]
    m32 = pkg.Matrix.generate(geo, layout=pkg.LAYOUT_LOCALITY)
    dz = torch.zeros(m32.rows, dtype=torch.int32, device="cuda")
    ratio = torch.zeros(m32.rows, dtype=torch.float32, device="cuda")
    fp = torch.zeros(m32.rows, dtype=torch.float32, device="cuda")
    G = []
    for k in picks:
        xt = torch.from_numpy(synth.phantom(geo, 20, seed=1000 + k)).cuda()
        m32.forward_project(xt.data_ptr(), dz.data_ptr(), ratio.data_ptr(), fp.data_ptr())
        torch.cuda.synchronize()
        G.append(synth.poisson_sinogram(fp.cpu().numpy().astype(np.float64), totals[k], seed=2000 + k))
    G = np.stack(G)
    F0 = np.stack([np.full(m32.cols, m32.initial_value(g), np.float32) for g in G])
    A, AT, norm = m32.csr(), m32.transpose(), m32.norm()
    m32.close()
    m16 = pkg.Matrix.generate(geo, value_type=pkg.VAL_F16, layout=pkg.LAYOUT_LOCALITY)
    out = m16.batch_run(G, np.full(len(G), iters, np.uint32), f0=F0)
    m16.close()
    for j, label in enumerate(("smallest", "median", "largest")):
        ref = O.mlem_f64_t(A, AT, G[j], norm, F0[j], iters)
        err = O.rel_l2(out[j], ref)
        print(f"\nbatched FP16, {label} total {totals[picks[j]]:.3g}, {iters} iterations: "
              f"image rel L2 vs FP64 oracle {err:.3e}")
        assert err < 1e-3
