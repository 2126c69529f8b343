"""MLEM benchmark: iterations/s of the single-device MLEM loop on GB300.

Workload (default): the 12 GB-class synthetic scanner — 16 rings x 144
detectors (r = 60 mm), 200x200x64 voxels of 0.4 mm, 2,653,056 LOR rows,
~1.43 B nonzeros of multi-ray Siddon lengths (11.5 GB in FP32, 23 GB with the
transpose) — plain FP32 MLEM, csr-vector forward projection + transposed
back projection, 100 iterations per step, seeded 20-ellipsoid phantom,
Poisson sinogram of 1e8 counts.  All inputs are synthetic (the reference's
measured data are not distributed).

value  : iterations/s with the matrix, sinogram and image resident in HBM
         (one step = one 100-iteration reconstruction through mlem_run_device).
e2e    : the same through mlem_run (the C ABI a user calls) from pinned host
         buffers: sinogram + initial image in, image out, every step.
roofline: the dominant kernel's algorithmic bytes / its CUDA-event duration
         against the measured HBM copy bandwidth.
cpu_baseline: the oracle's OpenMP MLEM (FP32 values, FP64 accumulation) on the
         full matrix, built on the host by the oracle's own generator.

--impl reference times the CPU implementation of the path (the reference has
no CPU path of its own; the oracle port, pinned bit-exact to the reference's
compiled code, stands in) on the full matrix, with inputs built by the
oracle alone (the product library is not loaded), and prints its line.  The line also carries
"reference_cuda": the reference's own kernel.cu, compiled unmodified for
sm_103a into oracle/_ref/mlemref_kernels.cubin, launched with the grids and
step order of its single-GPU MLEM loop on the same workload (all four
argv[7]/argv[8] modes).
"""
from __future__ import annotations

import argparse
import importlib.util
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))
PKG_DIR = ROOT / "bachelorarbeit-mlem_gb300"
PROFILES = ROOT / "profiles"

WORKLOADS = {
    "cyl3d_12gb": dict(iters=100, shapes=20, total=1e8),
    "cyl3d_mid": dict(iters=100, shapes=20, total=1e8),
    "ring2d": dict(iters=20, shapes=5, total=1e6),
}


def load_pkg():
    spec = importlib.util.spec_from_file_location("mlem_gb300_build", PKG_DIR / "build.py")
    b = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(b)
    b.build()
    spec = importlib.util.spec_from_file_location("mlem_gb300", PKG_DIR / "__init__.py",
                                                  submodule_search_locations=[str(PKG_DIR)])
    m = importlib.util.module_from_spec(spec)
    sys.modules["mlem_gb300"] = m
    spec.loader.exec_module(m)
    return m


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


# kernel of each autotuner choice
KERNEL_NAMES = {"direct": "k_csrvec", "persistent": "k_csrvec_pipe", "tma": "k_csr_tma", "d16": "k_csr_d16",
                "ilv": "k_csr_ilv", "sym": "k_sym_orbit"}


def algorithmic_bytes(rows, cols, nnz, sv, m=None, kinds=None):
    """Per-launch algorithmic bytes of the two kernels of an iteration.  With m
    given and an operand run on its D16 copy (kinds = the FP and BP kernel
    names, else the autotuner's choices), that operand is counted as its stored
    entries (2 index bytes + sv each, dummies and padding included) and its
    vector pointers and base columns."""
    fp = nnz * (sv + 4) + 8 * (rows + 1) + 4 * cols + 4 * rows + 4 * rows   # A, rowptr, x once, g, ratio
    bp = nnz * (sv + 4) + 8 * (cols + 1) + 4 * rows + 12 * cols             # Aᵀ, colptr, ratio once, norm, f r/w
    if m is not None and m.d16:
        kinds = kinds or (m.tuning(False)["kernel"], m.tuning(True)["kernel"])
        if kinds[0] == "d16":
            fp = m.d16["slots"] * (sv + 2) + 12 * rows + 8 + 4 * cols + 4 * rows + 4 * rows
        if kinds[1] == "d16":
            bp = m.d16["slots_t"] * (sv + 2) + 12 * cols + 8 + 4 * rows + 12 * cols
    return fp, bp


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = max(mx, float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx or None,
                "reasons": sorted(reasons), "samples": len(sm)}


def dist_init(n_gpus):
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if n_gpus > 0 else "gloo")
    return rank, world, local, dist


def barrier(dist, torch=None):
    if dist is not None:
        if torch is not None:
            dist.barrier(device_ids=[torch.cuda.current_device()])
        else:
            dist.barrier()


LAYOUT = 1  # device layout of the generated matrices (set from --layout)


def make_problem(pkg, name, torch, value_type=0, compress=False, interleave=True):
    from mlem_gb300 import synth
    cfg = WORKLOADS[name]
    geo = pkg.preset(name)
    t0 = time.time()
    m = pkg.Matrix.generate(geo, value_type=value_type, compress=compress, interleave=interleave, layout=LAYOUT)
    t_gen = time.time() - t0
    xt = synth.phantom(geo, cfg["shapes"], seed=1).astype(np.float32)
    dx = torch.from_numpy(xt).cuda()
    dz = torch.zeros(m.rows, dtype=torch.int32, device="cuda")
    ratio = torch.zeros(m.rows, dtype=torch.float32, device="cuda")
    fp = torch.zeros(m.rows, dtype=torch.float32, device="cuda")
    m.forward_project(dx.data_ptr(), dz.data_ptr(), ratio.data_ptr(), fp.data_ptr(),
                      stream=torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    g = synth.poisson_sinogram(fp.cpu().numpy().astype(np.float64), cfg["total"], seed=2)
    return m, geo, g, t_gen


def time_kernels(pkg, m, torch, g, f0, iters=20, **opts):
    """Mean CUDA-event duration of the forward and back projection stages of a
    real reconstruction (mlem_run with kernel_timing: events on the launching
    stream around every stage, eager launches)."""
    m.run(g, 3, f0=f0, **opts)  # tuning / plans / graphs settled
    _, st = m.run(g, iters, f0=f0, stats=True, kernel_timing=True, **opts)
    return {"fp": st["fp_ms"], "bp": st["bp_ms"]}


def import_pkg():
    """The package's Python modules (scanner presets, phantoms, sinograms)
    without building or loading its CUDA library."""
    if "mlem_gb300" in sys.modules:
        return sys.modules["mlem_gb300"]
    spec = importlib.util.spec_from_file_location("mlem_gb300", PKG_DIR / "__init__.py",
                                                  submodule_search_locations=[str(PKG_DIR)])
    m = importlib.util.module_from_spec(spec)
    sys.modules["mlem_gb300"] = m
    spec.loader.exec_module(m)
    return m


def cpu_problem(pkg, name):
    """The workload built on the host CPU by the oracle alone (the product
    library is neither built nor loaded): the full matrix A from the oracle's
    generator (bit-identical to the library's), Aᵀ by the oracle's stable
    transpose, FP64 column sums, the seeded phantom's Poisson sinogram and the
    reference initial image."""
    from oracle import oracle as O
    from mlem_gb300 import synth
    cfg = WORKLOADS[name]
    geo = pkg.preset(name)
    t0 = time.perf_counter()
    rp, col, val, cols = O.siddon(geo)
    AT = O.transpose(rp, col, val, cols)
    norm = O.colsum_t(AT, cols)
    xt = synth.phantom(geo, cfg["shapes"], seed=1)
    g = synth.poisson_sinogram(O.project_f64(rp, col, val, xt), cfg["total"], seed=2)
    f0 = np.full(cols, O.initial_value(g, norm), np.float32)
    return dict(A=(rp, col, val), AT=AT, rows=len(rp) - 1, cols=cols, nnz=len(col), g=g, norm=norm, f0=f0,
                prep_s=time.perf_counter() - t0)


def cpu_iterations(P, iters, nthreads):
    """Seconds per MLEM iteration of the oracle's OpenMP CSR MLEM (transposed
    form, FP32 values and image, FP64 accumulation) on the full matrix."""
    from oracle import oracle as O
    t0 = time.perf_counter()
    O.mlem_omp(P["A"], P["AT"], P["g"], P["norm"], P["f0"], iters, nthreads)
    return (time.perf_counter() - t0) / iters


def cpu_baseline(P, iters=3):
    """The CPU baseline on the full matrix: all host threads (one warm-up
    iteration, then `iters` timed) and one thread (one iteration)."""
    from oracle import oracle as O
    threads = O.max_threads()
    cpu_iterations(P, 1, threads)
    sec = cpu_iterations(P, iters, threads)
    sec1 = cpu_iterations(P, 1, 1)
    assert O.max_threads() == threads  # the one-thread run leaves the default alone
    fp_b, bp_b = algorithmic_bytes(P["rows"], P["cols"], P["nnz"], 4)
    return {"value": 1.0 / sec, "unit": "iter/s", "cores": threads, "kind": "port", "cpu_model": cpu_model(),
            "one_thread_value": 1.0 / sec1, "achieved_gbs": (fp_b + bp_b) / sec / 1e9,
            "one_thread_gbs": (fp_b + bp_b) / sec1 / 1e9,
            "sample": f"full matrix ({P['rows']} rows, {P['nnz']} nnz): {iters} OpenMP MLEM iterations on "
                      f"{threads} threads after 1 warm-up, and 1 iteration on 1 thread (FP32 values and image, "
                      f"FP64 accumulation, transposed form)",
            "input_prep_s": round(P["prep_s"], 1)}


def repo_libraries():
    """The shared libraries of this repository mapped into the process."""
    try:
        maps = Path("/proc/self/maps").read_text().splitlines()
    except OSError:
        return None
    root = str(ROOT) + os.sep
    return sorted({ln.split()[-1][len(root):] for ln in maps
                   if ln.split() and ln.split()[-1].startswith(root) and ".so" in ln.split()[-1]})


def workload_config(name, rows, cols, nnz, replicas, values="f32"):
    """The `config` both arms print for a workload."""
    return {"workload": name, "rows": rows, "cols": cols, "nnz": nnz, "values": values,
            "l2": f"inputs larger than L2 ({8 * nnz / 1e9:.1f} GB matrix + {8 * nnz / 1e9:.1f} GB transpose)",
            "replicas": replicas}


def cpu_model() -> str:
    """The host CPU's model name (lscpu, else /proc/cpuinfo, else the platform)."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for ln in out.splitlines():
            if ln.strip().lower().startswith("model name"):
                return ln.split(":", 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    try:
        for ln in open("/proc/cpuinfo"):
            if ln.lower().startswith("model name"):
                return ln.split(":", 1)[1].strip()
    except OSError:
        pass
    import platform
    return platform.machine()


def run_reference(args):
    """The CPU implementation of the path on the host cores (the oracle port:
    the reference's MLEM loop exists only as CUDA kernels).  Inputs come from
    the oracle's generator; the product library is not loaded.  Each step is
    one MLEM iteration over the full matrix on all host threads."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from oracle import oracle as O
    pkg = import_pkg()
    name = args.workload
    P = cpu_problem(pkg, name)
    threads = O.max_threads()
    for _ in range(max(1, args.warmup)):
        cpu_iterations(P, 1, threads)
    per_step = [cpu_iterations(P, 1, threads) for _ in range(args.steps)]
    total = sum(per_step)
    value = args.steps / total
    sec1 = cpu_iterations(P, 1, 1)
    line = {
        "impl": "reference", "metric": "MLEM iterations/s", "value": value, "unit": "iter/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": max(1, args.warmup), "ms_per_step": total / args.steps * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32 values, f64 accumulation",
        "data": "synthetic (seeded multi-ray Siddon matrix, ellipsoid phantom, Poisson sinogram)",
        "config": workload_config(name, P["rows"], P["cols"], P["nnz"], args.gpus),
        "iterations_per_step": 1,
        "form": "CPU CSR MLEM, transposed form, natural layout",
        "cpu_baseline": {"value": value, "unit": "iter/s", "cores": threads, "kind": "port",
                         "cpu_model": cpu_model(), "one_thread_value": 1.0 / sec1,
                         "achieved_gbs": sum(algorithmic_bytes(P["rows"], P["cols"], P["nnz"], 4)) * value / 1e9,
                         "sample": f"full matrix ({P['rows']} rows, {P['nnz']} nnz), one MLEM iteration per step "
                                   f"on {threads} threads; one_thread_value: one iteration on 1 thread",
                         "step_ms": [round(x * 1e3, 2) for x in per_step], "input_prep_s": round(P["prep_s"], 1)},
        "e2e": {"value": value, "unit": "iter/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "the reference's MLEM loop exists only as CUDA kernels + NCCL; its CPU-side restatement "
                "(oracle/mlem_oracle.c, pinned bit-exact to the reference's compiled kernels) is timed",
    }
    if not args.no_ref_cuda:
        line["reference_cuda"] = reference_cuda(P, name, args)
    line["repo_libraries_mapped"] = repo_libraries()
    print(json.dumps(line), flush=True)


def reference_cuda(P, name, args):
    """The reference's kernel.cu on this GPU, launched as its main.cu loop
    does, on the inputs of the CPU arm."""
    try:
        import torch
        from oracle import ref_cuda
    except Exception as e:  # pragma: no cover
        return {"unavailable": f"import failed: {e}"}
    if not torch.cuda.is_available():
        return {"unavailable": "no CUDA device"}
    if not ref_cuda.available():
        return {"unavailable": "oracle/_ref/mlemref_kernels.cubin not built (needs the reference sources)"}
    g, norm, f0, cols = P["g"], P["norm"], P["f0"], P["cols"]
    out = {"kind": "reference kernel.cu compiled unmodified for sm_103a; main.cu:302-449 loop replayed at 1 GPU "
                   "(blocksize 1024, secsize 5/5, host synchronisations and memsets included)",
           "workload": name, "modes": {}}
    iters = max(3, min(args.steps, 10))
    with ref_cuda.ReferenceCudaMLEM(P["A"], cols, P["AT"]) as R:
        for label, spmv, trans in (("csr_vector_trans", 1, 0), ("merge_trans", 0, 0),
                                   ("csr_vector_scatter", 1, 1), ("merge_scatter", 0, 1)):
            if spmv == 1 and not R.csr_vector_ok(trans):
                out["modes"][label] = {"unavailable": "row count not a multiple of 32"}
                continue
            t = R.time(g, norm, f0, iters, warmup=max(1, args.warmup), spmv=spmv, using_trans=trans)
            out["modes"][label] = {k: round(v, 4) for k, v in t.items()}
    best = max((m for m in out["modes"].values() if "iterations_per_s" in m),
               key=lambda m: m["iterations_per_s"], default=None)
    if best is not None:
        out["value"] = best["iterations_per_s"]
        out["unit"] = "iter/s"
    return out


def time_csr4_ingest(pkg, m):
    """Loading the matrix from a csr4 file (the reference's input format):
    mlem_matrix_load_csr4 (pinned staging + GPU split) against reading the file
    into host SoA arrays and uploading them (mlem_csr4_read + mlem_matrix_create).
    The file is read from the page cache in both cases (written just before)."""
    import shutil
    import tempfile
    d = tempfile.mkdtemp(prefix="mlem_csr4_")
    try:
        rp, col, val = m.csr()
        path = os.path.join(d, "m.csr4")
        pkg.csr4_write(path, rp, col, val, m.cols, geo=pkg.preset("cyl3d_mid"))
        size = os.path.getsize(path)
        del rp, col, val
        out = {"file_bytes": size}
        for label in ("host_path_s", "device_ingest_s"):
            t0 = time.perf_counter()
            if label == "device_ingest_s":
                mm = pkg.Matrix.from_csr4(path, build_transpose=False)
            else:
                r, c, v, _ = pkg.csr4_read(path)
                mm = pkg.Matrix.from_csr(r, c, v, m.cols, build_transpose=False)
                del r, c, v
            out[label] = time.perf_counter() - t0
            mm.close()
        out["device_ingest_gbs"] = size / out["device_ingest_s"] / 1e9
        return out
    except Exception as e:  # disk space or permissions on the host
        return {"unavailable": str(e)[:200]}
    finally:
        shutil.rmtree(d, ignore_errors=True)


def run_modes(pkg, torch, name):
    """The reference's switch combinations (argv[8] merge / csr-vector x argv[7]
    transposed / scatter), the fused single pass and a batched run (16
    sinograms, 10 iterations) on one workload: every projection kernel runs."""
    m, _, g, _ = make_problem(pkg, name, torch, interleave=False)
    f0 = np.full(m.cols, m.initial_value(g), np.float32)
    its = 10
    out = {}
    for label, spmv, bp in (("csr_vector_trans", 1, 0), ("merge_trans", 0, 0), ("csr_vector_scatter", 1, 1),
                            ("merge_scatter", 0, 1), ("fused", 1, 2)):
        m.run(g, 3, f0=f0, spmv=spmv, bp_mode=bp)
        _, st = m.run(g, its, f0=f0, spmv=spmv, bp_mode=bp, stats=True)
        out[label] = {"iterations_per_s": its / st["seconds_iterations"]}
    G = np.stack([np.roll(g, 17 * k) for k in range(16)]).astype(np.int32)
    _, st = m.batch_run(G, np.full(16, its, np.uint32), stats=True)
    out["batched_16"] = {"images_iterations_per_s": 16 * its / st["seconds_iterations"]}
    m.close()
    return out


def run_forms(pkg, torch, args):
    """FP16-value and batched forms (images*iterations/s)."""
    from mlem_gb300 import synth
    res = {}
    s = torch.cuda.current_stream()
    name = args.workload
    iters = WORKLOADS[name]["iters"]
    # FP16 values with 16-bit delta-coded indices (~4.4 B per nonzero), same workload
    m16, geo, g, _ = make_problem(pkg, name, torch, value_type=pkg.VAL_F16, compress=True, interleave=False)
    g_dev = torch.from_numpy(g).cuda()
    f0 = np.full(m16.cols, m16.initial_value(g), np.float32)
    f0_dev = torch.from_numpy(f0).cuda()
    f_dev = torch.empty_like(f0_dev)
    kt16 = time_kernels(pkg, m16, torch, g, f0)
    fb, bb = algorithmic_bytes(m16.rows, m16.cols, m16.nnz, 2, m16)
    pk, pkind = peaks()
    res["fp16_kernels"] = {"fp_ms": kt16["fp"], "bp_ms": kt16["bp"], "fp": m16.tuning(False), "bp": m16.tuning(True),
                           "device_bytes": m16.device_bytes, "d16": m16.d16,
                           "roofline": {"fp_bytes": fb, "bp_bytes": bb, "peak": pk, "peak_kind": pkind,
                                        "fp_gbs": fb / (kt16["fp"] * 1e-3) / 1e9,
                                        "bp_gbs": bb / (kt16["bp"] * 1e-3) / 1e9,
                                        "fp_frac": fb / (kt16["fp"] * 1e-3) / 1e9 / pk,
                                        "bp_frac": bb / (kt16["bp"] * 1e-3) / 1e9 / pk}}
    # each variant with its default lanes / vectors in flight (the tuned choice is above)
    variants = {}
    for label, kern in (("direct", pkg.KERNEL_DIRECT), ("d16", pkg.KERNEL_D16)):
        t = time_kernels(pkg, m16, torch, g, f0, iters=10, kernel=kern)
        variants[label] = {"fp_ms": t["fp"], "bp_ms": t["bp"]}
    res["fp16_kernels"]["variants_ms"] = variants
    for bp_mode, label in ((0, "fp16_trans"), (2, "fp16_fused")):
        f_dev.copy_(f0_dev)
        m16.run_device(g_dev.data_ptr(), f_dev.data_ptr(), 5, stream=s.cuda_stream, bp_mode=bp_mode)
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        f_dev.copy_(f0_dev)
        a.record(s)
        m16.run_device(g_dev.data_ptr(), f_dev.data_ptr(), iters, stream=s.cuda_stream, bp_mode=bp_mode)
        b.record(s)
        b.synchronize()
        res[label] = {"images_iterations_per_s": iters / (a.elapsed_time(b) * 1e-3)}
    m16.close()
    # FP32 values with the same 16-bit delta-coded indices (lossless: the FP32 matrix)
    m32d, _, g32, _ = make_problem(pkg, name, torch, value_type=pkg.VAL_F32, compress=True, interleave=False)
    g32_dev = torch.from_numpy(g32).cuda()
    f32_0 = torch.from_numpy(np.full(m32d.cols, m32d.initial_value(g32), np.float32)).cuda()
    f32_dev = torch.empty_like(f32_0)
    f32_dev.copy_(f32_0)
    m32d.run_device(g32_dev.data_ptr(), f32_dev.data_ptr(), 5, stream=s.cuda_stream)
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    f32_dev.copy_(f32_0)
    a.record(s)
    m32d.run_device(g32_dev.data_ptr(), f32_dev.data_ptr(), iters, stream=s.cuda_stream)
    b.record(s)
    b.synchronize()
    res["fp32_d16"] = {"iterations_per_s": iters / (a.elapsed_time(b) * 1e-3),
                       "fp": m32d.tuning(False)["kernel"], "bp": m32d.tuning(True)["kernel"],
                       "form": "FP32 values, 16-bit delta-coded indices (same matrix as the FP32 plain path)"}
    m32d.close()
    # plain FP32 on the smaller matrices (the baselines of the batched and served forms)
    for small in ("cyl3d_mid", "ring2d"):
        msm, _, gs, _ = make_problem(pkg, small, torch, interleave=False)
        gsd = torch.from_numpy(gs).cuda()
        f0s = torch.from_numpy(np.full(msm.cols, msm.initial_value(gs), np.float32)).cuda()
        fs = torch.empty_like(f0s)
        its = WORKLOADS[small]["iters"]
        fs.copy_(f0s)
        msm.run_device(gsd.data_ptr(), fs.data_ptr(), its, stream=s.cuda_stream)
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(s)
        for _ in range(3):
            fs.copy_(f0s)
            msm.run_device(gsd.data_ptr(), fs.data_ptr(), its, stream=s.cuda_stream)
        b.record(s)
        b.synchronize()
        res[f"fp32_plain_{small}"] = {"images_iterations_per_s": 3 * its / (a.elapsed_time(b) * 1e-3)}
        if small == "cyl3d_mid":
            # the reference's four switch combinations (argv[8] merge/csr-vector x argv[7]
            # transposed/scatter) and the fused single pass, FP32, 100 iterations each
            modes = {}
            for label, spmv, bp in (("csr_vector_trans", 1, 0), ("merge_trans", 0, 0),
                                    ("csr_vector_scatter", 1, 1), ("merge_scatter", 0, 1), ("fused", 1, 2)):
                fs.copy_(f0s)
                msm.run_device(gsd.data_ptr(), fs.data_ptr(), 5, stream=s.cuda_stream, spmv=spmv, bp_mode=bp)
                fs.copy_(f0s)
                a.record(s)
                msm.run_device(gsd.data_ptr(), fs.data_ptr(), its, stream=s.cuda_stream, spmv=spmv, bp_mode=bp)
                b.record(s)
                b.synchronize()
                modes[label] = {"iterations_per_s": its / (a.elapsed_time(b) * 1e-3)}
            res["modes_cyl3d_mid"] = modes
            res["csr4_ingest_cyl3d_mid"] = time_csr4_ingest(pkg, msm)
        msm.close()
    res["batched_fp16_64"] = run_batched(pkg, torch, res["fp32_plain_cyl3d_mid"]["images_iterations_per_s"])
    return res


def run_batched(pkg, torch, fp32_mid_rate=None):
    """Batched form: the 3-D mid matrix with FP16 values, 64 sinograms of seeded
    phantoms, counts log-U[1e5, 1e9], iterations U{10..200}, one batch_run."""
    from mlem_gb300 import synth
    s = torch.cuda.current_stream()
    mb = pkg.Matrix.generate(pkg.preset("cyl3d_mid"), value_type=pkg.VAL_F16, layout=LAYOUT)
    rng = np.random.Generator(np.random.PCG64(7))
    totals = np.exp(rng.uniform(np.log(1e5), np.log(1e9), 64))
    its = np.random.Generator(np.random.PCG64(8)).integers(10, 201, 64).astype(np.uint32)
    dz = torch.zeros(mb.rows, dtype=torch.int32, device="cuda")
    ratio = torch.zeros(mb.rows, dtype=torch.float32, device="cuda")
    fp = torch.zeros(mb.rows, dtype=torch.float32, device="cuda")
    G = np.zeros((64, mb.rows), np.int32)
    geo_b = pkg.preset("cyl3d_mid")
    for k in range(64):
        xt = torch.from_numpy(synth.phantom(geo_b, 20, seed=1000 + k)).cuda()
        mb.forward_project(xt.data_ptr(), dz.data_ptr(), ratio.data_ptr(), fp.data_ptr(), stream=s.cuda_stream)
        G[k] = synth.poisson_sinogram(fp.cpu().numpy().astype(np.float64), totals[k], seed=2000 + k)
    _, st = mb.batch_run(G[:8], np.full(8, 2, np.uint32), stats=True)  # autotune + warm-up
    _, st = mb.batch_run(G, its, stats=True)
    out = {"images_iterations_per_s": float(its.sum()) / st["seconds_iterations"],
           "wall_images_iterations_per_s": float(its.sum()) / st["seconds_total"],
           "workload": "cyl3d_mid fp16, 64 sinograms, iterations U{10..200}"}
    # each form explicitly: per-iteration graphs, and the persistent loop (the
    # iterations between two refills in one cooperative launch)
    for form, label in ((1, "graphs"), (2, "persistent")):
        mb.batch_run(G[:8], np.full(8, 2, np.uint32), form=form)
        _, st = mb.batch_run(G, its, stats=True, form=form)
        out[f"{label}_images_iterations_per_s"] = float(its.sum()) / st["seconds_iterations"]
        out[f"{label}_kernel_launches"] = int(st["kernel_launches"])
    if fp32_mid_rate:
        out["vs_fp32_plain_same_matrix"] = out["images_iterations_per_s"] / fp32_mid_rate
    mb.close()
    # the same 64 reconstructions one after the other on the plain FP32 matrix
    # (device-resident sinograms and images, CUDA events around all 64 runs)
    m32 = pkg.Matrix.generate(geo_b, value_type=pkg.VAL_F32, layout=LAYOUT)
    Gd = torch.from_numpy(G).cuda()
    F0 = torch.from_numpy(np.stack([np.full(m32.cols, m32.initial_value(G[k]), np.float32) for k in range(64)])).cuda()
    f = torch.empty(m32.cols, dtype=torch.float32, device="cuda")
    f.copy_(F0[0])
    m32.run_device(Gd[0].data_ptr(), f.data_ptr(), 5, stream=s.cuda_stream)  # tuning and graphs settled
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record(s)
    for k in range(64):
        f.copy_(F0[k])
        m32.run_device(Gd[k].data_ptr(), f.data_ptr(), int(its[k]), stream=s.cuda_stream)
    b.record(s)
    b.synchronize()
    out["sequential_fp32_images_iterations_per_s"] = float(its.sum()) / (a.elapsed_time(b) * 1e-3)
    out["vs_sequential_fp32"] = out["images_iterations_per_s"] / out["sequential_fp32_images_iterations_per_s"]
    m32.close()
    return out


def run_symmetry(pkg, torch, name):
    """Symmetry-compressed operands on the workload's scanner: the symmetric
    matrix A^ (16 symmetries), MLEM iterations/s with the autotuned kernels and
    with each of the compact (SYM) and full csr-vector (DIRECT) kernels on the
    same A^, the stage times and the device bytes; and how far the A^ image is
    from the image of the plain generated matrix on the same sinogram."""
    from mlem_gb300 import synth
    s = torch.cuda.current_stream()
    cfg = WORKLOADS[name]
    geo = pkg.preset(name)
    its = cfg["iters"]
    out = {"workload": f"{name}, natural layout, 16 symmetries"}
    plain = pkg.Matrix.generate(geo)
    xt = torch.from_numpy(synth.phantom(geo, cfg["shapes"], seed=1).astype(np.float32)).cuda()
    dz = torch.zeros(plain.rows, dtype=torch.int32, device="cuda")
    ratio = torch.zeros(plain.rows, dtype=torch.float32, device="cuda")
    fp = torch.zeros(plain.rows, dtype=torch.float32, device="cuda")
    plain.forward_project(xt.data_ptr(), dz.data_ptr(), ratio.data_ptr(), fp.data_ptr(), stream=s.cuda_stream)
    torch.cuda.synchronize()
    g = synth.poisson_sinogram(fp.cpu().numpy().astype(np.float64), cfg["total"], seed=2)
    f0 = np.full(plain.cols, plain.initial_value(g), np.float32)
    img_plain = plain.run(g, its, f0=f0)
    plain_bytes = plain.device_bytes
    plain.close()
    for vt, label in ((pkg.VAL_F32, "fp32"), (pkg.VAL_F16, "fp16")):
        t0 = time.time()
        m = pkg.Matrix.generate(geo, value_type=vt, symmetry=True)
        r = {"build_s": time.time() - t0, "device_bytes": m.device_bytes, "plain_fp32_device_bytes": plain_bytes,
             "nnz": m.nnz, "compact": m.symmetry}
        g_dev = torch.from_numpy(g).cuda()
        f0_dev = torch.from_numpy(f0).cuda()
        f_dev = torch.empty_like(f0_dev)
        for klabel, kern in (("autotuned", pkg.KERNEL_AUTO), ("sym", pkg.KERNEL_SYM), ("direct", pkg.KERNEL_DIRECT)):
            f_dev.copy_(f0_dev)
            m.run_device(g_dev.data_ptr(), f_dev.data_ptr(), 5, stream=s.cuda_stream, kernel=kern)
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            f_dev.copy_(f0_dev)
            a.record(s)
            m.run_device(g_dev.data_ptr(), f_dev.data_ptr(), its, stream=s.cuda_stream, kernel=kern)
            b.record(s)
            b.synchronize()
            kt = time_kernels(pkg, m, torch, g, f0, iters=10, kernel=kern)
            r[klabel] = {"iterations_per_s": its / (a.elapsed_time(b) * 1e-3), "fp_ms": kt["fp"], "bp_ms": kt["bp"]}
        r["tuning"] = {"fp": m.tuning(False), "bp": m.tuning(True)}
        img = m.run(g, its, f0=f0)
        r["image_rel_l2_vs_plain_matrix"] = float(np.linalg.norm(img.astype(np.float64) - img_plain)
                                                  / np.linalg.norm(img_plain.astype(np.float64)))
        m.close()
        out[label] = r
    return out


def run_serving(pkg, torch, n_requests=2000, rate=50.0, serial_every=10):
    """Serving form: three resident matrices (2-D ring FP32, 3-D mid FP32,
    12 GB class FP16), Poisson arrivals, continuous batching in the server.
    Then the serial plain-FP32 baseline, measured: every serial_every-th
    request of the same list run one at a time through mlem_run (host
    sinogram in, host image out) on FP32 matrices (the 12 GB class in FP32
    too)."""
    import threading as th
    from mlem_gb300 import synth
    s = torch.cuda.current_stream()
    specs = [("ring2d", pkg.VAL_F32, 0.5), ("cyl3d_mid", pkg.VAL_F32, 0.35), ("cyl3d_12gb", pkg.VAL_F16, 0.15)]
    mats, expect = [], []
    for name, vt, _ in specs:
        geo = pkg.preset(name)
        m = pkg.Matrix.generate(geo, value_type=vt, layout=LAYOUT)
        dz = torch.zeros(m.rows, dtype=torch.int32, device="cuda")
        ratio = torch.zeros(m.rows, dtype=torch.float32, device="cuda")
        fp = torch.zeros(m.rows, dtype=torch.float32, device="cuda")
        ex = []
        for k in range(4):  # four phantoms per matrix; requests rescale their counts
            xt = torch.from_numpy(synth.phantom(geo, WORKLOADS[name]["shapes"], seed=3000 + k)).cuda()
            m.forward_project(xt.data_ptr(), dz.data_ptr(), ratio.data_ptr(), fp.data_ptr(), stream=s.cuda_stream,
                              kernel=0)
            ex.append(fp.cpu().numpy().astype(np.float64))
        mats.append(m)
        expect.append(ex)
    rng = np.random.Generator(np.random.PCG64(11))
    arrivals = np.cumsum(rng.exponential(1.0 / rate, n_requests))
    which = rng.choice(3, size=n_requests, p=[p for _, _, p in specs])
    totals = np.exp(rng.uniform(np.log(1e5), np.log(1e9), n_requests))
    iters = rng.integers(20, 101, n_requests)
    sinos = [synth.poisson_sinogram(expect[w][i % 4], totals[i], seed=5000 + i) for i, w in enumerate(which)]
    lat = [None] * n_requests
    with pkg.Server() as srv:
        ids = [srv.add_matrix(m) for m in mats]
        # warm-up: one request per matrix (graphs captured, slot states allocated)
        for j in range(3):
            srv.wait(srv.submit(ids[j], sinos[int(np.argmax(which == j))], 2))
        rids = [None] * n_requests
        t0 = time.perf_counter()

        def submitter():
            for i in range(n_requests):
                d = t0 + arrivals[i] - time.perf_counter()
                if d > 0:
                    time.sleep(d)
                rids[i] = srv.submit(ids[which[i]], sinos[i], int(iters[i]))

        st = th.Thread(target=submitter)
        st.start()
        for i in range(n_requests):
            while rids[i] is None:
                time.sleep(0.0005)
            _, lat[i] = srv.wait(rids[i])
        st.join()
        wall = time.perf_counter() - t0
        stats = srv.stats()
    lat = np.array(lat)
    out = {"requests": n_requests, "arrival_rate_per_s": rate, "p50_latency_s": float(np.percentile(lat, 50)),
           "p99_latency_s": float(np.percentile(lat, 99)), "mean_latency_s": float(lat.mean()),
           "p99_tail_samples": int((lat >= np.percentile(lat, 99)).sum()),
           "reconstructions_per_s": n_requests / wall, "wall_s": wall,
           "iterations_done": int(stats["iterations_done"]),
           "mix": "ring2d fp32 0.5 / cyl3d_mid fp32 0.35 / cyl3d_12gb fp16 0.15, counts log-U[1e5,1e9], "
                  "iterations U{20..100}, autotuned slots per matrix, projections over the occupied slots, "
                  "small matrices (< 16 M nonzeros) on a high-priority stream, pinned staging of sinograms "
                  "and images"}
    for j, (name, _, _) in enumerate(specs):
        sel = which == j
        if sel.any():
            out[f"p50_latency_s_{name}"] = float(np.percentile(lat[sel], 50))
            out[f"p99_latency_s_{name}"] = float(np.percentile(lat[sel], 99))
    # serial plain FP32: the same requests one at a time through mlem_run
    mats[2].close()
    mats[2] = pkg.Matrix.generate(pkg.preset("cyl3d_12gb"), value_type=pkg.VAL_F32, layout=LAYOUT)
    sample = list(range(0, n_requests, serial_every))
    for j in range(3):  # tuning and plans settled outside the timed loop
        mats[j].run(sinos[int(np.argmax(which == j))], 2)
    t0 = time.perf_counter()
    for i in sample:
        mats[which[i]].run(sinos[i], int(iters[i]))
    serial_s = time.perf_counter() - t0
    out["serial_fp32_reconstructions_per_s"] = len(sample) / serial_s
    out["serial_fp32_sample"] = f"every {serial_every}th request of the list ({len(sample)} requests), " \
                                f"one at a time through mlem_run, FP32 matrices, {serial_s:.1f} s"
    out["vs_serial_fp32"] = out["reconstructions_per_s"] / out["serial_fp32_reconstructions_per_s"]
    for m in mats:
        m.close()
    return out


def forms_summary(forms, fp32_rate):
    """The headline figure of each form and its ratio to the FP32 plain path."""
    out = {"fp32_plain_iter_s": round(fp32_rate, 2)}
    fz = forms.get("fused_pass")
    if fz:
        out["fused_pass_iter_s"] = round(fz["iterations_per_s"], 2)
        out["fused_pass_vs_fp32_plain"] = round(fz["vs_fp32_plain"], 3)

    def put(key, val, ratio_to=None, nd=2):
        if val is None:
            return
        out[key] = round(val, nd)
        if ratio_to:
            out[key.replace("_s", "") + "_vs_fp32_plain"] = round(val / ratio_to, 3)

    put("fp16_d16_images_iter_s", forms.get("fp16_trans", {}).get("images_iterations_per_s"), fp32_rate)
    mid = forms.get("fp32_plain_cyl3d_mid", {}).get("images_iterations_per_s")
    put("mid_fp32_plain_iter_s", mid)
    put("ring2d_fp32_plain_iter_s", forms.get("fp32_plain_ring2d", {}).get("images_iterations_per_s"), nd=0)
    b = forms.get("batched_fp16_64", {})
    put("batched_fp16_64_images_iter_s", b.get("images_iterations_per_s"), mid)
    put("sequential_fp32_64_images_iter_s", b.get("sequential_fp32_images_iterations_per_s"))
    put("batched_vs_sequential_fp32", b.get("vs_sequential_fp32"), nd=3)
    put("batched_persistent_images_iter_s", b.get("persistent_images_iterations_per_s"))
    put("batched_graphs_images_iter_s", b.get("graphs_images_iterations_per_s"))
    modes = forms.get("modes_cyl3d_mid") or forms
    for k in ("csr_vector_trans", "merge_trans", "csr_vector_scatter", "merge_scatter", "fused"):
        if isinstance(modes.get(k), dict) and "iterations_per_s" in modes[k]:
            out[f"mid_{k}_iter_s"] = round(modes[k]["iterations_per_s"], 1)
    sv = forms.get("serving")
    if sv:
        out["serving"] = {k: (round(sv[k], 4) if isinstance(sv[k], float) else sv[k])
                          for k in ("requests", "p50_latency_s", "p99_latency_s", "reconstructions_per_s",
                                    "serial_fp32_reconstructions_per_s", "vs_serial_fp32", "p99_tail_samples")
                          if k in sv}
    sy = forms.get("symmetry", {}).get("fp32")
    if sy:
        out["symmetry_matrix_hat_fp32_iter_s"] = round(sy["autotuned"]["iterations_per_s"], 1)
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="cyl3d_12gb", choices=sorted(WORKLOADS))
    ap.add_argument("--forms", default="all", choices=["all", "none", "modes", "symmetry", "batched", "serving"],
                    help="all: FP16, batched, serving, symmetry and the modes on the smaller matrices; modes: only "
                         "the reference's switch combinations, the fused pass and a batched run on --workload; "
                         "symmetry: only the symmetry-compressed operands on --workload")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--detail-dir", default="bench_out",
                    help="folder (relative to the repository) for the per-variant detail of the forms")
    ap.add_argument("--spmv", default="csr-vector", choices=["csr-vector", "merge"],
                    help="SpMV of the timed reconstruction (the reference's argv[8])")
    ap.add_argument("--values", default="f32", choices=["f32", "f16", "bf16"],
                    help="value type of the timed matrix (f32: the plain path; FP32 accumulation always)")
    ap.add_argument("--kernel", default="auto", choices=["auto", "direct", "d16", "ilv", "tma", "persistent"],
                    help="csr-vector kernel of the timed path (auto: the autotuner's choice per operand; a fixed "
                         "choice keeps profiled runs on the same kernel as plain ones)")
    ap.add_argument("--compress", action="store_true",
                    help="also build the 16-bit delta-coded index copy (D16) of the timed matrix for the autotuner")
    ap.add_argument("--layout", default="locality", choices=["natural", "locality"],
                    help="device layout of the generated matrices (rows in LOR tubes, columns in voxel bricks)")
    ap.add_argument("--bp", default="trans", choices=["trans", "scatter", "fused"],
                    help="back projection of the timed reconstruction (argv[7]; fused: single pass)")
    ap.add_argument("--no-ref-cuda", action="store_true",
                    help="reference arm: skip timing the reference's CUDA kernels")
    ap.add_argument("--no-interleave", action="store_true",
                    help="skip the lane-interleaved matrix copy (halves device memory)")
    args = ap.parse_args()
    global LAYOUT
    LAYOUT = 1 if args.layout == "locality" else 0
    if args.impl == "reference":
        return run_reference(args)

    import torch
    rank, world, local, dist = dist_init(args.gpus)
    torch.cuda.set_device(local)
    pkg = load_pkg()
    name = args.workload
    iters = WORKLOADS[name]["iters"]
    vt = {"f32": pkg.VAL_F32, "f16": pkg.VAL_F16, "bf16": pkg.VAL_BF16}[args.values]
    sv = 4 if args.values == "f32" else 2
    m, geo, g, t_gen = make_problem(pkg, name, torch, value_type=vt, compress=args.compress,
                                    interleave=not args.no_interleave)
    s = torch.cuda.current_stream()
    g_dev = torch.from_numpy(g).cuda()
    f0 = np.full(m.cols, m.initial_value(g), np.float32)
    f0_dev = torch.from_numpy(f0).cuda()
    f_dev = torch.empty_like(f0_dev)

    SPMV = 0 if args.spmv == "merge" else 1
    BP = {"trans": 0, "scatter": 1, "fused": 2}[args.bp]
    KERN = {"auto": pkg.KERNEL_AUTO, "direct": pkg.KERNEL_DIRECT, "d16": pkg.KERNEL_D16, "ilv": pkg.KERNEL_ILV,
            "tma": pkg.KERNEL_TMA, "persistent": pkg.KERNEL_PERSISTENT}[args.kernel]
    default_form = SPMV == 1 and BP == 0 and args.values == "f32" and not args.compress and args.kernel == "auto"

    def step():
        f_dev.copy_(f0_dev)
        m.run_device(g_dev.data_ptr(), f_dev.data_ptr(), iters, stream=s.cuda_stream, spmv=SPMV, bp_mode=BP,
                     kernel=KERN)

    for _ in range(max(3, args.warmup)):
        step()
    torch.cuda.synchronize()
    barrier(dist, torch)
    n0 = pkg.kernel_launch_count()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        torch.cuda.synchronize()
        a.record(s)
        for _ in range(args.steps):
            step()
        b.record(s)
        torch.cuda.synchronize()
    launches = pkg.kernel_launch_count() - n0
    ms = a.elapsed_time(b)
    t = torch.tensor([ms], dtype=torch.float64, device="cuda")
    if dist is not None:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    ms = float(t.item())
    barrier(dist, torch)
    value = world * args.steps * iters / (ms * 1e-3)

    # e2e: through mlem_run from pinned host buffers (sinogram + f0 in, image out)
    g_pin = torch.from_numpy(g).pin_memory()
    f0_pin = torch.from_numpy(f0).pin_memory()
    out_pin = torch.empty(m.cols, dtype=torch.float32).pin_memory()
    import ctypes as C
    lib = pkg.load_library()
    ro = pkg.Matrix.run_opts(spmv=SPMV, bp_mode=BP, kernel=KERN)

    def e2e_step():
        st = lib.mlem_run(m.handle, C.c_void_p(g_pin.data_ptr()), C.c_void_p(f0_pin.data_ptr()), iters,
                          C.byref(ro), C.c_void_p(out_pin.data_ptr()), None, None)
        if st != 0:
            raise pkg.MlemError(st, lib.mlem_last_error().decode())

    e2e_step()
    torch.cuda.synchronize()
    barrier(dist, torch)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        e2e_step()
    torch.cuda.synchronize()
    e2e_s = time.perf_counter() - t0
    te = torch.tensor([e2e_s], dtype=torch.float64, device="cuda")
    if dist is not None:
        dist.all_reduce(te, op=dist.ReduceOp.MAX)
    e2e_value = world * args.steps * iters / float(te.item())

    # roofline of the dominant kernel
    kt = time_kernels(pkg, m, torch, g, f0, spmv=SPMV, bp_mode=BP, kernel=KERN)
    kt_direct = time_kernels(pkg, m, torch, g, f0, kernel=0)
    kt_tma = time_kernels(pkg, m, torch, g, f0, kernel=1)
    kt_pers = time_kernels(pkg, m, torch, g, f0, kernel=2)
    kinds = None if args.kernel == "auto" else (args.kernel, args.kernel)
    fp_b, bp_b = algorithmic_bytes(m.rows, m.cols, m.nnz, sv, m, kinds)
    dom = "fp" if kt["fp"] >= kt["bp"] else "bp"
    dom_bytes = fp_b if dom == "fp" else bp_b
    peak, peak_kind = peaks()
    achieved = dom_bytes / (kt[dom] * 1e-3) / 1e9
    iter_bytes = fp_b + bp_b
    traffic = None
    tf = PROFILES / "dram_traffic.json"
    if tf.exists() and default_form:
        key = f"{name}/{dom}" + ("/locality" if LAYOUT else "")
        traffic = json.loads(tf.read_text()).get(key)

    line = {
        "metric": "MLEM iterations/s", "value": value, "unit": "iter/s", "n_gpus": world,
        "steps": args.steps, "warmup": max(3, args.warmup), "ms_per_step": ms / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32" if args.values == "f32" else f"{args.values} values, f32 accumulation",
        "data": "synthetic (seeded multi-ray Siddon matrix, ellipsoid phantom, Poisson sinogram)",
        "config": workload_config(name, m.rows, m.cols, m.nnz, world, args.values),
        "iterations_per_step": iters,
        "form": (f"fp32 plain: {args.spmv} SpMV, {args.bp} BP, {args.layout} layout"
                 if args.values == "f32" and not args.compress else
                 f"{args.values} values{', D16 indices' if args.compress else ''}: {args.spmv} SpMV, "
                 f"{args.bp} BP, {args.layout} layout"),
        "device_bytes": m.device_bytes, "matrix_generation_s": round(t_gen, 2),
        "e2e": {"value": e2e_value, "unit": "iter/s", "h2d_bytes_per_step": int(4 * m.rows + 4 * m.cols),
                "d2h_bytes_per_step": int(4 * m.cols)},
        "gpu_launches": int(launches),
        "roofline": {"bound": "hbm", "kernel": KERNEL_NAMES.get(kinds[dom == "bp"] if kinds else
                                                               m.tuning(dom == "bp")["kernel"], "k_csrvec") + " "
                     + ("(FP, fused correlation)" if dom == "fp" else "(BP over Aᵀ, fused update)"),
                     "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "peak_kind": peak_kind, "traffic": traffic,
                     "algorithmic_bytes": dom_bytes, "kernel_ms": kt[dom],
                     "iteration": {"bytes": iter_bytes, "ms": ms / args.steps / iters,
                                   "achieved_gbs": iter_bytes / (ms / args.steps / iters * 1e-3) / 1e9,
                                   "frac": iter_bytes / (ms / args.steps / iters * 1e-3) / 1e9 / peak},
                     "fp_ms": kt["fp"], "bp_ms": kt["bp"],
                     "variants_ms": {"autotuned": kt, "direct": kt_direct, "tma": kt_tma, "persistent": kt_pers},
                     "autotuned": {"fp": m.tuning(False), "bp": m.tuning(True)}},
        "clocks": clk.summary(),
    }
    if default_form:
        # the fused single pass (argv[7]=1 arithmetic: A read once per
        # iteration, the back projection by atomic vector reductions) on the same matrix
        def fused_step():
            f_dev.copy_(f0_dev)
            m.run_device(g_dev.data_ptr(), f_dev.data_ptr(), iters, stream=s.cuda_stream, bp_mode=2,
                         kernel=pkg.KERNEL_AUTO)

        for _ in range(max(3, args.warmup)):
            fused_step()
        torch.cuda.synchronize()
        a.record(s)
        for _ in range(args.steps):
            fused_step()
        b.record(s)
        torch.cuda.synchronize()
        f_rate = args.steps * iters / (a.elapsed_time(b) * 1e-3)
        # its algorithmic bytes: one forward-projection stream (A once, the row
        # pointers, g, f) per iteration; the update's vectors are left out
        line["fused_pass"] = {"iterations_per_s": f_rate, "vs_fp32_plain": f_rate / (value / world),
                              "form": m.tuning(2), "bytes_per_iteration": fp_b,
                              "achieved_gbs": fp_b * f_rate / 1e9, "frac": fp_b * f_rate / 1e9 / peak}
    m.close()
    if args.forms == "modes":
        line["forms"] = run_modes(pkg, torch, name)
    if args.forms == "symmetry":
        line["forms"] = {"symmetry": run_symmetry(pkg, torch, name)}
    if args.forms == "batched":
        line["forms"] = {"batched_fp16_64": run_batched(pkg, torch)}
    if args.forms == "serving":
        line["forms"] = {"serving": run_serving(pkg, torch)}
    if args.forms == "all":
        line["forms"] = run_forms(pkg, torch, args)
        line["forms"]["fp32_plain"] = {"images_iterations_per_s": value / world}
        line["forms"]["serving"] = run_serving(pkg, torch)
        line["forms"]["symmetry"] = run_symmetry(pkg, torch, name)
    if rank == 0 and not args.no_cpu:
        P = cpu_problem(pkg, name)
        line["cpu_baseline"] = cpu_baseline(P)
        del P
    if "forms" in line:
        # the per-variant detail goes to a file; the line ends with the headline of each form
        forms = line.pop("forms")
        detail = ROOT / args.detail_dir / f"bench_forms_{name}.json"
        try:
            detail.parent.mkdir(parents=True, exist_ok=True)
            detail.write_text(json.dumps(forms, indent=1))
            line["forms_detail"] = str(detail.relative_to(ROOT))
        except OSError:
            line["forms"] = forms
        line["forms_summary"] = forms_summary(dict(forms, fused_pass=line.get("fused_pass")), value / world)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
