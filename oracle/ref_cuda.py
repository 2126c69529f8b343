"""The reference's own CUDA kernels, launched as its MLEM loop launches them.

Test and measurement infrastructure, never used by the library.  kernel.cu of
the reference is compiled unmodified into oracle/_ref/mlemref_kernels.cubin
(ref_build.build_cubin); this module loads that cubin through the CUDA driver
API and replays the single-GPU MLEM loop of main.cu with its grids and step
order:

  grids        main.cu:302-321 (blocksize 1024, main.cu:231): csr-vector one
               warp per row, ceil(n/32) blocks; merge-based
               ceil((n + nnz) / (1024 * secsize)) blocks; correl/update
               ceil(n/1024) blocks
  iteration    main.cu:329-449: FP (merge or csr-vector) -> calcCorrel ->
               [trans: AllReduce of temp, a no-op for one rank, + stream
               synchronize] -> BP (merge / csr-vector over A^T, or
               calcBwProj_none_trans over A) -> calcUpdate -> AllReduce of
               bwproj into f (one rank: a device-to-device copy) + stream
               synchronize -> memset bwproj, memset temp
  device data  main.cu:241-296: u32 row pointers, u32 columns, f32 values;
               temp and bwproj zeroed before the first iteration

The tests compare the library's images with the images these kernels compute
on the same inputs; the benchmark's reference arm times them.

Safety: mat_vec_mul_csr_vector (kernel.cu:297-336) calls __syncthreads()
inside its row loop, which the warps of a partial last block skip; csr-vector
modes are therefore only launched when the operand's row count is a multiple
of 32, so every warp of every block owns a row.
"""
from __future__ import annotations

import ctypes as C
import math
import time
from pathlib import Path

import numpy as np

CUBIN = Path(__file__).resolve().parent / "_ref" / "mlemref_kernels.cubin"
BLOCK = 1024  # main.cu:231

# Itanium-mangled names of the kernels declared in kernel.cuh:7-19.
KERNELS = {
    "correl": "_Z10calcCorrelPiPfj",
    "update": "_Z10calcUpdatePfS_S_j",
    "fp_merge": "_Z22calcFwProj_merge_basedPjS_PfS0_S0_jjj",
    "bp_merge": "_Z22calcBwProj_merge_basedPjS_PfS0_S0_jjj",
    "fp_csrvec": "_Z21calcFwProj_csr_vectorPjS_PfS0_S0_j",
    "bp_csrvec": "_Z21calcBwProj_csr_vectorPjS_PfS0_S0_j",
    "bp_none_trans": "_Z21calcBwProj_none_transPjS_PfS0_S0_j",
}


def available() -> bool:
    return CUBIN.exists()


class DriverError(RuntimeError):
    pass


class _Driver:
    def __init__(self, device: int):
        self.cu = C.CDLL("libcuda.so.1")
        self._check(self.cu.cuInit(0), "cuInit")
        dev = C.c_int()
        self._check(self.cu.cuDeviceGet(C.byref(dev), device), "cuDeviceGet")
        self.dev = dev
        ctx = C.c_void_p()
        self._check(self.cu.cuDevicePrimaryCtxRetain(C.byref(ctx), dev), "cuDevicePrimaryCtxRetain")
        self.ctx = ctx
        self._check(self.cu.cuCtxSetCurrent(ctx), "cuCtxSetCurrent")
        mod = C.c_void_p()
        image = CUBIN.read_bytes()
        self._image = C.create_string_buffer(image, len(image))
        self._check(self.cu.cuModuleLoadData(C.byref(mod), self._image), "cuModuleLoadData")
        self.mod = mod
        self.fn = {}
        for key, name in KERNELS.items():
            f = C.c_void_p()
            self._check(self.cu.cuModuleGetFunction(C.byref(f), mod, name.encode()), f"cuModuleGetFunction {name}")
            self.fn[key] = f
        self.cu.cuLaunchKernel.argtypes = [C.c_void_p, C.c_uint, C.c_uint, C.c_uint, C.c_uint, C.c_uint, C.c_uint,
                                           C.c_uint, C.c_void_p, C.POINTER(C.c_void_p), C.POINTER(C.c_void_p)]

    def _check(self, r: int, what: str):
        if r != 0:
            s = C.c_char_p()
            try:
                self.cu.cuGetErrorString(r, C.byref(s))
            except Exception:  # pragma: no cover
                pass
            raise DriverError(f"{what}: CUDA driver error {r} ({s.value.decode() if s.value else '?'})")

    def launch(self, key: str, grid: int, args, stream: int):
        held = []
        for a in args:
            held.append(C.c_void_p(a) if isinstance(a, _Ptr) else C.c_uint32(int(a)))
        params = (C.c_void_p * len(held))(*[C.cast(C.pointer(h), C.c_void_p) for h in held])
        self._check(self.cu.cuLaunchKernel(self.fn[key], int(grid), 1, 1, BLOCK, 1, 1, 0, C.c_void_p(stream),
                                           params, None), f"launch {key}")

    def close(self):
        if self.mod:
            self.cu.cuModuleUnload(self.mod)
            self.mod = None
        if self.ctx:
            self.cu.cuDevicePrimaryCtxRelease(self.dev)
            self.ctx = None


class _Ptr(int):
    """A device address passed as a pointer argument."""


def _ptr(t) -> _Ptr:
    return _Ptr(t.data_ptr())


class ReferenceCudaMLEM:
    """The reference's MLEM loop at one GPU on host CSR inputs.

    A: (rowptr, col, val) with rows and nnz below 2**32 (the reference keeps
    32-bit row pointers on the device); AT: the transpose in the same layout
    (sptrans output), needed by the transposed modes."""

    def __init__(self, A, cols: int, AT=None, device: int = 0):
        import torch
        if not available():
            raise FileNotFoundError(f"{CUBIN} is missing (built where the reference sources are)")
        self.torch = torch
        torch.cuda.set_device(device)
        torch.zeros(1, device="cuda")
        self.drv = _Driver(device)
        rp, col, val = A
        self.rows, self.cols, self.nnz = len(rp) - 1, int(cols), len(col)
        if self.nnz >= 2**32 or self.rows >= 2**32:
            raise ValueError("the reference's device CSR holds 32-bit row pointers")

        def up(a, dt):
            return torch.from_numpy(np.ascontiguousarray(a).astype(dt, copy=False).view(np.int32)).cuda()

        self.A = (up(rp, np.uint32), up(col, np.uint32), up(val, np.float32))
        self.AT = None
        if AT is not None:
            cp, ri, vt = AT
            self.AT = (up(cp, np.uint32), up(ri, np.uint32), up(vt, np.float32))
        dev = "cuda"
        self.temp = torch.zeros(self.rows, dtype=torch.float32, device=dev)
        self.bwproj = torch.zeros(self.cols, dtype=torch.float32, device=dev)
        self.f = torch.zeros(self.cols, dtype=torch.float32, device=dev)
        self.g = torch.zeros(self.rows, dtype=torch.int32, device=dev)
        self.norm = torch.zeros(self.cols, dtype=torch.float32, device=dev)

    def close(self):
        self.drv.close()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def csr_vector_ok(self, using_trans: int) -> bool:
        ok = self.rows % 32 == 0
        if using_trans == 0:
            ok = ok and self.cols % 32 == 0
        return ok

    def load(self, g, norm, f0):
        torch = self.torch
        self.g.copy_(torch.from_numpy(np.ascontiguousarray(g, np.int32)))
        self.norm.copy_(torch.from_numpy(np.ascontiguousarray(norm, np.float32)))
        self.f.copy_(torch.from_numpy(np.ascontiguousarray(f0, np.float32)))
        self.temp.zero_()
        self.bwproj.zero_()
        torch.cuda.synchronize()

    def iterate(self, iterations: int, spmv: int = 1, using_trans: int = 0, secsize_fp: int = 5,
                secsize_bp: int = 5, events=None):
        """Runs `iterations` MLEM steps on the loaded state (main.cu:329-449).

        events: optional list that receives (fp_start, fp_end, bp_start, bp_end)
        CUDA events of each iteration."""
        torch = self.torch
        if using_trans == 0 and self.AT is None:
            raise ValueError("transposed modes need AT")
        if spmv == 1 and not self.csr_vector_ok(using_trans):
            raise ValueError("csr-vector modes are launched only for row counts that are multiples of 32")
        s = torch.cuda.current_stream()
        h = s.cuda_stream
        rows, cols, nnz = self.rows, self.cols, self.nnz
        Ar, Ac, Av = (_ptr(t) for t in self.A)
        temp, bw, f, g, norm = _ptr(self.temp), _ptr(self.bwproj), _ptr(self.f), _ptr(self.g), _ptr(self.norm)
        if self.AT is not None:
            Tr, Tc, Tv = (_ptr(t) for t in self.AT)
        grid_correl = math.ceil(rows / BLOCK)
        grid_fp = math.ceil((rows + nnz) / (BLOCK * secsize_fp)) if spmv == 0 else math.ceil(rows / 32)
        if using_trans == 0:
            grid_update = math.ceil(cols / BLOCK)
            grid_bp = math.ceil((cols + nnz) / (BLOCK * secsize_bp)) if spmv == 0 else math.ceil(cols / 32)
        else:
            grid_update = math.ceil(cols / BLOCK)
            grid_bp = math.ceil(rows / 32)
        for _ in range(iterations):
            ev = [torch.cuda.Event(enable_timing=True) for _ in range(4)] if events is not None else None
            if ev:
                ev[0].record(s)
            if spmv == 0:
                self.drv.launch("fp_merge", grid_fp, (Ar, Ac, Av, f, temp, secsize_fp, rows, nnz), h)
            else:
                self.drv.launch("fp_csrvec", grid_fp, (Ar, Ac, Av, f, temp, rows), h)
            if ev:
                ev[1].record(s)
            self.drv.launch("correl", grid_correl, (g, temp, rows), h)
            if using_trans == 0:
                s.synchronize()  # AllReduce of temp over one rank + cudaStreamSynchronize
            if ev:
                ev[2].record(s)
            if using_trans == 0:
                if spmv == 0:
                    self.drv.launch("bp_merge", grid_bp, (Tr, Tc, Tv, temp, bw, secsize_bp, cols, nnz), h)
                else:
                    self.drv.launch("bp_csrvec", grid_bp, (Tr, Tc, Tv, temp, bw, cols), h)
            else:
                self.drv.launch("bp_none_trans", grid_bp, (Ar, Ac, Av, temp, bw, rows), h)
            if ev:
                ev[3].record(s)
            self.drv.launch("update", grid_update, (f, norm, bw, cols), h)
            self.f.copy_(self.bwproj)  # AllReduce(bwproj -> f) over one rank
            s.synchronize()
            self.bwproj.zero_()
            self.temp.zero_()
            if ev:
                events.append(ev)

    def run(self, g, norm, f0, iterations: int, **mode) -> np.ndarray:
        self.load(g, norm, f0)
        self.iterate(iterations, **mode)
        self.torch.cuda.synchronize()
        return self.f.cpu().numpy()

    def time(self, g, norm, f0, iterations: int, warmup: int = 1, **mode) -> dict:
        """Per-iteration wall time of the loop (host synchronisations included,
        as in the reference) and the mean FP / BP kernel times."""
        torch = self.torch
        self.load(g, norm, f0)
        self.iterate(warmup, **mode)
        torch.cuda.synchronize()
        events = []
        t0 = time.perf_counter()
        self.iterate(iterations, events=events, **mode)
        torch.cuda.synchronize()
        wall = (time.perf_counter() - t0) / iterations
        fp = float(np.mean([e[0].elapsed_time(e[1]) for e in events]))
        bp = float(np.mean([e[2].elapsed_time(e[3]) for e in events]))
        return {"ms_per_iteration": wall * 1e3, "iterations_per_s": 1.0 / wall, "fp_ms": fp, "bp_ms": bp}
