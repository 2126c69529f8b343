// loop.cu — whole MLEM iterations of a small (L2-resident) problem in one
// persistent cooperative launch.
//
// For a matrix whose operands fit in L2 (the 2-D ring scanner: 8 MB), an
// iteration's two projections take a few microseconds each and the launches
// around them dominate.  Here every iteration of a reconstruction runs inside
// one launch: the grid's lane groups stride over the rows of A (forward
// projection, calcCorrel, kernel.cu:11-19), pass a grid-wide barrier, stride
// over the rows of Aᵀ (back projection, calcUpdate, kernel.cu:28-39) and pass a
// second barrier, `iters` times.  Each row is summed exactly as the
// csr-vector kernel k_csrvec sums it for the same lanes per row and vectors in
// flight (lane l takes the 16-byte vectors l, l + L, ... of its row, U of them
// loaded before their gathers, FMAs in element order, a fixed xor butterfly
// over the group), so the images are bit-identical to the per-iteration path
// the autotuner configured.  The state gathered in one phase is written in the
// other, so the gathers use coherent loads, not the read-only path.  Every
// barrier wait is bounded (common.cuh: grid_barrier); a wait that runs out sets
// the workspace's error word, the launch ends and the host reports
// MLEM_ETIMEOUT.
#include "kernels.cuh"

#include <algorithm>

namespace mlem {

namespace {

__device__ __forceinline__ bool in_row_l(uint64_t e, uint64_t s, uint64_t t) { return e >= s && e < t; }

// Dot product of row [s, t) with x by lane `sub` of an lpr-lane group, in the
// order of k_csrvec's lane_dot<V, lpr, U>.
template <typename V, int U>
__device__ __forceinline__ float lane_dot_c(const uint32_t* __restrict__ idx, const V* __restrict__ val,
                                            const float* x, uint64_t s, uint64_t t, int sub, int lpr) {
    const uint4* idx4 = reinterpret_cast<const uint4*>(idx);
    const uint64_t v1 = (t + 3) >> 2;
    uint64_t v = (s >> 2) + sub;
    float acc = 0.f;
    for (; v + (uint64_t)(U - 1) * lpr < v1; v += (uint64_t)U * lpr) {
        uint4 c[U];
        float a[U][4], gq[U][4];
#pragma unroll
        for (int q = 0; q < U; ++q) {
            c[q] = __ldcs(idx4 + v + (uint64_t)q * lpr);
            Val4<V>::load(val, v + (uint64_t)q * lpr, a[q]);
        }
#pragma unroll
        for (int q = 0; q < U; ++q) {
            const uint64_t b = (v + (uint64_t)q * lpr) << 2;
            const uint32_t cs[4] = {c[q].x, c[q].y, c[q].z, c[q].w};
#pragma unroll
            for (int k = 0; k < 4; ++k) gq[q][k] = in_row_l(b + k, s, t) ? x[cs[k]] : 0.f;
        }
#pragma unroll
        for (int q = 0; q < U; ++q) {
            const uint64_t b = (v + (uint64_t)q * lpr) << 2;
#pragma unroll
            for (int k = 0; k < 4; ++k)
                if (in_row_l(b + k, s, t)) acc = fmaf(a[q][k], gq[q][k], acc);
        }
    }
    for (; v < v1; v += lpr) {
        const uint4 c = __ldcs(idx4 + v);
        float a[4], gp[4];
        Val4<V>::load(val, v, a);
        const uint64_t b = v << 2;
        const uint32_t cs[4] = {c.x, c.y, c.z, c.w};
#pragma unroll
        for (int k = 0; k < 4; ++k) gp[k] = in_row_l(b + k, s, t) ? x[cs[k]] : 0.f;
#pragma unroll
        for (int k = 0; k < 4; ++k)
            if (in_row_l(b + k, s, t)) acc = fmaf(a[k], gp[k], acc);
    }
    return acc;
}

// One projection over all rows of an operand by the grid's lane groups; the
// group leader applies the epilogue (CORREL: ratio = g / sum, zero guard;
// else the multiplicative update of f in place).
template <typename V, int U, bool CORREL>
__device__ __forceinline__ void loop_phase(const uint64_t* __restrict__ rp, const uint32_t* __restrict__ ix,
                                           const V* __restrict__ vl, uint32_t n, const float* x, int lpr,
                                           const int32_t* __restrict__ g, float* ratio, float* f,
                                           const float* __restrict__ norm) {
    const int lane = threadIdx.x & 31, sub = lane & (lpr - 1);
    const uint32_t gpw = 32u / (uint32_t)lpr;  // groups per warp
    const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t stride = ((gridDim.x * blockDim.x) >> 5) * gpw;
    for (uint32_t first = warp * gpw; first < n; first += stride) {  // warp-uniform
        const uint32_t row = first + (uint32_t)lane / (uint32_t)lpr;
        float acc = 0.f;
        if (row < n) acc = lane_dot_c<V, U>(ix, vl, x, rp[row], rp[row + 1], sub, lpr);
        for (int o = lpr / 2; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        if (row < n && sub == 0) {
            if (CORREL) {
                ratio[row] = (acc != 0.0f) ? __fdiv_rn((float)g[row], acc) : 0.0f;
            } else {
                const float t = __fmul_rn(f[row], acc);
                const float nn = norm[row];
                f[row] = (nn == 0.0f) ? t : __fdiv_rn(t, nn);
            }
        }
    }
}

template <typename V, int U>
__global__ void __launch_bounds__(256)
k_mlem_loop(const uint64_t* __restrict__ rp, const uint32_t* __restrict__ ix, const V* __restrict__ vl,
            uint32_t rows, int lpr_fp, const uint64_t* __restrict__ rpT, const uint32_t* __restrict__ ixT,
            const V* __restrict__ vlT, uint32_t cols, int lpr_bp, const int32_t* __restrict__ g, float* ratio,
            float* f, const float* __restrict__ norm, uint32_t iters, unsigned* count, int* err) {
    unsigned k = 0;
    for (uint32_t it = 0; it < iters; ++it) {
        loop_phase<V, U, true>(rp, ix, vl, rows, f, lpr_fp, g, ratio, f, norm);
        if (!grid_barrier(count, ++k, err)) return;
        loop_phase<V, U, false>(rpT, ixT, vlT, cols, ratio, lpr_bp, g, ratio, f, norm);
        if (!grid_barrier(count, ++k, err)) return;
    }
}

template <typename V, int U>
void loop_launch(const DevCsr& A, const DevCsr& AT, int lpr_fp, int lpr_bp, const int32_t* g, float* ratio,
                 float* f, const float* norm, uint32_t iters, unsigned* count, int* err, cudaStream_t s) {
    auto kern = k_mlem_loop<V, U>;
    static const int bps = [kern] {
        int b = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, kern, 256, 0) != cudaSuccess) {
            cudaGetLastError();
            b = 0;
        }
        return b;
    }();
    MLEM_REQUIRE(bps >= 1, MLEM_EUNSUPPORTED, "persistent MLEM loop does not fit on an SM");
    int dev = 0, sms = 0;
    MLEM_CUDA(cudaGetDevice(&dev));
    MLEM_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    // enough groups for the larger operand, at most half a resident wave, so
    // that two such launches on other streams fit beside each other
    const uint64_t need = std::max<uint64_t>((uint64_t)A.nrows * lpr_fp, (uint64_t)AT.nrows * lpr_bp);
    const unsigned cap = (unsigned)std::max(1, bps * sms / 2);
    const unsigned grid = (unsigned)std::max<uint64_t>(1, std::min<uint64_t>(cap, (need + 255) / 256));
    MLEM_CUDA(cudaMemsetAsync(count, 0, sizeof(unsigned), s));
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(256);
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    MLEM_CUDA(cudaLaunchKernelEx(&cfg, kern, (const uint64_t*)A.rowptr, (const uint32_t*)A.idx,
                                 static_cast<const V*>(A.val), A.nrows, lpr_fp, (const uint64_t*)AT.rowptr,
                                 (const uint32_t*)AT.idx, static_cast<const V*>(AT.val), AT.nrows, lpr_bp, g, ratio,
                                 f, norm, iters, count, err));
    count_launch();
}

template <typename V>
void loop_u(const DevCsr& A, const DevCsr& AT, int lpr_fp, int lpr_bp, int unroll, const int32_t* g, float* ratio,
            float* f, const float* norm, uint32_t iters, unsigned* count, int* err, cudaStream_t s) {
    switch (unroll) {
        case 1: loop_launch<V, 1>(A, AT, lpr_fp, lpr_bp, g, ratio, f, norm, iters, count, err, s); break;
        case 4: loop_launch<V, 4>(A, AT, lpr_fp, lpr_bp, g, ratio, f, norm, iters, count, err, s); break;
        default: loop_launch<V, 2>(A, AT, lpr_fp, lpr_bp, g, ratio, f, norm, iters, count, err, s);
    }
}

}  // namespace

void launch_mlem_loop(const DevCsr& A, const DevCsr& AT, int lanes_fp, int lanes_bp, int unroll, const int32_t* g,
                      float* ratio, float* f, const float* norm, uint32_t iters, unsigned* count, int* err,
                      cudaStream_t s) {
    if (iters == 0 || A.nrows == 0) return;
    MLEM_REQUIRE(A.vt == AT.vt, MLEM_EINVAL, "internal: operands of different value types");
    auto ok_lanes = [](int l) { return l == 4 || l == 8 || l == 16 || l == 32; };
    MLEM_REQUIRE(ok_lanes(lanes_fp) && ok_lanes(lanes_bp), MLEM_EINVAL, "internal: lanes per row must be 4..32");
    switch (A.vt) {
        case MLEM_VAL_F32: loop_u<float>(A, AT, lanes_fp, lanes_bp, unroll, g, ratio, f, norm, iters, count, err, s); break;
        case MLEM_VAL_F16: loop_u<__half>(A, AT, lanes_fp, lanes_bp, unroll, g, ratio, f, norm, iters, count, err, s); break;
        default: loop_u<__nv_bfloat16>(A, AT, lanes_fp, lanes_bp, unroll, g, ratio, f, norm, iters, count, err, s);
    }
}

}  // namespace mlem
