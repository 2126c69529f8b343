// spmv.cu — row-parallel projection kernels of the MLEM iteration.
//
//   forward projection + correlation   (calcFwProj_csr_vector + calcCorrel,
//                                        kernel.cu:118-130, 297-336, 11-19)
//   back projection over Aᵀ + update   (calcBwProj_csr_vector + calcUpdate,
//                                        kernel.cu:141-153, 28-39)
//   scatter back projection over A     (calcBwProj_none_trans, kernel.cu:165-177, 347-370)
//   fused single pass FP+correl+scatter (no reference counterpart; same arithmetic)
//
// Design: a group of LPR lanes owns one row; each lane streams aligned 16-byte
// vectors of column indices and values (4 elements per vector, the row head
// and tail are masked), gathers x[col] through the read-only path, accumulates
// with FMA in FP32 and the group reduces with a fixed xor butterfly, so every
// row sum has one deterministic order.  The correlation and the multiplicative
// update are applied by the group leader in the same kernel, so an MLEM
// iteration is two launches and never needs a memset.
#include "kernels.cuh"
#include "scatter.cuh"

#include <algorithm>
#include <map>
#include <mutex>

namespace mlem {

namespace {

__device__ __forceinline__ bool in_row(uint64_t e, uint64_t s, uint64_t t) { return e >= s && e < t; }

template <typename V>
struct Vec4 {
    uint4 c;
    float a[4];
    __device__ __forceinline__ void load(const uint4* idx4, const V* val, uint64_t v) {
        c = ld_cached(idx4 + v);
        Val4<V>::load_cached(val, v, a);
    }
};

// Gathers for one 4-element vector (masked), then the FMAs in element order.
__device__ __forceinline__ void gather4(const uint4& c, uint64_t base, uint64_t s, uint64_t t,
                                        const float* __restrict__ x, float g[4]) {
    g[0] = in_row(base + 0, s, t) ? __ldg(x + c.x) : 0.f;
    g[1] = in_row(base + 1, s, t) ? __ldg(x + c.y) : 0.f;
    g[2] = in_row(base + 2, s, t) ? __ldg(x + c.z) : 0.f;
    g[3] = in_row(base + 3, s, t) ? __ldg(x + c.w) : 0.f;
}

__device__ __forceinline__ float fma4(float acc, const float a[4], const float g[4], uint64_t base,
                                      uint64_t s, uint64_t t) {
#pragma unroll
    for (int k = 0; k < 4; ++k)
        if (in_row(base + k, s, t)) acc = fmaf(a[k], g[k], acc);
    return acc;
}

// Dot product of row [s, t) with x by one lane of an LPR-lane group; U
// vectors of 4 elements are loaded before their gathers are consumed.
template <typename V, int LPR, int U = 2>
__device__ __forceinline__ float lane_dot(const uint32_t* __restrict__ idx, const V* __restrict__ val,
                                          const float* __restrict__ x, uint64_t s, uint64_t t, int sub) {
    const uint4* idx4 = reinterpret_cast<const uint4*>(idx);
    const uint64_t v1 = (t + 3) >> 2;
    uint64_t v = (s >> 2) + sub;
    float acc = 0.f;
    for (; v + (U - 1) * LPR < v1; v += U * LPR) {
        Vec4<V> p[U];
#pragma unroll
        for (int q = 0; q < U; ++q) p[q].load(idx4, val, v + q * LPR);
        float gq[U][4];
#pragma unroll
        for (int q = 0; q < U; ++q) gather4(p[q].c, (v + q * LPR) << 2, s, t, x, gq[q]);
#pragma unroll
        for (int q = 0; q < U; ++q) acc = fma4(acc, p[q].a, gq[q], (v + q * LPR) << 2, s, t);
    }
    for (; v < v1; v += LPR) {
        Vec4<V> p;
        p.load(idx4, val, v);
        float gp[4];
        gather4(p.c, v << 2, s, t, x, gp);
        acc = fma4(acc, p.a, gp, v << 2, s, t);
    }
    return acc;
}

template <typename V, int LPR, int U>
__device__ __forceinline__ void load_step(Vec4<V> (&p)[U], const uint4* __restrict__ idx4,
                                          const V* __restrict__ val, uint64_t b, uint64_t v1, int sub) {
#pragma unroll
    for (int q = 0; q < U; ++q) {
        const uint64_t v = b + sub + (uint64_t)q * LPR;
        if (v < v1) p[q].load(idx4, val, v);
    }
}

// Software-pipelined form of lane_dot: the U vectors of the next step are
// loaded before the gathers of the current step, so the index/value stream
// stays in flight while the gathers wait.  Same per-lane order of additions
// as lane_dot (bit-identical results).
template <typename V, int LPR, int U>
__device__ __forceinline__ float lane_dot_pipe(const uint32_t* __restrict__ idx, const V* __restrict__ val,
                                               const float* __restrict__ x, uint64_t s, uint64_t t, int sub) {
    const uint4* idx4 = reinterpret_cast<const uint4*>(idx);
    const uint64_t v1 = (t + 3) >> 2;
    uint64_t b = s >> 2;
    Vec4<V> cur[U];
    load_step<V, LPR, U>(cur, idx4, val, b, v1, sub);
    float acc = 0.f;
    for (;;) {
        const bool last = b + (uint64_t)U * LPR >= v1;
        Vec4<V> nxt[U];
        if (!last) load_step<V, LPR, U>(nxt, idx4, val, b + (uint64_t)U * LPR, v1, sub);
        float gq[U][4];
#pragma unroll
        for (int q = 0; q < U; ++q) {
            const uint64_t v = b + sub + (uint64_t)q * LPR;
            if (v < v1) gather4(cur[q].c, v << 2, s, t, x, gq[q]);
        }
#pragma unroll
        for (int q = 0; q < U; ++q) {
            const uint64_t v = b + sub + (uint64_t)q * LPR;
            if (v < v1) acc = fma4(acc, cur[q].a, gq[q], v << 2, s, t);
        }
        if (last) break;
        b += (uint64_t)U * LPR;
#pragma unroll
        for (int q = 0; q < U; ++q) cur[q] = nxt[q];
    }
    return acc;
}

template <int LPR>
__device__ __forceinline__ float group_sum(float acc) {
#pragma unroll
    for (int o = LPR / 2; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    return acc;
}

// Epilogues (executed by the group leader only).
__device__ __forceinline__ void epi_correl(uint32_t r, float sum, const int32_t* __restrict__ g,
                                           float* __restrict__ ratio, float* __restrict__ fwproj) {
    // calcCorrel (kernel.cu:17-18): ratio stays 0 where the projection is 0.
    ratio[r] = (sum != 0.0f) ? __fdiv_rn((float)g[r], sum) : 0.0f;
    if (fwproj) fwproj[r] = sum;
}

__device__ __forceinline__ void epi_update(uint32_t c, float sum, float* __restrict__ f,
                                           const float* __restrict__ norm) {
    // calcUpdate (kernel.cu:34-37): f * bp / norm, evaluated left to right.
    const float t = __fmul_rn(f[c], sum);
    const float n = norm[c];
    f[c] = (n == 0.0f) ? t : __fdiv_rn(t, n);
}

template <typename V, int LPR, int EPI, int U, bool ORD, bool PIPE>
__global__ void __launch_bounds__(256)
k_csrvec(const uint64_t* __restrict__ rowptr, const uint32_t* __restrict__ idx,
         const V* __restrict__ val, const float* __restrict__ x, uint32_t nrows,
         const int32_t* __restrict__ g, float* __restrict__ out, float* __restrict__ fwproj,
         float* __restrict__ f, const float* __restrict__ norm, const uint32_t* __restrict__ order) {
    const uint32_t gt = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t k = gt / LPR;
    const int sub = threadIdx.x & (LPR - 1);
    float acc = 0.f;
    uint32_t row = k;
    if (k < nrows) {
        if (ORD) row = __ldg(order + k);
        const uint64_t s = rowptr[row], t = rowptr[row + 1];
        acc = PIPE ? lane_dot_pipe<V, LPR, U>(idx, val, x, s, t, sub) : lane_dot<V, LPR, U>(idx, val, x, s, t, sub);
    }
    acc = group_sum<LPR>(acc);
    if (sub == 0 && k < nrows) {
        if (EPI == (int)Epi::Correl) epi_correl(row, acc, g, out, fwproj);
        else if (EPI == (int)Epi::Update) epi_update(row, acc, f, norm);
        else out[row] = acc;
    }
}

// Persistent, software-pipelined variant.  The grid holds as many groups of
// LPR lanes as fit on the device; group k handles rows k, k+G, k+2G, ... (or
// order[k], order[k+G], ... in locality order).  A step is U vectors per
// lane; the index/value vectors of step i+1 (of the same row, or the first
// step of the group's next row, whose pointers were fetched one row ahead)
// are issued before the gathers of step i, so the HBM stream is in flight
// while the gathers wait on L2.  Each lane accumulates its vectors
// v = (s>>2)+sub, +LPR, +2*LPR, ... in increasing order and the group reduces
// with the same xor butterfly as k_csrvec<V, LPR>: the results are
// bit-identical to that kernel for every U.
template <int LPR>
__device__ __forceinline__ float group_sum_masked(float acc, unsigned mask) {
#pragma unroll
    for (int o = LPR / 2; o > 0; o >>= 1) acc += __shfl_xor_sync(mask, acc, o);
    return acc;
}

template <typename V, int LPR, int EPI, int U, bool ORD>
__global__ void __launch_bounds__(256)
k_csrvec_pipe(const uint64_t* __restrict__ rowptr, const uint32_t* __restrict__ idx,
              const V* __restrict__ val, const float* __restrict__ x, uint32_t nrows,
              const int32_t* __restrict__ g, float* __restrict__ out, float* __restrict__ fwproj,
              float* __restrict__ f, const float* __restrict__ norm, const uint32_t* __restrict__ order) {
    const uint32_t G = (gridDim.x * blockDim.x) / LPR;
    uint32_t k = (blockIdx.x * blockDim.x + threadIdx.x) / LPR;
    const int sub = threadIdx.x & (LPR - 1);
    const unsigned mask = LPR == 32 ? 0xffffffffu : (((1u << LPR) - 1u) << ((threadIdx.x & 31) & ~(LPR - 1)));
    if (k >= nrows) return;  // group-uniform
    const uint4* idx4 = reinterpret_cast<const uint4*>(idx);
    uint32_t row = ORD ? __ldg(order + k) : k;
    uint64_t s = rowptr[row], t = rowptr[row + 1];
    uint32_t kn = k + G, nrow = 0;
    uint64_t ns = 0, nt = 0;
    if (kn < nrows) {
        nrow = ORD ? __ldg(order + kn) : kn;
        ns = rowptr[nrow];
        nt = rowptr[nrow + 1];
    }
    uint64_t b = s >> 2, v1 = (t + 3) >> 2;
    Vec4<V> cur[U];
    load_step<V, LPR, U>(cur, idx4, val, b, v1, sub);
    float acc = 0.f;
    for (;;) {
        const bool last = b + (uint64_t)U * LPR >= v1;  // no vector of this row after this step
        const bool more = !last || kn < nrows;
        const uint64_t nb = last ? (ns >> 2) : b + (uint64_t)U * LPR;
        const uint64_t nv1 = last ? ((nt + 3) >> 2) : v1;
        Vec4<V> nxt[U];
        if (more) load_step<V, LPR, U>(nxt, idx4, val, nb, nv1, sub);
        float gq[U][4];
#pragma unroll
        for (int q = 0; q < U; ++q) {
            const uint64_t v = b + sub + (uint64_t)q * LPR;
            if (v < v1) gather4(cur[q].c, v << 2, s, t, x, gq[q]);
        }
#pragma unroll
        for (int q = 0; q < U; ++q) {
            const uint64_t v = b + sub + (uint64_t)q * LPR;
            if (v < v1) acc = fma4(acc, cur[q].a, gq[q], v << 2, s, t);
        }
        if (last) {
            acc = group_sum_masked<LPR>(acc, mask);
            if (sub == 0) {
                if (EPI == (int)Epi::Correl) epi_correl(row, acc, g, out, fwproj);
                else if (EPI == (int)Epi::Update) epi_update(row, acc, f, norm);
                else out[row] = acc;
            }
            acc = 0.f;
            if (!more) break;
            k = kn;
            row = nrow;
            s = ns;
            t = nt;
            kn = k + G;
            if (kn < nrows) {
                nrow = ORD ? __ldg(order + kn) : kn;
                ns = rowptr[nrow];
                nt = rowptr[nrow + 1];
            }
        }
        b = nb;
        v1 = nv1;
#pragma unroll
        for (int q = 0; q < U; ++q) cur[q] = nxt[q];
    }
}

// Scatters the products p[k] of four consecutive entries of a row (those
// with base + k in [s, t)) into bp (vector reductions, scatter.cuh).
__device__ __forceinline__ void scatter4(float* __restrict__ bp, uint32_t ncols, const uint4& c, const float p[4],
                                         uint64_t base, uint64_t s, uint64_t t) {
    unsigned use = 0;
#pragma unroll
    for (int k = 0; k < 4; ++k)
        if (in_row(base + k, s, t)) use |= 1u << k;
    scatter4_mask(bp, ncols, c, p, use);
}

// LPR lanes per row of A; each lane loads U 16-byte vectors of (column,
// value) before it scatters them (U loads per lane in flight).
template <typename V, int LPR, int U>
__global__ void __launch_bounds__(256)
k_scatter(const uint64_t* __restrict__ rowptr, const uint32_t* __restrict__ idx,
          const V* __restrict__ val, const float* __restrict__ ratio, uint32_t nrows,
          float* __restrict__ bp, uint32_t ncols) {
    const uint32_t gt = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t row = gt / LPR;
    const int sub = threadIdx.x & (LPR - 1);
    if (row >= nrows) return;
    // the ratio and the row bounds are loaded together (one round trip, not two)
    const float r = ratio[row];
    const uint64_t s = rowptr[row], t = rowptr[row + 1];
    if (r == 0.0f) return;  // adds of val*0 leave bp unchanged
    const uint4* idx4 = reinterpret_cast<const uint4*>(idx);
    const uint64_t v1 = (t + 3) >> 2;
    for (uint64_t v = (s >> 2) + sub; v < v1; v += (uint64_t)LPR * U) {
        Vec4<V> p[U];
#pragma unroll
        for (int u = 0; u < U; ++u)
            if (v + (uint64_t)u * LPR < v1) p[u].load(idx4, val, v + (uint64_t)u * LPR);
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const uint64_t vu = v + (uint64_t)u * LPR;
            if (vu < v1) {
                float prod[4];
#pragma unroll
                for (int k = 0; k < 4; ++k) prod[k] = __fmul_rn(p[u].a[k], r);
                scatter4(bp, ncols, p[u].c, prod, vu << 2, s, t);
            }
        }
    }
}

// One warp per row of A: the row's vectors stay in registers between the
// forward dot product and the scatter (rows longer than 512 elements re-read
// their tail, which is then L2-resident).
template <typename V>
__global__ void __launch_bounds__(256)
k_fused(const uint64_t* __restrict__ rowptr, const uint32_t* __restrict__ idx,
        const V* __restrict__ val, const float* __restrict__ x, const int32_t* __restrict__ g,
        uint32_t nrows, float* __restrict__ bp, float* __restrict__ fwproj, uint32_t ncols) {
    constexpr int Q = 4;
    const uint32_t row = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (row >= nrows) return;  // whole warp leaves together
    const uint64_t s = rowptr[row], t = rowptr[row + 1];
    const uint4* idx4 = reinterpret_cast<const uint4*>(idx);
    const uint64_t v0 = s >> 2, v1 = (t + 3) >> 2;
    Vec4<V> keep[Q];
    float gth[Q][4];
    float acc = 0.f;
#pragma unroll
    for (int q = 0; q < Q; ++q) {
        const uint64_t v = v0 + lane + 32 * q;
        if (v < v1) {
            keep[q].load(idx4, val, v);
            gather4(keep[q].c, v << 2, s, t, x, gth[q]);
        }
    }
#pragma unroll
    for (int q = 0; q < Q; ++q) {
        const uint64_t v = v0 + lane + 32 * q;
        if (v < v1) acc = fma4(acc, keep[q].a, gth[q], v << 2, s, t);
    }
    for (uint64_t v = v0 + lane + 32 * Q; v < v1; v += 32) {
        Vec4<V> p;
        p.load(idx4, val, v);
        float gp[4];
        gather4(p.c, v << 2, s, t, x, gp);
        acc = fma4(acc, p.a, gp, v << 2, s, t);
    }
    acc = group_sum<32>(acc);
    if (fwproj && lane == 0) fwproj[row] = acc;
    if (acc == 0.0f) return;
    const float r = __fdiv_rn((float)g[row], acc);
    if (r == 0.0f) return;
#pragma unroll
    for (int q = 0; q < Q; ++q) {
        const uint64_t v = v0 + lane + 32 * q;
        if (v < v1) {
            float prod[4];
#pragma unroll
            for (int k = 0; k < 4; ++k) prod[k] = __fmul_rn(keep[q].a[k], r);
            scatter4(bp, ncols, keep[q].c, prod, v << 2, s, t);
        }
    }
    for (uint64_t v = v0 + lane + 32 * Q; v < v1; v += 32) {
        Vec4<V> p;
        p.load(idx4, val, v);
        float prod[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) prod[k] = __fmul_rn(p.a[k], r);
        scatter4(bp, ncols, p.c, prod, v << 2, s, t);
    }
}

// Fused single pass at the occupancy of the projection kernels: a group of
// LPR lanes per row sums the row exactly as k_csrvec<V, LPR, U> does (same
// order of additions), computes the ratio, then walks the row a second time
// (its vectors were streamed a moment before, so L2 serves them) and
// scatters val * ratio with the grouped vector reductions.  A crosses HBM
// once per iteration.
template <typename V, int LPR, int U, bool ORD>
__global__ void __launch_bounds__(256)
k_fused_rescan(const uint64_t* __restrict__ rowptr, const uint32_t* __restrict__ idx,
               const V* __restrict__ val, const float* __restrict__ x, uint32_t nrows,
               const int32_t* __restrict__ g, float* __restrict__ bp, float* __restrict__ fwproj,
               uint32_t ncols, const uint32_t* __restrict__ order) {
    const uint32_t gt = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t k = gt / LPR;
    const int sub = threadIdx.x & (LPR - 1);
    float acc = 0.f;
    uint32_t row = k;
    uint64_t s = 0, t = 0;
    int32_t gr = 0;
    if (k < nrows) {
        if (ORD) row = __ldg(order + k);
        s = rowptr[row];
        t = rowptr[row + 1];
        gr = g[row];
        acc = lane_dot<V, LPR, U>(idx, val, x, s, t, sub);
    }
    acc = group_sum<LPR>(acc);
    if (k >= nrows) return;
    if (sub == 0 && fwproj) fwproj[row] = acc;
    const float r = (acc != 0.0f) ? __fdiv_rn((float)gr, acc) : 0.0f;
    if (r == 0.0f) return;  // adds of val*0 leave bp unchanged
    const uint4* idx4 = reinterpret_cast<const uint4*>(idx);
    const uint64_t v1 = (t + 3) >> 2;
    for (uint64_t v = (s >> 2) + sub; v < v1; v += LPR) {
        Vec4<V> p;
        p.load(idx4, val, v);
        float prod[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) prod[q] = __fmul_rn(p.a[q], r);
        scatter4(bp, ncols, p.c, prod, v << 2, s, t);
    }
}

// calcUpdate (kernel.cu:34-37) for the scatter forms: f * bp / norm, left to right.
__device__ __forceinline__ float update_one(float f, float b, float nn) {
    const float t = __fmul_rn(f, b);
    return (nn == 0.0f) ? t : __fdiv_rn(t, nn);
}

__global__ void k_update_zero(float* __restrict__ f, float* __restrict__ bp,
                              const float* __restrict__ norm, uint32_t n) {
    for (uint32_t c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += gridDim.x * blockDim.x) {
        const float b = bp[c];
        bp[c] = 0.0f;
        f[c] = update_one(f[c], b, norm[c]);
    }
}

// Four columns per thread with 16-byte accesses (16-byte aligned arrays); the
// n % 4 last columns go to the first threads of block 0.  Same arithmetic.
__global__ void k_update_zero4(float* __restrict__ f, float* __restrict__ bp, const float* __restrict__ norm,
                               uint32_t n) {
    const uint32_t n4 = n >> 2;
    float4* f4 = reinterpret_cast<float4*>(f);
    float4* b4 = reinterpret_cast<float4*>(bp);
    const float4* m4 = reinterpret_cast<const float4*>(norm);
    for (uint32_t c = blockIdx.x * blockDim.x + threadIdx.x; c < n4; c += gridDim.x * blockDim.x) {
        const float4 b = b4[c];
        const float4 x = f4[c];
        const float4 nn = __ldg(m4 + c);
        b4[c] = make_float4(0.f, 0.f, 0.f, 0.f);
        f4[c] = make_float4(update_one(x.x, b.x, nn.x), update_one(x.y, b.y, nn.y), update_one(x.z, b.z, nn.z),
                            update_one(x.w, b.w, nn.w));
    }
    if (blockIdx.x == 0 && threadIdx.x < (n & 3u)) {
        const uint32_t c = (n4 << 2) + threadIdx.x;
        const float b = bp[c];
        bp[c] = 0.0f;
        f[c] = update_one(f[c], b, norm[c]);
    }
}

__device__ __forceinline__ double block_sum_f64(double v, double* sh) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0) sh[w] = v;
    __syncthreads();
    double tot = 0.0;
    if (threadIdx.x == 0)
        for (int i = 0; i < (int)(blockDim.x >> 5); ++i) tot += sh[i];
    return tot;
}

__global__ void __launch_bounds__(256)
k_loglik_part(const int32_t* __restrict__ g, const float* __restrict__ fp, uint32_t rows,
              double* __restrict__ part) {
    __shared__ double sh[8];
    double acc = 0.0;
    for (uint32_t r = blockIdx.x * blockDim.x + threadIdx.x; r < rows; r += gridDim.x * blockDim.x) {
        const double p = (double)fp[r];
        if (p > 0.0) acc += (g[r] > 0 ? (double)g[r] * log(p) : 0.0) - p;
    }
    const double tot = block_sum_f64(acc, sh);
    if (threadIdx.x == 0) part[blockIdx.x] = tot;
}

__global__ void __launch_bounds__(1024) k_reduce_f64(const double* __restrict__ part, int n,
                                                     double* __restrict__ out) {
    __shared__ double sh[32];
    double v = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) v += part[i];
    const double tot = block_sum_f64(v, sh);
    if (threadIdx.x == 0) *out = tot;
}

template <typename V, int LPR, int U, bool ORD, bool PIPE>
void csrvec_dispatch_epi(const DevCsr& op, const float* x, const EpiArgs& e, L2Window win,
                         cudaStream_t s) {
    const uint64_t threads = (uint64_t)op.nrows * LPR;
    const dim3 grid(ceil_div_u(threads, 256)), block(256);
    const V* val = static_cast<const V*>(op.val);
    const uint32_t* ord = op.order;
    switch (e.kind) {
        case Epi::Correl:
            launch_ex(k_csrvec<V, LPR, (int)Epi::Correl, U, ORD, PIPE>, grid, block, 0, s, win, op.rowptr, op.idx,
                      val, x, op.nrows, e.g, e.out, e.fwproj, (float*)nullptr, (const float*)nullptr, ord);
            break;
        case Epi::Update:
            launch_ex(k_csrvec<V, LPR, (int)Epi::Update, U, ORD, PIPE>, grid, block, 0, s, win, op.rowptr, op.idx,
                      val, x, op.nrows, (const int32_t*)nullptr, (float*)nullptr, (float*)nullptr,
                      e.f, e.norm, ord);
            break;
        default:
            launch_ex(k_csrvec<V, LPR, (int)Epi::Raw, U, ORD, PIPE>, grid, block, 0, s, win, op.rowptr, op.idx,
                      val, x, op.nrows, (const int32_t*)nullptr, e.out, (float*)nullptr,
                      (float*)nullptr, (const float*)nullptr, ord);
    }
}

template <typename V, int LPR, int EPI, int U, bool ORD>
unsigned pipe_grid() {
    static std::mutex mu;
    static std::map<int, unsigned> cache;
    int dev = 0;
    MLEM_CUDA(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lk(mu);
    auto it = cache.find(dev);
    if (it != cache.end()) return it->second;
    int per_sm = 0, sms = 0;
    MLEM_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_csrvec_pipe<V, LPR, EPI, U, ORD>, 256, 0));
    MLEM_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    return cache[dev] = (unsigned)std::max(1, per_sm) * (unsigned)sms;
}

template <typename V, int LPR, int EPI, int U, bool ORD>
void pipe_launch(const DevCsr& op, const float* x, const EpiArgs& e, L2Window win, cudaStream_t s) {
    const unsigned grid =
        std::min(pipe_grid<V, LPR, EPI, U, ORD>(), std::max(1u, ceil_div_u((uint64_t)op.nrows * LPR, 256)));
    launch_ex(k_csrvec_pipe<V, LPR, EPI, U, ORD>, dim3(grid), dim3(256), 0, s, win, op.rowptr, op.idx,
              static_cast<const V*>(op.val), x, op.nrows, e.g, e.out, e.fwproj, e.f, e.norm,
              (const uint32_t*)op.order);
}

// kind: 0 = launch, 1 = settle the grid size only (outside stream captures).
template <typename V, int LPR, int U, bool ORD>
void pipe_epi(int kind, const DevCsr* op, const float* x, const EpiArgs* e, L2Window win, cudaStream_t s) {
    if (kind == 1) {
        pipe_grid<V, LPR, (int)Epi::Correl, U, ORD>();
        pipe_grid<V, LPR, (int)Epi::Update, U, ORD>();
        pipe_grid<V, LPR, (int)Epi::Raw, U, ORD>();
        return;
    }
    switch (e->kind) {
        case Epi::Correl: pipe_launch<V, LPR, (int)Epi::Correl, U, ORD>(*op, x, *e, win, s); break;
        case Epi::Update: pipe_launch<V, LPR, (int)Epi::Update, U, ORD>(*op, x, *e, win, s); break;
        default: pipe_launch<V, LPR, (int)Epi::Raw, U, ORD>(*op, x, *e, win, s);
    }
}

template <typename V, int LPR>
void pipe_u(int kind, const DevCsr* op, const float* x, const EpiArgs* e, int unroll, bool ordered, L2Window win,
            cudaStream_t s) {
    if (ordered) {
        if (unroll >= 2) pipe_epi<V, LPR, 2, true>(kind, op, x, e, win, s);
        else pipe_epi<V, LPR, 1, true>(kind, op, x, e, win, s);
    } else {
        if (unroll >= 2) pipe_epi<V, LPR, 2, false>(kind, op, x, e, win, s);
        else pipe_epi<V, LPR, 1, false>(kind, op, x, e, win, s);
    }
}

template <typename V>
void pipe_lanes(int kind, const DevCsr* op, const float* x, const EpiArgs* e, int lanes, int unroll, bool ordered,
                L2Window win, cudaStream_t s) {
    if (lanes >= 32) pipe_u<V, 32>(kind, op, x, e, unroll, ordered, win, s);
    else pipe_u<V, 16>(kind, op, x, e, unroll, ordered, win, s);
}

template <typename V, int LPR>
void csrvec_dispatch_u(const DevCsr& op, const float* x, const EpiArgs& e, int unroll, bool ordered, bool pipelined,
                       L2Window win, cudaStream_t s) {
    if constexpr (LPR >= 16) {
        const bool ord = ordered && op.order;
        if (pipelined) {
            if (ord) {
                if (unroll >= 2) csrvec_dispatch_epi<V, LPR, 2, true, true>(op, x, e, win, s);
                else csrvec_dispatch_epi<V, LPR, 1, true, true>(op, x, e, win, s);
            } else {
                if (unroll >= 2) csrvec_dispatch_epi<V, LPR, 2, false, true>(op, x, e, win, s);
                else csrvec_dispatch_epi<V, LPR, 1, false, true>(op, x, e, win, s);
            }
            return;
        }
        if (ord) {
            if (unroll >= 2) csrvec_dispatch_epi<V, LPR, 2, true, false>(op, x, e, win, s);
            else csrvec_dispatch_epi<V, LPR, 1, true, false>(op, x, e, win, s);
            return;
        }
    }
    if (unroll >= 4) csrvec_dispatch_epi<V, LPR, 4, false, false>(op, x, e, win, s);
    else if (unroll == 2) csrvec_dispatch_epi<V, LPR, 2, false, false>(op, x, e, win, s);
    else csrvec_dispatch_epi<V, LPR, 1, false, false>(op, x, e, win, s);
}

template <typename V>
void csrvec_dispatch_lanes(const DevCsr& op, const float* x, const EpiArgs& e, int lanes, int unroll,
                           bool ordered, bool pipelined, L2Window win, cudaStream_t s) {
    if (lanes >= 32) csrvec_dispatch_u<V, 32>(op, x, e, unroll, ordered, pipelined, win, s);
    else if (lanes >= 16) csrvec_dispatch_u<V, 16>(op, x, e, unroll, ordered, pipelined, win, s);
    else if (lanes >= 8) csrvec_dispatch_u<V, 8>(op, x, e, unroll, false, false, win, s);
    else csrvec_dispatch_u<V, 4>(op, x, e, unroll, false, false, win, s);
}

template <typename V>
void scatter_dispatch(const DevCsr& A, const float* ratio, float* bp, int lanes, int unroll, L2Window win,
                      cudaStream_t s) {
    const V* val = static_cast<const V*>(A.val);
    auto go = [&](auto kern, int lpr) {
        const uint64_t threads = (uint64_t)A.nrows * lpr;
        launch_ex(kern, dim3(ceil_div_u(threads, 256)), dim3(256), 0, s, win, A.rowptr, A.idx, val,
                  ratio, A.nrows, bp, A.ncols);
    };
    if (unroll >= 2) {
        if (lanes >= 32) go(k_scatter<V, 32, 2>, 32);
        else if (lanes >= 16) go(k_scatter<V, 16, 2>, 16);
        else go(k_scatter<V, 8, 2>, 8);
    } else {
        if (lanes >= 32) go(k_scatter<V, 32, 1>, 32);
        else if (lanes >= 16) go(k_scatter<V, 16, 1>, 16);
        else go(k_scatter<V, 8, 1>, 8);
    }
}

}  // namespace

int pick_lanes(uint64_t nnz, uint32_t rows) {
    const double mean = rows ? (double)nnz / rows : 0.0;
    if (mean >= 96.0) return 32;
    if (mean >= 40.0) return 16;
    if (mean >= 12.0) return 8;
    return 4;
}

void launch_csrvec(const DevCsr& op, const float* x, const EpiArgs& epi, int lanes, L2Window win,
                   cudaStream_t s, int unroll, bool ordered, bool pipelined) {
    if (op.nrows == 0) return;
    switch (op.vt) {
        case MLEM_VAL_F32: csrvec_dispatch_lanes<float>(op, x, epi, lanes, unroll, ordered, pipelined, win, s); break;
        case MLEM_VAL_F16:
            csrvec_dispatch_lanes<__half>(op, x, epi, lanes, unroll, ordered, pipelined, win, s);
            break;
        default: csrvec_dispatch_lanes<__nv_bfloat16>(op, x, epi, lanes, unroll, ordered, pipelined, win, s);
    }
}

void prepare_csrvec_pipe(mlem_value_type vt) {
    for (int lanes : {16, 32})
        for (int u : {1, 2})
            for (bool ord : {false, true}) {
                switch (vt) {
                    case MLEM_VAL_F32: pipe_lanes<float>(1, nullptr, nullptr, nullptr, lanes, u, ord, {}, 0); break;
                    case MLEM_VAL_F16: pipe_lanes<__half>(1, nullptr, nullptr, nullptr, lanes, u, ord, {}, 0); break;
                    default: pipe_lanes<__nv_bfloat16>(1, nullptr, nullptr, nullptr, lanes, u, ord, {}, 0);
                }
            }
}

void launch_csrvec_pipe(const DevCsr& op, const float* x, const EpiArgs& epi, int lanes, int unroll, bool ordered,
                        L2Window win, cudaStream_t s) {
    if (op.nrows == 0) return;
    MLEM_REQUIRE(lanes == 16 || lanes == 32, MLEM_EINVAL, "pipelined projection needs 16 or 32 lanes per row");
    MLEM_REQUIRE(!ordered || op.order != nullptr, MLEM_EINVAL, "operand has no row order");
    switch (op.vt) {
        case MLEM_VAL_F32: pipe_lanes<float>(0, &op, x, &epi, lanes, unroll, ordered, win, s); break;
        case MLEM_VAL_F16: pipe_lanes<__half>(0, &op, x, &epi, lanes, unroll, ordered, win, s); break;
        default: pipe_lanes<__nv_bfloat16>(0, &op, x, &epi, lanes, unroll, ordered, win, s);
    }
}

void launch_scatter(const DevCsr& A, const float* ratio, float* bp, int lanes, int unroll, L2Window win,
                    cudaStream_t s) {
    if (A.nrows == 0) return;
    switch (A.vt) {
        case MLEM_VAL_F32: scatter_dispatch<float>(A, ratio, bp, lanes, unroll, win, s); break;
        case MLEM_VAL_F16: scatter_dispatch<__half>(A, ratio, bp, lanes, unroll, win, s); break;
        default: scatter_dispatch<__nv_bfloat16>(A, ratio, bp, lanes, unroll, win, s);
    }
}

void launch_fused_fp_scatter(const DevCsr& A, const float* x, const int32_t* g, float* bp,
                             float* fwproj, L2Window win, cudaStream_t s) {
    if (A.nrows == 0) return;
    const dim3 grid(ceil_div_u((uint64_t)A.nrows * 32, 256)), block(256);
    switch (A.vt) {
        case MLEM_VAL_F32:
            launch_ex(k_fused<float>, grid, block, 0, s, win, A.rowptr, A.idx,
                      (const float*)A.val, x, g, A.nrows, bp, fwproj, A.ncols);
            break;
        case MLEM_VAL_F16:
            launch_ex(k_fused<__half>, grid, block, 0, s, win, A.rowptr, A.idx,
                      (const __half*)A.val, x, g, A.nrows, bp, fwproj, A.ncols);
            break;
        default:
            launch_ex(k_fused<__nv_bfloat16>, grid, block, 0, s, win, A.rowptr, A.idx,
                      (const __nv_bfloat16*)A.val, x, g, A.nrows, bp, fwproj, A.ncols);
    }
}

namespace {
template <typename V, int LPR, int U>
void rescan_ord(const DevCsr& A, const float* x, const int32_t* g, float* bp, float* fwproj, bool ordered,
                L2Window win, cudaStream_t s) {
    const dim3 grid(ceil_div_u((uint64_t)A.nrows * LPR, 256)), block(256);
    const V* val = static_cast<const V*>(A.val);
    if (ordered)
        launch_ex(k_fused_rescan<V, LPR, U, true>, grid, block, 0, s, win, A.rowptr, A.idx, val, x, A.nrows, g, bp,
                  fwproj, A.ncols, (const uint32_t*)A.order);
    else
        launch_ex(k_fused_rescan<V, LPR, U, false>, grid, block, 0, s, win, A.rowptr, A.idx, val, x, A.nrows, g, bp,
                  fwproj, A.ncols, (const uint32_t*)nullptr);
}
template <typename V>
void rescan_cfg(const DevCsr& A, const float* x, const int32_t* g, float* bp, float* fwproj, int lanes, int unroll,
                bool ordered, L2Window win, cudaStream_t s) {
    if (lanes >= 32) {
        if (unroll >= 2) rescan_ord<V, 32, 2>(A, x, g, bp, fwproj, ordered, win, s);
        else rescan_ord<V, 32, 1>(A, x, g, bp, fwproj, ordered, win, s);
    } else if (lanes >= 16) {
        if (unroll >= 2) rescan_ord<V, 16, 2>(A, x, g, bp, fwproj, ordered, win, s);
        else rescan_ord<V, 16, 1>(A, x, g, bp, fwproj, ordered, win, s);
    } else {
        if (unroll >= 2) rescan_ord<V, 8, 2>(A, x, g, bp, fwproj, ordered, win, s);
        else rescan_ord<V, 8, 1>(A, x, g, bp, fwproj, ordered, win, s);
    }
}
}  // namespace

void launch_fused_rescan(const DevCsr& A, const float* x, const int32_t* g, float* bp, float* fwproj, int lanes,
                         int unroll, bool ordered, L2Window win, cudaStream_t s) {
    if (A.nrows == 0) return;
    MLEM_REQUIRE(!ordered || A.order != nullptr, MLEM_EINVAL, "operand has no row order");
    switch (A.vt) {
        case MLEM_VAL_F32: rescan_cfg<float>(A, x, g, bp, fwproj, lanes, unroll, ordered, win, s); break;
        case MLEM_VAL_F16: rescan_cfg<__half>(A, x, g, bp, fwproj, lanes, unroll, ordered, win, s); break;
        default: rescan_cfg<__nv_bfloat16>(A, x, g, bp, fwproj, lanes, unroll, ordered, win, s);
    }
}

void launch_update_zero(float* f, float* bp, const float* norm, uint32_t n, cudaStream_t s) {
    if (n == 0) return;
    const bool aligned = ((reinterpret_cast<uintptr_t>(f) | reinterpret_cast<uintptr_t>(bp) |
                           reinterpret_cast<uintptr_t>(norm)) & 15u) == 0;
    if (aligned) {
        const unsigned grid = std::max(1u, std::min<unsigned>(ceil_div_u(n >> 2, 256), 152u * 16u));
        k_update_zero4<<<grid, 256, 0, s>>>(f, bp, norm, n);
    } else {
        const unsigned grid = std::min<unsigned>(ceil_div_u(n, 256), 152u * 16u);
        k_update_zero<<<grid, 256, 0, s>>>(f, bp, norm, n);
    }
    MLEM_LAUNCHED();
}

void launch_loglik(const int32_t* g, const float* fwproj, uint32_t rows, double* part,
                   double* out, cudaStream_t s) {
    k_loglik_part<<<kLoglikParts, 256, 0, s>>>(g, fwproj, rows, part);
    MLEM_LAUNCHED();
    k_reduce_f64<<<1, 1024, 0, s>>>(part, kLoglikParts, out);
    MLEM_LAUNCHED();
}

}  // namespace mlem
