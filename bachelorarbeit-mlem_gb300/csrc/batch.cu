// batch.cu — many sinograms against one resident matrix (batched SpMM).
//
// The matrix stream is shared by a tile of BT instances (8, 16 or 32): one
// warp per row; the warp loads 32 (index, value) pairs with one coalesced
// access each, broadcasts them with shuffles, and each lane multiplies them
// against its instance's entry of the interleaved image f[col*BT + b] (one
// 4*BT-byte coalesced gather per nonzero).  With BT < 32, 32/BT lane groups
// take every (32/BT)-th nonzero and are combined by a fixed xor tree, so an
// instance's arithmetic depends only on BT, never on which other slots are
// occupied: an instance gives the same bits alone and in a full batch.
//
// Per-slot iteration counters live on the device (remaining[b]); an
// iteration is FP, BP+update and a counter tick, replayable as one CUDA
// graph until the longest slot finishes.
#include "kernels.cuh"

#include <algorithm>

namespace mlem {

namespace {

template <typename V, int BT>
__device__ __forceinline__ void batch_row(const uint32_t* __restrict__ idx, const V* __restrict__ val,
                                          const float* __restrict__ x, uint64_t s, uint64_t t,
                                          int lane, float& acc) {
    constexpr int G = 32 / BT;       // lane groups
    const int grp = lane / BT, b = lane % BT;
    for (uint64_t base = s; base < t; base += 32) {
        const uint64_t e = base + lane;
        uint32_t c = 0;
        float v = 0.f;
        if (e < t) {
            c = __ldcs(idx + e);
            v = Val4<V>::one(val, e);
        }
        // every lane runs the same trip count so the shuffles stay converged
        const int n = (t - base) > 32 ? 32 : (int)(t - base);
        const int trips = (n + G - 1) / G;
#pragma unroll 4
        for (int q = 0; q < trips; ++q) {
            const int k = q * G + grp;
            const uint32_t ck = __shfl_sync(0xffffffffu, c, k);
            const float vk = __shfl_sync(0xffffffffu, v, k);
            if (k < n) acc = fmaf(vk, __ldg(x + (uint64_t)ck * BT + b), acc);
        }
    }
#pragma unroll
    for (int o = BT; o < 32; o <<= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
}

template <typename V, int BT>
__global__ void __launch_bounds__(256)
k_batch_fp(const uint64_t* __restrict__ rowptr, const uint32_t* __restrict__ idx,
           const V* __restrict__ val, const float* __restrict__ f, uint32_t rows,
           const int32_t* __restrict__ g, float* __restrict__ ratio) {
    const uint32_t row = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (row >= rows) return;
    float acc = 0.f;
    batch_row<V, BT>(idx, val, f, rowptr[row], rowptr[row + 1], lane, acc);
    if (lane < BT) {
        const uint64_t o = (uint64_t)row * BT + lane;
        ratio[o] = (acc != 0.0f) ? __fdiv_rn((float)g[o], acc) : 0.0f;
    }
}

template <typename V, int BT>
__global__ void __launch_bounds__(256)
k_batch_bp(const uint64_t* __restrict__ rowptr, const uint32_t* __restrict__ idx,
           const V* __restrict__ val, const float* __restrict__ ratio, uint32_t cols,
           const float* __restrict__ norm, const uint32_t* __restrict__ remaining,
           float* __restrict__ f) {
    const uint32_t c = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (c >= cols) return;
    float acc = 0.f;
    batch_row<V, BT>(idx, val, ratio, rowptr[c], rowptr[c + 1], lane, acc);
    if (lane < BT && remaining[lane] > 0) {
        const uint64_t o = (uint64_t)c * BT + lane;
        const float t = __fmul_rn(f[o], acc);
        const float n = norm[c];
        f[o] = (n == 0.0f) ? t : __fdiv_rn(t, n);
    }
}

template <typename V, int BT>
__global__ void __launch_bounds__(256)
k_batch_scatter(const uint64_t* __restrict__ rowptr, const uint32_t* __restrict__ idx,
                const V* __restrict__ val, const float* __restrict__ ratio, uint32_t rows,
                float* __restrict__ bp) {
    constexpr int G = 32 / BT;
    const uint32_t row = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31, grp = lane / BT, b = lane % BT;
    if (row >= rows) return;
    const float r = ratio[(uint64_t)row * BT + b];
    const uint64_t s = rowptr[row], t = rowptr[row + 1];
    for (uint64_t base = s; base < t; base += 32) {
        const uint64_t e = base + lane;
        uint32_t c = 0;
        float v = 0.f;
        if (e < t) {
            c = __ldcs(idx + e);
            v = Val4<V>::one(val, e);
        }
        const int n = (t - base) > 32 ? 32 : (int)(t - base);
        const int trips = (n + G - 1) / G;
        for (int q = 0; q < trips; ++q) {
            const int k = q * G + grp;
            const uint32_t ck = __shfl_sync(0xffffffffu, c, k);
            const float vk = __shfl_sync(0xffffffffu, v, k);
            if (k < n && r != 0.0f) atomicAdd(bp + (uint64_t)ck * BT + b, __fmul_rn(vk, r));
        }
    }
}

__global__ void k_batch_update_zero(const float* __restrict__ norm, uint32_t cols, uint32_t BT,
                                    const uint32_t* __restrict__ remaining, float* __restrict__ f,
                                    float* __restrict__ bp) {
    const uint64_t n = (uint64_t)cols * BT;
    for (uint64_t o = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; o < n;
         o += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t c = (uint32_t)(o / BT), b = (uint32_t)(o % BT);
        const float acc = bp[o];
        bp[o] = 0.0f;
        if (remaining[b] > 0) {
            const float t = __fmul_rn(f[o], acc);
            const float nn = norm[c];
            f[o] = (nn == 0.0f) ? t : __fdiv_rn(t, nn);
        }
    }
}

__global__ void k_batch_tick(uint32_t* remaining, uint32_t BT) {
    if (threadIdx.x < BT && remaining[threadIdx.x] > 0) remaining[threadIdx.x] -= 1;
}

template <int BT, typename V>
void fp_bt(const DevCsr& A, const BatchArgs& b, L2Window win, cudaStream_t s) {
    launch_ex(k_batch_fp<V, BT>, dim3(ceil_div_u((uint64_t)A.nrows * 32, 256)), dim3(256), 0, s, win,
              A.rowptr, A.idx, static_cast<const V*>(A.val), (const float*)b.f, A.nrows, b.g, b.ratio);
}

template <int BT, typename V>
void bp_bt(const DevCsr& AT, const float* norm, const BatchArgs& b, L2Window win, cudaStream_t s) {
    launch_ex(k_batch_bp<V, BT>, dim3(ceil_div_u((uint64_t)AT.nrows * 32, 256)), dim3(256), 0, s, win,
              AT.rowptr, AT.idx, static_cast<const V*>(AT.val), (const float*)b.ratio, AT.nrows, norm,
              (const uint32_t*)b.remaining, b.f);
}

template <int BT, typename V>
void sc_bt(const DevCsr& A, const BatchArgs& b, float* bp, cudaStream_t s) {
    k_batch_scatter<V, BT><<<ceil_div_u((uint64_t)A.nrows * 32, 256), 256, 0, s>>>(
        A.rowptr, A.idx, static_cast<const V*>(A.val), b.ratio, A.nrows, bp);
    MLEM_LAUNCHED();
}

template <typename V>
void fp_v(const DevCsr& A, const BatchArgs& b, L2Window win, cudaStream_t s) {
    if (b.tile == 32) fp_bt<32, V>(A, b, win, s);
    else if (b.tile == 16) fp_bt<16, V>(A, b, win, s);
    else fp_bt<8, V>(A, b, win, s);
}
template <typename V>
void bp_v(const DevCsr& AT, const float* norm, const BatchArgs& b, L2Window win, cudaStream_t s) {
    if (b.tile == 32) bp_bt<32, V>(AT, norm, b, win, s);
    else if (b.tile == 16) bp_bt<16, V>(AT, norm, b, win, s);
    else bp_bt<8, V>(AT, norm, b, win, s);
}
template <typename V>
void sc_v(const DevCsr& A, const BatchArgs& b, float* bp, cudaStream_t s) {
    if (b.tile == 32) sc_bt<32, V>(A, b, bp, s);
    else if (b.tile == 16) sc_bt<16, V>(A, b, bp, s);
    else sc_bt<8, V>(A, b, bp, s);
}

__global__ void k_slot_put(int32_t* __restrict__ G, float* __restrict__ F, uint32_t rows,
                           uint32_t cols, uint32_t BT, uint32_t b, const int32_t* __restrict__ g,
                           float init, const float* __restrict__ f0, uint32_t* __restrict__ remaining,
                           uint32_t iters, const uint32_t* __restrict__ lor_of, const uint32_t* __restrict__ vox_of) {
    const uint32_t n = rows > cols ? rows : cols;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        if (i < rows) G[(uint64_t)i * BT + b] = g[lor_of ? lor_of[i] : i];
        if (i < cols) F[(uint64_t)i * BT + b] = f0 ? f0[vox_of ? vox_of[i] : i] : init;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) remaining[b] = iters;
}

__global__ void k_slot_get(const float* __restrict__ F, uint32_t cols, uint32_t BT, uint32_t b,
                           float* __restrict__ out, const uint32_t* __restrict__ vox_of) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < cols; i += gridDim.x * blockDim.x)
        out[vox_of ? vox_of[i] : i] = F[(uint64_t)i * BT + b];
}

}  // namespace

void launch_slot_put(int32_t* G, float* F, uint32_t rows, uint32_t cols, uint32_t BT, uint32_t b,
                     const int32_t* g, float init, const float* f0, uint32_t* remaining,
                     uint32_t iters, const uint32_t* lor_of, const uint32_t* vox_of, cudaStream_t s) {
    const uint32_t n = std::max(rows, cols);
    const unsigned grid = std::max(1u, std::min<unsigned>(ceil_div_u(n, 256), 152u * 8u));
    k_slot_put<<<grid, 256, 0, s>>>(G, F, rows, cols, BT, b, g, init, f0, remaining, iters, lor_of, vox_of);
    MLEM_LAUNCHED();
}

void launch_slot_get(const float* F, uint32_t cols, uint32_t BT, uint32_t b, float* out,
                     const uint32_t* vox_of, cudaStream_t s) {
    const unsigned grid = std::max(1u, std::min<unsigned>(ceil_div_u(cols, 256), 152u * 8u));
    k_slot_get<<<grid, 256, 0, s>>>(F, cols, BT, b, out, vox_of);
    MLEM_LAUNCHED();
}

void launch_batch_fp(const DevCsr& A, const BatchArgs& b, L2Window win, cudaStream_t s) {
    if (A.nrows == 0) return;
    switch (A.vt) {
        case MLEM_VAL_F32: fp_v<float>(A, b, win, s); break;
        case MLEM_VAL_F16: fp_v<__half>(A, b, win, s); break;
        default: fp_v<__nv_bfloat16>(A, b, win, s);
    }
}

void launch_batch_bp_update(const DevCsr& AT, const float* norm, const BatchArgs& b, L2Window win,
                            cudaStream_t s) {
    if (AT.nrows == 0) return;
    switch (AT.vt) {
        case MLEM_VAL_F32: bp_v<float>(AT, norm, b, win, s); break;
        case MLEM_VAL_F16: bp_v<__half>(AT, norm, b, win, s); break;
        default: bp_v<__nv_bfloat16>(AT, norm, b, win, s);
    }
}

void launch_batch_tick(const BatchArgs& b, cudaStream_t s) {
    k_batch_tick<<<1, 32, 0, s>>>(b.remaining, b.tile);
    MLEM_LAUNCHED();
}

void launch_batch_scatter(const DevCsr& A, const BatchArgs& b, float* bp, cudaStream_t s) {
    if (A.nrows == 0) return;
    switch (A.vt) {
        case MLEM_VAL_F32: sc_v<float>(A, b, bp, s); break;
        case MLEM_VAL_F16: sc_v<__half>(A, b, bp, s); break;
        default: sc_v<__nv_bfloat16>(A, b, bp, s);
    }
}

void launch_batch_update_zero(const float* norm, uint32_t cols, const BatchArgs& b, float* bp,
                              cudaStream_t s) {
    const uint64_t n = (uint64_t)cols * b.tile;
    if (n == 0) return;
    const unsigned grid = std::max(1u, std::min<unsigned>(ceil_div_u(n, 256), 152u * 16u));
    k_batch_update_zero<<<grid, 256, 0, s>>>(norm, cols, b.tile, b.remaining, b.f, bp);
    MLEM_LAUNCHED();
}

}  // namespace mlem
