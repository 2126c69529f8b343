// transpose.cu — device-built CSR of Aᵀ and the sensitivity image.
//
// The reference transposes on the host with sptrans_scanTrans_specialized
// (sptrans.h:397-545): per-thread column histograms, an inter-thread prefix
// and intra-thread ranks, i.e. a stable counting sort of the nonzeros by
// column.  Its output therefore lists the entries of every column in
// increasing original position, independent of the thread count.
//
// Here the same permutation is produced by a stable LSD radix sort on the
// GPU: key = column index (8-bit digits, as many passes as the column count
// needs), payload = (row id, value bits).  Each pass is a per-tile digit
// histogram, an exclusive scan over (digit, tile) and a scatter in which every
// warp ranks its elements chunk by chunk with __match_any_sync, so equal
// digits keep their input order (stable).  The column pointer is a count +
// exclusive scan.  The result is bit-identical to the reference transpose.
#include "kernels.cuh"

#include <algorithm>
#include <vector>

namespace mlem {

namespace {

constexpr int kScanT = 256, kScanIpt = 16, kScanTile = kScanT * kScanIpt;
constexpr int kRsT = 256, kRsIpt = 16, kRsTile = kRsT * kRsIpt, kRsWarps = kRsT / 32;

template <typename T>
__device__ __forceinline__ T warp_incl_scan(T v) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const T u = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += u;
    }
    return v;
}

// Exclusive scan of the 256 per-thread sums of a block; returns the block total.
template <typename T>
__device__ __forceinline__ T block_excl_scan(T v, T& excl, T* sh /* [8] */) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const T inc = warp_incl_scan(v);
    if (lane == 31) sh[w] = inc;
    __syncthreads();
    if (w == 0) {
        T x = lane < (int)(blockDim.x >> 5) ? sh[lane] : (T)0;
        x = warp_incl_scan(x);
        if (lane < (int)(blockDim.x >> 5)) sh[lane] = x;
    }
    __syncthreads();
    const T wbase = w ? sh[w - 1] : (T)0;
    excl = wbase + inc - v;
    const T total = sh[(blockDim.x >> 5) - 1];
    __syncthreads();
    return total;
}

template <typename Tin, typename Tout>
__global__ void __launch_bounds__(kScanT) k_scan_reduce(const Tin* __restrict__ in, uint64_t n,
                                                        Tout* __restrict__ part) {
    __shared__ Tout sh[8];
    const uint64_t base = (uint64_t)blockIdx.x * kScanTile;
    Tout s = 0;
#pragma unroll 4
    for (int it = 0; it < kScanIpt; ++it) {
        const uint64_t e = base + (uint64_t)it * kScanT + threadIdx.x;
        if (e < n) s += (Tout)in[e];
    }
    Tout ex;
    const Tout tot = block_excl_scan<Tout>(s, ex, sh);
    if (threadIdx.x == 0) part[blockIdx.x] = tot;
}

template <typename Tin, typename Tout>
__global__ void __launch_bounds__(kScanT) k_scan_down(const Tin* __restrict__ in, uint64_t n,
                                                      const Tout* __restrict__ base_part,
                                                      Tout* __restrict__ out, Tout* __restrict__ total_out) {
    __shared__ Tout tile[kScanTile];
    __shared__ Tout sh[8];
    const uint64_t base = (uint64_t)blockIdx.x * kScanTile;
    for (int it = 0; it < kScanIpt; ++it) {
        const int u = it * kScanT + threadIdx.x;
        const uint64_t e = base + u;
        tile[u] = e < n ? (Tout)in[e] : (Tout)0;
    }
    __syncthreads();
    Tout loc[kScanIpt];
    Tout s = 0;
#pragma unroll
    for (int q = 0; q < kScanIpt; ++q) {
        loc[q] = tile[threadIdx.x * kScanIpt + q];
        s += loc[q];
    }
    Tout ex;
    const Tout tot = block_excl_scan<Tout>(s, ex, sh);
    Tout run = ex + (base_part ? base_part[blockIdx.x] : (Tout)0);
#pragma unroll
    for (int q = 0; q < kScanIpt; ++q) {
        tile[threadIdx.x * kScanIpt + q] = run;
        run += loc[q];
    }
    __syncthreads();
    for (int it = 0; it < kScanIpt; ++it) {
        const int u = it * kScanT + threadIdx.x;
        const uint64_t e = base + u;
        if (e < n) out[e] = tile[u];
    }
    if (total_out && blockIdx.x == gridDim.x - 1 && threadIdx.x == 0)
        *total_out = (base_part ? base_part[blockIdx.x] : (Tout)0) + tot;
}

// Exclusive scan in -> out (n elements); *total (device, optional) = sum.
template <typename Tin, typename Tout>
void scan_exclusive(const Tin* in, Tout* out, uint64_t n, Tout* total, cudaStream_t s) {
    if (n == 0) {
        if (total) MLEM_CUDA(cudaMemsetAsync(total, 0, sizeof(Tout), s));
        return;
    }
    const uint64_t nb = (n + kScanTile - 1) / kScanTile;
    if (nb == 1) {
        k_scan_down<Tin, Tout><<<1, kScanT, 0, s>>>(in, n, nullptr, out, total);
        MLEM_LAUNCHED();
        return;
    }
    Tout* part = nullptr;
    Tout* part_scan = nullptr;
    MLEM_CUDA(cudaMallocAsync(&part, sizeof(Tout) * nb, s));
    MLEM_CUDA(cudaMallocAsync(&part_scan, sizeof(Tout) * nb, s));
    k_scan_reduce<Tin, Tout><<<(unsigned)nb, kScanT, 0, s>>>(in, n, part);
    MLEM_LAUNCHED();
    scan_exclusive<Tout, Tout>(part, part_scan, nb, (Tout*)nullptr, s);
    k_scan_down<Tin, Tout><<<(unsigned)nb, kScanT, 0, s>>>(in, n, part_scan, out, total);
    MLEM_LAUNCHED();
    MLEM_CUDA(cudaFreeAsync(part, s));
    MLEM_CUDA(cudaFreeAsync(part_scan, s));
}

__global__ void k_col_count(const uint32_t* __restrict__ col, uint64_t nnz, uint32_t* __restrict__ cnt) {
    for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < nnz;
         e += (uint64_t)gridDim.x * blockDim.x)
        atomicAdd(cnt + col[e], 1u);
}

// payload[e] = row(e) | value_bits(e) << 32, one warp per row.
__global__ void k_row_payload(const uint64_t* __restrict__ rowptr, const float* __restrict__ val,
                              uint32_t rows, uint64_t* __restrict__ pay) {
    const uint32_t wid = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    const uint32_t nw = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t r = wid; r < rows; r += nw) {
        const uint64_t s = rowptr[r], t = rowptr[r + 1];
        for (uint64_t e = s + lane; e < t; e += 32)
            pay[e] = (uint64_t)r | ((uint64_t)__float_as_uint(val[e]) << 32);
    }
}

__global__ void __launch_bounds__(kRsT) k_radix_hist(const uint32_t* __restrict__ keys, uint64_t n,
                                                     int shift, uint32_t* __restrict__ hist,
                                                     uint64_t ntiles) {
    __shared__ uint32_t cnt[256];
    cnt[threadIdx.x] = 0;
    __syncthreads();
    const uint64_t base = blockIdx.x * (uint64_t)kRsTile;
#pragma unroll 4
    for (int it = 0; it < kRsIpt; ++it) {
        const uint64_t e = base + (uint64_t)it * kRsT + threadIdx.x;
        if (e < n) atomicAdd(&cnt[(keys[e] >> shift) & 255u], 1u);
    }
    __syncthreads();
    hist[(uint64_t)threadIdx.x * ntiles + blockIdx.x] = cnt[threadIdx.x];
}

// Stable scatter of one radix pass.  Warp w of the tile owns elements
// [tile + w*512, +512) and ranks them 32 at a time in order.
template <bool LAST>
__global__ void __launch_bounds__(kRsT)
k_radix_scatter(const uint32_t* __restrict__ keys_in, const uint64_t* __restrict__ pay_in,
                uint64_t n, int shift, const uint32_t* __restrict__ offs, uint64_t ntiles,
                uint32_t* __restrict__ keys_out, uint64_t* __restrict__ pay_out,
                uint32_t* __restrict__ row_out, float* __restrict__ val_out) {
    __shared__ uint32_t wcnt[kRsWarps][256];
    __shared__ uint32_t goff[256];
    for (int w = 0; w < kRsWarps; ++w) wcnt[w][threadIdx.x] = 0;
    goff[threadIdx.x] = offs[(uint64_t)threadIdx.x * ntiles + blockIdx.x];
    __syncthreads();
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const unsigned lt_mask = (1u << lane) - 1u;
    const uint64_t base = blockIdx.x * (uint64_t)kRsTile + (uint64_t)w * (32 * kRsIpt);
    uint32_t key[kRsIpt];
    uint64_t pay[kRsIpt];
    uint32_t pos[kRsIpt];
#pragma unroll
    for (int c = 0; c < kRsIpt; ++c) {
        const uint64_t e = base + c * 32 + lane;
        const bool valid = e < n;
        key[c] = valid ? keys_in[e] : 0u;
        pay[c] = valid ? pay_in[e] : 0ull;
    }
#pragma unroll
    for (int c = 0; c < kRsIpt; ++c) {
        const uint64_t e = base + c * 32 + lane;
        const bool valid = e < n;
        const unsigned vm = __ballot_sync(0xffffffffu, valid);
        const uint32_t d = (key[c] >> shift) & 255u;
        unsigned peers = 0, cnt = 0;
        if (valid) {
            peers = __match_any_sync(vm, d);
            cnt = wcnt[w][d];
            pos[c] = cnt + __popc(peers & lt_mask);
        }
        __syncwarp();
        if (valid && (peers & lt_mask) == 0) wcnt[w][d] = cnt + __popc(peers);
        __syncwarp();
    }
    __syncthreads();
    {  // exclusive prefix of the warp counts, per digit, in warp order
        uint32_t run = 0;
        for (int q = 0; q < kRsWarps; ++q) {
            const uint32_t c = wcnt[q][threadIdx.x];
            wcnt[q][threadIdx.x] = run;
            run += c;
        }
    }
    __syncthreads();
#pragma unroll
    for (int c = 0; c < kRsIpt; ++c) {
        const uint64_t e = base + c * 32 + lane;
        if (e < n) {
            const uint32_t d = (key[c] >> shift) & 255u;
            const uint64_t p = (uint64_t)goff[d] + wcnt[w][d] + pos[c];
            if (LAST) {
                row_out[p] = (uint32_t)pay[c];
                val_out[p] = __uint_as_float((uint32_t)(pay[c] >> 32));
            } else {
                keys_out[p] = key[c];
                pay_out[p] = pay[c];
            }
        }
    }
}

// norm[c] = Σ val over row c of Aᵀ, FP64, lane-strided then xor tree.
template <typename V>
__global__ void k_colsum_rows(const uint64_t* __restrict__ rowptr, const V* __restrict__ val,
                              uint32_t nrows, float* __restrict__ out) {
    const uint32_t wid = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    const uint32_t nw = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t r = wid; r < nrows; r += nw) {
        const uint64_t s = rowptr[r], t = rowptr[r + 1];
        double acc = 0.0;
        for (uint64_t e = s + lane; e < t; e += 32) acc += (double)Val4<V>::one(val, e);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        if (lane == 0) out[r] = (float)acc;
    }
}

template <typename V>
__global__ void k_colsum_scatter(const uint64_t* __restrict__ rowptr, const uint32_t* __restrict__ idx,
                                 const V* __restrict__ val, uint32_t rows, double* __restrict__ acc) {
    const uint32_t wid = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    const uint32_t nw = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t r = wid; r < rows; r += nw) {
        const uint64_t s = rowptr[r], t = rowptr[r + 1];
        for (uint64_t e = s + lane; e < t; e += 32)
            atomicAdd(acc + idx[e], (double)Val4<V>::one(val, e));
    }
}

__global__ void k_f64_to_f32(const double* __restrict__ in, float* __restrict__ out, uint64_t n) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
         i += (uint64_t)gridDim.x * blockDim.x)
        out[i] = (float)in[i];
}

template <typename V>
__global__ void k_to_lowp(const float* __restrict__ in, V* __restrict__ out, uint64_t n);
template <>
__global__ void k_to_lowp<__half>(const float* __restrict__ in, __half* __restrict__ out, uint64_t n) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
         i += (uint64_t)gridDim.x * blockDim.x)
        out[i] = __float2half_rn(in[i]);
}
template <>
__global__ void k_to_lowp<__nv_bfloat16>(const float* __restrict__ in, __nv_bfloat16* __restrict__ out,
                                         uint64_t n) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
         i += (uint64_t)gridDim.x * blockDim.x)
        out[i] = __float2bfloat16_rn(in[i]);
}

template <typename V>
__global__ void k_from_lowp(const V* __restrict__ in, float* __restrict__ out, uint64_t n) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
         i += (uint64_t)gridDim.x * blockDim.x)
        out[i] = Val4<V>::one(in, i);
}

__global__ void k_max_row(const uint64_t* __restrict__ rowptr, uint32_t rows, uint32_t* __restrict__ mx) {
    uint32_t m = 0;
    for (uint32_t r = blockIdx.x * blockDim.x + threadIdx.x; r < rows; r += gridDim.x * blockDim.x) {
        const uint64_t l = rowptr[r + 1] - rowptr[r];
        m = max(m, (uint32_t)(l > 0xffffffffull ? 0xffffffffull : l));
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) atomicMax(mx, m);
}

// flags: bit0 rowptr[0] != 0, bit1 decreasing rowptr, bit2 rowptr[rows] != nnz, bit3 col >= cols
__global__ void k_validate_rows(const uint64_t* __restrict__ rowptr, uint32_t rows, uint64_t nnz,
                                uint32_t* __restrict__ flags) {
    for (uint32_t r = blockIdx.x * blockDim.x + threadIdx.x; r < rows; r += gridDim.x * blockDim.x) {
        if (rowptr[r + 1] < rowptr[r]) atomicOr(flags, 2u);
        if (r == 0 && rowptr[0] != 0) atomicOr(flags, 1u);
        if (r == rows - 1 && rowptr[rows] != nnz) atomicOr(flags, 4u);
    }
}
__global__ void k_validate_cols(const uint32_t* __restrict__ idx, uint64_t nnz, uint32_t cols,
                                uint32_t* __restrict__ flags) {
    bool bad = false;
    for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < nnz;
         e += (uint64_t)gridDim.x * blockDim.x)
        bad |= idx[e] >= cols;
    if (__any_sync(0xffffffffu, bad) && (threadIdx.x & 31) == 0) atomicOr(flags, 8u);
}

unsigned grid_for(uint64_t n, unsigned per = 256, unsigned cap = 152u * 16u) {
    return std::max(1u, std::min<unsigned>(ceil_div_u(n, per), cap));
}

}  // namespace

void scan_counts_u64(const uint32_t* in, uint64_t* out, uint64_t n, cudaStream_t s) {
    scan_exclusive<uint32_t, uint64_t>(in, out, n, out + n, s);
}

void transpose_device(const DevCsr& A, DevCsr& AT, cudaStream_t s) {
    MLEM_REQUIRE(A.vt == MLEM_VAL_F32, MLEM_EINVAL, "transpose expects f32 values");
    MLEM_REQUIRE(A.nnz < (1ull << 32), MLEM_EUNSUPPORTED, "transpose: nnz must be < 2^32");
    const uint64_t n = A.nnz;
    AT.nrows = A.ncols;
    AT.ncols = A.nrows;
    AT.nnz = n;
    AT.vt = MLEM_VAL_F32;
    MLEM_CUDA(cudaMalloc(&AT.rowptr, sizeof(uint64_t) * ((uint64_t)AT.nrows + 1)));
    MLEM_CUDA(cudaMalloc(&AT.idx, sizeof(uint32_t) * padded(n)));
    MLEM_CUDA(cudaMalloc(&AT.val, sizeof(float) * padded(n)));
    MLEM_CUDA(cudaMemsetAsync(AT.idx, 0, sizeof(uint32_t) * padded(n), s));
    MLEM_CUDA(cudaMemsetAsync(AT.val, 0, sizeof(float) * padded(n), s));

    // column pointer: count + exclusive scan (cscColPtr of sptrans.h:455-463)
    uint32_t* cnt = nullptr;
    MLEM_CUDA(cudaMallocAsync(&cnt, sizeof(uint32_t) * std::max<uint64_t>(A.ncols, 1), s));
    MLEM_CUDA(cudaMemsetAsync(cnt, 0, sizeof(uint32_t) * std::max<uint64_t>(A.ncols, 1), s));
    if (n) {
        k_col_count<<<grid_for(n, 256, 152u * 32u), 256, 0, s>>>(A.idx, n, cnt);
        MLEM_LAUNCHED();
    }
    scan_counts_u64(cnt, AT.rowptr, A.ncols, s);
    MLEM_CUDA(cudaFreeAsync(cnt, s));
    if (n == 0) return;

    int bits = 0;
    while (bits < 32 && (1ull << bits) < (uint64_t)A.ncols) ++bits;
    const int passes = std::max(1, (bits + 7) / 8);
    const uint64_t ntiles = (n + kRsTile - 1) / kRsTile;

    uint32_t *kb[2] = {nullptr, nullptr}, *hist = nullptr, *offs = nullptr;
    uint64_t* pb[2] = {nullptr, nullptr};
    for (int q = 0; q < 2; ++q) {
        MLEM_CUDA(cudaMallocAsync(&kb[q], sizeof(uint32_t) * n, s));
        MLEM_CUDA(cudaMallocAsync(&pb[q], sizeof(uint64_t) * n, s));
    }
    MLEM_CUDA(cudaMallocAsync(&hist, sizeof(uint32_t) * 256 * ntiles, s));
    MLEM_CUDA(cudaMallocAsync(&offs, sizeof(uint32_t) * 256 * ntiles, s));

    k_row_payload<<<grid_for((uint64_t)A.nrows * 32, 256, 152u * 32u), 256, 0, s>>>(
        A.rowptr, static_cast<const float*>(A.val), A.nrows, pb[0]);
    MLEM_LAUNCHED();

    const uint32_t* kin = A.idx;
    int cur = 0;
    for (int p = 0; p < passes; ++p) {
        const int shift = 8 * p;
        const bool last = (p == passes - 1);
        k_radix_hist<<<(unsigned)ntiles, kRsT, 0, s>>>(kin, n, shift, hist, ntiles);
        MLEM_LAUNCHED();
        scan_exclusive<uint32_t, uint32_t>(hist, offs, 256 * ntiles, (uint32_t*)nullptr, s);
        if (last) {
            k_radix_scatter<true><<<(unsigned)ntiles, kRsT, 0, s>>>(
                kin, pb[cur], n, shift, offs, ntiles, nullptr, nullptr, AT.idx,
                static_cast<float*>(AT.val));
        } else {
            k_radix_scatter<false><<<(unsigned)ntiles, kRsT, 0, s>>>(
                kin, pb[cur], n, shift, offs, ntiles, kb[cur ^ 1], pb[cur ^ 1], nullptr, nullptr);
        }
        MLEM_LAUNCHED();
        kin = kb[cur ^ 1];
        cur ^= 1;
    }
    for (int q = 0; q < 2; ++q) {
        MLEM_CUDA(cudaFreeAsync(kb[q], s));
        MLEM_CUDA(cudaFreeAsync(pb[q], s));
    }
    MLEM_CUDA(cudaFreeAsync(hist, s));
    MLEM_CUDA(cudaFreeAsync(offs, s));
    AT.max_row = max_row_length(AT.rowptr, AT.nrows, s);
}

void colsum_from_transpose(const DevCsr& AT, float* norm, cudaStream_t s) {
    if (AT.nrows == 0) return;
    const unsigned grid = grid_for((uint64_t)AT.nrows * 32, 256, 152u * 32u);
    switch (AT.vt) {
        case MLEM_VAL_F32:
            k_colsum_rows<float><<<grid, 256, 0, s>>>(AT.rowptr, (const float*)AT.val, AT.nrows, norm);
            break;
        case MLEM_VAL_F16:
            k_colsum_rows<__half><<<grid, 256, 0, s>>>(AT.rowptr, (const __half*)AT.val, AT.nrows, norm);
            break;
        default:
            k_colsum_rows<__nv_bfloat16><<<grid, 256, 0, s>>>(AT.rowptr, (const __nv_bfloat16*)AT.val,
                                                              AT.nrows, norm);
    }
    MLEM_LAUNCHED();
}

void colsum_scatter(const DevCsr& A, float* norm, cudaStream_t s) {
    double* acc = nullptr;
    const uint64_t nc = std::max<uint64_t>(A.ncols, 1);
    MLEM_CUDA(cudaMallocAsync(&acc, sizeof(double) * nc, s));
    MLEM_CUDA(cudaMemsetAsync(acc, 0, sizeof(double) * nc, s));
    if (A.nrows) {
        const unsigned grid = grid_for((uint64_t)A.nrows * 32, 256, 152u * 32u);
        switch (A.vt) {
            case MLEM_VAL_F32:
                k_colsum_scatter<float><<<grid, 256, 0, s>>>(A.rowptr, A.idx, (const float*)A.val, A.nrows, acc);
                break;
            case MLEM_VAL_F16:
                k_colsum_scatter<__half><<<grid, 256, 0, s>>>(A.rowptr, A.idx, (const __half*)A.val, A.nrows, acc);
                break;
            default:
                k_colsum_scatter<__nv_bfloat16><<<grid, 256, 0, s>>>(A.rowptr, A.idx,
                                                                     (const __nv_bfloat16*)A.val, A.nrows, acc);
        }
        MLEM_LAUNCHED();
    }
    if (A.ncols) {
        k_f64_to_f32<<<grid_for(A.ncols), 256, 0, s>>>(acc, norm, A.ncols);
        MLEM_LAUNCHED();
    }
    MLEM_CUDA(cudaFreeAsync(acc, s));
}

void convert_values(const float* src, void* dst, mlem_value_type vt, uint64_t n, cudaStream_t s) {
    if (n == 0) return;
    if (vt == MLEM_VAL_F16) k_to_lowp<__half><<<grid_for(n, 256, 152u * 32u), 256, 0, s>>>(src, (__half*)dst, n);
    else if (vt == MLEM_VAL_BF16)
        k_to_lowp<__nv_bfloat16><<<grid_for(n, 256, 152u * 32u), 256, 0, s>>>(src, (__nv_bfloat16*)dst, n);
    else {
        MLEM_CUDA(cudaMemcpyAsync(dst, src, n * sizeof(float), cudaMemcpyDeviceToDevice, s));
        return;
    }
    MLEM_LAUNCHED();
}

void convert_values_back(const void* src, float* dst, mlem_value_type vt, uint64_t n, cudaStream_t s) {
    if (n == 0) return;
    if (vt == MLEM_VAL_F16) k_from_lowp<__half><<<grid_for(n, 256, 152u * 32u), 256, 0, s>>>((const __half*)src, dst, n);
    else if (vt == MLEM_VAL_BF16)
        k_from_lowp<__nv_bfloat16><<<grid_for(n, 256, 152u * 32u), 256, 0, s>>>((const __nv_bfloat16*)src, dst, n);
    else {
        MLEM_CUDA(cudaMemcpyAsync(dst, src, n * sizeof(float), cudaMemcpyDeviceToDevice, s));
        return;
    }
    MLEM_LAUNCHED();
}

uint32_t max_row_length(const uint64_t* rowptr, uint32_t rows, cudaStream_t s) {
    if (rows == 0) return 0;
    uint32_t* d = nullptr;
    MLEM_CUDA(cudaMallocAsync(&d, sizeof(uint32_t), s));
    MLEM_CUDA(cudaMemsetAsync(d, 0, sizeof(uint32_t), s));
    k_max_row<<<grid_for(rows), 256, 0, s>>>(rowptr, rows, d);
    MLEM_LAUNCHED();
    uint32_t h = 0;
    MLEM_CUDA(cudaMemcpyAsync(&h, d, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
    MLEM_CUDA(cudaStreamSynchronize(s));
    MLEM_CUDA(cudaFreeAsync(d, s));
    return h;
}

bool validate_csr(const DevCsr& A, cudaStream_t s) {
    uint32_t* d = nullptr;
    MLEM_CUDA(cudaMallocAsync(&d, sizeof(uint32_t), s));
    MLEM_CUDA(cudaMemsetAsync(d, 0, sizeof(uint32_t), s));
    if (A.nrows) {
        k_validate_rows<<<grid_for(A.nrows), 256, 0, s>>>(A.rowptr, A.nrows, A.nnz, d);
        MLEM_LAUNCHED();
    }
    if (A.nnz) {
        k_validate_cols<<<grid_for(A.nnz, 256, 152u * 32u), 256, 0, s>>>(A.idx, A.nnz, A.ncols, d);
        MLEM_LAUNCHED();
    }
    uint32_t h = 0;
    MLEM_CUDA(cudaMemcpyAsync(&h, d, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
    MLEM_CUDA(cudaStreamSynchronize(s));
    MLEM_CUDA(cudaFreeAsync(d, s));
    return h == 0;
}

}  // namespace mlem
