// spmv_d16.cu — projections over delta-compressed column indices (D16).
//
// Layout of an operand in D16 form (kept beside the u32 indices):
//   rowmeta[r] = first column of row r | (index of the row's first escape << 32)
//   d16[e]     = column(e) - column(e-1) for e inside a row (0 for the row's
//                first element), or 0xFFFF ("escape") when that difference is
//                negative or does not fit in 16 bits
//   esc[k]     = absolute column of the k-th escaped element (element order)
// With FP16 values a nonzero costs 4 bytes instead of 8 (u32 + f32).
//
// Kernel: one warp per row; a round covers 32 vectors of 8 consecutive
// elements (lane l owns vector l of the round).  The columns are the prefix
// sum of the deltas with resets at escapes: each lane summarises its vector
// (escape count; column after its last escape, or its delta sum), two warp
// scans (escape counts, then columns with the reset operator) give every
// lane the column before its vector, then the lane decodes its 8 columns,
// gathers x and accumulates in element order.  Deterministic.
#include "kernels.cuh"

#include <algorithm>
#include <vector>

namespace mlem {

namespace {

constexpr uint16_t kEsc = 0xFFFF;

template <typename V>
struct Val8;

template <>
struct Val8<float> {
    static __device__ __forceinline__ void load(const float* p, uint64_t v, float out[8]) {
        const float4* q = reinterpret_cast<const float4*>(p) + 2 * v;
        const float4 a = __ldcs(q), b = __ldcs(q + 1);
        out[0] = a.x; out[1] = a.y; out[2] = a.z; out[3] = a.w;
        out[4] = b.x; out[5] = b.y; out[6] = b.z; out[7] = b.w;
    }
};

template <>
struct Val8<__half> {
    static __device__ __forceinline__ void load(const __half* p, uint64_t v, float out[8]) {
        const uint4 u = __ldcs(reinterpret_cast<const uint4*>(p) + v);
        const uint32_t w[4] = {u.x, u.y, u.z, u.w};
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const float2 f = __half22float2(*reinterpret_cast<const __half2*>(&w[k]));
            out[2 * k] = f.x;
            out[2 * k + 1] = f.y;
        }
    }
};

template <>
struct Val8<__nv_bfloat16> {
    static __device__ __forceinline__ void load(const __nv_bfloat16* p, uint64_t v, float out[8]) {
        const uint4 u = __ldcs(reinterpret_cast<const uint4*>(p) + v);
        const uint32_t w[4] = {u.x, u.y, u.z, u.w};
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const float2 f = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(&w[k]));
            out[2 * k] = f.x;
            out[2 * k + 1] = f.y;
        }
    }
};

template <typename V, int EPI>
__global__ void __launch_bounds__(256)
k_csr_d16(const uint64_t* __restrict__ rowptr, const uint64_t* __restrict__ rowmeta,
          const uint16_t* __restrict__ d16, const V* __restrict__ val, const uint32_t* __restrict__ esc,
          const float* __restrict__ x, uint32_t nrows, const int32_t* __restrict__ g, float* __restrict__ out,
          float* __restrict__ fwproj, float* __restrict__ f, const float* __restrict__ norm) {
    const uint32_t row = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (row >= nrows) return;  // warp-uniform
    const uint64_t s = rowptr[row], t = rowptr[row + 1];
    const uint64_t meta = rowmeta[row];
    uint32_t carry_col = (uint32_t)meta;          // column before the next round
    uint64_t esc_next = meta >> 32;               // esc[] index of the next escape
    const uint64_t v1 = (t + 7) >> 3;
    float acc = 0.f;
    for (uint64_t vb = s >> 3; vb < v1; vb += 32) {
        const uint64_t v = vb + lane;
        const bool have = v < v1;
        uint32_t dw[4] = {0, 0, 0, 0};
        float a[8];
        if (have) {
            const uint4 u = __ldcs(reinterpret_cast<const uint4*>(d16) + v);
            dw[0] = u.x; dw[1] = u.y; dw[2] = u.z; dw[3] = u.w;
            Val8<V>::load(val, v, a);
        }
        uint32_t d[8];
        bool ok[8];
        uint32_t nesc = 0, sum = 0;
        bool reset = false;
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            d[j] = (dw[j >> 1] >> (16 * (j & 1))) & 0xFFFFu;
            const uint64_t e = (v << 3) + j;
            ok[j] = have && e >= s && e < t;
            if (ok[j]) {
                if (d[j] == kEsc) {
                    ++nesc;
                    reset = true;
                    sum = 0;
                } else {
                    sum += d[j];
                }
            }
        }
        // escape ordinals: exclusive scan of the per-lane escape counts
        uint32_t incl_n = nesc;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, incl_n, o);
            if (lane >= o) incl_n += y;
        }
        const uint64_t my_esc = esc_next + (incl_n - nesc);
        const uint32_t round_esc = __shfl_sync(0xffffffffu, incl_n, 31);
        // column after this lane's vector: last escape value + deltas after it
        uint32_t cv = sum;
        if (reset) cv = esc[my_esc + nesc - 1] + sum;
        // inclusive scan with resets: (r1, c1) then (r2, c2) -> r2 ? c2 : c1 + c2
        bool sr = reset;
        uint32_t sc = cv;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t yc = __shfl_up_sync(0xffffffffu, sc, o);
            const bool yr = __shfl_up_sync(0xffffffffu, sr ? 1u : 0u, o) != 0;
            if (lane >= o && !sr) {
                sc = yc + sc;
                sr = yr;
            }
        }
        // column before this lane's vector
        uint32_t pc = __shfl_up_sync(0xffffffffu, sc, 1);
        const bool pr = __shfl_up_sync(0xffffffffu, sr ? 1u : 0u, 1) != 0;
        uint32_t col = (lane == 0) ? carry_col : (pr ? pc : carry_col + pc);
        // next round's carry from lane 31
        const uint32_t c31 = __shfl_sync(0xffffffffu, sc, 31);
        const bool r31 = __shfl_sync(0xffffffffu, sr ? 1u : 0u, 31) != 0;
        // decode, gather, accumulate
        uint32_t cols[8];
        uint64_t k = my_esc;
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            if (ok[j]) col = (d[j] == kEsc) ? esc[k++] : col + d[j];
            cols[j] = col;
        }
        float gx[8];
#pragma unroll
        for (int j = 0; j < 8; ++j) gx[j] = ok[j] ? __ldg(x + cols[j]) : 0.f;
#pragma unroll
        for (int j = 0; j < 8; ++j)
            if (ok[j]) acc = fmaf(a[j], gx[j], acc);
        carry_col = r31 ? c31 : carry_col + c31;
        esc_next += round_esc;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane == 0) {
        if (EPI == (int)Epi::Correl) {
            out[row] = (acc != 0.0f) ? __fdiv_rn((float)g[row], acc) : 0.0f;
            if (fwproj) fwproj[row] = acc;
        } else if (EPI == (int)Epi::Update) {
            const float tt = __fmul_rn(f[row], acc);
            const float nn = norm[row];
            f[row] = (nn == 0.0f) ? tt : __fdiv_rn(tt, nn);
        } else {
            out[row] = acc;
        }
    }
}

// ---------------------------------------------------------------- conversion
__device__ __forceinline__ bool is_escape(const uint32_t* __restrict__ col, uint64_t e, uint64_t s) {
    if (e == s) return false;
    const uint32_t a = col[e - 1], b = col[e];
    return b < a || b - a >= kEsc;
}

__global__ void k_d16_count(const uint64_t* __restrict__ rowptr, const uint32_t* __restrict__ col, uint32_t rows,
                            uint32_t* __restrict__ cnt) {
    const uint32_t wid = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    const uint32_t nw = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t r = wid; r < rows; r += nw) {
        const uint64_t s = rowptr[r], t = rowptr[r + 1];
        uint32_t n = 0;
        for (uint64_t e = s + lane; e < t; e += 32) n += is_escape(col, e, s) ? 1u : 0u;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) n += __shfl_xor_sync(0xffffffffu, n, o);
        if (lane == 0) cnt[r] = n;
    }
}

__global__ void k_d16_fill(const uint64_t* __restrict__ rowptr, const uint32_t* __restrict__ col, uint32_t rows,
                           const uint64_t* __restrict__ escptr, uint64_t* __restrict__ rowmeta,
                           uint16_t* __restrict__ d16, uint32_t* __restrict__ esc) {
    const uint32_t wid = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    const uint32_t nw = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t r = wid; r < rows; r += nw) {
        const uint64_t s = rowptr[r], t = rowptr[r + 1];
        uint64_t k = escptr[r];
        if (lane == 0) rowmeta[r] = (uint64_t)(s < t ? col[s] : 0u) | (k << 32);
        for (uint64_t b = s; b < t; b += 32) {
            const uint64_t e = b + lane;
            const bool in = e < t;
            const bool x = in && is_escape(col, e, s);
            const unsigned bal = __ballot_sync(0xffffffffu, x);
            if (in) {
                if (x) {
                    d16[e] = kEsc;
                    esc[k + __popc(bal & ((1u << lane) - 1u))] = col[e];
                } else {
                    d16[e] = (uint16_t)(e == s ? 0u : col[e] - col[e - 1]);
                }
            }
            k += __popc(bal);
        }
    }
}

template <typename V, int EPI>
void d16_launch(const DevCsr& op, const float* x, const EpiArgs& e, L2Window win, cudaStream_t s) {
    launch_ex(k_csr_d16<V, EPI>, dim3(ceil_div_u((uint64_t)op.nrows * 32, 256)), dim3(256), 0, s, win, op.rowptr,
              op.rowmeta, op.d16, static_cast<const V*>(op.val), op.esc, x, op.nrows, e.g, e.out, e.fwproj, e.f,
              e.norm);
}

template <typename V>
void d16_dispatch(const DevCsr& op, const float* x, const EpiArgs& e, L2Window win, cudaStream_t s) {
    switch (e.kind) {
        case Epi::Correl: d16_launch<V, (int)Epi::Correl>(op, x, e, win, s); break;
        case Epi::Update: d16_launch<V, (int)Epi::Update>(op, x, e, win, s); break;
        default: d16_launch<V, (int)Epi::Raw>(op, x, e, win, s);
    }
}

unsigned grid_rows(uint32_t rows) {
    return std::max(1u, std::min<unsigned>(ceil_div_u((uint64_t)rows * 32, 256), 152u * 32u));
}

}  // namespace

void build_d16(DevCsr& op, cudaStream_t s) {
    MLEM_REQUIRE(op.nnz < (1ull << 32), MLEM_EUNSUPPORTED, "D16 indices: nnz must be < 2^32");
    uint32_t* cnt = nullptr;
    uint64_t* escptr = nullptr;
    const uint64_t R = std::max<uint32_t>(op.nrows, 1);
    MLEM_CUDA(cudaMallocAsync(&cnt, sizeof(uint32_t) * R, s));
    MLEM_CUDA(cudaMallocAsync(&escptr, sizeof(uint64_t) * (R + 1), s));
    if (op.nrows) {
        k_d16_count<<<grid_rows(op.nrows), 256, 0, s>>>(op.rowptr, op.idx, op.nrows, cnt);
        MLEM_LAUNCHED();
    }
    scan_counts_u64(cnt, escptr, op.nrows, s);
    uint64_t nesc = 0;
    MLEM_CUDA(cudaMemcpyAsync(&nesc, escptr + op.nrows, sizeof(uint64_t), cudaMemcpyDeviceToHost, s));
    MLEM_CUDA(cudaStreamSynchronize(s));
    op.nesc = nesc;
    MLEM_CUDA(cudaMalloc(&op.rowmeta, sizeof(uint64_t) * R));
    MLEM_CUDA(cudaMalloc(&op.d16, sizeof(uint16_t) * padded(op.nnz)));
    MLEM_CUDA(cudaMalloc(&op.esc, sizeof(uint32_t) * std::max<uint64_t>(nesc, 1)));
    MLEM_CUDA(cudaMemsetAsync(op.d16, 0, sizeof(uint16_t) * padded(op.nnz), s));
    if (op.nrows) {
        k_d16_fill<<<grid_rows(op.nrows), 256, 0, s>>>(op.rowptr, op.idx, op.nrows, escptr, op.rowmeta, op.d16,
                                                       op.esc);
        MLEM_LAUNCHED();
    }
    MLEM_CUDA(cudaFreeAsync(cnt, s));
    MLEM_CUDA(cudaFreeAsync(escptr, s));
    MLEM_CUDA(cudaStreamSynchronize(s));
}

void launch_csr_d16(const DevCsr& op, const float* x, const EpiArgs& epi, L2Window win, cudaStream_t s) {
    if (op.nrows == 0) return;
    MLEM_REQUIRE(op.d16 != nullptr, MLEM_EINVAL, "operand has no D16 indices");
    switch (op.vt) {
        case MLEM_VAL_F32: d16_dispatch<float>(op, x, epi, win, s); break;
        case MLEM_VAL_F16: d16_dispatch<__half>(op, x, epi, win, s); break;
        default: d16_dispatch<__nv_bfloat16>(op, x, epi, win, s);
    }
}

}  // namespace mlem
