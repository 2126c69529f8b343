// spmv_ilv.cu — projections over a lane-interleaved copy of the matrix.
//
// The nonzeros are permuted inside aligned blocks of 128: element
// 128*b + 32*j + l is stored at position 128*b + 4*l + j.  One 16-byte load
// by lane l then brings elements l, l+32, l+64, l+96 of the block, and the j-th
// gather instruction of the warp covers 32 consecutive elements of the row.
// Columns are ascending inside a row, so those 32 gathers fall on few cache
// lines, whereas the natural layout (lane l owning 4 consecutive elements)
// spreads one gather instruction over 128 elements.  Each lane accumulates
// its elements in increasing order — the lane-strided partial sums of
// mat_vec_mul_csr_vector (kernel.cu:316-318) — and the warp reduces them
// with a fixed xor tree.  Deterministic.
#include "kernels.cuh"

#include <algorithm>

namespace mlem {

namespace {

__device__ __forceinline__ uint64_t ilv_pos(uint64_t e) {
    return (e & ~127ull) | ((e & 31ull) << 2) | ((e >> 5) & 3ull);
}

template <typename V>
__global__ void k_ilv_build(const uint32_t* __restrict__ idx, const V* __restrict__ val, uint64_t n,
                            uint32_t* __restrict__ idx_i, V* __restrict__ val_i) {
    for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < n; e += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t p = ilv_pos(e);
        idx_i[p] = idx[e];
        val_i[p] = val[e];
    }
}

template <typename V, int EPI, int U>
__global__ void __launch_bounds__(256)
k_csr_ilv(const uint64_t* __restrict__ rowptr, const uint32_t* __restrict__ idx_i, const V* __restrict__ val_i,
          const float* __restrict__ x, uint32_t nrows, const int32_t* __restrict__ g, float* __restrict__ out,
          float* __restrict__ fwproj, float* __restrict__ f, const float* __restrict__ norm) {
    const uint32_t row = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (row >= nrows) return;  // warp-uniform
    const uint64_t s = rowptr[row], t = rowptr[row + 1];
    const uint4* idx4 = reinterpret_cast<const uint4*>(idx_i);
    const uint64_t b1 = (t + 127) >> 7;
    float acc = 0.f;
    for (uint64_t b = s >> 7; b < b1; b += U) {
        uint4 c[U];
        float a[U][4];
#pragma unroll
        for (int q = 0; q < U; ++q) {
            if (b + q < b1) {
                const uint64_t vi = ((b + q) << 5) + lane;
                c[q] = ld_stream(idx4 + vi);
                Val4<V>::load(val_i, vi, a[q]);
            }
        }
        float gx[U][4];
#pragma unroll
        for (int q = 0; q < U; ++q) {
            const uint32_t cs[4] = {c[q].x, c[q].y, c[q].z, c[q].w};
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const uint64_t e = ((b + q) << 7) + 32 * j + lane;
                gx[q][j] = (b + q < b1 && e >= s && e < t) ? __ldg(x + cs[j]) : 0.f;
            }
        }
#pragma unroll
        for (int q = 0; q < U; ++q)
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const uint64_t e = ((b + q) << 7) + 32 * j + lane;
                if (b + q < b1 && e >= s && e < t) acc = fmaf(a[q][j], gx[q][j], acc);
            }
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

template <typename V, int EPI, int U>
void ilv_launch(const DevCsr& op, const float* x, const EpiArgs& e, L2Window win, cudaStream_t s) {
    launch_ex(k_csr_ilv<V, EPI, U>, dim3(ceil_div_u((uint64_t)op.nrows * 32, 256)), dim3(256), 0, s, win,
              op.rowptr, op.idx_ilv, static_cast<const V*>(op.val_ilv), x, op.nrows, e.g, e.out, e.fwproj, e.f,
              e.norm);
}

template <typename V, int U>
void ilv_epi(const DevCsr& op, const float* x, const EpiArgs& e, L2Window win, cudaStream_t s) {
    switch (e.kind) {
        case Epi::Correl: ilv_launch<V, (int)Epi::Correl, U>(op, x, e, win, s); break;
        case Epi::Update: ilv_launch<V, (int)Epi::Update, U>(op, x, e, win, s); break;
        default: ilv_launch<V, (int)Epi::Raw, U>(op, x, e, win, s);
    }
}

template <typename V>
void ilv_u(const DevCsr& op, const float* x, const EpiArgs& e, int unroll, L2Window win, cudaStream_t s) {
    if (unroll >= 4) ilv_epi<V, 4>(op, x, e, win, s);
    else if (unroll == 2) ilv_epi<V, 2>(op, x, e, win, s);
    else ilv_epi<V, 1>(op, x, e, win, s);
}

}  // namespace

void build_ilv(DevCsr& op, cudaStream_t s) {
    const uint64_t n128 = (op.nnz + 127) / 128 * 128;
    MLEM_CUDA(cudaMalloc(&op.idx_ilv, sizeof(uint32_t) * std::max<uint64_t>(n128, 128)));
    MLEM_CUDA(cudaMalloc(&op.val_ilv, val_bytes(op.vt) * std::max<uint64_t>(n128, 128)));
    MLEM_CUDA(cudaMemsetAsync(op.idx_ilv, 0, sizeof(uint32_t) * std::max<uint64_t>(n128, 128), s));
    MLEM_CUDA(cudaMemsetAsync(op.val_ilv, 0, val_bytes(op.vt) * std::max<uint64_t>(n128, 128), s));
    op.ilv_len = std::max<uint64_t>(n128, 128);
    if (op.nnz) {
        const unsigned grid = std::max(1u, std::min<unsigned>(ceil_div_u(op.nnz, 256), 152u * 32u));
        switch (op.vt) {
            case MLEM_VAL_F32:
                k_ilv_build<float><<<grid, 256, 0, s>>>(op.idx, (const float*)op.val, op.nnz, op.idx_ilv,
                                                        (float*)op.val_ilv);
                break;
            case MLEM_VAL_F16:
                k_ilv_build<__half><<<grid, 256, 0, s>>>(op.idx, (const __half*)op.val, op.nnz, op.idx_ilv,
                                                         (__half*)op.val_ilv);
                break;
            default:
                k_ilv_build<__nv_bfloat16><<<grid, 256, 0, s>>>(op.idx, (const __nv_bfloat16*)op.val, op.nnz,
                                                                op.idx_ilv, (__nv_bfloat16*)op.val_ilv);
        }
        MLEM_LAUNCHED();
    }
    MLEM_CUDA(cudaStreamSynchronize(s));
}

void launch_csr_ilv(const DevCsr& op, const float* x, const EpiArgs& epi, int unroll, L2Window win,
                    cudaStream_t s) {
    if (op.nrows == 0) return;
    MLEM_REQUIRE(op.idx_ilv != nullptr, MLEM_EINVAL, "operand has no interleaved copy");
    switch (op.vt) {
        case MLEM_VAL_F32: ilv_u<float>(op, x, epi, unroll, win, s); break;
        case MLEM_VAL_F16: ilv_u<__half>(op, x, epi, unroll, win, s); break;
        default: ilv_u<__nv_bfloat16>(op, x, epi, unroll, win, s);
    }
}

}  // namespace mlem
