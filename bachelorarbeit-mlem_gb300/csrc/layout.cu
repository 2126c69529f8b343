// layout.cu — the locality layout of a matrix and the permutations at the
// entry points.
//
// With the locality layout the device operands are A' = P_L A P_Vᵀ: rows
// (LORs) in 4x4 detector-tube order, columns (voxels) in 4x4x2 brick order,
// every row's columns ascending again.  MLEM is invariant under the
// relabelling (ratio' = P_L ratio, f' = P_V f, norm' = P_V norm), so whole
// reconstructions run in the permuted space and only the sinogram, the images
// and single projections are permuted where they cross the C ABI.  Nearby
// LORs then gather nearby voxels from the same cache lines (and nearby voxels
// the ratios of nearby LORs), which lowers the L1 line lookups per nonzero of
// both projections.
//
// Rows of a matrix the library did not generate (no detector numbering to
// build tubes from) are ordered from the matrix itself: by the coarse voxel
// cells (about 1/12 of the grid across, 1/10 along z) of their lowest and of
// their highest column, so LORs that enter and leave the grid at nearly the
// same places — nearly parallel neighbours, like a detector tube — sit next to
// each other.
//
// Construction: rows are copied in the new order with the column map
// applied, then two stable transposes (transpose.cu) sort the columns of
// every row; the intermediate transpose is exactly the transpose of A' and is
// kept as Aᵀ.
#include "kernels.cuh"

#include <algorithm>

namespace mlem {

namespace {

__global__ void k_row_lengths(const uint64_t* __restrict__ rowptr, const uint32_t* __restrict__ row_src,
                              uint32_t rows, uint32_t* __restrict__ len) {
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < rows; k += gridDim.x * blockDim.x) {
        const uint32_t r = row_src ? row_src[k] : k;
        len[k] = (uint32_t)(rowptr[r + 1] - rowptr[r]);
    }
}

// One warp per new row: copy the source row with the column map applied.
__global__ void k_row_copy(const uint64_t* __restrict__ rowptr, const uint32_t* __restrict__ idx,
                           const float* __restrict__ val, const uint32_t* __restrict__ row_src,
                           const uint32_t* __restrict__ col_map, uint32_t rows,
                           const uint64_t* __restrict__ out_ptr, uint32_t* __restrict__ out_idx,
                           float* __restrict__ out_val) {
    const uint32_t lane = threadIdx.x & 31;
    for (uint64_t k = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5; k < rows;
         k += ((uint64_t)gridDim.x * blockDim.x) >> 5) {
        const uint32_t r = row_src ? row_src[k] : (uint32_t)k;
        const uint64_t s = rowptr[r], n = rowptr[r + 1] - s, o = out_ptr[k];
        for (uint64_t t = lane; t < n; t += 32) {
            const uint32_t c = idx[s + t];
            out_idx[o + t] = col_map ? col_map[c] : c;
            out_val[o + t] = val[s + t];
        }
    }
}

template <typename T>
__global__ void k_gather(T* __restrict__ out, const T* __restrict__ in, const uint32_t* __restrict__ map,
                         uint64_t n) {
    for (uint64_t k = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; k < n; k += (uint64_t)gridDim.x * blockDim.x)
        out[k] = in[map[k]];
}

template <typename T>
__global__ void k_scatter_perm(T* __restrict__ out, const T* __restrict__ in, const uint32_t* __restrict__ map,
                               uint64_t n) {
    for (uint64_t k = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; k < n; k += (uint64_t)gridDim.x * blockDim.x)
        out[map[k]] = in[k];
}

__global__ void k_invert(const uint32_t* __restrict__ map, uint32_t n, uint32_t* __restrict__ inv) {
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) inv[map[k]] = k;
}

unsigned grid_of(uint64_t n) { return std::max(1u, std::min<unsigned>(ceil_div_u(n, 256), 152u * 16u)); }

// Lowest and highest column of every row (one warp per row; ~0u / 0 when empty).
__global__ void k_row_minmax(const uint64_t* __restrict__ rowptr, const uint32_t* __restrict__ idx, uint32_t rows,
                             uint2* __restrict__ mm) {
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t nw = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t r = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < rows; r += nw) {
        uint32_t lo = 0xffffffffu, hi = 0u;
        for (uint64_t e = rowptr[r] + lane; e < rowptr[r + 1]; e += 32) {
            const uint32_t c = idx[e];
            lo = min(lo, c);
            hi = max(hi, c);
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            lo = min(lo, __shfl_xor_sync(0xffffffffu, lo, o));
            hi = max(hi, __shfl_xor_sync(0xffffffffu, hi, o));
        }
        if (lane == 0) mm[r] = make_uint2(lo, hi);
    }
}

}  // namespace

std::vector<uint32_t> derived_lor_order(const DevCsr& A, uint32_t nx, uint32_t ny, uint32_t nz, cudaStream_t s) {
    std::vector<uint2> mm(A.nrows);
    uint2* d_mm = nullptr;
    MLEM_CUDA(cudaMalloc(&d_mm, sizeof(uint2) * std::max<uint32_t>(A.nrows, 1)));
    if (A.nrows) {
        const unsigned grid = std::max(1u, std::min<unsigned>(ceil_div_u((uint64_t)A.nrows * 32, 256), 152u * 32u));
        k_row_minmax<<<grid, 256, 0, s>>>(A.rowptr, A.idx, A.nrows, d_mm);
        MLEM_LAUNCHED();
        MLEM_CUDA(cudaMemcpyAsync(mm.data(), d_mm, sizeof(uint2) * A.nrows, cudaMemcpyDeviceToHost, s));
    }
    MLEM_CUDA(cudaStreamSynchronize(s));
    cudaFree(d_mm);
    const uint32_t qxy = std::max(4u, (std::max(nx, ny) + 6) / 12), qz = std::max(2u, (nz + 5) / 10);
    const uint64_t cx = (nx + qxy - 1) / qxy, cy = (ny + qxy - 1) / qxy, cz = (nz + qz - 1) / qz;
    const uint64_t ncell = cx * cy * cz;
    auto cell = [&](uint32_t c) -> uint64_t {
        const uint32_t x = c % nx, y = (c / nx) % ny, z = c / (nx * ny);
        return (uint64_t)(z / qz) * cx * cy + (uint64_t)(y / qxy) * cx + x / qxy;
    };
    std::vector<uint64_t> key(A.nrows);
    for (uint32_t r = 0; r < A.nrows; ++r)
        key[r] = mm[r].x > mm[r].y ? ~0ull : cell(mm[r].x) * ncell + cell(mm[r].y);  // empty rows last
    std::vector<uint32_t> ord(A.nrows);
    for (uint32_t r = 0; r < A.nrows; ++r) ord[r] = r;
    std::stable_sort(ord.begin(), ord.end(), [&](uint32_t a, uint32_t b) { return key[a] < key[b]; });
    return ord;
}

void launch_gather_i32(int32_t* out, const int32_t* in, const uint32_t* map, uint64_t n, cudaStream_t s) {
    if (n == 0) return;
    k_gather<int32_t><<<grid_of(n), 256, 0, s>>>(out, in, map, n);
    MLEM_LAUNCHED();
}

void launch_gather_f32(float* out, const float* in, const uint32_t* map, uint64_t n, cudaStream_t s) {
    if (n == 0) return;
    k_gather<float><<<grid_of(n), 256, 0, s>>>(out, in, map, n);
    MLEM_LAUNCHED();
}

void launch_scatter_f32(float* out, const float* in, const uint32_t* map, uint64_t n, cudaStream_t s) {
    if (n == 0) return;
    k_scatter_perm<float><<<grid_of(n), 256, 0, s>>>(out, in, map, n);
    MLEM_LAUNCHED();
}

void launch_invert_perm(const uint32_t* map, uint32_t n, uint32_t* inv, cudaStream_t s) {
    if (n == 0) return;
    k_invert<<<grid_of(n), 256, 0, s>>>(map, n, inv);
    MLEM_LAUNCHED();
}

void remap_csr(const DevCsr& in, const uint32_t* row_src, const uint32_t* col_map, DevCsr& out, DevCsr* keep_t,
               cudaStream_t s) {
    MLEM_REQUIRE(in.vt == MLEM_VAL_F32, MLEM_EINVAL, "remap expects f32 values");
    DevCsr R, T;
    R.nrows = in.nrows;
    R.ncols = in.ncols;
    R.nnz = in.nnz;
    R.vt = MLEM_VAL_F32;
    uint32_t* len = nullptr;
    try {
        MLEM_CUDA(cudaMalloc(&R.rowptr, sizeof(uint64_t) * ((uint64_t)R.nrows + 1)));
        MLEM_CUDA(cudaMalloc(&R.idx, sizeof(uint32_t) * padded(R.nnz)));
        MLEM_CUDA(cudaMalloc(&R.val, sizeof(float) * padded(R.nnz)));
        MLEM_CUDA(cudaMemsetAsync(R.idx, 0, sizeof(uint32_t) * padded(R.nnz), s));
        MLEM_CUDA(cudaMemsetAsync(R.val, 0, sizeof(float) * padded(R.nnz), s));
        MLEM_CUDA(cudaMalloc(&len, sizeof(uint32_t) * std::max<uint32_t>(R.nrows, 1)));
        if (R.nrows) {
            k_row_lengths<<<grid_of(R.nrows), 256, 0, s>>>(in.rowptr, row_src, R.nrows, len);
            MLEM_LAUNCHED();
        }
        scan_counts_u64(len, R.rowptr, R.nrows, s);
        if (R.nrows) {
            k_row_copy<<<grid_of((uint64_t)R.nrows * 32), 256, 0, s>>>(
                in.rowptr, in.idx, static_cast<const float*>(in.val), row_src, col_map, R.nrows, R.rowptr, R.idx,
                static_cast<float*>(R.val));
            MLEM_LAUNCHED();
        }
        transpose_device(R, T, s);  // rows = new columns, entries ascending by new row
        MLEM_CUDA(cudaStreamSynchronize(s));
        cudaFree(R.rowptr);
        cudaFree(R.idx);
        cudaFree(R.val);
        R = DevCsr();
        transpose_device(T, out, s);  // rows = new rows, columns ascending
        out.max_row = max_row_length(out.rowptr, out.nrows, s);
        MLEM_CUDA(cudaStreamSynchronize(s));
    } catch (...) {
        cudaStreamSynchronize(s);
        cudaFree(len);
        cudaFree(R.rowptr);
        cudaFree(R.idx);
        cudaFree(R.val);
        cudaFree(T.rowptr);
        cudaFree(T.idx);
        cudaFree(T.val);
        throw;
    }
    cudaFree(len);
    if (keep_t) {
        *keep_t = T;
    } else {
        cudaFree(T.rowptr);
        cudaFree(T.idx);
        cudaFree(T.val);
    }
}

}  // namespace mlem
