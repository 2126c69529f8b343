// spmv_d16.cu — projections over 16-bit delta-coded column indices (D16).
//
// A row is cut into steps of 8·L entries, L = op.d16_lanes (4 or 8) lanes per
// row: position p of a row belongs to lane p % L as element p / L of that
// lane's sequence, so one gather instruction covers L consecutive entries of
// the row (few cache lines: its columns are ascending and close).  Each entry
// stores the difference between its column and the column L positions earlier
// (the previous element of the same lane; the row's first column for the first
// L positions): every lane decodes its own columns with one add per entry, no
// scans and no shuffles.  Layout of an operand in D16 form (beside the u32 CSR):
//   dvptr[r]  first 8-entry vector of row r (u64[nrows + 1]); vector
//             dvptr[r] + k·L + l holds lane l's elements 8k..8k+7
//   dbase[r]  first column of row r
//   d16[8 v + j], dval[8 v + j]  the delta and the value (the operand's type)
// A difference of 65,536 or more is bridged by dummy entries (value 0,
// column = the earlier column + 65,535); rows are padded to whole steps with
// delta 0 and value 0.  Dummies and padding add 4% (L = 4) to 9% (L = 8) on
// the generated matrices in the locality layout: with FP16 values ~4.2 bytes
// per nonzero instead of 8 (u32 + f32).  The lane sums are reduced by a fixed
// xor tree: deterministic.
#include "kernels.cuh"

#include <algorithm>
#include <cstring>
#include <vector>

namespace mlem {

namespace {

template <typename V>
struct Val8;

template <>
struct Val8<float> {
    static __device__ __forceinline__ void load(const float* p, uint64_t v, float out[8]) {
        const float4* q = reinterpret_cast<const float4*>(p) + 2 * v;
        const float4 a = ld_stream(q), b = ld_stream(q + 1);
        out[0] = a.x; out[1] = a.y; out[2] = a.z; out[3] = a.w;
        out[4] = b.x; out[5] = b.y; out[6] = b.z; out[7] = b.w;
    }
};

template <>
struct Val8<__half> {
    static __device__ __forceinline__ void load(const __half* p, uint64_t v, float out[8]) {
        const uint4 u = ld_stream(reinterpret_cast<const uint4*>(p) + v);
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
        const uint4 u = ld_stream(reinterpret_cast<const uint4*>(p) + v);
        const uint32_t w[4] = {u.x, u.y, u.z, u.w};
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const float2 f = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(&w[k]));
            out[2 * k] = f.x;
            out[2 * k + 1] = f.y;
        }
    }
};

template <typename V, int EPI, int LPR, int U>
__global__ void __launch_bounds__(256)
k_csr_d16(const uint64_t* __restrict__ dvptr, const uint32_t* __restrict__ dbase, const uint16_t* __restrict__ d16,
          const V* __restrict__ dval, const float* __restrict__ x, uint32_t nrows, const int32_t* __restrict__ g,
          float* __restrict__ out, float* __restrict__ fwproj, float* __restrict__ f, const float* __restrict__ norm) {
    const uint32_t row = (blockIdx.x * blockDim.x + threadIdx.x) / LPR;
    const uint32_t gl = threadIdx.x % LPR;
    const bool live = row < nrows;
    const uint64_t v0 = live ? dvptr[row] : 0, v1 = live ? dvptr[row + 1] : 0;
    const uint32_t nsteps = (uint32_t)((v1 - v0) / LPR);
    const uint4* dv = reinterpret_cast<const uint4*>(d16);
    if (live && gl == 0 && v1 > v0) {
        // the row's vectors into L2 ahead of the loads (whole 16-byte vectors)
        const uint64_t lo = reinterpret_cast<uint64_t>(dv + v0), nb = 16 * (v1 - v0);
        const uint64_t lv = reinterpret_cast<uint64_t>(dval) + 8 * sizeof(V) * v0, nv = 8 * sizeof(V) * (v1 - v0);
        for (uint64_t q = 0; q < nb; q += 65536)
            asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(lo + q),
                         "r"((uint32_t)(nb - q < 65536 ? nb - q : 65536)) : "memory");
        for (uint64_t q = 0; q < nv; q += 65536)
            asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(lv + q),
                         "r"((uint32_t)(nv - q < 65536 ? nv - q : 65536)) : "memory");
    }
    uint32_t prev = live ? dbase[row] : 0u;  // column of this lane's previous element
    float acc = 0.f;
    for (uint32_t k = 0; k < nsteps; k += U) {
        uint4 dw[U];
        float a[U][8];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            if (k + u < nsteps) {
                const uint64_t v = v0 + (uint64_t)(k + u) * LPR + gl;
                dw[u] = ld_stream(dv + v);
                Val8<V>::load(dval, v, a[u]);
            } else {
                dw[u] = make_uint4(0u, 0u, 0u, 0u);
#pragma unroll
                for (int j = 0; j < 8; ++j) a[u][j] = 0.f;
            }
        }
        uint32_t col[U][8];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const uint32_t w[4] = {dw[u].x, dw[u].y, dw[u].z, dw[u].w};
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                prev += (w[j >> 1] >> (16 * (j & 1))) & 0xFFFFu;
                col[u][j] = prev;
            }
        }
        float gx[U][8];
#pragma unroll
        for (int u = 0; u < U; ++u)
#pragma unroll
            for (int j = 0; j < 8; ++j) gx[u][j] = (k + u < nsteps) ? __ldg(x + col[u][j]) : 0.f;
#pragma unroll
        for (int u = 0; u < U; ++u)
#pragma unroll
            for (int j = 0; j < 8; ++j) acc = fmaf(a[u][j], gx[u][j], acc);
    }
#pragma unroll
    for (int o = LPR / 2; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o, LPR);
    if (live && gl == 0) {
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
// Sets *unsorted when some row lists a column below its predecessor.
__global__ void k_d16_check(const uint64_t* __restrict__ rowptr, const uint32_t* __restrict__ col, uint32_t rows,
                            int* __restrict__ unsorted) {
    const int lane = threadIdx.x & 31;
    const uint32_t nw = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t r = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < rows; r += nw) {
        const uint64_t s = rowptr[r], t = rowptr[r + 1];
        bool bad = false;
        for (uint64_t e = s + 1 + lane; e < t; e += 32) bad |= col[e] < col[e - 1];
        if (__any_sync(0xffffffffu, bad) && lane == 0) atomicOr(unsorted, 1);
    }
}

// Walks row r's positions: a dummy wherever the next column is 65,536 or more
// past the column L positions earlier.  emit(p, delta, e) for every position
// (e = entry index, or ~0 for a dummy); returns the positions used.
template <int L, class Emit>
__device__ __forceinline__ uint64_t d16_walk(const uint32_t* __restrict__ col, uint64_t s, uint64_t t, Emit&& emit) {
    if (s == t) return 0;
    uint32_t ring[L];
#pragma unroll
    for (int i = 0; i < L; ++i) ring[i] = col[s];
    uint64_t p = 0;
    for (uint64_t e = s; e < t;) {
        uint32_t earlier = ring[0];
#pragma unroll
        for (int i = 1; i < L; ++i)
            if ((p % L) == (uint64_t)i) earlier = ring[i];
        const uint32_t c = col[e];
        uint32_t now, d;
        uint64_t ent;
        if (c - earlier >= 65536u) {
            now = earlier + 65535u;
            d = 65535u;
            ent = ~0ull;
        } else {
            now = c;
            d = c - earlier;
            ent = e;
            ++e;
        }
        emit(p, d, ent);
#pragma unroll
        for (int i = 0; i < L; ++i)
            if ((p % L) == (uint64_t)i) ring[i] = now;
        ++p;
    }
    return p;
}

// Vectors per row (positions rounded up to whole steps of 8·L).  One thread per row.
template <int L>
__global__ void k_d16_count(const uint64_t* __restrict__ rowptr, const uint32_t* __restrict__ col, uint32_t rows,
                            uint32_t* __restrict__ nvec) {
    for (uint32_t r = blockIdx.x * blockDim.x + threadIdx.x; r < rows; r += gridDim.x * blockDim.x) {
        const uint64_t n = d16_walk<L>(col, rowptr[r], rowptr[r + 1], [](uint64_t, uint32_t, uint64_t) {});
        nvec[r] = (uint32_t)((n + 8 * L - 1) / (8 * L) * L);
    }
}

// Deltas and values at their positions (the arrays are zeroed beforehand,
// which is the padding).  One thread per row.
template <typename V, int L>
__global__ void k_d16_fill(const uint64_t* __restrict__ rowptr, const uint32_t* __restrict__ col,
                           const V* __restrict__ val, uint32_t rows, const uint64_t* __restrict__ dvptr,
                           uint32_t* __restrict__ dbase, uint16_t* __restrict__ d16, V* __restrict__ dval) {
    for (uint32_t r = blockIdx.x * blockDim.x + threadIdx.x; r < rows; r += gridDim.x * blockDim.x) {
        const uint64_t s = rowptr[r], t = rowptr[r + 1], v0 = dvptr[r];
        dbase[r] = s < t ? col[s] : 0u;
        d16_walk<L>(col, s, t, [&](uint64_t p, uint32_t d, uint64_t e) {
            // position p: step p / (8L), lane p % L, element (p / L) % 8
            const uint64_t v = v0 + (p / (8 * L)) * L + p % L, q = 8 * v + (p / L) % 8;
            d16[q] = (uint16_t)d;
            if (e != ~0ull) dval[q] = val[e];
        });
    }
}

unsigned grid_rows(uint32_t rows) {
    return std::max(1u, std::min<unsigned>(ceil_div_u((uint64_t)rows * 32, 256), 152u * 32u));
}

unsigned grid_threads(uint32_t rows) {
    return std::max(1u, std::min<unsigned>(ceil_div_u(rows, 128), 152u * 32u));
}

template <typename V>
void d16_fill(DevCsr& op, const uint32_t* idx, const void* val, cudaStream_t s) {
    if (op.d16_lanes == 4)
        k_d16_fill<V, 4><<<grid_threads(op.nrows), 128, 0, s>>>(op.rowptr, idx, static_cast<const V*>(val), op.nrows,
                                                                op.dvptr, op.dbase, op.d16, static_cast<V*>(op.dval));
    else
        k_d16_fill<V, 8><<<grid_threads(op.nrows), 128, 0, s>>>(op.rowptr, idx, static_cast<const V*>(val), op.nrows,
                                                                op.dvptr, op.dbase, op.d16, static_cast<V*>(op.dval));
    MLEM_LAUNCHED();
}

// A copy of the operand's entries with every row sorted by column (stable),
// made on the host: only for rows given out of order (generated and
// transposed operands are sorted already).
void sorted_copy(const DevCsr& op, uint32_t*& idx, void*& val, cudaStream_t s) {
    const size_t vb = val_bytes(op.vt);
    std::vector<uint64_t> rp(op.nrows + 1);
    std::vector<uint32_t> c(op.nnz);
    std::vector<unsigned char> v(op.nnz * vb);
    MLEM_CUDA(cudaMemcpyAsync(rp.data(), op.rowptr, sizeof(uint64_t) * rp.size(), cudaMemcpyDeviceToHost, s));
    MLEM_CUDA(cudaMemcpyAsync(c.data(), op.idx, sizeof(uint32_t) * op.nnz, cudaMemcpyDeviceToHost, s));
    MLEM_CUDA(cudaMemcpyAsync(v.data(), op.val, vb * op.nnz, cudaMemcpyDeviceToHost, s));
    MLEM_CUDA(cudaStreamSynchronize(s));
    std::vector<uint32_t> c2(op.nnz);
    std::vector<unsigned char> v2(op.nnz * vb);
#pragma omp parallel
    {
        std::vector<uint64_t> perm;
#pragma omp for schedule(dynamic, 64)
        for (int64_t r = 0; r < (int64_t)op.nrows; ++r) {
            const uint64_t a = rp[r], b = rp[r + 1];
            perm.resize(b - a);
            for (uint64_t e = a; e < b; ++e) perm[e - a] = e;
            std::stable_sort(perm.begin(), perm.end(), [&](uint64_t x, uint64_t y) { return c[x] < c[y]; });
            for (uint64_t k = 0; k < b - a; ++k) {
                c2[a + k] = c[perm[k]];
                std::memcpy(&v2[(a + k) * vb], &v[perm[k] * vb], vb);
            }
        }
    }
    MLEM_CUDA(cudaMalloc(&idx, sizeof(uint32_t) * std::max<uint64_t>(op.nnz, 1)));
    MLEM_CUDA(cudaMalloc(&val, vb * std::max<uint64_t>(op.nnz, 1)));
    MLEM_CUDA(cudaMemcpyAsync(idx, c2.data(), sizeof(uint32_t) * op.nnz, cudaMemcpyHostToDevice, s));
    MLEM_CUDA(cudaMemcpyAsync(val, v2.data(), vb * op.nnz, cudaMemcpyHostToDevice, s));
    MLEM_CUDA(cudaStreamSynchronize(s));
}

template <typename V, int EPI, int LPR, int U>
void d16_launch(const DevCsr& op, const float* x, const EpiArgs& e, L2Window win, cudaStream_t s) {
    launch_ex(k_csr_d16<V, EPI, LPR, U>, dim3(ceil_div_u((uint64_t)op.nrows * LPR, 256)), dim3(256), 0, s, win,
              op.dvptr, op.dbase, op.d16, static_cast<const V*>(op.dval), x, op.nrows, e.g, e.out, e.fwproj, e.f,
              e.norm);
}

template <typename V, int EPI>
void d16_shape(const DevCsr& op, const float* x, const EpiArgs& e, int unroll, L2Window win, cudaStream_t s) {
    if (op.d16_lanes == 4) {
        if (unroll >= 2) d16_launch<V, EPI, 4, 2>(op, x, e, win, s);
        else d16_launch<V, EPI, 4, 1>(op, x, e, win, s);
    } else {
        if (unroll >= 2) d16_launch<V, EPI, 8, 2>(op, x, e, win, s);
        else d16_launch<V, EPI, 8, 1>(op, x, e, win, s);
    }
}

template <typename V>
void d16_dispatch(const DevCsr& op, const float* x, const EpiArgs& e, int unroll, L2Window win, cudaStream_t s) {
    switch (e.kind) {
        case Epi::Correl: d16_shape<V, (int)Epi::Correl>(op, x, e, unroll, win, s); break;
        case Epi::Update: d16_shape<V, (int)Epi::Update>(op, x, e, unroll, win, s); break;
        default: d16_shape<V, (int)Epi::Raw>(op, x, e, unroll, win, s);
    }
}

}  // namespace

void build_d16(DevCsr& op, cudaStream_t s) {
    const uint64_t R = std::max<uint32_t>(op.nrows, 1);
    // 4 lanes per row for short rows, 8 for long ones (the padding to whole
    // steps of 8 L entries costs less than 10% either way)
    op.d16_lanes = op.nrows && op.nnz / op.nrows >= 256 ? 8 : 4;
    // deltas need every row in ascending column order
    const uint32_t* idx = op.idx;
    const void* val = op.val;
    uint32_t* sidx = nullptr;
    void* sval = nullptr;
    int* flag = nullptr;
    int unsorted = 0;
    MLEM_CUDA(cudaMallocAsync(&flag, sizeof(int), s));
    MLEM_CUDA(cudaMemsetAsync(flag, 0, sizeof(int), s));
    if (op.nrows) {
        k_d16_check<<<grid_rows(op.nrows), 256, 0, s>>>(op.rowptr, op.idx, op.nrows, flag);
        MLEM_LAUNCHED();
    }
    MLEM_CUDA(cudaMemcpyAsync(&unsorted, flag, sizeof(int), cudaMemcpyDeviceToHost, s));
    MLEM_CUDA(cudaFreeAsync(flag, s));
    MLEM_CUDA(cudaStreamSynchronize(s));
    if (unsorted) {
        sorted_copy(op, sidx, sval, s);
        idx = sidx;
        val = sval;
    }
    uint32_t* nvec = nullptr;
    try {
        MLEM_CUDA(cudaMallocAsync(&nvec, sizeof(uint32_t) * R, s));
        MLEM_CUDA(cudaMalloc(&op.dvptr, sizeof(uint64_t) * (R + 1)));
        if (op.nrows) {
            if (op.d16_lanes == 4) k_d16_count<4><<<grid_threads(op.nrows), 128, 0, s>>>(op.rowptr, idx, op.nrows, nvec);
            else k_d16_count<8><<<grid_threads(op.nrows), 128, 0, s>>>(op.rowptr, idx, op.nrows, nvec);
            MLEM_LAUNCHED();
        }
        scan_counts_u64(nvec, op.dvptr, op.nrows, s);
        uint64_t nv = 0;
        MLEM_CUDA(cudaMemcpyAsync(&nv, op.dvptr + op.nrows, sizeof(uint64_t), cudaMemcpyDeviceToHost, s));
        MLEM_CUDA(cudaStreamSynchronize(s));
        op.dvec = nv;
        const uint64_t slots = 8 * std::max<uint64_t>(nv, 1);
        MLEM_CUDA(cudaMalloc(&op.dbase, sizeof(uint32_t) * R));
        MLEM_CUDA(cudaMalloc(&op.d16, sizeof(uint16_t) * slots));
        MLEM_CUDA(cudaMalloc(&op.dval, val_bytes(op.vt) * slots));
        MLEM_CUDA(cudaMemsetAsync(op.d16, 0, sizeof(uint16_t) * slots, s));
        MLEM_CUDA(cudaMemsetAsync(op.dval, 0, val_bytes(op.vt) * slots, s));
        if (op.nrows) {
            switch (op.vt) {
                case MLEM_VAL_F32: d16_fill<float>(op, idx, val, s); break;
                case MLEM_VAL_F16: d16_fill<__half>(op, idx, val, s); break;
                default: d16_fill<__nv_bfloat16>(op, idx, val, s);
            }
        }
        MLEM_CUDA(cudaStreamSynchronize(s));
    } catch (...) {
        cudaStreamSynchronize(s);
        cudaFree(nvec);
        cudaFree(sidx);
        cudaFree(sval);
        throw;
    }
    cudaFree(nvec);
    cudaFree(sidx);
    cudaFree(sval);
}

void launch_csr_d16(const DevCsr& op, const float* x, const EpiArgs& epi, int unroll, L2Window win, cudaStream_t s) {
    if (op.nrows == 0) return;
    MLEM_REQUIRE(op.d16 != nullptr, MLEM_EINVAL, "operand has no D16 indices");
    switch (op.vt) {
        case MLEM_VAL_F32: d16_dispatch<float>(op, x, epi, unroll, win, s); break;
        case MLEM_VAL_F16: d16_dispatch<__half>(op, x, epi, unroll, win, s); break;
        default: d16_dispatch<__nv_bfloat16>(op, x, epi, unroll, win, s);
    }
}

}  // namespace mlem
