// batch.cu — many sinograms against one resident matrix (batched SpMM).
//
// The matrix stream is shared by the instances of a tile (BT = 8, 16 or 32
// slots, interleaved: slot b of voxel c is f[c*BT + b]).  A launch covers the
// first W slots (the active width, 4..BT, the smallest power of two holding
// every slot with iterations left): a row is handled by a segment of W lanes
// of a warp (32/W rows per warp); each lane owns 4 instances of a nonzero and
// reads their image entries with one 16-byte load, so W/4 lanes cover a
// nonzero and a segment takes 4 nonzeros per gather instruction.  The
// segment's lanes load the row 32 entries at a time (coalesced) and broadcast
// them with shuffles.
//
// Every instance sums its row in 4 chains — nonzero k of the row goes to
// chain k mod 4, each chain a sequential FMA chain in k order — combined as
// (c0 + c1) + (c2 + c3).  That order depends on neither W nor BT nor the slot,
// so an instance gives the same bits alone and in a full batch, in any tile.
//
// Per-slot iteration counters live on the device (remaining[b]); an
// iteration is FP, BP+update and a counter tick, replayable as one CUDA
// graph per width; a slot whose counter reached 0 is no longer updated.
#include "kernels.cuh"

#include <algorithm>

namespace mlem {

namespace {

// Row sums of one warp's 32/W rows (segment seg of W lanes holds row `row`,
// `ok` = the row exists).  On return the lanes sl < W/4 of each segment hold
// instances 4*sl..4*sl+3 of their row.
// NC: the gathered state is read through the read-only path (__ldg), which is
// right only when no block of the same launch writes it; the persistent loop
// below, whose phases write what the next phase gathers, uses plain loads.
template <bool NC>
__device__ __forceinline__ float4 load_state(const float* p) {
    if (NC) return __ldg(reinterpret_cast<const float4*>(p));
    return *reinterpret_cast<const float4*>(p);
}

template <typename V, int W, bool NC = true>
__device__ __forceinline__ void batch_rows(const uint64_t* __restrict__ rowptr, const uint32_t* __restrict__ idx,
                                           const V* __restrict__ val, const float* x, uint32_t BT,
                                           uint32_t row, bool ok, int lane, float4& acc) {
    constexpr int LPN = W / 4;  // lanes per nonzero
    constexpr int E = 32 / W;   // entries per lane per 32-entry chunk
    const int sl = lane % W, chain = sl / LPN, q4 = (sl % LPN) * 4, seg0 = lane - sl;
    uint64_t s = 0, t = 0;
    if (ok) {
        s = rowptr[row];
        t = rowptr[row + 1];
    }
    // the warp runs as many chunks as its longest row needs (shuffles stay converged)
    uint32_t chunks = (uint32_t)((t - s + 31) >> 5);
#pragma unroll
    for (int o = W; o < 32; o <<= 1) chunks = max(chunks, __shfl_xor_sync(0xffffffffu, chunks, o));
    for (uint32_t ch = 0; ch < chunks; ++ch) {
        const uint64_t base = s + 32ull * ch;
        // entry base + sl + i*W sits in slot i of lane sl
        uint32_t c[E];
        float v[E];
#pragma unroll
        for (int i = 0; i < E; ++i) {
            const uint64_t e = base + sl + (uint64_t)i * W;
            c[i] = 0;
            v[i] = 0.f;
            if (e < t) {
                c[i] = ld_stream(idx + e);
                v[i] = Val4<V>::one(val, e);
            }
        }
        // entries of this row left in the chunk, less the chain offset
        const int64_t left = (int64_t)t - (int64_t)base;
        const int r = (int)(left < 0 ? 0 : left > 32 ? 32 : left) - chain;
        // trip q: nonzero k = 4q + chain of the chunk, held by lane k % W in
        // slot k / W = 4q / W; k % W = 4q % W + chain since chain < 4 <= W
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            if (W == 32 && 4 * q >= r + chain) break;  // one row per warp: uniform
            const int src = seg0 + chain + (4 * q) % W;
            const uint32_t ck = __shfl_sync(0xffffffffu, c[(4 * q) / W], src);
            const float vk = __shfl_sync(0xffffffffu, v[(4 * q) / W], src);
            if (4 * q < r) {
                const float4 xv = load_state<NC>(x + (uint64_t)ck * BT + q4);
                acc.x = fmaf(vk, xv.x, acc.x);
                acc.y = fmaf(vk, xv.y, acc.y);
                acc.z = fmaf(vk, xv.z, acc.z);
                acc.w = fmaf(vk, xv.w, acc.w);
            }
        }
    }
    // (c0 + c1) + (c2 + c3): chains sit LPN lanes apart inside the segment
#pragma unroll
    for (int o = LPN; o < W; o <<= 1) {
        acc.x += __shfl_xor_sync(0xffffffffu, acc.x, o);
        acc.y += __shfl_xor_sync(0xffffffffu, acc.y, o);
        acc.z += __shfl_xor_sync(0xffffffffu, acc.z, o);
        acc.w += __shfl_xor_sync(0xffffffffu, acc.w, o);
    }
}

__device__ __forceinline__ float correl1(int32_t g, float fp) { return (fp != 0.0f) ? __fdiv_rn((float)g, fp) : 0.0f; }

__device__ __forceinline__ float update1(float f, float acc, float n) {
    const float t = __fmul_rn(f, acc);
    return (n == 0.0f) ? t : __fdiv_rn(t, n);
}

// ratio[row*BT + b] = g/(A f)_b for the first W slots.
template <typename V, int W>
__global__ void __launch_bounds__(256)
k_batch_fp(const uint64_t* __restrict__ rowptr, const uint32_t* __restrict__ idx,
           const V* __restrict__ val, const float* __restrict__ f, uint32_t rows, uint32_t BT,
           const int32_t* __restrict__ g, float* __restrict__ ratio) {
    const int lane = threadIdx.x & 31;
    const uint64_t first = ((blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5) * (32 / W);
    if (first >= rows) return;  // whole warp
    const uint64_t row = first + lane / W;
    const bool ok = row < rows;
    float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
    batch_rows<V, W>(rowptr, idx, val, f, BT, (uint32_t)row, ok, lane, acc);
    const int sl = lane % W;
    if (ok && sl < W / 4) {
        const uint64_t o = row * BT + sl * 4;
        const int4 gg = *reinterpret_cast<const int4*>(g + o);
        *reinterpret_cast<float4*>(ratio + o) =
            make_float4(correl1(gg.x, acc.x), correl1(gg.y, acc.y), correl1(gg.z, acc.z), correl1(gg.w, acc.w));
    }
}

// f[c*BT + b] = f·(Aᵀ ratio)_b / norm[c] for the slots b < W with iterations left.
template <typename V, int W>
__global__ void __launch_bounds__(256)
k_batch_bp(const uint64_t* __restrict__ rowptr, const uint32_t* __restrict__ idx,
           const V* __restrict__ val, const float* __restrict__ ratio, uint32_t cols, uint32_t BT,
           const float* __restrict__ norm, const uint32_t* __restrict__ remaining,
           float* __restrict__ f) {
    const int lane = threadIdx.x & 31;
    const uint64_t first = ((blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5) * (32 / W);
    if (first >= cols) return;  // whole warp
    const uint64_t c = first + lane / W;
    const bool ok = c < cols;
    float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
    batch_rows<V, W>(rowptr, idx, val, ratio, BT, (uint32_t)c, ok, lane, acc);
    const int sl = lane % W;
    if (ok && sl < W / 4) {
        const uint64_t o = c * BT + sl * 4;
        const uint4 rem = *reinterpret_cast<const uint4*>(remaining + sl * 4);
        const float n = norm[c];
        float4 fv = *reinterpret_cast<const float4*>(f + o);
        if (rem.x) fv.x = update1(fv.x, acc.x, n);
        if (rem.y) fv.y = update1(fv.y, acc.y, n);
        if (rem.z) fv.z = update1(fv.z, acc.z, n);
        if (rem.w) fv.w = update1(fv.w, acc.w, n);
        *reinterpret_cast<float4*>(f + o) = fv;
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
            c = ld_stream(idx + e);
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

// Persistent batched MLEM: `steps` iterations of the tile in one cooperative
// launch (every block resident).  Per iteration: forward projection and
// correlation over all rows of A, grid barrier, back projection and update
// over all rows of Aᵀ for the slots with iterations left, grid barrier, tick
// of the per-slot counters by block 0.  The warps of the grid stride over
// row groups; each row is summed exactly as by k_batch_fp / k_batch_bp (same
// chains, same order), so an instance's bits do not depend on which kernel
// form runs it.
template <typename V, int W>
__global__ void __launch_bounds__(256, W == 32 ? 8 : 6)
k_batch_loop(const uint64_t* __restrict__ rp, const uint32_t* __restrict__ ix, const V* __restrict__ vl,
             uint32_t rows, const uint64_t* __restrict__ rpT, const uint32_t* __restrict__ ixT,
             const V* __restrict__ vlT, uint32_t cols, const float* __restrict__ norm, uint32_t BT,
             const int32_t* __restrict__ g, float* f, float* ratio, uint32_t* remaining, uint32_t steps,
             unsigned* count, int* err) {
    constexpr uint32_t RPW = 32 / W;  // rows per warp
    const int lane = threadIdx.x & 31, sl = lane % W;
    // 32-bit row counters (rows, cols < 2^32; a resident grid has < 2^16 warps)
    const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t stride = ((gridDim.x * blockDim.x) >> 5) * RPW;
    unsigned k = 0;
    for (uint32_t step = 0; step < steps; ++step) {
        for (uint32_t first = warp * RPW; first < rows; first += stride) {
            const uint32_t row = first + lane / W;
            const bool ok = row < rows;
            float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
            batch_rows<V, W, false>(rp, ix, vl, f, BT, row, ok, lane, acc);
            if (ok && sl < W / 4) {
                const uint64_t o = (uint64_t)row * BT + sl * 4;
                const int4 gg = *reinterpret_cast<const int4*>(g + o);
                *reinterpret_cast<float4*>(ratio + o) = make_float4(correl1(gg.x, acc.x), correl1(gg.y, acc.y),
                                                                    correl1(gg.z, acc.z), correl1(gg.w, acc.w));
            }
        }
        if (!grid_barrier(count, ++k, err)) return;
        for (uint32_t first = warp * RPW; first < cols; first += stride) {
            const uint32_t c = first + lane / W;
            const bool ok = c < cols;
            float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
            batch_rows<V, W, false>(rpT, ixT, vlT, ratio, BT, c, ok, lane, acc);
            if (ok && sl < W / 4) {
                const uint64_t o = (uint64_t)c * BT + sl * 4;
                const uint4 rem = *reinterpret_cast<const uint4*>(remaining + sl * 4);
                const float n = norm[c];
                float4 fv = *reinterpret_cast<const float4*>(f + o);
                if (rem.x) fv.x = update1(fv.x, acc.x, n);
                if (rem.y) fv.y = update1(fv.y, acc.y, n);
                if (rem.z) fv.z = update1(fv.z, acc.z, n);
                if (rem.w) fv.w = update1(fv.w, acc.w, n);
                *reinterpret_cast<float4*>(f + o) = fv;
            }
        }
        if (!grid_barrier(count, ++k, err)) return;
        // every block has read `remaining` for this iteration; the tick is seen
        // by the next back projection through the next barrier
        if (blockIdx.x == 0 && threadIdx.x < BT && remaining[threadIdx.x] > 0) remaining[threadIdx.x] -= 1;
    }
}

template <int W, typename V>
void fp_w(const DevCsr& A, const BatchArgs& b, L2Window win, cudaStream_t s) {
    launch_ex(k_batch_fp<V, W>, dim3(ceil_div_u((uint64_t)A.nrows * W, 256)), dim3(256), 0, s, win, A.rowptr,
              A.idx, static_cast<const V*>(A.val), (const float*)b.f, A.nrows, b.tile, b.g, b.ratio);
}

template <int W, typename V>
void bp_w(const DevCsr& AT, const float* norm, const BatchArgs& b, L2Window win, cudaStream_t s) {
    launch_ex(k_batch_bp<V, W>, dim3(ceil_div_u((uint64_t)AT.nrows * W, 256)), dim3(256), 0, s, win, AT.rowptr,
              AT.idx, static_cast<const V*>(AT.val), (const float*)b.ratio, AT.nrows, b.tile, norm,
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
    switch (b.width()) {
        case 4: fp_w<4, V>(A, b, win, s); break;
        case 8: fp_w<8, V>(A, b, win, s); break;
        case 16: fp_w<16, V>(A, b, win, s); break;
        default: fp_w<32, V>(A, b, win, s);
    }
}
template <typename V>
void bp_v(const DevCsr& AT, const float* norm, const BatchArgs& b, L2Window win, cudaStream_t s) {
    switch (b.width()) {
        case 4: bp_w<4, V>(AT, norm, b, win, s); break;
        case 8: bp_w<8, V>(AT, norm, b, win, s); break;
        case 16: bp_w<16, V>(AT, norm, b, win, s); break;
        default: bp_w<32, V>(AT, norm, b, win, s);
    }
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

namespace {

template <typename V, int W>
void loop_w(const DevCsr& A, const DevCsr& AT, const float* norm, const BatchArgs& b, uint32_t steps,
            unsigned* count, int* err, cudaStream_t s) {
    auto kern = k_batch_loop<V, W>;
    // one resident wave: every block must be on the GPU at once for the barriers
    static const int bps = [kern] {
        int b = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, kern, 256, 0) != cudaSuccess) {
            cudaGetLastError();
            b = 0;
        }
        return b;
    }();
    int dev = 0, sms = 0;
    MLEM_CUDA(cudaGetDevice(&dev));
    MLEM_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    MLEM_REQUIRE(bps >= 1, MLEM_EUNSUPPORTED, "persistent batch kernel does not fit on an SM");
    MLEM_CUDA(cudaMemsetAsync(count, 0, sizeof(unsigned), s));
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)(bps * sms));
    cfg.blockDim = dim3(256);
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    MLEM_CUDA(cudaLaunchKernelEx(&cfg, kern, (const uint64_t*)A.rowptr, (const uint32_t*)A.idx,
                                 static_cast<const V*>(A.val), A.nrows, (const uint64_t*)AT.rowptr,
                                 (const uint32_t*)AT.idx, static_cast<const V*>(AT.val), AT.nrows, norm, b.tile,
                                 b.g, b.f, b.ratio, b.remaining, steps, count, err));
    count_launch();
}

template <typename V>
void loop_v(const DevCsr& A, const DevCsr& AT, const float* norm, const BatchArgs& b, uint32_t steps,
            unsigned* count, int* err, cudaStream_t s) {
    switch (b.width()) {
        case 4: loop_w<V, 4>(A, AT, norm, b, steps, count, err, s); break;
        case 8: loop_w<V, 8>(A, AT, norm, b, steps, count, err, s); break;
        case 16: loop_w<V, 16>(A, AT, norm, b, steps, count, err, s); break;
        default: loop_w<V, 32>(A, AT, norm, b, steps, count, err, s);
    }
}

}  // namespace

void launch_batch_loop(const DevCsr& A, const DevCsr& AT, const float* norm, const BatchArgs& b, uint32_t steps,
                       unsigned* count, int* err, cudaStream_t s) {
    if (steps == 0 || A.nrows == 0) return;
    switch (A.vt) {
        case MLEM_VAL_F32: loop_v<float>(A, AT, norm, b, steps, count, err, s); break;
        case MLEM_VAL_F16: loop_v<__half>(A, AT, norm, b, steps, count, err, s); break;
        default: loop_v<__nv_bfloat16>(A, AT, norm, b, steps, count, err, s);
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
