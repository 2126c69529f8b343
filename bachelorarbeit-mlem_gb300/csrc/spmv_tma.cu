// spmv_tma.cu — TMA-pipelined row-parallel projection (csr-vector switch).
//
// Same arithmetic contract as k_csrvec (spmv.cu): one warp owns a row, sums
// val*x[col] in a fixed order and applies the fused epilogue (correlation
// after the forward projection, multiplicative update after the back
// projection).  What changes is how the matrix reaches the SM: each warp runs
// a ring of STAGES shared-memory buffers; one elected lane streams the next
// chunks of its rows (CH elements of indices and values, 16-byte aligned,
// rows split at CH boundaries) with cp.async.bulk into the ring, completing on
// per-stage mbarriers, while the 32 lanes gather x[col] for the chunk that
// has landed.  The HBM stream therefore never waits on the gathers, and the
// row pointers are fetched 32 rows ahead.  Chunks never span rows, so every
// row sum has one deterministic order (lane-strided partials, xor tree).
//
// Every mbarrier wait is bounded: on expiry the warp records an error in
// *err, drains its own copies in flight (again bounded) and returns.
#include "kernels.cuh"
#include "scatter.cuh"
#include "tma.cuh"

#include <algorithm>
#include <map>
#include <mutex>

namespace mlem {

namespace {

constexpr int kTmaCh = 512;       // elements per chunk
constexpr int kTmaStages = 4;     // ring depth per warp
constexpr int kTmaWarps = 4;      // warps per CTA

// Staged values are read from shared memory with plain loads (the streaming
// global loads of Val4 are not valid on a shared-memory address).
__device__ __forceinline__ float staged(const float* p, uint32_t i) { return p[i]; }
__device__ __forceinline__ float staged(const __half* p, uint32_t i) { return __half2float(p[i]); }
__device__ __forceinline__ float staged(const __nv_bfloat16* p, uint32_t i) { return __bfloat162float(p[i]); }

struct ChunkMeta {
    uint32_t row;    // row index (0xffffffff: no chunk, the warp is done)
    uint32_t first;  // offset of the chunk's first element in the stage buffer
    uint32_t count;  // elements of the row in this chunk
    uint32_t last;   // 1 if the chunk ends its row
    float ratio;     // scatter: the row's ratio
};

template <typename V>
struct TmaSmem {
    uint32_t idx[kTmaStages][kTmaCh];
    V val[kTmaStages][kTmaCh];
    uint64_t bar[kTmaStages];
    ChunkMeta meta[kTmaStages];
};

template <typename V, int EPI>
__global__ void __launch_bounds__(kTmaWarps * 32)
k_csr_tma(const uint64_t* __restrict__ rowptr, const uint32_t* __restrict__ idx, const V* __restrict__ val,
          const float* __restrict__ x, uint32_t nrows, const int32_t* __restrict__ g, float* __restrict__ out,
          float* __restrict__ fwproj, float* __restrict__ f, const float* __restrict__ norm,
          uint32_t* __restrict__ err) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    TmaSmem<V>& S = reinterpret_cast<TmaSmem<V>*>(smem_raw)[w];
    const uint32_t gw = blockIdx.x * kTmaWarps + w;
    const uint32_t nw = gridDim.x * kTmaWarps;
    const uint64_t pol = evict_first_policy();

    if (lane == 0)
        for (int s = 0; s < kTmaStages; ++s) mbar_init(&S.bar[s], 1);
    fence_mbar_init();
    __syncwarp();

    // row pointers of this warp's rows, 32 at a time: batch kb holds rows
    // gw + (32*kb + lane) * nw
    auto load_batch = [&](uint32_t kb, uint64_t& s, uint64_t& t) {
        const uint64_t r = (uint64_t)gw + ((uint64_t)kb * 32 + lane) * nw;
        if (r < nrows) {
            s = rowptr[r];
            t = rowptr[r + 1];
        } else {
            s = t = 0;
        }
    };
    uint64_t cs, ct, ns, nt;
    uint32_t kb = 0;
    load_batch(0, cs, ct);
    load_batch(1, ns, nt);

    // producer state (identical in every lane)
    uint32_t pk = 0;          // row sequence number of the producer
    uint64_t pp = ~0ull;      // position inside that row (~0 = row start)
    auto issue = [&](int slot) {
        const uint64_t r = (uint64_t)gw + (uint64_t)pk * nw;
        if (r >= nrows) {
            if (lane == 0) S.meta[slot].row = 0xffffffffu;
            return;
        }
        if (pk / 32 != kb) {  // move to the next batch of row pointers
            cs = ns;
            ct = nt;
            ++kb;
            load_batch(kb + 1, ns, nt);
        }
        const uint64_t s = __shfl_sync(0xffffffffu, cs, pk % 32);
        const uint64_t t = __shfl_sync(0xffffffffu, ct, pk % 32);
        const uint64_t p = (pp == ~0ull) ? s : pp;
        const uint64_t a0 = p & ~7ull;
        const uint64_t e_end = t < a0 + kTmaCh ? t : a0 + kTmaCh;
        const uint64_t a1 = (e_end + 7) & ~7ull;
        const uint32_t ncopy = (uint32_t)(a1 - a0);
        if (lane == 0) {
            S.meta[slot].row = (uint32_t)r;
            S.meta[slot].first = (uint32_t)(p - a0);
            S.meta[slot].count = (uint32_t)(e_end - p);
            S.meta[slot].last = e_end == t ? 1u : 0u;
            if (ncopy) {
                mbar_arrive_tx(&S.bar[slot], ncopy * (uint32_t)(sizeof(uint32_t) + sizeof(V)));
                bulk_g2s(S.idx[slot], idx + a0, ncopy * (uint32_t)sizeof(uint32_t), &S.bar[slot], pol);
                bulk_g2s(S.val[slot], val + a0, ncopy * (uint32_t)sizeof(V), &S.bar[slot], pol);
            } else {
                mbar_arrive(&S.bar[slot]);
            }
        }
        if (e_end == t) {
            ++pk;
            pp = ~0ull;
        } else {
            pp = e_end;
        }
    };

    for (int s = 0; s < kTmaStages; ++s) issue(s);
    __syncwarp();

    uint32_t phase = 0;  // bit s = parity to wait for on stage s
    float acc = 0.f;
    int slot = 0;
    bool failed = false;
    while (true) {
        const ChunkMeta m = S.meta[slot];
        if (m.row == 0xffffffffu) break;
        if (!mbar_wait_timed(&S.bar[slot], (phase >> slot) & 1u)) {
            failed = true;
            break;
        }
        phase ^= 1u << slot;
        const uint32_t* ci = S.idx[slot] + m.first;
        const V* cv = S.val[slot] + m.first;
        // up to 16 elements per lane: 8 gathers in flight, then their FMAs
        uint32_t i = lane;
#pragma unroll 1
        for (; i + 224 < m.count; i += 256) {
            uint32_t c[8];
            float v[8], gx[8];
#pragma unroll
            for (int q = 0; q < 8; ++q) {
                c[q] = ci[i + 32 * q];
                v[q] = staged(cv, i + 32 * q);
            }
#pragma unroll
            for (int q = 0; q < 8; ++q) gx[q] = __ldg(x + c[q]);
#pragma unroll
            for (int q = 0; q < 8; ++q) acc = fmaf(v[q], gx[q], acc);
        }
        for (; i < m.count; i += 32) acc = fmaf(staged(cv, i), __ldg(x + ci[i]), acc);
        if (m.last) {
            float tot = acc;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) tot += __shfl_xor_sync(0xffffffffu, tot, o);
            if (lane == 0) {
                const uint32_t r = m.row;
                if (EPI == (int)Epi::Correl) {
                    out[r] = (tot != 0.0f) ? __fdiv_rn((float)g[r], tot) : 0.0f;
                    if (fwproj) fwproj[r] = tot;
                } else if (EPI == (int)Epi::Update) {
                    const float tt = __fmul_rn(f[r], tot);
                    const float nn = norm[r];
                    f[r] = (nn == 0.0f) ? tt : __fdiv_rn(tt, nn);
                } else {
                    out[r] = tot;
                }
            }
            acc = 0.f;
        }
        __syncwarp();  // every lane is done reading this stage
        issue(slot);   // refill it with the chunk kTmaStages ahead
        __syncwarp();
        slot = (slot + 1) % kTmaStages;
    }
    if (failed) {
        if (lane == 0) atomicOr(err, 1u);
        // drain this warp's copies still in flight before leaving
        for (int k = 0; k < kTmaStages; ++k) {
            const int sl = (slot + k) % kTmaStages;
            if (S.meta[sl].row != 0xffffffffu) mbar_wait_timed(&S.bar[sl], (phase >> sl) & 1u);
        }
    }
}

// Scatter back projection (calcBwProj_none_trans, kernel.cu:165-177) through
// the same per-warp rings.  The producer lane walks the warp's rows (gw,
// gw + nw, ...) with their bounds and ratios fetched 32 rows ahead, skips
// rows whose ratio is 0 (their products add nothing) and empty rows with one
// ballot per 32 rows, and streams pieces of at most kTmaCh elements of the
// others.  The 32 lanes scatter val * ratio of each staged piece with the
// grouped vector reductions, one aligned 4-entry vector per lane at a time.
// A row's pieces are independent (an entry needs only its row's ratio), so
// nothing waits for a row to complete, and the warps never wait on a gather:
// their only waits are for the copies, which the ring keeps ahead.
template <typename V>
__global__ void __launch_bounds__(kTmaWarps * 32)
k_scatter_tma(const uint64_t* __restrict__ rowptr, const uint32_t* __restrict__ idx, const V* __restrict__ val,
              const float* __restrict__ ratio, uint32_t nrows, float* __restrict__ bp, uint32_t ncols,
              uint32_t* __restrict__ err) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    TmaSmem<V>& S = reinterpret_cast<TmaSmem<V>*>(smem_raw)[w];
    const uint64_t gw = (uint64_t)blockIdx.x * kTmaWarps + w;
    const uint64_t nw = (uint64_t)gridDim.x * kTmaWarps;
    const uint64_t pol = evict_first_policy();

    if (lane == 0)
        for (int s = 0; s < kTmaStages; ++s) mbar_init(&S.bar[s], 1);
    fence_mbar_init();
    __syncwarp();

    // batch kb of the warp's rows: lane j holds row gw + (32*kb + j) * nw
    auto load_batch = [&](uint64_t kb, uint64_t& s, uint64_t& t, float& r) {
        const uint64_t row = gw + (kb * 32 + lane) * nw;
        if (row < nrows) {
            s = rowptr[row];
            t = rowptr[row + 1];
            r = ratio[row];
        } else {
            s = t = 0;
            r = 0.f;
        }
    };
    uint64_t cs, ct, ns, nt;
    float cr, nr;
    uint64_t kb = 0;
    load_batch(0, cs, ct, cr);
    load_batch(1, ns, nt, nr);
    unsigned live = __ballot_sync(0xffffffffu, cr != 0.0f && cs < ct);

    // producer state (identical in every lane)
    uint64_t pk = 0;       // position in the warp's row sequence
    uint64_t pp = ~0ull;   // position inside the current row (~0: find the next live row)
    uint64_t rs = 0, rt = 0;
    float rr = 0.f;
    bool done = false;
    auto issue = [&](int slot) {
        if (!done && pp == ~0ull) {
            for (;;) {
                if ((pk >> 5) != kb) {  // pk entered the next batch of 32 rows
                    ++kb;
                    if (gw + kb * 32 * nw >= nrows) {  // its first row is past the end
                        done = true;
                        break;
                    }
                    cs = ns;
                    ct = nt;
                    cr = nr;
                    load_batch(kb + 1, ns, nt, nr);
                    live = __ballot_sync(0xffffffffu, cr != 0.0f && cs < ct);
                }
                const unsigned m = live & (0xffffffffu << (unsigned)(pk & 31));
                if (m) {
                    pk = (pk & ~31ull) + (uint64_t)(__ffs(m) - 1);
                    break;
                }
                pk = (pk & ~31ull) + 32;  // no live row left in this batch
            }
            if (!done) {
                rs = __shfl_sync(0xffffffffu, cs, (int)(pk & 31));
                rt = __shfl_sync(0xffffffffu, ct, (int)(pk & 31));
                rr = __shfl_sync(0xffffffffu, cr, (int)(pk & 31));
                pp = rs;
            }
        }
        if (done) {
            if (lane == 0) S.meta[slot].row = 0xffffffffu;
            return;
        }
        const uint64_t a0 = pp & ~7ull;
        const uint64_t e_end = rt < a0 + kTmaCh ? rt : a0 + kTmaCh;
        const uint32_t ncopy = (uint32_t)(((e_end + 7) & ~7ull) - a0);
        if (lane == 0) {
            S.meta[slot].row = (uint32_t)(gw + pk * nw);
            S.meta[slot].first = (uint32_t)(pp - a0);
            S.meta[slot].count = (uint32_t)(e_end - pp);
            S.meta[slot].ratio = rr;
            mbar_arrive_tx(&S.bar[slot], ncopy * (uint32_t)(sizeof(uint32_t) + sizeof(V)));
            bulk_g2s(S.idx[slot], idx + a0, ncopy * (uint32_t)sizeof(uint32_t), &S.bar[slot], pol);
            bulk_g2s(S.val[slot], val + a0, ncopy * (uint32_t)sizeof(V), &S.bar[slot], pol);
        }
        if (e_end == rt) {
            ++pk;
            pp = ~0ull;
        } else {
            pp = e_end;
        }
    };

    for (int s = 0; s < kTmaStages; ++s) issue(s);
    __syncwarp();

    uint32_t phase = 0;  // bit s = parity to wait for on stage s
    int slot = 0;
    bool failed = false;
    while (true) {
        const ChunkMeta m = S.meta[slot];
        if (m.row == 0xffffffffu) break;
        if (!mbar_wait_timed(&S.bar[slot], (phase >> slot) & 1u)) {
            failed = true;
            break;
        }
        phase ^= 1u << slot;
        const uint4* ci = reinterpret_cast<const uint4*>(S.idx[slot]);
        const uint32_t e0 = m.first, e1 = m.first + m.count;
        for (uint32_t v = (e0 >> 2) + lane; v < (e1 + 3) >> 2; v += 32) {
            const uint32_t b = v * 4;
            unsigned use = 0;
#pragma unroll
            for (int k = 0; k < 4; ++k)
                if (b + k >= e0 && b + k < e1) use |= 1u << k;
            float a[4], pr[4];
            lds_val4(S.val[slot], v, a);
#pragma unroll
            for (int k = 0; k < 4; ++k) pr[k] = __fmul_rn(a[k], m.ratio);
            scatter4_mask(bp, ncols, ci[v], pr, use);
        }
        __syncwarp();  // every lane is done reading this stage
        issue(slot);   // refill it with the piece kTmaStages ahead
        __syncwarp();
        slot = (slot + 1) % kTmaStages;
    }
    if (failed) {
        if (lane == 0) atomicOr(err, 1u);
        // drain this warp's copies still in flight before leaving
        for (int k = 0; k < kTmaStages; ++k) {
            const int sl = (slot + k) % kTmaStages;
            if (S.meta[sl].row != 0xffffffffu) mbar_wait_timed(&S.bar[sl], (phase >> sl) & 1u);
        }
    }
}

template <typename V>
unsigned scatter_tma_grid() {
    static std::mutex mu;
    static std::map<int, unsigned> cache;
    int dev = 0;
    MLEM_CUDA(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lk(mu);
    auto it = cache.find(dev);
    if (it != cache.end()) return it->second;
    const size_t smem = sizeof(TmaSmem<V>) * kTmaWarps;
    MLEM_CUDA(cudaFuncSetAttribute(k_scatter_tma<V>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int per_sm = 0, sms = 0;
    MLEM_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_scatter_tma<V>, kTmaWarps * 32, smem));
    MLEM_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const unsigned grid = (unsigned)std::max(1, per_sm) * (unsigned)sms;
    cache[dev] = grid;
    return grid;
}

template <typename V>
void scatter_tma_launch(const DevCsr& A, const float* ratio, float* bp, uint32_t* err, L2Window win,
                        cudaStream_t s) {
    const unsigned grid = scatter_tma_grid<V>();
    const unsigned need = ceil_div_u(A.nrows, kTmaWarps);  // no more warps than rows
    launch_ex(k_scatter_tma<V>, dim3(std::min(grid, std::max(1u, need))), dim3(kTmaWarps * 32),
              sizeof(TmaSmem<V>) * kTmaWarps, s, win, (const uint64_t*)A.rowptr, (const uint32_t*)A.idx,
              static_cast<const V*>(A.val), ratio, A.nrows, bp, A.ncols, err);
}

template <typename V, int EPI>
unsigned tma_grid() {
    static std::mutex mu;
    static std::map<int, unsigned> cache;
    int dev = 0;
    cudaGetDevice(&dev);
    std::lock_guard<std::mutex> lk(mu);
    auto it = cache.find(dev);
    if (it != cache.end()) return it->second;
    const size_t smem = sizeof(TmaSmem<V>) * kTmaWarps;
    MLEM_CUDA(cudaFuncSetAttribute(k_csr_tma<V, EPI>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int per_sm = 0, sms = 0;
    MLEM_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_csr_tma<V, EPI>, kTmaWarps * 32, smem));
    MLEM_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const unsigned grid = (unsigned)std::max(1, per_sm) * (unsigned)sms;
    cache[dev] = grid;
    return grid;
}

template <typename V, int EPI>
void tma_launch(const DevCsr& op, const float* x, const EpiArgs& e, uint32_t* err, L2Window win, cudaStream_t s) {
    const unsigned grid = tma_grid<V, EPI>();
    const size_t smem = sizeof(TmaSmem<V>) * kTmaWarps;
    const unsigned need = ceil_div_u(op.nrows, kTmaWarps);  // no more warps than rows
    launch_ex(k_csr_tma<V, EPI>, dim3(std::min(grid, std::max(1u, need))), dim3(kTmaWarps * 32), smem, s, win,
              op.rowptr, op.idx, static_cast<const V*>(op.val), x, op.nrows, e.g, e.out, e.fwproj, e.f, e.norm, err);
}

template <typename V>
void tma_dispatch(const DevCsr& op, const float* x, const EpiArgs& e, uint32_t* err, L2Window win, cudaStream_t s) {
    switch (e.kind) {
        case Epi::Correl: tma_launch<V, (int)Epi::Correl>(op, x, e, err, win, s); break;
        case Epi::Update: tma_launch<V, (int)Epi::Update>(op, x, e, err, win, s); break;
        default: tma_launch<V, (int)Epi::Raw>(op, x, e, err, win, s);
    }
}

}  // namespace

void prepare_csr_tma(mlem_value_type vt) {
    // kernel attributes and occupancy are settled outside any stream capture
    switch (vt) {
        case MLEM_VAL_F32:
            tma_grid<float, 0>(); tma_grid<float, 1>(); tma_grid<float, 2>(); scatter_tma_grid<float>();
            break;
        case MLEM_VAL_F16:
            tma_grid<__half, 0>(); tma_grid<__half, 1>(); tma_grid<__half, 2>(); scatter_tma_grid<__half>();
            break;
        default:
            tma_grid<__nv_bfloat16, 0>(); tma_grid<__nv_bfloat16, 1>(); tma_grid<__nv_bfloat16, 2>();
            scatter_tma_grid<__nv_bfloat16>();
    }
}

void launch_scatter_tma(const DevCsr& A, const float* ratio, float* bp, uint32_t* err, L2Window win,
                        cudaStream_t s) {
    if (A.nrows == 0) return;
    MLEM_REQUIRE(err != nullptr, MLEM_EINVAL, "TMA scatter needs an error word");
    switch (A.vt) {
        case MLEM_VAL_F32: scatter_tma_launch<float>(A, ratio, bp, err, win, s); break;
        case MLEM_VAL_F16: scatter_tma_launch<__half>(A, ratio, bp, err, win, s); break;
        default: scatter_tma_launch<__nv_bfloat16>(A, ratio, bp, err, win, s);
    }
}

void launch_csr_tma(const DevCsr& op, const float* x, const EpiArgs& epi, uint32_t* err, L2Window win,
                    cudaStream_t s) {
    if (op.nrows == 0) return;
    switch (op.vt) {
        case MLEM_VAL_F32: tma_dispatch<float>(op, x, epi, err, win, s); break;
        case MLEM_VAL_F16: tma_dispatch<__half>(op, x, epi, err, win, s); break;
        default: tma_dispatch<__nv_bfloat16>(op, x, epi, err, win, s);
    }
}

}  // namespace mlem
