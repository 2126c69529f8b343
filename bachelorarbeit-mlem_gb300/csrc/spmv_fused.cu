// spmv_fused.cu — the fused single pass of the non-transposed iteration,
// staged through shared memory.
//
// One pass over A does the forward projection, the correlation and the
// scatter back projection (calcFwProj_csr_vector + calcCorrel +
// calcBwProj_none_trans, kernel.cu:118-130, 11-19, 165-177):
//     sum_r = A[r,:]·f,  ratio_r = g_r / sum_r (0 where sum_r = 0),
//     bp[c] += A[r,c] · ratio_r,
// so A crosses HBM once per iteration instead of twice.
//
// The rows are cut once per matrix into chunks of whole rows
// (fused_plan_build).  A persistent CTA takes chunks blockIdx.x,
// blockIdx.x + gridDim.x, ... through a ring of shared-memory stages:
// thread 0 streams a chunk's column indices, values and metadata with
// cp.async.bulk (completion on the stage's mbarrier), so two (FP32 values) or
// three (16-bit values) chunks are in flight while the CTA works on the
// current one.  The stage is cut into blocks of 128 entries (one 4-entry vector
// per lane); warp w owns blocks w, w + W, ... and the work runs in three
// phases separated by CTA barriers:
//   1. products  the warp gathers f[col] for its blocks (all in flight
//                together) and, for every piece (the part of one row inside
//                one block), sums the piece's products in a fixed order
//                (lane: entries in order; warp: xor tree);
//   2. ratios    one thread per row adds its pieces in block order, writes
//                the projection (log-likelihood) and ratio = g / sum;
//   3. scatter   the warp reloads its blocks and adds val · ratio of each
//                entry's row to bp; entries whose columns share a 16-byte
//                group of bp go out as one vector reduction.
// Every phase is balanced whatever the row lengths (blocks, not rows, are the
// unit of work), and the products of phase 1 never leave the registers.  A
// row longer than a stage is a chunk of its own, read from global memory by
// the whole CTA (dot, block reduction in a fixed order, scatter).
//
// Every mbarrier wait is bounded (kBarrierWaitNs of %globaltimer): on expiry
// the CTA sets *err, thread 0 waits (again bounded) for its copies still in
// flight, and the CTA returns; the host reports MLEM_ETIMEOUT.
//
// The other forms of the pass are k_fused_rescan and k_fused (spmv.cu); the
// run option `kernel` selects one, and AUTO times them all once per matrix
// (fused_form, runtime.cu).  On the scanners measured the rescan form wins:
// each CTA here works on one chunk at a time, so its gathers, its slowest
// warp and its reductions follow one another with 16-24 warps per SM to hide
// them.
#include "kernels.cuh"
#include "scatter.cuh"
#include "tma.cuh"

#include <algorithm>
#include <map>
#include <mutex>
#include <vector>

namespace mlem {

namespace {

constexpr int kNb = kFusedCap / kFusedBlk;                    // blocks per stage
constexpr int kMeta = (2 * (kFusedMaxRows + 1) + kNb + 3) & ~3;  // metadata words per stage
constexpr int kPieces = kNb + kFusedMaxRows;                    // pieces per chunk, at most

// Stages of the ring: 3 x 32 KB (FP32 values) or 4 x 24 KB (16-bit values),
// two CTAs per SM.
template <typename V>
constexpr int fused_stages() { return sizeof(V) == 4 ? 3 : 4; }

template <typename V, int T>
struct FusedSmem {
    static constexpr int S = fused_stages<V>();
    uint32_t idx[S][kFusedCap];
    V val[S][kFusedCap];
    uint32_t meta[S][kMeta];
    float psum[kPieces];        // piece sums
    float rr[kFusedMaxRows];    // ratio of each row of the chunk
    int32_t gs[kFusedMaxRows];  // counts of the chunk's rows
    FusedChunk desc[S];
    uint64_t bar[S];
    float wsum[T / 32];
    float bcast;
};

// A row longer than a stage, [s, t) of the global arrays, by the whole CTA.
template <typename V, int T>
__device__ __forceinline__ void wide_row(FusedSmem<V, T>& S, uint32_t row, uint64_t s, uint64_t t,
                                         const uint32_t* __restrict__ idx, const V* __restrict__ val,
                                         const float* __restrict__ x, const int32_t* __restrict__ g,
                                         float* __restrict__ bp, float* __restrict__ fwproj, uint32_t ncols) {
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const uint4* idx4 = reinterpret_cast<const uint4*>(idx);
    const uint64_t v1 = (t + 3) >> 2;
    float acc = 0.f;
    for (uint64_t v = (s >> 2) + tid; v < v1; v += T) {
        const uint4 c = ld_cached(idx4 + v);
        float a[4];
        Val4<V>::load_cached(val, v, a);
        const uint32_t cs[4] = {c.x, c.y, c.z, c.w};
        const uint64_t b = v << 2;
#pragma unroll
        for (int k = 0; k < 4; ++k)
            if (b + k >= s && b + k < t) acc = __fadd_rn(acc, __fmul_rn(a[k], __ldg(x + cs[k])));
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane == 0) S.wsum[warp] = acc;
    __syncthreads();
    if (tid == 0) {
        float tot = 0.f;
#pragma unroll
        for (int w = 0; w < T / 32; ++w) tot += S.wsum[w];
        if (fwproj) fwproj[row] = tot;
        S.bcast = (tot != 0.0f) ? __fdiv_rn((float)g[row], tot) : 0.0f;
    }
    __syncthreads();
    const float r = S.bcast;
    if (r == 0.0f) return;
    for (uint64_t v = (s >> 2) + tid; v < v1; v += T) {
        const uint4 c = ld_cached(idx4 + v);
        float a[4], pr[4];
        Val4<V>::load_cached(val, v, a);
        const uint64_t b = v << 2;
        unsigned use = 0;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            pr[k] = __fmul_rn(a[k], r);
            if (b + k >= s && b + k < t) use |= 1u << k;
        }
        scatter4_mask(bp, ncols, c, pr, use);
    }
}

template <typename V, int T>
__global__ void __launch_bounds__(T, 2)
k_fused_staged(const FusedChunk* __restrict__ chunks, uint64_t nchunks, const uint32_t* __restrict__ meta,
               const uint32_t* __restrict__ idx, const V* __restrict__ val, const float* __restrict__ x,
               const int32_t* __restrict__ g, float* __restrict__ bp, float* __restrict__ fwproj,
               uint32_t ncols, uint32_t* __restrict__ err) {
    constexpr int W = T / 32;
    constexpr int BPW = kNb / W;  // blocks per warp
    constexpr int S = FusedSmem<V, T>::S;
    static_assert(T >= kFusedMaxRows && kNb % W == 0, "one thread per row; whole blocks per warp");
    extern __shared__ __align__(128) unsigned char smem_raw[];
    auto& Sm = *reinterpret_cast<FusedSmem<V, T>*>(smem_raw);
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const uint64_t G = gridDim.x;

    uint64_t pol = 0;
    FusedChunk nd{};  // thread 0: the next chunk to stage
    auto stage = [&](int st, const FusedChunk& d) {
        Sm.desc[st] = d;
        const uint32_t nm = (d.mlen + 3u) & ~3u;  // metadata words, rounded up to 16 bytes
        const uint32_t ne = d.wide ? 0u : d.n8 * 8u;
        mbar_arrive_tx(&Sm.bar[st], nm * 4u + ne * (uint32_t)(sizeof(uint32_t) + sizeof(V)));
        bulk_g2s(Sm.meta[st], meta + d.meta_off, nm * 4u, &Sm.bar[st]);
        if (ne) {
            bulk_g2s(Sm.idx[st], idx + d.a0, ne * (uint32_t)sizeof(uint32_t), &Sm.bar[st], pol);
            bulk_g2s(Sm.val[st], val + d.a0, ne * (uint32_t)sizeof(V), &Sm.bar[st], pol);
        }
    };
    if (tid == 0) {
        pol = evict_first_policy();
        for (int i = 0; i < S; ++i) mbar_init(&Sm.bar[i], 1);
        fence_mbar_init();
        for (int i = 0; i < S; ++i)
            if (blockIdx.x + i * G < nchunks) stage(i, chunks[blockIdx.x + i * G]);
        if (blockIdx.x + S * G < nchunks) nd = chunks[blockIdx.x + S * G];
    }
    __syncthreads();

    uint64_t k = 0;
    for (uint64_t c = blockIdx.x; c < nchunks; c += G, ++k) {
        const int st = (int)(k % S);
        const uint32_t par = (uint32_t)((k / S) & 1);
        const bool ok = mbar_wait_timed(&Sm.bar[st], par);
        if (__syncthreads_or(!ok)) {
            if (tid == 0) {
                atomicOr(err, 1u);
                // the copies of this chunk and of the chunks staged after it may still land
                for (int i = 0; i < S; ++i)
                    if (c + i * G < nchunks)
                        mbar_wait_timed(&Sm.bar[(k + i) % S], (uint32_t)(((k + i) / S) & 1));
            }
            return;
        }
        const FusedChunk d = Sm.desc[st];
        const uint32_t* rs = Sm.meta[st];
        if (d.wide) {
            wide_row<V, T>(Sm, d.r0, d.a0 + rs[0], d.a0 + rs[1], idx, val, x, g, bp, fwproj, ncols);
        } else {
            const uint32_t nr = d.nr;
            const uint32_t* pf = rs + nr + 1;
            const uint32_t* bf = pf + nr + 1;
            const uint32_t lo = rs[0], hi = rs[nr];
            const uint32_t nb = (hi + kFusedBlk - 1) / kFusedBlk;
            const uint4* ci = reinterpret_cast<const uint4*>(Sm.idx[st]);
            const V* cv = Sm.val[st];
            // the counts of the chunk's rows travel with the gathers
            const int32_t gv = tid < (int)nr ? __ldg(g + d.r0 + tid) : 0;
            // phase 1: gathers and products of the warp's blocks, piece sums
            {
                uint4 cq[BPW];
                float pr[BPW][4];
#pragma unroll
                for (int i = 0; i < BPW; ++i) {
                    const uint32_t b = warp + W * i, v = b * 32 + lane;
                    if (b < nb) {
                        cq[i] = ci[v];
                        lds_val4(cv, v, pr[i]);
                    }
                }
#pragma unroll
                for (int i = 0; i < BPW; ++i) {
                    const uint32_t b = warp + W * i, e = (b * 32 + lane) * 4;
                    if (b < nb) {
                        const float x0 = (e + 0 >= lo && e + 0 < hi) ? __ldg(x + cq[i].x) : 0.f;
                        const float x1 = (e + 1 >= lo && e + 1 < hi) ? __ldg(x + cq[i].y) : 0.f;
                        const float x2 = (e + 2 >= lo && e + 2 < hi) ? __ldg(x + cq[i].z) : 0.f;
                        const float x3 = (e + 3 >= lo && e + 3 < hi) ? __ldg(x + cq[i].w) : 0.f;
                        pr[i][0] = __fmul_rn(pr[i][0], x0);
                        pr[i][1] = __fmul_rn(pr[i][1], x1);
                        pr[i][2] = __fmul_rn(pr[i][2], x2);
                        pr[i][3] = __fmul_rn(pr[i][3], x3);
                    }
                }
#pragma unroll
                for (int i = 0; i < BPW; ++i) {
                    const uint32_t b = warp + W * i;
                    if (b >= nb) continue;
                    const uint32_t b0 = b * kFusedBlk, b1 = b0 + kFusedBlk, e = (b * 32 + lane) * 4;
                    for (uint32_t j = bf[b]; j < nr && rs[j] < b1; ++j) {
                        const uint32_t ps = max(rs[j], b0), pe = min(rs[j + 1], b1);
                        if (ps >= pe) continue;  // empty row
                        float part = 0.f;
#pragma unroll
                        for (int kk = 0; kk < 4; ++kk)
                            if (e + kk >= ps && e + kk < pe) part += pr[i][kk];
#pragma unroll
                        for (int o = 16; o > 0; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
                        if (lane == 0) Sm.psum[pf[j] + (b - rs[j] / kFusedBlk)] = part;
                    }
                }
            }
            if (tid < (int)nr) Sm.gs[tid] = gv;
            __syncthreads();
            // phase 2: row sums from the pieces in block order, ratios
            if (tid < (int)nr) {
                float tot = 0.f;
                for (uint32_t q = pf[tid]; q < pf[tid + 1]; ++q) tot += Sm.psum[q];
                if (fwproj) fwproj[d.r0 + tid] = tot;
                Sm.rr[tid] = (tot != 0.0f) ? __fdiv_rn((float)Sm.gs[tid], tot) : 0.0f;
            }
            __syncthreads();
            // phase 3: scatter val * ratio of each entry's row (ratio 0 adds nothing)
#pragma unroll
            for (int i = 0; i < BPW; ++i) {
                const uint32_t b = warp + W * i, v = b * 32 + lane;
                if (b >= nb) continue;
                const uint32_t b0 = b * kFusedBlk, b1 = b0 + kFusedBlk, e = v * 4;
                float a[4], pr[4] = {0.f, 0.f, 0.f, 0.f};
                unsigned use = 0;
                lds_val4(cv, v, a);
                for (uint32_t j = bf[b]; j < nr && rs[j] < b1; ++j) {
                    const uint32_t ps = max(rs[j], b0), pe = min(rs[j + 1], b1);
                    const float r = Sm.rr[j];
                    if (ps >= pe || r == 0.0f) continue;
#pragma unroll
                    for (int kk = 0; kk < 4; ++kk)
                        if (e + kk >= ps && e + kk < pe) {
                            pr[kk] = __fmul_rn(a[kk], r);
                            use |= 1u << kk;
                        }
                }
                if (use) scatter4_mask(bp, ncols, ci[v], pr, use);
            }
        }
        __syncthreads();  // stage st is free again
        if (tid == 0 && c + S * G < nchunks) {
            stage(st, nd);
            if (c + (S + 1) * G < nchunks) nd = chunks[c + (S + 1) * G];
        }
    }
}

template <typename V, int T>
unsigned fused_grid() {
    static std::mutex mu;
    static std::map<int, unsigned> cache;
    int dev = 0;
    MLEM_CUDA(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lk(mu);
    auto it = cache.find(dev);
    if (it != cache.end()) return it->second;
    const size_t smem = sizeof(FusedSmem<V, T>);
    MLEM_CUDA(cudaFuncSetAttribute(k_fused_staged<V, T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int per_sm = 0, sms = 0;
    MLEM_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_fused_staged<V, T>, T, smem));
    MLEM_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const unsigned grid = (unsigned)std::max(1, per_sm) * (unsigned)sms;
    cache[dev] = grid;
    return grid;
}

template <typename V, int T>
void staged_launch(const DevCsr& A, const FusedPlan& p, const float* x, const int32_t* g, float* bp, float* fwproj,
                   uint32_t* err, L2Window win, cudaStream_t s) {
    const unsigned grid = (unsigned)std::min<uint64_t>(fused_grid<V, T>(), p.nchunks);
    launch_ex(k_fused_staged<V, T>, dim3(grid), dim3(T), sizeof(FusedSmem<V, T>), s, win,
              (const FusedChunk*)p.chunks, p.nchunks, (const uint32_t*)p.meta, (const uint32_t*)A.idx,
              static_cast<const V*>(A.val), x, g, bp, fwproj, A.ncols, err);
}

template <typename V>
void staged_threads(int threads, const DevCsr& A, const FusedPlan& p, const float* x, const int32_t* g, float* bp,
                    float* fwproj, uint32_t* err, L2Window win, cudaStream_t s) {
    if (threads == 512) staged_launch<V, 512>(A, p, x, g, bp, fwproj, err, win, s);
    else staged_launch<V, 256>(A, p, x, g, bp, fwproj, err, win, s);
}

}  // namespace

void FusedPlan::release() {
    cudaFree(chunks);
    cudaFree(meta);
    chunks = nullptr;
    meta = nullptr;
    nchunks = 0;
    meta_len = 0;
    built = false;
    staged_threads = 0;
    staged_ms = 0.f;
}

void fused_plan_build(const DevCsr& A, FusedPlan& p, cudaStream_t s) {
    p.release();
    const uint32_t R = A.nrows;
    std::vector<uint64_t> rp((size_t)R + 1, 0);
    MLEM_CUDA(cudaMemcpyAsync(rp.data(), A.rowptr, sizeof(uint64_t) * rp.size(), cudaMemcpyDeviceToHost, s));
    MLEM_CUDA(cudaStreamSynchronize(s));
    auto up8 = [](uint64_t e) { return (e + 7) & ~7ull; };
    std::vector<FusedChunk> ch;
    std::vector<uint32_t> meta;
    ch.reserve(A.nnz / (kFusedCap / 2) + R / kFusedMaxRows + 1);
    meta.reserve(2 * (size_t)R + 40 * ch.capacity());
    uint32_t r = 0;
    while (r < R) {
        FusedChunk d{};
        d.a0 = rp[r] & ~7ull;
        d.r0 = r;
        d.meta_off = meta.size();
        if (up8(rp[r + 1]) - d.a0 > (uint64_t)kFusedCap) {
            MLEM_REQUIRE(rp[r + 1] - d.a0 <= 0xffffffffull, MLEM_EINVAL, "row longer than 2^32 entries");
            d.nr = 1;
            d.wide = 1;
            meta.push_back((uint32_t)(rp[r] - d.a0));
            meta.push_back((uint32_t)(rp[r + 1] - d.a0));
        } else {
            uint32_t n = 0;
            while (r + n < R && n < (uint32_t)kFusedMaxRows && up8(rp[r + n + 1]) - d.a0 <= (uint64_t)kFusedCap) ++n;
            d.nr = (uint16_t)n;
            d.n8 = (uint32_t)((up8(rp[r + n]) - d.a0) / 8);
            const size_t rs0 = meta.size();
            for (uint32_t q = 0; q <= n; ++q) meta.push_back((uint32_t)(rp[r + q] - d.a0));
            // pf: first piece of each row (a non-empty row has one piece per block it touches)
            uint32_t acc = 0;
            for (uint32_t q = 0; q < n; ++q) {
                const uint32_t a = meta[rs0 + q], b = meta[rs0 + q + 1];
                meta.push_back(acc);
                if (b > a) acc += (b - 1) / kFusedBlk - a / kFusedBlk + 1;
            }
            meta.push_back(acc);
            // bf: first row that ends after each block starts
            const uint32_t hi = meta[rs0 + n], nb = (hi + kFusedBlk - 1) / kFusedBlk;
            uint32_t j = 0;
            for (uint32_t b = 0; b < nb; ++b) {
                while (meta[rs0 + j + 1] <= b * (uint32_t)kFusedBlk) ++j;
                meta.push_back(j);
            }
        }
        d.mlen = (uint32_t)(meta.size() - d.meta_off);
        while (meta.size() % 4) meta.push_back(0);
        ch.push_back(d);
        r += d.nr;
    }
    p.nchunks = ch.size();
    p.meta_len = meta.size();
    if (p.nchunks) {
        MLEM_CUDA(cudaMalloc(&p.chunks, sizeof(FusedChunk) * ch.size()));
        MLEM_CUDA(cudaMalloc(&p.meta, sizeof(uint32_t) * meta.size()));
        MLEM_CUDA(cudaMemcpyAsync(p.chunks, ch.data(), sizeof(FusedChunk) * ch.size(), cudaMemcpyHostToDevice, s));
        MLEM_CUDA(cudaMemcpyAsync(p.meta, meta.data(), sizeof(uint32_t) * meta.size(), cudaMemcpyHostToDevice, s));
        MLEM_CUDA(cudaStreamSynchronize(s));
    }
    p.built = true;
}

void prepare_fused_staged(mlem_value_type vt) {
    switch (vt) {
        case MLEM_VAL_F32: fused_grid<float, 256>(); fused_grid<float, 512>(); break;
        case MLEM_VAL_F16: fused_grid<__half, 256>(); fused_grid<__half, 512>(); break;
        default: fused_grid<__nv_bfloat16, 256>(); fused_grid<__nv_bfloat16, 512>();
    }
}

void launch_fused_staged(const DevCsr& A, const FusedPlan& p, int threads, const float* x, const int32_t* g,
                         float* bp, float* fwproj, uint32_t* err, L2Window win, cudaStream_t s) {
    if (A.nrows == 0 || p.nchunks == 0) return;
    MLEM_REQUIRE(threads == 256 || threads == 512, MLEM_EINVAL, "staged fused pass needs 256 or 512 threads");
    MLEM_REQUIRE(err != nullptr, MLEM_EINVAL, "staged fused pass needs an error word");
    switch (A.vt) {
        case MLEM_VAL_F32: staged_threads<float>(threads, A, p, x, g, bp, fwproj, err, win, s); break;
        case MLEM_VAL_F16: staged_threads<__half>(threads, A, p, x, g, bp, fwproj, err, win, s); break;
        default: staged_threads<__nv_bfloat16>(threads, A, p, x, g, bp, fwproj, err, win, s);
    }
}

}  // namespace mlem
