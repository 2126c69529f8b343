// merge.cu — merge-path SpMV (Merrill & Garland) for the merge-based switch
// (argv[8] = 0) of the reference: calcFwProj_merge_based / calcBwProj_merge_based
// (kernel.cu:52-105), merge_based_start (kernel.cu:190-241) and
// merge_based_work (kernel.cu:257-286).
//
// The merged list (row ends ∪ nonzeros) is cut into tiles whose start
// coordinates come from the reference search.  Library matrices use
// row-parallel tiles (k_merge_rows): a tile spans at least the stretch one
// 1024-thread block of the reference covers (1024 * secsize items) and about
// 32 average rows; its rows are shared out to 16-lane groups that read their
// part of the row with 16-byte vector loads.  Caller-owned arrays (the
// allocation-free entry point) use the per-thread form (k_merge_tile): thread
// t consumes secsize items from diagonal t*secsize, the tile's products are
// staged in shared memory and the per-thread carries are combined with a
// segmented scan in a fixed order.  Both apply the fused epilogue
// (correlation or update) to rows that end inside the tile and leave the
// first row of every tile to a small fix-up kernel that adds the carries of
// earlier tiles in tile order.  The reference instead adds every row fragment
// with a global atomicAdd (order nondeterministic); results here are
// deterministic.
#include "kernels.cuh"

#include <algorithm>
#include <cstdint>
#include <map>
#include <mutex>
#include <string>
#include <utility>

namespace mlem {

namespace {

// Restatement of the reference search loop (kernel.cu:202-229).  The
// reference can read csr_Rows[rows+1] (one past the end) when i reaches rows;
// either outcome of that comparison ends the loop at i = rows, so the probe
// is answered without the read.
__host__ __device__ __forceinline__ void search_ref(const uint64_t* rowptr, int64_t rows,
                                                    int64_t start, int64_t& oi, int64_t& oj) {
    int64_t lefti = 0, righti = rows;
    int64_t nexti = righti / 2;
    int64_t nextj = start - nexti;
    int64_t i = 0, j = start;
    while (i != nexti) {
        i = nexti;
        j = nextj;
        const bool right = (i + 1 > rows) ? true : ((int64_t)rowptr[i + 1] > j - 1);
        if (right) righti = i;
        else lefti = i + 1;
        nexti = (lefti + righti) / 2;
        nextj = start - nexti;
    }
    oi = i;
    oj = j;
}

__global__ void k_search_ref(const uint64_t* __restrict__ rowptr, uint32_t rows, uint32_t secsize,
                             uint64_t nthreads, int64_t* __restrict__ oi, int64_t* __restrict__ oj) {
    for (uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; t < nthreads;
         t += (uint64_t)gridDim.x * blockDim.x) {
        int64_t i, j;
        search_ref(rowptr, rows, (int64_t)(t * secsize), i, j);
        oi[t] = i;
        oj[t] = j;
    }
}

// Tile start coordinates at diagonals k*T*S; the end of the path is (rows, nnz).
__global__ void k_tile_coords(const uint64_t* __restrict__ rowptr, uint32_t rows, uint64_t nnz,
                              uint64_t tile_items, uint64_t ntiles, uint32_t* __restrict__ ti,
                              uint64_t* __restrict__ tj) {
    for (uint64_t k = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; k <= ntiles;
         k += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t d = k * tile_items;
        if (d >= (uint64_t)rows + nnz) {
            ti[k] = rows;
            tj[k] = nnz;
        } else {
            int64_t i, j;
            search_ref(rowptr, rows, (int64_t)d, i, j);
            ti[k] = (uint32_t)i;
            tj[k] = (uint64_t)j;
        }
    }
}

struct EpiDev {
    int kind;
    const int32_t* g;
    float* out;
    float* fwproj;
    float* f;
    const float* norm;
    __device__ __forceinline__ void operator()(uint32_t r, float sum) const {
        if (kind == (int)Epi::Correl) {
            out[r] = (sum != 0.0f) ? __fdiv_rn((float)g[r], sum) : 0.0f;
            if (fwproj) fwproj[r] = sum;
        } else if (kind == (int)Epi::Update) {
            const float t = __fmul_rn(f[r], sum);
            const float n = norm[r];
            f[r] = (n == 0.0f) ? t : __fdiv_rn(t, n);
        } else {
            out[r] = sum;
        }
    }
};

template <typename V>
__device__ __forceinline__ float load_val(const V* p, uint64_t e) { return Val4<V>::one(p, e); }

// One CTA per tile.  Dynamic shared memory: s_end[T*S+4] (u32, row ends
// relative to the tile's first nonzero) and s_prod[T*S] (val * x[col] of the
// tile's nonzeros).  The staging is element by element: consecutive lanes
// take consecutive nonzeros, so the loads are coalesced and one gather
// instruction covers 32 consecutive columns of a row (few cache lines).  Each
// product is formed once, and the walk along the merge path keeps the current
// row end in a register, so it reads one shared word per nonzero.
template <typename V>
__global__ void __launch_bounds__(256)
k_merge_tile(const uint64_t* __restrict__ rowptr, const uint32_t* __restrict__ idx,
             const V* __restrict__ val, const float* __restrict__ x, uint32_t rows,
             uint32_t S, const uint32_t* __restrict__ ti, const uint64_t* __restrict__ tj,
             float* __restrict__ carry, uint32_t* __restrict__ carry_row, float* __restrict__ head,
             EpiDev epi) {
    extern __shared__ __align__(16) unsigned char smem[];
    const uint32_t T = blockDim.x;
    const uint32_t TS = T * S;
    uint32_t* s_end = reinterpret_cast<uint32_t*>(smem);
    float* s_prod = reinterpret_cast<float*>(smem + sizeof(uint32_t) * (TS + 4));
    __shared__ float s_wv[32], s_inv[32];
    __shared__ int s_wk[32], s_ink[32];

    const uint64_t k = blockIdx.x;
    const uint32_t I0 = ti[k], I1 = ti[k + 1];
    const uint64_t J0 = tj[k], J1 = tj[k + 1];
    const uint32_t nrow_l = I1 - I0;            // row ends inside the tile
    const uint32_t nj = (uint32_t)(J1 - J0);    // nonzeros inside the tile
    const uint32_t total = nrow_l + nj;         // items of this tile (< TS only in the last)

    // Stage row ends (relative, clamped to nj+1) and the tile's nonzeros.
    for (uint32_t u = threadIdx.x; u <= nrow_l; u += T) {
        const uint64_t r = (uint64_t)I0 + u + 1;
        uint64_t e = (r <= rows) ? rowptr[r] : J1 + 1;
        e = e > J1 + 1 ? J1 + 1 : e;
        s_end[u] = (uint32_t)(e - J0);
    }
    for (uint32_t u = threadIdx.x; u < nj; u += T) {
        const uint64_t e = J0 + u;
        s_prod[u] = __fmul_rn(load_val<V>(val, e), __ldg(x + ld_stream(idx + e)));
    }
    __syncthreads();

    // Thread start coordinate: the same diagonal t*S as the reference's
    // global thread (blockIdx*T + threadIdx)*S, located inside the tile.
    const uint32_t dl = threadIdx.x * S;
    float acc = 0.f, first = 0.f;
    bool has_first = false;
    uint32_t first_row = 0;
    uint32_t i = nrow_l, j = nj;  // idle threads sit at the tile end
    if (dl < total) {
        uint32_t lo = dl > nj ? dl - nj : 0;
        uint32_t hi = dl < nrow_l ? dl : nrow_l;
        while (lo < hi) {
            const uint32_t mid = (lo + hi) >> 1;
            if (s_end[mid] + mid >= dl) hi = mid;
            else lo = mid + 1;
        }
        i = lo;
        j = dl - lo;
        first_row = i;
        const uint32_t steps = min(S, total - dl);
        uint32_t end_i = s_end[i];
        for (uint32_t st = 0; st < steps; ++st) {
            if (end_i > j) {
                acc = __fadd_rn(acc, s_prod[j]);
                ++j;
            } else {
                if (!has_first) {
                    first = acc;
                    has_first = true;
                } else {
                    epi(I0 + i, acc);  // row started and ended in this thread
                }
                acc = 0.f;
                ++i;
                end_i = s_end[i];
            }
        }
    }

    // Inclusive segmented scan of the carries (key = local row at the end
    // coordinate; keys are nondecreasing over threads).
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = T >> 5;
    float v = acc;
    const int key = (int)i;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const float vv = __shfl_up_sync(0xffffffffu, v, o);
        const int kk = __shfl_up_sync(0xffffffffu, key, o);
        if (lane >= o && kk == key) v = vv + v;
    }
    if (lane == 31) {
        s_wv[w] = v;
        s_wk[w] = key;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        float inv = 0.f;
        int ink = -1;
        for (int q = 0; q < nw; ++q) {
            s_inv[q] = inv;
            s_ink[q] = ink;
            float lv = s_wv[q];
            const int lk = s_wk[q];
            if (lk == ink) lv = inv + lv;
            inv = lv;
            ink = lk;
        }
    }
    __syncthreads();
    if (key == s_ink[w]) v = s_inv[w] + v;
    // carry into this thread = inclusive value of the previous thread
    float cin = __shfl_up_sync(0xffffffffu, v, 1);
    if (lane == 0) cin = (w == 0) ? 0.f : s_inv[w];
    if (threadIdx.x == 0) cin = 0.f;

    if (has_first) {
        const float tot = cin + first;
        if (first_row == 0) head[k] = tot;   // tile's first row: earlier tiles may add to it
        else epi(I0 + first_row, tot);
    }
    if (threadIdx.x == T - 1) {
        carry[k] = v;
        carry_row[k] = I0 + (uint32_t)key;
    }
}

// Rows that end in tile k but started earlier: sum of carries of the earlier
// tiles that ended inside the row (in tile order), plus the tile's head.
__global__ void k_merge_fixup(const uint32_t* __restrict__ ti, const float* __restrict__ carry,
                              const uint32_t* __restrict__ carry_row,
                              const float* __restrict__ head, uint64_t ntiles, EpiDev epi) {
    for (uint64_t k = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; k < ntiles;
         k += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t I0 = ti[k], I1 = ti[k + 1];
        if (I1 == I0) continue;  // the tile's first row does not end here
        int64_t q = (int64_t)k - 1;
        while (q >= 0 && carry_row[q] == I0) --q;
        float tot = 0.f;
        bool any = false;
        for (uint64_t p = (uint64_t)(q + 1); p < k; ++p) {
            tot = any ? tot + carry[p] : carry[p];
            any = true;
        }
        tot = any ? tot + head[k] : head[k];
        epi(I0, tot);
    }
}

// Row-parallel tile: the tile is the same stretch of the merge path as above
// (row ends and nonzeros from the reference search), but its rows are shared
// out to the CTA's warps.  A warp sums its row's part of the tile with
// 16-byte vector loads (the operand's arrays are padded and 16-byte aligned)
// and a fixed xor reduction; rows that end inside the tile get their
// epilogue here, the tile's first row (which began in an earlier tile) goes
// to head[k] and the row still open at the tile's end to carry[k], for the
// same fix-up kernel.  Deterministic.
template <typename V, int LPR, int U>
__device__ __forceinline__ float group_part_dot(const uint32_t* __restrict__ idx, const V* __restrict__ val,
                                                const float* __restrict__ x, uint64_t s, uint64_t t, int sub) {
    const uint4* idx4 = reinterpret_cast<const uint4*>(idx);
    const uint64_t v1 = (t + 3) >> 2;
    float acc = 0.f;
    // U = 2: two vectors per lane in flight; the FMAs still run in the lane's
    // vector order, so the sums are those of one vector at a time
    uint64_t v = (s >> 2) + sub;
    if constexpr (U == 2)
    for (; v + LPR < v1; v += 2 * LPR) {
        const uint4 c0 = ld_stream(idx4 + v), c1 = ld_stream(idx4 + v + LPR);
        float a0[4], a1[4];
        Val4<V>::load(val, v, a0);
        Val4<V>::load(val, v + LPR, a1);
        const uint32_t cs0[4] = {c0.x, c0.y, c0.z, c0.w}, cs1[4] = {c1.x, c1.y, c1.z, c1.w};
        // element 4v+k lies in [s, t) unless it is a masked head or tail element
        const uint32_t lo = (uint32_t)(s > 4 * v ? s - 4 * v : 0);
        const uint32_t hi1 = (uint32_t)(t - 4 * (v + LPR));  // the second vector starts past the head
        float g0[4], g1[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) g0[k] = (k >= (int)lo) ? __ldg(x + cs0[k]) : 0.f;
#pragma unroll
        for (int k = 0; k < 4; ++k) g1[k] = (k < (int)hi1) ? __ldg(x + cs1[k]) : 0.f;
#pragma unroll
        for (int k = 0; k < 4; ++k)
            if (k >= (int)lo) acc = fmaf(a0[k], g0[k], acc);
#pragma unroll
        for (int k = 0; k < 4; ++k)
            if (k < (int)hi1) acc = fmaf(a1[k], g1[k], acc);
    }
    for (; v < v1; v += LPR) {
        const uint4 c = ld_stream(idx4 + v);
        float a[4];
        Val4<V>::load(val, v, a);
        const uint32_t cs[4] = {c.x, c.y, c.z, c.w};
        const uint32_t lo = (uint32_t)(s > 4 * v ? s - 4 * v : 0), hi = (uint32_t)(t - 4 * v);
        float g[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) g[k] = (k >= (int)lo && k < (int)hi) ? __ldg(x + cs[k]) : 0.f;
#pragma unroll
        for (int k = 0; k < 4; ++k)
            if (k >= (int)lo && k < (int)hi) acc = fmaf(a[k], g[k], acc);
    }
    return acc;
}

template <typename V, int LPR, int U>
__global__ void __launch_bounds__(256, U == 1 ? 8 : 6)
k_merge_rows(const uint64_t* __restrict__ rowptr, const uint32_t* __restrict__ idx, const V* __restrict__ val,
             const float* __restrict__ x, uint32_t rows, const uint32_t* __restrict__ ti,
             const uint64_t* __restrict__ tj, float* __restrict__ carry, uint32_t* __restrict__ carry_row,
             float* __restrict__ head, EpiDev epi) {
    const uint64_t k = blockIdx.x;
    const uint32_t I0 = ti[k], I1 = ti[k + 1];
    const uint64_t J0 = tj[k], J1 = tj[k + 1];
    const uint32_t nrow_l = I1 - I0;  // rows that end inside the tile
    constexpr uint32_t NG = 256 / LPR;  // lane groups of the CTA
    const uint32_t grp = threadIdx.x / LPR;
    const int sub = threadIdx.x & (LPR - 1);
    const unsigned mask = LPR == 32 ? 0xffffffffu : (((1u << LPR) - 1u) << ((threadIdx.x & 31) & ~(LPR - 1)));
    for (uint32_t i = grp; i <= nrow_l; i += NG) {
        const uint32_t r = I0 + i;
        float acc = 0.f;
        if (r < rows) {
            uint64_t s = rowptr[r], t = rowptr[r + 1];
            s = s < J0 ? J0 : s;
            t = t > J1 ? J1 : t;
            if (s < t) acc = group_part_dot<V, LPR, U>(idx, val, x, s, t, sub);
        }
#pragma unroll
        for (int o = LPR / 2; o > 0; o >>= 1) acc += __shfl_xor_sync(mask, acc, o);
        if (sub == 0) {
            if (i == nrow_l) {  // still open at the tile's end (or past the last row)
                carry[k] = acc;
                carry_row[k] = r;
            } else if (i == 0) {
                head[k] = acc;  // began in an earlier tile: the fix-up adds their carries
            } else {
                epi(r, acc);
            }
        }
    }
}

template <typename V>
void merge_launch_t(const DevCsr& op, const MergePlan& p, const float* x, const EpiDev& e,
                    L2Window win, cudaStream_t s) {
    if (p.rows_kernel && p.rows_u == 2)
        launch_ex(k_merge_rows<V, 16, 2>, dim3((unsigned)p.ntiles), dim3(256), 0, s, win, op.rowptr, op.idx,
                  static_cast<const V*>(op.val), x, op.nrows, p.tile_i, p.tile_j, p.carry, p.carry_row, p.head, e);
    else if (p.rows_kernel)
        launch_ex(k_merge_rows<V, 16, 1>, dim3((unsigned)p.ntiles), dim3(256), 0, s, win, op.rowptr, op.idx,
                  static_cast<const V*>(op.val), x, op.nrows, p.tile_i, p.tile_j, p.carry, p.carry_row, p.head, e);
    else
        launch_ex(k_merge_tile<V>, dim3((unsigned)p.ntiles), dim3(p.threads), p.smem, s, win,
                  op.rowptr, op.idx, static_cast<const V*>(op.val), x, op.nrows, p.secsize,
                  p.tile_i, p.tile_j, p.carry, p.carry_row, p.head, e);
    const unsigned fg = std::max(1u, std::min<unsigned>(ceil_div_u(p.ntiles, 256), 152u * 8u));
    launch_ex(k_merge_fixup, dim3(fg), dim3(256), 0, s, L2Window{}, p.tile_i, p.carry,
              p.carry_row, p.head, p.ntiles, e);
}

}  // namespace

void MergePlan::release() {
    cudaFree(tile_i);
    cudaFree(tile_j);
    cudaFree(carry);
    cudaFree(carry_row);
    cudaFree(head);
    tile_i = nullptr;
    tile_j = nullptr;
    carry = nullptr;
    carry_row = nullptr;
    head = nullptr;
    ntiles = 0;
}

void launch_merge_search_ref(const uint64_t* rowptr, uint32_t rows, uint64_t nnz,
                             uint32_t secsize, uint64_t nthreads, int64_t* i_out,
                             int64_t* j_out, cudaStream_t s) {
    (void)nnz;
    if (nthreads == 0) return;
    const unsigned grid = std::min<unsigned>(ceil_div_u(nthreads, 256), 152u * 32u);
    k_search_ref<<<grid, 256, 0, s>>>(rowptr, rows, secsize, nthreads, i_out, j_out);
    MLEM_LAUNCHED();
}

void merge_plan_build(const DevCsr& op, uint32_t secsize, MergePlan& plan, cudaStream_t s) {
    MLEM_REQUIRE(secsize >= 1 && secsize <= 512, MLEM_EINVAL,
                 "merge section size must be in 1..512");
    plan.release();
    plan.secsize = secsize;
    // Row-parallel tiles of the merge path, 256 threads: at least the stretch
    // one 1024-thread block of the reference covers (1024 * secsize items),
    // and enough items for about 32 average rows so that the CTA's 8 warps
    // share the tile's rows evenly; at most 65536 items.
    plan.rows_kernel = true;
    plan.threads = 256;
    const uint64_t items = (uint64_t)op.nrows + op.nnz;
    const uint64_t per_row = op.nrows ? (items + op.nrows - 1) / op.nrows : 1;
    const uint64_t TS = std::min<uint64_t>(std::max<uint64_t>(1024ull * secsize, 32 * per_row), 65536ull);
    plan.ntiles = (items + TS - 1) / TS;
    MLEM_REQUIRE(plan.ntiles < (1ull << 31), MLEM_EUNSUPPORTED, "merge path: too many tiles");
    plan.smem = 0;
    const uint64_t nt = std::max<uint64_t>(plan.ntiles, 1);
    MLEM_CUDA(cudaMalloc(&plan.tile_i, sizeof(uint32_t) * (nt + 1)));
    MLEM_CUDA(cudaMalloc(&plan.tile_j, sizeof(uint64_t) * (nt + 1)));
    MLEM_CUDA(cudaMalloc(&plan.carry, sizeof(float) * nt));
    MLEM_CUDA(cudaMalloc(&plan.carry_row, sizeof(uint32_t) * nt));
    MLEM_CUDA(cudaMalloc(&plan.head, sizeof(float) * nt));
    // Opt in to the tile's shared memory outside any stream capture.  The
    // attribute belongs to the kernel, which all plans of a value type share,
    // so it only ever grows.
    {
        static std::mutex mu;
        static std::map<int, size_t> cur;  // (device * 4 + value type) -> bytes
        std::lock_guard<std::mutex> lk(mu);
        int dev = 0;
        cudaGetDevice(&dev);
        const int t = dev * 4 + (int)op.vt;
        if (plan.smem > cur[t]) {
            cudaError_t e;
            if (op.vt == MLEM_VAL_F32)
                e = cudaFuncSetAttribute(k_merge_tile<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)plan.smem);
            else if (op.vt == MLEM_VAL_F16)
                e = cudaFuncSetAttribute(k_merge_tile<__half>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)plan.smem);
            else
                e = cudaFuncSetAttribute(k_merge_tile<__nv_bfloat16>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)plan.smem);
            MLEM_CUDA(e);
            cur[t] = plan.smem;
        }
    }
    const unsigned grid = std::max(1u, std::min<unsigned>(ceil_div_u(plan.ntiles + 1, 256), 152u * 16u));
    k_tile_coords<<<grid, 256, 0, s>>>(op.rowptr, op.nrows, op.nnz, TS, plan.ntiles, plan.tile_i,
                                       plan.tile_j);
    MLEM_LAUNCHED();
}

void launch_merge_spmv(const DevCsr& op, const MergePlan& plan, const float* x, const EpiArgs& epi,
                       L2Window win, cudaStream_t s) {
    if (plan.ntiles == 0) return;
    EpiDev e{(int)epi.kind, epi.g, epi.out, epi.fwproj, epi.f, epi.norm};
    switch (op.vt) {
        case MLEM_VAL_F32: merge_launch_t<float>(op, plan, x, e, win, s); break;
        case MLEM_VAL_F16: merge_launch_t<__half>(op, plan, x, e, win, s); break;
        default: merge_launch_t<__nv_bfloat16>(op, plan, x, e, win, s);
    }
}

}  // namespace mlem

// ---------------------------------------------------------------------------
// Forward projection that allocates nothing.
//
// Some callers cannot call cudaMalloc: code that runs while a CUDA graph is
// being captured into a long-lived pool they do not own, host applications
// whose device memory is handed out once at start-up by their own pool
// (real-time reconstruction services, plugins inside a framework that
// accounts for every byte), and callers that must not trigger the implicit
// synchronisation an allocation can cause.  For them the merge-path forward
// projection keeps its per-tile scratch (tile coordinates, carries, heads) in
// one file-scope device array of fixed size instead of allocating it.
//
// The array belongs to the library image: every GPU that loads the library
// holds kNoAllocScratchBytes of it until the process exits.  All calls share
// it, so calls whose kernels overlap on the GPU race on it; serialise them
// (one stream, or events).  Nothing in it has to start at zero: every word a
// call reads was written earlier in the same call.
namespace mlem {
namespace {

constexpr size_t kNoAllocScratchBytes = 4u << 20;  // 4 MiB per device
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

// Identity of the current context: a number that the driver never reuses
// within the process (cuCtxGetId).  cudaDeviceReset destroys the primary
// context, and the module holding the array is loaded again into the next one,
// possibly at another address; keying the lookup on this identity keeps a
// stale address from being used.  The two driver calls are fetched through the
// runtime, so the library does not link libcuda.  Returns 0 where they are not
// available (the address is then looked up on every call).
unsigned long long current_context_id() {
    using GetCurrent = int (*)(void**);
    using GetId = int (*)(void*, unsigned long long*);
    static GetCurrent get_current = nullptr;
    static GetId get_id = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_current = reinterpret_cast<GetCurrent>(p);
        p = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_id = reinterpret_cast<GetId>(p);
    });
    void* ctx = nullptr;
    unsigned long long id = 0;
    if (!get_current || !get_id || get_current(&ctx) != 0 || ctx == nullptr || get_id(ctx, &id) != 0) return 0;
    return id;
}

// Device address of the array for the current device, looked up with that
// device current on the first call in each context (in host code the symbol
// itself is only a host-side stand-in, not a device address).
unsigned char* noalloc_scratch_address() {
    static std::mutex mu;
    static std::map<std::pair<int, unsigned long long>, unsigned char*> addr;
    int dev = -1;
    MLEM_CUDA(cudaGetDevice(&dev));
    const unsigned long long ctx = current_context_id();
    std::lock_guard<std::mutex> lk(mu);
    const auto key = std::make_pair(dev, ctx);
    if (ctx != 0) {
        auto it = addr.find(key);
        if (it != addr.end()) return it->second;
    }
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    MLEM_REQUIRE(e == cudaSuccess && p != nullptr, MLEM_ECUDA,
                 std::string("cudaGetSymbolAddress(scratch): ") + cudaGetErrorString(e));
    if (ctx != 0) addr[key] = static_cast<unsigned char*>(p);
    return static_cast<unsigned char*>(p);
}

inline size_t align256(size_t b) { return (b + 255) & ~size_t(255); }

}  // namespace
}  // namespace mlem

extern "C" mlem_status mlem_forward_project_merge_noalloc(const uint64_t* rowptr_dev, const uint32_t* col_dev,
                                                          const float* val_dev, uint32_t rows, uint32_t cols,
                                                          uint64_t nnz, const float* x_dev, const int32_t* g_dev,
                                                          float* ratio_dev, uint32_t secsize, void* stream) {
    using namespace mlem;
    try {
        MLEM_REQUIRE(rowptr_dev && x_dev && g_dev && ratio_dev && (nnz == 0 || (col_dev && val_dev)), MLEM_EINVAL,
                     "NULL argument");
        MLEM_REQUIRE(rows >= 1 && cols >= 1, MLEM_EINVAL, "matrix must have rows and columns");
        MLEM_REQUIRE(nnz <= UINT64_MAX - rows, MLEM_EINVAL, "allocation-free merge path: rows + nnz overflows");
        MLEM_REQUIRE(secsize >= 1 && secsize <= 125, MLEM_EINVAL,
                     "allocation-free merge path: secsize must be in 1..125");
        // tile of T threads * secsize items, sized so the tile's shared memory
        // stays within the default 48 KB (no opt-in call needed)
        uint32_t T = 4000 / secsize;
        T = std::max(32u, std::min(256u, T & ~31u));
        const uint64_t TS = (uint64_t)T * secsize;
        const uint64_t items = (uint64_t)rows + nnz;
        const uint64_t ntiles = (items + TS - 1) / TS;
        const size_t need = align256(sizeof(uint32_t) * (ntiles + 1)) + align256(sizeof(uint64_t) * (ntiles + 1)) +
                            3 * align256(sizeof(float) * ntiles);
        MLEM_REQUIRE(need <= kNoAllocScratchBytes, MLEM_EINVAL,
                     "allocation-free merge path: rows + nnz = " + std::to_string(items) + " needs " +
                         std::to_string(need) + " bytes of scratch, the fixed maximum is " +
                         std::to_string(kNoAllocScratchBytes) + " (use mlem_forward_project)");
        unsigned char* base = noalloc_scratch_address();
        MergePlan p;  // views into the static array; never released
        p.secsize = secsize;
        p.threads = T;
        p.ntiles = ntiles;
        p.smem = sizeof(uint32_t) * (TS + 4) + sizeof(float) * TS;
        size_t off = 0;
        p.tile_i = reinterpret_cast<uint32_t*>(base + off);
        off += align256(sizeof(uint32_t) * (ntiles + 1));
        p.tile_j = reinterpret_cast<uint64_t*>(base + off);
        off += align256(sizeof(uint64_t) * (ntiles + 1));
        p.carry = reinterpret_cast<float*>(base + off);
        off += align256(sizeof(float) * ntiles);
        p.carry_row = reinterpret_cast<uint32_t*>(base + off);
        off += align256(sizeof(float) * ntiles);
        p.head = reinterpret_cast<float*>(base + off);
        cudaStream_t s = static_cast<cudaStream_t>(stream);
        const unsigned grid = std::max(1u, std::min<unsigned>(ceil_div_u(ntiles + 1, 256), 152u * 16u));
        k_tile_coords<<<grid, 256, 0, s>>>(rowptr_dev, rows, nnz, TS, ntiles, p.tile_i, p.tile_j);
        MLEM_LAUNCHED();
        DevCsr A;
        A.nrows = rows;
        A.ncols = cols;
        A.nnz = nnz;
        A.rowptr = const_cast<uint64_t*>(rowptr_dev);
        A.idx = const_cast<uint32_t*>(col_dev);
        A.val = const_cast<float*>(val_dev);
        A.vt = MLEM_VAL_F32;
        EpiArgs e;
        e.kind = Epi::Correl;
        e.g = g_dev;
        e.out = ratio_dev;
        launch_merge_spmv(A, p, x_dev, e, L2Window{}, s);
        return MLEM_OK;
    } catch (const Error& err) {
        set_error(err.msg);
        return err.code;
    } catch (const std::exception& err) {
        set_error(err.what());
        return MLEM_EINVAL;
    }
}
