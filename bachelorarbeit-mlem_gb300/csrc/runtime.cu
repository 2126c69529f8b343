// runtime.cu — matrix handles, the MLEM iteration loop and the C ABI entry
// points of the single-reconstruction path.
//
// The reference mlem() (main.cu:167-514) allocates, uploads, runs
//   FP -> correl -> [AllReduce] -> BP -> update -> AllReduce(bp->f) -> 2x memset
// per iteration with host synchronisation after each collective, and frees
// everything at the end.  Here the matrix (A, the device-built Aᵀ and the
// sensitivity image) is a resident handle; one iteration is two kernels (FP
// with fused correlation, BP with fused update) or three in the scatter
// forms, enqueued on one stream and replayed as a CUDA graph; there is no
// memset, no collective and no host synchronisation inside the loop.
#include <chrono>
#include <cmath>
#include <cstring>
#include <limits>
#include <string>
#include <thread>

#include "runtime.h"

namespace mlem {

std::atomic<uint64_t> g_launches{0};
size_t g_max_window_bytes = 0;

namespace {
thread_local std::string t_error;
}

void set_error(const std::string& msg) { t_error = msg; }
const char* get_error() { return t_error.c_str(); }

[[noreturn]] void fail(mlem_status code, const std::string& msg) { throw Error{code, msg}; }

void Workspace::release() {
    for (auto& kv : graphs) cudaGraphExecDestroy(kv.second);
    graphs.clear();
    cudaFree(g);
    cudaFree(f);
    cudaFree(ratio);
    cudaFree(bp);
    cudaFree(fwproj);
    cudaFree(ll_part);
    cudaFree(ll_vals);
    cudaFree(err);
    cudaFree(tmp_rows);
    cudaFree(tmp_cols);
    *this = Workspace();
}

void BatchState::alloc(uint32_t rows, uint32_t cols, uint32_t t, bool scatter) {
    tile = t;
    const uint64_t R = std::max<uint32_t>(rows, 1), C = std::max<uint32_t>(cols, 1);
    MLEM_CUDA(cudaMalloc(&g, sizeof(int32_t) * R * t));
    MLEM_CUDA(cudaMalloc(&f, sizeof(float) * C * t));
    MLEM_CUDA(cudaMalloc(&ratio, sizeof(float) * R * t));
    MLEM_CUDA(cudaMalloc(&remaining, sizeof(uint32_t) * 32));
    MLEM_CUDA(cudaMalloc(&stage_g, sizeof(int32_t) * R));
    MLEM_CUDA(cudaMalloc(&stage_f, sizeof(float) * C));
    MLEM_CUDA(cudaMemset(g, 0, sizeof(int32_t) * R * t));
    MLEM_CUDA(cudaMemset(f, 0, sizeof(float) * C * t));
    MLEM_CUDA(cudaMemset(remaining, 0, sizeof(uint32_t) * 32));
    MLEM_CUDA(cudaMalloc(&bar, 64));
    MLEM_CUDA(cudaMemset(bar, 0, 64));
    err = reinterpret_cast<int*>(reinterpret_cast<char*>(bar) + 32);
    bytes = (sizeof(int32_t) + sizeof(float)) * R * t + sizeof(float) * C * t + 4 * R + 4 * C + 192;
    if (scatter) {
        MLEM_CUDA(cudaMalloc(&bp, sizeof(float) * C * t));
        MLEM_CUDA(cudaMemset(bp, 0, sizeof(float) * C * t));
        bytes += sizeof(float) * C * t;
    }
}

void BatchState::release() {
    for (cudaGraphExec_t ge : graph)
        if (ge) cudaGraphExecDestroy(ge);
    cudaFree(g);
    cudaFree(f);
    cudaFree(ratio);
    cudaFree(bp);
    cudaFree(remaining);
    cudaFree(stage_g);
    cudaFree(stage_f);
    cudaFree(bar);
    *this = BatchState();
}

static void free_csr(DevCsr& c) {
    cudaFree(c.rowptr);
    cudaFree(c.idx);
    cudaFree(c.val);
    cudaFree(c.dvptr);
    cudaFree(c.dbase);
    cudaFree(c.d16);
    cudaFree(c.dval);
    cudaFree(c.idx_ilv);
    cudaFree(c.val_ilv);
    cudaFree(c.order);
    c = DevCsr();
}

static uint64_t csr_bytes(const DevCsr& c) {
    if (!c.rowptr) return 0;
    uint64_t b = sizeof(uint64_t) * ((uint64_t)c.nrows + 1) + sizeof(uint32_t) * padded(c.nnz) +
                 val_bytes(c.vt) * padded(c.nnz);
    if (c.d16) b += 12ull * c.nrows + 8 + (sizeof(uint16_t) + val_bytes(c.vt)) * 8 * c.dvec;
    if (c.idx_ilv) b += (sizeof(uint32_t) + val_bytes(c.vt)) * c.ilv_len;
    if (c.order) b += sizeof(uint32_t) * c.nrows;
    return b;
}

void ensure_workspace(mlem_matrix* m) {
    Workspace& w = m->ws;
    if (w.ready) return;
    const uint64_t R = std::max<uint32_t>(m->A.nrows, 1), C = std::max<uint32_t>(m->A.ncols, 1);
    MLEM_CUDA(cudaMalloc(&w.g, sizeof(int32_t) * R));
    MLEM_CUDA(cudaMalloc(&w.f, sizeof(float) * C));
    MLEM_CUDA(cudaMalloc(&w.ratio, sizeof(float) * R));
    MLEM_CUDA(cudaMalloc(&w.bp, sizeof(float) * C));
    MLEM_CUDA(cudaMalloc(&w.fwproj, sizeof(float) * R));
    MLEM_CUDA(cudaMalloc(&w.ll_part, sizeof(double) * kLoglikParts));
    MLEM_CUDA(cudaMalloc(&w.err, sizeof(uint32_t)));
    MLEM_CUDA(cudaMemsetAsync(w.err, 0, sizeof(uint32_t), m->stream));
    MLEM_CUDA(cudaMemsetAsync(w.bp, 0, sizeof(float) * C, m->stream));
    MLEM_CUDA(cudaMemsetAsync(w.ratio, 0, sizeof(float) * R, m->stream));
    if (m->lor_of || m->vox_of) {
        MLEM_CUDA(cudaMalloc(&w.tmp_rows, sizeof(float) * R));
        MLEM_CUDA(cudaMalloc(&w.tmp_cols, sizeof(float) * C));
    }
    MLEM_CUDA(cudaStreamSynchronize(m->stream));
    w.ready = true;
}

// Entry-point permutations (identity copies when the matrix keeps its
// natural layout).  *_in: natural -> internal, *_out: internal -> natural;
// dst and src never alias.
static void rows_in_i32(const mlem_matrix* m, int32_t* dst, const int32_t* src, cudaStream_t s) {
    const uint64_t n = m->A.nrows;
    if (m->lor_of) launch_gather_i32(dst, src, m->lor_of, n, s);
    else MLEM_CUDA(cudaMemcpyAsync(dst, src, sizeof(int32_t) * n, cudaMemcpyDeviceToDevice, s));
}
static void rows_in_f32(const mlem_matrix* m, float* dst, const float* src, cudaStream_t s) {
    const uint64_t n = m->A.nrows;
    if (m->lor_of) launch_gather_f32(dst, src, m->lor_of, n, s);
    else MLEM_CUDA(cudaMemcpyAsync(dst, src, sizeof(float) * n, cudaMemcpyDeviceToDevice, s));
}
static void rows_out(const mlem_matrix* m, float* dst, const float* src, cudaStream_t s) {
    const uint64_t n = m->A.nrows;
    if (m->lor_of) launch_scatter_f32(dst, src, m->lor_of, n, s);
    else MLEM_CUDA(cudaMemcpyAsync(dst, src, sizeof(float) * n, cudaMemcpyDeviceToDevice, s));
}
static void cols_in(const mlem_matrix* m, float* dst, const float* src, cudaStream_t s) {
    const uint64_t n = m->A.ncols;
    if (m->vox_of) launch_gather_f32(dst, src, m->vox_of, n, s);
    else MLEM_CUDA(cudaMemcpyAsync(dst, src, sizeof(float) * n, cudaMemcpyDeviceToDevice, s));
}
static void cols_out(const mlem_matrix* m, float* dst, const float* src, cudaStream_t s) {
    const uint64_t n = m->A.ncols;
    if (m->vox_of) launch_scatter_f32(dst, src, m->vox_of, n, s);
    else MLEM_CUDA(cudaMemcpyAsync(dst, src, sizeof(float) * n, cudaMemcpyDeviceToDevice, s));
}
static bool permuted(const mlem_matrix* m) { return m->lor_of || m->vox_of; }

// Lanes per row of A (8, 16 or 32) and 16-byte vectors per lane in flight (1
// or 2) for the scatter back projection, timed once per matrix (ratio 1 into a
// scratch image), and whether the TMA-ring scatter beats the best of them.
// Returns the lanes; m->scatter_unroll holds the vectors, m->scatter_tma the
// choice of the TMA ring inside the MLEM iteration.
int scatter_lanes(mlem_matrix* m) {
    if (m->scatter_lanes) return m->scatter_lanes;
    const DevCsr& A = m->A;
    cudaStream_t s = m->stream;
    float *r = nullptr, *bp = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    int best_l = pick_lanes(A.nnz, A.nrows) < 8 ? 8 : pick_lanes(A.nnz, A.nrows), best_u = 1;
    float best = 1e30f;
    try {
        MLEM_CUDA(cudaMalloc(&r, sizeof(float) * std::max<uint32_t>(A.nrows, 1)));
        MLEM_CUDA(cudaMalloc(&bp, sizeof(float) * std::max<uint32_t>(A.ncols, 1)));
        std::vector<float> ones(std::max<uint32_t>(A.nrows, 1), 1.0f);
        MLEM_CUDA(cudaMemcpyAsync(r, ones.data(), sizeof(float) * ones.size(), cudaMemcpyHostToDevice, s));
        MLEM_CUDA(cudaMemsetAsync(bp, 0, sizeof(float) * std::max<uint32_t>(A.ncols, 1), s));
        MLEM_CUDA(cudaEventCreate(&e0));
        MLEM_CUDA(cudaEventCreate(&e1));
        for (int lanes : {8, 16, 32})
            for (int u : {1, 2}) {
                launch_scatter(A, r, bp, lanes, u, {}, s);
                MLEM_CUDA(cudaEventRecord(e0, s));
                for (int q = 0; q < 2; ++q) launch_scatter(A, r, bp, lanes, u, {}, s);
                MLEM_CUDA(cudaEventRecord(e1, s));
                MLEM_CUDA(cudaEventSynchronize(e1));
                float ms = 0.f;
                MLEM_CUDA(cudaEventElapsedTime(&ms, e0, e1));
                if (ms < best) {
                    best = ms;
                    best_l = lanes;
                    best_u = u;
                }
            }
        ensure_workspace(m);
        prepare_csr_tma(A.vt);
        launch_scatter_tma(A, r, bp, m->ws.err, {}, s);
        MLEM_CUDA(cudaEventRecord(e0, s));
        for (int q = 0; q < 2; ++q) launch_scatter_tma(A, r, bp, m->ws.err, {}, s);
        MLEM_CUDA(cudaEventRecord(e1, s));
        MLEM_CUDA(cudaEventSynchronize(e1));
        float ms = 0.f;
        MLEM_CUDA(cudaEventElapsedTime(&ms, e0, e1));
        check_device_error(m, s);
        m->scatter_tma = ms < best;
    } catch (...) {
        cudaStreamSynchronize(s);
        cudaFree(r);
        cudaFree(bp);
        if (e0) cudaEventDestroy(e0);
        if (e1) cudaEventDestroy(e1);
        throw;
    }
    cudaFree(r);
    cudaFree(bp);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    m->scatter_unroll = best_u;
    m->scatter_lanes = best_l;
    return best_l;
}

void launch_fused(mlem_matrix* m, const FusedForm& f, const float* x, const int32_t* g, float* bp, float* fwproj,
                  L2Window win, cudaStream_t s) {
    if (f.kind == 1) launch_fused_staged(m->A, m->fused, f.threads, x, g, bp, fwproj, m->ws.err, win, s);
    else if (f.kind == 2) launch_fused_rescan(m->A, x, g, bp, fwproj, f.lanes, f.unroll, f.ordered, win, s);
    else launch_fused_fp_scatter(m->A, x, g, bp, fwproj, win, s);
}

// Milliseconds of one fused pass of A in a form on an image and counts of
// ones into a scratch image, after one warm-up launch.
static float time_fused(mlem_matrix* m, const FusedForm& f) {
    const DevCsr& A = m->A;
    cudaStream_t s = m->stream;
    float *x = nullptr, *bp = nullptr;
    int32_t* g = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    float ms = 0.f;
    try {
        const uint32_t R = std::max<uint32_t>(A.nrows, 1), C = std::max<uint32_t>(A.ncols, 1);
        MLEM_CUDA(cudaMalloc(&x, sizeof(float) * C));
        MLEM_CUDA(cudaMalloc(&bp, sizeof(float) * C));
        MLEM_CUDA(cudaMalloc(&g, sizeof(int32_t) * R));
        std::vector<float> ones(C, 1.0f);
        std::vector<int32_t> gones(R, 1);
        MLEM_CUDA(cudaMemcpyAsync(x, ones.data(), sizeof(float) * C, cudaMemcpyHostToDevice, s));
        MLEM_CUDA(cudaMemcpyAsync(g, gones.data(), sizeof(int32_t) * R, cudaMemcpyHostToDevice, s));
        MLEM_CUDA(cudaMemsetAsync(bp, 0, sizeof(float) * C, s));
        MLEM_CUDA(cudaEventCreate(&e0));
        MLEM_CUDA(cudaEventCreate(&e1));
        launch_fused(m, f, x, g, bp, nullptr, {}, s);
        MLEM_CUDA(cudaEventRecord(e0, s));
        for (int q = 0; q < 2; ++q) launch_fused(m, f, x, g, bp, nullptr, {}, s);
        MLEM_CUDA(cudaEventRecord(e1, s));
        MLEM_CUDA(cudaEventSynchronize(e1));
        MLEM_CUDA(cudaEventElapsedTime(&ms, e0, e1));
        check_device_error(m, s);
    } catch (...) {
        cudaStreamSynchronize(s);
        cudaFree(x);
        cudaFree(bp);
        cudaFree(g);
        if (e0) cudaEventDestroy(e0);
        if (e1) cudaEventDestroy(e1);
        throw;
    }
    cudaFree(x);
    cudaFree(bp);
    cudaFree(g);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return ms / 2;
}

// Form of the fused single pass for the run's kernel switch: TMA = staged
// through shared memory (CTA size timed once per matrix), PERSISTENT = the
// register form, AUTO = the fastest of every form and configuration (timed
// once per matrix), any other = the rescan form with the run's lanes, vectors
// in flight and row order.
FusedForm fused_form(mlem_matrix* m, const mlem_run_opts& o) {
    FusedPlan& p = m->fused;
    FusedForm f;
    auto staged = [&]() {
        if (!p.staged_threads) {
            ensure_workspace(m);
            if (!p.built) fused_plan_build(m->A, p, m->stream);
            prepare_fused_staged(m->A.vt);
            FusedForm a, b;
            a.kind = b.kind = 1;
            a.threads = 256;
            b.threads = 512;
            const float ta = time_fused(m, a), tb = time_fused(m, b);
            p.staged_threads = tb < ta ? 512 : 256;
            p.staged_ms = std::min(ta, tb);
        }
        FusedForm r;
        r.kind = 1;
        r.threads = p.staged_threads;
        r.ms = p.staged_ms;
        return r;
    };
    if (o.kernel == MLEM_KERNEL_TMA) return staged();
    if (o.kernel == MLEM_KERNEL_PERSISTENT) return f;  // register form
    if (o.kernel != MLEM_KERNEL_AUTO) {
        f.kind = 2;
        f.lanes = o.lanes ? (int)std::max(8u, o.lanes) : std::max(8, pick_lanes(m->A.nnz, m->A.nrows));
        f.unroll = o.unroll == 1 ? 1 : 2;
        f.ordered = (o.kernel == MLEM_KERNEL_ORDERED || o.row_order) && m->A.order != nullptr;
        return f;
    }
    if (m->fused_auto.ms > 0.f) return m->fused_auto;
    FusedForm best = staged();
    FusedForm reg;
    reg.ms = time_fused(m, reg);
    if (reg.ms < best.ms) best = reg;
    for (int lanes : {8, 16, 32})
        for (int u : {1, 2})
            for (int ord = 0; ord <= (m->A.order ? 1 : 0); ++ord) {
                FusedForm c;
                c.kind = 2;
                c.lanes = lanes;
                c.unroll = u;
                c.ordered = ord != 0;
                c.ms = time_fused(m, c);
                if (c.ms < best.ms) best = c;
            }
    m->fused_auto = best;
    return best;
}

const MergePlan& merge_plan(mlem_matrix* m, bool transposed, uint32_t secsize) {
    auto& plans = transposed ? m->plan_AT : m->plan_A;
    auto it = plans.find(secsize);
    if (it != plans.end()) return it->second;
    MergePlan p;
    const DevCsr& op = transposed ? m->AT : m->A;
    cudaStream_t s = m->stream;
    merge_plan_build(op, secsize, p, s);
    MLEM_CUDA(cudaStreamSynchronize(s));
    if (p.rows_kernel && op.nnz) {
        // one or two vectors per lane in flight in the row kernel (6 or 8 blocks
        // per SM), timed with a Raw epilogue on an image of ones; same sums
        float *x = nullptr, *y = nullptr;
        cudaEvent_t e0 = nullptr, e1 = nullptr;
        float best = 1e30f;
        int pick = 1;
        try {
            MLEM_CUDA(cudaMalloc(&x, sizeof(float) * std::max<uint32_t>(op.ncols, 1)));
            MLEM_CUDA(cudaMalloc(&y, sizeof(float) * std::max<uint32_t>(op.nrows, 1)));
            std::vector<float> ones(std::max<uint32_t>(op.ncols, 1), 1.0f);
            MLEM_CUDA(cudaMemcpyAsync(x, ones.data(), sizeof(float) * ones.size(), cudaMemcpyHostToDevice, s));
            MLEM_CUDA(cudaEventCreate(&e0));
            MLEM_CUDA(cudaEventCreate(&e1));
            EpiArgs e;
            e.kind = Epi::Raw;
            e.out = y;
            for (int u : {1, 2}) {
                p.rows_u = u;
                launch_merge_spmv(op, p, x, e, L2Window{}, s);
                MLEM_CUDA(cudaEventRecord(e0, s));
                for (int q = 0; q < 2; ++q) launch_merge_spmv(op, p, x, e, L2Window{}, s);
                MLEM_CUDA(cudaEventRecord(e1, s));
                MLEM_CUDA(cudaEventSynchronize(e1));
                float ms = 0.f;
                MLEM_CUDA(cudaEventElapsedTime(&ms, e0, e1));
                if (ms < best) {
                    best = ms;
                    pick = u;
                }
            }
        } catch (...) {
            cudaStreamSynchronize(s);
            cudaFree(x);
            cudaFree(y);
            if (e0) cudaEventDestroy(e0);
            if (e1) cudaEventDestroy(e1);
            p.release();
            throw;
        }
        cudaFree(x);
        cudaFree(y);
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        p.rows_u = pick;
    }
    return plans.emplace(secsize, p).first->second;
}


void check_run_opts(const mlem_matrix* m, const mlem_run_opts& o) {
    MLEM_REQUIRE(o.kernel <= MLEM_KERNEL_SYM, MLEM_EINVAL,
                 "kernel must be 0 direct, 1 tma, 2 persistent, 3 auto, 4 d16, 5 ilv, 6 ordered or 7 sym");
    MLEM_REQUIRE(o.kernel != MLEM_KERNEL_SYM || m->sym.fp_rowptr != nullptr, MLEM_EINVAL,
                 "kernel SYM needs a matrix generated with symmetry = 1");
    MLEM_REQUIRE(o.lanes == 0 || o.lanes == 4 || o.lanes == 8 || o.lanes == 16 || o.lanes == 32, MLEM_EINVAL,
                 "lanes must be 0, 4, 8, 16 or 32");
    MLEM_REQUIRE(o.unroll == 0 || o.unroll == 1 || o.unroll == 2 || o.unroll == 4 ||
                     (o.unroll == 8 && o.kernel == MLEM_KERNEL_SYM),
                 MLEM_EINVAL, "unroll must be 0, 1, 2 or 4 (or 8 with kernel SYM)");
    MLEM_REQUIRE(o.kernel != MLEM_KERNEL_PERSISTENT || (o.lanes != 4 && o.lanes != 8 && o.unroll != 4),
                 MLEM_EINVAL, "the persistent kernel takes 16 or 32 lanes and unroll 1 or 2");
    MLEM_REQUIRE(o.row_order <= 1, MLEM_EINVAL, "row_order must be 0 or 1");
    MLEM_REQUIRE(o.pipeline <= 1, MLEM_EINVAL, "pipeline must be 0 or 1");
    MLEM_REQUIRE(!o.pipeline || o.lanes == 0 || o.lanes >= 16, MLEM_EINVAL, "pipeline needs 16 or 32 lanes");
    const bool ordered = o.kernel == MLEM_KERNEL_ORDERED ||
                         (o.row_order && (o.kernel == MLEM_KERNEL_DIRECT || o.kernel == MLEM_KERNEL_PERSISTENT));
    MLEM_REQUIRE(!ordered || o.lanes == 0 || o.lanes >= 16, MLEM_EINVAL, "row order needs 16 or 32 lanes");
    MLEM_REQUIRE(!ordered || o.spmv != MLEM_SPMV_CSR_VECTOR || m->A.order != nullptr, MLEM_EINVAL,
                 "row order needs a generated matrix");
    MLEM_REQUIRE(o.spmv == MLEM_SPMV_MERGE || o.spmv == MLEM_SPMV_CSR_VECTOR, MLEM_EINVAL,
                 "spmv must be 0 (merge-based) or 1 (csr-vector)");
    MLEM_REQUIRE(o.bp_mode == MLEM_BP_TRANS || o.bp_mode == MLEM_BP_SCATTER || o.bp_mode == MLEM_BP_FUSED,
                 MLEM_EINVAL, "bp_mode must be 0 (transposed), 1 (scatter) or 2 (fused)");
    MLEM_REQUIRE(o.secsize_fp >= 1 && o.secsize_fp <= 512 && o.secsize_bp >= 1 && o.secsize_bp <= 512,
                 MLEM_EINVAL, "section sizes must be in 1..512");
    MLEM_REQUIRE(o.loglik_rel_tol >= 0.0 && std::isfinite(o.loglik_rel_tol), MLEM_EINVAL,
                 "loglik_rel_tol must be a finite value >= 0");
    MLEM_REQUIRE(o.loglik_rel_tol == 0.0 || o.loglik_every > 0, MLEM_EINVAL,
                 "loglik_rel_tol needs loglik_every > 0");
    MLEM_REQUIRE(o.bp_mode != MLEM_BP_TRANS || m->has_t, MLEM_EINVAL,
                 "transposed back projection needs a matrix created with build_transpose = 1");
}

void check_device_error(mlem_matrix* m, cudaStream_t s) {
    Workspace& w = m->ws;
    if (!w.err) return;
    uint32_t h = 0;
    MLEM_CUDA(cudaMemcpyAsync(&h, w.err, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
    MLEM_CUDA(cudaStreamSynchronize(s));
    if (h) {
        MLEM_CUDA(cudaMemsetAsync(w.err, 0, sizeof(uint32_t), s));
        MLEM_CUDA(cudaStreamSynchronize(s));
        fail(MLEM_ETIMEOUT, "a pipelined projection kernel gave up waiting for its copies; results are invalid");
    }
}

static void launch_cfg(mlem_matrix* m, const DevCsr& op, const float* x, const EpiArgs& e, const ProjCfg& c,
                       L2Window win, cudaStream_t s) {
    if (c.kind == MLEM_KERNEL_TMA) {
        ensure_workspace(m);
        launch_csr_tma(op, x, e, m->ws.err, win, s);
    } else if (c.kind == MLEM_KERNEL_D16) {
        launch_csr_d16(op, x, e, c.unroll, win, s);
    } else if (c.kind == MLEM_KERNEL_SYM) {
        launch_sym(m->sym, &op == &m->AT, x, e, c.unroll, c.ordered, win, s);
    } else if (c.kind == MLEM_KERNEL_ILV) {
        launch_csr_ilv(op, x, e, c.unroll, win, s);
    } else if (c.kind == MLEM_KERNEL_PERSISTENT) {
        launch_csrvec_pipe(op, x, e, c.lanes, c.unroll, c.ordered, win, s);
    } else {
        launch_csrvec(op, x, e, c.lanes, win, s, c.unroll, c.ordered, c.pipelined);
    }
}

// Times every candidate configuration on the operand itself (Raw epilogue
// into a scratch vector, x = 1) and keeps the fastest.  Runs once per
// operand, outside any stream capture.
static void tune_projection(mlem_matrix* m, bool transposed) {
    if (m->tuned[transposed]) return;
    const DevCsr& op = transposed ? m->AT : m->A;
    cudaStream_t s = m->stream;
    std::vector<ProjCfg> cand;
    const int base = pick_lanes(op.nnz, op.nrows);
    for (int lanes : {base / 2, base, base * 2})
        if (lanes >= 4 && lanes <= 32) {
            for (int u : {1, 2, 4}) cand.push_back(ProjCfg{MLEM_KERNEL_DIRECT, lanes, u, 0.f, false, false});
            if (lanes >= 16)
                for (int u : {1, 2})
                    for (bool ord : {false, true})
                        for (bool pipe : {false, true})
                            if ((ord || pipe) && (!ord || op.order))
                                cand.push_back(ProjCfg{MLEM_KERNEL_DIRECT, lanes, u, 0.f, ord, pipe});
        }
    if (base >= 16) cand.push_back(ProjCfg{MLEM_KERNEL_PERSISTENT, base, 1, 0.f, false, false});
    cand.push_back(ProjCfg{MLEM_KERNEL_TMA, 32, 2, 0.f});
    if (op.d16)
        for (int u : {1, 2}) cand.push_back(ProjCfg{MLEM_KERNEL_D16, op.d16_lanes, u, 0.f});
    if (op.idx_ilv)
        for (int u : {1, 2, 4}) cand.push_back(ProjCfg{MLEM_KERNEL_ILV, 32, u, 0.f});
    if (m->sym.fp_rowptr)
        for (int u : {2, 4, 8})
            for (bool grouped : {false, true}) cand.push_back(ProjCfg{MLEM_KERNEL_SYM, 32, u, 0.f, grouped, false});
    prepare_csrvec_pipe(op.vt);
    prepare_csr_tma(op.vt);
    ensure_workspace(m);
    float *x = nullptr, *y = nullptr;
    MLEM_CUDA(cudaMalloc(&x, sizeof(float) * std::max<uint32_t>(op.ncols, 1)));
    MLEM_CUDA(cudaMalloc(&y, sizeof(float) * std::max<uint32_t>(op.nrows, 1)));
    cudaEvent_t e0, e1;
    MLEM_CUDA(cudaEventCreate(&e0));
    MLEM_CUDA(cudaEventCreate(&e1));
    ProjCfg best;
    best.ms = 1e30f;
    try {
        std::vector<float> ones(std::max<uint32_t>(op.ncols, 1), 1.0f);
        MLEM_CUDA(cudaMemcpyAsync(x, ones.data(), sizeof(float) * ones.size(), cudaMemcpyHostToDevice, s));
        EpiArgs e;
        e.kind = Epi::Raw;
        e.out = y;
        const int reps = op.nnz > (50ull << 20) ? 2 : 4;
        for (ProjCfg& c : cand) {
            launch_cfg(m, op, x, e, c, {}, s);  // warm-up
            MLEM_CUDA(cudaEventRecord(e0, s));
            for (int r = 0; r < reps; ++r) launch_cfg(m, op, x, e, c, {}, s);
            MLEM_CUDA(cudaEventRecord(e1, s));
            MLEM_CUDA(cudaEventSynchronize(e1));
            float ms = 0.f;
            MLEM_CUDA(cudaEventElapsedTime(&ms, e0, e1));
            c.ms = ms / reps;
            if (c.ms < best.ms) best = c;
        }
        check_device_error(m, s);
    } catch (...) {
        cudaFree(x);
        cudaFree(y);
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        throw;
    }
    cudaFree(x);
    cudaFree(y);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    m->proj[transposed] = best;
    m->tuned[transposed] = true;
}

void prepare_kernel(mlem_matrix* m, const mlem_run_opts& o) {
    if (o.kernel == MLEM_KERNEL_TMA) prepare_csr_tma(m->vt);
    else if (o.kernel == MLEM_KERNEL_PERSISTENT) prepare_csrvec_pipe(m->vt);
    else if (o.kernel == MLEM_KERNEL_AUTO) {
        tune_projection(m, false);
        if (m->has_t) tune_projection(m, true);
    }
}

// The csr-vector configuration a projection of A (or Aᵀ) uses under opts o.
static ProjCfg resolve_cfg(const mlem_matrix* m, bool transposed, const mlem_run_opts& o) {
    const DevCsr& op = transposed ? m->AT : m->A;
    ProjCfg c;
    if (o.kernel == MLEM_KERNEL_AUTO) {
        MLEM_REQUIRE(m->tuned[transposed], MLEM_EINVAL, "internal: projection used before autotuning");
        c = m->proj[transposed];
    } else if (o.kernel == MLEM_KERNEL_PERSISTENT && (o.lanes >= 16 || pick_lanes(op.nnz, op.nrows) >= 16)) {
        c.kind = MLEM_KERNEL_PERSISTENT;
        c.lanes = o.lanes ? (int)o.lanes : pick_lanes(op.nnz, op.nrows);
        c.unroll = o.unroll ? (int)o.unroll : 2;
        c.ordered = o.row_order && op.order && c.lanes >= 16;
    } else if (o.kernel == MLEM_KERNEL_TMA) {
        c.kind = MLEM_KERNEL_TMA;
    } else if (o.kernel == MLEM_KERNEL_D16) {
        MLEM_REQUIRE(op.d16 != nullptr, MLEM_EINVAL, "kernel D16 needs a matrix created with compress_indices = 1");
        c.kind = MLEM_KERNEL_D16;
        c.lanes = op.d16_lanes;
        c.unroll = o.unroll == 1 ? 1 : 2;
    } else if (o.kernel == MLEM_KERNEL_ORDERED) {
        MLEM_REQUIRE(op.order != nullptr, MLEM_EINVAL, "kernel ORDERED needs a generated matrix (row orders)");
        c.kind = MLEM_KERNEL_DIRECT;
        c.lanes = o.lanes ? (int)o.lanes : 32;
        c.unroll = o.unroll ? std::min<int>((int)o.unroll, 2) : 2;
        c.ordered = true;
        c.pipelined = o.pipeline != 0;
    } else if (o.kernel == MLEM_KERNEL_ILV) {
        MLEM_REQUIRE(op.idx_ilv != nullptr, MLEM_EINVAL, "kernel ILV needs a matrix created with interleave = 1");
        c.kind = MLEM_KERNEL_ILV;
        c.unroll = 2;
    } else if (o.kernel == MLEM_KERNEL_SYM) {
        c.kind = MLEM_KERNEL_SYM;
        c.unroll = (o.unroll == 0 || o.unroll >= 8) ? 8 : (o.unroll == 4 ? 4 : 2);
        c.ordered = o.row_order != 0;
    } else {
        c.kind = MLEM_KERNEL_DIRECT;
        c.lanes = o.lanes ? (int)o.lanes : pick_lanes(op.nnz, op.nrows);
        c.unroll = o.unroll ? (int)o.unroll : 2;
        c.ordered = o.row_order && op.order && c.lanes >= 16;
        c.pipelined = o.pipeline && c.lanes >= 16;
    }
    return c;
}

void project(mlem_matrix* m, bool transposed, const float* x, const EpiArgs& e, const mlem_run_opts& o,
             L2Window win, cudaStream_t s) {
    const DevCsr& op = transposed ? m->AT : m->A;
    if (o.spmv == MLEM_SPMV_MERGE) {
        launch_merge_spmv(op, merge_plan(m, transposed, transposed ? o.secsize_bp : o.secsize_fp), x, e, win, s);
        return;
    }
    launch_cfg(m, op, x, e, resolve_cfg(m, transposed, o), win, s);
}

// Both projections of an MLEM iteration run the symmetry-compressed kernels:
// they then hand each other their outputs in orbit order.
static bool sym_pair(const mlem_matrix* m, const mlem_run_opts& o) {
    return m->sym.fp_rowptr && o.spmv == MLEM_SPMV_CSR_VECTOR && o.bp_mode == MLEM_BP_TRANS &&
           resolve_cfg(m, false, o).kind == MLEM_KERNEL_SYM && resolve_cfg(m, true, o).kind == MLEM_KERNEL_SYM;
}

// One MLEM iteration on stream s using the matrix workspace.
void StageTimer::record(cudaStream_t s) {
    cudaEvent_t e = nullptr;
    MLEM_CUDA(cudaEventCreate(&e));
    ev.push_back(e);
    MLEM_CUDA(cudaEventRecord(e, s));
}

void StageTimer::means(double& fp_ms, double& bp_ms) const {
    double a = 0.0, b = 0.0;
    const size_t n = ev.size() / 4;
    for (size_t i = 0; i < n; ++i) {
        float x = 0.f, y = 0.f;
        MLEM_CUDA(cudaEventElapsedTime(&x, ev[4 * i], ev[4 * i + 1]));
        MLEM_CUDA(cudaEventElapsedTime(&y, ev[4 * i + 2], ev[4 * i + 3]));
        a += x;
        b += y;
    }
    fp_ms = n ? a / n : std::numeric_limits<double>::quiet_NaN();
    bp_ms = n ? b / n : std::numeric_limits<double>::quiet_NaN();
}

StageTimer::~StageTimer() {
    for (cudaEvent_t e : ev) cudaEventDestroy(e);
}

void enqueue_iteration(mlem_matrix* m, const mlem_run_opts& o, cudaStream_t s, double* ll_slot, StageTimer* timer,
                       bool sym_fused) {
    Workspace& w = m->ws;
    const DevCsr& A = m->A;
    const bool want_ll = ll_slot != nullptr;
    L2Window wf, wr;
    if (o.l2_window) {
        wf = {w.f, sizeof(float) * (size_t)A.ncols};
        wr = {w.ratio, sizeof(float) * (size_t)A.nrows};
    }
    if (o.bp_mode == MLEM_BP_FUSED) {
        const FusedForm ff = fused_form(m, o);
        if (timer) timer->record(s);
        launch_fused(m, ff, w.f, w.g, w.bp, want_ll ? w.fwproj : nullptr, wf, s);
        if (timer) {
            timer->record(s);
            timer->record(s);
        }
        launch_update_zero(w.f, w.bp, m->norm, A.ncols, s);
        if (timer) timer->record(s);
    } else {
        EpiArgs fe;
        fe.kind = Epi::Correl;
        fe.g = w.g;
        fe.out = w.ratio;
        fe.fwproj = want_ll ? w.fwproj : nullptr;
        if (sym_fused) {
            fe.orbit_out = m->sym.orb_r;
            fe.orbit_ready = true;
            fe.orbit_only = true;
        }
        if (timer) timer->record(s);
        project(m, false, w.f, fe, o, wf, s);
        if (timer) {
            timer->record(s);
            timer->record(s);
        }
        if (o.bp_mode == MLEM_BP_TRANS) {
            EpiArgs be;
            be.kind = Epi::Update;
            be.f = w.f;
            be.norm = m->norm;
            if (sym_fused) {
                be.orbit_out = m->sym.orb_x;
                be.orbit_ready = true;
                be.orbit_only = true;
            }
            project(m, true, w.ratio, be, o, wr, s);
        } else {
            const int sl = scatter_lanes(m);  // sets m->scatter_unroll / scatter_tma on the first call
            if (o.kernel == MLEM_KERNEL_TMA || (o.kernel == MLEM_KERNEL_AUTO && m->scatter_tma)) {
                ensure_workspace(m);
                launch_scatter_tma(A, w.ratio, w.bp, w.err, wr, s);
            }
            else launch_scatter(A, w.ratio, w.bp, sl, m->scatter_unroll, wr, s);
            launch_update_zero(w.f, w.bp, m->norm, A.ncols, s);
        }
        if (timer) timer->record(s);
    }
    if (want_ll) launch_loglik(w.g, w.fwproj, A.nrows, w.ll_part, ll_slot, s);
}

float reference_initial_value(const mlem_matrix* m, const int32_t* g) {
    // main.cu:83-97: FP32 running sum of norm in column order (kept with the
    // matrix), integer sum of g
    int64_t sum_g = 0;
    for (uint32_t i = 0; i < m->A.nrows; ++i) sum_g += g[i];
    return (float)sum_g / m->norm_sum;
}

static void enable_l2_persisting(int dev) {
    static std::mutex mu;
    static std::map<int, bool> done;
    std::lock_guard<std::mutex> lk(mu);
    if (done[dev]) return;
    done[dev] = true;
    int maxp = 0, maxw = 0;
    if (cudaDeviceGetAttribute(&maxp, cudaDevAttrMaxPersistingL2CacheSize, dev) == cudaSuccess && maxp > 0 &&
        cudaDeviceGetAttribute(&maxw, cudaDevAttrMaxAccessPolicyWindowSize, dev) == cudaSuccess && maxw > 0) {
        const size_t want = std::min<size_t>((size_t)maxp, 64ull << 20);
        // context-scoped set-aside: released with this process's context
        if (cudaDeviceSetLimit(cudaLimitPersistingL2CacheSize, want) == cudaSuccess)
            g_max_window_bytes = (size_t)maxw;
    }
    cudaGetLastError();
}

static uint32_t run_iterations(mlem_matrix* m, const mlem_run_opts& o, uint32_t iters, cudaStream_t s,
                               double* ll_dev, StageTimer* timer, bool fused);

// Runs `iters` iterations on the workspace (g and f already in place);
// returns the iterations run (fewer when the convergence stop ends the run).
static uint32_t run_loop(mlem_matrix* m, const mlem_run_opts& o, uint32_t iters, cudaStream_t s,
                         double* ll_dev, StageTimer* timer = nullptr) {
    // symmetry-compressed pair: the image and the sinogram are gathered into
    // orbit order once, the iterations stay in orbit order, and the image is
    // scattered back into natural order at the end
    const bool fused = iters > 0 && sym_pair(m, o);
    if (fused) {
        sym_gather_image(m->sym, m->ws.f, s);
        sym_gather_sinogram(m->sym, m->ws.g, s);
    }
    const uint32_t ran = run_iterations(m, o, iters, s, ll_dev, timer, fused);
    if (fused) sym_scatter_image(m->sym, m->ws.f, s);
    return ran;
}

static uint32_t run_iterations(mlem_matrix* m, const mlem_run_opts& o, uint32_t iters, cudaStream_t s,
                               double* ll_dev, StageTimer* timer, bool fused) {
    if (o.loglik_every > 0 || !o.use_graph || timer) {
        double prev = 0.0;
        bool have_prev = false;
        for (uint32_t it = 0; it < iters; ++it) {
            double* slot = (o.loglik_every > 0 && it % o.loglik_every == 0) ? ll_dev + it : nullptr;
            enqueue_iteration(m, o, s, slot, timer, fused);
            if (slot && o.loglik_rel_tol > 0.0) {
                // the log-likelihood L is evaluated on the image entering this
                // iteration; stop once an evaluation gains less than tol * |L|
                double v = 0.0;
                MLEM_CUDA(cudaMemcpyAsync(&v, slot, sizeof(double), cudaMemcpyDeviceToHost, s));
                MLEM_CUDA(cudaStreamSynchronize(s));
                if (have_prev && v - prev < o.loglik_rel_tol * std::fabs(v)) return it + 1;
                prev = v;
                have_prev = true;
            }
        }
        return iters;
    }
    constexpr uint32_t kChunk = 8;
    auto get_graph = [&](uint32_t chunk) -> cudaGraphExec_t {
        RunKey key{(int)o.spmv, (int)o.bp_mode, (int)o.secsize_fp, (int)o.secsize_bp, (int)o.l2_window,
                   (int)chunk, (int)(o.kernel | o.lanes << 8 | o.unroll << 16 | o.row_order << 24 | o.pipeline << 25)};
        auto it = m->ws.graphs.find(key);
        if (it != m->ws.graphs.end()) return it->second;
        // plans and kernel attributes must exist before capture
        if (o.spmv == MLEM_SPMV_CSR_VECTOR) prepare_kernel(m, o);
        if (o.spmv == MLEM_SPMV_MERGE && o.bp_mode != MLEM_BP_FUSED) {
            merge_plan(m, false, o.secsize_fp);
            if (o.bp_mode == MLEM_BP_TRANS) merge_plan(m, true, o.secsize_bp);
        }
        if (o.bp_mode == MLEM_BP_SCATTER) scatter_lanes(m);
        if (o.bp_mode == MLEM_BP_FUSED) fused_form(m, o);
        cudaStream_t cs = m->stream;
        cudaGraph_t graph = nullptr;
        const uint64_t l0 = g_launches.load();
        MLEM_CUDA(cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal));
        try {
            for (uint32_t q = 0; q < chunk; ++q) enqueue_iteration(m, o, cs, nullptr, nullptr, fused);
        } catch (...) {
            cudaStreamEndCapture(cs, &graph);
            if (graph) cudaGraphDestroy(graph);
            throw;
        }
        MLEM_CUDA(cudaStreamEndCapture(cs, &graph));
        // captured launches are counted when the graph is replayed, not here
        const uint64_t nodes = g_launches.load() - l0;
        g_launches.fetch_sub(nodes);
        cudaGraphExec_t exec = nullptr;
        const cudaError_t e = cudaGraphInstantiate(&exec, graph, 0);
        cudaGraphDestroy(graph);
        MLEM_CUDA(e);
        m->ws.graphs[key] = exec;
        m->ws.graph_nodes[key] = nodes;
        return exec;
    };
    const uint32_t full = iters / kChunk, rest = iters % kChunk;
    auto replay = [&](uint32_t chunk, uint32_t times) {
        cudaGraphExec_t ge = get_graph(chunk);
        const RunKey key{(int)o.spmv, (int)o.bp_mode, (int)o.secsize_fp, (int)o.secsize_bp,
                         (int)o.l2_window, (int)chunk, (int)(o.kernel | o.lanes << 8 | o.unroll << 16 | o.row_order << 24 | o.pipeline << 25)};
        const uint64_t nodes = m->ws.graph_nodes[key];
        for (uint32_t q = 0; q < times; ++q) {
            MLEM_CUDA(cudaGraphLaunch(ge, s));
            count_launch(nodes);
        }
    };
    if (full) replay(kChunk, full);
    if (rest) replay(1, rest);
    return iters;
}

static void postprocess_matrix(mlem_matrix* m, const mlem_matrix_opts& o) {
    cudaStream_t s = m->stream;
    DevCsr& A = m->A;
    A.max_row = max_row_length(A.rowptr, A.nrows, s);
    if (o.build_transpose && !m->has_t) {
        transpose_device(A, m->AT, s);
        m->has_t = true;
    }
    // low-precision storage first, so the sensitivity image is Aᵀ1 of the
    // matrix the projections actually use
    if (o.value_type != MLEM_VAL_F32) {
        auto lower = [&](DevCsr& c) {
            void* nv = nullptr;
            MLEM_CUDA(cudaMalloc(&nv, 2 * padded(c.nnz)));
            convert_values(static_cast<const float*>(c.val), nv, o.value_type, padded(c.nnz), s);
            MLEM_CUDA(cudaStreamSynchronize(s));
            cudaFree(c.val);
            c.val = nv;
            c.vt = o.value_type;
        };
        lower(A);
        if (m->has_t) lower(m->AT);
    }
    m->vt = o.value_type;
    if (o.compress_indices) {
        build_d16(A, s);
        if (m->has_t) build_d16(m->AT, s);
    }
    if (o.interleave) {
        build_ilv(A, s);
        if (m->has_t) build_ilv(m->AT, s);
    }
    MLEM_CUDA(cudaMalloc(&m->norm, sizeof(float) * std::max<uint32_t>(A.ncols, 1)));
    m->norm_host.resize(A.ncols);
    if (o.norm) {
        // given in natural column order
        if (m->vox_of && A.ncols) {
            float* nat = nullptr;
            MLEM_CUDA(cudaMalloc(&nat, sizeof(float) * A.ncols));
            MLEM_CUDA(cudaMemcpyAsync(nat, o.norm, sizeof(float) * A.ncols, cudaMemcpyHostToDevice, s));
            launch_gather_f32(m->norm, nat, m->vox_of, A.ncols, s);
            MLEM_CUDA(cudaStreamSynchronize(s));
            cudaFree(nat);
        } else {
            MLEM_CUDA(cudaMemcpyAsync(m->norm, o.norm, sizeof(float) * A.ncols, cudaMemcpyHostToDevice, s));
        }
        std::copy(o.norm, o.norm + A.ncols, m->norm_host.begin());
    } else {
        if (m->has_t) colsum_from_transpose(m->AT, m->norm, s);
        else colsum_scatter(A, m->norm, s);
        if (A.ncols)
            MLEM_CUDA(cudaMemcpyAsync(m->norm_host.data(), m->norm, sizeof(float) * A.ncols,
                                      cudaMemcpyDeviceToHost, s));
        MLEM_CUDA(cudaStreamSynchronize(s));
        if (m->vox_of) {  // back to natural order for the host copy
            std::vector<float> internal(m->norm_host);
            for (uint32_t p = 0; p < A.ncols; ++p) m->norm_host[m->vox_of_host[p]] = internal[p];
        }
    }
    MLEM_CUDA(cudaStreamSynchronize(s));
    m->norm_sum = 0.0f;
    for (float v : m->norm_host) m->norm_sum += v;
}

// Puts A (natural order, f32) into the locality layout.  lor: natural row of
// every internal row (empty = keep the row order); vox: natural column of
// every internal column.  keep_t: keep the transpose built on the way as Aᵀ.
static void apply_layout(mlem_matrix* m, const std::vector<uint32_t>& lor, const std::vector<uint32_t>& vox,
                         bool keep_t) {
    cudaStream_t s = m->stream;
    DevCsr& A = m->A;
    MLEM_REQUIRE(A.vt == MLEM_VAL_F32, MLEM_EINVAL, "internal: layout before value conversion");
    MLEM_REQUIRE(lor.empty() || lor.size() == A.nrows, MLEM_EINVAL, "internal: row order size");
    MLEM_REQUIRE(vox.size() == A.ncols, MLEM_EINVAL,
                 "locality layout: the voxel grid (nx*ny*nz) does not match the number of columns");
    std::vector<uint32_t> pos(A.ncols, UINT32_MAX);
    for (uint32_t p = 0; p < A.ncols; ++p) {
        MLEM_REQUIRE(vox[p] < A.ncols && pos[vox[p]] == UINT32_MAX, MLEM_EINVAL, "internal: voxel order");
        pos[vox[p]] = p;
    }
    uint32_t* d_pos = nullptr;
    try {
        if (!lor.empty()) {
            MLEM_CUDA(cudaMalloc(&m->lor_of, sizeof(uint32_t) * lor.size()));
            MLEM_CUDA(cudaMemcpy(m->lor_of, lor.data(), sizeof(uint32_t) * lor.size(), cudaMemcpyHostToDevice));
        }
        MLEM_CUDA(cudaMalloc(&m->vox_of, sizeof(uint32_t) * std::max<size_t>(vox.size(), 1)));
        MLEM_CUDA(cudaMalloc(&d_pos, sizeof(uint32_t) * std::max<size_t>(pos.size(), 1)));
        if (!vox.empty()) {
            MLEM_CUDA(cudaMemcpy(m->vox_of, vox.data(), sizeof(uint32_t) * vox.size(), cudaMemcpyHostToDevice));
            MLEM_CUDA(cudaMemcpy(d_pos, pos.data(), sizeof(uint32_t) * pos.size(), cudaMemcpyHostToDevice));
        }
        DevCsr An, Tn;
        remap_csr(A, m->lor_of, d_pos, An, keep_t ? &Tn : nullptr, s);
        free_csr(A);
        A = An;
        if (keep_t) {
            m->AT = Tn;
            m->has_t = true;
        }
    } catch (...) {
        cudaFree(d_pos);
        throw;
    }
    cudaFree(d_pos);
    m->vox_of_host = vox;
}

// The layout the options ask for, given the voxel grid and, for generated
// matrices, the detector-tube LOR order (empty: the order derived from the
// matrix's own columns).
static void maybe_apply_layout(mlem_matrix* m, const mlem_matrix_opts& o, uint32_t nx, uint32_t ny, uint32_t nz,
                               const std::vector<uint32_t>& lor) {
    if (o.layout == MLEM_LAYOUT_NATURAL) return;
    MLEM_REQUIRE(nx && ny && nz && (uint64_t)nx * ny * nz == m->A.ncols, MLEM_EINVAL,
                 "locality layout needs the voxel grid: nx*ny*nz must equal the number of columns");
    apply_layout(m, lor.empty() ? derived_lor_order(m->A, nx, ny, nz, m->stream) : lor,
                 voxel_brick_order(nx, ny, nz, 4, 4, 2), o.build_transpose != 0);
}

static mlem_matrix* new_matrix(const mlem_matrix_opts& o) {
    MLEM_REQUIRE(o.value_type == MLEM_VAL_F32 || o.value_type == MLEM_VAL_F16 ||
                     o.value_type == MLEM_VAL_BF16,
                 MLEM_EINVAL, "value_type must be F32, F16 or BF16");
    MLEM_REQUIRE(o.layout == MLEM_LAYOUT_NATURAL || o.layout == MLEM_LAYOUT_LOCALITY, MLEM_EINVAL,
                 "layout must be 0 (natural) or 1 (locality)");
    int ndev = 0;
    MLEM_CUDA(cudaGetDeviceCount(&ndev));
    MLEM_REQUIRE(o.device >= 0 && o.device < ndev, MLEM_EINVAL, "device ordinal out of range");
    auto* m = new mlem_matrix();
    m->device = o.device;
    MLEM_CUDA(cudaStreamCreateWithFlags(&m->stream, cudaStreamNonBlocking));
    enable_l2_persisting(o.device);
    return m;
}

static void destroy_matrix(mlem_matrix* m) {
    if (!m) return;
    DeviceGuard dg(m->device);
    if (m->stream) cudaStreamSynchronize(m->stream);
    m->ws.release();
    for (auto& kv : m->plan_A) kv.second.release();
    for (auto& kv : m->plan_AT) kv.second.release();
    m->fused.release();
    free_csr(m->A);
    free_csr(m->AT);
    m->sym.release();
    cudaFree(m->norm);
    cudaFree(m->lor_of);
    cudaFree(m->vox_of);
    if (m->stream) cudaStreamDestroy(m->stream);
    delete m;
}

static void check_host_csr(const mlem_csr_host* c) {
    MLEM_REQUIRE(c != nullptr, MLEM_EINVAL, "csr is NULL");
    MLEM_REQUIRE(c->rowptr != nullptr, MLEM_EINVAL, "csr rowptr is NULL");
    MLEM_REQUIRE(c->nnz == 0 || (c->col && c->val), MLEM_EINVAL, "csr col/val is NULL");
    MLEM_REQUIRE(c->rows >= 1 && c->cols >= 1, MLEM_EINVAL, "matrix must have rows and columns");
    MLEM_REQUIRE(c->rowptr[0] == 0, MLEM_EINVAL, "rowptr[0] must be 0");
    for (uint32_t r = 0; r < c->rows; ++r)
        MLEM_REQUIRE(c->rowptr[r + 1] >= c->rowptr[r], MLEM_EINVAL, "rowptr must be nondecreasing");
    MLEM_REQUIRE(c->rowptr[c->rows] == c->nnz, MLEM_EINVAL, "rowptr[rows] must equal nnz");
}

static void upload_csr(const mlem_csr_host* c, DevCsr& A, cudaStream_t s) {
    A.nrows = c->rows;
    A.ncols = c->cols;
    A.nnz = c->nnz;
    A.vt = MLEM_VAL_F32;
    MLEM_CUDA(cudaMalloc(&A.rowptr, sizeof(uint64_t) * ((uint64_t)c->rows + 1)));
    MLEM_CUDA(cudaMalloc(&A.idx, sizeof(uint32_t) * padded(c->nnz)));
    MLEM_CUDA(cudaMalloc(&A.val, sizeof(float) * padded(c->nnz)));
    MLEM_CUDA(cudaMemsetAsync(A.idx, 0, sizeof(uint32_t) * padded(c->nnz), s));
    MLEM_CUDA(cudaMemsetAsync(A.val, 0, sizeof(float) * padded(c->nnz), s));
    MLEM_CUDA(cudaMemcpyAsync(A.rowptr, c->rowptr, sizeof(uint64_t) * ((uint64_t)c->rows + 1),
                              cudaMemcpyHostToDevice, s));
    if (c->nnz) {
        MLEM_CUDA(cudaMemcpyAsync(A.idx, c->col, sizeof(uint32_t) * c->nnz, cudaMemcpyHostToDevice, s));
        MLEM_CUDA(cudaMemcpyAsync(A.val, c->val, sizeof(float) * c->nnz, cudaMemcpyHostToDevice, s));
    }
    MLEM_CUDA(cudaStreamSynchronize(s));
    MLEM_REQUIRE(validate_csr(A, s), MLEM_EINVAL, "csr column index >= cols or malformed row pointers");
}

mlem_matrix* create_matrix_filled(const mlem_matrix_opts& o, const std::function<void(mlem_matrix*)>& fill) {
    MLEM_REQUIRE(!o.symmetry, MLEM_EUNSUPPORTED,
                 "symmetry: create the matrix from host CSR arrays (mlem_matrix_create) or a geometry");
    DeviceGuard dg(o.device);
    mlem_matrix* m = new_matrix(o);
    try {
        fill(m);
        MLEM_CUDA(cudaStreamSynchronize(m->stream));
        MLEM_REQUIRE(validate_csr(m->A, m->stream), MLEM_EINVAL,
                     "csr column index >= cols or malformed row pointers");
        maybe_apply_layout(m, o, o.grid_nx, o.grid_ny, o.grid_nz, {});
        postprocess_matrix(m, o);
    } catch (...) {
        destroy_matrix(m);
        throw;
    }
    return m;
}

}  // namespace mlem

using namespace mlem;

uint64_t mlem_matrix::bytes() const {
    uint64_t b = csr_bytes(A) + csr_bytes(AT) + sizeof(float) * (uint64_t)A.ncols + sym.bytes();
    for (auto& kv : plan_A) b += kv.second.ntiles * 24;
    for (auto& kv : plan_AT) b += kv.second.ntiles * 24;
    b += fused.nchunks * sizeof(FusedChunk) + fused.meta_len * sizeof(uint32_t);
    if (ws.ready) b += (uint64_t)A.nrows * 12 + (uint64_t)A.ncols * 8;
    return b;
}

extern "C" {

const char* mlem_last_error(void) { return get_error(); }
const char* mlem_version(void) { return "mlem-gb300 1.0 (sm_103a)"; }
uint64_t mlem_kernel_launch_count(void) { return g_launches.load(); }

void mlem_matrix_opts_default(mlem_matrix_opts* o) {
    if (!o) return;
    o->value_type = MLEM_VAL_F32;
    o->build_transpose = 1;
    o->norm = nullptr;
    o->device = 0;
    o->compress_indices = 0;
    o->interleave = 0;
    o->layout = MLEM_LAYOUT_NATURAL;
    o->grid_nx = o->grid_ny = o->grid_nz = 0;
    o->symmetry = 0;
    o->sym_det_per_ring = o->sym_rings = 0;
}

void mlem_run_opts_default(mlem_run_opts* o) {
    if (!o) return;
    o->spmv = MLEM_SPMV_CSR_VECTOR;
    o->bp_mode = MLEM_BP_TRANS;
    o->secsize_fp = 5;
    o->secsize_bp = 5;
    o->use_graph = 1;
    o->loglik_every = 0;
    o->l2_window = 1;
    o->kernel = MLEM_KERNEL_AUTO;
    o->lanes = 0;
    o->unroll = 0;
    o->row_order = 0;
    o->pipeline = 0;
    o->kernel_timing = 0;
    o->loglik_rel_tol = 0.0;
}

mlem_status mlem_matrix_create(const mlem_csr_host* csr, const mlem_matrix_opts* opts, mlem_matrix** out) {
    return guarded([&] {
        MLEM_REQUIRE(out != nullptr, MLEM_EINVAL, "out is NULL");
        *out = nullptr;
        mlem_matrix_opts o;
        mlem_matrix_opts_default(&o);
        if (opts) o = *opts;
        check_host_csr(csr);
        DeviceGuard dg(o.device);
        mlem_matrix* m = new_matrix(o);
        try {
            upload_csr(csr, m->A, m->stream);
            if (o.symmetry) {
                MLEM_REQUIRE(o.layout == MLEM_LAYOUT_NATURAL, MLEM_EUNSUPPORTED,
                             "symmetry keeps the natural layout (the symmetric operands are compact already)");
                MLEM_REQUIRE(o.grid_nx == o.grid_ny, MLEM_EUNSUPPORTED, "symmetry needs a square voxel grid");
                DevCsr hat;
                try {
                    build_symmetric_checked(*csr, m->A, o.grid_nx, o.grid_nz, o.sym_det_per_ring, o.sym_rings, hat,
                                            m->AT, m->sym, m->stream);
                } catch (...) {
                    free_csr(hat);
                    throw;
                }
                free_csr(hat);  // equal to the caller's matrix, which stays
                m->has_t = true;
                postprocess_matrix(m, o);
                lower_symmetric_values(m->sym, o.value_type, m->stream);
                sym_set_norm(m->sym, m->norm, m->stream);
                MLEM_CUDA(cudaStreamSynchronize(m->stream));
            } else {
                maybe_apply_layout(m, o, o.grid_nx, o.grid_ny, o.grid_nz, {});
                postprocess_matrix(m, o);
            }
        } catch (...) {
            destroy_matrix(m);
            throw;
        }
        *out = m;
    });
}

mlem_status mlem_matrix_generate(const mlem_geometry* geo, const mlem_matrix_opts* opts, mlem_matrix** out) {
    return guarded([&] {
        MLEM_REQUIRE(out != nullptr && geo != nullptr, MLEM_EINVAL, "NULL argument");
        *out = nullptr;
        mlem_matrix_opts o;
        mlem_matrix_opts_default(&o);
        if (opts) o = *opts;
        DeviceGuard dg(o.device);
        mlem_matrix* m = new_matrix(o);
        try {
            if (o.symmetry) {
                MLEM_REQUIRE(o.layout == MLEM_LAYOUT_NATURAL, MLEM_EUNSUPPORTED,
                             "symmetry keeps the natural layout (the symmetric operands are compact already)");
                build_symmetric(*geo, m->A, m->AT, m->sym, m->stream);
                m->has_t = true;
                postprocess_matrix(m, o);
                lower_symmetric_values(m->sym, o.value_type, m->stream);
                sym_set_norm(m->sym, m->norm, m->stream);
                MLEM_CUDA(cudaStreamSynchronize(m->stream));
            } else {
                siddon_generate_device(*geo, m->A, m->stream);
                MLEM_REQUIRE(m->A.nrows >= 1, MLEM_EINVAL, "geometry produced no rows");
                maybe_apply_layout(m, o, geo->nx, geo->ny, geo->nz, siddon_lor_order(*geo));
                postprocess_matrix(m, o);
            }
            if (o.layout == MLEM_LAYOUT_NATURAL) {
                // locality orders of the rows (processing order only): LOR
                // tubes for A, voxel bricks for Aᵀ
                auto upload = [&](DevCsr& op, const std::vector<uint32_t>& ord) {
                    if (ord.size() != op.nrows || op.nrows == 0) return;
                    MLEM_CUDA(cudaMalloc(&op.order, sizeof(uint32_t) * ord.size()));
                    MLEM_CUDA(cudaMemcpy(op.order, ord.data(), sizeof(uint32_t) * ord.size(),
                                         cudaMemcpyHostToDevice));
                };
                upload(m->A, siddon_lor_order(*geo));
                if (m->has_t) upload(m->AT, voxel_brick_order(geo->nx, geo->ny, geo->nz));
            }
        } catch (...) {
            destroy_matrix(m);
            throw;
        }
        *out = m;
    });
}

mlem_status mlem_matrix_destroy(mlem_matrix* m) {
    return guarded([&] { destroy_matrix(m); });
}

mlem_status mlem_matrix_get_info(const mlem_matrix* m, mlem_matrix_info* info) {
    return guarded([&] {
        MLEM_REQUIRE(m && info, MLEM_EINVAL, "NULL argument");
        info->rows = m->A.nrows;
        info->cols = m->A.ncols;
        info->nnz = m->A.nnz;
        info->value_type = m->vt;
        info->has_transpose = m->has_t ? 1 : 0;
        info->device_bytes = m->bytes();
        info->max_row_nnz = m->A.max_row;
        info->max_col_nnz = m->has_t ? m->AT.max_row : 0;
        info->sym_lor_rows = m->sym.K;
        info->sym_voxel_rows = m->sym.J;
        info->sym_fp_nnz = m->sym.fp_nnz;
        info->sym_bp_nnz = m->sym.bp_nnz;
        info->d16_slots = 8 * m->A.dvec;
        info->d16_slots_t = m->has_t ? 8 * m->AT.dvec : 0;
        info->d16_lanes = (uint32_t)m->A.d16_lanes;
        info->d16_lanes_t = m->has_t ? (uint32_t)m->AT.d16_lanes : 0;
    });
}

mlem_status mlem_matrix_get_tuning(mlem_matrix* m, uint32_t transposed, int* kernel, int* lanes, int* unroll,
                                   int* ordered, int* pipelined, float* ms) {
    return guarded([&] {
        MLEM_REQUIRE(m && kernel && lanes && unroll && ordered && pipelined && ms, MLEM_EINVAL, "NULL argument");
        MLEM_REQUIRE(transposed <= 2, MLEM_EINVAL, "transposed must be 0, 1 or 2 (fused pass)");
        MLEM_REQUIRE(transposed != 1 || m->has_t, MLEM_EINVAL, "matrix has no transpose");
        std::lock_guard<std::mutex> lk(m->mu);
        DeviceGuard dg(m->device);
        if (transposed == 2) {
            mlem_run_opts o;
            mlem_run_opts_default(&o);
            o.bp_mode = MLEM_BP_FUSED;
            const FusedForm f = fused_form(m, o);
            *kernel = f.kind == 1 ? MLEM_KERNEL_TMA : f.kind == 0 ? MLEM_KERNEL_PERSISTENT : MLEM_KERNEL_DIRECT;
            *lanes = f.kind == 1 ? f.threads : f.kind == 2 ? f.lanes : 32;
            *unroll = f.kind == 2 ? f.unroll : 1;
            *ordered = f.kind == 2 && f.ordered ? 1 : 0;
            *pipelined = 0;
            *ms = f.ms;
            return;
        }
        tune_projection(m, transposed != 0);
        const ProjCfg& c = m->proj[transposed];
        *kernel = c.kind;
        *lanes = c.lanes;
        *unroll = c.unroll;
        *ordered = c.ordered ? 1 : 0;
        *pipelined = c.pipelined ? 1 : 0;
        *ms = c.ms;
    });
}

mlem_status mlem_matrix_get_norm(const mlem_matrix* m, float* norm_out) {
    return guarded([&] {
        MLEM_REQUIRE(m && norm_out, MLEM_EINVAL, "NULL argument");
        std::memcpy(norm_out, m->norm_host.data(), sizeof(float) * m->A.ncols);
    });
}

namespace mlem {
// Copies a device operand to host CSR arrays (values converted to f32).
static void copy_csr_to_host(const DevCsr& c, uint64_t* rowptr, uint32_t* idx, float* val, cudaStream_t s) {
    MLEM_CUDA(cudaMemcpy(rowptr, c.rowptr, sizeof(uint64_t) * ((uint64_t)c.nrows + 1), cudaMemcpyDeviceToHost));
    if (!c.nnz) return;
    MLEM_CUDA(cudaMemcpy(idx, c.idx, sizeof(uint32_t) * c.nnz, cudaMemcpyDeviceToHost));
    float* tmp = nullptr;
    MLEM_CUDA(cudaMalloc(&tmp, sizeof(float) * c.nnz));
    convert_values_back(c.val, tmp, c.vt, c.nnz, s);
    MLEM_CUDA(cudaStreamSynchronize(s));
    const cudaError_t e = cudaMemcpy(val, tmp, sizeof(float) * c.nnz, cudaMemcpyDeviceToHost);
    cudaFree(tmp);
    MLEM_CUDA(e);
}

// A (transposed = false) or Aᵀ of a matrix in the locality layout, back in
// natural order, as a new f32 device CSR.
static DevCsr natural_operand(const mlem_matrix* m, bool transposed) {
    cudaStream_t s = m->stream;
    const DevCsr& src = transposed ? m->AT : m->A;
    const uint32_t* perm_rows = transposed ? m->vox_of : m->lor_of;  // natural index of internal rows
    const uint32_t* col_map = transposed ? m->lor_of : m->vox_of;    // internal column -> natural
    DevCsr view = src, out;
    float* v32 = nullptr;
    uint32_t* inv = nullptr;
    try {
        if (src.vt != MLEM_VAL_F32) {
            MLEM_CUDA(cudaMalloc(&v32, sizeof(float) * padded(src.nnz)));
            convert_values_back(src.val, v32, src.vt, padded(src.nnz), s);
            view.val = v32;
            view.vt = MLEM_VAL_F32;
        }
        if (perm_rows) {
            MLEM_CUDA(cudaMalloc(&inv, sizeof(uint32_t) * std::max<uint32_t>(src.nrows, 1)));
            launch_invert_perm(perm_rows, src.nrows, inv, s);
        }
        remap_csr(view, inv, col_map, out, nullptr, s);
    } catch (...) {
        cudaStreamSynchronize(s);
        cudaFree(v32);
        cudaFree(inv);
        throw;
    }
    cudaFree(v32);
    cudaFree(inv);
    return out;
}
}  // namespace mlem

mlem_status mlem_matrix_get_transpose(const mlem_matrix* m, uint64_t* colptr, uint32_t* rowidx, float* val) {
    return guarded([&] {
        MLEM_REQUIRE(m && colptr && rowidx && val, MLEM_EINVAL, "NULL argument");
        MLEM_REQUIRE(m->has_t, MLEM_EINVAL, "matrix has no transpose");
        DeviceGuard dg(m->device);
        if (!permuted(m)) {
            copy_csr_to_host(m->AT, colptr, rowidx, val, m->stream);
            return;
        }
        DevCsr nat = natural_operand(m, true);
        try {
            copy_csr_to_host(nat, colptr, rowidx, val, m->stream);
        } catch (...) {
            free_csr(nat);
            throw;
        }
        free_csr(nat);
    });
}

mlem_status mlem_matrix_get_csr(const mlem_matrix* m, uint64_t* rowptr, uint32_t* col, float* val) {
    return guarded([&] {
        MLEM_REQUIRE(m && rowptr && col && val, MLEM_EINVAL, "NULL argument");
        DeviceGuard dg(m->device);
        if (!permuted(m)) {
            copy_csr_to_host(m->A, rowptr, col, val, m->stream);
            return;
        }
        DevCsr nat = natural_operand(m, false);
        try {
            copy_csr_to_host(nat, rowptr, col, val, m->stream);
        } catch (...) {
            free_csr(nat);
            throw;
        }
        free_csr(nat);
    });
}

mlem_status mlem_initial_value(const mlem_matrix* m, const int32_t* g, float* init_out) {
    return guarded([&] {
        MLEM_REQUIRE(m && g && init_out, MLEM_EINVAL, "NULL argument");
        *init_out = reference_initial_value(m, g);
    });
}

mlem_status mlem_run(mlem_matrix* m, const int32_t* g, const float* f0, uint32_t iterations,
                     const mlem_run_opts* opts, float* f_out, double* loglik_out, mlem_stats* stats) {
    return guarded([&] {
        const auto t0 = std::chrono::steady_clock::now();
        MLEM_REQUIRE(m && g && f_out, MLEM_EINVAL, "NULL argument");
        MLEM_REQUIRE(iterations > 0, MLEM_EINVAL, "iterations must be > 0");
        mlem_run_opts o;
        mlem_run_opts_default(&o);
        if (opts) o = *opts;
        check_run_opts(m, o);
        std::lock_guard<std::mutex> lk(m->mu);
        DeviceGuard dg(m->device);
        ensure_workspace(m);
        cudaStream_t s = m->stream;
        const uint32_t rows = m->A.nrows, cols = m->A.ncols;
        Workspace& w = m->ws;
        if (o.spmv == MLEM_SPMV_CSR_VECTOR) prepare_kernel(m, o);
        const bool perm = permuted(m);
        if (perm) {  // natural order staged, then permuted into the workspace
            int32_t* gt = reinterpret_cast<int32_t*>(w.tmp_rows);
            MLEM_CUDA(cudaMemcpyAsync(gt, g, sizeof(int32_t) * rows, cudaMemcpyHostToDevice, s));
            rows_in_i32(m, w.g, gt, s);
        } else {
            MLEM_CUDA(cudaMemcpyAsync(w.g, g, sizeof(int32_t) * rows, cudaMemcpyHostToDevice, s));
        }
        uint64_t h2d = sizeof(int32_t) * (uint64_t)rows;
        if (f0) {
            if (perm) {
                MLEM_CUDA(cudaMemcpyAsync(w.tmp_cols, f0, sizeof(float) * cols, cudaMemcpyHostToDevice, s));
                cols_in(m, w.f, w.tmp_cols, s);
            } else {
                MLEM_CUDA(cudaMemcpyAsync(w.f, f0, sizeof(float) * cols, cudaMemcpyHostToDevice, s));
            }
            h2d += sizeof(float) * (uint64_t)cols;
        } else {
            std::vector<float> init(cols, reference_initial_value(m, g));
            MLEM_CUDA(cudaMemcpyAsync(w.f, init.data(), sizeof(float) * cols, cudaMemcpyHostToDevice, s));
            MLEM_CUDA(cudaStreamSynchronize(s));
            h2d += sizeof(float) * (uint64_t)cols;
        }
        if (o.loglik_every > 0 && w.ll_cap < iterations) {
            cudaFree(w.ll_vals);
            w.ll_vals = nullptr;
            MLEM_CUDA(cudaMalloc(&w.ll_vals, sizeof(double) * iterations));
            w.ll_cap = iterations;
        }
        if (o.loglik_every > 0) {
            std::vector<double> nan(iterations, std::numeric_limits<double>::quiet_NaN());
            MLEM_CUDA(cudaMemcpyAsync(w.ll_vals, nan.data(), sizeof(double) * iterations, cudaMemcpyHostToDevice, s));
            MLEM_CUDA(cudaStreamSynchronize(s));
        }
        cudaEvent_t e0, e1;
        MLEM_CUDA(cudaEventCreate(&e0));
        MLEM_CUDA(cudaEventCreate(&e1));
        const uint64_t l0 = g_launches.load();
        StageTimer timer;
        MLEM_CUDA(cudaEventRecord(e0, s));
        const uint32_t ran = run_loop(m, o, iterations, s, w.ll_vals, o.kernel_timing ? &timer : nullptr);
        MLEM_CUDA(cudaEventRecord(e1, s));
        const uint64_t l1 = g_launches.load();
        if (perm) {
            cols_out(m, w.tmp_cols, w.f, s);
            MLEM_CUDA(cudaMemcpyAsync(f_out, w.tmp_cols, sizeof(float) * cols, cudaMemcpyDeviceToHost, s));
        } else {
            MLEM_CUDA(cudaMemcpyAsync(f_out, w.f, sizeof(float) * cols, cudaMemcpyDeviceToHost, s));
        }
        std::vector<double> ll;
        if (o.loglik_every > 0) {
            ll.resize(iterations);
            MLEM_CUDA(cudaMemcpyAsync(ll.data(), w.ll_vals, sizeof(double) * iterations, cudaMemcpyDeviceToHost, s));
        }
        MLEM_CUDA(cudaStreamSynchronize(s));
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        check_device_error(m, s);
        if (loglik_out) {
            for (uint32_t i = 0; i < iterations; ++i)
                loglik_out[i] = ll.empty() ? std::numeric_limits<double>::quiet_NaN() : ll[i];
        }
        if (stats) {
            stats->seconds_total =
                std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
            stats->seconds_iterations = ms * 1e-3;
            stats->iterations = ran;
            stats->kernel_launches = (uint32_t)(l1 - l0);
            stats->bytes_h2d = h2d;
            stats->bytes_d2h = sizeof(float) * (uint64_t)cols;
            stats->loglik_last = std::numeric_limits<double>::quiet_NaN();
            timer.means(stats->fp_ms, stats->bp_ms);
            for (uint32_t i = iterations; i-- > 0;)
                if (!ll.empty() && !std::isnan(ll[i])) {
                    stats->loglik_last = ll[i];
                    break;
                }
        }
    });
}

mlem_status mlem_run_device(mlem_matrix* m, const int32_t* g_dev, float* f_dev, uint32_t iterations,
                            const mlem_run_opts* opts, void* stream) {
    return guarded([&] {
        MLEM_REQUIRE(m && g_dev && f_dev, MLEM_EINVAL, "NULL argument");
        MLEM_REQUIRE(iterations > 0, MLEM_EINVAL, "iterations must be > 0");
        mlem_run_opts o;
        mlem_run_opts_default(&o);
        if (opts) o = *opts;
        MLEM_REQUIRE(o.loglik_every == 0, MLEM_EINVAL, "log-likelihood output needs mlem_run");
        check_run_opts(m, o);
        std::lock_guard<std::mutex> lk(m->mu);
        DeviceGuard dg(m->device);
        ensure_workspace(m);
        cudaStream_t s = static_cast<cudaStream_t>(stream);
        const uint32_t rows = m->A.nrows, cols = m->A.ncols;
        Workspace& w = m->ws;
        if (o.spmv == MLEM_SPMV_CSR_VECTOR) prepare_kernel(m, o);
        (void)rows;
        (void)cols;
        rows_in_i32(m, w.g, g_dev, s);
        cols_in(m, w.f, f_dev, s);
        run_loop(m, o, iterations, s, nullptr);
        cols_out(m, f_dev, w.f, s);
    });
}

mlem_status mlem_forward_project(mlem_matrix* m, const float* f_dev, const int32_t* g_dev, float* ratio_dev,
                                 float* fwproj_out_dev, const mlem_run_opts* opts, void* stream) {
    return guarded([&] {
        MLEM_REQUIRE(m && f_dev && g_dev && ratio_dev, MLEM_EINVAL, "NULL argument");
        mlem_run_opts o;
        mlem_run_opts_default(&o);
        if (opts) o = *opts;
        check_run_opts(m, o);
        std::lock_guard<std::mutex> lk(m->mu);
        DeviceGuard dg(m->device);
        cudaStream_t s = static_cast<cudaStream_t>(stream);
        if (o.spmv == MLEM_SPMV_CSR_VECTOR) prepare_kernel(m, o);
        EpiArgs fe;
        fe.kind = Epi::Correl;
        if (!permuted(m)) {
            fe.g = g_dev;
            fe.out = ratio_dev;
            fe.fwproj = fwproj_out_dev;
            project(m, false, f_dev, fe, o, {}, s);
        } else {  // internal order in the workspace, natural order at the boundary
            ensure_workspace(m);
            Workspace& w = m->ws;
            cols_in(m, w.tmp_cols, f_dev, s);
            rows_in_i32(m, w.g, g_dev, s);
            fe.g = w.g;
            fe.out = w.tmp_rows;
            fe.fwproj = fwproj_out_dev ? w.fwproj : nullptr;
            project(m, false, w.tmp_cols, fe, o, {}, s);
            rows_out(m, ratio_dev, w.tmp_rows, s);
            if (fwproj_out_dev) rows_out(m, fwproj_out_dev, w.fwproj, s);
        }
    });
}

mlem_status mlem_back_project(mlem_matrix* m, const float* ratio_dev, float* bp_dev, const mlem_run_opts* opts,
                              void* stream) {
    return guarded([&] {
        MLEM_REQUIRE(m && ratio_dev && bp_dev, MLEM_EINVAL, "NULL argument");
        mlem_run_opts o;
        mlem_run_opts_default(&o);
        if (opts) o = *opts;
        check_run_opts(m, o);
        std::lock_guard<std::mutex> lk(m->mu);
        DeviceGuard dg(m->device);
        cudaStream_t s = static_cast<cudaStream_t>(stream);
        const bool perm = permuted(m);
        const float* r = ratio_dev;
        float* out = bp_dev;
        if (perm) {  // internal order in the workspace, natural order at the boundary
            ensure_workspace(m);
            rows_in_f32(m, m->ws.tmp_rows, ratio_dev, s);
            r = m->ws.tmp_rows;
            out = m->ws.tmp_cols;
        }
        if (o.bp_mode == MLEM_BP_TRANS) {
            EpiArgs be;
            be.kind = Epi::Raw;
            be.out = out;
            if (o.spmv == MLEM_SPMV_CSR_VECTOR) prepare_kernel(m, o);
            project(m, true, r, be, o, {}, s);
        } else {
            MLEM_CUDA(cudaMemsetAsync(out, 0, sizeof(float) * m->A.ncols, s));
            const int sl = scatter_lanes(m);  // sets m->scatter_unroll on the first call
            launch_scatter(m->A, r, out, sl, m->scatter_unroll, {}, s);
        }
        if (perm) cols_out(m, bp_dev, out, s);
    });
}

mlem_status mlem_merge_path_search(const uint64_t* rowptr_dev, uint32_t rows, uint64_t nnz, uint32_t secsize,
                                   uint64_t nthreads, int64_t* i_out_dev, int64_t* j_out_dev, void* stream) {
    return guarded([&] {
        MLEM_REQUIRE(rowptr_dev && i_out_dev && j_out_dev, MLEM_EINVAL, "NULL argument");
        MLEM_REQUIRE(secsize >= 1, MLEM_EINVAL, "secsize must be > 0");
        launch_merge_search_ref(rowptr_dev, rows, nnz, secsize, nthreads, i_out_dev, j_out_dev,
                                static_cast<cudaStream_t>(stream));
    });
}

mlem_status mlem_transpose_host(const mlem_csr_host* csr, uint64_t* colptr, uint32_t* rowidx, float* val) {
    return guarded([&] {
        MLEM_REQUIRE(colptr && (csr == nullptr || csr->nnz == 0 || (rowidx && val)), MLEM_EINVAL, "NULL argument");
        check_host_csr(csr);
        DeviceGuard dg(0);
        cudaStream_t s = nullptr;
        MLEM_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
        DevCsr A, T;
        try {
            upload_csr(csr, A, s);
            transpose_device(A, T, s);
            MLEM_CUDA(cudaStreamSynchronize(s));
            MLEM_CUDA(cudaMemcpy(colptr, T.rowptr, sizeof(uint64_t) * ((uint64_t)T.nrows + 1), cudaMemcpyDeviceToHost));
            if (T.nnz) {
                MLEM_CUDA(cudaMemcpy(rowidx, T.idx, sizeof(uint32_t) * T.nnz, cudaMemcpyDeviceToHost));
                MLEM_CUDA(cudaMemcpy(val, T.val, sizeof(float) * T.nnz, cudaMemcpyDeviceToHost));
            }
        } catch (...) {
            free_csr(A);
            free_csr(T);
            cudaStreamDestroy(s);
            throw;
        }
        free_csr(A);
        free_csr(T);
        cudaStreamDestroy(s);
    });
}

mlem_status mlem_column_sums_host(const mlem_csr_host* csr, float* norm_out) {
    return guarded([&] {
        MLEM_REQUIRE(norm_out, MLEM_EINVAL, "NULL argument");
        check_host_csr(csr);
        DeviceGuard dg(0);
        cudaStream_t s = nullptr;
        MLEM_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
        DevCsr A, T;
        float* n = nullptr;
        try {
            upload_csr(csr, A, s);
            transpose_device(A, T, s);
            MLEM_CUDA(cudaMalloc(&n, sizeof(float) * csr->cols));
            colsum_from_transpose(T, n, s);
            MLEM_CUDA(cudaStreamSynchronize(s));
            MLEM_CUDA(cudaMemcpy(norm_out, n, sizeof(float) * csr->cols, cudaMemcpyDeviceToHost));
        } catch (...) {
            cudaFree(n);
            free_csr(A);
            free_csr(T);
            cudaStreamDestroy(s);
            throw;
        }
        cudaFree(n);
        free_csr(A);
        free_csr(T);
        cudaStreamDestroy(s);
    });
}

mlem_status mlem_partition_rows(const uint64_t* rowptr, uint64_t nnz, uint32_t rows, uint32_t nseg,
                                uint32_t* segments, uint32_t* seg_rows, uint32_t* seg_nnz, uint64_t* offsets) {
    return guarded([&] {
        MLEM_REQUIRE(rowptr && segments && seg_rows && seg_nnz && offsets, MLEM_EINVAL, "NULL argument");
        MLEM_REQUIRE(nseg >= 1, MLEM_EINVAL, "nseg must be > 0");
        // partitionMatrix (main.cu:593-611): segment s starts at the first row
        // whose start offset reaches s * nnz / nseg
        segments[0] = 0;
        segments[nseg] = rows;
        uint32_t i = 0;
        const double per = (double)nnz / (double)nseg;
        for (uint32_t sgm = 0; sgm < nseg; ++sgm) {
            for (; i <= rows; ++i)
                if ((double)rowptr[i] >= per * sgm) break;
            segments[sgm] = i;
        }
        for (uint32_t sgm = 0; sgm < nseg; ++sgm) {
            seg_rows[sgm] = segments[sgm + 1] - segments[sgm];
            seg_nnz[sgm] = (uint32_t)(rowptr[segments[sgm + 1]] - rowptr[segments[sgm]]);
            offsets[sgm] = rowptr[segments[sgm]];
        }
    });
}

mlem_status mlem_reconstruct(const uint64_t* csr_rows, const uint32_t* csr_cols, const float* csr_vals,
                             const uint64_t* csr_rows_trans, const uint32_t* csr_cols_trans,
                             const float* csr_vals_trans, const int32_t* g, const float* norm, const float* f,
                             float* result_f, uint32_t rows, uint32_t cols, uint64_t nnzs, uint32_t iterations,
                             uint32_t device_numbers, uint32_t matrix_vector_mul, uint32_t secsize_fp,
                             uint32_t secsize_bp, uint32_t using_trans) {
    return guarded([&] {
        MLEM_REQUIRE(device_numbers >= 1, MLEM_EINVAL, "device_numbers must be > 0");
        MLEM_REQUIRE(device_numbers == 1, MLEM_EUNSUPPORTED,
                     "one GPU per process: run independent replicas instead of device_numbers > 1");
        MLEM_REQUIRE(using_trans <= 1 && matrix_vector_mul <= 1, MLEM_EINVAL, "switches must be 0 or 1");
        MLEM_REQUIRE(g && f && result_f && norm, MLEM_EINVAL, "NULL argument");
        mlem_csr_host c{rows, cols, nnzs, csr_rows, csr_cols, csr_vals};
        mlem_matrix_opts mo;
        mlem_matrix_opts_default(&mo);
        mo.norm = norm;
        const bool host_t = using_trans == 0 && csr_rows_trans && (nnzs == 0 || (csr_cols_trans && csr_vals_trans));
        mo.build_transpose = (using_trans == 0 && !host_t) ? 1 : 0;
        mlem_matrix* m = nullptr;
        mlem_status st = mlem_matrix_create(&c, &mo, &m);
        if (st != MLEM_OK) fail(st, get_error());
        try {
            if (host_t) {
                // the caller supplied Aᵀ (as main.cu:100-105 does): upload it as is
                DeviceGuard dg(m->device);
                mlem_csr_host t{cols, rows, nnzs, csr_rows_trans, csr_cols_trans, csr_vals_trans};
                check_host_csr(&t);
                upload_csr(&t, m->AT, m->stream);
                m->AT.max_row = max_row_length(m->AT.rowptr, m->AT.nrows, m->stream);
                m->has_t = true;
            }
            mlem_run_opts o;
            mlem_run_opts_default(&o);
            o.spmv = matrix_vector_mul ? MLEM_SPMV_CSR_VECTOR : MLEM_SPMV_MERGE;
            o.bp_mode = using_trans ? MLEM_BP_SCATTER : MLEM_BP_TRANS;
            o.secsize_fp = secsize_fp;
            o.secsize_bp = secsize_bp;
            st = mlem_run(m, g, f, iterations, &o, result_f, nullptr, nullptr);
            if (st != MLEM_OK) fail(st, get_error());
        } catch (...) {
            destroy_matrix(m);
            throw;
        }
        destroy_matrix(m);
    });
}

}  // extern "C"
