// runtime.h — internal host-side objects behind the C ABI.
#pragma once

#include <condition_variable>
#include <functional>
#include <new>
#include <stdexcept>
#include <tuple>
#include <map>
#include <mutex>
#include <vector>

#include "kernels.cuh"

namespace mlem {

// Runs fn and converts exceptions into a status plus the thread's error text.
template <class F>
mlem_status guarded(F&& fn) {
    try {
        fn();
        return MLEM_OK;
    } catch (const Error& e) {
        set_error(e.msg);
        return e.code;
    } catch (const std::bad_alloc&) {
        set_error("host allocation failed");
        return MLEM_ENOMEM;
    } catch (const std::exception& e) {
        set_error(e.what());
        return MLEM_EINVAL;
    }
}

// Restores the caller's current device on scope exit.
struct DeviceGuard {
    int prev = -1;
    explicit DeviceGuard(int dev) {
        cudaGetDevice(&prev);
        if (prev != dev) MLEM_CUDA(cudaSetDevice(dev));
    }
    ~DeviceGuard() {
        int cur = -1;
        cudaGetDevice(&cur);
        if (prev >= 0 && cur != prev) cudaSetDevice(prev);
    }
};

struct RunKey {
    int spmv, bp, ss_fp, ss_bp, l2, chunk, pipe;
    bool operator<(const RunKey& o) const {
        return std::tie(spmv, bp, ss_fp, ss_bp, l2, chunk, pipe) <
               std::tie(o.spmv, o.bp, o.ss_fp, o.ss_bp, o.l2, o.chunk, o.pipe);
    }
};

// Per-matrix run state reused across calls (buffers and captured graphs).
struct Workspace {
    bool ready = false;
    int32_t* g = nullptr;      // [rows]
    float* f = nullptr;        // [cols]
    float* ratio = nullptr;    // [rows]
    float* bp = nullptr;       // [cols] accumulator of the scatter forms (kept zero)
    float* fwproj = nullptr;   // [rows] projection kept for the log-likelihood
    double* ll_part = nullptr; // [kLoglikParts]
    double* ll_vals = nullptr; // [ll_cap]
    uint32_t ll_cap = 0;
    uint32_t* err = nullptr;   // set by kernels whose bounded waits expired
    float* tmp_rows = nullptr; // [rows] staging in natural order (locality layout only)
    float* tmp_cols = nullptr; // [cols] staging in natural order (locality layout only)
    std::map<RunKey, cudaGraphExec_t> graphs;
    std::map<RunKey, uint64_t> graph_nodes;
    void release();
};

// Batched tile state (also the server's per-matrix slot state).
struct BatchState {
    uint32_t tile = 0;
    int32_t* g = nullptr;        // [rows][tile]
    float* f = nullptr;          // [cols][tile]
    float* ratio = nullptr;      // [rows][tile]
    float* bp = nullptr;         // [cols][tile] scatter form only
    uint32_t* remaining = nullptr;  // [tile]
    int32_t* stage_g = nullptr;  // [rows] contiguous staging
    float* stage_f = nullptr;    // [cols] contiguous staging
    unsigned* bar = nullptr;     // barrier word of the persistent form
    int* err = nullptr;          // set by the persistent form when a barrier wait ran out
    cudaGraphExec_t graph[4] = {};  // one iteration per projection width 4/8/16/32
    uint64_t graph_nodes[4] = {};
    uint64_t bytes = 0;
    void alloc(uint32_t rows, uint32_t cols, uint32_t tile, bool scatter);
    void release();
    // active: slots 0..active-1 may have iterations left (0 = all)
    BatchArgs args(uint32_t active = 0) const {
        BatchArgs a;
        a.tile = tile;
        a.active = active;
        a.g = g;
        a.f = f;
        a.ratio = ratio;
        a.remaining = remaining;
        return a;
    }
};

}  // namespace mlem

namespace mlem {
// Launch configuration of a csr-vector projection.
struct ProjCfg {
    int kind = 0;    // mlem_kernel: DIRECT, TMA, PERSISTENT, D16, ILV or SYM
    int lanes = 32;  // DIRECT: lanes per row
    int unroll = 2;  // DIRECT: 4-element vectors in flight per lane; SYM: entries in flight per lane
    float ms = 0.f;  // measured time of one launch
    bool ordered = false;    // DIRECT / PERSISTENT: rows in the operand's locality order; SYM: rows grouped by SM
    bool pipelined = false;  // DIRECT: next vectors loaded before the current gathers; SYM: next keys
};
}  // namespace mlem

struct mlem_matrix {
    int device = 0;
    mlem_value_type vt = MLEM_VAL_F32;
    mlem::DevCsr A, AT;
    bool has_t = false;
    float* norm = nullptr;
    std::vector<float> norm_host;     // host copy in natural column order (initial value)
    float norm_sum = 0.0f;            // FP32 running sum of norm_host in column order
    // Locality layout: natural row / column of each internal row / column
    // (NULL = natural order).
    mlem::SymOps sym;                 // symmetry-compressed operands (symmetry = 1)
    uint32_t* lor_of = nullptr;       // [rows]
    uint32_t* vox_of = nullptr;       // [cols]
    std::vector<uint32_t> vox_of_host;
    cudaStream_t stream = nullptr;
    mlem::Workspace ws;
    std::map<uint32_t, mlem::MergePlan> plan_A, plan_AT;
    uint32_t batch_tile = 0;          // autotuned batch tile (0 = not yet)
    uint32_t batch_form = 0;          // autotuned batch form: 1 graphs, 2 persistent (0 = not yet)
    int scatter_lanes = 0;            // autotuned lanes per row of the scatter back projection (0 = not yet)
    int scatter_unroll = 1;           // and its 16-byte vectors per lane in flight
    bool scatter_tma = false;         // the TMA-ring scatter timed faster than those lanes
    mlem::FusedPlan fused;            // chunks of the staged fused pass
    mlem::FusedForm fused_auto;       // fastest form of the fused pass (timed once; ms = 0: not yet)
    bool tuned[2] = {false, false};   // csr-vector configuration of A / Aᵀ measured
    mlem::ProjCfg proj[2];
    std::mutex mu;
    uint64_t bytes() const;
};

namespace mlem {
// Shared by the single, batched and server paths.
void ensure_workspace(mlem_matrix* m);
const MergePlan& merge_plan(mlem_matrix* m, bool transposed, uint32_t secsize);
// Form of the fused single pass for the run's options (timed once per matrix
// where the options leave it open).
FusedForm fused_form(mlem_matrix* m, const mlem_run_opts& o);
void launch_fused(mlem_matrix* m, const FusedForm& f, const float* x, const int32_t* g, float* bp, float* fwproj,
                  L2Window win, cudaStream_t s);
// CUDA events around the forward and back projection stages of eager
// iterations (mlem_run_opts.kernel_timing).
struct StageTimer {
    std::vector<cudaEvent_t> ev;  // 4 per iteration: FP start/end, BP start/end
    void record(cudaStream_t s);
    void means(double& fp_ms, double& bp_ms) const;
    ~StageTimer();
};
// sym_fused: both projections symmetry-compressed, the image orbit array
// current on entry (they exchange their outputs in orbit order)
void enqueue_iteration(mlem_matrix* m, const mlem_run_opts& o, cudaStream_t s, double* ll_slot,
                       StageTimer* timer = nullptr, bool sym_fused = false);
void enqueue_batch_iteration(mlem_matrix* m, BatchState& b, cudaStream_t s, uint32_t active);
float reference_initial_value(const mlem_matrix* m, const int32_t* g);
void check_run_opts(const mlem_matrix* m, const mlem_run_opts& o);
// Settles kernel attributes / occupancy of the selected variant (outside captures).
void prepare_kernel(mlem_matrix* m, const mlem_run_opts& o);
// Reads and clears the workspace error flag; fails with MLEM_ETIMEOUT if set.
void check_device_error(mlem_matrix* m, cudaStream_t s);
// One projection of `op` (A or Aᵀ) with the kernel the options select.
void project(mlem_matrix* m, bool transposed, const float* x, const EpiArgs& e, const mlem_run_opts& o,
             L2Window win, cudaStream_t s);
// Copies slot b of the interleaved batch state to/from contiguous device
// buffers in natural order (permuted for a matrix in the locality layout).
void batch_put_slot(const mlem_matrix* m, BatchState& b, uint32_t slot, const int32_t* g_dev, float init,
                    const float* f0_dev, uint32_t iters, cudaStream_t s);
void batch_get_slot(const mlem_matrix* m, const BatchState& b, uint32_t slot, float* f_dev, cudaStream_t s);
// A matrix whose operand A (FP32) is filled on the device by `fill` on the
// matrix stream, then validated and post-processed like mlem_matrix_create
// (transpose, value type, index copies, sensitivity image).
mlem_matrix* create_matrix_filled(const mlem_matrix_opts& o, const std::function<void(mlem_matrix*)>& fill);
}  // namespace mlem
