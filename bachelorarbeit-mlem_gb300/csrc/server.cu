// server.cu — batched reconstruction (many sinograms, one resident matrix)
// and the continuous-batching request server.
//
// Batched form: instances are packed into tiles of BT slots (interleaved
// image/ratio state, per-slot iteration counters on the device).  One
// iteration of a tile = batched FP, batched BP + update, counter tick; it is
// captured as a CUDA graph per projection width and replayed; a slot whose
// instance is done takes the next instance between two iterations.  The
// projections cover only the leading slots that still run (width
// 4/8/16/32), so a pool that is emptying, or a server matrix with few
// requests in flight, costs less per iteration.  BT is picked by timing
// 8/16/32 on the matrix (autotuner).
//
// Server: one worker thread owns per-matrix slot states; every matrix runs on
// its own stream and advances independently: when one of its iterations
// completes (event query), finished slots hand their images back, queued
// requests are admitted into free slots (a matrix's slot state is allocated
// on first use if it fits the HBM budget) and its next iteration is launched.
// Kernels of different matrices overlap on the GPU, and a small matrix is
// not paced by a large one.  A request's arithmetic depends on neither its
// slot, the tile size nor the width, so its result is the same alone and in
// a mix.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <numeric>
#include <thread>
#include <unordered_map>

#include "runtime.h"

namespace mlem {

void enqueue_batch_iteration(mlem_matrix* m, BatchState& b, cudaStream_t s, uint32_t active) {
    const BatchArgs a = b.args(m->has_t ? active : 0);  // the scatter form covers the whole tile
    launch_batch_fp(m->A, a, {}, s);
    if (m->has_t) {
        launch_batch_bp_update(m->AT, m->norm, a, {}, s);
    } else {
        launch_batch_scatter(m->A, a, b.bp, s);
        launch_batch_update_zero(m->norm, m->A.ncols, a, b.bp, s);
    }
    launch_batch_tick(a, s);
}

void batch_put_slot(const mlem_matrix* m, BatchState& b, uint32_t slot, const int32_t* g_dev, float init,
                    const float* f0_dev, uint32_t iters, cudaStream_t s) {
    launch_slot_put(b.g, b.f, m->A.nrows, m->A.ncols, b.tile, slot, g_dev, init, f0_dev, b.remaining, iters,
                    m->lor_of, m->vox_of, s);
}

void batch_get_slot(const mlem_matrix* m, const BatchState& b, uint32_t slot, float* f_dev, cudaStream_t s) {
    launch_slot_get(b.f, m->A.ncols, b.tile, slot, f_dev, m->vox_of, s);
}

static uint64_t batch_state_bytes(uint32_t rows, uint32_t cols, uint32_t tile, bool scatter) {
    const uint64_t R = std::max<uint32_t>(rows, 1), C = std::max<uint32_t>(cols, 1);
    return 8ull * R * tile + 4ull * C * tile * (scatter ? 2 : 1) + 4 * R + 4 * C + 192;
}

// Persistent launches of a device never run at the same time: a cooperative
// launch fills the GPU, and two of them partly resident could wait on each
// other's blocks.  mlem_batch_run holds this lock for the whole run when it
// uses the persistent form.
static std::mutex& persistent_lock(int dev) {
    static std::mutex mu;
    static std::map<int, std::unique_ptr<std::mutex>> locks;
    std::lock_guard<std::mutex> lk(mu);
    auto& p = locks[dev];
    if (!p) p.reset(new std::mutex());
    return *p;
}

// Reads and clears the error word of the persistent form (after the stream
// has drained).
static void check_persistent(const BatchState& b, cudaStream_t s) {
    int e = 0;
    MLEM_CUDA(cudaMemcpyAsync(&e, b.err, sizeof(int), cudaMemcpyDeviceToHost, s));
    MLEM_CUDA(cudaStreamSynchronize(s));
    if (e) {
        MLEM_CUDA(cudaMemsetAsync(b.err, 0, sizeof(int), s));
        fail(MLEM_ETIMEOUT, "persistent batch kernel: a grid barrier wait ran out");
    }
}

// Replays one iteration of the tile as a CUDA graph (one per projection
// width, captured on first use).  active: slots 0..active-1 may have
// iterations left; the projections cover the smallest width holding them.
static void batch_step(mlem_matrix* m, BatchState& b, cudaStream_t s, bool use_graph, uint32_t active) {
    if (!use_graph) {
        enqueue_batch_iteration(m, b, s, active);
        return;
    }
    const uint32_t w = m->has_t ? batch_width(b.tile, active) : b.tile;  // the scatter form covers the tile
    const int gi = w == 4 ? 0 : w == 8 ? 1 : w == 16 ? 2 : 3;
    if (!b.graph[gi]) {
        cudaStream_t cs = nullptr;
        MLEM_CUDA(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
        cudaGraph_t graph = nullptr;
        const uint64_t l0 = g_launches.load();
        MLEM_CUDA(cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal));
        try {
            enqueue_batch_iteration(m, b, cs, w);
        } catch (...) {
            cudaStreamEndCapture(cs, &graph);
            if (graph) cudaGraphDestroy(graph);
            cudaStreamDestroy(cs);
            throw;
        }
        MLEM_CUDA(cudaStreamEndCapture(cs, &graph));
        b.graph_nodes[gi] = g_launches.load() - l0;
        g_launches.fetch_sub(b.graph_nodes[gi]);
        const cudaError_t e = cudaGraphInstantiate(&b.graph[gi], graph, 0);
        cudaGraphDestroy(graph);
        cudaStreamDestroy(cs);
        MLEM_CUDA(e);
    }
    MLEM_CUDA(cudaGraphLaunch(b.graph[gi], s));
    count_launch(b.graph_nodes[gi]);
}

// Picks the batch tile with the highest images*iterations per second.
static uint32_t autotune_tile(mlem_matrix* m, cudaStream_t s) {
    if (m->batch_tile) return m->batch_tile;
    const uint32_t rows = m->A.nrows, cols = m->A.ncols;
    uint32_t best = 16;
    double best_rate = -1.0;
    cudaEvent_t e0, e1;
    MLEM_CUDA(cudaEventCreate(&e0));
    MLEM_CUDA(cudaEventCreate(&e1));
    for (uint32_t bt : {8u, 16u, 32u}) {
        BatchState b;
        try {
            b.alloc(rows, cols, bt, !m->has_t);
        } catch (const Error&) {
            b.release();
            cudaGetLastError();
            continue;
        }
        // representative data (image 1, counts 1) with every slot idle
        // (remaining = 0): the kernels run in full and f is left as is
        std::vector<float> ones((uint64_t)std::max(cols, 1u) * bt, 1.0f);
        std::vector<int32_t> cnt((uint64_t)std::max(rows, 1u) * bt, 1);
        MLEM_CUDA(cudaMemcpyAsync(b.f, ones.data(), sizeof(float) * ones.size(), cudaMemcpyHostToDevice, s));
        MLEM_CUDA(cudaMemcpyAsync(b.g, cnt.data(), sizeof(int32_t) * cnt.size(), cudaMemcpyHostToDevice, s));
        enqueue_batch_iteration(m, b, s, bt);  // warm-up
        MLEM_CUDA(cudaEventRecord(e0, s));
        for (int q = 0; q < 3; ++q) enqueue_batch_iteration(m, b, s, bt);
        MLEM_CUDA(cudaEventRecord(e1, s));
        MLEM_CUDA(cudaEventSynchronize(e1));
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        const double rate = bt / std::max(1e-6, (double)ms);
        if (rate > best_rate) {
            best_rate = rate;
            best = bt;
        }
        MLEM_CUDA(cudaStreamSynchronize(s));
        b.release();
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    m->batch_tile = best;
    return best;
}

// Picks the faster form at the matrix's tile: per-iteration launches or the
// persistent loop (same data as autotune_tile, every slot idle).
static uint32_t autotune_form(mlem_matrix* m, uint32_t tile, cudaStream_t s) {
    if (m->batch_form) return m->batch_form;
    if (!m->has_t) return m->batch_form = 1;  // the persistent form needs Aᵀ
    const uint32_t rows = m->A.nrows, cols = m->A.ncols;
    BatchState b;
    cudaEvent_t e[3] = {};
    float ms_graph = 0.f, ms_loop = 0.f;
    try {
        b.alloc(rows, cols, tile, false);
        std::vector<float> ones((uint64_t)std::max(cols, 1u) * tile, 1.0f);
        std::vector<int32_t> cnt((uint64_t)std::max(rows, 1u) * tile, 1);
        MLEM_CUDA(cudaMemcpyAsync(b.f, ones.data(), sizeof(float) * ones.size(), cudaMemcpyHostToDevice, s));
        MLEM_CUDA(cudaMemcpyAsync(b.g, cnt.data(), sizeof(int32_t) * cnt.size(), cudaMemcpyHostToDevice, s));
        for (auto& ev : e) MLEM_CUDA(cudaEventCreate(&ev));
        std::lock_guard<std::mutex> lk(persistent_lock(m->device));
        enqueue_batch_iteration(m, b, s, tile);
        launch_batch_loop(m->A, m->AT, m->norm, b.args(tile), 1, b.bar, b.err, s);  // warm-up
        MLEM_CUDA(cudaEventRecord(e[0], s));
        for (int q = 0; q < 3; ++q) enqueue_batch_iteration(m, b, s, tile);
        MLEM_CUDA(cudaEventRecord(e[1], s));
        launch_batch_loop(m->A, m->AT, m->norm, b.args(tile), 3, b.bar, b.err, s);
        MLEM_CUDA(cudaEventRecord(e[2], s));
        MLEM_CUDA(cudaEventSynchronize(e[2]));
        cudaEventElapsedTime(&ms_graph, e[0], e[1]);
        cudaEventElapsedTime(&ms_loop, e[1], e[2]);
        check_persistent(b, s);
    } catch (...) {
        cudaStreamSynchronize(s);
        for (auto& ev : e)
            if (ev) cudaEventDestroy(ev);
        b.release();
        throw;
    }
    for (auto& ev : e) cudaEventDestroy(ev);
    b.release();
    m->batch_form = ms_loop < ms_graph ? 2 : 1;
    return m->batch_form;
}

}  // namespace mlem

using namespace mlem;

// ------------------------------------------------------------------ server
namespace {

enum class ReqState { Queued, Running, Finishing, Done, Cancelled };

// Page-locked host buffers of one size (a sinogram or an image of one
// matrix), handed out to requests and returned when a request is done with
// them.  At most `cap` buffers exist; beyond that requests use pageable
// memory.  Guarded by the server mutex.
struct PinnedPool {
    size_t bytes = 0;
    uint32_t cap = 0, made = 0;
    std::vector<void*> free_list, all;
    // a free buffer, or nullptr with `make` set when the caller should
    // allocate a new one (outside the lock), or nullptr when the pool is full
    void* take(bool& make) {
        make = false;
        if (!free_list.empty()) {
            void* p = free_list.back();
            free_list.pop_back();
            return p;
        }
        if (made < cap) {
            ++made;
            make = true;
        }
        return nullptr;
    }
    void give(void* p) {
        if (p) free_list.push_back(p);
    }
    void release() {
        for (void* p : all) cudaFreeHost(p);
        all.clear();
        free_list.clear();
        made = 0;
    }
};

struct Request {
    uint64_t id = 0;
    uint32_t mid = 0;
    std::vector<int32_t> g;       // the sinogram when no pinned buffer was free
    int32_t* pin_g = nullptr;     // the sinogram in a pinned buffer of the matrix's pool
    float init = 0.f;             // reference initial value, computed at submit
    uint32_t iters = 0;
    std::chrono::steady_clock::time_point t_submit, t_done;
    ReqState state = ReqState::Queued;
    std::vector<float> result;    // the image when no pinned buffer was free
    float* pin_f = nullptr;       // the image in a pinned buffer (copy in flight while Finishing)
    cudaEvent_t copied = nullptr; // recorded after the image's device-to-host copy
};

struct MatrixSlots {
    mlem_matrix* m = nullptr;
    BatchState bs;
    bool allocated = false;
    cudaStream_t stream = nullptr;
    cudaEvent_t done = nullptr;       // recorded after each enqueued iteration
    bool inflight = false;            // an iteration is running on `stream`
    std::vector<uint64_t> slot_req;   // 0 = free
    std::vector<uint32_t> slot_left;
    uint32_t tile = 0;
    PinnedPool pin_g, pin_f;          // staging of sinograms in and images out
    bool active() const { return active_slots() > 0; }
    // one past the highest occupied slot
    uint32_t active_slots() const {
        for (uint32_t b = (uint32_t)slot_req.size(); b > 0; --b)
            if (slot_req[b - 1]) return b;
        return 0;
    }
};

}  // namespace

struct mlem_server {
    mlem_server_opts opts{};
    int device = 0;
    std::vector<MatrixSlots> mats;
    std::deque<uint64_t> queue;
    std::unordered_map<uint64_t, Request> reqs;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::thread worker;
    bool stop = false;
    bool started = false;
    uint64_t next_id = 1;
    uint64_t budget = 0, in_use = 0;
    mlem_server_stats st{};
    std::string worker_error;
    std::vector<uint64_t> finishing;    // requests whose image copy is in flight
    std::vector<cudaEvent_t> spare_events;

    void run();
    bool admit_locked();
    void finish_locked();
};

// Requests whose image copy to pinned memory has completed become Done.
void mlem_server::finish_locked() {
    for (size_t k = 0; k < finishing.size();) {
        Request& r = reqs[finishing[k]];
        const cudaError_t q = cudaEventQuery(r.copied);
        if (q == cudaErrorNotReady) {
            ++k;
            continue;
        }
        MLEM_CUDA(q);
        spare_events.push_back(r.copied);
        r.copied = nullptr;
        r.t_done = std::chrono::steady_clock::now();
        r.state = ReqState::Done;
        ++st.completed;
        finishing[k] = finishing.back();
        finishing.pop_back();
        cv_done.notify_all();
    }
}

bool mlem_server::admit_locked() {
    bool any = false;
    for (auto it = queue.begin(); it != queue.end();) {
        Request& r = reqs[*it];
        MatrixSlots& ms = mats[r.mid];
        const uint32_t rows = ms.m->A.nrows, cols = ms.m->A.ncols;
        if (ms.inflight) {  // its slots are being read by a running iteration
            ++it;
            continue;
        }
        if (!ms.allocated) {
            const uint64_t need = batch_state_bytes(rows, cols, ms.tile, !ms.m->has_t);
            if (in_use + need > budget) {
                // release the state of idle matrices, then retry once
                for (auto& o : mats)
                    if (o.allocated && !o.inflight && !o.active()) {
                        cudaStreamSynchronize(o.stream);
                        in_use -= o.bs.bytes;
                        o.bs.release();
                        o.allocated = false;
                    }
                if (in_use + need > budget) {
                    ++it;
                    continue;
                }
            }
            ms.bs.alloc(rows, cols, ms.tile, !ms.m->has_t);
            ms.allocated = true;
            in_use += ms.bs.bytes;
        }
        int slot = -1;
        for (uint32_t b = 0; b < ms.tile; ++b)
            if (ms.slot_req[b] == 0) {
                slot = (int)b;
                break;
            }
        if (slot < 0) {
            ++it;
            continue;
        }
        // Stream order makes the staging safe without waiting: the next
        // admission's copy into stage_g runs after this slot's put kernel.
        // A pinned sinogram is copied asynchronously; a pageable one is
        // consumed before cudaMemcpyAsync returns.
        MLEM_CUDA(cudaMemcpyAsync(ms.bs.stage_g, r.pin_g ? (const void*)r.pin_g : (const void*)r.g.data(),
                                  sizeof(int32_t) * rows, cudaMemcpyHostToDevice, ms.stream));
        batch_put_slot(ms.m, ms.bs, (uint32_t)slot, ms.bs.stage_g, r.init, nullptr, r.iters, ms.stream);
        ms.slot_req[slot] = r.id;
        ms.slot_left[slot] = r.iters;
        r.state = ReqState::Running;
        ++st.active;
        --st.queued;
        it = queue.erase(it);
        any = true;
    }
    return any;
}

void mlem_server::run() {
    DeviceGuard dg(device);
    // Each matrix advances on its own stream: as soon as one of its iterations
    // completes (event), finished slots are handed back, queued requests are
    // admitted into free slots and its next iteration is launched.  Small
    // matrices therefore iterate at their own pace next to large ones.
    while (true) {
        bool any_inflight = false;
        {
            std::unique_lock<std::mutex> lk(mu);
            if (stop) break;
            // 1. completions
            for (auto& ms : mats) {
                if (!ms.inflight) continue;
                const cudaError_t q = cudaEventQuery(ms.done);
                if (q == cudaErrorNotReady) continue;
                MLEM_CUDA(q);
                ms.inflight = false;
                const uint32_t cols = ms.m->A.ncols;
                for (uint32_t b = 0; b < ms.tile; ++b) {
                    if (ms.slot_req[b] == 0) continue;
                    ++st.iterations_done;
                    if (--ms.slot_left[b] > 0) continue;
                    Request& r = reqs[ms.slot_req[b]];
                    // the sinogram's copy completed before this iteration ran
                    ms.pin_g.give(r.pin_g);
                    r.pin_g = nullptr;
                    batch_get_slot(ms.m, ms.bs, b, ms.bs.stage_f, ms.stream);
                    bool make = false;
                    r.pin_f = static_cast<float*>(ms.pin_f.take(make));
                    if (make) {
                        void* p = nullptr;
                        if (cudaHostAlloc(&p, ms.pin_f.bytes, cudaHostAllocPortable) == cudaSuccess) {
                            ms.pin_f.all.push_back(p);
                            r.pin_f = static_cast<float*>(p);
                        } else {
                            cudaGetLastError();
                            --ms.pin_f.made;
                        }
                    }
                    if (r.pin_f) {
                        // asynchronous: the request is Done once the copy's event fires
                        MLEM_CUDA(cudaMemcpyAsync(r.pin_f, ms.bs.stage_f, sizeof(float) * cols,
                                                  cudaMemcpyDeviceToHost, ms.stream));
                        if (spare_events.empty()) {
                            cudaEvent_t e = nullptr;
                            MLEM_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
                            spare_events.push_back(e);
                        }
                        r.copied = spare_events.back();
                        spare_events.pop_back();
                        MLEM_CUDA(cudaEventRecord(r.copied, ms.stream));
                        r.state = ReqState::Finishing;
                        finishing.push_back(r.id);
                    } else {
                        r.result.resize(cols);
                        MLEM_CUDA(cudaMemcpyAsync(r.result.data(), ms.bs.stage_f, sizeof(float) * cols,
                                                  cudaMemcpyDeviceToHost, ms.stream));
                        MLEM_CUDA(cudaStreamSynchronize(ms.stream));
                        r.t_done = std::chrono::steady_clock::now();
                        r.state = ReqState::Done;
                        ++st.completed;
                        cv_done.notify_all();
                    }
                    ms.slot_req[b] = 0;
                    --st.active;
                }
            }
            finish_locked();
            // 2. admissions into free slots of idle matrices
            admit_locked();
            // 3. next iteration of every idle matrix with work
            for (auto& ms : mats) {
                if (!ms.inflight && ms.active()) {
                    batch_step(ms.m, ms.bs, ms.stream, true, ms.active_slots());
                    MLEM_CUDA(cudaEventRecord(ms.done, ms.stream));
                    ms.inflight = true;
                }
                any_inflight |= ms.inflight;
            }
            any_inflight |= !finishing.empty();
            if (!any_inflight) {
                cv_work.wait_for(lk, std::chrono::milliseconds(20));
                continue;
            }
        }
        std::this_thread::sleep_for(std::chrono::microseconds(20));
    }
}

extern "C" {

void mlem_batch_opts_default(mlem_batch_opts* o) {
    if (!o) return;
    o->tile = 0;
    o->use_graph = 1;
    o->order_by_iterations = 1;
    o->form = 0;
}

mlem_status mlem_batch_run(mlem_matrix* m, uint32_t count, const int32_t* g, const uint32_t* iterations,
                           const float* f0, const mlem_batch_opts* opts, float* f_out, mlem_stats* stats) {
    return guarded([&] {
        const auto t0 = std::chrono::steady_clock::now();
        MLEM_REQUIRE(m && g && iterations && f_out, MLEM_EINVAL, "NULL argument");
        mlem_batch_opts o;
        mlem_batch_opts_default(&o);
        if (opts) o = *opts;
        MLEM_REQUIRE(o.tile == 0 || o.tile == 8 || o.tile == 16 || o.tile == 32, MLEM_EINVAL,
                     "batch tile must be 0 (autotune), 8, 16 or 32");
        MLEM_REQUIRE(o.form <= 2, MLEM_EINVAL, "batch form must be 0 (autotune), 1 (graphs) or 2 (persistent)");
        MLEM_REQUIRE(o.form != 2 || m->has_t, MLEM_EINVAL, "the persistent batch form needs the transpose");
        std::lock_guard<std::mutex> lk(m->mu);
        DeviceGuard dg(m->device);
        cudaStream_t s = m->stream;
        const uint32_t rows = m->A.nrows, cols = m->A.ncols;
        const uint32_t tile = o.tile ? o.tile : autotune_tile(m, s);
        const bool persistent = (o.form ? o.form : autotune_form(m, tile, s)) == 2;
        std::unique_lock<std::mutex> plk(persistent_lock(m->device), std::defer_lock);
        if (persistent) plk.lock();
        std::vector<uint32_t> order(count);
        std::iota(order.begin(), order.end(), 0u);
        if (o.order_by_iterations)
            std::stable_sort(order.begin(), order.end(),
                             [&](uint32_t a, uint32_t b) { return iterations[a] > iterations[b]; });
        BatchState bs;
        bs.alloc(rows, cols, tile, !m->has_t);
        uint64_t h2d = 0, d2h = 0, iters_total = 0;
        cudaEvent_t e0 = nullptr, e1 = nullptr;
        double dev_seconds = 0.0;
        const uint64_t l0 = g_launches.load();
        // The tile's slots form a pool: the instances enter in `order`
        // (longest first when ordered), and a slot whose instance has run its
        // iterations hands the image back and takes the next instance before
        // the following iteration, so the pool stays full until the last
        // instances.  The host knows when every slot finishes (the counts are
        // fixed), so the refills are simply enqueued between iterations.
        std::vector<int64_t> slot_inst(tile, -1);
        std::vector<uint64_t> slot_end(tile, 0);
        uint32_t next = 0;
        uint64_t step = 0;
        // Sinograms in and images out pass through a small ring of pinned host
        // buffers, so a refill never waits for the GPU to drain (a pageable
        // copy would): buffer j is reused once its previous copy has completed.
        constexpr uint32_t kRing = 4;
        int32_t* pin_g = nullptr;
        float* pin_f = nullptr;
        cudaEvent_t ev_g[kRing] = {}, ev_f[kRing] = {};
        float* pending_f[kRing] = {};
        uint32_t ring_g = 0, ring_f = 0;
        const bool pinned =
            cudaHostAlloc((void**)&pin_g, sizeof(int32_t) * std::max<uint64_t>(rows, 1) * kRing, cudaHostAllocDefault) ==
                cudaSuccess &&
            cudaHostAlloc((void**)&pin_f, sizeof(float) * std::max<uint64_t>(cols, 1) * kRing, cudaHostAllocDefault) ==
                cudaSuccess;
        if (!pinned) cudaGetLastError();  // fall back to pageable copies
        auto drain_f = [&](uint32_t j) {  // completes the image copy held by ring buffer j
            if (!pending_f[j]) return;
            MLEM_CUDA(cudaEventSynchronize(ev_f[j]));
            std::memcpy(pending_f[j], pin_f + (uint64_t)j * cols, sizeof(float) * cols);
            pending_f[j] = nullptr;
        };
        auto admit = [&](uint32_t b) {
            const uint32_t i = order[next++];
            const int32_t* gi = g + (uint64_t)i * rows;
            if (pinned) {
                const uint32_t j = ring_g++ % kRing;
                if (ev_g[j]) MLEM_CUDA(cudaEventSynchronize(ev_g[j]));
                else MLEM_CUDA(cudaEventCreateWithFlags(&ev_g[j], cudaEventDisableTiming));
                int32_t* hb = pin_g + (uint64_t)j * rows;
                std::memcpy(hb, gi, sizeof(int32_t) * rows);
                MLEM_CUDA(cudaMemcpyAsync(bs.stage_g, hb, sizeof(int32_t) * rows, cudaMemcpyHostToDevice, s));
                MLEM_CUDA(cudaEventRecord(ev_g[j], s));
            } else {
                MLEM_CUDA(cudaMemcpyAsync(bs.stage_g, gi, sizeof(int32_t) * rows, cudaMemcpyHostToDevice, s));
            }
            h2d += sizeof(int32_t) * (uint64_t)rows;
            const float* f0d = nullptr;
            float init = 0.f;
            if (f0) {
                MLEM_CUDA(cudaMemcpyAsync(bs.stage_f, f0 + (uint64_t)i * cols, sizeof(float) * cols,
                                          cudaMemcpyHostToDevice, s));
                h2d += sizeof(float) * (uint64_t)cols;
                f0d = bs.stage_f;
            } else {
                init = reference_initial_value(m, gi);
            }
            batch_put_slot(m, bs, b, bs.stage_g, init, f0d, iterations[i], s);
            iters_total += iterations[i];
            slot_inst[b] = i;
            slot_end[b] = step + iterations[i];
        };
        auto hand_back = [&](uint32_t b) {
            const uint32_t i = (uint32_t)slot_inst[b];
            batch_get_slot(m, bs, b, bs.stage_f, s);
            if (pinned) {
                const uint32_t j = ring_f++ % kRing;
                if (ev_f[j]) drain_f(j);
                else MLEM_CUDA(cudaEventCreateWithFlags(&ev_f[j], cudaEventDisableTiming));
                MLEM_CUDA(cudaMemcpyAsync(pin_f + (uint64_t)j * cols, bs.stage_f, sizeof(float) * cols,
                                          cudaMemcpyDeviceToHost, s));
                MLEM_CUDA(cudaEventRecord(ev_f[j], s));
                pending_f[j] = f_out + (uint64_t)i * cols;
            } else {
                MLEM_CUDA(cudaMemcpyAsync(f_out + (uint64_t)i * cols, bs.stage_f, sizeof(float) * cols,
                                          cudaMemcpyDeviceToHost, s));
            }
            d2h += sizeof(float) * (uint64_t)cols;
            slot_inst[b] = -1;
        };
        auto release_ring = [&] {
            for (uint32_t j = 0; j < kRing; ++j) {
                if (ev_g[j]) cudaEventDestroy(ev_g[j]);
                if (ev_f[j]) cudaEventDestroy(ev_f[j]);
            }
            if (pin_g) cudaFreeHost(pin_g);
            if (pin_f) cudaFreeHost(pin_f);
        };
        try {
            MLEM_CUDA(cudaEventCreate(&e0));
            MLEM_CUDA(cudaEventCreate(&e1));
            MLEM_CUDA(cudaMemsetAsync(bs.remaining, 0, sizeof(uint32_t) * 32, s));
            // zero-iteration instances are their initial image
            for (uint32_t b = 0; b < tile && next < count; ++b) {
                admit(b);
                while (slot_end[b] == step) {
                    hand_back(b);
                    if (next == count) break;
                    admit(b);
                }
            }
            MLEM_CUDA(cudaEventRecord(e0, s));
            while (true) {
                uint32_t act = 0;
                for (uint32_t b = 0; b < tile; ++b)
                    if (slot_inst[b] >= 0) act = b + 1;
                if (act == 0) break;
                if (persistent) {
                    // every iteration up to the next slot refill in one launch
                    uint64_t n = ~0ull;
                    for (uint32_t b = 0; b < act; ++b)
                        if (slot_inst[b] >= 0) n = std::min(n, slot_end[b] - step);
                    launch_batch_loop(m->A, m->AT, m->norm, bs.args(act), (uint32_t)n, bs.bar, bs.err, s);
                    step += n;
                } else {
                    batch_step(m, bs, s, o.use_graph != 0, act);
                    ++step;
                }
                for (uint32_t b = 0; b < act; ++b) {
                    while (slot_inst[b] >= 0 && slot_end[b] == step) {
                        hand_back(b);
                        if (next < count) admit(b);
                    }
                }
            }
            MLEM_CUDA(cudaEventRecord(e1, s));
            MLEM_CUDA(cudaStreamSynchronize(s));
            if (persistent) check_persistent(bs, s);
            for (uint32_t j = 0; j < kRing; ++j) drain_f(j);
            float ms = 0.f;
            cudaEventElapsedTime(&ms, e0, e1);
            dev_seconds = ms * 1e-3;
        } catch (...) {
            cudaStreamSynchronize(s);
            release_ring();
            bs.release();
            if (e0) cudaEventDestroy(e0);
            if (e1) cudaEventDestroy(e1);
            throw;
        }
        release_ring();
        bs.release();
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        if (stats) {
            stats->seconds_total = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
            stats->seconds_iterations = dev_seconds;
            stats->iterations = (uint32_t)std::min<uint64_t>(iters_total, 0xffffffffu);
            stats->kernel_launches = (uint32_t)(g_launches.load() - l0);
            stats->bytes_h2d = h2d;
            stats->bytes_d2h = d2h;
            stats->loglik_last = std::nan("");
            stats->fp_ms = stats->bp_ms = std::nan("");
        }
    });
}

void mlem_server_opts_default(mlem_server_opts* o) {
    if (!o) return;
    o->slots_per_matrix = 0;
    o->hbm_budget_bytes = 0;
    o->hbm_reserve_bytes = 2ull << 30;
    o->queue_capacity = 4096;
    o->stream_priority = 1;
}

mlem_status mlem_server_create(const mlem_server_opts* opts, mlem_server** out) {
    return guarded([&] {
        MLEM_REQUIRE(out, MLEM_EINVAL, "NULL argument");
        *out = nullptr;
        auto* s = new mlem_server();
        mlem_server_opts_default(&s->opts);
        if (opts) s->opts = *opts;
        if (!(s->opts.slots_per_matrix == 0 || s->opts.slots_per_matrix == 8 || s->opts.slots_per_matrix == 16 ||
              s->opts.slots_per_matrix == 32)) {
            delete s;
            fail(MLEM_EINVAL, "slots_per_matrix must be 0 (autotuned), 8, 16 or 32");
        }
        if (s->opts.stream_priority > 2) {
            delete s;
            fail(MLEM_EINVAL, "stream_priority must be 0, 1 or 2");
        }
        cudaGetDevice(&s->device);
        if (s->opts.hbm_budget_bytes) {
            s->budget = s->opts.hbm_budget_bytes;
        } else {
            size_t fr = 0, tot = 0;
            MLEM_CUDA(cudaMemGetInfo(&fr, &tot));
            s->budget = fr > s->opts.hbm_reserve_bytes ? fr - s->opts.hbm_reserve_bytes : 0;
        }
        *out = s;
    });
}

mlem_status mlem_server_add_matrix(mlem_server* s, mlem_matrix* m, uint32_t* matrix_id) {
    return guarded([&] {
        MLEM_REQUIRE(s && m && matrix_id, MLEM_EINVAL, "NULL argument");
        std::lock_guard<std::mutex> lk(s->mu);
        MLEM_REQUIRE(!s->started, MLEM_EBUSY, "add matrices before the first submit");
        MLEM_REQUIRE(s->mats.empty() || m->device == s->device, MLEM_EINVAL, "all matrices must share a device");
        s->device = m->device;
        MatrixSlots ms;
        ms.m = m;
        DeviceGuard dg(m->device);
        // slots per matrix: fixed by the options, or the batch tile the
        // autotuner finds best for this matrix (the image tile of a large
        // matrix should stay L2-resident)
        ms.tile = s->opts.slots_per_matrix ? s->opts.slots_per_matrix : autotune_tile(m, m->stream);
        ms.slot_req.assign(ms.tile, 0);
        ms.slot_left.assign(ms.tile, 0);
        // pinned staging for up to two slot-fulls of sinograms and images
        ms.pin_g.bytes = sizeof(int32_t) * (size_t)std::max<uint32_t>(m->A.nrows, 1);
        ms.pin_f.bytes = sizeof(float) * (size_t)std::max<uint32_t>(m->A.ncols, 1);
        ms.pin_g.cap = ms.pin_f.cap = 2 * ms.tile;
        // smaller matrices can get higher stream priority, so their short
        // iterations are scheduled ahead of the CTAs of large ones.  The
        // default raises only small matrices: a matrix with requests in flight
        // runs its iterations back to back, so a mid-size matrix ranked above a
        // large one takes most of the GPU while few of its slots are occupied,
        // and the large matrix's requests pile up (3-matrix Poisson mix: p99
        // 5.8 s with three levels, 2.5 s with small-first-then-equal)
        int least = 0, greatest = 0;
        MLEM_CUDA(cudaDeviceGetStreamPriorityRange(&least, &greatest));
        int prio = least;
        const uint32_t pol = s->opts.stream_priority;
        if (pol != 2 && m->A.nnz < (16ull << 20)) prio = greatest;
        else if (pol == 0 && m->A.nnz < (512ull << 20)) prio = (least + greatest) / 2;
        MLEM_CUDA(cudaStreamCreateWithPriority(&ms.stream, cudaStreamNonBlocking, prio));
        MLEM_CUDA(cudaEventCreateWithFlags(&ms.done, cudaEventDisableTiming));
        s->mats.push_back(std::move(ms));
        *matrix_id = (uint32_t)(s->mats.size() - 1);
    });
}

mlem_status mlem_server_submit(mlem_server* s, uint32_t matrix_id, const int32_t* g, uint32_t iterations,
                               uint64_t* request_id) {
    return guarded([&] {
        const auto t_submit = std::chrono::steady_clock::now();
        MLEM_REQUIRE(s && g && request_id, MLEM_EINVAL, "NULL argument");
        MLEM_REQUIRE(iterations > 0, MLEM_EINVAL, "iterations must be > 0");
        uint32_t rows = 0;
        const mlem_matrix* mat = nullptr;
        int32_t* pin = nullptr;
        bool make = false;
        {
            std::lock_guard<std::mutex> lk(s->mu);
            MLEM_REQUIRE(matrix_id < s->mats.size(), MLEM_EINVAL, "unknown matrix id");
            if (!s->worker_error.empty()) fail(MLEM_ECUDA, "server worker stopped: " + s->worker_error);
            if (s->queue.size() >= s->opts.queue_capacity) {
                ++s->st.rejected;
                fail(MLEM_EBUSY, "server queue full");
            }
            MatrixSlots& ms = s->mats[matrix_id];
            mat = ms.m;
            rows = ms.m->A.nrows;
            pin = static_cast<int32_t*>(ms.pin_g.take(make));
        }
        // Outside the lock, so the worker keeps running: the sinogram goes to
        // a pinned buffer of the matrix (an asynchronous copy at admission) or,
        // when the pool is used up, to pageable memory; its sum gives the
        // reference initial value.
        Request r;
        if (make) {
            DeviceGuard dg(s->device);
            void* p = nullptr;
            if (cudaHostAlloc(&p, sizeof(int32_t) * (size_t)rows, cudaHostAllocPortable) == cudaSuccess)
                pin = static_cast<int32_t*>(p);
            else
                cudaGetLastError();
        }
        if (pin) std::memcpy(pin, g, sizeof(int32_t) * (size_t)rows);
        else r.g.assign(g, g + rows);
        r.pin_g = pin;
        r.init = reference_initial_value(mat, g);
        r.mid = matrix_id;
        r.iters = iterations;
        r.t_submit = t_submit;
        std::lock_guard<std::mutex> lk(s->mu);
        MatrixSlots& ms = s->mats[matrix_id];
        if (make) {
            if (pin) ms.pin_g.all.push_back(pin);
            else --ms.pin_g.made;
        }
        r.id = s->next_id++;
        *request_id = r.id;
        s->queue.push_back(r.id);
        s->reqs.emplace(r.id, std::move(r));
        ++s->st.submitted;
        ++s->st.queued;
        if (!s->started) {
            s->started = true;
            s->worker = std::thread([s] {
                try {
                    s->run();
                } catch (const Error& e) {
                    std::lock_guard<std::mutex> l2(s->mu);
                    s->worker_error = e.msg;
                    s->cv_done.notify_all();
                }
            });
        }
        s->cv_work.notify_one();
    });
}

mlem_status mlem_server_wait(mlem_server* s, uint64_t request_id, float* f_out, uint32_t timeout_ms,
                             double* latency_s) {
    return guarded([&] {
        MLEM_REQUIRE(s, MLEM_EINVAL, "NULL argument");
        std::unique_lock<std::mutex> lk(s->mu);
        auto it = s->reqs.find(request_id);
        MLEM_REQUIRE(it != s->reqs.end(), MLEM_EINVAL, "unknown request id");
        const bool ok = s->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), [&] {
            auto jt = s->reqs.find(request_id);
            return jt->second.state == ReqState::Done || jt->second.state == ReqState::Cancelled ||
                   !s->worker_error.empty();
        });
        Request& r = s->reqs.find(request_id)->second;
        if (r.state == ReqState::Cancelled) {
            s->reqs.erase(request_id);
            fail(MLEM_EINVAL, "request was cancelled");
        }
        if (r.state != ReqState::Done) {
            if (!s->worker_error.empty()) fail(MLEM_ECUDA, "server worker stopped: " + s->worker_error);
            MLEM_REQUIRE(ok, MLEM_ETIMEOUT, "request not finished within the timeout");
        }
        if (latency_s) *latency_s = std::chrono::duration<double>(r.t_done - r.t_submit).count();
        const uint32_t mid = r.mid;
        const size_t cols = s->mats[mid].m->A.ncols;
        float* pin = r.pin_f;
        std::vector<float> result = std::move(r.result);
        s->reqs.erase(request_id);
        // the image leaves the pinned buffer outside the lock
        lk.unlock();
        if (f_out) std::memcpy(f_out, pin ? pin : result.data(), sizeof(float) * cols);
        if (pin) {
            lk.lock();
            s->mats[mid].pin_f.give(pin);
        }
    });
}

mlem_status mlem_server_cancel(mlem_server* s, uint64_t request_id) {
    return guarded([&] {
        MLEM_REQUIRE(s, MLEM_EINVAL, "NULL argument");
        std::lock_guard<std::mutex> lk(s->mu);
        auto it = s->reqs.find(request_id);
        MLEM_REQUIRE(it != s->reqs.end(), MLEM_EINVAL, "unknown request id");
        MLEM_REQUIRE(it->second.state == ReqState::Queued, MLEM_EINVAL, "request is not queued");
        s->queue.erase(std::remove(s->queue.begin(), s->queue.end(), request_id), s->queue.end());
        s->mats[it->second.mid].pin_g.give(it->second.pin_g);
        it->second.pin_g = nullptr;
        it->second.state = ReqState::Cancelled;
        --s->st.queued;
        ++s->st.cancelled;
        s->cv_done.notify_all();
    });
}

mlem_status mlem_server_get_stats(mlem_server* s, mlem_server_stats* st) {
    return guarded([&] {
        MLEM_REQUIRE(s && st, MLEM_EINVAL, "NULL argument");
        std::lock_guard<std::mutex> lk(s->mu);
        *st = s->st;
        st->hbm_in_use = s->in_use;
    });
}

mlem_status mlem_server_destroy(mlem_server* s) {
    return guarded([&] {
        if (!s) return;
        {
            std::lock_guard<std::mutex> lk(s->mu);
            s->stop = true;
        }
        s->cv_work.notify_all();
        if (s->worker.joinable()) s->worker.join();
        DeviceGuard dg(s->device);
        for (auto& ms : s->mats) {
            if (ms.stream) cudaStreamSynchronize(ms.stream);
            ms.bs.release();
            ms.pin_g.release();
            ms.pin_f.release();
            if (ms.done) cudaEventDestroy(ms.done);
            if (ms.stream) cudaStreamDestroy(ms.stream);
        }
        for (auto& kv : s->reqs)
            if (kv.second.copied) cudaEventDestroy(kv.second.copied);
        for (cudaEvent_t e : s->spare_events) cudaEventDestroy(e);
        delete s;
    });
}

}  // extern "C"
