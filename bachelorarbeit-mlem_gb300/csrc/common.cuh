// common.cuh — error handling, launch accounting and small device helpers
// shared by every translation unit of the library.
#pragma once

#include <cuda_runtime.h>
#include <cuda_fp16.h>
#include <cuda_bf16.h>
#include <stdint.h>
#include <atomic>
#include <string>

#include "../../include/mlem.h"

namespace mlem {

// ------------------------------------------------------------ error state
void set_error(const std::string& msg);
const char* get_error();

struct Error {
    mlem_status code;
    std::string msg;
};

// Throwing helpers used inside the C++ runtime; every extern "C" entry point
// catches and converts to an mlem_status.
[[noreturn]] void fail(mlem_status code, const std::string& msg);

#define MLEM_CUDA(expr)                                                              \
    do {                                                                             \
        cudaError_t e_ = (expr);                                                     \
        if (e_ != cudaSuccess)                                                       \
            ::mlem::fail(e_ == cudaErrorMemoryAllocation ? MLEM_ENOMEM : MLEM_ECUDA, \
                         std::string(#expr) + ": " + cudaGetErrorString(e_));        \
    } while (0)

#define MLEM_REQUIRE(cond, code, msg)          \
    do {                                       \
        if (!(cond)) ::mlem::fail(code, msg);  \
    } while (0)

// Kernel launch accounting (reported as gpu_launches by the benchmark).
extern std::atomic<uint64_t> g_launches;
inline void count_launch(uint64_t n = 1) { g_launches.fetch_add(n, std::memory_order_relaxed); }

// Checks the launch that was just issued.
#define MLEM_LAUNCHED()                       \
    do {                                      \
        ::mlem::count_launch();               \
        MLEM_CUDA(cudaGetLastError());        \
    } while (0)

inline unsigned int ceil_div_u(uint64_t a, uint64_t b) { return (unsigned int)((a + b - 1) / b); }

// ------------------------------------------------------------ device helpers
// Loads of the matrix stream (column indices, values, delta words), in two
// policies chosen per kernel family by measurement on the GB300:
//   ld_stream  evict-first streaming loads (ld.global.cs): the merge-path,
//              D16, interleaved and batched kernels (on the 12 GB-class and
//              3-D mid matrices the cached path cost them 1-14%);
//   ld_cached  the read-only path, cached in L1 (ld.global.nc): the row
//              kernels of spmv.cu (csr-vector projections, scatter, fused
//              pass) and the symmetric kernels.  A row's head and tail vectors
//              are shared with its neighbours, which L1 then serves, and the
//              gathered vector stays in L2 through the access-policy window;
//              on the 12 GB-class matrix: transposed iteration 3.6% and fused
//              pass 6% faster, symmetric kernels 2%.
template <typename T>
__device__ __forceinline__ T ld_stream(const T* p) { return __ldcs(p); }
template <typename T>
__device__ __forceinline__ T ld_cached(const T* p) { return __ldg(p); }
__device__ __forceinline__ uint4 ld_stream_u4(const uint4* p) { return __ldcs(p); }
__device__ __forceinline__ uint2 ld_stream_u2(const uint2* p) { return __ldcs(p); }
__device__ __forceinline__ float4 ld_stream_f4(const float4* p) { return __ldcs(p); }

__device__ __forceinline__ uint64_t globaltimer_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned* p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// Grid-wide barrier of a cooperative launch: barrier k of the launch is
// passed once `count` (zeroed before the launch) reaches k * gridDim.x.  Every
// wait is bounded: after kBarrierWaitNs, or as soon as another block has given
// up, the block sets *err and the caller returns, so a failure ends the launch
// with an error flag the host reads instead of a hang.
constexpr uint64_t kBarrierWaitNs = 2000000000ull;  // 2 s; a phase takes milliseconds

__device__ __forceinline__ bool grid_barrier(unsigned* count, unsigned k, int* err) {
    __shared__ int s_ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        atomicAdd(count, 1u);
        const unsigned target = k * gridDim.x;
        const uint64_t t0 = globaltimer_ns();
        int ok = 1;
        while (ld_acquire_u32(count) < target) {
            if (*(volatile int*)err != 0 || globaltimer_ns() - t0 > kBarrierWaitNs) {
                atomicExch(err, 1);
                ok = 0;
                break;
            }
            __nanosleep(64);
        }
        __threadfence();
        s_ok = ok;
    }
    __syncthreads();
    return s_ok != 0;
}

// Value storage types: load 4 consecutive values (element index 4*v .. 4*v+3).
template <typename V>
struct Val4;

template <>
struct Val4<float> {
    static __device__ __forceinline__ void load(const float* p, uint64_t v, float out[4]) {
        float4 t = ld_stream_f4(reinterpret_cast<const float4*>(p) + v);
        out[0] = t.x; out[1] = t.y; out[2] = t.z; out[3] = t.w;
    }
    static __device__ __forceinline__ void load_cached(const float* p, uint64_t v, float out[4]) {
        float4 t = ld_cached(reinterpret_cast<const float4*>(p) + v);
        out[0] = t.x; out[1] = t.y; out[2] = t.z; out[3] = t.w;
    }
    static __device__ __forceinline__ float one(const float* p, uint64_t e) { return __ldcs(p + e); }
    static __device__ __forceinline__ float one_cached(const float* p, uint64_t e) { return __ldg(p + e); }
};

template <>
struct Val4<__half> {
    static __device__ __forceinline__ void load_cached(const __half* p, uint64_t v, float out[4]) {
        uint2 t = ld_cached(reinterpret_cast<const uint2*>(p) + v);
        __half2 a = *reinterpret_cast<__half2*>(&t.x);
        __half2 b = *reinterpret_cast<__half2*>(&t.y);
        float2 fa = __half22float2(a), fb = __half22float2(b);
        out[0] = fa.x; out[1] = fa.y; out[2] = fb.x; out[3] = fb.y;
    }
    static __device__ __forceinline__ void load(const __half* p, uint64_t v, float out[4]) {
        uint2 t = ld_stream_u2(reinterpret_cast<const uint2*>(p) + v);
        __half2 a = *reinterpret_cast<__half2*>(&t.x);
        __half2 b = *reinterpret_cast<__half2*>(&t.y);
        float2 fa = __half22float2(a), fb = __half22float2(b);
        out[0] = fa.x; out[1] = fa.y; out[2] = fb.x; out[3] = fb.y;
    }
    static __device__ __forceinline__ float one(const __half* p, uint64_t e) {
        return __half2float(p[e]);
    }
    static __device__ __forceinline__ float one_cached(const __half* p, uint64_t e) {
        return __half2float(__ldg(p + e));
    }
};

template <>
struct Val4<__nv_bfloat16> {
    static __device__ __forceinline__ void load_cached(const __nv_bfloat16* p, uint64_t v, float out[4]) {
        uint2 t = ld_cached(reinterpret_cast<const uint2*>(p) + v);
        __nv_bfloat162 a = *reinterpret_cast<__nv_bfloat162*>(&t.x);
        __nv_bfloat162 b = *reinterpret_cast<__nv_bfloat162*>(&t.y);
        float2 fa = __bfloat1622float2(a), fb = __bfloat1622float2(b);
        out[0] = fa.x; out[1] = fa.y; out[2] = fb.x; out[3] = fb.y;
    }
    static __device__ __forceinline__ void load(const __nv_bfloat16* p, uint64_t v, float out[4]) {
        uint2 t = ld_stream_u2(reinterpret_cast<const uint2*>(p) + v);
        __nv_bfloat162 a = *reinterpret_cast<__nv_bfloat162*>(&t.x);
        __nv_bfloat162 b = *reinterpret_cast<__nv_bfloat162*>(&t.y);
        float2 fa = __bfloat1622float2(a), fb = __bfloat1622float2(b);
        out[0] = fa.x; out[1] = fa.y; out[2] = fb.x; out[3] = fb.y;
    }
    static __device__ __forceinline__ float one(const __nv_bfloat16* p, uint64_t e) {
        return __bfloat162float(p[e]);
    }
    static __device__ __forceinline__ float one_cached(const __nv_bfloat16* p, uint64_t e) {
        return __bfloat162float(__ldg(p + e));
    }
};

// Elements of the col/val arrays are padded on the device to a multiple of
// this count (zeros), so vector loads never leave the allocation.
constexpr uint64_t kPad = 8;
inline uint64_t padded(uint64_t n) { return (n + kPad - 1) / kPad * kPad; }

inline size_t val_bytes(mlem_value_type t) { return t == MLEM_VAL_F32 ? 4 : 2; }

// Device CSR view (rows of A, or rows of Aᵀ = columns of A).
struct DevCsr {
    uint32_t nrows = 0;       // number of rows of this operand
    uint32_t ncols = 0;       // length of the vector it multiplies
    uint64_t nnz = 0;
    uint64_t* rowptr = nullptr;  // u64[nrows+1]
    uint32_t* idx = nullptr;     // u32[padded(nnz)]
    void* val = nullptr;         // f32/f16/bf16 [padded(nnz)]
    mlem_value_type vt = MLEM_VAL_F32;
    uint32_t max_row = 0;        // longest row
    // optional delta-coded copy (spmv_d16.cu): rows of 8-entry vectors
    uint64_t* dvptr = nullptr;   // [nrows+1] first vector of each row
    uint32_t* dbase = nullptr;   // [nrows] first column of each row
    uint16_t* d16 = nullptr;     // [8 dvec] column deltas (dummies and padding included)
    void* dval = nullptr;        // [8 dvec] values at the same positions
    uint64_t dvec = 0;           // vectors
    int d16_lanes = 0;           // lanes per row the D16 layout is built for (4 or 8)
    // optional processing order of the rows (locality of the gathers); the
    // k-th row group handles row order[k].  Results are written per row.
    uint32_t* order = nullptr;   // [nrows]
    // optional lane-interleaved copy (spmv_ilv.cu)
    uint32_t* idx_ilv = nullptr; // [ilv_len]
    void* val_ilv = nullptr;     // [ilv_len]
    uint64_t ilv_len = 0;
};

}  // namespace mlem
