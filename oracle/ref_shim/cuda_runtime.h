/* cuda_runtime.h — host emulation of the CUDA built-ins used by the
 * reference kernel.cu, so that file compiles unchanged with g++ and its
 * kernels run on the CPU (one emulated thread at a time, in an order the
 * launcher in ref_glue.cpp chooses).  Used only to build oracle/_ref. */
#ifndef REF_SHIM_CUDA_RUNTIME_H
#define REF_SHIM_CUDA_RUNTIME_H
#define __global__
#define __device__
#define __host__
#define __shared__ static
struct ref_emu_dim { unsigned int x, y, z; };
extern ref_emu_dim threadIdx, blockIdx, blockDim, gridDim;
static inline float atomicAdd(float* address, float v) {
    float old = *address;
    *address = old + v;
    return old;
}
static inline void __syncthreads(void) {}
#endif
