/*
 * Host shim that lets the reference's CUDA C device code compile as ordinary C++ so that its
 * own arithmetic can serve as a parity pin for the CPU oracle.  TEST INFRASTRUCTURE ONLY.
 *
 * Kernels run as sequential loops over virtual threads (host_launch below).  That is exact for
 * the one-thread-per-instance kernels of Kyber_GPU_Batched and NewHope_NIST_GPU, which never
 * synchronise between threads; it is not valid for kernels that rely on __syncthreads.
 */
#ifndef PQC_REF_SHIM_CUDA_RUNTIME_H
#define PQC_REF_SHIM_CUDA_RUNTIME_H
#include <stddef.h>
#include <stdint.h>
#include <stdio.h>

#define __device__
#define __global__
#define __host__
#define __constant__
#define __shared__ static
#define __forceinline__ inline

struct dim3 {
    unsigned x, y, z;
};
extern thread_local dim3 threadIdx, blockIdx, blockDim, gridDim;

typedef int cudaError_t;
typedef void *cudaStream_t;
typedef void *cudaEvent_t;
#define cudaSuccess 0
static inline const char *cudaGetErrorString(cudaError_t) { return "shim"; }

/* Evaluates the launch arguments once (the reference passes `nonce++` as an argument) and runs
 * grid x block virtual threads in order. */
template <class F, class... A>
void host_launch(unsigned grid, unsigned block, F f, A... a) {
    gridDim = {grid, 1, 1};
    blockDim = {block, 1, 1};
    for (unsigned g = 0; g < grid; g++)
        for (unsigned t = 0; t < block; t++) {
            blockIdx = {g, 0, 0};
            threadIdx = {t, 0, 0};
            f(a...);
        }
}
#endif
