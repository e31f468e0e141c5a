/*
 * Host shim for reference device code whose kernels synchronise inside a CTA -- TEST
 * INFRASTRUCTURE ONLY.  Like ref_shim/cuda_runtime.h it lets CUDA C compile as C++, but a launch
 * runs every CTA with one OS thread per CUDA thread, started together: __syncthreads() is a real
 * barrier across the CTA's threads, a thread that returns leaves the barrier, and __shared__
 * (static storage) is one array seen by all threads of the CTA.  CTAs run one after another.
 * Atomics are the host's atomics.  Memory "on the device" is host memory: cudaMemset /
 * cudaMemcpy / cudaMemcpyToSymbol are memset / memcpy.
 */
#ifndef PQC_REF_SHIM_SYNC_CUDA_RUNTIME_H
#define PQC_REF_SHIM_SYNC_CUDA_RUNTIME_H
#include <stddef.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>

#include <barrier>
#include <thread>
#include <vector>

#define __device__
#define __global__
#define __host__
#define __constant__
#define __shared__ static
#define __forceinline__ inline

struct dim3 {
    unsigned x, y, z;
    dim3(unsigned a = 1, unsigned b = 1, unsigned c = 1) : x(a), y(b), z(c) {}
};
extern thread_local dim3 threadIdx, blockIdx, blockDim, gridDim;
extern thread_local std::barrier<> *pqc_shim_cta_barrier;

typedef int cudaError_t;
typedef void *cudaStream_t;
typedef void *cudaEvent_t;
enum cudaMemcpyKind { cudaMemcpyHostToHost, cudaMemcpyHostToDevice, cudaMemcpyDeviceToHost, cudaMemcpyDeviceToDevice };
#define cudaSuccess 0
static inline const char *cudaGetErrorString(cudaError_t) { return "shim"; }
static inline cudaError_t cudaMemset(void *p, int v, size_t n) {
    memset(p, v, n);
    return cudaSuccess;
}
static inline cudaError_t cudaMemcpy(void *d, const void *s, size_t n, cudaMemcpyKind) {
    memcpy(d, s, n);
    return cudaSuccess;
}
template <class T>
cudaError_t cudaMemcpyToSymbol(T &sym, const void *s, size_t n, size_t off = 0, cudaMemcpyKind = cudaMemcpyHostToDevice) {
    memcpy(reinterpret_cast<char *>(&sym) + off, s, n);
    return cudaSuccess;
}
static inline void __syncthreads() {
    if (pqc_shim_cta_barrier) pqc_shim_cta_barrier->arrive_and_wait();
}
template <class T>
T atomicAdd(T *a, T v) {
    return __atomic_fetch_add(a, v, __ATOMIC_SEQ_CST);
}
template <class T>
T atomicSub(T *a, T v) {
    return __atomic_fetch_sub(a, v, __ATOMIC_SEQ_CST);
}

/* Evaluates the launch arguments once, then runs the grid CTA by CTA, each CTA's threads
 * concurrently. */
template <class F, class... A>
void host_launch(dim3 grid, dim3 block, F f, A... a) {
    const unsigned nthr = block.x * block.y * block.z;
    for (unsigned bz = 0; bz < grid.z; bz++)
        for (unsigned by = 0; by < grid.y; by++)
            for (unsigned bx = 0; bx < grid.x; bx++) {
                std::barrier<> bar((std::ptrdiff_t)nthr);
                std::vector<std::thread> ts;
                ts.reserve(nthr);
                for (unsigned t = 0; t < nthr; t++)
                    ts.emplace_back([&, t]() {
                        gridDim = grid;
                        blockDim = block;
                        blockIdx = dim3(bx, by, bz);
                        threadIdx = dim3(t % block.x, (t / block.x) % block.y, t / (block.x * block.y));
                        pqc_shim_cta_barrier = &bar;
                        f(a...);
                        pqc_shim_cta_barrier = nullptr;
                        bar.arrive_and_drop();
                    });
                for (auto &th : ts) th.join();
            }
}
#endif
