// Kyber encapsulation for callers that cannot allocate device memory.
//
// Some callers of this library run where cudaMalloc is not available to them: code that executes
// inside another framework's memory pool or allocator callback, drivers and plugins that are
// handed fixed device buffers and must not grow the process's footprint, and real-time paths that
// forbid allocation after start-up.  The regular batched calls need per-call scratch (96 bytes per
// instance between the encapsulation prologue, core and epilogue kernels) from the context arena,
// which is allocated on demand.  pqcgpu_kem_enc_batch_noalloc runs the same kernels with that
// scratch taken from a fixed array in device memory instead, and calls no allocating routine.
#include <cuda_runtime.h>
#include <stdint.h>

#include <mutex>

#include "pqcgpu_internal.h"

namespace {
constexpr size_t NOALLOC_MAX_INSTANCES = 65536;
constexpr size_t NOALLOC_SCRATCH_PER_INSTANCE = 96;  // m || r || K-bar of each encapsulation
constexpr int NOALLOC_MAX_DEVICES = 64;

// 6 MiB of scratch, resident on every GPU that loads the library until the process exits.  In
// host code this name is only a host-side stand-in for the device array: the kernels receive the
// device address that cudaGetSymbolAddress returns for the current device.
static __device__ __align__(256) uint8_t g_noalloc_scratch[NOALLOC_MAX_INSTANCES * NOALLOC_SCRATCH_PER_INSTANCE];

std::mutex g_noalloc_mu;
uint8_t *g_noalloc_addr[NOALLOC_MAX_DEVICES];  // device address of the array, per device

// First call on a device: upload the constant tables and look up the array's device address,
// with that device current.  Later calls on the device reuse the address.
int noalloc_setup(int device, uint8_t **addr) {
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if (!g_noalloc_addr[device]) {
        const int rc = pqc::device_ready(device);
        if (rc) return rc;
        void *p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) return pqc::set_error(PQCGPU_ECUDA, "cudaGetSymbolAddress of the scratch array failed");
        g_noalloc_addr[device] = static_cast<uint8_t *>(p);
    }
    *addr = g_noalloc_addr[device];
    return PQCGPU_OK;
}
}  // namespace

extern "C" int pqcgpu_kem_enc_batch_noalloc(pqcgpu_alg alg, size_t n, uint8_t *ct, uint8_t *ss, const uint8_t *pk,
                                            const uint8_t *coins, void *stream) {
    int variant, k;
    switch (alg) {
    case PQCGPU_KYBER512: variant = 3; k = 2; break;
    case PQCGPU_KYBER768: variant = 3; k = 3; break;
    case PQCGPU_KYBER1024: variant = 3; k = 4; break;
    case PQCGPU_KYBER1024_R2: variant = 2; k = 4; break;
    case PQCGPU_MLKEM512: variant = 3; k = 2; break;
    case PQCGPU_MLKEM768: variant = 3; k = 3; break;
    case PQCGPU_MLKEM1024: variant = 3; k = 4; break;
    default: return pqc::set_error(PQCGPU_EUNSUPPORTED, "the no-allocation encapsulation covers the Kyber algorithms");
    }
    if (n == 0) return PQCGPU_OK;
    if (n > NOALLOC_MAX_INSTANCES)
        return pqc::set_error(PQCGPU_EINVAL, "n exceeds the 65536 instances the no-allocation scratch array holds");
    if (!ct || !ss || !pk || !coins) return pqc::set_error(PQCGPU_EINVAL, "null buffer (coins are required)");
    if (((uintptr_t)ct | (uintptr_t)ss | (uintptr_t)pk | (uintptr_t)coins) & 15)
        return pqc::set_error(PQCGPU_EINVAL, "device buffers must be 16-byte aligned");
    int device = 0;
    if (cudaGetDevice(&device) != cudaSuccess || device < 0 || device >= NOALLOC_MAX_DEVICES)
        return pqc::set_error(PQCGPU_ECUDA, "no current CUDA device");
    uint8_t *scratch = nullptr;
    int rc = noalloc_setup(device, &scratch);
    if (rc) return rc;
    rc = pqc::kyber_enc_dev(variant, k, (int)n, ct, ss, pk, nullptr, coins, scratch, pqc::kyber_kem_mode(alg), 0,
                            (cudaStream_t)stream);
    if (rc) return pqc::set_error(rc, "kernel launch failed");
    return PQCGPU_OK;
}
