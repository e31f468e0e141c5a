// Internal interfaces between the C ABI layer (capi.cu) and the kernel translation units.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <atomic>
#include <string>
#include <vector>

#include "pqcgpu.h"

namespace pqc {
// dynamic shared memory a CTA may opt into on sm_103a (227 KB)
constexpr size_t MAX_SMEM_PER_CTA = 232448;

// Kernel launches issued by this library (all contexts); contexts report deltas.
extern std::atomic<uint64_t> g_launch_count;

// A launch shape -- a count (instances or row parts per CTA) and a thread count -- published as
// one 32-bit atomic word: a launch that reads it while pqcgpu_set_launch_shape changes it on
// another host thread sees the old pair or the new one, never half of each.  Shapes are
// process-wide: every context and device launches with them.
struct LaunchShape {
    std::atomic<uint32_t> w;
    constexpr LaunchShape(int count, int threads) : w(((uint32_t)count << 16) | (uint32_t)threads) {}
    void set(int count, int threads) { w.store(((uint32_t)count << 16) | (uint32_t)threads, std::memory_order_relaxed); }
    void get(int &count, int &threads) const {
        const uint32_t v = w.load(std::memory_order_relaxed);
        count = (int)(v >> 16);
        threads = (int)(v & 0xffffu);
    }
};

// Launch profiler (probe.cu): CUDA events around each launch on its stream when enabled.
// Set while a CUDA graph is being captured on this host thread: launch helpers then skip the
// profiler and attribute calls (both were done by the uncaptured warm-up pass).
void set_capturing(bool on);
bool capturing();
bool prof_enabled();
void *prof_begin(cudaStream_t st, const char *name, int k, int v);
void prof_end(cudaStream_t st, void *tok);
void prof_enable(bool on);
std::string prof_read();
bool prof_trace(char *buf, size_t cap, size_t *need);
int probe_peaks(int device, double *int_ops, double *keccak_perms);

// Every kernel launch of the library goes through this macro: counted, and timed when profiling.
#define PQC_LAUNCH(st, name, k, v, ...)                                      \
    do {                                                                     \
        void *pqc_tok_ = ::pqc::prof_enabled() ? ::pqc::prof_begin(st, name, k, v) : nullptr; \
        __VA_ARGS__;                                                         \
        if (pqc_tok_) ::pqc::prof_end(st, pqc_tok_);                         \
        ::pqc::g_launch_count++;                                             \
    } while (0)

// One device KEM operation (capi.cu): op 0 keypair (in0 coins -> out0 pk, out1 sk), 1 encaps (in0 pk,
// in1 coins -> out0 ct, out1 ss), 2 decaps (in0 ct, in1 sk -> out0 ss); device pointers.  flags:
// OP_PLAIN = Kyber's reference-style chain; OP_NH_BATCHED = NewHope on its batched kernels at every
// batch size (the serving loop: under concurrent load, the single-instance kernels' 512-thread CTAs
// raised the p99 latency of the FrodoKEM requests beside them).
constexpr int OP_PLAIN = 1, OP_NH_BATCHED = 2;
int op_dev(int alg, int op, int n, const uint8_t *in0, const uint8_t *in1, uint8_t *out0, uint8_t *out1,
           uint8_t *scr, int flags, cudaStream_t s);
size_t op_scratch_bytes(int alg, int op, int plain);
void op_io_sizes(int alg, int op, size_t sz[4]);

// Once-per-device set-up (constant tables) and the thread-local error text (capi.cu).
int device_ready(int device);
int set_error(int code, const char *what);

// A second stream of the calling host thread on the current device, for work of one call that may
// overlap the rest of the call: forked from and joined back into the call's stream with its events
// (stream capture follows them).  nullptr when it cannot be created (e.g. during a capture that
// forbids it): the caller then stays on its own stream.
struct SideStream {
    cudaStream_t s = nullptr;
    cudaEvent_t fork = nullptr, join = nullptr;
};
SideStream *side_stream();

// ---- Kyber (kyber.cu) ----
int kyber_init_constants();
// op: 0 keypair, 1 enc, 2 dec.  ni = instances per CTA of the core kernel, threads per CTA.
int kyber_set_shape(int op, int k, int ni, int threads);
// Launch bounds (threads per CTA, CTAs per SM) of the Kyber core kernels of op 1 (encapsulation),
// 2 (decapsulation's re-encryption stage, and CPA decryption) and 3 (decryption stage); op 0
// (keypair) is bounded by threads only.  The bound caps the registers ptxas may allocate
// (65536 / (threads x CTAs)) and so steers how it schedules the Keccak and basemul code: these
// pairs were the fastest measured on GB300 at 65536 instances (Kyber-768 re-encryption without the
// KDF: 1.079 ms at (256, 2), 104 registers, against 1.094 ms at (192, 3), 88 registers; the
// encapsulation kernel at (192, 3): 1.082 against 1.066 ms).  Shapes with more threads are refused.
constexpr int kyber_bound_threads(int op, int /*k*/) { return op == 1 ? 256 : op == 2 ? 256 : op == 3 ? 384 : 512; }
constexpr int kyber_bound_ctas(int op, int /*k*/) { return op == 1 ? 2 : op == 2 ? 2 : op == 3 ? 2 : 1; }
int kyber_get_shape(int op, int k, int *ni, int *threads);
// Scratch bytes per instance (op 0 keypair, 1 enc, 2 dec; plain = the per-stage baseline path).
size_t kyber_scratch_bytes(int k, int op, int plain);
// coins: d (CPA) or d||z (KEM) at `coins_stride`.  kem=1 writes the full KEM secret key.
// AES-256 CTR_DRBG without derivation function (SP 800-90A 10.2.1), as in the NIST KAT generator (kat.cu)
struct CtrDrbg {
    uint8_t key[32], v[16];
    uint64_t reseed_counter = 0;
    void instantiate(const uint8_t entropy[48], const uint8_t *personalization);
    void generate(uint8_t *out, size_t n);
    void update(const uint8_t *provided);
};
// One Kyber job of a mixed batch (round-3 arithmetic, k = 2, 3, 4; kem 1 FO or 2 ML-KEM), device
// pointers as in op_dev; scratch per kyber_scratch_bytes.  With PQCGPU_STAGE_KERNELS the core
// stages of all such jobs run as two persistent waves (kyber_mixed.cu): wave 0 holds every
// keypair core, encapsulation core and decryption stage, wave 1 every re-encryption stage; each
// job's serial hash kernels run around them through kyber_mixed_hash: phase 0 before wave 0
// (G(d) / H(pk), G / H(c)), phase 1 between the waves (decapsulation's G), phase 2 after its last
// wave (H(pk) into sk / the KDF).
struct MixedKyberJob {
    int k, kem, n;
    const uint8_t *in0, *in1;
    uint8_t *out0, *out1, *scratch;
};
constexpr int MIXED_COUNTER_WORDS = 8;  // zeroable device words a mixed batch gives its Kyber waves
constexpr int MIXED_NH_COUNTER_WORDS = 4;  // and its NewHope wave (after those 8)
int kyber_mixed_hash(int op, int phase, const MixedKyberJob &job, cudaStream_t st);
int kyber_mixed_wave(int wave, const std::vector<MixedKyberJob> (&jobs)[3], unsigned *counters, cudaStream_t st);
int kyber_mixed_init();  // constant tables of kyber_mixed.cu
int kyber_kem_mode(int alg);  // 1: round-2 / round-3 FO KEM, 2: ML-KEM (FIPS 203)
int kyber_keypair_dev(int variant, int k, int n, uint8_t *pk, uint8_t *sk, const uint8_t *coins, int coins_stride,
                      int kem, uint8_t *scratch, int plain, cudaStream_t st);
// kem=1: coins 32 B/instance, m ignored.  kem=0: CPA enc with m, coins.
int kyber_enc_dev(int variant, int k, int n, uint8_t *ct, uint8_t *ss, const uint8_t *pk, const uint8_t *m,
                  const uint8_t *coins, uint8_t *scratch, int kem, int plain, cudaStream_t st);
// kem=1: out = ss.  kem=0: out = m (CPA decryption).
int kyber_dec_dev(int variant, int k, int n, uint8_t *out, const uint8_t *ct, const uint8_t *sk, uint8_t *scratch,
                  int kem, int plain, cudaStream_t st);

// ---- NewHope-1024 and NewHope-512 (newhope.cu); N = 1024 or 512 coefficients ----
int newhope_init_constants();
int newhope_set_shape(int N, int op, int ni, int threads);
int newhope_get_shape(int N, int op, int *ni, int *threads);
// single_ok = false: the batched kernels even for batches that the single-instance kernels would take
int newhope_keypair_dev(int N, int n, uint8_t *pk, uint8_t *sk, const uint8_t *seed, int seed_stride, cudaStream_t st,
                        bool single_ok = true);
// kem=1: coins 32 B/instance, scratch >= 64 B/instance, ss written; kem=0: CPA with m and coins
int newhope_enc_dev(int N, int n, uint8_t *ct, uint8_t *ss, const uint8_t *pk, const uint8_t *m, const uint8_t *coins,
                    uint8_t *scratch, int kem, cudaStream_t st, bool single_ok = true);
// kem=1: out = ss (32 B); kem=0: out = message
int newhope_dec_dev(int N, int n, uint8_t *out, const uint8_t *ct, const uint8_t *sk, int kem, cudaStream_t st);
// One NewHope CPA-KEM job of a mixed batch (device pointers as in op_dev; scratch 64 B per instance
// for encapsulation).  With PQCGPU_STAGE_KERNELS their core kernels run as one persistent wave
// (newhope_mixed_wave), after each encapsulation job's prologue (newhope_mixed_pre).
struct NhMixedJob {
    int N, op, n;
    const uint8_t *in0, *in1;
    uint8_t *out0, *out1, *scratch;
};
int newhope_mixed_pre(const NhMixedJob &j, cudaStream_t st);
int newhope_mixed_wave(const std::vector<NhMixedJob> &jobs, unsigned *counters, int ncounters, cudaStream_t st);

// ---- FrodoKEM-640 / 976 / 1344 (frodo.cu); N = 640, 976 or 1344 ----
int frodo_init_constants();
// The FrodoKEM jobs of a mixed batch with PQCGPU_STAGE_KERNELS: each job's serial sponges run as
// its own kernels before (frodo_mixed_pre) and after (frodo_mixed_post) one persistent wave that
// holds the products of every job (frodo_mixed_wave: key generation rows of B = AS + E, and
// B' = S'A + E' of encapsulation and decapsulation).  kpc: keypair coins per instance.
struct FrMixedJob {
    int N, op, n, kpc;
    const uint8_t *in0, *in1;
    uint8_t *out0, *out1, *scratch;
};
constexpr int MIXED_FR_COUNTER_WORDS = 16;  // zeroable device words of the FrodoKEM waves (after the NewHope words)
int frodo_mixed_pre(const FrMixedJob &j, cudaStream_t st);
int frodo_mixed_wave(const std::vector<FrMixedJob> &jobs, unsigned *counters, int ncounters, cudaStream_t st);
int frodo_mixed_post(const FrMixedJob &j, cudaStream_t st);
size_t frodo_scratch_bytes(int N);  // per instance, all three operations
int frodo_keypair_dev(int N, int n, uint8_t *pk, uint8_t *sk, const uint8_t *coins, int cstride, uint8_t *scratch,
                      cudaStream_t st);
// pkh: optional SHAKE(pk, ss bytes) per instance (ss-size stride), e.g. from a resident secret key
int frodo_enc_dev(int N, int n, uint8_t *ct, uint8_t *ss, const uint8_t *pk, const uint8_t *mu, uint8_t *scratch,
                  cudaStream_t st, const uint8_t *pkh = nullptr);
int frodo_dec_dev(int N, int n, uint8_t *ss, const uint8_t *ct, const uint8_t *sk, uint8_t *scratch, cudaStream_t st);
// FrodoKEM parameter n of an algorithm id, 0 if it is not FrodoKEM
int frodo_n(int alg);
int frodo_set_shape(int op, int parts, int threads);
int frodo_get_shape(int op, int *parts, int *threads);
// Many encapsulations to one public key (A generated once, one matrix product for the batch).
// product: 1 CUDA cores, 2 tensor cores (tcgen05), 0 the measured default.
int frodo_set_shared_product(int product);
int frodo_get_shared_product();
size_t frodo_shared_extra_bytes(int N);
// error: a device word that the tensor-core product sets (never clears) when one of its waits runs out
// s16: fr_tc_s_bytes(N, n) bytes of device memory for the tensor-core product's S' tiles
int frodo_enc_shared_dev(int N, int n, uint8_t *ct, uint8_t *ss, const uint8_t *pk, const uint8_t *mu, uint8_t *scratch,
                         uint8_t *extra, uint16_t *s16, unsigned *error, cudaStream_t st);
// The tensor-core product G[x] = S'[x] A (frodo_tc.cu): planes = the split A from fr_gen_a, tiled as
// below; error = a zeroed device word, set if a wait in the kernel runs out.
int frodo_shared_tc_launch(int N, int n, const uint16_t *planes, uint16_t *s16, uint8_t *scratch, unsigned *error,
                           cudaStream_t st);
// A's two fp16 planes (A & 1023, A >> 10) as the product kernel reads them: one 16 KB tile per
// (plane, 128 output columns, 64 k), each tile already in the no-swizzle K-major core-matrix layout
// of a tcgen05 operand (8 columns x 8 k = 16-byte rows of one core matrix; core matrices 128 bytes
// apart along k and 1024 bytes apart along the columns), so the kernel moves a tile with one bulk
// copy.  Entries beyond N are zero (the buffer is cleared before fr_gen_a fills it).
constexpr int FR_TC_N = 128, FR_TC_KC = 64, FR_TC_TILE = FR_TC_N * FR_TC_KC;  // tile: u16 elements
__host__ __device__ constexpr int fr_tc_ntiles(int N) { return (N + FR_TC_N - 1) / FR_TC_N; }
__host__ __device__ constexpr int fr_tc_kchunks(int N) { return (N + FR_TC_KC - 1) / FR_TC_KC; }
__host__ __device__ constexpr size_t fr_tc_planes_elems(int N) {
    return (size_t)2 * fr_tc_ntiles(N) * fr_tc_kchunks(N) * FR_TC_TILE;
}
// u16 index of plane p's entry for output column j and k
__host__ __device__ constexpr size_t fr_tc_plane_index(int N, int p, int j, int k) {
    return ((size_t)(p * fr_tc_ntiles(N) + j / FR_TC_N) * fr_tc_kchunks(N) + k / FR_TC_KC) * FR_TC_TILE +
           ((j % FR_TC_N) >> 3) * 512 + ((k % FR_TC_KC) >> 3) * 64 + (j & 7) * 8 + (k & 7);
}
// The stacked S' (8 rows per instance) as fp16 in the same tiled layout: one 16 KB tile per (16
// instances, 64 k), converted from the instances' u16 copies by fr_s16_tiles (frodo_tc.cu); entries
// beyond n or N are zero.
__host__ __device__ constexpr size_t fr_tc_s_bytes(int N, int n) {
    return (size_t)((n + 15) / 16) * fr_tc_kchunks(N) * FR_TC_TILE * 2;
}
// u16 index of S'[i][k] of instance x
__host__ __device__ constexpr size_t fr_tc_s_index(int N, int x, int i, int k) {
    return ((size_t)(x / 16) * fr_tc_kchunks(N) + k / FR_TC_KC) * FR_TC_TILE + (x % 16) * 512 +
           ((k % FR_TC_KC) >> 3) * 64 + i * 8 + (k & 7);
}

}  // namespace pqc
