// Kyber dispatch on (k, variant) and the shared launch-shape table.
#include "pqcgpu_internal.h"

namespace pqc {
namespace kyber {
// Launch shape (instances per CTA, threads) of the core kernels, [op][k-2] with op 0 keypair, 1 enc,
// 2 dec (its re-encryption stage).  One thread per matrix entry (NI * k^2 jobs) sized against the shared memory each instance
// needs.  g_dec1: the decryption stage of decapsulation.  Defaults: the autotuner's GB300 optimum.
LaunchShape g_shape[3][3] = {{{16, 64}, {12, 128}, {4, 64}}, {{30, 128}, {14, 128}, {6, 96}},
                             {{30, 128}, {14, 128}, {8, 128}}};
LaunchShape g_dec1[3] = {{16, 256}, {4, 128}, {4, 128}};
// [k-2][op 0 keypair, 1 encapsulation, 2 decapsulation]: KEM batches of at most this many
// instances run on the single-instance kernels (one CTA per instance, kyber_single.cuh); larger ones
// on the batched chains.  Measured on GB300 (device buffers, median of 15, single-instance /
// batched, us): Kyber-512 single faster at every size up to 640 (encapsulation 57 / 124 at 448,
// 103 / 129 at 640); Kyber-768 encapsulation 75 / 122 at 256 but 135 / 121 at 320 (past 304 = two
// 512-thread CTAs per SM), keypair even at 320-384, decapsulation 87 / 93 at 512 and 113 / 95 at
// 640; Kyber-1024 keypair 73 / 95 at 256 but 114 / 96 at 320, encapsulation 97 / 132 and 180 /
// 133, decapsulation 103 / 107 at 384 and 103 / 89 at 448.
static constexpr int SINGLE_DEFAULT[3][3] = {{640, 640, 640}, {304, 304, 512}, {304, 304, 384}};
LaunchShape g_single[3][3] = {{{640, 0}, {640, 0}, {640, 0}}, {{304, 0}, {304, 0}, {512, 0}}, {{304, 0}, {304, 0}, {384, 0}}};
// Batches of at most this many instances run the serial hashes (H(pk), G, H(c), the KDF) with one
// warp per instance (25-lane permutation) instead of one thread.  Measured on GB300 (Kyber-768,
// device buffers, thread -> warp hash kernels): encapsulation 173 -> 139 us at 1536 instances and
// 173 -> 156 us at 2048, but 204 -> 225 us at 3072 (the warp form's ~7x issue slots then cost more
// than its shorter chain saves); the host-buffer step of 65536 pairs, whose first chunk is 2048,
// measured the same at 1024 and 2048 (3.35 ms) and slower at 4096 (3.41 ms).
LaunchShape g_warp_hash = {2048, 0};

#define PQC_KYBER_DECL(K, V)                                                                               \
    int keypair_##K##_##V(int, uint8_t *, uint8_t *, const uint8_t *, int, int, uint8_t *, int, cudaStream_t); \
    int enc_##K##_##V(int, uint8_t *, uint8_t *, const uint8_t *, const uint8_t *, const uint8_t *, uint8_t *, int, \
                      int, cudaStream_t);                                                                  \
    int dec_##K##_##V(int, uint8_t *, const uint8_t *, const uint8_t *, uint8_t *, int, int, cudaStream_t); \
    size_t smem_##K##_##V(int, int, int);                                                                \
    int init_##K##_##V();
PQC_KYBER_DECL(2, 3)
PQC_KYBER_DECL(3, 3)
PQC_KYBER_DECL(4, 3)
PQC_KYBER_DECL(2, 2)
PQC_KYBER_DECL(3, 2)
PQC_KYBER_DECL(4, 2)
}  // namespace kyber

#define PQC_KYBER_DISPATCH(FN, ...)                        \
    switch (variant * 10 + k) {                            \
    case 32: return kyber::FN##_2_3(__VA_ARGS__);          \
    case 33: return kyber::FN##_3_3(__VA_ARGS__);          \
    case 34: return kyber::FN##_4_3(__VA_ARGS__);          \
    case 22: return kyber::FN##_2_2(__VA_ARGS__);          \
    case 23: return kyber::FN##_3_2(__VA_ARGS__);          \
    case 24: return kyber::FN##_4_2(__VA_ARGS__);          \
    default: return PQCGPU_EINVAL;                         \
    }

int kyber_keypair_dev(int variant, int k, int n, uint8_t *pk, uint8_t *sk, const uint8_t *coins, int coins_stride,
                      int kem, uint8_t *scratch, int plain, cudaStream_t st) {
    PQC_KYBER_DISPATCH(keypair, n, pk, sk, coins, coins_stride, kem, scratch, plain, st)
}
int kyber_enc_dev(int variant, int k, int n, uint8_t *ct, uint8_t *ss, const uint8_t *pk, const uint8_t *m,
                  const uint8_t *coins, uint8_t *scratch, int kem, int plain, cudaStream_t st) {
    PQC_KYBER_DISPATCH(enc, n, ct, ss, pk, m, coins, scratch, kem, plain, st)
}
int kyber_dec_dev(int variant, int k, int n, uint8_t *out, const uint8_t *ct, const uint8_t *sk, uint8_t *scratch,
                  int kem, int plain, cudaStream_t st) {
    PQC_KYBER_DISPATCH(dec, n, out, ct, sk, scratch, kem, plain, st)
}
SideStream *side_stream() {
    static thread_local SideStream tbl[64];
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) {
        cudaGetLastError();
        return nullptr;
    }
    SideStream &ss = tbl[dev];
    if (!ss.s) {
        if (cudaStreamCreateWithFlags(&ss.s, cudaStreamNonBlocking) != cudaSuccess ||
            cudaEventCreateWithFlags(&ss.fork, cudaEventDisableTiming) != cudaSuccess ||
            cudaEventCreateWithFlags(&ss.join, cudaEventDisableTiming) != cudaSuccess) {
            cudaGetLastError();
            ss = SideStream{};
            return nullptr;
        }
    }
    return &ss;
}

size_t kyber_scratch_bytes(int k, int op, int plain) {
    if (plain) return (size_t)(k * k + 4 * k + 4) * 256 * 2 + 208;
    // keypair: rho || sigma (64); encaps: m || r || K-bar (96); decaps: H(c) (32) + m' r' K-bar' (96)
    return op == 1 ? 96 : (op == 2 ? 128 : 64);
}
int kyber_init_constants() {
    int (*inits[])() = {kyber::init_2_3, kyber::init_3_3, kyber::init_4_3,
                        kyber::init_2_2, kyber::init_3_2, kyber::init_4_2};
    for (auto f : inits) {
        const int rc = f();
        if (rc) return rc;
    }
    return kyber_mixed_init();
}
int kyber_set_shape(int op, int k, int ni, int threads) {
    if (op == 4) {  // the largest batch that takes the single-instance kernels, every operation of
                    // this k; 0 = never, -1 = the measured per-operation defaults
        if (k < 2 || k > 4 || ni < -1 || ni > 4096) return PQCGPU_EINVAL;
        for (int o = 0; o < 3; o++) kyber::g_single[k - 2][o].set(ni < 0 ? kyber::SINGLE_DEFAULT[k - 2][o] : ni, 0);
        return PQCGPU_OK;
    }
    if (op == 5) {  // the largest batch whose serial hashes run a warp per instance (all k); 0 = never
        if (ni < 0 || ni > 65535) return PQCGPU_EINVAL;  // a 16-bit field of the shape word
        kyber::g_warp_hash.set(ni, 0);
        return PQCGPU_OK;
    }
    if (op < 0 || op > 3 || k < 2 || k > 4 || ni <= 0 || ni > 128 || threads < 32 || threads % 32 ||
        threads > kyber_bound_threads(op, k))
        return PQCGPU_EINVAL;
    if (op == 3) {  // decapsulation, decryption stage: NI instances' polynomials, no staging
        const size_t sm1 = (k == 2 ? kyber::smem_2_3(2, ni, 0) : k == 3 ? kyber::smem_3_3(2, ni, 0) : kyber::smem_4_3(2, ni, 0));
        if (sm1 > MAX_SMEM_PER_CTA) return PQCGPU_EINVAL;
        kyber::g_dec1[k - 2].set(ni, threads);
        return PQCGPU_OK;
    }
    // the CTA's dynamic shared memory must fit the 227 KB a CTA may opt into on sm_103a
    const size_t sm = k == 2 ? kyber::smem_2_3(op, ni, threads) : k == 3 ? kyber::smem_3_3(op, ni, threads)
                                                                         : kyber::smem_4_3(op, ni, threads);
    if (sm > MAX_SMEM_PER_CTA) return PQCGPU_EINVAL;
    kyber::g_shape[op][k - 2].set(ni, threads);
    return PQCGPU_OK;
}
int kyber_get_shape(int op, int k, int *ni, int *threads) {
    if (op == 4) {  // the encapsulation's threshold of this k
        if (k < 2 || k > 4) return PQCGPU_EINVAL;
        kyber::g_single[k - 2][1].get(*ni, *threads);
        return PQCGPU_OK;
    }
    if (op == 5) {
        kyber::g_warp_hash.get(*ni, *threads);
        return PQCGPU_OK;
    }
    if (op < 0 || op > 3 || k < 2 || k > 4) return PQCGPU_EINVAL;
    if (op == 3) {
        kyber::g_dec1[k - 2].get(*ni, *threads);
        return PQCGPU_OK;
    }
    kyber::g_shape[op][k - 2].get(*ni, *threads);
    return PQCGPU_OK;
}

}  // namespace pqc
