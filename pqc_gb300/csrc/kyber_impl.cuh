// Batched Kyber (implementation header, instantiated per (k, variant) in kyber_k*_v*.cu)
// Batched Kyber (round-3 parameter sets k = 2/3/4 and the reference's round-2 k = 4 variant) for
// sm_103a: keypair, encapsulation and decapsulation.
//
// Each operation is a short chain of kernels over the batch:
//   *_hash kernels: one thread per instance, the serial sponges (H(pk), H(c), G, KDF);
//   *_core kernels: one CTA per group of NI instances.  Inside the CTA the work of the CPA
//     scheme runs as phases separated by __syncthreads:
//       - noise (PRF + CBD), one thread per polynomial, written straight into shared memory;
//       - forward / inverse NTT, one warp per polynomial (kyber_arith.cuh);
//       - the matrix: one thread per row streams SHAKE128 blocks, rejection-samples the entries
//         and multiplies them into the accumulator as they appear, so A never exists anywhere,
//         not in HBM and not even whole in shared memory;
//       - compression / packing, one warp per instance, straight to the output bytes.
// Shared memory holds only (2K+1) (3K for keypair) polynomials per instance.
//
// Reference call stacks replaced: indcpa_keypair / indcpa_enc / indcpa_dec
// (Kyber_GPU_Batched/indcpa.cu:474-733, ~52 launches at K = 4 with every intermediate in HBM) and
// the crypto_kem_* entry points the reference declares (Kyber_GPU_Batched/api.h:18-22).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "keccak.cuh"
#include "kyber_arith.cuh"
#include "pqcgpu_internal.h"

namespace pqc {
namespace kyber {

template <int K, int V>
struct P {
    static constexpr int ETA1 = (V == 3 && K == 2) ? 3 : 2;
    static constexpr int ETA2 = 2;
    static constexpr int DU = (V == 2 || K == 4) ? 11 : 10;
    static constexpr int DV = (V == 2 || K == 4) ? 5 : 4;
    static constexpr int POLYVECBYTES = K * 384;
    static constexpr int PKB = POLYVECBYTES + 32;
    static constexpr int SKCPA = POLYVECBYTES;
    static constexpr int SKB = SKCPA + PKB + 64;
    static constexpr int CTU = K * DU * 32;
    static constexpr int CTB = CTU + DV * 32;
};

// ---------------------------------------------------------------------------------------------
// Sponge helpers on a register state
// ---------------------------------------------------------------------------------------------

// The permutation of the core kernels' PRF and matrix phases runs its round loop rolled (one round
// of code instead of two).  Those kernels carry several phases of unrolled code, and the smaller
// loop body keeps the hot code within the instruction cache: measured on GB300 (Kyber-768
// encapsulation core at 65536 instances, the same kernel otherwise), 1.039x over the two-round body,
// with ncu's no-instruction stall halved (0.18 -> 0.09 warps per issue) and the ALU pipe busy
// 71.4 % of active cycles instead of 68.3 %; a four-round body was 7 % slower.
__device__ __forceinline__ void keccak_f1600_core(uint2 (&A)[25]) { keccak_f1600_rolled(A); }

// PRF(seed, nonce) = SHAKE256(seed || nonce); `seed` 8-byte aligned (global or shared).
__device__ __forceinline__ void prf_absorb(uint2 (&A)[25], const uint2 *seed, int nonce) {
    keccak_zero(A);
#pragma unroll
    for (int i = 0; i < 4; i++) A[i] = seed[i];
    A[4].x = (uint32_t)nonce | (DOM_SHAKE << 8);
    A[SHAKE256_LANES - 1].y ^= 0x80000000u;
    keccak_f1600_core(A);
}

// CBD eta=2 from the first 128 squeezed bytes: word w (bytes 4w..4w+3) gives coefficients
// 8w..8w+7 (cbd.cu:42-63).  Calls emit(c, coeff[8]) for each group of 8.
template <class F>
__device__ __forceinline__ void cbd2_from_state(const uint2 (&A)[25], F emit) {
#pragma unroll
    for (int w = 0; w < 32; w++) {
        const uint32_t t = (w & 1) ? A[w >> 1].y : A[w >> 1].x;
        uint32_t d = t & 0x55555555u;
        d += (t >> 1) & 0x55555555u;
        int16_t c[8];
#pragma unroll
        for (int j = 0; j < 8; j++) c[j] = (int16_t)((int)((d >> (4 * j)) & 3) - (int)((d >> (4 * j + 2)) & 3));
        emit(w, c);
    }
}

// CBD eta=3 from 192 bytes spread over two squeezes (136 + 56 bytes): words wa[0..33] from the
// first state, wb[0..13] from the second.  Triplet t (bytes 3t..3t+2) gives coefficients 4t..4t+3.
template <class F>
__device__ __forceinline__ void cbd3_from_words(const uint32_t (&w)[48], F emit) {
#pragma unroll
    for (int g = 0; g < 32; g++) {  // group of 8 coefficients = 2 triplets = 6 bytes
        int16_t c[8];
#pragma unroll
        for (int h = 0; h < 2; h++) {
            const int t = 2 * g + h, o = 3 * t, wi = o >> 2, sh = 8 * (o & 3);
            uint32_t v = (sh <= 8) ? (w[wi] >> sh) : __funnelshift_r(w[wi], w[wi + 1], sh);
            v &= 0x00ffffffu;
            uint32_t d = v & 0x00249249u;
            d += (v >> 1) & 0x00249249u;
            d += (v >> 2) & 0x00249249u;
#pragma unroll
            for (int j = 0; j < 4; j++)
                c[4 * h + j] = (int16_t)((int)((d >> (6 * j)) & 7) - (int)((d >> (6 * j + 3)) & 7));
        }
        emit(g, c);
    }
}

// Noise polynomial PRF(seed, nonce) -> CBD(eta), delivered to emit(group, coeff[8]).
template <int ETA, class F>
__device__ __forceinline__ void noise_poly(const uint2 *seed, int nonce, F emit) {
    uint2 A[25];
    prf_absorb(A, seed, nonce);
    if (ETA == 2) {
        cbd2_from_state(A, emit);
    } else {
        uint32_t w[48];
#pragma unroll
        for (int i = 0; i < 17; i++) {
            w[2 * i] = A[i].x;
            w[2 * i + 1] = A[i].y;
        }
        keccak_f1600_core(A);
#pragma unroll
        for (int i = 0; i < 7; i++) {
            w[34 + 2 * i] = A[i].x;
            w[35 + 2 * i] = A[i].y;
        }
        cbd3_from_words(w, emit);
    }
}

// ---------------------------------------------------------------------------------------------
// Matrix rows: stream SHAKE128(rho || x || y), rejection-sample, multiply into the accumulator.
// ---------------------------------------------------------------------------------------------

// One matrix entry per thread: stream SHAKE128(rho || x || y), rejection-sample in order, and as
// soon as a coefficient pair (2p, 2p+1) is complete multiply it with b (basemul) and add it into
// the shared accumulator with one 32-bit shared-memory atomic.  The two products are packed with a
// bias of 2q each: a basemul output lies in [-11, q + 11], so a biased term lies in (q, 4q) and the
// sum of at most four terms stays below 2^16 -- the halves never carry into each other.  The
// consumer subtracts K * 2q from each half, which yields the sum of the K products, before the
// Barrett of pointwise_acc.
constexpr uint32_t ACC_BIAS = 2 * Q;

// Per-thread staging of accepted candidates in shared memory: each Keccak block is parsed in parts
// of 28 candidates (round 3: 4 parts of 14 triplets; round 2: 3 parts of 14 little-endian words),
// consumed after each part.  A part yields at most 28 accepted coefficients, plus one carried over
// from the previous part (an unpaired even coefficient), so 30 int16 per thread suffice (29, kept
// even for the 32-bit pair loads).  Parts of 28 rather than halves of a block halve this area, which
// fits a 13th instance into a 128-thread CTA at three CTAs per SM (Kyber-768 encryption).
constexpr int STAGE_INT16 = 30;
template <int V>
__host__ __device__ constexpr int parts_per_block() {
    return V == 3 ? 4 : 3;
}

// Append the accepted candidates of part PART of a block to stg[n...] without branches (the store
// is unconditional, the count advances only on acceptance), in the order of the byte stream.
template <int V, int PART>
__device__ __forceinline__ void compact_part(const uint2 (&A)[25], int16_t *stg, int &n) {
    if (V == 3) {
        // 56 triplets per block, two 12-bit candidates each (round-3 Parse); this part: 14 triplets
#pragma unroll
        for (int tt = 0; tt < 14; tt++) {
            const int t = 14 * PART + tt, o = 3 * t, wi = o >> 2, sh = 8 * (o & 3);
            const uint32_t w0 = (wi & 1) ? A[wi >> 1].y : A[wi >> 1].x;
            uint32_t v;
            if (sh <= 8) {
                v = w0 >> sh;
            } else {
                const uint32_t w1 = ((wi + 1) & 1) ? A[(wi + 1) >> 1].y : A[(wi + 1) >> 1].x;
                v = __funnelshift_r(w0, w1, sh);
            }
            const uint32_t d0 = v & 0xfff, d1 = (v >> 12) & 0xfff;
            stg[n] = (int16_t)d0;
            n += (d0 < (uint32_t)Q);
            stg[n] = (int16_t)d1;
            n += (d1 < (uint32_t)Q);
        }
    } else {
        // 84 little-endian 16-bit candidates per block, v < 19q kept as v - (v >> 12) q
        // (rej_uniform, indcpa.cu:290-322); this part: 14 words, 28 candidates
#pragma unroll
        for (int tt = 0; tt < 14; tt++) {
            const int t = 14 * PART + tt;
            const uint32_t w0 = (t & 1) ? A[t >> 1].y : A[t >> 1].x;
            const uint32_t d0 = w0 & 0xffff, d1 = w0 >> 16;
            stg[n] = (int16_t)(d0 - (d0 >> 12) * Q);
            n += (d0 < (uint32_t)(19 * Q));
            stg[n] = (int16_t)(d1 - (d1 >> 12) * Q);
            n += (d1 < (uint32_t)(19 * Q));
        }
    }
}

// Multiply the complete pairs staged in stg[0..n) into the accumulator (pair index from ctr),
// stopping at 256 coefficients; an unpaired last coefficient moves to stg[0].
__device__ __forceinline__ void consume_pairs(int16_t *stg, int &n, int &ctr, const int16_t *b, uint32_t *acc,
                                              const int2 *tw) {
    int i = 0;
    for (; i + 1 < n && ctr < N; i += 2, ctr += 2) {
        const uint32_t av = *reinterpret_cast<const uint32_t *>(stg + i);
        const int p = ctr >> 1, o = phys(2 * p);
        const uint32_t bb = *reinterpret_cast<const uint32_t *>(b + o);
        // staged coefficients are in [0, 2^12) and the NTT output b in [0, q]: no sign extension
        int32_t r0, r1;
        basemul_plain(r0, r1, (int32_t)(av & 0xffff), (int32_t)(av >> 16), (int32_t)(bb & 0xffff), (int32_t)(bb >> 16),
                      pair_w(tw, p));
        atomicAdd(acc + (o >> 1), (uint32_t)(r0 + (int32_t)ACC_BIAS) | ((uint32_t)(r1 + (int32_t)ACC_BIAS) << 16));
    }
    const bool carry = (i < n) && (ctr < N);
    if (carry) stg[0] = stg[i];
    n = carry ? 1 : 0;
}

// Accumulate A[row][col] o b into acc (packed, biased pairs), where A[i][j] = XOF(rho || j || i)
// (gen_matrix, indcpa.cu:339-403) and the transposed matrix uses XOF(rho || i || j).  One thread
// per entry; the candidate stream is consumed strictly in order, so the entry equals the
// reference's rejection sampling coefficient for coefficient.
template <int V>
__device__ __forceinline__ void matrix_entry(const uint2 *rho, int row, int col, bool transposed, const int16_t *b,
                                             int16_t *acc16, const int2 *tw, int16_t *stg) {
    uint2 A[25];
    keccak_zero(A);
#pragma unroll
    for (int i = 0; i < 4; i++) A[i] = rho[i];
    const uint32_t x = transposed ? row : col, y = transposed ? col : row;
    A[4].x = x | (y << 8) | (DOM_SHAKE << 16);
    A[SHAKE128_LANES - 1].y ^= 0x80000000u;
    uint32_t *acc = reinterpret_cast<uint32_t *>(acc16);
    int ctr = 0, n = 0;
    while (ctr < N) {
        keccak_f1600_core(A);
        compact_part<V, 0>(A, stg, n);
        consume_pairs(stg, n, ctr, b, acc, tw);
        if (ctr >= N) break;
        compact_part<V, 1>(A, stg, n);
        consume_pairs(stg, n, ctr, b, acc, tw);
        if (ctr >= N) break;
        compact_part<V, 2>(A, stg, n);
        consume_pairs(stg, n, ctr, b, acc, tw);
        if constexpr (parts_per_block<V>() == 4) {
            if (ctr >= N) break;
            compact_part<V, 3>(A, stg, n);
            consume_pairs(stg, n, ctr, b, acc, tw);
        }
    }
}

// Undo the accumulator bias of K terms and apply pointwise_acc's Barrett.
template <int K>
__device__ __forceinline__ int32_t unbias(int32_t biased) {
    return barrett_hi((biased & 0xffff) - (int32_t)(K * ACC_BIAS));
}
__device__ __forceinline__ int32_t csubq32(int32_t a) {
    a -= Q;
    return a + ((a >> 31) & Q);
}

// Zero `npoly` consecutive shared polynomials starting at p (all threads of the CTA).
__device__ __forceinline__ void zero_polys(int16_t *p, int npoly) {
    uint4 *q = reinterpret_cast<uint4 *>(p);
    const int n16 = npoly * (POLY_PITCH / 8);
    for (int i = threadIdx.x; i < n16; i += blockDim.x) q[i] = make_uint4(0, 0, 0, 0);
}

// ---------------------------------------------------------------------------------------------
// Codecs (warp per instance, lane = group of 8 coefficients)
// ---------------------------------------------------------------------------------------------
template <int D>
__device__ __forceinline__ uint32_t compress_u(uint32_t x) {
    // x canonical in [0, q)
    return (((x << D) + Q / 2) / Q) & ((1u << D) - 1);
}
template <int D>
__device__ __forceinline__ uint32_t compress_d(int16_t x) { return compress_u<D>((uint16_t)x); }
template <int D>
__device__ __forceinline__ int16_t decompress_d(uint32_t t) {
    return (int16_t)((t * Q + (1u << (D - 1))) >> D);
}
// 8 D-bit values -> D bytes (little-endian bit order), via a 128-bit accumulator.
template <int D>
__device__ __forceinline__ void pack8(uint8_t (&out)[D], const uint32_t (&t)[8]) {
    uint64_t lo = 0, hi = 0;
#pragma unroll
    for (int j = 0; j < 8; j++) {
        const int bit = D * j;
        if (bit < 64) {
            lo |= (uint64_t)t[j] << bit;
            if (bit + D > 64) hi |= (uint64_t)t[j] >> (64 - bit);
        } else {
            hi |= (uint64_t)t[j] << (bit - 64);
        }
    }
#pragma unroll
    for (int b = 0; b < D; b++) out[b] = (uint8_t)(b < 8 ? (lo >> (8 * b)) : (hi >> (8 * (b - 8))));
}
template <int D>
__device__ __forceinline__ void unpack8(uint32_t (&t)[8], const uint8_t *in) {
    uint64_t lo = 0, hi = 0;
#pragma unroll
    for (int b = 0; b < D; b++) {
        if (b < 8) lo |= (uint64_t)in[b] << (8 * b);
        else hi |= (uint64_t)in[b] << (8 * (b - 8));
    }
#pragma unroll
    for (int j = 0; j < 8; j++) {
        const int bit = D * j;
        uint64_t v;
        if (bit < 64) {
            v = lo >> bit;
            if (bit + D > 64) v |= hi << (64 - bit);
        } else {
            v = hi >> (bit - 64);
        }
        t[j] = (uint32_t)v & ((1u << D) - 1);
    }
}

// ---------------------------------------------------------------------------------------------
// Kernel parameters
// ---------------------------------------------------------------------------------------------
// KEM layer: KEM_FO = the round-2 / round-3 Fujisaki-Okamoto transform (H(coins), KDF(K || H(c)));
// KEM_MLKEM = FIPS 203 (G(d || k), no message pre-hash, K used directly, rejection key J(z || c)).
constexpr int KEM_FO = 1, KEM_MLKEM = 2;

struct KpArgs {
    int n;
    uint8_t *pk;
    uint8_t *sk;             // CPA: sk_cpa (stride SKCPA); KEM: full sk (stride SKB)
    const uint8_t *coins;    // d (and z for KEM) per instance
    int coins_stride;
    int kem;                 // 1: write sk = sk_cpa || pk || (H(pk) later) || z
    const uint8_t *g_in;     // batches above KP_FUSED_MAX: (rho, sigma) per instance (64 B) computed by
                             // kyber_kp_hash_pre; null: the core kernel computes G itself
};
struct EncArgs {
    int n;
    uint8_t *ct;
    const uint8_t *pk;
    int pk_stride;
    const uint8_t *m;        // message (32 B) per instance
    int m_stride;
    const uint8_t *r;        // noise seed (32 B) per instance
    int r_stride;
};
struct DecArgs {
    int n;
    const uint8_t *ct;
    const uint8_t *sk;       // CPA: sk_cpa (stride SKCPA); KEM: full sk (stride SKB)
    uint8_t *m_out;          // CPA only: decrypted message
    uint8_t *ss;             // KEM only
    const uint8_t *hct;      // KEM only: H(c) per instance (32 B); ML-KEM: J(z || c)
    int kem;                 // 0 CPA, KEM_FO, KEM_MLKEM
    uint8_t *mr;             // two-stage decapsulation: m' || r' || K-bar' per instance (96 B)
    int kdf_post;            // KEM_FO: 1 = the re-encryption stage leaves the selected key (K-bar'
                             // or z) in mr + 64 and kyber_dec_hash_post derives ss from it
    int g_post;              // KEM: 1 = the decryption stage leaves m' in mr and kyber_dec_hash_mid
                             // computes (K-bar', r') = G(m' || h) into mr + 64 / mr + 32
};

// Decapsulation stages.  A KEM decapsulation runs as two kernels: decryption + G (warp-level
// phases, its own launch shape), then re-encryption + comparison + key selection, whose phases are
// those of encapsulation and which therefore runs at an encapsulation-like shape and efficiency.
// Measured on GB300 (Kyber-768, 65536): 0.29 + 1.54 ms against 2.03 ms as one kernel.  For
// batches above DEC_FUSED_MAX the two single-permutation hashes at the ends of the stages (G, the KDF) run
// as thread-per-instance kernels between and after them (DecArgs::g_post, kdf_post): inside a CTA
// each held its shared memory while NI threads permuted (0.26 -> 0.19 ms and 1.27 -> 1.10 ms for
// the two stages, 24 us per hash kernel).  CPA decryption alone (DEC_FUSED) stops after the message.
constexpr int DEC_FUSED = 0, DEC_DECRYPT = 1, DEC_REENCRYPT = 2;

// Shared-memory layout for a CTA of NI instances: twiddles, NPOLY polynomials per instance,
// SEEDB bytes of per-instance seeds / flags / noise bytes, and the per-thread staging areas.
template <int NPOLY, int SEEDB>
struct Layout {
    static __host__ __device__ constexpr size_t bytes(int ni, int threads) {
        return 2 * 128 * sizeof(int2) + (size_t)ni * NPOLY * POLY_PITCH * sizeof(int16_t) + (size_t)ni * SEEDB +
               (size_t)threads * STAGE_INT16 * sizeof(int16_t);
    }
};
// Per-thread staging area (after the seeds block).
template <int SEEDB>
__device__ __forceinline__ int16_t *stage_of(uint8_t *seeds, int ni) {
    return reinterpret_cast<int16_t *>(seeds + (size_t)ni * SEEDB) + (size_t)threadIdx.x * STAGE_INT16;
}
// Encryption seed block per instance: [0,32) m, [32,64) r, [64,96) K-bar, [96] flag, then the
// 128-byte PRF outputs of the K + 1 error polynomials e1_0..e1_{K-1}, e2 (eta2 = 2), whose CBD is
// applied in the packing phase.  The PRF output of r_i (64 eta1 bytes) is parked in the shared
// slot of the accumulator u_i, which is zeroed only after the NTT phase has consumed it.
template <int K, int V>
__host__ __device__ constexpr int enc_seed_bytes() {
    return 128 + 128 * (K + 1);
}

__device__ __forceinline__ void load_twiddles(int2 *tw, int2 *twi) {
    for (int i = threadIdx.x; i < 128; i += blockDim.x) {
        tw[i] = c_tw[i];
        twi[i] = c_twi[i];
    }
}

// 12-bit serialisation of 8 canonical coefficients -> 12 bytes (poly_tobytes, poly.cu:79-97)
__device__ __forceinline__ void tobytes8(uint8_t *out, const int16_t (&c)[8]) {
#pragma unroll
    for (int i = 0; i < 4; i++) {
        const uint16_t t0 = (uint16_t)c[2 * i], t1 = (uint16_t)c[2 * i + 1];
        out[3 * i] = (uint8_t)t0;
        out[3 * i + 1] = (uint8_t)((t0 >> 8) | ((t1 & 0xf) << 4));
        out[3 * i + 2] = (uint8_t)(t1 >> 4);
    }
}
__device__ __forceinline__ void tobytes8(uint8_t *out, const int32_t (&c)[8]) {
#pragma unroll
    for (int i = 0; i < 4; i++) {
        const uint32_t t0 = (uint32_t)c[2 * i], t1 = (uint32_t)c[2 * i + 1];
        out[3 * i] = (uint8_t)t0;
        out[3 * i + 1] = (uint8_t)((t0 >> 8) | (t1 << 4));
        out[3 * i + 2] = (uint8_t)(t1 >> 4);
    }
}
__device__ __forceinline__ void frombytes8(int16_t (&c)[8], const uint8_t *in) {
#pragma unroll
    for (int i = 0; i < 4; i++) {
        c[2 * i] = (int16_t)(in[3 * i] | (((uint16_t)in[3 * i + 1] & 0x0f) << 8));
        c[2 * i + 1] = (int16_t)((in[3 * i + 1] >> 4) | ((uint16_t)in[3 * i + 2] << 4));
    }
}
__device__ __forceinline__ void frombytes8(int32_t (&c)[8], const uint8_t *in) {
#pragma unroll
    for (int i = 0; i < 4; i++) {
        c[2 * i] = in[3 * i] | ((in[3 * i + 1] & 0x0f) << 8);
        c[2 * i + 1] = (in[3 * i + 1] >> 4) | (in[3 * i + 2] << 4);
    }
}

// ---------------------------------------------------------------------------------------------
// Encryption phases shared by encapsulation and the re-encryption inside decapsulation.
// Polynomial slots per instance: [0, K) = r-hat, [K, 2K) = u accumulators, 2K = v.
// ---------------------------------------------------------------------------------------------
template <int K, int V>
__device__ __forceinline__ int16_t *slot(int16_t *polys, int li, int s) {
    return polys + ((size_t)li * (2 * K + 1) + s) * POLY_PITCH;
}

template <int K, int V, bool DEC>
__device__ void encrypt_phases(int16_t *polys, uint8_t *seeds, const int2 *tw, const int2 *twi, int ni,
                               int ni_alloc, int base, const EncArgs &a, const uint8_t *ct_cmp) {
    using Pp = P<K, V>;
    constexpr int SB = enc_seed_bytes<K, V>();
    const int tid = threadIdx.x, nthr = blockDim.x, lane = tid & 31, warp = tid >> 5, nwarp = nthr >> 5;

    // (1) all 2K + 1 PRF permutations, one thread each: PRF(coins, i) output bytes -> the slot of
    //     u_i for r_i, the seed block for the errors (CBD applied in (2) for r, in (5) for the
    //     errors).  Every job runs the same code (eta1 = 3 needs a second squeeze: those r jobs come
    //     first, so a warp mixes the two lengths at most once).
    for (int job = tid; job < ni * (2 * K + 1); job += nthr) {
        const bool rj = job < ni * K;
        const int li = rj ? job / K : (job - ni * K) / (K + 1);
        const int i = rj ? job % K : K + (job - ni * K) % (K + 1);
        const uint2 *seed = DEC ? reinterpret_cast<const uint2 *>(seeds + li * SB + 32)
                                : reinterpret_cast<const uint2 *>(a.r + (size_t)(base + li) * a.r_stride);
        uint2 A[25];
        prf_absorb(A, seed, i);
        uint2 *o = rj ? reinterpret_cast<uint2 *>(slot<K, V>(polys, li, K + i))
                      : reinterpret_cast<uint2 *>(seeds + li * SB + 128 + 128 * (i - K));
        if (Pp::ETA1 == 3 && rj) {  // 192 bytes: the first squeeze (136) and 56 of the second
#pragma unroll
            for (int q = 0; q < 17; q++) o[q] = A[q];
            keccak_f1600_core(A);
#pragma unroll
            for (int q = 0; q < 7; q++) o[17 + q] = A[q];
        } else {
#pragma unroll
            for (int q = 0; q < 16; q++) o[q] = A[q];
        }
    }
    __syncthreads();
    // (2) r_i = CBD_eta1(PRF bytes in the slot of u_i), then zero u_i and r-hat_i = NTT(r_i): warp per
    //     polynomial, lane = 8 coefficients
    for (int w = warp; w < ni * K; w += nwarp) {
        const int li = w / K, i = w % K;
        int16_t *u = slot<K, V>(polys, li, K + i);
        const uint8_t *b = reinterpret_cast<const uint8_t *>(u);
        int16_t c[8];
        if (Pp::ETA1 == 2) {  // 4 bytes -> 8 coefficients (cbd.cu:42-63)
            const uint32_t t = reinterpret_cast<const uint32_t *>(b)[lane];
            uint32_t d = t & 0x55555555u;
            d += (t >> 1) & 0x55555555u;
#pragma unroll
            for (int q = 0; q < 8; q++) c[q] = (int16_t)((int)((d >> (4 * q)) & 3) - (int)((d >> (4 * q + 2)) & 3));
        } else {  // 6 bytes (two 3-byte groups) -> 8 coefficients
            const uint16_t *h = reinterpret_cast<const uint16_t *>(b + 6 * lane);
            const uint32_t lo = h[0] | ((uint32_t)h[1] << 16), hi = h[2];
#pragma unroll
            for (int g = 0; g < 2; g++) {
                const uint32_t v = g ? ((lo >> 24) | (hi << 8)) & 0x00ffffffu : lo & 0x00ffffffu;
                uint32_t d = v & 0x00249249u;
                d += (v >> 1) & 0x00249249u;
                d += (v >> 2) & 0x00249249u;
#pragma unroll
                for (int j = 0; j < 4; j++)
                    c[4 * g + j] = (int16_t)((int)((d >> (6 * j)) & 7) - (int)((d >> (6 * j + 3)) & 7));
            }
        }
        int16_t *p = slot<K, V>(polys, li, i);
        store8(p + phys(8 * lane), c);
        __syncwarp();
        uint4 *uz = reinterpret_cast<uint4 *>(u);
        for (int q = lane; q < POLY_PITCH / 8; q += 32) uz[q] = make_uint4(0, 0, 0, 0);
        ntt_warp(p, tw, lane);
    }
    __syncthreads();
    // (3) u_i += A^T[i][j] o r-hat_j, streamed from SHAKE128, one thread per matrix entry
    for (int job = tid; job < ni * K * K; job += nthr) {
        const int li = job / (K * K), i = (job / K) % K, j = job % K;
        const uint8_t *pk = a.pk + (size_t)(base + li) * a.pk_stride;
        matrix_entry<V>(reinterpret_cast<const uint2 *>(pk + Pp::POLYVECBYTES), i, j, true, slot<K, V>(polys, li, j),
                        slot<K, V>(polys, li, K + i), tw, stage_of<SB>(seeds, ni_alloc));
    }
    //     v = t-hat o r-hat (warp per instance, t-hat decoded from pk bytes; independent of (3))
    for (int li = warp; li < ni; li += nwarp) {
        const uint8_t *pk = a.pk + (size_t)(base + li) * a.pk_stride;
        int32_t acc[8];
        for (int j = 0; j < K; j++) {
            int32_t t[8], b[8], r[8];
            frombytes8(t, pk + 384 * j + 12 * lane);
            load8(b, slot<K, V>(polys, li, j) + phys(8 * lane));
#pragma unroll
            for (int q = 0; q < 4; q++)
                basemul_plain(r[2 * q], r[2 * q + 1], t[2 * q], t[2 * q + 1], b[2 * q], b[2 * q + 1],
                              pair_w(tw, 4 * lane + q));
#pragma unroll
            for (int q = 0; q < 8; q++) acc[q] = (j == 0) ? r[q] : acc[q] + r[q];
        }
#pragma unroll
        for (int q = 0; q < 8; q++) acc[q] = barrett_hi(acc[q]);
        store8(slot<K, V>(polys, li, 2 * K) + phys(8 * lane), acc);
    }
    __syncthreads();
    // (4) inverse NTT of u (K, accumulators unbiased + reduced on load) and v
    for (int w = warp; w < ni * (K + 1); w += nwarp) {
        int16_t *p = slot<K, V>(polys, w / (K + 1), K + w % (K + 1));
        if (w % (K + 1) < K) {
            int16_t c[8];
            load8(c, p + phys(8 * lane));
#pragma unroll
            for (int q = 0; q < 8; q++) c[q] = unbias<K>(c[q]);
            store8(p + phys(8 * lane), c);
            __syncwarp();
        }
        invntt_warp(p, twi, lane);
    }
    __syncthreads();
    // (5) warp per instance, lane = 8 coefficients: u += e1, v += e2 + msg (CBD_eta2 of the stored
    //     PRF bytes, cbd.cu:42-63), Barrett, compress, and pack (encaps) or compare with the
    //     received ciphertext (decaps)
    for (int li = warp; li < ni; li += nwarp) {
        uint8_t *out = DEC ? nullptr : a.ct + (size_t)(base + li) * Pp::CTB;
        const uint8_t *cmp = DEC ? ct_cmp + (size_t)(base + li) * Pp::CTB : nullptr;
        const uint8_t *msg = DEC ? seeds + li * SB : a.m + (size_t)(base + li) * a.m_stride;
        const uint8_t mb = msg[lane];
        uint32_t diff = 0;
        // With even DU and DV (k = 2, 3) every lane's byte group starts at an even offset of a
        // 16-byte-aligned row of even length, so the ciphertext moves as 16-bit words.  Decaps loads
        // the lane's words of the received ciphertext before the arithmetic, so their latency
        // overlaps it instead of following each polynomial (measured: the byte loads cost 5 % of
        // the Kyber-768 re-encryption stage).
        constexpr bool W16 = (Pp::DU % 2 == 0) && (Pp::DV % 2 == 0);
        constexpr int NW = K * (Pp::DU / 2) + Pp::DV / 2;
        uint32_t cw[DEC && W16 ? NW : 1];
        if constexpr (DEC && W16) {
#pragma unroll
            for (int i = 0; i < K; i++)
#pragma unroll
                for (int q = 0; q < Pp::DU / 2; q++)
                    cw[i * (Pp::DU / 2) + q] =
                        reinterpret_cast<const uint16_t *>(cmp + (size_t)i * Pp::DU * 32 + (size_t)lane * Pp::DU)[q];
#pragma unroll
            for (int q = 0; q < Pp::DV / 2; q++)
                cw[K * (Pp::DU / 2) + q] = reinterpret_cast<const uint16_t *>(cmp + (size_t)Pp::CTU + (size_t)lane * Pp::DV)[q];
        }
#pragma unroll
        for (int i = 0; i <= K; i++) {
            const uint32_t t = reinterpret_cast<const uint32_t *>(seeds + li * SB + 128 + 128 * i)[lane];
            uint32_t d = t & 0x55555555u;
            d += (t >> 1) & 0x55555555u;
            int16_t c[8];
            load8(c, slot<K, V>(polys, li, K + i) + phys(8 * lane));
            uint32_t cv[8];
#pragma unroll
            for (int q = 0; q < 8; q++) {
                const int16_t e = (int16_t)((int)((d >> (4 * q)) & 3) - (int)((d >> (4 * q + 2)) & 3));
                int16_t x = (int16_t)(c[q] + e);
                if (i == K) x = (int16_t)(x + (int16_t)(((mb >> q) & 1) ? (Q + 1) / 2 : 0));
                x = csubq(barrett(x));
                cv[q] = (i < K) ? compress_d<Pp::DU>(x) : compress_d<Pp::DV>(x);
            }
            if (i < K) {
                uint8_t b[Pp::DU];
                pack8<Pp::DU>(b, cv);
                const size_t off = (size_t)i * Pp::DU * 32 + (size_t)lane * Pp::DU;
                if constexpr (W16) {
#pragma unroll
                    for (int q = 0; q < Pp::DU / 2; q++) {
                        const uint32_t w = (uint32_t)b[2 * q] | ((uint32_t)b[2 * q + 1] << 8);
                        if constexpr (DEC) diff |= w ^ cw[i * (Pp::DU / 2) + q];
                        else reinterpret_cast<uint16_t *>(out + off)[q] = (uint16_t)w;
                    }
                } else {
#pragma unroll
                    for (int q = 0; q < Pp::DU; q++) {
                        if (DEC) diff |= (uint32_t)(b[q] ^ cmp[off + q]);
                        else out[off + q] = b[q];
                    }
                }
            } else {
                uint8_t b[Pp::DV];
                pack8<Pp::DV>(b, cv);
                const size_t off = (size_t)Pp::CTU + (size_t)lane * Pp::DV;
                if constexpr (W16) {
#pragma unroll
                    for (int q = 0; q < Pp::DV / 2; q++) {
                        const uint32_t w = (uint32_t)b[2 * q] | ((uint32_t)b[2 * q + 1] << 8);
                        if constexpr (DEC) diff |= w ^ cw[K * (Pp::DU / 2) + q];
                        else reinterpret_cast<uint16_t *>(out + off)[q] = (uint16_t)w;
                    }
                } else {
#pragma unroll
                    for (int q = 0; q < Pp::DV; q++) {
                        if (DEC) diff |= (uint32_t)(b[q] ^ cmp[off + q]);
                        else out[off + q] = b[q];
                    }
                }
            }
        }
        if (DEC) {
            diff = __any_sync(0xffffffffu, diff != 0);
            if (lane == 0) seeds[li * SB + 96] = (uint8_t)diff;
        }
    }
}


// ---------------------------------------------------------------------------------------------
// Kernels
// ---------------------------------------------------------------------------------------------
constexpr int CORE_MAX_THREADS = 512;

// Encapsulation of instances [base, base + NI) of `a` by the calling CTA (dynamic shared memory
// laid out for NI instances of this K).
template <int K, int V>
__device__ __forceinline__ void enc_core_body(const EncArgs &a, int NI, int base) {
    extern __shared__ __align__(16) uint8_t smem[];
    int2 *tw = reinterpret_cast<int2 *>(smem), *twi = tw + 128;
    int16_t *polys = reinterpret_cast<int16_t *>(twi + 128);
    uint8_t *seeds = reinterpret_cast<uint8_t *>(polys + (size_t)NI * (2 * K + 1) * POLY_PITCH);
    const int ni = min(NI, a.n - base);
    load_twiddles(tw, twi);
    __syncthreads();
    encrypt_phases<K, V, false>(polys, seeds, tw, twi, ni, NI, base, a, nullptr);
}
template <int K, int V>
__global__ void __launch_bounds__(kyber_bound_threads(1, K), kyber_bound_ctas(1, K)) kyber_enc_core(EncArgs a, int NI) {
    enc_core_body<K, V>(a, NI, blockIdx.x * NI);
}

// Decapsulation (stage STAGE) of instances [base, base + NI) of `d` by the calling CTA.
template <int K, int V, int STAGE>
__device__ __forceinline__ void dec_core_body(const DecArgs &d, int NI, int base) {
    using Pp = P<K, V>;
    constexpr int SB = enc_seed_bytes<K, V>();
    extern __shared__ __align__(16) uint8_t smem[];
    int2 *tw = reinterpret_cast<int2 *>(smem), *twi = tw + 128;
    int16_t *polys = reinterpret_cast<int16_t *>(twi + 128);
    uint8_t *seeds = reinterpret_cast<uint8_t *>(polys + (size_t)NI * (2 * K + 1) * POLY_PITCH);
    const int ni = min(NI, d.n - base);
    const int tid = threadIdx.x, nthr = blockDim.x, lane = tid & 31, warp = tid >> 5, nwarp = nthr >> 5;
    const int sks = d.kem ? Pp::SKB : Pp::SKCPA;
    load_twiddles(tw, twi);
    if constexpr (STAGE == DEC_REENCRYPT) {
        // m', r', K-bar' of the CTA's instances from the decryption stage
        for (int t = tid; t < ni * 12; t += nthr)
            reinterpret_cast<uint2 *>(seeds + (t / 12) * SB)[t % 12] =
                reinterpret_cast<const uint2 *>(d.mr + (size_t)(base + t / 12) * 96)[t % 12];
        __syncthreads();
    } else {
    // (a) decompress u' -> slots [K, 2K), v' -> slot 2K (unpack_ciphertext, indcpa.cu:264-275)
    for (int li = warp; li < ni; li += nwarp) {
        const uint8_t *ct = d.ct + (size_t)(base + li) * Pp::CTB;
        for (int i = 0; i <= K; i++) {
            uint32_t t[8];
            int16_t c[8];
            if (i < K) {
                unpack8<Pp::DU>(t, ct + (size_t)i * Pp::DU * 32 + (size_t)lane * Pp::DU);
#pragma unroll
                for (int q = 0; q < 8; q++) c[q] = decompress_d<Pp::DU>(t[q]);
            } else {
                unpack8<Pp::DV>(t, ct + Pp::CTU + (size_t)lane * Pp::DV);
#pragma unroll
                for (int q = 0; q < 8; q++) c[q] = decompress_d<Pp::DV>(t[q]);
            }
            store8(slot<K, V>(polys, li, K + i) + phys(8 * lane), c);
        }
    }
    __syncthreads();
    // (b) u-hat = NTT(u')
    for (int w = warp; w < ni * K; w += nwarp) ntt_warp(slot<K, V>(polys, w / K, K + w % K), tw, lane);
    __syncthreads();
    // (c) mp = s-hat o u-hat -> slot 0
    for (int li = warp; li < ni; li += nwarp) {
        const uint8_t *sk = d.sk + (size_t)(base + li) * sks;
        int32_t acc[8];
        for (int j = 0; j < K; j++) {
            int32_t s[8], b[8], r[8];
            frombytes8(s, sk + 384 * j + 12 * lane);
            load8(b, slot<K, V>(polys, li, K + j) + phys(8 * lane));
#pragma unroll
            for (int q = 0; q < 4; q++)
                basemul_plain(r[2 * q], r[2 * q + 1], s[2 * q], s[2 * q + 1], b[2 * q], b[2 * q + 1],
                              pair_w(tw, 4 * lane + q));
#pragma unroll
            for (int q = 0; q < 8; q++) acc[q] = (j == 0) ? r[q] : acc[q] + r[q];
        }
#pragma unroll
        for (int q = 0; q < 8; q++) acc[q] = barrett_hi(acc[q]);
        store8(slot<K, V>(polys, li, 0) + phys(8 * lane), acc);
    }
    __syncthreads();
    for (int w = warp; w < ni; w += nwarp) invntt_warp(slot<K, V>(polys, w, 0), twi, lane);
    __syncthreads();
    // (d) m' = tomsg(reduce(v - mp)), lane = message byte
    for (int li = warp; li < ni; li += nwarp) {
        int32_t v[8], mp[8];
        load8(v, slot<K, V>(polys, li, 2 * K) + phys(8 * lane));
        load8(mp, slot<K, V>(polys, li, 0) + phys(8 * lane));
        uint32_t byte = 0;
#pragma unroll
        for (int q = 0; q < 8; q++) byte |= compress_u<1>((uint32_t)csubq32(barrett_hi(v[q] - mp[q]))) << q;
        seeds[li * SB + lane] = (uint8_t)byte;
        if (!d.kem) d.m_out[(size_t)(base + li) * 32 + lane] = (uint8_t)byte;
        if (STAGE == DEC_DECRYPT && d.g_post) d.mr[(size_t)(base + li) * 96 + lane] = (uint8_t)byte;
    }
    if (!d.kem) return;
    // For large batches G leaves this CTA: one permutation on NI of its threads at its end moves to
    // kyber_dec_hash_mid, a thread per instance over the whole batch.
    if (STAGE == DEC_DECRYPT && d.g_post) return;
    __syncthreads();
    // (e) (K-bar', r') = G(m' || h)
    for (int li = tid; li < ni; li += nthr) {
        const uint8_t *sk = d.sk + (size_t)(base + li) * Pp::SKB;
        uint2 A[25];
        keccak_zero(A);
        const uint2 *m2 = reinterpret_cast<const uint2 *>(seeds + li * SB);
        const uint2 *h2 = reinterpret_cast<const uint2 *>(sk + Pp::SKB - 64);
#pragma unroll
        for (int i = 0; i < 4; i++) {
            A[i] = m2[i];
            A[4 + i] = h2[i];
        }
        A[8].x ^= DOM_SHA3;
        A[SHA3_512_LANES - 1].y ^= 0x80000000u;
        keccak_f1600_core(A);
        if constexpr (STAGE == DEC_DECRYPT) {
            uint2 *o = reinterpret_cast<uint2 *>(d.mr + (size_t)(base + li) * 96);
#pragma unroll
            for (int i = 0; i < 4; i++) {
                o[i] = m2[i];
                o[4 + i] = A[4 + i];  // r'
                o[8 + i] = A[i];      // K-bar'
            }
        } else {
            uint2 *kb = reinterpret_cast<uint2 *>(seeds + li * SB + 64), *rr = reinterpret_cast<uint2 *>(seeds + li * SB + 32);
#pragma unroll
            for (int i = 0; i < 4; i++) {
                kb[i] = A[i];
                rr[i] = A[4 + i];
            }
        }
    }
    if constexpr (STAGE == DEC_DECRYPT) return;
    __syncthreads();
    }  // STAGE != DEC_REENCRYPT
    // (f) re-encrypt m' with r' under the pk stored in sk and compare with the received ct
    EncArgs e;
    e.n = d.n;
    e.ct = nullptr;
    e.pk = d.sk + Pp::SKCPA;
    e.pk_stride = Pp::SKB;
    e.m = nullptr;
    e.m_stride = 0;
    e.r = nullptr;
    e.r_stride = 0;
    encrypt_phases<K, V, true>(polys, seeds, tw, twi, ni, NI, base, e, d.ct);
    __syncthreads();
    // (g) ML-KEM: ss = fail ? J(z || c) : K' (constant-time select, no hashing)
    if (d.kem == KEM_MLKEM) {
        for (int li = tid; li < ni; li += nthr) {
            const uint32_t mask = 0u - (uint32_t)(seeds[li * SB + 96] != 0);
            const uint2 *kb = reinterpret_cast<const uint2 *>(seeds + li * SB + 64);
            const uint2 *jz = reinterpret_cast<const uint2 *>(d.hct + (size_t)(base + li) * 32);
            uint2 *out = reinterpret_cast<uint2 *>(d.ss + (size_t)(base + li) * 32);
#pragma unroll
            for (int i = 0; i < 4; i++) {
                const uint2 kk = kb[i], jj = jz[i];
                out[i] = make_uint2(kk.x ^ (mask & (kk.x ^ jj.x)), kk.y ^ (mask & (kk.y ^ jj.y)));
            }
        }
        return;
    }
    // (g) ss = SHAKE256(fail ? z : K-bar' || H(c)), with a constant-time select.  For large
    //     batches only the select runs here: one permutation on NI threads at the end of every CTA
    //     (measured: 11 % of this kernel at 65536 Kyber-768 instances) moves to kyber_dec_hash_post,
    //     a thread per instance over the whole batch.
    if (d.kdf_post) {
        for (int t = tid; t < ni * 4; t += nthr) {
            const int li = t >> 2, i = t & 3;
            const uint32_t mask = 0u - (uint32_t)(seeds[li * SB + 96] != 0);
            const uint2 zk = reinterpret_cast<const uint2 *>(d.sk + (size_t)(base + li) * Pp::SKB + Pp::SKB - 32)[i];
            const uint2 kk = reinterpret_cast<const uint2 *>(seeds + li * SB + 64)[i];
            reinterpret_cast<uint2 *>(d.mr + (size_t)(base + li) * 96 + 64)[i] =
                make_uint2(kk.x ^ (mask & (kk.x ^ zk.x)), kk.y ^ (mask & (kk.y ^ zk.y)));
        }
        return;
    }
    for (int li = tid; li < ni; li += nthr) {
        const uint8_t *sk = d.sk + (size_t)(base + li) * Pp::SKB;
        const uint32_t mask = 0u - (uint32_t)(seeds[li * SB + 96] != 0);
        const uint2 *kb = reinterpret_cast<const uint2 *>(seeds + li * SB + 64);
        const uint2 *z = reinterpret_cast<const uint2 *>(sk + Pp::SKB - 32);
        const uint2 *hc = reinterpret_cast<const uint2 *>(d.hct + (size_t)(base + li) * 32);
        uint2 A[25];
        keccak_zero(A);
#pragma unroll
        for (int i = 0; i < 4; i++) {
            const uint2 zk = z[i], kk = kb[i];
            A[i] = make_uint2(kk.x ^ (mask & (kk.x ^ zk.x)), kk.y ^ (mask & (kk.y ^ zk.y)));
            A[4 + i] = hc[i];
        }
        A[8].x ^= DOM_SHAKE;
        A[SHAKE256_LANES - 1].y ^= 0x80000000u;
        keccak_f1600_core(A);
        uint2 *out = reinterpret_cast<uint2 *>(d.ss + (size_t)(base + li) * 32);
#pragma unroll
        for (int i = 0; i < 4; i++) out[i] = A[i];
    }
}
template <int K, int V, int STAGE>
__global__ void __launch_bounds__(kyber_bound_threads(2, K), kyber_bound_ctas(2, K)) kyber_dec_core(DecArgs d, int NI) {
    dec_core_body<K, V, STAGE>(d, NI, blockIdx.x * NI);
}
// The decryption stage alone: its bound keeps two 384-thread CTAs per SM (80 registers a thread).
template <int K, int V>
__global__ void __launch_bounds__(kyber_bound_threads(3, K), kyber_bound_ctas(3, K)) kyber_dec_decrypt(DecArgs d, int NI) {
    dec_core_body<K, V, DEC_DECRYPT>(d, NI, blockIdx.x * NI);
}


// Keypair of instances [base, base + NI) of `a` by the calling CTA.
// Slots [0,K) s, [K,2K) e, [2K,3K) t-hat; seeds [0,32) rho, [32,64) sigma.
template <int K, int V>
__device__ __forceinline__ void kp_core_body(const KpArgs &a, int NI, int base) {
    using Pp = P<K, V>;
    extern __shared__ __align__(16) uint8_t smem[];
    int2 *tw = reinterpret_cast<int2 *>(smem), *twi = tw + 128;
    int16_t *polys = reinterpret_cast<int16_t *>(twi + 128);
    uint8_t *seeds = reinterpret_cast<uint8_t *>(polys + (size_t)NI * (3 * K) * POLY_PITCH);
    auto kslot = [&](int li, int s) { return polys + ((size_t)li * (3 * K) + s) * POLY_PITCH; };
    const int ni = min(NI, a.n - base);
    const int tid = threadIdx.x, nthr = blockDim.x, lane = tid & 31, warp = tid >> 5, nwarp = nthr >> 5;
    load_twiddles(tw, twi);
    // (a) (rho, sigma) = G(d); ML-KEM: G(d || k) with the module rank as one byte (FIPS 203).  For
    //     large batches kyber_kp_hash_pre has computed them (a permutation on NI threads at the
    //     head of the CTA would hold its shared memory meanwhile): load them.
    if (a.g_in) {
        for (int t = tid; t < ni * 8; t += nthr)
            reinterpret_cast<uint2 *>(seeds + (t >> 3) * 128)[t & 7] =
                reinterpret_cast<const uint2 *>(a.g_in + (size_t)(base + (t >> 3)) * 64)[t & 7];
    }
    for (int li = tid; li < ni && !a.g_in; li += nthr) {
        const uint2 *dd = reinterpret_cast<const uint2 *>(a.coins + (size_t)(base + li) * a.coins_stride);
        uint2 A[25];
        keccak_zero(A);
#pragma unroll
        for (int i = 0; i < 4; i++) A[i] = dd[i];
        A[4].x = a.kem == KEM_MLKEM ? ((uint32_t)K | (DOM_SHA3 << 8)) : DOM_SHA3;
        A[SHA3_512_LANES - 1].y ^= 0x80000000u;
        keccak_f1600_core(A);
        uint2 *o = reinterpret_cast<uint2 *>(seeds + li * 128);
#pragma unroll
        for (int i = 0; i < 8; i++) o[i] = A[i];
    }
    __syncthreads();
    // (b) s_i = CBD(PRF(sigma, i)), e_i = CBD(PRF(sigma, K + i)); zero the t-hat accumulators
    for (int li = 0; li < ni; li++) zero_polys(kslot(li, 2 * K), K);
    for (int job = tid; job < ni * 2 * K; job += nthr) {
        const int li = job / (2 * K), i = job % (2 * K);
        int16_t *dst = kslot(li, i);
        noise_poly<Pp::ETA1>(reinterpret_cast<const uint2 *>(seeds + li * 128 + 32), i,
                             [&](int g, const int16_t(&c)[8]) { store8(dst + phys(8 * g), c); });
    }
    __syncthreads();
    for (int w = warp; w < ni * 2 * K; w += nwarp) ntt_warp(kslot(w / (2 * K), w % (2 * K)), tw, lane);
    __syncthreads();
    // (c) t-hat_i += A[i][j] o s-hat_j (not transposed), one thread per matrix entry
    for (int job = tid; job < ni * K * K; job += nthr) {
        const int li = job / (K * K), i = (job / K) % K, j = job % K;
        matrix_entry<V>(reinterpret_cast<const uint2 *>(seeds + li * 128), i, j, false, kslot(li, j), kslot(li, 2 * K + i),
                        tw, stage_of<128>(seeds, NI));
    }
    __syncthreads();
    // (d) t = reduce(frommont(t) + e); pack pk = t || rho and sk_cpa = s (warp per instance)
    for (int li = warp; li < ni; li += nwarp) {
        uint8_t *pk = a.pk + (size_t)(base + li) * Pp::PKB;
        uint8_t *sk = a.sk + (size_t)(base + li) * (a.kem ? Pp::SKB : Pp::SKCPA);
        for (int i = 0; i < K; i++) {
            int32_t t[8], e[8], s[8];
            load8(t, kslot(li, 2 * K + i) + phys(8 * lane));
            load8(e, kslot(li, K + i) + phys(8 * lane));
            load8(s, kslot(li, i) + phys(8 * lane));
#pragma unroll
            for (int q = 0; q < 8; q++) {
                // the plain basemul has no Montgomery factor for poly_tomont to undo
                t[q] = csubq32(barrett_hi(unbias<K>(t[q]) + e[q]));
                s[q] = csubq32(s[q]);
            }
            uint8_t bt[12], bs[12];
            tobytes8(bt, t);
            tobytes8(bs, s);
            const size_t off = (size_t)384 * i + 12 * lane;
#pragma unroll
            for (int q = 0; q < 12; q++) {
                pk[off + q] = bt[q];
                sk[off + q] = bs[q];
                if (a.kem) sk[Pp::SKCPA + off + q] = bt[q];
            }
        }
        if (lane < 4) {
            const uint2 rho = reinterpret_cast<const uint2 *>(seeds + li * 128)[lane];
            reinterpret_cast<uint2 *>(pk + Pp::POLYVECBYTES)[lane] = rho;
            if (a.kem) {
                reinterpret_cast<uint2 *>(sk + Pp::SKCPA + Pp::POLYVECBYTES)[lane] = rho;
                const uint2 z = reinterpret_cast<const uint2 *>(a.coins + (size_t)(base + li) * a.coins_stride + 32)[lane];
                reinterpret_cast<uint2 *>(sk + Pp::SKB - 32)[lane] = z;
            }
        }
    }
}
template <int K, int V>
__global__ void __launch_bounds__(CORE_MAX_THREADS) kyber_kp_core(KpArgs a, int NI) {
    kp_core_body<K, V>(a, NI, blockIdx.x * NI);
}

// ---- flat hash kernels: one thread per instance ----
// The long absorbs (H(pk), H(c)) stage their input blocks through shared memory, a column per
// thread of a 128-thread CTA (keccak_absorb_lanes_staged).
constexpr int HASH_THREADS = 128;
#define KY_HASH_STAGE __shared__ uint2 hstage[2 * SHA3_256_LANES * HASH_THREADS]
// encaps prologue: m = H(coins); (K-bar, r) = G(m || H(pk)); scratch = m || r || K-bar
// ML-KEM: m = coins (no pre-hash)
template <int K, int V>
__global__ void __launch_bounds__(HASH_THREADS) kyber_enc_hash_pre(int n, const uint8_t *pk, const uint8_t *coins,
                                                                   uint8_t *scratch, int kem) {
    using Pp = P<K, V>;
    KY_HASH_STAGE;
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= n) return;
    uint2 A[25], mh[8];
    const uint2 *cn = reinterpret_cast<const uint2 *>(coins + (size_t)x * 32);
    if (kem == KEM_MLKEM) {
#pragma unroll
        for (int i = 0; i < 4; i++) mh[i] = cn[i];
    } else {
        keccak_absorb_lanes<SHA3_256_LANES>(A, cn, 4, DOM_SHA3);
        keccak_f1600(A);
#pragma unroll
        for (int i = 0; i < 4; i++) mh[i] = A[i];
    }
    keccak_absorb_lanes_staged<SHA3_256_LANES>(A, reinterpret_cast<const uint2 *>(pk + (size_t)x * Pp::PKB), Pp::PKB / 8,
                                               DOM_SHA3, hstage, threadIdx.x, HASH_THREADS);
    keccak_f1600(A);
#pragma unroll
    for (int i = 0; i < 4; i++) mh[4 + i] = A[i];
    keccak_zero(A);
#pragma unroll
    for (int i = 0; i < 8; i++) A[i] = mh[i];
    A[8].x ^= DOM_SHA3;
    A[SHA3_512_LANES - 1].y ^= 0x80000000u;
    keccak_f1600(A);
    uint2 *o = reinterpret_cast<uint2 *>(scratch + (size_t)x * 96);
#pragma unroll
    for (int i = 0; i < 4; i++) {
        o[i] = mh[i];         // m
        o[4 + i] = A[4 + i];  // r
        o[8 + i] = A[i];      // K-bar
    }
}
// encaps epilogue: ss = KDF(K-bar || H(c))
// ML-KEM: ss = K (copied, no hashing)
template <int K, int V>
__global__ void __launch_bounds__(HASH_THREADS) kyber_enc_hash_post(int n, const uint8_t *ct, const uint8_t *scratch,
                                                                    uint8_t *ss, int kem) {
    using Pp = P<K, V>;
    KY_HASH_STAGE;
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= n) return;
    if (kem == KEM_MLKEM) {
        const uint2 *kb = reinterpret_cast<const uint2 *>(scratch + (size_t)x * 96 + 64);
        uint2 *o = reinterpret_cast<uint2 *>(ss + (size_t)x * 32);
#pragma unroll
        for (int i = 0; i < 4; i++) o[i] = kb[i];
        return;
    }
    uint2 A[25], hc[4];
    keccak_absorb_lanes_staged<SHA3_256_LANES>(A, reinterpret_cast<const uint2 *>(ct + (size_t)x * Pp::CTB), Pp::CTB / 8,
                                               DOM_SHA3, hstage, threadIdx.x, HASH_THREADS);
    keccak_f1600(A);
#pragma unroll
    for (int i = 0; i < 4; i++) hc[i] = A[i];
    const uint2 *kb = reinterpret_cast<const uint2 *>(scratch + (size_t)x * 96 + 64);
    keccak_zero(A);
#pragma unroll
    for (int i = 0; i < 4; i++) {
        A[i] = kb[i];
        A[4 + i] = hc[i];
    }
    A[8].x ^= DOM_SHAKE;
    A[SHAKE256_LANES - 1].y ^= 0x80000000u;
    keccak_f1600(A);
    uint2 *o = reinterpret_cast<uint2 *>(ss + (size_t)x * 32);
#pragma unroll
    for (int i = 0; i < 4; i++) o[i] = A[i];
}
// decaps prologue: H(c); ML-KEM: the rejection key J(z || c) = SHAKE256(z || c, 32)
template <int K, int V>
__global__ void __launch_bounds__(HASH_THREADS) kyber_dec_hash_pre(int n, const uint8_t *ct, const uint8_t *sk,
                                                                   uint8_t *hct, int kem) {
    using Pp = P<K, V>;
    KY_HASH_STAGE;
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= n) return;
    uint2 A[25];
    const uint2 *c = reinterpret_cast<const uint2 *>(ct + (size_t)x * Pp::CTB);
    if (kem == KEM_MLKEM)
        keccak_absorb_lanes2<SHAKE256_LANES>(A, reinterpret_cast<const uint2 *>(sk + (size_t)x * Pp::SKB + Pp::SKB - 32), 4,
                                             c, Pp::CTB / 8, DOM_SHAKE);
    else
        keccak_absorb_lanes_staged<SHA3_256_LANES>(A, c, Pp::CTB / 8, DOM_SHA3, hstage, threadIdx.x, HASH_THREADS);
    keccak_f1600(A);
    uint2 *o = reinterpret_cast<uint2 *>(hct + (size_t)x * 32);
#pragma unroll
    for (int i = 0; i < 4; i++) o[i] = A[i];
}
// decaps, between the two stages (large batches): (K-bar', r') = G(m' || h) with m' from the
// decryption stage and h = H(pk) from the secret key; mr = m' || r' || K-bar' per instance
template <int K, int V>
__global__ void __launch_bounds__(128) kyber_dec_hash_mid(int n, const uint8_t *sk, uint8_t *mr) {
    using Pp = P<K, V>;
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= n) return;
    uint2 *row = reinterpret_cast<uint2 *>(mr + (size_t)x * 96);
    const uint2 *h = reinterpret_cast<const uint2 *>(sk + (size_t)x * Pp::SKB + Pp::SKB - 64);
    uint2 A[25];
    keccak_zero(A);
#pragma unroll
    for (int i = 0; i < 4; i++) {
        A[i] = row[i];
        A[4 + i] = h[i];
    }
    A[8].x ^= DOM_SHA3;
    A[SHA3_512_LANES - 1].y ^= 0x80000000u;
    keccak_f1600(A);
#pragma unroll
    for (int i = 0; i < 4; i++) {
        row[4 + i] = A[4 + i];  // r'
        row[8 + i] = A[i];      // K-bar'
    }
}
// decaps epilogue (round-2 / round-3 KEM, large batches): ss = SHAKE256(key || H(c)), key being the
// constant-time selection (K-bar' or z) the re-encryption stage left in mr + 64
template <int K, int V>
__global__ void __launch_bounds__(128) kyber_dec_hash_post(int n, const uint8_t *mr, const uint8_t *hct, uint8_t *ss) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= n) return;
    const uint2 *key = reinterpret_cast<const uint2 *>(mr + (size_t)x * 96 + 64);
    const uint2 *hc = reinterpret_cast<const uint2 *>(hct + (size_t)x * 32);
    uint2 A[25];
    keccak_zero(A);
#pragma unroll
    for (int i = 0; i < 4; i++) {
        A[i] = key[i];
        A[4 + i] = hc[i];
    }
    A[8].x ^= DOM_SHAKE;
    A[SHAKE256_LANES - 1].y ^= 0x80000000u;
    keccak_f1600(A);
    uint2 *o = reinterpret_cast<uint2 *>(ss + (size_t)x * 32);
#pragma unroll
    for (int i = 0; i < 4; i++) o[i] = A[i];
}
// keypair prologue (large batches): (rho, sigma) = G(d) per instance into out (64 B each);
// ML-KEM: G(d || k)
template <int K, int V>
__global__ void __launch_bounds__(128) kyber_kp_hash_pre(int n, const uint8_t *coins, int coins_stride, int kem,
                                                         uint8_t *out) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= n) return;
    const uint2 *dd = reinterpret_cast<const uint2 *>(coins + (size_t)x * coins_stride);
    uint2 A[25];
    keccak_zero(A);
#pragma unroll
    for (int i = 0; i < 4; i++) A[i] = dd[i];
    A[4].x = kem == KEM_MLKEM ? ((uint32_t)K | (DOM_SHA3 << 8)) : DOM_SHA3;
    A[SHA3_512_LANES - 1].y ^= 0x80000000u;
    keccak_f1600(A);
    uint2 *o = reinterpret_cast<uint2 *>(out + (size_t)x * 64);
#pragma unroll
    for (int i = 0; i < 8; i++) o[i] = A[i];
}
// keypair epilogue: sk[SKB-64 .. SKB-32) = H(pk)
template <int K, int V>
__global__ void __launch_bounds__(HASH_THREADS) kyber_kp_hash_post(int n, const uint8_t *pk, uint8_t *sk) {
    using Pp = P<K, V>;
    KY_HASH_STAGE;
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= n) return;
    uint2 A[25];
    keccak_absorb_lanes_staged<SHA3_256_LANES>(A, reinterpret_cast<const uint2 *>(pk + (size_t)x * Pp::PKB), Pp::PKB / 8,
                                               DOM_SHA3, hstage, threadIdx.x, HASH_THREADS);
    keccak_f1600(A);
    uint2 *o = reinterpret_cast<uint2 *>(sk + (size_t)x * Pp::SKB + Pp::SKB - 64);
#pragma unroll
    for (int i = 0; i < 4; i++) o[i] = A[i];
}

// ---- the same serial hashes with one warp per instance: the latency path for small batches ----
// A thread-per-instance sponge of 9-11 permutations is a chain of ~50k dependent instructions; the
// 25-lane warp permutation (keccak.cuh) runs each permutation in about 60 % of the time, at ~7x the
// issue slots, so it is used while the batch is too small to fill the GPU (n <= warp_hash_max(),
// launch-shape op 5, default 2048).  Independently, keypair batches of at most KP_FUSED_MAX keep G(d)
// inside the core CTAs, and decapsulation batches of at most DEC_FUSED_MAX keep G and the KDF inside
// theirs (one launch fewer each).  Measured on GB300 (device buffers, fused -> split): Kyber-768
// decapsulation 103.6 -> 90.1 us at 512 instances and 109.9 -> 96.3 us at 1024 (Kyber-1024 108.8 ->
// 88.9 and 114.4 -> 96.5 us, Kyber-512 3 % faster), but keypair 93.5 -> 97.6 us at 512 (3-5 %
// slower for every k): the single-thread tails cost the decapsulation stages more than a launch.
constexpr int KP_FUSED_MAX = 1024;
constexpr int DEC_FUSED_MAX = 384;
#define KY_WARP_INSTANCE                                         \
    const int x = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;  \
    if (x >= n) return;                                          \
    const WarpKeccak w(threadIdx.x & 31)

template <int K, int V>
__global__ void __launch_bounds__(128) kyber_enc_hash_pre_w(int n, const uint8_t *pk, const uint8_t *coins,
                                                            uint8_t *scratch, int kem) {
    using Pp = P<K, V>;
    KY_WARP_INSTANCE;
    const uint2 *cn = reinterpret_cast<const uint2 *>(coins + (size_t)x * 32);
    uint2 m;
    if (kem == KEM_MLKEM) {
        m = w.lane < 4 ? cn[w.lane] : make_uint2(0, 0);
    } else {
        warp_absorb2<SHA3_256_LANES>(m, cn, 4, nullptr, 0, DOM_SHA3, w);
        keccak_f1600_warp(m, w);
    }
    uint2 h;
    warp_absorb2<SHA3_256_LANES>(h, reinterpret_cast<const uint2 *>(pk + (size_t)x * Pp::PKB), Pp::PKB / 8, nullptr, 0,
                                 DOM_SHA3, w);
    keccak_f1600_warp(h, w);
    const uint2 hs = shfl2(h, (w.lane - 4) & 31);
    uint2 g = w.lane < 4 ? m : (w.lane < 8 ? hs : make_uint2(0, 0));  // G(m || H(pk))
    if (w.lane == SHA3_512_LANES - 1) {
        g.x ^= DOM_SHA3;
        g.y ^= 0x80000000u;
    }
    keccak_f1600_warp(g, w);
    uint2 *o = reinterpret_cast<uint2 *>(scratch + (size_t)x * 96);
    if (w.lane < 4) {
        o[w.lane] = m;      // m
        o[8 + w.lane] = g;  // K-bar
    } else if (w.lane < 8) {
        o[w.lane] = g;  // r
    }
}
template <int K, int V>
__global__ void __launch_bounds__(128) kyber_enc_hash_post_w(int n, const uint8_t *ct, const uint8_t *scratch,
                                                             uint8_t *ss, int kem) {
    using Pp = P<K, V>;
    KY_WARP_INSTANCE;
    const uint2 *kb = reinterpret_cast<const uint2 *>(scratch + (size_t)x * 96 + 64);
    uint2 *o = reinterpret_cast<uint2 *>(ss + (size_t)x * 32);
    if (kem == KEM_MLKEM) {
        if (w.lane < 4) o[w.lane] = kb[w.lane];
        return;
    }
    uint2 h;
    warp_absorb2<SHA3_256_LANES>(h, reinterpret_cast<const uint2 *>(ct + (size_t)x * Pp::CTB), Pp::CTB / 8, nullptr, 0,
                                 DOM_SHA3, w);
    keccak_f1600_warp(h, w);
    const uint2 hs = shfl2(h, (w.lane - 4) & 31);
    uint2 a = w.lane < 4 ? kb[w.lane] : (w.lane < 8 ? hs : make_uint2(0, 0));  // KDF(K-bar || H(c))
    if (w.lane == 8) a.x ^= DOM_SHAKE;
    if (w.lane == SHAKE256_LANES - 1) a.y ^= 0x80000000u;
    keccak_f1600_warp(a, w);
    if (w.lane < 4) o[w.lane] = a;
}
template <int K, int V>
__global__ void __launch_bounds__(128) kyber_dec_hash_pre_w(int n, const uint8_t *ct, const uint8_t *sk, uint8_t *hct,
                                                            int kem) {
    using Pp = P<K, V>;
    KY_WARP_INSTANCE;
    const uint2 *c = reinterpret_cast<const uint2 *>(ct + (size_t)x * Pp::CTB);
    uint2 a;
    if (kem == KEM_MLKEM)
        warp_absorb2<SHAKE256_LANES>(a, reinterpret_cast<const uint2 *>(sk + (size_t)x * Pp::SKB + Pp::SKB - 32), 4, c,
                                     Pp::CTB / 8, DOM_SHAKE, w);
    else
        warp_absorb2<SHA3_256_LANES>(a, c, Pp::CTB / 8, nullptr, 0, DOM_SHA3, w);
    keccak_f1600_warp(a, w);
    if (w.lane < 4) reinterpret_cast<uint2 *>(hct + (size_t)x * 32)[w.lane] = a;
}
template <int K, int V>
__global__ void __launch_bounds__(128) kyber_kp_hash_post_w(int n, const uint8_t *pk, uint8_t *sk) {
    using Pp = P<K, V>;
    KY_WARP_INSTANCE;
    uint2 a;
    warp_absorb2<SHA3_256_LANES>(a, reinterpret_cast<const uint2 *>(pk + (size_t)x * Pp::PKB), Pp::PKB / 8, nullptr, 0,
                                 DOM_SHA3, w);
    keccak_f1600_warp(a, w);
    if (w.lane < 4) reinterpret_cast<uint2 *>(sk + (size_t)x * Pp::SKB + Pp::SKB - 64)[w.lane] = a;
}
#undef KY_WARP_INSTANCE

}  // namespace kyber
}  // namespace pqc
#include "kyber_single.cuh"
#include "kyber_plain.cuh"
namespace pqc {
namespace kyber {
// ---------------------------------------------------------------------------------------------
// Host launchers
// ---------------------------------------------------------------------------------------------
extern LaunchShape g_shape[3][3];  // [op][k-2]: instances per CTA, threads per CTA (kyber.cu)
extern LaunchShape g_dec1[3];      // [k-2]: the same for the decapsulation's decryption stage
extern LaunchShape g_warp_hash;    // batches of at most this many instances take the warp hash kernels
extern LaunchShape g_single[3][3];  // [k-2][op]: KEM batches of at most this many instances take
                                    // the single-instance kernels (count field; kyber.cu)

static inline int warp_hash_max() {
    int a, b;
    g_warp_hash.get(a, b);
    return a;
}
static inline int single_max(int k, int op) {
    int a, b;
    g_single[k - 2][op].get(a, b);
    return a;
}

// Every Kyber kernel asks for the largest shared-memory carveout of the SM's unified L1 / shared
// storage.  Kernels that run concurrently (the chunks of a host-buffer call, the jobs of a mixed
// batch, serving slots) then share one SM configuration: a hash kernel's CTAs, which need no shared
// memory, do not leave an SM configured with too little shared memory for a core kernel's CTAs.
template <class Kern>
static void prefer_shared(Kern kern) {
    if (cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout, (int)cudaSharedmemCarveoutMaxShared) !=
        cudaSuccess)
        cudaGetLastError();
}
template <int K, int V>
static void prefer_shared_all() {
    prefer_shared(kyber_enc_core<K, V>);
    prefer_shared(kyber_dec_core<K, V, DEC_FUSED>);
    prefer_shared(kyber_dec_decrypt<K, V>);
    prefer_shared(kyber_dec_core<K, V, DEC_REENCRYPT>);
    prefer_shared(kyber_kp_core<K, V>);
    prefer_shared(kyber_enc_hash_pre<K, V>);
    prefer_shared(kyber_enc_hash_post<K, V>);
    prefer_shared(kyber_dec_hash_pre<K, V>);
    prefer_shared(kyber_kp_hash_post<K, V>);
    prefer_shared(kyber_kp_hash_pre<K, V>);
    prefer_shared(kyber_dec_hash_mid<K, V>);
    prefer_shared(kyber_dec_hash_post<K, V>);
    prefer_shared(kyber_enc_hash_pre_w<K, V>);
    prefer_shared(kyber_enc_hash_post_w<K, V>);
    prefer_shared(kyber_dec_hash_pre_w<K, V>);
    prefer_shared(kyber_kp_hash_post_w<K, V>);
    prefer_shared(kyber_kp_single<K, V>);
    prefer_shared(kyber_enc_single<K, V>);
    prefer_shared(kyber_dec_single<K, V>);
}

template <class Kern>
static cudaError_t ensure_smem(Kern kern, size_t bytes) {
    if (capturing()) return cudaSuccess;  // set by the uncaptured warm-up pass
    const cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
    if (e != cudaSuccess) cudaGetLastError();  // leave no error behind for the caller's next CUDA call
    return e;
}

// Dynamic shared memory of the core kernel of `op` (0 keypair, 1 encaps, 2 decaps) at a launch shape.
template <int K, int V>
static size_t core_smem_bytes(int op, int ni, int threads) {
    return op == 0 ? Layout<3 * K, 128>::bytes(ni, threads) : Layout<2 * K + 1, enc_seed_bytes<K, V>()>::bytes(ni, threads);
}

template <int K, int V>
static int launch_keypair(int n, uint8_t *pk, uint8_t *sk, const uint8_t *coins, int coins_stride, int kem,
                          uint8_t *scratch, int plain, cudaStream_t st) {
    if (plain) return kem == KEM_FO ? plain_keypair<K, V>(n, pk, sk, coins, coins_stride, scratch, st) : PQCGPU_EUNSUPPORTED;
    if (kem && n <= single_max(K, 0)) {
        PQC_LAUNCH(st, "kyber_kp_single", K, V,
                   kyber_kp_single<K, V><<<n, SINGLE_THREADS, SingleSmem<K, V>::bytes(), st>>>(coins, coins_stride, pk, sk,
                                                                                              kem));
        return cudaGetLastError() == cudaSuccess ? PQCGPU_OK : PQCGPU_ECUDA;
    }
    int NI, NT;
    g_shape[0][K - 2].get(NI, NT);
    const size_t sm = Layout<3 * K, 128>::bytes(NI, NT);
    if (ensure_smem(kyber_kp_core<K, V>, sm) != cudaSuccess) return PQCGPU_ECUDA;
    const bool g_pre = scratch && n > KP_FUSED_MAX;  // G as its own kernel (scratch: 64 B per instance)
    KpArgs a{n, pk, sk, coins, coins_stride, kem, g_pre ? scratch : nullptr};
    if (g_pre)
        PQC_LAUNCH(st, "kyber_kp_hash_pre", K, V,
                   kyber_kp_hash_pre<K, V><<<(n + 127) / 128, 128, 0, st>>>(n, coins, coins_stride, kem, scratch));
    PQC_LAUNCH(st, "kyber_kp_core", K, V, kyber_kp_core<K, V><<<(n + NI - 1) / NI, NT, sm, st>>>(a, NI));
    if (kem && n <= warp_hash_max())
        PQC_LAUNCH(st, "kyber_kp_hash_post", K, V, kyber_kp_hash_post_w<K, V><<<(n + 3) / 4, 128, 0, st>>>(n, pk, sk));
    else if (kem)
        PQC_LAUNCH(st, "kyber_kp_hash_post", K, V, kyber_kp_hash_post<K, V><<<(n + 127) / 128, 128, 0, st>>>(n, pk, sk));
    return cudaGetLastError() == cudaSuccess ? PQCGPU_OK : PQCGPU_ECUDA;
}

template <int K, int V>
static int launch_enc(int n, uint8_t *ct, uint8_t *ss, const uint8_t *pk, const uint8_t *m, const uint8_t *coins,
                      uint8_t *scratch, int kem, int plain, cudaStream_t st) {
    if (plain) return kem == KEM_FO ? plain_enc<K, V>(n, ct, ss, pk, coins, scratch, st) : PQCGPU_EUNSUPPORTED;
    if (kem && n <= single_max(K, 1)) {
        PQC_LAUNCH(st, "kyber_enc_single", K, V,
                   kyber_enc_single<K, V><<<n, SINGLE_THREADS, SingleSmem<K, V>::bytes(), st>>>(pk, coins, ct, ss, kem));
        return cudaGetLastError() == cudaSuccess ? PQCGPU_OK : PQCGPU_ECUDA;
    }
    int NI, NT;
    g_shape[1][K - 2].get(NI, NT);
    const size_t sm = Layout<2 * K + 1, enc_seed_bytes<K, V>()>::bytes(NI, NT);
    if (ensure_smem(kyber_enc_core<K, V>, sm) != cudaSuccess) return PQCGPU_ECUDA;
    EncArgs a;
    a.n = n;
    a.ct = ct;
    a.pk = pk;
    a.pk_stride = P<K, V>::PKB;
    if (kem) {
        if (n <= warp_hash_max())
            PQC_LAUNCH(st, "kyber_enc_hash_pre", K, V,
                       kyber_enc_hash_pre_w<K, V><<<(n + 3) / 4, 128, 0, st>>>(n, pk, coins, scratch, kem));
        else
            PQC_LAUNCH(st, "kyber_enc_hash_pre", K, V,
                       kyber_enc_hash_pre<K, V><<<(n + 127) / 128, 128, 0, st>>>(n, pk, coins, scratch, kem));
        a.m = scratch;
        a.m_stride = 96;
        a.r = scratch + 32;
        a.r_stride = 96;
    } else {
        a.m = m;
        a.m_stride = 32;
        a.r = coins;
        a.r_stride = 32;
    }
    PQC_LAUNCH(st, "kyber_enc_core", K, V, kyber_enc_core<K, V><<<(n + NI - 1) / NI, NT, sm, st>>>(a, NI));
    if (kem) {
        if (n <= warp_hash_max())
            PQC_LAUNCH(st, "kyber_enc_hash_post", K, V,
                       kyber_enc_hash_post_w<K, V><<<(n + 3) / 4, 128, 0, st>>>(n, ct, scratch, ss, kem));
        else
            PQC_LAUNCH(st, "kyber_enc_hash_post", K, V,
                       kyber_enc_hash_post<K, V><<<(n + 127) / 128, 128, 0, st>>>(n, ct, scratch, ss, kem));
    }
    return cudaGetLastError() == cudaSuccess ? PQCGPU_OK : PQCGPU_ECUDA;
}

template <int K, int V>
static int launch_dec(int n, uint8_t *out, const uint8_t *ct, const uint8_t *sk, uint8_t *scratch, int kem,
                      int plain, cudaStream_t st) {
    if (plain) return kem == KEM_FO ? plain_dec<K, V>(n, out, ct, sk, scratch, st) : PQCGPU_EUNSUPPORTED;
    if (kem && n <= single_max(K, 2)) {
        PQC_LAUNCH(st, "kyber_dec_single", K, V,
                   kyber_dec_single<K, V><<<n, SINGLE_THREADS, SingleSmem<K, V>::bytes(), st>>>(ct, sk, out, kem));
        return cudaGetLastError() == cudaSuccess ? PQCGPU_OK : PQCGPU_ECUDA;
    }
    int NI, NT;
    g_shape[2][K - 2].get(NI, NT);
    const size_t sm = Layout<2 * K + 1, enc_seed_bytes<K, V>()>::bytes(NI, NT);
    DecArgs d;
    d.n = n;
    d.ct = ct;
    d.sk = sk;
    d.m_out = kem ? nullptr : out;
    d.ss = kem ? out : nullptr;
    d.hct = scratch;
    d.kem = kem;
    d.mr = scratch + (size_t)n * 32;
    d.kdf_post = (kem == KEM_FO && n > DEC_FUSED_MAX) ? 1 : 0;
    d.g_post = (kem && n > DEC_FUSED_MAX) ? 1 : 0;
    if (!kem) {
        if (ensure_smem(kyber_dec_core<K, V, DEC_FUSED>, sm) != cudaSuccess) return PQCGPU_ECUDA;
        PQC_LAUNCH(st, "kyber_dec_core", K, V,
                   kyber_dec_core<K, V, DEC_FUSED><<<(n + NI - 1) / NI, NT, sm, st>>>(d, NI));
        return cudaGetLastError() == cudaSuccess ? PQCGPU_OK : PQCGPU_ECUDA;
    }
    // With the KDF after the re-encryption stage (round-2 / round-3 KEM, batches above
    // DEC_FUSED_MAX), H(c)
    // is needed only by kyber_dec_hash_post: it runs on a side stream beside the decryption and
    // re-encryption stages, whose integer pipe it shares.
    SideStream *side = d.kdf_post ? side_stream() : nullptr;
    if (side && (cudaEventRecord(side->fork, st) != cudaSuccess || cudaStreamWaitEvent(side->s, side->fork, 0) != cudaSuccess)) {
        cudaGetLastError();
        side = nullptr;
    }
    const cudaStream_t hs = side ? side->s : st;
    if (n <= warp_hash_max())
        PQC_LAUNCH(hs, "kyber_dec_hash_pre", K, V,
                   kyber_dec_hash_pre_w<K, V><<<(n + 3) / 4, 128, 0, hs>>>(n, ct, sk, scratch, kem));
    else
        PQC_LAUNCH(hs, "kyber_dec_hash_pre", K, V,
                   kyber_dec_hash_pre<K, V><<<(n + 127) / 128, 128, 0, hs>>>(n, ct, sk, scratch, kem));
    int NI1, NT1;
    g_dec1[K - 2].get(NI1, NT1);
    const size_t sm1 = Layout<2 * K + 1, enc_seed_bytes<K, V>()>::bytes(NI1, 0);
    if (ensure_smem(kyber_dec_decrypt<K, V>, sm1) != cudaSuccess) return PQCGPU_ECUDA;
    if (ensure_smem(kyber_dec_core<K, V, DEC_REENCRYPT>, sm) != cudaSuccess) return PQCGPU_ECUDA;
    PQC_LAUNCH(st, "kyber_dec_decrypt", K, V,
               kyber_dec_decrypt<K, V><<<(n + NI1 - 1) / NI1, NT1, sm1, st>>>(d, NI1));
    if (d.g_post)
        PQC_LAUNCH(st, "kyber_dec_hash_mid", K, V,
                   kyber_dec_hash_mid<K, V><<<(n + 127) / 128, 128, 0, st>>>(n, d.sk, d.mr));
    PQC_LAUNCH(st, "kyber_dec_reencrypt", K, V,
               kyber_dec_core<K, V, DEC_REENCRYPT><<<(n + NI - 1) / NI, NT, sm, st>>>(d, NI));
    if (side && (cudaEventRecord(side->join, side->s) != cudaSuccess || cudaStreamWaitEvent(st, side->join, 0) != cudaSuccess))
        return PQCGPU_ECUDA;
    if (d.kdf_post)
        PQC_LAUNCH(st, "kyber_dec_hash_post", K, V,
                   kyber_dec_hash_post<K, V><<<(n + 127) / 128, 128, 0, st>>>(n, d.mr, d.hct, d.ss));
    return cudaGetLastError() == cudaSuccess ? PQCGPU_OK : PQCGPU_ECUDA;
}

}  // namespace kyber
}  // namespace pqc

// One translation unit per (K, V) instantiates the kernels and exports these entry points.
#define PQC_KYBER_INSTANTIATE(K, V)                                                                        \
    namespace pqc {                                                                                        \
    namespace kyber {                                                                                      \
    int keypair_##K##_##V(int n, uint8_t *pk, uint8_t *sk, const uint8_t *coins, int cs, int kem,         \
                          uint8_t *scratch, int plain, cudaStream_t st) {                                  \
        return launch_keypair<K, V>(n, pk, sk, coins, cs, kem, scratch, plain, st);                       \
    }                                                                                                      \
    int enc_##K##_##V(int n, uint8_t *ct, uint8_t *ss, const uint8_t *pk, const uint8_t *m,               \
                      const uint8_t *coins, uint8_t *scratch, int kem, int plain, cudaStream_t st) {       \
        return launch_enc<K, V>(n, ct, ss, pk, m, coins, scratch, kem, plain, st);                        \
    }                                                                                                      \
    int dec_##K##_##V(int n, uint8_t *out, const uint8_t *ct, const uint8_t *sk, uint8_t *scratch, int kem, \
                      int plain, cudaStream_t st) {                                                        \
        return launch_dec<K, V>(n, out, ct, sk, scratch, kem, plain, st);                                 \
    }                                                                                                      \
    size_t smem_##K##_##V(int op, int ni, int threads) { return core_smem_bytes<K, V>(op, ni, threads); }     \
    int init_##K##_##V() {                                                                                 \
        uint2 rc[24];                                                                                      \
        keccak_rc_host(rc);                                                                                \
        int16_t z[128], zi[128];                                                                           \
        kyber_twiddles_host(z, zi);                                                                        \
        if (cudaMemcpyToSymbol(c_keccak_rc, rc, sizeof rc) != cudaSuccess) return PQCGPU_ECUDA;           \
        if (cudaMemcpyToSymbol(c_zetas, z, sizeof z) != cudaSuccess) return PQCGPU_ECUDA;                 \
        if (cudaMemcpyToSymbol(c_zetas_inv, zi, sizeof zi) != cudaSuccess) return PQCGPU_ECUDA;           \
        int2 tw[128], twi[128];                                                                            \
        kyber_twiddles_shoup_host(tw, twi);                                                                \
        if (cudaMemcpyToSymbol(c_tw, tw, sizeof tw) != cudaSuccess) return PQCGPU_ECUDA;                  \
        if (cudaMemcpyToSymbol(c_twi, twi, sizeof twi) != cudaSuccess) return PQCGPU_ECUDA;               \
        prefer_shared_all<K, V>();                                                                         \
        return PQCGPU_OK;                                                                                  \
    }                                                                                                      \
    }                                                                                                      \
    }
