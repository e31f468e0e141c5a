// Batched FrodoKEM-640 / 976 / 1344 (SHAKE) for sm_103a.
//
// Replaces crypto_kem_keypair_gpu / enc / dec (FrodoKEM_GPU/frodo976.cu:87-690: one instance per
// call, A written to and re-read from HBM, host SHAKE for pk / ct) with, per operation:
//   * a warp-per-instance kernel for the serial sponges -- the S/E noise stream
//     (SHAKE(0x5F / 0x96 || seedSE), 230-231 permutations for n = 976), G1 = SHAKE(pk) (115), G2
//     and the final F = SHAKE(ct || k) (116) -- with the Keccak state spread over the warp to cut
//     the latency of these chains, the noise sampled with the CDF table on the fly;
//   * a core kernel that regenerates A row by row from SHAKE128(le16(i) || seedA) and multiplies
//     it as it appears, so A (1.9 MB per key) never exists in HBM or whole in shared memory:
//       - keypair, B = A S + E: one thread per row, which owns the 8 outputs of that row;
//       - encaps / decaps, B' = S' A + E': each thread squeezes one 168-byte block of its row per
//         round into shared memory, then the CTA contracts the staged 84 columns over its rows
//         (exact mod 2^16 with uint32 multiply-accumulate) and adds the partial sums into the
//         8 x 976 accumulator with shared-memory atomics;
//   * codecs (log q-bit MSB-first pack, B-bit key encode / decode) inside the same kernels.
// Host flow and arithmetic follow FrodoKEM_GPU/kem.c:13-214, frodo_macrify_reference.cu:55-360,
// util.cu:18-113, noise.c:10-29 and the CDF table of frodo976.cu:21.  The reference builds only
// n = 976 (FrodoKEM_GPU/params.h:17-30); FrodoKEM-640 and -1344 run the same flow with the other
// parameter sets of the FrodoKEM specification: n, log q (15 for 640), B (2 / 3 / 4 encoded bits),
// 16 / 24 / 32-byte seeds and keys, SHAKE128 (640) or SHAKE256 (976, 1344) for every hash and for
// the noise stream, and their CDF tables.  Every value is computed mod 2^16 and reduced mod q when
// packed, compared or decoded.
#include <cuda_fp16.h>

#include <algorithm>
#include <vector>
#include <cuda_runtime.h>
#include <stdint.h>

#include "keccak.cuh"
#include "pqcgpu_internal.h"

namespace pqc {
namespace frodo {

constexpr int NB = 8, SEEDA = 16;

// Parameter set with n = N: LOGQ bits per value, B encoded bits, SSB = length of s, seedSE, k, pkh
// and ss (= MUB, the length of mu), RATE = Keccak rate in 64-bit lanes of the hash (SHAKE128 for
// n = 640, SHAKE256 otherwise), CDF table length.
template <int N>
struct FP {
    static constexpr int LOGQ = N == 640 ? 15 : 16, B = N == 640 ? 2 : N == 976 ? 3 : 4;
    static constexpr int SSB = 8 * B, MUB = 8 * B, NW = SSB / 8;
    static constexpr int RATE = N == 640 ? SHAKE128_LANES : SHAKE256_LANES;
    static constexpr int CDF_LEN = N == 640 ? 13 : N == 976 ? 11 : 7;
    static constexpr uint32_t MASKQ = (1u << LOGQ) - 1;
    static constexpr int C1B = LOGQ * N * NB / 8;   // packed N x NBAR (or NBAR x N) matrix
    static constexpr int C2B = LOGQ * NB * NB / 8;  // packed NBAR x NBAR matrix
    static constexpr int PKB = SEEDA + C1B, CTB = C1B + C2B, SKB = SSB + PKB + 2 * N * NB + SSB;
    static constexpr int ROW_BLOCKS = (2 * N + 167) / 168;  // SHAKE128 blocks per row of A
    // scratch per instance: noise (Sp, Ep: N x 8, Epp: 8 x 8 u16) + seeds (k at +0, mu at +32,
    // fail flag at +64, the F key at +72), then the u32 accumulator of B' (8 x N) used when the
    // rows of A are split over several CTAs
    static constexpr int NOISE_U16 = 2 * N * NB + NB * NB;
    static constexpr size_t GACC_OFF = (size_t)NOISE_U16 * 2 + 128;
    static constexpr size_t SCRATCH = GACC_OFF + (size_t)NB * N * 4;
};
static_assert(FP<976>::PKB == 15632 && FP<976>::SKB == 31296 && FP<976>::CTB == 15744, "FrodoKEM-976 sizes");
static_assert(FP<640>::PKB == 9616 && FP<640>::SKB == 19888 && FP<640>::CTB == 9720, "FrodoKEM-640 sizes");
static_assert(FP<1344>::PKB == 21520 && FP<1344>::SKB == 43088 && FP<1344>::CTB == 21632, "FrodoKEM-1344 sizes");

static __constant__ uint16_t c_cdf640[13], c_cdf976[11], c_cdf1344[7];

// ---- helpers ---------------------------------------------------------------------------------
// CDF sampler of one 16-bit value (noise.c:10-29)
template <int N>
__device__ __forceinline__ uint16_t cdf_sample(uint32_t r) {
    const uint16_t *cdf = N == 640 ? c_cdf640 : N == 976 ? c_cdf976 : c_cdf1344;
    uint32_t sample = 0;
    const uint32_t prnd = (r & 0xffff) >> 1, sign = r & 1;
#pragma unroll
    for (int j = 0; j < FP<N>::CDF_LEN - 1; j++) sample += ((uint32_t)cdf[j] - prnd) >> 31 & 1;
    return (uint16_t)((((0u - sign) ^ sample) + sign) & 0xffff);
}

// Pack / unpack of 8 consecutive values (util.cu:18-113, MSB first): LOGQ bytes.  For LOGQ = 16
// this is big-endian u16.
template <int LOGQ>
__device__ __forceinline__ void pack8(uint8_t *o, const uint32_t (&v)[8]) {
    if (LOGQ == 16) {
#pragma unroll
        for (int k = 0; k < 8; k++) {
            o[2 * k] = (uint8_t)(v[k] >> 8);
            o[2 * k + 1] = (uint8_t)v[k];
        }
    } else {
        uint64_t hi = 0, lo = 0;  // 8 x LOGQ <= 128 bits, value 0 first (most significant)
#pragma unroll
        for (int k = 0; k < 8; k++) {
            const uint64_t x = v[k] & ((1u << LOGQ) - 1);
            hi = (hi << LOGQ) | (lo >> (64 - LOGQ));
            lo = (lo << LOGQ) | x;
        }
        // 8 * LOGQ bits, left-aligned at bit 8*LOGQ - 1 of (hi:lo)
#pragma unroll
        for (int b = 0; b < LOGQ; b++) {
            const int sh = 8 * (LOGQ - 1 - b);  // bit offset of byte b from the right
            o[b] = (uint8_t)(sh >= 64 ? (hi >> (sh - 64)) : ((lo >> sh) | (sh > 0 ? (hi << (64 - sh)) : 0)));
        }
    }
}
// value k (0..7) of the 8-value group packed at p
template <int LOGQ>
__device__ __forceinline__ uint32_t unpack_at(const uint8_t *p, int k) {
    if (LOGQ == 16) return ((uint32_t)p[2 * k] << 8) | p[2 * k + 1];
    const int bit = LOGQ * k, byte = bit >> 3, off = bit & 7;  // MSB-first bit offset
    const uint32_t w = ((uint32_t)p[byte] << 16) | ((uint32_t)p[byte + 1] << 8) | (byte + 2 < LOGQ ? p[byte + 2] : 0u);
    return (w >> (24 - off - LOGQ)) & ((1u << LOGQ) - 1);
}

// SHAKE128 row generator for A: absorb le16(row) || seedA, squeeze block by block.
__device__ __forceinline__ void row_absorb(uint2 (&A)[25], int row, const uint2 *seedA) {
    keccak_zero(A);
    // bytes: row_lo row_hi seedA[0..15] -> lanes
    const uint2 s0 = seedA[0], s1 = seedA[1];
    A[0] = make_uint2((uint32_t)(row & 0xffff) | (s0.x << 16), (s0.x >> 16) | (s0.y << 16));
    A[1] = make_uint2((s0.y >> 16) | (s1.x << 16), (s1.x >> 16) | (s1.y << 16));
    A[2] = make_uint2((s1.y >> 16) | (DOM_SHAKE << 16), 0);
    A[SHAKE128_LANES - 1].y ^= 0x80000000u;
}

// element e of a packed matrix (8-value groups of LOGQ bytes)
template <int LOGQ>
__device__ __forceinline__ uint32_t ld_packed(const uint8_t *base, int e) {
    return unpack_at<LOGQ>(base + (size_t)LOGQ * (e >> 3), e & 7);
}

// ---------------------------------------------------------------------------------------------
// Serial sponges: one warp per instance (warp-cooperative Keccak, keccak.cuh)
// ---------------------------------------------------------------------------------------------
// Message lane m of prefix || seed (1 + 8 NW bytes) followed by the SHAKE domain byte, where the
// seed is given as NW little-endian 64-bit words (lane m < NW holds seed word m shifted by a byte).
template <int NW>
__device__ __forceinline__ uint2 prefixed_lane(int m, uint32_t prefix, const uint64_t (&s)[NW]) {
    uint64_t v = m == 0 ? prefix : 0;
#pragma unroll
    for (int i = 0; i < NW; i++) {
        if (m == i) v |= s[i] << 8;
        if (m == i + 1) v |= s[i] >> 56;
    }
    if (m == NW) v |= (uint64_t)DOM_SHAKE << 8;
    return make_uint2((uint32_t)v, (uint32_t)(v >> 32));
}
__device__ __forceinline__ uint64_t u64(uint2 v) { return (uint64_t)v.x | ((uint64_t)v.y << 32); }

// State absorbing prefix || seed (one block, not yet permuted).
template <int N>
__device__ __forceinline__ uint2 seeded_state(uint32_t prefix, const uint64_t (&s)[FP<N>::NW], const WarpKeccak &w) {
    uint2 a = w.lane <= FP<N>::NW ? prefixed_lane<FP<N>::NW>(w.lane, prefix, s) : make_uint2(0, 0);
    if (w.lane == FP<N>::RATE - 1) a.y ^= 0x80000000u;
    return a;
}

// Squeeze the noise stream (state absorbed, not permuted): lanes 0..RATE-1 hold 4 u16 values each
// per block; value at stream position p is CDF-sampled and handed to emit(p, v).
template <int N, class F>
__device__ __forceinline__ void warp_noise_stream(uint2 &a, int count, const WarpKeccak &w, F emit) {
    constexpr int R = FP<N>::RATE;
    for (int base = 0; base < count; base += 4 * R) {
        keccak_f1600_warp(a, w);
        if (w.lane < R) {
#pragma unroll
            for (int q = 0; q < 4; q++) {
                const int p = base + 4 * w.lane + q;
                const uint32_t word = q < 2 ? a.x : a.y;
                if (p < count) emit(p, cdf_sample<N>((word >> (16 * (q & 1))) & 0xffff));
            }
        }
    }
}

template <int N>
__device__ __forceinline__ void write_spt(uint8_t *scr, int p, uint16_t v) {
    uint16_t *Spt = reinterpret_cast<uint16_t *>(scr), *Ep = Spt + N * NB, *Epp = Ep + N * NB;
    if (p < N * NB) Spt[(p % N) * NB + p / N] = v;  // stream S'[i*N + k] -> Spt[k*8 + i]
    else if (p < 2 * N * NB) Ep[p - N * NB] = v;
    else Epp[p - 2 * N * NB] = v;
}

#define FR_WARP_INSTANCE                                         \
    const int x = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;  \
    if (x >= n) return;                                          \
    const WarpKeccak w(threadIdx.x & 31)

// keypair: seedA = SHAKE(z, 16) -> pk[0..16); S (as St[j][k], N x 8) and E (N x 8) -> scratch
template <int N>
__global__ void __launch_bounds__(128) fr_kp_pre(int n, const uint8_t *coins, int cstride, uint8_t *pk, uint8_t *scratch) {
    using P = FP<N>;
    FR_WARP_INSTANCE;
    const uint8_t *c = coins + (size_t)x * cstride;  // s(SSB) || seedSE(SSB) || z(16)
    uint2 a;
    warp_absorb2<P::RATE>(a, reinterpret_cast<const uint2 *>(c + 2 * P::SSB), 2, nullptr, 0, DOM_SHAKE, w);
    keccak_f1600_warp(a, w);
    if (w.lane < 2) reinterpret_cast<uint2 *>(pk + (size_t)x * P::PKB)[w.lane] = a;
    const uint64_t *sd = reinterpret_cast<const uint64_t *>(c + P::SSB);
    uint64_t seed[P::NW];
#pragma unroll
    for (int i = 0; i < P::NW; i++) seed[i] = sd[i];
    a = seeded_state<N>(0x5F, seed, w);
    uint16_t *St = reinterpret_cast<uint16_t *>(scratch + (size_t)x * P::SCRATCH), *E = St + N * NB;
    // stream order: S[k*N + j] (k < 8, j < N) then E[i*8 + k]
    warp_noise_stream<N>(a, 2 * N * NB, w, [&](int p, uint16_t v) {
        if (p < N * NB) St[(p % N) * NB + p / N] = v;
        else E[p - N * NB] = v;
    });
}

// G2(pkh || mu) with pkh in lanes 0..NW-1 of `a`, mu at `mu`; then the S' / E' / E'' noise stream.
// Writes k (SSB bytes) and mu (MUB bytes) into the scratch seed area.
template <int N>
__device__ __forceinline__ void g2_and_noise(uint2 a, const uint8_t *mu, uint8_t *scr, const WarpKeccak &w) {
    using P = FP<N>;
    constexpr int NW = P::NW;
    const uint2 *m = reinterpret_cast<const uint2 *>(mu);
    uint2 g = w.lane < NW ? a : (w.lane < 2 * NW ? m[w.lane - NW] : make_uint2(0, 0));
    if (w.lane == 2 * NW) g.x ^= DOM_SHAKE;
    if (w.lane == P::RATE - 1) g.y ^= 0x80000000u;
    keccak_f1600_warp(g, w);
    uint2 *kk = reinterpret_cast<uint2 *>(scr + P::NOISE_U16 * 2), *mm = reinterpret_cast<uint2 *>(scr + P::NOISE_U16 * 2 + 32);
    if (w.lane >= NW && w.lane < 2 * NW) kk[w.lane - NW] = g;
    const uint2 mv = w.lane < NW ? m[w.lane] : make_uint2(0, 0);
    __syncwarp();
    if (w.lane < NW && mu != scr + P::NOISE_U16 * 2 + 32) mm[w.lane] = mv;
    uint64_t seed[NW];
#pragma unroll
    for (int i = 0; i < NW; i++) seed[i] = u64(shfl2(g, i));
    uint2 st = seeded_state<N>(0x96, seed, w);
    warp_noise_stream<N>(st, P::NOISE_U16, w, [&](int p, uint16_t v) { write_spt<N>(scr, p, v); });
}

// encaps prologue: pkh = G1(pk); (seedSE || k) = G2(pkh || mu); S', E', E'' sampled -> scratch.
// scratch: Spt (N x 8: Spt[k][i] = S'[i][k]), Ep (8 x N), Epp (8 x 8), then k (24) at +NOISE*2,
// mu (24) at +NOISE*2 + 32.
template <int N>
__device__ __forceinline__ void zero_gacc(uint8_t *scr, int lane) {
    uint4 *g = reinterpret_cast<uint4 *>(scr + FP<N>::GACC_OFF);
    for (int i = lane; i < NB * N / 4; i += 32) g[i] = make_uint4(0, 0, 0, 0);
}

// pkh != nullptr: pkh = SHAKE(pk, SSB) is given (the tail of a resident secret key, SSB bytes at
// pkh + x * pkh_stride; stride 0 when every instance encapsulates to one key), which skips the
// serial permutations of hashing the public key.
template <int N>
__global__ void __launch_bounds__(128) fr_enc_pre(int n, const uint8_t *pk, const uint8_t *mu, uint8_t *scratch,
                                                  int split, const uint8_t *pkh, int pkh_stride) {
    using P = FP<N>;
    FR_WARP_INSTANCE;
    if (split > 1) zero_gacc<N>(scratch + (size_t)x * P::SCRATCH, w.lane);
    uint2 a;
    if (pkh) {
        const uint2 *h = reinterpret_cast<const uint2 *>(pkh + (size_t)x * pkh_stride);
        a = w.lane < P::NW ? h[w.lane] : make_uint2(0, 0);
    } else {
        warp_absorb2<P::RATE>(a, reinterpret_cast<const uint2 *>(pk + (size_t)x * P::PKB), P::PKB / 8, nullptr, 0,
                              DOM_SHAKE, w);
        keccak_f1600_warp(a, w);
    }
    g2_and_noise<N>(a, mu + (size_t)x * P::MUB, scratch + (size_t)x * P::SCRATCH, w);
}

// decaps, step 1 (CTA per instance): W = C - B' S (frodo_mul_bs + frodo_sub), mu' = decode(W)
// -> scratch mu' slot.  B' and S are staged in shared memory with coalesced loads.
template <int N>
__global__ void __launch_bounds__(256) fr_dec_w(int n, const uint8_t *ct, const uint8_t *sk, uint8_t *scratch) {
    using P = FP<N>;
    constexpr int LOGQ = P::LOGQ, B = P::B;
    __shared__ __align__(16) uint16_t Bp[NB * N];
    __shared__ __align__(16) uint16_t S[NB * N];
    __shared__ uint32_t W[64];
    const int x = blockIdx.x, tid = threadIdx.x;
    const uint8_t *c = ct + (size_t)x * P::CTB, *sS = sk + (size_t)x * P::SKB + P::SSB + P::PKB;
    for (int e = tid; e < NB * N; e += blockDim.x) {
        Bp[e] = (uint16_t)ld_packed<LOGQ>(c, e);
        S[e] = (uint16_t)(sS[2 * e] | (sS[2 * e + 1] << 8));
    }
    if (tid < 64) W[tid] = 0;
    __syncthreads();
    // W[i][j] = sum_k Bp[i][k] S[j][k]: 4 threads per output, k interleaved
    {
        const int o = tid & 63, part = tid >> 6, i = o >> 3, j = o & 7;
        uint32_t sum = 0;
        for (int k = part; k < N; k += 4) sum += (uint32_t)Bp[i * N + k] * S[j * N + k];
        atomicAdd(&W[o], sum);
    }
    __syncthreads();
    if (tid < 8) {  // word g = tid: 8 pieces of B bits (key_decode)
        const int g = tid;
        uint32_t templong = 0;
        for (int jj = 0; jj < 8; jj++) {
            const uint32_t wv = (ld_packed<LOGQ>(c + P::C1B, g * NB + jj) - W[g * NB + jj]) & P::MASKQ;
            const uint32_t t = (wv + (1u << (LOGQ - B - 1))) >> (LOGQ - B);
            templong |= (t & ((1u << B) - 1)) << (B * jj);
        }
        uint8_t *mu = scratch + (size_t)x * P::SCRATCH + P::NOISE_U16 * 2 + 32;
#pragma unroll
        for (int b = 0; b < B; b++) mu[B * g + b] = (uint8_t)(templong >> (8 * b));
    }
}

// decaps, step 2 (warp per instance): (seedSE' || k') = G2(pkh || mu'); S', E', E'' -> scratch
template <int N>
__global__ void __launch_bounds__(128) fr_dec_pre(int n, const uint8_t *sk, uint8_t *scratch, int split) {
    using P = FP<N>;
    FR_WARP_INSTANCE;
    uint8_t *scr = scratch + (size_t)x * P::SCRATCH;
    if (split > 1) zero_gacc<N>(scr, w.lane);
    const uint2 *pkh = reinterpret_cast<const uint2 *>(sk + (size_t)x * P::SKB + P::SSB + P::PKB + 2 * N * NB);
    const uint2 a = w.lane < P::NW ? pkh[w.lane] : make_uint2(0, 0);
    g2_and_noise<N>(a, scr + P::NOISE_U16 * 2 + 32, scr, w);
}

// F = SHAKE(ct || key, SSB): encaps key = k; decaps key = fail ? s : k' (constant-time select)
template <int N>
__global__ void __launch_bounds__(128) fr_post(int n, const uint8_t *ct, uint8_t *scratch, const uint8_t *sk, uint8_t *ss) {
    using P = FP<N>;
    FR_WARP_INSTANCE;
    uint8_t *scr = scratch + (size_t)x * P::SCRATCH;
    const uint2 *k = reinterpret_cast<const uint2 *>(scr + P::NOISE_U16 * 2);
    uint2 *key = reinterpret_cast<uint2 *>(scr + P::NOISE_U16 * 2 + 72);
    if (w.lane < P::NW) {
        uint2 kv = k[w.lane];
        if (sk) {
            const uint32_t mask = 0u - (uint32_t)(scr[P::NOISE_U16 * 2 + 64] != 0);
            const uint2 sv = reinterpret_cast<const uint2 *>(sk + (size_t)x * P::SKB)[w.lane];
            kv = make_uint2(kv.x ^ (mask & (kv.x ^ sv.x)), kv.y ^ (mask & (kv.y ^ sv.y)));
        }
        key[w.lane] = kv;
    }
    __syncwarp();
    uint2 a;
    warp_absorb2<P::RATE>(a, reinterpret_cast<const uint2 *>(ct + (size_t)x * P::CTB), P::CTB / 8, key, P::NW, DOM_SHAKE,
                          w);
    keccak_f1600_warp(a, w);
    if (w.lane < P::NW) reinterpret_cast<uint2 *>(ss + (size_t)x * P::SSB)[w.lane] = a;
}

// keypair epilogue: sk = s || pk || S (u16 LE, S[k*N + j]) || SHAKE(pk, SSB)
template <int N>
__global__ void __launch_bounds__(128) fr_kp_post(int n, const uint8_t *coins, int cstride, const uint8_t *pk,
                                                  const uint8_t *scratch, uint8_t *sk) {
    using P = FP<N>;
    FR_WARP_INSTANCE;
    uint8_t *s = sk + (size_t)x * P::SKB;
    const uint8_t *p = pk + (size_t)x * P::PKB;
    const uint16_t *St = reinterpret_cast<const uint16_t *>(scratch + (size_t)x * P::SCRATCH);
    if (w.lane < P::NW)
        reinterpret_cast<uint2 *>(s)[w.lane] = reinterpret_cast<const uint2 *>(coins + (size_t)x * cstride)[w.lane];
    for (int i = w.lane; i < P::PKB / 8; i += 32)
        reinterpret_cast<uint2 *>(s + P::SSB)[i] = reinterpret_cast<const uint2 *>(p)[i];
    uint16_t *dS = reinterpret_cast<uint16_t *>(s + P::SSB + P::PKB);
    for (int e = w.lane; e < N * NB; e += 32) {
        const int k = e / N, j = e % N;
        dS[e] = St[j * NB + k];
    }
    uint2 a;
    warp_absorb2<P::RATE>(a, reinterpret_cast<const uint2 *>(p), P::PKB / 8, nullptr, 0, DOM_SHAKE, w);
    keccak_f1600_warp(a, w);
    if (w.lane < P::NW) reinterpret_cast<uint2 *>(s + P::SSB + P::PKB + 2 * N * NB)[w.lane] = a;
}

// ---------------------------------------------------------------------------------------------
// Core kernels: A generated on the fly
// ---------------------------------------------------------------------------------------------
// B = A S + E, one thread per row of A; CTA = (instance, group of rows); St in shared memory.
template <int N>
__device__ __forceinline__ void fr_kp_core_body(uint8_t *pk, const uint8_t *scratch, int x, int rb, uint16_t *St) {
    using P = FP<N>;
    const uint16_t *gSt = reinterpret_cast<const uint16_t *>(scratch + (size_t)x * P::SCRATCH), *E = gSt + N * NB;
    for (int i = threadIdx.x; i < N * NB / 8; i += blockDim.x)
        reinterpret_cast<uint4 *>(St)[i] = reinterpret_cast<const uint4 *>(gSt)[i];
    __syncthreads();
    const int row = rb * blockDim.x + threadIdx.x;
    if (row >= N) return;
    uint8_t *p = pk + (size_t)x * P::PKB;
    uint2 A[25];
    row_absorb(A, row, reinterpret_cast<const uint2 *>(p));
    uint32_t acc[NB];
#pragma unroll
    for (int k = 0; k < NB; k++) acc[k] = E[row * NB + k];
    for (int blk = 0; blk < P::ROW_BLOCKS; blk++) {
        keccak_f1600(A);
        const int j0 = blk * 84;
#pragma unroll
        for (int w = 0; w < 42; w++) {
            const uint32_t t = (w & 1) ? A[w >> 1].y : A[w >> 1].x;
#pragma unroll
            for (int h = 0; h < 2; h++) {
                const int j = j0 + 2 * w + h;
                if (j < N) {
                    const uint32_t a = h ? (t >> 16) : (t & 0xffff);
                    const uint4 sv = reinterpret_cast<const uint4 *>(St)[j];
                    acc[0] += a * (sv.x & 0xffff);
                    acc[1] += a * (sv.x >> 16);
                    acc[2] += a * (sv.y & 0xffff);
                    acc[3] += a * (sv.y >> 16);
                    acc[4] += a * (sv.z & 0xffff);
                    acc[5] += a * (sv.z >> 16);
                    acc[6] += a * (sv.w & 0xffff);
                    acc[7] += a * (sv.w >> 16);
                }
            }
        }
    }
    // pack B row (8 values, LOGQ bits each, MSB first) at pk[16 + LOGQ row]
    pack8<P::LOGQ>(p + SEEDA + P::LOGQ * row, acc);
}
template <int N>
__global__ void __launch_bounds__(256) fr_kp_core(int n, uint8_t *pk, const uint8_t *scratch) {
    __shared__ __align__(16) uint16_t St[N * NB];
    fr_kp_core_body<N>(pk, scratch, blockIdx.y, blockIdx.x, St);
}

// Epilogue of B' = S' A + E': V = S' B + E'' (B = unpack(pk_b), N x 8; 64 outputs, k split over
// the CTA, into acc[NB*N ..]), then B' -> c1 and C = V + encode(mu) -> c2, packed LOGQ bits MSB
// first, or compared mod q with the received ciphertext (cmp != nullptr; the fail flag goes to
// scratch).  acc holds B' (8 x N, u32, wrapped mod 2^32) and E'' in its last 64 words; Spt is S'
// (N x 8).  Packing works on groups of 8 consecutive values (LOGQ bytes each).
template <int N>
__device__ void sa_epilogue(uint32_t *acc, const uint16_t *Spt, const uint8_t *p, uint8_t *scr, uint8_t *ct,
                            const uint8_t *ct_cmp, int x) {
    using P = FP<N>;
    constexpr int LOGQ = P::LOGQ, B = P::B;
    const int tid = threadIdx.x, nthr = blockDim.x;
    {
        // V = S' B (8 x 8, sums over N): thread = (row i of S', k residue kb mod KS); each step reads
        // one whole row of B (8 values; 16 bytes when LOGQ = 16) and updates the thread's 8 sums;
        // the KS / 4 residues of a warp are summed by shuffles, then one shared atomic per output
        const uint8_t *pb = p + SEEDA;
        const int ks = nthr / NB, i = tid % NB, kb = tid / NB;
        // 16-bit rows as two 8-byte loads when B is 8-byte aligned (the public key inside a
        // FrodoKEM-976 secret key starts 24 bytes in, so 16-byte alignment is not given)
        const bool wide = LOGQ == 16 && (reinterpret_cast<uintptr_t>(pb) & 7) == 0;
        uint32_t v[NB];
#pragma unroll
        for (int l = 0; l < NB; l++) v[l] = 0;
        for (int k = kb; k < N; k += ks) {
            const uint32_t sv = Spt[k * NB + i];
            uint32_t b[NB];
            if (wide) {
                const uint2 r0 = reinterpret_cast<const uint2 *>(pb + (size_t)16 * k)[0];
                const uint2 r1 = reinterpret_cast<const uint2 *>(pb + (size_t)16 * k)[1];
                const uint32_t w[4] = {r0.x, r0.y, r1.x, r1.y};
#pragma unroll
                for (int l = 0; l < NB; l++) {  // big-endian 16-bit values
                    const uint32_t h = (w[l >> 1] >> (16 * (l & 1))) & 0xffff;
                    b[l] = ((h & 0xff) << 8) | (h >> 8);
                }
            } else {
#pragma unroll
                for (int l = 0; l < NB; l++) b[l] = unpack_at<LOGQ>(pb + (size_t)LOGQ * k, l);
            }
#pragma unroll
            for (int l = 0; l < NB; l++) v[l] += sv * b[l];
        }
#pragma unroll
        for (int l = 0; l < NB; l++) {
            v[l] += __shfl_xor_sync(0xffffffffu, v[l], 8);
            v[l] += __shfl_xor_sync(0xffffffffu, v[l], 16);
        }
        if ((tid & 31) < NB) {
#pragma unroll
            for (int l = 0; l < NB; l++) atomicAdd(acc + NB * N + i * NB + l, v[l]);
        }
    }
    __syncthreads();
    const uint8_t *mu = scr + P::NOISE_U16 * 2 + 32;
    uint32_t diff = 0;
    for (int g8 = tid; g8 < NB * N / 8; g8 += nthr) {  // groups of 8 values of B'
        uint32_t v[8];
#pragma unroll
        for (int k = 0; k < 8; k++) v[k] = acc[8 * g8 + k] & P::MASKQ;
        if (ct_cmp) {
            const uint8_t *c = ct_cmp + (size_t)x * P::CTB + (size_t)LOGQ * g8;
#pragma unroll
            for (int k = 0; k < 8; k++) diff |= v[k] ^ unpack_at<LOGQ>(c, k);
        } else {
            pack8<LOGQ>(ct + (size_t)x * P::CTB + (size_t)LOGQ * g8, v);
        }
    }
    for (int g = tid; g < 8; g += nthr) {  // C = V + encode(mu), row g: B bytes of mu -> 8 values
        uint32_t temp = 0;
#pragma unroll
        for (int b = 0; b < B; b++) temp |= (uint32_t)mu[B * g + b] << (8 * b);
        uint32_t v[8];
#pragma unroll
        for (int j = 0; j < 8; j++) {
            const uint32_t enc = ((temp >> (B * j)) & ((1u << B) - 1)) << (LOGQ - B);
            v[j] = (acc[NB * N + 8 * g + j] + enc) & P::MASKQ;
        }
        if (ct_cmp) {
            const uint8_t *c = ct_cmp + (size_t)x * P::CTB + P::C1B + (size_t)LOGQ * g;
#pragma unroll
            for (int j = 0; j < 8; j++) diff |= v[j] ^ unpack_at<LOGQ>(c, j);
        } else {
            pack8<LOGQ>(ct + (size_t)x * P::CTB + P::C1B + (size_t)LOGQ * g, v);
        }
    }
    if (ct_cmp) {
        const int any = __syncthreads_or(diff != 0);
        if (tid == 0) scr[P::NOISE_U16 * 2 + 64] = (uint8_t)any;
    }
}

// B' = S' A + E' (and V, C), CTA (instance x = blockIdx.x, row part blockIdx.y of gridDim.y).
// With one part the CTA owns the whole product and runs the epilogue.  With several, the CTA
// contracts only its rows of A and adds its partial B' into the instance's u32 accumulator in
// scratch (zeroed by the prologue kernel); fr_sa_final then finishes.  Sums are mod 2^32, hence
// exact mod 2^16 in any order.  cmp == nullptr: pack into ct; else compare with ct.
constexpr int SA_THREADS = 256;
constexpr int STAGE_PITCH = 86;  // u16 per staged row block (84 used; odd word pitch)
constexpr int BLK_COLS = 84;     // u16 values per SHAKE128 block
template <int N>
__device__ __forceinline__ void fr_sa_core_body(uint8_t *ct, const uint8_t *ct_cmp, const uint8_t *pk, int pk_stride,
                                                uint8_t *scratch, int x, int part, int parts, uint8_t *smem) {
    using P = FP<N>;
    uint16_t *Spt = reinterpret_cast<uint16_t *>(smem);                       // N x 8
    uint32_t *acc = reinterpret_cast<uint32_t *>(smem + N * NB * 2);          // 8 x N (+64 for V)
    uint16_t *stage = reinterpret_cast<uint16_t *>(smem + N * NB * 2 + (NB * N + 64) * 4);  // threads x 86
    const int tid = threadIdx.x, nthr = blockDim.x;
    const int rows_per = (N + parts - 1) / parts, rbeg = part * rows_per, rend = min(N, rbeg + rows_per);
    uint8_t *scr = scratch + (size_t)x * P::SCRATCH;
    const uint16_t *gSpt = reinterpret_cast<const uint16_t *>(scr), *Ep = gSpt + N * NB, *Epp = Ep + N * NB;
    const uint8_t *p = pk + (size_t)x * pk_stride;
    for (int i = tid; i < N * NB / 8; i += nthr) reinterpret_cast<uint4 *>(Spt)[i] = reinterpret_cast<const uint4 *>(gSpt)[i];
    for (int i = tid; i < NB * N; i += nthr) acc[i] = parts == 1 ? Ep[i] : 0u;
    for (int i = tid; i < 64; i += nthr) acc[NB * N + i] = Epp[i];
    __syncthreads();
    // rows pass by pass; within a pass each thread owns one row and squeezes one block per round,
    // then the CTA contracts the staged block: work item (column j, row slice) per thread
    const int nslice = max(1, nthr / BLK_COLS);
    for (int r0 = rbeg; r0 < rend; r0 += nthr) {
        const int rows = min(nthr, rend - r0);
        uint2 A[25];
        if (tid < rows) row_absorb(A, r0 + tid, reinterpret_cast<const uint2 *>(p));
        for (int blk = 0; blk < P::ROW_BLOCKS; blk++) {
            if (tid < rows) {
                keccak_f1600(A);
                uint32_t *st = reinterpret_cast<uint32_t *>(stage + tid * STAGE_PITCH);
#pragma unroll
                for (int w = 0; w < 42; w++) st[w] = (w & 1) ? A[w >> 1].y : A[w >> 1].x;
            }
            __syncthreads();
            const int per = (rows + nslice - 1) / nslice;
            for (int t = tid; t < BLK_COLS * nslice; t += nthr) {
                const int j = t % BLK_COLS, slice = t / BLK_COLS, col = blk * BLK_COLS + j;
                if (col >= N) continue;
                const int k0 = slice * per, k1 = min(rows, k0 + per);
                uint32_t s[NB] = {0, 0, 0, 0, 0, 0, 0, 0};
                for (int k = k0; k < k1; k++) {
                    const uint32_t a = stage[k * STAGE_PITCH + j];
                    const uint4 sv = reinterpret_cast<const uint4 *>(Spt)[r0 + k];
                    s[0] += a * (sv.x & 0xffff);
                    s[1] += a * (sv.x >> 16);
                    s[2] += a * (sv.y & 0xffff);
                    s[3] += a * (sv.y >> 16);
                    s[4] += a * (sv.z & 0xffff);
                    s[5] += a * (sv.z >> 16);
                    s[6] += a * (sv.w & 0xffff);
                    s[7] += a * (sv.w >> 16);
                }
#pragma unroll
                for (int i = 0; i < NB; i++) atomicAdd(acc + i * N + col, s[i]);
            }
            __syncthreads();
        }
    }
    if (parts > 1) {
        uint32_t *g = reinterpret_cast<uint32_t *>(scr + P::GACC_OFF);
        for (int i = tid; i < NB * N; i += nthr) atomicAdd(g + i, acc[i]);
        return;
    }
    sa_epilogue<N>(acc, Spt, p, scr, ct, ct_cmp, x);
}
template <int N>
__global__ void __launch_bounds__(SA_THREADS) fr_sa_core(int n, uint8_t *ct, const uint8_t *ct_cmp, const uint8_t *pk,
                                                         int pk_stride, uint8_t *scratch) {
    extern __shared__ __align__(16) uint8_t smem[];
    fr_sa_core_body<N>(ct, ct_cmp, pk, pk_stride, scratch, blockIdx.x, blockIdx.y, gridDim.y, smem);
}

// Finish a split product: acc = (sum of the parts) + E', then the same epilogue.  CTA per instance.
template <int N>
__global__ void __launch_bounds__(SA_THREADS) fr_sa_final(int n, uint8_t *ct, const uint8_t *ct_cmp, const uint8_t *pk,
                                                          int pk_stride, uint8_t *scratch) {
    using P = FP<N>;
    extern __shared__ __align__(16) uint8_t smem[];
    uint16_t *Spt = reinterpret_cast<uint16_t *>(smem);
    uint32_t *acc = reinterpret_cast<uint32_t *>(smem + N * NB * 2);
    const int x = blockIdx.x, tid = threadIdx.x, nthr = blockDim.x;
    uint8_t *scr = scratch + (size_t)x * P::SCRATCH;
    const uint16_t *gSpt = reinterpret_cast<const uint16_t *>(scr), *Ep = gSpt + N * NB, *Epp = Ep + N * NB;
    const uint32_t *g = reinterpret_cast<const uint32_t *>(scr + P::GACC_OFF);
    for (int i = tid; i < N * NB / 8; i += nthr) reinterpret_cast<uint4 *>(Spt)[i] = reinterpret_cast<const uint4 *>(gSpt)[i];
    for (int i = tid; i < NB * N; i += nthr) acc[i] = g[i] + Ep[i];
    for (int i = tid; i < 64; i += nthr) acc[NB * N + i] = Epp[i];
    __syncthreads();
    sa_epilogue<N>(acc, Spt, pk + (size_t)x * pk_stride, scr, ct, ct_cmp, x);
}

// ---------------------------------------------------------------------------------------------
// Many encapsulations to one public key: A is generated once for the whole batch and the products
// of every instance form one matrix product, [S'_0; S'_1; ...] (8n x N) times A (N x N).
// ---------------------------------------------------------------------------------------------
// A (N x N, u16, row-major) from seedA, one thread per row (frodo_macrify_reference.cu:164-188);
// with planes != nullptr also the tensor-core operands: plane 0 = A & 1023 and plane 1 = A >> 10 as fp16
// bit patterns (exact: both below 2048), column j / row k of A at fr_tc_plane_index.  CTA 0's first
// warp computes pkh = SHAKE(pk, SSB) meanwhile (fr_pkh_one's work, 115 serial permutations for
// n = 976), so the two fixed latencies of a shared-key batch overlap.
template <int N>
__global__ void __launch_bounds__(128) fr_gen_a(const uint8_t *pk, uint16_t *A, uint16_t *planes, uint8_t *pkh) {
    using P = FP<N>;
    if (blockIdx.x == 0) {
        if (threadIdx.x >= 32) return;
        const WarpKeccak w(threadIdx.x);
        uint2 a;
        warp_absorb2<P::RATE>(a, reinterpret_cast<const uint2 *>(pk), P::PKB / 8, nullptr, 0, DOM_SHAKE, w);
        keccak_f1600_warp(a, w);
        if (w.lane < P::NW) reinterpret_cast<uint2 *>(pkh)[w.lane] = a;
        return;
    }
    const int row = (blockIdx.x - 1) * blockDim.x + threadIdx.x;
    if (row >= N) return;
    uint2 S[25];
    row_absorb(S, row, reinterpret_cast<const uint2 *>(pk));
    for (int blk = 0; blk < P::ROW_BLOCKS; blk++) {
        keccak_f1600(S);
#pragma unroll
        for (int w = 0; w < 42; w++) {
            const uint32_t t = (w & 1) ? S[w >> 1].y : S[w >> 1].x;
#pragma unroll
            for (int h = 0; h < 2; h++) {
                const int j = blk * BLK_COLS + 2 * w + h;
                if (j < N) {
                    const uint32_t a = h ? (t >> 16) : (t & 0xffff);
                    A[(size_t)row * N + j] = (uint16_t)a;
                    if (planes) {
                        planes[fr_tc_plane_index(N, 0, j, row)] = __half_as_ushort(__uint2half_rn(a & 1023));
                        planes[fr_tc_plane_index(N, 1, j, row)] = __half_as_ushort(__uint2half_rn(a >> 10));
                    }
                }
            }
        }
    }
}

// CUDA-core product: G[x][i][j] = sum_k S'[x][i][k] A[k][j] (mod 2^32, exact mod 2^16) into the
// instances' u32 accumulators (scratch, GACC_OFF).  CTA = 4 instances x 128 columns, thread =
// one instance's 8 rows x 2 columns; A and S' staged through shared memory in chunks of 32 k.
constexpr int SH_INST = 4, SH_COLS = 128, SH_KC = 32, SH_THREADS = 256;
template <int N>
__global__ void __launch_bounds__(SH_THREADS) fr_sa_shared_simt(int n, const uint16_t *A, uint8_t *scratch) {
    using P = FP<N>;
    __shared__ __align__(16) uint16_t sA[SH_KC][SH_COLS];
    __shared__ __align__(16) uint16_t sS[SH_INST][SH_KC][NB];
    const int x0 = blockIdx.x * SH_INST, c0 = blockIdx.y * SH_COLS, tid = threadIdx.x;
    const int li = tid >> 6, cc = (tid & 63) * 2;  // instance in the CTA, first of its two columns
    uint32_t acc[NB][2];
#pragma unroll
    for (int i = 0; i < NB; i++) acc[i][0] = acc[i][1] = 0;
    for (int k0 = 0; k0 < N; k0 += SH_KC) {
        for (int t = tid; t < SH_KC * SH_COLS / 2; t += SH_THREADS) {  // A rows k0.., 2 columns a thread
            const int kk = t / (SH_COLS / 2), j = c0 + 2 * (t % (SH_COLS / 2)), k = k0 + kk;
            uint32_t v = 0;
            if (k < N && j < N) v = *reinterpret_cast<const uint32_t *>(A + (size_t)k * N + j);  // N even
            reinterpret_cast<uint32_t *>(&sA[kk][0])[t % (SH_COLS / 2)] = v;
        }
        for (int t = tid; t < SH_INST * SH_KC; t += SH_THREADS) {  // S'^T rows: 8 values per (instance, k)
            const int xi = t / SH_KC, kk = t % SH_KC, x = x0 + xi, k = k0 + kk;
            uint4 v = make_uint4(0, 0, 0, 0);
            if (x < n && k < N) v = reinterpret_cast<const uint4 *>(scratch + (size_t)x * P::SCRATCH)[k];
            *reinterpret_cast<uint4 *>(&sS[xi][kk][0]) = v;
        }
        __syncthreads();
#pragma unroll 4
        for (int kk = 0; kk < SH_KC; kk++) {
            const uint4 sv = *reinterpret_cast<const uint4 *>(&sS[li][kk][0]);
            const uint32_t a2 = *reinterpret_cast<const uint32_t *>(&sA[kk][cc]);
            const uint32_t a0 = a2 & 0xffff, a1 = a2 >> 16;
            const uint32_t s[NB] = {sv.x & 0xffff, sv.x >> 16, sv.y & 0xffff, sv.y >> 16,
                                    sv.z & 0xffff, sv.z >> 16, sv.w & 0xffff, sv.w >> 16};
#pragma unroll
            for (int i = 0; i < NB; i++) {
                acc[i][0] += s[i] * a0;
                acc[i][1] += s[i] * a1;
            }
        }
        __syncthreads();
    }
    const int x = x0 + li, j = c0 + cc;
    if (x >= n || j >= N) return;
    uint32_t *g = reinterpret_cast<uint32_t *>(scratch + (size_t)x * P::SCRATCH + P::GACC_OFF);
#pragma unroll
    for (int i = 0; i < NB; i++) *reinterpret_cast<uint2 *>(g + (size_t)i * N + j) = make_uint2(acc[i][0], acc[i][1]);
}

static size_t sa_smem(int N, int threads) {
    return (size_t)N * NB * 2 + ((size_t)NB * N + 64) * 4 + (size_t)threads * STAGE_PITCH * 2;
}
static size_t sa_final_smem(int N) { return (size_t)N * NB * 2 + ((size_t)NB * N + 64) * 4; }

// ---- persistent wave for the FrodoKEM jobs of a mixed batch ----
// One launch holds the products of every FrodoKEM job (n = 640, 976 and 1344): key generation's
// B = AS + E in tiles of 256 rows of one instance, and the B' = S'A + E' of encapsulation and
// decapsulation in tiles of one instance or one part of it (the job's row split, as in its own
// launch).  SMs x 2 CTAs of 256 threads take tiles from a global counter, products first.
constexpr int FRW_THREADS = 256, FRW_MAX_JOBS = 32;
struct FrWaveJob {
    int kind;                // 0 key generation rows, 1 B' = S'A + E'
    int N, first, per;       // first tile; tiles per instance (row blocks or parts)
    uint8_t *pk;             // kind 0: the public keys being formed
    uint8_t *ct;             // kind 1: ciphertexts out (encapsulation) or nullptr
    const uint8_t *cmp;      // kind 1: received ciphertexts (decapsulation) or nullptr
    const uint8_t *pkp;      // kind 1: public keys (stride pk_stride)
    int pk_stride;
    uint8_t *scratch;
};
struct FrWaveTable {
    int njobs, tiles;
    FrWaveJob j[FRW_MAX_JOBS];
};

// counter: a zeroed word of device memory for this launch.  One kernel per stage (KIND 0: key
// generation rows; KIND 1: B' = S'A + E' of encapsulations and decapsulations) and parameter set:
// with several bodies in one kernel they spilled at the 128 registers that two CTAs per SM allow.
template <int KIND, int N>
__global__ void __launch_bounds__(FRW_THREADS, 2) fr_stage_persistent(const __grid_constant__ FrWaveTable t,
                                                                     unsigned *counter) {
    extern __shared__ __align__(16) uint8_t smem[];
    __shared__ int s_tile;
    for (;;) {
        if (threadIdx.x == 0) s_tile = (int)atomicAdd(counter, 1u);
        __syncthreads();
        const int tile = s_tile;
        if (tile >= t.tiles) break;
        int lo = 0, hi = t.njobs - 1;  // the job whose tiles start at or before `tile`
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (t.j[mid].first <= tile) lo = mid;
            else hi = mid - 1;
        }
        const int per = t.j[lo].per, local = tile - t.j[lo].first, x = local / per, sub = local % per;
        if constexpr (KIND == 0)
            fr_kp_core_body<N>(t.j[lo].pk, t.j[lo].scratch, x, sub, reinterpret_cast<uint16_t *>(smem));
        else
            fr_sa_core_body<N>(t.j[lo].ct, t.j[lo].cmp, t.j[lo].pkp, t.j[lo].pk_stride, t.j[lo].scratch, x, sub, per,
                               smem);
        __syncthreads();  // the next tile reuses shared memory (and s_tile)
    }
}

// A wave's dynamic shared memory.
static size_t frw_smem(int kind, int N) { return kind == 0 ? (size_t)N * NB * 2 : sa_smem(N, FRW_THREADS); }
template <int KIND, int N>
static cudaError_t frw_attr() {
    return cudaFuncSetAttribute(fr_stage_persistent<KIND, N>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)frw_smem(KIND, N));
}
// One persistent launch of stage KIND of parameter set N over the table's jobs.
template <int KIND, int N>
static int frw_launch(const FrWaveTable &t, unsigned *counter, cudaStream_t st) {
    int dev = 0, sms = 0, per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fr_stage_persistent<KIND, N>, FRW_THREADS,
                                                      frw_smem(KIND, N)) != cudaSuccess ||
        per_sm < 1) {
        cudaGetLastError();
        per_sm = 1;
    }
    if (cudaMemsetAsync(counter, 0, sizeof(unsigned), st) != cudaSuccess) return PQCGPU_ECUDA;
    const int grid = std::min(t.tiles, sms * per_sm);
    PQC_LAUNCH(st, "fr_stage_persistent", N, KIND,
               fr_stage_persistent<KIND, N><<<grid, FRW_THREADS, frw_smem(KIND, N), st>>>(t, counter));
    return cudaGetLastError() == cudaSuccess ? PQCGPU_OK : PQCGPU_ECUDA;
}

}  // namespace frodo

using namespace frodo;

int frodo_init_constants() {
    // CDF tables of the FrodoKEM parameter sets (n = 976: FrodoKEM_GPU/frodo976.cu:21)
    const uint16_t cdf640[13] = {4643, 13363, 20579, 25843, 29227, 31145, 32103, 32525, 32689, 32745, 32762, 32766, 32767};
    const uint16_t cdf976[11] = {5638, 15915, 23689, 28571, 31116, 32217, 32613, 32731, 32760, 32766, 32767};
    const uint16_t cdf1344[7] = {9142, 23462, 30338, 32361, 32725, 32765, 32767};
    uint2 rc[24];
    keccak_rc_host(rc);
    if (cudaMemcpyToSymbol(c_keccak_rc, rc, sizeof rc) != cudaSuccess) return PQCGPU_ECUDA;
    if (cudaMemcpyToSymbol(c_cdf640, cdf640, sizeof cdf640) != cudaSuccess) return PQCGPU_ECUDA;
    if (cudaMemcpyToSymbol(c_cdf976, cdf976, sizeof cdf976) != cudaSuccess) return PQCGPU_ECUDA;
    if (cudaMemcpyToSymbol(c_cdf1344, cdf1344, sizeof cdf1344) != cudaSuccess) return PQCGPU_ECUDA;
    // the FrodoKEM wave's shared-memory bound, once, so that no launch (captured or not) depends on
    // an earlier one having set it
    if (frw_attr<0, 640>() || frw_attr<0, 976>() || frw_attr<0, 1344>() || frw_attr<1, 640>() || frw_attr<1, 976>() ||
        frw_attr<1, 1344>())
        return PQCGPU_ECUDA;
    return PQCGPU_OK;
}
size_t frodo_scratch_bytes(int N) {
    return N == 640 ? FP<640>::SCRATCH : N == 976 ? FP<976>::SCRATCH : N == 1344 ? FP<1344>::SCRATCH : 0;
}

// Launch shapes.  Keypair: threads per CTA of fr_kp_core (one row of A per thread).  Encaps /
// decaps: row parts per instance for B' = S' A + E' and threads per CTA of fr_sa_core.  0 = chosen
// by batch size: small batches split an instance over several CTAs (latency), large ones keep one
// CTA per instance (no split traffic).  Set through pqcgpu_set_launch_shape (the autotuner); the
// settings apply to every FrodoKEM parameter set.
int frodo_set_shared_product(int product);
int frodo_get_shared_product();
// (parts, threads) per operation, one atomic word each; parts 0 = chosen by batch size.
static LaunchShape g_fr_shape[3] = {{0, 0}, {0, 0}, {0, 0}};

static void fr_shape(int op, int n, int *parts, int *threads) {
    int p, t;
    g_fr_shape[op].get(p, t);
    if (op == 0) {
        *parts = 1;
        *threads = t ? t : (n >= 152 ? 256 : 64);
        return;
    }
    if (p) {
        *parts = p;
        *threads = t;
        return;
    }
    if (n >= 304) *parts = 1, *threads = 256;
    else if (n >= 152) *parts = 2, *threads = 256;
    else if (n >= 76) *parts = 4, *threads = 256;
    else if (n >= 10) *parts = 8, *threads = 128;
    else *parts = 16, *threads = 256;  // at most 144 CTAs, one per SM (measured on GB300 at n = 1, 8 x 128 ->
                                       // 16 x 256: FrodoKEM-1344 encapsulation 1884 -> 1775 us, decapsulation
                                       // 1413 -> 1305 us; FrodoKEM-976 1267 -> 1248 and 981 -> 963 us)
}

int frodo_set_shape(int op, int parts, int threads) {
    if (op == 3) return frodo_set_shared_product(parts);  // the shared-key product
    if (op == 0) {
        if (parts > 1 || !(threads == 0 || threads == 64 || threads == 128 || threads == 256)) return PQCGPU_EINVAL;
        g_fr_shape[0].set(0, threads);
        return PQCGPU_OK;
    }
    if (op != 1 && op != 2) return PQCGPU_EINVAL;
    if (parts == 0) {
        g_fr_shape[op].set(0, 0);
        return PQCGPU_OK;
    }
    if (!(parts == 1 || parts == 2 || parts == 4 || parts == 8 || parts == 16) || !(threads == 128 || threads == 256))
        return PQCGPU_EINVAL;
    g_fr_shape[op].set(parts, threads);
    return PQCGPU_OK;
}

int frodo_get_shape(int op, int *parts, int *threads) {
    if (op == 3) {
        *parts = frodo_get_shared_product();
        *threads = 0;
        return PQCGPU_OK;
    }
    if (op < 0 || op > 2) return PQCGPU_EINVAL;
    int p, t;
    g_fr_shape[op].get(p, t);
    *parts = op == 0 ? 1 : p;
    *threads = t;
    return PQCGPU_OK;
}

namespace {
template <int N>
int keypair_n(int n, uint8_t *pk, uint8_t *sk, const uint8_t *coins, int cstride, uint8_t *scratch, cudaStream_t st) {
    int parts, thr;
    fr_shape(0, n, &parts, &thr);
    PQC_LAUNCH(st, "fr_kp_pre", N, 0, fr_kp_pre<N><<<(n + 3) / 4, 128, 0, st>>>(n, coins, cstride, pk, scratch));
    PQC_LAUNCH(st, "fr_kp_core", N, 0, fr_kp_core<N><<<dim3((N + thr - 1) / thr, n), thr, 0, st>>>(n, pk, scratch));
    PQC_LAUNCH(st, "fr_kp_post", N, 0, fr_kp_post<N><<<(n + 3) / 4, 128, 0, st>>>(n, coins, cstride, pk, scratch, sk));
    return cudaGetLastError() == cudaSuccess ? PQCGPU_OK : PQCGPU_ECUDA;
}

// B' = S' A + E' and the ciphertext epilogue: one CTA per instance, or `parts` CTAs per instance
// plus fr_sa_final.
template <int N>
void launch_sa(int n, uint8_t *ct, const uint8_t *ct_cmp, const uint8_t *pk, int pk_stride, uint8_t *scratch, int parts,
               int thr, cudaStream_t st) {
    PQC_LAUNCH(st, "fr_sa_core", N, 0,
               fr_sa_core<N><<<dim3(n, parts), thr, sa_smem(N, thr), st>>>(n, ct, ct_cmp, pk, pk_stride, scratch));
    if (parts > 1)
        PQC_LAUNCH(st, "fr_sa_final", N, 0,
                   fr_sa_final<N><<<n, SA_THREADS, sa_final_smem(N), st>>>(n, ct, ct_cmp, pk, pk_stride, scratch));
}

template <int N>
int sa_attrs() {
    if (capturing()) return PQCGPU_OK;
    if (cudaFuncSetAttribute(fr_sa_core<N>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sa_smem(N, SA_THREADS)) !=
            cudaSuccess ||
        cudaFuncSetAttribute(fr_sa_final<N>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sa_final_smem(N)) !=
            cudaSuccess) {
        cudaGetLastError();
        return PQCGPU_ECUDA;
    }
    return PQCGPU_OK;
}

template <int N>
int enc_n(int n, uint8_t *ct, uint8_t *ss, const uint8_t *pk, const uint8_t *mu, uint8_t *scratch, cudaStream_t st,
          const uint8_t *pkh) {
    if (sa_attrs<N>()) return PQCGPU_ECUDA;
    int parts, thr;
    fr_shape(1, n, &parts, &thr);
    PQC_LAUNCH(st, "fr_enc_pre", N, 0,
               fr_enc_pre<N><<<(n + 3) / 4, 128, 0, st>>>(n, pk, mu, scratch, parts, pkh, FP<N>::SSB));
    launch_sa<N>(n, ct, nullptr, pk, FP<N>::PKB, scratch, parts, thr, st);
    PQC_LAUNCH(st, "fr_post", N, 0, fr_post<N><<<(n + 3) / 4, 128, 0, st>>>(n, ct, scratch, nullptr, ss));
    return cudaGetLastError() == cudaSuccess ? PQCGPU_OK : PQCGPU_ECUDA;
}

template <int N>
int dec_n(int n, uint8_t *ss, const uint8_t *ct, const uint8_t *sk, uint8_t *scratch, cudaStream_t st) {
    using P = FP<N>;
    if (sa_attrs<N>()) return PQCGPU_ECUDA;
    int parts, thr;
    fr_shape(2, n, &parts, &thr);
    PQC_LAUNCH(st, "fr_dec_w", N, 0, fr_dec_w<N><<<n, 256, 0, st>>>(n, ct, sk, scratch));
    PQC_LAUNCH(st, "fr_dec_pre", N, 0, fr_dec_pre<N><<<(n + 3) / 4, 128, 0, st>>>(n, sk, scratch, parts));
    launch_sa<N>(n, nullptr, ct, sk + P::SSB, P::SKB, scratch, parts, thr, st);
    PQC_LAUNCH(st, "fr_post", N, 0, fr_post<N><<<(n + 3) / 4, 128, 0, st>>>(n, ct, scratch, sk, ss));
    return cudaGetLastError() == cudaSuccess ? PQCGPU_OK : PQCGPU_ECUDA;
}
}  // namespace

// Product of a shared-key batch: 1 CUDA cores (mad.lo, fr_sa_shared_simt), 2 tensor cores
// (tcgen05 kind::f16 on split A, fr_sa_shared_tc); 0 = the default below, chosen by measurement on
// GB300 at 2048 encapsulations to one key (product kernel, CUDA cores -> tensor cores):
// FrodoKEM-976 product 1.070 -> 0.116 ms (S' conversion included); the whole batch, FrodoKEM-640 /
// 976 / 1344: 1.43 -> 1.88, 0.70 -> 1.01 and 0.45 -> 0.73 M encapsulations/s.
static LaunchShape g_fr_shared = {0, 0};
constexpr int FR_SHARED_DEFAULT = 2;

int frodo_set_shared_product(int product) {
    if (product < 0 || product > 2) return PQCGPU_EINVAL;
    g_fr_shared.set(product, 0);
    return PQCGPU_OK;
}
int frodo_get_shared_product() {
    int p, t;
    g_fr_shared.get(p, t);
    return p;
}
size_t frodo_shared_extra_bytes(int N) { return 256 + (size_t)N * N * 2 + fr_tc_planes_elems(N) * 2; }

namespace {
template <int N>
int enc_shared_n(int n, uint8_t *ct, uint8_t *ss, const uint8_t *pk, const uint8_t *mu, uint8_t *scratch, uint8_t *extra,
                 uint16_t *s16, unsigned *error, cudaStream_t st) {
    if (sa_attrs<N>()) return PQCGPU_ECUDA;
    int product = frodo_get_shared_product();
    if (product == 0) product = FR_SHARED_DEFAULT;
    uint8_t *pkh = extra;
    uint16_t *A = reinterpret_cast<uint16_t *>(extra + 256), *planes = A + (size_t)N * N;
    if (product == 2 && cudaMemsetAsync(planes, 0, fr_tc_planes_elems(N) * 2, st) != cudaSuccess) return PQCGPU_ECUDA;
    PQC_LAUNCH(st, "fr_gen_a", N, 0,
               fr_gen_a<N><<<1 + (N + 127) / 128, 128, 0, st>>>(pk, A, product == 2 ? planes : nullptr, pkh));
    PQC_LAUNCH(st, "fr_enc_pre", N, 0, fr_enc_pre<N><<<(n + 3) / 4, 128, 0, st>>>(n, pk, mu, scratch, 1, pkh, 0));
    if (product == 2) {
        const int rc = frodo_shared_tc_launch(N, n, planes, s16, scratch, error, st);
        if (rc) return rc;
    } else {
        PQC_LAUNCH(st, "fr_sa_shared_simt", N, 0,
                   fr_sa_shared_simt<N><<<dim3((n + SH_INST - 1) / SH_INST, (N + SH_COLS - 1) / SH_COLS), SH_THREADS, 0,
                                          st>>>(n, A, scratch));
    }
    PQC_LAUNCH(st, "fr_sa_final", N, 0,
               fr_sa_final<N><<<n, SA_THREADS, sa_final_smem(N), st>>>(n, ct, nullptr, pk, 0, scratch));
    PQC_LAUNCH(st, "fr_post", N, 0, fr_post<N><<<(n + 3) / 4, 128, 0, st>>>(n, ct, scratch, nullptr, ss));
    return cudaGetLastError() == cudaSuccess ? PQCGPU_OK : PQCGPU_ECUDA;
}
}  // namespace

// n encapsulations to one public key pk (PKB bytes), mu per instance; scratch: n x
// frodo_scratch_bytes(N), extra: frodo_shared_extra_bytes(N) (256-byte aligned): pkh at +0, A
// (N x N u16) at +256, then its two tiled fp16 planes.
int frodo_enc_shared_dev(int N, int n, uint8_t *ct, uint8_t *ss, const uint8_t *pk, const uint8_t *mu, uint8_t *scratch,
                         uint8_t *extra, uint16_t *s16, unsigned *error, cudaStream_t st) {
    if (N == 640) return enc_shared_n<640>(n, ct, ss, pk, mu, scratch, extra, s16, error, st);
    if (N == 976) return enc_shared_n<976>(n, ct, ss, pk, mu, scratch, extra, s16, error, st);
    if (N == 1344) return enc_shared_n<1344>(n, ct, ss, pk, mu, scratch, extra, s16, error, st);
    return PQCGPU_EINVAL;
}

int frodo_keypair_dev(int N, int n, uint8_t *pk, uint8_t *sk, const uint8_t *coins, int cstride, uint8_t *scratch,
                      cudaStream_t st) {
    if (N == 640) return keypair_n<640>(n, pk, sk, coins, cstride, scratch, st);
    if (N == 976) return keypair_n<976>(n, pk, sk, coins, cstride, scratch, st);
    if (N == 1344) return keypair_n<1344>(n, pk, sk, coins, cstride, scratch, st);
    return PQCGPU_EINVAL;
}

int frodo_enc_dev(int N, int n, uint8_t *ct, uint8_t *ss, const uint8_t *pk, const uint8_t *mu, uint8_t *scratch,
                  cudaStream_t st, const uint8_t *pkh) {
    if (N == 640) return enc_n<640>(n, ct, ss, pk, mu, scratch, st, pkh);
    if (N == 976) return enc_n<976>(n, ct, ss, pk, mu, scratch, st, pkh);
    if (N == 1344) return enc_n<1344>(n, ct, ss, pk, mu, scratch, st, pkh);
    return PQCGPU_EINVAL;
}

int frodo_dec_dev(int N, int n, uint8_t *ss, const uint8_t *ct, const uint8_t *sk, uint8_t *scratch, cudaStream_t st) {
    if (N == 640) return dec_n<640>(n, ss, ct, sk, scratch, st);
    if (N == 976) return dec_n<976>(n, ss, ct, sk, scratch, st);
    if (N == 1344) return dec_n<1344>(n, ss, ct, sk, scratch, st);
    return PQCGPU_EINVAL;
}

// ---- the FrodoKEM jobs of a mixed batch (persistent wave: fr_stage_persistent) ----
namespace {
template <int N>
int mixed_pre_n(const FrMixedJob &j, cudaStream_t st) {
    using P = FP<N>;
    const int n = j.n;
    int parts, thr;
    if (j.op == 0) {
        PQC_LAUNCH(st, "fr_kp_pre", N, 0, fr_kp_pre<N><<<(n + 3) / 4, 128, 0, st>>>(n, j.in0, j.kpc, j.out0, j.scratch));
    } else if (j.op == 1) {
        fr_shape(1, n, &parts, &thr);
        PQC_LAUNCH(st, "fr_enc_pre", N, 0,
                   fr_enc_pre<N><<<(n + 3) / 4, 128, 0, st>>>(n, j.in0, j.in1, j.scratch, parts, nullptr, P::SSB));
    } else {
        fr_shape(2, n, &parts, &thr);
        PQC_LAUNCH(st, "fr_dec_w", N, 0, fr_dec_w<N><<<n, 256, 0, st>>>(n, j.in0, j.in1, j.scratch));
        PQC_LAUNCH(st, "fr_dec_pre", N, 0, fr_dec_pre<N><<<(n + 3) / 4, 128, 0, st>>>(n, j.in1, j.scratch, parts));
    }
    return cudaGetLastError() == cudaSuccess ? PQCGPU_OK : PQCGPU_ECUDA;
}

template <int N>
int mixed_post_n(const FrMixedJob &j, cudaStream_t st) {
    using P = FP<N>;
    const int n = j.n;
    int parts, thr;
    if (j.op == 0) {
        PQC_LAUNCH(st, "fr_kp_post", N, 0,
                   fr_kp_post<N><<<(n + 3) / 4, 128, 0, st>>>(n, j.in0, j.kpc, j.out0, j.scratch, j.out1));
        return cudaGetLastError() == cudaSuccess ? PQCGPU_OK : PQCGPU_ECUDA;
    }
    if (sa_attrs<N>()) return PQCGPU_ECUDA;
    fr_shape(j.op, n, &parts, &thr);
    const bool enc = j.op == 1;
    uint8_t *ct = enc ? j.out0 : nullptr;
    const uint8_t *cmp = enc ? nullptr : j.in0, *pkp = enc ? j.in0 : j.in1 + P::SSB;
    const int pk_stride = enc ? P::PKB : P::SKB;
    if (parts > 1)
        PQC_LAUNCH(st, "fr_sa_final", N, 0,
                   fr_sa_final<N><<<n, SA_THREADS, sa_final_smem(N), st>>>(n, ct, cmp, pkp, pk_stride, j.scratch));
    if (enc)
        PQC_LAUNCH(st, "fr_post", N, 0, fr_post<N><<<(n + 3) / 4, 128, 0, st>>>(n, j.out0, j.scratch, nullptr, j.out1));
    else
        PQC_LAUNCH(st, "fr_post", N, 0, fr_post<N><<<(n + 3) / 4, 128, 0, st>>>(n, j.in0, j.scratch, j.in1, j.out0));
    return cudaGetLastError() == cudaSuccess ? PQCGPU_OK : PQCGPU_ECUDA;
}

}  // namespace

int frodo_mixed_pre(const FrMixedJob &j, cudaStream_t st) {
    if (j.n <= 0) return PQCGPU_OK;
    if (j.N == 640) return mixed_pre_n<640>(j, st);
    if (j.N == 976) return mixed_pre_n<976>(j, st);
    if (j.N == 1344) return mixed_pre_n<1344>(j, st);
    return PQCGPU_EINVAL;
}
int frodo_mixed_post(const FrMixedJob &j, cudaStream_t st) {
    if (j.n <= 0) return PQCGPU_OK;
    if (j.N == 640) return mixed_post_n<640>(j, st);
    if (j.N == 976) return mixed_post_n<976>(j, st);
    if (j.N == 1344) return mixed_post_n<1344>(j, st);
    return PQCGPU_EINVAL;
}

// The persistent launches of the FrodoKEM jobs: per stage (products first) and parameter set, one
// launch per FRW_MAX_JOBS jobs; counters: ncounters zeroable words, one per launch.
int frodo_mixed_wave(const std::vector<FrMixedJob> &jobs, unsigned *counters, int ncounters, cudaStream_t st) {
    std::vector<FrWaveJob> items;
    for (const FrMixedJob &j : jobs) {
        if (j.n <= 0) continue;
        FrWaveJob m{};
        m.N = j.N;
        m.scratch = j.scratch;
        if (j.op == 0) {
            m.kind = 0;
            m.per = (j.N + FRW_THREADS - 1) / FRW_THREADS;
            m.pk = j.out0;
        } else {
            int parts, thr;
            fr_shape(j.op, j.n, &parts, &thr);
            m.kind = 1;
            m.per = parts;
            const bool enc = j.op == 1;
            const int pkb = (int)(j.N == 640 ? FP<640>::PKB : j.N == 976 ? FP<976>::PKB : FP<1344>::PKB);
            const int ssb = (int)(j.N == 640 ? FP<640>::SSB : j.N == 976 ? FP<976>::SSB : FP<1344>::SSB);
            const int skb = (int)(j.N == 640 ? FP<640>::SKB : j.N == 976 ? FP<976>::SKB : FP<1344>::SKB);
            m.ct = enc ? j.out0 : nullptr;
            m.cmp = enc ? nullptr : j.in0;
            m.pkp = enc ? j.in0 : j.in1 + ssb;
            m.pk_stride = enc ? pkb : skb;
        }
        m.first = j.n;  // instances, for the ordering below; replaced by the first tile
        items.push_back(m);
    }
    int w = 0;
    for (int kind = 1; kind >= 0; kind--)  // the products first; one launch per (stage, N, FRW_MAX_JOBS jobs)
        for (int N : {1344, 976, 640}) {
            std::vector<FrWaveJob> ks;
            for (const FrWaveJob &m : items)
                if (m.kind == kind && m.N == N) ks.push_back(m);
            for (size_t from = 0; from < ks.size(); from += FRW_MAX_JOBS, w++) {
                if (w >= ncounters) return PQCGPU_EINVAL;
                FrWaveTable t{};
                t.njobs = (int)std::min(ks.size() - from, (size_t)FRW_MAX_JOBS);
                for (int i = 0; i < t.njobs; i++) {
                    t.j[i] = ks[from + i];
                    const int n = t.j[i].first;
                    t.j[i].first = t.tiles;
                    t.tiles += n * t.j[i].per;
                }
                int rc;
                if (kind) rc = N == 640 ? frw_launch<1, 640>(t, counters + w, st)
                               : N == 976 ? frw_launch<1, 976>(t, counters + w, st) : frw_launch<1, 1344>(t, counters + w, st);
                else rc = N == 640 ? frw_launch<0, 640>(t, counters + w, st)
                          : N == 976 ? frw_launch<0, 976>(t, counters + w, st) : frw_launch<0, 1344>(t, counters + w, st);
                if (rc) return rc;
            }
        }
    return PQCGPU_OK;
}

}  // namespace pqc
