// Batched FrodoKEM-976 (SHAKE) for sm_103a.
//
// Replaces crypto_kem_keypair_gpu / enc / dec (FrodoKEM_GPU/frodo976.cu:87-690: one instance per
// call, A written to and re-read from HBM, host SHAKE for pk / ct) with, per operation:
//   * a warp-per-instance kernel for the serial sponges -- the S/E noise stream
//     (SHAKE256(0x5F / 0x96 || seedSE), 230-231 permutations), G1 = SHAKE256(pk) (115), G2 and
//     the final F = SHAKE256(ct || k) (116) -- with the Keccak state spread over the warp to cut
//     the latency of these chains, the noise sampled with the CDF table on the fly;
//   * a core kernel that regenerates A row by row from SHAKE128(le16(i) || seedA) and multiplies
//     it as it appears, so A (1.9 MB per key) never exists in HBM or whole in shared memory:
//       - keypair, B = A S + E: one thread per row, which owns the 8 outputs of that row;
//       - encaps / decaps, B' = S' A + E': each thread squeezes one 168-byte block of its row per
//         round into shared memory, then the CTA contracts the staged 84 columns over its rows
//         (exact mod 2^16 with uint32 multiply-accumulate) and adds the partial sums into the
//         8 x 976 accumulator with shared-memory atomics;
//   * codecs (16-bit big-endian pack, 3-bit key encode / decode) inside the same kernels.
// Host flow and arithmetic follow FrodoKEM_GPU/kem.c:13-214, frodo_macrify_reference.cu:55-360,
// util.cu:18-113, noise.c:10-29 and the CDF table of frodo976.cu:21.
#include <cuda_runtime.h>
#include <stdint.h>

#include "keccak.cuh"
#include "pqcgpu_internal.h"

namespace pqc {
namespace frodo {

constexpr int N = 976, NB = 8;
constexpr int PKB = 15632, SKB = 31296, CTB = 15744, SSB = 24, SEEDA = 16, MUB = 24;
constexpr int C1B = 2 * N * NB;  // 15616: packed N x NBAR (or NBAR x N) matrix
constexpr int ROW_BLOCKS = 12;   // 1952 bytes of SHAKE128 per row = 11 full blocks + 104 bytes
// scratch per instance: noise (Sp 7808 + Ep 7808 + Epp 64 u16) + seeds (seedSE/k 48, mu 24, flag),
// then the u32 accumulator of B' (8 x N) used when the rows of A are split over several CTAs
constexpr int NOISE_U16 = 2 * N * NB + NB * NB;
constexpr size_t GACC_OFF = (size_t)NOISE_U16 * 2 + 128;
constexpr size_t SCRATCH = GACC_OFF + (size_t)NB * N * 4;

static __constant__ uint16_t c_cdf[11];

// ---- helpers ---------------------------------------------------------------------------------
// CDF sampler of one 16-bit value (noise.c:10-29)
__device__ __forceinline__ uint16_t cdf_sample(uint32_t r) {
    uint32_t sample = 0;
    const uint32_t prnd = (r & 0xffff) >> 1, sign = r & 1;
#pragma unroll
    for (int j = 0; j < 10; j++) sample += ((uint32_t)c_cdf[j] - prnd) >> 31 & 1;
    return (uint16_t)((((0u - sign) ^ sample) + sign) & 0xffff);
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

__device__ __forceinline__ uint32_t ld_be16(const uint8_t *p) { return ((uint32_t)p[0] << 8) | p[1]; }

// ---------------------------------------------------------------------------------------------
// Serial sponges: one warp per instance (warp-cooperative Keccak, keccak.cuh)
// ---------------------------------------------------------------------------------------------
// Message lane m (0..3) of prefix || seed (25 bytes) followed by the SHAKE domain byte, where the
// 24-byte seed is given as three little-endian 64-bit words.
__device__ __forceinline__ uint2 prefixed_lane(int m, uint32_t prefix, uint64_t s0, uint64_t s1, uint64_t s2) {
    uint64_t v;
    if (m == 0) v = prefix | (s0 << 8);
    else if (m == 1) v = (s0 >> 56) | (s1 << 8);
    else if (m == 2) v = (s1 >> 56) | (s2 << 8);
    else v = (s2 >> 56) | ((uint64_t)DOM_SHAKE << 8);
    return make_uint2((uint32_t)v, (uint32_t)(v >> 32));
}
__device__ __forceinline__ uint64_t u64(uint2 v) { return (uint64_t)v.x | ((uint64_t)v.y << 32); }

// State absorbing prefix || seed (one block, not yet permuted).
__device__ __forceinline__ uint2 seeded_state(uint32_t prefix, uint64_t s0, uint64_t s1, uint64_t s2, const WarpKeccak &w) {
    uint2 a = w.lane < 4 ? prefixed_lane(w.lane, prefix, s0, s1, s2) : make_uint2(0, 0);
    if (w.lane == SHAKE256_LANES - 1) a.y ^= 0x80000000u;
    return a;
}

// Squeeze the noise stream (state absorbed, not permuted): lanes 0..16 hold 4 u16 values each per
// block; value at stream position p is CDF-sampled and handed to emit(p, v).
template <class F>
__device__ __forceinline__ void warp_noise_stream(uint2 &a, int count, const WarpKeccak &w, F emit) {
    for (int base = 0; base < count; base += 68) {
        keccak_f1600_warp(a, w);
        if (w.lane < 17) {
#pragma unroll
            for (int q = 0; q < 4; q++) {
                const int p = base + 4 * w.lane + q;
                const uint32_t word = q < 2 ? a.x : a.y;
                if (p < count) emit(p, cdf_sample((word >> (16 * (q & 1))) & 0xffff));
            }
        }
    }
}

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

// keypair: seedA = SHAKE256(z, 16) -> pk[0..16); S (as St[j][k], N x 8) and E (N x 8) -> scratch
__global__ void __launch_bounds__(128) fr_kp_pre(int n, const uint8_t *coins, int cstride, uint8_t *pk, uint8_t *scratch) {
    FR_WARP_INSTANCE;
    const uint8_t *c = coins + (size_t)x * cstride;  // s(24) || seedSE(24) || z(16)
    uint2 a;
    warp_absorb2<SHAKE256_LANES>(a, reinterpret_cast<const uint2 *>(c + 48), 2, nullptr, 0, DOM_SHAKE, w);
    keccak_f1600_warp(a, w);
    if (w.lane < 2) reinterpret_cast<uint2 *>(pk + (size_t)x * PKB)[w.lane] = a;
    const uint64_t *sd = reinterpret_cast<const uint64_t *>(c + 24);
    a = seeded_state(0x5F, sd[0], sd[1], sd[2], w);
    uint16_t *St = reinterpret_cast<uint16_t *>(scratch + (size_t)x * SCRATCH), *E = St + N * NB;
    // stream order: S[k*N + j] (k < 8, j < N) then E[i*8 + k]
    warp_noise_stream(a, 2 * N * NB, w, [&](int p, uint16_t v) {
        if (p < N * NB) St[(p % N) * NB + p / N] = v;
        else E[p - N * NB] = v;
    });
}

// G2(pkh || mu) with pkh in lanes 0..2 of `a`, mu at `mu`; then the S' / E' / E'' noise stream.
// Writes k (24 B) and mu (24 B) into the scratch seed area.
__device__ __forceinline__ void g2_and_noise(uint2 a, const uint8_t *mu, uint8_t *scr, const WarpKeccak &w) {
    const uint2 *m = reinterpret_cast<const uint2 *>(mu);
    uint2 g = w.lane < 3 ? a : (w.lane < 6 ? m[w.lane - 3] : make_uint2(0, 0));
    if (w.lane == 6) g.x ^= DOM_SHAKE;
    if (w.lane == SHAKE256_LANES - 1) g.y ^= 0x80000000u;
    keccak_f1600_warp(g, w);
    uint2 *kk = reinterpret_cast<uint2 *>(scr + NOISE_U16 * 2), *mm = reinterpret_cast<uint2 *>(scr + NOISE_U16 * 2 + 32);
    if (w.lane >= 3 && w.lane < 6) kk[w.lane - 3] = g;
    const uint2 mv = w.lane < 3 ? m[w.lane] : make_uint2(0, 0);
    __syncwarp();
    if (w.lane < 3 && mu != scr + NOISE_U16 * 2 + 32) mm[w.lane] = mv;
    const uint64_t s0 = u64(shfl2(g, 0)), s1 = u64(shfl2(g, 1)), s2 = u64(shfl2(g, 2));
    uint2 st = seeded_state(0x96, s0, s1, s2, w);
    warp_noise_stream(st, NOISE_U16, w, [&](int p, uint16_t v) { write_spt(scr, p, v); });
}

// encaps prologue: pkh = G1(pk); (seedSE || k) = G2(pkh || mu); S', E', E'' sampled -> scratch.
// scratch: Spt (N x 8: Spt[k][i] = S'[i][k]), Ep (8 x N), Epp (8 x 8), then k (24) at +NOISE*2,
// mu (24) at +NOISE*2 + 32.
__device__ __forceinline__ void zero_gacc(uint8_t *scr, int lane) {
    uint4 *g = reinterpret_cast<uint4 *>(scr + GACC_OFF);
    for (int i = lane; i < NB * N / 4; i += 32) g[i] = make_uint4(0, 0, 0, 0);
}

// pkh != nullptr: pkh = SHAKE256(pk, 24) is given (the tail of a resident secret key, 24 bytes at
// pkh + x * 24), which skips the 115 serial permutations of hashing the public key.
__global__ void __launch_bounds__(128) fr_enc_pre(int n, const uint8_t *pk, const uint8_t *mu, uint8_t *scratch,
                                                  int split, const uint8_t *pkh) {
    FR_WARP_INSTANCE;
    if (split > 1) zero_gacc(scratch + (size_t)x * SCRATCH, w.lane);
    uint2 a;
    if (pkh) {
        const uint2 *h = reinterpret_cast<const uint2 *>(pkh + (size_t)x * 24);
        a = w.lane < 3 ? h[w.lane] : make_uint2(0, 0);
    } else {
        warp_absorb2<SHAKE256_LANES>(a, reinterpret_cast<const uint2 *>(pk + (size_t)x * PKB), PKB / 8, nullptr, 0,
                                     DOM_SHAKE, w);
        keccak_f1600_warp(a, w);
    }
    g2_and_noise(a, mu + (size_t)x * MUB, scratch + (size_t)x * SCRATCH, w);
}

// decaps, step 1 (CTA per instance): W = C - B' S (frodo_mul_bs + frodo_sub), mu' = decode(W)
// -> scratch mu' slot.  B' and S are staged in shared memory with coalesced loads.
__global__ void __launch_bounds__(256) fr_dec_w(int n, const uint8_t *ct, const uint8_t *sk, uint8_t *scratch) {
    __shared__ __align__(16) uint16_t Bp[NB * N];
    __shared__ __align__(16) uint16_t S[NB * N];
    __shared__ uint32_t W[64];
    const int x = blockIdx.x, tid = threadIdx.x;
    const uint8_t *c = ct + (size_t)x * CTB, *sS = sk + (size_t)x * SKB + SSB + PKB;
    for (int e = tid; e < NB * N; e += blockDim.x) {
        Bp[e] = (uint16_t)ld_be16(c + 2 * e);
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
    if (tid < 8) {  // word g = tid: 8 pieces of 3 bits (key_decode)
        const int g = tid;
        uint32_t templong = 0;
        for (int jj = 0; jj < 8; jj++) {
            const uint32_t wv = (ld_be16(c + C1B + 2 * (g * NB + jj)) - W[g * NB + jj]) & 0xffff;
            const uint32_t t = (wv + (1u << 12)) >> 13;
            templong |= (t & 7) << (3 * jj);
        }
        uint8_t *mu = scratch + (size_t)x * SCRATCH + NOISE_U16 * 2 + 32;
        mu[3 * g] = (uint8_t)templong;
        mu[3 * g + 1] = (uint8_t)(templong >> 8);
        mu[3 * g + 2] = (uint8_t)(templong >> 16);
    }
}

// decaps, step 2 (warp per instance): (seedSE' || k') = G2(pkh || mu'); S', E', E'' -> scratch
__global__ void __launch_bounds__(128) fr_dec_pre(int n, const uint8_t *sk, uint8_t *scratch, int split) {
    FR_WARP_INSTANCE;
    uint8_t *scr = scratch + (size_t)x * SCRATCH;
    if (split > 1) zero_gacc(scr, w.lane);
    const uint2 *pkh = reinterpret_cast<const uint2 *>(sk + (size_t)x * SKB + SSB + PKB + C1B);
    const uint2 a = w.lane < 3 ? pkh[w.lane] : make_uint2(0, 0);
    g2_and_noise(a, scr + NOISE_U16 * 2 + 32, scr, w);
}

// F = SHAKE256(ct || key, 24): encaps key = k; decaps key = fail ? s : k' (constant-time select)
__global__ void __launch_bounds__(128) fr_post(int n, const uint8_t *ct, uint8_t *scratch, const uint8_t *sk, uint8_t *ss) {
    FR_WARP_INSTANCE;
    uint8_t *scr = scratch + (size_t)x * SCRATCH;
    const uint2 *k = reinterpret_cast<const uint2 *>(scr + NOISE_U16 * 2);
    uint2 *key = reinterpret_cast<uint2 *>(scr + NOISE_U16 * 2 + 72);
    if (w.lane < 3) {
        uint2 kv = k[w.lane];
        if (sk) {
            const uint32_t mask = 0u - (uint32_t)(scr[NOISE_U16 * 2 + 64] != 0);
            const uint2 sv = reinterpret_cast<const uint2 *>(sk + (size_t)x * SKB)[w.lane];
            kv = make_uint2(kv.x ^ (mask & (kv.x ^ sv.x)), kv.y ^ (mask & (kv.y ^ sv.y)));
        }
        key[w.lane] = kv;
    }
    __syncwarp();
    uint2 a;
    warp_absorb2<SHAKE256_LANES>(a, reinterpret_cast<const uint2 *>(ct + (size_t)x * CTB), CTB / 8, key, 3, DOM_SHAKE, w);
    keccak_f1600_warp(a, w);
    if (w.lane < 3) reinterpret_cast<uint2 *>(ss + (size_t)x * SSB)[w.lane] = a;
}

// keypair epilogue: sk = s || pk || S (u16 LE, S[k*N + j]) || SHAKE256(pk, 24)
__global__ void __launch_bounds__(128) fr_kp_post(int n, const uint8_t *coins, int cstride, const uint8_t *pk,
                                                  const uint8_t *scratch, uint8_t *sk) {
    FR_WARP_INSTANCE;
    uint8_t *s = sk + (size_t)x * SKB;
    const uint8_t *p = pk + (size_t)x * PKB;
    const uint16_t *St = reinterpret_cast<const uint16_t *>(scratch + (size_t)x * SCRATCH);
    if (w.lane < 3) reinterpret_cast<uint2 *>(s)[w.lane] = reinterpret_cast<const uint2 *>(coins + (size_t)x * cstride)[w.lane];
    for (int i = w.lane; i < PKB / 8; i += 32) reinterpret_cast<uint2 *>(s + SSB)[i] = reinterpret_cast<const uint2 *>(p)[i];
    uint16_t *dS = reinterpret_cast<uint16_t *>(s + SSB + PKB);
    for (int e = w.lane; e < N * NB; e += 32) {
        const int k = e / N, j = e % N;
        dS[e] = St[j * NB + k];
    }
    uint2 a;
    warp_absorb2<SHAKE256_LANES>(a, reinterpret_cast<const uint2 *>(p), PKB / 8, nullptr, 0, DOM_SHAKE, w);
    keccak_f1600_warp(a, w);
    if (w.lane < 3) reinterpret_cast<uint2 *>(s + SSB + PKB + C1B)[w.lane] = a;
}

// ---------------------------------------------------------------------------------------------
// Core kernels: A generated on the fly
// ---------------------------------------------------------------------------------------------
// B = A S + E, one thread per row of A; CTA = (instance, group of rows); St in shared memory.
__global__ void __launch_bounds__(256) fr_kp_core(int n, uint8_t *pk, const uint8_t *scratch) {
    __shared__ __align__(16) uint16_t St[N * NB];
    const int x = blockIdx.y;
    const uint16_t *gSt = reinterpret_cast<const uint16_t *>(scratch + (size_t)x * SCRATCH), *E = gSt + N * NB;
    for (int i = threadIdx.x; i < N * NB / 8; i += blockDim.x)
        reinterpret_cast<uint4 *>(St)[i] = reinterpret_cast<const uint4 *>(gSt)[i];
    __syncthreads();
    const int row = blockIdx.x * blockDim.x + threadIdx.x;
    if (row >= N) return;
    uint8_t *p = pk + (size_t)x * PKB;
    uint2 A[25];
    row_absorb(A, row, reinterpret_cast<const uint2 *>(p));
    uint32_t acc[NB];
#pragma unroll
    for (int k = 0; k < NB; k++) acc[k] = E[row * NB + k];
    for (int blk = 0; blk < ROW_BLOCKS; blk++) {
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
    // pack B row (8 values, 16-bit big-endian) at pk[16 + 16 row]
    uint8_t *o = p + SEEDA + 16 * row;
#pragma unroll
    for (int k = 0; k < NB; k++) {
        o[2 * k] = (uint8_t)(acc[k] >> 8);
        o[2 * k + 1] = (uint8_t)acc[k];
    }
}

// Epilogue of B' = S' A + E': V = S' B + E'' (B = unpack(pk_b), N x 8; 64 outputs, k split over
// the CTA, into acc[NB*N ..]), then B' -> c1 and C = V + encode(mu) -> c2, 16-bit big-endian, or
// compared with the received ciphertext (cmp != nullptr; the fail flag goes to scratch).
// acc holds B' (8 x N, u32, wrapped mod 2^32) and E'' in its last 64 words; Spt is S' (N x 8).
__device__ void sa_epilogue(uint32_t *acc, const uint16_t *Spt, const uint8_t *p, uint8_t *scr, uint8_t *ct,
                            const uint8_t *ct_cmp, int x) {
    const int tid = threadIdx.x, nthr = blockDim.x;
    {
        const uint8_t *pb = p + SEEDA;
        for (int t = tid; t < 64 * 4; t += nthr) {
            const int o = t & 63, part = t >> 6, i = o >> 3, l = o & 7;
            uint32_t sum = 0;
            for (int k = part; k < N; k += 4) sum += (uint32_t)Spt[k * NB + i] * ld_be16(pb + 2 * (k * NB + l));
            atomicAdd(acc + NB * N + o, sum);
        }
    }
    __syncthreads();
    const uint8_t *mu = scr + NOISE_U16 * 2 + 32;
    uint32_t diff = 0;
    for (int e = tid; e < NB * N; e += nthr) {
        const uint32_t v = acc[e] & 0xffff;
        if (ct_cmp) diff |= v ^ ld_be16(ct_cmp + (size_t)x * CTB + 2 * e);
        else {
            ct[(size_t)x * CTB + 2 * e] = (uint8_t)(v >> 8);
            ct[(size_t)x * CTB + 2 * e + 1] = (uint8_t)v;
        }
    }
    for (int e = tid; e < 64; e += nthr) {
        const int g = e >> 3, j = e & 7;
        const uint32_t temp = (uint32_t)mu[3 * g] | ((uint32_t)mu[3 * g + 1] << 8) | ((uint32_t)mu[3 * g + 2] << 16);
        const uint32_t enc = ((temp >> (3 * j)) & 7) << 13;
        const uint32_t v = (acc[NB * N + e] + enc) & 0xffff;
        if (ct_cmp) diff |= v ^ ld_be16(ct_cmp + (size_t)x * CTB + C1B + 2 * e);
        else {
            ct[(size_t)x * CTB + C1B + 2 * e] = (uint8_t)(v >> 8);
            ct[(size_t)x * CTB + C1B + 2 * e + 1] = (uint8_t)v;
        }
    }
    if (ct_cmp) {
        const int any = __syncthreads_or(diff != 0);
        if (tid == 0) scr[NOISE_U16 * 2 + 64] = (uint8_t)any;
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
__global__ void __launch_bounds__(SA_THREADS) fr_sa_core(int n, uint8_t *ct, const uint8_t *ct_cmp, const uint8_t *pk,
                                                         int pk_stride, uint8_t *scratch) {
    extern __shared__ __align__(16) uint8_t smem[];
    uint16_t *Spt = reinterpret_cast<uint16_t *>(smem);                       // N x 8
    uint32_t *acc = reinterpret_cast<uint32_t *>(smem + N * NB * 2);          // 8 x N (+64 for V)
    uint16_t *stage = reinterpret_cast<uint16_t *>(smem + N * NB * 2 + (NB * N + 64) * 4);  // threads x 86
    const int x = blockIdx.x, tid = threadIdx.x, nthr = blockDim.x, parts = gridDim.y;
    const int rows_per = (N + parts - 1) / parts, rbeg = blockIdx.y * rows_per, rend = min(N, rbeg + rows_per);
    uint8_t *scr = scratch + (size_t)x * SCRATCH;
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
        for (int blk = 0; blk < ROW_BLOCKS; blk++) {
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
        uint32_t *g = reinterpret_cast<uint32_t *>(scr + GACC_OFF);
        for (int i = tid; i < NB * N; i += nthr) atomicAdd(g + i, acc[i]);
        return;
    }
    sa_epilogue(acc, Spt, p, scr, ct, ct_cmp, x);
}

// Finish a split product: acc = (sum of the parts) + E', then the same epilogue.  CTA per instance.
__global__ void __launch_bounds__(SA_THREADS) fr_sa_final(int n, uint8_t *ct, const uint8_t *ct_cmp, const uint8_t *pk,
                                                          int pk_stride, uint8_t *scratch) {
    extern __shared__ __align__(16) uint8_t smem[];
    uint16_t *Spt = reinterpret_cast<uint16_t *>(smem);
    uint32_t *acc = reinterpret_cast<uint32_t *>(smem + N * NB * 2);
    const int x = blockIdx.x, tid = threadIdx.x, nthr = blockDim.x;
    uint8_t *scr = scratch + (size_t)x * SCRATCH;
    const uint16_t *gSpt = reinterpret_cast<const uint16_t *>(scr), *Ep = gSpt + N * NB, *Epp = Ep + N * NB;
    const uint32_t *g = reinterpret_cast<const uint32_t *>(scr + GACC_OFF);
    for (int i = tid; i < N * NB / 8; i += nthr) reinterpret_cast<uint4 *>(Spt)[i] = reinterpret_cast<const uint4 *>(gSpt)[i];
    for (int i = tid; i < NB * N; i += nthr) acc[i] = g[i] + Ep[i];
    for (int i = tid; i < 64; i += nthr) acc[NB * N + i] = Epp[i];
    __syncthreads();
    sa_epilogue(acc, Spt, pk + (size_t)x * pk_stride, scr, ct, ct_cmp, x);
}

static size_t sa_smem(int threads) { return (size_t)N * NB * 2 + ((size_t)NB * N + 64) * 4 + (size_t)threads * STAGE_PITCH * 2; }
static size_t sa_final_smem() { return (size_t)N * NB * 2 + ((size_t)NB * N + 64) * 4; }

}  // namespace frodo

using namespace frodo;

int frodo_init_constants() {
    const uint16_t cdf[11] = {5638, 15915, 23689, 28571, 31116, 32217, 32613, 32731, 32760, 32766, 32767};
    uint2 rc[24];
    keccak_rc_host(rc);
    if (cudaMemcpyToSymbol(c_keccak_rc, rc, sizeof rc) != cudaSuccess) return PQCGPU_ECUDA;
    if (cudaMemcpyToSymbol(c_cdf, cdf, sizeof cdf) != cudaSuccess) return PQCGPU_ECUDA;
    return PQCGPU_OK;
}
size_t frodo_scratch_bytes() { return SCRATCH; }

// Launch shapes.  Keypair: threads per CTA of fr_kp_core (one row of A per thread).  Encaps /
// decaps: row parts per instance for B' = S' A + E' and threads per CTA of fr_sa_core.  0 = chosen
// by batch size: small batches split an instance over several CTAs (latency), large ones keep one
// CTA per instance (no split traffic).  Set through pqcgpu_set_launch_shape (the autotuner).
static int g_fr_parts[3] = {0, 0, 0}, g_fr_threads[3] = {0, 0, 0};

static void fr_shape(int op, int n, int *parts, int *threads) {
    if (op == 0) {
        *parts = 1;
        *threads = g_fr_threads[0] ? g_fr_threads[0] : (n >= 152 ? 256 : 64);
        return;
    }
    if (g_fr_parts[op]) {
        *parts = g_fr_parts[op];
        *threads = g_fr_threads[op];
        return;
    }
    if (n >= 304) *parts = 1, *threads = 256;
    else if (n >= 152) *parts = 2, *threads = 256;
    else if (n >= 76) *parts = 4, *threads = 256;
    else *parts = 8, *threads = 128;
}

int frodo_set_shape(int op, int parts, int threads) {
    if (op == 0) {
        if (parts > 1 || !(threads == 0 || threads == 64 || threads == 128 || threads == 256)) return PQCGPU_EINVAL;
        g_fr_threads[0] = threads;
        return PQCGPU_OK;
    }
    if (op != 1 && op != 2) return PQCGPU_EINVAL;
    if (parts == 0) {
        g_fr_parts[op] = g_fr_threads[op] = 0;
        return PQCGPU_OK;
    }
    if (!(parts == 1 || parts == 2 || parts == 4 || parts == 8 || parts == 16) || !(threads == 128 || threads == 256))
        return PQCGPU_EINVAL;
    g_fr_parts[op] = parts;
    g_fr_threads[op] = threads;
    return PQCGPU_OK;
}

int frodo_get_shape(int op, int *parts, int *threads) {
    if (op < 0 || op > 2) return PQCGPU_EINVAL;
    *parts = op == 0 ? 1 : g_fr_parts[op];
    *threads = g_fr_threads[op];
    return PQCGPU_OK;
}

int frodo_keypair_dev(int n, uint8_t *pk, uint8_t *sk, const uint8_t *coins, int cstride, uint8_t *scratch,
                      cudaStream_t st) {
    int parts, thr;
    fr_shape(0, n, &parts, &thr);
    PQC_LAUNCH(st, "fr_kp_pre", 976, 0, fr_kp_pre<<<(n + 3) / 4, 128, 0, st>>>(n, coins, cstride, pk, scratch));
    PQC_LAUNCH(st, "fr_kp_core", 976, 0, fr_kp_core<<<dim3((N + thr - 1) / thr, n), thr, 0, st>>>(n, pk, scratch));
    PQC_LAUNCH(st, "fr_kp_post", 976, 0, fr_kp_post<<<(n + 3) / 4, 128, 0, st>>>(n, coins, cstride, pk, scratch, sk));
    return cudaGetLastError() == cudaSuccess ? PQCGPU_OK : PQCGPU_ECUDA;
}

// B' = S' A + E' and the ciphertext epilogue: one CTA per instance, or `parts` CTAs per instance
// plus fr_sa_final.
static void launch_sa(int n, uint8_t *ct, const uint8_t *ct_cmp, const uint8_t *pk, int pk_stride, uint8_t *scratch,
                      int parts, int thr, cudaStream_t st) {
    PQC_LAUNCH(st, "fr_sa_core", 976, 0,
               fr_sa_core<<<dim3(n, parts), thr, sa_smem(thr), st>>>(n, ct, ct_cmp, pk, pk_stride, scratch));
    if (parts > 1)
        PQC_LAUNCH(st, "fr_sa_final", 976, 0,
                   fr_sa_final<<<n, SA_THREADS, sa_final_smem(), st>>>(n, ct, ct_cmp, pk, pk_stride, scratch));
}

static int sa_attrs() {
    if (capturing()) return PQCGPU_OK;
    if (cudaFuncSetAttribute(fr_sa_core, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sa_smem(SA_THREADS)) !=
        cudaSuccess) {
        cudaGetLastError();
        return PQCGPU_ECUDA;
    }
    return PQCGPU_OK;
}

int frodo_enc_dev(int n, uint8_t *ct, uint8_t *ss, const uint8_t *pk, const uint8_t *mu, uint8_t *scratch,
                  cudaStream_t st, const uint8_t *pkh) {
    if (sa_attrs()) return PQCGPU_ECUDA;
    int parts, thr;
    fr_shape(1, n, &parts, &thr);
    PQC_LAUNCH(st, "fr_enc_pre", 976, 0, fr_enc_pre<<<(n + 3) / 4, 128, 0, st>>>(n, pk, mu, scratch, parts, pkh));
    launch_sa(n, ct, nullptr, pk, PKB, scratch, parts, thr, st);
    PQC_LAUNCH(st, "fr_post", 976, 0, fr_post<<<(n + 3) / 4, 128, 0, st>>>(n, ct, scratch, nullptr, ss));
    return cudaGetLastError() == cudaSuccess ? PQCGPU_OK : PQCGPU_ECUDA;
}

int frodo_dec_dev(int n, uint8_t *ss, const uint8_t *ct, const uint8_t *sk, uint8_t *scratch, cudaStream_t st) {
    if (sa_attrs()) return PQCGPU_ECUDA;
    int parts, thr;
    fr_shape(2, n, &parts, &thr);
    PQC_LAUNCH(st, "fr_dec_w", 976, 0, fr_dec_w<<<n, 256, 0, st>>>(n, ct, sk, scratch));
    PQC_LAUNCH(st, "fr_dec_pre", 976, 0, fr_dec_pre<<<(n + 3) / 4, 128, 0, st>>>(n, sk, scratch, parts));
    launch_sa(n, nullptr, ct, sk + SSB, SKB, scratch, parts, thr, st);
    PQC_LAUNCH(st, "fr_post", 976, 0, fr_post<<<(n + 3) / 4, 128, 0, st>>>(n, ct, scratch, sk, ss));
    return cudaGetLastError() == cudaSuccess ? PQCGPU_OK : PQCGPU_ECUDA;
}

}  // namespace pqc
