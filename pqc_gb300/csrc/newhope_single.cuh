// Single-instance NewHope KEM kernels: the latency path for small batches (implementation header,
// included by newhope.cu after the batched bodies, whose samplers, transforms and codecs it uses).
//
// One CTA of NHS_WARPS warps runs a whole keypair or encapsulation of one instance in one launch,
// in the manner of the reference's single-instance build (NewHope_NIST_GPU_Single: a CTA of
// cooperating threads per operation, ntt.cu:1015-1091, poly.cu:299-411):
//   * the serial hashes (SHAKE256 of the seed or of the coins, and ss = SHAKE256(m)) run on the
//     25-lane warp permutation (keccak.cuh), about half the latency of a one-thread permutation;
//   * the noise chunks (one-block SHAKE256 sponges, 32 or 48 of them) run a thread each, all at
//     once on one or two warps;
//   * the public polynomial a-hat is sampled beside the noise, a chunk per warp on the other
//     warps: after each SHAKE128 block every lane checks its four 16-bit candidates, and three
//     ballots give each lane its prefix count, so the accepted values land in stream order, the
//     first 64 of each chunk exactly as in the thread sampler (poly_uniform, poly.cu:332-372);
//     a-hat is staged in shared memory and used once the noise is in the NTT domain;
//   * the transforms are the batched kernels' (a warp per 1024-point polynomial, a half-warp per
//     512-point one), and the pointwise products, the noise additions, the message encoding and
//     the codecs run on all threads, with the batched bodies' arithmetic expression for
//     expression, so every byte equals the batched path's.
#pragma once

namespace pqc {
namespace newhope {

constexpr int NHS_WARPS = 16;
constexpr int NHS_THREADS = NHS_WARPS * 32;

// Shared memory of one instance: five polynomials (s, e, a-hat, v, e''), the public key, 128 B of
// seeds.
template <int N>
struct NhSingleSmem {
    uint16_t *s, *e, *a, *v, *e2;
    uint8_t *pk;
    uint2 *seeds;  // [0, 4) m or publicseed, [4, 8) coin or noiseseed
    __device__ __forceinline__ explicit NhSingleSmem(uint8_t *smem) {
        s = reinterpret_cast<uint16_t *>(smem);
        e = s + Nh<N>::PITCH;
        a = e + Nh<N>::PITCH;
        v = a + Nh<N>::PITCH;
        e2 = v + Nh<N>::PITCH;
        pk = reinterpret_cast<uint8_t *>(e2 + Nh<N>::PITCH);
        seeds = reinterpret_cast<uint2 *>(pk + ((Nh<N>::PKB + 15) & ~15));
    }
    static __host__ __device__ constexpr size_t bytes() {
        return (size_t)5 * Nh<N>::PITCH * 2 + ((Nh<N>::PKB + 15) & ~15) + 128;
    }
};

// poly_uniform chunk `chunk` of SHAKE128(seed || chunk) by one warp: emit(j, value) for the first
// 64 candidates below 5q in stream order (lane l < 21 holds candidates 4l .. 4l + 3 of a block).
template <class F>
__device__ __forceinline__ void warp_uniform_chunk(const uint2 *seed, int chunk, F emit, const WarpKeccak &w) {
    uint2 a = w.lane < 4 ? seed[w.lane] : make_uint2(0, 0);
    if (w.lane == 4) a.x = (uint32_t)chunk | (DOM_SHAKE << 8);
    if (w.lane == SHAKE128_LANES - 1) a.y ^= 0x80000000u;
    const unsigned below = (1u << w.lane) - 1u;
    int cnt = 0;
    while (cnt < 64) {  // warp-uniform
        keccak_f1600_warp(a, w);
        const uint32_t c[4] = {a.x & 0xffff, a.x >> 16, a.y & 0xffff, a.y >> 16};
        bool ok[4];
        int k = 0;
#pragma unroll
        for (int i = 0; i < 4; i++) {
            ok[i] = w.lane < SHAKE128_LANES && c[i] < 5 * Q;
            k += ok[i];
        }
        const unsigned b0 = __ballot_sync(0xffffffffu, k & 1), b1 = __ballot_sync(0xffffffffu, k & 2),
                       b2 = __ballot_sync(0xffffffffu, k & 4);
        int pos = cnt + __popc(b0 & below) + 2 * __popc(b1 & below) + 4 * __popc(b2 & below);
#pragma unroll
        for (int i = 0; i < 4; i++)
            if (ok[i]) {
                if (pos < 64) emit(pos, c[i]);
                pos++;
            }
        cnt += __popc(b0) + 2 * __popc(b1) + 4 * __popc(b2);
    }
    __syncwarp();
}

// SHAKE256 of 32 bytes (lanes 0-3 of `in`) by one warp; lanes 0-7 of the result (64 bytes).
__device__ __forceinline__ uint2 warp_shake256_32(const uint2 *in, const WarpKeccak &w) {
    uint2 a = w.lane < 4 ? in[w.lane] : make_uint2(0, 0);
    if (w.lane == 4) a.x ^= DOM_SHAKE;
    if (w.lane == SHAKE256_LANES - 1) a.y ^= 0x80000000u;
    keccak_f1600_warp(a, w);
    return a;
}

// The two forward transforms of s and e (1024: a warp each, warps 0 and 1; 512: warp 0, a half each).
template <int N>
__device__ __forceinline__ void nhs_ntt2(const NhSingleSmem<N> &S, int warp, int lane) {
    if constexpr (N == 1024) {
        if (warp < 2) ntt_warp(warp ? S.e : S.s, lane);
    } else {
        if (warp == 0) ntt512_half(lane < 16 ? S.s : S.e, lane & 15, true);
    }
}

// Keypair: (publicseed, noiseseed) = SHAKE256(seed, 64); s, e noise; a-hat; b-hat = e-hat + s-hat o
// a-hat; pk = b-hat || publicseed, sk = s-hat (cpapke_keypair, NewHope_NIST_GPU/cpapke.cu:265-316).
template <int N>
__global__ void __launch_bounds__(NHS_THREADS) nh_kp_single(const uint8_t *seed, int seed_stride, uint8_t *pk,
                                                            uint8_t *sk) {
    using P = Nh<N>;
    constexpr int NCH = P::NCH;
    extern __shared__ __align__(16) uint8_t smem[];
    const NhSingleSmem<N> S(smem);
    const int x = blockIdx.x, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const WarpKeccak w(lane);
    if (warp == 0) {
        const uint2 h = warp_shake256_32(reinterpret_cast<const uint2 *>(seed + (size_t)x * seed_stride), w);
        if (lane < 8) S.seeds[lane] = h;
    }
    __syncthreads();
    if (warp == 1) {  // s (nonce 0) and e (nonce 1): a chunk per thread
        if (lane < 2 * NCH) {
            const int pl = lane / NCH, ch = lane % NCH;
            uint16_t *dst = pl ? S.e : S.s;
            sample_chunk(S.seeds + 4, pl, ch, [&](int j, uint32_t c0, uint32_t c1) {
                *reinterpret_cast<uint32_t *>(dst + phys(64 * ch + j)) = (c0 & 0xffff) | (c1 << 16);
            });
        }
    } else if (warp >= 2) {  // a-hat, a chunk per warp, meanwhile
        for (int ch = warp - 2; ch < NCH; ch += NHS_WARPS - 2)
            warp_uniform_chunk(S.seeds, ch, [&](int j, uint32_t av) { S.a[phys(64 * ch + j)] = (uint16_t)av; }, w);
    }
    __syncthreads();
    nhs_ntt2<N>(S, warp, lane);
    __syncthreads();
    for (int i = tid; i < N; i += NHS_THREADS) {  // b-hat = e-hat + s-hat o a-hat (nh_kp_body)
        const int idx = phys(i);
        const uint32_t t = mont(3186u * S.a[idx]);
        const uint32_t r = mont((uint32_t)S.s[idx] * t);
        S.e[idx] = (uint16_t)((S.e[idx] + r) % Q);
    }
    __syncthreads();
    uint8_t *ski = sk + (size_t)x * P::SKB, *pki = pk + (size_t)x * P::PKB;
    for (int g = tid; g < N / 4; g += NHS_THREADS) {
        uint8_t o[7];
        tobytes4(o, S.s[phys(4 * g)], S.s[phys(4 * g + 1)], S.s[phys(4 * g + 2)], S.s[phys(4 * g + 3)]);
#pragma unroll
        for (int q = 0; q < 7; q++) ski[7 * g + q] = o[q];
        tobytes4(o, S.e[phys(4 * g)], S.e[phys(4 * g + 1)], S.e[phys(4 * g + 2)], S.e[phys(4 * g + 3)]);
#pragma unroll
        for (int q = 0; q < 7; q++) pki[7 * g + q] = o[q];
    }
    if (tid < 4) reinterpret_cast<uint2 *>(pki + P::POLYBYTES)[tid] = S.seeds[tid];
}

// Encryption: s', e', e'' noise from coin; a-hat; u-hat = a-hat o s'-hat + e'-hat, v = invNTT(b-hat o
// s'-hat) + e'' + encode(m); ct = u-hat || compress(v) (cpapke_enc, NewHope_NIST_GPU/cpapke.cu:
// 333-404).  KEM: (m, coin) = SHAKE256(coins, 64) and ss = SHAKE256(m, 32) (the CPA-KEM); CPA: m and
// coin are given (32 bytes each per instance at coins and m_in), ss is not written.
template <int N, bool KEM>
__global__ void __launch_bounds__(NHS_THREADS) nh_enc_single(const uint8_t *pk, const uint8_t *coins, const uint8_t *m_in,
                                                             uint8_t *ct, uint8_t *ss) {
    using P = Nh<N>;
    constexpr int NCH = P::NCH;
    extern __shared__ __align__(16) uint8_t smem[];
    const NhSingleSmem<N> S(smem);
    const int x = blockIdx.x, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const WarpKeccak w(lane);
    const uint8_t *pki = pk + (size_t)x * P::PKB;
    for (int i = tid; i < P::PKB / 8; i += NHS_THREADS)  // the public key, coalesced
        reinterpret_cast<uint2 *>(S.pk)[i] = reinterpret_cast<const uint2 *>(pki)[i];
    if (warp == 0) {
        if constexpr (KEM) {
            const uint2 h = warp_shake256_32(reinterpret_cast<const uint2 *>(coins + (size_t)x * 32), w);
            if (lane < 8) S.seeds[4 + lane] = h;  // [4, 8) m, [8, 12) coin
        } else if (lane < 8) {
            S.seeds[4 + lane] = reinterpret_cast<const uint2 *>(lane < 4 ? m_in + (size_t)x * 32 : coins + (size_t)x * 32)[lane & 3];
        }
    }
    __syncthreads();
    const uint2 *m2 = S.seeds + 4, *coin = S.seeds + 8;
    if (warp == 0) {  // KEM: ss = SHAKE256(m, 32); then e'' (nonce 2): a chunk per thread
        if constexpr (KEM) {
            const uint2 h = warp_shake256_32(m2, w);
            if (lane < 4) reinterpret_cast<uint2 *>(ss + (size_t)x * 32)[lane] = h;
        }
        if (lane < NCH)
            sample_chunk(coin, 2, lane, [&](int j, uint32_t c0, uint32_t c1) {
                *reinterpret_cast<uint32_t *>(S.e2 + phys(64 * lane + j)) = (c0 & 0xffff) | (c1 << 16);
            });
    } else if (warp == 1) {  // s' (nonce 0) and e' (nonce 1)
        if (lane < 2 * NCH) {
            const int pl = lane / NCH, ch = lane % NCH;
            uint16_t *dst = pl ? S.e : S.s;
            sample_chunk(coin, pl, ch, [&](int j, uint32_t c0, uint32_t c1) {
                *reinterpret_cast<uint32_t *>(dst + phys(64 * ch + j)) = (c0 & 0xffff) | (c1 << 16);
            });
        }
    } else {  // a-hat from the public seed, a chunk per warp, meanwhile
        const uint2 *pseed = reinterpret_cast<const uint2 *>(S.pk + P::POLYBYTES);
        for (int ch = warp - 2; ch < NCH; ch += NHS_WARPS - 2)
            warp_uniform_chunk(pseed, ch, [&](int j, uint32_t av) { S.a[phys(64 * ch + j)] = (uint16_t)av; }, w);
    }
    __syncthreads();
    nhs_ntt2<N>(S, warp, lane);
    __syncthreads();
    for (int i = tid; i < N; i += NHS_THREADS) {  // u-hat = a-hat o s' + e'; v = b-hat o s' (nh_enc_body)
        const int idx = phys(i);
        const uint32_t t = mont(3186u * S.s[idx]);
        const uint32_t u = mont((uint32_t)S.a[idx] * t);
        S.e[idx] = (uint16_t)((u + S.e[idx]) % Q);
        uint32_t bh[4];
        frombytes4(bh, S.pk + 7 * (i >> 2));
        S.v[idx] = (uint16_t)mont(bh[i & 3] * t);
    }
    __syncthreads();
    if constexpr (N == 1024) {
        if (warp == 0) invntt_warp(S.v, lane);
    } else {
        if (warp == 0) invntt512_half(S.v, lane & 15, lane < 16);
    }
    __syncthreads();
    const uint8_t *m = reinterpret_cast<const uint8_t *>(m2);
    for (int i = tid; i < N; i += NHS_THREADS) {  // v += e'' + encode(m), compress
        const int idx = phys(i);
        uint32_t xv = (S.v[idx] + (uint32_t)S.e2[idx]) % Q;
        const uint32_t mb = (m[(i & 255) >> 3] >> (i & 7)) & 1;
        xv = (xv + (mb ? Q / 2 : 0)) % Q;
        S.v[idx] = (uint16_t)compress_coeff(xv);
    }
    __syncthreads();
    uint8_t *cti = ct + (size_t)x * P::CTB;
    for (int g = tid; g < N / 4; g += NHS_THREADS) {
        uint8_t o[7];
        tobytes4(o, S.e[phys(4 * g)], S.e[phys(4 * g + 1)], S.e[phys(4 * g + 2)], S.e[phys(4 * g + 3)]);
#pragma unroll
        for (int q = 0; q < 7; q++) cti[7 * g + q] = o[q];
    }
    for (int g = tid; g < N / 8; g += NHS_THREADS) {  // 8 compressed 3-bit values -> 3 bytes
        uint32_t t[8];
#pragma unroll
        for (int q = 0; q < 8; q++) t[q] = S.v[phys(8 * g + q)];
        uint8_t *r = cti + P::POLYBYTES + 3 * g;
        r[0] = (uint8_t)(t[0] | (t[1] << 3) | (t[2] << 6));
        r[1] = (uint8_t)((t[2] >> 2) | (t[3] << 1) | (t[4] << 4) | (t[5] << 7));
        r[2] = (uint8_t)((t[5] >> 1) | (t[6] << 2) | (t[7] << 5));
    }
}

}  // namespace newhope
}  // namespace pqc
