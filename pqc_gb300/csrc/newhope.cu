// Batched NewHope-1024 CPA-PKE and CPA-KEM for sm_103a.
//
// Replaces cpapke_keypair / cpapke_enc / cpapke_dec (NewHope_NIST_GPU/cpapke.cu:265-476, one thread
// per instance, every polynomial in HBM in a coefficient-major layout) with one core kernel per
// operation:
//   - noise and the public polynomial a-hat in chunks of 64 coefficients, one Keccak permutation
//     per thread (poly_sample / poly_uniform, NewHope_NIST_GPU/poly.cu:332-444), written straight
//     into shared memory or consumed on the spot (a-hat never exists whole);
//   - the 1024-point NTT by one warp per polynomial, 32 coefficients per lane, two passes of five
//     layers in registers with one transpose through shared memory;
//   - packing by one warp per instance;
//   - Keccak with the round loop rolled (keccak_f1600_rolled): the kernels have several sampler
//     call sites, and the unrolled copies stalled instruction fetch (encapsulation +2.5 %).
// Arithmetic mirrors the reference operation for operation (NewHope_NIST_GPU/reduce.cu:22-47,
// ntt.cu:92-234, poly.cu:19-508), uint16 truncations and uint32 wrap-around included, so every
// intermediate value equals the reference's.
#include <cuda_runtime.h>
#include <stdint.h>

#include "keccak.cuh"
#include "pqcgpu_internal.h"

namespace pqc {
namespace newhope {

constexpr int N = 1024;
constexpr uint32_t Q = 12289;
constexpr int POLYBYTES = 1792, PKB = 1824, SKB = 1792, CTB = 2176, COMPB = 384;
constexpr int PITCH = 1280;  // uint16 per shared polynomial: 8 pad after every 32 coefficients

// Tables generated on the host (g = 7, mont = 2^18 mod q; NewHope_NIST_GPU/precomp.cu:27-29).
static __device__ uint16_t d_gammas_bitrev[N];
static __device__ uint16_t d_omegas_inv_bitrev[N / 2];
static __device__ uint16_t d_gammas_inv[N];

__device__ __forceinline__ int phys(int i) { return i + ((i >> 5) << 3); }

__device__ __forceinline__ uint32_t mont(uint32_t a) {
    uint32_t u = a * 12287u;
    u &= (1u << 18) - 1;
    u *= Q;
    a = a + u;
    return (a >> 18) & 0xffffu;
}
__device__ __forceinline__ uint32_t barrett(uint32_t a16) {
    const uint32_t a = a16 & 0xffffu;
    uint32_t u = (a * 5) >> 16;
    u *= Q;
    return (a - u) & 0xffffu;
}
__device__ __forceinline__ uint32_t freeze(uint32_t x) {
    const uint32_t r = (x & 0xffffu) % Q;
    const uint32_t m = (r - Q) & 0xffffu;
    const int32_t c = (int16_t)m >> 15;
    return (m ^ ((r ^ m) & (uint32_t)c)) & 0xffffu;
}
__device__ __forceinline__ uint32_t flipabs(uint32_t x) {
    int32_t r = (int16_t)freeze(x);
    r = (int16_t)(r - (int32_t)(Q / 2));
    const int32_t m = (int16_t)r >> 15;
    return (uint32_t)((r + m) ^ m) & 0xffffu;
}
// butterfly of ntt(): a <- a + b (even layer) or barrett(a + b) (odd layer); b <- mont(W (a + 3q - b))
__device__ __forceinline__ void bfly(uint32_t &a, uint32_t &b, uint32_t W, bool odd) {
    const uint32_t temp = a;
    a = odd ? barrett(temp + b) : ((temp + b) & 0xffffu);
    b = mont(W * (temp + 3 * Q - b));
}

// Forward transform (poly_ntt, poly.cu:519-531): mul_coefficients(gammas_bitrev) then
// ntt(gammas_bitrev as omega).  Layer i pairs j, j + 2^i with twiddle omega[j >> (i + 1)].
__device__ void ntt_warp(uint16_t *p, int lane) {
    uint32_t r[32];
    uint16_t *pa = p + phys(32 * lane);
#pragma unroll
    for (int v = 0; v < 4; v++) {
        const uint4 w = reinterpret_cast<const uint4 *>(pa)[v];
        const uint32_t ws[4] = {w.x, w.y, w.z, w.w};
#pragma unroll
        for (int h = 0; h < 4; h++) {
            r[8 * v + 2 * h] = ws[h] & 0xffffu;
            r[8 * v + 2 * h + 1] = ws[h] >> 16;
        }
    }
#pragma unroll
    for (int q = 0; q < 32; q++) r[q] = mont(r[q] * __ldg(&d_gammas_bitrev[32 * lane + q]));
#pragma unroll
    for (int i = 0; i < 5; i++)
#pragma unroll
        for (int q = 0; q < 32; q++)
            if (!((q >> i) & 1)) bfly(r[q], r[q + (1 << i)], __ldg(&d_gammas_bitrev[(32 * lane + q) >> (i + 1)]), i & 1);
#pragma unroll
    for (int v = 0; v < 4; v++)
        reinterpret_cast<uint4 *>(pa)[v] =
            make_uint4(r[8 * v] | (r[8 * v + 1] << 16), r[8 * v + 2] | (r[8 * v + 3] << 16),
                       r[8 * v + 4] | (r[8 * v + 5] << 16), r[8 * v + 6] | (r[8 * v + 7] << 16));
    __syncwarp();
#pragma unroll
    for (int q = 0; q < 32; q++) r[q] = p[phys(lane + 32 * q)];
#pragma unroll
    for (int i = 5; i < 10; i++)
#pragma unroll
        for (int q = 0; q < 32; q++)
            if (!((q >> (i - 5)) & 1)) bfly(r[q], r[q + (1 << (i - 5))], __ldg(&d_gammas_bitrev[q >> (i - 4)]), i & 1);
#pragma unroll
    for (int q = 0; q < 32; q++) p[phys(lane + 32 * q)] = (uint16_t)r[q];
    __syncwarp();
}

// Inverse transform (poly_invntt, poly.cu:541-547): bitrev_vector, ntt(omegas_inv_bitrev),
// mul_coefficients(gammas_inv).  The bit reversal is folded into the first pass's loads.
__device__ void invntt_warp(uint16_t *p, int lane) {
    uint32_t r[32];
    const int lrev = __brev(lane) >> 27;
#pragma unroll
    for (int q = 0; q < 32; q++) {
        const int qrev = __brev(q) >> 27;
        r[q] = p[phys(32 * qrev + lrev)];  // x'[32 lane + q] = x[brv10(32 lane + q)]
    }
    __syncwarp();
#pragma unroll
    for (int i = 0; i < 5; i++)
#pragma unroll
        for (int q = 0; q < 32; q++)
            if (!((q >> i) & 1))
                bfly(r[q], r[q + (1 << i)], __ldg(&d_omegas_inv_bitrev[(32 * lane + q) >> (i + 1)]), i & 1);
    uint16_t *pa = p + phys(32 * lane);
#pragma unroll
    for (int v = 0; v < 4; v++)
        reinterpret_cast<uint4 *>(pa)[v] =
            make_uint4(r[8 * v] | (r[8 * v + 1] << 16), r[8 * v + 2] | (r[8 * v + 3] << 16),
                       r[8 * v + 4] | (r[8 * v + 5] << 16), r[8 * v + 6] | (r[8 * v + 7] << 16));
    __syncwarp();
#pragma unroll
    for (int q = 0; q < 32; q++) r[q] = p[phys(lane + 32 * q)];
#pragma unroll
    for (int i = 5; i < 10; i++)
#pragma unroll
        for (int q = 0; q < 32; q++)
            if (!((q >> (i - 5)) & 1))
                bfly(r[q], r[q + (1 << (i - 5))], __ldg(&d_omegas_inv_bitrev[q >> (i - 4)]), i & 1);
#pragma unroll
    for (int q = 0; q < 32; q++) p[phys(lane + 32 * q)] = (uint16_t)mont(r[q] * __ldg(&d_gammas_inv[lane + 32 * q]));
    __syncwarp();
}

// ---- samplers (one 64-coefficient chunk per thread) ----
// poly_sample chunk i: SHAKE256(seed || nonce || i) 128 bytes, coeff = HW(b[2j]) + q - HW(b[2j+1])
template <class F>
__device__ __forceinline__ void sample_chunk(const uint2 *seed, int nonce, int chunk, F emit) {
    uint2 A[25];
    keccak_zero(A);
#pragma unroll
    for (int i = 0; i < 4; i++) A[i] = seed[i];
    A[4].x = (uint32_t)nonce | ((uint32_t)chunk << 8) | (DOM_SHAKE << 16);
    A[SHAKE256_LANES - 1].y ^= 0x80000000u;
    keccak_f1600_rolled(A);
#pragma unroll
    for (int w = 0; w < 32; w++) {  // word w = bytes 4w..4w+3 -> coefficients 2w, 2w+1
        const uint32_t t = (w & 1) ? A[w >> 1].y : A[w >> 1].x;
        const uint32_t c0 = __popc(t & 0xff) + Q - __popc((t >> 8) & 0xff);
        const uint32_t c1 = __popc((t >> 16) & 0xff) + Q - __popc(t >> 24);
        emit(2 * w, c0, c1);
    }
}
// poly_uniform chunk i: SHAKE128(seed || i), 16-bit candidates < 5q, 64 accepted (kept unreduced)
template <class F>
__device__ __forceinline__ void uniform_chunk(const uint2 *seed, int chunk, F emit) {
    uint2 A[25];
    keccak_zero(A);
#pragma unroll
    for (int i = 0; i < 4; i++) A[i] = seed[i];
    A[4].x = (uint32_t)chunk | (DOM_SHAKE << 8);
    A[SHAKE128_LANES - 1].y ^= 0x80000000u;
    int ctr = 0;
    while (ctr < 64) {
        keccak_f1600_rolled(A);
#pragma unroll
        for (int w = 0; w < 42; w++) {
            const uint32_t t = (w & 1) ? A[w >> 1].y : A[w >> 1].x;
            const uint32_t v0 = t & 0xffff, v1 = t >> 16;
            if (v0 < 5 * Q && ctr < 64) emit(ctr++, v0);
            if (v1 < 5 * Q && ctr < 64) emit(ctr++, v1);
        }
    }
}

// ---- codecs ----
// 14-bit serialisation of 4 coefficients -> 7 bytes (poly_tobytes, poly.cu:104-124)
__device__ __forceinline__ void tobytes4(uint8_t *r, uint32_t a, uint32_t b, uint32_t c, uint32_t d) {
    const uint32_t t0 = freeze(a), t1 = freeze(b), t2 = freeze(c), t3 = freeze(d);
    r[0] = (uint8_t)t0;
    r[1] = (uint8_t)((t0 >> 8) | (t1 << 6));
    r[2] = (uint8_t)(t1 >> 2);
    r[3] = (uint8_t)((t1 >> 10) | (t2 << 4));
    r[4] = (uint8_t)(t2 >> 4);
    r[5] = (uint8_t)((t2 >> 12) | (t3 << 2));
    r[6] = (uint8_t)(t3 >> 6);
}
__device__ __forceinline__ void frombytes4(uint32_t (&c)[4], const uint8_t *a) {
    c[0] = a[0] | (((uint32_t)a[1] & 0x3f) << 8);
    c[1] = (a[1] >> 6) | ((uint32_t)a[2] << 2) | (((uint32_t)a[3] & 0x0f) << 10);
    c[2] = (a[3] >> 4) | ((uint32_t)a[4] << 4) | (((uint32_t)a[5] & 0x03) << 12);
    c[3] = (a[5] >> 2) | ((uint32_t)a[6] << 6);
}
// coefficient i of the polynomial serialised at `bytes` (14 bits)
__device__ __forceinline__ uint32_t coeff_from_bytes(const uint8_t *bytes, int i) {
    uint32_t c[4];
    frombytes4(c, bytes + 7 * (i >> 2));
    return c[i & 3];
}
__device__ __forceinline__ uint32_t decompress_coeff(const uint8_t *cb, int i) {
    // 3-bit values packed LSB-first, 8 per 3 bytes (poly_decompress, poly.cu:197-216)
    const int bit = 3 * i;
    const uint32_t w = cb[bit >> 3] | ((uint32_t)cb[(bit >> 3) + 1 < COMPB ? (bit >> 3) + 1 : (bit >> 3)] << 8);
    const uint32_t t = (w >> (bit & 7)) & 7;
    return (t * Q + 4) >> 3;
}
__device__ __forceinline__ uint32_t compress_coeff(uint32_t x) { return (((freeze(x) << 3) + Q / 2) / Q) & 7; }

// ---------------------------------------------------------------------------------------------
// Kernels.  Shared layout: NPOLY polynomials per instance, then 128 B of seeds per instance.
// ---------------------------------------------------------------------------------------------
struct KpArgs {
    int n;
    uint8_t *pk, *sk;
    const uint8_t *seed;  // 32 B per instance
    int seed_stride;
};
struct EncArgs {
    int n;
    uint8_t *ct;
    const uint8_t *pk;
    const uint8_t *m, *coin;  // 32 B each per instance
    int m_stride, coin_stride;
};
struct DecArgs {
    int n;
    uint8_t *m_out;  // CPA: message; KEM: ss = SHAKE256(message, 32)
    const uint8_t *ct, *sk;
    int kem;
};

__device__ __forceinline__ uint16_t *npoly(uint16_t *polys, int per, int li, int s) {
    return polys + ((size_t)li * per + s) * PITCH;
}

// keypair: slots 0 s-hat, 1 e-hat -> b-hat
__global__ void __launch_bounds__(256) nh_kp_core(KpArgs a, int NI) {
    extern __shared__ __align__(16) uint8_t smem[];
    uint16_t *polys = reinterpret_cast<uint16_t *>(smem);
    uint8_t *seeds = smem + (size_t)NI * 2 * PITCH * 2;
    const int base = blockIdx.x * NI, ni = min(NI, a.n - base);
    const int tid = threadIdx.x, nthr = blockDim.x, lane = tid & 31, warp = tid >> 5, nwarp = nthr >> 5;
    // publicseed || noiseseed = SHAKE256(seed, 64)
    for (int li = tid; li < ni; li += nthr) {
        uint2 A[25];
        keccak_absorb_lanes<SHAKE256_LANES>(A, reinterpret_cast<const uint2 *>(a.seed + (size_t)(base + li) * a.seed_stride),
                                            4, DOM_SHAKE);
        keccak_f1600_rolled(A);
        uint2 *o = reinterpret_cast<uint2 *>(seeds + li * 128);
#pragma unroll
        for (int i = 0; i < 8; i++) o[i] = A[i];
    }
    __syncthreads();
    for (int job = tid; job < ni * 32; job += nthr) {
        const int li = job >> 5, pl = (job >> 4) & 1, ch = job & 15;
        uint16_t *dst = npoly(polys, 2, li, pl);
        sample_chunk(reinterpret_cast<const uint2 *>(seeds + li * 128 + 32), pl, ch, [&](int j, uint32_t c0, uint32_t c1) {
            *reinterpret_cast<uint32_t *>(dst + phys(64 * ch + j)) = (c0 & 0xffff) | (c1 << 16);
        });
    }
    __syncthreads();
    for (int w = warp; w < ni * 2; w += nwarp) ntt_warp(npoly(polys, 2, w >> 1, w & 1), lane);
    __syncthreads();
    // b-hat = e-hat + pointwise(s-hat, a-hat), a-hat generated chunk by chunk
    for (int job = tid; job < ni * 16; job += nthr) {
        const int li = job >> 4, ch = job & 15;
        uint16_t *s = npoly(polys, 2, li, 0), *e = npoly(polys, 2, li, 1);
        uniform_chunk(reinterpret_cast<const uint2 *>(seeds + li * 128), ch, [&](int j, uint32_t av) {
            const int idx = phys(64 * ch + j);
            const uint32_t t = mont(3186u * av);
            const uint32_t r = mont((uint32_t)s[idx] * t);
            e[idx] = (uint16_t)((e[idx] + r) % Q);
        });
    }
    __syncthreads();
    for (int li = warp; li < ni; li += nwarp) {
        uint8_t *sk = a.sk + (size_t)(base + li) * SKB, *pk = a.pk + (size_t)(base + li) * PKB;
        const uint16_t *s = npoly(polys, 2, li, 0), *b = npoly(polys, 2, li, 1);
        for (int g = lane; g < N / 4; g += 32) {
            uint8_t o[7];
            tobytes4(o, s[phys(4 * g)], s[phys(4 * g + 1)], s[phys(4 * g + 2)], s[phys(4 * g + 3)]);
#pragma unroll
            for (int q = 0; q < 7; q++) sk[7 * g + q] = o[q];
            tobytes4(o, b[phys(4 * g)], b[phys(4 * g + 1)], b[phys(4 * g + 2)], b[phys(4 * g + 3)]);
#pragma unroll
            for (int q = 0; q < 7; q++) pk[7 * g + q] = o[q];
        }
        if (lane < 4) reinterpret_cast<uint2 *>(pk + POLYBYTES)[lane] = reinterpret_cast<const uint2 *>(seeds + li * 128)[lane];
    }
}

// encryption: slots 0 s', 1 e' -> u-hat, 2 v'
__global__ void __launch_bounds__(256) nh_enc_core(EncArgs a, int NI) {
    extern __shared__ __align__(16) uint8_t smem[];
    uint16_t *polys = reinterpret_cast<uint16_t *>(smem);
    const int base = blockIdx.x * NI, ni = min(NI, a.n - base);
    const int tid = threadIdx.x, nthr = blockDim.x, lane = tid & 31, warp = tid >> 5, nwarp = nthr >> 5;
    for (int job = tid; job < ni * 32; job += nthr) {
        const int li = job >> 5, pl = (job >> 4) & 1, ch = job & 15;
        uint16_t *dst = npoly(polys, 3, li, pl);
        sample_chunk(reinterpret_cast<const uint2 *>(a.coin + (size_t)(base + li) * a.coin_stride), pl, ch,
                     [&](int j, uint32_t c0, uint32_t c1) {
                         *reinterpret_cast<uint32_t *>(dst + phys(64 * ch + j)) = (c0 & 0xffff) | (c1 << 16);
                     });
    }
    __syncthreads();
    for (int w = warp; w < ni * 2; w += nwarp) ntt_warp(npoly(polys, 3, w >> 1, w & 1), lane);
    __syncthreads();
    // u-hat = pointwise(a-hat, s') + e' (a-hat chunk by chunk); v' = pointwise(b-hat, s')
    for (int job = tid; job < ni * 16; job += nthr) {
        const int li = job >> 4, ch = job & 15;
        const uint8_t *pk = a.pk + (size_t)(base + li) * PKB;
        uint16_t *s = npoly(polys, 3, li, 0), *e = npoly(polys, 3, li, 1), *v = npoly(polys, 3, li, 2);
        uniform_chunk(reinterpret_cast<const uint2 *>(pk + POLYBYTES), ch, [&](int j, uint32_t av) {
            const int idx = phys(64 * ch + j);
            const uint32_t t = mont(3186u * s[idx]);
            const uint32_t u = mont(av * t);
            e[idx] = (uint16_t)((u + e[idx]) % Q);
        });
        for (int j = 0; j < 64; j += 4) {
            uint32_t bh[4];
            frombytes4(bh, pk + 7 * ((64 * ch + j) >> 2));
#pragma unroll
            for (int q = 0; q < 4; q++) {
                const int idx = phys(64 * ch + j + q);
                const uint32_t t = mont(3186u * s[idx]);
                v[idx] = (uint16_t)mont(bh[q] * t);
            }
        }
    }
    __syncthreads();
    for (int w = warp; w < ni; w += nwarp) invntt_warp(npoly(polys, 3, w, 2), lane);
    __syncthreads();
    // v' = v' + e'' + msg, compress (chunk jobs, noise nonce 2)
    for (int job = tid; job < ni * 16; job += nthr) {
        const int li = job >> 4, ch = job & 15;
        uint16_t *v = npoly(polys, 3, li, 2);
        const uint8_t *m = a.m + (size_t)(base + li) * a.m_stride;
        sample_chunk(reinterpret_cast<const uint2 *>(a.coin + (size_t)(base + li) * a.coin_stride), 2, ch,
                     [&](int j, uint32_t c0, uint32_t c1) {
                         const uint32_t cs[2] = {c0, c1};
#pragma unroll
                         for (int h = 0; h < 2; h++) {
                             const int i = 64 * ch + j + h, idx = phys(i);
                             uint32_t x = (v[idx] + (cs[h] & 0xffff)) % Q;
                             const uint32_t mb = (m[(i & 255) >> 3] >> (i & 7)) & 1;
                             x = (x + (mb ? Q / 2 : 0)) % Q;
                             v[idx] = (uint16_t)compress_coeff(x);
                         }
                     });
    }
    __syncthreads();
    for (int li = warp; li < ni; li += nwarp) {
        uint8_t *ct = a.ct + (size_t)(base + li) * CTB;
        const uint16_t *u = npoly(polys, 3, li, 1), *v = npoly(polys, 3, li, 2);
        for (int g = lane; g < N / 4; g += 32) {
            uint8_t o[7];
            tobytes4(o, u[phys(4 * g)], u[phys(4 * g + 1)], u[phys(4 * g + 2)], u[phys(4 * g + 3)]);
#pragma unroll
            for (int q = 0; q < 7; q++) ct[7 * g + q] = o[q];
        }
        for (int g = lane; g < N / 8; g += 32) {  // 8 compressed 3-bit values -> 3 bytes
            uint32_t t[8];
#pragma unroll
            for (int q = 0; q < 8; q++) t[q] = v[phys(8 * g + q)];
            uint8_t *r = ct + POLYBYTES + 3 * g;
            r[0] = (uint8_t)(t[0] | (t[1] << 3) | (t[2] << 6));
            r[1] = (uint8_t)((t[2] >> 2) | (t[3] << 1) | (t[4] << 4) | (t[5] << 7));
            r[2] = (uint8_t)((t[5] >> 1) | (t[6] << 2) | (t[7] << 5));
        }
    }
}

// decryption: tmp = invntt(pointwise(s-hat, u-hat)); m = tomsg(tmp - v')
__global__ void __launch_bounds__(256) nh_dec_core(DecArgs d, int NI) {
    extern __shared__ __align__(16) uint8_t smem[];
    uint16_t *polys = reinterpret_cast<uint16_t *>(smem);
    const int base = blockIdx.x * NI, ni = min(NI, d.n - base);
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nwarp = blockDim.x >> 5;
    for (int li = warp; li < ni; li += nwarp) {
        const uint8_t *sk = d.sk + (size_t)(base + li) * SKB, *ct = d.ct + (size_t)(base + li) * CTB;
        uint16_t *t = npoly(polys, 1, li, 0);
        for (int g = lane; g < N / 4; g += 32) {
            uint32_t s[4], u[4];
            frombytes4(s, sk + 7 * g);
            frombytes4(u, ct + 7 * g);
#pragma unroll
            for (int q = 0; q < 4; q++) t[phys(4 * g + q)] = (uint16_t)mont(s[q] * mont(3186u * u[q]));
        }
        __syncwarp();
        invntt_warp(t, lane);
        // lane = message byte: bits 8 lane + b use coefficients i, i+256, i+512, i+768
        const uint8_t *cv = ct + POLYBYTES;
        uint32_t byte = 0;
#pragma unroll
        for (int b = 0; b < 8; b++) {
            const int i = 8 * lane + b;
            uint32_t acc = 0;
#pragma unroll
            for (int qq = 0; qq < 4; qq++) {
                const int c = i + 256 * qq;
                const uint32_t x = (t[phys(c)] + 3 * Q - decompress_coeff(cv, c)) % Q;
                acc = (acc + flipabs(x)) & 0xffff;
            }
            acc = (acc - Q) & 0xffff;
            byte |= (acc >> 15) << b;
        }
        uint8_t *out = d.m_out + (size_t)(base + li) * 32;
        if (!d.kem) {
            out[lane] = (uint8_t)byte;
        } else {
            // ss = SHAKE256(m', 32): gather the 32 message bytes into lane 0's Keccak state
            uint2 A[25];
            keccak_zero(A);
#pragma unroll
            for (int w = 0; w < 4; w++) {
                uint32_t lo = 0, hi = 0;
#pragma unroll
                for (int b = 0; b < 4; b++) {
                    lo |= (__shfl_sync(0xffffffffu, byte, 8 * w + b) & 0xff) << (8 * b);
                    hi |= (__shfl_sync(0xffffffffu, byte, 8 * w + 4 + b) & 0xff) << (8 * b);
                }
                A[w] = make_uint2(lo, hi);
            }
            if (lane == 0) {
                A[4].x ^= DOM_SHAKE;
                A[SHAKE256_LANES - 1].y ^= 0x80000000u;
                keccak_f1600_rolled(A);
                uint2 *o = reinterpret_cast<uint2 *>(out);
#pragma unroll
                for (int w = 0; w < 4; w++) o[w] = A[w];
            }
        }
    }
}

// CPA-KEM encapsulation prologue: buf = SHAKE256(coins, 64) -> m || coin; ss = SHAKE256(m, 32)
__global__ void __launch_bounds__(128) nh_enc_hash_pre(int n, const uint8_t *coins, uint8_t *scratch, uint8_t *ss) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= n) return;
    uint2 A[25], buf[8];
    keccak_absorb_lanes<SHAKE256_LANES>(A, reinterpret_cast<const uint2 *>(coins + (size_t)x * 32), 4, DOM_SHAKE);
    keccak_f1600_rolled(A);
#pragma unroll
    for (int i = 0; i < 8; i++) buf[i] = A[i];
    uint2 *o = reinterpret_cast<uint2 *>(scratch + (size_t)x * 64);
#pragma unroll
    for (int i = 0; i < 8; i++) o[i] = buf[i];
    keccak_zero(A);
#pragma unroll
    for (int i = 0; i < 4; i++) A[i] = buf[i];
    A[4].x ^= DOM_SHAKE;
    A[SHAKE256_LANES - 1].y ^= 0x80000000u;
    keccak_f1600_rolled(A);
    uint2 *s = reinterpret_cast<uint2 *>(ss + (size_t)x * 32);
#pragma unroll
    for (int i = 0; i < 4; i++) s[i] = A[i];
}

static int g_shape[3][2] = {{8, 128}, {4, 64}, {4, 128}};  // [op] = {instances per CTA, threads}

template <class Kern>
static int prep(Kern k, size_t sm) {
    if (capturing()) return PQCGPU_OK;
    if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm) == cudaSuccess) return PQCGPU_OK;
    cudaGetLastError();  // leave no error behind for the caller's next CUDA call
    return PQCGPU_ECUDA;
}
// per-instance shared memory of the core kernel of op (0 keypair, 1 encaps, 2 decaps)
static size_t smem_per_instance(int op) { return op == 0 ? 2 * PITCH * 2 + 128 : op == 1 ? 3 * PITCH * 2 : PITCH * 2; }

}  // namespace newhope

using namespace newhope;

int newhope_init_constants() {
    const long q = Q, g = 7, mont = (1L << 18) % q;
    auto pw = [&](long b, long e) {
        long r = 1;
        b %= q;
        while (e) {
            if (e & 1) r = r * b % q;
            b = b * b % q;
            e >>= 1;
        }
        return r;
    };
    const long ginv = pw(g, q - 2), ninv = pw(N, q - 2);
    static uint16_t gb[N], oi[N / 2], gi[N];
    auto brv = [](int i) { int r = 0; for (int b = 0; b < 10; b++) r |= ((i >> b) & 1) << (9 - b); return r; };
    for (int i = 0; i < N; i++) gb[i] = (uint16_t)(pw(g, brv(i)) * mont % q);
    for (int i = 0; i < N / 2; i++) oi[i] = (uint16_t)(pw(ginv, 2L * brv(2 * i)) * mont % q);
    for (int i = 0; i < N; i++) gi[i] = (uint16_t)(pw(ginv, i) * ninv % q * mont % q);
    uint2 rc[24];
    keccak_rc_host(rc);
    if (cudaMemcpyToSymbol(c_keccak_rc, rc, sizeof rc) != cudaSuccess) return PQCGPU_ECUDA;
    if (cudaMemcpyToSymbol(d_gammas_bitrev, gb, sizeof gb) != cudaSuccess) return PQCGPU_ECUDA;
    if (cudaMemcpyToSymbol(d_omegas_inv_bitrev, oi, sizeof oi) != cudaSuccess) return PQCGPU_ECUDA;
    if (cudaMemcpyToSymbol(d_gammas_inv, gi, sizeof gi) != cudaSuccess) return PQCGPU_ECUDA;
    return PQCGPU_OK;
}

int newhope_set_shape(int op, int ni, int threads) {
    if (op < 0 || op > 2 || ni < 1 || ni > 64 || threads < 32 || threads > 256 || threads % 32) return PQCGPU_EINVAL;
    if ((size_t)ni * smem_per_instance(op) > MAX_SMEM_PER_CTA) return PQCGPU_EINVAL;
    g_shape[op][0] = ni;
    g_shape[op][1] = threads;
    return PQCGPU_OK;
}

int newhope_get_shape(int op, int *ni, int *threads) {
    if (op < 0 || op > 2) return PQCGPU_EINVAL;
    *ni = g_shape[op][0];
    *threads = g_shape[op][1];
    return PQCGPU_OK;
}

int newhope_keypair_dev(int n, uint8_t *pk, uint8_t *sk, const uint8_t *seed, int seed_stride, cudaStream_t st) {
    const int NI = g_shape[0][0], NT = g_shape[0][1];
    const size_t sm = (size_t)NI * smem_per_instance(0);
    if (prep(nh_kp_core, sm)) return PQCGPU_ECUDA;
    KpArgs a{n, pk, sk, seed, seed_stride};
    PQC_LAUNCH(st, "nh_kp_core", 1024, 0, nh_kp_core<<<(n + NI - 1) / NI, NT, sm, st>>>(a, NI));
    return cudaGetLastError() == cudaSuccess ? PQCGPU_OK : PQCGPU_ECUDA;
}

// kem: coins 32 B per instance -> (m, coin) via the prologue into scratch (64 B / instance), ss
int newhope_enc_dev(int n, uint8_t *ct, uint8_t *ss, const uint8_t *pk, const uint8_t *m, const uint8_t *coins,
                    uint8_t *scratch, int kem, cudaStream_t st) {
    const int NI = g_shape[1][0], NT = g_shape[1][1];
    const size_t sm = (size_t)NI * smem_per_instance(1);
    if (prep(nh_enc_core, sm)) return PQCGPU_ECUDA;
    EncArgs a{n, ct, pk, m, coins, 32, 32};
    if (kem) {
        PQC_LAUNCH(st, "nh_enc_hash_pre", 1024, 0, nh_enc_hash_pre<<<(n + 127) / 128, 128, 0, st>>>(n, coins, scratch, ss));
        a.m = scratch;
        a.coin = scratch + 32;
        a.m_stride = a.coin_stride = 64;
    }
    PQC_LAUNCH(st, "nh_enc_core", 1024, 0, nh_enc_core<<<(n + NI - 1) / NI, NT, sm, st>>>(a, NI));
    return cudaGetLastError() == cudaSuccess ? PQCGPU_OK : PQCGPU_ECUDA;
}

int newhope_dec_dev(int n, uint8_t *out, const uint8_t *ct, const uint8_t *sk, int kem, cudaStream_t st) {
    const int NI = g_shape[2][0], NT = g_shape[2][1];
    const size_t sm = (size_t)NI * smem_per_instance(2);
    if (prep(nh_dec_core, sm)) return PQCGPU_ECUDA;
    DecArgs d{n, out, ct, sk, kem};
    PQC_LAUNCH(st, "nh_dec_core", 1024, 0, nh_dec_core<<<(n + NI - 1) / NI, NT, sm, st>>>(d, NI));
    return cudaGetLastError() == cudaSuccess ? PQCGPU_OK : PQCGPU_ECUDA;
}

}  // namespace pqc
