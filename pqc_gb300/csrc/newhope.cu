// Batched NewHope-1024 and NewHope-512 CPA-PKE and CPA-KEM for sm_103a.
//
// Replaces cpapke_keypair / cpapke_enc / cpapke_dec (NewHope_NIST_GPU/cpapke.cu:265-476, one thread
// per instance, every polynomial in HBM in a coefficient-major layout) with one core kernel per
// operation:
//   - noise and the public polynomial a-hat in chunks of 64 coefficients, one Keccak permutation
//     per thread (poly_sample / poly_uniform, NewHope_NIST_GPU/poly.cu:332-444), written straight
//     into shared memory or consumed on the spot (a-hat never exists whole);
//   - the 1024-point NTT by one warp per polynomial, 32 coefficients per lane, two passes of five
//     layers in registers with one transpose through shared memory; the 512-point NTT by a
//     half-warp per polynomial (two polynomials per warp), 32 coefficients per lane, five + four
//     layers;
//   - packing by one warp per instance;
//   - Keccak with the round loop rolled (keccak_f1600_rolled): the kernels have several sampler
//     call sites, and the unrolled copies stalled instruction fetch (encapsulation +2.5 %).
// Arithmetic mirrors the reference operation for operation (NewHope_NIST_GPU/reduce.cu:22-47,
// ntt.cu:92-234, poly.cu:19-508), uint16 truncations and uint32 wrap-around included, so every
// intermediate value equals the reference's.  For n = 512 the transform follows the reference's
// scalar 512-point ntt (ntt.cu:143-181), which reduces odd layers with `% q` where the 1024-point
// one uses barrett_reduce; each message bit occupies n / 256 coefficients (poly.cu:226-291).
#include <cuda_runtime.h>

#include <algorithm>
#include <vector>
#include <stdint.h>

#include "keccak.cuh"
#include "pqcgpu_internal.h"

namespace pqc {
namespace newhope {

constexpr uint32_t Q = 12289;

// Sizes of the parameter set with n coefficients (NewHope_NIST_GPU/params.h:25-31).
// PITCH = uint16 per shared polynomial: 8 pad after every 32 coefficients; for n = 512 another 16
// so that the two polynomials of a warp's half-warps start 8 banks apart.
template <int N>
struct Nh {
    static constexpr int POLYBYTES = 14 * N / 8, PKB = POLYBYTES + 32, SKB = POLYBYTES, COMPB = 3 * N / 8,
                         CTB = POLYBYTES + COMPB, NCH = N / 64, PITCH = N + N / 4 + (N == 512 ? 16 : 0);
};

// Tables generated on the host (g = 7 for n = 1024, g = 10968 for n = 512; mont = 2^18 mod q;
// NewHope_NIST_GPU/precomp.cu:27-29, :75-183).
static __device__ uint16_t d_gammas_bitrev[1024];
static __device__ uint16_t d_omegas_inv_bitrev[512];
static __device__ uint16_t d_gammas_inv[1024];
static __device__ uint16_t d_gammas_bitrev512[512];
static __device__ uint16_t d_omegas_inv_bitrev512[256];
static __device__ uint16_t d_gammas_inv512[512];

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
// butterfly of ntt(): a <- a + b (even layer) or, on odd layers, barrett(a + b) (n = 1024) /
// (a + b) % q (n = 512); b <- mont(W (a + 3q - b))
template <int N>
__device__ __forceinline__ void bfly(uint32_t &a, uint32_t &b, uint32_t W, bool odd) {
    const uint32_t temp = a;
    if (N == 1024)
        a = odd ? barrett(temp + b) : ((temp + b) & 0xffffu);
    else
        a = odd ? (temp + b) % Q : ((temp + b) & 0xffffu);
    b = mont(W * (temp + 3 * Q - b));
}

// Forward transform (poly_ntt, poly.cu:519-531): mul_coefficients(gammas_bitrev) then
// ntt(gammas_bitrev as omega).  Layer i pairs j, j + 2^i with twiddle omega[j >> (i + 1)].
__device__ void ntt_warp(uint16_t *p, int lane) {  // n = 1024
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
            if (!((q >> i) & 1)) bfly<1024>(r[q], r[q + (1 << i)], __ldg(&d_gammas_bitrev[(32 * lane + q) >> (i + 1)]), i & 1);
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
            if (!((q >> (i - 5)) & 1)) bfly<1024>(r[q], r[q + (1 << (i - 5))], __ldg(&d_gammas_bitrev[q >> (i - 4)]), i & 1);
#pragma unroll
    for (int q = 0; q < 32; q++) p[phys(lane + 32 * q)] = (uint16_t)r[q];
    __syncwarp();
}

// Inverse transform (poly_invntt, poly.cu:541-547): bitrev_vector, ntt(omegas_inv_bitrev),
// mul_coefficients(gammas_inv).  The bit reversal is folded into the first pass's loads.
__device__ void invntt_warp(uint16_t *p, int lane) {  // n = 1024
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
                bfly<1024>(r[q], r[q + (1 << i)], __ldg(&d_omegas_inv_bitrev[(32 * lane + q) >> (i + 1)]), i & 1);
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
                bfly<1024>(r[q], r[q + (1 << (i - 5))], __ldg(&d_omegas_inv_bitrev[q >> (i - 4)]), i & 1);
#pragma unroll
    for (int q = 0; q < 32; q++) p[phys(lane + 32 * q)] = (uint16_t)mont(r[q] * __ldg(&d_gammas_inv[lane + 32 * q]));
    __syncwarp();
}

// n = 512 transforms by a half-warp: lane l (0..15) of each half holds 32 coefficients.  Pass 1
// (layers 0-4, distances 1..16) on the 32 consecutive coefficients 32 l + q, pass 2 (layers 5-8,
// distances 32..256) on the coefficients l + 16 q.  Both halves call together (the __syncwarp
// calls need all 32 lanes); a half with act == false touches no memory.
__device__ void ntt512_half(uint16_t *p, int l, bool act) {
    uint32_t r[32];
    if (act) {
        uint16_t *pa = p + phys(32 * l);
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
        for (int q = 0; q < 32; q++) r[q] = mont(r[q] * __ldg(&d_gammas_bitrev512[32 * l + q]));
#pragma unroll
        for (int i = 0; i < 5; i++)
#pragma unroll
            for (int q = 0; q < 32; q++)
                if (!((q >> i) & 1))
                    bfly<512>(r[q], r[q + (1 << i)], __ldg(&d_gammas_bitrev512[(32 * l + q) >> (i + 1)]), i & 1);
#pragma unroll
        for (int v = 0; v < 4; v++)
            reinterpret_cast<uint4 *>(pa)[v] =
                make_uint4(r[8 * v] | (r[8 * v + 1] << 16), r[8 * v + 2] | (r[8 * v + 3] << 16),
                           r[8 * v + 4] | (r[8 * v + 5] << 16), r[8 * v + 6] | (r[8 * v + 7] << 16));
    }
    __syncwarp();
    if (act) {
#pragma unroll
        for (int q = 0; q < 32; q++) r[q] = p[phys(l + 16 * q)];
        // layer i pairs j, j + 2^i; with j = l + 16 q that is q, q + 2^(i-4), twiddle j >> (i+1) = q >> (i-3)
#pragma unroll
        for (int i = 5; i < 9; i++)
#pragma unroll
            for (int q = 0; q < 32; q++)
                if (!((q >> (i - 4)) & 1))
                    bfly<512>(r[q], r[q + (1 << (i - 4))], __ldg(&d_gammas_bitrev512[q >> (i - 3)]), i & 1);
#pragma unroll
        for (int q = 0; q < 32; q++) p[phys(l + 16 * q)] = (uint16_t)r[q];
    }
    __syncwarp();
}

// Inverse (poly_invntt): bit reversal folded into the first loads, x'[32 l + q] = x[brv9(32 l + q)]
// = x[16 brv5(q) + brv4(l)], then the two passes with omegas_inv, then gammas_inv.
__device__ void invntt512_half(uint16_t *p, int l, bool act) {
    uint32_t r[32];
    if (act) {
        const int lrev = __brev(l) >> 28;
#pragma unroll
        for (int q = 0; q < 32; q++) {
            const int qrev = __brev(q) >> 27;
            r[q] = p[phys(16 * qrev + lrev)];
        }
    }
    __syncwarp();
    if (act) {
#pragma unroll
        for (int i = 0; i < 5; i++)
#pragma unroll
            for (int q = 0; q < 32; q++)
                if (!((q >> i) & 1))
                    bfly<512>(r[q], r[q + (1 << i)], __ldg(&d_omegas_inv_bitrev512[(32 * l + q) >> (i + 1)]), i & 1);
        uint16_t *pa = p + phys(32 * l);
#pragma unroll
        for (int v = 0; v < 4; v++)
            reinterpret_cast<uint4 *>(pa)[v] =
                make_uint4(r[8 * v] | (r[8 * v + 1] << 16), r[8 * v + 2] | (r[8 * v + 3] << 16),
                           r[8 * v + 4] | (r[8 * v + 5] << 16), r[8 * v + 6] | (r[8 * v + 7] << 16));
    }
    __syncwarp();
    if (act) {
#pragma unroll
        for (int q = 0; q < 32; q++) r[q] = p[phys(l + 16 * q)];
#pragma unroll
        for (int i = 5; i < 9; i++)
#pragma unroll
            for (int q = 0; q < 32; q++)
                if (!((q >> (i - 4)) & 1))
                    bfly<512>(r[q], r[q + (1 << (i - 4))], __ldg(&d_omegas_inv_bitrev512[q >> (i - 3)]), i & 1);
#pragma unroll
        for (int q = 0; q < 32; q++)
            p[phys(l + 16 * q)] = (uint16_t)mont(r[q] * __ldg(&d_gammas_inv512[l + 16 * q]));
    }
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
template <int N>
__device__ __forceinline__ uint32_t decompress_coeff(const uint8_t *cb, int i) {
    // 3-bit values packed LSB-first, 8 per 3 bytes (poly_decompress, poly.cu:197-216)
    constexpr int COMPB = Nh<N>::COMPB;
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

template <int N>
__device__ __forceinline__ uint16_t *npoly(uint16_t *polys, int per, int li, int s) {
    return polys + ((size_t)li * per + s) * Nh<N>::PITCH;
}

// keypair: slots 0 s-hat, 1 e-hat -> b-hat
template <int N>
__device__ __forceinline__ void nh_kp_body(const KpArgs &a, int NI, int base) {
    using P = Nh<N>;
    constexpr int NCH = P::NCH;
    extern __shared__ __align__(16) uint8_t smem[];
    uint16_t *polys = reinterpret_cast<uint16_t *>(smem);
    uint8_t *seeds = smem + (size_t)NI * 2 * P::PITCH * 2;
    const int ni = min(NI, a.n - base);
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
    for (int job = tid; job < ni * 2 * NCH; job += nthr) {
        const int li = job / (2 * NCH), pl = (job / NCH) & 1, ch = job % NCH;
        uint16_t *dst = npoly<N>(polys, 2, li, pl);
        sample_chunk(reinterpret_cast<const uint2 *>(seeds + li * 128 + 32), pl, ch, [&](int j, uint32_t c0, uint32_t c1) {
            *reinterpret_cast<uint32_t *>(dst + phys(64 * ch + j)) = (c0 & 0xffff) | (c1 << 16);
        });
    }
    __syncthreads();
    if constexpr (N == 1024) {
        for (int w = warp; w < ni * 2; w += nwarp) ntt_warp(npoly<N>(polys, 2, w >> 1, w & 1), lane);
    } else {  // one instance per warp: s-hat on lanes 0-15, e-hat on lanes 16-31
        for (int w = warp; w < ni; w += nwarp) ntt512_half(npoly<N>(polys, 2, w, lane >> 4), lane & 15, true);
    }
    __syncthreads();
    // b-hat = e-hat + pointwise(s-hat, a-hat), a-hat generated chunk by chunk
    for (int job = tid; job < ni * NCH; job += nthr) {
        const int li = job / NCH, ch = job % NCH;
        uint16_t *s = npoly<N>(polys, 2, li, 0), *e = npoly<N>(polys, 2, li, 1);
        uniform_chunk(reinterpret_cast<const uint2 *>(seeds + li * 128), ch, [&](int j, uint32_t av) {
            const int idx = phys(64 * ch + j);
            const uint32_t t = mont(3186u * av);
            const uint32_t r = mont((uint32_t)s[idx] * t);
            e[idx] = (uint16_t)((e[idx] + r) % Q);
        });
    }
    __syncthreads();
    for (int li = warp; li < ni; li += nwarp) {
        uint8_t *sk = a.sk + (size_t)(base + li) * P::SKB, *pk = a.pk + (size_t)(base + li) * P::PKB;
        const uint16_t *s = npoly<N>(polys, 2, li, 0), *b = npoly<N>(polys, 2, li, 1);
        for (int g = lane; g < N / 4; g += 32) {
            uint8_t o[7];
            tobytes4(o, s[phys(4 * g)], s[phys(4 * g + 1)], s[phys(4 * g + 2)], s[phys(4 * g + 3)]);
#pragma unroll
            for (int q = 0; q < 7; q++) sk[7 * g + q] = o[q];
            tobytes4(o, b[phys(4 * g)], b[phys(4 * g + 1)], b[phys(4 * g + 2)], b[phys(4 * g + 3)]);
#pragma unroll
            for (int q = 0; q < 7; q++) pk[7 * g + q] = o[q];
        }
        if (lane < 4) reinterpret_cast<uint2 *>(pk + P::POLYBYTES)[lane] = reinterpret_cast<const uint2 *>(seeds + li * 128)[lane];
    }
}

// encryption: slots 0 s', 1 e' -> u-hat, 2 v'
template <int N>
__device__ __forceinline__ void nh_enc_body(const EncArgs &a, int NI, int base) {
    using P = Nh<N>;
    constexpr int NCH = P::NCH;
    extern __shared__ __align__(16) uint8_t smem[];
    uint16_t *polys = reinterpret_cast<uint16_t *>(smem);
    const int ni = min(NI, a.n - base);
    const int tid = threadIdx.x, nthr = blockDim.x, lane = tid & 31, warp = tid >> 5, nwarp = nthr >> 5;
    for (int job = tid; job < ni * 2 * NCH; job += nthr) {
        const int li = job / (2 * NCH), pl = (job / NCH) & 1, ch = job % NCH;
        uint16_t *dst = npoly<N>(polys, 3, li, pl);
        sample_chunk(reinterpret_cast<const uint2 *>(a.coin + (size_t)(base + li) * a.coin_stride), pl, ch,
                     [&](int j, uint32_t c0, uint32_t c1) {
                         *reinterpret_cast<uint32_t *>(dst + phys(64 * ch + j)) = (c0 & 0xffff) | (c1 << 16);
                     });
    }
    __syncthreads();
    if constexpr (N == 1024) {
        for (int w = warp; w < ni * 2; w += nwarp) ntt_warp(npoly<N>(polys, 3, w >> 1, w & 1), lane);
    } else {  // one instance per warp: s' on lanes 0-15, e' on lanes 16-31
        for (int w = warp; w < ni; w += nwarp) ntt512_half(npoly<N>(polys, 3, w, lane >> 4), lane & 15, true);
    }
    __syncthreads();
    // u-hat = pointwise(a-hat, s') + e' (a-hat chunk by chunk); v' = pointwise(b-hat, s')
    for (int job = tid; job < ni * NCH; job += nthr) {
        const int li = job / NCH, ch = job % NCH;
        const uint8_t *pk = a.pk + (size_t)(base + li) * P::PKB;
        uint16_t *s = npoly<N>(polys, 3, li, 0), *e = npoly<N>(polys, 3, li, 1), *v = npoly<N>(polys, 3, li, 2);
        uniform_chunk(reinterpret_cast<const uint2 *>(pk + P::POLYBYTES), ch, [&](int j, uint32_t av) {
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
    if constexpr (N == 1024) {
        for (int w = warp; w < ni; w += nwarp) invntt_warp(npoly<N>(polys, 3, w, 2), lane);
    } else {  // two instances per warp
        for (int w = warp; 2 * w < ni; w += nwarp) {
            const int li = 2 * w + (lane >> 4);
            invntt512_half(npoly<N>(polys, 3, li < ni ? li : 0, 2), lane & 15, li < ni);
        }
    }
    __syncthreads();
    // v' = v' + e'' + msg, compress (chunk jobs, noise nonce 2)
    for (int job = tid; job < ni * NCH; job += nthr) {
        const int li = job / NCH, ch = job % NCH;
        uint16_t *v = npoly<N>(polys, 3, li, 2);
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
        uint8_t *ct = a.ct + (size_t)(base + li) * P::CTB;
        const uint16_t *u = npoly<N>(polys, 3, li, 1), *v = npoly<N>(polys, 3, li, 2);
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
            uint8_t *r = ct + P::POLYBYTES + 3 * g;
            r[0] = (uint8_t)(t[0] | (t[1] << 3) | (t[2] << 6));
            r[1] = (uint8_t)((t[2] >> 2) | (t[3] << 1) | (t[4] << 4) | (t[5] << 7));
            r[2] = (uint8_t)((t[5] >> 1) | (t[6] << 2) | (t[7] << 5));
        }
    }
}

// decryption: tmp = invntt(pointwise(s-hat, u-hat)); m = tomsg(tmp - v')
// n = 1024: one warp per instance.  n = 512: one half-warp per instance (two per warp).
template <int N>
__device__ __forceinline__ void nh_dec_body(const DecArgs &d, int NI, int base) {
    using P = Nh<N>;
    if constexpr (N == 1024) {
    extern __shared__ __align__(16) uint8_t smem[];
    uint16_t *polys = reinterpret_cast<uint16_t *>(smem);
    const int ni = min(NI, d.n - base);
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nwarp = blockDim.x >> 5;
    for (int li = warp; li < ni; li += nwarp) {
        const uint8_t *sk = d.sk + (size_t)(base + li) * P::SKB, *ct = d.ct + (size_t)(base + li) * P::CTB;
        uint16_t *t = npoly<N>(polys, 1, li, 0);
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
        const uint8_t *cv = ct + P::POLYBYTES;
        uint32_t byte = 0;
#pragma unroll
        for (int b = 0; b < 8; b++) {
            const int i = 8 * lane + b;
            uint32_t acc = 0;
#pragma unroll
            for (int qq = 0; qq < 4; qq++) {
                const int c = i + 256 * qq;
                const uint32_t x = (t[phys(c)] + 3 * Q - decompress_coeff<N>(cv, c)) % Q;
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
    } else {
        extern __shared__ __align__(16) uint8_t smem[];
        uint16_t *polys = reinterpret_cast<uint16_t *>(smem);
        const int ni = min(NI, d.n - base);
        const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nwarp = blockDim.x >> 5;
        const int l = lane & 15, half = lane >> 4;
        for (int w = warp; 2 * w < ni; w += nwarp) {
            const int li = 2 * w + half;
            const bool act = li < ni;
            const int lc = act ? li : 0;
            const uint8_t *sk = d.sk + (size_t)(base + lc) * P::SKB, *ct = d.ct + (size_t)(base + lc) * P::CTB;
            uint16_t *t = npoly<N>(polys, 1, lc, 0);
            if (act)
                for (int g = l; g < N / 4; g += 16) {
                    uint32_t s[4], u[4];
                    frombytes4(s, sk + 7 * g);
                    frombytes4(u, ct + 7 * g);
#pragma unroll
                    for (int q = 0; q < 4; q++) t[phys(4 * g + q)] = (uint16_t)mont(s[q] * mont(3186u * u[q]));
                }
            __syncwarp();
            invntt512_half(t, l, act);
            // lane l of the half = message bytes 2l, 2l+1: bit 8 byte + b uses coefficients i, i+256
            const uint8_t *cv = ct + P::POLYBYTES;
            uint32_t bytes2 = 0;
            if (act)
#pragma unroll
                for (int b = 0; b < 16; b++) {
                    const int i = 16 * l + b;
                    uint32_t acc = 0;
#pragma unroll
                    for (int qq = 0; qq < 2; qq++) {
                        const int c = i + 256 * qq;
                        const uint32_t x = (t[phys(c)] + 3 * Q - decompress_coeff<N>(cv, c)) % Q;
                        acc = (acc + flipabs(x)) & 0xffff;
                    }
                    acc = (acc - Q / 2) & 0xffff;
                    bytes2 |= (acc >> 15) << b;
                }
            uint8_t *out = d.m_out + (size_t)(base + lc) * 32;
            if (!d.kem) {
                if (act) {
                    out[2 * l] = (uint8_t)bytes2;
                    out[2 * l + 1] = (uint8_t)(bytes2 >> 8);
                }
            } else {
                // ss = SHAKE256(m', 32): the half's lane 0 gathers its 32 message bytes (two per lane)
                uint2 A[25];
                keccak_zero(A);
#pragma unroll
                for (int w4 = 0; w4 < 4; w4++) {
                    uint32_t lo = 0, hi = 0;
#pragma unroll
                    for (int b = 0; b < 2; b++) {
                        lo |= (__shfl_sync(0xffffffffu, bytes2, 16 * half + 4 * w4 + b) & 0xffff) << (16 * b);
                        hi |= (__shfl_sync(0xffffffffu, bytes2, 16 * half + 4 * w4 + 2 + b) & 0xffff) << (16 * b);
                    }
                    A[w4] = make_uint2(lo, hi);
                }
                if (act && l == 0) {
                    A[4].x ^= DOM_SHAKE;
                    A[SHAKE256_LANES - 1].y ^= 0x80000000u;
                    keccak_f1600_rolled(A);
                    uint2 *o = reinterpret_cast<uint2 *>(out);
#pragma unroll
                    for (int w4 = 0; w4 < 4; w4++) o[w4] = A[w4];
                }
            }
            __syncwarp();
        }
    }
}

}  // namespace newhope
}  // namespace pqc
#include "newhope_single.cuh"
namespace pqc {
namespace newhope {

template <int N>
__global__ void __launch_bounds__(256) nh_kp_core(KpArgs a, int NI) {
    nh_kp_body<N>(a, NI, blockIdx.x * NI);
}
// (256, 1): no register cap below 255 (the n = 512 instance spilled at 128)
template <int N>
__global__ void __launch_bounds__(256, 1) nh_enc_core(EncArgs a, int NI) {
    nh_enc_body<N>(a, NI, blockIdx.x * NI);
}
template <int N>
__global__ void __launch_bounds__(256) nh_dec_core(DecArgs d, int NI) {
    nh_dec_body<N>(d, NI, blockIdx.x * NI);
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

// [n index: 0 = 1024, 1 = 512][op] = {instances per CTA, threads}
static LaunchShape g_shape[2][3] = {{{8, 128}, {4, 64}, {4, 128}}, {{16, 128}, {16, 128}, {4, 64}}};
// [0 keypair, 1 encapsulation]: key generations and encapsulations (CPA and KEM) of at most this
// many instances run on the single-instance kernels (newhope_single.cuh); larger batches on the
// batched core kernels (both n).  One 512-thread CTA per SM, so the single-instance time steps up
// past each multiple of 152 instances.  Measured on GB300 (NewHope-1024, single-instance / batched,
// us): keypair 22.0 / 31.4 and encapsulation 26.5 / 58.2 at n = 1; 38.9 / 43.1 and 49.0 / 70.5 at
// 304; 52.7 / 42.8 and 66.2 / 70.6 at 384; 54.9 / 42.8 and 68.8 / 71.9 at 456; 67.5 / 43.3 and 84.3
// / 72.5 at 512 (NewHope-512 alike).
static constexpr int NH_SINGLE_DEFAULT[2] = {304, 456};
static LaunchShape g_nh_single[2] = {{304, 0}, {456, 0}};
static int nh_single_max(int op) {
    int v, t;
    g_nh_single[op].get(v, t);
    return v;
}
static int nidx(int N) { return N == 1024 ? 0 : 1; }

template <class Kern>
static int prep(Kern k, size_t sm) {
    if (capturing()) return PQCGPU_OK;
    if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm) == cudaSuccess) return PQCGPU_OK;
    cudaGetLastError();  // leave no error behind for the caller's next CUDA call
    return PQCGPU_ECUDA;
}
// per-instance shared memory of the core kernel of op (0 keypair, 1 encaps, 2 decaps)
static size_t smem_per_instance(int N, int op) {
    const size_t pitch = N == 1024 ? Nh<1024>::PITCH : Nh<512>::PITCH;
    return op == 0 ? 2 * pitch * 2 + 128 : op == 1 ? 3 * pitch * 2 : pitch * 2;
}

// twiddle tables of the n-point transform (formulas of NewHope_NIST_GPU/precomp.cu:27-29)
static void make_tables(int n, int logn, long g, uint16_t *gb, uint16_t *oi, uint16_t *gi) {
    const long q = Q, mont = (1L << 18) % q;
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
    const long ginv = pw(g, q - 2), ninv = pw(n, q - 2);
    auto brv = [&](int i) {
        int r = 0;
        for (int b = 0; b < logn; b++) r |= ((i >> b) & 1) << (logn - 1 - b);
        return r;
    };
    for (int i = 0; i < n; i++) gb[i] = (uint16_t)(pw(g, brv(i)) * mont % q);
    for (int i = 0; i < n / 2; i++) oi[i] = (uint16_t)(pw(ginv, 2L * brv(2 * i)) * mont % q);
    for (int i = 0; i < n; i++) gi[i] = (uint16_t)(pw(ginv, i) * ninv % q * mont % q);
}

}  // namespace newhope

using namespace newhope;

int newhope_init_constants() {
    static uint16_t gb[1024], oi[512], gi[1024], gb5[512], oi5[256], gi5[512];
    make_tables(1024, 10, 7, gb, oi, gi);
    make_tables(512, 9, 10968, gb5, oi5, gi5);
    uint2 rc[24];
    keccak_rc_host(rc);
    if (cudaMemcpyToSymbol(c_keccak_rc, rc, sizeof rc) != cudaSuccess) return PQCGPU_ECUDA;
    if (cudaMemcpyToSymbol(d_gammas_bitrev, gb, sizeof gb) != cudaSuccess) return PQCGPU_ECUDA;
    if (cudaMemcpyToSymbol(d_omegas_inv_bitrev, oi, sizeof oi) != cudaSuccess) return PQCGPU_ECUDA;
    if (cudaMemcpyToSymbol(d_gammas_inv, gi, sizeof gi) != cudaSuccess) return PQCGPU_ECUDA;
    if (cudaMemcpyToSymbol(d_gammas_bitrev512, gb5, sizeof gb5) != cudaSuccess) return PQCGPU_ECUDA;
    if (cudaMemcpyToSymbol(d_omegas_inv_bitrev512, oi5, sizeof oi5) != cudaSuccess) return PQCGPU_ECUDA;
    if (cudaMemcpyToSymbol(d_gammas_inv512, gi5, sizeof gi5) != cudaSuccess) return PQCGPU_ECUDA;
    return PQCGPU_OK;
}

int newhope_set_shape(int N, int op, int ni, int threads) {
    if (op == 3) {  // the largest batch that takes the single-instance kernels, keypair and
                    // encapsulation, both n; 0 = never, -1 = the measured defaults
        if ((N != 1024 && N != 512) || ni < -1 || ni > 4096) return PQCGPU_EINVAL;
        for (int o = 0; o < 2; o++) g_nh_single[o].set(ni < 0 ? NH_SINGLE_DEFAULT[o] : ni, 0);
        return PQCGPU_OK;
    }
    if ((N != 1024 && N != 512) || op < 0 || op > 2 || ni < 1 || ni > 64 || threads < 32 || threads > 256 || threads % 32)
        return PQCGPU_EINVAL;
    if ((size_t)ni * smem_per_instance(N, op) > MAX_SMEM_PER_CTA) return PQCGPU_EINVAL;
    g_shape[nidx(N)][op].set(ni, threads);
    return PQCGPU_OK;
}

int newhope_get_shape(int N, int op, int *ni, int *threads) {
    if (op == 3 && (N == 1024 || N == 512)) {  // the encapsulation's threshold
        g_nh_single[1].get(*ni, *threads);
        return PQCGPU_OK;
    }
    if ((N != 1024 && N != 512) || op < 0 || op > 2) return PQCGPU_EINVAL;
    g_shape[nidx(N)][op].get(*ni, *threads);
    return PQCGPU_OK;
}

template <int N>
static int keypair_n(int n, uint8_t *pk, uint8_t *sk, const uint8_t *seed, int seed_stride, bool single_ok,
                     cudaStream_t st) {
    if (single_ok && n <= nh_single_max(0)) {
        PQC_LAUNCH(st, "nh_kp_single", N, 0,
                   nh_kp_single<N><<<n, NHS_THREADS, NhSingleSmem<N>::bytes(), st>>>(seed, seed_stride, pk, sk));
        return cudaGetLastError() == cudaSuccess ? PQCGPU_OK : PQCGPU_ECUDA;
    }
    int NI, NT;
    g_shape[nidx(N)][0].get(NI, NT);
    const size_t sm = (size_t)NI * smem_per_instance(N, 0);
    if (prep(nh_kp_core<N>, sm)) return PQCGPU_ECUDA;
    KpArgs a{n, pk, sk, seed, seed_stride};
    PQC_LAUNCH(st, "nh_kp_core", N, 0, nh_kp_core<N><<<(n + NI - 1) / NI, NT, sm, st>>>(a, NI));
    return cudaGetLastError() == cudaSuccess ? PQCGPU_OK : PQCGPU_ECUDA;
}

template <int N>
static int enc_n(int n, uint8_t *ct, uint8_t *ss, const uint8_t *pk, const uint8_t *m, const uint8_t *coins,
                 uint8_t *scratch, int kem, bool single_ok, cudaStream_t st) {
    int NI, NT;
    g_shape[nidx(N)][1].get(NI, NT);
    const size_t sm = (size_t)NI * smem_per_instance(N, 1);
    if (prep(nh_enc_core<N>, sm)) return PQCGPU_ECUDA;
    if (single_ok && n <= nh_single_max(1)) {
        if (kem)
            PQC_LAUNCH(st, "nh_enc_single", N, 0,
                       nh_enc_single<N, true><<<n, NHS_THREADS, NhSingleSmem<N>::bytes(), st>>>(pk, coins, nullptr, ct, ss));
        else
            PQC_LAUNCH(st, "nh_enc_single", N, 0,
                       nh_enc_single<N, false><<<n, NHS_THREADS, NhSingleSmem<N>::bytes(), st>>>(pk, coins, m, ct, nullptr));
        return cudaGetLastError() == cudaSuccess ? PQCGPU_OK : PQCGPU_ECUDA;
    }
    EncArgs a{n, ct, pk, m, coins, 32, 32};
    if (kem) {
        PQC_LAUNCH(st, "nh_enc_hash_pre", N, 0, nh_enc_hash_pre<<<(n + 127) / 128, 128, 0, st>>>(n, coins, scratch, ss));
        a.m = scratch;
        a.coin = scratch + 32;
        a.m_stride = a.coin_stride = 64;
    }
    PQC_LAUNCH(st, "nh_enc_core", N, 0, nh_enc_core<N><<<(n + NI - 1) / NI, NT, sm, st>>>(a, NI));
    return cudaGetLastError() == cudaSuccess ? PQCGPU_OK : PQCGPU_ECUDA;
}

template <int N>
static int dec_n(int n, uint8_t *out, const uint8_t *ct, const uint8_t *sk, int kem, cudaStream_t st) {
    int NI, NT;
    g_shape[nidx(N)][2].get(NI, NT);
    const size_t sm = (size_t)NI * smem_per_instance(N, 2);
    if (prep(nh_dec_core<N>, sm)) return PQCGPU_ECUDA;
    DecArgs d{n, out, ct, sk, kem};
    PQC_LAUNCH(st, "nh_dec_core", N, 0, nh_dec_core<N><<<(n + NI - 1) / NI, NT, sm, st>>>(d, NI));
    return cudaGetLastError() == cudaSuccess ? PQCGPU_OK : PQCGPU_ECUDA;
}

// ---- persistent wave for the NewHope jobs of a mixed batch ----
// One launch holds the keypair, encapsulation and decapsulation tiles of every NewHope job (n = 1024
// and 512): SMs x (CTAs per SM) CTAs of 128 threads take tiles from a global counter, heaviest first,
// as the Kyber waves do (kyber_mixed.cu).  Instances per CTA per (n, op) at 128 threads.
namespace {
constexpr int NHW_MAX_JOBS = 40, NHW_THREADS = 128;
constexpr int NHW_NI[2][3] = {{8, 4, 4}, {16, 16, 8}};  // [n index][op]
struct NhWaveJob {
    int nidx, op, ni, first;
    KpArgs kp;
    EncArgs e;
    DecArgs d;
};
struct NhWaveTable {
    int njobs, tiles;
    NhWaveJob j[NHW_MAX_JOBS];
};
template <int N>
__device__ __forceinline__ void nhw_run(const NhWaveJob &m, int base) {
    if (m.op == 0) nh_kp_body<N>(m.kp, m.ni, base);
    else if (m.op == 1) nh_enc_body<N>(m.e, m.ni, base);
    else nh_dec_body<N>(m.d, m.ni, base);
}
__global__ void __launch_bounds__(NHW_THREADS, 2) nh_stage_persistent(const __grid_constant__ NhWaveTable t,
                                                                      unsigned *counter) {
    __shared__ int s_tile;
    for (;;) {
        if (threadIdx.x == 0) s_tile = (int)atomicAdd(counter, 1u);
        __syncthreads();
        const int tile = s_tile;
        if (tile >= t.tiles) break;
        int lo = 0, hi = t.njobs - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (t.j[mid].first <= tile) lo = mid;
            else hi = mid - 1;
        }
        const NhWaveJob &m = t.j[lo];
        const int base = (tile - m.first) * m.ni;
        if (m.nidx == 0) nhw_run<1024>(m, base);
        else nhw_run<512>(m, base);
        __syncthreads();
    }
}
}  // namespace

int newhope_mixed_wave(const std::vector<NhMixedJob> &jobs, unsigned *counters, int ncounters, cudaStream_t st) {
    std::vector<const NhMixedJob *> order;
    for (int op : {1, 0, 2})  // encapsulation tiles are the heaviest, decapsulation the lightest
        for (int N : {1024, 512})
            for (const auto &j : jobs)
                if (j.op == op && j.N == N && j.n > 0) order.push_back(&j);
    for (size_t from = 0, w = 0; from < order.size(); from += NHW_MAX_JOBS, w++) {
        if ((int)w >= ncounters) return PQCGPU_EINVAL;
        const size_t to = std::min(order.size(), from + NHW_MAX_JOBS);
        NhWaveTable t;
        t.njobs = (int)(to - from);
        t.tiles = 0;
        size_t sm = 0;
        for (size_t i = from; i < to; i++) {
            const NhMixedJob &j = *order[i];
            NhWaveJob &m = t.j[i - from];
            m.nidx = nidx(j.N);
            m.op = j.op;
            m.ni = NHW_NI[m.nidx][j.op];
            m.first = t.tiles;
            m.kp = KpArgs{j.n, j.out0, j.out1, j.in0, 32};
            m.e = EncArgs{j.n, j.out0, j.in0, j.scratch, j.scratch + 32, 64, 64};
            m.d = DecArgs{j.n, j.out0, j.in0, j.in1, 1};
            t.tiles += (j.n + m.ni - 1) / m.ni;
            sm = std::max(sm, (size_t)m.ni * smem_per_instance(j.N, j.op));
        }
        if (prep(nh_stage_persistent, sm)) return PQCGPU_ECUDA;
        int dev = 0, sms = 0, per_sm = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, nh_stage_persistent, NHW_THREADS, sm) != cudaSuccess ||
            per_sm < 1)
            per_sm = 1;
        if (cudaMemsetAsync(counters + w, 0, sizeof(unsigned), st) != cudaSuccess) return PQCGPU_ECUDA;
        PQC_LAUNCH(st, "nh_stage_persistent", 0, 0,
                   nh_stage_persistent<<<std::min(t.tiles, sms * per_sm), NHW_THREADS, sm, st>>>(t, counters + w));
        if (cudaGetLastError() != cudaSuccess) return PQCGPU_ECUDA;
    }
    return PQCGPU_OK;
}

// The CPA-KEM encapsulation prologue of one job of a mixed batch (before its wave).
int newhope_mixed_pre(const NhMixedJob &j, cudaStream_t st) {
    if (j.op != 1 || j.n <= 0) return PQCGPU_OK;
    PQC_LAUNCH(st, "nh_enc_hash_pre", j.N, 0,
               nh_enc_hash_pre<<<(j.n + 127) / 128, 128, 0, st>>>(j.n, j.in1, j.scratch, j.out1));
    return cudaGetLastError() == cudaSuccess ? PQCGPU_OK : PQCGPU_ECUDA;
}

int newhope_keypair_dev(int N, int n, uint8_t *pk, uint8_t *sk, const uint8_t *seed, int seed_stride, cudaStream_t st,
                        bool single_ok) {
    if (N == 1024) return keypair_n<1024>(n, pk, sk, seed, seed_stride, single_ok, st);
    if (N == 512) return keypair_n<512>(n, pk, sk, seed, seed_stride, single_ok, st);
    return PQCGPU_EINVAL;
}

// kem: coins 32 B per instance -> (m, coin) via the prologue into scratch (64 B / instance), ss
int newhope_enc_dev(int N, int n, uint8_t *ct, uint8_t *ss, const uint8_t *pk, const uint8_t *m, const uint8_t *coins,
                    uint8_t *scratch, int kem, cudaStream_t st, bool single_ok) {
    if (N == 1024) return enc_n<1024>(n, ct, ss, pk, m, coins, scratch, kem, single_ok, st);
    if (N == 512) return enc_n<512>(n, ct, ss, pk, m, coins, scratch, kem, single_ok, st);
    return PQCGPU_EINVAL;
}

int newhope_dec_dev(int N, int n, uint8_t *out, const uint8_t *ct, const uint8_t *sk, int kem, cudaStream_t st) {
    if (N == 1024) return dec_n<1024>(n, out, ct, sk, kem, st);
    if (N == 512) return dec_n<512>(n, out, ct, sk, kem, st);
    return PQCGPU_EINVAL;
}

}  // namespace pqc
