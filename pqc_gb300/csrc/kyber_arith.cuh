// Kyber modular arithmetic and warp-cooperative NTT for sm_103a.
//
// Two families.  The int16 functions are the reference's (Kyber_GPU_Batched/reduce.cu:21-66:
// Montgomery with R = 2^16 and QINV = 62209, Barrett with v = floor(2^26 / q) + 1, conditional
// subtraction; ntt.cu:152-259 butterflies) and serve the per-stage path.  The fused kernels use
// plain residues with reductions that run on the multiply pipe (IMAD / IMAD.HI) instead of the
// integer ALU, which Keccak saturates: multiplication by a twiddle is Shoup's multiplication by a
// precomputed constant and a product is reduced by a Barrett high multiply.  These compute the same polynomials modulo q as the reference, with other representatives
// in between; every value that leaves a kernel (packed keys, compressed ciphertexts, messages) is
// first brought to [0, q) by the reference's Barrett and conditional subtraction, so the bytes are
// the reference's.
#pragma once
#include <stdint.h>

namespace pqc {
namespace kyber {

constexpr int N = 256;
constexpr int Q = 3329;
constexpr int POLY_PITCH = 296;  // int16 per shared-memory polynomial (256 + 8 per 64, +16 pad)

static __constant__ int16_t c_zetas[128];
static __constant__ int16_t c_zetas_inv[128];
// Twiddles of the fused kernels as Shoup pairs {w, floor(w 2^32 / q)}, w the representative of the
// plain twiddle in (-q/2, q/2); entry 127 of the inverse table is 1/128 mod q.
static __constant__ int2 c_tw[128];
static __constant__ int2 c_twi[128];

// zetas[i] = MONT * 17^brv7(i) mod q and the inverse-NTT table of the reference's generation
// recipe (Kyber_GPU_Batched/ntt.cu:8-48), computed on the host at init.
static inline void kyber_twiddles_host(int16_t zetas[128], int16_t zetas_inv[128]) {
    const long MONT = 2285;
    long pw[129];
    pw[0] = 1;
    for (int i = 1; i <= 128; i++) pw[i] = (pw[i - 1] * 17) % Q;
    auto brv7 = [](int x) { int r = 0; for (int i = 0; i < 7; i++) r |= ((x >> i) & 1) << (6 - i); return r; };
    auto modq = [](long v) { long r = v % Q; return (int16_t)(r < 0 ? r + Q : r); };
    for (int i = 0; i < 128; i++) zetas[i] = modq(MONT * pw[brv7(i)]);
    int k = 0;
    for (int i = 64; i >= 1; i >>= 1)
        for (int j = i; j < 2 * i; j++) zetas_inv[k++] = modq(-MONT * pw[128 - brv7(j)]);
    zetas_inv[127] = (int16_t)((MONT * ((MONT * (Q - 1) * ((Q - 1) / 128)) % Q)) % Q);
}

// Plain twiddles of the forward and inverse NTT (the reference's tables without the Montgomery
// factor) as Shoup pairs, and 1/128 for the end of the inverse transform.
static inline void kyber_twiddles_shoup_host(int2 tw[128], int2 twi[128]) {
    long pw[129];
    pw[0] = 1;
    for (int i = 1; i <= 128; i++) pw[i] = (pw[i - 1] * 17) % Q;
    auto brv7 = [](int x) { int r = 0; for (int i = 0; i < 7; i++) r |= ((x >> i) & 1) << (6 - i); return r; };
    auto pair = [](long v) {
        long w = v % Q;
        if (w < 0) w += Q;
        if (w > Q / 2) w -= Q;
        const long long num = (long long)w << 32;
        long long ws = num / Q;
        if (num % Q != 0 && num < 0) ws -= 1;  // floor
        return make_int2((int)w, (int)ws);
    };
    for (int i = 0; i < 128; i++) tw[i] = pair(pw[brv7(i)]);
    int k = 0;
    for (int i = 64; i >= 1; i >>= 1)
        for (int j = i; j < 2 * i; j++) twi[k++] = pair(-pw[128 - brv7(j)]);
    twi[127] = pair(3303);  // 128 * 3303 = 1 mod q
}

__device__ __forceinline__ int16_t mont_reduce(int32_t a) {
    const int16_t u = (int16_t)((uint32_t)a * 62209u);
    return (int16_t)((a - (int32_t)u * Q) >> 16);
}
__device__ __forceinline__ int16_t fqmul(int16_t a, int16_t b) { return mont_reduce((int32_t)a * b); }
__device__ __forceinline__ int16_t barrett(int16_t a) {
    const int32_t t = ((int32_t)20159 * a) >> 26;
    return (int16_t)(a - t * Q);
}
__device__ __forceinline__ int16_t csubq(int16_t a) {
    a = (int16_t)(a - Q);
    return (int16_t)(a + ((a >> 15) & Q));
}

// Physical index of coefficient i inside a shared-memory polynomial: 8 int16 of padding after
// every 64 coefficients keeps all three NTT access patterns free of bank conflicts while each run
// of 8 coefficients stays 16-byte aligned.
__device__ __forceinline__ int phys(int i) { return i + ((i >> 6) << 3); }

// basemul in Z_q[X]/(X^2 - zeta), Kyber_GPU_Batched/ntt.cu:249-259
__device__ __forceinline__ void basemul(int16_t &r0, int16_t &r1, int16_t a0, int16_t a1, int16_t b0, int16_t b1,
                                        int16_t zeta) {
    r0 = fqmul(a1, b1);
    r0 = fqmul(r0, zeta);
    r0 = (int16_t)(r0 + fqmul(a0, b0));
    r1 = fqmul(a0, b1);
    r1 = (int16_t)(r1 + fqmul(a1, b0));
}
// zeta of coefficient pair p (coefficients 2p, 2p+1): +zetas[64 + p/2] for even p, minus for odd.
__device__ __forceinline__ int16_t pair_zeta(const int16_t *sz, int p) {
    const int16_t z = sz[64 + (p >> 1)];
    return (p & 1) ? (int16_t)-z : z;
}

// Plain twiddle of coefficient pair p for the fused kernels' basemul: +w[64 + p/2] for even p, minus
// for odd.
__device__ __forceinline__ int32_t pair_w(const int2 *tw, int p) {
    const int32_t w = tw[64 + (p >> 1)].x;
    return (p & 1) ? -w : w;
}

// 32-bit forms for the NTTs.  The reference computes in int16, but no value of its transforms leaves
// the int16 range (forward inputs |x| < q grow by at most q per layer: < 8q after 7 layers; the
// inverse reduces every layer), so its truncations never take effect and the same arithmetic on
// 32-bit values gives the same numbers without a sign extension after every add and subtract.
// Only Montgomery's mod-2^16 step truncates.
__device__ __forceinline__ int32_t fqmul32(int32_t a, int32_t b) {
    const int32_t x = a * b;
    const int32_t u = (int16_t)((uint32_t)x * 62209u);
    return (x - u * Q) >> 16;
}
__device__ __forceinline__ int32_t barrett32(int32_t a) { return a - ((20159 * a) >> 26) * Q; }
__device__ __forceinline__ void ct_bfly32(int32_t &a, int32_t &b, int32_t z) {
    const int32_t t = fqmul32(z, b);
    b = a - t;
    a = a + t;
}
__device__ __forceinline__ void gs_bfly32(int32_t &a, int32_t &b, int32_t z) {
    const int32_t t = a;
    a = barrett32(t + b);
    b = fqmul32(z, t - b);
}
// basemul of the 32-bit forms: each Montgomery product is below q in magnitude, so r0 < 2q and
// r1 < 2q, the bounds of the reference's int16 basemul, and sums of K <= 4 of them stay below 8q.
__device__ __forceinline__ void basemul32(int32_t &r0, int32_t &r1, int32_t a0, int32_t a1, int32_t b0, int32_t b1,
                                          int32_t zeta) {
    r0 = fqmul32(fqmul32(a1, b1), zeta) + fqmul32(a0, b0);
    r1 = fqmul32(a0, b1) + fqmul32(a1, b0);
}
// Multiplication by a twiddle (Shoup, "NTL: MulModPrecon"): for |b| < 2^15 the estimated quotient
// floor(b w' / 2^32), w' = floor(w 2^32 / q), is off by less than 2^-17, so the result is the
// representative of b w in [0, q].  Three multiply-pipe instructions.
__device__ __forceinline__ int32_t mulc(int32_t b, int2 w) { return b * w.x - __mulhi(b, w.y) * Q; }
// Barrett reduction of a product sum |x| < 2^25 by a high multiply with floor(2^32 / q): result in
// [-11, q + 11].
__device__ __forceinline__ int32_t red_prod(int32_t x) { return x - __mulhi(x, 1290167) * Q; }
// The reference's Barrett, floor(20159 a / 2^26) taken as the high word of a * (20159 * 2^6):
// the same quotient, result in [0, q].
__device__ __forceinline__ int32_t barrett_hi(int32_t a) { return a - __mulhi(a, 20159 << 6) * Q; }
// basemul in Z_q[X]/(X^2 - zeta) on plain residues (ntt.cu:249-259 without the Montgomery factor):
// one reduction per product sum.  |a| < 2^12 (packed 12-bit or sampled coefficients), b in [0, q]
// (reduced NTT output), |zeta| < q/2: results in [-11, q + 11].
__device__ __forceinline__ void basemul_plain(int32_t &r0, int32_t &r1, int32_t a0, int32_t a1, int32_t b0, int32_t b1,
                                              int32_t zeta) {
    r0 = red_prod(red_prod(a1 * b1) * zeta + a0 * b0);
    r1 = red_prod(a0 * b1 + a1 * b0);
}
// Forward butterfly: t in [0, q], so a coefficient grows by at most q a layer (< 8q after seven
// layers from |x| <= q, within int16 for the shared-memory passes).
__device__ __forceinline__ void ct_bfly_s(int32_t &a, int32_t &b, int2 w) {
    const int32_t t = mulc(b, w);
    b = a - t;
    a = a + t;
}
// Inverse butterfly (ntt.cu:194-224 without the Montgomery factor): both outputs in [0, q].
__device__ __forceinline__ void gs_bfly_s(int32_t &a, int32_t &b, int2 w) {
    const int32_t t = a;
    a = barrett_hi(t + b);
    b = mulc(t - b, w);
}
__device__ __forceinline__ void load8(int32_t (&r)[8], const int16_t *p) {
    const uint4 v = *reinterpret_cast<const uint4 *>(p);
    const uint32_t w[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
    for (int i = 0; i < 4; i++) {
        r[2 * i] = (int16_t)(w[i] & 0xffff);
        r[2 * i + 1] = (int32_t)w[i] >> 16;
    }
}
__device__ __forceinline__ void store8(int16_t *p, const int32_t (&r)[8]) {
    auto pk2 = [](int32_t lo, int32_t hi) { return ((uint32_t)lo & 0xffffu) | ((uint32_t)hi << 16); };
    *reinterpret_cast<uint4 *>(p) = make_uint4(pk2(r[0], r[1]), pk2(r[2], r[3]), pk2(r[4], r[5]), pk2(r[6], r[7]));
}

__device__ __forceinline__ void ct_bfly(int16_t &a, int16_t &b, int16_t z) {
    const int16_t t = fqmul(z, b);
    b = (int16_t)(a - t);
    a = (int16_t)(a + t);
}
__device__ __forceinline__ void gs_bfly(int16_t &a, int16_t &b, int16_t z) {
    const int16_t t = a;
    a = barrett((int16_t)(t + b));
    b = (int16_t)(t - b);
    b = fqmul(z, b);
}

__device__ __forceinline__ void load8(int16_t (&r)[8], const int16_t *p) {
    const uint4 v = *reinterpret_cast<const uint4 *>(p);
    r[0] = (int16_t)(v.x & 0xffff); r[1] = (int16_t)(v.x >> 16);
    r[2] = (int16_t)(v.y & 0xffff); r[3] = (int16_t)(v.y >> 16);
    r[4] = (int16_t)(v.z & 0xffff); r[5] = (int16_t)(v.z >> 16);
    r[6] = (int16_t)(v.w & 0xffff); r[7] = (int16_t)(v.w >> 16);
}
__device__ __forceinline__ uint32_t pack2(int16_t a, int16_t b) { return (uint16_t)a | ((uint32_t)(uint16_t)b << 16); }
__device__ __forceinline__ void store8(int16_t *p, const int16_t (&r)[8]) {
    *reinterpret_cast<uint4 *>(p) = make_uint4(pack2(r[0], r[1]), pack2(r[2], r[3]), pack2(r[4], r[5]), pack2(r[6], r[7]));
}

// Forward NTT + Barrett (poly_ntt, poly.cu:153-157) of one shared-memory polynomial by one warp,
// on plain residues (output in [0, q]).
// Three passes, each doing the butterflies of a 3-bit (or 2-bit) slice of the index in registers:
//   pass 1: lane = bits 4..0, registers = bits 7,6,5   -> layers len 128, 64, 32
//   pass 2: lane = bits 6,5,2,1,0, registers = 7,4,3   -> layers len 16, 8
//   pass 3: lane = bits 7..3, registers = bits 2,1,0   -> layers len 4, 2, then Barrett
// `tw` is the twiddle table in shared memory (lane-dependent indices in passes 2 and 3).
__device__ __forceinline__ void ntt_warp(int16_t *p, const int2 *tw, int lane) {
    int32_t r[8];
#pragma unroll
    for (int m = 0; m < 8; m++) r[m] = p[phys(32 * m + lane)];
    {
        const int2 z = tw[1];
#pragma unroll
        for (int m = 0; m < 4; m++) ct_bfly_s(r[m], r[m + 4], z);
    }
#pragma unroll
    for (int m = 0; m < 8; m++)
        if (!(m & 2)) ct_bfly_s(r[m], r[m + 2], tw[2 + (m >> 2)]);
#pragma unroll
    for (int m = 0; m < 8; m += 2) ct_bfly_s(r[m], r[m + 1], tw[4 + (m >> 1)]);
#pragma unroll
    for (int m = 0; m < 8; m++) p[phys(32 * m + lane)] = (int16_t)r[m];
    __syncwarp();

    const int l65 = lane >> 3, l210 = lane & 7;
#pragma unroll
    for (int q = 0; q < 8; q++)
        r[q] = p[phys(128 * (q >> 2) + 32 * l65 + 16 * ((q >> 1) & 1) + 8 * (q & 1) + l210)];
#pragma unroll
    for (int q = 0; q < 8; q++)
        if (!(q & 2)) ct_bfly_s(r[q], r[q + 2], tw[8 + 4 * (q >> 2) + l65]);
#pragma unroll
    for (int q = 0; q < 8; q += 2) ct_bfly_s(r[q], r[q + 1], tw[16 + 8 * (q >> 2) + 2 * l65 + ((q >> 1) & 1)]);
#pragma unroll
    for (int q = 0; q < 8; q++)
        p[phys(128 * (q >> 2) + 32 * l65 + 16 * ((q >> 1) & 1) + 8 * (q & 1) + l210)] = (int16_t)r[q];
    __syncwarp();

    int16_t *p8 = p + phys(8 * lane);
    load8(r, p8);
    {
        const int2 z = tw[32 + lane];
#pragma unroll
        for (int q = 0; q < 4; q++) ct_bfly_s(r[q], r[q + 4], z);
    }
#pragma unroll
    for (int q = 0; q < 8; q++)
        if (!(q & 2)) ct_bfly_s(r[q], r[q + 2], tw[64 + 2 * lane + (q >> 2)]);
#pragma unroll
    for (int q = 0; q < 8; q++) r[q] = barrett_hi(r[q]);
    store8(p8, r);
    __syncwarp();
}

// Inverse NTT including the final multiplication by 1/128 (invntt, ntt.cu:194-224, whose mont^2/128
// also undoes the Montgomery factor of its basemul); the passes mirror ntt_warp in reverse order.
// `twi` is the inverse twiddle table in shared memory.  Output in [0, q].
__device__ __forceinline__ void invntt_warp(int16_t *p, const int2 *twi, int lane) {
    int32_t r[8];
    int16_t *p8 = p + phys(8 * lane);
    load8(r, p8);
#pragma unroll
    for (int q = 0; q < 8; q++)
        if (!(q & 2)) gs_bfly_s(r[q], r[q + 2], twi[2 * lane + (q >> 2)]);
    {
        const int2 z = twi[64 + lane];
#pragma unroll
        for (int q = 0; q < 4; q++) gs_bfly_s(r[q], r[q + 4], z);
    }
    store8(p8, r);
    __syncwarp();

    const int l65 = lane >> 3, l210 = lane & 7;
#pragma unroll
    for (int q = 0; q < 8; q++)
        r[q] = p[phys(128 * (q >> 2) + 32 * l65 + 16 * ((q >> 1) & 1) + 8 * (q & 1) + l210)];
#pragma unroll
    for (int q = 0; q < 8; q += 2) gs_bfly_s(r[q], r[q + 1], twi[96 + 8 * (q >> 2) + 2 * l65 + ((q >> 1) & 1)]);
#pragma unroll
    for (int q = 0; q < 8; q++)
        if (!(q & 2)) gs_bfly_s(r[q], r[q + 2], twi[112 + 4 * (q >> 2) + l65]);
#pragma unroll
    for (int q = 0; q < 8; q++)
        p[phys(128 * (q >> 2) + 32 * l65 + 16 * ((q >> 1) & 1) + 8 * (q & 1) + l210)] = (int16_t)r[q];
    __syncwarp();

#pragma unroll
    for (int m = 0; m < 8; m++) r[m] = p[phys(32 * m + lane)];
#pragma unroll
    for (int m = 0; m < 8; m += 2) gs_bfly_s(r[m], r[m + 1], twi[120 + (m >> 1)]);
#pragma unroll
    for (int m = 0; m < 8; m++)
        if (!(m & 2)) gs_bfly_s(r[m], r[m + 2], twi[124 + (m >> 2)]);
    {
        const int2 z = twi[126];
#pragma unroll
        for (int m = 0; m < 4; m++) gs_bfly_s(r[m], r[m + 4], z);
    }
    const int2 f = twi[127];
#pragma unroll
    for (int m = 0; m < 8; m++) p[phys(32 * m + lane)] = (int16_t)mulc(r[m], f);
    __syncwarp();
}

}  // namespace kyber
}  // namespace pqc
