// Keccak-f[1600] and FIPS-202 sponges for sm_103a, one state per thread, all 25 lanes held in
// registers as 32-bit halves (uint2 {lo, hi}).
//
// Same function as the reference permutation (Kyber_GPU_Batched/fips202.cu:393-447) and sponge
// (:462-689), laid out for the GPU integer pipe instead of a rolled loop over a local array:
//   theta parity and chi are single LOP3 instructions (0x96 = a^b^c, 0xD2 = a^(~b&c)); theta's
//   D[x] = C[x-1] ^ rot(C[x+1], 1) is never formed: each lane takes A ^ C[x-1] ^ rot(C[x+1], 1) in
//   one LOP3, 180 ALU instructions a round instead of 190 (measured 4.18 -> 4.41 G permutations/s),
//   rho is two funnel shifts (SHF.L.W) per lane, pi is pure register renaming,
//   the round constants sit in constant memory (uniform access).
// Every index into the state is a compile-time constant after unrolling, so the state never
// touches local memory (checked with -Xptxas -v: 0 bytes stack).
#pragma once
#include <stdint.h>

namespace pqc {

__device__ __forceinline__ uint32_t lop3_xor3(uint32_t a, uint32_t b, uint32_t c) {
    uint32_t r;
    asm("lop3.b32 %0, %1, %2, %3, 0x96;" : "=r"(r) : "r"(a), "r"(b), "r"(c));
    return r;
}
// a ^ (~b & c)
__device__ __forceinline__ uint32_t lop3_chi(uint32_t a, uint32_t b, uint32_t c) {
    uint32_t r;
    asm("lop3.b32 %0, %1, %2, %3, 0xD2;" : "=r"(r) : "r"(a), "r"(b), "r"(c));
    return r;
}

__device__ __forceinline__ uint2 xor2(uint2 a, uint2 b) { return make_uint2(a.x ^ b.x, a.y ^ b.y); }

// 64-bit rotate-left of {lo, hi} by a compile-time-known n (0..63) via funnel shifts.
__device__ __forceinline__ uint2 rotl64(uint2 v, const int n) {
    if (n == 0) return v;
    if (n == 32) return make_uint2(v.y, v.x);
    if (n < 32) return make_uint2(__funnelshift_l(v.y, v.x, n), __funnelshift_l(v.x, v.y, n));
    return make_uint2(__funnelshift_l(v.x, v.y, n - 32), __funnelshift_l(v.y, v.x, n - 32));
}

// Rotation offsets r[x + 5y] (FIPS 202 Algorithm 2).
__device__ __forceinline__ constexpr int keccak_rho(int i) {
    constexpr int R[25] = {0, 1, 62, 28, 27, 36, 44, 6, 55, 20, 3, 10, 43, 25, 39,
                           41, 45, 15, 21, 8, 18, 2, 61, 56, 14};
    return R[i];
}

// Per translation unit; each .cu that includes this header uploads the table in its init function.
static __constant__ uint2 c_keccak_rc[24];

// Round constants from the rc(t) LFSR of FIPS 202 Algorithm 5 (host side, used at init).
static inline void keccak_rc_host(uint2 out[24]) {
    for (int ir = 0; ir < 24; ir++) {
        unsigned long long rc = 0;
        for (int j = 0; j <= 6; j++) {
            const int t = j + 7 * ir;
            int bit;
            if (t % 255 == 0) {
                bit = 1;
            } else {
                int R[9] = {1, 0, 0, 0, 0, 0, 0, 0, 0};
                for (int i = 1; i <= t % 255; i++) {
                    int Rn[9];
                    Rn[0] = 0;
                    for (int b = 0; b < 8; b++) Rn[b + 1] = R[b];
                    Rn[0] ^= Rn[8];
                    Rn[4] ^= Rn[8];
                    Rn[5] ^= Rn[8];
                    Rn[6] ^= Rn[8];
                    for (int b = 0; b < 9; b++) R[b] = Rn[b];
                }
                bit = R[0];
            }
            if (bit) rc |= 1ULL << ((1u << j) - 1);
        }
        out[ir] = make_uint2((unsigned)(rc & 0xffffffffu), (unsigned)(rc >> 32));
    }
}

// One round: theta, rho+pi into B, chi back into A, iota.
__device__ __forceinline__ void keccak_round(uint2 (&A)[25], const uint2 rc) {
    uint2 C[5], E[5], B[25];
#pragma unroll
    for (int x = 0; x < 5; x++) {
        C[x].x = lop3_xor3(lop3_xor3(A[x].x, A[x + 5].x, A[x + 10].x), A[x + 15].x, A[x + 20].x);
        C[x].y = lop3_xor3(lop3_xor3(A[x].y, A[x + 5].y, A[x + 10].y), A[x + 15].y, A[x + 20].y);
    }
#pragma unroll
    for (int x = 0; x < 5; x++) E[x] = rotl64(C[(x + 1) % 5], 1);
    // pi: B[X][Y] = rot(A[(X + 3Y) % 5][X]) -- output lane (X, Y) takes input lane (x, y) with
    // X = y, Y = 2x + 3y.
#pragma unroll
    for (int Y = 0; Y < 5; Y++)
#pragma unroll
        for (int X = 0; X < 5; X++) {
            const int sx = (X + 3 * Y) % 5, sy = X, li = sx + 5 * sy;
            const uint2 cm = C[(sx + 4) % 5];
            const uint2 t = make_uint2(lop3_xor3(A[li].x, cm.x, E[sx].x), lop3_xor3(A[li].y, cm.y, E[sx].y));
            B[X + 5 * Y] = rotl64(t, keccak_rho(li));
        }
#pragma unroll
    for (int Y = 0; Y < 5; Y++)
#pragma unroll
        for (int X = 0; X < 5; X++) {
            A[X + 5 * Y].x = lop3_chi(B[X + 5 * Y].x, B[(X + 1) % 5 + 5 * Y].x, B[(X + 2) % 5 + 5 * Y].x);
            A[X + 5 * Y].y = lop3_chi(B[X + 5 * Y].y, B[(X + 1) % 5 + 5 * Y].y, B[(X + 2) % 5 + 5 * Y].y);
        }
    A[0] = xor2(A[0], rc);
}

__device__ __forceinline__ void keccak_f1600(uint2 (&A)[25]) {
#pragma unroll 2
    for (int r = 0; r < 24; r++) keccak_round(A, c_keccak_rc[r]);
}

// The same permutation with the round loop rolled: half the code of keccak_f1600, for kernels whose
// several call sites would otherwise overflow the instruction cache.
__device__ __forceinline__ void keccak_f1600_rolled(uint2 (&A)[25]) {
#pragma unroll 1
    for (int r = 0; r < 24; r++) keccak_round(A, c_keccak_rc[r]);
}

__device__ __forceinline__ void keccak_zero(uint2 (&A)[25]) {
#pragma unroll
    for (int i = 0; i < 25; i++) A[i] = make_uint2(0, 0);
}

// XOR `pad` into byte 0 of lane `pos` (runtime pos < rate lanes) and 0x80 into the last rate byte.
template <int RATE_LANES>
__device__ __forceinline__ void keccak_pad(uint2 (&A)[25], int pos, uint32_t pad) {
#pragma unroll
    for (int i = 0; i < RATE_LANES; i++)
        if (i == pos) A[i].x ^= pad;
    A[RATE_LANES - 1].y ^= 0x80000000u;
}

// Absorb a message of `nlanes` 8-byte lanes (message length = 8 * nlanes) from memory that is
// 8-byte aligned, apply pad10*1 with domain byte `dom`, and leave the state ready to squeeze
// (the final permutation is NOT applied).  Works for global or shared pointers.
template <int RATE_LANES>
__device__ __forceinline__ void keccak_absorb_lanes(uint2 (&A)[25], const uint2 *in, int nlanes, uint32_t dom) {
    keccak_zero(A);
    while (nlanes >= RATE_LANES) {
#pragma unroll
        for (int i = 0; i < RATE_LANES; i++) A[i] = xor2(A[i], in[i]);
        keccak_f1600(A);
        in += RATE_LANES;
        nlanes -= RATE_LANES;
    }
#pragma unroll
    for (int i = 0; i < RATE_LANES; i++)
        if (i < nlanes) A[i] = xor2(A[i], in[i]);
    keccak_pad<RATE_LANES>(A, nlanes, dom);
}

// Asynchronous 8-byte copy global -> shared (LDGSTS: no register holds the data in flight).
__device__ __forceinline__ void cp_async8(void *smem, const void *gmem) {
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int PENDING>
__device__ __forceinline__ void cp_async_wait() {
    asm volatile("cp.async.wait_group %0;" ::"n"(PENDING) : "memory");
}

// keccak_absorb_lanes for a long message in global memory, one sponge per thread: block b + 1 is
// copied into shared memory while block b is permuted, so the loads' latency hides behind the
// permutation instead of stalling before each block.  `stage` is [2][RATE_LANES][nslots] uint2 of
// shared memory, of which this thread uses column `slot` (consecutive threads, consecutive 8-byte
// words: no bank conflicts); each thread reads only what its own copies wrote.
template <int RATE_LANES>
__device__ __forceinline__ void keccak_absorb_lanes_staged(uint2 (&A)[25], const uint2 *in, int nlanes, uint32_t dom,
                                                           uint2 *stage, int slot, int nslots) {
    keccak_zero(A);
    const int nb = nlanes / RATE_LANES;
    auto fetch = [&](int buf, const uint2 *src, int cnt) {
        uint2 *d = stage + buf * RATE_LANES * nslots + slot;
#pragma unroll
        for (int i = 0; i < RATE_LANES; i++)
            if (i < cnt) cp_async8(d + i * nslots, src + i);
        cp_async_commit();
    };
    fetch(0, in, nlanes < RATE_LANES ? nlanes : RATE_LANES);
    for (int b = 0; b < nb; b++) {
        const int left = nlanes - (b + 1) * RATE_LANES;
        fetch((b + 1) & 1, in + (b + 1) * RATE_LANES, left < RATE_LANES ? left : RATE_LANES);
        cp_async_wait<1>();
        const uint2 *s = stage + (b & 1) * RATE_LANES * nslots + slot;
#pragma unroll
        for (int i = 0; i < RATE_LANES; i++) A[i] = xor2(A[i], s[i * nslots]);
        keccak_f1600(A);
    }
    cp_async_wait<0>();
    const int rem = nlanes - nb * RATE_LANES;
    const uint2 *s = stage + (nb & 1) * RATE_LANES * nslots + slot;
#pragma unroll
    for (int i = 0; i < RATE_LANES; i++)
        if (i < rem) A[i] = xor2(A[i], s[i * nslots]);
    keccak_pad<RATE_LANES>(A, rem, dom);
}

// Absorb pre[0..npre) || in[0..nlanes) (whole lanes) and pad; the state is ready to permute.
template <int RATE_LANES>
__device__ __forceinline__ void keccak_absorb_lanes2(uint2 (&A)[25], const uint2 *pre, int npre, const uint2 *in,
                                                     int nlanes, uint32_t dom) {
    keccak_zero(A);
    const int total = npre + nlanes;
    int pos = 0;
    for (; total - pos >= RATE_LANES; pos += RATE_LANES) {
#pragma unroll
        for (int i = 0; i < RATE_LANES; i++) {
            const int g = pos + i;
            A[i] = xor2(A[i], g < npre ? pre[g] : in[g - npre]);
        }
        keccak_f1600(A);
    }
    const int rem = total - pos;
#pragma unroll
    for (int i = 0; i < RATE_LANES; i++)
        if (i < rem) {
            const int g = pos + i;
            A[i] = xor2(A[i], g < npre ? pre[g] : in[g - npre]);
        }
    keccak_pad<RATE_LANES>(A, rem, dom);
}

constexpr int SHAKE128_LANES = 21;  // rate 168
constexpr int SHAKE256_LANES = 17;  // rate 136
constexpr int SHA3_256_LANES = 17;  // rate 136
constexpr int SHA3_512_LANES = 9;   // rate 72
constexpr uint32_t DOM_SHAKE = 0x1F;
constexpr uint32_t DOM_SHA3 = 0x06;

}  // namespace pqc

// ---------------------------------------------------------------------------------------------
// One Keccak state spread over a warp: lane l < 25 holds state lane l (x = l % 5, y = l / 5).
// For long serial sponges (FrodoKEM's noise stream, G1 over a 15.6 KB key, F over a 15.7 KB
// ciphertext) the permutation's latency, not its throughput, bounds the batch: spreading the
// state over 25 lanes cuts the instructions on the critical path about six-fold, and message
// lanes are loaded (and output lanes stored) by consecutive threads.
// ---------------------------------------------------------------------------------------------
namespace pqc {

__device__ __forceinline__ uint2 shfl2(uint2 v, int src) {
    return make_uint2(__shfl_sync(0xffffffffu, v.x, src), __shfl_sync(0xffffffffu, v.y, src));
}
// rotate-left by a per-lane amount n in [0, 63]
__device__ __forceinline__ uint2 rotl64_var(uint2 v, int n) {
    const bool sw = n >= 32;
    const uint32_t lo = sw ? v.y : v.x, hi = sw ? v.x : v.y;
    n &= 31;
    return make_uint2(__funnelshift_l(hi, lo, n), __funnelshift_l(lo, hi, n));
}

struct WarpKeccak {
    int lane, rho, src_pi, src_pi1, src_pi2, col0, col1, col2, col3, xm1, xp1;
    __device__ __forceinline__ explicit WarpKeccak(int ln) {
        lane = ln;
        const int l = ln < 25 ? ln : 0;  // lanes 25..31 mirror lane 0; their values are never read
        const int x = l % 5, y = l / 5;
        constexpr int R[25] = {0, 1, 62, 28, 27, 36, 44, 6, 55, 20, 3, 10, 43, 25, 39,
                               41, 45, 15, 21, 8, 18, 2, 61, 56, 14};
        int r = 0;
#pragma unroll
        for (int i = 0; i < 25; i++)
            if (i == l) r = R[i];
        rho = r;
        // pi: lane (X, Y) takes A[(X + 3Y) % 5][X]; chi also needs what lanes (X+1, Y) and (X+2, Y)
        // take, so all three are gathered straight from the rotated state in one shuffle step
        src_pi = (x + 3 * y) % 5 + 5 * x;
        const int x1 = (x + 1) % 5, x2 = (x + 2) % 5;
        src_pi1 = (x1 + 3 * y) % 5 + 5 * x1;
        src_pi2 = (x2 + 3 * y) % 5 + 5 * x2;
        col0 = x + 5 * ((y + 1) % 5);
        col1 = x + 5 * ((y + 2) % 5);
        col2 = x + 5 * ((y + 3) % 5);
        col3 = x + 5 * ((y + 4) % 5);
        xm1 = (x + 4) % 5 + 5 * y;
        xp1 = (x + 1) % 5 + 5 * y;
    }
};

__device__ __forceinline__ void keccak_f1600_warp(uint2 &a, const WarpKeccak &w) {
#pragma unroll 1
    for (int r = 0; r < 24; r++) {
        uint2 c = xor2(xor2(a, shfl2(a, w.col0)), xor2(shfl2(a, w.col1), xor2(shfl2(a, w.col2), shfl2(a, w.col3))));
        const uint2 cm = shfl2(c, w.xm1), cp = shfl2(c, w.xp1);
        a = xor2(a, xor2(cm, rotl64(cp, 1)));
        a = rotl64_var(a, w.rho);
        const uint2 b = shfl2(a, w.src_pi), b1 = shfl2(a, w.src_pi1), b2 = shfl2(a, w.src_pi2);
        a.x = lop3_chi(b.x, b1.x, b2.x);
        a.y = lop3_chi(b.y, b1.y, b2.y);
        if (w.lane == 0) a = xor2(a, c_keccak_rc[r]);
    }
}

// Absorb the concatenation of two lane-aligned messages (n1 + n2 lanes) into a fresh warp state,
// with pad10*1 and domain byte `dom`; the final permutation is left to the caller.
template <int R>
__device__ __forceinline__ void warp_absorb2(uint2 &a, const uint2 *p1, int n1, const uint2 *p2, int n2, uint32_t dom,
                                             const WarpKeccak &w) {
    a = make_uint2(0, 0);
    const int total = n1 + n2;
    int done = 0;
    for (; total - done >= R; done += R) {
        const int i = done + w.lane;
        if (w.lane < R) a = xor2(a, i < n1 ? p1[i] : p2[i - n1]);
        keccak_f1600_warp(a, w);
    }
    const int i = done + w.lane;
    if (w.lane < total - done) a = xor2(a, i < n1 ? p1[i] : p2[i - n1]);
    if (w.lane == total - done) a.x ^= dom;
    if (w.lane == R - 1) a.y ^= 0x80000000u;
}

}  // namespace pqc
