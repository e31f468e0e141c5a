// Single-instance Kyber KEM kernels: the latency path for small batches (implementation header,
// included by kyber_impl.cuh and instantiated per (k, variant)).
//
// One CTA of SINGLE_WARPS warps runs a whole keypair, encapsulation or decapsulation of one
// instance, with no intermediate launch.  Every sponge runs on the 25-lane warp permutation
// (keccak.cuh), whose latency is about half that of a one-thread permutation, and independent
// sponges run on different warps at the same time:
//   * the matrix entries are sampled by warps while the serial hashes run -- H(pk) (and H(coins))
//     in encapsulation, H(c) in decapsulation -- since A depends only on rho;
//   * rejection sampling is warp-parallel: after each SHAKE128 block every lane parses the
//     candidates in its own state lane (plus one shuffle for 12-bit triplets that straddle two
//     lanes) and three ballots give each lane its prefix count, so the accepted coefficients land
//     in stream order, the first 256 of them exactly as in the reference's rej_uniform
//     (Kyber_GPU_Batched/indcpa.cu:290-322);
//   * noise, NTTs, products, codecs and the FO / FIPS 203 layer are the batched kernels' steps,
//     a warp per polynomial.
// Decapsulation keeps its H(c) warp outside the CTA barrier: the other warps synchronise on a
// named barrier (bar.sync 1) through decryption, G, re-encryption and the comparison, and all
// warps meet once before the final key derivation.
//
// Reference call stacks replaced for one instance: indcpa_keypair / enc / dec
// (Kyber_GPU_Batched/indcpa.cu:474-733) behind the crypto_kem_* entry points
// (Kyber_GPU_Batched/api.h:18-22); the single-CTA design of NewHope_NIST_GPU_Single (a CTA of
// cooperating threads per operation, NewHope_NIST_GPU_Single/ntt.cu:1015-1091).
#pragma once

namespace pqc {
namespace kyber {

constexpr int SINGLE_WARPS = 16;
constexpr int SINGLE_THREADS = SINGLE_WARPS * 32;

// Shared-memory layout of one instance.
template <int K, int V>
struct SingleSmem {
    static constexpr int PRFB = 192;  // bytes per PRF output (eta = 3 needs 192, eta = 2 uses 128)
    static constexpr int NPOLY = 3 * K + 2;
    int2 *tw, *twi;
    int16_t *A;      // K*K sampled matrix entries (NTT domain), entry i*K + j
    int16_t *polys;  // NPOLY polynomials
    uint8_t *prf;    // (2K + 1) PRF outputs
    uint8_t *buf;    // encapsulation: pk copy, then the ciphertext; decapsulation: ct copy; keypair: pk
    static_assert(P<K, V>::PKB <= 1600 && P<K, V>::CTB <= 1600, "buf holds a public key or a ciphertext");
    uint2 *seeds;    // 32 lanes: [0,4) m, [4,8) h, [8,12) K-bar, [12,16) r, [16,20) rho, [20,24) sigma,
                     // [24,28) H(c) or J(z || c), [28] fail flag
    __device__ __forceinline__ explicit SingleSmem(uint8_t *s) {
        tw = reinterpret_cast<int2 *>(s);
        twi = tw + 128;
        A = reinterpret_cast<int16_t *>(twi + 128);
        polys = A + K * K * POLY_PITCH;
        prf = reinterpret_cast<uint8_t *>(polys + NPOLY * POLY_PITCH);
        buf = prf + (2 * K + 1) * PRFB;
        seeds = reinterpret_cast<uint2 *>(buf + 1600);
    }
    __device__ __forceinline__ int16_t *poly(int i) const { return polys + i * POLY_PITCH; }
    static __host__ __device__ constexpr size_t bytes() {
        return 2 * 128 * sizeof(int2) + (size_t)(K * K + NPOLY) * POLY_PITCH * sizeof(int16_t) + (2 * K + 1) * PRFB +
               1600 + 32 * sizeof(uint2);
    }
};

// Named barrier among the warps [1, SINGLE_WARPS) of the CTA (warp 0 runs a serial hash meanwhile).
__device__ __forceinline__ void single_bar_rest() {
    asm volatile("bar.sync 1, %0;" ::"r"((SINGLE_WARPS - 1) * 32) : "memory");
}

// PRF(seed, nonce) = SHAKE256(seed || nonce) by one warp; 128 bytes (eta = 2) or 192 (eta = 3)
// into `out` (shared, 8-byte aligned).
template <int ETA>
__device__ __forceinline__ void warp_prf(const uint2 *seed, int nonce, uint8_t *out, const WarpKeccak &w) {
    uint2 a = w.lane < 4 ? seed[w.lane] : make_uint2(0, 0);
    if (w.lane == 4) a.x = (uint32_t)nonce | (DOM_SHAKE << 8);
    if (w.lane == SHAKE256_LANES - 1) a.y ^= 0x80000000u;
    keccak_f1600_warp(a, w);
    uint2 *o = reinterpret_cast<uint2 *>(out);
    if (ETA == 2) {
        if (w.lane < 16) o[w.lane] = a;
    } else {
        if (w.lane < 17) o[w.lane] = a;
        keccak_f1600_warp(a, w);
        if (w.lane < 7) o[17 + w.lane] = a;
    }
    __syncwarp();
}

// Matrix entry XOF(rho || x || y) rejection-sampled by one warp into dst (shared polynomial,
// coefficients in [0, q) as the reference's int16 values).  Round 3: 12-bit candidates < q from
// 3-byte groups; round 2: 16-bit candidates < 19q reduced by v - (v >> 12) q.
template <int V>
__device__ void warp_sample_entry(const uint2 *rho, int x, int y, int16_t *dst, const WarpKeccak &w) {
    uint2 a = w.lane < 4 ? rho[w.lane] : make_uint2(0, 0);
    if (w.lane == 4) a.x = (uint32_t)x | ((uint32_t)y << 8) | (DOM_SHAKE << 16);
    if (w.lane == SHAKE128_LANES - 1) a.y ^= 0x80000000u;
    const unsigned below = (1u << w.lane) - 1u;
    int cnt = 0;
    while (cnt < N) {  // warp-uniform
        keccak_f1600_warp(a, w);
        uint32_t c[6];
        bool ok[6];
        if (V == 3) {
            // lane l < 21 holds bytes [8l, 8l + 8) of the block; the 3-byte groups starting there
            // begin at offsets r, r + 3, r + 6 (r = l mod 3; two groups when r = 2)
            const uint2 nx = shfl2(a, (w.lane + 1) & 31);
            const uint32_t q0 = a.x, q1 = a.y, q2 = nx.x;
            const int r = w.lane % 3;
            const int ntrip = w.lane < SHAKE128_LANES ? (r == 2 ? 2 : 3) : 0;
#pragma unroll
            for (int t = 0; t < 3; t++) {
                const int o = r + 3 * t, sh = 8 * (o & 3);
                const uint32_t lo = (o >> 2) ? q1 : q0, hi = (o >> 2) ? q2 : q1;
                const uint32_t v = __funnelshift_r(lo, hi, sh) & 0xffffffu;
                c[2 * t] = v & 0xfff;
                c[2 * t + 1] = v >> 12;
                ok[2 * t] = t < ntrip && c[2 * t] < (uint32_t)Q;
                ok[2 * t + 1] = t < ntrip && c[2 * t + 1] < (uint32_t)Q;
            }
        } else {
            // lane l < 21 holds the 16-bit candidates 4l .. 4l + 3
            const bool valid = w.lane < SHAKE128_LANES;
            c[0] = a.x & 0xffff;
            c[1] = a.x >> 16;
            c[2] = a.y & 0xffff;
            c[3] = a.y >> 16;
#pragma unroll
            for (int i = 0; i < 4; i++) {
                ok[i] = valid && c[i] < (uint32_t)(19 * Q);
                c[i] = c[i] - (c[i] >> 12) * Q;
            }
            ok[4] = ok[5] = false;
        }
        int k = 0;
#pragma unroll
        for (int i = 0; i < 6; i++) k += ok[i];
        const unsigned b0 = __ballot_sync(0xffffffffu, k & 1), b1 = __ballot_sync(0xffffffffu, k & 2),
                       b2 = __ballot_sync(0xffffffffu, k & 4);
        int pos = cnt + __popc(b0 & below) + 2 * __popc(b1 & below) + 4 * __popc(b2 & below);
#pragma unroll
        for (int i = 0; i < 6; i++)
            if (ok[i]) {
                if (pos < N) dst[phys(pos)] = (int16_t)c[i];
                pos++;
            }
        cnt += __popc(b0) + 2 * __popc(b1) + 4 * __popc(b2);
    }
    __syncwarp();
}

// CBD of a PRF output into a shared polynomial, a warp: lane = 8 coefficients (cbd.cu:42-63).
template <int ETA>
__device__ __forceinline__ void warp_cbd(const uint8_t *b, int16_t *p, int lane) {
    int16_t c[8];
    if (ETA == 2) {
        const uint32_t t = reinterpret_cast<const uint32_t *>(b)[lane];
        uint32_t d = t & 0x55555555u;
        d += (t >> 1) & 0x55555555u;
#pragma unroll
        for (int q = 0; q < 8; q++) c[q] = (int16_t)((int)((d >> (4 * q)) & 3) - (int)((d >> (4 * q + 2)) & 3));
    } else {
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
    store8(p + phys(8 * lane), c);
    __syncwarp();
}

// acc[8] (lane's 8 coefficients) = sum_j x_j o y_j with x_j from `xa` (shared polynomials at stride
// xs) or, when xb is given, decoded from 12-bit bytes at stride 384 (a packed t-hat or s-hat), and
// y_j the shared polynomials at ya (stride POLY_PITCH); result reduced to [0, q].
template <int K>
__device__ __forceinline__ void warp_dot(int32_t (&acc)[8], const int16_t *xa, int xs, const uint8_t *xb,
                                         const int16_t *ya, const int2 *tw, int lane) {
#pragma unroll
    for (int q = 0; q < 8; q++) acc[q] = 0;
    for (int j = 0; j < K; j++) {
        int32_t x[8], y[8], r[8];
        if (xb) frombytes8(x, xb + 384 * j + 12 * lane);
        else load8(x, xa + j * xs + phys(8 * lane));
        load8(y, ya + j * POLY_PITCH + phys(8 * lane));
#pragma unroll
        for (int q = 0; q < 4; q++)
            basemul_plain(r[2 * q], r[2 * q + 1], x[2 * q], x[2 * q + 1], y[2 * q], y[2 * q + 1], pair_w(tw, 4 * lane + q));
#pragma unroll
        for (int q = 0; q < 8; q++) acc[q] += r[q];
    }
#pragma unroll
    for (int q = 0; q < 8; q++) acc[q] = barrett_hi(acc[q]);
}

// Encryption tail of polynomial t (t < K: u_t with e1_t, t = K: v with e2 and the message): add
// the noise, compress and pack the lane's bytes into the ciphertext at `out` (shared), or (CMP)
// compare them with `cmp` and return whether they differ.
template <int K, int V, bool CMP>
__device__ __forceinline__ uint32_t warp_pack_ct(const int16_t *p, const uint8_t *ebytes, uint8_t msgbyte, int t,
                                                 uint8_t *out, const uint8_t *cmp, int lane) {
    using Pp = P<K, V>;
    const uint32_t tt = reinterpret_cast<const uint32_t *>(ebytes)[lane];
    uint32_t d = tt & 0x55555555u;
    d += (tt >> 1) & 0x55555555u;
    int16_t c[8];
    load8(c, p + phys(8 * lane));
    uint32_t cv[8];
#pragma unroll
    for (int q = 0; q < 8; q++) {
        const int16_t e = (int16_t)((int)((d >> (4 * q)) & 3) - (int)((d >> (4 * q + 2)) & 3));
        int16_t x = (int16_t)(c[q] + e);
        if (t == K) x = (int16_t)(x + (int16_t)(((msgbyte >> q) & 1) ? (Q + 1) / 2 : 0));
        x = csubq(barrett(x));
        cv[q] = (t < K) ? compress_d<Pp::DU>(x) : compress_d<Pp::DV>(x);
    }
    uint32_t diff = 0;
    if (t < K) {
        uint8_t b[Pp::DU];
        pack8<Pp::DU>(b, cv);
        const int off = t * Pp::DU * 32 + lane * Pp::DU;
#pragma unroll
        for (int q = 0; q < Pp::DU; q++) {
            if (CMP) diff |= (uint32_t)(b[q] ^ cmp[off + q]);
            else out[off + q] = b[q];
        }
    } else {
        uint8_t b[Pp::DV];
        pack8<Pp::DV>(b, cv);
        const int off = Pp::CTU + lane * Pp::DV;
#pragma unroll
        for (int q = 0; q < Pp::DV; q++) {
            if (CMP) diff |= (uint32_t)(b[q] ^ cmp[off + q]);
            else out[off + q] = b[q];
        }
    }
    return diff;
}

// Re-encryption / encryption body after (m, r) sit in S.seeds, run by the warps [w0, w0 + nw):
// PRFs, noise NTT, the products with the sampled matrix and t-hat (pk bytes at pkb), inverse NTT,
// and the ciphertext (CMP: comparison with cmp, the result ORed into the fail flag).  `sync` is
// the barrier shared by those warps.  Polynomials: [0, K) r-hat, [K, 2K + 1) u and v.
template <int K, int V, bool CMP, class Sync>
__device__ __forceinline__ void single_encrypt(const SingleSmem<K, V> &S, const uint8_t *pkb, const uint8_t *cmp,
                                               int w0, int nw, Sync sync) {
    using Pp = P<K, V>;
    constexpr int SP = SingleSmem<K, V>::PRFB;
    const int lane = threadIdx.x & 31, warp = (threadIdx.x >> 5) - w0;
    const WarpKeccak w(lane);
    const uint2 *r = S.seeds + 12;
    for (int j = warp; j < 2 * K + 1; j += nw) {
        if (j < K) warp_prf<Pp::ETA1>(r, j, S.prf + j * SP, w);
        else warp_prf<2>(r, j, S.prf + j * SP, w);
    }
    sync();
    for (int j = warp; j < K; j += nw) {
        warp_cbd<Pp::ETA1>(S.prf + j * SP, S.poly(j), lane);
        ntt_warp(S.poly(j), S.tw, lane);
    }
    sync();
    // u_t = sum_j A^T[t][j] o r-hat_j (entry t*K + j was sampled with x = t, y = j); v = t-hat o r-hat
    for (int t = warp; t <= K; t += nw) {
        int32_t acc[8];
        if (t < K) warp_dot<K>(acc, S.A + t * K * POLY_PITCH, POLY_PITCH, nullptr, S.poly(0), S.tw, lane);
        else warp_dot<K>(acc, nullptr, 0, pkb, S.poly(0), S.tw, lane);
        int16_t *u = S.poly(K + t);
        store8(u + phys(8 * lane), acc);
        __syncwarp();
        invntt_warp(u, S.twi, lane);
    }
    sync();
    const uint8_t *msg = reinterpret_cast<const uint8_t *>(S.seeds);
    uint32_t *fail = reinterpret_cast<uint32_t *>(S.seeds + 28);
    for (int t = warp; t <= K; t += nw) {
        const uint32_t d = warp_pack_ct<K, V, CMP>(S.poly(K + t), S.prf + (K + t) * SP, msg[lane], t, S.buf, cmp, lane);
        if (CMP && __any_sync(0xffffffffu, d != 0) && lane == 0) atomicOr(fail, 1u);
    }
}

// ---- kernels: one CTA of SINGLE_THREADS per instance ------------------------------------------

// Encapsulation (KEM_FO: m = H(coins), ss = KDF(K-bar || H(c)); KEM_MLKEM: m = coins, ss = K).
template <int K, int V>
__global__ void __launch_bounds__(SINGLE_THREADS) kyber_enc_single(const uint8_t *pk, const uint8_t *coins,
                                                                   uint8_t *ct, uint8_t *ss, int kem) {
    using Pp = P<K, V>;
    extern __shared__ __align__(16) uint8_t smem[];
    const SingleSmem<K, V> S(smem);
    const int x = blockIdx.x, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const WarpKeccak w(lane);
    const uint8_t *pki = pk + (size_t)x * Pp::PKB;
    load_twiddles(S.tw, S.twi);
    // the public key to shared memory in one coalesced pass: H(pk), the matrix seed rho and t-hat
    // are read from there, so no global-load latency sits inside the serial H(pk) sponge (the
    // ciphertext overwrites this copy only after t-hat has been used)
    for (int i = tid; i < Pp::PKB / 8; i += SINGLE_THREADS)
        reinterpret_cast<uint2 *>(S.buf)[i] = reinterpret_cast<const uint2 *>(pki)[i];
    const uint2 *rho = reinterpret_cast<const uint2 *>(S.buf + Pp::POLYVECBYTES);
    __syncthreads();
    if (warp == 0) {  // m
        const uint2 *cn = reinterpret_cast<const uint2 *>(coins + (size_t)x * 32);
        uint2 m;
        if (kem == KEM_MLKEM) {
            m = lane < 4 ? cn[lane] : make_uint2(0, 0);
        } else {
            warp_absorb2<SHA3_256_LANES>(m, cn, 4, nullptr, 0, DOM_SHA3, w);
            keccak_f1600_warp(m, w);
        }
        if (lane < 4) S.seeds[lane] = m;
    } else if (warp == 1) {  // H(pk)
        uint2 h;
        warp_absorb2<SHA3_256_LANES>(h, reinterpret_cast<const uint2 *>(S.buf), Pp::PKB / 8, nullptr, 0, DOM_SHA3, w);
        keccak_f1600_warp(h, w);
        if (lane < 4) S.seeds[4 + lane] = h;
    } else {  // the matrix entries A^T[i][j] = XOF(rho || i || j), meanwhile
        for (int e = warp - 2; e < K * K; e += SINGLE_WARPS - 2)
            warp_sample_entry<V>(rho, e / K, e % K, S.A + e * POLY_PITCH, w);
    }
    __syncthreads();
    if (warp == 0) {  // (K-bar, r) = G(m || H(pk))
        uint2 g = lane < 8 ? S.seeds[lane] : make_uint2(0, 0);
        if (lane == SHA3_512_LANES - 1) {
            g.x ^= DOM_SHA3;
            g.y ^= 0x80000000u;
        }
        keccak_f1600_warp(g, w);
        if (lane < 8) S.seeds[8 + lane] = g;  // lanes 0-3 K-bar, 4-7 r
    }
    __syncthreads();
    single_encrypt<K, V, false>(S, S.buf, nullptr, 0, SINGLE_WARPS, [] { __syncthreads(); });
    __syncthreads();
    uint8_t *cti = ct + (size_t)x * Pp::CTB;
    for (int i = tid; i < Pp::CTB / 8; i += SINGLE_THREADS)
        reinterpret_cast<uint2 *>(cti)[i] = reinterpret_cast<const uint2 *>(S.buf)[i];
    if (warp == 0) {
        uint2 *o = reinterpret_cast<uint2 *>(ss + (size_t)x * 32);
        if (kem == KEM_MLKEM) {
            if (lane < 4) o[lane] = S.seeds[8 + lane];
        } else {  // KDF(K-bar || H(c))
            uint2 h;
            warp_absorb2<SHA3_256_LANES>(h, reinterpret_cast<const uint2 *>(S.buf), Pp::CTB / 8, nullptr, 0, DOM_SHA3, w);
            keccak_f1600_warp(h, w);
            const uint2 hs = shfl2(h, (lane - 4) & 31);
            uint2 a = lane < 4 ? S.seeds[8 + lane] : (lane < 8 ? hs : make_uint2(0, 0));
            if (lane == 8) a.x ^= DOM_SHAKE;
            if (lane == SHAKE256_LANES - 1) a.y ^= 0x80000000u;
            keccak_f1600_warp(a, w);
            if (lane < 4) o[lane] = a;
        }
    }
}

// Decapsulation: warp 0 computes H(c) (KEM_MLKEM: the rejection key J(z || c)) while the other
// warps decrypt, derive (K-bar', r') = G(m' || h), sample the matrix and re-encrypt; then the
// constant-time selection and (KEM_FO) the KDF.
template <int K, int V>
__global__ void __launch_bounds__(SINGLE_THREADS) kyber_dec_single(const uint8_t *ct, const uint8_t *sk, uint8_t *ss,
                                                                   int kem) {
    using Pp = P<K, V>;
    extern __shared__ __align__(16) uint8_t smem[];
    const SingleSmem<K, V> S(smem);
    const int x = blockIdx.x, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const WarpKeccak w(lane);
    const uint8_t *cti, *ski = sk + (size_t)x * Pp::SKB;
    const uint8_t *pki = ski + Pp::SKCPA;
    load_twiddles(S.tw, S.twi);
    // the ciphertext to shared memory in one coalesced pass: H(c), the decryption and the
    // comparison read it from there (the serial H(c) sponge then waits on no global load)
    for (int i = tid; i < Pp::CTB / 8; i += SINGLE_THREADS)
        reinterpret_cast<uint2 *>(S.buf)[i] = reinterpret_cast<const uint2 *>(ct + (size_t)x * Pp::CTB)[i];
    cti = S.buf;
    if (tid < 4) {
        S.seeds[16 + tid] = reinterpret_cast<const uint2 *>(pki + Pp::POLYVECBYTES)[tid];  // rho
        S.seeds[4 + tid] = reinterpret_cast<const uint2 *>(ski + Pp::SKB - 64)[tid];       // h = H(pk)
    }
    if (tid == 0) reinterpret_cast<uint32_t *>(S.seeds + 28)[0] = 0;
    __syncthreads();
    if (warp == 0) {
        uint2 h;
        if (kem == KEM_MLKEM)
            warp_absorb2<SHAKE256_LANES>(h, reinterpret_cast<const uint2 *>(ski + Pp::SKB - 32), 4,
                                         reinterpret_cast<const uint2 *>(cti), Pp::CTB / 8, DOM_SHAKE, w);
        else
            warp_absorb2<SHA3_256_LANES>(h, reinterpret_cast<const uint2 *>(cti), Pp::CTB / 8, nullptr, 0, DOM_SHA3, w);
        keccak_f1600_warp(h, w);
        if (lane < 4) S.seeds[24 + lane] = h;
    } else {
        const int rw = warp - 1;  // warps 1 .. SINGLE_WARPS - 1
        if (rw == 0) {
            // decryption by one warp: u' = decompress (slots [K, 2K)), u-hat = NTT, mp = s-hat^T u-hat,
            // v' = decompress (slot 2K), m' = tomsg(v' - invNTT(mp)) (indcpa.cu:690-733)
            for (int i = 0; i <= K; i++) {
                uint32_t t[8];
                int16_t c[8];
                if (i < K) {
                    unpack8<Pp::DU>(t, cti + (size_t)i * Pp::DU * 32 + (size_t)lane * Pp::DU);
#pragma unroll
                    for (int q = 0; q < 8; q++) c[q] = decompress_d<Pp::DU>(t[q]);
                } else {
                    unpack8<Pp::DV>(t, cti + Pp::CTU + (size_t)lane * Pp::DV);
#pragma unroll
                    for (int q = 0; q < 8; q++) c[q] = decompress_d<Pp::DV>(t[q]);
                }
                store8(S.poly(K + i) + phys(8 * lane), c);
                __syncwarp();
                if (i < K) ntt_warp(S.poly(K + i), S.tw, lane);
            }
            int32_t mp[8];
            warp_dot<K>(mp, nullptr, 0, ski, S.poly(K), S.tw, lane);
            store8(S.poly(0) + phys(8 * lane), mp);
            __syncwarp();
            invntt_warp(S.poly(0), S.twi, lane);
            int32_t v[8], m2[8];
            load8(v, S.poly(2 * K) + phys(8 * lane));
            load8(m2, S.poly(0) + phys(8 * lane));
            uint32_t byte = 0;
#pragma unroll
            for (int q = 0; q < 8; q++) byte |= compress_u<1>((uint32_t)csubq32(barrett_hi(v[q] - m2[q]))) << q;
            reinterpret_cast<uint8_t *>(S.seeds)[lane] = (uint8_t)byte;  // m'
            __syncwarp();
            uint2 g = lane < 8 ? S.seeds[lane] : make_uint2(0, 0);  // G(m' || h)
            if (lane == SHA3_512_LANES - 1) {
                g.x ^= DOM_SHA3;
                g.y ^= 0x80000000u;
            }
            keccak_f1600_warp(g, w);
            if (lane < 8) S.seeds[8 + lane] = g;  // lanes 0-3 K-bar', 4-7 r'
        } else {
            for (int e = rw - 1; e < K * K; e += SINGLE_WARPS - 2)
                warp_sample_entry<V>(S.seeds + 16, e / K, e % K, S.A + e * POLY_PITCH, w);
        }
        single_bar_rest();
        single_encrypt<K, V, true>(S, pki, cti, 1, SINGLE_WARPS - 1, [] { single_bar_rest(); });
    }
    __syncthreads();
    if (warp == 0) {
        const uint32_t mask = 0u - reinterpret_cast<const uint32_t *>(S.seeds + 28)[0];
        uint2 *o = reinterpret_cast<uint2 *>(ss + (size_t)x * 32);
        uint2 kk = lane < 4 ? S.seeds[8 + lane] : make_uint2(0, 0);
        if (kem == KEM_MLKEM) {  // ss = fail ? J(z || c) : K'
            const uint2 jj = lane < 4 ? S.seeds[24 + lane] : make_uint2(0, 0);
            if (lane < 4) o[lane] = make_uint2(kk.x ^ (mask & (kk.x ^ jj.x)), kk.y ^ (mask & (kk.y ^ jj.y)));
        } else {  // ss = KDF((fail ? z : K-bar') || H(c))
            const uint2 zk = lane < 4 ? reinterpret_cast<const uint2 *>(ski + Pp::SKB - 32)[lane] : make_uint2(0, 0);
            uint2 a = lane < 4 ? make_uint2(kk.x ^ (mask & (kk.x ^ zk.x)), kk.y ^ (mask & (kk.y ^ zk.y)))
                               : (lane < 8 ? S.seeds[24 + lane - 4] : make_uint2(0, 0));
            if (lane == 8) a.x ^= DOM_SHAKE;
            if (lane == SHAKE256_LANES - 1) a.y ^= 0x80000000u;
            keccak_f1600_warp(a, w);
            if (lane < 4) o[lane] = a;
        }
    }
}

// Keypair (KEM): (rho, sigma) = G(d) (ML-KEM: G(d || k)); s, e noise and the matrix entries
// A[i][j] = XOF(rho || j || i) on the warps at once; t-hat = A s-hat + e-hat; pk, sk; H(pk).
template <int K, int V>
__global__ void __launch_bounds__(SINGLE_THREADS) kyber_kp_single(const uint8_t *coins, int coins_stride, uint8_t *pk,
                                                                  uint8_t *sk, int kem) {
    using Pp = P<K, V>;
    constexpr int SP = SingleSmem<K, V>::PRFB;
    extern __shared__ __align__(16) uint8_t smem[];
    const SingleSmem<K, V> S(smem);
    const int x = blockIdx.x, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const WarpKeccak w(lane);
    const uint8_t *cn = coins + (size_t)x * coins_stride;
    uint8_t *pki = pk + (size_t)x * Pp::PKB, *ski = sk + (size_t)x * Pp::SKB;
    load_twiddles(S.tw, S.twi);
    if (warp == 0) {
        uint2 g = lane < 4 ? reinterpret_cast<const uint2 *>(cn)[lane] : make_uint2(0, 0);
        if (lane == 4) g.x = kem == KEM_MLKEM ? ((uint32_t)K | (DOM_SHA3 << 8)) : DOM_SHA3;
        if (lane == SHA3_512_LANES - 1) g.y ^= 0x80000000u;
        keccak_f1600_warp(g, w);
        if (lane < 8) S.seeds[16 + lane] = g;  // lanes 16-19 rho, 20-23 sigma
    }
    __syncthreads();
    // the 2K noise PRFs first (nonces 0 .. 2K-1: s then e), then the K*K matrix entries
    for (int t = warp; t < 2 * K + K * K; t += SINGLE_WARPS) {
        if (t < 2 * K) warp_prf<Pp::ETA1>(S.seeds + 20, t, S.prf + t * SP, w);
        else {
            const int e = t - 2 * K, i = e / K, j = e % K;
            warp_sample_entry<V>(S.seeds + 16, j, i, S.A + e * POLY_PITCH, w);
        }
    }
    __syncthreads();
    for (int t = warp; t < 2 * K; t += SINGLE_WARPS) {  // polys [0, K) s-hat, [K, 2K) e-hat
        warp_cbd<Pp::ETA1>(S.prf + t * SP, S.poly(t), lane);
        ntt_warp(S.poly(t), S.tw, lane);
    }
    __syncthreads();
    for (int i = warp; i < K; i += SINGLE_WARPS) {
        int32_t t[8], e[8], s[8];
        warp_dot<K>(t, S.A + i * K * POLY_PITCH, POLY_PITCH, nullptr, S.poly(0), S.tw, lane);
        load8(e, S.poly(K + i) + phys(8 * lane));
        load8(s, S.poly(i) + phys(8 * lane));
#pragma unroll
        for (int q = 0; q < 8; q++) {
            t[q] = csubq32(barrett_hi(t[q] + e[q]));
            s[q] = csubq32(s[q]);
        }
        uint8_t bt[12], bs[12];
        tobytes8(bt, t);
        tobytes8(bs, s);
        const int off = 384 * i + 12 * lane;
#pragma unroll
        for (int q = 0; q < 12; q++) {
            S.buf[off + q] = bt[q];
            ski[off + q] = bs[q];
        }
    }
    if (tid < 4) reinterpret_cast<uint2 *>(S.buf + Pp::POLYVECBYTES)[tid] = S.seeds[16 + tid];  // rho
    __syncthreads();
    for (int i = tid; i < Pp::PKB / 8; i += SINGLE_THREADS) {
        const uint2 v = reinterpret_cast<const uint2 *>(S.buf)[i];
        reinterpret_cast<uint2 *>(pki)[i] = v;
        reinterpret_cast<uint2 *>(ski + Pp::SKCPA)[i] = v;
    }
    if (warp == 1 && lane < 4)
        reinterpret_cast<uint2 *>(ski + Pp::SKB - 32)[lane] = reinterpret_cast<const uint2 *>(cn + 32)[lane];  // z
    if (warp == 0) {  // sk[SKB - 64, SKB - 32) = H(pk)
        uint2 h;
        warp_absorb2<SHA3_256_LANES>(h, reinterpret_cast<const uint2 *>(S.buf), Pp::PKB / 8, nullptr, 0, DOM_SHA3, w);
        keccak_f1600_warp(h, w);
        if (lane < 4) reinterpret_cast<uint2 *>(ski + Pp::SKB - 64)[lane] = h;
    }
}

}  // namespace kyber
}  // namespace pqc
