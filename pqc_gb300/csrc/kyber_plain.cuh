// Plain per-stage Kyber path: the baseline the fused kernels are measured against.
//
// Same decomposition as the reference's indcpa_keypair / indcpa_enc / indcpa_dec
// (Kyber_GPU_Batched/indcpa.cu:474-733): one kernel per stage, one thread per instance, every
// intermediate polynomial (the matrix A included) in HBM in the reference's coefficient-major
// structure-of-arrays layout (coefficient c of instance x at c * n + x, poly.h:12-22), plus the KEM
// hashing kernels shared with the fused path.  It uses this library's arithmetic and register
// Keccak, so the fused / plain ratio measures the fusion and batching, not a slower primitive.
// Included from kyber_impl.cuh.
#pragma once

namespace pqc {
namespace kyber {
namespace plain {
namespace {  // internal linkage: this header is compiled into one translation unit per (k, variant)

struct Soa {
    int16_t *p;
    int n;
    __device__ __forceinline__ int16_t &at(int c, int x) const { return p[(size_t)c * n + x]; }
    __host__ __device__ __forceinline__ Soa poly(int i) const { return Soa{p + (size_t)i * N * n, n}; }
};

// ---- per-thread polynomial stages on SoA memory (thread x owns column x) ----
__device__ __forceinline__ void ntt_soa(Soa r, int x) {
    int k = 1;
    for (int len = 128; len >= 2; len >>= 1)
        for (int start = 0; start < N; start += 2 * len) {
            const int16_t z = c_zetas[k++];
            for (int j = start; j < start + len; j++) {
                int16_t a = r.at(j, x), b = r.at(j + len, x);
                ct_bfly(a, b, z);
                r.at(j, x) = a;
                r.at(j + len, x) = b;
            }
        }
    for (int j = 0; j < N; j++) r.at(j, x) = barrett(r.at(j, x));
}
__device__ __forceinline__ void invntt_soa(Soa r, int x) {
    int k = 0;
    for (int len = 2; len <= 128; len <<= 1)
        for (int start = 0; start < N; start += 2 * len) {
            const int16_t z = c_zetas_inv[k++];
            for (int j = start; j < start + len; j++) {
                int16_t a = r.at(j, x), b = r.at(j + len, x);
                gs_bfly(a, b, z);
                r.at(j, x) = a;
                r.at(j + len, x) = b;
            }
        }
    for (int j = 0; j < N; j++) r.at(j, x) = fqmul(r.at(j, x), c_zetas_inv[127]);
}

template <int K>
__global__ void k_ntt(int n, Soa v, int npoly) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= n) return;
    for (int i = 0; i < npoly; i++) ntt_soa(v.poly(i), x);
}
template <int K>
__global__ void k_invntt(int n, Soa v, int npoly) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= n) return;
    for (int i = 0; i < npoly; i++) invntt_soa(v.poly(i), x);
}
// r = sum_j a_j o b_j, then Barrett (polyvec_pointwise_acc_n, polyvec.cu:161-177)
template <int K>
__global__ void k_pointwise_acc(int n, Soa r, Soa a, Soa b) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= n) return;
    for (int p = 0; p < N / 2; p++) {
        int16_t acc0 = 0, acc1 = 0;
        for (int j = 0; j < K; j++) {
            int16_t r0, r1;
            const Soa aj = a.poly(j), bj = b.poly(j);
            basemul(r0, r1, aj.at(2 * p, x), aj.at(2 * p + 1, x), bj.at(2 * p, x), bj.at(2 * p + 1, x),
                    (p & 1) ? (int16_t)-c_zetas[64 + (p >> 1)] : c_zetas[64 + (p >> 1)]);
            acc0 = (int16_t)(acc0 + r0);
            acc1 = (int16_t)(acc1 + r1);
        }
        r.at(2 * p, x) = barrett(acc0);
        r.at(2 * p + 1, x) = barrett(acc1);
    }
}
__global__ void k_frommont(int n, Soa r, int npoly) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= n) return;
    for (int i = 0; i < npoly; i++)
        for (int c = 0; c < N; c++) r.poly(i).at(c, x) = mont_reduce((int32_t)r.poly(i).at(c, x) * 1353);
}
// r = a + s * b for npoly polynomials (s = +1 add, -1 sub: r = a - b)
__global__ void k_addsub(int n, Soa r, Soa a, Soa b, int npoly, int sub) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= n) return;
    for (int i = 0; i < npoly; i++)
        for (int c = 0; c < N; c++) {
            const int16_t u = a.poly(i).at(c, x), v = b.poly(i).at(c, x);
            r.poly(i).at(c, x) = sub ? (int16_t)(u - v) : (int16_t)(u + v);
        }
}
__global__ void k_reduce(int n, Soa r, int npoly) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= n) return;
    for (int i = 0; i < npoly; i++)
        for (int c = 0; c < N; c++) r.poly(i).at(c, x) = barrett(r.poly(i).at(c, x));
}

// getnoise: one polynomial per launch, as the reference launches poly_getnoise per nonce
template <int ETA>
__global__ void k_getnoise(int n, Soa r, const uint8_t *seed, int seed_stride, int nonce) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= n) return;
    noise_poly<ETA>(reinterpret_cast<const uint2 *>(seed + (size_t)x * seed_stride), nonce,
                    [&](int g, const int16_t(&c)[8]) {
#pragma unroll
                        for (int q = 0; q < 8; q++) r.at(8 * g + q, x) = c[q];
                    });
}

// gen_matrix: all K*K entries by the instance's thread, written to HBM
template <int K, int V>
__global__ void k_gen_matrix(int n, Soa A, const uint8_t *rho, int rho_stride, int transposed) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= n) return;
    const uint2 *r = reinterpret_cast<const uint2 *>(rho + (size_t)x * rho_stride);
    for (int i = 0; i < K; i++)
        for (int j = 0; j < K; j++) {
            Soa e = A.poly(i * K + j);
            uint2 S[25];
            keccak_zero(S);
#pragma unroll
            for (int l = 0; l < 4; l++) S[l] = r[l];
            const uint32_t xx = transposed ? i : j, yy = transposed ? j : i;
            S[4].x = xx | (yy << 8) | (DOM_SHAKE << 16);
            S[SHAKE128_LANES - 1].y ^= 0x80000000u;
            int ctr = 0;
            auto take = [&](uint32_t d) {
                const uint32_t bound = (V == 2) ? (uint32_t)(19 * Q) : (uint32_t)Q;
                if (d < bound && ctr < N) e.at(ctr++, x) = (V == 2) ? (int16_t)(d - (d >> 12) * Q) : (int16_t)d;
            };
            while (ctr < N) {
                keccak_f1600(S);
                if (V == 3) {
#pragma unroll
                    for (int t = 0; t < 56; t++) {
                        const int o = 3 * t, wi = o >> 2, sh = 8 * (o & 3);
                        const uint32_t w0 = (wi & 1) ? S[wi >> 1].y : S[wi >> 1].x;
                        uint32_t v;
                        if (sh <= 8) {
                            v = w0 >> sh;
                        } else {
                            const uint32_t w1 = ((wi + 1) & 1) ? S[(wi + 1) >> 1].y : S[(wi + 1) >> 1].x;
                            v = __funnelshift_r(w0, w1, sh);
                        }
                        take(v & 0xfff);
                        take((v >> 12) & 0xfff);
                    }
                } else {
#pragma unroll
                    for (int t = 0; t < 42; t++) {
                        const uint32_t w0 = (t & 1) ? S[t >> 1].y : S[t >> 1].x;
                        take(w0 & 0xffff);
                        take(w0 >> 16);
                    }
                }
            }
        }
}

// ---- codecs (thread per instance) ----
template <int K>
__global__ void k_frombytes(int n, Soa r, const uint8_t *src, int stride, int npoly) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= n) return;
    const uint8_t *b = src + (size_t)x * stride;
    for (int i = 0; i < npoly; i++)
        for (int g = 0; g < 32; g++) {
            int16_t c[8];
            frombytes8(c, b + 384 * i + 12 * g);
#pragma unroll
            for (int q = 0; q < 8; q++) r.poly(i).at(8 * g + q, x) = c[q];
        }
}
template <int K>
__global__ void k_tobytes(int n, uint8_t *dst, int stride, Soa r, int npoly) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= n) return;
    uint8_t *b = dst + (size_t)x * stride;
    for (int i = 0; i < npoly; i++)
        for (int g = 0; g < 32; g++) {
            int16_t c[8];
#pragma unroll
            for (int q = 0; q < 8; q++) c[q] = csubq(r.poly(i).at(8 * g + q, x));
            uint8_t o[12];
            tobytes8(o, c);
#pragma unroll
            for (int q = 0; q < 12; q++) b[384 * i + 12 * g + q] = o[q];
        }
}
__global__ void k_frommsg(int n, Soa r, const uint8_t *m, int stride) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= n) return;
    for (int i = 0; i < 32; i++) {
        const uint8_t b = m[(size_t)x * stride + i];
        for (int j = 0; j < 8; j++) r.at(8 * i + j, x) = ((b >> j) & 1) ? (int16_t)((Q + 1) / 2) : (int16_t)0;
    }
}
__global__ void k_tomsg(int n, uint8_t *m, int stride, Soa r) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= n) return;
    for (int i = 0; i < 32; i++) {
        uint32_t byte = 0;
        for (int j = 0; j < 8; j++) {
            const int16_t v = csubq(r.at(8 * i + j, x));
            byte |= (((((uint32_t)v << 1) + Q / 2) / Q) & 1) << j;
        }
        m[(size_t)x * stride + i] = (uint8_t)byte;
    }
}
// pack_ciphertext (compress du / dv); with cmp != nullptr compare instead and write fail flags
template <int K, int V>
__global__ void k_pack_ct(int n, uint8_t *ct, const uint8_t *cmp, uint8_t *fail, Soa u, Soa v) {
    using Pp = P<K, V>;
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= n) return;
    uint32_t diff = 0;
    for (int i = 0; i <= K; i++) {
        const Soa p = (i < K) ? u.poly(i) : v;
        for (int g = 0; g < 32; g++) {
            uint32_t t[8];
            for (int q = 0; q < 8; q++) {
                const int16_t c = csubq(p.at(8 * g + q, x));
                t[q] = (i < K) ? compress_d<Pp::DU>(c) : compress_d<Pp::DV>(c);
            }
            if (i < K) {
                uint8_t b[Pp::DU];
                pack8<Pp::DU>(b, t);
                const size_t off = (size_t)x * Pp::CTB + (size_t)i * Pp::DU * 32 + (size_t)g * Pp::DU;
                for (int q = 0; q < Pp::DU; q++) {
                    if (cmp) diff |= b[q] ^ cmp[off + q];
                    else ct[off + q] = b[q];
                }
            } else {
                uint8_t b[Pp::DV];
                pack8<Pp::DV>(b, t);
                const size_t off = (size_t)x * Pp::CTB + Pp::CTU + (size_t)g * Pp::DV;
                for (int q = 0; q < Pp::DV; q++) {
                    if (cmp) diff |= b[q] ^ cmp[off + q];
                    else ct[off + q] = b[q];
                }
            }
        }
    }
    if (cmp) fail[x] = diff ? 1 : 0;
}
template <int K, int V>
__global__ void k_unpack_ct(int n, Soa u, Soa v, const uint8_t *ct) {
    using Pp = P<K, V>;
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= n) return;
    const uint8_t *c = ct + (size_t)x * Pp::CTB;
    for (int i = 0; i <= K; i++)
        for (int g = 0; g < 32; g++) {
            uint32_t t[8];
            if (i < K) {
                unpack8<Pp::DU>(t, c + (size_t)i * Pp::DU * 32 + (size_t)g * Pp::DU);
                for (int q = 0; q < 8; q++) u.poly(i).at(8 * g + q, x) = decompress_d<Pp::DU>(t[q]);
            } else {
                unpack8<Pp::DV>(t, c + Pp::CTU + (size_t)g * Pp::DV);
                for (int q = 0; q < 8; q++) v.at(8 * g + q, x) = decompress_d<Pp::DV>(t[q]);
            }
        }
}

// G(m || h) for decapsulation: seeds[x] = m' || r' || K-bar' (96 B, the encaps scratch layout)
template <int K, int V>
__global__ void k_dec_g(int n, uint8_t *seeds, const uint8_t *sk) {
    using Pp = P<K, V>;
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= n) return;
    uint2 A[25];
    keccak_zero(A);
    const uint2 *m = reinterpret_cast<const uint2 *>(seeds + (size_t)x * 96);
    const uint2 *h = reinterpret_cast<const uint2 *>(sk + (size_t)x * Pp::SKB + Pp::SKB - 64);
#pragma unroll
    for (int i = 0; i < 4; i++) {
        A[i] = m[i];
        A[4 + i] = h[i];
    }
    A[8].x ^= DOM_SHA3;
    A[SHA3_512_LANES - 1].y ^= 0x80000000u;
    keccak_f1600(A);
    uint2 *o = reinterpret_cast<uint2 *>(seeds + (size_t)x * 96);
#pragma unroll
    for (int i = 0; i < 4; i++) {
        o[4 + i] = A[4 + i];  // r'
        o[8 + i] = A[i];      // K-bar'
    }
}
// ss = KDF(fail ? z : K-bar' || H(c))
template <int K, int V>
__global__ void k_dec_kdf(int n, uint8_t *ss, const uint8_t *seeds, const uint8_t *fail, const uint8_t *hct,
                          const uint8_t *sk) {
    using Pp = P<K, V>;
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= n) return;
    const uint32_t mask = 0u - (uint32_t)(fail[x] != 0);
    const uint2 *kb = reinterpret_cast<const uint2 *>(seeds + (size_t)x * 96 + 64);
    const uint2 *z = reinterpret_cast<const uint2 *>(sk + (size_t)x * Pp::SKB + Pp::SKB - 32);
    const uint2 *hc = reinterpret_cast<const uint2 *>(hct + (size_t)x * 32);
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
    keccak_f1600(A);
    uint2 *o = reinterpret_cast<uint2 *>(ss + (size_t)x * 32);
#pragma unroll
    for (int i = 0; i < 4; i++) o[i] = A[i];
}
// keypair: (rho, sigma) = G(d) -> seeds (64 B per instance)
__global__ void k_kp_g(int n, uint8_t *seeds, const uint8_t *coins, int stride) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= n) return;
    uint2 A[25];
    keccak_zero(A);
    const uint2 *d = reinterpret_cast<const uint2 *>(coins + (size_t)x * stride);
#pragma unroll
    for (int i = 0; i < 4; i++) A[i] = d[i];
    A[4].x ^= DOM_SHA3;
    A[SHA3_512_LANES - 1].y ^= 0x80000000u;
    keccak_f1600(A);
    uint2 *o = reinterpret_cast<uint2 *>(seeds + (size_t)x * 64);
#pragma unroll
    for (int i = 0; i < 8; i++) o[i] = A[i];
}
// keypair: pk tail rho, sk = sk_cpa || pk || . || z
template <int K, int V>
__global__ void k_kp_finish(int n, uint8_t *pk, uint8_t *sk, const uint8_t *seeds, const uint8_t *coins, int stride) {
    using Pp = P<K, V>;
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= n) return;
    for (int i = 0; i < 32; i++) pk[(size_t)x * Pp::PKB + Pp::POLYVECBYTES + i] = seeds[(size_t)x * 64 + i];
    for (int i = 0; i < Pp::PKB; i++) sk[(size_t)x * Pp::SKB + Pp::SKCPA + i] = pk[(size_t)x * Pp::PKB + i];
    for (int i = 0; i < 32; i++) sk[(size_t)x * Pp::SKB + Pp::SKB - 32 + i] = coins[(size_t)x * stride + 32 + i];
}

// Scratch (bytes per instance) the plain path needs from the arena.
template <int K>
constexpr size_t scratch_per_instance() {
    return (size_t)(K * K + 4 * K + 4) * N * 2 + 96 + 64 + 32 + 16;
}

}  // namespace
}  // namespace plain

// ---- plain host sequences (every stage one launch, as in indcpa.cu) ----
#define PL(name, kern, ...) PQC_LAUNCH(st, "plain_" name, K, V, kern<<<g, TPB, 0, st>>>(__VA_ARGS__))

template <int K, int V>
static int plain_encrypt(int n, uint8_t *scratch, const uint8_t *pk, int pk_stride, const uint8_t *seeds,
                         uint8_t *ct, const uint8_t *cmp, uint8_t *fail, cudaStream_t st) {
    using namespace plain;
    using Pp = P<K, V>;
    const int TPB = 128, g = (n + TPB - 1) / TPB;
    int16_t *base = reinterpret_cast<int16_t *>(scratch);
    Soa At{base, n}, sp{base + (size_t)K * K * N * n, n}, ep = sp.poly(K), bp = sp.poly(2 * K),
        pkpv = sp.poly(3 * K), v = sp.poly(4 * K), epp = sp.poly(4 * K + 1), kp = sp.poly(4 * K + 2);
    (void)pk_stride;
    // unpack_pk + frommsg + gen_matrix(transposed) + getnoise x (2K+1)
    PL("frombytes", k_frombytes<K>, n, pkpv, pk, pk_stride, K);
    PL("frommsg", k_frommsg, n, kp, seeds, 96);
    auto gm = k_gen_matrix<K, V>;
    PL("gen_matrix", gm, n, At, pk + Pp::POLYVECBYTES, pk_stride, 1);
    for (int i = 0; i < K; i++) PL("getnoise", k_getnoise<Pp::ETA1>, n, sp.poly(i), seeds + 32, 96, i);
    for (int i = 0; i < K; i++) PL("getnoise", k_getnoise<Pp::ETA2>, n, ep.poly(i), seeds + 32, 96, K + i);
    PL("getnoise", k_getnoise<Pp::ETA2>, n, epp, seeds + 32, 96, 2 * K);
    PL("ntt", k_ntt<K>, n, sp, K);
    for (int i = 0; i < K; i++) PL("pointwise_acc", k_pointwise_acc<K>, n, bp.poly(i), At.poly(i * K), sp);
    PL("pointwise_acc", k_pointwise_acc<K>, n, v, pkpv, sp);
    PL("invntt", k_invntt<K>, n, bp, K);
    PL("invntt", k_invntt<K>, n, v, 1);
    PL("add", k_addsub, n, bp, bp, ep, K, 0);
    PL("add", k_addsub, n, v, v, epp, 1, 0);
    PL("add", k_addsub, n, v, v, kp, 1, 0);
    PL("reduce", k_reduce, n, bp, K);
    PL("reduce", k_reduce, n, v, 1);
    auto pc = k_pack_ct<K, V>;
    PL("pack_ct", pc, n, ct, cmp, fail, bp, v);
    return cudaGetLastError() == cudaSuccess ? PQCGPU_OK : PQCGPU_ECUDA;
}

template <int K, int V>
static int plain_enc(int n, uint8_t *ct, uint8_t *ss, const uint8_t *pk, const uint8_t *coins, uint8_t *scratch,
                     cudaStream_t st) {
    using Pp = P<K, V>;
    const int TPB = 128, g = (n + TPB - 1) / TPB;
    uint8_t *seeds = scratch + plain::scratch_per_instance<K>() * n - (size_t)(96 + 64 + 32 + 16) * n;
    PQC_LAUNCH(st, "plain_enc_hash_pre", K, V, kyber_enc_hash_pre<K, V><<<g, TPB, 0, st>>>(n, pk, coins, seeds, KEM_FO));
    const int rc = plain_encrypt<K, V>(n, scratch, pk, Pp::PKB, seeds, ct, nullptr, nullptr, st);
    if (rc) return rc;
    PQC_LAUNCH(st, "plain_enc_hash_post", K, V, kyber_enc_hash_post<K, V><<<g, TPB, 0, st>>>(n, ct, seeds, ss, KEM_FO));
    return cudaGetLastError() == cudaSuccess ? PQCGPU_OK : PQCGPU_ECUDA;
}

template <int K, int V>
static int plain_dec(int n, uint8_t *ss, const uint8_t *ct, const uint8_t *sk, uint8_t *scratch, cudaStream_t st) {
    using namespace plain;
    using Pp = P<K, V>;
    const int TPB = 128, g = (n + TPB - 1) / TPB;
    uint8_t *tail = scratch + scratch_per_instance<K>() * n - (size_t)(96 + 64 + 32 + 16) * n;
    uint8_t *seeds = tail, *hct = tail + (size_t)160 * n, *fail = tail + (size_t)192 * n;
    int16_t *base = reinterpret_cast<int16_t *>(scratch);
    Soa bp{base, n}, skpv = bp.poly(K), v = bp.poly(2 * K), mp = bp.poly(2 * K + 1);
    PQC_LAUNCH(st, "plain_dec_hash_pre", K, V, kyber_dec_hash_pre<K, V><<<g, TPB, 0, st>>>(n, ct, sk, hct, KEM_FO));
    auto uc = k_unpack_ct<K, V>;
    PL("unpack_ct", uc, n, bp, v, ct);
    PL("frombytes", k_frombytes<K>, n, skpv, sk, Pp::SKB, K);
    PL("ntt", k_ntt<K>, n, bp, K);
    PL("pointwise_acc", k_pointwise_acc<K>, n, mp, skpv, bp);
    PL("invntt", k_invntt<K>, n, mp, 1);
    PL("sub", k_addsub, n, mp, v, mp, 1, 1);
    PL("reduce", k_reduce, n, mp, 1);
    PL("tomsg", k_tomsg, n, seeds, 96, mp);
    auto dg = k_dec_g<K, V>;
    PL("dec_g", dg, n, seeds, sk);
    int rc = plain_encrypt<K, V>(n, scratch, sk + Pp::SKCPA, Pp::SKB, seeds, nullptr, ct, fail, st);
    if (rc) return rc;
    auto dk = k_dec_kdf<K, V>;
    PL("dec_kdf", dk, n, ss, seeds, fail, hct, sk);
    return cudaGetLastError() == cudaSuccess ? PQCGPU_OK : PQCGPU_ECUDA;
}

template <int K, int V>
static int plain_keypair(int n, uint8_t *pk, uint8_t *sk, const uint8_t *coins, int coins_stride, uint8_t *scratch,
                         cudaStream_t st) {
    using namespace plain;
    using Pp = P<K, V>;
    const int TPB = 128, g = (n + TPB - 1) / TPB;
    uint8_t *seeds = scratch + scratch_per_instance<K>() * n - (size_t)(96 + 64 + 32 + 16) * n;
    int16_t *base = reinterpret_cast<int16_t *>(scratch);
    Soa A{base, n}, s{base + (size_t)K * K * N * n, n}, e = s.poly(K), t = s.poly(2 * K);
    PL("kp_g", k_kp_g, n, seeds, coins, coins_stride);
    auto gm = k_gen_matrix<K, V>;
    PL("gen_matrix", gm, n, A, seeds, 64, 0);
    for (int i = 0; i < K; i++) PL("getnoise", k_getnoise<Pp::ETA1>, n, s.poly(i), seeds + 32, 64, i);
    for (int i = 0; i < K; i++) PL("getnoise", k_getnoise<Pp::ETA1>, n, e.poly(i), seeds + 32, 64, K + i);
    PL("ntt", k_ntt<K>, n, s, K);
    PL("ntt", k_ntt<K>, n, e, K);
    for (int i = 0; i < K; i++) {
        PL("pointwise_acc", k_pointwise_acc<K>, n, t.poly(i), A.poly(i * K), s);
        PL("frommont", k_frommont, n, t.poly(i), 1);
    }
    PL("add", k_addsub, n, t, t, e, K, 0);
    PL("reduce", k_reduce, n, t, K);
    PL("tobytes", k_tobytes<K>, n, sk, Pp::SKB, s, K);
    PL("tobytes", k_tobytes<K>, n, pk, Pp::PKB, t, K);
    auto kf = k_kp_finish<K, V>;
    PL("kp_finish", kf, n, pk, sk, seeds, coins, coins_stride);
    PQC_LAUNCH(st, "plain_kp_hash_post", K, V, kyber_kp_hash_post<K, V><<<g, TPB, 0, st>>>(n, pk, sk));
    return cudaGetLastError() == cudaSuccess ? PQCGPU_OK : PQCGPU_ECUDA;
}
#undef PL

}  // namespace kyber
}  // namespace pqc
