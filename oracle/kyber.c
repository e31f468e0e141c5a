/*
 * Kyber CPA-PKE and KEM restated in plain C -- TEST INFRASTRUCTURE (CPU oracle), never shipped.
 *
 * Arithmetic follows the reference exactly, so every intermediate value (not only the result
 * mod q) is the one the reference computes:
 *   montgomery_reduce / barrett_reduce / csubq   Kyber_GPU_Batched/reduce.cu:21-66
 *   zetas / zetas_inv (generated here from 17, MONT = 2^16 mod q, the bit-reversal tree)
 *                                                Kyber_GPU_Batched/ntt.cu:8-68 (generation recipe)
 *   forward / inverse NTT, basemul               Kyber_GPU_Batched/ntt.cu:152-259
 *   poly_basemul, pointwise_acc + reduce         Kyber_GPU_Batched/poly.cu:204-225, polyvec.cu:161-177
 *   frommont (x 2^32 mod q, Montgomery)          Kyber_GPU_Batched/poly.cu:235-247
 *   cbd (eta = 2)                                Kyber_GPU_Batched/cbd.cu:42-63
 *   rej_uniform 16-bit / 19q, gen_matrix         Kyber_GPU_Batched/indcpa.cu:290-403
 *   codecs, compress du=11 / dv=5, msg           Kyber_GPU_Batched/poly.cu:22-116, :367-417,
 *                                                polyvec.cu:18-82
 *   CPA orchestration                            Kyber_GPU_Batched/indcpa.cu:474-733, with the seed
 *                                                plumbing of the NIST flow ((rho, sigma) = G(d) per
 *                                                instance; the reference's in-place race at
 *                                                indcpa.cu:500 is not reproduced).
 * Round-3 additions restated from the Kyber round-3 specification: 12-bit rejection sampling,
 * CBD eta = 3, compress du = 10 / dv = 4, parameter sets k = 2/3/4.
 * KEM: the Fujisaki-Okamoto transform of the Kyber submission (keypair sk = sk_cpa||pk||H(pk)||z;
 * encaps m = H(coins), (K, r) = G(m||H(pk)), ss = SHAKE256(K||H(c)); decaps re-encrypts and
 * substitutes z on mismatch).  The reference declares these entry points (Kyber_GPU_Batched/
 * api.h:18-22) but its kem.cu is absent from the tree.
 */
#include <string.h>
#include "oracle.h"

#define KN 256
#define KQ 3329
#define KQINV 62209 /* q^-1 mod 2^16 */
#define KMONT 2285  /* 2^16 mod q */

extern _Thread_local uint64_t oracle_g_butterfly_count;

typedef struct {
    int16_t c[KN];
} kpoly;

typedef struct {
    int variant, k, eta1, eta2, du, dv;
    size_t polyvecbytes, polycomp, polyveccomp, pk, skcpa, sk, ct;
} kparams;

static int16_t zetas[128], zetas_inv[128];

static int brv7(int x) {
    int r = 0;
    for (int i = 0; i < 7; i++) r |= ((x >> i) & 1) << (6 - i);
    return r;
}

static int modq(long v) {
    long r = v % KQ;
    return (int)(r < 0 ? r + KQ : r);
}

__attribute__((constructor)) static void kyber_tables_init(void) {
    long pw[129];
    pw[0] = 1;
    for (int i = 1; i <= 128; i++) pw[i] = (pw[i - 1] * 17) % KQ;
    for (int i = 0; i < 128; i++) zetas[i] = (int16_t)modq((long)KMONT * pw[brv7(i)]);
    int k = 0;
    for (int i = 64; i >= 1; i >>= 1)
        for (int j = i; j < 2 * i; j++) zetas_inv[k++] = (int16_t)modq(-(long)KMONT * pw[128 - brv7(j)]);
    zetas_inv[127] = (int16_t)((KMONT * ((KMONT * (KQ - 1) * ((KQ - 1) / 128)) % KQ)) % KQ);
}

static int kparams_get(int variant, int k, kparams *p) {
    if (k < 2 || k > 4) return -1;
    p->variant = variant;
    p->k = k;
    if (variant == 2) {
        p->eta1 = p->eta2 = 2;
        p->du = 11;
        p->dv = 5;
    } else if (variant == 3) {
        p->eta1 = (k == 2) ? 3 : 2;
        p->eta2 = 2;
        p->du = (k == 4) ? 11 : 10;
        p->dv = (k == 4) ? 5 : 4;
    } else {
        return -1;
    }
    p->polyvecbytes = (size_t)k * 384;
    p->polycomp = (size_t)p->dv * 32;
    p->polyveccomp = (size_t)k * p->du * 32;
    p->pk = p->polyvecbytes + 32;
    p->skcpa = p->polyvecbytes;
    p->sk = p->skcpa + p->pk + 64;
    p->ct = p->polyveccomp + p->polycomp;
    return 0;
}

int oracle_kyber_sizes(int variant, int k, size_t *pk, size_t *sk_cpa, size_t *sk, size_t *ct) {
    kparams p;
    if (kparams_get(variant, k, &p)) return -1;
    if (pk) *pk = p.pk;
    if (sk_cpa) *sk_cpa = p.skcpa;
    if (sk) *sk = p.sk;
    if (ct) *ct = p.ct;
    return 0;
}

/* ---- reductions (reduce.cu:21-66) ---- */
static int16_t mont_reduce(int32_t a) {
    int16_t u = (int16_t)(uint16_t)((uint32_t)a * (uint32_t)KQINV);
    int32_t t = (int32_t)u * KQ;
    t = a - t;
    return (int16_t)(t >> 16);
}
static int16_t barrett(int16_t a) {
    const int32_t v = (1 << 26) / KQ + 1;
    int32_t t = v * a;
    t >>= 26;
    t *= KQ;
    return (int16_t)(a - t);
}
static int16_t csubq(int16_t a) {
    a = (int16_t)(a - KQ);
    a = (int16_t)(a + ((a >> 15) & KQ));
    return a;
}
static int16_t fqmul(int16_t a, int16_t b) { return mont_reduce((int32_t)a * b); }

/* ---- NTT (ntt.cu:152-224) ---- */
static void ntt(int16_t r[KN]) {
    unsigned k = 1;
    for (unsigned len = 128; len >= 2; len >>= 1) {
        for (unsigned start = 0; start < KN; start += 2 * len) {
            int16_t zeta = zetas[k++];
            for (unsigned j = start; j < start + len; j++) {
                int16_t t = fqmul(zeta, r[j + len]);
                r[j + len] = (int16_t)(r[j] - t);
                r[j] = (int16_t)(r[j] + t);
                oracle_g_butterfly_count++;
            }
        }
    }
}
static void invntt(int16_t r[KN]) {
    unsigned k = 0;
    for (unsigned len = 2; len <= 128; len <<= 1) {
        for (unsigned start = 0; start < KN; start += 2 * len) {
            int16_t zeta = zetas_inv[k++];
            for (unsigned j = start; j < start + len; j++) {
                int16_t t = r[j];
                r[j] = barrett((int16_t)(t + r[j + len]));
                r[j + len] = (int16_t)(t - r[j + len]);
                r[j + len] = fqmul(zeta, r[j + len]);
                oracle_g_butterfly_count++;
            }
        }
    }
    for (unsigned j = 0; j < KN; j++) r[j] = fqmul(r[j], zetas_inv[127]);
}

static void poly_reduce(kpoly *r) {
    for (int i = 0; i < KN; i++) r->c[i] = barrett(r->c[i]);
}
static void poly_csubq(kpoly *r) {
    for (int i = 0; i < KN; i++) r->c[i] = csubq(r->c[i]);
}
static void poly_ntt(kpoly *r) {
    ntt(r->c);
    poly_reduce(r);
}

static void basemul(int16_t r[2], const int16_t a[2], const int16_t b[2], int16_t zeta) {
    r[0] = fqmul(a[1], b[1]);
    r[0] = fqmul(r[0], zeta);
    r[0] = (int16_t)(r[0] + fqmul(a[0], b[0]));
    r[1] = fqmul(a[0], b[1]);
    r[1] = (int16_t)(r[1] + fqmul(a[1], b[0]));
}
static void poly_basemul(kpoly *r, const kpoly *a, const kpoly *b) {
    for (int i = 0; i < KN / 4; i++) {
        basemul(r->c + 4 * i, a->c + 4 * i, b->c + 4 * i, zetas[64 + i]);
        basemul(r->c + 4 * i + 2, a->c + 4 * i + 2, b->c + 4 * i + 2, (int16_t)-zetas[64 + i]);
    }
}
static void pointwise_acc(kpoly *r, const kpoly *a, const kpoly *b, int k) {
    kpoly t;
    poly_basemul(r, &a[0], &b[0]);
    for (int i = 1; i < k; i++) {
        poly_basemul(&t, &a[i], &b[i]);
        for (int j = 0; j < KN; j++) r->c[j] = (int16_t)(r->c[j] + t.c[j]);
    }
    poly_reduce(r);
}
static void poly_frommont(kpoly *r) {
    const int16_t f = (int16_t)((1ULL << 32) % KQ);
    for (int i = 0; i < KN; i++) r->c[i] = mont_reduce((int32_t)r->c[i] * f);
}

/* ---- codecs ---- */
static void poly_tobytes(uint8_t *r, kpoly *a) {
    poly_csubq(a);
    for (int i = 0; i < KN / 2; i++) {
        uint16_t t0 = (uint16_t)a->c[2 * i], t1 = (uint16_t)a->c[2 * i + 1];
        r[3 * i] = (uint8_t)t0;
        r[3 * i + 1] = (uint8_t)((t0 >> 8) | ((t1 & 0xf) << 4));
        r[3 * i + 2] = (uint8_t)(t1 >> 4);
    }
}
static void poly_frombytes(kpoly *r, const uint8_t *a) {
    for (int i = 0; i < KN / 2; i++) {
        r->c[2 * i] = (int16_t)(a[3 * i] | ((uint16_t)a[3 * i + 1] & 0x0f) << 8);
        r->c[2 * i + 1] = (int16_t)(a[3 * i + 1] >> 4 | ((uint16_t)a[3 * i + 2]) << 4);
    }
}
/* compress to d bits: round(2^d x / q) mod 2^d on canonical x; little-endian bit packing */
static uint32_t compress_coeff(int16_t x, int d) {
    return (uint32_t)(((((uint32_t)(uint16_t)x << d) + KQ / 2) / KQ) & ((1u << d) - 1));
}
static int16_t decompress_coeff(uint32_t t, int d) { return (int16_t)((t * KQ + (1u << (d - 1))) >> d); }

static void pack_bits(uint8_t *out, const uint32_t *v, int n, int d) {
    /* LSB-first packing of n d-bit values: identical byte layout to the unrolled packers in
     * poly.cu:22-43 (d = 5), polyvec.cu:18-50 (d = 11) and the round-3 d = 4 / 10 packers. */
    memset(out, 0, (size_t)n * d / 8);
    int bit = 0;
    for (int i = 0; i < n; i++)
        for (int b = 0; b < d; b++, bit++)
            if ((v[i] >> b) & 1) out[bit >> 3] |= (uint8_t)(1u << (bit & 7));
}
static void unpack_bits(uint32_t *v, const uint8_t *in, int n, int d) {
    int bit = 0;
    for (int i = 0; i < n; i++) {
        uint32_t t = 0;
        for (int b = 0; b < d; b++, bit++) t |= (uint32_t)((in[bit >> 3] >> (bit & 7)) & 1) << b;
        v[i] = t;
    }
}
static void poly_compress(uint8_t *r, kpoly *a, int d) {
    uint32_t t[KN];
    poly_csubq(a);
    for (int i = 0; i < KN; i++) t[i] = compress_coeff(a->c[i], d);
    pack_bits(r, t, KN, d);
}
static void poly_decompress(kpoly *r, const uint8_t *a, int d) {
    uint32_t t[KN];
    unpack_bits(t, a, KN, d);
    for (int i = 0; i < KN; i++) r->c[i] = decompress_coeff(t[i], d);
}
static void poly_frommsg(kpoly *r, const uint8_t msg[32]) {
    for (int i = 0; i < 32; i++)
        for (int j = 0; j < 8; j++) {
            int16_t mask = (int16_t)-((msg[i] >> j) & 1);
            r->c[8 * i + j] = (int16_t)(mask & ((KQ + 1) / 2));
        }
}
static void poly_tomsg(uint8_t msg[32], kpoly *a) {
    poly_csubq(a);
    for (int i = 0; i < 32; i++) {
        msg[i] = 0;
        for (int j = 0; j < 8; j++) {
            uint16_t t = (uint16_t)((((a->c[8 * i + j] << 1) + KQ / 2) / KQ) & 1);
            msg[i] |= (uint8_t)(t << j);
        }
    }
}

/* ---- sampling ---- */
static void cbd(kpoly *r, const uint8_t *buf, int eta) {
    if (eta == 2) {
        for (int i = 0; i < KN / 8; i++) {
            uint32_t t = (uint32_t)buf[4 * i] | (uint32_t)buf[4 * i + 1] << 8 | (uint32_t)buf[4 * i + 2] << 16 |
                         (uint32_t)buf[4 * i + 3] << 24;
            uint32_t d = t & 0x55555555u;
            d += (t >> 1) & 0x55555555u;
            for (int j = 0; j < 8; j++) {
                int16_t a = (int16_t)((d >> (4 * j)) & 3), b = (int16_t)((d >> (4 * j + 2)) & 3);
                r->c[8 * i + j] = (int16_t)(a - b);
            }
        }
    } else { /* eta = 3 */
        for (int i = 0; i < KN / 4; i++) {
            uint32_t t = (uint32_t)buf[3 * i] | (uint32_t)buf[3 * i + 1] << 8 | (uint32_t)buf[3 * i + 2] << 16;
            uint32_t d = t & 0x00249249u;
            d += (t >> 1) & 0x00249249u;
            d += (t >> 2) & 0x00249249u;
            for (int j = 0; j < 4; j++) {
                int16_t a = (int16_t)((d >> (6 * j)) & 7), b = (int16_t)((d >> (6 * j + 3)) & 7);
                r->c[4 * i + j] = (int16_t)(a - b);
            }
        }
    }
}
static void getnoise(kpoly *r, const uint8_t seed[32], uint8_t nonce, int eta) {
    uint8_t ext[33], buf[3 * KN / 4];
    memcpy(ext, seed, 32);
    ext[32] = nonce;
    oracle_shake256(buf, (size_t)eta * KN / 4, ext, 33);
    cbd(r, buf, eta);
}

/* incremental SHAKE128 used for the matrix XOF: absorb once, squeeze 168-byte blocks */
typedef struct {
    uint64_t s[25];
} xof_t;
static void xof_absorb(xof_t *x, const uint8_t *in, size_t inlen) {
    uint8_t blk[168];
    memset(x->s, 0, sizeof x->s);
    memset(blk, 0, sizeof blk);
    memcpy(blk, in, inlen); /* inlen < 168 */
    blk[inlen] ^= 0x1F;
    blk[167] ^= 0x80;
    for (int i = 0; i < 21; i++) {
        uint64_t w = 0;
        for (int b = 0; b < 8; b++) w |= (uint64_t)blk[8 * i + b] << (8 * b);
        x->s[i] ^= w;
    }
}
static void xof_squeeze(xof_t *x, uint8_t out[168]) {
    oracle_keccakf1600(x->s);
    for (int i = 0; i < 168; i++) out[i] = (uint8_t)(x->s[i / 8] >> (8 * (i % 8)));
}

/* A[i][j] = Parse(XOF(rho || j || i)); transposed swaps the two index bytes (indcpa.cu:339-403). */
static void gen_matrix(kpoly *a, const uint8_t rho[32], int transposed, const kparams *p) {
    int k = p->k;
    for (int i = 0; i < k; i++)
        for (int j = 0; j < k; j++) {
            uint8_t ext[34], buf[168];
            xof_t x;
            memcpy(ext, rho, 32);
            ext[32] = (uint8_t)(transposed ? i : j);
            ext[33] = (uint8_t)(transposed ? j : i);
            xof_absorb(&x, ext, 34);
            kpoly *r = &a[i * k + j];
            int ctr = 0;
            while (ctr < KN) {
                xof_squeeze(&x, buf);
                if (p->variant == 2) {
                    for (int pos = 0; pos + 2 <= 168 && ctr < KN; pos += 2) {
                        uint16_t val = (uint16_t)(buf[pos] | ((uint16_t)buf[pos + 1] << 8));
                        if (val < 19 * KQ) {
                            val = (uint16_t)(val - (val >> 12) * KQ);
                            r->c[ctr++] = (int16_t)val;
                        }
                    }
                } else {
                    for (int pos = 0; pos + 3 <= 168 && ctr < KN; pos += 3) {
                        uint16_t v0 = (uint16_t)(((buf[pos] >> 0) | ((uint16_t)buf[pos + 1] << 8)) & 0xFFF);
                        uint16_t v1 = (uint16_t)(((buf[pos + 1] >> 4) | ((uint16_t)buf[pos + 2] << 4)) & 0xFFF);
                        if (v0 < KQ) r->c[ctr++] = (int16_t)v0;
                        if (ctr < KN && v1 < KQ) r->c[ctr++] = (int16_t)v1;
                    }
                }
            }
        }
}

/* ---- CPA-PKE ---- */
/* (rho, sigma) = G(d) for Kyber (indcpa.cu:495-500); ML-KEM (FIPS 203, K-PKE.KeyGen) hashes
 * d || k, the module rank as one byte, for domain separation between parameter sets. */
static void cpa_keypair_g(const kparams *p, uint8_t *pk, uint8_t *sk, const uint8_t d[32], int mlkem) {
    int k = p->k;
    uint8_t buf[64], din[33];
    kpoly a[16], s[4], e[4], t[4];
    memcpy(din, d, 32);
    din[32] = (uint8_t)k;
    oracle_sha3_512(buf, din, mlkem ? 33 : 32);
    const uint8_t *rho = buf, *sigma = buf + 32;
    gen_matrix(a, rho, 0, p);
    uint8_t nonce = 0;
    for (int i = 0; i < k; i++) getnoise(&s[i], sigma, nonce++, p->eta1);
    for (int i = 0; i < k; i++) getnoise(&e[i], sigma, nonce++, p->eta1);
    for (int i = 0; i < k; i++) poly_ntt(&s[i]);
    for (int i = 0; i < k; i++) poly_ntt(&e[i]);
    for (int i = 0; i < k; i++) {
        pointwise_acc(&t[i], &a[i * k], s, k);
        poly_frommont(&t[i]);
    }
    for (int i = 0; i < k; i++)
        for (int j = 0; j < KN; j++) t[i].c[j] = (int16_t)(t[i].c[j] + e[i].c[j]);
    for (int i = 0; i < k; i++) poly_reduce(&t[i]);
    for (int i = 0; i < k; i++) poly_tobytes(sk + 384 * i, &s[i]);
    for (int i = 0; i < k; i++) poly_tobytes(pk + 384 * i, &t[i]);
    memcpy(pk + p->polyvecbytes, rho, 32);
}
static void cpa_keypair(const kparams *p, uint8_t *pk, uint8_t *sk, const uint8_t d[32]) {
    cpa_keypair_g(p, pk, sk, d, 0);
}

static void cpa_enc(const kparams *p, uint8_t *ct, const uint8_t m[32], const uint8_t *pk, const uint8_t coins[32]) {
    int k = p->k;
    kpoly at[16], sp[4] = {{{0}}}, ep[4], bp[4], pkpv[4], v, kmsg, epp;
    uint8_t rho[32];
    for (int i = 0; i < k; i++) poly_frombytes(&pkpv[i], pk + 384 * i);
    memcpy(rho, pk + p->polyvecbytes, 32);
    poly_frommsg(&kmsg, m);
    gen_matrix(at, rho, 1, p);
    uint8_t nonce = 0;
    for (int i = 0; i < k; i++) getnoise(&sp[i], coins, nonce++, p->eta1);
    for (int i = 0; i < k; i++) getnoise(&ep[i], coins, nonce++, p->eta2);
    getnoise(&epp, coins, nonce++, p->eta2);
    for (int i = 0; i < k; i++) poly_ntt(&sp[i]);
    for (int i = 0; i < k; i++) pointwise_acc(&bp[i], &at[i * k], sp, k);
    pointwise_acc(&v, pkpv, sp, k);
    for (int i = 0; i < k; i++) invntt(bp[i].c);
    invntt(v.c);
    for (int i = 0; i < k; i++)
        for (int j = 0; j < KN; j++) bp[i].c[j] = (int16_t)(bp[i].c[j] + ep[i].c[j]);
    for (int j = 0; j < KN; j++) v.c[j] = (int16_t)(v.c[j] + epp.c[j]);
    for (int j = 0; j < KN; j++) v.c[j] = (int16_t)(v.c[j] + kmsg.c[j]);
    for (int i = 0; i < k; i++) poly_reduce(&bp[i]);
    poly_reduce(&v);
    for (int i = 0; i < k; i++) poly_compress(ct + (size_t)i * p->du * 32, &bp[i], p->du);
    poly_compress(ct + p->polyveccomp, &v, p->dv);
}

static void cpa_dec(const kparams *p, uint8_t m[32], const uint8_t *ct, const uint8_t *sk) {
    int k = p->k;
    kpoly bp[4], skpv[4], v, mp;
    for (int i = 0; i < k; i++) poly_decompress(&bp[i], ct + (size_t)i * p->du * 32, p->du);
    poly_decompress(&v, ct + p->polyveccomp, p->dv);
    for (int i = 0; i < k; i++) poly_frombytes(&skpv[i], sk + 384 * i);
    for (int i = 0; i < k; i++) poly_ntt(&bp[i]);
    pointwise_acc(&mp, skpv, bp, k);
    invntt(mp.c);
    for (int j = 0; j < KN; j++) mp.c[j] = (int16_t)(v.c[j] - mp.c[j]);
    poly_reduce(&mp);
    poly_tomsg(m, &mp);
}

int oracle_kyber_indcpa_keypair(int variant, int k, uint8_t *pk, uint8_t *sk, const uint8_t d[32]) {
    kparams p;
    if (kparams_get(variant, k, &p)) return -1;
    cpa_keypair(&p, pk, sk, d);
    return 0;
}
int oracle_kyber_indcpa_enc(int variant, int k, uint8_t *ct, const uint8_t m[32], const uint8_t *pk,
                            const uint8_t coins[32]) {
    kparams p;
    if (kparams_get(variant, k, &p)) return -1;
    cpa_enc(&p, ct, m, pk, coins);
    return 0;
}
int oracle_kyber_indcpa_dec(int variant, int k, uint8_t m[32], const uint8_t *ct, const uint8_t *sk) {
    kparams p;
    if (kparams_get(variant, k, &p)) return -1;
    cpa_dec(&p, m, ct, sk);
    return 0;
}

/* ---- KEM (Fujisaki-Okamoto transform) ---- */
int oracle_kyber_kem_keypair(int variant, int k, uint8_t *pk, uint8_t *sk, const uint8_t coins[64]) {
    kparams p;
    if (kparams_get(variant, k, &p)) return -1;
    cpa_keypair(&p, pk, sk, coins);
    memcpy(sk + p.skcpa, pk, p.pk);
    oracle_sha3_256(sk + p.sk - 64, pk, p.pk);
    memcpy(sk + p.sk - 32, coins + 32, 32);
    return 0;
}

int oracle_kyber_kem_enc(int variant, int k, uint8_t *ct, uint8_t ss[32], const uint8_t *pk, const uint8_t coins[32]) {
    kparams p;
    if (kparams_get(variant, k, &p)) return -1;
    uint8_t buf[64], kr[64];
    oracle_sha3_256(buf, coins, 32);      /* m = H(coins) */
    oracle_sha3_256(buf + 32, pk, p.pk);  /* H(pk) */
    oracle_sha3_512(kr, buf, 64);         /* (K, r) = G(m || H(pk)) */
    cpa_enc(&p, ct, buf, pk, kr + 32);
    oracle_sha3_256(kr + 32, ct, p.ct);   /* H(c) */
    oracle_shake256(ss, 32, kr, 64);      /* KDF(K || H(c)) */
    return 0;
}

int oracle_kyber_kem_dec(int variant, int k, uint8_t ss[32], const uint8_t *ct, const uint8_t *sk) {
    kparams p;
    if (kparams_get(variant, k, &p)) return -1;
    uint8_t buf[64], kr[64], cmp[1568 + 16];
    const uint8_t *pk = sk + p.skcpa;
    cpa_dec(&p, buf, ct, sk);
    memcpy(buf + 32, sk + p.sk - 64, 32);
    oracle_sha3_512(kr, buf, 64);
    cpa_enc(&p, cmp, buf, pk, kr + 32);
    uint8_t diff = 0;
    for (size_t i = 0; i < p.ct; i++) diff |= (uint8_t)(ct[i] ^ cmp[i]);
    oracle_sha3_256(kr + 32, ct, p.ct);
    if (diff) memcpy(kr, sk + p.sk - 32, 32);
    oracle_shake256(ss, 32, kr, 64);
    return 0;
}

/* ---- ML-KEM (FIPS 203): the same K-PKE with G(d || k), and a KEM layer without the message
 * pre-hash and without the final KDF.  Keys are laid out as in round 3:
 * dk = dk_pke || ek || H(ek) || z; the shared key is K from (K, r) = G(m || H(ek)); decapsulation
 * rejects to J(z || c) = SHAKE256(z || c, 32).  Sizes equal the round-3 sets (k = 2, 3, 4). ---- */
int oracle_mlkem_keypair(int k, uint8_t *pk, uint8_t *sk, const uint8_t coins[64]) {
    kparams p;
    if (kparams_get(3, k, &p)) return -1;
    cpa_keypair_g(&p, pk, sk, coins, 1);
    memcpy(sk + p.skcpa, pk, p.pk);
    oracle_sha3_256(sk + p.sk - 64, pk, p.pk);
    memcpy(sk + p.sk - 32, coins + 32, 32);
    return 0;
}

int oracle_mlkem_enc(int k, uint8_t *ct, uint8_t ss[32], const uint8_t *pk, const uint8_t m[32]) {
    kparams p;
    if (kparams_get(3, k, &p)) return -1;
    uint8_t buf[64], kr[64];
    memcpy(buf, m, 32);
    oracle_sha3_256(buf + 32, pk, p.pk);  /* H(ek) */
    oracle_sha3_512(kr, buf, 64);         /* (K, r) = G(m || H(ek)) */
    cpa_enc(&p, ct, m, pk, kr + 32);
    memcpy(ss, kr, 32);
    return 0;
}

int oracle_mlkem_dec(int k, uint8_t ss[32], const uint8_t *ct, const uint8_t *sk) {
    kparams p;
    if (kparams_get(3, k, &p)) return -1;
    uint8_t buf[64], kr[64], kbar[32], cmp[1568 + 16], zc[32 + 1568];
    const uint8_t *pk = sk + p.skcpa;
    cpa_dec(&p, buf, ct, sk);
    memcpy(buf + 32, sk + p.sk - 64, 32);  /* h = H(ek) */
    oracle_sha3_512(kr, buf, 64);          /* (K', r') = G(m' || h) */
    memcpy(zc, sk + p.sk - 32, 32);
    memcpy(zc + 32, ct, p.ct);
    oracle_shake256(kbar, 32, zc, 32 + p.ct);  /* J(z || c) */
    cpa_enc(&p, cmp, buf, pk, kr + 32);
    uint8_t diff = 0;
    for (size_t i = 0; i < p.ct; i++) diff |= (uint8_t)(ct[i] ^ cmp[i]);
    const uint8_t mask = (uint8_t)(0u - (uint8_t)(diff != 0));
    for (int i = 0; i < 32; i++) ss[i] = (uint8_t)(kr[i] ^ (mask & (kr[i] ^ kbar[i])));
    return 0;
}
