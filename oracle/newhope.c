/*
 * NewHope-1024 and NewHope-512 CPA-PKE and CPA-KEM restated in plain C -- TEST INFRASTRUCTURE
 * (CPU oracle).
 *
 * Every integer step mirrors the reference so intermediate (lazily reduced) values agree:
 *   montgomery_reduce (R = 2^18, qinv = 12287), barrett (a*5 >> 16)
 *                                         NewHope_NIST_GPU/reduce.cu:22-47
 *   twiddle tables, generated here from g = 7 (n = 1024; a primitive 2048-th root of unity mod
 *   12289) or g = 10968 (n = 512; a primitive 1024-th root) and mont = 2^18 mod q with the formulas
 *   documented at NewHope_NIST_GPU/precomp.cu:27-29, :69-71:
 *     gammas_bitrev[i] = g^brv(i) * mont, omegas_inv_bitrev[i] = g^(-2 brv(2i)) * mont,
 *     gammas_inv[i] = g^(-i) * n^-1 * mont   (all lifted to [0, q))
 *   These equal the reference's tables for both n (precomp.cu:75-183 for n = 512).
 *   bitrev_vector, mul_coefficients, lazy ntt: 10 layers with barrett_reduce on odd layers for
 *   n = 1024 (NewHope_NIST_GPU/ntt.cu:92-234); 9 layers with `% q` on odd layers for n = 512,
 *   the reference's scalar n = 512 transform (ntt.cu:143-181)
 *   poly_uniform (n/64 x SHAKE128(seed||i), 16-bit samples < 5q)
 *   poly_sample (n/64 x SHAKE256(seed||nonce||i) 128 B, HW(a) + q - HW(b))
 *   pointwise (3186 = R^2 mod q), add / sub with %, codecs, msg (each message bit in n/256
 *   coefficients; tomsg subtracts q for n = 1024, q/2 for n = 512, poly.cu:226-291)
 *                                         NewHope_NIST_GPU/poly.cu:19-508
 *   cpapke_keypair / enc / dec            NewHope_NIST_GPU/cpapke.cu:265-476, with the seed layout
 *     of the NIST flow (publicseed || noiseseed = SHAKE256(seed, 64) per instance; the
 *     reference's temp_2 layout at cpapke.cu:283-284 is not reproduced).
 * CPA-KEM (the reference only fixes its sizes, NewHope_NIST_GPU/api.h:11-14): the NIST
 * NewHope CPA-KEM without domain-separation prefixes, matching the reference's unprefixed seed
 * expansion: buf = SHAKE256(coins, 64); ct = Enc(pk, buf[0:32], buf[32:64]);
 * ss = SHAKE256(buf[0:32], 32); decaps ss = SHAKE256(Dec(ct), 32).
 */
#include <string.h>
#include "oracle.h"

#define NMAX 1024
#define NQ 12289

extern _Thread_local uint64_t oracle_g_butterfly_count;

/* per-n tables; NN, NPOLYBYTES below refer to the parameter set in use */
typedef struct {
    int n, logn;
    uint16_t br[NMAX], gb[NMAX], oib[NMAX / 2], gi[NMAX];
} NhTables;
static NhTables T1024, T512;
static _Thread_local const NhTables *T = &T1024;
#define NN (T->n)
#define NPOLYBYTES (14 * NN / 8)
#define bitrev (T->br)
#define gammas_bitrev (T->gb)
#define omegas_inv_bitrev (T->oib)
#define gammas_inv (T->gi)

static long powmod(long b, long e, long m) {
    long r = 1;
    b %= m;
    if (b < 0) b += m;
    while (e) {
        if (e & 1) r = r * b % m;
        b = b * b % m;
        e >>= 1;
    }
    return r;
}

static void tables_init(NhTables *t, int n, int logn, long g) {
    const long mont = (1L << 18) % NQ;
    const long ginv = powmod(g, NQ - 2, NQ), ninv = powmod(n, NQ - 2, NQ);
    t->n = n;
    t->logn = logn;
    for (int i = 0; i < n; i++) {
        int r = 0;
        for (int b = 0; b < logn; b++) r |= ((i >> b) & 1) << (logn - 1 - b);
        t->br[i] = (uint16_t)r;
    }
    for (int i = 0; i < n; i++) t->gb[i] = (uint16_t)(powmod(g, t->br[i], NQ) * mont % NQ);
    for (int i = 0; i < n / 2; i++) t->oib[i] = (uint16_t)(powmod(ginv, 2L * t->br[2 * i], NQ) * mont % NQ);
    for (int i = 0; i < n; i++) t->gi[i] = (uint16_t)(powmod(ginv, i, NQ) * ninv % NQ * mont % NQ);
}
__attribute__((constructor)) static void newhope_tables_init(void) {
    tables_init(&T1024, 1024, 10, 7);
    tables_init(&T512, 512, 9, 10968);
}

static uint16_t nh_mont(uint32_t a) {
    uint32_t u = a * 12287u;
    u &= (1u << 18) - 1;
    u *= NQ;
    a = a + u;
    return (uint16_t)(a >> 18);
}
static uint16_t nh_barrett(uint16_t a) {
    uint32_t u = ((uint32_t)a * 5) >> 16;
    u *= NQ;
    a = (uint16_t)(a - u);
    return a;
}
static uint16_t freeze(uint16_t x) {
    uint16_t r = (uint16_t)(x % NQ);
    uint16_t m = (uint16_t)(r - NQ);
    int16_t c = (int16_t)m;
    c >>= 15;
    return (uint16_t)(m ^ ((r ^ m) & (uint16_t)c));
}
static uint16_t flipabs(uint16_t x) {
    int16_t r = (int16_t)freeze(x), m;
    r = (int16_t)(r - NQ / 2);
    m = (int16_t)(r >> 15);
    return (uint16_t)((r + m) ^ m);
}

static void mul_coeffs(uint16_t *p, const uint16_t *f) {
    for (int i = 0; i < NN; i++) p[i] = nh_mont((uint32_t)p[i] * f[i]);
}
static void bitrev_vec(uint16_t *p) {
    for (int i = 0; i < NN; i++) {
        int r = bitrev[i];
        if (i < r) {
            uint16_t t = p[i];
            p[i] = p[r];
            p[r] = t;
        }
    }
}
static void nh_ntt(uint16_t *a, const uint16_t *omega) {
    const int layers = T->logn;
    for (int i = 0; i < layers; i += 2) {
        int distance = 1 << i;
        for (int start = 0; start < distance; start++) {
            int jt = 0;
            for (int j = start; j < NN - 1; j += 2 * distance) {
                uint16_t W = omega[jt++], temp = a[j];
                a[j] = (uint16_t)(temp + a[j + distance]);
                a[j + distance] = nh_mont((uint32_t)W * ((uint32_t)temp + 3 * NQ - a[j + distance]));
                oracle_g_butterfly_count++;
            }
        }
        if (i + 1 >= layers) break;
        distance <<= 1;
        for (int start = 0; start < distance; start++) {
            int jt = 0;
            for (int j = start; j < NN - 1; j += 2 * distance) {
                uint16_t W = omega[jt++], temp = a[j];
                if (NN == 1024)
                    a[j] = nh_barrett((uint16_t)(temp + a[j + distance]));
                else
                    a[j] = (uint16_t)((temp + a[j + distance]) % NQ);
                a[j + distance] = nh_mont((uint32_t)W * ((uint32_t)temp + 3 * NQ - a[j + distance]));
                oracle_g_butterfly_count++;
            }
        }
    }
}
static void poly_ntt(uint16_t *r) {
    mul_coeffs(r, gammas_bitrev);
    nh_ntt(r, gammas_bitrev);
}
static void poly_invntt(uint16_t *r) {
    bitrev_vec(r);
    nh_ntt(r, omegas_inv_bitrev);
    mul_coeffs(r, gammas_inv);
}
static void poly_pointwise(uint16_t *r, const uint16_t *a, const uint16_t *b) {
    for (int i = 0; i < NN; i++) {
        uint16_t t = nh_mont(3186u * b[i]);
        r[i] = nh_mont((uint32_t)a[i] * t);
    }
}
static void poly_add(uint16_t *r, const uint16_t *a, const uint16_t *b) {
    for (int i = 0; i < NN; i++) r[i] = (uint16_t)((a[i] + b[i]) % NQ);
}
static void poly_sub(uint16_t *r, const uint16_t *a, const uint16_t *b) {
    for (int i = 0; i < NN; i++) r[i] = (uint16_t)((a[i] + 3 * NQ - b[i]) % NQ);
}
static void poly_tobytes(uint8_t *r, const uint16_t *p) {
    for (int i = 0; i < NN / 4; i++) {
        uint16_t t0 = freeze(p[4 * i]), t1 = freeze(p[4 * i + 1]), t2 = freeze(p[4 * i + 2]),
                 t3 = freeze(p[4 * i + 3]);
        r[7 * i + 0] = (uint8_t)(t0 & 0xff);
        r[7 * i + 1] = (uint8_t)((t0 >> 8) | (t1 << 6));
        r[7 * i + 2] = (uint8_t)(t1 >> 2);
        r[7 * i + 3] = (uint8_t)((t1 >> 10) | (t2 << 4));
        r[7 * i + 4] = (uint8_t)(t2 >> 4);
        r[7 * i + 5] = (uint8_t)((t2 >> 12) | (t3 << 2));
        r[7 * i + 6] = (uint8_t)(t3 >> 6);
    }
}
static void poly_frombytes(uint16_t *r, const uint8_t *a) {
    for (int i = 0; i < NN / 4; i++) {
        r[4 * i + 0] = (uint16_t)(a[7 * i + 0] | (((uint16_t)a[7 * i + 1] & 0x3f) << 8));
        r[4 * i + 1] = (uint16_t)((a[7 * i + 1] >> 6) | (((uint16_t)a[7 * i + 2]) << 2) |
                                  (((uint16_t)a[7 * i + 3] & 0x0f) << 10));
        r[4 * i + 2] = (uint16_t)((a[7 * i + 3] >> 4) | (((uint16_t)a[7 * i + 4]) << 4) |
                                  (((uint16_t)a[7 * i + 5] & 0x03) << 12));
        r[4 * i + 3] = (uint16_t)((a[7 * i + 5] >> 2) | (((uint16_t)a[7 * i + 6]) << 6));
    }
}
static void poly_compress(uint8_t *r, const uint16_t *p) {
    for (int i = 0, k = 0; i < NN; i += 8, k += 3) {
        uint32_t t[8];
        for (int j = 0; j < 8; j++) {
            t[j] = freeze(p[i + j]);
            t[j] = (((t[j] << 3) + NQ / 2) / NQ) & 0x7;
        }
        r[k] = (uint8_t)(t[0] | (t[1] << 3) | (t[2] << 6));
        r[k + 1] = (uint8_t)((t[2] >> 2) | (t[3] << 1) | (t[4] << 4) | (t[5] << 7));
        r[k + 2] = (uint8_t)((t[5] >> 1) | (t[6] << 2) | (t[7] << 5));
    }
}
static void poly_decompress(uint16_t *r, const uint8_t *a) {
    for (int i = 0; i < NN; i += 8, a += 3) {
        r[i + 0] = a[0] & 7;
        r[i + 1] = (a[0] >> 3) & 7;
        r[i + 2] = (uint16_t)((a[0] >> 6) | ((a[1] << 2) & 4));
        r[i + 3] = (a[1] >> 1) & 7;
        r[i + 4] = (a[1] >> 4) & 7;
        r[i + 5] = (uint16_t)((a[1] >> 7) | ((a[2] << 1) & 6));
        r[i + 6] = (a[2] >> 2) & 7;
        r[i + 7] = (a[2] >> 5);
        for (int j = 0; j < 8; j++) r[i + j] = (uint16_t)(((uint32_t)r[i + j] * NQ + 4) >> 3);
    }
}
static void poly_frommsg(uint16_t *r, const uint8_t *msg) {
    for (int i = 0; i < 32; i++)
        for (int j = 0; j < 8; j++) {
            uint16_t mask = (uint16_t)-((msg[i] >> j) & 1);
            uint16_t v = (uint16_t)(mask & (NQ / 2));
            for (int c = 8 * i + j; c < NN; c += 256) r[c] = v;
        }
}
static void poly_tomsg(uint8_t *msg, const uint16_t *x) {
    memset(msg, 0, 32);
    for (int i = 0; i < 256; i++) {
        uint16_t t = 0;
        for (int c = i; c < NN; c += 256) t = (uint16_t)(t + flipabs(x[c]));
        t = (uint16_t)(t - (NN == 1024 ? NQ : NQ / 2));
        t >>= 15;
        msg[i >> 3] |= (uint8_t)(t << (i & 7));
    }
}

static void poly_uniform(uint16_t *a, const uint8_t *seed) {
    uint8_t ext[33], buf[168];
    uint64_t s[25];
    memcpy(ext, seed, 32);
    for (int i = 0; i < NN / 64; i++) {
        ext[32] = (uint8_t)i;
        /* absorb the 33-byte input (single block) */
        uint8_t blk[168];
        memset(blk, 0, sizeof blk);
        memcpy(blk, ext, 33);
        blk[33] ^= 0x1F;
        blk[167] ^= 0x80;
        memset(s, 0, sizeof s);
        for (int w = 0; w < 21; w++) {
            uint64_t v = 0;
            for (int b = 0; b < 8; b++) v |= (uint64_t)blk[8 * w + b] << (8 * b);
            s[w] ^= v;
        }
        int ctr = 0;
        while (ctr < 64) {
            oracle_keccakf1600(s);
            for (int b = 0; b < 168; b++) buf[b] = (uint8_t)(s[b / 8] >> (8 * (b % 8)));
            for (int j = 0; j < 168 && ctr < 64; j += 2) {
                uint16_t val = (uint16_t)(buf[j] | ((uint16_t)buf[j + 1] << 8));
                if (val < 5 * NQ) a[i * 64 + ctr++] = val;
            }
        }
    }
}
static uint8_t hw8(uint8_t a) {
    uint8_t r = 0;
    for (int i = 0; i < 8; i++) r = (uint8_t)(r + ((a >> i) & 1));
    return r;
}
static void poly_sample(uint16_t *r, const uint8_t *seed, uint8_t nonce) {
    uint8_t ext[34], buf[128];
    memcpy(ext, seed, 32);
    ext[32] = nonce;
    for (int i = 0; i < NN / 64; i++) {
        ext[33] = (uint8_t)i;
        oracle_shake256(buf, 128, ext, 34);
        for (int j = 0; j < 64; j++) r[64 * i + j] = (uint16_t)(hw8(buf[2 * j]) + NQ - hw8(buf[2 * j + 1]));
    }
}

static int cpa_keypair(uint8_t *pk, uint8_t *sk, const uint8_t seed[32]) {
    static _Thread_local uint16_t ahat[NMAX], ehat[NMAX], ahat_shat[NMAX], bhat[NMAX], shat[NMAX];
    uint8_t z[64];
    oracle_shake256(z, 64, seed, 32);
    const uint8_t *publicseed = z, *noiseseed = z + 32;
    poly_uniform(ahat, publicseed);
    poly_sample(shat, noiseseed, 0);
    poly_ntt(shat);
    poly_sample(ehat, noiseseed, 1);
    poly_ntt(ehat);
    poly_pointwise(ahat_shat, shat, ahat);
    poly_add(bhat, ehat, ahat_shat);
    poly_tobytes(sk, shat);
    poly_tobytes(pk, bhat);
    memcpy(pk + NPOLYBYTES, publicseed, 32);
    return 0;
}

static int cpa_enc(uint8_t *ct, const uint8_t m[32], const uint8_t *pk, const uint8_t coin[32]) {
    static _Thread_local uint16_t sprime[NMAX], eprime[NMAX], vprime[NMAX], ahat[NMAX], bhat[NMAX], epp[NMAX], uhat[NMAX], v[NMAX];
    poly_frommsg(v, m);
    poly_frombytes(bhat, pk);
    poly_uniform(ahat, pk + NPOLYBYTES);
    poly_sample(sprime, coin, 0);
    poly_sample(eprime, coin, 1);
    poly_sample(epp, coin, 2);
    poly_ntt(sprime);
    poly_ntt(eprime);
    poly_pointwise(uhat, ahat, sprime);
    poly_add(uhat, uhat, eprime);
    poly_pointwise(vprime, bhat, sprime);
    poly_invntt(vprime);
    poly_add(vprime, vprime, epp);
    poly_add(vprime, vprime, v);
    poly_tobytes(ct, uhat);
    poly_compress(ct + NPOLYBYTES, vprime);
    return 0;
}

static int cpa_dec(uint8_t m[32], const uint8_t *ct, const uint8_t *sk) {
    static _Thread_local uint16_t vprime[NMAX], uhat[NMAX], tmp[NMAX], shat[NMAX];
    poly_frombytes(shat, sk);
    poly_frombytes(uhat, ct);
    poly_decompress(vprime, ct + NPOLYBYTES);
    poly_pointwise(tmp, shat, uhat);
    poly_invntt(tmp);
    poly_sub(tmp, tmp, vprime);
    poly_tomsg(m, tmp);
    return 0;
}

static int kem_enc(uint8_t *ct, uint8_t ss[32], const uint8_t *pk, const uint8_t coins[32]) {
    uint8_t buf[64];
    oracle_shake256(buf, 64, coins, 32);
    cpa_enc(ct, buf, pk, buf + 32);
    oracle_shake256(ss, 32, buf, 32);
    return 0;
}
static int kem_dec(uint8_t ss[32], const uint8_t *ct, const uint8_t *sk) {
    uint8_t m[32];
    cpa_dec(m, ct, sk);
    oracle_shake256(ss, 32, m, 32);
    return 0;
}

/* public entry points: NewHope-1024 (oracle_newhope_*) and NewHope-512 (oracle_newhope512_*) */
#define NH_ENTRY(prefix, tables)                                                                         \
    int prefix##_cpapke_keypair(uint8_t *pk, uint8_t *sk, const uint8_t seed[32]) {                      \
        T = &tables;                                                                                     \
        return cpa_keypair(pk, sk, seed);                                                                \
    }                                                                                                    \
    int prefix##_cpapke_enc(uint8_t *ct, const uint8_t m[32], const uint8_t *pk, const uint8_t coin[32]) { \
        T = &tables;                                                                                     \
        return cpa_enc(ct, m, pk, coin);                                                                 \
    }                                                                                                    \
    int prefix##_cpapke_dec(uint8_t m[32], const uint8_t *ct, const uint8_t *sk) {                       \
        T = &tables;                                                                                     \
        return cpa_dec(m, ct, sk);                                                                       \
    }                                                                                                    \
    int prefix##_kem_keypair(uint8_t *pk, uint8_t *sk, const uint8_t coins[32]) {                       \
        T = &tables;                                                                                     \
        return cpa_keypair(pk, sk, coins);                                                               \
    }                                                                                                    \
    int prefix##_kem_enc(uint8_t *ct, uint8_t ss[32], const uint8_t *pk, const uint8_t coins[32]) {      \
        T = &tables;                                                                                     \
        return kem_enc(ct, ss, pk, coins);                                                               \
    }                                                                                                    \
    int prefix##_kem_dec(uint8_t ss[32], const uint8_t *ct, const uint8_t *sk) {                         \
        T = &tables;                                                                                     \
        return kem_dec(ss, ct, sk);                                                                      \
    }
NH_ENTRY(oracle_newhope, T1024)
NH_ENTRY(oracle_newhope512, T512)
