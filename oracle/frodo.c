/*
 * FrodoKEM-640 / 976 / 1344 (SHAKE variant, round-2 parameters) restated in plain C -- TEST
 * INFRASTRUCTURE.
 *
 * Host flow restated from FrodoKEM_GPU/kem.c:13-214 (keypair / enc / dec with the 0x5F / 0x96
 * domain bytes, G1 = SHAKE256 over pk, G2 over pkh || mu, F over ct || k, implicit rejection
 * with s).  Matrix arithmetic restated from the kernels' definitions:
 *   A row i = SHAKE128(le16(i) || seedA, 2n bytes) as little-endian u16
 *                                     FrodoKEM_GPU/frodo_macrify_reference.cu:164-188
 *   B  = A S + E   (S stored transposed, nbar x n)      :55-99 and :190-212
 *   B' = S' A + E'                                     :102-159 and :215-234
 *   W  = B' S,  V = S' B + E''                         :237-281
 *   add / sub / key encode / key decode (3 bits)        :284-360
 *   log q-bit pack / unpack (MSB-first bit order)       FrodoKEM_GPU/util.cu:18-113
 *   CDF sampler                                         FrodoKEM_GPU/noise.c:10-29 with the
 *                                                       table of FrodoKEM_GPU/frodo976.cu:21
 * The S / E stream is the standard SHAKE256(0x5F || seedSE) of kem.c:39 (resp. 0x96 at kem.c:96),
 * not the reference GPU path's shake256_kernel_single.
 * FrodoKEM-976 is pinned to the reference's own code: tests/golden/ref_frodo976_kem.json holds the
 * outputs of kem.c run with the reference's sampler, codecs, SHAKE and matrix kernels
 * (oracle/ref_glue_frodo.cpp), and this restatement reproduces them.
 * All arithmetic is mod 2^16 (uint16 wrap-around), so the matrix products are exact; for log q = 15
 * values are reduced mod q where they are packed, compared or decoded.
 *
 * The reference builds only n = 976 (FrodoKEM_GPU/params.h:17-30).  FrodoKEM-640 and -1344 run the
 * same flow with the other parameter sets of the FrodoKEM specification (round 2): n = 640 / 1344,
 * log q = 15 / 16, B = 2 / 4 encoded bits, 16 / 32-byte s, seedSE, z-derived keys, k, pkh, ss and mu,
 * SHAKE128 (640) or SHAKE256 (1344) for every hash and the noise stream, and the CDF tables
 * {4643, 13363, 20579, 25843, 29227, 31145, 32103, 32525, 32689, 32745, 32762, 32766, 32767} and
 * {9142, 23462, 30338, 32361, 32725, 32765, 32767}.  Nothing in the reference pins these two: their
 * parity rests on this restatement (the 976 instance of the same code is pinned by its sizes and
 * CDF table against the reference).
 */
#include <stdlib.h>
#include <string.h>
#include "oracle.h"

#define FNBAR 8
#define FSEEDA 16
#define FNMAX 1344

typedef struct {
    int n, logq, b, ss; /* ss: length of s, seedSE, k, pkh, ss and mu */
    int shake256;       /* hash = SHAKE256 (else SHAKE128) */
    int cdf_len;
    const uint16_t *cdf;
    size_t pk, sk, ct;
} FrodoP;
static const uint16_t CDF640[13] = {4643, 13363, 20579, 25843, 29227, 31145, 32103, 32525, 32689, 32745, 32762, 32766, 32767};
static const uint16_t CDF976[11] = {5638, 15915, 23689, 28571, 31116, 32217, 32613, 32731, 32760, 32766, 32767};
static const uint16_t CDF1344[7] = {9142, 23462, 30338, 32361, 32725, 32765, 32767};
static const FrodoP P640 = {640, 15, 2, 16, 0, 13, CDF640, 9616, 19888, 9720};
static const FrodoP P976 = {976, 16, 3, 24, 1, 11, CDF976, 15632, 31296, 15744};
static const FrodoP P1344 = {1344, 16, 4, 32, 1, 7, CDF1344, 21520, 43088, 21632};

static _Thread_local const FrodoP *F = &P976;
#define FN (F->n)
#define FPK (F->pk)
#define FSK (F->sk)
#define FCT (F->ct)
#define FSS (F->ss)
#define FMU (F->ss)
#define FC1 ((size_t)F->logq * FN * FNBAR / 8) /* packed N x NBAR matrix */
#define FMASK ((uint16_t)((1u << F->logq) - 1))

static void shake(uint8_t *out, size_t outlen, const uint8_t *in, size_t inlen) {
    if (F->shake256) oracle_shake256(out, outlen, in, inlen);
    else oracle_shake128(out, outlen, in, inlen);
}

static void sample_n(uint16_t *s, size_t n) {
    for (size_t i = 0; i < n; i++) {
        uint8_t sample = 0;
        uint16_t prnd = (uint16_t)(s[i] >> 1);
        uint8_t sign = (uint8_t)(s[i] & 1);
        for (int j = 0; j < F->cdf_len - 1; j++) sample = (uint8_t)(sample + ((uint16_t)(F->cdf[j] - prnd) >> 15));
        s[i] = (uint16_t)(((uint16_t)-sign ^ sample) + sign);
    }
}

static void le_bytes_to_u16(uint16_t *out, const uint8_t *in, size_t n) {
    for (size_t i = 0; i < n; i++) out[i] = (uint16_t)(in[2 * i] | (in[2 * i + 1] << 8));
}
static void u16_to_le_bytes(uint8_t *out, const uint16_t *in, size_t n) {
    for (size_t i = 0; i < n; i++) {
        out[2 * i] = (uint8_t)in[i];
        out[2 * i + 1] = (uint8_t)(in[i] >> 8);
    }
}
/* pack of util.cu: the low log q bits of each value, most significant bit first (for log q = 16,
 * big-endian u16) */
static void pack16(uint8_t *out, const uint16_t *in, size_t n) {
    const int d = F->logq;
    memset(out, 0, (size_t)d * n / 8);
    size_t bit = 0;
    for (size_t i = 0; i < n; i++)
        for (int b = d - 1; b >= 0; b--, bit++)
            if ((in[i] >> b) & 1) out[bit >> 3] |= (uint8_t)(0x80 >> (bit & 7));
}
static void unpack16(uint16_t *out, const uint8_t *in, size_t n) {
    const int d = F->logq;
    size_t bit = 0;
    for (size_t i = 0; i < n; i++) {
        uint16_t v = 0;
        for (int b = 0; b < d; b++, bit++) v = (uint16_t)((v << 1) | ((in[bit >> 3] >> (7 - (bit & 7))) & 1));
        out[i] = v;
    }
}

static void gen_row(uint16_t *row, const uint8_t seedA[16], int i) {
    uint8_t in[18], buf[2 * FNMAX];
    in[0] = (uint8_t)i;
    in[1] = (uint8_t)(i >> 8);
    memcpy(in + 2, seedA, 16);
    oracle_shake128(buf, 2 * FN, in, 18);
    le_bytes_to_u16(row, buf, FN);
}

/* out (n x nbar) = A s + e, with s stored transposed (nbar x n) */
static void mul_add_as_plus_e(uint16_t *out, const uint16_t *s, const uint16_t *e, const uint8_t seedA[16]) {
    uint16_t row[FNMAX];
    memcpy(out, e, sizeof(uint16_t) * FN * FNBAR);
    for (int i = 0; i < FN; i++) {
        gen_row(row, seedA, i);
        for (int k = 0; k < FNBAR; k++) {
            uint16_t sum = 0;
            for (int j = 0; j < FN; j++) sum = (uint16_t)(sum + row[j] * s[k * FN + j]);
            out[i * FNBAR + k] = (uint16_t)(out[i * FNBAR + k] + sum);
        }
    }
}
/* out (nbar x n) = s' A + e' */
static void mul_add_sa_plus_e(uint16_t *out, const uint16_t *s, const uint16_t *e, const uint8_t seedA[16]) {
    uint16_t row[FNMAX];
    memcpy(out, e, sizeof(uint16_t) * FN * FNBAR);
    for (int kk = 0; kk < FN; kk++) {
        gen_row(row, seedA, kk);
        for (int i = 0; i < FNBAR; i++) {
            uint16_t sp = s[i * FN + kk];
            for (int j = 0; j < FN; j++) out[i * FN + j] = (uint16_t)(out[i * FN + j] + sp * row[j]);
        }
    }
}
static void mul_bs(uint16_t *out, const uint16_t *b, const uint16_t *s) {
    for (int i = 0; i < FNBAR; i++)
        for (int j = 0; j < FNBAR; j++) {
            uint32_t sum = 0;
            for (int k = 0; k < FN; k++) sum += (uint32_t)b[i * FN + k] * s[j * FN + k];
            out[i * FNBAR + j] = (uint16_t)sum;
        }
}
static void mul_add_sb_plus_e(uint16_t *out, const uint16_t *b, const uint16_t *s, const uint16_t *e) {
    for (int k = 0; k < FNBAR; k++)
        for (int i = 0; i < FNBAR; i++) {
            uint32_t sum = e[k * FNBAR + i];
            for (int j = 0; j < FN; j++) sum += (uint32_t)s[k * FN + j] * b[j * FNBAR + i];
            out[k * FNBAR + i] = (uint16_t)sum;
        }
}
/* B bits of mu per value, scaled by q / 2^B (frodo_macrify_reference.cu:311-360) */
static void key_encode(uint16_t *out, const uint8_t *mu) {
    const int B = F->b, sh = F->logq - B;
    for (int i = 0; i < 8; i++) {
        uint32_t temp = 0;
        for (int j = 0; j < B; j++) temp |= (uint32_t)mu[B * i + j] << (8 * j);
        for (int j = 0; j < 8; j++) {
            out[8 * i + j] = (uint16_t)((temp & ((1u << B) - 1)) << sh);
            temp >>= B;
        }
    }
}
static void key_decode(uint8_t *mu, const uint16_t *in) {
    const int B = F->b, sh = F->logq - B;
    for (int i = 0; i < 8; i++) {
        uint32_t templong = 0;
        for (int j = 0; j < 8; j++) {
            uint16_t temp = (uint16_t)(((in[8 * i + j] & FMASK) + (1 << (sh - 1))) >> sh);
            templong |= (uint32_t)(temp & ((1u << B) - 1)) << (B * j);
        }
        for (int j = 0; j < B; j++) mu[B * i + j] = (uint8_t)(templong >> (8 * j));
    }
}

static int kem_keypair(uint8_t *pk, uint8_t *sk, const uint8_t *coins) {
    const uint8_t *rs = coins, *rseedSE = coins + FSS, *rz = coins + 2 * FSS;
    uint16_t *S = malloc(sizeof(uint16_t) * 2 * FN * FNBAR), *B = malloc(sizeof(uint16_t) * FN * FNBAR);
    uint8_t *buf = malloc(4 * FN * FNBAR), in[1 + 32];
    shake(pk, FSEEDA, rz, FSEEDA);
    in[0] = 0x5F;
    memcpy(in + 1, rseedSE, FSS);
    shake(buf, 4 * FN * FNBAR, in, 1 + FSS);
    le_bytes_to_u16(S, buf, 2 * FN * FNBAR);
    uint16_t *E = S + FN * FNBAR;
    sample_n(S, FN * FNBAR);
    sample_n(E, FN * FNBAR);
    mul_add_as_plus_e(B, S, E, pk);
    pack16(pk + FSEEDA, B, FN * FNBAR);
    memcpy(sk, rs, FSS);
    memcpy(sk + FSS, pk, FPK);
    u16_to_le_bytes(sk + FSS + FPK, S, FN * FNBAR);
    shake(sk + FSS + FPK + 2 * FN * FNBAR, FSS, pk, FPK);
    free(S);
    free(B);
    free(buf);
    return 0;
}

/* Sp, Ep (n*nbar each) and Epp (nbar*nbar) from SHAKE(0x96 || seedSE) */
static void sample_sp(uint16_t *Sp, const uint8_t *seedSE) {
    size_t n = (2 * FN + FNBAR) * FNBAR;
    uint8_t *buf = malloc(2 * n), in[1 + 32];
    in[0] = 0x96;
    memcpy(in + 1, seedSE, FSS);
    shake(buf, 2 * n, in, 1 + FSS);
    le_bytes_to_u16(Sp, buf, n);
    sample_n(Sp, n);
    free(buf);
}

static int kem_enc(uint8_t *ct, uint8_t *ss, const uint8_t *pk, const uint8_t *coins) {
    size_t nsp = (2 * FN + FNBAR) * FNBAR;
    uint16_t *Sp = malloc(sizeof(uint16_t) * nsp), *Bp = malloc(sizeof(uint16_t) * FN * FNBAR),
             *B = malloc(sizeof(uint16_t) * FN * FNBAR);
    uint16_t V[64], C[64];
    uint8_t G2in[64], G2out[64], *Fin = malloc(FCT + FSS);
    shake(G2in, FSS, pk, FPK);
    memcpy(G2in + FSS, coins, FMU);
    shake(G2out, 2 * FSS, G2in, FSS + FMU);
    sample_sp(Sp, G2out);
    uint16_t *Ep = Sp + FN * FNBAR, *Epp = Sp + 2 * FN * FNBAR;
    mul_add_sa_plus_e(Bp, Sp, Ep, pk);
    pack16(ct, Bp, FN * FNBAR);
    unpack16(B, pk + FSEEDA, FN * FNBAR);
    mul_add_sb_plus_e(V, B, Sp, Epp);
    key_encode(C, coins);
    for (int i = 0; i < 64; i++) C[i] = (uint16_t)(V[i] + C[i]);
    pack16(ct + FC1, C, 64);
    memcpy(Fin, ct, FCT);
    memcpy(Fin + FCT, G2out + FSS, FSS);
    shake(ss, FSS, Fin, FCT + FSS);
    free(Sp);
    free(Bp);
    free(B);
    free(Fin);
    return 0;
}

static int kem_dec(uint8_t *ss, const uint8_t *ct, const uint8_t *sk) {
    size_t nsp = (2 * FN + FNBAR) * FNBAR;
    uint16_t *Sp = malloc(sizeof(uint16_t) * nsp), *Bp = malloc(sizeof(uint16_t) * FN * FNBAR),
             *BBp = malloc(sizeof(uint16_t) * FN * FNBAR), *B = malloc(sizeof(uint16_t) * FN * FNBAR),
             *S = malloc(sizeof(uint16_t) * FN * FNBAR);
    uint16_t W[64], C[64], CC[64];
    uint8_t G2in[64], G2out[64], *Fin = malloc(FCT + FSS);
    const uint8_t *sk_s = sk, *sk_pk = sk + FSS, *sk_S = sk + FSS + FPK, *sk_pkh = sk + FSS + FPK + 2 * FN * FNBAR;
    unpack16(Bp, ct, FN * FNBAR);
    unpack16(C, ct + FC1, 64);
    le_bytes_to_u16(S, sk_S, FN * FNBAR);
    mul_bs(W, Bp, S);
    for (int i = 0; i < 64; i++) W[i] = (uint16_t)(C[i] - W[i]);
    memcpy(G2in, sk_pkh, FSS);
    key_decode(G2in + FSS, W);
    shake(G2out, 2 * FSS, G2in, FSS + FMU);
    sample_sp(Sp, G2out);
    uint16_t *Ep = Sp + FN * FNBAR, *Epp = Sp + 2 * FN * FNBAR;
    mul_add_sa_plus_e(BBp, Sp, Ep, sk_pk);
    unpack16(B, sk_pk + FSEEDA, FN * FNBAR);
    mul_add_sb_plus_e(W, B, Sp, Epp);
    key_encode(CC, G2in + FSS);
    for (int i = 0; i < 64; i++) CC[i] = (uint16_t)(W[i] + CC[i]);
    memcpy(Fin, ct, FCT);
    int eq = 1; /* compare mod q (Bp and C come unpacked from log q bits) */
    for (int i = 0; i < FN * FNBAR; i++) eq &= (uint16_t)(BBp[i] & FMASK) == Bp[i];
    for (int i = 0; i < 64; i++) eq &= (uint16_t)(CC[i] & FMASK) == C[i];
    memcpy(Fin + FCT, eq ? G2out + FSS : sk_s, FSS);
    shake(ss, FSS, Fin, FCT + FSS);
    free(Sp);
    free(Bp);
    free(BBp);
    free(B);
    free(S);
    free(Fin);
    return 0;
}

/* public entry points per parameter set */
#define FRODO_ENTRY(prefix, params)                                                             \
    int prefix##_kem_keypair(uint8_t *pk, uint8_t *sk, const uint8_t *coins) {                    \
        F = &params;                                                                            \
        return kem_keypair(pk, sk, coins);                                                      \
    }                                                                                           \
    int prefix##_kem_enc(uint8_t *ct, uint8_t *ss, const uint8_t *pk, const uint8_t *coins) {     \
        F = &params;                                                                            \
        return kem_enc(ct, ss, pk, coins);                                                      \
    }                                                                                           \
    int prefix##_kem_dec(uint8_t *ss, const uint8_t *ct, const uint8_t *sk) {                     \
        F = &params;                                                                            \
        return kem_dec(ss, ct, sk);                                                             \
    }
FRODO_ENTRY(oracle_frodo, P976)
FRODO_ENTRY(oracle_frodo640, P640)
FRODO_ENTRY(oracle_frodo1344, P1344)
