/*
 * Keccak-f[1600] and the FIPS-202 sponge functions, restated from FIPS 202 (sections 3.2, 4, 6).
 * TEST INFRASTRUCTURE: part of the CPU oracle; never linked into the product library.
 *
 * Reference behaviour followed: Kyber_GPU_Batched/fips202.cu:393-447 (permutation),
 * :462-530 (absorb / squeeze with pad10*1 and domain byte), :543-689 (SHAKE128 / SHAKE256 /
 * SHA3-256 / SHA3-512 with rates 168 / 136 / 136 / 72 and domain bytes 0x1F / 0x06).
 * The round constants and rotation offsets are derived here from their FIPS 202 definitions
 * (the rc(t) LFSR of Algorithm 5 and the (t+1)(t+2)/2 offsets of Algorithm 2) rather than
 * typed in as tables.
 */
#include <string.h>
#include "oracle.h"

static uint64_t RC[24];
static unsigned ROT[25];
static _Thread_local uint64_t g_keccak_count;
_Thread_local uint64_t oracle_g_butterfly_count;

/* FIPS 202 Algorithm 5: rc(t) from the LFSR x^8 + x^6 + x^5 + x^4 + 1. */
static int rc_bit(int t) {
    if (t % 255 == 0) return 1;
    /* R = 10000000; each step: R = 0 || R; R[0,4,5,6] ^= R[8]; R = Trunc8(R). */
    int R[9] = {1, 0, 0, 0, 0, 0, 0, 0, 0};
    for (int i = 1; i <= t % 255; i++) {
        int Rn[9];
        Rn[0] = 0;
        for (int j = 0; j < 8; j++) Rn[j + 1] = R[j];
        Rn[0] ^= Rn[8];
        Rn[4] ^= Rn[8];
        Rn[5] ^= Rn[8];
        Rn[6] ^= Rn[8];
        for (int j = 0; j < 9; j++) R[j] = Rn[j];
    }
    return R[0];
}

__attribute__((constructor)) static void keccak_tables_init(void) {
    for (int ir = 0; ir < 24; ir++) {
        uint64_t rc = 0;
        for (int j = 0; j <= 6; j++)
            if (rc_bit(j + 7 * ir)) rc |= (uint64_t)1 << ((1u << j) - 1);
        RC[ir] = rc;
    }
    ROT[0] = 0;
    int x = 1, y = 0;
    for (int t = 0; t < 24; t++) {
        ROT[x + 5 * y] = (unsigned)(((t + 1) * (t + 2) / 2) % 64);
        int nx = y, ny = (2 * x + 3 * y) % 5;
        x = nx;
        y = ny;
    }
}

static inline uint64_t rol64(uint64_t v, unsigned n) { return n ? (v << n) | (v >> (64 - n)) : v; }

void oracle_keccakf1600(uint64_t A[25]) {
    g_keccak_count++;
    for (int ir = 0; ir < 24; ir++) {
        uint64_t C[5], D[5], B[25];
        for (int x = 0; x < 5; x++) C[x] = A[x] ^ A[x + 5] ^ A[x + 10] ^ A[x + 15] ^ A[x + 20];
        for (int x = 0; x < 5; x++) D[x] = C[(x + 4) % 5] ^ rol64(C[(x + 1) % 5], 1);
        for (int i = 0; i < 25; i++) A[i] ^= D[i % 5];
        /* rho + pi: B[y][2x+3y] = rot(A[x][y]) */
        for (int x = 0; x < 5; x++)
            for (int y = 0; y < 5; y++) B[y + 5 * ((2 * x + 3 * y) % 5)] = rol64(A[x + 5 * y], ROT[x + 5 * y]);
        /* chi */
        for (int y = 0; y < 5; y++)
            for (int x = 0; x < 5; x++)
                A[x + 5 * y] = B[x + 5 * y] ^ ((~B[(x + 1) % 5 + 5 * y]) & B[(x + 2) % 5 + 5 * y]);
        /* iota */
        A[0] ^= RC[ir];
    }
}

/* Sponge with byte-oriented absorb / squeeze; `pad` is the domain byte (0x1F SHAKE, 0x06 SHA3). */
static void sponge(uint8_t *out, size_t outlen, const uint8_t *in, size_t inlen, unsigned rate, uint8_t pad) {
    uint64_t s[25];
    uint8_t blk[200];
    memset(s, 0, sizeof s);
    while (inlen >= rate) {
        for (unsigned i = 0; i < rate / 8; i++) {
            uint64_t w = 0;
            for (int b = 0; b < 8; b++) w |= (uint64_t)in[8 * i + b] << (8 * b);
            s[i] ^= w;
        }
        oracle_keccakf1600(s);
        in += rate;
        inlen -= rate;
    }
    memset(blk, 0, sizeof blk);
    memcpy(blk, in, inlen);
    blk[inlen] ^= pad;
    blk[rate - 1] ^= 0x80;
    for (unsigned i = 0; i < rate / 8; i++) {
        uint64_t w = 0;
        for (int b = 0; b < 8; b++) w |= (uint64_t)blk[8 * i + b] << (8 * b);
        s[i] ^= w;
    }
    for (;;) {
        oracle_keccakf1600(s);
        size_t take = outlen < rate ? outlen : rate;
        for (size_t i = 0; i < take; i++) out[i] = (uint8_t)(s[i / 8] >> (8 * (i % 8)));
        out += take;
        outlen -= take;
        if (!outlen) break;
    }
}

void oracle_shake128(uint8_t *out, size_t outlen, const uint8_t *in, size_t inlen) {
    sponge(out, outlen, in, inlen, 168, 0x1F);
}
void oracle_shake256(uint8_t *out, size_t outlen, const uint8_t *in, size_t inlen) {
    sponge(out, outlen, in, inlen, 136, 0x1F);
}
void oracle_sha3_256(uint8_t out[32], const uint8_t *in, size_t inlen) { sponge(out, 32, in, inlen, 136, 0x06); }
void oracle_sha3_512(uint8_t out[64], const uint8_t *in, size_t inlen) { sponge(out, 64, in, inlen, 72, 0x06); }

void oracle_counters_reset(void) {
    g_keccak_count = 0;
    oracle_g_butterfly_count = 0;
}
uint64_t oracle_counter_keccak(void) { return g_keccak_count; }
uint64_t oracle_counter_butterfly(void) { return oracle_g_butterfly_count; }
