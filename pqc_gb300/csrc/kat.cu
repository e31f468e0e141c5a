// NIST known-answer-test randomness: AES-256 CTR_DRBG without a derivation function
// (SP 800-90A section 10.2.1, instantiated as in the NIST PQC KAT generator's randombytes),
// selectable as the library DRBG so that the single-instance crypto_kem_* entry points and the KAT
// harness (pqc_gb300/kat.py) draw the same coins, in the same calls, as a NIST submission package.
//
// Host code only.  AES-256 follows FIPS 197 directly: the S-box is computed at first use from the
// multiplicative inverse in GF(2^8) and the affine map, the key schedule uses Nk = 8, Nr = 14.
#include <stdint.h>
#include <string.h>

#include <mutex>

#include "pqcgpu_internal.h"

namespace pqc {
namespace {

uint8_t g_sbox[256];
std::once_flag g_sbox_once;

uint8_t gf_mul(uint8_t a, uint8_t b) {
    uint8_t r = 0;
    while (b) {
        if (b & 1) r ^= a;
        a = (uint8_t)((a << 1) ^ ((a & 0x80) ? 0x1b : 0));
        b >>= 1;
    }
    return r;
}

void build_sbox() {
    for (int x = 0; x < 256; x++) {
        uint8_t inv = 0;  // 0 maps to 0; otherwise the unique y with x * y = 1
        if (x)
            for (int y = 1; y < 256; y++)
                if (gf_mul((uint8_t)x, (uint8_t)y) == 1) {
                    inv = (uint8_t)y;
                    break;
                }
        uint8_t s = inv;  // affine map: b ^ rotl(b,1) ^ rotl(b,2) ^ rotl(b,3) ^ rotl(b,4) ^ 0x63
        for (int r = 1; r <= 4; r++) s ^= (uint8_t)((inv << r) | (inv >> (8 - r)));
        g_sbox[x] = (uint8_t)(s ^ 0x63);
    }
}

struct Aes256 {
    uint8_t rk[15][16];
    explicit Aes256(const uint8_t key[32]) {
        std::call_once(g_sbox_once, build_sbox);
        uint8_t w[60][4];
        for (int i = 0; i < 8; i++) memcpy(w[i], key + 4 * i, 4);
        uint8_t rcon = 1;
        for (int i = 8; i < 60; i++) {
            uint8_t t[4];
            memcpy(t, w[i - 1], 4);
            if (i % 8 == 0) {
                const uint8_t t0 = t[0];
                t[0] = (uint8_t)(g_sbox[t[1]] ^ rcon);
                t[1] = g_sbox[t[2]];
                t[2] = g_sbox[t[3]];
                t[3] = g_sbox[t0];
                rcon = gf_mul(rcon, 2);
            } else if (i % 8 == 4) {
                for (int j = 0; j < 4; j++) t[j] = g_sbox[t[j]];
            }
            for (int j = 0; j < 4; j++) w[i][j] = (uint8_t)(w[i - 8][j] ^ t[j]);
        }
        for (int r = 0; r < 15; r++)
            for (int c = 0; c < 4; c++) memcpy(rk[r] + 4 * c, w[4 * r + c], 4);
    }
    // state byte (row r, column c) at s[4c + r]
    void encrypt(uint8_t out[16], const uint8_t in[16]) const {
        uint8_t s[16];
        for (int i = 0; i < 16; i++) s[i] = (uint8_t)(in[i] ^ rk[0][i]);
        for (int round = 1; round <= 14; round++) {
            uint8_t t[16];
            for (int c = 0; c < 4; c++)  // SubBytes + ShiftRows: row r moves left by r
                for (int r = 0; r < 4; r++) t[4 * c + r] = g_sbox[s[4 * ((c + r) & 3) + r]];
            if (round != 14)
                for (int c = 0; c < 4; c++) {  // MixColumns
                    const uint8_t a0 = t[4 * c], a1 = t[4 * c + 1], a2 = t[4 * c + 2], a3 = t[4 * c + 3];
                    t[4 * c] = (uint8_t)(gf_mul(a0, 2) ^ gf_mul(a1, 3) ^ a2 ^ a3);
                    t[4 * c + 1] = (uint8_t)(a0 ^ gf_mul(a1, 2) ^ gf_mul(a2, 3) ^ a3);
                    t[4 * c + 2] = (uint8_t)(a0 ^ a1 ^ gf_mul(a2, 2) ^ gf_mul(a3, 3));
                    t[4 * c + 3] = (uint8_t)(gf_mul(a0, 3) ^ a1 ^ a2 ^ gf_mul(a3, 2));
                }
            for (int i = 0; i < 16; i++) s[i] = (uint8_t)(t[i] ^ rk[round][i]);
        }
        memcpy(out, s, 16);
    }
};

void incr_be(uint8_t v[16]) {
    for (int i = 15; i >= 0; i--)
        if (++v[i]) break;
}

}  // namespace

// CTR_DRBG state (SP 800-90A 10.2.1): Key (32), V (16); seedlen = 48.
void CtrDrbg::update(const uint8_t *provided) {
    const Aes256 aes(key);
    uint8_t temp[48];
    for (int i = 0; i < 3; i++) {
        incr_be(v);
        aes.encrypt(temp + 16 * i, v);
    }
    if (provided)
        for (int i = 0; i < 48; i++) temp[i] ^= provided[i];
    memcpy(key, temp, 32);
    memcpy(v, temp + 32, 16);
}

void CtrDrbg::instantiate(const uint8_t entropy[48], const uint8_t *personalization) {
    uint8_t seed[48];
    memcpy(seed, entropy, 48);
    if (personalization)
        for (int i = 0; i < 48; i++) seed[i] ^= personalization[i];
    memset(key, 0, sizeof key);
    memset(v, 0, sizeof v);
    update(seed);
    reseed_counter = 1;
}

void CtrDrbg::generate(uint8_t *out, size_t n) {
    const Aes256 aes(key);
    uint8_t block[16];
    while (n) {
        incr_be(v);
        aes.encrypt(block, v);
        const size_t take = n < 16 ? n : 16;
        memcpy(out, block, take);
        out += take;
        n -= take;
    }
    update(nullptr);
    reseed_counter++;
}

}  // namespace pqc
