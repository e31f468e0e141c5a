/*
 * CPU oracle for the batched KEM path -- TEST INFRASTRUCTURE ONLY.
 *
 * This library restates, in plain C, the algorithms the reference implements on the GPU:
 * Keccak / FIPS-202, Kyber (round-2 variant as coded in the reference, and the round-3
 * parameter sets), NewHope-1024 CPA-PKE + CPA-KEM and FrodoKEM-976 (SHAKE).  It is the checker
 * for the CUDA path: only tests, the smoke check and the CPU-baseline leg of the benchmark
 * load it.  The product library (libpqcgpu) never links or calls it.
 *
 * Parity status:
 *   - Keccak family: pinned against Python hashlib (tests/golden/keccak.json).
 *   - Kyber round-2 CPA (k = 2, 3, 4) and NewHope-1024 / -512 CPA: pinned against golden vectors
 *     produced by the reference's own device code compiled for the host (oracle/build_ref.sh,
 *     tests/golden/ref_*.json).
 *   - FrodoKEM-976: pinned against the reference's own host KEM flow (FrodoKEM_GPU/kem.c) run with
 *     the reference's sampler, pack / unpack, SHAKE, A generation and matrix kernels
 *     (oracle/ref_glue_frodo.cpp, tests/golden/ref_frodo976_kem.json).
 *   - ML-KEM-768 / -1024 (FIPS 203): pinned against an independent implementation, the
 *     `cryptography` package (tests/golden/gen_fips203.py); this also pins the K-PKE arithmetic
 *     that round-3 Kyber shares with ML-KEM.
 *   - Round-3 Kyber's KEM hash layer, ML-KEM-512, NewHope CPA-KEM and FrodoKEM-640 / -1344:
 *     restated from the published algorithms; parity unpinned by outputs of other code (the
 *     reference tree has no code or KAT files for them).
 */
#ifndef PQC_ORACLE_H
#define PQC_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- FIPS-202 ------------------------------------------------------------------------ */
void oracle_keccakf1600(uint64_t s[25]);
void oracle_shake128(uint8_t *out, size_t outlen, const uint8_t *in, size_t inlen);
void oracle_shake256(uint8_t *out, size_t outlen, const uint8_t *in, size_t inlen);
void oracle_sha3_256(uint8_t out[32], const uint8_t *in, size_t inlen);
void oracle_sha3_512(uint8_t out[64], const uint8_t *in, size_t inlen);

/* Work counters (Keccak permutations, NTT butterflies) accumulated per calling thread. */
void oracle_counters_reset(void);
uint64_t oracle_counter_keccak(void);
uint64_t oracle_counter_butterfly(void);

/* ---- Kyber ----------------------------------------------------------------------------
 * variant 2: round-2 semantics as coded in Kyber_GPU_Batched (eta = 2, 16-bit 19q rejection,
 *            du = 11, dv = 5; only k = 4 is meaningful, as in the reference).
 * variant 3: round-3 parameter sets (k = 2: eta1 = 3; du/dv 10/4 for k = 2,3 and 11/5 for k = 4).
 */
int oracle_kyber_sizes(int variant, int k, size_t *pk, size_t *sk_cpa, size_t *sk, size_t *ct);
int oracle_kyber_indcpa_keypair(int variant, int k, uint8_t *pk, uint8_t *sk, const uint8_t d[32]);
int oracle_kyber_indcpa_enc(int variant, int k, uint8_t *ct, const uint8_t m[32], const uint8_t *pk,
                            const uint8_t coins[32]);
int oracle_kyber_indcpa_dec(int variant, int k, uint8_t m[32], const uint8_t *ct, const uint8_t *sk);
int oracle_kyber_kem_keypair(int variant, int k, uint8_t *pk, uint8_t *sk, const uint8_t coins[64]);
int oracle_kyber_kem_enc(int variant, int k, uint8_t *ct, uint8_t ss[32], const uint8_t *pk,
                         const uint8_t coins[32]);
int oracle_kyber_kem_dec(int variant, int k, uint8_t ss[32], const uint8_t *ct, const uint8_t *sk);
/* ML-KEM (FIPS 203), k = 2, 3, 4: coins = d || z (keypair), m (encapsulation) */
int oracle_mlkem_keypair(int k, uint8_t *pk, uint8_t *sk, const uint8_t coins[64]);
int oracle_mlkem_enc(int k, uint8_t *ct, uint8_t ss[32], const uint8_t *pk, const uint8_t m[32]);
int oracle_mlkem_dec(int k, uint8_t ss[32], const uint8_t *ct, const uint8_t *sk);

/* ---- NewHope-1024 (oracle_newhope_*) and NewHope-512 (oracle_newhope512_*) -------------- */
int oracle_newhope_cpapke_keypair(uint8_t *pk, uint8_t *sk, const uint8_t seed[32]);
int oracle_newhope_cpapke_enc(uint8_t *ct, const uint8_t m[32], const uint8_t *pk, const uint8_t coin[32]);
int oracle_newhope_cpapke_dec(uint8_t m[32], const uint8_t *ct, const uint8_t *sk);
int oracle_newhope_kem_keypair(uint8_t *pk, uint8_t *sk, const uint8_t coins[32]);
int oracle_newhope_kem_enc(uint8_t *ct, uint8_t ss[32], const uint8_t *pk, const uint8_t coins[32]);
int oracle_newhope_kem_dec(uint8_t ss[32], const uint8_t *ct, const uint8_t *sk);
int oracle_newhope512_cpapke_keypair(uint8_t *pk, uint8_t *sk, const uint8_t seed[32]);
int oracle_newhope512_cpapke_enc(uint8_t *ct, const uint8_t m[32], const uint8_t *pk, const uint8_t coin[32]);
int oracle_newhope512_cpapke_dec(uint8_t m[32], const uint8_t *ct, const uint8_t *sk);
int oracle_newhope512_kem_keypair(uint8_t *pk, uint8_t *sk, const uint8_t coins[32]);
int oracle_newhope512_kem_enc(uint8_t *ct, uint8_t ss[32], const uint8_t *pk, const uint8_t coins[32]);
int oracle_newhope512_kem_dec(uint8_t ss[32], const uint8_t *ct, const uint8_t *sk);

/* ---- FrodoKEM-976 (oracle_frodo_*), -640 and -1344 (SHAKE) ------------------------------
 * keypair coins = s || seedSE || z (2 ss + 16 bytes), encapsulation coins = mu (ss bytes), with
 * ss = 24 / 16 / 32 bytes for n = 976 / 640 / 1344 */
int oracle_frodo_kem_keypair(uint8_t *pk, uint8_t *sk, const uint8_t *coins);
int oracle_frodo_kem_enc(uint8_t *ct, uint8_t *ss, const uint8_t *pk, const uint8_t *coins);
int oracle_frodo_kem_dec(uint8_t *ss, const uint8_t *ct, const uint8_t *sk);
int oracle_frodo640_kem_keypair(uint8_t *pk, uint8_t *sk, const uint8_t *coins);
int oracle_frodo640_kem_enc(uint8_t *ct, uint8_t *ss, const uint8_t *pk, const uint8_t *coins);
int oracle_frodo640_kem_dec(uint8_t *ss, const uint8_t *ct, const uint8_t *sk);
int oracle_frodo1344_kem_keypair(uint8_t *pk, uint8_t *sk, const uint8_t *coins);
int oracle_frodo1344_kem_enc(uint8_t *ct, uint8_t *ss, const uint8_t *pk, const uint8_t *coins);
int oracle_frodo1344_kem_dec(uint8_t *ss, const uint8_t *ct, const uint8_t *sk);

/* ---- Batched drivers (OpenMP over instances; nthreads <= 0 means all cores) -------------
 * alg: 0..2 = Kyber-512/768/1024 (round 3), 3 = Kyber-1024 round 2, 4 = NewHope-1024 CPA-KEM,
 * 5 = FrodoKEM-976, 6..8 = ML-KEM-512/768/1024 (FIPS 203), 9 = NewHope-512 CPA-KEM,
 * 10 = FrodoKEM-640, 11 = FrodoKEM-1344.
 * Buffers are instance-major, each instance at a fixed stride. */
int oracle_batch_keypair(int alg, size_t n, uint8_t *pk, uint8_t *sk, const uint8_t *coins, int nthreads);
int oracle_batch_enc(int alg, size_t n, uint8_t *ct, uint8_t *ss, const uint8_t *pk, const uint8_t *coins,
                     int nthreads);
int oracle_batch_dec(int alg, size_t n, uint8_t *ss, const uint8_t *ct, const uint8_t *sk, int nthreads);
int oracle_alg_sizes(int alg, size_t *pk, size_t *sk, size_t *ct, size_t *ss, size_t *kp_coins,
                     size_t *enc_coins);

#ifdef __cplusplus
}
#endif
#endif
