/*
 * Batched drivers over the CPU oracle (OpenMP across instances) -- TEST INFRASTRUCTURE.
 * Used by the tests as the checker and by the benchmark's CPU-baseline leg; the instance-major
 * layout (instance i at offset i * size) is the one the product's C ABI uses.
 */
#include <omp.h>
#include "oracle.h"

int oracle_alg_sizes(int alg, size_t *pk, size_t *sk, size_t *ct, size_t *ss, size_t *kp_coins, size_t *enc_coins) {
    size_t a = 0, b = 0, c = 0, d = 32, e = 64, f = 32;
    switch (alg) {
    case 0: case 1: case 2:
        oracle_kyber_sizes(3, alg + 2, &a, 0, &b, &c);
        break;
    case 3:
        oracle_kyber_sizes(2, 4, &a, 0, &b, &c);
        break;
    case 4:
        a = 1824; b = 1792; c = 2176; e = 32;
        break;
    case 5:
        a = 15632; b = 31296; c = 15744; d = 24; e = 64; f = 24;
        break;
    case 6: case 7: case 8:
        oracle_kyber_sizes(3, alg - 4, &a, 0, &b, &c);
        break;
    case 9:
        a = 928; b = 896; c = 1088; e = 32;
        break;
    case 10:
        a = 9616; b = 19888; c = 9720; d = 16; e = 48; f = 16;
        break;
    case 11:
        a = 21520; b = 43088; c = 21632; d = 32; e = 80; f = 32;
        break;
    default:
        return -1;
    }
    if (pk) *pk = a;
    if (sk) *sk = b;
    if (ct) *ct = c;
    if (ss) *ss = d;
    if (kp_coins) *kp_coins = e;
    if (enc_coins) *enc_coins = f;
    return 0;
}

static int one_keypair(int alg, uint8_t *pk, uint8_t *sk, const uint8_t *coins) {
    if (alg <= 2) return oracle_kyber_kem_keypair(3, alg + 2, pk, sk, coins);
    if (alg == 3) return oracle_kyber_kem_keypair(2, 4, pk, sk, coins);
    if (alg == 4) return oracle_newhope_kem_keypair(pk, sk, coins);
    if (alg == 9) return oracle_newhope512_kem_keypair(pk, sk, coins);
    if (alg == 10) return oracle_frodo640_kem_keypair(pk, sk, coins);
    if (alg == 11) return oracle_frodo1344_kem_keypair(pk, sk, coins);
    if (alg >= 6) return oracle_mlkem_keypair(alg - 4, pk, sk, coins);
    return oracle_frodo_kem_keypair(pk, sk, coins);
}
static int one_enc(int alg, uint8_t *ct, uint8_t *ss, const uint8_t *pk, const uint8_t *coins) {
    if (alg <= 2) return oracle_kyber_kem_enc(3, alg + 2, ct, ss, pk, coins);
    if (alg == 3) return oracle_kyber_kem_enc(2, 4, ct, ss, pk, coins);
    if (alg == 4) return oracle_newhope_kem_enc(ct, ss, pk, coins);
    if (alg == 9) return oracle_newhope512_kem_enc(ct, ss, pk, coins);
    if (alg == 10) return oracle_frodo640_kem_enc(ct, ss, pk, coins);
    if (alg == 11) return oracle_frodo1344_kem_enc(ct, ss, pk, coins);
    if (alg >= 6) return oracle_mlkem_enc(alg - 4, ct, ss, pk, coins);
    return oracle_frodo_kem_enc(ct, ss, pk, coins);
}
static int one_dec(int alg, uint8_t *ss, const uint8_t *ct, const uint8_t *sk) {
    if (alg <= 2) return oracle_kyber_kem_dec(3, alg + 2, ss, ct, sk);
    if (alg == 3) return oracle_kyber_kem_dec(2, 4, ss, ct, sk);
    if (alg == 4) return oracle_newhope_kem_dec(ss, ct, sk);
    if (alg == 9) return oracle_newhope512_kem_dec(ss, ct, sk);
    if (alg == 10) return oracle_frodo640_kem_dec(ss, ct, sk);
    if (alg == 11) return oracle_frodo1344_kem_dec(ss, ct, sk);
    if (alg >= 6) return oracle_mlkem_dec(alg - 4, ss, ct, sk);
    return oracle_frodo_kem_dec(ss, ct, sk);
}

int oracle_batch_keypair(int alg, size_t n, uint8_t *pk, uint8_t *sk, const uint8_t *coins, int nthreads) {
    size_t P, S, C, SS, KC, EC;
    if (oracle_alg_sizes(alg, &P, &S, &C, &SS, &KC, &EC)) return -1;
    if (nthreads <= 0) nthreads = omp_get_num_procs();
#pragma omp parallel for schedule(dynamic, 16) num_threads(nthreads)
    for (long i = 0; i < (long)n; i++) one_keypair(alg, pk + i * P, sk + i * S, coins + i * KC);
    return 0;
}
int oracle_batch_enc(int alg, size_t n, uint8_t *ct, uint8_t *ss, const uint8_t *pk, const uint8_t *coins,
                     int nthreads) {
    size_t P, S, C, SS, KC, EC;
    if (oracle_alg_sizes(alg, &P, &S, &C, &SS, &KC, &EC)) return -1;
    if (nthreads <= 0) nthreads = omp_get_num_procs();
#pragma omp parallel for schedule(dynamic, 16) num_threads(nthreads)
    for (long i = 0; i < (long)n; i++) one_enc(alg, ct + i * C, ss + i * SS, pk + i * P, coins + i * EC);
    return 0;
}
int oracle_batch_dec(int alg, size_t n, uint8_t *ss, const uint8_t *ct, const uint8_t *sk, int nthreads) {
    size_t P, S, C, SS, KC, EC;
    if (oracle_alg_sizes(alg, &P, &S, &C, &SS, &KC, &EC)) return -1;
    if (nthreads <= 0) nthreads = omp_get_num_procs();
#pragma omp parallel for schedule(dynamic, 16) num_threads(nthreads)
    for (long i = 0; i < (long)n; i++) one_dec(alg, ss + i * SS, ct + i * C, sk + i * S);
    return 0;
}
