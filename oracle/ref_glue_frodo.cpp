/*
 * FrodoKEM-976 as the reference computes it, on the CPU -- TEST INFRASTRUCTURE ONLY.
 *
 * The reference's host KEM flow (FrodoKEM_GPU/kem.c:13-214) calls the FrodoKEM matrix functions
 * in their host form (frodo_mul_add_as_plus_e, frodo_mul_bs, frodo_key_encode, ...), which the
 * reference tree does not define: it has only their kernel form (FrodoKEM_GPU/
 * frodo_macrify_reference.cu).  Each function below runs the reference's kernel with the launch
 * shape the reference's GPU flow gives it (frodo976.cu:356-361, 572-576; the two big products
 * through the reference's own frodo_mul_add_as_plus_e_gpu / frodo_mul_add_sa_plus_e_gpu, which
 * generate A with generateMatA2 and multiply with matMulKernelTile / matMulKernelSA).  Kernels
 * run through ref_shim_sync, whose CTAs have real __syncthreads barriers.  The sampler
 * (noise.c), pack / unpack (util.cu) and SHAKE256 (fips202.cu) are the reference's host code.
 *
 * kem.c draws its randomness with randombytes(); here randombytes() hands out the coins the
 * caller passed: keypair s || seedSE || z (64 bytes), encapsulation mu (24 bytes) -- the layout
 * of the batched API's coin buffers.
 */
#include <stdlib.h>
#include <string.h>

#include "api.h"
#include "fips202.h"
#include "frodo_macrify.h"
#include "params.h"
#include "random.h"

thread_local dim3 threadIdx, blockIdx, blockDim, gridDim;
thread_local std::barrier<> *pqc_shim_cta_barrier = nullptr;

// FrodoKEM-976's CDF table as the reference defines it (frodo976.cu:21), staged by build_ref.sh
#include "ref_cdf_table.h"

int crypto_kem_keypair(unsigned char *pk, unsigned char *sk);
int crypto_kem_enc(unsigned char *ct, unsigned char *ss, const unsigned char *pk);
int crypto_kem_dec(unsigned char *ss, const unsigned char *ct, const unsigned char *sk);

static thread_local const unsigned char *g_coins = nullptr;
static thread_local unsigned int g_coins_left = 0;

int randombytes(unsigned char *out, unsigned int nbytes) {
    if (nbytes > g_coins_left) return -1;
    memcpy(out, g_coins, nbytes);
    g_coins += nbytes;
    g_coins_left -= nbytes;
    return 0;
}

void frodo_mul_add_as_plus_e(uint16_t *out, const uint16_t *s, const uint16_t *e, const uint8_t *seed_A) {
    uint16_t *A = (uint16_t *)malloc(sizeof(uint16_t) * PARAMS_N * PARAMS_N);
    frodo_mul_add_as_plus_e_gpu(out, (uint16_t *)s, (uint16_t *)e, seed_A, A);
    free(A);
}
void frodo_mul_add_sa_plus_e(uint16_t *out, const uint16_t *s, const uint16_t *e, const uint8_t *seed_A) {
    uint16_t *A = (uint16_t *)malloc(sizeof(uint16_t) * PARAMS_N * PARAMS_N);
    frodo_mul_add_sa_plus_e_gpu(out, (uint16_t *)s, (uint16_t *)e, seed_A, A);
    free(A);
}
void frodo_mul_add_sb_plus_e(uint16_t *out, const uint16_t *b, const uint16_t *s, const uint16_t *e) {
    host_launch(8, 8, frodo_mul_add_sb_plus_e_kernel, out, (uint16_t *)b, (uint16_t *)s, (uint16_t *)e);
}
void frodo_mul_bs(uint16_t *out, const uint16_t *b, const uint16_t *s) {
    host_launch(8, 8, frodo_mul_bs_kernel, out, (uint16_t *)b, (uint16_t *)s);
}
void frodo_add(uint16_t *out, const uint16_t *a, const uint16_t *b) {
    host_launch(8, 8, frodo_add_kernel, out, (uint16_t *)a, (uint16_t *)b);
}
void frodo_sub(uint16_t *out, const uint16_t *a, const uint16_t *b) {
    host_launch(8, 8, frodo_sub_kernel, out, (uint16_t *)a, (uint16_t *)b);
}
void frodo_key_encode(uint16_t *out, const uint16_t *in) {
    host_launch(1, 8, frodo_key_encode_kernel, out, (uint16_t *)in);
}
void frodo_key_decode(uint16_t *out, const uint16_t *in) {
    host_launch(1, 8, frodo_key_decode_kernel, out, (uint16_t *)in);
}

extern "C" int ref_frodo976_keypair(unsigned char *pk, unsigned char *sk, const unsigned char *coins) {
    g_coins = coins;
    g_coins_left = 2 * CRYPTO_BYTES + BYTES_SEED_A;
    return crypto_kem_keypair(pk, sk);
}
extern "C" int ref_frodo976_enc(unsigned char *ct, unsigned char *ss, const unsigned char *pk, const unsigned char *mu) {
    g_coins = mu;
    g_coins_left = BYTES_MU;
    return crypto_kem_enc(ct, ss, pk);
}
extern "C" int ref_frodo976_dec(unsigned char *ss, const unsigned char *ct, const unsigned char *sk) {
    return crypto_kem_dec(ss, ct, sk);
}
