/*
 * Driver around the reference's own NewHope_NIST_GPU device code, compiled for the host via
 * ref_shim/.  TEST INFRASTRUCTURE: it produces golden vectors that pin the CPU oracle.
 *
 * cpapke_enc / cpapke_dec are the reference's functions unchanged (NewHope_NIST_GPU/
 * cpapke.cu:353-476).  The keypair re-sequences the reference's kernels as cpapke_keypair does
 * (cpapke.cu:265-338) but splits SHAKE256(seed, 64) into publicseed / noiseseed per instance at
 * stride 32, instead of reading noiseseed at temp_2 + 32 * N_TESTS (cpapke.cu:283-284), which for
 * batches up to 8192 is memory the preceding kernel never wrote.
 */
#include <stdlib.h>
#include <string.h>
#include "cpapke.h"
#include "fips202.h"
#include "poly.h"

thread_local dim3 threadIdx, blockIdx, blockDim, gridDim;
int SELECTED_GPU = GPU_V100;

__global__ void encode_pk(int COUNT, unsigned char *r, poly *pk, unsigned char *seed);
__global__ void gen_a(int COUNT, poly *a, unsigned char *seed);

void HandleError(cudaError_t err, const char *file, int line) {
    if (err != cudaSuccess) {
        fprintf(stderr, "%s in %s at line %d\n", cudaGetErrorString(err), file, line);
        abort();
    }
}

static void alloc_set(poly_set4 *ps) {
    poly **p[8] = {&ps->a, &ps->b, &ps->c, &ps->d, &ps->e, &ps->f, &ps->g, &ps->h};
    for (int i = 0; i < 8; i++) *p[i] = (poly *)calloc(1, sizeof(poly));
    ps->seed = (unsigned char *)calloc(N_TESTS, 32);
    ps->seed_2x = (unsigned char *)calloc(N_TESTS, 64);
    ps->large_buffer_a = (unsigned char *)calloc(N_TESTS, LARGE_BUFFER_SZ);
}
static void free_set(poly_set4 *ps) {
    poly *p[8] = {ps->a, ps->b, ps->c, ps->d, ps->e, ps->f, ps->g, ps->h};
    for (int i = 0; i < 8; i++) free(p[i]);
    free(ps->seed); free(ps->seed_2x); free(ps->large_buffer_a);
}

extern "C" int ref_newhope_max_count(void) { return N_TESTS; }

extern "C" int ref_newhope_cpa_keypair(int count, unsigned char *pk, unsigned char *sk, const unsigned char *seed) {
    if (count <= 0 || count > N_TESTS) return -1;
    poly_set4 ps;
    alloc_set(&ps);
    const unsigned g = (count + 31) / 32, b = 32;
    unsigned char *in = (unsigned char *)malloc((size_t)count * 32);
    unsigned char *z = (unsigned char *)malloc((size_t)count * 64);
    unsigned char *pub = (unsigned char *)malloc((size_t)count * 32);
    unsigned char *noise = (unsigned char *)malloc((size_t)count * 32);
    memcpy(in, seed, (size_t)count * 32);
    host_launch(g, b, shake256_n, count, z, 64ULL, in, 32ULL, ps.large_buffer_a);
    for (int x = 0; x < count; x++) {
        memcpy(pub + 32 * x, z + 64 * x, 32);
        memcpy(noise + 32 * x, z + 64 * x + 32, 32);
    }
    poly *ahat = ps.a, *ehat = ps.b, *ahat_shat = ps.c, *bhat = ps.d, *shat = ps.e;
    host_launch(g, b, gen_a, count, ahat, pub);
    host_launch(g, b, poly_sample, count, shat, noise, (unsigned char)0);
    host_launch(g, b, poly_ntt, count, shat);
    host_launch(g, b, poly_sample, count, ehat, noise, (unsigned char)1);
    host_launch(g, b, poly_ntt, count, ehat);
    host_launch(g, b, poly_mul_pointwise, count, ahat_shat, shat, ahat);
    host_launch(g, b, poly_add, count, bhat, ehat, ahat_shat);
    host_launch(g, b, poly_tobytes_n, count, sk, shat);
    host_launch(g, b, encode_pk, count, pk, bhat, pub);
    free(in); free(z); free(pub); free(noise);
    free_set(&ps);
    return 0;
}

extern "C" int ref_newhope_cpa_enc(int count, unsigned char *ct, unsigned char *m, unsigned char *pk, unsigned char *coin) {
    if (count <= 0 || count > N_TESTS) return -1;
    poly_set4 ps;
    alloc_set(&ps);
    cpapke_enc(count, &ps, ct, m, pk, coin, 0);
    free_set(&ps);
    return 0;
}

extern "C" int ref_newhope_cpa_dec(int count, unsigned char *m, unsigned char *ct, unsigned char *sk) {
    if (count <= 0 || count > N_TESTS) return -1;
    poly_set4 ps;
    alloc_set(&ps);
    cpapke_dec(count, &ps, m, ct, sk, 0);
    free_set(&ps);
    return 0;
}
