/*
 * Driver that runs the reference's own batched Kyber kernels (Kyber_GPU_Batched, round-2
 * arithmetic, one thread per instance, every intermediate in HBM) compiled by nvcc for sm_103a.
 * It is a measurement baseline and a GPU-side parity check, never part of libpqcgpu: the
 * kernels and orchestration (indcpa_keypair / indcpa_enc / indcpa_dec, Kyber_GPU_Batched/
 * indcpa.cu:474-733) are the reference's, unmodified; this file only allocates their scratch
 * (the poly_set4 of Kyber_GPU_Batched/main.cu:77-97) and exposes them through extern "C".
 *
 * Launch shapes: the reference picks block sizes from a GPU table (indcpa.cu:74-79); the V100
 * column is used, whose block sizes are all powers of two <= 256.  Every entry point requires a
 * count that is a multiple of 256 and <= N_TESTS, so each launched thread maps to an instance and
 * every index stays inside the N_TESTS-sized buffers, including the kernels that do not test
 * X < COUNT.
 *
 * refgpu_cpa_keypair runs indcpa_keypair as the reference does (its in-place sha3_512_n at
 * indcpa.cu:500 lets instance X read other instances' G output, so its keys are only good for
 * timing).  refgpu_cpa_keypair_nist issues the same kernels with G(d) written to a separate
 * buffer and split into rho / sigma per instance, which gives the NIST keys used for parity.
 */
#include <cuda_runtime.h>
#include <stdint.h>
#include <stdlib.h>

#include "fips202.h"
#include "indcpa.h"
#include "poly.h"
#include "polyvec.h"

int SELECTED_GPU = GPU_V100;

__global__ void gen_matrix_n(int COUNT, polyvec *a, unsigned char *seed, int transposed, unsigned char *large_bufA);
__global__ void pack_pk_n(int COUNT, unsigned char *r, polyvec *pk, unsigned char *seed);
__global__ void pack_sk_n(int COUNT, unsigned char *r, polyvec *sk);

extern "C" void refgpu_destroy(void *h);

namespace {
struct RefCtx {
    poly_set4 ps;
    unsigned char *gout, *rho, *sigma;  // NIST keypair: G(d) and its two halves, N_TESTS each
};

bool count_ok(int count) { return count > 0 && count <= N_TESTS && count % 256 == 0; }
}  // namespace

extern "C" int refgpu_k(void) { return KYBER_K; }
extern "C" int refgpu_max_count(void) { return N_TESTS; }

extern "C" void *refgpu_create(void) {
    RefCtx *c = (RefCtx *)calloc(1, sizeof(RefCtx));
    if (!c) return nullptr;
    poly_set4 *p = &c->ps;
    bool ok = true;
    ok &= cudaMalloc(&p->a, sizeof(poly)) == cudaSuccess;
    ok &= cudaMalloc(&p->b, sizeof(poly)) == cudaSuccess;
    ok &= cudaMalloc(&p->c, sizeof(poly)) == cudaSuccess;
    ok &= cudaMalloc(&p->d, sizeof(poly)) == cudaSuccess;
    ok &= cudaMalloc(&p->av, sizeof(polyvec)) == cudaSuccess;
    ok &= cudaMalloc(&p->bv, sizeof(polyvec)) == cudaSuccess;
    ok &= cudaMalloc(&p->cv, sizeof(polyvec)) == cudaSuccess;
    ok &= cudaMalloc(&p->dv, sizeof(polyvec)) == cudaSuccess;
    ok &= cudaMalloc(&p->ev, sizeof(polyvec)) == cudaSuccess;
    ok &= cudaMalloc(&p->fv, sizeof(polyvec)) == cudaSuccess;
    ok &= cudaMalloc(&p->AV, sizeof(polyvec) * 4) == cudaSuccess;
    ok &= cudaMalloc(&p->seed, (size_t)KYBER_SYMBYTES * 2 * N_TESTS) == cudaSuccess;
    ok &= cudaMalloc(&p->large_buffer_a, (size_t)LARGE_BUFFER_SZ * N_TESTS) == cudaSuccess;
    ok &= cudaMalloc(&p->large_buffer_b, (size_t)LARGE_BUFFER_SZ * N_TESTS) == cudaSuccess;
    ok &= cudaMalloc(&c->gout, (size_t)64 * N_TESTS) == cudaSuccess;
    ok &= cudaMalloc(&c->rho, (size_t)32 * N_TESTS) == cudaSuccess;
    ok &= cudaMalloc(&c->sigma, (size_t)32 * N_TESTS) == cudaSuccess;
    if (!ok) {
        refgpu_destroy(c);
        return nullptr;
    }
    return c;
}

extern "C" void refgpu_destroy(void *h) {
    RefCtx *c = (RefCtx *)h;
    if (!c) return;
    poly_set4 *p = &c->ps;
    void *all[] = {p->a, p->b, p->c, p->d, p->av, p->bv, p->cv, p->dv, p->ev, p->fv, p->AV,
                   p->seed, p->large_buffer_a, p->large_buffer_b, c->gout, c->rho, c->sigma};
    for (void *q : all)
        if (q) cudaFree(q);
    free(c);
}

// The reference's indcpa_keypair, unchanged (rng_buf: count * 64 bytes, d in the first 32 of each
// 64, overwritten in place).
extern "C" int refgpu_cpa_keypair(void *h, int count, unsigned char *pk, unsigned char *sk, unsigned char *rng_buf,
                                  cudaStream_t stream) {
    if (!h || !count_ok(count)) return -1;
    indcpa_keypair(count, &((RefCtx *)h)->ps, pk, sk, rng_buf, stream);
    return cudaGetLastError() == cudaSuccess ? 0 : -3;
}

// Same kernels as indcpa_keypair, NIST seed plumbing: (rho, sigma) = G(d) per instance.
extern "C" int refgpu_cpa_keypair_nist(void *h, int count, unsigned char *pk, unsigned char *sk, unsigned char *d,
                                       cudaStream_t stream) {
    if (!h || !count_ok(count)) return -1;
    RefCtx *c = (RefCtx *)h;
    poly_set4 *ps = &c->ps;
    const int b = 256, g = count / b;
    sha3_512_n<<<g, b, 0, stream>>>(count, c->gout, d, 32ULL);
    cudaMemcpy2DAsync(c->rho, 32, c->gout, 64, 32, count, cudaMemcpyDeviceToDevice, stream);
    cudaMemcpy2DAsync(c->sigma, 32, c->gout + 32, 64, 32, count, cudaMemcpyDeviceToDevice, stream);
    polyvec *a = ps->AV, *e = ps->av, *pkpv = ps->bv, *skpv = ps->cv;
    poly *tmp = ps->a;
    unsigned char nonce = 0;
    gen_matrix_n<<<g, b, 0, stream>>>(count, a, c->rho, 0, ps->large_buffer_a);
    for (int i = 0; i < KYBER_K; i++) poly_getnoise<<<g, b, 0, stream>>>(count, skpv->vec + i, c->sigma, nonce++);
    for (int i = 0; i < KYBER_K; i++) poly_getnoise<<<g, b, 0, stream>>>(count, e->vec + i, c->sigma, nonce++);
    polyvec_ntt_n<<<g, b, 0, stream>>>(count, skpv);
    polyvec_ntt_n<<<g, b, 0, stream>>>(count, e);
    for (int i = 0; i < KYBER_K; i++) {
        polyvec_pointwise_acc_n<<<g, b, 0, stream>>>(count, &(pkpv->vec[i]), &(a[i]), skpv, tmp);
        poly_frommont_n<<<g, b, 0, stream>>>(count, &(pkpv->vec[i]));
    }
    polyvec_add_n<<<g, b, 0, stream>>>(count, pkpv, pkpv, e);
    polyvec_reduce_n<<<g, b, 0, stream>>>(count, pkpv);
    pack_sk_n<<<g, b, 0, stream>>>(count, sk, skpv);
    pack_pk_n<<<g, b, 0, stream>>>(count, pk, pkpv, c->rho);
    return cudaGetLastError() == cudaSuccess ? 0 : -3;
}

extern "C" int refgpu_cpa_enc(void *h, int count, unsigned char *ct, unsigned char *m, unsigned char *pk,
                              unsigned char *coins, cudaStream_t stream) {
    if (!h || !count_ok(count)) return -1;
    indcpa_enc(count, &((RefCtx *)h)->ps, ct, m, pk, coins, stream);
    return cudaGetLastError() == cudaSuccess ? 0 : -3;
}

extern "C" int refgpu_cpa_dec(void *h, int count, unsigned char *m, unsigned char *ct, unsigned char *sk,
                              cudaStream_t stream) {
    if (!h || !count_ok(count)) return -1;
    indcpa_dec(count, &((RefCtx *)h)->ps, m, ct, sk, stream);
    return cudaGetLastError() == cudaSuccess ? 0 : -3;
}
