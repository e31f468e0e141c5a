/*
 * Glue for host-compiling the reference's NewHope_NIST_GPU with NEWHOPE_N = 512 -- TEST
 * INFRASTRUCTURE.  For n = 512 the reference defines only the scalar transform
 * `void ntt(uint16_t *a, const uint16_t *omega)` (NewHope_NIST_GPU/ntt.cu:143-181), while
 * poly_ntt / poly_invntt (poly.cu:519-547) call the batched `ntt(poly *, const uint16_t *)`
 * declared in ntt.h:17, which exists only for n = 1024.  This file supplies the batched form as
 * the reference's own scalar transform applied to the calling virtual thread's instance:
 * gather its coefficients, call the reference's ntt, scatter them back.
 */
#include "ntt.h"

void ntt(uint16_t *a, const uint16_t *omega);  // the reference's n = 512 transform

void ntt(poly *p, const uint16_t *omega) {
    const int X = threadIdx.x + blockIdx.x * blockDim.x;
    uint16_t a[NEWHOPE_N];
    for (int i = 0; i < NEWHOPE_N; i++) a[i] = p->coeffs[i].threads[X];
    ntt(a, omega);
    for (int i = 0; i < NEWHOPE_N; i++) p->coeffs[i].threads[X] = a[i];
}
