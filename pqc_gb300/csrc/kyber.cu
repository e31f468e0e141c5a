// Kyber dispatch on (k, variant) and the shared launch-shape table.
#include "pqcgpu_internal.h"

namespace pqc {
namespace kyber {
int g_ni[3][3] = {{16, 16, 16}, {16, 16, 16}, {16, 16, 16}};

#define PQC_KYBER_DECL(K, V)                                                                               \
    int keypair_##K##_##V(int, uint8_t *, uint8_t *, const uint8_t *, int, int, cudaStream_t);            \
    int enc_##K##_##V(int, uint8_t *, uint8_t *, const uint8_t *, const uint8_t *, const uint8_t *, uint8_t *, int, \
                      cudaStream_t);                                                                       \
    int dec_##K##_##V(int, uint8_t *, const uint8_t *, const uint8_t *, uint8_t *, int, cudaStream_t);     \
    int init_##K##_##V();
PQC_KYBER_DECL(2, 3)
PQC_KYBER_DECL(3, 3)
PQC_KYBER_DECL(4, 3)
PQC_KYBER_DECL(2, 2)
PQC_KYBER_DECL(3, 2)
PQC_KYBER_DECL(4, 2)
}  // namespace kyber

#define PQC_KYBER_DISPATCH(FN, ...)                        \
    switch (variant * 10 + k) {                            \
    case 32: return kyber::FN##_2_3(__VA_ARGS__);          \
    case 33: return kyber::FN##_3_3(__VA_ARGS__);          \
    case 34: return kyber::FN##_4_3(__VA_ARGS__);          \
    case 22: return kyber::FN##_2_2(__VA_ARGS__);          \
    case 23: return kyber::FN##_3_2(__VA_ARGS__);          \
    case 24: return kyber::FN##_4_2(__VA_ARGS__);          \
    default: return PQCGPU_EINVAL;                         \
    }

int kyber_keypair_dev(int variant, int k, int n, uint8_t *pk, uint8_t *sk, const uint8_t *coins, int coins_stride,
                      int kem, cudaStream_t st) {
    PQC_KYBER_DISPATCH(keypair, n, pk, sk, coins, coins_stride, kem, st)
}
int kyber_enc_dev(int variant, int k, int n, uint8_t *ct, uint8_t *ss, const uint8_t *pk, const uint8_t *m,
                  const uint8_t *coins, uint8_t *scratch, int kem, cudaStream_t st) {
    PQC_KYBER_DISPATCH(enc, n, ct, ss, pk, m, coins, scratch, kem, st)
}
int kyber_dec_dev(int variant, int k, int n, uint8_t *out, const uint8_t *ct, const uint8_t *sk, uint8_t *scratch,
                  int kem, cudaStream_t st) {
    PQC_KYBER_DISPATCH(dec, n, out, ct, sk, scratch, kem, st)
}
int kyber_init_constants() {
    int (*inits[])() = {kyber::init_2_3, kyber::init_3_3, kyber::init_4_3,
                        kyber::init_2_2, kyber::init_3_2, kyber::init_4_2};
    for (auto f : inits) {
        const int rc = f();
        if (rc) return rc;
    }
    return PQCGPU_OK;
}
void kyber_set_ni(int op, int k, int ni) {
    if (op >= 0 && op < 3 && k >= 2 && k <= 4 && ni > 0) kyber::g_ni[op][k - 2] = ni;
}
int kyber_get_ni(int op, int k) { return (op >= 0 && op < 3 && k >= 2 && k <= 4) ? kyber::g_ni[op][k - 2] : -1; }

}  // namespace pqc
