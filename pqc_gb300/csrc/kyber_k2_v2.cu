// Kyber kernels instantiated for k = 2, variant 2.
#include "kyber_impl.cuh"
PQC_KYBER_INSTANTIATE(2, 2)
