// Kyber kernels instantiated for k = 4, variant 2.
#include "kyber_impl.cuh"
PQC_KYBER_INSTANTIATE(4, 2)
