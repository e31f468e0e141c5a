// Kyber kernels instantiated for k = 2, variant 3.
#include "kyber_impl.cuh"
PQC_KYBER_INSTANTIATE(2, 3)
