// Kyber kernels instantiated for k = 3, variant 2.
#include "kyber_impl.cuh"
PQC_KYBER_INSTANTIATE(3, 2)
