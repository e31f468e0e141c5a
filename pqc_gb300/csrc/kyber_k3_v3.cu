// Kyber kernels instantiated for k = 3, variant 3.
#include "kyber_impl.cuh"
PQC_KYBER_INSTANTIATE(3, 3)
