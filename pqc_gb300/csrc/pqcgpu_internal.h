// Internal interfaces between the C ABI layer (capi.cu) and the kernel translation units.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <atomic>

#include "pqcgpu.h"

namespace pqc {

// Kernel launches issued by this library (all contexts); contexts report deltas.
extern std::atomic<uint64_t> g_launch_count;

// ---- Kyber (kyber.cu) ----
int kyber_init_constants();
// op: 0 keypair, 1 enc, 2 dec.  ni = instances per CTA of the core kernel.
void kyber_set_ni(int op, int k, int ni);
int kyber_get_ni(int op, int k);
// coins: d (CPA) or d||z (KEM) at `coins_stride`.  kem=1 writes the full KEM secret key.
int kyber_keypair_dev(int variant, int k, int n, uint8_t *pk, uint8_t *sk, const uint8_t *coins, int coins_stride,
                      int kem, cudaStream_t st);
// kem=1: coins 32 B/instance, scratch >= 96 B/instance, m ignored.  kem=0: CPA enc with m, coins.
int kyber_enc_dev(int variant, int k, int n, uint8_t *ct, uint8_t *ss, const uint8_t *pk, const uint8_t *m,
                  const uint8_t *coins, uint8_t *scratch, int kem, cudaStream_t st);
// kem=1: out = ss, scratch >= 32 B/instance.  kem=0: out = m (CPA decryption).
int kyber_dec_dev(int variant, int k, int n, uint8_t *out, const uint8_t *ct, const uint8_t *sk, uint8_t *scratch,
                  int kem, cudaStream_t st);

}  // namespace pqc
