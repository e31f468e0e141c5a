"""The reference's own batched Kyber kernels, compiled for sm_103a (baseline/_ref, built by
baseline/build_ref_gpu.sh), against this library on the same GPU: round-2 CPA keypair (NIST seed
plumbing), encryption and decryption, byte for byte, for k = 3 and k = 4."""
import os
import sys

import pytest

from conftest import ROOT
from pqc_gb300 import drbg

pytestmark = pytest.mark.gpu
sys.path.insert(0, os.path.join(ROOT, "baseline"))


@pytest.mark.parametrize("k", [3, 4])
@pytest.mark.parametrize("n", [256, 1280])
def test_reference_kernels_match_library(k, n):
    import refgpu
    if not refgpu.available(k):
        pytest.skip("reference kernels not built (baseline/build_ref_gpu.sh found no staged sources)")
    import ctypes

    import torch
    from pqc_gb300 import kem
    dev = torch.device("cuda:0")
    seed = drbg.seed48(7000 + 10 * n + k)

    def t(label, nbytes):
        return torch.frombuffer(bytearray(drbg.stream(seed, label, nbytes)), dtype=torch.uint8).to(dev)

    s = kem.kyber_cpa_sizes(2, k)
    d, m, coins = t(b"d", 32 * n), t(b"m", 32 * n), t(b"coins", 32 * n)
    ctx = kem.Context(0)
    ref = refgpu.RefGPU(k)
    try:
        stream = torch.cuda.Stream()
        ctx.set_stream(stream.cuda_stream)
        sh = ctypes.c_void_p(stream.cuda_stream)
        pk_r, sk_r, ct_r, m_r = (torch.zeros(n * x, dtype=torch.uint8, device=dev) for x in (s["pk"], s["sk"], s["ct"], 32))
        pk_o, sk_o, ct_o, m_o = (torch.zeros(n * x, dtype=torch.uint8, device=dev) for x in (s["pk"], s["sk"], s["ct"], 32))
        torch.cuda.synchronize()
        ref.keypair_nist(n, pk_r, sk_r, d, sh)
        ref.enc(n, ct_r, m, pk_r, coins, sh)
        ref.dec(n, m_r, ct_r, sk_r, sh)
        lib, P = ctx.lib, (lambda x: ctypes.c_void_p(x.data_ptr()))
        F = kem.DEVICE_PTRS
        assert lib.pqcgpu_kyber_indcpa_keypair_batch(ctx.h, 2, k, n, P(pk_o), P(sk_o), P(d), F) == 0
        assert lib.pqcgpu_kyber_indcpa_enc_batch(ctx.h, 2, k, n, P(ct_o), P(m), P(pk_o), P(coins), F) == 0
        assert lib.pqcgpu_kyber_indcpa_dec_batch(ctx.h, 2, k, n, P(m_o), P(ct_o), P(sk_o), F) == 0
        stream.synchronize()
        assert torch.equal(pk_r, pk_o)
        assert torch.equal(sk_r, sk_o)
        assert torch.equal(ct_r, ct_o)
        assert torch.equal(m_r, m)
        assert torch.equal(m_o, m)
    finally:
        ref.close()
        ctx.close()
