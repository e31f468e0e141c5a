"""The encapsulation entry point that allocates nothing (pqcgpu_kem_enc_batch_noalloc).

It serves callers that cannot call cudaMalloc -- code running inside another framework's memory
pool or allocator callback, plugins handed fixed device buffers, real-time paths that forbid
allocation after start-up.  Its scratch is a fixed device array shared by all calls.  This test
calls it through the C ABI several times in a row -- batches above 1024 instances (thread-per-
instance hash kernels) and at or below it (warp-per-instance hash kernels, 1000 and 1) -- and checks
each result byte for byte against the regular batched encapsulation.  It runs last (file name) and
needs a GPU.
"""
import ctypes

import pytest

from pqc_gb300 import drbg

pytestmark = pytest.mark.gpu


def test_noalloc_encaps_matches_batched_encaps():
    import torch
    from pqc_gb300 import _lib, kem
    lib = _lib.load()
    dev = torch.device("cuda:0")
    torch.cuda.set_device(dev)
    alg = "kyber768"
    s = kem.sizes(alg)
    ctx = kem.Context(0)
    seed = drbg.seed48(2024)
    nmax = 5000
    up = lambda b: torch.frombuffer(bytearray(b), dtype=torch.uint8).to(dev)
    kc = up(drbg.stream(seed, b"kp", nmax * s["kp_coins"]))
    pk = torch.empty(nmax * s["pk"], dtype=torch.uint8, device=dev)
    sk = torch.empty(nmax * s["sk"], dtype=torch.uint8, device=dev)
    torch.cuda.synchronize()
    ctx.keypair_dev(alg, nmax, pk, sk, kc)
    ctx.wait()
    stream = torch.cuda.current_stream(dev)
    p = lambda t: ctypes.c_void_p(t.data_ptr())
    for call, n in enumerate((nmax, 1234, 1000, 1)):  # calls in a row share the scratch array
        coins = up(drbg.stream(seed, b"enc%d" % call, n * s["enc_coins"]))
        ct = torch.empty(n * s["ct"], dtype=torch.uint8, device=dev)
        ss = torch.empty(n * s["ss"], dtype=torch.uint8, device=dev)
        ct_ref, ss_ref = torch.empty_like(ct), torch.empty_like(ss)
        torch.cuda.synchronize()
        rc = lib.pqcgpu_kem_enc_batch_noalloc(kem.alg_id(alg), n, p(ct), p(ss), p(pk), p(coins),
                                              ctypes.c_void_p(stream.cuda_stream))
        assert rc == 0, lib.pqcgpu_last_error()
        stream.synchronize()
        ctx.enc_dev(alg, n, ct_ref, ss_ref, pk, coins)
        ctx.wait()
        assert torch.equal(ct, ct_ref), call
        assert torch.equal(ss, ss_ref), call
        dec = torch.empty_like(ss)
        ctx.dec_dev(alg, n, dec, ct, sk)
        ctx.wait()
        assert torch.equal(dec, ss), call
    too_many = lib.pqcgpu_kem_enc_batch_noalloc(kem.alg_id(alg), 65537, p(ct), p(ss), p(pk), p(coins), None)
    assert too_many == -1
    assert b"65536" in lib.pqcgpu_last_error()
    ctx.close()
