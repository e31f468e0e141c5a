"""Empty batches: n = 0 is accepted by every operation of every algorithm, with host buffers and
with device buffers, returns PQCGPU_OK, writes nothing and launches no kernel."""
import ctypes

import pytest

pytestmark = pytest.mark.gpu

ALGS = ["kyber512", "kyber768", "kyber1024", "kyber1024r2", "mlkem512", "mlkem768", "mlkem1024", "newhope1024",
        "newhope512", "frodo640", "frodo976", "frodo1344"]


@pytest.mark.parametrize("device_ptrs", [False, True])
def test_empty_batches_are_no_ops(device_ptrs):
    import torch

    from pqc_gb300 import _lib, kem
    lib = _lib.load()
    ctx = kem.Context(0)
    try:
        if device_ptrs:
            bufs = [torch.full((64,), 0xA5, dtype=torch.uint8, device="cuda") for _ in range(3)]
            ptr = [ctypes.c_void_p(b.data_ptr()) for b in bufs]
            flags = kem.DEVICE_PTRS
        else:
            bufs = [ctypes.create_string_buffer(b"\xa5" * 64, 64) for _ in range(3)]
            ptr = [ctypes.cast(b, ctypes.c_void_p) for b in bufs]
            flags = 0
        before = lib.pqcgpu_ctx_launches(ctx.h)
        for alg in ALGS:
            a = kem.alg_id(alg)
            assert lib.pqcgpu_kem_keypair_batch(ctx.h, a, 0, ptr[0], ptr[1], ptr[2], flags) == 0, alg
            assert lib.pqcgpu_kem_enc_batch(ctx.h, a, 0, ptr[0], ptr[1], ptr[2], ptr[2], flags) == 0, alg
            assert lib.pqcgpu_kem_dec_batch(ctx.h, a, 0, ptr[0], ptr[1], ptr[2], flags) == 0, alg
        ctx.wait()
        assert lib.pqcgpu_ctx_launches(ctx.h) == before
        if device_ptrs:
            assert all(bool((b == 0xA5).all()) for b in bufs)
        else:
            assert all(b.raw == b"\xa5" * 64 for b in bufs)
    finally:
        ctx.close()
