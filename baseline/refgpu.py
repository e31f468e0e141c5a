"""ctypes binding of baseline/_ref/librefgpu_kyber{3,4}.so: the reference's own batched Kyber
kernels (Kyber_GPU_Batched, round-2 arithmetic) compiled for sm_103a by baseline/build_ref_gpu.sh.

Used by the benchmark (the reference-kernels reference point) and by a GPU parity test; never by
the library.  All buffers are torch.uint8 CUDA tensors, instance-major, `n` a multiple of 256 and
at most `max_count`.
"""
import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))


def path(k):
    return os.path.join(HERE, "_ref", "librefgpu_kyber%d.so" % k)


def available(k):
    return os.path.exists(path(k))


def _p(t):
    return ctypes.c_void_p(t.data_ptr())


class RefGPU:
    def __init__(self, k):
        lib = ctypes.CDLL(path(k))
        vp, ci = ctypes.c_void_p, ctypes.c_int
        lib.refgpu_create.restype = vp
        lib.refgpu_destroy.argtypes = [vp]
        lib.refgpu_k.restype = ci
        lib.refgpu_max_count.restype = ci
        for f in ("refgpu_cpa_keypair", "refgpu_cpa_keypair_nist", "refgpu_cpa_dec"):
            getattr(lib, f).argtypes = [vp, ci, vp, vp, vp, vp]
            getattr(lib, f).restype = ci
        lib.refgpu_cpa_enc.argtypes = [vp, ci, vp, vp, vp, vp, vp]
        lib.refgpu_cpa_enc.restype = ci
        self.lib = lib
        self.k = lib.refgpu_k()
        self.max_count = lib.refgpu_max_count()
        self.h = lib.refgpu_create()
        if not self.h:
            raise RuntimeError("refgpu_create failed (device memory)")

    def close(self):
        if self.h:
            self.lib.refgpu_destroy(self.h)
            self.h = None

    def _check(self, rc, what):
        if rc != 0:
            raise RuntimeError("%s returned %d" % (what, rc))

    def keypair(self, n, pk, sk, rng_buf, stream):
        """The reference's indcpa_keypair as it is (rng_buf n*64 bytes, overwritten)."""
        self._check(self.lib.refgpu_cpa_keypair(self.h, n, _p(pk), _p(sk), _p(rng_buf), stream), "keypair")

    def keypair_nist(self, n, pk, sk, d, stream):
        self._check(self.lib.refgpu_cpa_keypair_nist(self.h, n, _p(pk), _p(sk), _p(d), stream), "keypair_nist")

    def enc(self, n, ct, m, pk, coins, stream):
        self._check(self.lib.refgpu_cpa_enc(self.h, n, _p(ct), _p(m), _p(pk), _p(coins), stream), "enc")

    def dec(self, n, m, ct, sk, stream):
        self._check(self.lib.refgpu_cpa_dec(self.h, n, _p(m), _p(ct), _p(sk), stream), "dec")
