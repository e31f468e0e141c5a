"""Python mirror of the batched KEM C ABI (include/pqcgpu.h), used by the tests and the benchmark.

Host path: methods take / return `bytes` (instance-major), synchronous.
Device path: the *_dev methods take torch.uint8 CUDA tensors (instance-major, 16-byte aligned),
asynchronous on the context stream.
"""
import ctypes
import json

from . import _lib

ALGS = {"kyber512": 0, "kyber768": 1, "kyber1024": 2, "kyber1024r2": 3, "newhope1024": 4, "frodo976": 5,
        "mlkem512": 6, "mlkem768": 7, "mlkem1024": 8, "newhope512": 9, "frodo640": 10, "frodo1344": 11}
DEVICE_PTRS = 0x1
PLAIN = 0x2
STAGE_KERNELS = 0x4


def alg_id(alg):
    return ALGS[alg] if isinstance(alg, str) else int(alg)


def sizes(alg):
    lib = _lib.load()
    v = [ctypes.c_size_t() for _ in range(6)]
    _lib.check(lib.pqcgpu_alg_sizes(alg_id(alg), *[ctypes.byref(x) for x in v]))
    return dict(zip(("pk", "sk", "ct", "ss", "kp_coins", "enc_coins"), (x.value for x in v)))


def newhope_cpa_sizes(poly_n):
    """NewHope CPA-PKE byte sizes for n = 1024 or 512 coefficients."""
    pb = 14 * poly_n // 8
    return {"pk": pb + 32, "sk": pb, "ct": pb + 3 * poly_n // 8}


def kyber_cpa_sizes(variant, k):
    du, dv = (11, 5) if (variant == 2 or k == 4) else (10, 4)
    return {"pk": 384 * k + 32, "sk": 384 * k, "ct": k * du * 32 + dv * 32}


OPS = {"keypair": 0, "enc": 1, "dec": 2}


def profile_enable(on=True):
    """Bracket every kernel launch and host-buffer copy with CUDA events (all contexts)."""
    _lib.check(_lib.load().pqcgpu_profile_enable(1 if on else 0))


def profile_trace():
    """The profiler's records since the last read as a Chrome trace-event dict, then clears them.
    Write it with json.dump and open it in chrome://tracing or Perfetto."""
    lib = _lib.load()
    need = ctypes.c_size_t(0)
    while True:
        buf = ctypes.create_string_buffer(need.value) if need.value else None
        if lib.pqcgpu_profile_trace(buf, ctypes.byref(need)) == 0:
            return json.loads(buf.value.decode())
        if buf is not None and len(buf) >= need.value:
            _lib.check(-1)  # failed for another reason


def set_host_pipeline(chunk_max=0, chunk_first=0, chunk_last=0, streams=0):
    """Chunking of host-buffer calls (all contexts); zeros select the defaults."""
    _lib.check(_lib.load().pqcgpu_set_host_pipeline(chunk_max, chunk_first, chunk_last, streams))


def get_host_pipeline():
    """(chunk_max, chunk_first, chunk_last, streams) of host-buffer calls."""
    a, b, c, d = ctypes.c_size_t(), ctypes.c_size_t(), ctypes.c_size_t(), ctypes.c_int()
    _lib.check(_lib.load().pqcgpu_get_host_pipeline(ctypes.byref(a), ctypes.byref(b), ctypes.byref(c),
                                                    ctypes.byref(d)))
    return a.value, b.value, c.value, d.value


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


def make_jobs(jobs):
    """jobs: iterable of (alg, op, n, in0, in1, out0, out1) with torch CUDA tensors (or None)."""
    arr = (_lib.Job * len(jobs))()
    for i, (alg, op, n, in0, in1, out0, out1) in enumerate(jobs):
        arr[i].alg = alg_id(alg)
        arr[i].op = OPS[op] if isinstance(op, str) else int(op)
        arr[i].n = n
        for name, t in (("in0", in0), ("in1", in1), ("out0", out0), ("out1", out1)):
            setattr(arr[i], name, t.data_ptr() if t is not None else None)
    return arr


class shared_product:
    """Context manager: the product of FrodoKEM shared-key encapsulation (1 CUDA cores, 2 tensor cores)
    for the duration of a block, restored afterwards; None leaves it unchanged."""

    def __init__(self, alg, product):
        self.alg, self.product, self.old = alg, product, None

    def __enter__(self):
        if self.product is not None:
            lib = _lib.load()
            a, b = ctypes.c_int(), ctypes.c_int()
            _lib.check(lib.pqcgpu_get_launch_shape(alg_id(self.alg), 3, ctypes.byref(a), ctypes.byref(b)))
            self.old = a.value
            _lib.check(lib.pqcgpu_set_launch_shape(alg_id(self.alg), 3, self.product, 0))
        return self

    def __exit__(self, *exc):
        if self.old is not None:
            _lib.load().pqcgpu_set_launch_shape(alg_id(self.alg), 3, self.old, 0)


class Graph:
    """A captured mixed job list (pqcgpu_graph_capture); launch() replays it on the context stream."""

    def __init__(self, ctx, jobs, flags=0):
        self.ctx = ctx
        self.arr = make_jobs(jobs)
        h = ctypes.c_void_p()
        _lib.check(ctx.lib.pqcgpu_graph_capture(ctx.h, self.arr, len(jobs), flags | DEVICE_PTRS, ctypes.byref(h)))
        self.h = h

    def launch(self):
        _lib.check(self.ctx.lib.pqcgpu_graph_launch(self.h))

    def close(self):
        if self.h:
            self.ctx.lib.pqcgpu_graph_destroy(self.h)
            self.h = None


class Context:
    def __init__(self, device=0, budget=0):
        self.lib = _lib.load()
        h = ctypes.c_void_p()
        _lib.check(self.lib.pqcgpu_ctx_create(ctypes.byref(h), device, budget))
        self.h = h

    def close(self):
        if self.h:
            self.lib.pqcgpu_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def wait(self):
        _lib.check(self.lib.pqcgpu_ctx_wait(self.h))

    @property
    def launches(self):
        return int(self.lib.pqcgpu_ctx_launches(self.h))

    @property
    def stream(self):
        return self.lib.pqcgpu_ctx_stream(self.h)

    def set_stream(self, stream_handle):
        _lib.check(self.lib.pqcgpu_ctx_set_stream(self.h, ctypes.c_void_p(stream_handle)))

    # ---- host buffers (bytes) ----
    def keypair(self, alg, n, coins=None, flags=0):
        s = sizes(alg)
        pk = ctypes.create_string_buffer(n * s["pk"])
        sk = ctypes.create_string_buffer(n * s["sk"])
        _lib.check(self.lib.pqcgpu_kem_keypair_batch(self.h, alg_id(alg), n, pk, sk, coins, flags))
        return pk.raw, sk.raw

    def enc(self, alg, n, pk, coins=None, flags=0):
        s = sizes(alg)
        ct = ctypes.create_string_buffer(n * s["ct"])
        ss = ctypes.create_string_buffer(n * s["ss"])
        _lib.check(self.lib.pqcgpu_kem_enc_batch(self.h, alg_id(alg), n, ct, ss, pk, coins, flags))
        return ct.raw, ss.raw

    def dec(self, alg, n, ct, sk, flags=0):
        s = sizes(alg)
        ss = ctypes.create_string_buffer(n * s["ss"])
        _lib.check(self.lib.pqcgpu_kem_dec_batch(self.h, alg_id(alg), n, ss, ct, sk, flags))
        return ss.raw

    def frodo_enc_shared(self, alg, n, pk, coins=None, product=None, flags=0):
        """n FrodoKEM encapsulations to the one public key pk (host bytes); product: None (default),
        1 CUDA cores, 2 tensor cores.  Returns (ct, ss)."""
        s = sizes(alg)
        ct = ctypes.create_string_buffer(n * s["ct"])
        ss = ctypes.create_string_buffer(n * s["ss"])
        with shared_product(alg, product):
            _lib.check(self.lib.pqcgpu_frodo_enc_shared_key_batch(self.h, alg_id(alg), n, ct, ss, pk, coins, flags))
        return ct.raw, ss.raw

    def frodo_enc_shared_dev(self, alg, n, ct, ss, pk, coins, flags=0):
        _lib.check(self.lib.pqcgpu_frodo_enc_shared_key_batch(self.h, alg_id(alg), n, _ptr(ct), _ptr(ss), _ptr(pk),
                                                              _ptr(coins), flags | DEVICE_PTRS))

    def kyber_cpa_keypair(self, variant, k, n, d, flags=0):
        s = kyber_cpa_sizes(variant, k)
        pk = ctypes.create_string_buffer(n * s["pk"])
        sk = ctypes.create_string_buffer(n * s["sk"])
        _lib.check(self.lib.pqcgpu_kyber_indcpa_keypair_batch(self.h, variant, k, n, pk, sk, d, flags))
        return pk.raw, sk.raw

    def kyber_cpa_enc(self, variant, k, n, m, pk, coins, flags=0):
        s = kyber_cpa_sizes(variant, k)
        ct = ctypes.create_string_buffer(n * s["ct"])
        _lib.check(self.lib.pqcgpu_kyber_indcpa_enc_batch(self.h, variant, k, n, ct, m, pk, coins, flags))
        return ct.raw

    def kyber_cpa_dec(self, variant, k, n, ct, sk, flags=0):
        m = ctypes.create_string_buffer(n * 32)
        _lib.check(self.lib.pqcgpu_kyber_indcpa_dec_batch(self.h, variant, k, n, m, ct, sk, flags))
        return m.raw

    # NewHope CPA-PKE; poly_n = 1024 (pqcgpu_newhope_*) or 512 (pqcgpu_newhope512_*)
    def _nh(self, poly_n, what):
        return getattr(self.lib, "pqcgpu_newhope%s_cpapke_%s_batch" % ("" if poly_n == 1024 else "512", what))

    def newhope_cpa_keypair(self, n, seed, flags=0, poly_n=1024):
        s = newhope_cpa_sizes(poly_n)
        pk = ctypes.create_string_buffer(n * s["pk"])
        sk = ctypes.create_string_buffer(n * s["sk"])
        _lib.check(self._nh(poly_n, "keypair")(self.h, n, pk, sk, seed, flags))
        return pk.raw, sk.raw

    def newhope_cpa_enc(self, n, m, pk, coin, flags=0, poly_n=1024):
        ct = ctypes.create_string_buffer(n * newhope_cpa_sizes(poly_n)["ct"])
        _lib.check(self._nh(poly_n, "enc")(self.h, n, ct, m, pk, coin, flags))
        return ct.raw

    def newhope_cpa_dec(self, n, ct, sk, flags=0, poly_n=1024):
        m = ctypes.create_string_buffer(n * 32)
        _lib.check(self._nh(poly_n, "dec")(self.h, n, m, ct, sk, flags))
        return m.raw

    # ---- device tensors (torch.uint8 on this context's device), asynchronous ----
    def keypair_dev(self, alg, n, pk, sk, coins, flags=0):
        _lib.check(self.lib.pqcgpu_kem_keypair_batch(self.h, alg_id(alg), n, _ptr(pk), _ptr(sk), _ptr(coins),
                                                     flags | DEVICE_PTRS))

    def enc_dev(self, alg, n, ct, ss, pk, coins, flags=0):
        _lib.check(self.lib.pqcgpu_kem_enc_batch(self.h, alg_id(alg), n, _ptr(ct), _ptr(ss), _ptr(pk), _ptr(coins),
                                                 flags | DEVICE_PTRS))

    def dec_dev(self, alg, n, ss, ct, sk, flags=0):
        _lib.check(self.lib.pqcgpu_kem_dec_batch(self.h, alg_id(alg), n, _ptr(ss), _ptr(ct), _ptr(sk),
                                                 flags | DEVICE_PTRS))

    def mixed_dev(self, jobs, flags=0):
        """Run a list of (alg, op, n, in0, in1, out0, out1) jobs at once (device tensors, async)."""
        arr = make_jobs(jobs)
        _lib.check(self.lib.pqcgpu_kem_mixed_batch(self.h, arr, len(jobs), flags | DEVICE_PTRS))

    def graph(self, jobs, flags=0):
        return Graph(self, jobs, flags)

    # host-pointer call on raw addresses (pinned torch tensors), synchronous
    def enc_host_ptrs(self, alg, n, ct, ss, pk, coins, flags=0):
        _lib.check(self.lib.pqcgpu_kem_enc_batch(self.h, alg_id(alg), n, _ptr(ct), _ptr(ss), _ptr(pk), _ptr(coins),
                                                 flags))

    def dec_host_ptrs(self, alg, n, ss, ct, sk, flags=0):
        _lib.check(self.lib.pqcgpu_kem_dec_batch(self.h, alg_id(alg), n, _ptr(ss), _ptr(ct), _ptr(sk), flags))
