"""Python handle on the native serving loop (pqcgpu_server_* in include/pqcgpu.h).

The dispatcher, batching, key store and load generator are native (pqc_gb300/csrc/server.cu);
this module only marshals requests for tests and the serving benchmark.
"""
import ctypes

from . import _lib, kem


class Ticket:
    __slots__ = ("id", "bufs", "op", "alg")

    def __init__(self, tid, bufs, op, alg):
        self.id, self.bufs, self.op, self.alg = tid, bufs, op, alg


class Server:
    def __init__(self, device=0, budget=16 << 30, max_inflight=4, max_batch=4096):
        self.lib = _lib.load()
        h = ctypes.c_void_p()
        _lib.check(self.lib.pqcgpu_server_create(ctypes.byref(h), device, budget, max_inflight, max_batch))
        self.h = h

    def close(self):
        if self.h:
            self.lib.pqcgpu_server_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def submit(self, alg, op, key=0, pk=None, inp=None):
        """Submit one request; returns a Ticket whose `bufs` hold the outputs after wait()."""
        s = kem.sizes(alg)
        op = kem.OPS[op] if isinstance(op, str) else op
        r = _lib.Request()
        r.alg, r.op, r.key = kem.alg_id(alg), op, key
        bufs = {}
        if pk is not None:
            bufs["pk_in"] = ctypes.create_string_buffer(bytes(pk), len(pk))
            r.pk = ctypes.addressof(bufs["pk_in"])
        if inp is not None:
            bufs["in"] = ctypes.create_string_buffer(bytes(inp), len(inp))
            r.in_ = ctypes.addressof(bufs["in"])
        if op == 0:
            bufs["pk"] = ctypes.create_string_buffer(s["pk"])
            bufs["key"] = ctypes.c_uint64(0)
            r.out0 = ctypes.addressof(bufs["pk"])
            r.key_out = ctypes.addressof(bufs["key"])
        elif op == 1:
            bufs["ct"] = ctypes.create_string_buffer(s["ct"])
            bufs["ss"] = ctypes.create_string_buffer(s["ss"])
            r.out0, r.out1 = ctypes.addressof(bufs["ct"]), ctypes.addressof(bufs["ss"])
        else:
            bufs["ss"] = ctypes.create_string_buffer(s["ss"])
            r.out0 = ctypes.addressof(bufs["ss"])
        tid = ctypes.c_uint64()
        _lib.check(self.lib.pqcgpu_server_submit(self.h, ctypes.byref(r), ctypes.byref(tid)))
        return Ticket(tid.value, bufs, op, alg)

    def wait(self, t, timeout_ms=-1):
        _lib.check(self.lib.pqcgpu_server_wait(self.h, t.id, timeout_ms))
        b = t.bufs
        if t.op == 0:
            return b["key"].value, b["pk"].raw
        if t.op == 1:
            return b["ct"].raw, b["ss"].raw
        return b["ss"].raw

    def keypair(self, alg, coins=None):
        return self.wait(self.submit(alg, 0, inp=coins))

    def enc(self, alg, key=0, pk=None, coins=None):
        return self.wait(self.submit(alg, 1, key=key, pk=pk, inp=coins))

    def dec(self, alg, key, ct):
        return self.wait(self.submit(alg, 2, key=key, inp=ct))

    def release(self, key):
        _lib.check(self.lib.pqcgpu_server_key_release(self.h, key))

    def drain(self):
        _lib.check(self.lib.pqcgpu_server_drain(self.h))

    def stats(self, reset=False):
        st = _lib.ServerStats()
        _lib.check(self.lib.pqcgpu_server_get_stats(self.h, ctypes.byref(st), 1 if reset else 0))
        return {f: getattr(st, f) for f, _ in _lib.ServerStats._fields_}

    def group_stats(self, alg, op):
        """Latency of the completed (alg, op) requests since the last reset."""
        st = _lib.ServerStats()
        _lib.check(self.lib.pqcgpu_server_get_group_stats(self.h, kem.alg_id(alg), kem.OPS[op] if isinstance(op, str)
                                                          else op, ctypes.byref(st)))
        return {f: getattr(st, f) for f in ("completed", "p50_ms", "p99_ms", "mean_ms", "max_ms")}

    def run_poisson(self, mix, rate, seconds, seed=0):
        """mix: list of (alg, op, weight).  Returns the load report as a dict; the latency samples of
        the run stay readable through stats() / group_stats() until the next reset."""
        arr = (_lib.MixEntry * len(mix))()
        for i, (alg, op, w) in enumerate(mix):
            arr[i].alg, arr[i].op, arr[i].weight = kem.alg_id(alg), kem.OPS[op] if isinstance(op, str) else op, w
        rep = _lib.LoadReport()
        _lib.check(self.lib.pqcgpu_server_run_poisson(self.h, arr, len(mix), float(rate), float(seconds), seed,
                                                      ctypes.byref(rep)))
        return {f: getattr(rep, f) for f, _ in _lib.LoadReport._fields_}


# The serving mix of the benchmark: 60 % Kyber (512 / 768 / 1024 evenly), 20 % NewHope-1024,
# 20 % FrodoKEM-976, each operation equiprobable.
SERVING_MIX = [(alg, op, w / 3.0) for alg, w in (("kyber512", 0.2), ("kyber768", 0.2), ("kyber1024", 0.2),
                                                 ("newhope1024", 0.2), ("frodo976", 0.2))
               for op in ("keypair", "enc", "dec")]
