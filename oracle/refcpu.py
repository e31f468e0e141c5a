"""The reference's own Kyber code on the host cores, as a CPU timing baseline -- TEST INFRASTRUCTURE.

oracle/_ref/librefkyber{2,3,4}.so is the reference's batched Kyber device code (round-2 arithmetic,
Kyber_GPU_Batched) compiled for the host by oracle/build_ref.sh.  The reference has no KEM layer,
so what it can time for Kyber-768 is its own CPA encryption + decryption (indcpa_enc / indcpa_dec,
Kyber_GPU_Batched/indcpa.cu:578-733) of k = 3 instances.

Its host code is not thread-safe: every launch rewrites the file-scope `blockSize` / `gridSize`
(Kyber_GPU_Batched/indcpa.cu:404-405) through its TIMING_START macro.  So the baseline runs one
process per core (started with `spawn`), each with its own state (the reference's poly_set4, about
300 MB at its N_TESTS = 16384) and its own range of instances, and times the whole job from the
parent.  Only bench.py's CPU-baseline leg and reference arm use this module.
"""
import concurrent.futures as cf
import ctypes
import multiprocessing as mp
import os
import time

HERE = os.path.dirname(os.path.abspath(__file__))
_L = None
_STATE = None


def lib_path(k=3):
    return os.path.join(HERE, "_ref", "librefkyber%d.so" % k)


def available(k=3):
    return os.path.exists(lib_path(k))


def _init(path):
    global _L, _STATE
    _L = ctypes.CDLL(path)
    _L.ref_kyber_state_new.restype = ctypes.c_void_p
    _L.ref_kyber_state_free.argtypes = [ctypes.c_void_p]
    _L.ref_kyber_cpa_enc_state.argtypes = [ctypes.c_void_p, ctypes.c_int] + [ctypes.c_char_p] * 4
    _L.ref_kyber_cpa_dec_state.argtypes = [ctypes.c_void_p, ctypes.c_int] + [ctypes.c_char_p] * 3
    _STATE = _L.ref_kyber_state_new()


def _work(task):
    """reps x (CPA encryption + decryption of `count` instances); returns whether every message
    decrypted to itself."""
    count, pk, sk, m, coins, reps, ct_len = task
    ct = ctypes.create_string_buffer(count * ct_len)
    m2 = ctypes.create_string_buffer(count * 32)
    ok = True
    for _ in range(reps):
        if _L.ref_kyber_cpa_enc_state(_STATE, count, ct, m, pk, coins) != 0:
            return False
        if _L.ref_kyber_cpa_dec_state(_STATE, count, m2, ct.raw, sk) != 0:
            return False
        ok = ok and m2.raw == m
    return ok


class RefKyberCPU:
    """A pool of `procs` processes, each holding the reference's state, with keys for `chunk`
    instances per process made by the reference's own keypair."""

    def __init__(self, k=3, procs=None, chunk=256, seed=5):
        import sys
        sys.path.insert(0, os.path.dirname(HERE))
        from pqc_gb300 import drbg
        self.k = k
        self.procs = procs or os.cpu_count()
        self.chunk = chunk
        L = ctypes.CDLL(lib_path(k))
        pkb, skb = 384 * k + 32, 384 * k
        self.ct_len = k * 11 * 32 + 5 * 32  # the reference's round-2 du = 11, dv = 5 for every k
        s = drbg.seed48(seed)
        self.inputs = []
        for p in range(self.procs):
            d = drbg.stream(s, b"d%d" % p, 32 * chunk)
            pk = ctypes.create_string_buffer(chunk * pkb)
            sk = ctypes.create_string_buffer(chunk * skb)
            if L.ref_kyber_cpa_keypair(chunk, pk, sk, d) != 0:
                raise RuntimeError("reference keypair failed")
            self.inputs.append((pk.raw, sk.raw, drbg.stream(s, b"m%d" % p, 32 * chunk),
                                drbg.stream(s, b"c%d" % p, 32 * chunk)))
        self.pool = cf.ProcessPoolExecutor(self.procs, mp_context=mp.get_context("spawn"), initializer=_init,
                                           initargs=(lib_path(k),))

    def run(self, reps):
        """All processes, reps rounds each; returns (pairs, seconds, all_ok)."""
        tasks = [(self.chunk, pk, sk, m, c, reps, self.ct_len) for pk, sk, m, c in self.inputs]
        t0 = time.perf_counter()
        oks = list(self.pool.map(_work, tasks))
        el = time.perf_counter() - t0
        return self.procs * self.chunk * reps, el, all(oks)

    def close(self):
        self.pool.shutdown()


def cpu_model():
    try:
        with open("/proc/cpuinfo") as f:
            for line in f:
                if line.lower().startswith(("model name", "cpu part")):
                    return line.split(":", 1)[1].strip()
    except OSError:
        pass
    import platform
    return platform.processor() or platform.machine()
