"""ctypes bindings for the CPU oracle (oracle/_build/liboracle.so) -- TEST INFRASTRUCTURE.

Only the tests, the smoke check and the CPU-baseline leg of bench.py import this module; the
product package never does.  `build()` compiles the library with the Makefile beside this file.
"""
import ctypes
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")

# alg ids shared with the batched drivers in batch.c
KYBER512, KYBER768, KYBER1024, KYBER1024_R2, NEWHOPE1024, FRODO976 = range(6)
MLKEM512, MLKEM768, MLKEM1024 = 6, 7, 8
NEWHOPE512, FRODO640, FRODO1344 = 9, 10, 11
ALG_NAMES = {
    "newhope512": NEWHOPE512,
    "frodo640": FRODO640,
    "frodo1344": FRODO1344,
    "mlkem512": MLKEM512,
    "mlkem768": MLKEM768,
    "mlkem1024": MLKEM1024,
    "kyber512": KYBER512,
    "kyber768": KYBER768,
    "kyber1024": KYBER1024,
    "kyber1024r2": KYBER1024_R2,
    "newhope1024": NEWHOPE1024,
    "frodo976": FRODO976,
}

_lib = None


def build(force=False):
    if force or not os.path.exists(LIB_PATH):
        subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB_PATH)
        u8p = ctypes.c_char_p
        sz = ctypes.c_size_t
        L.oracle_keccakf1600.argtypes = [ctypes.c_void_p]
        for f in ("oracle_shake128", "oracle_shake256"):
            getattr(L, f).argtypes = [ctypes.c_void_p, sz, u8p, sz]
        for f in ("oracle_sha3_256", "oracle_sha3_512"):
            getattr(L, f).argtypes = [ctypes.c_void_p, u8p, sz]
        L.oracle_counter_keccak.restype = ctypes.c_uint64
        L.oracle_counter_butterfly.restype = ctypes.c_uint64
        L.oracle_alg_sizes.argtypes = [ctypes.c_int] + [ctypes.POINTER(sz)] * 6
        L.oracle_batch_keypair.argtypes = [ctypes.c_int, sz, ctypes.c_void_p, ctypes.c_void_p, u8p, ctypes.c_int]
        L.oracle_batch_enc.argtypes = [ctypes.c_int, sz, ctypes.c_void_p, ctypes.c_void_p, u8p, u8p, ctypes.c_int]
        L.oracle_batch_dec.argtypes = [ctypes.c_int, sz, ctypes.c_void_p, u8p, u8p, ctypes.c_int]
        L.oracle_kyber_sizes.argtypes = [ctypes.c_int, ctypes.c_int] + [ctypes.POINTER(sz)] * 4
        L.oracle_kyber_indcpa_keypair.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, u8p]
        L.oracle_kyber_indcpa_enc.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_void_p, u8p, u8p, u8p]
        L.oracle_kyber_indcpa_dec.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_void_p, u8p, u8p]
        for pre in ("oracle_newhope", "oracle_newhope512"):
            getattr(L, pre + "_cpapke_keypair").argtypes = [ctypes.c_void_p, ctypes.c_void_p, u8p]
            getattr(L, pre + "_cpapke_enc").argtypes = [ctypes.c_void_p, u8p, u8p, u8p]
            getattr(L, pre + "_cpapke_dec").argtypes = [ctypes.c_void_p, u8p, u8p]
        _lib = L
    return _lib


def shake128(data, n):
    out = ctypes.create_string_buffer(n)
    lib().oracle_shake128(out, n, bytes(data), len(data))
    return out.raw


def shake256(data, n):
    out = ctypes.create_string_buffer(n)
    lib().oracle_shake256(out, n, bytes(data), len(data))
    return out.raw


def sha3_256(data):
    out = ctypes.create_string_buffer(32)
    lib().oracle_sha3_256(out, bytes(data), len(data))
    return out.raw


def sha3_512(data):
    out = ctypes.create_string_buffer(64)
    lib().oracle_sha3_512(out, bytes(data), len(data))
    return out.raw


def alg_sizes(alg):
    vals = [ctypes.c_size_t() for _ in range(6)]
    if lib().oracle_alg_sizes(alg, *[ctypes.byref(v) for v in vals]):
        raise ValueError("unknown alg %r" % alg)
    keys = ("pk", "sk", "ct", "ss", "kp_coins", "enc_coins")
    return dict(zip(keys, (v.value for v in vals)))


def batch_keypair(alg, n, coins, nthreads=0):
    s = alg_sizes(alg)
    assert len(coins) == n * s["kp_coins"]
    pk = ctypes.create_string_buffer(n * s["pk"])
    sk = ctypes.create_string_buffer(n * s["sk"])
    lib().oracle_batch_keypair(alg, n, pk, sk, bytes(coins), nthreads)
    return pk.raw, sk.raw


def batch_enc(alg, n, pk, coins, nthreads=0):
    s = alg_sizes(alg)
    assert len(pk) == n * s["pk"] and len(coins) == n * s["enc_coins"]
    ct = ctypes.create_string_buffer(n * s["ct"])
    ss = ctypes.create_string_buffer(n * s["ss"])
    lib().oracle_batch_enc(alg, n, ct, ss, bytes(pk), bytes(coins), nthreads)
    return ct.raw, ss.raw


def batch_dec(alg, n, ct, sk, nthreads=0):
    s = alg_sizes(alg)
    assert len(ct) == n * s["ct"] and len(sk) == n * s["sk"]
    ss = ctypes.create_string_buffer(n * s["ss"])
    lib().oracle_batch_dec(alg, n, ss, bytes(ct), bytes(sk), nthreads)
    return ss.raw


def kyber_sizes(variant, k):
    vals = [ctypes.c_size_t() for _ in range(4)]
    lib().oracle_kyber_sizes(variant, k, *[ctypes.byref(v) for v in vals])
    return dict(zip(("pk", "sk_cpa", "sk", "ct"), (v.value for v in vals)))


def kyber_indcpa_keypair(variant, k, d):
    s = kyber_sizes(variant, k)
    pk = ctypes.create_string_buffer(s["pk"])
    sk = ctypes.create_string_buffer(s["sk_cpa"])
    lib().oracle_kyber_indcpa_keypair(variant, k, pk, sk, bytes(d))
    return pk.raw, sk.raw


def kyber_indcpa_enc(variant, k, m, pk, coins):
    s = kyber_sizes(variant, k)
    ct = ctypes.create_string_buffer(s["ct"])
    lib().oracle_kyber_indcpa_enc(variant, k, ct, bytes(m), bytes(pk), bytes(coins))
    return ct.raw


def kyber_indcpa_dec(variant, k, ct, sk):
    m = ctypes.create_string_buffer(32)
    lib().oracle_kyber_indcpa_dec(variant, k, m, bytes(ct), bytes(sk))
    return m.raw


# NewHope CPA-PKE sizes by n: (pk, sk, ct)
NEWHOPE_CPA_SIZES = {1024: (1824, 1792, 2176), 512: (928, 896, 1088)}


def _nh(n):
    return "oracle_newhope" if n == 1024 else "oracle_newhope512"


def newhope_cpapke_keypair(seed, n=1024):
    pkb, skb, _ = NEWHOPE_CPA_SIZES[n]
    pk = ctypes.create_string_buffer(pkb)
    sk = ctypes.create_string_buffer(skb)
    getattr(lib(), _nh(n) + "_cpapke_keypair")(pk, sk, bytes(seed))
    return pk.raw, sk.raw


def newhope_cpapke_enc(m, pk, coin, n=1024):
    ct = ctypes.create_string_buffer(NEWHOPE_CPA_SIZES[n][2])
    getattr(lib(), _nh(n) + "_cpapke_enc")(ct, bytes(m), bytes(pk), bytes(coin))
    return ct.raw


def newhope_cpapke_dec(ct, sk, n=1024):
    m = ctypes.create_string_buffer(32)
    getattr(lib(), _nh(n) + "_cpapke_dec")(m, bytes(ct), bytes(sk))
    return m.raw


def counters_reset():
    lib().oracle_counters_reset()


def counters():
    return int(lib().oracle_counter_keccak()), int(lib().oracle_counter_butterfly())
