"""Host-side checks of the native library that need no GPU: it loads, exports every entry point
declared in include/pqcgpu.h, reports sizes consistent with the oracle, fails cleanly without a
device, and its DRBG is the SHAKE-256 stream it documents."""
import ctypes
import hashlib
import os
import re

import pytest

from conftest import ROOT


@pytest.fixture(scope="module")
def lib():
    from pqc_gb300 import _lib
    return _lib.load()


def declared_symbols():
    names = set()
    for h in os.listdir(os.path.join(ROOT, "include")):
        if h.endswith(".h"):
            txt = open(os.path.join(ROOT, "include", h)).read()
            txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
            names |= set(re.findall(r"\b(pqcgpu_\w+)\s*\(", txt))
    return names


def test_exports_every_declared_symbol(lib):
    from pqc_gb300 import _lib
    names = declared_symbols()
    assert len(names) >= 20
    for n in sorted(names):
        assert hasattr(lib, n), n
    assert set(_lib.SIGNATURES) == names


def test_sizes_match_oracle(lib, oracle):
    from pqc_gb300 import kem
    for name, alg in kem.ALGS.items():
        assert kem.sizes(alg) == oracle.alg_sizes(alg), name


def test_bad_arguments_return_errors(lib):
    assert lib.pqcgpu_alg_sizes(99, *([None] * 6)) == -1
    assert lib.pqcgpu_ctx_create(None, 0, 0) == -1
    assert lib.pqcgpu_kem_keypair_batch(None, 1, 1, None, None, None, 0) == -1


def test_drbg_is_shake256_stream(lib):
    seed = bytes(range(48))
    assert lib.pqcgpu_randombytes_init(seed) == 0
    a = ctypes.create_string_buffer(100)
    b = ctypes.create_string_buffer(300)
    lib.pqcgpu_randombytes(a, 100)
    lib.pqcgpu_randombytes(b, 300)
    assert a.raw + b.raw == hashlib.shake_256(seed).digest(400)


def test_no_device_is_a_clean_error(lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    h = ctypes.c_void_p()
    rc = lib.pqcgpu_ctx_create(ctypes.byref(h), 0, 0)
    assert rc == -3
    assert b"device" in lib.pqcgpu_last_error() or b"CUDA" in lib.pqcgpu_last_error()


def test_frodo_launch_shape_validation():
    """Shape setting is host-only (no device needed); bad splits / block sizes are refused."""
    from pqc_gb300 import _lib, kem
    lib = _lib.load()
    fr = kem.alg_id("frodo976")
    assert lib.pqcgpu_set_launch_shape(fr, 1, 3, 256) != 0
    assert lib.pqcgpu_set_launch_shape(fr, 1, 2, 96) != 0
    assert lib.pqcgpu_set_launch_shape(fr, 0, 2, 256) != 0
    assert lib.pqcgpu_set_launch_shape(fr, 0, 0, 0) == 0


def test_kyber_single_instance_thresholds():
    """Kyber op 4 sets the single-instance threshold of every operation of one k (0 = never); -1
    restores the measured per-operation defaults; get returns the encapsulation's."""
    import ctypes

    from pqc_gb300 import _lib, kem
    lib = _lib.load()
    ni, thr = ctypes.c_int(), ctypes.c_int()

    def enc_limit(alg):
        assert lib.pqcgpu_get_launch_shape(kem.alg_id(alg), 4, ctypes.byref(ni), ctypes.byref(thr)) == 0
        return ni.value

    assert (enc_limit("kyber512"), enc_limit("kyber768"), enc_limit("kyber1024")) == (640, 304, 304)
    assert enc_limit("mlkem768") == 304  # shared by every variant of one k
    try:
        assert lib.pqcgpu_set_launch_shape(kem.alg_id("kyber768"), 4, 4097, 0) != 0
        assert lib.pqcgpu_set_launch_shape(kem.alg_id("kyber768"), 4, -2, 0) != 0
        assert lib.pqcgpu_set_launch_shape(kem.alg_id("kyber768"), 4, 0, 0) == 0
        assert enc_limit("kyber768") == 0 and enc_limit("kyber512") == 640
    finally:
        assert lib.pqcgpu_set_launch_shape(kem.alg_id("kyber768"), 4, -1, 0) == 0
    assert enc_limit("kyber768") == 304


def test_newhope_single_instance_thresholds():
    """NewHope op 3 sets the single-instance threshold of keypair and encapsulation (both n); -1
    restores the measured defaults (304 / 456); get returns the encapsulation's."""
    import ctypes

    from pqc_gb300 import _lib, kem
    lib = _lib.load()
    a = kem.alg_id("newhope1024")
    ni, thr = ctypes.c_int(), ctypes.c_int()
    assert lib.pqcgpu_get_launch_shape(a, 3, ctypes.byref(ni), ctypes.byref(thr)) == 0
    assert ni.value == 456
    try:
        assert lib.pqcgpu_set_launch_shape(a, 3, -2, 0) != 0
        assert lib.pqcgpu_set_launch_shape(a, 3, 0, 0) == 0
        assert lib.pqcgpu_get_launch_shape(kem.alg_id("newhope512"), 3, ctypes.byref(ni), ctypes.byref(thr)) == 0
        assert ni.value == 0
    finally:
        assert lib.pqcgpu_set_launch_shape(a, 3, -1, 0) == 0
    assert lib.pqcgpu_get_launch_shape(a, 3, ctypes.byref(ni), ctypes.byref(thr)) == 0
    assert ni.value == 456


def test_kyber_warp_hash_threshold():
    """Kyber op 5 (the largest batch whose serial hashes run a warp per instance) takes 0..65535,
    shared by every k; the setting round-trips and the default is restored."""
    import ctypes

    from pqc_gb300 import _lib, kem
    lib = _lib.load()
    ky = kem.alg_id("kyber768")
    ni, thr = ctypes.c_int(), ctypes.c_int()
    assert lib.pqcgpu_get_launch_shape(ky, 5, ctypes.byref(ni), ctypes.byref(thr)) == 0
    default = ni.value
    assert default == 2048
    try:
        assert lib.pqcgpu_set_launch_shape(ky, 5, 65536, 0) != 0
        assert lib.pqcgpu_set_launch_shape(ky, 5, -1, 0) != 0
        assert lib.pqcgpu_set_launch_shape(ky, 5, 4096, 0) == 0
        assert lib.pqcgpu_get_launch_shape(kem.alg_id("kyber1024"), 5, ctypes.byref(ni), ctypes.byref(thr)) == 0
        assert ni.value == 4096
    finally:
        lib.pqcgpu_set_launch_shape(ky, 5, default, 0)


class _CtrDrbgRestated:
    """SP 800-90A AES-256 CTR_DRBG (no derivation function), restated over an independent AES
    (the `cryptography` package) to check the library's own AES and DRBG."""

    def __init__(self, aes_ecb, entropy, personalization=None):
        self.aes = aes_ecb
        seed = bytes(a ^ b for a, b in zip(entropy, personalization or bytes(48)))
        self.key, self.v = bytes(32), bytes(16)
        self._update(seed)

    def _inc(self):
        self.v = ((int.from_bytes(self.v, "big") + 1) % (1 << 128)).to_bytes(16, "big")

    def _update(self, provided):
        temp = b""
        for _ in range(3):
            self._inc()
            temp += self.aes(self.key, self.v)
        if provided is not None:
            temp = bytes(a ^ b for a, b in zip(temp, provided))
        self.key, self.v = temp[:32], temp[32:]

    def generate(self, n):
        out = b""
        while len(out) < n:
            self._inc()
            out += self.aes(self.key, self.v)
        self._update(None)
        return out[:n]


def test_nist_ctr_drbg_matches_independent_aes():
    pytest.importorskip("cryptography")
    import ctypes

    from cryptography.hazmat.primitives.ciphers import Cipher, algorithms, modes

    from pqc_gb300 import _lib, kem

    def aes(key, block):
        e = Cipher(algorithms.AES(key), modes.ECB()).encryptor()
        return e.update(block) + e.finalize()

    lib = _lib.load()
    entropy = bytes(range(48))
    pers = bytes((7 * i + 3) & 0xff for i in range(48))
    for p in (None, pers):
        ref = _CtrDrbgRestated(aes, entropy, p)
        assert lib.pqcgpu_randombytes_init_nist(entropy, p) == 0
        for n in (48, 32, 32, 1, 17, 100, 16):
            buf = ctypes.create_string_buffer(n)
            assert lib.pqcgpu_randombytes(buf, n) == 0
            assert buf.raw == ref.generate(n), (p is not None, n)
    # coins of one crypto_kem_* call: Kyber keypair = two draws of 32, ML-KEM / FrodoKEM one draw
    for alg, splits in (("kyber768", (32, 32)), ("mlkem768", (64,)), ("frodo976", (64,))):
        ref = _CtrDrbgRestated(aes, entropy)
        lib.pqcgpu_randombytes_init_nist(entropy, None)
        buf = ctypes.create_string_buffer(64)
        assert lib.pqcgpu_nist_coins(kem.alg_id(alg), 0, buf) == 0
        assert buf.raw == b"".join(ref.generate(s) for s in splits), alg
    lib.pqcgpu_randombytes_init(bytes(48))


def test_launch_shapes_that_exceed_shared_memory_are_refused():
    """A shape whose CTA would need more than the 227 KB of shared memory is refused when set
    (host-only check, no device needed), so no launch can fail on it later."""
    from pqc_gb300 import _lib, kem
    lib = _lib.load()
    import ctypes
    k768, nh = kem.alg_id("kyber768"), kem.alg_id("newhope1024")
    ni, thr = ctypes.c_int(), ctypes.c_int()
    assert lib.pqcgpu_get_launch_shape(k768, 2, ctypes.byref(ni), ctypes.byref(thr)) == 0
    try:
        assert lib.pqcgpu_set_launch_shape(k768, 2, 48, 192) != 0  # 48 x 4.8 KB + staging > 227 KB
        assert lib.pqcgpu_set_launch_shape(k768, 2, 30, 192) == 0
        assert lib.pqcgpu_set_launch_shape(k768, 2, 8, 288) != 0   # above the kernel's launch bound (256)
        assert lib.pqcgpu_set_launch_shape(nh, 1, 64, 256) != 0   # 64 x 7.5 KB
    finally:
        lib.pqcgpu_set_launch_shape(k768, 2, ni.value, thr.value)


def test_host_pipeline_shape_validation():
    """The host-buffer pipeline shape: zeros select the defaults, out-of-range values are refused
    and leave the shape unchanged."""
    from pqc_gb300 import kem
    from pqc_gb300 import _lib
    lib = _lib.load()
    default = kem.get_host_pipeline()
    assert default == (16384, 2048, 4096, 8)
    try:
        kem.set_host_pipeline(32768, 0, 0, 4)
        assert kem.get_host_pipeline() == (32768, 4096, 8192, 4)
        kem.set_host_pipeline(8192, 2048, 8192, 8)
        assert kem.get_host_pipeline() == (8192, 2048, 8192, 8)
        assert lib.pqcgpu_set_host_pipeline(32, 0, 0, 0) != 0         # chunk_max < 64
        assert lib.pqcgpu_set_host_pipeline(4096, 8192, 0, 0) != 0     # chunk_first > chunk_max
        assert lib.pqcgpu_set_host_pipeline(4096, 0, 8192, 0) != 0     # chunk_last > chunk_max
        assert lib.pqcgpu_set_host_pipeline(0, 0, 0, 9) != 0           # more streams than the context has
        assert kem.get_host_pipeline() == (8192, 2048, 8192, 8)
    finally:
        kem.set_host_pipeline(*default)
    assert kem.get_host_pipeline() == default


def test_profile_trace_without_records(lib):
    """The trace call reports the size it needs and returns an empty timeline when nothing ran."""
    from pqc_gb300 import kem
    need = ctypes.c_size_t(0)
    assert lib.pqcgpu_profile_trace(None, ctypes.byref(need)) != 0
    assert need.value == len('{"traceEvents": []}') + 1
    assert kem.profile_trace() == {"traceEvents": []}
