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
