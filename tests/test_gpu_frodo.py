"""FrodoKEM-976 on the GPU through the C ABI, bit-exact against the oracle (restated from the
reference's host flow FrodoKEM_GPU/kem.c and its matrix kernels)."""
import hashlib

import pytest

from conftest import load_golden
from pqc_gb300 import drbg

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    from pqc_gb300 import kem
    c = kem.Context(0)
    yield c
    c.close()


@pytest.mark.parametrize("n", [1, 3, 17])
def test_kem_matches_oracle(ctx, oracle, n):
    alg, a = "frodo976", oracle.FRODO976
    seed = drbg.seed48(900 + n)
    kc = drbg.stream(seed, b"kp", n * 64)
    ec = drbg.stream(seed, b"enc", n * 24)
    pk, sk = ctx.keypair(alg, n, kc)
    opk, osk = oracle.batch_keypair(a, n, kc)
    assert pk == opk
    assert sk == osk
    ct, ss = ctx.enc(alg, n, pk, ec)
    oct_, oss = oracle.batch_enc(a, n, pk, ec)
    assert ct == oct_
    assert ss == oss
    assert ctx.dec(alg, n, ct, sk) == oss


def test_implicit_rejection(ctx, oracle):
    alg, a, n = "frodo976", oracle.FRODO976, 4
    seed = drbg.seed48(77)
    pk, sk = ctx.keypair(alg, n, drbg.stream(seed, b"kp", n * 64))
    ct, ss = ctx.enc(alg, n, pk, drbg.stream(seed, b"enc", n * 24))
    bad = bytearray(ct)
    bad[5] ^= 1                      # instance 0: c1
    bad[2 * 15744 - 1] ^= 0x80       # instance 1: c2
    got = ctx.dec(alg, n, bytes(bad), sk)
    assert got == oracle.batch_dec(a, n, bytes(bad), sk)
    assert got[:24] != ss[:24] and got[24:48] != ss[24:48]
    assert got[48:] == ss[48:]


def test_restated_fixture(ctx):
    g = load_golden("restated_frodo976.json")
    n = g["n"]
    seed = drbg.seed48(g["drbg_seed"])
    pk, sk = ctx.keypair("frodo976", n, drbg.stream(seed, b"kp", n * 64))
    ct, ss = ctx.enc("frodo976", n, pk, drbg.stream(seed, b"enc", n * 24))
    sha = lambda b: hashlib.sha256(b).hexdigest()
    assert [sha(pk[i * 15632:(i + 1) * 15632]) for i in range(n)] == g["pk_sha256"]
    assert [sha(ct[i * 15744:(i + 1) * 15744]) for i in range(n)] == g["ct_sha256"]
    assert ss.hex() == g["ss"]


@pytest.mark.parametrize("parts,threads", [(1, 256), (1, 128), (2, 256), (4, 128), (8, 128), (16, 128), (16, 256)])
def test_row_split_shapes_match_oracle(ctx, oracle, parts, threads):
    """Every split of the rows of A over CTAs (and every keypair block size) gives the same bytes."""
    from pqc_gb300 import _lib, kem
    lib = _lib.load()
    alg, a, n = "frodo976", oracle.FRODO976, 5
    fr = kem.alg_id(alg)
    seed = drbg.seed48(4400 + parts * 7 + threads)
    kc = drbg.stream(seed, b"kp", n * 64)
    ec = drbg.stream(seed, b"enc", n * 24)
    kp_threads = {128: 64, 256: 256}[threads] if parts != 16 else 128
    try:
        assert lib.pqcgpu_set_launch_shape(fr, 0, 0, kp_threads) == 0
        assert lib.pqcgpu_set_launch_shape(fr, 1, parts, threads) == 0
        assert lib.pqcgpu_set_launch_shape(fr, 2, parts, threads) == 0
        pk, sk = ctx.keypair(alg, n, kc)
        opk, osk = oracle.batch_keypair(a, n, kc)
        assert (pk, sk) == (opk, osk)
        ct, ss = ctx.enc(alg, n, pk, ec)
        oct_, oss = oracle.batch_enc(a, n, pk, ec)
        assert (ct, ss) == (oct_, oss)
        assert ctx.dec(alg, n, ct, sk) == oss
        bad = bytearray(ct)
        bad[100] ^= 1  # one B' coefficient of instance 0: decaps must reject it implicitly
        ss_bad = ctx.dec(alg, n, bytes(bad), sk)
        assert ss_bad[24:] == oss[24:] and ss_bad[:24] != oss[:24]
    finally:
        for op in (0, 1, 2):
            lib.pqcgpu_set_launch_shape(fr, op, 0, 0)

