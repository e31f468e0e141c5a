"""FrodoKEM-976, -640 and -1344 on the GPU through the C ABI, bit-exact against the oracle (restated
from the reference's host flow FrodoKEM_GPU/kem.c and its matrix kernels; -640 / -1344 with their
parameter sets)."""
import hashlib

import pytest

from conftest import load_golden
from pqc_gb300 import drbg

pytestmark = pytest.mark.gpu

ALGS = ["frodo976", "frodo640", "frodo1344"]


@pytest.fixture(scope="module")
def ctx():
    from pqc_gb300 import kem
    c = kem.Context(0)
    yield c
    c.close()


def _sizes(alg):
    from pqc_gb300 import kem
    return kem.sizes(alg)


@pytest.mark.parametrize("alg", ALGS)
@pytest.mark.parametrize("n", [1, 3, 17])
def test_kem_matches_oracle(ctx, oracle, alg, n):
    a, s = oracle.ALG_NAMES[alg], _sizes(alg)
    seed = drbg.seed48(900 + n)
    kc = drbg.stream(seed, b"kp", n * s["kp_coins"])
    ec = drbg.stream(seed, b"enc", n * s["enc_coins"])
    pk, sk = ctx.keypair(alg, n, kc)
    opk, osk = oracle.batch_keypair(a, n, kc)
    assert pk == opk
    assert sk == osk
    ct, ss = ctx.enc(alg, n, pk, ec)
    oct_, oss = oracle.batch_enc(a, n, pk, ec)
    assert ct == oct_
    assert ss == oss
    assert ctx.dec(alg, n, ct, sk) == oss


@pytest.mark.parametrize("alg", ALGS)
def test_implicit_rejection(ctx, oracle, alg):
    a, s, n = oracle.ALG_NAMES[alg], _sizes(alg), 4
    SS, CT = s["ss"], s["ct"]
    seed = drbg.seed48(77)
    pk, sk = ctx.keypair(alg, n, drbg.stream(seed, b"kp", n * s["kp_coins"]))
    ct, ss = ctx.enc(alg, n, pk, drbg.stream(seed, b"enc", n * s["enc_coins"]))
    bad = bytearray(ct)
    bad[5] ^= 1                      # instance 0: c1
    bad[2 * CT - 1] ^= 0x80          # instance 1: c2
    got = ctx.dec(alg, n, bytes(bad), sk)
    assert got == oracle.batch_dec(a, n, bytes(bad), sk)
    assert got[:SS] != ss[:SS] and got[SS:2 * SS] != ss[SS:2 * SS]
    assert got[2 * SS:] == ss[2 * SS:]


@pytest.mark.parametrize("alg", ALGS)
def test_restated_fixture(ctx, alg):
    s = _sizes(alg)
    g = load_golden("restated_%s.json" % alg)
    n = g["n"]
    seed = drbg.seed48(g["drbg_seed"])
    pk, sk = ctx.keypair(alg, n, drbg.stream(seed, b"kp", n * s["kp_coins"]))
    ct, ss = ctx.enc(alg, n, pk, drbg.stream(seed, b"enc", n * s["enc_coins"]))
    sha = lambda b: hashlib.sha256(b).hexdigest()  # noqa: E731
    assert [sha(pk[i * s["pk"]:(i + 1) * s["pk"]]) for i in range(n)] == g["pk_sha256"]
    assert [sha(sk[i * s["sk"]:(i + 1) * s["sk"]]) for i in range(n)] == g["sk_sha256"]
    assert [sha(ct[i * s["ct"]:(i + 1) * s["ct"]]) for i in range(n)] == g["ct_sha256"]
    assert ss.hex() == g["ss"]


@pytest.mark.parametrize("alg", ALGS)
@pytest.mark.parametrize("parts,threads", [(1, 256), (1, 128), (2, 256), (4, 128), (8, 128), (16, 128), (16, 256)])
def test_row_split_shapes_match_oracle(ctx, oracle, alg, parts, threads):
    """Every split of the rows of A over CTAs (and every keypair block size) gives the same bytes."""
    from pqc_gb300 import _lib, kem
    lib = _lib.load()
    a, s, n = oracle.ALG_NAMES[alg], _sizes(alg), 5
    SS = s["ss"]
    fr = kem.alg_id(alg)
    seed = drbg.seed48(4400 + parts * 7 + threads)
    kc = drbg.stream(seed, b"kp", n * s["kp_coins"])
    ec = drbg.stream(seed, b"enc", n * s["enc_coins"])
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
        assert ss_bad[SS:] == oss[SS:] and ss_bad[:SS] != oss[:SS]
    finally:
        for op in (0, 1, 2):
            lib.pqcgpu_set_launch_shape(fr, op, 0, 0)
