"""NewHope-1024 on the GPU through the C ABI: CPA-PKE against the reference's own golden vectors
and the oracle, CPA-KEM against the oracle."""
import hashlib

import pytest

from conftest import load_golden
from pqc_gb300 import drbg

pytestmark = pytest.mark.gpu


def sha(b):
    return hashlib.sha256(b).hexdigest()


def split(b, sz):
    return [b[i * sz:(i + 1) * sz] for i in range(len(b) // sz)]


@pytest.fixture(scope="module")
def ctx():
    from pqc_gb300 import kem
    c = kem.Context(0)
    yield c
    c.close()


def test_cpa_matches_reference_vectors(ctx):
    g = load_golden("ref_newhope1024_cpa.json")
    n = g["n"]
    seed, m, coins = (bytes.fromhex(g[x]) for x in ("seed", "m", "coins"))
    pk, sk = ctx.newhope_cpa_keypair(n, seed)
    assert [sha(x) for x in split(pk, 1824)] == g["pk_sha256"]
    assert [sha(x) for x in split(sk, 1792)] == g["sk_sha256"]
    ct = ctx.newhope_cpa_enc(n, m, pk, coins)
    assert [sha(x) for x in split(ct, 2176)] == g["ct_sha256"]
    assert ctx.newhope_cpa_dec(n, ct, sk).hex() == g["m_dec"]


@pytest.mark.parametrize("n", [1, 5, 33, 257])
def test_cpa_matches_oracle(ctx, oracle, n):
    seed = drbg.seed48(500 + n)
    d = drbg.stream(seed, b"d", 32 * n)
    m = drbg.stream(seed, b"m", 32 * n)
    coins = drbg.stream(seed, b"coins", 32 * n)
    pk, sk = ctx.newhope_cpa_keypair(n, d)
    ct = ctx.newhope_cpa_enc(n, m, pk, coins)
    for x in range(n):
        opk, osk = oracle.newhope_cpapke_keypair(d[32 * x:32 * x + 32])
        assert pk[1824 * x:1824 * (x + 1)] == opk, x
        assert sk[1792 * x:1792 * (x + 1)] == osk, x
        assert ct[2176 * x:2176 * (x + 1)] == oracle.newhope_cpapke_enc(m[32 * x:32 * x + 32], opk, coins[32 * x:32 * x + 32]), x
    assert ctx.newhope_cpa_dec(n, ct, sk) == m


@pytest.mark.parametrize("n", [1, 63, 1000])
def test_kem_matches_oracle(ctx, oracle, n):
    alg = "newhope1024"
    a = oracle.NEWHOPE1024
    seed = drbg.seed48(600 + n)
    kc = drbg.stream(seed, b"kp", n * 32)
    ec = drbg.stream(seed, b"enc", n * 32)
    pk, sk = ctx.keypair(alg, n, kc)
    assert (pk, sk) == oracle.batch_keypair(a, n, kc)
    ct, ss = ctx.enc(alg, n, pk, ec)
    assert (ct, ss) == oracle.batch_enc(a, n, pk, ec)
    assert ctx.dec(alg, n, ct, sk) == ss
    bad = bytearray(ct)
    bad[-1] ^= 0xE0
    bad[100] ^= 0x3
    assert ctx.dec(alg, n, bytes(bad), sk) == oracle.batch_dec(a, n, bytes(bad), sk)


def test_restated_fixture(ctx):
    from pqc_gb300 import kem
    g = load_golden("restated_newhope1024.json")
    n = g["n"]
    seed = drbg.seed48(g["drbg_seed"])
    pk, sk = ctx.keypair("newhope1024", n, drbg.stream(seed, b"kp", n * 32))
    ct, ss = ctx.enc("newhope1024", n, pk, drbg.stream(seed, b"enc", n * 32))
    assert [sha(x) for x in split(pk, 1824)] == g["pk_sha256"]
    assert [sha(x) for x in split(ct, 2176)] == g["ct_sha256"]
    assert ss.hex() == g["ss"]
