"""NewHope-1024 and NewHope-512 on the GPU through the C ABI: CPA-PKE against the reference's own
golden vectors (n = 512: the reference built with NEWHOPE_N=512) and the oracle, CPA-KEM against the
oracle."""
import hashlib

import pytest

from conftest import load_golden
from pqc_gb300 import drbg

pytestmark = pytest.mark.gpu

ALG = {1024: "newhope1024", 512: "newhope512"}


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


@pytest.mark.parametrize("poly_n", [1024, 512])
def test_cpa_matches_reference_vectors(ctx, poly_n):
    from pqc_gb300.kem import newhope_cpa_sizes
    s = newhope_cpa_sizes(poly_n)
    g = load_golden("ref_newhope%d_cpa.json" % poly_n)
    n = g["n"]
    seed, m, coins = (bytes.fromhex(g[x]) for x in ("seed", "m", "coins"))
    pk, sk = ctx.newhope_cpa_keypair(n, seed, poly_n=poly_n)
    assert [sha(x) for x in split(pk, s["pk"])] == g["pk_sha256"]
    assert [sha(x) for x in split(sk, s["sk"])] == g["sk_sha256"]
    ct = ctx.newhope_cpa_enc(n, m, pk, coins, poly_n=poly_n)
    assert [sha(x) for x in split(ct, s["ct"])] == g["ct_sha256"]
    assert ctx.newhope_cpa_dec(n, ct, sk, poly_n=poly_n).hex() == g["m_dec"]


@pytest.mark.parametrize("poly_n", [1024, 512])
@pytest.mark.parametrize("n", [1, 5, 33, 257])
def test_cpa_matches_oracle(ctx, oracle, n, poly_n):
    from pqc_gb300.kem import newhope_cpa_sizes
    s = newhope_cpa_sizes(poly_n)
    P, S, C = s["pk"], s["sk"], s["ct"]
    seed = drbg.seed48(500 + n + poly_n)
    d = drbg.stream(seed, b"d", 32 * n)
    m = drbg.stream(seed, b"m", 32 * n)
    coins = drbg.stream(seed, b"coins", 32 * n)
    pk, sk = ctx.newhope_cpa_keypair(n, d, poly_n=poly_n)
    ct = ctx.newhope_cpa_enc(n, m, pk, coins, poly_n=poly_n)
    for x in range(n):
        opk, osk = oracle.newhope_cpapke_keypair(d[32 * x:32 * x + 32], poly_n)
        assert pk[P * x:P * (x + 1)] == opk, x
        assert sk[S * x:S * (x + 1)] == osk, x
        oct_ = oracle.newhope_cpapke_enc(m[32 * x:32 * x + 32], opk, coins[32 * x:32 * x + 32], poly_n)
        assert ct[C * x:C * (x + 1)] == oct_, x
    assert ctx.newhope_cpa_dec(n, ct, sk, poly_n=poly_n) == m


@pytest.mark.parametrize("poly_n", [1024, 512])
@pytest.mark.parametrize("n", [1, 63, 400, 1000])  # 400: batched keypair, single-instance encapsulation
def test_kem_matches_oracle(ctx, oracle, n, poly_n):
    alg = ALG[poly_n]
    a = oracle.ALG_NAMES[alg]
    seed = drbg.seed48(600 + n + poly_n)
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


@pytest.mark.parametrize("poly_n", [1024, 512])
@pytest.mark.parametrize("n", [1, 7, 64])
def test_single_instance_kernels_equal_batched(ctx, poly_n, n):
    """Key generations and KEM encapsulations of small batches run on the single-instance kernels
    (one 512-thread CTA per operation); the bytes equal the batched kernels' (launch-shape op 3 = 0
    forces those), and decapsulation recovers the key."""
    import ctypes
    from pqc_gb300 import _lib, kem
    lib = _lib.load()
    alg = ALG[poly_n]
    a = kem.alg_id(alg)
    seed = drbg.seed48(700 + n + poly_n)
    kc = drbg.stream(seed, b"kp", n * 32)
    ec = drbg.stream(seed, b"enc", n * 32)
    single, t = ctypes.c_int(), ctypes.c_int()
    assert lib.pqcgpu_get_launch_shape(a, 3, ctypes.byref(single), ctypes.byref(t)) == 0
    assert n <= single.value
    pk, sk = ctx.keypair(alg, n, kc)
    ct, ss = ctx.enc(alg, n, pk, ec)
    try:
        assert lib.pqcgpu_set_launch_shape(a, 3, 0, 0) == 0
        assert ctx.keypair(alg, n, kc) == (pk, sk)
        assert ctx.enc(alg, n, pk, ec) == (ct, ss)
    finally:
        lib.pqcgpu_set_launch_shape(a, 3, -1, 0)
    assert ctx.dec(alg, n, ct, sk) == ss


@pytest.mark.parametrize("poly_n", [1024, 512])
def test_restated_fixture(ctx, poly_n):
    from pqc_gb300 import kem
    alg = ALG[poly_n]
    s = kem.sizes(alg)
    g = load_golden("restated_%s.json" % alg)
    n = g["n"]
    seed = drbg.seed48(g["drbg_seed"])
    pk, sk = ctx.keypair(alg, n, drbg.stream(seed, b"kp", n * 32))
    ct, ss = ctx.enc(alg, n, pk, drbg.stream(seed, b"enc", n * 32))
    assert [sha(x) for x in split(pk, s["pk"])] == g["pk_sha256"]
    assert [sha(x) for x in split(ct, s["ct"])] == g["ct_sha256"]
    assert ss.hex() == g["ss"]


@pytest.mark.parametrize("shape", [(1, 32), (3, 96), (7, 64), (32, 256)])
def test_newhope512_launch_shapes_match_oracle(ctx, oracle, shape):
    """Odd and even instance counts per CTA (the half-warp NTT pairs two instances per warp and idles
    a half when the count is odd) give the same bytes at every shape."""
    import ctypes

    from pqc_gb300 import _lib, kem
    lib = _lib.load()
    alg = "newhope512"
    a = oracle.ALG_NAMES[alg]
    n = 45
    seed = drbg.seed48(77)
    kc = drbg.stream(seed, b"kp", n * 32)
    ec = drbg.stream(seed, b"enc", n * 32)
    opk, osk = oracle.batch_keypair(a, n, kc)
    oct_, oss = oracle.batch_enc(a, n, opk, ec)
    saved = []
    for op in range(3):
        ni, thr = ctypes.c_int(), ctypes.c_int()
        assert lib.pqcgpu_get_launch_shape(kem.alg_id(alg), op, ctypes.byref(ni), ctypes.byref(thr)) == 0
        saved.append((ni.value, thr.value))
    try:
        for op in range(3):
            assert lib.pqcgpu_set_launch_shape(kem.alg_id(alg), op, *shape) == 0
        assert ctx.keypair(alg, n, kc) == (opk, osk)
        assert ctx.enc(alg, n, opk, ec) == (oct_, oss)
        assert ctx.dec(alg, n, oct_, osk) == oss
    finally:
        for op in range(3):
            lib.pqcgpu_set_launch_shape(kem.alg_id(alg), op, *saved[op])
