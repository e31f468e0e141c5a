"""Kyber on the GPU through the C ABI, bit-exact against the reference's own code (round-2 CPA
golden vectors) and the CPU oracle (round-3 KEM)."""
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


@pytest.mark.parametrize("k", [2, 3, 4])
def test_r2_cpa_matches_reference_vectors(ctx, k):
    g = load_golden("ref_kyber_r2_k%d_cpa.json" % k)
    n = g["n"]
    d, m, coins = (bytes.fromhex(g[x]) for x in ("d", "m", "coins"))
    pk, sk = ctx.kyber_cpa_keypair(2, k, n, d)
    from pqc_gb300.kem import kyber_cpa_sizes
    s = kyber_cpa_sizes(2, k)
    assert [sha(x) for x in split(pk, s["pk"])] == g["pk_sha256"]
    assert [sha(x) for x in split(sk, s["sk"])] == g["sk_sha256"]
    ct = ctx.kyber_cpa_enc(2, k, n, m, pk, coins)
    assert [sha(x) for x in split(ct, s["ct"])] == g["ct_sha256"]
    assert ctx.kyber_cpa_dec(2, k, n, ct, sk).hex() == g["m_dec"]


@pytest.mark.parametrize("variant,k", [(3, 2), (3, 3), (3, 4), (2, 4)])
@pytest.mark.parametrize("n", [1, 17, 33, 130])
def test_cpa_matches_oracle(ctx, oracle, variant, k, n):
    seed = drbg.seed48(1000 + n)
    d = drbg.stream(seed, b"d", 32 * n)
    m = drbg.stream(seed, b"m", 32 * n)
    coins = drbg.stream(seed, b"coins", 32 * n)
    pk, sk = ctx.kyber_cpa_keypair(variant, k, n, d)
    ct = ctx.kyber_cpa_enc(variant, k, n, m, pk, coins)
    md = ctx.kyber_cpa_dec(variant, k, n, ct, sk)
    s = oracle.kyber_sizes(variant, k)
    for x in range(n):
        opk, osk = oracle.kyber_indcpa_keypair(variant, k, d[32 * x:32 * x + 32])
        assert pk[x * s["pk"]:(x + 1) * s["pk"]] == opk, x
        assert sk[x * s["sk_cpa"]:(x + 1) * s["sk_cpa"]] == osk, x
        oct_ = oracle.kyber_indcpa_enc(variant, k, m[32 * x:32 * x + 32], opk, coins[32 * x:32 * x + 32])
        assert ct[x * s["ct"]:(x + 1) * s["ct"]] == oct_, x
    assert md == m


@pytest.mark.parametrize("alg", ["kyber512", "kyber768", "kyber1024", "kyber1024r2", "mlkem512", "mlkem768",
                                 "mlkem1024"])
@pytest.mark.parametrize("n", [1, 31, 257, 768, 1536, 4099])
def test_kem_matches_oracle(ctx, oracle, alg, n):
    from pqc_gb300 import kem
    s = kem.sizes(alg)
    a = oracle.ALG_NAMES[alg]
    seed = drbg.seed48(n)
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


@pytest.mark.parametrize("alg", ["kyber512", "kyber768", "kyber1024", "kyber1024r2", "mlkem512", "mlkem768",
                                 "mlkem1024"])
# 768 and 2048: the key selection leaves the CTA and the KDF runs after it, hashes a warp per
# instance; 4096: the same with the hashes a thread per instance
@pytest.mark.parametrize("n", [64, 768, 2048, 4096])
def test_kem_implicit_rejection(ctx, oracle, alg, n):
    from pqc_gb300 import kem
    s = kem.sizes(alg)
    a = oracle.ALG_NAMES[alg]
    seed = drbg.seed48(77)
    pk, sk = ctx.keypair(alg, n, drbg.stream(seed, b"kp", n * s["kp_coins"]))
    ct, ss = ctx.enc(alg, n, pk, drbg.stream(seed, b"enc", n * s["enc_coins"]))
    bad = bytearray(ct)
    for x in range(0, n, 2):  # tamper every other instance at a different byte
        bad[x * s["ct"] + (x * 37) % s["ct"]] ^= 1 << (x % 8)
    got = ctx.dec(alg, n, bytes(bad), sk)
    assert got == oracle.batch_dec(a, n, bytes(bad), sk)
    for x in range(n):
        same = got[x * 32:(x + 1) * 32] == ss[x * 32:(x + 1) * 32]
        assert same == (x % 2 == 1), x


@pytest.mark.parametrize("name", ["kyber512", "kyber768", "kyber1024", "kyber1024r2", "mlkem512", "mlkem768",
                                  "mlkem1024"])
def test_restated_fixtures(ctx, name):
    from pqc_gb300 import kem
    g = load_golden("restated_%s.json" % name)
    s = kem.sizes(name)
    n = g["n"]
    seed = drbg.seed48(g["drbg_seed"])
    pk, sk = ctx.keypair(name, n, drbg.stream(seed, b"kp", n * s["kp_coins"]))
    ct, ss = ctx.enc(name, n, pk, drbg.stream(seed, b"enc", n * s["enc_coins"]))
    assert [sha(x) for x in split(pk, s["pk"])] == g["pk_sha256"]
    assert [sha(x) for x in split(sk, s["sk"])] == g["sk_sha256"]
    assert [sha(x) for x in split(ct, s["ct"])] == g["ct_sha256"]
    assert ss.hex() == g["ss"]
    assert ctx.dec(name, n, ct, sk).hex() == g["ss"]


def test_device_pointer_path_matches_host_path(ctx):
    import torch
    from pqc_gb300 import kem
    alg, n = "kyber768", 1000
    s = kem.sizes(alg)
    seed = drbg.seed48(5)
    kc = drbg.stream(seed, b"kp", n * s["kp_coins"])
    ec = drbg.stream(seed, b"enc", n * s["enc_coins"])
    pk, sk = ctx.keypair(alg, n, kc)
    ct, ss = ctx.enc(alg, n, pk, ec)
    dev = torch.device("cuda:0")
    t = lambda b: torch.frombuffer(bytearray(b), dtype=torch.uint8).to(dev)
    dpk, dsk, dct = (torch.empty(n * s[x], dtype=torch.uint8, device=dev) for x in ("pk", "sk", "ct"))
    dss, dss2 = (torch.empty(n * 32, dtype=torch.uint8, device=dev) for _ in range(2))
    dkc, dec_ = t(kc), t(ec)  # inputs must outlive the asynchronous calls
    torch.cuda.synchronize()
    ctx.keypair_dev(alg, n, dpk, dsk, dkc)
    ctx.enc_dev(alg, n, dct, dss, dpk, dec_)
    ctx.dec_dev(alg, n, dss2, dct, dsk)
    ctx.wait()
    assert bytes(dpk.cpu().numpy()) == pk
    assert bytes(dsk.cpu().numpy()) == sk
    assert bytes(dct.cpu().numpy()) == ct
    assert bytes(dss.cpu().numpy()) == ss
    assert bytes(dss2.cpu().numpy()) == ss


def test_deterministic_replay(ctx):
    alg, n = "kyber768", 2048
    seed = drbg.seed48(9)
    from pqc_gb300 import kem
    s = kem.sizes(alg)
    kc = drbg.stream(seed, b"kp", n * s["kp_coins"])
    assert ctx.keypair(alg, n, kc) == ctx.keypair(alg, n, kc)


def test_nist_single_instance_api(oracle):
    import ctypes
    from pqc_gb300 import _lib
    lib = _lib.load()
    seed = bytes(range(48))
    for name, a in (("kyber512", 0), ("kyber768", 1), ("kyber1024", 2)):
        s = oracle.alg_sizes(a)
        pk = ctypes.create_string_buffer(s["pk"])
        sk = ctypes.create_string_buffer(s["sk"])
        ct = ctypes.create_string_buffer(s["ct"])
        ss = ctypes.create_string_buffer(32)
        ss2 = ctypes.create_string_buffer(32)
        assert lib.pqcgpu_randombytes_init(seed) == 0
        assert getattr(lib, "pqcgpu_%s_crypto_kem_keypair" % name)(pk, sk) == 0
        assert getattr(lib, "pqcgpu_%s_crypto_kem_enc" % name)(ct, ss, pk) == 0
        assert getattr(lib, "pqcgpu_%s_crypto_kem_dec" % name)(ss2, ct, sk) == 0
        assert ss.raw == ss2.raw
        stream = hashlib.shake_256(seed).digest(s["kp_coins"] + s["enc_coins"])
        opk, osk = oracle.batch_keypair(a, 1, stream[:s["kp_coins"]])
        assert pk.raw == opk and sk.raw == osk
        oct_, oss = oracle.batch_enc(a, 1, opk, stream[s["kp_coins"]:])
        assert ct.raw == oct_ and ss.raw == oss


@pytest.mark.parametrize("alg", ["kyber512", "kyber768", "kyber1024", "kyber1024r2"])
def test_plain_path_matches_oracle(ctx, oracle, alg):
    """The per-stage baseline path (flag PQCGPU_PLAIN) produces the same bytes as the oracle."""
    from pqc_gb300 import kem
    s = kem.sizes(alg)
    a = oracle.ALG_NAMES[alg]
    n = 300
    seed = drbg.seed48(31)
    kc = drbg.stream(seed, b"kp", n * s["kp_coins"])
    ec = drbg.stream(seed, b"enc", n * s["enc_coins"])
    pk, sk = ctx.keypair(alg, n, kc, flags=kem.PLAIN)
    opk, osk = oracle.batch_keypair(a, n, kc)
    assert (pk, sk) == (opk, osk)
    ct, ss = ctx.enc(alg, n, pk, ec, flags=kem.PLAIN)
    oct_, oss = oracle.batch_enc(a, n, pk, ec)
    assert (ct, ss) == (oct_, oss)
    bad = bytearray(ct)
    bad[7] ^= 4
    assert ctx.dec(alg, n, bytes(bad), sk, flags=kem.PLAIN) == oracle.batch_dec(a, n, bytes(bad), sk)


@pytest.mark.parametrize("alg", ["kyber512", "kyber768", "kyber1024", "kyber1024r2", "mlkem512", "mlkem768",
                                  "mlkem1024"])
@pytest.mark.parametrize("n", [1, 33, 300])
def test_single_instance_and_batched_paths_match_oracle(ctx, oracle, alg, n):
    """Small KEM batches run on the single-instance kernels (one CTA per instance) up to a size
    threshold per k and operation (launch-shape op 4 sets every operation of a k; -1 restores the
    measured defaults); both that path and the batched chains must give the oracle's bytes,
    including implicit rejection."""
    from pqc_gb300 import _lib, kem
    lib = _lib.load()
    s = kem.sizes(alg)
    a = oracle.ALG_NAMES[alg]
    seed = drbg.seed48(7000 + n)
    kc = drbg.stream(seed, b"kp", n * s["kp_coins"])
    ec = drbg.stream(seed, b"enc", n * s["enc_coins"])
    opk, osk = oracle.batch_keypair(a, n, kc)
    oct_, oss = oracle.batch_enc(a, n, opk, ec)
    bad = bytearray(oct_)
    for x in range(0, n, 2):
        bad[x * s["ct"] + (x * 53) % s["ct"]] ^= 1 << (x % 8)
    orej = oracle.batch_dec(a, n, bytes(bad), osk)
    try:
        for limit in (4096, 0):  # every batch single-instance, then never
            assert lib.pqcgpu_set_launch_shape(kem.alg_id(alg), 4, limit, 0) == 0
            assert ctx.keypair(alg, n, kc) == (opk, osk), limit
            assert ctx.enc(alg, n, opk, ec) == (oct_, oss), limit
            assert ctx.dec(alg, n, oct_, osk) == oss, limit
            assert ctx.dec(alg, n, bytes(bad), osk) == orej, limit
    finally:
        assert lib.pqcgpu_set_launch_shape(kem.alg_id(alg), 4, -1, 0) == 0
