"""CPU oracle pinned against the golden fixtures (hashlib and the reference's own code)."""
import hashlib

import pytest

from conftest import load_golden
from pqc_gb300 import drbg


def sha(b):
    return hashlib.sha256(b).hexdigest()


def split(b, sz):
    return [b[i * sz:(i + 1) * sz] for i in range(len(b) // sz)]


def test_keccak_vectors(oracle):
    g = load_golden("keccak.json")
    for v in g["vectors"]:
        data = bytes.fromhex(v["in"])
        assert oracle.shake128(data, 256).hex() == v["shake128_256"]
        assert oracle.shake256(data, 256).hex() == v["shake256_256"]
        assert oracle.sha3_256(data).hex() == v["sha3_256"]
        assert oracle.sha3_512(data).hex() == v["sha3_512"]


@pytest.mark.parametrize("k", [2, 3, 4])
def test_kyber_r2_cpa_matches_reference(oracle, k):
    g = load_golden("ref_kyber_r2_k%d_cpa.json" % k)
    d, m, coins = (bytes.fromhex(g[x]) for x in ("d", "m", "coins"))
    for x in range(g["n"]):
        pk, sk = oracle.kyber_indcpa_keypair(2, k, d[32 * x:32 * x + 32])
        assert sha(pk) == g["pk_sha256"][x]
        assert sha(sk) == g["sk_sha256"][x]
        ct = oracle.kyber_indcpa_enc(2, k, m[32 * x:32 * x + 32], pk, coins[32 * x:32 * x + 32])
        assert sha(ct) == g["ct_sha256"][x]
        assert oracle.kyber_indcpa_dec(2, k, ct, sk).hex() == g["m_dec"][64 * x:64 * x + 64]
        if x == 0:
            assert (pk.hex(), sk.hex(), ct.hex()) == (g["pk0"], g["sk0"], g["ct0"])


@pytest.mark.parametrize("poly_n", [1024, 512])
def test_newhope_cpa_matches_reference(oracle, poly_n):
    """The CPA-PKE restatement against the reference's own NewHope_NIST_GPU code (n = 512: built
    with NEWHOPE_N=512 and the reference's scalar 512-point transform)."""
    g = load_golden("ref_newhope%d_cpa.json" % poly_n)
    seed, m, coins = (bytes.fromhex(g[x]) for x in ("seed", "m", "coins"))
    for x in range(g["n"]):
        pk, sk = oracle.newhope_cpapke_keypair(seed[32 * x:32 * x + 32], poly_n)
        assert sha(pk) == g["pk_sha256"][x]
        assert sha(sk) == g["sk_sha256"][x]
        ct = oracle.newhope_cpapke_enc(m[32 * x:32 * x + 32], pk, coins[32 * x:32 * x + 32], poly_n)
        assert sha(ct) == g["ct_sha256"][x]
        assert oracle.newhope_cpapke_dec(ct, sk, poly_n).hex() == g["m_dec"][64 * x:64 * x + 64]


@pytest.mark.parametrize("name", ["kyber512", "kyber768", "kyber1024", "kyber1024r2", "newhope1024", "frodo976",
                                  "mlkem512", "mlkem768", "mlkem1024", "newhope512", "frodo640", "frodo1344"])
def test_restated_kem_vectors(oracle, name):
    g = load_golden("restated_%s.json" % name)
    alg = oracle.ALG_NAMES[name]
    sz = oracle.alg_sizes(alg)
    n = g["n"]
    seed = drbg.seed48(g["drbg_seed"])
    pk, sk = oracle.batch_keypair(alg, n, drbg.stream(seed, b"kp", n * sz["kp_coins"]))
    ct, ss = oracle.batch_enc(alg, n, pk, drbg.stream(seed, b"enc", n * sz["enc_coins"]))
    assert [sha(x) for x in split(pk, sz["pk"])] == g["pk_sha256"]
    assert [sha(x) for x in split(sk, sz["sk"])] == g["sk_sha256"]
    assert [sha(x) for x in split(ct, sz["ct"])] == g["ct_sha256"]
    assert ss.hex() == g["ss"]
    assert oracle.batch_dec(alg, n, ct, sk) == ss


@pytest.mark.parametrize("name", ["kyber512", "kyber768", "kyber1024", "kyber1024r2", "frodo976", "mlkem512",
                                  "mlkem768", "mlkem1024"])
def test_implicit_rejection(oracle, name):
    """A tampered ciphertext decapsulates to a different key (Kyber / Frodo: the z / s fallback).
    NewHope's CPA-KEM has no re-encryption check, so a small ciphertext change may decode to the
    same message; it is not part of this test."""
    alg = oracle.ALG_NAMES[name]
    sz = oracle.alg_sizes(alg)
    n = 2
    seed = drbg.seed48(7)
    pk, sk = oracle.batch_keypair(alg, n, drbg.stream(seed, b"kp", n * sz["kp_coins"]))
    ct, ss = oracle.batch_enc(alg, n, pk, drbg.stream(seed, b"enc", n * sz["enc_coins"]))
    bad = bytearray(ct)
    bad[3] ^= 0x40
    bad[2 * sz["ct"] - 1] ^= 0x01
    ss2 = oracle.batch_dec(alg, n, bytes(bad), sk)
    assert ss2[:sz["ss"]] != ss[:sz["ss"]]
    assert ss2[sz["ss"]:] != ss[sz["ss"]:]
    assert oracle.batch_dec(alg, n, ct, sk) == ss


def test_work_counters(oracle):
    """Kyber-768 encaps + decaps: permutation / butterfly counts used as the algorithmic work unit."""
    sz = oracle.alg_sizes(oracle.KYBER768)
    seed = drbg.seed48(0)
    pk, sk = oracle.batch_keypair(oracle.KYBER768, 1, drbg.stream(seed, b"kp", sz["kp_coins"]), nthreads=1)
    oracle.counters_reset()
    ct, ss = oracle.batch_enc(oracle.KYBER768, 1, pk, drbg.stream(seed, b"enc", sz["enc_coins"]), nthreads=1)
    oracle.batch_dec(oracle.KYBER768, 1, ct, sk, nthreads=1)
    perms, bfly = oracle.counters()
    assert 90 <= perms <= 110
    assert bfly == (3 + 4 + 3 + 1 + 3 + 4) * 896


@pytest.mark.parametrize("k", [2, 3, 4])
def test_mlkem_hash_layer_against_hashlib(oracle, k):
    """The FIPS 203 steps that differ from round 3, checked with hashlib on the oracle's outputs:
    rho = G(d || k)[:32] ends the encapsulation key; H(ek) and z sit at the end of dk; the shared
    key is G(m || H(ek))[:32]; a rejected ciphertext decapsulates to J(z || c) = SHAKE256(z || c, 32)."""
    import hashlib
    alg = oracle.ALG_NAMES["mlkem%d" % {2: 512, 3: 768, 4: 1024}[k]]
    sz = oracle.alg_sizes(alg)
    seed = drbg.seed48(600 + k)
    coins = drbg.stream(seed, b"kp", sz["kp_coins"])
    m = drbg.stream(seed, b"enc", 32)
    pk, sk = oracle.batch_keypair(alg, 1, coins)
    d, z = coins[:32], coins[32:64]
    assert pk[-32:] == hashlib.sha3_512(d + bytes([k])).digest()[:32]
    assert sk[-64:-32] == hashlib.sha3_256(pk).digest()
    assert sk[-32:] == z
    assert sk[384 * k:384 * k + len(pk)] == pk
    ct, ss = oracle.batch_enc(alg, 1, pk, m)
    assert ss == hashlib.sha3_512(m + hashlib.sha3_256(pk).digest()).digest()[:32]
    assert oracle.batch_dec(alg, 1, ct, sk) == ss
    bad = bytearray(ct)
    bad[len(bad) // 2] ^= 0x10
    assert oracle.batch_dec(alg, 1, bytes(bad), sk) == hashlib.shake_256(z + bytes(bad)).digest(32)
    # the module rank in G separates ML-KEM keys from round-3 keys of the same seed
    kpk, _ = oracle.batch_keypair(alg - 6, 1, coins)
    assert kpk != pk


def _fips203_tamper(ct, i):
    b = bytearray(ct)
    b[(37 * i) % len(b)] ^= 1 << (i % 8)
    return bytes(b)


@pytest.mark.parametrize("name", ["mlkem768", "mlkem1024"])
def test_mlkem_oracle_against_fips203_fixtures(oracle, name):
    """The oracle against the committed answers of an independent FIPS 203 implementation (the
    `cryptography` package, tests/golden/gen_fips203.py): encapsulation keys, the encapsulation of
    sampled instances (whose ciphertexts that implementation decapsulated to the same key), its own
    ciphertexts decapsulated here, and its implicit-rejection keys for tampered ciphertexts."""
    import base64
    g = load_golden("fips203_%s.json" % name)
    alg = oracle.ALG_NAMES[name]
    sz = oracle.alg_sizes(alg)
    for case in g["cases"]:
        n = case["n"]
        seed = drbg.seed48(case["drbg_seed"])
        kc = drbg.stream(seed, b"kp", n * sz["kp_coins"])
        ec = drbg.stream(seed, b"enc", n * sz["enc_coins"])
        keys = {}
        for r in case["samples"][:64]:
            i = r["i"]
            pk, sk = oracle.batch_keypair(alg, 1, kc[i * 64:(i + 1) * 64])
            keys[i] = sk
            assert sha(pk) == r["pk_sha256"], (n, i)
            ct, ss = oracle.batch_enc(alg, 1, pk, ec[i * 32:(i + 1) * 32])
            assert sha(ct) == r["ct_sha256"], (n, i)
            assert ss.hex() == r["ss"], (n, i)
        for f in case["foreign"][:8]:
            i = f["i"]
            sk = keys.get(i) or oracle.batch_keypair(alg, 1, kc[i * 64:(i + 1) * 64])[1]
            ct = base64.b64decode(f["ct_b64"])
            assert oracle.batch_dec(alg, 1, ct, sk).hex() == f["ss"], (n, i)
            assert oracle.batch_dec(alg, 1, _fips203_tamper(ct, i), sk).hex() == f["tampered_ss"], (n, i)


@pytest.mark.parametrize("name", ["mlkem768", "mlkem1024"])
def test_mlkem_oracle_against_cryptography_live(oracle, name):
    """The same four checks against the `cryptography` package itself, on 20 fresh seeds, where it is
    installed (it is not on every machine that runs these tests)."""
    import os
    mlkem = pytest.importorskip("cryptography.hazmat.primitives.asymmetric.mlkem")
    cls = {"mlkem768": mlkem.MLKEM768PrivateKey, "mlkem1024": mlkem.MLKEM1024PrivateKey}[name]
    alg = oracle.ALG_NAMES[name]
    for t in range(20):
        d_z, m = os.urandom(64), os.urandom(32)
        key = cls.from_seed_bytes(d_z)
        pk, sk = oracle.batch_keypair(alg, 1, d_z)
        assert pk == key.public_key().public_bytes_raw()
        ct, ss = oracle.batch_enc(alg, 1, pk, m)
        assert key.decapsulate(ct) == ss
        ss_c, ct_c = key.public_key().encapsulate()
        assert oracle.batch_dec(alg, 1, ct_c, sk) == ss_c
        bad = _fips203_tamper(ct_c, t)
        assert oracle.batch_dec(alg, 1, bad, sk) == key.decapsulate(bad)


def test_frodo976_oracle_matches_reference(oracle):
    """The FrodoKEM-976 restatement against the reference's own host KEM flow (FrodoKEM_GPU/kem.c)
    with the reference's sampler, pack / unpack, SHAKE, A generation and matrix kernels
    (tests/golden/ref_frodo976_kem.json): keys, ciphertexts, shared secrets, and the implicit
    rejection of a tampered ciphertext."""
    g = load_golden("ref_frodo976_kem.json")
    a = oracle.FRODO976
    sz = oracle.alg_sizes(a)
    n = g["n"]
    seed = drbg.seed48(g["drbg_seed"])
    pk, sk = oracle.batch_keypair(a, n, drbg.stream(seed, b"kp", n * sz["kp_coins"]))
    ct, ss = oracle.batch_enc(a, n, pk, drbg.stream(seed, b"enc", n * sz["enc_coins"]))
    assert [sha(x) for x in split(pk, sz["pk"])] == g["pk_sha256"]
    assert [sha(x) for x in split(sk, sz["sk"])] == g["sk_sha256"]
    assert [sha(x) for x in split(ct, sz["ct"])] == g["ct_sha256"]
    assert [x.hex() for x in split(ss, sz["ss"])] == g["ss"]
    bad = bytearray(ct)
    for i in range(n):
        bad[i * sz["ct"] + (37 * i + 11) % sz["ct"]] ^= 1 << (i % 8)
    got = oracle.batch_dec(a, n, bytes(bad), sk)
    assert [x.hex() for x in split(got, sz["ss"])] == g["tampered_ss"]
