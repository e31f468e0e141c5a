"""FrodoKEM-976, -640 and -1344 on the GPU through the C ABI, bit-exact against the oracle (restated
from the reference's host flow FrodoKEM_GPU/kem.c and its matrix kernels; -640 / -1344 with their
parameter sets), and FrodoKEM-976 against the reference's own code (its host KEM flow with its
sampler, codecs, SHAKE and matrix kernels: tests/golden/ref_frodo976_kem.json)."""
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


def test_frodo976_matches_reference_vectors(ctx):
    g = load_golden("ref_frodo976_kem.json")
    s = _sizes("frodo976")
    n = g["n"]
    seed = drbg.seed48(g["drbg_seed"])
    pk, sk = ctx.keypair("frodo976", n, drbg.stream(seed, b"kp", n * s["kp_coins"]))
    ct, ss = ctx.enc("frodo976", n, pk, drbg.stream(seed, b"enc", n * s["enc_coins"]))
    sha = lambda b: hashlib.sha256(b).hexdigest()  # noqa: E731
    rows = lambda b, sz: [b[i * sz:(i + 1) * sz] for i in range(n)]  # noqa: E731
    assert [sha(x) for x in rows(pk, s["pk"])] == g["pk_sha256"]
    assert [sha(x) for x in rows(sk, s["sk"])] == g["sk_sha256"]
    assert [sha(x) for x in rows(ct, s["ct"])] == g["ct_sha256"]
    assert [x.hex() for x in rows(ss, s["ss"])] == g["ss"]
    assert ctx.dec("frodo976", n, ct, sk) == ss
    bad = bytearray(ct)
    for i in range(n):
        bad[i * s["ct"] + (37 * i + 11) % s["ct"]] ^= 1 << (i % 8)
    assert [x.hex() for x in rows(ctx.dec("frodo976", n, bytes(bad), sk), s["ss"])] == g["tampered_ss"]


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


@pytest.mark.parametrize("alg", ALGS)
@pytest.mark.parametrize("product", [1, 2])
@pytest.mark.parametrize("n", [1, 17, 40])
def test_shared_key_encaps_matches_oracle(ctx, oracle, alg, product, n):
    """n encapsulations to one public key (A generated once, one matrix product on the CUDA cores
    (product 1) or the tensor cores (2)) give the per-instance encapsulation's bytes, and decapsulate
    to the same keys; tampered ciphertexts take the implicit-rejection key."""
    a, s = oracle.ALG_NAMES[alg], _sizes(alg)
    seed = drbg.seed48(9100 + n)
    pk, sk = oracle.batch_keypair(a, 1, drbg.stream(seed, b"kp", s["kp_coins"]))
    mu = drbg.stream(seed, b"enc", n * s["enc_coins"])
    ct, ss = ctx.frodo_enc_shared(alg, n, pk, mu, product=product)
    oct_, oss = oracle.batch_enc(a, n, pk * n, mu)
    assert ct == oct_
    assert ss == oss
    bad = bytearray(ct)
    for x in range(0, n, 3):
        bad[x * s["ct"] + (x * 89) % s["ct"]] ^= 0x04
    assert ctx.dec(alg, n, bytes(bad), sk * n) == oracle.batch_dec(a, n, bytes(bad), sk * n)


@pytest.mark.parametrize("alg", ALGS)
def test_shared_key_products_agree_at_2048(ctx, alg):
    """At 2048 instances (every tile of both products in use) the tensor-core and CUDA-core products
    and the per-instance path give the same ciphertexts and keys."""
    import torch
    s = _sizes(alg)
    n = 2048
    seed = drbg.seed48(9200)
    pk, _ = ctx.keypair(alg, 1, drbg.stream(seed, b"kp", s["kp_coins"]))
    mu = drbg.stream(seed, b"enc", n * s["enc_coins"])
    ref = ctx.enc(alg, n, pk * n, mu)
    for product in (1, 2):
        assert ctx.frodo_enc_shared(alg, n, pk, mu, product=product) == ref, product
    dev = torch.device("cuda:0")
    up = lambda b: torch.frombuffer(bytearray(b), dtype=torch.uint8).to(dev)  # noqa: E731
    dpk, dmu = up(pk), up(mu)
    dct = torch.empty(n * s["ct"], dtype=torch.uint8, device=dev)
    dss = torch.empty(n * s["ss"], dtype=torch.uint8, device=dev)
    torch.cuda.synchronize()
    ctx.frodo_enc_shared_dev(alg, n, dct, dss, dpk, dmu)
    ctx.wait()
    assert (bytes(dct.cpu().numpy()), bytes(dss.cpu().numpy())) == ref
