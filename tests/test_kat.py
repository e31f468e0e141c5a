"""NIST KAT harness (pqc_gb300/kat.py): the committed .rsp fixtures (CTR_DRBG seeds and coins,
oracle outputs) are reproduced by the oracle on CPU and by the GPU path through the C ABI."""
import os

import pytest

from conftest import GOLDEN

ALGS = ["kyber512", "kyber768", "kyber1024", "newhope1024", "frodo976", "mlkem512", "mlkem768", "mlkem1024",
        "newhope512", "frodo640", "frodo1344"]


def _fixture(name):
    with open(os.path.join(GOLDEN, "kat_%s.rsp" % name)) as f:
        return f.read()


@pytest.mark.parametrize("name", ALGS)
def test_kat_fixture_reproduced_by_oracle(oracle, name):
    from pqc_gb300 import kat
    text = _fixture(name)
    recs = kat.parse_rsp(text)
    assert [r["seed"] for r in recs] == kat.seeds(len(recs))
    alg = oracle.ALG_NAMES[name]
    for r in recs:
        kc, ec = kat.coins_for(name, r["seed"])
        pk, sk = oracle.batch_keypair(alg, 1, kc)
        ct, ss = oracle.batch_enc(alg, 1, pk, ec)
        assert (pk, sk, ct, ss) == (r["pk"], r["sk"], r["ct"], r["ss"]), r["count"]
    assert kat.format_rsp(name, recs) == text


@pytest.mark.gpu
@pytest.mark.parametrize("name", ALGS)
def test_kat_fixture_reproduced_on_gpu(name):
    from pqc_gb300 import kat
    text = _fixture(name)
    n = len(kat.parse_rsp(text))
    assert kat.generate(name, n) == text
    assert kat.check(name, text) == (n, None)


@pytest.mark.gpu
def test_single_instance_nist_api_draws_the_kat_coins():
    """crypto_kem_keypair / enc of the NIST single-instance API, DRBG re-instantiated with a KAT seed,
    give the record's keys and ciphertext (the same coins as the batched harness)."""
    import ctypes

    from pqc_gb300 import _lib, kat, kem
    lib = _lib.load()
    for name in ("kyber768", "mlkem768", "frodo976"):
        r = kat.parse_rsp(_fixture(name))[0]
        s = kem.sizes(name)
        pk, sk = ctypes.create_string_buffer(s["pk"]), ctypes.create_string_buffer(s["sk"])
        ct, ss = ctypes.create_string_buffer(s["ct"]), ctypes.create_string_buffer(s["ss"])
        assert lib.pqcgpu_randombytes_init_nist(r["seed"], None) == 0
        assert getattr(lib, "pqcgpu_%s_crypto_kem_keypair" % name)(pk, sk) == 0
        assert getattr(lib, "pqcgpu_%s_crypto_kem_enc" % name)(ct, ss, pk) == 0
        assert (pk.raw, sk.raw, ct.raw, ss.raw) == (r["pk"], r["sk"], r["ct"], r["ss"]), name
    lib.pqcgpu_randombytes_init(bytes(48))
