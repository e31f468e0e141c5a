"""ML-KEM-768 / -1024 on the GPU against an independent FIPS 203 implementation.

The answers come from the `cryptography` package (OpenSSL backend), committed as fixtures by
tests/golden/gen_fips203.py because the GPU machine does not have that package.  At batch sizes
1, 1025 and 65536 (the Kyber-768 headline batch), for instances sampled from every CTA-sized region
of the batch:
  * the batched keypair's encapsulation key equals cryptography's for the same seed d || z;
  * the batched encapsulation's ciphertext and shared key are the ones cryptography decapsulates
    back to that key;
  * ciphertexts made by cryptography's own encapsulate() decapsulate on the GPU to its shared key;
  * the same ciphertexts with one bit flipped decapsulate to cryptography's implicit-rejection key
    J(z || c).
Round-3 Kyber shares the K-PKE arithmetic these checks exercise (the same kernels run it); only
G(d) against G(d || k) and the KEM hash layer differ.
"""
import base64
import hashlib

import pytest

from conftest import load_golden
from pqc_gb300 import drbg

pytestmark = pytest.mark.gpu


def sha(b):
    return hashlib.sha256(b).hexdigest()


def tamper(ct, i):
    b = bytearray(ct)
    b[(37 * i) % len(b)] ^= 1 << (i % 8)
    return bytes(b)


@pytest.fixture(scope="module")
def ctx():
    from pqc_gb300 import kem
    c = kem.Context(0)
    yield c
    c.close()


@pytest.mark.parametrize("name", ["mlkem768", "mlkem1024"])
@pytest.mark.parametrize("case_no", [0, 1, 2])
def test_mlkem_matches_fips203_implementation(ctx, name, case_no):
    from pqc_gb300 import kem
    g = load_golden("fips203_%s.json" % name)
    case = g["cases"][case_no]
    n = case["n"]
    s = kem.sizes(name)
    seed = drbg.seed48(case["drbg_seed"])
    kc = drbg.stream(seed, b"kp", n * s["kp_coins"])
    ec = drbg.stream(seed, b"enc", n * s["enc_coins"])
    pk, sk = ctx.keypair(name, n, kc)
    ct, ss = ctx.enc(name, n, pk, ec)
    for r in case["samples"]:
        i = r["i"]
        assert sha(pk[i * s["pk"]:(i + 1) * s["pk"]]) == r["pk_sha256"], i
        assert sha(ct[i * s["ct"]:(i + 1) * s["ct"]]) == r["ct_sha256"], i
        assert ss[i * 32:(i + 1) * 32].hex() == r["ss"], i
    # cryptography's ciphertexts, intact and tampered, in place of the GPU's own at their indices
    good, bad = bytearray(ct), bytearray(ct)
    for f in case["foreign"]:
        i = f["i"]
        c = base64.b64decode(f["ct_b64"])
        good[i * s["ct"]:(i + 1) * s["ct"]] = c
        bad[i * s["ct"]:(i + 1) * s["ct"]] = tamper(c, i)
    got = ctx.dec(name, n, bytes(good), sk)
    rej = ctx.dec(name, n, bytes(bad), sk)
    foreign = {f["i"] for f in case["foreign"]}
    for f in case["foreign"]:
        i = f["i"]
        assert got[i * 32:(i + 1) * 32].hex() == f["ss"], i
        assert rej[i * 32:(i + 1) * 32].hex() == f["tampered_ss"], i
    # every other instance still decapsulates its own ciphertext to its encapsulated key
    for i in range(n):
        if i not in foreign:
            assert got[i * 32:(i + 1) * 32] == ss[i * 32:(i + 1) * 32], i
