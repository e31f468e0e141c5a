"""Generate tests/golden/fips203_mlkem{768,1024}.json from an independent FIPS 203 implementation.

The `cryptography` package (50.x, OpenSSL backend) implements ML-KEM-768 and ML-KEM-1024.  It
shares no code with this repository, so its outputs pin the K-PKE arithmetic (12-bit rejection
sampling, CBD eta = 2, NTT, du / dv compression, byte encodings) and the FIPS 203 KEM layer of the
GPU path.  The GPU machine has no `cryptography`, so its answers are committed here:

    python tests/golden/gen_fips203.py

For each batch size n in (1, 1025, 65536) the batch inputs are the same DRBG streams the GPU test
draws (pqc_gb300.drbg, labels b"kp" and b"enc"); a sample of instance indices spread over every
CTA-sized region of the batch carries:
  * pk_sha256  -- SHA-256 of cryptography's encapsulation key for seed d || z
                  (MLKEM*PrivateKey.from_seed_bytes(d || z)), the coins of that instance;
  * ct_sha256, ss -- the encapsulation with message m = the instance's enc coins.  cryptography has
                  no deterministic encapsulation, so these bytes come from the oracle and are kept
                  only after cryptography's decapsulation of that ciphertext returned the same ss;
and a smaller subset ("foreign") carries a ciphertext made by cryptography's own encapsulate(),
its shared secret, and the implicit-rejection key cryptography returns for the same ciphertext
with one bit flipped (byte (37 i) mod |ct|, bit i mod 8, i the instance index).
"""
import base64
import hashlib
import json
import os
import random
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import pyoracle as O  # noqa: E402
from pqc_gb300 import drbg  # noqa: E402

CASES = ((1, 301), (1025, 302), (65536, 303))


def sample_indices(n, count, seed):
    """One index from each of `count` equal strata of [0, n) plus both ends of the batch."""
    if n <= count:
        return list(range(n))
    rng = random.Random(seed)
    idx = {0, n - 1}
    for s in range(count):
        lo, hi = s * n // count, (s + 1) * n // count
        idx.add(rng.randrange(lo, hi))
    return sorted(idx)


def tamper(ct, i):
    b = bytearray(ct)
    b[(37 * i) % len(b)] ^= 1 << (i % 8)
    return bytes(b)


def generate(name):
    from cryptography.hazmat.primitives.asymmetric import mlkem
    cls = {"mlkem768": mlkem.MLKEM768PrivateKey, "mlkem1024": mlkem.MLKEM1024PrivateKey}[name]
    a = O.ALG_NAMES[name]
    s = O.alg_sizes(a)
    cases = []
    for n, sd in CASES:
        seed = drbg.seed48(sd)
        kc = drbg.stream(seed, b"kp", n * s["kp_coins"])
        ec = drbg.stream(seed, b"enc", n * s["enc_coins"])
        idx = sample_indices(n, 256, sd)
        foreign = idx if n == 1 else sample_indices(n, 48 if n > 2048 else 16, sd + 1)
        recs = []
        for i in idx:
            d_z = kc[i * 64:(i + 1) * 64]
            key = cls.from_seed_bytes(d_z)
            pk = key.public_key().public_bytes_raw()
            opk, osk = O.batch_keypair(a, 1, d_z)
            assert opk == pk, (name, n, i)
            ct, ss = O.batch_enc(a, 1, pk, ec[i * 32:(i + 1) * 32])
            assert key.decapsulate(ct) == ss, (name, n, i)
            recs.append({"i": i, "pk_sha256": hashlib.sha256(pk).hexdigest(),
                         "ct_sha256": hashlib.sha256(ct).hexdigest(), "ss": ss.hex()})
        frs = []
        for i in foreign:
            key = cls.from_seed_bytes(kc[i * 64:(i + 1) * 64])
            ss, ct = key.public_key().encapsulate()
            rej = key.decapsulate(tamper(ct, i))
            assert rej != ss
            frs.append({"i": i, "ct_b64": base64.b64encode(ct).decode(), "ss": ss.hex(), "tampered_ss": rej.hex()})
        cases.append({"n": n, "drbg_seed": sd, "samples": recs, "foreign": frs})
    out = {
        "source": "cryptography %s ML-KEM (FIPS 203, OpenSSL backend), independent of this repository" %
                  __import__("cryptography").__version__,
        "alg": name,
        "labels": {"keypair_coins": "kp (d || z per instance)", "enc_coins": "enc (m per instance)"},
        "tamper": "byte (37 i) mod len(ct), bit i mod 8",
        "cases": cases,
    }
    with open(os.path.join(HERE, "fips203_%s.json" % name), "w") as f:
        json.dump(out, f, indent=0, sort_keys=True)
        f.write("\n")


if __name__ == "__main__":
    for nm in ("mlkem768", "mlkem1024"):
        generate(nm)
    print("fixtures written to", HERE)
