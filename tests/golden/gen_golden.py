"""Generate the committed golden fixtures in tests/golden/.

Run here (x86 container with the reference tree) after `oracle/build_ref.sh`:
    python tests/golden/gen_golden.py

Fixture kinds:
  * keccak.json     -- FIPS-202 outputs from Python hashlib (independent implementation).
  * ref_*.json      -- outputs of the reference's OWN device code (Kyber_GPU_Batched for k = 2/3/4,
                       round-2 semantics; NewHope_NIST_GPU for n = 1024 and n = 512), compiled for
                       the host by oracle/build_ref.sh and driven with the NIST per-instance seed
                       layout; and of the reference's FrodoKEM-976 host KEM flow (FrodoKEM_GPU/
                       kem.c with its sampler, pack / unpack, SHAKE and matrix kernels, run with
                       CTA barriers through oracle/ref_shim_sync).
  * kat_*.rsp       -- NIST-format KAT records (AES-256 CTR_DRBG seeds and coins, oracle outputs).
  * restated_*.json -- outputs of the CPU oracle for paths the reference has no code for (Kyber
                       round-3 KEM, NewHope CPA-KEM, FrodoKEM-976, ML-KEM): regression pins, parity
                       unpinned by reference outputs.
Inputs come from pqc_gb300.drbg with fixed seeds; every output is stored as SHA-256 per instance,
and instance 0 is also stored in full.
"""
import ctypes
import hashlib
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import pyoracle as O  # noqa: E402
from pqc_gb300 import drbg  # noqa: E402

REF = os.path.join(ROOT, "oracle", "_ref")


def h(b):
    return hashlib.sha256(b).hexdigest()


def chunks(b, sz):
    return [b[i * sz:(i + 1) * sz] for i in range(len(b) // sz)]


def dump(name, obj):
    with open(os.path.join(HERE, name), "w") as f:
        json.dump(obj, f, indent=1, sort_keys=True)
        f.write("\n")


def keccak():
    vec = []
    seed = drbg.seed48(100)
    for i, n in enumerate([0, 1, 31, 32, 33, 71, 72, 73, 135, 136, 137, 167, 168, 169, 500, 1184, 2400]):
        data = drbg.stream(seed, b"keccak%d" % i, n)
        vec.append({
            "in": data.hex(),
            "shake128_256": hashlib.shake_128(data).hexdigest(256),
            "shake256_256": hashlib.shake_256(data).hexdigest(256),
            "sha3_256": hashlib.sha3_256(data).hexdigest(),
            "sha3_512": hashlib.sha3_512(data).hexdigest(),
        })
    dump("keccak.json", {"source": "python hashlib", "vectors": vec})


def ref_kyber(k, n=16, s=1):
    L = ctypes.CDLL(os.path.join(REF, "librefkyber%d.so" % k))
    sz = O.kyber_sizes(2, k)
    seed = drbg.seed48(s)
    d = drbg.stream(seed, b"d", 32 * n)
    m = drbg.stream(seed, b"m", 32 * n)
    coins = drbg.stream(seed, b"coins", 32 * n)
    pk = ctypes.create_string_buffer(n * sz["pk"])
    sk = ctypes.create_string_buffer(n * sz["sk_cpa"])
    ct = ctypes.create_string_buffer(n * sz["ct"])
    m2 = ctypes.create_string_buffer(32 * n)
    assert L.ref_kyber_cpa_keypair(n, pk, sk, d) == 0
    assert L.ref_kyber_cpa_enc(n, ct, m, pk.raw, coins) == 0
    assert L.ref_kyber_cpa_dec(n, m2, ct.raw, sk.raw) == 0
    dump("ref_kyber_r2_k%d_cpa.json" % k, {
        "source": "reference Kyber_GPU_Batched device code (KYBER_K=%d), host-compiled via oracle/build_ref.sh" % k,
        "variant": 2, "k": k, "n": n, "drbg_seed": s,
        "d": d.hex(), "m": m.hex(), "coins": coins.hex(),
        "pk_sha256": [h(x) for x in chunks(pk.raw, sz["pk"])],
        "sk_sha256": [h(x) for x in chunks(sk.raw, sz["sk_cpa"])],
        "ct_sha256": [h(x) for x in chunks(ct.raw, sz["ct"])],
        "m_dec": m2.raw.hex(),
        "pk0": pk.raw[:sz["pk"]].hex(), "sk0": sk.raw[:sz["sk_cpa"]].hex(), "ct0": ct.raw[:sz["ct"]].hex(),
    })


def ref_newhope(n=16, s=2, poly_n=1024):
    L = ctypes.CDLL(os.path.join(REF, "librefnewhope.so" if poly_n == 1024 else "librefnewhope512.so"))
    pkb, skb, ctb = O.NEWHOPE_CPA_SIZES[poly_n]
    seed = drbg.seed48(s)
    kp = drbg.stream(seed, b"d", 32 * n)
    m = drbg.stream(seed, b"m", 32 * n)
    coins = drbg.stream(seed, b"coins", 32 * n)
    pk = ctypes.create_string_buffer(n * pkb)
    sk = ctypes.create_string_buffer(n * skb)
    ct = ctypes.create_string_buffer(n * ctb)
    m2 = ctypes.create_string_buffer(32 * n)
    assert L.ref_newhope_cpa_keypair(n, pk, sk, kp) == 0
    assert L.ref_newhope_cpa_enc(n, ct, m, pk.raw, coins) == 0
    assert L.ref_newhope_cpa_dec(n, m2, ct.raw, sk.raw) == 0
    src = "reference NewHope_NIST_GPU device code, host-compiled via oracle/build_ref.sh"
    if poly_n == 512:
        src += " (NEWHOPE_N=512, with the reference's scalar n = 512 ntt applied per instance)"
    dump("ref_newhope%d_cpa.json" % poly_n, {
        "source": src,
        "n": n, "drbg_seed": s, "seed": kp.hex(), "m": m.hex(), "coins": coins.hex(),
        "pk_sha256": [h(x) for x in chunks(pk.raw, pkb)],
        "sk_sha256": [h(x) for x in chunks(sk.raw, skb)],
        "ct_sha256": [h(x) for x in chunks(ct.raw, ctb)],
        "m_dec": m2.raw.hex(),
        "pk0": pk.raw[:pkb].hex(), "sk0": sk.raw[:skb].hex(), "ct0": ct.raw[:ctb].hex(),
    })


def ref_frodo976(n=3, s=6):
    """FrodoKEM-976 keypair / encapsulation / decapsulation by the reference's own code
    (oracle/_ref/librefrodo976.so, about 10 s per keypair: A.S runs 1024 CTAs of 128 host threads),
    plus the decapsulation of a tampered ciphertext (byte (37 i + 11) mod |ct|, bit i mod 8)."""
    L = ctypes.CDLL(os.path.join(REF, "librefrodo976.so"))
    sz = O.alg_sizes(O.FRODO976)
    seed = drbg.seed48(s)
    kc = drbg.stream(seed, b"kp", n * sz["kp_coins"])
    ec = drbg.stream(seed, b"enc", n * sz["enc_coins"])
    pks, sks, cts, sss, rej = [], [], [], [], []
    for i in range(n):
        pk = ctypes.create_string_buffer(sz["pk"])
        sk = ctypes.create_string_buffer(sz["sk"])
        ct = ctypes.create_string_buffer(sz["ct"])
        ss = ctypes.create_string_buffer(sz["ss"])
        ss2 = ctypes.create_string_buffer(sz["ss"])
        assert L.ref_frodo976_keypair(pk, sk, kc[i * sz["kp_coins"]:(i + 1) * sz["kp_coins"]]) == 0
        assert L.ref_frodo976_enc(ct, ss, pk.raw, ec[i * sz["enc_coins"]:(i + 1) * sz["enc_coins"]]) == 0
        assert L.ref_frodo976_dec(ss2, ct.raw, sk.raw) == 0 and ss2.raw == ss.raw
        bad = bytearray(ct.raw)
        bad[(37 * i + 11) % len(bad)] ^= 1 << (i % 8)
        assert L.ref_frodo976_dec(ss2, bytes(bad), sk.raw) == 0 and ss2.raw != ss.raw
        pks.append(h(pk.raw)), sks.append(h(sk.raw)), cts.append(h(ct.raw)), sss.append(ss.raw.hex())
        rej.append(ss2.raw.hex())
    dump("ref_frodo976_kem.json", {
        "source": "reference FrodoKEM_GPU host KEM flow (kem.c) with its sampler, pack/unpack, SHAKE and "
                  "matrix kernels, host-compiled via oracle/build_ref.sh (CTA barriers: oracle/ref_shim_sync)",
        "n": n, "drbg_seed": s, "labels": {"keypair_coins": "kp", "enc_coins": "enc"},
        "tamper": "byte (37 i + 11) mod len(ct), bit i mod 8",
        "pk_sha256": pks, "sk_sha256": sks, "ct_sha256": cts, "ss": sss, "tampered_ss": rej,
    })


def restated(name, alg, n, s):
    sz = O.alg_sizes(alg)
    seed = drbg.seed48(s)
    kc = drbg.stream(seed, b"kp", n * sz["kp_coins"])
    ec = drbg.stream(seed, b"enc", n * sz["enc_coins"])
    pk, sk = O.batch_keypair(alg, n, kc)
    ct, ss = O.batch_enc(alg, n, pk, ec)
    ss2 = O.batch_dec(alg, n, ct, sk)
    assert ss2 == ss
    dump("restated_%s.json" % name, {
        "source": "CPU oracle restatement (parity unpinned by reference outputs)",
        "alg": name, "n": n, "drbg_seed": s,
        "labels": {"keypair_coins": "kp", "enc_coins": "enc"},
        "pk_sha256": [h(x) for x in chunks(pk, sz["pk"])],
        "sk_sha256": [h(x) for x in chunks(sk, sz["sk"])],
        "ct_sha256": [h(x) for x in chunks(ct, sz["ct"])],
        "ss": ss.hex(),
    })


def kat_rsp(name, alg, count=3):
    """A NIST-format .rsp of `count` records, coins from the KAT CTR_DRBG flow (pqc_gb300.kat),
    keys / ciphertexts from the oracle: a regression pin for the harness and the GPU path."""
    from pqc_gb300 import kat
    seed_list = kat.seeds(count)
    sz = O.alg_sizes(alg)
    recs = []
    for i, sd in enumerate(seed_list):
        kc, ec = kat.coins_for(name, sd)
        pk, sk = O.batch_keypair(alg, 1, kc)
        ct, ss = O.batch_enc(alg, 1, pk, ec)
        assert O.batch_dec(alg, 1, ct, sk) == ss
        recs.append({"count": i, "seed": sd, "pk": pk, "sk": sk, "ct": ct, "ss": ss})
    assert all(len(r["pk"]) == sz["pk"] for r in recs)
    with open(os.path.join(HERE, "kat_%s.rsp" % name), "w") as f:
        f.write(kat.format_rsp(name, recs))


if __name__ == "__main__":
    keccak()
    for k in (2, 3, 4):
        ref_kyber(k)
    ref_newhope()
    ref_newhope(16, 3, 512)
    ref_frodo976()
    restated("kyber512", O.KYBER512, 16, 0)
    restated("kyber768", O.KYBER768, 16, 0)
    restated("kyber1024", O.KYBER1024, 16, 0)
    restated("kyber1024r2", O.KYBER1024_R2, 16, 0)
    restated("newhope1024", O.NEWHOPE1024, 16, 0)
    restated("newhope512", O.NEWHOPE512, 16, 0)
    restated("frodo640", O.FRODO640, 4, 0)
    restated("frodo1344", O.FRODO1344, 2, 0)
    restated("frodo976", O.FRODO976, 4, 0)
    restated("mlkem512", O.MLKEM512, 16, 0)
    restated("mlkem768", O.MLKEM768, 16, 0)
    restated("mlkem1024", O.MLKEM1024, 16, 0)
    for name in ("kyber512", "kyber768", "kyber1024", "newhope1024", "frodo976", "mlkem512", "mlkem768", "mlkem1024",
                 "newhope512", "frodo640", "frodo1344"):
        kat_rsp(name, O.ALG_NAMES[name], 1 if name.startswith("frodo") else 3)
    print("fixtures written to", HERE)
