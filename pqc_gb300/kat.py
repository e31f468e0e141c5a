"""NIST known-answer-test (.rsp) files for the KEMs of this library, generated or checked on the GPU.

    python -m pqc_gb300.kat --alg kyber768 --count 100 --out PQCkemKAT_2400.rsp
    python -m pqc_gb300.kat --alg kyber768 --check PQCkemKAT_2400.rsp

The flow is the NIST PQC KAT generator's:
* the DRBG is the AES-256 CTR_DRBG instantiated with entropy 0, 1, ..., 47;
* each count's 48-byte seed is one 48-byte draw from it;
* the DRBG is then re-instantiated with that seed before the count's crypto_kem_keypair and
  crypto_kem_enc, and their coins come from it in the calls the algorithm's submission package
  makes (`pqcgpu_nist_coins`).

This module derives every count's coins that way on the host and then runs all counts as single
batched keypair / encapsulation / decapsulation calls on the GPU. The bytes equal those of calling
the single-instance crypto_kem_* once per count. `--check` regenerates the pk, sk, ct and ss of
every record of an existing .rsp file from its seed and reports the first difference.
"""
import argparse
import ctypes
import sys

from . import _lib, kem

ALG_NAMES = {
    "kyber512": "Kyber512", "kyber768": "Kyber768", "kyber1024": "Kyber1024",
    "kyber1024r2": "Kyber1024-round2", "newhope1024": "NewHope1024-CPAKEM", "newhope512": "NewHope512-CPAKEM",
    "frodo976": "FrodoKEM-976-SHAKE", "frodo640": "FrodoKEM-640-SHAKE", "frodo1344": "FrodoKEM-1344-SHAKE",
    "mlkem512": "ML-KEM-512", "mlkem768": "ML-KEM-768",
    "mlkem1024": "ML-KEM-1024",
}


def _draw(lib, n):
    buf = ctypes.create_string_buffer(n)
    _lib.check(lib.pqcgpu_randombytes(buf, n))
    return buf.raw


def seeds(count):
    """The per-count seeds: 48-byte draws of the CTR_DRBG instantiated with 0..47."""
    lib = _lib.load()
    _lib.check(lib.pqcgpu_randombytes_init_nist(bytes(range(48)), None))
    return [_draw(lib, 48) for _ in range(count)]


def coins_for(alg, seed):
    """(keypair coins, encapsulation coins) of one count, as its crypto_kem_* calls draw them."""
    lib = _lib.load()
    s = kem.sizes(alg)
    _lib.check(lib.pqcgpu_randombytes_init_nist(seed, None))
    kc = ctypes.create_string_buffer(s["kp_coins"])
    ec = ctypes.create_string_buffer(s["enc_coins"])
    _lib.check(lib.pqcgpu_nist_coins(kem.alg_id(alg), 0, kc))
    _lib.check(lib.pqcgpu_nist_coins(kem.alg_id(alg), 1, ec))
    return kc.raw[:s["kp_coins"]], ec.raw[:s["enc_coins"]]


def records(alg, seed_list, ctx=None):
    """KAT records (dicts of count, seed, pk, sk, ct, ss) for the given seeds, computed in batches."""
    s = kem.sizes(alg)
    n = len(seed_list)
    kcs, ecs = zip(*(coins_for(alg, sd) for sd in seed_list)) if n else ((), ())
    own = ctx is None
    ctx = ctx or kem.Context(0)
    try:
        pk, sk = ctx.keypair(alg, n, b"".join(kcs))
        ct, ss = ctx.enc(alg, n, pk, b"".join(ecs))
        ss2 = ctx.dec(alg, n, ct, sk)
    finally:
        if own:
            ctx.close()
    if ss2 != ss:
        raise RuntimeError("decapsulation disagrees with encapsulation")
    cut = lambda b, sz, i: b[i * sz:(i + 1) * sz]  # noqa: E731
    return [{"count": i, "seed": seed_list[i], "pk": cut(pk, s["pk"], i), "sk": cut(sk, s["sk"], i),
             "ct": cut(ct, s["ct"], i), "ss": cut(ss, s["ss"], i)} for i in range(n)]


def format_rsp(alg, recs):
    out = ["# %s\n\n" % ALG_NAMES[alg]]
    for r in recs:
        out.append("count = %d\n" % r["count"])
        for f in ("seed", "pk", "sk", "ct", "ss"):
            out.append("%s = %s\n" % (f, r[f].hex().upper()))
        out.append("\n")
    return "".join(out)


def parse_rsp(text):
    recs, cur = [], None
    for line in text.splitlines():
        line = line.strip()
        if not line or line.startswith("#"):
            continue
        key, _, val = (p.strip() for p in line.partition("="))
        if key == "count":
            cur = {"count": int(val)}
            recs.append(cur)
        elif cur is not None and key in ("seed", "pk", "sk", "ct", "ss"):
            cur[key] = bytes.fromhex(val)
    return recs


def generate(alg, count):
    return format_rsp(alg, records(alg, seeds(count)))


def check(alg, text):
    """Returns (number of records checked, None) or (index, field) of the first mismatch."""
    want = parse_rsp(text)
    got = records(alg, [r["seed"] for r in want])
    for w, g in zip(want, got):
        for f in ("pk", "sk", "ct", "ss"):
            if f in w and w[f] != g[f]:
                return w["count"], f
    return len(want), None


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--alg", required=True, choices=sorted(ALG_NAMES))
    ap.add_argument("--count", type=int, default=100)
    ap.add_argument("--out", help="write the .rsp here (default: stdout)")
    ap.add_argument("--check", help="verify an existing .rsp file")
    a = ap.parse_args(argv)
    if a.check:
        with open(a.check) as f:
            n, field = check(a.alg, f.read())
        if field:
            print("MISMATCH at count %d: %s" % (n, field))
            return 1
        print("ok: %d records of %s match" % (n, a.check))
        return 0
    text = generate(a.alg, a.count)
    if a.out:
        with open(a.out, "w") as f:
            f.write(text)
    else:
        sys.stdout.write(text)
    return 0


if __name__ == "__main__":
    sys.exit(main())
