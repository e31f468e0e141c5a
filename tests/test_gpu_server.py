"""The serving loop: continuous batching gives every request the same bytes alone and in a mix,
keys stay resident, the memory budget is enforced, and the Poisson load generator runs."""
import random

import pytest

from pqc_gb300 import drbg

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def server():
    from pqc_gb300 import serve
    s = serve.Server(0, budget=4 << 30, max_inflight=4, max_batch=512)
    yield s
    s.close()


def test_keypair_enc_dec_match_batched_api(server):
    from pqc_gb300 import kem
    ctx = kem.Context(0)
    for alg in ("kyber512", "kyber768", "kyber1024", "kyber1024r2", "newhope1024", "frodo976", "mlkem768", "newhope512",
                "frodo640", "frodo1344"):
        s = kem.sizes(alg)
        seed = drbg.seed48(hash(alg) & 0xffff)
        kc = drbg.stream(seed, b"kp", s["kp_coins"])
        ec = drbg.stream(seed, b"enc", s["enc_coins"])
        key, pk = server.keypair(alg, kc)
        bpk, bsk = ctx.keypair(alg, 1, kc)
        assert pk == bpk, alg
        ct, ss = server.enc(alg, key=key, coins=ec)
        bct, bss = ctx.enc(alg, 1, bpk, ec)
        assert (ct, ss) == (bct, bss), alg
        assert server.enc(alg, pk=pk, coins=ec) == (ct, ss), alg  # by pk bytes instead of handle
        assert server.dec(alg, key, ct) == ss, alg
        server.release(key)
    ctx.close()


def test_each_result_same_alone_and_in_the_mix(server):
    rng = random.Random(3)
    algs = ["kyber512", "kyber768", "kyber1024", "newhope1024", "frodo976"]
    from pqc_gb300 import kem
    keys = {}
    for alg in algs:
        s = kem.sizes(alg)
        keys[alg] = [server.keypair(alg, drbg.stream(drbg.seed48(7), alg.encode() + bytes([i]), s["kp_coins"]))
                     for i in range(3)]
    reqs = []
    for i in range(300):
        alg = rng.choice(algs)
        s = kem.sizes(alg)
        op = rng.choice(["keypair", "enc", "dec"])
        coins = drbg.stream(drbg.seed48(100 + i), b"c", s["kp_coins"] if op == "keypair" else s["enc_coins"])
        key, pk = rng.choice(keys[alg])
        reqs.append((alg, op, key, coins))
    # ciphertexts for the decapsulations, produced alone first
    cts = {}
    for i, (alg, op, key, coins) in enumerate(reqs):
        if op == "dec":
            cts[i] = server.enc(alg, key=key, coins=drbg.stream(drbg.seed48(900 + i), b"e", kem.sizes(alg)["enc_coins"]))[0]

    def run(i, alg, op, key, coins):
        if op == "keypair":
            return server.submit(alg, 0, inp=coins)
        if op == "enc":
            return server.submit(alg, 1, key=key, inp=coins)
        return server.submit(alg, 2, key=key, inp=cts[i])

    def strip(op, res):
        return res[1] if op == "keypair" else res  # keypair: compare the pk bytes, not the handle

    alone = [strip(op, server.wait(run(i, alg, op, key, coins))) for i, (alg, op, key, coins) in enumerate(reqs)]
    tickets = [run(i, *r) for i, r in enumerate(reqs)]  # all in flight together
    mixed = [strip(r[1], server.wait(t)) for r, t in zip(reqs, tickets)]
    assert alone == mixed
    st = server.stats()
    assert st["completed"] > 0 and st["p99_ms"] > 0


def test_bad_key_and_budget():
    from pqc_gb300 import serve
    with serve.Server(0, budget=8 << 20, max_inflight=2, max_batch=64) as small:
        with pytest.raises(RuntimeError):
            small.keypair("frodo976")  # key store of 1024 FrodoKEM keys does not fit 8 MiB
        with pytest.raises(RuntimeError):
            small.dec("kyber768", (1 << 48) | 12345, bytes(1088))


def test_poisson_load(server):
    from pqc_gb300 import serve
    rep = server.run_poisson(serve.SERVING_MIX, rate=2000, seconds=0.5, seed=1)
    assert rep["completed"] == rep["submitted"] > 0
    assert 0 < rep["p50_ms"] <= rep["p99_ms"]


def _kernels_launched(lib, fn):
    """Names of the library kernels launched while fn runs (the library's launch profiler)."""
    import ctypes
    import json

    from pqc_gb300 import _lib
    buf = ctypes.create_string_buffer(1 << 16)
    _lib.check(lib.pqcgpu_profile_read(buf, len(buf)))  # drop older records
    lib.pqcgpu_profile_enable(1)
    try:
        fn()
    finally:
        lib.pqcgpu_profile_enable(0)
    _lib.check(lib.pqcgpu_profile_read(buf, len(buf)))
    return set(json.loads(buf.value.decode()))


def test_newhope_requests_take_the_batched_kernels(server):
    """The serving loop runs NewHope on its batched kernels at every batch size: the
    single-instance kernels, which a direct call of a small batch takes, crowd the FrodoKEM
    requests beside them under load.  Same bytes either way."""
    from pqc_gb300 import _lib, kem
    lib = _lib.load()
    alg = "newhope1024"
    s = kem.sizes(alg)
    seed = drbg.seed48(91)
    kc, ec = drbg.stream(seed, b"kp", s["kp_coins"]), drbg.stream(seed, b"enc", s["enc_coins"])
    out = {}

    def served():
        key, pk = server.keypair(alg, kc)
        ct, ss = server.enc(alg, key=key, coins=ec)
        out["served"] = (pk, ct, ss, server.dec(alg, key, ct))
        server.release(key)

    names = _kernels_launched(lib, served)
    assert {"nh_kp_core<1024,0>", "nh_enc_core<1024,0>", "nh_dec_core<1024,0>"} <= names, names
    assert not any("single" in n for n in names), names
    ctx = kem.Context(0)

    def direct():
        pk, sk = ctx.keypair(alg, 1, kc)
        ct, ss = ctx.enc(alg, 1, pk, ec)
        out["direct"] = (pk, ct, ss, ctx.dec(alg, 1, ct, sk))

    names = _kernels_launched(lib, direct)
    ctx.close()
    assert {"nh_kp_single<1024,0>", "nh_enc_single<1024,0>"} <= names, names
    assert out["served"] == out["direct"]
    assert out["served"][2] == out["served"][3]
