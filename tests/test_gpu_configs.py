"""Parity at the benchmark configurations' own sizes, against the CPU oracle.

* C1: Kyber-512, 256 keypair -> encaps -> decaps chains, every input from the DRBG of integer seed 0;
  pk, sk, ct and ss equal the oracle's for every chain.
* Kyber-768 at the headline batch of 65536: every output equals the oracle's.
* C2: NewHope-1024 CPA-KEM at 16384: every output equals the oracle's.
* C4: FrodoKEM-976 at 2048 (a distinct seedA per key): the GPU runs the whole batch; the oracle
  (about 40 ms per instance and operation on one core) recomputes 96 instances sampled over the
  batch, and every decapsulation of the batch is checked against its encapsulation.
* C3: the mixed Kyber batch (24 launches, k = 2/3/4 at 40/40/20, n ~ U{1..65536}, 780690
  instances), through the mixed-batch call with each job's own kernels and with one kernel per
  core stage; the oracle recomputes up to 512 instances of every job, sampled over its batch.
Instances are independent, so the oracle's outputs for a sample of them are exactly the batch's
outputs at those indices.
"""
import random

import pytest

from pqc_gb300 import drbg

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    from pqc_gb300 import kem
    c = kem.Context(0)
    yield c
    c.close()


def rows(b, sz, idx):
    return b"".join(b[i * sz:(i + 1) * sz] for i in idx)


def sample(n, count, seed):
    if n <= count:
        return list(range(n))
    rng = random.Random(seed)
    idx = {0, n - 1}
    for s in range(count - 2):
        idx.add(rng.randrange(s * n // (count - 2), (s + 1) * n // (count - 2)))
    return sorted(idx)


@pytest.mark.parametrize("alg,n,seed_no", [("kyber512", 256, 0), ("kyber768", 65536, 1), ("newhope1024", 16384, 2)])
def test_config_full_batch_matches_oracle(ctx, oracle, alg, n, seed_no):
    from pqc_gb300 import kem
    s = kem.sizes(alg)
    a = oracle.ALG_NAMES[alg]
    seed = drbg.seed48(seed_no)
    kc = drbg.stream(seed, b"kp", n * s["kp_coins"])
    ec = drbg.stream(seed, b"enc", n * s["enc_coins"])
    pk, sk = ctx.keypair(alg, n, kc)
    ct, ss = ctx.enc(alg, n, pk, ec)
    ss2 = ctx.dec(alg, n, ct, sk)
    opk, osk = oracle.batch_keypair(a, n, kc)
    assert pk == opk
    assert sk == osk
    oct_, oss = oracle.batch_enc(a, n, opk, ec)
    assert ct == oct_
    assert ss == oss
    assert ss2 == oss
    # implicit rejection over the whole batch (NewHope's CPA-KEM has no re-encryption check)
    if alg.startswith("kyber"):
        bad = bytearray(ct)
        for x in range(0, n, 3):
            bad[x * s["ct"] + (x * 29) % s["ct"]] ^= 1 << (x % 8)
        assert ctx.dec(alg, n, bytes(bad), sk) == oracle.batch_dec(a, n, bytes(bad), sk)


def test_c4_frodo976_batch_2048(ctx, oracle):
    from pqc_gb300 import kem
    alg, n = "frodo976", 2048
    s = kem.sizes(alg)
    a = oracle.FRODO976
    seed = drbg.seed48(4)
    kc = drbg.stream(seed, b"kp", n * s["kp_coins"])
    ec = drbg.stream(seed, b"enc", n * s["enc_coins"])
    pk, sk = ctx.keypair(alg, n, kc)
    ct, ss = ctx.enc(alg, n, pk, ec)
    assert ctx.dec(alg, n, ct, sk) == ss
    idx = sample(n, 96, 44)
    opk, osk = oracle.batch_keypair(a, len(idx), rows(kc, s["kp_coins"], idx))
    assert rows(pk, s["pk"], idx) == opk
    assert rows(sk, s["sk"], idx) == osk
    oct_, oss = oracle.batch_enc(a, len(idx), opk, rows(ec, s["enc_coins"], idx))
    assert rows(ct, s["ct"], idx) == oct_
    assert rows(ss, s["ss"], idx) == oss
    # distinct seedA per key: the first 16 bytes of pk differ across the sample
    assert len({pk[i * s["pk"]:i * s["pk"] + 16] for i in idx}) == len(idx)
    bad = bytearray(ct)
    for j, i in enumerate(idx[::4]):
        bad[i * s["ct"] + (j * 131) % s["ct"]] ^= 0x20
    got = ctx.dec(alg, n, bytes(bad), sk)
    tidx = idx[::4]
    assert rows(got, s["ss"], tidx) == oracle.batch_dec(a, len(tidx), rows(bytes(bad), s["ct"], tidx),
                                                         rows(sk, s["sk"], tidx))


@pytest.mark.parametrize("stage_kernels", [False, True])
def test_c3_mixed_kyber_full_size(ctx, oracle, stage_kernels):
    import torch
    from pqc_gb300 import kem
    from pqc_gb300.workload import mixed_kyber_spec
    dev = torch.device("cuda:0")
    up = lambda b: torch.frombuffer(bytearray(b), dtype=torch.uint8).to(dev)  # noqa: E731
    spec = mixed_kyber_spec()
    assert sum(n for _, _, n in spec) == 780690
    jobs, host = [], []
    for j, (alg, op, n) in enumerate(spec):
        s = kem.sizes(alg)
        seed = drbg.seed48(200 + j)
        kc = drbg.stream(seed, b"kp", n * s["kp_coins"])
        if op == "keypair":
            jobs.append((alg, op, n, up(kc), None, torch.empty(n * s["pk"], dtype=torch.uint8, device=dev),
                         torch.empty(n * s["sk"], dtype=torch.uint8, device=dev)))
            host.append((kc, None))
            continue
        pk, sk = ctx.keypair(alg, n, kc)
        ec = drbg.stream(seed, b"enc", n * s["enc_coins"])
        if op == "enc":
            jobs.append((alg, op, n, up(pk), up(ec), torch.empty(n * s["ct"], dtype=torch.uint8, device=dev),
                         torch.empty(n * s["ss"], dtype=torch.uint8, device=dev)))
            host.append((pk, ec))
        else:
            ct, _ = ctx.enc(alg, n, pk, ec)
            bad = bytearray(ct)
            for x in range(0, n, 5):  # every fifth instance tampered: implicit rejection inside the mix
                bad[x * s["ct"] + (x * 41) % s["ct"]] ^= 1 << (x % 8)
            jobs.append((alg, op, n, up(bytes(bad)), up(sk), torch.empty(n * s["ss"], dtype=torch.uint8, device=dev),
                         None))
            host.append((bytes(bad), sk))
    torch.cuda.synchronize()
    ctx.mixed_dev(jobs, kem.STAGE_KERNELS if stage_kernels else 0)
    ctx.wait()
    for j, ((alg, op, n, _, _, o0, o1), (h0, h1)) in enumerate(zip(jobs, host)):
        s = kem.sizes(alg)
        a = oracle.ALG_NAMES[alg]
        idx = sample(n, 512, j)
        out0 = bytes(o0.cpu().numpy())
        if op == "keypair":
            opk, osk = oracle.batch_keypair(a, len(idx), rows(h0, s["kp_coins"], idx))
            assert rows(out0, s["pk"], idx) == opk, (j, alg, op, n)
            assert rows(bytes(o1.cpu().numpy()), s["sk"], idx) == osk, (j, alg, op, n)
        elif op == "enc":
            oct_, oss = oracle.batch_enc(a, len(idx), rows(h0, s["pk"], idx), rows(h1, s["enc_coins"], idx))
            assert rows(out0, s["ct"], idx) == oct_, (j, alg, op, n)
            assert rows(bytes(o1.cpu().numpy()), s["ss"], idx) == oss, (j, alg, op, n)
        else:
            oss = oracle.batch_dec(a, len(idx), rows(h0, s["ct"], idx), rows(h1, s["sk"], idx))
            assert rows(out0, s["ss"], idx) == oss, (j, alg, op, n)
