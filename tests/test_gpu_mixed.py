"""Mixed batches (pqcgpu_kem_mixed_batch), CUDA-graph capture / replay and the autotuner: every
output bit-exact against the per-algorithm batched calls (themselves checked against the oracle)."""
import random

import pytest

from pqc_gb300 import drbg

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def env():
    import torch
    from pqc_gb300 import kem
    c = kem.Context(0)
    yield c, torch, torch.device("cuda:0")
    c.close()


def make_case(torch, dev, alg, op, n, seed):
    """Inputs and output buffers for one job, plus the expected outputs from the single-alg API."""
    from pqc_gb300 import kem
    s = kem.sizes(alg)
    up = lambda b: torch.frombuffer(bytearray(b), dtype=torch.uint8).to(dev)
    kc = drbg.stream(seed, b"kp", n * s["kp_coins"])
    return s, up, kc


def build_jobs(ctx, torch, dev, spec, seed_base):
    """spec: list of (alg, op, n). Returns (jobs, expected) with expected from the batched calls."""
    from pqc_gb300 import kem
    jobs, expected, keep = [], [], []
    for idx, (alg, op, n) in enumerate(spec):
        s = kem.sizes(alg)
        seed = drbg.seed48(seed_base + idx)
        up = lambda b: torch.frombuffer(bytearray(b), dtype=torch.uint8).to(dev)
        kc = drbg.stream(seed, b"kp", n * s["kp_coins"])
        ec = drbg.stream(seed, b"enc", n * s["enc_coins"])
        pk, sk = ctx.keypair(alg, n, kc)
        ct, ss = ctx.enc(alg, n, pk, ec)
        if op == "keypair":
            ins, outs, exp = (up(kc), None), (torch.empty(n * s["pk"], dtype=torch.uint8, device=dev),
                                              torch.empty(n * s["sk"], dtype=torch.uint8, device=dev)), (pk, sk)
        elif op == "enc":
            ins, outs, exp = (up(pk), up(ec)), (torch.empty(n * s["ct"], dtype=torch.uint8, device=dev),
                                                torch.empty(n * s["ss"], dtype=torch.uint8, device=dev)), (ct, ss)
        else:
            ins, outs, exp = (up(ct), up(sk)), (torch.empty(n * s["ss"], dtype=torch.uint8, device=dev), None), (ss, None)
        jobs.append((alg, op, n, ins[0], ins[1], outs[0], outs[1]))
        expected.append(exp)
    return jobs, expected


def check(jobs, expected):
    for (alg, op, n, _, _, o0, o1), (e0, e1) in zip(jobs, expected):
        assert bytes(o0.cpu().numpy()) == e0, (alg, op, n)
        if e1 is not None:
            assert bytes(o1.cpu().numpy()) == e1, (alg, op, n)


@pytest.mark.parametrize("stage_kernels", [False, True])
def test_mixed_batch_all_algorithms(env, stage_kernels):
    """Every algorithm and operation in one mixed batch: each job's own kernels over the streams, or
    (STAGE_KERNELS) the persistent waves of the Kyber, NewHope and FrodoKEM jobs; every output equal
    to the single-algorithm calls'."""
    from pqc_gb300 import kem
    ctx, torch, dev = env
    rng = random.Random(5)
    algs = ["kyber512", "kyber768", "kyber1024", "kyber1024r2", "newhope1024", "frodo976", "mlkem768", "newhope512",
            "frodo640", "frodo1344"]
    spec = []
    for alg in algs:
        for op in ("keypair", "enc", "dec"):
            spec.append((alg, op, rng.randint(1, 3) if alg.startswith("frodo") else rng.randint(1, 700)))
    rng.shuffle(spec)
    jobs, expected = build_jobs(ctx, torch, dev, spec, 3000)
    torch.cuda.synchronize()
    ctx.mixed_dev(jobs, kem.STAGE_KERNELS if stage_kernels else 0)
    ctx.wait()
    check(jobs, expected)


def test_mixed_frodo_waves_every_split(env):
    """FrodoKEM jobs of all three parameter sets in the persistent waves (STAGE_KERNELS) at batch
    sizes that take each row split of B' = S'A + E' (1, 2, 4 and 8 tiles an instance) and the
    key generation's row tiles; outputs equal to the single-algorithm calls'."""
    from pqc_gb300 import kem
    ctx, torch, dev = env
    spec = [("frodo640", "enc", 320), ("frodo976", "dec", 160), ("frodo1344", "enc", 80), ("frodo640", "dec", 9),
            ("frodo976", "keypair", 40), ("frodo1344", "keypair", 5), ("frodo976", "enc", 17), ("frodo1344", "dec", 2)]
    jobs, expected = build_jobs(ctx, torch, dev, spec, 4600)
    torch.cuda.synchronize()
    ctx.mixed_dev(jobs, kem.STAGE_KERNELS)
    ctx.wait()
    check(jobs, expected)


@pytest.mark.parametrize("stage_kernels", [False, True])
def test_mixed_kyber_uneven_sizes(env, stage_kernels):
    """The mixed-Kyber configuration: k = 2/3/4 at 40/40/20 (plus ML-KEM), uneven sizes, ops 1/3
    each; every job's own kernels, or one kernel per core stage for the Kyber jobs (STAGE_KERNELS)."""
    from pqc_gb300 import kem
    ctx, torch, dev = env
    rng = random.Random(11)
    spec = []
    for _ in range(12):
        alg = rng.choices(["kyber512", "kyber768", "kyber1024"], [0.4, 0.4, 0.2])[0]
        spec.append((alg, rng.choice(["keypair", "enc", "dec"]), rng.randint(1, 5000)))
    spec += [("mlkem768", "enc", 333), ("mlkem1024", "dec", 1500), ("kyber1024r2", "dec", 257)]
    jobs, expected = build_jobs(ctx, torch, dev, spec, 4000)
    torch.cuda.synchronize()
    ctx.mixed_dev(jobs, kem.STAGE_KERNELS if stage_kernels else 0)
    ctx.wait()
    check(jobs, expected)


@pytest.mark.parametrize("stage_kernels", [False, True])
def test_graph_replay(env, stage_kernels):
    from pqc_gb300 import kem
    ctx, torch, dev = env
    spec = [("kyber768", "enc", 3000), ("kyber768", "dec", 3000), ("kyber512", "keypair", 777), ("newhope1024", "enc", 100),
            ("kyber1024", "enc", 500)]
    jobs, expected = build_jobs(ctx, torch, dev, spec, 5000)
    torch.cuda.synchronize()
    g = ctx.graph(jobs, kem.STAGE_KERNELS if stage_kernels else 0)
    check(jobs, expected)  # the warm-up pass already computed the outputs
    for t in (j[5] for j in jobs):
        t.zero_()
    torch.cuda.synchronize()
    g.launch()
    ctx.wait()
    check(jobs, expected)
    # new inputs in the same buffers, replay again
    jobs2, expected2 = build_jobs(ctx, torch, dev, spec, 6000)
    for (a, b) in zip(jobs, jobs2):
        a[3].copy_(b[3])
        if a[4] is not None:
            a[4].copy_(b[4])
    torch.cuda.synchronize()
    g.launch()
    ctx.wait()
    check(jobs, expected2)
    g.close()


def test_autotune_roundtrip(env, tmp_path):
    """Tunes Kyber-768 at a small batch, saves and reloads the cache, and runs a mixed batch at the
    tuned shapes; the shapes in force before are restored afterwards, so later tests do not depend
    on this one's timing noise."""
    from pqc_gb300 import _lib, autotune
    lib = _lib.load()
    before = {op: autotune.get_shape(lib, "kyber768", op) for op in range(4)}
    try:
        t = autotune.tune(batch=2048, algs=("kyber768",), reps=1, log=lambda *a: None)
        assert set(t["shapes"]) == {"kyber768/0", "kyber768/1", "kyber768/2", "kyber768/3"}
        p = str(tmp_path / "tuning.json")
        autotune.save(t, p)
        assert autotune.load_cached(p, gpu_name=t["gpu"]) is not None
        ctx, torch, dev = env
        jobs, expected = build_jobs(ctx, torch, dev, [("kyber768", "enc", 999), ("kyber768", "dec", 999)], 7000)
        torch.cuda.synchronize()
        ctx.mixed_dev(jobs)
        ctx.wait()
        check(jobs, expected)
    finally:
        for op, sh in before.items():
            assert lib.pqcgpu_set_launch_shape(1, op, sh[0], sh[1]) == 0


@pytest.mark.parametrize("op,shape", [(1, (8, 96)), (1, (20, 192)), (2, (14, 256)), (2, (6, 64)), (3, (4, 64)),
                                      (3, (24, 384)), (0, (6, 96))])
def test_kyber768_non_default_shapes_match_oracle(env, oracle, op, shape):
    """Kyber-768 at launch shapes other than the defaults (including re-encryption at its 256-thread
    bound), against the oracle, with tampered ciphertexts for decapsulation."""
    from pqc_gb300 import _lib, autotune, kem
    ctx, torch, dev = env
    lib = _lib.load()
    before = autotune.get_shape(lib, "kyber768", op)
    alg, n = "kyber768", 777
    s = kem.sizes(alg)
    a = oracle.KYBER768
    seed = drbg.seed48(8800 + op)
    kc = drbg.stream(seed, b"kp", n * s["kp_coins"])
    ec = drbg.stream(seed, b"enc", n * s["enc_coins"])
    opk, osk = oracle.batch_keypair(a, n, kc)
    oct_, oss = oracle.batch_enc(a, n, opk, ec)
    bad = bytearray(oct_)
    for x in range(0, n, 4):
        bad[x * s["ct"] + (x * 13) % s["ct"]] ^= 0x08
    try:
        assert lib.pqcgpu_set_launch_shape(kem.alg_id(alg), op, shape[0], shape[1]) == 0
        if op == 0:
            assert ctx.keypair(alg, n, kc) == (opk, osk)
        elif op == 1:
            assert ctx.enc(alg, n, opk, ec) == (oct_, oss)
        else:
            assert ctx.dec(alg, n, bytes(bad), osk) == oracle.batch_dec(a, n, bytes(bad), osk)
    finally:
        assert lib.pqcgpu_set_launch_shape(kem.alg_id(alg), op, before[0], before[1]) == 0
