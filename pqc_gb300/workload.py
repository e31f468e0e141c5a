"""Fixed-size batched KEM workload on one GPU, for throughput checks and profiler captures.

    python -m pqc_gb300.workload --alg kyber768 --n 16384 --reps 2
    python -m pqc_gb300.workload --alg newhope512,frodo640 --n 16384,256 --reps 1
    python -m pqc_gb300.workload --alg frodo976 --n 2048 --ops shared --product 2
    python -m pqc_gb300.workload --mixed 8 --with-others --stage --reps 2

For each algorithm in turn (a comma list, with one batch size each or one for all): generates n key
pairs once, then runs `reps` rounds of encapsulation + decapsulation of n instances through the C
ABI with device buffers (`PQCGPU_DEVICE_PTRS`), timing each operation with CUDA events on the
library stream.  Inputs come from the seeded SHAKE-256 DRBG, so every run of the same command
launches the same kernels on the same data.  Exits non-zero if any decapsulated key differs from
the encapsulated one.  `--ops shared` (FrodoKEM) runs n encapsulations to the first key with the
shared-key call instead, on the CUDA-core or tensor-core product (`--product`).  `--mixed S` runs
the mixed Kyber batch (`mixed_kyber_spec`, every batch size divided by S; `--with-others` adds
NewHope-1024 / 512 and FrodoKEM-640 / 976 / 1344 jobs of every operation) through one mixed-batch
call per round, on the per-job kernels or (`--stage`) the persistent per-stage waves.
"""
import argparse
import sys

import torch

from . import drbg, kem


def mixed_kyber_spec(njobs=24, seed=12):
    """The mixed Kyber batch: per launch (job) a parameter set k = 2 / 3 / 4 with probabilities
    0.4 / 0.4 / 0.2, an operation keypair / enc / dec with 1/3 each, and a batch size drawn uniformly
    from 1..65536.  Returns [(alg, op, n)]; job j draws its inputs from DRBG seed 200 + j."""
    import random
    rng = random.Random(seed)
    spec = []
    for _ in range(njobs):
        alg = rng.choices(["kyber512", "kyber768", "kyber1024"], [0.4, 0.4, 0.2])[0]
        op = rng.choice(["keypair", "enc", "dec"])
        spec.append((alg, op, rng.randint(1, 65536)))
    return spec


def run(alg, n, reps, want, fl, product=None):
    ctx = kem.Context(0)
    s = kem.sizes(alg)
    dev = torch.device("cuda:0")
    seed = drbg.seed48(0)

    def dev_bytes(label, nbytes):
        return torch.frombuffer(bytearray(drbg.stream(seed, label, nbytes)), dtype=torch.uint8).to(dev)

    kc = dev_bytes(b"kp", n * s["kp_coins"])
    ec = dev_bytes(b"enc", n * s["enc_coins"])
    pk = torch.empty(n * s["pk"], dtype=torch.uint8, device=dev)
    sk = torch.empty(n * s["sk"], dtype=torch.uint8, device=dev)
    ct = torch.empty(n * s["ct"], dtype=torch.uint8, device=dev)
    ss = torch.empty(n * s["ss"], dtype=torch.uint8, device=dev)
    ss2 = torch.empty_like(ss)
    torch.cuda.synchronize()
    st = torch.cuda.ExternalStream(ctx.stream)
    ops = {
        "keypair": lambda: ctx.keypair_dev(alg, n, pk, sk, kc, fl),
        "enc": lambda: ctx.enc_dev(alg, n, ct, ss, pk, ec, fl),
        "dec": lambda: ctx.dec_dev(alg, n, ss2, ct, sk, fl),
        # FrodoKEM: n encapsulations to instance 0's key (pqcgpu_frodo_enc_shared_key_batch)
        "shared": lambda: ctx.frodo_enc_shared_dev(alg, n, ct, ss, pk[:s["pk"]], ec),
    }
    ops["keypair"]()
    ctx.wait()
    if product is not None:
        from ctypes import c_int
        from . import _lib
        _lib.check(_lib.load().pqcgpu_set_launch_shape(kem.alg_id(alg), 3, c_int(product), 0))
    ok = True
    for rep in range(reps):
        line = []
        for o in want:
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(st)
            ops[o]()
            e1.record(st)
            e1.synchronize()
            ms = e0.elapsed_time(e1)
            line.append("%s %.3f ms (%.2f M/s)" % (o, ms, n / ms / 1e3))
        if "enc" in want and "dec" in want:
            ctx.wait()
            same = torch.equal(ss, ss2)
            ok = ok and same
            line.append("ss match %s" % same)
        print("%s n=%d rep %d: %s" % (alg, n, rep, ", ".join(line)), flush=True)
    ctx.close()
    return ok


def mixed_jobs(scale, with_others):
    """[(alg, op, n)]: the mixed Kyber spec with every n divided by `scale` (at least 1), and with
    `with_others` one job of every operation of NewHope-1024 / 512 (4096 / scale instances) and of
    FrodoKEM-640 / 976 / 1344 (256 / scale)."""
    spec = [(alg, op, max(1, n // scale)) for alg, op, n in mixed_kyber_spec()]
    if with_others:
        for alg, n in (("newhope1024", 4096), ("newhope512", 4096), ("frodo640", 256), ("frodo976", 256),
                       ("frodo1344", 256)):
            spec += [(alg, op, max(1, n // scale)) for op in ("keypair", "enc", "dec")]
    return spec


def run_mixed(scale, with_others, stage, reps):
    """One mixed-batch call per round over mixed_jobs(); the decapsulated keys are checked against
    the encapsulations that made their ciphertexts."""
    ctx = kem.Context(0)
    dev = torch.device("cuda:0")
    jobs, keep, total = [], [], 0

    def dev_bytes(seed, label, nbytes):
        return torch.frombuffer(bytearray(drbg.stream(seed, label, nbytes)), dtype=torch.uint8).to(dev)

    for j, (alg, op, n) in enumerate(mixed_jobs(scale, with_others)):
        s = kem.sizes(alg)
        seed = drbg.seed48(200 + j)
        kc = dev_bytes(seed, b"kp", n * s["kp_coins"])
        pk, sk = (torch.empty(n * s[x], dtype=torch.uint8, device=dev) for x in ("pk", "sk"))
        ctx.keypair_dev(alg, n, pk, sk, kc)
        if op == "keypair":
            jobs.append((alg, op, n, kc, None, torch.empty_like(pk), torch.empty_like(sk)))
        else:
            ec = dev_bytes(seed, b"enc", n * s["enc_coins"])
            ct = torch.empty(n * s["ct"], dtype=torch.uint8, device=dev)
            ss = torch.empty(n * s["ss"], dtype=torch.uint8, device=dev)
            ctx.enc_dev(alg, n, ct, ss, pk, ec)
            if op == "enc":
                jobs.append((alg, op, n, pk, ec, torch.empty_like(ct), torch.empty_like(ss)))
            else:
                jobs.append((alg, op, n, ct, sk, torch.empty_like(ss), None))
                keep.append((len(jobs) - 1, ss))
        total += n
    ctx.wait()
    st = torch.cuda.ExternalStream(ctx.stream)
    ok = True
    for rep in range(reps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        ctx.mixed_dev(jobs, kem.STAGE_KERNELS if stage else 0)
        e1.record(st)
        e1.synchronize()
        ms = e0.elapsed_time(e1)
        same = all(torch.equal(jobs[i][5], ss) for i, ss in keep)
        ok = ok and same
        print("mixed %d jobs, %d instances, %s rep %d: %.3f ms (%.2f M ops/s), decaps match %s" %
              (len(jobs), total, "stage waves" if stage else "per job", rep, ms, total / ms / 1e3, same), flush=True)
    ctx.close()
    return ok


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--alg", default="kyber768", help="algorithm or comma list of: " + ", ".join(sorted(kem.ALGS)))
    ap.add_argument("--n", default="16384", help="batch size, or one per algorithm (comma list)")
    ap.add_argument("--reps", type=int, default=2)
    ap.add_argument("--ops", default="enc,dec", help="comma list of keypair, enc, dec to repeat")
    ap.add_argument("--plain", action="store_true", help="per-stage path instead of the fused kernels")
    ap.add_argument("--product", type=int, default=None,
                    help="FrodoKEM shared-key product for --ops shared: 1 CUDA cores, 2 tensor cores")
    ap.add_argument("--mixed", type=int, default=0, metavar="S",
                    help="run the mixed batch with every batch size divided by S instead")
    ap.add_argument("--with-others", action="store_true", help="--mixed: add NewHope and FrodoKEM jobs")
    ap.add_argument("--stage", action="store_true", help="--mixed: the persistent per-stage waves")
    args = ap.parse_args(argv)
    if args.mixed:
        return 0 if run_mixed(args.mixed, args.with_others, args.stage, args.reps) else 1
    algs = [a for a in args.alg.split(",") if a]
    ns = [int(x) for x in args.n.split(",") if x]
    if any(a not in kem.ALGS for a in algs):
        ap.error("unknown algorithm in %r" % args.alg)
    if len(ns) == 1:
        ns = ns * len(algs)
    if len(ns) != len(algs):
        ap.error("give one batch size, or one per algorithm")
    want = [o for o in args.ops.split(",") if o]
    for o in want:
        if o not in ("keypair", "enc", "dec", "shared"):
            ap.error("unknown op %r" % o)
    fl = kem.PLAIN if args.plain else 0
    ok = True
    for alg, n in zip(algs, ns):
        ok = run(alg, n, args.reps, want, fl, args.product) and ok
    return 0 if ok else 1


if __name__ == "__main__":
    sys.exit(main())
