"""Benchmark: Kyber-768 encapsulation + decapsulation throughput on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--batch B]
                    [--path fused|plain]

One step = one Kyber-768 encapsulation batch of B instances followed by the decapsulation of its
ciphertexts (B = 65536 per GPU), keys resident in HBM (generated once before timing), fresh
encapsulation coins for every step.  `value` is enc+dec pairs per second over all ranks with the
inputs already in HBM, timed with CUDA events on the library's stream; `e2e` is the same metric
through the host-buffer C ABI (pinned host memory; H2D of pk, coins, ct, sk and D2H of ct and both
shared secrets inside the timed region).  The fused path is the headline; the plain per-stage path
(one kernel per stage, thread per instance, intermediates in HBM) is timed beside it.

Multi-GPU (torchrun): every rank runs an independent replica on its own GPU (KEM instances are
independent; no collective on the data path), `value` = pairs of all ranks / max rank time.
--impl reference: times the reference's own code on the host cores of rank 0 -- its Kyber device
code (round-2 arithmetic; it has no KEM layer) compiled for the host by oracle/build_ref.sh, one
process per core, Kyber-768 CPA encryption + decryption pairs -- and prints the reference line;
where that build is missing, the CPU restatement of the KEM workload (oracle/) instead.

The default line also carries three secondary measurements, each with its own clock record:
serving at 50 % of the measured peak (p50 / p99), the mixed Kyber batch (k = 2/3/4, n ~
U{1..65536}), and Kyber-768 single-instance latency.  --no-extras leaves them out.

--config prints one line per configuration instead:
* kyber512, kyber1024, newhope1024, frodo976, newhope512, frodo640, frodo1344: keypair / enc / dec
  rates;
* mixed: concurrent mixed Kyber batches, stage kernels, graph replay;
* serving: continuous batching at 10-90 % of the measured peak;
* refgpu: the reference's own Kyber kernels recompiled for sm_103a, beside ours;
* latency: single-instance latencies;
* frodo_shared: FrodoKEM encapsulations to one public key, CUDA-core vs tensor-core product;
* all: every one of them.
"""
import argparse
import json
import os

# many concurrent streams (mixed batches, serving slots): 32 hardware work queues instead of 8,
# set before any CUDA context exists
os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

ALG = "kyber768"
METRIC = "Kyber-768 encaps+decaps/sec (batched, bit-exact)"
UNIT = "enc+dec pairs/s"
# Keccak-f[1600] cost in this implementation's 32-bit formulation, per permutation: 24 rounds x
# (theta parity 20 LOP3 + rot(C, 1) 10 SHF + theta apply 50 LOP3 + rho 48 SHF + chi 50 LOP3 + iota 2)
OPS_PER_PERM = 24 * 180
# One Kyber butterfly in 32-bit arithmetic: Montgomery multiply (3 IMAD + sign-extend + shift) + add + sub
OPS_PER_BUTTERFLY = 7
# Serial sponges of a Kyber-768 KEM (SHA3 rate 136, SHA3-512 rate 72): permutations per instance
# H(coins) 1, H(pk) 9, G 1 (encaps prologue); H(c) 9, KDF 1 (encaps epilogue / decaps)
ENC_HASH_PERMS = 1 + 9 + 1 + 9 + 1
DEC_HASH_PRE_PERMS = 9


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=60)
    p.add_argument("--warmup", type=int, default=5)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--batch", type=int, default=65536)
    p.add_argument("--path", default="fused", choices=["fused", "plain"])
    p.add_argument("--no-plain", action="store_true", help="skip timing the plain path beside the fused one")
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--no-extras", action="store_true", help="skip the serving / mixed / latency keys of the default line")
    p.add_argument("--slots", type=int, default=12, help="serving: batches in flight (worker threads)")
    p.add_argument("--config", default=None,
                   choices=["kyber512", "kyber1024", "newhope1024", "frodo976", "newhope512", "frodo640", "frodo1344", "mixed", "serving",
                            "refgpu", "latency", "frodo_shared", "all"],
                   help="measure another configuration (extra JSON lines) instead of the headline")
    return p.parse_args()


def max_over_ranks(x, world, device=None):
    """The maximum of x over all ranks (x itself on one rank): the slowest replica bounds the job."""
    if world <= 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(units_per_rank, world, max_ms):
    """Units of all ranks per second over the slowest rank's time (weak scaling: fixed work per GPU)."""
    return world * units_per_rank / (max_ms * 1e-3)


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class ClockSampler:
    """nvidia-smi sampling of SM clocks / throttle reasons during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
            # nvidia-smi takes a moment to print its first line: wait for it (at most 3 s), so that
            # a short region still has the sample taken as it starts, then one every 200 ms
            t0 = time.time()
            while not self.lines and time.time() - t0 < 3 and self.proc.poll() is None:
                time.sleep(0.01)
            self.first = max(0, len(self.lines) - 1)
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in self.lines[getattr(self, "first", 0):]:
            f = [x.strip() for x in l.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "samples": len(sm), "reasons": sorted(reasons)}


def cpu_baseline_port(nsample=16384, nthreads=0):
    """The CPU restatement (oracle/, C with OpenMP) of the Kyber-768 KEM on a bounded sample."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle as O
    from pqc_gb300 import drbg
    a = O.KYBER768
    s = O.alg_sizes(a)
    seed = drbg.seed48(12345)
    pk, sk = O.batch_keypair(a, nsample, drbg.stream(seed, b"kp", nsample * s["kp_coins"]), nthreads)
    ec = drbg.stream(seed, b"enc", nsample * s["enc_coins"])
    t0 = time.perf_counter()
    ct, ss = O.batch_enc(a, nsample, pk, ec, nthreads)
    ss2 = O.batch_dec(a, nsample, ct, sk, nthreads)
    el = time.perf_counter() - t0
    assert ss == ss2
    cores = nthreads if nthreads > 0 else os.cpu_count()
    return {"value": nsample / el, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": "%d Kyber-768 KEM enc+dec pairs (round 3) by the CPU restatement, keys pre-generated, "
                      "OpenMP over instances" % nsample, "seconds": el}


REF_SAMPLE = ("Kyber-768 CPA encryption + decryption pairs by the reference's own code (Kyber_GPU_Batched "
              "indcpa_enc / indcpa_dec, round-2 arithmetic; the reference has no KEM layer), host-compiled "
              "from its sources (oracle/build_ref.sh), one process per core, %d pairs per round")


def reference_cpu(reps=4, chunk=256):
    """The reference's own host-compiled Kyber code on all host cores (oracle/refcpu.py), or None
    where its build is missing."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import refcpu
    if not refcpu.available(3):
        return None
    r = refcpu.RefKyberCPU(3, chunk=chunk)
    try:
        r.run(1)  # warm-up: the processes allocate their state
        pairs, el, ok = r.run(reps)
    finally:
        r.close()
    return {"value": pairs / el, "unit": UNIT, "cores": r.procs, "kind": "reference",
            "sample": REF_SAMPLE % (r.procs * chunk), "pairs": pairs, "seconds": el, "roundtrip_ok": ok,
            "cpu": refcpu.cpu_model()}


def cpu_baseline():
    """The reference's own code where it built (kind "reference"), with the port beside it."""
    port = cpu_baseline_port()
    ref = reference_cpu()
    if ref is None:
        return port
    ref["port"] = port
    return ref


def work_per_pair():
    """Keccak permutations and NTT butterflies per Kyber-768 enc and dec, counted by the oracle's
    instrumented permutation / butterfly functions on 64 instances (single thread)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle as O
    from pqc_gb300 import drbg
    a = O.KYBER768
    s = O.alg_sizes(a)
    n = 64
    seed = drbg.seed48(4242)
    pk, sk = O.batch_keypair(a, n, drbg.stream(seed, b"kp", n * s["kp_coins"]), 1)
    O.counters_reset()
    ct, _ = O.batch_enc(a, n, pk, drbg.stream(seed, b"enc", n * s["enc_coins"]), 1)
    ep, eb = O.counters()
    O.counters_reset()
    O.batch_dec(a, n, ct, sk, 1)
    dp, db = O.counters()
    return {"enc_perms": ep / n, "enc_bfly": eb / n, "dec_perms": dp / n, "dec_bfly": db / n}


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import refcpu
    if refcpu.available(3):
        chunk = 256
        r = refcpu.RefKyberCPU(3, chunk=chunk)
        times, pairs, ok = [], 0, True
        try:
            for step in range(args.warmup + args.steps):
                n, el, good = r.run(1)
                ok = ok and good
                if step >= args.warmup:
                    times.append(el)
                    pairs += n
        finally:
            r.close()
        kind, cores, sample = "reference", r.procs, REF_SAMPLE % (r.procs * chunk)
        extra = {"roundtrip_ok": ok, "cpu": refcpu.cpu_model(), "port_kem": cpu_baseline_port()}
    else:
        import pyoracle as O
        from pqc_gb300 import drbg
        a = O.KYBER768
        s = O.alg_sizes(a)
        sample_n = 16384
        seed = drbg.seed48(777)
        pk, sk = O.batch_keypair(a, sample_n, drbg.stream(seed, b"kp", sample_n * s["kp_coins"]))
        times, pairs = [], 0
        for step in range(args.warmup + args.steps):
            ec = drbg.stream(seed, b"enc%d" % step, sample_n * s["enc_coins"])
            t0 = time.perf_counter()
            ct, ss = O.batch_enc(a, sample_n, pk, ec)
            ss2 = O.batch_dec(a, sample_n, ct, sk)
            el = time.perf_counter() - t0
            assert ss == ss2
            if step >= args.warmup:
                times.append(el)
                pairs += sample_n
        kind, cores = "port", os.cpu_count()
        sample = ("%d Kyber-768 KEM pairs per step by the CPU restatement (oracle/, C + OpenMP): the reference's "
                  "host build is missing" % sample_n)
        extra = {}
    tot = sum(times)
    v = pairs / tot
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * tot / len(times),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int16",
        "data": "synthetic (SHAKE-256 DRBG seeded coins)",
        "config": {"workload": "kyber768 enc+dec, a bounded sample per step on the host cores",
                   "alg": ALG, "batch": args.batch, "parallelism": "host processes"},
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": cores, "kind": kind, "sample": sample},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    line.update(extra)
    print(json.dumps(line), flush=True)


def clocked(fn, device=0):
    """Run fn() with the nvidia-smi clock sampler around it; returns (result, clocks)."""
    c = ClockSampler(device)
    c.start()
    try:
        r = fn()
    finally:
        clk = c.stop()
    return r, clk


def make_timer(ctx, st):
    import torch

    def timed(fn, reps):
        fn()
        ctx.wait()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        for _ in range(reps):
            fn()
        e1.record(st)
        e1.synchronize()
        return e0.elapsed_time(e1) / reps
    return timed


def measure_mixed(ctx, dev, up, timed, reps=3):
    """The mixed Kyber batch (pqc_gb300.workload.mixed_kyber_spec: 24 launches, k = 2/3/4 at
    40/40/20, n ~ U{1..65536}, ops 1/3 each) through the mixed-batch call, its graph replay, one
    kernel per stage, and the single-job calls one after another."""
    import torch
    from pqc_gb300 import drbg, kem
    from pqc_gb300.workload import mixed_kyber_spec
    jobs, total, keep = [], 0, []
    for j, (alg, op, n) in enumerate(mixed_kyber_spec()):
        s = kem.sizes(alg)
        seed = drbg.seed48(200 + j)
        kc = up(drbg.stream(seed, b"kp", n * s["kp_coins"]))
        pk, sk = (torch.empty(n * s[x], dtype=torch.uint8, device=dev) for x in ("pk", "sk"))
        ctx.keypair_dev(alg, n, pk, sk, kc)
        if op == "keypair":
            jobs.append((alg, op, n, kc, None, torch.empty_like(pk), torch.empty_like(sk)))
        else:
            ec = up(drbg.stream(seed, b"enc", n * s["enc_coins"]))
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
    t_mixed = timed(lambda: ctx.mixed_dev(jobs), reps)
    ok = all(torch.equal(jobs[i][5], ss) for i, ss in keep)
    t_stage = timed(lambda: ctx.mixed_dev(jobs, kem.STAGE_KERNELS), reps)
    ok = ok and all(torch.equal(jobs[i][5], ss) for i, ss in keep)
    g = ctx.graph(jobs)
    t_graph = timed(g.launch, reps)
    ok = ok and all(torch.equal(jobs[i][5], ss) for i, ss in keep)
    g.close()

    def sequential():
        for alg, op, n, in0, in1, out0, out1 in jobs:
            if op == "keypair":
                ctx.keypair_dev(alg, n, out0, out1, in0)
            elif op == "enc":
                ctx.enc_dev(alg, n, out0, out1, in0, in1)
            else:
                ctx.dec_dev(alg, n, out0, in0, in1)

    t_seq = timed(sequential, reps)
    return {"metric": "mixed Kyber batch ops/s", "jobs": len(jobs), "instances": total,
            "mixed_batch_per_s": total / t_mixed * 1e3, "graph_replay_per_s": total / t_graph * 1e3,
            "sequential_per_s": total / t_seq * 1e3, "stage_kernels_per_s": total / t_stage * 1e3,
            "what": "mixed_batch (default): every job's own kernels over 8 streams; stage_kernels: one kernel per "
                    "Kyber core stage for all jobs; sequential: the single-job calls one after another",
            "mix": "k=2/3/4 at 40/40/20, n ~ U{1..65536}, ops 1/3 each", "bit_exact_decaps": bool(ok)}


def measure_frodo_shared(ctx, dev, up, timed, n=2048, algs=("frodo640", "frodo976", "frodo1344")):
    """n FrodoKEM encapsulations to one public key: A generated once and one matrix product for the
    batch, on the CUDA cores (mad.lo) or the tensor cores (tcgen05 kind::f16 on the split A), beside
    the per-instance path (A regenerated by every encapsulation); outputs compared byte for byte.
    The product kernels' own times come from the library's launch profiler."""
    import ctypes

    import torch
    from pqc_gb300 import _lib, drbg, kem
    lib = _lib.load()
    out = {}
    for alg in algs:
        s = kem.sizes(alg)
        seed = drbg.seed48(17)
        pk1 = torch.empty(s["pk"], dtype=torch.uint8, device=dev)
        sk1 = torch.empty(s["sk"], dtype=torch.uint8, device=dev)
        ctx.keypair_dev(alg, 1, pk1, sk1, up(drbg.stream(seed, b"kp", s["kp_coins"])))
        mu = up(drbg.stream(seed, b"enc", n * s["enc_coins"]))
        pkn = pk1.repeat(n)
        ct, ss = (torch.empty(n * s[x], dtype=torch.uint8, device=dev) for x in ("ct", "ss"))
        res = {}
        t_inst = timed(lambda: ctx.enc_dev(alg, n, ct, ss, pkn, mu), 3)
        ref = (ct.clone(), ss.clone())
        res["per_instance_per_s"] = n / t_inst * 1e3
        for name, product in (("cuda_cores", 1), ("tensor_cores", 2)):
            with kem.shared_product(alg, product):
                t = timed(lambda: ctx.frodo_enc_shared_dev(alg, n, ct, ss, pk1, mu), 3)
                same = torch.equal(ct, ref[0]) and torch.equal(ss, ref[1])
                lib.pqcgpu_profile_enable(1)
                ctx.frodo_enc_shared_dev(alg, n, ct, ss, pk1, mu)
                ctx.wait()
                lib.pqcgpu_profile_enable(0)
                buf = ctypes.create_string_buffer(1 << 16)
                _lib.check(lib.pqcgpu_profile_read(buf, len(buf)))
                prof = json.loads(buf.value.decode())
            kern = {k: round(v[1], 4) for k, v in prof.items()}
            res[name] = {"per_s": n / t * 1e3, "ms": t, "bit_exact_vs_per_instance": bool(same), "kernels_ms": kern}
        out[alg] = res
    return {"metric": "FrodoKEM encapsulations to one public key, per second (device-resident)", "batch": n,
            "algs": out}


def measure_serving(slots, fractions=(0.1, 0.3, 0.5, 0.7, 0.9), seconds=1.5):
    """Continuous batching under Poisson load at fractions of the measured peak (native load
    generator, pqcgpu_server_run_poisson); the peak is the rate achieved at saturation."""
    from pqc_gb300 import serve
    with serve.Server(0, budget=16 << 30, max_inflight=slots, max_batch=4096) as srv:
        sat = srv.run_poisson(serve.SERVING_MIX, rate=2e6, seconds=1.0, seed=1)
        peak = sat["achieved_per_s"]
        # Saturation forms only large batches; a short low-load pass (discarded) makes the first
        # launches of the small-batch kernels (and their lazy module loads) before any timed point.
        srv.run_poisson(serve.SERVING_MIX, rate=0.05 * peak, seconds=0.5, seed=7)
        points = []
        for frac in fractions:
            r = srv.run_poisson(serve.SERVING_MIX, rate=frac * peak, seconds=seconds, seed=int(frac * 100))
            groups = {"%s/%s" % (alg, op): srv.group_stats(alg, op) for alg, op, _ in serve.SERVING_MIX}
            points.append({"load": frac, "offered_per_s": r["offered_per_s"], "achieved_per_s": r["achieved_per_s"],
                           "p50_ms": r["p50_ms"], "p99_ms": r["p99_ms"], "max_ms": r["max_ms"],
                           "batches": r["batches"],
                           "p99_ms_by_group": {g: round(v["p99_ms"], 3) for g, v in groups.items()},
                           "p50_ms_by_group": {g: round(v["p50_ms"], 3) for g, v in groups.items()}})
    return {"metric": "KEM serving latency under Poisson load", "slots": slots,
            "mix": "60% Kyber-512/768/1024, 20% NewHope-1024, 20% FrodoKEM-976, ops equiprobable",
            "keys": "resident on the device", "hbm_budget_gb": 16, "measured_peak_per_s": peak, "points": points}


def run_configs(args):
    """Secondary configurations, one JSON line each (not the headline metric), each with the clock
    record of its own measurement."""
    import torch
    from pqc_gb300 import drbg, kem
    dev = torch.device("cuda", 0)
    ctx = kem.Context(0)
    st = torch.cuda.ExternalStream(ctx.stream, device=dev)
    up = lambda b: torch.frombuffer(bytearray(b), dtype=torch.uint8).to(dev)
    which = (["kyber512", "kyber1024", "newhope1024", "frodo976", "newhope512", "frodo640", "frodo1344", "mixed", "serving", "refgpu",
              "latency", "frodo_shared"] if args.config == "all" else [args.config])
    timed = make_timer(ctx, st)

    for cfg in which:
        if cfg in ("kyber512", "kyber1024", "newhope1024", "frodo976", "newhope512", "frodo640", "frodo1344"):
            alg = cfg
            n = {"kyber512": 65536, "kyber1024": 65536, "newhope1024": 16384, "frodo976": 2048, "newhope512": 16384, "frodo640": 2048,
                 "frodo1344": 2048}[cfg]
            s = kem.sizes(alg)
            seed = drbg.seed48(5)
            kc, ec = up(drbg.stream(seed, b"kp", n * s["kp_coins"])), up(drbg.stream(seed, b"enc", n * s["enc_coins"]))
            pk, sk, ct = (torch.empty(n * s[x], dtype=torch.uint8, device=dev) for x in ("pk", "sk", "ct"))
            ss, ss2 = (torch.empty(n * s["ss"], dtype=torch.uint8, device=dev) for _ in range(2))
            torch.cuda.synchronize()
            reps = 3 if alg.startswith("frodo") else 10

            def rates():
                tk = timed(lambda: ctx.keypair_dev(alg, n, pk, sk, kc), reps)
                te = timed(lambda: ctx.enc_dev(alg, n, ct, ss, pk, ec), reps)
                td = timed(lambda: ctx.dec_dev(alg, n, ss2, ct, sk), reps)
                return tk, te, td

            (tk, te, td), clk = clocked(rates)
            ctx.wait()
            print(json.dumps({"config": cfg, "batch": n, "metric": "%s ops/s per operation (device-resident)" % alg,
                              "keypair_per_s": n / tk * 1e3, "enc_per_s": n / te * 1e3, "dec_per_s": n / td * 1e3,
                              "keypair_enc_dec_chains_per_s": n / (tk + te + td) * 1e3,
                              "bit_exact_roundtrip": bool(torch.equal(ss, ss2)), "clocks": clk}), flush=True)
        elif cfg == "mixed":
            r, clk = clocked(lambda: measure_mixed(ctx, dev, up, timed))
            r.update({"config": "mixed", "clocks": clk})
            print(json.dumps(r), flush=True)
        elif cfg == "frodo_shared":
            r, clk = clocked(lambda: measure_frodo_shared(ctx, dev, up, timed))
            r.update({"config": "frodo_shared", "clocks": clk})
            print(json.dumps(r), flush=True)
        elif cfg == "refgpu":
            run_refgpu(ctx, dev, up, timed)
        elif cfg == "latency":
            r, clk = clocked(lambda: measure_latency(ctx, dev, up))
            r.update({"config": "latency", "clocks": clk})
            print(json.dumps(r), flush=True)
        elif cfg == "serving":
            r, clk = clocked(lambda: measure_serving(args.slots))
            r.update({"config": "serving", "clocks": clk})
            print(json.dumps(r), flush=True)
    ctx.close()


LATENCY_ALGS = ("kyber512", "kyber768", "kyber1024", "mlkem768", "newhope1024", "newhope512", "frodo640", "frodo976",
                "frodo1344")


def measure_latency(ctx, dev, up, algs=LATENCY_ALGS, reps=50):
    """Single-instance latency (n = 1) of every operation, device-resident buffers, CUDA events
    around each call on the library stream: p50 and p99 over `reps` calls."""
    import torch
    from pqc_gb300 import drbg, kem
    st = torch.cuda.ExternalStream(ctx.stream, device=dev)
    out = {}
    for alg in algs:
        s = kem.sizes(alg)
        seed = drbg.seed48(77)
        kc, ec = up(drbg.stream(seed, b"kp", s["kp_coins"])), up(drbg.stream(seed, b"enc", s["enc_coins"]))
        pk, sk, ct = (torch.empty(s[x], dtype=torch.uint8, device=dev) for x in ("pk", "sk", "ct"))
        ss, ss2 = (torch.empty(s["ss"], dtype=torch.uint8, device=dev) for _ in range(2))
        ops = {"keypair": lambda: ctx.keypair_dev(alg, 1, pk, sk, kc), "enc": lambda: ctx.enc_dev(alg, 1, ct, ss, pk, ec),
               "dec": lambda: ctx.dec_dev(alg, 1, ss2, ct, sk)}
        res = {}
        for op, f in ops.items():
            f()
            ctx.wait()
            ts = []
            for _ in range(reps):
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(st)
                f()
                e1.record(st)
                e1.synchronize()
                ts.append(e0.elapsed_time(e1))
            ts.sort()
            res[op] = {"p50_ms": ts[len(ts) // 2], "p99_ms": ts[min(len(ts) - 1, int(0.99 * len(ts)))]}
        ctx.wait()
        res["roundtrip_ok"] = bool(torch.equal(ss, ss2))
        out[alg] = res
    return {"metric": "single-instance latency (n = 1), device-resident", "reps": reps, "algs": out}


def run_refgpu(ctx, dev, up, timed):
    """The reference's own batched Kyber kernels (round-2 CPA, k = 4 and 3) recompiled for sm_103a
    (baseline/_ref) beside this library's fused kernels on the same GPU, same inputs, same batch
    (the reference's maximum, N_TESTS = 16384); outputs compared byte for byte."""
    import ctypes

    import torch
    from pqc_gb300 import drbg, kem
    sys.path.insert(0, os.path.join(ROOT, "baseline"))
    import refgpu
    for k in (4, 3):
        if not refgpu.available(k):
            print(json.dumps({"config": "refgpu", "k": k, "unavailable": "reference kernels not built "
                              "(baseline/build_ref_gpu.sh had no staged sources)"}), flush=True)
            continue
        ref = refgpu.RefGPU(k)
        n = ref.max_count
        cs = kem.kyber_cpa_sizes(2, k)
        seed = drbg.seed48(31 + k)
        d, m, coins = (up(drbg.stream(seed, lab, 32 * n)) for lab in (b"d", b"m", b"coins"))
        rng = up(drbg.stream(seed, b"rng", 64 * n))
        buf = lambda sz: torch.zeros(n * sz, dtype=torch.uint8, device=dev)  # noqa: E731
        pk_r, sk_r, ct_r, m_r, pk_t, sk_t = (buf(cs[x]) if x in cs else buf(32)
                                             for x in ("pk", "sk", "ct", "m", "pk", "sk"))
        pk_o, sk_o, ct_o, m_o = (buf(cs[x]) if x in cs else buf(32) for x in ("pk", "sk", "ct", "m"))
        sh = ctypes.c_void_p(ctx.stream)
        L, F = ctx.lib, kem.DEVICE_PTRS
        P = lambda t: ctypes.c_void_p(t.data_ptr())  # noqa: E731

        def ok(rc):
            if rc != 0:
                raise RuntimeError("pqcgpu call returned %d" % rc)

        ours = {
            "keypair": lambda: ok(L.pqcgpu_kyber_indcpa_keypair_batch(ctx.h, 2, k, n, P(pk_o), P(sk_o), P(d), F)),
            "enc": lambda: ok(L.pqcgpu_kyber_indcpa_enc_batch(ctx.h, 2, k, n, P(ct_o), P(m), P(pk_o), P(coins), F)),
            "dec": lambda: ok(L.pqcgpu_kyber_indcpa_dec_batch(ctx.h, 2, k, n, P(m_o), P(ct_o), P(sk_o), F)),
        }
        theirs = {
            # indcpa_keypair as the reference runs it (its in-place G makes these keys timing-only)
            "keypair": lambda: ref.keypair(n, pk_t, sk_t, rng, sh),
            "enc": lambda: ref.enc(n, ct_r, m, pk_r, coins, sh),
            "dec": lambda: ref.dec(n, m_r, ct_r, sk_r, sh),
        }
        torch.cuda.synchronize()
        ref.keypair_nist(n, pk_r, sk_r, d, sh)
        for op in ("keypair", "enc", "dec"):
            if op != "keypair":  # the reference's keys for parity come from keypair_nist above
                theirs[op]()
            ours[op]()
        ctx.wait()
        same = {"pk": torch.equal(pk_r, pk_o), "sk": torch.equal(sk_r, sk_o), "ct": torch.equal(ct_r, ct_o),
                "m_dec_ref": torch.equal(m_r, m), "m_dec_ours": torch.equal(m_o, m)}
        tr = {op: timed(f, 10) for op, f in theirs.items()}
        to = {op: timed(f, 10) for op, f in ours.items()}
        ref.close()
        chains = lambda t: n / (t["keypair"] + t["enc"] + t["dec"]) * 1e3  # noqa: E731
        print(json.dumps({
            "config": "refgpu", "metric": "Kyber round-2 CPA (k=%d) keypair+enc+dec chains/s, device-resident" % k,
            "k": k, "batch": n,
            "reference_kernels_sm103a": {"ms": tr, "chains_per_s": chains(tr),
                                         "what": "Kyber_GPU_Batched indcpa_* recompiled by nvcc for sm_103a, V100 "
                                                 "block sizes, thread per instance, intermediates in HBM"},
            "ours_fused": {"ms": to, "chains_per_s": chains(to)},
            "speedup": {op: tr[op] / to[op] for op in tr},
            "speedup_chain": chains(to) / chains(tr),
            "bit_exact": same}), flush=True)


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    if args.config:
        return run_configs(args)
    import torch
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=dev)
    from pqc_gb300 import _lib, drbg, kem
    lib = _lib.load()
    B, K, W = args.batch, args.steps, args.warmup
    s = kem.sizes(ALG)
    ctx = kem.Context(local)
    st = torch.cuda.ExternalStream(ctx.stream, device=dev)

    def barrier():
        torch.cuda.synchronize(dev)
        if world > 1:
            torch.distributed.barrier()

    seed = drbg.seed48(1000 + rank)
    up = lambda b: torch.frombuffer(bytearray(b), dtype=torch.uint8).to(dev)
    pk = torch.empty(B * s["pk"], dtype=torch.uint8, device=dev)
    sk = torch.empty(B * s["sk"], dtype=torch.uint8, device=dev)
    ct = torch.empty(B * s["ct"], dtype=torch.uint8, device=dev)
    ss = torch.empty(B * s["ss"], dtype=torch.uint8, device=dev)
    ss2 = torch.empty_like(ss)
    kc = up(drbg.stream(seed, b"kp", B * s["kp_coins"]))
    coins = [up(drbg.stream(seed, b"enc%d" % i, B * s["enc_coins"])) for i in range(W + K)]
    torch.cuda.synchronize(dev)
    ctx.keypair_dev(ALG, B, pk, sk, kc)
    ctx.wait()
    flags = kem.PLAIN if args.path == "plain" else 0

    def step(i, fl=flags):
        ctx.enc_dev(ALG, B, ct, ss, pk, coins[i], fl)
        ctx.dec_dev(ALG, B, ss2, ct, sk, fl)

    for i in range(W):
        step(i)
    ctx.wait()
    barrier()
    ok = torch.equal(ss, ss2)

    # ---- timed region (device-resident inputs) ----
    clocks = ClockSampler(local)
    clocks.start()
    lib.pqcgpu_profile_enable(1)
    launches0 = ctx.launches
    barrier()
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(K)]
    for i in range(K):
        evs[i][0].record(st)
        step(W + i)
        evs[i][1].record(st)
    ctx.wait()
    barrier()
    launches = ctx.launches - launches0
    lib.pqcgpu_profile_enable(0)
    buf = __import__("ctypes").create_string_buffer(1 << 16)
    _lib.check(lib.pqcgpu_profile_read(buf, len(buf)))
    prof = json.loads(buf.value.decode())
    clk = clocks.stop()
    ok = ok and torch.equal(ss, ss2)
    # the last timed step's outputs against the oracle on a sample spread over the batch
    oracle_ok = oracle_sample_check(ALG, B, pk, coins[W + K - 1], ct, ss)
    ok = ok and oracle_ok
    step_ms = [a.elapsed_time(b) for a, b in evs]
    total_ms = evs[0][0].elapsed_time(evs[-1][1])
    total_ms = max_over_ranks(total_ms, world, dev)
    value = whole_job_rate(B * K, world, total_ms)

    # ---- plain path beside it (same inputs, same outputs) ----
    plain = None
    if not args.no_plain and args.path == "fused":
        try:
            step(0, kem.PLAIN)
            ctx.wait()
            ref_ss = ss.clone()
            step(0, 0)
            ctx.wait()
            same = torch.equal(ref_ss, ss)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(st)
            for i in range(min(K, 3)):
                step(W + i, kem.PLAIN)
            e1.record(st)
            ctx.wait()
            pms = e0.elapsed_time(e1) / min(K, 3)
            plain = {"value": B / (pms * 1e-3), "unit": UNIT, "ms_per_step": pms, "bit_exact_vs_fused": same}
        except RuntimeError as e:
            plain = {"unavailable": str(e)}

    # ---- end to end through the host-buffer C ABI ----
    e2e = None
    if not args.no_e2e:
        h = {k: torch.empty(B * s[k], dtype=torch.uint8).pin_memory() for k in ("pk", "sk", "ct")}
        h["ss"] = torch.empty(B * s["ss"], dtype=torch.uint8).pin_memory()
        h["ss2"] = torch.empty(B * s["ss"], dtype=torch.uint8).pin_memory()
        h["pk"].copy_(pk.cpu())
        h["sk"].copy_(sk.cpu())
        hcoins = [c.cpu().pin_memory() for c in coins]

        def hstep(i):
            ctx.enc_host_ptrs(ALG, B, h["ct"], h["ss"], h["pk"], hcoins[i])
            ctx.dec_host_ptrs(ALG, B, h["ss2"], h["ct"], h["sk"])

        for i in range(min(W, 2)):
            hstep(i)
        barrier()
        t0 = time.perf_counter()
        for i in range(K):
            hstep(W + i)
        el = time.perf_counter() - t0
        el = max_over_ranks(el, world, dev)
        ok = ok and torch.equal(h["ss"], h["ss2"])
        e2e = {"value": whole_job_rate(B * K, world, 1e3 * el), "unit": UNIT,
               "h2d_bytes_per_step": B * (s["pk"] + s["enc_coins"] + s["ct"] + s["sk"]),
               "d2h_bytes_per_step": B * (s["ct"] + 2 * s["ss"]), "ms_per_step": 1e3 * el / K}

    if rank != 0:
        if world > 1:
            torch.distributed.destroy_process_group()
        return

    # ---- roofline of the dominant kernel (integer pipe) ----
    w = work_per_pair()
    io = ctypes_peaks(lib, local)
    dom = max(prof.items(), key=lambda kv: kv[1][1]) if prof else None
    roof = None
    if dom:
        name, (nl, tms) = dom
        per_launch_ms = tms / nl
        dec_stage1_bfly = 4 * 896  # decryption stage: NTT of u' (k = 3) and the inverse NTT of s^T u
        if "enc_core" in name:
            perms, bfly = w["enc_perms"] - ENC_HASH_PERMS, w["enc_bfly"]
        elif "dec_core" in name:
            perms, bfly = w["dec_perms"] - DEC_HASH_PRE_PERMS, w["dec_bfly"]
        elif "dec_reencrypt" in name:  # re-encryption stage: all but G, the decryption NTTs and the
            # KDF when kyber_dec_hash_post runs it (batches above 1024)
            kdf_out = 1 if any("dec_hash_post" in k for k in prof) else 0
            perms, bfly = w["dec_perms"] - DEC_HASH_PRE_PERMS - 1 - kdf_out, w["dec_bfly"] - dec_stage1_bfly
        elif "dec_decrypt" in name:
            perms, bfly = 1, dec_stage1_bfly
        else:
            perms, bfly = ENC_HASH_PERMS, 0
        ops = B * (perms * OPS_PER_PERM + bfly * OPS_PER_BUTTERFLY)
        achieved = ops / (per_launch_ms * 1e-3) / 1e12
        peak = io["int_ops_per_s"] / 1e12
        traffic = None
        tfile = os.path.join(ROOT, "profiles", "traffic.json")
        if os.path.exists(tfile):
            tj = json.load(open(tfile))
            if name in tj:
                traffic = tj[name]["dram_bytes_per_instance"] * B
        roof = {"bound": "alu", "kernel": name, "achieved": achieved, "peak": peak, "unit": "Tops/s (int32)",
                "frac": achieved / peak, "traffic": traffic,
                "peak_source": "measured in this run: LOP3 throughput probe (pqcgpu_probe_peaks)",
                "algorithmic_ops_per_launch": ops, "launch_ms": per_launch_ms,
                "keccak_perms_per_s": B * perms / (per_launch_ms * 1e-3),
                "keccak_perm_peak_per_s": io["keccak_perms_per_s"]}
    io_bytes = B * (s["pk"] + s["enc_coins"] + s["ct"] + s["ss"] + s["ct"] + s["sk"] + s["ss"])
    hbm_peak = measured_hbm_peak()
    io_gbs = io_bytes / (total_ms / K * 1e-3) / 1e9
    hbm_io = {"gbs": io_gbs, "bytes_per_step": io_bytes, "peak_gbs": hbm_peak,
              "frac": (io_gbs / hbm_peak) if hbm_peak else None,
              "what": "batch I/O of one step (enc: pk, coins in, ct, ss out; dec: ct, sk in, ss out) over the step "
                      "time; peak = MEASURED_PEAKS.json hbm_gbs (of measured)"}
    if roof:
        roof["hbm_gbs_io"] = hbm_io
    base = cpu_baseline()
    extras = {}
    if not args.no_extras:
        timed = make_timer(ctx, st)
        r, clk = clocked(lambda: measure_serving(args.slots, fractions=(0.5,)), local)
        p50 = r["points"][0]
        extras["serving"] = {"load": 0.5, "measured_peak_per_s": r["measured_peak_per_s"],
                             "achieved_per_s": p50["achieved_per_s"], "p50_ms": p50["p50_ms"], "p99_ms": p50["p99_ms"],
                             "max_ms": p50["max_ms"], "slots": args.slots, "mix": r["mix"], "clocks": clk}
        r, clk = clocked(lambda: measure_mixed(ctx, dev, up, timed), local)
        extras["mixed"] = {k: r[k] for k in ("instances", "jobs", "mixed_batch_per_s", "graph_replay_per_s",
                                             "stage_kernels_per_s", "sequential_per_s", "bit_exact_decaps", "mix")}
        extras["mixed"]["clocks"] = clk
        r, clk = clocked(lambda: measure_latency(ctx, dev, up, algs=(ALG,)), local)
        extras["latency_n1"] = dict(r["algs"][ALG], clocks=clk, alg=ALG)
    lat = sorted(step_ms)
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": K, "warmup": W,
        "ms_per_step": total_ms / K, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "int16", "data": "synthetic (keys and coins from a seeded SHAKE-256 DRBG)",
        "config": {"workload": "kyber768 encaps+decaps, batch %d per GPU, keys resident in HBM" % B,
                   "alg": ALG, "batch": B, "path": args.path, "parallelism": "replicas x%d" % world,
                   "l2": "inputs larger than L2 (%.0f MB of pk/sk/ct/coins per step)" %
                         (B * (s["pk"] + s["sk"] + s["ct"] + s["enc_coins"]) / 1e6)},
        "bit_exact_check": bool(ok),
        "bit_exact_vs_oracle_sample": bool(oracle_ok),
        "latency_ms": {"p50": lat[len(lat) // 2], "p99": lat[min(len(lat) - 1, int(0.99 * len(lat)))],
                       "what": "one enc+dec batch of %d" % B},
        "plain": plain,
        "fused_over_plain": (value / world / plain["value"]) if plain and "value" in plain else None,
        "e2e": e2e,
        "gpu_launches": launches,
        "kernels": {k: {"launches": v[0], "total_ms": v[1]} for k, v in prof.items()},
        "roofline": roof,
        "cpu_baseline": base,
        "clocks": clk,
    }
    line.update(extras)
    print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def oracle_sample_check(alg, n, pk, coins, ct, ss, count=256):
    """The ciphertexts and shared secrets of one batched encapsulation (device tensors) against the
    CPU oracle at `count` instance indices spread over the batch (instances are independent)."""
    import random
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle as O
    from pqc_gb300 import kem
    s = kem.sizes(alg)
    rng = random.Random(n)
    idx = sorted({0, n - 1} | {rng.randrange(i * n // count, (i + 1) * n // count) for i in range(count)})
    hb = lambda t: bytes(t.cpu().numpy())  # noqa: E731
    pkh, ch, cth, ssh = hb(pk), hb(coins), hb(ct), hb(ss)
    rows = lambda b, sz: b"".join(b[i * sz:(i + 1) * sz] for i in idx)  # noqa: E731
    oct_, oss = O.batch_enc(O.ALG_NAMES[alg], len(idx), rows(pkh, s["pk"]), rows(ch, s["enc_coins"]))
    return oct_ == rows(cth, s["ct"]) and oss == rows(ssh, s["ss"])


def measured_hbm_peak():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            return float(json.load(f)["hbm_gbs"])
    except (OSError, KeyError, ValueError):
        return None


def ctypes_peaks(lib, device):
    import ctypes
    a, b = ctypes.c_double(), ctypes.c_double()
    rc = lib.pqcgpu_probe_peaks(device, ctypes.byref(a), ctypes.byref(b))
    if rc != 0:
        raise RuntimeError("peak probe failed")
    return {"int_ops_per_s": a.value, "keccak_perms_per_s": b.value}


if __name__ == "__main__":
    main()
