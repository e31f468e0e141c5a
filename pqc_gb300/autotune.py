"""Autotuner for the core-kernel launch shapes (instances per CTA, threads per CTA).

Replaces the reference's ANALYSIS_MODE block-size sweep (Kyber_GPU_Batched/indcpa.cu:21-70), which
re-ran every launch over ten block sizes and printed the best: here each (algorithm, operation) is
timed with CUDA events over a candidate grid at a given batch size (FrodoKEM: the split of an
instance's rows of A over CTAs, at serving-size batches), the fastest shape is applied
through pqcgpu_set_launch_shape, and the choice is persisted in a JSON cache keyed by GPU name and
library version so later processes load it instead of re-tuning.  A candidate counts only if its
outputs equal the outputs at the shape in force when tuning started (byte for byte); a candidate
that is refused, fails or differs is skipped, and an operation keeps its shape when none is left.

    python -m pqc_gb300.autotune [--batch 65536] [--out tuning.json]
"""
import argparse
import ctypes
import json
import os

from . import _lib, drbg, kem

DEFAULT_CACHE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "_build", "tuning.json")
TUNABLE = ("kyber512", "kyber768", "kyber1024", "newhope1024", "newhope512", "frodo976")


def candidates(alg, op):
    if alg.startswith("kyber") and op == 3:  # decapsulation, decryption stage (warp-level phases)
        return [(ni, thr) for ni in (4, 6, 8, 12, 16, 24, 32) for thr in (64, 128, 192, 256, 384)]
    if alg.startswith("kyber"):
        k = {"kyber512": 2, "kyber768": 3, "kyber1024": 4}[alg]
        out = []
        for ni in (4, 6, 8, 10, 11, 12, 13, 14, 15, 16, 18, 20, 24, 28, 30, 32, 36, 40, 48):
            jobs = ni * k * k
            for thr in (64, 96, 128, 160, 192, 224, 256, 288, 320, 384):
                lo = min(((jobs + 31) // 32) * 32, 384) - 64
                if lo <= thr <= ((jobs + 31) // 32) * 32 + 32:
                    out.append((ni, thr))
        return out
    if alg == "frodo976":
        # keypair: threads of the row CTAs; encaps / decaps: CTAs per instance (row split) x threads
        if op == 0:
            return [(0, thr) for thr in (64, 128, 256)]
        return [(parts, thr) for parts in (1, 2, 4, 8, 16) for thr in (128, 256)]
    if alg == "newhope512":  # half the shared memory per instance of NewHope-1024
        return [(ni, thr) for ni in (2, 4, 8, 12, 16, 24, 32) for thr in (32, 64, 128, 256)]
    return [(ni, thr) for ni in (1, 2, 4, 8) for thr in (64, 128, 256) if thr // 32 >= 1]


def get_shape(lib, alg, op):
    a, b = ctypes.c_int(), ctypes.c_int()
    if lib.pqcgpu_get_launch_shape(kem.alg_id(alg), op, ctypes.byref(a), ctypes.byref(b)) != 0:
        return None
    return a.value, b.value


def tune(batch=65536, algs=TUNABLE, reps=3, device=0, log=print):
    import torch
    lib = _lib.load()
    ctx = kem.Context(device)
    dev = torch.device("cuda", device)
    st = torch.cuda.ExternalStream(ctx.stream, device=dev)
    result = {}
    for alg in algs:
        s = kem.sizes(alg)
        n = {"newhope1024": min(batch, 16384), "newhope512": min(batch, 16384),
             "frodo976": min(batch, 256)}.get(alg, batch)
        seed = drbg.seed48(99)
        up = lambda b: torch.frombuffer(bytearray(b), dtype=torch.uint8).to(dev)
        kc = up(drbg.stream(seed, b"kp", n * s["kp_coins"]))
        ec = up(drbg.stream(seed, b"enc", n * s["enc_coins"]))
        pk, sk = (torch.empty(n * s[x], dtype=torch.uint8, device=dev) for x in ("pk", "sk"))
        ct = torch.empty(n * s["ct"], dtype=torch.uint8, device=dev)
        ss, ss2 = (torch.empty(n * s["ss"], dtype=torch.uint8, device=dev) for _ in range(2))
        torch.cuda.synchronize(dev)
        ctx.keypair_dev(alg, n, pk, sk, kc)
        ctx.enc_dev(alg, n, ct, ss, pk, ec)
        ctx.wait()
        # a tampered copy of every third ciphertext, so that the decapsulation check also runs
        # the implicit-rejection path at each candidate shape
        ct_bad = ct.clone()
        ct_bad[::3 * s["ct"]] ^= 1
        fns = {0: lambda: ctx.keypair_dev(alg, n, pk, sk, kc), 1: lambda: ctx.enc_dev(alg, n, ct, ss, pk, ec),
               2: lambda: ctx.dec_dev(alg, n, ss2, ct_bad, sk), 3: lambda: ctx.dec_dev(alg, n, ss2, ct_bad, sk)}
        outs = {0: (pk, sk), 1: (ct, ss), 2: (ss2,), 3: (ss2,)}
        for op in ((0, 1, 3, 2) if alg.startswith("kyber") else (0, 1, 2)):
            start = get_shape(lib, alg, op)
            fns[op]()
            ctx.wait()
            want = [t.clone() for t in outs[op]]
            best = None
            for ni, thr in candidates(alg, op):
                if lib.pqcgpu_set_launch_shape(kem.alg_id(alg), op, ni, thr) != 0:
                    continue
                try:
                    for t in outs[op]:
                        t.zero_()
                    fns[op]()
                    ctx.wait()
                    if not all(torch.equal(t, w) for t, w in zip(outs[op], want)):
                        log("%s op %d: ni=%d threads=%d gives different outputs; skipped" % (alg, op, ni, thr))
                        continue
                    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                    e0.record(st)
                    for _ in range(reps):
                        fns[op]()
                    e1.record(st)
                    e1.synchronize()
                    ms = e0.elapsed_time(e1) / reps
                except RuntimeError:
                    continue
                if best is None or ms < best[0]:
                    best = (ms, ni, thr)
            if best is None:
                if start is not None:
                    lib.pqcgpu_set_launch_shape(kem.alg_id(alg), op, start[0], start[1])
                log("%s op %d: no candidate ran; shape kept at %s" % (alg, op, start))
                continue
            lib.pqcgpu_set_launch_shape(kem.alg_id(alg), op, best[1], best[2])
            result["%s/%d" % (alg, op)] = {"ni": best[1], "threads": best[2], "ms": best[0], "batch": n}
            log("%s op %d: ni=%d threads=%d  %.3f ms" % (alg, op, best[1], best[2], best[0]))
    ctx.close()
    return {"gpu": torch.cuda.get_device_name(dev), "library": library_version(), "shapes": result}


def library_version():
    return _lib.load().pqcgpu_version().decode()


def save(tuning, path=DEFAULT_CACHE):
    os.makedirs(os.path.dirname(path), exist_ok=True)
    with open(path, "w") as f:
        json.dump(tuning, f, indent=1)


def apply(tuning, log=print):
    """Apply a tuning dict (or a path to its JSON) to the loaded library.  An entry the library
    refuses (e.g. a shape outside the current kernels' launch bounds) is skipped with a message."""
    if isinstance(tuning, str):
        with open(tuning) as f:
            tuning = json.load(f)
    lib = _lib.load()
    for key, v in tuning["shapes"].items():
        alg, op = key.split("/")
        if lib.pqcgpu_set_launch_shape(kem.alg_id(alg), int(op), v["ni"], v["threads"]) != 0:
            log("tuning entry %s (%d, %d) refused by this library; default kept" % (key, v["ni"], v["threads"]))
    return tuning


def load_cached(path=DEFAULT_CACHE, gpu_name=None):
    """Apply the cached tuning if it exists and was made on this GPU model with this library
    version; returns it or None."""
    if not os.path.exists(path):
        return None
    with open(path) as f:
        t = json.load(f)
    if gpu_name is not None and t.get("gpu") != gpu_name:
        return None
    if t.get("library") != library_version():
        return None
    return apply(t)


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--batch", type=int, default=65536)
    ap.add_argument("--out", default=DEFAULT_CACHE)
    ap.add_argument("--algs", default=",".join(TUNABLE), help="comma list of algorithms to tune")
    a = ap.parse_args()
    t = tune(a.batch, algs=[x for x in a.algs.split(",") if x])
    save(t, a.out)
    print("saved", a.out)
