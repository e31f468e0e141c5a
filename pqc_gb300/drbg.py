"""Deterministic randomness for batches: a SHAKE-256 stream keyed by a 48-byte seed.

seed48(s) = SHAKE256(b"pqcgpu-seed" || le64(s))[0:48]; the bytes for a purpose `label` are
SHAKE256(seed48 || label) read from the start.  Every coins buffer passed to the batched API in
the tests and the benchmark comes from here, so the GPU path and the oracle see the same inputs.
"""
import hashlib


def seed48(s: int) -> bytes:
    return hashlib.shake_256(b"pqcgpu-seed" + int(s).to_bytes(8, "little")).digest(48)


def stream(seed: bytes, label: bytes, n: int) -> bytes:
    if len(seed) != 48:
        raise ValueError("seed must be 48 bytes")
    return hashlib.shake_256(seed + label).digest(n)
