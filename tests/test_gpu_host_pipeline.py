"""The host-buffer path splits a batch into chunks (small first and last chunks, large ones in
between). Copies in and out run on their own streams and each chunk's kernels on a compute stream
of falling priority; up to 16 device buffer slots are used and then reused. These tests run
batches that need several chunks, reuse the slots (many chunks, or a budget that holds one or two
slots), and check that the bytes equal those of the device-pointer path on the same inputs."""
import pytest

from pqc_gb300 import drbg

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    from pqc_gb300 import kem
    c = kem.Context(0)
    yield c
    c.close()


# chunks of the host path with the default shape: Kyber-768 x 20000 -> 4096 3616 8192 4096;
# Kyber-512 x 40000 -> 4096 8192 15424 8192 4096; FrodoKEM-976 x 2200 (at most 2048 per chunk by
# slot size) -> 1100 1100.  Shape (1024, 256, 512, 5): Kyber-768 x 20000 -> 256 512 + 19 middle
# chunks + 512, so slots are reused, over 5 compute streams.
CASES = [("kyber768", 20000, None), ("kyber512", 40000, None), ("frodo976", 2200, None),
         ("kyber768", 20000, (1024, 256, 512, 5))]


@pytest.mark.parametrize("alg,n,shape", CASES)
def test_chunked_host_path_matches_device_path(ctx, alg, n, shape):
    import torch
    from pqc_gb300 import kem
    s = kem.sizes(alg)
    seed = drbg.seed48(4242 + n)
    kc = drbg.stream(seed, b"kp", n * s["kp_coins"])
    ec = drbg.stream(seed, b"enc", n * s["enc_coins"])
    default = kem.get_host_pipeline()
    if shape:
        kem.set_host_pipeline(*shape)
    try:
        pk, sk = ctx.keypair(alg, n, kc)
        ct, ss = ctx.enc(alg, n, pk, ec)
        ss2 = ctx.dec(alg, n, ct, sk)
    finally:
        kem.set_host_pipeline(*default)
    assert ss2 == ss

    dev = torch.device("cuda:0")
    t = lambda b: torch.frombuffer(bytearray(b), dtype=torch.uint8).to(dev)  # noqa: E731
    dpk, dsk, dct = (torch.empty(n * s[x], dtype=torch.uint8, device=dev) for x in ("pk", "sk", "ct"))
    dss, dss2 = (torch.empty(n * s["ss"], dtype=torch.uint8, device=dev) for _ in range(2))
    dkc, dec_ = t(kc), t(ec)
    torch.cuda.synchronize()
    ctx.keypair_dev(alg, n, dpk, dsk, dkc)
    ctx.enc_dev(alg, n, dct, dss, dpk, dec_)
    ctx.dec_dev(alg, n, dss2, dct, dsk)
    ctx.wait()
    assert bytes(dpk.cpu().numpy()) == pk
    assert bytes(dsk.cpu().numpy()) == sk
    assert bytes(dct.cpu().numpy()) == ct
    assert bytes(dss.cpu().numpy()) == ss
    assert bytes(dss2.cpu().numpy()) == ss


@pytest.mark.parametrize("budget", [8 << 20, 40 << 20])
def test_host_path_with_a_small_budget(ctx, budget):
    """A context whose budget holds only one or a few slots reuses them, with smaller chunks when
    even one full-size slot does not fit; the bytes do not change."""
    from pqc_gb300 import kem
    alg, n = "kyber768", 12000
    s = kem.sizes(alg)
    seed = drbg.seed48(77)
    kc = drbg.stream(seed, b"kp", n * s["kp_coins"])
    ec = drbg.stream(seed, b"enc", n * s["enc_coins"])
    pk, sk = ctx.keypair(alg, n, kc)
    ct, ss = ctx.enc(alg, n, pk, ec)
    small = kem.Context(0, budget=budget)
    try:
        assert small.keypair(alg, n, kc) == (pk, sk)
        assert small.enc(alg, n, pk, ec) == (ct, ss)
        assert small.dec(alg, n, ct, sk) == ss
    finally:
        small.close()


def test_profile_trace_of_a_host_buffer_call(ctx):
    """The Chrome-trace timeline of a chunked host-buffer call holds its copies in and out and its
    kernels, on several streams, with well-formed times; reading it clears the records."""
    from pqc_gb300 import kem
    alg, n = "kyber768", 20000
    s = kem.sizes(alg)
    seed = drbg.seed48(31)
    pk, _ = ctx.keypair(alg, n, drbg.stream(seed, b"kp", n * s["kp_coins"]))
    kem.profile_trace()  # drop anything recorded before
    kem.profile_enable(True)
    try:
        ctx.enc(alg, n, pk, drbg.stream(seed, b"enc", n * s["enc_coins"]))
    finally:
        kem.profile_enable(False)
    ev = kem.profile_trace()["traceEvents"]
    names = {e["name"] for e in ev}
    assert {"copy H2D", "copy D2H", "kyber_enc_core<3,3>"} <= names
    assert len({e["tid"] for e in ev}) >= 3  # copies in, copies out, compute streams
    assert all(e["ph"] == "X" and e["ts"] >= 0 and e["dur"] >= 0 for e in ev)
    assert min(e["ts"] for e in ev) == 0
    # every chunk's kernels start after its copy in began
    first_h2d = min(e["ts"] for e in ev if e["name"] == "copy H2D")
    assert all(e["ts"] >= first_h2d for e in ev if e["name"].startswith("kyber_"))
    assert kem.profile_trace() == {"traceEvents": []}
