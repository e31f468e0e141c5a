// C ABI of libpqcgpu: contexts, the device arena, host-buffer staging, the DRBG and the NIST
// single-instance entry points.  Declarations and conventions: include/pqcgpu.h.
#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>

#include <atomic>
#include <mutex>
#include <string>
#include <vector>

#include <sys/random.h>

#include "pqcgpu_internal.h"

namespace pqc {
std::atomic<uint64_t> g_launch_count{0};
}

using namespace pqc;

static thread_local std::string g_last_error;
static int set_err(int code, const char *what) {
    g_last_error = what;
    return code;
}
static int cuda_err(cudaError_t e, const char *where) {
    if (e == cudaSuccess) return PQCGPU_OK;
    g_last_error = std::string(where) + ": " + cudaGetErrorString(e);
    return PQCGPU_ECUDA;
}

// ---------------------------------------------------------------------------------------------
// Host SHAKE-256 (for the DRBG only; all batch hashing runs on the GPU)
// ---------------------------------------------------------------------------------------------
namespace {
struct HostShake {
    uint64_t s[25];
    unsigned pos;  // squeeze position within the current block
    static uint64_t rol(uint64_t v, int n) { return n ? (v << n) | (v >> (64 - n)) : v; }
    // round constants (FIPS 202 rc(t) LFSR) and rotation offsets, built once; a function-local
    // static is initialised thread-safely, so concurrent first calls from several threads are fine
    struct Tables {
        uint64_t RC[24];
        int R[25];
    };
    static const Tables &tables() {
        static const Tables t = [] {
            Tables tb{};
            for (int ir = 0; ir < 24; ir++) {
                uint64_t v = 0;
                for (int j = 0; j <= 6; j++) {
                    const int tt = j + 7 * ir;
                    int bit = 1;
                    if (tt % 255) {
                        int Rr[9] = {1, 0, 0, 0, 0, 0, 0, 0, 0};
                        for (int i = 1; i <= tt % 255; i++) {
                            int Rn[9];
                            Rn[0] = 0;
                            for (int b = 0; b < 8; b++) Rn[b + 1] = Rr[b];
                            Rn[0] ^= Rn[8];
                            Rn[4] ^= Rn[8];
                            Rn[5] ^= Rn[8];
                            Rn[6] ^= Rn[8];
                            for (int b = 0; b < 9; b++) Rr[b] = Rn[b];
                        }
                        bit = Rr[0];
                    }
                    if (bit) v |= 1ULL << ((1u << j) - 1);
                }
                tb.RC[ir] = v;
            }
            tb.R[0] = 0;
            int x = 1, y = 0;
            for (int t2 = 0; t2 < 24; t2++) {
                tb.R[x + 5 * y] = ((t2 + 1) * (t2 + 2) / 2) % 64;
                const int nx = y, ny = (2 * x + 3 * y) % 5;
                x = nx;
                y = ny;
            }
            return tb;
        }();
        return t;
    }
    static void permute(uint64_t A[25]) {
        const uint64_t *RC = tables().RC;
        const int *R = tables().R;
        for (int ir = 0; ir < 24; ir++) {
            uint64_t C[5], D[5], B[25];
            for (int i = 0; i < 5; i++) C[i] = A[i] ^ A[i + 5] ^ A[i + 10] ^ A[i + 15] ^ A[i + 20];
            for (int i = 0; i < 5; i++) D[i] = C[(i + 4) % 5] ^ rol(C[(i + 1) % 5], 1);
            for (int i = 0; i < 25; i++) A[i] ^= D[i % 5];
            for (int xx = 0; xx < 5; xx++)
                for (int yy = 0; yy < 5; yy++) B[yy + 5 * ((2 * xx + 3 * yy) % 5)] = rol(A[xx + 5 * yy], R[xx + 5 * yy]);
            for (int yy = 0; yy < 5; yy++)
                for (int xx = 0; xx < 5; xx++)
                    A[xx + 5 * yy] = B[xx + 5 * yy] ^ (~B[(xx + 1) % 5 + 5 * yy] & B[(xx + 2) % 5 + 5 * yy]);
            A[0] ^= RC[ir];
        }
    }
    void init(const uint8_t *in, size_t len) {
        memset(s, 0, sizeof s);
        uint8_t blk[136];
        while (len >= 136) {
            for (int i = 0; i < 17; i++) {
                uint64_t w = 0;
                for (int b = 0; b < 8; b++) w |= (uint64_t)in[8 * i + b] << (8 * b);
                s[i] ^= w;
            }
            permute(s);
            in += 136;
            len -= 136;
        }
        memset(blk, 0, sizeof blk);
        memcpy(blk, in, len);
        blk[len] ^= 0x1F;
        blk[135] ^= 0x80;
        for (int i = 0; i < 17; i++) {
            uint64_t w = 0;
            for (int b = 0; b < 8; b++) w |= (uint64_t)blk[8 * i + b] << (8 * b);
            s[i] ^= w;
        }
        pos = 136;
    }
    void squeeze(uint8_t *out, size_t n) {
        while (n) {
            if (pos == 136) {
                permute(s);
                pos = 0;
            }
            const size_t take = (n < 136 - pos) ? n : 136 - pos;
            for (size_t i = 0; i < take; i++) out[i] = (uint8_t)(s[(pos + i) / 8] >> (8 * ((pos + i) % 8)));
            pos += (unsigned)take;
            out += take;
            n -= take;
        }
    }
};

std::mutex g_drbg_mu;
HostShake g_drbg;
bool g_drbg_seeded = false;
bool g_drbg_nist = false;  // pqcgpu_randombytes_init_nist: AES-256 CTR_DRBG (kat.cu) instead of SHAKE256
pqc::CtrDrbg g_ctr;

// 48 bytes of operating-system entropy (getrandom, else /dev/urandom); false if neither works.
bool os_entropy(uint8_t seed[48]) {
    size_t got = 0;
    while (got < 48) {
        const ssize_t r = getrandom(seed + got, 48 - got, 0);
        if (r <= 0) break;
        got += (size_t)r;
    }
    if (got == 48) return true;
    FILE *f = fopen("/dev/urandom", "rb");
    if (!f) return false;
    got = fread(seed, 1, 48, f);
    fclose(f);
    return got == 48;
}

// Fills out from the library DRBG (the caller holds g_drbg_mu).  The SHAKE-256 DRBG seeds itself
// from the operating system on first use; without an entropy source it refuses (returns false)
// rather than produce predictable keys.
bool drbg_bytes_locked(uint8_t *out, size_t n) {
    if (g_drbg_nist) {
        g_ctr.generate(out, n);
        return true;
    }
    if (!g_drbg_seeded) {
        uint8_t seed[48];
        if (!os_entropy(seed)) return false;
        g_drbg.init(seed, sizeof seed);
        g_drbg_seeded = true;
    }
    g_drbg.squeeze(out, n);
    return true;
}
bool drbg_bytes(uint8_t *out, size_t n) {
    std::lock_guard<std::mutex> lk(g_drbg_mu);
    return drbg_bytes_locked(out, n);
}

struct AlgInfo {
    size_t pk, sk, ct, ss, kpc, encc;
};
bool alg_info(int alg, AlgInfo *a) {
    switch (alg) {
    case PQCGPU_KYBER512: *a = {800, 1632, 768, 32, 64, 32}; return true;
    case PQCGPU_KYBER768: *a = {1184, 2400, 1088, 32, 64, 32}; return true;
    case PQCGPU_KYBER1024: *a = {1568, 3168, 1568, 32, 64, 32}; return true;
    case PQCGPU_KYBER1024_R2: *a = {1568, 3168, 1568, 32, 64, 32}; return true;
    case PQCGPU_MLKEM512: *a = {800, 1632, 768, 32, 64, 32}; return true;
    case PQCGPU_MLKEM768: *a = {1184, 2400, 1088, 32, 64, 32}; return true;
    case PQCGPU_MLKEM1024: *a = {1568, 3168, 1568, 32, 64, 32}; return true;
    case PQCGPU_NEWHOPE1024: *a = {1824, 1792, 2176, 32, 32, 32}; return true;
    case PQCGPU_NEWHOPE512: *a = {928, 896, 1088, 32, 32, 32}; return true;
    case PQCGPU_FRODO976: *a = {15632, 31296, 15744, 24, 64, 24}; return true;
    case PQCGPU_FRODO640: *a = {9616, 19888, 9720, 16, 48, 16}; return true;
    case PQCGPU_FRODO1344: *a = {21520, 43088, 21632, 32, 80, 32}; return true;
    default: return false;
    }
}
bool kyber_alg(int alg, int *variant, int *k) {
    switch (alg) {
    case PQCGPU_KYBER512: *variant = 3; *k = 2; return true;
    case PQCGPU_KYBER768: *variant = 3; *k = 3; return true;
    case PQCGPU_KYBER1024: *variant = 3; *k = 4; return true;
    case PQCGPU_KYBER1024_R2: *variant = 2; *k = 4; return true;
    case PQCGPU_MLKEM512: *variant = 3; *k = 2; return true;
    case PQCGPU_MLKEM768: *variant = 3; *k = 3; return true;
    case PQCGPU_MLKEM1024: *variant = 3; *k = 4; return true;
    default: return false;
    }
}
}  // namespace
namespace pqc {
// KEM layer of a Kyber-family algorithm: 1 = Fujisaki-Okamoto as in rounds 2 / 3, 2 = FIPS 203
int kyber_kem_mode(int alg) { return (alg >= PQCGPU_MLKEM512 && alg <= PQCGPU_MLKEM1024) ? 2 : 1; }
int frodo_n(int alg) {
    return alg == PQCGPU_FRODO976 ? 976 : alg == PQCGPU_FRODO640 ? 640 : alg == PQCGPU_FRODO1344 ? 1344 : 0;
}
}  // namespace pqc

// ---------------------------------------------------------------------------------------------
// Context
// ---------------------------------------------------------------------------------------------
struct pqcgpu_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    static constexpr int NPAR = 8;  // concurrent streams for mixed batches
    cudaStream_t par[NPAR] = {};
    // Host-buffer calls: ordered copies in and out on their own streams; chunk i uses buffer slot
    // i % (slots of the call).  Its kernels run on one of the pipeline streams, whose priorities
    // fall from pipe[0] to pipe[NPAR - 1]; chunks map to them in order, so earlier chunks take the
    // SMs first and later ones fill the gaps.
    static constexpr int NSLOT = 16;
    cudaStream_t copy_in = nullptr, copy_out = nullptr;
    cudaStream_t pipe[NPAR] = {};
    cudaEvent_t in_ev[NSLOT] = {}, done_ev[NSLOT] = {}, free_ev[NSLOT] = {};
    cudaEvent_t fork_ev = nullptr, join_ev[NPAR] = {};
    cudaEvent_t stage_ev[NPAR] = {}, stage_ev2[NPAR] = {}, core_ev = nullptr;  // mixed Kyber waves and their hashes
    cudaEvent_t fr_ev[NPAR] = {}, fr_core_ev = nullptr;                        // the FrodoKEM wave and its sponges
    bool own_stream = true;
    size_t budget = 0;
    uint8_t *arena = nullptr;
    size_t arena_size = 0;
    uint64_t launches_at_create = 0;
    // a device word set by kernels whose bounded waits ran out (FrodoKEM's tensor-core product);
    // allocated on first use, read and cleared by the call (host buffers) or by pqcgpu_ctx_wait
    unsigned *dev_err = nullptr;
    bool dev_err_pending = false;
    std::recursive_mutex mu;

    // Read and clear the device error word (the stream must be synchronised).
    int take_dev_err() {
        dev_err_pending = false;
        if (!dev_err) return PQCGPU_OK;
        unsigned e = 0;
        if (cudaMemcpy(&e, dev_err, sizeof e, cudaMemcpyDeviceToHost) != cudaSuccess) {
            cudaGetLastError();
            return set_err(PQCGPU_ECUDA, "reading the device error word failed");
        }
        if (!e) return PQCGPU_OK;
        cudaMemset(dev_err, 0, sizeof e);
        return set_err(PQCGPU_ECUDA, "tensor-core product: a wait ran out (outputs of that call are undefined)");
    }

    // Arena: one device allocation, grown on demand within the budget; sub-buffers are carved
    // per call (calls on a context are serialised, so a call owns the whole arena).
    int reserve(size_t bytes) {
        if (bytes <= arena_size) return PQCGPU_OK;
        if (bytes > budget) return set_err(PQCGPU_EBUDGET, "request exceeds the context's device-memory budget");
        if (arena) {
            cudaStreamSynchronize(stream);
            cudaStreamSynchronize(copy_in);
            cudaStreamSynchronize(copy_out);
            for (auto s : par) cudaStreamSynchronize(s);
            for (auto s : pipe) cudaStreamSynchronize(s);
            cudaFree(arena);
            arena = nullptr;
            arena_size = 0;
        }
        size_t want = bytes + bytes / 4;
        if (want > budget) want = budget;
        if (cudaMalloc(&arena, want) != cudaSuccess) {
            cudaGetLastError();
            return set_err(PQCGPU_ENOMEM, "cudaMalloc of the context arena failed");
        }
        arena_size = want;
        return PQCGPU_OK;
    }
};

static bool g_constants_ready[64];
static std::mutex g_init_mu;

static int ensure_device_init(int device) {
    std::lock_guard<std::mutex> lk(g_init_mu);
    if (device < 0 || device >= 64) return set_err(PQCGPU_EINVAL, "bad device");
    if (g_constants_ready[device]) return PQCGPU_OK;
    int rc = kyber_init_constants();
    if (rc) return set_err(rc, "uploading Kyber constants failed");
    rc = newhope_init_constants();
    if (rc) return set_err(rc, "uploading NewHope constants failed");
    rc = frodo_init_constants();
    if (rc) return set_err(rc, "uploading FrodoKEM constants failed");
    g_constants_ready[device] = true;
    return PQCGPU_OK;
}

namespace pqc {
// Per-device set-up shared with entry points that work without a context: uploads the constant
// tables once per device (the current device must be `device`).
int device_ready(int device) { return ensure_device_init(device); }
int set_error(int code, const char *what) { return set_err(code, what); }
}  // namespace pqc

extern "C" int pqcgpu_ctx_create(pqcgpu_ctx **out, int device, size_t budget) {
    if (!out) return set_err(PQCGPU_EINVAL, "out is NULL");
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return set_err(PQCGPU_ECUDA, "no CUDA device available");
    }
    if (device < 0 || device >= ndev) return set_err(PQCGPU_EINVAL, "device index out of range");
    int rc = cuda_err(cudaSetDevice(device), "cudaSetDevice");
    if (rc) return rc;
    rc = ensure_device_init(device);
    if (rc) return rc;
    pqcgpu_ctx *c = new pqcgpu_ctx();
    c->device = device;
    c->budget = budget ? budget : ((size_t)4 << 30);
    if ((rc = cuda_err(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking), "stream")) ||
        (rc = cuda_err(cudaStreamCreateWithFlags(&c->copy_in, cudaStreamNonBlocking), "stream")) ||
        (rc = cuda_err(cudaStreamCreateWithFlags(&c->copy_out, cudaStreamNonBlocking), "stream"))) {
        pqcgpu_ctx_destroy(c);
        return rc;
    }
    for (int i = 0; i < pqcgpu_ctx::NPAR; i++) {
        if ((rc = cuda_err(cudaStreamCreateWithFlags(&c->par[i], cudaStreamNonBlocking), "stream")) ||
            (rc = cuda_err(cudaEventCreateWithFlags(&c->join_ev[i], cudaEventDisableTiming), "event")) ||
            (rc = cuda_err(cudaEventCreateWithFlags(&c->stage_ev[i], cudaEventDisableTiming), "event")) ||
            (rc = cuda_err(cudaEventCreateWithFlags(&c->stage_ev2[i], cudaEventDisableTiming), "event")) ||
            (rc = cuda_err(cudaEventCreateWithFlags(&c->fr_ev[i], cudaEventDisableTiming), "event"))) {
            pqcgpu_ctx_destroy(c);
            return rc;
        }
    }
    int least = 0, greatest = 0;
    if ((rc = cuda_err(cudaDeviceGetStreamPriorityRange(&least, &greatest), "stream priorities"))) {
        pqcgpu_ctx_destroy(c);
        return rc;
    }
    for (int i = 0; i < pqcgpu_ctx::NPAR; i++) {
        const int prio = greatest + (int)(((long)(least - greatest) * i + (pqcgpu_ctx::NPAR - 1) / 2) / (pqcgpu_ctx::NPAR - 1));
        if ((rc = cuda_err(cudaStreamCreateWithPriority(&c->pipe[i], cudaStreamNonBlocking, prio), "stream"))) {
            pqcgpu_ctx_destroy(c);
            return rc;
        }
    }
    for (int i = 0; i < pqcgpu_ctx::NSLOT; i++) {
        if ((rc = cuda_err(cudaEventCreateWithFlags(&c->in_ev[i], cudaEventDisableTiming), "event")) ||
            (rc = cuda_err(cudaEventCreateWithFlags(&c->done_ev[i], cudaEventDisableTiming), "event")) ||
            (rc = cuda_err(cudaEventCreateWithFlags(&c->free_ev[i], cudaEventDisableTiming), "event"))) {
            pqcgpu_ctx_destroy(c);
            return rc;
        }
    }
    if ((rc = cuda_err(cudaEventCreateWithFlags(&c->fork_ev, cudaEventDisableTiming), "event")) ||
        (rc = cuda_err(cudaEventCreateWithFlags(&c->core_ev, cudaEventDisableTiming), "event")) ||
        (rc = cuda_err(cudaEventCreateWithFlags(&c->fr_core_ev, cudaEventDisableTiming), "event"))) {
        pqcgpu_ctx_destroy(c);
        return rc;
    }
    c->launches_at_create = g_launch_count.load();
    *out = c;
    return PQCGPU_OK;
}

extern "C" int pqcgpu_ctx_destroy(pqcgpu_ctx *c) {
    if (!c) return PQCGPU_EINVAL;
    cudaSetDevice(c->device);
    cudaDeviceSynchronize();
    if (c->arena) cudaFree(c->arena);
    if (c->dev_err) cudaFree(c->dev_err);
    if (c->own_stream && c->stream) cudaStreamDestroy(c->stream);
    if (c->copy_in) cudaStreamDestroy(c->copy_in);
    for (auto s : c->pipe)
        if (s) cudaStreamDestroy(s);
    if (c->copy_out) cudaStreamDestroy(c->copy_out);
    for (int i = 0; i < pqcgpu_ctx::NSLOT; i++) {
        if (c->in_ev[i]) cudaEventDestroy(c->in_ev[i]);
        if (c->done_ev[i]) cudaEventDestroy(c->done_ev[i]);
        if (c->free_ev[i]) cudaEventDestroy(c->free_ev[i]);
    }
    for (int i = 0; i < pqcgpu_ctx::NPAR; i++) {
        if (c->par[i]) cudaStreamDestroy(c->par[i]);
        if (c->join_ev[i]) cudaEventDestroy(c->join_ev[i]);
        if (c->stage_ev[i]) cudaEventDestroy(c->stage_ev[i]);
        if (c->stage_ev2[i]) cudaEventDestroy(c->stage_ev2[i]);
        if (c->fr_ev[i]) cudaEventDestroy(c->fr_ev[i]);
    }
    if (c->fork_ev) cudaEventDestroy(c->fork_ev);
    if (c->core_ev) cudaEventDestroy(c->core_ev);
    if (c->fr_core_ev) cudaEventDestroy(c->fr_core_ev);
    delete c;
    return PQCGPU_OK;
}

extern "C" int pqcgpu_ctx_set_stream(pqcgpu_ctx *c, void *s) {
    if (!c) return PQCGPU_EINVAL;
    std::lock_guard<std::recursive_mutex> lk(c->mu);
    if (c->own_stream && c->stream) cudaStreamDestroy(c->stream);
    c->stream = (cudaStream_t)s;
    c->own_stream = false;
    return PQCGPU_OK;
}
extern "C" void *pqcgpu_ctx_stream(pqcgpu_ctx *c) { return c ? (void *)c->stream : nullptr; }
extern "C" int pqcgpu_ctx_wait(pqcgpu_ctx *c) {
    if (!c) return PQCGPU_EINVAL;
    std::lock_guard<std::recursive_mutex> lk(c->mu);
    const int rc = cuda_err(cudaStreamSynchronize(c->stream), "cudaStreamSynchronize");
    if (rc) return rc;
    return c->dev_err_pending ? c->take_dev_err() : PQCGPU_OK;
}
extern "C" uint64_t pqcgpu_ctx_launches(pqcgpu_ctx *c) { return c ? g_launch_count.load() - c->launches_at_create : 0; }
extern "C" const char *pqcgpu_last_error(void) { return g_last_error.c_str(); }
extern "C" const char *pqcgpu_version(void) { return "pqcgpu 0.1 (sm_103a)"; }

extern "C" int pqcgpu_alg_sizes(pqcgpu_alg alg, size_t *pk, size_t *sk, size_t *ct, size_t *ss, size_t *kpc,
                                size_t *encc) {
    AlgInfo a;
    if (!alg_info(alg, &a)) return set_err(PQCGPU_EINVAL, "unknown algorithm");
    if (pk) *pk = a.pk;
    if (sk) *sk = a.sk;
    if (ct) *ct = a.ct;
    if (ss) *ss = a.ss;
    if (kpc) *kpc = a.kpc;
    if (encc) *encc = a.encc;
    return PQCGPU_OK;
}

extern "C" int pqcgpu_randombytes_init(const uint8_t seed[48]) {
    if (!seed) return PQCGPU_EINVAL;
    std::lock_guard<std::mutex> lk(g_drbg_mu);
    g_drbg.init(seed, 48);
    g_drbg_seeded = true;
    g_drbg_nist = false;
    return PQCGPU_OK;
}
extern "C" int pqcgpu_randombytes_init_nist(const uint8_t entropy[48], const uint8_t *personalization) {
    if (!entropy) return PQCGPU_EINVAL;
    std::lock_guard<std::mutex> lk(g_drbg_mu);
    g_ctr.instantiate(entropy, personalization);
    g_drbg_nist = true;
    return PQCGPU_OK;
}
extern "C" int pqcgpu_randombytes(uint8_t *out, size_t n) {
    if (!out && n) return PQCGPU_EINVAL;
    if (!drbg_bytes(out, n)) return set_err(PQCGPU_EUNSUPPORTED, "no operating-system entropy to seed the DRBG");
    return PQCGPU_OK;
}

// ---------------------------------------------------------------------------------------------
// Operation plumbing.  An op is described by its per-instance input / output sizes and a device
// function over a contiguous chunk.  The host-buffer path pipelines chunks: copies in run in
// order on one stream, copies out on another, and the kernels of consecutive chunks on different
// streams, so the copies of one chunk overlap the kernels of its neighbours.
// ---------------------------------------------------------------------------------------------
namespace {
constexpr int MAXIO = 3;
struct OpDesc {
    int nin = 0, nout = 0;
    const uint8_t *in[MAXIO];
    size_t in_sz[MAXIO];
    uint8_t *out[MAXIO];
    size_t out_sz[MAXIO];
    size_t scratch_per = 0;
};
// Shape of the host-buffer pipeline (process-wide, pqcgpu_set_host_pipeline): the largest chunk,
// the first and the last chunk, and the number of compute streams.  A chunk's device buffers are
// also capped at SLOT_BYTES_MAX, which caps FrodoKEM chunks at 2048 instances.
struct PipeShape {
    size_t chunk_max = 16384, chunk_first = 2048, chunk_last = 4096;
    int streams = 8;
};
PipeShape g_pipe;
std::mutex g_pipe_mu;
constexpr size_t SLOT_BYTES_MAX = (size_t)256 << 20;

// Chunk sizes for a host-buffer call of n instances.  The first chunk's copies in and the last
// chunk's copies out overlap no kernels, so chunks may start at `first` and double up to cmax, and
// shrink from cmax to `last` at the end; the middle is split evenly into chunks of at most cmax.
// 65536 instances with cmax = 16384, first = 2048, last = 4096 (the default): 2048, 4096, 8192,
// 12971, 12971, 12970, 8192, 4096; with cmax = 8192, first = 4096, last = 8192: 4096, 8 x 7680.
// The default was measured on GB300 (Kyber-768 encapsulation + decapsulation of 65536 instances
// through host buffers, median of three): first / last chunk 2048 / 4096 3.37 ms a step, 4096 /
// 4096 3.42 ms, 1024 / 4096 3.47 ms, 1024 / 8192 3.40 ms, 512 / 4096 3.64 ms; chunks of at most
// 24576 or 12288 instances 3.45 and 3.66 ms.
std::vector<size_t> chunk_plan(size_t n, size_t cmax, size_t first, size_t last) {
    std::vector<size_t> head, tail;
    size_t ramp = 0;
    for (size_t c = first; c < cmax; c *= 2) {
        head.push_back(c);
        ramp += c;
    }
    for (size_t c = last; c < cmax; c *= 2) {
        tail.push_back(c);
        ramp += c;
    }
    while (ramp > n) {  // drop the largest ramp chunks until the ramps fit
        std::vector<size_t> &v = (tail.empty() || (!head.empty() && head.back() >= tail.back())) ? head : tail;
        ramp -= v.back();
        v.pop_back();
    }
    std::vector<size_t> plan(head);
    const size_t mid = n - ramp;
    if (mid) {
        const size_t parts = (mid + cmax - 1) / cmax, each = (mid + parts - 1) / parts;
        for (size_t left = mid; left;) {
            const size_t m = left < each ? left : each;
            plan.push_back(m);
            left -= m;
        }
    }
    plan.insert(plan.end(), tail.rbegin(), tail.rend());
    return plan;
}

// One copy of the host-buffer pipeline, recorded by the launch profiler when it is on.
cudaError_t copy_async(void *dst, const void *src, size_t bytes, cudaMemcpyKind kind, cudaStream_t s) {
    const bool h2d = kind == cudaMemcpyHostToDevice;
    void *tok = prof_enabled() ? prof_begin(s, h2d ? "copy H2D" : "copy D2H", -1, 0) : nullptr;
    const cudaError_t e = cudaMemcpyAsync(dst, src, bytes, kind, s);
    if (tok) prof_end(s, tok);
    return e;
}

// run(n, din[], dout[], scratch, stream)
template <class Run>
int run_op(pqcgpu_ctx *c, size_t n, const OpDesc &d, unsigned flags, Run run) {
    if (n == 0) return PQCGPU_OK;
    if (n > (size_t)1 << 30) return set_err(PQCGPU_EINVAL, "batch too large");
    std::lock_guard<std::recursive_mutex> lk(c->mu);
    int rc = cuda_err(cudaSetDevice(c->device), "cudaSetDevice");
    if (rc) return rc;
    for (int i = 0; i < d.nin; i++)
        if (!d.in[i]) return set_err(PQCGPU_EINVAL, "null input buffer");
    for (int i = 0; i < d.nout; i++)
        if (!d.out[i]) return set_err(PQCGPU_EINVAL, "null output buffer");
    if (flags & PQCGPU_DEVICE_PTRS) {
        for (int i = 0; i < d.nin; i++)
            if ((uintptr_t)d.in[i] & 15) return set_err(PQCGPU_EINVAL, "device buffers must be 16-byte aligned");
        for (int i = 0; i < d.nout; i++)
            if ((uintptr_t)d.out[i] & 15) return set_err(PQCGPU_EINVAL, "device buffers must be 16-byte aligned");
        const size_t need = d.scratch_per * n + 256;
        if ((rc = c->reserve(need))) return rc;
        rc = run((int)n, d.in, d.out, c->arena, c->stream);
        if (rc) return rc;
        return cuda_err(cudaGetLastError(), "kernel launch");
    }
    // host buffers: the pipeline
    auto r256 = [](size_t v) { return (v + 255) & ~(size_t)255; };
    auto slot_bytes = [&](size_t m) {
        size_t b = r256(d.scratch_per * m);
        for (int i = 0; i < d.nin; i++) b += r256(d.in_sz[i] * m);
        for (int i = 0; i < d.nout; i++) b += r256(d.out_sz[i] * m);
        return b;
    };
    PipeShape shape;
    {
        std::lock_guard<std::mutex> lk(g_pipe_mu);
        shape = g_pipe;
    }
    size_t cmax = shape.chunk_max, first = shape.chunk_first, last = shape.chunk_last;
    while (cmax > 64 && slot_bytes(cmax) > SLOT_BYTES_MAX) cmax /= 2;
    // slots: one per chunk up to NSLOT (a slot is reused only by a later chunk), fewer if the
    // budget says so; chunks halve only when not even one slot fits
    std::vector<size_t> plan;
    size_t set_bytes = 0, mc = 0;
    int nslot = 1;
    for (;;) {
        if (first > cmax) first = cmax;
        if (last > cmax) last = cmax;
        plan = chunk_plan(n, cmax, first, last);
        mc = 0;
        for (size_t m : plan) mc = m > mc ? m : mc;
        set_bytes = slot_bytes(mc);
        size_t fit = c->budget / set_bytes;
        if (fit > plan.size()) fit = plan.size();
        if (fit > (size_t)pqcgpu_ctx::NSLOT) fit = pqcgpu_ctx::NSLOT;
        nslot = fit ? (int)fit : 1;
        if (fit || cmax <= 64) break;
        cmax /= 2;
    }
    // compute streams: nstream of the pipeline streams spread over the priority range; chunk ci
    // goes to bin ci * nstream / chunks, so the bins follow the chunk order
    const int nstream = (size_t)shape.streams < plan.size() ? shape.streams : (int)plan.size();
    cudaStream_t cst[pqcgpu_ctx::NPAR];
    for (int i = 0; i < nstream; i++) cst[i] = c->pipe[nstream > 1 ? i * (pqcgpu_ctx::NPAR - 1) / (nstream - 1) : 0];
    if ((rc = c->reserve(set_bytes * nslot))) return rc;
    cudaEvent_t ev;
    if ((rc = cuda_err(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming), "event"))) return rc;
    cudaEventRecord(ev, c->stream);  // order after prior work on the main stream
    cudaStreamWaitEvent(c->copy_in, ev, 0);
    cudaStreamWaitEvent(c->copy_out, ev, 0);
    for (int i = 0; i < nstream; i++) cudaStreamWaitEvent(cst[i], ev, 0);
    size_t off = 0;
    for (size_t ci = 0; ci < plan.size() && !rc; off += plan[ci], ci++) {
        const size_t m = plan[ci];
        const int sl = (int)(ci % (size_t)nslot);
        cudaStream_t cs = cst[ci * (size_t)nstream / plan.size()];
        // a slot's buffers sit at the same offsets for every chunk (sized for the largest), so a
        // chunk's copies in never touch the previous chunk's results still being copied out
        uint8_t *p = c->arena + (size_t)sl * set_bytes;
        const uint8_t *din[MAXIO];
        uint8_t *dout[MAXIO];
        // inputs: once the kernels of the slot's previous chunk have consumed theirs
        if (ci >= (size_t)nslot) cudaStreamWaitEvent(c->copy_in, c->done_ev[sl], 0);
        for (int i = 0; i < d.nin && !rc; i++) {
            uint8_t *q = p;
            p += r256(d.in_sz[i] * mc);
            rc = cuda_err(copy_async(q, d.in[i] + off * d.in_sz[i], m * d.in_sz[i], cudaMemcpyHostToDevice, c->copy_in),
                          "H2D");
            din[i] = q;
        }
        if (rc) break;
        cudaEventRecord(c->in_ev[sl], c->copy_in);
        for (int i = 0; i < d.nout; i++) {
            dout[i] = p;
            p += r256(d.out_sz[i] * mc);
        }
        // kernels: once the inputs are in and the slot's previous results are out
        cudaStreamWaitEvent(cs, c->in_ev[sl], 0);
        if (ci >= (size_t)nslot) cudaStreamWaitEvent(cs, c->free_ev[sl], 0);
        if ((rc = run((int)m, din, dout, p, cs))) break;
        cudaEventRecord(c->done_ev[sl], cs);
        cudaStreamWaitEvent(c->copy_out, c->done_ev[sl], 0);
        for (int i = 0; i < d.nout && !rc; i++)
            rc = cuda_err(copy_async(d.out[i] + off * d.out_sz[i], dout[i], m * d.out_sz[i], cudaMemcpyDeviceToHost,
                                     c->copy_out),
                          "D2H");
        cudaEventRecord(c->free_ev[sl], c->copy_out);
    }
    cudaError_t e = cudaStreamSynchronize(c->copy_out);
    cudaError_t e_in = cudaStreamSynchronize(c->copy_in);
    for (int i = 0; i < nstream; i++) {
        cudaError_t ei = cudaStreamSynchronize(cst[i]);
        if (e == cudaSuccess) e = ei;
    }
    if (e == cudaSuccess) e = e_in;
    cudaEventDestroy(ev);
    if (rc) return rc;
    if ((rc = cuda_err(e, "sync"))) return rc;
    return cuda_err(cudaGetLastError(), "kernel");
}

// coins == NULL: draw from the DRBG into a host buffer (or a temporary device copy)
struct CoinsHolder {
    uint8_t *host = nullptr;
    ~CoinsHolder() { free(host); }
};
}  // namespace

static int coins_or_drbg(pqcgpu_ctx *c, const uint8_t *&coins, size_t bytes, unsigned &flags, CoinsHolder &h,
                         const uint8_t **others, int nothers) {
    (void)c;
    (void)others;
    (void)nothers;
    if (coins) return PQCGPU_OK;
    if (flags & PQCGPU_DEVICE_PTRS)
        return set_err(PQCGPU_EINVAL, "coins == NULL needs host buffers (or pass device coins)");
    h.host = (uint8_t *)malloc(bytes ? bytes : 1);
    if (!h.host) return set_err(PQCGPU_ENOMEM, "malloc");
    if (!drbg_bytes(h.host, bytes))
        return set_err(PQCGPU_EUNSUPPORTED, "no operating-system entropy to seed the DRBG");
    coins = h.host;
    return PQCGPU_OK;
}

// ---------------------------------------------------------------------------------------------
// One device operation: op 0 keypair (in0 coins -> out0 pk, out1 sk), 1 encaps (in0 pk, in1 coins ->
// out0 ct, out1 ss), 2 decaps (in0 ct, in1 sk -> out0 ss).  All pointers on the device.
// ---------------------------------------------------------------------------------------------
namespace pqc {
size_t op_scratch_bytes(int alg, int op, int plain) {
    int variant, k;
    if (kyber_alg(alg, &variant, &k)) return kyber_scratch_bytes(k, op, plain);
    if (alg == PQCGPU_NEWHOPE1024 || alg == PQCGPU_NEWHOPE512) return op == 1 ? 64 : 0;
    if (frodo_n(alg)) return frodo_scratch_bytes(frodo_n(alg));
    return 0;
}
int op_dev(int alg, int op, int n, const uint8_t *in0, const uint8_t *in1, uint8_t *out0, uint8_t *out1,
           uint8_t *scr, int flags, cudaStream_t s) {
    AlgInfo ai;
    if (!alg_info(alg, &ai) || op < 0 || op > 2) return PQCGPU_EINVAL;
    const int plain = flags & OP_PLAIN;
    if (n <= 0) return PQCGPU_OK;
    int variant, k;
    if (kyber_alg(alg, &variant, &k)) {
        const int kem = kyber_kem_mode(alg);
        if (op == 0) return kyber_keypair_dev(variant, k, n, out0, out1, in0, (int)ai.kpc, kem, scr, plain, s);
        if (op == 1) return kyber_enc_dev(variant, k, n, out0, out1, in0, nullptr, in1, scr, kem, plain, s);
        return kyber_dec_dev(variant, k, n, out0, in0, in1, scr, kem, plain, s);
    }
    if (plain) return PQCGPU_EUNSUPPORTED;
    if (alg == PQCGPU_NEWHOPE1024 || alg == PQCGPU_NEWHOPE512) {
        const int N = alg == PQCGPU_NEWHOPE1024 ? 1024 : 512;
        const bool single_ok = !(flags & OP_NH_BATCHED);
        if (op == 0) return newhope_keypair_dev(N, n, out0, out1, in0, 32, s, single_ok);
        if (op == 1) return newhope_enc_dev(N, n, out0, out1, in0, nullptr, in1, scr, 1, s, single_ok);
        return newhope_dec_dev(N, n, out0, in0, in1, 1, s);
    }
    const int fn = frodo_n(alg);
    if (op == 0) return frodo_keypair_dev(fn, n, out0, out1, in0, (int)ai.kpc, scr, s);
    if (op == 1) return frodo_enc_dev(fn, n, out0, out1, in0, in1, scr, s);
    return frodo_dec_dev(fn, n, out0, in0, in1, scr, s);
}
// Per-instance byte sizes of the op's buffers (in0, in1, out0, out1; 0 = unused).
void op_io_sizes(int alg, int op, size_t sz[4]) {
    AlgInfo ai{};
    alg_info(alg, &ai);
    if (op == 0) { sz[0] = ai.kpc; sz[1] = 0; sz[2] = ai.pk; sz[3] = ai.sk; }
    else if (op == 1) { sz[0] = ai.pk; sz[1] = ai.encc; sz[2] = ai.ct; sz[3] = ai.ss; }
    else { sz[0] = ai.ct; sz[1] = ai.sk; sz[2] = ai.ss; sz[3] = 0; }
}
}  // namespace pqc

static int kem_op(pqcgpu_ctx *c, int alg, int op, size_t n, const uint8_t *in0, const uint8_t *in1, uint8_t *out0,
                  uint8_t *out1, unsigned flags) {
    AlgInfo ai;
    if (!c || !alg_info(alg, &ai)) return set_err(PQCGPU_EINVAL, "bad context or algorithm");
    const int plain = (flags & PQCGPU_PLAIN) ? 1 : 0;
    int variant, k;
    if (plain && (!kyber_alg(alg, &variant, &k) || kyber_kem_mode(alg) != 1))
        return set_err(PQCGPU_EUNSUPPORTED, "the plain path covers the round-2 / round-3 Kyber KEMs only");
    size_t sz[4];
    op_io_sizes(alg, op, sz);
    OpDesc d;
    const uint8_t *ins[2] = {in0, in1};
    uint8_t *outs[2] = {out0, out1};
    for (int i = 0; i < 2; i++)
        if (sz[i]) {
            d.in[d.nin] = ins[i];
            d.in_sz[d.nin++] = sz[i];
        }
    for (int i = 0; i < 2; i++)
        if (sz[2 + i]) {
            d.out[d.nout] = outs[i];
            d.out_sz[d.nout++] = sz[2 + i];
        }
    d.scratch_per = op_scratch_bytes(alg, op, plain);
    return run_op(c, n, d, flags, [&](int m, const uint8_t *const *in, uint8_t *const *out, uint8_t *scr, cudaStream_t s) {
        return op_dev(alg, op, m, in[0], d.nin > 1 ? in[1] : nullptr, out[0], d.nout > 1 ? out[1] : nullptr, scr, plain, s);
    });
}

extern "C" int pqcgpu_kem_keypair_batch(pqcgpu_ctx *c, pqcgpu_alg alg, size_t n, uint8_t *pk, uint8_t *sk,
                                        const uint8_t *coins, unsigned flags) {
    AlgInfo ai;
    if (!c || !alg_info(alg, &ai)) return set_err(PQCGPU_EINVAL, "bad context or algorithm");
    CoinsHolder h;
    int rc = coins_or_drbg(c, coins, n * ai.kpc, flags, h, nullptr, 0);
    if (rc) return rc;
    return kem_op(c, alg, 0, n, coins, nullptr, pk, sk, flags);
}

extern "C" int pqcgpu_kem_enc_batch(pqcgpu_ctx *c, pqcgpu_alg alg, size_t n, uint8_t *ct, uint8_t *ss,
                                    const uint8_t *pk, const uint8_t *coins, unsigned flags) {
    AlgInfo ai;
    if (!c || !alg_info(alg, &ai)) return set_err(PQCGPU_EINVAL, "bad context or algorithm");
    CoinsHolder h;
    int rc = coins_or_drbg(c, coins, n * ai.encc, flags, h, nullptr, 0);
    if (rc) return rc;
    return kem_op(c, alg, 1, n, pk, coins, ct, ss, flags);
}

extern "C" int pqcgpu_kem_dec_batch(pqcgpu_ctx *c, pqcgpu_alg alg, size_t n, uint8_t *ss, const uint8_t *ct,
                                    const uint8_t *sk, unsigned flags) {
    return kem_op(c, alg, 2, n, ct, sk, ss, nullptr, flags);
}

// ---------------------------------------------------------------------------------------------
// Mixed batches and CUDA graphs
// ---------------------------------------------------------------------------------------------
static int check_jobs(const pqcgpu_job *jobs, size_t njobs, int plain, size_t *scratch_total, size_t *offs) {
    if (!jobs && njobs) return set_err(PQCGPU_EINVAL, "jobs is NULL");
    size_t tot = 0;
    for (size_t i = 0; i < njobs; i++) {
        AlgInfo ai;
        const pqcgpu_job &j = jobs[i];
        if (!alg_info(j.alg, &ai) || j.op < 0 || j.op > 2 || j.n > ((uint64_t)1 << 30))
            return set_err(PQCGPU_EINVAL, "bad job (alg, op or n)");
        size_t sz[4];
        op_io_sizes(j.alg, j.op, sz);
        const void *ptrs[4] = {j.in0, j.in1, j.out0, j.out1};
        for (int q = 0; q < 4; q++) {
            if (sz[q] && j.n && !ptrs[q]) return set_err(PQCGPU_EINVAL, "null buffer in a job");
            if (sz[q] && ((uintptr_t)ptrs[q] & 15)) return set_err(PQCGPU_EINVAL, "device buffers must be 16-byte aligned");
        }
        if (offs) offs[i] = tot;
        tot += (op_scratch_bytes(j.alg, j.op, plain) * j.n + 255) & ~(size_t)255;
    }
    if (offs) offs[njobs] = tot;  // 256 bytes past the jobs' scratch: the persistent waves' counters
    *scratch_total = tot;
    return PQCGPU_OK;
}

// Fork the jobs over the context's parallel streams after the work already on `main`, join back.
static int launch_jobs(pqcgpu_ctx *c, const pqcgpu_job *jobs, size_t njobs, uint8_t *scratch, const size_t *offs,
                       int plain, cudaStream_t main, bool stage_kernels) {
    int rc = cuda_err(cudaEventRecord(c->fork_ev, main), "event record");
    if (rc) return rc;
    const int used = pqcgpu_ctx::NPAR;  // every parallel stream joins back (some may stay idle)
    for (int i = 0; i < used; i++)
        if ((rc = cuda_err(cudaStreamWaitEvent(c->par[i], c->fork_ev, 0), "wait event"))) return rc;
    // With stage_kernels, the Kyber key generations, encapsulations and decapsulations of round-3
    // arithmetic (all k, FO or ML-KEM) run their core stages as two persistent waves for all of them
    // (kyber_mixed.cu) on par[0], followed there by the NewHope jobs' wave; their per-job hash
    // kernels spread over the first HS parallel streams around the waves.  The FrodoKEM jobs' serial
    // sponges run per job on the remaining streams before and after the FrodoKEM waves (frodo.cu),
    // which run on the last stream; the other jobs round-robin over the remaining streams.
    // Otherwise every job's own kernels round-robin over all streams.
    constexpr int HS = pqcgpu_ctx::NPAR / 2;
    std::vector<MixedKyberJob> mix[3];
    std::vector<NhMixedJob> nhmix;
    std::vector<FrMixedJob> frmix;
    std::vector<size_t> rest;
    for (size_t i = 0; i < njobs; i++) {
        const pqcgpu_job &j = jobs[i];
        int variant = 0, k = 0;
        if (!plain && stage_kernels && kyber_alg(j.alg, &variant, &k) && variant == 3 && j.n > 0)
            mix[j.op].push_back(MixedKyberJob{k, kyber_kem_mode(j.alg), (int)j.n, j.in0, j.in1, j.out0, j.out1,
                                              scratch + offs[i]});
        else if (!plain && stage_kernels && (j.alg == PQCGPU_NEWHOPE1024 || j.alg == PQCGPU_NEWHOPE512) && j.n > 0)
            nhmix.push_back(NhMixedJob{j.alg == PQCGPU_NEWHOPE1024 ? 1024 : 512, j.op, (int)j.n, j.in0, j.in1, j.out0,
                                       j.out1, scratch + offs[i]});
        else if (!plain && stage_kernels && frodo_n(j.alg) && j.n > 0) {
            AlgInfo ai;
            alg_info(j.alg, &ai);
            frmix.push_back(FrMixedJob{frodo_n(j.alg), j.op, (int)j.n, (int)ai.kpc, j.in0, j.in1, j.out0, j.out1,
                                       scratch + offs[i]});
        } else
            rest.push_back(i);
    }
    const bool mixed = mix[0].size() + mix[1].size() + mix[2].size() + nhmix.size() + frmix.size() >= 2;
    if (!mixed) {
        rest.clear();
        for (size_t i = 0; i < njobs; i++) rest.push_back(i);
    }
    const int first = mixed ? HS : 0, nrest = pqcgpu_ctx::NPAR - first;
    for (size_t q = 0; q < rest.size(); q++) {
        const pqcgpu_job &j = jobs[rest[q]];
        rc = op_dev(j.alg, j.op, (int)j.n, j.in0, j.in1, j.out0, j.out1, scratch + offs[rest[q]], plain,
                    c->par[first + (int)(q % (size_t)nrest)]);
        if (rc) return set_err(rc, "job launch failed");
    }
    if (mixed && !frmix.empty()) {
        // FrodoKEM: per-job sponges on par[HS ..), the waves on par[NPAR - 1] once all of them are
        // done, the per-job sponges after the waves once those are
        unsigned *fr_counters =
            reinterpret_cast<unsigned *>(scratch + offs[njobs]) + MIXED_COUNTER_WORDS + MIXED_NH_COUNTER_WORDS;
        constexpr int FL = pqcgpu_ctx::NPAR - 1;
        int q = 0;
        for (const auto &j : frmix)
            if ((rc = frodo_mixed_pre(j, c->par[HS + q++ % (pqcgpu_ctx::NPAR - HS)]))) return set_err(rc, "job launch failed");
        for (int i = HS; i < FL; i++)
            if ((rc = cuda_err(cudaEventRecord(c->fr_ev[i], c->par[i]), "event record")) ||
                (rc = cuda_err(cudaStreamWaitEvent(c->par[FL], c->fr_ev[i], 0), "wait event")))
                return rc;
        if ((rc = frodo_mixed_wave(frmix, fr_counters, MIXED_FR_COUNTER_WORDS, c->par[FL])))
            return set_err(rc, "mixed FrodoKEM launch failed");
        if ((rc = cuda_err(cudaEventRecord(c->fr_core_ev, c->par[FL]), "event record"))) return rc;
        for (int i = HS; i < FL; i++)
            if ((rc = cuda_err(cudaStreamWaitEvent(c->par[i], c->fr_core_ev, 0), "wait event"))) return rc;
        q = 0;
        for (const auto &j : frmix)
            if ((rc = frodo_mixed_post(j, c->par[HS + q++ % (pqcgpu_ctx::NPAR - HS)]))) return set_err(rc, "job launch failed");
    }
    if (mixed) {
        unsigned *counters = reinterpret_cast<unsigned *>(scratch + offs[njobs]);
        auto join_into_main = [&](cudaEvent_t *evs) {  // par[0] waits for par[1 .. HS)
            for (int i = 1; i < HS; i++) {
                int r = cuda_err(cudaEventRecord(evs[i], c->par[i]), "event record");
                if (!r) r = cuda_err(cudaStreamWaitEvent(c->par[0], evs[i], 0), "wait event");
                if (r) return r;
            }
            return (int)PQCGPU_OK;
        };
        auto fork_from_main = [&]() {  // par[1 .. HS) wait for par[0]
            int r = cuda_err(cudaEventRecord(c->core_ev, c->par[0]), "event record");
            for (int i = 1; i < HS && !r; i++) r = cuda_err(cudaStreamWaitEvent(c->par[i], c->core_ev, 0), "wait event");
            return r;
        };
        int q = 0;
        for (int op = 0; op <= 2; op++)  // phase 0 hashes
            for (const auto &j : mix[op])
                if ((rc = kyber_mixed_hash(op, 0, j, c->par[q++ % HS]))) return set_err(rc, "job launch failed");
        for (const auto &j : nhmix)
            if ((rc = newhope_mixed_pre(j, c->par[q++ % HS]))) return set_err(rc, "job launch failed");
        if ((rc = join_into_main(c->stage_ev))) return rc;
        if ((rc = kyber_mixed_wave(0, mix, counters, c->par[0]))) return set_err(rc, "mixed Kyber launch failed");
        if ((rc = fork_from_main())) return rc;
        // the NewHope wave follows Kyber's first wave on par[0], while the Kyber jobs' G kernels run
        // on the other streams
        if (!nhmix.empty() &&
            (rc = newhope_mixed_wave(nhmix, counters + MIXED_COUNTER_WORDS, MIXED_NH_COUNTER_WORDS, c->par[0])))
            return set_err(rc, "mixed NewHope launch failed");
        q = 1;
        for (const auto &j : mix[2])  // decapsulation's G between the waves, on par[1 .. HS)
            if ((rc = kyber_mixed_hash(2, 1, j, c->par[1 + (q++ - 1) % (HS - 1)]))) return set_err(rc, "job launch failed");
        if (!mix[2].empty()) {
            if ((rc = join_into_main(c->stage_ev2))) return rc;
            if ((rc = kyber_mixed_wave(1, mix, counters, c->par[0]))) return set_err(rc, "mixed Kyber launch failed");
        }
        q = 1;
        for (int op = 0; op <= 1; op++)  // keypair / encapsulation phase 2 hashes, after wave 0
            for (const auto &j : mix[op])
                if ((rc = kyber_mixed_hash(op, 2, j, c->par[1 + (q++ - 1) % (HS - 1)]))) return set_err(rc, "job launch failed");
        if (!mix[2].empty()) {
            if ((rc = fork_from_main())) return rc;
            q = 1;
            for (const auto &j : mix[2])
                if ((rc = kyber_mixed_hash(2, 2, j, c->par[1 + (q++ - 1) % (HS - 1)]))) return set_err(rc, "job launch failed");
        }
    }
    for (int i = 0; i < used; i++) {
        if ((rc = cuda_err(cudaEventRecord(c->join_ev[i], c->par[i]), "event record"))) return rc;
        if ((rc = cuda_err(cudaStreamWaitEvent(main, c->join_ev[i], 0), "wait event"))) return rc;
    }
    return PQCGPU_OK;
}

extern "C" int pqcgpu_kem_mixed_batch(pqcgpu_ctx *c, const pqcgpu_job *jobs, size_t njobs, unsigned flags) {
    if (!c) return set_err(PQCGPU_EINVAL, "bad context");
    if (!(flags & PQCGPU_DEVICE_PTRS)) return set_err(PQCGPU_EINVAL, "mixed batches take device pointers");
    const int plain = (flags & PQCGPU_PLAIN) ? 1 : 0;
    std::lock_guard<std::recursive_mutex> lk(c->mu);
    int rc = cuda_err(cudaSetDevice(c->device), "cudaSetDevice");
    if (rc) return rc;
    std::vector<size_t> offs(njobs + 1);
    size_t tot = 0;
    if ((rc = check_jobs(jobs, njobs, plain, &tot, offs.data()))) return rc;
    if ((rc = c->reserve(tot + 256))) return rc;
    return launch_jobs(c, jobs, njobs, c->arena, offs.data(), plain, c->stream, (flags & PQCGPU_STAGE_KERNELS) != 0);
}

struct pqcgpu_graph {
    pqcgpu_ctx *ctx = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    uint8_t *scratch = nullptr;
};

extern "C" int pqcgpu_graph_capture(pqcgpu_ctx *c, const pqcgpu_job *jobs, size_t njobs, unsigned flags,
                                    pqcgpu_graph **out) {
    if (!c || !out) return set_err(PQCGPU_EINVAL, "bad context or output");
    *out = nullptr;
    if (!(flags & PQCGPU_DEVICE_PTRS)) return set_err(PQCGPU_EINVAL, "graphs take device pointers");
    const int plain = (flags & PQCGPU_PLAIN) ? 1 : 0;
    std::lock_guard<std::recursive_mutex> lk(c->mu);
    int rc = cuda_err(cudaSetDevice(c->device), "cudaSetDevice");
    if (rc) return rc;
    std::vector<size_t> offs(njobs + 1);
    size_t tot = 0;
    if ((rc = check_jobs(jobs, njobs, plain, &tot, offs.data()))) return rc;
    pqcgpu_graph *g = new pqcgpu_graph();
    g->ctx = c;
    if (cudaMalloc(&g->scratch, tot + 256) != cudaSuccess) {
        cudaGetLastError();
        delete g;
        return set_err(PQCGPU_ENOMEM, "graph scratch allocation failed");
    }
    // one uncaptured pass: loads the kernels and sets their shared-memory attributes
    rc = launch_jobs(c, jobs, njobs, g->scratch, offs.data(), plain, c->stream, (flags & PQCGPU_STAGE_KERNELS) != 0);
    if (!rc) rc = cuda_err(cudaStreamSynchronize(c->stream), "warm-up");
    if (!rc) {
        set_capturing(true);
        rc = cuda_err(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal), "begin capture");
        if (!rc) {
            const int lrc = launch_jobs(c, jobs, njobs, g->scratch, offs.data(), plain, c->stream,
                                        (flags & PQCGPU_STAGE_KERNELS) != 0);
            const int erc = cuda_err(cudaStreamEndCapture(c->stream, &g->graph), "end capture");
            rc = lrc ? lrc : erc;
        }
        set_capturing(false);
    }
    if (!rc) rc = cuda_err(cudaGraphInstantiate(&g->exec, g->graph, 0), "graph instantiate");
    if (rc) {
        if (g->graph) cudaGraphDestroy(g->graph);
        cudaFree(g->scratch);
        delete g;
        return rc;
    }
    *out = g;
    return PQCGPU_OK;
}
extern "C" int pqcgpu_graph_launch(pqcgpu_graph *g) {
    if (!g) return set_err(PQCGPU_EINVAL, "null graph");
    std::lock_guard<std::recursive_mutex> lk(g->ctx->mu);
    return cuda_err(cudaGraphLaunch(g->exec, g->ctx->stream), "graph launch");
}
extern "C" int pqcgpu_graph_destroy(pqcgpu_graph *g) {
    if (!g) return PQCGPU_EINVAL;
    cudaStreamSynchronize(g->ctx->stream);
    if (g->exec) cudaGraphExecDestroy(g->exec);
    if (g->graph) cudaGraphDestroy(g->graph);
    if (g->scratch) cudaFree(g->scratch);
    delete g;
    return PQCGPU_OK;
}

// ---- many FrodoKEM encapsulations to one public key ----
extern "C" int pqcgpu_frodo_enc_shared_key_batch(pqcgpu_ctx *c, pqcgpu_alg alg, size_t n, uint8_t *ct, uint8_t *ss,
                                                 const uint8_t *pk, const uint8_t *coins, unsigned flags) {
    AlgInfo ai;
    const int N = frodo_n(alg);
    if (!c || !N || !alg_info(alg, &ai)) return set_err(PQCGPU_EINVAL, "bad context, or not a FrodoKEM algorithm");
    if (n == 0) return PQCGPU_OK;
    if (n > ((size_t)1 << 20)) return set_err(PQCGPU_EINVAL, "n above 2^20");
    if (!ct || !ss || !pk) return set_err(PQCGPU_EINVAL, "null buffer");
    CoinsHolder h;
    int rc = coins_or_drbg(c, coins, n * ai.encc, flags, h, nullptr, 0);
    if (rc) return rc;
    const bool dev = (flags & PQCGPU_DEVICE_PTRS) != 0;
    if (dev && (((uintptr_t)ct | (uintptr_t)ss | (uintptr_t)pk | (uintptr_t)coins) & 15))
        return set_err(PQCGPU_EINVAL, "device buffers must be 16-byte aligned");
    std::lock_guard<std::recursive_mutex> lk(c->mu);
    if ((rc = cuda_err(cudaSetDevice(c->device), "cudaSetDevice"))) return rc;
    auto up = [](size_t b) { return (b + 255) & ~(size_t)255; };
    const size_t scr = up(n * frodo_scratch_bytes(N)), extra = up(frodo_shared_extra_bytes(N));
    const size_t s16b = up(fr_tc_s_bytes(N, (int)n));
    const size_t io = dev ? 0 : up(ai.pk) + up(n * ai.encc) + up(n * ai.ct) + up(n * ai.ss);
    if ((rc = c->reserve(scr + extra + s16b + io))) return rc;
    uint8_t *b = c->arena, *scratch = b, *ex = b + scr;
    uint16_t *s16 = reinterpret_cast<uint16_t *>(b + scr + extra);
    const uint8_t *dpk = pk, *dmu = coins;
    uint8_t *dct = ct, *dss = ss;
    cudaStream_t st = c->stream;
    if (!dev) {
        uint8_t *q = b + scr + extra + s16b;
        uint8_t *bpk = q, *bmu = q + up(ai.pk);
        dct = bmu + up(n * ai.encc);
        dss = dct + up(n * ai.ct);
        if ((rc = cuda_err(cudaMemcpyAsync(bpk, pk, ai.pk, cudaMemcpyHostToDevice, st), "copy in")) ||
            (rc = cuda_err(cudaMemcpyAsync(bmu, coins, n * ai.encc, cudaMemcpyHostToDevice, st), "copy in")))
            return rc;
        dpk = bpk;
        dmu = bmu;
    }
    if (!c->dev_err) {
        if (cudaMalloc(&c->dev_err, 256) != cudaSuccess) {
            cudaGetLastError();
            return set_err(PQCGPU_ENOMEM, "cudaMalloc of the error word failed");
        }
        if ((rc = cuda_err(cudaMemsetAsync(c->dev_err, 0, sizeof(unsigned), st), "memset"))) return rc;
    }
    if ((rc = frodo_enc_shared_dev(N, (int)n, dct, dss, dpk, dmu, scratch, ex, s16, c->dev_err, st)))
        return set_err(rc, "launch failed");
    c->dev_err_pending = true;
    if (dev) return PQCGPU_OK;  // pqcgpu_ctx_wait reports a wait that ran out
    if ((rc = cuda_err(cudaMemcpyAsync(ct, dct, n * ai.ct, cudaMemcpyDeviceToHost, st), "copy out")) ||
        (rc = cuda_err(cudaMemcpyAsync(ss, dss, n * ai.ss, cudaMemcpyDeviceToHost, st), "copy out")) ||
        (rc = cuda_err(cudaStreamSynchronize(st), "synchronize")))
        return rc;
    return c->take_dev_err();
}

// ---- launch shapes (autotuner) ----
extern "C" int pqcgpu_set_launch_shape(pqcgpu_alg alg, int op, int ni, int threads) {
    int variant, k, rc;
    if (kyber_alg(alg, &variant, &k)) rc = kyber_set_shape(op, k, ni, threads);
    else if (alg == PQCGPU_NEWHOPE1024) rc = newhope_set_shape(1024, op, ni, threads);
    else if (alg == PQCGPU_NEWHOPE512) rc = newhope_set_shape(512, op, ni, threads);
    else if (frodo_n(alg)) rc = frodo_set_shape(op, ni, threads);
    else rc = PQCGPU_EUNSUPPORTED;
    return rc ? set_err(rc, "launch shape not accepted") : PQCGPU_OK;
}
extern "C" int pqcgpu_get_launch_shape(pqcgpu_alg alg, int op, int *ni, int *threads) {
    int variant, k;
    if (!ni || !threads) return set_err(PQCGPU_EINVAL, "null output");
    if (kyber_alg(alg, &variant, &k)) return kyber_get_shape(op, k, ni, threads);
    if (alg == PQCGPU_NEWHOPE1024) return newhope_get_shape(1024, op, ni, threads);
    if (alg == PQCGPU_NEWHOPE512) return newhope_get_shape(512, op, ni, threads);
    if (frodo_n(alg)) return frodo_get_shape(op, ni, threads);
    return set_err(PQCGPU_EUNSUPPORTED, "no tunable launch shape for this algorithm");
}

// ---- CPA level ----
static bool kyber_vk_ok(int variant, int k) { return (variant == 2 || variant == 3) && k >= 2 && k <= 4; }
static size_t kyber_cpa_ct(int variant, int k) {
    const int du = (variant == 2 || k == 4) ? 11 : 10, dv = (variant == 2 || k == 4) ? 5 : 4;
    return (size_t)k * du * 32 + (size_t)dv * 32;
}

extern "C" int pqcgpu_kyber_indcpa_keypair_batch(pqcgpu_ctx *c, int variant, int k, size_t n, uint8_t *pk,
                                                 uint8_t *sk, const uint8_t *dseed, unsigned flags) {
    if (!c || !kyber_vk_ok(variant, k)) return set_err(PQCGPU_EINVAL, "bad context, variant or k");
    OpDesc d;
    d.nin = 1;
    d.in[0] = dseed;
    d.in_sz[0] = 32;
    d.nout = 2;
    d.out[0] = pk;
    d.out_sz[0] = 384 * k + 32;
    d.out[1] = sk;
    d.out_sz[1] = 384 * k;
    return run_op(c, n, d, flags, [&](int m, const uint8_t *const *in, uint8_t *const *out, uint8_t *, cudaStream_t s) {
        return kyber_keypair_dev(variant, k, m, out[0], out[1], in[0], 32, 0, nullptr, 0, s);
    });
}
extern "C" int pqcgpu_kyber_indcpa_enc_batch(pqcgpu_ctx *c, int variant, int k, size_t n, uint8_t *ct,
                                             const uint8_t *msg, const uint8_t *pk, const uint8_t *coins,
                                             unsigned flags) {
    if (!c || !kyber_vk_ok(variant, k)) return set_err(PQCGPU_EINVAL, "bad context, variant or k");
    OpDesc d;
    d.nin = 3;
    d.in[0] = pk;
    d.in_sz[0] = 384 * k + 32;
    d.in[1] = msg;
    d.in_sz[1] = 32;
    d.in[2] = coins;
    d.in_sz[2] = 32;
    d.nout = 1;
    d.out[0] = ct;
    d.out_sz[0] = kyber_cpa_ct(variant, k);
    return run_op(c, n, d, flags, [&](int m, const uint8_t *const *in, uint8_t *const *out, uint8_t *, cudaStream_t s) {
        return kyber_enc_dev(variant, k, m, out[0], nullptr, in[0], in[1], in[2], nullptr, 0, 0, s);
    });
}
extern "C" int pqcgpu_kyber_indcpa_dec_batch(pqcgpu_ctx *c, int variant, int k, size_t n, uint8_t *msg,
                                             const uint8_t *ct, const uint8_t *sk, unsigned flags) {
    if (!c || !kyber_vk_ok(variant, k)) return set_err(PQCGPU_EINVAL, "bad context, variant or k");
    OpDesc d;
    d.nin = 2;
    d.in[0] = ct;
    d.in_sz[0] = kyber_cpa_ct(variant, k);
    d.in[1] = sk;
    d.in_sz[1] = 384 * k;
    d.nout = 1;
    d.out[0] = msg;
    d.out_sz[0] = 32;
    return run_op(c, n, d, flags, [&](int m, const uint8_t *const *in, uint8_t *const *out, uint8_t *, cudaStream_t s) {
        return kyber_dec_dev(variant, k, m, out[0], in[0], in[1], nullptr, 0, 0, s);
    });
}

extern "C" int pqcgpu_set_host_pipeline(size_t chunk_max, size_t chunk_first, size_t chunk_last, int streams) {
    PipeShape p;
    if (chunk_max) p.chunk_max = chunk_max;
    p.chunk_first = chunk_first ? chunk_first : p.chunk_max / 8;
    p.chunk_last = chunk_last ? chunk_last : p.chunk_max / 4;
    if (streams) p.streams = streams;
    if (p.chunk_max < 64 || p.chunk_max > ((size_t)1 << 24))
        return set_err(PQCGPU_EINVAL, "chunk_max must lie in [64, 2^24]");
    if (p.chunk_first < 1 || p.chunk_first > p.chunk_max || p.chunk_last < 1 || p.chunk_last > p.chunk_max)
        return set_err(PQCGPU_EINVAL, "chunk_first and chunk_last must lie in [1, chunk_max]");
    if (p.streams < 1 || p.streams > pqcgpu_ctx::NPAR) return set_err(PQCGPU_EINVAL, "streams must lie in [1, 8]");
    std::lock_guard<std::mutex> lk(g_pipe_mu);
    g_pipe = p;
    return PQCGPU_OK;
}
extern "C" int pqcgpu_get_host_pipeline(size_t *chunk_max, size_t *chunk_first, size_t *chunk_last, int *streams) {
    if (!chunk_max || !chunk_first || !chunk_last || !streams) return set_err(PQCGPU_EINVAL, "NULL argument");
    std::lock_guard<std::mutex> lk(g_pipe_mu);
    *chunk_max = g_pipe.chunk_max;
    *chunk_first = g_pipe.chunk_first;
    *chunk_last = g_pipe.chunk_last;
    *streams = g_pipe.streams;
    return PQCGPU_OK;
}

extern "C" int pqcgpu_profile_enable(int on) {
    prof_enable(on != 0);
    return PQCGPU_OK;
}
extern "C" int pqcgpu_profile_read(char *buf, size_t len) {
    const std::string s = prof_read();
    if (!buf || len < s.size() + 1) return set_err(PQCGPU_EINVAL, "profile buffer too small");
    memcpy(buf, s.c_str(), s.size() + 1);
    return PQCGPU_OK;
}
extern "C" int pqcgpu_profile_trace(char *buf, size_t *len) {
    if (!len) return set_err(PQCGPU_EINVAL, "len is NULL");
    size_t need = 0;
    const bool ok = prof_trace(buf, *len, &need);
    *len = need;
    return ok ? PQCGPU_OK : set_err(PQCGPU_EINVAL, "trace buffer too small (the records are kept; *len = bytes needed)");
}
extern "C" int pqcgpu_probe_peaks(int device, double *int_ops_per_s, double *keccak_perms_per_s) {
    const int rc = probe_peaks(device, int_ops_per_s, keccak_perms_per_s);
    return rc ? set_err(rc, "probe failed") : PQCGPU_OK;
}

// ---- NewHope CPA level (replaces cpapke_* of NewHope_NIST_GPU/cpapke.h:14-24; N = 1024 or 512
// as the reference's NEWHOPE_N, params.h:9-11) ----
static int nh_cpa_keypair(int N, pqcgpu_ctx *c, size_t n, uint8_t *pk, uint8_t *sk, const uint8_t *seed, unsigned flags) {
    if (!c) return set_err(PQCGPU_EINVAL, "bad context");
    const size_t pb = 14 * (size_t)N / 8;
    OpDesc d;
    d.nin = 1;
    d.in[0] = seed;
    d.in_sz[0] = 32;
    d.nout = 2;
    d.out[0] = pk;
    d.out_sz[0] = pb + 32;
    d.out[1] = sk;
    d.out_sz[1] = pb;
    return run_op(c, n, d, flags, [&](int m, const uint8_t *const *in, uint8_t *const *out, uint8_t *, cudaStream_t s) {
        return newhope_keypair_dev(N, m, out[0], out[1], in[0], 32, s);
    });
}
static int nh_cpa_enc(int N, pqcgpu_ctx *c, size_t n, uint8_t *ct, const uint8_t *msg, const uint8_t *pk,
                      const uint8_t *coin, unsigned flags) {
    if (!c) return set_err(PQCGPU_EINVAL, "bad context");
    const size_t pb = 14 * (size_t)N / 8;
    OpDesc d;
    d.nin = 3;
    d.in[0] = pk;
    d.in_sz[0] = pb + 32;
    d.in[1] = msg;
    d.in_sz[1] = 32;
    d.in[2] = coin;
    d.in_sz[2] = 32;
    d.nout = 1;
    d.out[0] = ct;
    d.out_sz[0] = pb + 3 * (size_t)N / 8;
    return run_op(c, n, d, flags, [&](int m, const uint8_t *const *in, uint8_t *const *out, uint8_t *, cudaStream_t s) {
        return newhope_enc_dev(N, m, out[0], nullptr, in[0], in[1], in[2], nullptr, 0, s);
    });
}
static int nh_cpa_dec(int N, pqcgpu_ctx *c, size_t n, uint8_t *msg, const uint8_t *ct, const uint8_t *sk,
                      unsigned flags) {
    if (!c) return set_err(PQCGPU_EINVAL, "bad context");
    const size_t pb = 14 * (size_t)N / 8;
    OpDesc d;
    d.nin = 2;
    d.in[0] = ct;
    d.in_sz[0] = pb + 3 * (size_t)N / 8;
    d.in[1] = sk;
    d.in_sz[1] = pb;
    d.nout = 1;
    d.out[0] = msg;
    d.out_sz[0] = 32;
    return run_op(c, n, d, flags, [&](int m, const uint8_t *const *in, uint8_t *const *out, uint8_t *, cudaStream_t s) {
        return newhope_dec_dev(N, m, out[0], in[0], in[1], 0, s);
    });
}
extern "C" int pqcgpu_newhope_cpapke_keypair_batch(pqcgpu_ctx *c, size_t n, uint8_t *pk, uint8_t *sk,
                                                   const uint8_t *seed, unsigned flags) {
    return nh_cpa_keypair(1024, c, n, pk, sk, seed, flags);
}
extern "C" int pqcgpu_newhope_cpapke_enc_batch(pqcgpu_ctx *c, size_t n, uint8_t *ct, const uint8_t *msg,
                                               const uint8_t *pk, const uint8_t *coin, unsigned flags) {
    return nh_cpa_enc(1024, c, n, ct, msg, pk, coin, flags);
}
extern "C" int pqcgpu_newhope_cpapke_dec_batch(pqcgpu_ctx *c, size_t n, uint8_t *msg, const uint8_t *ct,
                                               const uint8_t *sk, unsigned flags) {
    return nh_cpa_dec(1024, c, n, msg, ct, sk, flags);
}
extern "C" int pqcgpu_newhope512_cpapke_keypair_batch(pqcgpu_ctx *c, size_t n, uint8_t *pk, uint8_t *sk,
                                                      const uint8_t *seed, unsigned flags) {
    return nh_cpa_keypair(512, c, n, pk, sk, seed, flags);
}
extern "C" int pqcgpu_newhope512_cpapke_enc_batch(pqcgpu_ctx *c, size_t n, uint8_t *ct, const uint8_t *msg,
                                                  const uint8_t *pk, const uint8_t *coin, unsigned flags) {
    return nh_cpa_enc(512, c, n, ct, msg, pk, coin, flags);
}
extern "C" int pqcgpu_newhope512_cpapke_dec_batch(pqcgpu_ctx *c, size_t n, uint8_t *msg, const uint8_t *ct,
                                                  const uint8_t *sk, unsigned flags) {
    return nh_cpa_dec(512, c, n, msg, ct, sk, flags);
}

// ---- NIST single-instance API (default context on device 0) ----
static pqcgpu_ctx *g_default_ctx = nullptr;
static std::mutex g_default_mu;
static pqcgpu_ctx *default_ctx() {
    std::lock_guard<std::mutex> lk(g_default_mu);
    if (!g_default_ctx) pqcgpu_ctx_create(&g_default_ctx, 0, (size_t)256 << 20);
    return g_default_ctx;
}
// The coins of one NIST crypto_kem_* call are drawn from the library DRBG in the calls the
// algorithm's submission package makes to randombytes, so that with the CTR_DRBG of the NIST KAT
// generator (pqcgpu_randombytes_init_nist) the keys and ciphertexts are those of its .rsp files:
// Kyber (rounds 2 / 3) keypair d then z (32 + 32: indcpa_keypair, then crypto_kem_keypair);
// ML-KEM keypair d || z in one call (the derandomized FIPS 203 API); FrodoKEM s || seedSE || z in
// one call; one call for every encapsulation (m, or mu for FrodoKEM).
extern "C" int pqcgpu_nist_coins(pqcgpu_alg alg, int op, uint8_t *coins) {
    AlgInfo ai;
    if (!coins || !alg_info(alg, &ai) || op < 0 || op > 1) return PQCGPU_EINVAL;
    int variant, k;
    const bool split = op == 0 && kyber_alg(alg, &variant, &k) && kyber_kem_mode(alg) == 1;
    bool ok;
    if (split) {  // two draws, not interleaved with other threads' draws
        std::lock_guard<std::mutex> lk(g_drbg_mu);
        ok = drbg_bytes_locked(coins, 32) && drbg_bytes_locked(coins + 32, 32);
    } else {
        ok = drbg_bytes(coins, op == 0 ? ai.kpc : ai.encc);
    }
    return ok ? PQCGPU_OK : set_err(PQCGPU_EUNSUPPORTED, "no operating-system entropy to seed the DRBG");
}

#define PQC_NIST(NAME, ALG)                                                                              \
    extern "C" int pqcgpu_##NAME##_crypto_kem_keypair(unsigned char *pk, unsigned char *sk) {             \
        pqcgpu_ctx *c = default_ctx();                                                                   \
        uint8_t coins[128]; /* >= every kp_coins / enc_coins size (at most 80) */                         \
        if (!c) return PQCGPU_ECUDA;                                                                     \
        if (int rc_ = pqcgpu_nist_coins(ALG, 0, coins)) return rc_;                                      \
        return pqcgpu_kem_keypair_batch(c, ALG, 1, pk, sk, coins, 0);                                    \
    }                                                                                                    \
    extern "C" int pqcgpu_##NAME##_crypto_kem_enc(unsigned char *ct, unsigned char *ss, const unsigned char *pk) { \
        pqcgpu_ctx *c = default_ctx();                                                                   \
        uint8_t coins[128]; /* >= every kp_coins / enc_coins size (at most 80) */                         \
        if (!c) return PQCGPU_ECUDA;                                                                     \
        if (int rc_ = pqcgpu_nist_coins(ALG, 1, coins)) return rc_;                                      \
        return pqcgpu_kem_enc_batch(c, ALG, 1, ct, ss, pk, coins, 0);                                    \
    }                                                                                                    \
    extern "C" int pqcgpu_##NAME##_crypto_kem_dec(unsigned char *ss, const unsigned char *ct, const unsigned char *sk) { \
        pqcgpu_ctx *c = default_ctx();                                                                   \
        return c ? pqcgpu_kem_dec_batch(c, ALG, 1, ss, ct, sk, 0) : PQCGPU_ECUDA;                        \
    }
PQC_NIST(mlkem512, PQCGPU_MLKEM512)
PQC_NIST(mlkem768, PQCGPU_MLKEM768)
PQC_NIST(mlkem1024, PQCGPU_MLKEM1024)
PQC_NIST(kyber512, PQCGPU_KYBER512)
PQC_NIST(kyber768, PQCGPU_KYBER768)
PQC_NIST(kyber1024, PQCGPU_KYBER1024)
PQC_NIST(newhope1024, PQCGPU_NEWHOPE1024)
PQC_NIST(newhope512, PQCGPU_NEWHOPE512)
PQC_NIST(frodo976, PQCGPU_FRODO976)
PQC_NIST(frodo640, PQCGPU_FRODO640)
PQC_NIST(frodo1344, PQCGPU_FRODO1344)
