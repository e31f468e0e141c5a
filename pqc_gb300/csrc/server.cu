// Serving loop: continuous batching of mixed KEM requests with device-resident keys.
//
// The reference has no serving path: its drivers run one fixed-size batch at a time from main()
// (Kyber_GPU_Batched/main.cu:371-503).  Here a dispatcher thread turns a stream of individual
// requests (keypair / encapsulation / decapsulation, any algorithm) into GPU batches:
//   * requests queue up; whenever an in-flight slot (a stream + staging buffers) is free, the
//     dispatcher takes the (algorithm, operation) group of the oldest waiting request, up to
//     max_batch requests of it, packs their inputs into pinned memory, copies them up, runs the
//     batched kernels and copies the results back -- all on the slot's stream;
//   * up to max_inflight batches run at once, so requests that arrive while others are on the GPU
//     are admitted as soon as a slot is free and overlap with them on the device;
//   * keys live on the device: a keypair stores pk / sk in a per-algorithm key store and returns a
//     handle; encapsulation / decapsulation by handle gather the keys on the device;
//   * admission is by device-memory budget: the key stores and the slots' buffers together stay
//     within the budget given at creation (a batch is cut short, or waits, when it would not fit).
// Results are identical to the batched entry points: every instance of a batch is independent,
// so a request's bytes do not depend on what it was batched with.
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <memory>
#include <mutex>
#include <random>
#include <thread>
#include <unordered_map>
#include <vector>

#include "pqcgpu_internal.h"

namespace pqc {
namespace {

using Clock = std::chrono::steady_clock;

// copy rows of `row` bytes (multiple of 16): dst[i] = src[idx[i]] (gather) or dst[idx[i]] = src[i]
__global__ void rows_gather(uint4 *dst, const uint4 *src, const uint32_t *idx, int n, int row16) {
    const int r = blockIdx.y * 8 + (threadIdx.x >> 5);
    if (r >= n) return;
    const uint4 *s = src + (size_t)idx[r] * row16;
    uint4 *d = dst + (size_t)r * row16;
    for (int i = threadIdx.x & 31; i < row16; i += 32) d[i] = s[i];
}
__global__ void rows_scatter(uint4 *dst, const uint4 *src, const uint32_t *idx, int n, int row16) {
    const int r = blockIdx.y * 8 + (threadIdx.x >> 5);
    if (r >= n) return;
    const uint4 *s = src + (size_t)r * row16;
    uint4 *d = dst + (size_t)idx[r] * row16;
    for (int i = threadIdx.x & 31; i < row16; i += 32) d[i] = s[i];
}
// dst[i] = `words` 8-byte words at byte offset `off` of row idx[i] of src (row, off 8-byte aligned)
__global__ void rows_tail_gather(uint2 *dst, const uint8_t *src, const uint32_t *idx, int n, size_t row, size_t off,
                                 int words) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n * words) return;
    const int i = t / words, w = t % words;
    dst[t] = reinterpret_cast<const uint2 *>(src + (size_t)idx[i] * row + off)[w];
}

void launch_rows(bool gather, uint8_t *dst, const uint8_t *src, const uint32_t *idx, int n, size_t row, cudaStream_t st) {
    if (n <= 0) return;
    const dim3 grid(1, (n + 7) / 8);
    if (gather)
        PQC_LAUNCH(st, "rows_gather", 0, 0,
                   rows_gather<<<grid, 256, 0, st>>>((uint4 *)dst, (const uint4 *)src, idx, n, (int)(row / 16)));
    else
        PQC_LAUNCH(st, "rows_scatter", 0, 0,
                   rows_scatter<<<grid, 256, 0, st>>>((uint4 *)dst, (const uint4 *)src, idx, n, (int)(row / 16)));
}

struct Req {
    pqcgpu_request r;
    uint64_t ticket;
    Clock::time_point t0;
    int status = 1;  // 1 pending, 0 done, < 0 error
    uint32_t key_slot = 0;
};

struct KeyStore {
    size_t pkb = 0, skb = 0;
    uint8_t *dpk = nullptr, *dsk = nullptr;
    uint32_t cap = 0;
    std::vector<uint32_t> free_slots;
    std::vector<uint8_t> used;
};

// One in-flight batch: a stream, staging buffers and a worker thread that packs the inputs, runs
// the copies and kernels, waits for them and hands the results back.  The dispatcher fills in the
// job under the server mutex; the worker runs it without the mutex.
struct Slot {
    cudaStream_t stream = nullptr;     // the stream of the current job (hi or lo)
    cudaStream_t hi = nullptr, lo = nullptr;  // light algorithms run at high priority, FrodoKEM at low
    cudaEvent_t done = nullptr;
    uint8_t *dbuf = nullptr;  // device staging
    size_t dcap = 0;
    uint8_t *hbuf = nullptr;  // pinned host staging
    size_t hcap = 0;
    bool busy = false;     // assigned by the dispatcher, until the worker has completed it
    bool has_job = false;  // handed over, not yet picked up by the worker
    std::condition_variable cv;
    std::thread th;
    // the job
    int alg = 0, op = 0, n = 0;
    bool by_handle = false;
    bool use_pkh = false;  // FrodoKEM encaps by handle: pkh = SHAKE256(pk) taken from the resident sk
    std::vector<Req *> reqs;
    std::vector<uint32_t> idx;
    uint8_t *kpk = nullptr, *ksk = nullptr;  // key store rows of `alg` (stable while any slot is busy)
    size_t pkb = 0, skb = 0;
    // staging layout, device and host alike: [idx | host inputs | gathered input | out0 | out1 | scratch]
    size_t off_in0 = 0, off_in1 = 0, off_out0 = 0, off_out1 = 0, off_scr = 0, off_pkh = 0, h2d_bytes = 0, d2h_bytes = 0;
};

size_t r256(size_t v) { return (v + 255) & ~(size_t)255; }

}  // namespace
}  // namespace pqc

using namespace pqc;

struct pqcgpu_server {
    int device = 0;
    size_t budget = 0, used = 0;
    int max_inflight = 4, max_batch = 4096;
    std::vector<std::unique_ptr<Slot>> slots;
    KeyStore ks[PQCGPU_NUM_ALGS];
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    uint64_t events = 0;  // bumped on every submit and completion; the dispatcher sleeps until it moves
    // one FIFO per (algorithm, operation); the dispatcher serves the group with the oldest head
    std::deque<Req *> groups[PQCGPU_NUM_ALGS][3];
    size_t pending = 0;
    int heavy_running = 0;  // in-flight FrodoKEM batches (at most all slots but a quarter)
    int grow_alg = -1;      // a key store waits to grow: no new batch starts until all slots are idle
    uint32_t grow_need = 0;
    std::unordered_map<uint64_t, std::unique_ptr<Req>> reqs;
    uint64_t next_ticket = 1;
    bool stop = false, stop_workers = false;
    std::thread th;
    std::vector<double> lat_ms;
    std::vector<double> lat_grp[PQCGPU_NUM_ALGS][3];  // the same samples per (algorithm, operation)
    uint64_t completed = 0, batches = 0;
    std::string error;

    int alloc_dev(uint8_t **p, size_t bytes) {
        if (used + bytes > budget) return PQCGPU_EBUDGET;
        if (cudaMalloc(p, bytes) != cudaSuccess) {
            cudaGetLastError();
            return PQCGPU_ENOMEM;
        }
        used += bytes;
        return PQCGPU_OK;
    }
    void free_dev(uint8_t *p, size_t bytes) {
        if (p) {
            cudaFree(p);
            used -= bytes;
        }
    }
    bool any_busy() const {
        for (auto &sl : slots)
            if (sl->busy) return true;
        return false;
    }
    // Grow the key store of `alg` to at least `need` rows.  Only called with every slot idle: the
    // rows move to new arrays, and no batch may hold the old pointers.
    int grow_keys(int alg, uint32_t need) {
        KeyStore &k = ks[alg];
        if (need <= k.cap) return PQCGPU_OK;
        uint32_t cap = std::max<uint32_t>(need, std::max<uint32_t>(1024, k.cap * 2));
        uint8_t *npk = nullptr, *nsk = nullptr;
        int rc = alloc_dev(&npk, (size_t)cap * k.pkb);
        if (rc) return rc;
        if ((rc = alloc_dev(&nsk, (size_t)cap * k.skb))) {
            free_dev(npk, (size_t)cap * k.pkb);
            return rc;
        }
        if (k.cap) {
            cudaDeviceSynchronize();
            cudaMemcpy(npk, k.dpk, (size_t)k.cap * k.pkb, cudaMemcpyDeviceToDevice);
            cudaMemcpy(nsk, k.dsk, (size_t)k.cap * k.skb, cudaMemcpyDeviceToDevice);
            free_dev(k.dpk, (size_t)k.cap * k.pkb);
            free_dev(k.dsk, (size_t)k.cap * k.skb);
        }
        for (uint32_t i = cap; i > k.cap; i--) k.free_slots.push_back(i - 1);
        k.used.resize(cap, 0);
        k.dpk = npk;
        k.dsk = nsk;
        k.cap = cap;
        return PQCGPU_OK;
    }
    bool key_ok(uint64_t h, int alg, uint32_t *slot) {
        if ((int)(h >> 48) != alg) return false;
        const uint64_t s = (h & 0xffffffffffffull);
        if (s == 0 || s > ks[alg].cap || !ks[alg].used[s - 1]) return false;
        *slot = (uint32_t)(s - 1);
        return true;
    }

    void finish(Req *q, int status, double ms) {
        q->status = status;
        if (status == 0) {
            lat_ms.push_back(ms);
            lat_grp[q->r.alg][q->r.op].push_back(ms);
            completed++;
        }
    }

    // Pick the next batch and hand it to a free slot's worker (mutex held).  Returns false when
    // nothing can start now.
    bool assign_one() {
        if (!pending) return false;
        Slot *slot = nullptr;
        for (auto &s : slots)
            if (!s->busy) {
                slot = s.get();
                break;
            }
        if (!slot) return false;
        if (grow_alg >= 0) {
            if (any_busy()) return false;
            const int ga = grow_alg;
            grow_alg = -1;
            if (grow_keys(ga, ks[ga].cap + grow_need)) {
                // no memory for more keys: refuse the waiting keypair requests of that algorithm
                auto &g = groups[ga][PQCGPU_OP_KEYPAIR];
                while (!g.empty() && ks[ga].free_slots.empty()) {
                    finish(g.front(), PQCGPU_EBUDGET, 0);
                    g.pop_front();
                    pending--;
                }
                cv_done.notify_all();
            }
        }
        // oldest group head.  FrodoKEM batches are long (about a millisecond of serial sponges) and
        // its three operations queue separately, so they may use all slots but a quarter (at least
        // two), which stay for the light algorithms.
        const int heavy_max = std::max(1, max_inflight - std::max(2, max_inflight / 4));
        int alg = -1, op = -1;
        Clock::time_point oldest;
        for (int a = 0; a < PQCGPU_NUM_ALGS; a++)
            for (int o = 0; o < 3; o++) {
                auto &g = groups[a][o];
                if (g.empty() || (frodo_n(a) && heavy_running >= heavy_max)) continue;
                if (alg < 0 || g.front()->t0 < oldest) {
                    alg = a;
                    op = o;
                    oldest = g.front()->t0;
                }
            }
        if (alg < 0) return false;
        const int cap = frodo_n(alg) ? std::min(max_batch, 256) : max_batch;
        auto &grp = groups[alg][op];
        KeyStore &k = ks[alg];
        const size_t take_n = std::min<size_t>(grp.size(), (size_t)cap);
        if (op == PQCGPU_OP_KEYPAIR && k.free_slots.size() < take_n) {
            if (any_busy()) {  // grow once every in-flight batch is done
                grow_alg = alg;
                grow_need = (uint32_t)(take_n - k.free_slots.size());
                return false;
            }
            if (grow_keys(alg, k.cap + (uint32_t)(take_n - k.free_slots.size())) && k.free_slots.empty()) {
                finish(grp.front(), PQCGPU_EBUDGET, 0);
                grp.pop_front();
                pending--;
                cv_done.notify_all();
                return true;
            }
        }
        std::vector<Req *> ok;
        std::vector<uint32_t> idx;
        while (!grp.empty() && (int)ok.size() < cap) {
            Req *q = grp.front();
            uint32_t ksl = 0;
            if (op == PQCGPU_OP_KEYPAIR) {
                if (k.free_slots.empty()) break;
                ksl = k.free_slots.back();
                k.free_slots.pop_back();
                k.used[ksl] = 1;
            } else if (q->r.key || op == PQCGPU_OP_DEC) {
                if (!key_ok(q->r.key, alg, &ksl)) {
                    grp.pop_front();
                    pending--;
                    finish(q, PQCGPU_EINVAL, 0);
                    cv_done.notify_all();
                    continue;
                }
            }
            // an encapsulation batch is either all by handle or all by explicit pk
            if (op == PQCGPU_OP_ENC && !ok.empty() && ((q->r.key != 0) != (ok[0]->r.key != 0))) break;
            grp.pop_front();
            pending--;
            q->key_slot = ksl;
            idx.push_back(ksl);
            ok.push_back(q);
        }
        if (ok.empty()) return true;
        const int n = (int)ok.size();
        const bool by_handle = (op == PQCGPU_OP_DEC) || (op == PQCGPU_OP_ENC && ok[0]->r.key != 0);
        size_t sz[4];
        op_io_sizes(alg, op, sz);
        Slot &s = *slot;
        // staging layout: idx, host-packed inputs, gathered input, outputs, scratch
        size_t d = r256(4 * (size_t)n), in0 = 0, in1 = 0;
        if (op == PQCGPU_OP_KEYPAIR) {
            in0 = d; d += r256(sz[0] * n);
        } else if (op == PQCGPU_OP_ENC) {
            in1 = d; d += r256(sz[1] * n);            // coins
            if (!by_handle) { in0 = d; d += r256(sz[0] * n); }
        } else {
            in0 = d; d += r256(sz[0] * n);            // ct
        }
        const size_t h2d = d;
        if (op == PQCGPU_OP_ENC && by_handle) { in0 = d; d += r256(sz[0] * n); }   // pk gathered
        if (op == PQCGPU_OP_DEC) { in1 = d; d += r256(sz[1] * n); }                // sk gathered
        // FrodoKEM keeps pkh = SHAKE(pk) as the last ss-size bytes of its secret key
        const bool use_pkh = frodo_n(alg) && op == PQCGPU_OP_ENC && by_handle;
        const size_t pkhb = sz[3];  // the shared-secret size = the pkh size
        size_t pkh = 0;
        if (use_pkh) { pkh = d; d += r256(pkhb * (size_t)n); }
        const size_t out0 = d;
        d += r256(sz[2] * n);
        const size_t out1 = d;
        d += r256(sz[3] * n);
        const size_t hneed = d;
        const size_t d2h = (op == PQCGPU_OP_KEYPAIR) ? sz[2] * n : (op == PQCGPU_OP_ENC ? out1 + sz[3] * n - out0 : sz[2] * n);
        const size_t scr = d;
        d += r256(op_scratch_bytes(alg, op, 0) * n);
        if (d > s.dcap) {
            free_dev(s.dbuf, s.dcap);
            s.dbuf = nullptr;
            s.dcap = 0;
            size_t want = d + d / 2;
            if (alloc_dev(&s.dbuf, want) && alloc_dev(&s.dbuf, d)) {
                const bool others = any_busy();
                for (auto it = ok.rbegin(); it != ok.rend(); ++it) {
                    Req *q = *it;
                    if (op == PQCGPU_OP_KEYPAIR) {
                        k.used[q->key_slot] = 0;
                        k.free_slots.push_back(q->key_slot);
                    }
                    if (others) {  // wait for in-flight batches to free memory
                        grp.push_front(q);
                        pending++;
                    } else {
                        finish(q, PQCGPU_EBUDGET, 0);  // nothing will free memory: refuse
                    }
                }
                if (!others) cv_done.notify_all();
                return !others;
            }
            s.dcap = (s.dbuf && used >= want) ? want : d;
        }
        if (hneed > s.hcap) {
            if (s.hbuf) cudaFreeHost(s.hbuf);
            s.hbuf = nullptr;
            s.hcap = 0;
            if (cudaMallocHost(&s.hbuf, hneed + hneed / 2) != cudaSuccess) {
                cudaGetLastError();
                for (Req *q : ok) {
                    if (op == PQCGPU_OP_KEYPAIR) {
                        k.used[q->key_slot] = 0;
                        k.free_slots.push_back(q->key_slot);
                    }
                    finish(q, PQCGPU_ENOMEM, 0);
                }
                cv_done.notify_all();
                return true;
            }
            s.hcap = hneed + hneed / 2;
        }
        s.alg = alg;
        s.op = op;
        s.n = n;
        s.by_handle = by_handle;
        s.reqs.swap(ok);
        s.idx.swap(idx);
        s.kpk = k.dpk;
        s.ksk = k.dsk;
        s.pkb = k.pkb;
        s.skb = k.skb;
        s.off_in0 = in0;
        s.off_in1 = in1;
        s.off_out0 = out0;
        s.off_out1 = out1;
        s.off_scr = scr;
        s.use_pkh = use_pkh;
        s.off_pkh = pkh;
        s.h2d_bytes = h2d;
        s.d2h_bytes = d2h;
        s.stream = frodo_n(alg) ? s.lo : s.hi;
        s.busy = true;
        s.has_job = true;
        if (frodo_n(alg)) heavy_running++;
        s.cv.notify_one();
        return true;
    }

    // The worker's half of a batch (no mutex): pack, copy up, run, copy down, wait, unpack.
    int execute(Slot &s) {
        size_t sz[4];
        op_io_sizes(s.alg, s.op, sz);
        const int n = s.n, op = s.op, alg = s.alg;
        uint8_t *H = s.hbuf, *D = s.dbuf;
        memcpy(H, s.idx.data(), 4 * (size_t)n);
        size_t missing = 0;  // coins drawn from the library DRBG in one call
        for (int i = 0; i < n; i++) {
            const pqcgpu_request &r = s.reqs[i]->r;
            if (op == PQCGPU_OP_KEYPAIR) {
                if (r.in) memcpy(H + s.off_in0 + (size_t)i * sz[0], r.in, sz[0]);
                else missing++;
            } else if (op == PQCGPU_OP_ENC) {
                if (!s.by_handle) memcpy(H + s.off_in0 + (size_t)i * sz[0], r.pk, sz[0]);
                if (r.in) memcpy(H + s.off_in1 + (size_t)i * sz[1], r.in, sz[1]);
                else missing++;
            } else {
                memcpy(H + s.off_in0 + (size_t)i * sz[0], r.in, sz[0]);
            }
        }
        if (missing) {
            const size_t off = op == PQCGPU_OP_KEYPAIR ? s.off_in0 : s.off_in1, b = sz[op == PQCGPU_OP_KEYPAIR ? 0 : 1];
            for (int i = 0; i < n; i++)
                if (!s.reqs[i]->r.in && pqcgpu_randombytes(H + off + (size_t)i * b, b) != PQCGPU_OK)
                    return PQCGPU_EUNSUPPORTED;  // no entropy: fail the batch rather than use weak coins
        }
        cudaStream_t st = s.stream;
        const uint32_t *didx = (const uint32_t *)D;
        cudaMemcpyAsync(D, H, s.h2d_bytes, cudaMemcpyHostToDevice, st);
        int rc = PQCGPU_OK;
        if (op == PQCGPU_OP_KEYPAIR) {
            rc = op_dev(alg, op, n, D + s.off_in0, nullptr, D + s.off_out0, D + s.off_out1, D + s.off_scr, OP_NH_BATCHED,
                        st);
            launch_rows(false, s.kpk, D + s.off_out0, didx, n, s.pkb, st);
            launch_rows(false, s.ksk, D + s.off_out1, didx, n, s.skb, st);
        } else if (op == PQCGPU_OP_ENC) {
            if (s.by_handle) launch_rows(true, D + s.off_in0, s.kpk, didx, n, s.pkb, st);
            if (s.use_pkh) {
                size_t io[4];
                op_io_sizes(alg, op, io);
                const int words = (int)(io[3] / 8);  // pkh = ss size
                PQC_LAUNCH(st, "rows_tail_gather", 0, 0,
                           rows_tail_gather<<<(n * words + 255) / 256, 256, 0, st>>>(
                               (uint2 *)(D + s.off_pkh), s.ksk, didx, n, s.skb, s.skb - 8 * words, words));
                rc = frodo_enc_dev(frodo_n(alg), n, D + s.off_out0, D + s.off_out1, D + s.off_in0, D + s.off_in1,
                                   D + s.off_scr, st, D + s.off_pkh);
            } else {
                rc = op_dev(alg, op, n, D + s.off_in0, D + s.off_in1, D + s.off_out0, D + s.off_out1, D + s.off_scr,
                            OP_NH_BATCHED, st);
            }
        } else {
            launch_rows(true, D + s.off_in1, s.ksk, didx, n, s.skb, st);
            rc = op_dev(alg, op, n, D + s.off_in0, D + s.off_in1, D + s.off_out0, nullptr, D + s.off_scr, OP_NH_BATCHED,
                        st);
        }
        cudaMemcpyAsync(H + s.off_out0, D + s.off_out0, s.d2h_bytes, cudaMemcpyDeviceToHost, st);
        cudaEventRecord(s.done, st);
        // poll, yielding the core between polls: up to 16 workers share the host's cores
        cudaError_t q;
        while ((q = cudaEventQuery(s.done)) == cudaErrorNotReady) std::this_thread::yield();
        if (q != cudaSuccess || cudaGetLastError() != cudaSuccess) rc = PQCGPU_ECUDA;
        if (rc) return rc;
        for (int i = 0; i < n; i++) {
            Req *q = s.reqs[i];
            if (op == PQCGPU_OP_KEYPAIR) {
                if (q->r.out0) memcpy(q->r.out0, H + s.off_out0 + (size_t)i * sz[2], sz[2]);
                if (q->r.key_out) *q->r.key_out = ((uint64_t)alg << 48) | (uint64_t)(q->key_slot + 1);
            } else if (op == PQCGPU_OP_ENC) {
                memcpy(q->r.out0, H + s.off_out0 + (size_t)i * sz[2], sz[2]);
                memcpy(q->r.out1, H + s.off_out1 + (size_t)i * sz[3], sz[3]);
            } else {
                memcpy(q->r.out0, H + s.off_out0 + (size_t)i * sz[2], sz[2]);
            }
        }
        return PQCGPU_OK;
    }

    // Record the batch's outcome and free the slot (mutex held).
    void complete(Slot &s, int rc) {
        const auto now = Clock::now();
        for (Req *q : s.reqs) {
            if (rc && s.op == PQCGPU_OP_KEYPAIR) {
                ks[s.alg].used[q->key_slot] = 0;
                ks[s.alg].free_slots.push_back(q->key_slot);
            }
            finish(q, rc, std::chrono::duration<double, std::milli>(now - q->t0).count());
        }
        if (rc && error.empty()) error = "a batch failed on the device";
        s.reqs.clear();
        s.busy = false;
        if (frodo_n(s.alg)) heavy_running--;
        batches++;
        events++;
        cv_work.notify_one();
        cv_done.notify_all();
    }

    void work(Slot *s) {
        cudaSetDevice(device);
        std::unique_lock<std::mutex> lk(mu);
        while (true) {
            s->cv.wait(lk, [&] { return s->has_job || stop_workers; });
            if (!s->has_job) break;
            s->has_job = false;
            lk.unlock();
            const int rc = execute(*s);
            lk.lock();
            complete(*s, rc);
        }
    }

    void run() {
        cudaSetDevice(device);
        std::unique_lock<std::mutex> lk(mu);
        while (true) {
            const uint64_t seen = events;
            while (assign_one()) {
            }
            if (stop && !pending && !any_busy()) break;
            cv_work.wait(lk, [&] { return events != seen || (stop && !pending && !any_busy()); });
        }
    }
};

extern "C" int pqcgpu_server_create(pqcgpu_server **out, int device, size_t budget, int max_inflight, int max_batch) {
    if (!out) return set_error(PQCGPU_EINVAL, "out is NULL");
    *out = nullptr;
    if (cudaSetDevice(device) != cudaSuccess) {
        cudaGetLastError();
        return set_error(PQCGPU_ECUDA, "no such CUDA device");
    }
    int rc = device_ready(device);
    if (rc) return rc;
    auto *s = new pqcgpu_server();
    s->device = device;
    s->budget = budget ? budget : ((size_t)16 << 30);
    s->max_inflight = max_inflight > 0 ? std::min(max_inflight, 16) : 4;
    s->max_batch = max_batch > 0 ? max_batch : 4096;
    // light batches (Kyber, NewHope: tens of microseconds of GPU time) get the high-priority
    // streams so that their CTAs are scheduled ahead of waiting FrodoKEM CTAs
    int prio_lo = 0, prio_hi = 0;
    cudaDeviceGetStreamPriorityRange(&prio_lo, &prio_hi);
    for (int i = 0; i < s->max_inflight; i++) {
        s->slots.emplace_back(new Slot());
        Slot *sl = s->slots.back().get();
        cudaStreamCreateWithPriority(&sl->hi, cudaStreamNonBlocking, prio_hi);
        cudaStreamCreateWithPriority(&sl->lo, cudaStreamNonBlocking, prio_lo);
        sl->stream = sl->hi;
        cudaEventCreateWithFlags(&sl->done, cudaEventDisableTiming);
    }
    for (int a = 0; a < PQCGPU_NUM_ALGS; a++) {
        size_t sz[4];
        op_io_sizes(a, PQCGPU_OP_KEYPAIR, sz);
        s->ks[a].pkb = sz[2];
        s->ks[a].skb = sz[3];
    }
    for (auto &sl : s->slots) {
        Slot *p = sl.get();
        p->th = std::thread([s, p] { s->work(p); });
    }
    s->th = std::thread([s] { s->run(); });
    *out = s;
    return PQCGPU_OK;
}

extern "C" int pqcgpu_server_submit(pqcgpu_server *s, const pqcgpu_request *req, uint64_t *ticket) {
    if (!s || !req) return set_error(PQCGPU_EINVAL, "null server or request");
    size_t sz[4];
    if (req->alg < 0 || req->alg >= PQCGPU_NUM_ALGS || req->op < 0 || req->op > 2)
        return set_error(PQCGPU_EINVAL, "bad algorithm or operation");
    op_io_sizes(req->alg, req->op, sz);
    if (req->op == PQCGPU_OP_ENC && !req->key && !req->pk) return set_error(PQCGPU_EINVAL, "encapsulation needs a key or pk");
    if ((req->op == PQCGPU_OP_ENC && (!req->out0 || !req->out1)) || (req->op == PQCGPU_OP_DEC && (!req->in || !req->out0)))
        return set_error(PQCGPU_EINVAL, "missing buffer");
    auto q = std::make_unique<Req>();
    q->r = *req;
    q->t0 = Clock::now();
    Req *raw = q.get();
    {
        std::lock_guard<std::mutex> lk(s->mu);
        if (s->stop) return set_error(PQCGPU_EINVAL, "server is shutting down");
        raw->ticket = s->next_ticket++;
        s->reqs[raw->ticket] = std::move(q);
        s->groups[req->alg][req->op].push_back(raw);
        s->pending++;
        s->events++;
    }
    s->cv_work.notify_one();
    if (ticket) *ticket = raw->ticket;
    return PQCGPU_OK;
}

extern "C" int pqcgpu_server_wait(pqcgpu_server *s, uint64_t ticket, int timeout_ms) {
    if (!s) return PQCGPU_EINVAL;
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->reqs.find(ticket);
    if (it == s->reqs.end()) return set_error(PQCGPU_EINVAL, "unknown ticket");
    Req *q = it->second.get();
    auto pred = [&] { return q->status != 1; };
    if (timeout_ms < 0) s->cv_done.wait(lk, pred);
    else if (!s->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), pred)) return PQCGPU_ETIMEOUT;
    const int st = q->status;
    s->reqs.erase(it);
    return st;
}

extern "C" int pqcgpu_server_drain(pqcgpu_server *s) {
    if (!s) return PQCGPU_EINVAL;
    std::unique_lock<std::mutex> lk(s->mu);
    s->cv_done.wait(lk, [&] { return !s->pending && !s->any_busy(); });
    return PQCGPU_OK;
}

extern "C" int pqcgpu_server_key_release(pqcgpu_server *s, uint64_t key) {
    if (!s) return PQCGPU_EINVAL;
    std::lock_guard<std::mutex> lk(s->mu);
    const int alg = (int)(key >> 48);
    uint32_t slot;
    if (alg < 0 || alg >= PQCGPU_NUM_ALGS || !s->key_ok(key, alg, &slot)) return set_error(PQCGPU_EINVAL, "unknown key");
    s->ks[alg].used[slot] = 0;
    s->ks[alg].free_slots.push_back(slot);
    return PQCGPU_OK;
}

namespace {
void fill_latency(std::vector<double> v, pqcgpu_server_stats *out) {
    if (v.empty()) return;
    std::sort(v.begin(), v.end());
    out->p50_ms = v[v.size() / 2];
    out->p99_ms = v[std::min(v.size() - 1, (size_t)(0.99 * v.size()))];
    out->max_ms = v.back();
    double sum = 0;
    for (double x : v) sum += x;
    out->mean_ms = sum / v.size();
}
}  // namespace

extern "C" int pqcgpu_server_get_stats(pqcgpu_server *s, pqcgpu_server_stats *out, int reset) {
    if (!s || !out) return PQCGPU_EINVAL;
    std::lock_guard<std::mutex> lk(s->mu);
    memset(out, 0, sizeof *out);
    out->completed = s->completed;
    out->batches = s->batches;
    out->hbm_used = s->used;
    for (auto &k : s->ks)
        for (auto u : k.used) out->keys_resident += u;
    fill_latency(s->lat_ms, out);
    if (reset) {
        s->lat_ms.clear();
        for (auto &a : s->lat_grp)
            for (auto &g : a) g.clear();
        s->completed = 0;
        s->batches = 0;
    }
    return PQCGPU_OK;
}

extern "C" int pqcgpu_server_get_group_stats(pqcgpu_server *s, int alg, int op, pqcgpu_server_stats *out) {
    if (!s || !out || alg < 0 || alg >= PQCGPU_NUM_ALGS || op < 0 || op > 2) return PQCGPU_EINVAL;
    std::lock_guard<std::mutex> lk(s->mu);
    memset(out, 0, sizeof *out);
    out->completed = s->lat_grp[alg][op].size();
    out->hbm_used = s->used;
    fill_latency(s->lat_grp[alg][op], out);
    return PQCGPU_OK;
}

extern "C" int pqcgpu_server_destroy(pqcgpu_server *s) {
    if (!s) return PQCGPU_EINVAL;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
    }
    s->cv_work.notify_all();
    if (s->th.joinable()) s->th.join();  // returns once nothing is pending or in flight
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop_workers = true;
    }
    for (auto &sl : s->slots) {
        sl->cv.notify_all();
        if (sl->th.joinable()) sl->th.join();
    }
    cudaSetDevice(s->device);
    cudaDeviceSynchronize();
    for (auto &sl : s->slots) {
        s->free_dev(sl->dbuf, sl->dcap);
        if (sl->hbuf) cudaFreeHost(sl->hbuf);
        cudaStreamDestroy(sl->hi);
        cudaStreamDestroy(sl->lo);
        cudaEventDestroy(sl->done);
    }
    for (auto &k : s->ks) {
        s->free_dev(k.dpk, (size_t)k.cap * k.pkb);
        s->free_dev(k.dsk, (size_t)k.cap * k.skb);
    }
    delete s;
    return PQCGPU_OK;
}

// ---------------------------------------------------------------------------------------------
// Open-loop Poisson load: keys and ciphertexts are prepared first (resident keys), then requests
// are submitted at exponential inter-arrival times for `seconds`, then the server is drained.
// ---------------------------------------------------------------------------------------------
extern "C" int pqcgpu_server_run_poisson(pqcgpu_server *s, const pqcgpu_mix_entry *mix, size_t nmix, double rate,
                                         double seconds, uint64_t seed, pqcgpu_load_report *out) {
    if (!s || !mix || !nmix || rate <= 0 || seconds <= 0 || !out) return set_error(PQCGPU_EINVAL, "bad load arguments");
    std::mt19937_64 rng(seed);
    // per-algorithm pools: resident keys and matching ciphertexts
    constexpr int POOL = 64;
    struct Pool {
        std::vector<uint64_t> keys;
        std::vector<std::vector<uint8_t>> cts;
    } pools[PQCGPU_NUM_ALGS];
    for (size_t m = 0; m < nmix; m++) {
        const int a = mix[m].alg;
        if (a < 0 || a >= PQCGPU_NUM_ALGS || mix[m].op < 0 || mix[m].op > 2) return set_error(PQCGPU_EINVAL, "bad mix entry");
        if (!pools[a].keys.empty()) continue;
        size_t kz[4], ez[4];
        op_io_sizes(a, PQCGPU_OP_KEYPAIR, kz);
        op_io_sizes(a, PQCGPU_OP_ENC, ez);
        pools[a].keys.resize(POOL);
        std::vector<uint64_t> tk(POOL);
        for (int i = 0; i < POOL; i++) {
            pqcgpu_request r{};
            r.alg = a;
            r.op = PQCGPU_OP_KEYPAIR;
            r.key_out = &pools[a].keys[i];
            int rc = pqcgpu_server_submit(s, &r, &tk[i]);
            if (rc) return rc;
        }
        for (int i = 0; i < POOL; i++)
            if (pqcgpu_server_wait(s, tk[i], -1) != 0) return set_error(PQCGPU_ECUDA, "pool keypair failed");
        pools[a].cts.assign(POOL, std::vector<uint8_t>(ez[2]));
        std::vector<uint8_t> ss(ez[3]);
        for (int i = 0; i < POOL; i++) {
            pqcgpu_request r{};
            r.alg = a;
            r.op = PQCGPU_OP_ENC;
            r.key = pools[a].keys[i];
            r.out0 = pools[a].cts[i].data();
            r.out1 = ss.data();
            int rc = pqcgpu_server_submit(s, &r, &tk[i]);
            if (rc) return rc;
            if (pqcgpu_server_wait(s, tk[i], -1) != 0) return set_error(PQCGPU_ECUDA, "pool encaps failed");
        }
    }
    pqcgpu_server_drain(s);
    {
        pqcgpu_server_stats st;
        pqcgpu_server_get_stats(s, &st, 1);
    }
    double wsum = 0;
    for (size_t m = 0; m < nmix; m++) wsum += mix[m].weight;
    std::exponential_distribution<double> gap(rate);
    std::uniform_real_distribution<double> uni(0.0, wsum);
    // output sinks (results are discarded; one buffer per alg/op, largest sizes)
    static thread_local std::vector<uint8_t> sink0(1 << 16), sink1(1 << 16);
    std::deque<uint64_t> key_outs;  // handles of the keypairs the run made (a deque: stable addresses)
    const auto t_start = Clock::now();
    double t = 0;
    uint64_t submitted = 0;
    while (t < seconds) {
        t += gap(rng);
        const auto due = t_start + std::chrono::duration_cast<Clock::duration>(std::chrono::duration<double>(t));
        while (Clock::now() < due) {
            const auto left = due - Clock::now();
            if (left > std::chrono::microseconds(200)) std::this_thread::sleep_for(left - std::chrono::microseconds(100));
        }
        double u = uni(rng);
        size_t m = 0;
        while (m + 1 < nmix && u >= mix[m].weight) {
            u -= mix[m].weight;
            m++;
        }
        const int a = mix[m].alg, op = mix[m].op;
        const int i = (int)(rng() % POOL);
        pqcgpu_request r{};
        r.alg = a;
        r.op = op;
        if (op == PQCGPU_OP_KEYPAIR) {
            key_outs.push_back(0);
            r.key_out = &key_outs.back();
        } else if (op == PQCGPU_OP_ENC) {
            r.key = pools[a].keys[i];
            r.out0 = sink0.data();
            r.out1 = sink1.data();
        } else {
            r.key = pools[a].keys[i];
            r.in = pools[a].cts[i].data();
            r.out0 = sink0.data();
        }
        uint64_t tk;
        if (pqcgpu_server_submit(s, &r, &tk) == 0) submitted++;
    }
    const auto t_sub = Clock::now();
    pqcgpu_server_drain(s);
    const auto t_end = Clock::now();
    pqcgpu_server_stats st;
    pqcgpu_server_get_stats(s, &st, 0);  // samples stay readable (per group too) until the next reset
    {
        // forget the tickets of the load run and release the keys it generated
        std::lock_guard<std::mutex> lk(s->mu);
        s->reqs.clear();
    }
    for (uint64_t k : key_outs)
        if (k) pqcgpu_server_key_release(s, k);
    out->offered_per_s = rate;
    out->seconds = std::chrono::duration<double>(t_end - t_start).count();
    out->submit_seconds = std::chrono::duration<double>(t_sub - t_start).count();
    out->submitted = submitted;
    out->completed = st.completed;
    out->batches = st.batches;
    out->achieved_per_s = st.completed / out->seconds;
    out->p50_ms = st.p50_ms;
    out->p99_ms = st.p99_ms;
    out->mean_ms = st.mean_ms;
    out->max_ms = st.max_ms;
    return PQCGPU_OK;
}
