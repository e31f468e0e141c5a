// Roofline probes and the launch profiler.
//
// Probes: the integer (LOP3) pipe peak and the register-resident Keccak-f[1600] permutation rate of
// this GPU, measured with CUDA events.  bench.py reports kernel throughput against them, since the
// KEM path is bound by the integer pipe, a figure no vendor table or copy/GEMM benchmark gives.
//
// Profiler: when enabled, every kernel launch of the library is bracketed by CUDA events recorded
// on the launching stream; per-kernel launch counts and summed durations can be read back as JSON.
#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>

#include <mutex>
#include <string>
#include <vector>

#include "keccak.cuh"
#include "pqcgpu_internal.h"

namespace pqc {

// 8 independent LOP3 chains per thread; the immediate mixes all three inputs so nothing folds.
__global__ void probe_lop3_kernel(uint32_t *out, int iters) {
    uint32_t a[8];
#pragma unroll
    for (int i = 0; i < 8; i++) a[i] = threadIdx.x * 0x9E3779B9u + i * 0x85EBCA6Bu + blockIdx.x;
    const uint32_t b = blockIdx.x * 0x27D4EB2Fu, c = threadIdx.x ^ 0x165667B1u;
    for (int it = 0; it < iters; it++) {
#pragma unroll
        for (int r = 0; r < 16; r++) {
#pragma unroll
            for (int i = 0; i < 8; i++) asm volatile("lop3.b32 %0, %0, %1, %2, 0x96;" : "+r"(a[i]) : "r"(b), "r"(c));
        }
    }
    uint32_t x = 0;
#pragma unroll
    for (int i = 0; i < 8; i++) x ^= a[i];
    if (x == 0x12345678u) out[0] = x;  // practically never; keeps the chains live
}

__global__ void probe_keccak_kernel(uint32_t *out, int iters) {
    uint2 A[25];
#pragma unroll
    for (int i = 0; i < 25; i++) A[i] = make_uint2(threadIdx.x + i, blockIdx.x * 7 + i);
    for (int it = 0; it < iters; it++) keccak_f1600(A);
    if (A[0].x == 0x12345678u) out[0] = A[0].y;
}

static int time_kernel(void (*launch)(uint32_t *, int, cudaStream_t), uint32_t *buf, int iters, cudaStream_t st,
                       float *ms) {
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    launch(buf, iters / 4 + 1, st);  // warm-up
    cudaEventRecord(e0, st);
    launch(buf, iters, st);
    cudaEventRecord(e1, st);
    cudaError_t e = cudaEventSynchronize(e1);
    cudaEventElapsedTime(ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return e == cudaSuccess ? PQCGPU_OK : PQCGPU_ECUDA;
}

static int g_probe_blocks = 0;
static void launch_lop3(uint32_t *b, int it, cudaStream_t st) { probe_lop3_kernel<<<g_probe_blocks, 256, 0, st>>>(b, it); }
static void launch_keccak(uint32_t *b, int it, cudaStream_t st) {
    probe_keccak_kernel<<<g_probe_blocks, 128, 0, st>>>(b, it);
}

int probe_peaks(int device, double *int_ops, double *keccak_perms) {
    if (cudaSetDevice(device) != cudaSuccess) return PQCGPU_ECUDA;
    uint2 rc[24];
    keccak_rc_host(rc);
    if (cudaMemcpyToSymbol(c_keccak_rc, rc, sizeof rc) != cudaSuccess) return PQCGPU_ECUDA;
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    g_probe_blocks = sms * 8;
    uint32_t *buf = nullptr;
    if (cudaMalloc(&buf, 64) != cudaSuccess) return PQCGPU_ENOMEM;
    cudaStream_t st;
    cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
    float ms = 0;
    int rc1 = PQCGPU_OK;
    if (int_ops) {
        const int iters = 4000;
        rc1 = time_kernel(launch_lop3, buf, iters, st, &ms);
        *int_ops = (double)g_probe_blocks * 256 * iters * 16 * 8 / (ms * 1e-3);
    }
    if (!rc1 && keccak_perms) {
        const int iters = 400;
        rc1 = time_kernel(launch_keccak, buf, iters, st, &ms);
        *keccak_perms = (double)g_probe_blocks * 128 * iters / (ms * 1e-3);
    }
    cudaStreamDestroy(st);
    cudaFree(buf);
    return rc1;
}

// ---- launch profiler ----
namespace {
struct Rec {
    std::string name;
    cudaStream_t st;
    cudaEvent_t e0, e1;
};
std::mutex g_prof_mu;
std::vector<Rec> g_recs;
bool g_prof_on = false;
}  // namespace

static thread_local bool g_capturing = false;
void set_capturing(bool on) { g_capturing = on; }
bool capturing() { return g_capturing; }
bool prof_enabled() { return g_prof_on && !g_capturing; }
void *prof_begin(cudaStream_t st, const char *name, int k, int v) {
    Rec *r = new Rec();
    char buf[96];
    if (k < 0)  // copies and other non-kernel records carry no template arguments
        snprintf(buf, sizeof buf, "%s", name);
    else
        snprintf(buf, sizeof buf, "%s<%d,%d>", name, k, v);
    r->name = buf;
    r->st = st;
    cudaEventCreate(&r->e0);
    cudaEventCreate(&r->e1);
    cudaEventRecord(r->e0, st);
    return r;
}
void prof_end(cudaStream_t st, void *tok) {
    Rec *r = (Rec *)tok;
    cudaEventRecord(r->e1, st);
    std::lock_guard<std::mutex> lk(g_prof_mu);
    g_recs.push_back(*r);
    delete r;
}
void prof_enable(bool on) {
    std::lock_guard<std::mutex> lk(g_prof_mu);
    g_prof_on = on;
}
// Aggregates and clears the records: {"name": [launches, total_ms], ...}
std::string prof_read() {
    std::lock_guard<std::mutex> lk(g_prof_mu);
    std::vector<std::pair<std::string, std::pair<int, double>>> agg;
    for (auto &r : g_recs) {
        float ms = 0;
        cudaEventSynchronize(r.e1);
        cudaEventElapsedTime(&ms, r.e0, r.e1);
        cudaEventDestroy(r.e0);
        cudaEventDestroy(r.e1);
        bool found = false;
        for (auto &a : agg)
            if (a.first == r.name) {
                a.second.first++;
                a.second.second += ms;
                found = true;
            }
        if (!found) agg.push_back({r.name, {1, (double)ms}});
    }
    g_recs.clear();
    std::string s = "{";
    for (size_t i = 0; i < agg.size(); i++) {
        char buf[200];
        snprintf(buf, sizeof buf, "%s\"%s\": [%d, %.6f]", i ? ", " : "", agg[i].first.c_str(), agg[i].second.first,
                 agg[i].second.second);
        s += buf;
    }
    return s + "}";
}


// The records as a timeline in the Chrome trace-event format: one complete event ("ph": "X") per
// record, times in microseconds from the earliest record, one "tid" per stream in order of first
// use.  Returns false (records kept) when `cap` is too small; *need = the bytes with the NUL.
bool prof_trace(char *buf, size_t cap, size_t *need) {
    std::lock_guard<std::mutex> lk(g_prof_mu);
    std::vector<double> t0(g_recs.size()), t1(g_recs.size());
    std::vector<cudaStream_t> streams;
    double lo = 0;
    for (size_t i = 0; i < g_recs.size(); i++) {
        float a = 0, b = 0;
        cudaEventSynchronize(g_recs[i].e1);
        cudaEventElapsedTime(&a, g_recs[0].e0, g_recs[i].e0);
        cudaEventElapsedTime(&b, g_recs[0].e0, g_recs[i].e1);
        t0[i] = a;
        t1[i] = b;
        lo = i == 0 || a < lo ? a : lo;
    }
    std::string s = "{\"traceEvents\": [";
    for (size_t i = 0; i < g_recs.size(); i++) {
        size_t tid = 0;
        while (tid < streams.size() && streams[tid] != g_recs[i].st) tid++;
        if (tid == streams.size()) streams.push_back(g_recs[i].st);
        char b[256];
        snprintf(b, sizeof b, "%s{\"name\": \"%s\", \"ph\": \"X\", \"pid\": 0, \"tid\": %zu, \"ts\": %.3f, \"dur\": %.3f}",
                 i ? ", " : "", g_recs[i].name.c_str(), tid, 1e3 * (t0[i] - lo), 1e3 * (t1[i] - t0[i]));
        s += b;
    }
    s += "]}";
    *need = s.size() + 1;
    if (!buf || cap < s.size() + 1) return false;
    memcpy(buf, s.c_str(), s.size() + 1);
    for (auto &r : g_recs) {
        cudaEventDestroy(r.e0);
        cudaEventDestroy(r.e1);
    }
    g_recs.clear();
    return true;
}

}  // namespace pqc
