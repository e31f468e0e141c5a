// FrodoKEM shared-key product on the tensor cores (tcgen05, sm_103a).
//
// For n encapsulations to one public key the products B'_x = S'_x A (frodo_macrify_reference.cu:
// 102-159, matMulKernelSA) form one matrix product: the 8-row blocks S'_x stacked into an 8n x N
// matrix times A (N x N), all mod 2^16.  The tensor cores of this GPU take no 8-bit integer MMA
// (ptxas for sm_103a refuses tcgen05.mma kind::i8), so the product runs exactly in fp16 with fp32
// accumulation:
//   A = 1024 A_hi + A_lo with A_lo = A & 1023 and A_hi = A >> 10, both exact in fp16 (< 2048);
//   S' entries are small signed integers (|s| <= 12 for every FrodoKEM parameter set), exact;
//   every partial sum of S' A_lo is below 1344 * 12 * 1023 < 2^24 and of S' A_hi below
//   1344 * 12 * 63, so the fp32 accumulators hold exact integers;
//   G = 1024 round(D_hi) + round(D_lo) (mod 2^32) equals S' A mod 2^16 in its low half.
// The result goes to each instance's u32 accumulator in scratch, which fr_sa_final turns into
// B' + E', V, C and the ciphertext.
//
// Kernel layout: CTA = 128 rows of the stacked S' (16 instances) x 128 columns of A, 4 warps, K in
// chunks of 64 through two shared-memory stages, so that chunk c + 1 is fetched while the tensor
// cores work on chunk c.  Every operand tile is 16 KB, stored pre-tiled in global memory in the
// no-swizzle K-major core-matrix layout of a tcgen05 operand (8 rows x 16 bytes per core matrix;
// LBO = 128 bytes between core matrices along K, SBO = 1024 bytes between 8-row groups):
//   * A's two fp16 planes by fr_gen_a (fr_tc_plane_index), once per batch;
//   * S' in fp16 by fr_s16_tiles (fr_tc_s_index) from the instances' u16 copies, a tile per CTA
//     with coalesced loads and stores, once (each S' tile feeds all the CTAs of its row);
// so one thread moves a chunk's three tiles with three bulk copies (cp.async.bulk, completion
// counted in bytes on the stage's mbarrier), issues the tcgen05.mma kind::f16 instructions
// (M = 128, N = 128, K = 16 each) into two fp32 accumulators in tensor memory, and commits them to
// the stage's second mbarrier, which says when the stage may be refilled.
// The epilogue reads the accumulators with tcgen05.ld (warp w: lanes 32w..32w+31 = rows).
// Every wait is bounded: a wait that runs out sets an error word (extra buffer) and the CTA frees
// its tensor memory and returns.
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "pqcgpu_internal.h"

namespace pqc {
namespace frodo_tc {

constexpr int NB = 8;
constexpr int TC_M = 128, TC_N = 128, TC_KC = 64, TC_THREADS = 128;
constexpr int TC_TMEM_COLS = 2 * TC_N;  // two fp32 accumulators
constexpr uint32_t LBO = 128, SBO = (TC_KC / 8) * 128;
constexpr int OP_BYTES = TC_M * TC_KC * 2;  // one 128 x 64 fp16 operand tile
// Operand stages (three 16 KB tiles each).  Dynamic shared memory per CTA: two stages, 96 KB, so
// that at most two CTAs share an SM, whose 512 tensor-memory columns then hold both CTAs' 256.
constexpr int NSTAGE = 2;
constexpr int TC_SMEM = NSTAGE * 3 * (TC_M * TC_KC * 2);
constexpr int WAIT_LIMIT = 1 << 22;

// Scratch layout per instance (frodo.cu FP<N>): S'^T (N x 8 u16) first, the u32 accumulator at GACC_OFF.
__host__ __device__ constexpr size_t gacc_off(int N) { return (size_t)(2 * N * NB + NB * NB) * 2 + 128; }
__host__ __device__ constexpr size_t scratch_bytes(int N) { return gacc_off(N) + (size_t)NB * N * 4; }

__device__ __forceinline__ uint32_t smem_addr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

// Shared-memory matrix descriptor, no swizzle (sm_100-family descriptor, version field 1).
__device__ __forceinline__ uint64_t sdesc(uint32_t saddr) {
    uint64_t d = (uint64_t)((saddr >> 4) & 0x3FFF);
    d |= (uint64_t)((LBO >> 4) & 0x3FFF) << 16;
    d |= (uint64_t)((SBO >> 4) & 0x3FFF) << 32;
    d |= (uint64_t)1 << 46;
    return d;
}
// Instruction descriptor of kind::f16: D f32 (bits 4-5 = 1), A and B f16 (0), both K-major, N >> 3
// at bits 17-22, M >> 4 at bits 24-28.
constexpr uint32_t IDESC = (1u << 4) | ((uint32_t)(TC_N >> 3) << 17) | ((uint32_t)(TC_M >> 4) << 24);

__device__ __forceinline__ void mma_f16(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t accumulate) {
    asm volatile(
        "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
        "l"(a), "l"(b), "r"(IDESC), "r"(accumulate));
}
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity) {
    for (int i = 0; i < WAIT_LIMIT; i++) {
        uint32_t done;
        asm volatile(
            "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done)
            : "r"(bar), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}

__device__ __forceinline__ void mbar_init(uint32_t bar) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar) : "memory");
}
// The stage's three operand tiles of chunk c: one bulk copy each, completion counted in bytes on `bar`.
__device__ __forceinline__ void bulk_tile(uint32_t dst, const uint16_t *src, uint32_t bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
                 "l"(src), "r"(OP_BYTES), "r"(bar)
                 : "memory");
}
__device__ __forceinline__ void issue_tiles(uint32_t bar, uint32_t dst, const uint16_t *s_src, const uint16_t *lo_src,
                                            const uint16_t *hi_src) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(3 * OP_BYTES) : "memory");
    bulk_tile(dst, s_src, bar);
    bulk_tile(dst + OP_BYTES, lo_src, bar);
    bulk_tile(dst + 2 * OP_BYTES, hi_src, bar);
}

// S'^T (scratch, u16 two's complement, N x 8 per instance) -> the fp16 operand tiles of S'
// (fr_tc_s_index).  CTA = one 16 KB tile (16 instances x 64 k): thread = (instance g, k block kb)
// loads the instance's 8 S'^T rows of its k block (128 contiguous bytes), converts and transposes
// them in registers, and stores 8 rows of 16 bytes; entries beyond n or N are written as zero.
template <int N>
__global__ void __launch_bounds__(128) fr_s16_tiles(int n, const uint8_t *scratch, uint16_t *s16) {
    constexpr int KCH = fr_tc_kchunks(N);
    const int mt = blockIdx.x / KCH, c = blockIdx.x % KCH, tid = threadIdx.x, g = tid >> 3, kb = tid & 7;
    const int x = mt * 16 + g, k = c * TC_KC + 8 * kb;
    const uint4 *sp = reinterpret_cast<const uint4 *>(scratch + (size_t)x * scratch_bytes(N));
    uint4 v[8];  // v[kk] = S'^T row k + kk (8 u16: i = 0..7)
#pragma unroll
    for (int kk = 0; kk < 8; kk++) v[kk] = (x < n && k + kk < N) ? sp[k + kk] : make_uint4(0, 0, 0, 0);
    uint4 *out = reinterpret_cast<uint4 *>(s16 + fr_tc_s_index(N, mt * 16 + g, 0, k));  // row i at +8 i
#pragma unroll
    for (int i = 0; i < 8; i++) {
        uint32_t h[8];
#pragma unroll
        for (int kk = 0; kk < 8; kk++) {
            const uint32_t w = (i < 2 ? v[kk].x : i < 4 ? v[kk].y : i < 6 ? v[kk].z : v[kk].w) >> (16 * (i & 1));
            h[kk] = __half_as_ushort(__short2half_rn((int16_t)(w & 0xffff)));
        }
        out[i] = make_uint4(h[0] | (h[1] << 16), h[2] | (h[3] << 16), h[4] | (h[5] << 16), h[6] | (h[7] << 16));
    }
}

// planes: A's two fp16 planes (fr_tc_plane_index); s16: S' in fp16 (fr_tc_s_index); error: a word
// set on a wait that ran out.
template <int N>
__global__ void __launch_bounds__(TC_THREADS, 1) fr_sa_shared_tc(int n, const uint16_t *planes, const uint16_t *s16,
                                                                 uint8_t *scratch, unsigned *error) {
    constexpr int NT = fr_tc_ntiles(N), KCH = fr_tc_kchunks(N);
    static_assert(FR_TC_N == TC_N && FR_TC_KC == TC_KC && FR_TC_TILE * 2 == OP_BYTES, "tiles are the operand tiles");
    static_assert(N % 16 == 0, "whole K = 16 steps");
    extern __shared__ __align__(128) uint8_t smem[];  // stage s: S' tile, plane-lo tile, plane-hi tile
    __shared__ __align__(8) uint64_t full[NSTAGE], mdone[NSTAGE];
    __shared__ uint32_t tmem_slot;
    __shared__ int s_abort;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int mt = blockIdx.x, x0 = mt * (TC_M / NB), nt = blockIdx.y, n0 = nt * TC_N;
    auto opA = [&](int st) { return smem + st * 3 * OP_BYTES; };
    auto full_a = [&](int st) { return smem_addr(&full[st]); };
    auto mdone_a = [&](int st) { return smem_addr(&mdone[st]); };
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(&tmem_slot)),
                     "r"(TC_TMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (tid == 0) {
        for (int i = 0; i < NSTAGE; i++) {
            mbar_init(full_a(i));
            mbar_init(mdone_a(i));
        }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        s_abort = 0;
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = tmem_slot, d_lo = tmem, d_hi = tmem + TC_N;

    if (tid == 0) {
        // one thread moves the tiles and issues the MMAs; stage c % NSTAGE holds chunk c.  The MMAs
        // of chunk c are queued before the thread waits for those of chunk c - 1, whose stage then
        // takes chunk c - 1 + NSTAGE, so the tensor cores always have the next chunk queued.
        auto issue = [&](int c) {
            issue_tiles(full_a(c % NSTAGE), smem_addr(opA(c % NSTAGE)), s16 + ((size_t)mt * KCH + c) * FR_TC_TILE,
                        planes + ((size_t)nt * KCH + c) * FR_TC_TILE, planes + ((size_t)(NT + nt) * KCH + c) * FR_TC_TILE);
        };
        int issued = 0, landed = 0, committed = -1;  // copies issued / waited for: chunks [0, issued) / [0, landed)
        bool ok = true;
        for (; issued < NSTAGE && issued < KCH; issued++) issue(issued);
        for (int c = 0; c < KCH; c++) {
            const int st = c % NSTAGE;
            if (!mbar_wait(full_a(st), (uint32_t)((c / NSTAGE) & 1))) {
                ok = false;
                break;
            }
            landed = c + 1;
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const int steps = min(TC_KC, N - c * TC_KC) / 16;
            const uint32_t a = smem_addr(opA(st)), lo = a + OP_BYTES, hi = a + 2 * OP_BYTES;
            for (int ks = 0; ks < steps; ks++) {
                const uint32_t off = ks * 2 * LBO;  // K = 16: two core matrices
                const uint32_t acc = (c > 0 || ks > 0) ? 1u : 0u;
                mma_f16(d_lo, sdesc(a + off), sdesc(lo + off), acc);
                mma_f16(d_hi, sdesc(a + off), sdesc(hi + off), acc);
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mdone_a(st))
                         : "memory");
            committed = c;
            if (c >= 1 && issued < KCH) {  // refill the stage of chunk c - 1 once its MMAs are done
                const int p = c - 1;
                if (!mbar_wait(mdone_a(p % NSTAGE), (uint32_t)((p / NSTAGE) & 1))) {
                    ok = false;
                    break;
                }
                issue(issued++);
            }
        }
        if (ok) {  // the last commit covers every MMA issued before it
            ok = mbar_wait(mdone_a((KCH - 1) % NSTAGE), (uint32_t)(((KCH - 1) / NSTAGE) & 1));
        } else {
            // leave nothing in flight: wait (bounded) for the copies not yet consumed and the
            // last committed MMAs
            for (int c = landed; c < issued; c++) mbar_wait(full_a(c % NSTAGE), (uint32_t)((c / NSTAGE) & 1));
            if (committed >= 0) mbar_wait(mdone_a(committed % NSTAGE), (uint32_t)((committed / NSTAGE) & 1));
        }
        if (!ok) {
            atomicOr(error, 1u);
            s_abort = 1;
        }
    }
    __syncthreads();
    const bool ok = !s_abort;
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (ok) {
        // epilogue: warp w holds rows 32w .. 32w + 31 (tensor-memory lanes)
        const int r = 32 * warp + lane, x = x0 + (r >> 3), i = r & 7;
        uint32_t *gacc = reinterpret_cast<uint32_t *>(scratch + (size_t)x * scratch_bytes(N) + gacc_off(N)) + (size_t)i * N;
        const uint32_t lane_base = (uint32_t)(32 * warp) << 16;
        for (int c0 = 0; c0 < TC_N; c0 += 16) {
            uint32_t lo[16], hi[16];
            asm volatile(
                "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
                : "=r"(lo[0]), "=r"(lo[1]), "=r"(lo[2]), "=r"(lo[3]), "=r"(lo[4]), "=r"(lo[5]), "=r"(lo[6]), "=r"(lo[7]),
                  "=r"(lo[8]), "=r"(lo[9]), "=r"(lo[10]), "=r"(lo[11]), "=r"(lo[12]), "=r"(lo[13]), "=r"(lo[14]),
                  "=r"(lo[15])
                : "r"(d_lo + lane_base + c0));
            asm volatile(
                "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
                : "=r"(hi[0]), "=r"(hi[1]), "=r"(hi[2]), "=r"(hi[3]), "=r"(hi[4]), "=r"(hi[5]), "=r"(hi[6]), "=r"(hi[7]),
                  "=r"(hi[8]), "=r"(hi[9]), "=r"(hi[10]), "=r"(hi[11]), "=r"(hi[12]), "=r"(hi[13]), "=r"(hi[14]),
                  "=r"(hi[15])
                : "r"(d_hi + lane_base + c0));
            asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
            const int j = n0 + c0;
            if (x < n && j < N) {
                uint32_t o[16];
#pragma unroll
                for (int q = 0; q < 16; q++)
                    o[q] = ((uint32_t)__float2int_rn(__uint_as_float(hi[q])) << 10) +
                           (uint32_t)__float2int_rn(__uint_as_float(lo[q]));
#pragma unroll
                for (int q = 0; q < 16; q += 4)
                    if (j + q < N) *reinterpret_cast<uint4 *>(gacc + j + q) = make_uint4(o[q], o[q + 1], o[q + 2], o[q + 3]);
            }
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TC_TMEM_COLS) : "memory");
}

template <int N>
int launch(int n, const uint16_t *planes, uint16_t *s16, uint8_t *scratch, unsigned *error, cudaStream_t st) {
    if (!capturing() &&
        cudaFuncSetAttribute(fr_sa_shared_tc<N>, cudaFuncAttributeMaxDynamicSharedMemorySize, TC_SMEM) != cudaSuccess) {
        cudaGetLastError();
        return PQCGPU_ECUDA;
    }
    const int mtiles = (8 * n + TC_M - 1) / TC_M;
    PQC_LAUNCH(st, "fr_s16_tiles", N, 0,
               fr_s16_tiles<N><<<mtiles * fr_tc_kchunks(N), 128, 0, st>>>(n, scratch, s16));
    const dim3 grid(mtiles, (N + TC_N - 1) / TC_N);
    PQC_LAUNCH(st, "fr_sa_shared_tc", N, 0, fr_sa_shared_tc<N><<<grid, TC_THREADS, TC_SMEM, st>>>(n, planes, s16, scratch, error));
    return cudaGetLastError() == cudaSuccess ? PQCGPU_OK : PQCGPU_ECUDA;
}

}  // namespace frodo_tc

// error: a device word the caller zeroed; set when a wait in the kernel runs out
int frodo_shared_tc_launch(int N, int n, const uint16_t *planes, uint16_t *s16, uint8_t *scratch, unsigned *error,
                           cudaStream_t st) {
    if (N == 640) return frodo_tc::launch<640>(n, planes, s16, scratch, error, st);
    if (N == 976) return frodo_tc::launch<976>(n, planes, s16, scratch, error, st);
    if (N == 1344) return frodo_tc::launch<1344>(n, planes, s16, scratch, error, st);
    return PQCGPU_EINVAL;
}

}  // namespace pqc
