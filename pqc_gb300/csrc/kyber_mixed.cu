// Persistent per-stage kernels for the Kyber jobs of a mixed batch.
//
// A mixed batch (pqcgpu_kem_mixed_batch with PQCGPU_STAGE_KERNELS) may hold Kyber key generations,
// encapsulations and decapsulations of all three module ranks (round 3 and ML-KEM) with uneven
// batch sizes.  Instead of one chain of kernels per job, their core stages run in two persistent
// launches:
//   wave A: every keypair core, encapsulation core and decapsulation's decryption stage;
//   wave B: every decapsulation's re-encryption stage (after G, which needs wave A's m').
// Each wave launches the SMs x (CTAs per SM) that fit at once.  A CTA takes a tile (a job and a
// group of NI instances) from a global atomic counter, runs that job's stage body for its k on it,
// and takes the next, so uneven jobs share the GPU without a tail per job and without a launch
// per job.  The tiles are ordered heaviest first (encapsulation, then keypair, then decryption;
// larger k first), so the long tiles start early and the short ones fill the end.
// The per-job serial hash kernels (G(d), H(pk), G, H(c), KDF) stay per job on the caller's streams
// between the waves (thread or warp per instance, as in the single-job path).
//
// One launch has one block size and one dynamic shared-memory size: every stage runs at 128
// threads, with instances per CTA chosen per (stage, k) so that every tile needs at most the
// 76.7 KB of Kyber-768 encapsulation's tuned shape (three CTAs per SM).
//
// Replaces the reference's fixed per-operation launch chains, one parameter set per build
// (Kyber_GPU_Batched/indcpa.cu:474-733).
#include <algorithm>
#include <vector>

#include "kyber_impl.cuh"

namespace pqc {
namespace kyber {
namespace {

constexpr int MIX_MAX_JOBS = 40;  // jobs per wave table (a kernel parameter, about 6.5 KB)
constexpr int MIX_THREADS = 128;
enum StageKind { ST_ENC = 0, ST_KP = 1, ST_DEC1 = 2, ST_DEC2 = 3 };
// instances per CTA by stage and k (index k - 2), every tile within 76.7 KB of shared memory
constexpr int MIX_NI[4][3] = {{19, 14, 8}, {16, 12, 8}, {21, 15, 12}, {19, 14, 8}};

struct MixJob {
    int kind, k, ni, first;  // stage, module rank, instances per CTA, first tile of the job
    KpArgs kp;
    EncArgs e;
    DecArgs d;
};
struct MixTable {
    int njobs, tiles;
    MixJob j[MIX_MAX_JOBS];
};

__device__ __forceinline__ int mix_find(const MixTable &t, int tile) {
    int lo = 0, hi = t.njobs - 1;  // the last job whose first tile <= tile
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (t.j[mid].first <= tile) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

template <int K>
__device__ __forceinline__ void mix_run(const MixJob &m, int base) {
    switch (m.kind) {
    case ST_ENC: enc_core_body<K, 3>(m.e, m.ni, base); break;
    case ST_KP: kp_core_body<K, 3>(m.kp, m.ni, base); break;
    case ST_DEC1: dec_core_body<K, 3, DEC_DECRYPT>(m.d, m.ni, base); break;
    default: dec_core_body<K, 3, DEC_REENCRYPT>(m.d, m.ni, base); break;
    }
}

// counter: a zeroed word of device memory for this launch
__global__ void __launch_bounds__(MIX_THREADS, 3) kyber_stage_persistent(const __grid_constant__ MixTable t,
                                                                      unsigned *counter) {
    __shared__ int s_tile;
    for (;;) {
        if (threadIdx.x == 0) s_tile = (int)atomicAdd(counter, 1u);
        __syncthreads();
        const int tile = s_tile;
        if (tile >= t.tiles) break;
        const MixJob &m = t.j[mix_find(t, tile)];
        const int base = (tile - m.first) * m.ni;
        if (m.k == 2) mix_run<2>(m, base);
        else if (m.k == 3) mix_run<3>(m, base);
        else mix_run<4>(m, base);
        __syncthreads();  // the next tile reuses shared memory (and s_tile)
    }
}

template <int K>
size_t tile_smem(int kind, int ni) {
    switch (kind) {
    case ST_KP: return Layout<3 * K, 128>::bytes(ni, MIX_THREADS);
    case ST_DEC1: return Layout<2 * K + 1, enc_seed_bytes<K, 3>()>::bytes(ni, 0);
    default: return Layout<2 * K + 1, enc_seed_bytes<K, 3>()>::bytes(ni, MIX_THREADS);
    }
}
size_t tile_smem(int kind, int k, int ni) {
    return k == 2 ? tile_smem<2>(kind, ni) : k == 3 ? tile_smem<3>(kind, ni) : tile_smem<4>(kind, ni);
}

int pkb(int k) { return k * 384 + 32; }

void fill_job(MixJob &m, int kind, const MixedKyberJob &j) {
    m.kind = kind;
    m.k = j.k;
    m.ni = MIX_NI[kind][j.k - 2];
    m.kp = KpArgs{};
    m.e = EncArgs{};
    m.d = DecArgs{};
    if (kind == ST_KP) {
        m.kp = KpArgs{j.n, j.out0, j.out1, j.in0, 64, j.kem, j.scratch};
    } else if (kind == ST_ENC) {
        m.e.n = j.n;
        m.e.ct = j.out0;
        m.e.pk = j.in0;
        m.e.pk_stride = pkb(j.k);
        m.e.m = j.scratch;
        m.e.m_stride = 96;
        m.e.r = j.scratch + 32;
        m.e.r_stride = 96;
    } else {
        m.d.n = j.n;
        m.d.ct = j.in0;
        m.d.sk = j.in1;
        m.d.ss = j.out0;
        m.d.hct = j.scratch;
        m.d.kem = j.kem;
        m.d.mr = j.scratch + (size_t)j.n * 32;
        m.d.g_post = 1;                              // G runs between the waves (kyber_dec_hash_mid)
        m.d.kdf_post = j.kem == KEM_FO ? 1 : 0;      // the KDF after wave B (kyber_dec_hash_post)
    }
}

// The largest tile of any job kind: the kernel's dynamic shared-memory bound, set once at init so
// that no launch (captured into a graph or not) depends on an earlier launch having raised it.
size_t max_tile_smem() {
    size_t sm = 0;
    for (int kind = 0; kind < 4; kind++)
        for (int k = 2; k <= 4; k++) sm = std::max(sm, tile_smem(kind, k, MIX_NI[kind][k - 2]));
    return sm;
}

// One persistent launch over `items` (kind, job) on st; counter = a zeroed word of device memory.
int launch_wave(const std::vector<std::pair<int, const MixedKyberJob *>> &items, unsigned *counter, cudaStream_t st) {
    for (size_t from = 0; from < items.size(); from += MIX_MAX_JOBS) {
        const size_t to = std::min(items.size(), from + MIX_MAX_JOBS);
        MixTable t;
        t.njobs = (int)(to - from);
        t.tiles = 0;
        size_t sm = 0;
        for (size_t i = from; i < to; i++) {
            MixJob &m = t.j[i - from];
            fill_job(m, items[i].first, *items[i].second);
            m.first = t.tiles;
            t.tiles += (items[i].second->n + m.ni - 1) / m.ni;
            sm = std::max(sm, tile_smem(m.kind, m.k, m.ni));
        }
        if (sm > max_tile_smem()) return PQCGPU_EINVAL;  // the bound set at init covers every job kind
        int dev = 0, sms = 0, per_sm = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kyber_stage_persistent, MIX_THREADS, sm) != cudaSuccess ||
            per_sm < 1)
            per_sm = 1;
        const int grid = std::min(t.tiles, sms * per_sm);
        unsigned *ctr = counter + from / MIX_MAX_JOBS;
        if (cudaMemsetAsync(ctr, 0, sizeof(unsigned), st) != cudaSuccess) return PQCGPU_ECUDA;
        PQC_LAUNCH(st, "kyber_stage_persistent", 0, 3, kyber_stage_persistent<<<grid, MIX_THREADS, sm, st>>>(t, ctr));
        if (cudaGetLastError() != cudaSuccess) return PQCGPU_ECUDA;
    }
    return PQCGPU_OK;
}

// the per-job hash kernels, thread or warp per instance as in the single-job path
template <int K>
void job_hash(int op, int phase, const MixedKyberJob &j, cudaStream_t st) {
    const int n = j.n;
    const bool w = n <= warp_hash_max();
    if (op == 0) {
        if (phase == 0)
            PQC_LAUNCH(st, "kyber_kp_hash_pre", K, 3,
                       kyber_kp_hash_pre<K, 3><<<(n + 127) / 128, 128, 0, st>>>(n, j.in0, 64, j.kem, j.scratch));
        else if (phase == 2 && w)
            PQC_LAUNCH(st, "kyber_kp_hash_post", K, 3, kyber_kp_hash_post_w<K, 3><<<(n + 3) / 4, 128, 0, st>>>(n, j.out0, j.out1));
        else if (phase == 2)
            PQC_LAUNCH(st, "kyber_kp_hash_post", K, 3,
                       kyber_kp_hash_post<K, 3><<<(n + 127) / 128, 128, 0, st>>>(n, j.out0, j.out1));
    } else if (op == 1) {
        if (phase == 0 && w)
            PQC_LAUNCH(st, "kyber_enc_hash_pre", K, 3,
                       kyber_enc_hash_pre_w<K, 3><<<(n + 3) / 4, 128, 0, st>>>(n, j.in0, j.in1, j.scratch, j.kem));
        else if (phase == 0)
            PQC_LAUNCH(st, "kyber_enc_hash_pre", K, 3,
                       kyber_enc_hash_pre<K, 3><<<(n + 127) / 128, 128, 0, st>>>(n, j.in0, j.in1, j.scratch, j.kem));
        else if (phase == 2 && w)
            PQC_LAUNCH(st, "kyber_enc_hash_post", K, 3,
                       kyber_enc_hash_post_w<K, 3><<<(n + 3) / 4, 128, 0, st>>>(n, j.out0, j.scratch, j.out1, j.kem));
        else if (phase == 2)
            PQC_LAUNCH(st, "kyber_enc_hash_post", K, 3,
                       kyber_enc_hash_post<K, 3><<<(n + 127) / 128, 128, 0, st>>>(n, j.out0, j.scratch, j.out1, j.kem));
    } else {
        if (phase == 0 && w)
            PQC_LAUNCH(st, "kyber_dec_hash_pre", K, 3,
                       kyber_dec_hash_pre_w<K, 3><<<(n + 3) / 4, 128, 0, st>>>(n, j.in0, j.in1, j.scratch, j.kem));
        else if (phase == 0)
            PQC_LAUNCH(st, "kyber_dec_hash_pre", K, 3,
                       kyber_dec_hash_pre<K, 3><<<(n + 127) / 128, 128, 0, st>>>(n, j.in0, j.in1, j.scratch, j.kem));
        else if (phase == 1)
            PQC_LAUNCH(st, "kyber_dec_hash_mid", K, 3,
                       kyber_dec_hash_mid<K, 3><<<(n + 127) / 128, 128, 0, st>>>(n, j.in1, j.scratch + (size_t)n * 32));
        else if (j.kem == KEM_FO)
            PQC_LAUNCH(st, "kyber_dec_hash_post", K, 3,
                       kyber_dec_hash_post<K, 3><<<(n + 127) / 128, 128, 0, st>>>(n, j.scratch + (size_t)n * 32, j.scratch,
                                                                                 j.out0));
    }
}

}  // namespace
}  // namespace kyber

// This translation unit's copies of the constant tables (Keccak round constants, NTT twiddles):
// every translation unit that instantiates the kernels holds its own.
int kyber_mixed_init() {
    uint2 rc[24];
    keccak_rc_host(rc);
    int16_t z[128], zi[128];
    kyber::kyber_twiddles_host(z, zi);
    if (cudaMemcpyToSymbol(c_keccak_rc, rc, sizeof rc) != cudaSuccess) return PQCGPU_ECUDA;
    if (cudaMemcpyToSymbol(kyber::c_zetas, z, sizeof z) != cudaSuccess) return PQCGPU_ECUDA;
    if (cudaMemcpyToSymbol(kyber::c_zetas_inv, zi, sizeof zi) != cudaSuccess) return PQCGPU_ECUDA;
    int2 tw[128], twi[128];
    kyber::kyber_twiddles_shoup_host(tw, twi);
    if (cudaMemcpyToSymbol(kyber::c_tw, tw, sizeof tw) != cudaSuccess) return PQCGPU_ECUDA;
    if (cudaMemcpyToSymbol(kyber::c_twi, twi, sizeof twi) != cudaSuccess) return PQCGPU_ECUDA;
    kyber::prefer_shared(kyber::kyber_stage_persistent);
    if (cudaFuncSetAttribute(kyber::kyber_stage_persistent, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)kyber::max_tile_smem()) != cudaSuccess)
        return PQCGPU_ECUDA;
    return PQCGPU_OK;
}

int kyber_mixed_hash(int op, int phase, const MixedKyberJob &j, cudaStream_t st) {
    if (op < 0 || op > 2 || phase < 0 || phase > 3) return PQCGPU_EINVAL;
    if (j.n > 0) {
        if (j.k == 2) kyber::job_hash<2>(op, phase, j, st);
        else if (j.k == 3) kyber::job_hash<3>(op, phase, j, st);
        else kyber::job_hash<4>(op, phase, j, st);
    }
    return cudaGetLastError() == cudaSuccess ? PQCGPU_OK : PQCGPU_ECUDA;
}

// wave 0: keypair cores, encapsulation cores, decryption stages; wave 1: re-encryption stages.
// jobs[op] lists the jobs of operation op; counters: MIXED_COUNTER_WORDS zeroable words.
int kyber_mixed_wave(int wave, const std::vector<MixedKyberJob> (&jobs)[3], unsigned *counters, cudaStream_t st) {
    using namespace kyber;
    std::vector<std::pair<int, const MixedKyberJob *>> items;
    auto add = [&](int kind, int op) {
        for (int k = 4; k >= 2; k--)  // heavier k first
            for (const auto &j : jobs[op])
                if (j.k == k && j.n > 0) items.push_back({kind, &j});
    };
    if (wave == 0) {
        add(ST_ENC, 1);
        add(ST_KP, 0);
        add(ST_DEC1, 2);
    } else {
        add(ST_DEC2, 2);
    }
    if (items.empty()) return PQCGPU_OK;
    if (items.size() > (size_t)MIX_MAX_JOBS * (MIXED_COUNTER_WORDS / 2)) return PQCGPU_EINVAL;
    return launch_wave(items, counters + wave * (MIXED_COUNTER_WORDS / 2), st);
}

}  // namespace pqc
