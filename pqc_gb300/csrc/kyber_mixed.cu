// One kernel per stage for the Kyber jobs of a mixed batch.
//
// A mixed batch (pqcgpu_kem_mixed_batch) may hold Kyber encapsulations and decapsulations of all
// three module ranks (round 3 and ML-KEM) with uneven batch sizes.  Instead of one chain of kernels
// per job, the core stages of all such jobs run as single launches: each CTA looks up its job in a
// small table passed as a __grid_constant__ kernel parameter (the job's k, instances per CTA and
// buffers) and runs that k's stage body on its instances.  Jobs are ordered by k, heaviest first,
// so the long CTAs start early and the short ones fill the tail.  The per-job serial hash kernels
// (H(pk), G, H(c), KDF) stay per job; the caller spreads them over streams.
#include <algorithm>
#include <vector>

#include "kyber_impl.cuh"

namespace pqc {
namespace kyber {
namespace {

constexpr int MIX_MAX_JOBS = 32;  // jobs per table (a kernel parameter of about 4.6 KB)
constexpr int MIX_THREADS = 128, MIX_THREADS_DEC1 = 384;
// instances per CTA by k (index k - 2): at 128 threads about one thread per matrix entry of the
// encryption phases; the decryption stage is warp-level and runs 12 warps per CTA
constexpr int MIX_NI_ENC[3] = {24, 14, 8};
constexpr int MIX_NI_DEC1[3] = {32, 24, 12};

struct MixJob {
    int k, ni, first;  // module rank, instances per CTA, first CTA of the job
    EncArgs e;         // encapsulation jobs
    DecArgs d;         // decapsulation jobs
};
struct MixTable {
    int njobs;
    MixJob j[MIX_MAX_JOBS];
};

__device__ __forceinline__ const MixJob &mix_job(const MixTable &t, int b) {
    int j = 0;
    while (j + 1 < t.njobs && b >= t.j[j + 1].first) j++;
    return t.j[j];
}

__global__ void __launch_bounds__(MIX_THREADS) kyber_enc_core_mixed(const __grid_constant__ MixTable t) {
    const MixJob &m = mix_job(t, blockIdx.x);
    const int base = (blockIdx.x - m.first) * m.ni;
    if (m.k == 2) enc_core_body<2, 3>(m.e, m.ni, base);
    else if (m.k == 3) enc_core_body<3, 3>(m.e, m.ni, base);
    else enc_core_body<4, 3>(m.e, m.ni, base);
}

template <int STAGE>
__global__ void __launch_bounds__(MIX_THREADS_DEC1) kyber_dec_core_mixed(const __grid_constant__ MixTable t) {
    const MixJob &m = mix_job(t, blockIdx.x);
    const int base = (blockIdx.x - m.first) * m.ni;
    if (m.k == 2) dec_core_body<2, 3, STAGE>(m.d, m.ni, base);
    else if (m.k == 3) dec_core_body<3, 3, STAGE>(m.d, m.ni, base);
    else dec_core_body<4, 3, STAGE>(m.d, m.ni, base);
}

template <int K>
size_t enc_smem(int ni) { return Layout<2 * K + 1, enc_seed_bytes<K, 3>()>::bytes(ni, MIX_THREADS); }
template <int K>
size_t dec1_smem(int ni) { return Layout<2 * K + 1, enc_seed_bytes<K, 3>()>::bytes(ni, 0); }
size_t stage_smem(int k, bool dec1) {
    const int ni = (dec1 ? MIX_NI_DEC1 : MIX_NI_ENC)[k - 2];
    if (k == 2) return dec1 ? dec1_smem<2>(ni) : enc_smem<2>(ni);
    if (k == 3) return dec1 ? dec1_smem<3>(ni) : enc_smem<3>(ni);
    return dec1 ? dec1_smem<4>(ni) : enc_smem<4>(ni);
}

// the per-job hash kernels, thread or warp per instance as in the single-job path
template <int K>
void enc_hashes(bool pre, const MixedKyberJob &j, cudaStream_t st) {
    const int n = j.n;
    if (pre) {
        if (n <= WARP_HASH_MAX)
            PQC_LAUNCH(st, "kyber_enc_hash_pre", K, 3,
                       kyber_enc_hash_pre_w<K, 3><<<(n + 3) / 4, 128, 0, st>>>(n, j.in0, j.in1, j.scratch, j.kem));
        else
            PQC_LAUNCH(st, "kyber_enc_hash_pre", K, 3,
                       kyber_enc_hash_pre<K, 3><<<(n + 127) / 128, 128, 0, st>>>(n, j.in0, j.in1, j.scratch, j.kem));
    } else {
        if (n <= WARP_HASH_MAX)
            PQC_LAUNCH(st, "kyber_enc_hash_post", K, 3,
                       kyber_enc_hash_post_w<K, 3><<<(n + 3) / 4, 128, 0, st>>>(n, j.out0, j.scratch, j.out1, j.kem));
        else
            PQC_LAUNCH(st, "kyber_enc_hash_post", K, 3,
                       kyber_enc_hash_post<K, 3><<<(n + 127) / 128, 128, 0, st>>>(n, j.out0, j.scratch, j.out1, j.kem));
    }
}
template <int K>
void dec_hash(const MixedKyberJob &j, cudaStream_t st) {
    const int n = j.n;
    if (n <= WARP_HASH_MAX)
        PQC_LAUNCH(st, "kyber_dec_hash_pre", K, 3,
                   kyber_dec_hash_pre_w<K, 3><<<(n + 3) / 4, 128, 0, st>>>(n, j.in0, j.in1, j.scratch, j.kem));
    else
        PQC_LAUNCH(st, "kyber_dec_hash_pre", K, 3,
                   kyber_dec_hash_pre<K, 3><<<(n + 127) / 128, 128, 0, st>>>(n, j.in0, j.in1, j.scratch, j.kem));
}
void hashes(int op, bool pre, const MixedKyberJob &j, cudaStream_t st) {
    if (op == 1) {
        if (j.k == 2) enc_hashes<2>(pre, j, st);
        else if (j.k == 3) enc_hashes<3>(pre, j, st);
        else enc_hashes<4>(pre, j, st);
    } else if (pre) {
        if (j.k == 2) dec_hash<2>(j, st);
        else if (j.k == 3) dec_hash<3>(j, st);
        else dec_hash<4>(j, st);
    }
}

int pkb(int k) { return k * 384 + 32; }

// Fill a table with jobs [from, to) of `js` (sorted by k, heaviest first) for the stage.
int fill_table(MixTable &t, int op, bool dec1, const MixedKyberJob *js, int from, int to, size_t *smem) {
    t.njobs = to - from;
    int blocks = 0;
    *smem = 0;
    for (int i = from; i < to; i++) {
        const MixedKyberJob &j = js[i];
        MixJob &m = t.j[i - from];
        m.k = j.k;
        m.ni = (dec1 ? MIX_NI_DEC1 : MIX_NI_ENC)[j.k - 2];
        m.first = blocks;
        blocks += (j.n + m.ni - 1) / m.ni;
        *smem = std::max(*smem, stage_smem(j.k, dec1));
        if (op == 1) {
            m.e = EncArgs{};
            m.e.n = j.n;
            m.e.ct = j.out0;
            m.e.pk = j.in0;
            m.e.pk_stride = pkb(j.k);
            m.e.m = j.scratch;
            m.e.m_stride = 96;
            m.e.r = j.scratch + 32;
            m.e.r_stride = 96;
        } else {
            m.d = DecArgs{};
            m.d.n = j.n;
            m.d.ct = j.in0;
            m.d.sk = j.in1;
            m.d.m_out = nullptr;
            m.d.ss = j.out0;
            m.d.hct = j.scratch;
            m.d.kem = j.kem;
            m.d.mr = j.scratch + (size_t)j.n * 32;
        }
    }
    return blocks;
}

template <class Kern>
int launch_stage(Kern kern, const char *name, const MixTable &t, int blocks, int threads, size_t sm, cudaStream_t st) {
    if (!capturing() && cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm) != cudaSuccess) {
        cudaGetLastError();
        return PQCGPU_ECUDA;
    }
    PQC_LAUNCH(st, name, 0, 3, kern<<<blocks, threads, sm, st>>>(t));
    return cudaGetLastError() == cudaSuccess ? PQCGPU_OK : PQCGPU_ECUDA;
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
    kyber::prefer_shared(kyber::kyber_enc_core_mixed);
    kyber::prefer_shared(kyber::kyber_dec_core_mixed<kyber::DEC_DECRYPT>);
    kyber::prefer_shared(kyber::kyber_dec_core_mixed<kyber::DEC_REENCRYPT>);
    return PQCGPU_OK;
}

int kyber_mixed_hash(int op, bool pre, const MixedKyberJob &j, cudaStream_t st) {
    if (op != 1 && op != 2) return PQCGPU_EINVAL;
    if (j.n > 0) kyber::hashes(op, pre, j, st);
    return cudaGetLastError() == cudaSuccess ? PQCGPU_OK : PQCGPU_ECUDA;
}

int kyber_mixed_core(int op, const MixedKyberJob *jobs_in, int njobs, cudaStream_t st) {
    using namespace kyber;
    if (op != 1 && op != 2) return PQCGPU_EINVAL;
    std::vector<MixedKyberJob> js;
    for (int i = 0; i < njobs; i++)
        if (jobs_in[i].n > 0) js.push_back(jobs_in[i]);
    std::stable_sort(js.begin(), js.end(), [](const MixedKyberJob &a, const MixedKyberJob &b) { return a.k > b.k; });
    const int nj = (int)js.size();
    for (int from = 0; from < nj; from += MIX_MAX_JOBS) {
        const int to = std::min(nj, from + MIX_MAX_JOBS);
        MixTable t;
        size_t sm = 0;
        int rc;
        if (op == 1) {
            const int blocks = fill_table(t, 1, false, js.data(), from, to, &sm);
            rc = launch_stage(kyber_enc_core_mixed, "kyber_enc_core_mixed", t, blocks, MIX_THREADS, sm, st);
        } else {
            int blocks = fill_table(t, 2, true, js.data(), from, to, &sm);
            rc = launch_stage(kyber_dec_core_mixed<DEC_DECRYPT>, "kyber_dec_decrypt_mixed", t, blocks, MIX_THREADS_DEC1, sm,
                              st);
            if (!rc) {
                blocks = fill_table(t, 2, false, js.data(), from, to, &sm);
                rc = launch_stage(kyber_dec_core_mixed<DEC_REENCRYPT>, "kyber_dec_reencrypt_mixed", t, blocks, MIX_THREADS,
                                  sm, st);
            }
        }
        if (rc) return rc;
    }
    return PQCGPU_OK;
}

}  // namespace pqc
