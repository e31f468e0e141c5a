/*
 * pqcgpu -- batched post-quantum KEMs on one NVIDIA GB300 (sm_103a).  C ABI.
 *
 * This header is the drop-in boundary for the reference's KEM path.  The reference exposes, per
 * compile-time parameter set, the NIST/SUPERCOP API
 *     int crypto_kem_keypair(unsigned char *pk, unsigned char *sk);
 *     int crypto_kem_enc(unsigned char *ct, unsigned char *ss, const unsigned char *pk);
 *     int crypto_kem_dec(unsigned char *ss, const unsigned char *ct, const unsigned char *sk);
 * (Kyber_GPU_Batched/api.h:18-22, FrodoKEM_GPU/api.h:20-24, sizes in the CRYPTO_* macros of
 * Kyber_GPU_Batched/api.h:11-14, NewHope_NIST_GPU/api.h:11-14, FrodoKEM_GPU/api.h:11-14), and
 * internally batched CPA entry points taking an instance count
 *     indcpa_keypair / indcpa_enc / indcpa_dec(int COUNT, poly_set4*, ..., cudaStream_t)
 *       (Kyber_GPU_Batched/indcpa.h:16-26)
 *     cpapke_keypair / cpapke_enc / cpapke_dec(int COUNT, poly_set4*, ..., cudaStream_t)
 *       (NewHope_NIST_GPU/cpapke.h:14-24).
 * Here every parameter set lives in one library, selected at run time by pqcgpu_alg, and the
 * batch count is an argument.
 *
 * Conventions (all functions):
 *   - Return 0 (PQCGPU_OK) on success or a negative pqcgpu_status; never exit().
 *   - Buffers are instance-major: instance i of an n-batch starts at i * <size>.
 *   - Caller owns every buffer.  Without PQCGPU_DEVICE_PTRS the pointers are host memory
 *     (pinned memory is fastest) and the call is synchronous.  With PQCGPU_DEVICE_PTRS they are
 *     device pointers on the context's device and the call is asynchronous on the context stream
 *     (pqcgpu_ctx_wait synchronises).
 *   - Randomness is explicit: `coins` holds kp_coins / enc_coins bytes per instance (sizes from
 *     pqcgpu_alg_sizes).  Passing coins == NULL draws them from the library's SHAKE-256 DRBG.
 *   - A decapsulation whose re-encryption check fails is not an error: it returns 0 with the
 *     implicit-rejection key, as the NIST API requires.
 *   - A context may be used from several host threads; calls are serialised internally.
 */
#ifndef PQCGPU_H
#define PQCGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    PQCGPU_KYBER512 = 0,     /* round-3 Kyber-512:  k=2, eta1=3, eta2=2, du=10, dv=4 */
    PQCGPU_KYBER768 = 1,     /* round-3 Kyber-768:  k=3, eta=2, du=10, dv=4 */
    PQCGPU_KYBER1024 = 2,    /* round-3 Kyber-1024: k=4, eta=2, du=11, dv=5 */
    PQCGPU_KYBER1024_R2 = 3, /* the reference's round-2 Kyber (Kyber_GPU_Batched/params.h), k=4 */
    PQCGPU_NEWHOPE1024 = 4,  /* NewHope1024-CPAKEM (NewHope_NIST_GPU) */
    PQCGPU_FRODO976 = 5,     /* FrodoKEM-976, SHAKE (FrodoKEM_GPU) */
    PQCGPU_MLKEM512 = 6,     /* ML-KEM-512 (FIPS 203): round-3 Kyber-512 K-PKE with G(d || k), K direct, */
    PQCGPU_MLKEM768 = 7,     /*   rejection key J(z || c); same sizes as the round-3 sets.  The FIPS 203 */
    PQCGPU_MLKEM1024 = 8,    /*   input checks (ek modulus, dk hash) are left to the caller. */
    PQCGPU_NEWHOPE512 = 9,   /* NewHope512-CPAKEM (NewHope_NIST_GPU built with NEWHOPE_N = 512) */
    PQCGPU_FRODO640 = 10,    /* FrodoKEM-640, SHAKE: the FrodoKEM-976 flow with the 640 parameter set */
    PQCGPU_FRODO1344 = 11,   /* FrodoKEM-1344, SHAKE: the same with the 1344 parameter set */
    PQCGPU_NUM_ALGS = 12
} pqcgpu_alg;

typedef enum {
    PQCGPU_OK = 0,
    PQCGPU_EINVAL = -1,      /* bad argument (unknown alg, null pointer, n out of range) */
    PQCGPU_ENOMEM = -2,      /* device or pinned-host allocation failed */
    PQCGPU_ECUDA = -3,       /* a CUDA call failed; pqcgpu_last_error() has the text */
    PQCGPU_EBUDGET = -4,     /* the request does not fit the context's device-memory budget */
    PQCGPU_ETIMEOUT = -5,    /* a bounded device-side wait gave up */
    PQCGPU_EUNSUPPORTED = -6 /* operation not available for this algorithm / variant */
} pqcgpu_status;

/* flags */
#define PQCGPU_DEVICE_PTRS 0x1u /* all buffer arguments are device pointers; asynchronous */
#define PQCGPU_PLAIN 0x2u       /* use the plain per-stage path (one kernel per stage, thread per
                                   instance, intermediates in HBM) instead of the fused path */
#define PQCGPU_STAGE_KERNELS 0x4u /* mixed batches: persistent per-stage kernels for all Kyber, FrodoKEM and
                                     NewHope jobs instead of every job's own kernels on the
                                     concurrent streams */

typedef struct pqcgpu_ctx pqcgpu_ctx;

/* ---- context lifecycle ----------------------------------------------------------------- */
/* Create a context on `device` with a device-memory budget for its arena (0 = 4 GiB). */
int pqcgpu_ctx_create(pqcgpu_ctx **out, int device, size_t hbm_budget_bytes);
int pqcgpu_ctx_destroy(pqcgpu_ctx *ctx);
/* Use an external cudaStream_t (passed as void*) instead of the context's own stream. */
int pqcgpu_ctx_set_stream(pqcgpu_ctx *ctx, void *cuda_stream);
void *pqcgpu_ctx_stream(pqcgpu_ctx *ctx);
int pqcgpu_ctx_wait(pqcgpu_ctx *ctx);
/* Number of kernels this context launched since creation (for launch accounting). */
uint64_t pqcgpu_ctx_launches(pqcgpu_ctx *ctx);
const char *pqcgpu_last_error(void);
const char *pqcgpu_version(void);

/* ---- sizes ------------------------------------------------------------------------------ */
int pqcgpu_alg_sizes(pqcgpu_alg alg, size_t *pk, size_t *sk, size_t *ct, size_t *ss, size_t *kp_coins,
                     size_t *enc_coins);

/* ---- batched KEM (the batched extension of crypto_kem_*) ---------------------------------- */
int pqcgpu_kem_keypair_batch(pqcgpu_ctx *ctx, pqcgpu_alg alg, size_t n, uint8_t *pk, uint8_t *sk,
                             const uint8_t *coins, unsigned flags);
int pqcgpu_kem_enc_batch(pqcgpu_ctx *ctx, pqcgpu_alg alg, size_t n, uint8_t *ct, uint8_t *ss, const uint8_t *pk,
                         const uint8_t *coins, unsigned flags);
int pqcgpu_kem_dec_batch(pqcgpu_ctx *ctx, pqcgpu_alg alg, size_t n, uint8_t *ss, const uint8_t *ct,
                         const uint8_t *sk, unsigned flags);

/* ---- encapsulation without allocation --------------------------------------------------------
 * No counterpart in the reference.  For callers that cannot call cudaMalloc (code running inside
 * another framework's allocator or memory pool, plugins handed fixed device buffers, real-time
 * paths that forbid allocation after start-up): a Kyber encapsulation (alg = one of the Kyber
 * algorithms) that allocates nothing and needs no context.  All pointers are caller-owned device
 * buffers on the current device (16-byte aligned, coins required); work is enqueued on `stream`
 * (a cudaStream_t, NULL = legacy default stream) and the call returns without waiting.
 * Its scratch is one fixed 6 MiB device array (96 bytes for each of up to 65536 instances), held
 * by every GPU that loads the library until the process exits; n > 65536 returns PQCGPU_EINVAL.
 * Every call shares that array: calls whose work overlaps on the GPU (other streams, other host
 * threads) race and must be serialised by the caller.  Each call writes every scratch byte it
 * reads before reading it, so nothing left by an earlier call needs clearing.  The first call on
 * a device does the set-up (constant tables, lookup of the array's device address); make that
 * first call before any stream capture.  The address is kept for the life of the process, so a
 * device reset (cudaDeviceReset) between calls is not supported.  Leave the launch profiler off
 * for this call. */
int pqcgpu_kem_enc_batch_noalloc(pqcgpu_alg alg, size_t n, uint8_t *ct, uint8_t *ss, const uint8_t *pk,
                                 const uint8_t *coins, void *stream);

/* ---- many FrodoKEM encapsulations to one public key --------------------------------------------
 * n encapsulations to the one public key pk (alg = a FrodoKEM algorithm, pk = one key of
 * CRYPTO_PUBLICKEYBYTES), coins = mu per instance (NULL: library DRBG, host buffers only): ct and ss
 * per instance, the same bytes as pqcgpu_kem_enc_batch with pk repeated n times.  Replaces n calls of
 * crypto_kem_enc (FrodoKEM_GPU/kem.c:66-131 via frodo976.cu:229-425), each of which regenerates
 * the key's matrix A: here A is generated once per call, and the products B'_x = S'_x A of all
 * instances (frodo_macrify_reference.cu:102-159) run as one matrix product, on the CUDA cores or on
 * the tensor cores (launch-shape op 3 of the FrodoKEM algorithms: ni = 1 CUDA cores, 2 tensor
 * cores, 0 the measured default).  Host buffers: synchronous; PQCGPU_DEVICE_PTRS: asynchronous on
 * the context stream.  Every wait inside the tensor-core product is bounded: one that runs out (a
 * device fault, never seen in normal operation) makes the call (host buffers) or the next
 * pqcgpu_ctx_wait (device pointers) return PQCGPU_ECUDA, and that call's outputs are undefined. */
int pqcgpu_frodo_enc_shared_key_batch(pqcgpu_ctx *ctx, pqcgpu_alg alg, size_t n, uint8_t *ct, uint8_t *ss,
                                      const uint8_t *pk, const uint8_t *coins, unsigned flags);

/* ---- batched CPA-PKE (replaces indcpa_* of Kyber_GPU_Batched/indcpa.h:16-26) -------------
 * variant 2 = the reference's round-2 arithmetic, variant 3 = round-3 parameter sets; k = 2..4.
 * keypair: d = 32 bytes per instance; pk = KYBER_INDCPA_PUBLICKEYBYTES, sk = K*384.
 * enc: m and coins 32 bytes per instance.  dec: m out 32 bytes per instance. */
int pqcgpu_kyber_indcpa_keypair_batch(pqcgpu_ctx *ctx, int variant, int k, size_t n, uint8_t *pk, uint8_t *sk,
                                      const uint8_t *d, unsigned flags);
int pqcgpu_kyber_indcpa_enc_batch(pqcgpu_ctx *ctx, int variant, int k, size_t n, uint8_t *ct, const uint8_t *m,
                                  const uint8_t *pk, const uint8_t *coins, unsigned flags);
int pqcgpu_kyber_indcpa_dec_batch(pqcgpu_ctx *ctx, int variant, int k, size_t n, uint8_t *m, const uint8_t *ct,
                                  const uint8_t *sk, unsigned flags);

/* ---- batched NewHope CPA-PKE (replaces cpapke_* of NewHope_NIST_GPU/cpapke.h:14-24) ----------
 * NewHope-1024 (pqcgpu_newhope_*): keypair: seed 32 bytes per instance -> pk 1824, sk 1792; enc: msg
 * and coin 32 bytes per instance -> ct 2176; dec: msg out 32 bytes per instance.
 * NewHope-512 (pqcgpu_newhope512_*, the reference's NEWHOPE_N = 512 build, params.h:9-11): pk 928,
 * sk 896, ct 1088. */
int pqcgpu_newhope_cpapke_keypair_batch(pqcgpu_ctx *ctx, size_t n, uint8_t *pk, uint8_t *sk, const uint8_t *seed,
                                        unsigned flags);
int pqcgpu_newhope_cpapke_enc_batch(pqcgpu_ctx *ctx, size_t n, uint8_t *ct, const uint8_t *msg, const uint8_t *pk,
                                    const uint8_t *coin, unsigned flags);
int pqcgpu_newhope_cpapke_dec_batch(pqcgpu_ctx *ctx, size_t n, uint8_t *msg, const uint8_t *ct, const uint8_t *sk,
                                    unsigned flags);
int pqcgpu_newhope512_cpapke_keypair_batch(pqcgpu_ctx *ctx, size_t n, uint8_t *pk, uint8_t *sk, const uint8_t *seed,
                                           unsigned flags);
int pqcgpu_newhope512_cpapke_enc_batch(pqcgpu_ctx *ctx, size_t n, uint8_t *ct, const uint8_t *msg, const uint8_t *pk,
                                       const uint8_t *coin, unsigned flags);
int pqcgpu_newhope512_cpapke_dec_batch(pqcgpu_ctx *ctx, size_t n, uint8_t *msg, const uint8_t *ct, const uint8_t *sk,
                                       unsigned flags);

/* ---- mixed batches and CUDA graphs --------------------------------------------------------
 * A job is one (algorithm, operation, batch) with its device buffers:
 *   op PQCGPU_OP_KEYPAIR: in0 coins          -> out0 pk, out1 sk
 *   op PQCGPU_OP_ENC:     in0 pk,  in1 coins -> out0 ct, out1 ss
 *   op PQCGPU_OP_DEC:     in0 ct,  in1 sk    -> out0 ss
 * pqcgpu_kem_mixed_batch runs any mix of jobs (parameter sets, operations, uneven sizes) at once,
 * after the work already queued on the context stream and joined back into it (asynchronous;
 * device pointers only, PQCGPU_DEVICE_PTRS): every job's kernels run on the context's concurrent
 * streams.  With PQCGPU_STAGE_KERNELS the core stages of the Kyber jobs (round 3 and ML-KEM, all
 * k, every operation) run instead as two persistent waves -- keypair, encapsulation and decryption
 * tiles, then re-encryption tiles -- those of the NewHope jobs (n = 1024 and 512) as one more, and
 * the products of the FrodoKEM jobs as one wave per stage and parameter set: SMs x (CTAs per SM)
 * CTAs take (job, instance group) tiles from an atomic counter, heaviest first (the per-job hash
 * kernels and the other jobs still spread over the streams).  The default is the faster of the
 * two on GB300 (`bench.py --config mixed` reports both).
 * pqcgpu_graph_capture records such a job list once into a CUDA graph (with its own scratch) and
 * pqcgpu_graph_launch replays it on the context stream: same buffers, no per-kernel launch cost. */
#define PQCGPU_OP_KEYPAIR 0
#define PQCGPU_OP_ENC 1
#define PQCGPU_OP_DEC 2
typedef struct {
    int32_t alg; /* pqcgpu_alg */
    int32_t op;  /* PQCGPU_OP_* */
    uint64_t n;  /* instances */
    const uint8_t *in0, *in1;
    uint8_t *out0, *out1;
} pqcgpu_job;
typedef struct pqcgpu_graph pqcgpu_graph;
int pqcgpu_kem_mixed_batch(pqcgpu_ctx *ctx, const pqcgpu_job *jobs, size_t njobs, unsigned flags);
int pqcgpu_graph_capture(pqcgpu_ctx *ctx, const pqcgpu_job *jobs, size_t njobs, unsigned flags, pqcgpu_graph **out);
int pqcgpu_graph_launch(pqcgpu_graph *graph);
int pqcgpu_graph_destroy(pqcgpu_graph *graph);

/* ---- serving loop ----------------------------------------------------------------------------
 * A server owns a dispatcher thread that batches individual requests continuously: whenever one of
 * its max_inflight slots (stream + staging buffers) is free it takes up to max_batch waiting
 * requests of the oldest request's (algorithm, operation), runs them as one GPU batch on that
 * slot's stream, and completes each request when its batch finishes, so requests arriving while
 * others are on the GPU join the next batch and overlap with them.  Keys stay on the device: a
 * KEYPAIR request stores pk / sk in the server's key store and returns a handle; ENC / DEC use the
 * handle (ENC may pass pk bytes instead).  Device memory (key stores + staging) is admitted against
 * hbm_budget_bytes (0 = 16 GiB); a request that cannot fit while nothing else is in flight fails
 * with PQCGPU_EBUDGET.  Buffers of a request (host memory) must stay valid until it completes.
 * Results are byte-identical to the batched entry points for the same inputs. */
typedef struct pqcgpu_server pqcgpu_server;
typedef struct {
    int32_t alg;        /* pqcgpu_alg */
    int32_t op;         /* PQCGPU_OP_* */
    uint64_t key;       /* ENC / DEC: key handle (ENC: 0 = use pk) */
    const uint8_t *pk;  /* ENC without a handle: public key */
    const uint8_t *in;  /* KEYPAIR / ENC: coins (NULL = library DRBG); DEC: ciphertext */
    uint8_t *out0;      /* KEYPAIR: pk (may be NULL); ENC: ct; DEC: ss */
    uint8_t *out1;      /* ENC: ss */
    uint64_t *key_out;  /* KEYPAIR: receives the key handle (may be NULL) */
} pqcgpu_request;
typedef struct {
    uint64_t completed, batches, keys_resident;
    size_t hbm_used;
    double p50_ms, p99_ms, mean_ms, max_ms; /* submit-to-completion latency of completed requests */
} pqcgpu_server_stats;
typedef struct {
    int32_t alg, op;
    double weight;
} pqcgpu_mix_entry;
typedef struct {
    double offered_per_s, achieved_per_s, seconds, submit_seconds, p50_ms, p99_ms, mean_ms, max_ms;
    uint64_t submitted, completed, batches;
} pqcgpu_load_report;
int pqcgpu_server_create(pqcgpu_server **out, int device, size_t hbm_budget_bytes, int max_inflight, int max_batch);
int pqcgpu_server_submit(pqcgpu_server *server, const pqcgpu_request *req, uint64_t *ticket);
/* 0 when done, a negative status if the request failed, PQCGPU_ETIMEOUT (timeout_ms < 0: wait forever) */
int pqcgpu_server_wait(pqcgpu_server *server, uint64_t ticket, int timeout_ms);
int pqcgpu_server_drain(pqcgpu_server *server);
int pqcgpu_server_get_stats(pqcgpu_server *server, pqcgpu_server_stats *out, int reset);
/* Latency of the completed requests of one (algorithm, operation) since the last reset;
 * `completed` counts them, `batches` and `keys_resident` are 0. */
int pqcgpu_server_get_group_stats(pqcgpu_server *server, int alg, int op, pqcgpu_server_stats *out);
int pqcgpu_server_key_release(pqcgpu_server *server, uint64_t key);
int pqcgpu_server_destroy(pqcgpu_server *server);
/* Open-loop load for the serving benchmark: resident key / ciphertext pools per algorithm of the
 * mix are prepared first, then requests drawn from the weighted (alg, op) mix are submitted at
 * Poisson arrival times at rate_per_s for `seconds`, and the server is drained. */
int pqcgpu_server_run_poisson(pqcgpu_server *server, const pqcgpu_mix_entry *mix, size_t nmix, double rate_per_s,
                              double seconds, uint64_t seed, pqcgpu_load_report *out);

/* ---- launch-shape tuning (used by the autotuner, pqc_gb300/autotune.py) --------------------
 * Core-kernel launch shape per (algorithm, operation): ni = instances per CTA, threads per CTA
 * (multiple of 32).  Kyber also takes op 3: the decryption stage of decapsulation (op 2 is then
 * its re-encryption stage), and op 4: ni = the largest KEM batch that runs on the single-instance
 * kernels (one CTA per instance), set for every operation of this k (0 = never, -1 = the measured
 * per-operation defaults; get returns the encapsulation's; threads ignored), and op 5:
 * ni = the largest batch whose serial hashes (H(pk), G, H(c), the KDF) run one warp per instance
 * instead of one thread (0..65535, default 2048; all k; threads ignored).  Kyber: ni
 * 1..128, threads from 32 up to the core kernel's launch bound (keypair 512, encapsulation 256,
 * re-encryption 256, decryption stage 384; shared by the round-2 and round-3 sets of the same k);
 * NewHope: ni 1..64, threads 32..256; op 3: ni = the largest batch whose key generations and
 * encapsulations (CPA and KEM) run on the single-instance kernels (one CTA per instance; both n;
 * 0 = never, -1 = the measured defaults, 304 for keypair and 456 for encapsulation; get returns
 * the encapsulation's).  FrodoKEM: keypair ni 0 or 1, threads 64 / 128 / 256 (one row of A per thread); encaps / decaps ni = CTAs per instance sharing the rows of A (1, 2, 4, 8,
 * 16) with threads 128 / 256, or ni = 0 to choose by batch size (the default); op 3: ni = the
 * product of pqcgpu_frodo_enc_shared_key_batch (1 CUDA cores, 2 tensor cores, 0 default).
 * Applies to all contexts of the process; a launch reads the pair atomically. */
int pqcgpu_set_launch_shape(pqcgpu_alg alg, int op, int ni, int threads);
int pqcgpu_get_launch_shape(pqcgpu_alg alg, int op, int *ni, int *threads);

/* Shape of the host-buffer pipeline; there is no counterpart in the reference, whose drivers copy a
 * whole batch before and after the kernels. A host-buffer call splits its batch into chunks:
 * `chunk_first` instances, doubling up to `chunk_max`, an even split of the middle into chunks of
 * at most `chunk_max`, then doubling down to `chunk_last`.
 * Copies in run in order on one stream and copies out on another. Each chunk's kernels start as
 * soon as its inputs are in, on one of `streams` compute streams (1..8) in turn. Each chunk has
 * its own device buffers, up to 16 chunks and the context budget; later chunks reuse them.
 * Zeros select the defaults: chunk_max 16384, chunk_first = chunk_max / 8, chunk_last =
 * chunk_max / 4, 8 streams (measured best on GB300 for Kyber-768 at 65536 instances).
 * Applies to all contexts of the process. */
int pqcgpu_set_host_pipeline(size_t chunk_max, size_t chunk_first, size_t chunk_last, int streams);
int pqcgpu_get_host_pipeline(size_t *chunk_max, size_t *chunk_first, size_t *chunk_last, int *streams);

/* ---- tracing and roofline probes ------------------------------------------------------------
 * These replace the reference's TIMING_START / TIMING_END event pairs
 * (Kyber_GPU_Batched/indcpa.cu:21-84).
 * pqcgpu_profile_enable(1): every kernel launch, and every copy of a host-buffer call ("copy H2D",
 * "copy D2H"), is bracketed by CUDA events on its stream.
 * pqcgpu_profile_read: JSON {"kernel<k,v>": [launches, total_ms], ...} of the records since the
 * last read (synchronises on them), then clears them.
 * pqcgpu_profile_trace: the same records as a timeline in the Chrome trace-event format
 * ({"traceEvents": [{"name", "ph": "X", "tid" = stream, "ts", "dur"}]}, microseconds from the
 * earliest record), for chrome://tracing or Perfetto. *len: in, the capacity of buf; out, the bytes
 * needed with the NUL. If buf is NULL or too small, PQCGPU_EINVAL and the records are kept.
 * Otherwise it clears them.
 * pqcgpu_probe_peaks: measured integer-pipe (LOP3) op rate and register-resident Keccak-f[1600]
 * permutation rate of `device`, the denominators of the integer roofline. */
int pqcgpu_profile_enable(int on);
int pqcgpu_profile_read(char *buf, size_t len);
int pqcgpu_profile_trace(char *buf, size_t *len);
int pqcgpu_probe_peaks(int device, double *int_ops_per_s, double *keccak_perms_per_s);

/* ---- NIST single-instance API per parameter set (crypto_kem_* of each api.h) -------------
 * Randomness comes from the library DRBG (pqcgpu_randombytes_init); device 0, default context. */
int pqcgpu_randombytes_init(const uint8_t seed[48]);
int pqcgpu_randombytes(uint8_t *out, size_t n);
/* Switch the library DRBG to the NIST KAT generator's AES-256 CTR_DRBG (SP 800-90A, no derivation
 * function), instantiated with entropy[48] xor personalization[48] (NULL: none).
 * pqcgpu_randombytes_init returns to the SHAKE-256 DRBG. */
int pqcgpu_randombytes_init_nist(const uint8_t entropy[48], const uint8_t *personalization);
/* The coins of one crypto_kem_keypair (op 0) or crypto_kem_enc (op 1) of `alg`, drawn from the
 * library DRBG in the randombytes calls of that algorithm's submission package; kp_coins or
 * enc_coins bytes (pqcgpu_alg_sizes) are written. */
int pqcgpu_nist_coins(pqcgpu_alg alg, int op, uint8_t *coins);

int pqcgpu_kyber512_crypto_kem_keypair(unsigned char *pk, unsigned char *sk);
int pqcgpu_kyber512_crypto_kem_enc(unsigned char *ct, unsigned char *ss, const unsigned char *pk);
int pqcgpu_kyber512_crypto_kem_dec(unsigned char *ss, const unsigned char *ct, const unsigned char *sk);
int pqcgpu_kyber768_crypto_kem_keypair(unsigned char *pk, unsigned char *sk);
int pqcgpu_kyber768_crypto_kem_enc(unsigned char *ct, unsigned char *ss, const unsigned char *pk);
int pqcgpu_kyber768_crypto_kem_dec(unsigned char *ss, const unsigned char *ct, const unsigned char *sk);
int pqcgpu_kyber1024_crypto_kem_keypair(unsigned char *pk, unsigned char *sk);
int pqcgpu_kyber1024_crypto_kem_enc(unsigned char *ct, unsigned char *ss, const unsigned char *pk);
int pqcgpu_kyber1024_crypto_kem_dec(unsigned char *ss, const unsigned char *ct, const unsigned char *sk);
int pqcgpu_newhope1024_crypto_kem_keypair(unsigned char *pk, unsigned char *sk);
int pqcgpu_newhope1024_crypto_kem_enc(unsigned char *ct, unsigned char *ss, const unsigned char *pk);
int pqcgpu_newhope1024_crypto_kem_dec(unsigned char *ss, const unsigned char *ct, const unsigned char *sk);
int pqcgpu_newhope512_crypto_kem_keypair(unsigned char *pk, unsigned char *sk);
int pqcgpu_newhope512_crypto_kem_enc(unsigned char *ct, unsigned char *ss, const unsigned char *pk);
int pqcgpu_newhope512_crypto_kem_dec(unsigned char *ss, const unsigned char *ct, const unsigned char *sk);
int pqcgpu_frodo976_crypto_kem_keypair(unsigned char *pk, unsigned char *sk);
int pqcgpu_frodo976_crypto_kem_enc(unsigned char *ct, unsigned char *ss, const unsigned char *pk);
int pqcgpu_frodo976_crypto_kem_dec(unsigned char *ss, const unsigned char *ct, const unsigned char *sk);
int pqcgpu_frodo640_crypto_kem_keypair(unsigned char *pk, unsigned char *sk);
int pqcgpu_frodo640_crypto_kem_enc(unsigned char *ct, unsigned char *ss, const unsigned char *pk);
int pqcgpu_frodo640_crypto_kem_dec(unsigned char *ss, const unsigned char *ct, const unsigned char *sk);
int pqcgpu_frodo1344_crypto_kem_keypair(unsigned char *pk, unsigned char *sk);
int pqcgpu_frodo1344_crypto_kem_enc(unsigned char *ct, unsigned char *ss, const unsigned char *pk);
int pqcgpu_frodo1344_crypto_kem_dec(unsigned char *ss, const unsigned char *ct, const unsigned char *sk);
int pqcgpu_mlkem512_crypto_kem_keypair(unsigned char *pk, unsigned char *sk);
int pqcgpu_mlkem512_crypto_kem_enc(unsigned char *ct, unsigned char *ss, const unsigned char *pk);
int pqcgpu_mlkem512_crypto_kem_dec(unsigned char *ss, const unsigned char *ct, const unsigned char *sk);
int pqcgpu_mlkem768_crypto_kem_keypair(unsigned char *pk, unsigned char *sk);
int pqcgpu_mlkem768_crypto_kem_enc(unsigned char *ct, unsigned char *ss, const unsigned char *pk);
int pqcgpu_mlkem768_crypto_kem_dec(unsigned char *ss, const unsigned char *ct, const unsigned char *sk);
int pqcgpu_mlkem1024_crypto_kem_keypair(unsigned char *pk, unsigned char *sk);
int pqcgpu_mlkem1024_crypto_kem_enc(unsigned char *ct, unsigned char *ss, const unsigned char *pk);
int pqcgpu_mlkem1024_crypto_kem_dec(unsigned char *ss, const unsigned char *ct, const unsigned char *sk);

#ifdef __cplusplus
}
#endif
#endif
