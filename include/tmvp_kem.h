/*
 * tmvp_kem.h — C ABI of libtmvpkem: batched Saber/Sable KEM on one GB300 GPU.
 *
 * The entry points replace the reference's host API and keep its byte
 * layouts:
 *   - saber_enc / saber_dec        TMVP-Saber/SABER-GPU/include/cuda_kernel.cuh:6-7
 *                                  (bodies: TMVP-Saber/SABER-GPU/src/cuda_kernel.cu:25-479)
 *   - SABLE_enc / SABLE_dec        TMVP_SABLE/include/SABLE_indcpa.cuh:8-10
 *                                  (bodies: TMVP_SABLE/src/SABLE_indcpa.cu:24-610)
 *   - crypto_kem_keypair/enc/dec and indcpa_kem_keypair/enc/dec: the Saber
 *     reference C API whose byte layouts the reference's kernels implement
 *     (pk = pack_p(b) || seed_A; sk = pack(s) || pk || H(pk) || z;
 *      ct = pack_p(b') || pack_T(c_m); all little-endian bit streams).
 *   - tmvp_kem_*_batch: derandomised batched forms of the same operations;
 *     the reference's equivalent is its BATCH-wide launch sequence
 *     (saber_enc / saber_dec above).
 *   - tmvp_matvec_batch: the MatrixVectorMul step on its own
 *     (TMVP-Saber/SABER-GPU/src/poly.cu:269-376 schoolbook,
 *      :1396-1453 TMVP on CUDA cores, :1455-1500 TMVP on tensor cores).
 *
 * Conventions: caller-owned buffers, contiguous [n][bytes]; a buffer may be
 * host memory (pageable or pinned) or device memory of the context's GPU.
 * Calls return TMVP_OK or a negative TMVP_E* code; no exception crosses the
 * ABI.  A context is safe to share between host threads (calls on one
 * context are serialised).  The reference's void shims report their status
 * through tmvp_last_error().
 */
#ifndef TMVP_KEM_H
#define TMVP_KEM_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Parameter sets.  Saber family: TMVP-Saber/SABER-GPU/include/params.h:1-50
 * (L = 2, 3, 4).  Sable family: TMVP_SABLE/include/SABLE_params.h:1-73
 * (Saber_type 1, 2, 3). */
typedef enum {
  TMVP_LIGHTSABER = 0,
  TMVP_SABER = 1,
  TMVP_FIRESABER = 2,
  TMVP_LIGHTSABLE = 3,
  TMVP_SABLE = 4,
  TMVP_FIRESABLE = 5
} tmvp_param_set;

/* Polynomial-multiplication form (the reference's `mode` argument,
 * TMVP-Saber/SABER-GPU/main.cu:25-33, cuda_kernel.cu:140-163):
 *   CUDA_CORE     TMVP on CUDA cores (reference mode 1)
 *   INT8_TC       TMVP on INT8 tensor cores (mma.sync): s8 secrets x u8 limbs,
 *                 s32 accumulate
 *   FP8_TC        TMVP on FP8 tensor cores (mma.sync): e4m3 secrets x radix-8
 *                 digits biased by 8, f32 accumulate; every partial sum is an
 *                 integer below 2^24, so the result is exact
 *   AUTO          the fastest exact tensor-core form on this GPU (FP8_TCGEN05)
 *   SCHOOLBOOK    plain negacyclic schoolbook on CUDA cores (reference mode 2)
 *   FP8_TCGEN05   TMVP on the 5th-generation tensor cores (tcgen05.mma,
 *                 operands in shared memory, accumulator in tensor memory):
 *                 e4m3 secrets x radix-16 digits, f32 accumulate, exact
 *   DP2A          TMVP on CUDA cores with dp2a (two 16-bit x 8-bit products
 *                 per instruction), the DPSaber form of the reference's unused
 *                 DoDP4Av7 kernels (SABER poly.cu:32-224); secrets |s| <= 63
 *   TOOM_COOK     Toom-Cook 4-way on CUDA cores (the reference's pol_mul,
 *                 TMVP_SABLE pack.cu:505-732): seven 64x64 products per
 *                 polynomial pair, accumulated over the module index before
 *                 one interpolation */
typedef enum {
  TMVP_FORM_CUDA_CORE = 0,
  TMVP_FORM_INT8_TC = 1,
  TMVP_FORM_FP8_TC = 2,
  TMVP_FORM_AUTO = 3,
  TMVP_FORM_SCHOOLBOOK = 4,
  TMVP_FORM_FP8_TCGEN05 = 5,
  TMVP_FORM_DP2A = 6,
  TMVP_FORM_TOOM_COOK = 7
} tmvp_form;

enum {
  TMVP_OK = 0,
  TMVP_EINVAL = -1,   /* bad argument (null pointer, unknown set/form, n too large) */
  TMVP_ENOMEM = -2,   /* device workspace does not fit the context's memory budget */
  TMVP_EDEVICE = -3,  /* CUDA runtime error                                         */
  TMVP_ETIMEOUT = -4, /* a bounded device-side wait gave up                         */
  TMVP_ENOTSUP = -5   /* no usable GPU / unsupported architecture                  */
};

typedef struct {
  int l, eq, ep, et, mu;
  size_t pk_bytes, sk_bytes, ct_bytes, ss_bytes;
  size_t indcpa_pk_bytes, indcpa_sk_bytes;
} tmvp_sizes;

typedef struct tmvp_ctx tmvp_ctx;

/* Sizes of a parameter set. */
int tmvp_param_sizes(tmvp_param_set set, tmvp_sizes *out);
const char *tmvp_strerror(int code);
/* Status of the last call on this host thread (for the void shims). */
int tmvp_last_error(void);

/* Context: owns device workspace on `device`.  mem_budget caps the workspace
 * in bytes (0 = no cap).  Workspace grows on demand up to the cap. */
int tmvp_ctx_create(int device, size_t mem_budget, tmvp_ctx **out);
void tmvp_ctx_destroy(tmvp_ctx *ctx);
/* Device bytes of workspace the context holds now. */
size_t tmvp_ctx_workspace_bytes(const tmvp_ctx *ctx);
/* Number of kernel launches the context issued since creation. */
uint64_t tmvp_ctx_launch_count(const tmvp_ctx *ctx);
/* Per-stage timing (profiling aid; no counterpart in the reference, which
 * brackets whole operations with cudaEvent pairs, cuda_kernel.cu:114-188).
 * When enabled, every kernel launch is bracketed by CUDA events on its own
 * stream.  tmvp_ctx_stage_stats(ctx, -1, ...) returns the number of stages;
 * for idx >= 0 it fills the stage's kernel name, launch count and summed
 * device milliseconds (it waits for pending launches).  Disabling clears the
 * statistics. */
int tmvp_ctx_set_timing(tmvp_ctx *ctx, int enable);
int tmvp_ctx_stage_stats(tmvp_ctx *ctx, int idx, char *name, size_t name_len,
                         uint64_t *launches, double *total_ms);
/* The stage's busy milliseconds: the union of its launches' intervals, the
 * time during which at least one of them ran.  Launches of one stage on
 * several streams (the chunk chains of a decapsulation) overlap, so their
 * summed milliseconds overstate the time the stage took. */
int tmvp_ctx_stage_busy(tmvp_ctx *ctx, int idx, double *busy_ms);

/* Batched, derandomised KEM.  stream: a cudaStream_t (NULL = legacy default).
 * A secret key whose coefficients are outside the tensor-core forms' range
 * (|s| <= 7; real keys have |s| <= 5) makes the call return TMVP_EINVAL when
 * the call synchronises (host buffers).
 * keypair coins per instance: seed_A(32) | seed_s(32) | z(32).
 * enc coins per instance: 32 bytes (hashed into the message, as saber_enc
 * does with its 32 random bytes, cuda_kernel.cu:116).
 * The calls are asynchronous with respect to the host only when every buffer
 * is device memory; with host buffers they return after the results are in
 * host memory. */
int tmvp_kem_keypair_batch(tmvp_ctx *ctx, tmvp_param_set set, size_t n, uint8_t *pk,
                           uint8_t *sk, const uint8_t *coins, tmvp_form form, void *stream);
int tmvp_kem_enc_batch(tmvp_ctx *ctx, tmvp_param_set set, size_t n, uint8_t *ct, uint8_t *ss,
                       const uint8_t *pk, const uint8_t *coins, tmvp_form form, void *stream);
int tmvp_kem_dec_batch(tmvp_ctx *ctx, tmvp_param_set set, size_t n, uint8_t *ss,
                       const uint8_t *ct, const uint8_t *sk, tmvp_form form, void *stream);

/* Expanded public matrices kept per key (no counterpart in the reference,
 * which expands A on every call: GenMatrix, saber_enc / saber_dec
 * cuda_kernel.cu:116-127, :383).  tmvp_genmatrix_batch writes
 * a_stream[i] = SHAKE-128(seed_A of pk + i * pk_stride), the
 * tmvp_genmatrix_bytes(set) bytes that GenMatrix unpacks; the _a variants of
 * encapsulation and decapsulation take those streams (one per instance, in
 * device memory) instead of expanding A themselves, which removes 23 of the
 * 39 Keccak-f of a Saber decapsulation.  Results equal the plain calls for
 * the same keys.  a_stream and pk of tmvp_genmatrix_batch must be device
 * memory (TMVP_EINVAL otherwise). */
size_t tmvp_genmatrix_bytes(tmvp_param_set set);
int tmvp_genmatrix_batch(tmvp_ctx *ctx, tmvp_param_set set, size_t n, uint8_t *a_stream,
                         const uint8_t *pk, size_t pk_stride, void *stream);
int tmvp_kem_enc_batch_a(tmvp_ctx *ctx, tmvp_param_set set, size_t n, uint8_t *ct, uint8_t *ss,
                         const uint8_t *pk, const uint8_t *coins, const uint8_t *a_stream,
                         tmvp_form form, void *stream);
int tmvp_kem_dec_batch_a(tmvp_ctx *ctx, tmvp_param_set set, size_t n, uint8_t *ss,
                         const uint8_t *ct, const uint8_t *sk, const uint8_t *a_stream,
                         tmvp_form form, void *stream);
/* Decapsulation of n ciphertexts under ONE secret key (sk: sk_bytes, host or
 * device; ct, ss as in tmvp_kem_dec_batch): a server holding one long-term
 * key.  The key's GenMatrix runs once, then the cached-A chain (16 instead
 * of 39 Keccak-f per ciphertext), and with the tcgen05 form one CTA decrypts
 * 5 or 8 ciphertexts against the key's staged secret.  Same bytes as
 * tmvp_kem_dec_batch with sk repeated n times.  The reference's saber_dec
 * and SABLE_dec also decapsulate their whole batch under one key
 * (TMVP-Saber/SABER-GPU/src/cuda_kernel.cu:320-321, TMVP_SABLE/src/
 * SABLE_indcpa.cu:402-408), through per-instance buffers. */
int tmvp_kem_dec_batch_onekey(tmvp_ctx *ctx, tmvp_param_set set, size_t n, uint8_t *ss, const uint8_t *ct,
                              const uint8_t *sk, tmvp_form form, void *stream);

/* Batched IND-CPA (indcpa_kem_* of the Saber reference API, n instances). */
int tmvp_indcpa_keypair_batch(tmvp_ctx *ctx, tmvp_param_set set, size_t n, uint8_t *pk,
                              uint8_t *sk, const uint8_t *seeds /*[n][64]: seed_A|seed_s*/,
                              tmvp_form form, void *stream);
int tmvp_indcpa_enc_batch(tmvp_ctx *ctx, tmvp_param_set set, size_t n, uint8_t *ct,
                          const uint8_t *m /*[n][32]*/, const uint8_t *noiseseed /*[n][32]*/,
                          const uint8_t *pk, tmvp_form form, void *stream);
int tmvp_indcpa_dec_batch(tmvp_ctx *ctx, tmvp_param_set set, size_t n, uint8_t *m,
                          const uint8_t *sk, const uint8_t *ct, tmvp_form form, void *stream);

/* MatrixVectorMul alone: out[i] = sum_j A[i][j] * s[j] mod 2^eq
 * (transpose: A[j][i]); A uint16 [n][l][l][256] (values < 2^eq), s int8
 * [n][l][256], out uint16 [n][l][256].  l in 2..4, eq <= 13.  The
 * tensor-core forms take |s| <= 7 (CBD secrets have |s| <= 5) and return
 * TMVP_EINVAL otherwise; the CUDA-core forms take any int8 secret. */
int tmvp_matvec_batch(tmvp_ctx *ctx, size_t n, int l, int eq, int transpose, uint16_t *out,
                      const uint16_t *A, const int8_t *s, tmvp_form form, void *stream);

/* Reserve `bytes` of device workspace up front (so that later calls do not
 * allocate).  Fails with TMVP_ENOMEM above the context's budget. */
int tmvp_ctx_reserve(tmvp_ctx *ctx, size_t bytes);
/* Batched decapsulation with host-resident ct / sk copies and processes them
 * in chunks of n instances (one copy stream running ahead of the kernels), so
 * that copies overlap the kernels of earlier chunks; 0 = one copy, then the
 * kernels.  Unless set here (or chosen by tmvp_autotune for the batch size),
 * a call of b instances uses about b / 4, from 4096 to 16384.  n must be 0
 * or >= 1024.  Results do not depend on it. */
int tmvp_ctx_set_host_chunk(tmvp_ctx *ctx, size_t n);
/* The first `steps` chunks of such a call are n >> steps, n >> (steps - 1),
 * ..., n >> 1 instances (at least 256), so that the kernels start after a
 * short first copy; 0 = all chunks n.  Default 1; 0 <= steps <= 4.  Results
 * do not depend on it.  No counterpart in the reference (its calls are
 * synchronous, with the whole batch copied first). */
int tmvp_ctx_set_host_ramp(tmvp_ctx *ctx, int steps);
/* Batched decapsulation with device-resident buffers splits batches larger
 * than n into chunks whose decryption / G / re-encryption / final-key chains
 * run on four of the context's streams (joined back into the caller's), so
 * that one chunk's re-encryption overlaps the next chunk's GenMatrix and
 * decryption; 0 = one chain over the whole batch.  Default 32768; n must
 * be 0 or >= 1024.  Results do not depend on it. */
int tmvp_ctx_set_dev_chunk(tmvp_ctx *ctx, size_t n);
/* on != 0: decapsulation runs every stage on the caller's stream, one after
 * the other, unchunked and with the Keccak front uncapped (no side stream, no
 * lanes), so that the per-stage
 * timing (tmvp_ctx_set_timing) measures each kernel alone on the GPU.  Slower;
 * for measurement.  Results do not depend on it.  Default 0. */
int tmvp_ctx_set_serial(tmvp_ctx *ctx, int on);
/* Caps the Keccak front of decapsulation (GenMatrix + H(c), one launch beside
 * the decryption) at blocks_per_sm 64-thread blocks per SM, its threads then
 * striding over the sponges, so that decryption CTAs fit beside it on every
 * SM; 0 (the default) launches one thread per sponge.  0..64.  Results do
 * not depend on it. */
int tmvp_ctx_set_front_cap(tmvp_ctx *ctx, int blocks_per_sm);
/* The form of each Keccak launch (GenMatrix, GenSecret, H, G, the final
 * key).  Launches of at most warp_hash sponges run one warp per sponge, the
 * state spread over the warp's lanes (~2.1 us per permutation while the GPU
 * is far from full); larger ones of at most pair_hash sponges run two threads
 * per sponge, each holding half of every state lane (~3.3 us per permutation
 * up to ~10 K sponges); larger ones one thread per sponge (~4.7 us per
 * permutation, the best rate once the GPU is full).  Launches of short
 * sponges (G, the final key, the key-generation tail) count four times
 * against warp_hash and twice against pair_hash.  Defaults 1024 and 32768;
 * 0 turns a form off.  Results do not depend on them.  No counterpart in the reference, whose hash kernels run as one
 * block of one thread per instance
 * (TMVP-Saber/SABER-GPU/src/cuda_kernel.cu:116-127). */
int tmvp_ctx_set_warp_hash(tmvp_ctx *ctx, size_t max_sponges);
int tmvp_ctx_set_pair_hash(tmvp_ctx *ctx, size_t max_sponges);

/* ---------------------------------------------------------------------------
 * Request-serving loop with device-resident keys and continuous batching.
 * No counterpart in the reference (its host API runs one fixed batch per call).
 *
 * Requests (one KEM operation each) are queued per (parameter set, op).  A
 * scheduler thread turns the queue with the oldest waiting request into a
 * batch whenever one of `slots` batch slots is free (each slot owns a context
 * and CUDA stream, so up to `slots` batches run on the GPU at once while new
 * requests keep arriving).  Memory admission: every batch in flight holds a
 * block of one device arena (mem_budget bytes, or by default what `slots`
 * batches of max_batch requests of the largest set need) for its inputs,
 * outputs, gathered keys and matrices and KEM workspace; a batch takes as many
 * requests (up to max_batch) as the largest free block holds for its own set
 * and operation, and waits for a batch to finish when not even one fits.
 * Keys live in device tables (outside the arena) and are gathered per batch
 * by index.
 *   encaps: in = 32 random bytes,   out = ct || ss   (ct_bytes + 32 bytes)
 *   decaps: in = ct (ct_bytes),     out = ss         (32 bytes)
 * `in` and `out` must stay valid until the request completes.
 * ------------------------------------------------------------------------- */
typedef struct tmvp_server tmvp_server;
typedef struct {
  int device;
  size_t mem_budget; /* device bytes of the batch arena (0 = default);
                        must hold one request of every set             */
  int max_batch;     /* largest batch per launch, 1..65536 (0 = 4096)  */
  int slots;         /* batches in flight (0 = 4)                      */
  int form;          /* tmvp_form used for every batch                 */
} tmvp_server_config;
typedef struct {
  uint64_t submitted, completed, batches;
  double mean_batch;          /* requests per batch             */
  double p50_us, p99_us, max_us; /* submit-to-completion latency */
  double elapsed_s, throughput;  /* since the last reset         */
  int slots;                     /* batch slots                  */
  uint64_t failed;               /* requests of batches whose launch failed
                                    (their outputs are not written) */
  uint64_t one_key_batches;      /* decapsulation batches whose requests all
                                    used one key (tmvp_kem_dec_batch_onekey) */
  uint64_t arena_bytes;          /* device bytes of the batch arena */
  uint64_t peak_arena_bytes;     /* most arena bytes held at once   */
  uint64_t admission_waits;      /* times a batch waited for arena memory */
  uint64_t admission_splits;     /* batches cut short by arena memory     */
  uint64_t checked, mismatched;  /* load generator: decapsulations checked
                                    against the encapsulated key, and wrong */
} tmvp_server_stats;
enum { TMVP_OP_ENCAPS = 0, TMVP_OP_DECAPS = 1 };
int tmvp_server_create(const tmvp_server_config *cfg, tmvp_server **out);
void tmvp_server_destroy(tmvp_server *srv);
/* Copies n key pairs of one parameter set into the device key table and
 * returns their ids (key_ids[n]). */
int tmvp_server_add_keys(tmvp_server *srv, tmvp_param_set set, size_t n, const uint8_t *pk,
                         const uint8_t *sk, uint32_t *key_ids);
int tmvp_server_submit(tmvp_server *srv, int op, uint32_t key_id, const uint8_t *in, uint8_t *out,
                       uint64_t *ticket);
/* 0 when the request has completed, TMVP_ETIMEOUT otherwise. */
int tmvp_server_wait(tmvp_server *srv, uint64_t ticket, int timeout_ms);
int tmvp_server_drain(tmvp_server *srv, int timeout_ms);
int tmvp_server_get_stats(tmvp_server *srv, tmvp_server_stats *out);
void tmvp_server_reset_stats(tmvp_server *srv);
/* Load generator for benchmarking: Poisson arrivals at `rate` requests/s for
 * `seconds`, keys drawn uniformly from key_ids, decapsulations with
 * probability decaps_fraction (of a ciphertext made once per key), seeded.
 * Every decapsulation's key is checked against the encapsulated one
 * (stats.checked / stats.mismatched).  Waits are bounded: TMVP_ETIMEOUT if the
 * server does not finish the requests in time (their buffers then stay with
 * the server until it is destroyed). */
int tmvp_server_loadgen(tmvp_server *srv, double rate, double seconds, uint64_t seed,
                        const uint32_t *key_ids, size_t nkeys, double decaps_fraction,
                        uint64_t *submitted);

/* ---------------------------------------------------------------------------
 * Launch shapes and the autotuner (FP8_TCGEN05 form).  No counterpart in the
 * reference, whose kernels have fixed launch shapes (cuda_kernel.cu:140-163).
 *
 * Every IND-CPA step runs either as one CTA per instance (shape -1) or as the
 * persistent, pipelined kernel with `shape` CTAs per SM (0 = as many as fit);
 * the choice is kept per (step, parameter set), process-wide.
 * tmvp_autotune times every shape of every step for `set` on n synthetic
 * instances (key pairs and ciphertexts made with this library; every shape
 * must decapsulate to the same keys), keeps the fastest and, if `shapes` is
 * not NULL, writes them to shapes[5] (indexed by step).  It then picks the
 * decapsulation pass settings for n's batch bucket (ceil(log2 n), 256 ..
 * 2^20): the device chunk (tmvp_ctx_set_dev_chunk) and Keccak-front cap
 * (tmvp_ctx_set_front_cap) on device buffers, the host chunk and ramp
 * (tmvp_ctx_set_host_chunk / _ramp) on pinned host buffers, each the fastest
 * of its candidates that gives the same keys.  Decapsulations of that set and
 * bucket then use them, in every context, for each setting the context's
 * caller did not set explicitly.  n is clamped to 1024 .. 65536.  Run it with
 * no other call in flight on `ctx`.  If $TMVP_TUNE_CACHE names a file, the
 * choices are saved there after tuning and loaded from it when the first
 * context of the process is created.
 * ------------------------------------------------------------------------- */
enum {
  TMVP_STEP_DECRYPT = 0,
  TMVP_STEP_ENCRYPT = 1,
  TMVP_STEP_REENC = 2,
  TMVP_STEP_KEYGEN = 3,
  TMVP_STEP_MATVEC = 4
};
int tmvp_tune_set(int step, tmvp_param_set set, int shape);
int tmvp_tune_get(int step, tmvp_param_set set);
int tmvp_autotune(tmvp_ctx *ctx, tmvp_param_set set, size_t n, int *shapes);
/* The pass settings of (set, n's batch bucket): choice[4] = device chunk,
 * Keccak-front cap, host chunk, host ramp (the ranges of the tmvp_ctx_set_*
 * calls).  _get returns 1 and fills choice if the bucket has a choice, 0 if
 * not, TMVP_EINVAL on a bad argument. */
int tmvp_tune_pass_set(tmvp_param_set set, size_t n, const int *choice);
int tmvp_tune_pass_get(tmvp_param_set set, size_t n, int *choice);
/* Forget every choice (launch shapes back to one CTA per instance). */
void tmvp_tune_clear(void);
/* Write / read the choices as a text file (TMVP_EINVAL if it cannot be
 * written or read, or holds a malformed line; good lines are still loaded). */
int tmvp_tune_save(const char *path);
int tmvp_tune_load(const char *path);

/* Waits for `stream`, then reads and clears the context's device status:
 * TMVP_EINVAL if a secret was outside the tensor-core range, TMVP_ETIMEOUT if
 * a bounded device wait gave up, TMVP_OK otherwise.  For work launched without
 * a host synchronisation (device buffers, graphs). */
int tmvp_ctx_sync_status(tmvp_ctx *ctx, void *stream);
/* Failure-detection self-test: launches one tcgen05 matrix-vector instance
 * whose input barrier is told to expect 16 bytes more than its copies bring,
 * so the kernel's bounded wait (about two seconds, then a second bounded
 * wait for anything still in flight) gives up, frees its tensor memory and
 * reports.  Returns TMVP_ETIMEOUT when that path works as designed (after
 * about four seconds); the context stays usable.  No counterpart in the
 * reference, which has no device-side waits. */
int tmvp_selftest_bounded_wait(tmvp_ctx *ctx, void *stream);
/* Tensor-core issue cost of the exact kinds available to the IND-CPA kernels:
 * kind 0 = tcgen05.mma kind::f8f6f4 (e4m3, K = 32), kind 1 = kind::f16 (f16,
 * K = 16), M = 128, N = n (16, 32, 64, 128 or 256).  ctas_per_sm CTAs on
 * every SM each issue `iters` MMAs back to back; out[0] = median cycles per
 * MMA of one CTA (issue to completion), out[1] = out[0] / ctas_per_sm, the
 * SM's cycles per MMA.  A diagnostic with no counterpart in the reference. */
int tmvp_diag_umma_rate(tmvp_ctx *ctx, int kind, int n, int ctas_per_sm, int iters, double *out);
/* Keccak-f[1600] permutation rate at full occupancy (one register-resident
 * state per thread, the hash stages' permutation, `perms` per thread, as
 * many 64-thread blocks as fit on every SM): out[0] = permutations per
 * second over the GPU, out[1] = resident blocks per SM.  The integer-pipe
 * ceiling of the hash stages.  A diagnostic with no counterpart in the
 * reference. */
int tmvp_diag_keccak_rate(tmvp_ctx *ctx, int perms, double *out);

/* ---------------------------------------------------------------------------
 * Mixed-parameter decapsulation.  No counterpart in the reference (one
 * parameter set per build, params.h:4).
 *
 * Up to 64 groups (at most 2^30 instances in all), each with its own
 * parameter set (any of the six) and its own device buffers (16-byte aligned,
 * this context's GPU), decapsulate in one pass: every stage is ONE launch over
 * all groups -- GenMatrix, H(c), G and the final key as Keccak kernels, the two
 * IND-CPA steps on the tcgen05 tensor cores (one CTA per instance, or the
 * persistent pipelined kernel where the autotuner chose it for every set in
 * the pass).  tmvp_mixed_plan_create
 * captures the pass for fixed buffers into a CUDA graph (the plan owns its
 * workspace); tmvp_mixed_plan_launch replays it, so the caller refills the
 * ciphertext / key buffers and relaunches.  Asynchronous on `stream`; use
 * tmvp_ctx_sync_status for the device status.
 * ------------------------------------------------------------------------- */
typedef struct {
  tmvp_param_set set;
  size_t n;
  uint8_t *ss;        /* [n][32]       */
  const uint8_t *ct;  /* [n][ct_bytes] */
  const uint8_t *sk;  /* [n][sk_bytes] */
} tmvp_dec_group;
int tmvp_kem_dec_mixed(tmvp_ctx *ctx, size_t ngroups, const tmvp_dec_group *groups, void *stream);
typedef struct tmvp_mixed_plan tmvp_mixed_plan;
int tmvp_mixed_plan_create(tmvp_ctx *ctx, size_t ngroups, const tmvp_dec_group *groups,
                           tmvp_mixed_plan **out);
int tmvp_mixed_plan_launch(tmvp_mixed_plan *plan, void *stream);
void tmvp_mixed_plan_destroy(tmvp_mixed_plan *plan);

/* Decapsulation that allocates nothing.  No counterpart in the reference.
 * For callers that cannot call cudaMalloc: a host whose GPU memory is owned
 * by its own pool allocator, or a serving process that forbids allocation
 * after start-up so that its latency stays flat.
 * Instead of a context workspace it uses one fixed array in device global
 * memory (7.4 MiB, sized for TMVP_NOALLOC_MAX_BATCH instances of the largest
 * parameter set), which every GPU that loads the library holds until the
 * process exits.  n <= TMVP_NOALLOC_MAX_BATCH
 * (larger n returns TMVP_EINVAL and launches nothing); ss, ct and sk must be
 * 16-byte-aligned device memory of the current GPU.
 * The return value covers the arguments and the launches only.  Errors that
 * the GPU finds (a secret outside a tensor-core form's exact range, a bounded
 * device wait that gave up) arrive in *status: when the stream reaches the
 * end of the call the GPU writes TMVP_OK, TMVP_EINVAL or TMVP_ETIMEOUT there.
 * status is a 4-byte-aligned int in device memory of the current GPU or in
 * host memory mapped into it (cudaHostAlloc); NULL drops the report.
 * The first call on a device (and the first after its context was replaced,
 * e.g. by cudaDeviceReset) looks up the array's address with that device
 * current: make it before any stream capture.  All calls share the array,
 * which keeps the last call's contents, so calls that overlap on the GPU
 * race; issue them in order on one stream.  The call is asynchronous on
 * `stream` and calls no cudaMalloc, cudaFree or allocating library routine. */
#define TMVP_NOALLOC_MAX_BATCH 1024
int tmvp_kem_dec_batch_noalloc(tmvp_param_set set, size_t n, uint8_t *ss, const uint8_t *ct,
                               const uint8_t *sk, tmvp_form form, int *status, void *stream);

/* NIST-style single-instance API for the default parameter set (Saber unless
 * changed).  Randomness comes from the randombytes hook (default: the
 * operating system's getrandom).  Return 0 on success. */
int crypto_kem_keypair(uint8_t *pk, uint8_t *sk);
int crypto_kem_enc(uint8_t *ct, uint8_t *ss, const uint8_t *pk);
int crypto_kem_dec(uint8_t *ss, const uint8_t *ct, const uint8_t *sk);
int indcpa_kem_keypair(uint8_t *pk, uint8_t *sk);
int indcpa_kem_enc(const uint8_t m[32], const uint8_t seed_sp[32], const uint8_t *pk,
                   uint8_t *ciphertext);
int indcpa_kem_dec(const uint8_t *sk, const uint8_t *ciphertext, uint8_t m[32]);
typedef void (*tmvp_randombytes_fn)(uint8_t *out, size_t len);
void tmvp_set_randombytes(tmvp_randombytes_fn fn);
int tmvp_set_default_param_set(tmvp_param_set set);

/* Reference-compatible shims.  mode: 0 = tensor cores (AUTO), 1 = CUDA-core
 * TMVP, other = schoolbook, as in the reference.  They process
 * tmvp_ref_batch(scheme) instances (defaults: Saber 1 and Sable 512, the
 * reference's BATCH values, cuda_kernel.cuh:1 and SABLE_indcpa.cuh:6) over
 * contiguous [batch][bytes] host arrays.  Unlike the reference they do not
 * overwrite h_pk / h_sk with built-in test vectors: the caller's keys are
 * used, and the 32 random bytes per encapsulation come from the randombytes
 * hook.  h_pk is unused by the decapsulation shims (sk embeds pk). */
void saber_enc(uint8_t mode, uint8_t *h_k, uint8_t *h_pk, uint8_t *h_c);
void saber_dec(uint8_t mode, uint8_t *h_c, uint8_t *h_pk, uint8_t *h_sk, uint8_t *h_k);
void SABLE_enc(uint8_t *h_k, uint8_t *h_pk, uint8_t *h_c, int mode);
void SABLE_dec(uint8_t *h_c, uint8_t *h_pk, uint8_t *h_sk, uint8_t *h_k, int mode);
/* scheme: 0 = Saber shims, 1 = Sable shims. */
int tmvp_ref_set_batch(int scheme, size_t n);
size_t tmvp_ref_batch(int scheme);

#ifdef __cplusplus
}
#endif
#endif /* TMVP_KEM_H */
