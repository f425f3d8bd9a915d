/*
 * z0p_gpu.h — C ABI of the GB300 (sm_103a) proving backend for z0p.
 *
 * The backend replaces the CPU prove path of z0p (FutureProofsTech/z0p,
 * a pure-Rust crate) behind its own API: the same parameter structs and
 * validation rules, the same Fiat-Shamir transcript and the same VERSION=6
 * proof bytes. Every declaration below names the reference item it stands in
 * for (paths inside the z0p repository). All structs are plain C with fixed
 * widths, so a `z0p-gpu-sys` crate can mirror them with #[repr(C)].
 *
 * Conventions
 *  - Field elements are canonical BabyBear values (< 2013265921) as uint32_t.
 *  - Status codes: 0 = Ok; 1..9 mirror the variants of z0p::Error in
 *    declaration order (src/error.rs:7-40); >= 100 are backend errors.
 *    z0p_gpu_last_reason() returns the thread-local message of the last
 *    failure on this thread and consumes it (a second read returns ""); the
 *    pointer stays valid until the next read on the same thread.
 *  - Proof-producing calls write into a caller-owned host buffer. When `cap`
 *    is too small they write the required size to *len and return
 *    Z0P_ERR_BUFFER_TOO_SMALL before any device work.
 *  - A context owns one CUDA stream and the device workspace; calls on one
 *    context are serialised by an internal mutex. Outputs are deterministic.
 */
#ifndef Z0P_GPU_H
#define Z0P_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define Z0P_GPU_ABI_VERSION 1

/* Status codes. 1..9 follow z0p::Error (src/error.rs:7-40) in order. */
enum {
    Z0P_OK = 0,
    Z0P_ERR_EMPTY_INPUT = 1,             /* Error::EmptyInput */
    Z0P_ERR_INDEX_OUT_OF_BOUNDS = 2,     /* Error::IndexOutOfBounds */
    Z0P_ERR_INVALID_DOMAIN_SIZE = 3,     /* Error::InvalidDomainSize */
    Z0P_ERR_INVALID_BLOWUP = 4,          /* Error::InvalidBlowup */
    Z0P_ERR_NO_QUERIES = 5,              /* Error::NoQueries */
    Z0P_ERR_BAD_MERKLE_PATH = 6,         /* Error::BadMerklePath */
    Z0P_ERR_FRI_VERIFICATION_FAILED = 7, /* Error::FriVerificationFailed */
    Z0P_ERR_MALFORMED_INPUT = 8,         /* Error::MalformedInput */
    Z0P_ERR_RNG_UNAVAILABLE = 9,         /* Error::RngUnavailable */
    Z0P_ERR_BUFFER_TOO_SMALL = 100,
    Z0P_ERR_CUDA = 101,
    Z0P_ERR_OUT_OF_MEMORY = 102,
    Z0P_ERR_UNSUPPORTED = 103,
    Z0P_ERR_DEVICE_TIMEOUT = 104,        /* a bounded device wait gave up */
    Z0P_ERR_ADMISSION = 105,             /* job larger than the HBM budget */
    Z0P_ERR_INVALID_ARGUMENT = 106,
    Z0P_ERR_CANCELLED = 107
};

/* air::Params (src/air.rs:31-54). usize fields are widened to uint64_t. */
typedef struct {
    uint64_t n_steps;
    uint64_t blowup;
    uint64_t num_queries;
    uint64_t final_size;
    uint32_t grinding_bits;
    uint64_t cap_height;
    uint32_t a0;
    uint32_t b0;
    uint32_t b_last;
} z0p_air_params;

/* range::Params (src/range.rs:30-51). */
typedef struct {
    uint64_t n_rows;
    uint64_t n_bits;
    uint64_t blowup;
    uint64_t num_queries;
    uint64_t final_size;
    uint32_t grinding_bits;
    uint64_t cap_height;
    uint32_t value;
} z0p_range_params;

/*
 * Transcript state (src/transcript.rs:54-57: Transcript{history: Hasher,
 * counter}; src/hash.rs:233-240: Hasher{buf[start..], stack, stack_len,
 * next_index, total_len}). `tail` holds the unprocessed history bytes
 * (always < 2048 after an absorb). Exporting a z0p Transcript into this POD
 * and importing it back after a prove call leaves it exactly where the CPU
 * prover would have left it, so proofs can be chained on one transcript.
 */
typedef struct {
    uint8_t tail[2048];
    uint32_t tail_len;
    uint8_t stack[54][32];
    uint32_t stack_len;
    uint64_t next_index;
    uint64_t total_len;
    uint64_t counter;
} z0p_transcript_state;

typedef struct z0p_gpu_ctx z0p_gpu_ctx;

/*
 * ChaCha20 stream state (src/rng.rs:81-87: key, nonce, block counter, the
 * buffered 64-byte block and how much of it is used), for the masking
 * randomness of zero-knowledge proofs. ChaCha20::new(key, nonce) is
 * {key, nonce, 0, zeros, 64}. A prove call advances it exactly as the
 * reference's prove_zk advances its `&mut ChaCha20`.
 */
typedef struct {
    uint8_t key[32];
    uint8_t nonce[12];
    uint32_t counter;
    uint8_t block[64];
    uint32_t used;
} z0p_chacha20_state;

/* ------------------------------------------------------------ misc ---- */
int z0p_gpu_abi_version(void);
const char *z0p_gpu_last_reason(void);

/* ------------------------------------------------- transcript (host) ---- */
/* Transcript::new (src/transcript.rs:62-69). */
int z0p_transcript_init(z0p_transcript_state *st, const uint8_t *label, size_t label_len);
/* Transcript::absorb (src/transcript.rs:72-77). */
int z0p_transcript_absorb(z0p_transcript_state *st, const uint8_t *label, size_t label_len,
                          const uint8_t *data, size_t data_len);
/* Transcript::challenge_bytes (src/transcript.rs:95-97 via squeeze_raw :162-171). */
int z0p_transcript_challenge_bytes(z0p_transcript_state *st, const uint8_t *label,
                                   size_t label_len, uint8_t out[32]);
/* Transcript::challenge_ext (src/transcript.rs:136-141): 4 canonical coordinates. */
int z0p_transcript_challenge_ext(z0p_transcript_state *st, const uint8_t *label,
                                 size_t label_len, uint32_t out[4]);
/* Transcript::challenge_index (src/transcript.rs:148-160); MALFORMED_INPUT
 * where the reference returns None. */
int z0p_transcript_challenge_index(z0p_transcript_state *st, const uint8_t *label,
                                   size_t label_len, uint64_t domain, uint64_t *out);

/* ------------------------------------------------------ params (host) ---- */
/* air::Params::new (src/air.rs:62-102). */
int z0p_air_params_new(uint64_t n_steps, uint64_t blowup, uint64_t num_queries,
                       uint64_t final_size, uint32_t a0, uint32_t b0, uint32_t b_last,
                       z0p_air_params *out);
/* air::Params::for_security (src/air.rs:127-158). */
int z0p_air_params_for_security(uint64_t n_steps, uint32_t a0, uint32_t b0, uint32_t b_last,
                                uint32_t target_bits, z0p_air_params *out);
/* range::Params::new (src/range.rs:57-99). */
int z0p_range_params_new(uint64_t n_rows, uint64_t n_bits, uint64_t blowup,
                         uint64_t num_queries, uint64_t final_size, uint32_t value,
                         z0p_range_params *out);
/* range::Params::for_security (src/range.rs:124-161). */
int z0p_range_params_for_security(uint64_t n_rows, uint64_t n_bits, uint32_t value,
                                  uint32_t target_bits, z0p_range_params *out);
/* Exact length of air::Proof::to_bytes (src/air.rs:262-281) for `params`. */
int z0p_air_proof_size(const z0p_air_params *params, size_t *len);
/* Exact length of range::Proof::to_bytes (src/range.rs:253-269) for `params`. */
int z0p_range_proof_size(const z0p_range_params *params, size_t *len);

/* ---------------------------------------------------------- contexts ---- */
/* Creates a prover context on CUDA device `device` (one stream, lazily grown
 * device workspace).
 * A prove call queues the small folds at the end of a FRI commitment, the PoW
 * search and the openings gather ahead of their inputs, each waiting on a
 * gate word that the calling thread opens once it has written them. The
 * gates are off (each such launch follows its inputs) when the environment
 * sets Z0P_GATES=0 or CUDA_LAUNCH_BLOCKING=1, or when a tool is injected
 * through CUDA_INJECTION64_PATH; proofs are the same bytes either way. */
int z0p_gpu_ctx_create(int device, z0p_gpu_ctx **out);
/* Gated launches on (nonzero, the default) or off for this context. On, a
 * single proof's latency is lower; off, the launches wait for their inputs
 * on the host instead of on the GPU, which suits contexts proving side by
 * side (a pool of more than one worker turns them off on its own contexts:
 * launches waiting at their gates hold SM slots the other streams could
 * use). Proofs are the same bytes either way. */
int z0p_gpu_ctx_set_gates(z0p_gpu_ctx *ctx, int on);
void z0p_gpu_ctx_destroy(z0p_gpu_ctx *ctx);
/* The context's cudaStream_t (as void*), for callers that time or order work. */
void *z0p_gpu_ctx_stream(z0p_gpu_ctx *ctx);
/* Bytes of device memory currently held by the context. */
size_t z0p_gpu_ctx_device_bytes(z0p_gpu_ctx *ctx);
/* Hands the context's proof workspace (trace, LDE, trees, FRI layers) back to
 * the library's device memory pool, queued on the context's stream; the next
 * prove call takes it again. No counterpart in the reference (its buffers are
 * per-call Vecs); a serving loop uses it to keep held memory near the sum of
 * the running jobs' footprints. */
int z0p_gpu_ctx_trim(z0p_gpu_ctx *ctx);
/* Reserves the context's per-proof constant slots for proof groups of up to
 * max_group (1..64) statements, so that later group calls neither wait for
 * nor compete for them. The process has 168 slots in all (64 KiB of constant
 * memory); every context holds at least one. Returns Z0P_ERR_OUT_OF_MEMORY
 * when no max_group free slots are contiguous: the context then keeps its
 * previous reservation, and a group call larger than the reservation is
 * proved as consecutive smaller groups. No counterpart in the reference. */
int z0p_gpu_ctx_reserve_group(z0p_gpu_ctx *ctx, uint32_t max_group);
/* Cumulative counters of a context (launches are process-wide). */
typedef struct {
    uint64_t launches;   /* kernels launched by this library in this process */
    uint64_t h2d_bytes;  /* host-to-device bytes copied by this context */
    uint64_t d2h_bytes;  /* device-to-host bytes copied by this context */
    uint64_t syncs;      /* stream synchronisations (host round trips) */
    uint64_t proofs;     /* proofs completed */
    uint64_t sync_wait_ns; /* host time blocked in those synchronisations */
    uint64_t prove_ns;     /* host wall time inside prove calls */
} z0p_gpu_stats;
int z0p_gpu_ctx_stats(z0p_gpu_ctx *ctx, z0p_gpu_stats *out);
/* Diagnostic per-stage timing: while on, every kernel stage is bracketed by
 * CUDA events on the context stream. z0p_gpu_ctx_profile writes a JSON
 * object {"stage": {"ms": total, "calls": n, "kernels": k}, ...} covering
 * the stages since the previous call (calls: bracketed stage calls; kernels:
 * kernel launches inside them), then clears it. Profiling uses a process-wide hook, so
 * only one context should profile at a time. */
int z0p_gpu_ctx_set_profiling(z0p_gpu_ctx *ctx, int on);
int z0p_gpu_ctx_profile(z0p_gpu_ctx *ctx, char *json, size_t cap, size_t *len);
/* Device bytes a proof of `params` needs (the admission footprint). */
int z0p_gpu_air_footprint(const z0p_air_params *params, size_t *bytes);
int z0p_gpu_range_footprint(const z0p_range_params *params, size_t *bytes);

/* ------------------------------------------------------------ prove ---- */
/*
 * air::prove (src/air.rs:365-372) followed by Proof::to_bytes
 * (src/air.rs:262-281). `transcript` is read and advanced exactly as the
 * reference advances its &mut Transcript.
 */
int z0p_gpu_air_prove(z0p_gpu_ctx *ctx, const z0p_air_params *params,
                      z0p_transcript_state *transcript, uint8_t *out, size_t cap,
                      size_t *len);
/* range::prove (src/range.rs:337-343) followed by Proof::to_bytes
 * (src/range.rs:253-269). range::prove's columns each repeat one value, so
 * the device builds every tree as runs of equal leaves (one chain of node
 * hashes per run) and every FRI layer as per-coset constants, with the same
 * bytes as transforming and hashing every row; shapes outside that form
 * (final layers below 4 values, or an out-of-range value with final layers
 * below the blowup or fewer than 4 rows) take the row-by-row path. */
int z0p_gpu_range_prove(z0p_gpu_ctx *ctx, const z0p_range_params *params,
                        z0p_transcript_state *transcript, uint8_t *out, size_t cap,
                        size_t *len);
/* range::prove_zk (src/range.rs:393-418): every column masked with n_rand
 * maskers drawn from `rng`, column after column (value first); the LDE runs
 * over 2^ceil(log2(n_rows + n_rand)) rows. n_rand < num_queries is
 * Z0P_ERR_MALFORMED_INPUT. On error neither the transcript nor the stream
 * moves. */
int z0p_range_proof_size_zk(const z0p_range_params *params, size_t n_rand, size_t *len);
int z0p_gpu_range_prove_zk(z0p_gpu_ctx *ctx, const z0p_range_params *params, size_t n_rand,
                           z0p_chacha20_state *rng, z0p_transcript_state *transcript,
                           uint8_t *out, size_t cap, size_t *out_len);
/* range::prove_with_columns (src/range.rs:353-375): the caller's value column
 * and n_bits bit columns, n_rows canonical words each. Any values prove
 * structurally (invalid columns fail verify). Shapes that differ from the
 * params are Z0P_ERR_MALFORMED_INPUT (after the params' own checks). */
int z0p_gpu_range_prove_with_columns(z0p_gpu_ctx *ctx, const z0p_range_params *params,
                                     const uint32_t *v_col, size_t v_len,
                                     const uint32_t *const *bit_cols, const size_t *bit_lens,
                                     size_t n_bit_cols, z0p_transcript_state *transcript,
                                     uint8_t *out, size_t cap, size_t *out_len);

/* air::prove_with_trace (src/air.rs:381-399): the caller's two columns of
 * n_steps canonical words, each interpolated and extended (no linked
 * column). Same proof length as z0p_gpu_air_prove. */
int z0p_gpu_air_prove_with_trace(z0p_gpu_ctx *ctx, const z0p_air_params *params,
                                 const uint32_t *col_a, const uint32_t *col_b, size_t len,
                                 z0p_transcript_state *transcript, uint8_t *out, size_t cap,
                                 size_t *out_len);
/* air::prove_zk (src/air.rs:439-464, masking of src/blind.rs:40-78): both
 * columns masked with n_rand values each drawn from `rng` (n_rand >= 16 *
 * num_queries); the LDE grows to the next power of two of n_steps + n_rand
 * times blowup. On error neither the transcript nor the stream changes. */
int z0p_air_proof_size_zk(const z0p_air_params *params, size_t n_rand, size_t *len);
int z0p_gpu_air_prove_zk(z0p_gpu_ctx *ctx, const z0p_air_params *params, size_t n_rand,
                         z0p_chacha20_state *rng, z0p_transcript_state *transcript, uint8_t *out,
                         size_t cap, size_t *out_len);

/* table::Params (src/table.rs:27-45): a constant column `value` proved to lie
 * in a public table of canonical entries. */
typedef struct {
    uint64_t n_rows;
    uint64_t blowup;
    uint64_t num_queries;
    uint64_t final_size;
    uint32_t grinding_bits;
    uint64_t cap_height;
    uint32_t value;
} z0p_table_params;
/* table::Params::new (src/table.rs:55-88) and ::for_security (:114-170). */
int z0p_table_params_new(uint64_t n_rows, uint64_t blowup, uint64_t num_queries,
                         uint64_t final_size, uint32_t value, z0p_table_params *out);
int z0p_table_params_for_security(uint64_t n_rows, uint64_t table_len, uint32_t value,
                                  uint32_t target_bits, z0p_table_params *out);
/* Exact length of table::Proof::to_bytes (src/table.rs:244-262); n_rand = 0
 * for table::prove. */
int z0p_table_proof_size(const z0p_table_params *params, size_t table_len, size_t n_rand,
                         size_t *len);
/* table::prove (src/table.rs:305-317) and table::prove_zk (:329-356, n_rand
 * >= num_queries maskers drawn from `rng`). */
int z0p_gpu_table_prove(z0p_gpu_ctx *ctx, const z0p_table_params *params, const uint32_t *table,
                        size_t table_len, z0p_transcript_state *transcript, uint8_t *out,
                        size_t cap, size_t *out_len);
int z0p_gpu_table_prove_zk(z0p_gpu_ctx *ctx, const z0p_table_params *params,
                           const uint32_t *table, size_t table_len, size_t n_rand,
                           z0p_chacha20_state *rng, z0p_transcript_state *transcript,
                           uint8_t *out, size_t cap, size_t *out_len);

/* Proof groups (no counterpart in the reference): n statements of one shape
 * -- the same n_steps / n_rows (and n_bits), blowup, num_queries,
 * final_size, grinding_bits and cap_height -- proved in lockstep, so each
 * kernel launch and each host round trip serves the whole group. Proof i
 * lands in outs[i] (caps[i] bytes; lens[i] receives its length when lens is
 * non-null) with transcripts[i] advanced exactly as z0p_gpu_air_prove /
 * z0p_gpu_range_prove would leave it for that statement alone; on any error
 * no transcript is changed. Groups larger than the library's group limit are
 * proved in consecutive groups. */
int z0p_gpu_air_prove_group(z0p_gpu_ctx *ctx, size_t n, const z0p_air_params *params,
                            z0p_transcript_state *const *transcripts, uint8_t *const *outs,
                            const size_t *caps, size_t *lens);
int z0p_gpu_range_prove_group(z0p_gpu_ctx *ctx, size_t n, const z0p_range_params *params,
                              z0p_transcript_state *const *transcripts, uint8_t *const *outs,
                              const size_t *caps, size_t *lens);

/* --------------------------------------- FRI as a polynomial commitment ---- */
/* fri::Params (src/fri.rs:103-126): fields and validation as the reference. */
typedef struct {
    uint64_t blowup;
    uint64_t num_queries;
    uint64_t final_size;
    uint32_t grinding_bits;
    uint64_t cap_height;
} z0p_fri_params;
/* Input forms of the commit call:
 *   Z0P_FRI_COEFFS      fri::commit            (src/fri.rs:407-433), n coefficients
 *   Z0P_FRI_COEFFS_EXT  fri::commit_ext        (src/fri.rs:443-460), n Ext4 coefficients
 *   Z0P_FRI_EVALS       fri::commit_evals      (src/fri.rs:473-499), n LDE values
 *   Z0P_FRI_EVALS_EXT   fri::commit_ext_evals  (src/fri.rs:508-549), n Ext4 LDE values
 * Ext4 values are 4 words each (coordinates a, b, c, d of a + bu + cv + duv);
 * the evaluation forms take natural-order values on the 31-coset and a
 * degree_bound (ignored by the coefficient forms, whose bound is n - 1). */
enum { Z0P_FRI_COEFFS = 0, Z0P_FRI_COEFFS_EXT = 1, Z0P_FRI_EVALS = 2, Z0P_FRI_EVALS_EXT = 3 };
/* fri::Params::for_security (src/fri.rs:232-255): blowup 16, queries and
 * grinding from the target, size-optimal final layer and cap height. */
int z0p_fri_params_for_security(uint64_t poly_len, uint32_t target_bits, z0p_fri_params *out);
/* Byte lengths of Commitment::to_bytes and Proof::to_bytes for these inputs
 * (src/fri.rs:331-336, 875-880), after the same checks as the commit call. */
int z0p_fri_sizes(const z0p_fri_params *params, int form, size_t n, uint64_t degree_bound,
                  size_t *commitment_len, size_t *proof_len);
/* Commits to host `values` and writes Commitment::to_bytes to `out` (cap
 * bytes; *len receives the length, also when cap is too small). The
 * transcript advances as the reference's commit call leaves it. Checks run
 * in the reference's order before any device work; a word >= p gives
 * Z0P_ERR_MALFORMED_INPUT. The committed layers and trees (ProverState,
 * src/fri.rs:276-295) stay on the device for z0p_gpu_fri_open until any
 * other call on this context uses its workspace. */
int z0p_gpu_fri_commit(z0p_gpu_ctx *ctx, const z0p_fri_params *params, int form,
                       const uint32_t *values, size_t n, uint64_t degree_bound,
                       z0p_transcript_state *transcript, uint8_t *out, size_t cap, size_t *len);
/* fri::open (src/fri.rs:645-666) of the context's last commitment: grinds,
 * draws the query indices (num_queries entries into `indices`, may be null)
 * and writes Proof::to_bytes. Z0P_ERR_INVALID_ARGUMENT when there is no
 * commitment to open. On error the transcript is left untouched. */
int z0p_gpu_fri_open(z0p_gpu_ctx *ctx, z0p_transcript_state *transcript, uint8_t *out, size_t cap,
                     size_t *len, uint64_t *indices);

/* -------------------------------------------------------- folded IVC ---- */
/* fold::Params (src/fold.rs:42-64): rows per segment, FRI shape, and the
 * global claims (input A, B; output B). */
typedef struct {
    uint64_t seg_steps;
    uint64_t blowup;
    uint64_t num_queries;
    uint64_t final_size;
    uint32_t grinding_bits;
    uint64_t cap_height;
    uint32_t in_a;
    uint32_t in_b;
    uint32_t out_b;
} z0p_fold_params;
/* fold::Params::new (src/fold.rs:72-111) and ::for_security (:136-171). */
int z0p_fold_params_new(uint64_t seg_steps, uint64_t blowup, uint64_t num_queries,
                        uint64_t final_size, uint32_t in_a, uint32_t in_b, uint32_t out_b,
                        z0p_fold_params *out);
int z0p_fold_params_for_security(uint64_t seg_steps, uint32_t in_a, uint32_t in_b, uint32_t out_b,
                                 uint32_t target_bits, z0p_fold_params *out);
/* fold::Accumulator (src/fold.rs:362-561) on a context: every segment's column
 * LDEs and row tree stay on the device until finalize. Calls on an
 * accumulator are serialised by its context's mutex. */
typedef struct z0p_gpu_fold z0p_gpu_fold;
int z0p_gpu_fold_create(z0p_gpu_ctx *ctx, const z0p_fold_params *params, z0p_gpu_fold **out);
void z0p_gpu_fold_destroy(z0p_gpu_fold *acc);
size_t z0p_gpu_fold_len(const z0p_gpu_fold *acc);
/* Accumulator::add_segment (src/fold.rs:407-488): columns of seg_steps
 * canonical words each; on error the transcript is left untouched. */
int z0p_gpu_fold_add_segment(z0p_gpu_fold *acc, const uint32_t *col_a, const uint32_t *col_b,
                             size_t len, z0p_transcript_state *transcript);
/* Exact length of IvcProof::to_bytes (src/fold.rs:281-309) for the segments so far. */
int z0p_gpu_fold_proof_size(const z0p_gpu_fold *acc, size_t *len);
/* Accumulator::finalize (src/fold.rs:494-561): writes IvcProof::to_bytes; the
 * accumulator accepts no further segment afterwards. */
int z0p_gpu_fold_finalize(z0p_gpu_fold *acc, z0p_transcript_state *transcript, uint8_t *out,
                          size_t cap, size_t *len);

/* ------------------------------------------------- batching / serving ---- */
/*
 * Many independent proofs (the batched and served configurations). A pool
 * owns `workers` contexts, each with its own stream and host thread, and a
 * FIFO job queue. A job starts once its device footprint
 * (z0p_gpu_*_footprint) fits the pool's HBM budget next to the jobs already
 * running. Jobs whose footprint exceeds the whole budget are rejected with
 * Z0P_ERR_ADMISSION. Proofs are deterministic: a job's bytes and transcript
 * post-state are the same alone and in any mix. The reference has no
 * counterpart: it proves one statement per call (air::prove / range::prove).
 */
enum { Z0P_JOB_AIR = 0, Z0P_JOB_RANGE = 1 };
typedef struct {
    int kind;                          /* Z0P_JOB_AIR or Z0P_JOB_RANGE */
    z0p_air_params air;                /* used when kind == Z0P_JOB_AIR */
    z0p_range_params range;            /* used when kind == Z0P_JOB_RANGE */
    z0p_transcript_state *transcript;  /* in/out, owned by the caller */
    uint8_t *out;                      /* proof bytes (caller-owned) */
    size_t cap;
    size_t len;                        /* written: proof length */
    int status;                        /* written: the prove call's status */
    double submit_s, start_s, end_s;   /* written: pool clock, seconds */
} z0p_job;
typedef struct z0p_gpu_pool z0p_gpu_pool;
/* hbm_budget = 0 means 90% of the device's free memory at creation. */
int z0p_gpu_pool_create(int device, int workers, size_t hbm_budget, z0p_gpu_pool **out);
void z0p_gpu_pool_destroy(z0p_gpu_pool *pool);
/* Queues a job (it must stay valid until it completes); *ticket identifies it. */
int z0p_gpu_pool_submit(z0p_gpu_pool *pool, z0p_job *job, uint64_t *ticket);
/* Waits up to timeout_ms (< 0: forever) for a ticket; Z0P_ERR_DEVICE_TIMEOUT
 * if it is still pending. Returns the job's status once done. */
int z0p_gpu_pool_wait(z0p_gpu_pool *pool, uint64_t ticket, int timeout_ms);
/* Proves all jobs (largest footprint first) and waits; 0 if every job returned 0. */
int z0p_gpu_pool_prove_all(z0p_gpu_pool *pool, z0p_job *jobs, size_t n);
/* Seconds on the pool's clock (the clock of the job timestamps). */
double z0p_gpu_pool_clock(z0p_gpu_pool *pool);

/* ------------------------------------------ per-stage kernels (device) ---- */
/*
 * ntt::reed_solomon_extend (src/ntt.rs:436-439) over `batch` columns of
 * length n (power of two): d_out[c*n*blowup + k] = LDE of column c at the
 * natural-order point GENERATOR * omega_{n*blowup}^k. Device pointers; runs on
 * the context stream and synchronises before returning.
 */
int z0p_gpu_rs_extend(z0p_gpu_ctx *ctx, const uint32_t *d_values, uint64_t n, uint64_t batch,
                      uint64_t blowup, uint32_t *d_out);
/*
 * Allocation-free variant of z0p_gpu_rs_extend. It has no counterpart in the
 * reference. It serves callers that may not allocate device memory: a process
 * whose device heap is owned by another allocator that must see every byte, a
 * latency-critical loop where cudaMalloc/cudaFree would synchronise the
 * device, or a deployment whose memory budget is fixed when the library loads.
 * It needs no context. It allocates nothing, and it calls no allocating
 * library routine.
 *
 * Its working memory is static device arrays inside this library: 12 MiB of
 * scratch plus 240 KiB of power tables, held on every device that loads the
 * library until the process exits.
 * - Limit: n * batch * blowup <= 1048576 output elements; larger sizes
 *   return Z0P_ERR_UNSUPPORTED. The other checks and their codes are
 *   z0p_gpu_rs_extend's (batch * blowup > 65535 is
 *   Z0P_ERR_INVALID_DOMAIN_SIZE there and here).
 * - Set-up: the first call on a device, with that device current, resolves
 *   the arrays' device addresses, uploads the tables through the legacy
 *   default stream and waits for that upload, so the first call's work is
 *   correct on any stream, non-blocking ones included. Make that first call
 *   before any stream capture.
 * - Semantics: the same output as z0p_gpu_rs_extend. The work is enqueued on
 *   `stream` (NULL = legacy default stream) and the call returns without
 *   waiting.
 * - Concurrency: every call shares the one scratch area, so calls whose work
 *   overlaps on the GPU race. Serialise them on one stream.
 */
int z0p_gpu_rs_extend_noalloc(const uint32_t *d_values, uint64_t n, uint64_t batch,
                              uint64_t blowup, uint32_t *d_out, void *stream);
/*
 * air::compose (src/air.rs:847-929) as one device stage, the composition
 * evaluation of z0p_gpu_air_prove with the caller's alphas in place of the
 * transcript's "fib/alpha" draws: the Fibonacci trace of *p (n_steps, a0, b0;
 * b_last enters the boundary term), its LDE at p->blowup and the composition
 * (src/air.rs:938-962 value by value). alphas: 5 Ext4 as 20 canonical words
 * (non-canonical: Z0P_ERR_MALFORMED_INPUT). d_out (device, 4 * m words for
 * m = n_steps * blowup) receives FRI layer 0: position P holds the value at
 * LDE row brev_{log m}(P), the point 31 * omega_m^row (src/fri.rs:584-586).
 * Parameter checks are z0p_gpu_air_prove's. Runs on the context stream and
 * synchronises before returning.
 */
int z0p_gpu_air_compose(z0p_gpu_ctx *ctx, const z0p_air_params *p, const uint32_t alphas[20],
                        uint32_t *d_out);
/*
 * MerkleTree::from_flat64 (src/merkle.rs:93-110) + cap (src/merkle.rs:229-232):
 * builds the BLAKE3 tree over len/64 64-byte leaves of the device buffer
 * d_flat, padded to a power of two by duplicating the last leaf
 * (src/merkle.rs:350-360), and copies cap level min(cap_height, depth) to
 * the host buffer h_cap (2^drop * 32 bytes; *cap_count receives the count).
 */
int z0p_gpu_merkle_flat64_cap(z0p_gpu_ctx *ctx, const uint8_t *d_flat, uint64_t len,
                              uint64_t cap_height, uint8_t *h_cap, uint64_t *cap_count);
/*
 * fri::fold_layer (src/fri.rs:1273-1302) for layer `depth` of an FRI stack
 * over an LDE of length lde_len: folds n bit-reversed Ext4 values (d_in,
 * 4*n uint32) with challenges ch[12] into n/4 values (d_out). The quad
 * leader points are derived from (lde_len, depth) exactly as fri::point_at
 * (src/fri.rs:1108-1115) defines them.
 */
int z0p_gpu_fri_fold(z0p_gpu_ctx *ctx, const uint32_t *d_in, uint64_t n, uint64_t lde_len,
                     uint64_t depth, const uint32_t ch[12], uint32_t *d_out);
/* ------------------------------------------- launch schedule autotuning ---- */
/* No counterpart in the reference (its prover has no device schedule).
 * Launch choices the kernels read, one schedule per device, process-wide.
 * Every schedule gives byte-identical proofs; only the time changes.
 *  - ntt_log_n1[l]: for a four-step NTT of length 2^l (13 <= l <= 26),
 *    log2 of the first pass's transform length, within
 *    [max(7, l - 13), min(13, l - 6)]; 0 = the balanced split ceil(l / 2).
 *    Other entries must be 0.
 *  - ntt_radix32[l]: the pass variant of the same transforms, 0 outside
 *    13 <= l <= 26. 0: shared-memory passes in register groups of 16
 *    elements (512 threads a CTA); 1: the same in groups of 32 (256
 *    threads); 2: register passes (each half of 2^L points as two register
 *    passes of radix 2^(L/2) with one shared-memory transpose, tiles loaded
 *    by TMA), used when both halves are even and within 2^6..2^12 and the
 *    input is 16-byte aligned, variant 0 otherwise; 3: the register passes
 *    streamed (a resident grid, each CTA walking many tiles through two
 *    buffers so the next tile's copy overlaps the current transform; a half
 *    above 2^10 takes variant 2's kernel), same conditions. The default schedule
 *    (z0p_schedule_default) has variant 2 at 2^16, 2^20 and 2^24, whose
 *    balanced splits have two even halves, and 0 elsewhere.
 *  - merkle_top_log: a Merkle tree's levels are one launch each while they
 *    hold more than 2^merkle_top_log nodes; one top kernel hashes the rest
 *    (10..18).
 *  - grind_ctas_per_sm: proof-of-work grid, CTAs per SM (1..16, clamped to
 *    the occupancy limit). */
typedef struct {
    uint8_t ntt_log_n1[32];
    uint8_t ntt_radix32[32];
    uint32_t merkle_top_log;
    uint32_t grind_ctas_per_sm;
} z0p_schedule;
/* What z0p_gpu_autotune measured, device time per candidate set (µs):
 * the default and the chosen schedule for each LDE transform size (16
 * cosets of 2^l; 0 where not tuned), for a 2^21-leaf Merkle tree above its
 * leaves, and for eight single 20-bit proof-of-work searches. */
typedef struct {
    float ntt_default_us[32];
    float ntt_best_us[32];
    float merkle_default_us, merkle_best_us;
    float grind_default_us, grind_best_us;
    float wall_ms;  /* tuning time, host clock */
} z0p_tune_report;
int z0p_schedule_default(z0p_schedule *out);
/* Read or replace a device's schedule; set validates every field first
 * (Z0P_ERR_INVALID_ARGUMENT, schedule unchanged). Neither touches the GPU. */
int z0p_gpu_schedule_get(int device, z0p_schedule *out);
int z0p_gpu_schedule_set(int device, const z0p_schedule *schedule);
/* Times the candidates of every field on the context's device (LDE
 * transforms up to 16 x 2^min(max_log_n, 22) points, in the context's
 * workspace), keeps a candidate only when it beats the default by 3% or
 * more, installs the result as the device's schedule and writes it to *out.
 * The proof-of-work candidates must agree on the nonce (else
 * Z0P_ERR_UNSUPPORTED). `report` may be NULL. */
int z0p_gpu_autotune(z0p_gpu_ctx *ctx, uint32_t max_log_n, z0p_schedule *out,
                     z0p_tune_report *report);

/* Diagnostic, no counterpart in the reference: the device's BLAKE3
 * throughput ceiling in G compressions/s, measured with register-resident
 * chains of Merkle-node hashes (no memory traffic). The hashing stages'
 * roofline fraction is taken against it. */
int z0p_gpu_blake3_ceiling(z0p_gpu_ctx *ctx, double *gcompress_per_s);

/*
 * Transcript::grind core (src/transcript.rs:263-281): the smallest nonce
 * whose BLAKE3(head || LE64(nonce)) has >= bits leading zero bits, MSB first.
 * head_len + 8 must fit one BLAKE3 block (head_len <= 56); bits <= 32.
 */
int z0p_gpu_grind(z0p_gpu_ctx *ctx, const uint8_t *head, size_t head_len, uint32_t bits,
                  uint64_t *nonce);

#ifdef __cplusplus
}
#endif
#endif
