/*
 * z0p CPU oracle: a plain-C restatement of the z0p STARK prove/verify path.
 *
 * TEST INFRASTRUCTURE ONLY. This library is the checker for the GPU prover
 * and the timed CPU baseline; the shipped prover never links or calls it.
 *
 * Every function restates the reference crate FutureProofsTech/z0p
 * (Rust, zero dependencies) and cites the file:line it follows.
 * Status codes mirror the reference `Error` enum (src/error.rs:7-40).
 */
#ifndef Z0P_ORACLE_H
#define Z0P_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
    ZO_OK = 0,
    ZO_EMPTY_INPUT = 1,
    ZO_INDEX_OUT_OF_BOUNDS = 2,
    ZO_INVALID_DOMAIN_SIZE = 3,
    ZO_INVALID_BLOWUP = 4,
    ZO_NO_QUERIES = 5,
    ZO_BAD_MERKLE_PATH = 6,
    ZO_FRI_VERIFICATION_FAILED = 7,
    ZO_MALFORMED_INPUT = 8,
    ZO_RNG_UNAVAILABLE = 9,
    ZO_BUFFER_TOO_SMALL = 100,
    ZO_OUT_OF_MEMORY = 101
};

/* Field (src/babybear.rs) */
uint32_t zo_f_mul(uint32_t a, uint32_t b);
uint32_t zo_f_pow(uint32_t a, uint64_t e);
uint32_t zo_f_inv(uint32_t a);
uint32_t zo_f_from_u64(uint64_t v);
void zo_batch_invert(uint32_t *values, size_t n);
uint64_t zo_splitmix64(uint64_t *state);

/* Ext4 (src/ext4.rs): 4 coordinates a + b u + c v + d uv */
void zo_e_mul(const uint32_t a[4], const uint32_t b[4], uint32_t out[4]);
void zo_e_inv(const uint32_t a[4], uint32_t out[4]);

/* BLAKE3 (src/hash.rs) */
void zo_blake3(const uint8_t *data, size_t len, uint8_t out[32]);
void zo_leaf64_digest(const uint8_t block[64], uint8_t out[32]);
void zo_node_digest(const uint8_t left[32], const uint8_t right[32], uint8_t out[32]);
void zo_leaf_digest(const uint8_t *data, size_t len, uint8_t out[32]);

/* Transcript (src/transcript.rs). Opaque handle. */
typedef struct zo_transcript zo_transcript;
zo_transcript *zo_transcript_new(const uint8_t *label, size_t len);
zo_transcript *zo_transcript_clone(const zo_transcript *t);
void zo_transcript_free(zo_transcript *t);
void zo_transcript_absorb(zo_transcript *t, const uint8_t *label, size_t llen,
                          const uint8_t *data, size_t dlen);
void zo_transcript_challenge_bytes(zo_transcript *t, const uint8_t *label, size_t llen,
                                   uint8_t out[32]);
void zo_transcript_challenge_ext(zo_transcript *t, const uint8_t *label, size_t llen,
                                 uint32_t out[4]);
/* Returns 0 and writes *out, or -1 for a non-power-of-two / zero domain. */
int zo_transcript_challenge_index(zo_transcript *t, const uint8_t *label, size_t llen,
                                  uint64_t domain, uint64_t *out);
uint64_t zo_transcript_grind(zo_transcript *t, const uint8_t *label, size_t llen,
                             uint32_t bits);
int zo_transcript_verify_grind(zo_transcript *t, const uint8_t *label, size_t llen,
                               uint64_t nonce, uint32_t bits);
/* Serialises the streaming state in the layout of z0p_transcript_state
 * (include/z0p_gpu.h) so GPU-side transcripts can be compared. */
void zo_transcript_export(const zo_transcript *t, uint8_t *tail, uint32_t *tail_len,
                          uint8_t stack[54][32], uint32_t *stack_len, uint64_t *next_index,
                          uint64_t *total_len, uint64_t *counter);

/* NTT (src/ntt.rs) */
int zo_ntt_forward(uint32_t *values, size_t n);
int zo_ntt_inverse(uint32_t *values, size_t n);
int zo_evaluate_on_coset(const uint32_t *coeffs, size_t n, size_t blowup, uint32_t shift,
                         uint32_t *out);

/* Merkle (src/merkle.rs): roots / caps of a tree built over flat leaves. */
int zo_merkle_flat64_cap(const uint8_t *flat, size_t len, size_t cap_height,
                         uint8_t *cap_out, size_t *cap_count);
int zo_merkle_flat_cap(const uint8_t *flat, size_t len, size_t leaf_len, size_t cap_height,
                       uint8_t *cap_out, size_t *cap_count);

/* FRI pieces (src/fri.rs) */
void zo_fold_values(const uint32_t quad[16], uint32_t inv_point, const uint32_t ch[12],
                    uint32_t unit, uint32_t out[4]);
void zo_fri_tune_shape(size_t lde_len, size_t num_queries, size_t col_lde,
                       size_t col_value_bytes, int has_column, size_t *final_size,
                       size_t *cap_height);
void zo_fri_tune_strength(uint32_t target_bits, uint32_t millibits, size_t *queries,
                          uint32_t *grinding);
uint32_t zo_fri_composition_millibits(size_t lde_len, size_t degree_bound);

/* AIR (src/air.rs) */
typedef struct {
    uint64_t n_steps;
    uint64_t blowup;
    uint64_t num_queries;
    uint64_t final_size;
    uint32_t grinding_bits;
    uint64_t cap_height;
    uint32_t a0, b0, b_last;
} zo_air_params;

int zo_air_params_new(uint64_t n_steps, uint64_t blowup, uint64_t num_queries,
                      uint64_t final_size, uint32_t a0, uint32_t b0, uint32_t b_last,
                      zo_air_params *out);
int zo_air_for_security(uint64_t n_steps, uint32_t a0, uint32_t b0, uint32_t b_last,
                        uint32_t target_bits, zo_air_params *out);
void zo_air_build_trace(uint32_t a0, uint32_t b0, size_t n, uint32_t *a, uint32_t *b);
/* Proves; writes the VERSION=6 proof bytes (malloc'd, caller frees with zo_free). */
int zo_air_prove(const zo_air_params *params, zo_transcript *t, uint8_t **proof,
                 size_t *proof_len);
/* Proves from explicit trace columns (air::prove_with_trace). */
int zo_air_prove_with_trace(const zo_air_params *params, const uint32_t *col_a,
                            const uint32_t *col_b, zo_transcript *t, uint8_t **proof,
                            size_t *proof_len);
int zo_air_verify(const zo_air_params *params, const uint8_t *proof, size_t proof_len,
                  zo_transcript *t);
/* air::compose over caller-chosen points (alphas: 5 Ext4 as 20 words; out:
 * m Ext4) and air::composition_at at one point (out: 4 words). */
int zo_air_compose(const uint32_t *ca, const uint32_t *cb, const uint32_t *pts, size_t m,
                   uint32_t w_last, uint32_t a0, uint32_t b0, uint32_t b_last, size_t n,
                   size_t offset, const uint32_t *alphas, uint32_t *out);
void zo_air_composition_at(uint32_t a, uint32_t b, uint32_t an, uint32_t bn, uint32_t x,
                           uint32_t w_last, uint32_t a0, uint32_t b0, uint32_t b_last, size_t n,
                           const uint32_t *alphas, uint32_t *out);

/* Range AIR (src/range.rs) */
typedef struct {
    uint64_t n_rows;
    uint64_t n_bits;
    uint64_t blowup;
    uint64_t num_queries;
    uint64_t final_size;
    uint32_t grinding_bits;
    uint64_t cap_height;
    uint32_t value;
} zo_range_params;

int zo_range_params_new(uint64_t n_rows, uint64_t n_bits, uint64_t blowup,
                        uint64_t num_queries, uint64_t final_size, uint32_t value,
                        zo_range_params *out);
int zo_range_for_security(uint64_t n_rows, uint64_t n_bits, uint32_t value,
                          uint32_t target_bits, zo_range_params *out);
int zo_range_prove_with_columns(const zo_range_params *params, const uint32_t *cols,
                                zo_transcript *t, uint8_t **proof, size_t *proof_len);
int zo_range_prove(const zo_range_params *params, zo_transcript *t, uint8_t **proof,
                   size_t *proof_len);
int zo_range_verify(const zo_range_params *params, const uint8_t *proof, size_t proof_len,
                    zo_transcript *t);

/* Kernel-sweep helper: LDE := reed_solomon_extend(values, blowup) (ntt.rs:436-439). */
int zo_reed_solomon_extend(const uint32_t *values, size_t n, size_t blowup, uint32_t *out);
/* Kernel-sweep helper: one FRI fold over bit-reversed Ext4 values with first points. */
void zo_fold_layer(const uint32_t *values, size_t n, const uint32_t *first_points,
                   const uint32_t ch[12], uint32_t *out_values, uint32_t *out_points);

/* FRI as a polynomial commitment (src/fri.rs:400-858): commit to
 * coefficients or LDE evaluations (base field, or Ext4 as 4 coordinates per
 * value), open, verify. The state handle holds the layers and trees. */
typedef struct {
    uint64_t blowup, num_queries, final_size;
    uint32_t grinding_bits;
    uint64_t cap_height;
} zo_fri_params;
enum { ZO_FRI_COEFFS = 0, ZO_FRI_COEFFS_EXT = 1, ZO_FRI_EVALS = 2, ZO_FRI_EVALS_EXT = 3 };
int zo_fri_commit(const zo_fri_params *params, int form, const uint32_t *values, size_t n,
                  uint64_t degree_bound, zo_transcript *t, void **state, uint8_t **commitment,
                  size_t *commitment_len);
int zo_fri_open(void *state, zo_transcript *t, uint8_t **proof, size_t *proof_len,
                uint64_t *indices);
void zo_fri_state_free(void *state);
int zo_fri_verify(const zo_fri_params *params, const uint8_t *commitment, size_t commitment_len,
                  const uint8_t *proof, size_t proof_len, zo_transcript *t, uint64_t *indices);

/* fold.rs: hash-chained Fibonacci segments plus one batched FRI (IVC).
 * The accumulator handle holds every segment's LDEs, tree and composition. */
typedef struct {
    uint64_t seg_steps, blowup, num_queries, final_size;
    uint32_t grinding_bits;
    uint64_t cap_height;
    uint32_t in_a, in_b, out_b;
} zo_fold_params;
int zo_fold_params_new(uint64_t seg_steps, uint64_t blowup, uint64_t num_queries,
                       uint64_t final_size, uint32_t in_a, uint32_t in_b, uint32_t out_b,
                       zo_fold_params *out);
int zo_fold_for_security(uint64_t seg_steps, uint32_t in_a, uint32_t in_b, uint32_t out_b,
                         uint32_t target_bits, zo_fold_params *out);
void *zo_fold_new(const zo_fold_params *params);
int zo_fold_add_segment(void *acc, const uint32_t *col_a, const uint32_t *col_b, size_t len,
                        zo_transcript *t);
int zo_fold_finalize(void *acc, zo_transcript *t, uint8_t **proof, size_t *proof_len);
void zo_fold_free(void *acc);
int zo_fold_verify(const zo_fold_params *params, const uint8_t *proof, size_t proof_len,
                   zo_transcript *t);

/* ChaCha20 stream (src/rng.rs, RFC 8439) and the zero-knowledge AIR prover
 * (src/air.rs:439-464 with src/blind.rs:40-78). The state layout is the
 * reference's fields, in order. */
typedef struct {
    uint8_t key[32];
    uint8_t nonce[12];
    uint32_t counter;
    uint8_t block[64];
    uint32_t used;
} zo_chacha20;
void zo_chacha20_block(const uint8_t key[32], uint32_t counter, const uint8_t nonce[12],
                       uint8_t out[64]);
void zo_chacha20_init(zo_chacha20 *s, const uint8_t key[32], const uint8_t nonce[12]);
void zo_chacha20_fill(zo_chacha20 *s, uint8_t *out, size_t n);
int zo_range_prove_zk(const zo_range_params *params, size_t n_rand, zo_chacha20 *rng,
                      zo_transcript *t, uint8_t **proof, size_t *proof_len);
uint32_t zo_chacha20_next_field(zo_chacha20 *s);
int zo_air_prove_zk(const zo_air_params *params, size_t n_rand, zo_chacha20 *rng,
                    zo_transcript *t, uint8_t **proof, size_t *proof_len);

/* table.rs: membership of a committed constant value in a public table. */
typedef struct {
    uint64_t n_rows, blowup, num_queries, final_size;
    uint32_t grinding_bits;
    uint64_t cap_height;
    uint32_t value;
} zo_table_params;
int zo_table_params_new(uint64_t n_rows, uint64_t blowup, uint64_t num_queries,
                        uint64_t final_size, uint32_t value, zo_table_params *out);
int zo_table_for_security(uint64_t n_rows, uint64_t table_len, uint32_t value,
                          uint32_t target_bits, zo_table_params *out);
int zo_table_prove(const zo_table_params *params, const uint32_t *table, size_t table_len,
                   zo_transcript *t, uint8_t **proof, size_t *proof_len);
int zo_table_prove_zk(const zo_table_params *params, const uint32_t *table, size_t table_len,
                      size_t n_rand, zo_chacha20 *rng, zo_transcript *t, uint8_t **proof,
                      size_t *proof_len);
int zo_table_verify(const zo_table_params *params, const uint32_t *table, size_t table_len,
                    const uint8_t *proof, size_t proof_len, zo_transcript *t);

void zo_free(void *p);
/* Worker-thread cap for the parallel paths (0 = all online cores). */
void zo_set_max_workers(size_t workers);
size_t zo_max_workers(void);

#ifdef __cplusplus
}
#endif
#endif
