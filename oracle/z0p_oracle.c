/*
 * z0p CPU oracle — TEST INFRASTRUCTURE, not the product.
 *
 * A plain-C restatement of the z0p (FutureProofsTech/z0p, pure Rust) STARK
 * prove/verify path: BabyBear + Fp4 arithmetic, BLAKE3 and its streaming
 * hasher, the Fiat-Shamir transcript and proof-of-work grind, Merkle trees
 * with caps, the radix-2 NTT and coset LDE, FRI commit/open/verify, the
 * Fibonacci AIR and the range-check AIR, and the VERSION=6 wire codec.
 *
 * Only tests, the smoke check and the CPU-baseline leg of the benchmark load
 * it. The parallel structure follows src/par.rs (std::thread::scope over
 * disjoint chunks with the same per-call thresholds) so its timings are a
 * fair stand-in for the reference's multithreaded CPU prover.
 */
#define _GNU_SOURCE
#include "z0p_oracle.h"

#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>

/* ------------------------------------------------------------------------ */
/* par.rs:17-56 — worker counts and chunked parallel loops                   */
/* ------------------------------------------------------------------------ */

static size_t g_max_workers = 0;

void zo_set_max_workers(size_t workers) { g_max_workers = workers; }

size_t zo_max_workers(void) {
    if (g_max_workers) return g_max_workers;
    long n = sysconf(_SC_NPROCESSORS_ONLN);
    return n > 0 ? (size_t)n : 1;
}

/* par.rs:30-34 */
static size_t worker_count(size_t units, size_t min_per_thread) {
    size_t floor = min_per_thread ? min_per_thread : 1;
    size_t by_work = units / floor;
    size_t w = by_work < zo_max_workers() ? by_work : zo_max_workers();
    if (w < 1) w = 1;
    size_t cap = units ? units : 1;
    return w < cap ? w : cap;
}

typedef void (*par_fn)(void *ctx, size_t base, size_t len);
typedef struct { par_fn fn; void *ctx; size_t base, len; } par_job;

static void *par_trampoline(void *arg) {
    par_job *j = (par_job *)arg;
    j->fn(j->ctx, j->base, j->len);
    return NULL;
}

/* Runs fn over `workers` disjoint chunks of [0, n) (one thread each). */
static void par_chunks(size_t n, size_t workers, par_fn fn, void *ctx) {
    if (workers <= 1 || n == 0) { fn(ctx, 0, n); return; }
    size_t chunk = (n + workers - 1) / workers;
    size_t count = (n + chunk - 1) / chunk;
    pthread_t *th = malloc(count * sizeof(pthread_t));
    par_job *jobs = malloc(count * sizeof(par_job));
    for (size_t k = 0; k < count; k++) {
        jobs[k].fn = fn; jobs[k].ctx = ctx; jobs[k].base = k * chunk;
        jobs[k].len = (k + 1) * chunk > n ? n - k * chunk : chunk;
        pthread_create(&th[k], NULL, par_trampoline, &jobs[k]);
    }
    for (size_t k = 0; k < count; k++) pthread_join(th[k], NULL);
    free(th); free(jobs);
}

/* par.rs:38-56 for_each_indexed */
static void for_each_indexed(size_t n, size_t min_chunk, par_fn fn, void *ctx) {
    par_chunks(n, worker_count(n, min_chunk), fn, ctx);
}

void zo_free(void *p) { free(p); }

/* ------------------------------------------------------------------------ */
/* babybear.rs — p = 2^31 - 2^27 + 1                                         */
/* ------------------------------------------------------------------------ */

#define P 2013265921u
#define TWO_ADICITY 27u
#define GENERATOR 31u

static inline uint32_t f_add(uint32_t a, uint32_t b) {  /* :75-84 */
    uint32_t s = a + b;
    return s >= P ? s - P : s;
}
static inline uint32_t f_sub(uint32_t a, uint32_t b) {  /* :89-96 */
    return a >= b ? a - b : P - (b - a);
}
static inline uint32_t f_neg(uint32_t a) { return a ? P - a : 0; } /* :101-107 */

/* babybear.rs:121-131 Barrett multiply with MU = floor(2^64 / p). */
static inline uint32_t f_mul(uint32_t a, uint32_t b) {
    const uint64_t MU = 9162596893ull;
    uint64_t x = (uint64_t)a * b;
    uint64_t q = ((x >> 32) * MU) >> 32;
    uint64_t r = x - q * (uint64_t)P;
    while (r >= P) r -= P;
    return (uint32_t)r;
}
uint32_t zo_f_mul(uint32_t a, uint32_t b) { return f_mul(a, b); }

/* babybear.rs:147-158 */
static uint32_t f_pow(uint32_t base, uint64_t exp) {
    uint32_t acc = 1;
    while (exp > 0) {
        if (exp & 1) acc = f_mul(acc, base);
        base = f_mul(base, base);
        exp >>= 1;
    }
    return acc;
}
uint32_t zo_f_pow(uint32_t a, uint64_t e) { return f_pow(a, e); }
/* babybear.rs:167-169 Fermat inverse, zero maps to zero. */
static uint32_t f_inv(uint32_t a) { return f_pow(a, P - 2); }
uint32_t zo_f_inv(uint32_t a) { return f_inv(a); }
/* babybear.rs:173-177 */
static inline uint32_t f_halve(uint32_t a) { return (a + (a & 1) * P) >> 1; }
/* babybear.rs:66-69 */
static inline uint32_t f_from_u64(uint64_t v) { return (uint32_t)(v % P); }
uint32_t zo_f_from_u64(uint64_t v) { return f_from_u64(v); }

/* babybear.rs:183-193 */
static int two_adic_generator(uint32_t bits, uint32_t *out) {
    if (bits > TWO_ADICITY) return ZO_INVALID_DOMAIN_SIZE;
    *out = f_pow(GENERATOR, ((uint64_t)(P - 1)) >> bits);
    return ZO_OK;
}
static int is_pow2(uint64_t x) { return x && !(x & (x - 1)); }
static uint32_t log2u(uint64_t x) { return (uint32_t)__builtin_ctzll(x); }
/* babybear.rs:200-208 */
static int primitive_root(uint64_t size, uint32_t *out) {
    if (!is_pow2(size)) return ZO_INVALID_DOMAIN_SIZE;
    uint32_t bits = log2u(size);
    if (bits > TWO_ADICITY) return ZO_INVALID_DOMAIN_SIZE;
    return two_adic_generator(bits, out);
}

/* babybear.rs:307-331 Montgomery-trick batch inversion; zeros stay zero. */
void zo_batch_invert(uint32_t *values, size_t n) {
    if (n == 0) return;
    uint32_t *prefix = malloc(n * sizeof(uint32_t));
    uint32_t acc = 1;
    for (size_t i = 0; i < n; i++) {
        if (values[i] != 0) acc = f_mul(acc, values[i]);
        prefix[i] = acc;
    }
    uint32_t suffix = f_inv(acc);
    for (size_t i = n; i-- > 0;) {
        uint32_t v = values[i];
        if (v == 0) continue;
        uint32_t before = i == 0 ? 1 : prefix[i - 1];
        values[i] = f_mul(before, suffix);
        suffix = f_mul(suffix, v);
    }
    free(prefix);
}

/* gf2.rs:425-431 */
uint64_t zo_splitmix64(uint64_t *state) {
    *state += 0x9E3779B97F4A7C15ull;
    uint64_t z = *state;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

/* ------------------------------------------------------------------------ */
/* ext4.rs — Fp4 = Fp2[v]/(v^2 - u), Fp2 = Fp[u]/(u^2 - 11)                  */
/* ------------------------------------------------------------------------ */

typedef struct { uint32_t c[4]; } ext4;
#define NONRESIDUE 11u

static inline ext4 e_from_base(uint32_t a) { ext4 r = {{a, 0, 0, 0}}; return r; }
static inline ext4 e_add(ext4 a, ext4 b) {
    ext4 r; for (int i = 0; i < 4; i++) r.c[i] = f_add(a.c[i], b.c[i]); return r;
}
static inline ext4 e_sub(ext4 a, ext4 b) {
    ext4 r; for (int i = 0; i < 4; i++) r.c[i] = f_sub(a.c[i], b.c[i]); return r;
}
static inline ext4 e_halve(ext4 a) {
    ext4 r; for (int i = 0; i < 4; i++) r.c[i] = f_halve(a.c[i]); return r;
}
static inline ext4 e_mul_base(ext4 a, uint32_t s) {  /* ext4.rs:121-123 */
    ext4 r; for (int i = 0; i < 4; i++) r.c[i] = f_mul(a.c[i], s); return r;
}
static inline int e_eq(ext4 a, ext4 b) { return memcmp(&a, &b, sizeof a) == 0; }
static inline int e_is_zero(ext4 a) { return !(a.c[0] | a.c[1] | a.c[2] | a.c[3]); }

/* ext4.rs:189-194 */
static inline void fp2_mul(const uint32_t x[2], const uint32_t y[2], uint32_t o[2]) {
    uint32_t real = f_mul(x[0], y[0]);
    uint32_t imag = f_mul(x[1], y[1]);
    uint32_t cross = f_sub(f_sub(f_mul(f_add(x[0], x[1]), f_add(y[0], y[1])), real), imag);
    o[0] = f_add(real, f_mul(imag, NONRESIDUE));
    o[1] = cross;
}

/* ext4.rs:106-117 Karatsuba tower multiply */
static ext4 e_mul(ext4 s, ext4 o) {
    uint32_t a[2] = {s.c[0], s.c[1]}, b[2] = {o.c[0], o.c[1]};
    uint32_t c[2] = {s.c[2], s.c[3]}, d[2] = {o.c[2], o.c[3]};
    uint32_t ac[2], bd[2], t[2];
    fp2_mul(a, b, ac);
    fp2_mul(c, d, bd);
    uint32_t apc[2] = {f_add(a[0], c[0]), f_add(a[1], c[1])};
    uint32_t bpd[2] = {f_add(b[0], d[0]), f_add(b[1], d[1])};
    fp2_mul(apc, bpd, t);
    uint32_t cross0 = f_sub(f_sub(t[0], ac[0]), bd[0]);
    uint32_t cross1 = f_sub(f_sub(t[1], ac[1]), bd[1]);
    uint32_t bdu0 = f_mul(bd[1], NONRESIDUE), bdu1 = bd[0];
    ext4 r = {{f_add(ac[0], bdu0), f_add(ac[1], bdu1), cross0, cross1}};
    return r;
}
void zo_e_mul(const uint32_t a[4], const uint32_t b[4], uint32_t out[4]) {
    ext4 x, y; memcpy(x.c, a, 16); memcpy(y.c, b, 16);
    ext4 r = e_mul(x, y); memcpy(out, r.c, 16);
}

/* ext4.rs:155-165 tower-norm inverse (0 -> 0) */
static ext4 e_inv(ext4 s) {
    uint32_t c[2] = {s.c[0], s.c[1]}, d[2] = {s.c[2], s.c[3]};
    uint32_t cc[2], dd[2];
    fp2_mul(c, c, cc);
    fp2_mul(d, d, dd);
    uint32_t ddu[2] = {f_mul(dd[1], NONRESIDUE), dd[0]};
    uint32_t norm[2] = {f_sub(cc[0], ddu[0]), f_sub(cc[1], ddu[1])};
    /* fp2_inv, ext4.rs:215-220 */
    uint32_t n2 = f_sub(f_mul(norm[0], norm[0]), f_mul(f_mul(NONRESIDUE, norm[1]), norm[1]));
    uint32_t n2i = f_inv(n2);
    uint32_t ninv[2] = {f_mul(norm[0], n2i), f_mul(f_neg(norm[1]), n2i)};
    uint32_t re[2], im[2];
    fp2_mul(c, ninv, re);
    fp2_mul(d, ninv, im);
    ext4 r = {{re[0], re[1], f_neg(im[0]), f_neg(im[1])}};
    return r;
}
void zo_e_inv(const uint32_t a[4], uint32_t out[4]) {
    ext4 x; memcpy(x.c, a, 16); ext4 r = e_inv(x); memcpy(out, r.c, 16);
}

static inline void put_u32(uint8_t *p, uint32_t v) {
    p[0] = (uint8_t)v; p[1] = (uint8_t)(v >> 8); p[2] = (uint8_t)(v >> 16); p[3] = (uint8_t)(v >> 24);
}
static inline void put_u64(uint8_t *p, uint64_t v) {
    for (int i = 0; i < 8; i++) p[i] = (uint8_t)(v >> (8 * i));
}
static inline uint32_t get_u32(const uint8_t *p) {
    return (uint32_t)p[0] | ((uint32_t)p[1] << 8) | ((uint32_t)p[2] << 16) | ((uint32_t)p[3] << 24);
}
static inline uint64_t get_u64(const uint8_t *p) {
    uint64_t v = 0;
    for (int i = 0; i < 8; i++) v |= (uint64_t)p[i] << (8 * i);
    return v;
}
/* ext4.rs:169-175 */
static inline void e_to_bytes(ext4 a, uint8_t out[16]) {
    for (int i = 0; i < 4; i++) put_u32(out + 4 * i, a.c[i]);
}

/* ------------------------------------------------------------------------ */
/* hash.rs — BLAKE3-256 (unkeyed) from the specification                     */
/* ------------------------------------------------------------------------ */

static const uint32_t IV[8] = {0x6A09E667u, 0xBB67AE85u, 0x3C6EF372u, 0xA54FF53Au,
                               0x510E527Fu, 0x9B05688Cu, 0x1F83D9ABu, 0x5BE0CD19u};
static const int PERM[16] = {2, 6, 3, 10, 7, 0, 4, 13, 1, 11, 12, 5, 9, 14, 15, 8};
enum { CHUNK_START = 1, CHUNK_END = 2, PARENT = 4, ROOT = 8 };
#define CHUNK_LEN 1024
#define MAX_STACK 54

static inline uint32_t rotr(uint32_t x, int n) { return (x >> n) | (x << (32 - n)); }

/* hash.rs:47-80 */
static inline void g_mix(uint32_t s[16], int a, int b, int c, int d, uint32_t x, uint32_t y) {
    s[a] = s[a] + s[b] + x; s[d] = rotr(s[d] ^ s[a], 16);
    s[c] = s[c] + s[d];     s[b] = rotr(s[b] ^ s[c], 12);
    s[a] = s[a] + s[b] + y; s[d] = rotr(s[d] ^ s[a], 8);
    s[c] = s[c] + s[d];     s[b] = rotr(s[b] ^ s[c], 7);
}

/* hash.rs:93-133 */
static void compress(const uint32_t cv[8], const uint32_t block[16], uint64_t counter,
                     uint32_t block_len, uint32_t flags, uint32_t out[16]) {
    uint32_t s[16], m[16], t[16];
    memcpy(s, cv, 32);
    memcpy(s + 8, IV, 16);
    s[12] = (uint32_t)counter; s[13] = (uint32_t)(counter >> 32);
    s[14] = block_len; s[15] = flags;
    memcpy(m, block, 64);
    for (int r = 0; r < 7; r++) {
        g_mix(s, 0, 4, 8, 12, m[0], m[1]);
        g_mix(s, 1, 5, 9, 13, m[2], m[3]);
        g_mix(s, 2, 6, 10, 14, m[4], m[5]);
        g_mix(s, 3, 7, 11, 15, m[6], m[7]);
        g_mix(s, 0, 5, 10, 15, m[8], m[9]);
        g_mix(s, 1, 6, 11, 12, m[10], m[11]);
        g_mix(s, 2, 7, 8, 13, m[12], m[13]);
        g_mix(s, 3, 4, 9, 14, m[14], m[15]);
        if (r < 6) {
            for (int i = 0; i < 16; i++) t[i] = m[PERM[i]];
            memcpy(m, t, 64);
        }
    }
    for (int i = 0; i < 8; i++) { s[i] ^= s[i + 8]; s[i + 8] ^= cv[i]; }
    memcpy(out, s, 64);
}

static void words_from_bytes(const uint8_t *b, size_t len, uint32_t w[16]) {
    uint8_t blk[64] = {0};
    memcpy(blk, b, len);
    for (int i = 0; i < 16; i++) w[i] = get_u32(blk + 4 * i);
}
static void cv_bytes(const uint32_t *words, uint8_t out[32]) {
    for (int i = 0; i < 8; i++) put_u32(out + 4 * i, words[i]);
}

/* hash.rs:151-182 parent chaining value / root */
static void parent_digest(const uint8_t l[32], const uint8_t r[32], uint32_t flags,
                          uint8_t out[32]) {
    uint8_t blk[64];
    memcpy(blk, l, 32); memcpy(blk + 32, r, 32);
    uint32_t w[16], o[16];
    words_from_bytes(blk, 64, w);
    compress(IV, w, 0, 64, flags, o);
    cv_bytes(o, out);
}

/* hash.rs:186-225 chunk_output over 1..=16 blocks */
static void chunk_output(const uint8_t *data, size_t len, uint64_t counter, int root,
                         uint8_t out[32]) {
    uint32_t cv[8], w[16], o[16];
    memcpy(cv, IV, 32);
    size_t blocks = (len + 63) / 64;
    for (size_t i = 0; i < blocks; i++) {
        size_t bl = (i + 1 == blocks) ? len - 64 * i : 64;
        words_from_bytes(data + 64 * i, bl, w);
        uint32_t flags = 0;
        if (i == 0) flags |= CHUNK_START;
        if (i + 1 == blocks) { flags |= CHUNK_END; if (root) flags |= ROOT; }
        compress(cv, w, counter, (uint32_t)bl, flags, o);
        memcpy(cv, o, 32);
    }
    cv_bytes(cv, out);
}

/* hash.rs:233-324 streaming Hasher */
typedef struct {
    uint8_t *buf; size_t len, cap, start;
    uint8_t stack[MAX_STACK][32];
    size_t stack_len;
    uint64_t next_index;
    uint64_t total_len;
} hasher;

static void hasher_init(hasher *h) { memset(h, 0, sizeof *h); }
static void hasher_free(hasher *h) { free(h->buf); h->buf = NULL; }
static void hasher_clone(hasher *dst, const hasher *src) {
    *dst = *src;
    size_t tail = src->len - src->start;
    dst->buf = malloc(tail ? tail : 1);
    memcpy(dst->buf, src->buf + src->start, tail);
    dst->len = tail; dst->cap = tail ? tail : 1; dst->start = 0;
}

/* hash.rs:305-318 */
static void push_merged(hasher *h, const uint8_t cv[32]) {
    memcpy(h->stack[h->stack_len++], cv, 32);
    h->next_index++;
    uint64_t total = h->next_index;
    while (total % 2 == 0) {
        uint8_t merged[32];
        parent_digest(h->stack[h->stack_len - 2], h->stack[h->stack_len - 1], PARENT, merged);
        h->stack_len -= 2;
        memcpy(h->stack[h->stack_len++], merged, 32);
        total /= 2;
    }
}

/* hash.rs:256-272 */
static void hasher_update(hasher *h, const uint8_t *in, size_t n) {
    h->total_len += n;
    if (h->len + n > h->cap) {
        size_t nc = h->cap ? h->cap * 2 : 256;
        while (nc < h->len + n) nc *= 2;
        h->buf = realloc(h->buf, nc); h->cap = nc;
    }
    memcpy(h->buf + h->len, in, n);
    h->len += n;
    while (h->len - h->start >= 2 * CHUNK_LEN) {
        uint8_t cv[32];
        chunk_output(h->buf + h->start, CHUNK_LEN, h->next_index, 0, cv);
        push_merged(h, cv);
        h->start += CHUNK_LEN;
    }
    if (h->start >= 65536) {
        memmove(h->buf, h->buf + h->start, h->len - h->start);
        h->len -= h->start; h->start = 0;
    }
}

/* hash.rs:276-302; non-consuming (works on a private copy of the tail). */
static void hasher_finalize(const hasher *src, uint8_t out[32]) {
    if (src->total_len == 0) {
        uint32_t w[16] = {0}, o[16];
        compress(IV, w, 0, 0, CHUNK_START | CHUNK_END | ROOT, o);
        cv_bytes(o, out);
        return;
    }
    hasher h; hasher_clone(&h, src);
    size_t tail = h.len - h.start;
    if (tail > CHUNK_LEN) {
        uint8_t cv[32];
        chunk_output(h.buf + h.start, CHUNK_LEN, h.next_index, 0, cv);
        push_merged(&h, cv);
        h.start += CHUNK_LEN;
    }
    const uint8_t *partial = h.buf + h.start;
    size_t plen = h.len - h.start;
    if (h.stack_len == 0) {
        chunk_output(partial, plen, h.next_index, 1, out);
        hasher_free(&h);
        return;
    }
    uint8_t cur[32];
    chunk_output(partial, plen, h.next_index, 0, cur);
    for (size_t i = h.stack_len - 1; i >= 1; i--) {
        uint8_t nx[32];
        parent_digest(h.stack[i], cur, PARENT, nx);
        memcpy(cur, nx, 32);
    }
    parent_digest(h.stack[0], cur, PARENT | ROOT, out);
    hasher_free(&h);
}

void zo_blake3(const uint8_t *data, size_t len, uint8_t out[32]) {  /* hash.rs:334-338 */
    hasher h; hasher_init(&h);
    hasher_update(&h, data, len);
    hasher_finalize(&h, out);
    hasher_free(&h);
}

/* hash.rs:692-707 single-chunk fast path (same digest as zo_blake3) */
static void blake3_small(const uint8_t *data, size_t len, uint8_t out[32]) {
    if (len == 0 || len > CHUNK_LEN) { zo_blake3(data, len, out); return; }
    chunk_output(data, len, 0, 1, out);
}

/* hash.rs:388-397 */
void zo_leaf64_digest(const uint8_t block[64], uint8_t out[32]) {
    uint32_t w[16], o[16];
    words_from_bytes(block, 64, w);
    compress(IV, w, 0, 64, CHUNK_START | CHUNK_END | ROOT, o);
    cv_bytes(o, out);
}

/* hash.rs:417-443 node = BLAKE3(0x01 || l || r) */
void zo_node_digest(const uint8_t l[32], const uint8_t r[32], uint8_t out[32]) {
    uint8_t pre[65];
    pre[0] = 0x01; memcpy(pre + 1, l, 32); memcpy(pre + 33, r, 32);
    chunk_output(pre, 65, 0, 1, out);
}

/* hash.rs:351-381 leaf = BLAKE3(0x00 || data) */
void zo_leaf_digest(const uint8_t *data, size_t len, uint8_t out[32]) {
    uint8_t stackbuf[CHUNK_LEN + 1];
    uint8_t *pre = len < CHUNK_LEN ? stackbuf : malloc(len + 1);
    pre[0] = 0x00; memcpy(pre + 1, data, len);
    blake3_small(pre, len + 1, out);
    if (pre != stackbuf) free(pre);
}

/* ------------------------------------------------------------------------ */
/* transcript.rs — Fiat-Shamir over streaming BLAKE3                         */
/* ------------------------------------------------------------------------ */

struct zo_transcript { hasher h; uint64_t counter; };

/* transcript.rs:72-77 */
void zo_transcript_absorb(zo_transcript *t, const uint8_t *label, size_t llen,
                          const uint8_t *data, size_t dlen) {
    uint8_t len8[8];
    put_u64(len8, llen); hasher_update(&t->h, len8, 8);
    hasher_update(&t->h, label, llen);
    put_u64(len8, dlen); hasher_update(&t->h, len8, 8);
    hasher_update(&t->h, data, dlen);
}

/* transcript.rs:62-69 */
zo_transcript *zo_transcript_new(const uint8_t *label, size_t len) {
    zo_transcript *t = calloc(1, sizeof *t);
    hasher_init(&t->h);
    zo_transcript_absorb(t, (const uint8_t *)"domain", 6, label, len);
    return t;
}
zo_transcript *zo_transcript_clone(const zo_transcript *src) {
    zo_transcript *t = calloc(1, sizeof *t);
    hasher_clone(&t->h, &src->h);
    t->counter = src->counter;
    return t;
}
void zo_transcript_free(zo_transcript *t) {
    if (!t) return;
    hasher_free(&t->h); free(t);
}

void zo_transcript_export(const zo_transcript *t, uint8_t *tail, uint32_t *tail_len,
                          uint8_t stack[54][32], uint32_t *stack_len, uint64_t *next_index,
                          uint64_t *total_len, uint64_t *counter) {
    size_t tl = t->h.len - t->h.start;
    memcpy(tail, t->h.buf + t->h.start, tl);
    *tail_len = (uint32_t)tl;
    memcpy(stack, t->h.stack, sizeof t->h.stack);
    *stack_len = (uint32_t)t->h.stack_len;
    *next_index = t->h.next_index;
    *total_len = t->h.total_len;
    *counter = t->counter;
}

/* transcript.rs:162-171 */
static void squeeze_raw(zo_transcript *t, const uint8_t *label, size_t llen, uint8_t out[32]) {
    hasher h; hasher_clone(&h, &t->h);
    uint8_t len8[8];
    put_u64(len8, llen); hasher_update(&h, len8, 8);
    hasher_update(&h, label, llen);
    put_u64(len8, t->counter); hasher_update(&h, len8, 8);
    t->counter++;
    hasher_finalize(&h, out);
    hasher_free(&h);
    zo_transcript_absorb(t, label, llen, out, 32);
}

void zo_transcript_challenge_bytes(zo_transcript *t, const uint8_t *label, size_t llen,
                                   uint8_t out[32]) {
    squeeze_raw(t, label, llen, out);
}

/* transcript.rs:136-141 + ext4.rs:179-187 (coordinates reduced mod p) */
void zo_transcript_challenge_ext(zo_transcript *t, const uint8_t *label, size_t llen,
                                 uint32_t out[4]) {
    uint8_t b[32];
    squeeze_raw(t, label, llen, b);
    for (int i = 0; i < 4; i++) out[i] = get_u32(b + 4 * i) % P;
}
static ext4 challenge_ext(zo_transcript *t, const char *label) {
    ext4 r;
    zo_transcript_challenge_ext(t, (const uint8_t *)label, strlen(label), r.c);
    return r;
}

/* transcript.rs:148-160 */
int zo_transcript_challenge_index(zo_transcript *t, const uint8_t *label, size_t llen,
                                  uint64_t domain, uint64_t *out) {
    if (!is_pow2(domain)) return -1;
    uint8_t b[32];
    squeeze_raw(t, label, llen, b);
    *out = get_u64(b) & (domain - 1);
    return 0;
}

/* transcript.rs:341-351 leading zero bits, MSB first */
static uint32_t leading_zero_bits(const uint8_t d[32]) {
    uint32_t count = 0;
    for (int i = 0; i < 32; i++) {
        uint32_t z = d[i] ? (uint32_t)__builtin_clz((unsigned)d[i]) - 24 : 8;
        count += z;
        if (z < 8) break;
    }
    return count;
}

/* transcript.rs:182-189 head = H(history) || LE64(|label|) || label */
static size_t pow_head(const zo_transcript *t, const uint8_t *label, size_t llen,
                       uint8_t *head) {
    hasher_finalize(&t->h, head);
    put_u64(head + 32, llen);
    memcpy(head + 40, label, llen);
    return 40 + llen;
}

/* transcript.rs:251-260 */
static void pow_digest(const uint8_t *head, size_t hlen, uint64_t nonce, uint8_t out[32]) {
    uint8_t in[CHUNK_LEN + 64];
    memcpy(in, head, hlen);
    put_u64(in + hlen, nonce);
    blake3_small(in, hlen + 8, out);
}

/* transcript.rs:284-303 */
static int scan_range(const uint8_t *head, size_t hlen, uint64_t start, uint64_t count,
                      uint32_t bits, uint64_t *found) {
    uint8_t d[32];
    uint64_t nonce = start;
    for (uint64_t i = 0; i < count; i++) {
        pow_digest(head, hlen, nonce, d);
        if (leading_zero_bits(d) >= bits) { *found = nonce; return 1; }
        nonce++;
    }
    return 0;
}

typedef struct {
    const uint8_t *head; size_t hlen; uint32_t bits; uint64_t per_worker;
    uint64_t base; int *hit; uint64_t *val;
} grind_ctx;

static void grind_worker(void *vctx, size_t w0, size_t wn) {
    grind_ctx *c = vctx;
    for (size_t w = w0; w < w0 + wn; w++) {
        uint64_t f = 0;
        c->hit[w] = scan_range(c->head, c->hlen, c->base + w * c->per_worker, c->per_worker,
                               c->bits, &f);
        c->val[w] = f;
    }
}

/* transcript.rs:310-338 banded parallel scan == sequential minimum nonce */
static uint64_t grind_parallel(const uint8_t *head, size_t hlen, uint32_t bits,
                               size_t workers) {
    grind_ctx c = {head, hlen, bits, 1ull << (bits < 16 ? bits : 16), 0, NULL, NULL};
    c.hit = calloc(workers, sizeof(int));
    c.val = calloc(workers, sizeof(uint64_t));
    for (;;) {
        par_chunks(workers, workers, grind_worker, &c);
        int any = 0; uint64_t best = 0;
        for (size_t w = 0; w < workers; w++)
            if (c.hit[w] && (!any || c.val[w] < best)) { any = 1; best = c.val[w]; }
        if (any) { free(c.hit); free(c.val); return best; }
        c.base += workers * c.per_worker;
    }
}

/* transcript.rs:206-228 */
uint64_t zo_transcript_grind(zo_transcript *t, const uint8_t *label, size_t llen,
                             uint32_t bits) {
    uint8_t z[8] = {0};
    if (bits > 32) {
        zo_transcript_absorb(t, label, llen, z, 8);
        return 0;
    }
    uint8_t head[CHUNK_LEN];
    size_t hlen = pow_head(t, label, llen, head);
    size_t workers = worker_count((size_t)1 << bits, 4096);
    uint64_t nonce;
    if (workers > 1) {
        nonce = grind_parallel(head, hlen, bits, workers);
    } else {
        nonce = 0;
        while (!scan_range(head, hlen, nonce, 1, bits, &nonce)) nonce++;
    }
    uint8_t n8[8]; put_u64(n8, nonce);
    zo_transcript_absorb(t, label, llen, n8, 8);
    return nonce;
}

/* transcript.rs:236-246 */
int zo_transcript_verify_grind(zo_transcript *t, const uint8_t *label, size_t llen,
                               uint64_t nonce, uint32_t bits) {
    if (bits > 256) return 0;
    uint8_t head[CHUNK_LEN], d[32];
    size_t hlen = pow_head(t, label, llen, head);
    pow_digest(head, hlen, nonce, d);
    if (leading_zero_bits(d) < bits) return 0;
    uint8_t n8[8]; put_u64(n8, nonce);
    zo_transcript_absorb(t, label, llen, n8, 8);
    return 1;
}

static void absorb_s(zo_transcript *t, const char *label, const uint8_t *d, size_t n) {
    zo_transcript_absorb(t, (const uint8_t *)label, strlen(label), d, n);
}

/* ------------------------------------------------------------------------ */
/* merkle.rs — BLAKE3 Merkle trees, duplicate-last padding, caps             */
/* ------------------------------------------------------------------------ */

typedef uint8_t digest[32];
typedef struct { size_t n_layers; size_t *len; digest **layer; } mtree;

static void mtree_free(mtree *t) {
    for (size_t i = 0; i < t->n_layers; i++) free(t->layer[i]);
    free(t->layer); free(t->len);
    memset(t, 0, sizeof *t);
}

typedef struct { const digest *prev; digest *next; } level_ctx;
static void hash_level_worker(void *vctx, size_t base, size_t len) {  /* merkle.rs:367-376 */
    level_ctx *c = vctx;
    for (size_t i = base; i < base + len; i++)
        zo_node_digest(c->prev[2 * i], c->prev[2 * i + 1], c->next[i]);
}

/* merkle.rs:350-360 finish(): pad by duplicating the last leaf, hash up. */
static void mtree_finish(mtree *t, digest *leaves, size_t count) {
    size_t target = 1;
    while (target < count) target <<= 1;
    if (target != count) {
        leaves = realloc(leaves, target * sizeof(digest));
        for (size_t i = count; i < target; i++) memcpy(leaves[i], leaves[count - 1], 32);
    }
    size_t depth = log2u(target);
    t->n_layers = depth + 1;
    t->len = malloc(t->n_layers * sizeof(size_t));
    t->layer = malloc(t->n_layers * sizeof(digest *));
    t->layer[0] = leaves; t->len[0] = target;
    for (size_t l = 1; l <= depth; l++) {
        t->len[l] = t->len[l - 1] / 2;
        t->layer[l] = malloc(t->len[l] * sizeof(digest));
        level_ctx c = {(const digest *)t->layer[l - 1], t->layer[l]};
        for_each_indexed(t->len[l], 1024, hash_level_worker, &c);
    }
}

typedef struct { const uint8_t *flat; size_t leaf_len; digest *out; } leaf_ctx;
static void leaf64_worker(void *vctx, size_t base, size_t len) {
    leaf_ctx *c = vctx;
    for (size_t i = base; i < base + len; i++) zo_leaf64_digest(c->flat + 64 * i, c->out[i]);
}
static void leaf_worker(void *vctx, size_t base, size_t len) {
    leaf_ctx *c = vctx;
    for (size_t i = base; i < base + len; i++)
        zo_leaf_digest(c->flat + c->leaf_len * i, c->leaf_len, c->out[i]);
}

/* merkle.rs:93-110 */
static int mtree_from_flat64(const uint8_t *flat, size_t len, mtree *t) {
    if (len == 0) return ZO_EMPTY_INPUT;
    if (len % 64) return ZO_MALFORMED_INPUT;
    size_t count = len / 64;
    digest *leaves = malloc(count * sizeof(digest));
    leaf_ctx c = {flat, 64, leaves};
    for_each_indexed(count, 1024, leaf64_worker, &c);
    mtree_finish(t, leaves, count);
    return ZO_OK;
}
/* merkle.rs:63-80 */
static int mtree_from_flat(const uint8_t *flat, size_t len, size_t leaf_len, mtree *t) {
    if (len == 0 || leaf_len == 0) return ZO_EMPTY_INPUT;
    if (len % leaf_len) return ZO_MALFORMED_INPUT;
    size_t count = len / leaf_len;
    digest *leaves = malloc(count * sizeof(digest));
    leaf_ctx c = {flat, leaf_len, leaves};
    for_each_indexed(count, 1024, leaf_worker, &c);
    mtree_finish(t, leaves, count);
    return ZO_OK;
}

static size_t mtree_num_leaves(const mtree *t) { return t->len[0]; }

/* merkle.rs:229-232: cap = layer depth - min(dropped, depth) */
static const digest *mtree_cap(const mtree *t, size_t dropped, size_t *count) {
    size_t depth = t->n_layers - 1;
    size_t l = depth - (dropped < depth ? dropped : depth);
    *count = t->len[l];
    return (const digest *)t->layer[l];
}

typedef struct { uint8_t sib[32]; uint8_t is_left; } pstep;
typedef struct { pstep *s; size_t n; } path_t;

/* merkle.rs:139-158 + 240-245 (capped: keep the first depth - drop steps) */
static int mtree_prove_capped(const mtree *t, size_t index, size_t drop, path_t *out) {
    if (index >= mtree_num_leaves(t)) return ZO_INDEX_OUT_OF_BOUNDS;
    size_t full = t->n_layers - 1;
    size_t d = drop < full ? drop : full;
    out->n = full - d;
    out->s = malloc((out->n ? out->n : 1) * sizeof(pstep));
    for (size_t l = 0; l < out->n; l++) {
        int left = index % 2 == 0;
        memcpy(out->s[l].sib, t->layer[l][left ? index + 1 : index - 1], 32);
        out->s[l].is_left = (uint8_t)left;
        index /= 2;
    }
    return ZO_OK;
}

/* merkle.rs:320-324 */
static int directions_match(size_t index, const path_t *p) {
    for (size_t l = 0; l < p->n; l++)
        if (p->s[l].is_left != (((index >> l) & 1) == 0)) return 0;
    return 1;
}
static void walk_path(uint8_t cur[32], const path_t *p) {
    for (size_t l = 0; l < p->n; l++) {
        uint8_t nx[32];
        if (p->s[l].is_left) zo_node_digest(cur, p->s[l].sib, nx);
        else zo_node_digest(p->s[l].sib, cur, nx);
        memcpy(cur, nx, 32);
    }
}
/* merkle.rs:254-277 */
static int verify_capped64(const uint8_t entry[32], const uint8_t leaf[64], size_t index,
                           size_t total_depth, const path_t *p) {
    if (total_depth >= 64 || p->n > total_depth || (index >> total_depth) != 0 ||
        !directions_match(index, p))
        return 0;
    uint8_t cur[32];
    zo_leaf64_digest(leaf, cur);
    walk_path(cur, p);
    return memcmp(cur, entry, 32) == 0;
}
/* merkle.rs:286-309 */
static int verify_capped(const uint8_t entry[32], const uint8_t *leaf, size_t llen,
                         size_t index, size_t total_depth, const path_t *p) {
    if (total_depth >= 64 || p->n > total_depth || (index >> total_depth) != 0 ||
        !directions_match(index, p))
        return 0;
    uint8_t cur[32];
    zo_leaf_digest(leaf, llen, cur);
    walk_path(cur, p);
    return memcmp(cur, entry, 32) == 0;
}

/* merkle.rs:333-337 */
static void capped_shape(size_t num_leaves, size_t cap_height, size_t *drop, size_t *depth) {
    *depth = log2u(num_leaves);
    *drop = cap_height < *depth ? cap_height : *depth;
}

int zo_merkle_flat64_cap(const uint8_t *flat, size_t len, size_t cap_height,
                         uint8_t *cap_out, size_t *cap_count) {
    mtree t;
    int rc = mtree_from_flat64(flat, len, &t);
    if (rc) return rc;
    size_t n;
    const digest *cap = mtree_cap(&t, cap_height, &n);
    memcpy(cap_out, cap, 32 * n);
    *cap_count = n;
    mtree_free(&t);
    return ZO_OK;
}
int zo_merkle_flat_cap(const uint8_t *flat, size_t len, size_t leaf_len, size_t cap_height,
                       uint8_t *cap_out, size_t *cap_count) {
    mtree t;
    int rc = mtree_from_flat(flat, len, leaf_len, &t);
    if (rc) return rc;
    size_t n;
    const digest *cap = mtree_cap(&t, cap_height, &n);
    memcpy(cap_out, cap, 32 * n);
    *cap_count = n;
    mtree_free(&t);
    return ZO_OK;
}

/* ------------------------------------------------------------------------ */
/* ntt.rs — radix-2 DIT Cooley-Tukey, natural-order output                  */
/* ------------------------------------------------------------------------ */

static inline uint64_t rev64(uint64_t x) {
    x = ((x >> 1) & 0x5555555555555555ull) | ((x & 0x5555555555555555ull) << 1);
    x = ((x >> 2) & 0x3333333333333333ull) | ((x & 0x3333333333333333ull) << 2);
    x = ((x >> 4) & 0x0F0F0F0F0F0F0F0Full) | ((x & 0x0F0F0F0F0F0F0F0Full) << 4);
    x = ((x >> 8) & 0x00FF00FF00FF00FFull) | ((x & 0x00FF00FF00FF00FFull) << 8);
    x = ((x >> 16) & 0x0000FFFF0000FFFFull) | ((x & 0x0000FFFF0000FFFFull) << 16);
    return (x >> 32) | (x << 32);
}
static inline size_t brev(size_t i, uint32_t bits) {
    return bits ? (size_t)(rev64((uint64_t)i) >> (64 - bits)) : 0;
}

typedef struct { const void *src; void *dst; uint32_t bits; size_t esize; } brev_ctx;
static void brev_worker(void *vctx, size_t base, size_t len) {
    brev_ctx *c = vctx;
    const uint8_t *s = c->src; uint8_t *d = c->dst;
    for (size_t i = base; i < base + len; i++)
        memcpy(d + i * c->esize, s + brev(i, c->bits) * c->esize, c->esize);
}

/* ntt.rs:21-68 bit reversal; large arrays gather in parallel (chunks 2^14) */
static void bit_reverse_permute(void *v, size_t n, size_t esize, size_t par_threshold) {
    if (n <= 1) return;
    uint32_t bits = log2u(n);
    uint8_t *b = v;
    if (n < par_threshold) {
        uint8_t tmp[16];
        for (size_t i = 0; i < n; i++) {
            size_t r = brev(i, bits);
            if (i < r) {
                memcpy(tmp, b + i * esize, esize);
                memcpy(b + i * esize, b + r * esize, esize);
                memcpy(b + r * esize, tmp, esize);
            }
        }
        return;
    }
    void *out = malloc(n * esize);
    brev_ctx c = {v, out, bits, esize};
    for_each_indexed(n, 1 << 14, brev_worker, &c);
    memcpy(v, out, n * esize);
    free(out);
}

/* ntt.rs:180-187 */
static uint32_t *twiddle_table(uint32_t root, size_t n) {
    size_t h = n / 2 ? n / 2 : 1;
    uint32_t *t = malloc(h * sizeof(uint32_t));
    t[0] = 1;
    for (size_t i = 1; i < n / 2; i++) t[i] = f_mul(t[i - 1], root);
    return t;
}

#define PAR_NTT (1u << 16)
#define PAR_BUTTERFLIES_PER_THREAD (1u << 14)

/* ntt.rs:292-310 */
static void butterfly_range(uint32_t *block, size_t half, size_t j0, size_t j1,
                            const uint32_t *tw, size_t stride, int scale, uint32_t inv) {
    for (size_t j = j0; j < j1; j++) {
        uint32_t u = block[j];
        uint32_t v = f_mul(block[j + half], tw[j * stride]);
        uint32_t s = f_add(u, v), d = f_sub(u, v);
        if (scale) { s = f_mul(s, inv); d = f_mul(d, inv); }
        block[j] = s; block[j + half] = d;
    }
}

typedef struct {
    uint32_t *v; size_t len, half, stride; const uint32_t *tw; int scale; uint32_t inv;
    size_t blocks_per_chunk; uint32_t *block; size_t chunk;
} stage_ctx;
static void stage_blocks_worker(void *vctx, size_t base, size_t len) {
    stage_ctx *c = vctx;
    for (size_t b = base; b < base + len; b++)
        butterfly_range(c->v + b * c->len, c->half, 0, c->half, c->tw, c->stride, c->scale, c->inv);
}
static void stage_inner_worker(void *vctx, size_t base, size_t len) {
    stage_ctx *c = vctx;
    butterfly_range(c->block, c->half, base, base + len, c->tw, c->stride, c->scale, c->inv);
}

/* ntt.rs:207-247 one stage, parallel over blocks or within a block */
static void butterfly_stage(uint32_t *v, size_t n, size_t len, const uint32_t *tw,
                            size_t stride, int scale, uint32_t inv) {
    size_t half = len / 2, blocks = n / len, bflies = blocks * half;
    size_t workers = n < PAR_NTT ? 1 : worker_count(bflies, PAR_BUTTERFLIES_PER_THREAD);
    stage_ctx c = {v, len, half, stride, tw, scale, inv, 0, NULL, 0};
    if (workers <= 1) { stage_blocks_worker(&c, 0, blocks); return; }
    if (blocks >= workers) { par_chunks(blocks, workers, stage_blocks_worker, &c); return; }
    for (size_t b = 0; b < blocks; b++) {
        c.block = v + b * len;
        par_chunks(half, workers, stage_inner_worker, &c);
    }
}

static int check_domain(size_t n) {  /* ntt.rs:441-446 */
    if (!is_pow2(n) || n > ((size_t)1 << TWO_ADICITY)) return ZO_INVALID_DOMAIN_SIZE;
    return ZO_OK;
}

/* ntt.rs:116-149 forward NTT (bit_reverse_permute then stages) */
static int ntt_forward_owned(uint32_t *v, size_t n) {
    int rc = check_domain(n);
    if (rc) return rc;
    if (n == 1) return ZO_OK;
    uint32_t omega = 0;
    primitive_root(n, &omega);
    bit_reverse_permute(v, n, 4, 1 << 18);
    uint32_t *tw = twiddle_table(omega, n);
    for (size_t len = 2; len <= n; len *= 2) butterfly_stage(v, n, len, tw, n / len, 0, 0);
    free(tw);
    return ZO_OK;
}
int zo_ntt_forward(uint32_t *v, size_t n) { return ntt_forward_owned(v, n); }

/* ntt.rs:158-177 inverse NTT, 1/n folded into the last stage */
int zo_ntt_inverse(uint32_t *v, size_t n) {
    int rc = check_domain(n);
    if (rc) return rc;
    if (n == 1) return ZO_OK;
    uint32_t omega = 0;
    primitive_root(n, &omega);
    uint32_t *tw = twiddle_table(f_inv(omega), n);
    uint32_t n_inv = f_inv(f_from_u64(n));
    bit_reverse_permute(v, n, 4, 1 << 18);
    for (size_t len = 2; len < n; len *= 2) butterfly_stage(v, n, len, tw, n / len, 0, 0);
    butterfly_stage(v, n, n, tw, 1, 1, n_inv);
    free(tw);
    return ZO_OK;
}

/* ntt.rs:341-363 evaluate on the coset shift * <omega_m>, m = n * blowup */
int zo_evaluate_on_coset(const uint32_t *coeffs, size_t n, size_t blowup, uint32_t shift,
                         uint32_t *out) {
    if (!is_pow2(blowup)) return ZO_INVALID_BLOWUP;
    int rc = check_domain(n);
    if (rc) return rc;
    size_t m = n * blowup;
    if (m > ((size_t)1 << TWO_ADICITY)) return ZO_INVALID_DOMAIN_SIZE;
    memset(out, 0, m * sizeof(uint32_t));
    uint32_t power = 1;
    for (size_t i = 0; i < n; i++) {
        out[i] = f_mul(coeffs[i], power);
        power = f_mul(power, shift);
    }
    return ntt_forward_owned(out, m);
}

/* ntt.rs:436-439 */
int zo_reed_solomon_extend(const uint32_t *values, size_t n, size_t blowup, uint32_t *out) {
    uint32_t *c = malloc(n * sizeof(uint32_t));
    memcpy(c, values, n * sizeof(uint32_t));
    int rc = zo_ntt_inverse(c, n);
    if (!rc) rc = zo_evaluate_on_coset(c, n, blowup, GENERATOR, out);
    free(c);
    return rc;
}

/* ------------------------------------------------------------------------ */
/* codec.rs — VERSION = 6 writer / fail-closed reader                        */
/* ------------------------------------------------------------------------ */

#define VERSION 6
#define MAX_QUERIES (1u << 20)
#define MAX_FOLDS 64u
#define MAX_PATH_STEPS 128u
#define MAX_CAP_DIGESTS 256u
#define MAX_ELEMS (1u << 27)

typedef struct { uint8_t *b; size_t n, cap; } writer;
static void w_bytes(writer *w, const void *d, size_t n) {
    if (w->n + n > w->cap) {
        size_t nc = w->cap ? w->cap * 2 : 4096;
        while (nc < w->n + n) nc *= 2;
        w->b = realloc(w->b, nc); w->cap = nc;
    }
    memcpy(w->b + w->n, d, n); w->n += n;
}
static void w_byte(writer *w, uint8_t v) { w_bytes(w, &v, 1); }
static void w_u32(writer *w, uint32_t v) { uint8_t b[4]; put_u32(b, v); w_bytes(w, b, 4); }
static void w_u64(writer *w, uint64_t v) { uint8_t b[8]; put_u64(b, v); w_bytes(w, b, 8); }
static void w_ext4(writer *w, ext4 e) { uint8_t b[16]; e_to_bytes(e, b); w_bytes(w, b, 16); }
static void w_path(writer *w, const path_t *p) {  /* codec.rs:95-101 */
    w_u32(w, (uint32_t)p->n);
    for (size_t i = 0; i < p->n; i++) { w_bytes(w, p->s[i].sib, 32); w_byte(w, p->s[i].is_left); }
}
static void w_cap(writer *w, const digest *cap, size_t n) {  /* codec.rs:104-109 */
    w_u32(w, (uint32_t)n);
    w_bytes(w, cap, 32 * n);
}

typedef struct { const uint8_t *in; size_t n, pos; int err; } reader;
static const uint8_t *r_take(reader *r, size_t n) {
    if (r->err || n > r->n - r->pos) { r->err = 1; return NULL; }
    const uint8_t *p = r->in + r->pos; r->pos += n; return p;
}
static uint8_t r_byte(reader *r) { const uint8_t *p = r_take(r, 1); return p ? *p : 0; }
static uint32_t r_u32(reader *r) { const uint8_t *p = r_take(r, 4); return p ? get_u32(p) : 0; }
static uint64_t r_u64(reader *r) { const uint8_t *p = r_take(r, 8); return p ? get_u64(p) : 0; }
static uint32_t r_field(reader *r) {  /* codec.rs:197-207 rejects >= p */
    uint32_t v = r_u32(r);
    if (v >= P) r->err = 1;
    return v;
}
static ext4 r_ext4(reader *r) {
    ext4 e; for (int i = 0; i < 4; i++) e.c[i] = r_field(r); return e;
}
static size_t r_count(reader *r, uint32_t max) {  /* codec.rs:231-242 */
    uint32_t n = r_u32(r);
    if (n > max) { r->err = 1; return 0; }
    return r->err ? 0 : n;
}
/* codec.rs:245-251; entries are 33 bytes so a count must fit the input. */
static void r_path(reader *r, path_t *p) {
    size_t n = r_count(r, MAX_PATH_STEPS);
    p->n = 0; p->s = NULL;
    if (r->err) return;
    if (n * 33 > r->n - r->pos) { r->err = 1; return; }
    p->s = malloc((n ? n : 1) * sizeof(pstep));
    for (size_t i = 0; i < n; i++) {
        const uint8_t *d = r_take(r, 32);
        if (!d) return;
        memcpy(p->s[i].sib, d, 32);
        uint8_t dir = r_byte(r);
        if (dir > 1) { r->err = 1; return; }
        p->s[i].is_left = dir;
        p->n = i + 1;
    }
}
static digest *r_cap(reader *r, size_t *count) {  /* codec.rs:254-260 */
    size_t n = r_count(r, MAX_CAP_DIGESTS);
    *count = 0;
    if (r->err) return NULL;
    const uint8_t *d = r_take(r, 32 * n);
    if (!d) return NULL;
    digest *c = malloc((n ? n : 1) * 32);
    memcpy(c, d, 32 * n);
    *count = n;
    return c;
}

/* ------------------------------------------------------------------------ */
/* fri.rs — params, tuners, commit, fold, open, verify                       */
/* ------------------------------------------------------------------------ */

#define LDE_SHIFT GENERATOR
#define MAX_FINAL_SIZE (1u << 10)

typedef struct {
    size_t blowup, num_queries, final_size; uint32_t grinding_bits; size_t cap_height;
} fri_params;

/* fri.rs:152-171 */
static int fri_params_new(size_t blowup, size_t q, size_t final_size, fri_params *o) {
    if (blowup < 2 || !is_pow2(blowup)) return ZO_INVALID_BLOWUP;
    if (q == 0) return ZO_NO_QUERIES;
    if (final_size < 2 || !is_pow2(final_size) || final_size > MAX_FINAL_SIZE)
        return ZO_INVALID_DOMAIN_SIZE;
    o->blowup = blowup; o->num_queries = q; o->final_size = final_size;
    o->grinding_bits = 0; o->cap_height = 0;
    return ZO_OK;
}
/* fri.rs:163-196 */
static int fri_params_validate(const fri_params *p) {
    if (p->blowup < 2 || !is_pow2(p->blowup)) return ZO_INVALID_BLOWUP;
    if (p->num_queries == 0) return ZO_NO_QUERIES;
    if (p->num_queries > MAX_QUERIES) return ZO_MALFORMED_INPUT;
    if (p->final_size < 2 || !is_pow2(p->final_size) || p->final_size > MAX_FINAL_SIZE)
        return ZO_INVALID_DOMAIN_SIZE;
    if (p->grinding_bits > 32) return ZO_MALFORMED_INPUT;
    if (p->cap_height > 8) return ZO_MALFORMED_INPUT;
    return ZO_OK;
}

/* fri.rs:935-939 */
static size_t fri_drop_top(size_t leaves, size_t cap_height) {
    size_t d = log2u(leaves);
    return cap_height < d ? cap_height : d;
}

/* fri.rs:945-955 */
static size_t fri_layer_sizes(size_t len, size_t final_size, size_t *out) {
    size_t k = 0;
    for (;;) {
        out[k++] = len;
        if (len <= final_size) break;
        len /= 4;
    }
    return k;
}
static size_t sat_add(size_t a, size_t b) { size_t s = a + b; return s < a ? SIZE_MAX : s; }

/* fri.rs:962-979 */
static size_t estimate_fri_bytes(const size_t *layers, size_t nl, size_t q, size_t cap_height) {
    size_t total = 24 + 8;
    for (size_t i = 0; i < nl; i++) {
        size_t v = layers[i];
        size_t leaves = v % 4 == 0 ? v / 4 : v;
        size_t depth = log2u(leaves);
        size_t drop = cap_height < depth ? cap_height : depth;
        total = sat_add(total, (size_t)32 << (drop < 16 ? drop : 16));
        if (i + 1 < nl) total += q * (64 + 33 * (depth - drop));
    }
    return total;
}
/* fri.rs:985-998 */
static size_t estimate_col_bytes(size_t lde_len, size_t q, size_t vb, size_t cap_height) {
    size_t depth = log2u(lde_len);
    size_t drop = cap_height < depth ? cap_height : depth;
    return sat_add((size_t)32 << (drop < 16 ? drop : 16), q * (vb + 33 * (depth - drop)));
}

/* fri.rs:1009-1043 */
void zo_fri_tune_shape(size_t lde_len, size_t q, size_t col_lde, size_t col_vb, int has_col,
                       size_t *final_out, size_t *cap_out) {
    size_t shifted = lde_len / 4 > 2 ? lde_len / 4 : 2;
    while (shifted > 32) shifted /= 4;
    size_t best_f = shifted, best_h = 0, best_bytes = SIZE_MAX;
    size_t layers[64];
    for (;;) {
        size_t nl = fri_layer_sizes(lde_len, shifted, layers);
        for (size_t h = 0; h <= 4; h++) {
            size_t total = estimate_fri_bytes(layers, nl, q, h);
            if (has_col) total = sat_add(total, estimate_col_bytes(col_lde, q, col_vb, h));
            if (total < best_bytes) { best_bytes = total; best_f = shifted; best_h = h; }
        }
        if (shifted <= 1) break;
        shifted /= 4;
        if (shifted < 1) break;
    }
    *final_out = best_f; *cap_out = best_h;
}

/* fri.rs:1050-1056 */
uint32_t zo_fri_composition_millibits(size_t lde_len, size_t degree_bound) {
    size_t den = 1;
    while (den < degree_bound + 1) den <<= 1;
    if (den == 0 || lde_len < den) return 500;
    return 500 * (log2u(lde_len) - log2u(den));
}
/* fri.rs:1064-1074 */
void zo_fri_tune_strength(uint32_t target, uint32_t millibits, size_t *queries,
                          uint32_t *grinding) {
    uint32_t g = target / 2 < 20 ? target / 2 : 20;
    uint64_t remaining = (uint64_t)(target > g ? target - g : 0) * 1000;
    uint64_t per = millibits ? millibits : 1;
    uint64_t qn = (remaining + per - 1) / per;
    if (qn < 1) qn = 1;
    if (qn > 1000000) qn = 1000000;
    *queries = (size_t)qn; *grinding = g;
}

/* fri.rs:1130-1140 */
static int check_layers(size_t lde_len, size_t final_size) {
    if (final_size >= lde_len || lde_len % final_size) return ZO_INVALID_DOMAIN_SIZE;
    size_t ratio = lde_len / final_size;
    if (!is_pow2(ratio) || log2u(ratio) % 2) return ZO_INVALID_DOMAIN_SIZE;
    return ZO_OK;
}

/* fri.rs:1311-1331 fold one quad (x, -x, j0 x, -j0 x) */
static ext4 fold_values(const ext4 q[4], uint32_t inv_point, const ext4 ch[3], uint32_t unit) {
    ext4 even_sum = e_add(e_add(q[0], q[1]), e_add(q[2], q[3]));
    ext4 odd_diff = e_sub(q[0], q[1]);
    ext4 skew_diff = e_sub(q[2], q[3]);
    ext4 mean = e_halve(e_halve(even_sum));
    ext4 odd = e_halve(e_halve(e_sub(odd_diff, e_mul_base(skew_diff, unit))));
    ext4 even = e_halve(e_halve(e_sub(e_add(q[0], q[1]), e_add(q[2], q[3]))));
    ext4 skew = e_halve(e_halve(e_add(odd_diff, e_mul_base(skew_diff, unit))));
    ext4 acc = e_add(e_mul_base(e_add(e_mul_base(e_mul(ch[2], skew), inv_point),
                                      e_mul(ch[1], even)), inv_point),
                     e_mul(ch[0], odd));
    return e_add(mean, e_mul_base(acc, inv_point));
}
void zo_fold_values(const uint32_t quad[16], uint32_t inv_point, const uint32_t ch[12],
                    uint32_t unit, uint32_t out[4]) {
    ext4 q[4], c[3];
    memcpy(q, quad, 64); memcpy(c, ch, 48);
    ext4 r = fold_values(q, inv_point, c, unit);
    memcpy(out, r.c, 16);
}

typedef struct {
    const ext4 *values; const uint32_t *inv_points; const ext4 *ch; uint32_t unit; ext4 *out;
} fold_ctx;
static void fold_worker(void *vctx, size_t base, size_t len) {
    fold_ctx *c = vctx;
    for (size_t i = base; i < base + len; i++)
        c->out[i] = fold_values(c->values + 4 * i, c->inv_points[i], c->ch, c->unit);
}

/* fri.rs:1273-1302 */
static void fold_layer(const ext4 *values, size_t n, const uint32_t *first_points,
                       const ext4 ch[3], uint32_t unit, ext4 *next, uint32_t *next_points) {
    size_t quarter = n / 4;
    uint32_t *inv = malloc(quarter * sizeof(uint32_t));
    memcpy(inv, first_points, quarter * sizeof(uint32_t));
    zo_batch_invert(inv, quarter);
    fold_ctx c = {values, inv, ch, unit, next};
    for_each_indexed(quarter, 512, fold_worker, &c);
    for (size_t j = 0; j < quarter / 4; j++) {
        uint32_t s = f_mul(first_points[4 * j], first_points[4 * j]);
        next_points[j] = f_mul(s, s);
    }
    free(inv);
}
void zo_fold_layer(const uint32_t *values, size_t n, const uint32_t *first_points,
                   const uint32_t ch[12], uint32_t *out_values, uint32_t *out_points) {
    uint32_t unit;
    two_adic_generator(2, &unit);
    ext4 c[3];
    memcpy(c, ch, 48);
    fold_layer((const ext4 *)values, n, first_points, c, unit, (ext4 *)out_values, out_points);
}

/* fri.rs:1401-1428 commit one layer */
static int commit_layer(const ext4 *layer, size_t n, mtree *t) {
    uint8_t *flat = malloc(16 * n);
    for (size_t i = 0; i < n; i++) e_to_bytes(layer[i], flat + 16 * i);
    int rc = n % 4 == 0 ? mtree_from_flat64(flat, 16 * n, t) : mtree_from_flat(flat, 16 * n, 16, t);
    free(flat);
    return rc;
}

typedef struct {
    size_t n_layers;
    ext4 **layers; size_t *layer_len;
    mtree *trees;
    size_t lde_len, poly_len, degree_bound;
    fri_params params;
} fri_state;

static void fri_state_free(fri_state *s) {
    for (size_t i = 0; i < s->n_layers; i++) { free(s->layers[i]); mtree_free(&s->trees[i]); }
    free(s->layers); free(s->layer_len); free(s->trees);
    memset(s, 0, sizeof *s);
}

/* fri.rs:1450-1456 */
static void encode_dims(size_t lde, size_t poly, size_t deg, uint8_t out[24]) {
    put_u64(out, lde); put_u64(out + 8, poly); put_u64(out + 16, deg);
}

/* fri.rs:551-633 commit_inner; takes ownership of `current` */
static int fri_commit_inner(ext4 *current, size_t lde_len, size_t degree_bound,
                            size_t poly_len, const fri_params *params, zo_transcript *t,
                            fri_state *st) {
    int rc = fri_params_validate(params);
    if (!rc) rc = check_layers(lde_len, params->final_size);
    if (!rc && (lde_len < 2 || degree_bound + 1 > lde_len / 2)) rc = ZO_MALFORMED_INPUT;
    if (rc) { free(current); return rc; }
    uint32_t folds = log2u(lde_len / params->final_size) / 2;
    size_t residual = degree_bound >> (2 * folds);
    if (residual + 1 >= params->final_size) { free(current); return ZO_MALFORMED_INPUT; }
    uint8_t dims[24];
    encode_dims(lde_len, poly_len, degree_bound, dims);
    absorb_s(t, "fri-dims", dims, 24);

    uint32_t omega = 0;
    primitive_root(lde_len, &omega);
    size_t nfp = lde_len / 4;
    uint32_t *first = malloc((nfp ? nfp : 1) * sizeof(uint32_t));
    uint32_t cur = LDE_SHIFT;  /* fri.rs:1086-1094 */
    for (size_t i = 0; i < nfp; i++) { first[i] = cur; cur = f_mul(cur, omega); }
    bit_reverse_permute(current, lde_len, 16, 1 << 24);
    bit_reverse_permute(first, nfp, 4, 1 << 18);
    uint32_t unit;
    two_adic_generator(2, &unit);

    size_t max_layers = folds + 1;
    memset(st, 0, sizeof *st);
    st->layers = calloc(max_layers, sizeof(ext4 *));
    st->layer_len = calloc(max_layers, sizeof(size_t));
    st->trees = calloc(max_layers, sizeof(mtree));
    st->layers[0] = current; st->layer_len[0] = lde_len; st->n_layers = 1;
    for (;;) {
        size_t idx = st->n_layers - 1;
        commit_layer(st->layers[idx], st->layer_len[idx], &st->trees[idx]);
        size_t ncap;
        const digest *cap = mtree_cap(&st->trees[idx],
                                      fri_drop_top(mtree_num_leaves(&st->trees[idx]), params->cap_height),
                                      &ncap);
        for (size_t i = 0; i < ncap; i++) absorb_s(t, "fri-layer-root", cap[i], 32);
        if (st->layer_len[idx] == params->final_size) break;
        ext4 ch[3];
        for (int k = 0; k < 3; k++) ch[k] = challenge_ext(t, "fri-fold");
        size_t n = st->layer_len[idx];
        ext4 *next = malloc((n / 4) * sizeof(ext4));
        uint32_t *next_first = malloc(((n / 16) ? n / 16 : 1) * sizeof(uint32_t));
        fold_layer(st->layers[idx], n, first, ch, unit, next, next_first);
        free(first);
        first = next_first;
        st->layers[idx + 1] = next; st->layer_len[idx + 1] = n / 4; st->n_layers++;
    }
    free(first);
    size_t fl = st->layer_len[st->n_layers - 1];
    uint8_t *enc = malloc(16 * fl);
    for (size_t i = 0; i < fl; i++) e_to_bytes(st->layers[st->n_layers - 1][i], enc + 16 * i);
    absorb_s(t, "fri-final", enc, 16 * fl);
    free(enc);
    st->lde_len = lde_len; st->poly_len = poly_len; st->degree_bound = degree_bound;
    st->params = *params;
    return ZO_OK;
}

/* fri.rs:896-904 Commitment::write_body */
static void fri_write_commitment(writer *w, const fri_state *st) {
    w_u64(w, st->lde_len); w_u64(w, st->poly_len); w_u64(w, st->degree_bound);
    w_u32(w, (uint32_t)st->n_layers);
    for (size_t i = 0; i < st->n_layers; i++) {
        size_t n;
        const digest *cap = mtree_cap(&st->trees[i],
                                      fri_drop_top(mtree_num_leaves(&st->trees[i]), st->params.cap_height), &n);
        w_cap(w, cap, n);
    }
}

/* fri.rs:645-666 open + fri.rs:1229-1260 open_one + fri.rs:352-368 write_body */
static int fri_open_write(const fri_state *st, zo_transcript *t, writer *w, uint64_t *indices) {
    uint64_t nonce = 0;
    if (st->params.grinding_bits > 0)
        nonce = zo_transcript_grind(t, (const uint8_t *)"fri-pow", 7, st->params.grinding_bits);
    size_t fl = st->layer_len[st->n_layers - 1];
    w_u32(w, (uint32_t)fl);
    for (size_t i = 0; i < fl; i++) w_ext4(w, st->layers[st->n_layers - 1][i]);
    w_u64(w, nonce);
    w_u32(w, (uint32_t)st->params.num_queries);
    for (size_t qi = 0; qi < st->params.num_queries; qi++) {
        uint64_t leaf;
        if (zo_transcript_challenge_index(t, (const uint8_t *)"fri-query", 9, st->lde_len, &leaf))
            return ZO_FRI_VERIFICATION_FAILED;
        indices[qi] = leaf;
        w_u32(w, (uint32_t)(st->n_layers - 1));
        size_t index = leaf;
        for (size_t d = 0; d + 1 < st->n_layers; d++) {
            size_t base = index / 4 * 4;
            for (int k = 0; k < 4; k++) w_ext4(w, st->layers[d][base + k]);
            path_t p;
            int rc = mtree_prove_capped(&st->trees[d], base / 4,
                                        fri_drop_top(mtree_num_leaves(&st->trees[d]), st->params.cap_height), &p);
            if (rc) return rc;
            w_path(w, &p);
            free(p.s);
            index /= 4;
        }
    }
    return ZO_OK;
}

/* fri.rs:1108-1115 point j of bit-reversed layer `depth` */
static uint32_t point_at(size_t lde_len, size_t depth, size_t j) {
    uint32_t log_m = log2u(lde_len);
    uint32_t bits = log_m - 2 * (uint32_t)depth;
    uint32_t omega = 0;
    primitive_root(lde_len, &omega);
    uint32_t base = f_mul(LDE_SHIFT, f_pow(omega, brev(j, bits)));
    return f_pow(base, 1ull << (2 * depth));
}

/* fri.rs:1339-1362 divided-difference degree check */
static int check_degree_ext(const uint32_t *pts, const ext4 *vals, size_t n, size_t bound) {
    if (n == 0) return 0;
    if (bound >= n - 1) return 1;
    ext4 *tab = malloc(n * sizeof(ext4));
    memcpy(tab, vals, n * sizeof(ext4));
    size_t last = bound + 1 < n - 1 ? bound + 1 : n - 1;
    int ok = 1;
    for (size_t order = 1; order <= last && ok; order++) {
        for (size_t i = 0; i < n - order; i++) {
            uint32_t den = f_sub(pts[i + order], pts[i]);
            if (den == 0) { ok = 0; break; }
            tab[i] = e_mul(e_sub(tab[i + 1], tab[i]), e_from_base(f_inv(den)));
        }
        if (ok && order > bound)
            for (size_t i = 0; i < n - order; i++) if (!e_is_zero(tab[i])) { ok = 0; break; }
    }
    free(tab);
    return ok;
}

/* Decoded FRI commitment/proof (fri.rs:260-326) */
typedef struct { ext4 v[4]; path_t path; } fold_wit;
typedef struct { fold_wit *f; size_t n; } query_t;
typedef struct {
    digest **caps; size_t *cap_n; size_t n_caps;
    size_t lde_len, poly_len, degree_bound;
    ext4 *final_poly; size_t final_n;
    query_t *q; size_t nq;
    uint64_t nonce;
} fri_decoded;

static void fri_decoded_free(fri_decoded *d) {
    for (size_t i = 0; i < d->n_caps; i++) free(d->caps[i]);
    free(d->caps); free(d->cap_n); free(d->final_poly);
    for (size_t i = 0; i < d->nq; i++) {
        for (size_t k = 0; k < d->q[i].n; k++) free(d->q[i].f[k].path.s);
        free(d->q[i].f);
    }
    free(d->q);
    memset(d, 0, sizeof *d);
}

/* fri.rs:908-925 Commitment::read_body + fri.rs:370-397 Proof::read_body */
/* fri.rs:906-925 Commitment::read_body */
static void fri_read_commitment(reader *r, fri_decoded *d) {
    memset(d, 0, sizeof *d);
    d->lde_len = r_u64(r); d->poly_len = r_u64(r); d->degree_bound = r_u64(r);
    size_t nc = r_count(r, MAX_FOLDS);
    if (r->err) return;
    d->caps = calloc(nc ? nc : 1, sizeof(digest *));
    d->cap_n = calloc(nc ? nc : 1, sizeof(size_t));
    for (size_t i = 0; i < nc && !r->err; i++) { d->caps[i] = r_cap(r, &d->cap_n[i]); d->n_caps = i + 1; }
}

/* fri.rs:370-397 Proof::read_body, into the same decoded record */
static void fri_read_proof(reader *r, fri_decoded *d) {
    size_t fn = r_count(r, MAX_ELEMS);
    if (r->err) return;
    if (fn * 16 > r->n - r->pos) { r->err = 1; return; }
    d->final_poly = malloc((fn ? fn : 1) * sizeof(ext4));
    for (size_t i = 0; i < fn; i++) d->final_poly[i] = r_ext4(r);
    d->final_n = fn;
    d->nonce = r_u64(r);
    size_t nq = r_count(r, MAX_QUERIES);
    if (r->err) return;
    if (nq * 4 > r->n - r->pos) { r->err = 1; return; }
    d->q = calloc(nq ? nq : 1, sizeof(query_t));
    for (size_t i = 0; i < nq && !r->err; i++) {
        d->nq = i + 1;
        size_t nf = r_count(r, MAX_FOLDS);
        if (r->err) return;
        d->q[i].f = calloc(nf ? nf : 1, sizeof(fold_wit));
        for (size_t k = 0; k < nf && !r->err; k++) {
            d->q[i].n = k + 1;
            for (int j = 0; j < 4; j++) d->q[i].f[k].v[j] = r_ext4(r);
            r_path(r, &d->q[i].f[k].path);
        }
    }
}

static void fri_read(reader *r, fri_decoded *d) {
    fri_read_commitment(r, d);
    if (!r->err) fri_read_proof(r, d);
}

/* fri.rs:1153-1227 */
static int verify_one(const fri_decoded *d, const ext4 (*fold_ch)[3], const query_t *q,
                      size_t leaf_index, uint32_t unit, size_t cap_height) {
    size_t index = leaf_index;
    for (size_t depth = 0; depth < q->n; depth++) {
        const fold_wit *w = &q->f[depth];
        size_t layer_len = d->lde_len >> (2 * depth);
        size_t base = index / 4 * 4;
        if (base + 3 >= layer_len) return ZO_FRI_VERIFICATION_FAILED;
        size_t quad_len = layer_len / 4;
        size_t depth_bits = log2u(quad_len);
        size_t drop = cap_height < depth_bits ? cap_height : depth_bits;
        if (w->path.n != depth_bits - drop) return ZO_BAD_MERKLE_PATH;
        size_t quad_index = base / 4;
        size_t ei = quad_index >> (depth_bits - drop);
        if (ei >= d->cap_n[depth]) return ZO_BAD_MERKLE_PATH;
        uint32_t x = point_at(d->lde_len, depth, base);
        uint8_t leaf[64], node[32];
        for (int k = 0; k < 4; k++) e_to_bytes(w->v[k], leaf + 16 * k);
        zo_leaf64_digest(leaf, node);
        size_t pos = quad_index;
        for (size_t s = 0; s < w->path.n; s++) {
            if (w->path.s[s].is_left != ((pos & 1) == 0)) return ZO_BAD_MERKLE_PATH;
            uint8_t nx[32];
            if (w->path.s[s].is_left) zo_node_digest(node, w->path.s[s].sib, nx);
            else zo_node_digest(w->path.s[s].sib, node, nx);
            memcpy(node, nx, 32);
            pos >>= 1;
        }
        if (memcmp(node, d->caps[depth][ei], 32)) return ZO_BAD_MERKLE_PATH;
        ext4 parent = fold_values(w->v, f_inv(x), fold_ch[depth], unit);
        if (depth + 1 == q->n) {
            size_t fi = index / 4;
            if (fi >= d->final_n || !e_eq(d->final_poly[fi], parent)) return ZO_FRI_VERIFICATION_FAILED;
        } else {
            if (!e_eq(q->f[depth + 1].v[(index / 4) % 4], parent)) return ZO_FRI_VERIFICATION_FAILED;
        }
        index /= 4;
    }
    return ZO_OK;
}

/* fri.rs:686-859 verify; writes the sampled indices (num_queries of them) */
static int fri_verify(const fri_decoded *d, const fri_params *params, zo_transcript *t,
                      uint64_t *indices) {
    int rc = fri_params_validate(params);
    if (rc) return rc;
    if (d->nq != params->num_queries) return ZO_FRI_VERIFICATION_FAILED;
    if (d->final_n != params->final_size) return ZO_FRI_VERIFICATION_FAILED;
    if (d->n_caps == 0) return ZO_FRI_VERIFICATION_FAILED;
    if (!is_pow2(d->lde_len) || d->lde_len > ((size_t)1 << TWO_ADICITY)) return ZO_INVALID_DOMAIN_SIZE;
    if (d->degree_bound >= d->lde_len) return ZO_FRI_VERIFICATION_FAILED;
    if (!is_pow2(d->poly_len)) return ZO_FRI_VERIFICATION_FAILED;
    if (d->poly_len != d->lde_len) {
        if (d->poly_len > SIZE_MAX / params->blowup ||
            d->lde_len != d->poly_len * params->blowup)
            return ZO_FRI_VERIFICATION_FAILED;
    }
    if (d->lde_len < 2 || d->degree_bound + 1 > d->lde_len / 2) return ZO_FRI_VERIFICATION_FAILED;
    size_t folds = d->n_caps - 1;
    if (folds == 0 || folds > 30 || (d->lde_len >> (2 * folds)) != params->final_size)
        return ZO_FRI_VERIFICATION_FAILED;
    for (size_t i = 0; i < d->n_caps; i++) {
        size_t layer_len = d->lde_len >> (2 * i);
        size_t leaves = layer_len % 4 == 0 ? layer_len / 4 : layer_len;
        size_t depth = log2u(leaves);
        size_t drop = params->cap_height < depth ? params->cap_height : depth;
        if (d->cap_n[i] != ((size_t)1 << drop)) return ZO_BAD_MERKLE_PATH;
    }
    uint8_t dims[24];
    encode_dims(d->lde_len, d->poly_len, d->degree_bound, dims);
    absorb_s(t, "fri-dims", dims, 24);
    ext4 (*fold_ch)[3] = malloc(d->n_caps * sizeof(ext4[3]));
    for (size_t i = 0; i < d->n_caps; i++) {
        for (size_t k = 0; k < d->cap_n[i]; k++) absorb_s(t, "fri-layer-root", d->caps[i][k], 32);
        if (i + 1 < d->n_caps)
            for (int k = 0; k < 3; k++) fold_ch[i][k] = challenge_ext(t, "fri-fold");
    }
    uint8_t *enc = malloc(16 * d->final_n);
    for (size_t i = 0; i < d->final_n; i++) e_to_bytes(d->final_poly[i], enc + 16 * i);
    absorb_s(t, "fri-final", enc, 16 * d->final_n);
    free(enc);
    rc = ZO_OK;
    if (params->grinding_bits == 0) {
        if (d->nonce != 0) rc = ZO_FRI_VERIFICATION_FAILED;
    } else if (!zo_transcript_verify_grind(t, (const uint8_t *)"fri-pow", 7, d->nonce,
                                           params->grinding_bits)) {
        rc = ZO_FRI_VERIFICATION_FAILED;
    }
    uint32_t unit;
    two_adic_generator(2, &unit);
    size_t residual = d->degree_bound >> (2 * folds);
    if (!rc && residual + 1 >= params->final_size) rc = ZO_FRI_VERIFICATION_FAILED;
    if (!rc) {
        uint32_t *fp = malloc(params->final_size * sizeof(uint32_t));
        for (size_t j = 0; j < params->final_size; j++) fp[j] = point_at(d->lde_len, folds, j);
        if (!check_degree_ext(fp, d->final_poly, d->final_n, residual)) rc = ZO_FRI_VERIFICATION_FAILED;
        free(fp);
    }
    if (!rc) {  /* final cap must be the cap of final_poly (fri.rs:828-833) */
        mtree ft;
        commit_layer(d->final_poly, d->final_n, &ft);
        size_t n;
        const digest *cap = mtree_cap(&ft, fri_drop_top(mtree_num_leaves(&ft), params->cap_height), &n);
        if (n != d->cap_n[d->n_caps - 1] || memcmp(cap, d->caps[d->n_caps - 1], 32 * n))
            rc = ZO_FRI_VERIFICATION_FAILED;
        mtree_free(&ft);
    }
    if (!rc) {
        for (size_t i = 0; i < d->nq; i++)
            if (zo_transcript_challenge_index(t, (const uint8_t *)"fri-query", 9, d->lde_len, &indices[i]))
                { rc = ZO_FRI_VERIFICATION_FAILED; break; }
    }
    for (size_t i = 0; !rc && i < d->nq; i++) {
        if (d->q[i].n != folds) { rc = ZO_FRI_VERIFICATION_FAILED; break; }
        rc = verify_one(d, (const ext4 (*)[3])fold_ch, &d->q[i], indices[i], unit, params->cap_height);
    }
    free(fold_ch);
    return rc;
}

/* ------------------------------------------------------------------------ */
/* fri.rs public commit / open / verify (the PCS entry points)               */
/* ------------------------------------------------------------------------ */

static fri_params fri_from_public(const zo_fri_params *p) {
    fri_params f;
    f.blowup = p->blowup; f.num_queries = p->num_queries; f.final_size = p->final_size;
    f.grinding_bits = p->grinding_bits; f.cap_height = p->cap_height;
    return f;
}

/* fri.rs:407-433 commit, :443-460 commit_ext, :473-499 commit_evals,
 * :508-549 commit_ext_evals(_owned): entry checks, encoding, then
 * commit_inner (fri_commit_inner). Ext4 input is 4 coordinates per value. */
int zo_fri_commit(const zo_fri_params *params, int form, const uint32_t *values, size_t n,
                  uint64_t degree_bound, zo_transcript *t, void **state, uint8_t **commitment,
                  size_t *commitment_len) {
    fri_params fp = fri_from_public(params);
    int rc = fri_params_validate(&fp);
    if (rc) return rc;
    if (form < ZO_FRI_COEFFS || form > ZO_FRI_EVALS_EXT) return ZO_MALFORMED_INPUT;
    const int ext = form == ZO_FRI_COEFFS_EXT || form == ZO_FRI_EVALS_EXT;
    const int evals = form >= ZO_FRI_EVALS;
    if (n == 0) return ZO_EMPTY_INPUT;
    if (!is_pow2(n)) return ZO_INVALID_DOMAIN_SIZE;
    size_t lde_len, poly_len, bound;
    ext4 *current;
    if (!evals) {
        /* ntt.rs:341-363 (per coordinate for ext, ntt.rs:394-403) */
        if (n > SIZE_MAX / fp.blowup || n * fp.blowup > ((size_t)1 << TWO_ADICITY))
            return ZO_INVALID_DOMAIN_SIZE;
        lde_len = n * fp.blowup; poly_len = n; bound = n - 1;
        current = calloc(lde_len, sizeof(ext4));
        uint32_t *coord = malloc(n * 4), *lde = malloc(lde_len * 4);
        for (int c = 0; c < (ext ? 4 : 1); c++) {
            for (size_t i = 0; i < n; i++) coord[i] = values[ext ? 4 * i + c : i];
            zo_evaluate_on_coset(coord, n, fp.blowup, LDE_SHIFT, lde);
            for (size_t k = 0; k < lde_len; k++) current[k].c[c] = lde[k];
        }
        free(coord); free(lde);
    } else {
        if (n > ((size_t)1 << TWO_ADICITY)) return ZO_INVALID_DOMAIN_SIZE;
        if (degree_bound >= n) return ZO_MALFORMED_INPUT;
        lde_len = n; poly_len = n; bound = degree_bound;
        current = calloc(lde_len, sizeof(ext4));
        for (size_t k = 0; k < n; k++)
            for (int c = 0; c < (ext ? 4 : 1); c++) current[k].c[c] = values[ext ? 4 * k + c : k];
    }
    fri_state *st = calloc(1, sizeof(fri_state));
    rc = fri_commit_inner(current, lde_len, bound, poly_len, &fp, t, st);
    if (rc) { free(st); return rc; }
    writer w = {0};
    w_byte(&w, VERSION);
    fri_write_commitment(&w, st);
    *state = st;
    *commitment = w.b; *commitment_len = w.n;
    return ZO_OK;
}

/* fri.rs:645-666 open, bytes per fri.rs:331-336 Proof::to_bytes */
int zo_fri_open(void *state, zo_transcript *t, uint8_t **proof, size_t *proof_len,
                uint64_t *indices) {
    fri_state *st = state;
    writer w = {0};
    w_byte(&w, VERSION);
    int rc = fri_open_write(st, t, &w, indices);
    if (rc) { free(w.b); return rc; }
    *proof = w.b; *proof_len = w.n;
    return ZO_OK;
}

void zo_fri_state_free(void *state) {
    if (!state) return;
    fri_state_free(state);
    free(state);
}

/* fri.rs:694-858 verify over Commitment::from_bytes / Proof::from_bytes */
int zo_fri_verify(const zo_fri_params *params, const uint8_t *commitment, size_t commitment_len,
                  const uint8_t *proof, size_t proof_len, zo_transcript *t, uint64_t *indices) {
    fri_params fp = fri_from_public(params);
    reader rc_ = {commitment, commitment_len, 0, 0}, rp = {proof, proof_len, 0, 0};
    fri_decoded d;
    memset(&d, 0, sizeof d);
    int bad = r_byte(&rc_) != VERSION;
    if (!bad) fri_read_commitment(&rc_, &d);
    bad = bad || rc_.err || rc_.pos != rc_.n;
    if (!bad) bad = r_byte(&rp) != VERSION;
    if (!bad) fri_read_proof(&rp, &d);
    bad = bad || rp.err || rp.pos != rp.n;
    int rc = bad ? ZO_MALFORMED_INPUT : fri_verify(&d, &fp, t, indices);
    fri_decoded_free(&d);
    return rc;
}

/* ------------------------------------------------------------------------ */
/* air.rs — Fibonacci AIR                                                    */
/* ------------------------------------------------------------------------ */

static const size_t MAX_DOMAIN = (size_t)1 << TWO_ADICITY;

/* air.rs:62-102 */
int zo_air_params_new(uint64_t n, uint64_t blowup, uint64_t q, uint64_t final_size,
                      uint32_t a0, uint32_t b0, uint32_t b_last, zo_air_params *o) {
    if (n < 2 || !is_pow2(n)) return ZO_INVALID_DOMAIN_SIZE;
    if (blowup < 4 || !is_pow2(blowup)) return ZO_INVALID_BLOWUP;
    if (q == 0) return ZO_NO_QUERIES;
    if (final_size < 2 || !is_pow2(final_size)) return ZO_INVALID_DOMAIN_SIZE;
    if (n > UINT64_MAX / blowup || n * blowup > MAX_DOMAIN) return ZO_INVALID_DOMAIN_SIZE;
    o->n_steps = n; o->blowup = blowup; o->num_queries = q; o->final_size = final_size;
    o->grinding_bits = 0; o->cap_height = 0;
    o->a0 = a0 % P; o->b0 = b0 % P; o->b_last = b_last % P;
    return ZO_OK;
}

/* air.rs:127-158 */
int zo_air_for_security(uint64_t n, uint32_t a0, uint32_t b0, uint32_t b_last,
                        uint32_t target, zo_air_params *o) {
    if (n < 2 || !is_pow2(n)) return ZO_INVALID_DOMAIN_SIZE;
    uint64_t blowup = 16;
    if (n > UINT64_MAX / blowup || n * blowup > MAX_DOMAIN) return ZO_INVALID_DOMAIN_SIZE;
    size_t lde = n * blowup;
    uint32_t mb = zo_fri_composition_millibits(lde, n - 1);
    size_t q; uint32_t g;
    zo_fri_tune_strength(target, mb, &q, &g);
    size_t fs, ch;
    zo_fri_tune_shape(lde, q, lde, 24, 1, &fs, &ch);
    o->n_steps = n; o->blowup = blowup; o->num_queries = q; o->final_size = fs;
    o->grinding_bits = g; o->cap_height = ch;
    o->a0 = a0 % P; o->b0 = b0 % P; o->b_last = b_last % P;
    return ZO_OK;
}

/* air.rs:181-211 */
static int air_validate(const zo_air_params *p) {
    if (p->n_steps < 2 || !is_pow2(p->n_steps)) return ZO_INVALID_DOMAIN_SIZE;
    if (p->blowup < 4 || !is_pow2(p->blowup)) return ZO_INVALID_BLOWUP;
    if (p->num_queries == 0) return ZO_NO_QUERIES;
    if (p->final_size < 2 || !is_pow2(p->final_size)) return ZO_INVALID_DOMAIN_SIZE;
    if (p->cap_height > 8) return ZO_MALFORMED_INPUT;
    if (p->n_steps > UINT64_MAX / p->blowup || p->n_steps * p->blowup > MAX_DOMAIN)
        return ZO_INVALID_DOMAIN_SIZE;
    return ZO_OK;
}

/* air.rs:163-169 */
static int air_fri_params(const zo_air_params *p, fri_params *f) {
    int rc = fri_params_new(p->blowup, p->num_queries, p->final_size, f);
    if (rc) return rc;
    f->grinding_bits = p->grinding_bits; f->cap_height = p->cap_height;
    return ZO_OK;
}

/* air.rs:341-354 */
void zo_air_build_trace(uint32_t a0, uint32_t b0, size_t n, uint32_t *a, uint32_t *b) {
    if (n == 0) return;
    a[0] = a0; b[0] = b0;
    for (size_t i = 0; i + 1 < n; i++) { a[i + 1] = b[i]; b[i + 1] = f_add(a[i], b[i]); }
}

/* air.rs:754-766 */
static void air_absorb_params(const zo_air_params *p, zo_transcript *t) {
    uint8_t buf[56];
    put_u64(buf, p->n_steps); put_u64(buf + 8, p->blowup); put_u64(buf + 16, p->num_queries);
    put_u64(buf + 24, p->final_size); put_u32(buf + 32, p->grinding_bits);
    put_u64(buf + 36, p->cap_height); put_u32(buf + 44, p->a0); put_u32(buf + 48, p->b0);
    put_u32(buf + 52, p->b_last);
    absorb_s(t, "fib/params", buf, 56);
}

/* air.rs:770-779 (sequential chain of m multiplies, as in the reference) */
static uint32_t *lde_points(size_t m) {
    uint32_t omega = 0;
    primitive_root(m, &omega);
    uint32_t *pts = malloc(m * sizeof(uint32_t));
    uint32_t cur = LDE_SHIFT;
    for (size_t i = 0; i < m; i++) { pts[i] = cur; cur = f_mul(cur, omega); }
    return pts;
}

typedef struct {
    const uint32_t *lde_a; uint32_t *out; size_t m, n, offset;
    uint32_t omega_m, ratio, p0, w_last, coeff;
} linked_ctx;
static void linked_worker(void *vctx, size_t base, size_t len) {  /* air.rs:822-842 */
    linked_ctx *c = vctx;
    uint32_t x = f_mul(LDE_SHIFT, f_pow(c->omega_m, base));
    uint32_t xn = f_mul(c->p0, f_pow(c->ratio, base));
    uint32_t *den = malloc(len * sizeof(uint32_t)), *van = malloc(len * sizeof(uint32_t));
    for (size_t j = 0; j < len; j++) {
        den[j] = f_sub(x, c->w_last); van[j] = f_sub(xn, 1);
        x = f_mul(x, c->omega_m); xn = f_mul(xn, c->ratio);
    }
    zo_batch_invert(den, len);
    for (size_t j = 0; j < len; j++) {
        size_t i = base + j, s = i + c->offset;
        if (s >= c->m) s -= c->m;
        c->out[i] = f_add(c->lde_a[s], f_mul(f_mul(c->coeff, van[j]), den[j]));
    }
    free(den); free(van);
}

/* air.rs:806-844 B(x) = A(omega_n x) + delta * L_{n-1}(x) */
static int linked_lde(const uint32_t *lde_a, size_t m, size_t n, uint32_t b_last, uint32_t a0,
                      uint32_t *out) {
    if (!is_pow2(n) || m % n) return ZO_MALFORMED_INPUT;
    linked_ctx c;
    c.lde_a = lde_a; c.out = out; c.m = m; c.n = n; c.offset = m / n;
    primitive_root(m, &c.omega_m);
    uint32_t omega_n = 0;
    primitive_root(n, &omega_n);
    c.w_last = f_pow(omega_n, n - 1);
    c.ratio = f_pow(c.omega_m, n);
    c.p0 = f_pow(LDE_SHIFT, n);
    uint32_t n_inv = f_inv(f_from_u64(n));
    c.coeff = f_mul(f_mul(f_sub(b_last, a0), c.w_last), n_inv);
    for_each_indexed(m, 2048, linked_worker, &c);
    return ZO_OK;
}

typedef struct {
    const uint32_t *ca, *cb, *pts; ext4 *out; size_t m, offset;
    uint32_t w_last, a0, b0, b_last, p0, ratio; const ext4 *alpha;
} compose_ctx;
static void compose_worker(void *vctx, size_t base, size_t len) {  /* air.rs:886-928 */
    compose_ctx *c = vctx;
    uint32_t *da = malloc(len * 4), *db = malloc(len * 4), *iz = malloc(len * 4);
    uint32_t cur = f_mul(c->p0, f_pow(c->ratio, base));
    for (size_t j = 0; j < len; j++) {
        size_t i = base + j;
        da[j] = f_sub(c->pts[i], c->w_last);
        db[j] = f_sub(c->pts[i], 1);
        iz[j] = f_sub(cur, 1);
        cur = f_mul(cur, c->ratio);
    }
    zo_batch_invert(da, len);
    zo_batch_invert(db, len);
    for (size_t j = 0; j < len; j++) iz[j] = f_mul(iz[j], da[j]);
    zo_batch_invert(iz, len);
    for (size_t j = 0; j < len; j++) {
        size_t i = base + j, nx = i + c->offset;
        if (nx >= c->m) nx -= c->m;
        uint32_t a = c->ca[i], b = c->cb[i];
        uint32_t t1 = f_mul(f_sub(c->ca[nx], b), iz[j]);
        uint32_t t2 = f_mul(f_sub(c->cb[nx], f_add(a, b)), iz[j]);
        uint32_t ba = f_mul(f_sub(a, c->a0), db[j]);
        uint32_t bb = f_mul(f_sub(b, c->b0), db[j]);
        uint32_t bo = f_mul(f_sub(b, c->b_last), da[j]);
        ext4 acc = e_mul_base(c->alpha[0], t1);
        acc = e_add(acc, e_mul_base(c->alpha[1], t2));
        acc = e_add(acc, e_mul_base(c->alpha[2], ba));
        acc = e_add(acc, e_mul_base(c->alpha[3], bb));
        acc = e_add(acc, e_mul_base(c->alpha[4], bo));
        c->out[i] = acc;
    }
    free(da); free(db); free(iz);
}

/* air.rs:938-962 (used by verify) */
static ext4 air_composition_at(uint32_t a, uint32_t b, uint32_t an, uint32_t bn, uint32_t x,
                               uint32_t w_last, const zo_air_params *p, size_t n,
                               const ext4 alpha[5]) {
    uint32_t van = f_sub(f_pow(x, n), 1);
    uint32_t zt = f_mul(van, f_inv(f_sub(x, w_last)));
    uint32_t t1 = f_mul(f_sub(an, b), f_inv(zt));
    uint32_t t2 = f_mul(f_sub(bn, f_add(a, b)), f_inv(zt));
    uint32_t ba = f_mul(f_sub(a, p->a0), f_inv(f_sub(x, 1)));
    uint32_t bb = f_mul(f_sub(b, p->b0), f_inv(f_sub(x, 1)));
    uint32_t bo = f_mul(f_sub(b, p->b_last), f_inv(f_sub(x, w_last)));
    ext4 acc = e_mul_base(alpha[0], t1);
    acc = e_add(acc, e_mul_base(alpha[1], t2));
    acc = e_add(acc, e_mul_base(alpha[2], ba));
    acc = e_add(acc, e_mul_base(alpha[3], bb));
    return e_add(acc, e_mul_base(alpha[4], bo));
}

/* air.rs:847-929 compose over caller-chosen points, as the reference's own
 * batched-vs-scalar test calls it (air.rs:1155-1242): LDE points and the unit
 * domain, whose singular rows map zero denominators to zero. Fewer than two
 * points take the scalar fallback (air.rs:863-882). */
int zo_air_compose(const uint32_t *ca, const uint32_t *cb, const uint32_t *pts, size_t m,
                   uint32_t w_last, uint32_t a0, uint32_t b0, uint32_t b_last, size_t n,
                   size_t offset, const uint32_t *alphas, uint32_t *out) {
    ext4 alpha[5];
    for (int k = 0; k < 5; k++)
        for (int e = 0; e < 4; e++) alpha[k].c[e] = alphas[4 * k + e];
    if (m < 2) {
        zo_air_params p = {0};
        p.a0 = a0; p.b0 = b0; p.b_last = b_last;
        for (size_t i = 0; i < m; i++) {
            size_t nx = (i + offset) % m;
            ext4 v = air_composition_at(ca[i], cb[i], ca[nx], cb[nx], pts[i], w_last, &p, n, alpha);
            memcpy(out + 4 * i, v.c, 16);
        }
        return ZO_OK;
    }
    compose_ctx c;
    c.ca = ca; c.cb = cb; c.pts = pts; c.m = m; c.offset = offset;
    c.w_last = w_last; c.a0 = a0; c.b0 = b0; c.b_last = b_last;
    c.p0 = f_pow(pts[0], n);
    c.ratio = f_pow(f_mul(pts[1], f_inv(pts[0])), n);
    c.alpha = alpha;
    c.out = (ext4 *)out;
    for_each_indexed(m, 2048, compose_worker, &c);
    return ZO_OK;
}

/* air.rs:938-962 composition_at at one point */
void zo_air_composition_at(uint32_t a, uint32_t b, uint32_t an, uint32_t bn, uint32_t x,
                           uint32_t w_last, uint32_t a0, uint32_t b0, uint32_t b_last, size_t n,
                           const uint32_t *alphas, uint32_t *out) {
    ext4 alpha[5];
    for (int k = 0; k < 5; k++)
        for (int e = 0; e < 4; e++) alpha[k].c[e] = alphas[4 * k + e];
    zo_air_params p = {0};
    p.a0 = a0; p.b0 = b0; p.b_last = b_last;
    ext4 v = air_composition_at(a, b, an, bn, x, w_last, &p, n, alpha);
    memcpy(out, v.c, 16);
}

/* air.rs:485-599 prove_inner; lde_b given (from linked_lde or a second NTT) */
static int air_prove_inner(const zo_air_params *params, uint32_t *lde_a, uint32_t *lde_b,
                           size_t m, size_t degree_bound, zo_transcript *t, uint8_t **proof,
                           size_t *proof_len) {
    /* m = LDE length: n * blowup, or the padded masked length (air.rs:505-513) */
    size_t n = params->n_steps, offset = m / n;
    uint32_t omega_base = 0;
    primitive_root(n, &omega_base);
    /* Joint rows A || B, 8 bytes each; 64-byte leaves of 8 rows (air.rs:520-531). */
    uint8_t *flat = malloc(8 * m);
    for (size_t i = 0; i < m; i++) { put_u32(flat + 8 * i, lde_a[i]); put_u32(flat + 8 * i + 4, lde_b[i]); }
    mtree tree;
    mtree_from_flat64(flat, 8 * m, &tree);
    size_t drop, depth;
    capped_shape(m / 8, params->cap_height, &drop, &depth);
    size_t ncap;
    const digest *cap = mtree_cap(&tree, drop, &ncap);
    absorb_s(t, "fib/trace", (const uint8_t *)cap, 32 * ncap);
    ext4 alpha[5];
    for (int k = 0; k < 5; k++) alpha[k] = challenge_ext(t, "fib/alpha");

    uint32_t *pts = lde_points(m);
    compose_ctx c;
    c.ca = lde_a; c.cb = lde_b; c.pts = pts; c.m = m; c.offset = offset;
    c.w_last = f_pow(omega_base, n - 1);
    c.a0 = params->a0; c.b0 = params->b0; c.b_last = params->b_last;
    c.p0 = f_pow(pts[0], n);
    c.ratio = f_pow(f_mul(pts[1], f_inv(pts[0])), n);
    c.alpha = alpha;
    c.out = malloc(m * sizeof(ext4));
    for_each_indexed(m, 2048, compose_worker, &c);
    free(pts);

    fri_params fp;
    air_fri_params(params, &fp);
    fri_state st;
    /* fri.rs:527-549 commit_ext_evals_owned: poly_len echoes lde_len. */
    int rc = fri_commit_inner(c.out, m, degree_bound, m, &fp, t, &st);
    if (rc) { mtree_free(&tree); free(flat); return rc; }

    writer w = {0};
    w_byte(&w, VERSION);
    w_cap(&w, cap, ncap);
    fri_write_commitment(&w, &st);
    uint64_t *idx = malloc(params->num_queries * sizeof(uint64_t));
    rc = fri_open_write(&st, t, &w, idx);
    if (!rc) {
        /* air.rs:565-591 trace openings */
        uint32_t log_m = log2u(m);
        w_u32(&w, (uint32_t)params->num_queries);
        for (size_t k = 0; k < params->num_queries; k++) {
            size_t index = brev(idx[k], log_m);
            size_t shifted = (index + offset) % m;
            size_t base = index & ~(size_t)7, sbase = shifted & ~(size_t)7;
            path_t p1, p2;
            mtree_prove_capped(&tree, base / 8, drop, &p1);
            mtree_prove_capped(&tree, sbase / 8, drop, &p2);
            w_u64(&w, index);
            w_u32(&w, lde_a[index]); w_u32(&w, lde_b[index]);
            w_u32(&w, lde_a[shifted]); w_u32(&w, lde_b[shifted]);
            w_path(&w, &p1); w_path(&w, &p2);
            w_bytes(&w, flat + 8 * base, 64);
            w_bytes(&w, flat + 8 * sbase, 64);
            free(p1.s); free(p2.s);
        }
    }
    free(idx);
    fri_state_free(&st);
    mtree_free(&tree);
    free(flat);
    if (rc) { free(w.b); return rc; }
    *proof = w.b; *proof_len = w.n;
    return ZO_OK;
}

/* air.rs:365-372 prove: trace -> interpolate -> LDE A -> linked LDE B */
int zo_air_prove(const zo_air_params *params, zo_transcript *t, uint8_t **proof,
                 size_t *proof_len) {
    int rc = air_validate(params);
    if (rc) return rc;
    size_t n = params->n_steps, m = n * params->blowup;
    uint32_t *a = malloc(n * 4), *b = malloc(n * 4);
    zo_air_build_trace(params->a0, params->b0, n, a, b);
    uint32_t actual_b_last = b[n - 1];
    zo_ntt_inverse(a, n);
    air_absorb_params(params, t);
    uint32_t *lde_a = malloc(m * 4), *lde_b = malloc(m * 4);
    zo_evaluate_on_coset(a, n, params->blowup, LDE_SHIFT, lde_a);
    linked_lde(lde_a, m, n, actual_b_last, params->a0, lde_b);
    rc = air_prove_inner(params, lde_a, lde_b, m, n - 1, t, proof, proof_len);
    free(a); free(b); free(lde_a); free(lde_b);
    return rc;
}

/* air.rs:381-399 prove_with_trace: two independent NTTs */
int zo_air_prove_with_trace(const zo_air_params *params, const uint32_t *col_a,
                            const uint32_t *col_b, zo_transcript *t, uint8_t **proof,
                            size_t *proof_len) {
    int rc = air_validate(params);
    if (rc) return rc;
    size_t n = params->n_steps, m = n * params->blowup;
    uint32_t *ca = malloc(n * 4), *cb = malloc(n * 4);
    memcpy(ca, col_a, n * 4); memcpy(cb, col_b, n * 4);
    zo_ntt_inverse(ca, n); zo_ntt_inverse(cb, n);
    air_absorb_params(params, t);
    uint32_t *lde_a = malloc(m * 4), *lde_b = malloc(m * 4);
    zo_evaluate_on_coset(ca, n, params->blowup, LDE_SHIFT, lde_a);
    zo_evaluate_on_coset(cb, n, params->blowup, LDE_SHIFT, lde_b);
    rc = air_prove_inner(params, lde_a, lde_b, m, n - 1, t, proof, proof_len);
    free(ca); free(cb); free(lde_a); free(lde_b);
    return rc;
}

/* rng.rs:22-35 quarter round, :40-73 block (RFC 8439 section 2.3) */
static void chacha_qr(uint32_t *x, int a, int b, int c, int d) {
    x[a] += x[b]; x[d] ^= x[a]; x[d] = (x[d] << 16) | (x[d] >> 16);
    x[c] += x[d]; x[b] ^= x[c]; x[b] = (x[b] << 12) | (x[b] >> 20);
    x[a] += x[b]; x[d] ^= x[a]; x[d] = (x[d] << 8) | (x[d] >> 24);
    x[c] += x[d]; x[b] ^= x[c]; x[b] = (x[b] << 7) | (x[b] >> 25);
}
void zo_chacha20_block(const uint8_t key[32], uint32_t counter, const uint8_t nonce[12],
                       uint8_t out[64]) {
    uint32_t x[16], in[16];
    in[0] = 0x61707865u; in[1] = 0x3320646eu; in[2] = 0x79622d32u; in[3] = 0x6b206574u;
    for (int i = 0; i < 8; i++) in[4 + i] = get_u32(key + 4 * i);
    in[12] = counter;
    for (int i = 0; i < 3; i++) in[13 + i] = get_u32(nonce + 4 * i);
    memcpy(x, in, sizeof x);
    for (int r = 0; r < 10; r++) {
        chacha_qr(x, 0, 4, 8, 12); chacha_qr(x, 1, 5, 9, 13);
        chacha_qr(x, 2, 6, 10, 14); chacha_qr(x, 3, 7, 11, 15);
        chacha_qr(x, 0, 5, 10, 15); chacha_qr(x, 1, 6, 11, 12);
        chacha_qr(x, 2, 7, 8, 13); chacha_qr(x, 3, 4, 9, 14);
    }
    for (int i = 0; i < 16; i++) put_u32(out + 4 * i, x[i] + in[i]);
}

/* rng.rs:101-112 ChaCha20::new */
void zo_chacha20_init(zo_chacha20 *s, const uint8_t key[32], const uint8_t nonce[12]) {
    memcpy(s->key, key, 32); memcpy(s->nonce, nonce, 12);
    s->counter = 0; memset(s->block, 0, 64); s->used = 64;
}
/* rng.rs:115-131 fill_bytes */
void zo_chacha20_fill(zo_chacha20 *s, uint8_t *out, size_t n) {
    size_t done = 0;
    while (done < n) {
        if (s->used == 64) {
            zo_chacha20_block(s->key, s->counter, s->nonce, s->block);
            s->counter += 1;
            s->used = 0;
        }
        size_t take = 64 - s->used < n - done ? 64 - s->used : n - done;
        memcpy(out + done, s->block + s->used, take);
        s->used += (uint32_t)take;
        done += take;
    }
}
/* rng.rs:157-167 next_field: rejection above 2p */
uint32_t zo_chacha20_next_field(zo_chacha20 *s) {
    const uint64_t limit = (((uint64_t)1 << 32) / P) * P;
    for (;;) {
        uint8_t w[4];
        zo_chacha20_fill(s, w, 4);
        uint64_t v = get_u32(w);
        if (v < limit) return (uint32_t)(v % P);
    }
}

/* blind.rs:40-78 mask_coeffs: T + (x^n - 1) R, padded to a power of two */
static uint32_t *mask_coeffs(const uint32_t *coeffs, size_t n, size_t n_rand, zo_chacha20 *rng,
                             size_t *padded_out) {
    size_t total = n + n_rand, padded = 1;
    while (padded < total) padded <<= 1;
    uint32_t *r = malloc((n_rand ? n_rand : 1) * 4);
    for (size_t i = 0; i < n_rand; i++) r[i] = zo_chacha20_next_field(rng);
    uint32_t *out = calloc(padded, 4);
    for (size_t i = 0; i < n; i++) out[i] = f_add(out[i], coeffs[i]);
    for (size_t i = 0; i < n_rand; i++) {
        out[i + n] = f_add(out[i + n], r[i]);
        out[i] = f_sub(out[i], r[i]);
    }
    free(r);
    *padded_out = padded;
    return out;
}

/* air.rs:439-464 prove_zk: both columns masked, then prove_from_coeffs */
int zo_air_prove_zk(const zo_air_params *params, size_t n_rand, zo_chacha20 *rng,
                    zo_transcript *t, uint8_t **proof, size_t *proof_len) {
    int rc = air_validate(params);
    if (rc) return rc;
    if (params->num_queries > SIZE_MAX / 16) return ZO_MALFORMED_INPUT;
    if (n_rand < 16 * params->num_queries) return ZO_MALFORMED_INPUT;
    size_t n = params->n_steps;
    uint32_t *a = malloc(n * 4), *b = malloc(n * 4);
    zo_air_build_trace(params->a0, params->b0, n, a, b);
    zo_ntt_inverse(a, n);
    zo_ntt_inverse(b, n);
    size_t pa = 0, pb = 0;
    if (n + n_rand < n) { free(a); free(b); return ZO_INVALID_DOMAIN_SIZE; }
    size_t total = n + n_rand, padded = 1;
    while (padded < total) padded <<= 1;
    if (padded > ((size_t)1 << TWO_ADICITY)) { free(a); free(b); return ZO_INVALID_DOMAIN_SIZE; }
    uint32_t *ma = mask_coeffs(a, n, n_rand, rng, &pa);
    uint32_t *mb = mask_coeffs(b, n, n_rand, rng, &pb);
    free(a); free(b);
    size_t m = pa * params->blowup;
    if (pa > SIZE_MAX / params->blowup || m > ((size_t)1 << TWO_ADICITY)) {
        free(ma); free(mb); return ZO_INVALID_DOMAIN_SIZE;
    }
    air_absorb_params(params, t);
    uint32_t *lde_a = malloc(m * 4), *lde_b = malloc(m * 4);
    zo_evaluate_on_coset(ma, pa, params->blowup, LDE_SHIFT, lde_a);
    zo_evaluate_on_coset(mb, pb, params->blowup, LDE_SHIFT, lde_b);
    free(ma); free(mb);
    rc = air_prove_inner(params, lde_a, lde_b, m, n + n_rand - 1, t, proof, proof_len);
    free(lde_a); free(lde_b);
    return rc;
}

typedef struct {
    size_t index; uint32_t a, b, an, bn; path_t path, spath; uint8_t leaf[64], sleaf[64];
} air_open_t;

/* air.rs:607-752 verify (decodes with air.rs:291-331 from_bytes) */
int zo_air_verify(const zo_air_params *params, const uint8_t *proof, size_t proof_len,
                  zo_transcript *t) {
    int rc = air_validate(params);
    if (rc) return rc;
    reader r = {proof, proof_len, 0, 0};
    if (r_byte(&r) != VERSION) return ZO_MALFORMED_INPUT;
    size_t ncap;
    digest *column_cap = r_cap(&r, &ncap);
    fri_decoded d;
    fri_read(&r, &d);
    size_t nopen = r_count(&r, MAX_QUERIES);
    air_open_t *op = NULL;
    size_t got = 0;
    if (!r.err && nopen * 8 <= r.n - r.pos) {
        op = calloc(nopen ? nopen : 1, sizeof(air_open_t));
        for (size_t k = 0; k < nopen && !r.err; k++) {
            got = k + 1;
            op[k].index = r_u64(&r);
            op[k].a = r_field(&r); op[k].b = r_field(&r);
            op[k].an = r_field(&r); op[k].bn = r_field(&r);
            r_path(&r, &op[k].path); r_path(&r, &op[k].spath);
            const uint8_t *l = r_take(&r, 64);
            if (l) memcpy(op[k].leaf, l, 64);
            const uint8_t *s = r_take(&r, 64);
            if (s) memcpy(op[k].sleaf, s, 64);
        }
    } else r.err = 1;
    if (r.err || r.pos != r.n) { rc = ZO_MALFORMED_INPUT; goto out; }

    size_t n = params->n_steps;
    size_t m = d.lde_len;
    if (params->blowup > SIZE_MAX / n) { rc = ZO_FRI_VERIFICATION_FAILED; goto out; }
    size_t expected_m = n * params->blowup;
    if (m < expected_m || m % expected_m) { rc = ZO_FRI_VERIFICATION_FAILED; goto out; }
    if (m == expected_m) {
        if (d.degree_bound != n - 1) { rc = ZO_FRI_VERIFICATION_FAILED; goto out; }
    } else if (d.degree_bound >= m / params->blowup) { rc = ZO_FRI_VERIFICATION_FAILED; goto out; }
    if (d.poly_len != m) { rc = ZO_FRI_VERIFICATION_FAILED; goto out; }
    size_t offset = m / n;
    air_absorb_params(params, t);
    if (nopen != params->num_queries) { rc = ZO_FRI_VERIFICATION_FAILED; goto out; }
    absorb_s(t, "fib/trace", (const uint8_t *)column_cap, 32 * ncap);
    ext4 alpha[5];
    for (int k = 0; k < 5; k++) alpha[k] = challenge_ext(t, "fib/alpha");
    fri_params fp;
    if ((rc = air_fri_params(params, &fp))) goto out;
    uint64_t *idx = malloc((d.nq ? d.nq : 1) * sizeof(uint64_t));
    rc = fri_verify(&d, &fp, t, idx);
    if (!rc) {
        uint32_t omega_base = 0, omega_m = 0;
        primitive_root(n, &omega_base);
        primitive_root(m, &omega_m);
        uint32_t w_last = f_pow(omega_base, n - 1);
        uint32_t log_m = log2u(m);
        for (size_t k = 0; k < nopen && !rc; k++) {
            size_t index = brev(idx[k], log_m);
            if (op[k].index != index) { rc = ZO_FRI_VERIFICATION_FAILED; break; }
            if (m % 8) { rc = ZO_FRI_VERIFICATION_FAILED; break; }
            size_t drop, depth;
            capped_shape(m / 8, params->cap_height, &drop, &depth);
            if (ncap != ((size_t)1 << drop) || op[k].path.n != depth - drop ||
                op[k].spath.n != depth - drop) { rc = ZO_BAD_MERKLE_PATH; break; }
            size_t ro = (index & 7) * 8;
            if (get_u32(op[k].leaf + ro) != op[k].a || get_u32(op[k].leaf + ro + 4) != op[k].b)
                { rc = ZO_BAD_MERKLE_PATH; break; }
            size_t ei = (index / 8) >> (depth - drop);
            if (ei >= ncap || !verify_capped64(column_cap[ei], op[k].leaf, index / 8, depth, &op[k].path))
                { rc = ZO_BAD_MERKLE_PATH; break; }
            size_t shifted = (index + offset) % m;
            size_t so = (shifted & 7) * 8;
            if (get_u32(op[k].sleaf + so) != op[k].an || get_u32(op[k].sleaf + so + 4) != op[k].bn)
                { rc = ZO_BAD_MERKLE_PATH; break; }
            size_t sei = (shifted / 8) >> (depth - drop);
            if (sei >= ncap || !verify_capped64(column_cap[sei], op[k].sleaf, shifted / 8, depth, &op[k].spath))
                { rc = ZO_BAD_MERKLE_PATH; break; }
            uint32_t x = f_mul(LDE_SHIFT, f_pow(omega_m, index));
            ext4 expected = air_composition_at(op[k].a, op[k].b, op[k].an, op[k].bn, x, w_last,
                                               params, n, alpha);
            if (d.q[k].n == 0) { rc = ZO_FRI_VERIFICATION_FAILED; break; }
            if (!e_eq(d.q[k].f[0].v[idx[k] % 4], expected)) { rc = ZO_FRI_VERIFICATION_FAILED; break; }
        }
    }
    free(idx);
out:
    for (size_t k = 0; k < got; k++) { free(op[k].path.s); free(op[k].spath.s); }
    free(op);
    free(column_cap);
    fri_decoded_free(&d);
    return rc;
}

/* ------------------------------------------------------------------------ */
/* fold.rs — hash-chained Fibonacci segments with one batched FRI (IVC)     */
/* ------------------------------------------------------------------------ */

/* fold.rs:72-111 Params::new */
int zo_fold_params_new(uint64_t seg, uint64_t blowup, uint64_t q, uint64_t final_size,
                       uint32_t in_a, uint32_t in_b, uint32_t out_b, zo_fold_params *o) {
    if (seg < 2 || !is_pow2(seg)) return ZO_INVALID_DOMAIN_SIZE;
    if (blowup < 4 || !is_pow2(blowup)) return ZO_INVALID_BLOWUP;
    if (q == 0) return ZO_NO_QUERIES;
    if (final_size < 2 || !is_pow2(final_size)) return ZO_INVALID_DOMAIN_SIZE;
    if (seg > UINT64_MAX / blowup || seg * blowup > MAX_DOMAIN) return ZO_INVALID_DOMAIN_SIZE;
    o->seg_steps = seg; o->blowup = blowup; o->num_queries = q; o->final_size = final_size;
    o->grinding_bits = 0; o->cap_height = 0;
    o->in_a = in_a % P; o->in_b = in_b % P; o->out_b = out_b % P;
    return ZO_OK;
}

/* fold.rs:136-171 Params::for_security */
int zo_fold_for_security(uint64_t seg, uint32_t in_a, uint32_t in_b, uint32_t out_b,
                         uint32_t target, zo_fold_params *o) {
    if (seg < 2 || !is_pow2(seg)) return ZO_INVALID_DOMAIN_SIZE;
    uint64_t blowup = 16;
    if (seg > UINT64_MAX / blowup || seg * blowup > MAX_DOMAIN) return ZO_INVALID_DOMAIN_SIZE;
    size_t lde = seg * blowup;
    uint32_t mb = zo_fri_composition_millibits(lde, seg - 1);
    size_t q; uint32_t g;
    zo_fri_tune_strength(target, mb, &q, &g);
    size_t fs, ch;
    zo_fri_tune_shape(lde, q, lde, 24, 1, &fs, &ch);
    o->seg_steps = seg; o->blowup = blowup; o->num_queries = q; o->final_size = fs;
    o->grinding_bits = g; o->cap_height = ch;
    o->in_a = in_a % P; o->in_b = in_b % P; o->out_b = out_b % P;
    return ZO_OK;
}

/* fold.rs:186-222 validate */
static int fold_validate(const zo_fold_params *p) {
    if (p->seg_steps < 2 || !is_pow2(p->seg_steps)) return ZO_INVALID_DOMAIN_SIZE;
    if (p->blowup < 4 || !is_pow2(p->blowup)) return ZO_INVALID_BLOWUP;
    if (p->num_queries == 0) return ZO_NO_QUERIES;
    if (p->final_size < 2 || !is_pow2(p->final_size)) return ZO_INVALID_DOMAIN_SIZE;
    if (p->cap_height > 8) return ZO_MALFORMED_INPUT;
    if (p->seg_steps > UINT64_MAX / p->blowup || p->seg_steps * p->blowup > MAX_DOMAIN)
        return ZO_INVALID_DOMAIN_SIZE;
    return ZO_OK;
}

/* fold.rs:177-184 fri_params */
static int fold_fri_params(const zo_fold_params *p, fri_params *f) {
    int rc = fri_params_new(p->blowup, p->num_queries, p->final_size, f);
    if (rc) return rc;
    f->grinding_bits = p->grinding_bits; f->cap_height = p->cap_height;
    return ZO_OK;
}

/* fold.rs:729-741 */
static void fold_absorb_params(const zo_fold_params *p, zo_transcript *t) {
    uint8_t b[64];
    put_u64(b, p->seg_steps); put_u64(b + 8, p->blowup); put_u64(b + 16, p->num_queries);
    put_u64(b + 24, p->final_size); put_u32(b + 32, p->grinding_bits);
    put_u64(b + 36, p->cap_height); put_u32(b + 44, p->in_a); put_u32(b + 48, p->in_b);
    put_u32(b + 52, p->out_b);
    absorb_s(t, "fold/params", b, 56);
}

typedef struct { uint32_t in_a, in_b, out_a, out_b; } fold_claims;

/* fold.rs:743-751 */
static void fold_absorb_step(const fold_claims *c, zo_transcript *t) {
    uint8_t b[16];
    put_u32(b, c->in_a); put_u32(b + 4, c->in_b); put_u32(b + 8, c->out_a); put_u32(b + 12, c->out_b);
    absorb_s(t, "fold/step", b, 16);
}

typedef struct {
    fold_claims claims;
    uint32_t *lde[2];
    mtree tree;
    ext4 *composition;
} fold_step;

typedef struct {
    zo_fold_params params;
    fold_step *steps;
    size_t n, cap;
} fold_acc;

void *zo_fold_new(const zo_fold_params *p) {  /* fold.rs:379-384 */
    fold_acc *a = calloc(1, sizeof *a);
    a->params = *p;
    return a;
}

void zo_fold_free(void *acc) {
    fold_acc *a = acc;
    if (!a) return;
    for (size_t i = 0; i < a->n; i++) {
        free(a->steps[i].lde[0]); free(a->steps[i].lde[1]);
        mtree_free(&a->steps[i].tree); free(a->steps[i].composition);
    }
    free(a->steps);
    free(a);
}

/* fold.rs:856-879 composition_at (quotient form) */
static ext4 fold_composition_at(uint32_t a, uint32_t b, uint32_t an, uint32_t bn, uint32_t x,
                                uint32_t w_last, const fold_claims *c, size_t s,
                                const ext4 alpha[6]) {
    uint32_t vanishing = f_sub(f_pow(x, s), 1);
    uint32_t z_trans = f_mul(vanishing, f_inv(f_sub(x, w_last)));
    uint32_t inv_z = f_inv(z_trans);
    uint32_t inv_b = f_inv(f_sub(x, 1)), inv_a = f_inv(f_sub(x, w_last));
    uint32_t t[6] = {
        f_mul(f_sub(an, b), inv_z), f_mul(f_sub(bn, f_add(a, b)), inv_z),
        f_mul(f_sub(a, c->in_a), inv_b), f_mul(f_sub(b, c->in_b), inv_b),
        f_mul(f_sub(a, c->out_a), inv_a), f_mul(f_sub(b, c->out_b), inv_a),
    };
    ext4 acc = e_mul_base(alpha[0], t[0]);
    for (int k = 1; k < 6; k++) acc = e_add(acc, e_mul_base(alpha[k], t[k]));
    return acc;
}

/* fold.rs:407-488 add_segment */
int zo_fold_add_segment(void *acc, const uint32_t *col_a, const uint32_t *col_b, size_t len,
                        zo_transcript *t) {
    fold_acc *a = acc;
    int rc = fold_validate(&a->params);
    if (rc) return rc;
    size_t s = a->params.seg_steps;
    if (len != s) return ZO_MALFORMED_INPUT;
    fold_claims c = {col_a[0] % P, col_b[0] % P, col_a[s - 1] % P, col_b[s - 1] % P};
    if (a->n == 0) fold_absorb_params(&a->params, t);
    fold_absorb_step(&c, t);
    size_t m = s * a->params.blowup;
    fold_step st;
    memset(&st, 0, sizeof st);
    st.claims = c;
    for (int k = 0; k < 2; k++) {
        uint32_t *coeffs = malloc(s * 4);
        for (size_t i = 0; i < s; i++) coeffs[i] = (k ? col_b : col_a)[i] % P;
        zo_ntt_inverse(coeffs, s);
        st.lde[k] = malloc(m * 4);
        zo_evaluate_on_coset(coeffs, s, a->params.blowup, LDE_SHIFT, st.lde[k]);
        free(coeffs);
    }
    size_t offset = m / s;
    uint8_t *flat = malloc(m * 8);
    for (size_t i = 0; i < m; i++) { put_u32(flat + 8 * i, st.lde[0][i]); put_u32(flat + 8 * i + 4, st.lde[1][i]); }
    mtree_from_flat(flat, m * 8, 8, &st.tree);
    free(flat);
    size_t drop, depth;
    capped_shape(m, a->params.cap_height, &drop, &depth);
    size_t ncap;
    const digest *cap = mtree_cap(&st.tree, drop, &ncap);
    absorb_s(t, "fold/trace", (const uint8_t *)cap, 32 * ncap);
    ext4 alpha[6];
    for (int k = 0; k < 6; k++) alpha[k] = challenge_ext(t, "fold/alpha");
    /* compose_step (fold.rs:785-850): batched inverses over the whole domain */
    uint32_t omega_m, omega_s;
    primitive_root(m, &omega_m);
    primitive_root(s, &omega_s);
    uint32_t w_last = f_pow(omega_s, s - 1);
    uint32_t *da = malloc(m * 4), *db = malloc(m * 4), *zt = malloc(m * 4), *xs = malloc(m * 4);
    uint32_t x = LDE_SHIFT;
    for (size_t i = 0; i < m; i++) {
        xs[i] = x;
        da[i] = f_sub(x, w_last);
        db[i] = f_sub(x, 1);
        x = f_mul(x, omega_m);
    }
    zo_batch_invert(da, m);
    zo_batch_invert(db, m);
    for (size_t i = 0; i < m; i++) zt[i] = f_mul(f_sub(f_pow(xs[i], s), 1), da[i]);
    zo_batch_invert(zt, m);
    st.composition = malloc(m * sizeof(ext4));
    for (size_t i = 0; i < m; i++) {
        uint32_t av = st.lde[0][i], bv = st.lde[1][i];
        uint32_t an = st.lde[0][(i + offset) % m], bn = st.lde[1][(i + offset) % m];
        uint32_t tv[6] = {
            f_mul(f_sub(an, bv), zt[i]), f_mul(f_sub(bn, f_add(av, bv)), zt[i]),
            f_mul(f_sub(av, c.in_a), db[i]), f_mul(f_sub(bv, c.in_b), db[i]),
            f_mul(f_sub(av, c.out_a), da[i]), f_mul(f_sub(bv, c.out_b), da[i]),
        };
        ext4 accv = e_mul_base(alpha[0], tv[0]);
        for (int k = 1; k < 6; k++) accv = e_add(accv, e_mul_base(alpha[k], tv[k]));
        st.composition[i] = accv;
    }
    free(da); free(db); free(zt); free(xs);
    if (a->n == a->cap) {
        a->cap = a->cap ? 2 * a->cap : 4;
        a->steps = realloc(a->steps, a->cap * sizeof(fold_step));
    }
    a->steps[a->n++] = st;
    return ZO_OK;
}

static size_t bit_reverse_index(size_t x, uint32_t bits) {  /* fold.rs:881-888 */
    size_t out = 0;
    for (uint32_t i = 0; i < bits; i++) { out = (out << 1) | (x & 1); x >>= 1; }
    return out;
}

/* fold.rs:494-560 finalize, bytes per fold.rs:281-309 */
int zo_fold_finalize(void *acc, zo_transcript *t, uint8_t **proof, size_t *proof_len) {
    fold_acc *a = acc;
    if (a->n == 0) return ZO_EMPTY_INPUT;
    const zo_fold_params *p = &a->params;
    size_t s = p->seg_steps, m = s * p->blowup;
    ext4 *gamma = malloc(a->n * sizeof(ext4));
    for (size_t k = 0; k < a->n; k++) gamma[k] = challenge_ext(t, "fold/gamma");
    ext4 *combined = calloc(m, sizeof(ext4));
    for (size_t i = 0; i < m; i++)
        for (size_t k = 0; k < a->n; k++)
            combined[i] = e_add(combined[i], e_mul(gamma[k], a->steps[k].composition[i]));
    free(gamma);
    fri_params fp;
    int rc = fold_fri_params(p, &fp);
    if (rc) { free(combined); return rc; }
    /* fri::commit_ext_evals (fri.rs:508-549): the bound check, then commit_inner */
    rc = fri_params_validate(&fp);
    if (!rc && s - 1 >= m) rc = ZO_MALFORMED_INPUT;
    if (rc) { free(combined); return rc; }
    fri_state st;
    rc = fri_commit_inner(combined, m, s - 1, m, &fp, t, &st);
    if (rc) return rc;
    writer fc = {0}, fo = {0};
    fri_write_commitment(&fc, &st);
    uint64_t *idx = malloc(p->num_queries * sizeof(uint64_t));
    rc = fri_open_write(&st, t, &fo, idx);
    if (rc) { fri_state_free(&st); free(fc.b); free(fo.b); free(idx); return rc; }
    uint32_t log_m = log2u(m);
    size_t offset = m / s, drop, depth;
    capped_shape(m, p->cap_height, &drop, &depth);
    writer w = {0};
    w_byte(&w, VERSION);
    w_u32(&w, (uint32_t)a->n);
    for (size_t k = 0; k < a->n && !rc; k++) {
        fold_step *sp = &a->steps[k];
        w_u32(&w, sp->claims.in_a); w_u32(&w, sp->claims.in_b);
        w_u32(&w, sp->claims.out_a); w_u32(&w, sp->claims.out_b);
        size_t ncap;
        const digest *cap = mtree_cap(&sp->tree, drop, &ncap);
        w_cap(&w, cap, ncap);
        w_u32(&w, (uint32_t)p->num_queries);
        for (size_t qi = 0; qi < p->num_queries && !rc; qi++) {
            size_t index = bit_reverse_index(idx[qi], log_m);
            size_t shifted = (index + offset) % m;
            w_u64(&w, index);
            w_u32(&w, sp->lde[0][index]); w_u32(&w, sp->lde[1][index]);
            w_u32(&w, sp->lde[0][shifted]); w_u32(&w, sp->lde[1][shifted]);
            path_t pa, pb;
            rc = mtree_prove_capped(&sp->tree, index, drop, &pa);
            if (rc) break;
            rc = mtree_prove_capped(&sp->tree, shifted, drop, &pb);
            if (rc) { free(pa.s); break; }
            w_path(&w, &pa); w_path(&w, &pb);
            free(pa.s); free(pb.s);
        }
    }
    if (!rc) { w_bytes(&w, fc.b, fc.n); w_bytes(&w, fo.b, fo.n); }
    fri_state_free(&st);
    free(fc.b); free(fo.b); free(idx);
    if (rc) { free(w.b); return rc; }
    *proof = w.b; *proof_len = w.n;
    return ZO_OK;
}

typedef struct { size_t index; uint32_t cols[4]; path_t path, spath; } fold_open_t;
typedef struct { fold_claims claims; digest *cap; size_t ncap; fold_open_t *op; size_t nop; } fold_step_t;

/* fold.rs:572-667 verify (decoding per fold.rs:312-355) */
int zo_fold_verify(const zo_fold_params *p, const uint8_t *proof, size_t proof_len,
                   zo_transcript *t) {
    int rc = fold_validate(p);
    if (rc) return rc;
    reader r = {proof, proof_len, 0, 0};
    if (r_byte(&r) != VERSION) return ZO_MALFORMED_INPUT;
    size_t nsteps = r_count(&r, 1u << 20);
    if (r.err) return ZO_MALFORMED_INPUT;
    if (nsteps * 20 > r.n - r.pos) return ZO_MALFORMED_INPUT;
    fold_step_t *st = calloc(nsteps ? nsteps : 1, sizeof(fold_step_t));
    size_t got = 0;
    fri_decoded d;
    memset(&d, 0, sizeof d);
    for (size_t k = 0; k < nsteps && !r.err; k++) {
        got = k + 1;
        st[k].claims.in_a = r_field(&r); st[k].claims.in_b = r_field(&r);
        st[k].claims.out_a = r_field(&r); st[k].claims.out_b = r_field(&r);
        st[k].cap = r_cap(&r, &st[k].ncap);
        size_t no = r_count(&r, MAX_QUERIES);
        if (r.err || no * 24 > r.n - r.pos) { r.err = 1; break; }
        st[k].op = calloc(no ? no : 1, sizeof(fold_open_t));
        for (size_t i = 0; i < no && !r.err; i++) {
            st[k].nop = i + 1;
            st[k].op[i].index = r_u64(&r);
            for (int c = 0; c < 4; c++) st[k].op[i].cols[c] = r_field(&r);
            r_path(&r, &st[k].op[i].path);
            r_path(&r, &st[k].op[i].spath);
        }
    }
    if (!r.err) fri_read(&r, &d);
    if (r.err || r.pos != r.n) { rc = ZO_MALFORMED_INPUT; goto out; }
    if (nsteps == 0) { rc = ZO_EMPTY_INPUT; goto out; }
    size_t s = p->seg_steps, m = s * p->blowup, offset = m / s;
    if (d.lde_len != m || d.poly_len != m || d.degree_bound != s - 1) { rc = ZO_FRI_VERIFICATION_FAILED; goto out; }
    fold_absorb_params(p, t);
    /* check_chain (fold.rs:710-727) */
    if (st[0].claims.in_a != p->in_a || st[0].claims.in_b != p->in_b) { rc = ZO_FRI_VERIFICATION_FAILED; goto out; }
    for (size_t k = 0; k + 1 < nsteps; k++)
        if (st[k].claims.out_a != st[k + 1].claims.in_a || st[k].claims.out_b != st[k + 1].claims.in_b)
            { rc = ZO_FRI_VERIFICATION_FAILED; goto out; }
    if (st[nsteps - 1].claims.out_b != p->out_b) { rc = ZO_FRI_VERIFICATION_FAILED; goto out; }
    uint32_t omega_s, omega_m;
    primitive_root(s, &omega_s);
    primitive_root(m, &omega_m);
    uint32_t w_last = f_pow(omega_s, s - 1);
    ext4 (*alpha)[6] = malloc(nsteps * sizeof(ext4[6]));
    for (size_t k = 0; k < nsteps && !rc; k++) {
        fold_absorb_step(&st[k].claims, t);
        absorb_s(t, "fold/trace", (const uint8_t *)st[k].cap, 32 * st[k].ncap);
        for (int j = 0; j < 6; j++) alpha[k][j] = challenge_ext(t, "fold/alpha");
        if (st[k].nop != p->num_queries) rc = ZO_FRI_VERIFICATION_FAILED;
    }
    ext4 *gamma = malloc(nsteps * sizeof(ext4));
    for (size_t k = 0; k < nsteps && !rc; k++) gamma[k] = challenge_ext(t, "fold/gamma");
    fri_params fp;
    uint64_t *idx = NULL;
    if (!rc) rc = fold_fri_params(p, &fp);
    if (!rc) {
        idx = malloc((d.nq ? d.nq : 1) * sizeof(uint64_t));
        rc = fri_verify(&d, &fp, t, idx);
    }
    size_t drop, depth;
    capped_shape(m, p->cap_height, &drop, &depth);
    uint32_t log_m = log2u(m);
    for (size_t qi = 0; !rc && qi < d.nq; qi++) {
        size_t index = bit_reverse_index(idx[qi], log_m);
        uint32_t x = f_mul(LDE_SHIFT, f_pow(omega_m, index));
        ext4 combined = {{0, 0, 0, 0}};
        for (size_t k = 0; k < nsteps && !rc; k++) {
            fold_open_t *o = &st[k].op[qi];
            if (o->index != index) { rc = ZO_FRI_VERIFICATION_FAILED; break; }
            /* check_step_openings (fold.rs:669-708) */
            if (st[k].ncap != ((size_t)1 << drop) || o->path.n != depth - drop ||
                o->spath.n != depth - drop) { rc = ZO_BAD_MERKLE_PATH; break; }
            uint8_t row[8];
            put_u32(row, o->cols[0]); put_u32(row + 4, o->cols[1]);
            size_t e = index >> (depth - drop);
            if (e >= st[k].ncap || !verify_capped(st[k].cap[e], row, 8, index, depth, &o->path))
                { rc = ZO_BAD_MERKLE_PATH; break; }
            size_t sh = (index + offset) % m;
            put_u32(row, o->cols[2]); put_u32(row + 4, o->cols[3]);
            e = sh >> (depth - drop);
            if (e >= st[k].ncap || !verify_capped(st[k].cap[e], row, 8, sh, depth, &o->spath))
                { rc = ZO_BAD_MERKLE_PATH; break; }
            combined = e_add(combined, e_mul(gamma[k],
                fold_composition_at(o->cols[0], o->cols[1], o->cols[2], o->cols[3], x, w_last,
                                    &st[k].claims, s, alpha[k])));
        }
        if (rc) break;
        if (d.q[qi].n == 0) { rc = ZO_FRI_VERIFICATION_FAILED; break; }
        if (!e_eq(d.q[qi].f[0].v[idx[qi] % 4], combined)) rc = ZO_FRI_VERIFICATION_FAILED;
    }
    free(idx); free(alpha); free(gamma);
out:
    for (size_t k = 0; k < got; k++) {
        free(st[k].cap);
        for (size_t i = 0; i < st[k].nop; i++) { free(st[k].op[i].path.s); free(st[k].op[i].spath.s); }
        free(st[k].op);
    }
    free(st);
    fri_decoded_free(&d);
    return rc;
}

/* ------------------------------------------------------------------------ */
/* table.rs — membership of a committed value in a public table              */
/* ------------------------------------------------------------------------ */

/* table.rs:55-88 Params::new */
int zo_table_params_new(uint64_t n_rows, uint64_t blowup, uint64_t q, uint64_t final_size,
                        uint32_t value, zo_table_params *o) {
    if (n_rows < 2 || !is_pow2(n_rows)) return ZO_INVALID_DOMAIN_SIZE;
    if (blowup < 2 || !is_pow2(blowup)) return ZO_INVALID_BLOWUP;
    if (q == 0) return ZO_NO_QUERIES;
    if (final_size < 2 || !is_pow2(final_size)) return ZO_INVALID_DOMAIN_SIZE;
    if (n_rows > UINT64_MAX / blowup || n_rows * blowup > MAX_DOMAIN) return ZO_INVALID_DOMAIN_SIZE;
    o->n_rows = n_rows; o->blowup = blowup; o->num_queries = q; o->final_size = final_size;
    o->grinding_bits = 0; o->cap_height = 0; o->value = value % P;
    return ZO_OK;
}

/* table.rs:114-170 Params::for_security */
int zo_table_for_security(uint64_t n_rows, uint64_t table_len, uint32_t value, uint32_t target,
                          zo_table_params *o) {
    if (n_rows < 2 || !is_pow2(n_rows)) return ZO_INVALID_DOMAIN_SIZE;
    if (table_len < 2) return ZO_MALFORMED_INPUT;
    if (n_rows - 1 > UINT64_MAX / table_len || table_len * (n_rows - 1) < n_rows) return ZO_MALFORMED_INPUT;
    uint64_t bound = table_len * (n_rows - 1) - n_rows;
    uint64_t need = bound + 1, blowup = 4, lde;
    for (;;) {
        if (n_rows > UINT64_MAX / blowup) return ZO_INVALID_DOMAIN_SIZE;
        lde = n_rows * blowup;
        if (need <= lde / 4 || blowup >= ((uint64_t)1 << 27)) break;
        blowup *= 2;
    }
    if (lde > MAX_DOMAIN || need > lde / 4) return ZO_INVALID_DOMAIN_SIZE;
    uint32_t mb = zo_fri_composition_millibits(lde, bound);
    size_t q; uint32_t g;
    zo_fri_tune_strength(target, mb, &q, &g);
    size_t fs, ch;
    zo_fri_tune_shape(lde, q, lde, 12, 1, &fs, &ch);
    o->n_rows = n_rows; o->blowup = blowup; o->num_queries = q; o->final_size = fs;
    o->grinding_bits = g; o->cap_height = ch; o->value = value % P;
    return ZO_OK;
}

/* table.rs:220-250 validate */
static int table_validate(const zo_table_params *p) {
    if (p->n_rows < 2 || !is_pow2(p->n_rows)) return ZO_INVALID_DOMAIN_SIZE;
    if (p->blowup < 2 || !is_pow2(p->blowup)) return ZO_INVALID_BLOWUP;
    if (p->num_queries == 0) return ZO_NO_QUERIES;
    if (p->final_size < 2 || !is_pow2(p->final_size)) return ZO_INVALID_DOMAIN_SIZE;
    if (p->cap_height > 8) return ZO_MALFORMED_INPUT;
    if (p->n_rows > UINT64_MAX / p->blowup || p->n_rows * p->blowup > MAX_DOMAIN) return ZO_INVALID_DOMAIN_SIZE;
    return ZO_OK;
}

/* table.rs:364-374 membership_bound (saturating) */
static uint64_t membership_bound(uint64_t tlen, uint64_t n, uint64_t n_rand) {
    uint64_t a = n + n_rand < n ? UINT64_MAX : n + n_rand;
    a = a ? a - 1 : 0;
    uint64_t prod = (a && tlen > UINT64_MAX / a) ? UINT64_MAX : tlen * a;
    return prod > n ? prod - n : 0;
}

/* table.rs:540-554 absorb_params */
static void table_absorb_params(const zo_table_params *p, const uint32_t *table, size_t tlen,
                                zo_transcript *t) {
    size_t len = 56 + 4 * tlen;
    uint8_t *b = malloc(len);
    put_u64(b, p->n_rows); put_u64(b + 8, p->blowup); put_u64(b + 16, p->num_queries);
    put_u64(b + 24, p->final_size); put_u32(b + 32, p->grinding_bits); put_u64(b + 36, p->cap_height);
    put_u32(b + 44, p->value); put_u64(b + 48, tlen);
    for (size_t i = 0; i < tlen; i++) put_u32(b + 56 + 4 * i, table[i]);
    absorb_s(t, "table/params", b, len);
    free(b);
}

/* table.rs:646-660 composition_at */
static ext4 table_composition_at(uint32_t v, uint32_t x, const uint32_t *table, size_t tlen,
                                 uint32_t value, size_t n, ext4 am, ext4 ab) {
    uint32_t z_inv = f_inv(f_sub(f_pow(x, n), 1));
    uint32_t prod = 1;
    for (size_t i = 0; i < tlen; i++) prod = f_mul(prod, f_sub(v, table[i]));
    return e_add(e_mul_base(am, f_mul(prod, z_inv)),
                 e_mul_base(ab, f_mul(f_sub(v, value), f_inv(f_sub(x, 1)))));
}

/* table.rs:376-424 prove_from_coeffs; bytes per table.rs:244-262 */
static int table_prove_coeffs(const zo_table_params *p, const uint32_t *table, size_t tlen,
                              const uint32_t *coeffs, size_t len, uint64_t degree_bound,
                              zo_transcript *t, uint8_t **proof, size_t *proof_len) {
    size_t n = p->n_rows, m = len * p->blowup;
    if (len > SIZE_MAX / p->blowup || m > MAX_DOMAIN) return ZO_INVALID_DOMAIN_SIZE;
    table_absorb_params(p, table, tlen, t);
    uint32_t *lde = malloc(m * 4);
    zo_evaluate_on_coset(coeffs, len, p->blowup, LDE_SHIFT, lde);
    uint8_t *flat = malloc(m * 4);
    for (size_t i = 0; i < m; i++) put_u32(flat + 4 * i, lde[i]);
    mtree tree;
    mtree_from_flat(flat, m * 4, 4, &tree);
    free(flat);
    size_t drop, depth;
    capped_shape(m, p->cap_height, &drop, &depth);
    size_t ncap;
    const digest *cap = mtree_cap(&tree, drop, &ncap);
    absorb_s(t, "table/column", (const uint8_t *)cap, 32 * ncap);
    ext4 am = challenge_ext(t, "table/alpha"), ab = challenge_ext(t, "table/alpha");
    uint32_t omega;
    primitive_root(m, &omega);
    ext4 *comp = malloc(m * sizeof(ext4));
    uint32_t *dz = malloc(m * 4), *db = malloc(m * 4);
    uint32_t x = LDE_SHIFT;
    for (size_t i = 0; i < m; i++) {
        dz[i] = f_sub(f_pow(x, n), 1);
        db[i] = f_sub(x, 1);
        x = f_mul(x, omega);
    }
    zo_batch_invert(dz, m);
    zo_batch_invert(db, m);
    for (size_t i = 0; i < m; i++) {
        uint32_t prod = 1;
        for (size_t k = 0; k < tlen; k++) prod = f_mul(prod, f_sub(lde[i], table[k]));
        comp[i] = e_add(e_mul_base(am, f_mul(prod, dz[i])),
                        e_mul_base(ab, f_mul(f_sub(lde[i], p->value), db[i])));
    }
    free(dz); free(db);
    fri_params fp;
    int rc = fri_params_new(p->blowup, p->num_queries, p->final_size, &fp);
    if (!rc) { fp.grinding_bits = p->grinding_bits; fp.cap_height = p->cap_height; rc = fri_params_validate(&fp); }
    if (!rc && degree_bound >= m) rc = ZO_MALFORMED_INPUT;
    if (rc) { free(comp); free(lde); mtree_free(&tree); return rc; }
    fri_state st;
    rc = fri_commit_inner(comp, m, degree_bound, m, &fp, t, &st);
    if (rc) { free(lde); mtree_free(&tree); return rc; }
    writer w = {0};
    w_byte(&w, VERSION);
    w_cap(&w, cap, ncap);
    fri_write_commitment(&w, &st);
    uint64_t *idx = malloc(p->num_queries * sizeof(uint64_t));
    rc = fri_open_write(&st, t, &w, idx);
    if (!rc) {
        w_u32(&w, (uint32_t)p->num_queries);
        uint32_t log_m = log2u(m);
        for (size_t k = 0; k < p->num_queries && !rc; k++) {
            size_t index = brev(idx[k], log_m);
            path_t pa;
            rc = mtree_prove_capped(&tree, index, drop, &pa);
            if (rc) break;
            w_u64(&w, index);
            w_u32(&w, lde[index]);
            w_path(&w, &pa);
            free(pa.s);
        }
    }
    free(idx); free(lde);
    fri_state_free(&st);
    mtree_free(&tree);
    if (rc) { free(w.b); return rc; }
    *proof = w.b; *proof_len = w.n;
    return ZO_OK;
}

/* table.rs:305-317 prove */
int zo_table_prove(const zo_table_params *p, const uint32_t *table, size_t tlen, zo_transcript *t,
                   uint8_t **proof, size_t *proof_len) {
    int rc = table_validate(p);
    if (rc) return rc;
    if (tlen < 2) return ZO_MALFORMED_INPUT;  /* table.rs:291-298 */
    size_t n = p->n_rows;
    uint32_t *c = calloc(n, 4);
    for (size_t i = 0; i < n; i++) c[i] = p->value;
    zo_ntt_inverse(c, n);
    rc = table_prove_coeffs(p, table, tlen, c, n, membership_bound(tlen, n, 0), t, proof, proof_len);
    free(c);
    return rc;
}

/* table.rs:329-356 prove_zk */
int zo_table_prove_zk(const zo_table_params *p, const uint32_t *table, size_t tlen, size_t n_rand,
                      zo_chacha20 *rng, zo_transcript *t, uint8_t **proof, size_t *proof_len) {
    int rc = table_validate(p);
    if (rc) return rc;
    if (tlen < 2) return ZO_MALFORMED_INPUT;
    if (n_rand < p->num_queries) return ZO_MALFORMED_INPUT;
    size_t n = p->n_rows;
    uint32_t *c = calloc(n, 4);
    for (size_t i = 0; i < n; i++) c[i] = p->value;
    zo_ntt_inverse(c, n);
    size_t total = n + n_rand, padded = 1;
    while (padded < total) padded <<= 1;
    if (padded > MAX_DOMAIN) { free(c); return ZO_INVALID_DOMAIN_SIZE; }
    size_t pl;
    uint32_t *masked = mask_coeffs(c, n, n_rand, rng, &pl);
    free(c);
    rc = table_prove_coeffs(p, table, tlen, masked, pl, membership_bound(tlen, n, n_rand), t, proof,
                            proof_len);
    free(masked);
    return rc;
}

/* table.rs:430-538 verify (decoding per table.rs:265-289) */
int zo_table_verify(const zo_table_params *p, const uint32_t *table, size_t tlen,
                    const uint8_t *proof, size_t proof_len, zo_transcript *t) {
    int rc = table_validate(p);
    if (rc) return rc;
    if (tlen < 2) return ZO_MALFORMED_INPUT;
    reader r = {proof, proof_len, 0, 0};
    if (r_byte(&r) != VERSION) return ZO_MALFORMED_INPUT;
    size_t ncap;
    digest *cap = r_cap(&r, &ncap);
    fri_decoded d;
    memset(&d, 0, sizeof d);
    if (!r.err) fri_read(&r, &d);
    size_t no = r.err ? 0 : r_count(&r, MAX_QUERIES);
    typedef struct { size_t index; uint32_t v; path_t path; } top_t;
    top_t *op = NULL;
    size_t got = 0;
    if (!r.err && no * 12 <= r.n - r.pos) {
        op = calloc(no ? no : 1, sizeof(top_t));
        for (size_t k = 0; k < no && !r.err; k++) {
            got = k + 1;
            op[k].index = r_u64(&r);
            op[k].v = r_field(&r);
            r_path(&r, &op[k].path);
        }
    } else r.err = 1;
    if (r.err || r.pos != r.n) { rc = ZO_MALFORMED_INPUT; goto out; }
    size_t n = p->n_rows, m = d.lde_len, expected = n * p->blowup;
    if (m < expected || m % expected) { rc = ZO_FRI_VERIFICATION_FAILED; goto out; }
    if (m == expected) {
        if (d.degree_bound != membership_bound(tlen, n, 0)) { rc = ZO_FRI_VERIFICATION_FAILED; goto out; }
    } else {
        size_t padded = m / p->blowup;
        if (padded - 1 > UINT64_MAX / tlen || tlen * (padded - 1) < n) { rc = ZO_FRI_VERIFICATION_FAILED; goto out; }
        if (d.degree_bound > tlen * (padded - 1) - n) { rc = ZO_FRI_VERIFICATION_FAILED; goto out; }
    }
    if (d.poly_len != m) { rc = ZO_FRI_VERIFICATION_FAILED; goto out; }
    table_absorb_params(p, table, tlen, t);
    if (no != p->num_queries) { rc = ZO_FRI_VERIFICATION_FAILED; goto out; }
    absorb_s(t, "table/column", (const uint8_t *)cap, 32 * ncap);
    ext4 am = challenge_ext(t, "table/alpha"), ab = challenge_ext(t, "table/alpha");
    fri_params fp;
    rc = fri_params_new(p->blowup, p->num_queries, p->final_size, &fp);
    if (rc) goto out;
    fp.grinding_bits = p->grinding_bits; fp.cap_height = p->cap_height;
    uint64_t *idx = malloc((d.nq ? d.nq : 1) * sizeof(uint64_t));
    rc = fri_verify(&d, &fp, t, idx);
    uint32_t log_m = log2u(m), omega;
    primitive_root(m, &omega);
    size_t drop, depth;
    capped_shape(m, p->cap_height, &drop, &depth);
    for (size_t k = 0; !rc && k < d.nq; k++) {
        size_t index = brev(idx[k], log_m);
        if (op[k].index != index) { rc = ZO_FRI_VERIFICATION_FAILED; break; }
        if (ncap != ((size_t)1 << drop) || op[k].path.n != depth - drop) { rc = ZO_BAD_MERKLE_PATH; break; }
        uint8_t vb[4];
        put_u32(vb, op[k].v);
        size_t e = index >> (depth - drop);
        if (e >= ncap || !verify_capped(cap[e], vb, 4, index, depth, &op[k].path)) { rc = ZO_BAD_MERKLE_PATH; break; }
        uint32_t x = f_mul(LDE_SHIFT, f_pow(omega, index));
        ext4 want = table_composition_at(op[k].v, x, table, tlen, p->value, n, am, ab);
        if (d.q[k].n == 0) { rc = ZO_FRI_VERIFICATION_FAILED; break; }
        if (!e_eq(d.q[k].f[0].v[idx[k] % 4], want)) rc = ZO_FRI_VERIFICATION_FAILED;
    }
    free(idx);
out:
    for (size_t k = 0; k < got; k++) free(op[k].path.s);
    free(op);
    free(cap);
    fri_decoded_free(&d);
    return rc;
}

/* ------------------------------------------------------------------------ */
/* range.rs — range-check AIR                                                */
/* ------------------------------------------------------------------------ */

/* range.rs:57-99 */
int zo_range_params_new(uint64_t n_rows, uint64_t n_bits, uint64_t blowup, uint64_t q,
                        uint64_t final_size, uint32_t value, zo_range_params *o) {
    if (n_rows < 2 || !is_pow2(n_rows)) return ZO_INVALID_DOMAIN_SIZE;
    if (n_bits == 0 || n_bits > 24) return ZO_MALFORMED_INPUT;
    if (blowup < 2 || !is_pow2(blowup)) return ZO_INVALID_BLOWUP;
    if (q == 0) return ZO_NO_QUERIES;
    if (final_size < 2 || !is_pow2(final_size)) return ZO_INVALID_DOMAIN_SIZE;
    if (n_rows > UINT64_MAX / blowup || n_rows * blowup > MAX_DOMAIN) return ZO_INVALID_DOMAIN_SIZE;
    o->n_rows = n_rows; o->n_bits = n_bits; o->blowup = blowup; o->num_queries = q;
    o->final_size = final_size; o->grinding_bits = 0; o->cap_height = 0; o->value = value % P;
    return ZO_OK;
}

/* range.rs:124-161 */
int zo_range_for_security(uint64_t n_rows, uint64_t n_bits, uint32_t value, uint32_t target,
                          zo_range_params *o) {
    if (n_rows < 2 || !is_pow2(n_rows)) return ZO_INVALID_DOMAIN_SIZE;
    if (n_bits == 0 || n_bits > 24) return ZO_MALFORMED_INPUT;
    uint64_t blowup = 16;
    if (n_rows > UINT64_MAX / blowup || n_rows * blowup > MAX_DOMAIN) return ZO_INVALID_DOMAIN_SIZE;
    size_t lde = n_rows * blowup;
    uint32_t mb = zo_fri_composition_millibits(lde, n_rows - 1);
    size_t q; uint32_t g;
    zo_fri_tune_strength(target, mb, &q, &g);
    size_t fs, ch;
    zo_fri_tune_shape(lde, q, lde, 8 + 4 * (n_bits + 1), 1, &fs, &ch);
    o->n_rows = n_rows; o->n_bits = n_bits; o->blowup = blowup; o->num_queries = q;
    o->final_size = fs; o->grinding_bits = g; o->cap_height = ch; o->value = value % P;
    return ZO_OK;
}

/* range.rs:185-218 */
static int range_validate(const zo_range_params *p) {
    if (p->n_rows < 2 || !is_pow2(p->n_rows)) return ZO_INVALID_DOMAIN_SIZE;
    if (p->n_bits == 0 || p->n_bits > 24) return ZO_MALFORMED_INPUT;
    if (p->blowup < 2 || !is_pow2(p->blowup)) return ZO_INVALID_BLOWUP;
    if (p->num_queries == 0) return ZO_NO_QUERIES;
    if (p->final_size < 2 || !is_pow2(p->final_size)) return ZO_INVALID_DOMAIN_SIZE;
    if (p->cap_height > 8) return ZO_MALFORMED_INPUT;
    if (p->n_rows > UINT64_MAX / p->blowup || p->n_rows * p->blowup > MAX_DOMAIN)
        return ZO_INVALID_DOMAIN_SIZE;
    return ZO_OK;
}

/* range.rs:634-645 */
static void range_absorb_params(const zo_range_params *p, zo_transcript *t) {
    uint8_t buf[56];
    put_u64(buf, p->n_rows); put_u64(buf + 8, p->n_bits); put_u64(buf + 16, p->blowup);
    put_u64(buf + 24, p->num_queries); put_u64(buf + 32, p->final_size);
    put_u32(buf + 40, p->grinding_bits); put_u64(buf + 44, p->cap_height);
    put_u32(buf + 52, p->value);
    absorb_s(t, "range/params", buf, 56);
}

typedef struct {
    uint32_t **ldes; size_t nbits; const uint32_t *pts; ext4 *out;
    uint32_t p0, ratio, value; ext4 ad, ab; const ext4 *abits;
} rcompose_ctx;
static void rcompose_worker(void *vctx, size_t base, size_t len) {  /* range.rs:712-739 */
    rcompose_ctx *c = vctx;
    uint32_t *dz = malloc(len * 4), *dbn = malloc(len * 4);
    uint32_t cur = f_mul(c->p0, f_pow(c->ratio, base));
    for (size_t j = 0; j < len; j++) {
        dz[j] = f_sub(cur, 1);
        dbn[j] = f_sub(c->pts[base + j], 1);
        cur = f_mul(cur, c->ratio);
    }
    zo_batch_invert(dz, len);
    zo_batch_invert(dbn, len);
    for (size_t j = 0; j < len; j++) {
        size_t i = base + j;
        uint32_t rec = 0, power = 1;
        for (size_t k = 0; k < c->nbits; k++) {
            rec = f_add(rec, f_mul(power, c->ldes[1 + k][i]));
            power = f_add(power, power);
        }
        uint32_t v = c->ldes[0][i];
        ext4 acc = e_mul_base(c->ad, f_mul(f_sub(v, rec), dz[j]));
        for (size_t k = 0; k < c->nbits; k++) {
            uint32_t bit = c->ldes[1 + k][i];
            acc = e_add(acc, e_mul_base(c->abits[k], f_mul(f_mul(bit, f_sub(bit, 1)), dz[j])));
        }
        acc = e_add(acc, e_mul_base(c->ab, f_mul(f_sub(v, c->value), dbn[j])));
        c->out[i] = acc;
    }
    free(dz); free(dbn);
}

/* range.rs:753-774 */
static ext4 range_composition_at(uint32_t v, const uint32_t *bits, size_t nbits, uint32_t x,
                                 uint32_t value, size_t n, ext4 ad, const ext4 *abits, ext4 ab) {
    uint32_t zinv = f_inv(f_sub(f_pow(x, n), 1));
    uint32_t rec = 0, power = 1;
    for (size_t k = 0; k < nbits; k++) { rec = f_add(rec, f_mul(power, bits[k])); power = f_add(power, power); }
    ext4 acc = e_mul_base(ad, f_mul(f_sub(v, rec), zinv));
    for (size_t k = 0; k < nbits; k++)
        acc = e_add(acc, e_mul_base(abits[k], f_mul(f_mul(bits[k], f_sub(bits[k], 1)), zinv)));
    return e_add(acc, e_mul_base(ab, f_mul(f_sub(v, value), f_inv(f_sub(x, 1)))));
}

/* range.rs:337-343 prove -> 353-375 prove_with_columns -> 425-514 prove_from_columns */
static int range_prove_cols(const zo_range_params *params, const uint32_t *cols, zo_transcript *t,
                            uint8_t **proof, size_t *proof_len);

int zo_range_prove(const zo_range_params *params, zo_transcript *t, uint8_t **proof,
                   size_t *proof_len) {
    int rc = range_validate(params);
    if (rc) return rc;
    size_t n = params->n_rows, ncol = params->n_bits + 1;
    uint32_t *cols = malloc(ncol * n * 4);
    for (size_t k = 0; k < ncol; k++) {  /* range.rs:316-330 build_columns */
        uint32_t v = k == 0 ? params->value
                            : ((k - 1) < 32 ? (params->value >> (k - 1)) & 1 : 0);
        for (size_t i = 0; i < n; i++) cols[k * n + i] = v;
    }
    rc = range_prove_cols(params, cols, t, proof, proof_len);
    free(cols);
    return rc;
}

/* range.rs:353-375 prove_with_columns: ncol x n_rows words, column-major,
 * value column first (lengths are the caller's to check). */
int zo_range_prove_with_columns(const zo_range_params *params, const uint32_t *cols,
                                zo_transcript *t, uint8_t **proof, size_t *proof_len) {
    int rc = range_validate(params);
    if (rc) return rc;
    return range_prove_cols(params, cols, t, proof, proof_len);
}

/* range.rs:425-514 prove_from_columns over coefficient columns of length L
 * (power of two; takes ownership of coeffs). */
static int range_prove_coeffs(const zo_range_params *params, uint32_t **coeffs, size_t L,
                              uint64_t degree_bound, zo_transcript *t, uint8_t **proof,
                              size_t *proof_len);

static int range_prove_cols(const zo_range_params *params, const uint32_t *cols, zo_transcript *t,
                            uint8_t **proof, size_t *proof_len) {
    size_t n = params->n_rows, ncol = params->n_bits + 1;
    uint32_t **coeffs = malloc(ncol * sizeof(uint32_t *));
    for (size_t k = 0; k < ncol; k++) {  /* range.rs:370-374 interpolate */
        coeffs[k] = malloc(n * 4);
        memcpy(coeffs[k], cols + k * n, n * 4);
        zo_ntt_inverse(coeffs[k], n);
    }
    return range_prove_coeffs(params, coeffs, n, n - 1, t, proof, proof_len);
}

/* range.rs:393-418 prove_zk: every column masked with n_rand maskers from the
 * stream, column after column (value first). */
int zo_range_prove_zk(const zo_range_params *params, size_t n_rand, zo_chacha20 *rng,
                      zo_transcript *t, uint8_t **proof, size_t *proof_len) {
    int rc = range_validate(params);
    if (rc) return rc;
    if (n_rand < params->num_queries) return ZO_MALFORMED_INPUT;
    size_t n = params->n_rows, ncol = params->n_bits + 1, pl = 0;
    uint32_t **coeffs = malloc(ncol * sizeof(uint32_t *));
    uint32_t *c = malloc(n * 4);
    for (size_t k = 0; k < ncol; k++) {
        uint32_t v = k == 0 ? params->value
                            : ((k - 1) < 32 ? (params->value >> (k - 1)) & 1 : 0);
        for (size_t i = 0; i < n; i++) c[i] = v;
        zo_ntt_inverse(c, n);
        coeffs[k] = mask_coeffs(c, n, n_rand, rng, &pl);
    }
    free(c);
    if (pl > MAX_DOMAIN) {
        for (size_t k = 0; k < ncol; k++) free(coeffs[k]);
        free(coeffs);
        return ZO_INVALID_DOMAIN_SIZE;
    }
    return range_prove_coeffs(params, coeffs, pl, n + 2 * n_rand - 2, t, proof, proof_len);
}

static int range_prove_coeffs(const zo_range_params *params, uint32_t **coeffs, size_t L,
                              uint64_t degree_bound, zo_transcript *t, uint8_t **proof,
                              size_t *proof_len) {
    int rc;
    size_t n = params->n_rows, ncol = params->n_bits + 1;
    if (L > SIZE_MAX / params->blowup || L * params->blowup > MAX_DOMAIN) {
        for (size_t k = 0; k < ncol; k++) free(coeffs[k]);
        free(coeffs);
        return ZO_INVALID_DOMAIN_SIZE;
    }
    size_t m = L * params->blowup;
    uint32_t **ldes = malloc(ncol * sizeof(uint32_t *));
    range_absorb_params(params, t);  /* range.rs:437 */
    for (size_t k = 0; k < ncol; k++) {  /* range.rs:441-448 */
        ldes[k] = malloc(m * 4);
        zo_evaluate_on_coset(coeffs[k], L, params->blowup, LDE_SHIFT, ldes[k]);
        free(coeffs[k]);
    }
    free(coeffs);
    size_t row_len = 4 * ncol;
    uint8_t *flat = malloc(row_len * m);
    for (size_t i = 0; i < m; i++)
        for (size_t k = 0; k < ncol; k++) put_u32(flat + row_len * i + 4 * k, ldes[k][i]);
    mtree tree;
    mtree_from_flat(flat, row_len * m, row_len, &tree);
    size_t drop, depth;
    capped_shape(m, params->cap_height, &drop, &depth);
    size_t ncap;
    const digest *cap = mtree_cap(&tree, drop, &ncap);
    absorb_s(t, "range/column", (const uint8_t *)cap, 32 * ncap);
    ext4 ad = challenge_ext(t, "range/alpha");
    ext4 *abits = malloc(params->n_bits * sizeof(ext4));
    for (size_t k = 0; k < params->n_bits; k++) abits[k] = challenge_ext(t, "range/alpha");
    ext4 ab = challenge_ext(t, "range/alpha");

    uint32_t *pts = lde_points(m);
    rcompose_ctx c;
    c.ldes = ldes; c.nbits = params->n_bits; c.pts = pts; c.value = params->value;
    c.p0 = f_pow(pts[0], n);
    c.ratio = f_pow(f_mul(pts[1], f_inv(pts[0])), n);
    c.ad = ad; c.ab = ab; c.abits = abits;
    c.out = malloc(m * sizeof(ext4));
    for_each_indexed(m, 2048, rcompose_worker, &c);
    free(pts);
    fri_params fp;
    fri_params_new(params->blowup, params->num_queries, params->final_size, &fp);
    fp.grinding_bits = params->grinding_bits; fp.cap_height = params->cap_height;
    fri_state st;
    rc = fri_params_validate(&fp);
    if (!rc && degree_bound >= m) rc = ZO_MALFORMED_INPUT;
    if (!rc) rc = fri_commit_inner(c.out, m, degree_bound, m, &fp, t, &st);
    else free(c.out);
    if (!rc) {
        writer w = {0};
        w_byte(&w, VERSION);
        w_cap(&w, cap, ncap);
        fri_write_commitment(&w, &st);
        uint64_t *idx = malloc(params->num_queries * sizeof(uint64_t));
        rc = fri_open_write(&st, t, &w, idx);
        if (!rc) {
            uint32_t log_m = log2u(m);
            w_u32(&w, (uint32_t)params->num_queries);
            for (size_t k = 0; k < params->num_queries; k++) {
                size_t index = brev(idx[k], log_m);
                w_u64(&w, index);
                w_u32(&w, ldes[0][index]);
                w_u32(&w, (uint32_t)params->n_bits);
                for (size_t b = 1; b < ncol; b++) w_u32(&w, ldes[b][index]);
                path_t p;
                mtree_prove_capped(&tree, index, drop, &p);
                w_path(&w, &p);
                free(p.s);
            }
        }
        free(idx);
        fri_state_free(&st);
        if (rc) free(w.b); else { *proof = w.b; *proof_len = w.n; }
    }
    mtree_free(&tree);
    free(flat); free(abits);
    for (size_t k = 0; k < ncol; k++) free(ldes[k]);
    free(ldes);
    return rc;
}

typedef struct { size_t index; uint32_t v; uint32_t *bits; size_t nb; path_t path; } range_open_t;

/* range.rs:521-632 verify (decodes with range.rs:282-312 from_bytes) */
int zo_range_verify(const zo_range_params *params, const uint8_t *proof, size_t proof_len,
                    zo_transcript *t) {
    int rc = range_validate(params);
    if (rc) return rc;
    reader r = {proof, proof_len, 0, 0};
    if (r_byte(&r) != VERSION) return ZO_MALFORMED_INPUT;
    size_t ncap;
    digest *column_cap = r_cap(&r, &ncap);
    fri_decoded d;
    fri_read(&r, &d);
    size_t nopen = r_count(&r, MAX_QUERIES);
    range_open_t *op = NULL;
    size_t got = 0;
    if (!r.err && nopen * 8 <= r.n - r.pos) {
        op = calloc(nopen ? nopen : 1, sizeof(range_open_t));
        for (size_t k = 0; k < nopen && !r.err; k++) {
            got = k + 1;
            op[k].index = r_u64(&r);
            op[k].v = r_field(&r);
            size_t nb = r_count(&r, MAX_ELEMS);
            if (r.err || nb * 4 > r.n - r.pos) { r.err = 1; break; }
            op[k].bits = malloc((nb ? nb : 1) * 4);
            op[k].nb = nb;
            for (size_t b = 0; b < nb; b++) op[k].bits[b] = r_field(&r);
            r_path(&r, &op[k].path);
        }
    } else r.err = 1;
    if (r.err || r.pos != r.n) { rc = ZO_MALFORMED_INPUT; goto out; }

    size_t n = params->n_rows, m = d.lde_len;
    if (params->blowup > SIZE_MAX / n) { rc = ZO_FRI_VERIFICATION_FAILED; goto out; }
    size_t expected_m = n * params->blowup;
    if (m < expected_m || m % expected_m) { rc = ZO_FRI_VERIFICATION_FAILED; goto out; }
    if (m == expected_m) {
        if (d.degree_bound != n - 1) { rc = ZO_FRI_VERIFICATION_FAILED; goto out; }
    } else {
        size_t padded = m / params->blowup;
        if (2 * padded < n + 2 || d.degree_bound > 2 * padded - (n + 2))
            { rc = ZO_FRI_VERIFICATION_FAILED; goto out; }
    }
    if (d.poly_len != m) { rc = ZO_FRI_VERIFICATION_FAILED; goto out; }
    range_absorb_params(params, t);
    if (nopen != params->num_queries) { rc = ZO_FRI_VERIFICATION_FAILED; goto out; }
    absorb_s(t, "range/column", (const uint8_t *)column_cap, 32 * ncap);
    ext4 ad = challenge_ext(t, "range/alpha");
    ext4 *abits = malloc((params->n_bits ? params->n_bits : 1) * sizeof(ext4));
    for (size_t k = 0; k < params->n_bits; k++) abits[k] = challenge_ext(t, "range/alpha");
    ext4 ab = challenge_ext(t, "range/alpha");
    fri_params fp;
    fri_params_new(params->blowup, params->num_queries, params->final_size, &fp);
    fp.grinding_bits = params->grinding_bits; fp.cap_height = params->cap_height;
    uint64_t *idx = malloc((d.nq ? d.nq : 1) * sizeof(uint64_t));
    rc = fri_verify(&d, &fp, t, idx);
    if (!rc) {
        uint32_t log_m = log2u(m), omega_m = 0;
        primitive_root(m, &omega_m);
        size_t ncol = params->n_bits + 1;
        uint8_t *row = malloc(4 * ncol);
        for (size_t k = 0; k < nopen && !rc; k++) {
            size_t index = brev(idx[k], log_m);
            if (op[k].index != index || op[k].nb != params->n_bits) { rc = ZO_FRI_VERIFICATION_FAILED; break; }
            put_u32(row, op[k].v);
            for (size_t b = 0; b < op[k].nb; b++) put_u32(row + 4 + 4 * b, op[k].bits[b]);
            size_t drop, depth;
            capped_shape(m, params->cap_height, &drop, &depth);
            if (ncap != ((size_t)1 << drop) || op[k].path.n != depth - drop) { rc = ZO_BAD_MERKLE_PATH; break; }
            size_t ei = index >> (depth - drop);
            if (ei >= ncap || !verify_capped(column_cap[ei], row, 4 * ncol, index, depth, &op[k].path))
                { rc = ZO_BAD_MERKLE_PATH; break; }
            uint32_t x = f_mul(LDE_SHIFT, f_pow(omega_m, index));
            ext4 expected = range_composition_at(op[k].v, op[k].bits, op[k].nb, x, params->value,
                                                 n, ad, abits, ab);
            if (d.q[k].n == 0) { rc = ZO_FRI_VERIFICATION_FAILED; break; }
            if (!e_eq(d.q[k].f[0].v[idx[k] % 4], expected)) { rc = ZO_FRI_VERIFICATION_FAILED; break; }
        }
        free(row);
    }
    free(idx); free(abits);
out:
    for (size_t k = 0; k < got; k++) { free(op[k].bits); free(op[k].path.s); }
    free(op);
    free(column_cap);
    fri_decoded_free(&d);
    return rc;
}
