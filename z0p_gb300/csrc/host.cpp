// Host-side protocol logic of the z0p GB300 prover: the parts of the prove
// path that are sequential by nature (Fiat-Shamir transcript, parameter
// validation and tuning, proof shapes). Each function names the reference
// item it reproduces.
#include "host.h"

#include <cstring>

namespace z0p {
namespace host {

static thread_local std::string g_reason;
void set_reason(const std::string& r) { g_reason = r; }
const char* reason() { return g_reason.c_str(); }

uint32_t fpow(uint32_t a, uint64_t e) {  // src/babybear.rs:147-158
  uint32_t acc = 1;
  while (e) {
    if (e & 1) acc = fmul(acc, a);
    a = fmul(a, a);
    e >>= 1;
  }
  return acc;
}

uint32_t two_adic_generator(uint32_t bits) {  // src/babybear.rs:183-193
  return fpow(GENERATOR, (uint64_t)(P - 1) >> bits);
}

uint64_t brev(uint64_t x, uint32_t bits) {
  uint64_t r = 0;
  for (uint32_t i = 0; i < bits; i++) r = (r << 1) | ((x >> i) & 1);
  return r;
}

// ---------------------------------------------------------------- BLAKE3 ----
static const uint32_t IV[8] = {0x6A09E667u, 0xBB67AE85u, 0x3C6EF372u, 0xA54FF53Au,
                               0x510E527Fu, 0x9B05688Cu, 0x1F83D9ABu, 0x5BE0CD19u};
static const uint8_t MSG_PERM[16] = {2, 6, 3, 10, 7, 0, 4, 13, 1, 11, 12, 5, 9, 14, 15, 8};
enum : uint32_t { CHUNK_START = 1, CHUNK_END = 2, PARENT = 4, ROOT = 8 };
constexpr size_t CHUNK_LEN = 1024;

static inline uint32_t rotr(uint32_t x, int n) { return (x >> n) | (x << (32 - n)); }
static inline uint32_t le32(const uint8_t* p) {
  return (uint32_t)p[0] | ((uint32_t)p[1] << 8) | ((uint32_t)p[2] << 16) | ((uint32_t)p[3] << 24);
}
static inline void put32(uint8_t* p, uint32_t v) {
  p[0] = (uint8_t)v; p[1] = (uint8_t)(v >> 8); p[2] = (uint8_t)(v >> 16); p[3] = (uint8_t)(v >> 24);
}
static inline void put64(uint8_t* p, uint64_t v) {
  for (int i = 0; i < 8; i++) p[i] = (uint8_t)(v >> (8 * i));
}

static inline void gmix(uint32_t s[16], int a, int b, int c, int d, uint32_t x, uint32_t y) {
  s[a] += s[b] + x; s[d] = rotr(s[d] ^ s[a], 16);
  s[c] += s[d];     s[b] = rotr(s[b] ^ s[c], 12);
  s[a] += s[b] + y; s[d] = rotr(s[d] ^ s[a], 8);
  s[c] += s[d];     s[b] = rotr(s[b] ^ s[c], 7);
}

// BLAKE3 compression (specification; src/hash.rs:93-133). Returns the
// chaining value (first 8 output words).
static void compress_cv(const uint32_t cv[8], const uint32_t block[16], uint64_t counter,
                        uint32_t len, uint32_t flags, uint32_t out[8]) {
  uint32_t s[16], m[16], t[16];
  std::memcpy(s, cv, 32);
  std::memcpy(s + 8, IV, 16);
  s[12] = (uint32_t)counter; s[13] = (uint32_t)(counter >> 32); s[14] = len; s[15] = flags;
  std::memcpy(m, block, 64);
  for (int r = 0; r < 7; r++) {
    gmix(s, 0, 4, 8, 12, m[0], m[1]);
    gmix(s, 1, 5, 9, 13, m[2], m[3]);
    gmix(s, 2, 6, 10, 14, m[4], m[5]);
    gmix(s, 3, 7, 11, 15, m[6], m[7]);
    gmix(s, 0, 5, 10, 15, m[8], m[9]);
    gmix(s, 1, 6, 11, 12, m[10], m[11]);
    gmix(s, 2, 7, 8, 13, m[12], m[13]);
    gmix(s, 3, 4, 9, 14, m[14], m[15]);
    for (int i = 0; i < 16; i++) t[i] = m[MSG_PERM[i]];
    std::memcpy(m, t, 64);
  }
  for (int i = 0; i < 8; i++) out[i] = s[i] ^ s[i + 8];
}

static void block_words(const uint8_t* p, size_t len, uint32_t w[16]) {
  uint8_t b[64] = {0};
  std::memcpy(b, p, len);
  for (int i = 0; i < 16; i++) w[i] = le32(b + 4 * i);
}

// Output of one chunk of 1..1024 bytes (src/hash.rs:186-225).
static void chunk_output(const uint8_t* data, size_t len, uint64_t counter, bool root,
                         uint8_t out[32]) {
  uint32_t cv[8], w[16];
  std::memcpy(cv, IV, 32);
  size_t blocks = (len + 63) / 64;
  for (size_t i = 0; i < blocks; i++) {
    size_t bl = i + 1 == blocks ? len - 64 * i : 64;
    block_words(data + 64 * i, bl, w);
    uint32_t flags = (i == 0 ? (uint32_t)CHUNK_START : 0u) |
                     (i + 1 == blocks ? ((uint32_t)CHUNK_END | (root ? (uint32_t)ROOT : 0u)) : 0u);
    compress_cv(cv, w, counter, (uint32_t)bl, flags, cv);
  }
  for (int i = 0; i < 8; i++) put32(out + 4 * i, cv[i]);
}

static void parent(const uint8_t l[32], const uint8_t r[32], uint32_t flags, uint8_t out[32]) {
  uint8_t b[64];
  std::memcpy(b, l, 32);
  std::memcpy(b + 32, r, 32);
  uint32_t w[16], cv[8];
  block_words(b, 64, w);
  compress_cv(IV, w, 0, 64, flags, cv);
  for (int i = 0; i < 8; i++) put32(out + 4 * i, cv[i]);
}

// Hasher::push_merged (src/hash.rs:305-318).
static void push_merged(z0p_transcript_state* st, const uint8_t cv[32]) {
  std::memcpy(st->stack[st->stack_len++], cv, 32);
  st->next_index++;
  uint64_t total = st->next_index;
  while (total % 2 == 0) {
    uint8_t merged[32];
    parent(st->stack[st->stack_len - 2], st->stack[st->stack_len - 1], PARENT, merged);
    st->stack_len -= 2;
    std::memcpy(st->stack[st->stack_len++], merged, 32);
    total /= 2;
  }
}

// Hasher::update (src/hash.rs:256-272). The tail never reaches 2048 bytes
// between calls: whenever it does, its first chunk is known not to be the
// last one and is compressed, exactly as the reference's loop does.
void hasher_update(z0p_transcript_state* st, const uint8_t* data, size_t len) {
  st->total_len += len;
  while (len) {
    size_t room = 2 * CHUNK_LEN - st->tail_len;
    size_t take = len < room ? len : room;
    std::memcpy(st->tail + st->tail_len, data, take);
    st->tail_len += (uint32_t)take;
    data += take;
    len -= take;
    if (st->tail_len == 2 * CHUNK_LEN) {
      uint8_t cv[32];
      chunk_output(st->tail, CHUNK_LEN, st->next_index, false, cv);
      push_merged(st, cv);
      std::memmove(st->tail, st->tail + CHUNK_LEN, CHUNK_LEN);
      st->tail_len = CHUNK_LEN;
    }
  }
}

// Hasher::finalize (src/hash.rs:276-302) on a copy of the state.
void hasher_finalize(const z0p_transcript_state* src, uint8_t out[32]) {
  if (src->total_len == 0) {
    uint32_t w[16] = {0}, cv[8];
    compress_cv(IV, w, 0, 0, CHUNK_START | CHUNK_END | ROOT, cv);
    for (int i = 0; i < 8; i++) put32(out + 4 * i, cv[i]);
    return;
  }
  z0p_transcript_state st = *src;
  const uint8_t* tail = st.tail;
  size_t tl = st.tail_len;
  if (tl > CHUNK_LEN) {
    uint8_t cv[32];
    chunk_output(tail, CHUNK_LEN, st.next_index, false, cv);
    push_merged(&st, cv);
    tail += CHUNK_LEN;
    tl -= CHUNK_LEN;
  }
  if (st.stack_len == 0) {
    chunk_output(tail, tl, st.next_index, true, out);
    return;
  }
  uint8_t cur[32];
  chunk_output(tail, tl, st.next_index, false, cur);
  for (uint32_t i = st.stack_len - 1; i >= 1; i--) {
    uint8_t nx[32];
    parent(st.stack[i], cur, PARENT, nx);
    std::memcpy(cur, nx, 32);
  }
  parent(st.stack[0], cur, PARENT | ROOT, out);
}

void blake3(const uint8_t* data, size_t len, uint8_t out[32]) {
  z0p_transcript_state st;
  std::memset(&st, 0, sizeof st);
  hasher_update(&st, data, len);
  hasher_finalize(&st, out);
}

// ------------------------------------------------------------- transcript ----
void transcript_absorb_raw(z0p_transcript_state* st, const uint8_t* label, size_t llen,
                           const uint8_t* data, size_t len) {  // src/transcript.rs:72-77
  uint8_t b[8];
  put64(b, llen);
  hasher_update(st, b, 8);
  hasher_update(st, label, llen);
  put64(b, len);
  hasher_update(st, b, 8);
  hasher_update(st, data, len);
}
void transcript_absorb(z0p_transcript_state* st, const char* label, const uint8_t* data,
                       size_t len) {
  transcript_absorb_raw(st, (const uint8_t*)label, std::strlen(label), data, len);
}
void transcript_init(z0p_transcript_state* st, const uint8_t* label, size_t len) {
  std::memset(st, 0, sizeof *st);  // src/transcript.rs:62-69
  transcript_absorb(st, "domain", label, len);
}
void squeeze_raw(z0p_transcript_state* st, const uint8_t* label, size_t llen, uint8_t out[32]) {
  z0p_transcript_state h = *st;  // src/transcript.rs:162-171
  uint8_t b[8];
  put64(b, llen);
  hasher_update(&h, b, 8);
  hasher_update(&h, label, llen);
  put64(b, st->counter);
  hasher_update(&h, b, 8);
  st->counter++;
  hasher_finalize(&h, out);
  transcript_absorb_raw(st, label, llen, out, 32);
}
void challenge_ext(z0p_transcript_state* st, const char* label, uint32_t out[4]) {
  uint8_t b[32];  // src/transcript.rs:136-141, src/ext4.rs:179-187
  squeeze_raw(st, (const uint8_t*)label, std::strlen(label), b);
  for (int i = 0; i < 4; i++) out[i] = le32(b + 4 * i) % P;
}
uint64_t challenge_index(z0p_transcript_state* st, const char* label, uint64_t domain) {
  uint8_t b[32];  // src/transcript.rs:148-160 (domain checked by the caller)
  squeeze_raw(st, (const uint8_t*)label, std::strlen(label), b);
  uint64_t v = 0;
  for (int i = 0; i < 8; i++) v |= (uint64_t)b[i] << (8 * i);
  return v & (domain - 1);
}
std::vector<uint8_t> pow_head(const z0p_transcript_state* st, const char* label) {
  size_t ll = std::strlen(label);
  std::vector<uint8_t> head(40 + ll);
  hasher_finalize(st, head.data());
  put64(head.data() + 32, ll);
  std::memcpy(head.data() + 40, label, ll);
  return head;
}

// ----------------------------------------------------------------- params ----
int fri_params_new(uint64_t blowup, uint64_t q, uint64_t final_size, FriParams* o) {
  if (blowup < 2 || !is_pow2(blowup)) return Z0P_ERR_INVALID_BLOWUP;  // src/fri.rs:152-171
  if (q == 0) return Z0P_ERR_NO_QUERIES;
  if (final_size < 2 || !is_pow2(final_size) || final_size > 1024) return Z0P_ERR_INVALID_DOMAIN_SIZE;
  *o = FriParams{blowup, q, final_size, 0, 0};
  return Z0P_OK;
}
int fri_params_validate(const FriParams& p) {  // src/fri.rs:163-196
  if (p.blowup < 2 || !is_pow2(p.blowup)) return Z0P_ERR_INVALID_BLOWUP;
  if (p.num_queries == 0) return Z0P_ERR_NO_QUERIES;
  if (p.num_queries > (1u << 20)) { set_reason("num_queries above protocol cap"); return Z0P_ERR_MALFORMED_INPUT; }
  if (p.final_size < 2 || !is_pow2(p.final_size) || p.final_size > 1024) return Z0P_ERR_INVALID_DOMAIN_SIZE;
  if (p.grinding_bits > 32) { set_reason("grinding_bits above 32"); return Z0P_ERR_MALFORMED_INPUT; }
  if (p.cap_height > 8) { set_reason("cap_height above 8"); return Z0P_ERR_MALFORMED_INPUT; }
  return Z0P_OK;
}

static uint64_t sat_add(uint64_t a, uint64_t b) { uint64_t s = a + b; return s < a ? UINT64_MAX : s; }

static std::vector<uint64_t> layer_sizes(uint64_t len, uint64_t final_size) {  // src/fri.rs:945-955
  std::vector<uint64_t> out;
  for (;;) {
    out.push_back(len);
    if (len <= final_size) break;
    len /= 4;
  }
  return out;
}
static uint64_t est_fri(const std::vector<uint64_t>& layers, uint64_t q, uint64_t h) {
  uint64_t total = 24 + 8;  // src/fri.rs:962-979
  for (size_t i = 0; i < layers.size(); i++) {
    uint64_t v = layers[i];
    uint64_t leaves = v % 4 == 0 ? v / 4 : v;
    uint64_t depth = log2u(leaves), drop = h < depth ? h : depth;
    total = sat_add(total, 32ull << (drop < 16 ? drop : 16));
    if (i + 1 < layers.size()) total += q * (64 + 33 * (depth - drop));
  }
  return total;
}
static uint64_t est_col(uint64_t lde, uint64_t q, uint64_t vb, uint64_t h) {  // src/fri.rs:985-998
  uint64_t depth = log2u(lde), drop = h < depth ? h : depth;
  return sat_add(32ull << (drop < 16 ? drop : 16), q * (vb + 33 * (depth - drop)));
}
void tune_shape(uint64_t lde_len, uint64_t q, uint64_t col_lde, uint64_t col_vb,
                uint64_t* final_size, uint64_t* cap_height) {  // src/fri.rs:1009-1043
  uint64_t shifted = lde_len / 4 > 2 ? lde_len / 4 : 2;
  while (shifted > 32) shifted /= 4;
  uint64_t best_f = shifted, best_h = 0, best = UINT64_MAX;
  for (;;) {
    auto layers = layer_sizes(lde_len, shifted);
    for (uint64_t h = 0; h <= 4; h++) {
      uint64_t total = sat_add(est_fri(layers, q, h), est_col(col_lde, q, col_vb, h));
      if (total < best) { best = total; best_f = shifted; best_h = h; }
    }
    if (shifted <= 1) break;
    shifted /= 4;
    if (shifted < 1) break;
  }
  *final_size = best_f;
  *cap_height = best_h;
}
uint32_t composition_millibits(uint64_t lde_len, uint64_t degree_bound) {  // src/fri.rs:1050-1056
  uint64_t den = 1;
  while (den < degree_bound + 1) den <<= 1;
  if (lde_len < den) return 500;
  return 500 * (log2u(lde_len) - log2u(den));
}
void tune_strength(uint32_t target, uint32_t millibits, uint64_t* q, uint32_t* g) {  // src/fri.rs:1064-1074
  uint32_t grind = target / 2 < 20 ? target / 2 : 20;
  uint64_t remaining = (uint64_t)(target > grind ? target - grind : 0) * 1000;
  uint64_t per = millibits ? millibits : 1;
  uint64_t qn = (remaining + per - 1) / per;
  if (qn < 1) qn = 1;
  if (qn > 1000000) qn = 1000000;
  *q = qn;
  *g = grind;
}

int air_validate(const z0p_air_params& p) {  // src/air.rs:181-211
  if (p.n_steps < 2 || !is_pow2(p.n_steps)) return Z0P_ERR_INVALID_DOMAIN_SIZE;
  if (p.blowup < 4 || !is_pow2(p.blowup)) return Z0P_ERR_INVALID_BLOWUP;
  if (p.num_queries == 0) return Z0P_ERR_NO_QUERIES;
  if (p.final_size < 2 || !is_pow2(p.final_size)) return Z0P_ERR_INVALID_DOMAIN_SIZE;
  if (p.cap_height > 8) { set_reason("cap_height above 8"); return Z0P_ERR_MALFORMED_INPUT; }
  if (p.n_steps > UINT64_MAX / p.blowup || p.n_steps * p.blowup > MAX_DOMAIN)
    return Z0P_ERR_INVALID_DOMAIN_SIZE;
  if (p.a0 >= P || p.b0 >= P || p.b_last >= P) {
    set_reason("field elements must be canonical (< p)");
    return Z0P_ERR_MALFORMED_INPUT;
  }
  return Z0P_OK;
}

int range_validate(const z0p_range_params& p) {  // src/range.rs:185-218
  if (p.n_rows < 2 || !is_pow2(p.n_rows)) return Z0P_ERR_INVALID_DOMAIN_SIZE;
  if (p.n_bits == 0 || p.n_bits > 24) { set_reason("n_bits must be within 1..=24"); return Z0P_ERR_MALFORMED_INPUT; }
  if (p.blowup < 2 || !is_pow2(p.blowup)) return Z0P_ERR_INVALID_BLOWUP;
  if (p.num_queries == 0) return Z0P_ERR_NO_QUERIES;
  if (p.final_size < 2 || !is_pow2(p.final_size)) return Z0P_ERR_INVALID_DOMAIN_SIZE;
  if (p.cap_height > 8) { set_reason("cap_height above 8"); return Z0P_ERR_MALFORMED_INPUT; }
  if (p.n_rows > UINT64_MAX / p.blowup || p.n_rows * p.blowup > MAX_DOMAIN)
    return Z0P_ERR_INVALID_DOMAIN_SIZE;
  if (p.value >= P) { set_reason("field elements must be canonical (< p)"); return Z0P_ERR_MALFORMED_INPUT; }
  return Z0P_OK;
}

int fri_shape(uint64_t m, uint64_t degree_bound, const FriParams& fp, FriShape* out) {
  int rc = fri_params_validate(fp);  // src/fri.rs:551-575
  if (rc) return rc;
  if (fp.final_size >= m || m % fp.final_size) return Z0P_ERR_INVALID_DOMAIN_SIZE;  // :1130-1140
  uint64_t ratio = m / fp.final_size;
  if (!is_pow2(ratio) || log2u(ratio) % 2) return Z0P_ERR_INVALID_DOMAIN_SIZE;
  if (m < 2 || degree_bound + 1 > m / 2) { set_reason("degree bound implies rate >= 1/2"); return Z0P_ERR_MALFORMED_INPUT; }
  uint32_t folds = log2u(ratio) / 2;
  uint64_t residual = degree_bound >> (2 * folds);
  if (residual + 1 >= fp.final_size) {
    set_reason("final layer too small for a non-vacuous degree check");
    return Z0P_ERR_MALFORMED_INPUT;
  }
  out->m = m;
  out->len = layer_sizes(m, fp.final_size);
  out->leaves.clear(); out->depth.clear(); out->drop.clear();
  for (uint64_t len : out->len) {
    uint64_t leaves = len % 4 == 0 ? len / 4 : len;
    uint32_t d = log2u(leaves);
    out->leaves.push_back(leaves);
    out->depth.push_back(d);
    out->drop.push_back(fp.cap_height < d ? (uint32_t)fp.cap_height : d);  // src/fri.rs:935-939
  }
  return Z0P_OK;
}

uint64_t fri_bytes(const FriShape& s, uint64_t q) {
  // Commitment body (src/fri.rs:896-904) + proof body (src/fri.rs:352-368).
  uint64_t total = 24 + 4;
  for (size_t i = 0; i < s.len.size(); i++) total += 4 + 32ull * (1ull << s.drop[i]);
  total += 4 + 16 * s.len.back() + 8 + 4;
  uint64_t per_query = 4;
  for (size_t d = 0; d + 1 < s.len.size(); d++) per_query += 64 + 4 + 33ull * (s.depth[d] - s.drop[d]);
  return total + q * per_query;
}

}  // namespace host
}  // namespace z0p
