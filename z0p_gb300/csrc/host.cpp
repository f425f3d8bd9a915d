// Host-side protocol logic of the z0p GB300 prover: the parts of the prove
// path that are sequential by nature (Fiat-Shamir transcript, parameter
// validation and tuning, proof shapes). Each function names the reference
// item it reproduces.
#include "host.h"

#include <cstring>

namespace z0p {
namespace host {

// The message of the last failure on this thread. Reading it consumes it, so
// a later failure that sets no message of its own reports none rather than
// an older one.
static thread_local std::string g_reason, g_read;
void set_reason(const std::string& r) { g_reason = r; }
const char* reason() {
  g_read.swap(g_reason);
  g_reason.clear();
  return g_read.c_str();
}

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

#define Z0P_HG(a, b, c, d, x, y)  \
  do {                            \
    a = a + b + (x);              \
    d = rotr(d ^ a, 16);          \
    c = c + d;                    \
    b = rotr(b ^ c, 12);          \
    a = a + b + (y);              \
    d = rotr(d ^ a, 8);           \
    c = c + d;                    \
    b = rotr(b ^ c, 7);           \
  } while (0)

// The message words each round reads (specification: the permutation applied
// after every round), as compile-time indices, so the message stays in
// registers instead of being permuted through memory seven times.
struct MsgSchedule {
  uint8_t at[7][16];
};
static constexpr MsgSchedule make_schedule() {
  constexpr uint8_t perm[16] = {2, 6, 3, 10, 7, 0, 4, 13, 1, 11, 12, 5, 9, 14, 15, 8};
  MsgSchedule r{};
  for (int i = 0; i < 16; i++) r.at[0][i] = (uint8_t)i;
  for (int k = 1; k < 7; k++)
    for (int i = 0; i < 16; i++) r.at[k][i] = r.at[k - 1][perm[i]];
  return r;
}
static constexpr MsgSchedule SCHEDULE = make_schedule();

template <int R>
static inline void blake3_round(uint32_t (&v)[16], const uint32_t (&m)[16]) {
  constexpr const uint8_t* S = SCHEDULE.at[R];
  Z0P_HG(v[0], v[4], v[8], v[12], m[S[0]], m[S[1]]);
  Z0P_HG(v[1], v[5], v[9], v[13], m[S[2]], m[S[3]]);
  Z0P_HG(v[2], v[6], v[10], v[14], m[S[4]], m[S[5]]);
  Z0P_HG(v[3], v[7], v[11], v[15], m[S[6]], m[S[7]]);
  Z0P_HG(v[0], v[5], v[10], v[15], m[S[8]], m[S[9]]);
  Z0P_HG(v[1], v[6], v[11], v[12], m[S[10]], m[S[11]]);
  Z0P_HG(v[2], v[7], v[8], v[13], m[S[12]], m[S[13]]);
  Z0P_HG(v[3], v[4], v[9], v[14], m[S[14]], m[S[15]]);
}

// BLAKE3 compression (specification; src/hash.rs:93-133). Returns the
// chaining value (first 8 output words); out may alias cv.
static void compress_cv(const uint32_t cv[8], const uint32_t block[16], uint64_t counter,
                        uint32_t len, uint32_t flags, uint32_t out[8]) {
  uint32_t m[16];
  std::memcpy(m, block, 64);
  uint32_t v[16] = {cv[0], cv[1], cv[2], cv[3], cv[4], cv[5], cv[6], cv[7],
                    IV[0], IV[1], IV[2], IV[3], (uint32_t)counter, (uint32_t)(counter >> 32), len,
                    flags};
  blake3_round<0>(v, m);
  blake3_round<1>(v, m);
  blake3_round<2>(v, m);
  blake3_round<3>(v, m);
  blake3_round<4>(v, m);
  blake3_round<5>(v, m);
  blake3_round<6>(v, m);
  for (int i = 0; i < 8; i++) out[i] = v[i] ^ v[8 + i];
}
#undef Z0P_HG

static void block_words(const uint8_t* p, size_t len, uint32_t w[16]) {
#if defined(__BYTE_ORDER__) && __BYTE_ORDER__ == __ORDER_LITTLE_ENDIAN__
  if (len == 64) {  // a full block is its words' bytes in order
    std::memcpy(w, p, 64);
    return;
  }
#endif
  uint8_t b[64] = {0};
  std::memcpy(b, p, len);
  for (int i = 0; i < 16; i++) w[i] = le32(b + 4 * i);
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

// Block i of a chunk whose first `len` bytes are at p, zero-padded.
static void chunk_block(const uint8_t* p, size_t len, uint32_t i, uint32_t w[16]) {
  size_t off = 64 * (size_t)i;
  block_words(p + off, len - off < 64 ? len - off : 64, w);
}

// The block cache of the last transcript this thread finished with. A prove
// call works on a copy of the caller's state and hands it back, so the next
// call usually starts from the same tail: its chunks' cached chaining values
// are taken over instead of re-hashing up to 2 KiB. Chunk h's entry is used
// only for a state with the same chunk count whose tail repeats the cached
// blocks byte for byte, with a byte after them inside the chunk (so none of
// them is the chunk's last); its chaining value depends on nothing else.
namespace {
struct CacheMemo {
  bool valid = false;
  uint64_t next_index = 0;
  uint32_t cv[2][8];
  uint32_t nblk[2];
  uint8_t blocks[2 * CHUNK_LEN];  // the cached blocks' bytes, at their tail offsets
};
thread_local CacheMemo g_memo;
}  // namespace

Hasher::Hasher(z0p_transcript_state* s) : st(s) {
  const CacheMemo& m = g_memo;
  const bool same_chunks = m.valid && m.next_index == st->next_index && st->tail_len < 2 * CHUNK_LEN;
  for (int h = 0; h < 2; h++) {
    std::memcpy(cv[h], IV, 32);
    nblk[h] = 0;
    if (!same_chunks || m.nblk[h] == 0) continue;
    const size_t base = CHUNK_LEN * h, covered = 64 * (size_t)m.nblk[h];
    if (st->tail_len > base + covered && covered < CHUNK_LEN &&
        std::memcmp(st->tail + base, m.blocks + base, covered) == 0) {
      std::memcpy(cv[h], m.cv[h], 32);
      nblk[h] = m.nblk[h];
    }
  }
  advance();
}

void Hasher::remember() const {
  CacheMemo& m = g_memo;
  m.valid = true;
  m.next_index = st->next_index;
  for (int h = 0; h < 2; h++) {
    std::memcpy(m.cv[h], cv[h], 32);
    m.nblk[h] = nblk[h];
    std::memcpy(m.blocks + CHUNK_LEN * h, st->tail + CHUNK_LEN * h, 64 * (size_t)nblk[h]);
  }
}

// Folds into cv[h] every block of tail chunk h that has at least one byte
// after it inside the chunk: such a block is never its chunk's last block, so
// its compression (flags CHUNK_START or none, counter = chunk index) is final.
void Hasher::advance() {
  for (uint32_t h = 0; h < 2; h++) {
    size_t base = CHUNK_LEN * h;
    if (st->tail_len <= base) break;
    size_t len = st->tail_len - base < CHUNK_LEN ? st->tail_len - base : CHUNK_LEN;
    while (64 * ((size_t)nblk[h] + 1) < len) {
      uint32_t w[16];
      chunk_block(st->tail + base, len, nblk[h], w);
      compress_cv(cv[h], w, st->next_index + h, 64, nblk[h] == 0 ? (uint32_t)CHUNK_START : 0u,
                  cv[h]);
      nblk[h]++;
    }
  }
}

// Hasher::update (src/hash.rs:256-272). The tail never reaches 2048 bytes
// between calls: whenever it does, its first chunk is known not to be the
// last one and is compressed, exactly as the reference's loop does.
void Hasher::update(const uint8_t* data, size_t len) {
  st->total_len += len;
  while (len) {
    size_t room = 2 * CHUNK_LEN - st->tail_len;
    size_t take = len < room ? len : room;
    std::memcpy(st->tail + st->tail_len, data, take);
    st->tail_len += (uint32_t)take;
    data += take;
    len -= take;
    advance();
    if (st->tail_len == 2 * CHUNK_LEN) {
      // Blocks 0..14 of the first chunk are folded; its last block ends it.
      uint32_t w[16], out[8];
      chunk_block(st->tail, CHUNK_LEN, 15, w);
      compress_cv(cv[0], w, st->next_index, 64, CHUNK_END, out);
      uint8_t cvb[32];
      for (int i = 0; i < 8; i++) put32(cvb + 4 * i, out[i]);
      push_merged(st, cvb);
      std::memmove(st->tail, st->tail + CHUNK_LEN, CHUNK_LEN);
      st->tail_len = CHUNK_LEN;
      std::memcpy(cv[0], cv[1], 32);
      nblk[0] = nblk[1];
      std::memcpy(cv[1], IV, 32);
      nblk[1] = 0;
    }
  }
}

// The first of two tail chunks ends with block 15 (flags CHUNK_END, counter
// next_index); push_merged of its output on a virtual copy of the stack
// leaves stack[0..top_sl) and top_cv. Kept for this next_index.
void Hasher::first_chunk_top() const {
  if (top_ok && top_index == st->next_index) return;
  uint32_t w[16], o[8];
  chunk_block(st->tail, CHUNK_LEN, 15, w);
  compress_cv(cv[0], w, st->next_index, 64, CHUNK_END, o);
  for (int i = 0; i < 8; i++) put32(top_cv + 4 * i, o[i]);
  uint32_t sl = st->stack_len;
  uint64_t total = st->next_index + 1;
  while (total % 2 == 0) {
    parent(st->stack[sl - 1], top_cv, PARENT, top_cv);
    sl--;
    total /= 2;
  }
  top_sl = sl;
  top_index = st->next_index;
  top_ok = true;
}
void Hasher::prime() const {
  if (st->total_len && st->tail_len > CHUNK_LEN) first_chunk_top();
}

// Hasher::finalize (src/hash.rs:276-302) without touching the state: the
// first chunk's output, when the tail holds two, is merged into a virtual
// copy of the stack top; the last chunk needs only its last block.
void Hasher::finalize(uint8_t out[32]) const {
  if (st->total_len == 0) {
    uint32_t w[16] = {0}, o[8];
    compress_cv(IV, w, 0, 0, CHUNK_START | CHUNK_END | ROOT, o);
    for (int i = 0; i < 8; i++) put32(out + 4 * i, o[i]);
    return;
  }
  size_t tl = st->tail_len;
  uint32_t sl = st->stack_len;
  const uint8_t* top = nullptr;
  bool have_top = false;  // virtual stack = stack[0..sl) (+ top)
  uint32_t h = 0;
  if (tl > CHUNK_LEN) {
    first_chunk_top();
    top = top_cv;
    sl = top_sl;
    have_top = true;
    h = 1;
  }
  const uint8_t* chunk = st->tail + CHUNK_LEN * h;
  size_t len = tl - CHUNK_LEN * h;
  uint32_t last = (uint32_t)((len + 63) / 64) - 1;  // == nblk[h]
  size_t depth = sl + (have_top ? 1 : 0);
  uint32_t w[16], o[8];
  chunk_block(chunk, len, last, w);
  uint32_t flags = (last == 0 ? (uint32_t)CHUNK_START : 0u) | CHUNK_END | (depth == 0 ? ROOT : 0u);
  compress_cv(cv[h], w, st->next_index + h, (uint32_t)(len - 64 * (size_t)last), flags, o);
  uint8_t cur[32];
  for (int i = 0; i < 8; i++) put32(cur + 4 * i, o[i]);
  if (depth == 0) {
    std::memcpy(out, cur, 32);
    return;
  }
  auto entry = [&](size_t i) -> const uint8_t* { return i < sl ? st->stack[i] : top; };
  for (size_t i = depth - 1; i >= 1; i--) parent(entry(i), cur, PARENT, cur);
  parent(entry(0), cur, PARENT | ROOT, out);
}

void blake3(const uint8_t* data, size_t len, uint8_t out[32]) {
  z0p_transcript_state st;
  std::memset(&st, 0, sizeof st);
  Hasher hs(&st);
  hs.update(data, len);
  hs.finalize(out);
}

// ------------------------------------------------------------- transcript ----
void Transcript::absorb_raw(const uint8_t* label, size_t llen, const uint8_t* data,
                            size_t len) {  // src/transcript.rs:72-77
  uint8_t hdr[16 + 64];
  if (llen <= 64) {  // LE64(|label|) || label || LE64(|data|) in one update
    put64(hdr, llen);
    std::memcpy(hdr + 8, label, llen);
    put64(hdr + 8 + llen, len);
    h_.update(hdr, 16 + llen);
  } else {
    put64(hdr, llen);
    h_.update(hdr, 8);
    h_.update(label, llen);
    put64(hdr, len);
    h_.update(hdr, 8);
  }
  h_.update(data, len);
}
void Transcript::absorb(const char* label, const uint8_t* data, size_t len) {
  absorb_raw((const uint8_t*)label, std::strlen(label), data, len);
}
void Transcript::absorb_each(const char* label, const uint8_t* data, size_t count, size_t len) {
  const size_t llen = std::strlen(label), item = 16 + llen + len;
  if (llen > 64 || item > 1024) {
    for (size_t i = 0; i < count; i++) absorb_raw((const uint8_t*)label, llen, data + i * len, len);
    return;
  }
  uint8_t buf[2048];  // whole framed items, LE64(|label|) || label || LE64(len) || item
  size_t n = 0;
  for (size_t i = 0; i < count; i++) {
    if (n + item > sizeof buf) {
      h_.update(buf, n);
      n = 0;
    }
    put64(buf + n, llen);
    std::memcpy(buf + n + 8, label, llen);
    put64(buf + n + 8 + llen, len);
    std::memcpy(buf + n + 16 + llen, data + i * len, len);
    n += item;
  }
  if (n) h_.update(buf, n);
}
void Transcript::squeeze(const uint8_t* label, size_t llen, uint8_t out[32]) {
  // src/transcript.rs:162-171 on a copy of the history: only the parts in
  // use (tail bytes, stack entries, counts) are copied.
  const z0p_transcript_state& s = *h_.st;
  z0p_transcript_state copy;
  copy.tail_len = s.tail_len;
  std::memcpy(copy.tail, s.tail, s.tail_len);
  copy.stack_len = s.stack_len;
  std::memcpy(copy.stack, s.stack, 32 * (size_t)s.stack_len);
  copy.next_index = s.next_index;
  copy.total_len = s.total_len;
  copy.counter = s.counter;
  h_.prime();  // the copy inherits the first chunk's merged entry
  Hasher hc = h_;
  hc.st = &copy;
  uint8_t sfx[16 + 64];
  if (llen <= 64) {  // LE64(|label|) || label || LE64(counter) in one update
    put64(sfx, llen);
    std::memcpy(sfx + 8, label, llen);
    put64(sfx + 8 + llen, s.counter);
    hc.update(sfx, 16 + llen);
  } else {
    put64(sfx, llen);
    hc.update(sfx, 8);
    hc.update(label, llen);
    put64(sfx, s.counter);
    hc.update(sfx, 8);
  }
  h_.st->counter++;
  hc.finalize(out);
  absorb_raw(label, llen, out, 32);
}
void Transcript::challenge_ext(const char* label, uint32_t out[4]) {
  uint8_t b[32];  // src/transcript.rs:136-141, src/ext4.rs:179-187
  squeeze((const uint8_t*)label, std::strlen(label), b);
  for (int i = 0; i < 4; i++) out[i] = le32(b + 4 * i) % P;
}
uint64_t Transcript::challenge_index(const char* label, uint64_t domain) {
  uint8_t b[32];  // src/transcript.rs:148-160 (domain checked by the caller)
  squeeze((const uint8_t*)label, std::strlen(label), b);
  uint64_t v = 0;
  for (int i = 0; i < 8; i++) v |= (uint64_t)b[i] << (8 * i);
  return v & (domain - 1);
}
std::vector<uint8_t> Transcript::pow_head(const char* label) const {
  size_t ll = std::strlen(label);  // src/transcript.rs:182-189
  std::vector<uint8_t> head(40 + ll);
  h_.finalize(head.data());
  put64(head.data() + 32, ll);
  std::memcpy(head.data() + 40, label, ll);
  return head;
}

void transcript_init(z0p_transcript_state* st, const uint8_t* label, size_t len) {
  std::memset(st, 0, sizeof *st);  // src/transcript.rs:62-69
  Transcript(st).absorb("domain", label, len);
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
      uint64_t total = est_fri(layers, q, h);
      if (col_lde) total = sat_add(total, est_col(col_lde, q, col_vb, h));  // 0: no column
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

// ---------------------------------------------------------------- ChaCha20 ----
// RFC 8439 section 2.3: 20 rounds (10 column/diagonal double rounds) over the
// constant, key, counter and nonce words, plus the input (src/rng.rs:22-73).
static inline uint32_t rotl32(uint32_t x, int n) { return (x << n) | (x >> (32 - n)); }
static inline void chacha_qr(uint32_t* x, int a, int b, int c, int d) {
  x[a] += x[b]; x[d] = rotl32(x[d] ^ x[a], 16);
  x[c] += x[d]; x[b] = rotl32(x[b] ^ x[c], 12);
  x[a] += x[b]; x[d] = rotl32(x[d] ^ x[a], 8);
  x[c] += x[d]; x[b] = rotl32(x[b] ^ x[c], 7);
}
void chacha20_block(const uint8_t key[32], uint32_t counter, const uint8_t nonce[12],
                    uint8_t out[64]) {
  uint32_t in[16] = {0x61707865u, 0x3320646eu, 0x79622d32u, 0x6b206574u};
  for (int i = 0; i < 8; i++) in[4 + i] = le32(key + 4 * i);
  in[12] = counter;
  for (int i = 0; i < 3; i++) in[13 + i] = le32(nonce + 4 * i);
  uint32_t x[16];
  for (int i = 0; i < 16; i++) x[i] = in[i];
  for (int r = 0; r < 10; r++) {
    chacha_qr(x, 0, 4, 8, 12); chacha_qr(x, 1, 5, 9, 13);
    chacha_qr(x, 2, 6, 10, 14); chacha_qr(x, 3, 7, 11, 15);
    chacha_qr(x, 0, 5, 10, 15); chacha_qr(x, 1, 6, 11, 12);
    chacha_qr(x, 2, 7, 8, 13); chacha_qr(x, 3, 4, 9, 14);
  }
  for (int i = 0; i < 16; i++) {
    const uint32_t v = x[i] + in[i];
    for (int b = 0; b < 4; b++) out[4 * i + b] = (uint8_t)(v >> (8 * b));
  }
}
void chacha20_fill(z0p_chacha20_state* s, uint8_t* out, size_t n) {  // src/rng.rs:115-131
  size_t done = 0;
  while (done < n) {
    if (s->used >= 64) {
      chacha20_block(s->key, s->counter, s->nonce, s->block);
      s->counter += 1;
      s->used = 0;
    }
    size_t take = 64 - s->used < n - done ? 64 - s->used : n - done;
    for (size_t i = 0; i < take; i++) out[done + i] = s->block[s->used + i];
    s->used += (uint32_t)take;
    done += take;
  }
}
uint32_t chacha20_next_field(z0p_chacha20_state* s) {  // src/rng.rs:157-167
  const uint64_t limit = ((1ull << 32) / P) * P;
  for (;;) {
    uint8_t w[4];
    chacha20_fill(s, w, 4);
    const uint64_t v = le32(w);
    if (v < limit) return (uint32_t)(v % P);
  }
}

}  // namespace host
}  // namespace z0p
