// Host-side pieces of the z0p GB300 prover: BabyBear scalar arithmetic, the
// streaming BLAKE3 hasher and Fiat-Shamir transcript over the C-ABI state,
// parameter rules and tuners, and the proof shape/size arithmetic.
#pragma once
#include <cstddef>
#include <cstdint>
#include <string>
#include <vector>

#include "../../include/z0p_gpu.h"

namespace z0p {
namespace host {

constexpr uint32_t P = 2013265921u;
constexpr uint32_t GENERATOR = 31u;
constexpr uint32_t TWO_ADICITY = 27u;
constexpr uint64_t MAX_DOMAIN = 1ull << 27;

inline uint32_t fadd(uint32_t a, uint32_t b) { uint32_t s = a + b; return s >= P ? s - P : s; }
inline uint32_t fsub(uint32_t a, uint32_t b) { return a >= b ? a - b : P - (b - a); }
inline uint32_t fmul(uint32_t a, uint32_t b) { return (uint32_t)((uint64_t)a * b % P); }
uint32_t fpow(uint32_t a, uint64_t e);
inline uint32_t finv(uint32_t a) { return fpow(a, P - 2); }
inline uint32_t to_mont(uint32_t a) { return (uint32_t)(((uint64_t)a << 32) % P); }
inline bool is_pow2(uint64_t x) { return x && !(x & (x - 1)); }
inline uint32_t log2u(uint64_t x) { return (uint32_t)__builtin_ctzll(x); }
uint32_t two_adic_generator(uint32_t bits);  // bits <= 27
uint64_t brev(uint64_t x, uint32_t bits);

// BLAKE3 (unkeyed, 32-byte output).
void blake3(const uint8_t* data, size_t len, uint8_t out[32]);

// Streaming BLAKE3 hasher of src/hash.rs:233-324 over the C-ABI state. The
// state bytes evolve exactly as the reference's do; beside them, cv[h] holds
// tail chunk h (tail bytes 1024h..) after its first nblk[h] blocks — every
// block known not to be its chunk's last — so finalize compresses only the
// last block of each open chunk instead of re-hashing the whole tail.
struct Hasher {
  z0p_transcript_state* st;
  uint32_t cv[2][8];
  uint32_t nblk[2];
  explicit Hasher(z0p_transcript_state* s);  // builds the cache from the state
  void update(const uint8_t* data, size_t len);
  void finalize(uint8_t out[32]) const;
  // Leaves this cache for the next Hasher this thread builds on the same
  // tail (host.cpp, CacheMemo).
  void remember() const;
  // Computes the merged first-chunk entry finalize needs (below) now, so
  // that copies of this hasher start with it.
  void prime() const;

 private:
  void advance();
  void first_chunk_top() const;
  // While the tail holds two chunks, finalize merges the first chunk's
  // output into the stack: the result (stack[0..top_sl) then top_cv) is
  // fixed until the first chunk is pushed, i.e. for one next_index.
  mutable bool top_ok = false;
  mutable uint64_t top_index = 0;
  mutable uint32_t top_sl = 0;
  mutable uint8_t top_cv[32];
};

// Fiat-Shamir transcript (src/transcript.rs:54-189) over the C-ABI state.
class Transcript {
 public:
  explicit Transcript(z0p_transcript_state* st) : h_(st) {}
  ~Transcript() { h_.remember(); }
  void absorb_raw(const uint8_t* label, size_t llen, const uint8_t* data, size_t len);
  void absorb(const char* label, const uint8_t* data, size_t len);
  // `count` absorbs under one label of consecutive `len`-byte items: the same
  // bytes as that many absorb calls, hashed in a few large updates.
  void absorb_each(const char* label, const uint8_t* data, size_t count, size_t len);
  void squeeze(const uint8_t* label, size_t llen, uint8_t out[32]);
  void challenge_ext(const char* label, uint32_t out[4]);
  uint64_t challenge_index(const char* label, uint64_t domain);
  // pow_head (src/transcript.rs:182-189): H(history) || LE64(|label|) || label.
  std::vector<uint8_t> pow_head(const char* label) const;

 private:
  Hasher h_;
};

void transcript_init(z0p_transcript_state* st, const uint8_t* label, size_t len);
inline void transcript_absorb(Transcript& t, const char* label, const uint8_t* data, size_t len) {
  t.absorb(label, data, len);
}
inline void challenge_ext(Transcript& t, const char* label, uint32_t out[4]) {
  t.challenge_ext(label, out);
}
inline uint64_t challenge_index(Transcript& t, const char* label, uint64_t domain) {
  return t.challenge_index(label, domain);
}
inline std::vector<uint8_t> pow_head(const Transcript& t, const char* label) {
  return t.pow_head(label);
}

// FRI parameter rules (src/fri.rs:105-196) and tuners (src/fri.rs:945-1074).
struct FriParams {
  uint64_t blowup, num_queries, final_size;
  uint32_t grinding_bits;
  uint64_t cap_height;
};
int fri_params_new(uint64_t blowup, uint64_t q, uint64_t final_size, FriParams* out);
int fri_params_validate(const FriParams& p);
// col_lde = 0: no opened column beside the FRI layers (fri::Params::for_security).
void tune_shape(uint64_t lde_len, uint64_t q, uint64_t col_lde, uint64_t col_vb,
                uint64_t* final_size, uint64_t* cap_height);
void tune_strength(uint32_t target, uint32_t millibits, uint64_t* q, uint32_t* g);
uint32_t composition_millibits(uint64_t lde_len, uint64_t degree_bound);

int air_validate(const z0p_air_params& p);
int range_validate(const z0p_range_params& p);

// Shape of the FRI layer stack and trees for an LDE of length m.
struct FriShape {
  uint64_t m;
  std::vector<uint64_t> len;      // layer lengths, m down to final_size
  std::vector<uint64_t> leaves;   // Merkle leaves per layer
  std::vector<uint32_t> depth;    // log2(leaves)
  std::vector<uint32_t> drop;     // cap level drop = min(cap_height, depth)
};
// Checks commit_inner's preconditions (src/fri.rs:551-575) and builds the shape.
int fri_shape(uint64_t m, uint64_t degree_bound, const FriParams& fp, FriShape* out);
uint64_t fri_bytes(const FriShape& s, uint64_t q);  // commitment + proof bodies

void set_reason(const std::string& r);

// ChaCha20 (RFC 8439) stream over the C-ABI state (src/rng.rs:40-167).
void chacha20_block(const uint8_t key[32], uint32_t counter, const uint8_t nonce[12],
                    uint8_t out[64]);
void chacha20_fill(z0p_chacha20_state* s, uint8_t* out, size_t n);
uint32_t chacha20_next_field(z0p_chacha20_state* s);  // rejection above 2p

}  // namespace host
}  // namespace z0p
