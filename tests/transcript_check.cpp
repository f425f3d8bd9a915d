// Long-lived transcript check: one host Transcript object (with its cached
// chunk chaining values) against the oracle's transcript over random absorb /
// squeeze sequences that cross the 64-, 1024- and 2048-byte boundaries.
// Built and run by tests/test_host_transcript.py; prints "ok <ops>" or the
// first mismatch, and the host cost of a squeeze on a long transcript.
#include <chrono>
#include <cstdio>
#include <cstring>
#include <vector>

#include "host.h"

extern "C" {
#include "z0p_oracle.h"
}

using z0p::host::Transcript;

static uint64_t rng = 0x9E3779B97F4A7C15ull;
static uint64_t next() {
  rng ^= rng << 13;
  rng ^= rng >> 7;
  rng ^= rng << 17;
  return rng;
}

static bool same_state(const z0p_transcript_state& s, const zo_transcript* o) {
  z0p_transcript_state e;
  std::memset(&e, 0, sizeof e);
  zo_transcript_export(o, e.tail, &e.tail_len, e.stack, &e.stack_len, &e.next_index, &e.total_len,
                       &e.counter);
  return s.tail_len == e.tail_len && std::memcmp(s.tail, e.tail, s.tail_len) == 0 &&
         s.stack_len == e.stack_len && std::memcmp(s.stack, e.stack, 32 * s.stack_len) == 0 &&
         s.next_index == e.next_index && s.total_len == e.total_len && s.counter == e.counter;
}

int main() {
  const size_t sizes[] = {0, 1, 7, 31, 32, 33, 63, 64, 65, 127, 128, 960, 1000, 1023, 1024, 1025, 2047, 2048, 2049, 5000};
  long ops = 0;
  for (int trial = 0; trial < 60; trial++) {
    uint8_t label[16];
    int ll = std::snprintf((char*)label, sizeof label, "trial-%d", trial);
    z0p_transcript_state st;
    z0p::host::transcript_init(&st, label, (size_t)ll);
    Transcript t(&st);
    zo_transcript* o = zo_transcript_new(label, (size_t)ll);
    int steps = 20 + (int)(next() % 200);
    for (int k = 0; k < steps; k++, ops++) {
      uint64_t op = next() % 10;
      if (op < 5) {
        size_t n = sizes[next() % (sizeof sizes / sizeof sizes[0])];
        std::vector<uint8_t> d(n);
        for (auto& x : d) x = (uint8_t)next();
        t.absorb_raw((const uint8_t*)"fri-layer-root", 14, d.data(), n);
        zo_transcript_absorb(o, (const uint8_t*)"fri-layer-root", 14, d.data(), n);
      } else if (op < 8) {
        uint8_t a[32], b[32];
        t.squeeze((const uint8_t*)"fri-query", 9, a);
        zo_transcript_challenge_bytes(o, (const uint8_t*)"fri-query", 9, b);
        if (std::memcmp(a, b, 32)) {
          std::printf("squeeze mismatch trial %d step %d\n", trial, k);
          return 1;
        }
      } else {
        std::vector<uint8_t> h = t.pow_head("fri-pow");
        zo_transcript* c = zo_transcript_clone(o);
        uint8_t b[32];  // H(history) is the first 32 bytes of the head
        z0p_transcript_state e;
        std::memset(&e, 0, sizeof e);
        zo_transcript_export(c, e.tail, &e.tail_len, e.stack, &e.stack_len, &e.next_index,
                             &e.total_len, &e.counter);
        z0p::host::Hasher hh(&e);
        hh.finalize(b);
        zo_transcript_free(c);
        if (std::memcmp(h.data(), b, 32)) {
          std::printf("pow head mismatch trial %d step %d\n", trial, k);
          return 1;
        }
      }
      if (!same_state(st, o)) {
        std::printf("state mismatch trial %d step %d\n", trial, k);
        return 1;
      }
    }
    zo_transcript_free(o);
  }
  // Host cost of one squeeze on a transcript with a part-filled second chunk.
  z0p_transcript_state st;
  z0p::host::transcript_init(&st, (const uint8_t*)"t", 1);
  Transcript t(&st);
  std::vector<uint8_t> d(1500, 7);
  t.absorb("x", d.data(), d.size());
  const int n = 20000;
  uint8_t out[32];
  auto t0 = std::chrono::steady_clock::now();
  for (int i = 0; i < n; i++) t.squeeze((const uint8_t*)"fri-query", 9, out);
  double us = std::chrono::duration<double, std::micro>(std::chrono::steady_clock::now() - t0).count() / n;
  std::printf("ok %ld squeeze_us %.3f\n", ops, us);
  return 0;
}
