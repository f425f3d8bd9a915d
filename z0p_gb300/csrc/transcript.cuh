// Device Fiat-Shamir transcript: the streaming BLAKE3 hasher of
// src/hash.rs:233-324 and the transcript of src/transcript.rs:54-189 over a
// DevTranscript record in shared memory, so that a proof's challenges are
// drawn where its commitments are made and the launches after them need no
// host round trip.
//
// One warp per proof. A BLAKE3 stream is one chain of compressions, so lane 0
// does every compression, through one non-inlined routine reading its block
// straight from the record's tail in shared memory; the warp
// writes the framed messages into the tail in parallel and moves records and
// absorbed data between global and shared memory. The record evolves exactly
// as the host's Transcript (host.cpp) evolves the same state: tail bytes,
// chaining-value stack, chunk and byte counts, squeeze counter, block cache.
#pragma once

namespace dtr {

constexpr uint32_t kChunk = 1024;
constexpr uint32_t kTail = 2 * kChunk;
constexpr uint32_t kStackMax = 54;

// The one copy of the compression in this kernel: a single warp runs through
// the hasher's straight-line code once, so every inlined copy would be
// fetched cold; this one stays in the instruction cache. Chaining values and
// blocks come by pointer (shared or local memory, 4-byte aligned); out may
// alias cv.
__device__ __noinline__ void compress_at(const uint32_t* cv, const uint32_t* w, uint64_t counter,
                                         uint32_t len, uint32_t flags, uint32_t* out) {
  uint32_t c[8], m[16], o[8];
#pragma unroll
  for (int i = 0; i < 8; i++) c[i] = cv[i];
#pragma unroll
  for (int i = 0; i < 16; i++) m[i] = w[i];
  blake3_compress(c, m, (uint32_t)counter, (uint32_t)(counter >> 32), len, flags, o);
#pragma unroll
  for (int i = 0; i < 8; i++) out[i] = o[i];
}

// Parent node of two chaining values (src/hash.rs:161-176).
__device__ __noinline__ void parent_at(const uint32_t* l, const uint32_t* r, uint32_t flags,
                                       uint32_t* out) {
  uint32_t w[16], iv[8];
#pragma unroll
  for (int i = 0; i < 8; i++) {
    w[i] = l[i];
    w[8 + i] = r[i];
  }
  iv_words(iv);
  compress_at(iv, w, 0ull, 64u, flags, out);
}

// The hasher's block cache: cv[h] is tail chunk h after its first nb[h]
// blocks (laid out as DevTranscript's cv and nblk).
struct Cache {
  uint32_t cv[2][8];
  uint32_t nb[2];
};
__device__ __forceinline__ Cache& cache_of(DevTranscript& T) {
  return *reinterpret_cast<Cache*>(&T.cv[0][0]);
}
static_assert(offsetof(DevTranscript, nblk) == offsetof(DevTranscript, cv) + offsetof(Cache, nb),
              "the cache fields are laid out as Cache");

// Folds into the cache every block of the tail (tail_len bytes) that has a
// byte after it in its chunk: such a block is never its chunk's last, so its
// compression (CHUNK_START or no flag, counter = chunk index) is final.
__device__ __noinline__ void advance(const uint8_t* tail, uint32_t tail_len, uint64_t next_index,
                                     Cache& c) {
  for (uint32_t h = 0; h < 2; h++) {
    const uint32_t base = kChunk * h;
    if (tail_len <= base) break;
    const uint32_t len = tail_len - base < kChunk ? tail_len - base : kChunk;
    while (64 * (c.nb[h] + 1) < len) {
      const uint32_t* blk = reinterpret_cast<const uint32_t*>(tail + base + 64 * c.nb[h]);
      compress_at(c.cv[h], blk, next_index + h, 64u, c.nb[h] == 0 ? kChunkStart : 0u, c.cv[h]);
      c.nb[h]++;
    }
  }
}

// Hasher::push_merged (src/hash.rs:305-318) on the record's stack.
__device__ __noinline__ void push_merged(DevTranscript& T, uint32_t* cv) {
  z0p_transcript_state& s = T.st;
  uint32_t sl = s.stack_len;
  const uint64_t n = s.next_index + 1;
  for (uint64_t total = n; (total & 1ull) == 0; total >>= 1) {
    --sl;
    parent_at(reinterpret_cast<const uint32_t*>(s.stack[sl]), cv, kParent, cv);
  }
  uint32_t* dst = reinterpret_cast<uint32_t*>(s.stack[sl++]);
  for (int i = 0; i < 8; i++) dst[i] = cv[i];
  s.stack_len = sl;
  s.next_index = n;
}

// The last block of a chunk holding len bytes (1..1024), zero padded.
__device__ __forceinline__ void last_block(const uint8_t* chunk, uint32_t len, uint32_t w[16]) {
  const uint32_t b = (len - 1) / 64, n = len - 64 * b;
  const uint32_t* q = reinterpret_cast<const uint32_t*>(chunk + 64 * b);
  for (int j = 0; j < 16; j++) {
    const int rem = (int)n - 4 * j;
    w[j] = rem <= 0 ? 0u : rem < 4 ? q[j] & ((1u << (8 * rem)) - 1u) : q[j];
  }
}

// Hasher::finalize (src/hash.rs:276-302) of the record's stack with a tail of
// tail_len bytes and the cache c, without changing either.
__device__ __noinline__ void finalize(const DevTranscript& T, uint32_t tail_len,
                                      uint64_t total_len, const Cache& c, uint32_t* out) {
  const z0p_transcript_state& s = T.st;
  uint32_t w[16], iv[8];
  iv_words(iv);
  if (total_len == 0) {
    for (int i = 0; i < 16; i++) w[i] = 0u;
    compress_at(iv, w, 0ull, 0u, kChunkStart | kChunkEnd | kRoot, out);
    return;
  }
  uint32_t sl = s.stack_len;
  uint32_t top[8], cur[8];
  bool have_top = false;  // virtual stack: stack[0..sl) and then top
  if (tail_len > kChunk) {
    // The first tail chunk ends here: merged as push_merged would, virtually.
    compress_at(c.cv[0], reinterpret_cast<const uint32_t*>(s.tail + 64 * 15), s.next_index, 64u,
                kChunkEnd, top);
    for (uint64_t total = s.next_index + 1; (total & 1ull) == 0; total >>= 1) {
      --sl;
      parent_at(reinterpret_cast<const uint32_t*>(s.stack[sl]), top, kParent, top);
    }
    have_top = true;
    const uint32_t len = tail_len - kChunk, last = (len - 1) / 64;
    last_block(s.tail + kChunk, len, w);
    compress_at(c.cv[1], w, s.next_index + 1, len - 64 * last,
                (last == 0 ? kChunkStart : 0u) | kChunkEnd, cur);
  } else {
    const uint32_t len = tail_len, last = (len - 1) / 64;
    last_block(s.tail, len, w);
    compress_at(c.cv[0], w, s.next_index, len - 64 * last,
                (last == 0 ? kChunkStart : 0u) | kChunkEnd | (sl == 0 ? kRoot : 0u), cur);
  }
  const uint32_t depth = sl + (have_top ? 1u : 0u);
  if (depth == 0) {
    for (int i = 0; i < 8; i++) out[i] = cur[i];
    return;
  }
  // Merge from the top of the virtual stack down; the bottom one is the root.
  for (uint32_t i = depth - 1;; i--) {
    const uint32_t* l = i < sl ? reinterpret_cast<const uint32_t*>(s.stack[i]) : top;
    if (i == 0) {
      parent_at(l, cur, kParent | kRoot, out);
      return;
    }
    parent_at(l, cur, kParent, cur);
  }
}

// The bytes of framed messages, item after item: for each item,
// LE64(|label|) || label || LE64(word) || data, where word = |data| for an
// absorb (src/transcript.rs:72-77) and the squeeze counter, with no data, for
// a squeeze's suffix (src/transcript.rs:162-171).
struct Msg {
  const char* label;
  uint32_t llen;
  uint64_t word;
  const uint8_t* data;  // item j's bytes at data + j * dlen (shared memory)
  uint32_t dlen;
  uint32_t count;
  __device__ __forceinline__ uint32_t size() const { return (16 + llen + dlen) * count; }
  __device__ __forceinline__ uint8_t at(uint32_t i) const {
    const uint32_t S = 16 + llen + dlen, j = i / S, o = i - j * S;
    if (o < 8) return (uint8_t)((uint64_t)llen >> (8 * o));
    if (o < 8 + llen) return (uint8_t)label[o - 8];
    if (o < 16 + llen) return (uint8_t)(word >> (8 * (o - 8 - llen)));
    return data[(size_t)j * dlen + (o - 16 - llen)];
  }
};

// Hasher::update (src/hash.rs:256-272) of a message, with the warp. The tail
// is filled in parallel up to two chunks; lane 0 then folds its finished
// blocks, and when the tail is full, ends its first chunk and pushes it, and
// the warp moves the second chunk down. Every lane must call it.
__device__ void update(DevTranscript& T, const Msg& m) {
  const uint32_t lane = threadIdx.x, n = m.size();
  uint32_t done = 0;
  while (done < n) {
    __syncwarp();
    const uint32_t tl = T.st.tail_len;
    const uint32_t take = n - done < kTail - tl ? n - done : kTail - tl;
    for (uint32_t i = lane; i < take; i += 32) T.st.tail[tl + i] = m.at(done + i);
    __syncwarp();
    int full = 0;
    if (lane == 0) {
      Cache& c = cache_of(T);
      advance(T.st.tail, tl + take, T.st.next_index, c);
      T.st.tail_len = tl + take;
      T.st.total_len += take;
      if (tl + take == kTail) {
        // Blocks 0..14 of the first chunk are folded; its last block ends it.
        uint32_t out[8];
        compress_at(c.cv[0], reinterpret_cast<const uint32_t*>(T.st.tail + 64 * 15),
                    T.st.next_index, 64u, kChunkEnd, out);
        push_merged(T, out);
        for (int i = 0; i < 8; i++) c.cv[0][i] = c.cv[1][i];
        c.nb[0] = c.nb[1];
        iv_words(c.cv[1]);
        c.nb[1] = 0;
        T.st.tail_len = kChunk;
        full = 1;
      }
    }
    full = __shfl_sync(0xffffffffu, full, 0);
    if (full) {
      __syncwarp();
      uint4* t = reinterpret_cast<uint4*>(T.st.tail);
      for (uint32_t i = lane; i < kChunk / 16; i += 32) t[i] = t[kChunk / 16 + i];
    }
    done += take;
  }
  __syncwarp();
}

// Copies `bytes` (a multiple of 16, both ends 16-byte aligned) with the warp.
__device__ __forceinline__ void warp_copy16(void* dst, const void* src, uint32_t bytes) {
  uint4* d = reinterpret_cast<uint4*>(dst);
  const uint4* s = reinterpret_cast<const uint4*>(src);
  for (uint32_t i = threadIdx.x; i < bytes / 16; i += 32) d[i] = s[i];
}

// Copies `bytes` from any address to a 16-byte aligned buffer with the warp,
// in 16-byte words when the source allows.
__device__ __forceinline__ void warp_stage(uint8_t* dst, const uint8_t* src, uint32_t bytes) {
  if ((reinterpret_cast<uintptr_t>(src) & 15u) == 0 && (bytes & 15u) == 0) {
    warp_copy16(dst, src, bytes);
  } else {
    for (uint32_t i = threadIdx.x; i < bytes; i += 32) dst[i] = src[i];
  }
}

// The meaningful part of a record (tail and stack in use, counters, cache).
__device__ __forceinline__ void warp_clone(DevTranscript& C, const DevTranscript& T) {
  const uint32_t tail16 = (T.st.tail_len + 15) / 16 * 16;
  warp_copy16(C.st.tail, T.st.tail, tail16);
  for (uint32_t i = threadIdx.x; i < 8 * T.st.stack_len; i += 32)
    reinterpret_cast<uint32_t*>(C.st.stack)[i] = reinterpret_cast<const uint32_t*>(T.st.stack)[i];
  if (threadIdx.x == 0) {
    C.st.tail_len = T.st.tail_len;
    C.st.stack_len = T.st.stack_len;
    C.st.next_index = T.st.next_index;
    C.st.total_len = T.st.total_len;
    C.st.counter = T.st.counter;
  }
  if (threadIdx.x < 16) (&C.cv[0][0])[threadIdx.x] = (&T.cv[0][0])[threadIdx.x];
  if (threadIdx.x < 2) C.nblk[threadIdx.x] = T.nblk[threadIdx.x];
  __syncwarp();
}

// squeeze_raw (src/transcript.rs:162-171): the hash of the history with the
// label and counter appended, which is then absorbed. When the suffix fits
// in the tail, it is written past the record's bytes and hashed from a copy
// of the cache (the absorb that follows overwrites it); otherwise a copy of
// the record is extended. Every lane must call it; lane 0 receives out.
__device__ void squeeze(DevTranscript& T, DevTranscript& C, uint8_t* out_bytes, const char* label,
                        uint32_t llen, uint32_t out[8]) {
  const uint32_t lane = threadIdx.x;
  __syncwarp();
  const Msg suffix{label, llen, T.st.counter, nullptr, 0, 1};
  const uint32_t S = suffix.size(), tl = T.st.tail_len;
  if (tl + S < kTail) {
    for (uint32_t i = lane; i < S; i += 32) T.st.tail[tl + i] = suffix.at(i);
    __syncwarp();
    if (lane == 0) {
      Cache& c = cache_of(C);  // the copy's cache area is free here
      c = cache_of(T);
      advance(T.st.tail, tl + S, T.st.next_index, c);
      finalize(T, tl + S, T.st.total_len + S, c, out);
    }
  } else {
    warp_clone(C, T);
    update(C, suffix);
    if (lane == 0) finalize(C, C.st.tail_len, C.st.total_len, cache_of(C), out);
  }
  if (lane == 0) {
    T.st.counter++;
#pragma unroll
    for (int i = 0; i < 8; i++) reinterpret_cast<uint32_t*>(out_bytes)[i] = out[i];
  }
  __syncwarp();
  update(T, Msg{label, llen, 32, out_bytes, 32, 1});
}

}  // namespace dtr

// Runs one TranscriptArgs program for proof blockIdx.x (one warp).
__global__ void __launch_bounds__(32) transcript_kernel(const __grid_constant__ TranscriptArgs a) {
  __shared__ __align__(16) DevTranscript T;
  __shared__ __align__(16) DevTranscript C;
  __shared__ __align__(16) uint8_t stage[kTrStage];
  __shared__ __align__(16) uint8_t sq[32];
  const uint32_t k = blockIdx.x, lane = threadIdx.x;
  dtr::warp_copy16(&T, a.in + k, sizeof(DevTranscript));
  __syncwarp();
  // A record the hasher could run out of bounds on is left alone. (The stack
  // holds one value per set bit of the chunk count, so it never outgrows a
  // consistent record.)
  if (T.st.tail_len >= dtr::kTail || T.st.stack_len > dtr::kStackMax ||
      (uint32_t)__popcll(T.st.next_index) != T.st.stack_len || (T.st.next_index >> 53) != 0 ||
      T.nblk[0] > 15 || T.nblk[1] > 15) {
    if (lane == 0 && a.fault) atomicOr(a.fault, 4u);
    return;
  }
  for (uint32_t o = 0; o < a.nops; o++) {
    const TranscriptOp& op = a.op[o];
    if (op.kind == kTrAbsorb) {
      if (op.len == 0 || op.len > kTrStage) {  // the launcher refuses these
        if (lane == 0 && a.fault) atomicOr(a.fault, 4u);
        continue;
      }
      const uint8_t* src = static_cast<const uint8_t*>(op.src) + k * op.src_stride;
      const uint32_t per = kTrStage / op.len;
      for (uint32_t i0 = 0; i0 < op.count; i0 += per) {
        const uint32_t n = op.count - i0 < per ? op.count - i0 : per;
        __syncwarp();
        dtr::warp_stage(stage, src + (size_t)i0 * op.len, n * op.len);
        __syncwarp();
        dtr::update(T, dtr::Msg{op.label, op.label_len, op.len, stage, op.len, n});
      }
    } else if (op.kind == kTrFoldTables) {
      // challenge_ext x 3 (src/transcript.rs:136-141), then the tables of
      // r_k / 4 for e4_mul_tab.
      uint32_t ch[3][4];
#pragma unroll 1
      for (int r = 0; r < 3; r++) {
        uint32_t d[8] = {};
        dtr::squeeze(T, C, sq, op.label, op.label_len, d);
#pragma unroll
        for (int e = 0; e < 4; e++) ch[r][e] = __shfl_sync(0xffffffffu, d[e] % kP, 0);
      }
      if (lane < 16) {
        // Product by q in the tower (src/ext4.rs:106-117, u^2 = 11): output
        // coordinate c takes input coordinate i times q[kIdx], times 11
        // where kW11 says so; word 4c + i of each table.
        const uint32_t e = (0x0123103232012310ull >> (4 * lane)) & 0xfu;  // kIdx[lane]
        const bool w11 = (0x0a8eu >> lane) & 1u;                            // kW11[lane]
        const uint32_t inv4 = 1509949441u;  // 4^-1 mod p
#pragma unroll
        for (int r = 0; r < 3; r++) {
          const uint32_t q = e == 0 ? ch[r][0] : e == 1 ? ch[r][1] : e == 2 ? ch[r][2] : ch[r][3];
          uint64_t v = (uint64_t)q * inv4 % kP;
          if (w11) v = 11ull * v % kP;
          op.dst[k * op.dst_stride + 16 * r + lane] = to_mont((uint32_t)v);
        }
      }
    } else if (op.kind == kTrPowHead) {
      // H(history) || LE64(|label|) || label, as little-endian words.
      uint32_t d[8] = {};
      if (lane == 0) dtr::finalize(T, T.st.tail_len, T.st.total_len, dtr::cache_of(T), d);
      uint32_t v = 0;
#pragma unroll
      for (int i = 0; i < 8; i++) {
        const uint32_t di = __shfl_sync(0xffffffffu, d[i], 0);
        if ((uint32_t)i == lane) v = di;
      }
      if (lane >= 8 && lane < kPowHeadWords) {
        v = 0;
        for (uint32_t b = 0; b < 4; b++) {
          const uint32_t at = 4 * lane + b;  // byte of the head, 32 and up
          uint32_t x = 0;
          if (at < 40) x = (uint32_t)((uint64_t)op.label_len >> (8 * (at - 32)));
          else if (at < 40 + op.label_len) x = (uint8_t)op.label[at - 40];
          v |= (x & 0xffu) << (8 * b);
        }
      }
      if (lane < kPowHeadWords) op.dst[k * op.dst_stride + lane] = v;
    }
    __syncwarp();
  }
  __syncwarp();
  dtr::warp_copy16(a.out + k, &T, sizeof(DevTranscript));
}
