// Device Fiat-Shamir transcript: the streaming BLAKE3 hasher of
// src/hash.rs:233-324 and the transcript of src/transcript.rs:54-189 over a
// DevTranscript record in shared memory, so that a proof's challenges are
// drawn where its commitments are made and the launches after them need no
// host round trip.
//
// One warp per proof. Lane 0 does the hashing (a BLAKE3 stream is one chain
// of compressions); the warp moves records and absorbed data between global
// and shared memory. The record evolves exactly as the host's Transcript
// (host.cpp) evolves the same state: the tail bytes, the chaining-value stack,
// the chunk and byte counts, the squeeze counter and the block cache.
#pragma once

namespace dtr {

constexpr uint32_t kChunk = 1024;
constexpr uint32_t kTail = 2 * kChunk;
constexpr uint32_t kStackMax = 54;

// Block i of a chunk whose first len bytes are at p (4-byte aligned, inside
// a record's tail), zero padded past len.
__device__ __forceinline__ void chunk_block(const uint8_t* p, uint32_t len, uint32_t i,
                                            uint32_t w[16]) {
  const uint32_t off = 64 * i;
  const uint32_t n = len - off < 64 ? len - off : 64;
  const uint32_t* q = reinterpret_cast<const uint32_t*>(p + off);
#pragma unroll
  for (int j = 0; j < 16; j++) {
    const int rem = (int)n - 4 * j;
    uint32_t v = rem > 0 ? q[j] : 0u;
    if (rem > 0 && rem < 4) v &= (1u << (8 * rem)) - 1u;
    w[j] = v;
  }
}

__device__ __forceinline__ void compress(const uint32_t cv[8], uint32_t w[16], uint64_t counter,
                                         uint32_t len, uint32_t flags, uint32_t out[8]) {
  blake3_compress(cv, w, (uint32_t)counter, (uint32_t)(counter >> 32), len, flags, out);
}

__device__ __forceinline__ void load8(const uint8_t* p, uint32_t v[8]) {
  const uint32_t* q = reinterpret_cast<const uint32_t*>(p);
#pragma unroll
  for (int i = 0; i < 8; i++) v[i] = q[i];
}
__device__ __forceinline__ void store8(uint8_t* p, const uint32_t v[8]) {
  uint32_t* q = reinterpret_cast<uint32_t*>(p);
#pragma unroll
  for (int i = 0; i < 8; i++) q[i] = v[i];
}

// Parent node of two chaining values (src/hash.rs:161-176).
__device__ __forceinline__ void parent(const uint32_t l[8], const uint32_t r[8], uint32_t flags,
                                       uint32_t out[8]) {
  uint32_t w[16], iv[8];
#pragma unroll
  for (int i = 0; i < 8; i++) {
    w[i] = l[i];
    w[8 + i] = r[i];
  }
  iv_words(iv);
  compress(iv, w, 0ull, 64u, flags, out);
}

// Hasher::push_merged (src/hash.rs:305-318).
__device__ void push_merged(DevTranscript& T, const uint32_t cv[8]) {
  z0p_transcript_state& s = T.st;
  store8(s.stack[s.stack_len++], cv);
  s.next_index++;
  for (uint64_t total = s.next_index; (total & 1ull) == 0; total >>= 1) {
    uint32_t l[8], r[8], m[8];
    load8(s.stack[s.stack_len - 2], l);
    load8(s.stack[s.stack_len - 1], r);
    parent(l, r, kParent, m);
    s.stack_len--;
    store8(s.stack[s.stack_len - 1], m);
  }
}

// Folds into cv[h] every block of tail chunk h that has a byte after it in
// its chunk (such a block is never its chunk's last, so its compression is
// final), as the host hasher's cache does.
__device__ void advance(DevTranscript& T) {
  for (uint32_t h = 0; h < 2; h++) {
    const uint32_t base = kChunk * h;
    if (T.st.tail_len <= base) break;
    const uint32_t len = T.st.tail_len - base < kChunk ? T.st.tail_len - base : kChunk;
    while (64 * (T.nblk[h] + 1) < len) {
      uint32_t w[16];
      chunk_block(T.st.tail + base, len, T.nblk[h], w);
      compress(T.cv[h], w, T.st.next_index + h, 64u, T.nblk[h] == 0 ? kChunkStart : 0u, T.cv[h]);
      T.nblk[h]++;
    }
  }
}

// Hasher::update (src/hash.rs:256-272); data in any address space.
__device__ void update(DevTranscript& T, const uint8_t* data, uint32_t len) {
  z0p_transcript_state& s = T.st;
  s.total_len += len;
  while (len) {
    const uint32_t room = kTail - s.tail_len;
    const uint32_t take = len < room ? len : room;
    for (uint32_t i = 0; i < take; i++) s.tail[s.tail_len + i] = data[i];
    s.tail_len += take;
    data += take;
    len -= take;
    advance(T);
    if (s.tail_len == kTail) {
      // Blocks 0..14 of the first chunk are folded; its last block ends it.
      uint32_t w[16], out[8];
      chunk_block(s.tail, kChunk, 15, w);
      compress(T.cv[0], w, s.next_index, 64u, kChunkEnd, out);
      push_merged(T, out);
      uint32_t* tw = reinterpret_cast<uint32_t*>(s.tail);
      for (uint32_t i = 0; i < kChunk / 4; i++) tw[i] = tw[kChunk / 4 + i];
      s.tail_len = kChunk;
#pragma unroll
      for (int i = 0; i < 8; i++) {
        T.cv[0][i] = T.cv[1][i];
      }
      T.nblk[0] = T.nblk[1];
      iv_words(T.cv[1]);
      T.nblk[1] = 0;
    }
  }
}

__device__ __forceinline__ void update_u64(DevTranscript& T, uint64_t v) {
  uint8_t b[8];
#pragma unroll
  for (int i = 0; i < 8; i++) b[i] = (uint8_t)(v >> (8 * i));
  update(T, b, 8);
}

// Hasher::finalize (src/hash.rs:276-302), leaving the record unchanged.
__device__ void finalize(const DevTranscript& T, uint32_t out[8]) {
  const z0p_transcript_state& s = T.st;
  uint32_t iv[8];
  iv_words(iv);
  if (s.total_len == 0) {
    uint32_t w[16];
#pragma unroll
    for (int i = 0; i < 16; i++) w[i] = 0u;
    compress(iv, w, 0ull, 0u, kChunkStart | kChunkEnd | kRoot, out);
    return;
  }
  const uint32_t tl = s.tail_len;
  uint32_t sl = s.stack_len;
  uint32_t top[8];
  bool have_top = false;  // virtual stack: stack[0..sl) and then top
  uint32_t h = 0;
  if (tl > kChunk) {
    uint32_t w[16];
    chunk_block(s.tail, kChunk, 15, w);
    compress(T.cv[0], w, s.next_index, 64u, kChunkEnd, top);
    for (uint64_t total = s.next_index + 1; (total & 1ull) == 0; total >>= 1) {
      uint32_t l[8];
      load8(s.stack[sl - 1], l);
      parent(l, top, kParent, top);
      sl--;
    }
    have_top = true;
    h = 1;
  }
  const uint32_t len = tl - kChunk * h;
  const uint32_t last = (len + 63) / 64 - 1;
  const uint32_t depth = sl + (have_top ? 1u : 0u);
  uint32_t w[16], cur[8];
  chunk_block(s.tail + kChunk * h, len, last, w);
  const uint32_t flags =
      (last == 0 ? kChunkStart : 0u) | kChunkEnd | (depth == 0 ? kRoot : 0u);
  compress(T.cv[h], w, s.next_index + h, len - 64 * last, flags, cur);
  if (depth == 0) {
#pragma unroll
    for (int i = 0; i < 8; i++) out[i] = cur[i];
    return;
  }
  for (uint32_t i = depth - 1; i >= 1; i--) {
    uint32_t l[8];
    if (i < sl) load8(s.stack[i], l);
    else
#pragma unroll
      for (int j = 0; j < 8; j++) l[j] = top[j];
    parent(l, cur, kParent, cur);
  }
  uint32_t l[8];
  if (sl > 0) load8(s.stack[0], l);
  else
#pragma unroll
    for (int j = 0; j < 8; j++) l[j] = top[j];
  parent(l, cur, kParent | kRoot, out);
}

// Transcript::absorb (src/transcript.rs:72-77).
__device__ void absorb(DevTranscript& T, const char* label, uint32_t llen, const uint8_t* data,
                       uint32_t len) {
  update_u64(T, llen);
  update(T, reinterpret_cast<const uint8_t*>(label), llen);
  update_u64(T, len);
  update(T, data, len);
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

// squeeze_raw (src/transcript.rs:162-171): the hash of a copy of the history
// with the label and counter appended; the output is then absorbed. The warp
// makes the copy; lane 0 hashes. Every lane must call it.
__device__ void squeeze(DevTranscript& T, DevTranscript& C, const char* label, uint32_t llen,
                        uint32_t out[8]) {
  __syncwarp();
  warp_copy16(&C, &T, sizeof(DevTranscript));
  __syncwarp();
  if (threadIdx.x == 0) {
    update_u64(C, llen);
    update(C, reinterpret_cast<const uint8_t*>(label), llen);
    update_u64(C, T.st.counter);
    T.st.counter++;
    finalize(C, out);
    uint8_t b[32];
#pragma unroll
    for (int i = 0; i < 32; i++) b[i] = (uint8_t)(out[i / 4] >> (8 * (i % 4)));
    absorb(T, label, llen, b, 32);
  }
  __syncwarp();
}

}  // namespace dtr

// Runs one TranscriptArgs program for proof blockIdx.x (one warp).
__global__ void __launch_bounds__(32) transcript_kernel(const __grid_constant__ TranscriptArgs a) {
  __shared__ __align__(16) DevTranscript T;
  __shared__ __align__(16) DevTranscript C;
  __shared__ __align__(16) uint8_t stage[kTrStage];
  const uint32_t k = blockIdx.x, lane = threadIdx.x;
  dtr::warp_copy16(&T, a.in + k, sizeof(DevTranscript));
  __syncwarp();
  // A record the hasher could run out of bounds on is left alone.
  // (The stack holds one value per set bit of the chunk count, so it never
  // outgrows a consistent record.)
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
        if (lane == 0)
          for (uint32_t i = 0; i < n; i++)
            dtr::absorb(T, op.label, op.label_len, stage + (size_t)i * op.len, op.len);
      }
    } else if (op.kind == kTrFoldTables) {
      // challenge_ext x 3 (src/transcript.rs:136-141), then the tables of
      // r_k / 4 for e4_mul_tab: T[c][i] holds the coefficient of input
      // coordinate i in output coordinate c, times 2^32 (Montgomery).
      uint32_t ch[3][4];
      for (int r = 0; r < 3; r++) {
        uint32_t d[8];
        dtr::squeeze(T, C, op.label, op.label_len, d);
#pragma unroll
        for (int e = 0; e < 4; e++) ch[r][e] = d[e] % kP;
      }
      // Lane 0 drew the challenges; the 48 table words are spread over the
      // warp (lanes 0..15 each write table r's word for r = 0, 1, 2).
#pragma unroll
      for (int r = 0; r < 3; r++)
#pragma unroll
        for (int e = 0; e < 4; e++) ch[r][e] = __shfl_sync(0xffffffffu, ch[r][e], 0);
      if (lane < 16) {
        // Product by q in the tower (src/ext4.rs:106-117, u^2 = 11): output
        // coordinate c takes input coordinate i times q[kIdx], times 11
        // where kW11 says so.
        constexpr uint8_t kIdx[16] = {0, 1, 3, 2, 1, 0, 2, 3, 2, 3, 0, 1, 3, 2, 1, 0};
        constexpr uint8_t kW11[16] = {0, 1, 1, 1, 0, 0, 0, 1, 0, 1, 0, 1, 0, 0, 0, 0};
        const uint32_t inv4 = 1509949441u;  // 4^-1 mod p
#pragma unroll
        for (int r = 0; r < 3; r++) {
          uint64_t v = (uint64_t)ch[r][kIdx[lane]] * inv4 % kP;
          if (kW11[lane]) v = 11ull * v % kP;
          op.dst[k * op.dst_stride + 16 * r + lane] = to_mont((uint32_t)v);
        }
      }
    } else if (op.kind == kTrPowHead) {
      if (lane == 0) {
        uint32_t d[8];
        dtr::finalize(T, d);
        uint8_t head[64];
        for (int i = 0; i < 64; i++) head[i] = 0;
        for (int i = 0; i < 32; i++) head[i] = (uint8_t)(d[i / 4] >> (8 * (i % 4)));
        for (int i = 0; i < 8; i++) head[32 + i] = (uint8_t)((uint64_t)op.label_len >> (8 * i));
        for (uint32_t i = 0; i < op.label_len && 40 + i < 64; i++) head[40 + i] = (uint8_t)op.label[i];
        uint32_t* dst = op.dst + k * op.dst_stride;
        for (int i = 0; i < 16; i++)
          dst[i] = (uint32_t)head[4 * i] | ((uint32_t)head[4 * i + 1] << 8) |
                   ((uint32_t)head[4 * i + 2] << 16) | ((uint32_t)head[4 * i + 3] << 24);
      }
    }
    __syncwarp();
  }
  __syncwarp();
  dtr::warp_copy16(a.out + k, &T, sizeof(DevTranscript));
}
