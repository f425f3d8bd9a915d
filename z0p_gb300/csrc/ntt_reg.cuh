// Register-pass four-step NTT (included by kernels.cu after the shared-memory
// passes, whose NttArgs, helpers and twiddle tables it shares).
//
// Same transform as ntt_pass1_kernel / ntt_pass2_kernel (decimation in
// frequency, src/ntt.rs:116-177 values), organised around the registers:
// a half of 2^L points (L = 2H even) is two register passes of radix R = 2^H
// with a single shared-memory transpose between them.
//  * Pass A: thread (c, l) holds elements l + R r (r < R) of column c and
//    runs the H stages of distance R 2^k (k = H-1..0) in registers. Their
//    twiddles omega_{2D}^(l + R (r mod 2^k)) come from per-stage tables in
//    shared memory (stage s at offset 2^s - R), read at a per-thread base plus
//    compile-time offsets: lanes that share l read one word, so no bank
//    conflicts.
//  * Transpose: element i goes to position i + (i >> H) of its column, whose
//    stride is 4 mod 32 words: the eight columns of a warp start on distinct
//    banks, and both access patterns below touch 32 distinct banks.
//  * Pass B: thread (c, h) holds elements R h + r (r < R) and runs the H
//    stages of distance 2^k < R. Their twiddles omega_{2^(k+1)}^(r mod 2^k)
//    are compile-time constants (immediates), and the index-0 ones are 1.
//  * Pass 1 of the LDE takes its C x n1 column tile with TMA
//    (cp.async.bulk.tensor, a 3-D tensor map over the caller's input,
//    completion on an mbarrier), applies the coset twist on the way into
//    registers, and after pass B multiplies by the four-step twiddles as a
//    geometric chain and stores 32-byte row segments directly.
//  * Pass 2 takes its eight contiguous rows with cp.async.bulk, one copy per
//    row into a padded row slot, and stores eight consecutive output words
//    per lane group (natural order).
//  * The streamed kernels (schedule variant 3, halves up to 2^10) run the
//    same tiles from a resident grid, each CTA walking its tiles through two
//    buffers: the next tile's copy is in flight while the current one is
//    transformed, and the pass-A twiddles are loaded once per CTA.
// Every mbarrier wait is bounded: a CTA that gives up sets Tables::fault
// (read by the host after its next synchronisation) and returns.

namespace reg_ntt {

constexpr uint32_t kC = 8;  // columns (pass 1) or rows (pass 2) per CTA

constexpr uint32_t cpow(uint32_t b, uint64_t e) {
  uint64_t r = 1, x = b;
  while (e) {
    if (e & 1) r = r * x % kP;
    x = x * x % kP;
    e >>= 1;
  }
  return (uint32_t)r;
}

// omega_{2^(S+1)}^(+-X), canonical, with its Shoup quotient: compile-time.
template <int S, int X, bool INV>
struct Tw {
  static constexpr uint32_t root = cpow(31u, (uint64_t)(kP - 1) >> (S + 1));
  static constexpr uint32_t w = cpow(INV ? cpow(root, (2ull << S) - 1) : root, X);
  static constexpr uint32_t q = (uint32_t)(((uint64_t)w << 32) / kP);
};

// Column (row) stride in words: at least 2^L + R for the skewed layout, and
// 4 mod 32 so that eight columns start on distinct banks.
__host__ __device__ constexpr uint32_t stride(uint32_t L) {
  return (1u << L) + (1u << (L / 2)) + ((4u - (1u << (L / 2))) & 31u);
}

template <int H>
__device__ __forceinline__ constexpr int brev_c(int x) {
  int r = 0;
  for (int i = 0; i < H; i++) r |= ((x >> i) & 1) << (H - 1 - i);
  return r;
}

// Pass A: stages of distance R 2^k, k = H-1..0, on x[r] = element l + R r.
template <int H>
__device__ __forceinline__ void pass_a(uint32_t (&x)[1 << H], const uint2* tw, uint32_t l) {
  constexpr int R = 1 << H;
#pragma unroll
  for (int k = H - 1; k >= 0; k--) {
    const uint2* t = tw + ((R << k) - R) + l;
#pragma unroll
    for (int r = 0; r < R; r++) {
      if (r & (1 << k)) continue;
      const uint32_t u = x[r], v = x[r + (1 << k)];
      const uint2 w = t[R * (r & ((1 << k) - 1))];
      x[r] = fadd(u, v);
      x[r + (1 << k)] = shoup_mul(u + kP - v, w.x, w.y);
    }
  }
}

// One butterfly of pass B: pair I of the stage of distance 2^S.
template <int S, bool INV, int I, int R>
__device__ __forceinline__ void bfly_b(uint32_t (&x)[R]) {
  constexpr int D = 1 << S;
  constexpr int r = ((I >> S) << (S + 1)) | (I & (D - 1));
  constexpr int X = I & (D - 1);
  const uint32_t u = x[r], v = x[r + D];
  x[r] = fadd(u, v);
  if constexpr (X == 0)
    x[r + D] = fsub(u, v);
  else
    x[r + D] = shoup_mul(u + kP - v, Tw<S, X, INV>::w, Tw<S, X, INV>::q);
}
template <int S, bool INV, int R, int... I>
__device__ __forceinline__ void stage_b(uint32_t (&x)[R], std::integer_sequence<int, I...>) {
  (bfly_b<S, INV, I, R>(x), ...);
}
// Pass B: stages of distance 2^S, S = H-1..0, on x[r] = element R h + r.
template <int S, bool INV, int R>
__device__ __forceinline__ void pass_b(uint32_t (&x)[R]) {
  stage_b<S, INV, R>(x, std::make_integer_sequence<int, R / 2>{});
  if constexpr (S > 0) pass_b<S - 1, INV, R>(x);
}

__device__ __forceinline__ uint32_t saddr(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(uint64_t* bar) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(saddr(bar)) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(saddr(bar)), "r"(bytes)
               : "memory");
}
// Waits for the phase of bar with parity `par` (0 for its first use, 1 for
// its second, ...), giving up after about 2^31 cycles (about a second at
// full clock).
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t par = 0) {
  const long long t0 = clock64();
  for (;;) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(saddr(bar)), "r"(par)
        : "memory");
    if (ok) return true;
    if (clock64() - t0 > (1ll << 31)) return false;
  }
}
__device__ __forceinline__ void bulk_load(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          saddr(dst)),
      "l"(src), "r"(bytes), "r"(saddr(bar))
      : "memory");
}
__device__ __forceinline__ void tensor_load_3d(void* dst, const CUtensorMap* map, uint32_t x, uint32_t y,
                                               uint32_t z, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(saddr(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(saddr(bar))
      : "memory");
}

// Every thread waits on bar (phase parity par); the CTA goes on only if all
// of them saw the copies land. Otherwise the host learns of it through
// fault, and the CTA gives its copies a second bounded wait (and those of
// `other`, a prefetch in flight on another barrier, one) before it leaves.
__device__ __forceinline__ bool cta_wait(uint64_t* bar, unsigned int* fault, uint32_t par = 0,
                                         uint64_t* other = nullptr, uint32_t other_par = 0) {
  const bool ok = mbar_wait(bar, par);
  if (__syncthreads_or(!ok)) {
    if (threadIdx.x == 0 && fault) atomicOr(fault, 1u);
    if (!ok) mbar_wait(bar, par);
    if (other) mbar_wait(other, other_par);
    return false;
  }
  return true;
}
// Orders this thread's generic-proxy accesses of shared memory before the
// async-proxy (TMA / bulk copy) writes that a later barrier lets start.
__device__ __forceinline__ void fence_proxy_async() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// Pass-A stage twiddles: entry 2^s - R + x = omega_{2^(s+1)}^(+-x), s = H..L-1,
// which is the contiguous range [R - 1, 2^L - 1) of the per-context table.
template <int L>
__device__ __forceinline__ void load_pass_a_twiddles(uint2* tw, const NttArgs& a) {
  constexpr uint32_t R = 1u << (L / 2), n = 1u << L;
  const uint2* src = a.tb.stw + (a.inverse ? kStwInverse : 0u) + (R - 1);
  for (uint32_t i = threadIdx.x; i < n - R; i += blockDim.x) tw[i] = __ldg(src + i);
}

// Dynamic shared memory of the two kernels (bytes), 128 of them slack for
// aligning the TMA destination.
__host__ __device__ constexpr uint32_t pass1_words(uint32_t L) {
  return (kC << L) > kC * stride(L) ? (kC << L) : kC * stride(L);
}
__host__ __device__ constexpr size_t pass1_smem(uint32_t L) {
  return 128 + 4 * (size_t)pass1_words(L) + 8 * ((1u << L) - (1u << (L / 2))) + 4 * (1u << L) + 16;
}
__host__ __device__ constexpr size_t pass2_smem(uint32_t L) {
  return 128 + 4 * (size_t)kC * stride(L) + 8 * ((1u << L) - (1u << (L / 2))) + 16;
}
// The streamed kernels hold two tile buffers and two barriers.
__host__ __device__ constexpr size_t pass1s_smem(uint32_t L) {
  return 128 + 8 * (size_t)pass1_words(L) + 8 * ((1u << L) - (1u << (L / 2))) + 4 * (1u << L) + 16;
}
__host__ __device__ constexpr size_t pass2s_smem(uint32_t L) {
  return 128 + 8 * (size_t)kC * stride(L) + 8 * ((1u << L) - (1u << (L / 2))) + 16;
}
// Halves the streamed kernels take: two buffers fit in shared memory up to
// 2^10 points (80 KB for pass 1), not at 2^12 (266 KB).
__host__ __device__ constexpr bool streamed_ok(uint32_t L) { return L <= 10; }

}  // namespace reg_ntt

// Pass 1 on one tile: n1 = 2^L point columns i2 = c0 .. c0+7 of block b,
// whose copy (kC words per row, rows i1 = 0 .. n1-1) has landed in `data`;
// twisted by w^(j i) on load (twist[i1], filled when j != 0); writes
// yt[k1][i2] times the four-step twiddle. Ends with `data` read (the
// transpose's barriers are inside): a caller that reuses it adds a barrier.
// PLAIN: a.bad is null and a.pre_gamma is 0 (the LDE), so the per-element
// word check and scaling are compiled out.
template <int L, bool INV, bool PLAIN = false>
__device__ __forceinline__ void reg1_tile(uint32_t* data, const uint2* tw, const uint32_t* twist,
                                          uint32_t* __restrict__ yt, const NttArgs& a, uint32_t b,
                                          uint32_t c0, uint32_t j) {
  using namespace reg_ntt;
  constexpr int H = L / 2;
  constexpr uint32_t R = 1u << H, CS = stride(L);
  const uint32_t tid = threadIdx.x;
  const uint32_t logn2 = a.logn - L;
  const uint32_t n = 1u << a.logn;
  const uint32_t c = tid & (kC - 1), l = tid / kC;
  uint32_t x[R];
  if constexpr (PLAIN) {
    // Coset 0 of an LDE has no twist; the others twist every element.
    if (j) {
#pragma unroll
      for (uint32_t r = 0; r < R; r++) x[r] = mmul(data[(l + R * r) * kC + c], twist[l + R * r]);
    } else {
#pragma unroll
      for (uint32_t r = 0; r < R; r++) x[r] = data[(l + R * r) * kC + c];
    }
  } else {
#pragma unroll
    for (uint32_t r = 0; r < R; r++) {
      const uint32_t i1 = l + R * r;
      uint32_t v = data[i1 * kC + c];
      if (a.bad && v >= kP) atomicOr(a.bad, 1u);
      if (a.pre_gamma) v = mmul(v < kP ? v : 0u, gamma_pow(a.tb, (i1 << logn2) + c0 + c));
      if (j) v = mmul(v, twist[i1]);
      x[r] = v;
    }
  }
  pass_a<H>(x, tw, l);
  __syncthreads();  // the tile has been read: its space takes the skewed columns
  uint32_t* col = data + c * CS;
#pragma unroll
  for (uint32_t r = 0; r < R; r++) col[l + (R + 1) * r] = x[r];
  __syncthreads();
#pragma unroll
  for (uint32_t r = 0; r < R; r++) x[r] = col[(R + 1) * l + r];
  pass_b<H - 1, INV, (int)R>(x);
  // Output k1 = brev_L(R h + r) = (brev_H(r) << H) | brev_H(h), h = l. The
  // twiddle of (k1, i2) is w^(i2 (tw_exp(k1) + j << twist_shift)): a base
  // for brev_H(h) times q^e for e = brev_H(r).
  const uint32_t i2 = c0 + c;
  const uint32_t shift = kRootBits - a.logn;
  const uint32_t hb = brev_bits(l, H);
  // Four interleaved chains (e = 4 t + u) keep the products independent.
  const uint32_t e_base = i2 * (tw_exp(hb, shift, INV) + (j << a.twist_shift));
  const uint32_t e_q = i2 * tw_exp(R, shift, INV);
  uint32_t w[4];
#pragma unroll
  for (int u = 0; u < 4; u++) w[u] = root_pow(a.tb, e_base + (uint32_t)u * e_q);
  const uint32_t q4 = root_pow(a.tb, 4u * e_q);
  // Row k1 = (e << H) | hb at dst + k1 n2: a base for hb, then e rows of
  // 2^H n2 words apart.
  uint32_t* dst = yt + (size_t)b * n + i2 + ((size_t)hb << logn2);
  const size_t step = (size_t)1 << (H + logn2);
#pragma unroll
  for (int e = 0; e < (int)R; e++) {
    dst[(size_t)e * step] = mmul(x[brev_c<H>(e)], w[e & 3]);
    w[e & 3] = mmul(w[e & 3], q4);
  }
}

// Pass 2 on one tile: rows k1 = r0 .. r0+7 of block b of yt, n2 = 2^L
// points each, landed in `data` (row stride stride(L)); output k = k1 + n1
// k2 (natural order), optionally times 31^k / n. Same reuse rule as pass 1.
template <int L, bool INV>
__device__ __forceinline__ void reg2_tile(uint32_t* data, const uint2* tw, uint32_t* __restrict__ out,
                                          const NttArgs& a, uint32_t b, uint32_t r0) {
  using namespace reg_ntt;
  constexpr int H = L / 2;
  constexpr uint32_t R = 1u << H, RS = stride(L);
  const uint32_t tid = threadIdx.x;
  const uint32_t logn1 = a.logn - L;
  const uint32_t n = 1u << a.logn;
  const uint32_t rho = tid & (kC - 1), l = tid / kC;
  uint32_t* row = data + rho * RS;
  uint32_t x[R];
#pragma unroll
  for (uint32_t r = 0; r < R; r++) x[r] = row[l + R * r];
  pass_a<H>(x, tw, l);
  __syncthreads();
#pragma unroll
  for (uint32_t r = 0; r < R; r++) row[l + (R + 1) * r] = x[r];
  __syncthreads();
#pragma unroll
  for (uint32_t r = 0; r < R; r++) x[r] = row[(R + 1) * l + r];
  pass_b<H - 1, INV, (int)R>(x);
  const uint32_t hb = brev_bits(l, H);
  // Output k = r0 + rho + n1 k2 for k2 = (e << H) | hb: a base for hb, then e
  // steps of 2^H n1 words.
  uint32_t* dst = out + (size_t)b * n + r0 + rho + ((size_t)hb << logn1);
  const size_t step = (size_t)1 << (H + logn1);
  if (a.post_gamma) {
    // 31^k / n for k = r0 + rho + n1 k2, k2 = (e << H) | hb: four chains in e.
    const uint32_t k0 = r0 + rho + (hb << logn1);
    uint32_t g[4];
#pragma unroll
    for (int u = 0; u < 4; u++) g[u] = mmul(gamma_pow(a.tb, k0 + ((uint32_t)u * R << logn1)), a.ninv_m);
    const uint32_t g4 = gamma_pow(a.tb, 4u * R << logn1);
#pragma unroll
    for (int e = 0; e < (int)R; e++) {
      dst[(size_t)e * step] = mmul(x[brev_c<H>(e)], g[e & 3]);
      g[e & 3] = mmul(g[e & 3], g4);
    }
  } else {
#pragma unroll
    for (int e = 0; e < (int)R; e++) dst[(size_t)e * step] = x[brev_c<H>(e)];
  }
}

namespace reg_ntt {
__device__ __forceinline__ uint32_t* align128(uint32_t* p) {
  return reinterpret_cast<uint32_t*>((reinterpret_cast<uintptr_t>(p) + 127) & ~uintptr_t(127));
}
// The twist w^(j i1 n2) of pass-1 rows i1 for coset j != 0.
template <int L>
__device__ __forceinline__ void fill_twist(uint32_t* twist, const NttArgs& a, uint32_t j, uint32_t logn2) {
  for (uint32_t i1 = threadIdx.x; i1 < (1u << L); i1 += blockDim.x)
    twist[i1] = root_pow(a.tb, ((j * i1) << logn2) << a.twist_shift);
}
// Issues the tensor copies of pass-1 tile (b, c0) into dst (one thread).
template <int L>
__device__ __forceinline__ void fetch1(uint32_t* dst, const CUtensorMap* tmap, uint32_t b, uint32_t c0,
                                       const NttArgs& a, uint64_t* bar) {
  constexpr uint32_t n1 = 1u << L, BOX = n1 < 256 ? n1 : 256;  // rows per tensor copy
  mbar_expect(bar, kC * n1 * 4u);
  for (uint32_t y = 0; y < n1; y += BOX) tensor_load_3d(dst + y * kC, tmap, c0, y, b / a.in_div, bar);
}
// Issues the row copies of pass-2 tile (b, r0) into dst (one thread).
template <int L>
__device__ __forceinline__ void fetch2(uint32_t* dst, const uint32_t* yt, uint32_t b, uint32_t r0,
                                       const NttArgs& a, uint64_t* bar) {
  constexpr uint32_t n2 = 1u << L;
  mbar_expect(bar, kC * n2 * 4u);
  const uint32_t* src = yt + ((size_t)b << a.logn) + ((size_t)r0 << L);
  for (uint32_t rho = 0; rho < kC; rho++) bulk_load(dst + rho * stride(L), src + ((size_t)rho << L), n2 * 4u, bar);
}
}  // namespace reg_ntt

// Pass 1, one tile per CTA: columns c0 = blockIdx.x * 8 .. of the input
// viewed as [n1][n2] (the tensor map's x = i2, y = i1, z = input block
// b / in_div), block b = blockIdx.y.
template <int L, bool INV, bool PLAIN>
__global__ void __launch_bounds__(reg_ntt::kC << (L / 2), L == 10 ? 4 : 1)
    ntt_reg1_kernel(const __grid_constant__ CUtensorMap tmap, uint32_t* __restrict__ yt, NttArgs a) {
  pdl_wait();
  using namespace reg_ntt;
  constexpr uint32_t R = 1u << (L / 2), n1 = 1u << L;
  extern __shared__ uint32_t sm_raw[];
  uint32_t* data = align128(sm_raw);
  uint2* tw = reinterpret_cast<uint2*>(data + pass1_words(L));
  uint32_t* twist = reinterpret_cast<uint32_t*>(tw + (n1 - R));
  uint64_t* bar = reinterpret_cast<uint64_t*>(twist + n1);
  const uint32_t b = blockIdx.y, c0 = blockIdx.x * kC;
  const uint32_t j = b % a.twist_mod;
  if (threadIdx.x == 0) mbar_init(bar);
  __syncthreads();
  if (threadIdx.x == 0) fetch1<L>(data, &tmap, b, c0, a, bar);
  load_pass_a_twiddles<L>(tw, a);
  if (j) fill_twist<L>(twist, a, j, a.logn - L);
  if (!cta_wait(bar, a.tb.fault)) return;  // (also orders the tables above)
  reg1_tile<L, INV, PLAIN>(data, tw, twist, yt, a, b, c0, j);
}

// Pass 2, one tile per CTA: rows r0 = blockIdx.x * 8 .. of block b =
// blockIdx.y, one bulk copy per row.
template <int L, bool INV>
__global__ void __launch_bounds__(reg_ntt::kC << (L / 2))
    ntt_reg2_kernel(const uint32_t* __restrict__ yt, uint32_t* __restrict__ out, NttArgs a) {
  pdl_wait();
  using namespace reg_ntt;
  constexpr uint32_t R = 1u << (L / 2), n2 = 1u << L;
  extern __shared__ uint32_t sm_raw[];
  uint32_t* data = align128(sm_raw);
  uint2* tw = reinterpret_cast<uint2*>(data + kC * stride(L));
  uint64_t* bar = reinterpret_cast<uint64_t*>(tw + (n2 - R));
  const uint32_t b = blockIdx.y, r0 = blockIdx.x * kC;
  if (threadIdx.x == 0) mbar_init(bar);
  __syncthreads();
  if (threadIdx.x == 0) fetch2<L>(data, yt, b, r0, a, bar);
  load_pass_a_twiddles<L>(tw, a);
  if (!cta_wait(bar, a.tb.fault)) return;
  reg2_tile<L, INV>(data, tw, out, a, b, r0);
}

// Streamed pass 1: a resident grid whose CTAs walk the tiles t = blockIdx.x,
// blockIdx.x + gridDim.x, ... < tiles (tile t: block t / (n2/8), columns
// 8 (t mod n2/8) ..) through two tile buffers, so that the copy of a CTA's
// next tile is in flight while it transforms the current one, and the
// pass-A twiddles are loaded once per CTA rather than once per tile.
// Buffer s = k mod 2 of a CTA's k-th tile completes its barrier's phase
// k / 2, waited for with parity (k / 2) mod 2.
template <int L, bool INV>
__global__ void __launch_bounds__(reg_ntt::kC << (L / 2), L == 10 ? 2 : 4)
    ntt_reg1s_kernel(const __grid_constant__ CUtensorMap tmap, uint32_t* __restrict__ yt, NttArgs a,
                     uint32_t tiles) {
  pdl_wait();
  using namespace reg_ntt;
  constexpr uint32_t R = 1u << (L / 2), n1 = 1u << L, W = pass1_words(L);
  extern __shared__ uint32_t sm_raw[];
  uint32_t* buf = align128(sm_raw);
  uint2* tw = reinterpret_cast<uint2*>(buf + 2 * W);
  uint32_t* twist = reinterpret_cast<uint32_t*>(tw + (n1 - R));
  uint64_t* bar = reinterpret_cast<uint64_t*>(twist + n1);
  const uint32_t logn2 = a.logn - L;
  const uint32_t per_b = (1u << logn2) / kC;
  if (threadIdx.x == 0) {
    mbar_init(bar);
    mbar_init(bar + 1);
  }
  __syncthreads();
  if (threadIdx.x == 0 && blockIdx.x < tiles)
    fetch1<L>(buf, &tmap, blockIdx.x / per_b, (blockIdx.x % per_b) * kC, a, bar);
  load_pass_a_twiddles<L>(tw, a);
  uint32_t k = 0;
  for (uint32_t t = blockIdx.x; t < tiles; t += gridDim.x, k++) {
    const uint32_t s = k & 1u, tn = t + gridDim.x;
    // The other buffer was last read before the barrier that ended the
    // previous tile (and its proxy fences).
    if (threadIdx.x == 0 && tn < tiles) fetch1<L>(buf + (s ^ 1u) * W, &tmap, tn / per_b, (tn % per_b) * kC, a, bar + (s ^ 1u));
    const uint32_t b = t / per_b, c0 = (t % per_b) * kC;
    const uint32_t j = b % a.twist_mod;
    if (j) fill_twist<L>(twist, a, j, logn2);
    if (!cta_wait(bar + s, a.tb.fault, (k >> 1) & 1u, tn < tiles ? bar + (s ^ 1u) : nullptr,
                  ((k + 1) >> 1) & 1u))
      return;
    reg1_tile<L, INV>(buf + s * W, tw, twist, yt, a, b, c0, j);
    fence_proxy_async();
    __syncthreads();  // buffer s and the twist table are free
  }
}

// Streamed pass 2: the same walk over the row tiles (tile t: block
// t / (n1/8), rows 8 (t mod n1/8) ..).
template <int L, bool INV>
__global__ void __launch_bounds__(reg_ntt::kC << (L / 2), L == 10 ? 2 : 4)
    ntt_reg2s_kernel(const uint32_t* __restrict__ yt, uint32_t* __restrict__ out, NttArgs a, uint32_t tiles) {
  pdl_wait();
  using namespace reg_ntt;
  constexpr uint32_t R = 1u << (L / 2), n2 = 1u << L, W = kC * stride(L);
  extern __shared__ uint32_t sm_raw[];
  uint32_t* buf = align128(sm_raw);
  uint2* tw = reinterpret_cast<uint2*>(buf + 2 * W);
  uint64_t* bar = reinterpret_cast<uint64_t*>(tw + (n2 - R));
  const uint32_t per_b = (1u << (a.logn - L)) / kC;
  if (threadIdx.x == 0) {
    mbar_init(bar);
    mbar_init(bar + 1);
  }
  __syncthreads();
  if (threadIdx.x == 0 && blockIdx.x < tiles)
    fetch2<L>(buf, yt, blockIdx.x / per_b, (blockIdx.x % per_b) * kC, a, bar);
  load_pass_a_twiddles<L>(tw, a);
  uint32_t k = 0;
  for (uint32_t t = blockIdx.x; t < tiles; t += gridDim.x, k++) {
    const uint32_t s = k & 1u, tn = t + gridDim.x;
    if (threadIdx.x == 0 && tn < tiles) fetch2<L>(buf + (s ^ 1u) * W, yt, tn / per_b, (tn % per_b) * kC, a, bar + (s ^ 1u));
    if (!cta_wait(bar + s, a.tb.fault, (k >> 1) & 1u, tn < tiles ? bar + (s ^ 1u) : nullptr,
                  ((k + 1) >> 1) & 1u))
      return;
    reg2_tile<L, INV>(buf + s * W, tw, out, a, t / per_b, (t % per_b) * kC);
    fence_proxy_async();
    __syncthreads();
  }
}
