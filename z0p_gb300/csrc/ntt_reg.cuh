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
// Waits for phase 0 of bar, giving up after about 2^31 cycles (about a
// second at full clock).
__device__ __forceinline__ bool mbar_wait(uint64_t* bar) {
  const long long t0 = clock64();
  for (;;) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], 0;\n"
        " selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(saddr(bar))
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

// Every thread waits on bar; the CTA goes on only if all of them saw the
// copies land. Otherwise the host learns of it through fault, and the CTA
// gives its copies a second bounded wait before it leaves.
__device__ __forceinline__ bool cta_wait(uint64_t* bar, unsigned int* fault) {
  const bool ok = mbar_wait(bar);
  if (__syncthreads_or(!ok)) {
    if (threadIdx.x == 0 && fault) atomicOr(fault, 1u);
    if (!ok) mbar_wait(bar);
    return false;
  }
  return true;
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

}  // namespace reg_ntt

// Pass 1: n1 = 2^L point columns i2 = c0 .. c0+7 of the input viewed as
// [n1][n2] (the tensor map's x = i2, y = i1, z = input block b / in_div),
// twisted by w^(j i) on load; writes yt[k1][i2] times the four-step twiddle.
template <int L, bool INV>
__global__ void __launch_bounds__(reg_ntt::kC << (L / 2), L == 10 ? 4 : 1)
    ntt_reg1_kernel(const __grid_constant__ CUtensorMap tmap, uint32_t* __restrict__ yt, NttArgs a) {
  using namespace reg_ntt;
  constexpr int H = L / 2;
  constexpr uint32_t R = 1u << H, n1 = 1u << L, CS = stride(L), T = kC * R;
  constexpr uint32_t BOX = n1 < 256 ? n1 : 256;  // rows per tensor copy
  extern __shared__ uint32_t sm_raw[];
  uint32_t* data = reinterpret_cast<uint32_t*>((reinterpret_cast<uintptr_t>(sm_raw) + 127) & ~uintptr_t(127));
  uint2* tw = reinterpret_cast<uint2*>(data + pass1_words(L));
  uint32_t* twist = reinterpret_cast<uint32_t*>(tw + (n1 - R));
  uint64_t* bar = reinterpret_cast<uint64_t*>(twist + n1);
  const uint32_t tid = threadIdx.x;
  const uint32_t logn2 = a.logn - L;
  const uint32_t n = 1u << a.logn;
  const uint32_t b = blockIdx.y, c0 = blockIdx.x * kC;
  const uint32_t j = b % a.twist_mod;
  if (tid == 0) mbar_init(bar);
  __syncthreads();
  if (tid == 0) {
    mbar_expect(bar, kC * n1 * 4u);
    for (uint32_t y = 0; y < n1; y += BOX) tensor_load_3d(data + y * kC, &tmap, c0, y, b / a.in_div, bar);
  }
  load_pass_a_twiddles<L>(tw, a);
  if (j)
    for (uint32_t i1 = tid; i1 < n1; i1 += T) twist[i1] = root_pow(a.tb, ((j * i1) << logn2) << a.twist_shift);
  if (!cta_wait(bar, a.tb.fault)) return;  // (also orders the tables above)
  const uint32_t c = tid & (kC - 1), l = tid / kC;
  uint32_t x[R];
#pragma unroll
  for (uint32_t r = 0; r < R; r++) {
    const uint32_t i1 = l + R * r;
    uint32_t v = data[i1 * kC + c];
    if (a.bad && v >= kP) atomicOr(a.bad, 1u);
    if (a.pre_gamma) v = mmul(v < kP ? v : 0u, gamma_pow(a.tb, (i1 << logn2) + c0 + c));
    if (j) v = mmul(v, twist[i1]);
    x[r] = v;
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
  uint32_t* dst = yt + (size_t)b * n + i2;
#pragma unroll
  for (int e = 0; e < (int)R; e++) {
    dst[(size_t)(((uint32_t)e << H) | hb) << logn2] = mmul(x[brev_c<H>(e)], w[e & 3]);
    w[e & 3] = mmul(w[e & 3], q4);
  }
}

// Pass 2: rows k1 = r0 .. r0+7 of yt, n2 = 2^L points each, one bulk copy
// per row; output k = k1 + n1 k2 (natural order), optionally times 31^k / n.
template <int L, bool INV>
__global__ void __launch_bounds__(reg_ntt::kC << (L / 2))
    ntt_reg2_kernel(const uint32_t* __restrict__ yt, uint32_t* __restrict__ out, NttArgs a) {
  using namespace reg_ntt;
  constexpr int H = L / 2;
  constexpr uint32_t R = 1u << H, n2 = 1u << L, RS = stride(L);
  extern __shared__ uint32_t sm_raw[];
  uint32_t* data = reinterpret_cast<uint32_t*>((reinterpret_cast<uintptr_t>(sm_raw) + 127) & ~uintptr_t(127));
  uint2* tw = reinterpret_cast<uint2*>(data + kC * RS);
  uint64_t* bar = reinterpret_cast<uint64_t*>(tw + (n2 - R));
  const uint32_t tid = threadIdx.x;
  const uint32_t logn1 = a.logn - L;
  const uint32_t n = 1u << a.logn;
  const uint32_t b = blockIdx.y, r0 = blockIdx.x * kC;
  if (tid == 0) mbar_init(bar);
  __syncthreads();
  if (tid == 0) {
    mbar_expect(bar, kC * n2 * 4u);
    const uint32_t* src = yt + (size_t)b * n + ((size_t)r0 << L);
    for (uint32_t rho = 0; rho < kC; rho++) bulk_load(data + rho * RS, src + ((size_t)rho << L), n2 * 4u, bar);
  }
  load_pass_a_twiddles<L>(tw, a);
  if (!cta_wait(bar, a.tb.fault)) return;
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
  uint32_t* dst = out + (size_t)b * n + r0 + rho;
  if (a.post_gamma) {
    // 31^k / n for k = r0 + rho + n1 k2, k2 = (e << H) | hb: four chains in e.
    const uint32_t k0 = r0 + rho + (hb << logn1);
    uint32_t g[4];
#pragma unroll
    for (int u = 0; u < 4; u++) g[u] = mmul(gamma_pow(a.tb, k0 + ((uint32_t)u * R << logn1)), a.ninv_m);
    const uint32_t g4 = gamma_pow(a.tb, 4u * R << logn1);
#pragma unroll
    for (int e = 0; e < (int)R; e++) {
      dst[(size_t)(((uint32_t)e << H) | hb) << logn1] = mmul(x[brev_c<H>(e)], g[e & 3]);
      g[e & 3] = mmul(g[e & 3], g4);
    }
  } else {
#pragma unroll
    for (int e = 0; e < (int)R; e++) dst[(size_t)(((uint32_t)e << H) | hb) << logn1] = x[brev_c<H>(e)];
  }
}
