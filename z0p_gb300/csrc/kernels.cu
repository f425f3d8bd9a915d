// sm_103a kernels of the z0p GB300 prover.
//
// Layout conventions shared by all kernels:
//  * An LDE of blowup B = 2^logB over N = 2^logN trace rows is stored
//    coset-major: row k = B*q + j (natural order, src/air.rs:520-531) lives at
//    [j][q] = j*N + q. Coset j is the N-point NTT of the coefficients twisted
//    by (31 * omega_m^j)^i, so each coset is one contiguous, coalesced stream;
//    the next-row shift k -> k + B (src/air.rs:519) becomes q -> q + 1.
//  * FRI layer 0 is bitrev(composition) (src/fri.rs:584-586). Its quad P
//    holds rows k0 + s*m/4 (s = 0..3) with k0 = brev_{log m - 2}(P), i.e.
//    rows q0 + s*N/4 of a single coset, so a thread that owns one quad reads
//    four coalesced streams and writes its 64-byte leaf contiguously.
//  * Merkle trees are stored level-contiguous: level l of a tree with L
//    leaves starts at digest 2L - 2(L >> l); a digest is 8 little-endian
//    words, byte-identical to the reference's [u8; 32].
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>

#include <atomic>
#include <cstdint>
#include <mutex>
#include <utility>

#include "device.cuh"
#include "kernels.h"

namespace z0p {

namespace {

constexpr int kThreads = 256;

inline unsigned grid_for(uint64_t n, int threads = kThreads) {
  return (unsigned)((n + threads - 1) / threads);
}

// Programmatic dependent launch. Every kernel of this file starts with
// pdl_wait(): it returns once the stream's preceding kernel has completed and
// its writes are visible (at once for a kernel launched without the
// attribute). launch_dep launches with programmatic stream serialization, so
// the kernel is scheduled as its predecessor's CTAs exit instead of after the
// predecessor's completion has been processed: about 2 µs less between two
// dependent kernels on a GB300.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

template <typename... KArgs, typename... Args>
void launch_dep(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t st,
                Args&&... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  // A failed launch is left in the runtime's last error, which every
  // launcher reads next (cudaGetLastError), as after <<< >>>.
  (void)cudaLaunchKernelEx(&cfg, kernel, std::forward<Args>(args)...);
}

__device__ __forceinline__ uint32_t tw_exp(uint32_t e, uint32_t shift, uint32_t inverse) {
  uint32_t x = e << shift;
  return inverse ? 0u - x : x;
}

__device__ __forceinline__ void load_digest(const uint32_t* p, uint32_t d[8]) {
  uint4 a = *reinterpret_cast<const uint4*>(p);
  uint4 b = *reinterpret_cast<const uint4*>(p + 4);
  d[0] = a.x; d[1] = a.y; d[2] = a.z; d[3] = a.w;
  d[4] = b.x; d[5] = b.y; d[6] = b.z; d[7] = b.w;
}
__device__ __forceinline__ void store_digest(uint32_t* p, const uint32_t d[8]) {
  *reinterpret_cast<uint4*>(p) = make_uint4(d[0], d[1], d[2], d[3]);
  *reinterpret_cast<uint4*>(p + 4) = make_uint4(d[4], d[5], d[6], d[7]);
}

// ------------------------------------------------------------ trace gen ----
// (A_i, B_i) = M^i (a0, b0) with M = [[0,1],[1,1]] (src/air.rs:341-354).
// Lane l of a warp owns rows base + l + 32 j (j < per_lane): it jumps to its
// first row with the binary powers of M, then steps by M^32, so every store
// of the warp covers 32 consecutive rows.
__constant__ ProofConsts g_consts[kConstSlots];

struct FibMats {
  uint32_t m[32][4];  // M^(2^k), Montgomery form
};

// Coset j's constants (ZinvArgs) for proof blockIdx.y: zinv is shared by
// the group, cb is per proof.
__device__ __forceinline__ void coset_constants(const ZinvArgs& z, const Tables& tb, uint32_t j) {
  const uint32_t pk = blockIdx.y;
  if (j >= (1u << z.logB)) return;
  uint32_t xn = mmul(z.gamma_n_m, root_pow(tb, j << (kRootBits - z.logB)));
  uint32_t xn1 = fsub(xn, kR);
  if (pk == 0) {
    uint32_t inv = minv(xn1);
    z.zinv[j] = inv;
    z.zinv2[j] = mmul(inv, kR2);
  }
  if (z.cb) z.cb[((size_t)pk << z.logB) + j] = mmul(g_consts[z.slot + pk].coeff, xn1);
}

// CTAs from trace_ctas on compute the per-coset constants (when z.zinv).
__global__ void fib_trace_kernel(uint32_t* __restrict__ col_a, uint32_t* __restrict__ col_b,
                                 uint32_t n, uint32_t slot, FibMats mats,
                                 uint32_t per_lane, uint32_t trace_ctas, ZinvArgs z, Tables tb) {
  pdl_wait();
  if (blockIdx.x >= trace_ctas) {
    coset_constants(z, tb, (blockIdx.x - trace_ctas) * blockDim.x + threadIdx.x);
    return;
  }
  const uint32_t pk = blockIdx.y;  // proof of the group
  col_a += (size_t)pk * n;
  col_b += (size_t)pk * n;
  const uint32_t a0 = g_consts[slot + pk].a0, b0 = g_consts[slot + pk].b0;
  const uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const uint64_t start = (t >> 5) * 32 * per_lane + (t & 31);
  if (start >= n) return;
  // R = M^start in Montgomery form (the powers of M commute), one reduction
  // per entry of each product.
  uint32_t r00 = kR, r01 = 0, r10 = 0, r11 = kR;
  for (int k = 0; k < 32; k++) {
    if ((start >> k) & 1u) {
      const uint32_t* q = mats.m[k];
      const uint32_t n00 = mdot2(r00, q[0], r01, q[2]);
      const uint32_t n01 = mdot2(r00, q[1], r01, q[3]);
      const uint32_t n10 = mdot2(r10, q[0], r11, q[2]);
      const uint32_t n11 = mdot2(r10, q[1], r11, q[3]);
      r00 = n00; r01 = n01; r10 = n10; r11 = n11;
    }
  }
  // Montgomery R times canonical (a0, b0): canonical rows.
  uint32_t a = mdot2(r00, a0, r01, b0);
  uint32_t b = mdot2(r10, a0, r11, b0);
  const uint32_t s00 = mats.m[5][0], s01 = mats.m[5][1];
  const uint32_t s10 = mats.m[5][2], s11 = mats.m[5][3];
  for (uint32_t j = 0; j < per_lane; j++) {
    const uint64_t i = start + 32ull * j;
    if (i >= n) break;
    col_a[i] = a;
    col_b[i] = b;
    const uint32_t na = mdot2(a, s00, b, s01);
    b = mdot2(a, s10, b, s11);
    a = na;
  }
}

__global__ void fill_columns_kernel(uint32_t* cols, uint32_t n, uint32_t ncols,
                                    const uint32_t* __restrict__ values) {
  pdl_wait();
  const uint32_t pk = blockIdx.y;
  uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (uint64_t)n * ncols) return;
  cols[(uint64_t)pk * n * ncols + i] = values[(size_t)pk * ncols + i / n];
}

// ----------------------------------------------------------------- NTT ----
// Exact arithmetic: any transform order gives the reference's values
// (src/ntt.rs:116-177 is radix-2 DIT). These kernels run decimation in
// frequency with a bit-reversed read-out. Each column of 2^L values sits in
// shared memory at the skewed index i + i/32 (no bank conflicts for unit or
// power-of-two strides); its stages are done four at a time in registers, one
// 16-element group per thread per pass. L is a template parameter, so every
// shared-memory offset inside a group is a compile-time immediate: for a
// group base i0 whose bits [s_lo, s_lo + K) are zero,
// spos(i0 + (t << s_lo)) = spos(i0) + (t << s_lo) + ((t << s_lo) >> 5).
struct NttArgs {
  uint32_t logn, inverse, in_div, twist_mod, twist_shift, post_gamma, ninv_m;
  Tables tb;
  unsigned int* bad;    // see NttPlan::bad
  uint32_t pre_gamma;   // see NttPlan::pre_gamma
};

__device__ __forceinline__ uint32_t spos(uint32_t i) { return i + (i >> 5); }
// Stage-twiddle table position: one padding entry per 16 spreads the
// power-of-two strides at which a warp's threads read twiddles over the banks.
__host__ __device__ constexpr uint32_t tpos(uint32_t i) { return i + (i >> 4); }
__host__ __device__ constexpr uint32_t tw_entries(uint32_t L) {
  return L ? tpos(1u << (L - 1)) : 0u;
}
__host__ __device__ constexpr uint32_t skewed_len(uint32_t n) { return n + (n >> 5); }

// K DIF stages (distances 2^S_HI .. 2^(S_HI-K+1)) on group g of a column at
// col (skewed); tw[e] = (w^e, quotient) for the column root w of order 2^L,
// canonical with its Shoup quotient. Butterfly (u + v, (u - v) w): u - v + p
// < 2^32 is a valid Shoup operand without a prior reduction. In the last
// pass (S_LO = 0) the butterflies whose twiddle index is 0 multiply by 1,
// known at compile time, and reduce to a subtraction.
template <int L, int S_HI, int K>
__device__ __forceinline__ void dif_group_t(uint32_t* col, const uint2* tw, uint32_t g) {
  constexpr int S_LO = S_HI + 1 - K;
  const uint32_t g_lo = g & ((1u << S_LO) - 1u);
  const uint32_t i0 = g_lo | ((g >> S_LO) << (S_HI + 1));
  uint32_t* base = col + spos(i0);
  uint32_t x[1 << K];
#pragma unroll
  for (int t = 0; t < (1 << K); t++) x[t] = base[(t << S_LO) + ((t << S_LO) >> 5)];
#pragma unroll
  for (int st = K - 1; st >= 0; st--) {
    const int d = 1 << st;
    const uint32_t tshift = L - (S_LO + st) - 1;
    const uint32_t tbase = g_lo << tshift;
#pragma unroll
    for (int t = 0; t < (1 << K); t++) {
      if (t & d) continue;
      const uint32_t u = x[t], v = x[t + d];
      x[t] = fadd(u, v);
      if (S_LO == 0 && (t & (d - 1)) == 0) {
        x[t + d] = fsub(u, v);
      } else {
        const uint2 w = tw[tpos(tbase + ((uint32_t)(t & (d - 1)) << (S_LO + tshift)))];
        x[t + d] = shoup_mul(u + kP - v, w.x, w.y);
      }
    }
  }
#pragma unroll
  for (int t = 0; t < (1 << K); t++) base[(t << S_LO) + ((t << S_LO) >> 5)] = x[t];
}

template <int L, int S_HI, int KM = 4>
__device__ __forceinline__ void dif_passes_t(uint32_t* s, const uint2* tw, uint32_t ncols,
                                             uint32_t cstride) {
  constexpr int K = S_HI + 1 < KM ? S_HI + 1 : KM;
  constexpr uint32_t groups = 1u << (L - K);
  const uint32_t total = groups * ncols;
  for (uint32_t idx = threadIdx.x; idx < total; idx += blockDim.x)
    dif_group_t<L, S_HI, K>(s + (idx >> (L - K)) * cstride, tw, idx & (groups - 1u));
  __syncthreads();
  if constexpr (S_HI - K >= 0) dif_passes_t<L, S_HI - K, KM>(s, tw, ncols, cstride);
}

// KM: register group of 2^KM elements per thread and pass (16 or 32).
template <int L, int KM = 4>
__device__ __forceinline__ void smem_dif_t(uint32_t* s, const uint2* tw, uint32_t ncols,
                                           uint32_t cstride) {
  if constexpr (L > 0) dif_passes_t<L, L - 1, KM>(s, tw, ncols, cstride);
}

// Stage twiddles of a 2^L-point transform: (w^i, Shoup quotient), canonical,
// for i < 2^(L-1) (w^-1 for the inverse transform), entry i at tpos(i).
template <int L>
__device__ __forceinline__ void stage_twiddles(uint2* tw, const NttArgs& a) {
  if constexpr (L > 0) {
    if (a.tb.stw) {
      const uint2* src = a.tb.stw + (a.inverse ? kStwInverse : 0u) + ((1u << (L - 1)) - 1u);
      for (uint32_t i = threadIdx.x; i < (1u << (L - 1)); i += blockDim.x) tw[tpos(i)] = __ldg(src + i);
    } else {
      for (uint32_t i = threadIdx.x; i < (1u << (L - 1)); i += blockDim.x)
        tw[tpos(i)] = shoup_pair(from_mont(root_pow(a.tb, tw_exp(i, kRootBits - L, a.inverse))));
    }
  }
}

// Word offset of the stage-twiddle table after `words` of shared memory
// (8-byte aligned for the uint2 entries).
__host__ __device__ constexpr uint32_t tw_offset(uint32_t words) { return (words + 1u) & ~1u; }

// One transform of length 2^L per CTA (L <= 12).
template <int L>
__global__ void __launch_bounds__(512) ntt_small_kernel(const uint32_t* __restrict__ in,
                                                        uint32_t* __restrict__ out, NttArgs a) {
  pdl_wait();
  extern __shared__ uint32_t sm[];
  constexpr uint32_t n = 1u << L;
  uint32_t* s = sm;
  uint2* tw = reinterpret_cast<uint2*>(sm + tw_offset(skewed_len(n)));
  const uint32_t b = blockIdx.x;
  const uint32_t* src = in + (size_t)(b / a.in_div) * n;
  const uint32_t j = b % a.twist_mod;
  stage_twiddles<L>(tw, a);
  // twist w^(j i): a geometric chain per thread (stride blockDim)
  uint32_t tw_cur = 0, tw_step = 0;
  if (j) {
    tw_cur = root_pow(a.tb, (j * threadIdx.x) << a.twist_shift);
    tw_step = root_pow(a.tb, (j * blockDim.x) << a.twist_shift);
  }
  for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) {
    uint32_t v = src[i];
    if (a.bad && v >= kP) atomicOr(a.bad, 1u);
    if (a.pre_gamma) v = mmul(v < kP ? v : 0u, gamma_pow(a.tb, i));
    if (j) {
      v = mmul(v, tw_cur);
      tw_cur = mmul(tw_cur, tw_step);
    }
    s[spos(i)] = v;
  }
  __syncthreads();
  smem_dif_t<L>(s, tw, 1, 0);
  uint32_t* dst = out + (size_t)b * n;
  uint32_t g_cur = 0, g_step = 0;
  if (a.post_gamma) {
    g_cur = mmul(gamma_pow(a.tb, threadIdx.x), a.ninv_m);
    g_step = gamma_pow(a.tb, blockDim.x);
  }
  for (uint32_t k = threadIdx.x; k < n; k += blockDim.x) {
    uint32_t v = s[spos(brev_bits(k, L))];
    if (a.post_gamma) {
      v = mmul(v, g_cur);
      g_cur = mmul(g_cur, g_step);
    }
    dst[k] = v;
  }
}

// Column stride (words) of C skewed columns of length 2^L: congruent to 32/C
// mod 32 so the transposing store of a C-wide row hits distinct banks.
__host__ __device__ constexpr uint32_t col_stride(uint32_t L, uint32_t C) {
  return skewed_len(1u << L) + ((32u / C - (skewed_len(1u << L) & 31u)) & 31u);
}

// Four-step pass 1: for C columns i2 of x viewed as [n1][n2] (n1 = 2^L1),
// n1-point transforms over i1. The coset twist w^(j i), i = n2 i1 + i2,
// splits into a per-CTA table over i1 (applied on load) and a per-column
// factor folded into the four-step twiddle on the way out; each thread then
// writes C consecutive words of row k1 of yt (32 bytes for C = 8), with the
// twiddles w_k1(i2) a geometric chain in i2.
template <int L1, int LOGC, int KM>
__global__ void __launch_bounds__(512) ntt_pass1_kernel(const uint32_t* __restrict__ in,
                                                        uint32_t* __restrict__ yt, NttArgs a) {
  pdl_wait();
  constexpr uint32_t C = 1u << LOGC;
  constexpr uint32_t n1 = 1u << L1;
  constexpr uint32_t cstride = col_stride(L1, C);
  extern __shared__ uint32_t sm[];
  const uint32_t logn2 = a.logn - L1;
  const uint32_t n = 1u << a.logn;
  uint32_t* s = sm;
  uint2* tw = reinterpret_cast<uint2*>(sm + tw_offset(C * cstride));
  uint32_t* twist = reinterpret_cast<uint32_t*>(tw + tw_entries(L1));
  const uint32_t b = blockIdx.y;
  const uint32_t c0 = blockIdx.x * C;
  const uint32_t* src = in + (size_t)(b / a.in_div) * n;
  const uint32_t j = b % a.twist_mod;
  stage_twiddles<L1>(tw, a);
  if (j)
    for (uint32_t i1 = threadIdx.x; i1 < n1; i1 += blockDim.x)
      twist[i1] = root_pow(a.tb, ((j * i1) << logn2) << a.twist_shift);
  __syncthreads();
  for (uint32_t e = threadIdx.x; e < (n1 << LOGC); e += blockDim.x) {
    const uint32_t i1 = e >> LOGC, c = e & (C - 1);
    uint32_t v = src[(i1 << logn2) + c0 + c];
    if (a.bad && v >= kP) atomicOr(a.bad, 1u);
    if (a.pre_gamma) v = mmul(v < kP ? v : 0u, gamma_pow(a.tb, (i1 << logn2) + c0 + c));
    if (j) v = mmul(v, twist[i1]);
    s[c * cstride + spos(i1)] = v;
  }
  __syncthreads();
  smem_dif_t<L1, KM>(s, tw, C, cstride);
  uint32_t* dst = yt + (size_t)b * n;
  const uint32_t shift = kRootBits - a.logn;
  for (uint32_t k1 = threadIdx.x; k1 < n1; k1 += blockDim.x) {
    const uint32_t p = spos(brev_bits(k1, L1));
    // exponent of the twiddle for column i2: tw_exp(i2 k1) + (j i2 << twist_shift)
    const uint32_t step = tw_exp(k1, shift, a.inverse) + (j << a.twist_shift);
    uint32_t w = root_pow(a.tb, step * c0);
    const uint32_t wstep = root_pow(a.tb, step);
    uint32_t v[C];
#pragma unroll
    for (uint32_t c = 0; c < C; c++) {
      v[c] = mmul(s[c * cstride + p], w);
      w = mmul(w, wstep);
    }
    uint32_t* row = dst + ((size_t)k1 << logn2) + c0;
#pragma unroll
    for (uint32_t c = 0; c < C; c += 4)
      *reinterpret_cast<uint4*>(row + c) = make_uint4(v[c], v[c + 1], v[c + 2], v[c + 3]);
  }
}

// Four-step pass 2: for R rows k1 of yt, n2-point transforms over i2 (n2 =
// 2^L2); output k = k1 + n1 k2 (natural order). Each thread writes R
// consecutive words of out, optionally scaled by 31^k / n (a chain in k).
template <int L2, int LOGR, int KM>
__global__ void __launch_bounds__(512) ntt_pass2_kernel(const uint32_t* __restrict__ yt,
                                                        uint32_t* __restrict__ out, NttArgs a) {
  pdl_wait();
  constexpr uint32_t R = 1u << LOGR;
  constexpr uint32_t n2 = 1u << L2;
  constexpr uint32_t rstride = col_stride(L2, R);
  extern __shared__ uint32_t sm[];
  const uint32_t logn1 = a.logn - L2;
  const uint32_t n = 1u << a.logn;
  uint32_t* s = sm;
  uint2* tw = reinterpret_cast<uint2*>(sm + tw_offset(R * rstride));
  const uint32_t b = blockIdx.y;
  const uint32_t r0 = blockIdx.x * R;
  stage_twiddles<L2>(tw, a);
  const uint4* src = reinterpret_cast<const uint4*>(yt + (size_t)b * n + ((size_t)r0 << L2));
  for (uint32_t e = threadIdx.x; e < (R << L2) / 4; e += blockDim.x) {
    const uint32_t r = (4 * e) >> L2, i2 = (4 * e) & (n2 - 1);
    const uint4 v = src[e];
    uint32_t* dstrow = s + r * rstride + spos(i2);  // i2 % 4 == 0: no skew step inside
    dstrow[0] = v.x;
    dstrow[1] = v.y;
    dstrow[2] = v.z;
    dstrow[3] = v.w;
  }
  __syncthreads();
  smem_dif_t<L2, KM>(s, tw, R, rstride);
  uint32_t* dst = out + (size_t)b * n;
  for (uint32_t k2 = threadIdx.x; k2 < n2; k2 += blockDim.x) {
    const uint32_t p = spos(brev_bits(k2, L2));
    const uint32_t k0 = r0 + (k2 << logn1);
    uint32_t v[R];
    if (a.post_gamma) {
      uint32_t g = mmul(gamma_pow(a.tb, k0), a.ninv_m);
      const uint32_t gamma_m = to_mont(31u);
#pragma unroll
      for (uint32_t r = 0; r < R; r++) {
        v[r] = mmul(s[r * rstride + p], g);
        g = mmul(g, gamma_m);
      }
    } else {
#pragma unroll
      for (uint32_t r = 0; r < R; r++) v[r] = s[r * rstride + p];
    }
    uint32_t* o = dst + k0;
#pragma unroll
    for (uint32_t r = 0; r < R; r += 4)
      *reinterpret_cast<uint4*>(o + r) = make_uint4(v[r], v[r + 1], v[r + 2], v[r + 3]);
  }
}

#include "ntt_reg.cuh"

// Per coset j: 1 / (x^N - 1) with x^N = 31^N * omega_B^j (constant on the
// coset), in Montgomery form, the same value times 2^32 once more, and the
// linked-column constant C_j = coeff * (x^N - 1) (canonical).
__global__ void coset_zinv_kernel(ZinvArgs z, Tables tb) {
  pdl_wait();
  coset_constants(z, tb, blockIdx.x * blockDim.x + threadIdx.x);
}

// B at row k = B q + j of the LDE from A: A[j][q+1] + C_j / (x_k - w_last),
// given the Montgomery-form inverse of (x_k - w_last).
__device__ __forceinline__ uint32_t linked_b(const uint32_t* lde_a, uint32_t logN, uint32_t j,
                                             uint32_t q, uint32_t cbj, uint32_t inv_den_m) {
  const uint32_t N = 1u << logN;
  return fadd(__ldg(lde_a + ((size_t)j << logN) + ((q + 1u) & (N - 1u))), mmul(cbj, inv_den_m));
}

// ------------------------------------------------------------- subtrees ----
// Level-contiguous tree offset (level l at digest 2L - 2(L >> l), L leaves).
__device__ __forceinline__ uint64_t level_offset(uint64_t leaves, uint32_t level) {
  return 2 * leaves - 2 * (leaves >> level);
}

// Digests sit in shared memory at a stride of 9 words (2-way bank conflicts
// at most when a thread reads its two children).
constexpr int kTopStride = 9;

template <bool kMad = true>
__device__ __forceinline__ void hash_pair_smem(const uint32_t* pair, uint32_t* out_s,
                                               uint32_t* out_g, uint32_t* out_cap) {
  uint32_t a[8], b[8], d[8];
#pragma unroll
  for (int i = 0; i < 8; i++) { a[i] = pair[i]; b[i] = pair[kTopStride + i]; }
  blake3_node<kMad>(a, b, d);
#pragma unroll
  for (int i = 0; i < 8; i++) out_s[i] = d[i];
  store_digest(out_g, d);
  if (out_cap) store_digest(out_cap, d);
}

// Levels lsub+1..top of a tree whose CTAs have each written one root at
// level lsub (leaves >> lsub == gridDim.x; thread 0 wrote the CTA's root).
// Without a grid barrier: the CTA that arrives last (one atomic per CTA on
// `counter`, after a release fence; nobody waits) loads the roots into
// shared memory (buf: 2 * 9 * gridDim.x words) and hashes the remaining
// levels there, each node to the tree and level `top` also to `cap`. It puts
// the counter back to zero for the next launch. Every thread calls it.
template <bool kMad = true>
__device__ __forceinline__ void last_cta_levels(uint32_t* tree, uint64_t leaves, uint32_t lsub,
                                                uint32_t top, unsigned int* counter,
                                                uint32_t* cap, uint32_t* buf) {
  __shared__ int s_last;
  if (threadIdx.x == 0) {
    __threadfence();
    s_last = (atomicAdd(counter, 1u) == gridDim.x - 1);
  }
  __syncthreads();
  if (!s_last) return;
  __threadfence();
  uint64_t n = leaves >> lsub;
  const uint32_t* roots = tree + 8 * level_offset(leaves, lsub);
  for (uint64_t i = threadIdx.x; i < n; i += blockDim.x) {
    const uint4* p = reinterpret_cast<const uint4*>(roots + 8 * i);
    uint4 v0 = __ldcg(p), v1 = __ldcg(p + 1);
    uint32_t* o = buf + kTopStride * i;
    o[0] = v0.x; o[1] = v0.y; o[2] = v0.z; o[3] = v0.w;
    o[4] = v1.x; o[5] = v1.y; o[6] = v1.z; o[7] = v1.w;
  }
  uint32_t* cur = buf;
  uint32_t* nxt = buf + kTopStride * n;
  __syncthreads();
  for (uint32_t l = lsub; l < top; l++) {
    n >>= 1;
    uint32_t* next = tree + 8 * level_offset(leaves, l + 1);
    for (uint64_t i = threadIdx.x; i < n; i += blockDim.x)
      hash_pair_smem<kMad>(cur + 2 * kTopStride * i, nxt + kTopStride * i, next + 8 * i,
                     (cap && l + 1 == top) ? cap + 8 * i : nullptr);
    uint32_t* tmp = cur;
    cur = nxt;
    nxt = tmp;
    __syncthreads();
  }
  if (threadIdx.x == 0) *counter = 0u;
}

// Levels 1..min(log2(nt), top) of the subtree over one CTA's nt consecutive
// leaves (leaf first + t holds thread t's digest d), hashed in shared memory
// right where the leaves are made: each node goes to the tree and, at level
// `top`, to `cap` (as does the leaf itself when top == 0). Every thread of
// the CTA calls it; nt is a power of two no larger than the CTA, and buf
// holds 2 * nt * 9 words. With a `counter` (every CTA full, so one root per
// CTA) the last CTA to finish also hashes the levels above the roots up to
// `top` (last_cta_levels; buf then holds 2 * 9 * max(nt, gridDim.x) words).
__device__ __forceinline__ void cta_subtree(const uint32_t d[8], uint32_t* buf, uint32_t nt,
                                            uint64_t first, uint32_t* tree, uint64_t leaves,
                                            uint32_t top, uint32_t* cap, unsigned int* counter) {
  const uint32_t t = threadIdx.x;
  if (t < nt) {
    if (cap && top == 0) store_digest(cap + 8 * (first + t), d);
#pragma unroll
    for (int i = 0; i < 8; i++) buf[9 * t + i] = d[i];
  }
  uint32_t levels = 0;
  while ((2u << levels) <= nt && levels < top) levels++;
  uint32_t* cur = buf;
  uint32_t* nxt = buf + 9 * nt;
  __syncthreads();
  for (uint32_t l = 1; l <= levels; l++) {
    const uint32_t per = nt >> l;
    if (t < per) {
      uint32_t a[8], b[8], o[8];
#pragma unroll
      for (int i = 0; i < 8; i++) { a[i] = cur[18 * t + i]; b[i] = cur[18 * t + 9 + i]; }
      blake3_node(a, b, o);
#pragma unroll
      for (int i = 0; i < 8; i++) nxt[9 * t + i] = o[i];
      const uint64_t n = (first >> l) + t;
      store_digest(tree + 8 * (level_offset(leaves, l) + n), o);
      if (cap && l == top) store_digest(cap + 8 * n, o);
    }
    uint32_t* tmp = cur;
    cur = nxt;
    nxt = tmp;
    __syncthreads();
  }
  if (counter && levels < top) last_cta_levels(tree, leaves, levels, top, counter, cap, buf);
}

// --------------------------------------------------------------- Merkle ----
// Trace tree leaf L = rows 8L..8L+7 packed A||B (src/air.rs:520-531), hashed
// as one 64-byte block (src/merkle.rs:93-110). B comes from A (linked_b):
// eight (x - w_last) inverses per thread in one batch, also stored coset-major
// in tinv for the composition.
constexpr uint32_t kTraceLeafThreads = 256;
template <bool kLinked>  // B derived from A (lde_b null), decided once per launch
__global__ void __launch_bounds__(kTraceLeafThreads) air_trace_leaves_kernel(
    const uint32_t* __restrict__ lde_a, const uint32_t* __restrict__ cb, uint32_t w_last_m,
    uint32_t* __restrict__ leaves, uint32_t* __restrict__ tinv, uint32_t logN, uint32_t logB,
    uint32_t nleaves, uint32_t top, uint32_t* cap, unsigned int* counter, uint64_t tree_stride,
    uint64_t cap_stride, const uint32_t* __restrict__ lde_b, Tables tb) {
  pdl_wait();
  __shared__ uint32_t buf[2 * kTraceLeafThreads * 9];  // >= 2 * 9 * (kFuseMaxLeaves / 256) roots
  {
    const uint32_t pk = blockIdx.y;  // proof of the group
    const size_t m = (size_t)nleaves * 8;
    lde_a += pk * m;
    cb += (size_t)pk << logB;
    tinv += pk * m;
    leaves += pk * tree_stride;
    if (cap) cap += pk * cap_stride;
    if (counter) counter += pk;
  }
  const uint32_t nt = nleaves < kTraceLeafThreads ? nleaves : kTraceLeafThreads;
  const uint32_t L = blockIdx.x * kTraceLeafThreads + threadIdx.x;
  uint32_t d[8];
  if (threadIdx.x < nt) {
  const uint32_t logm = logN + logB;
  // Rows 8L..8L+7 are consecutive powers of omega_m: x_{k+1} = x_k omega_m.
  const uint32_t step = root_pow(tb, 1u << (kRootBits - logm));
  uint32_t x = mmul(to_mont(31u), root_pow(tb, (8u * L) << (kRootBits - logm)));
  uint32_t den[8];
#pragma unroll
  for (int r = 0; r < 8; r++) {
    den[r] = fsub(x, w_last_m);
    x = mmul(x, step);
  }
  batch_minv(den);
  uint32_t m[16];
#pragma unroll
  for (int r = 0; r < 8; r++) {
    uint32_t k = 8u * L + r;
    uint32_t j = k & ((1u << logB) - 1u), q = k >> logB;
    m[2 * r] = __ldg(lde_a + ((size_t)j << logN) + q);
    if constexpr (kLinked)
      m[2 * r + 1] = linked_b(lde_a, logN, j, q, __ldg(cb + j), den[r]);
    else
      m[2 * r + 1] = __ldg(lde_b + ((size_t)j << logN) + q);
    tinv[((size_t)j << logN) + q] = den[r];
  }
  blake3_leaf64(m, d);
  store_digest(leaves + 8 * (size_t)L, d);
  }
  cta_subtree(d, buf, nt, (uint64_t)blockIdx.x * kTraceLeafThreads, leaves, nleaves, top, cap,
              counter);
}

// The same leaves for trees that are not finished in the launch (more than
// kFuseMaxLeaves leaves): thread t makes leaves 2t and 2t + 1, rows 16t ..
// 16t + 15, with one batch inversion of their sixteen (x - w_last) (one
// field inversion per sixteen rows instead of eight). With 16 cosets, the
// warp's loads of one row index r read 32 consecutive q of coset r.
// kLinked: B is derived from A (lde_b is null), decided once per launch.
template <bool kLinked>
__global__ void __launch_bounds__(kTraceLeafThreads) air_trace_leaves2_kernel(
    const uint32_t* __restrict__ lde_a, const uint32_t* __restrict__ cb, uint32_t w_last_m,
    uint32_t* __restrict__ leaves, uint32_t* __restrict__ tinv, uint32_t logN, uint32_t logB,
    uint32_t nleaves, uint64_t tree_stride, const uint32_t* __restrict__ lde_b, Tables tb) {
  pdl_wait();
  {
    const uint32_t pk = blockIdx.y;  // proof of the group
    const size_t m = (size_t)nleaves * 8;
    lde_a += pk * m;
    cb += (size_t)pk << logB;
    tinv += pk * m;
    leaves += pk * tree_stride;
  }
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (2 * t >= nleaves) return;
  const uint32_t logm = logN + logB;
  // Rows 16t .. 16t+15 are consecutive powers of omega_m: x_{k+1} = x_k omega_m.
  const uint32_t step = root_pow(tb, 1u << (kRootBits - logm));
  uint32_t x = mmul(to_mont(31u), root_pow(tb, (16u * t) << (kRootBits - logm)));
  uint32_t den[16];
#pragma unroll
  for (int r = 0; r < 16; r++) {
    den[r] = fsub(x, w_last_m);
    x = mmul(x, step);
  }
  batch_minv(den);
#pragma unroll
  for (int h = 0; h < 2; h++) {
    uint32_t msg[16], d[8];
#pragma unroll
    for (int r = 0; r < 8; r++) {
      const uint32_t k = 16u * t + 8u * h + r;
      const uint32_t j = k & ((1u << logB) - 1u), q = k >> logB;
      msg[2 * r] = __ldg(lde_a + ((size_t)j << logN) + q);
      if constexpr (kLinked)
        msg[2 * r + 1] = linked_b(lde_a, logN, j, q, __ldg(cb + j), den[8 * h + r]);
      else
        msg[2 * r + 1] = __ldg(lde_b + ((size_t)j << logN) + q);
      tinv[((size_t)j << logN) + q] = den[8 * h + r];
    }
    blake3_leaf64(msg, d);
    store_digest(leaves + 8 * (2 * (size_t)t + h), d);
  }
}

// Range tree leaf k = BLAKE3(0x00 || row k) with the row = ncols LE words
// (src/range.rs:452-460, src/hash.rs:351-381). Threads walk rows in
// coset-major order so column reads coalesce; digests land at index k.
// kFused (trees of <= kFuseMaxLeaves leaves): thread u makes leaf k = u and
// the launch hashes the tree up to `top` (cta_subtree); otherwise
// consecutive threads read consecutive LDE rows of a coset.
template <bool kFused>
__global__ void __launch_bounds__(kThreads) range_trace_leaves_kernel(
    const uint32_t* __restrict__ lde, uint32_t* __restrict__ leaves, uint32_t logN, uint32_t logB,
    uint32_t ncols, uint64_t tree_stride, unsigned int* counter, uint32_t top, uint32_t* cap,
    uint64_t cap_stride) {
  pdl_wait();
  __shared__ uint32_t buf[kFused ? 2 * kThreads * kTopStride : 1];
  const uint32_t u = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t m = 1u << (logN + logB);
  lde += (size_t)blockIdx.y * ncols * m;
  leaves += blockIdx.y * tree_stride;
  if (kFused) {
    counter += blockIdx.y;
    if (cap) cap += blockIdx.y * cap_stride;
  }
  uint32_t o[8];
  if (u < m) {
    uint32_t j, q, k;
    if (kFused) {
      k = u;
      j = k & ((1u << logB) - 1u);
      q = k >> logB;
    } else {
      j = u >> logN;
      q = u & ((1u << logN) - 1u);
      k = (q << logB) | j;
    }
    const size_t at = ((size_t)j << logN) + q;
    uint32_t w[32];
#pragma unroll
    for (int c = 0; c < 32; c++) w[c] = 0u;
#pragma unroll
    for (int c = 0; c < 25; c++)
      if ((uint32_t)c < ncols) w[c] = __ldg(lde + ((size_t)c << (logN + logB)) + at);
    row_leaf_digest(w, ncols, o);
    store_digest(leaves + 8 * (size_t)k, o);
  }
  if constexpr (kFused)
    cta_subtree(o, buf, m < kThreads ? m : kThreads, (uint64_t)blockIdx.x * kThreads, leaves, m,
                top, cap, counter);
}

// A small IVC segment's commit in one CTA (src/fold.rs:430-458): both
// columns interpolated on <omega_S> with outputs times 31^i / S
// (src/ntt.rs:316-321, 353-358), each extended to the B cosets of 2^logm
// rows (src/ntt.rs:341-363, written coset-major per column like the
// two-launch path), the 8-byte A || B row leaves hashed
// (src/merkle.rs:63-80) and their tree built up to `top`, every level into
// `tree` and level `top` into `cap`. One thread per LDE row (m = S B <=
// kSegmentMaxRows); the 2 + 2B transforms of S = 2^L points share the
// shared-memory DIF of the one-CTA NTT. The columns are read where the
// caller left them (the mapped buffer) and checked as they load.
constexpr uint32_t kSegmentMaxRows = 256;
template <int L>
__global__ void __launch_bounds__(kSegmentMaxRows) fold_segment_kernel(
    const uint32_t* __restrict__ cols, unsigned int* bad, uint32_t* __restrict__ lde,
    uint32_t* __restrict__ tree, uint32_t* __restrict__ cap, uint32_t logB, uint32_t top,
    uint32_t ninv_m, Tables tb) {
  pdl_wait();
  constexpr uint32_t S = 1u << L;
  constexpr uint32_t cs = (skewed_len(S) + 1u) & ~1u;  // column stride (words)
  extern __shared__ uint32_t sm[];
  const uint32_t B = 1u << logB, logm = L + logB, m = S << logB;
  uint32_t* coef = sm;                                   // 2 columns
  uint32_t* ext = coef + 2 * cs;                         // 2B cosets
  uint2* tw_inv = reinterpret_cast<uint2*>(ext + 2 * B * cs);
  uint2* tw_fwd = tw_inv + tw_entries(L);
  uint32_t* buf = reinterpret_cast<uint32_t*>(tw_fwd + tw_entries(L));  // 2 * 9 * m words
  const uint32_t t = threadIdx.x;  // blockDim.x == m: two LDE inputs per thread
  // The columns (mapped host memory) are requested first; the twiddles and
  // each input's twist factor load while they arrive.
  uint32_t v_in = 0u;
  if (t < 2 * S) v_in = cols[t];
  NttArgs a{};
  a.tb = tb;
  a.inverse = 1;
  stage_twiddles<L>(tw_inv, a);
  a.inverse = 0;
  stage_twiddles<L>(tw_fwd, a);
  // Input e = b S + i of coset b = c B + j takes coefficient i of column c
  // times 31^i / S, twisted by omega_m^(j i).
  uint32_t fac[2];
#pragma unroll
  for (int h = 0; h < 2; h++) {
    const uint32_t e = t + (uint32_t)h * m;
    const uint32_t b = e >> L, i = e & (S - 1u), j = b & (B - 1u);
    fac[h] = mmul(gamma_pow(tb, i), ninv_m);
    if (j) fac[h] = mmul(fac[h], root_pow(tb, (j * i) << (kRootBits - logm)));
  }
  if (t < 2 * S) {
    if (v_in >= kP) {
      // Visible to the host before any word of the cap (written after the
      // barrier below), which the host may read before the launch retires.
      atomicOr_system(bad, 1u);
      __threadfence_system();
    }
    coef[(t >> L) * cs + spos(t & (S - 1u))] = v_in;
  }
  __syncthreads();
  smem_dif_t<L>(coef, tw_inv, 2, cs);
#pragma unroll
  for (int h = 0; h < 2; h++) {
    const uint32_t e = t + (uint32_t)h * m;
    const uint32_t b = e >> L, i = e & (S - 1u);
    const uint32_t c = b >> logB;
    ext[b * cs + spos(i)] = mmul(coef[c * cs + spos(brev_bits(i, L))], fac[h]);
  }
  __syncthreads();
  smem_dif_t<L>(ext, tw_fwd, 2 * B, cs);
  uint32_t d[8];
  if (t < m) {
    const uint32_t j = t & (B - 1u), q = t >> logB;  // row t = B q + j
    const uint32_t p = spos(brev_bits(q, L));
    uint32_t w[32];
#pragma unroll
    for (int k = 0; k < 32; k++) w[k] = 0u;
    w[0] = ext[j * cs + p];
    w[1] = ext[(B + j) * cs + p];
    lde[(j << L) + q] = w[0];
    lde[m + (j << L) + q] = w[1];
    row_leaf_digest(w, 2, d);
    store_digest(tree + 8 * t, d);
  }
  cta_subtree(d, buf, m, 0, tree, m, top, cap, nullptr);
}

// Merkle trees whose leaves repeat in runs (kernels.h, UniformTree): one CTA
// per tree. Each group's chain is one thread's sequence of node hashes of a
// digest with itself; the group roots then go up as an ordinary tree in
// shared memory.
constexpr uint32_t kUniformMaxGroups = 512;
__global__ void __launch_bounds__(128) uniform_trees_kernel(const UniformTree* trees) {
  pdl_wait();
  __shared__ uint32_t top[2 * kUniformMaxGroups * 8];
  const UniformTree t = trees[blockIdx.x];
  if (t.G == 0 || t.G > kUniformMaxGroups || (t.G & (t.G - 1u)) || t.logS > 31 ||
      (t.row ? (t.seed_words == 0 || t.seed_words > 25) : t.seed_words != 16))
    return;  // the launcher's caller validates; never index past the buffers
  const uint32_t L = t.logS + 1;
  for (uint32_t g = threadIdx.x; g < t.G; g += blockDim.x) {
    const uint32_t* sd = t.seeds + (size_t)g * t.seed_words;
    uint32_t d[8];
    if (!t.row) {
      uint32_t m[16];
#pragma unroll
      for (int i = 0; i < 16; i++) m[i] = sd[i];
      blake3_leaf64(m, d);
    } else {
      uint32_t w[32];
#pragma unroll
      for (int c = 0; c < 32; c++) w[c] = (uint32_t)c < t.seed_words ? sd[c] : 0u;
      row_leaf_digest(w, t.seed_words, d);
    }
    uint32_t* o = t.out + 8 * ((size_t)g * L);
    store_digest(o, d);
    for (uint32_t l = 1; l < L; l++) {
      uint32_t n[8];
      blake3_node(d, d, n);
#pragma unroll
      for (int i = 0; i < 8; i++) d[i] = n[i];
      store_digest(o + 8 * l, d);
    }
#pragma unroll
    for (int i = 0; i < 8; i++) top[8 * g + i] = d[i];
  }
  __syncthreads();
  uint32_t* dst = t.out + 8 * ((size_t)t.G * L);
  for (uint32_t g = threadIdx.x; g < t.G; g += blockDim.x) store_digest(dst + 8 * g, top + 8 * g);
  uint32_t off = 0, cnt = t.G;
  while (cnt > 1) {
    for (uint32_t i = threadIdx.x; i < cnt / 2; i += blockDim.x) {
      uint32_t a[8], b[8], n[8];
#pragma unroll
      for (int w = 0; w < 8; w++) {
        a[w] = top[8 * (off + 2 * i) + w];
        b[w] = top[8 * (off + 2 * i + 1) + w];
      }
      blake3_node(a, b, n);
#pragma unroll
      for (int w = 0; w < 8; w++) top[8 * (off + cnt + i) + w] = n[w];
      store_digest(dst + 8 * (off + cnt + i), n);
    }
    off += cnt;
    cnt >>= 1;
    __syncthreads();
  }
}

// One tree level; `cap` (may be null) receives a second copy of the level
// when it is the tree's cap level.
__global__ void merkle_level_kernel(const uint32_t* __restrict__ prev, uint32_t* __restrict__ next,
                                    uint64_t count, uint32_t* __restrict__ cap, uint64_t stride,
                                    uint64_t cap_stride) {
  pdl_wait();
  uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  prev += blockIdx.y * stride;
  next += blockIdx.y * stride;
  if (cap) cap += blockIdx.y * cap_stride;
  uint32_t l[8], r[8], d[8];
  load_digest(prev + 16 * i, l);
  load_digest(prev + 16 * i + 8, r);
  blake3_node(l, r, d);
  store_digest(next + 8 * i, d);
  if (cap) store_digest(cap + 8 * i, d);
}

// Two tree levels in one launch: thread i hashes nodes 2i and 2i+1 of level
// l+1 from nodes 4i..4i+3 of level l (two independent node hashes the
// scheduler interleaves), then their parent, node i of level l+2, without
// reading level l+1 back. `count` = nodes at level l+2; `cap` (may be null)
// receives level l+2 when it is the tree's cap level.
__global__ void merkle_level2_kernel(const uint32_t* __restrict__ prev, uint32_t* __restrict__ mid,
                                     uint32_t* __restrict__ next, uint64_t count,
                                     uint32_t* __restrict__ cap, uint64_t stride, uint64_t cap_stride) {
  pdl_wait();
  uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  prev += blockIdx.y * stride;
  mid += blockIdx.y * stride;
  next += blockIdx.y * stride;
  if (cap) cap += blockIdx.y * cap_stride;
  uint32_t a[8], b[8], c[8], e[8], d0[8], d1[8], d[8];
  load_digest(prev + 32 * i, a);
  load_digest(prev + 32 * i + 8, b);
  load_digest(prev + 32 * i + 16, c);
  load_digest(prev + 32 * i + 24, e);
  blake3_node(a, b, d0);
  blake3_node(c, e, d1);
  store_digest(mid + 16 * i, d0);
  store_digest(mid + 16 * i + 8, d1);
  blake3_node(d0, d1, d);
  store_digest(next + 8 * i, d);
  if (cap) store_digest(cap + 8 * i, d);
}

__global__ void copy_words_kernel(const uint32_t* __restrict__ src, uint32_t* __restrict__ dst,
                                  uint64_t n, uint64_t src_stride, uint64_t dst_stride) {
  pdl_wait();
  uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) dst[blockIdx.y * dst_stride + i] = src[blockIdx.y * src_stride + i];
}

// Upper levels of a tree without a grid barrier: CTA b hashes the 2T nodes
// [2T b, 2T b + 2T) of level l0 up to one node at level l0 + log2(2T) (or
// up to `top`), keeping each level in shared memory and writing it to
// global; the last CTA to finish hashes the rest (last_cta_levels).
constexpr int kTopThreads = 256;
constexpr int kTopMaxRoots = 512;  // level-l0 nodes <= 2^18, 512 per CTA

// `cap` (may be null) receives a copy of level `top`. The CTA that finishes
// the tree puts `counter` back to zero for the next launch. Its node hashes
// keep every G addition on the ALU pipe: with the multiply-add G step this
// kernel measured about 8% slower on a GB300 (24.5 -> 26.5 us a launch).
__global__ void __launch_bounds__(kTopThreads) merkle_top_kernel(uint32_t* tree, uint64_t leaves,
                                                                 uint32_t l0, uint32_t top,
                                                                 unsigned int* counter,
                                                                 uint32_t* cap, uint64_t stride,
                                                                 uint64_t cap_stride) {
  pdl_wait();
  __shared__ uint32_t sm[2][kTopMaxRoots * kTopStride];
  tree += blockIdx.y * stride;  // proof of the group: its tree, counter and cap
  counter += blockIdx.y;
  if (cap) cap += blockIdx.y * cap_stride;
  const uint32_t lsub = l0 + 9 < top ? l0 + 9 : top;  // last level done per CTA
  // level l0+1: thread t hashes children 2(base+t), 2(base+t)+1
  uint64_t cnt = leaves >> (l0 + 1);                    // nodes at level l0+1
  uint64_t per = 1ull << (lsub - l0 - 1);               // nodes per CTA at level l0+1
  uint64_t node = (uint64_t)blockIdx.x * per + threadIdx.x;
  int cur = 0;
  if (threadIdx.x < per && node < cnt) {
    const uint32_t* prev = tree + 8 * level_offset(leaves, l0);
    uint32_t d[8];
    uint32_t a[8], b[8];
    load_digest(prev + 16 * node, a);
    load_digest(prev + 16 * node + 8, b);
    blake3_node<false>(a, b, d);
    store_digest(tree + 8 * (level_offset(leaves, l0 + 1) + node), d);
    if (cap && l0 + 1 == top) store_digest(cap + 8 * node, d);
#pragma unroll
    for (int i = 0; i < 8; i++) sm[cur][kTopStride * threadIdx.x + i] = d[i];
  }
  __syncthreads();
  for (uint32_t l = l0 + 1; l < lsub; l++) {
    per >>= 1;
    if (threadIdx.x < per) {
      uint64_t n = (uint64_t)blockIdx.x * per + threadIdx.x;
      hash_pair_smem<false>(sm[cur] + 2 * kTopStride * threadIdx.x, sm[cur ^ 1] + kTopStride * threadIdx.x,
                     tree + 8 * (level_offset(leaves, l + 1) + n),
                     (cap && l + 1 == top) ? cap + 8 * n : nullptr);
    }
    cur ^= 1;
    __syncthreads();
  }
  if (lsub == top) return;
  last_cta_levels<false>(tree, leaves, lsub, top, counter, cap, &sm[0][0]);
}

// 64-byte leaves (four Ext4 values) of an in-memory FRI layer
// (src/fri.rs:1408-1414) or of any flat buffer.
// Leaf digests i < npad of `count` 64-byte leaves; i >= count repeats the
// last leaf (power-of-two padding, src/merkle.rs:350-360).
__global__ void leaf64_kernel(const uint32_t* __restrict__ flat, uint32_t* __restrict__ leaves,
                              uint64_t count, uint64_t npad, uint64_t in_stride,
                              uint64_t out_stride) {
  pdl_wait();
  uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= npad) return;
  flat += blockIdx.y * in_stride;
  leaves += blockIdx.y * out_stride;
  uint32_t m[16];
  const uint4* p = reinterpret_cast<const uint4*>(flat + 16 * (i < count ? i : count - 1));
#pragma unroll
  for (int k = 0; k < 4; k++) {
    uint4 v = p[k];
    m[4 * k] = v.x; m[4 * k + 1] = v.y; m[4 * k + 2] = v.z; m[4 * k + 3] = v.w;
  }
  uint32_t d[8];
  blake3_leaf64(m, d);
  store_digest(leaves + 8 * i, d);
}

// 0x00-prefixed 16-byte leaves for layers whose length is not a multiple of
// four (src/fri.rs:1422-1428).
__global__ void leaf16_kernel(const uint32_t* __restrict__ values, uint32_t* __restrict__ leaves,
                              uint64_t n, uint64_t in_stride, uint64_t out_stride) {
  pdl_wait();
  uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  values += blockIdx.y * in_stride;
  leaves += blockIdx.y * out_stride;
  uint32_t w[4] = {values[4 * i], values[4 * i + 1], values[4 * i + 2], values[4 * i + 3]};
  uint32_t d[8];
  blake3_prefixed_leaf<4>(w, d);
  store_digest(leaves + 8 * i, d);
}

// The four rows k0 + s m/4 of a layer-0 quad share a coset and sit at
// x0 omega_4^s: x1 = x0 omega_4, x2 = -x0, x3 = -x1 (omega_4^2 = -1), all in
// Montgomery form.
__device__ __forceinline__ void quad_points(const Tables& tb, uint32_t k0, uint32_t logm,
                                            uint32_t x[4]) {
  x[0] = mmul(to_mont(31u), root_pow(tb, k0 << (kRootBits - logm)));
  x[1] = mmul(x[0], kOmega4M);
  x[2] = fneg(x[0]);
  x[3] = fneg(x[1]);
}

// -------------------------------------------------------------- compose ----
// AIR composition (src/air.rs:847-929 == composition_at :938-962) on the four
// rows of layer-0 quad P, written bit-reversed as one 64-byte leaf and hashed.
//
// No inversion here. With T(q) = 1/(x_q - w_last) from the trace-leaf pass and
// w_last = omega_N^-1, x_{q+1} = omega_N x_q on a coset:
//   1/(x - w_last)          = T(q)
//   1/(omega_N x - w_last)  = T(q+1)        (B at the next row)
//   1/(x - 1)               = omega_N^-1 T(q-1)   (folded into alpha_2, alpha_3)
// and with B(x) = A(omega_N x) + C_j/(x - w_last) the first transition term
// (A(omega_N x) - B(x)) (x - w_last)/Z(x) is the constant -coeff, so
// alpha_0 times it is the per-proof constant kc. All arithmetic is exact, so
// the values equal the reference's term by term.
// With a.counter (small trees), thread u makes leaf P = u, so a CTA's leaves
// are consecutive and it hashes their subtree (cta_subtree); otherwise
// consecutive threads read consecutive LDE rows and leaf P is bit-reversed.
// The four composition values of layer-0 quad k0 (rows k0 + s quarter), each
// at its leaf position 4P + brev2(s); `a` already offset to its proof.
// kParams: the statement and weights come from a (one proof a launch),
// otherwise from the proof's constant slot.
template <bool kParams>
__device__ __forceinline__ void compose_quad(const AirComposeArgs& a, const Tables& tb, uint32_t k0,
                                             uint32_t logm, uint32_t (&leaf)[16]) {
  const uint32_t N = 1u << a.logN, B = 1u << a.logB, quarter = 1u << (logm - 2);
  uint32_t xs[4];
  quad_points(tb, k0, logm, xs);
#pragma unroll
  for (int s = 0; s < 4; s++) {
    const uint32_t k = k0 + (uint32_t)s * quarter;
    const uint32_t j = k & (B - 1u), q = k >> a.logB;
    const uint32_t qm = (q - 1u) & (N - 1u), qn = (q + 1u) & (N - 1u), qnn = (q + 2u) & (N - 1u);
    const size_t base = (size_t)j << a.logN;
    const uint32_t av = __ldg(a.lde_a + base + q);
    const uint32_t avn = __ldg(a.lde_a + base + qn);
    const uint32_t avnn = __ldg(a.lde_a + base + qnn);
    const uint32_t tm = __ldg(a.tinv + base + qm);
    const uint32_t t0 = __ldg(a.tinv + base + q);
    const uint32_t tn = __ldg(a.tinv + base + qn);
    const uint32_t cbj = __ldg(a.cb + j);
    // Differences that only feed a Montgomery product stay unreduced.
    const uint32_t zt = mmul(fsub_lazy(xs[s], a.w_last_m), __ldg(a.zinv + j));  // (x - w_last)/Z
    const uint32_t bv = fadd(avn, mmul(cbj, t0));
    const uint32_t bvn = fadd(avnn, mmul(cbj, tn));
    const uint32_t t2 = mmul(fsub_lazy(bvn, fadd(av, bv)), zt);
    const uint32_t a0 = kParams ? a.a0 : g_consts[a.slot].a0;
    const uint32_t b0 = kParams ? a.b0 : g_consts[a.slot].b0;
    const uint32_t b_last = kParams ? a.b_last : g_consts[a.slot].b_last;
    const uint32_t ba = mmul(fsub_lazy(av, a0), tm);
    const uint32_t bb = mmul(fsub_lazy(bv, b0), tm);
    const uint32_t bo = mmul(fsub_lazy(bv, b_last), t0);
    const int t = (s == 1) ? 2 : (s == 2) ? 1 : s;  // position 4P + brev2(s)
#pragma unroll
    for (int c = 0; c < 4; c++) {
      const uint32_t* al = kParams ? a.alpha[c] : g_consts[a.slot].alpha[c];
      const uint32_t kc = kParams ? a.kc[c] : g_consts[a.slot].kc[c];
      leaf[4 * t + c] = fadd(mdot4(t2, al[1], ba, al[2], bb, al[3], bo, al[4]), kc);
    }
  }
}

__device__ __forceinline__ void compose_for_proof(AirComposeArgs& a, uint32_t logm) {
  const uint32_t pk = blockIdx.y;  // proof of the group
  a.lde_a += (size_t)pk << logm;
  a.tinv += (size_t)pk << logm;
  a.cb += (size_t)pk << a.logB;
  a.layer0 += pk * a.layer_stride;
  a.leaves += pk * a.tree_stride;
  a.slot += pk;
  if (a.counter) a.counter += pk;
  if (a.cap) a.cap += pk * a.cap_stride;
}

__device__ __forceinline__ void store_leaf_values(const AirComposeArgs& a, uint32_t P,
                                                  const uint32_t (&leaf)[16]) {
  uint4* dst = reinterpret_cast<uint4*>(a.layer0 + 16 * (size_t)P);
#pragma unroll
  for (int t = 0; t < 4; t++)
    dst[t] = make_uint4(leaf[4 * t], leaf[4 * t + 1], leaf[4 * t + 2], leaf[4 * t + 3]);
}

template <bool kFused, bool kParams>
__global__ void __launch_bounds__(kThreads) air_compose_leaves_kernel(AirComposeArgs a, Tables tb) {
  pdl_wait();
  // >= 2 * 9 * (kFuseMaxLeaves / 256) roots when fused
  __shared__ uint32_t buf[kFused ? 2 * kThreads * kTopStride : 1];
  if (!kFused) a.counter = nullptr;
  const uint32_t logm = a.logN + a.logB;
  const uint32_t quarter = 1u << (logm - 2);
  const uint32_t u = blockIdx.x * blockDim.x + threadIdx.x;
  compose_for_proof(a, logm);
  const uint32_t nt = quarter < kThreads ? quarter : kThreads;
  uint32_t d[8];
  if (u < quarter) {
    const uint32_t N = 1u << a.logN;
    uint32_t k0, P;
    if (a.counter) {
      P = u;
      k0 = brev_bits(u, logm - 2);
    } else {
      if (a.logN >= 2) {
        uint32_t j = u >> (a.logN - 2), q0 = u & ((N >> 2) - 1u);
        k0 = (q0 << a.logB) | j;
      } else {
        k0 = u;
      }
      P = brev_bits(k0, logm - 2);
    }
    uint32_t leaf[16];
    compose_quad<kParams>(a, tb, k0, logm, leaf);
    store_leaf_values(a, P, leaf);
    blake3_leaf64(leaf, d);
    store_digest(a.leaves + 8 * (size_t)P, d);
  }
  if constexpr (kFused)
    cta_subtree(d, buf, nt, (uint64_t)blockIdx.x * kThreads, a.leaves, quarter, a.top, a.cap,
                a.counter);
}


// Range-check composition (src/range.rs:678-741 == composition_at :746-774).
__global__ void __launch_bounds__(kThreads) range_compose_leaves_kernel(RangeComposeArgs a,
                                                                        Tables tb) {
  pdl_wait();
  const uint32_t logm = a.logN + a.logB;
  const uint32_t quarter = 1u << (logm - 2);
  uint32_t u = blockIdx.x * blockDim.x + threadIdx.x;
  if (u >= quarter) return;
  {
    const uint32_t pk = blockIdx.y;  // proof of the group
    a.lde += ((size_t)pk * (a.n_bits + 1)) << logm;
    a.alphas += (size_t)pk * 4 * (a.n_bits + 2);
    a.layer0 += pk * a.layer_stride;
    a.leaves += pk * a.tree_stride;
    a.slot += pk;
  }
  const uint32_t N = 1u << a.logN, B = 1u << a.logB;
  uint32_t k0;
  if (a.logN >= 2) {
    uint32_t j = u >> (a.logN - 2), q0 = u & ((N >> 2) - 1u);
    k0 = (q0 << a.logB) | j;
  } else {
    k0 = u;
  }
  const uint32_t P = brev_bits(k0, logm - 2);
  uint32_t den[4], kk[4], xs[4];
  quad_points(tb, k0, logm, xs);
#pragma unroll
  for (int s = 0; s < 4; s++) {
    kk[s] = k0 + (uint32_t)s * quarter;
    den[s] = fsub(xs[s], kR);
  }
  batch_minv(den);
  const uint32_t nb = a.n_bits;
  uint32_t leaf[16];
#pragma unroll
  for (int s = 0; s < 4; s++) {
    uint32_t k = kk[s];
    uint32_t j = k & (B - 1u), q = k >> a.logB;
    size_t row = ((size_t)j << a.logN) + q;
    size_t colstride = (size_t)1 << logm;
    uint32_t v = __ldg(a.lde + row);
    const uint32_t zrow = j * a.r + (q & (a.r - 1u));
    uint32_t zi = __ldg(a.zinv + zrow), zi2 = __ldg(a.zinv2 + zrow);
    // Bit columns four at a time, highest first (columns past nb read as 0):
    // rec = sum bit_c 2^c by Horner, and per coordinate
    // sum_c alpha_c bit_c (bit_c - 1) as one lazy four-term dot product per
    // group (mmul(bit, bit - 1) carries 2^-32 and so does the dot product;
    // zinv2 = zinv 2^64 restores both at the end).
    uint32_t rec = 0u;
    E4 acc = {{0u, 0u, 0u, 0u}};
    const uint32_t groups = (nb + 3u) >> 2;
#pragma unroll 2
    for (uint32_t g = groups; g-- > 0;) {
      uint32_t b2[4];
      const uint32_t* al[4];
#pragma unroll
      for (int i = 3; i >= 0; i--) {
        const uint32_t c = 4u * g + (uint32_t)i;
        const uint32_t bit = c < nb ? __ldg(a.lde + (c + 1) * colstride + row) : 0u;
        rec = fadd(fadd(rec, rec), bit);
        b2[i] = mmul(bit, fsub_lazy(bit, 1u));
        al[i] = a.alphas + 4 * (1 + (c < nb ? c : nb - 1u));
      }
#pragma unroll
      for (int e = 0; e < 4; e++)
        acc.c[e] = fadd(acc.c[e], mdot4(b2[0], __ldg(al[0] + e), b2[1], __ldg(al[1] + e), b2[2],
                                        __ldg(al[2] + e), b2[3], __ldg(al[3] + e)));
    }
#pragma unroll
    for (int e = 0; e < 4; e++) acc.c[e] = mmul(acc.c[e], zi2);
    uint32_t dterm = mmul(fsub(v, rec), zi);
    uint32_t bound = mmul(fsub(v, g_consts[a.slot].value), den[s]);
    const uint32_t* ad = a.alphas;
    const uint32_t* ab = a.alphas + 4 * (1 + nb);
    const int t = (s == 1) ? 2 : (s == 2) ? 1 : s;
#pragma unroll
    for (int e = 0; e < 4; e++) {
      uint32_t x = mmul(dterm, __ldg(ad + e));
      x = fadd(x, acc.c[e]);
      x = fadd(x, mmul(bound, __ldg(ab + e)));
      leaf[4 * t + e] = x;
    }
  }
  uint4* dst = reinterpret_cast<uint4*>(a.layer0 + 16 * (size_t)P);
#pragma unroll
  for (int t = 0; t < 4; t++)
    dst[t] = make_uint4(leaf[4 * t], leaf[4 * t + 1], leaf[4 * t + 2], leaf[4 * t + 3]);
  uint32_t d[8];
  blake3_leaf64(leaf, d);
  store_digest(a.leaves + 8 * (size_t)P, d);
}

// -------------------------------------------- general two-column AIR ----
// air::prove_zk's masking (src/blind.rs:40-78) on coefficients that already
// carry the coset twist 31^k: plane c of `out` (padded words) is
//   c_k 31^k - r_k 31^k [k < n_rand] + r_(k-n) 31^k [n <= k < n + n_rand],
// zero beyond, i.e. T + (x^n - 1) R with R = r[c] (canonical, n_rand words).
__global__ void mask_pad_kernel(const uint32_t* __restrict__ coeffs, const uint32_t* __restrict__ r,
                                uint32_t* __restrict__ out, uint32_t n, uint32_t n_rand,
                                uint32_t padded, Tables tb) {
  pdl_wait();
  const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x, c = blockIdx.y;
  if (k >= padded) return;
  uint32_t v = k < n ? coeffs[(size_t)c * n + k] : 0u;
  const uint32_t g = gamma_pow(tb, k);
  if (k < n_rand) v = fsub(v, mmul(r[(size_t)c * n_rand + k], g));
  if (k >= n && k - n < n_rand) v = fadd(v, mmul(r[(size_t)c * n_rand + (k - n)], g));
  out[(size_t)c * padded + k] = v;
}

// AIR composition on two committed columns (src/air.rs:847-929 with
// cols[1] its own LDE, the prove_with_trace / prove_zk path): quad P as in
// air_compose_leaves_kernel, over an LDE of B cosets of N' = 2^logN rows whose
// next trace row is r = N' / n rows further in a coset (r = 1 unpadded).
//   1/z_trans = (x - w_last) / (x^n - 1),  x^n periodic in q with period r
//   1/(x - w_last) = T(q),  1/(x - 1) = omega_n^-1 T(q - r)  (in alpha_2, alpha_3)
__global__ void __launch_bounds__(kThreads) air_compose_general_kernel(AirComposeArgs a,
                                                                       const uint32_t* lde_b,
                                                                       uint32_t r, Tables tb) {
  pdl_wait();
  const uint32_t logm = a.logN + a.logB;
  const uint32_t quarter = 1u << (logm - 2);
  const uint32_t u = blockIdx.x * blockDim.x + threadIdx.x;
  if (u >= quarter) return;
  const uint32_t N = 1u << a.logN, B = 1u << a.logB;
  uint32_t k0 = u;
  if (a.logN >= 2) {
    const uint32_t j = u >> (a.logN - 2), q0 = u & ((N >> 2) - 1u);
    k0 = (q0 << a.logB) | j;
  }
  const uint32_t P = brev_bits(k0, logm - 2);
  uint32_t xs[4];
  quad_points(tb, k0, logm, xs);
  const ProofConsts& pc = g_consts[a.slot];
  uint32_t leaf[16];
#pragma unroll
  for (int s = 0; s < 4; s++) {
    const uint32_t k = k0 + (uint32_t)s * quarter;
    const uint32_t j = k & (B - 1u), q = k >> a.logB;
    const size_t base = (size_t)j << a.logN;
    const uint32_t qn = (q + r) & (N - 1u), qm = (q - r) & (N - 1u);
    const uint32_t av = __ldg(a.lde_a + base + q), bv = __ldg(lde_b + base + q);
    const uint32_t an = __ldg(a.lde_a + base + qn), bn = __ldg(lde_b + base + qn);
    const uint32_t tm = __ldg(a.tinv + base + qm), t0 = __ldg(a.tinv + base + q);
    const uint32_t iz = mmul(fsub_lazy(xs[s], a.w_last_m), __ldg(a.zinv + j * r + (q & (r - 1u))));
    const uint32_t t1 = mmul(fsub_lazy(an, bv), iz);
    const uint32_t t2 = mmul(fsub_lazy(bn, fadd(av, bv)), iz);
    const uint32_t ba = mmul(fsub_lazy(av, pc.a0), tm);
    const uint32_t bb = mmul(fsub_lazy(bv, pc.b0), tm);
    const uint32_t bo = mmul(fsub_lazy(bv, pc.b_last), t0);
    const int t = (s == 1) ? 2 : (s == 2) ? 1 : s;  // position 4P + brev2(s)
#pragma unroll
    for (int c = 0; c < 4; c++)
      leaf[4 * t + c] = fadd(mdot4(t1, pc.alpha[c][0], t2, pc.alpha[c][1], ba, pc.alpha[c][2], bb,
                                   pc.alpha[c][3]),
                             mmul(bo, pc.alpha[c][4]));
  }
  uint4* dst = reinterpret_cast<uint4*>(a.layer0 + 16 * (size_t)P);
#pragma unroll
  for (int t = 0; t < 4; t++)
    dst[t] = make_uint4(leaf[4 * t], leaf[4 * t + 1], leaf[4 * t + 2], leaf[4 * t + 3]);
  uint32_t d[8];
  blake3_leaf64(leaf, d);
  store_digest(a.leaves + 8 * (size_t)P, d);
}

// Table membership composition (src/table.rs:597-644 == composition_at
// :646-660) on layer-0 quads, as the AIR kernels lay them out:
//   alpha_m prod_t (v - t) / (x^n - 1) + alpha_b (v - value) / (x - 1)
// with 1/(x^n - 1) periodic in q (period r = N'/n) and 1/(x - 1) =
// omega_n^-1 T(q - r), omega_n^-1 folded into alpha_b. The product runs as a
// chain of Montgomery products of canonical factors and is brought back to
// canonical by one product with R^len.
__global__ void __launch_bounds__(kThreads) table_compose_kernel(TableComposeArgs a, Tables tb) {
  pdl_wait();
  const uint32_t logm = a.logN + a.logB;
  const uint32_t quarter = 1u << (logm - 2);
  const uint32_t u = blockIdx.x * blockDim.x + threadIdx.x;
  if (u >= quarter) return;
  const uint32_t N = 1u << a.logN, B = 1u << a.logB;
  uint32_t k0 = u;
  if (a.logN >= 2) {
    const uint32_t j = u >> (a.logN - 2), q0 = u & ((N >> 2) - 1u);
    k0 = (q0 << a.logB) | j;
  }
  const uint32_t P = brev_bits(k0, logm - 2);
  uint32_t leaf[16];
#pragma unroll
  for (int s = 0; s < 4; s++) {
    const uint32_t k = k0 + (uint32_t)s * quarter;
    const uint32_t j = k & (B - 1u), q = k >> a.logB;
    const size_t base = (size_t)j << a.logN;
    const uint32_t v = __ldg(a.lde + base + q);
    const uint32_t tm = __ldg(a.tinv + base + ((q - a.r) & (N - 1u)));
    const uint32_t iz = __ldg(a.zinv + j * a.r + (q & (a.r - 1u)));
    uint32_t prod = fsub(v, __ldg(a.table));
    for (uint32_t i = 1; i < a.table_len; i++) prod = mmul(prod, fsub(v, __ldg(a.table + i)));
    prod = mmul(mmul(prod, a.corr_m), iz);
    const uint32_t bd = mmul(fsub_lazy(v, a.value), tm);
    const int t = (s == 1) ? 2 : (s == 2) ? 1 : s;  // position 4P + brev2(s)
#pragma unroll
    for (int c = 0; c < 4; c++) leaf[4 * t + c] = mdot2(prod, a.alpha_m[c], bd, a.alpha_b[c]);
  }
  uint4* dst = reinterpret_cast<uint4*>(a.layer0 + 16 * (size_t)P);
#pragma unroll
  for (int t = 0; t < 4; t++)
    dst[t] = make_uint4(leaf[4 * t], leaf[4 * t + 1], leaf[4 * t + 2], leaf[4 * t + 3]);
  uint32_t d[8];
  blake3_leaf64(leaf, d);
  store_digest(a.leaves + 8 * (size_t)P, d);
}

// ------------------------------------------------- FRI commitment input ----
// fri::commit on coefficients (src/fri.rs:407-433, 443-460): evaluate_on_coset
// scales c_i by 31^i before the forward transform (src/ntt.rs:353-358). One
// launch per coordinate (grid y); Ext4 input is interleaved, 4 words per
// value. Values >= p raise *bad (the C boundary takes canonical elements).
__global__ void gamma_scale_kernel(const uint32_t* __restrict__ in, uint32_t* __restrict__ out,
                                   uint32_t n, uint32_t ext, unsigned int* bad, Tables tb) {
  pdl_wait();
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x, c = blockIdx.y;
  if (i >= n) return;
  const uint32_t v = in[ext ? 4 * (size_t)i + c : i];
  if (v >= kP) atomicOr(bad, 1u);
  out[(size_t)c * n + i] = mmul(v < kP ? v : 0u, gamma_pow(tb, i));
}

// FRI layer 0 of a commitment (src/fri.rs:584-586): the LDE bit-reversed as
// Ext4 values, written as 64-byte quad leaves and hashed, as in the AIR
// composition kernel (quad P holds rows k0 + s m/4, k0 = brev(P)). The LDE is
// either coset-major per coordinate (fri::commit: `coset_major`, ncomp 1 or
// 4 coordinate planes of m words) or the caller's natural-order evaluations
// (fri::commit_evals: 1 or 4 words per value, checked canonical into *bad).
struct Layer0Args {
  const uint32_t* src;
  uint32_t* layer0;
  uint32_t* leaves;
  unsigned int* bad;
  uint32_t logm, logB, ncomp, coset_major;
  unsigned int* counter;  // fused tree (kFused): zero counter, cap level and cap
  uint32_t top;
  uint32_t* cap;
};
// kFused (trees of <= kFuseMaxLeaves leaves): thread u makes leaf P = u and
// the launch hashes the tree up to `top`, as air_compose_leaves does.
template <bool kFused>
__global__ void __launch_bounds__(kThreads) layer0_leaves_kernel(Layer0Args a) {
  pdl_wait();
  __shared__ uint32_t buf[kFused ? 2 * kThreads * kTopStride : 1];
  const uint32_t quarter = 1u << (a.logm - 2);
  const uint32_t u = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t nt = quarter < kThreads ? quarter : kThreads;
  uint32_t d[8];
  if (u < quarter) {
  const uint32_t logN = a.logm - a.logB;
  uint32_t k0 = u, P;
  if (kFused) {
    P = u;
    k0 = brev_bits(u, a.logm - 2);
  } else {
    if (a.coset_major && logN >= 2) {  // consecutive threads read consecutive q
      const uint32_t j = u >> (logN - 2), q0 = u & ((1u << (logN - 2)) - 1u);
      k0 = (q0 << a.logB) | j;
    }
    P = brev_bits(k0, a.logm - 2);
  }
  const size_t m = (size_t)1 << a.logm;
  uint32_t leaf[16];
  unsigned int over = 0;
#pragma unroll
  for (int s = 0; s < 4; s++) {
    const uint32_t k = k0 + (uint32_t)s * quarter;
    const int t = (s == 1) ? 2 : (s == 2) ? 1 : s;  // position 4P + brev2(s)
    size_t idx = k;
    if (a.coset_major) idx = ((size_t)(k & ((1u << a.logB) - 1u)) << logN) + (k >> a.logB);
#pragma unroll
    for (int c = 0; c < 4; c++) {
      uint32_t v = 0u;
      if ((uint32_t)c < a.ncomp)
        v = a.coset_major ? a.src[(size_t)c * m + idx] : a.src[idx * a.ncomp + c];
      over |= v >= kP;
      leaf[4 * t + c] = v;
    }
  }
  if (over) atomicOr(a.bad, 1u);
  uint4* dst = reinterpret_cast<uint4*>(a.layer0 + 16 * (size_t)P);
#pragma unroll
  for (int t = 0; t < 4; t++)
    dst[t] = make_uint4(leaf[4 * t], leaf[4 * t + 1], leaf[4 * t + 2], leaf[4 * t + 3]);
  blake3_leaf64(leaf, d);
  store_digest(a.leaves + 8 * (size_t)P, d);
  }
  if constexpr (kFused)
    cta_subtree(d, buf, nt, (uint64_t)blockIdx.x * kThreads, a.leaves, quarter, a.top, a.cap,
                a.counter);
}

// ---------------------------------------------------------- folded IVC ----

// 1/(x_k - w_last) for rows k = 8L..8L+7 (consecutive powers of omega_m), one
// batched inversion per thread, stored coset-major at [j][q], k = B q + j.
__global__ void row_inverses_kernel(uint32_t* __restrict__ tinv, uint32_t w_last_m, uint32_t logN,
                                    uint32_t logB, Tables tb) {
  pdl_wait();
  const uint32_t logm = logN + logB;
  const uint32_t L = blockIdx.x * blockDim.x + threadIdx.x;
  if (L >= (1u << (logm - 3))) return;
  const uint32_t step = root_pow(tb, 1u << (kRootBits - logm));
  uint32_t x = mmul(to_mont(31u), root_pow(tb, (8u * L) << (kRootBits - logm)));
  uint32_t den[8];
#pragma unroll
  for (int r = 0; r < 8; r++) {
    den[r] = fsub(x, w_last_m);
    x = mmul(x, step);
  }
  batch_minv(den);
#pragma unroll
  for (int r = 0; r < 8; r++) {
    const uint32_t k = 8u * L + r;
    tinv[((size_t)(k & ((1u << logB) - 1u)) << logN) + (k >> logB)] = den[r];
  }
}

// One thread per layer-0 quad (the composition kernel's mapping): for each of
// its four rows, the six quotient terms of every segment (src/fold.rs:833-847)
// times gamma_k alpha_t, summed over the segments; then the 64-byte leaf.
//   1/z_trans = (x - w_last) / (x^s - 1)     (x^s constant on a coset)
//   1/(x - w_last) = T(q),  1/(x - 1) = omega_s^-1 T(q-1)  (folded into ga[2], ga[3])
// All arithmetic is exact, so the sum equals sum_k gamma_k C_k term by term.
// kFused (small layer 0, a.counter): thread u makes leaf P = u and the launch
// builds the layer-0 tree (cta_subtree); each thread inverts its four rows'
// x - w_last and x omega_s^-1 - w_last (= x_{q-1} - w_last on a coset) in
// one batch instead of reading T.
// The segments go by in the outer loop, their table entries staged in shared
// memory kCombineStage at a time: per segment a thread issues the sixteen
// column loads of its four rows together, so a segment costs one memory
// latency rather than four dependent pairs of them.
constexpr uint32_t kCombineStage = 32;
template <bool kFused>
__global__ void __launch_bounds__(kThreads) fold_combine_kernel(FoldCombineArgs a, Tables tb) {
  pdl_wait();
  __shared__ uint32_t buf[kFused ? 2 * kThreads * kTopStride : 1];
  __shared__ FoldStepDev stage[kCombineStage];
  static_assert(sizeof(FoldStepDev) % 4 == 0, "staged as words");
  const uint32_t logm = a.logN + a.logB;
  const uint32_t quarter = 1u << (logm - 2);
  const uint32_t u = blockIdx.x * blockDim.x + threadIdx.x;
  const bool live = u < quarter;
  const uint32_t nt = quarter < kThreads ? quarter : kThreads;
  const uint32_t N = 1u << a.logN, B = 1u << a.logB;
  uint32_t k0 = u, P = 0;
  size_t at[4] = {}, atn[4] = {};
  uint32_t tm[4] = {}, t0[4] = {}, iz[4] = {};
  if (live) {
    if (kFused) {
      P = u;
      k0 = brev_bits(u, logm - 2);
    } else {
      if (a.logN >= 2) {
        const uint32_t j = u >> (a.logN - 2), q0 = u & ((N >> 2) - 1u);
        k0 = (q0 << a.logB) | j;
      }
      P = brev_bits(k0, logm - 2);
    }
    uint32_t xs[4];
    quad_points(tb, k0, logm, xs);
    uint32_t inv[8];  // kFused: T(q) of row s at s, T(q - 1) at 4 + s
    if (kFused) {
#pragma unroll
      for (int s = 0; s < 4; s++) {
        inv[s] = fsub(xs[s], a.w_last_m);
        inv[4 + s] = fsub(mmul(xs[s], a.w_last_m), a.w_last_m);
      }
      batch_minv(inv);
    }
#pragma unroll
    for (int s = 0; s < 4; s++) {
      const uint32_t k = k0 + (uint32_t)s * quarter;
      const uint32_t j = k & (B - 1u), q = k >> a.logB;
      const size_t base = (size_t)j << a.logN;
      at[s] = base + q;
      atn[s] = base + ((q + 1u) & (N - 1u));
      tm[s] = kFused ? inv[4 + s] : __ldg(a.tinv + base + ((q - 1u) & (N - 1u)));
      t0[s] = kFused ? inv[s] : __ldg(a.tinv + at[s]);
      iz[s] = mmul(fsub_lazy(xs[s], a.w_last_m), __ldg(a.zinv + j));
    }
  }
  uint32_t acc[4][4] = {};
  for (uint32_t c0 = 0; c0 < a.nsteps; c0 += kCombineStage) {
    const uint32_t cn = a.nsteps - c0 < kCombineStage ? a.nsteps - c0 : kCombineStage;
    __syncthreads();
    const uint32_t* src = reinterpret_cast<const uint32_t*>(a.steps + c0);
    for (uint32_t i = threadIdx.x; i < cn * (uint32_t)(sizeof(FoldStepDev) / 4); i += blockDim.x)
      reinterpret_cast<uint32_t*>(stage)[i] = __ldg(src + i);
    __syncthreads();
    if (!live) continue;
    for (uint32_t st = 0; st < cn; st++) {
      const FoldStepDev& S = stage[st];
      uint32_t av[4], bv[4], an[4], bn[4];
#pragma unroll
      for (int s = 0; s < 4; s++) {
        av[s] = __ldg(S.a + at[s]);
        bv[s] = __ldg(S.b + at[s]);
        an[s] = __ldg(S.a + atn[s]);
        bn[s] = __ldg(S.b + atn[s]);
      }
#pragma unroll
      for (int s = 0; s < 4; s++) {
        const uint32_t tr1 = mmul(fsub_lazy(an[s], bv[s]), iz[s]);
        const uint32_t tr2 = mmul(fsub_lazy(bn[s], fadd(av[s], bv[s])), iz[s]);
        const uint32_t ia = mmul(fsub_lazy(av[s], S.in_a), tm[s]);
        const uint32_t ib = mmul(fsub_lazy(bv[s], S.in_b), tm[s]);
        const uint32_t oa = mmul(fsub_lazy(av[s], S.out_a), t0[s]);
        const uint32_t ob = mmul(fsub_lazy(bv[s], S.out_b), t0[s]);
#pragma unroll
        for (int c = 0; c < 4; c++) {
          const uint32_t v = fadd(mdot4(tr1, S.ga[0][c], tr2, S.ga[1][c], ia, S.ga[2][c], ib,
                                        S.ga[3][c]),
                                  mdot2(oa, S.ga[4][c], ob, S.ga[5][c]));
          acc[s][c] = fadd(acc[s][c], v);
        }
      }
    }
  }
  uint32_t d[8];
  if (live) {
    uint32_t leaf[16];
#pragma unroll
    for (int s = 0; s < 4; s++) {
      const int t = (s == 1) ? 2 : (s == 2) ? 1 : s;  // position 4P + brev2(s)
#pragma unroll
      for (int c = 0; c < 4; c++) leaf[4 * t + c] = acc[s][c];
    }
    uint4* dst = reinterpret_cast<uint4*>(a.layer0 + 16 * (size_t)P);
#pragma unroll
    for (int t = 0; t < 4; t++)
      dst[t] = make_uint4(leaf[4 * t], leaf[4 * t + 1], leaf[4 * t + 2], leaf[4 * t + 3]);
    blake3_leaf64(leaf, d);
    store_digest(a.leaves + 8 * (size_t)P, d);
  }
  if constexpr (kFused)
    cta_subtree(d, buf, nt, (uint64_t)blockIdx.x * kThreads, a.leaves, quarter, a.top, a.cap,
                a.counter);
}

// CTA (query i, step k): 4 column words, then the two capped row paths.
__global__ void __launch_bounds__(64) fold_openings_kernel(const FoldStepDev* steps,
                                                          const uint64_t* leaves, uint32_t nq,
                                                          uint32_t logN, uint32_t logB,
                                                          uint32_t path_steps, uint32_t* out,
                                                          uint32_t stride) {
  pdl_wait();
  const uint32_t qi = blockIdx.x, k = blockIdx.y;
  const FoldStepDev& S = steps[k];
  const uint32_t logm = logN + logB;
  const uint64_t m = 1ull << logm;
  const uint64_t index = brev_bits((uint32_t)leaves[qi], logm);
  const uint64_t shifted = (index + (1ull << logB)) & (m - 1);
  uint32_t* o = out + ((size_t)k * nq + qi) * stride;
  for (uint32_t t = threadIdx.x; t < 4 + 16 * path_steps; t += blockDim.x) {
    if (t < 4) {
      const uint64_t idx = t < 2 ? index : shifted;
      const size_t at = ((size_t)(idx & ((1u << logB) - 1u)) << logN) + (idx >> logB);
      o[t] = (t & 1u) ? S.b[at] : S.a[at];
    } else {
      const uint32_t h = (t - 4) / (8 * path_steps), r = (t - 4) % (8 * path_steps);
      const uint32_t lv = r >> 3, w = r & 7u;
      const uint64_t sib = ((h ? shifted : index) >> lv) ^ 1ull;
      o[t] = S.tree[8 * (2 * m - 2 * (m >> lv) + sib) + w];
    }
  }
}

// ---------------------------------------------------------------- gates ----
// A launch queued before the host has written its inputs waits here: thread 0
// polls the device-mapped gate word until it holds `epoch` (acquire at system
// scope, so the inputs the host wrote before it are visible), at most about
// 2^31 cycles, after which it sets bit 3 of *fault and the CTA runs on.
__device__ __noinline__ void wait_gate(const unsigned int* go, unsigned int epoch,
                                       unsigned int* fault) {
  if (threadIdx.x == 0) {
    const long long t0 = clock64();
    for (;;) {
      unsigned int v;
      asm volatile("ld.acquire.sys.global.u32 %0, [%1];" : "=r"(v) : "l"(go) : "memory");
      if (v == epoch) break;
      if (clock64() - t0 > (1ll << 31)) {
        if (fault) atomicOr(fault, 8u);
        break;
      }
      __nanosleep(64);
    }
  }
  __syncthreads();
}

// ----------------------------------------------------------------- FRI ----
// fold_values (src/fri.rs:1311-1331): A + x^-1 (r0 B + x^-1 (r1 C + x^-1 r2 D))
// with B, C, D the quarter-scaled differences; the 1/4 is folded into the
// challenge tables (r_k / 4), so only the mean is halved twice here.
using FoldTab = uint32_t[3][4][4];
__device__ __forceinline__ E4 fold_quad(const E4& q0, const E4& q1, const E4& q2, const E4& q3,
                                        uint32_t xinv_m, const FoldArgs& a, const FoldTab& tab) {
  E4 s01 = e4_add(q0, q1), s23 = e4_add(q2, q3);
  E4 odd_diff = e4_sub(q0, q1);
  E4 skew_u = e4_mul_base(e4_sub_lazy(q2, q3), a.unit_m);
  E4 mean = e4_quarter(e4_add(s01, s23));
  E4 odd4 = e4_sub(odd_diff, skew_u);
  E4 even4 = e4_sub(s01, s23);
  E4 skew4 = e4_add(odd_diff, skew_u);
  // The Horner sums only feed the next product by x^-1: left unreduced.
  E4 acc = e4_add_lazy(e4_mul_base(e4_mul_tab(skew4, tab[2]), xinv_m),
                       e4_mul_tab(even4, tab[1]));
  acc = e4_add_lazy(e4_mul_base(acc, xinv_m), e4_mul_tab(odd4, tab[0]));
  return e4_add(mean, e4_mul_base(acc, xinv_m));
}

// x^-1 of quad P's leader on a layer of length 2^logn: the layer domain is
// 31^(4^depth) <omega_n> in bit-reversed order (src/fri.rs:1108-1115), so no
// field inversion is needed.
__device__ __forceinline__ uint32_t quad_xinv(const Tables& tb, const FoldArgs& a, uint32_t P) {
  uint32_t e = brev_bits(P, a.logn - 2);
  return mmul(a.ginv_m, root_pow(tb, 0u - (e << (kRootBits - a.logn))));
}

// Thread per next-layer leaf: folds four quads (256 contiguous input bytes,
// staged through shared memory), writes the 64-byte next leaf and its digest.
constexpr int kFoldThreads = 128;
__device__ __forceinline__ void fold_for_proof(FoldArgs& a) {
  const uint32_t pk = blockIdx.y;  // proof of the group
  a.in += pk * a.in_stride;
  a.out += pk * a.out_stride;
  a.leaves += pk * a.tree_stride;
  if (a.cap) a.cap += pk * a.cap_stride;
  if (a.counter) a.counter += pk;
  if (a.final_vals) a.final_vals += pk * a.final_stride;
  if (a.tab) a.tab += pk * kFoldTabWords;
  a.slot += pk;
}

// A small fold's challenge tables, staged once per CTA from a.tab (every
// thread reads all of them), after the fold's gate when it has one; the
// tables are read past the L1.
__device__ __forceinline__ void stage_fold_tab(const FoldArgs& a, const Tables& tb, FoldTab& t) {
  if (a.go) wait_gate(a.go, a.go_epoch, tb.fault);
  const volatile uint32_t* src = a.tab;
  for (uint32_t i = threadIdx.x; i < kFoldTabWords; i += blockDim.x) (&t[0][0][0])[i] = src[i];
  __syncthreads();
}

// Large layers (and folds that stop at their CTAs' subtrees): the tables are
// constant-bank operands of the products.
// kWide: the input (and its per-proof stride) is 32-byte aligned, and each
// thread reads its 256 bytes as eight 32-byte loads.
template <bool kWide>
__global__ void __launch_bounds__(kFoldThreads) fri_fold_leaf_kernel(FoldArgs a, Tables tb) {
  pdl_wait();
  __shared__ uint32_t sm[2 * kTopStride * kFoldThreads];  // the CTA's subtree levels
  fold_for_proof(a);
  a.counter = nullptr;
  const uint64_t nleaf = 1ull << (a.logn - 4);
  const uint64_t first = (uint64_t)blockIdx.x * kFoldThreads;
  const uint32_t avail = nleaf < (uint64_t)kFoldThreads ? (uint32_t)nleaf : (uint32_t)kFoldThreads;
  uint64_t Pn = first + threadIdx.x;
  uint32_t d[8];
  if (threadIdx.x < avail) {
  // The thread's 256 input bytes are contiguous. With kWide, eight 32-byte
  // loads: every lane of a warp load takes a whole sector (a 16-byte load
  // leaves half of each sector to the next load, which finds it evicted from
  // L1 often enough to read it again from L2).
  const uint32_t* src = a.in + Pn * 64;
  uint32_t leaf[16];
#pragma unroll
  for (int t = 0; t < 4; t++) {
    E4 q[4];
#pragma unroll
    for (int i = 0; i < 4; i += 2) {
      if constexpr (kWide) {
        asm volatile(
            "ld.global.nc.L1::no_allocate.v8.u32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
            : "=r"(q[i].c[0]), "=r"(q[i].c[1]), "=r"(q[i].c[2]), "=r"(q[i].c[3]),
              "=r"(q[i + 1].c[0]), "=r"(q[i + 1].c[1]), "=r"(q[i + 1].c[2]), "=r"(q[i + 1].c[3])
            : "l"(src + 16 * t + 4 * i));
      } else {
#pragma unroll
        for (int u = 0; u < 2; u++) {
          const uint4 v = __ldcs(reinterpret_cast<const uint4*>(src + 16 * t + 4 * (i + u)));
          q[i + u].c[0] = v.x; q[i + u].c[1] = v.y; q[i + u].c[2] = v.z; q[i + u].c[3] = v.w;
        }
      }
    }
    uint32_t P = (uint32_t)(4 * Pn + t);
    E4 r = fold_quad(q[0], q[1], q[2], q[3], quad_xinv(tb, a, P), a, g_consts[a.slot].tab);
#pragma unroll
    for (int c = 0; c < 4; c++) leaf[4 * t + c] = r.c[c];
  }
  uint4* dst = reinterpret_cast<uint4*>(a.out + 16 * Pn);
#pragma unroll
  for (int t = 0; t < 4; t++)
    dst[t] = make_uint4(leaf[4 * t], leaf[4 * t + 1], leaf[4 * t + 2], leaf[4 * t + 3]);
  if (a.final_vals) {
    uint4* fin = reinterpret_cast<uint4*>(a.final_vals + 16 * Pn);
#pragma unroll
    for (int t = 0; t < 4; t++)
      fin[t] = make_uint4(leaf[4 * t], leaf[4 * t + 1], leaf[4 * t + 2], leaf[4 * t + 3]);
  }
  blake3_leaf64(leaf, d);
  store_digest(a.leaves + 8 * Pn, d);
  }
  cta_subtree(d, sm, avail, first, a.leaves, nleaf, a.top, a.cap, a.counter);
}

// The small-layer fold (trees of at most kFuseMaxLeaves leaves, latency-
// bound launches of a few CTAs), which also finishes the tree in its last
// CTA: four threads per next leaf, one quad each, so a thread waits on one
// fold's loads and products instead of four; the leaf's four values meet in
// its first lane by warp shuffles, which hashes the leaf. 128 leaves per CTA,
// so each CTA hashes a subtree of 128 leaves.
constexpr int kFold4Threads = 4 * kFoldThreads;
__global__ void __launch_bounds__(kFold4Threads) fri_fold_quad_kernel(FoldArgs a, Tables tb) {
  pdl_wait();
  __shared__ uint32_t sm[2 * kTopStride * (kFuseMaxLeaves / kFoldThreads)];
  __shared__ FoldTab tab;
  fold_for_proof(a);
  stage_fold_tab(a, tb, tab);
  const uint64_t nleaf = 1ull << (a.logn - 4);
  const uint64_t first = (uint64_t)blockIdx.x * kFoldThreads;
  const uint32_t avail = nleaf < (uint64_t)kFoldThreads ? (uint32_t)nleaf : (uint32_t)kFoldThreads;
  const uint32_t tl = threadIdx.x >> 2, tq = threadIdx.x & 3u;  // leaf in the CTA, its quad
  const uint64_t Pn = first + tl;
  uint32_t r[4] = {0u, 0u, 0u, 0u};
  if (tl < avail) {
    const uint4* src = reinterpret_cast<const uint4*>(a.in) + Pn * 16 + 4 * tq;
    E4 q[4];
#pragma unroll
    for (int i = 0; i < 4; i++) {
      uint4 v = __ldcs(src + i);
      q[i].c[0] = v.x; q[i].c[1] = v.y; q[i].c[2] = v.z; q[i].c[3] = v.w;
    }
    const E4 f = fold_quad(q[0], q[1], q[2], q[3], quad_xinv(tb, a, (uint32_t)(4 * Pn + tq)), a, tab);
#pragma unroll
    for (int c = 0; c < 4; c++) r[c] = f.c[c];
    const uint4 o = make_uint4(r[0], r[1], r[2], r[3]);
    reinterpret_cast<uint4*>(a.out + 16 * Pn)[tq] = o;
    if (a.final_vals) reinterpret_cast<uint4*>(a.final_vals + 16 * Pn)[tq] = o;
  }
  // Lanes 4 tl .. 4 tl + 3 of a warp hold leaf tl's four values.
  const uint32_t lane = threadIdx.x & 31u;
  uint32_t leaf[16];
#pragma unroll
  for (int s2 = 0; s2 < 4; s2++)
#pragma unroll
    for (int c = 0; c < 4; c++) leaf[4 * s2 + c] = __shfl_sync(0xffffffffu, r[c], (lane & ~3u) | s2);
  if (tl < avail && tq == 0) {
    uint32_t d[8];
    blake3_leaf64(leaf, d);
    store_digest(a.leaves + 8 * Pn, d);
#pragma unroll
    for (int i = 0; i < 8; i++) sm[kTopStride * tl + i] = d[i];
  }
  __syncthreads();
  uint32_t d[8];
#pragma unroll
  for (int i = 0; i < 8; i++) d[i] = threadIdx.x < avail ? sm[kTopStride * threadIdx.x + i] : 0u;
  __syncthreads();
  cta_subtree(d, sm, avail, first, a.leaves, nleaf, a.top, a.cap, a.counter);
}

// Thread per next-layer value (small layers; leaves hashed separately).
__global__ void fri_fold_plain_kernel(FoldArgs a, Tables tb) {
  pdl_wait();
  __shared__ FoldTab tab;
  fold_for_proof(a);
  stage_fold_tab(a, tb, tab);
  uint32_t P = blockIdx.x * blockDim.x + threadIdx.x;
  if (P >= (1u << (a.logn - 2))) return;
  E4 q[4];
#pragma unroll
  for (int i = 0; i < 4; i++) {
    uint4 v = reinterpret_cast<const uint4*>(a.in)[4 * P + i];
    q[i].c[0] = v.x; q[i].c[1] = v.y; q[i].c[2] = v.z; q[i].c[3] = v.w;
  }
  E4 r = fold_quad(q[0], q[1], q[2], q[3], quad_xinv(tb, a, P), a, tab);
  reinterpret_cast<uint4*>(a.out)[P] = make_uint4(r.c[0], r.c[1], r.c[2], r.c[3]);
  if (a.final_vals)
    reinterpret_cast<uint4*>(a.final_vals)[P] = make_uint4(r.c[0], r.c[1], r.c[2], r.c[3]);
}

// ------------------------------------------------------------------ PoW ----
// Transcript::grind (src/transcript.rs:206-228): smallest nonce n with
// BLAKE3(head || LE64(n)) having >= bits leading zero bits (MSB first). CTAs
// take nonce chunks in increasing order from a counter and stop once a chunk
// starts above the best nonce found: every chunk below the final minimum was
// taken and finished, so the result equals the sequential scan. The chunk
// counter is capped (max_chunks), after which the kernel sets status and
// returns instead of spinning.
constexpr int kGrindThreads = 256;
constexpr int kGrindPerThread = 4;
constexpr uint64_t kGrindChunk = (uint64_t)kGrindThreads * kGrindPerThread;

// state: [0] best nonce, [1] next chunk, [2] status (1 = chunk cap reached),
// [3] CTAs finished. The last CTA to finish copies {best, status} to `out`
// and puts the state back to {~0, 0, 0, 0} for the next launch.
struct GrindArgs {
  const uint32_t* head;  // proof k's head at head + k * kPowHeadWords
  const unsigned int* go;  // optional gate (wait_gate) before the head is read
  unsigned int go_epoch;
  unsigned int* fault;
  uint32_t bits;
  unsigned long long* state;
  unsigned long long* out;
  unsigned long long max_chunks;
};

__device__ __forceinline__ void grind_finish(const GrindArgs& a) {
  if (threadIdx.x != 0) return;
  __threadfence();
  if (atomicAdd(a.state + 3, 1ull) != gridDim.x - 1) return;
  __threadfence();
  // The cap flag first: the host may read the nonce word as soon as it
  // lands, and the flag with it.
  a.out[1] = atomicAdd(a.state + 2, 0ull);
  __threadfence_system();
  a.out[0] = atomicAdd(a.state + 0, 0ull);
  a.state[0] = ~0ull;
  a.state[1] = 0ull;
  a.state[2] = 0ull;
  a.state[3] = 0ull;
  __threadfence();
}

// The preimage is head (47 bytes) || LE64(nonce): one 55-byte block.
constexpr uint32_t kPowHeadLen = 47;

__global__ void __launch_bounds__(kGrindThreads) grind_kernel(GrindArgs a) {
  pdl_wait();
  a.head += kPowHeadWords * blockIdx.y;  // proof of the group: its head, search state and result
  a.state += 4 * blockIdx.y;
  a.out += 2 * blockIdx.y;
  constexpr int W = kPowHeadLen / 4, SH = (kPowHeadLen % 4) * 8;
  static_assert(kPowHeadLen + 8 <= 64 && SH != 0, "head and nonce must fit one block");
  __shared__ unsigned long long s_chunk;
  __shared__ int s_stop;
  __shared__ uint32_t s_head[W + 1];
  if (a.go) wait_gate(a.go, a.go_epoch, a.fault);
  if (threadIdx.x <= (unsigned)W)
    s_head[threadIdx.x] = reinterpret_cast<const volatile uint32_t*>(a.head)[threadIdx.x];
  __syncthreads();
  uint32_t head[W + 1];  // the head's words, kept in registers for every attempt
#pragma unroll
  for (int i = 0; i <= W; i++) head[i] = s_head[i];
  const volatile unsigned long long* best_p = a.state;
  for (;;) {
    if (threadIdx.x == 0) {
      unsigned long long c = atomicAdd(a.state + 1, 1ull);
      s_chunk = c;
      unsigned long long best = *best_p;
      s_stop = (c >= a.max_chunks) ? 2 : (c * kGrindChunk > best ? 1 : 0);
      if (s_stop == 2) atomicOr(a.state + 2, 1ull);
    }
    __syncthreads();
    unsigned long long c = s_chunk;
    int stop = s_stop;
    __syncthreads();
    if (stop) {
      grind_finish(a);
      return;
    }
    // Nonces above the best hit so far cannot be the minimum: a thread
    // leaves the chunk once its next nonce passes the best it last read.
    unsigned long long best = ~0ull;
#pragma unroll 1
    for (int k = 0; k < kGrindPerThread; k++) {
      unsigned long long nonce = c * kGrindChunk + (unsigned long long)k * kGrindThreads + threadIdx.x;
      if (nonce > best) break;
      best = *best_p;
      const uint32_t lo = (uint32_t)nonce, hi = (uint32_t)(nonce >> 32);
      uint32_t m[16];
#pragma unroll
      for (int i = 0; i < 16; i++) m[i] = i < W ? head[i] : 0u;
      m[W] = head[W] | (lo << SH);
      m[W + 1] = (lo >> (32 - SH)) | (hi << SH);
      m[W + 2] = hi >> (32 - SH);
      uint32_t cv[8], o[8];
      iv_words(cv);
      blake3_compress(cv, m, 0u, 0u, kPowHeadLen + 8u, kChunkStart | kChunkEnd | kRoot, o);
      uint32_t lz = __clz(__byte_perm(o[0], 0, 0x0123));
      if (lz >= a.bits) atomicMin(a.state, nonce);
    }
  }
}

// Coset-major [c][j][q] -> natural [c][k], k = B q + j (for callers that
// want reed_solomon_extend's natural order, src/ntt.rs:436-439).
// Coset-major [j][q] to natural k = B q + j: per column a transpose of the
// B x n matrix, through shared memory in tiles of up to 32 cosets x 64 rows,
// so the loads read 256 contiguous bytes per coset and the stores write
// 64 B contiguous words (B <= 32) or 128-byte runs.
constexpr uint32_t kNatTileQ = 64;
__global__ void __launch_bounds__(256) coset_to_natural_kernel(const uint32_t* __restrict__ in,
                                                               uint32_t* __restrict__ out,
                                                               uint32_t logN, uint32_t logB) {
  pdl_wait();
  __shared__ uint32_t tile[32][kNatTileQ + 1];
  const uint64_t n = 1ull << logN, m = n << logB;
  const uint64_t q0 = (uint64_t)blockIdx.x * kNatTileQ, j0 = (uint64_t)blockIdx.y * 32;
  const uint32_t ltj = logB < 5 ? logB : 5, tj = 1u << ltj;  // B - j0 >= 32 whenever B > 32
  const uint32_t tq = (uint32_t)(n - q0 < kNatTileQ ? n - q0 : kNatTileQ);
  in += (uint64_t)blockIdx.z * m;
  out += (uint64_t)blockIdx.z * m;
  for (uint32_t i = threadIdx.x; i < tj * kNatTileQ; i += blockDim.x) {
    const uint32_t jj = i / kNatTileQ, qq = i % kNatTileQ;
    if (qq < tq) tile[jj][qq] = in[((j0 + jj) << logN) + q0 + qq];
  }
  __syncthreads();
  for (uint32_t i = threadIdx.x; i < tj * kNatTileQ; i += blockDim.x) {
    const uint32_t qq = i >> ltj, jj = i & (tj - 1u);
    if (qq < tq) out[((q0 + qq) << logB) + j0 + jj] = tile[jj][qq];
  }
}

// ------------------------------------------------------- hash ceiling ----
// Throughput reference for the hashing stages: each thread chains `iters`
// Merkle-node hashes (two compressions each) in registers, so the kernel is
// bound by the BLAKE3 arithmetic alone, with no memory traffic.
__global__ void __launch_bounds__(256) hash_ceiling_kernel(const uint32_t* __restrict__ in,
                                                           uint32_t* __restrict__ out, int iters) {
  pdl_wait();
  const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  uint32_t l[8], r[8];
  load_digest(in + 16 * t, l);
  load_digest(in + 16 * t + 8, r);
#pragma unroll 1
  for (int it = 0; it < iters; it++) {
    uint32_t o[8];
    blake3_node(l, r, o);
#pragma unroll
    for (int i = 0; i < 8; i++) { l[i] = r[i]; r[i] = o[i]; }
  }
  store_digest(out + 8 * t, r);
}

// ------------------------------------------------------------- openings ----
// Every opened value and Merkle path of one proof, gathered straight from the
// device-resident layers and trees into the proof-order block of each query
// (src/fri.rs:1229-1260 for FRI, src/air.rs:565-591 and src/range.rs:483-500
// for the trace). One CTA per query; the block layout is OpenArgs'.
// The argument block stays in parameter space (__grid_constant__): the
// layer table is indexed at run time without a per-thread local copy.
__device__ __forceinline__ void gather_query(const OpenArgs& a);

__global__ void __launch_bounds__(128) openings_kernel(const __grid_constant__ OpenArgs a) {
  pdl_wait();
  const uint32_t qi = blockIdx.x, pk = blockIdx.y;  // query, proof of the group
  if (a.go) wait_gate(a.go_per_query ? a.go + qi : a.go, a.go_epoch, a.fault);
  gather_query(a);
  // The block is written: its done word, for a host that reads blocks as
  // they land.
  if (a.done) {
    __syncthreads();
    if (threadIdx.x == 0) {
      __threadfence_system();
      asm volatile("st.release.sys.global.u32 [%0], %1;" ::"l"(a.done + (size_t)pk * a.nq + qi),
                   "r"(a.go_epoch)
                   : "memory");
    }
  }
}

// Query blockIdx.x of proof blockIdx.y: its opening block.
__device__ __forceinline__ void gather_query(const OpenArgs& a) {
  const uint32_t qi = blockIdx.x, pk = blockIdx.y;
  uint32_t* out = a.out + ((size_t)pk * a.nq + qi) * a.stride;
  // Indices are positions in layer 0 (a power of two); masking leaves valid
  // ones unchanged and keeps every read inside the layers and trees, whatever
  // the mapped buffer holds (a gate opened on an early return).
  const uint64_t dom = a.nlayers ? 4ull * a.layer[0].leaves : 1ull << (a.logN + a.logB);
  const uint64_t leaf =
      *reinterpret_cast<const volatile uint64_t*>(a.indices + (size_t)pk * a.nq + qi) & (dom - 1);
  const uint64_t vo = pk * a.fri_val_stride, to = pk * a.fri_tree_stride;
  const uint32_t* lde = a.lde + pk * a.lde_stride;
  const uint32_t* ttree = a.ttree + pk * a.ttree_stride;
  const uint32_t* cb = a.cb ? a.cb + ((size_t)pk << a.logB) : nullptr;
  const uint32_t* tinv = a.tinv ? a.tinv + ((size_t)pk << (a.logN + a.logB)) : nullptr;
  // FRI layers: 16 words of values, then steps x 8 words of siblings, the
  // layers' blocks back to back from word 0. The words of all layers are one
  // index range, so a CTA's loads are in flight together rather than one
  // layer's latency after another's.
  const uint32_t fri_words =
      a.nlayers ? a.layer[a.nlayers - 1].off + 16 + 8 * a.layer[a.nlayers - 1].steps : 0u;
  uint32_t d = 0;
  for (uint32_t wi = threadIdx.x; wi < fri_words; wi += blockDim.x) {
    while (d + 1 < a.nlayers && wi >= a.layer[d + 1].off) d++;
    const OpenLayer& L = a.layer[d];
    const uint32_t t = wi - L.off;
    const uint64_t base = (leaf >> (2 * d)) & ~3ull;
    if (t < 16) {
      out[wi] = L.values[vo + 4 * base + t];
    } else {
      const uint32_t st = (t - 16) >> 3, w = (t - 16) & 7u;
      const uint64_t sib = ((base >> 2) >> st) ^ 1ull;
      out[wi] = L.tree[to + 8 * (2 * L.leaves - 2 * (L.leaves >> st) + sib) + w];
    }
  }
  if (a.no_trace) return;
  // Trace openings.
  const uint32_t logm = a.logN + a.logB;
  const uint32_t N = 1u << a.logN, B = 1u << a.logB;
  const uint64_t m = 1ull << logm;
  const uint64_t index = brev_bits((uint32_t)leaf, logm);
  uint32_t* o = out + a.trace_off;
  if (a.ncol == 0) {
    // AIR: rows base..base+7 of `index` and of `index + B`, A || B each, with
    // B = A(q+1) + C_j * tinv[j][q] (the linked column).
    const uint64_t shift = a.shift ? a.shift : B;
    const uint32_t per = 16 + 8 * a.tsteps;  // both rows' blocks in one index range
    for (uint32_t ti = threadIdx.x; ti < 2 * per; ti += blockDim.x) {
      const uint32_t h = ti >= per, t = ti - h * per;
      const uint64_t at = h ? (index + shift) % m : index;
      const uint64_t base = at & ~7ull;
      uint32_t* oh = o + h * per;
      {
        if (t < 16) {
          const uint32_t k = (uint32_t)base + (t >> 1);
          const uint32_t j = k & (B - 1u), q = k >> a.logB;
          const size_t cj = (size_t)j << a.logN;
          uint32_t v = lde[cj + q];
          if (t & 1u)
            v = a.lde_b ? a.lde_b[cj + q]
                        : fadd(lde[cj + ((q + 1u) & (N - 1u))], mmul(cb[j], tinv[cj + q]));
          oh[t] = v;
        } else {
          const uint32_t st = (t - 16) >> 3, w = (t - 16) & 7u;
          const uint64_t sib = ((base >> 3) >> st) ^ 1ull;
          oh[t] = ttree[8 * (2 * a.tleaves - 2 * (a.tleaves >> st) + sib) + w];
        }
      }
    }
  } else {
    // Range: the ncol column values at `index`, then its path.
    const uint32_t j = (uint32_t)index & (B - 1u), q = (uint32_t)(index >> a.logB);
    for (uint32_t t = threadIdx.x; t < a.ncol + 8 * a.tsteps; t += blockDim.x) {
      if (t < a.ncol) {
        o[t] = lde[(size_t)t * m + ((size_t)j << a.logN) + q];
      } else {
        const uint32_t st = (t - a.ncol) >> 3, w = (t - a.ncol) & 7u;
        const uint64_t sib = (index >> st) ^ 1ull;
        o[t] = ttree[8 * (2 * a.tleaves - 2 * (a.tleaves >> st) + sib) + w];
      }
    }
  }
}


}  // namespace

// ============================================================= launchers ====
void e4_table(const uint32_t r[4], uint32_t T[4][4]) {
  auto m = [](uint64_t x) { return (uint32_t)(((x % kP) << 32) % kP); };
  const uint64_t r0 = r[0], r1 = r[1], r2 = r[2], r3 = r[3];
  const uint64_t e1 = 11 * r1, e2 = 11 * r2, e3 = 11 * r3;
  const uint64_t rows[4][4] = {{r0, e1, e3, e2}, {r1, r0, r2, e3}, {r2, e3, r0, e1}, {r3, r2, r1, r0}};
  for (int c = 0; c < 4; c++)
    for (int i = 0; i < 4; i++) T[c][i] = m(rows[c][i]);
}

namespace launch {

static std::atomic<uint64_t> g_launches{0};
static StageRecorder* g_recorder = nullptr;
uint64_t launch_count() { return g_launches.load(); }
void set_recorder(StageRecorder* r) { g_recorder = r; }

// Counts the launches of one stage and brackets them with the recorder.
struct Stage {
  const char* name;
  cudaStream_t st;
  Stage(const char* n, cudaStream_t s) : name(n), st(s) {
    if (g_recorder) g_recorder->begin(name, st);
  }
  ~Stage() {
    if (g_recorder) g_recorder->end(name, st);
  }
  void launched(int k = 1) {
    g_launches += k;
    if (g_recorder) g_recorder->launched(name, k);
  }
};

cudaError_t const_slot_address(int slot, void** ptr) {
  if (slot < 0 || slot >= kConstSlots) return cudaErrorInvalidValue;
  void* base = nullptr;
  cudaError_t e = cudaGetSymbolAddress(&base, g_consts);
  if (e != cudaSuccess) return e;
  *ptr = static_cast<char*>(base) + (size_t)slot * sizeof(ProofConsts);
  return cudaSuccess;
}

cudaError_t fib_trace(cudaStream_t st, uint32_t* col_a, uint32_t* col_b, uint32_t n, uint32_t slot,
                      const uint32_t mats[32][4], uint32_t nproofs, const ZinvArgs* zinv,
                      const Tables* tb) {
  if (zinv && !tb) return cudaErrorInvalidValue;
  FibMats fm;  // M^(2^k) in Montgomery form
  for (int k = 0; k < 32; k++)
    for (int i = 0; i < 4; i++) fm.m[k][i] = (uint32_t)(((uint64_t)mats[k][i] << 32) % kP);
  const uint32_t per_lane = 16;  // rows per lane; a warp covers 512 consecutive rows
  const uint64_t threads = 32 * ((n + 32 * per_lane - 1) / (32 * per_lane));
  const uint32_t trace_ctas = (uint32_t)grid_for(threads);
  const ZinvArgs z = zinv ? *zinv : ZinvArgs{};
  const uint32_t extra = zinv ? (uint32_t)grid_for(1ull << zinv->logB) : 0u;
  Stage stg("trace", st);
  stg.launched();
  launch_dep(fib_trace_kernel, dim3(trace_ctas + extra, nproofs), kThreads, 0, st, col_a, col_b, n,
             slot, fm, per_lane, trace_ctas, z, tb ? *tb : Tables{});
  return cudaGetLastError();
}

cudaError_t fill_constant_columns(cudaStream_t st, uint32_t* cols, uint32_t n, uint32_t ncols,
                                  const uint32_t* d_values, uint32_t nproofs) {
  Stage stg("fill_columns", st);
  stg.launched();
  launch_dep(fill_columns_kernel, dim3(grid_for((uint64_t)n * ncols), nproofs), kThreads, 0, st,
             cols, n, ncols, d_values);
  return cudaGetLastError();
}

// Levels cta_subtree builds for a CTA of nt leaves under a tree capped at `top`.
uint32_t subtree_levels(uint32_t nt, uint32_t top) {
  uint32_t l = 0;
  while ((2u << l) <= nt && l < top) l++;
  return l;
}

// ------------------------------------------------------------ schedule ----
namespace {
constexpr int kMaxDevices = 64;
std::mutex g_sched_mu;
Schedule g_sched[kMaxDevices];

// Allows the pass-`pass` kernel `func` for half-length 2^L `smem` bytes of
// dynamic shared memory, with the largest carveout, on the current device. Each kernel's need is fixed by
// L, so the attribute is set once per kernel and device, not per launch.
// cudaFuncSetAttribute acts on the current device only, so what has been
// raised is recorded per device, and only after the call has succeeded (a
// failed raise is returned and retried on the next launch).
template <typename K>
cudaError_t raise_smem(K* func, int pass, uint32_t L, size_t smem) {
  static std::mutex mu;
  static size_t done[kMaxDevices][16][32] = {};
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lk(mu);
  if (done[dev][pass][L] >= smem) return cudaSuccess;
  e = cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  // The largest shared-memory carveout (a hint): several CTAs of 40-50 KB
  // fit beside one another on an SM only with it.
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(func, cudaFuncAttributePreferredSharedMemoryCarveout,
                             (int)cudaSharedmemCarveoutMaxShared);
  if (e == cudaSuccess) done[dev][pass][L] = smem;
  return e;
}

Schedule current_schedule() {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) dev = 0;
  std::lock_guard<std::mutex> lk(g_sched_mu);
  return g_sched[dev];
}
}  // namespace

// Pass 1 is instantiated for 2^7..2^13 points and pass 2 for 2^6..2^13.
void ntt_split_range(uint32_t logn, uint32_t* lo, uint32_t* hi) {
  if (logn <= 12 || logn > 26) {
    *lo = 1;
    *hi = 0;
    return;
  }
  *lo = logn >= 20 ? logn - 13 : 7;
  *hi = logn - 6 < 13 ? logn - 6 : 13;
}

uint32_t ntt_default_split(uint32_t logn) { return (logn + 1) / 2; }

bool schedule_valid(const Schedule& s) {
  for (uint32_t l = 0; l < 32; l++) {
    uint32_t lo, hi;
    ntt_split_range(l, &lo, &hi);
    if (s.ntt_radix32[l] > 3 || (s.ntt_radix32[l] && lo > hi)) return false;
    if (!s.ntt_log_n1[l]) continue;
    if (s.ntt_log_n1[l] < lo || s.ntt_log_n1[l] > hi) return false;
  }
  return s.merkle_top_log >= 10 && s.merkle_top_log <= 18 && s.grind_ctas_per_sm >= 1 &&
         s.grind_ctas_per_sm <= 16;
}

Schedule get_schedule(int device) {
  std::lock_guard<std::mutex> lk(g_sched_mu);
  return g_sched[device >= 0 && device < kMaxDevices ? device : 0];
}

void set_schedule(int device, const Schedule& s) {
  if (device < 0 || device >= kMaxDevices) return;
  std::lock_guard<std::mutex> lk(g_sched_mu);
  g_sched[device] = s;
}

// Halves the register passes cover: 2^6..2^12 points, L even.
bool reg_split_ok(uint32_t L) { return L >= 6 && L <= 12 && (L & 1u) == 0; }

namespace {
PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) !=
            cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      p = nullptr;
    return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  }();
  return fn;
}

// CTAs of `func` (threads, smem) resident on the current device at once:
// the grid of a streamed kernel. Cached per kernel slot and device.
template <typename K>
uint32_t resident_ctas(K* func, int slot, uint32_t L, int threads, size_t smem) {
  static std::mutex mu;
  static uint32_t cached[kMaxDevices][4][32] = {};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) dev = 0;
  std::lock_guard<std::mutex> lk(mu);
  uint32_t& c = cached[dev][slot][L];
  if (!c) {
    int sms = 0, per = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, func, threads, smem);
    c = (uint32_t)((sms > 0 ? sms : 1) * (per > 0 ? per : 1));
  }
  return c;
}

template <int L, bool INV>
cudaError_t reg_pass1(cudaStream_t st, const CUtensorMap& map, uint32_t* yt, const NttArgs& a, dim3 g,
                      bool streamed) {
  constexpr int threads = reg_ntt::kC << (L / 2);
  if constexpr (reg_ntt::streamed_ok(L)) {
    if (streamed) {
      constexpr size_t smem = reg_ntt::pass1s_smem(L);
      if (cudaError_t e = raise_smem(ntt_reg1s_kernel<L, INV>, 10 + INV, L, smem)) return e;
      const uint32_t tiles = g.x * g.y;
      const uint32_t res = resident_ctas(ntt_reg1s_kernel<L, INV>, INV, L, threads, smem);
      const uint32_t ctas = tiles < res ? tiles : res;
      launch_dep(ntt_reg1s_kernel<L, INV>, ctas, threads, smem, st, map, yt, a, tiles);
      return cudaGetLastError();
    }
  }
  constexpr size_t smem = reg_ntt::pass1_smem(L);
  if (!a.bad && !a.pre_gamma) {  // the LDE: no word check, no 31^i scaling
    if (cudaError_t e = raise_smem(ntt_reg1_kernel<L, INV, true>, 14 + INV, L, smem)) return e;
    launch_dep(ntt_reg1_kernel<L, INV, true>, g, threads, smem, st, map, yt, a);
    return cudaGetLastError();
  }
  if (cudaError_t e = raise_smem(ntt_reg1_kernel<L, INV, false>, 6 + INV, L, smem)) return e;
  launch_dep(ntt_reg1_kernel<L, INV, false>, g, threads, smem, st, map, yt, a);
  return cudaGetLastError();
}
template <int L, bool INV>
cudaError_t reg_pass2(cudaStream_t st, const uint32_t* yt, uint32_t* out, const NttArgs& a, dim3 g,
                      bool streamed) {
  constexpr int threads = reg_ntt::kC << (L / 2);
  if constexpr (reg_ntt::streamed_ok(L)) {
    if (streamed) {
      constexpr size_t smem = reg_ntt::pass2s_smem(L);
      if (cudaError_t e = raise_smem(ntt_reg2s_kernel<L, INV>, 12 + INV, L, smem)) return e;
      const uint32_t tiles = g.x * g.y;
      const uint32_t res = resident_ctas(ntt_reg2s_kernel<L, INV>, 2 + INV, L, threads, smem);
      const uint32_t ctas = tiles < res ? tiles : res;
      launch_dep(ntt_reg2s_kernel<L, INV>, ctas, threads, smem, st, yt, out, a, tiles);
      return cudaGetLastError();
    }
  }
  constexpr size_t smem = reg_ntt::pass2_smem(L);
  if (cudaError_t e = raise_smem(ntt_reg2_kernel<L, INV>, 8 + INV, L, smem)) return e;
  launch_dep(ntt_reg2_kernel<L, INV>, g, threads, smem, st, yt, out, a);
  return cudaGetLastError();
}
}  // namespace

// Register-pass four-step transform (ntt_reg.cuh): pass 1 reads its column
// tiles through a tensor map over `in`, viewed as [in blocks][n1][n2] words.
cudaError_t ntt_reg(cudaStream_t st, const NttArgs& a, const NttPlan& plan, const uint32_t* in,
                    uint32_t* out, uint32_t* scratch, uint32_t logn1, uint32_t logn2, bool streamed) {
  PFN_cuTensorMapEncodeTiled_v12000 encode = tensor_map_encoder();
  if (!encode) return cudaErrorNotSupported;
  const uint32_t in_div = plan.in_div ? plan.in_div : 1;
  CUtensorMap map;
  const cuuint64_t dims[3] = {1ull << logn2, 1ull << logn1, (plan.batch + in_div - 1) / in_div};
  const cuuint64_t strides[2] = {4ull << logn2, 4ull << plan.logn};
  const cuuint32_t box[3] = {reg_ntt::kC, logn1 < 8 ? (1u << logn1) : 256u, 1u};
  const cuuint32_t elem[3] = {1u, 1u, 1u};
  if (encode(&map, CU_TENSOR_MAP_DATA_TYPE_UINT32, 3, const_cast<uint32_t*>(in), dims, strides, box, elem,
             CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
             CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
    return cudaErrorInvalidValue;
  const dim3 g1((1u << logn2) / reg_ntt::kC, plan.batch), g2((1u << logn1) / reg_ntt::kC, plan.batch);
  Stage stg(plan.inverse ? "intt" : "ntt", st);
  stg.launched(2);
  cudaError_t e = cudaErrorInvalidValue;
  const bool inv = plan.inverse != 0;
  switch (logn1) {
#define Z0P_R1(Lv) \
  case Lv:                                                                                         \
    e = inv ? reg_pass1<Lv, true>(st, map, scratch, a, g1, streamed)                               \
            : reg_pass1<Lv, false>(st, map, scratch, a, g1, streamed);                             \
    break;
    Z0P_R1(8) Z0P_R1(10) Z0P_R1(12)  // pass 1 is at least 2^7 points
#undef Z0P_R1
  }
  if (e != cudaSuccess) return e;
  e = cudaErrorInvalidValue;
  switch (logn2) {
#define Z0P_R2(Lv) \
  case Lv:                                                                                         \
    e = inv ? reg_pass2<Lv, true>(st, scratch, out, a, g2, streamed)                               \
            : reg_pass2<Lv, false>(st, scratch, out, a, g2, streamed);                             \
    break;
    Z0P_R2(6) Z0P_R2(8) Z0P_R2(10) Z0P_R2(12)
#undef Z0P_R2
  }
  return e;
}

cudaError_t ntt(cudaStream_t st, const Tables& tb, const NttPlan& plan, const uint32_t* in,
                uint32_t* out, uint32_t* scratch) {
  NttArgs a;
  a.logn = plan.logn;
  a.inverse = plan.inverse;
  a.in_div = plan.in_div ? plan.in_div : 1;
  a.twist_mod = plan.twist_mod ? plan.twist_mod : 1;
  a.twist_shift = plan.twist_shift;
  a.post_gamma = plan.post_gamma;
  a.bad = plan.bad;  // with in_div > 1 a word is checked once per reader: the flag is idempotent
  a.pre_gamma = plan.pre_gamma;
  // n^-1 in Montgomery form: (2^-logn) * 2^32 mod p.
  {
    uint64_t inv2 = (kP + 1) / 2;  // 2^-1 mod p
    uint64_t v = 1;
    for (uint32_t i = 0; i < plan.logn; i++) v = v * inv2 % kP;
    a.ninv_m = (uint32_t)((v << 32) % kP);
  }
  a.tb = tb;
  const uint32_t n = 1u << plan.logn;
  if (plan.logn <= 12) {
    size_t smem = (size_t)(tw_offset(skewed_len(n)) + 2 * tw_entries(plan.logn) + 2) * 4;
    int threads = n >= 2048 ? 512 : (n >= 256 ? 256 : 128);
    Stage stg(plan.inverse ? "intt" : "ntt", st);
    stg.launched();
    switch (plan.logn) {
#define Z0P_SMALL(Lv) \
  case Lv: launch_dep(ntt_small_kernel<Lv>, plan.batch, threads, smem, st, in, out, a); break;
      Z0P_SMALL(0) Z0P_SMALL(1) Z0P_SMALL(2) Z0P_SMALL(3) Z0P_SMALL(4) Z0P_SMALL(5)
      Z0P_SMALL(6) Z0P_SMALL(7) Z0P_SMALL(8) Z0P_SMALL(9) Z0P_SMALL(10) Z0P_SMALL(11)
      Z0P_SMALL(12)
#undef Z0P_SMALL
    }
    return cudaGetLastError();
  }
  const Schedule sched = current_schedule();
  uint32_t logn1 = ntt_default_split(plan.logn);
  if (plan.logn < 32 && sched.ntt_log_n1[plan.logn]) {
    uint32_t lo, hi;
    ntt_split_range(plan.logn, &lo, &hi);
    if (sched.ntt_log_n1[plan.logn] >= lo && sched.ntt_log_n1[plan.logn] <= hi)
      logn1 = sched.ntt_log_n1[plan.logn];
  }
  const uint32_t logn2 = plan.logn - logn1;
  const uint32_t n1 = 1u << logn1, n2 = 1u << logn2;
  const uint32_t variant = plan.logn < 32 ? sched.ntt_radix32[plan.logn] : 0u;
  if (variant >= 2 && reg_split_ok(logn1) && reg_split_ok(logn2) && tb.stw &&
      (reinterpret_cast<uintptr_t>(in) & 15u) == 0)
    return ntt_reg(st, a, plan, in, out, scratch, logn1, logn2, variant == 3);
  // C = R = 8 columns per CTA (32-byte global segments), 4 for the largest halves.
  const int logc = logn1 > 12 ? 2 : 3;
  const int logr = logn2 > 12 ? 2 : 3;
  size_t smem1 =
      ((size_t)tw_offset(col_stride(logn1, 1u << logc) << logc) + 2 * tw_entries(logn1) + n1) * 4;
  size_t smem2 = ((size_t)tw_offset(col_stride(logn2, 1u << logr) << logr) + 2 * tw_entries(logn2)) * 4;
  dim3 g1(n2 >> logc, plan.batch), g2(n1 >> logr, plan.batch);
  // Register groups of 32 (two shared-memory passes for a 2^10 half) run
  // 256 threads a CTA; groups of 16 run 512.
  const bool r32 = plan.logn < 32 && sched.ntt_radix32[plan.logn] == 1;
  const int threads = r32 ? 256 : 512, slot = r32 ? 3 : 0;
  Stage stg(plan.inverse ? "intt" : "ntt", st);
  stg.launched(2);
  switch (logn1) {
#define Z0P_P1K(Lv, LC, KM)                                                                      \
    if (cudaError_t re = raise_smem(ntt_pass1_kernel<Lv, LC, KM>, 1 + slot, Lv, smem1))          \
      return re;                                                                                 \
    launch_dep(ntt_pass1_kernel<Lv, LC, KM>, g1, threads, smem1, st, in, scratch, a);
#define Z0P_P1(Lv, LC)                                                                           \
  case Lv:                                                                                       \
    if (r32) { Z0P_P1K(Lv, LC, 5) } else { Z0P_P1K(Lv, LC, 4) }                                  \
    break;
    Z0P_P1(7, 3) Z0P_P1(8, 3) Z0P_P1(9, 3) Z0P_P1(10, 3) Z0P_P1(11, 3) Z0P_P1(12, 3) Z0P_P1(13, 2)
#undef Z0P_P1
#undef Z0P_P1K
    default: return cudaErrorInvalidValue;
  }
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  switch (logn2) {
#define Z0P_P2K(Lv, LR, KM)                                                                      \
    if (cudaError_t re = raise_smem(ntt_pass2_kernel<Lv, LR, KM>, 2 + slot, Lv, smem2))          \
      return re;                                                                                 \
    launch_dep(ntt_pass2_kernel<Lv, LR, KM>, g2, threads, smem2, st, scratch, out, a);
#define Z0P_P2(Lv, LR)                                                                           \
  case Lv:                                                                                       \
    if (r32) { Z0P_P2K(Lv, LR, 5) } else { Z0P_P2K(Lv, LR, 4) }                                  \
    break;
    Z0P_P2(6, 3) Z0P_P2(7, 3) Z0P_P2(8, 3) Z0P_P2(9, 3) Z0P_P2(10, 3) Z0P_P2(11, 3) Z0P_P2(12, 3)
    Z0P_P2(13, 2)
#undef Z0P_P2
#undef Z0P_P2K
    default: return cudaErrorInvalidValue;
  }
  (void)n;
  return cudaGetLastError();
}

cudaError_t coset_zinv(cudaStream_t st, const Tables& tb, uint32_t* zinv, uint32_t* zinv2,
                       uint32_t logB, uint32_t gamma_n_m, uint32_t* cb, uint32_t slot,
                       uint32_t nproofs) {
  Stage stg("coset_zinv", st);
  stg.launched();
  const ZinvArgs z{zinv, zinv2, logB, gamma_n_m, cb, slot};
  launch_dep(coset_zinv_kernel, dim3(grid_for(1ull << logB), nproofs), kThreads, 0, st, z, tb);
  return cudaGetLastError();
}

cudaError_t air_trace_leaves(cudaStream_t st, const Tables& tb, const uint32_t* lde_a,
                             const uint32_t* cb, uint32_t w_last_m, uint32_t* leaves,
                             uint32_t* tinv, uint32_t logN, uint32_t logB, uint32_t top,
                             uint32_t* cap, unsigned int* counter, uint32_t* levels,
                             uint32_t nproofs, uint64_t tree_stride, uint64_t cap_stride,
                             const uint32_t* lde_b) {
  uint32_t nleaves = 1u << (logN + logB - 3);
  if (nleaves > kFuseMaxLeaves) {
    top = 0;  // no subtree; merkle_build does every level
    cap = nullptr;
    counter = nullptr;
  }
  *levels = counter ? top
                    : subtree_levels(nleaves < kTraceLeafThreads ? nleaves : kTraceLeafThreads, top);
  Stage stg("trace_leaves", st);
  stg.launched();
  if (nleaves > kFuseMaxLeaves && !lde_b)  // two leaves a thread, no subtree
    launch_dep(air_trace_leaves2_kernel<true>,
               dim3(grid_for(nleaves / 2, kTraceLeafThreads), nproofs), kTraceLeafThreads, 0, st,
               lde_a, cb, w_last_m, leaves, tinv, logN, logB, nleaves, tree_stride, lde_b, tb);
  else if (nleaves > kFuseMaxLeaves)
    launch_dep(air_trace_leaves2_kernel<false>,
               dim3(grid_for(nleaves / 2, kTraceLeafThreads), nproofs), kTraceLeafThreads, 0, st,
               lde_a, cb, w_last_m, leaves, tinv, logN, logB, nleaves, tree_stride, lde_b, tb);
  else if (!lde_b)
    launch_dep(air_trace_leaves_kernel<true>, dim3(grid_for(nleaves, kTraceLeafThreads), nproofs),
               kTraceLeafThreads, 0, st, lde_a, cb, w_last_m, leaves, tinv, logN, logB, nleaves,
               top, cap, counter, tree_stride, cap_stride, lde_b, tb);
  else
    launch_dep(air_trace_leaves_kernel<false>, dim3(grid_for(nleaves, kTraceLeafThreads), nproofs),
               kTraceLeafThreads, 0, st, lde_a, cb, w_last_m, leaves, tinv, logN, logB, nleaves,
               top, cap, counter, tree_stride, cap_stride, lde_b, tb);
  return cudaGetLastError();
}

bool fold_segment_ok(uint32_t logN, uint32_t logB) {
  return logN >= 1 && logN <= 8 && (1u << (logN + logB)) <= kSegmentMaxRows && logN + logB >= 5;
}

cudaError_t fold_segment(cudaStream_t st, const Tables& tb, const uint32_t* cols, unsigned int* bad,
                         uint32_t* lde, uint32_t* tree, uint32_t* cap, uint32_t logN, uint32_t logB,
                         uint32_t top) {
  if (!fold_segment_ok(logN, logB) || !tb.stw) return cudaErrorInvalidValue;
  const uint32_t S = 1u << logN, B = 1u << logB, m = S * B;
  const uint32_t cs = (skewed_len(S) + 1u) & ~1u;
  const size_t smem = 4 * ((size_t)2 * cs + 2ull * B * cs + 4ull * tw_entries(logN) + 18ull * m);
  uint64_t inv2 = (kP + 1) / 2, v = 1;  // S^-1 in Montgomery form
  for (uint32_t i = 0; i < logN; i++) v = v * inv2 % kP;
  const uint32_t ninv_m = (uint32_t)((v << 32) % kP);
  Stage stg("fold_segment", st);
  stg.launched();
  switch (logN) {
#define Z0P_SEG(Lv)                                                                              \
  case Lv:                                                                                         \
    launch_dep(fold_segment_kernel<Lv>, 1, m, smem, st, cols, bad, lde, tree, cap, logB, top,     \
               ninv_m, tb);                                                                      \
    break;
    Z0P_SEG(1) Z0P_SEG(2) Z0P_SEG(3) Z0P_SEG(4) Z0P_SEG(5) Z0P_SEG(6) Z0P_SEG(7) Z0P_SEG(8)
#undef Z0P_SEG
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

cudaError_t range_trace_leaves(cudaStream_t st, const uint32_t* lde, uint32_t* leaves,
                               uint32_t logN, uint32_t logB, uint32_t ncols, uint32_t nproofs,
                               uint64_t tree_stride, unsigned int* counter, uint32_t top,
                               uint32_t* cap, uint64_t cap_stride, uint32_t* levels) {
  if (ncols < 1 || ncols > 25) return cudaErrorInvalidValue;
  const uint64_t m = 1ull << (logN + logB);
  const bool fused = counter && m <= kFuseMaxLeaves;
  if (levels) *levels = fused ? top : 0u;
  Stage stg("trace_leaves", st);
  stg.launched();
  const dim3 grid(grid_for(m), nproofs);
  if (fused)
    launch_dep(range_trace_leaves_kernel<true>, grid, kThreads, 0, st, lde, leaves, logN, logB,
               ncols, tree_stride, counter, top, cap, cap_stride);
  else
    launch_dep(range_trace_leaves_kernel<false>, grid, kThreads, 0, st, lde, leaves, logN, logB,
               ncols, tree_stride, nullptr, 0, nullptr, 0);
  return cudaGetLastError();
}

cudaError_t merkle_build(cudaStream_t st, uint32_t* tree, uint64_t leaves, uint32_t top,
                         unsigned int* counter, uint32_t* cap, uint32_t from, uint32_t nproofs,
                         uint64_t stride, uint64_t cap_stride) {
  if (from > 0 && from >= top) return cudaSuccess;  // the leaf kernel built up to the cap
  Stage stg("merkle_levels", st);
  if (top == 0) {  // the cap is the leaf level itself
    if (!cap) return cudaSuccess;
    stg.launched();
    launch_dep(copy_words_kernel, dim3(grid_for(8 * leaves), nproofs), kThreads, 0, st, tree, cap,
               8 * leaves, stride, cap_stride);
    return cudaGetLastError();
  }
  // Levels with more than 2^16 nodes fill the GPU on their own: one launch
  // each. The rest (at most 2^16 nodes at l0, so at most 128 CTAs of 512
  // children, whose roots fit the last CTA's shared memory) go to one launch
  // of merkle_top_kernel. (Starting the top kernel anywhere from 2^12 to 2^18
  // nodes measured within 7% on a 2^21-leaf tree; 2^16 was the fastest.)
  uint32_t level = from;
  const uint32_t top_log = current_schedule().merkle_top_log;
  // Pairs of levels while both source levels are above the top kernel's.
  while (level + 2 <= top && (leaves >> (level + 1)) > (1ull << top_log)) {
    uint64_t cnt = leaves >> (level + 2);
    const uint32_t* prev = tree + 8 * (2 * leaves - 2 * (leaves >> level));
    uint32_t* mid = tree + 8 * (2 * leaves - 2 * (leaves >> (level + 1)));
    uint32_t* next = tree + 8 * (2 * leaves - 2 * (leaves >> (level + 2)));
    stg.launched();
    launch_dep(merkle_level2_kernel, dim3(grid_for(cnt), nproofs), kThreads, 0, st, prev, mid, next,
               cnt, level + 2 == top ? cap : nullptr, stride, cap_stride);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    level += 2;
  }
  while (level < top && (leaves >> level) > (1ull << top_log)) {
    uint64_t cnt = leaves >> (level + 1);
    const uint32_t* prev = tree + 8 * (2 * leaves - 2 * (leaves >> level));
    uint32_t* next = tree + 8 * (2 * leaves - 2 * (leaves >> (level + 1)));
    stg.launched();
    launch_dep(merkle_level_kernel, dim3(grid_for(cnt), nproofs), kThreads, 0, st, prev, next, cnt,
               level + 1 == top ? cap : nullptr, stride, cap_stride);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    level++;
  }
  if (level >= top) return cudaSuccess;
  const uint32_t lsub = level + 9 < top ? level + 9 : top;
  const uint64_t per_cta_children = 2ull << (lsub - level - 1);  // level-l0 nodes per CTA
  const uint64_t blocks = ((leaves >> level) + per_cta_children - 1) / per_cta_children;
  stg.launched();
  launch_dep(merkle_top_kernel, dim3((unsigned)blocks, nproofs), kTopThreads, 0, st, tree, leaves,
             level, top, counter, cap, stride, cap_stride);
  return cudaGetLastError();
}

cudaError_t air_compose_leaves(cudaStream_t st, const Tables& tb, const AirComposeArgs& a,
                               uint32_t nproofs, uint32_t* levels) {
  uint32_t quarter = 1u << (a.logN + a.logB - 2);
  AirComposeArgs f = a;
  if (quarter > kFuseMaxLeaves || !f.counter) {
    f.counter = nullptr;  // merkle_build does every level
    f.top = 0;
    f.cap = nullptr;
  }
  if (levels) *levels = f.counter ? f.top : 0;
  Stage stg("air_compose_leaves", st);
  stg.launched();
  const bool params = nproofs == 1;  // one proof: the weights travel as kernel parameters
  if (f.counter && params)
    launch_dep(air_compose_leaves_kernel<true, true>, dim3(grid_for(quarter), nproofs), kThreads, 0,
               st, f, tb);
  else if (f.counter)
    launch_dep(air_compose_leaves_kernel<true, false>, dim3(grid_for(quarter), nproofs), kThreads,
               0, st, f, tb);
  else if (params)
    launch_dep(air_compose_leaves_kernel<false, true>, dim3(grid_for(quarter), nproofs), kThreads,
               0, st, f, tb);
  else
    launch_dep(air_compose_leaves_kernel<false, false>, dim3(grid_for(quarter), nproofs), kThreads,
               0, st, f, tb);
  return cudaGetLastError();
}

cudaError_t range_compose_leaves(cudaStream_t st, const Tables& tb, const RangeComposeArgs& a,
                                 uint32_t nproofs) {
  uint32_t quarter = 1u << (a.logN + a.logB - 2);
  Stage stg("range_compose_leaves", st);
  stg.launched();
  launch_dep(range_compose_leaves_kernel, dim3(grid_for(quarter), nproofs), kThreads, 0, st, a, tb);
  return cudaGetLastError();
}

bool fri_fold_uses_slot(const FoldArgs& a) {
  return a.logn >= 4 && (!a.counter || (1ull << (a.logn - 4)) > kFuseMaxLeaves);
}

cudaError_t fri_fold(cudaStream_t st, const Tables& tb, const FoldArgs& a, uint32_t* levels,
                     uint32_t nproofs) {
  *levels = 0;
  if (a.logn < 2) return cudaErrorInvalidValue;
  if (a.logn >= 4) {
    uint64_t nleaf = 1ull << (a.logn - 4);
    FoldArgs f = a;
    if (nleaf > kFuseMaxLeaves) {
      f.top = 0;  // no subtree; merkle_build does every level
      f.cap = nullptr;
      f.counter = nullptr;
    }
    *levels = f.counter ? f.top
                        : subtree_levels(nleaf < (uint64_t)kFoldThreads ? (uint32_t)nleaf
                                                                        : kFoldThreads,
                                         f.top);
    const bool slot = fri_fold_uses_slot(a);
    if (slot ? a.slot + nproofs > (uint32_t)kConstSlots : !a.tab) return cudaErrorInvalidValue;
    Stage stg("fri_fold_leaves", st);
    stg.launched();
    const dim3 grid(grid_for(nleaf, kFoldThreads), nproofs);
    const bool wide = (reinterpret_cast<uintptr_t>(f.in) & 31u) == 0 && (f.in_stride & 7u) == 0;
    if (slot && wide)
      launch_dep(fri_fold_leaf_kernel<true>, grid, kFoldThreads, 0, st, f, tb);
    else if (slot)
      launch_dep(fri_fold_leaf_kernel<false>, grid, kFoldThreads, 0, st, f, tb);
    else
      launch_dep(fri_fold_quad_kernel, grid, kFold4Threads, 0, st, f, tb);
    return cudaGetLastError();
  }
  if (!a.tab) return cudaErrorInvalidValue;
  {
    Stage stg("fri_fold_small", st);
    stg.launched();
    launch_dep(fri_fold_plain_kernel, dim3(1, nproofs), 32, 0, st, a, tb);
  }
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  return layer_leaves(st, a.out, 1ull << (a.logn - 2), a.leaves, nproofs, a.out_stride,
                      a.tree_stride);
}

cudaError_t layer_leaves(cudaStream_t st, const uint32_t* values, uint64_t len, uint32_t* leaves,
                         uint32_t nproofs, uint64_t in_stride, uint64_t out_stride) {
  Stage stg("layer_leaves", st);
  stg.launched();
  if (len % 4 == 0) {
    launch_dep(leaf64_kernel, dim3(grid_for(len / 4), nproofs), kThreads, 0, st, values, leaves,
               len / 4, len / 4, in_stride, out_stride);
  } else {
    launch_dep(leaf16_kernel, dim3(grid_for(len), nproofs), kThreads, 0, st, values, leaves, len,
               in_stride, out_stride);
  }
  return cudaGetLastError();
}

cudaError_t merkle_flat64_leaves(cudaStream_t st, const uint32_t* flat, uint64_t count,
                                 uint64_t npad, uint32_t* leaves) {
  if (!count || npad < count) return cudaErrorInvalidValue;
  Stage stg("leaf64", st);
  stg.launched();
  launch_dep(leaf64_kernel, grid_for(npad), kThreads, 0, st, flat, leaves, count, npad, 0, 0);
  return cudaGetLastError();
}

bool grind_supports(uint32_t head_len) { return head_len == kPowHeadLen; }

cudaError_t grind(cudaStream_t st, const uint32_t* head, uint32_t head_len, uint32_t bits,
                  unsigned long long* state, unsigned long long* out, uint64_t max_nonces,
                  uint32_t nproofs, const unsigned int* go, unsigned int go_epoch,
                  unsigned int* fault) {
  if (!grind_supports(head_len) || bits > 32 || !head || nproofs == 0 || nproofs > 65535u)
    return cudaErrorInvalidValue;
  GrindArgs a;
  a.head = head;
  a.go = go;
  a.go_epoch = go_epoch;
  a.fault = fault;
  a.bits = bits;
  a.state = state;
  a.out = out;
  a.max_chunks = (max_nonces + kGrindChunk - 1) / kGrindChunk;
  // Per device: SM count and the grind kernel's resident CTAs.
  static std::mutex mu;
  static int cached_sms[kMaxDevices] = {}, cached_max[kMaxDevices] = {};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) dev = 0;
  int sms, max_ctas;
  {
    std::lock_guard<std::mutex> lk(mu);
    if (!cached_max[dev]) {
      int per = 0;
      cudaDeviceGetAttribute(&cached_sms[dev], cudaDevAttrMultiProcessorCount, dev);
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, grind_kernel, kGrindThreads, 0);
      cached_max[dev] = cached_sms[dev] * (per > 0 ? per : 1);
    }
    sms = cached_sms[dev];
    max_ctas = cached_max[dev];
  }
  // The search expects 2^bits nonces. A thread stops at its next nonce once
  // that passes the best hit, so at most one nonce per thread is hashed past
  // the answer: the grid can fill the GPU (four CTAs per SM reach the hash
  // ceiling) without wasting much, but stays below the expected search.
  // A search of a few bits (2^bits within a few chunks) takes that many CTAs,
  // not a full grid: the answer is the same, the launch and the last-CTA
  // handshake shorter.
  uint64_t want = (1ull << bits) / kGrindChunk;
  const int per_sm = (int)current_schedule().grind_ctas_per_sm;
  int ctas = want > (uint64_t)(per_sm * sms) ? per_sm * sms : (int)want;
  if (ctas > max_ctas) ctas = max_ctas;
  if (ctas < 1) ctas = 1;
  Stage stg("grind", st);
  stg.launched();
  launch_dep(grind_kernel, dim3(ctas, nproofs), kGrindThreads, 0, st, a);
  return cudaGetLastError();
}

cudaError_t uniform_trees(cudaStream_t st, const UniformTree* trees, uint32_t ntrees) {
  if (ntrees == 0) return cudaSuccess;
  Stage stg("uniform_trees", st);
  stg.launched();
  launch_dep(uniform_trees_kernel, ntrees, 128, 0, st, trees);
  return cudaGetLastError();
}

cudaError_t mask_pad(cudaStream_t st, const Tables& tb, const uint32_t* coeffs, const uint32_t* r,
                     uint32_t* out, uint32_t n, uint32_t n_rand, uint32_t padded, uint32_t ncols) {
  Stage stg("mask_pad", st);
  stg.launched();
  launch_dep(mask_pad_kernel, dim3(grid_for(padded), ncols), kThreads, 0, st, coeffs, r, out, n,
             n_rand, padded, tb);
  return cudaGetLastError();
}

cudaError_t table_compose(cudaStream_t st, const Tables& tb, const TableComposeArgs& a) {
  Stage stg("table_compose", st);
  stg.launched();
  launch_dep(table_compose_kernel, grid_for(1ull << (a.logN + a.logB - 2)), kThreads, 0, st, a, tb);
  return cudaGetLastError();
}

cudaError_t air_compose_general(cudaStream_t st, const Tables& tb, const AirComposeArgs& a,
                                const uint32_t* lde_b, uint32_t r) {
  Stage stg("air_compose_leaves", st);
  stg.launched();
  launch_dep(air_compose_general_kernel,
             grid_for(1ull << (a.logN + a.logB - 2)), kThreads, 0, st, a, lde_b, r, tb);
  return cudaGetLastError();
}

cudaError_t gamma_scale(cudaStream_t st, const Tables& tb, const uint32_t* in, uint32_t* out,
                        uint32_t n, uint32_t ext, unsigned int* bad) {
  Stage stg("fri_input", st);
  stg.launched();
  launch_dep(gamma_scale_kernel, dim3(grid_for(n), ext ? 4 : 1), kThreads, 0, st, in, out, n, ext,
             bad, tb);
  return cudaGetLastError();
}

cudaError_t layer0_leaves(cudaStream_t st, const uint32_t* src, uint32_t* layer0, uint32_t* leaves,
                          unsigned int* bad, uint32_t logm, uint32_t logB, uint32_t ncomp,
                          bool coset_major, unsigned int* counter, uint32_t top, uint32_t* cap,
                          uint32_t* levels) {
  if (logm < 2) return cudaErrorInvalidValue;
  const uint64_t quarter = 1ull << (logm - 2);
  const bool fused = counter && quarter <= kFuseMaxLeaves;
  Layer0Args a{src, layer0, leaves, bad, logm, coset_major ? logB : 0u, ncomp,
               coset_major ? 1u : 0u, fused ? counter : nullptr, fused ? top : 0u,
               fused ? cap : nullptr};
  if (levels) *levels = fused ? top : 0u;
  Stage stg("layer0_leaves", st);
  stg.launched();
  if (fused)
    launch_dep(layer0_leaves_kernel<true>, grid_for(quarter), kThreads, 0, st, a);
  else
    launch_dep(layer0_leaves_kernel<false>, grid_for(quarter), kThreads, 0, st, a);
  return cudaGetLastError();
}

cudaError_t row_inverses(cudaStream_t st, const Tables& tb, uint32_t* tinv, uint32_t w_last_m,
                         uint32_t logN, uint32_t logB) {
  if (logN + logB < 3) return cudaErrorInvalidValue;
  Stage stg("row_inverses", st);
  stg.launched();
  launch_dep(row_inverses_kernel,
             grid_for(1ull << (logN + logB - 3)), kThreads, 0, st, tinv, w_last_m, logN, logB, tb);
  return cudaGetLastError();
}


cudaError_t fold_combine(cudaStream_t st, const Tables& tb, const FoldCombineArgs& a,
                         uint32_t* levels) {
  if (a.logN + a.logB < 3) return cudaErrorInvalidValue;
  const uint64_t quarter = 1ull << (a.logN + a.logB - 2);
  const bool fused = a.counter && quarter <= kFuseMaxLeaves;
  if (!fused && !a.tinv) return cudaErrorInvalidValue;  // the unfused kernel reads T
  if (levels) *levels = fused ? a.top : 0u;
  Stage stg("fold_combine", st);
  stg.launched();
  if (fused)
    launch_dep(fold_combine_kernel<true>, grid_for(quarter), kThreads, 0, st, a, tb);
  else
    launch_dep(fold_combine_kernel<false>, grid_for(quarter), kThreads, 0, st, a, tb);
  return cudaGetLastError();
}

cudaError_t fold_openings(cudaStream_t st, const FoldStepDev* steps, uint32_t nsteps,
                          const uint64_t* leaves, uint32_t nq, uint32_t logN, uint32_t logB,
                          uint32_t path_steps, uint32_t* out, uint32_t stride) {
  Stage stg("fold_openings", st);
  stg.launched();
  launch_dep(fold_openings_kernel, dim3(nq, nsteps), 64, 0, st, steps, leaves, nq, logN, logB,
             path_steps, out, stride);
  return cudaGetLastError();
}

cudaError_t hash_ceiling(cudaStream_t st, const uint32_t* in, uint32_t* out, uint32_t blocks,
                         int iters) {
  launch_dep(hash_ceiling_kernel, blocks, 256, 0, st, in, out, iters);
  return cudaGetLastError();
}

cudaError_t openings(cudaStream_t st, const OpenArgs& a, uint32_t nproofs) {
  if (a.nlayers > kMaxOpenLayers) return cudaErrorInvalidValue;
  if (!a.nq) return cudaSuccess;
  Stage stg("gather", st);
  stg.launched();
  launch_dep(openings_kernel, dim3(a.nq, nproofs), 128, 0, st, a);
  return cudaGetLastError();
}

cudaError_t coset_to_natural(cudaStream_t st, const uint32_t* in, uint32_t* out, uint32_t logN,
                             uint32_t logB, uint64_t batch) {
  if (batch == 0) return cudaSuccess;
  if (batch > 65535 || (logB > 5 && (1ull << (logB - 5)) > 65535)) return cudaErrorInvalidValue;
  const uint64_t qt = ((1ull << logN) + kNatTileQ - 1) / kNatTileQ;
  const uint32_t jt = logB > 5 ? 1u << (logB - 5) : 1u;
  if (qt > 0x7fffffffull) return cudaErrorInvalidValue;
  Stage stg("coset_to_natural", st);
  stg.launched();
  launch_dep(coset_to_natural_kernel, dim3((unsigned)qt, jt, (unsigned)batch), 256, 0, st, in, out,
             logN, logB);
  return cudaGetLastError();
}


}  // namespace launch
}  // namespace z0p

// ====================================================== allocation-free LDE ====
// z0p_gpu_rs_extend_noalloc: the Reed-Solomon extension of z0p_gpu_rs_extend
// for callers that may not allocate device memory. Such callers include a
// process whose device heap is owned by another allocator (a framework's
// caching pool that must see every byte), a latency-critical loop in which
// cudaMalloc/cudaFree would synchronise the device, and a deployment with a
// fixed memory budget that must be fully accounted when the library loads.
// Its working memory is the static arrays below. They are sized for at most
// kNoAllocMaxElems output elements and stay resident on every device that
// loads this library until the process exits.
#include <mutex>
#include <vector>

#include "../../include/z0p_gpu.h"
#include "host.h"

namespace {

// Largest n * batch * blowup the allocation-free entry accepts (4 MiB per region).
constexpr uint64_t kNoAllocMaxElems = 1ull << 20;
constexpr size_t kNoAllocTableWords = (1u << 14) + (1u << 13) + (1u << 12) + (1u << 15);

// Three regions of kNoAllocMaxElems words: coefficients, four-step
// intermediate, coset-major LDE (12 MiB in total).
static __device__ __align__(256) uint32_t g_noalloc_scratch[3 * kNoAllocMaxElems];
// omega_{2^27} and 31 power tables (same contents as a context's tables).
static __device__ __align__(256) uint32_t g_noalloc_tables[kNoAllocTableWords];

struct NoAllocDevice {
  bool ready = false;
  uint32_t* scratch = nullptr;
  uint32_t* tables = nullptr;
};
std::mutex g_noalloc_mu;
NoAllocDevice g_noalloc_dev[64];

// Once per device, with that device current: resolve the device addresses of
// the static arrays (host code cannot use their names as pointers) and fill
// the power tables. The copy goes through the legacy default stream, and the
// set-up waits for it to finish before any call uses the tables.
int noalloc_setup(int dev, NoAllocDevice** out) {
  std::lock_guard<std::mutex> lk(g_noalloc_mu);
  NoAllocDevice& d = g_noalloc_dev[dev];
  if (!d.ready) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) {
      z0p::host::set_reason(std::string("cudaGetSymbolAddress(scratch): ") + cudaGetErrorString(e));
      return Z0P_ERR_CUDA;
    }
    d.scratch = static_cast<uint32_t*>(p);
    e = cudaGetSymbolAddress(&p, g_noalloc_tables);
    if (e != cudaSuccess) {
      z0p::host::set_reason(std::string("cudaGetSymbolAddress(tables): ") + cudaGetErrorString(e));
      return Z0P_ERR_CUDA;
    }
    d.tables = static_cast<uint32_t*>(p);
    using namespace z0p::host;
    std::vector<uint32_t> t(kNoAllocTableWords);
    uint32_t* w_lo = t.data();
    uint32_t* w_hi = w_lo + (1u << 14);
    uint32_t* g_lo = w_hi + (1u << 13);
    uint32_t* g_hi = g_lo + (1u << 12);
    const uint32_t omega = two_adic_generator(27);
    uint32_t x = 1;
    for (uint32_t i = 0; i < (1u << 14); i++) { w_lo[i] = to_mont(x); x = fmul(x, omega); }
    const uint32_t wstep = fpow(omega, 1u << 14);
    x = 1;
    for (uint32_t i = 0; i < (1u << 13); i++) { w_hi[i] = to_mont(x); x = fmul(x, wstep); }
    x = 1;
    for (uint32_t i = 0; i < (1u << 12); i++) { g_lo[i] = to_mont(x); x = fmul(x, GENERATOR); }
    const uint32_t gstep = fpow(GENERATOR, 1u << 12);
    x = 1;
    for (uint32_t i = 0; i < (1u << 15); i++) { g_hi[i] = to_mont(x); x = fmul(x, gstep); }
    e = cudaMemcpyToSymbol(g_noalloc_tables, t.data(), t.size() * sizeof(uint32_t));
    // A copy from pageable memory may return before its DMA has landed, and a
    // caller's non-blocking stream is not ordered after the legacy stream: wait
    // for the tables here, before any call can enqueue work that reads them.
    if (e == cudaSuccess) e = cudaStreamSynchronize(0);
    if (e != cudaSuccess) {
      z0p::host::set_reason(std::string("cudaMemcpyToSymbol(tables): ") + cudaGetErrorString(e));
      return Z0P_ERR_CUDA;
    }
    d.ready = true;
  }
  *out = &d;
  return Z0P_OK;
}

}  // namespace

extern "C" int z0p_gpu_rs_extend_noalloc(const uint32_t* d_values, uint64_t n, uint64_t batch,
                                         uint64_t blowup, uint32_t* d_out, void* stream) {
  using namespace z0p;
  // The argument, domain and blowup checks are z0p_gpu_rs_extend's, with its codes.
  if (!d_values || !d_out || batch == 0 || batch > 65535) return Z0P_ERR_INVALID_ARGUMENT;
  if (!host::is_pow2(n) || n > host::MAX_DOMAIN) return Z0P_ERR_INVALID_DOMAIN_SIZE;
  if (!host::is_pow2(blowup)) return Z0P_ERR_INVALID_BLOWUP;
  if (n * blowup > host::MAX_DOMAIN || batch * blowup > 65535) {
    host::set_reason("z0p_gpu_rs_extend_noalloc: batch * blowup exceeds the 65535 transforms "
                     "of one launch, or n * blowup exceeds the largest domain");
    return Z0P_ERR_INVALID_DOMAIN_SIZE;
  }
  // Only this limit is particular to the static scratch.
  if (n * blowup > kNoAllocMaxElems || n * batch * blowup > kNoAllocMaxElems) {
    host::set_reason("z0p_gpu_rs_extend_noalloc: n * batch * blowup exceeds the static scratch "
                     "limit of 1048576 output elements");
    return Z0P_ERR_UNSUPPORTED;
  }
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess || dev < 0 || dev >= 64) {
    host::set_reason("z0p_gpu_rs_extend_noalloc: no usable current CUDA device");
    return Z0P_ERR_CUDA;
  }
  NoAllocDevice* d = nullptr;
  int rc = noalloc_setup(dev, &d);
  if (rc != Z0P_OK) return rc;
  Tables tb;
  tb.w_lo = d->tables;
  tb.w_hi = d->tables + (1u << 14);
  tb.g_lo = d->tables + (1u << 14) + (1u << 13);
  tb.g_hi = d->tables + (1u << 14) + (1u << 13) + (1u << 12);
  uint32_t* coeffs = d->scratch;
  uint32_t* four_step = d->scratch + kNoAllocMaxElems;
  uint32_t* coset_major = d->scratch + 2 * kNoAllocMaxElems;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const uint32_t logn = host::log2u(n), logb = host::log2u(blowup);
  NttPlan ip;
  ip.logn = logn;
  ip.batch = (uint32_t)batch;
  ip.inverse = 1;
  ip.post_gamma = 1;
  e = launch::ntt(st, tb, ip, d_values, coeffs, four_step);
  NttPlan lp;
  lp.logn = logn;
  lp.batch = (uint32_t)(batch * blowup);
  lp.in_div = (uint32_t)blowup;
  lp.twist_mod = (uint32_t)blowup;
  lp.twist_shift = 27 - (logn + logb);
  if (e == cudaSuccess) e = launch::ntt(st, tb, lp, coeffs, coset_major, four_step);
  if (e == cudaSuccess) e = launch::coset_to_natural(st, coset_major, d_out, logn, logb, batch);
  if (e != cudaSuccess) {
    host::set_reason(std::string("z0p_gpu_rs_extend_noalloc: ") + cudaGetErrorString(e));
    return Z0P_ERR_CUDA;
  }
  return Z0P_OK;
}
