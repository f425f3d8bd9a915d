// Device arithmetic for the z0p GB300 prover: BabyBear in Montgomery form,
// the Fp4 tower and the BLAKE3 compression function.
//
// Representation rule used by every kernel: data values (trace, LDE,
// composition and FRI layer values) stay canonical (< p) because they are
// hashed and serialised byte-exactly; constants and derived denominators
// (twiddles, coset points, challenges, inverses) are held in Montgomery form
// (x * 2^32 mod p). mmul(canonical, montgomery) then yields a canonical
// product in one reduction, so no conversions appear on the hot paths.
#pragma once
#include <cstdint>

#include "kernels.h"

namespace z0p {

constexpr uint32_t kP = 0x78000001u;      // 2^31 - 2^27 + 1 (src/babybear.rs:26)
constexpr uint32_t kPInv = 0x88000001u;   // p^-1 mod 2^32
constexpr uint32_t kR = 0x0FFFFFFEu;      // 2^32 mod p  (Montgomery one)
constexpr uint32_t kR2 = 0x45DDDDE3u;     // 2^64 mod p
constexpr uint32_t k11R = 939524073u;     // 11 * 2^32 mod p (Fp2 non-residue)
constexpr int kRootBits = 27;             // omega = 31^((p-1)/2^27)
constexpr uint32_t kOmega4M = 473486609u; // omega_4 = 31^((p-1)/4) = 1728404513, Montgomery form
constexpr int kWLoBits = 14;
constexpr int kWHiBits = kRootBits - kWLoBits;
constexpr int kGLoBits = 12;
constexpr int kGHiBits = kRootBits - kGLoBits;


// Final corrections as an unsigned min: with x < 2p < 2^32, exactly one of
// x and x - p (or x + p) lies in [0, p), and the other wraps above 2^32 - p.
__device__ __forceinline__ uint32_t fadd(uint32_t a, uint32_t b) {
  uint32_t s = a + b;
  return min(s, s - kP);
}
__device__ __forceinline__ uint32_t fsub(uint32_t a, uint32_t b) {
  uint32_t d = a - b;
  return min(d, d + kP);
}
__device__ __forceinline__ uint32_t fneg(uint32_t a) { return a ? kP - a : 0u; }
// a - b + p for a, b < p: in (0, 2p), not reduced. Valid only as an operand
// of mmul beside an operand below p (the product stays below p * 2^32).
__device__ __forceinline__ uint32_t fsub_lazy(uint32_t a, uint32_t b) { return a + kP - b; }
__device__ __forceinline__ uint32_t fhalve(uint32_t a) { return (a + ((a & 1u) ? kP : 0u)) >> 1; }

// Montgomery product a*b*2^-32 mod p for a*b < p * 2^32, e.g. a, b < p or
// a < 2p and b < p (Montgomery 1985, with the signed "hi - hi(m p)"
// reduction so no 64-bit addition is needed).
__device__ __forceinline__ uint32_t mmul(uint32_t a, uint32_t b) {
  uint32_t lo = a * b;
  uint32_t hi = __umulhi(a, b);
  uint32_t m = lo * kPInv;
  uint32_t mp = __umulhi(m, kP);
  uint32_t r = hi - mp;  // hi, mp < p: r in (-p, p)
  return min(r, r + kP);
}
// (a0 b0 + a1 b1) * 2^-32 mod p for canonical a_i and b_i < p: the sum of
// the two products is below 2p^2 < p * 2^32, so one signed Montgomery
// reduction covers both (lazy reduction of a two-term dot product).
__device__ __forceinline__ uint32_t mdot2(uint32_t a0, uint32_t b0, uint32_t a1, uint32_t b1) {
  uint64_t t = (uint64_t)a0 * b0 + (uint64_t)a1 * b1;
  uint32_t lo = (uint32_t)t, hi = (uint32_t)(t >> 32);
  uint32_t m = lo * kPInv;
  uint32_t mp = __umulhi(m, kP);
  uint32_t r = hi - mp;
  return min(r, r + kP);
}
// (a0 b0 + a1 b1 + a2 b2 + a3 b3) * 2^-32 mod p for a_i, b_i < p: the sum is
// below 4p^2 < 2^64, so one Montgomery reduction covers the four products.
// Its high word is below 1.9p; reducing it once first keeps the signed
// reduction in (-p, p).
__device__ __forceinline__ uint32_t mdot4(uint32_t a0, uint32_t b0, uint32_t a1, uint32_t b1,
                                          uint32_t a2, uint32_t b2, uint32_t a3, uint32_t b3) {
  uint64_t t = (uint64_t)a0 * b0 + (uint64_t)a1 * b1 + (uint64_t)a2 * b2 + (uint64_t)a3 * b3;
  uint32_t lo = (uint32_t)t, hi = (uint32_t)(t >> 32);
  hi = min(hi, hi - kP);
  uint32_t m = lo * kPInv;
  uint32_t mp = __umulhi(m, kP);
  uint32_t r = hi - mp;
  return min(r, r + kP);
}
// a * w mod p for any a < 2^32 and canonical w, with wq = floor(w 2^32 / p)
// precomputed (Shoup's product): q = floor(a wq / 2^32) leaves a w - q p in
// [0, 2p), so one correction gives the canonical product.
__device__ __forceinline__ uint32_t shoup_mul(uint32_t a, uint32_t w, uint32_t wq) {
  uint32_t q = __umulhi(a, wq);
  uint32_t r = a * w - q * kP;
  return min(r, r - kP);
}
// (w, floor(w 2^32 / p)) for canonical w.
__device__ __forceinline__ uint2 shoup_pair(uint32_t w) {
  return make_uint2(w, (uint32_t)(((uint64_t)w << 32) / kP));
}
// Canonical x canonical -> canonical.
__device__ __forceinline__ uint32_t fmul(uint32_t a, uint32_t b) { return mmul(mmul(a, b), kR2); }
__device__ __forceinline__ uint32_t to_mont(uint32_t a) { return mmul(a, kR2); }
__device__ __forceinline__ uint32_t from_mont(uint32_t a) { return mmul(a, 1u); }

// x^(p-2) in the Montgomery domain (inverse, zero maps to zero as in
// src/babybear.rs:167-169). p - 2 = 0b1110 followed by 27 ones: a 3-bit
// window chain of 30 squarings and 11 multiplications.
__device__ __forceinline__ uint32_t minv(uint32_t x) {
  uint32_t x2 = mmul(x, x);
  uint32_t x3 = mmul(x2, x);
  uint32_t x6 = mmul(x3, x3);
  uint32_t x7 = mmul(x6, x);
  uint32_t r = mmul(x7, x7);  // exponent 0b1110
#pragma unroll
  for (int g = 0; g < 9; g++) {
    r = mmul(r, r);
    r = mmul(r, r);
    r = mmul(r, r);
    r = mmul(r, x7);
  }
  return r;
}

// Montgomery-trick batch inversion of K Montgomery-form values in registers;
// zeros stay zero and are skipped (src/babybear.rs:307-331 semantics).
template <int K>
__device__ __forceinline__ void batch_minv(uint32_t (&v)[K]) {
  uint32_t prefix[K];
  uint32_t acc = kR;
#pragma unroll
  for (int i = 0; i < K; i++) {
    if (v[i] != 0u) acc = mmul(acc, v[i]);
    prefix[i] = acc;
  }
  uint32_t suffix = minv(acc);
#pragma unroll
  for (int i = K - 1; i >= 0; i--) {
    uint32_t x = v[i];
    if (x == 0u) continue;
    uint32_t before = i == 0 ? kR : prefix[i - 1];
    v[i] = mmul(before, suffix);
    suffix = mmul(suffix, x);
  }
}

// omega_{2^27}^e (Montgomery form), e taken mod 2^27.
__device__ __forceinline__ uint32_t root_pow(const Tables& t, uint32_t e) {
  e &= (1u << kRootBits) - 1u;
  return mmul(__ldg(t.w_hi + (e >> kWLoBits)), __ldg(t.w_lo + (e & ((1u << kWLoBits) - 1u))));
}
// 31^i (Montgomery form), i < 2^27.
__device__ __forceinline__ uint32_t gamma_pow(const Tables& t, uint32_t i) {
  return mmul(__ldg(t.g_hi + (i >> kGLoBits)), __ldg(t.g_lo + (i & ((1u << kGLoBits) - 1u))));
}

__device__ __forceinline__ uint32_t brev_bits(uint32_t x, int bits) {
  return bits ? (__brev(x) >> (32 - bits)) : 0u;
}

// ----------------------------------------------------------------- Fp4 ----
// a + b u + c v + d uv, u^2 = 11, v^2 = u (src/ext4.rs:24).
struct E4 {
  uint32_t c[4];
};

__device__ __forceinline__ E4 e4_add(const E4& a, const E4& b) {
  E4 r;
#pragma unroll
  for (int i = 0; i < 4; i++) r.c[i] = fadd(a.c[i], b.c[i]);
  return r;
}
__device__ __forceinline__ E4 e4_sub(const E4& a, const E4& b) {
  E4 r;
#pragma unroll
  for (int i = 0; i < 4; i++) r.c[i] = fsub(a.c[i], b.c[i]);
  return r;
}
// Unreduced sums and differences (components below 2p), for operands of
// e4_mul_base only (see fsub_lazy).
__device__ __forceinline__ E4 e4_add_lazy(const E4& a, const E4& b) {
  E4 r;
#pragma unroll
  for (int i = 0; i < 4; i++) r.c[i] = a.c[i] + b.c[i];
  return r;
}
__device__ __forceinline__ E4 e4_sub_lazy(const E4& a, const E4& b) {
  E4 r;
#pragma unroll
  for (int i = 0; i < 4; i++) r.c[i] = fsub_lazy(a.c[i], b.c[i]);
  return r;
}
__device__ __forceinline__ E4 e4_quarter(const E4& a) {
  E4 r;
#pragma unroll
  for (int i = 0; i < 4; i++) r.c[i] = fhalve(fhalve(a.c[i]));
  return r;
}
// Fp4 (components below 2p) times a Montgomery-form base scalar -> canonical.
__device__ __forceinline__ E4 e4_mul_base(const E4& a, uint32_t sM) {
  E4 r;
#pragma unroll
  for (int i = 0; i < 4; i++) r.c[i] = mmul(a.c[i], sM);
  return r;
}
// canonical Fp4 times Montgomery-form Fp4 -> canonical (src/ext4.rs:106-117:
// Karatsuba over Fp2 with the u-twist on the d-part).
__device__ __forceinline__ void fp2_mul_cm(uint32_t x0, uint32_t x1, uint32_t y0, uint32_t y1,
                                           uint32_t& o0, uint32_t& o1) {
  uint32_t real = mmul(x0, y0);
  uint32_t imag = mmul(x1, y1);
  uint32_t cross = fsub(fsub(mmul(fadd(x0, x1), fadd(y0, y1)), real), imag);
  o0 = fadd(real, mmul(imag, k11R));
  o1 = cross;
}
__device__ __forceinline__ E4 e4_mul_cm(const E4& v, const E4& rM) {
  uint32_t ac0, ac1, bd0, bd1, t0, t1;
  fp2_mul_cm(v.c[0], v.c[1], rM.c[0], rM.c[1], ac0, ac1);
  fp2_mul_cm(v.c[2], v.c[3], rM.c[2], rM.c[3], bd0, bd1);
  fp2_mul_cm(fadd(v.c[0], v.c[2]), fadd(v.c[1], v.c[3]), fadd(rM.c[0], rM.c[2]),
             fadd(rM.c[1], rM.c[3]), t0, t1);
  E4 r;
  r.c[0] = fadd(ac0, mmul(bd1, k11R));
  r.c[1] = fadd(ac1, bd0);
  r.c[2] = fsub(fsub(t0, ac0), bd0);
  r.c[3] = fsub(fsub(t1, ac1), bd1);
  return r;
}

// Canonical Fp4 times a constant r, given r's product table T (Montgomery
// form): coordinate c of v*r is sum_i v_i T[c][i] with
//   T[0] = (r0, 11 r1, 11 r3, 11 r2)   T[1] = (r1, r0, r2, 11 r3)
//   T[2] = (r2, 11 r3, r0, 11 r1)      T[3] = (r3, r2, r1, r0)
// (the tower product of src/ext4.rs:106-117 written out), i.e. two lazy
// two-term reductions per coordinate.
__device__ __forceinline__ E4 e4_mul_tab(const E4& v, const uint32_t (&T)[4][4]) {
  E4 r;
#pragma unroll
  for (int c = 0; c < 4; c++)
    r.c[c] = mdot4(v.c[0], T[c][0], v.c[1], T[c][1], v.c[2], T[c][2], v.c[3], T[c][3]);
  return r;
}

// ------------------------------------------------------------- BLAKE3 ----
// Compression function per the BLAKE3 specification (src/hash.rs:93-133).
constexpr uint32_t kIV0 = 0x6A09E667u, kIV1 = 0xBB67AE85u, kIV2 = 0x3C6EF372u,
                   kIV3 = 0xA54FF53Au, kIV4 = 0x510E527Fu, kIV5 = 0x9B05688Cu,
                   kIV6 = 0x1F83D9ABu, kIV7 = 0x5BE0CD19u;
constexpr uint32_t kChunkStart = 1u, kChunkEnd = 2u, kParent = 4u, kRoot = 8u;

__device__ __forceinline__ uint32_t rotr16(uint32_t x) { return __byte_perm(x, 0, 0x1032); }
__device__ __forceinline__ uint32_t rotr8(uint32_t x) { return __byte_perm(x, 0, 0x0321); }
__device__ __forceinline__ uint32_t rotr12(uint32_t x) { return __funnelshift_r(x, x, 12); }
__device__ __forceinline__ uint32_t rotr7(uint32_t x) { return __funnelshift_r(x, x, 7); }

// A one the compiler cannot fold, so that x * k_unit + y stays a multiply-add.
// The G function is bound by the integer ALU pipe (additions, XORs, byte
// permutes and funnel shifts all issue there). Issuing three of its four
// additions as multiply-adds by one moves them to the FMA pipe. A GB300
// probe (311,296 threads, each hashing two chains of 64 nodes) measured
// 35.9 -> 38.6 G compressions/s with this mix and identical digests. Moving all four
// measured 37.5; moving only the c-additions measured 34.8. Z0P_G_ALU keeps
// every addition on the ALU pipe (the tree-top kernel measured faster so).
static __constant__ uint32_t k_unit = 1u;

__device__ __forceinline__ uint32_t mad_unit(uint32_t x, uint32_t y) {
  uint32_t r;
  asm("mad.lo.u32 %0, %1, %2, %3;" : "=r"(r) : "r"(x), "r"(k_unit), "r"(y));
  return r;
}

#define Z0P_G(a, b, c, d, x, y)    \
  do {                             \
    a = mad_unit(b, a + (x));      \
    d = rotr16(d ^ a);             \
    c = c + d;                     \
    b = rotr12(b ^ c);             \
    a = mad_unit(b, a + (y));      \
    d = rotr8(d ^ a);              \
    c = mad_unit(d, c);            \
    b = rotr7(b ^ c);              \
  } while (0)

#define Z0P_G_ALU(a, b, c, d, x, y) \
  do {                              \
    a = a + b + (x);                \
    d = rotr16(d ^ a);              \
    c = c + d;                      \
    b = rotr12(b ^ c);              \
    a = a + b + (y);                \
    d = rotr8(d ^ a);               \
    c = c + d;                      \
    b = rotr7(b ^ c);               \
  } while (0)

// out[0..8] = first 8 words of the compression output (the chaining value /
// root digest). m is consumed (permuted in place). kMad selects the G step
// with multiply-adds (true) or all additions on the ALU pipe (false); both
// compute the same function.
template <bool kMad = true>
__device__ __forceinline__ void blake3_compress(const uint32_t cv[8], uint32_t m[16],
                                                uint32_t counter_lo, uint32_t counter_hi,
                                                uint32_t block_len, uint32_t flags,
                                                uint32_t out[8]) {
  uint32_t s0 = cv[0], s1 = cv[1], s2 = cv[2], s3 = cv[3];
  uint32_t s4 = cv[4], s5 = cv[5], s6 = cv[6], s7 = cv[7];
  uint32_t s8 = kIV0, s9 = kIV1, s10 = kIV2, s11 = kIV3;
  uint32_t s12 = counter_lo, s13 = counter_hi, s14 = block_len, s15 = flags;
#pragma unroll
  for (int r = 0; r < 7; r++) {
    if (kMad) {
      Z0P_G(s0, s4, s8, s12, m[0], m[1]);
      Z0P_G(s1, s5, s9, s13, m[2], m[3]);
      Z0P_G(s2, s6, s10, s14, m[4], m[5]);
      Z0P_G(s3, s7, s11, s15, m[6], m[7]);
      Z0P_G(s0, s5, s10, s15, m[8], m[9]);
      Z0P_G(s1, s6, s11, s12, m[10], m[11]);
      Z0P_G(s2, s7, s8, s13, m[12], m[13]);
      Z0P_G(s3, s4, s9, s14, m[14], m[15]);
    } else {
      Z0P_G_ALU(s0, s4, s8, s12, m[0], m[1]);
      Z0P_G_ALU(s1, s5, s9, s13, m[2], m[3]);
      Z0P_G_ALU(s2, s6, s10, s14, m[4], m[5]);
      Z0P_G_ALU(s3, s7, s11, s15, m[6], m[7]);
      Z0P_G_ALU(s0, s5, s10, s15, m[8], m[9]);
      Z0P_G_ALU(s1, s6, s11, s12, m[10], m[11]);
      Z0P_G_ALU(s2, s7, s8, s13, m[12], m[13]);
      Z0P_G_ALU(s3, s4, s9, s14, m[14], m[15]);
    }
    if (r < 6) {  // message permutation (src/hash.rs:30)
      uint32_t t0 = m[2], t1 = m[6], t2 = m[3], t3 = m[10], t4 = m[7], t5 = m[0], t6 = m[4],
               t7 = m[13], t8 = m[1], t9 = m[11], t10 = m[12], t11 = m[5], t12 = m[9],
               t13 = m[14], t14 = m[15], t15 = m[8];
      m[0] = t0; m[1] = t1; m[2] = t2; m[3] = t3; m[4] = t4; m[5] = t5; m[6] = t6; m[7] = t7;
      m[8] = t8; m[9] = t9; m[10] = t10; m[11] = t11; m[12] = t12; m[13] = t13; m[14] = t14;
      m[15] = t15;
    }
  }
  out[0] = s0 ^ s8; out[1] = s1 ^ s9; out[2] = s2 ^ s10; out[3] = s3 ^ s11;
  out[4] = s4 ^ s12; out[5] = s5 ^ s13; out[6] = s6 ^ s14; out[7] = s7 ^ s15;
}

__device__ __forceinline__ void iv_words(uint32_t cv[8]) {
  cv[0] = kIV0; cv[1] = kIV1; cv[2] = kIV2; cv[3] = kIV3;
  cv[4] = kIV4; cv[5] = kIV5; cv[6] = kIV6; cv[7] = kIV7;
}

// BLAKE3 root of one full 64-byte block (src/hash.rs:388-397).
__device__ __forceinline__ void blake3_leaf64(uint32_t m[16], uint32_t out[8]) {
  uint32_t cv[8];
  iv_words(cv);
  blake3_compress(cv, m, 0u, 0u, 64u, kChunkStart | kChunkEnd | kRoot, out);
}

// BLAKE3(0x01 || l || r): 65 bytes, two compressions (src/hash.rs:417-443).
template <bool kMad = true>
__device__ __forceinline__ void blake3_node(const uint32_t l[8], const uint32_t r[8],
                                            uint32_t out[8]) {
  uint32_t m[16];
  m[0] = 0x01u | (l[0] << 8);
#pragma unroll
  for (int i = 1; i < 8; i++) m[i] = __funnelshift_l(l[i - 1], l[i], 8);
  m[8] = __funnelshift_l(l[7], r[0], 8);
#pragma unroll
  for (int i = 1; i < 8; i++) m[8 + i] = __funnelshift_l(r[i - 1], r[i], 8);
  uint32_t cv[8], mid[8];
  iv_words(cv);
  blake3_compress<kMad>(cv, m, 0u, 0u, 64u, kChunkStart, mid);
  uint32_t m2[16];
  m2[0] = r[7] >> 24;
#pragma unroll
  for (int i = 1; i < 16; i++) m2[i] = 0u;
  blake3_compress<kMad>(mid, m2, 0u, 0u, 1u, kChunkEnd | kRoot, out);
}

// BLAKE3(0x00 || data) for data of `nwords` 32-bit words (<= 25, i.e. at most
// two blocks): the leaf digest of src/hash.rs:351-381 for short rows.
template <int NW>
__device__ __forceinline__ void blake3_prefixed_leaf(const uint32_t (&d)[NW], uint32_t out[8]) {
  static_assert(NW >= 1 && NW <= 31, "row must fit two BLAKE3 blocks");
  constexpr int kLen = 4 * NW + 1;
  constexpr int kBlocks = (kLen + 63) / 64;
  // byte stream: 0x00, d bytes; word w = (d[w-1] >> 24) | (d[w] << 8)
  uint32_t pre[32];
#pragma unroll
  for (int w = 0; w < 32; w++) {
    uint32_t lo = (w >= 1 && w - 1 < NW) ? d[w - 1] : 0u;
    uint32_t hi = (w < NW) ? d[w] : 0u;
    pre[w] = __funnelshift_l(lo, hi, 8);
  }
  uint32_t cv[8];
  iv_words(cv);
#pragma unroll
  for (int b = 0; b < kBlocks; b++) {
    uint32_t m[16];
#pragma unroll
    for (int i = 0; i < 16; i++) m[i] = pre[16 * b + i];
    uint32_t flags = (b == 0 ? kChunkStart : 0u) | (b == kBlocks - 1 ? (kChunkEnd | kRoot) : 0u);
    uint32_t bl = b == kBlocks - 1 ? (uint32_t)(kLen - 64 * b) : 64u;
    uint32_t o[8];
    blake3_compress(cv, m, 0u, 0u, bl, flags, o);
#pragma unroll
    for (int i = 0; i < 8; i++) cv[i] = o[i];
  }
#pragma unroll
  for (int i = 0; i < 8; i++) out[i] = cv[i];
}

// BLAKE3 of 0x00 || ncols little-endian words (a Merkle leaf over one row,
// src/merkle.rs:93-110; ncols <= 25, so one or two blocks). w[ncols..32)
// must be zero.
__device__ __forceinline__ void row_leaf_digest(const uint32_t (&w)[32], uint32_t ncols,
                                                uint32_t o[8]) {
  // 0x00 || row: word i = (w[i-1] >> 24) | (w[i] << 8).
  const uint32_t len = 4u * ncols + 1u;
  uint32_t cv[8];
  iv_words(cv);
  uint32_t blk[16];
#pragma unroll
  for (int i = 0; i < 16; i++) blk[i] = __funnelshift_l(i ? w[i - 1] : 0u, w[i], 8);
  const bool one = len <= 64u;
  blake3_compress(cv, blk, 0u, 0u, one ? len : 64u,
                  one ? (kChunkStart | kChunkEnd | kRoot) : kChunkStart, o);
  if (!one) {
#pragma unroll
    for (int i = 0; i < 16; i++) blk[i] = __funnelshift_l(w[15 + i], w[16 + i], 8);
    uint32_t o2[8];
    blake3_compress(o, blk, 0u, 0u, len - 64u, kChunkEnd | kRoot, o2);
#pragma unroll
    for (int i = 0; i < 8; i++) o[i] = o2[i];
  }
}

}  // namespace z0p
