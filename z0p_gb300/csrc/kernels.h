// Launchers for the z0p GB300 kernels (host-callable, C++ linkage).
// Every launcher enqueues on `st` and returns the launch status; none of them
// synchronises. Pointers are device pointers unless stated otherwise.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

namespace z0p {

struct Tables {
  const uint32_t* w_lo;  // omega_{2^27}^i,          i < 2^14 (Montgomery)
  const uint32_t* w_hi;  // omega_{2^27}^(i * 2^14), i < 2^13
  const uint32_t* g_lo;  // 31^i,                    i < 2^12
  const uint32_t* g_hi;  // 31^(i * 2^12),           i < 2^15
};

// Batched NTT of length 2^logn. Transform b reads in + (b / in_div) * n,
// multiplies input i by omega_{2^27}^((j*i) << twist_shift) with
// j = b % twist_mod (a coset twist), transforms forward or inverse, optionally
// multiplies output k by 31^k / n, and writes out + b * n (natural order).
struct NttPlan {
  uint32_t logn = 0;
  uint32_t batch = 1;
  uint32_t inverse = 0;
  uint32_t in_div = 1;
  uint32_t twist_mod = 1;
  uint32_t twist_shift = 0;
  uint32_t post_gamma = 0;
};

struct AirComposeArgs {
  const uint32_t* lde_a;  // coset-major [j][q]
  const uint32_t* lde_b;
  const uint32_t* zinv;   // per coset 1 / (x^N - 1) (Montgomery)
  uint32_t* layer0;       // FRI layer 0, bit-reversed Ext4 values
  uint32_t* leaves;       // layer-0 tree, leaf digests
  uint32_t logN, logB;
  uint32_t a0, b0, b_last;  // canonical
  uint32_t w_last_m;        // omega_N^(N-1) (Montgomery)
  uint32_t alpha[5][4];     // Montgomery
};

struct RangeComposeArgs {
  const uint32_t* lde;     // column-major: column c, coset j, row q at (c*B + j)*N + q
  const uint32_t* zinv;    // per coset 1 / (x^N - 1) (Montgomery)
  const uint32_t* zinv2;   // per coset 1 / (x^N - 1) * 2^64 mod p
  const uint32_t* alphas;  // (n_bits + 2) Ext4 in Montgomery form: decomp, bits..., bound
  uint32_t* layer0;
  uint32_t* leaves;
  uint32_t logN, logB, n_bits;
  uint32_t value;  // canonical
};

struct FoldArgs {
  const uint32_t* in;  // layer values (4 words each), bit-reversed, length 2^logn
  uint32_t* out;       // next layer, length 2^(logn-2)
  uint32_t* leaves;    // next layer's leaf digests (fused variant only)
  uint32_t logn;
  uint32_t ginv_m;     // (31^(4^depth))^-1 (Montgomery)
  uint32_t unit_m;     // two_adic_generator(2) (Montgomery)
  uint32_t ch[3][4];   // fold challenges (Montgomery)
};

namespace launch {

// Number of kernel launches issued by this library in this process.
uint64_t launch_count();
// Optional per-stage timing: when a recorder is installed, every launcher
// brackets its kernels with CUDA events on the launching stream.
struct StageRecorder {
  virtual ~StageRecorder() = default;
  virtual void begin(const char* stage, cudaStream_t st) = 0;
  virtual void end(const char* stage, cudaStream_t st) = 0;
};
void set_recorder(StageRecorder* r);

cudaError_t fib_trace(cudaStream_t st, uint32_t* col_a, uint32_t* col_b, uint32_t n, uint32_t a0,
                      uint32_t b0, const uint32_t mats[32][4]);
cudaError_t fill_constant_columns(cudaStream_t st, uint32_t* cols, uint32_t n, uint32_t ncols,
                                  const uint32_t* h_values);
cudaError_t ntt(cudaStream_t st, const Tables& tb, const NttPlan& plan, const uint32_t* in,
                uint32_t* out, uint32_t* scratch);
cudaError_t coset_zinv(cudaStream_t st, const Tables& tb, uint32_t* zinv, uint32_t* zinv2,
                       uint32_t logB, uint32_t gamma_n_m);
cudaError_t air_trace_leaves(cudaStream_t st, const uint32_t* lde_a, const uint32_t* lde_b,
                             uint32_t* leaves, uint32_t logN, uint32_t logB);
cudaError_t range_trace_leaves(cudaStream_t st, const uint32_t* lde, uint32_t* leaves,
                               uint32_t logN, uint32_t logB, uint32_t ncols);
// Builds every level above the leaves of a tree stored level-contiguous
// (level l at digest offset 2L - 2(L >> l), L = leaves, power of two).
cudaError_t merkle_build(cudaStream_t st, uint32_t* tree, uint64_t leaves);
cudaError_t air_compose_leaves(cudaStream_t st, const Tables& tb, const AirComposeArgs& a);
cudaError_t range_compose_leaves(cudaStream_t st, const Tables& tb, const RangeComposeArgs& a);
// Folds one FRI layer; hashes the next layer's 64-byte leaves when it has a
// multiple of four values, its 0x00-prefixed 16-byte leaves otherwise.
cudaError_t fri_fold(cudaStream_t st, const Tables& tb, const FoldArgs& a);
// Leaf digests of an FRI layer held in memory (64-byte quads or 16-byte values).
cudaError_t layer_leaves(cudaStream_t st, const uint32_t* values, uint64_t len, uint32_t* leaves);
cudaError_t merkle_flat64_leaves(cudaStream_t st, const uint32_t* flat, uint64_t nleaves,
                                 uint32_t* leaves);
// Minimum-nonce proof-of-work search; `state` is 3 device words of scratch:
// best (u64), next chunk (u64), status (u32, 1 = iteration cap reached).
cudaError_t grind(cudaStream_t st, const uint8_t* head, uint32_t head_len, uint32_t bits,
                  unsigned long long* state, uint64_t max_nonces);
bool grind_supports(uint32_t head_len);
// Reorders `batch` coset-major LDEs ([j][q]) into natural order ([B q + j]).
cudaError_t coset_to_natural(cudaStream_t st, const uint32_t* in, uint32_t* out, uint32_t logN,
                             uint32_t logB, uint64_t batch);
// out[i] = 16 bytes at device address addr[i].
cudaError_t gather16(cudaStream_t st, const uint64_t* addr, void* out, uint32_t n);
// out[i] = 4 bytes at device address addr[i].
cudaError_t gather4(cudaStream_t st, const uint64_t* addr, uint32_t* out, uint32_t n);

}  // namespace launch
}  // namespace z0p
