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
  // NTT stage twiddles (w, floor(w 2^32 / p)), w = omega_{2^L}^(+-i)
  // canonical, i < 2^(L-1), for L = 1..13: the forward table at
  // stw + 2^(L-1) - 1, the inverse one kStwInverse entries further. Null:
  // the transforms compute them.
  const uint2* stw = nullptr;
  // Device-mapped status word: a kernel whose bounded wait gave up sets it
  // (nonzero) and returns; the host checks it after synchronising. Null: no
  // report.
  unsigned int* fault = nullptr;
};
constexpr uint32_t kStwInverse = 1u << 13;

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
  // Non-null: every input word is checked on load, and a value >= p sets
  // *bad (a caller's columns; the C boundary takes canonical elements).
  unsigned int* bad = nullptr;
  // Nonzero: input i is multiplied by 31^i on load (coefficients of
  // fri::commit, src/ntt.rs:353-358); non-canonical inputs read as 0.
  uint32_t pre_gamma = 0;
};

// Column B of the Fibonacci trace is never transformed: on the LDE,
// B(x) = A(omega_N x) + C_j / (x - w_last) with C_j constant on coset j
// (src/air.rs:806-844, linked_lde), so kernels that need B derive it from A.
// Values that change from one proof to the next on the same shape: the
// statement, the Fiat-Shamir challenges in the forms the kernels use. Each
// context owns one slot of them in constant memory, filled by a stream-
// ordered copy before the kernels that read it, so a captured launch
// sequence replays unchanged for every proof of its shape.
struct ProofConsts {
  uint32_t a0, b0, b_last;  // AIR statement (canonical)
  uint32_t coeff;           // linked-column coefficient (B[N-1] - a0) w_last / N
  uint32_t value;           // range statement
  uint32_t kc[4];           // alpha_0 * (-coeff): the composition's constant term
  // Composition weights, coordinate c at [c][k] (Montgomery): alpha_1,
  // alpha_2 and alpha_3 times omega_N^-1, alpha_4 ([c][0] unused).
  uint32_t alpha[4][5];
  uint32_t tab[3][4][4];    // a large fold's e4_mul_tab tables of r_k / 4
};
constexpr int kConstSlots = 168;  // 168 x 308 bytes of the 64 KiB constant bank
// Largest proof group one launch sequence covers (per-proof counters and PoW
// states are sized for it).
constexpr int kMaxGroup = 64;

// Words of one fold's challenge tables (ProofConsts::tab) and of one PoW head
// (47 bytes, little-endian words, zero padded), per proof.
constexpr uint32_t kFoldTabWords = 48;
constexpr uint32_t kPowHeadWords = 16;

// Per coset j of an LDE of 2^logB cosets (x^N = 31^N omega_B^j, gamma_n_m =
// 31^N in Montgomery form): zinv = 1/(x^N - 1) (Montgomery), zinv2 = zinv *
// 2^32, and, when cb is non-null, cb = coeff * (x^N - 1) (canonical; coeff
// from the slot), the linked-column constant.
struct ZinvArgs {
  uint32_t* zinv;
  uint32_t* zinv2;
  uint32_t logB;
  uint32_t gamma_n_m;
  uint32_t* cb;
  uint32_t slot;
};

struct AirComposeArgs {
  const uint32_t* lde_a;  // coset-major [j][q]
  const uint32_t* cb;     // per coset C_j (canonical)
  const uint32_t* zinv;   // per coset 1 / (x^N - 1) (Montgomery)
  const uint32_t* tinv;   // coset-major 1 / (x - w_last) (Montgomery), from air_trace_leaves
  uint32_t* layer0;       // FRI layer 0, bit-reversed Ext4 values
  uint32_t* leaves;       // layer-0 tree, leaf digests
  uint32_t logN, logB;
  uint32_t w_last_m;      // omega_N^(N-1) (Montgomery)
  uint32_t slot;          // ProofConsts slot of the first proof: statement, alphas, kc
  uint64_t layer_stride = 0, tree_stride = 0;  // per-proof strides (words) of layer0 / leaves
  // Fused layer-0 tree (air_compose_leaves, trees of <= kFuseMaxLeaves
  // leaves): one zero counter per proof; the launch then hashes the tree up
  // to level `top` and writes that level to cap (proof k at k * cap_stride).
  unsigned int* counter = nullptr;
  uint32_t top = 0;
  uint32_t* cap = nullptr;
  uint64_t cap_stride = 0;
  // A launch of one proof reads its statement and weights from here (kernel
  // parameters, fixed offsets) rather than from its constant slot, which is
  // indexed at run time; groups read the slots.
  uint32_t a0 = 0, b0 = 0, b_last = 0;
  uint32_t kc[4] = {};
  uint32_t alpha[4][5] = {};
};

struct RangeComposeArgs {
  const uint32_t* lde;     // column-major: column c, coset j, row q at (c*B + j)*N + q
  const uint32_t* zinv;    // per coset 1 / (x^N - 1) (Montgomery)
  const uint32_t* zinv2;   // per coset 1 / (x^N - 1) * 2^64 mod p
  const uint32_t* alphas;  // (n_bits + 2) Ext4 in Montgomery form: decomp, bits..., bound
  uint32_t* layer0;
  uint32_t* leaves;
  uint32_t logN, logB, n_bits;  // logN: rows per coset of the LDE (padded when masked)
  uint32_t slot;  // ProofConsts slot of the first proof: the claimed value
  uint64_t layer_stride = 0, tree_stride = 0;  // per-proof strides (words) of layer0 / leaves
  // zinv / zinv2 hold B x r values, [j][q mod r]: x^n is periodic in q with
  // period r = padded rows / n (1 unpadded).
  uint32_t r = 1;
};

struct FoldArgs {
  const uint32_t* in;  // layer values (4 words each), bit-reversed, length 2^logn
  uint32_t* out;       // next layer, length 2^(logn-2)
  uint32_t* leaves;    // next layer's tree (level-contiguous; leaf digests first)
  uint32_t top = 0;    // the next tree's cap level: subtree levels stop there
  uint32_t* cap = nullptr;  // receives the cap level when the fold reaches it
  uint32_t logn;
  uint32_t ginv_m;     // (31^(4^depth))^-1 (Montgomery)
  uint32_t unit_m;     // two_adic_generator(2) (Montgomery)
  // The fold's challenge tables: small layers (the launches that finish their
  // tree) read them from `tab` (kFoldTabWords per proof, device-visible, e.g.
  // mapped host memory, so no copy is queued before a latency-bound fold);
  // large layers from the constant slots, first proof's at `slot`.
  const uint32_t* tab = nullptr;
  uint32_t slot = 0;
  // Optional gate for a fold queued before its challenges exist (small
  // layers): every CTA first waits until *go == go_epoch (a device-mapped
  // word the host writes after the tables), at most about 2^31 cycles, after
  // which it sets bit 3 of Tables::fault and runs on.
  const unsigned int* go = nullptr;
  unsigned int go_epoch = 0;
  // One zero device word per proof: with it, a small tree is finished up to
  // `top` by the fold's last CTA (nullptr: the fold stops at its subtrees).
  unsigned int* counter = nullptr;
  // Receives a second copy of the output values when the output is the final
  // layer (device-visible, e.g. mapped host memory; nullptr: none).
  uint32_t* final_vals = nullptr;
  // Per-proof strides (words) of in, out, leaves, cap and final_vals for a
  // proof group.
  uint64_t in_stride = 0, out_stride = 0, tree_stride = 0, cap_stride = 0, final_stride = 0;
};

// Openings of one proof, gathered on the device into one block per query.
// Block layout (32-bit words): for each non-final FRI layer d, at layer[d].off,
// the 16 words of the opened quad then steps x 8 words of sibling digests
// (leaf upward); at trace_off, the trace part: for the AIR, twice (row index,
// then row index + B) the 16 words A0 B0 .. A7 B7 of the 8-row leaf and
// tsteps x 8 words of siblings; for the range AIR, the ncol column values of
// the row then tsteps x 8 words of siblings.
constexpr uint32_t kMaxOpenLayers = 16;
struct OpenLayer {
  const uint32_t* values;  // layer values (Ext4, 4 words each)
  const uint32_t* tree;    // level-contiguous tree
  uint64_t leaves;
  uint32_t steps;          // path length (depth - cap drop)
  uint32_t off;            // word offset of this layer inside a query block
};
struct OpenArgs {
  const uint64_t* indices;  // nq FRI query indices (layer-0 positions) per proof
  uint32_t* out;            // nq blocks of `stride` words per proof
  uint32_t nq, nlayers, stride, trace_off;
  OpenLayer layer[kMaxOpenLayers];
  const uint32_t* lde;      // AIR: column A coset-major; range: ncol columns
  const uint32_t* cb;       // AIR: per-coset linked-column constant
  const uint32_t* tinv;     // AIR: 1 / (x - w_last), coset-major
  const uint32_t* ttree;    // trace tree
  uint64_t tleaves;
  uint32_t tsteps, logN, logB;
  uint32_t ncol;            // 0 for the AIR, else the range AIR's column count
  uint32_t no_trace = 0;    // 1: FRI openings only (a FRI commitment on its own)
  // AIR with two committed columns: column B's own LDE (nullptr: linked B)
  // and the next-row distance in LDE index units (0: B).
  const uint32_t* lde_b = nullptr;
  uint64_t shift = 0;
  // Per-proof strides (words) for a proof group: FRI layer values and trees,
  // trace LDE and trace tree (cb and tinv follow from B and m).
  uint64_t fri_val_stride = 0, fri_tree_stride = 0, lde_stride = 0, ttree_stride = 0;
  // Optional gate (as FoldArgs::go): the launch waits for *go == go_epoch
  // before it reads the indices; a wait that runs out sets bit 3 of *fault.
  // With go_per_query, query qi's CTAs wait on go[qi] instead, so that each
  // gathers as soon as its own index is written.
  const unsigned int* go = nullptr;
  unsigned int go_epoch = 0;
  unsigned int go_per_query = 0;
  unsigned int* fault = nullptr;
  // Optional: word pk * nq + qi is set to go_epoch (store-release, system
  // scope) once the block of query qi of proof pk is written.
  unsigned int* done = nullptr;
};

// Product table of the Fp4 constant r (canonical coordinates) in the layout
// e4_mul_tab expects, in Montgomery form.
void e4_table(const uint32_t r[4], uint32_t T[4][4]);

// Leaf kernels (trace leaves, FRI fold) hash their CTA's Merkle subtree only
// for trees of at most kFuseMaxLeaves leaves: such launches do not fill the
// GPU, so the shrinking levels' latency is paid either way and the separate
// level launches are saved. Larger trees keep the flat level kernels, which
// run the hash at the ALU ceiling where fused levels would leave warps idle.
constexpr uint64_t kFuseMaxLeaves = 1ull << 15;

// Folded IVC (src/fold.rs): one accumulated segment as the combination
// kernel reads it. `a`/`b` are the segment's column LDEs, coset-major
// [j][q]; `ga[t]` is gamma_k * alpha_t (Montgomery form, canonical
// coordinates), with the boundary-at-1 terms (t = 2, 3) also carrying
// omega_s^-1 (1/(x - 1) = omega_s^-1 T(q-1)); `tree` is the segment's row tree.
struct FoldStepDev {
  const uint32_t* a;
  const uint32_t* b;
  const uint32_t* tree;
  uint32_t in_a, in_b, out_a, out_b;
  uint32_t ga[6][4];
};
struct FoldCombineArgs {
  const FoldStepDev* steps;
  uint32_t nsteps;
  const uint32_t* tinv;  // coset-major 1/(x - w_last) (Montgomery)
  const uint32_t* zinv;  // per coset 1/(x^s - 1) (Montgomery)
  uint32_t* layer0;      // FRI layer 0 (bit-reversed Ext4 values)
  uint32_t* leaves;      // its leaf digests
  uint32_t logN, logB;   // segment rows s = 2^logN, blowup 2^logB
  uint32_t w_last_m;     // omega_s^(s-1) (Montgomery)
  // Non-null counter (layer 0 of at most kFuseMaxLeaves leaves): the launch
  // computes its rows' 1/(x - w_last) itself (tinv unused) and builds the
  // layer-0 tree up to `top`, that level also into `cap`.
  unsigned int* counter = nullptr;
  uint32_t top = 0;
  uint32_t* cap = nullptr;
};
// Table membership composition inputs (src/table.rs:597-644).
struct TableComposeArgs {
  const uint32_t* lde;    // the value column's LDE, coset-major [j][q]
  const uint32_t* tinv;   // 1/(x - omega_n^-1) per row, coset-major (Montgomery)
  const uint32_t* zinv;   // B x r values 1/(x^n - 1) (Montgomery)
  const uint32_t* table;  // public table entries (canonical)
  uint32_t table_len;
  uint32_t corr_m;        // R^table_len mod p: restores the product chain to canonical
  uint32_t value;         // claimed member (canonical)
  uint32_t alpha_m[4];    // alpha_member (Montgomery)
  uint32_t alpha_b[4];    // alpha_bound * omega_n^-1 (Montgomery)
  uint32_t* layer0;
  uint32_t* leaves;
  uint32_t logN, logB, r;
};
// A Merkle tree whose leaves repeat in runs (a constant trace, or an FRI
// layer of per-coset constants): G groups of 2^logS equal consecutive leaves,
// group g's leaf hashed from seed g. Every node of a group's subtree at level
// l is one digest, chain[g][l]; the G group roots then form an ordinary
// tree. `out` (16-byte aligned) receives chain[g][l] at digest g * (logS + 1)
// + l, then the tree over the roots, level-contiguous (2G - 1 digests).
struct UniformTree {
  const uint32_t* seeds;  // G seeds of seed_words words each
  uint32_t* out;
  uint32_t G;             // power of two, <= 512
  uint32_t logS;
  uint32_t row;           // 0: a 64-byte block leaf (16 words); 1: a 0x00-prefixed row
  uint32_t seed_words;    // 16 for a block; 1..25 for a row
};

namespace launch {

// Launch schedule: choices that change how work is split across launches,
// CTAs and passes but never a result. One per device, process-wide; the
// launchers read the current device's on every call.
struct Schedule {
  // The default: register passes (variant 2) wherever the balanced split has
  // two even halves within 2^6..2^12 (2^16, 2^20 and 2^24 points), the
  // shared-memory passes in groups of 16 elsewhere.
  Schedule() {
    for (uint32_t l = 13; l <= 26; l++) {
      const uint32_t s = (l + 1) / 2;
      if ((s & 1u) == 0 && ((l - s) & 1u) == 0 && s <= 12 && l - s >= 6) ntt_radix32[l] = 2;
    }
  }
  // Four-step NTT of length 2^logn (13 <= logn <= 26): log2 of the pass-1
  // transform length; 0 = the balanced default ceil(logn / 2).
  uint8_t ntt_log_n1[32] = {};
  // Pass variant of a 2^logn transform: 0 = shared-memory passes in register
  // groups of 16 elements (512 threads a CTA), 1 = the same in groups of 32
  // (256 threads), 2 = register passes (two register passes of radix
  // 2^(L/2) per half of 2^L points, one shared-memory transpose, the tiles
  // loaded by TMA; both halves even and within 2^6..2^12, else variant 0),
  // 3 = the register passes streamed: a resident grid whose CTAs each walk
  // many tiles through two buffers (halves up to 2^10; a 2^12 half takes
  // variant 2's kernel).
  uint8_t ntt_radix32[32] = {};
  // A Merkle tree's levels go one launch each while they have more than
  // 2^merkle_top_log nodes; the rest go to one top kernel (10..18).
  uint32_t merkle_top_log = 16;
  // Proof-of-work grid: CTAs per SM (1..16, clamped to the occupancy limit).
  uint32_t grind_ctas_per_sm = 4;
};
// Valid pass-1 lengths for an NTT of length 2^logn: [lo, hi] (empty if
// logn is served by the one-kernel path).
void ntt_split_range(uint32_t logn, uint32_t* lo, uint32_t* hi);
uint32_t ntt_default_split(uint32_t logn);
// Range checks of every field; false names no field (the caller reports).
bool schedule_valid(const Schedule& s);
// True when a half of 2^L points can take the register passes (variant 2).
bool reg_split_ok(uint32_t L);
Schedule get_schedule(int device);
void set_schedule(int device, const Schedule& s);

// One CTA per tree (kernels.h, UniformTree); `trees` is device-readable.
cudaError_t uniform_trees(cudaStream_t st, const UniformTree* trees, uint32_t ntrees);

// Number of kernel launches issued by this library in this process.
uint64_t launch_count();
// Optional per-stage timing: when a recorder is installed, every launcher
// brackets its kernels with CUDA events on the launching stream.
struct StageRecorder {
  virtual ~StageRecorder() = default;
  virtual void begin(const char* stage, cudaStream_t st) = 0;
  virtual void end(const char* stage, cudaStream_t st) = 0;
  // `kernels` kernel launches issued inside the open stage `stage`.
  virtual void launched(const char* stage, int kernels) { (void)stage; (void)kernels; }
};
void set_recorder(StageRecorder* r);

// Device address of constant slot `slot` (a ProofConsts).
cudaError_t const_slot_address(int slot, void** ptr);

// (a0, b0) from the slot.
//
// Proof groups: the launchers below take `nproofs` proofs of one shape at
// once (grid y = proof). Proof k's buffers sit at the given per-proof strides
// from proof 0's, its ProofConsts in slot + k, and its counters and search
// state at index k.
// With `zinv` the launch also computes the per-coset constants (extra CTAs
// beside the trace's, as coset_zinv would).
cudaError_t fib_trace(cudaStream_t st, uint32_t* col_a, uint32_t* col_b, uint32_t n, uint32_t slot,
                      const uint32_t mats[32][4], uint32_t nproofs = 1, const ZinvArgs* zinv = nullptr,
                      const Tables* tb = nullptr);
// Proof k: cols + k n ncols, values + k ncols.
cudaError_t fill_constant_columns(cudaStream_t st, uint32_t* cols, uint32_t n, uint32_t ncols,
                                  const uint32_t* d_values, uint32_t nproofs = 1);
cudaError_t ntt(cudaStream_t st, const Tables& tb, const NttPlan& plan, const uint32_t* in,
                uint32_t* out, uint32_t* scratch);
// The per-coset constants of ZinvArgs in a launch of their own.
cudaError_t coset_zinv(cudaStream_t st, const Tables& tb, uint32_t* zinv, uint32_t* zinv2,
                       uint32_t logB, uint32_t gamma_n_m, uint32_t* cb, uint32_t slot,
                       uint32_t nproofs = 1);
// Trace leaves of the AIR: rows 8L..8L+7 as A || B with B derived from A.
// Also writes tinv (m words, coset-major): 1 / (x - w_last) per LDE row.
// For trees of at most kFuseMaxLeaves leaves the kernel also hashes each
// CTA's subtree (up to the cap level `top`; nodes to the tree, the cap level
// to `cap`), and with `counter` (one zero device word per proof) its last CTA
// finishes the tree up to `top`. *levels receives how many levels above the
// leaves are done, the start level for merkle_build.
// With `lde_b`, column B is read from its own LDE (same layout) instead of
// being derived from A.
cudaError_t air_trace_leaves(cudaStream_t st, const Tables& tb, const uint32_t* lde_a,
                             const uint32_t* cb, uint32_t w_last_m, uint32_t* leaves,
                             uint32_t* tinv, uint32_t logN, uint32_t logB, uint32_t top,
                             uint32_t* cap, unsigned int* counter, uint32_t* levels,
                             uint32_t nproofs = 1, uint64_t tree_stride = 0,
                             uint64_t cap_stride = 0, const uint32_t* lde_b = nullptr);
// air::prove_zk masking of both columns' twisted coefficients into planes of
// `padded` words (r: 2 x n_rand canonical masking values).
cudaError_t mask_pad(cudaStream_t st, const Tables& tb, const uint32_t* coeffs, const uint32_t* r,
                     uint32_t* out, uint32_t n, uint32_t n_rand, uint32_t padded, uint32_t ncols = 2);
cudaError_t table_compose(cudaStream_t st, const Tables& tb, const TableComposeArgs& a);
// Composition with column B from its own LDE (next row r rows further in a
// coset; a.zinv holds B x r values 1/(x^n - 1)); the slot's alpha[.][0..4]
// are alpha_0..alpha_4 with alpha_2, alpha_3 times omega_n^-1.
cudaError_t air_compose_general(cudaStream_t st, const Tables& tb, const AirComposeArgs& a,
                                const uint32_t* lde_b, uint32_t r);
// A small IVC segment's commit in one launch (2 <= S = 2^logN <= 2^8,
// 32 <= S B <= 256): interpolation of the two columns at `cols` (checked on
// load, a non-canonical word sets *bad), their coset-major LDEs at `lde`
// (column A, then column B), the 8-byte row leaves and the tree up to `top`,
// level `top` also into `cap`. The same words as the two NTTs and the row
// leaves of range_trace_leaves with two columns.
bool fold_segment_ok(uint32_t logN, uint32_t logB);
cudaError_t fold_segment(cudaStream_t st, const Tables& tb, const uint32_t* cols, unsigned int* bad,
                         uint32_t* lde, uint32_t* tree, uint32_t* cap, uint32_t logN, uint32_t logB,
                         uint32_t top);
// With a counter (one zero word per proof) and at most kFuseMaxLeaves rows,
// the launch also builds the tree up to `top` and writes that level to cap
// (proof k at k * cap_stride); *levels receives the levels built (0:
// merkle_build does them all).
cudaError_t range_trace_leaves(cudaStream_t st, const uint32_t* lde, uint32_t* leaves,
                               uint32_t logN, uint32_t logB, uint32_t ncols, uint32_t nproofs = 1,
                               uint64_t tree_stride = 0, unsigned int* counter = nullptr,
                               uint32_t top = 0, uint32_t* cap = nullptr, uint64_t cap_stride = 0,
                               uint32_t* levels = nullptr);
// Builds levels 1..top of a tree stored level-contiguous (level l at digest
// offset 2L - 2(L >> l), L = leaves, power of two). Levels above the cap
// level are never read (caps and capped paths stop there), so callers pass
// top = depth - drop.
// `counter` is one device word, zero before the call and zero again after it
// (the upper levels are finished by the last CTA to arrive; nothing waits).
// `cap` (may be null; device-visible, e.g. mapped host memory) receives a copy
// of level `top`, 32 bytes per node.
// Levels below `from` must already be built (0: from the leaves).
cudaError_t merkle_build(cudaStream_t st, uint32_t* tree, uint64_t leaves, uint32_t top,
                         unsigned int* counter, uint32_t* cap, uint32_t from = 0,
                         uint32_t nproofs = 1, uint64_t stride = 0, uint64_t cap_stride = 0);
// With a.counter set and a tree of at most kFuseMaxLeaves leaves, the
// launch also builds the tree up to a.top; *levels receives the levels it
// built (0: merkle_build does them all).
cudaError_t air_compose_leaves(cudaStream_t st, const Tables& tb, const AirComposeArgs& a,
                               uint32_t nproofs = 1, uint32_t* levels = nullptr);
cudaError_t range_compose_leaves(cudaStream_t st, const Tables& tb, const RangeComposeArgs& a,
                                 uint32_t nproofs = 1);
// Folds one FRI layer; hashes the next layer's 64-byte leaves when it has a
// multiple of four values, its 0x00-prefixed 16-byte leaves otherwise. With
// 64-byte leaves it also hashes each CTA's subtree up to a.top (writing the
// cap level to a.cap), and the last CTA finishes the tree when a.counter is
// set; *levels receives the levels done above the leaves.
cudaError_t fri_fold(cudaStream_t st, const Tables& tb, const FoldArgs& a, uint32_t* levels,
                     uint32_t nproofs = 1);
// Whether fri_fold reads the tables of `a` from the constant slots (true) or
// from a.tab (false).
bool fri_fold_uses_slot(const FoldArgs& a);
// fri::commit input: out[c][i] = in[c-th coordinate of value i] * 31^i (one
// coordinate, or four for Ext4 input interleaved 4 words per value); *bad
// receives 1 when an input word is not a canonical field element.
cudaError_t gamma_scale(cudaStream_t st, const Tables& tb, const uint32_t* in, uint32_t* out,
                        uint32_t n, uint32_t ext, unsigned int* bad);
// FRI layer 0 of a commitment and its leaf digests, from coset-major
// coordinate LDEs (coset_major; ncomp planes of m = 2^logm words, 2^logB
// cosets) or from natural-order evaluations (ncomp words per value, checked
// canonical into *bad).
// With a counter and a tree of at most kFuseMaxLeaves leaves, the launch
// also builds the tree up to `top` and writes that level to cap; *levels
// receives the levels built (0: merkle_build does them all).
cudaError_t layer0_leaves(cudaStream_t st, const uint32_t* src, uint32_t* layer0, uint32_t* leaves,
                          unsigned int* bad, uint32_t logm, uint32_t logB, uint32_t ncomp,
                          bool coset_major, unsigned int* counter = nullptr, uint32_t top = 0,
                          uint32_t* cap = nullptr, uint32_t* levels = nullptr);
// Words of 1 / (x_k - w_last) for every LDE row, stored coset-major.
cudaError_t row_inverses(cudaStream_t st, const Tables& tb, uint32_t* tinv, uint32_t w_last_m,
                         uint32_t logN, uint32_t logB);
// combined(x) = sum_k gamma_k C_k(x) over the accumulated segments, written
// as FRI layer 0 with its leaf digests (src/fold.rs:494-517, 785-850).
cudaError_t fold_combine(cudaStream_t st, const Tables& tb, const FoldCombineArgs& a,
                         uint32_t* levels = nullptr);
// Step openings (src/fold.rs:527-552): for step k and query i, at
// out + (k nq + i) stride: A, B at index = brev(leaf) and at index + B
// (mod m), then the capped paths of both rows (steps x 8 words each).
cudaError_t fold_openings(cudaStream_t st, const FoldStepDev* steps, uint32_t nsteps,
                          const uint64_t* leaves, uint32_t nq, uint32_t logN, uint32_t logB,
                          uint32_t path_steps, uint32_t* out, uint32_t stride);
// Leaf digests of an FRI layer held in memory (64-byte quads or 16-byte values).
cudaError_t layer_leaves(cudaStream_t st, const uint32_t* values, uint64_t len, uint32_t* leaves,
                         uint32_t nproofs = 1, uint64_t in_stride = 0, uint64_t out_stride = 0);
// Digests of `count` 64-byte leaves, padded to npad (a power of two) by
// repeating the last leaf.
cudaError_t merkle_flat64_leaves(cudaStream_t st, const uint32_t* flat, uint64_t count,
                                 uint64_t npad, uint32_t* leaves);
// Minimum-nonce proof-of-work search. `state` is 4 device u64s holding
// {~0, 0, 0, 0} before the call and again after it; `out` (device-visible)
// receives {best nonce, status}, status 1 when the nonce cap was reached.
// Proof k's head (head_len bytes) is at head + k * kPowHeadWords
// (device-visible). With `go`, the launch first waits at that gate (as
// FoldArgs::go) for go_epoch; a wait that runs out sets bit 3 of *fault.
cudaError_t grind(cudaStream_t st, const uint32_t* head, uint32_t head_len, uint32_t bits,
                  unsigned long long* state, unsigned long long* out, uint64_t max_nonces,
                  uint32_t nproofs = 1, const unsigned int* go = nullptr,
                  unsigned int go_epoch = 0, unsigned int* fault = nullptr);

bool grind_supports(uint32_t head_len);
// Reorders `batch` coset-major LDEs ([j][q]) into natural order ([B q + j]).
cudaError_t coset_to_natural(cudaStream_t st, const uint32_t* in, uint32_t* out, uint32_t logN,
                             uint32_t logB, uint64_t batch);
cudaError_t openings(cudaStream_t st, const OpenArgs& a, uint32_t nproofs = 1);
// blocks x 256 threads, each chaining `iters` node hashes from 16 words of
// `in` (blocks * 256 * 64 bytes) and writing 8 words of `out`.
cudaError_t hash_ceiling(cudaStream_t st, const uint32_t* in, uint32_t* out, uint32_t blocks,
                         int iters);

}  // namespace launch
}  // namespace z0p
