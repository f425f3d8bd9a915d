// GB300 prove path for z0p: device workspace, the Fibonacci-AIR and
// range-check provers, and the C ABI declared in include/z0p_gpu.h.
//
// Dataflow of one AIR proof (src/air.rs:485-599), all stages on one stream:
//   trace (parallel 2x2 matrix powers) -> iNTT of both columns, outputs
//   pre-multiplied by 31^i / N -> 2B coset NTTs written coset-major ->
//   trace leaves + tree -> [host: cap, alphas] -> composition written as
//   bit-reversed FRI layer 0 with its leaf digests -> tree -> [host: cap,
//   fold challenges] -> fold + next-layer leaves -> tree -> ... -> final
//   layer -> [host: head] -> PoW grind -> [host: query indices] -> one
//   gather of every opened value and path -> proof bytes on the host.
// The host holds the transcript; each bracket is one stream synchronisation.
#include <cuda_runtime.h>

#include <array>
#include <chrono>
#include <functional>
#include <map>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/z0p_gpu.h"
#include "host.h"
#include "kernels.h"

using namespace z0p;
using namespace z0p::host;

namespace z0p {
namespace host {
const char* reason();
}
}  // namespace z0p

#define CK(expr)                                                              \
  do {                                                                        \
    cudaError_t _e = (expr);                                                  \
    if (_e != cudaSuccess) {                                                  \
      set_reason(std::string(#expr) + ": " + cudaGetErrorString(_e));         \
      return _e == cudaErrorMemoryAllocation ? Z0P_ERR_OUT_OF_MEMORY : Z0P_ERR_CUDA; \
    }                                                                         \
  } while (0)

#define RC(expr)              \
  do {                        \
    int _r = (expr);          \
    if (_r != Z0P_OK) return _r; \
  } while (0)

namespace {

struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
};

// Little-endian byte writer (src/codec.rs:38-114) straight into the caller's
// buffer; the proof length is known from its shape before the first byte.
struct Writer {
  uint8_t* p;
  size_t n = 0, cap;
  Writer(uint8_t* out, size_t c) : p(out), cap(c) {}
  bool ok() const { return n <= cap; }
  void byte(uint8_t v) {
    if (n < cap) p[n] = v;
    n++;
  }
  void u32(uint32_t v) {
    if (n + 4 <= cap) for (int i = 0; i < 4; i++) p[n + i] = (uint8_t)(v >> (8 * i));
    n += 4;
  }
  void u64(uint64_t v) {
    if (n + 8 <= cap) for (int i = 0; i < 8; i++) p[n + i] = (uint8_t)(v >> (8 * i));
    n += 8;
  }
  void bytes(const void* src, size_t k) {
    if (n + k <= cap) std::memcpy(p + n, src, k);
    n += k;
  }
};

}  // namespace

// Per-stage CUDA-event timing on the launching stream (diagnostic mode).
struct EventRecorder final : launch::StageRecorder {
  struct Mark {
    std::string stage;
    cudaEvent_t a, b;
    uint64_t kernels = 0;
  };
  std::vector<Mark> marks;
  std::vector<cudaEvent_t> pool;
  cudaEvent_t take() {
    if (!pool.empty()) {
      cudaEvent_t e = pool.back();
      pool.pop_back();
      return e;
    }
    cudaEvent_t e;
    cudaEventCreate(&e);
    return e;
  }
  void begin(const char* stage, cudaStream_t st) override {
    Mark m{stage, take(), take()};
    cudaEventRecord(m.a, st);
    marks.push_back(m);
  }
  void end(const char* stage, cudaStream_t st) override {
    for (size_t i = marks.size(); i-- > 0;)
      if (marks[i].stage == stage) {
        cudaEventRecord(marks[i].b, st);
        return;
      }
  }
  void launched(const char* stage, int kernels) override {
    for (size_t i = marks.size(); i-- > 0;)
      if (marks[i].stage == stage) {
        marks[i].kernels += (uint64_t)kernels;
        return;
      }
  }
  ~EventRecorder() override {
    for (auto& m : marks) { cudaEventDestroy(m.a); cudaEventDestroy(m.b); }
    for (auto e : pool) cudaEventDestroy(e);
  }
};

namespace z0p {
struct FriPending;
}

struct z0p_gpu_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  std::mutex mu;
  Tables tb{};
  DevBuf tables, cols, coeffs, scratch, lde, ttree, layers, ftrees, misc, state;
  // Mapped pinned buffer for what a proof hands to the host (caps, final
  // layer, PoW result, query indices, openings): kernels write it directly,
  // so no copy operation is queued for them.
  uint8_t* hio = nullptr;
  uint8_t* hio_d = nullptr;  // its device address
  size_t hio_bytes = 0;
  // Mapped status word of the bounded device waits (Tables::fault): nonzero
  // once a kernel of this context gave up waiting.
  unsigned int* fault = nullptr;
  // The context's constant slots of per-proof values (slot .. slot+nslots-1,
  // one per proof of a group) and their pinned staging copies: the host
  // fills `consts`, push_consts queues the copy into the slots.
  int slot = -1, nslots = 0;
  void* slot_dev = nullptr;
  ProofConsts* consts = nullptr;  // kMaxGroup entries
  size_t held = 0;
  uint64_t h2d = 0, d2h = 0, syncs = 0, proofs = 0, sync_ns = 0, prove_ns = 0;
  bool profiling = false;
  EventRecorder rec;
  struct HostSite {
    uint64_t calls = 0, wait_ns = 0, before_ns = 0;
  };
  std::map<std::string, HostSite> sites;
  uint64_t last_sync_ns = 0;  // 0 = no prove call in progress
  uint64_t tail_ns = 0;       // host time after a prove call's last synchronisation
  // Every call that uses the workspace or the mapped buffer counts here; a
  // FRI commitment stays openable only while no other such call came after it.
  uint64_t work_serial = 0;
  z0p::FriPending* fri = nullptr;
  // Gated FRI tails (run_fri_commit): one event per layer, and the value the
  // current commitment writes into its gate words.
  std::vector<cudaEvent_t> gate_ev;
  uint32_t go_epoch = 0;
  bool gates = true;  // z0p_gpu_ctx_set_gates
  // Openings read as they land (run_fri_openings with `defer`): while
  // open_epoch is non-zero, open_block waits for the query's done word in
  // the mapped buffer (at open_done) to hold it.
  uint32_t open_epoch = 0;
  size_t open_done = 0;
};
using HostSite = z0p_gpu_ctx::HostSite;

namespace {

uint64_t now_ns() {
  return (uint64_t)std::chrono::duration_cast<std::chrono::nanoseconds>(
             std::chrono::steady_clock::now().time_since_epoch())
      .count();
}
// Every stream synchronisation of a prove call goes through here (with
// `upto`, the wait ends at that event rather than at the stream's end). With
// profiling on, it also records, per call site, the time blocked and the host
// time since the previous synchronisation returned (the GPU is idle for part
// of the latter, from the moment its queue drains until the next launch).
cudaError_t sync(z0p_gpu_ctx* c, const char* site = "other", cudaEvent_t upto = nullptr) {
  c->syncs++;
  uint64_t t0 = now_ns();
  cudaError_t e = upto ? cudaEventSynchronize(upto) : cudaStreamSynchronize(c->stream);
  uint64_t t1 = now_ns();
  if (e == cudaSuccess && c->fault && *reinterpret_cast<volatile unsigned int*>(c->fault)) {
    *c->fault = 0u;  // reported once; the context stays usable
    e = cudaErrorLaunchTimeout;
  }
  c->sync_ns += t1 - t0;
  if (c->profiling) {
    HostSite& h = c->sites[site];
    h.calls++;
    h.wait_ns += t1 - t0;
    if (c->last_sync_ns) h.before_ns += t0 - c->last_sync_ns;
  }
  c->last_sync_ns = t1;
  return e;
}

// Spins until done() holds, querying `upto` (or the stream) every 64
// passes so that a launch that failed, or a word that legitimately equals
// its sentinel, ends the wait at the work's completion; accounted like sync.
template <class Done>
cudaError_t wait_mapped(z0p_gpu_ctx* c, const char* site, cudaEvent_t upto, Done done) {
  c->syncs++;
  const uint64_t t0 = now_ns();
  cudaError_t e = cudaSuccess;
  for (uint32_t pass = 0; !done(); pass++) {
    if ((pass & 63u) != 63u) continue;
    e = upto ? cudaEventQuery(upto) : cudaStreamQuery(c->stream);
    if (e != cudaErrorNotReady) break;
    e = cudaSuccess;
  }
  __atomic_thread_fence(__ATOMIC_ACQUIRE);
  const uint64_t t1 = now_ns();
  if (e == cudaSuccess && c->fault && *reinterpret_cast<volatile unsigned int*>(c->fault)) {
    *c->fault = 0u;  // reported once; the context stays usable
    e = cudaErrorLaunchTimeout;
  }
  c->sync_ns += t1 - t0;
  if (c->profiling) {
    HostSite& hs = c->sites[site];
    hs.calls++;
    hs.wait_ns += t1 - t0;
    if (c->last_sync_ns) hs.before_ns += t0 - c->last_sync_ns;
  }
  c->last_sync_ns = t1;
  return e;
}

// A Merkle cap the device writes into the mapped buffer can be read as soon
// as its last word lands, before the kernel that wrote it has retired and
// the stream's completion has reached the host. arm_cap fills the cap's
// region with kCapSentinel; it must run before the kernels that write the
// cap are queued (after them, it could overwrite digests already written).
// wait_cap then waits until no word of the region holds the sentinel (a
// digest word equal to it, one chance in 2^32 a word, only sends the wait
// on to the work's completion).
constexpr uint32_t kCapSentinel = 0x6A09E667u;

void arm_cap(z0p_gpu_ctx* c, size_t off, size_t bytes) {
  uint32_t* w = reinterpret_cast<uint32_t*>(c->hio + off);
  for (size_t i = 0; i < bytes / 4; i++) w[i] = kCapSentinel;
  __atomic_thread_fence(__ATOMIC_SEQ_CST);
}

cudaError_t wait_cap(z0p_gpu_ctx* c, const char* site, size_t off, size_t bytes,
                     cudaEvent_t upto = nullptr) {
  const volatile uint32_t* w = reinterpret_cast<const volatile uint32_t*>(c->hio + off);
  const size_t n = bytes / 4;
  size_t i = 0;  // words before i are written (each is written once)
  return wait_mapped(c, site, upto, [&] {
    while (i < n && w[i] != kCapSentinel) i++;
    return i == n;
  });
}

// The same for the PoW results (per proof the nonce word, then the cap
// flag, which the search writes first): a nonce word is below 2^40 or all
// ones, never kPowSentinel.
constexpr uint64_t kPowSentinel = ~1ull;

void arm_pow(z0p_gpu_ctx* c, size_t off, uint32_t K) {
  for (uint32_t k = 0; k < K; k++) std::memcpy(c->hio + off + 16 * k, &kPowSentinel, 8);
  __atomic_thread_fence(__ATOMIC_SEQ_CST);
}

cudaError_t wait_pow(z0p_gpu_ctx* c, size_t off, uint32_t K, cudaEvent_t upto = nullptr) {
  uint32_t k = 0;
  return wait_mapped(c, "grind", upto, [&] {
    while (k < K && *reinterpret_cast<const volatile uint64_t*>(c->hio + off + 16 * k) != kPowSentinel) k++;
    return k == K;
  });
}

// Workspace comes from one stream-ordered memory pool per device that keeps
// freed memory for reuse: growing or releasing a context's buffers is queued
// on its own stream and never synchronises the device, so contexts proving
// side by side do not stall one another.
cudaError_t device_pool(int device, cudaMemPool_t* out) {
  static std::mutex mu;
  static std::map<int, cudaMemPool_t> pools;
  std::lock_guard<std::mutex> lk(mu);
  auto it = pools.find(device);
  if (it != pools.end()) {
    *out = it->second;
    return cudaSuccess;
  }
  cudaMemPoolProps props{};
  props.allocType = cudaMemAllocationTypePinned;
  props.handleTypes = cudaMemHandleTypeNone;
  props.location.type = cudaMemLocationTypeDevice;
  props.location.id = device;
  cudaMemPool_t pool;
  cudaError_t e = cudaMemPoolCreate(&pool, &props);
  if (e != cudaSuccess) return e;
  uint64_t keep = UINT64_MAX;
  e = cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
  if (e != cudaSuccess) return e;
  pools[device] = pool;
  *out = pool;
  return cudaSuccess;
}

void release(z0p_gpu_ctx* c, DevBuf& b) {
  if (!b.p) return;
  cudaFreeAsync(b.p, c->stream);
  c->held -= b.bytes;
  b.p = nullptr;
  b.bytes = 0;
}

int ensure(z0p_gpu_ctx* c, DevBuf& b, size_t bytes) {
  if (bytes <= b.bytes) return Z0P_OK;
  release(c, b);
  size_t want = bytes + bytes / 8;  // headroom so near sizes reuse the buffer
  cudaMemPool_t pool;
  CK(device_pool(c->device, &pool));
  CK(cudaMallocFromPoolAsync(&b.p, want, pool, c->stream));
  b.bytes = want;
  c->held += want;
  return Z0P_OK;
}

// Constant slots are handed to contexts as contiguous ranges (one slot per
// proof of a group), first fit.
std::mutex g_slot_mu;
bool g_slot_used[kConstSlots] = {};

int take_slots_locked(int n) {
  for (int i = 0; i + n <= kConstSlots; i++) {
    int j = 0;
    while (j < n && !g_slot_used[i + j]) j++;
    if (j == n) {
      for (j = 0; j < n; j++) g_slot_used[i + j] = true;
      return i;
    }
    i += j;
  }
  return -1;
}
int take_slots(int n) {
  std::lock_guard<std::mutex> lk(g_slot_mu);
  return take_slots_locked(n);
}
void give_slots_locked(int first, int n) {
  for (int i = first; i >= 0 && i < first + n && i < kConstSlots; i++) g_slot_used[i] = false;
}
void give_slots(int first, int n) {
  std::lock_guard<std::mutex> lk(g_slot_mu);
  give_slots_locked(first, n);
}

// The context holds at least K contiguous slots. A context only grows its
// range between prove calls, after its stream has drained. When no K free
// slots are contiguous, the context keeps a range of its previous size
// (which always fits again: the exchange holds the lock throughout) and the
// call reports Z0P_ERR_OUT_OF_MEMORY; callers then prove smaller groups.
int ensure_slots(z0p_gpu_ctx* c, uint32_t K) {
  if ((int)K <= c->nslots) return Z0P_OK;
  CK(cudaStreamSynchronize(c->stream));
  bool grown;
  {
    std::lock_guard<std::mutex> lk(g_slot_mu);
    const int old = c->nslots;
    give_slots_locked(c->slot, old);
    int first = take_slots_locked((int)K);
    grown = first >= 0;
    if (grown) {
      c->nslots = (int)K;
    } else {
      first = take_slots_locked(old > 0 ? old : 1);
      c->nslots = first < 0 ? 0 : (old > 0 ? old : 1);
    }
    c->slot = first;
  }
  if (c->nslots > 0) CK(launch::const_slot_address(c->slot, &c->slot_dev));
  if (!grown) {
    set_reason("no free constant slots for a group of this size");
    return Z0P_ERR_OUT_OF_MEMORY;
  }
  return Z0P_OK;
}

// Queues the copy of the first K proofs' values into the context's slots.
// The host changes c->consts only after the stream has synchronised past the
// previous copy.
cudaError_t push_consts(z0p_gpu_ctx* c, uint32_t K) {
  c->h2d += (uint64_t)K * sizeof(ProofConsts);
  return cudaMemcpyAsync(c->slot_dev, c->consts, (size_t)K * sizeof(ProofConsts),
                         cudaMemcpyHostToDevice, c->stream);
}

// PoW head bytes as kPowHeadWords little-endian words, zero padded.
void set_head(uint32_t* words, const uint8_t* head, size_t len) {
  for (uint32_t i = 0; i < kPowHeadWords; i++) words[i] = 0;
  for (size_t i = 0; i < len && i < 4 * kPowHeadWords; i++)
    words[i / 4] |= (uint32_t)head[i] << (8 * (i % 4));
}

int ensure_hio(z0p_gpu_ctx* c, size_t bytes) {
  if (bytes <= c->hio_bytes) return Z0P_OK;
  if (c->hio) {
    CK(sync(c));
    CK(cudaFreeHost(c->hio));
    c->hio = c->hio_d = nullptr;
    c->hio_bytes = 0;
  }
  size_t want = bytes + bytes / 4 < (4u << 20) ? (4u << 20) : bytes + bytes / 4;
  CK(cudaHostAlloc((void**)&c->hio, want, cudaHostAllocMapped));
  CK(cudaHostGetDevicePointer((void**)&c->hio_d, c->hio, 0));
  c->hio_bytes = want;
  return Z0P_OK;
}
template <class T>
T* hio_dev(z0p_gpu_ctx* c, size_t off) {
  return reinterpret_cast<T*>(c->hio_d + off);
}

int build_tables(z0p_gpu_ctx* c) {
  const int lo_w = 1 << 14, hi_w = 1 << 13, lo_g = 1 << 12, hi_g = 1 << 15;
  std::vector<uint32_t> t(lo_w + hi_w + lo_g + hi_g);
  uint32_t omega = two_adic_generator(27);
  uint32_t* w_lo = t.data();
  uint32_t* w_hi = w_lo + lo_w;
  uint32_t* g_lo = w_hi + hi_w;
  uint32_t* g_hi = g_lo + lo_g;
  uint32_t x = 1;
  for (int i = 0; i < lo_w; i++) { w_lo[i] = to_mont(x); x = fmul(x, omega); }
  uint32_t step = fpow(omega, lo_w);
  x = 1;
  for (int i = 0; i < hi_w; i++) { w_hi[i] = to_mont(x); x = fmul(x, step); }
  x = 1;
  for (int i = 0; i < lo_g; i++) { g_lo[i] = to_mont(x); x = fmul(x, GENERATOR); }
  step = fpow(GENERATOR, lo_g);
  x = 1;
  for (int i = 0; i < hi_g; i++) { g_hi[i] = to_mont(x); x = fmul(x, step); }
  // NTT stage twiddles with their Shoup quotients (kernels.h, Tables::stw).
  const size_t stw_at = t.size();  // in words; t.size() is even
  t.resize(stw_at + 4 * (size_t)kStwInverse, 0u);
  for (uint32_t inv = 0; inv < 2; inv++)
    for (uint32_t L = 1; L <= 13; L++) {
      const uint32_t root = two_adic_generator(L);
      uint32_t w = 1;
      const uint32_t step = inv ? finv(root) : root;
      uint32_t* dst = t.data() + stw_at + 2 * ((size_t)inv * kStwInverse + (1u << (L - 1)) - 1);
      for (uint32_t i = 0; i < (1u << (L - 1)); i++) {
        dst[2 * i] = w;
        dst[2 * i + 1] = (uint32_t)(((uint64_t)w << 32) / P);
        w = fmul(w, step);
      }
    }
  RC(ensure(c, c->tables, t.size() * 4));
  CK(cudaMemcpyAsync(c->tables.p, t.data(), t.size() * 4, cudaMemcpyHostToDevice, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  const uint32_t* d = (const uint32_t*)c->tables.p;
  c->tb.w_lo = d;
  c->tb.w_hi = d + lo_w;
  c->tb.g_lo = d + lo_w + hi_w;
  c->tb.g_hi = d + lo_w + hi_w + lo_g;
  c->tb.stw = reinterpret_cast<const uint2*>(d + stw_at);
  return Z0P_OK;
}

inline uint64_t tree_digests(uint64_t leaves) { return 2 * leaves - 1; }

// Device counters that kernels leave as they found them, set once when the
// context is created, one per proof of a group: the Merkle last-CTA counters
// (kMaxGroup words) and the PoW search states (kMaxGroup x 4 u64).
inline unsigned int* merkle_counter(z0p_gpu_ctx* c) { return (unsigned int*)c->state.p; }
inline unsigned long long* grind_state(z0p_gpu_ctx* c) {
  return reinterpret_cast<unsigned long long*>((char*)c->state.p + 4 * kMaxGroup);
}
constexpr uint32_t kPowHeadBytes = 40 + 7;  // H(history) || LE64(7) || "fri-pow"


inline uint64_t level_off(uint64_t leaves, uint32_t l) { return 2 * leaves - 2 * (leaves >> l); }

// One FRI commitment + opening of one proof (src/fri.rs:551-666 from the
// first layer-root absorb onward).
struct FriOut {
  std::vector<std::vector<uint8_t>> caps;
  std::vector<uint32_t> final_vals;
  uint64_t nonce = 0;
  std::vector<uint64_t> indices;
};

// Device FRI layers and trees of a proof group: proof k's layer l values at
// layer[l] + k * val_stride and its layer-l tree at tree[l] + k * tree_stride
// (words).
struct FriBufs {
  std::vector<uint32_t*> layer;  // proof 0's values per layer (layer 0 included)
  std::vector<uint32_t*> tree;   // proof 0's trees per layer
  uint64_t val_stride = 0, tree_stride = 0;
};

int plan_fri_buffers(z0p_gpu_ctx* c, const FriShape& s, uint32_t K, FriBufs* fb) {
  size_t vals = 0, digs = 0;
  for (size_t i = 0; i < s.len.size(); i++) {
    vals += 4 * s.len[i];
    digs += 8 * tree_digests(s.leaves[i]);
  }
  RC(ensure(c, c->layers, (size_t)K * vals * 4));
  RC(ensure(c, c->ftrees, (size_t)K * digs * 4));
  fb->val_stride = vals;
  fb->tree_stride = digs;
  uint32_t* v = (uint32_t*)c->layers.p;
  uint32_t* d = (uint32_t*)c->ftrees.p;
  fb->layer.clear();
  fb->tree.clear();
  for (size_t i = 0; i < s.len.size(); i++) {
    fb->layer.push_back(v);
    fb->tree.push_back(d);
    v += 4 * s.len[i];
    d += 8 * tree_digests(s.leaves[i]);
  }
  return Z0P_OK;
}

// Where a group's host-visible pieces land in the mapped buffer. Each piece
// is one region holding the K proofs' copies back to back, so kernels reach
// proof k's at a fixed stride: the trace cap and each FRI layer's cap (tree
// kernels), the final layers, the PoW results, the query indices (host),
// the opening blocks (openings kernel; layout in kernels.h, OpenArgs) and
// small per-proof inputs read by kernels in place.
struct HioPlan {
  uint32_t K = 1;
  uint64_t queries = 0;
  size_t trace_cap = 0, trace_cap_bytes = 0;
  std::vector<size_t> fri_cap, fri_cap_bytes;
  size_t final_vals = 0, final_bytes = 0, grind = 0, indices = 0, open = 0;
  // Read by kernels in place: the small folds' challenge tables, per layer
  // ([layer][proof][kFoldTabWords]), the gate words (one per fold, then the
  // PoW search's, then one per query for the gather) and the PoW heads.
  size_t tabs = 0, gates = 0, heads = 0;
  size_t done = 0;  // the gather's done word per (proof, query)
  size_t extra = 0, extra_bytes = 0;
  uint32_t stride = 0, trace_off = 0;  // one opening block, in words
  std::vector<uint32_t> layer_off;     // per non-final FRI layer, in words
};

int plan_hio(z0p_gpu_ctx* c, const FriShape& s, uint64_t queries, uint32_t tdrop,
             uint32_t trace_words, uint32_t K, HioPlan* h, size_t extra_bytes = 0) {
  size_t at = 0;
  auto take = [&](size_t bytes) {  // a region of K copies, 16-byte aligned
    size_t r = at;
    at += ((size_t)K * bytes + 15) & ~(size_t)15;
    return r;
  };
  h->K = K;
  h->queries = queries;
  h->trace_cap_bytes = 32ull << tdrop;
  h->trace_cap = take(h->trace_cap_bytes);
  h->fri_cap.clear();
  h->fri_cap_bytes.clear();
  for (size_t l = 0; l < s.len.size(); l++) {
    h->fri_cap_bytes.push_back(32ull << s.drop[l]);
    h->fri_cap.push_back(take(h->fri_cap_bytes.back()));
  }
  h->final_bytes = 16 * s.len.back();
  h->final_vals = take(h->final_bytes);
  h->grind = take(16);
  h->tabs = take(4 * kFoldTabWords * s.len.size());
  h->gates = take(4 * (s.len.size() + (queries ? queries : 1)));
  h->heads = take(4 * kPowHeadWords);
  h->indices = take(8 * queries);
  h->done = take(4 * (queries ? queries : 1));
  size_t L = s.len.size() - 1;
  if (L > kMaxOpenLayers) {
    set_reason("more FRI layers than the openings kernel supports");
    return Z0P_ERR_UNSUPPORTED;
  }
  h->layer_off.clear();
  uint32_t w = 0;
  for (size_t d = 0; d < L; d++) {
    h->layer_off.push_back(w);
    w += 16 + 8 * (s.depth[d] - s.drop[d]);
  }
  h->trace_off = w;
  h->stride = (w + trace_words + 3) & ~3u;
  h->open = take(4ull * h->stride * queries);
  h->extra_bytes = extra_bytes;
  h->extra = take(extra_bytes);
  return ensure_hio(c, at);
}

// The PoW search of a group whose heads are at `heads` (device-visible,
// kPowHeadWords per proof): results at res_at in the mapped buffer.
cudaError_t queue_grind(z0p_gpu_ctx* c, const FriParams& fp, const uint32_t* heads, size_t res_at,
                        uint32_t K) {
  return launch::grind(c->stream, heads, kPowHeadBytes, fp.grinding_bits, grind_state(c),
                       hio_dev<unsigned long long>(c, res_at), 1ull << 40, K);
}
int check_grind(z0p_gpu_ctx* c, size_t res_at, uint32_t k, uint64_t* nonce) {
  unsigned long long res[2];
  std::memcpy(res, c->hio + res_at + 16 * k, 16);
  c->d2h += 16;
  if (res[1] != 0 || res[0] == ~0ull) {
    set_reason("proof-of-work search reached its nonce cap without a solution");
    return Z0P_ERR_DEVICE_TIMEOUT;
  }
  *nonce = res[0];
  return Z0P_OK;
}

// Gated launches need a host thread that queues ahead and opens the gates
// while they wait. A process whose launches block (CUDA_LAUNCH_BLOCKING=1)
// or run under an injected tool that serialises them (profilers and
// checkers set CUDA_INJECTION64_PATH) would leave each gated launch waiting
// out its bound, so there the folds are launched after their tables, as
// the large ones are. Z0P_GATES=0 turns gates off as well.
bool gates_enabled() {
  static const bool on = [] {
    const char* g = std::getenv("Z0P_GATES");
    if (g && std::strcmp(g, "0") == 0) return false;
    const char* b = std::getenv("CUDA_LAUNCH_BLOCKING");
    if (b && std::strcmp(b, "1") == 0) return false;
    const char* inj = std::getenv("CUDA_INJECTION64_PATH");
    return !(inj && *inj);
  }();
  return on;
}

// Whether folds l, l+1, ... to the final layer are all small folds (one
// launch that also finishes the next layer's tree, tables read in place),
// so that they can be queued ahead behind gates.
bool gated_tail(const z0p_gpu_ctx* c, const FriShape& s, size_t l) {
  if (!c->gates || !gates_enabled() || l + 1 >= s.len.size()) return false;
  for (size_t j = l; j + 1 < s.len.size(); j++)
    if (s.len[j] < 16 || s.leaves[j + 1] > kFuseMaxLeaves) return false;
  return true;
}

// The gate words of one gated tail, opened in order. Whatever is still
// closed when it is dropped (an early return) is opened then, so that no
// launch queued behind a gate waits out its bound.
struct GateRelease {
  volatile unsigned int* gates = nullptr;
  size_t next = 0, end = 0;
  uint32_t epoch = 0;
  GateRelease() = default;
  GateRelease(const GateRelease&) = delete;  // one owner opens each gate once
  GateRelease& operator=(const GateRelease&) = delete;
  void open_next() {  // after the host has written the inputs behind it
    __atomic_store_n(const_cast<unsigned int*>(gates + next), epoch, __ATOMIC_RELEASE);
    next++;
  }
  ~GateRelease() {
    while (next < end) open_next();
  }
};

// What follows a FRI commitment in a prover: the PoW search and the openings
// gather (prepared, kernels.h OpenArgs), then `after`. When the commitment's
// tail is gated, run_fri_commit queues them behind more gates: the PoW
// search's (word L - 1, L the layer count) and one per query for the gather
// (words L .. L + Q - 1), opened as the host draws each query's index.
struct FriTail {
  OpenArgs* oa = nullptr;
  std::function<cudaError_t()> after;
  bool queued = false;
  GateRelease gates;
};

// FRI commit of one group (src/fri.rs:551-633), layer 0 and its tree
// already queued: fold tables proof by proof on the host, the device work
// of each round for the whole group. A large fold reads its tables from the
// constant slots, a small one from the mapped buffer in place. Once every
// remaining fold is small, they are all queued at once, each behind a gate
// word in the mapped buffer: the host then waits for a layer's event, absorbs
// its cap, writes the next fold's tables and opens its gate, so no launch
// stands between a challenge and its fold.
// cap0_armed: layer 0's cap region was armed (arm_cap) before the kernels
// that write it were queued, so its wait can end as soon as it lands.
int run_fri_commit(z0p_gpu_ctx* c, const FriShape& s, const FriParams& fp, const FriBufs& fb,
                   uint64_t poly_len, uint64_t degree_bound, Transcript* const* ts, uint32_t K,
                   const HioPlan& h, FriOut* outs, FriTail* tail = nullptr, bool cap0_armed = false) {
  uint8_t dims[24];  // src/fri.rs:1450-1456
  for (int i = 0; i < 8; i++) {
    dims[i] = (uint8_t)(s.m >> (8 * i));
    dims[8 + i] = (uint8_t)(poly_len >> (8 * i));
    dims[16 + i] = (uint8_t)(degree_bound >> (8 * i));
  }
  for (uint32_t k = 0; k < K; k++) {
    transcript_absorb(*ts[k], "fri-dims", dims, 24);
    outs[k].caps.assign(s.len.size(), {});
  }
  const size_t L = s.len.size();
  std::vector<bool> armed(L, false);  // cap regions armed before their writers were queued
  armed[0] = cap0_armed;
  auto arm = [&](size_t l) {
    arm_cap(c, h.fri_cap[l], (size_t)h.fri_cap_bytes[l] * K);
    armed[l] = true;
  };
  // Waits for layer l's cap (and, for the last layer, the values in the
  // clear) in the mapped buffer.
  auto wait_layer = [&](size_t l, cudaEvent_t upto) -> cudaError_t {
    if (l + 1 == L) return sync(c, "cap+final", upto);
    if (armed[l]) return wait_cap(c, "cap", h.fri_cap[l], (size_t)h.fri_cap_bytes[l] * K, upto);
    return sync(c, "cap", upto);
  };
  const uint32_t unit_m = to_mont(two_adic_generator(2));
  const uint64_t fl = s.len.back();
  auto tabs = [&](size_t l) {  // layer l's fold tables, proof 0's
    return reinterpret_cast<uint32_t(*)[3][4][4]>(c->hio + h.tabs + 4ull * kFoldTabWords * K * l);
  };
  auto fold_args = [&](size_t l) {
    FoldArgs fa;
    fa.in = fb.layer[l];
    fa.out = fb.layer[l + 1];
    fa.leaves = fb.tree[l + 1];
    fa.logn = log2u(s.len[l]);
    fa.counter = merkle_counter(c);
    fa.slot = (uint32_t)c->slot;
    fa.tab = hio_dev<uint32_t>(c, h.tabs + 4ull * kFoldTabWords * K * l);
    // layer-l domain is 31^(4^l) <omega_len>; its inverse shift:
    uint32_t g = GENERATOR;
    for (size_t i = 0; i < l; i++) g = fpow(g, 4);
    fa.ginv_m = to_mont(finv(g));
    fa.unit_m = unit_m;
    fa.top = s.depth[l + 1] - s.drop[l + 1];
    fa.cap = hio_dev<uint32_t>(c, h.fri_cap[l + 1]);
    fa.in_stride = fa.out_stride = fb.val_stride;
    fa.tree_stride = fb.tree_stride;
    fa.cap_stride = h.fri_cap_bytes[l + 1] / 4;
    if (l + 2 == L) {  // this fold makes the final layer
      fa.final_vals = hio_dev<uint32_t>(c, h.final_vals);
      fa.final_stride = h.final_bytes / 4;
    }
    return fa;
  };
  auto absorb_cap = [&](size_t l) {
    for (uint32_t k = 0; k < K; k++) {
      const uint8_t* cap = c->hio + h.fri_cap[l] + k * h.fri_cap_bytes[l];
      outs[k].caps[l].assign(cap, cap + h.fri_cap_bytes[l]);
      c->d2h += h.fri_cap_bytes[l];  // written by the tree kernel into the mapped buffer
      ts[k]->absorb_each("fri-layer-root", cap, h.fri_cap_bytes[l] / 32, 32);
    }
  };
  // Fold l's challenges into its tables (src/fri.rs:603-606): the constant
  // slots for a large fold, the mapped buffer for a small one.
  auto fold_tables = [&](size_t l, bool slot) {
    const uint32_t inv4 = finv(4);
    for (uint32_t k = 0; k < K; k++) {
      uint32_t ch[3][4];
      for (int r = 0; r < 3; r++) challenge_ext(*ts[k], "fri-fold", ch[r]);
      for (int r = 0; r < 3; r++) {
        uint32_t q[4];
        for (int e = 0; e < 4; e++) q[e] = fmul(ch[r][e], inv4);
        e4_table(q, slot ? c->consts[k].tab[r] : tabs(l)[k][r]);
      }
    }
    if (!slot) c->h2d += 4ull * kFoldTabWords * K;  // read by the fold in place
  };
  if (L == 1) {  // the final layer is layer 0: its values come back by copy
    c->d2h += (uint64_t)K * h.final_bytes;
    CK(cudaMemcpy2DAsync(c->hio + h.final_vals, h.final_bytes, fb.layer.back(), 4 * fb.val_stride,
                         h.final_bytes, K, cudaMemcpyDeviceToHost, c->stream));
  }
  for (size_t l = 0;; l++) {
    if (gated_tail(c, s, l)) {
      while (c->gate_ev.size() < L + 1) {
        cudaEvent_t e;
        CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        c->gate_ev.push_back(e);
      }
      const uint32_t epoch = ++c->go_epoch;
      unsigned int* gates_dev = hio_dev<unsigned int>(c, h.gates);
      GateRelease local;
      GateRelease& rel = tail ? tail->gates : local;
      rel.gates = reinterpret_cast<volatile unsigned int*>(c->hio + h.gates);
      rel.epoch = epoch;
      rel.next = l;
      rel.end = tail ? L + (h.queries ? h.queries : 1) : L - 1;
      // Close every gate of this tail before anything is queued behind it: the
      // mapped buffer is shared by all calls and shapes, so a word left there
      // could otherwise already hold this epoch.
      for (size_t g = l; g < rel.end; g++)
        __atomic_store_n(const_cast<unsigned int*>(rel.gates + g), epoch - 1u, __ATOMIC_RELAXED);
      if (tail) {  // the gather's done words too (open_block reads a block once its word is `epoch`)
        unsigned int* done = reinterpret_cast<unsigned int*>(c->hio + h.done);
        for (size_t i = 0; i < (size_t)K * h.queries; i++)
          __atomic_store_n(done + i, epoch - 1u, __ATOMIC_RELAXED);
      }
      __atomic_thread_fence(__ATOMIC_SEQ_CST);
      for (size_t j = l + 1; j + 1 < L; j++) arm(j);  // written by the folds queued below
      CK(cudaEventRecord(c->gate_ev[l], c->stream));  // layer l's cap
      for (size_t j = l; j + 1 < L; j++) {
        FoldArgs fa = fold_args(j);
        fa.go = gates_dev + j;
        fa.go_epoch = epoch;
        uint32_t built = 0;
        CK(launch::fri_fold(c->stream, c->tb, fa, &built, K));
        CK(cudaEventRecord(c->gate_ev[j + 1], c->stream));  // layer j+1's cap
      }
      if (tail) {
        if (fp.grinding_bits > 0) arm_pow(c, h.grind, K);
        if (fp.grinding_bits > 0)
          CK(launch::grind(c->stream, hio_dev<uint32_t>(c, h.heads), kPowHeadBytes,
                           fp.grinding_bits, grind_state(c),
                           hio_dev<unsigned long long>(c, h.grind), 1ull << 40, K,
                           gates_dev + (L - 1), epoch, c->tb.fault));
        CK(cudaEventRecord(c->gate_ev[L], c->stream));  // the PoW results
        tail->oa->go = gates_dev + L;
        tail->oa->go_per_query = 1;
        tail->oa->go_epoch = epoch;
        tail->oa->done = hio_dev<unsigned int>(c, h.done);
        tail->oa->fault = c->tb.fault;
        CK(launch::openings(c->stream, *tail->oa, K));
        if (tail->after) CK(tail->after());
        tail->queued = true;
      }
      c->d2h += (uint64_t)K * h.final_bytes;  // written by the last fold
      for (size_t j = l;; j++) {
        const bool last = j + 1 == L;
        CK(wait_layer(j, c->gate_ev[j]));
        absorb_cap(j);
        if (last) break;
        fold_tables(j, false);
        rel.open_next();  // gate j
      }
      break;
    }
    const bool last = l + 1 == L;
    // A layer's caps are in the mapped buffer once its trees are done; the
    // last layer's values (sent in the clear) come back in the same trip,
    // written there by the last fold (or copied, when there is no fold).
    if (last && l > 0) c->d2h += (uint64_t)K * h.final_bytes;
    CK(wait_layer(l, nullptr));
    absorb_cap(l);
    if (last) break;
    if (l + 2 < L) arm(l + 1);  // written by this fold or the tree launches after it
    FoldArgs fa = fold_args(l);
    const bool slot = launch::fri_fold_uses_slot(fa);
    fold_tables(l, slot);
    if (slot) CK(push_consts(c, K));
    uint32_t built = 0;  // tree levels the fold kernel hashed itself
    CK(launch::fri_fold(c->stream, c->tb, fa, &built, K));
    // Levels above `built` remain, if any. A tree capped at its leaves has
    // its cap written by the fold only when the fold hashed its subtree (64-
    // byte leaves, small tree); otherwise merkle_build copies it.
    const bool fused = s.len[l] >= 16 && s.leaves[l + 1] <= kFuseMaxLeaves;
    if (built < fa.top || (fa.top == 0 && !fused))
      CK(launch::merkle_build(c->stream, fb.tree[l + 1], s.leaves[l + 1], fa.top,
                              merkle_counter(c), fa.cap, built, K, fb.tree_stride, fa.cap_stride));
  }
  // Final layer in the clear (src/fri.rs:620-621).
  for (uint32_t k = 0; k < K; k++) {
    outs[k].final_vals.resize(4 * fl);
    std::memcpy(outs[k].final_vals.data(), c->hio + h.final_vals + k * h.final_bytes, 16 * fl);
    transcript_absorb(*ts[k], "fri-final", (const uint8_t*)outs[k].final_vals.data(), 16 * fl);
    outs[k].nonce = 0;
  }
  return Z0P_OK;
}

// FRI open of one group up to the openings (src/fri.rs:645-666): the PoW
// nonce, then the query indices.
int run_fri_open(z0p_gpu_ctx* c, const FriShape& s, const FriParams& fp, Transcript* const* ts,
                 uint32_t K, const HioPlan& h, FriOut* outs) {
  // Proof of work (src/fri.rs:645-650, src/transcript.rs:206-228); the heads
  // are read by the search in place.
  if (fp.grinding_bits > 0) {
    uint32_t* heads = reinterpret_cast<uint32_t*>(c->hio + h.heads);
    for (uint32_t k = 0; k < K; k++) {
      std::vector<uint8_t> head = pow_head(*ts[k], "fri-pow");
      set_head(heads + kPowHeadWords * k, head.data(), head.size());
    }
    c->h2d += 4ull * kPowHeadWords * K;
    arm_pow(c, h.grind, K);
    CK(queue_grind(c, fp, hio_dev<uint32_t>(c, h.heads), h.grind, K));
    CK(wait_pow(c, h.grind, K));
    for (uint32_t k = 0; k < K; k++) {
      RC(check_grind(c, h.grind, k, &outs[k].nonce));
      uint8_t nb[8];
      for (int i = 0; i < 8; i++) nb[i] = (uint8_t)(outs[k].nonce >> (8 * i));
      transcript_absorb(*ts[k], "fri-pow", nb, 8);
    }
  }
  for (uint32_t k = 0; k < K; k++) {
    outs[k].indices.resize(fp.num_queries);
    for (uint64_t i = 0; i < fp.num_queries; i++)
      outs[k].indices[i] = challenge_index(*ts[k], "fri-query", s.m);
  }
  return Z0P_OK;
}

// The openings gather's arguments (kernels.h, OpenArgs) for a group: every
// opening lands in the mapped buffer; `oa` arrives with its trace fields and
// strides set.
void prepare_openings(z0p_gpu_ctx* c, const FriShape& s, const FriBufs& fb, const HioPlan& h,
                      OpenArgs& oa) {
  const uint64_t Q = h.queries;
  oa.indices = hio_dev<uint64_t>(c, h.indices);
  oa.out = hio_dev<uint32_t>(c, h.open);
  oa.nq = (uint32_t)Q;
  oa.nlayers = (uint32_t)(s.len.size() - 1);
  oa.stride = h.stride;
  oa.trace_off = h.trace_off;
  oa.fri_val_stride = fb.val_stride;
  oa.fri_tree_stride = fb.tree_stride;
  for (uint32_t d = 0; d < oa.nlayers; d++)
    oa.layer[d] = OpenLayer{fb.layer[d], fb.tree[d], s.leaves[d], s.depth[d] - s.drop[d],
                            h.layer_off[d]};
}

void write_indices(z0p_gpu_ctx* c, const HioPlan& h, const FriOut* outs, uint32_t K) {
  const uint64_t Q = h.queries;
  for (uint32_t k = 0; k < K; k++)
    std::memcpy(c->hio + h.indices + 8 * Q * k, outs[k].indices.data(), 8 * Q);
  c->h2d += 8 * Q * K;                  // indices read in place
  c->d2h += 4ull * h.stride * Q * K;    // opening blocks
}

// Gathers every opening of the group on the device, the query indices known.
int run_openings(z0p_gpu_ctx* c, const FriShape& s, const FriBufs& fb, const HioPlan& h,
                 const FriOut* outs, uint32_t K, OpenArgs& oa) {
  write_indices(c, h, outs, K);
  prepare_openings(c, s, fb, h, oa);
  CK(launch::openings(c->stream, oa, K));
  CK(sync(c, "openings"));
  return Z0P_OK;
}

// A prover's FRI commitment, opening and openings gather (src/fri.rs:551-666
// and the proof's query loop), `oa` carrying the trace fields, `after` any
// kernels that read the query indices after the gather. With a gated tail
// the PoW search and the gather are queued with the folds; the host then
// fills their inputs and opens their gates in turn. Ends with the openings
// in the mapped buffer.
// With `defer` (no `after` kernels), a gated gather is not waited for here:
// the caller reads the blocks through open_block as they land and then calls
// finish_openings; otherwise the openings are complete on return.
int run_fri_openings(z0p_gpu_ctx* c, const FriShape& s, const FriParams& fp, const FriBufs& fb,
                     uint64_t poly_len, uint64_t degree_bound, Transcript* const* ts, uint32_t K,
                     const HioPlan& h, FriOut* outs, OpenArgs& oa,
                     std::function<cudaError_t()> after = {}, bool cap0_armed = false,
                     bool defer = false) {
  c->open_epoch = 0;
  prepare_openings(c, s, fb, h, oa);
  FriTail tail;
  tail.oa = &oa;
  tail.after = after;
  RC(run_fri_commit(c, s, fp, fb, poly_len, degree_bound, ts, K, h, outs, &tail, cap0_armed));
  if (!tail.queued) {
    RC(run_fri_open(c, s, fp, ts, K, h, outs));
    write_indices(c, h, outs, K);
    CK(launch::openings(c->stream, oa, K));
    if (after) CK(after());
    CK(sync(c, "openings"));
    return Z0P_OK;
  }
  if (fp.grinding_bits > 0) {  // src/fri.rs:645-650, src/transcript.rs:206-228
    uint32_t* heads = reinterpret_cast<uint32_t*>(c->hio + h.heads);
    for (uint32_t k = 0; k < K; k++) {
      std::vector<uint8_t> head = pow_head(*ts[k], "fri-pow");
      set_head(heads + kPowHeadWords * k, head.data(), head.size());
    }
    c->h2d += 4ull * kPowHeadWords * K;
    tail.gates.open_next();  // the PoW search's gate
    CK(wait_pow(c, h.grind, K, c->gate_ev[s.len.size()]));
    for (uint32_t k = 0; k < K; k++) {
      RC(check_grind(c, h.grind, k, &outs[k].nonce));
      uint8_t nb[8];
      for (int i = 0; i < 8; i++) nb[i] = (uint8_t)(outs[k].nonce >> (8 * i));
      transcript_absorb(*ts[k], "fri-pow", nb, 8);
    }
  } else {
    tail.gates.open_next();  // nothing behind it
  }
  // Query i's gather starts once index i of every proof is in the mapped
  // buffer, while the host draws the next ones.
  for (uint32_t k = 0; k < K; k++) outs[k].indices.resize(fp.num_queries);
  const uint64_t Q = h.queries;
  for (uint64_t i = 0; i < fp.num_queries; i++) {
    for (uint32_t k = 0; k < K; k++) {
      const uint64_t v = challenge_index(*ts[k], "fri-query", s.m);
      outs[k].indices[i] = v;
      std::memcpy(c->hio + h.indices + 8 * (Q * k + i), &v, 8);
    }
    tail.gates.open_next();  // query i's gate
  }
  while (tail.gates.next < tail.gates.end) tail.gates.open_next();  // (none left: Q queries)
  c->h2d += 8 * Q * K;                // indices read in place
  c->d2h += 4ull * h.stride * Q * K;  // opening blocks
  if (defer && !after) {
    c->open_done = h.done;
    c->open_epoch = tail.gates.epoch;
    return Z0P_OK;
  }
  CK(sync(c, "openings"));
  return Z0P_OK;
}

void write_path(Writer& w, const uint8_t* digests, uint64_t leaf, uint32_t steps) {
  w.u32(steps);  // src/codec.rs:95-101: digest then direction byte (1 = left)
  const size_t len = 33ull * steps;
  if (w.n + len <= w.cap) {  // one capacity check for the whole path
    uint8_t* o = w.p + w.n;
    for (uint32_t s = 0; s < steps; s++, o += 33) {
      std::memcpy(o, digests + 32 * s, 32);
      o[32] = (uint8_t)(((leaf >> s) & 1u) ^ 1u);
    }
  }
  w.n += len;
}

// Opening block of query qi of proof k.
// With openings read as they land, first waits for the block's done word
// (querying the stream every 64 passes: a stream that has drained, or
// failed, ends the wait; the failure is reported by finish_openings).
const uint32_t* open_block(z0p_gpu_ctx* c, const HioPlan& h, uint32_t k, size_t qi) {
  if (c->open_epoch) {
    const volatile uint32_t* w =
        reinterpret_cast<const volatile uint32_t*>(c->hio + c->open_done) + (size_t)k * h.queries + qi;
    for (uint32_t pass = 0; *w != c->open_epoch; pass++)
      if ((pass & 63u) == 63u && cudaStreamQuery(c->stream) != cudaErrorNotReady) break;
    __atomic_thread_fence(__ATOMIC_ACQUIRE);
  }
  return reinterpret_cast<const uint32_t*>(c->hio + h.open) +
         (size_t)h.stride * ((size_t)k * h.queries + qi);
}

// Ends openings read as they land: the stream's synchronisation, after the
// proof bytes are written.
cudaError_t finish_openings(z0p_gpu_ctx* c) {
  c->open_epoch = 0;
  return sync(c, "openings");
}

// Commitment::write_body (src/fri.rs:896-904).
void write_fri_commitment(Writer& w, const FriShape& s, const FriOut& fo, uint64_t poly_len,
                          uint64_t degree_bound) {
  w.u64(s.m);
  w.u64(poly_len);
  w.u64(degree_bound);
  w.u32((uint32_t)fo.caps.size());
  for (auto& cap : fo.caps) {
    w.u32((uint32_t)(cap.size() / 32));
    w.bytes(cap.data(), cap.size());
  }
}

// Proof::write_body (src/fri.rs:352-368), openings from proof k's blocks.
void write_fri_proof(Writer& w, z0p_gpu_ctx* c, const FriShape& s, const FriOut& fo,
                     const HioPlan& h, uint32_t k) {
  w.u32((uint32_t)(fo.final_vals.size() / 4));
  w.bytes(fo.final_vals.data(), 4 * fo.final_vals.size());
  w.u64(fo.nonce);
  w.u32((uint32_t)fo.indices.size());
  size_t L = s.len.size() - 1;
  for (size_t qi = 0; qi < fo.indices.size(); qi++) {
    const uint32_t* blk = open_block(c, h, k, qi);
    w.u32((uint32_t)L);
    uint64_t index = fo.indices[qi];
    for (size_t d = 0; d < L; d++) {
      const uint32_t* at = blk + h.layer_off[d];
      w.bytes(at, 64);
      write_path(w, (const uint8_t*)(at + 16), index / 4, s.depth[d] - s.drop[d]);
      index /= 4;
    }
  }
}

void write_fri(Writer& w, z0p_gpu_ctx* c, const FriShape& s, const FriOut& fo, uint64_t poly_len,
               uint64_t degree_bound, const HioPlan& h, uint32_t k) {
  write_fri_commitment(w, s, fo, poly_len, degree_bound);
  write_fri_proof(w, c, s, fo, h, k);
}

int air_shape(const z0p_air_params& p, FriParams* fp, FriShape* s) {
  RC(air_validate(p));
  // fri_params (src/air.rs:163-169) then commit_ext_evals_owned's checks.
  RC(fri_params_new(p.blowup, p.num_queries, p.final_size, fp));
  fp->grinding_bits = p.grinding_bits;
  fp->cap_height = p.cap_height;
  return fri_shape(p.n_steps * p.blowup, p.n_steps - 1, *fp, s);
}

int range_shape(const z0p_range_params& p, FriParams* fp, FriShape* s) {
  RC(range_validate(p));
  RC(fri_params_new(p.blowup, p.num_queries, p.final_size, fp));
  fp->grinding_bits = p.grinding_bits;
  fp->cap_height = p.cap_height;
  return fri_shape(p.n_rows * p.blowup, p.n_rows - 1, *fp, s);
}

// range::prove_zk's shape (src/range.rs:393-418): rows padded to
// 2^ceil(log2(n + n_rand)), composition bound n + 2 n_rand - 2.
int range_zk_shape(const z0p_range_params& p, uint64_t n_rand, FriParams* fp, FriShape* s) {
  RC(range_validate(p));
  if (n_rand < p.num_queries) {
    set_reason("n_rand must cover num_queries for hiding");
    return Z0P_ERR_MALFORMED_INPUT;
  }
  if (n_rand > MAX_DOMAIN) return Z0P_ERR_INVALID_DOMAIN_SIZE;
  uint64_t lp = 1;
  while (lp < p.n_rows + n_rand) lp <<= 1;
  if (lp > MAX_DOMAIN / p.blowup) return Z0P_ERR_INVALID_DOMAIN_SIZE;
  RC(fri_params_new(p.blowup, p.num_queries, p.final_size, fp));
  fp->grinding_bits = p.grinding_bits;
  fp->cap_height = p.cap_height;
  const uint64_t bound = p.n_rows + 2 * n_rand - 2;
  if (bound >= lp * p.blowup) {
    set_reason("degree bound must be below LDE size (rate < 1)");
    return Z0P_ERR_MALFORMED_INPUT;
  }
  return fri_shape(lp * p.blowup, bound, *fp, s);
}

uint64_t air_size(const z0p_air_params& p, const FriShape& s) {
  uint64_t m = s.m, leaves = m / 8;
  uint32_t depth = log2u(leaves), drop = p.cap_height < depth ? (uint32_t)p.cap_height : depth;
  uint64_t st = depth - drop;  // src/air.rs:262-281
  return 1 + 4 + 32 * (1ull << drop) + fri_bytes(s, p.num_queries) + 4 +
         p.num_queries * (8 + 16 + 4 + 33 * st + 4 + 33 * st + 128);
}

uint64_t range_size(const z0p_range_params& p, const FriShape& s) {
  uint32_t depth = log2u(s.m), drop = p.cap_height < depth ? (uint32_t)p.cap_height : depth;
  uint64_t st = depth - drop;  // src/range.rs:253-269
  return 1 + 4 + 32 * (1ull << drop) + fri_bytes(s, p.num_queries) + 4 +
         p.num_queries * (8 + 4 + 4 + 4 * p.n_bits + 4 + 33 * st);
}

void fib_mats(uint32_t mats[32][4]) {
  uint32_t m00 = 0, m01 = 1, m10 = 1, m11 = 1;  // M = [[0,1],[1,1]]
  for (int k = 0; k < 32; k++) {
    mats[k][0] = m00; mats[k][1] = m01; mats[k][2] = m10; mats[k][3] = m11;
    uint32_t n00 = fadd(fmul(m00, m00), fmul(m01, m10));
    uint32_t n01 = fadd(fmul(m00, m01), fmul(m01, m11));
    uint32_t n10 = fadd(fmul(m10, m00), fmul(m11, m10));
    uint32_t n11 = fadd(fmul(m10, m01), fmul(m11, m11));
    m00 = n00; m01 = n01; m10 = n10; m11 = n11;
  }
}

// One proof of a group: its statement, transcript and output buffer.
template <class Params>
struct Task {
  const Params* p;
  Transcript* ts;
  uint8_t* out;
  size_t cap;
  size_t* len;
  // Composition stage only (z0p_gpu_air_compose): alphas chosen by the
  // caller instead of drawn, and FRI layer 0 copied to this device buffer
  // before the call returns, with no FRI, openings or proof bytes.
  const uint32_t* fixed_alpha = nullptr;
  uint32_t* layer0_out = nullptr;
};
using AirTask = Task<z0p_air_params>;
using RangeTask = Task<z0p_range_params>;

bool same_air_shape(const z0p_air_params& a, const z0p_air_params& b) {
  return a.n_steps == b.n_steps && a.blowup == b.blowup && a.num_queries == b.num_queries &&
         a.final_size == b.final_size && a.grinding_bits == b.grinding_bits &&
         a.cap_height == b.cap_height;
}
bool same_range_shape(const z0p_range_params& a, const z0p_range_params& b) {
  return a.n_rows == b.n_rows && a.n_bits == b.n_bits && a.blowup == b.blowup &&
         a.num_queries == b.num_queries && a.final_size == b.final_size &&
         a.grinding_bits == b.grinding_bits && a.cap_height == b.cap_height;
}

// Validation, sizes and output buffers of a group, before any device work.
template <class T, class Shape, class Size, class Same>
int check_group(const T* tasks, uint32_t K, Shape shape, Size size, Same same, FriParams* fp,
                FriShape* s, uint64_t* need) {
  if (!K || K > (uint32_t)kMaxGroup) return Z0P_ERR_INVALID_ARGUMENT;
  RC(shape(*tasks[0].p, fp, s));
  *need = size(*tasks[0].p, *s);
  for (uint32_t k = 0; k < K; k++) {
    if (k) {
      if (!same(*tasks[0].p, *tasks[k].p)) {
        set_reason("proofs of a group must share their shape (sizes and schedule)");
        return Z0P_ERR_INVALID_ARGUMENT;
      }
      FriParams f2;
      FriShape s2;
      RC(shape(*tasks[k].p, &f2, &s2));  // statement checks (canonical values)
    }
    if (tasks[k].len) *tasks[k].len = *need;
  }
  for (uint32_t k = 0; k < K; k++)
    if (!tasks[k].out || tasks[k].cap < *need) {
      set_reason("output buffer too small for the proof");
      return Z0P_ERR_BUFFER_TOO_SMALL;
    }
  return Z0P_OK;
}

// air::prove_with_trace / prove_zk (src/air.rs:381-399, 439-464) through
// prove_inner (:485-599) with column B committed on its own: both columns
// interpolated (caller's columns, or the Fibonacci trace), masked and padded
// to Lp = 2^ceil(log2(n + n_rand)) coefficients when n_rand > 0, extended to
// m = Lp * blowup, tree over 8-row A || B leaves, the general composition
// (next row m / n further), the FRI and the openings at index and index + m/n.
struct GeneralAir {
  const uint32_t* host_a = nullptr;  // caller's columns (prove_with_trace), else the trace
  const uint32_t* host_b = nullptr;
  uint64_t n_rand = 0;
  const uint32_t* rand = nullptr;    // 2 x n_rand canonical masking values
};

uint64_t padded_len(uint64_t n, uint64_t n_rand) {
  uint64_t total = n + n_rand, lp = 1;
  while (lp < total) lp <<= 1;
  return lp;
}

int general_shape(const z0p_air_params& p, uint64_t n_rand, FriParams* fp, FriShape* s) {
  RC(air_validate(p));
  if (n_rand > (1ull << 27)) return Z0P_ERR_INVALID_DOMAIN_SIZE;
  const uint64_t lp = padded_len(p.n_steps, n_rand);
  if (lp > (1ull << 27)) return Z0P_ERR_INVALID_DOMAIN_SIZE;   // src/blind.rs:62-64
  if (lp > (1ull << 27) / p.blowup) return Z0P_ERR_INVALID_DOMAIN_SIZE;  // src/ntt.rs:347-352
  RC(fri_params_new(p.blowup, p.num_queries, p.final_size, fp));
  fp->grinding_bits = p.grinding_bits;
  fp->cap_height = p.cap_height;
  return fri_shape(lp * p.blowup, p.n_steps + n_rand - 1, *fp, s);
}

int air_prove_general(z0p_gpu_ctx* c, const z0p_air_params& p, const GeneralAir& g,
                      z0p_transcript_state* tsp, uint8_t* out) {
  FriParams fp;
  FriShape s;
  RC(general_shape(p, g.n_rand, &fp, &s));
  const uint64_t N = p.n_steps, B = p.blowup, Lp = padded_len(N, g.n_rand), m = Lp * B;
  const uint32_t logN = log2u(N), logL = log2u(Lp), logB = log2u(B), logm = logL + logB;
  const uint32_t r = (uint32_t)(Lp / N);
  const uint64_t need = air_size(p, s);
  cudaStream_t st = c->stream;
  RC(ensure(c, c->cols, 8 * N));
  RC(ensure(c, c->coeffs, 8 * (N + Lp)));
  RC(ensure(c, c->scratch, 8 * m));
  RC(ensure(c, c->lde, 8 * m));
  const uint64_t tleaves = m / 8, ttree_words = 8 * tree_digests(tleaves);
  RC(ensure(c, c->ttree, 4 * ttree_words));
  RC(ensure(c, c->misc, 64 + 4 * B * r + 8 * g.n_rand));
  FriBufs fb;
  RC(plan_fri_buffers(c, s, 1, &fb));
  const uint32_t tdepth = log2u(tleaves);
  const uint32_t tdrop = p.cap_height < tdepth ? (uint32_t)p.cap_height : tdepth;
  const uint32_t tsteps = tdepth - tdrop;
  HioPlan h;
  RC(plan_hio(c, s, p.num_queries, tdrop, 2 * (16 + 8 * tsteps), 1, &h, 16));
  uint32_t* cols = (uint32_t*)c->cols.p;
  uint32_t* coeffs = (uint32_t*)c->coeffs.p;
  uint32_t* padded = coeffs + 2 * N;
  uint32_t* lde_a = (uint32_t*)c->lde.p;
  uint32_t* lde_b = lde_a + m;
  uint32_t* ttree = (uint32_t*)c->ttree.p;
  uint32_t* zinv = (uint32_t*)c->misc.p + 16;
  uint32_t* rdev = zinv + B * r;
  unsigned int* bad_h = reinterpret_cast<unsigned int*>(c->hio + h.extra);
  *bad_h = 0;
  z0p_transcript_state work = *tsp;
  Transcript t(&work);
  {  // absorb_params (src/air.rs:754-766)
    uint8_t pb[56];
    auto p64 = [&](int off, uint64_t v) { for (int i = 0; i < 8; i++) pb[off + i] = (uint8_t)(v >> (8 * i)); };
    auto p32 = [&](int off, uint32_t v) { for (int i = 0; i < 4; i++) pb[off + i] = (uint8_t)(v >> (8 * i)); };
    p64(0, p.n_steps); p64(8, p.blowup); p64(16, p.num_queries); p64(24, p.final_size);
    p32(32, p.grinding_bits); p64(36, p.cap_height); p32(44, p.a0); p32(48, p.b0); p32(52, p.b_last);
    transcript_absorb(t, "fib/params", pb, 56);
  }
  ProofConsts& pc = c->consts[0];
  pc.a0 = p.a0; pc.b0 = p.b0; pc.b_last = p.b_last;
  CK(push_consts(c, 1));
  if (g.host_a) {
    CK(cudaMemcpyAsync(cols, g.host_a, 4 * N, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(cols + N, g.host_b, 4 * N, cudaMemcpyHostToDevice, st));
    c->h2d += 8 * N;  // checked as the interpolation loads them (NttPlan::bad)
  } else {
    uint32_t mats[32][4];
    fib_mats(mats);
    CK(launch::fib_trace(st, cols, cols + N, (uint32_t)N, (uint32_t)c->slot, mats, 1));
  }
  NttPlan ip;  // interpolate both columns; outputs times 31^i / ... (coset twist included)
  ip.logn = logN; ip.batch = 2; ip.inverse = 1; ip.post_gamma = 1;
  if (g.host_a) ip.bad = hio_dev<unsigned int>(c, h.extra);
  CK(launch::ntt(st, c->tb, ip, cols, coeffs, (uint32_t*)c->scratch.p));
  const uint32_t* lde_in = coeffs;
  if (Lp != N || g.n_rand) {  // T + (x^n - 1) R, zero-padded (src/blind.rs:40-78)
    if (g.n_rand) {
      CK(cudaMemcpyAsync(rdev, g.rand, 8 * g.n_rand, cudaMemcpyHostToDevice, st));
      c->h2d += 8 * g.n_rand;
    }
    CK(launch::mask_pad(st, c->tb, coeffs, rdev, padded, (uint32_t)N, (uint32_t)g.n_rand,
                        (uint32_t)Lp));
    lde_in = padded;
  }
  NttPlan lp;
  lp.logn = logL; lp.batch = (uint32_t)(2 * B); lp.in_div = (uint32_t)B; lp.twist_mod = (uint32_t)B;
  lp.twist_shift = 27 - logm;
  CK(launch::ntt(st, c->tb, lp, lde_in, lde_a, (uint32_t*)c->scratch.p));
  // 1/(x^n - 1) per coset j and q mod r: x^n = (31 omega_m^j omega_Lp^q)^n.
  const uint32_t omega_n = two_adic_generator(logN);
  const uint32_t w_last = fpow(omega_n, N - 1);
  {
    std::vector<uint32_t> zt(B * r);
    const uint32_t omega_m = two_adic_generator(logm), omega_l = two_adic_generator(logL);
    for (uint64_t j = 0; j < B; j++)
      for (uint32_t q = 0; q < r; q++) {
        const uint32_t x = fmul(fmul(GENERATOR, fpow(omega_m, j)), fpow(omega_l, q));
        zt[j * r + q] = to_mont(finv(fsub(fpow(x, N), 1)));
      }
    CK(cudaMemcpyAsync(zinv, zt.data(), 4 * B * r, cudaMemcpyHostToDevice, st));
  }
  // Joint trace tree over 8-row A || B leaves (src/air.rs:520-537) and T.
  uint32_t* tinv = (uint32_t*)c->scratch.p;
  uint32_t built = 0;
  CK(launch::air_trace_leaves(st, c->tb, lde_a, nullptr, to_mont(w_last), ttree, tinv, logL, logB,
                              tsteps, hio_dev<uint32_t>(c, h.trace_cap), merkle_counter(c), &built,
                              1, ttree_words, h.trace_cap_bytes / 4, lde_b));
  if (built < tsteps || (tsteps == 0 && tleaves > kFuseMaxLeaves))
    CK(launch::merkle_build(st, ttree, tleaves, tsteps, merkle_counter(c),
                            hio_dev<uint32_t>(c, h.trace_cap), built, 1, ttree_words,
                            h.trace_cap_bytes / 4));
  CK(sync(c, "cap"));
  if (*reinterpret_cast<volatile unsigned int*>(bad_h)) {
    set_reason("field elements must be canonical (< p)");
    return Z0P_ERR_MALFORMED_INPUT;
  }
  std::vector<uint8_t> column_cap(c->hio + h.trace_cap, c->hio + h.trace_cap + h.trace_cap_bytes);
  c->d2h += h.trace_cap_bytes;
  transcript_absorb(t, "fib/trace", column_cap.data(), column_cap.size());
  uint32_t alpha[5][4];
  for (int i = 0; i < 5; i++) challenge_ext(t, "fib/alpha", alpha[i]);
  const uint32_t omega_inv = finv(omega_n);
  for (int e = 0; e < 4; e++) {
    pc.alpha[e][0] = to_mont(alpha[0][e]);
    pc.alpha[e][1] = to_mont(alpha[1][e]);
    pc.alpha[e][2] = to_mont(fmul(alpha[2][e], omega_inv));
    pc.alpha[e][3] = to_mont(fmul(alpha[3][e], omega_inv));
    pc.alpha[e][4] = to_mont(alpha[4][e]);
  }
  CK(push_consts(c, 1));
  AirComposeArgs ca;
  ca.lde_a = lde_a; ca.cb = nullptr; ca.zinv = zinv; ca.tinv = tinv;
  ca.layer0 = fb.layer[0]; ca.leaves = fb.tree[0];
  ca.logN = logL; ca.logB = logB;
  ca.w_last_m = to_mont(w_last);
  ca.slot = (uint32_t)c->slot;
  CK(launch::air_compose_general(st, c->tb, ca, lde_b, r));
  CK(launch::merkle_build(st, fb.tree[0], s.leaves[0], s.depth[0] - s.drop[0], merkle_counter(c),
                          hio_dev<uint32_t>(c, h.fri_cap[0]), 0, 1, fb.tree_stride,
                          h.fri_cap_bytes[0] / 4));
  Transcript* ts[1] = {&t};
  FriOut fo;
  const uint64_t offset = m / N;
  OpenArgs oa{};
  oa.lde = lde_a; oa.lde_b = lde_b; oa.shift = offset;
  oa.ttree = ttree; oa.tleaves = tleaves; oa.tsteps = tsteps;
  oa.logN = logL; oa.logB = logB; oa.ncol = 0;
  RC(run_fri_openings(c, s, fp, fb, m, N + g.n_rand - 1, ts, 1, h, &fo, oa));
  Writer w(out, need);  // air::Proof::to_bytes (src/air.rs:262-281)
  w.byte(6);
  w.u32((uint32_t)(column_cap.size() / 32));
  w.bytes(column_cap.data(), column_cap.size());
  write_fri(w, c, s, fo, m, N + g.n_rand - 1, h, 0);
  w.u32((uint32_t)fo.indices.size());
  for (size_t qi = 0; qi < fo.indices.size(); qi++) {
    const uint64_t index = brev(fo.indices[qi], logm);
    const uint64_t shifted = (index + offset) % m;
    const uint32_t* rows = open_block(c, h, 0, qi) + h.trace_off;
    const uint32_t* srows = rows + 16 + 8 * tsteps;
    w.u64(index);
    w.u32(rows[2 * (index & 7)]);
    w.u32(rows[2 * (index & 7) + 1]);
    w.u32(srows[2 * (shifted & 7)]);
    w.u32(srows[2 * (shifted & 7) + 1]);
    write_path(w, (const uint8_t*)(rows + 16), index / 8, tsteps);
    write_path(w, (const uint8_t*)(srows + 16), shifted / 8, tsteps);
    w.bytes(rows, 64);
    w.bytes(srows, 64);
  }
  if (w.n != need) {
    set_reason("internal error: proof length differs from its shape");
    return Z0P_ERR_CUDA;
  }
  *tsp = work;
  return Z0P_OK;
}

// table::prove / prove_zk (src/table.rs:305-424) on the device: the value
// column is the constant polynomial [v, 0, ..] (interpolate of a constant),
// masked and padded for prove_zk, extended, hashed as 4-byte row leaves; the
// membership composition, the FRI, and one opening per query.
int table_validate(const z0p_table_params& p) {  // src/table.rs:220-250
  if (p.n_rows < 2 || !is_pow2(p.n_rows)) return Z0P_ERR_INVALID_DOMAIN_SIZE;
  if (p.blowup < 2 || !is_pow2(p.blowup)) return Z0P_ERR_INVALID_BLOWUP;
  if (p.num_queries == 0) return Z0P_ERR_NO_QUERIES;
  if (p.final_size < 2 || !is_pow2(p.final_size)) return Z0P_ERR_INVALID_DOMAIN_SIZE;
  if (p.cap_height > 8) { set_reason("cap_height above 8"); return Z0P_ERR_MALFORMED_INPUT; }
  if (p.n_rows > (1ull << 27) / p.blowup) return Z0P_ERR_INVALID_DOMAIN_SIZE;
  if (p.value >= P) { set_reason("field elements must be canonical (< p)"); return Z0P_ERR_MALFORMED_INPUT; }
  return Z0P_OK;
}

uint64_t membership_bound(uint64_t tlen, uint64_t n, uint64_t n_rand) {  // src/table.rs:364-374
  uint64_t a = n + n_rand < n ? UINT64_MAX : n + n_rand;
  a = a ? a - 1 : 0;
  const uint64_t prod = (a && tlen > UINT64_MAX / a) ? UINT64_MAX : tlen * a;
  return prod > n ? prod - n : 0;
}

int table_shape(const z0p_table_params& p, const uint32_t* table, size_t tlen, uint64_t n_rand,
                FriParams* fp, FriShape* s, uint64_t* bytes) {
  RC(table_validate(p));
  if (tlen < 2) {  // src/table.rs:291-298
    set_reason("table needs at least two entries");
    return Z0P_ERR_MALFORMED_INPUT;
  }
  if (n_rand && n_rand < p.num_queries) {  // src/table.rs:338-342
    set_reason("n_rand must cover num_queries for hiding");
    return Z0P_ERR_MALFORMED_INPUT;
  }
  if (table)
    for (size_t i = 0; i < tlen; i++)
      if (table[i] >= P) {
        set_reason("field elements must be canonical (< p)");
        return Z0P_ERR_MALFORMED_INPUT;
      }
  const uint64_t lp = padded_len(p.n_rows, n_rand);
  if (lp > (1ull << 27) || lp > (1ull << 27) / p.blowup) return Z0P_ERR_INVALID_DOMAIN_SIZE;
  RC(fri_params_new(p.blowup, p.num_queries, p.final_size, fp));
  fp->grinding_bits = p.grinding_bits;
  fp->cap_height = p.cap_height;
  const uint64_t m = lp * p.blowup;
  const uint64_t bound = membership_bound(tlen, p.n_rows, n_rand);
  if (bound >= m) {
    set_reason("degree bound must be below LDE size (rate < 1)");
    return Z0P_ERR_MALFORMED_INPUT;
  }
  RC(fri_shape(m, bound, *fp, s));
  const uint32_t depth = log2u(m), drop = p.cap_height < depth ? (uint32_t)p.cap_height : depth;
  *bytes = 1 + 4 + 32ull * (1ull << drop) + fri_bytes(*s, p.num_queries) + 4 +
           p.num_queries * (8 + 4 + 4 + 33ull * (depth - drop));  // src/table.rs:244-262
  return Z0P_OK;
}

// ------------------------------------------------- constant traces ----
// range::prove builds every column as one repeated value (src/range.rs:
// 316-330), and table::prove one column of one value (src/table.rs:305-317).
// The coset LDE of a constant is that constant, so:
//  - every trace row is the same, and each level of the trace tree is one
//    repeated digest;
//  - the composition is one Ext4 constant K_j per coset j: for range
//    (src/range.rs:678-774), (v - sum 2^c b_c) zinv_j alpha_d, since the
//    boolean terms vanish (bits are 0 or 1) and so does the boundary term
//    (v = value); for table (src/table.rs:646-660), alpha_m prod_k (v - T_k)
//    zinv_j. K is zero for an in-range value or a table member;
//  - an arity-4 fold of four equal values returns that value (the three
//    non-constant components of the quad are zero), and the four rows of a
//    quad share their coset while the layer holds at least 4B values. So
//    FRI layer l, of length L >= B, holds K_j at position x with
//    j = brev(x >> (log L - log B), log B): runs of L / B equal values, in
//    every layer, whatever the fold challenges.
// Each tree is then G groups of equal leaves (UniformTree): one chain of
// node hashes per group and a tree over the group roots. The proof bytes are
// the generic path's (tests compare both against the oracle).
struct CompactTree {
  const uint8_t* out;  // UniformTree::out, as the host holds it
  uint32_t G, logS;
  const uint8_t* node(uint32_t l, uint64_t i) const {
    if (l <= logS) return out + 32 * ((i >> (logS - l)) * (logS + 1) + l);
    const uint32_t tl = l - logS;
    return out + 32 * ((uint64_t)G * (logS + 1) + (2ull * G - 2ull * (G >> tl)) + i);
  }
  // Siblings from the leaf up to the cap (`steps` levels) into buf.
  const uint8_t* path(uint64_t leaf, uint32_t steps, std::vector<uint8_t>& buf) const {
    buf.resize(32 * (size_t)steps);
    for (uint32_t l = 0; l < steps; l++) std::memcpy(&buf[32 * l], node(l, (leaf >> l) ^ 1), 32);
    return buf.data();
  }
};

// A compact tree as one launch of uniform_trees builds it: its seeds go in,
// its digests come back into `bytes`.
struct ConstTree {
  uint32_t G = 1, logS = 0, row = 0, words = 16;
  std::vector<uint32_t> seeds;  // G x words
  std::vector<uint8_t> bytes;   // G (logS + 1) + 2G - 1 digests
  CompactTree view() const { return CompactTree{bytes.data(), G, logS}; }
};

// Builds every tree in one launch through the mapped buffer and waits.
int build_const_trees(z0p_gpu_ctx* c, std::vector<ConstTree*>& trees, const char* site) {
  size_t at = 0;
  auto take = [&](size_t bytes) {
    size_t r = at;
    at += (bytes + 15) & ~(size_t)15;
    return r;
  };
  const size_t n = trees.size();
  const size_t desc = take(sizeof(UniformTree) * n);
  std::vector<size_t> sd(n), od(n);
  for (size_t i = 0; i < n; i++) {
    const ConstTree& t = *trees[i];
    if (t.G == 0 || t.G > 512 || (t.G & (t.G - 1)) || t.seeds.size() != (size_t)t.G * t.words) {
      set_reason("internal error: compact tree shape");
      return Z0P_ERR_CUDA;
    }
    sd[i] = take(4 * t.seeds.size());
    od[i] = take(32ull * ((uint64_t)t.G * (t.logS + 1) + 2 * t.G - 1));
  }
  RC(ensure_hio(c, at));
  UniformTree* u = reinterpret_cast<UniformTree*>(c->hio + desc);
  for (size_t i = 0; i < n; i++) {
    const ConstTree& t = *trees[i];
    std::memcpy(c->hio + sd[i], t.seeds.data(), 4 * t.seeds.size());
    u[i] = UniformTree{hio_dev<uint32_t>(c, sd[i]), hio_dev<uint32_t>(c, od[i]), t.G, t.logS, t.row,
                       t.words};
    c->h2d += 4 * t.seeds.size() + sizeof(UniformTree);
  }
  CK(launch::uniform_trees(c->stream, hio_dev<UniformTree>(c, desc), (uint32_t)n));
  CK(sync(c, site));
  for (size_t i = 0; i < n; i++) {
    ConstTree& t = *trees[i];
    t.bytes.assign(c->hio + od[i], c->hio + od[i] + 32ull * ((uint64_t)t.G * (t.logS + 1) + 2 * t.G - 1));
    c->d2h += t.bytes.size();
  }
  return Z0P_OK;
}

// FRI over a composition that is one Ext4 constant per coset (kc: 4B words,
// canonical; null: zero), as fri::commit_ext_evals then fri::open
// (src/fri.rs:551-666) drive the transcript, from compact trees. Layer l of
// length 2^logL >= B holds K_j at x, j = brev(x >> (logL - logB), logB).
struct ConstFri {
  const uint32_t* kc = nullptr;
  uint32_t logB = 0;
  std::vector<ConstTree> trees;  // per layer
  FriOut fo;
  const uint32_t* val(uint32_t logL, uint64_t x) const {
    static const uint32_t z4[4] = {0, 0, 0, 0};
    return kc ? kc + 4 * brev(x >> (logL - logB), logB) : z4;
  }
};

bool const_fri_ok(const FriShape& s, bool zero, uint64_t rows, uint64_t blowup) {
  if (s.len.back() < 4) return false;  // quad leaves in every layer
  for (size_t l = 0; l < s.len.size(); l++)
    if (s.leaves[l] * 4 != s.len[l]) return false;
  if (zero) return true;
  return rows >= 4 && s.len.back() >= blowup && blowup <= 512;
}

// The seeds of every FRI tree of K proofs (their K_j known); `all`
// receives the trees to build.
void prepare_const_fri(const FriShape& s, uint32_t K, ConstFri* fr, std::vector<ConstTree*>* all) {
  const size_t nl = s.len.size();
  for (uint32_t k = 0; k < K; k++) {
    ConstFri& f = fr[k];
    const uint32_t logB = f.logB;
    f.trees.assign(nl, ConstTree{});
    for (size_t l = 0; l < nl; l++) {
      ConstTree& t = f.trees[l];
      const uint32_t logL = log2u(s.len[l]), logNL = logL - 2;
      if (!f.kc) {
        t.G = 1;
        t.logS = logNL;
      } else if (logL >= logB + 2) {
        t.G = 1u << logB;
        t.logS = logNL - logB;
      } else {
        t.G = 1u << logNL;
        t.logS = 0;
      }
      t.seeds.resize(16ull * t.G);
      for (uint32_t g = 0; g < t.G; g++) {
        const uint64_t leaf = (uint64_t)g << t.logS;  // any leaf of the group
        for (int q = 0; q < 4; q++) std::memcpy(&t.seeds[16 * g + 4 * q], f.val(logL, 4 * leaf + q), 16);
      }
      all->push_back(&t);
    }
  }
}

// With `built`, the trees are already there (a zero composition's trees
// depend on the shape alone and go with the trace tree's launch).
int const_fri(z0p_gpu_ctx* c, const FriShape& s, const FriParams& fp, uint64_t poly_len,
              uint64_t degree_bound, Transcript* const* ts, uint32_t K, ConstFri* fr,
              bool built = false) {
  const size_t nl = s.len.size();
  if (!built) {
    std::vector<ConstTree*> all;
    prepare_const_fri(s, K, fr, &all);
    RC(build_const_trees(c, all, "cap"));
  }
  uint8_t dims[24];  // src/fri.rs:1450-1456
  for (int i = 0; i < 8; i++) {
    dims[i] = (uint8_t)(s.m >> (8 * i));
    dims[8 + i] = (uint8_t)(poly_len >> (8 * i));
    dims[16 + i] = (uint8_t)(degree_bound >> (8 * i));
  }
  const uint64_t F = s.len.back();
  for (uint32_t k = 0; k < K; k++) {
    Transcript& t = *ts[k];
    ConstFri& f = fr[k];
    transcript_absorb(t, "fri-dims", dims, 24);
    f.fo.caps.assign(nl, {});
    for (size_t l = 0; l < nl; l++) {
      const CompactTree tr = f.trees[l].view();
      const uint32_t steps = s.depth[l] - s.drop[l];
      std::vector<uint8_t>& cap = f.fo.caps[l];
      cap.resize(32ull << s.drop[l]);
      for (uint64_t i = 0; i < (1ull << s.drop[l]); i++) std::memcpy(&cap[32 * i], tr.node(steps, i), 32);
      t.absorb_each("fri-layer-root", cap.data(), cap.size() / 32, 32);
      if (l + 1 == nl) break;
      uint32_t ch[4];
      for (int r = 0; r < 3; r++) challenge_ext(t, "fri-fold", ch);  // the values do not depend on them
    }
    f.fo.final_vals.resize(4 * F);
    const uint32_t logF = log2u(F);
    for (uint64_t x = 0; x < F; x++) std::memcpy(&f.fo.final_vals[4 * x], f.val(logF, x), 16);
    transcript_absorb(t, "fri-final", (const uint8_t*)f.fo.final_vals.data(), 16 * F);
    f.fo.nonce = 0;
  }
  if (fp.grinding_bits > 0) {  // src/fri.rs:645-650
    const size_t heads_at = 16ull * K;  // results first, then the heads
    RC(ensure_hio(c, heads_at + 4ull * kPowHeadWords * K));
    uint32_t* heads = reinterpret_cast<uint32_t*>(c->hio + heads_at);
    for (uint32_t k = 0; k < K; k++) {
      std::vector<uint8_t> head = pow_head(*ts[k], "fri-pow");
      set_head(heads + kPowHeadWords * k, head.data(), head.size());
    }
    c->h2d += 4ull * kPowHeadWords * K;
    arm_pow(c, 0, K);
    CK(queue_grind(c, fp, hio_dev<uint32_t>(c, heads_at), 0, K));
    CK(wait_pow(c, 0, K));
    for (uint32_t k = 0; k < K; k++) {
      RC(check_grind(c, 0, k, &fr[k].fo.nonce));
      uint8_t nb[8];
      for (int i = 0; i < 8; i++) nb[i] = (uint8_t)(fr[k].fo.nonce >> (8 * i));
      transcript_absorb(*ts[k], "fri-pow", nb, 8);
    }
  }
  for (uint32_t k = 0; k < K; k++) {
    fr[k].fo.indices.resize(fp.num_queries);
    for (uint64_t i = 0; i < fp.num_queries; i++)
      fr[k].fo.indices[i] = challenge_index(*ts[k], "fri-query", s.m);
  }
  return Z0P_OK;
}

// Commitment::to_bytes and Proof::to_bytes (src/fri.rs:352-368, 896-904)
// of a ConstFri.
void write_const_fri(Writer& w, const FriShape& s, const ConstFri& f, uint64_t poly_len,
                     uint64_t degree_bound) {
  write_fri_commitment(w, s, f.fo, poly_len, degree_bound);
  const uint64_t F = s.len.back();
  const size_t nl = s.len.size();
  w.u32((uint32_t)F);
  w.bytes(f.fo.final_vals.data(), 16 * F);
  w.u64(f.fo.nonce);
  w.u32((uint32_t)f.fo.indices.size());
  std::vector<uint8_t> pbuf;
  for (size_t qi = 0; qi < f.fo.indices.size(); qi++) {
    w.u32((uint32_t)(nl - 1));
    uint64_t index = f.fo.indices[qi];
    for (size_t d = 0; d + 1 < nl; d++) {
      const uint32_t logL = log2u(s.len[d]);
      const uint64_t leaf = index / 4;
      for (int q = 0; q < 4; q++) {
        const uint32_t* v = f.val(logL, 4 * leaf + q);
        for (int e = 0; e < 4; e++) w.u32(v[e]);
      }
      const uint32_t steps = s.depth[d] - s.drop[d];
      write_path(w, f.trees[d].view().path(leaf, steps, pbuf), leaf, steps);
      index /= 4;
    }
  }
}

// The trace trees of constant rows: K rows of `words` words, one tree of m
// equal leaves each; returns the trees (digest chains) and their caps.
int const_trace_trees(z0p_gpu_ctx* c, const std::vector<std::vector<uint32_t>>& rows,
                      uint32_t logm, uint32_t tdrop, std::vector<ConstTree>* trees,
                      std::vector<std::vector<uint8_t>>* caps,
                      std::vector<ConstTree*> all = {}) {  // `all`: more trees for the same launch
  const size_t K = rows.size();
  trees->assign(K, ConstTree{});
  for (size_t k = 0; k < K; k++) {
    ConstTree& t = (*trees)[k];
    t.G = 1;
    t.logS = logm;
    t.row = 1;
    t.words = (uint32_t)rows[k].size();
    t.seeds = rows[k];
    all.push_back(&t);
  }
  RC(build_const_trees(c, all, "cap"));
  caps->assign(K, {});
  for (size_t k = 0; k < K; k++) {
    const CompactTree tt = (*trees)[k].view();
    (*caps)[k].resize(32ull << tdrop);
    for (uint64_t i = 0; i < (1ull << tdrop); i++)
      std::memcpy(&(*caps)[k][32 * i], tt.node(logm - tdrop, i), 32);
  }
  return Z0P_OK;
}

// table::prove on its constant column (src/table.rs:305-317 proves
// vec![value; n]): the trace tree is one chain of equal leaves and the
// composition (src/table.rs:646-660) is alpha_m prod_k (value - T_k) zinv_j
// per coset (the boundary term vanishes, v = value); see range_prove_const.
int table_prove_const(z0p_gpu_ctx* c, const z0p_table_params& p, const uint32_t* table, size_t tlen,
                      const FriParams& fp, const FriShape& s, uint64_t need,
                      z0p_transcript_state* tsp, uint8_t* out) {
  const uint64_t N = p.n_rows, B = p.blowup, m = N * B;
  const uint32_t logB = log2u(B), logm = log2u(m);
  const uint32_t tdrop = p.cap_height < logm ? (uint32_t)p.cap_height : logm;
  const uint32_t tsteps = logm - tdrop;
  z0p_transcript_state work = *tsp;
  Transcript t(&work);
  {  // absorb_params (src/table.rs:540-554)
    std::vector<uint8_t> pb(56 + 4 * tlen);
    auto p64 = [&](size_t off, uint64_t v) { for (int i = 0; i < 8; i++) pb[off + i] = (uint8_t)(v >> (8 * i)); };
    auto p32 = [&](size_t off, uint32_t v) { for (int i = 0; i < 4; i++) pb[off + i] = (uint8_t)(v >> (8 * i)); };
    p64(0, p.n_rows); p64(8, p.blowup); p64(16, p.num_queries); p64(24, p.final_size);
    p32(32, p.grinding_bits); p64(36, p.cap_height); p32(44, p.value); p64(48, tlen);
    for (size_t i = 0; i < tlen; i++) p32(56 + 4 * i, table[i]);
    transcript_absorb(t, "table/params", pb.data(), pb.size());
  }
  uint32_t prod = 1;
  for (size_t i = 0; i < tlen; i++) prod = fmul(prod, fsub(p.value, table[i]));
  ConstFri fr;
  fr.logB = logB;
  std::vector<ConstTree*> early;  // a member's FRI trees: all-zero layers
  if (!prod) prepare_const_fri(s, 1, &fr, &early);
  std::vector<ConstTree> ttrees;
  std::vector<std::vector<uint8_t>> tcap;
  RC(const_trace_trees(c, {{p.value}}, logm, tdrop, &ttrees, &tcap, early));  // from_flat(.., 4) leaves
  transcript_absorb(t, "table/column", tcap[0].data(), tcap[0].size());
  uint32_t am[4], ab[4];
  challenge_ext(t, "table/alpha", am);
  challenge_ext(t, "table/alpha", ab);
  std::vector<uint32_t> kc;
  if (prod) {
    kc.assign(4 * B, 0u);
    const uint32_t wB = two_adic_generator(logB);
    uint32_t xn = fpow(GENERATOR, N);  // x^N on coset j: 31^N omega_B^j
    for (uint64_t j = 0; j < B; j++) {
      const uint32_t base = fmul(prod, finv(fsub(xn, 1)));
      for (int e = 0; e < 4; e++) kc[4 * j + e] = fmul(base, am[e]);
      xn = fmul(xn, wB);
    }
    fr.kc = kc.data();
  }
  const uint64_t bound = membership_bound(tlen, N, 0);
  Transcript* ts[1] = {&t};
  RC(const_fri(c, s, fp, m, bound, ts, 1, &fr, !prod));
  Writer w(out, need);  // table::Proof::to_bytes (src/table.rs:244-262)
  w.byte(6);
  w.u32((uint32_t)(tcap[0].size() / 32));
  w.bytes(tcap[0].data(), tcap[0].size());
  write_const_fri(w, s, fr, m, bound);
  w.u32((uint32_t)fr.fo.indices.size());
  const CompactTree tt = ttrees[0].view();
  std::vector<uint8_t> pbuf;
  for (size_t qi = 0; qi < fr.fo.indices.size(); qi++) {
    const uint64_t index = brev(fr.fo.indices[qi], logm);
    w.u64(index);
    w.u32(p.value);
    write_path(w, tt.path(index, tsteps, pbuf), index, tsteps);
  }
  if (w.n != need) {
    set_reason("internal error: proof length differs from its shape");
    return Z0P_ERR_CUDA;
  }
  *tsp = work;
  return Z0P_OK;
}

int table_prove_dev(z0p_gpu_ctx* c, const z0p_table_params& p, const uint32_t* table, size_t tlen,
                    uint64_t n_rand, const uint32_t* rand, z0p_transcript_state* tsp,
                    uint8_t* out) {
  FriParams fp;
  FriShape s;
  uint64_t need = 0;
  RC(table_shape(p, table, tlen, n_rand, &fp, &s, &need));
  if (n_rand == 0) {
    uint32_t prod = 1;
    for (size_t i = 0; i < tlen; i++) prod = fmul(prod, fsub(p.value, table[i]));
    if (const_fri_ok(s, prod == 0, p.n_rows, p.blowup))
      return table_prove_const(c, p, table, tlen, fp, s, need, tsp, out);
  }
  const uint64_t N = p.n_rows, B = p.blowup, Lp = padded_len(N, n_rand), m = Lp * B;
  const uint32_t logN = log2u(N), logL = log2u(Lp), logB = log2u(B), logm = logL + logB;
  const uint32_t r = (uint32_t)(Lp / N);
  cudaStream_t st = c->stream;
  RC(ensure(c, c->coeffs, 4 * (N + Lp)));
  RC(ensure(c, c->scratch, 4 * m));
  RC(ensure(c, c->lde, 4 * m));
  const uint64_t ttree_words = 8 * tree_digests(m);
  RC(ensure(c, c->ttree, 4 * ttree_words));
  RC(ensure(c, c->misc, 64 + 4 * B * r + 4 * n_rand + 4 * tlen + 4 * m));
  FriBufs fb;
  RC(plan_fri_buffers(c, s, 1, &fb));
  const uint32_t tdrop = p.cap_height < logm ? (uint32_t)p.cap_height : logm;
  const uint32_t tsteps = logm - tdrop;
  HioPlan h;
  RC(plan_hio(c, s, p.num_queries, tdrop, 1 + 8 * tsteps, 1, &h));
  uint32_t* coeffs = (uint32_t*)c->coeffs.p;
  uint32_t* lde = (uint32_t*)c->lde.p;
  uint32_t* ttree = (uint32_t*)c->ttree.p;
  uint32_t* zinv = (uint32_t*)c->misc.p + 16;
  uint32_t* rdev = zinv + B * r;
  uint32_t* tdev = rdev + n_rand;
  uint32_t* tinv = tdev + tlen;
  z0p_transcript_state work = *tsp;
  Transcript t(&work);
  {  // absorb_params (src/table.rs:540-554)
    std::vector<uint8_t> pb(56 + 4 * tlen);
    auto p64 = [&](size_t off, uint64_t v) { for (int i = 0; i < 8; i++) pb[off + i] = (uint8_t)(v >> (8 * i)); };
    auto p32 = [&](size_t off, uint32_t v) { for (int i = 0; i < 4; i++) pb[off + i] = (uint8_t)(v >> (8 * i)); };
    p64(0, p.n_rows); p64(8, p.blowup); p64(16, p.num_queries); p64(24, p.final_size);
    p32(32, p.grinding_bits); p64(36, p.cap_height); p32(44, p.value); p64(48, tlen);
    for (size_t i = 0; i < tlen; i++) p32(56 + 4 * i, table[i]);
    transcript_absorb(t, "table/params", pb.data(), pb.size());
  }
  // interpolate(vec![value; n]) = [value, 0, ..] (src/table.rs:307-309).
  CK(cudaMemsetAsync(coeffs, 0, 4 * N, st));
  CK(cudaMemcpyAsync(coeffs, &p.value, 4, cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(tdev, table, 4 * tlen, cudaMemcpyHostToDevice, st));
  c->h2d += 4 + 4 * tlen;
  const uint32_t* lde_in = coeffs;
  if (Lp != N || n_rand) {
    if (n_rand) {
      CK(cudaMemcpyAsync(rdev, rand, 4 * n_rand, cudaMemcpyHostToDevice, st));
      c->h2d += 4 * n_rand;
    }
    CK(launch::mask_pad(st, c->tb, coeffs, rdev, coeffs + N, (uint32_t)N, (uint32_t)n_rand,
                        (uint32_t)Lp, 1));
    lde_in = coeffs + N;
  }
  // The twisted coefficients: [value, 0, ..] already equal c_k 31^k.
  NttPlan lp;
  lp.logn = logL; lp.batch = (uint32_t)B; lp.in_div = (uint32_t)B; lp.twist_mod = (uint32_t)B;
  lp.twist_shift = 27 - logm;
  CK(launch::ntt(st, c->tb, lp, lde_in, lde, (uint32_t*)c->scratch.p));
  uint32_t tbuilt = 0;  // from_flat(.., 4) leaves; small trees finished in the launch
  CK(launch::range_trace_leaves(st, lde, ttree, logL, logB, 1, 1, 0, merkle_counter(c), tsteps,
                                hio_dev<uint32_t>(c, h.trace_cap), 0, &tbuilt));
  if (tbuilt == 0)
    CK(launch::merkle_build(st, ttree, m, tsteps, merkle_counter(c), hio_dev<uint32_t>(c, h.trace_cap)));
  const uint32_t omega_n = two_adic_generator(logN);
  const uint32_t omega_inv = finv(omega_n);
  CK(launch::row_inverses(st, c->tb, tinv, to_mont(omega_inv), logL, logB));
  {
    std::vector<uint32_t> zt(B * r);
    const uint32_t omega_m = two_adic_generator(logm), omega_l = two_adic_generator(logL);
    for (uint64_t j = 0; j < B; j++)
      for (uint32_t q = 0; q < r; q++) {
        const uint32_t x = fmul(fmul(GENERATOR, fpow(omega_m, j)), fpow(omega_l, q));
        zt[j * r + q] = to_mont(finv(fsub(fpow(x, N), 1)));
      }
    CK(cudaMemcpyAsync(zinv, zt.data(), 4 * B * r, cudaMemcpyHostToDevice, st));
  }
  CK(sync(c, "cap"));
  std::vector<uint8_t> column_cap(c->hio + h.trace_cap, c->hio + h.trace_cap + h.trace_cap_bytes);
  c->d2h += h.trace_cap_bytes;
  transcript_absorb(t, "table/column", column_cap.data(), column_cap.size());
  uint32_t am[4], ab[4];
  challenge_ext(t, "table/alpha", am);
  challenge_ext(t, "table/alpha", ab);
  TableComposeArgs ca;
  ca.lde = lde; ca.tinv = tinv; ca.zinv = zinv; ca.table = tdev;
  ca.table_len = (uint32_t)tlen;
  ca.corr_m = fpow((uint32_t)((1ull << 32) % P), tlen);
  ca.value = p.value;
  for (int e = 0; e < 4; e++) {
    ca.alpha_m[e] = to_mont(am[e]);
    ca.alpha_b[e] = to_mont(fmul(ab[e], omega_inv));
  }
  ca.layer0 = fb.layer[0]; ca.leaves = fb.tree[0];
  ca.logN = logL; ca.logB = logB; ca.r = r;
  CK(launch::table_compose(st, c->tb, ca));
  CK(launch::merkle_build(st, fb.tree[0], s.leaves[0], s.depth[0] - s.drop[0], merkle_counter(c),
                          hio_dev<uint32_t>(c, h.fri_cap[0]), 0, 1, fb.tree_stride,
                          h.fri_cap_bytes[0] / 4));
  Transcript* ts[1] = {&t};
  FriOut fo;
  const uint64_t bound = membership_bound(tlen, N, n_rand);
  OpenArgs oa{};  // src/table.rs:412-420
  oa.lde = lde; oa.ttree = ttree; oa.tleaves = m; oa.tsteps = tsteps;
  oa.logN = logL; oa.logB = logB; oa.ncol = 1;
  RC(run_fri_openings(c, s, fp, fb, m, bound, ts, 1, h, &fo, oa));
  Writer w(out, need);  // table::Proof::to_bytes (src/table.rs:244-262)
  w.byte(6);
  w.u32((uint32_t)(column_cap.size() / 32));
  w.bytes(column_cap.data(), column_cap.size());
  write_fri(w, c, s, fo, m, bound, h, 0);
  w.u32((uint32_t)fo.indices.size());
  for (size_t qi = 0; qi < fo.indices.size(); qi++) {
    const uint64_t index = brev(fo.indices[qi], logm);
    const uint32_t* row = open_block(c, h, 0, qi) + h.trace_off;
    w.u64(index);
    w.u32(row[0]);
    write_path(w, (const uint8_t*)(row + 1), index, tsteps);
  }
  if (w.n != need) {
    set_reason("internal error: proof length differs from its shape");
    return Z0P_ERR_CUDA;
  }
  *tsp = work;
  return Z0P_OK;
}

// src/air.rs:365-372 -> 485-599 on the device, for K proofs of one shape in
// lockstep: every launch covers the group (grid y = proof) and every
// Fiat-Shamir round trip serves it.
int air_prove(z0p_gpu_ctx* c, const AirTask* tasks, uint32_t K) {
  FriParams fp;
  FriShape s;
  uint64_t need = 0;
  RC(check_group(tasks, K, air_shape, air_size, same_air_shape, &fp, &s, &need));
  const z0p_air_params& p0 = *tasks[0].p;
  const uint64_t N = p0.n_steps, B = p0.blowup, m = N * B;
  const uint32_t logN = log2u(N), logB = log2u(B), logm = logN + logB;
  cudaStream_t st = c->stream;

  RC(ensure_slots(c, K));
  RC(ensure(c, c->cols, 8 * N * K));
  RC(ensure(c, c->coeffs, 4 * N * K));
  RC(ensure(c, c->scratch, 4 * m * K));
  RC(ensure(c, c->lde, 4 * m * K));
  const uint64_t tleaves = m / 8, ttree_words = 8 * tree_digests(tleaves);
  RC(ensure(c, c->ttree, 4 * ttree_words * K));
  RC(ensure(c, c->misc, 64 + 8 * B + 4 * B * K));
  FriBufs fb;
  RC(plan_fri_buffers(c, s, K, &fb));
  const uint32_t tdepth = log2u(tleaves);
  const uint32_t tdrop = p0.cap_height < tdepth ? (uint32_t)p0.cap_height : tdepth;
  const uint32_t tsteps = tdepth - tdrop;
  HioPlan h;
  RC(plan_hio(c, s, p0.num_queries, tdrop, 2 * (16 + 8 * tsteps), K, &h));
  uint32_t* cols = (uint32_t*)c->cols.p;
  uint32_t* coeffs = (uint32_t*)c->coeffs.p;
  uint32_t* lde = (uint32_t*)c->lde.p;
  uint32_t* ttree = (uint32_t*)c->ttree.p;
  uint32_t* zinv = (uint32_t*)c->misc.p + 16;
  uint32_t* zinv2 = zinv + B;
  uint32_t* cb = zinv2 + B;  // K x B: per-proof linked-column constants

  uint32_t mats[32][4];
  fib_mats(mats);
  // C_j = coeff * (x^N - 1) with coeff = (B[N-1] - a0) w_last / N, where
  // B[N-1] is the actual last trace value (src/air.rs:366-371, 817-821).
  const uint32_t omega_n = two_adic_generator(logN);
  const uint32_t w_last = fpow(omega_n, N - 1);
  const uint32_t n_inv = finv((uint32_t)(N % P));
  // (A[N-1], B[N-1]) = M^(N-1) (a0, b0) from the binary powers of M.
  uint32_t r00 = 1, r01 = 0, r10 = 0, r11 = 1;
  for (int k = 0; k < 32; k++)
    if (((N - 1) >> k) & 1) {
      const uint32_t* q = mats[k];
      uint32_t n00 = fadd(fmul(r00, q[0]), fmul(r01, q[2])), n01 = fadd(fmul(r00, q[1]), fmul(r01, q[3]));
      uint32_t n10 = fadd(fmul(r10, q[0]), fmul(r11, q[2])), n11 = fadd(fmul(r10, q[1]), fmul(r11, q[3]));
      r00 = n00; r01 = n01; r10 = n10; r11 = n11;
    }
  std::vector<uint32_t> coeff(K);
  for (uint32_t k = 0; k < K; k++) {
    const z0p_air_params& p = *tasks[k].p;
    // absorb_params (src/air.rs:754-766)
    uint8_t pb[56];
    auto p64 = [&](int off, uint64_t v) { for (int i = 0; i < 8; i++) pb[off + i] = (uint8_t)(v >> (8 * i)); };
    auto p32 = [&](int off, uint32_t v) { for (int i = 0; i < 4; i++) pb[off + i] = (uint8_t)(v >> (8 * i)); };
    p64(0, p.n_steps); p64(8, p.blowup); p64(16, p.num_queries); p64(24, p.final_size);
    p32(32, p.grinding_bits); p64(36, p.cap_height); p32(44, p.a0); p32(48, p.b0); p32(52, p.b_last);
    transcript_absorb(*tasks[k].ts, "fib/params", pb, 56);
    const uint32_t b_actual = fadd(fmul(r10, p.a0), fmul(r11, p.b0));
    coeff[k] = fmul(fmul(fsub(b_actual, p.a0), w_last), n_inv);
    ProofConsts& pc = c->consts[k];
    pc.a0 = p.a0; pc.b0 = p.b0; pc.b_last = p.b_last;
    pc.coeff = coeff[k];
  }
  const uint32_t slot = (uint32_t)c->slot;
  // Trace, interpolation of column A (times 31^i / N) and its coset LDE.
  // Column B is derived from A wherever it is needed (linked_lde,
  // src/air.rs:806-844): B(x) = A(omega_N x) + C_j / (x - w_last).
  CK(push_consts(c, K));
  // The per-coset constants come from extra CTAs of the trace launch.
  const ZinvArgs za{zinv, zinv2, logB, to_mont(fpow(GENERATOR, N)), cb, slot};
  CK(launch::fib_trace(st, cols, cols + N * K, (uint32_t)N, slot, mats, K, &za, &c->tb));
  NttPlan ip;
  ip.logn = logN; ip.batch = K; ip.inverse = 1; ip.post_gamma = 1;
  CK(launch::ntt(st, c->tb, ip, cols, coeffs, (uint32_t*)c->scratch.p));
  NttPlan lp;
  lp.logn = logN; lp.batch = (uint32_t)(B * K); lp.in_div = (uint32_t)B; lp.twist_mod = (uint32_t)B;
  lp.twist_shift = 27 - logm;
  CK(launch::ntt(st, c->tb, lp, coeffs, lde, (uint32_t*)c->scratch.p));
  const uint32_t* lde_a = lde;
  const uint32_t w_last_m = to_mont(w_last);

  // Joint trace tree over 8-row 64-byte leaves (src/air.rs:520-537).
  uint32_t* tinv = (uint32_t*)c->scratch.p;  // the NTT's scratch is free from here on
  uint32_t built = 0;  // subtree levels the leaf kernel hashed itself
  const uint64_t tcap_stride = h.trace_cap_bytes / 4;
  arm_cap(c, h.trace_cap, (size_t)h.trace_cap_bytes * K);
  CK(launch::air_trace_leaves(st, c->tb, lde_a, cb, w_last_m, ttree, tinv, logN, logB, tsteps,
                              hio_dev<uint32_t>(c, h.trace_cap), merkle_counter(c), &built, K,
                              ttree_words, tcap_stride));
  if (built < tsteps || (tsteps == 0 && tleaves > kFuseMaxLeaves))
    CK(launch::merkle_build(st, ttree, tleaves, tsteps, merkle_counter(c),
                            hio_dev<uint32_t>(c, h.trace_cap), built, K, ttree_words, tcap_stride));
  CK(wait_cap(c, "cap", h.trace_cap, (size_t)h.trace_cap_bytes * K));
  std::vector<std::vector<uint8_t>> column_cap(K);
  const uint32_t omega_inv = finv(omega_n);
  for (uint32_t k = 0; k < K; k++) {
    const uint8_t* cap = c->hio + h.trace_cap + k * h.trace_cap_bytes;
    column_cap[k].assign(cap, cap + h.trace_cap_bytes);
    c->d2h += h.trace_cap_bytes;
    transcript_absorb(*tasks[k].ts, "fib/trace", cap, h.trace_cap_bytes);
    uint32_t alpha[5][4];
    for (int i = 0; i < 5; i++) challenge_ext(*tasks[k].ts, "fib/alpha", alpha[i]);
    if (tasks[k].fixed_alpha)
      for (int i = 0; i < 5; i++)
        for (int e = 0; e < 4; e++) alpha[i][e] = tasks[k].fixed_alpha[4 * i + e];
    ProofConsts& pc = c->consts[k];
    const uint32_t neg_coeff = fsub(0, coeff[k]);
    for (int e = 0; e < 4; e++) {
      pc.alpha[e][0] = 0;
      pc.alpha[e][1] = to_mont(alpha[1][e]);
      pc.alpha[e][2] = to_mont(fmul(alpha[2][e], omega_inv));
      pc.alpha[e][3] = to_mont(fmul(alpha[3][e], omega_inv));
      pc.alpha[e][4] = to_mont(alpha[4][e]);
      pc.kc[e] = fmul(alpha[0][e], neg_coeff);
    }
  }

  // Composition as bit-reversed FRI layer 0 with its leaves (src/air.rs:847-929).
  AirComposeArgs ca;
  ca.lde_a = lde_a; ca.cb = cb; ca.zinv = zinv; ca.tinv = tinv;
  ca.layer0 = fb.layer[0]; ca.leaves = fb.tree[0];
  ca.logN = logN; ca.logB = logB;
  ca.w_last_m = w_last_m;
  ca.slot = slot;
  ca.layer_stride = fb.val_stride;
  ca.tree_stride = fb.tree_stride;
  CK(push_consts(c, K));
  if (K == 1) {  // one proof: its statement and weights as kernel parameters
    const ProofConsts& p0 = c->consts[0];
    ca.a0 = p0.a0; ca.b0 = p0.b0; ca.b_last = p0.b_last;
    std::memcpy(ca.kc, p0.kc, sizeof ca.kc);
    std::memcpy(ca.alpha, p0.alpha, sizeof ca.alpha);
  }
  ca.counter = merkle_counter(c);  // small layer-0 trees are finished inside the launch
  ca.top = s.depth[0] - s.drop[0];
  ca.cap = hio_dev<uint32_t>(c, h.fri_cap[0]);
  ca.cap_stride = h.fri_cap_bytes[0] / 4;
  uint32_t built0 = 0;
  arm_cap(c, h.fri_cap[0], (size_t)h.fri_cap_bytes[0] * K);
  CK(launch::air_compose_leaves(st, c->tb, ca, K, &built0));
  if (built0 == 0)
    CK(launch::merkle_build(st, fb.tree[0], s.leaves[0], s.depth[0] - s.drop[0], merkle_counter(c),
                            hio_dev<uint32_t>(c, h.fri_cap[0]), 0, K, fb.tree_stride,
                            h.fri_cap_bytes[0] / 4));
  if (tasks[0].layer0_out) {  // composition stage: layer 0 out, nothing further
    CK(cudaMemcpyAsync(tasks[0].layer0_out, fb.layer[0], 16 * m, cudaMemcpyDeviceToDevice, st));
    CK(sync(c));
    return Z0P_OK;
  }

  std::vector<Transcript*> ts(K);
  for (uint32_t k = 0; k < K; k++) ts[k] = tasks[k].ts;
  std::vector<FriOut> fo(K);
  // Openings: FRI queries plus the two trace leaves per query (src/air.rs:565-591).
  OpenArgs oa{};
  oa.lde = lde_a; oa.cb = cb; oa.tinv = tinv;
  oa.ttree = ttree; oa.tleaves = tleaves; oa.tsteps = tsteps;
  oa.logN = logN; oa.logB = logB; oa.ncol = 0;
  oa.lde_stride = m;
  oa.ttree_stride = ttree_words;
  RC(run_fri_openings(c, s, fp, fb, m, N - 1, ts.data(), K, h, fo.data(), oa, {}, true, true));
  // The proof bytes are written as the opening blocks land.
  struct OpenGuard {
    z0p_gpu_ctx* c;
    ~OpenGuard() { c->open_epoch = 0; }
  } open_guard{c};

  for (uint32_t k = 0; k < K; k++) {
    Writer w(tasks[k].out, need);  // air::Proof::to_bytes (src/air.rs:262-281)
    w.byte(6);
    w.u32((uint32_t)(column_cap[k].size() / 32));
    w.bytes(column_cap[k].data(), column_cap[k].size());
    write_fri(w, c, s, fo[k], m, N - 1, h, k);
    w.u32((uint32_t)fo[k].indices.size());
    for (size_t qi = 0; qi < fo[k].indices.size(); qi++) {
      uint64_t index = brev(fo[k].indices[qi], logm);
      uint64_t shifted = (index + B) % m;
      const uint32_t* rows = open_block(c, h, k, qi) + h.trace_off;  // A0 B0 .. A7 B7, path
      const uint32_t* srows = rows + 16 + 8 * tsteps;
      w.u64(index);
      w.u32(rows[2 * (index & 7)]);
      w.u32(rows[2 * (index & 7) + 1]);
      w.u32(srows[2 * (shifted & 7)]);
      w.u32(srows[2 * (shifted & 7) + 1]);
      write_path(w, (const uint8_t*)(rows + 16), index / 8, tsteps);
      write_path(w, (const uint8_t*)(srows + 16), shifted / 8, tsteps);
      w.bytes(rows, 64);
      w.bytes(srows, 64);
    }
    if (w.n != need) {
      set_reason("internal error: proof length differs from its shape");
      return Z0P_ERR_CUDA;
    }
  }
  CK(finish_openings(c));
  return Z0P_OK;
}

bool range_const_ok(const z0p_range_params& p, const FriShape& s) {
  return const_fri_ok(s, p.value < (1u << p.n_bits), p.n_rows, p.blowup);
}

int range_prove_const(z0p_gpu_ctx* c, const RangeTask* tasks, uint32_t K, const FriParams& fp,
                      const FriShape& s, uint64_t need) {
  const z0p_range_params& p0 = *tasks[0].p;
  const uint64_t N = p0.n_rows, B = p0.blowup, m = N * B, ncol = p0.n_bits + 1;
  const uint32_t logB = log2u(B), logm = log2u(m);
  const uint32_t tdrop = p0.cap_height < logm ? (uint32_t)p0.cap_height : logm;
  const uint32_t tsteps = logm - tdrop;
  std::vector<std::vector<uint32_t>> rows(K);
  for (uint32_t k = 0; k < K; k++) {
    const z0p_range_params& p = *tasks[k].p;
    rows[k].assign(ncol, 0u);
    rows[k][0] = p.value;  // build_columns (src/range.rs:316-330)
    for (uint64_t j = 0; j < p.n_bits; j++) rows[k][1 + j] = (p.value >> j) & 1u;
    uint8_t pb[56];  // absorb_params (src/range.rs:634-645)
    auto p64 = [&](int off, uint64_t x) { for (int i = 0; i < 8; i++) pb[off + i] = (uint8_t)(x >> (8 * i)); };
    auto p32 = [&](int off, uint32_t x) { for (int i = 0; i < 4; i++) pb[off + i] = (uint8_t)(x >> (8 * i)); };
    p64(0, p.n_rows); p64(8, p.n_bits); p64(16, p.blowup); p64(24, p.num_queries);
    p64(32, p.final_size); p32(40, p.grinding_bits); p64(44, p.cap_height); p32(52, p.value);
    transcript_absorb(*tasks[k].ts, "range/params", pb, 56);
  }
  // In-range values only: every FRI layer is zero, and its trees go with
  // the trace trees' launch.
  std::vector<ConstFri> fr(K);
  bool all_zero = true;
  for (uint32_t k = 0; k < K; k++) {
    fr[k].logB = logB;
    all_zero &= tasks[k].p->value < (1u << p0.n_bits);
  }
  std::vector<ConstTree*> early;
  if (all_zero) prepare_const_fri(s, K, fr.data(), &early);
  std::vector<ConstTree> ttrees;
  std::vector<std::vector<uint8_t>> tcap;
  RC(const_trace_trees(c, rows, logm, tdrop, &ttrees, &tcap, early));
  // Composition (src/range.rs:678-774) on coset j: (value - rec) zinv_j alpha_d.
  const uint32_t gN = fpow(GENERATOR, N), wB = two_adic_generator(logB);
  std::vector<std::vector<uint32_t>> kc(K);
  std::vector<Transcript*> ts(K);
  for (uint32_t k = 0; k < K; k++) {
    ts[k] = tasks[k].ts;
    transcript_absorb(*ts[k], "range/column", tcap[k].data(), tcap[k].size());
    uint32_t alpha_d[4];
    for (uint64_t i = 0; i < ncol + 1; i++) {  // decomposition, n_bits booleans, boundary
      uint32_t a[4];
      challenge_ext(*ts[k], "range/alpha", a);
      if (i == 0) std::memcpy(alpha_d, a, 16);
    }
    const uint32_t value = tasks[k].p->value, rec = value & ((1u << p0.n_bits) - 1u);
    if (value != rec) {
      kc[k].assign(4 * B, 0u);
      uint32_t xn = gN;  // x^N on coset j: 31^N omega_B^j
      for (uint64_t j = 0; j < B; j++) {
        const uint32_t base = fmul(fsub(value, rec), finv(fsub(xn, 1)));
        for (int e = 0; e < 4; e++) kc[k][4 * j + e] = fmul(base, alpha_d[e]);
        xn = fmul(xn, wB);
      }
      fr[k].kc = kc[k].data();
    }
  }
  RC(const_fri(c, s, fp, m, N - 1, ts.data(), K, fr.data(), all_zero));
  std::vector<uint8_t> pbuf;
  for (uint32_t k = 0; k < K; k++) {
    const z0p_range_params& p = *tasks[k].p;
    Writer w(tasks[k].out, need);  // range::Proof::to_bytes (src/range.rs:253-269)
    w.byte(6);
    w.u32((uint32_t)(tcap[k].size() / 32));
    w.bytes(tcap[k].data(), tcap[k].size());
    write_const_fri(w, s, fr[k], m, N - 1);
    w.u32((uint32_t)fr[k].fo.indices.size());
    const CompactTree tt = ttrees[k].view();
    for (size_t qi = 0; qi < fr[k].fo.indices.size(); qi++) {
      const uint64_t index = brev(fr[k].fo.indices[qi], logm);
      w.u64(index);
      w.u32(rows[k][0]);
      w.u32((uint32_t)p.n_bits);
      for (uint64_t b = 0; b < p.n_bits; b++) w.u32(rows[k][1 + b]);
      write_path(w, tt.path(index, tsteps, pbuf), index, tsteps);
    }
    if (w.n != need) {
      set_reason("internal error: proof length differs from its shape");
      return Z0P_ERR_CUDA;
    }
  }
  return Z0P_OK;
}

// src/range.rs:353-375 -> 425-514 on the device for any columns, for K
// proofs of one shape in lockstep: the columns of range::prove (host_cols
// null: value and its bits, filled on the device) or, for K = 1, the
// caller's n_bits + 1 columns of n_rows words, value column first.
// With n_rand (K = 1), every column is masked as range::prove_zk does
// (src/range.rs:393-418) with rand[c * n_rand + k] and the LDE runs over the
// padded rows.
int range_prove_columns(z0p_gpu_ctx* c, const RangeTask* tasks, uint32_t K, const FriParams& fp,
                        const FriShape& s, uint64_t need, const uint32_t* const* host_cols,
                        uint64_t n_rand = 0, const uint32_t* rand = nullptr) {
  const z0p_range_params& p0 = *tasks[0].p;
  const uint64_t N = p0.n_rows, B = p0.blowup, ncol = p0.n_bits + 1;
  uint64_t Lp = N;  // rows per coset of the LDE: padded to 2^ceil(log2(n + n_rand)) when masked
  while (n_rand && Lp < N + n_rand) Lp <<= 1;
  const uint64_t m = Lp * B, r = Lp / N;
  const uint32_t logN = log2u(N), logL = log2u(Lp), logB = log2u(B), logm = logL + logB;
  const uint64_t bound = n_rand ? N + 2 * n_rand - 2 : N - 1;  // src/range.rs:417
  cudaStream_t st = c->stream;
  RC(ensure_slots(c, K));
  RC(ensure(c, c->cols, 4 * N * ncol * K));
  RC(ensure(c, c->coeffs, 4 * (N * ncol * K + (n_rand ? Lp * ncol : 0))));
  RC(ensure(c, c->scratch, 4 * m * ncol * K));
  RC(ensure(c, c->lde, 4 * m * ncol * K));
  const uint64_t ttree_words = 8 * tree_digests(m);
  RC(ensure(c, c->ttree, 4 * ttree_words * K));
  RC(ensure(c, c->misc, 4 * (16 + 2 * B * r + ncol * n_rand)));
  FriBufs fb;
  RC(plan_fri_buffers(c, s, K, &fb));
  uint32_t* cols = (uint32_t*)c->cols.p;
  uint32_t* coeffs = (uint32_t*)c->coeffs.p;
  uint32_t* lde = (uint32_t*)c->lde.p;
  uint32_t* ttree = (uint32_t*)c->ttree.p;
  uint32_t* zinv = (uint32_t*)c->misc.p + 16;
  uint32_t* zinv2 = zinv + B * r;
  uint32_t* rdev = zinv2 + B * r;
  const uint32_t tdepth = logm;
  const uint32_t tdrop = p0.cap_height < tdepth ? (uint32_t)p0.cap_height : tdepth;
  const uint32_t tsteps = tdepth - tdrop;
  // Per-proof inputs read in place: the column values (ncol words, all proofs
  // first) then the alphas (ncol + 1 Ext4 per proof).
  HioPlan h;
  RC(plan_hio(c, s, p0.num_queries, tdrop, (uint32_t)ncol + 8 * tsteps, K, &h,
              4 * ncol + 16 * (ncol + 1) + 16));
  uint32_t* hvals = reinterpret_cast<uint32_t*>(c->hio + h.extra);
  uint32_t* halpha = hvals + ncol * K;
  const size_t bad_at = h.extra + (4 * ncol + 16 * (ncol + 1)) * K;  // caller's columns: a non-canonical value
  const uint32_t* dvals = hio_dev<uint32_t>(c, h.extra);
  const uint32_t* dalpha = dvals + ncol * K;
  c->h2d += (4 * ncol + 16 * (ncol + 1)) * K;

  const uint32_t slot = (uint32_t)c->slot;
  for (uint32_t k = 0; k < K; k++) {
    const z0p_range_params& p = *tasks[k].p;
    // build_columns (src/range.rs:316-330): V = value, C_j = bit j of value.
    uint32_t* v = hvals + ncol * k;
    v[0] = p.value;
    for (uint64_t j = 0; j < p.n_bits; j++) v[1 + j] = j < 32 ? (p.value >> j) & 1 : 0;
    uint8_t pb[56];  // absorb_params (src/range.rs:634-645)
    auto p64 = [&](int off, uint64_t x) { for (int i = 0; i < 8; i++) pb[off + i] = (uint8_t)(x >> (8 * i)); };
    auto p32 = [&](int off, uint32_t x) { for (int i = 0; i < 4; i++) pb[off + i] = (uint8_t)(x >> (8 * i)); };
    p64(0, p.n_rows); p64(8, p.n_bits); p64(16, p.blowup); p64(24, p.num_queries);
    p64(32, p.final_size); p32(40, p.grinding_bits); p64(44, p.cap_height); p32(52, p.value);
    transcript_absorb(*tasks[k].ts, "range/params", pb, 56);
    c->consts[k].value = p.value;
  }
  CK(push_consts(c, K));
  if (host_cols) {
    for (uint64_t j = 0; j < ncol; j++)
      CK(cudaMemcpyAsync(cols + j * N, host_cols[j], 4 * N, cudaMemcpyHostToDevice, st));
    c->h2d += 4 * N * ncol;
    *reinterpret_cast<unsigned int*>(c->hio + bad_at) = 0u;  // checked by the interpolation
  } else {
    CK(launch::fill_constant_columns(st, cols, (uint32_t)N, (uint32_t)ncol, dvals, K));
  }
  NttPlan ip;
  ip.logn = logN; ip.batch = (uint32_t)(ncol * K); ip.inverse = 1; ip.post_gamma = 1;
  if (host_cols) ip.bad = hio_dev<unsigned int>(c, bad_at);
  CK(launch::ntt(st, c->tb, ip, cols, coeffs, (uint32_t*)c->scratch.p));
  const uint32_t* lde_in = coeffs;
  if (n_rand) {  // T + (x^n - 1) R per column, zero-padded (src/blind.rs:40-78)
    CK(cudaMemcpyAsync(rdev, rand, 4 * ncol * n_rand, cudaMemcpyHostToDevice, st));
    c->h2d += 4 * ncol * n_rand;
    CK(launch::mask_pad(st, c->tb, coeffs, rdev, coeffs + N * ncol, (uint32_t)N, (uint32_t)n_rand,
                        (uint32_t)Lp, (uint32_t)ncol));
    lde_in = coeffs + N * ncol;
  }
  NttPlan lp;
  lp.logn = logL; lp.batch = (uint32_t)(ncol * B * K); lp.in_div = (uint32_t)B;
  lp.twist_mod = (uint32_t)B;
  lp.twist_shift = 27 - logm;
  CK(launch::ntt(st, c->tb, lp, lde_in, lde, (uint32_t*)c->scratch.p));
  const uint64_t tcap_stride = h.trace_cap_bytes / 4;
  uint32_t tbuilt = 0;  // small trees finished in the launch
  CK(launch::range_trace_leaves(st, lde, ttree, logL, logB, (uint32_t)ncol, K, ttree_words,
                                merkle_counter(c), tsteps, hio_dev<uint32_t>(c, h.trace_cap),
                                tcap_stride, &tbuilt));
  if (tbuilt == 0)
    CK(launch::merkle_build(st, ttree, m, tsteps, merkle_counter(c),
                            hio_dev<uint32_t>(c, h.trace_cap), 0, K, ttree_words, tcap_stride));
  if (r == 1) {
    CK(launch::coset_zinv(st, c->tb, zinv, zinv2, logB, to_mont(fpow(GENERATOR, N)), nullptr, slot));
  } else {  // 1/(x^n - 1) for coset j and q mod r, x = 31 omega_m^j omega_Lp^q
    std::vector<uint32_t> zt(2 * B * r);
    const uint32_t omega_m = two_adic_generator(logm), omega_l = two_adic_generator(logL);
    for (uint64_t j = 0; j < B; j++)
      for (uint64_t q = 0; q < r; q++) {
        const uint32_t x = fmul(fmul(GENERATOR, fpow(omega_m, j)), fpow(omega_l, q));
        const uint32_t zm = to_mont(finv(fsub(fpow(x, N), 1)));
        zt[j * r + q] = zm;
        zt[B * r + j * r + q] = to_mont(zm);  // times 2^64
      }
    CK(cudaMemcpyAsync(zinv, zt.data(), 8 * B * r, cudaMemcpyHostToDevice, st));
    c->h2d += 8 * B * r;
  }
  CK(sync(c, "cap"));
  if (host_cols && *reinterpret_cast<volatile unsigned int*>(c->hio + bad_at)) {
    set_reason("field elements must be canonical (< p)");
    return Z0P_ERR_MALFORMED_INPUT;
  }
  std::vector<std::vector<uint8_t>> column_cap(K);
  for (uint32_t k = 0; k < K; k++) {
    const uint8_t* cap = c->hio + h.trace_cap + k * h.trace_cap_bytes;
    column_cap[k].assign(cap, cap + h.trace_cap_bytes);
    c->d2h += h.trace_cap_bytes;
    transcript_absorb(*tasks[k].ts, "range/column", cap, h.trace_cap_bytes);
    for (uint64_t i = 0; i < ncol + 1; i++) {  // decomposition, n_bits booleans, boundary
      uint32_t a[4];
      challenge_ext(*tasks[k].ts, "range/alpha", a);
      for (int e = 0; e < 4; e++) halpha[4 * (ncol + 1) * k + 4 * i + e] = to_mont(a[e]);
    }
  }

  RangeComposeArgs ca;
  ca.lde = lde; ca.zinv = zinv; ca.zinv2 = zinv2;
  ca.alphas = dalpha;
  ca.layer0 = fb.layer[0]; ca.leaves = fb.tree[0];
  ca.logN = logL; ca.logB = logB; ca.n_bits = (uint32_t)p0.n_bits; ca.slot = slot;
  ca.r = (uint32_t)r;
  ca.layer_stride = fb.val_stride;
  ca.tree_stride = fb.tree_stride;
  CK(launch::range_compose_leaves(st, c->tb, ca, K));
  CK(launch::merkle_build(st, fb.tree[0], s.leaves[0], s.depth[0] - s.drop[0], merkle_counter(c),
                          hio_dev<uint32_t>(c, h.fri_cap[0]), 0, K, fb.tree_stride,
                          h.fri_cap_bytes[0] / 4));

  std::vector<Transcript*> ts(K);
  for (uint32_t k = 0; k < K; k++) ts[k] = tasks[k].ts;
  std::vector<FriOut> fo(K);
  OpenArgs oa{};  // src/range.rs:483-500
  oa.lde = lde; oa.ttree = ttree; oa.tleaves = m; oa.tsteps = tsteps;
  oa.logN = logL; oa.logB = logB; oa.ncol = (uint32_t)ncol;
  oa.lde_stride = m * ncol;
  oa.ttree_stride = ttree_words;
  RC(run_fri_openings(c, s, fp, fb, m, bound, ts.data(), K, h, fo.data(), oa));

  for (uint32_t k = 0; k < K; k++) {
    const z0p_range_params& p = *tasks[k].p;
    Writer w(tasks[k].out, need);  // range::Proof::to_bytes (src/range.rs:253-269)
    w.byte(6);
    w.u32((uint32_t)(column_cap[k].size() / 32));
    w.bytes(column_cap[k].data(), column_cap[k].size());
    write_fri(w, c, s, fo[k], m, bound, h, k);
    w.u32((uint32_t)fo[k].indices.size());
    for (size_t qi = 0; qi < fo[k].indices.size(); qi++) {
      uint64_t index = brev(fo[k].indices[qi], logm);
      const uint32_t* row = open_block(c, h, k, qi) + h.trace_off;
      w.u64(index);
      w.u32(row[0]);
      w.u32((uint32_t)p.n_bits);
      for (uint64_t b = 0; b < p.n_bits; b++) w.u32(row[1 + b]);
      write_path(w, (const uint8_t*)(row + ncol), index, tsteps);
    }
    if (w.n != need) {
      set_reason("internal error: proof length differs from its shape");
      return Z0P_ERR_CUDA;
    }
  }
  return Z0P_OK;
}

// src/range.rs:337-343 (range::prove) for K proofs of one shape in lockstep:
// the constant-trace path whenever its conditions hold, else the columns path.
int range_prove(z0p_gpu_ctx* c, const RangeTask* tasks, uint32_t K) {
  FriParams fp;
  FriShape s;
  uint64_t need = 0;
  RC(check_group(tasks, K, range_shape, range_size, same_range_shape, &fp, &s, &need));
  bool constant_ok = true;
  for (uint32_t k = 0; k < K && constant_ok; k++) constant_ok = range_const_ok(*tasks[k].p, s);
  if (constant_ok) return range_prove_const(c, tasks, K, fp, s, need);
  return range_prove_columns(c, tasks, K, fp, s, need, nullptr);
}

int with_device(z0p_gpu_ctx* c) {
  CK(cudaSetDevice(c->device));
  return Z0P_OK;
}


// ====================================================== FRI as a PCS ====
// fri::commit* and fri::open (src/fri.rs:400-666) on the device. Between the
// two calls the committed layers and trees (ProverState, src/fri.rs:276-295)
// stay in the context's workspace; fri.serial pins them to the workspace
// state they were made in.
struct FriInput {
  FriParams fp{};
  FriShape s;
  bool ext = false, evals = false;
  uint64_t n = 0, m = 0, poly_len = 0, bound = 0;
  uint64_t commitment_bytes = 0, proof_bytes = 0;
};

// The entry checks of src/fri.rs:407-549 in the reference's order, then
// commit_inner's (fri_shape), and the byte lengths of both outputs.
int fri_input(const z0p_fri_params* p, int form, size_t n, uint64_t degree_bound, FriInput* in) {
  if (!p || form < Z0P_FRI_COEFFS || form > Z0P_FRI_EVALS_EXT) return Z0P_ERR_INVALID_ARGUMENT;
  in->fp = FriParams{p->blowup, p->num_queries, p->final_size, p->grinding_bits, p->cap_height};
  RC(fri_params_validate(in->fp));
  in->ext = form == Z0P_FRI_COEFFS_EXT || form == Z0P_FRI_EVALS_EXT;
  in->evals = form >= Z0P_FRI_EVALS;
  if (n == 0) return Z0P_ERR_EMPTY_INPUT;
  if (!is_pow2(n)) return Z0P_ERR_INVALID_DOMAIN_SIZE;
  const uint64_t max_domain = 1ull << 27;  // Field::TWO_ADICITY
  in->n = n;
  if (!in->evals) {  // src/ntt.rs:341-352
    if (n > max_domain / in->fp.blowup) return Z0P_ERR_INVALID_DOMAIN_SIZE;
    in->m = n * in->fp.blowup;
    in->bound = n - 1;
  } else {
    if (n > max_domain) return Z0P_ERR_INVALID_DOMAIN_SIZE;
    if (degree_bound >= n) {
      set_reason("degree bound must be below LDE size (rate < 1)");
      return Z0P_ERR_MALFORMED_INPUT;
    }
    in->m = n;
    in->bound = degree_bound;
  }
  in->poly_len = n;
  RC(fri_shape(in->m, in->bound, in->fp, &in->s));
  const FriShape& s = in->s;
  uint64_t cb = 1 + 24 + 4;  // Commitment::to_bytes
  for (size_t i = 0; i < s.len.size(); i++) cb += 4 + 32ull * (1ull << s.drop[i]);
  uint64_t per_query = 4;  // Proof::to_bytes
  for (size_t d = 0; d + 1 < s.len.size(); d++) per_query += 64 + 4 + 33ull * (s.depth[d] - s.drop[d]);
  in->commitment_bytes = cb;
  in->proof_bytes = 1 + 4 + 16 * s.len.back() + 8 + 4 + in->fp.num_queries * per_query;
  return Z0P_OK;
}

}  // namespace

namespace z0p {
struct FriPending {
  bool valid = false;
  uint64_t serial = 0;
  FriInput in;
  FriBufs fb;
  HioPlan h;
  FriOut out;
};
}  // namespace z0p

namespace {

int fri_commit(z0p_gpu_ctx* c, const FriInput& in, const uint32_t* values,
               z0p_transcript_state* t, uint8_t* out) {
  const FriShape& s = in.s;
  const uint32_t ncomp = in.ext ? 4 : 1;
  const uint32_t logm = log2u(in.m), logn = log2u(in.n), logB = log2u(in.fp.blowup);
  cudaStream_t st = c->stream;
  const uint64_t in_words = in.n * ncomp;
  RC(ensure(c, c->cols, 4 * in_words));
  if (!in.evals) {
    RC(ensure(c, c->coeffs, 4ull * ncomp * in.n));
    RC(ensure(c, c->lde, 4ull * ncomp * in.m));
    RC(ensure(c, c->scratch, 4ull * ncomp * in.m));
  }
  if (!c->fri) c->fri = new FriPending();
  FriPending& f = *c->fri;
  f.valid = false;
  f.in = in;
  RC(plan_fri_buffers(c, s, 1, &f.fb));
  RC(plan_hio(c, s, in.fp.num_queries, 0, 0, 1, &f.h, 16));
  unsigned int* bad_h = reinterpret_cast<unsigned int*>(c->hio + f.h.extra);
  unsigned int* bad = hio_dev<unsigned int>(c, f.h.extra);
  *bad_h = 0;
  uint32_t* src = (uint32_t*)c->cols.p;
  CK(cudaMemcpyAsync(src, values, 4 * in_words, cudaMemcpyHostToDevice, st));
  c->h2d += 4 * in_words;
  if (!in.evals) {
    uint32_t* coeffs = (uint32_t*)c->coeffs.p;
    uint32_t* lde = (uint32_t*)c->lde.p;
    NttPlan lp;
    lp.logn = logn;
    lp.batch = ncomp << logB;
    lp.in_div = 1u << logB;
    lp.twist_mod = 1u << logB;
    lp.twist_shift = 27 - logm;
    if (in.ext) {  // de-interleave the Ext4 coordinates, scaled by 31^i
      CK(launch::gamma_scale(st, c->tb, src, coeffs, (uint32_t)in.n, 1u, bad));
      CK(launch::ntt(st, c->tb, lp, coeffs, lde, (uint32_t*)c->scratch.p));
    } else {  // base coefficients: the transform scales and checks them as it loads
      lp.pre_gamma = 1;
      lp.bad = bad;
      CK(launch::ntt(st, c->tb, lp, src, lde, (uint32_t*)c->scratch.p));
    }
  }
  // Small layer-0 trees are finished inside the leaf launch.
  const uint32_t top0 = s.depth[0] - s.drop[0];
  uint32_t* cap0 = hio_dev<uint32_t>(c, f.h.fri_cap[0]);
  uint32_t built0 = 0;
  arm_cap(c, f.h.fri_cap[0], f.h.fri_cap_bytes[0]);  // the bad flag is read after the last wait
  const bool from_lde = !in.evals;  // coefficients were extended (coset-major LDE)
  CK(launch::layer0_leaves(st, from_lde ? (const uint32_t*)c->lde.p : src, f.fb.layer[0],
                           f.fb.tree[0], bad, logm, from_lde ? logB : 0, ncomp, from_lde,
                           merkle_counter(c), top0, cap0, &built0));
  if (built0 == 0)
    CK(launch::merkle_build(st, f.fb.tree[0], s.leaves[0], top0, merkle_counter(c), cap0, 0, 1,
                            f.fb.tree_stride, f.h.fri_cap_bytes[0] / 4));
  z0p_transcript_state work = *t;
  Transcript tr(&work);
  Transcript* ts[1] = {&tr};
  RC(run_fri_commit(c, s, in.fp, f.fb, in.poly_len, in.bound, ts, 1, f.h, &f.out, nullptr, true));
  if (*reinterpret_cast<volatile unsigned int*>(bad_h)) {  // read after the stream drained
    set_reason("field elements must be canonical (< p)");
    return Z0P_ERR_MALFORMED_INPUT;
  }
  Writer w(out, in.commitment_bytes);
  w.byte(6);  // VERSION (src/codec.rs:21)
  write_fri_commitment(w, s, f.out, in.poly_len, in.bound);
  *t = work;
  f.valid = true;
  f.serial = c->work_serial;
  return Z0P_OK;
}

int fri_open(z0p_gpu_ctx* c, z0p_transcript_state* t, uint8_t* out, uint64_t* indices) {
  FriPending& f = *c->fri;
  const FriShape& s = f.in.s;
  z0p_transcript_state work = *t;
  Transcript tr(&work);
  Transcript* ts[1] = {&tr};
  RC(run_fri_open(c, s, f.in.fp, ts, 1, f.h, &f.out));
  OpenArgs oa{};
  oa.no_trace = 1;
  RC(run_openings(c, s, f.fb, f.h, &f.out, 1, oa));
  Writer w(out, f.in.proof_bytes);
  w.byte(6);  // VERSION (src/codec.rs:21)
  write_fri_proof(w, c, s, f.out, f.h, 0);
  if (indices)
    for (size_t i = 0; i < f.out.indices.size(); i++) indices[i] = f.out.indices[i];
  *t = work;
  f.valid = false;
  return Z0P_OK;
}

// ====================================================== folded IVC ====
// fold::Accumulator (src/fold.rs:362-561) on the device: each segment's two
// column LDEs and row tree stay resident; finalize combines every segment's
// composition into FRI layer 0 in one pass, commits it with the FRI engine
// and gathers the step openings.
// Ext4 product on the host (src/ext4.rs:106-117): with x = x0 + x1 v over
// Fp2 = Fp[u]/(u^2 - 11) and v^2 = u, xy = (x0 y0 + u x1 y1) + (x0 y1 + x1 y0) v.
void e4_mul_host(const uint32_t x[4], const uint32_t y[4], uint32_t out[4]) {
  auto fp2 = [](uint32_t a0, uint32_t a1, uint32_t b0, uint32_t b1, uint32_t o[2]) {
    o[0] = fadd(fmul(a0, b0), fmul(11, fmul(a1, b1)));
    o[1] = fadd(fmul(a0, b1), fmul(a1, b0));
  };
  uint32_t p00[2], p11[2], p01[2], p10[2];
  fp2(x[0], x[1], y[0], y[1], p00);
  fp2(x[2], x[3], y[2], y[3], p11);
  fp2(x[0], x[1], y[2], y[3], p01);
  fp2(x[2], x[3], y[0], y[1], p10);
  out[0] = fadd(p00[0], fmul(11, p11[1]));  // u (a + b u) = 11 b + a u
  out[1] = fadd(p00[1], p11[0]);
  out[2] = fadd(p01[0], p10[0]);
  out[3] = fadd(p01[1], p10[1]);
}

int fold_validate(const z0p_fold_params& p) {  // src/fold.rs:186-222
  if (p.seg_steps < 2 || !is_pow2(p.seg_steps)) return Z0P_ERR_INVALID_DOMAIN_SIZE;
  if (p.blowup < 4 || !is_pow2(p.blowup)) return Z0P_ERR_INVALID_BLOWUP;
  if (p.num_queries == 0) return Z0P_ERR_NO_QUERIES;
  if (p.final_size < 2 || !is_pow2(p.final_size)) return Z0P_ERR_INVALID_DOMAIN_SIZE;
  if (p.cap_height > 8) { set_reason("cap_height above 8"); return Z0P_ERR_MALFORMED_INPUT; }
  if (p.seg_steps > (1ull << 27) / p.blowup) return Z0P_ERR_INVALID_DOMAIN_SIZE;
  if (p.in_a >= P || p.in_b >= P || p.out_b >= P) {
    set_reason("field elements must be canonical (< p)");
    return Z0P_ERR_MALFORMED_INPUT;
  }
  return Z0P_OK;
}

int fold_fri(const z0p_fold_params& p, FriParams* fp, FriShape* s) {  // src/fold.rs:177-184
  RC(fri_params_new(p.blowup, p.num_queries, p.final_size, fp));
  fp->grinding_bits = p.grinding_bits;
  fp->cap_height = p.cap_height;
  const uint64_t m = p.seg_steps * p.blowup;
  if (p.seg_steps - 1 >= m) return Z0P_ERR_MALFORMED_INPUT;  // fri::commit_ext_evals
  return fri_shape(m, p.seg_steps - 1, *fp, s);
}

struct FoldStepHost {
  uint32_t claims[4];  // in_a, in_b, out_a, out_b
  uint32_t alpha[6][4];
  std::vector<uint8_t> cap;
  // In one of the accumulator's slabs: [A planes | B planes] coset-major,
  // then the level-contiguous row tree.
  uint32_t* lde = nullptr;
  uint32_t* tree = nullptr;
};

}  // namespace

struct z0p_gpu_fold {
  z0p_gpu_ctx* ctx = nullptr;
  z0p_fold_params p{};
  std::vector<FoldStepHost> steps;
  DevBuf tinv, table;  // row inverses; FoldStepDev table + per-coset 1/(x^s - 1)
  // Segments' LDEs and trees, several segments to an allocation: slabs of 4,
  // 8, 16, ... segments, each at most 16 MB (one segment where that is
  // less), so a short chain makes one allocation, not two per segment.
  std::vector<DevBuf> slabs;
  size_t slab_cap = 0, slab_used = 0;
  bool finalized = false;
};

namespace {

uint64_t fold_proof_bytes(const z0p_fold_params& p, size_t nsteps, const FriShape& s) {
  const uint64_t m = p.seg_steps * p.blowup;
  const uint32_t depth = log2u(m), drop = p.cap_height < depth ? (uint32_t)p.cap_height : depth;
  const uint64_t path = 4 + 33ull * (depth - drop);
  const uint64_t per_step = 16 + 4 + 32ull * (1ull << drop) + 4 + p.num_queries * (8 + 16 + 2 * path);
  return 1 + 4 + nsteps * per_step + fri_bytes(s, p.num_queries);
}

void fold_absorb_params(const z0p_fold_params& p, Transcript& t) {  // src/fold.rs:729-741
  uint8_t b[56];
  auto u64 = [&](int at, uint64_t v) { for (int i = 0; i < 8; i++) b[at + i] = (uint8_t)(v >> (8 * i)); };
  auto u32 = [&](int at, uint32_t v) { for (int i = 0; i < 4; i++) b[at + i] = (uint8_t)(v >> (8 * i)); };
  u64(0, p.seg_steps); u64(8, p.blowup); u64(16, p.num_queries); u64(24, p.final_size);
  u32(32, p.grinding_bits); u64(36, p.cap_height); u32(44, p.in_a); u32(48, p.in_b); u32(52, p.out_b);
  transcript_absorb(t, "fold/params", b, 56);
}

int fold_add(z0p_gpu_fold* f, const uint32_t* col_a, const uint32_t* col_b,
             z0p_transcript_state* ts) {
  z0p_gpu_ctx* c = f->ctx;
  const z0p_fold_params& p = f->p;
  const uint64_t S = p.seg_steps, B = p.blowup, m = S * B;
  const uint32_t logN = log2u(S), logB = log2u(B), logm = logN + logB;
  cudaStream_t st = c->stream;
  RC(ensure(c, c->cols, 8 * S));
  RC(ensure(c, c->coeffs, 8 * S));
  RC(ensure(c, c->scratch, 8 * m));
  FoldStepHost step;
  const size_t lde_bytes = (8 * m + 255) & ~(size_t)255;
  const size_t seg_bytes = lde_bytes + ((32 * tree_digests(m) + 255) & ~(size_t)255);
  if (f->slab_used == f->slab_cap) {
    size_t n = f->steps.empty() ? 4 : 2 * f->steps.size();
    const size_t fit = ((size_t)16 << 20) / seg_bytes;
    if (n > fit) n = fit > 0 ? fit : 1;
    DevBuf slab;
    RC(ensure(c, slab, n * seg_bytes));
    f->slabs.push_back(slab);
    f->slab_cap = n;
    f->slab_used = 0;
  }
  char* seg = static_cast<char*>(f->slabs.back().p) + f->slab_used * seg_bytes;
  step.lde = reinterpret_cast<uint32_t*>(seg);
  step.tree = reinterpret_cast<uint32_t*>(seg + lde_bytes);
  const uint32_t depth = logm, drop = p.cap_height < depth ? (uint32_t)p.cap_height : depth;
  const size_t cap_bytes = 32ull << drop;
  // Segments of up to 2^12 rows are interpolated by the one-CTA transform,
  // which reads the two columns straight from the mapped buffer: no copy
  // operation is queued for them. Larger ones are copied to the device.
  const bool mapped_cols = logN <= 12;
  const size_t cols_at = 64 + cap_bytes;
  RC(ensure_hio(c, cols_at + (mapped_cols ? 8 * S : 0)));
  unsigned int* bad_h = reinterpret_cast<unsigned int*>(c->hio);
  *bad_h = 0;
  uint32_t* cols = (uint32_t*)c->cols.p;
  if (mapped_cols) {
    std::memcpy(c->hio + cols_at, col_a, 4 * S);
    std::memcpy(c->hio + cols_at + 4 * S, col_b, 4 * S);
    cols = hio_dev<uint32_t>(c, cols_at);
  } else {
    CK(cudaMemcpyAsync(cols, col_a, 4 * S, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(cols + S, col_b, 4 * S, cudaMemcpyHostToDevice, st));
  }
  c->h2d += 8 * S;
  uint32_t* lde = step.lde;
  uint32_t* tree = step.tree;
  const bool one_launch = mapped_cols && launch::fold_segment_ok(logN, logB);
  if (one_launch) {
    // Small segments: interpolation, LDE, row leaves and tree in one launch,
    // which publishes a bad column word before any word of the cap: the cap
    // is read as soon as it lands (arm_cap, wait_cap).
    arm_cap(c, 64, cap_bytes);
    CK(launch::fold_segment(st, c->tb, cols, hio_dev<unsigned int>(c, 0), lde, tree,
                            hio_dev<uint32_t>(c, 64), logN, logB, depth - drop));
  } else {
    NttPlan ip;  // interpolate (src/ntt.rs:316-321), outputs times 31^i / S
    ip.logn = logN; ip.batch = 2; ip.inverse = 1; ip.post_gamma = 1;
    ip.bad = hio_dev<unsigned int>(c, 0);  // the columns are checked as they load
    CK(launch::ntt(st, c->tb, ip, cols, (uint32_t*)c->coeffs.p, (uint32_t*)c->scratch.p));
    NttPlan lp;  // evaluate_on_coset (src/ntt.rs:341-363), coset-major per column
    lp.logn = logN; lp.batch = (uint32_t)(2 * B); lp.in_div = (uint32_t)B; lp.twist_mod = (uint32_t)B;
    lp.twist_shift = 27 - logm;
    CK(launch::ntt(st, c->tb, lp, (uint32_t*)c->coeffs.p, lde, (uint32_t*)c->scratch.p));
    // Row tree over A || B (src/fold.rs:448-458: MerkleTree::from_flat, 8-byte rows).
    uint32_t built = 0;  // small segment trees finished in the launch
    CK(launch::range_trace_leaves(st, lde, tree, logN, logB, 2, 1, 0, merkle_counter(c), depth - drop,
                                  hio_dev<uint32_t>(c, 64), 0, &built));
    if (built == 0)
      CK(launch::merkle_build(st, tree, m, depth - drop, merkle_counter(c), hio_dev<uint32_t>(c, 64)));
  }
  CK(one_launch ? wait_cap(c, "cap", 64, cap_bytes) : sync(c, "cap"));
  if (*reinterpret_cast<volatile unsigned int*>(bad_h)) {
    set_reason("field elements must be canonical (< p)");
    return Z0P_ERR_MALFORMED_INPUT;
  }
  step.claims[0] = col_a[0]; step.claims[1] = col_b[0];
  step.claims[2] = col_a[S - 1]; step.claims[3] = col_b[S - 1];
  step.cap.assign(c->hio + 64, c->hio + 64 + cap_bytes);
  c->d2h += cap_bytes;
  z0p_transcript_state work = *ts;
  Transcript t(&work);
  if (f->steps.empty()) fold_absorb_params(p, t);
  uint8_t cl[16];
  for (int i = 0; i < 16; i++) cl[i] = (uint8_t)(step.claims[i / 4] >> (8 * (i % 4)));
  transcript_absorb(t, "fold/step", cl, 16);
  transcript_absorb(t, "fold/trace", step.cap.data(), cap_bytes);
  for (int k = 0; k < 6; k++) challenge_ext(t, "fold/alpha", step.alpha[k]);
  *ts = work;
  f->steps.push_back(std::move(step));
  f->slab_used++;  // the segment's slot stays taken only once it is added
  return Z0P_OK;
}

int fold_finalize(z0p_gpu_fold* f, z0p_transcript_state* ts, uint8_t* out) {
  z0p_gpu_ctx* c = f->ctx;
  const z0p_fold_params& p = f->p;
  const uint64_t S = p.seg_steps, B = p.blowup, m = S * B;
  const uint32_t logN = log2u(S), logB = log2u(B), logm = logN + logB;
  const uint32_t K = (uint32_t)f->steps.size();
  cudaStream_t st = c->stream;
  FriParams fp;
  FriShape s;
  RC(fold_fri(p, &fp, &s));
  const uint32_t depth = logm, drop = p.cap_height < depth ? (uint32_t)p.cap_height : depth;
  const uint32_t psteps = depth - drop;
  z0p_transcript_state work = *ts;
  Transcript t(&work);
  // Combination challenges (src/fold.rs:500-504), folded with each step's alphas.
  const uint32_t omega_s = two_adic_generator(logN);
  const uint32_t omega_inv = finv(omega_s);
  const uint32_t w_last = fpow(omega_s, S - 1);
  std::vector<FoldStepDev> table(K);
  for (uint32_t k = 0; k < K; k++) {
    uint32_t g[4];
    challenge_ext(t, "fold/gamma", g);
    FoldStepHost& h = f->steps[k];
    FoldStepDev& d = table[k];
    d.a = h.lde;
    d.b = d.a + m;
    d.tree = h.tree;
    d.in_a = h.claims[0]; d.in_b = h.claims[1]; d.out_a = h.claims[2]; d.out_b = h.claims[3];
    for (int j = 0; j < 6; j++) {
      uint32_t ga[4];
      e4_mul_host(g, h.alpha[j], ga);
      for (int e = 0; e < 4; e++)
        d.ga[j][e] = to_mont(j == 2 || j == 3 ? fmul(ga[e], omega_inv) : ga[e]);
    }
  }
  // Per-coset 1/(x^S - 1), x^S = 31^S omega_m^(j S) = 31^S omega_B^j
  // (src/fold.rs:818-825), inverted together: one inversion and three
  // products per coset (Montgomery's batch inversion).
  std::vector<uint32_t> zinv(B), pre(B);
  {
    const uint32_t omega_b = two_adic_generator(logB);
    uint32_t x = fpow(GENERATOR, S), run = 1;
    for (uint64_t j = 0; j < B; j++) {
      zinv[j] = fsub(x, 1);  // nonzero: 31^S is outside the subgroup of order B
      pre[j] = run;
      run = fmul(run, zinv[j]);
      x = fmul(x, omega_b);
    }
    uint32_t inv = finv(run);
    for (uint64_t j = B; j-- > 0;) {
      const uint32_t d = zinv[j];
      zinv[j] = to_mont(fmul(inv, pre[j]));
      inv = fmul(inv, d);
    }
  }
  const size_t tbytes = (size_t)K * sizeof(FoldStepDev), zoff = (tbytes + 15) & ~(size_t)15;
  FriBufs fb;
  RC(plan_fri_buffers(c, s, 1, &fb));
  const uint32_t stride = (4 + 16 * psteps + 3) & ~3u;
  // The mapped buffer's extra region: the segments' opening blocks, then the
  // step table and the coset inverses (read there in place by a small
  // combination, else staged for one pinned, asynchronous copy).
  const size_t open_bytes = 4ull * stride * fp.num_queries * K;
  HioPlan h;
  RC(plan_hio(c, s, fp.num_queries, 0, 0, 1, &h, open_bytes + zoff + 4 * B));
  uint8_t* staged = c->hio + h.extra + open_bytes;
  std::memcpy(staged, table.data(), tbytes);
  std::memcpy(staged + zoff, zinv.data(), 4 * B);
  c->h2d += tbytes + 4 * B;
  // Small layers 0: the combination launch inverts its rows' denominators
  // itself and builds the layer-0 tree, and its few CTAs read the table in
  // place (staged once per CTA), so no copy is queued before it. Larger ones
  // read a table of inverses and a device copy of the step table.
  const bool fused_combine = (m / 4) <= kFuseMaxLeaves;  // fold_combine's own test
  const FoldStepDev* steps_dev = hio_dev<const FoldStepDev>(c, h.extra + open_bytes);
  if (!fused_combine) {
    RC(ensure(c, f->table, zoff + 4 * B));
    CK(cudaMemcpyAsync(f->table.p, staged, zoff + 4 * B, cudaMemcpyHostToDevice, st));
    steps_dev = (const FoldStepDev*)f->table.p;
    RC(ensure(c, f->tinv, 4 * m));
    CK(launch::row_inverses(st, c->tb, (uint32_t*)f->tinv.p, to_mont(w_last), logN, logB));
  }
  FoldCombineArgs ca;
  ca.steps = steps_dev;
  ca.nsteps = K;
  ca.tinv = fused_combine ? nullptr : (const uint32_t*)f->tinv.p;
  ca.zinv = (const uint32_t*)((const char*)steps_dev + zoff);
  ca.layer0 = fb.layer[0];
  ca.leaves = fb.tree[0];
  ca.logN = logN; ca.logB = logB;
  ca.w_last_m = to_mont(w_last);
  if (fused_combine) {
    ca.counter = merkle_counter(c);
    ca.top = s.depth[0] - s.drop[0];
    ca.cap = hio_dev<uint32_t>(c, h.fri_cap[0]);
  }
  uint32_t built0 = 0;
  arm_cap(c, h.fri_cap[0], h.fri_cap_bytes[0]);
  CK(launch::fold_combine(st, c->tb, ca, &built0));
  if (built0 == 0)
    CK(launch::merkle_build(st, fb.tree[0], s.leaves[0], s.depth[0] - s.drop[0], merkle_counter(c),
                            hio_dev<uint32_t>(c, h.fri_cap[0]), 0, 1, fb.tree_stride,
                            h.fri_cap_bytes[0] / 4));
  // fri::commit_ext_evals(combined, S - 1) and fri::open (src/fold.rs:517-520).
  Transcript* tp[1] = {&t};
  FriOut fo;
  OpenArgs oa{};
  oa.no_trace = 1;
  // The step openings read the same indices after the gather (stream order):
  // both gathers end at one synchronisation.
  RC(run_fri_openings(c, s, fp, fb, m, S - 1, tp, 1, h, &fo, oa, [&]() {
    return launch::fold_openings(st, ca.steps, K, hio_dev<uint64_t>(c, h.indices),
                                 (uint32_t)fp.num_queries, logN, logB, psteps,
                                 hio_dev<uint32_t>(c, h.extra), stride);
  }, true));
  // IvcProof::to_bytes (src/fold.rs:281-309).
  Writer w(out, fold_proof_bytes(p, K, s));
  w.byte(6);
  w.u32(K);
  const uint32_t* blocks = reinterpret_cast<const uint32_t*>(c->hio + h.extra);
  for (uint32_t k = 0; k < K; k++) {
    const FoldStepHost& sh = f->steps[k];
    for (int i = 0; i < 4; i++) w.u32(sh.claims[i]);
    w.u32((uint32_t)(sh.cap.size() / 32));
    w.bytes(sh.cap.data(), sh.cap.size());
    w.u32((uint32_t)fp.num_queries);
    for (uint64_t qi = 0; qi < fp.num_queries; qi++) {
      const uint32_t* blk = blocks + ((size_t)k * fp.num_queries + qi) * stride;
      const uint64_t index = brev(fo.indices[qi], logm);
      const uint64_t shifted = (index + B) % m;
      w.u64(index);
      for (int i = 0; i < 4; i++) w.u32(blk[i]);
      write_path(w, (const uint8_t*)(blk + 4), index, psteps);
      write_path(w, (const uint8_t*)(blk + 4 + 8 * psteps), shifted, psteps);
    }
  }
  c->d2h += 4ull * stride * fp.num_queries * K;
  write_fri_commitment(w, s, fo, m, S - 1);
  write_fri_proof(w, c, s, fo, h, 0);
  *ts = work;
  f->finalized = true;
  return Z0P_OK;
}
}  // namespace

struct ProfileScope {
  bool on;
  explicit ProfileScope(z0p_gpu_ctx* c) : on(c->profiling) {
    if (on) launch::set_recorder(&c->rec);
  }
  ~ProfileScope() {
    if (on) launch::set_recorder(nullptr);
  }
};

// Proves n statements of one shape in groups of at most kMaxGroup, each on
// working copies of the transcripts; the copies are written back only when
// every proof succeeded, so a failing call leaves every transcript untouched.
template <class Params, class Fn>
int prove_group_abi(z0p_gpu_ctx* c, size_t n, const Params* params,
                    z0p_transcript_state* const* transcripts, uint8_t* const* outs,
                    const size_t* caps, size_t* lens, Fn prove) {
  if (!c || !n || !params || !transcripts || !outs || !caps) return Z0P_ERR_INVALID_ARGUMENT;
  for (size_t i = 0; i < n; i++)
    if (!transcripts[i]) return Z0P_ERR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> lk(c->mu);
  c->work_serial++;
  RC(with_device(c));
  ProfileScope ps(c);
  const uint64_t t0 = now_ns();
  std::vector<z0p_transcript_state> work(n);
  for (size_t i = 0; i < n; i++) work[i] = *transcripts[i];
  // Group size: up to kMaxGroup proofs, but no more than the context's
  // constant slots. When the process-wide slots are short (many contexts),
  // the group is proved in smaller consecutive groups instead of failing.
  size_t G = n < (size_t)kMaxGroup ? n : (size_t)kMaxGroup;
  if (ensure_slots(c, (uint32_t)G) != Z0P_OK) {
    if (c->nslots < 1) return Z0P_ERR_OUT_OF_MEMORY;  // reason already set
    G = (size_t)c->nslots;
  }
  int rc = Z0P_OK;
  for (size_t at = 0; at < n && rc == Z0P_OK; at += G) {
    const uint32_t K = (uint32_t)(n - at < G ? n - at : G);
    std::vector<Transcript> tr;
    tr.reserve(K);
    std::vector<Task<Params>> tasks(K);
    for (uint32_t k = 0; k < K; k++) {
      tr.emplace_back(&work[at + k]);
      tasks[k] = Task<Params>{&params[at + k], &tr[k], outs[at + k], caps[at + k],
                              lens ? &lens[at + k] : nullptr};
    }
    c->last_sync_ns = now_ns();
    rc = prove(c, tasks.data(), K);
    if (c->profiling && c->last_sync_ns) c->tail_ns += now_ns() - c->last_sync_ns;
    c->last_sync_ns = 0;
  }
  c->prove_ns += now_ns() - t0;
  if (rc != Z0P_OK) return rc;
  for (size_t i = 0; i < n; i++) *transcripts[i] = work[i];
  c->proofs += n;
  return Z0P_OK;
}

// ================================================================ C ABI ====
extern "C" {

int z0p_gpu_abi_version(void) { return Z0P_GPU_ABI_VERSION; }
const char* z0p_gpu_last_reason(void) { return z0p::host::reason(); }

int z0p_transcript_init(z0p_transcript_state* st, const uint8_t* label, size_t len) {
  if (!st || (!label && len)) return Z0P_ERR_INVALID_ARGUMENT;
  transcript_init(st, label, len);
  return Z0P_OK;
}
int z0p_transcript_absorb(z0p_transcript_state* st, const uint8_t* label, size_t llen,
                          const uint8_t* data, size_t dlen) {
  if (!st || (!label && llen) || (!data && dlen)) return Z0P_ERR_INVALID_ARGUMENT;
  Transcript(st).absorb_raw(label, llen, data, dlen);
  return Z0P_OK;
}
int z0p_transcript_challenge_bytes(z0p_transcript_state* st, const uint8_t* label, size_t llen,
                                   uint8_t out[32]) {
  if (!st || !out || (!label && llen)) return Z0P_ERR_INVALID_ARGUMENT;
  Transcript(st).squeeze(label, llen, out);
  return Z0P_OK;
}
int z0p_transcript_challenge_ext(z0p_transcript_state* st, const uint8_t* label, size_t llen,
                                 uint32_t out[4]) {
  if (!st || !out || (!label && llen)) return Z0P_ERR_INVALID_ARGUMENT;
  uint8_t b[32];
  Transcript(st).squeeze(label, llen, b);
  for (int i = 0; i < 4; i++)
    out[i] = ((uint32_t)b[4 * i] | ((uint32_t)b[4 * i + 1] << 8) | ((uint32_t)b[4 * i + 2] << 16) |
              ((uint32_t)b[4 * i + 3] << 24)) % P;
  return Z0P_OK;
}
int z0p_transcript_challenge_index(z0p_transcript_state* st, const uint8_t* label, size_t llen,
                                   uint64_t domain, uint64_t* out) {
  if (!st || !out || (!label && llen)) return Z0P_ERR_INVALID_ARGUMENT;
  if (!is_pow2(domain)) {
    set_reason("challenge_index domain must be a nonzero power of two");
    return Z0P_ERR_MALFORMED_INPUT;
  }
  uint8_t b[32];
  Transcript(st).squeeze(label, llen, b);
  uint64_t v = 0;
  for (int i = 0; i < 8; i++) v |= (uint64_t)b[i] << (8 * i);
  *out = v & (domain - 1);
  return Z0P_OK;
}

int z0p_air_params_new(uint64_t n, uint64_t blowup, uint64_t q, uint64_t final_size, uint32_t a0,
                       uint32_t b0, uint32_t b_last, z0p_air_params* o) {
  if (!o) return Z0P_ERR_INVALID_ARGUMENT;  // src/air.rs:62-102
  if (n < 2 || !is_pow2(n)) return Z0P_ERR_INVALID_DOMAIN_SIZE;
  if (blowup < 4 || !is_pow2(blowup)) return Z0P_ERR_INVALID_BLOWUP;
  if (q == 0) return Z0P_ERR_NO_QUERIES;
  if (final_size < 2 || !is_pow2(final_size)) return Z0P_ERR_INVALID_DOMAIN_SIZE;
  if (n > UINT64_MAX / blowup || n * blowup > MAX_DOMAIN) return Z0P_ERR_INVALID_DOMAIN_SIZE;
  *o = z0p_air_params{n, blowup, q, final_size, 0, 0, a0 % P, b0 % P, b_last % P};
  return Z0P_OK;
}
int z0p_air_params_for_security(uint64_t n, uint32_t a0, uint32_t b0, uint32_t b_last,
                                uint32_t target, z0p_air_params* o) {
  if (!o) return Z0P_ERR_INVALID_ARGUMENT;  // src/air.rs:127-158
  if (n < 2 || !is_pow2(n)) return Z0P_ERR_INVALID_DOMAIN_SIZE;
  if (n > UINT64_MAX / 16 || n * 16 > MAX_DOMAIN) return Z0P_ERR_INVALID_DOMAIN_SIZE;
  uint64_t lde = n * 16, q, fs, ch;
  uint32_t g;
  tune_strength(target, composition_millibits(lde, n - 1), &q, &g);
  tune_shape(lde, q, lde, 24, &fs, &ch);
  *o = z0p_air_params{n, 16, q, fs, g, ch, a0 % P, b0 % P, b_last % P};
  return Z0P_OK;
}
int z0p_range_params_new(uint64_t n_rows, uint64_t n_bits, uint64_t blowup, uint64_t q,
                         uint64_t final_size, uint32_t value, z0p_range_params* o) {
  if (!o) return Z0P_ERR_INVALID_ARGUMENT;  // src/range.rs:57-99
  if (n_rows < 2 || !is_pow2(n_rows)) return Z0P_ERR_INVALID_DOMAIN_SIZE;
  if (n_bits == 0 || n_bits > 24) { set_reason("n_bits must be within 1..=24"); return Z0P_ERR_MALFORMED_INPUT; }
  if (blowup < 2 || !is_pow2(blowup)) return Z0P_ERR_INVALID_BLOWUP;
  if (q == 0) return Z0P_ERR_NO_QUERIES;
  if (final_size < 2 || !is_pow2(final_size)) return Z0P_ERR_INVALID_DOMAIN_SIZE;
  if (n_rows > UINT64_MAX / blowup || n_rows * blowup > MAX_DOMAIN) return Z0P_ERR_INVALID_DOMAIN_SIZE;
  *o = z0p_range_params{n_rows, n_bits, blowup, q, final_size, 0, 0, value % P};
  return Z0P_OK;
}
int z0p_range_params_for_security(uint64_t n_rows, uint64_t n_bits, uint32_t value,
                                  uint32_t target, z0p_range_params* o) {
  if (!o) return Z0P_ERR_INVALID_ARGUMENT;  // src/range.rs:124-161
  if (n_rows < 2 || !is_pow2(n_rows)) return Z0P_ERR_INVALID_DOMAIN_SIZE;
  if (n_bits == 0 || n_bits > 24) { set_reason("n_bits must be within 1..=24"); return Z0P_ERR_MALFORMED_INPUT; }
  if (n_rows > UINT64_MAX / 16 || n_rows * 16 > MAX_DOMAIN) return Z0P_ERR_INVALID_DOMAIN_SIZE;
  uint64_t lde = n_rows * 16, q, fs, ch;
  uint32_t g;
  tune_strength(target, composition_millibits(lde, n_rows - 1), &q, &g);
  tune_shape(lde, q, lde, 8 + 4 * (n_bits + 1), &fs, &ch);
  *o = z0p_range_params{n_rows, n_bits, 16, q, fs, g, ch, value % P};
  return Z0P_OK;
}

int z0p_air_proof_size(const z0p_air_params* p, size_t* len) {
  if (!p || !len) return Z0P_ERR_INVALID_ARGUMENT;
  FriParams fp;
  FriShape s;
  RC(air_shape(*p, &fp, &s));
  *len = air_size(*p, s);
  return Z0P_OK;
}
int z0p_range_proof_size(const z0p_range_params* p, size_t* len) {
  if (!p || !len) return Z0P_ERR_INVALID_ARGUMENT;
  FriParams fp;
  FriShape s;
  RC(range_shape(*p, &fp, &s));
  *len = range_size(*p, s);
  return Z0P_OK;
}

int z0p_gpu_air_footprint(const z0p_air_params* p, size_t* bytes) {
  if (!p || !bytes) return Z0P_ERR_INVALID_ARGUMENT;
  FriParams fp;
  FriShape s;
  RC(air_shape(*p, &fp, &s));
  uint64_t N = p->n_steps, m = s.m, total = 16 * N + 8 * m + 32 * tree_digests(m / 8);
  for (size_t i = 0; i < s.len.size(); i++) total += 16 * s.len[i] + 32 * tree_digests(s.leaves[i]);
  *bytes = total;
  return Z0P_OK;
}
int z0p_gpu_range_footprint(const z0p_range_params* p, size_t* bytes) {
  if (!p || !bytes) return Z0P_ERR_INVALID_ARGUMENT;
  FriParams fp;
  FriShape s;
  RC(range_shape(*p, &fp, &s));
  uint64_t ncol = p->n_bits + 1, N = p->n_rows, m = s.m;
  if (range_const_ok(*p, s)) {
    // The constant-trace path keeps its compact trees in the mapped buffer
    // and no device arrays: its device footprint is the PoW search state.
    *bytes = 1ull << 16;
    return Z0P_OK;
  }
  uint64_t total = 8 * N * ncol + 8 * m * ncol + 32 * tree_digests(m);
  for (size_t i = 0; i < s.len.size(); i++) total += 16 * s.len[i] + 32 * tree_digests(s.leaves[i]);
  *bytes = total;
  return Z0P_OK;
}

int z0p_gpu_ctx_create(int device, z0p_gpu_ctx** out) {
  if (!out) return Z0P_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  int count = 0;
  CK(cudaGetDeviceCount(&count));
  if (device < 0 || device >= count) {
    set_reason("no such CUDA device");
    return Z0P_ERR_INVALID_ARGUMENT;
  }
  z0p_gpu_ctx* c = new z0p_gpu_ctx();
  c->device = device;
  cudaError_t e = cudaSetDevice(device);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    set_reason(std::string("context creation: ") + cudaGetErrorString(e));
    delete c;
    return Z0P_ERR_CUDA;
  }
  int rc = build_tables(c);
  if (rc == Z0P_OK) {
    unsigned int* fault_d = nullptr;
    if (cudaHostAlloc((void**)&c->fault, 64, cudaHostAllocMapped) != cudaSuccess ||
        cudaHostGetDevicePointer((void**)&fault_d, c->fault, 0) != cudaSuccess) {
      set_reason("context creation: status word setup failed");
      rc = Z0P_ERR_CUDA;
    } else {
      *c->fault = 0u;
      c->tb.fault = fault_d;
    }
  }
  if (rc == Z0P_OK) {
    c->slot = take_slots(1);
    c->nslots = c->slot < 0 ? 0 : 1;
    if (c->slot < 0) {
      set_reason("context creation: every constant slot is taken (too many contexts)");
      rc = Z0P_ERR_OUT_OF_MEMORY;
    } else if (launch::const_slot_address(c->slot, &c->slot_dev) != cudaSuccess ||
               cudaHostAlloc((void**)&c->consts, kMaxGroup * sizeof(ProofConsts),
                             cudaHostAllocDefault) != cudaSuccess) {
      set_reason("context creation: constant slot setup failed");
      rc = Z0P_ERR_CUDA;
    } else {
      std::memset(c->consts, 0, kMaxGroup * sizeof(ProofConsts));
    }
  }
  const size_t state_bytes = 4 * kMaxGroup + 32 * kMaxGroup;
  if (rc == Z0P_OK) rc = ensure(c, c->state, state_bytes);
  if (rc == Z0P_OK) {
    // Merkle counters 0; PoW states {best = ~0, next chunk 0, status 0, done 0}.
    std::vector<uint64_t> init(state_bytes / 8, 0);
    for (int k = 0; k < kMaxGroup; k++) init[kMaxGroup / 2 + 4 * k] = ~0ull;
    if (cudaMemcpyAsync(c->state.p, init.data(), state_bytes, cudaMemcpyHostToDevice, c->stream) !=
            cudaSuccess ||
        cudaStreamSynchronize(c->stream) != cudaSuccess) {
      set_reason("context creation: state upload failed");
      rc = Z0P_ERR_CUDA;
    }
  }
  if (rc) {
    z0p_gpu_ctx_destroy(c);
    return rc;
  }
  *out = c;
  return Z0P_OK;
}

void z0p_gpu_ctx_destroy(z0p_gpu_ctx* c) {
  if (!c) return;
  cudaSetDevice(c->device);
  if (c->stream) cudaStreamSynchronize(c->stream);
  for (DevBuf* b : {&c->tables, &c->cols, &c->coeffs, &c->scratch, &c->lde, &c->ttree, &c->layers,
                    &c->ftrees, &c->misc, &c->state})
    release(c, *b);
  if (c->stream) cudaStreamSynchronize(c->stream);
  if (c->hio) cudaFreeHost(c->hio);
  if (c->fault) cudaFreeHost(c->fault);
  if (c->consts) cudaFreeHost(c->consts);
  for (cudaEvent_t e : c->gate_ev) cudaEventDestroy(e);
  give_slots(c->slot, c->nslots);
  if (c->stream) cudaStreamDestroy(c->stream);
  delete c->fri;
  delete c;
}

int z0p_gpu_ctx_set_gates(z0p_gpu_ctx* c, int on) {
  if (!c) return Z0P_ERR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> lk(c->mu);
  c->gates = on != 0;
  return Z0P_OK;
}

int z0p_gpu_ctx_trim(z0p_gpu_ctx* c) {
  if (!c) return Z0P_ERR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> lk(c->mu);
  c->work_serial++;
  RC(with_device(c));
  for (DevBuf* b : {&c->cols, &c->coeffs, &c->scratch, &c->lde, &c->ttree, &c->layers, &c->ftrees,
                    &c->misc})
    release(c, *b);
  return Z0P_OK;
}

int z0p_fri_params_for_security(uint64_t poly_len, uint32_t target_bits, z0p_fri_params* out) {
  if (!out) return Z0P_ERR_INVALID_ARGUMENT;  // src/fri.rs:232-255
  if (poly_len == 0) return Z0P_ERR_EMPTY_INPUT;
  if (!is_pow2(poly_len)) return Z0P_ERR_INVALID_DOMAIN_SIZE;
  const uint64_t blowup = 16;
  if (poly_len > (1ull << 27) / blowup) return Z0P_ERR_INVALID_DOMAIN_SIZE;
  uint64_t q = 0, fs = 0, ch = 0;
  uint32_t g = 0;
  tune_strength(target_bits, 2000, &q, &g);
  tune_shape(poly_len * blowup, q, 0, 0, &fs, &ch);
  *out = z0p_fri_params{blowup, q, fs, g, ch};
  return Z0P_OK;
}

int z0p_fri_sizes(const z0p_fri_params* p, int form, size_t n, uint64_t degree_bound,
                  size_t* commitment_len, size_t* proof_len) {
  FriInput in;
  RC(fri_input(p, form, n, degree_bound, &in));
  if (commitment_len) *commitment_len = in.commitment_bytes;
  if (proof_len) *proof_len = in.proof_bytes;
  return Z0P_OK;
}

int z0p_gpu_fri_commit(z0p_gpu_ctx* c, const z0p_fri_params* p, int form, const uint32_t* values,
                       size_t n, uint64_t degree_bound, z0p_transcript_state* t, uint8_t* out,
                       size_t cap, size_t* len) {
  if (!c || !t || (!values && n)) return Z0P_ERR_INVALID_ARGUMENT;
  FriInput in;
  RC(fri_input(p, form, n, degree_bound, &in));
  if (len) *len = in.commitment_bytes;
  if (!out || cap < in.commitment_bytes) {
    set_reason("output buffer too small for the commitment");
    return Z0P_ERR_BUFFER_TOO_SMALL;
  }
  std::lock_guard<std::mutex> lk(c->mu);
  c->work_serial++;
  RC(with_device(c));
  ProfileScope ps(c);
  return fri_commit(c, in, values, t, out);
}

int z0p_gpu_fri_open(z0p_gpu_ctx* c, z0p_transcript_state* t, uint8_t* out, size_t cap,
                     size_t* len, uint64_t* indices) {
  if (!c || !t) return Z0P_ERR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> lk(c->mu);
  if (!c->fri || !c->fri->valid || c->fri->serial != c->work_serial) {
    set_reason("no FRI commitment to open on this context");
    return Z0P_ERR_INVALID_ARGUMENT;
  }
  if (len) *len = c->fri->in.proof_bytes;
  if (!out || cap < c->fri->in.proof_bytes) {
    set_reason("output buffer too small for the proof");
    return Z0P_ERR_BUFFER_TOO_SMALL;
  }
  RC(with_device(c));
  ProfileScope ps(c);
  return fri_open(c, t, out, indices);
}

int z0p_gpu_air_prove_with_trace(z0p_gpu_ctx* c, const z0p_air_params* p, const uint32_t* col_a,
                                 const uint32_t* col_b, size_t len, z0p_transcript_state* t,
                                 uint8_t* out, size_t cap, size_t* out_len) {
  if (!c || !p || !t || !col_a || !col_b) return Z0P_ERR_INVALID_ARGUMENT;
  FriParams fp;
  FriShape s;
  RC(general_shape(*p, 0, &fp, &s));
  if (len != p->n_steps) {  // src/air.rs:389-394
    set_reason("trace columns must match n_steps");
    return Z0P_ERR_MALFORMED_INPUT;
  }
  const uint64_t need = air_size(*p, s);
  if (out_len) *out_len = need;
  if (!out || cap < need) {
    set_reason("output buffer too small for the proof");
    return Z0P_ERR_BUFFER_TOO_SMALL;
  }
  std::lock_guard<std::mutex> lk(c->mu);
  c->work_serial++;
  RC(with_device(c));
  ProfileScope ps(c);
  GeneralAir g;
  g.host_a = col_a;
  g.host_b = col_b;
  return air_prove_general(c, *p, g, t, out);
}

int z0p_air_proof_size_zk(const z0p_air_params* p, size_t n_rand, size_t* len) {
  if (!p || !len) return Z0P_ERR_INVALID_ARGUMENT;
  FriParams fp;
  FriShape s;
  RC(general_shape(*p, n_rand, &fp, &s));
  *len = air_size(*p, s);
  return Z0P_OK;
}

int z0p_gpu_air_prove_zk(z0p_gpu_ctx* c, const z0p_air_params* p, size_t n_rand,
                         z0p_chacha20_state* rng, z0p_transcript_state* t, uint8_t* out,
                         size_t cap, size_t* out_len) {
  if (!c || !p || !t || !rng || rng->used > 64) return Z0P_ERR_INVALID_ARGUMENT;
  RC(air_validate(*p));  // src/air.rs:445-458: the hiding budget first
  if (p->num_queries > SIZE_MAX / 16) {
    set_reason("query budget overflows the hiding requirement");
    return Z0P_ERR_MALFORMED_INPUT;
  }
  if (n_rand < 16 * p->num_queries) {
    set_reason("n_rand must cover every revealed leaf row for hiding");
    return Z0P_ERR_MALFORMED_INPUT;
  }
  FriParams fp;
  FriShape s;
  RC(general_shape(*p, n_rand, &fp, &s));
  const uint64_t need = air_size(*p, s);
  if (out_len) *out_len = need;
  if (!out || cap < need) {
    set_reason("output buffer too small for the proof");
    return Z0P_ERR_BUFFER_TOO_SMALL;
  }
  // Masking values: n_rand for column A, then n_rand for column B
  // (src/air.rs:461-462, src/blind.rs:65), on a copy of the stream.
  z0p_chacha20_state r = *rng;
  std::vector<uint32_t> rand(2 * n_rand);
  for (auto& v : rand) v = chacha20_next_field(&r);
  std::lock_guard<std::mutex> lk(c->mu);
  c->work_serial++;
  RC(with_device(c));
  ProfileScope ps(c);
  GeneralAir g;
  g.n_rand = n_rand;
  g.rand = rand.data();
  RC(air_prove_general(c, *p, g, t, out));
  *rng = r;
  return Z0P_OK;
}

int z0p_table_params_new(uint64_t n_rows, uint64_t blowup, uint64_t num_queries,
                         uint64_t final_size, uint32_t value, z0p_table_params* out) {
  if (!out) return Z0P_ERR_INVALID_ARGUMENT;  // src/table.rs:55-88
  if (n_rows < 2 || !is_pow2(n_rows)) return Z0P_ERR_INVALID_DOMAIN_SIZE;
  if (blowup < 2 || !is_pow2(blowup)) return Z0P_ERR_INVALID_BLOWUP;
  if (num_queries == 0) return Z0P_ERR_NO_QUERIES;
  if (final_size < 2 || !is_pow2(final_size)) return Z0P_ERR_INVALID_DOMAIN_SIZE;
  if (n_rows > (1ull << 27) / blowup) return Z0P_ERR_INVALID_DOMAIN_SIZE;
  if (value >= P) { set_reason("field elements must be canonical (< p)"); return Z0P_ERR_MALFORMED_INPUT; }
  *out = z0p_table_params{n_rows, blowup, num_queries, final_size, 0, 0, value};
  return Z0P_OK;
}

int z0p_table_params_for_security(uint64_t n_rows, uint64_t table_len, uint32_t value,
                                  uint32_t target_bits, z0p_table_params* out) {
  if (!out) return Z0P_ERR_INVALID_ARGUMENT;  // src/table.rs:114-170
  if (n_rows < 2 || !is_pow2(n_rows)) return Z0P_ERR_INVALID_DOMAIN_SIZE;
  if (table_len < 2) { set_reason("table needs at least two entries"); return Z0P_ERR_MALFORMED_INPUT; }
  if (n_rows - 1 > UINT64_MAX / table_len || table_len * (n_rows - 1) < n_rows) {
    set_reason("table length overflows composition bound");
    return Z0P_ERR_MALFORMED_INPUT;
  }
  if (value >= P) { set_reason("field elements must be canonical (< p)"); return Z0P_ERR_MALFORMED_INPUT; }
  const uint64_t bound = table_len * (n_rows - 1) - n_rows, need = bound + 1;
  uint64_t blowup = 4, lde = 0;
  for (;;) {
    if (n_rows > UINT64_MAX / blowup) return Z0P_ERR_INVALID_DOMAIN_SIZE;
    lde = n_rows * blowup;
    if (need <= lde / 4 || blowup >= (1ull << 27)) break;
    blowup *= 2;
  }
  if (lde > (1ull << 27) || need > lde / 4) return Z0P_ERR_INVALID_DOMAIN_SIZE;
  uint64_t q = 0, fs = 0, ch = 0;
  uint32_t g = 0;
  tune_strength(target_bits, composition_millibits(lde, bound), &q, &g);
  tune_shape(lde, q, lde, 12, &fs, &ch);
  *out = z0p_table_params{n_rows, blowup, q, fs, g, ch, value};
  return Z0P_OK;
}

int z0p_table_proof_size(const z0p_table_params* p, size_t table_len, size_t n_rand, size_t* len) {
  if (!p || !len) return Z0P_ERR_INVALID_ARGUMENT;
  FriParams fp;
  FriShape s;
  uint64_t bytes = 0;
  RC(table_shape(*p, nullptr, table_len, n_rand, &fp, &s, &bytes));
  *len = bytes;
  return Z0P_OK;
}

int z0p_gpu_table_prove(z0p_gpu_ctx* c, const z0p_table_params* p, const uint32_t* table,
                        size_t table_len, z0p_transcript_state* t, uint8_t* out, size_t cap,
                        size_t* out_len) {
  if (!c || !p || !t || (!table && table_len)) return Z0P_ERR_INVALID_ARGUMENT;
  FriParams fp;
  FriShape s;
  uint64_t need = 0;
  RC(table_shape(*p, table, table_len, 0, &fp, &s, &need));
  if (out_len) *out_len = need;
  if (!out || cap < need) { set_reason("output buffer too small for the proof"); return Z0P_ERR_BUFFER_TOO_SMALL; }
  std::lock_guard<std::mutex> lk(c->mu);
  c->work_serial++;
  RC(with_device(c));
  ProfileScope ps(c);
  return table_prove_dev(c, *p, table, table_len, 0, nullptr, t, out);
}

int z0p_gpu_table_prove_zk(z0p_gpu_ctx* c, const z0p_table_params* p, const uint32_t* table,
                           size_t table_len, size_t n_rand, z0p_chacha20_state* rng,
                           z0p_transcript_state* t, uint8_t* out, size_t cap, size_t* out_len) {
  if (!c || !p || !t || !rng || rng->used > 64 || (!table && table_len)) return Z0P_ERR_INVALID_ARGUMENT;
  RC(table_validate(*p));  // src/table.rs:336-343
  if (table_len < 2) { set_reason("table needs at least two entries"); return Z0P_ERR_MALFORMED_INPUT; }
  if (n_rand < p->num_queries) {
    set_reason("n_rand must cover num_queries for hiding");
    return Z0P_ERR_MALFORMED_INPUT;
  }
  FriParams fp;
  FriShape s;
  uint64_t need = 0;
  RC(table_shape(*p, table, table_len, n_rand, &fp, &s, &need));
  if (out_len) *out_len = need;
  if (!out || cap < need) { set_reason("output buffer too small for the proof"); return Z0P_ERR_BUFFER_TOO_SMALL; }
  z0p_chacha20_state r = *rng;
  std::vector<uint32_t> rand(n_rand);
  for (auto& v : rand) v = chacha20_next_field(&r);
  std::lock_guard<std::mutex> lk(c->mu);
  c->work_serial++;
  RC(with_device(c));
  ProfileScope ps(c);
  RC(table_prove_dev(c, *p, table, table_len, n_rand, rand.data(), t, out));
  *rng = r;
  return Z0P_OK;
}

int z0p_fold_params_new(uint64_t seg_steps, uint64_t blowup, uint64_t num_queries,
                        uint64_t final_size, uint32_t in_a, uint32_t in_b, uint32_t out_b,
                        z0p_fold_params* out) {
  if (!out) return Z0P_ERR_INVALID_ARGUMENT;  // src/fold.rs:72-111
  if (seg_steps < 2 || !is_pow2(seg_steps)) return Z0P_ERR_INVALID_DOMAIN_SIZE;
  if (blowup < 4 || !is_pow2(blowup)) return Z0P_ERR_INVALID_BLOWUP;
  if (num_queries == 0) return Z0P_ERR_NO_QUERIES;
  if (final_size < 2 || !is_pow2(final_size)) return Z0P_ERR_INVALID_DOMAIN_SIZE;
  if (seg_steps > (1ull << 27) / blowup) return Z0P_ERR_INVALID_DOMAIN_SIZE;
  if (in_a >= P || in_b >= P || out_b >= P) {
    set_reason("field elements must be canonical (< p)");
    return Z0P_ERR_MALFORMED_INPUT;
  }
  *out = z0p_fold_params{seg_steps, blowup, num_queries, final_size, 0, 0, in_a, in_b, out_b};
  return Z0P_OK;
}

int z0p_fold_params_for_security(uint64_t seg_steps, uint32_t in_a, uint32_t in_b, uint32_t out_b,
                                 uint32_t target_bits, z0p_fold_params* out) {
  if (!out) return Z0P_ERR_INVALID_ARGUMENT;  // src/fold.rs:136-171
  if (seg_steps < 2 || !is_pow2(seg_steps)) return Z0P_ERR_INVALID_DOMAIN_SIZE;
  const uint64_t blowup = 16;
  if (seg_steps > (1ull << 27) / blowup) return Z0P_ERR_INVALID_DOMAIN_SIZE;
  if (in_a >= P || in_b >= P || out_b >= P) {
    set_reason("field elements must be canonical (< p)");
    return Z0P_ERR_MALFORMED_INPUT;
  }
  const uint64_t lde = seg_steps * blowup;
  uint64_t q = 0, fs = 0, ch = 0;
  uint32_t g = 0;
  tune_strength(target_bits, composition_millibits(lde, seg_steps - 1), &q, &g);
  tune_shape(lde, q, lde, 24, &fs, &ch);
  *out = z0p_fold_params{seg_steps, blowup, q, fs, g, ch, in_a, in_b, out_b};
  return Z0P_OK;
}

int z0p_gpu_fold_create(z0p_gpu_ctx* c, const z0p_fold_params* p, z0p_gpu_fold** out) {
  if (!c || !p || !out) return Z0P_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  z0p_gpu_fold* f = new z0p_gpu_fold();
  f->ctx = c;
  f->p = *p;
  *out = f;
  return Z0P_OK;
}

void z0p_gpu_fold_destroy(z0p_gpu_fold* f) {
  if (!f) return;
  {
    std::lock_guard<std::mutex> lk(f->ctx->mu);
    cudaSetDevice(f->ctx->device);
    for (DevBuf& b : f->slabs) release(f->ctx, b);
    release(f->ctx, f->tinv);
    release(f->ctx, f->table);
  }
  delete f;
}

size_t z0p_gpu_fold_len(const z0p_gpu_fold* f) { return f ? f->steps.size() : 0; }

int z0p_gpu_fold_add_segment(z0p_gpu_fold* f, const uint32_t* col_a, const uint32_t* col_b,
                             size_t len, z0p_transcript_state* t) {
  if (!f || !t || !col_a || !col_b) return Z0P_ERR_INVALID_ARGUMENT;
  if (f->finalized) {
    set_reason("the accumulator was finalized");
    return Z0P_ERR_INVALID_ARGUMENT;
  }
  RC(fold_validate(f->p));
  if (len != f->p.seg_steps) {
    set_reason("segment columns must match seg_steps");
    return Z0P_ERR_MALFORMED_INPUT;
  }
  std::lock_guard<std::mutex> lk(f->ctx->mu);
  f->ctx->work_serial++;
  RC(with_device(f->ctx));
  ProfileScope ps(f->ctx);
  return fold_add(f, col_a, col_b, t);
}

int z0p_gpu_fold_proof_size(const z0p_gpu_fold* f, size_t* len) {
  if (!f || !len) return Z0P_ERR_INVALID_ARGUMENT;
  if (f->steps.empty()) return Z0P_ERR_EMPTY_INPUT;
  FriParams fp;
  FriShape s;
  RC(fold_fri(f->p, &fp, &s));
  *len = fold_proof_bytes(f->p, f->steps.size(), s);
  return Z0P_OK;
}

int z0p_gpu_fold_finalize(z0p_gpu_fold* f, z0p_transcript_state* t, uint8_t* out, size_t cap,
                          size_t* len) {
  if (!f || !t) return Z0P_ERR_INVALID_ARGUMENT;
  if (f->finalized) {
    set_reason("the accumulator was finalized");
    return Z0P_ERR_INVALID_ARGUMENT;
  }
  if (f->steps.empty()) return Z0P_ERR_EMPTY_INPUT;  // src/fold.rs:495-497
  size_t need = 0;
  RC(z0p_gpu_fold_proof_size(f, &need));
  if (len) *len = need;
  if (!out || cap < need) {
    set_reason("output buffer too small for the proof");
    return Z0P_ERR_BUFFER_TOO_SMALL;
  }
  std::lock_guard<std::mutex> lk(f->ctx->mu);
  f->ctx->work_serial++;
  RC(with_device(f->ctx));
  ProfileScope ps(f->ctx);
  return fold_finalize(f, t, out);
}

int z0p_gpu_ctx_reserve_group(z0p_gpu_ctx* c, uint32_t max_group) {
  if (!c || max_group < 1 || max_group > (uint32_t)kMaxGroup) return Z0P_ERR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> lk(c->mu);
  RC(with_device(c));
  return ensure_slots(c, max_group);
}

void* z0p_gpu_ctx_stream(z0p_gpu_ctx* c) { return c ? (void*)c->stream : nullptr; }
size_t z0p_gpu_ctx_device_bytes(z0p_gpu_ctx* c) { return c ? c->held : 0; }


int z0p_gpu_air_prove(z0p_gpu_ctx* c, const z0p_air_params* p, z0p_transcript_state* ts,
                      uint8_t* out, size_t cap, size_t* len) {
  if (!c || !p || !ts) return Z0P_ERR_INVALID_ARGUMENT;
  return prove_group_abi(c, 1, p, &ts, &out, &cap, len, air_prove);
}

int z0p_gpu_air_compose(z0p_gpu_ctx* c, const z0p_air_params* p, const uint32_t* alphas,
                        uint32_t* d_out) {
  if (!c || !p || !alphas || !d_out) return Z0P_ERR_INVALID_ARGUMENT;
  for (int i = 0; i < 20; i++)
    if (alphas[i] >= P) {
      set_reason("alphas must be canonical field elements");
      return Z0P_ERR_MALFORMED_INPUT;
    }
  size_t need = 0;
  RC(z0p_air_proof_size(p, &need));
  std::vector<uint8_t> unused(need);
  z0p_transcript_state work;
  RC(z0p_transcript_init(&work, (const uint8_t*)"compose", 7));
  std::lock_guard<std::mutex> lk(c->mu);
  c->work_serial++;
  RC(with_device(c));
  RC(ensure_slots(c, 1));
  Transcript tr(&work);
  AirTask task{p, &tr, unused.data(), need, nullptr};
  task.fixed_alpha = alphas;
  task.layer0_out = d_out;
  return air_prove(c, &task, 1);
}

int z0p_gpu_air_prove_group(z0p_gpu_ctx* c, size_t n, const z0p_air_params* params,
                            z0p_transcript_state* const* transcripts, uint8_t* const* outs,
                            const size_t* caps, size_t* lens) {
  return prove_group_abi(c, n, params, transcripts, outs, caps, lens, air_prove);
}

int z0p_gpu_ctx_stats(z0p_gpu_ctx* c, z0p_gpu_stats* out) {
  if (!c || !out) return Z0P_ERR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> lk(c->mu);
  *out = z0p_gpu_stats{launch::launch_count(), c->h2d, c->d2h, c->syncs, c->proofs, c->sync_ns,
                       c->prove_ns};
  return Z0P_OK;
}

int z0p_gpu_ctx_set_profiling(z0p_gpu_ctx* c, int on) {
  if (!c) return Z0P_ERR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> lk(c->mu);
  c->profiling = on != 0;
  return Z0P_OK;
}

int z0p_gpu_ctx_profile(z0p_gpu_ctx* c, char* json, size_t cap, size_t* len) {
  if (!c || !len) return Z0P_ERR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> lk(c->mu);
  RC(with_device(c));
  CK(sync(c));
  struct Agg {
    std::string stage;
    double ms = 0;
    uint64_t calls = 0, kernels = 0;
  };
  std::vector<Agg> agg;
  for (auto& m : c->rec.marks) {
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, m.a, m.b) != cudaSuccess) ms = 0.f;
    size_t i = 0;
    while (i < agg.size() && agg[i].stage != m.stage) i++;
    if (i == agg.size()) agg.push_back({m.stage});
    agg[i].ms += ms;
    agg[i].calls += 1;
    agg[i].kernels += m.kernels;
  }
  std::string s = "{";
  for (size_t i = 0; i < agg.size(); i++) {
    char buf[200];
    snprintf(buf, sizeof buf, "%s\"%s\": {\"ms\": %.6f, \"calls\": %llu, \"kernels\": %llu}",
             i ? ", " : "", agg[i].stage.c_str(), agg[i].ms, (unsigned long long)agg[i].calls,
             (unsigned long long)agg[i].kernels);
    s += buf;
  }
  s += agg.empty() ? "\"host\": {" : ", \"host\": {";
  bool first = true;
  for (auto& kv : c->sites) {
    char buf[200];
    snprintf(buf, sizeof buf, "%s\"%s\": {\"calls\": %llu, \"wait_ms\": %.6f, \"before_ms\": %.6f}",
             first ? "" : ", ", kv.first.c_str(), (unsigned long long)kv.second.calls,
             kv.second.wait_ns * 1e-6, kv.second.before_ns * 1e-6);
    s += buf;
    first = false;
  }
  char tb[80];
  snprintf(tb, sizeof tb, "%s\"tail\": {\"ms\": %.6f}", first ? "" : ", ", c->tail_ns * 1e-6);
  s += tb;
  s += "}}";
  *len = s.size() + 1;
  if (!json || cap < s.size() + 1) return Z0P_ERR_BUFFER_TOO_SMALL;
  std::memcpy(json, s.c_str(), s.size() + 1);
  for (auto& m : c->rec.marks) {
    c->rec.pool.push_back(m.a);
    c->rec.pool.push_back(m.b);
  }
  c->rec.marks.clear();
  c->sites.clear();
  c->tail_ns = 0;
  return Z0P_OK;
}

int z0p_gpu_range_prove(z0p_gpu_ctx* c, const z0p_range_params* p, z0p_transcript_state* ts,
                        uint8_t* out, size_t cap, size_t* len) {
  if (!c || !p || !ts) return Z0P_ERR_INVALID_ARGUMENT;
  return prove_group_abi(c, 1, p, &ts, &out, &cap, len, range_prove);
}

int z0p_range_proof_size_zk(const z0p_range_params* p, size_t n_rand, size_t* len) {
  if (!p || !len) return Z0P_ERR_INVALID_ARGUMENT;
  FriParams fp;
  FriShape s;
  RC(range_zk_shape(*p, n_rand, &fp, &s));
  *len = range_size(*p, s);
  return Z0P_OK;
}

int z0p_gpu_range_prove_zk(z0p_gpu_ctx* c, const z0p_range_params* p, size_t n_rand,
                           z0p_chacha20_state* rng, z0p_transcript_state* t, uint8_t* out,
                           size_t cap, size_t* out_len) {
  if (!c || !p || !t || !rng || rng->used > 64) return Z0P_ERR_INVALID_ARGUMENT;
  FriParams fp;
  FriShape s;
  RC(range_zk_shape(*p, n_rand, &fp, &s));  // src/range.rs:399-404, then the shape
  const uint64_t need = range_size(*p, s);
  if (out_len) *out_len = need;
  if (!out || cap < need) {
    set_reason("output buffer too small for the proof");
    return Z0P_ERR_BUFFER_TOO_SMALL;
  }
  // Masking values, column after column (value first), n_rand each
  // (src/range.rs:411-414, src/blind.rs:65), on a copy of the stream.
  const uint64_t ncol = p->n_bits + 1;
  z0p_chacha20_state r = *rng;
  std::vector<uint32_t> rand(ncol * n_rand);
  for (auto& v : rand) v = chacha20_next_field(&r);
  std::lock_guard<std::mutex> lk(c->mu);
  c->work_serial++;
  RC(with_device(c));
  RC(ensure_slots(c, 1));
  ProfileScope ps(c);
  z0p_transcript_state work = *t;
  Transcript tr(&work);
  RangeTask task{p, &tr, out, cap, out_len};
  c->last_sync_ns = now_ns();
  const int rc = range_prove_columns(c, &task, 1, fp, s, need, nullptr, n_rand, rand.data());
  c->last_sync_ns = 0;
  if (rc != Z0P_OK) return rc;
  *t = work;
  *rng = r;
  c->proofs++;
  return Z0P_OK;
}

int z0p_gpu_range_prove_with_columns(z0p_gpu_ctx* c, const z0p_range_params* p,
                                     const uint32_t* v_col, size_t v_len,
                                     const uint32_t* const* bit_cols, const size_t* bit_lens,
                                     size_t n_bit_cols, z0p_transcript_state* t, uint8_t* out,
                                     size_t cap, size_t* out_len) {
  if (!c || !p || !t || (!v_col && v_len) || (n_bit_cols && (!bit_cols || !bit_lens)))
    return Z0P_ERR_INVALID_ARGUMENT;
  RC(range_validate(*p));  // src/range.rs:359-366: params, then the column shapes
  bool shape_ok = v_len == p->n_rows && n_bit_cols == p->n_bits;
  for (size_t i = 0; shape_ok && i < n_bit_cols; i++)
    shape_ok = bit_cols[i] && bit_lens[i] == p->n_rows;
  if (!shape_ok) {
    set_reason("range columns must match n_rows/n_bits");
    return Z0P_ERR_MALFORMED_INPUT;
  }
  FriParams fp;
  FriShape s;
  RC(range_shape(*p, &fp, &s));
  const uint64_t need = range_size(*p, s);
  if (out_len) *out_len = need;
  if (!out || cap < need) {
    set_reason("output buffer too small for the proof");
    return Z0P_ERR_BUFFER_TOO_SMALL;
  }
  std::vector<const uint32_t*> cols(n_bit_cols + 1);
  cols[0] = v_col;
  for (size_t i = 0; i < n_bit_cols; i++) cols[i + 1] = bit_cols[i];
  std::lock_guard<std::mutex> lk(c->mu);
  c->work_serial++;
  RC(with_device(c));
  RC(ensure_slots(c, 1));
  ProfileScope ps(c);
  z0p_transcript_state work = *t;
  Transcript tr(&work);
  RangeTask task{p, &tr, out, cap, out_len};
  c->last_sync_ns = now_ns();
  const int rc = range_prove_columns(c, &task, 1, fp, s, need, cols.data());
  c->last_sync_ns = 0;
  if (rc != Z0P_OK) return rc;
  *t = work;
  c->proofs++;
  return Z0P_OK;
}

int z0p_gpu_range_prove_group(z0p_gpu_ctx* c, size_t n, const z0p_range_params* params,
                              z0p_transcript_state* const* transcripts, uint8_t* const* outs,
                              const size_t* caps, size_t* lens) {
  return prove_group_abi(c, n, params, transcripts, outs, caps, lens, range_prove);
}

int z0p_gpu_rs_extend(z0p_gpu_ctx* c, const uint32_t* d_values, uint64_t n, uint64_t batch,
                      uint64_t blowup, uint32_t* d_out) {
  if (!c || !d_values || !d_out || batch == 0 || batch > 65535) return Z0P_ERR_INVALID_ARGUMENT;
  if (!is_pow2(n) || n > MAX_DOMAIN) return Z0P_ERR_INVALID_DOMAIN_SIZE;  // src/ntt.rs:441-446
  if (!is_pow2(blowup)) return Z0P_ERR_INVALID_BLOWUP;
  if (n * blowup > MAX_DOMAIN || batch * blowup > 65535) return Z0P_ERR_INVALID_DOMAIN_SIZE;
  std::lock_guard<std::mutex> lk(c->mu);
  c->work_serial++;
  RC(with_device(c));
  ProfileScope ps(c);
  uint32_t logn = log2u(n), logm = logn + log2u(blowup);
  RC(ensure(c, c->coeffs, 4 * n * batch));
  RC(ensure(c, c->scratch, 4 * n * batch * blowup));
  NttPlan ip;
  ip.logn = logn; ip.batch = (uint32_t)batch; ip.inverse = 1; ip.post_gamma = 1;
  CK(launch::ntt(c->stream, c->tb, ip, d_values, (uint32_t*)c->coeffs.p, (uint32_t*)c->scratch.p));
  // The LDE kernels write coset-major [c][j][q]; this entry returns the
  // natural order [c][k], k = B q + j.
  RC(ensure(c, c->lde, 4 * n * batch * blowup));
  NttPlan lp;
  lp.logn = logn; lp.batch = (uint32_t)(batch * blowup); lp.in_div = (uint32_t)blowup;
  lp.twist_mod = (uint32_t)blowup; lp.twist_shift = 27 - logm;
  CK(launch::ntt(c->stream, c->tb, lp, (uint32_t*)c->coeffs.p, (uint32_t*)c->lde.p,
                 (uint32_t*)c->scratch.p));
  CK(launch::coset_to_natural(c->stream, (const uint32_t*)c->lde.p, d_out, logn, log2u(blowup),
                              batch));
  CK(sync(c));
  return Z0P_OK;
}

int z0p_gpu_merkle_flat64_cap(z0p_gpu_ctx* c, const uint8_t* d_flat, uint64_t len,
                              uint64_t cap_height, uint8_t* h_cap, uint64_t* cap_count) {
  if (!c || !d_flat || !h_cap || !cap_count) return Z0P_ERR_INVALID_ARGUMENT;
  if (len == 0) return Z0P_ERR_EMPTY_INPUT;  // src/merkle.rs:93-110
  if (len % 64) return Z0P_ERR_MALFORMED_INPUT;
  const uint64_t count = len / 64;
  uint64_t leaves = 1;  // padded by duplicating the last leaf (src/merkle.rs:350-360)
  while (leaves < count) leaves <<= 1;
  std::lock_guard<std::mutex> lk(c->mu);
  c->work_serial++;
  RC(with_device(c));
  ProfileScope ps(c);
  RC(ensure(c, c->ttree, 32 * tree_digests(leaves)));
  uint32_t* tree = (uint32_t*)c->ttree.p;
  uint32_t depth = log2u(leaves), drop = cap_height < depth ? (uint32_t)cap_height : depth;
  RC(ensure_hio(c, 32ull << drop));
  CK(launch::merkle_flat64_leaves(c->stream, (const uint32_t*)d_flat, count, leaves, tree));
  CK(launch::merkle_build(c->stream, tree, leaves, depth - drop, merkle_counter(c),
                          hio_dev<uint32_t>(c, 0)));
  CK(sync(c));
  std::memcpy(h_cap, c->hio, 32ull << drop);
  *cap_count = 1ull << drop;
  return Z0P_OK;
}

int z0p_gpu_fri_fold(z0p_gpu_ctx* c, const uint32_t* d_in, uint64_t n, uint64_t lde_len,
                     uint64_t depth, const uint32_t ch[12], uint32_t* d_out) {
  if (!c || !d_in || !d_out || !ch) return Z0P_ERR_INVALID_ARGUMENT;
  if (!is_pow2(n) || n < 4 || !is_pow2(lde_len) || lde_len > MAX_DOMAIN || depth > 13 ||
      (lde_len >> (2 * depth)) != n)
    return Z0P_ERR_INVALID_DOMAIN_SIZE;
  std::lock_guard<std::mutex> lk(c->mu);
  c->work_serial++;
  RC(with_device(c));
  ProfileScope ps(c);
  RC(ensure(c, c->ftrees, 32 * (n / 4 + 4)));
  FoldArgs fa;
  fa.in = d_in;
  fa.out = d_out;
  fa.leaves = (uint32_t*)c->ftrees.p;
  fa.logn = log2u(n);
  uint32_t g = GENERATOR;
  for (uint64_t i = 0; i < depth; i++) g = fpow(g, 4);
  fa.ginv_m = to_mont(finv(g));
  fa.unit_m = to_mont(two_adic_generator(2));
  const uint32_t inv4 = finv(4);
  RC(ensure_hio(c, 4 * kFoldTabWords));
  // Without a tree counter the fold reads the slot (n >= 16), or, below 16
  // values, the tables in the mapped buffer in place: both are filled.
  uint32_t(*tab)[4][4] = reinterpret_cast<uint32_t(*)[4][4]>(c->hio);
  for (int k = 0; k < 3; k++) {
    uint32_t q[4];
    for (int e = 0; e < 4; e++) q[e] = fmul(ch[4 * k + e] % P, inv4);
    e4_table(q, c->consts->tab[k]);
    std::memcpy(tab[k], c->consts->tab[k], sizeof tab[k]);
  }
  fa.tab = hio_dev<uint32_t>(c, 0);
  fa.slot = (uint32_t)c->slot;
  CK(push_consts(c, 1));
  uint32_t built = 0;
  CK(launch::fri_fold(c->stream, c->tb, fa, &built));  // top 0, no cap: leaves only
  CK(sync(c));
  return Z0P_OK;
}

int z0p_gpu_blake3_ceiling(z0p_gpu_ctx* c, double* gcompress_per_s) {
  if (!c || !gcompress_per_s) return Z0P_ERR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> lk(c->mu);
  c->work_serial++;
  RC(with_device(c));
  int sms = 0;
  CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c->device));
  const uint32_t blocks = 8u * (uint32_t)sms;
  const size_t threads = 256ull * blocks;
  const int iters = 256;
  RC(ensure(c, c->scratch, threads * 64 + threads * 32));
  uint32_t* in = (uint32_t*)c->scratch.p;
  uint32_t* outp = in + 16 * threads;
  CK(cudaMemsetAsync(in, 0x5a, threads * 64, c->stream));
  cudaEvent_t e0, e1;
  CK(cudaEventCreate(&e0));
  CK(cudaEventCreate(&e1));
  cudaError_t e = launch::hash_ceiling(c->stream, in, outp, blocks, iters);  // warm-up
  float best = 0.f;
  for (int rep = 0; rep < 3 && e == cudaSuccess; rep++) {
    e = cudaEventRecord(e0, c->stream);
    if (e == cudaSuccess) e = launch::hash_ceiling(c->stream, in, outp, blocks, iters);
    if (e == cudaSuccess) e = cudaEventRecord(e1, c->stream);
    if (e == cudaSuccess) e = cudaEventSynchronize(e1);
    float ms = 0.f;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
    if (e == cudaSuccess && ms > 0.f) {
      float g = (float)(2.0 * threads * iters / (ms * 1e-3) / 1e9);
      if (g > best) best = g;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  CK(e);
  *gcompress_per_s = best;
  return Z0P_OK;
}

static launch::Schedule from_abi(const z0p_schedule& s) {
  launch::Schedule o;
  std::memcpy(o.ntt_log_n1, s.ntt_log_n1, sizeof o.ntt_log_n1);
  std::memcpy(o.ntt_radix32, s.ntt_radix32, sizeof o.ntt_radix32);
  o.merkle_top_log = s.merkle_top_log;
  o.grind_ctas_per_sm = s.grind_ctas_per_sm;
  return o;
}

static z0p_schedule to_abi(const launch::Schedule& s) {
  z0p_schedule o;
  std::memcpy(o.ntt_log_n1, s.ntt_log_n1, sizeof o.ntt_log_n1);
  std::memcpy(o.ntt_radix32, s.ntt_radix32, sizeof o.ntt_radix32);
  o.merkle_top_log = s.merkle_top_log;
  o.grind_ctas_per_sm = s.grind_ctas_per_sm;
  return o;
}

int z0p_schedule_default(z0p_schedule* out) {
  if (!out) return Z0P_ERR_INVALID_ARGUMENT;
  *out = to_abi(launch::Schedule{});
  return Z0P_OK;
}

int z0p_gpu_schedule_get(int device, z0p_schedule* out) {
  if (!out || device < 0 || device >= 64) return Z0P_ERR_INVALID_ARGUMENT;
  *out = to_abi(launch::get_schedule(device));
  return Z0P_OK;
}

int z0p_gpu_schedule_set(int device, const z0p_schedule* s) {
  if (!s || device < 0 || device >= 64) return Z0P_ERR_INVALID_ARGUMENT;
  const launch::Schedule v = from_abi(*s);
  if (!launch::schedule_valid(v)) {
    set_reason("schedule field out of range");
    return Z0P_ERR_INVALID_ARGUMENT;
  }
  launch::set_schedule(device, v);
  return Z0P_OK;
}

// Device time of `run` (ms): the fastest of `reps` event-timed calls after
// one untimed call.
static cudaError_t time_best(z0p_gpu_ctx* c, cudaEvent_t e0, cudaEvent_t e1, int reps,
                             const std::function<cudaError_t()>& run, float* ms) {
  cudaError_t e = run();
  *ms = 0.f;
  for (int r = 0; r < reps && e == cudaSuccess; r++) {
    e = cudaEventRecord(e0, c->stream);
    if (e == cudaSuccess) e = run();
    if (e == cudaSuccess) e = cudaEventRecord(e1, c->stream);
    if (e == cudaSuccess) e = cudaEventSynchronize(e1);
    float t = 0.f;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&t, e0, e1);
    if (e == cudaSuccess && (r == 0 || t < *ms)) *ms = t;
  }
  return e;
}

static int autotune_locked(z0p_gpu_ctx* c, uint32_t max_log_n, launch::Schedule* best,
                           z0p_tune_report* rep, cudaEvent_t e0, cudaEvent_t e1) {
  constexpr float kKeep = 0.97f;  // a candidate must beat the default by 3%
  constexpr uint32_t B = 16;      // LDE cosets: the production blowup
  const launch::Schedule base{};
  *best = base;
  auto use = [&](const launch::Schedule& s) { launch::set_schedule(c->device, s); };

  // Four-step NTT splits and register-group radix, one LDE of 16 cosets of
  // 2^l per run.
  const uint32_t top_l = max_log_n < 22 ? max_log_n : 22;
  if (top_l >= 13) {
    const size_t n_max = 1ull << top_l;
    RC(ensure(c, c->coeffs, 4 * n_max));
    RC(ensure(c, c->lde, 4 * B * n_max));
    RC(ensure(c, c->scratch, 4 * B * n_max));
    CK(cudaMemsetAsync(c->coeffs.p, 0x11, 4 * n_max, c->stream));
  }
  for (uint32_t l = 13; l <= top_l; l++) {
    NttPlan plan;
    plan.logn = l;
    plan.batch = B;
    plan.in_div = B;
    plan.twist_mod = B;
    plan.twist_shift = 27 - (l + log2u(B));
    auto run = [&]() {
      return launch::ntt(c->stream, c->tb, plan, (const uint32_t*)c->coeffs.p, (uint32_t*)c->lde.p,
                         (uint32_t*)c->scratch.p);
    };
    uint32_t lo, hi;
    launch::ntt_split_range(l, &lo, &hi);
    const uint32_t def = launch::ntt_default_split(l);
    const uint32_t def_r = base.ntt_radix32[l];  // the default schedule's variant
    float t_def = 0.f, t_best = 0.f;
    uint32_t pick = 0, pick_r32 = 0;
    for (uint32_t s1 = (def > lo + 2 ? def - 2 : lo); s1 <= hi && s1 <= def + 2; s1++)
      for (uint32_t r32 = 0; r32 < 4; r32++) {
        if (r32 >= 2 && !(launch::reg_split_ok(s1) && launch::reg_split_ok(l - s1))) continue;
        launch::Schedule s = base;
        s.ntt_log_n1[l] = (uint8_t)s1;
        s.ntt_radix32[l] = (uint8_t)r32;
        use(s);
        float t = 0.f;
        CK(time_best(c, e0, e1, 3, run, &t));
        if (s1 == def && r32 == def_r) t_def = t;
        if (pick == 0 || t < t_best) {
          t_best = t;
          pick = s1;
          pick_r32 = r32;
        }
      }
    if ((pick != def || pick_r32 != def_r) && t_best > kKeep * t_def) {
      pick = def;
      pick_r32 = def_r;
      t_best = t_def;
    }
    best->ntt_log_n1[l] = pick == def ? 0 : (uint8_t)pick;
    best->ntt_radix32[l] = (uint8_t)pick_r32;
    if (rep) {
      rep->ntt_default_us[l] = 1e3f * t_def;
      rep->ntt_best_us[l] = 1e3f * t_best;
    }
  }

  // Merkle top level, on a 2^21-leaf tree (the trace tree of a 2^20-step
  // proof), every level above the leaves.
  {
    const uint64_t leaves = 1ull << 21;
    RC(ensure(c, c->ttree, 32 * tree_digests(leaves)));
    uint32_t* tree = (uint32_t*)c->ttree.p;
    CK(cudaMemsetAsync(tree, 0x5a, 32 * leaves, c->stream));
    const uint32_t top = 21 - 4;
    auto run = [&]() {
      return launch::merkle_build(c->stream, tree, leaves, top, merkle_counter(c), nullptr, 0, 1, 0, 0);
    };
    float t_def = 0.f, t_best = 0.f;
    uint32_t pick = 0;
    for (uint32_t tl = 12; tl <= 18; tl++) {
      launch::Schedule s = base;
      s.merkle_top_log = tl;
      use(s);
      float t = 0.f;
      CK(time_best(c, e0, e1, 3, run, &t));
      if (tl == base.merkle_top_log) t_def = t;
      if (pick == 0 || t < t_best) {
        t_best = t;
        pick = tl;
      }
    }
    if (t_best > kKeep * t_def) {
      pick = base.merkle_top_log;
      t_best = t_def;
    }
    best->merkle_top_log = pick;
    if (rep) {
      rep->merkle_default_us = 1e3f * t_def;
      rep->merkle_best_us = 1e3f * t_best;
    }
  }

  // Proof-of-work grid: 20-bit searches on eight fixed heads, timed together
  // (a search's time depends on where its first hit lies); every grid must
  // find the same nonces.
  {
    constexpr int kHeads = 8;
    const size_t heads_at = 16 * kHeads;  // results first, then the heads
    RC(ensure_hio(c, heads_at + 4 * kPowHeadWords * kHeads));
    for (int h = 0; h < kHeads; h++) {
      uint8_t head[kPowHeadBytes];
      for (uint32_t i = 0; i < kPowHeadBytes; i++) head[i] = (uint8_t)(0x3c ^ (7 * i) ^ (29 * h));
      set_head(reinterpret_cast<uint32_t*>(c->hio + heads_at) + kPowHeadWords * h, head, sizeof head);
    }
    auto run = [&]() {  // eight single searches, one after the other, as proofs run them
      cudaError_t e = cudaSuccess;
      for (int h = 0; h < kHeads && e == cudaSuccess; h++)
        e = launch::grind(c->stream, hio_dev<uint32_t>(c, heads_at) + kPowHeadWords * h,
                          kPowHeadBytes, 20, grind_state(c),
                          hio_dev<unsigned long long>(c, 16 * h), 1ull << 40, 1);
      return e;
    };
    float t_def = 0.f, t_best = 0.f;
    uint32_t pick = 0;
    unsigned long long nonce0[kHeads] = {};
    for (uint32_t per : {1u, 2u, 3u, 4u, 6u, 8u}) {
      launch::Schedule s = base;
      s.grind_ctas_per_sm = per;
      use(s);
      float t = 0.f;
      CK(time_best(c, e0, e1, 3, run, &t));
      for (int h = 0; h < kHeads; h++) {
        unsigned long long res[2];
        std::memcpy(res, c->hio + 16 * h, 16);  // the last run's result; the stream is idle
        if (res[1] != 0 || res[0] == ~0ull || (pick != 0 && res[0] != nonce0[h])) {
          set_reason("autotune: proof-of-work grids disagree on the nonce");
          return Z0P_ERR_UNSUPPORTED;
        }
        nonce0[h] = res[0];
      }
      if (per == base.grind_ctas_per_sm) t_def = t;
      if (pick == 0 || t < t_best) {
        t_best = t;
        pick = per;
      }
    }
    if (t_best > kKeep * t_def) {
      pick = base.grind_ctas_per_sm;
      t_best = t_def;
    }
    best->grind_ctas_per_sm = pick;
    if (rep) {
      rep->grind_default_us = 1e3f * t_def;
      rep->grind_best_us = 1e3f * t_best;
    }
  }
  return Z0P_OK;
}

int z0p_gpu_autotune(z0p_gpu_ctx* c, uint32_t max_log_n, z0p_schedule* out, z0p_tune_report* rep) {
  if (!c || !out || max_log_n > 26) return Z0P_ERR_INVALID_ARGUMENT;
  const auto w0 = std::chrono::steady_clock::now();
  std::lock_guard<std::mutex> lk(c->mu);
  c->work_serial++;
  RC(with_device(c));
  if (rep) std::memset(rep, 0, sizeof *rep);
  const launch::Schedule before = launch::get_schedule(c->device);
  cudaEvent_t e0, e1;
  CK(cudaEventCreate(&e0));
  if (cudaEventCreate(&e1) != cudaSuccess) {
    cudaEventDestroy(e0);
    set_reason("cudaEventCreate failed");
    return Z0P_ERR_CUDA;
  }
  launch::Schedule best;
  const int rc = autotune_locked(c, max_log_n, &best, rep, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  launch::set_schedule(c->device, rc == Z0P_OK ? best : before);
  if (rc != Z0P_OK) return rc;
  *out = to_abi(best);
  if (rep)
    rep->wall_ms = (float)std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - w0).count();
  return Z0P_OK;
}

int z0p_gpu_grind(z0p_gpu_ctx* c, const uint8_t* head, size_t head_len, uint32_t bits,
                  uint64_t* nonce) {
  if (!c || !head || !nonce) return Z0P_ERR_INVALID_ARGUMENT;
  if (bits > 32) {
    set_reason("grinding difficulty above 32 bits");
    return Z0P_ERR_MALFORMED_INPUT;
  }
  if (!launch::grind_supports((uint32_t)head_len)) {
    set_reason("grind head length not supported by the device kernel");
    return Z0P_ERR_UNSUPPORTED;
  }
  std::lock_guard<std::mutex> lk(c->mu);
  c->work_serial++;
  RC(with_device(c));
  ProfileScope ps(c);
  RC(ensure_hio(c, 16 + 4 * kPowHeadWords));  // the result, then the head
  set_head(reinterpret_cast<uint32_t*>(c->hio + 16), head, head_len);
  c->h2d += 4 * kPowHeadWords;
  CK(launch::grind(c->stream, hio_dev<uint32_t>(c, 16), (uint32_t)head_len, bits, grind_state(c),
                   hio_dev<unsigned long long>(c, 0), 1ull << 40));
  CK(sync(c));
  unsigned long long res[2];
  std::memcpy(res, c->hio, 16);
  if (res[1] != 0 || res[0] == ~0ull) {
    set_reason("proof-of-work search reached its nonce cap without a solution");
    return Z0P_ERR_DEVICE_TIMEOUT;
  }
  *nonce = res[0];
  return Z0P_OK;
}

}  // extern "C"
