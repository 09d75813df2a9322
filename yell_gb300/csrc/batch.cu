// Batched polymul over polynomials of uneven degree N and limb count L.
//
// The batch is split into size buckets (one per degree).  Each bucket is
// flattened into device-resident lists of limb pointers and modulus indices,
// so one launch sequence (1 kernel for whole-limb degrees, 4 for two-pass
// degrees) covers every polymul of that degree whatever its L.  Buckets run
// concurrently on forked streams.  The whole fork/launch/join sequence is
// captured once into a CUDA graph per batch shape (the ordered list of
// (degree, limb count) buckets); later batches of the same shape upload their
// pointer lists and replay the graph.
#include <algorithm>
#include <array>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "kernels.h"
#include "runtime.h"
#include "yell_gb300.h"

using namespace yell_gb300;

namespace {

constexpr int kDegrees = (int)(kMaxLogN - kMinLogN + 1);

struct CachedGraph {
  cudaGraphExec_t exec = nullptr;
  uint64_t launches = 0;
};

struct BatchState {
  std::mutex mu;
  uint8_t* d_lists = nullptr;  // device: pointer lists + modulus lists of every bucket
  size_t lists_bytes = 0;
  uint8_t* h_lists = nullptr;  // pinned staging of the same
  size_t h_bytes = 0;
  uint64_t* d_scratch = nullptr;
  size_t scratch_words = 0;
  uint64_t generation = 0;  // bumps when a buffer moves (cached graphs are stale)
  cudaStream_t side[kDegrees] = {};
  cudaEvent_t fork = nullptr, staged = nullptr, user_ev = nullptr, done_ev = nullptr;
  cudaEvent_t join[kDegrees] = {};
  std::map<std::string, CachedGraph> graphs;
  bool ready = false;

  int init() {
    for (int i = 0; i < kDegrees; ++i) {
      cudaError_t e = cudaStreamCreateWithFlags(&side[i], cudaStreamNonBlocking);
      if (e != cudaSuccess) return fail_cuda(e, "cudaStreamCreate(batch)");
      e = cudaEventCreateWithFlags(&join[i], cudaEventDisableTiming);
      if (e != cudaSuccess) return fail_cuda(e, "cudaEventCreate(batch)");
    }
    cudaEvent_t* evs[] = {&fork, &staged, &user_ev, &done_ev};
    for (cudaEvent_t* ev : evs) {
      cudaError_t e = cudaEventCreateWithFlags(ev, cudaEventDisableTiming);
      if (e != cudaSuccess) return fail_cuda(e, "cudaEventCreate(batch)");
    }
    ready = true;
    return kOk;
  }

  void drop_graphs() {
    for (auto& kv : graphs) cudaGraphExecDestroy(kv.second.exec);
    graphs.clear();
    ++generation;
  }

  int reserve_lists(size_t bytes) {
    if (bytes <= lists_bytes && bytes <= h_bytes) return kOk;
    // the previous upload must have finished before the staging is replaced
    cudaEventSynchronize(staged);
    drop_graphs();
    if (d_lists) cudaFree(d_lists);
    if (h_lists) cudaFreeHost(h_lists);
    d_lists = nullptr;
    h_lists = nullptr;
    lists_bytes = h_bytes = 0;
    const size_t want = std::max<size_t>(bytes, 1 << 16) * 2;
    cudaError_t e = cudaMalloc(&d_lists, want);
    if (e != cudaSuccess) return fail_cuda(e, "cudaMalloc(batch lists)");
    e = cudaMallocHost(&h_lists, want);
    if (e != cudaSuccess) return fail_cuda(e, "cudaMallocHost(batch lists)");
    lists_bytes = h_bytes = want;
    return kOk;
  }

  int reserve_scratch(size_t words) {
    if (words <= scratch_words) return kOk;
    drop_graphs();
    if (d_scratch) cudaFree(d_scratch);
    d_scratch = nullptr;
    scratch_words = 0;
    cudaError_t e = cudaMalloc(&d_scratch, words * sizeof(uint64_t));
    if (e != cudaSuccess) return fail_cuda(e, "cudaMalloc(batch scratch)");
    scratch_words = words;
    return kOk;
  }
};

BatchState* batch_state(int dev, int* st) {
  static std::mutex mu;
  static std::array<std::unique_ptr<BatchState>, 64> states;
  std::lock_guard<std::mutex> g(mu);
  if (!states[dev]) {
    std::unique_ptr<BatchState> s(new BatchState());
    *st = s->init();
    if (*st != kOk) return nullptr;
    states[dev] = std::move(s);
  }
  *st = kOk;
  return states[dev].get();
}

struct BucketLayout {
  uint32_t log_n = 0;
  uint32_t limbs = 0;
  size_t c_off = 0, a_off = 0, b_off = 0, cm_off = 0;  // byte offsets in the lists
  size_t scratch_off = 0;                              // word offset in the scratch
  const DevMod* mods = nullptr;
};

int validate(const yell_polymul_desc& d) {
  if (!d.c || !d.a || !d.b) return fail(kInvalidArgument, "null pointer in a batch entry");
  if (d.c == d.a || d.c == d.b) return fail(kInvalidArgument, "batch entry output aliases an operand");
  const uintptr_t m = reinterpret_cast<uintptr_t>(d.c) | reinterpret_cast<uintptr_t>(d.a) |
                      reinterpret_cast<uintptr_t>(d.b);
  if (m % 16) return fail(kInvalidArgument, "batch entry pointers must be 16-byte aligned");
  int st = check_degree(d.log_n);
  if (st != kOk) return st;
  return check_moduli(d.cm0, d.L);
}

}  // namespace

extern "C" int yell_dev_polymul_batch(const yell_polymul_desc* descs, uint32_t n, void* stream) {
  if (!descs || n == 0) return fail(kInvalidArgument, "empty batch");
  for (uint32_t i = 0; i < n; ++i) {
    const int st = validate(descs[i]);
    if (st != kOk) return st;
  }
  int st = kOk;
  DeviceContext* ctx = DeviceContext::current(&st);
  if (!ctx) return st;
  BatchState* bs = batch_state(ctx->device(), &st);
  if (!bs) return st;
  std::lock_guard<std::mutex> g(bs->mu);

  // ---- buckets and their list layout -----------------------------------
  std::vector<BucketLayout> buckets;
  std::array<int, kDegrees> index;
  index.fill(-1);
  std::array<std::vector<uint32_t>, kDegrees> members;
  for (uint32_t i = 0; i < n; ++i) members[descs[i].log_n - kMinLogN].push_back(i);
  size_t bytes = 0, scratch = 0;
  for (int k = 0; k < kDegrees; ++k) {
    if (members[k].empty()) continue;
    BucketLayout b;
    b.log_n = kMinLogN + k;
    std::vector<uint32_t> cms;
    for (uint32_t i : members[k]) {
      b.limbs += descs[i].L;
      for (uint32_t l = 0; l < descs[i].L; ++l) cms.push_back(descs[i].cm0 + l);
    }
    st = ctx->ensure_tables_list(b.log_n, cms.data(), (uint32_t)cms.size(), &b.mods);
    if (st != kOk) return st;
    b.c_off = bytes;
    bytes += 8 * (size_t)b.limbs;
    b.a_off = bytes;
    bytes += 8 * (size_t)b.limbs;
    b.b_off = bytes;
    bytes += 8 * (size_t)b.limbs;
    b.cm_off = bytes;
    bytes += ((4 * (size_t)b.limbs + 15) / 16) * 16;
    b.scratch_off = scratch;
    scratch += polymul_scratch_words(b.limbs, b.log_n, ctx->shape);
    index[k] = (int)buckets.size();
    buckets.push_back(b);
  }
  st = bs->reserve_lists(bytes);
  if (st != kOk) return st;
  st = bs->reserve_scratch(std::max<size_t>(scratch, 2));
  if (st != kOk) return st;

  // ---- fill the pinned staging (after the previous upload has drained) ---
  cudaError_t e = cudaEventSynchronize(bs->staged);
  if (e != cudaSuccess) return fail_cuda(e, "batch staging wait");
  for (const BucketLayout& b : buckets) {
    uint64_t* c = reinterpret_cast<uint64_t*>(bs->h_lists + b.c_off);
    uint64_t* a = reinterpret_cast<uint64_t*>(bs->h_lists + b.a_off);
    uint64_t* bb = reinterpret_cast<uint64_t*>(bs->h_lists + b.b_off);
    uint32_t* cm = reinterpret_cast<uint32_t*>(bs->h_lists + b.cm_off);
    size_t k = 0;
    const size_t nw = (size_t)1 << b.log_n;
    for (uint32_t i : members[b.log_n - kMinLogN]) {
      const yell_polymul_desc& d = descs[i];
      for (uint32_t l = 0; l < d.L; ++l, ++k) {
        c[k] = reinterpret_cast<uint64_t>(d.c + l * nw);
        a[k] = reinterpret_cast<uint64_t>(d.a + l * nw);
        bb[k] = reinterpret_cast<uint64_t>(d.b + l * nw);
        cm[k] = d.cm0 + l;
      }
    }
  }

  cudaStream_t s = ctx->stream();
  if (stream) {
    e = cudaEventRecord(bs->user_ev, static_cast<cudaStream_t>(stream));
    if (e == cudaSuccess) e = cudaStreamWaitEvent(s, bs->user_ev, 0);
    if (e != cudaSuccess) return fail_cuda(e, "batch stream ordering");
  }
  e = cudaMemcpyAsync(bs->d_lists, bs->h_lists, bytes, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaEventRecord(bs->staged, s);
  if (e != cudaSuccess) return fail_cuda(e, "batch list upload");

  // ---- graph per batch shape --------------------------------------------
  std::string sig = std::to_string(bs->generation);
  for (const BucketLayout& b : buckets) sig += ";" + std::to_string(b.log_n) + ":" + std::to_string(b.limbs);
  auto it = bs->graphs.find(sig);
  if (it == bs->graphs.end()) {
    const uint64_t launches0 = g_kernel_launches.load();
    e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return fail_cuda(e, "batch capture begin");
    cudaError_t le = cudaEventRecord(bs->fork, s);
    for (size_t i = 0; i < buckets.size() && le == cudaSuccess; ++i) {
      const BucketLayout& b = buckets[i];
      cudaStream_t side = bs->side[b.log_n - kMinLogN];
      le = cudaStreamWaitEvent(side, bs->fork, 0);
      if (le != cudaSuccess) break;
      LimbSet c;
      c.base = nullptr;
      c.ptrs = reinterpret_cast<uint64_t* const*>(bs->d_lists + b.c_off);
      c.cms = reinterpret_cast<const uint32_t*>(bs->d_lists + b.cm_off);
      c.count = b.limbs;
      c.L = 1;
      c.cm0 = 0;
      c.pad_ = 0;
      ConstLimbSet a{nullptr, reinterpret_cast<const uint64_t* const*>(bs->d_lists + b.a_off), c.cms,
                     b.limbs, 1, 0, 0};
      ConstLimbSet bb{nullptr, reinterpret_cast<const uint64_t* const*>(bs->d_lists + b.b_off), c.cms,
                      b.limbs, 1, 0, 0};
      le = launch_polymul(c, a, bb, b.log_n, b.mods, bs->d_scratch + b.scratch_off, ctx->shape, side);
      if (le == cudaSuccess) le = cudaEventRecord(bs->join[b.log_n - kMinLogN], side);
      if (le == cudaSuccess) le = cudaStreamWaitEvent(s, bs->join[b.log_n - kMinLogN], 0);
    }
    cudaGraph_t graph = nullptr;
    e = cudaStreamEndCapture(s, &graph);
    if (le != cudaSuccess) {
      if (graph) cudaGraphDestroy(graph);
      return fail_cuda(le, "batch capture");
    }
    if (e != cudaSuccess) return fail_cuda(e, "batch capture end");
    CachedGraph cg;
    e = cudaGraphInstantiate(&cg.exec, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) return fail_cuda(e, "batch graph instantiate");
    cg.launches = g_kernel_launches.load() - launches0;
    g_kernel_launches -= cg.launches;  // counted when the graph runs
    it = bs->graphs.emplace(sig, cg).first;
  }
  e = cudaGraphLaunch(it->second.exec, s);
  if (e != cudaSuccess) return fail_cuda(e, "batch graph launch");
  g_kernel_launches += it->second.launches;
  if (stream) {
    e = cudaEventRecord(bs->done_ev, s);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(static_cast<cudaStream_t>(stream), bs->done_ev, 0);
    if (e != cudaSuccess) return fail_cuda(e, "batch stream ordering");
  }
  return kOk;
}
