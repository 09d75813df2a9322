// Batched polymul over polynomials of uneven degree N and limb count L.
//
// The batch is split into size buckets (one per degree).  Each bucket is
// flattened into device-resident lists of limb pointers and modulus indices,
// so one launch sequence (1 kernel for whole-limb degrees, 3 for two-pass
// degrees) covers every polymul of that degree whatever its L.  Buckets run
// concurrently on forked streams, launched in degree order (starting the
// largest buckets first measured 1% slower on the 512-polymul uneven batch).  With graphs on, the whole fork/launch/join
// sequence is captured once per batch shape (the ordered list of (degree,
// limb count) buckets); later batches of the same shape upload their pointer
// lists and replay the graph.
#include "batch.h"

#include <algorithm>
#include <array>

#include "batch_queue.h"
#include "profiler.h"
#include <cstring>
#include <memory>

namespace yell_gb300 {

int BatchExecutor::init() {
  for (int i = 0; i < kDegrees; ++i) {
    cudaError_t e = cudaStreamCreateWithFlags(&side_[i], cudaStreamNonBlocking);
    if (e != cudaSuccess) return fail_cuda(e, "cudaStreamCreate(batch)");
    e = cudaEventCreateWithFlags(&join_[i], cudaEventDisableTiming);
    if (e != cudaSuccess) return fail_cuda(e, "cudaEventCreate(batch)");
  }
  cudaError_t e = cudaEventCreateWithFlags(&fork_, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&staged_, cudaEventDisableTiming);
  if (e != cudaSuccess) return fail_cuda(e, "cudaEventCreate(batch)");
  return kOk;
}

BatchExecutor::~BatchExecutor() {
  // Graphs and buffers belong to the CUDA context, which is torn down at exit.
  if (staged_) cudaEventSynchronize(staged_);
  for (auto& kv : graphs_) cudaGraphExecDestroy(kv.second.exec);
  if (d_lists_) cudaFree(d_lists_);
  if (h_lists_) cudaFreeHost(h_lists_);
  if (d_scratch_) cudaFree(d_scratch_);
  if (d_queue_ctl_) cudaFree(d_queue_ctl_);
  for (int i = 0; i < kDegrees; ++i) {
    if (side_[i]) cudaStreamDestroy(side_[i]);
    if (join_[i]) cudaEventDestroy(join_[i]);
  }
  if (fork_) cudaEventDestroy(fork_);
  if (staged_) cudaEventDestroy(staged_);
}

void BatchExecutor::drop_graphs() {
  for (auto& kv : graphs_) cudaGraphExecDestroy(kv.second.exec);
  graphs_.clear();
  ++generation_;
}

int BatchExecutor::reserve_lists(size_t bytes) {
  if (bytes <= lists_bytes_) return kOk;
  cudaEventSynchronize(staged_);  // the previous upload must have drained
  drop_graphs();
  if (d_lists_) cudaFree(d_lists_);
  if (h_lists_) cudaFreeHost(h_lists_);
  d_lists_ = nullptr;
  h_lists_ = nullptr;
  lists_bytes_ = 0;
  const size_t want = std::max<size_t>(bytes, 1 << 16) * 2;
  cudaError_t e = lib_malloc(&d_lists_, want);
  if (e != cudaSuccess) return fail_cuda(e, "cudaMalloc(batch lists)");
  e = lib_malloc_host(&h_lists_, want);
  if (e != cudaSuccess) return fail_cuda(e, "cudaMallocHost(batch lists)");
  lists_bytes_ = want;
  return kOk;
}

int BatchExecutor::reserve_scratch(size_t words) {
  if (words <= scratch_words_) return kOk;
  drop_graphs();
  if (d_scratch_) cudaFree(d_scratch_);
  d_scratch_ = nullptr;
  scratch_words_ = 0;
  cudaError_t e = lib_malloc(&d_scratch_, words * sizeof(uint64_t));
  if (e != cudaSuccess) return fail_cuda(e, "cudaMalloc(batch scratch)");
  scratch_words_ = words;
  return kOk;
}

int BatchExecutor::reserve_limbs(size_t limbs) {
  const int st = reserve_lists(limbs * (4 * 8 + 4) + kDegrees * 16);
  return st != kOk ? st : reserve_scratch(2);
}

cudaError_t BatchExecutor::launch_buckets(const std::vector<Bucket>& buckets, cudaStream_t s,
                                          bool scratch_lists, bool fork) {
  PlainLaunches plain;  // buckets run side by side
  fork = fork && buckets.size() > 1;
  cudaError_t le = fork ? cudaEventRecord(fork_, s) : cudaSuccess;
  for (size_t i = 0; i < buckets.size() && le == cudaSuccess; ++i) {
    const Bucket& b = buckets[i];
    const int k = (int)(b.log_n - kMinLogN);
    cudaStream_t side = fork ? side_[k] : s;
    if (fork) le = cudaStreamWaitEvent(side, fork_, 0);
    if (le != cudaSuccess) break;
    LimbSet c;
    c.base = nullptr;
    c.ptrs = reinterpret_cast<uint64_t* const*>(d_lists_ + b.c_off);
    c.cms = reinterpret_cast<const uint32_t*>(d_lists_ + b.cm_off);
    c.count = b.limbs;
    c.L = 1;
    c.cm0 = 0;
    c.pad_ = 0;
    ConstLimbSet a{nullptr, reinterpret_cast<const uint64_t* const*>(d_lists_ + b.a_off), c.cms,
                   b.limbs, 1, 0, 0};
    ConstLimbSet bb{nullptr, reinterpret_cast<const uint64_t* const*>(d_lists_ + b.b_off), c.cms,
                    b.limbs, 1, 0, 0};
    uint64_t* const* sptrs =
        scratch_lists ? reinterpret_cast<uint64_t* const*>(d_lists_ + b.s_off) : nullptr;
    le = launch_polymul(c, a, bb, b.log_n, b.mods, d_scratch_ + b.scratch_off, NttShape{}, side, sptrs);
    if (fork && le == cudaSuccess) le = cudaEventRecord(join_[k], side);
    if (fork && le == cudaSuccess) le = cudaStreamWaitEvent(s, join_[k], 0);
  }
  return le;
}

int BatchExecutor::run(DeviceContext* ctx, const yell_polymul_desc* descs, uint64_t* const* desc_scratch,
                       uint32_t n, cudaStream_t s, bool use_graph, bool fork) {
  TraceRange trace("yell batch");
  // ---- buckets and their list layout -----------------------------------
  std::array<std::vector<uint32_t>, kDegrees> members;
  for (uint32_t i = 0; i < n; ++i) members[descs[i].log_n - kMinLogN].push_back(i);
  std::vector<Bucket> buckets;
  size_t bytes = 0, scratch = 0;
  for (int k = 0; k < kDegrees; ++k) {
    if (members[k].empty()) continue;
    Bucket b;
    b.log_n = kMinLogN + k;
    for (uint32_t i : members[k]) b.limbs += descs[i].L;
    b.mods = ctx->mods_if_ready(b.log_n);
    if (!b.mods) return fail(kInvalidArgument, "batch: twiddle tables not built");
    b.c_off = bytes;
    bytes += 8 * (size_t)b.limbs;
    b.a_off = bytes;
    bytes += 8 * (size_t)b.limbs;
    b.b_off = bytes;
    bytes += 8 * (size_t)b.limbs;
    b.s_off = bytes;
    bytes += 8 * (size_t)b.limbs;
    b.cm_off = bytes;
    bytes += ((4 * (size_t)b.limbs + 15) / 16) * 16;
    b.scratch_off = scratch;
    if (!desc_scratch) scratch += polymul_scratch_words(b.limbs, b.log_n, NttShape{});
    buckets.push_back(b);
  }
  int st = reserve_lists(bytes);
  if (st != kOk) return st;
  st = reserve_scratch(std::max<size_t>(scratch, 2));
  if (st != kOk) return st;

  // ---- fill the pinned staging after the previous upload has drained ----
  cudaError_t e = cudaEventSynchronize(staged_);
  if (e != cudaSuccess) return fail_cuda(e, "batch staging wait");
  for (const Bucket& b : buckets) {
    uint64_t* c = reinterpret_cast<uint64_t*>(h_lists_ + b.c_off);
    uint64_t* a = reinterpret_cast<uint64_t*>(h_lists_ + b.a_off);
    uint64_t* bb = reinterpret_cast<uint64_t*>(h_lists_ + b.b_off);
    uint64_t* sc = reinterpret_cast<uint64_t*>(h_lists_ + b.s_off);
    uint32_t* cm = reinterpret_cast<uint32_t*>(h_lists_ + b.cm_off);
    size_t k = 0;
    const size_t nw = (size_t)1 << b.log_n;
    for (uint32_t i : members[b.log_n - kMinLogN]) {
      const yell_polymul_desc& d = descs[i];
      for (uint32_t l = 0; l < d.L; ++l, ++k) {
        c[k] = reinterpret_cast<uint64_t>(d.c + l * nw);
        a[k] = reinterpret_cast<uint64_t>(d.a + l * nw);
        bb[k] = reinterpret_cast<uint64_t>(d.b + l * nw);
        sc[k] = desc_scratch && desc_scratch[i] ? reinterpret_cast<uint64_t>(desc_scratch[i] + l * nw) : 0;
        cm[k] = d.cm0 + l;
      }
    }
  }
  e = cudaMemcpyAsync(d_lists_, h_lists_, bytes, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaEventRecord(staged_, s);
  if (e != cudaSuccess) return fail_cuda(e, "batch list upload");

  const bool scratch_lists = desc_scratch != nullptr;
  if (!use_graph) {
    const uint64_t l0 = g_kernel_launches.load();
    e = launch_buckets(buckets, s, scratch_lists, fork);
    last_launches_ = g_kernel_launches.load() - l0;
    if (e != cudaSuccess) return fail_cuda(e, "batch launch");
    return kOk;
  }
  std::string sig = std::to_string(generation_) + (scratch_lists ? "s" : "o") + (fork ? "f" : "q");
  for (const Bucket& b : buckets) sig += ";" + std::to_string(b.log_n) + ":" + std::to_string(b.limbs);
  auto it = graphs_.find(sig);
  if (it == graphs_.end()) {
    const uint64_t launches0 = g_kernel_launches.load();
    e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return fail_cuda(e, "batch capture begin");
    const cudaError_t le = launch_buckets(buckets, s, scratch_lists, fork);
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
    if (graphs_.size() >= 64) drop_graphs();
    it = graphs_.emplace(sig, cg).first;
  }
  e = cudaGraphLaunch(it->second.exec, s);
  if (e != cudaSuccess) return fail_cuda(e, "batch graph launch");
  g_kernel_launches += it->second.launches;
  last_launches_ = it->second.launches;
  return kOk;
}

int BatchExecutor::reserve_queue_ctl(size_t words) {
  if (words <= queue_ctl_words_) return kOk;
  // keep the sticky status word across the regrowth
  uint32_t status = 0;
  if (d_queue_ctl_) {
    cudaError_t e = cudaMemcpy(&status, d_queue_ctl_, 4, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return fail_cuda(e, "queue status");
    cudaFree(d_queue_ctl_);
    d_queue_ctl_ = nullptr;
    queue_ctl_words_ = 0;
  }
  const size_t want = std::max<size_t>(words, 4096) * 2;
  cudaError_t e = lib_malloc(&d_queue_ctl_, want * sizeof(uint32_t));
  if (e == cudaSuccess) e = cudaMemset(d_queue_ctl_, 0, want * sizeof(uint32_t));
  if (e == cudaSuccess) e = cudaMemcpy(d_queue_ctl_, &status, 4, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return fail_cuda(e, "cudaMalloc(queue control)");
  queue_ctl_words_ = want;
  return kOk;
}

int BatchExecutor::run_queue(DeviceContext* ctx, const yell_polymul_desc* descs, uint32_t n, cudaStream_t s,
                             uint64_t timeout_ns, bool phased) {
  TraceRange trace(phased ? "yell batch phases" : "yell batch queue");
  if (!phased && !queue_attrs_) {
    const cudaError_t e = queue_set_attributes();
    if (e != cudaSuccess) return fail_cuda(e, "queue kernel attributes");
    queue_attrs_ = true;
  }
  if (phased && !phase_attrs_) {
    const cudaError_t e = phases_set_attributes();
    if (e != cudaSuccess) return fail_cuda(e, "phase kernel attributes");
    phase_attrs_ = true;
  }
  // ---- buckets: limb lists, scratch for the two-pass degrees -------------
  std::array<std::vector<uint32_t>, kDegrees> members;
  for (uint32_t i = 0; i < n; ++i) members[descs[i].log_n - kMinLogN].push_back(i);
  std::vector<Bucket> buckets;
  std::vector<uint32_t> counter_off;
  size_t bytes = 0, scratch = 0, counters = 0;
  for (int k = 0; k < kDegrees; ++k) {
    if (members[k].empty()) continue;
    Bucket b;
    b.log_n = kMinLogN + k;
    for (uint32_t i : members[k]) b.limbs += descs[i].L;
    b.mods = ctx->mods_if_ready(b.log_n);
    if (!b.mods) return fail(kInvalidArgument, "batch: twiddle tables not built");
    b.c_off = bytes;
    bytes += 8 * (size_t)b.limbs;
    b.a_off = bytes;
    bytes += 8 * (size_t)b.limbs;
    b.b_off = bytes;
    bytes += 8 * (size_t)b.limbs;
    b.s_off = bytes;
    bytes += 8 * (size_t)b.limbs;
    b.cm_off = bytes;
    bytes += ((4 * (size_t)b.limbs + 15) / 16) * 16;
    b.scratch_off = scratch;
    counter_off.push_back((uint32_t)counters);
    if (b.log_n >= kQueueFirstTwoPass) {
      scratch += (size_t)b.limbs << b.log_n;
      counters += 2 * (size_t)b.limbs;
    }
    buckets.push_back(b);
  }
  if (buckets.size() > kQueueMaxBuckets) return fail(kInvalidArgument, "batch: too many buckets");
  // ---- queue: forward column passes, whole-limb tiles, row steps, inverse
  // column passes.  All resident CTAs run the same kind of item most of the
  // time, so the SMs' instruction caches hold one body at a time.
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device());
  const uint32_t resident = (uint32_t)std::max(sms, 1) * 2;
  std::vector<QueueItem> items;
  uint32_t phase_items[4] = {0, 0, 0, 0};
  for (int phase = 0; phase < 4; ++phase)
    for (size_t bi = 0; bi < buckets.size(); ++bi) {
      const Bucket& b = buckets[bi];
      const bool two_pass = b.log_n >= kQueueFirstTwoPass;
      if (two_pass == (phase == 1)) continue;  // phase 1 holds the whole-limb tiles only
      uint32_t kind, tiles;
      if (two_pass) {
        kind = phase == 0 ? kItemColFwd : (phase == 2 ? kItemRows : kItemColInv);
        tiles = b.limbs << (b.log_n - kQueueTileLog);
      } else {
        kind = kItemWhole;
        const uint32_t t = b.log_n >= 4 ? kQueueTileLog : kQueueTileLog - 1;
        const uint32_t per = 1u << (t - b.log_n);
        tiles = (b.limbs + per - 1) / per;
      }
      for (uint32_t t = 0; t < tiles; ++t) items.push_back(QueueItem{(uint32_t)bi << 8 | kind, t});
      phase_items[phase] += tiles;
    }
  const size_t buckets_off = (bytes + 15) / 16 * 16;
  bytes = buckets_off + buckets.size() * sizeof(QueueBucket);
  const size_t items_off = (bytes + 15) / 16 * 16;
  bytes = items_off + items.size() * sizeof(QueueItem);
  int st = reserve_lists(bytes);
  if (st == kOk) st = reserve_scratch(std::max<size_t>(scratch, 2));
  if (st == kOk) st = reserve_queue_ctl(2 + std::max<size_t>(counters, 1));
  if (st != kOk) return st;

  // ---- host staging after the previous upload has drained -------------------
  cudaError_t e = cudaEventSynchronize(staged_);
  if (e != cudaSuccess) return fail_cuda(e, "batch staging wait");
  QueueBucket* qb = reinterpret_cast<QueueBucket*>(h_lists_ + buckets_off);
  for (size_t bi = 0; bi < buckets.size(); ++bi) {
    const Bucket& b = buckets[bi];
    uint64_t* c = reinterpret_cast<uint64_t*>(h_lists_ + b.c_off);
    uint64_t* a = reinterpret_cast<uint64_t*>(h_lists_ + b.a_off);
    uint64_t* bb = reinterpret_cast<uint64_t*>(h_lists_ + b.b_off);
    uint64_t* sc = reinterpret_cast<uint64_t*>(h_lists_ + b.s_off);
    uint32_t* cm = reinterpret_cast<uint32_t*>(h_lists_ + b.cm_off);
    const size_t nw = (size_t)1 << b.log_n;
    size_t k = 0;
    for (uint32_t i : members[b.log_n - kMinLogN]) {
      const yell_polymul_desc& d = descs[i];
      for (uint32_t l = 0; l < d.L; ++l, ++k) {
        c[k] = reinterpret_cast<uint64_t>(d.c + l * nw);
        a[k] = reinterpret_cast<uint64_t>(d.a + l * nw);
        bb[k] = reinterpret_cast<uint64_t>(d.b + l * nw);
        sc[k] = reinterpret_cast<uint64_t>(d_scratch_ + b.scratch_off + k * nw);
        cm[k] = d.cm0 + l;
      }
    }
    QueueBucket q;
    const uint32_t* cms = reinterpret_cast<const uint32_t*>(d_lists_ + b.cm_off);
    q.c = LimbSet{nullptr, reinterpret_cast<uint64_t* const*>(d_lists_ + b.c_off), cms, b.limbs, 1, 0, 0};
    q.a = ConstLimbSet{nullptr, reinterpret_cast<const uint64_t* const*>(d_lists_ + b.a_off), cms, b.limbs, 1, 0, 0};
    q.b = ConstLimbSet{nullptr, reinterpret_cast<const uint64_t* const*>(d_lists_ + b.b_off), cms, b.limbs, 1, 0, 0};
    q.s = LimbSet{nullptr, reinterpret_cast<uint64_t* const*>(d_lists_ + b.s_off), cms, b.limbs, 1, 0, 0};
    q.mods = b.mods + kPolymulConsts;  // the fused polymul's copy of the constants
    q.log_n = b.log_n;
    q.counter_off = counter_off[bi];
    qb[bi] = q;
  }
  std::memcpy(h_lists_ + items_off, items.data(), items.size() * sizeof(QueueItem));
  e = cudaMemcpyAsync(d_lists_, h_lists_, bytes, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaEventRecord(staged_, s);
  // ticket counter and limb counters start at zero; the status word (index 0) is sticky
  if (e == cudaSuccess && !phased) e = cudaMemsetAsync(d_queue_ctl_ + 1, 0, (1 + counters) * sizeof(uint32_t), s);
  if (e != cudaSuccess) return fail_cuda(e, "queue upload");

  QueueLaunch ql;
  ql.buckets = reinterpret_cast<const QueueBucket*>(d_lists_ + buckets_off);
  ql.items = reinterpret_cast<const QueueItem*>(d_lists_ + items_off);
  ql.n_items = (uint32_t)items.size();
  ql.n_buckets = (uint32_t)buckets.size();
  ql.status = d_queue_ctl_;
  ql.next = d_queue_ctl_ + 1;
  ql.done = d_queue_ctl_ + 2;
  ql.timeout_ns = timeout_ns;
  ql.grid = (uint32_t)std::min<size_t>(items.size(), resident);
  const uint64_t l0 = g_kernel_launches.load();
  if (phased) {
    // forward column passes and whole-limb tiles, row steps, inverse column passes
    const uint32_t counts[3] = {phase_items[0] + phase_items[1], phase_items[2], phase_items[3]};
    e = launch_batch_phases(qb, (uint32_t)buckets.size(), ql.items, counts, s);
  } else {
    e = launch_batch_queue(ql, s);
  }
  last_launches_ = g_kernel_launches.load() - l0;
  return e == cudaSuccess ? kOk : fail_cuda(e, phased ? "phase launch" : "queue launch");
}

int BatchExecutor::queue_status(cudaStream_t s, uint32_t* status) {
  *status = 0;
  if (!d_queue_ctl_) return kOk;
  cudaError_t e = cudaStreamSynchronize(s);
  if (e == cudaSuccess) e = cudaMemcpy(status, d_queue_ctl_, 4, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemset(d_queue_ctl_, 0, 4);
  return e == cudaSuccess ? kOk : fail_cuda(e, "queue status");
}

int BatchExecutor::queue_wait_check(DeviceContext* ctx, cudaStream_t s, uint64_t timeout_ns, uint32_t* status) {
  // one N = 2^14 limb whose column passes are never queued: its 4 row steps
  // and 4 inverse column passes each wait on a counter nothing increments
  constexpr uint32_t log_n = 14;
  const DevMod* mods;
  int st = ctx->ensure_tables(log_n, 0, 1, &mods);
  if (st != kOk) return st;
  if (!queue_attrs_) {
    const cudaError_t e = queue_set_attributes();
    if (e != cudaSuccess) return fail_cuda(e, "queue kernel attributes");
    queue_attrs_ = true;
  }
  const size_t nw = (size_t)1 << log_n;
  st = reserve_scratch(3 * nw);  // c, a = b, scratch: real buffers, the items touch them
  if (st == kOk) st = reserve_lists(4096);
  if (st == kOk) st = reserve_queue_ctl(4);
  if (st != kOk) return st;
  cudaError_t e = cudaEventSynchronize(staged_);
  if (e != cudaSuccess) return fail_cuda(e, "batch staging wait");
  uint64_t* ptrs = reinterpret_cast<uint64_t*>(h_lists_);
  ptrs[0] = reinterpret_cast<uint64_t>(d_scratch_);           // c
  ptrs[1] = reinterpret_cast<uint64_t>(d_scratch_ + nw);      // a, b
  ptrs[2] = reinterpret_cast<uint64_t>(d_scratch_ + 2 * nw);  // scratch
  reinterpret_cast<uint32_t*>(h_lists_ + 32)[0] = 0;          // cm
  QueueBucket q;
  const uint32_t* cms = reinterpret_cast<const uint32_t*>(d_lists_ + 32);
  q.c = LimbSet{nullptr, reinterpret_cast<uint64_t* const*>(d_lists_), cms, 1, 1, 0, 0};
  q.a = ConstLimbSet{nullptr, reinterpret_cast<const uint64_t* const*>(d_lists_ + 8), cms, 1, 1, 0, 0};
  q.b = q.a;
  q.s = LimbSet{nullptr, reinterpret_cast<uint64_t* const*>(d_lists_ + 16), cms, 1, 1, 0, 0};
  q.mods = mods + kPolymulConsts;
  q.log_n = log_n;
  q.counter_off = 0;
  std::memcpy(h_lists_ + 64, &q, sizeof q);
  QueueItem* items = reinterpret_cast<QueueItem*>(h_lists_ + 64 + sizeof(QueueBucket) + 16);
  const uint32_t tiles = 1u << (log_n - kQueueTileLog);
  for (uint32_t t = 0; t < tiles; ++t) {
    items[t] = QueueItem{kItemRows, t};
    items[tiles + t] = QueueItem{kItemColInv, t};
  }
  const size_t bytes = 64 + sizeof(QueueBucket) + 16 + 2 * tiles * sizeof(QueueItem);
  e = cudaMemsetAsync(d_scratch_, 0, 3 * nw * sizeof(uint64_t), s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(d_lists_, h_lists_, bytes, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaEventRecord(staged_, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(d_queue_ctl_ + 1, 0, 3 * sizeof(uint32_t), s);
  if (e != cudaSuccess) return fail_cuda(e, "queue check upload");
  QueueLaunch ql;
  ql.buckets = reinterpret_cast<const QueueBucket*>(d_lists_ + 64);
  ql.items = reinterpret_cast<const QueueItem*>(d_lists_ + 64 + sizeof(QueueBucket) + 16);
  ql.n_items = 2 * tiles;
  ql.n_buckets = 1;
  ql.status = d_queue_ctl_;
  ql.next = d_queue_ctl_ + 1;
  ql.done = d_queue_ctl_ + 2;
  ql.timeout_ns = timeout_ns;
  ql.grid = 2;
  e = launch_batch_queue(ql, s);
  if (e != cudaSuccess) return fail_cuda(e, "queue check launch");
  return queue_status(s, status);
}

}  // namespace yell_gb300

using namespace yell_gb300;

namespace {

// Bound of each dependency wait in the persistent batch kernel.
constexpr uint64_t kQueueWaitNs = 2'000'000'000ull;

int validate(const yell_polymul_desc& d) {
  if (!d.c || !d.a || !d.b) return fail(kInvalidArgument, "null pointer in a batch entry");
  if (d.c == d.a || d.c == d.b) return fail(kInvalidArgument, "batch entry output aliases an operand");
  const uintptr_t m = reinterpret_cast<uintptr_t>(d.c) | reinterpret_cast<uintptr_t>(d.a) |
                      reinterpret_cast<uintptr_t>(d.b);
  if (m % 16) return fail(kInvalidArgument, "batch entry pointers must be 16-byte aligned");
  const int st = check_degree(d.log_n);
  if (st != kOk) return st;
  return check_moduli(d.cm0, d.L);
}

// Every entry valid, and the limbs of each degree (one bucket, one launch
// sequence) within what one launch covers.
int validate_batch(const yell_polymul_desc* descs, uint32_t n) {
  uint64_t limbs[kMaxLogN + 1] = {};
  for (uint32_t i = 0; i < n; ++i) {
    const int st = validate(descs[i]);
    if (st != kOk) return st;
    limbs[descs[i].log_n] += descs[i].L;
  }
  for (uint32_t k = kMinLogN; k <= kMaxLogN; ++k) {
    if (!limbs[k]) continue;
    const int st = check_limbs(limbs[k], 1, k, nullptr);
    if (st != kOk) return st;
  }
  return kOk;
}

struct DeviceBatch {
  std::mutex mu;
  BatchExecutor exec;
  cudaEvent_t user_ev = nullptr, done_ev = nullptr;
};

DeviceBatch* device_batch(int dev, int* st) {
  static std::mutex mu;
  static std::array<std::unique_ptr<DeviceBatch>, 64> states;
  std::lock_guard<std::mutex> g(mu);
  if (!states[dev]) {
    std::unique_ptr<DeviceBatch> b(new DeviceBatch());
    *st = b->exec.init();
    if (*st != kOk) return nullptr;
    cudaError_t e = cudaEventCreateWithFlags(&b->user_ev, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->done_ev, cudaEventDisableTiming);
    if (e != cudaSuccess) {
      *st = fail_cuda(e, "cudaEventCreate(batch)");
      return nullptr;
    }
    states[dev] = std::move(b);
  }
  *st = kOk;
  return states[dev].get();
}

}  // namespace

extern "C" int yell_dev_polymul_batch(const yell_polymul_desc* descs, uint32_t n, void* stream) {
  if (!descs || n == 0) return fail(kInvalidArgument, "empty batch");
  int st = validate_batch(descs, n);
  if (st != kOk) return st;
  DeviceContext* ctx = DeviceContext::current(&st);
  if (!ctx) return st;
  // tables first (this may allocate and synchronise)
  for (uint32_t i = 0; i < n; ++i) {
    const DevMod* mods;
    st = ctx->ensure_tables(descs[i].log_n, descs[i].cm0, descs[i].L, &mods);
    if (st != kOk) return st;
  }
  DeviceBatch* db = device_batch(ctx->device(), &st);
  if (!db) return st;
  std::lock_guard<std::mutex> g(db->mu);
  cudaStream_t s = ctx->stream();
  cudaError_t e;
  if (stream) {
    e = cudaEventRecord(db->user_ev, static_cast<cudaStream_t>(stream));
    if (e == cudaSuccess) e = cudaStreamWaitEvent(s, db->user_ev, 0);
    if (e != cudaSuccess) return fail_cuda(e, "batch stream ordering");
  }
  st = db->exec.run(ctx, descs, nullptr, n, s, true);
  if (st != kOk) return st;
  if (stream) {
    e = cudaEventRecord(db->done_ev, s);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(static_cast<cudaStream_t>(stream), db->done_ev, 0);
    if (e != cudaSuccess) return fail_cuda(e, "batch stream ordering");
  }
  return kOk;
}

namespace {

int batch_queue_entry(const yell_polymul_desc* descs, uint32_t n, void* stream, bool phased) {
  if (!descs || n == 0) return fail(kInvalidArgument, "empty batch");
  int st = validate_batch(descs, n);
  if (st != kOk) return st;
  DeviceContext* ctx = DeviceContext::current(&st);
  if (!ctx) return st;
  for (uint32_t i = 0; i < n; ++i) {
    const DevMod* mods;
    st = ctx->ensure_tables(descs[i].log_n, descs[i].cm0, descs[i].L, &mods);
    if (st != kOk) return st;
  }
  DeviceBatch* db = device_batch(ctx->device(), &st);
  if (!db) return st;
  std::lock_guard<std::mutex> g(db->mu);
  cudaStream_t s = ctx->stream();
  cudaError_t e;
  if (stream) {
    e = cudaEventRecord(db->user_ev, static_cast<cudaStream_t>(stream));
    if (e == cudaSuccess) e = cudaStreamWaitEvent(s, db->user_ev, 0);
    if (e != cudaSuccess) return fail_cuda(e, "batch stream ordering");
  }
  st = db->exec.run_queue(ctx, descs, n, s, kQueueWaitNs, phased);
  if (st != kOk) return st;
  if (stream) {
    e = cudaEventRecord(db->done_ev, s);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(static_cast<cudaStream_t>(stream), db->done_ev, 0);
    if (e != cudaSuccess) return fail_cuda(e, "batch stream ordering");
  }
  return kOk;
}

}  // namespace

extern "C" int yell_dev_polymul_batch_queue(const yell_polymul_desc* descs, uint32_t n, void* stream) {
  return batch_queue_entry(descs, n, stream, false);
}

extern "C" int yell_dev_polymul_batch_phased(const yell_polymul_desc* descs, uint32_t n, void* stream) {
  return batch_queue_entry(descs, n, stream, true);
}

extern "C" int yell_batch_queue_status(uint32_t* status) {
  if (!status) return fail(kInvalidArgument, "null output");
  int st = kOk;
  DeviceContext* ctx = DeviceContext::current(&st);
  if (!ctx) return st;
  DeviceBatch* db = device_batch(ctx->device(), &st);
  if (!db) return st;
  std::lock_guard<std::mutex> g(db->mu);
  return db->exec.queue_status(ctx->stream(), status);
}

extern "C" int yell_batch_queue_wait_check(uint64_t timeout_ns, uint32_t* status) {
  if (!status) return fail(kInvalidArgument, "null output");
  if (timeout_ns == 0 || timeout_ns > 10'000'000'000ull) return fail(kInvalidArgument, "timeout must be in (0, 10 s]");
  int st = kOk;
  DeviceContext* ctx = DeviceContext::current(&st);
  if (!ctx) return st;
  DeviceBatch* db = device_batch(ctx->device(), &st);
  if (!db) return st;
  std::lock_guard<std::mutex> g(db->mu);
  return db->exec.queue_wait_check(ctx, ctx->stream(), timeout_ns, status);
}
