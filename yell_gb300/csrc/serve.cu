// Serving loop: continuous batching of polymul requests of mixed size.
//
// Requests are queued by yell_server_submit.  A scheduler thread owns
// `max_inflight` stream slots.  Whenever a slot is free it admits queued
// requests in arrival order while the HBM budget (a pre-allocated arena
// carved by a range allocator) can hold their device buffers, forms one batch
// of everything admitted, and launches it on the slot: host operands are
// copied in, the batch executor runs one launch sequence per degree bucket,
// host results are copied out, and an event marks completion.  Requests that
// arrive while other batches are on the GPU are admitted into the next free
// slot, so their work overlaps on the device with the batches in flight.
// Every host wait is bounded; failures are per-request status codes.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "batch.h"
#include "profiler.h"
#include "range_alloc.h"
#include "runtime.h"
#include "yell_gb300.h"

using namespace yell_gb300;

namespace {

using Clock = std::chrono::steady_clock;

double us_between(Clock::time_point a, Clock::time_point b) {
  return std::chrono::duration<double, std::micro>(b - a).count();
}

struct Request {
  uint64_t id = 0;
  yell_polymul_request req{};
  size_t words = 0;       // L * N
  size_t footprint = 0;   // device bytes held while admitted
  size_t off = 0;         // arena offset of the footprint
  bool has_mem = false;
  uint64_t* d_a = nullptr;
  uint64_t* d_b = nullptr;
  uint64_t* d_c = nullptr;
  uint64_t* d_s = nullptr;
  int status = -1;  // -1 while queued or running
  bool cancelled = false;
  Clock::time_point t_submit, t_start, t_done;
};
using ReqPtr = std::shared_ptr<Request>;

struct Slot {
  cudaStream_t stream = nullptr;
  cudaEvent_t done = nullptr;
  BatchExecutor exec;
  std::vector<ReqPtr> reqs;
  bool busy = false;
};

}  // namespace

struct yell_server {
  int device = 0;
  DeviceContext* ctx = nullptr;
  yell_server_config cfg{};
  uint8_t* arena = nullptr;
  RangeAllocator pool;
  std::vector<std::unique_ptr<Slot>> slots;

  std::mutex mu;
  std::condition_variable cv_sched;  // wakes the scheduler
  std::condition_variable cv_done;   // wakes waiters
  std::deque<ReqPtr> pending;
  std::unordered_map<uint64_t, ReqPtr> requests;
  uint64_t next_id = 1;
  bool stop = false;
  bool paused = false;
  uint32_t inject_failures = 0;
  std::thread thread;

  // statistics since the last reset
  std::vector<double> latencies;
  uint64_t submitted = 0, completed = 0, rejected = 0, cancelled = 0, failed = 0, batches = 0;
  double limb_ntts = 0;
  Clock::time_point window_start = Clock::now();
  Clock::time_point last_done = Clock::now();

  int init(const yell_server_config* c);
  void loop();
  void finish(Slot& s);
  bool admit(std::vector<ReqPtr>* batch);
  int launch(Slot& s, std::vector<ReqPtr>& batch);
  void complete(const ReqPtr& r, int status, Clock::time_point t);
  void shutdown();
};

namespace {

bool is_ntt(const yell_polymul_request& r) { return r.flags & (YELL_REQ_NTT_FORWARD | YELL_REQ_NTT_BACKWARD); }

size_t footprint_of(const yell_polymul_request& r, size_t words, uint32_t log_n) {
  size_t bytes = 0;
  const size_t limb_bytes = words * sizeof(uint64_t);
  const bool device = r.flags & YELL_REQ_DEVICE;
  if (is_ntt(r)) {  // the transform runs in place in the output buffer
    if (!device || (r.flags & YELL_REQ_DISCARD_OUTPUT)) bytes += RangeAllocator::round(limb_bytes);
    return bytes;
  }
  if (!device) bytes += 2 * RangeAllocator::round(limb_bytes);  // a, b
  if (!device || (r.flags & YELL_REQ_DISCARD_OUTPUT)) bytes += RangeAllocator::round(limb_bytes);  // c
  if (polymul_scratch_words(1, log_n, NttShape{})) bytes += RangeAllocator::round(limb_bytes);  // two-pass scratch
  return bytes;
}

struct DeviceGuard {
  int prev = -1;
  explicit DeviceGuard(int dev) {
    if (cudaGetDevice(&prev) == cudaSuccess && prev != dev) cudaSetDevice(dev);
    else prev = -1;
  }
  ~DeviceGuard() {
    if (prev >= 0) cudaSetDevice(prev);
  }
};

}  // namespace

int yell_server::init(const yell_server_config* c) {
  cfg = *c;
  if (cfg.max_inflight == 0) cfg.max_inflight = 4;
  if (cfg.max_batch == 0) cfg.max_batch = 1024;
  inject_failures = cfg.inject_alloc_failures;
  int st = kOk;
  cudaError_t e = cudaGetDevice(&device);
  if (e != cudaSuccess) return fail_cuda(e, "cudaGetDevice");
  ctx = DeviceContext::current(&st);
  if (!ctx) return st;
  size_t free_b = 0, total_b = 0;
  e = cudaMemGetInfo(&free_b, &total_b);
  if (e != cudaSuccess) return fail_cuda(e, "cudaMemGetInfo");
  size_t budget = cfg.hbm_budget_bytes ? cfg.hbm_budget_bytes : (size_t)120 << 30;
  const size_t margin = (size_t)4 << 30;
  if (budget + margin > free_b) {
    if (cfg.hbm_budget_bytes) return fail(kOutOfMemory, "HBM budget exceeds the free device memory");
    budget = free_b > 2 * margin ? free_b - 2 * margin : free_b / 2;
  }
  e = lib_malloc(&arena, budget);
  if (e != cudaSuccess) return fail_cuda(e, "cudaMalloc(server arena)");
  pool.reset(budget);
  cfg.hbm_budget_bytes = budget;
  for (uint32_t i = 0; i < cfg.max_inflight; ++i) {
    std::unique_ptr<Slot> s(new Slot());
    e = cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&s->done, cudaEventDisableTiming);
    if (e != cudaSuccess) return fail_cuda(e, "server slot");
    st = s->exec.init();
    if (st == kOk) st = s->exec.reserve_limbs((size_t)cfg.max_batch * 64);  // no growth in steady state
    if (st != kOk) return st;
    slots.push_back(std::move(s));
  }
  thread = std::thread([this] { loop(); });
  return kOk;
}

void yell_server::complete(const ReqPtr& r, int status, Clock::time_point t) {
  // caller holds mu
  r->status = status;
  r->t_done = t;
  if (r->has_mem) {
    pool.free(r->off, r->footprint);
    r->has_mem = false;
  }
  if (status == kOk) {
    ++completed;
    latencies.push_back(us_between(r->t_submit, t));
    limb_ntts += (is_ntt(r->req) ? 1.0 : 3.0) * r->req.L;
    last_done = t;
  } else if (status == kCancelled) {
    ++cancelled;
  } else {
    ++failed;
  }
  if (r->req.flags & YELL_REQ_DISCARD_OUTPUT) requests.erase(r->id);
}

void yell_server::finish(Slot& s) {
  const Clock::time_point t = Clock::now();
  const cudaError_t e = cudaEventQuery(s.done);
  std::lock_guard<std::mutex> g(mu);
  for (const ReqPtr& r : s.reqs) complete(r, e == cudaSuccess ? kOk : kCudaError, t);
  s.reqs.clear();
  s.busy = false;
  cv_done.notify_all();
}

// Takes queued requests in arrival order while the arena can hold them.
bool yell_server::admit(std::vector<ReqPtr>* batch) {
  std::lock_guard<std::mutex> g(mu);
  const Clock::time_point t = Clock::now();
  while (!pending.empty() && batch->size() < cfg.max_batch) {
    ReqPtr r = pending.front();
    if (r->cancelled) {
      pending.pop_front();
      complete(r, kCancelled, t);
      continue;
    }
    size_t off = 0;
    if (inject_failures > 0) {  // host-side fault injection: a refused allocation
      --inject_failures;
      pending.pop_front();
      complete(r, kOutOfMemory, t);
      cv_done.notify_all();
      continue;
    }
    if (!pool.alloc(r->footprint, &off)) break;  // waits for memory to free up
    pending.pop_front();
    r->off = off;
    r->has_mem = true;
    uint8_t* p = arena + off;
    const size_t lb = RangeAllocator::round(r->words * sizeof(uint64_t));
    const bool device = r->req.flags & YELL_REQ_DEVICE;
    if (is_ntt(r->req)) {
      r->d_a = device ? const_cast<uint64_t*>(r->req.a) : nullptr;  // host input goes straight to c
      r->d_b = nullptr;
    } else if (!device) {
      r->d_a = reinterpret_cast<uint64_t*>(p);
      p += lb;
      r->d_b = reinterpret_cast<uint64_t*>(p);
      p += lb;
    } else {
      r->d_a = const_cast<uint64_t*>(r->req.a);
      r->d_b = const_cast<uint64_t*>(r->req.b);
    }
    if (!device || (r->req.flags & YELL_REQ_DISCARD_OUTPUT)) {
      r->d_c = reinterpret_cast<uint64_t*>(p);
      p += lb;
    } else {
      r->d_c = r->req.c;
    }
    r->d_s = (polymul_scratch_words(1, r->req.log_n, NttShape{}) && !is_ntt(r->req)) ? reinterpret_cast<uint64_t*>(p)
                                                                                  : nullptr;
    r->t_start = t;
    batch->push_back(r);
  }
  return !batch->empty();
}

// Host operands: pageable ones move by kernels that access them in place
// where the device can (a copy from or to pageable memory would hold the
// scheduler thread until it completes); pinned ones by the copy engines.
static cudaError_t host_in(DeviceContext* ctx, uint64_t* dev, const uint64_t* host, uint32_t limbs, uint32_t log_n,
                           cudaStream_t st) {
  if (ctx->host_access() && pageable_host(host)) return gather_host_contiguous(dev, host, limbs, log_n, st);
  return cudaMemcpyAsync(dev, host, ((size_t)limbs << log_n) * sizeof(uint64_t), cudaMemcpyHostToDevice, st);
}

static cudaError_t host_out(DeviceContext* ctx, uint64_t* host, const uint64_t* dev, uint32_t limbs, uint32_t log_n,
                            cudaStream_t st) {
  if (ctx->host_access() && pageable_host(host)) return scatter_host_contiguous(host, dev, limbs, log_n, st);
  return cudaMemcpyAsync(host, dev, ((size_t)limbs << log_n) * sizeof(uint64_t), cudaMemcpyDeviceToHost, st);
}

int yell_server::launch(Slot& s, std::vector<ReqPtr>& batch) {
  TraceRange trace("yell serve step");
  PlainLaunches plain;  // batches of other slots run beside this one
  const size_t n = batch.size();
  std::vector<yell_polymul_desc> descs;
  std::vector<uint64_t*> scratch;
  descs.reserve(n);
  scratch.reserve(n);
  cudaError_t e = cudaSuccess;
  for (size_t i = 0; i < n && e == cudaSuccess; ++i) {
    Request& r = *batch[i];
    const size_t bytes = r.words * sizeof(uint64_t);
    if (is_ntt(r.req)) {  // input into the output buffer, transformed there in place
      if (!(r.req.flags & YELL_REQ_DEVICE))
        e = host_in(ctx, r.d_c, r.req.a, r.req.L, r.req.log_n, s.stream);
      else if (r.d_c != r.d_a)
        e = cudaMemcpyAsync(r.d_c, r.d_a, bytes, cudaMemcpyDeviceToDevice, s.stream);
      continue;
    }
    if (!(r.req.flags & YELL_REQ_DEVICE)) {
      e = host_in(ctx, r.d_a, r.req.a, r.req.L, r.req.log_n, s.stream);
      if (e == cudaSuccess) e = host_in(ctx, r.d_b, r.req.b, r.req.L, r.req.log_n, s.stream);
    }
    descs.push_back(yell_polymul_desc{r.d_c, r.d_a, r.d_b, r.req.log_n, r.req.L, r.req.cm0, 0});
    scratch.push_back(r.d_s);
  }
  if (e != cudaSuccess) return fail_cuda(e, "server H2D");
  if (!descs.empty()) {
    const int st = s.exec.run(ctx, descs.data(), scratch.data(), (uint32_t)descs.size(), s.stream, false, false);
    if (st != kOk) return st;
  }
  for (size_t i = 0; i < n && e == cudaSuccess; ++i) {  // NTT requests: one launch sequence each
    Request& r = *batch[i];
    if (!is_ntt(r.req)) continue;
    const DevMod* mods = ctx->tables_ready(r.req.log_n, r.req.cm0, r.req.L);
    if (!mods) return fail(kInvalidArgument, "server: twiddle tables not built");
    LimbSet ls;
    ls.base = r.d_c;
    ls.ptrs = nullptr;
    ls.cms = nullptr;
    ls.count = r.req.L;
    ls.L = r.req.L;
    ls.cm0 = r.req.cm0;
    ls.pad_ = 0;
    e = launch_ntt(ls, r.req.log_n, mods,
                   (r.req.flags & YELL_REQ_NTT_FORWARD) ? NttDir::kForward : NttDir::kBackward, ctx->shape,
                   s.stream);
  }
  for (size_t i = 0; i < n && e == cudaSuccess; ++i) {
    Request& r = *batch[i];
    if (!(r.req.flags & YELL_REQ_DEVICE)) e = host_out(ctx, r.req.c, r.d_c, r.req.L, r.req.log_n, s.stream);
  }
  if (e == cudaSuccess) e = cudaEventRecord(s.done, s.stream);
  if (e != cudaSuccess) return fail_cuda(e, "server launch");
  return kOk;
}

void yell_server::loop() {
  cudaSetDevice(device);
  while (true) {
    bool progress = false, any_busy = false;
    for (auto& sp : slots) {
      Slot& s = *sp;
      if (s.busy && cudaEventQuery(s.done) != cudaErrorNotReady) {
        finish(s);
        progress = true;
      }
      any_busy |= s.busy;
    }
    {
      std::unique_lock<std::mutex> g(mu);
      if (stop && pending.empty() && !any_busy) break;
    }
    bool paused_now;
    {
      std::lock_guard<std::mutex> g(mu);
      paused_now = paused;
    }
    if (!paused_now) {
      for (auto& sp : slots) {
        Slot& s = *sp;
        if (s.busy) continue;
        std::vector<ReqPtr> batch;
        if (!admit(&batch)) break;
        const int st = launch(s, batch);
        if (st != kOk) {
          // the batch failed to launch: fail its requests, keep serving
          cudaStreamSynchronize(s.stream);
          std::lock_guard<std::mutex> g(mu);
          for (const ReqPtr& r : batch) complete(r, st, Clock::now());
          cv_done.notify_all();
          continue;
        }
        s.reqs = std::move(batch);
        s.busy = true;
        {
          std::lock_guard<std::mutex> g(mu);
          ++batches;
        }
        progress = true;
        any_busy = true;
      }
    }
    if (!progress) {
      if (any_busy) {
        std::this_thread::yield();  // poll the in-flight batches closely
      } else {
        std::unique_lock<std::mutex> g(mu);
        cv_sched.wait_for(g, std::chrono::milliseconds(1),
                          [this] { return stop || (!pending.empty() && !paused); });
      }
    }
  }
}

void yell_server::shutdown() {
  {
    std::lock_guard<std::mutex> g(mu);
    stop = true;
    paused = false;
  }
  cv_sched.notify_all();
  if (thread.joinable()) thread.join();
  for (auto& s : slots) {
    if (s->stream) cudaStreamSynchronize(s->stream);
  }
}

// ---------------------------------------------------------------------------

extern "C" {

int yell_server_create(const yell_server_config* cfg, yell_server** out) {
  if (!out) return fail(kInvalidArgument, "null output");
  yell_server_config def{};
  std::unique_ptr<yell_server> s(new yell_server());
  const int st = s->init(cfg ? cfg : &def);
  if (st != kOk) {
    s->shutdown();
    if (s->arena) cudaFree(s->arena);
    return st;
  }
  *out = s.release();
  return kOk;
}

int yell_server_destroy(yell_server* s) {
  if (!s) return fail(kInvalidArgument, "null server");
  s->shutdown();
  if (s->arena) cudaFree(s->arena);
  delete s;
  return kOk;
}

int yell_server_submit(yell_server* s, const yell_polymul_request* r, uint64_t* id) {
  if (!s || !r || !id) return fail(kInvalidArgument, "null argument");
  const bool ntt = is_ntt(*r);
  if ((r->flags & YELL_REQ_NTT_FORWARD) && (r->flags & YELL_REQ_NTT_BACKWARD))
    return fail(kInvalidArgument, "a request is a forward or a backward NTT, not both");
  if (!r->a || (!ntt && !r->b) || (!r->c && !(r->flags & YELL_REQ_DISCARD_OUTPUT)))
    return fail(kInvalidArgument, "null operand");
  if (!ntt && (r->flags & YELL_REQ_DEVICE) && !(r->flags & YELL_REQ_DISCARD_OUTPUT) &&
      (r->c == r->a || r->c == r->b))
    return fail(kInvalidArgument, "a device polymul's output may not overwrite an operand");
  int st = check_degree(r->log_n);
  if (st != kOk) return st;
  st = check_moduli(r->cm0, r->L);
  if (st != kOk) return st;
  if (r->flags & YELL_REQ_DEVICE) {
    const uintptr_t m = reinterpret_cast<uintptr_t>(r->a) | reinterpret_cast<uintptr_t>(r->b) |
                        reinterpret_cast<uintptr_t>(r->c);  // b may be null for an NTT
    if (m % 16) return fail(kInvalidArgument, "device operands must be 16-byte aligned");
  }
  auto req = std::make_shared<Request>();
  req->req = *r;
  req->words = (size_t)r->L << r->log_n;
  req->footprint = footprint_of(*r, req->words, r->log_n);
  if (req->footprint > s->pool.capacity()) {
    std::lock_guard<std::mutex> g(s->mu);
    ++s->rejected;
    return fail(kBudget, "request needs " + std::to_string(req->footprint) + " bytes of HBM; the budget is " +
                             std::to_string(s->pool.capacity()));
  }
  {
    DeviceGuard dg(s->device);
    const DevMod* mods;
    st = s->ctx->ensure_tables(r->log_n, r->cm0, r->L, &mods);
    if (st != kOk) return st;
  }
  {
    std::lock_guard<std::mutex> g(s->mu);
    req->id = s->next_id++;
    req->t_submit = Clock::now();
    s->requests[req->id] = req;
    s->pending.push_back(req);
    ++s->submitted;
    *id = req->id;
  }
  s->cv_sched.notify_one();
  return kOk;
}

int yell_server_wait(yell_server* s, uint64_t id, double timeout_s, yell_request_result* out) {
  if (!s) return fail(kInvalidArgument, "null server");
  std::unique_lock<std::mutex> g(s->mu);
  auto it = s->requests.find(id);
  if (it == s->requests.end()) return fail(kNotFound, "unknown request id " + std::to_string(id));
  ReqPtr r = it->second;
  const auto deadline = Clock::now() + std::chrono::duration_cast<Clock::duration>(
                                           std::chrono::duration<double>(timeout_s > 0 ? timeout_s : 0));
  while (r->status < 0) {
    if (s->cv_done.wait_until(g, deadline) == std::cv_status::timeout && r->status < 0)
      return fail(kTimeout, "request " + std::to_string(id) + " not finished within the timeout");
  }
  if (out) {
    out->status = r->status;
    out->queue_us = us_between(r->t_submit, r->t_start);
    out->latency_us = us_between(r->t_submit, r->t_done);
  }
  s->requests.erase(id);
  if (r->status != kOk) {
    return fail(r->status, r->status == kCancelled ? "request cancelled" : "request failed");
  }
  return kOk;
}

int yell_server_cancel(yell_server* s, uint64_t id) {
  if (!s) return fail(kInvalidArgument, "null server");
  std::lock_guard<std::mutex> g(s->mu);
  auto it = s->requests.find(id);
  if (it == s->requests.end()) return fail(kNotFound, "unknown request id");
  for (auto p = s->pending.begin(); p != s->pending.end(); ++p) {
    if ((*p)->id == id) {
      ReqPtr r = *p;
      s->pending.erase(p);
      s->complete(r, kCancelled, Clock::now());
      s->cv_done.notify_all();
      return kOk;
    }
  }
  return fail(kNotFound, "request already running or finished");
}

int yell_server_pause(yell_server* s, int paused) {
  if (!s) return fail(kInvalidArgument, "null server");
  {
    std::lock_guard<std::mutex> g(s->mu);
    s->paused = paused != 0;
  }
  s->cv_sched.notify_all();
  return kOk;
}

int yell_server_get_stats(yell_server* s, int reset, yell_server_stats* out) {
  if (!s || !out) return fail(kInvalidArgument, "null argument");
  std::lock_guard<std::mutex> g(s->mu);
  std::memset(out, 0, sizeof(*out));
  out->submitted = s->submitted;
  out->completed = s->completed;
  out->rejected = s->rejected;
  out->cancelled = s->cancelled;
  out->failed = s->failed;
  out->batches = s->batches;
  out->queued = s->pending.size();
  out->hbm_budget = s->pool.capacity();
  out->hbm_in_use = s->pool.in_use();
  out->hbm_peak = s->pool.peak();
  out->limb_ntts = s->limb_ntts;
  const double span = us_between(s->window_start, s->last_done) * 1e-6;
  out->window_s = span;
  out->limb_ntts_per_s = span > 0 ? s->limb_ntts / span : 0;
  out->requests_per_s = span > 0 ? s->completed / span : 0;
  std::vector<double> v = s->latencies;
  if (!v.empty()) {
    std::sort(v.begin(), v.end());
    auto pct = [&](double q) { return v[std::min(v.size() - 1, (size_t)(q * (v.size() - 1) + 0.5))]; };
    out->p50_us = pct(0.50);
    out->p99_us = pct(0.99);
    out->max_us = v.back();
    double sum = 0;
    for (double x : v) sum += x;
    out->mean_us = sum / v.size();
  }
  if (reset) {
    s->latencies.clear();
    s->submitted = s->completed = s->rejected = s->cancelled = s->failed = s->batches = 0;
    s->limb_ntts = 0;
    s->window_start = s->last_done = Clock::now();
  }
  return kOk;
}

// Poisson arrivals at offered_rps for duration_s, requests drawn round-robin
// from the templates (each submitted with YELL_REQ_DISCARD_OUTPUT), then a
// bounded drain; stats cover exactly the requests of this run.
int yell_server_load_test(yell_server* s, const yell_polymul_request* templates, uint32_t n,
                          double offered_rps, double duration_s, uint64_t seed, yell_server_stats* out) {
  if (!s || !templates || n == 0 || !out || offered_rps <= 0 || duration_s <= 0)
    return fail(kInvalidArgument, "bad load-test arguments");
  yell_server_stats scratch;
  int st = yell_server_get_stats(s, 1, &scratch);
  if (st != kOk) return st;
  {
    std::lock_guard<std::mutex> g(s->mu);
    s->window_start = s->last_done = Clock::now();
  }
  uint64_t state = seed;
  auto uniform = [&state]() {  // splitmix64 -> (0, 1]
    uint64_t z = (state += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    return ((z >> 11) + 1) * (1.0 / 9007199254740992.0);
  };
  const Clock::time_point t0 = Clock::now();
  double t_next = 0;
  uint64_t k = 0;
  while (t_next < duration_s) {
    const Clock::time_point due = t0 + std::chrono::duration_cast<Clock::duration>(std::chrono::duration<double>(t_next));
    while (Clock::now() < due) {
      if (due - Clock::now() > std::chrono::microseconds(200))
        std::this_thread::sleep_for(std::chrono::microseconds(100));
    }
    yell_polymul_request r = templates[k % n];
    r.flags |= YELL_REQ_DISCARD_OUTPUT;
    uint64_t id;
    st = yell_server_submit(s, &r, &id);
    if (st != kOk && st != kBudget) return st;
    ++k;
    t_next += -std::log(uniform()) / offered_rps;
  }
  // drain (bounded)
  const Clock::time_point limit = Clock::now() + std::chrono::seconds(120);
  while (true) {
    {
      std::lock_guard<std::mutex> g(s->mu);
      if (s->completed + s->failed + s->cancelled + s->rejected >= s->submitted) break;
    }
    if (Clock::now() > limit) return fail(kTimeout, "load test did not drain within 120 s");
    std::this_thread::sleep_for(std::chrono::microseconds(200));
  }
  return yell_server_get_stats(s, 0, out);
}

}  // extern "C"
