// Autotuner: times every launch variant of a degree (same butterflies, other
// work splits) on the current device and keeps the fastest.  Choices can be
// persisted to a small text file named by YELL_GB300_TUNE_FILE, one line per
// choice: "<device name>|<log_n>|<variant name>".
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <mutex>
#include <sstream>
#include <string>
#include <vector>

#include "kernels.h"
#include "ntt_variants.h"
#include "runtime.h"
#include "yell_gb300.h"

using namespace yell_gb300;

namespace {

std::mutex g_file_mu;

std::string device_name(int dev) {
  cudaDeviceProp prop;
  if (cudaGetDeviceProperties(&prop, dev) != cudaSuccess) return "unknown";
  return prop.name;
}

void persist(int dev, uint32_t log_n, const std::string& vname) {
  const char* path = std::getenv("YELL_GB300_TUNE_FILE");
  if (!path || !*path) return;
  std::lock_guard<std::mutex> g(g_file_mu);
  const std::string key = device_name(dev) + "|" + std::to_string(log_n) + "|";
  std::vector<std::string> lines;
  {
    std::ifstream in(path);
    std::string line;
    while (std::getline(in, line))
      if (line.compare(0, key.size(), key) != 0) lines.push_back(line);
  }
  lines.push_back(key + vname);
  std::ofstream out(path, std::ios::trunc);
  for (const std::string& l : lines) out << l << "\n";
}

}  // namespace

namespace yell_gb300 {

// Applies the persisted choices of this device (called once per context).
void load_tuning(int dev) {
  const char* path = std::getenv("YELL_GB300_TUNE_FILE");
  if (!path || !*path) return;
  std::lock_guard<std::mutex> g(g_file_mu);
  std::ifstream in(path);
  const std::string prefix = device_name(dev) + "|";
  std::string line;
  while (std::getline(in, line)) {
    if (line.compare(0, prefix.size(), prefix) != 0) continue;
    std::istringstream ss(line.substr(prefix.size()));
    std::string deg, vname;
    if (!std::getline(ss, deg, '|') || !std::getline(ss, vname)) continue;
    const uint32_t log_n = (uint32_t)std::atoi(deg.c_str());
    if (log_n < kMinLogN || log_n > kMaxLogN) continue;
    const std::vector<Variant>& vs = variants_of(log_n);
    for (uint32_t v = 0; v < vs.size(); ++v)
      if (vname == vs[v].name) select_variant(dev, log_n, v);
  }
}

}  // namespace yell_gb300

extern "C" {

int yell_variant_count(uint32_t log_n, uint32_t* count) {
  if (!count) return fail(kInvalidArgument, "null output");
  const int st = check_degree(log_n);
  if (st != kOk) return st;
  *count = (uint32_t)variants_of(log_n).size();
  return kOk;
}

int yell_variant_name(uint32_t log_n, uint32_t variant, char* buf, size_t len) {
  if (!buf || len == 0) return fail(kInvalidArgument, "null output");
  const int st = check_degree(log_n);
  if (st != kOk) return st;
  const std::vector<Variant>& vs = variants_of(log_n);
  if (variant >= vs.size()) return fail(kInvalidArgument, "no such variant");
  std::snprintf(buf, len, "%s", vs[variant].name);
  return kOk;
}

int yell_set_variant(uint32_t log_n, uint32_t variant) {
  int st = check_degree(log_n);
  if (st != kOk) return st;
  if (variant >= variants_of(log_n).size()) return fail(kInvalidArgument, "no such variant");
  DeviceContext* ctx = DeviceContext::current(&st);
  if (!ctx) return st;
  select_variant(ctx->device(), log_n, variant);
  return kOk;
}

int yell_get_variant(uint32_t log_n, uint32_t* variant) {
  if (!variant) return fail(kInvalidArgument, "null output");
  int st = check_degree(log_n);
  if (st != kOk) return st;
  DeviceContext* ctx = DeviceContext::current(&st);
  if (!ctx) return st;
  *variant = selected_variant(ctx->device(), log_n);
  return kOk;
}

int yell_autotune(uint32_t log_n, uint32_t L, uint32_t pairs, uint32_t* best, double* best_ms) {
  int st = check_degree(log_n);
  if (st != kOk) return st;
  st = check_moduli(0, L);
  if (st != kOk) return st;
  if (pairs == 0) return fail(kInvalidArgument, "pairs is 0");
  DeviceContext* ctx = DeviceContext::current(&st);
  if (!ctx) return st;
  const DevMod* mods;
  st = ctx->ensure_tables(log_n, 0, L, &mods);
  if (st != kOk) return st;
  const size_t count = (size_t)pairs * L;
  const size_t words = count << log_n;
  const size_t sw = polymul_scratch_words((uint32_t)count, log_n, NttShape{});
  uint64_t* buf = nullptr;
  cudaError_t e = lib_malloc(&buf, (3 * words + sw + 2) * sizeof(uint64_t));
  if (e != cudaSuccess) return fail_cuda(e, "cudaMalloc(autotune)");
  cudaStream_t s = ctx->stream();
  // Any words will do: the arithmetic is branch-free, so timing does not depend on them.
  e = cudaMemsetAsync(buf, 0x5a, 2 * words * sizeof(uint64_t), s);
  LimbSet c{buf + 2 * words, nullptr, nullptr, (uint32_t)count, L, 0, 0};
  ConstLimbSet a{buf, nullptr, nullptr, (uint32_t)count, L, 0, 0};
  ConstLimbSet b{buf + words, nullptr, nullptr, (uint32_t)count, L, 0, 0};
  uint64_t* scratch = sw ? buf + 3 * words : nullptr;
  const std::vector<Variant>& vs = variants_of(log_n);
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  uint32_t best_v = 0;
  double best_t = 1e30;
  for (uint32_t v = 0; v < vs.size() && e == cudaSuccess; ++v) {
    float t = 1e30f;
    for (int rep = 0; rep < 4 && e == cudaSuccess; ++rep) {
      e = cudaEventRecord(e0, s);
      if (e == cudaSuccess) e = vs[v].polymul(c, a, b, mods, scratch, nullptr, s);
      if (e == cudaSuccess) e = cudaEventRecord(e1, s);
      if (e == cudaSuccess) e = cudaEventSynchronize(e1);
      float ms = 0;
      if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
      if (rep > 0 && ms < t) t = ms;  // rep 0 warms up
    }
    if (t < best_t) {
      best_t = t;
      best_v = v;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(buf);
  if (e != cudaSuccess) return fail_cuda(e, "autotune run");
  select_variant(ctx->device(), log_n, best_v);
  persist(ctx->device(), log_n, vs[best_v].name);
  if (best) *best = best_v;
  if (best_ms) *best_ms = best_t;
  return kOk;
}

}  // extern "C"
