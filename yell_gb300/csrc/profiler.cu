#include "profiler.h"

#include <map>
#include <mutex>

namespace yell_gb300 {

std::atomic<bool> g_profiling{false};

namespace {
std::mutex g_mu;
std::vector<ProfileRecord> g_records;
std::vector<cudaEvent_t> g_pool;
size_t g_pool_next = 0;
struct Total {
  uint64_t launches = 0;
  double ms = 0.0;
};
std::vector<std::pair<std::string, Total>> g_totals;
}  // namespace

cudaEvent_t profile_event() {
  std::lock_guard<std::mutex> g(g_mu);
  if (g_pool_next == g_pool.size()) {
    cudaEvent_t e;
    if (cudaEventCreate(&e) != cudaSuccess) return nullptr;
    g_pool.push_back(e);
  }
  return g_pool[g_pool_next++];
}

void profile_push(const char* name, cudaEvent_t start, cudaEvent_t stop) {
  std::lock_guard<std::mutex> g(g_mu);
  g_records.push_back({name, start, stop});
}

int profile_start() {
  std::lock_guard<std::mutex> g(g_mu);
  g_records.clear();
  g_totals.clear();
  g_pool_next = 0;
  g_profiling.store(true);
  return 0;
}

int profile_stop() {
  g_profiling.store(false);
  std::lock_guard<std::mutex> g(g_mu);
  std::map<std::string, Total> acc;
  std::vector<std::string> order;
  for (const ProfileRecord& r : g_records) {
    if (cudaEventSynchronize(r.stop) != cudaSuccess) return -1;
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, r.start, r.stop) != cudaSuccess) return -1;
    if (!acc.count(r.name)) order.push_back(r.name);
    Total& t = acc[r.name];
    t.launches += 1;
    t.ms += ms;
  }
  g_totals.clear();
  for (const std::string& n : order) g_totals.push_back({n, acc[n]});
  g_records.clear();
  return 0;
}

int profile_count() {
  std::lock_guard<std::mutex> g(g_mu);
  return (int)g_totals.size();
}

int profile_get(int i, std::string* name, uint64_t* launches, double* total_ms) {
  std::lock_guard<std::mutex> g(g_mu);
  if (i < 0 || i >= (int)g_totals.size()) return -1;
  *name = g_totals[i].first;
  *launches = g_totals[i].second.launches;
  *total_ms = g_totals[i].second.ms;
  return 0;
}

}  // namespace yell_gb300
