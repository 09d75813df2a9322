// Unit test of the server's HBM range allocator (host-only code).
#include <cstdio>
#include <cstdlib>
#include <vector>
#include "range_alloc.h"

#define CHECK(c) do { if (!(c)) { std::printf("FAIL %s:%d %s\n", __FILE__, __LINE__, #c); return 1; } } while (0)

int main() {
  using yell_gb300::RangeAllocator;
  RangeAllocator a(1 << 20);
  CHECK(a.capacity() == (1u << 20));
  size_t o1, o2, o3;
  CHECK(a.alloc(1000, &o1) && o1 == 0);
  CHECK(a.alloc(256, &o2) && o2 == 1024);
  CHECK(a.alloc(4096, &o3) && o3 == 1280);
  CHECK(a.in_use() == 1024 + 256 + 4096);
  a.free(o2, 256);
  size_t o4;
  CHECK(a.alloc(100, &o4) && o4 == 1024);  // first fit reuses the hole
  a.free(o4, 100);
  a.free(o1, 1000);
  a.free(o3, 4096);
  CHECK(a.in_use() == 0 && a.free_ranges() == 1 && a.largest_free() == (1u << 20));
  size_t big;
  CHECK(!a.alloc((1 << 20) + 1, &big));
  CHECK(a.alloc(1 << 20, &big) && big == 0);
  a.free(big, 1 << 20);
  // random churn keeps the books straight
  std::vector<std::pair<size_t, size_t>> live;
  std::srand(7);
  for (int i = 0; i < 20000; ++i) {
    if (!live.empty() && (std::rand() % 2)) {
      size_t k = std::rand() % live.size();
      a.free(live[k].first, live[k].second);
      live.erase(live.begin() + k);
    } else {
      size_t sz = 1 + std::rand() % 20000, off;
      if (a.alloc(sz, &off)) live.push_back({off, sz});
    }
  }
  for (auto& l : live) a.free(l.first, l.second);
  CHECK(a.in_use() == 0 && a.free_ranges() == 1);
  CHECK(a.peak() <= a.capacity());
  std::printf("OK\n");
  return 0;
}
