// Host runtime: prime table, twiddle-table registry, per-device context,
// error reporting.
#pragma once
#include <atomic>
#include <cstddef>
#include <cstdint>
#include <mutex>
#include <string>
#include <vector>
#include <cuda_runtime.h>
#include "common.cuh"
#include "kernels.h"

namespace yell_gb300 {

constexpr uint32_t kMaxModuli = 1000;       // params_64.hpp:19 kMaxNbModuli
constexpr uint32_t kLogMaxDegree = 20;      // params_64.hpp:21 kMaxPolyDegree = 2^20

struct PrimeEntry {
  uint64_t p, pn, root;
};
const PrimeEntry& prime_entry(uint32_t cm);

// Status codes (mirrors enum yell_status_code in include/yell_gb300.h).
enum Status : int {
  kOk = 0,
  kInvalidArgument = 1,
  kUnsupportedDegree = 2,
  kInvalidModulus = 3,
  kCudaError = 4,
  kOutOfMemory = 5,
  kBudget = 6,
  kTimeout = 7,
  kCancelled = 8,
  kNotFound = 9,
  kNoDevice = 10,
};

// Records a thread-local message for yell_last_error() and returns `code`.
int fail(int code, const std::string& msg);
int fail_cuda(cudaError_t e, const char* what);
const char* last_error();
void clear_error();

// Applies persisted autotuner choices for a device (YELL_GB300_TUNE_FILE).
void load_tuning(int device);

// Argument checks shared by the entry points.
int check_degree(uint32_t log_n);
int check_moduli(uint32_t cm0, uint32_t L);
// count polys (or pairs) of L limbs each: rejects a zero count and a limb
// total of one call that would not fit its launch grid (in particular any
// count * L >= 2^32).  On success *limbs = count * L (when limbs != nullptr).
int check_limbs(uint64_t count, uint32_t L, uint32_t log_n, uint32_t* limbs);

// Looks up, once per device, the device address of the fixed scratch array
// of yell_dev_polymul_noalloc (which loads the module holding it, so the
// array is in device memory from then on).  Called with that device current.
int noalloc_prepare(int device);
// The address noalloc_prepare found for `device`, or nullptr.
uint64_t* noalloc_scratch(int device);

// Builds the reference's tables for (log_n, cm) on the host
// (include/yell/details/ntt.hpp:28-77): out4n = phi, phi', invphi, invphi'
// (N words each, bit-reversed); sc4 = N^-1, (N^-1)', N^-1*invphi[1], its '.
void build_host_tables(uint32_t log_n, uint32_t cm, uint64_t* out4n, uint64_t* sc4);

// One per CUDA device, created on first use with that device current.
// Direct host-memory access by kernels, on devices that support it (on by
// default; yell_set_host_access).
extern std::atomic<bool> g_host_access;

class DeviceContext {
 public:
  // Context of the current device; nullptr and a recorded error on failure.
  static DeviceContext* current(int* status);

  int device() const { return device_; }
  cudaStream_t stream() const { return stream_; }

  // DevMod array of this degree (kMaxModuli entries, device memory) with the
  // tables of every listed modulus built and resident.  Safe to call from
  // several threads; building takes the registry lock.  Issues no CUDA call
  // when every table is already resident (so it is safe inside capture).
  int ensure_tables(uint32_t log_n, uint32_t cm0, uint32_t L, const DevMod** mods);
  int ensure_tables_list(uint32_t log_n, const uint32_t* cms, uint32_t n, const DevMod** mods);
  const DevMod* mods_if_ready(uint32_t log_n) const;
  // DevMod array of this degree if the tables of moduli cm0 .. cm0+L-1 are
  // all resident, else nullptr.  Makes no CUDA call and allocates nothing.
  const DevMod* tables_ready(uint32_t log_n, uint32_t cm0, uint32_t L) const;

  // Device buffer of at least `words` words owned by the context; grows on
  // demand.  The caller holds `lock` for as long as it uses the buffer.
  struct Buffer {
    std::mutex lock;
    uint64_t* ptr = nullptr;
    size_t words = 0;
    int reserve(size_t words);  // under lock
    ~Buffer();
  };
  Buffer staging;   // host-pointer drop-ins: operands / results

  // Stream-ordered scratch for device-resident calls made without caller
  // scratch: taken from this context's memory pool on the caller's stream
  // and given back on that stream after the kernels that use it, so the call
  // returns before its work completes and concurrent calls on different
  // streams each get their own.  The pool keeps freed memory for reuse (no
  // release threshold), so after the first call of a size no memory is
  // obtained from the driver.
  int scratch_alloc_async(size_t words, cudaStream_t st, uint64_t** out);
  int scratch_free_async(uint64_t* p, cudaStream_t st);

  // Pinned host memory mapped into this device's address space, for small
  // host-pointer calls: the caller's words are copied in on the host and the
  // kernel reads and writes them in place, so a call is one launch and one
  // stream synchronisation instead of copy calls around the launch.  Three
  // operands of kSmallCallWords words each; allocated on first use.
  static constexpr size_t kSmallCallWords = size_t(1) << 15;
  struct HostMapped {
    std::mutex lock;
    uint64_t* host = nullptr;  // host address
    uint64_t* dev = nullptr;   // the same memory as the device sees it
    int ensure();              // under lock
  };
  HostMapped small;

  // Pipelined host polymul, under `pipe_lock`: one stream each for H2D,
  // compute and D2H; kPipeSlots device buffer sets cycled by the chunks, with
  // per-slot events ordering reuse of a slot's buffers.
  std::mutex pipe_lock;
  static constexpr int kPipeSlots = 3;
  cudaStream_t pipe_stream[3] = {};  // 0: H2D, 1: compute, 2: D2H
  cudaEvent_t pipe_h2d[kPipeSlots] = {}, pipe_comp[kPipeSlots] = {}, pipe_d2h[kPipeSlots] = {};
  Buffer pipe_buf[kPipeSlots];

  NttShape shape;  // launch shape (autotuner may adjust)

  // The device loads and stores pageable host memory through the host's page
  // tables (cudaDevAttrPageableMemoryAccess and
  // cudaDevAttrPageableMemoryAccessUsesHostPageTables), and direct host access
  // is enabled (yell_set_host_access): host-pointer calls then move the
  // caller's limbs with gather / scatter kernels instead of pageable copies.
  bool host_access() const;

 private:
  explicit DeviceContext(int device);
  int init();

  int device_;
  bool pageable_access_ = false;
  cudaStream_t stream_ = nullptr;
  cudaMemPool_t pool_ = nullptr;
  mutable std::mutex tables_mu_;
  DevMod* d_mods_[kMaxLogN + 1] = {};
  std::vector<uint8_t> built_[kMaxLogN + 1];
  std::vector<void*> table_allocs_;
};

}  // namespace yell_gb300
