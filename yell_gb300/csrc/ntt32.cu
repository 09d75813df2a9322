// 32-bit moduli mode of the hot path (the reference built with
// -DYELL_USE_32BITS_MODULI: include/yell/params_32.hpp, 291 30-bit primes,
// uint32 words and uint64 products, degrees up to kMaxPolyDegree = 2^15).
//
// The kernels reuse the tile engine of the 64-bit path at 32-bit words.  A CTA
// holds whole limbs in shared memory (2^T words, T = max(log_n, 11), several
// limbs per CTA below 2^11); every word is read from HBM once and written
// once.  The single-CTA fused polymul keeps one operand tile in shared memory
// at a time: NTT(a) leaves its last forward round in registers and parks the
// reduced words in the output limb (the same thread reads them back, so they
// stay in L2), NTT(b) then runs in the same buffer, and the product, inverse
// rounds and scaled last layer follow.  At 2^14 and 2^15 a limb is split over
// a CTA pair whose operands arrive by bulk asynchronous copies, b's while a
// computes, and a's NTT waits in shared memory.  The butterflies, their order
// and their twiddle indices are the reference's, so lazy words match it
// exactly.
#include <algorithm>
#include <cstring>
#include <memory>
#include <mutex>
#include <string>
#include <utility>
#include <vector>

#include <cooperative_groups.h>

#include "async_copy.cuh"
#include "kernels.h"
#include "ntt_tile.cuh"
#include "profiler.h"
#include "runtime.h"
#include "yell_gb300.h"

namespace yell_gb300 {
namespace {

constexpr uint32_t kMaxModuli32 = 291;   // params_32.hpp kMaxNbModuli
constexpr uint32_t kLogMaxDegree32 = 15; // kMaxPolyDegree = 2^15
constexpr uint32_t kMinLogN32 = 3;

// ---- prime table -------------------------------------------------------------
// params_32.hpp:15-34: p = 2^30 - j * 2^16 + 1 for increasing j, kept when
// prime (the stated 2^14 step, restricted to p = 1 mod 2^16 so that a
// primitive 2^16-th root exists); Pn = low word of floor(2^64 / p);
// primitive_roots[cm] = g^((p - 1) / 2^16), g the least primitive root.
struct Prime32 {
  uint32_t p, pn, root;
};

uint32_t pow32(uint64_t b, uint64_t e, uint32_t m) {
  uint64_t r = 1;
  b %= m;
  while (e) {
    if (e & 1) r = r * b % m;
    b = b * b % m;
    e >>= 1;
  }
  return (uint32_t)r;
}

bool is_prime32(uint32_t n) {
  if (n < 2) return false;
  for (uint32_t q : {2u, 7u, 61u})
    if (n % q == 0) return n == q;
  uint32_t d = n - 1;
  int s = 0;
  while (!(d & 1)) d >>= 1, ++s;
  for (uint32_t a : {2u, 7u, 61u}) {
    uint64_t x = pow32(a, d, n);
    if (x == 1 || x == n - 1) continue;
    bool comp = true;
    for (int r = 1; r < s && comp; ++r) {
      x = x * x % n;
      if (x == n - 1) comp = false;
    }
    if (comp) return false;
  }
  return true;
}

uint32_t least_primitive_root32(uint32_t p) {
  std::vector<uint32_t> f;
  uint32_t m = p - 1;
  for (uint32_t q = 2; q * q <= m; ++q)
    if (m % q == 0) {
      f.push_back(q);
      while (m % q == 0) m /= q;
    }
  if (m > 1) f.push_back(m);
  for (uint32_t g = 2;; ++g) {
    bool ok = true;
    for (uint32_t q : f) ok = ok && pow32(g, (p - 1) / q, p) != 1;
    if (ok) return g;
  }
}

const std::vector<Prime32>& primes32() {
  static std::vector<Prime32> table = [] {
    std::vector<Prime32> t;
    for (uint32_t j = 1; t.size() < kMaxModuli32; ++j) {
      const uint32_t p = (1u << 30) - j * (1u << 16) + 1;
      if (!is_prime32(p)) continue;
      t.push_back({p, (uint32_t)(~0ull / p), pow32(least_primitive_root32(p), (p - 1) >> 16, p)});
    }
    return t;
  }();
  return table;
}

uint32_t shoupify32(uint32_t x, uint32_t p) { return (uint32_t)(((uint64_t)x << 32) / p); }

// details/ntt.hpp:28-77 at 32-bit words: psi = root^(2^(15 - log_n)); phi and
// invphi powers with Shoup forms, bit-reversed; N^-1 and N^-1 * invphi[1].
void build_host_tables32(uint32_t log_n, uint32_t cm, uint32_t* out4n, uint32_t* sc4) {
  const Prime32& pe = primes32()[cm];
  const uint32_t p = pe.p, n = 1u << log_n;
  uint32_t psi = pe.root;
  for (uint32_t i = 0; i < kLogMaxDegree32 - log_n; ++i) psi = (uint32_t)((uint64_t)psi * psi % p);
  const uint32_t ipsi = pow32(psi, 2ull * n - 1, p);
  uint32_t a = 1, b = 1;
  for (uint32_t i = 0; i < n; ++i) {
    uint32_t r = 0;
    for (uint32_t k = 0; k < log_n; ++k) r |= ((i >> k) & 1u) << (log_n - 1 - k);
    out4n[r] = a;
    out4n[n + r] = shoupify32(a, p);
    out4n[2 * n + r] = b;
    out4n[3 * n + r] = shoupify32(b, p);
    a = (uint32_t)((uint64_t)a * psi % p);
    b = (uint32_t)((uint64_t)b * ipsi % p);
  }
  const uint32_t inv_n = pow32(n % p, p - 2, p);
  const uint32_t inv_n_iphi = (uint32_t)((uint64_t)inv_n * out4n[2 * n + 1] % p);
  sc4[0] = inv_n;
  sc4[1] = shoupify32(inv_n, p);
  sc4[2] = inv_n_iphi;
  sc4[3] = shoupify32(inv_n_iphi, p);
}

// ---- device tables -------------------------------------------------------------
struct DeviceTables32 {
  std::mutex mu;
  DevMod32* mods[kLogMaxDegree32 + 1] = {};
  std::vector<uint8_t> built[kLogMaxDegree32 + 1];
};

DeviceTables32& tables_of(int device) {
  static std::mutex mu;
  static std::vector<std::unique_ptr<DeviceTables32>> all;
  std::lock_guard<std::mutex> g(mu);
  if ((int)all.size() <= device) all.resize(device + 1);
  if (!all[device]) all[device].reset(new DeviceTables32);
  return *all[device];
}

int ensure32(int device, uint32_t log_n, uint32_t cm0, uint32_t L, const DevMod32** out) {
  DeviceTables32& t = tables_of(device);
  std::lock_guard<std::mutex> g(t.mu);
  std::vector<uint8_t>& built = t.built[log_n];
  if (built.empty()) built.assign(kMaxModuli32, 0);
  cudaError_t e;
  if (!t.mods[log_n]) {
    // [cm]: transforms and element-wise ops; [kMaxModuli32 + cm]: the fused
    // polymul (Montgomery product, inverse scaled by N^-1 * 2^32)
    e = lib_malloc(&t.mods[log_n], 2 * kMaxModuli32 * sizeof(DevMod32));
    if (e != cudaSuccess) {
      t.mods[log_n] = nullptr;
      return fail_cuda(e, "cudaMalloc(DevMod32 table)");
    }
    e = cudaMemset(t.mods[log_n], 0, 2 * kMaxModuli32 * sizeof(DevMod32));
    if (e != cudaSuccess) return fail_cuda(e, "cudaMemset(DevMod32 table)");
  }
  const uint32_t n = 1u << log_n;
  std::vector<uint32_t> host(4 * (size_t)n), packed(4 * (size_t)n);
  for (uint32_t cm = cm0; cm < cm0 + L; ++cm) {
    if (built[cm]) continue;
    uint32_t sc[4];
    build_host_tables32(log_n, cm, host.data(), sc);
    for (uint32_t k = 0; k < n; ++k) {  // {w, w'} pairs: fwd then inv
      packed[2 * k] = host[k];
      packed[2 * k + 1] = host[n + k];
      packed[2 * (size_t)n + 2 * k] = host[2 * n + k];
      packed[2 * (size_t)n + 2 * k + 1] = host[3 * n + k];
    }
    uint32_t* d = nullptr;
    e = lib_malloc(&d, packed.size() * sizeof(uint32_t));
    if (e != cudaSuccess) return fail_cuda(e, "cudaMalloc(twiddles32)");
    e = cudaMemcpy(d, packed.data(), packed.size() * sizeof(uint32_t), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return fail_cuda(e, "upload twiddles32");
    DevMod32 m;
    m.fwd = reinterpret_cast<const uint2*>(d);
    m.inv = reinterpret_cast<const uint2*>(d + 2 * (size_t)n);
    m.p = primes32()[cm].p;
    m.pn = primes32()[cm].pn;
    m.inv_n = sc[0];
    m.inv_n_s = sc[1];
    m.inv_n_iphi = sc[2];
    m.inv_n_iphi_s = sc[3];
    e = cudaMemcpy(t.mods[log_n] + cm, &m, sizeof m, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return fail_cuda(e, "upload DevMod32");
    DevMod32 pm = m;
    uint32_t inv = m.p;  // p * p = 1 mod 8; Newton's iteration doubles the correct low bits
    for (int i = 0; i < 4; ++i) inv *= 2u - m.p * inv;
    const uint64_t r32 = (1ull << 32) % m.p;
    pm.pn = 0u - inv;
    pm.inv_n = (uint32_t)(m.inv_n * r32 % m.p);
    pm.inv_n_s = shoupify32(pm.inv_n, m.p);
    pm.inv_n_iphi = (uint32_t)(m.inv_n_iphi * r32 % m.p);
    pm.inv_n_iphi_s = shoupify32(pm.inv_n_iphi, m.p);
    e = cudaMemcpy(t.mods[log_n] + kMaxModuli32 + cm, &pm, sizeof pm, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return fail_cuda(e, "upload DevMod32");
    built[cm] = 1;
  }
  *out = t.mods[log_n];
  return kOk;
}

// ---- kernels -------------------------------------------------------------------
// Tile geometry per degree: whole limbs, 2^LOGE words per thread.
template <int LOGN>
struct Cfg32 {
  static constexpr int T = LOGN > 11 ? LOGN : 11;
  static constexpr int LOGE = LOGN < 4 ? LOGN : (T == 15 ? 5 : 4);
  using C = TileCfg<T, LOGN, 0, LOGE>;
  static constexpr size_t kSmem = Smem<uint32_t>::words(1u << T) * sizeof(uint32_t);
};

struct Limbs32 {
  uint32_t count, L, cm0;
  __device__ __forceinline__ uint32_t cm(uint32_t k) const { return cm0 + k % L; }
};

// Tile <- limbs limb0 .. (16-byte global loads and shared stores).  All of a
// thread's loads are issued before its first store.
template <class C>
__device__ __forceinline__ void stage_in32(uint32_t* s, const uint32_t* g, uint32_t limb0, uint32_t count) {
  constexpr int IT = (1 << C::T) / (C::THREADS * 4);
  static_assert(IT * C::THREADS * 4 == (1 << C::T), "tile not a whole number of 16-byte chunks per thread");
  uint4 d[IT];
#pragma unroll
  for (int i = 0; i < IT; ++i) {
    const uint32_t v = (threadIdx.x + i * C::THREADS) * 4;
    const uint32_t limb = limb0 + (v >> C::K);
    if (limb < count)
      d[i] = __ldg(reinterpret_cast<const uint4*>(g + ((size_t)limb << C::K) + (v & ((1u << C::K) - 1u))));
  }
#pragma unroll
  for (int i = 0; i < IT; ++i) {
    const uint32_t v = (threadIdx.x + i * C::THREADS) * 4;
    if (limb0 + (v >> C::K) < count) *reinterpret_cast<uint4*>(s + Smem<uint32_t>::idx(v)) = d[i];
  }
}

template <class C>
__device__ __forceinline__ void stage_out32(const uint32_t* s, uint32_t* g, uint32_t limb0, const Limbs32& ls,
                                            const DevMod32* __restrict__ mods, bool reduce) {
  for (uint32_t v = threadIdx.x * 4; v < (1u << C::T); v += C::THREADS * 4) {
    const uint32_t limb = limb0 + (v >> C::K);
    if (limb < ls.count) {
      uint4 d = *reinterpret_cast<const uint4*>(s + Smem<uint32_t>::idx(v));
      if (reduce) {
        const uint32_t p = __ldg(&mods[ls.cm(limb)].p), p2 = p << 1;
        d.x = fwd_correct(d.x, p, p2);
        d.y = fwd_correct(d.y, p, p2);
        d.z = fwd_correct(d.z, p, p2);
        d.w = fwd_correct(d.w, p, p2);
      }
      *reinterpret_cast<uint4*>(g + ((size_t)limb << C::K) + (v & ((1u << C::K) - 1u))) = d;
    }
  }
}

// DIR: 0 forward (reduced to [0, p)), 1 forward lazy ([0, 4p)), 2 backward.
template <class C, int DIR>
__global__ void __launch_bounds__(C::THREADS, 1024 / C::THREADS) k32_ntt(uint32_t* data, Limbs32 ls, const DevMod32* __restrict__ mods) {
  extern __shared__ __align__(16) uint32_t smem32[];
  constexpr int NR = C::NR;
  const uint32_t tid = threadIdx.x;
  const uint32_t limb0 = blockIdx.x << (C::T - C::K);
  const uint32_t my_limb = limb0 + C::sub(tid);
  const bool active = my_limb < ls.count;
  const DevMod32 m = load_mod(mods, ls.cm(active ? my_limb : 0));
  stage_in32<C>(smem32, data, limb0, ls.count);
  __syncthreads();
  if constexpr (DIR != 2) {
    fwd_rounds<C, 0, NR>(smem32, tid, 0, 0, m.fwd, m.p, active);
  } else {
    inv_rounds<C, NR - 1, -1, true>(smem32, tid, (uint32_t)C::K, 0, 0, m, active);
  }
  stage_out32<C>(smem32, data, limb0, ls, mods, DIR == 0);
}

// c = INTT(NTT(a) * NTT(b)) per limb; c must not alias a or b.
template <class C>
__global__ void __launch_bounds__(C::THREADS, 1024 / C::THREADS) k32_polymul(uint32_t* c, const uint32_t* a, const uint32_t* b,
                                                          Limbs32 ls, const DevMod32* __restrict__ mods) {
  extern __shared__ __align__(16) uint32_t smem32[];
  constexpr int NR = C::NR, E = 1 << C::LOGE;
  using RB = Round<C, NR - 1>;
  static_assert(RB::R == C::LOGE && RB::BETA == 0 && RB::EB == 0, "bottom round must own contiguous words");
  const uint32_t tid = threadIdx.x;
  const uint32_t limb0 = blockIdx.x << (C::T - C::K);
  const uint32_t my_limb = limb0 + C::sub(tid);
  const bool active = my_limb < ls.count;
  const DevMod32 m = load_mod(mods, ls.cm(active ? my_limb : 0));
  const uint32_t p = m.p, p2 = p << 1;
  const uint32_t bb = RB::base(tid);
  // the thread's E contiguous words of the output tile (in limb my_limb)
  uint32_t* park = c + ((size_t)my_limb << C::K) + (bb & ((1u << C::K) - 1u));
  uint32_t x[E];
  // NTT(a), parked in c
  stage_in32<C>(smem32, a, limb0, ls.count);
  __syncthreads();
  fwd_rounds<C, 0, NR - 1>(smem32, tid, 0, 0, m.fwd, p, active);
  if (active) {
    smem_load<RB>(x, smem32, bb);
    ct_round<RB>(x, m.fwd, (uint32_t)RB::HI, RB::gr(bb, 0), p);
#pragma unroll
    for (int i = 0; i < E; i += 4)
      *reinterpret_cast<uint4*>(park + i) =
          make_uint4(csub(x[i], p2), csub(x[i + 1], p2), csub(x[i + 2], p2), csub(x[i + 3], p2));
  }
  __syncthreads();
  // NTT(b), product, inverse
  stage_in32<C>(smem32, b, limb0, ls.count);
  __syncthreads();
  fwd_rounds<C, 0, NR - 1>(smem32, tid, 0, 0, m.fwd, p, active);
  if (active) {
    smem_load<RB>(x, smem32, bb);
    ct_round<RB>(x, m.fwd, (uint32_t)RB::HI, RB::gr(bb, 0), p);
#pragma unroll
    for (int i = 0; i < E; i += 4) {
      const uint4 ah = *reinterpret_cast<const uint4*>(park + i);  // written above by this thread
      x[i] = mont_mul(ah.x, csub(x[i], p2), p, m.pn);
      x[i + 1] = mont_mul(ah.y, csub(x[i + 1], p2), p, m.pn);
      x[i + 2] = mont_mul(ah.z, csub(x[i + 2], p2), p, m.pn);
      x[i + 3] = mont_mul(ah.w, csub(x[i + 3], p2), p, m.pn);
    }
    gs_round<RB, NR == 1>(x, (uint32_t)C::K, (uint32_t)RB::BETA, RB::gr(bb, 0), m);
    smem_store<RB>(x, smem32, bb);
  }
  __syncthreads();
  inv_rounds<C, NR - 2, -1, true>(smem32, tid, (uint32_t)C::K, 0, 0, m, active);
  stage_out32<C>(smem32, c, limb0, ls, mods, false);
}


// ---- polymul by a CTA pair (thread-block cluster of 2) ------------------------
// For N = 2^14 and 2^15 one limb is split over two CTAs of one cluster, each
// holding half of it (2^(log N - 1) words, 64 KB at 2^15).  The forward stage
// that pairs words N/2 apart (stage 0, twiddle w[1]) is applied while
// loading: each CTA reads both halves (the second read of a word comes from
// L2) and keeps the butterfly output of its own half.  Stages 1 .. log N - 1
// stay inside a half (group G = the CTA's rank).  The inverse's last layer
// (N^-1 scaling fused) pairs the halves again: after a cluster barrier each
// CTA reads the peer's words through distributed shared memory and writes its
// own half of the outputs.
//
// The stages inside a half limb of 2^H words run as two tiles of the engine:
// the top KTOP (pair distances 2^(H-1) .. 2^(H-KTOP)) across the CTA (CA:
// columns of stride 2^(H-KTOP), CTA barriers), the other H - KTOP in rows of
// 2^(H-KTOP) words (CB), each row held by the threads of one warp, so the
// rounds inside a row need only warp barriers.  The bottom round gives each
// thread 2^LOGE consecutive words.
template <int H, int LOGE, int KTOP>
struct HalfSplit {
  using CA = TileCfg<H, KTOP, H - KTOP, LOGE>;
  using CB = TileCfg<H, H - KTOP, 0, LOGE>;
  static constexpr int KB = H - KTOP, KTOP_STAGES = KTOP;
  static_assert(CA::THREADS == CB::THREADS && CB::LOCAL_BARRIER == 1, "rows must stay inside a warp");
  // Row index within the whole limb (the sub-transform group of CB's top stage).
  __device__ static __forceinline__ uint32_t row_group(uint32_t r, uint32_t tid) {
    return (r << KTOP) + CB::sub(tid);
  }
};

// Geometry of a CTA-pair kernel: half limbs of 2^(LOGN-1) words, 2^LOGE words
// per thread, the top KTOP stages of the half across the CTA.
template <int LOGN, int LOGE_, int KTOP_>
struct PairGeom32 {
  static constexpr int H = LOGN - 1;
  static constexpr int LOGE = LOGE_;
  static constexpr int KTOP = KTOP_;
  using C = TileCfg<H, H, 0, LOGE>;
  using S = HalfSplit<H, LOGE, KTOP>;
  static constexpr int MIN_BLOCKS = C::THREADS <= 256 ? 3 : (C::THREADS <= 512 ? 2 : 1);
  static constexpr size_t kSmem = Smem<uint32_t>::words(1u << H) * sizeof(uint32_t);
};

// Polymul.  2^14: 256-thread CTAs of 32 words per thread, three per SM at 80
// registers.  2^15: 1024-thread CTAs of 16 words per thread, one per SM at 64
// registers, top 7 stages across the CTA and rows of 128 words: the same 32
// resident warps per SM as two 512-thread CTAs of 32 words, without their
// 216 bytes of register spills, and 1024 CTA-sized units per 512-limb launch
// fill 6.7 waves of 152 SMs where limb pairs filled 3.4 waves of 304 slots.
// Measured on GB300 (N = 2^15, L = 32, 16 pairs): 0.2228 ms, the same as two
// 512-thread CTAs per SM (0.2228 ms); with the top 6 or 8 stages across the
// CTA 0.2238 and 0.2273 ms.  Staged (k32_polymul_pair_staged, one CTA per SM
// by its shared memory), 512-thread CTAs of 32 words at 128 registers took
// 0.2087 / 0.2195 / 0.2353 ms with the top 5 / 6 / 7 stages across the CTA,
// against 0.2053 ms for this geometry.
template <int LOGN>
using PairCfg32 = PairGeom32<LOGN, (LOGN >= 15 ? 4 : 5), (LOGN >= 15 ? 7 : 5)>;

// NTT alone: 32 words per thread at both degrees; at 2^15 two 512-thread CTAs
// per SM (64 registers, no spills) with the top 5 stages across the CTA:
// rounds of 5 stages, one exchange fewer per transform.  Measured (2^15,
// L = 32, 16 polys): backward 90.7 -> 77.1 us, forward 83.4 / 83.8 us.
template <int LOGN>
using NttPairCfg32 = PairGeom32<LOGN, 5, 5>;

// Forward NTT of one half limb of `src` (the limb's first word) into the
// bottom-round registers x of this thread: stage 0 while loading, stages
// 1 .. log N - 1 in shared memory, the last round in registers.
template <class PC, bool CLUSTER_SYNC = false>
__device__ __forceinline__ void pair_forward(uint32_t* x, const uint32_t* __restrict__ src, uint32_t* smem32,
                                             uint32_t tid, uint32_t r, const DevMod32& m, uint2 w1) {
  using C = typename PC::C;
  using S = typename PC::S;
  constexpr int H = C::K, NR = C::NR;
  constexpr uint32_t half = 1u << H;
  constexpr int IT = (int)(half / (C::THREADS * 4));
  constexpr int BATCH = IT < 2 ? IT : 2;  // loads in flight per thread: 2 x BATCH x 16 bytes
  using RB = Round<C, NR - 1>;
  const uint32_t p = m.p, p2 = p << 1, np = 0u - p;
#pragma unroll 1  // unrolled, the loads of every batch get hoisted together and spill
  for (int i0 = 0; i0 < IT; i0 += BATCH) {
    uint4 lo[BATCH], hi[BATCH];
#pragma unroll
    for (int i = 0; i < BATCH; ++i) {
      const uint32_t v = (tid + (i0 + i) * C::THREADS) * 4;
      lo[i] = __ldg(reinterpret_cast<const uint4*>(src + v));
      hi[i] = __ldg(reinterpret_cast<const uint4*>(src + half + v));
    }
#pragma unroll
    for (int i = 0; i < BATCH; ++i) {
      const uint32_t v = (tid + (i0 + i) * C::THREADS) * 4;
      uint32_t u0[4] = {lo[i].x, lo[i].y, lo[i].z, lo[i].w}, u1[4] = {hi[i].x, hi[i].y, hi[i].z, hi[i].w};
#pragma unroll
      for (int k = 0; k < 4; ++k) ct_bfly(u0[k], u1[k], w1.x, w1.y, np, p2);
      *reinterpret_cast<uint4*>(smem32 + Smem<uint32_t>::idx(v)) =
          r == 0 ? make_uint4(u0[0], u0[1], u0[2], u0[3]) : make_uint4(u1[0], u1[1], u1[2], u1[3]);
    }
  }
  // an in-place transform may overwrite src only once both CTAs have read it
  if constexpr (CLUSTER_SYNC) cooperative_groups::this_cluster().sync();
  else __syncthreads();
  using CA = typename S::CA;
  using CB = typename S::CB;
  using RBB = Round<CB, CB::NR - 1>;
  static_assert(RBB::R == RB::R && RBB::BETA == 0 && RBB::EB == 0, "same bottom round as one tile over the half");
  constexpr uint32_t s_rows = 1 + S::KTOP_STAGES;  // first stage of the rows
  fwd_rounds<CA, 0, CA::NR>(smem32, tid, 1, r, m.fwd, p, true);  // stages 1..KTOP, CTA barriers
  const uint32_t G = S::row_group(r, tid);
  fwd_rounds<CB, 0, CB::NR - 1, CB::LOCAL_BARRIER>(smem32, tid, s_rows, G, m.fwd, p, true);
  const uint32_t bb = RBB::base(tid);
  smem_load<RBB>(x, smem32, bb);
  ct_round<RBB>(x, m.fwd, s_rows + RBB::HI, RBB::gr(bb, G), p);
}

// Inverse stages inside the half limb from the bottom-round registers x:
// rows (warp barriers), then the top KTOP across the CTA; the words end in
// shared memory.  CB's last round is followed by a CTA barrier.
template <class PC>
__device__ __forceinline__ void pair_inverse(uint32_t* x, uint32_t* smem32, uint32_t tid, uint32_t r,
                                             uint32_t bb, const DevMod32& m) {
  using C = typename PC::C;
  using S = typename PC::S;
  using CA = typename S::CA;
  using CB = typename S::CB;
  using RBB = Round<CB, CB::NR - 1>;
  constexpr uint32_t log_n = C::K + 1;
  const uint32_t G = S::row_group(r, tid);
  gs_round<RBB, false>(x, log_n, (uint32_t)RBB::BETA, RBB::gr(bb, G), m);
  smem_store<RBB>(x, smem32, bb);
  round_barrier<CB, CB::LOCAL_BARRIER>(tid);
  inv_rounds<CB, CB::NR - 2, 0, false, CB::LOCAL_BARRIER>(smem32, tid, log_n, 0, G, m, true);
  inv_rounds<CB, 0, -1, false>(smem32, tid, log_n, 0, G, m, true);  // CTA barrier after
  inv_rounds<CA, CA::NR - 1, -1, false>(smem32, tid, log_n, S::KB, r, m, true);
}

// Last inverse layer across the pair with the N^-1 scaling: u = word i
// (rank 0), w = word i + N/2 (rank 1); each CTA writes its own half.
template <class PC, bool UNROLL>
__device__ __forceinline__ void pair_last_layer(uint32_t* dst, const uint32_t* smem32, const uint32_t* peer,
                                                uint32_t tid, uint32_t r, const DevMod32& m) {
  using C = typename PC::C;
  constexpr int IT = (int)((1u << C::K) / (C::THREADS * 4));
  const uint32_t p2 = m.p << 1;
#pragma unroll(UNROLL ? IT : 1)
  for (int i = 0; i < IT; ++i) {
    const uint32_t v = (tid + i * C::THREADS) * 4;
    const uint4 own = *reinterpret_cast<const uint4*>(smem32 + Smem<uint32_t>::idx(v));
    const uint4 oth = *reinterpret_cast<const uint4*>(peer + Smem<uint32_t>::idx(v));
    const uint32_t o[4] = {own.x, own.y, own.z, own.w}, q[4] = {oth.x, oth.y, oth.z, oth.w};
    uint32_t res[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const uint32_t u = r == 0 ? o[k] : q[k], w = r == 0 ? q[k] : o[k];
      res[k] = r == 0 ? mulmod_shoup(u + w, m.inv_n, m.inv_n_s, m.p)
                      : mulmod_shoup(u - w + p2, m.inv_n_iphi, m.inv_n_iphi_s, m.p);
    }
    *reinterpret_cast<uint4*>(dst + v) = make_uint4(res[0], res[1], res[2], res[3]);
  }
}

template <class PC>
__global__ void __cluster_dims__(2, 1, 1) __launch_bounds__(PC::C::THREADS, PC::MIN_BLOCKS)
    k32_polymul_pair(uint32_t* c, const uint32_t* a, const uint32_t* b, Limbs32 ls,
                     const DevMod32* __restrict__ mods) {
  namespace cg = cooperative_groups;
  using C = typename PC::C;
  extern __shared__ __align__(16) uint32_t smem32[];
  constexpr int H = C::K, NR = C::NR, E = 1 << C::LOGE;
  constexpr uint32_t log_n = H + 1, half = 1u << H;
  constexpr int IT = (int)(half / (C::THREADS * 4));
  using RB = Round<C, NR - 1>;
  static_assert(RB::R == C::LOGE && RB::BETA == 0 && RB::EB == 0, "bottom round must own contiguous words");
  static_assert(IT * C::THREADS * 4 == (int)half, "half limb not a whole number of 16-byte chunks per thread");
  static_assert(IT % 2 == 0 || IT == 1, "stage-in batches of two");
  cg::cluster_group cluster = cg::this_cluster();
  const uint32_t r = cluster.block_rank();  // which half of the limb
  const uint32_t limb = blockIdx.x >> 1;    // grid = 2 x limbs, every CTA active
  const uint32_t tid = threadIdx.x;
  const DevMod32 m = load_mod(mods, ls.cm(limb));
  const uint32_t p = m.p, p2 = p << 1;
  const uint2 w1 = __ldg(m.fwd + 1);
  const size_t lbase = (size_t)limb << log_n;
  const uint32_t bb = RB::base(tid);
  uint32_t* park = c + lbase + r * half + bb;
  uint32_t x[E];
  pair_forward<PC>(x, a + lbase, smem32, tid, r, m, w1);
#pragma unroll
  for (int i = 0; i < E; i += 4)
    *reinterpret_cast<uint4*>(park + i) =
        make_uint4(csub(x[i], p2), csub(x[i + 1], p2), csub(x[i + 2], p2), csub(x[i + 3], p2));
  __syncthreads();  // the buffer is reused for b
  pair_forward<PC>(x, b + lbase, smem32, tid, r, m, w1);
#pragma unroll
  for (int i = 0; i < E; i += 4) {
    const uint4 ah = *reinterpret_cast<const uint4*>(park + i);  // written above by this thread
    x[i] = mont_mul(ah.x, csub(x[i], p2), p, m.pn);
    x[i + 1] = mont_mul(ah.y, csub(x[i + 1], p2), p, m.pn);
    x[i + 2] = mont_mul(ah.z, csub(x[i + 2], p2), p, m.pn);
    x[i + 3] = mont_mul(ah.w, csub(x[i + 3], p2), p, m.pn);
  }
  pair_inverse<PC>(x, smem32, tid, r, bb, m);
  cluster.sync();
  pair_last_layer<PC, true>(c + lbase + r * half, smem32, cluster.map_shared_rank(smem32, (int)(r ^ 1u)), tid, r, m);
  cluster.sync();  // the peer may still be reading this CTA's shared memory
}

// ---- polymul by a CTA pair with staged operands ------------------------------
// The same butterflies as k32_polymul_pair, with the operands moved by bulk
// asynchronous copies (cp.async.bulk, completion counted on an mbarrier):
// both halves of a's limb land in a raw staging area S of shared memory; the
// stage-0 butterflies read them from there; then b's copy into S starts and
// runs while a's remaining stages compute.  a's reduced NTT stays in the work
// tile W where its bottom round left it, and b is transformed in place in S
// (its own-half outputs overwrite the raw words once every thread has read
// its pairs).  Shared memory: W (half limb) + S (whole limb) + the mbarrier.
// Every wait on the mbarrier is bounded; one that runs out records
// YELL_ERR_TIMEOUT in g_k32_wait_status and the kernel carries on, so that
// every thread still reaches every barrier.
__device__ uint32_t g_k32_wait_status;

// Bounded wait on the staged kernel's mbarrier; a wait that runs out records
// YELL_ERR_TIMEOUT in g_k32_wait_status.
__device__ __forceinline__ bool mbar_wait32(uint64_t* mbar, uint32_t parity,
                                            uint64_t timeout_ns = 1000000000ull) {
  return mbar_wait(mbar, parity, &g_k32_wait_status, (uint32_t)YELL_ERR_TIMEOUT, timeout_ns);
}

// Check of that bounded wait: one CTA announces 16 bytes of copies on an
// mbarrier, starts none, and waits on it the way the staged kernel does; the
// wait runs out after timeout_ns and records YELL_ERR_TIMEOUT.  No copy is in
// flight when the CTA exits.
__global__ void k32_wait_check(uint64_t timeout_ns) {
  __shared__ uint64_t mbar;
  if (threadIdx.x == 0) {
    mbar_init(&mbar, 1);
    mbar_expect(&mbar, 16);
  }
  __syncthreads();
  mbar_wait32(&mbar, 0, timeout_ns);
}

// Stage 0 (pairs N/2 apart, twiddle w[1]) from the raw halves of a limb in
// S_lo and S_hi into this CTA's half in `dst` (swizzled tile layout).  With
// IN_PLACE, dst overlaps S_lo: every thread keeps its outputs in registers
// until all raw words are read.
// Ends with a CTA barrier.
template <class PC, bool IN_PLACE>
__device__ __forceinline__ void stage0_from_smem(uint32_t* dst, const uint32_t* S_lo, const uint32_t* S_hi,
                                                 uint32_t tid, uint32_t r, uint32_t p, uint2 w1) {
  using C = typename PC::C;
  constexpr uint32_t half = 1u << C::K;
  constexpr int IT = (int)(half / (C::THREADS * 4));
  const uint32_t p2 = p << 1, np = 0u - p;
  uint4 out[IN_PLACE ? IT : 1];
#pragma unroll
  for (int i = 0; i < IT; ++i) {
    const uint32_t v = (tid + i * C::THREADS) * 4;
    const uint4 lo = *reinterpret_cast<const uint4*>(S_lo + v);
    const uint4 hi = *reinterpret_cast<const uint4*>(S_hi + v);
    uint32_t u0[4] = {lo.x, lo.y, lo.z, lo.w}, u1[4] = {hi.x, hi.y, hi.z, hi.w};
#pragma unroll
    for (int k = 0; k < 4; ++k) ct_bfly(u0[k], u1[k], w1.x, w1.y, np, p2);
    const uint4 o = r == 0 ? make_uint4(u0[0], u0[1], u0[2], u0[3]) : make_uint4(u1[0], u1[1], u1[2], u1[3]);
    if constexpr (IN_PLACE) out[i] = o;
    else *reinterpret_cast<uint4*>(dst + Smem<uint32_t>::idx(v)) = o;
  }
  if constexpr (IN_PLACE) {
    __syncthreads();
#pragma unroll
    for (int i = 0; i < IT; ++i)
      *reinterpret_cast<uint4*>(dst + Smem<uint32_t>::idx((tid + i * C::THREADS) * 4)) = out[i];
  }
  __syncthreads();
}

// Stages 1 .. log N - 1 of the half limb in `work` (after stage 0), the last
// round into the registers x; the same rounds as pair_forward.
template <class PC>
__device__ __forceinline__ void pair_forward_rounds(uint32_t* x, uint32_t* work, uint32_t tid, uint32_t r,
                                                    const DevMod32& m) {
  using C = typename PC::C;
  using S = typename PC::S;
  using CA = typename S::CA;
  using CB = typename S::CB;
  using RBB = Round<CB, CB::NR - 1>;
  constexpr uint32_t s_rows = 1 + S::KTOP_STAGES;
  fwd_rounds<CA, 0, CA::NR>(work, tid, 1, r, m.fwd, m.p, true);
  const uint32_t G = S::row_group(r, tid);
  fwd_rounds<CB, 0, CB::NR - 1, CB::LOCAL_BARRIER>(work, tid, s_rows, G, m.fwd, m.p, true);
  const uint32_t bb = RBB::base(tid);
  smem_load<RBB>(x, work, bb);
  ct_round<RBB>(x, m.fwd, s_rows + RBB::HI, RBB::gr(bb, G), m.p);
}

template <int LOGN>
struct StagedCfg32 {
  using PC = PairCfg32<LOGN>;
  static constexpr uint32_t kHalf = 1u << (LOGN - 1);
  static constexpr size_t kSmem = 3 * (size_t)kHalf * sizeof(uint32_t) + 16;  // W, S, mbarrier
  static constexpr int MIN_BLOCKS = (int)(228 * 1024 / (kSmem + 1024)) < PC::MIN_BLOCKS
                                        ? (int)(228 * 1024 / (kSmem + 1024))
                                        : PC::MIN_BLOCKS;
};

template <int LOGN>
__global__ void __cluster_dims__(2, 1, 1)
    __launch_bounds__(PairCfg32<LOGN>::C::THREADS, StagedCfg32<LOGN>::MIN_BLOCKS)
    k32_polymul_pair_staged(uint32_t* c, const uint32_t* a, const uint32_t* b, Limbs32 ls,
                            const DevMod32* __restrict__ mods) {
  namespace cg = cooperative_groups;
  using PC = PairCfg32<LOGN>;
  using C = typename PC::C;
  extern __shared__ __align__(128) uint32_t smem_st[];
  constexpr int H = C::K, NR = C::NR, E = 1 << C::LOGE;
  constexpr uint32_t log_n = H + 1, half = 1u << H;
  using RB = Round<C, NR - 1>;
  static_assert(RB::R == C::LOGE && RB::BETA == 0 && RB::EB == 0, "bottom round must own contiguous words");
  uint32_t* W = smem_st;             // a's tile, then a's parked NTT
  uint32_t* S = smem_st + half;      // raw limb (2 halves); b's tile after its stage 0
  uint64_t* mbar = reinterpret_cast<uint64_t*>(smem_st + 3 * half);
  cg::cluster_group cluster = cg::this_cluster();
  const uint32_t r = cluster.block_rank();
  const uint32_t limb = blockIdx.x >> 1;
  const uint32_t tid = threadIdx.x;
  const DevMod32 m = load_mod(mods, ls.cm(limb));
  const uint32_t p = m.p, p2 = p << 1;
  const uint2 w1 = __ldg(m.fwd + 1);
  const size_t lbase = (size_t)limb << log_n;
  const uint32_t bb = RB::base(tid);
  grid_dep_launch();
  grid_dep_wait();  // the stream's previous kernel may produce a or b, or read c
  if (tid == 0) {
    mbar_init(mbar, 1);
    mbar_expect(mbar, 2 * half * (uint32_t)sizeof(uint32_t));
    bulk_g2s(S, a + lbase, half * (uint32_t)sizeof(uint32_t), mbar);
    bulk_g2s(S + half, a + lbase + half, half * (uint32_t)sizeof(uint32_t), mbar);
  }
  __syncthreads();  // the mbarrier is initialised before anyone polls it
  mbar_wait32(mbar, 0);
  stage0_from_smem<PC, false>(W, S, S + half, tid, r, p, w1);
  if (tid == 0) {
    // S was read through the generic proxy; the copies write it through the async one
    fence_proxy_async();
    mbar_expect(mbar, 2 * half * (uint32_t)sizeof(uint32_t));
    bulk_g2s(S, b + lbase, half * (uint32_t)sizeof(uint32_t), mbar);
    bulk_g2s(S + half, b + lbase + half, half * (uint32_t)sizeof(uint32_t), mbar);
  }
  uint32_t x[E];
  pair_forward_rounds<PC>(x, W, tid, r, m);
  // park a's words (in [0, 2p)) where its bottom round read them (only this thread's positions)
#pragma unroll
  for (int i = 0; i < E; ++i) x[i] = csub(x[i], p2);
  smem_store<RB>(x, W, bb);
  mbar_wait32(mbar, 1);
  stage0_from_smem<PC, true>(S, S, S + half, tid, r, p, w1);
  pair_forward_rounds<PC>(x, S, tid, r, m);
  {
    const uint32_t ib = Smem<uint32_t>::idx(bb);
#pragma unroll
    for (int i = 0; i < E; i += 4) {
      const uint4 ah = *reinterpret_cast<const uint4*>(W + (ib ^ (uint32_t)i));
      x[i] = mont_mul(ah.x, csub(x[i], p2), p, m.pn);
      x[i + 1] = mont_mul(ah.y, csub(x[i + 1], p2), p, m.pn);
      x[i + 2] = mont_mul(ah.z, csub(x[i + 2], p2), p, m.pn);
      x[i + 3] = mont_mul(ah.w, csub(x[i + 3], p2), p, m.pn);
    }
  }
  pair_inverse<PC>(x, S, tid, r, bb, m);
  cluster.sync();
  pair_last_layer<PC, true>(c + lbase + r * half, S, cluster.map_shared_rank(S, (int)(r ^ 1u)), tid, r, m);
  cluster.sync();  // the peer may still be reading this CTA's shared memory
}

// In-place NTT of one limb by a CTA pair (DIR: 0 forward, 1 forward lazy,
// 2 backward), same split as k32_polymul_pair.
template <class PC, int DIR>
__global__ void __cluster_dims__(2, 1, 1) __launch_bounds__(PC::C::THREADS, PC::MIN_BLOCKS)
    k32_ntt_pair(uint32_t* data, Limbs32 ls, const DevMod32* __restrict__ mods) {
  namespace cg = cooperative_groups;
  using C = typename PC::C;
  using S = typename PC::S;
  extern __shared__ __align__(16) uint32_t smem32[];
  constexpr int H = C::K, NR = C::NR, E = 1 << C::LOGE;
  constexpr uint32_t log_n = H + 1, half = 1u << H;
  constexpr int IT = (int)(half / (C::THREADS * 4));
  using RB = Round<C, NR - 1>;
  cg::cluster_group cluster = cg::this_cluster();
  const uint32_t r = cluster.block_rank();
  const uint32_t limb = blockIdx.x >> 1;
  const uint32_t tid = threadIdx.x;
  const DevMod32 m = load_mod(mods, ls.cm(limb));
  const uint32_t p = m.p, p2 = p << 1;
  uint32_t* base = data + ((size_t)limb << log_n);
  if constexpr (DIR != 2) {
    uint32_t x[E];
    pair_forward<PC, true>(x, base, smem32, tid, r, m, __ldg(m.fwd + 1));
    uint32_t* out = base + r * half + RB::base(tid);
#pragma unroll
    for (int i = 0; i < E; i += 4) {
      uint4 v = make_uint4(x[i], x[i + 1], x[i + 2], x[i + 3]);
      if (DIR == 0) v = make_uint4(fwd_correct(v.x, p, p2), fwd_correct(v.y, p, p2), fwd_correct(v.z, p, p2),
                                   fwd_correct(v.w, p, p2));
      *reinterpret_cast<uint4*>(out + i) = v;
    }
  } else {
    const uint32_t* own = base + r * half;
#pragma unroll 1
    for (int i = 0; i < IT; ++i) {
      const uint32_t v = (tid + i * C::THREADS) * 4;
      *reinterpret_cast<uint4*>(smem32 + Smem<uint32_t>::idx(v)) = __ldg(reinterpret_cast<const uint4*>(own + v));
    }
    __syncthreads();
    {
      using CA = typename S::CA;
      using CB = typename S::CB;
      const uint32_t G = S::row_group(r, tid);
      inv_rounds<CB, CB::NR - 1, 0, false, CB::LOCAL_BARRIER>(smem32, tid, log_n, 0, G, m, true);
      inv_rounds<CB, 0, -1, false>(smem32, tid, log_n, 0, G, m, true);  // CTA barrier after
      inv_rounds<CA, CA::NR - 1, -1, false>(smem32, tid, log_n, S::KB, r, m, true);
    }
    cluster.sync();
    pair_last_layer<PC, false>(base + r * half, smem32, cluster.map_shared_rank(smem32, (int)(r ^ 1u)), tid, r, m);
    cluster.sync();
  }
}

template <int OP>
__global__ void k32_elementwise(uint32_t* dst, const uint32_t* a, const uint32_t* b, size_t total, uint32_t log_n,
                                Limbs32 ls, const DevMod32* __restrict__ mods) {
  for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < total; k += (size_t)gridDim.x * blockDim.x) {
    const uint32_t cm = ls.cm((uint32_t)(k >> log_n));
    const uint32_t p = __ldg(&mods[cm].p);
    if constexpr (OP == YELL_OP_MULMOD) dst[k] = mulmod_barrett(a[k], b[k], p, __ldg(&mods[cm].pn));
    else if constexpr (OP == YELL_OP_ADDMOD) dst[k] = addmod(a[k], b[k], p);
    else if constexpr (OP == YELL_OP_SUBMOD) dst[k] = submod(a[k], b[k], p);
    else if constexpr (OP == YELL_OP_MULADD) dst[k] = muladd_barrett(dst[k], a[k], b[k], p, __ldg(&mods[cm].pn));
    else dst[k] = p - a[k];
  }
}

// ---- launch ----------------------------------------------------------------------
// Degrees whose polymul runs on a CTA pair, with staged operands
// (k32_polymul_pair_staged; measured on GB300 at L = 32 and 2^20 words per
// operand: 2^15 203.6 us against 223.3 us for k32_polymul_pair, 2^14 176.4
// against 195.9 us).
constexpr int kMinPairLogN = 14;
constexpr int kStagedMinLogN = 14;
// Host-pointer calls up to this degree (single-CTA kernels) run in place on
// the context's pinned, device-mapped host buffer.
constexpr uint32_t kSmallCall32LogN = 13;

template <int LOGN>
cudaError_t set_attrs32() {
  using C = typename Cfg32<LOGN>::C;
  const int smem = (int)Cfg32<LOGN>::kSmem;
  cudaError_t e = cudaSuccess;
  for (auto k : {k32_ntt<C, 0>, k32_ntt<C, 1>, k32_ntt<C, 2>})
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  if (e == cudaSuccess) e = cudaFuncSetAttribute(k32_polymul<C>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  if constexpr (LOGN >= kMinPairLogN) {
    using PC = PairCfg32<LOGN>;
    using NC = NttPairCfg32<LOGN>;
    for (auto k : {k32_ntt_pair<NC, 0>, k32_ntt_pair<NC, 1>, k32_ntt_pair<NC, 2>})
      if (e == cudaSuccess) e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)NC::kSmem);
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(k32_polymul_pair<PC>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)PC::kSmem);
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(k32_polymul_pair_staged<LOGN>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)StagedCfg32<LOGN>::kSmem);
  }
  return e;
}

template <int LOGN>
cudaError_t launch32(int kind, uint32_t* c, const uint32_t* a, const uint32_t* b, const Limbs32& ls,
                     const DevMod32* mods, cudaStream_t st) {
  using CF = Cfg32<LOGN>;
  using C = typename CF::C;
  const uint32_t blocks = (ls.count + (1u << (C::T - LOGN)) - 1) >> (C::T - LOGN);
  if (kind == 3) mods += kMaxModuli32;  // the fused polymul's copy of the constants
  if constexpr (LOGN >= kMinPairLogN) {
    using PC = PairCfg32<LOGN>;
    using P = typename PC::C;
    using NC = NttPairCfg32<LOGN>;
    using NP = typename NC::C;
    const uint32_t g = 2 * ls.count;
    if (kind == 0) k32_ntt_pair<NC, 0><<<g, NP::THREADS, NC::kSmem, st>>>(c, ls, mods);
    else if (kind == 1) k32_ntt_pair<NC, 1><<<g, NP::THREADS, NC::kSmem, st>>>(c, ls, mods);
    else if (kind == 2) k32_ntt_pair<NC, 2><<<g, NP::THREADS, NC::kSmem, st>>>(c, ls, mods);
    else if (LOGN >= kStagedMinLogN)  // a programmatic dependent of the stream's previous kernel
      launch_dependent(k32_polymul_pair_staged<LOGN>, g, P::THREADS, StagedCfg32<LOGN>::kSmem, st, c, a, b, ls,
                       mods);
    else k32_polymul_pair<PC><<<g, P::THREADS, PC::kSmem, st>>>(c, a, b, ls, mods);
    return cudaGetLastError();
  }
  if (kind == 0) k32_ntt<C, 0><<<blocks, C::THREADS, CF::kSmem, st>>>(c, ls, mods);
  else if (kind == 1) k32_ntt<C, 1><<<blocks, C::THREADS, CF::kSmem, st>>>(c, ls, mods);
  else if (kind == 2) k32_ntt<C, 2><<<blocks, C::THREADS, CF::kSmem, st>>>(c, ls, mods);
  else k32_polymul<C><<<blocks, C::THREADS, CF::kSmem, st>>>(c, a, b, ls, mods);
  return cudaGetLastError();
}

template <int... L>
cudaError_t dispatch32(std::integer_sequence<int, L...>, uint32_t log_n, int kind, uint32_t* c, const uint32_t* a,
                       const uint32_t* b, const Limbs32& ls, const DevMod32* mods, cudaStream_t st) {
  cudaError_t e = cudaErrorInvalidValue;
  ((log_n == (uint32_t)(L + kMinLogN32) ? (e = launch32<L + kMinLogN32>(kind, c, a, b, ls, mods, st), 0) : 0), ...);
  return e;
}

template <int... L>
cudaError_t attrs32(std::integer_sequence<int, L...>) {
  cudaError_t e = cudaSuccess;
  ((e = (e == cudaSuccess ? set_attrs32<L + kMinLogN32>() : e)), ...);
  return e;
}

using Degrees32 = std::make_integer_sequence<int, kLogMaxDegree32 - kMinLogN32 + 1>;

int prepare32(uint32_t log_n, uint32_t cm0, uint32_t L, DeviceContext** ctx, const DevMod32** mods) {
  if (log_n < kMinLogN32 || log_n > kLogMaxDegree32)
    return fail(kUnsupportedDegree, "32-bit moduli: log_n must be in [3, 15]");
  if (L == 0 || cm0 >= kMaxModuli32 || L > kMaxModuli32 - cm0)
    return fail(kInvalidModulus, "32-bit moduli: indices must lie in [0, 291)");
  int st = kOk;
  *ctx = DeviceContext::current(&st);
  if (!*ctx) return st;
  {
    static std::mutex mu;
    static std::vector<int> done;
    std::lock_guard<std::mutex> g(mu);
    const int dev = (*ctx)->device();
    if (std::find(done.begin(), done.end(), dev) == done.end()) {
      const cudaError_t e = attrs32(Degrees32{});
      if (e != cudaSuccess) return fail_cuda(e, "32-bit kernel attributes");
      done.push_back(dev);
    }
  }
  return ensure32((*ctx)->device(), log_n, cm0, L, mods);
}

int aligned16(const void* p, const char* what) {
  return reinterpret_cast<uintptr_t>(p) % 16 ? fail(kInvalidArgument, std::string(what) + " is not 16-byte aligned")
                                             : kOk;
}

int run32(int kind, uint32_t* c, const uint32_t* a, const uint32_t* b, uint32_t count, uint32_t L, uint32_t log_n,
          uint32_t cm0, void* stream) {
  DeviceContext* ctx;
  const DevMod32* mods;
  int st = check_limbs(count, L, log_n, nullptr);
  if (st != kOk) return st;
  st = prepare32(log_n, cm0, L, &ctx, &mods);
  if (st != kOk) return st;
  if ((st = aligned16(c, "output")) != kOk) return st;
  if (a && (st = aligned16(a, "a")) != kOk) return st;
  if (b && (st = aligned16(b, "b")) != kOk) return st;
  const Limbs32 ls{count * L, L, cm0};
  cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : ctx->stream();
  static const char* names[4] = {"ntt32_forward", "ntt32_forward_lazy", "ntt32_backward", "polymul32"};
  LaunchScope ps(names[kind], s);
  const cudaError_t e = dispatch32(Degrees32{}, log_n, kind, c, a, b, ls, mods, s);
  g_kernel_launches += 1;
  return e == cudaSuccess ? kOk : fail_cuda(e, names[kind]);
}

// Host-memory single-limb transform through the staging buffer.
int host_ntt32(int kind, uint32_t* op, uint32_t log_n, uint32_t cm) {
  if (!op) return fail(kInvalidArgument, "null pointer");
  DeviceContext* ctx;
  const DevMod32* mods;
  int st = prepare32(log_n, cm, 1, &ctx, &mods);
  if (st != kOk) return st;
  const size_t n = (size_t)1 << log_n;
  cudaStream_t s = ctx->stream();
  if (log_n <= kSmallCall32LogN) {
    // small call: one single-CTA launch in place on the mapped host buffer
    std::lock_guard<std::mutex> g(ctx->small.lock);
    st = ctx->small.ensure();
    if (st != kOk) return st;
    uint32_t* h = reinterpret_cast<uint32_t*>(ctx->small.host);
    std::memcpy(h, op, n * 4);
    st = run32(kind, reinterpret_cast<uint32_t*>(ctx->small.dev), nullptr, nullptr, 1, 1, log_n, cm, s);
    if (st != kOk) return st;
    const cudaError_t e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return fail_cuda(e, "synchronize");
    std::memcpy(op, h, n * 4);
    return kOk;
  }
  std::lock_guard<std::mutex> g(ctx->staging.lock);
  st = ctx->staging.reserve(n);
  if (st != kOk) return st;
  uint32_t* d = reinterpret_cast<uint32_t*>(ctx->staging.ptr);
  cudaError_t e = cudaMemcpyAsync(d, op, n * 4, cudaMemcpyHostToDevice, s);
  if (e != cudaSuccess) return fail_cuda(e, "H2D");
  st = run32(kind, d, nullptr, nullptr, 1, 1, log_n, cm, s);
  if (st != kOk) return st;
  e = cudaMemcpyAsync(op, d, n * 4, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  return e == cudaSuccess ? kOk : fail_cuda(e, "D2H");
}

}  // namespace
}  // namespace yell_gb300

using namespace yell_gb300;

extern "C" {

uint32_t yell32_max_moduli(void) { return kMaxModuli32; }
uint32_t yell32_max_log_degree(void) { return kLogMaxDegree32; }
uint32_t yell32_prime(uint32_t cm) { return cm < kMaxModuli32 ? primes32()[cm].p : 0; }
uint32_t yell32_prime_pn(uint32_t cm) { return cm < kMaxModuli32 ? primes32()[cm].pn : 0; }
uint32_t yell32_primitive_root(uint32_t cm) { return cm < kMaxModuli32 ? primes32()[cm].root : 0; }

int yell32_ntt_tables(uint32_t log_n, uint32_t cm, uint32_t* out4n, uint32_t* scalars4) {
  if (!out4n || !scalars4) return fail(kInvalidArgument, "null output");
  if (log_n < 1 || log_n > kLogMaxDegree32) return fail(kUnsupportedDegree, "log_n must be in [1, 15]");
  if (cm >= kMaxModuli32) return fail(kInvalidModulus, "modulus index out of range");
  build_host_tables32(log_n, cm, out4n, scalars4);
  return kOk;
}

int yell32_init_ntt_tables(uint32_t log_n, uint32_t cm0, uint32_t L) {
  DeviceContext* ctx;
  const DevMod32* mods;
  return prepare32(log_n, cm0, L, &ctx, &mods);
}

int yell32_ntt_forward(uint32_t* op, uint32_t log_n, uint32_t cm) { return host_ntt32(0, op, log_n, cm); }
int yell32_ntt_forward_lazy(uint32_t* op, uint32_t log_n, uint32_t cm) { return host_ntt32(1, op, log_n, cm); }
int yell32_ntt_backward(uint32_t* op, uint32_t log_n, uint32_t cm) { return host_ntt32(2, op, log_n, cm); }

int yell32_dev_ntt(uint32_t* d_polys, uint32_t count, uint32_t L, uint32_t log_n, uint32_t cm0, int direction,
                   void* stream) {
  if (!d_polys || count == 0) return fail(kInvalidArgument, "null pointer or zero count");
  if (direction < 0 || direction > 2) return fail(kInvalidArgument, "bad direction");
  return run32(direction, d_polys, nullptr, nullptr, count, L, log_n, cm0, stream);
}

int yell32_dev_polymul(uint32_t* d_c, const uint32_t* d_a, const uint32_t* d_b, uint32_t pairs, uint32_t L,
                       uint32_t log_n, uint32_t cm0, void* stream) {
  if (!d_c || !d_a || !d_b || pairs == 0) return fail(kInvalidArgument, "null pointer or zero pairs");
  if (d_c == d_a || d_c == d_b) return fail(kInvalidArgument, "the product may not overwrite an operand");
  return run32(3, d_c, d_a, d_b, pairs, L, log_n, cm0, stream);
}

int yell32_wait_check(uint64_t timeout_ns, uint32_t* status) {
  if (!status) return fail(kInvalidArgument, "null output");
  if (timeout_ns == 0 || timeout_ns > 10'000'000'000ull) return fail(kInvalidArgument, "timeout must be in (0, 10 s]");
  int st = kOk;
  DeviceContext* ctx = DeviceContext::current(&st);
  if (!ctx) return st;
  k32_wait_check<<<1, 32, 0, ctx->stream()>>>(timeout_ns);
  g_kernel_launches += 1;
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return fail_cuda(e, "wait check");
  return yell32_wait_status(status);
}

int yell32_wait_status(uint32_t* status) {
  if (!status) return fail(kInvalidArgument, "null output");
  int st = kOk;
  DeviceContext* ctx = DeviceContext::current(&st);
  if (!ctx) return st;
  cudaError_t e = cudaDeviceSynchronize();
  if (e != cudaSuccess) return fail_cuda(e, "synchronize");
  uint32_t v = 0;
  e = cudaMemcpyFromSymbol(&v, g_k32_wait_status, sizeof(v));
  if (e != cudaSuccess) return fail_cuda(e, "read wait status");
  if (v != 0) {
    const uint32_t zero = 0;
    e = cudaMemcpyToSymbol(g_k32_wait_status, &zero, sizeof(zero));
    if (e != cudaSuccess) return fail_cuda(e, "clear wait status");
  }
  *status = v;
  return kOk;
}

int yell32_dev_elementwise(int op, uint32_t* d_dst, const uint32_t* d_a, const uint32_t* d_b, uint32_t count,
                           uint32_t L, uint32_t log_n, uint32_t cm0, void* stream) {
  if (!d_dst || !d_a || (op != YELL_OP_NEGATE && !d_b) || count == 0)
    return fail(kInvalidArgument, "null pointer or zero count");
  if (op < YELL_OP_MULMOD || op > YELL_OP_NEGATE) return fail(kInvalidArgument, "bad op");
  DeviceContext* ctx;
  const DevMod32* mods;
  int st = check_limbs(count, L, log_n, nullptr);
  if (st != kOk) return st;
  st = prepare32(log_n, cm0, L, &ctx, &mods);
  if (st != kOk) return st;
  cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : ctx->stream();
  const size_t total = ((size_t)count * L) << log_n;
  const Limbs32 ls{count * L, L, cm0};
  const int grid = (int)std::min<size_t>((total + 255) / 256, 152 * 16);
  LaunchScope ps("elementwise32", s);
  switch (op) {
    case YELL_OP_MULMOD: k32_elementwise<YELL_OP_MULMOD><<<grid, 256, 0, s>>>(d_dst, d_a, d_b, total, log_n, ls, mods); break;
    case YELL_OP_ADDMOD: k32_elementwise<YELL_OP_ADDMOD><<<grid, 256, 0, s>>>(d_dst, d_a, d_b, total, log_n, ls, mods); break;
    case YELL_OP_SUBMOD: k32_elementwise<YELL_OP_SUBMOD><<<grid, 256, 0, s>>>(d_dst, d_a, d_b, total, log_n, ls, mods); break;
    case YELL_OP_MULADD: k32_elementwise<YELL_OP_MULADD><<<grid, 256, 0, s>>>(d_dst, d_a, d_b, total, log_n, ls, mods); break;
    default: k32_elementwise<YELL_OP_NEGATE><<<grid, 256, 0, s>>>(d_dst, d_a, d_b, total, log_n, ls, mods); break;
  }
  g_kernel_launches += 1;
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? kOk : fail_cuda(e, "elementwise32");
}

// ---- host-memory poly<N> drop-ins (limb pointer arrays, moduli 0 .. L-1) ----
// The reference's poly<N> members in 32-bit mode (details/poly.hpp:118-186 and
// the operators of include/yell/poly.hpp:163-168): limbs staged through device memory,
// one launch over all limbs, copied back; synchronous.

static int host_poly32(int kind, int op, uint32_t* const* dst, const uint32_t* const* a, const uint32_t* const* b,
                       uint32_t L, uint32_t log_n) {
  // kind 0..2: NTT of dst in place; kind 3: element-wise op
  if (!dst || L == 0) return fail(kInvalidArgument, "null limb array or zero limbs");
  const bool binary = kind == 3 && op != YELL_OP_NEGATE;
  if (kind == 3 && (!a || (binary && !b))) return fail(kInvalidArgument, "null limb array");
  for (uint32_t l = 0; l < L; ++l)
    if (!dst[l] || (kind == 3 && !a[l]) || (binary && !b[l])) return fail(kInvalidArgument, "null limb pointer");
  DeviceContext* ctx;
  const DevMod32* mods;
  int st = prepare32(log_n, 0, L, &ctx, &mods);
  if (st != kOk) return st;
  const size_t n = (size_t)1 << log_n, w = n * L;
  cudaStream_t s = ctx->stream();
  const bool need_dst = kind != 3 || op == YELL_OP_MULADD;
  if (log_n <= kSmallCall32LogN && w <= 2 * DeviceContext::kSmallCallWords) {
    // small call: the kernel works on the mapped host buffer (three operands
    // of w 32-bit words fit its 3 x kSmallCallWords 64-bit words)
    std::lock_guard<std::mutex> g(ctx->small.lock);
    st = ctx->small.ensure();
    if (st != kOk) return st;
    uint32_t* hd = reinterpret_cast<uint32_t*>(ctx->small.host);
    uint32_t* ha = hd + w;
    uint32_t* hb = ha + w;
    for (uint32_t l = 0; l < L; ++l) {
      if (need_dst) std::memcpy(hd + l * n, dst[l], n * 4);
      if (kind == 3) std::memcpy(ha + l * n, a[l], n * 4);
      if (binary) std::memcpy(hb + l * n, b[l], n * 4);
    }
    uint32_t* vd = reinterpret_cast<uint32_t*>(ctx->small.dev);
    st = kind == 3 ? yell32_dev_elementwise(op, vd, vd + w, binary ? vd + 2 * w : nullptr, 1, L, log_n, 0, s)
                   : run32(kind, vd, nullptr, nullptr, 1, L, log_n, 0, s);
    if (st != kOk) return st;
    const cudaError_t e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return fail_cuda(e, "synchronize");
    for (uint32_t l = 0; l < L; ++l) std::memcpy(dst[l], hd + l * n, n * 4);
    return kOk;
  }
  std::lock_guard<std::mutex> g(ctx->staging.lock);
  st = ctx->staging.reserve((3 * w + 1) / 2);  // three uint32 operands in uint64 words
  if (st != kOk) return st;
  uint32_t* dd = reinterpret_cast<uint32_t*>(ctx->staging.ptr);
  uint32_t* da = dd + w;
  uint32_t* db = da + w;
  cudaError_t e = cudaSuccess;
  for (uint32_t l = 0; l < L && e == cudaSuccess; ++l) {
    if (need_dst) e = cudaMemcpyAsync(dd + l * n, dst[l], n * 4, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess && kind == 3) e = cudaMemcpyAsync(da + l * n, a[l], n * 4, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess && binary) e = cudaMemcpyAsync(db + l * n, b[l], n * 4, cudaMemcpyHostToDevice, s);
  }
  if (e != cudaSuccess) return fail_cuda(e, "H2D limbs");
  st = kind == 3 ? yell32_dev_elementwise(op, dd, da, binary ? db : nullptr, 1, L, log_n, 0, s)
                 : run32(kind, dd, nullptr, nullptr, 1, L, log_n, 0, s);
  if (st != kOk) return st;
  for (uint32_t l = 0; l < L && e == cudaSuccess; ++l)
    e = cudaMemcpyAsync(dst[l], dd + l * n, n * 4, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  return e == cudaSuccess ? kOk : fail_cuda(e, "D2H limbs");
}

int yell32_poly_forward(uint32_t* const* limbs, uint32_t L, uint32_t log_n) {
  return host_poly32(0, 0, limbs, nullptr, nullptr, L, log_n);
}
int yell32_poly_forward_lazy(uint32_t* const* limbs, uint32_t L, uint32_t log_n) {
  return host_poly32(1, 0, limbs, nullptr, nullptr, L, log_n);
}
int yell32_poly_backward(uint32_t* const* limbs, uint32_t L, uint32_t log_n) {
  return host_poly32(2, 0, limbs, nullptr, nullptr, L, log_n);
}
int yell32_poly_mulmod(uint32_t* const* dst, const uint32_t* const* a, const uint32_t* const* b, uint32_t L,
                       uint32_t log_n) {
  return host_poly32(3, YELL_OP_MULMOD, dst, a, b, L, log_n);
}
int yell32_poly_addmod(uint32_t* const* dst, const uint32_t* const* a, const uint32_t* const* b, uint32_t L,
                       uint32_t log_n) {
  return host_poly32(3, YELL_OP_ADDMOD, dst, a, b, L, log_n);
}
int yell32_poly_submod(uint32_t* const* dst, const uint32_t* const* a, const uint32_t* const* b, uint32_t L,
                       uint32_t log_n) {
  return host_poly32(3, YELL_OP_SUBMOD, dst, a, b, L, log_n);
}
int yell32_poly_add_product_of(uint32_t* const* acc, const uint32_t* const* a, const uint32_t* const* b, uint32_t L,
                               uint32_t log_n) {
  return host_poly32(3, YELL_OP_MULADD, acc, a, b, L, log_n);
}
int yell32_poly_negate(uint32_t* const* limbs, uint32_t L, uint32_t log_n) {
  return host_poly32(3, YELL_OP_NEGATE, limbs, limbs, nullptr, L, log_n);
}

}  // extern "C"
