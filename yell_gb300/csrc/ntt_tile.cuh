// Tile engine shared by every NTT kernel.
//
// A CTA holds a tile of 2^T uint64 words in shared memory.  The transform
// acts on the bit range [lb, lb + K) of the tile index v ("u" bits); the other
// bits select independent sub-transforms (columns below lb, blocks or limbs
// above lb + K).  Each thread owns E = 2^LOGE words per round and applies R
// consecutive radix-2 stages to them in registers; rounds exchange through
// shared memory.  The butterflies, their order within a dependency chain and
// their twiddle indices are exactly the reference's (lib/ntt.cpp:89-210), so
// the lazy words produced are identical to the reference's, not only
// congruent: a radix-2 butterfly is a pure function of its two inputs and its
// twiddle, and every butterfly here sees the same inputs as its reference
// counterpart.
//
// Twiddle indices.  Forward stage s (m = 2^s groups, half-size h = N/2^(s+1))
// uses w[m + (i >> (log_n - s))] for the pair at global index i
// (lib/ntt.cpp:105-110).  Inverse stage sigma (h = 2^sigma,
// m = N/2^(sigma+1)) uses w[m + (i >> (sigma + 1))] (lib/ntt.cpp:193-198).
// Inside a round both reduce to a per-thread group number gr plus the top
// bits of the in-register index j, worked out in ct_round/gs_round below.
#pragma once
#include "common.cuh"

namespace yell_gb300 {

// One pad word after every 16 words: rows of 16 words shift by two banks,
// which keeps the strided per-thread access of the low-bit rounds at the
// two-wavefront minimum for 8-byte accesses.
constexpr uint32_t kPadShift = 4;
__device__ __forceinline__ uint32_t sidx(uint32_t v) { return v + (v >> kPadShift); }
__host__ __device__ constexpr uint32_t padded_words(uint32_t n) { return n + (n >> kPadShift); }

// Round split of a K-stage transform into rounds of at most LOGE stages.  The
// round on the lowest u bits always has LOGE stages, so every other round has
// beta >= LOGE and can take its (LOGE - R) extra in-register bits from the
// lowest u bits.  Forward rounds run from the top bits down (CT, stage 0 has
// the largest distance); inverse rounds run from the bottom up (GS).
struct RoundPlan {
  uint32_t n;     // number of rounds
  uint32_t q;     // base width of the rounds above the bottom one
  uint32_t rem;   // the first `rem` of those are one stage wider
  uint32_t K;
  uint32_t loge;
  bool inverse;

  // Width R and lowest butterfly bit beta of round r in execution order.
  __device__ __forceinline__ void geom(uint32_t r, uint32_t& R, uint32_t& beta) const {
    const uint32_t i = inverse ? n - 1 - r : r;   // index counted from the top bits
    if (i + 1 == n) {
      R = (n == 1) ? K : loge;
      beta = 0;
    } else {
      R = q + (i < rem ? 1u : 0u);
      beta = K - (i + 1) * q - ((i + 1) < rem ? (i + 1) : rem);
    }
  }
};

__device__ __forceinline__ RoundPlan make_plan(uint32_t K, uint32_t LOGE, bool inverse) {
  RoundPlan pl;
  pl.n = (K + LOGE - 1) / LOGE;
  pl.K = K;
  pl.loge = LOGE;
  pl.inverse = inverse;
  if (pl.n > 1) {
    const uint32_t rest = K - LOGE;
    pl.q = rest / (pl.n - 1);
    pl.rem = rest % (pl.n - 1);
  } else {
    pl.q = K;
    pl.rem = 0;
  }
  return pl;
}

// Tile index of this thread's element (ex = 0, j = 0) in a round with
// butterfly bits [beta, beta + R) and extra bits [0, LOGE - R) of u.  The
// thread id fills the remaining tile bits in increasing order, so consecutive
// lanes take consecutive columns (bits below lb) first.
template <int LOGE, int R>
__device__ __forceinline__ uint32_t thread_base(uint32_t tid, uint32_t lb, uint32_t beta) {
  constexpr uint32_t e = LOGE - R;
  const uint32_t mid = beta - e;
  uint32_t v = tid & ((1u << lb) - 1u);
  v |= ((tid >> lb) & ((1u << mid) - 1u)) << (lb + e);
  v |= (tid >> (lb + mid)) << (lb + beta + R);
  return v;
}

template <int LOGE, int R>
__device__ __forceinline__ void load_regs(uint64_t* x, const uint64_t* s, uint32_t base, uint32_t lb,
                                          uint32_t beta) {
  constexpr int E = 1 << (LOGE - R);
#pragma unroll
  for (int ex = 0; ex < E; ++ex)
#pragma unroll
    for (int j = 0; j < (1 << R); ++j)
      x[(ex << R) | j] = s[sidx(base + ((uint32_t)ex << lb) + ((uint32_t)j << (lb + beta)))];
}

template <int LOGE, int R>
__device__ __forceinline__ void store_regs(const uint64_t* x, uint64_t* s, uint32_t base, uint32_t lb,
                                           uint32_t beta) {
  constexpr int E = 1 << (LOGE - R);
#pragma unroll
  for (int ex = 0; ex < E; ++ex)
#pragma unroll
    for (int j = 0; j < (1 << R); ++j)
      s[sidx(base + ((uint32_t)ex << lb) + ((uint32_t)j << (lb + beta)))] = x[(ex << R) | j];
}

// Forward (CT) round on registers.  s_first: absolute stage of the round's
// first sub-stage.  gr: group number of this thread at stage s_first.  At
// sub-stage k the pair (j, j + 2^(R-1-k)) uses twiddle
// w[2^(s_first+k) + (gr << k) + (j >> (R-k))].  Sub-stages recurse at compile
// time so every loop bound and register index is a constant.
template <int LOGE, int R, int k>
__device__ __forceinline__ void ct_stage(uint64_t* x, uint32_t s_first, uint32_t gr,
                                         const ulonglong2* __restrict__ tw, uint64_t p, uint64_t p2) {
  if constexpr (k < R) {
    constexpr int E = 1 << (LOGE - R);
    constexpr int d = 1 << (R - 1 - k);
    constexpr int NJ = 1 << k;
    const uint32_t tbase = (1u << (s_first + k)) + (gr << k);
#pragma unroll
    for (int jj = 0; jj < NJ; ++jj) {
      const ulonglong2 w = __ldg(tw + tbase + jj);
#pragma unroll
      for (int ex = 0; ex < E; ++ex)
#pragma unroll
        for (int q = 0; q < d; ++q) {
          const int j = jj * 2 * d + q;
          ct_bfly(x[(ex << R) | j], x[(ex << R) | (j + d)], w.x, w.y, p, p2);
        }
    }
    ct_stage<LOGE, R, k + 1>(x, s_first, gr, tw, p, p2);
  }
}

template <int LOGE, int R>
__device__ __forceinline__ void ct_round(uint64_t* x, uint32_t s_first, uint32_t gr,
                                         const ulonglong2* __restrict__ tw, uint64_t p, uint64_t p2) {
  ct_stage<LOGE, R, 0>(x, s_first, gr, tw, p, p2);
}

// Inverse (GS) round on registers.  sigma_first: absolute inverse stage of
// the first sub-stage (pair distance 2^sigma in the global index).  At
// sub-stage k the pair (j, j + 2^k) uses twiddle
// w[2^(log_n-1-sigma) + (gr << (R-1-k)) + (j >> (k+1))].  With LAST, the
// round's final sub-stage is the reference's last layer with the N^-1
// scaling fused (include/yell/details/ntt.hpp:220-228) instead of a GS stage.
template <int LOGE, int R, bool LAST, int k>
__device__ __forceinline__ void gs_stage(uint64_t* x, uint32_t log_n, uint32_t sigma_first,
                                         uint32_t gr, const ulonglong2* __restrict__ itw,
                                         const DevMod& m) {
  if constexpr (k < R) {
    constexpr int E = 1 << (LOGE - R);
    constexpr int d = 1 << k;
    if constexpr (LAST && k == R - 1) {
#pragma unroll
      for (int ex = 0; ex < E; ++ex)
#pragma unroll
        for (int q = 0; q < d; ++q) gs_last(x[(ex << R) | q], x[(ex << R) | (q + d)], m);
    } else {
      constexpr int NJ = 1 << (R - 1 - k);
      const uint64_t p = m.p, p2 = m.p << 1;
      const uint32_t tbase = (1u << (log_n - 1 - (sigma_first + k))) + (gr << (R - 1 - k));
#pragma unroll
      for (int jj = 0; jj < NJ; ++jj) {
        const ulonglong2 w = __ldg(itw + tbase + jj);
#pragma unroll
        for (int ex = 0; ex < E; ++ex)
#pragma unroll
          for (int q = 0; q < d; ++q) {
            const int j = jj * 2 * d + q;
            gs_bfly(x[(ex << R) | j], x[(ex << R) | (j + d)], w.x, w.y, p, p2);
          }
      }
      gs_stage<LOGE, R, LAST, k + 1>(x, log_n, sigma_first, gr, itw, m);
    }
  }
}

template <int LOGE, int R, bool LAST>
__device__ __forceinline__ void gs_round(uint64_t* x, uint32_t log_n, uint32_t sigma_first, uint32_t gr,
                                         const ulonglong2* __restrict__ itw, const DevMod& m) {
  gs_stage<LOGE, R, LAST, 0>(x, log_n, sigma_first, gr, itw, m);
}

// Reads the DevMod for modulus index cm with read-only loads.
__device__ __forceinline__ DevMod load_mod(const DevMod* __restrict__ mods, uint32_t cm) {
  DevMod m;
  const ulonglong2* src = reinterpret_cast<const ulonglong2*>(mods + cm);
  ulonglong2 a = __ldg(src), b = __ldg(src + 1), c = __ldg(src + 2), d = __ldg(src + 3);
  m.fwd = reinterpret_cast<const ulonglong2*>(a.x);
  m.inv = reinterpret_cast<const ulonglong2*>(a.y);
  m.p = b.x;
  m.pn = b.y;
  m.inv_n = c.x;
  m.inv_n_s = c.y;
  m.inv_n_iphi = d.x;
  m.inv_n_iphi_s = d.y;
  return m;
}

// Runs one forward round of the plan on the tile in shared memory.
//   lb, K     : position and width of the transform bits in the tile index
//   s_off     : absolute stage of the transform's u-bit K-1 (0 for a whole
//               NTT or a column pass, k1 for a row pass)
//   G         : group number of the sub-transform at stage s_off
//   active    : false for threads whose sub-transform is padding
template <int LOGE, int R>
__device__ __forceinline__ void fwd_round_smem(uint64_t* s, uint32_t tid, uint32_t lb, uint32_t K,
                                               uint32_t beta, uint32_t s_off, uint32_t G,
                                               const ulonglong2* tw, uint64_t p, bool active) {
  uint64_t x[1 << LOGE];
  const uint32_t base = thread_base<LOGE, R>(tid, lb, beta);
  if (active) {
    load_regs<LOGE, R>(x, s, base, lb, beta);
    const uint32_t hi_bits = K - beta - R;
    const uint32_t u_hi = (base >> (lb + beta + R)) & ((1u << hi_bits) - 1u);
    const uint32_t gr = (G << hi_bits) + u_hi;
    ct_round<LOGE, R>(x, s_off + hi_bits, gr, tw, p, p << 1);
    store_regs<LOGE, R>(x, s, base, lb, beta);
  }
}

// Inverse counterpart.  sig_off: absolute inverse stage of the transform's
// u-bit 0 (0 for a whole NTT or a row pass, log2(B) for a column pass).
template <int LOGE, int R, bool LAST>
__device__ __forceinline__ void inv_round_smem(uint64_t* s, uint32_t tid, uint32_t lb, uint32_t K,
                                               uint32_t beta, uint32_t log_n, uint32_t sig_off,
                                               uint32_t G, const DevMod& m, bool active) {
  uint64_t x[1 << LOGE];
  const uint32_t base = thread_base<LOGE, R>(tid, lb, beta);
  if (active) {
    load_regs<LOGE, R>(x, s, base, lb, beta);
    const uint32_t hi_bits = K - beta - R;
    const uint32_t u_hi = (base >> (lb + beta + R)) & ((1u << hi_bits) - 1u);
    const uint32_t gr = (G << hi_bits) + u_hi;
    gs_round<LOGE, R, LAST>(x, log_n, sig_off + beta, gr, m.inv, m);
    store_regs<LOGE, R>(x, s, base, lb, beta);
  }
}

// One forward round of width R (runtime) at bit beta, dispatched to the
// compile-time round.
template <int LOGE>
__device__ __forceinline__ void fwd_round(uint64_t* s, uint32_t tid, uint32_t lb, uint32_t K,
                                          uint32_t R, uint32_t beta, uint32_t s_off, uint32_t G,
                                          const ulonglong2* tw, uint64_t p, bool active) {
  switch (R) {
#define YELL_FWD_CASE(RR)                                                       \
  case RR:                                                                      \
    if constexpr (RR <= LOGE)                                                   \
      fwd_round_smem<LOGE, RR>(s, tid, lb, K, beta, s_off, G, tw, p, active);   \
    break;
    YELL_FWD_CASE(1)
    YELL_FWD_CASE(2)
    YELL_FWD_CASE(3)
    YELL_FWD_CASE(4)
#undef YELL_FWD_CASE
    default: break;
  }
}

template <int LOGE>
__device__ __forceinline__ void inv_round(uint64_t* s, uint32_t tid, uint32_t lb, uint32_t K,
                                          uint32_t R, uint32_t beta, uint32_t log_n,
                                          uint32_t sig_off, uint32_t G, const DevMod& m,
                                          bool active, bool last) {
  switch (R) {
#define YELL_INV_CASE(RR)                                                                   \
  case RR:                                                                                  \
    if constexpr (RR <= LOGE) {                                                             \
      if (last)                                                                             \
        inv_round_smem<LOGE, RR, true>(s, tid, lb, K, beta, log_n, sig_off, G, m, active);  \
      else                                                                                  \
        inv_round_smem<LOGE, RR, false>(s, tid, lb, K, beta, log_n, sig_off, G, m, active); \
    }                                                                                       \
    break;
    YELL_INV_CASE(1)
    YELL_INV_CASE(2)
    YELL_INV_CASE(3)
    YELL_INV_CASE(4)
#undef YELL_INV_CASE
    default: break;
  }
}

// All rounds of a forward transform over the tile (syncs between rounds).
// G is this thread's sub-transform group number at stage s_off; tw, p and
// active may differ per thread (per limb).  A thread's sub-transform is the
// same in every round: its tile bits above lb + K are tid >> (lb + K - LOGE).
template <int LOGE>
__device__ __forceinline__ void fwd_tile(uint64_t* s, uint32_t tid, uint32_t lb, uint32_t K,
                                         uint32_t s_off, uint32_t G, const ulonglong2* tw,
                                         uint64_t p, bool active) {
  const RoundPlan pl = make_plan(K, LOGE, false);
  for (uint32_t r = 0; r < pl.n; ++r) {
    uint32_t R, beta;
    pl.geom(r, R, beta);
    fwd_round<LOGE>(s, tid, lb, K, R, beta, s_off, G, tw, p, active);
    __syncthreads();
  }
}

// All rounds of an inverse transform over the tile.  With has_last, the
// final sub-stage is the scaled last layer (only when the tile's transform
// contains the global top bit).
template <int LOGE>
__device__ __forceinline__ void inv_tile(uint64_t* s, uint32_t tid, uint32_t lb, uint32_t K,
                                         uint32_t log_n, uint32_t sig_off, uint32_t G,
                                         const DevMod& m, bool active, bool has_last) {
  const RoundPlan pl = make_plan(K, LOGE, true);
  for (uint32_t r = 0; r < pl.n; ++r) {
    uint32_t R, beta;
    pl.geom(r, R, beta);
    inv_round<LOGE>(s, tid, lb, K, R, beta, log_n, sig_off, G, m, active,
                    has_last && (r + 1 == pl.n));
    __syncthreads();
  }
}

}  // namespace yell_gb300
