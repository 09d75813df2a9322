// Tile engine shared by every NTT kernel (all geometry known at compile time).
//
// A CTA owns a tile of 2^T uint64 words.  The transform acts on the bit range
// [LB, LB + K) of the tile index v (the "u" bits); the other bits select
// independent sub-transforms (columns below LB; blocks or limbs above
// LB + K).  Each thread owns 2^LOGE words per round and applies R consecutive
// radix-2 stages to them in registers; rounds exchange through shared memory.
// The butterflies, their pairing and their twiddle indices are exactly the
// reference's (lib/ntt.cpp:89-210), so the lazy words produced are identical
// to the reference's, not only congruent: a radix-2 butterfly is a pure
// function of its two inputs and its twiddle, and every butterfly here sees
// the same inputs as its reference counterpart.
//
// Rounds.  A K-stage transform is split into NR = ceil(K / LOGE) rounds.  The
// round on the lowest u bits always has LOGE stages, so every other round has
// beta >= LOGE and takes its LOGE - R extra in-register bits from the lowest
// u bits.  Forward (CT) rounds run from the top bits down, inverse (GS)
// rounds from the bottom up.  Round geometry is indexed by its position I
// counted from the top bits.
//
// Twiddle indices.  Forward stage s (m = 2^s groups, half-size N/2^(s+1))
// uses w[m + (i >> (log_n - s))] for the pair at global index i
// (lib/ntt.cpp:105-110); inverse stage sigma (pair distance 2^sigma,
// m = N/2^(sigma+1)) uses w[m + (i >> (sigma + 1))] (lib/ntt.cpp:193-198).
// Inside a round both reduce to a per-thread group number gr plus the top
// bits of the in-register index j.
//
// Shared memory layout: word v lives at v + 2*(v >> 4) (two pad words per
// 16), which keeps 16-byte alignment for adjacent pairs and spreads the
// strided accesses of the low-bit rounds across banks.
#pragma once
#include "common.cuh"

namespace yell_gb300 {

__host__ __device__ constexpr uint32_t sidx(uint32_t v) { return v + ((v >> 4) << 1); }
__host__ __device__ constexpr uint32_t tile_smem_words(uint32_t n) { return n + (n >> 3); }

// Shared-memory layout per word type.  64-bit words: sidx (2 pad words per
// 16), an additive map: idx(base + off) = idx(base) + idx(off) for the
// disjoint bit fields a round combines.  32-bit words: no padding; in each
// 32-word row, 4-word groups are XOR-swizzled by the row index (bits 2..4 ^=
// bits 5..7), a linear map over GF(2): idx(base ^ off) = idx(base) ^ idx(off),
// every 4-word group stays contiguous and 16-byte aligned, and contiguous,
// paired and 16-byte-per-lane accesses all spread over the 32 banks.
template <class W> struct Smem;
template <> struct Smem<uint64_t> {
  static constexpr bool kXor = false;
  __host__ __device__ static constexpr uint32_t idx(uint32_t v) { return sidx(v); }
  __host__ __device__ static constexpr uint32_t words(uint32_t n) { return tile_smem_words(n); }
};
template <> struct Smem<uint32_t> {
  static constexpr bool kXor = true;
  __host__ __device__ static constexpr uint32_t idx(uint32_t v) { return v ^ (((v >> 5) & 7u) << 2); }
  __host__ __device__ static constexpr uint32_t words(uint32_t n) { return n; }
};

template <int T_, int K_, int LB_, int LOGE_>
struct TileCfg {
  static constexpr int T = T_, K = K_, LB = LB_, LOGE = LOGE_;
  static constexpr int THREADS = 1 << (T - LOGE);
  static constexpr int NR = (K + LOGE - 1) / LOGE;
  static constexpr int Q = NR > 1 ? (K - LOGE) / (NR - 1) : K;
  static constexpr int REM = NR > 1 ? (K - LOGE) % (NR - 1) : 0;
  __host__ __device__ static constexpr int width(int i) { return (i + 1 == NR) ? (NR == 1 ? K : LOGE) : Q + (i < REM ? 1 : 0); }
  __host__ __device__ static constexpr int beta(int i) {
    return (i + 1 == NR) ? 0 : K - (i + 1) * Q - ((i + 1) < REM ? (i + 1) : REM);
  }
  // Tile bits above LB + K (sub-transform index) of thread tid.
  __device__ static __forceinline__ uint32_t sub(uint32_t tid) { return tid >> (LB + K - LOGE); }
  // A thread keeps its sub-transform in every round (the tid bits above the
  // lowest K - LOGE select it), so with contiguous sub-transforms (LB = 0)
  // every exchange between rounds stays among the GROUP threads of one
  // sub-transform.  The barrier between rounds for a caller that does no
  // CTA-wide staging around them: 1 = the warp's (GROUP <= 32), 2 = a named
  // barrier per sub-transform (at most 15 in the CTA), 0 = the CTA's.
  static constexpr int GROUP = 1 << (K - LOGE);
  static constexpr int LOCAL_BARRIER =
      LB != 0 ? 0 : (GROUP <= 32 ? 1 : ((GROUP < THREADS && THREADS / GROUP <= 15) ? 2 : 0));
  static_assert(K >= LOGE, "transform narrower than a thread's word set");
  static_assert(T >= K + LB, "tile smaller than one sub-transform");
};

// Geometry of round I of tile C.
template <class C, int I>
struct Round {
  static constexpr int R = C::width(I);
  static constexpr int BETA = C::beta(I);
  static constexpr int LB = C::LB, LOGE = C::LOGE, K = C::K;
  static constexpr int EB = LOGE - R;          // extra (non-butterfly) bits per thread
  static constexpr int E = 1 << EB;
  static constexpr int MID = BETA - EB;        // u bits between the extra and butterfly bits
  static constexpr int HI = K - BETA - R;      // u bits above the butterfly bits
  // Adjacent word pairs (ex = 2m, 2m+1) when the extra bits are the tile's
  // lowest bits: moved as one 16-byte access.
  static constexpr bool PAIRS = (LB == 0 && EB >= 1);
  // The bottom round of a row-type tile: each thread's words are 2^R
  // consecutive words, moved as 16-byte pairs.
  static constexpr bool CONTIG = (LB == 0 && EB == 0 && BETA == 0 && R >= 1);
  static_assert(MID >= 0, "round plan broke the extra-bits-below rule");

  // Tile index of the thread's element (ex = 0, j = 0): thread id bits fill
  // [0, LB), [LB + EB, LB + BETA) and [LB + BETA + R, T) in increasing order.
  __device__ static __forceinline__ uint32_t base(uint32_t tid) {
    uint32_t v = tid & ((1u << LB) - 1u);
    v |= ((tid >> LB) & ((1u << MID) - 1u)) << (LB + EB);
    v |= (tid >> (LB + MID)) << (LB + BETA + R);
    return v;
  }
  __host__ __device__ static constexpr uint32_t off(int ex, int j) {
    return ((uint32_t)ex << LB) + ((uint32_t)j << (LB + BETA));
  }
  // Group number at the round's first stage: sub-transform group G (at the
  // transform's top stage) followed by the u bits above the butterfly range.
  __device__ static __forceinline__ uint32_t gr(uint32_t base_v, uint32_t G) {
    return (G << HI) + ((base_v >> (LB + BETA + R)) & ((1u << HI) - 1u));
  }
};

// ---- register <-> shared memory ----------------------------------------------
// A 32-bit round whose thread owns 2^R consecutive words starting at a
// multiple of 16 (the bottom round of a row tile).
template <class RG, class W>
constexpr bool kContig32 = sizeof(W) == 4 && RG::EB == 0 && RG::BETA == 0 && RG::LB == 0 && RG::R >= 4;

template <class RG, class W>
__device__ __forceinline__ void smem_load(W* x, const W* s, uint32_t base_v) {
  constexpr int R = RG::R;
  using PW = typename PairOf<W>::type;
  using SL = Smem<W>;
  if constexpr (kContig32<RG, W>) {
    // base_v has no bits below 2^R (R >= 4): idx(base_v + j) = idx(base_v) ^ j
    const uint32_t ib = SL::idx(base_v);
#pragma unroll
    for (int j = 0; j < (1 << R); j += 4) {
      const uint4 v = *reinterpret_cast<const uint4*>(s + (ib ^ (uint32_t)j));
      x[j] = v.x;
      x[j + 1] = v.y;
      x[j + 2] = v.z;
      x[j + 3] = v.w;
    }
  } else if constexpr (SL::kXor) {
    const uint32_t ib = SL::idx(base_v);
    if constexpr (RG::PAIRS) {
#pragma unroll
      for (int m = 0; m < RG::E / 2; ++m)
#pragma unroll
        for (int j = 0; j < (1 << R); ++j) {
          const PW v = *reinterpret_cast<const PW*>(s + (ib ^ SL::idx(RG::off(2 * m, j))));
          x[((2 * m) << R) | j] = v.x;
          x[((2 * m + 1) << R) | j] = v.y;
        }
    } else {
#pragma unroll
      for (int ex = 0; ex < RG::E; ++ex)
#pragma unroll
        for (int j = 0; j < (1 << R); ++j) x[(ex << R) | j] = s[ib ^ SL::idx(RG::off(ex, j))];
    }
  } else if constexpr (RG::PAIRS) {
    // base_v and the offsets occupy disjoint bits, so idx(base_v + off) = idx(base_v) + idx(off)
    const W* sb = s + SL::idx(base_v);
#pragma unroll
    for (int m = 0; m < RG::E / 2; ++m)
#pragma unroll
      for (int j = 0; j < (1 << R); ++j) {
        const PW v = *reinterpret_cast<const PW*>(sb + SL::idx(RG::off(2 * m, j)));
        x[((2 * m) << R) | j] = v.x;
        x[((2 * m + 1) << R) | j] = v.y;
      }
  } else {
    const W* sb = s + SL::idx(base_v);
#pragma unroll
    for (int ex = 0; ex < RG::E; ++ex)
#pragma unroll
      for (int j = 0; j < (1 << R); ++j) x[(ex << R) | j] = sb[SL::idx(RG::off(ex, j))];
  }
}

template <class RG, class W>
__device__ __forceinline__ void smem_store(const W* x, W* s, uint32_t base_v) {
  constexpr int R = RG::R;
  using PW = typename PairOf<W>::type;
  using SL = Smem<W>;
  if constexpr (kContig32<RG, W>) {
    const uint32_t ib = SL::idx(base_v);
#pragma unroll
    for (int j = 0; j < (1 << R); j += 4)
      *reinterpret_cast<uint4*>(s + (ib ^ (uint32_t)j)) = make_uint4(x[j], x[j + 1], x[j + 2], x[j + 3]);
  } else if constexpr (SL::kXor) {
    const uint32_t ib = SL::idx(base_v);
    if constexpr (RG::PAIRS) {
#pragma unroll
      for (int m = 0; m < RG::E / 2; ++m)
#pragma unroll
        for (int j = 0; j < (1 << R); ++j)
          *reinterpret_cast<PW*>(s + (ib ^ SL::idx(RG::off(2 * m, j)))) =
              PairOf<W>::make(x[((2 * m) << R) | j], x[((2 * m + 1) << R) | j]);
    } else {
#pragma unroll
      for (int ex = 0; ex < RG::E; ++ex)
#pragma unroll
        for (int j = 0; j < (1 << R); ++j) s[ib ^ SL::idx(RG::off(ex, j))] = x[(ex << R) | j];
    }
  } else if constexpr (RG::PAIRS) {
    W* sb = s + SL::idx(base_v);
#pragma unroll
    for (int m = 0; m < RG::E / 2; ++m)
#pragma unroll
      for (int j = 0; j < (1 << R); ++j)
        *reinterpret_cast<PW*>(sb + SL::idx(RG::off(2 * m, j))) =
            PairOf<W>::make(x[((2 * m) << R) | j], x[((2 * m + 1) << R) | j]);
  } else {
    W* sb = s + SL::idx(base_v);
#pragma unroll
    for (int ex = 0; ex < RG::E; ++ex)
#pragma unroll
      for (int j = 0; j < (1 << R); ++j) sb[SL::idx(RG::off(ex, j))] = x[(ex << R) | j];
  }
}

// NN consecutive twiddle pairs from src, which is aligned to NN pairs (every
// caller's offset is a multiple of NN).  8-byte pairs (32-bit words) move
// two per 16-byte load.
template <int NN, class PW>
__device__ __forceinline__ void ld_twiddles(PW* dst, const PW* __restrict__ src) {
  if constexpr (sizeof(PW) == 8 && NN >= 2) {
    const uint4* s4 = reinterpret_cast<const uint4*>(src);
#pragma unroll
    for (int i = 0; i < NN / 2; ++i) {
      const uint4 v = __ldg(s4 + i);
      dst[2 * i] = PW{v.x, v.y};
      dst[2 * i + 1] = PW{v.z, v.w};
    }
  } else {
#pragma unroll
    for (int i = 0; i < NN; ++i) dst[i] = __ldg(src + i);
  }
}

// ---- butterfly stages on registers -------------------------------------------
// Forward sub-stage k of a round pairs (j, j + 2^(R-1-k)) with twiddle
// w[2^(s_first+k) + (gr << k) + (j >> (R-k))].  The twiddles of sub-stage
// k+1 are requested before sub-stage k computes.
template <int R, int E, int k, class W, class PW>
__device__ __forceinline__ void ct_stages(W* x, const PW* __restrict__ tw, uint32_t s_first, uint32_t gr,
                                          W np, W p2, const PW* wk) {
  if constexpr (k < R) {
    constexpr int d = 1 << (R - 1 - k);
    constexpr int NJ = 1 << k;
    constexpr int NN = (k + 1 < R) ? (2 << k) : 1;
    PW wn[NN];
    if constexpr (k + 1 < R) {
      ld_twiddles<NN>(wn, tw + (1u << (s_first + k + 1)) + (gr << (k + 1)));
    }
#pragma unroll
    for (int jj = 0; jj < NJ; ++jj)
#pragma unroll
      for (int ex = 0; ex < E; ++ex)
#pragma unroll
        for (int q = 0; q < d; ++q) {
          const int j = jj * 2 * d + q;
          ct_bfly(x[(ex << R) | j], x[(ex << R) | (j + d)], wk[jj].x, wk[jj].y, np, p2);
        }
    ct_stages<R, E, k + 1>(x, tw, s_first, gr, np, p2, wn);
  }
}

template <class RG, class W, class PW>
__device__ __forceinline__ void ct_round(W* x, const PW* __restrict__ tw, uint32_t s_first, uint32_t gr, W p) {
  PW w0[1];
  w0[0] = __ldg(tw + (1u << s_first) + gr);
  ct_stages<RG::R, RG::E, 0>(x, tw, s_first, gr, (W)(0 - p), (W)(p << 1), w0);
}

// The same round applied to two operands that share twiddles (the two
// inputs of a polymul at the same limb and position).  The twiddles of
// sub-stage k+1 are requested before sub-stage k computes.
template <int R, int E, int k, class W, class PW>
__device__ __forceinline__ void ct_stages2p(W* x, W* y, const PW* __restrict__ tw, uint32_t s_first, uint32_t gr,
                                            W np, W p2, const PW* wk) {
  if constexpr (k < R) {
    constexpr int d = 1 << (R - 1 - k);
    constexpr int NJ = 1 << k;
    constexpr int NN = (k + 1 < R) ? (2 << k) : 1;
    PW wn[NN];
    if constexpr (k + 1 < R) {
      ld_twiddles<NN>(wn, tw + (1u << (s_first + k + 1)) + (gr << (k + 1)));
    }
#pragma unroll
    for (int jj = 0; jj < NJ; ++jj)
#pragma unroll
      for (int ex = 0; ex < E; ++ex)
#pragma unroll
        for (int q = 0; q < d; ++q) {
          const int j = jj * 2 * d + q;
          ct_bfly(x[(ex << R) | j], x[(ex << R) | (j + d)], wk[jj].x, wk[jj].y, np, p2);
          ct_bfly(y[(ex << R) | j], y[(ex << R) | (j + d)], wk[jj].x, wk[jj].y, np, p2);
        }
    ct_stages2p<R, E, k + 1>(x, y, tw, s_first, gr, np, p2, wn);
  }
}

// Two-operand round with its first sub-stage's twiddle loaded here.
template <int R, int E, class W, class PW>
__device__ __forceinline__ void ct_stages2(W* x, W* y, const PW* __restrict__ tw, uint32_t s_first, uint32_t gr,
                                           W np, W p2) {
  PW w0[1];
  w0[0] = __ldg(tw + (1u << s_first) + gr);
  ct_stages2p<R, E, 0>(x, y, tw, s_first, gr, np, p2, w0);
}

// Inverse sub-stage k pairs (j, j + 2^k) with twiddle
// w[2^(log_n-1-sigma_first-k) + (gr << (R-1-k)) + (j >> (k+1))].  With
// LAST, the round's final sub-stage is the reference's last layer with the
// N^-1 scaling fused (include/yell/details/ntt.hpp:144-159).
// top = log_n - 1 - sigma_first, so sub-stage k uses m = 2^(top - k).
template <int R, int E, bool LAST, int k, class W, class PW, class M>
__device__ __forceinline__ void gs_stages(W* x, const PW* __restrict__ itw, uint32_t top, uint32_t gr,
                                          const M& m, const PW* wk) {
  if constexpr (k < R) {
    constexpr int d = 1 << k;
    if constexpr (LAST && k == R - 1) {
#pragma unroll
      for (int ex = 0; ex < E; ++ex)
#pragma unroll
        for (int q = 0; q < d; ++q) gs_last(x[(ex << R) | q], x[(ex << R) | (q + d)], m);
    } else {
      constexpr int NJ = 1 << (R - 1 - k);
      constexpr bool NEXT = (k + 1 < R) && !(LAST && k + 2 == R);
      constexpr int NN = NEXT ? (1 << (R - 2 - k)) : 1;
      PW wn[NN];
      if constexpr (NEXT) {
        ld_twiddles<NN>(wn, itw + (1u << (top - k - 1)) + (gr << (R - 2 - k)));
      }
      const W np = (W)(0 - m.p), p2 = (W)(m.p << 1);
#pragma unroll
      for (int jj = 0; jj < NJ; ++jj)
#pragma unroll
        for (int ex = 0; ex < E; ++ex)
#pragma unroll
          for (int q = 0; q < d; ++q) {
            const int j = jj * 2 * d + q;
            gs_bfly(x[(ex << R) | j], x[(ex << R) | (j + d)], wk[jj].x, wk[jj].y, np, p2);
          }
      gs_stages<R, E, LAST, k + 1>(x, itw, top, gr, m, wn);
    }
  }
}

// Twiddles of an inverse round's first sub-stage (loaded ahead by callers
// that have other work to cover their latency with).
template <class RG, bool LAST>
struct GsFirst {
  static constexpr bool ONLY_LAST = LAST && RG::R == 1;
  static constexpr int N0 = ONLY_LAST ? 1 : (1 << (RG::R - 1));
  template <class PW>
  __device__ static __forceinline__ void load(PW* w0, const PW* __restrict__ itw, uint32_t log_n,
                                              uint32_t sigma_first, uint32_t gr) {
    if constexpr (!ONLY_LAST) {
      ld_twiddles<N0>(w0, itw + (1u << (log_n - 1 - sigma_first)) + (gr << (RG::R - 1)));
    }
  }
};

// Inverse round with its first sub-stage's twiddles already loaded.
template <class RG, bool LAST, class W, class M, class PW>
__device__ __forceinline__ void gs_round_w(W* x, uint32_t log_n, uint32_t sigma_first, uint32_t gr, const M& m,
                                           const PW* w0) {
  gs_stages<RG::R, RG::E, LAST, 0>(x, m.inv, log_n - 1 - sigma_first, gr, m, w0);
}

template <class RG, bool LAST, class W, class M>
__device__ __forceinline__ void gs_round(W* x, uint32_t log_n, uint32_t sigma_first, uint32_t gr, const M& m) {
  using PW = typename PairOf<W>::type;
  PW w0[GsFirst<RG, LAST>::N0];
  GsFirst<RG, LAST>::load(w0, m.inv, log_n, sigma_first, gr);
  gs_round_w<RG, LAST>(x, log_n, sigma_first, gr, m, w0);
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

__device__ __forceinline__ DevMod32 load_mod(const DevMod32* __restrict__ mods, uint32_t cm) {
  DevMod32 m;
  const ulonglong2* src = reinterpret_cast<const ulonglong2*>(mods + cm);
  const ulonglong2 a = __ldg(src);
  const uint4 b = __ldg(reinterpret_cast<const uint4*>(src + 1));
  const uint2 c = __ldg(reinterpret_cast<const uint2*>(src + 2));
  m.fwd = reinterpret_cast<const uint2*>(a.x);
  m.inv = reinterpret_cast<const uint2*>(a.y);
  m.p = b.x;
  m.pn = b.y;
  m.inv_n = b.z;
  m.inv_n_s = b.w;
  m.inv_n_iphi = c.x;
  m.inv_n_iphi_s = c.y;
  return m;
}

// ---- whole rounds through shared memory ---------------------------------------
// Forward round I: load from s, CT stages, store to s.  s_off: absolute stage
// of the transform's top u bit; G: the thread's sub-transform group number.
template <class C, int I, class W, class PW>
__device__ __forceinline__ void fwd_round_smem(W* s, uint32_t tid, uint32_t s_off, uint32_t G, const PW* tw, W p,
                                               bool active) {
  using RG = Round<C, I>;
  W x[1 << C::LOGE];
  const uint32_t b = RG::base(tid);
  if (active) {
    smem_load<RG>(x, s, b);
    ct_round<RG>(x, tw, s_off + RG::HI, RG::gr(b, G), p);
    smem_store<RG>(x, s, b);
  }
}

// Inverse round at top-index I: sig_off is the absolute inverse stage of the
// transform's u-bit 0.
template <class C, int I, bool LAST, class W, class M>
__device__ __forceinline__ void inv_round_smem(W* s, uint32_t tid, uint32_t log_n, uint32_t sig_off, uint32_t G,
                                               const M& m, bool active) {
  using RG = Round<C, I>;
  W x[1 << C::LOGE];
  const uint32_t b = RG::base(tid);
  if (active) {
    smem_load<RG>(x, s, b);
    gs_round<RG, LAST>(x, log_n, sig_off + RG::BETA, RG::gr(b, G), m);
    smem_store<RG>(x, s, b);
  }
}

// Barrier between rounds of kind BK (TileCfg::LOCAL_BARRIER, or 0 for the
// CTA's).  Named barrier 1 + g serves sub-transform g (barrier 0 is the
// CTA's); every thread of the group takes it, active or not.
template <class C, int BK>
__device__ __forceinline__ void round_barrier(uint32_t tid) {
  if constexpr (BK == 1) {
    __syncwarp();
  } else if constexpr (BK == 2) {
    asm volatile("bar.sync %0, %1;" ::"r"(1u + C::sub(tid)), "r"((uint32_t)C::GROUP) : "memory");
  } else {
    __syncthreads();
  }
}

// Forward rounds [I, I1) through shared memory, a barrier after each.
template <class C, int I, int I1, int BK = 0, class W, class PW>
__device__ __forceinline__ void fwd_rounds(W* s, uint32_t tid, uint32_t s_off, uint32_t G, const PW* tw, W p,
                                           bool active) {
  if constexpr (I < I1) {
    fwd_round_smem<C, I>(s, tid, s_off, G, tw, p, active);
    round_barrier<C, BK>(tid);
    fwd_rounds<C, I + 1, I1, BK>(s, tid, s_off, G, tw, p, active);
  }
}

// Forward rounds [I, I1) of two operands at the same positions (shared
// twiddles), a barrier after each.
template <class C, int I, int I1, int BK = 0, class W, class PW>
__device__ __forceinline__ void fwd_rounds2(W* sa, W* sb, uint32_t tid, uint32_t s_off, uint32_t G, const PW* tw,
                                            W p, bool active) {
  if constexpr (I < I1) {
    using RG = Round<C, I>;
    W xa[1 << C::LOGE], xb[1 << C::LOGE];
    const uint32_t b = RG::base(tid);
    if (active) {
      smem_load<RG>(xa, sa, b);
      smem_load<RG>(xb, sb, b);
      ct_stages2<RG::R, RG::E>(xa, xb, tw, s_off + RG::HI, RG::gr(b, G), (W)(0 - p), (W)(p << 1));
      smem_store<RG>(xa, sa, b);
      smem_store<RG>(xb, sb, b);
    }
    round_barrier<C, BK>(tid);
    fwd_rounds2<C, I + 1, I1, BK>(sa, sb, tid, s_off, G, tw, p, active);
  }
}

// Inverse rounds from top-index I down to I1 (exclusive), bottom-up order.
// The round at top-index 0 carries the scaled last layer when HAS_LAST.
template <class C, int I, int I1, bool HAS_LAST, int BK = 0, class W, class M>
__device__ __forceinline__ void inv_rounds(W* s, uint32_t tid, uint32_t log_n, uint32_t sig_off, uint32_t G,
                                           const M& m, bool active) {
  if constexpr (I > I1) {
    inv_round_smem<C, I, HAS_LAST && I == 0>(s, tid, log_n, sig_off, G, m, active);
    round_barrier<C, BK>(tid);
    inv_rounds<C, I - 1, I1, HAS_LAST, BK>(s, tid, log_n, sig_off, G, m, active);
  }
}

}  // namespace yell_gb300
