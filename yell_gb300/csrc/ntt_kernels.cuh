// NTT and fused polymul kernels for sm_103a (templates; see ntt_variants.h).
//
// Paths (per degree N = 2^log_n):
//   * whole-limb: N <= 2^13.  One CTA holds whole limbs in shared memory
//     (several limbs per CTA below 2^12), reads each word from HBM once and
//     writes it once.
//   * two-pass: N >= 2^14.  N = C x B with C = 2^k1.  The column pass applies
//     forward stages 0..k1-1, which pair words B*2^t apart (columns of stride
//     B); the row pass applies stages k1..log_n-1, which stay inside
//     contiguous blocks of B words.  The inverse runs the same passes in the
//     opposite order; its column pass ends with the scaled last layer.
//   * fused polymul: NTT(a), NTT(b), pointwise product and INTT in one kernel
//     (whole-limb) or three (two-pass: column pass of a and of b, one row
//     kernel doing forward rows of both, the product and inverse rows, then
//     the inverse column pass).  The last forward round of both operands,
//     the product and the first inverse round share one register set.
//
// Global I/O goes straight between registers and HBM in rounds whose lanes
// cover contiguous words (the top round of a row tile, every round of a
// column tile); the other ends are staged through shared memory so that the
// HBM accesses stay coalesced.
#pragma once
#include <atomic>
#include <cstring>
#include <utility>

#include "kernels.h"
#include "ntt_tile.cuh"
#include "profiler.h"
#include "ntt_variants.h"
#include <cstdio>

namespace yell_gb300 {

// Everything below has internal linkage: each translation unit that includes
// this header instantiates the kernels of its own degrees and variants.
namespace {

constexpr int kTileLog = 12;  // 4096 words per two-pass tile

__device__ __forceinline__ ulonglong2 ld_pair(const uint64_t* p) {
  return __ldg(reinterpret_cast<const ulonglong2*>(p));
}

// Loads of words another CTA of the same launch wrote (the persistent batch
// kernel's intermediates): through L2, never the non-coherent read-only path.
__device__ __forceinline__ ulonglong2 ld_pair_cg(const uint64_t* p) {
  ulonglong2 v;
  asm volatile("ld.global.cg.v2.u64 {%0, %1}, [%2];" : "=l"(v.x), "=l"(v.y) : "l"(p));
  return v;
}
__device__ __forceinline__ uint64_t ld_cg(const uint64_t* p) {
  uint64_t v;
  asm volatile("ld.global.cg.u64 %0, [%1];" : "=l"(v) : "l"(p));
  return v;
}
template <bool COH>
__device__ __forceinline__ ulonglong2 ld_pair_t(const uint64_t* p) {
  if constexpr (COH) return ld_pair_cg(p);
  else return ld_pair(p);
}
template <bool COH>
__device__ __forceinline__ uint64_t ld_word_t(const uint64_t* p) {
  if constexpr (COH) return ld_cg(p);
  else return __ldg(p);
}

__device__ __forceinline__ void st_pair(uint64_t* p, uint64_t a, uint64_t b) {
  *reinterpret_cast<ulonglong2*>(p) = make_ulonglong2(a, b);
}

// ---- direct global access for one round ---------------------------------------
// Row-type region: word u of the region at g[u]; base_u and offsets are
// u-space (tile bits below LB + K, LB = 0).
template <class RG, bool COH = false>
__device__ __forceinline__ void gload_rows(uint64_t* x, const uint64_t* g, uint32_t base_u) {
  constexpr int R = RG::R;
  const uint64_t* gb = g + base_u;
  if constexpr (RG::PAIRS) {
#pragma unroll
    for (int m = 0; m < RG::E / 2; ++m)
#pragma unroll
      for (int j = 0; j < (1 << R); ++j) {
        const ulonglong2 v = ld_pair_t<COH>(gb + RG::off(2 * m, j));
        x[((2 * m) << R) | j] = v.x;
        x[((2 * m + 1) << R) | j] = v.y;
      }
  } else if constexpr (RG::CONTIG) {
#pragma unroll
    for (int j = 0; j < (1 << R); j += 2) {
      const ulonglong2 v = ld_pair_t<COH>(gb + j);
      x[j] = v.x;
      x[j + 1] = v.y;
    }
  } else {
#pragma unroll
    for (int ex = 0; ex < RG::E; ++ex)
#pragma unroll
      for (int j = 0; j < (1 << R); ++j) x[(ex << R) | j] = ld_word_t<COH>(gb + RG::off(ex, j));
  }
}

template <class RG>
__device__ __forceinline__ void gstore_rows(const uint64_t* x, uint64_t* g, uint32_t base_u) {
  constexpr int R = RG::R;
  uint64_t* gb = g + base_u;
  if constexpr (RG::PAIRS) {
#pragma unroll
    for (int m = 0; m < RG::E / 2; ++m)
#pragma unroll
      for (int j = 0; j < (1 << R); ++j)
        st_pair(gb + RG::off(2 * m, j), x[((2 * m) << R) | j], x[((2 * m + 1) << R) | j]);
  } else if constexpr (RG::CONTIG) {
#pragma unroll
    for (int j = 0; j < (1 << R); j += 2) st_pair(gb + j, x[j], x[j + 1]);
  } else {
#pragma unroll
    for (int ex = 0; ex < RG::E; ++ex)
#pragma unroll
      for (int j = 0; j < (1 << R); ++j) gb[RG::off(ex, j)] = x[(ex << R) | j];
  }
}

// Column tile: tile word v (row c = v >> LB, column v & (2^LB - 1)) is at
// g[(c << LOGB) + column], g = limb + first column of the tile.
template <class RG, int LOGB>
__device__ __forceinline__ size_t col_base(uint32_t base_v) {
  return ((size_t)(base_v >> RG::LB) << LOGB) + (base_v & ((1u << RG::LB) - 1u));
}

template <class RG, int LOGB, bool COH = false>
__device__ __forceinline__ void gload_cols(uint64_t* x, const uint64_t* g, uint32_t base_v) {
  constexpr int R = RG::R;
  const uint64_t* gb = g + col_base<RG, LOGB>(base_v);
#pragma unroll
  for (int ex = 0; ex < RG::E; ++ex)
#pragma unroll
    for (int j = 0; j < (1 << R); ++j)
      x[(ex << R) | j] = ld_word_t<COH>(gb + ((size_t)(RG::off(ex, j) >> RG::LB) << LOGB));
}

template <class RG, int LOGB>
__device__ __forceinline__ void gstore_cols(const uint64_t* x, uint64_t* g, uint32_t base_v) {
  constexpr int R = RG::R;
  uint64_t* gb = g + col_base<RG, LOGB>(base_v);
#pragma unroll
  for (int ex = 0; ex < RG::E; ++ex)
#pragma unroll
    for (int j = 0; j < (1 << R); ++j) gb[(size_t)(RG::off(ex, j) >> RG::LB) << LOGB] = x[(ex << R) | j];
}

// ---- staged (coalesced) copies between a whole tile and HBM ------------------
// Whole-limb tile: 2^T words = 2^(T-K) limbs of 2^K words.
template <class C>
__device__ __forceinline__ void stage_in_limbs(uint64_t* s, const ConstLimbSet& src, uint32_t limb0,
                                               uint32_t count, uint32_t log_n) {
  for (uint32_t v = threadIdx.x * 2; v < (1u << C::T); v += C::THREADS * 2) {
    const uint32_t limb = limb0 + (v >> C::K);
    if (limb < count)
      *reinterpret_cast<ulonglong2*>(s + sidx(v)) =
          ld_pair(src.limb(limb, log_n) + (v & ((1u << C::K) - 1u)));
  }
}

// Copies the tile out; `reduce` applies ntt<N>::forward's final reduction.
template <class C>
__device__ __forceinline__ void stage_out_limbs(const uint64_t* s, const LimbSet& dst, uint32_t limb0,
                                                uint32_t log_n, const DevMod* __restrict__ mods,
                                                bool reduce) {
  for (uint32_t v = threadIdx.x * 2; v < (1u << C::T); v += C::THREADS * 2) {
    const uint32_t limb = limb0 + (v >> C::K);
    if (limb < dst.count) {
      ulonglong2 d = *reinterpret_cast<const ulonglong2*>(s + sidx(v));
      if (reduce) {
        const uint64_t p = __ldg(&mods[dst.cm(limb)].p);
        d.x = fwd_correct(d.x, p, p << 1);
        d.y = fwd_correct(d.y, p, p << 1);
      }
      *reinterpret_cast<ulonglong2*>(dst.limb(limb, log_n) + (v & ((1u << C::K) - 1u))) = d;
    }
  }
}

// Contiguous 2^T-word region.
template <class C>
__device__ __forceinline__ void stage_in_region(uint64_t* s, const uint64_t* g) {
  for (uint32_t v = threadIdx.x * 2; v < (1u << C::T); v += C::THREADS * 2)
    *reinterpret_cast<ulonglong2*>(s + sidx(v)) = ld_pair(g + v);
}

template <class C>
__device__ __forceinline__ void stage_out_region(const uint64_t* s, uint64_t* g, uint64_t p, bool reduce) {
  for (uint32_t v = threadIdx.x * 2; v < (1u << C::T); v += C::THREADS * 2) {
    ulonglong2 d = *reinterpret_cast<const ulonglong2*>(s + sidx(v));
    if (reduce) {
      d.x = fwd_correct(d.x, p, p << 1);
      d.y = fwd_correct(d.y, p, p << 1);
    }
    st_pair(g + v, d.x, d.y);
  }
}

__host__ __device__ ConstLimbSet as_const(const LimbSet& l) {
  ConstLimbSet c;
  c.base = l.base;
  c.ptrs = l.ptrs;
  c.cms = l.cms;
  c.count = l.count;
  c.L = l.L;
  c.cm0 = l.cm0;
  c.pad_ = 0;
  return c;
}

// Whole-limb NTT tiles holding several limbs (sub-transforms of fewer
// threads than the CTA, each with its own barrier) move the bottom round
// between HBM and registers directly; one-limb tiles stage it coalesced.
template <class C>
constexpr bool kDirectBottom = C::LOCAL_BARRIER != 0 && C::GROUP < C::THREADS;

// ===========================================================================
// Whole-limb NTT.  DIR: 0 forward (reduced), 1 forward lazy, 2 backward.
// ===========================================================================
// Three 256-thread CTAs per SM (at most 85 registers, a few bytes spilled;
// the compiler's own choice of up to 106 gave two): 2^12 NTTs 7% faster.
template <class C, int DIR>
__global__ void __launch_bounds__(C::THREADS, C::THREADS <= 256 ? 3 : 1) k_ntt_whole(LimbSet ls, const DevMod* __restrict__ mods) {
  extern __shared__ __align__(16) uint64_t smem[];
  constexpr int K = C::K, NR = C::NR;
  const uint32_t log_n = K;
  const uint32_t tid = threadIdx.x;
  const uint32_t limb0 = blockIdx.x << (C::T - K);
  const uint32_t my_limb = limb0 + C::sub(tid);
  const bool active = my_limb < ls.count;
  const DevMod m = load_mod(mods, ls.cm(active ? my_limb : 0));
  const uint32_t umask = (1u << K) - 1u;
  if constexpr (DIR != 2) {
    // forward: round 0 straight from HBM when it is not also the last round
    if constexpr (NR > 1) {
      // barriers over a limb's threads between rounds; with one limb per CTA
      // the CTA's before the cooperative (coalesced) stage-out, with several
      // the bottom round goes to HBM straight from registers and the CTA
      // barrier disappears (2^10: 16% faster)
      constexpr int BK = C::LOCAL_BARRIER;
      using RG = Round<C, 0>;
      uint64_t x[1 << C::LOGE];
      const uint32_t b = RG::base(tid);
      if (active) {
        gload_rows<RG>(x, ls.limb(my_limb, log_n), b & umask);
        ct_round<RG>(x, m.fwd, RG::HI, RG::gr(b, 0), m.p);
        smem_store<RG>(x, smem, b);
      }
      round_barrier<C, BK>(tid);
      fwd_rounds<C, 1, NR - 1, BK>(smem, tid, 0, 0, m.fwd, m.p, active);
      if constexpr (kDirectBottom<C>) {
        using RB = Round<C, NR - 1>;
        const uint32_t bb = RB::base(tid);
        if (active) {
          smem_load<RB>(x, smem, bb);
          ct_round<RB>(x, m.fwd, RB::HI, RB::gr(bb, 0), m.p);
          if constexpr (DIR == 0) {
#pragma unroll
            for (int i = 0; i < (1 << C::LOGE); ++i) x[i] = fwd_correct(x[i], m.p, m.p << 1);
          }
          gstore_rows<RB>(x, ls.limb(my_limb, log_n), bb & umask);
        }
        return;
      }
      fwd_rounds<C, NR - 1, NR>(smem, tid, 0, 0, m.fwd, m.p, active);
    } else {
      stage_in_limbs<C>(smem, as_const(ls), limb0, ls.count, log_n);
      __syncthreads();
      fwd_rounds<C, 0, NR>(smem, tid, 0, 0, m.fwd, m.p, active);
    }
    stage_out_limbs<C>(smem, ls, limb0, log_n, mods, DIR == 0);
  } else {
    if constexpr (NR > 1) {
      if constexpr (kDirectBottom<C>) {
        // several limbs per CTA: the bottom round straight from HBM
        using RB = Round<C, NR - 1>;
        uint64_t xb[1 << C::LOGE];
        const uint32_t bb = RB::base(tid);
        if (active) {
          gload_rows<RB>(xb, ls.limb(my_limb, log_n), bb & umask);
          gs_round<RB, false>(xb, log_n, RB::BETA, RB::gr(bb, 0), m);
          smem_store<RB>(xb, smem, bb);
        }
        round_barrier<C, C::LOCAL_BARRIER>(tid);
        inv_rounds<C, NR - 2, 0, true, C::LOCAL_BARRIER>(smem, tid, log_n, 0, 0, m, active);
      } else {
        // after the cooperative stage-in, barriers over a limb's threads only
        stage_in_limbs<C>(smem, as_const(ls), limb0, ls.count, log_n);
        __syncthreads();
        inv_rounds<C, NR - 1, 0, true, C::LOCAL_BARRIER>(smem, tid, log_n, 0, 0, m, active);
      }
      using RG = Round<C, 0>;
      uint64_t x[1 << C::LOGE];
      const uint32_t b = RG::base(tid);
      if (active) {
        smem_load<RG>(x, smem, b);
        gs_round<RG, true>(x, log_n, RG::BETA, RG::gr(b, 0), m);
        gstore_rows<RG>(x, ls.limb(my_limb, log_n), b & umask);
      }
    } else {
      stage_in_limbs<C>(smem, as_const(ls), limb0, ls.count, log_n);
      __syncthreads();
      inv_rounds<C, 0, -1, true>(smem, tid, log_n, 0, 0, m, active);
      stage_out_limbs<C>(smem, ls, limb0, log_n, mods, false);
    }
  }
}

// ===========================================================================
// Two-pass column pass.  Tile = 2^K rows x 2^LB columns (K + LB = 12);
// limb word (c << LOGB) + col0 + col.  Forward: stages 0..K-1; inverse:
// stages LOGB..log_n-1 with the scaled last layer.  src and dst may alias.
// ===========================================================================
template <class C, int LOGB, bool INV, bool COH = false>
__device__ __forceinline__ void col_pass_body(ConstLimbSet src, LimbSet dst, const DevMod* __restrict__ mods,
                                              uint32_t bid) {
  extern __shared__ __align__(16) uint64_t smem[];
  constexpr int K = C::K, LB = C::LB, NR = C::NR;
  constexpr uint32_t log_n = K + LOGB;
  constexpr int TPL = LOGB - LB;  // log2(tiles per limb)
  const uint32_t tid = threadIdx.x;
  const uint32_t limb = dst.ordered(bid >> TPL);
  const uint32_t col0 = (bid & ((1u << TPL) - 1u)) << LB;
  const uint64_t* in = src.limb(limb, log_n) + col0;
  uint64_t* out = dst.limb(limb, log_n) + col0;
  const DevMod m = load_mod(mods, dst.cm(limb));
  uint64_t x[1 << C::LOGE];
  if constexpr (!INV) {
    using R0 = Round<C, 0>;
    const uint32_t b0 = R0::base(tid);
    gload_cols<R0, LOGB, COH>(x, in, b0);
    ct_round<R0>(x, m.fwd, R0::HI, R0::gr(b0, 0), m.p);
    if constexpr (NR == 1) {
      gstore_cols<R0, LOGB>(x, out, b0);
    } else {
      smem_store<R0>(x, smem, b0);
      __syncthreads();
      fwd_rounds<C, 1, NR - 1>(smem, tid, 0, 0, m.fwd, m.p, true);
      using RL = Round<C, NR - 1>;
      const uint32_t bl = RL::base(tid);
      smem_load<RL>(x, smem, bl);
      ct_round<RL>(x, m.fwd, RL::HI, RL::gr(bl, 0), m.p);
      gstore_cols<RL, LOGB>(x, out, bl);
    }
  } else {
    using RB = Round<C, NR - 1>;  // bottom round, executed first
    const uint32_t bb = RB::base(tid);
    gload_cols<RB, LOGB, COH>(x, in, bb);
    if constexpr (NR == 1) {
      gs_round<RB, true>(x, log_n, LOGB + RB::BETA, RB::gr(bb, 0), m);
      gstore_cols<RB, LOGB>(x, out, bb);
    } else {
      gs_round<RB, false>(x, log_n, LOGB + RB::BETA, RB::gr(bb, 0), m);
      smem_store<RB>(x, smem, bb);
      __syncthreads();
      inv_rounds<C, NR - 2, 0, false>(smem, tid, log_n, LOGB, 0, m, true);
      using RT = Round<C, 0>;
      const uint32_t bt = RT::base(tid);
      smem_load<RT>(x, smem, bt);
      gs_round<RT, true>(x, log_n, LOGB + RT::BETA, RT::gr(bt, 0), m);
      gstore_cols<RT, LOGB>(x, out, bt);
    }
  }
}

// The standalone column pass keeps its own copy of the body above: compiled
// as one kernel it schedules better at k1 = 9 (1.131 vs 1.141 ms for the
// N = 2^16, L = 32, 16-pair polymul on GB300) than the inlined body.  The
// inverse pass waits mostly on its strided column loads: capped at 64
// registers (a few bytes spilled) it runs four CTAs per SM instead of three,
// and that polymul takes 1.117 instead of 1.127 ms.  The forward pass (NTT
// calls) fits three CTAs per SM at 80 registers without spilling.
// Minimum resident CTAs for a launch-bounds target of `threads` per SM.
constexpr int min_blocks(int threads_per_sm, int cta_threads) {
  return threads_per_sm / cta_threads > 1 ? threads_per_sm / cta_threads : 1;
}

template <class C, int LOGB, bool INV>
__global__ void __launch_bounds__(C::THREADS, min_blocks(INV ? 1024 : 768, C::THREADS))
    k_col_pass(ConstLimbSet src, LimbSet dst, const DevMod* __restrict__ mods) {
  extern __shared__ __align__(16) uint64_t smem[];
  constexpr int K = C::K, LB = C::LB, NR = C::NR;
  constexpr uint32_t log_n = K + LOGB;
  constexpr int TPL = LOGB - LB;  // log2(tiles per limb)
  grid_dep_launch();
  // when launched as a dependent: the previous kernel's words, and limb or
  // modulus lists it may have written, are read only after this
  grid_dep_wait();
  const uint32_t tid = threadIdx.x;
  const uint32_t limb = dst.ordered(blockIdx.x >> TPL);
  const uint32_t col0 = (blockIdx.x & ((1u << TPL) - 1u)) << LB;
  const uint64_t* in = src.limb(limb, log_n) + col0;
  uint64_t* out = dst.limb(limb, log_n) + col0;
  const DevMod m = load_mod(mods, dst.cm(limb));
  uint64_t x[1 << C::LOGE];
  if constexpr (!INV) {
    using R0 = Round<C, 0>;
    const uint32_t b0 = R0::base(tid);
    gload_cols<R0, LOGB>(x, in, b0);
    ct_round<R0>(x, m.fwd, R0::HI, R0::gr(b0, 0), m.p);
    if constexpr (NR == 1) {
      gstore_cols<R0, LOGB>(x, out, b0);
    } else {
      smem_store<R0>(x, smem, b0);
      __syncthreads();
      fwd_rounds<C, 1, NR - 1>(smem, tid, 0, 0, m.fwd, m.p, true);
      using RL = Round<C, NR - 1>;
      const uint32_t bl = RL::base(tid);
      smem_load<RL>(x, smem, bl);
      ct_round<RL>(x, m.fwd, RL::HI, RL::gr(bl, 0), m.p);
      gstore_cols<RL, LOGB>(x, out, bl);
    }
  } else {
    using RB = Round<C, NR - 1>;  // bottom round, executed first
    const uint32_t bb = RB::base(tid);
    gload_cols<RB, LOGB>(x, in, bb);
    if constexpr (NR == 1) {
      gs_round<RB, true>(x, log_n, LOGB + RB::BETA, RB::gr(bb, 0), m);
      gstore_cols<RB, LOGB>(x, out, bb);
    } else {
      gs_round<RB, false>(x, log_n, LOGB + RB::BETA, RB::gr(bb, 0), m);
      smem_store<RB>(x, smem, bb);
      __syncthreads();
      inv_rounds<C, NR - 2, 0, false>(smem, tid, log_n, LOGB, 0, m, true);
      using RT = Round<C, 0>;
      const uint32_t bt = RT::base(tid);
      smem_load<RT>(x, smem, bt);
      gs_round<RT, true>(x, log_n, LOGB + RT::BETA, RT::gr(bt, 0), m);
      gstore_cols<RT, LOGB>(x, out, bt);
    }
  }
}

// ===========================================================================
// Two-pass row pass over 4096 contiguous words (2^(12-K) blocks of 2^K).
// Forward: stages k1..log_n-1 (+ the final reduction when reduce); inverse:
// stages 0..K-1.  In place.
// ===========================================================================
template <class C, int K1, bool INV>
__global__ void __launch_bounds__(C::THREADS) k_row_pass(LimbSet ls, const DevMod* __restrict__ mods,
                                                         int reduce) {
  extern __shared__ __align__(16) uint64_t smem[];
  constexpr int K = C::K, NR = C::NR;
  constexpr uint32_t log_n = K + K1;
  constexpr int TPL = log_n - kTileLog;
  grid_dep_launch();
  grid_dep_wait();  // as in k_col_pass
  const uint32_t tid = threadIdx.x;
  const uint32_t limb = ls.ordered(blockIdx.x >> TPL);
  const uint32_t off = (blockIdx.x & ((1u << TPL) - 1u)) << kTileLog;
  uint64_t* data = ls.limb(limb, log_n) + off;
  const DevMod m = load_mod(mods, ls.cm(limb));
  const uint32_t G = (off >> K) + C::sub(tid);
  if constexpr (!INV) {
    using R0 = Round<C, 0>;
    uint64_t x[1 << C::LOGE];
    const uint32_t b0 = R0::base(tid);
    gload_rows<R0>(x, data, b0);
    ct_round<R0>(x, m.fwd, K1 + R0::HI, R0::gr(b0, G), m.p);
    smem_store<R0>(x, smem, b0);
    // barriers over a row's threads between rounds; the CTA's only before
    // the cooperative stage-out
    round_barrier<C, C::LOCAL_BARRIER>(tid);
    fwd_rounds<C, 1, NR - 1, C::LOCAL_BARRIER>(smem, tid, K1, G, m.fwd, m.p, true);
    fwd_rounds<C, NR - 1, NR>(smem, tid, K1, G, m.fwd, m.p, true);
    stage_out_region<C>(smem, data, m.p, reduce != 0);
  } else {
    stage_in_region<C>(smem, data);
    __syncthreads();
    // after the cooperative stage-in, barriers over a row's threads only
    inv_rounds<C, NR - 1, 0, false, C::LOCAL_BARRIER>(smem, tid, log_n, 0, G, m, true);
    using RT = Round<C, 0>;
    uint64_t x[1 << C::LOGE];
    const uint32_t bt = RT::base(tid);
    smem_load<RT>(x, smem, bt);
    gs_round<RT, false>(x, log_n, RT::BETA, RT::gr(bt, G), m);
    gstore_rows<RT>(x, data, bt);
  }
}

// ===========================================================================
// Fused product round shared by both polymul kernels: the bottom forward
// round (R = LOGE at bit 0) of both operands with shared twiddles, the
// pointwise product and the bottom inverse round, on one register set.  The
// product is a Montgomery product of the lazy forward words (one conditional
// subtraction each instead of ntt<N>::forward's reduction and the Barrett
// reduction of ops::mulmod): x*y*2^-64 in [0, 2p), congruent to the
// reference's product times 2^-64, which the inverse's scaling constants
// (N^-1 * 2^64, the polymul copy of the constants) cancel, so the output
// words equal the reference's.
// ===========================================================================
// First twiddle of the fused product round (its forward top sub-stage), for
// callers that request it a round ahead.
template <class C>
__device__ __forceinline__ ulonglong2 fused_w0(uint32_t b, uint32_t s_off, uint32_t G, const DevMod& m) {
  using RB = Round<C, C::NR - 1>;
  return __ldg(m.fwd + (1u << (s_off + RB::HI)) + RB::gr(b, G));
}

template <class C, bool INV_LAST>
__device__ __forceinline__ void fused_product(uint64_t* xa, uint64_t* xb, uint32_t b, uint32_t log_n,
                                              uint32_t s_off, uint32_t G, const DevMod& m, ulonglong2 w0) {
  using RB = Round<C, C::NR - 1>;
  static_assert(RB::R == C::LOGE && RB::BETA == 0, "bottom round must be full width");
  constexpr int E = 1 << C::LOGE;
  const uint64_t p = m.p, p2 = m.p << 1;
  const uint32_t gr = RB::gr(b, G);
  ct_stages2p<RB::R, RB::E, 0>(xa, xb, m.fwd, s_off + RB::HI, gr, 0 - p, p2, &w0);
  // the inverse round's first twiddles load while the products compute
  ulonglong2 wg[GsFirst<RB, INV_LAST>::N0];
  GsFirst<RB, INV_LAST>::load(wg, m.inv, log_n, 0, gr);
  // m is the polymul copy of the constants: m.pn = -p^-1 mod 2^64
#pragma unroll
  for (int i = 0; i < E; ++i) xa[i] = mont_mul(csub(xa[i], p2), csub(xb[i], p2), p, m.pn);
  gs_round_w<RB, INV_LAST>(xa, log_n, 0, gr, m, wg);
}

// Whole-limb fused polymul: c = INTT(NTT(a) * NTT(b)), N <= 2^13.
template <class C>
__device__ __forceinline__ void polymul_whole_body(LimbSet c, ConstLimbSet a, ConstLimbSet b,
                                                   const DevMod* __restrict__ mods, uint32_t bid) {
  extern __shared__ __align__(16) uint64_t smem[];
  constexpr int K = C::K, NR = C::NR;
  constexpr uint32_t log_n = K;
  uint64_t* sa = smem;
  uint64_t* sb = smem + tile_smem_words(1u << C::T);
  const uint32_t tid = threadIdx.x;
  const uint32_t limb0 = bid << (C::T - K);
  const uint32_t my_limb = limb0 + C::sub(tid);
  const bool active = my_limb < c.count;
  const DevMod m = load_mod(mods, c.cm(active ? my_limb : 0));
  const uint32_t umask = (1u << K) - 1u;
  constexpr int E = 1 << C::LOGE;
  uint64_t xa[E], xb[E];
  if constexpr (NR == 1) {
    using RB = Round<C, 0>;
    const uint32_t bb = RB::base(tid);
    const ulonglong2 w0 = fused_w0<C>(bb, 0, 0, m);
    stage_in_limbs<C>(sa, a, limb0, c.count, log_n);
    stage_in_limbs<C>(sb, b, limb0, c.count, log_n);
    __syncthreads();
    if (active) {
      smem_load<RB>(xa, sa, bb);
      smem_load<RB>(xb, sb, bb);
      fused_product<C, true>(xa, xb, bb, log_n, 0, 0, m, w0);
      smem_store<RB>(xa, sa, bb);
    }
    __syncthreads();
    stage_out_limbs<C>(sa, c, limb0, log_n, mods, false);
  } else {
    // no CTA-wide staging on this path: barriers over a limb's threads only
    constexpr int BK = C::LOCAL_BARRIER;
    using R0 = Round<C, 0>;
    const uint32_t b0 = R0::base(tid);
    if (active) {
      gload_rows<R0>(xa, a.limb(my_limb, log_n), b0 & umask);
      gload_rows<R0>(xb, b.limb(my_limb, log_n), b0 & umask);
      ct_stages2<R0::R, R0::E>(xa, xb, m.fwd, R0::HI, R0::gr(b0, 0), 0 - m.p, m.p << 1);
      smem_store<R0>(xa, sa, b0);
      smem_store<R0>(xb, sb, b0);
    }
    round_barrier<C, BK>(tid);
    using RB = Round<C, NR - 1>;
    const uint32_t bb = RB::base(tid);
    const ulonglong2 w0 = fused_w0<C>(bb, 0, 0, m);
    fwd_rounds2<C, 1, NR - 1, BK>(sa, sb, tid, 0, 0, m.fwd, m.p, active);
    if (active) {
      smem_load<RB>(xa, sa, bb);
      smem_load<RB>(xb, sb, bb);
      fused_product<C, false>(xa, xb, bb, log_n, 0, 0, m, w0);
      smem_store<RB>(xa, sa, bb);
    }
    round_barrier<C, BK>(tid);
    inv_rounds<C, NR - 2, 0, true, BK>(sa, tid, log_n, 0, 0, m, active);
    if (active) {
      smem_load<R0>(xa, sa, b0);
      gs_round<R0, true>(xa, log_n, R0::BETA, R0::gr(b0, 0), m);
      gstore_rows<R0>(xa, c.limb(my_limb, log_n), b0 & umask);
    }
  }
}

// Two 256-thread CTAs per SM (at most 128 registers, a few bytes spilled):
// left to itself the compiler took 152-158 registers at the 2^12 tile, one
// CTA per SM, and a 2^12 polymul ran 20% longer.
template <class C>
__global__ void __launch_bounds__(C::THREADS, C::THREADS <= 256 ? 2 : 1) k_polymul_whole(LimbSet c, ConstLimbSet a, ConstLimbSet b,
                                                              const DevMod* __restrict__ mods) {
  polymul_whole_body<C>(c, a, b, mods, blockIdx.x);
}

// Forward column pass of both polymul operands in one CTA: each thread
// applies the same butterflies to a's and b's words at the same positions,
// so every twiddle load serves two butterflies.  a -> ca, b -> cb.
template <class C, int LOGB>
__device__ __forceinline__ void col_pass2_body(ConstLimbSet a, ConstLimbSet b, LimbSet ca, LimbSet cb,
                                               const DevMod* __restrict__ mods, uint32_t bid) {
  extern __shared__ __align__(16) uint64_t smem[];
  constexpr int K = C::K, LB = C::LB, NR = C::NR;
  constexpr uint32_t log_n = K + LOGB;
  constexpr int TPL = LOGB - LB;
  uint64_t* sa = smem;
  uint64_t* sb = smem + tile_smem_words(1u << kTileLog);
  const uint32_t tid = threadIdx.x;
  const uint32_t limb = ca.ordered(bid >> TPL);
  const uint32_t col0 = (bid & ((1u << TPL) - 1u)) << LB;
  const DevMod m = load_mod(mods, ca.cm(limb));
  const uint64_t np = 0 - m.p, p2 = m.p << 1;
  constexpr int E = 1 << C::LOGE;
  uint64_t xa[E], xb[E];
  using R0 = Round<C, 0>;
  const uint32_t b0 = R0::base(tid);
  gload_cols<R0, LOGB>(xa, a.limb(limb, log_n) + col0, b0);
  gload_cols<R0, LOGB>(xb, b.limb(limb, log_n) + col0, b0);
  ct_stages2<R0::R, R0::E>(xa, xb, m.fwd, R0::HI, R0::gr(b0, 0), np, p2);
  if constexpr (NR == 1) {
    gstore_cols<R0, LOGB>(xa, ca.limb(limb, log_n) + col0, b0);
    gstore_cols<R0, LOGB>(xb, cb.limb(limb, log_n) + col0, b0);
  } else {
    smem_store<R0>(xa, sa, b0);
    smem_store<R0>(xb, sb, b0);
    __syncthreads();
    fwd_rounds2<C, 1, NR - 1>(sa, sb, tid, 0, 0, m.fwd, m.p, true);
    using RL = Round<C, NR - 1>;
    const uint32_t bl = RL::base(tid);
    smem_load<RL>(xa, sa, bl);
    smem_load<RL>(xb, sb, bl);
    ct_stages2<RL::R, RL::E>(xa, xb, m.fwd, RL::HI, RL::gr(bl, 0), np, p2);
    gstore_cols<RL, LOGB>(xa, ca.limb(limb, log_n) + col0, bl);
    gstore_cols<RL, LOGB>(xb, cb.limb(limb, log_n) + col0, bl);
  }
}

template <class C, int LOGB>
__global__ void __launch_bounds__(C::THREADS, min_blocks(512, C::THREADS))
    k_col_pass2(ConstLimbSet a, ConstLimbSet b, LimbSet ca, LimbSet cb, const DevMod* __restrict__ mods) {
  grid_dep_launch();
  grid_dep_wait();  // as in k_col_pass
  col_pass2_body<C, LOGB>(a, b, ca, cb, mods, blockIdx.x);
}

// Two-pass fused row step: ca holds a's column-pass output and receives the
// row-pass output of the product; sbuf holds b's column-pass output.
template <class C, int K1, bool COH = false>
__device__ __forceinline__ void polymul_rows_body(LimbSet ca, ConstLimbSet sbuf, const DevMod* __restrict__ mods,
                                                  uint32_t bid) {
  extern __shared__ __align__(16) uint64_t smem[];
  constexpr int K = C::K, NR = C::NR;
  // rows stay with their threads: barriers over a row's threads only
  constexpr int BK = C::LOCAL_BARRIER;
  constexpr uint32_t log_n = K + K1;
  constexpr int TPL = log_n - kTileLog;
  uint64_t* sa = smem;
  uint64_t* sb = smem + tile_smem_words(1u << kTileLog);
  const uint32_t tid = threadIdx.x;
  const uint32_t limb = ca.ordered(bid >> TPL);
  const uint32_t off = (bid & ((1u << TPL) - 1u)) << kTileLog;
  uint64_t* pa = ca.limb(limb, log_n) + off;
  const uint64_t* pb = sbuf.limb(limb, log_n) + off;
  const DevMod m = load_mod(mods, ca.cm(limb));
  const uint32_t G = (off >> K) + C::sub(tid);
  constexpr int E = 1 << C::LOGE;
  uint64_t xa[E], xb[E];
  using R0 = Round<C, 0>;
  const uint32_t b0 = R0::base(tid);
  gload_rows<R0, COH>(xa, pa, b0);
  gload_rows<R0, COH>(xb, pb, b0);
  ct_stages2<R0::R, R0::E>(xa, xb, m.fwd, K1 + R0::HI, R0::gr(b0, G), 0 - m.p, m.p << 1);
  smem_store<R0>(xa, sa, b0);
  smem_store<R0>(xb, sb, b0);
  round_barrier<C, BK>(tid);
  using RB = Round<C, NR - 1>;
  const uint32_t bb = RB::base(tid);
  const ulonglong2 w0 = fused_w0<C>(bb, K1, G, m);
  fwd_rounds2<C, 1, NR - 1, BK>(sa, sb, tid, K1, G, m.fwd, m.p, true);
  smem_load<RB>(xa, sa, bb);
  smem_load<RB>(xb, sb, bb);
  fused_product<C, false>(xa, xb, bb, log_n, K1, G, m, w0);
  smem_store<RB>(xa, sa, bb);
  round_barrier<C, BK>(tid);
  inv_rounds<C, NR - 2, 0, false, BK>(sa, tid, log_n, 0, G, m, true);
  smem_load<R0>(xa, sa, b0);
  gs_round<R0, false>(xa, log_n, R0::BETA, R0::gr(b0, G), m);
  gstore_rows<R0>(xa, pa, b0);
}

template <class C, int K1>
__global__ void __launch_bounds__(C::THREADS, min_blocks(512, C::THREADS))
    k_polymul_rows(LimbSet ca, ConstLimbSet sbuf, const DevMod* __restrict__ mods) {
  grid_dep_launch();
  grid_dep_wait();  // as in k_col_pass
  // tiles in the reverse of the column pass's order: the first rows read the
  // words the column pass wrote last, still in L2, and the inverse column
  // pass (forward order) starts on the rows written last
  polymul_rows_body<C, K1>(ca, sbuf, mods, gridDim.x - 1 - blockIdx.x);
}

// ===========================================================================
// Pipelined two-pass polymul: the same three kernels as persistent CTAs that
// copy the next tile's words into shared memory (cp.async, 16 bytes per copy,
// into the padded layout) while they compute the current tile.  A tile's
// first round then reads shared memory instead of waiting on HBM, and the
// copy of tile t + grid overlaps the last round and the stores of tile t.
// Same butterflies, same words as the kernels above.
// ===========================================================================
__device__ __forceinline__ void cp_async16(void* smem_dst, const void* gsrc) {
  const uint32_t d = (uint32_t)__cvta_generic_to_shared(smem_dst);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(d), "l"(gsrc) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
// Waits for this thread's copies; a CTA barrier after it publishes everyone's.
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

// Column tile (rows of 2^LB words, stride 2^LOGB) -> padded shared layout.
template <class C, int LOGB>
__device__ __forceinline__ void stage_cols_async(uint64_t* s, const uint64_t* g) {
  static_assert(C::LB >= 1, "column pairs per 16-byte copy");
  for (uint32_t v = threadIdx.x * 2; v < (1u << C::T); v += C::THREADS * 2)
    cp_async16(s + sidx(v), g + ((size_t)(v >> C::LB) << LOGB) + (v & ((1u << C::LB) - 1u)));
}

// Contiguous 2^T-word region -> padded shared layout.
template <class C>
__device__ __forceinline__ void stage_region_async(uint64_t* s, const uint64_t* g) {
  for (uint32_t v = threadIdx.x * 2; v < (1u << C::T); v += C::THREADS * 2) cp_async16(s + sidx(v), g + v);
}

template <class C, int LOGB>
__global__ void __launch_bounds__(C::THREADS, min_blocks(512, C::THREADS))
    k_col_pass2_pipe(ConstLimbSet a, ConstLimbSet b, LimbSet ca, LimbSet cb, const DevMod* __restrict__ mods,
                     uint32_t tiles) {
  extern __shared__ __align__(16) uint64_t smem[];
  constexpr int K = C::K, LB = C::LB, NR = C::NR;
  constexpr uint32_t log_n = K + LOGB;
  constexpr int TPL = LOGB - LB;
  static_assert(NR >= 2, "the last round reads shared memory before the next tile is staged");
  uint64_t* sa = smem;
  uint64_t* sb = smem + tile_smem_words(1u << kTileLog);
  const uint32_t tid = threadIdx.x;
  constexpr int E = 1 << C::LOGE;
  uint64_t xa[E], xb[E];
  uint32_t bid = blockIdx.x;
  if (bid < tiles) {
    const uint32_t limb = ca.ordered(bid >> TPL), col0 = (bid & ((1u << TPL) - 1u)) << LB;
    stage_cols_async<C, LOGB>(sa, a.limb(limb, log_n) + col0);
    stage_cols_async<C, LOGB>(sb, b.limb(limb, log_n) + col0);
    cp_async_commit();
  }
  for (; bid < tiles; bid += gridDim.x) {
    const uint32_t limb = ca.ordered(bid >> TPL), col0 = (bid & ((1u << TPL) - 1u)) << LB;
    const DevMod m = load_mod(mods, ca.cm(limb));
    const uint64_t np = 0 - m.p, p2 = m.p << 1;
    cp_async_wait_all();
    __syncthreads();
    using R0 = Round<C, 0>;
    const uint32_t b0 = R0::base(tid);
    smem_load<R0>(xa, sa, b0);
    smem_load<R0>(xb, sb, b0);
    ct_stages2<R0::R, R0::E>(xa, xb, m.fwd, R0::HI, R0::gr(b0, 0), np, p2);
    smem_store<R0>(xa, sa, b0);  // the words this thread read: no barrier needed before
    smem_store<R0>(xb, sb, b0);
    __syncthreads();
    fwd_rounds2<C, 1, NR - 1>(sa, sb, tid, 0, 0, m.fwd, m.p, true);
    using RL = Round<C, NR - 1>;
    const uint32_t bl = RL::base(tid);
    smem_load<RL>(xa, sa, bl);
    smem_load<RL>(xb, sb, bl);
    __syncthreads();  // the tile is in registers: the buffers take the next one
    const uint32_t nb = bid + gridDim.x;
    if (nb < tiles) {
      const uint32_t nl = ca.ordered(nb >> TPL), nc = (nb & ((1u << TPL) - 1u)) << LB;
      stage_cols_async<C, LOGB>(sa, a.limb(nl, log_n) + nc);
      stage_cols_async<C, LOGB>(sb, b.limb(nl, log_n) + nc);
      cp_async_commit();
    }
    ct_stages2<RL::R, RL::E>(xa, xb, m.fwd, RL::HI, RL::gr(bl, 0), np, p2);
    gstore_cols<RL, LOGB>(xa, ca.limb(limb, log_n) + col0, bl);
    gstore_cols<RL, LOGB>(xb, cb.limb(limb, log_n) + col0, bl);
  }
}

template <class C, int K1>
__global__ void __launch_bounds__(C::THREADS, min_blocks(512, C::THREADS))
    k_polymul_rows_pipe(LimbSet ca, ConstLimbSet sbuf, const DevMod* __restrict__ mods, uint32_t tiles) {
  extern __shared__ __align__(16) uint64_t smem[];
  constexpr int K = C::K, NR = C::NR;
  constexpr int BK = C::LOCAL_BARRIER;
  constexpr uint32_t log_n = K + K1;
  constexpr int TPL = log_n - kTileLog;
  uint64_t* sa = smem;
  uint64_t* sb = smem + tile_smem_words(1u << kTileLog);
  const uint32_t tid = threadIdx.x;
  constexpr int E = 1 << C::LOGE;
  uint64_t xa[E], xb[E];
  uint32_t bid = blockIdx.x;
  if (bid < tiles) {
    const uint32_t limb = ca.ordered(bid >> TPL), off = (bid & ((1u << TPL) - 1u)) << kTileLog;
    stage_region_async<C>(sa, ca.limb(limb, log_n) + off);
    stage_region_async<C>(sb, sbuf.limb(limb, log_n) + off);
    cp_async_commit();
  }
  for (; bid < tiles; bid += gridDim.x) {
    const uint32_t limb = ca.ordered(bid >> TPL), off = (bid & ((1u << TPL) - 1u)) << kTileLog;
    const DevMod m = load_mod(mods, ca.cm(limb));
    const uint32_t G = (off >> K) + C::sub(tid);
    cp_async_wait_all();
    __syncthreads();
    using R0 = Round<C, 0>;
    const uint32_t b0 = R0::base(tid);
    smem_load<R0>(xa, sa, b0);
    smem_load<R0>(xb, sb, b0);
    ct_stages2<R0::R, R0::E>(xa, xb, m.fwd, K1 + R0::HI, R0::gr(b0, G), 0 - m.p, m.p << 1);
    smem_store<R0>(xa, sa, b0);
    smem_store<R0>(xb, sb, b0);
    round_barrier<C, BK>(tid);
    using RB = Round<C, NR - 1>;
    const uint32_t bb = RB::base(tid);
    const ulonglong2 w0 = fused_w0<C>(bb, K1, G, m);
    fwd_rounds2<C, 1, NR - 1, BK>(sa, sb, tid, K1, G, m.fwd, m.p, true);
    smem_load<RB>(xa, sa, bb);
    smem_load<RB>(xb, sb, bb);
    fused_product<C, false>(xa, xb, bb, log_n, K1, G, m, w0);
    smem_store<RB>(xa, sa, bb);
    round_barrier<C, BK>(tid);
    inv_rounds<C, NR - 2, 0, false, BK>(sa, tid, log_n, 0, G, m, true);
    smem_load<R0>(xa, sa, b0);
    __syncthreads();  // every row is in registers: the buffers take the next tile
    const uint32_t nb = bid + gridDim.x;
    if (nb < tiles) {
      const uint32_t nl = ca.ordered(nb >> TPL), no = (nb & ((1u << TPL) - 1u)) << kTileLog;
      stage_region_async<C>(sa, ca.limb(nl, log_n) + no);
      stage_region_async<C>(sb, sbuf.limb(nl, log_n) + no);
      cp_async_commit();
    }
    gs_round<R0, false>(xa, log_n, R0::BETA, R0::gr(b0, G), m);
    gstore_rows<R0>(xa, ca.limb(limb, log_n) + off, b0);
  }
}

// Inverse column pass, in place on ca.
template <class C, int LOGB>
__global__ void __launch_bounds__(C::THREADS, min_blocks(1024, C::THREADS))
    k_col_inv_pipe(LimbSet ca, const DevMod* __restrict__ mods, uint32_t tiles) {
  extern __shared__ __align__(16) uint64_t smem[];
  constexpr int K = C::K, LB = C::LB, NR = C::NR;
  constexpr uint32_t log_n = K + LOGB;
  constexpr int TPL = LOGB - LB;
  static_assert(NR >= 2, "the top round reads shared memory before the next tile is staged");
  const uint32_t tid = threadIdx.x;
  uint64_t x[1 << C::LOGE];
  uint32_t bid = blockIdx.x;
  if (bid < tiles) {
    const uint32_t limb = ca.ordered(bid >> TPL), col0 = (bid & ((1u << TPL) - 1u)) << LB;
    stage_cols_async<C, LOGB>(smem, ca.limb(limb, log_n) + col0);
    cp_async_commit();
  }
  for (; bid < tiles; bid += gridDim.x) {
    const uint32_t limb = ca.ordered(bid >> TPL), col0 = (bid & ((1u << TPL) - 1u)) << LB;
    const DevMod m = load_mod(mods, ca.cm(limb));
    cp_async_wait_all();
    __syncthreads();
    using RB = Round<C, NR - 1>;  // bottom round, executed first
    const uint32_t bb = RB::base(tid);
    smem_load<RB>(x, smem, bb);
    gs_round<RB, false>(x, log_n, LOGB + RB::BETA, RB::gr(bb, 0), m);
    smem_store<RB>(x, smem, bb);
    __syncthreads();
    inv_rounds<C, NR - 2, 0, false>(smem, tid, log_n, LOGB, 0, m, true);
    using RT = Round<C, 0>;
    const uint32_t bt = RT::base(tid);
    smem_load<RT>(x, smem, bt);
    __syncthreads();  // the tile is in registers: the buffer takes the next one
    const uint32_t nb = bid + gridDim.x;
    if (nb < tiles) {
      const uint32_t nl = ca.ordered(nb >> TPL), nc = (nb & ((1u << TPL) - 1u)) << LB;
      stage_cols_async<C, LOGB>(smem, ca.limb(nl, log_n) + nc);
      cp_async_commit();
    }
    gs_round<RT, true>(x, log_n, LOGB + RT::BETA, RT::gr(bt, 0), m);
    gstore_cols<RT, LOGB>(x, ca.limb(limb, log_n) + col0, bt);
  }
}

// Resident CTAs of `kernel` on the current device (the persistent grids).
template <typename KernelT>
uint32_t resident_ctas(KernelT kernel, int threads, size_t smem) {
  int dev = 0, sms = 0, per = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kernel, threads, smem) != cudaSuccess || per < 1)
    return 152;
  return (uint32_t)(sms * per);
}

// ===========================================================================
// Launch templates.  A variant is (degree, tile size T) for whole-limb
// degrees and (degree, column stages K1) for two-pass degrees.
// ===========================================================================
template <typename KernelT>
cudaError_t set_smem(KernelT kernel, size_t bytes) {
  return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}

// Whole-limb tile: 2^T words (T >= log_n); 16 words per thread (8 at N = 8).
template <int LOGN, int T>
using WholeCfg = TileCfg<T, LOGN, 0, (LOGN >= 4 ? 4 : 3)>;
// Two-pass tiles: 4096 words, 2^LOGE words per thread per round (radix-2^LOGE
// rounds): LOGE = 4 is 256 threads, LOGE = 3 is 512 threads per tile.
template <int LOGN, int K1, int LOGE = 4>
using ColCfg = TileCfg<kTileLog, K1, kTileLog - K1, LOGE>;
template <int LOGN, int K1, int LOGE = 4>
using RowCfg = TileCfg<kTileLog, LOGN - K1, 0, LOGE>;

constexpr size_t tile_bytes(int T) { return tile_smem_words(1u << T) * sizeof(uint64_t); }
constexpr size_t kTileSmemBytes = tile_bytes(kTileLog);

template <int LOGN, int T>
cudaError_t launch_whole_ntt(const LimbSet& ls, const DevMod* mods, NttDir dir, cudaStream_t st) {
  using C = WholeCfg<LOGN, T>;
  const uint32_t per = 1u << (T - LOGN);
  const uint32_t grid = (ls.count + per - 1) / per;
  const size_t smem = tile_bytes(T);
  LaunchScope ps(dir == NttDir::kBackward ? "ntt_whole_inv" : "ntt_whole_fwd", st);
  switch (dir) {
    case NttDir::kForward: k_ntt_whole<C, 0><<<grid, C::THREADS, smem, st>>>(ls, mods); break;
    case NttDir::kForwardLazy: k_ntt_whole<C, 1><<<grid, C::THREADS, smem, st>>>(ls, mods); break;
    case NttDir::kBackward: k_ntt_whole<C, 2><<<grid, C::THREADS, smem, st>>>(ls, mods); break;
  }
  g_kernel_launches += 1;
  return cudaGetLastError();
}

template <int LOGN, int T>
cudaError_t launch_whole_polymul(const LimbSet& c, const ConstLimbSet& a, const ConstLimbSet& b,
                                 const DevMod* mods, uint64_t*, uint64_t* const*, cudaStream_t st) {
  mods += kPolymulConsts;  // the fused polymul's copy of the constants
  using C = WholeCfg<LOGN, T>;
  const uint32_t per = 1u << (T - LOGN);
  const uint32_t grid = (c.count + per - 1) / per;
  LaunchScope ps("polymul_whole", st);
  k_polymul_whole<C><<<grid, C::THREADS, 2 * tile_bytes(T), st>>>(c, a, b, mods);
  g_kernel_launches += 1;
  return cudaGetLastError();
}

template <int LOGN, int T>
cudaError_t set_attrs_whole() {
  using C = WholeCfg<LOGN, T>;
  const size_t s = tile_bytes(T);
  cudaError_t e;
  if ((e = set_smem(k_ntt_whole<C, 0>, s)) != cudaSuccess) return e;
  if ((e = set_smem(k_ntt_whole<C, 1>, s)) != cudaSuccess) return e;
  if ((e = set_smem(k_ntt_whole<C, 2>, s)) != cudaSuccess) return e;
  return set_smem(k_polymul_whole<C>, 2 * s);
}

template <int LOGN, int K1, int LC = 4, int LR = 4>
cudaError_t launch_two_pass_ntt(const LimbSet& ls, const DevMod* mods, NttDir dir, cudaStream_t st) {
  constexpr int LOGB = LOGN - K1;
  using CC = ColCfg<LOGN, K1, LC>;
  using RC = RowCfg<LOGN, K1, LR>;
  const uint32_t tiles = ls.count << (LOGN - kTileLog);
  const ConstLimbSet cls = as_const(ls);
  if (dir == NttDir::kBackward) {
    {
      LaunchScope ps("row_pass_inv", st);
      launch_dependent(k_row_pass<RC, K1, true>, tiles, RC::THREADS, kTileSmemBytes, st, ls, mods, 0);
    }
    LaunchScope ps("col_pass_inv", st);
    launch_dependent(k_col_pass<CC, LOGB, true>, tiles, CC::THREADS, kTileSmemBytes, st, cls, ls, mods);
  } else {
    {
      LaunchScope ps("col_pass_fwd", st);
      launch_dependent(k_col_pass<CC, LOGB, false>, tiles, CC::THREADS, kTileSmemBytes, st, cls, ls, mods);
    }
    LaunchScope ps("row_pass_fwd", st);
    launch_dependent(k_row_pass<RC, K1, false>, tiles, RC::THREADS, kTileSmemBytes, st, ls, mods,
                     dir == NttDir::kForward ? 1 : 0);
  }
  g_kernel_launches += 2;
  return cudaGetLastError();
}

template <int LOGN, int K1, int LC = 4, int LR = 4>
cudaError_t launch_two_pass_polymul(const LimbSet& c, const ConstLimbSet& a, const ConstLimbSet& b,
                                    const DevMod* mods, uint64_t* scratch, uint64_t* const* scratch_ptrs,
                                    cudaStream_t st) {
  mods += kPolymulConsts;  // the fused polymul's copy of the constants
  constexpr int LOGB = LOGN - K1;
  using CC = ColCfg<LOGN, K1, LC>;
  using RC = RowCfg<LOGN, K1, LR>;
  const uint32_t tiles = c.count << (LOGN - kTileLog);
  LimbSet sl = c;
  sl.base = scratch_ptrs ? nullptr : scratch;
  sl.ptrs = scratch_ptrs;
  {
    LaunchScope ps("polymul_col_fwd", st);
    launch_dependent(k_col_pass2<CC, LOGB>, tiles, CC::THREADS, 2 * kTileSmemBytes, st, a, b, c, sl, mods);
  }
  {
    LaunchScope ps("polymul_rows", st);
    launch_dependent(k_polymul_rows<RC, K1>, tiles, RC::THREADS, 2 * kTileSmemBytes, st, c, as_const(sl), mods);
  }
  {
    LaunchScope ps("polymul_col_inv", st);
    launch_dependent(k_col_pass<CC, LOGB, true>, tiles, CC::THREADS, kTileSmemBytes, st, as_const(c), c, mods);
  }
  g_kernel_launches += 3;
  return cudaGetLastError();
}

template <int LOGN, int K1, int LC = 4, int LR = 4>
cudaError_t set_attrs_two_pass() {
  constexpr int LOGB = LOGN - K1;
  using CC = ColCfg<LOGN, K1, LC>;
  using RC = RowCfg<LOGN, K1, LR>;
  cudaError_t e;
  if ((e = set_smem(k_col_pass<CC, LOGB, false>, kTileSmemBytes)) != cudaSuccess) return e;
  if ((e = set_smem(k_col_pass<CC, LOGB, true>, kTileSmemBytes)) != cudaSuccess) return e;
  if ((e = set_smem(k_row_pass<RC, K1, false>, kTileSmemBytes)) != cudaSuccess) return e;
  if ((e = set_smem(k_row_pass<RC, K1, true>, kTileSmemBytes)) != cudaSuccess) return e;
  if ((e = set_smem(k_col_pass2<CC, LOGB>, 2 * kTileSmemBytes)) != cudaSuccess) return e;
  return set_smem(k_polymul_rows<RC, K1>, 2 * kTileSmemBytes);
}

// Persistent grid of a pipelined kernel: its resident CTAs on this device,
// computed once per device (the attributes are set before the first launch).
template <typename KernelT>
uint32_t persistent_grid(KernelT kernel, int threads, size_t smem, uint32_t tiles) {
  static std::atomic<uint32_t> cached[64];
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) dev = 0;
  uint32_t g = cached[dev].load(std::memory_order_relaxed);
  if (g == 0) {
    g = resident_ctas(kernel, threads, smem);
    cached[dev].store(g, std::memory_order_relaxed);
  }
  return g < tiles ? g : tiles;
}

template <int LOGN, int K1, int LC = 4, int LR = 4>
cudaError_t launch_two_pass_polymul_pipe(const LimbSet& c, const ConstLimbSet& a, const ConstLimbSet& b,
                                         const DevMod* mods, uint64_t* scratch, uint64_t* const* scratch_ptrs,
                                         cudaStream_t st) {
  mods += kPolymulConsts;  // the fused polymul's copy of the constants
  constexpr int LOGB = LOGN - K1;
  using CC = ColCfg<LOGN, K1, LC>;
  using RC = RowCfg<LOGN, K1, LR>;
  const uint32_t tiles = c.count << (LOGN - kTileLog);
  if (tiles == 0) return cudaSuccess;
  LimbSet sl = c;
  sl.base = scratch_ptrs ? nullptr : scratch;
  sl.ptrs = scratch_ptrs;
  {
    LaunchScope ps("polymul_col_fwd", st);
    const uint32_t g = persistent_grid(k_col_pass2_pipe<CC, LOGB>, CC::THREADS, 2 * kTileSmemBytes, tiles);
    k_col_pass2_pipe<CC, LOGB><<<g, CC::THREADS, 2 * kTileSmemBytes, st>>>(a, b, c, sl, mods, tiles);
  }
  {
    LaunchScope ps("polymul_rows", st);
    const uint32_t g = persistent_grid(k_polymul_rows_pipe<RC, K1>, RC::THREADS, 2 * kTileSmemBytes, tiles);
    k_polymul_rows_pipe<RC, K1><<<g, RC::THREADS, 2 * kTileSmemBytes, st>>>(c, as_const(sl), mods, tiles);
  }
  {
    LaunchScope ps("polymul_col_inv", st);
    const uint32_t g = persistent_grid(k_col_inv_pipe<CC, LOGB>, CC::THREADS, kTileSmemBytes, tiles);
    k_col_inv_pipe<CC, LOGB><<<g, CC::THREADS, kTileSmemBytes, st>>>(c, mods, tiles);
  }
  g_kernel_launches += 3;
  return cudaGetLastError();
}

template <int LOGN, int K1, int LC = 4, int LR = 4>
cudaError_t set_attrs_two_pass_pipe() {
  constexpr int LOGB = LOGN - K1;
  using CC = ColCfg<LOGN, K1, LC>;
  using RC = RowCfg<LOGN, K1, LR>;
  cudaError_t e;
  if ((e = set_attrs_two_pass<LOGN, K1, LC, LR>()) != cudaSuccess) return e;
  if ((e = set_smem(k_col_pass2_pipe<CC, LOGB>, 2 * kTileSmemBytes)) != cudaSuccess) return e;
  if ((e = set_smem(k_polymul_rows_pipe<RC, K1>, 2 * kTileSmemBytes)) != cudaSuccess) return e;
  return set_smem(k_col_inv_pipe<CC, LOGB>, kTileSmemBytes);
}

template <int LOGN, int T>
Variant whole_variant() {
  Variant v;
  std::snprintf(v.name, sizeof(v.name), "whole-limb tile 2^%d (%d threads, %d limbs/CTA)", T,
                1 << (T - (LOGN >= 4 ? 4 : 3)), 1 << (T - LOGN));
  v.ntt = &launch_whole_ntt<LOGN, T>;
  v.polymul = &launch_whole_polymul<LOGN, T>;
  v.set_attrs = &set_attrs_whole<LOGN, T>;
  v.ntt_launches = 1;
  v.polymul_launches = 1;
  return v;
}

// Named "two-pass k1=K1 (...)"; variants whose column or row tiles use other
// than 16 words per thread name both word counts.
template <int LOGN, int K1, int LC = 4, int LR = 4>
Variant two_pass_variant() {
  Variant v;
  if (LC == 4 && LR == 4)
    std::snprintf(v.name, sizeof(v.name), "two-pass k1=%d (columns of 2^%d, rows of 2^%d)", K1, K1, LOGN - K1);
  else
    std::snprintf(v.name, sizeof(v.name), "two-pass k1=%d (columns of 2^%d, rows of 2^%d; %d/%d words per thread)",
                  K1, K1, LOGN - K1, 1 << LC, 1 << LR);
  v.ntt = &launch_two_pass_ntt<LOGN, K1, LC, LR>;
  v.polymul = &launch_two_pass_polymul<LOGN, K1, LC, LR>;
  v.set_attrs = &set_attrs_two_pass<LOGN, K1, LC, LR>;
  v.ntt_launches = 2;
  v.polymul_launches = 3;
  v.polymul_scratch = true;
  return v;
}

// The same split with the pipelined (persistent, copy-ahead) polymul kernels;
// the NTT keeps the one-tile-per-CTA kernels.
template <int LOGN, int K1, int LC = 4, int LR = 4>
Variant two_pass_pipe_variant() {
  Variant v = two_pass_variant<LOGN, K1, LC, LR>();
  const size_t n = std::strlen(v.name);
  std::snprintf(v.name + n - 1, sizeof(v.name) - (n - 1), "; pipelined)");
  v.polymul = &launch_two_pass_polymul_pipe<LOGN, K1, LC, LR>;
  v.set_attrs = &set_attrs_two_pass_pipe<LOGN, K1, LC, LR>;
  return v;
}

}  // namespace
}  // namespace yell_gb300
