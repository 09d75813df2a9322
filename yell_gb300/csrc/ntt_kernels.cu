// NTT, fused polymul and element-wise kernels for sm_103a.
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
//   * fused polymul: NTT(a), NTT(b), Barrett product and INTT in one kernel
//     (whole-limb) or three (two-pass: column pass of a and b, then one row
//     kernel doing forward rows of both, the product and inverse rows, then
//     the inverse column pass).  The last forward round of both operands,
//     the product and the first inverse round share one register set.
#include "kernels.h"
#include "ntt_tile.cuh"

namespace yell_gb300 {

namespace {

constexpr uint32_t kTwoPassTileLog = 12;  // 4096 words per two-pass tile
constexpr uint32_t kTwoPassThreads = 1u << (kTwoPassTileLog - 4);

__device__ __forceinline__ ulonglong2 ld_pair(const uint64_t* p) {
  return __ldg(reinterpret_cast<const ulonglong2*>(p));
}

__device__ __forceinline__ void st_pair(uint64_t* p, uint64_t a, uint64_t b) {
  *reinterpret_cast<ulonglong2*>(p) = make_ulonglong2(a, b);
}

// ---------------------------------------------------------------------------
// Whole-limb NTT.  Tile of 2^T words = 2^(T - log_n) limbs; 2^(T - LOGE)
// threads.  dir: 0 forward (reduced), 1 forward lazy, 2 backward.
// ---------------------------------------------------------------------------
template <int LOGE>
__global__ void __launch_bounds__(512) k_ntt_whole(LimbSet ls, uint32_t log_n, uint32_t T,
                                                   const DevMod* __restrict__ mods, int dir) {
  extern __shared__ __align__(16) uint64_t smem[];
  const uint32_t tid = threadIdx.x;
  const uint32_t K = log_n, N = 1u << K, words = 1u << T;
  const uint32_t limb0 = blockIdx.x << (T - K);
  for (uint32_t v = tid * 2; v < words; v += blockDim.x * 2) {
    const uint32_t limb = limb0 + (v >> K);
    if (limb < ls.count) {
      const ulonglong2 d = ld_pair(ls.limb(limb, log_n) + (v & (N - 1)));
      smem[sidx(v)] = d.x;
      smem[sidx(v + 1)] = d.y;
    }
  }
  __syncthreads();
  const uint32_t my_limb = limb0 + (tid >> (K - LOGE));
  const bool active = my_limb < ls.count;
  const DevMod m = load_mod(mods, ls.cm(active ? my_limb : 0));
  if (dir == 2)
    inv_tile<LOGE>(smem, tid, 0, K, log_n, 0, 0, m, active, true);
  else
    fwd_tile<LOGE>(smem, tid, 0, K, 0, 0, m.fwd, m.p, active);
  for (uint32_t v = tid * 2; v < words; v += blockDim.x * 2) {
    const uint32_t limb = limb0 + (v >> K);
    if (limb < ls.count) {
      uint64_t a = smem[sidx(v)], b = smem[sidx(v + 1)];
      if (dir == 0) {
        const uint64_t p = __ldg(&mods[ls.cm(limb)].p);
        a = fwd_correct(a, p, p << 1);
        b = fwd_correct(b, p, p << 1);
      }
      st_pair(ls.limb(limb, log_n) + (v & (N - 1)), a, b);
    }
  }
}

// ---------------------------------------------------------------------------
// Two-pass: column pass.  Tile = C x ncols words, C = 2^k1, ncols = 2^lb,
// lb = 12 - k1; tile word v = c * ncols + col is global word c*B + col0 + col.
// Forward: stages 0..k1-1.  Inverse: stages log2(B)..log_n-1 ending with the
// scaled last layer.  src and dst may be the same limbs (in place).
// ---------------------------------------------------------------------------
template <bool INV>
__global__ void __launch_bounds__(256) k_col_pass(ConstLimbSet src, LimbSet dst, uint32_t log_n,
                                                  uint32_t k1, const DevMod* __restrict__ mods) {
  extern __shared__ __align__(16) uint64_t smem[];
  const uint32_t tid = threadIdx.x;
  const uint32_t lb = kTwoPassTileLog - k1, logB = log_n - k1;
  const uint32_t tpl_log = logB - lb;  // log2(tiles per limb)
  const uint32_t limb = blockIdx.x >> tpl_log;
  const uint32_t col0 = (blockIdx.x & ((1u << tpl_log) - 1u)) << lb;
  const uint64_t* in = src.limb(limb, log_n);
  uint64_t* out = dst.limb(limb, log_n);
  const uint32_t cmask = (1u << lb) - 1u;
  for (uint32_t v = tid * 2; v < (1u << kTwoPassTileLog); v += kTwoPassThreads * 2) {
    const ulonglong2 d = ld_pair(in + ((size_t)(v >> lb) << logB) + col0 + (v & cmask));
    smem[sidx(v)] = d.x;
    smem[sidx(v + 1)] = d.y;
  }
  __syncthreads();
  const DevMod m = load_mod(mods, dst.cm(limb));
  if (INV)
    inv_tile<4>(smem, tid, lb, k1, log_n, logB, 0, m, true, true);
  else
    fwd_tile<4>(smem, tid, lb, k1, 0, 0, m.fwd, m.p, true);
  for (uint32_t v = tid * 2; v < (1u << kTwoPassTileLog); v += kTwoPassThreads * 2)
    st_pair(out + ((size_t)(v >> lb) << logB) + col0 + (v & cmask), smem[sidx(v)], smem[sidx(v + 1)]);
}

// ---------------------------------------------------------------------------
// Two-pass: row pass over 4096 contiguous words (4096 / B blocks of B).
// Forward: stages k1..log_n-1 (+ the reduction of ntt::forward when
// fwd_full); inverse: stages 0..log2(B)-1.  In place.
// ---------------------------------------------------------------------------
template <bool INV>
__global__ void __launch_bounds__(256) k_row_pass(LimbSet ls, uint32_t log_n, uint32_t k1,
                                                  const DevMod* __restrict__ mods, int fwd_full) {
  extern __shared__ __align__(16) uint64_t smem[];
  const uint32_t tid = threadIdx.x;
  const uint32_t logB = log_n - k1;
  const uint32_t tpl_log = log_n - kTwoPassTileLog;
  const uint32_t limb = blockIdx.x >> tpl_log;
  const uint32_t off = (blockIdx.x & ((1u << tpl_log) - 1u)) << kTwoPassTileLog;
  uint64_t* data = ls.limb(limb, log_n) + off;
  for (uint32_t v = tid * 2; v < (1u << kTwoPassTileLog); v += kTwoPassThreads * 2) {
    const ulonglong2 d = ld_pair(data + v);
    smem[sidx(v)] = d.x;
    smem[sidx(v + 1)] = d.y;
  }
  __syncthreads();
  const DevMod m = load_mod(mods, ls.cm(limb));
  const uint32_t G = (off >> logB) + (tid >> (logB - 4));
  if (INV)
    inv_tile<4>(smem, tid, 0, logB, log_n, 0, G, m, true, false);
  else
    fwd_tile<4>(smem, tid, 0, logB, k1, G, m.fwd, m.p, true);
  const uint64_t p = m.p, p2 = m.p << 1;
  for (uint32_t v = tid * 2; v < (1u << kTwoPassTileLog); v += kTwoPassThreads * 2) {
    uint64_t a = smem[sidx(v)], b = smem[sidx(v + 1)];
    if (!INV && fwd_full) {
      a = fwd_correct(a, p, p2);
      b = fwd_correct(b, p, p2);
    }
    st_pair(data + v, a, b);
  }
}

// ---------------------------------------------------------------------------
// Fused product step shared by both polymul kernels: the last forward round
// (R = LOGE at bit 0) of both operands, the reduction of ntt::forward, the
// Barrett product of ops::mulmod and the first inverse round (R = LOGE at bit
// 0), all on one register set; the result goes back to sa.
// ---------------------------------------------------------------------------
template <int LOGE>
__device__ __forceinline__ void fused_product_round(uint64_t* sa, const uint64_t* sb, uint32_t tid,
                                                    uint32_t K, uint32_t log_n, uint32_t s_off,
                                                    uint32_t G, const DevMod& m, bool active,
                                                    bool inv_last) {
  constexpr int E = 1 << LOGE;
  if (!active) return;
  const uint32_t base = thread_base<LOGE, LOGE>(tid, 0, 0);
  const uint32_t hi_bits = K - LOGE;
  const uint32_t u_hi = (base >> LOGE) & ((1u << hi_bits) - 1u);
  const uint32_t gr = (G << hi_bits) + u_hi;
  const uint64_t p = m.p, p2 = m.p << 1;
  uint64_t xa[E], xb[E];
  load_regs<LOGE, LOGE>(xa, sa, base, 0, 0);
  ct_round<LOGE, LOGE>(xa, s_off + hi_bits, gr, m.fwd, p, p2);
  load_regs<LOGE, LOGE>(xb, sb, base, 0, 0);
  ct_round<LOGE, LOGE>(xb, s_off + hi_bits, gr, m.fwd, p, p2);
#pragma unroll
  for (int i = 0; i < E; ++i)
    xa[i] = mulmod_barrett(fwd_correct(xa[i], p, p2), fwd_correct(xb[i], p, p2), p, m.pn);
  if (inv_last)
    gs_round<LOGE, LOGE, true>(xa, log_n, 0, gr, m.inv, m);
  else
    gs_round<LOGE, LOGE, false>(xa, log_n, 0, gr, m.inv, m);
  store_regs<LOGE, LOGE>(xa, sa, base, 0, 0);
}

// Whole-limb fused polymul: c = INTT(NTT(a) * NTT(b)), N <= 2^13.
template <int LOGE>
__global__ void __launch_bounds__(512) k_polymul_whole(LimbSet c, ConstLimbSet a, ConstLimbSet b,
                                                       uint32_t log_n, uint32_t T,
                                                       const DevMod* __restrict__ mods) {
  extern __shared__ __align__(16) uint64_t smem[];
  uint64_t* sa = smem;
  uint64_t* sb = smem + padded_words(1u << T);
  const uint32_t tid = threadIdx.x;
  const uint32_t K = log_n, N = 1u << K, words = 1u << T;
  const uint32_t limb0 = blockIdx.x << (T - K);
  for (uint32_t v = tid * 2; v < words; v += blockDim.x * 2) {
    const uint32_t limb = limb0 + (v >> K);
    if (limb < c.count) {
      const ulonglong2 da = ld_pair(a.limb(limb, log_n) + (v & (N - 1)));
      const ulonglong2 db = ld_pair(b.limb(limb, log_n) + (v & (N - 1)));
      sa[sidx(v)] = da.x;
      sa[sidx(v + 1)] = da.y;
      sb[sidx(v)] = db.x;
      sb[sidx(v + 1)] = db.y;
    }
  }
  __syncthreads();
  const uint32_t my_limb = limb0 + (tid >> (K - LOGE));
  const bool active = my_limb < c.count;
  const DevMod m = load_mod(mods, c.cm(active ? my_limb : 0));
  const RoundPlan fp = make_plan(K, LOGE, false);
  for (uint32_t r = 0; r + 1 < fp.n; ++r) {
    uint32_t R, beta;
    fp.geom(r, R, beta);
    fwd_round<LOGE>(sa, tid, 0, K, R, beta, 0, 0, m.fwd, m.p, active);
    fwd_round<LOGE>(sb, tid, 0, K, R, beta, 0, 0, m.fwd, m.p, active);
    __syncthreads();
  }
  fused_product_round<LOGE>(sa, sb, tid, K, log_n, 0, 0, m, active, fp.n == 1);
  __syncthreads();
  const RoundPlan ip = make_plan(K, LOGE, true);
  for (uint32_t r = 1; r < ip.n; ++r) {
    uint32_t R, beta;
    ip.geom(r, R, beta);
    inv_round<LOGE>(sa, tid, 0, K, R, beta, log_n, 0, 0, m, active, r + 1 == ip.n);
    __syncthreads();
  }
  for (uint32_t v = tid * 2; v < words; v += blockDim.x * 2) {
    const uint32_t limb = limb0 + (v >> K);
    if (limb < c.count) st_pair(c.limb(limb, log_n) + (v & (N - 1)), sa[sidx(v)], sa[sidx(v + 1)]);
  }
}

// Two-pass fused row step: ca holds a's column-pass output and receives the
// row-pass output of the product; sbuf holds b's column-pass output.
__global__ void __launch_bounds__(256, 2) k_polymul_rows(LimbSet ca, ConstLimbSet sbuf,
                                                         uint32_t log_n, uint32_t k1,
                                                         const DevMod* __restrict__ mods) {
  extern __shared__ __align__(16) uint64_t smem[];
  uint64_t* sa = smem;
  uint64_t* sb = smem + padded_words(1u << kTwoPassTileLog);
  const uint32_t tid = threadIdx.x;
  const uint32_t logB = log_n - k1;
  const uint32_t tpl_log = log_n - kTwoPassTileLog;
  const uint32_t limb = blockIdx.x >> tpl_log;
  const uint32_t off = (blockIdx.x & ((1u << tpl_log) - 1u)) << kTwoPassTileLog;
  uint64_t* pa = ca.limb(limb, log_n) + off;
  const uint64_t* pb = sbuf.limb(limb, log_n) + off;
  for (uint32_t v = tid * 2; v < (1u << kTwoPassTileLog); v += kTwoPassThreads * 2) {
    const ulonglong2 da = ld_pair(pa + v);
    const ulonglong2 db = ld_pair(pb + v);
    sa[sidx(v)] = da.x;
    sa[sidx(v + 1)] = da.y;
    sb[sidx(v)] = db.x;
    sb[sidx(v + 1)] = db.y;
  }
  __syncthreads();
  const DevMod m = load_mod(mods, ca.cm(limb));
  const uint32_t G = (off >> logB) + (tid >> (logB - 4));
  const RoundPlan fp = make_plan(logB, 4, false);
  for (uint32_t r = 0; r + 1 < fp.n; ++r) {
    uint32_t R, beta;
    fp.geom(r, R, beta);
    fwd_round<4>(sa, tid, 0, logB, R, beta, k1, G, m.fwd, m.p, true);
    fwd_round<4>(sb, tid, 0, logB, R, beta, k1, G, m.fwd, m.p, true);
    __syncthreads();
  }
  fused_product_round<4>(sa, sb, tid, logB, log_n, k1, G, m, true, false);
  __syncthreads();
  const RoundPlan ip = make_plan(logB, 4, true);
  for (uint32_t r = 1; r < ip.n; ++r) {
    uint32_t R, beta;
    ip.geom(r, R, beta);
    inv_round<4>(sa, tid, 0, logB, R, beta, log_n, 0, G, m, true, false);
    __syncthreads();
  }
  for (uint32_t v = tid * 2; v < (1u << kTwoPassTileLog); v += kTwoPassThreads * 2)
    st_pair(pa + v, sa[sidx(v)], sa[sidx(v + 1)]);
}

// ---------------------------------------------------------------------------
// Element-wise ops, two words per thread with 128-bit accesses.
// ---------------------------------------------------------------------------
template <int OP>
__global__ void __launch_bounds__(256) k_elementwise(LimbSet dst, ConstLimbSet a, ConstLimbSet b,
                                                     uint32_t log_n, const DevMod* __restrict__ mods) {
  const size_t pairs = ((size_t)dst.count << log_n) >> 1;
  const uint32_t nmask = (1u << log_n) - 1u;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < pairs;
       i += (size_t)gridDim.x * blockDim.x) {
    const size_t v = i * 2;
    const uint32_t limb = (uint32_t)(v >> log_n);
    const uint32_t off = (uint32_t)v & nmask;
    const uint32_t cm = dst.cm(limb);
    const uint64_t p = __ldg(&mods[cm].p);
    const ulonglong2 x = ld_pair(a.limb(limb, log_n) + off);
    uint64_t* d = dst.limb(limb, log_n) + off;
    uint64_t r0, r1;
    if (OP == (int)EwOp::kNegate) {
      r0 = p - x.x;
      r1 = p - x.y;
    } else {
      const ulonglong2 y = ld_pair(b.limb(limb, log_n) + off);
      if (OP == (int)EwOp::kAddmod) {
        r0 = addmod(x.x, y.x, p);
        r1 = addmod(x.y, y.y, p);
      } else if (OP == (int)EwOp::kSubmod) {
        r0 = submod(x.x, y.x, p);
        r1 = submod(x.y, y.y, p);
      } else {
        const uint64_t pn = __ldg(&mods[cm].pn);
        if (OP == (int)EwOp::kMulmod) {
          r0 = mulmod_barrett(x.x, y.x, p, pn);
          r1 = mulmod_barrett(x.y, y.y, p, pn);
        } else {
          const ulonglong2 acc = *reinterpret_cast<const ulonglong2*>(d);
          r0 = muladd_barrett(acc.x, x.x, y.x, p, pn);
          r1 = muladd_barrett(acc.y, x.y, y.y, p, pn);
        }
      }
    }
    st_pair(d, r0, r1);
  }
}

int g_num_sms = 0;

int num_sms() {
  if (g_num_sms == 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&g_num_sms, cudaDevAttrMultiProcessorCount, dev);
    if (g_num_sms <= 0) g_num_sms = 1;
  }
  return g_num_sms;
}

template <typename KernelT>
cudaError_t set_smem(KernelT kernel, size_t bytes) {
  return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}

inline uint32_t whole_tile_log(uint32_t log_n) { return log_n > 12 ? log_n : 12u; }
inline int whole_loge(uint32_t log_n) { return log_n >= 4 ? 4 : 3; }

ConstLimbSet as_const(const LimbSet& l) {
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

}  // namespace

uint32_t default_k1(uint32_t log_n) {
  uint32_t k1 = log_n / 2;
  return k1 > 8 ? 8u : k1;
}

static uint32_t pick_k1(uint32_t log_n, const NttShape& shape) {
  uint32_t k1 = shape.k1 ? shape.k1 : default_k1(log_n);
  // column tiles need >= 2 columns (lb >= 1) and rows must fit a 4096-word tile
  if (k1 > kTwoPassTileLog - 1) k1 = kTwoPassTileLog - 1;
  if (log_n - k1 > kTwoPassTileLog) k1 = log_n - kTwoPassTileLog;
  if (log_n - k1 < 4) k1 = log_n - 4;
  return k1;
}

static bool use_whole(uint32_t log_n, const NttShape& shape) {
  return log_n <= shape.single_cta_max_log_n && log_n <= 13;
}

cudaError_t launch_ntt(const LimbSet& ls, uint32_t log_n, const DevMod* mods, NttDir dir,
                       const NttShape& shape, cudaStream_t st) {
  if (ls.count == 0) return cudaSuccess;
  if (use_whole(log_n, shape)) {
    const uint32_t T = whole_tile_log(log_n);
    const uint32_t grid = (ls.count + (1u << (T - log_n)) - 1) >> (T - log_n);
    const size_t smem = padded_words(1u << T) * sizeof(uint64_t);
    if (whole_loge(log_n) == 4) {
      k_ntt_whole<4><<<grid, 1u << (T - 4), smem, st>>>(ls, log_n, T, mods, (int)dir);
    } else {
      k_ntt_whole<3><<<grid, 1u << (T - 3), smem, st>>>(ls, log_n, T, mods, (int)dir);
    }
    g_kernel_launches += 1;
    return cudaGetLastError();
  }
  const uint32_t k1 = pick_k1(log_n, shape);
  const size_t smem = padded_words(1u << kTwoPassTileLog) * sizeof(uint64_t);
  const uint32_t tiles = ls.count << (log_n - kTwoPassTileLog);
  const ConstLimbSet cls = as_const(ls);
  if (dir == NttDir::kBackward) {
    k_row_pass<true><<<tiles, kTwoPassThreads, smem, st>>>(ls, log_n, k1, mods, 0);
    k_col_pass<true><<<tiles, kTwoPassThreads, smem, st>>>(cls, ls, log_n, k1, mods);
  } else {
    k_col_pass<false><<<tiles, kTwoPassThreads, smem, st>>>(cls, ls, log_n, k1, mods);
    k_row_pass<false><<<tiles, kTwoPassThreads, smem, st>>>(ls, log_n, k1, mods,
                                                            dir == NttDir::kForward ? 1 : 0);
  }
  g_kernel_launches += 2;
  return cudaGetLastError();
}

cudaError_t init_kernel_attributes() {
  const size_t whole = padded_words(1u << 13) * sizeof(uint64_t);
  const size_t tile = padded_words(1u << kTwoPassTileLog) * sizeof(uint64_t);
  cudaError_t e;
  if ((e = set_smem(k_ntt_whole<4>, whole)) != cudaSuccess) return e;
  if ((e = set_smem(k_ntt_whole<3>, whole)) != cudaSuccess) return e;
  if ((e = set_smem(k_polymul_whole<4>, 2 * whole)) != cudaSuccess) return e;
  if ((e = set_smem(k_polymul_whole<3>, 2 * whole)) != cudaSuccess) return e;
  if ((e = set_smem(k_polymul_rows, 2 * tile)) != cudaSuccess) return e;
  if ((e = set_smem(k_col_pass<false>, tile)) != cudaSuccess) return e;
  if ((e = set_smem(k_col_pass<true>, tile)) != cudaSuccess) return e;
  if ((e = set_smem(k_row_pass<false>, tile)) != cudaSuccess) return e;
  if ((e = set_smem(k_row_pass<true>, tile)) != cudaSuccess) return e;
  return cudaSuccess;
}

uint32_t ntt_launch_count(uint32_t log_n, const NttShape& shape) {
  return use_whole(log_n, shape) ? 1u : 2u;
}

uint32_t polymul_launch_count(uint32_t log_n, const NttShape& shape) {
  return use_whole(log_n, shape) ? 1u : 4u;
}

size_t polymul_scratch_words(uint32_t count, uint32_t log_n, const NttShape& shape) {
  return use_whole(log_n, shape) ? 0 : ((size_t)count << log_n);
}

cudaError_t launch_polymul(const LimbSet& c, const ConstLimbSet& a, const ConstLimbSet& b,
                           uint32_t log_n, const DevMod* mods, uint64_t* scratch,
                           const NttShape& shape, cudaStream_t st) {
  if (c.count == 0) return cudaSuccess;
  if (use_whole(log_n, shape)) {
    const uint32_t T = whole_tile_log(log_n);
    const uint32_t grid = (c.count + (1u << (T - log_n)) - 1) >> (T - log_n);
    const size_t smem = 2 * padded_words(1u << T) * sizeof(uint64_t);
    if (whole_loge(log_n) == 4) {
      k_polymul_whole<4><<<grid, 1u << (T - 4), smem, st>>>(c, a, b, log_n, T, mods);
    } else {
      k_polymul_whole<3><<<grid, 1u << (T - 3), smem, st>>>(c, a, b, log_n, T, mods);
    }
    g_kernel_launches += 1;
    return cudaGetLastError();
  }
  if (scratch == nullptr) return cudaErrorInvalidValue;
  const uint32_t k1 = pick_k1(log_n, shape);
  const size_t smem = padded_words(1u << kTwoPassTileLog) * sizeof(uint64_t);
  const uint32_t tiles = c.count << (log_n - kTwoPassTileLog);
  LimbSet sl = c;
  sl.base = scratch;
  sl.ptrs = nullptr;
  k_col_pass<false><<<tiles, kTwoPassThreads, smem, st>>>(a, c, log_n, k1, mods);
  k_col_pass<false><<<tiles, kTwoPassThreads, smem, st>>>(b, sl, log_n, k1, mods);
  k_polymul_rows<<<tiles, kTwoPassThreads, 2 * smem, st>>>(c, as_const(sl), log_n, k1, mods);
  k_col_pass<true><<<tiles, kTwoPassThreads, smem, st>>>(as_const(c), c, log_n, k1, mods);
  g_kernel_launches += 4;
  return cudaGetLastError();
}

cudaError_t launch_elementwise(EwOp op, const LimbSet& dst, const ConstLimbSet& a,
                               const ConstLimbSet& b, uint32_t log_n, const DevMod* mods,
                               cudaStream_t st) {
  if (dst.count == 0) return cudaSuccess;
  const size_t pairs = ((size_t)dst.count << log_n) >> 1;
  const size_t want = (pairs + 255) / 256;
  const size_t cap = (size_t)num_sms() * 8;
  const uint32_t grid = (uint32_t)(want < cap ? want : cap);
  switch (op) {
    case EwOp::kMulmod: k_elementwise<0><<<grid, 256, 0, st>>>(dst, a, b, log_n, mods); break;
    case EwOp::kAddmod: k_elementwise<1><<<grid, 256, 0, st>>>(dst, a, b, log_n, mods); break;
    case EwOp::kSubmod: k_elementwise<2><<<grid, 256, 0, st>>>(dst, a, b, log_n, mods); break;
    case EwOp::kMuladd: k_elementwise<3><<<grid, 256, 0, st>>>(dst, a, b, log_n, mods); break;
    case EwOp::kNegate: k_elementwise<4><<<grid, 256, 0, st>>>(dst, a, b, log_n, mods); break;
  }
  g_kernel_launches += 1;
  return cudaGetLastError();
}

}  // namespace yell_gb300
