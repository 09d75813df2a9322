// Shared device arithmetic and descriptors for the YELL GB300 kernels.
//
// Residues are uint64 words modulo 62-bit primes p (p < 2^62), exactly as in
// the reference (include/yell/params_64.hpp:19-24).  Every formula below is
// the reference's own, evaluated with the same wrap-around uint64 semantics,
// so a kernel that applies the same sequence of butterflies produces the same
// words as the reference, not just the same residues.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace yell_gb300 {

// Per-(log_n, cm) constants resident on the device.  fwd/inv point at N
// {w, w'} pairs in the reference's bit-reversed order
// (include/yell/details/ntt.hpp:45-71): fwd = phiTbl/shoupPhiTbl,
// inv = invphiTbl/shoupInvphiTbl.
struct alignas(16) DevMod {
  const ulonglong2* fwd;
  const ulonglong2* inv;
  uint64_t p;
  uint64_t pn;               // low word of floor(2^128/p) (params_64.hpp:29-31)
  uint64_t inv_n, inv_n_s;   // N^-1 and its Shoup form (include/yell/details/ntt.hpp:73,75)
  uint64_t inv_n_iphi, inv_n_iphi_s;  // N^-1 * invphiTbl[1] and Shoup form (include/yell/details/ntt.hpp:74,76)
};

// Which limbs a launch touches.  Limb k of the launch lives at
// ptrs ? ptrs[k] : base + k * N, and uses modulus index
// cms ? cms[k] : cm0 + k % L.
struct LimbSet {
  uint64_t* base;
  uint64_t* const* ptrs;
  const uint32_t* cms;
  uint32_t count;
  uint32_t L;
  uint32_t cm0;
  uint32_t pad_;

  __device__ __forceinline__ uint64_t* limb(uint32_t k, uint32_t log_n) const {
    return ptrs ? ptrs[k] : base + ((size_t)k << log_n);
  }
  __device__ __forceinline__ uint32_t cm(uint32_t k) const {
    return cms ? cms[k] : cm0 + k % L;
  }
  // Launch order -> limb index.  Contiguous batches of whole polys are
  // visited modulus-major (limb l of every poly, then limb l + 1), so the
  // twiddle table of one prime stays resident in L2 while it is in use.
  __device__ __forceinline__ uint32_t ordered(uint32_t i) const {
    if (ptrs || L <= 1 || count % L != 0) return i;
    const uint32_t polys = count / L;
    return (i % polys) * L + i / polys;
  }
};

struct ConstLimbSet {
  const uint64_t* base;
  const uint64_t* const* ptrs;
  const uint32_t* cms;
  uint32_t count;
  uint32_t L;
  uint32_t cm0;
  uint32_t pad_;

  __device__ __forceinline__ const uint64_t* limb(uint32_t k, uint32_t log_n) const {
    return ptrs ? ptrs[k] : base + ((size_t)k << log_n);
  }
};

// ---------------------------------------------------------------------------
// Modular arithmetic.  64-bit products are formed from 32-bit IMAD/IMAD.HI by
// the compiler; there is no 64-bit multiplier on the SM.
// ---------------------------------------------------------------------------

// lo64(a*w + q*np) from 32-bit IMAD.WIDE / IMAD: with np = 2^64 - p this is
// a*w - q*p (mod 2^64) without a 64-bit subtraction.
__device__ __forceinline__ uint64_t lo_mul_add(uint64_t a, uint64_t w, uint64_t q, uint64_t np) {
  uint64_t r;
  asm("{\n\t"
      ".reg .u32 a0, a1, w0, w1, q0, q1, n0, n1, rl, rh;\n\t"
      ".reg .u64 t;\n\t"
      "mov.b64 {a0, a1}, %1;\n\t"
      "mov.b64 {w0, w1}, %2;\n\t"
      "mov.b64 {q0, q1}, %3;\n\t"
      "mov.b64 {n0, n1}, %4;\n\t"
      "mul.wide.u32 t, a0, w0;\n\t"
      "mad.wide.u32 t, q0, n0, t;\n\t"
      "mov.b64 {rl, rh}, t;\n\t"
      "mad.lo.u32 rh, a0, w1, rh;\n\t"
      "mad.lo.u32 rh, a1, w0, rh;\n\t"
      "mad.lo.u32 rh, q0, n1, rh;\n\t"
      "mad.lo.u32 rh, q1, n0, rh;\n\t"
      "mov.b64 %0, {rl, rh};\n\t"
      "}"
      : "=l"(r)
      : "l"(a), "l"(w), "l"(q), "l"(np));
  return r;
}

// u >= m ? u - m : u, as a borrow mask and a bitwise select per 32-bit half.
__device__ __forceinline__ uint64_t csub(uint64_t u, uint64_t m) {
  uint64_t r;
  asm("{\n\t"
      ".reg .u32 ul, uh, ml, mh, dl, dh, b;\n\t"
      "mov.b64 {ul, uh}, %1;\n\t"
      "mov.b64 {ml, mh}, %2;\n\t"
      "sub.cc.u32 dl, ul, ml;\n\t"
      "subc.cc.u32 dh, uh, mh;\n\t"
      "subc.u32 b, 0, 0;\n\t"
      "lop3.b32 dl, ul, dl, b, 0xE4;\n\t"
      "lop3.b32 dh, uh, dh, b, 0xE4;\n\t"
      "mov.b64 %0, {dl, dh};\n\t"
      "}"
      : "=l"(r)
      : "l"(u), "l"(m));
  return r;
}

// hi64(a*b) as one carry chain of 32-bit multiply-adds (the low word of the
// product is never formed; only its carries are).  Same value as
// __umul64hi; in the Gentleman-Sande butterfly, where the multiplicand is
// computed just before, it schedules better (8% more register-resident GS
// butterflies per second on GB300; 2% fewer CT ones, which keep __umul64hi).
__device__ __forceinline__ uint64_t hi64_chain(uint64_t a, uint64_t b) {
  uint64_t r;
  asm("{\n\t"
      ".reg .u32 a0, a1, b0, b1, t1, t2, t3;\n\t"
      "mov.b64 {a0, a1}, %1;\n\t"
      "mov.b64 {b0, b1}, %2;\n\t"
      "mul.hi.u32 t1, a0, b0;\n\t"
      "mad.lo.cc.u32 t1, a0, b1, t1;\n\t"
      "madc.hi.cc.u32 t2, a0, b1, 0;\n\t"
      "addc.u32 t3, 0, 0;\n\t"
      "mad.lo.cc.u32 t1, a1, b0, t1;\n\t"
      "madc.hi.cc.u32 t2, a1, b0, t2;\n\t"
      "addc.u32 t3, t3, 0;\n\t"
      "mad.lo.cc.u32 t2, a1, b1, t2;\n\t"
      "madc.hi.u32 t3, a1, b1, t3;\n\t"
      "mov.b64 %0, {t2, t3};\n\t"
      "}"
      : "=l"(r)
      : "l"(a), "l"(b));
  return r;
}

// Shoup product with the precomputed companion w' = floor(w * 2^64 / p):
// x*w - hi64(x*w')*p (mod 2^64).  For x < 2^64 the value lies in [0, 2p).
// lib/ntt.cpp:59-62 (GS) and :79-80 (CT).  np = 2^64 - p.
__device__ __forceinline__ uint64_t shoup_lazy(uint64_t x, uint64_t w, uint64_t wp, uint64_t np) {
  return lo_mul_add(x, w, __umul64hi(x, wp), np);
}

__device__ __forceinline__ uint64_t shoup_lazy_gs(uint64_t x, uint64_t w, uint64_t wp, uint64_t np) {
  return lo_mul_add(x, w, hi64_chain(x, wp), np);
}

// Cooley-Tukey butterfly, lib/ntt.cpp:69-83.  In/out [0, 4p).
__device__ __forceinline__ void ct_bfly(uint64_t& x0, uint64_t& x1, uint64_t w, uint64_t wp,
                                        uint64_t np, uint64_t p2) {
  const uint64_t u0 = csub(x0, p2);
  const uint64_t t = shoup_lazy(x1, w, wp, np);
  x0 = u0 + t;
  x1 = u0 - t + p2;
}

// Gentleman-Sande butterfly, lib/ntt.cpp:47-63.  In/out [0, 2p).
__device__ __forceinline__ void gs_bfly(uint64_t& x0, uint64_t& x1, uint64_t w, uint64_t wp,
                                        uint64_t np, uint64_t p2) {
  const uint64_t u0 = x0, u1 = x1;
  const uint64_t t1 = u0 - u1 + p2;
  x0 = csub(u0 + u1, p2);
  x1 = shoup_lazy_gs(t1, w, wp, np);
}

// ops::mulmod_shoup, include/yell/ops.hpp:122-132: Shoup product plus one
// conditional subtraction of p.
__device__ __forceinline__ uint64_t mulmod_shoup(uint64_t x, uint64_t y, uint64_t yp, uint64_t p) {
  return csub(shoup_lazy(x, y, yp, 0 - p), p);
}

// Last inverse layer with the N^-1 scaling fused in,
// include/yell/details/ntt.hpp:144-159.
__device__ __forceinline__ void gs_last(uint64_t& x0, uint64_t& x1, const DevMod& m) {
  const uint64_t u = x0, v = x1;
  x0 = mulmod_shoup(u + v, m.inv_n, m.inv_n_s, m.p);
  x1 = mulmod_shoup(u - v + (m.p << 1), m.inv_n_iphi, m.inv_n_iphi_s, m.p);
}

// Final correction of ntt<N>::forward, include/yell/details/ntt.hpp:111-118:
// v -= 2p if v >= 2p; v -= p if v >= p.
__device__ __forceinline__ uint64_t fwd_correct(uint64_t v, uint64_t p, uint64_t p2) {
  return csub(csub(v, p2), p);
}

// Barrett reduction of the 128-bit value (xh:xl), lib/ops.cpp:5-21:
// q = Pn*xh + (x << 2) (mod 2^128); r = xl - hi64(q)*p (mod 2^64);
// one conditional subtraction.
__device__ __forceinline__ uint64_t barrett128(uint64_t xh, uint64_t xl, uint64_t p, uint64_t pn) {
  const uint64_t pl = pn * xh;
  const uint64_t ph = __umul64hi(pn, xh);
  const uint64_t sl = xl << 2;
  const uint64_t sh = (xh << 2) | (xl >> 62);
  const uint64_t lo = pl + sl;
  const uint64_t qh = ph + sh + (lo < pl ? 1ull : 0ull);
  const uint64_t r = xl - qh * p;
  return (r >= p) ? r - p : r;
}

// ops::mulmod, include/yell/ops.hpp:103-112.
__device__ __forceinline__ uint64_t mulmod_barrett(uint64_t x, uint64_t y, uint64_t p, uint64_t pn) {
  return barrett128(__umul64hi(x, y), x * y, p, pn);
}

// Montgomery product x*y*2^-64 mod p, lazily in [0, 2p), for x, y < 2p:
// t = (x*y + m*p) / 2^64 with m = lo64(x*y) * (-p^-1) mod 2^64.  The low words
// of x*y and m*p sum to 0 or 2^64, so their carry is (lo64(x*y) != 0); and
// t < (4p^2 + 2^64 p) / 2^64 < 2p since 4p < 2^64.  Used for the fused
// polymul's product, where only the final fully reduced words are observable
// and the 2^-64 is cancelled by the inverse's scaling constant.
__device__ __forceinline__ uint64_t mont_mul(uint64_t x, uint64_t y, uint64_t p, uint64_t neg_pinv) {
  const uint64_t lo = x * y, hi = __umul64hi(x, y);
  const uint64_t m = lo * neg_pinv;
  return hi + __umul64hi(m, p) + (lo != 0 ? 1ull : 0ull);
}

// ops::muladd, include/yell/ops.hpp:144-158: barrett(x*y + rop).
__device__ __forceinline__ uint64_t muladd_barrett(uint64_t rop, uint64_t x, uint64_t y, uint64_t p,
                                                   uint64_t pn) {
  const uint64_t lo = x * y;
  const uint64_t s = lo + rop;
  const uint64_t hi = __umul64hi(x, y) + (s < lo ? 1ull : 0ull);
  return barrett128(hi, s, p, pn);
}

// ops::addmod / ops::submod, include/yell/ops.hpp:54-83 (mod_correct :46-52).
__device__ __forceinline__ uint64_t addmod(uint64_t x, uint64_t y, uint64_t p) {
  x += y;
  return (x >= p) ? x - p : x;
}

__device__ __forceinline__ uint64_t submod(uint64_t x, uint64_t y, uint64_t p) {
  x += (p - y);
  return (x >= p) ? x - p : x;
}

// ---------------------------------------------------------------------------
// 32-bit moduli mode (include/yell/params_32.hpp: 30-bit primes, uint32
// words, uint64 products).  The reference runs the same generic code with
// bit_width = 32; the functions below are those formulas at 32-bit words.
// ---------------------------------------------------------------------------

// Per-(log_n, cm) constants of a 32-bit modulus; fwd/inv point at N {w, w'}
// pairs, bit-reversed, w' = floor(w * 2^32 / p).
struct alignas(16) DevMod32 {
  const uint2* fwd;
  const uint2* inv;
  uint32_t p;
  uint32_t pn;  // low word of floor(2^64/p) (params_32.hpp Pn)
  uint32_t inv_n, inv_n_s;
  uint32_t inv_n_iphi, inv_n_iphi_s;
};

// u >= m ? u - m : u for 0 < m: u - m wraps above u exactly when u < m.
__device__ __forceinline__ uint32_t csub(uint32_t u, uint32_t m) { return min(u, u - m); }

// x*w - hi32(x*w')*p (mod 2^32), in [0, 2p); np = 2^32 - p.
__device__ __forceinline__ uint32_t shoup_lazy(uint32_t x, uint32_t w, uint32_t wp, uint32_t np) {
  return x * w + __umulhi(x, wp) * np;
}

__device__ __forceinline__ void ct_bfly(uint32_t& x0, uint32_t& x1, uint32_t w, uint32_t wp, uint32_t np,
                                        uint32_t p2) {
  const uint32_t u0 = csub(x0, p2);
  const uint32_t t = shoup_lazy(x1, w, wp, np);
  x0 = u0 + t;
  x1 = u0 - t + p2;
}

__device__ __forceinline__ void gs_bfly(uint32_t& x0, uint32_t& x1, uint32_t w, uint32_t wp, uint32_t np,
                                        uint32_t p2) {
  const uint32_t u0 = x0, u1 = x1;
  const uint32_t t1 = u0 - u1 + p2;
  x0 = csub(u0 + u1, p2);
  x1 = shoup_lazy(t1, w, wp, np);
}

__device__ __forceinline__ uint32_t mulmod_shoup(uint32_t x, uint32_t y, uint32_t yp, uint32_t p) {
  return csub(shoup_lazy(x, y, yp, 0u - p), p);
}

__device__ __forceinline__ void gs_last(uint32_t& x0, uint32_t& x1, const DevMod32& m) {
  const uint32_t u = x0, v = x1;
  x0 = mulmod_shoup(u + v, m.inv_n, m.inv_n_s, m.p);
  x1 = mulmod_shoup(u - v + (m.p << 1), m.inv_n_iphi, m.inv_n_iphi_s, m.p);
}

__device__ __forceinline__ uint32_t fwd_correct(uint32_t v, uint32_t p, uint32_t p2) {
  return csub(csub(v, p2), p);
}

// lib/ops.cpp:5-21 at shift 32, delta 2: q = Pn*(x >> 32) + (x << 2)
// (mod 2^64); r = lo32(x) - hi32(q)*p (mod 2^32); one correction.
__device__ __forceinline__ uint32_t barrett64(uint64_t x, uint32_t p, uint32_t pn) {
  const uint64_t q = (uint64_t)pn * (x >> 32) + (x << 2);
  return csub((uint32_t)x - (uint32_t)(q >> 32) * p, p);
}

__device__ __forceinline__ uint32_t mulmod_barrett(uint32_t x, uint32_t y, uint32_t p, uint32_t pn) {
  return barrett64((uint64_t)x * y, p, pn);
}

// Montgomery product x*y*2^-32 mod p, lazily in [0, 2p), for x, y < 2p and
// 4p < 2^32: (x*y + m*p) / 2^32 with m = lo32(x*y) * (-p^-1) mod 2^32, the sum
// exact in 64 bits (below 2^63).  The fused polymul's product; its 2^-32 is
// cancelled by the inverse's scaling constants.
__device__ __forceinline__ uint32_t mont_mul(uint32_t x, uint32_t y, uint32_t p, uint32_t neg_pinv) {
  const uint64_t t = (uint64_t)x * y;
  const uint32_t m = (uint32_t)t * neg_pinv;
  return (uint32_t)((t + (uint64_t)m * p) >> 32);
}

__device__ __forceinline__ uint32_t muladd_barrett(uint32_t rop, uint32_t x, uint32_t y, uint32_t p,
                                                   uint32_t pn) {
  return barrett64((uint64_t)x * y + rop, p, pn);
}

__device__ __forceinline__ uint32_t addmod(uint32_t x, uint32_t y, uint32_t p) { return csub(x + y, p); }
__device__ __forceinline__ uint32_t submod(uint32_t x, uint32_t y, uint32_t p) { return csub(x + (p - y), p); }

// Twiddle pair type of a word type.
template <class W> struct PairOf;
template <> struct PairOf<uint64_t> {
  using type = ulonglong2;
  __device__ static __forceinline__ type make(uint64_t a, uint64_t b) { return make_ulonglong2(a, b); }
};
template <> struct PairOf<uint32_t> {
  using type = uint2;
  __device__ static __forceinline__ type make(uint32_t a, uint32_t b) { return make_uint2(a, b); }
};

// ---------------------------------------------------------------------------
// Programmatic dependent launch.  Kernels launched with programmatic stream
// serialization (launch_dependent, kernels.h) may have their CTAs resident
// while the stream's previous kernel still runs its last CTAs;
// grid_dep_wait() returns once that kernel has completed with its writes
// visible (at once for a kernel launched without the attribute, or when the
// stream's previous work is not a kernel), and every such kernel calls it
// before it reads or writes global memory other than the library's own
// tables.  grid_dep_launch() at the start of a CTA lets the stream's next
// kernel begin launching once every CTA of this one has started.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void grid_dep_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void grid_dep_launch() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

}  // namespace yell_gb300
