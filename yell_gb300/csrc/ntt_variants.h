// Launch variants of the NTT / fused polymul per degree (internal).
//
// Each degree has one or more variants that apply exactly the same
// butterflies (so produce the same words) with a different split of the work:
// the tile size of the whole-limb path (limbs per CTA) or the number of
// column stages k1 of the two-pass path (columns of 2^k1 words, rows of
// 2^(log_n - k1) words).  Variant 0 is the default; the autotuner times every
// variant of a degree on the current device and keeps the fastest.
#pragma once
#include <vector>

#include "kernels.h"

namespace yell_gb300 {

struct Variant {
  char name[96] = {};
  cudaError_t (*ntt)(const LimbSet&, const DevMod*, NttDir, cudaStream_t) = nullptr;
  cudaError_t (*polymul)(const LimbSet&, const ConstLimbSet&, const ConstLimbSet&, const DevMod*,
                         uint64_t* scratch, uint64_t* const* scratch_ptrs, cudaStream_t) = nullptr;
  cudaError_t (*set_attrs)() = nullptr;
  uint32_t ntt_launches = 0;
  uint32_t polymul_launches = 0;
  bool polymul_scratch = false;  // the polymul needs one operand's worth of scratch words
};

// Registration, one per translation unit (by_degree has kMaxLogN + 1 entries).
void add_whole_variants_small(std::vector<Variant>* by_degree);  // 2^3 .. 2^8
void add_whole_variants_large(std::vector<Variant>* by_degree);  // 2^9 .. 2^13 (and two-pass 2^13)
void add_two_pass_variants_a(std::vector<Variant>* by_degree);   // 2^14, 2^15
void add_two_pass_variants_b(std::vector<Variant>* by_degree);   // 2^16, 2^17
void add_two_pass_variants_c(std::vector<Variant>* by_degree);   // 2^18 .. 2^20
void add_two_pass_variants_d(std::vector<Variant>* by_degree);   // more 2^16 splits and round widths
void add_two_pass_variants_e(std::vector<Variant>* by_degree);   // pipelined polymul, 2^16

// Variant table of a degree, and the variant selected on the current device.
const std::vector<Variant>& variants_of(uint32_t log_n);
uint32_t selected_variant(int device, uint32_t log_n);
void select_variant(int device, uint32_t log_n, uint32_t v);

}  // namespace yell_gb300
