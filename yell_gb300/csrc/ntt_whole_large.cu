// Whole-limb variants, degrees 2^9 .. 2^13, and the two-pass variants of
// 2^13 (tiles of 4096 words: two CTAs of 256 threads per SM where the
// whole-limb 2^13 tile fits one of 512; 9% faster at 512 limbs on GB300).
#include "ntt_kernels.cuh"

namespace yell_gb300 {

void add_whole_variants_large(std::vector<Variant>* by) {
  by[9].push_back(whole_variant<9, 12>());
  by[9].push_back(whole_variant<9, 13>());
  by[10].push_back(whole_variant<10, 12>());
  by[10].push_back(whole_variant<10, 13>());
  by[11].push_back(whole_variant<11, 12>());
  by[11].push_back(whole_variant<11, 13>());
  by[12].push_back(whole_variant<12, 12>());
  by[12].push_back(whole_variant<12, 13>());
  by[13].push_back(whole_variant<13, 13>());
  by[13].push_back(two_pass_variant<13, 6>());
  by[13].push_back(two_pass_variant<13, 7>());
}

}  // namespace yell_gb300
