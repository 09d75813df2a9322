// Whole-limb variants, degrees 2^9 .. 2^13.
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
}

}  // namespace yell_gb300
