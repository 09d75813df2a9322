// Whole-limb variants, degrees 2^3 .. 2^8.
#include "ntt_kernels.cuh"

namespace yell_gb300 {

void add_whole_variants_small(std::vector<Variant>* by) {
  by[3].push_back(whole_variant<3, 12>());
  by[4].push_back(whole_variant<4, 12>());
  by[4].push_back(whole_variant<4, 13>());
  by[5].push_back(whole_variant<5, 12>());
  by[5].push_back(whole_variant<5, 13>());
  by[6].push_back(whole_variant<6, 12>());
  by[6].push_back(whole_variant<6, 13>());
  by[7].push_back(whole_variant<7, 12>());
  by[7].push_back(whole_variant<7, 13>());
  by[8].push_back(whole_variant<8, 12>());
  by[8].push_back(whole_variant<8, 13>());
}

}  // namespace yell_gb300
