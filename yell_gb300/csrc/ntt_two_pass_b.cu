// Two-pass variants, degrees 2^16 and 2^17 (k1 = column stages).
#include "ntt_kernels.cuh"

namespace yell_gb300 {

void add_two_pass_variants_b(std::vector<Variant>* by) {
  by[16].push_back(two_pass_variant<16, 7>());
  by[16].push_back(two_pass_variant<16, 8>());
  by[16].push_back(two_pass_variant<16, 9>());
  by[17].push_back(two_pass_variant<17, 8>());
  by[17].push_back(two_pass_variant<17, 9>());
}

}  // namespace yell_gb300
