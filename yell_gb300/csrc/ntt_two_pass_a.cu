// Two-pass variants, degrees 2^14 and 2^15 (k1 = column stages).
#include "ntt_kernels.cuh"

namespace yell_gb300 {

void add_two_pass_variants_a(std::vector<Variant>* by) {
  by[14].push_back(two_pass_variant<14, 7>());
  by[14].push_back(two_pass_variant<14, 6>());
  by[14].push_back(two_pass_variant<14, 8>());
  by[15].push_back(two_pass_variant<15, 7>());
  by[15].push_back(two_pass_variant<15, 6>());
  by[15].push_back(two_pass_variant<15, 8>());
}

}  // namespace yell_gb300
