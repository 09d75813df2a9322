// Two-pass variants, degrees 2^18 .. 2^20 (the reference's kMaxPolyDegree,
// include/yell/params_64.hpp:21).  Rows stay within one 4096-word tile
// (log N - k1 <= 12), columns of 2^8 or 2^9 words as at 2^16 and 2^17.
#include "ntt_kernels.cuh"

namespace yell_gb300 {

void add_two_pass_variants_c(std::vector<Variant>* by) {
  by[18].push_back(two_pass_variant<18, 8>());
  by[18].push_back(two_pass_variant<18, 9>());
  by[19].push_back(two_pass_variant<19, 8>());
  by[19].push_back(two_pass_variant<19, 9>());
  by[20].push_back(two_pass_variant<20, 8>());
  by[20].push_back(two_pass_variant<20, 9>());
}

}  // namespace yell_gb300
