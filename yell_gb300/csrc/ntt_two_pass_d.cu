// Two-pass variants of degree 2^16 with other splits or other round widths:
// k1 = 6 (rows of 2^10 words), and column or row tiles of 8 words per thread
// (512 threads per 4096-word tile, radix-8 rounds).
#include "ntt_kernels.cuh"

namespace yell_gb300 {

void add_two_pass_variants_d(std::vector<Variant>* by) {
  by[16].push_back(two_pass_variant<16, 6>());
  by[16].push_back(two_pass_variant<16, 7, 3, 4>());
  by[16].push_back(two_pass_variant<16, 7, 4, 3>());
  by[16].push_back(two_pass_variant<16, 7, 3, 3>());
  by[16].push_back(two_pass_variant<16, 8, 3, 4>());
  by[16].push_back(two_pass_variant<16, 6, 4, 3>());
}

}  // namespace yell_gb300
