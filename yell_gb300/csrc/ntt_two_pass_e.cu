// The 2^16 split k1 = 7 with the pipelined polymul kernels (persistent CTAs
// that copy the next tile into shared memory while computing the current
// one).  Measured on GB300 at 32 limbs x 16 pairs: 1.277 ms per step against
// 1.101 ms for the one-tile-per-CTA kernels, every pass slower (the staged
// first round adds a shared-memory round trip, and two resident CTAs per SM
// already overlap one CTA's loads with the other's butterflies); kept as an
// autotuner candidate.
#include "ntt_kernels.cuh"

namespace yell_gb300 {

void add_two_pass_variants_e(std::vector<Variant>* by) { by[16].push_back(two_pass_pipe_variant<16, 7>()); }

}  // namespace yell_gb300
