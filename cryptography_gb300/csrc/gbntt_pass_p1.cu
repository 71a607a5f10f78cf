// gbntt_pass_p1.cu — pass kernels of prime index 1 (see gbntt_pass.cuh).
#include "gbntt_pass.cuh"

namespace gbntt {
template cudaError_t launch_pass_prime<1>(int log_l, int dir, int ld, const PassArgs &a, cudaStream_t st);
template cudaError_t launch_inner_fused_prime<1>(int log_l, const PassArgs &a, cudaStream_t st);
template cudaError_t launch_build_pass_twiddles<1>(uint64_t *table, const uint64_t *hi, const uint64_t *lo, int log_m,
                                                 int log_s, int use_scale, uint64_t scale, cudaStream_t st);
}  // namespace gbntt
