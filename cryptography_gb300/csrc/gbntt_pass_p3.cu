// gbntt_pass_p3.cu — pass kernels of the 32-bit prime p3 (see gbntt_pass.cuh).
#include "gbntt_pass.cuh"

namespace gbntt {
template cudaError_t launch_pass_prime<3>(int log_l, int dir, int ld, const PassArgs &a, cudaStream_t st);
template cudaError_t launch_inner_fused_prime<3>(int log_l, const PassArgs &a, cudaStream_t st);
template cudaError_t launch_build_pass_twiddles<3>(uint64_t *table, const uint64_t *hi, const uint64_t *lo, int log_m,
                                                 int log_s, int use_scale, uint64_t scale, cudaStream_t st);
}  // namespace gbntt
