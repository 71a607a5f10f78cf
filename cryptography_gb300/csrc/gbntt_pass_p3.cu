// gbntt_pass_p3.cu — pass kernels of the 32-bit prime p3 (see gbntt_pass.cuh).
#include "gbntt_pass.cuh"

namespace gbntt {
template cudaError_t launch_pass_prime<3>(int log_l, int dir, int ld, const PassArgs &a, cudaStream_t st);
}  // namespace gbntt
