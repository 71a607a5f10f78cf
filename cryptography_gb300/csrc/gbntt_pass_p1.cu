// gbntt_pass_p1.cu — pass kernels of prime index 1 (see gbntt_pass.cuh).
#include "gbntt_pass.cuh"

namespace gbntt {
template cudaError_t launch_pass_prime<1>(int log_l, int dir, int ld, const PassArgs &a, cudaStream_t st);
}  // namespace gbntt
