// gbntt_pass_p4.cu — pass kernels of q0 in lazy normal form (see gbntt_pass.cuh).
#include "gbntt_pass.cuh"

namespace gbntt {
template cudaError_t launch_pass_prime<4>(int log_l, int dir, int ld, const PassArgs &a, cudaStream_t st);
}  // namespace gbntt
