// Complex-RBM kernels instantiated for K = 2 hidden units per lane (M <= 64).
#include "rbm_impl.cuh"

namespace rbmg {
template cudaError_t rbm_mc_launch_k<2>(const RbmDev&, const OpDev*, const McLaunch&, cudaStream_t);
template cudaError_t rbm_est_launch_k<2>(const RbmDev&, const OpDev*, const RbmDev*, const EstLaunch&, cudaStream_t);
}  // namespace rbmg
