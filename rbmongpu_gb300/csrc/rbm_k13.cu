// Complex-RBM kernels instantiated for K = 13 hidden units per lane (M <= 416).
#include "rbm_impl.cuh"

namespace rbmg {
template cudaError_t rbm_mc_launch_k<13>(const RbmDev&, const OpDev*, const McLaunch&, cudaStream_t);
template cudaError_t rbm_est_launch_k<13>(const RbmDev&, const OpDev*, const RbmDev*, const EstLaunch&, cudaStream_t);
}  // namespace rbmg
