// Chooses the instantiated hidden-units-per-lane count K for an RBM of M hidden units.
#include "kernels.h"

namespace rbmg {

template <int K>
cudaError_t rbm_mc_launch_k(const RbmDev&, const OpDev*, const McLaunch&, cudaStream_t);
template <int K>
cudaError_t rbm_est_launch_k(const RbmDev&, const OpDev*, const RbmDev*, const EstLaunch&, cudaStream_t);

static const int kInstantiated[] = {1, 2, 4, 8, 13, 18};

int rbm_lanes_k(int M) {
    const int need = (M + 31) / 32;
    for (int k : kInstantiated)
        if (k >= need) return k;
    return -1;
}

cudaError_t launch_rbm_mc(const RbmDev& P, const OpDev* op, const McLaunch& L, cudaStream_t st) {
    switch (P.Mpad / 32) {
        case 1: return rbm_mc_launch_k<1>(P, op, L, st);
        case 2: return rbm_mc_launch_k<2>(P, op, L, st);
        case 4: return rbm_mc_launch_k<4>(P, op, L, st);
        case 8: return rbm_mc_launch_k<8>(P, op, L, st);
        case 13: return rbm_mc_launch_k<13>(P, op, L, st);
        case 18: return rbm_mc_launch_k<18>(P, op, L, st);
        default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_rbm_estimate(const RbmDev& P, const OpDev* op, const RbmDev* PP, const EstLaunch& L,
                                cudaStream_t st) {
    if (PP && PP->Mpad != P.Mpad) return cudaErrorInvalidValue;
    switch (P.Mpad / 32) {
        case 1: return rbm_est_launch_k<1>(P, op, PP, L, st);
        case 2: return rbm_est_launch_k<2>(P, op, PP, L, st);
        case 4: return rbm_est_launch_k<4>(P, op, PP, L, st);
        case 8: return rbm_est_launch_k<8>(P, op, PP, L, st);
        case 13: return rbm_est_launch_k<13>(P, op, PP, L, st);
        case 18: return rbm_est_launch_k<18>(P, op, PP, L, st);
        default: return cudaErrorInvalidValue;
    }
}

}  // namespace rbmg
