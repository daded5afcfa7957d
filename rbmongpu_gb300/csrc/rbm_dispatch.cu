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

// Wq [N][KP][32], bq [KP][32] (KP = ceil(K / 2)): entry (row, kk, lane) holds units
// j0 = lane + 32 (2 kk) and j1 = j0 + 32; row N is the bias
__global__ void rbm_pairs_kernel(int N, int Mpad, int KP, const float2* W, const float2* b, float4* Wq, float4* bq) {
    const long idx = static_cast<long>(blockIdx.x) * blockDim.x + threadIdx.x;
    const long per_row = static_cast<long>(KP) * 32;
    if (idx >= (N + 1) * per_row) return;
    const int row = static_cast<int>(idx / per_row);
    const int rem = static_cast<int>(idx - row * per_row);
    const int kk = rem / 32, lane = rem % 32;
    const int j0 = lane + 32 * (2 * kk), j1 = j0 + 32;
    const float2* src = row < N ? W + static_cast<long>(row) * Mpad : b;
    const float2 a = j0 < Mpad ? src[j0] : make_float2(0.0f, 0.0f);
    const float2 c = j1 < Mpad ? src[j1] : make_float2(0.0f, 0.0f);
    (row < N ? Wq[idx] : bq[rem]) = make_float4(a.x, c.x, a.y, c.y);
}

// Wt4 [Mpad / 2][N]: entry (p, i) = (x_j, x_j+4, y_j, y_j+4) of W[i], j = 8 (p / 4) + p % 4
__global__ void rbm_transpose_kernel(int N, int Mpad, const float2* W, float4* Wt4) {
    const long idx = static_cast<long>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (idx >= static_cast<long>(N) * (Mpad / 2)) return;
    const int p = static_cast<int>(idx / N), i = static_cast<int>(idx - static_cast<long>(p) * N);
    const int j = 8 * (p / 4) + p % 4;
    const float2 a = W[static_cast<long>(i) * Mpad + j], c = W[static_cast<long>(i) * Mpad + j + 4];
    Wt4[idx] = make_float4(a.x, c.x, a.y, c.y);
}

cudaError_t launch_rbm_pairs(int N, int Mpad, const float2* W, const float2* b, float4* Wq, float4* bq,
                             float4* Wt, cudaStream_t st) {
    const int KP = (Mpad / 32 + 1) / 2;
    const long n = static_cast<long>(N + 1) * KP * 32;
    rbm_pairs_kernel<<<static_cast<int>((n + 255) / 256), 256, 0, st>>>(N, Mpad, KP, W, b, Wq, bq);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess || !Wt) return e;
    const long m = static_cast<long>(N) * (Mpad / 2);
    rbm_transpose_kernel<<<static_cast<int>((m + 255) / 256), 256, 0, st>>>(N, Mpad, W, Wt);
    return cudaGetLastError();
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
