// FP64 per-sample pass of the Hilbert-space distance (rbm64.cu).
#pragma once

#include <algorithm>
#include <cstdint>
#include <cuda_runtime.h>

#include "kernels.h"

namespace rbmg {

struct Rbm64 {
    int N, M;
    const double2* W;   // [N][M]
    const double2* b;   // [M]
};

struct Hsd64Launch {
    int count;
    uint64_t enum_base;
    int enumerate;
    const uint64_t* spins;
    double2* eloc;      // [count] local energy of the operator under psi, or null
    double2* logpsi;    // [count] log psi, or null
    double2* dlogpsi;   // [count] log psi' - log psi
};

cudaError_t launch_rbm_hsd64(const Rbm64& P, const Rbm64& PP, const OpDev& op, const Hsd64Launch& L,
                             cudaStream_t st);
cudaError_t launch_hsd_terms64(int count, const double2* eloc, const double2* dl, int is_unitary, double2* omega,
                               double2* pr, double2* nn, cudaStream_t st);
cudaError_t launch_hsd2_terms64(int count, const double2* e1, const double2* e2, const double2* dl, double2* omega,
                                double2* pr, double2* nn, cudaStream_t st);
// mode 0: w B_s, mode 1: w Re B_s, mode 2: w Im(conj(<omega>) omega_s), each times scale
// (the host folds the final 1/v^2 / d^nu into scale so the FP32 reduction stays in range)
cudaError_t launch_hsd_coef(int count, const double* w, const double2* omega, const double2* pr,
                            double2 conj_omega_bar, double v, double u, double nn_bar, int mode, double scale,
                            double2* c, cudaStream_t st);

// free quantum axis of the Hilbert-space distance (source/network_functions/
// HilbertSpaceDistance.cu:47-81, 109-122).  qa [4][N]: da = alpha' - alpha, db = beta' - beta,
// cos(alpha' + alpha), sin(alpha' + alpha).
// out[t N + i] = configuration t with spin i flipped
cudaError_t launch_flip_each(int count, int N, const uint64_t* spins, uint64_t enum_base, int enumerate,
                             uint64_t* out, cudaStream_t st);
// per configuration: r_i = exp(lpf[t N + i] - lp[t]) into r [t][N] (if r), and
// dl[t] += sum_i (da_i s_i r_i + i db_i (r_i cos_i - s_i sin_i))
cudaError_t launch_fqa_terms(int count, int N, const uint64_t* spins, uint64_t enum_base, int enumerate,
                             const double2* lp, const double2* lpf, const double* qa, double2* dl, double2* r,
                             cudaStream_t st);
// out[k] = sum_t c_t conj(O_k(t)) for the 2N angles: O_alpha_i = s_i r_i,
// O_beta_i = i (r_i cos_i - s_i sin_i); fixed summation order
cudaError_t launch_fqa_grad(int count, int N, const uint64_t* spins, uint64_t enum_base, int enumerate,
                            const double2* c, const double2* r, const double* qa, double2* out, cudaStream_t st);

}  // namespace rbmg
