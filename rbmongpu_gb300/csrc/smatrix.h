// S-matrix kernels (smatrix.cu), driven from capi.cu::rbmg_s_matrix.
#pragma once

#include <cstddef>
#include <cstdint>

#include <cuda_runtime.h>

namespace rbmg {

// one chunk of samples whose O_k rows (k >= 2N, L of them) enter the S matrix
struct SmSource {
    int kind;                // 0 complex RBM (rows formed from tanh(theta) and the spins), 1 FP64 rows
    int count, L;
    int N, M, Mpad, nw;      // RBM shape
    int enumerate;           // configurations are enum_base + s (exact summation without a sector)
    uint64_t enum_base;
    const uint64_t* spins;   // [count][nw] when not enumerated
    const float2* T;         // RBM: tanh(theta) [count][Mpad]
    const double2* rows;     // kind 1: O_k rows [count][ld]
    long ld;
    const double* w;         // per-sample weights (exact summation), used when weighted
    int weighted;
    const double2* shift;    // [L] subtracted from every row before the products, or null
};

// S [L][L] += sum_s c_s G_s^T conj(G_s) on the upper tiles, G_s = F_s - shift (c_s = w_s
// when weighted, else 1); mean [L] += sum_s c_s G_s when mean is not null
cudaError_t launch_sm_accumulate(const SmSource& src, double2* S, double2* mean, int num_sms, cudaStream_t st);
// mean [L] += sum_s c_s G_s alone
cudaError_t launch_sm_mean(const SmSource& src, double2* mean, cudaStream_t st);
// out [L] = sum_s F_s / count (unweighted, unshifted): the shift of a centred S matrix
cudaError_t launch_sm_row_mean(const SmSource& src, double2* out, cudaStream_t st);
// the same products on the tensor cores (smatrix_tc.cu): BF16 hi / mid / lo operand planes
// of the chunk in `planes` (sm_tc_planes_bytes(L, count) bytes), one operand pass and one
// persistent MMA launch on num_sms CTAs (counted into *launches); a tensor-core wait that
// gives up sets *error
size_t sm_tc_planes_bytes(int L, int count);
cudaError_t launch_sm_tc_accumulate(const SmSource& src, double2* S, void* planes, int* error, int* launches,
                                    int num_sms, cudaStream_t st);
// out [off + r][off + c] (ldo columns) = S / Z with the lower triangle mirrored; centred:
// minus (mean / Z)(mean / Z)^dagger
cudaError_t launch_sm_finish(int L, const double2* S, const double2* mean, double inv_z, int centered,
                             double2* out, long ldo, int off, cudaStream_t st);

}  // namespace rbmg
