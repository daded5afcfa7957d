// Launchers of the deterministic per-sample reductions (reduce_kernels.cu).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace rbmg {

constexpr int kMaxSeries = 6;
constexpr int kSumBlocks = 512;

struct SeriesSet {
    int n;
    const double2* v[kMaxSeries];
};

// out[r][j] += sum_s c[s] f(A[s][j]) g_r(s), g_0 = 1, g_{1+i} = s_i; f = conj if conj_a.
// partial: scratch of max_splits * (1+N) * M double2.
cudaError_t launch_outer_reduce(int count, int N, int nw, int M, const uint64_t* spins, uint64_t enum_base,
                                int enumerate, const double2* c, const float2* A, int lda, int conj_a, double2* out,
                                double2* partial, int max_splits, cudaStream_t st);
// out[1+i][j] += -2 sum_s w[s] s_i sum_{slots of site i} X[s][slot][j]; with cw the per-sample
// coefficient is the complex cw[s] (w ignored)
cudaError_t launch_vterm_reduce(int count, int N, int nw, int M, int Mpad, const uint64_t* spins, uint64_t enum_base,
                                int enumerate, const double* w, const float2* X, int num_offdiag,
                                const int* site_ptr, const int* site_slots, double2* out, double2* partial,
                                int max_splits, cudaStream_t st, const double2* cw = nullptr);
// sums[q] += sum_s w[s] v_q[s]; block_scratch: kSumBlocks * kMaxSeries double2
cudaError_t launch_weighted_sums(int count, const double* w, const SeriesSet& set, double2* block_scratch,
                                 double2* sums, cudaStream_t st);
cudaError_t launch_max_re2(int count, const double2* lp, double* block_max, int* blocks_out, cudaStream_t st);
cudaError_t launch_exp_weights(int count, const double2* lp, double shift, double* w, cudaStream_t st);
// c[s] = scale w[s] (v[s] - shift), or scale w[s] when v is null
cudaError_t launch_coef(int count, const double* w, const double2* v, double scale, double2* c, cudaStream_t st,
                        double2 shift = make_double2(0.0, 0.0));
cudaError_t launch_abs2(int count, const double2* v, double2* out, cudaStream_t st);
// c[s] = w[s] conj(v[s] - shift)
cudaError_t launch_coef_conj(int count, const double* w, const double2* v, double2 shift, double2* c,
                             cudaStream_t st);
// c[s] = (w[s] (Re v[s] - shift), 0)
cudaError_t launch_coef_real(int count, const double* w, const double2* v, double shift, double2* c,
                             cudaStream_t st);
// rw[s] = w[s] |psi(s) / psi'(s)|^2 from log psi and log psi', rwc[s] = (rw[s], 0)
cudaError_t launch_ratio_weights(int count, const double* w, const double2* lp, const double2* lpp, double* rw,
                                 double2* rwc, cudaStream_t st);
// a[s] = exp(2 Im E + Re(E E - E)), the weight of ExpectationValue::corrected
cudaError_t launch_corrected_terms(int count, const double2* e, double2* a, cudaStream_t st);
cudaError_t launch_hsd_terms(int count, const double2* eloc, const double2* lp, const double2* lpp, int is_unitary,
                             double2* omega, double2* pr, double2* nn, cudaStream_t st);

}  // namespace rbmg
