// Host-visible descriptions of the device buffers and the kernel launchers.
// Everything here is plain data: the launchers are implemented in the .cu files
// and called by the C ABI layer (capi.cu).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace rbmg {

constexpr int kMaxWords = 4;   // N <= 256 spins
constexpr int kWarpsPerBlock = 4;

// complex RBM, FP32 on the device: W is [N][Mpad] row-major, zero padded to
// Mpad = 32 * K so that lane l owns hidden units j = l + 32 k.
struct RbmDev {
    int N, M, Mpad;
    const float2* W;
    const float2* b;
    // the same parameters with hidden units k and k + 1 of a lane side by side (lane l,
    // pair kk: units j = l + 32 (2 kk) and l + 32 (2 kk + 1)), as (x_j0, x_j1, y_j0, y_j1):
    // Wq [N][ceil(K / 2)][32], bq [ceil(K / 2)][32]; the unit beyond an odd K is zero
    const float4* Wq;
    const float4* bq;
    // W transposed with units j and j + 4 side by side (the local-energy kernel's pairs):
    // Wt4 [Mpad / 2][N], entry (p, i) = (x_j, x_j+4, y_j, y_j+4) of spin i's row,
    // j = 8 (p / 4) + p % 4
    const float4* Wt4;
};

// build Wq, bq from W [N][Mpad], b [Mpad] (K = Mpad / 32 hidden units per lane), and Wt4
cudaError_t launch_rbm_pairs(int N, int Mpad, const float2* W, const float2* b, float4* Wq, float4* bq,
                             float4* Wt4, cudaStream_t st);

// Pauli-string operator in compact form (built from the reference's padded
// table, include/operator/Operator.hpp:30-88).
struct OpDev {
    int S;                     // strings
    const double2* coef;       // [S]
    const int* ypow;           // [S] number of Y factors mod 4  -> (-i)^ypow
    const uint64_t* zmask;     // [S][kMaxWords] sites whose original spin multiplies the coefficient
    const int* nflip;          // [S] sites flipped an odd number of times
    const int* flip_off;       // [S] offset into flip_sites
    const int* flip_sites;     // flat
    const int* offdiag_slot;   // [S] index among off-diagonal strings, -1 if diagonal
    int num_offdiag;
    const float2* coef32;      // [S] coefficients rounded to FP32 (local-energy sums)
    const int* site1;          // [S] the flipped site of a single-flip string, -1 otherwise
    const int* next1;          // [S + 1] next1[n]: first single-flip string >= n (S if none)
    const int* offdiag;        // [num_offdiag] the off-diagonal strings in order
};

// Metropolis launch: one warp per walker (include/spin_ensembles/MonteCarloLoop.hpp:55-256)
struct McLaunch {
    int B;                      // walkers in this launch
    uint32_t walker_base;       // global index of walker 0 (Philox stream id)
    uint64_t seed;
    uint64_t* spins;            // [B][NW] chain state, in/out
    uint64_t* rng_index;        // [B] next Philox word, in/out
    int init;                   // 1: draw fresh random start spins
    int total_z, sector;        // S_z-conserving pair updates
    int fast_tries;             // > 0: fast sweep, multi-spin masks (the AND of fast_tries random words)
    int n_therm;                // sweeps before the first sample
    int n_samples;              // samples recorded by this launch
    int sweeps_per_sample;
    int sample_base;            // index of the first recorded sample within the output rows
    uint64_t* sample_spins;     // [rows][B][NW] or null
    unsigned long long* accepts;   // [B], accumulated
    unsigned long long* proposals; // [B], accumulated
};

// Per-sample estimator pass over a list of configurations (warp per sample).
enum : int {
    EST_ELOC = 1,       // local energy -> eloc[s]
    EST_LOGPSI = 2,     // log psi -> logpsi[s]
    EST_GRADVEC = 4,    // T[s][j] = tanh(theta_j), U[s][j] = sum_n e_n tanh(theta''_nj) + E_diag T, X[s][n][j]
    EST_PRIME = 8,      // log psi'(s) -> logpsi_prime[s] and T'[s][j] (HSD)
    EST_ENUMERATE = 16  // configuration s = sample index (exact summation), spins buffer ignored
};

struct EstLaunch {
    int count;                  // samples in this chunk
    uint64_t enum_base;         // first basis index when EST_ENUMERATE
    const uint64_t* spins;      // [count][NW]
    int flags;
    double2* eloc;              // [count]
    double2* logpsi;            // [count]
    float2* T;                  // [count][Mpad]
    float2* U;                  // [count][Mpad]
    float2* X;                  // [count][num_offdiag][Mpad]
    double2* logpsi_prime;      // [count]
    float2* Tp;                 // [count][Mpad'] tanh of psi' angles
    double2 e_shift;            // U is stored as U - e_shift * T (centred E_k sums)
};

// PsiDeep net on the device (include/quantum_state/PsiDeep.hpp:38-84): per layer the
// lhs connections / weights [conn][size], biases [size]; rhs lists (CSR over the
// units of layer l, entries c * size_{l+1} + j of layer l+1) for the reverse pass.
struct DeepNetDev {
    int N, L, P, width, units, real_net, ti;
    int size[3], conn[3], begin_params[3], begin_angle[3];
    const int* cidx[3];
    const float2* w[3];
    const float2* b[3];
    const double2* w64[3];
    const double2* b64[3];
    const int* rptr[3];
    const int* rq[3];
    const float2* fw;
    const double2* fw64;
    // layer 0's connections grouped by input spin: entries c * size[0] + unit of spin i in
    // sq[sptr[i] .. sptr[i + 1]) (the single-flip update of its pre-activations)
    const int* sptr;
    const int* sq;
};

// ---- launchers (return cudaError_t) ----
cudaError_t launch_rbm_mc(const RbmDev& psi, const OpDev* op, const McLaunch& L, cudaStream_t st);
cudaError_t launch_rbm_estimate(const RbmDev& psi, const OpDev* op, const RbmDev* psi_prime, const EstLaunch& L,
                                cudaStream_t st);

int rbm_lanes_k(int M);   // instantiated hidden units per lane for M, -1 if too large

}  // namespace rbmg
