/*
 * CPU restatement ("oracle") of RBMonGPU's variational hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product library links or calls this
 * code: the tests, the smoke check and the benchmark's CPU-baseline leg use it
 * as the checker of the CUDA kernels in rbmongpu_gb300/csrc.
 *
 * Two arithmetic modes:
 *   OR_PREC_REF64  follows the reference's own host path (FP64, sequential sums,
 *                  Metropolis revert-on-reject), so that with OR_RNG_MT19937 it
 *                  reproduces the reference's spins and accept counts exactly.
 *   OR_PREC_GPU32  follows the documented FP32 operation order of the CUDA
 *                  sampler (explicit fmaf, fixed warp-butterfly reduction,
 *                  per-sweep angle refresh), so that with OR_RNG_PHILOX it
 *                  reproduces the GPU chains bit for bit.
 *
 * Complex numbers are passed as interleaved (re, im) doubles.
 * Spin configurations are bitsets of ceil(N/64) uint64 words; bit i set <=> s_i = +1
 * (reference include/Spins.h:125-129).
 */
#ifndef RBMG_ORACLE_H
#define RBMG_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define OR_MAX_WORDS 4          /* N <= 256 */
#define OR_MAX_LAYERS 3

enum { OR_RNG_MT19937 = 0, OR_RNG_PHILOX = 1 };
enum { OR_PREC_REF64 = 0, OR_PREC_GPU32 = 1 };
enum { OR_PSI_RBM = 0, OR_PSI_DEEP = 1, OR_PSI_PAIR = 2 };

typedef struct {
    int S, L;                 /* strings x table width */
    const double* coef;       /* [2*S] */
    const int* types;         /* [S*L] 0=I 1=X 2=Y 3=Z */
    const int* idx;           /* [S*L] site, -1 terminates a row */
} or_op;

typedef struct {
    int kind;
    int N;
    double prefactor;
    /* RBM: b[2M], W[2*N*M] row-major W[i*M+j] */
    int M;
    const double* b;
    const double* W;
    /* PsiDeep (complex, kind 1) or PsiPair (kind 2: real part nets in *_re, imag in *_im) */
    int num_layers;
    int size[OR_MAX_LAYERS];
    int conn[OR_MAX_LAYERS];
    const unsigned* lhs_conn[OR_MAX_LAYERS];   /* [conn*size], entry i*size+j */
    const double* lhs_w[OR_MAX_LAYERS];        /* kind 1: complex [2*conn*size]; kind 2: real parts */
    const double* bias[OR_MAX_LAYERS];         /* kind 1: complex [2*size];      kind 2: real parts */
    const double* final_w;                     /* kind 1: complex [2*last];      kind 2: real parts */
    const double* lhs_w_im[OR_MAX_LAYERS];     /* kind 2 only */
    const double* bias_im[OR_MAX_LAYERS];
    const double* final_w_im;
    int translational_invariance;
    /* free quantum axis (PsiBase.hpp:164): the Hilbert-space distance of a psi with it set
     * adds the alpha / beta rotation terms (HilbertSpaceDistance.cu:47-81); alpha, beta [N]
     * real, NULL = zeros */
    int free_quantum_axis;
    const double* alpha;
    const double* beta;
} or_psi;

/* ---- random streams ---- */
void or_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);
uint32_t or_philox_word(uint64_t seed, uint32_t walker, uint64_t index);
void or_mt_words(uint32_t seed, int count, uint32_t* out);

/* ---- activation ---- */
void or_logcosh(double re, double im, double* out);   /* out[2] */
void or_tanh(double re, double im, double* out);
float or_lc_re_f32(float x, float y);
void or_div_pos_f32_n(const float* num, const float* den, float* out, long n);
void or_lc_f32(float x, float y, float* out);
void or_tanh_f32(float x, float y, float* out);
float or_expf_det(float x);
float or_logf_det(float x);

/* ---- wave functions ---- */
int or_num_params(const or_psi* psi);
void or_log_psi(const or_psi* psi, const uint64_t* spins, double* out);
void or_O_k(const or_psi* psi, const uint64_t* spins, double* out /* [2*P] */);
/* PsiPair: O_k of the real (part=0) or imaginary (part=1) net, real valued [P] */
void or_O_k_pair(const or_psi* psi, int part, const uint64_t* spins, double* out);
void or_rbm_angles(const or_psi* psi, const uint64_t* spins, double* theta /* [2M] */);

/* ---- operator ---- */
void or_local_energy(const or_psi* psi, const or_op* op, const uint64_t* spins, const double* log_psi, double* out);
/* E_k(s) = sum_n E_{s s'_n} O_k(s'_n), accumulated with weight into acc [2*P] */
void or_E_k_accumulate(const or_psi* psi, const or_op* op, const uint64_t* spins, const double* log_psi,
                       double weight, double* acc);

/* ---- exact summation (reference weights: prefactor^2 |psi|^2, i.e. the value the
 *      reference returns after dividing by num_steps) ---- */
double or_exact_norm(const or_psi* psi);
void or_psi_vector(const or_psi* psi, double* out /* [2 * 2^N] */);
void or_exact_value(const or_psi* psi, const or_op* op, double* E);
void or_exact_fluctuation(const or_psi* psi, const or_op* op, double* E, double* sigma);
void or_exact_gradient(const or_psi* psi, const or_op* op, double* grad /* [2P] */, double* E);
double or_exact_hsd(const or_psi* psi, const or_psi* psi_prime, const or_op* op, int is_unitary,
                    double nu, double* grad /* [2P'] or NULL */);

/* ---- Metropolis Monte Carlo (reference MonteCarloLoop) ----
 * Runs chains [chain_begin, chain_begin+num_chains) of a MonteCarloLoop with
 * total_chains chains.  Each chain: random start, num_therm*N proposals,
 * then samples_per_chain x (num_sweeps*N proposals, measurement).
 * spins_out [samples][num_chains][nwords]; log_psi_out, eloc_out [samples][num_chains][2];
 * any output may be NULL.  eloc is only computed when op != NULL. */
typedef struct {
    int total_chains;
    int chain_begin;
    int num_chains;
    int samples_per_chain;
    int num_sweeps;
    int num_therm;
    int rng;            /* OR_RNG_* ; MT19937 is seeded with the chain index */
    uint64_t seed;      /* Philox key */
    int prec;           /* OR_PREC_* */
    int fast_sweep_tries;   /* 0 = single-spin sweeps */
    int total_z;            /* 1 = S_z-conserving pair updates */
    int sector;
    /* optional persistent state of the chains (Philox streams only): when state_spins is
     * set and resume != 0 the chains continue from these configurations and stream
     * positions instead of drawing fresh starts; both are updated on return */
    uint64_t* state_spins;   /* [num_chains][nwords] */
    uint64_t* state_rng;     /* [num_chains] next Philox word */
    int resume;
} or_mc_cfg;

int or_mc_run(const or_psi* psi, const or_op* op, const or_mc_cfg* cfg,
              uint64_t* spins_out, double* log_psi_out, double* eloc_out,
              uint64_t* accepts, uint64_t* rejects);

/* Estimators over externally supplied samples (equal weights), FP64.
 * grad_out: reference gradient formula with the E_k term (ExpectationValue.cu:177-256). */
void or_samples_gradient(const or_psi* psi, const or_op* op, int num_samples, const uint64_t* spins,
                         double* grad, double* E);
double or_samples_hsd(const or_psi* psi, const or_psi* psi_prime, const or_op* op, int is_unitary,
                      int num_samples, const uint64_t* spins, double nu, double* grad);

#ifdef __cplusplus
}
#endif
/* learned-proposal chain: FP32 replay of the frozen Metropolis-Hastings steps of
 * rbmongpu_gb300/csrc/proposal.cu fed the device's logits (see oracle.c) */
int or_learned_replay(int N, int M, int Mpad, const float* Wr, const float* Wi, int B, int steps, uint64_t seed,
                      uint32_t walker_base, const uint64_t* spins0, const uint64_t* rng0, const float* theta0,
                      const float* re0, const float* logits0, const float* logits_prop, int* site, int* len,
                      float* logq, uint64_t* spins_out, uint8_t* accepted, uint64_t* rng_end);

#endif
