/*
 * rbmg — C ABI of the GB300 implementation of RBMonGPU's variational hot path.
 *
 * Plain C: opaque handles, host pointers and sizes, int status codes.  Complex
 * numbers are interleaved (re, im) doubles, exactly the memory layout of
 * numpy.complex128 / std::complex<double>.  Spin configurations are bitsets of
 * ceil(N/64) uint64 words, bit i set <=> s_i = +1 (reference include/Spins.h:125-129).
 *
 * Every call is synchronous: results are on the host when it returns, as in the
 * reference.  Handles are not thread-safe (the reference's objects are not either).
 *
 * Each declaration names the reference interface it replaces (paths relative to
 * the RBMonGPU source tree; the Python names are those of pyRBMonGPU/main.cpp).
 */
#ifndef RBMG_H
#define RBMG_H

#include <stdint.h>

#if defined(__GNUC__)
#define RBMG_API __attribute__((visibility("default")))
#else
#define RBMG_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* status codes: the reference throws std::runtime_error / calls exit
 * (include/types.h:40-48, 83-97); here every failure is returned. */
#define RBMG_OK 0
#define RBMG_EINVAL 1        /* bad argument or shape */
#define RBMG_ENOMEM 2        /* device allocation failed */
#define RBMG_ECUDA 3         /* CUDA runtime error (message in rbmg_last_error) */
#define RBMG_ETIMEOUT 4      /* a bounded device wait gave up */
#define RBMG_ENAN 5          /* non-finite parameters or results */
#define RBMG_EUNSUPPORTED 6  /* combination not provided (mirrors a missing reference instantiation) */

typedef struct rbmg_psi rbmg_psi;
typedef struct rbmg_operator rbmg_operator;
typedef struct rbmg_ensemble rbmg_ensemble;

/* last error message of the calling thread */
RBMG_API const char* rbmg_last_error(void);
/* library version string */
RBMG_API const char* rbmg_version(void);

/* setDevice (source/RBMonGPU.cu:7-9, pyRBMonGPU/main.cpp:611) */
RBMG_API int rbmg_set_device(int device);
/* start_profiling / stop_profiling (source/RBMonGPU.cu:11-17) */
RBMG_API int rbmg_profiler_start(void);
RBMG_API int rbmg_profiler_stop(void);

/* activation_function (pyRBMonGPU/main.cpp:607-609): the reference's rational
 * log-cosh, include/quantum_state/psi_functions.hpp:49-57, evaluated in FP64. */
RBMG_API int rbmg_activation(double re, double im, double* out /* [2] */);

/* ---------------------------------------------------------------- Psi (RBM)
 * Psi(alpha, beta, b, W, prefactor, free_quantum_axis, gpu)
 * (include/quantum_state/Psi.hpp:220-238, pyRBMonGPU/main.cpp:50-59).
 * alpha, beta: [N] real; b: [M] complex; W: [N, M] complex row-major.
 * Like the reference (include/quantum_state/PsiBase.hpp:168-178, 183-192) beta is
 * initialised from alpha.  free_quantum_axis != 0 makes the Hilbert-space distance of this
 * psi add the alpha / beta rotation terms (source/network_functions/HilbertSpaceDistance.cu:
 * 47-81, 109-122); the reference uses the flag nowhere else on this path. */
RBMG_API int rbmg_psi_create(int N, int M, const double* alpha, const double* beta, const double* b, const double* W,
                    double prefactor, int free_quantum_axis, rbmg_psi** out);

/* PsiDeep(alpha, beta, b_list, connections_list, W_list, final_weights, prefactor,
 * free_quantum_axis, gpu) (include/quantum_state/PsiDeep.hpp:339-400,
 * pyRBMonGPU/main.cpp:97-108) and, with pair != 0, PsiPair(...) with the same
 * arguments (include/quantum_state/PsiPair.hpp:166-205, main.cpp:138-149).
 * Layer l has sizes[l] units and conns[l] inputs per unit; connections[l] is
 * [conns[l], sizes[l]] uint32, biases[l] [sizes[l]] complex, weights[l]
 * [conns[l], sizes[l]] complex, final_weights [sizes[L-1]] complex. */
RBMG_API int rbmg_psi_deep_create(int N, int num_layers, const int* sizes, const int* conns,
                         const uint32_t* const* connections, const double* const* biases,
                         const double* const* weights, const double* final_weights, const double* alpha,
                         const double* beta, double prefactor, int free_quantum_axis, int pair, rbmg_psi** out);

/* Psi.copy() / PsiDeep.copy() (source/quantum_state/Psi.cu:17-29); all fields are
 * copied, including the O_k length the reference's copy drops. */
RBMG_API int rbmg_psi_copy(const rbmg_psi* psi, rbmg_psi** out);
RBMG_API int rbmg_psi_destroy(rbmg_psi* psi);

/* free_quantum_axis (pyRBMonGPU/main.cpp:91, 132, 166) */
RBMG_API int rbmg_psi_free_quantum_axis(const rbmg_psi* psi, int* on);
/* psi kind: 0 Psi, 1 PsiDeep, 2 PsiPair */
RBMG_API int rbmg_psi_kind(const rbmg_psi* psi, int* kind);
/* N, M (RBM) or width (deep), num_params (include/quantum_state/Psi.hpp:233, PsiDeep.cu:34-66) */
RBMG_API int rbmg_psi_shape(const rbmg_psi* psi, int* N, int* M, int* num_params);
/* params getter / setter, layout [alpha(N), beta(N), ...] (Psi.cu:71-92, PsiDeep.cu:120-177,
 * PsiPair.cu:34-76); values cross as complex128, the device holds complex64. */
RBMG_API int rbmg_psi_get_params(const rbmg_psi* psi, double* params /* [2 P] */);
RBMG_API int rbmg_psi_set_params(rbmg_psi* psi, const double* params /* [2 P] */);
RBMG_API int rbmg_psi_get_prefactor(const rbmg_psi* psi, double* prefactor);
RBMG_API int rbmg_psi_set_prefactor(rbmg_psi* psi, double prefactor);
/* PsiDeep.translational_invariance (pyRBMonGPU/main.cpp:111) */
RBMG_API int rbmg_psi_set_translational_invariance(rbmg_psi* psi, int on);

/* log psi(s) for a batch of configurations (Psi::log_psi_s_std, source/quantum_state/Psi.cu:57-58),
 * without the prefactor; out [2 count]. */
RBMG_API int rbmg_psi_log_psi(const rbmg_psi* psi, int count, const uint64_t* spins, double* out);

/* Psi.vector: psi over all 2^N basis states, index = bit pattern
 * (source/network_functions/PsiVector.cu:13-51); out [2 * 2^N]. */
RBMG_API int rbmg_psi_vector(const rbmg_psi* psi, double* out);

/* psi.norm(exact_summation) = sqrt(sum_s prefactor^2 |psi(s)|^2)
 * (source/network_functions/PsiNorm.cu:13-44), via an FP64 log-sum-exp. */
RBMG_API int rbmg_psi_norm(const rbmg_psi* psi, rbmg_ensemble* exact_summation, double* norm);

/* psi_O_k_vector(psi, spins) (source/network_functions/PsiOkVector.cu:9-44); entries [0, 2N) are 0. */
RBMG_API int rbmg_psi_O_k_vector(const rbmg_psi* psi, const uint64_t* spins, double* out /* [2 P] */);

/* ---------------------------------------------------------------- Operator
 * Operator(coefficients[S], pauli_types[S, L], pauli_indices[S, L], gpu)
 * (include/operator/Operator.hpp:212-227, pyRBMonGPU/main.cpp:240-245): types
 * 0 = I, 1 = X, 2 = Y, 3 = Z; an index of -1 ends a string. */
RBMG_API int rbmg_operator_create(int num_strings, int max_string_length, const double* coefficients, const int* pauli_types,
                         const int* pauli_indices, rbmg_operator** out);
RBMG_API int rbmg_operator_destroy(rbmg_operator* op);
/* num_strings, max_string_length, coefficients / pauli_types / pauli_indices getters (main.cpp:252-256) */
RBMG_API int rbmg_operator_shape(const rbmg_operator* op, int* num_strings, int* max_string_length);
RBMG_API int rbmg_operator_tables(const rbmg_operator* op, double* coefficients, int* pauli_types, int* pauli_indices);

/* ---------------------------------------------------------------- ensembles
 * MonteCarloLoop(num_samples, num_sweeps, num_thermalization_sweeps, num_markov_chains, gpu)
 * (source/spin_ensembles/MonteCarloLoop.cu:20-42, pyRBMonGPU/main.cpp:276-284).
 * Each chain is a Philox4x32-10 stream keyed by `seed`; num_samples must be a
 * multiple of num_markov_chains (MonteCarloLoop.cu:78). */
RBMG_API int rbmg_mc_create(uint32_t num_samples, uint32_t num_sweeps, uint32_t num_thermalization_sweeps,
                   uint32_t num_markov_chains, uint64_t seed, rbmg_ensemble** out);
/* MonteCarloLoop(MonteCarloLoop&) (MonteCarloLoop.cu:44-66): same settings, fresh streams */
RBMG_API int rbmg_mc_copy(const rbmg_ensemble* other, rbmg_ensemble** out);
/* set_total_z_symmetry / set_fast_sweep (include/spin_ensembles/MonteCarloLoop.hpp:283-291).
 * Fast sweep: each update flips the AND of num_tries random configurations (num_tries 0
 * draws one, like the reference's loop; above 64 is RBMG_EINVAL); a thermalisation sweep is
 * N updates, a sampling sweep one (MonteCarloLoop.hpp:108-113, 139-151, 162-171).  Both
 * networks accept on the change of Re log psi with the flipped sites' angles (the
 * reference's Psi keeps its angles for these moves and accepts every one); with
 * total_z symmetry a sampling call returns RBMG_EUNSUPPORTED. */
RBMG_API int rbmg_mc_set_total_z_symmetry(rbmg_ensemble* mc, int sector);
RBMG_API int rbmg_mc_set_fast_sweep(rbmg_ensemble* mc, uint32_t num_tries);
/* acceptance counters of the last sampling call (MonteCarloLoop.hpp:215-219), summed
 * over chains; per_chain_accepts may be NULL or [num_markov_chains]. */
RBMG_API int rbmg_mc_acceptance(const rbmg_ensemble* mc, uint64_t* accepts, uint64_t* proposals, uint64_t* per_chain_accepts);

/* ExactSummation(N, gpu) (source/spin_ensembles/ExactSummation.cu:16-24, main.cpp:288-291) */
RBMG_API int rbmg_exact_create(uint32_t num_spins, rbmg_ensemble** out);
/* ExactSummation.set_total_z_symmetry (ExactSummation.cu:26-45) */
RBMG_API int rbmg_exact_set_total_z_symmetry(rbmg_ensemble* exact, int sector);

/* num_steps (main.cpp:281, 291) */
RBMG_API int rbmg_ensemble_num_steps(const rbmg_ensemble* ens, uint64_t* num_steps);
RBMG_API int rbmg_ensemble_destroy(rbmg_ensemble* ens);
/* Extension (no reference counterpart; the reference's ensembles always sample or enumerate):
 * a fixed set of `count` configurations, spins [count][ceil(N/64)], each with weight 1 / count,
 * as a MonteCarloLoop pass that produced them (rbmg_ensemble_samples).  Every estimator
 * accepts it, e.g. the gradient of an energy estimated earlier, on the same samples. */
RBMG_API int rbmg_samples_create(uint32_t num_spins, uint32_t count, const uint64_t* spins, rbmg_ensemble** out);

/* Runs the ensemble's foreach (MonteCarloLoop.hpp:294-339) and records, per sample
 * index (step * chains + chain), the configuration, log psi and local energy.
 * spins [num_steps * nwords], log_psi / eloc [2 * num_steps]; any may be NULL;
 * eloc needs op.  (Extension: the reference exposes this only to C++ lambdas.) */
RBMG_API int rbmg_ensemble_samples(rbmg_ensemble* ens, const rbmg_psi* psi, const rbmg_operator* op, uint64_t* spins,
                          double* log_psi, double* eloc);

/* ---------------------------------------------------------------- ExpectationValue
 * (source/network_functions/ExpectationValue.cu, pyRBMonGPU/main.cpp:295-339) */
/* __call__(psi, operator, ensemble) -> <O>                        (:17-73)  */
RBMG_API int rbmg_ev_value(const rbmg_psi* psi, const rbmg_operator* op, rbmg_ensemble* ens, double* value /* [2] */);
/* __call__(psi, [operators], ensemble) -> [<O_i>]                 (:448-518)
 * one pass over the ensemble: every operator on the same configurations */
RBMG_API int rbmg_ev_values(const rbmg_psi* psi, const rbmg_operator* const* ops, int num_ops, rbmg_ensemble* ens,
                   double* values /* [2 num_ops] */);
/* fluctuation_gradient -> grad[P], the gradient of sigma = sqrt(<|E|^2> - |<E>|^2)   (:258-348)
 * grad_k = (2 conj(<E* E_k> - <E>* <E_k>) - 2 <E>* <E O_k*> + 2 <O_k>* (2|<E>|^2 - <|E|^2>)) / (2 sigma);
 * entries k < 2N are zero; sigma (may be NULL) receives sigma.  Psi and PsiDeep. */
RBMG_API int rbmg_ev_fluctuation_gradient(const rbmg_psi* psi, const rbmg_operator* op, rbmg_ensemble* ens,
                                          double* grad /* [2P] */, double* sigma);
/* difference(psi, psi_prime, [operators], ensemble) -> [<E'_i> - <r E_i> / <r>]   (:350-446)
 * over psi's ensemble, E' the local energy under psi_prime, r = |psi / psi_prime|^2; Psi only
 * (its instantiations), psi_prime with psi's N and padded M. */
RBMG_API int rbmg_ev_difference(const rbmg_psi* psi, const rbmg_psi* psi_prime, const rbmg_operator* const* ops,
                                int num_ops, rbmg_ensemble* ens, double* values /* [2 num_ops] */);
/* corrected(psi, operator, operator2, ensemble) -> (<E> / <a>, <a>), a = exp(2 Im E + Re(E E - E))
 * (:76-127); as in the reference the local energy is taken with the first operator twice and
 * operator2 is not used.  The reference binds it for PsiDeep; every network is accepted. */
RBMG_API int rbmg_ev_corrected(const rbmg_psi* psi, const rbmg_operator* op, const rbmg_operator* op2,
                               rbmg_ensemble* ens, double* value /* [2] */, double* abs2);
/* fluctuation -> (sigma, <O>)                                     (:130-175) */
RBMG_API int rbmg_ev_fluctuation(const rbmg_psi* psi, const rbmg_operator* op, rbmg_ensemble* ens, double* sigma,
                        double* value /* [2] */);
/* gradient -> (grad[P], <O>), grad_k = <E O_k*> + conj<E_k> - 2 <E> <O_k*>   (:177-256) */
RBMG_API int rbmg_ev_gradient(const rbmg_psi* psi, const rbmg_operator* op, rbmg_ensemble* ens, double* grad /* [2P] */,
                     double* value /* [2] */);

/* Extension (no reference counterpart): local energies of `count` given configurations
 * (spins [count][ceil(N/64)]) -> out [2 count]; the reference computes them only inside
 * its ensembles' foreach (include/operator/Operator.hpp:90-115). */
RBMG_API int rbmg_local_energies(const rbmg_psi* psi, const rbmg_operator* op, int count, const uint64_t* spins,
                                 double* out);
/* Extension: hidden angles theta = b + s W of `count` given configurations -> out
 * [2 count M] (complex), built on the tensor cores (spins exact in BF16, W as three BF16
 * parts, FP32 accumulation); the reference evaluates them one at a time
 * (kernel::Psi::angle, include/quantum_state/Psi.hpp:43-53).  Complex RBM. */
RBMG_API int rbmg_psi_angles(const rbmg_psi* psi, int count, const uint64_t* spins, double* out);
/* Extension: gradient of the local energy in PyTorch's convention for a real loss L:
 * grad_k = dL/dRe(theta_k) + i dL/dIm(theta_k).  score = 0: L = Re <E_loc> over the
 * ensemble's samples held fixed; score = 1: L = <H>, adding the sampling term.  PsiDeep: a
 * hand-written adjoint (reverse mode) kernel that recomputes every forward pass; score = 1
 * equals rbmg_ev_gradient except at the final weights (include/quantum_state/PsiDeep.hpp:285-292
 * scales their O_k by log psi; here d log psi / d w_final = activation).  Psi: formed from
 * the estimator sums, conj<E_k - E O_k> (+ 2 <(Re E - <Re E>) O_k*> for score = 1). */
RBMG_API int rbmg_ev_eloc_gradient(const rbmg_psi* psi, const rbmg_operator* op, rbmg_ensemble* ens, int score,
                                   double* grad /* [2P] */, double* value /* [2] */);

/* ---------------------------------------------------------------- HilbertSpaceDistance
 * (source/network_functions/HilbertSpaceDistance.cu:14-269, HilbertSpaceDistance_PsiPair.cu:99-169,
 * pyRBMonGPU/main.cpp:342-418).  The ensemble samples psi. */
RBMG_API int rbmg_hsd_distance(const rbmg_psi* psi, const rbmg_psi* psi_prime, const rbmg_operator* op, int is_unitary,
                      rbmg_ensemble* ens, double* distance);
/* distance_2nd_order (source/network_functions/HilbertSpaceDistance_2nd_order.cu:69-95,
 * pyRBMonGPU/main.cpp:352-363 builds op = Operator(expr) and op2 = Operator(expr * expr)):
 * the distance between exp(A) psi, expanded to second order, and psi_prime, with
 * omega_s = exp(E_A + (E_A2 - E_A^2) / 2 + conj(log psi' - log psi)). */
RBMG_API int rbmg_hsd_distance_2nd_order(const rbmg_psi* psi, const rbmg_psi* psi_prime, const rbmg_operator* op,
                                         const rbmg_operator* op2, rbmg_ensemble* ens, double* distance);
/* DiagDensityOp(sub_system_size, gpu)(psi, op, spin_ensemble) (pyRBMonGPU/main.cpp:497-533,
 * source/network_functions/DiagDensityOp.cu:12-50): out [2^sub_system_size] =
 * <|E_loc|^2 binned by the configuration of the first sub_system_size spins>, each bin's
 * weighted sum over num_steps.  Psi, PsiDeep and PsiPair, both ensembles (the reference
 * instantiates PsiDeep and PsiExact); sub_system_size <= min(N, 30). */
RBMG_API int rbmg_diag_density(const rbmg_psi* psi, const rbmg_operator* op, rbmg_ensemble* ens,
                               int sub_system_size, double* out);
/* KullbackLeibler(num_params, gpu) value / gradient (source/network_functions/
 * KullbackLeibler.cu:14-137, pyRBMonGPU/main.cpp:421-470) with D = log psi' - log psi:
 * value = sqrt(<|D|^2> - |<D>|^2), grad_k = (<D O_k*> - <D><O_k*>) / max(value, 1e-6)^nu
 * over psi's ensemble (O_k of psi_prime).  The reference instantiates it with PsiClassical
 * or PsiExact as psi, types outside this library; here psi and psi_prime are any of
 * Psi / PsiDeep / PsiPair (PsiPair psi_prime: value only).  grad [2P] nullable. */
RBMG_API int rbmg_kl_gradient(const rbmg_psi* psi, const rbmg_psi* psi_prime, rbmg_ensemble* ens, double nu,
                              double* grad, double* value);
RBMG_API int rbmg_hsd_gradient(const rbmg_psi* psi, const rbmg_psi* psi_prime, const rbmg_operator* op, int is_unitary,
                      rbmg_ensemble* ens, float nu, double* grad /* [2 P'] */, double* distance);

/* ---------------------------------------------------------------- persistent chains
 * Extension without a reference counterpart: the reference's foreach re-draws and
 * re-thermalises its chains on every call (include/spin_ensembles/MonteCarloLoop.hpp:79-105);
 * a chain handle keeps the walkers' configurations and Philox positions on the device
 * between calls, for long runs measured sweep by sweep (autocorrelation times).
 * The step is the reference's MonteCarloLoop step (MonteCarloLoop.hpp:153-256). */
typedef struct rbmg_chain rbmg_chain;
RBMG_API int rbmg_chain_create(const rbmg_psi* psi, uint32_t num_walkers, uint64_t seed, rbmg_chain** out);
RBMG_API int rbmg_chain_destroy(rbmg_chain* chain);
/* Runs n_sweeps sweeps (N proposals each) of every walker; after every
 * `measure_every`-th sweep the local energies of all walkers are written to
 * d_eloc_out, a DEVICE array of double2 [n_sweeps / measure_every][num_walkers]
 * (NULL: no measurement).  `stream` is a cudaStream_t (NULL: the library's stream);
 * the call returns without synchronising. */
RBMG_API int rbmg_chain_sweep_async(rbmg_chain* chain, const rbmg_psi* psi, const rbmg_operator* op, int n_sweeps,
                                    int measure_every, void* d_eloc_out, void* stream);
/* host copies of the walkers' configurations [num_walkers * nwords] and acceptance counters */
/* walker checkpoint (the reference checkpoints no chain state): spins [walkers][ceil(N/64)],
 * next Philox word, accept and proposal counters [walkers]; restoring continues bit for bit */
RBMG_API int rbmg_chain_get_checkpoint(const rbmg_chain* chain, uint64_t* spins, uint64_t* rng_index,
                                       uint64_t* accepts, uint64_t* proposals);
RBMG_API int rbmg_chain_set_checkpoint(rbmg_chain* chain, const uint64_t* spins, const uint64_t* rng_index,
                                       const uint64_t* accepts, const uint64_t* proposals);
RBMG_API int rbmg_chain_state(const rbmg_chain* chain, uint64_t* spins, uint64_t* accepts, uint64_t* proposals);
/* the library's CUDA stream of the calling thread, as a cudaStream_t */
RBMG_API int rbmg_stream(void** stream);

/* <op> under ExactSummation(num_spins) for a complex RBM, computed without allocating any
 * device memory.  It agrees with rbmg_ev_value on an ExactSummation ensemble to within
 * 1e-5 relative, not bit for bit: log psi is evaluated in FP64 from the device's FP32
 * (complex64) parameters, while rbmg_ev_value's exact path uses the FP64 parameters.
 * No counterpart in the reference: it is for callers that cannot call cudaMalloc, such as a
 * framework that owns all device memory through its own pool, or a latency-critical loop
 * that cannot afford the device-wide synchronisation of cudaFree.
 * The scratch is a fixed 1 MiB array in device global memory, held by every GPU that loads
 * the library until the process exits; it limits num_spins to 14 (larger sizes return
 * RBMG_EINVAL).  The first call on a device looks up the array's address with
 * cudaGetSymbolAddress (set-up done once per device, on the current device), so make that
 * first call before any stream capture.  Each call returns once the result is on the host.
 * Every call uses the same array and clears the sums it accumulates; calls that overlap on
 * the GPU (other host threads, other streams) race.  After a cudaDeviceReset the cached
 * address is stale: do not call it on a device that was reset. */
RBMG_API int rbmg_ev_value_exact_noalloc(const rbmg_psi* psi, const rbmg_operator* op, int num_spins,
                                         double* value /* [2] */);

/* ---------------------------------------------------------------- learned proposal
 * Extension (no reference counterpart): an MLP on the spins (BF16 operands, FP32
 * accumulation; N -> 256 -> 256 SiLU -> N seed + 8 length logits) proposes flipping the
 * contiguous cluster {i, ..., i+l-1}; the Metropolis-Hastings ratio includes the forward and
 * reverse proposal densities, so the chain's stationary law stays |psi|^2 (the step of
 * include/spin_ensembles/MonteCarloLoop.hpp:153-256 with a different proposal).  The net
 * is trained online with Adam, by default on the cross-entropy to the locally balanced
 * proposal over all cluster moves (rbmg_proposal_set_objective selects the objective). */
typedef struct rbmg_proposal rbmg_proposal;
RBMG_API int rbmg_proposal_create(int N, uint64_t seed, float lr, rbmg_proposal** out);
RBMG_API int rbmg_proposal_destroy(rbmg_proposal* proposal);
RBMG_API int rbmg_proposal_num_params(const rbmg_proposal* proposal, int64_t* num_params);
/* parameters, FP32, order W1 [N][256], b1, W2 [256][256], b2, W3 [256][N+8], b3 */
RBMG_API int rbmg_proposal_get_params(const rbmg_proposal* proposal, float* params);
RBMG_API int rbmg_proposal_set_params(rbmg_proposal* proposal, const float* params);
/* forward on `count` configurations -> logits [count][N+8]; with dlogits [count][N+8] also
 * the backward pass -> grads [num_params] (host buffers; a test hook of the kernels) */
RBMG_API int rbmg_proposal_eval(rbmg_proposal* proposal, int count, const uint64_t* spins, const float* dlogits,
                                float* logits, float* grads);
/* waits for the device and reports RBMG_ETIMEOUT (once) if a tensor-core pass of the
 * network gave up waiting for its MMAs since the last call */
RBMG_API int rbmg_proposal_status(rbmg_proposal* proposal);
/* one Adam step (lr of the proposal, beta 0.9 / 0.999, eps 1e-8) with the given gradient */
RBMG_API int rbmg_proposal_adam(rbmg_proposal* proposal, const float* grads);
/* training objective of rbmg_chain_learned_async: cross-entropy to the locally balanced
 * proposal p*(i, l) propto |psi(s')/psi(s)| over all N x 8 cluster moves of the training
 * walkers (default), or REINFORCE on the acceptance, reward min(1, a) * l */
#define RBMG_PROPOSAL_LOCALLY_BALANCED 0
#define RBMG_PROPOSAL_REINFORCE 1
RBMG_API int rbmg_proposal_set_objective(rbmg_proposal* proposal, int objective);
/* training state for checkpoints: FP32 parameters, Adam moments [num_params] each, Adam steps */
RBMG_API int rbmg_proposal_get_state(const rbmg_proposal* proposal, float* params, float* m, float* v, int64_t* steps);
RBMG_API int rbmg_proposal_set_state(rbmg_proposal* proposal, const float* params, const float* m, const float* v,
                                     int64_t steps);
/* n_steps learned Metropolis-Hastings steps of every walker of the chain.  train = 0 keeps
 * the weights (the chain is then exactly |psi|^2-stationary); train > 0 follows every step
 * with one update (objective of rbmg_proposal_set_objective) + Adam step on the first
 * `train` walkers (adaptive chain: use it to train, then measure with train = 0).  Local energies every
 * measure_every steps into d_eloc_out [n_steps / measure_every][walkers] (device double2),
 * as in rbmg_chain_sweep_async.  N must exceed 8. */
RBMG_API int rbmg_chain_learned_async(rbmg_chain* chain, const rbmg_psi* psi, const rbmg_operator* op,
                                      rbmg_proposal* proposal, int n_steps, int train, int measure_every,
                                      void* d_eloc_out, void* stream);
/* Measurement hook (no reference counterpart): n_steps frozen learned steps on one stream
 * with CUDA events around each tensor-core network pass and each accept pass; mean
 * durations in ms (the bench's per-kernel roofline of a learned step). */
RBMG_API int rbmg_chain_learned_kernel_times(rbmg_chain* chain, const rbmg_psi* psi, rbmg_proposal* proposal,
                                             int n_steps, double* ms_network, double* ms_accept);
/* Test hook (no reference counterpart): the locally balanced training target of `count`
 * configurations spins [count][nw] with the given logits [count][N+8]:
 * dl [count][N+8] = (q - p*) / count, p*(i, l) propto |psi(s')/psi(s)| over all N x 8 moves
 * (seed and length marginals), the gradient of the mean cross-entropy. */
RBMG_API int rbmg_proposal_lb_target(rbmg_proposal* proposal, const rbmg_psi* psi, int count, const uint64_t* spins,
                                     const float* logits, float* dl);
/* Test hook (no reference counterpart): n_steps frozen learned steps with the state copied
 * out around every launch, for a CPU replay of the draws and Metropolis-Hastings decisions.
 * Before the first step: spins0 [B][nw], rng0 [B] (next Philox word), the angles theta0
 * [B][Mpad][2] (re, im; Mpad = M rounded up to 32), their Re f re0 [B][Mpad] and the
 * current states' logits logits0 [B][N+8].  Per step t: the proposed states' logits
 * logits_prop [t][B][N+8], the move (site, len, logq = log q(s'|s)) [t][B], and after the
 * accept pass spins [t][B][nw] and the accept counters [t][B]; rng_end [B] at the end.
 * Networks with N + 8 <= 128. */
RBMG_API int rbmg_chain_learned_trace(rbmg_chain* chain, const rbmg_psi* psi, rbmg_proposal* proposal, int n_steps,
                                      uint64_t* spins0, uint64_t* rng0, float* theta0, float* re0, float* logits0,
                                      float* logits_prop, int* site, int* len, float* logq, uint64_t* spins,
                                      uint64_t* accepts, uint64_t* rng_end);
/* Extension: the frozen learned steps of a chain run its walkers as `streams` (1 to 4)
 * independent slices on as many streams (one slice's network pass overlapping another's
 * accept pass); 0 (default) picks 2 from 8192 walkers on.  Every walker
 * keeps its Philox stream, so the chains do not depend on the choice. */
RBMG_API int rbmg_chain_set_learned_streams(rbmg_chain* chain, int streams);


/* ---------------------------------------------------------------- batched serving
 * Extension (no reference counterpart; the reference runs one network per call,
 * include/spin_ensembles/MonteCarloLoop.hpp:294-339): many complex RBMs of uneven N and M,
 * each with its own operator, walkers and Philox seed, sampled, given local energies and
 * the O_k gradient 2 (<E O*> - <E> <O*>) in one persistent launch replayed from a CUDA
 * graph.  Walker w of instance i draws the Philox stream (seeds[i], w), as a Chain of
 * that instance would.  The instances' psi and operator handles must outlive the batch. */
typedef struct rbmg_batch rbmg_batch;
RBMG_API int rbmg_batch_create(int num_instances, const rbmg_psi* const* psis, const rbmg_operator* const* ops,
                               const uint32_t* walkers, const uint64_t* seeds, rbmg_batch** out);
RBMG_API int rbmg_batch_destroy(rbmg_batch* batch);
/* one replay: the first draws random start spins and runs `therm` + `sweeps` sweeps, later
 * ones continue the chains for `sweeps` sweeps; then every walker's local energy and the
 * per-instance O_k sums.  RBMG_ETIMEOUT if a reduction task gave up waiting. */
RBMG_API int rbmg_batch_run(rbmg_batch* batch, int therm, int sweeps);
/* launch shape: warps per block in {2, 4, 8}, reduction tile rows in {8, 16} */
RBMG_API int rbmg_batch_set_shape(rbmg_batch* batch, int warps_per_block, int rows);
RBMG_API int rbmg_batch_get_shape(const rbmg_batch* batch, int* warps_per_block, int* rows, int* blocks);
/* wall-clock limit of a reduction task's wait for its instance's walkers (default 20 s),
 * and walkers to wait for beyond each instance's (default 0): with extra_walkers > 0 the
 * wait runs out and the next replay returns RBMG_ETIMEOUT, leaving the device usable (the
 * test of the bounded wait). */
RBMG_API int rbmg_batch_set_wait(rbmg_batch* batch, double seconds, uint32_t extra_walkers);
/* register cap per thread of the persistent kernel: 255 (none), 128 or 96 (the largest
 * walker task sets the kernel's register count; a cap trades spills for resident warps) */
RBMG_API int rbmg_batch_set_register_cap(rbmg_batch* batch, int regs);
RBMG_API int rbmg_batch_get_register_cap(const rbmg_batch* batch, int* regs);
/* times the 18 shapes (register cap x warps per block x tile rows) on `reps` replays of
 * `sweeps` sweeps each and keeps the fastest; ms [18] (nullable) gets their mean replay
 * times, caps 255, 128, 96 in turn, each in the order (2,8) (2,16) (4,8) (4,16) (8,8) (8,16) */
RBMG_API int rbmg_batch_autotune(rbmg_batch* batch, int sweeps, int reps, double* ms);
/* last replay's results of instance i: energy [2], grad [2P] (nullable) -- the reference's
 * estimator <E O*> + conj<E_k> - 2 <E> <O*> (source/network_functions/ExpectationValue.cu:243-253)
 * over the instance's walkers, summed in a fixed order -- and eloc [2 walkers] (nullable) */
RBMG_API int rbmg_batch_result(const rbmg_batch* batch, int instance, double* energy, double* grad, double* eloc);
/* the configurations of instance i's walkers after the last replay, spins [walkers][ceil(N/64)] */
RBMG_API int rbmg_batch_spins(const rbmg_batch* batch, int instance, uint64_t* spins);
RBMG_API int rbmg_batch_info(const rbmg_batch* batch, int* num_instances, uint64_t* accepts, double* tuned_ms);

/* ---------------------------------------------------------------- optimisers
 * The reference's gradient-descent methods (pyRBMonGPU/gradient_descent.py, Python on the
 * host) as device kernels with their state on the device.  hyper[5] = {eta, gamma or
 * beta1, beta2, epsilon, p}; unused entries are ignored:
 *   VANILLA eta (:14-22)            MOMENTUM eta, gamma (:37-47)     NAG eta, gamma (:51-61)
 *   ADAGRAD eta, eps (:70-83)       ADADELTA gamma, eps (:86-108)    RMSPROP eta, gamma, eps (:111-126)
 *   ADAM beta1, beta2, eta, eps (:135-152)   PADAM beta1, beta2, eta, eps, p (:161-181)
 *   ADAMAX beta1, beta2, eta, eps (:190-214)
 * Adam divides by 1 - beta (no power of the step count) as the reference does
 * (:147-148) unless flags has RBMG_OPT_STANDARD_BIAS (Kingma & Ba's 1 - beta^t). */
#define RBMG_OPT_VANILLA 0
#define RBMG_OPT_MOMENTUM 1
#define RBMG_OPT_NAG 2
#define RBMG_OPT_ADAGRAD 3
#define RBMG_OPT_ADADELTA 4
#define RBMG_OPT_RMSPROP 5
#define RBMG_OPT_ADAM 6
#define RBMG_OPT_PADAM 7
#define RBMG_OPT_ADAMAX 8
#define RBMG_OPT_STANDARD_BIAS 1
typedef struct rbmg_optimizer rbmg_optimizer;
RBMG_API int rbmg_optimizer_create(int method, int num_params, const double* hyper, int num_hyper, int flags,
                                   rbmg_optimizer** out);
RBMG_API int rbmg_optimizer_destroy(rbmg_optimizer* opt);
/* zero the state (velocities, moments) and the step count */
RBMG_API int rbmg_optimizer_reset(rbmg_optimizer* opt);
RBMG_API int rbmg_optimizer_num_steps(const rbmg_optimizer* opt, uint64_t* steps);
/* one step of the generators' loop body with a host gradient (the reference's
 * gradient_function): params [2P] in/out, grad [2P]; eta >= 0 overrides hyper[0] for this
 * step (the reference's callable eta), eta < 0 keeps it */
RBMG_API int rbmg_optimizer_update(rbmg_optimizer* opt, double* params, const double* grad, double eta);
/* NAG's evaluation point params - gamma velocity (:56) -> out [2P] */
RBMG_API int rbmg_optimizer_lookahead(rbmg_optimizer* opt, const double* params, double* out);
/* Fused ground-state step (the groundstate branch of set_params_and_return_gradient,
 * pyRBMonGPU/LearningByGradientDescent.py:128-137, with the optimiser's update): the
 * energy gradient of rbmg_ev_gradient formed on the device, the update applied to the
 * device copy of psi's parameters, and psi's device parameters rewritten; only the
 * energy <H> [2] (at the parameters before the update) comes back.  NAG takes the
 * gradient at params - gamma velocity.  psi's host parameters follow on the next read. */
RBMG_API int rbmg_optimizer_step_energy(rbmg_optimizer* opt, rbmg_psi* psi, const rbmg_operator* op,
                                        rbmg_ensemble* ens, double eta, double* energy /* [2] */);

/* ---------------------------------------------------------------- S matrix
 * get_S_matrix (source/network_functions/S_matrix.cu:10-53; the reference instantiates it
 * for Psi with ExactSummation and binds it to no Python name): S [P][P] complex128,
 * S[k][k'] = sum_s O_k(s) conj(O_k'(s)) / num_steps over every configuration of the
 * ensemble.  As in the reference the exact-summation weight |psi|^2 is not applied and
 * entries k < 2N are zero.  flags: RBMG_S_WEIGHTED weights each configuration by its
 * normalised |psi|^2 (no change for MonteCarloLoop, whose samples carry weight 1);
 * RBMG_S_CENTERED subtracts <O_k> conj(<O_k'>) (the covariance of stochastic
 * reconfiguration).  Psi and PsiDeep, both ensembles; PsiPair has no O_k.  The products
 * run on the tensor cores (BF16 hi / mid / lo parts of the complex64 rows, FP32 sums of at
 * most 1024 samples, FP64 matrix); RBMG_S_SIMT (extension) takes the FP32 CUDA-core tile
 * kernel instead.  A tensor-core wait that gives up returns RBMG_ETIMEOUT. */
#define RBMG_S_WEIGHTED 1
#define RBMG_S_CENTERED 2
#define RBMG_S_SIMT 4
RBMG_API int rbmg_s_matrix(const rbmg_psi* psi, rbmg_ensemble* ens, int flags, double* out /* [2 P P] */);
/* Extension: device time (CUDA events) of the last rbmg_s_matrix call's accumulation
 * launches on this thread, and the number of kernels they launched (the measurement hook
 * of the benchmark). */
RBMG_API int rbmg_s_matrix_timing(double* ms, int* launches);

/* FP32 FMA throughput of the current device in TFLOP/s (a probe kernel of `iters`
 * x 128 independent FMAs per thread), the roofline denominator of the sampler. */
RBMG_API int rbmg_probe_fp32_tflops(int iters, double* tflops);
/* the same probe on packed pairs (fma.rn.f32x2, two FMAs per instruction) */
RBMG_API int rbmg_probe_fp32x2_tflops(int iters, double* tflops);

#ifdef __cplusplus
}
#endif
#endif
