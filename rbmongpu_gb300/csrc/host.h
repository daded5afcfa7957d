// Host-side objects behind the C ABI handles, shared by capi.cu and deep.cu.
#pragma once

#include <complex>
#include <cstdint>
#include <cstring>
#include <functional>
#include <memory>
#include <string>
#include <vector>

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "../../include/rbmg.h"
#include "kernels.h"

namespace rbmg {

using cplx = std::complex<double>;

void set_error(const std::string& msg);
int fail(int code, const std::string& msg);
int cuda_fail(cudaError_t e, const char* where);

#define RBMG_CK(call)                                                    \
    do {                                                                 \
        cudaError_t e__ = (call);                                        \
        if (e__ != cudaSuccess) return ::rbmg::cuda_fail(e__, #call);    \
    } while (0)

// grow-only device buffer
struct DevBuf {
    void* p = nullptr;
    size_t bytes = 0;
    DevBuf() = default;
    DevBuf(const DevBuf&) = delete;
    DevBuf& operator=(const DevBuf&) = delete;
    ~DevBuf() { release(); }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
    }
    cudaError_t ensure(size_t n) {
        if (n <= bytes) return cudaSuccess;
        release();
        cudaError_t e = cudaMalloc(&p, n);
        if (e != cudaSuccess) { p = nullptr; return e; }
        bytes = n;
        return cudaSuccess;
    }
    template <typename T>
    T* as() const { return static_cast<T*>(p); }
};

cudaStream_t stream();

inline int nwords_of(int N) { return (N + 63) / 64; }

struct DeepLayerHost {
    int size = 0, conn = 0;
    std::vector<uint32_t> connections;   // [conn][size]
    std::vector<cplx> biases;            // [size]
    std::vector<cplx> weights;           // [conn][size]
};

struct DeepDev;   // deep.cu

}  // namespace rbmg

struct rbmg_psi {
    int kind = 0;     // 0 RBM, 1 PsiDeep, 2 PsiPair
    int N = 0;
    double prefactor = 1.0;
    std::vector<double> alpha, beta;
    int free_quantum_axis = 0;   // the Hilbert-space distance's alpha / beta terms (PsiBase.hpp:164)
    // RBM
    int M = 0, Mpad = 0;
    std::vector<rbmg::cplx> b, W;
    rbmg::DevBuf dW, db, dWq, dbq;     // complex64 rows, and the sampler's paired copies (kernels.h)
    rbmg::DevBuf dWt;                  // W transposed, units paired [Mpad / 2][N] (RbmDev::Wt4)
    rbmg::DevBuf dWtc;                 // W as BF16 hi / mid / lo tensor-core operands (angles_tc.cu), if supported
    rbmg::DevBuf tc_error;             // set when a tensor-core pass of this psi gave up waiting
    mutable rbmg::DevBuf dW64, db64;   // FP64 copies for the Hilbert-space distance pass, uploaded on use
    mutable bool f64_valid = false;
    // deep / pair
    std::vector<rbmg::DeepLayerHost> layers;
    std::vector<rbmg::cplx> final_weights;
    int translational_invariance = 0;
    rbmg::DeepNetDev deep_dev[2] = {};     // device nets (deep.cu): complex net, or PsiPair real / imaginary
    std::shared_ptr<void> deep_host;       // owner of the device buffers behind deep_dev
    int width = 0;

    // device master copy of the packed parameter vector [P] complex128, written by the
    // device optimiser (optim.cu); while host_stale is set the vectors above are out of
    // date and psi_sync_host refreshes them before any host read
    rbmg::DevBuf dmaster;
    bool master_valid = false;
    mutable bool host_stale = false;

    int num_params() const;
    rbmg::RbmDev rbm_dev() const {
        return rbmg::RbmDev{N, M, Mpad, static_cast<const float2*>(dW.p), static_cast<const float2*>(db.p),
                            static_cast<const float4*>(dWq.p), static_cast<const float4*>(dbq.p),
                            static_cast<const float4*>(dWt.p)};
    }
};

namespace rbmg {
// optim.cu: host copy of the parameters from the device master when the optimiser
// has moved them; packed device master from the host copy; device parameters (the
// layouts the kernels read) from a packed vector on the device
int psi_sync_host(const rbmg_psi* psi);
int psi_master_ensure(rbmg_psi* psi);
int psi_scatter(rbmg_psi* psi, const double2* packed);
// capi.cu: the energy gradient formed on the device, d_grad [P]; energy to value[2]
int ev_gradient_device(const rbmg_psi* psi, const rbmg_operator* op, rbmg_ensemble* ens, double2* d_grad,
                       double* value);
// angles_tc.cu: hidden angles from scratch on the tensor cores
bool rbm_tc_supported(int N, int Mpad);
size_t rbm_tc_pack_elems(int Mpad, int Kp);
int rbm_tc_kp(int N);
cudaError_t launch_rbm_tc_pack(int N, int M, int Mpad, const float2* W, __nv_bfloat16* out, cudaStream_t st);
cudaError_t launch_angles_tc(int count, int N, int Mpad, const uint64_t* spins, const float2* b,
                             const __nv_bfloat16* images, float4* theta, float2* re, float2* plain, int* error,
                             cudaStream_t st);
// density.cu: out = a - b elementwise
cudaError_t launch_sub(int count, const double2* a, const double2* b, double2* out, cudaStream_t st);
// density.cu: out [2^na] += w_s |eloc_s|^2 at the bin of the first na spins
cudaError_t launch_diag_density(int count, int enumerate, uint64_t enum_base, const uint64_t* spins, int nw,
                                const double* w, const double2* eloc, int na, double* out, cudaStream_t st);
cudaError_t launch_grad_final(const double2* O, const double2* EO, const double2* Ek, const double2* sums,
                              double norm, double2 E0, int first, long count, double2* grad, cudaStream_t st);
}  // namespace rbmg

struct rbmg_operator {
    int S = 0, L = 0;
    std::vector<rbmg::cplx> coef;
    std::vector<int> types, idx;
    // compact form
    std::vector<int> ypow, nflip, flip_off, flip_sites, offdiag_slot;
    std::vector<uint64_t> zmask;
    int num_offdiag = 0;
    int max_site = -1;
    rbmg::DevBuf d_coef, d_coef32, d_site1, d_next1, d_ypow, d_zmask, d_nflip, d_flip_off, d_flip_sites, d_slot;
    rbmg::DevBuf d_offdiag;
    // per-site CSR of the off-diagonal slots whose string flips the site (E_k term)
    std::vector<int> site_ptr, site_slots;
    rbmg::DevBuf d_site_ptr, d_site_slots;
    int site_ptr_N = -1;
    rbmg::OpDev dev() const {
        return rbmg::OpDev{S,
                           d_coef.as<double2>(),
                           d_ypow.as<int>(),
                           d_zmask.as<uint64_t>(),
                           d_nflip.as<int>(),
                           d_flip_off.as<int>(),
                           d_flip_sites.as<int>(),
                           d_slot.as<int>(),
                           num_offdiag,
                           d_coef32.as<float2>(),
                           d_site1.as<int>(),
                           d_next1.as<int>(),
                           d_offdiag.as<int>()};
    }
};

// per-site lists of the off-diagonal strings flipping each site, built (once per N) on the
// device for the E_k term (capi.cu)
int op_site_lists(rbmg_operator* op, int N);

struct rbmg_ensemble {
    int kind = 0;   // 0 MonteCarloLoop, 1 ExactSummation, 2 fixed sample set
    // MonteCarloLoop
    uint32_t num_samples = 0, num_sweeps = 1, num_therm = 0, num_chains = 1;
    uint64_t seed = 0;
    int total_z = 0, sector = 0;
    uint32_t fast_sweep_tries = 0;
    rbmg::DevBuf spins, rng_index, accepts, proposals;
    int spins_words = 0;
    std::vector<uint64_t> last_accepts, last_proposals;
    // ExactSummation
    uint32_t num_spins = 0;
    int exact_total_z = 0;
    std::vector<uint64_t> allowed;          // sector configurations
    rbmg::DevBuf d_allowed;                 // sector configurations; fixed sample set (kind 2)
    uint64_t fixed_count = 0;               // fixed sample set: number of configurations

    uint64_t num_steps() const;
};

// walkers that persist on the device between calls (capi.cu); the learned-proposal
// steps (proposal.cu) keep their angles and logits in `learned`
struct rbmg_chain {
    int N = 0, nw = 0;
    uint32_t walkers = 0;
    uint64_t seed = 0;
    rbmg::DevBuf spins, rng_index, accepts, proposals;
    bool initialised = false;
    int learned_streams = 0;   // frozen learned steps on 1 to 4 streams; 0: automatic
    std::shared_ptr<void> learned;
};
