// Exact-summation energy of a complex RBM without any device allocation.
//
// For callers that cannot call cudaMalloc: host threads of a framework that owns all
// device memory through its own pool (where a foreign cudaMalloc would break its
// accounting or fail under its memory cap), or latency-critical loops where an
// allocation and the device-wide synchronisation of cudaFree are not allowed.
// rbmg_ev_value grows a per-thread
// workspace on demand; this entry point instead works in one fixed array in device
// global memory, reserved when the library is loaded and held by every GPU that
// loads it until the process exits.
#include <atomic>
#include <cmath>

#include <cuda_runtime.h>

#include "host.h"
#include "reduce.h"

namespace rbmg {
namespace {

constexpr int kNoAllocMaxSpins = 14;                          // 2^14 = 16384 basis states
constexpr size_t kNoAllocStates = size_t(1) << kNoAllocMaxSpins;
constexpr size_t kNoAllocBytes = size_t(1) << 20;             // 1 MiB

// The scratch.  In host code this name is only a stand-in for the device symbol: its
// device address comes from cudaGetSymbolAddress (noalloc_scratch() below).
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

// layout inside the scratch (byte offsets, 256-byte aligned)
constexpr size_t kOffLogPsi = 0;                                            // double2 [states]
constexpr size_t kOffWeights = kOffLogPsi + kNoAllocStates * sizeof(double2);   // double  [states]
constexpr size_t kOffEloc = kOffWeights + kNoAllocStates * sizeof(double);      // double2 [states]
constexpr size_t kOffBlocks = kOffEloc + kNoAllocStates * sizeof(double2);      // double2 [kSumBlocks * kMaxSeries]
constexpr size_t kOffBlockMax = kOffBlocks + kSumBlocks * kMaxSeries * sizeof(double2);   // double [kSumBlocks]
constexpr size_t kOffSums = kOffBlockMax + kSumBlocks * sizeof(double);         // double2 [kMaxSeries]
static_assert(kOffSums + kMaxSeries * sizeof(double2) <= kNoAllocBytes, "no-alloc scratch too small");

// FP64 log psi of basis state t, from the FP32 device parameters (one warp per state)
__global__ void logpsi64_from32_kernel(RbmDev P, int count, double2* out) {
    const int lane = threadIdx.x & 31;
    const long t = static_cast<long>(blockIdx.x) * kWarpsPerBlock + (threadIdx.x >> 5);
    if (t >= count) return;
    const uint64_t s = static_cast<uint64_t>(t);
    double lr = 0.0, li = 0.0;
    for (int j = lane; j < P.M; j += 32) {
        double ar = P.b[j].x, ai = P.b[j].y;
        for (int i = 0; i < P.N; i++) {
            const float2 w = P.W[static_cast<long>(i) * P.Mpad + j];
            const double sg = ((s >> i) & 1ull) ? 1.0 : -1.0;
            ar += sg * w.x;
            ai += sg * w.y;
        }
        // include/quantum_state/psi_functions.hpp:49-57 in FP64
        const double sgn = ar > 0.0 ? 1.0 : -1.0;
        double tr = sgn * 3.746646023906276 + ar, ti = ai;
        double nr = ar * tr - ai * ti + 7.771429504240965, ni = ar * ti + ai * tr;
        tr = ar * nr - ai * ni + sgn * 10.2180213465;
        ti = ar * ni + ai * nr;
        nr = ar * tr - ai * ti + 9.19376335670885;
        ni = ar * ti + ai * tr;
        const double ur = 5.49914721954 - sgn * 2.16564366435 * ar, ui = -sgn * 2.16564366435 * ai;
        const double den = nr * nr + ni * ni;
        lr += sgn * 0.9003320053750442 * ar + (ur * nr + ui * ni) / den - 0.598139;
        li += sgn * 0.9003320053750442 * ai + (ui * nr - ur * ni) / den;
    }
    for (int off = 16; off >= 1; off >>= 1) {
        lr += __shfl_xor_sync(0xffffffffu, lr, off);
        li += __shfl_xor_sync(0xffffffffu, li, off);
    }
    if (lane == 0) out[t] = make_double2(lr, li);
}

// device address of the scratch on the current device, looked up once per device.  Host
// threads may race on the first lookup; they all store the same address, and the atomic
// entries make that well defined.  A cudaDeviceReset reloads the module, after which the
// cached address is stale: a process that resets a device must not call the entry point
// on that device again.
int noalloc_scratch(unsigned char** out) {
    static std::atomic<unsigned char*> addr[64];
    int dev = 0;
    RBMG_CK(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) return fail(RBMG_EINVAL, "no-alloc: device index out of range");
    unsigned char* a = addr[dev].load(std::memory_order_acquire);
    if (!a) {
        void* p = nullptr;
        RBMG_CK(cudaGetSymbolAddress(&p, g_noalloc_scratch));
        a = static_cast<unsigned char*>(p);
        addr[dev].store(a, std::memory_order_release);
    }
    *out = a;
    return RBMG_OK;
}

}  // namespace
}  // namespace rbmg

using namespace rbmg;

extern "C" int rbmg_ev_value_exact_noalloc(const rbmg_psi* psi, const rbmg_operator* op, int num_spins,
                                           double* value) {
    if (!psi || !op || !value) return fail(RBMG_EINVAL, "no-alloc energy: null argument");
    if (psi->kind != 0) return fail(RBMG_EUNSUPPORTED, "no-alloc energy: complex RBM (Psi) only");
    if (num_spins != psi->N) return fail(RBMG_EINVAL, "no-alloc energy: num_spins does not match psi");
    if (num_spins < 1 || num_spins > kNoAllocMaxSpins)
        return fail(RBMG_EINVAL, "no-alloc energy: N must be between 1 and 14 (scratch holds 2^14 basis states)");
    if (op->max_site >= psi->N) return fail(RBMG_EINVAL, "no-alloc energy: operator acts on a site >= N");
    unsigned char* base = nullptr;
    const int r = noalloc_scratch(&base);
    if (r != RBMG_OK) return r;
    double2* lp = reinterpret_cast<double2*>(base + kOffLogPsi);
    double* w = reinterpret_cast<double*>(base + kOffWeights);
    double2* eloc = reinterpret_cast<double2*>(base + kOffEloc);
    double2* blocks = reinterpret_cast<double2*>(base + kOffBlocks);
    double* bmax = reinterpret_cast<double*>(base + kOffBlockMax);
    double2* sums = reinterpret_cast<double2*>(base + kOffSums);
    cudaStream_t st = stream();
    const int count = 1 << num_spins;
    const RbmDev P = psi->rbm_dev();
    // log psi of every basis state and the FP64 log-sum-exp normalisation
    logpsi64_from32_kernel<<<(count + kWarpsPerBlock - 1) / kWarpsPerBlock, 32 * kWarpsPerBlock, 0, st>>>(P, count, lp);
    RBMG_CK(cudaGetLastError());
    int blocks_used = 0;
    RBMG_CK(launch_max_re2(count, lp, bmax, &blocks_used, st));
    double hmax[kSumBlocks];
    RBMG_CK(cudaMemcpyAsync(hmax, bmax, sizeof(double) * blocks_used, cudaMemcpyDeviceToHost, st));
    RBMG_CK(cudaStreamSynchronize(st));
    double mx = hmax[0];
    for (int b = 1; b < blocks_used; b++) mx = std::fmax(mx, hmax[b]);
    if (!std::isfinite(mx)) return fail(RBMG_ENAN, "no-alloc energy: non-finite log psi");
    RBMG_CK(launch_exp_weights(count, lp, mx, w, st));
    // the sum is accumulated: it must start at zero on every call
    RBMG_CK(cudaMemsetAsync(sums, 0, sizeof(double2) * kMaxSeries, st));
    // local energies (the same estimator kernel as rbmg_ev_value)
    EstLaunch L{};
    L.count = count;
    L.flags = EST_ELOC | EST_ENUMERATE;
    L.eloc = eloc;
    const OpDev od = op->dev();
    RBMG_CK(launch_rbm_estimate(P, &od, nullptr, L, st));
    SeriesSet eset{};
    eset.n = 1;
    eset.v[0] = eloc;
    RBMG_CK(launch_weighted_sums(count, w, eset, blocks, sums, st));
    double2 h;
    RBMG_CK(cudaMemcpyAsync(&h, sums, sizeof(h), cudaMemcpyDeviceToHost, st));
    RBMG_CK(cudaStreamSynchronize(st));
    // reference weights prefactor^2 |psi|^2 (ExactSummation.hpp:75), with w = |psi|^2 e^-mx:
    // <O> = prefactor^2 e^mx sum_s w_s E_s
    const double scale = std::exp(2.0 * std::log(psi->prefactor) + mx);
    value[0] = scale * h.x;
    value[1] = scale * h.y;
    if (!std::isfinite(value[0]) || !std::isfinite(value[1])) return fail(RBMG_ENAN, "no-alloc energy: non-finite");
    return RBMG_OK;
}
