// Gradient-descent optimisers on the device, and the fused variational step.
//
// The reference runs its optimisers in Python on the host (pyRBMonGPU/gradient_descent.py)
// and reaches the device through set_params_and_return_gradient
// (pyRBMonGPU/LearningByGradientDescent.py:103-157): every step copies the parameters
// host->device and the gradient device->host.  Here the packed parameter vector
// (complex128, the reference's layout [alpha, beta, network parameters]) has a master
// copy on the device; one step forms the energy gradient from the sampler's sums on the
// device, applies the optimiser's update to the master and writes the parameters the
// kernels read (complex64 padded RBM rows, PsiDeep layers).  Only the energy comes back.
//
// Every method of the reference works elementwise on the real vector
// hstack(params.real, params.imag) (gradient_descent.py:5-11); the kernels work on the
// interleaved (re, im) doubles, the same arithmetic in another order of the elements.
// The operations are rounded one by one (no contraction into FMA), in the order of the
// reference's numpy expressions, so that they give the reference's values.
#include <algorithm>
#include <cmath>
#include <memory>
#include <vector>

#include "host.h"

namespace rbmg {

namespace {

struct OptHp {
    double eta, gamma, beta2, eps, p;   // gamma doubles as beta1
};

// one step on n doubles; s0..s2 are the method's state vectors (zero at the start)
__global__ void optim_update_kernel(int method, long n, double* __restrict__ p, const double* __restrict__ g,
                                    double* __restrict__ s0, double* __restrict__ s1, double* __restrict__ s2,
                                    OptHp hp, double bc1, double bc2) {
    const long i = static_cast<long>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double gi = g[i];
    double pi = p[i];
    const double one_g = __dsub_rn(1.0, hp.gamma), one_b2 = __dsub_rn(1.0, hp.beta2);
    switch (method) {
        case RBMG_OPT_VANILLA:   // :19  params -= eta * gradient
            pi = __dsub_rn(pi, __dmul_rn(hp.eta, gi));
            break;
        case RBMG_OPT_MOMENTUM:  // :42-44  velocity = gamma velocity + eta gradient; params -= velocity
        case RBMG_OPT_NAG: {     // :56-58  (gradient taken at params - gamma velocity)
            const double v = __dadd_rn(__dmul_rn(hp.gamma, s0[i]), __dmul_rn(hp.eta, gi));
            s0[i] = v;
            pi = __dsub_rn(pi, v);
            break;
        }
        case RBMG_OPT_ADAGRAD: {  // :77-80  G += g^2; params -= eta / (G + eps) g
            const double G = __dadd_rn(s0[i], __dmul_rn(gi, gi));
            s0[i] = G;
            pi = __dsub_rn(pi, __dmul_rn(__ddiv_rn(hp.eta, __dadd_rn(G, hp.eps)), gi));
            break;
        }
        case RBMG_OPT_ADADELTA: {  // :96-105
            const double dp_old = s0[i];
            const double Edp2 = __dadd_rn(__dmul_rn(hp.gamma, s1[i]), __dmul_rn(one_g, __dmul_rn(dp_old, dp_old)));
            const double Eg2 = __dadd_rn(__dmul_rn(hp.gamma, s2[i]), __dmul_rn(one_g, __dmul_rn(gi, gi)));
            const double rms_g = __dsqrt_rn(__dadd_rn(Eg2, hp.eps));
            const double rms_dp = __dsqrt_rn(__dadd_rn(Edp2, hp.eps));
            const double dp = __dmul_rn(__ddiv_rn(-rms_dp, rms_g), gi);
            s0[i] = dp;
            s1[i] = Edp2;
            s2[i] = Eg2;
            pi = __dadd_rn(pi, dp);
            break;
        }
        case RBMG_OPT_RMSPROP: {  // :119-123  G = gamma G + (1 - gamma) g^2; params -= eta / (G + eps) g
            const double G = __dadd_rn(__dmul_rn(hp.gamma, s0[i]), __dmul_rn(one_g, __dmul_rn(gi, gi)));
            s0[i] = G;
            pi = __dsub_rn(pi, __dmul_rn(__ddiv_rn(hp.eta, __dadd_rn(G, hp.eps)), gi));
            break;
        }
        case RBMG_OPT_ADAM: {  // :144-150  bias corrections bc1, bc2 from the host
            const double m = __dadd_rn(__dmul_rn(hp.gamma, s0[i]), __dmul_rn(one_g, gi));
            const double v = __dadd_rn(__dmul_rn(hp.beta2, s1[i]), __dmul_rn(one_b2, __dmul_rn(gi, gi)));
            s0[i] = m;
            s1[i] = v;
            const double mh = __ddiv_rn(m, bc1), vh = __ddiv_rn(v, bc2);
            pi = __dsub_rn(pi, __dmul_rn(__ddiv_rn(hp.eta, __dadd_rn(__dsqrt_rn(vh), hp.eps)), mh));
            break;
        }
        case RBMG_OPT_PADAM: {  // :170-179  v_hat = max(v_hat, v); params -= eta / (v_hat^p + eps) m
            const double m = __dadd_rn(__dmul_rn(hp.gamma, s0[i]), __dmul_rn(one_g, gi));
            const double v = __dadd_rn(__dmul_rn(hp.beta2, s1[i]), __dmul_rn(one_b2, __dmul_rn(gi, gi)));
            const double vhat = fmax(s2[i], v);
            s0[i] = m;
            s1[i] = v;
            s2[i] = vhat;
            const double vp = hp.p == 0.5 ? __dsqrt_rn(vhat) : (hp.p == 1.0 ? vhat : pow(vhat, hp.p));
            pi = __dsub_rn(pi, __dmul_rn(__ddiv_rn(hp.eta, __dadd_rn(vp, hp.eps)), m));
            break;
        }
        case RBMG_OPT_ADAMAX: {  // :200-206  u = max(beta2 u, |g|); params -= eta / (u + eps) m / (1 - beta1)
            const double m = __dadd_rn(__dmul_rn(hp.gamma, s0[i]), __dmul_rn(one_g, gi));
            const double u = fmax(__dmul_rn(hp.beta2, s1[i]), fabs(gi));
            s0[i] = m;
            s1[i] = u;
            const double mh = __ddiv_rn(m, one_g);
            pi = __dsub_rn(pi, __dmul_rn(__ddiv_rn(hp.eta, __dadd_rn(u, hp.eps)), mh));
            break;
        }
        default: break;
    }
    p[i] = pi;
}

// NAG's evaluation point params - gamma velocity (gradient_descent.py:56)
__global__ void lookahead_kernel(long n, const double* p, const double* v, double gamma, double* out) {
    const long i = static_cast<long>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i < n) out[i] = __dsub_rn(p[i], __dmul_rn(gamma, v[i]));
}

// ExpectationValue.cu:243-253: grad = <E O*> + conj<E_k> - 2 <E> <O*>, from the centred
// sums EO' = sum w (E - E0) O*, Ek' = sum w (E_k - E0 O):
// grad = EO' + conj(Ek') + (E0 + conj(E0) - 2 <E>) conj<O>   (all sums times norm)
__global__ void grad_final_kernel(const double2* O, const double2* EO, const double2* Ek, const double2* sums,
                                  double norm, double2 E0, int first, long count, double2* grad) {
    const long k = static_cast<long>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (k < first) grad[k] = make_double2(0.0, 0.0);
    if (k >= count) return;
    const double Er = __dmul_rn(sums[0].x, norm), Ei = __dmul_rn(sums[0].y, norm);
    const double sr = __dsub_rn(__dadd_rn(E0.x, E0.x), __dmul_rn(2.0, Er));
    const double si = __dsub_rn(__dsub_rn(E0.y, E0.y), __dmul_rn(2.0, Ei));
    const double orr = __dmul_rn(O[k].x, norm), oi = __dmul_rn(O[k].y, norm);
    const double eor = __dmul_rn(EO[k].x, norm), eoi = __dmul_rn(EO[k].y, norm);
    const double ekr = __dmul_rn(Ek[k].x, norm), eki = __dmul_rn(Ek[k].y, norm);
    // shift * conj(o) = (sr + i si)(orr - i oi)
    const double tr = __dadd_rn(__dmul_rn(sr, orr), __dmul_rn(si, oi));
    const double ti = __dsub_rn(__dmul_rn(si, orr), __dmul_rn(sr, oi));
    grad[first + k] = make_double2(__dadd_rn(__dadd_rn(eor, ekr), tr), __dadd_rn(__dsub_rn(eoi, eki), ti));
}

// RBM parameters the kernels read: b [Mpad], W [N][Mpad] complex64 (zero padding untouched)
__global__ void rbm_scatter_kernel(const double2* packed, int N, int M, int Mpad, float2* b, float2* W) {
    const long q = static_cast<long>(blockIdx.x) * blockDim.x + threadIdx.x;
    const long total = static_cast<long>(M) + static_cast<long>(N) * M;
    if (q >= total) return;
    const double2 z = packed[2 * N + q];
    const float2 f = make_float2(static_cast<float>(z.x), static_cast<float>(z.y));
    if (q < M) {
        b[q] = f;
    } else {
        const long r = q - M;
        const long i = r / M, j = r - i * M;
        W[i * Mpad + j] = f;
    }
}

struct ScatterSeg {
    long src;        // first packed index
    int count;
    int part;        // 0 complex (or PsiPair real part), 1 PsiPair imaginary part
    int real_only;   // PsiPair: the part goes in as a real number
    float2* d32;
    double2* d64;
};
constexpr int kMaxSegs = 16;
struct ScatterTable {
    int n;
    ScatterSeg seg[kMaxSegs];
};

__global__ void deep_scatter_kernel(const double2* packed, ScatterTable t) {
    const ScatterSeg& s = t.seg[blockIdx.y];
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < s.count; q += gridDim.x * blockDim.x) {
        double2 z = packed[s.src + q];
        if (s.real_only) z = make_double2(s.part == 0 ? z.x : z.y, 0.0);
        s.d32[q] = make_float2(static_cast<float>(z.x), static_cast<float>(z.y));
        s.d64[q] = z;
    }
}

int blocks_of(long n, int threads) { return static_cast<int>((n + threads - 1) / threads); }

void pack_host(const rbmg_psi* psi, std::vector<cplx>& out) {
    out.assign(psi->num_params(), cplx(0.0, 0.0));
    const int N = psi->N;
    for (int i = 0; i < N; i++) {
        out[i] = cplx(psi->alpha[i], 0.0);
        out[N + i] = cplx(psi->beta[i], 0.0);
    }
    size_t k = 2 * N;
    if (psi->kind == 0) {
        for (const auto& v : psi->b) out[k++] = v;
        for (const auto& v : psi->W) out[k++] = v;
    } else {
        for (const auto& L : psi->layers) {
            for (const auto& v : L.biases) out[k++] = v;
            for (const auto& v : L.weights) out[k++] = v;
        }
        for (const auto& v : psi->final_weights) out[k++] = v;
    }
}

}  // namespace

cudaError_t launch_grad_final(const double2* O, const double2* EO, const double2* Ek, const double2* sums,
                              double norm, double2 E0, int first, long count, double2* grad, cudaStream_t st) {
    const long n = std::max<long>(count, first);
    grad_final_kernel<<<blocks_of(n, 256), 256, 0, st>>>(O, EO, Ek, sums, norm, E0, first, count, grad);
    return cudaGetLastError();
}

int psi_sync_host(const rbmg_psi* cpsi) {
    if (!cpsi->host_stale) return RBMG_OK;
    rbmg_psi* psi = const_cast<rbmg_psi*>(cpsi);
    std::vector<cplx> v(psi->num_params());
    RBMG_CK(cudaMemcpyAsync(v.data(), psi->dmaster.p, sizeof(cplx) * v.size(), cudaMemcpyDeviceToHost, stream()));
    RBMG_CK(cudaStreamSynchronize(stream()));
    const int N = psi->N;
    for (int i = 0; i < N; i++) {
        psi->alpha[i] = v[i].real();
        psi->beta[i] = v[N + i].real();
    }
    size_t k = 2 * N;
    if (psi->kind == 0) {
        for (auto& x : psi->b) x = v[k++];
        for (auto& x : psi->W) x = v[k++];
    } else {
        for (auto& L : psi->layers) {
            for (auto& x : L.biases) x = v[k++];
            for (auto& x : L.weights) x = v[k++];
        }
        for (auto& x : psi->final_weights) x = v[k++];
    }
    psi->host_stale = false;
    return RBMG_OK;
}

int psi_master_ensure(rbmg_psi* psi) {
    if (psi->master_valid) return RBMG_OK;
    std::vector<cplx> v;
    pack_host(psi, v);
    RBMG_CK(psi->dmaster.ensure(sizeof(cplx) * v.size()));
    RBMG_CK(cudaMemcpyAsync(psi->dmaster.p, v.data(), sizeof(cplx) * v.size(), cudaMemcpyHostToDevice, stream()));
    RBMG_CK(cudaStreamSynchronize(stream()));
    psi->master_valid = true;
    return RBMG_OK;
}

int psi_scatter(rbmg_psi* psi, const double2* packed) {
    if (psi->kind == 0) {
        const long total = static_cast<long>(psi->M) + static_cast<long>(psi->N) * psi->M;
        rbm_scatter_kernel<<<blocks_of(total, 256), 256, 0, stream()>>>(packed, psi->N, psi->M, psi->Mpad,
                                                                         psi->db.as<float2>(), psi->dW.as<float2>());
        RBMG_CK(cudaGetLastError());
        RBMG_CK(launch_rbm_pairs(psi->N, psi->Mpad, psi->dW.as<float2>(), psi->db.as<float2>(), psi->dWq.as<float4>(),
                                 psi->dbq.as<float4>(), psi->dWt.as<float4>(), stream()));
        if (psi->dWtc.p)
            RBMG_CK(launch_rbm_tc_pack(psi->N, psi->M, psi->Mpad, psi->dW.as<float2>(),
                                       psi->dWtc.as<__nv_bfloat16>(), stream()));
        // the FP64 copies (exact-summation weights, Hilbert-space distance) in the host
        // layout b [M], W [N][M] are the packed vector's tail as it stands
        const size_t M = psi->M, NM = static_cast<size_t>(psi->N) * psi->M;
        RBMG_CK(psi->db64.ensure(sizeof(cplx) * M));
        RBMG_CK(psi->dW64.ensure(sizeof(cplx) * NM));
        RBMG_CK(cudaMemcpyAsync(psi->db64.p, packed + 2 * psi->N, sizeof(cplx) * M, cudaMemcpyDeviceToDevice,
                                stream()));
        RBMG_CK(cudaMemcpyAsync(psi->dW64.p, packed + 2 * psi->N + M, sizeof(cplx) * NM, cudaMemcpyDeviceToDevice,
                                stream()));
        psi->f64_valid = true;
        return RBMG_OK;
    }
    ScatterTable t{};
    const int parts = psi->kind == 2 ? 2 : 1;
    const int L = static_cast<int>(psi->layers.size());
    int maxc = 1;
    for (int part = 0; part < parts; part++) {
        const DeepNetDev& d = psi->deep_dev[part];
        long k = 2 * psi->N;
        auto add = [&](long src, int count, const float2* d32, const double2* d64) {
            ScatterSeg& s = t.seg[t.n++];
            s.src = src;
            s.count = count;
            s.part = part;
            s.real_only = psi->kind == 2;
            s.d32 = const_cast<float2*>(d32);
            s.d64 = const_cast<double2*>(d64);
            maxc = std::max(maxc, count);
        };
        for (int l = 0; l < L; l++) {
            const auto& Ly = psi->layers[l];
            add(k, Ly.size, d.b[l], d.b64[l]);
            add(k + Ly.size, Ly.conn * Ly.size, d.w[l], d.w64[l]);
            k += Ly.size + static_cast<long>(Ly.conn) * Ly.size;
        }
        add(k, static_cast<int>(psi->final_weights.size()), d.fw, d.fw64);
    }
    const dim3 grid(std::min(blocks_of(maxc, 256), 64), t.n);
    deep_scatter_kernel<<<grid, 256, 0, stream()>>>(packed, t);
    RBMG_CK(cudaGetLastError());
    return RBMG_OK;
}

}  // namespace rbmg

using namespace rbmg;

struct rbmg_optimizer {
    int method = 0, P = 0, flags = 0;
    OptHp hp{};
    uint64_t steps = 0;
    DevBuf s0, s1, s2, grad, look, io;
};

namespace {

int state_reset(rbmg_optimizer* o) {
    const size_t bytes = sizeof(double) * 2 * static_cast<size_t>(o->P);
    RBMG_CK(cudaMemsetAsync(o->s0.p, 0, bytes, stream()));
    RBMG_CK(cudaMemsetAsync(o->s1.p, 0, bytes, stream()));
    RBMG_CK(cudaMemsetAsync(o->s2.p, 0, bytes, stream()));
    RBMG_CK(cudaStreamSynchronize(stream()));
    o->steps = 0;
    return RBMG_OK;
}

// update of the packed vector `p` (device, P complex) with the gradient o->grad
int apply(rbmg_optimizer* o, double* p, double eta) {
    OptHp hp = o->hp;
    if (!(eta < 0.0)) hp.eta = eta;
    double bc1 = 1.0 - hp.gamma, bc2 = 1.0 - hp.beta2;   // gradient_descent.py:147-148, no step power
    if (o->method == RBMG_OPT_ADAM && (o->flags & RBMG_OPT_STANDARD_BIAS)) {
        bc1 = 1.0 - std::pow(hp.gamma, static_cast<double>(o->steps + 1));
        bc2 = 1.0 - std::pow(hp.beta2, static_cast<double>(o->steps + 1));
    }
    const long n = 2L * o->P;
    optim_update_kernel<<<blocks_of(n, 256), 256, 0, stream()>>>(o->method, n, p, o->grad.as<double>(),
                                                                 o->s0.as<double>(), o->s1.as<double>(),
                                                                 o->s2.as<double>(), hp, bc1, bc2);
    RBMG_CK(cudaGetLastError());
    o->steps++;
    return RBMG_OK;
}

}  // namespace

extern "C" int rbmg_optimizer_create(int method, int num_params, const double* hyper, int num_hyper, int flags,
                                     rbmg_optimizer** out) {
    if (!out || num_params <= 0 || method < RBMG_OPT_VANILLA || method > RBMG_OPT_ADAMAX)
        return fail(RBMG_EINVAL, "optimizer: bad method or size");
    if (num_hyper < 0 || num_hyper > 5 || (num_hyper > 0 && !hyper)) return fail(RBMG_EINVAL, "optimizer: hyper[5]");
    auto o = std::make_unique<rbmg_optimizer>();
    o->method = method;
    o->P = num_params;
    o->flags = flags;
    double h[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
    for (int i = 0; i < num_hyper; i++) h[i] = hyper[i];
    o->hp = OptHp{h[0], h[1], h[2], h[3], h[4]};
    const size_t bytes = sizeof(double) * 2 * static_cast<size_t>(num_params);
    RBMG_CK(o->s0.ensure(bytes));
    RBMG_CK(o->s1.ensure(bytes));
    RBMG_CK(o->s2.ensure(bytes));
    RBMG_CK(o->grad.ensure(bytes));
    RBMG_CK(o->io.ensure(bytes));
    const int r = state_reset(o.get());
    if (r != RBMG_OK) return r;
    *out = o.release();
    return RBMG_OK;
}

extern "C" int rbmg_optimizer_destroy(rbmg_optimizer* opt) {
    delete opt;
    return RBMG_OK;
}

extern "C" int rbmg_optimizer_reset(rbmg_optimizer* opt) {
    if (!opt) return fail(RBMG_EINVAL, "optimizer: null");
    return state_reset(opt);
}

extern "C" int rbmg_optimizer_num_steps(const rbmg_optimizer* opt, uint64_t* steps) {
    if (!opt || !steps) return fail(RBMG_EINVAL, "optimizer: null");
    *steps = opt->steps;
    return RBMG_OK;
}

extern "C" int rbmg_optimizer_update(rbmg_optimizer* opt, double* params, const double* grad, double eta) {
    if (!opt || !params || !grad) return fail(RBMG_EINVAL, "optimizer update: null");
    const size_t bytes = sizeof(double) * 2 * static_cast<size_t>(opt->P);
    RBMG_CK(cudaMemcpyAsync(opt->io.p, params, bytes, cudaMemcpyHostToDevice, stream()));
    RBMG_CK(cudaMemcpyAsync(opt->grad.p, grad, bytes, cudaMemcpyHostToDevice, stream()));
    const int r = apply(opt, opt->io.as<double>(), eta);
    if (r != RBMG_OK) return r;
    RBMG_CK(cudaMemcpyAsync(params, opt->io.p, bytes, cudaMemcpyDeviceToHost, stream()));
    RBMG_CK(cudaStreamSynchronize(stream()));
    return RBMG_OK;
}

extern "C" int rbmg_optimizer_lookahead(rbmg_optimizer* opt, const double* params, double* out) {
    if (!opt || !params || !out) return fail(RBMG_EINVAL, "optimizer lookahead: null");
    const size_t bytes = sizeof(double) * 2 * static_cast<size_t>(opt->P);
    RBMG_CK(opt->look.ensure(bytes));
    RBMG_CK(cudaMemcpyAsync(opt->io.p, params, bytes, cudaMemcpyHostToDevice, stream()));
    const long n = 2L * opt->P;
    lookahead_kernel<<<blocks_of(n, 256), 256, 0, stream()>>>(n, opt->io.as<double>(), opt->s0.as<double>(),
                                                              opt->hp.gamma, opt->look.as<double>());
    RBMG_CK(cudaGetLastError());
    RBMG_CK(cudaMemcpyAsync(out, opt->look.p, bytes, cudaMemcpyDeviceToHost, stream()));
    RBMG_CK(cudaStreamSynchronize(stream()));
    return RBMG_OK;
}

extern "C" int rbmg_optimizer_step_energy(rbmg_optimizer* opt, rbmg_psi* psi, const rbmg_operator* op,
                                          rbmg_ensemble* ens, double eta, double* energy) {
    if (!opt || !psi || !op || !ens || !energy) return fail(RBMG_EINVAL, "optimizer step: null");
    if (psi->num_params() != opt->P) return fail(RBMG_EINVAL, "optimizer step: num_params differs from the optimizer's");
    int r = psi_master_ensure(psi);
    if (r != RBMG_OK) return r;
    double2* master = psi->dmaster.as<double2>();
    const long n = 2L * opt->P;
    if (opt->method == RBMG_OPT_NAG) {
        // the gradient is taken at params - gamma velocity (gradient_descent.py:56)
        RBMG_CK(opt->look.ensure(sizeof(double) * n));
        lookahead_kernel<<<blocks_of(n, 256), 256, 0, stream()>>>(n, psi->dmaster.as<double>(), opt->s0.as<double>(),
                                                                  opt->hp.gamma, opt->look.as<double>());
        RBMG_CK(cudaGetLastError());
        r = psi_scatter(psi, opt->look.as<double2>());
        if (r != RBMG_OK) return r;
    }
    r = ev_gradient_device(psi, op, ens, opt->grad.as<double2>(), energy);
    if (r != RBMG_OK) return r;
    r = apply(opt, psi->dmaster.as<double>(), eta);
    if (r != RBMG_OK) return r;
    r = psi_scatter(psi, master);
    if (r != RBMG_OK) return r;
    psi->host_stale = true;
    RBMG_CK(cudaStreamSynchronize(stream()));
    if (!std::isfinite(energy[0]) || !std::isfinite(energy[1])) return fail(RBMG_ENAN, "optimizer step: energy not finite");
    return RBMG_OK;
}
