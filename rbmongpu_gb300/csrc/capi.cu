// C ABI of the library (include/rbmg.h): handles, the ensembles' sample streams
// and the estimators of ExpectationValue / HilbertSpaceDistance, orchestrating the
// CUDA kernels of rbm_impl.cuh, deep.cu and reduce_kernels.cu.
#include <algorithm>
#include <cmath>
#include <functional>
#include <memory>
#include <thread>
#include <vector>
#include <unistd.h>

#include <cuda_profiler_api.h>

#include "host.h"
#include "smatrix.h"
#include "rbm64.h"
#include "reduce.h"

namespace rbmg {

// ---------------------------------------------------------------- errors
static thread_local std::string g_last_error;

void set_error(const std::string& msg) { g_last_error = msg; }

int fail(int code, const std::string& msg) {
    g_last_error = msg;
    return code;
}

int cuda_fail(cudaError_t e, const char* where) {
    g_last_error = std::string(where) + ": " + cudaGetErrorString(e);
    return e == cudaErrorMemoryAllocation ? RBMG_ENOMEM : RBMG_ECUDA;
}

cudaStream_t stream() {
    static thread_local cudaStream_t st = nullptr;
    static thread_local int st_dev = -1;
    int dev = 0;
    cudaGetDevice(&dev);
    if (!st || st_dev != dev) {
        cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
        st_dev = dev;
    }
    return st;
}

// deep.cu
int deep_upload(rbmg_psi* psi);
int deep_log_psi(const rbmg_psi* psi, int count, const uint64_t* d_spins, uint64_t enum_base, int enumerate,
                 double2* d_out, cudaStream_t st);

// ---------------------------------------------------------------- workspace
// Grow-only scratch buffers shared by all calls on this thread's device.
struct Workspace {
    DevBuf sample_spins, eloc, logpsi, logpsi_p, T, U, X, Tp, weights, coef1, coef2, coef3, omega, pr, nn;
    DevBuf partial, block_scratch, sums, acc_O, acc_EO, acc_Ek, acc_wO, acc_pO, block_max, zsum;
    DevBuf smat, smean, okrows, sshift, splanes, serror, sout;
    DevBuf acc_B, eabs2, lsums, rw, rwc, acc_C2, acc_C3;
    DevBuf fqa_qa, fqa_r, fqa_flip, fqa_lpf, fqa_lp, fqa_out;   // free-quantum-axis terms of the HSD
};

static Workspace& ws() {
    static thread_local Workspace w;
    return w;
}


}  // namespace rbmg

using namespace rbmg;

int rbmg_psi::num_params() const {
    if (kind == 0) return 2 * N + M + N * M;
    int P = 2 * N;
    for (const auto& l : layers) P += l.size + l.conn * l.size;
    return P + (layers.empty() ? 0 : layers.back().size);
}

uint64_t rbmg_ensemble::num_steps() const {
    if (kind == 0) return num_samples;
    if (kind == 2) return fixed_count;
    if (exact_total_z) return allowed.size();
    return 1ull << num_spins;
}

// ====================================================================== misc
extern "C" const char* rbmg_last_error(void) { return g_last_error.c_str(); }
extern "C" const char* rbmg_version(void) { return "rbmg 0.1 (sm_103a)"; }

extern "C" int rbmg_set_device(int device) {
    RBMG_CK(cudaSetDevice(device));
    return RBMG_OK;
}

extern "C" int rbmg_profiler_start(void) {
    RBMG_CK(cudaProfilerStart());
    return RBMG_OK;
}

extern "C" int rbmg_profiler_stop(void) {
    RBMG_CK(cudaProfilerStop());
    return RBMG_OK;
}

extern "C" int rbmg_activation(double re, double im, double* out) {
    if (!out) return fail(RBMG_EINVAL, "activation: null output");
    // include/quantum_state/psi_functions.hpp:49-57 in FP64
    const cplx z(re, im);
    const double sign = re > 0.0 ? 1.0 : -1.0;
    const cplx den = 9.19376335670885 + z * (sign * 10.2180213465 + z * (7.771429504240965 + z * (sign * 3.746646023906276 + z)));
    const cplx r = sign * 0.9003320053750442 * z + (5.49914721954 - sign * 2.16564366435 * z) / den - 0.598139;
    out[0] = r.real();
    out[1] = r.imag();
    return RBMG_OK;
}

// ====================================================================== Psi
static int rbm_upload(rbmg_psi* p) {
    for (const auto& v : p->b)
        if (!std::isfinite(v.real()) || !std::isfinite(v.imag())) return fail(RBMG_ENAN, "Psi: non-finite b");
    for (const auto& v : p->W)
        if (!std::isfinite(v.real()) || !std::isfinite(v.imag())) return fail(RBMG_ENAN, "Psi: non-finite W");
    std::vector<float2> hb(p->Mpad, make_float2(0.f, 0.f)), hW(static_cast<size_t>(p->N) * p->Mpad,
                                                               make_float2(0.f, 0.f));
    for (int j = 0; j < p->M; j++) hb[j] = make_float2(float(p->b[j].real()), float(p->b[j].imag()));
    for (int i = 0; i < p->N; i++)
        for (int j = 0; j < p->M; j++) {
            const cplx w = p->W[static_cast<size_t>(i) * p->M + j];
            hW[static_cast<size_t>(i) * p->Mpad + j] = make_float2(float(w.real()), float(w.imag()));
        }
    RBMG_CK(p->db.ensure(hb.size() * sizeof(float2)));
    RBMG_CK(p->dW.ensure(hW.size() * sizeof(float2)));
    RBMG_CK(cudaMemcpyAsync(p->db.p, hb.data(), hb.size() * sizeof(float2), cudaMemcpyHostToDevice, stream()));
    RBMG_CK(cudaMemcpyAsync(p->dW.p, hW.data(), hW.size() * sizeof(float2), cudaMemcpyHostToDevice, stream()));
    const size_t kp = static_cast<size_t>((p->Mpad / 32 + 1) / 2) * 32;
    RBMG_CK(p->dWq.ensure(sizeof(float4) * kp * p->N));
    RBMG_CK(p->dbq.ensure(sizeof(float4) * kp));
    RBMG_CK(p->dWt.ensure(sizeof(float2) * static_cast<size_t>(p->Mpad) * p->N));
    RBMG_CK(launch_rbm_pairs(p->N, p->Mpad, p->dW.as<float2>(), p->db.as<float2>(), p->dWq.as<float4>(),
                             p->dbq.as<float4>(), p->dWt.as<float4>(), stream()));
    if (rbm_tc_supported(p->N, p->Mpad)) {
        RBMG_CK(p->dWtc.ensure(sizeof(__nv_bfloat16) * rbm_tc_pack_elems(p->Mpad, rbm_tc_kp(p->N))));
        RBMG_CK(launch_rbm_tc_pack(p->N, p->M, p->Mpad, p->dW.as<float2>(), p->dWtc.as<__nv_bfloat16>(), stream()));
    }
    RBMG_CK(p->tc_error.ensure(sizeof(int)));
    RBMG_CK(cudaMemsetAsync(p->tc_error.p, 0, sizeof(int), stream()));
    RBMG_CK(cudaStreamSynchronize(stream()));
    p->f64_valid = false;
    return RBMG_OK;
}

// FP64 parameter copies for the Hilbert-space distance pass, uploaded on first use
static int rbm_upload64(const rbmg_psi* p) {
    if (p->f64_valid) return RBMG_OK;
    const int rs = psi_sync_host(p);
    if (rs != RBMG_OK) return rs;
    RBMG_CK(p->db64.ensure(sizeof(cplx) * p->M));
    RBMG_CK(p->dW64.ensure(sizeof(cplx) * p->W.size()));
    RBMG_CK(cudaMemcpyAsync(p->db64.p, p->b.data(), sizeof(cplx) * p->M, cudaMemcpyHostToDevice, stream()));
    RBMG_CK(cudaMemcpyAsync(p->dW64.p, p->W.data(), sizeof(cplx) * p->W.size(), cudaMemcpyHostToDevice, stream()));
    RBMG_CK(cudaStreamSynchronize(stream()));
    p->f64_valid = true;
    return RBMG_OK;
}

static Rbm64 rbm64(const rbmg_psi* p) { return Rbm64{p->N, p->M, p->dW64.as<double2>(), p->db64.as<double2>()}; }

extern "C" int rbmg_psi_create(int N, int M, const double* alpha, const double* beta, const double* b,
                               const double* W, double prefactor, int free_quantum_axis, rbmg_psi** out) {
    (void)beta;
    if (!out || N <= 0 || M <= 0 || !b || !W) return fail(RBMG_EINVAL, "Psi: bad arguments");
    if (N > 64 * kMaxWords) return fail(RBMG_EINVAL, "Psi: N exceeds 256 spins");
    const int K = rbm_lanes_k(M);
    if (K < 0) return fail(RBMG_EINVAL, "Psi: M exceeds the largest instantiated hidden layer (576)");
    auto p = std::make_unique<rbmg_psi>();
    p->kind = 0;
    p->N = N;
    p->M = M;
    p->Mpad = 32 * K;
    p->prefactor = prefactor;
    p->free_quantum_axis = free_quantum_axis ? 1 : 0;
    p->alpha.assign(N, 0.0);
    if (alpha) p->alpha.assign(alpha, alpha + N);
    p->beta = p->alpha;   // include/quantum_state/PsiBase.hpp:176, 190: beta_array(alpha)
    p->b.resize(M);
    p->W.resize(static_cast<size_t>(N) * M);
    std::memcpy(p->b.data(), b, sizeof(cplx) * M);
    std::memcpy(p->W.data(), W, sizeof(cplx) * N * M);
    const int r = rbm_upload(p.get());
    if (r != RBMG_OK) return r;
    *out = p.release();
    return RBMG_OK;
}

extern "C" int rbmg_psi_deep_create(int N, int num_layers, const int* sizes, const int* conns,
                                    const uint32_t* const* connections, const double* const* biases,
                                    const double* const* weights, const double* final_weights, const double* alpha,
                                    const double* beta, double prefactor, int free_quantum_axis, int pair,
                                    rbmg_psi** out) {
    (void)beta;
    if (!out || N <= 0 || num_layers <= 0 || num_layers > 3 || !sizes || !conns || !connections || !biases ||
        !weights || !final_weights)
        return fail(RBMG_EINVAL, "PsiDeep: bad arguments");
    if (N > 64 * kMaxWords) return fail(RBMG_EINVAL, "PsiDeep: N exceeds 256 spins");
    auto p = std::make_unique<rbmg_psi>();
    p->kind = pair ? 2 : 1;
    p->N = N;
    p->prefactor = prefactor;
    p->free_quantum_axis = free_quantum_axis ? 1 : 0;
    p->alpha.assign(N, 0.0);
    if (alpha) p->alpha.assign(alpha, alpha + N);
    p->beta = p->alpha;
    int prev = N;
    p->width = N;
    for (int l = 0; l < num_layers; l++) {
        DeepLayerHost L;
        L.size = sizes[l];
        L.conn = conns[l];
        if (L.size <= 0 || L.conn <= 0) return fail(RBMG_EINVAL, "PsiDeep: empty layer");
        L.connections.assign(connections[l], connections[l] + static_cast<size_t>(L.conn) * L.size);
        for (uint32_t c : L.connections)
            if (static_cast<int>(c) >= prev) return fail(RBMG_EINVAL, "PsiDeep: connection index out of range");
        L.biases.resize(L.size);
        std::memcpy(L.biases.data(), biases[l], sizeof(cplx) * L.size);
        L.weights.resize(static_cast<size_t>(L.conn) * L.size);
        std::memcpy(L.weights.data(), weights[l], sizeof(cplx) * L.conn * L.size);
        p->width = std::max(p->width, L.size);
        prev = L.size;
        p->layers.push_back(std::move(L));
    }
    p->final_weights.resize(prev);
    std::memcpy(p->final_weights.data(), final_weights, sizeof(cplx) * prev);
    const int r = deep_upload(p.get());
    if (r != RBMG_OK) return r;
    *out = p.release();
    return RBMG_OK;
}

extern "C" int rbmg_psi_copy(const rbmg_psi* psi, rbmg_psi** out) {
    if (!psi || !out) return fail(RBMG_EINVAL, "copy: null handle");
    const int rs = psi_sync_host(psi);
    if (rs != RBMG_OK) return rs;
    auto p = std::make_unique<rbmg_psi>();
    p->kind = psi->kind;
    p->N = psi->N;
    p->prefactor = psi->prefactor;
    p->alpha = psi->alpha;
    p->beta = psi->beta;
    p->free_quantum_axis = psi->free_quantum_axis;
    p->M = psi->M;
    p->Mpad = psi->Mpad;
    p->b = psi->b;
    p->W = psi->W;
    p->layers = psi->layers;
    p->final_weights = psi->final_weights;
    p->translational_invariance = psi->translational_invariance;
    p->width = psi->width;
    const int r = p->kind == 0 ? rbm_upload(p.get()) : deep_upload(p.get());
    if (r != RBMG_OK) return r;
    *out = p.release();
    return RBMG_OK;
}

extern "C" int rbmg_psi_destroy(rbmg_psi* psi) {
    delete psi;
    return RBMG_OK;
}

extern "C" int rbmg_psi_kind(const rbmg_psi* psi, int* kind) {
    if (!psi || !kind) return fail(RBMG_EINVAL, "kind: null");
    *kind = psi->kind;
    return RBMG_OK;
}

extern "C" int rbmg_psi_shape(const rbmg_psi* psi, int* N, int* M, int* num_params) {
    if (!psi) return fail(RBMG_EINVAL, "shape: null handle");
    if (N) *N = psi->N;
    if (M) *M = psi->kind == 0 ? psi->M : psi->width;
    if (num_params) *num_params = psi->num_params();
    return RBMG_OK;
}

extern "C" int rbmg_psi_get_params(const rbmg_psi* psi, double* params) {
    if (!psi || !params) return fail(RBMG_EINVAL, "get_params: null");
    const int rs = psi_sync_host(psi);
    if (rs != RBMG_OK) return rs;
    cplx* out = reinterpret_cast<cplx*>(params);
    const int N = psi->N;
    for (int i = 0; i < N; i++) {
        out[i] = cplx(psi->alpha[i], 0.0);
        out[N + i] = cplx(psi->beta[i], 0.0);
    }
    size_t k = 2 * N;
    if (psi->kind == 0) {      // source/quantum_state/Psi.cu:71-78
        for (const auto& v : psi->b) out[k++] = v;
        for (const auto& v : psi->W) out[k++] = v;
    } else {                   // source/quantum_state/PsiDeep.cu:120-140
        for (const auto& L : psi->layers) {
            for (const auto& v : L.biases) out[k++] = v;
            for (const auto& v : L.weights) out[k++] = v;
        }
        for (const auto& v : psi->final_weights) out[k++] = v;
    }
    return RBMG_OK;
}

extern "C" int rbmg_psi_set_params(rbmg_psi* psi, const double* params) {
    if (!psi || !params) return fail(RBMG_EINVAL, "set_params: null");
    const cplx* in = reinterpret_cast<const cplx*>(params);
    const int N = psi->N;
    const int P = psi->num_params();
    for (int k = 0; k < P; k++)
        if (!std::isfinite(in[k].real()) || !std::isfinite(in[k].imag())) return fail(RBMG_ENAN, "set_params: non-finite");
    psi->host_stale = false;     // the host copy is the truth again; the device master
    psi->master_valid = false;   // is rebuilt from it by the next device optimiser step
    for (int i = 0; i < N; i++) {
        psi->alpha[i] = in[i].real();
        psi->beta[i] = in[N + i].real();
    }
    size_t k = 2 * N;
    if (psi->kind == 0) {      // source/quantum_state/Psi.cu:80-92
        for (auto& v : psi->b) v = in[k++];
        for (auto& v : psi->W) v = in[k++];
        return rbm_upload(psi);
    }
    for (auto& L : psi->layers) {   // source/quantum_state/PsiDeep.cu:143-177 (PsiPair.cu:55-76 splits re/im)
        for (auto& v : L.biases) v = in[k++];
        for (auto& v : L.weights) v = in[k++];
    }
    for (auto& v : psi->final_weights) v = in[k++];
    return deep_upload(psi);
}

extern "C" int rbmg_psi_free_quantum_axis(const rbmg_psi* psi, int* on) {
    if (!psi || !on) return fail(RBMG_EINVAL, "free_quantum_axis: null");
    *on = psi->free_quantum_axis;
    return RBMG_OK;
}

extern "C" int rbmg_psi_get_prefactor(const rbmg_psi* psi, double* prefactor) {
    if (!psi || !prefactor) return fail(RBMG_EINVAL, "prefactor: null");
    *prefactor = psi->prefactor;
    return RBMG_OK;
}

extern "C" int rbmg_psi_set_prefactor(rbmg_psi* psi, double prefactor) {
    if (!psi) return fail(RBMG_EINVAL, "prefactor: null");
    psi->prefactor = prefactor;
    return RBMG_OK;
}

extern "C" int rbmg_psi_set_translational_invariance(rbmg_psi* psi, int on) {
    if (!psi) return fail(RBMG_EINVAL, "translational_invariance: null");
    if (psi->kind == 0) return fail(RBMG_EINVAL, "translational_invariance: PsiDeep only");
    if (on && psi->N > 64) return fail(RBMG_EUNSUPPORTED, "translational_invariance: N <= 64 (Spins.h:280-285)");
    psi->translational_invariance = on ? 1 : 0;
    return RBMG_OK;
}

// ====================================================================== Operator
// Compact form of the padded table (include/operator/Operator.hpp:45-88): X flips,
// Y flips and multiplies by -i s_i, Z multiplies by s_i, with the ORIGINAL spins.
static int op_compile(rbmg_operator* op) {
    op->ypow.assign(op->S, 0);
    op->nflip.assign(op->S, 0);
    op->flip_off.assign(op->S, 0);
    op->offdiag_slot.assign(op->S, -1);
    op->zmask.assign(static_cast<size_t>(op->S) * kMaxWords, 0);
    op->flip_sites.clear();
    op->num_offdiag = 0;
    op->max_site = -1;
    for (int n = 0; n < op->S; n++) {
        uint64_t flips[kMaxWords] = {0, 0, 0, 0};
        int yp = 0;
        for (int c = 0; c < op->L; c++) {
            const int i = op->idx[static_cast<size_t>(n) * op->L + c];
            if (i < 0) break;
            if (i >= 64 * kMaxWords) return fail(RBMG_EINVAL, "Operator: site index exceeds 256");
            const int t = op->types[static_cast<size_t>(n) * op->L + c];
            if (t < 0 || t > 3) return fail(RBMG_EINVAL, "Operator: pauli type must be 0..3");
            op->max_site = std::max(op->max_site, i);
            const uint64_t bit = 1ull << (i & 63);
            if (t == 1 || t == 2) flips[i >> 6] ^= bit;
            if (t == 2 || t == 3) op->zmask[static_cast<size_t>(n) * kMaxWords + (i >> 6)] ^= bit;
            if (t == 2) yp++;
        }
        op->ypow[n] = yp & 3;
        op->flip_off[n] = static_cast<int>(op->flip_sites.size());
        for (int w = 0; w < kMaxWords; w++)
            for (int bpos = 0; bpos < 64; bpos++)
                if ((flips[w] >> bpos) & 1ull) op->flip_sites.push_back(64 * w + bpos);
        op->nflip[n] = static_cast<int>(op->flip_sites.size()) - op->flip_off[n];
        if (op->nflip[n] > 0) op->offdiag_slot[n] = op->num_offdiag++;
    }
    if (op->flip_sites.empty()) op->flip_sites.push_back(0);
    auto up = [](DevBuf& d, const void* h, size_t bytes) -> cudaError_t {
        cudaError_t e = d.ensure(std::max<size_t>(bytes, 16));
        if (e != cudaSuccess) return e;
        return cudaMemcpy(d.p, h, bytes, cudaMemcpyHostToDevice);
    };
    RBMG_CK(up(op->d_coef, op->coef.data(), sizeof(cplx) * op->S));
    std::vector<float2> c32(op->S);
    for (int n = 0; n < op->S; n++)
        c32[n] = make_float2(static_cast<float>(op->coef[n].real()), static_cast<float>(op->coef[n].imag()));
    RBMG_CK(up(op->d_coef32, c32.data(), sizeof(float2) * op->S));
    std::vector<int> site1(op->S, -1), next1(op->S + 1, op->S);
    for (int n = 0; n < op->S; n++)
        if (op->nflip[n] == 1) site1[n] = op->flip_sites[op->flip_off[n]];
    for (int n = op->S - 1; n >= 0; n--) next1[n] = site1[n] >= 0 ? n : next1[n + 1];
    RBMG_CK(up(op->d_site1, site1.data(), sizeof(int) * op->S));
    RBMG_CK(up(op->d_next1, next1.data(), sizeof(int) * (op->S + 1)));
    RBMG_CK(up(op->d_ypow, op->ypow.data(), sizeof(int) * op->S));
    RBMG_CK(up(op->d_zmask, op->zmask.data(), sizeof(uint64_t) * op->zmask.size()));
    RBMG_CK(up(op->d_nflip, op->nflip.data(), sizeof(int) * op->S));
    RBMG_CK(up(op->d_flip_off, op->flip_off.data(), sizeof(int) * op->S));
    RBMG_CK(up(op->d_flip_sites, op->flip_sites.data(), sizeof(int) * op->flip_sites.size()));
    RBMG_CK(up(op->d_slot, op->offdiag_slot.data(), sizeof(int) * op->S));
    std::vector<int> offdiag;
    for (int n = 0; n < op->S; n++)
        if (op->offdiag_slot[n] >= 0) offdiag.push_back(n);
    if (offdiag.empty()) offdiag.push_back(0);
    RBMG_CK(up(op->d_offdiag, offdiag.data(), sizeof(int) * offdiag.size()));
    return RBMG_OK;
}

// per-site lists of off-diagonal slots flipping that site, for the E_k term
int op_site_lists(rbmg_operator* op, int N) {
    if (op->site_ptr_N == N) return RBMG_OK;
    std::vector<std::vector<int>> per(N);
    for (int n = 0; n < op->S; n++) {
        if (op->offdiag_slot[n] < 0) continue;
        for (int q = 0; q < op->nflip[n]; q++) {
            const int site = op->flip_sites[op->flip_off[n] + q];
            if (site < N) per[site].push_back(op->offdiag_slot[n]);
        }
    }
    op->site_ptr.assign(N + 1, 0);
    op->site_slots.clear();
    for (int i = 0; i < N; i++) {
        op->site_ptr[i] = static_cast<int>(op->site_slots.size());
        op->site_slots.insert(op->site_slots.end(), per[i].begin(), per[i].end());
    }
    op->site_ptr[N] = static_cast<int>(op->site_slots.size());
    if (op->site_slots.empty()) op->site_slots.push_back(0);
    RBMG_CK(op->d_site_ptr.ensure(sizeof(int) * (N + 1)));
    RBMG_CK(op->d_site_slots.ensure(sizeof(int) * op->site_slots.size()));
    RBMG_CK(cudaMemcpy(op->d_site_ptr.p, op->site_ptr.data(), sizeof(int) * (N + 1), cudaMemcpyHostToDevice));
    RBMG_CK(cudaMemcpy(op->d_site_slots.p, op->site_slots.data(), sizeof(int) * op->site_slots.size(),
                       cudaMemcpyHostToDevice));
    op->site_ptr_N = N;
    return RBMG_OK;
}

extern "C" int rbmg_operator_create(int num_strings, int max_string_length, const double* coefficients,
                                    const int* pauli_types, const int* pauli_indices, rbmg_operator** out) {
    if (!out || num_strings <= 0 || max_string_length <= 0 || !coefficients || !pauli_types || !pauli_indices)
        return fail(RBMG_EINVAL, "Operator: bad arguments");
    auto op = std::make_unique<rbmg_operator>();
    op->S = num_strings;
    op->L = max_string_length;
    op->coef.resize(num_strings);
    std::memcpy(op->coef.data(), coefficients, sizeof(cplx) * num_strings);
    for (const auto& c : op->coef)
        if (!std::isfinite(c.real()) || !std::isfinite(c.imag())) return fail(RBMG_ENAN, "Operator: non-finite coefficient");
    const size_t cells = static_cast<size_t>(num_strings) * max_string_length;
    op->types.assign(pauli_types, pauli_types + cells);
    op->idx.assign(pauli_indices, pauli_indices + cells);
    const int r = op_compile(op.get());
    if (r != RBMG_OK) return r;
    *out = op.release();
    return RBMG_OK;
}

extern "C" int rbmg_operator_destroy(rbmg_operator* op) {
    delete op;
    return RBMG_OK;
}

extern "C" int rbmg_operator_shape(const rbmg_operator* op, int* num_strings, int* max_string_length) {
    if (!op) return fail(RBMG_EINVAL, "operator: null");
    if (num_strings) *num_strings = op->S;
    if (max_string_length) *max_string_length = op->L;
    return RBMG_OK;
}

extern "C" int rbmg_operator_tables(const rbmg_operator* op, double* coefficients, int* pauli_types,
                                    int* pauli_indices) {
    if (!op) return fail(RBMG_EINVAL, "operator: null");
    if (coefficients) std::memcpy(coefficients, op->coef.data(), sizeof(cplx) * op->S);
    if (pauli_types) std::memcpy(pauli_types, op->types.data(), sizeof(int) * op->types.size());
    if (pauli_indices) std::memcpy(pauli_indices, op->idx.data(), sizeof(int) * op->idx.size());
    return RBMG_OK;
}

// ====================================================================== ensembles
extern "C" int rbmg_mc_create(uint32_t num_samples, uint32_t num_sweeps, uint32_t num_therm, uint32_t num_chains,
                              uint64_t seed, rbmg_ensemble** out) {
    if (!out || num_chains == 0 || num_samples == 0 || num_sweeps == 0)
        return fail(RBMG_EINVAL, "MonteCarloLoop: zero samples, sweeps or chains");
    if (num_samples % num_chains != 0)   // source/spin_ensembles/MonteCarloLoop.cu:78
        return fail(RBMG_EINVAL, "MonteCarloLoop: num_samples must be a multiple of num_markov_chains");
    auto e = std::make_unique<rbmg_ensemble>();
    e->kind = 0;
    e->num_samples = num_samples;
    e->num_sweeps = num_sweeps;
    e->num_therm = num_therm;
    e->num_chains = num_chains;
    e->seed = seed;
    RBMG_CK(e->rng_index.ensure(sizeof(uint64_t) * num_chains));
    RBMG_CK(cudaMemset(e->rng_index.p, 0, sizeof(uint64_t) * num_chains));
    RBMG_CK(e->accepts.ensure(sizeof(unsigned long long) * num_chains));
    RBMG_CK(e->proposals.ensure(sizeof(unsigned long long) * num_chains));
    e->last_accepts.assign(num_chains, 0);
    e->last_proposals.assign(num_chains, 0);
    *out = e.release();
    return RBMG_OK;
}

extern "C" int rbmg_mc_copy(const rbmg_ensemble* o, rbmg_ensemble** out) {
    if (!o || o->kind != 0) return fail(RBMG_EINVAL, "MonteCarloLoop copy: not a MonteCarloLoop");
    int r = rbmg_mc_create(o->num_samples, o->num_sweeps, o->num_therm, o->num_chains, o->seed, out);
    if (r != RBMG_OK) return r;
    (*out)->total_z = o->total_z;
    (*out)->sector = o->sector;
    (*out)->fast_sweep_tries = o->fast_sweep_tries;
    return RBMG_OK;
}

extern "C" int rbmg_mc_set_total_z_symmetry(rbmg_ensemble* mc, int sector) {
    if (!mc || mc->kind != 0) return fail(RBMG_EINVAL, "set_total_z_symmetry: not a MonteCarloLoop");
    mc->total_z = 1;
    mc->sector = sector;
    return RBMG_OK;
}

// set_fast_sweep (MonteCarloLoop.hpp:288-291): multi-spin masks, the AND of num_tries random
// configurations (0 draws one, as the reference's loop does); a sampling sweep is then one
// update instead of N
extern "C" int rbmg_mc_set_fast_sweep(rbmg_ensemble* mc, uint32_t num_tries) {
    if (!mc || mc->kind != 0) return fail(RBMG_EINVAL, "set_fast_sweep: not a MonteCarloLoop");
    if (num_tries > 64) return fail(RBMG_EINVAL, "set_fast_sweep: num_tries above 64 flips no spin");
    mc->fast_sweep_tries = std::max(1u, num_tries);
    return RBMG_OK;
}

extern "C" int rbmg_mc_acceptance(const rbmg_ensemble* mc, uint64_t* accepts, uint64_t* proposals,
                                  uint64_t* per_chain) {
    if (!mc || mc->kind != 0) return fail(RBMG_EINVAL, "acceptance: not a MonteCarloLoop");
    uint64_t a = 0, p = 0;
    for (size_t c = 0; c < mc->last_accepts.size(); c++) {
        a += mc->last_accepts[c];
        p += mc->last_proposals[c];
        if (per_chain) per_chain[c] = mc->last_accepts[c];
    }
    if (accepts) *accepts = a;
    if (proposals) *proposals = p;
    return RBMG_OK;
}

extern "C" int rbmg_exact_create(uint32_t num_spins, rbmg_ensemble** out) {
    if (!out || num_spins == 0 || num_spins > 30) return fail(RBMG_EINVAL, "ExactSummation: 1 <= N <= 30");
    auto e = std::make_unique<rbmg_ensemble>();
    e->kind = 1;
    e->num_spins = num_spins;
    *out = e.release();
    return RBMG_OK;
}

extern "C" int rbmg_exact_set_total_z_symmetry(rbmg_ensemble* ex, int sector) {
    if (!ex || ex->kind != 1) return fail(RBMG_EINVAL, "set_total_z_symmetry: not an ExactSummation");
    // source/spin_ensembles/ExactSummation.cu:26-45
    ex->allowed.clear();
    const uint64_t dim = 1ull << ex->num_spins;
    for (uint64_t x = 0; x < dim; x++) {
        const int tz = 2 * __builtin_popcountll(x) - static_cast<int>(ex->num_spins);
        if (tz == sector) ex->allowed.push_back(x);
    }
    ex->exact_total_z = 1;
    RBMG_CK(ex->d_allowed.ensure(sizeof(uint64_t) * std::max<size_t>(1, ex->allowed.size())));
    if (!ex->allowed.empty())
        RBMG_CK(cudaMemcpy(ex->d_allowed.p, ex->allowed.data(), sizeof(uint64_t) * ex->allowed.size(),
                           cudaMemcpyHostToDevice));
    return RBMG_OK;
}

// A fixed set of configurations visited with equal weights 1 / count: the samples of an
// earlier MonteCarloLoop pass (rbmg_ensemble_samples) evaluated again, e.g. the gradient
// of the energy an earlier call estimated, on the same configurations.
extern "C" int rbmg_samples_create(uint32_t num_spins, uint32_t count, const uint64_t* spins, rbmg_ensemble** out) {
    if (!out || !spins || count == 0 || num_spins == 0 || num_spins > 256)
        return fail(RBMG_EINVAL, "fixed samples: need 1 <= N <= 256 and at least one configuration");
    const int nw = nwords_of(static_cast<int>(num_spins));
    const size_t n = static_cast<size_t>(count) * nw;
    if (num_spins % 64)
        for (uint32_t t = 0; t < count; t++)
            if (spins[static_cast<size_t>(t) * nw + nw - 1] >> (num_spins % 64))
                return fail(RBMG_EINVAL, "fixed samples: a configuration sets a bit at or beyond N");
    auto e = std::make_unique<rbmg_ensemble>();
    e->kind = 2;
    e->num_spins = num_spins;
    e->spins_words = nw;
    e->fixed_count = count;
    RBMG_CK(e->d_allowed.ensure(sizeof(uint64_t) * n));
    RBMG_CK(cudaMemcpy(e->d_allowed.p, spins, sizeof(uint64_t) * n, cudaMemcpyHostToDevice));
    *out = e.release();
    return RBMG_OK;
}

extern "C" int rbmg_ensemble_num_steps(const rbmg_ensemble* ens, uint64_t* n) {
    if (!ens || !n) return fail(RBMG_EINVAL, "num_steps: null");
    *n = ens->num_steps();
    return RBMG_OK;
}

extern "C" int rbmg_ensemble_destroy(rbmg_ensemble* ens) {
    delete ens;
    return RBMG_OK;
}

// ====================================================================== sample streams
static int rbm_upload64(const rbmg_psi* p);
static Rbm64 rbm64(const rbmg_psi* p);

namespace rbmg {

// One chunk of samples: spins on the device (or basis indices when enumerate),
// per-sample weights (null = equal weights) and, for MC, the sampler's log psi / E_loc.
struct Chunk {
    int count = 0;
    const uint64_t* spins = nullptr;
    int enumerate = 0;
    uint64_t enum_base = 0;
    const double* weights = nullptr;
    const double2* eloc = nullptr;      // filled by the sampler when requested
};

struct StreamResult {
    double norm_factor = 1.0;   // reference weight scale: sum_s prefactor^2 |psi|^2 (exact) or 1/num_samples (MC)
    double log_norm = 0.0;      // log of sum_s prefactor^2 |psi|^2 (exact)
};

// FP64 log psi of a batch of configurations (exact-summation weights, psi vector,
// log_psi queries): the rational activation cancels to ~1e-7 absolute near theta = 0 in
// FP32, a bias that would shift the normalisation sum by ~1e-6 relative.
static int psi_log_psi_dev(const rbmg_psi* psi, int count, const uint64_t* d_spins, uint64_t enum_base,
                           int enumerate, double2* d_out) {
    if (psi->kind == 0) {
        const int r = ::rbm_upload64(psi);
        if (r != RBMG_OK) return r;
        Hsd64Launch L{};
        L.count = count;
        L.enum_base = enum_base;
        L.enumerate = enumerate;
        L.spins = d_spins;
        L.logpsi = d_out;
        OpDev none{};
        Rbm64 nopp{};
        nopp.N = psi->N;
        nopp.M = psi->M;
        RBMG_CK(launch_rbm_hsd64(::rbm64(psi), nopp, none, L, stream()));
        return RBMG_OK;
    }
    return deep_log_psi(psi, count, d_spins, enum_base, enumerate, d_out, stream());
}

constexpr int kExactChunk = 1 << 16;

// MonteCarloLoop::foreach (include/spin_ensembles/MonteCarloLoop.hpp:294-339): every call
// re-draws the start configurations and thermalises; the chains' Philox streams continue.
static int mc_stream(rbmg_ensemble* e, const rbmg_psi* psi, const rbmg_operator* op, bool want_eloc,
                     size_t max_chunk_samples, const std::function<int(const Chunk&)>& fn) {
    if (psi->kind != 0) return fail(RBMG_EUNSUPPORTED, "MonteCarloLoop: PsiDeep / PsiPair chains are sampled by deep.cu");
    if (e->fast_sweep_tries && e->total_z)
        return fail(RBMG_EUNSUPPORTED, "fast sweep with total_z symmetry (the reference pairs a mask with an unset site)");
    if (e->total_z && psi->N > 64) return fail(RBMG_EUNSUPPORTED, "total_z symmetry needs N <= 64");
    const int nw = nwords_of(psi->N);
    const int B = static_cast<int>(e->num_chains);
    const int steps = static_cast<int>(e->num_samples / e->num_chains);
    RBMG_CK(e->spins.ensure(sizeof(uint64_t) * nw * B));
    e->spins_words = nw;
    RBMG_CK(cudaMemsetAsync(e->accepts.p, 0, sizeof(unsigned long long) * B, stream()));
    RBMG_CK(cudaMemsetAsync(e->proposals.p, 0, sizeof(unsigned long long) * B, stream()));
    Workspace& W = ws();
    const int rows_per_chunk = static_cast<int>(std::max<size_t>(1, std::min<size_t>(steps, max_chunk_samples / B)));
    RBMG_CK(W.sample_spins.ensure(sizeof(uint64_t) * nw * B * rows_per_chunk));
    if (want_eloc) RBMG_CK(W.eloc.ensure(sizeof(double2) * B * rows_per_chunk));
    OpDev od;
    if (op) od = op->dev();
    bool first = true;
    for (int row0 = 0; row0 < steps; row0 += rows_per_chunk) {
        const int rows = std::min(rows_per_chunk, steps - row0);
        McLaunch L{};
        L.B = B;
        L.walker_base = 0;
        L.seed = e->seed;
        L.spins = e->spins.as<uint64_t>();
        L.rng_index = e->rng_index.as<uint64_t>();
        L.init = first ? 1 : 0;
        L.total_z = e->total_z;
        L.sector = e->sector;
        L.fast_tries = static_cast<int>(e->fast_sweep_tries);
        L.n_therm = first ? static_cast<int>(e->num_therm) : 0;
        L.n_samples = rows;
        L.sweeps_per_sample = static_cast<int>(e->num_sweeps);
        L.sample_base = 0;
        L.sample_spins = W.sample_spins.as<uint64_t>();
        L.accepts = e->accepts.as<unsigned long long>();
        L.proposals = e->proposals.as<unsigned long long>();
        RBMG_CK(launch_rbm_mc(psi->rbm_dev(), nullptr, L, stream()));
        first = false;
        Chunk c;
        c.count = rows * B;
        c.spins = W.sample_spins.as<uint64_t>();
        if (want_eloc && op) {
            EstLaunch E{};
            E.count = c.count;
            E.spins = c.spins;
            E.flags = EST_ELOC;
            E.eloc = W.eloc.as<double2>();
            RBMG_CK(launch_rbm_estimate(psi->rbm_dev(), &od, nullptr, E, stream()));
            c.eloc = W.eloc.as<double2>();
        }
        const int r = fn(c);
        if (r != RBMG_OK) return r;
    }
    std::vector<unsigned long long> a(B), p(B);
    RBMG_CK(cudaMemcpyAsync(a.data(), e->accepts.p, sizeof(unsigned long long) * B, cudaMemcpyDeviceToHost, stream()));
    RBMG_CK(cudaMemcpyAsync(p.data(), e->proposals.p, sizeof(unsigned long long) * B, cudaMemcpyDeviceToHost, stream()));
    RBMG_CK(cudaStreamSynchronize(stream()));
    e->last_accepts.assign(a.begin(), a.end());
    e->last_proposals.assign(p.begin(), p.end());
    return RBMG_OK;
}

// ExactSummation::foreach (include/spin_ensembles/ExactSummation.hpp:36-84): weights
// prefactor^2 |psi(s)|^2, computed as w_s = exp(2 Re log psi_s - L) (L = FP64
// log-sum-exp over the basis) times the returned norm factor exp(2 log prefactor + L).
static int exact_stream(rbmg_ensemble* e, const rbmg_psi* psi, StreamResult* res,
                        const std::function<int(const Chunk&)>& fn) {
    if (static_cast<int>(e->num_spins) != psi->N) return fail(RBMG_EINVAL, "ExactSummation: N does not match psi");
    const uint64_t total = e->num_steps();
    if (total == 0) return fail(RBMG_EINVAL, "ExactSummation: empty sector");
    Workspace& W = ws();
    RBMG_CK(W.logpsi.ensure(sizeof(double2) * total));
    RBMG_CK(W.weights.ensure(sizeof(double) * total));
    const int enumerate = e->exact_total_z ? 0 : 1;
    const uint64_t* sp = e->exact_total_z ? e->d_allowed.as<uint64_t>() : nullptr;
    for (uint64_t base = 0; base < total; base += kExactChunk) {
        const int cnt = static_cast<int>(std::min<uint64_t>(kExactChunk, total - base));
        const int r = psi_log_psi_dev(psi, cnt, sp ? sp + base : nullptr, base, enumerate,
                                      W.logpsi.as<double2>() + base);
        if (r != RBMG_OK) return r;
    }
    // FP64 log-sum-exp of 2 Re log psi
    RBMG_CK(W.block_max.ensure(sizeof(double) * kSumBlocks));
    int blocks = 0;
    RBMG_CK(launch_max_re2(static_cast<int>(total), W.logpsi.as<double2>(), W.block_max.as<double>(), &blocks, stream()));
    std::vector<double> bm(blocks);
    RBMG_CK(cudaMemcpyAsync(bm.data(), W.block_max.p, sizeof(double) * blocks, cudaMemcpyDeviceToHost, stream()));
    RBMG_CK(cudaStreamSynchronize(stream()));
    const double mx = *std::max_element(bm.begin(), bm.end());
    if (!std::isfinite(mx)) return fail(RBMG_ENAN, "ExactSummation: non-finite log psi");
    RBMG_CK(launch_exp_weights(static_cast<int>(total), W.logpsi.as<double2>(), mx, W.weights.as<double>(), stream()));
    RBMG_CK(W.block_scratch.ensure(sizeof(double2) * kSumBlocks * kMaxSeries));
    RBMG_CK(W.zsum.ensure(sizeof(double2) * kMaxSeries));
    RBMG_CK(cudaMemsetAsync(W.zsum.p, 0, sizeof(double2) * kMaxSeries, stream()));
    // sum of the weights (its own accumulator: the caller's sums are already armed)
    RBMG_CK(W.coef1.ensure(sizeof(double2) * total));
    RBMG_CK(launch_coef(static_cast<int>(total), W.weights.as<double>(), nullptr, 1.0, W.coef1.as<double2>(), stream()));
    SeriesSet set{};
    set.n = 1;
    set.v[0] = W.coef1.as<double2>();
    RBMG_CK(launch_weighted_sums(static_cast<int>(total), nullptr, set, W.block_scratch.as<double2>(),
                                 W.zsum.as<double2>(), stream()));
    double2 z;
    RBMG_CK(cudaMemcpyAsync(&z, W.zsum.p, sizeof(double2), cudaMemcpyDeviceToHost, stream()));
    RBMG_CK(cudaStreamSynchronize(stream()));
    const double logZ = mx + std::log(z.x);
    // normalised weights w_s = |psi_s|^2 / Z
    RBMG_CK(launch_exp_weights(static_cast<int>(total), W.logpsi.as<double2>(), logZ, W.weights.as<double>(), stream()));
    res->log_norm = 2.0 * std::log(psi->prefactor) + logZ;
    res->norm_factor = std::exp(res->log_norm);
    for (uint64_t base = 0; base < total; base += kExactChunk) {
        Chunk c;
        c.count = static_cast<int>(std::min<uint64_t>(kExactChunk, total - base));
        c.enumerate = enumerate;
        c.enum_base = base;
        c.spins = sp ? sp + base : nullptr;
        c.weights = W.weights.as<double>() + base;
        const int r = fn(c);
        if (r != RBMG_OK) return r;
    }
    return RBMG_OK;
}

}  // namespace rbmg

extern "C" int rbmg_psi_norm(const rbmg_psi* psi, rbmg_ensemble* ex, double* norm) {
    if (!psi || !ex || !norm) return fail(RBMG_EINVAL, "norm: null");
    if (ex->kind != 1) return fail(RBMG_EINVAL, "norm: needs an ExactSummation");
    StreamResult res;
    const int r = exact_stream(ex, psi, &res, [](const Chunk&) { return RBMG_OK; });
    if (r != RBMG_OK) return r;
    *norm = std::exp(0.5 * res.log_norm);
    return RBMG_OK;
}

extern "C" int rbmg_psi_log_psi(const rbmg_psi* psi, int count, const uint64_t* spins, double* out) {
    if (!psi || count < 0 || (count > 0 && (!spins || !out))) return fail(RBMG_EINVAL, "log_psi: bad arguments");
    if (count == 0) return RBMG_OK;
    const int nw = nwords_of(psi->N);
    Workspace& W = ws();
    RBMG_CK(W.sample_spins.ensure(sizeof(uint64_t) * nw * count));
    RBMG_CK(W.logpsi_p.ensure(sizeof(double2) * count));
    RBMG_CK(cudaMemcpyAsync(W.sample_spins.p, spins, sizeof(uint64_t) * nw * count, cudaMemcpyHostToDevice, stream()));
    const int r = psi_log_psi_dev(psi, count, W.sample_spins.as<uint64_t>(), 0, 0, W.logpsi_p.as<double2>());
    if (r != RBMG_OK) return r;
    RBMG_CK(cudaMemcpyAsync(out, W.logpsi_p.p, sizeof(double2) * count, cudaMemcpyDeviceToHost, stream()));
    RBMG_CK(cudaStreamSynchronize(stream()));
    return RBMG_OK;
}

extern "C" int rbmg_psi_vector(const rbmg_psi* psi, double* out) {
    if (!psi || !out) return fail(RBMG_EINVAL, "vector: null");
    if (psi->N > 30) return fail(RBMG_EINVAL, "vector: N <= 30");
    const uint64_t dim = 1ull << psi->N;
    Workspace& W = ws();
    RBMG_CK(W.logpsi.ensure(sizeof(double2) * dim));
    for (uint64_t base = 0; base < dim; base += kExactChunk) {
        const int cnt = static_cast<int>(std::min<uint64_t>(kExactChunk, dim - base));
        const int r = psi_log_psi_dev(psi, cnt, nullptr, base, 1, W.logpsi.as<double2>() + base);
        if (r != RBMG_OK) return r;
    }
    std::vector<double2> lp(dim);
    RBMG_CK(cudaMemcpyAsync(lp.data(), W.logpsi.p, sizeof(double2) * dim, cudaMemcpyDeviceToHost, stream()));
    RBMG_CK(cudaStreamSynchronize(stream()));
    const double lpf = std::log(psi->prefactor);   // PsiVector.cu:23-39: exp(log prefactor + log psi)
    cplx* o = reinterpret_cast<cplx*>(out);
    for (uint64_t x = 0; x < dim; x++) o[x] = std::exp(cplx(lpf + lp[x].x, lp[x].y));
    return RBMG_OK;
}

// ====================================================================== estimators
namespace rbmg {

struct Sums {
    cplx E{0, 0};
    double E2 = 0.0;
};

int deep_gradient_chunk(const rbmg_psi* psi, const rbmg_operator* op, const Chunk& c, double2 e_shift,
                        double2* d_eloc, double2* acc_O, double2* acc_EO, double2* acc_Ek, double2* coef1,
                        double2* coef2, cudaStream_t st,
                        double2* acc_B = nullptr, double2* coef3 = nullptr);
int deep_eloc_chunk(const rbmg_psi* psi, const rbmg_operator* op, const Chunk& c, double2* d_eloc, cudaStream_t st);
int deep_stream(rbmg_ensemble* e, const rbmg_psi* psi, const rbmg_operator* op, bool want_eloc,
                size_t max_chunk_samples, const std::function<int(const Chunk&)>& fn);

// local energies of one chunk into W.eloc (unless the sampler already produced them)
static int chunk_eloc(const rbmg_psi* psi, const rbmg_operator* op, const Chunk& c, const double2** out) {
    if (c.eloc) {
        *out = c.eloc;
        return RBMG_OK;
    }
    Workspace& W = ws();
    RBMG_CK(W.eloc.ensure(sizeof(double2) * c.count));
    if (psi->kind != 0) {
        const int r = deep_eloc_chunk(psi, op, c, W.eloc.as<double2>(), stream());
        if (r != RBMG_OK) return r;
        *out = W.eloc.as<double2>();
        return RBMG_OK;
    }
    EstLaunch L{};
    L.count = c.count;
    L.enum_base = c.enum_base;
    L.spins = c.spins;
    L.flags = EST_ELOC | (c.enumerate ? EST_ENUMERATE : 0);
    L.eloc = W.eloc.as<double2>();
    const OpDev od = op->dev();
    RBMG_CK(launch_rbm_estimate(psi->rbm_dev(), &od, nullptr, L, stream()));
    *out = W.eloc.as<double2>();
    return RBMG_OK;
}

// weighted mean of a per-sample complex series over one chunk (sum w v / sum w)
static int chunk_mean(const Chunk& c, const double2* v, cplx* out) {
    Workspace& W = ws();
    RBMG_CK(W.coef3.ensure(sizeof(double2) * c.count));
    RBMG_CK(launch_coef(c.count, c.weights, nullptr, 1.0, W.coef3.as<double2>(), stream()));
    RBMG_CK(W.zsum.ensure(sizeof(double2) * kMaxSeries));
    RBMG_CK(W.block_scratch.ensure(sizeof(double2) * kSumBlocks * kMaxSeries));
    RBMG_CK(cudaMemsetAsync(W.zsum.p, 0, sizeof(double2) * kMaxSeries, stream()));
    SeriesSet set{};
    set.n = 2;
    set.v[0] = v;
    set.v[1] = W.coef3.as<double2>();   // the weights themselves, summed with unit weight below
    RBMG_CK(launch_weighted_sums(c.count, c.weights, set, W.block_scratch.as<double2>(), W.zsum.as<double2>(),
                                 stream()));
    double2 m[2];
    RBMG_CK(cudaMemcpyAsync(m, W.zsum.p, sizeof(m), cudaMemcpyDeviceToHost, stream()));
    RBMG_CK(cudaStreamSynchronize(stream()));
    // m[1] = sum w * w when weighted; the weight total needs the plain sum: recompute it
    double wtot = static_cast<double>(c.count);
    if (c.weights) {
        SeriesSet s1{};
        s1.n = 1;
        s1.v[0] = W.coef3.as<double2>();
        RBMG_CK(cudaMemsetAsync(W.zsum.p, 0, sizeof(double2) * kMaxSeries, stream()));
        RBMG_CK(launch_weighted_sums(c.count, nullptr, s1, W.block_scratch.as<double2>(), W.zsum.as<double2>(),
                                     stream()));
        double2 t;
        RBMG_CK(cudaMemcpyAsync(&t, W.zsum.p, sizeof(t), cudaMemcpyDeviceToHost, stream()));
        RBMG_CK(cudaStreamSynchronize(stream()));
        wtot = t.x;
    }
    *out = wtot > 0.0 ? cplx(m[0].x, m[0].y) / wtot : cplx(0.0, 0.0);
    return RBMG_OK;
}

// the configurations of a fixed sample set, equal weights
static int fixed_stream(rbmg_ensemble* e, const rbmg_psi* psi, size_t max_chunk, StreamResult* res,
                        const std::function<int(const Chunk&)>& fn) {
    if (static_cast<int>(e->num_spins) != psi->N) return fail(RBMG_EINVAL, "fixed samples: N does not match psi");
    const uint64_t total = e->num_steps();
    res->norm_factor = 1.0 / static_cast<double>(total);
    const uint64_t per = std::max<uint64_t>(1, max_chunk);
    for (uint64_t base = 0; base < total; base += per) {
        Chunk c;
        c.count = static_cast<int>(std::min<uint64_t>(per, total - base));
        c.spins = e->d_allowed.as<uint64_t>() + base * e->spins_words;
        const int r = fn(c);
        if (r != RBMG_OK) return r;
    }
    return RBMG_OK;
}

static int run_stream(rbmg_ensemble* ens, const rbmg_psi* psi, const rbmg_operator* op, bool sampler_eloc,
                      size_t max_chunk, StreamResult* res, const std::function<int(const Chunk&)>& fn) {
    if (ens->kind == 1) return exact_stream(ens, psi, res, fn);
    if (ens->kind == 2) return fixed_stream(ens, psi, max_chunk, res, fn);
    res->norm_factor = 1.0 / static_cast<double>(ens->num_samples);
    if (psi->kind != 0) return deep_stream(ens, psi, op, sampler_eloc, max_chunk, fn);
    return mc_stream(ens, psi, op, sampler_eloc, max_chunk, fn);
}

// <E> and <|E|^2> with reference weights
static int energy_sums(const rbmg_psi* psi, const rbmg_operator* op, rbmg_ensemble* ens, Sums* out) {
    Workspace& W = ws();
    RBMG_CK(W.sums.ensure(sizeof(double2) * kMaxSeries));
    RBMG_CK(W.block_scratch.ensure(sizeof(double2) * kSumBlocks * kMaxSeries));
    RBMG_CK(cudaMemsetAsync(W.sums.p, 0, sizeof(double2) * kMaxSeries, stream()));
    StreamResult res;
    int r = run_stream(ens, psi, op, true, size_t(1) << 22, &res, [&](const Chunk& c) -> int {
        const double2* e = nullptr;
        int rr = chunk_eloc(psi, op, c, &e);
        if (rr != RBMG_OK) return rr;
        RBMG_CK(W.coef2.ensure(sizeof(double2) * c.count));
        RBMG_CK(launch_abs2(c.count, e, W.coef2.as<double2>(), stream()));
        SeriesSet set{};
        set.n = 2;
        set.v[0] = e;
        set.v[1] = W.coef2.as<double2>();
        RBMG_CK(launch_weighted_sums(c.count, c.weights, set, W.block_scratch.as<double2>(), W.sums.as<double2>(),
                                     stream()));
        return RBMG_OK;
    });
    if (r != RBMG_OK) return r;
    double2 s[2];
    RBMG_CK(cudaMemcpyAsync(s, W.sums.p, sizeof(s), cudaMemcpyDeviceToHost, stream()));
    RBMG_CK(cudaStreamSynchronize(stream()));
    out->E = cplx(s[0].x, s[0].y) * res.norm_factor;
    out->E2 = s[1].x * res.norm_factor;
    if (!std::isfinite(out->E.real()) || !std::isfinite(out->E.imag())) return fail(RBMG_ENAN, "non-finite energy");
    return RBMG_OK;
}

static int check_pair(const rbmg_psi* psi, const rbmg_operator* op, const rbmg_ensemble* ens) {
    if (!psi || !ens) return fail(RBMG_EINVAL, "null handle");
    if (op && op->max_site >= psi->N) return fail(RBMG_EINVAL, "operator acts on a site >= N");
    if (ens->kind == 1 && static_cast<int>(ens->num_spins) != psi->N)
        return fail(RBMG_EINVAL, "ExactSummation size does not match psi");
    if (ens->kind == 2 && static_cast<int>(ens->num_spins) != psi->N)
        return fail(RBMG_EINVAL, "fixed sample set: N does not match psi");
    return RBMG_OK;
}

}  // namespace rbmg

extern "C" int rbmg_ev_value(const rbmg_psi* psi, const rbmg_operator* op, rbmg_ensemble* ens, double* value) {
    if (!op || !value) return fail(RBMG_EINVAL, "ev: null");
    int r = check_pair(psi, op, ens);
    if (r != RBMG_OK) return r;
    Sums s;
    r = energy_sums(psi, op, ens, &s);
    if (r != RBMG_OK) return r;
    value[0] = s.E.real();
    value[1] = s.E.imag();
    return RBMG_OK;
}

namespace rbmg {
// device accumulators of `n` complex sums, zeroed
static int zero_sums(DevBuf& b, int n) {
    RBMG_CK(b.ensure(sizeof(double2) * std::max(1, n)));
    RBMG_CK(cudaMemsetAsync(b.p, 0, sizeof(double2) * std::max(1, n), stream()));
    return RBMG_OK;
}

// sums[0] += sum_s w[s] v[s]
static int add_sum(const Chunk& c, const double* w, const double2* v, double2* sum) {
    Workspace& W = ws();
    RBMG_CK(W.block_scratch.ensure(sizeof(double2) * kSumBlocks * kMaxSeries));
    SeriesSet set{};
    set.n = 1;
    set.v[0] = v;
    RBMG_CK(launch_weighted_sums(c.count, w, set, W.block_scratch.as<double2>(), sum, stream()));
    return RBMG_OK;
}
}  // namespace rbmg

// ExpectationValue::operator() of an operator list (ExpectationValue.cu:448-518): one pass
// over the ensemble, every operator's local energy on the same configurations.
extern "C" int rbmg_ev_values(const rbmg_psi* psi, const rbmg_operator* const* ops, int num_ops, rbmg_ensemble* ens,
                              double* values) {
    if (!ops || num_ops < 0 || (num_ops > 0 && !values)) return fail(RBMG_EINVAL, "ev list: bad arguments");
    if (num_ops == 0) return RBMG_OK;
    for (int q = 0; q < num_ops; q++) {
        if (!ops[q]) return fail(RBMG_EINVAL, "ev list: null operator");
        const int r = check_pair(psi, ops[q], ens);
        if (r != RBMG_OK) return r;
    }
    Workspace& W = ws();
    int r = zero_sums(W.lsums, num_ops);
    if (r != RBMG_OK) return r;
    StreamResult res;
    r = run_stream(ens, psi, nullptr, false, size_t(1) << 22, &res, [&](const Chunk& c) -> int {
        for (int q = 0; q < num_ops; q++) {
            const double2* e = nullptr;
            int rr = chunk_eloc(psi, ops[q], c, &e);
            if (rr == RBMG_OK) rr = add_sum(c, c.weights, e, W.lsums.as<double2>() + q);
            if (rr != RBMG_OK) return rr;
        }
        return RBMG_OK;
    });
    if (r != RBMG_OK) return r;
    std::vector<double2> h(num_ops);
    RBMG_CK(cudaMemcpyAsync(h.data(), W.lsums.p, sizeof(double2) * num_ops, cudaMemcpyDeviceToHost, stream()));
    RBMG_CK(cudaStreamSynchronize(stream()));
    for (int q = 0; q < num_ops; q++) {
        values[2 * q] = h[q].x * res.norm_factor;
        values[2 * q + 1] = h[q].y * res.norm_factor;
    }
    return RBMG_OK;
}

// ExpectationValue::difference (ExpectationValue.cu:350-446), Psi only (its instantiations):
// per operator <E'> - <r E> / <r> over psi's ensemble, E' the local energy under psi_prime,
// r = |psi / psi_prime|^2.
extern "C" int rbmg_ev_difference(const rbmg_psi* psi, const rbmg_psi* psi_prime, const rbmg_operator* const* ops,
                                  int num_ops, rbmg_ensemble* ens, double* values) {
    if (!psi || !psi_prime || !ops || num_ops < 0 || (num_ops > 0 && !values))
        return fail(RBMG_EINVAL, "difference: bad arguments");
    if (psi->kind != 0 || psi_prime->kind != 0)
        return fail(RBMG_EUNSUPPORTED, "difference: instantiated for Psi only (ExpectationValue.cu:529, 575)");
    if (psi_prime->N != psi->N || psi_prime->Mpad != psi->Mpad)
        return fail(RBMG_EUNSUPPORTED, "difference: psi_prime must have psi's N and padded M");
    if (num_ops == 0) return RBMG_OK;
    for (int q = 0; q < num_ops; q++) {
        if (!ops[q]) return fail(RBMG_EINVAL, "difference: null operator");
        const int r = check_pair(psi, ops[q], ens);
        if (r != RBMG_OK) return r;
    }
    Workspace& W = ws();
    int r = zero_sums(W.lsums, 2 * num_ops + 1);
    if (r != RBMG_OK) return r;
    double2* sums = W.lsums.as<double2>();
    StreamResult res;
    r = run_stream(ens, psi, nullptr, false, size_t(1) << 22, &res, [&](const Chunk& c) -> int {
        RBMG_CK(W.logpsi.ensure(sizeof(double2) * c.count));
        RBMG_CK(W.logpsi_p.ensure(sizeof(double2) * c.count));
        RBMG_CK(W.rw.ensure(sizeof(double) * c.count));
        RBMG_CK(W.rwc.ensure(sizeof(double2) * c.count));
        EstLaunch L{};
        L.count = c.count;
        L.enum_base = c.enum_base;
        L.spins = c.spins;
        L.flags = EST_LOGPSI | EST_PRIME | (c.enumerate ? EST_ENUMERATE : 0);
        L.logpsi = W.logpsi.as<double2>();
        L.logpsi_prime = W.logpsi_p.as<double2>();
        const RbmDev d = psi->rbm_dev(), dp = psi_prime->rbm_dev();
        RBMG_CK(launch_rbm_estimate(d, nullptr, &dp, L, stream()));
        RBMG_CK(launch_ratio_weights(c.count, c.weights, W.logpsi.as<double2>(), W.logpsi_p.as<double2>(),
                                     W.rw.as<double>(), W.rwc.as<double2>(), stream()));
        int rr = add_sum(c, nullptr, W.rwc.as<double2>(), sums + 2 * num_ops);
        for (int q = 0; q < num_ops && rr == RBMG_OK; q++) {
            const double2* e = nullptr;
            rr = chunk_eloc(psi, ops[q], c, &e);
            if (rr == RBMG_OK) rr = add_sum(c, W.rw.as<double>(), e, sums + num_ops + q);
            if (rr == RBMG_OK) rr = chunk_eloc(psi_prime, ops[q], c, &e);
            if (rr == RBMG_OK) rr = add_sum(c, c.weights, e, sums + q);
        }
        return rr;
    });
    if (r != RBMG_OK) return r;
    std::vector<double2> h(2 * num_ops + 1);
    RBMG_CK(cudaMemcpyAsync(h.data(), sums, sizeof(double2) * h.size(), cudaMemcpyDeviceToHost, stream()));
    RBMG_CK(cudaStreamSynchronize(stream()));
    const double f = res.norm_factor;
    const double p = h[2 * num_ops].x * f;
    for (int q = 0; q < num_ops; q++) {
        const cplx a = cplx(h[q].x, h[q].y) * f, b = cplx(h[num_ops + q].x, h[num_ops + q].y) * f;
        const cplx v = a - b / p;
        values[2 * q] = v.real();
        values[2 * q + 1] = v.imag();
    }
    return RBMG_OK;
}

// ExpectationValue::corrected (ExpectationValue.cu:76-127).  As in the reference the local
// energy is evaluated with the first operator twice (operator2 is accepted and not used):
// value = <E> / <a>, abs2 = <a>, a = exp(2 Im E + Re(E E - E)).
extern "C" int rbmg_ev_corrected(const rbmg_psi* psi, const rbmg_operator* op, const rbmg_operator* op2,
                                 rbmg_ensemble* ens, double* value, double* abs2) {
    if (!op || !op2 || !value || !abs2) return fail(RBMG_EINVAL, "corrected: null");
    int r = check_pair(psi, op, ens);
    if (r != RBMG_OK) return r;
    Workspace& W = ws();
    r = zero_sums(W.lsums, 2);
    if (r != RBMG_OK) return r;
    double2* sums = W.lsums.as<double2>();
    StreamResult res;
    r = run_stream(ens, psi, op, true, size_t(1) << 22, &res, [&](const Chunk& c) -> int {
        const double2* e = nullptr;
        int rr = chunk_eloc(psi, op, c, &e);
        if (rr != RBMG_OK) return rr;
        RBMG_CK(W.eabs2.ensure(sizeof(double2) * c.count));
        RBMG_CK(launch_corrected_terms(c.count, e, W.eabs2.as<double2>(), stream()));
        rr = add_sum(c, c.weights, e, sums);
        if (rr == RBMG_OK) rr = add_sum(c, c.weights, W.eabs2.as<double2>(), sums + 1);
        return rr;
    });
    if (r != RBMG_OK) return r;
    double2 h[2];
    RBMG_CK(cudaMemcpyAsync(h, sums, sizeof(h), cudaMemcpyDeviceToHost, stream()));
    RBMG_CK(cudaStreamSynchronize(stream()));
    const cplx A = cplx(h[0].x, h[0].y) * res.norm_factor;
    const double a = h[1].x * res.norm_factor;
    value[0] = (A / a).real();
    value[1] = (A / a).imag();
    *abs2 = a;
    return RBMG_OK;
}

extern "C" int rbmg_ev_fluctuation(const rbmg_psi* psi, const rbmg_operator* op, rbmg_ensemble* ens, double* sigma,
                                   double* value) {
    if (!op || !sigma || !value) return fail(RBMG_EINVAL, "fluctuation: null");
    int r = check_pair(psi, op, ens);
    if (r != RBMG_OK) return r;
    Sums s;
    r = energy_sums(psi, op, ens, &s);
    if (r != RBMG_OK) return r;
    *sigma = std::sqrt(s.E2 - std::norm(s.E));   // ExpectationValue.cu:171-174
    value[0] = s.E.real();
    value[1] = s.E.imag();
    return RBMG_OK;
}

// The gradient's sums, left on the device: acc_O = sum w O, acc_EO = sum w (E - E0) O*,
// acc_Ek = sum w (E_k - E0 O) over the O_k entries k >= 2N, sums[0] = sum w E; E0 (the
// first chunk's mean local energy) and the ensemble's normalisation factor come back.
// fluct: also B = sum w conj(E - E0) (E_k - E0 O_k) into acc_B and sum w |E|^2 into sums[1]
// (the further sums of ExpectationValue::fluctuation_gradient).  adjoint (complex RBM): also
// C2 = sum w (E - E0) O_k into acc_C2 and C3 = sum w (Re E - Re E0) conj(O_k) into acc_C3
// (the derivative of <E_loc>, rbmg_ev_eloc_gradient).
static int ev_gradient_sums(const rbmg_psi* psi, const rbmg_operator* op, rbmg_ensemble* ens, cplx* E0_out,
                            double* norm_out, bool fluct = false, bool adjoint = false) {
    int r = check_pair(psi, op, ens);
    if (r != RBMG_OK) return r;
    const int N = psi->N, P = psi->num_params();
    const int nw = nwords_of(N);
    Workspace& W = ws();
    const size_t ok_len = static_cast<size_t>(P - 2 * N);   // O_k entries the accumulators hold
    RBMG_CK(W.acc_O.ensure(sizeof(double2) * ok_len));
    RBMG_CK(W.acc_EO.ensure(sizeof(double2) * ok_len));
    RBMG_CK(W.acc_Ek.ensure(sizeof(double2) * ok_len));
    RBMG_CK(cudaMemsetAsync(W.acc_O.p, 0, sizeof(double2) * ok_len, stream()));
    RBMG_CK(cudaMemsetAsync(W.acc_EO.p, 0, sizeof(double2) * ok_len, stream()));
    RBMG_CK(cudaMemsetAsync(W.acc_Ek.p, 0, sizeof(double2) * ok_len, stream()));
    if (fluct) {
        RBMG_CK(W.acc_B.ensure(sizeof(double2) * ok_len));
        RBMG_CK(cudaMemsetAsync(W.acc_B.p, 0, sizeof(double2) * ok_len, stream()));
    }
    if (adjoint) {
        if (psi->kind != 0) return fail(RBMG_EUNSUPPORTED, "adjoint sums: complex RBM only");
        RBMG_CK(W.acc_C2.ensure(sizeof(double2) * ok_len));
        RBMG_CK(W.acc_C3.ensure(sizeof(double2) * ok_len));
        RBMG_CK(cudaMemsetAsync(W.acc_C2.p, 0, sizeof(double2) * ok_len, stream()));
        RBMG_CK(cudaMemsetAsync(W.acc_C3.p, 0, sizeof(double2) * ok_len, stream()));
    }
    RBMG_CK(W.sums.ensure(sizeof(double2) * kMaxSeries));
    RBMG_CK(W.block_scratch.ensure(sizeof(double2) * kSumBlocks * kMaxSeries));
    RBMG_CK(cudaMemsetAsync(W.sums.p, 0, sizeof(double2) * kMaxSeries, stream()));
    constexpr int kSplits = 64;
    size_t per_sample = 0;
    if (psi->kind == 0) {
        r = op_site_lists(const_cast<rbmg_operator*>(op), N);
        if (r != RBMG_OK) return r;
        per_sample = sizeof(float2) * psi->Mpad * (2 + op->num_offdiag) + 64;
        RBMG_CK(W.partial.ensure(sizeof(double2) * kSplits * (1 + N) * psi->M));
    }
    const size_t max_chunk = psi->kind == 0 ? std::max<size_t>(256, (size_t(512) << 20) / per_sample) : 4096;
    // The sums are centred on E0, the mean local energy of the first chunk:
    // EO' = sum w (E - E0) O*, Ek' = sum w (E_k - E0 O), so that FP32 partial sums keep
    // the small covariance the gradient is made of (see the formula below).
    cplx E0(0.0, 0.0);
    bool have_shift = false;
    StreamResult res;
    r = run_stream(ens, psi, op, false, max_chunk, &res, [&](const Chunk& c) -> int {
        RBMG_CK(W.eloc.ensure(sizeof(double2) * c.count));
        if (psi->kind != 0) {
            if (!have_shift) {
                const double2* e0 = nullptr;
                const int rr0 = chunk_eloc(psi, op, c, &e0);
                if (rr0 != RBMG_OK) return rr0;
                const int rr1 = chunk_mean(c, e0, &E0);
                if (rr1 != RBMG_OK) return rr1;
                have_shift = true;
            }
            RBMG_CK(W.coef1.ensure(sizeof(double2) * c.count));
            RBMG_CK(W.coef2.ensure(sizeof(double2) * c.count));
            if (fluct) RBMG_CK(W.coef3.ensure(sizeof(double2) * c.count));
            const int rr = deep_gradient_chunk(psi, op, c, make_double2(E0.real(), E0.imag()), W.eloc.as<double2>(),
                                               W.acc_O.as<double2>(), W.acc_EO.as<double2>(), W.acc_Ek.as<double2>(),
                                               W.coef1.as<double2>(), W.coef2.as<double2>(), stream(),
                                               fluct ? W.acc_B.as<double2>() : nullptr,
                                               fluct ? W.coef3.as<double2>() : nullptr);
            if (rr != RBMG_OK) return rr;
        } else {
            const OpDev od = op->dev();
            if (!have_shift) {
                const double2* e0 = nullptr;
                const int rr0 = chunk_eloc(psi, op, c, &e0);
                if (rr0 != RBMG_OK) return rr0;
                const int rr1 = chunk_mean(c, e0, &E0);
                if (rr1 != RBMG_OK) return rr1;
                have_shift = true;
            }
            RBMG_CK(W.T.ensure(sizeof(float2) * c.count * psi->Mpad));
            RBMG_CK(W.U.ensure(sizeof(float2) * c.count * psi->Mpad));
            RBMG_CK(W.X.ensure(sizeof(float2) * std::max<size_t>(1, size_t(c.count) * op->num_offdiag * psi->Mpad)));
            EstLaunch L{};
            L.count = c.count;
            L.enum_base = c.enum_base;
            L.spins = c.spins;
            L.flags = EST_ELOC | EST_GRADVEC | (c.enumerate ? EST_ENUMERATE : 0);
            L.eloc = W.eloc.as<double2>();
            L.T = W.T.as<float2>();
            L.U = W.U.as<float2>();
            L.X = W.X.as<float2>();
            L.e_shift = make_double2(E0.real(), E0.imag());
            RBMG_CK(launch_rbm_estimate(psi->rbm_dev(), &od, nullptr, L, stream()));
            RBMG_CK(W.coef1.ensure(sizeof(double2) * c.count));
            RBMG_CK(W.coef2.ensure(sizeof(double2) * c.count));
            RBMG_CK(launch_coef(c.count, c.weights, nullptr, 1.0, W.coef1.as<double2>(), stream()));
            RBMG_CK(launch_coef(c.count, c.weights, W.eloc.as<double2>(), 1.0, W.coef2.as<double2>(), stream(),
                                make_double2(E0.real(), E0.imag())));
            double2* part = W.partial.as<double2>();
            RBMG_CK(launch_outer_reduce(c.count, N, nw, psi->M, c.spins, c.enum_base, c.enumerate,
                                        W.coef1.as<double2>(), W.T.as<float2>(), psi->Mpad, 0,
                                        W.acc_O.as<double2>(), part, kSplits, stream()));
            RBMG_CK(launch_outer_reduce(c.count, N, nw, psi->M, c.spins, c.enum_base, c.enumerate,
                                        W.coef2.as<double2>(), W.T.as<float2>(), psi->Mpad, 1,
                                        W.acc_EO.as<double2>(), part, kSplits, stream()));
            RBMG_CK(launch_outer_reduce(c.count, N, nw, psi->M, c.spins, c.enum_base, c.enumerate,
                                        W.coef1.as<double2>(), W.U.as<float2>(), psi->Mpad, 0,
                                        W.acc_Ek.as<double2>(), part, kSplits, stream()));
            RBMG_CK(launch_vterm_reduce(c.count, N, nw, psi->M, psi->Mpad, c.spins, c.enum_base, c.enumerate,
                                        c.weights, W.X.as<float2>(), op->num_offdiag, op->d_site_ptr.as<int>(),
                                        op->d_site_slots.as<int>(), W.acc_Ek.as<double2>(), part, kSplits,
                                        stream()));
            if (adjoint) {
                RBMG_CK(launch_outer_reduce(c.count, N, nw, psi->M, c.spins, c.enum_base, c.enumerate,
                                            W.coef2.as<double2>(), W.T.as<float2>(), psi->Mpad, 0,
                                            W.acc_C2.as<double2>(), part, kSplits, stream()));
                RBMG_CK(W.coef3.ensure(sizeof(double2) * c.count));
                RBMG_CK(launch_coef_real(c.count, c.weights, W.eloc.as<double2>(), E0.real(), W.coef3.as<double2>(),
                                         stream()));
                RBMG_CK(launch_outer_reduce(c.count, N, nw, psi->M, c.spins, c.enum_base, c.enumerate,
                                            W.coef3.as<double2>(), W.T.as<float2>(), psi->Mpad, 1,
                                            W.acc_C3.as<double2>(), part, kSplits, stream()));
            }
            if (fluct) {
                RBMG_CK(W.coef3.ensure(sizeof(double2) * c.count));
                RBMG_CK(launch_coef_conj(c.count, c.weights, W.eloc.as<double2>(), make_double2(E0.real(), E0.imag()),
                                         W.coef3.as<double2>(), stream()));
                RBMG_CK(launch_outer_reduce(c.count, N, nw, psi->M, c.spins, c.enum_base, c.enumerate,
                                            W.coef3.as<double2>(), W.U.as<float2>(), psi->Mpad, 0,
                                            W.acc_B.as<double2>(), part, kSplits, stream()));
                RBMG_CK(launch_vterm_reduce(c.count, N, nw, psi->M, psi->Mpad, c.spins, c.enum_base, c.enumerate,
                                            nullptr, W.X.as<float2>(), op->num_offdiag, op->d_site_ptr.as<int>(),
                                            op->d_site_slots.as<int>(), W.acc_B.as<double2>(), part, kSplits,
                                            stream(), W.coef3.as<double2>()));
            }
        }
        SeriesSet set{};
        set.n = 1;
        set.v[0] = W.eloc.as<double2>();
        if (fluct) {
            RBMG_CK(W.eabs2.ensure(sizeof(double2) * c.count));
            RBMG_CK(launch_abs2(c.count, W.eloc.as<double2>(), W.eabs2.as<double2>(), stream()));
            set.n = 2;
            set.v[1] = W.eabs2.as<double2>();
        }
        RBMG_CK(launch_weighted_sums(c.count, c.weights, set, W.block_scratch.as<double2>(), W.sums.as<double2>(),
                                     stream()));
        return RBMG_OK;
    });
    if (r != RBMG_OK) return r;
    *E0_out = E0;
    *norm_out = res.norm_factor;
    return RBMG_OK;
}

extern "C" int rbmg_ev_gradient(const rbmg_psi* psi, const rbmg_operator* op, rbmg_ensemble* ens, double* grad,
                                double* value) {
    if (!op || !grad || !value) return fail(RBMG_EINVAL, "gradient: null");
    cplx E0;
    double f = 0.0;
    int r = ev_gradient_sums(psi, op, ens, &E0, &f);
    if (r != RBMG_OK) return r;
    const int N = psi->N;
    const size_t ok_len = static_cast<size_t>(psi->num_params() - 2 * N);
    Workspace& W = ws();
    std::vector<double2> O(ok_len), EO(ok_len), Ek(ok_len);
    double2 Es;
    RBMG_CK(cudaMemcpyAsync(O.data(), W.acc_O.p, sizeof(double2) * ok_len, cudaMemcpyDeviceToHost, stream()));
    RBMG_CK(cudaMemcpyAsync(EO.data(), W.acc_EO.p, sizeof(double2) * ok_len, cudaMemcpyDeviceToHost, stream()));
    RBMG_CK(cudaMemcpyAsync(Ek.data(), W.acc_Ek.p, sizeof(double2) * ok_len, cudaMemcpyDeviceToHost, stream()));
    RBMG_CK(cudaMemcpyAsync(&Es, W.sums.p, sizeof(double2), cudaMemcpyDeviceToHost, stream()));
    RBMG_CK(cudaStreamSynchronize(stream()));
    // ExpectationValue.cu:243-253: grad = <E O*> + conj<E_k> - 2 <E> <O*>.  With the centred
    // sums <E O*> = EO' + E0 conj<O> and <E_k> = Ek' + E0 <O>, so
    // grad = EO' + conj(Ek') + (E0 + conj(E0) - 2 <E>) conj<O>.
    const cplx E = cplx(Es.x, Es.y) * f;
    const cplx shift_sum = E0 + std::conj(E0) - 2.0 * E;
    cplx* g = reinterpret_cast<cplx*>(grad);
    for (int k = 0; k < 2 * N; k++) g[k] = 0.0;
    for (size_t k = 0; k < ok_len; k++) {
        const cplx o = cplx(O[k].x, O[k].y) * f, eo = cplx(EO[k].x, EO[k].y) * f, ek = cplx(Ek[k].x, Ek[k].y) * f;
        g[2 * N + k] = eo + std::conj(ek) + shift_sum * std::conj(o);
    }
    value[0] = E.real();
    value[1] = E.imag();
    return RBMG_OK;
}

// ExpectationValue::fluctuation_gradient (ExpectationValue.cu:258-348): the gradient of
// sigma = sqrt(<|E|^2> - |<E>|^2),
//   1 / (2 sigma) (2 conj(<E* E_k> - <E>* <E_k>) - 2 <E>* <E O_k*> + 2 <O_k>* (2 |<E>|^2 - <|E|^2>)),
// formed from sums centred on E0 (the first chunk's mean local energy):
//   <E* E_k> - <E>* <E_k> = B + E0 conj(EO') - conj(<E> - E0) <E_k>,  <E_k> = Ek' + E0 <O>,
//   -2 <E>* <E O*> + 2 <O>* (2 |<E>|^2 - <|E|^2>) = -2 <E>* EO' + 2 <O>* (<E>* (<E> - E0) - sigma^2),
// with EO' = <(E - E0) O*>, Ek' = <E_k - E0 O>, B = <(E - E0)* (E_k - E0 O)>.
extern "C" int rbmg_ev_fluctuation_gradient(const rbmg_psi* psi, const rbmg_operator* op, rbmg_ensemble* ens,
                                            double* grad, double* sigma) {
    if (!op || !grad) return fail(RBMG_EINVAL, "fluctuation_gradient: null");
    cplx E0;
    double f = 0.0;
    int r = ev_gradient_sums(psi, op, ens, &E0, &f, true);
    if (r != RBMG_OK) return r;
    const int N = psi->N;
    const size_t ok_len = static_cast<size_t>(psi->num_params() - 2 * N);
    Workspace& W = ws();
    std::vector<double2> O(ok_len), EO(ok_len), Ek(ok_len), B(ok_len);
    double2 Es[2];
    RBMG_CK(cudaMemcpyAsync(O.data(), W.acc_O.p, sizeof(double2) * ok_len, cudaMemcpyDeviceToHost, stream()));
    RBMG_CK(cudaMemcpyAsync(EO.data(), W.acc_EO.p, sizeof(double2) * ok_len, cudaMemcpyDeviceToHost, stream()));
    RBMG_CK(cudaMemcpyAsync(Ek.data(), W.acc_Ek.p, sizeof(double2) * ok_len, cudaMemcpyDeviceToHost, stream()));
    RBMG_CK(cudaMemcpyAsync(B.data(), W.acc_B.p, sizeof(double2) * ok_len, cudaMemcpyDeviceToHost, stream()));
    RBMG_CK(cudaMemcpyAsync(Es, W.sums.p, sizeof(Es), cudaMemcpyDeviceToHost, stream()));
    RBMG_CK(cudaStreamSynchronize(stream()));
    const cplx E = cplx(Es[0].x, Es[0].y) * f;
    const double E2 = Es[1].x * f;
    const double var = std::max(0.0, E2 - std::norm(E));
    const double sig = std::sqrt(var);
    cplx* g = reinterpret_cast<cplx*>(grad);
    for (int k = 0; k < 2 * N; k++) g[k] = 0.0;
    const cplx de = E - E0;
    for (size_t k = 0; k < ok_len; k++) {
        const cplx o = cplx(O[k].x, O[k].y) * f, eo = cplx(EO[k].x, EO[k].y) * f;
        const cplx ek = cplx(Ek[k].x, Ek[k].y) * f, b = cplx(B[k].x, B[k].y) * f;
        const cplx eka = ek + E0 * o;
        const cplx t1 = 2.0 * std::conj(b + E0 * std::conj(eo) - std::conj(de) * eka);
        const cplx t23 = -2.0 * std::conj(E) * eo + 2.0 * std::conj(o) * (std::conj(E) * de - var);
        g[2 * N + k] = (t1 + t23) / (2.0 * sig);
    }
    if (sigma) *sigma = sig;
    return RBMG_OK;
}

// The same gradient left on the device: d_grad [P] complex128 (entries below 2N zero),
// formed by launch_grad_final from the sums above; the energy comes back to the host.
int rbmg::ev_gradient_device(const rbmg_psi* psi, const rbmg_operator* op, rbmg_ensemble* ens, double2* d_grad,
                       double* value) {
    if (!op || !d_grad || !value) return fail(RBMG_EINVAL, "gradient: null");
    cplx E0;
    double f = 0.0;
    int r = ev_gradient_sums(psi, op, ens, &E0, &f);
    if (r != RBMG_OK) return r;
    Workspace& W = ws();
    const int N = psi->N;
    const long ok_len = psi->num_params() - 2 * N;
    RBMG_CK(launch_grad_final(W.acc_O.as<double2>(), W.acc_EO.as<double2>(), W.acc_Ek.as<double2>(),
                              W.sums.as<double2>(), f, make_double2(E0.real(), E0.imag()), 2 * N, ok_len, d_grad,
                              stream()));
    double2 Es;
    RBMG_CK(cudaMemcpyAsync(&Es, W.sums.p, sizeof(double2), cudaMemcpyDeviceToHost, stream()));
    RBMG_CK(cudaStreamSynchronize(stream()));
    value[0] = Es.x * f;
    value[1] = Es.y * f;
    return RBMG_OK;
}

// Extension: the hidden angles theta = b + s W of given configurations (spins
// [count][ceil(N/64)]) -> out [2 count M] (complex), from the tensor-core kernel
// (reference: kernel::Psi::angle, include/quantum_state/Psi.hpp:43-53, one angle at a time)
extern "C" int rbmg_psi_angles(const rbmg_psi* psi, int count, const uint64_t* spins, double* out) {
    if (!psi || count < 0 || (count > 0 && (!spins || !out))) return fail(RBMG_EINVAL, "angles: bad arguments");
    if (psi->kind != 0) return fail(RBMG_EUNSUPPORTED, "angles: complex RBM (Psi) only");
    if (!psi->dWtc.p) return fail(RBMG_EUNSUPPORTED, "angles: no tensor-core operands for this psi");
    if (count == 0) return RBMG_OK;
    const int nw = nwords_of(psi->N);
    Workspace& W = ws();
    RBMG_CK(W.sample_spins.ensure(sizeof(uint64_t) * nw * count));
    RBMG_CK(W.Tp.ensure(sizeof(float2) * static_cast<size_t>(count) * psi->Mpad));
    RBMG_CK(cudaMemcpyAsync(W.sample_spins.p, spins, sizeof(uint64_t) * nw * count, cudaMemcpyHostToDevice, stream()));
    RBMG_CK(launch_angles_tc(count, psi->N, psi->Mpad, W.sample_spins.as<uint64_t>(), psi->db.as<float2>(),
                             psi->dWtc.as<__nv_bfloat16>(), nullptr, nullptr, W.Tp.as<float2>(),
                             psi->tc_error.as<int>(), stream()));
    std::vector<float2> h(static_cast<size_t>(count) * psi->Mpad);
    int err = 0;
    RBMG_CK(cudaMemcpyAsync(h.data(), W.Tp.p, sizeof(float2) * h.size(), cudaMemcpyDeviceToHost, stream()));
    RBMG_CK(cudaMemcpyAsync(&err, psi->tc_error.p, sizeof(int), cudaMemcpyDeviceToHost, stream()));
    RBMG_CK(cudaStreamSynchronize(stream()));
    if (err) {
        RBMG_CK(cudaMemset(psi->tc_error.p, 0, sizeof(int)));
        return fail(RBMG_ETIMEOUT, "angles: a tensor-core wait gave up");
    }
    for (int t = 0; t < count; t++)
        for (int j = 0; j < psi->M; j++) {
            const float2 v = h[static_cast<size_t>(t) * psi->Mpad + j];
            out[2 * (static_cast<size_t>(t) * psi->M + j)] = v.x;
            out[2 * (static_cast<size_t>(t) * psi->M + j) + 1] = v.y;
        }
    return RBMG_OK;
}

// local energies of given configurations (extension: the reference evaluates them only
// inside its ensembles' foreach, Operator.hpp:90-115); FP64 estimator path for PsiDeep
extern "C" int rbmg_local_energies(const rbmg_psi* psi, const rbmg_operator* op, int count, const uint64_t* spins,
                                   double* out) {
    if (!psi || !op || count < 0 || (count > 0 && (!spins || !out))) return fail(RBMG_EINVAL, "local energies: bad arguments");
    if (op->max_site >= psi->N) return fail(RBMG_EINVAL, "local energies: operator acts on a site >= N");
    if (count == 0) return RBMG_OK;
    const int nw = nwords_of(psi->N);
    Workspace& W = ws();
    RBMG_CK(W.sample_spins.ensure(sizeof(uint64_t) * nw * count));
    RBMG_CK(cudaMemcpyAsync(W.sample_spins.p, spins, sizeof(uint64_t) * nw * count, cudaMemcpyHostToDevice, stream()));
    Chunk c;
    c.count = count;
    c.spins = W.sample_spins.as<uint64_t>();
    const double2* e = nullptr;
    const int r = chunk_eloc(psi, op, c, &e);
    if (r != RBMG_OK) return r;
    RBMG_CK(cudaMemcpyAsync(out, e, sizeof(double2) * count, cudaMemcpyDeviceToHost, stream()));
    RBMG_CK(cudaStreamSynchronize(stream()));
    return RBMG_OK;
}

// ====================================================================== adjoint
namespace rbmg {
int deep_adjoint_chunk(const rbmg_psi* psi, const rbmg_operator* op, const Chunk& c, int score, double2* d_eloc,
                       double2* G, double2* GO, const std::vector<size_t>& goff, cudaStream_t st);
}  // namespace rbmg

// Gradient of the local energy by the adjoint kernel (extension, PsiDeep): in PyTorch's
// convention for a real loss, grad_k = dL/dRe(theta_k) + i dL/dIm(theta_k), with
//   score = 0: L = Re <E_loc> over the ensemble's samples held fixed, i.e.
//              grad = conj(<sum_n e_n O(s'_n) - E_loc O(s)>);
//   score = 1: L = <H>, adding the sampling term 2 <(Re E_loc - <Re E>) O*>, so that
//              grad equals the reference's estimator (ExpectationValue.cu:243-253) except
//              at the final weights, whose derivative is the last layer's activation here
//              and activation * log psi there (PsiDeep.hpp:285-292).
// The complex RBM's derivative of <E_loc> in PyTorch's convention (dL/dRe + i dL/dIm of
// L = Re <E_loc>).  E_loc(s) is holomorphic in the parameters with
// dE_loc(s)/dtheta_k = E_k(s) - E_loc(s) O_k(s) (E_k the estimator vector of
// Operator.hpp:145-179), so the fixed-sample part is conj(<E_k - E O_k>) = conj(C1 - C2)
// (C1 = <E_k - E0 O_k>, C2 = <(E - E0) O_k>); the sampling term (score) adds
// 2 <(Re E - <Re E>) O_k*> = 2 (C3 - (<Re E> - Re E0) <O_k>*).
static int rbm_eloc_gradient(const rbmg_psi* psi, const rbmg_operator* op, rbmg_ensemble* ens, int score,
                             double* grad, double* value) {
    cplx E0;
    double f = 0.0;
    int r = ev_gradient_sums(psi, op, ens, &E0, &f, false, true);
    if (r != RBMG_OK) return r;
    const int N = psi->N;
    const size_t ok_len = static_cast<size_t>(psi->num_params() - 2 * N);
    Workspace& W = ws();
    std::vector<double2> O(ok_len), C1(ok_len), C2(ok_len), C3(ok_len);
    double2 Es;
    RBMG_CK(cudaMemcpyAsync(O.data(), W.acc_O.p, sizeof(double2) * ok_len, cudaMemcpyDeviceToHost, stream()));
    RBMG_CK(cudaMemcpyAsync(C1.data(), W.acc_Ek.p, sizeof(double2) * ok_len, cudaMemcpyDeviceToHost, stream()));
    RBMG_CK(cudaMemcpyAsync(C2.data(), W.acc_C2.p, sizeof(double2) * ok_len, cudaMemcpyDeviceToHost, stream()));
    RBMG_CK(cudaMemcpyAsync(C3.data(), W.acc_C3.p, sizeof(double2) * ok_len, cudaMemcpyDeviceToHost, stream()));
    RBMG_CK(cudaMemcpyAsync(&Es, W.sums.p, sizeof(double2), cudaMemcpyDeviceToHost, stream()));
    RBMG_CK(cudaStreamSynchronize(stream()));
    const cplx E = cplx(Es.x, Es.y) * f;
    const double dre = E.real() - E0.real();
    cplx* g = reinterpret_cast<cplx*>(grad);
    for (int k = 0; k < 2 * N; k++) g[k] = 0.0;
    for (size_t k = 0; k < ok_len; k++) {
        const cplx c1 = cplx(C1[k].x, C1[k].y) * f, c2 = cplx(C2[k].x, C2[k].y) * f;
        cplx v = std::conj(c1 - c2);
        if (score) {
            const cplx o = cplx(O[k].x, O[k].y) * f, c3 = cplx(C3[k].x, C3[k].y) * f;
            v += 2.0 * (c3 - dre * std::conj(o));
        }
        g[2 * N + k] = v;
    }
    value[0] = E.real();
    value[1] = E.imag();
    return RBMG_OK;
}

extern "C" int rbmg_ev_eloc_gradient(const rbmg_psi* psi, const rbmg_operator* op, rbmg_ensemble* ens, int score,
                                     double* grad, double* value) {
    if (!op || !grad || !value) return fail(RBMG_EINVAL, "adjoint: null");
    int r = check_pair(psi, op, ens);
    if (r != RBMG_OK) return r;
    if (psi->kind == 0) return rbm_eloc_gradient(psi, op, ens, score, grad, value);
    if (psi->kind != 1) return fail(RBMG_EUNSUPPORTED, "adjoint: PsiDeep and Psi only");
    if (psi->translational_invariance) return fail(RBMG_EUNSUPPORTED, "adjoint: translational averaging not provided");
    const int N = psi->N, P = psi->num_params();
    const int L = static_cast<int>(psi->layers.size());
    std::vector<size_t> goff;
    size_t tot = 0;
    for (int l = 0; l < L; l++) {
        const int size = psi->layers[l].size, in = l == 0 ? N : psi->layers[l - 1].size;
        goff.push_back(tot);
        tot += static_cast<size_t>(size) * in;
        goff.push_back(tot);
        tot += size;
    }
    goff.push_back(tot);
    tot += psi->layers[L - 1].size;
    Workspace& W = ws();
    // G: sum over configurations of alpha delta (x) a; GO: sum over samples of w O(s)
    RBMG_CK(W.acc_O.ensure(sizeof(double2) * tot));
    RBMG_CK(W.acc_EO.ensure(sizeof(double2) * tot));
    RBMG_CK(cudaMemsetAsync(W.acc_O.p, 0, sizeof(double2) * tot, stream()));
    RBMG_CK(cudaMemsetAsync(W.acc_EO.p, 0, sizeof(double2) * tot, stream()));
    RBMG_CK(W.sums.ensure(sizeof(double2) * kMaxSeries));
    RBMG_CK(W.block_scratch.ensure(sizeof(double2) * kSumBlocks * kMaxSeries));
    RBMG_CK(cudaMemsetAsync(W.sums.p, 0, sizeof(double2) * kMaxSeries, stream()));
    StreamResult res;
    r = run_stream(ens, psi, op, false, 4096, &res, [&](const Chunk& c) -> int {
        RBMG_CK(W.eloc.ensure(sizeof(double2) * c.count));
        const int rr = deep_adjoint_chunk(psi, op, c, score, W.eloc.as<double2>(), W.acc_O.as<double2>(),
                                          W.acc_EO.as<double2>(), goff, stream());
        if (rr != RBMG_OK) return rr;
        SeriesSet set{};
        set.n = 1;
        set.v[0] = W.eloc.as<double2>();
        RBMG_CK(launch_weighted_sums(c.count, c.weights, set, W.block_scratch.as<double2>(), W.sums.as<double2>(),
                                     stream()));
        return RBMG_OK;
    });
    if (r != RBMG_OK) return r;
    std::vector<double2> G(tot), GO(tot);
    double2 Es;
    RBMG_CK(cudaMemcpyAsync(G.data(), W.acc_O.p, sizeof(double2) * tot, cudaMemcpyDeviceToHost, stream()));
    RBMG_CK(cudaMemcpyAsync(GO.data(), W.acc_EO.p, sizeof(double2) * tot, cudaMemcpyDeviceToHost, stream()));
    RBMG_CK(cudaMemcpyAsync(&Es, W.sums.p, sizeof(double2), cudaMemcpyDeviceToHost, stream()));
    RBMG_CK(cudaStreamSynchronize(stream()));
    const double f = res.norm_factor;
    const double e_mean = score ? Es.x * f : 0.0;   // <Re E_loc> of this same pass
    cplx* g = reinterpret_cast<cplx*>(grad);
    for (int k = 0; k < P; k++) g[k] = 0.0;
    auto put = [&](size_t k, size_t q) {
        const cplx v = cplx(G[q].x, G[q].y) - 2.0 * e_mean * cplx(GO[q].x, GO[q].y);
        g[k] = std::conj(v * f);
    };
    size_t k = 2 * static_cast<size_t>(N);
    for (int l = 0; l < L; l++) {
        const DeepLayerHost& ly = psi->layers[l];
        const int in = l == 0 ? N : psi->layers[l - 1].size;
        for (int j = 0; j < ly.size; j++) put(k + j, goff[2 * l + 1] + j);
        k += ly.size;
        for (int c = 0; c < ly.conn; c++)
            for (int j = 0; j < ly.size; j++) {
                const int i = static_cast<int>(ly.connections[static_cast<size_t>(c) * ly.size + j]);
                put(k + static_cast<size_t>(c) * ly.size + j, goff[2 * l] + static_cast<size_t>(j) * in + i);
            }
        k += static_cast<size_t>(ly.conn) * ly.size;
    }
    for (int j = 0; j < psi->layers[L - 1].size; j++) put(k + j, goff[2 * L] + j);
    value[0] = Es.x * f;
    value[1] = Es.y * f;
    return RBMG_OK;
}

// ====================================================================== HSD
namespace rbmg {
int deep_hsd64_chunk(const rbmg_psi* psi, const rbmg_psi* pp, const rbmg_operator* op, const Chunk& c,
                     double2* d_eloc, double2* d_dlp, cudaStream_t st);
int deep_hsd_okreduce(const rbmg_psi* pp, int pair_part, int count, const uint64_t* d_spins, uint64_t enum_base,
                      int enumerate, const double2* d_coef, double2* acc, cudaStream_t st);
}  // namespace rbmg

// Hilbert-space distance and its gradient w.r.t. psi' (HilbertSpaceDistance.cu:14-269).
// Stage 1 streams the ensemble of psi and computes, in FP64, omega_s, ratio_s and
// norm_s per sample, keeping the samples; stage 2 forms the gradient numerator as
//   u'_k v - u v'_k = sum_s w_s conj(O_k(s)) B_s,  B_s = conj(<omega>) omega_s v - u <norm> ratio_s,
// an exact rewrite in which the nearly cancelling terms are combined per sample in
// FP64 before the FP32 O_k reduction.  PsiPair uses the two-pass real / imaginary
// form of HilbertSpaceDistance_PsiPair.cu:99-169, each pass drawing its own samples.
extern "C" int rbmg_hsd_gradient(const rbmg_psi* psi, const rbmg_psi* pp, const rbmg_operator* op, int is_unitary,
                                 rbmg_ensemble* ens, float nu, double* grad, double* distance) {
    if (!pp || !op || !distance) return fail(RBMG_EINVAL, "hsd: null");
    int r = check_pair(psi, op, ens);
    if (r != RBMG_OK) return r;
    if (pp->N != psi->N) return fail(RBMG_EINVAL, "hsd: psi and psi_prime differ in N");
    if (psi->kind != pp->kind) return fail(RBMG_EUNSUPPORTED, "hsd: psi and psi_prime must be of the same kind");
    if (psi->kind == 0 && pp->M != psi->M) return fail(RBMG_EUNSUPPORTED, "hsd: psi and psi_prime need the same M");
    const bool want_grad = grad != nullptr;
    const int N = pp->N, P = pp->num_params();
    const int nw = nwords_of(N);
    const size_t ok_len = static_cast<size_t>(P - 2 * N);
    Workspace& W = ws();
    constexpr int kSplits = 64;
    const int passes = (pp->kind == 2 && want_grad) ? 2 : 1;
    const uint64_t total = ens->num_steps();
    std::vector<cplx> gout(P, 0.0);
    double dist = 0.0;
    const OpDev od = op->dev();
    if (psi->kind == 0) {
        r = rbm_upload64(psi);
        if (r == RBMG_OK) r = rbm_upload64(pp);
        if (r != RBMG_OK) return r;
    }
    // free quantum axis of psi (HilbertSpaceDistance.cu:47-81, 109-122): log psi' of every
    // sample gains sum_i [da_i s_i r_i + i db_i (r_i cos_i - s_i sin_i)], r_i = psi'(s with
    // spin i flipped) / psi'(s), and the gradient its alpha / beta entries; the PsiPair
    // gradient (HilbertSpaceDistance_PsiPair.cu) has no such branch
    const bool fqa = psi->free_quantum_axis && !(pp->kind == 2 && want_grad);
    if (fqa) {
        std::vector<double> qa(4 * static_cast<size_t>(N));
        for (int i = 0; i < N; i++) {
            qa[i] = pp->alpha[i] - psi->alpha[i];
            qa[N + i] = pp->beta[i] - psi->beta[i];
            qa[2 * N + i] = std::cos(pp->alpha[i] + psi->alpha[i]);
            qa[3 * N + i] = std::sin(pp->alpha[i] + psi->alpha[i]);
        }
        RBMG_CK(W.fqa_qa.ensure(sizeof(double) * qa.size()));
        RBMG_CK(cudaMemcpyAsync(W.fqa_qa.p, qa.data(), sizeof(double) * qa.size(), cudaMemcpyHostToDevice, stream()));
        if (want_grad) RBMG_CK(W.fqa_r.ensure(sizeof(double2) * total * N));
    }
    // the free-quantum-axis terms of one chunk of samples, in sub-chunks of <= 2^20 flips
    auto fqa_chunk = [&](const Chunk& c, uint64_t offset) -> int {
        const int per = std::max(1, (1 << 20) / N);
        RBMG_CK(W.fqa_flip.ensure(sizeof(uint64_t) * static_cast<size_t>(per) * N * nw));
        RBMG_CK(W.fqa_lpf.ensure(sizeof(double2) * static_cast<size_t>(per) * N));
        RBMG_CK(W.fqa_lp.ensure(sizeof(double2) * per));
        if (!want_grad) RBMG_CK(W.fqa_r.ensure(sizeof(double2) * static_cast<size_t>(per) * N));
        for (int b0 = 0; b0 < c.count; b0 += per) {
            const int n = std::min(per, c.count - b0);
            const uint64_t* sp = c.spins ? c.spins + static_cast<size_t>(b0) * nw : nullptr;
            const uint64_t eb = c.enum_base + static_cast<uint64_t>(b0);
            RBMG_CK(launch_flip_each(n, N, sp, eb, c.enumerate, W.fqa_flip.as<uint64_t>(), stream()));
            int rr = psi_log_psi_dev(pp, n * N, W.fqa_flip.as<uint64_t>(), 0, 0, W.fqa_lpf.as<double2>());
            if (rr == RBMG_OK) rr = psi_log_psi_dev(pp, n, sp, eb, c.enumerate, W.fqa_lp.as<double2>());
            if (rr != RBMG_OK) return rr;
            double2* rout = want_grad ? W.fqa_r.as<double2>() + (offset + b0) * static_cast<size_t>(N)
                                      : W.fqa_r.as<double2>();
            RBMG_CK(launch_fqa_terms(n, N, sp, eb, c.enumerate, W.fqa_lp.as<double2>(), W.fqa_lpf.as<double2>(),
                                     W.fqa_qa.as<double>(), W.logpsi_p.as<double2>() + b0, rout, stream()));
        }
        return RBMG_OK;
    };
    for (int pass = 0; pass < passes; pass++) {
        // ---- stage 1
        RBMG_CK(W.omega.ensure(sizeof(double2) * total));
        RBMG_CK(W.pr.ensure(sizeof(double2) * total));
        RBMG_CK(W.nn.ensure(sizeof(double2) * total));
        RBMG_CK(W.coef3.ensure(sizeof(double) * total));      // weights of all samples
        RBMG_CK(W.Tp.ensure(sizeof(uint64_t) * nw * total));   // spins of all samples
        RBMG_CK(W.sums.ensure(sizeof(double2) * kMaxSeries));
        RBMG_CK(W.block_scratch.ensure(sizeof(double2) * kSumBlocks * kMaxSeries));
        RBMG_CK(cudaMemsetAsync(W.sums.p, 0, sizeof(double2) * kMaxSeries, stream()));
        uint64_t* all_spins = W.Tp.as<uint64_t>();
        double* all_w = W.coef3.as<double>();
        bool weighted = false, enumerated = false;
        uint64_t offset = 0;
        StreamResult res;
        r = run_stream(ens, psi, op, false, size_t(1) << 20, &res, [&](const Chunk& c) -> int {
            RBMG_CK(W.eloc.ensure(sizeof(double2) * c.count));
            RBMG_CK(W.logpsi_p.ensure(sizeof(double2) * c.count));
            if (psi->kind == 0) {
                Hsd64Launch L{};
                L.count = c.count;
                L.enum_base = c.enum_base;
                L.enumerate = c.enumerate;
                L.spins = c.spins;
                L.eloc = W.eloc.as<double2>();
                L.dlogpsi = W.logpsi_p.as<double2>();
                RBMG_CK(launch_rbm_hsd64(rbm64(psi), rbm64(pp), od, L, stream()));
            } else {
                const int rr = deep_hsd64_chunk(psi, pp, op, c, W.eloc.as<double2>(), W.logpsi_p.as<double2>(),
                                                stream());
                if (rr != RBMG_OK) return rr;
            }
            if (fqa) {
                const int rr = fqa_chunk(c, offset);
                if (rr != RBMG_OK) return rr;
            }
            RBMG_CK(launch_hsd_terms64(c.count, W.eloc.as<double2>(), W.logpsi_p.as<double2>(), is_unitary,
                                       W.omega.as<double2>() + offset, W.pr.as<double2>() + offset,
                                       W.nn.as<double2>() + offset, stream()));
            if (c.spins) {
                RBMG_CK(cudaMemcpyAsync(all_spins + offset * nw, c.spins, sizeof(uint64_t) * nw * c.count,
                                        cudaMemcpyDeviceToDevice, stream()));
            } else {
                enumerated = true;
            }
            if (c.weights) {
                weighted = true;
                RBMG_CK(cudaMemcpyAsync(all_w + offset, c.weights, sizeof(double) * c.count, cudaMemcpyDeviceToDevice,
                                        stream()));
            }
            offset += c.count;
            return RBMG_OK;
        });
        if (r != RBMG_OK) return r;
        const int count = static_cast<int>(offset);
        SeriesSet set{};
        set.n = 3;
        set.v[0] = W.omega.as<double2>();
        set.v[1] = W.pr.as<double2>();
        set.v[2] = W.nn.as<double2>();
        RBMG_CK(launch_weighted_sums(count, weighted ? all_w : nullptr, set, W.block_scratch.as<double2>(),
                                     W.sums.as<double2>(), stream()));
        double2 s3[3];
        RBMG_CK(cudaMemcpyAsync(s3, W.sums.p, sizeof(s3), cudaMemcpyDeviceToHost, stream()));
        RBMG_CK(cudaStreamSynchronize(stream()));
        const double f = res.norm_factor;
        const cplx omega = cplx(s3[0].x, s3[0].y) * f;
        const double pr = s3[1].x * f, nn = s3[2].x * f;
        const double u = std::norm(omega);   // HilbertSpaceDistance.cu:216-220, 248-250
        const double v = nn * pr;
        dist = std::sqrt(1.0 - u / v);
        if (!want_grad) break;
        // ---- stage 2: sum_s w_s c_s O_k(s) over the kept samples
        const int mode = passes == 1 ? 0 : (pass == 0 ? 1 : 2);
        const double pf = std::pow(dist, static_cast<double>(nu));
        const double scale = mode == 0 ? 1.0 / (v * v * pf) : (mode == 1 ? 1.0 / (v * v * dist) : 1.0 / (v * dist));
        RBMG_CK(W.coef1.ensure(sizeof(double2) * count));
        RBMG_CK(launch_hsd_coef(count, weighted ? all_w : nullptr, W.omega.as<double2>(), W.pr.as<double2>(),
                                make_double2(omega.real(), -omega.imag()), v, u, nn, mode, scale,
                                W.coef1.as<double2>(), stream()));
        RBMG_CK(W.acc_wO.ensure(sizeof(double2) * ok_len));
        RBMG_CK(cudaMemsetAsync(W.acc_wO.p, 0, sizeof(double2) * ok_len, stream()));
        const uint64_t* sp = enumerated ? (ens->exact_total_z ? ens->d_allowed.as<uint64_t>() : nullptr) : all_spins;
        const int enumerate = (enumerated && !ens->exact_total_z) ? 1 : 0;
        if (pp->kind == 0) {
            RBMG_CK(W.partial.ensure(sizeof(double2) * kSplits * (1 + N) * pp->M));
            const int chunk = std::max(1024, static_cast<int>((size_t(256) << 20) / (sizeof(float2) * pp->Mpad)));
            RBMG_CK(W.T.ensure(sizeof(float2) * std::min(chunk, count) * pp->Mpad));
            RBMG_CK(W.logpsi.ensure(sizeof(double2) * std::min(chunk, count)));
            const RbmDev pd = pp->rbm_dev();
            for (int base = 0; base < count; base += chunk) {
                const int cnt = std::min(chunk, count - base);
                EstLaunch L{};
                L.count = cnt;
                L.enum_base = static_cast<uint64_t>(base);
                L.spins = sp ? sp + static_cast<size_t>(base) * nw : nullptr;
                L.flags = EST_PRIME | (enumerate ? EST_ENUMERATE : 0);
                L.logpsi_prime = W.logpsi.as<double2>();
                L.Tp = W.T.as<float2>();
                RBMG_CK(launch_rbm_estimate(pd, nullptr, &pd, L, stream()));
                RBMG_CK(launch_outer_reduce(cnt, N, nw, pp->M, L.spins, L.enum_base, enumerate,
                                            W.coef1.as<double2>() + base, W.T.as<float2>(), pp->Mpad, 1,
                                            W.acc_wO.as<double2>(), W.partial.as<double2>(), kSplits, stream()));
            }
        } else {
            const int rr = deep_hsd_okreduce(pp, passes == 2 ? pass : -1, count, sp, 0, enumerate,
                                             W.coef1.as<double2>(), W.acc_wO.as<double2>(), stream());
            if (rr != RBMG_OK) return rr;
        }
        std::vector<double2> acc(ok_len);
        RBMG_CK(cudaMemcpyAsync(acc.data(), W.acc_wO.p, sizeof(double2) * ok_len, cudaMemcpyDeviceToHost, stream()));
        std::vector<double2> acc_qa(fqa ? 2 * static_cast<size_t>(N) : 0);
        if (fqa) {   // the alpha / beta entries (mode 0 only: fqa is off for the PsiPair gradient)
            RBMG_CK(W.fqa_out.ensure(sizeof(double2) * 2 * N));
            RBMG_CK(launch_fqa_grad(count, N, sp, 0, enumerate, W.coef1.as<double2>(), W.fqa_r.as<double2>(),
                                    W.fqa_qa.as<double>(), W.fqa_out.as<double2>(), stream()));
            RBMG_CK(cudaMemcpyAsync(acc_qa.data(), W.fqa_out.p, sizeof(double2) * 2 * N, cudaMemcpyDeviceToHost,
                                    stream()));
        }
        RBMG_CK(cudaStreamSynchronize(stream()));
        for (size_t k = 0; k < acc_qa.size(); k++) gout[k] = -(cplx(acc_qa[k].x, acc_qa[k].y) * f);
        // the coefficients already carry 1/v^2/d^nu (mode 0), 1/v^2/d (mode 1), 1/v/d (mode 2)
        if (mode == 0) {          // HilbertSpaceDistance.cu:253-263
            for (size_t k = 0; k < ok_len; k++) gout[2 * N + k] = -(cplx(acc[k].x, acc[k].y) * f);
        } else if (mode == 1) {   // HilbertSpaceDistance_PsiPair.cu:121-133
            for (size_t k = 0; k < ok_len; k++) gout[2 * N + k] = cplx(-(acc[k].x * f), 0.0);
        } else {                  // HilbertSpaceDistance_PsiPair.cu:153-163
            for (size_t k = 0; k < ok_len; k++) gout[2 * N + k] += cplx(0.0, -(acc[k].x * f));
        }
    }
    *distance = dist;
    if (want_grad) std::memcpy(grad, gout.data(), sizeof(cplx) * P);
    return RBMG_OK;
}

// KullbackLeibler::value / gradient (source/network_functions/KullbackLeibler.cu:14-137)
// with D = log psi' - log psi per configuration (FP64):
//   value = sqrt(<|D|^2> - |<D>|^2),  grad_k = (<D O_k*> - <D><O_k*>) / max(value, 1e-6)^nu
// (O_k of psi').  The reference instantiates it with PsiClassical / PsiExact as psi; the
// formula holds for any pair of states, here every pair of this library's kinds with the
// same N (PsiPair psi' for the value only).  The gradient sums w (D - <D>) O_k*, the same
// quantity with the mean taken out first.
extern "C" int rbmg_kl_gradient(const rbmg_psi* psi, const rbmg_psi* pp, rbmg_ensemble* ens, double nu,
                                double* grad, double* value) {
    if (!psi || !pp || !ens || !value) return fail(RBMG_EINVAL, "KullbackLeibler: null");
    if (pp->N != psi->N) return fail(RBMG_EINVAL, "KullbackLeibler: psi and psi_prime differ in N");
    if (ens->kind == 1 && static_cast<int>(ens->num_spins) != psi->N)
        return fail(RBMG_EINVAL, "KullbackLeibler: ExactSummation size differs from psi's N");
    if (grad && pp->kind == 2) return fail(RBMG_EUNSUPPORTED, "KullbackLeibler: gradient for a PsiPair psi_prime");
    int r = RBMG_OK;
    if (psi->kind == 0) r = rbm_upload64(psi);
    if (r == RBMG_OK && pp->kind == 0) r = rbm_upload64(pp);
    if (r != RBMG_OK) return r;
    const int N = pp->N, P = pp->num_params(), nw = nwords_of(N);
    const size_t ok_len = static_cast<size_t>(P - 2 * N);
    const uint64_t total = ens->num_steps();
    Workspace& W = ws();
    RBMG_CK(W.omega.ensure(sizeof(double2) * total));      // D of every sample
    RBMG_CK(W.coef3.ensure(sizeof(double) * total));       // weights of every sample
    RBMG_CK(W.Tp.ensure(sizeof(uint64_t) * nw * total));  // spins of every sample
    RBMG_CK(W.sums.ensure(sizeof(double2) * kMaxSeries));
    RBMG_CK(W.block_scratch.ensure(sizeof(double2) * kSumBlocks * kMaxSeries));
    RBMG_CK(cudaMemsetAsync(W.sums.p, 0, sizeof(double2) * kMaxSeries, stream()));
    double2* D = W.omega.as<double2>();
    uint64_t* all_spins = W.Tp.as<uint64_t>();
    double* all_w = W.coef3.as<double>();
    bool weighted = false, enumerated = false;
    uint64_t offset = 0;
    StreamResult res;
    r = run_stream(ens, psi, nullptr, false, size_t(1) << 20, &res, [&](const Chunk& c) -> int {
        RBMG_CK(W.pr.ensure(sizeof(double2) * c.count));
        RBMG_CK(W.nn.ensure(sizeof(double2) * c.count));
        RBMG_CK(W.coef2.ensure(sizeof(double2) * c.count));
        int rr = psi_log_psi_dev(psi, c.count, c.spins, c.enum_base, c.enumerate, W.pr.as<double2>());
        if (rr == RBMG_OK) rr = psi_log_psi_dev(pp, c.count, c.spins, c.enum_base, c.enumerate, W.nn.as<double2>());
        if (rr != RBMG_OK) return rr;
        RBMG_CK(launch_sub(c.count, W.nn.as<double2>(), W.pr.as<double2>(), D + offset, stream()));
        RBMG_CK(launch_abs2(c.count, D + offset, W.coef2.as<double2>(), stream()));
        SeriesSet set{};
        set.n = 2;
        set.v[0] = D + offset;
        set.v[1] = W.coef2.as<double2>();
        RBMG_CK(launch_weighted_sums(c.count, c.weights, set, W.block_scratch.as<double2>(), W.sums.as<double2>(),
                                     stream()));
        if (c.spins) {
            RBMG_CK(cudaMemcpyAsync(all_spins + offset * nw, c.spins, sizeof(uint64_t) * nw * c.count,
                                    cudaMemcpyDeviceToDevice, stream()));
        } else {
            enumerated = true;
        }
        if (c.weights) {
            weighted = true;
            RBMG_CK(cudaMemcpyAsync(all_w + offset, c.weights, sizeof(double) * c.count, cudaMemcpyDeviceToDevice,
                                    stream()));
        }
        offset += c.count;
        return RBMG_OK;
    });
    if (r != RBMG_OK) return r;
    double2 s2[2];
    RBMG_CK(cudaMemcpyAsync(s2, W.sums.p, sizeof(s2), cudaMemcpyDeviceToHost, stream()));
    RBMG_CK(cudaStreamSynchronize(stream()));
    const double f = res.norm_factor;
    const cplx mean = cplx(s2[0].x, s2[0].y) * f;
    const double v = std::sqrt(s2[1].x * f - std::norm(mean));   // KullbackLeibler.cu:100-104
    *value = v;
    if (!grad) return RBMG_OK;
    const int count = static_cast<int>(offset);
    const double factor = std::pow(std::max(v, 1e-6), nu);        // :119-121
    RBMG_CK(W.coef1.ensure(sizeof(double2) * count));
    RBMG_CK(launch_coef(count, weighted ? all_w : nullptr, D, f / factor, W.coef1.as<double2>(), stream(),
                        make_double2(mean.real(), mean.imag())));
    RBMG_CK(W.acc_wO.ensure(sizeof(double2) * ok_len));
    RBMG_CK(cudaMemsetAsync(W.acc_wO.p, 0, sizeof(double2) * ok_len, stream()));
    const uint64_t* sp = enumerated ? (ens->exact_total_z ? ens->d_allowed.as<uint64_t>() : nullptr) : all_spins;
    const int enumerate = (enumerated && !ens->exact_total_z) ? 1 : 0;
    if (pp->kind == 0) {
        constexpr int kSplits = 64;
        RBMG_CK(W.partial.ensure(sizeof(double2) * kSplits * (1 + N) * pp->M));
        const int chunk = std::max(1024, static_cast<int>((size_t(256) << 20) / (sizeof(float2) * pp->Mpad)));
        RBMG_CK(W.T.ensure(sizeof(float2) * std::min(chunk, count) * pp->Mpad));
        RBMG_CK(W.logpsi_p.ensure(sizeof(double2) * std::min(chunk, count)));
        const RbmDev pd = pp->rbm_dev();
        for (int base = 0; base < count; base += chunk) {
            const int cnt = std::min(chunk, count - base);
            EstLaunch L{};
            L.count = cnt;
            L.enum_base = static_cast<uint64_t>(base);
            L.spins = sp ? sp + static_cast<size_t>(base) * nw : nullptr;
            L.flags = EST_PRIME | (enumerate ? EST_ENUMERATE : 0);
            L.logpsi_prime = W.logpsi_p.as<double2>();
            L.Tp = W.T.as<float2>();
            RBMG_CK(launch_rbm_estimate(pd, nullptr, &pd, L, stream()));
            RBMG_CK(launch_outer_reduce(cnt, N, nw, pp->M, L.spins, L.enum_base, enumerate,
                                        W.coef1.as<double2>() + base, W.T.as<float2>(), pp->Mpad, 1,
                                        W.acc_wO.as<double2>(), W.partial.as<double2>(), kSplits, stream()));
        }
    } else {
        const int rr = deep_hsd_okreduce(pp, -1, count, sp, 0, enumerate, W.coef1.as<double2>(),
                                         W.acc_wO.as<double2>(), stream());
        if (rr != RBMG_OK) return rr;
    }
    std::vector<double2> acc(ok_len);
    RBMG_CK(cudaMemcpyAsync(acc.data(), W.acc_wO.p, sizeof(double2) * ok_len, cudaMemcpyDeviceToHost, stream()));
    RBMG_CK(cudaStreamSynchronize(stream()));
    cplx* g = reinterpret_cast<cplx*>(grad);
    for (int k = 0; k < 2 * N; k++) g[k] = 0.0;
    for (size_t k = 0; k < ok_len; k++) g[2 * N + k] = cplx(acc[k].x, acc[k].y);
    return RBMG_OK;
}

// DiagDensityOp(sub_system_size)(psi, op, ensemble) (source/network_functions/DiagDensityOp.cu:
// 12-50): densities [2^N_A] = sum_s weight |E_loc(s)|^2 binned by the first N_A spins, over
// num_steps (the reference's local_energy1 * conj(local_energy2) of one operator)
extern "C" int rbmg_diag_density(const rbmg_psi* psi, const rbmg_operator* op, rbmg_ensemble* ens,
                                 int sub_system_size, double* out) {
    if (!out) return fail(RBMG_EINVAL, "DiagDensityOp: null");
    int r = check_pair(psi, op, ens);
    if (r != RBMG_OK) return r;
    if (sub_system_size < 0 || sub_system_size > std::min(psi->N, 30))
        return fail(RBMG_EINVAL, "DiagDensityOp: sub_system_size must lie in [0, min(N, 30)]");
    const int na = sub_system_size, bins = 1 << na, nw = nwords_of(psi->N);
    Workspace& W = ws();
    RBMG_CK(W.coef3.ensure(sizeof(double) * bins));
    RBMG_CK(cudaMemsetAsync(W.coef3.p, 0, sizeof(double) * bins, stream()));
    StreamResult res;
    r = run_stream(ens, psi, op, true, size_t(1) << 20, &res, [&](const Chunk& c) -> int {
        const double2* e = nullptr;
        const int rr = chunk_eloc(psi, op, c, &e);
        if (rr != RBMG_OK) return rr;
        RBMG_CK(launch_diag_density(c.count, c.enumerate, c.enum_base, c.spins, nw, c.weights, e, na,
                                    W.coef3.as<double>(), stream()));
        return RBMG_OK;
    });
    if (r != RBMG_OK) return r;
    RBMG_CK(cudaMemcpyAsync(out, W.coef3.p, sizeof(double) * bins, cudaMemcpyDeviceToHost, stream()));
    RBMG_CK(cudaStreamSynchronize(stream()));
    for (int i = 0; i < bins; i++) out[i] *= res.norm_factor;
    return RBMG_OK;
}

// HilbertSpaceDistance::distance_2nd_order (source/network_functions/HilbertSpaceDistance_2nd_order.cu:
// 14-95): the distance to psi' of the state exp(A) psi expanded to second order, with the
// local energies of A (op) and of A^2 (op2) in FP64
extern "C" int rbmg_hsd_distance_2nd_order(const rbmg_psi* psi, const rbmg_psi* pp, const rbmg_operator* op,
                                           const rbmg_operator* op2, rbmg_ensemble* ens, double* distance) {
    if (!pp || !op || !op2 || !distance) return fail(RBMG_EINVAL, "hsd 2nd order: null");
    int r = check_pair(psi, op, ens);
    if (r == RBMG_OK) r = check_pair(psi, op2, ens);
    if (r != RBMG_OK) return r;
    if (pp->N != psi->N) return fail(RBMG_EINVAL, "hsd 2nd order: psi and psi_prime differ in N");
    if (psi->kind != pp->kind) return fail(RBMG_EUNSUPPORTED, "hsd 2nd order: psi and psi_prime must be of the same kind");
    if (psi->kind == 2) return fail(RBMG_EUNSUPPORTED, "hsd 2nd order: not instantiated for PsiPair");
    if (psi->kind == 0) {
        r = rbm_upload64(psi);
        if (r == RBMG_OK) r = rbm_upload64(pp);
        if (r != RBMG_OK) return r;
    }
    Workspace& W = ws();
    RBMG_CK(W.sums.ensure(sizeof(double2) * kMaxSeries));
    RBMG_CK(W.block_scratch.ensure(sizeof(double2) * kSumBlocks * kMaxSeries));
    RBMG_CK(cudaMemsetAsync(W.sums.p, 0, sizeof(double2) * kMaxSeries, stream()));
    const OpDev od = op->dev(), od2 = op2->dev();
    StreamResult res;
    r = run_stream(ens, psi, op, false, size_t(1) << 20, &res, [&](const Chunk& c) -> int {
        RBMG_CK(W.eloc.ensure(sizeof(double2) * c.count));
        RBMG_CK(W.coef2.ensure(sizeof(double2) * c.count));
        RBMG_CK(W.logpsi_p.ensure(sizeof(double2) * c.count));
        RBMG_CK(W.omega.ensure(sizeof(double2) * c.count));
        RBMG_CK(W.pr.ensure(sizeof(double2) * c.count));
        RBMG_CK(W.nn.ensure(sizeof(double2) * c.count));
        for (int which = 0; which < 2; which++) {
            double2* e = which == 0 ? W.eloc.as<double2>() : W.coef2.as<double2>();
            if (psi->kind == 0) {
                Hsd64Launch L{};
                L.count = c.count;
                L.enum_base = c.enum_base;
                L.enumerate = c.enumerate;
                L.spins = c.spins;
                L.eloc = e;
                L.dlogpsi = W.logpsi_p.as<double2>();
                RBMG_CK(launch_rbm_hsd64(rbm64(psi), rbm64(pp), which == 0 ? od : od2, L, stream()));
            } else {
                const int rr = deep_hsd64_chunk(psi, pp, which == 0 ? op : op2, c, e, W.logpsi_p.as<double2>(),
                                                stream());
                if (rr != RBMG_OK) return rr;
            }
        }
        RBMG_CK(launch_hsd2_terms64(c.count, W.eloc.as<double2>(), W.coef2.as<double2>(), W.logpsi_p.as<double2>(),
                                    W.omega.as<double2>(), W.pr.as<double2>(), W.nn.as<double2>(), stream()));
        SeriesSet set{};
        set.n = 3;
        set.v[0] = W.omega.as<double2>();
        set.v[1] = W.pr.as<double2>();
        set.v[2] = W.nn.as<double2>();
        RBMG_CK(launch_weighted_sums(c.count, c.weights, set, W.block_scratch.as<double2>(), W.sums.as<double2>(),
                                     stream()));
        return RBMG_OK;
    });
    if (r != RBMG_OK) return r;
    double2 s3[3];
    RBMG_CK(cudaMemcpyAsync(s3, W.sums.p, sizeof(s3), cudaMemcpyDeviceToHost, stream()));
    RBMG_CK(cudaStreamSynchronize(stream()));
    const double f = res.norm_factor;   // HilbertSpaceDistance_2nd_order.cu:83-94
    const cplx omega = cplx(s3[0].x, s3[0].y) * f;
    const double pr = s3[1].x * f, nn = s3[2].x * f;
    *distance = std::sqrt(1.0 - std::norm(omega) / (nn * pr));
    return RBMG_OK;
}

extern "C" int rbmg_hsd_distance(const rbmg_psi* psi, const rbmg_psi* pp, const rbmg_operator* op, int is_unitary,
                                 rbmg_ensemble* ens, double* distance) {
    return rbmg_hsd_gradient(psi, pp, op, is_unitary, ens, 1.0f, nullptr, distance);
}

// ====================================================================== samples / O_k
extern "C" int rbmg_ensemble_samples(rbmg_ensemble* ens, const rbmg_psi* psi, const rbmg_operator* op,
                                     uint64_t* spins, double* log_psi, double* eloc) {
    int r = check_pair(psi, op, ens);
    if (r != RBMG_OK) return r;
    if (eloc && !op) return fail(RBMG_EINVAL, "samples: local energies need an operator");
    const int nw = nwords_of(psi->N);
    Workspace& W = ws();
    uint64_t offset = 0;
    StreamResult res;
    r = run_stream(ens, psi, op, eloc != nullptr, size_t(1) << 22, &res, [&](const Chunk& c) -> int {
        if (spins) {
            if (c.spins) {
                RBMG_CK(cudaMemcpyAsync(spins + offset * nw, c.spins, sizeof(uint64_t) * nw * c.count,
                                        cudaMemcpyDeviceToHost, stream()));
            } else {
                for (int t = 0; t < c.count; t++) {
                    spins[(offset + t) * nw] = c.enum_base + t;
                    for (int k = 1; k < nw; k++) spins[(offset + t) * nw + k] = 0;
                }
            }
        }
        if (log_psi) {
            RBMG_CK(W.logpsi_p.ensure(sizeof(double2) * c.count));
            const int rr = psi_log_psi_dev(psi, c.count, c.spins, c.enum_base, c.enumerate, W.logpsi_p.as<double2>());
            if (rr != RBMG_OK) return rr;
            RBMG_CK(cudaMemcpyAsync(log_psi + 2 * offset, W.logpsi_p.p, sizeof(double2) * c.count,
                                    cudaMemcpyDeviceToHost, stream()));
        }
        if (eloc) {
            const double2* e = nullptr;
            const int rr = chunk_eloc(psi, op, c, &e);
            if (rr != RBMG_OK) return rr;
            RBMG_CK(cudaMemcpyAsync(eloc + 2 * offset, e, sizeof(double2) * c.count, cudaMemcpyDeviceToHost, stream()));
        }
        RBMG_CK(cudaStreamSynchronize(stream()));
        offset += c.count;
        return RBMG_OK;
    });
    return r;
}

namespace rbmg {
int deep_ok_vector(const rbmg_psi* psi, const uint64_t* d_spins, double2* d_out, cudaStream_t st);
}  // namespace rbmg

extern "C" int rbmg_psi_O_k_vector(const rbmg_psi* psi, const uint64_t* spins, double* out) {
    if (!psi || !spins || !out) return fail(RBMG_EINVAL, "O_k_vector: null");
    const int N = psi->N, P = psi->num_params();
    const int nw = nwords_of(N);
    Workspace& W = ws();
    RBMG_CK(W.sample_spins.ensure(sizeof(uint64_t) * nw));
    RBMG_CK(cudaMemcpyAsync(W.sample_spins.p, spins, sizeof(uint64_t) * nw, cudaMemcpyHostToDevice, stream()));
    cplx* o = reinterpret_cast<cplx*>(out);
    for (int k = 0; k < P; k++) o[k] = 0.0;
    if (psi->kind == 0) {
        RBMG_CK(W.Tp.ensure(sizeof(float2) * psi->Mpad));
        RBMG_CK(W.logpsi_p.ensure(sizeof(double2)));
        EstLaunch L{};
        L.count = 1;
        L.spins = W.sample_spins.as<uint64_t>();
        L.flags = EST_PRIME;    // psi itself as psi': writes tanh(theta) into Tp
        L.logpsi_prime = W.logpsi_p.as<double2>();
        L.Tp = W.Tp.as<float2>();
        const RbmDev d = psi->rbm_dev();
        RBMG_CK(launch_rbm_estimate(d, nullptr, &d, L, stream()));
        std::vector<float2> T(psi->Mpad);
        RBMG_CK(cudaMemcpyAsync(T.data(), W.Tp.p, sizeof(float2) * psi->Mpad, cudaMemcpyDeviceToHost, stream()));
        RBMG_CK(cudaStreamSynchronize(stream()));
        const int M = psi->M;   // Psi.hpp:165-178
        for (int j = 0; j < M; j++) {
            const cplx t(T[j].x, T[j].y);
            o[2 * N + j] = t;
            for (int i = 0; i < N; i++) {
                const bool up = (spins[i >> 6] >> (i & 63)) & 1ull;
                o[2 * N + M + static_cast<size_t>(i) * M + j] = up ? t : -t;
            }
        }
        return RBMG_OK;
    }
    RBMG_CK(W.acc_O.ensure(sizeof(double2) * P));
    const int r = deep_ok_vector(psi, W.sample_spins.as<uint64_t>(), W.acc_O.as<double2>(), stream());
    if (r != RBMG_OK) return r;
    RBMG_CK(cudaMemcpyAsync(out + 4 * N, W.acc_O.p, sizeof(double2) * (P - 2 * N), cudaMemcpyDeviceToHost, stream()));
    RBMG_CK(cudaStreamSynchronize(stream()));
    return RBMG_OK;
}

// ====================================================================== persistent chains
static thread_local double g_sm_timing_ms = 0.0;
static thread_local int g_sm_timing_launches = 0;

namespace rbmg {
int deep_ok_rows(const rbmg_psi* psi, int count, const uint64_t* d_spins, uint64_t enum_base, int enumerate,
                 double2* rows, long ld, cudaStream_t st);
}  // namespace rbmg

// Writes one word of every page of a large host output from several threads while the GPU
// works, so that the device-to-host copy of the result does not take the first-touch page
// faults of a freshly allocated array one by one (joined before the copy).
class Prefault {
  public:
    Prefault(void* p, size_t bytes) {
        const size_t page = static_cast<size_t>(std::max(4096L, sysconf(_SC_PAGESIZE)));
        if (bytes < (size_t(64) << 20)) return;
        const int n = static_cast<int>(std::min(16u, std::max(1u, std::thread::hardware_concurrency())));
        const size_t pages = (bytes + page - 1) / page, per = (pages + n - 1) / n;
        char* base = static_cast<char*>(p);
        for (int t = 0; t < n; t++) {
            const size_t p0 = t * per, p1 = std::min(pages, p0 + per);
            if (p0 >= p1) break;
            threads_.emplace_back([=]() {
                for (size_t q = p0; q < p1; q++) *reinterpret_cast<volatile char*>(base + q * page) = 0;
            });
        }
    }
    void join() {
        for (auto& t : threads_) t.join();
        threads_.clear();
    }
    ~Prefault() { join(); }

  private:
    std::vector<std::thread> threads_;
};

// get_S_matrix (source/network_functions/S_matrix.cu:10-53, instantiated for Psi with
// ExactSummation only): S[k][k'] = sum_s O_k(s) conj(O_k'(s)) / num_steps over every
// configuration of the ensemble, without the ensemble's weight (the reference ignores the
// weight its foreach passes); flags add the weight and / or centre it (the SR covariance).
extern "C" int rbmg_s_matrix(const rbmg_psi* psi, rbmg_ensemble* ens, int flags, double* out) {
    if (!psi || !ens || !out) return fail(RBMG_EINVAL, "S_matrix: null");
    if (psi->kind == 2) return fail(RBMG_EUNSUPPORTED, "S_matrix: PsiPair has no O_k (PsiPair.hpp:73-76)");
    if (ens->kind == 1 && static_cast<int>(ens->num_spins) != psi->N)
        return fail(RBMG_EINVAL, "S_matrix: ExactSummation size differs from psi's N");
    const int N = psi->N, P = psi->num_params(), L = P - 2 * N, nw = nwords_of(N);
    const bool weighted = (flags & RBMG_S_WEIGHTED) != 0, centered = (flags & RBMG_S_CENTERED) != 0;
    const bool use_tc = (flags & RBMG_S_SIMT) == 0;
    Workspace& W = ws();
    const size_t sbytes = sizeof(double2) * static_cast<size_t>(L) * L;
    Prefault prefault(out, sizeof(double2) * static_cast<size_t>(P) * P);
    RBMG_CK(W.smat.ensure(sbytes));
    RBMG_CK(W.smean.ensure(sizeof(double2) * L));
    RBMG_CK(cudaMemsetAsync(W.smat.p, 0, sbytes, stream()));
    RBMG_CK(cudaMemsetAsync(W.smean.p, 0, sizeof(double2) * L, stream()));
    int dev = 0, sms = 0;
    RBMG_CK(cudaGetDevice(&dev));
    RBMG_CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    uint64_t total = 0;
    StreamResult res;
    // centred: every row is shifted by the first chunk's mean row (in FP64) before the FP32
    // products, so that the covariance is not the small difference of two large sums
    RBMG_CK(W.sshift.ensure(sizeof(double2) * L));
    bool have_shift = false;
    auto with_shift = [&](SmSource& a) -> cudaError_t {
        if (!centered) return cudaSuccess;
        if (!have_shift) {
            const cudaError_t e = launch_sm_row_mean(a, W.sshift.as<double2>(), stream());
            if (e != cudaSuccess) return e;
            have_shift = true;
        }
        a.shift = W.sshift.as<double2>();
        return cudaSuccess;
    };
    if (use_tc) {
        RBMG_CK(W.serror.ensure(sizeof(int)));
        RBMG_CK(cudaMemsetAsync(W.serror.p, 0, sizeof(int), stream()));
    }
    int nlaunch = 0;
    // the products of one chunk (tensor cores, or the FP32 tile kernel) and its mean row
    auto accumulate = [&](const SmSource& a) -> cudaError_t {
        cudaError_t e;
        if (use_tc) {
            e = W.splanes.ensure(sm_tc_planes_bytes(L, a.count));
            if (e != cudaSuccess) return e;
            e = launch_sm_tc_accumulate(a, W.smat.as<double2>(), W.splanes.p, W.serror.as<int>(), &nlaunch, sms,
                                        stream());
        } else {
            e = launch_sm_accumulate(a, W.smat.as<double2>(), nullptr, sms, stream());
            nlaunch++;
        }
        if (e != cudaSuccess || !centered) return e;
        nlaunch++;
        return launch_sm_mean(a, W.smean.as<double2>(), stream());
    };
    // CUDA events around every accumulation launch (rbmg_s_matrix_timing)
    std::vector<cudaEvent_t> ev;
    auto mark = [&]() -> cudaError_t {
        cudaEvent_t e;
        cudaError_t err = cudaEventCreate(&e);
        if (err != cudaSuccess) return err;
        ev.push_back(e);
        return cudaEventRecord(e, stream());
    };
    struct EvFree {
        std::vector<cudaEvent_t>& v;
        ~EvFree() {
            for (auto e : v) cudaEventDestroy(e);
        }
    } ev_free{ev};
    const int r = run_stream(ens, psi, nullptr, false, 4096, &res, [&](const Chunk& c) -> int {
        total += static_cast<uint64_t>(c.count);
        SmSource a{};
        a.L = L;
        a.N = N;
        a.M = psi->M;
        a.Mpad = psi->Mpad;
        a.nw = nw;
        a.weighted = weighted && c.weights;
        if (psi->kind == 0) {
            RBMG_CK(W.Tp.ensure(sizeof(float2) * static_cast<size_t>(c.count) * psi->Mpad));
            RBMG_CK(W.logpsi_p.ensure(sizeof(double2) * c.count));
            EstLaunch E{};
            E.count = c.count;
            E.enum_base = c.enum_base;
            E.spins = c.spins;
            E.flags = EST_PRIME | (c.enumerate ? EST_ENUMERATE : 0);
            E.logpsi_prime = W.logpsi_p.as<double2>();
            E.Tp = W.Tp.as<float2>();
            const RbmDev d = psi->rbm_dev();
            RBMG_CK(launch_rbm_estimate(d, nullptr, &d, E, stream()));
            a.kind = 0;
            a.count = c.count;
            a.enumerate = c.enumerate;
            a.enum_base = c.enum_base;
            a.spins = c.spins;
            a.T = W.Tp.as<float2>();
            a.w = c.weights;
            RBMG_CK(with_shift(a));
            RBMG_CK(mark());
            RBMG_CK(accumulate(a));
            RBMG_CK(mark());
            return RBMG_OK;
        }
        // PsiDeep: FP64 O_k rows, in pieces of at most 256 MB
        const int piece = static_cast<int>(std::max<size_t>(1, (size_t(256) << 20) / (sizeof(double2) * L)));
        RBMG_CK(W.okrows.ensure(sizeof(double2) * static_cast<size_t>(std::min(piece, c.count)) * L));
        for (int base = 0; base < c.count; base += piece) {
            const int cnt = std::min(piece, c.count - base);
            const uint64_t* sp = c.spins ? c.spins + static_cast<size_t>(base) * nw : nullptr;
            const int rr = deep_ok_rows(psi, cnt, sp, c.enum_base + base, c.enumerate, W.okrows.as<double2>(), L,
                                        stream());
            if (rr != RBMG_OK) return rr;
            a.kind = 1;
            a.count = cnt;
            a.rows = W.okrows.as<double2>();
            a.ld = L;
            a.w = c.weights ? c.weights + base : nullptr;
            a.weighted = weighted && a.w;
            RBMG_CK(with_shift(a));
            RBMG_CK(mark());
            RBMG_CK(accumulate(a));
            RBMG_CK(mark());
        }
        return RBMG_OK;
    });
    if (r != RBMG_OK) return r;
    if (total == 0) return fail(RBMG_EINVAL, "S_matrix: the ensemble has no samples");
    // the exact-summation weights are normalised to sum 1; otherwise divide by the count
    const double z = (weighted && ens->kind == 1) ? 1.0 : static_cast<double>(total);
    // the P x P result on the device (zero rows and columns below 2N), then one contiguous copy
    const size_t obytes = sizeof(double2) * static_cast<size_t>(P) * P;
    RBMG_CK(W.sout.ensure(obytes));
    RBMG_CK(cudaMemsetAsync(W.sout.p, 0, sizeof(double2) * static_cast<size_t>(2 * N) * P, stream()));
    if (N > 0)
        RBMG_CK(cudaMemset2DAsync(W.sout.as<double2>() + static_cast<size_t>(2 * N) * P, sizeof(double2) * P, 0,
                                  sizeof(double2) * 2 * N, L, stream()));
    RBMG_CK(launch_sm_finish(L, W.smat.as<double2>(), W.smean.as<double2>(), 1.0 / z, centered ? 1 : 0,
                             W.sout.as<double2>(), P, 2 * N, stream()));
    prefault.join();
    RBMG_CK(cudaMemcpyAsync(out, W.sout.p, obytes, cudaMemcpyDeviceToHost, stream()));
    int tc_err = 0;
    if (use_tc) RBMG_CK(cudaMemcpyAsync(&tc_err, W.serror.p, sizeof(int), cudaMemcpyDeviceToHost, stream()));
    RBMG_CK(cudaStreamSynchronize(stream()));
    if (tc_err) return fail(RBMG_ETIMEOUT, "S_matrix: a tensor-core wait gave up");
    double ms = 0.0;
    for (size_t q = 0; q + 1 < ev.size(); q += 2) {
        float t = 0.0f;
        RBMG_CK(cudaEventElapsedTime(&t, ev[q], ev[q + 1]));
        ms += t;
    }
    g_sm_timing_ms = ms;
    g_sm_timing_launches = nlaunch;
    return RBMG_OK;
}

extern "C" int rbmg_s_matrix_timing(double* ms, int* launches) {
    if (!ms || !launches) return fail(RBMG_EINVAL, "S_matrix timing: null");
    *ms = g_sm_timing_ms;
    *launches = g_sm_timing_launches;
    return RBMG_OK;
}

extern "C" int rbmg_stream(void** st) {
    if (!st) return fail(RBMG_EINVAL, "stream: null");
    *st = static_cast<void*>(stream());
    return RBMG_OK;
}

extern "C" int rbmg_chain_create(const rbmg_psi* psi, uint32_t num_walkers, uint64_t seed, rbmg_chain** out) {
    if (!psi || !out || num_walkers == 0) return fail(RBMG_EINVAL, "chain: bad arguments");
    if (psi->kind != 0) return fail(RBMG_EUNSUPPORTED, "chain: complex RBM only");
    auto c = std::make_unique<rbmg_chain>();
    c->N = psi->N;
    c->nw = nwords_of(psi->N);
    c->walkers = num_walkers;
    c->seed = seed;
    RBMG_CK(c->spins.ensure(sizeof(uint64_t) * c->nw * num_walkers));
    RBMG_CK(c->rng_index.ensure(sizeof(uint64_t) * num_walkers));
    RBMG_CK(c->accepts.ensure(sizeof(unsigned long long) * num_walkers));
    RBMG_CK(c->proposals.ensure(sizeof(unsigned long long) * num_walkers));
    RBMG_CK(cudaMemset(c->rng_index.p, 0, sizeof(uint64_t) * num_walkers));
    RBMG_CK(cudaMemset(c->accepts.p, 0, sizeof(unsigned long long) * num_walkers));
    RBMG_CK(cudaMemset(c->proposals.p, 0, sizeof(unsigned long long) * num_walkers));
    *out = c.release();
    return RBMG_OK;
}

extern "C" int rbmg_chain_destroy(rbmg_chain* c) {
    delete c;
    return RBMG_OK;
}

extern "C" int rbmg_chain_sweep_async(rbmg_chain* c, const rbmg_psi* psi, const rbmg_operator* op, int n_sweeps,
                                      int measure_every, void* d_eloc_out, void* st) {
    if (!c || !psi || n_sweeps < 0) return fail(RBMG_EINVAL, "chain sweep: bad arguments");
    if (psi->kind != 0 || psi->N != c->N) return fail(RBMG_EINVAL, "chain sweep: psi does not match the chain");
    if (d_eloc_out && (!op || measure_every <= 0)) return fail(RBMG_EINVAL, "chain sweep: measurement needs op");
    if (op && op->max_site >= psi->N) return fail(RBMG_EINVAL, "chain sweep: operator acts on a site >= N");
    if (n_sweeps == 0) return RBMG_OK;
    cudaStream_t cs = st ? static_cast<cudaStream_t>(st) : stream();
    const RbmDev P = psi->rbm_dev();
    OpDev od;
    if (op) od = op->dev();
    McLaunch L{};
    L.B = static_cast<int>(c->walkers);
    L.walker_base = 0;
    L.seed = c->seed;
    L.spins = c->spins.as<uint64_t>();
    L.rng_index = c->rng_index.as<uint64_t>();
    L.sweeps_per_sample = 1;
    L.accepts = c->accepts.as<unsigned long long>();
    L.proposals = c->proposals.as<unsigned long long>();
    auto sweeps = [&](int n) -> int {
        if (n <= 0) return RBMG_OK;
        L.init = c->initialised ? 0 : 1;
        L.n_therm = n;
        L.n_samples = 0;
        RBMG_CK(launch_rbm_mc(P, nullptr, L, cs));
        c->initialised = true;
        return RBMG_OK;
    };
    if (!d_eloc_out) return sweeps(n_sweeps);
    // n_sweeps % measure_every leading sweeps, then (measure_every sweeps, measurement) rows
    int r = sweeps(n_sweeps % measure_every);
    if (r != RBMG_OK) return r;
    double2* out = static_cast<double2*>(d_eloc_out);
    for (int row = 0; row < n_sweeps / measure_every; row++) {
        r = sweeps(measure_every);
        if (r != RBMG_OK) return r;
        EstLaunch E{};
        E.count = static_cast<int>(c->walkers);
        E.spins = c->spins.as<uint64_t>();
        E.flags = EST_ELOC;
        E.eloc = out + static_cast<size_t>(row) * c->walkers;
        RBMG_CK(launch_rbm_estimate(P, &od, nullptr, E, cs));
    }
    return RBMG_OK;
}

// checkpoint of the walkers: spins [walkers][nw], next Philox word [walkers], accept and
// proposal counters [walkers]; restoring it continues the chains bit for bit
extern "C" int rbmg_chain_get_checkpoint(const rbmg_chain* c, uint64_t* spins, uint64_t* rng_index, uint64_t* accepts,
                                         uint64_t* proposals) {
    if (!c || !spins || !rng_index || !accepts || !proposals) return fail(RBMG_EINVAL, "chain checkpoint: null");
    if (!c->initialised) return fail(RBMG_EINVAL, "chain checkpoint: the chain has not started");
    RBMG_CK(cudaDeviceSynchronize());
    const size_t B = c->walkers;
    RBMG_CK(cudaMemcpy(spins, c->spins.p, sizeof(uint64_t) * c->nw * B, cudaMemcpyDeviceToHost));
    RBMG_CK(cudaMemcpy(rng_index, c->rng_index.p, sizeof(uint64_t) * B, cudaMemcpyDeviceToHost));
    RBMG_CK(cudaMemcpy(accepts, c->accepts.p, sizeof(uint64_t) * B, cudaMemcpyDeviceToHost));
    RBMG_CK(cudaMemcpy(proposals, c->proposals.p, sizeof(uint64_t) * B, cudaMemcpyDeviceToHost));
    return RBMG_OK;
}

extern "C" int rbmg_chain_set_checkpoint(rbmg_chain* c, const uint64_t* spins, const uint64_t* rng_index,
                                         const uint64_t* accepts, const uint64_t* proposals) {
    if (!c || !spins || !rng_index || !accepts || !proposals) return fail(RBMG_EINVAL, "chain checkpoint: null");
    const size_t B = c->walkers;
    for (size_t w = 0; w < B; w++)
        if (c->N % 64 && (spins[w * c->nw + c->nw - 1] >> (c->N % 64)))
            return fail(RBMG_EINVAL, "chain checkpoint: spin bits beyond N");
    RBMG_CK(cudaDeviceSynchronize());
    RBMG_CK(cudaMemcpy(c->spins.p, spins, sizeof(uint64_t) * c->nw * B, cudaMemcpyHostToDevice));
    RBMG_CK(cudaMemcpy(c->rng_index.p, rng_index, sizeof(uint64_t) * B, cudaMemcpyHostToDevice));
    RBMG_CK(cudaMemcpy(c->accepts.p, accepts, sizeof(uint64_t) * B, cudaMemcpyHostToDevice));
    RBMG_CK(cudaMemcpy(c->proposals.p, proposals, sizeof(uint64_t) * B, cudaMemcpyHostToDevice));
    c->initialised = true;
    return RBMG_OK;
}

extern "C" int rbmg_chain_state(const rbmg_chain* c, uint64_t* spins, uint64_t* accepts, uint64_t* proposals) {
    if (!c) return fail(RBMG_EINVAL, "chain state: null");
    RBMG_CK(cudaDeviceSynchronize());
    if (spins) RBMG_CK(cudaMemcpy(spins, c->spins.p, sizeof(uint64_t) * c->nw * c->walkers, cudaMemcpyDeviceToHost));
    std::vector<unsigned long long> a(c->walkers), p(c->walkers);
    RBMG_CK(cudaMemcpy(a.data(), c->accepts.p, sizeof(unsigned long long) * c->walkers, cudaMemcpyDeviceToHost));
    RBMG_CK(cudaMemcpy(p.data(), c->proposals.p, sizeof(unsigned long long) * c->walkers, cudaMemcpyDeviceToHost));
    uint64_t sa = 0, sp = 0;
    for (uint32_t w = 0; w < c->walkers; w++) {
        sa += a[w];
        sp += p[w];
    }
    if (accepts) *accepts = sa;
    if (proposals) *proposals = sp;
    return RBMG_OK;
}

