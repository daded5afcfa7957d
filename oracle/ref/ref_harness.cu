// Golden-vector generator: drives the RBMonGPU reference's own host path
// (objects constructed with gpu=false) through its public C++ API and writes
// the results as raw binary files.  Used only by tests/golden/make_golden.py.
//
// usage: ref_harness <case_dir>
// The case directory holds meta.txt ("key value" lines) and raw little-endian
// arrays; results are written back into the same directory as out_*.bin and
// out_scalars.txt.
#include "quantum_states.hpp"
#include "spin_ensembles.hpp"
#include "operator/Operator.hpp"
#include "network_functions/ExpectationValue.hpp"
#include "network_functions/HilbertSpaceDistance.hpp"
#include "network_functions/PsiNorm.hpp"
#include "network_functions/PsiVector.hpp"
#include "network_functions/PsiOkVector.hpp"
#include "network_functions/S_matrix.hpp"
#include "network_functions/DiagDensityOp.hpp"
#include "network_functions/KullbackLeibler.hpp"
// The reference's KullbackLeibler source, compiled in place in this unit: it instantiates
// the templates only for PsiClassical / PsiExact as psi (types this harness does not
// build), so the complex-RBM pair is instantiated below, for the golden vectors only.
#include "../source/network_functions/KullbackLeibler.cu"

#include <complex>
#include <cstdio>
#include <fstream>
#include <map>
#include <sstream>
#include <string>
#include <vector>

using namespace rbm_on_gpu;
using cplx = std::complex<double>;

namespace rbm_on_gpu {
template double KullbackLeibler::value(const Psi& psi, const Psi& psi_prime, ExactSummation& spin_ensemble);
template double KullbackLeibler::gradient(std::complex<double>* result, const Psi& psi, const Psi& psi_prime,
                                          ExactSummation& spin_ensemble, const double nu);
}  // namespace rbm_on_gpu

static std::string g_dir;
static std::map<std::string, std::string> g_meta;

template <typename T>
static std::vector<T> load(const std::string& name) {
    std::ifstream f(g_dir + "/" + name, std::ios::binary | std::ios::ate);
    if (!f) { fprintf(stderr, "missing %s\n", name.c_str()); exit(2); }
    const auto bytes = static_cast<size_t>(f.tellg());
    std::vector<T> v(bytes / sizeof(T));
    f.seekg(0);
    f.read(reinterpret_cast<char*>(v.data()), bytes);
    return v;
}

template <typename T>
static void save(const std::string& name, const T* data, size_t n) {
    std::ofstream f(g_dir + "/out_" + name + ".bin", std::ios::binary);
    f.write(reinterpret_cast<const char*>(data), n * sizeof(T));
}

static std::ofstream g_scalars;
static void scalar(const std::string& k, double v) {
    char buf[64];
    snprintf(buf, sizeof(buf), "%.17g", v);
    g_scalars << k << " " << buf << "\n";
}

static long meta_i(const std::string& k, long def = 0) { return g_meta.count(k) ? std::stol(g_meta[k]) : def; }
static double meta_d(const std::string& k, double def = 0) { return g_meta.count(k) ? std::stod(g_meta[k]) : def; }

template <typename T, size_t D>
static xt::pytensor<T, D> tensor(std::vector<T> v, std::array<long, D> shape) {
    return xt::pytensor<T, D>(shape, std::move(v));
}

static Operator load_operator(const std::string& prefix) {
    const auto coef = load<cplx>(prefix + "coef.bin");
    const auto types = load<int>(prefix + "types.bin");
    const auto idx = load<int>(prefix + "idx.bin");
    const long S = static_cast<long>(coef.size());
    const long L = static_cast<long>(types.size()) / S;
    return Operator(tensor<cplx, 1>(coef, {S}), tensor<int, 2>(types, {S, L}), tensor<int, 2>(idx, {S, L}), false);
}

// the alpha angles of a free-quantum-axis case (meta fqa = 1), zeros otherwise
static std::vector<double> load_alpha(const std::string& prefix, long N) {
    return meta_i("fqa", 0) ? load<double>(prefix + "alpha.bin") : std::vector<double>(N, 0.0);
}

static Psi load_rbm(const std::string& prefix, long N, long M) {
    const auto alpha = load_alpha(prefix, N);
    return Psi(tensor<double, 1>(alpha, {N}), tensor<double, 1>(alpha, {N}),
               tensor<cplx, 1>(load<cplx>(prefix + "b.bin"), {M}),
               tensor<cplx, 2>(load<cplx>(prefix + "W.bin"), {N, M}), meta_d("prefactor", 1.0),
               meta_i("fqa", 0) != 0, false);
}

template <typename Deep>
static Deep load_deep(const std::string& prefix, long N) {
    const long L = meta_i("layers");
    std::vector<xt::pytensor<cplx, 1>> b;
    std::vector<xt::pytensor<unsigned, 2>> conn;
    std::vector<xt::pytensor<cplx, 2>> W;
    for (long l = 0; l < L; l++) {
        const long size = meta_i("size" + std::to_string(l));
        const long c = meta_i("conn" + std::to_string(l));
        b.push_back(tensor<cplx, 1>(load<cplx>(prefix + "b" + std::to_string(l) + ".bin"), {size}));
        conn.push_back(tensor<unsigned, 2>(load<unsigned>(prefix + "conn" + std::to_string(l) + ".bin"), {c, size}));
        W.push_back(tensor<cplx, 2>(load<cplx>(prefix + "W" + std::to_string(l) + ".bin"), {c, size}));
    }
    const long last = meta_i("size" + std::to_string(L - 1));
    const auto alpha = load_alpha(prefix, N);
    return Deep(tensor<double, 1>(alpha, {N}), tensor<double, 1>(alpha, {N}), b, conn, W,
                tensor<cplx, 1>(load<cplx>(prefix + "fw.bin"), {last}), meta_d("prefactor", 1.0),
                meta_i("fqa", 0) != 0, false);
}

template <typename P>
static void exact_outputs(P& psi, P& psi_prime, const Operator& op, long N, long num_params) {
    ExactSummation es(static_cast<unsigned>(N), false);
    scalar("norm", psi_norm(psi, es));
    std::vector<cplx> vec(1ul << N);
    psi_vector(vec.data(), psi);
    save("vector", vec.data(), vec.size());

    ExpectationValue ev(false);
    const cplx E = ev(psi, op, es);
    scalar("E_re", E.real());
    scalar("E_im", E.imag());
    const auto fl = ev.fluctuation(psi, op, es);
    scalar("sigma", fl.first);
    std::vector<cplx> grad(num_params);
    const cplx E2 = ev.gradient(grad.data(), psi, op, es);
    scalar("gradE_re", E2.real());
    scalar("gradE_im", E2.imag());
    save("gradient", grad.data(), grad.size());

    HilbertSpaceDistance hsd(static_cast<unsigned>(N), static_cast<unsigned>(num_params), false);
    const auto hop = load_operator("hop_");
    const bool unitary = meta_i("hsd_unitary", 1) != 0;
    const float nu = static_cast<float>(meta_d("hsd_nu", 1.0));
    scalar("hsd_distance", hsd.distance(psi, psi_prime, hop, unitary, es));
    std::vector<cplx> hgrad(num_params);
    scalar("hsd_grad_distance", hsd.gradient(hgrad.data(), psi, psi_prime, hop, unitary, es, nu));
    save("hsd_gradient", hgrad.data(), hgrad.size());
}

template <typename P>
static void ok_vectors(P& psi, long num_params) {
    const auto configs = load<unsigned long long>("ok_spins.bin");
    std::vector<cplx> all;
    for (auto c : configs) {
        std::vector<cplx> ok(num_params, cplx(0.0, 0.0));
        psi_O_k_vector(ok.data(), psi, Spins(c, static_cast<unsigned>(meta_i("N"))));
        // entries [0, 2N) are left unwritten by the reference; report them as zero
        for (long k = 0; k < 2 * meta_i("N"); k++) ok[k] = 0.0;
        all.insert(all.end(), ok.begin(), ok.end());
    }
    save("ok_vectors", all.data(), all.size());
}

template <typename P>
static void mc_outputs(P& psi, const Operator& op, long N, long num_params) {
    const unsigned samples = static_cast<unsigned>(meta_i("mc_samples"));
    const unsigned sweeps = static_cast<unsigned>(meta_i("mc_sweeps", 1));
    const unsigned therm = static_cast<unsigned>(meta_i("mc_therm", 0));
    {
        MonteCarloLoop mc(samples, sweeps, therm, 1, false);
        std::vector<unsigned long long> spins(samples);
        std::vector<double> logpsi(2 * samples);
        auto* sp = spins.data();
        auto* lp = logpsi.data();
        mc.foreach(psi, [=] __host__ __device__ (const unsigned idx, const Spins s, const complex_t log_psi,
                                                 const typename P::Angles&, const double) {
            sp[idx] = s.configuration();
            lp[2 * idx] = log_psi.real();
            lp[2 * idx + 1] = log_psi.imag();
        });
        save("mc_spins", spins.data(), spins.size());
        save("mc_logpsi", logpsi.data(), logpsi.size());
        scalar("mc_accept", mc.acceptances_ar.front());
        scalar("mc_reject", mc.rejections_ar.front());
    }
    {
        MonteCarloLoop mc(samples, sweeps, therm, 1, false);
        ExpectationValue ev(false);
        const cplx E = ev(psi, op, mc);
        scalar("mc_E_re", E.real());
        scalar("mc_E_im", E.imag());
    }
    if (meta_i("mc_gradient", 0)) {
        MonteCarloLoop mc(samples, sweeps, therm, 1, false);
        ExpectationValue ev(false);
        std::vector<cplx> grad(num_params);
        const cplx E = ev.gradient(grad.data(), psi, op, mc);
        scalar("mc_gradE_re", E.real());
        scalar("mc_gradE_im", E.imag());
        save("mc_gradient", grad.data(), grad.size());
    }
}

int main(int argc, char** argv) {
    if (argc < 2) { fprintf(stderr, "usage: %s <case_dir>\n", argv[0]); return 2; }
    g_dir = argv[1];
    {
        std::ifstream f(g_dir + "/meta.txt");
        std::string k, v;
        while (f >> k >> v) g_meta[k] = v;
    }
    g_scalars.open(g_dir + "/out_scalars.txt");
    const std::string kind = g_meta["kind"];
    const long N = meta_i("N");
    const Operator op = load_operator("op_");

    if (kind == "rbm") {
        const long M = meta_i("M");
        Psi psi = load_rbm("", N, M);
        const long P = psi.num_params;
        if (meta_i("normalize", 0)) {
            ExactSummation es(static_cast<unsigned>(N), false);
            psi.prefactor /= psi_norm(psi, es);
            scalar("prefactor", psi.prefactor);
        }
        if (meta_i("exact", 0)) {
            Psi psi_prime = load_rbm("pp_", N, M);
            exact_outputs(psi, psi_prime, op, N, P);
        }
        if (meta_i("ok", 0)) ok_vectors(psi, P);
        if (meta_i("mc_samples", 0)) mc_outputs(psi, op, N, P);
        if (meta_i("ev_extra", 0)) {
            // ExpectationValue::fluctuation_gradient, the operator-list call and difference
            // (source/network_functions/ExpectationValue.cu:258-348, 350-446, 448-518)
            Psi psi_prime = load_rbm("pp_", N, M);
            const auto hop = load_operator("hop_");
            ExactSummation es(static_cast<unsigned>(N), false);
            ExpectationValue ev(false);
            std::vector<cplx> fg(P);
            ev.fluctuation_gradient(fg.data(), psi, op, es);
            save("fluct_gradient", fg.data(), fg.size());
            const auto vals = ev(psi, std::vector<Operator>{op, hop}, es);
            save("ev_list", vals.data(), vals.size());
            const auto diff = ev.difference(psi, psi_prime, std::vector<Operator>{op, hop}, es);
            save("ev_difference", diff.data(), diff.size());
        }
        if (meta_i("kl", 0)) {
            // KullbackLeibler value / gradient (source/network_functions/KullbackLeibler.cu:91-137)
            Psi psi_prime = load_rbm("pp_", N, M);
            ExactSummation es(static_cast<unsigned>(N), false);
            KullbackLeibler kl(static_cast<unsigned>(P), false);
            scalar("kl_value", kl.value(psi, psi_prime, es));
            std::vector<cplx> g(P);
            scalar("kl_grad_value", kl.gradient(g.data(), psi, psi_prime, es, meta_d("hsd_nu", 1.0)));
            save("kl_gradient", g.data(), g.size());
        }
        if (meta_i("smatrix", 0)) {
            // get_S_matrix (source/network_functions/S_matrix.cu:10-53), ExactSummation
            ExactSummation es(static_cast<unsigned>(N), false);
            auto S = get_S_matrix(psi, es);
            std::vector<cplx> out(static_cast<size_t>(P) * P);
            for (size_t q = 0; q < out.size(); q++) out[q] = cplx(S[q].real(), S[q].imag());
            save("smatrix", out.data(), out.size());
        }
        // activation function samples
        const auto z = load<cplx>("act_in.bin");
        std::vector<cplx> lc(z.size()), th(z.size());
        for (size_t i = 0; i < z.size(); i++) {
            lc[i] = my_logcosh(complex_t(z[i].real(), z[i].imag())).to_std();
            th[i] = my_tanh(complex_t(z[i].real(), z[i].imag())).to_std();
        }
        save("logcosh", lc.data(), lc.size());
        save("tanh", th.data(), th.size());
    } else if (kind == "deep") {
        PsiDeep psi = load_deep<PsiDeep>("", N);
        PsiDeep psi_prime = load_deep<PsiDeep>("pp_", N);
        const long P = psi.num_params;
        if (meta_i("normalize", 0)) {
            ExactSummation es(static_cast<unsigned>(N), false);
            psi.prefactor = 1.0;
            psi.prefactor /= psi_norm(psi, es);
            scalar("prefactor", psi.prefactor);
        }
        if (meta_i("exact", 0)) exact_outputs(psi, psi_prime, op, N, P);
        if (meta_i("ok", 0)) ok_vectors(psi, P);
        if (meta_i("mc_samples", 0)) mc_outputs(psi, op, N, P);
        if (meta_i("ev_extra", 0)) {
            // ExpectationValue::fluctuation_gradient, the operator-list call and corrected
            // (source/network_functions/ExpectationValue.cu:258-348, 448-518, 76-127)
            const auto hop = load_operator("hop_");
            ExactSummation es(static_cast<unsigned>(N), false);
            ExpectationValue ev(false);
            std::vector<cplx> fg(P);
            ev.fluctuation_gradient(fg.data(), psi, op, es);
            save("fluct_gradient", fg.data(), fg.size());
            const auto vals = ev(psi, std::vector<Operator>{op, hop}, es);
            save("ev_list", vals.data(), vals.size());
            const auto cr = ev.corrected(psi, op, hop, es);
            scalar("corrected_re", cr.first.real());
            scalar("corrected_im", cr.first.imag());
            scalar("corrected_abs2", cr.second);
        }
        if (meta_i("hsd2", 0)) {
            // HilbertSpaceDistance::distance_2nd_order (HilbertSpaceDistance_2nd_order.cu:69-95)
            const auto op_a = load_operator("h2a_");
            const auto op_b = load_operator("h2b_");
            ExactSummation es(static_cast<unsigned>(N), false);
            HilbertSpaceDistance hsd(static_cast<unsigned>(N), static_cast<unsigned>(P), false);
            scalar("hsd2_distance", hsd.distance_2nd_order(psi, psi_prime, op_a, op_b, es));
        }
        if (meta_i("diag_density", 0)) {
            // DiagDensityOp::operator() (source/network_functions/DiagDensityOp.cu:12-50)
            const unsigned na = static_cast<unsigned>(meta_i("diag_density"));
            ExactSummation es(static_cast<unsigned>(N), false);
            DiagDensityOp dd(na, false);
            dd(psi, op, es);
            std::vector<double> v(1u << na);
            for (size_t q = 0; q < v.size(); q++) v[q] = dd.diag_densities_ar[q];
            save("diag_density", v.data(), v.size());
        }
    } else if (kind == "pair") {
        PsiPair psi = load_deep<PsiPair>("", N);
        PsiPair psi_prime = load_deep<PsiPair>("pp_", N);
        const long P = psi.psi_real.num_params;
        ExactSummation es(static_cast<unsigned>(N), false);
        if (meta_i("normalize", 0)) {
            psi.prefactor /= psi_norm(psi, es);
            psi.update_kernel();
            scalar("prefactor", psi.prefactor);
        }
        scalar("norm", psi_norm(psi, es));
        std::vector<cplx> vec(1ul << N);
        psi_vector(vec.data(), psi);
        save("vector", vec.data(), vec.size());
        ExpectationValue ev(false);
        const cplx E = ev(psi, op, es);
        scalar("E_re", E.real());
        scalar("E_im", E.imag());
        HilbertSpaceDistance hsd(static_cast<unsigned>(N), static_cast<unsigned>(P), false);
        const auto hop = load_operator("hop_");
        const bool unitary = meta_i("hsd_unitary", 1) != 0;
        scalar("hsd_distance", hsd.distance(psi, psi_prime, hop, unitary, es));
        std::vector<cplx> hgrad(P);
        scalar("hsd_grad_distance", hsd.gradient(hgrad.data(), psi, psi_prime, hop, unitary, es, 1.0f));
        save("hsd_gradient", hgrad.data(), hgrad.size());
    } else {
        fprintf(stderr, "unknown kind %s\n", kind.c_str());
        return 2;
    }
    return 0;
}
