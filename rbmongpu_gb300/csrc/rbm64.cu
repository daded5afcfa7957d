// FP64 per-sample pass for the Hilbert-space distance of complex RBMs.
//
// The distance between nearby states is a difference of nearly equal averages
// (d^2 = 1 - |<omega>|^2 / (<norm><ratio>) is ~1e-6 for the perturbed copies the
// reference tests), so the per-sample terms omega_s = exp(conj(log psi'_s - log psi_s)) E_s
// and ratio_s are computed here in FP64, from FP64 copies of the parameters,
// with log psi' - log psi summed angle by angle as differences.  One warp per sample,
// angles and activations of the warp's sample in shared memory.
#include <cuda_runtime.h>

#include "kernels.h"
#include "rbm64.h"

namespace rbmg {

namespace {

__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
    return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

// include/quantum_state/psi_functions.hpp:49-57 in FP64
__device__ __forceinline__ double2 lc64(double2 z) {
    const double s = z.x > 0.0 ? 1.0 : -1.0;
    double2 t = make_double2(s * 3.746646023906276 + z.x, z.y);
    t = cmul(z, t);
    t.x += 7.771429504240965;
    t = cmul(z, t);
    t.x += s * 10.2180213465;
    t = cmul(z, t);
    t.x += 9.19376335670885;
    const double2 num = make_double2(5.49914721954 - s * 2.16564366435 * z.x, -s * 2.16564366435 * z.y);
    const double den = t.x * t.x + t.y * t.y;
    const double qr = (num.x * t.x + num.y * t.y) / den, qi = (num.y * t.x - num.x * t.y) / den;
    return make_double2(s * 0.9003320053750442 * z.x + qr - 0.598139, s * 0.9003320053750442 * z.y + qi);
}

__device__ __forceinline__ double2 warp_sum64(double2 v) {
#pragma unroll
    for (int off = 16; off >= 1; off >>= 1) {
        v.x += __shfl_xor_sync(0xffffffffu, v.x, off);
        v.y += __shfl_xor_sync(0xffffffffu, v.y, off);
    }
    return v;
}

__device__ __forceinline__ bool spin_up(const uint64_t* s, int i) { return (s[i >> 6] >> (i & 63)) & 1ull; }

// shared memory per warp: theta[M], f[M] (double2 each).  op.S = 0 skips the local
// energy and PP.W = null skips log psi'; with both it is the FP64 log psi pass that the
// exact-summation weights and the psi vector use.
__global__ void rbm_hsd64_kernel(Rbm64 P, Rbm64 PP, OpDev op, Hsd64Launch L) {
    extern __shared__ double2 smem[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const long t = static_cast<long>(blockIdx.x) * kWarpsPerBlock + warp;
    if (t >= L.count) return;
    const int M = P.M, N = P.N;
    double2* th = smem + static_cast<long>(warp) * 2 * M;
    double2* f = th + M;
    uint64_t s[kMaxWords] = {0, 0, 0, 0};
    const int nw = (N + 63) / 64;
    if (L.enumerate) {
        const uint64_t idx = L.enum_base + static_cast<uint64_t>(t);
        s[0] = N >= 64 ? idx : (idx & ((1ull << N) - 1ull));
    } else {
        for (int k = 0; k < nw; k++) s[k] = L.spins[t * nw + k];
    }
    double2 lp = make_double2(0.0, 0.0);
    for (int j = lane; j < M; j += 32) {
        double2 a = P.b[j];
        for (int i = 0; i < N; i++) {
            const double2 w = P.W[static_cast<long>(i) * M + j];
            if (spin_up(s, i)) { a.x += w.x; a.y += w.y; }
            else { a.x -= w.x; a.y -= w.y; }
        }
        th[j] = a;
        f[j] = lc64(a);
        lp.x += f[j].x;
        lp.y += f[j].y;
    }
    lp = warp_sum64(lp);
    __syncwarp();
    // local energy (include/operator/Operator.hpp:90-115) with per-angle differences
    double er = 0.0, ei = 0.0;
    for (int n = 0; n < op.S; n++) {
        int parity = 0;
        for (int k = 0; k < nw; k++) parity += __popcll(op.zmask[n * kMaxWords + k] & ~s[k]);
        const double sg = (parity & 1) ? -1.0 : 1.0;
        const double2 c0 = op.coef[n];
        const int yp = op.ypow[n] & 3;
        double2 cf = yp == 0 ? c0 : (yp == 1 ? make_double2(c0.y, -c0.x) : (yp == 2 ? make_double2(-c0.x, -c0.y)
                                                                                  : make_double2(-c0.y, c0.x)));
        cf.x *= sg;
        cf.y *= sg;
        const int nf = op.nflip[n];
        if (nf == 0) {
            er += cf.x;
            ei += cf.y;
            continue;
        }
        const int off = op.flip_off[n];
        double2 d = make_double2(0.0, 0.0);
        for (int j = lane; j < M; j += 32) {
            double2 a = th[j];
            for (int q = 0; q < nf; q++) {
                const int site = op.flip_sites[off + q];
                const double2 w = P.W[static_cast<long>(site) * M + j];
                const double two_s = spin_up(s, site) ? -2.0 : 2.0;
                a.x += two_s * w.x;
                a.y += two_s * w.y;
            }
            const double2 g = lc64(a);
            d.x += g.x - f[j].x;
            d.y += g.y - f[j].y;
        }
        d = warp_sum64(d);
        const double m = exp(d.x);
        const double2 x = make_double2(m * cos(d.y), m * sin(d.y));
        er += cf.x * x.x - cf.y * x.y;
        ei += cf.x * x.y + cf.y * x.x;
    }
    // log psi'(s) - log psi(s), angle by angle
    double2 dl = make_double2(0.0, 0.0);
    for (int j = lane; PP.W && j < M; j += 32) {
        double2 a = PP.b[j];
        for (int i = 0; i < N; i++) {
            const double2 w = PP.W[static_cast<long>(i) * M + j];
            if (spin_up(s, i)) { a.x += w.x; a.y += w.y; }
            else { a.x -= w.x; a.y -= w.y; }
        }
        const double2 g = lc64(a);
        dl.x += g.x - f[j].x;
        dl.y += g.y - f[j].y;
    }
    dl = warp_sum64(dl);
    if (lane == 0) {
        if (L.eloc) L.eloc[t] = make_double2(er, ei);
        if (L.logpsi) L.logpsi[t] = lp;
        if (L.dlogpsi) L.dlogpsi[t] = dl;
    }
}

__global__ void hsd_terms64_kernel(int count, const double2* __restrict__ eloc, const double2* __restrict__ dl,
                                   int is_unitary, double2* omega, double2* pr, double2* nn) {
    for (long s = blockIdx.x * 256L + threadIdx.x; s < count; s += static_cast<long>(gridDim.x) * 256) {
        const double2 e = eloc[s];
        const double dr = dl[s].x, di = -dl[s].y;   // conj(log psi' - log psi)
        double2 om;
        double n;
        if (is_unitary) {   // source/network_functions/HilbertSpaceDistance.cu:88-94
            const double m = exp(dr);
            const double ar = m * cos(di), ai = m * sin(di);
            om = make_double2(ar * e.x - ai * e.y, ar * e.y + ai * e.x);
            n = e.x * e.x + e.y * e.y;
        } else {            // :95-101
            const double m = exp(e.x + dr);
            om = make_double2(m * cos(e.y + di), m * sin(e.y + di));
            n = exp(2.0 * e.x);
        }
        omega[s] = om;
        pr[s] = make_double2(exp(2.0 * dl[s].x), 0.0);   // :102
        nn[s] = make_double2(n, 0.0);
    }
}

// per-sample gradient coefficients w_s * B_s (see capi.cu, rbmg_hsd_gradient)
__global__ void hsd_coef_kernel(int count, const double* __restrict__ w, const double2* __restrict__ omega,
                                const double2* __restrict__ pr, double2 conj_omega_bar, double v, double u,
                                double nn_bar, int mode, double scale, double2* c) {
    for (long s = blockIdx.x * 256L + threadIdx.x; s < count; s += static_cast<long>(gridDim.x) * 256) {
        const double ws = w ? w[s] : 1.0;
        const double2 om = omega[s];
        const double2 a = cmul(conj_omega_bar, om);
        double2 r;
        if (mode == 2) {
            r = make_double2(a.y, 0.0);                                  // Im(conj(<omega>) omega_s)
        } else {
            r = make_double2(a.x * v - u * nn_bar * pr[s].x, a.y * v);   // B_s
            if (mode == 1) r.y = 0.0;                                     // Re B_s
        }
        c[s] = make_double2(scale * ws * r.x, scale * ws * r.y);
    }
}

__device__ __forceinline__ double spin_of(const uint64_t* spins, uint64_t enum_base, int enumerate, long t, int N,
                                          int i) {
    const int nw = (N + 63) / 64;
    const uint64_t word = enumerate ? ((i >> 6) == 0 ? enum_base + static_cast<uint64_t>(t) : 0ull)
                                    : spins[t * nw + (i >> 6)];
    return ((word >> (i & 63)) & 1ull) ? 1.0 : -1.0;
}

__global__ void flip_each_kernel(int count, int N, const uint64_t* spins, uint64_t enum_base, int enumerate,
                                 uint64_t* out) {
    const int nw = (N + 63) / 64;
    const long total = static_cast<long>(count) * N;
    for (long q = blockIdx.x * 256L + threadIdx.x; q < total; q += static_cast<long>(gridDim.x) * 256) {
        const long t = q / N;
        const int i = static_cast<int>(q - t * N);
        for (int k = 0; k < nw; k++) {
            uint64_t w = enumerate ? (k == 0 ? enum_base + static_cast<uint64_t>(t) : 0ull) : spins[t * nw + k];
            if ((i >> 6) == k) w ^= 1ull << (i & 63);
            out[q * nw + k] = w;
        }
    }
}

__global__ void fqa_terms_kernel(int count, int N, const uint64_t* spins, uint64_t enum_base, int enumerate,
                                 const double2* lp, const double2* lpf, const double* qa, double2* dl, double2* r) {
    for (long t = blockIdx.x * 256L + threadIdx.x; t < count; t += static_cast<long>(gridDim.x) * 256) {
        const double2 l0 = lp[t];
        double cx = 0.0, cy = 0.0;
        for (int i = 0; i < N; i++) {
            const double2 li = lpf[t * N + i];
            const double m = exp(li.x - l0.x);
            const double rx = m * cos(li.y - l0.y), ry = m * sin(li.y - l0.y);
            if (r) r[t * N + i] = make_double2(rx, ry);
            const double sg = spin_of(spins, enum_base, enumerate, t, N, i);
            const double da = qa[i], db = qa[N + i], cs = qa[2 * N + i], sn = qa[3 * N + i];
            // da s_i r_i + i db (r_i cos - s_i sin)
            cx += da * sg * rx - db * (ry * cs);
            cy += da * sg * ry + db * (rx * cs - sg * sn);
        }
        dl[t] = make_double2(dl[t].x + cx, dl[t].y + cy);
    }
}

// one block per angle k (alpha_i: k = i, beta_i: k = N + i)
__global__ void fqa_grad_kernel(int count, int N, const uint64_t* spins, uint64_t enum_base, int enumerate,
                                const double2* c, const double2* r, const double* qa, double2* out) {
    __shared__ double2 red[256];
    const int k = blockIdx.x, i = k % N;
    const bool beta = k >= N;
    double ax = 0.0, ay = 0.0;
    for (long t = threadIdx.x; t < count; t += 256) {
        const double2 rv = r[t * N + i];
        const double sg = spin_of(spins, enum_base, enumerate, t, N, i);
        double ox, oy;
        if (beta) {   // i (r cos - s sin)
            ox = -(rv.y * qa[2 * N + i]);
            oy = rv.x * qa[2 * N + i] - sg * qa[3 * N + i];
        } else {      // s r
            ox = sg * rv.x;
            oy = sg * rv.y;
        }
        const double2 cv = c[t];
        // c conj(O)
        ax += cv.x * ox + cv.y * oy;
        ay += cv.y * ox - cv.x * oy;
    }
    red[threadIdx.x] = make_double2(ax, ay);
    __syncthreads();
    for (int h = 128; h >= 1; h >>= 1) {
        if (threadIdx.x < h)
            red[threadIdx.x] = make_double2(red[threadIdx.x].x + red[threadIdx.x + h].x,
                                            red[threadIdx.x].y + red[threadIdx.x + h].y);
        __syncthreads();
    }
    if (threadIdx.x == 0) out[k] = red[0];
}

}  // namespace

cudaError_t launch_flip_each(int count, int N, const uint64_t* spins, uint64_t enum_base, int enumerate,
                             uint64_t* out, cudaStream_t st) {
    if (count <= 0) return cudaSuccess;
    const long total = static_cast<long>(count) * N;
    flip_each_kernel<<<static_cast<int>(std::min(4096L, (total + 255) / 256)), 256, 0, st>>>(count, N, spins, enum_base,
                                                                                           enumerate, out);
    return cudaGetLastError();
}

cudaError_t launch_fqa_terms(int count, int N, const uint64_t* spins, uint64_t enum_base, int enumerate,
                             const double2* lp, const double2* lpf, const double* qa, double2* dl, double2* r,
                             cudaStream_t st) {
    if (count <= 0) return cudaSuccess;
    fqa_terms_kernel<<<static_cast<int>(std::min(1024L, (count + 255L) / 256)), 256, 0, st>>>(
        count, N, spins, enum_base, enumerate, lp, lpf, qa, dl, r);
    return cudaGetLastError();
}

cudaError_t launch_fqa_grad(int count, int N, const uint64_t* spins, uint64_t enum_base, int enumerate,
                            const double2* c, const double2* r, const double* qa, double2* out, cudaStream_t st) {
    if (count <= 0) return cudaSuccess;
    fqa_grad_kernel<<<2 * N, 256, 0, st>>>(count, N, spins, enum_base, enumerate, c, r, qa, out);
    return cudaGetLastError();
}

cudaError_t launch_rbm_hsd64(const Rbm64& P, const Rbm64& PP, const OpDev& op, const Hsd64Launch& L,
                             cudaStream_t st) {
    if (L.count <= 0) return cudaSuccess;
    const size_t smem = sizeof(double2) * 2 * P.M * kWarpsPerBlock;
    if (smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(rbm_hsd64_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             static_cast<int>(smem));
        if (e != cudaSuccess) return e;
    }
    rbm_hsd64_kernel<<<(L.count + kWarpsPerBlock - 1) / kWarpsPerBlock, 32 * kWarpsPerBlock, smem, st>>>(P, PP, op, L);
    return cudaGetLastError();
}

// second order (HilbertSpaceDistance_2nd_order.cu:44-60): x = E1 + (E2 - E1^2) / 2,
// omega = exp(x + conj(log psi' - log psi)), norm = exp(2 Re x), ratio = exp(2 Re(log psi' - log psi))
__global__ void hsd2_terms64_kernel(int count, const double2* __restrict__ e1, const double2* __restrict__ e2,
                                    const double2* __restrict__ dl, double2* omega, double2* pr, double2* nn) {
    for (long s = blockIdx.x * 256L + threadIdx.x; s < count; s += static_cast<long>(gridDim.x) * 256) {
        const double2 a = e1[s], b = e2[s];
        const double xr = a.x + 0.5 * (b.x - (a.x * a.x - a.y * a.y));
        const double xi = a.y + 0.5 * (b.y - 2.0 * a.x * a.y);
        const double m = exp(xr + dl[s].x);
        const double ph = xi - dl[s].y;
        omega[s] = make_double2(m * cos(ph), m * sin(ph));
        nn[s] = make_double2(exp(2.0 * xr), 0.0);
        pr[s] = make_double2(exp(2.0 * dl[s].x), 0.0);
    }
}

cudaError_t launch_hsd2_terms64(int count, const double2* e1, const double2* e2, const double2* dl, double2* omega,
                                double2* pr, double2* nn, cudaStream_t st) {
    if (count <= 0) return cudaSuccess;
    const int blocks = std::min((count + 255) / 256, 4096);
    hsd2_terms64_kernel<<<blocks, 256, 0, st>>>(count, e1, e2, dl, omega, pr, nn);
    return cudaGetLastError();
}

cudaError_t launch_hsd_terms64(int count, const double2* eloc, const double2* dl, int is_unitary, double2* omega,
                               double2* pr, double2* nn, cudaStream_t st) {
    if (count <= 0) return cudaSuccess;
    hsd_terms64_kernel<<<static_cast<int>(std::min(1024L, (count + 255L) / 256)), 256, 0, st>>>(
        count, eloc, dl, is_unitary, omega, pr, nn);
    return cudaGetLastError();
}

cudaError_t launch_hsd_coef(int count, const double* w, const double2* omega, const double2* pr,
                            double2 conj_omega_bar, double v, double u, double nn_bar, int mode, double scale,
                            double2* c, cudaStream_t st) {
    if (count <= 0) return cudaSuccess;
    hsd_coef_kernel<<<static_cast<int>(std::min(1024L, (count + 255L) / 256)), 256, 0, st>>>(
        count, w, omega, pr, conj_omega_bar, v, u, nn_bar, mode, scale, c);
    return cudaGetLastError();
}

}  // namespace rbmg
