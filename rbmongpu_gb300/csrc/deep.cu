// PsiDeep / PsiPair kernels (include/quantum_state/PsiDeep.hpp:89-293, PsiPair.hpp:36-119).
//
// One CTA per configuration: thread j owns unit j of the layer being evaluated;
// the estimator kernels (local energies, O_k and E_k rows) run in FP64 -- for these
// nets log psi(s') - log psi(s) is the difference of two full forward passes, so FP32
// would cost ~1e-7 |log psi| per local-energy term -- while the Metropolis sampler runs
// in FP32;
// the layer's inputs, angles and activations live in shared memory; weights are read
// coalesced over j ([connectivity][size] layout, as the reference stores them).
// The backward pass gathers over the rhs connection lists compiled on the host in
// the reference's order (source/quantum_state/PsiDeep.cu:85-117).
#include <cstdlib>
#include <algorithm>
#include <functional>
#include <memory>

#include "device_math.cuh"
#include "host.h"
#include "reduce.h"

namespace rbmg {

struct Chunk {
    int count = 0;
    const uint64_t* spins = nullptr;
    int enumerate = 0;
    uint64_t enum_base = 0;
    const double* weights = nullptr;
    const double2* eloc = nullptr;
};

namespace {

// ---------------------------------------------------------------- complex helpers
__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double2 cadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
    return make_float2(fmaf(a.x, b.x, -a.y * b.y), fmaf(a.x, b.y, a.y * b.x));
}
__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
    return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
template <typename V> __device__ __forceinline__ V czero();
template <> __device__ __forceinline__ float2 czero<float2>() { return make_float2(0.f, 0.f); }
template <> __device__ __forceinline__ double2 czero<double2>() { return make_double2(0.0, 0.0); }
template <typename V> __device__ __forceinline__ V creal(double x);
template <> __device__ __forceinline__ float2 creal<float2>(double x) { return make_float2(float(x), 0.f); }
template <> __device__ __forceinline__ double2 creal<double2>(double x) { return make_double2(x, 0.0); }

__device__ __forceinline__ double2 lc64(double2 z) {
    const double s = z.x > 0.0 ? 1.0 : -1.0;
    double2 t = make_double2(s * 3.746646023906276 + z.x, z.y);
    t = cmul(z, t); t.x += 7.771429504240965;
    t = cmul(z, t); t.x += s * 10.2180213465;
    t = cmul(z, t); t.x += 9.19376335670885;
    const double2 num = make_double2(5.49914721954 - s * 2.16564366435 * z.x, -s * 2.16564366435 * z.y);
    const double den = t.x * t.x + t.y * t.y;
    return make_double2(s * 0.9003320053750442 * z.x + (num.x * t.x + num.y * t.y) / den - 0.598139,
                        s * 0.9003320053750442 * z.y + (num.y * t.x - num.x * t.y) / den);
}

// activation: the reference's rational log-cosh for complex nets, ReLU for the real
// nets of a PsiPair (include/quantum_state/psi_functions.hpp:118-125)
template <bool REAL> __device__ __forceinline__ float2 act(float2 a) {
    return REAL ? make_float2(a.x > 0.f ? a.x : 0.f, 0.f) : lc_c(a.x, a.y);
}
template <bool REAL> __device__ __forceinline__ double2 act(double2 a) {
    return REAL ? make_double2(a.x > 0.0 ? a.x : 0.0, 0.0) : lc64(a);
}
// derivative: my_tanh for complex nets, 1 for the real nets (psi_functions.hpp:127-136)
template <bool REAL> __device__ __forceinline__ float2 dact(float2 a) {
    return REAL ? make_float2(1.f, 0.f) : tanh_c(a.x, a.y);
}
// my_tanh in FP64 (psi_functions.hpp:97-114)
__device__ __forceinline__ double2 tanh64(double2 z) {
    const double s = z.x > 0.0 ? 1.0 : -1.0;
    const double2 u = make_double2(s * z.x, s * z.y);
    double2 d = make_double2(u.x + 3.746646023906276, u.y);
    d = cmul(u, d); d.x += 7.771429504240965;
    d = cmul(u, d); d.x += 10.218021346543315;
    d = cmul(u, d); d.x += 9.19376335670885;
    double2 q = make_double2(6.746450656267947 + 0.9003320053750442 * u.x, 0.9003320053750442 * u.y);
    q = cmul(u, q); q.x += 26.632014683761202;
    q = cmul(u, q); q.x += 70.82878897882324;
    q = cmul(u, q); q.x += 146.36284300074402;
    q = cmul(u, q); q.x += 199.24474920889975;
    q = cmul(u, q); q.x += 177.6769746361748;
    q = cmul(u, q); q.x += 83.68563506532087;
    q = cmul(u, q);
    const double2 d2 = cmul(d, d);
    const double den = d2.x * d2.x + d2.y * d2.y;
    const double2 h = make_double2((q.x * d2.x + q.y * d2.y) / den, (q.y * d2.x - q.x * d2.y) / den);
    return make_double2(s * h.x, s * h.y);
}
template <bool REAL> __device__ __forceinline__ double2 dact(double2 a) {
    return REAL ? make_double2(1.0, 0.0) : tanh64(a);
}

template <typename V> struct W_of;
template <> struct W_of<float2> {
    static __device__ __forceinline__ const float2* w(const DeepNetDev& n, int l) { return n.w[l]; }
    static __device__ __forceinline__ const float2* b(const DeepNetDev& n, int l) { return n.b[l]; }
    static __device__ __forceinline__ const float2* fw(const DeepNetDev& n) { return n.fw; }
};
template <> struct W_of<double2> {
    static __device__ __forceinline__ const double2* w(const DeepNetDev& n, int l) { return n.w64[l]; }
    static __device__ __forceinline__ const double2* b(const DeepNetDev& n, int l) { return n.b64[l]; }
    static __device__ __forceinline__ const double2* fw(const DeepNetDev& n) { return n.fw64; }
};

// deterministic block sum of one complex value per thread; all threads receive it
template <typename V>
__device__ __forceinline__ V block_sum(V v, V* red) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = (blockDim.x + 31) >> 5;
#pragma unroll
    for (int off = 16; off >= 1; off >>= 1) {
        v.x += __shfl_xor_sync(0xffffffffu, v.x, off);
        v.y += __shfl_xor_sync(0xffffffffu, v.y, off);
    }
    __syncthreads();
    if (lane == 0) red[warp] = v;
    __syncthreads();
    V t = czero<V>();
    for (int q = 0; q < nwarps; q++) t = cadd(t, red[q]);
    return t;
}

__device__ __forceinline__ bool bit_up(const uint64_t* s, int i) { return (s[i >> 6] >> (i & 63)) & 1ull; }

// shared-memory layout of one configuration's evaluation
template <typename V>
struct Work {
    V* in;        // [width]
    V* out;       // [width]
    V* angles;    // [units] or null
    V* acts;      // [units] or null
    V* red;       // [32]
    uint64_t* s;  // [kMaxWords] spins being evaluated
};

// forward pass (PsiDeep.hpp:89-133) of one net on the spins in w.s; returns
// sum_j act_j * final_w_j; with STORE keeps every angle and activation
template <typename V, bool REAL, bool STORE>
__device__ V forward_once(const DeepNetDev& net, const uint64_t* s, Work<V>& w) {
    const int t = threadIdx.x;
    if (t < net.N) w.in[t] = creal<V>(bit_up(s, t) ? 1.0 : -1.0);
    __syncthreads();
    V* in = w.in;
    V* out = w.out;
    for (int l = 0; l < net.L; l++) {
        const int size = net.size[l], conn = net.conn[l];
        if (t < size) {
            const V* wl = W_of<V>::w(net, l);
            const int* ci = net.cidx[l];
            V a = czero<V>();
            for (int c = 0; c < conn; c++) a = cadd(a, cmul(wl[c * size + t], in[ci[c * size + t]]));
            a = cadd(a, W_of<V>::b(net, l)[t]);
            const V y = act<REAL>(a);
            if (STORE) {
                w.angles[net.begin_angle[l] + t] = a;
                w.acts[net.begin_angle[l] + t] = y;
            }
            out[t] = y;
        }
        __syncthreads();
        V* tmp = in;
        in = out;
        out = tmp;
    }
    const int last = net.size[net.L - 1];
    V term = czero<V>();
    if (t < last) term = cmul(in[t], W_of<V>::fw(net)[t]);
    return block_sum(term, w.red);
}

// layer 0's pre-activations of the spins s (the order of forward_once's layer 0)
__device__ void layer0_pre(const DeepNetDev& net, const uint64_t* s, float2* z0) {
    const int size = net.size[0], conn = net.conn[0];
    for (int u = threadIdx.x; u < size; u += blockDim.x) {
        const float2* wl = net.w[0];
        const int* ci = net.cidx[0];
        float2 a = czero<float2>();
        for (int c = 0; c < conn; c++)
            a = cadd(a, cmul(wl[c * size + u], creal<float2>(bit_up(s, ci[c * size + u]) ? 1.0 : -1.0)));
        z0[u] = cadd(a, net.b[0][u]);
    }
}

// forward pass of a complex net from its layer-0 pre-activations z0 (the rest as
// forward_once; with STORE keeps every angle and activation)
template <bool STORE = false>
__device__ float2 forward_from_z0(const DeepNetDev& net, const float2* z0, Work<float2>& w) {
    const int t = threadIdx.x;
    const int size0 = net.size[0];
    for (int u = t; u < size0; u += blockDim.x) {
        const float2 y = act<false>(z0[u]);
        if (STORE) {
            w.angles[net.begin_angle[0] + u] = z0[u];
            w.acts[net.begin_angle[0] + u] = y;
        }
        w.in[u] = y;
    }
    __syncthreads();
    float2* in = w.in;
    float2* out = w.out;
    for (int l = 1; l < net.L; l++) {
        const int size = net.size[l], conn = net.conn[l];
        if (t < size) {
            const float2* wl = net.w[l];
            const int* ci = net.cidx[l];
            float2 a = czero<float2>();
            for (int c = 0; c < conn; c++) a = cadd(a, cmul(wl[c * size + t], in[ci[c * size + t]]));
            a = cadd(a, net.b[l][t]);
            const float2 y = act<false>(a);
            if (STORE) {
                w.angles[net.begin_angle[l] + t] = a;
                w.acts[net.begin_angle[l] + t] = y;
            }
            out[t] = y;
        }
        __syncthreads();
        float2* tmp = in;
        in = out;
        out = tmp;
    }
    const int last = net.size[net.L - 1];
    float2 term = czero<float2>();
    if (t < last) term = cmul(in[t], net.fw[t]);
    return block_sum(term, w.red);
}

// log psi of one net with optional translational averaging (PsiDeep.hpp:135-169)
template <typename V, bool REAL>
__device__ V net_log_psi(const DeepNetDev& net, const uint64_t* s, Work<V>& w, uint64_t* shifted) {
    if (!net.ti) return forward_once<V, REAL, false>(net, s, w);
    V r = czero<V>();
    for (int shift = 0; shift < net.N; shift++) {
        __syncthreads();
        if (threadIdx.x == 0) {   // Spins_t<1>::rotate_left (include/Spins.h:280-285)
            const uint64_t x = s[0];
            uint64_t y = shift == 0 ? x : ((x << shift) | (x >> (net.N - shift)));
            if (net.N < 64) y &= (1ull << net.N) - 1ull;
            shifted[0] = y;
        }
        __syncthreads();
        r = cadd(r, forward_once<V, REAL, false>(net, shifted, w));
    }
    const double inv = 1.0 / net.N;
    r.x *= inv;
    r.y *= inv;
    return r;
}

// log psi of the state: one complex net, or (Re, Im) from the two real nets of a PsiPair
template <typename V>
__device__ V state_log_psi(const DeepNetDev& n0, const DeepNetDev& n1, int pair, const uint64_t* s, Work<V>& w,
                           uint64_t* shifted) {
    if (!pair) return net_log_psi<V, false>(n0, s, w, shifted);
    const V re = net_log_psi<V, true>(n0, s, w, shifted);
    const V im = net_log_psi<V, true>(n1, s, w, shifted);
    V r;
    r.x = re.x;
    r.y = im.x;
    return r;
}

// reverse pass (PsiDeep.hpp:214-293) after forward_once<STORE>; emit(k, value) with k
// counted from the first O_k entry (parameter index - 2N)
template <typename V, bool REAL, typename Emit>
__device__ void backward(const DeepNetDev& net, const uint64_t* s, Work<V>& w, V log_psi, Emit emit) {
    const int t = threadIdx.x;
    const int L = net.L;
    V* cur = w.in;
    V* nxt = w.out;
    for (int l = L - 1; l >= 0; l--) {
        const int size = net.size[l];
        V d = czero<V>();
        if (t < size) {
            const V ang = w.angles[net.begin_angle[l] + t];
            if (l == L - 1) {
                d = cmul(W_of<V>::fw(net)[t], dact<REAL>(ang));
            } else {
                const int nsize = net.size[l + 1];
                V acc = czero<V>();
                const V* wn = W_of<V>::w(net, l + 1);
                for (int e = net.rptr[l][t]; e < net.rptr[l][t + 1]; e++) {
                    const int q = net.rq[l][e];
                    acc = cadd(acc, cmul(wn[q], nxt[q % nsize]));
                }
                d = cmul(acc, dact<REAL>(ang));
            }
        }
        __syncthreads();
        if (t < size) {
            cur[t] = d;
            const int base = net.begin_params[l];
            emit(base + t, d);
            const int conn = net.conn[l];
            for (int c = 0; c < conn; c++) {
                const int src = net.cidx[l][c * size + t];
                const V in = l == 0 ? creal<V>(bit_up(s, src) ? 1.0 : -1.0) : w.acts[net.begin_angle[l - 1] + src];
                emit(base + size + c * size + t, cmul(d, in));
            }
        }
        __syncthreads();
        V* tmp = cur;
        cur = nxt;
        nxt = tmp;
    }
    // final weights: log psi * activation of the last layer (PsiDeep.hpp:285-292)
    const int last = net.size[L - 1];
    if (t < last) emit(net.P - 2 * net.N - last + t, cmul(log_psi, w.acts[net.begin_angle[L - 1] + t]));
    __syncthreads();
}

template <typename V>
__device__ Work<V> carve(void* base, const DeepNetDev& net, bool store) {
    Work<V> w;
    V* p = static_cast<V*>(base);
    const int width = net.width;
    w.red = p;
    p += 32;
    w.in = p;
    p += width;
    w.out = p;
    p += width;
    w.angles = store ? p : nullptr;
    if (store) p += net.units;
    w.acts = store ? p : nullptr;
    if (store) p += net.units;
    w.s = reinterpret_cast<uint64_t*>(p);
    return w;
}

__device__ __forceinline__ void load_config(const uint64_t* spins, uint64_t enum_base, int enumerate, long t, int N,
                                            uint64_t* s) {
    const int nw = (N + 63) / 64;
    if (threadIdx.x < kMaxWords) {
        uint64_t v = 0;
        if (enumerate) {
            if (threadIdx.x == 0) {
                v = enum_base + static_cast<uint64_t>(t);
                if (N < 64) v &= (1ull << N) - 1ull;
            }
        } else if (static_cast<int>(threadIdx.x) < nw) {
            v = spins[t * nw + threadIdx.x];
        }
        s[threadIdx.x] = v;
    }
    __syncthreads();
}

// string n applied to s: flipped configuration into sp, returns coef * phase (Operator.hpp:45-88)
__device__ double2 apply_string(const OpDev& op, int n, const uint64_t* s, uint64_t* sp) {
    int parity = 0;
    for (int k = 0; k < kMaxWords; k++) parity += __popcll(op.zmask[n * kMaxWords + k] & ~s[k]);
    const double sg = (parity & 1) ? -1.0 : 1.0;
    const double2 c = op.coef[n];
    const int yp = op.ypow[n] & 3;
    double2 r = yp == 0 ? c : (yp == 1 ? make_double2(c.y, -c.x) : (yp == 2 ? make_double2(-c.x, -c.y)
                                                                            : make_double2(-c.y, c.x)));
    __syncthreads();
    if (threadIdx.x < kMaxWords) {
        uint64_t v = s[threadIdx.x];
        for (int q = 0; q < op.nflip[n]; q++) {
            const int site = op.flip_sites[op.flip_off[n] + q];
            if ((site >> 6) == static_cast<int>(threadIdx.x)) v ^= 1ull << (site & 63);
        }
        sp[threadIdx.x] = v;
    }
    __syncthreads();
    return make_double2(sg * r.x, sg * r.y);
}

// ---------------------------------------------------------------- kernels
template <typename V>
__global__ void deep_logpsi_kernel(DeepNetDev n0, DeepNetDev n1, int pair, int count, const uint64_t* spins,
                                   uint64_t enum_base, int enumerate, double2* out) {
    extern __shared__ __align__(16) unsigned char smem[];
    Work<V> w = carve<V>(smem, n0, false);
    uint64_t* shifted = w.s + kMaxWords;
    const long t = blockIdx.x;
    if (t >= count) return;
    load_config(spins, enum_base, enumerate, t, n0.N, w.s);
    const V lp = state_log_psi<V>(n0, n1, pair, w.s, w, shifted);
    if (threadIdx.x == 0) out[t] = make_double2(lp.x, lp.y);
}

// local energy (Operator.hpp:90-115); FP32 or FP64 evaluation; with PRIME also
// log psi'(s) - log psi(s) for the Hilbert-space distance
template <typename V, bool PRIME>
__global__ void deep_eloc_kernel(DeepNetDev n0, DeepNetDev n1, int pair, DeepNetDev p0, DeepNetDev p1, OpDev op,
                                 int count, const uint64_t* spins, uint64_t enum_base, int enumerate, double2* eloc,
                                 double2* dlp) {
    extern __shared__ __align__(16) unsigned char smem[];
    Work<V> w = carve<V>(smem, n0.width >= p0.width ? n0 : p0, false);
    uint64_t* sp = w.s + kMaxWords;
    uint64_t* shifted = sp + kMaxWords;
    const long t = blockIdx.x;
    if (t >= count) return;
    load_config(spins, enum_base, enumerate, t, n0.N, w.s);
    const V lp = state_log_psi<V>(n0, n1, pair, w.s, w, shifted);
    double er = 0.0, ei = 0.0;
    for (int n = 0; n < op.S; n++) {
        const double2 cf = apply_string(op, n, w.s, sp);
        if (op.nflip[n] == 0) {
            er += cf.x;
            ei += cf.y;
            continue;
        }
        const V lq = state_log_psi<V>(n0, n1, pair, sp, w, shifted);
        const double dr = static_cast<double>(lq.x) - static_cast<double>(lp.x);
        const double di = static_cast<double>(lq.y) - static_cast<double>(lp.y);
        const double m = exp(dr);
        const double xr = m * cos(di), xi = m * sin(di);
        er += cf.x * xr - cf.y * xi;
        ei += cf.x * xi + cf.y * xr;
    }
    double2 d = make_double2(0.0, 0.0);
    if (PRIME) {
        const V lq = state_log_psi<V>(p0, p1, pair, w.s, w, shifted);
        d = make_double2(static_cast<double>(lq.x) - static_cast<double>(lp.x),
                         static_cast<double>(lq.y) - static_cast<double>(lp.y));
    }
    if (threadIdx.x == 0) {
        if (eloc) eloc[t] = make_double2(er, ei);
        if (PRIME) dlp[t] = d;
    }
}

// O_k rows [count][P - 2N] of one net (complex, or a real PsiPair net stored as (x, 0))
template <bool REAL>
__global__ void deep_ok_kernel(DeepNetDev net, int count, const uint64_t* spins, uint64_t enum_base, int enumerate,
                               double2* rows, long ld) {
    extern __shared__ __align__(16) unsigned char smem[];
    Work<double2> w = carve<double2>(smem, net, true);
    const long t = blockIdx.x;
    if (t >= count) return;
    load_config(spins, enum_base, enumerate, t, net.N, w.s);
    const double2 lp = forward_once<double2, REAL, true>(net, w.s, w);
    double2* row = rows + t * ld;
    backward<double2, REAL>(net, w.s, w, lp, [&](int k, double2 v) { row[k] = v; });
}

// per sample (FP64): E_loc, O_k(s) row, and the centred E_k row
//   Ek[s] = (E_diag - E0) O(s) + sum_{off-diagonal n} e_n O(s'_n)
// (Operator.hpp:145-179 with the shift of the gradient estimator)
__global__ void deep_grad_kernel(DeepNetDev net, OpDev op, int count, const uint64_t* spins, uint64_t enum_base,
                                 int enumerate, double2 e_shift, double2* eloc, double2* Orows, double2* Ekrows,
                                 long ld) {
    extern __shared__ __align__(16) unsigned char smem[];
    Work<double2> w = carve<double2>(smem, net, true);
    uint64_t* sp = w.s + kMaxWords;
    const long t = blockIdx.x;
    if (t >= count) return;
    load_config(spins, enum_base, enumerate, t, net.N, w.s);
    double2* orow = Orows + t * ld;
    double2* erow = Ekrows + t * ld;
    const double2 lp = forward_once<double2, false, true>(net, w.s, w);
    backward<double2, false>(net, w.s, w, lp, [&](int k, double2 v) { orow[k] = v; });
    double dr_ = 0.0, di_ = 0.0;
    for (int n = 0; n < op.S; n++) {
        if (op.nflip[n] != 0) continue;
        const double2 cf = apply_string(op, n, w.s, sp);
        dr_ += cf.x;
        di_ += cf.y;
    }
    double er = dr_, ei = di_;
    {
        const double2 c = make_double2(dr_ - e_shift.x, di_ - e_shift.y);
        const int P = net.P - 2 * net.N;
        for (int k = threadIdx.x; k < P; k += blockDim.x) erow[k] = cmul(c, orow[k]);
    }
    __syncthreads();
    for (int n = 0; n < op.S; n++) {
        if (op.nflip[n] == 0) continue;
        const double2 cf = apply_string(op, n, w.s, sp);
        const double2 lq = forward_once<double2, false, true>(net, sp, w);
        const double dr = lq.x - lp.x, di = lq.y - lp.y;
        const double m = exp(dr);
        const double xr = m * cos(di), xi = m * sin(di);
        const double2 e = make_double2(cf.x * xr - cf.y * xi, cf.x * xi + cf.y * xr);
        er += e.x;
        ei += e.y;
        backward<double2, false>(net, sp, w, lq, [&](int k, double2 v) { erow[k] = cadd(erow[k], cmul(e, v)); });
    }
    if (threadIdx.x == 0) eloc[t] = make_double2(er, ei);
}

// out[k] += sum_s c[s] f(A[s][k]) over count samples, f = conj if conj_a (FP64)
__global__ void col_reduce_kernel(int count, int P, const double2* __restrict__ c, const double2* __restrict__ A,
                                  long ld, int conj_a, double2* __restrict__ partial, int per_split) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    const long s0 = static_cast<long>(blockIdx.y) * per_split;
    const long s1 = min(static_cast<long>(count), s0 + per_split);
    if (k >= P) return;
    double2 acc = make_double2(0.0, 0.0);
    for (long s = s0; s < s1; s++) {
        double2 a = A[s * ld + k];
        if (conj_a) a.y = -a.y;
        acc = cadd(acc, cmul(c[s], a));
    }
    partial[static_cast<long>(blockIdx.y) * P + k] = acc;
}

__global__ void col_finish_kernel(int P, int splits, const double2* __restrict__ partial, double2* out) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= P) return;
    double2 a = make_double2(0.0, 0.0);
    for (int z = 0; z < splits; z++) {
        a.x += partial[static_cast<long>(z) * P + k].x;
        a.y += partial[static_cast<long>(z) * P + k].y;
    }
    out[k].x += a.x;
    out[k].y += a.y;
}

// Metropolis for PsiDeep / PsiPair: one CTA per walker, full forward pass per proposal
// (PsiDeep.hpp:191-194: angles are not updated incrementally; single flips of a complex
// net move layer 0 incrementally here, and run several walkers per CTA in
// deep_mc_multi_kernel).  Fast sweep
// (MonteCarloLoop.hpp:162-171): the proposal flips the AND of fast_tries random
// configurations, N such updates per thermalisation sweep and one per sampling sweep.
__global__ void deep_mc_kernel(DeepNetDev n0, DeepNetDev n1, int pair, McLaunch L) {
    extern __shared__ __align__(16) unsigned char smem[];
    Work<float2> w = carve<float2>(smem, n0, false);
    uint64_t* sp = w.s + kMaxWords;
    uint64_t* shifted = sp + kMaxWords;
    const int walker = blockIdx.x;
    if (walker >= L.B) return;
    const int N = n0.N, nw = (N + 63) / 64;
    WalkerRng rng;
    rng.init(L.seed, L.walker_base + static_cast<uint32_t>(walker), L.rng_index[walker]);
    // every thread draws the same words, so all threads agree without a broadcast
    uint64_t s[kMaxWords] = {0, 0, 0, 0};
    if (L.init) {
        for (int k = 0; k < nw; k++) {
            const uint64_t lo = rng.next();
            const uint64_t hi = rng.next();
            s[k] = lo | (hi << 32);
        }
        if (N / 64 < nw) s[N / 64] &= (1ull << (N % 64)) - 1ull;
    } else {
        for (int k = 0; k < nw; k++) s[k] = L.spins[static_cast<long>(walker) * nw + k];
    }
    if (threadIdx.x < kMaxWords) w.s[threadIdx.x] = s[threadIdx.x];
    __syncthreads();
    float lpr = state_log_psi<float2>(n0, n1, pair, w.s, w, shifted).x;
    // single-flip proposals of a complex net move layer 0's pre-activations by the flipped
    // spin's connections (z0' = z0 - 2 s_i W0[i, :]) and evaluate the later layers only;
    // z0 and log psi are recomputed from the spins at the start of every sweep
    const bool incr = L.fast_tries == 0 && !pair && !n0.ti;
    float2* z0 = reinterpret_cast<float2*>(shifted + kMaxWords);   // [size[0]] the state's
    float2* z0p = z0 + n0.size[0];                                   // [size[0]] a proposal's
    unsigned long long acc = 0, props = 0;
    const int total = L.n_therm + L.n_samples * L.sweeps_per_sample;
    int sample = 0;
    for (int sw = 0; sw < total; sw++) {
        const int updates = (L.fast_tries > 0 && sw >= L.n_therm) ? 1 : N;
        if (incr) {
            __syncthreads();
            layer0_pre(n0, w.s, z0);
            __syncthreads();
            lpr = forward_from_z0(n0, z0, w).x;
        }
        for (int p = 0; p < updates; p++) {
            int site = -1;
            if (L.fast_tries > 0) {
                // every thread draws the same mask words
                uint64_t m[kMaxWords] = {0, 0, 0, 0};
                for (int t = 0; t < L.fast_tries; t++) {
                    for (int k = 0; k < nw; k++) {
                        const uint64_t lo = rng.next();
                        const uint64_t hi = rng.next();
                        const uint64_t v = lo | (hi << 32);
                        m[k] = t == 0 ? v : (m[k] & v);
                    }
                }
                if (N / 64 < nw) m[N / 64] &= (1ull << (N % 64)) - 1ull;
                __syncthreads();
                if (threadIdx.x < kMaxWords) {
                    uint64_t v = w.s[threadIdx.x];
                    for (int k = 0; k < kMaxWords; k++)
                        if (k == static_cast<int>(threadIdx.x)) v ^= m[k];
                    sp[threadIdx.x] = v;
                }
            } else {
                site = static_cast<int>(rng.next() % static_cast<uint32_t>(N));
                __syncthreads();
                if (threadIdx.x < kMaxWords) {
                    uint64_t v = w.s[threadIdx.x];
                    if ((site >> 6) == static_cast<int>(threadIdx.x)) v ^= 1ull << (site & 63);
                    sp[threadIdx.x] = v;
                }
                if (incr)
                    for (int u = threadIdx.x; u < n0.size[0]; u += blockDim.x) z0p[u] = z0[u];
            }
            __syncthreads();
            float nl;
            if (incr && site >= 0) {
                const float two_s = bit_up(w.s, site) ? -2.0f : 2.0f;
                const int size0 = n0.size[0];
                for (int q = n0.sptr[site] + threadIdx.x; q < n0.sptr[site + 1]; q += blockDim.x) {
                    const int e = n0.sq[q];
                    const float2 wv = n0.w[0][e];
                    float2* z = z0p + e % size0;
                    atomicAdd(&z->x, two_s * wv.x);
                    atomicAdd(&z->y, two_s * wv.y);
                }
                __syncthreads();
                nl = forward_from_z0(n0, z0p, w).x;
            } else {
                nl = state_log_psi<float2>(n0, n1, pair, sp, w, shifted).x;
            }
            const float delta = nl - lpr;
            bool accept = delta > 0.0f;
            if (!accept) accept = rng.uniform() <= expf_det(2.0f * delta);
            __syncthreads();
            if (accept) {
                if (threadIdx.x < kMaxWords) w.s[threadIdx.x] = sp[threadIdx.x];
                lpr = nl;
                acc++;
                if (incr && site >= 0) {
                    float2* tz = z0;
                    z0 = z0p;
                    z0p = tz;
                }
            }
            props++;
            __syncthreads();
        }
        const int done = sw + 1 - L.n_therm;
        if (done > 0 && done % L.sweeps_per_sample == 0) {
            const long row = static_cast<long>(L.sample_base + sample) * L.B + walker;
            if (L.sample_spins && threadIdx.x < nw) L.sample_spins[row * nw + threadIdx.x] = w.s[threadIdx.x];
            sample++;
        }
    }
    __syncthreads();
    if (threadIdx.x < nw) L.spins[static_cast<long>(walker) * nw + threadIdx.x] = w.s[threadIdx.x];
    if (threadIdx.x == 0) {
        L.rng_index[walker] = rng.index;
        L.accepts[walker] += acc;
        L.proposals[walker] += props;
    }
}

// The same chains as deep_mc_kernel's incremental path (a complex net, single-flip
// proposals, no pair or translation sums), WPC walkers per CTA: one thread per unit
// evaluates that unit for all WPC walkers, so each weight and connection index read from
// L1 serves WPC independent multiply-add chains.  Walker k's Philox stream is drawn by
// thread k alone (site, uniform, start spins) and published through shared memory; every
// walker's arithmetic is deep_mc_kernel's, in the same order, so spins, accept counts and
// stream positions are identical.
// forward_from_z0 for WPC configurations at once: configuration k's layer-0
// pre-activations are zof(k)[0 .. size[0]); with STORE its angles and activations go to
// angles / acts + k * units
template <int WPC, bool STORE, typename ZOf>
__device__ __forceinline__ void forward_multi(const DeepNetDev& net, ZOf zof, float2* in, float2* out,
                                              float2* angles, float2* acts, float2* red, float2 lp[WPC]) {
    const int t = threadIdx.x;
    const int width = net.width, size0 = net.size[0], units = net.units;
#pragma unroll
    for (int k = 0; k < WPC; k++) {
        const float2* zk = zof(k);
        for (int u = t; u < size0; u += blockDim.x) {
            const float2 y = act<false>(zk[u]);
            if (STORE) {
                angles[k * units + net.begin_angle[0] + u] = zk[u];
                acts[k * units + net.begin_angle[0] + u] = y;
            }
            in[k * width + u] = y;
        }
    }
    __syncthreads();
    for (int l = 1; l < net.L; l++) {
        const int size = net.size[l], conn = net.conn[l];
        if (t < size) {
            const float2* wl = net.w[l];
            const int* ci = net.cidx[l];
            float2 a[WPC];
#pragma unroll
            for (int k = 0; k < WPC; k++) a[k] = czero<float2>();
            for (int c = 0; c < conn; c++) {
                const float2 wv = wl[c * size + t];
                const int i = ci[c * size + t];
#pragma unroll
                for (int k = 0; k < WPC; k++) a[k] = cadd(a[k], cmul(wv, in[k * width + i]));
            }
            const float2 bv = net.b[l][t];
#pragma unroll
            for (int k = 0; k < WPC; k++) {
                const float2 z = cadd(a[k], bv);
                const float2 y = act<false>(z);
                if (STORE) {
                    angles[k * units + net.begin_angle[l] + t] = z;
                    acts[k * units + net.begin_angle[l] + t] = y;
                }
                out[k * width + t] = y;
            }
        }
        __syncthreads();
        float2* tmp = in;
        in = out;
        out = tmp;
    }
    // each configuration's block_sum of its terms, in block_sum's order
    const int last = net.size[net.L - 1];
    const int lane = t & 31, warp = t >> 5, nwarps = (blockDim.x + 31) >> 5;
    float2 v[WPC];
#pragma unroll
    for (int k = 0; k < WPC; k++) {
        v[k] = t < last ? cmul(in[k * width + t], net.fw[t]) : czero<float2>();
#pragma unroll
        for (int off = 16; off >= 1; off >>= 1) {
            v[k].x += __shfl_xor_sync(0xffffffffu, v[k].x, off);
            v[k].y += __shfl_xor_sync(0xffffffffu, v[k].y, off);
        }
    }
    __syncthreads();
    if (lane == 0)
#pragma unroll
        for (int k = 0; k < WPC; k++) red[k * 32 + warp] = v[k];
    __syncthreads();
#pragma unroll
    for (int k = 0; k < WPC; k++) {
        float2 r = czero<float2>();
        for (int q = 0; q < nwarps; q++) r = cadd(r, red[k * 32 + q]);
        lp[k] = r;
    }
}

size_t deep_mc_multi_smem(const DeepNetDev& n, int wpc) {
    return wpc * (sizeof(float2) * (32 + 2 * n.width + 2 * n.size[0]) + sizeof(uint64_t) * kMaxWords +
                  2 * sizeof(int));
}

template <int WPC>
__global__ void deep_mc_multi_kernel(DeepNetDev n0, McLaunch L) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int width = n0.width, size0 = n0.size[0];
    float2* red = reinterpret_cast<float2*>(smem);                     // [WPC][32]
    float2* in = red + WPC * 32;                                       // [WPC][width]
    float2* out = in + WPC * width;                                    // [WPC][width]
    float2* zb = out + WPC * width;                                    // [WPC][2][size0]
    uint64_t* s = reinterpret_cast<uint64_t*>(zb + 2 * WPC * size0);   // [WPC][kMaxWords]
    int* site_sh = reinterpret_cast<int*>(s + WPC * kMaxWords);        // [WPC]
    int* flag_sh = site_sh + WPC;                                      // [WPC]
    const int N = n0.N, nw = (N + 63) / 64;
    const int first = blockIdx.x * WPC;
    const int t = threadIdx.x;
    // thread k < WPC owns walker first + k: its stream, spins updates and counters
    const int mine = first + t;
    const bool owner = t < WPC && mine < L.B;
    WalkerRng rng;
    unsigned long long acc = 0, props = 0;
    if (t < WPC) {
        rng.init(L.seed, L.walker_base + static_cast<uint32_t>(mine), owner ? L.rng_index[mine] : 0);
        uint64_t* sk = s + t * kMaxWords;
        for (int k = 0; k < kMaxWords; k++) sk[k] = 0;
        if (owner) {
            if (L.init) {
                for (int k = 0; k < nw; k++) {
                    const uint64_t lo = rng.next();
                    const uint64_t hi = rng.next();
                    sk[k] = lo | (hi << 32);
                }
                if (N / 64 < nw) sk[N / 64] &= (1ull << (N % 64)) - 1ull;
            } else {
                for (int k = 0; k < nw; k++) sk[k] = L.spins[static_cast<long>(mine) * nw + k];
            }
        }
    }
    float lpr[WPC];
    float2 nl[WPC], lp0[WPC];
    int cur = 0;   // bit k: the half of walker k's layer-0 pair that holds its state
    const int total = L.n_therm + L.n_samples * L.sweeps_per_sample;
    int sample = 0;
    for (int sw = 0; sw < total; sw++) {
        // layer 0 and log psi of every state from its spins
        __syncthreads();
#pragma unroll
        for (int k = 0; k < WPC; k++) layer0_pre(n0, s + k * kMaxWords, zb + (2 * k + ((cur >> k) & 1)) * size0);
        __syncthreads();
        forward_multi<WPC, false>(n0, [&](int k) { return zb + (2 * k + ((cur >> k) & 1)) * size0; }, in, out,
                                  nullptr, nullptr, red, lp0);
#pragma unroll
        for (int k = 0; k < WPC; k++) lpr[k] = lp0[k].x;
        for (int p = 0; p < N; p++) {
            if (owner) site_sh[t] = static_cast<int>(rng.next() % static_cast<uint32_t>(N));
            // a proposal's layer 0: its state's moved by the flipped spin's connections
#pragma unroll
            for (int k = 0; k < WPC; k++) {
                const int h = (cur >> k) & 1;
                const float2* src = zb + (2 * k + h) * size0;
                float2* dst = zb + (2 * k + 1 - h) * size0;
                for (int u = t; u < size0; u += blockDim.x) dst[u] = src[u];
            }
            __syncthreads();
#pragma unroll
            for (int k = 0; k < WPC; k++) {
                if (first + k >= L.B) continue;
                const int site = site_sh[k];
                const float two_s = bit_up(s + k * kMaxWords, site) ? -2.0f : 2.0f;
                float2* dst = zb + (2 * k + 1 - ((cur >> k) & 1)) * size0;
                for (int q = n0.sptr[site] + t; q < n0.sptr[site + 1]; q += blockDim.x) {
                    const int e = n0.sq[q];
                    const float2 wv = n0.w[0][e];
                    float2* zz = dst + e % size0;
                    atomicAdd(&zz->x, two_s * wv.x);
                    atomicAdd(&zz->y, two_s * wv.y);
                }
            }
            __syncthreads();
            forward_multi<WPC, false>(n0, [&](int k) { return zb + (2 * k + 1 - ((cur >> k) & 1)) * size0; }, in,
                                      out, nullptr, nullptr, red, nl);
            if (t < WPC) {
                float mnl = nl[0].x, mlp = lpr[0];
#pragma unroll
                for (int k = 1; k < WPC; k++)
                    if (k == t) {
                        mnl = nl[k].x;
                        mlp = lpr[k];
                    }
                bool accept = false;
                if (owner) {
                    const float delta = mnl - mlp;
                    accept = delta > 0.0f;
                    if (!accept) accept = rng.uniform() <= expf_det(2.0f * delta);
                    if (accept) {
                        const int site = site_sh[t];
                        s[t * kMaxWords + (site >> 6)] ^= 1ull << (site & 63);
                        acc++;
                    }
                    props++;
                }
                flag_sh[t] = accept ? 1 : 0;
            }
            __syncthreads();
#pragma unroll
            for (int k = 0; k < WPC; k++)
                if (flag_sh[k]) {
                    lpr[k] = nl[k].x;
                    cur ^= 1 << k;
                }
        }
        const int done = sw + 1 - L.n_therm;
        if (done > 0 && done % L.sweeps_per_sample == 0) {
            const long row0 = static_cast<long>(L.sample_base + sample) * L.B;
            if (L.sample_spins)
                for (int i = t; i < WPC * nw; i += blockDim.x) {
                    const int k = i / nw, word = i % nw;
                    if (first + k < L.B) L.sample_spins[(row0 + first + k) * nw + word] = s[k * kMaxWords + word];
                }
            sample++;
        }
    }
    __syncthreads();
    for (int i = t; i < WPC * nw; i += blockDim.x) {
        const int k = i / nw, word = i % nw;
        if (first + k < L.B) L.spins[static_cast<long>(first + k) * nw + word] = s[k * kMaxWords + word];
    }
    if (owner) {
        L.rng_index[mine] = rng.index;
        L.accepts[mine] += acc;
        L.proposals[mine] += props;
    }
}

// ---------------------------------------------------------------- adjoint of E_loc
// Extension (no reference counterpart): reverse-mode derivative of the local energy,
//   d E_loc(s) / d theta = sum_n e_n O(s'_n) - E_loc(s) O(s),  e_n = c_n psi(s'_n) / psi(s),
// with O = d log psi / d theta (holomorphic, final weights d log psi / d fw_j = act_j).
// Per configuration x the reverse pass yields the error vector delta_l(x) = d log psi /
// d z_l of every layer; the parameter gradient is then the weighted sum over
// configurations of the outer products delta_l(x) (x) a_{l-1}(x), formed as batched
// reductions over all configurations of a chunk.  Every forward pass is recomputed
// from the spins (no angles are kept per walker between calls).

// delta_l for every layer after forward_once<STORE>; emit(layer, unit, delta)
template <typename V, bool REAL, typename Emit>
__device__ void backward_deltas(const DeepNetDev& net, Work<V>& w, Emit emit) {
    const int t = threadIdx.x;
    const int L = net.L;
    V* cur = w.in;
    V* nxt = w.out;
    for (int l = L - 1; l >= 0; l--) {
        const int size = net.size[l];
        V d = czero<V>();
        if (t < size) {
            const V ang = w.angles[net.begin_angle[l] + t];
            if (l == L - 1) {
                d = cmul(W_of<V>::fw(net)[t], dact<REAL>(ang));
            } else {
                const int nsize = net.size[l + 1];
                V acc = czero<V>();
                const V* wn = W_of<V>::w(net, l + 1);
                for (int e = net.rptr[l][t]; e < net.rptr[l][t + 1]; e++) {
                    const int q = net.rq[l][e];
                    acc = cadd(acc, cmul(wn[q], nxt[q % nsize]));
                }
                d = cmul(acc, dact<REAL>(ang));
            }
        }
        __syncthreads();
        if (t < size) {
            cur[t] = d;
            emit(l, t, d);
        }
        __syncthreads();
        V* tmp = cur;
        cur = nxt;
        nxt = tmp;
    }
}

// One CTA per sample: E_loc(s) (FP32 passes, FP64 sum), then for every configuration x
// of the sample (x = s first, then s'_n for the off-diagonal strings in order) its spins,
// activations and alpha_x * delta_l(x), with alpha_{s'_n} = w_s e_n and
// alpha_s = w_s (-sum_{off-diagonal n} e_n + score * 2 Re E_loc(s)) (diagonal strings leave
// the configuration unchanged and drop out of the derivative).  With score, also
// w_s delta_l(s) and w_s (dltsO, alphaO) for the -2 <Re E> <O*> part of the sampling term.
__global__ void deep_adjoint_kernel(DeepNetDev net, OpDev op, int count, const uint64_t* spins, uint64_t enum_base,
                                    int enumerate, const double* weights, int score, double2* eloc, float2* acts,
                                    float2* dlts, float2* alpha, uint64_t* xspins, int xs, float2* dltsO,
                                    float2* alphaO) {
    extern __shared__ __align__(16) unsigned char smem[];
    Work<float2> w = carve<float2>(smem, net, true);
    uint64_t* sp = w.s + kMaxWords;
    // layer 0's pre-activations of the sample and of a neighbour
    float2* z0s = reinterpret_cast<float2*>(w.s + 4 * kMaxWords);
    float2* z0n = z0s + net.size[0];
    const long t = blockIdx.x;
    if (t >= count) return;
    const int nw = (net.N + 63) / 64;
    const int size0 = net.size[0];
    load_config(spins, enum_base, enumerate, t, net.N, w.s);
    __syncthreads();
    layer0_pre(net, w.s, z0s);
    __syncthreads();
    const float2 lp = forward_from_z0(net, z0s, w);
    double er = 0.0, ei = 0.0, eor = 0.0, eoi = 0.0;
    for (int n = 0; n < op.S; n++) {
        if (op.nflip[n] != 0) continue;
        const double2 cf = apply_string(op, n, w.s, sp);
        er += cf.x;
        ei += cf.y;
    }
    const double ws = weights ? weights[t] : 1.0;
    const float wsf = static_cast<float>(ws);
    // the stored forward pass and the reverse pass of configuration xi with coefficient af
    auto pass = [&](const uint64_t* x, long xi, float2 af, bool self) {
        for (int k = threadIdx.x; k < net.units; k += blockDim.x) acts[xi * net.units + k] = w.acts[k];
        if (threadIdx.x < nw) xspins[xi * nw + threadIdx.x] = x[threadIdx.x];
        if (threadIdx.x == 0) alpha[xi] = af;
        backward_deltas<float2, false>(net, w, [&](int l, int j, float2 d) {
            dlts[xi * net.units + net.begin_angle[l] + j] = cmul(af, d);
            if (self) dltsO[t * net.units + net.begin_angle[l] + j] = make_float2(wsf * d.x, wsf * d.y);
        });
    };
    // each off-diagonal string's neighbour: one stored forward pass gives its term of the
    // local energy and feeds its reverse pass (coefficient w_s e_n)
    int q = 0;
    for (int n = 0; n < op.S; n++) {
        if (op.nflip[n] == 0) continue;
        q++;
        const double2 cf = apply_string(op, n, w.s, sp);
        // the neighbour's layer 0: the sample's moved by the flipped spins' connections
        for (int u = threadIdx.x; u < size0; u += blockDim.x) z0n[u] = z0s[u];
        __syncthreads();
        for (int f = 0; f < op.nflip[n]; f++) {
            const int site = op.flip_sites[op.flip_off[n] + f];
            const float two_s = bit_up(w.s, site) ? -2.0f : 2.0f;
            for (int k = net.sptr[site] + threadIdx.x; k < net.sptr[site + 1]; k += blockDim.x) {
                const int e = net.sq[k];
                const float2 wv = net.w[0][e];
                float2* z = z0n + e % size0;
                atomicAdd(&z->x, two_s * wv.x);
                atomicAdd(&z->y, two_s * wv.y);
            }
            // one site at a time: each unit meets a site once, so the sums do not
            // depend on the order of the atomic additions
            __syncthreads();
        }
        const float2 lq = forward_from_z0<true>(net, z0n, w);
        const double dr = static_cast<double>(lq.x) - lp.x, di = static_cast<double>(lq.y) - lp.y;
        const double m = exp(dr);
        const double2 e = make_double2(m * (cf.x * cos(di) - cf.y * sin(di)), m * (cf.x * sin(di) + cf.y * cos(di)));
        eor += e.x;
        eoi += e.y;
        pass(sp, t * xs + q, make_float2(static_cast<float>(ws * e.x), static_cast<float>(ws * e.y)), false);
    }
    er += eor;
    ei += eoi;
    // the configuration itself last: its coefficient -sum_n e_n (+ 2 E_loc with the
    // sampling term) needs every neighbour's term
    {
        double2 a = make_double2(-eor, -eoi);
        if (score) a.x += 2.0 * er;
        forward_from_z0<true>(net, z0s, w);
        pass(w.s, t * xs, make_float2(static_cast<float>(ws * a.x), static_cast<float>(ws * a.y)), score != 0);
        if (score && threadIdx.x == 0) alphaO[t] = make_float2(wsf, 0.f);
    }
    if (threadIdx.x == 0) eloc[t] = make_double2(er, ei);
}

// backward_deltas for NB configurations at once (configuration k's angles at angles +
// k * units, its error buffers at cur / nxt + k * width); emit(k, layer, unit, delta) for
// k < nb
template <int NB, typename Emit>
__device__ void backward_multi(const DeepNetDev& net, const float2* angles, float2* cur, float2* nxt, int nb,
                               Emit emit) {
    const int t = threadIdx.x;
    const int L = net.L, width = net.width, units = net.units;
    for (int l = L - 1; l >= 0; l--) {
        const int size = net.size[l];
        float2 d[NB];
#pragma unroll
        for (int k = 0; k < NB; k++) d[k] = czero<float2>();
        if (t < size) {
            const int at = net.begin_angle[l] + t;
            if (l == L - 1) {
                const float2 f = net.fw[t];
#pragma unroll
                for (int k = 0; k < NB; k++) d[k] = cmul(f, dact<false>(angles[k * units + at]));
            } else {
                const int nsize = net.size[l + 1];
                float2 acc[NB];
#pragma unroll
                for (int k = 0; k < NB; k++) acc[k] = czero<float2>();
                const float2* wn = net.w[l + 1];
                for (int e = net.rptr[l][t]; e < net.rptr[l][t + 1]; e++) {
                    const int q = net.rq[l][e];
                    const float2 wv = wn[q];
                    const int j = q % nsize;
#pragma unroll
                    for (int k = 0; k < NB; k++) acc[k] = cadd(acc[k], cmul(wv, nxt[k * width + j]));
                }
#pragma unroll
                for (int k = 0; k < NB; k++) d[k] = cmul(acc[k], dact<false>(angles[k * units + at]));
            }
        }
        __syncthreads();
        if (t < size)
#pragma unroll
            for (int k = 0; k < NB; k++) {
                cur[k * width + t] = d[k];
                if (k < nb) emit(k, l, t, d[k]);
            }
        __syncthreads();
        float2* tmp = cur;
        cur = nxt;
        nxt = tmp;
    }
}

size_t deep_adjoint_multi_smem(const DeepNetDev& n, int nb) {
    return sizeof(float2) * (nb * (32 + 2 * n.width + 2 * n.units + n.size[0]) + n.size[0]) +
           sizeof(uint64_t) * (1 + nb) * kMaxWords;
}

// deep_adjoint_kernel with the off-diagonal neighbours of a sample taken NB at a time: the
// thread of a unit evaluates it (forward and reverse) for all NB neighbours, so each weight
// read serves NB chains.  Every configuration's arithmetic and the local energy's order of
// summation are deep_adjoint_kernel's: the outputs are identical.
template <int NB>
__global__ void deep_adjoint_multi_kernel(DeepNetDev net, OpDev op, int count, const uint64_t* spins,
                                          uint64_t enum_base, int enumerate, const double* weights, int score,
                                          double2* eloc, float2* acts, float2* dlts, float2* alpha, uint64_t* xspins,
                                          int xs, float2* dltsO, float2* alphaO) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int width = net.width, size0 = net.size[0], units = net.units;
    float2* red = reinterpret_cast<float2*>(smem);                   // [NB][32]
    float2* in = red + NB * 32;                                      // [NB][width]
    float2* out = in + NB * width;                                   // [NB][width]
    float2* angles = out + NB * width;                               // [NB][units]
    float2* actsb = angles + NB * units;                             // [NB][units]
    float2* z0s = actsb + NB * units;                                // [size0] the sample's layer 0
    float2* z0n = z0s + size0;                                       // [NB][size0] the neighbours'
    uint64_t* s = reinterpret_cast<uint64_t*>(z0n + NB * size0);     // [kMaxWords] the sample
    uint64_t* sp = s + kMaxWords;                                    // [NB][kMaxWords] the neighbours
    const long t = blockIdx.x;
    if (t >= count) return;
    const int nw = (net.N + 63) / 64;
    load_config(spins, enum_base, enumerate, t, net.N, s);
    __syncthreads();
    layer0_pre(net, s, z0s);
    __syncthreads();
    auto self_z = [&](int) { return static_cast<const float2*>(z0s); };
    float2 lp1[1];
    forward_multi<1, false>(net, self_z, in, out, nullptr, nullptr, red, lp1);
    const float2 lp = lp1[0];
    double er = 0.0, ei = 0.0, eor = 0.0, eoi = 0.0;
    for (int n = 0; n < op.S; n++) {
        if (op.nflip[n] != 0) continue;
        const double2 cf = apply_string(op, n, s, sp);
        er += cf.x;
        ei += cf.y;
    }
    const double ws = weights ? weights[t] : 1.0;
    const float wsf = static_cast<float>(ws);
    int q = 0;   // neighbours done
    int n = 0;   // next string to scan
    for (;;) {
        // the next (up to) NB off-diagonal strings, their neighbours' spins and coefficients
        double2 cf[NB];
        int ns[NB];
        int nb = 0;
#pragma unroll
        for (int k = 0; k < NB; k++) {
            while (n < op.S && op.nflip[n] == 0) n++;
            ns[k] = -1;
            cf[k] = make_double2(0.0, 0.0);
            if (n < op.S) {
                cf[k] = apply_string(op, n, s, sp + k * kMaxWords);
                ns[k] = n;
                nb = k + 1;
                n++;
            }
        }
        if (nb == 0) break;
        // each neighbour's layer 0: the sample's moved by the flipped spins' connections
        for (int i = threadIdx.x; i < NB * size0; i += blockDim.x) z0n[i] = z0s[i % size0];
        __syncthreads();
#pragma unroll
        for (int k = 0; k < NB; k++) {
            if (k >= nb) break;
            const int m = ns[k];
            for (int f = 0; f < op.nflip[m]; f++) {
                const int site = op.flip_sites[op.flip_off[m] + f];
                const float two_s = bit_up(s, site) ? -2.0f : 2.0f;
                for (int e = net.sptr[site] + threadIdx.x; e < net.sptr[site + 1]; e += blockDim.x) {
                    const int c = net.sq[e];
                    const float2 wv = net.w[0][c];
                    float2* z = z0n + k * size0 + c % size0;
                    atomicAdd(&z->x, two_s * wv.x);
                    atomicAdd(&z->y, two_s * wv.y);
                }
                // one site at a time: each unit meets a site once, so the sums do not
                // depend on the order of the atomic additions
                __syncthreads();
            }
        }
        float2 lq[NB];
        forward_multi<NB, true>(net, [&](int k) { return static_cast<const float2*>(z0n + k * size0); }, in, out,
                                angles, actsb, red, lq);
        float2 af[NB];
#pragma unroll
        for (int k = 0; k < NB; k++) {
            af[k] = make_float2(0.f, 0.f);
            if (k < nb) {
                const double dr = static_cast<double>(lq[k].x) - lp.x, di = static_cast<double>(lq[k].y) - lp.y;
                const double mg = exp(dr);
                const double2 e = make_double2(mg * (cf[k].x * cos(di) - cf[k].y * sin(di)),
                                               mg * (cf[k].x * sin(di) + cf[k].y * cos(di)));
                eor += e.x;
                eoi += e.y;
                af[k] = make_float2(static_cast<float>(ws * e.x), static_cast<float>(ws * e.y));
            }
        }
        // stored activations, spins and weights of the neighbours, then their reverse passes
        const long x0 = t * xs + q + 1;
        for (int i = threadIdx.x; i < nb * units; i += blockDim.x)
            acts[(x0 + i / units) * units + i % units] = actsb[i];
        for (int i = threadIdx.x; i < nb * nw; i += blockDim.x)
            xspins[(x0 + i / nw) * nw + i % nw] = sp[(i / nw) * kMaxWords + i % nw];
        if (threadIdx.x < nb)
#pragma unroll
            for (int k = 0; k < NB; k++)
                if (k == static_cast<int>(threadIdx.x)) alpha[x0 + k] = af[k];
        backward_multi<NB>(net, angles, in, out, nb, [&](int k, int l, int j, float2 d) {
            dlts[(x0 + k) * units + net.begin_angle[l] + j] = cmul(af[k], d);
        });
        q += nb;
    }
    er += eor;
    ei += eoi;
    // the configuration itself last: its coefficient -sum_n e_n (+ 2 E_loc with the
    // sampling term) needs every neighbour's term
    double2 a = make_double2(-eor, -eoi);
    if (score) a.x += 2.0 * er;
    const float2 afs = make_float2(static_cast<float>(ws * a.x), static_cast<float>(ws * a.y));
    forward_multi<1, true>(net, self_z, in, out, angles, actsb, red, lp1);
    const long xi = t * xs;
    for (int i = threadIdx.x; i < units; i += blockDim.x) acts[xi * units + i] = actsb[i];
    if (threadIdx.x < nw) xspins[xi * nw + threadIdx.x] = s[threadIdx.x];
    if (threadIdx.x == 0) alpha[xi] = afs;
    backward_multi<1>(net, angles, in, out, 1, [&](int, int l, int j, float2 d) {
        dlts[xi * units + net.begin_angle[l] + j] = cmul(afs, d);
        if (score) dltsO[t * units + net.begin_angle[l] + j] = make_float2(wsf * d.x, wsf * d.y);
    });
    if (score && threadIdx.x == 0) alphaO[t] = make_float2(wsf, 0.f);
    if (threadIdx.x == 0) eloc[t] = make_double2(er, ei);
}

// partial[z][m][n] = sum over the configurations x of split z of D[x][m] * A(x, n), where
// D[x][m] = D[x * ldd + m] and A(x, n) = A[x * lda + n] (A_ACTS), +-1 for spin n of the
// spin row xsp + x * xld (A_SPINS) or 1 (A_ONES).  FP32 products and sums within a split,
// FP64 partials.
enum : int { A_ACTS = 0, A_SPINS = 1, A_ONES = 2 };
template <int AMODE>
__global__ void __launch_bounds__(256) adj_cgemm_kernel(int K, int M, int Nn, const float2* __restrict__ D, int ldd,
                                                        const float2* __restrict__ A, int lda,
                                                        const uint64_t* __restrict__ xsp, int xld, int per_split,
                                                        double2* __restrict__ partial) {
    __shared__ float2 sD[32][33];
    __shared__ float2 sA[32][33];
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    const int m0 = blockIdx.x * 32, n0 = blockIdx.y * 32;
    const int k0 = blockIdx.z * per_split, k1 = min(K, k0 + per_split);
    float2 acc[2][2];
#pragma unroll
    for (int i = 0; i < 2; i++)
#pragma unroll
        for (int j = 0; j < 2; j++) acc[i][j] = make_float2(0.f, 0.f);
    for (int kb = k0; kb < k1; kb += 32) {
        for (int e = threadIdx.x; e < 32 * 32; e += 256) {
            const int kk = e >> 5, c = e & 31;
            const int x = kb + kk;
            const bool ok = x < k1;
            sD[kk][c] = (ok && m0 + c < M) ? D[static_cast<long>(x) * ldd + m0 + c] : make_float2(0.f, 0.f);
            float2 av = make_float2(0.f, 0.f);
            if (ok && n0 + c < Nn) {
                if (AMODE == A_ACTS) av = A[static_cast<long>(x) * lda + n0 + c];
                else if (AMODE == A_SPINS) {
                    const int i = n0 + c;
                    av.x = ((xsp[static_cast<long>(x) * xld + (i >> 6)] >> (i & 63)) & 1ull) ? 1.f : -1.f;
                } else av.x = 1.f;
            }
            sA[kk][c] = av;
        }
        __syncthreads();
#pragma unroll 8
        for (int kk = 0; kk < 32; kk++) {
            const float2 d0 = sD[kk][ty], d1 = sD[kk][ty + 16];
            const float2 a0 = sA[kk][tx], a1 = sA[kk][tx + 16];
            acc[0][0] = cadd(acc[0][0], cmul(d0, a0));
            acc[0][1] = cadd(acc[0][1], cmul(d0, a1));
            acc[1][0] = cadd(acc[1][0], cmul(d1, a0));
            acc[1][1] = cadd(acc[1][1], cmul(d1, a1));
        }
        __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < 2; i++)
#pragma unroll
        for (int j = 0; j < 2; j++) {
            const int m = m0 + ty + 16 * i, n = n0 + tx + 16 * j;
            if (m < M && n < Nn)
                partial[(static_cast<long>(blockIdx.z) * M + m) * Nn + n] =
                    make_double2(acc[i][j].x, acc[i][j].y);
        }
}

// G[m][n] += sum over splits (in order) of partial[z][m][n]
__global__ void adj_split_sum_kernel(int M, int Nn, int splits, const double2* __restrict__ partial, double2* G) {
    const long t = static_cast<long>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (t >= static_cast<long>(M) * Nn) return;
    double2 a = make_double2(0.0, 0.0);
    for (int z = 0; z < splits; z++) {
        const double2 v = partial[static_cast<long>(z) * M * Nn + t];
        a.x += v.x;
        a.y += v.y;
    }
    G[t].x += a.x;
    G[t].y += a.y;
}

int threads_for(const DeepNetDev& n) {
    const int width = std::max(n.width, n.N);
    return std::min(1024, std::max(32, (width + 31) / 32 * 32));
}

size_t smem_for(const DeepNetDev& n, size_t vbytes, bool store) {
    return vbytes * (32 + 2 * n.width + (store ? 2 * n.units : 0)) + sizeof(uint64_t) * 4 * kMaxWords;
}

template <typename K>
cudaError_t set_smem(K kernel, size_t bytes) {
    if (bytes <= 48 * 1024) return cudaSuccess;
    return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(bytes));
}

}  // namespace

// ---------------------------------------------------------------- host side
struct DeepHost {
    std::vector<std::unique_ptr<DevBuf>> bufs;
    DeepNetDev net[2];
};

static std::vector<std::unique_ptr<DeepHost>>& deep_registry() {
    static std::vector<std::unique_ptr<DeepHost>> r;
    return r;
}

template <typename T>
static cudaError_t upload(DeepHost* h, const std::vector<T>& v, const T** out) {
    auto b = std::make_unique<DevBuf>();
    cudaError_t e = b->ensure(std::max<size_t>(16, sizeof(T) * v.size()));
    if (e != cudaSuccess) return e;
    if (!v.empty()) e = cudaMemcpy(b->p, v.data(), sizeof(T) * v.size(), cudaMemcpyHostToDevice);
    *out = static_cast<const T*>(b->p);
    h->bufs.push_back(std::move(b));
    return e;
}

// Device copy of the net(s): part 0 = complex net (PsiDeep) or real part (PsiPair), 1 = imaginary part.
int deep_upload(rbmg_psi* psi) {
    auto h = std::make_unique<DeepHost>();
    const int nets = psi->kind == 2 ? 2 : 1;
    const int L = static_cast<int>(psi->layers.size());
    for (int part = 0; part < nets; part++) {
        DeepNetDev& d = h->net[part];
        d = DeepNetDev{};
        d.N = psi->N;
        d.L = L;
        d.real_net = psi->kind == 2;
        d.ti = psi->translational_invariance;
        d.P = psi->num_params();
        d.width = psi->width;
        int k = 2 * psi->N, a = 0;
        for (int l = 0; l < L; l++) {
            const auto& Ly = psi->layers[l];
            d.size[l] = Ly.size;
            d.conn[l] = Ly.conn;
            d.begin_params[l] = k - 2 * psi->N;
            d.begin_angle[l] = a;
            k += Ly.size + Ly.conn * Ly.size;
            a += Ly.size;
            auto pick = [&](const cplx& z) -> cplx {
                if (psi->kind != 2) return z;
                return part == 0 ? cplx(z.real(), 0.0) : cplx(z.imag(), 0.0);
            };
            std::vector<float2> w32(Ly.weights.size()), b32(Ly.biases.size());
            std::vector<double2> w64(Ly.weights.size()), b64(Ly.biases.size());
            for (size_t q = 0; q < Ly.weights.size(); q++) {
                const cplx z = pick(Ly.weights[q]);
                w32[q] = make_float2(float(z.real()), float(z.imag()));
                w64[q] = make_double2(z.real(), z.imag());
            }
            for (size_t q = 0; q < Ly.biases.size(); q++) {
                const cplx z = pick(Ly.biases[q]);
                b32[q] = make_float2(float(z.real()), float(z.imag()));
                b64[q] = make_double2(z.real(), z.imag());
            }
            std::vector<int> ci(Ly.connections.begin(), Ly.connections.end());
            RBMG_CK(upload(h.get(), w32, &d.w[l]));
            RBMG_CK(upload(h.get(), b32, &d.b[l]));
            RBMG_CK(upload(h.get(), w64, &d.w64[l]));
            RBMG_CK(upload(h.get(), b64, &d.b64[l]));
            RBMG_CK(upload(h.get(), ci, &d.cidx[l]));
        }
        d.units = a;
        // rhs lists of layer l from the lhs connections of layer l+1, in the order of
        // source/quantum_state/PsiDeep.cu:101-111 (next unit j ascending, connection c inner)
        for (int l = 0; l + 1 < L; l++) {
            const auto& Nx = psi->layers[l + 1];
            const int size = psi->layers[l].size;
            std::vector<std::vector<int>> lists(size);
            for (int j = 0; j < Nx.size; j++)
                for (int c = 0; c < Nx.conn; c++) lists[Nx.connections[c * Nx.size + j]].push_back(c * Nx.size + j);
            std::vector<int> ptr(size + 1, 0), q;
            for (int i = 0; i < size; i++) {
                ptr[i] = static_cast<int>(q.size());
                q.insert(q.end(), lists[i].begin(), lists[i].end());
            }
            ptr[size] = static_cast<int>(q.size());
            RBMG_CK(upload(h.get(), ptr, &d.rptr[l]));
            RBMG_CK(upload(h.get(), q, &d.rq[l]));
        }
        {
            const auto& L0 = psi->layers[0];
            std::vector<std::vector<int>> lists(psi->N);
            for (int c = 0; c < L0.conn; c++)
                for (int j = 0; j < L0.size; j++) {
                    const int i = static_cast<int>(L0.connections[static_cast<size_t>(c) * L0.size + j]);
                    if (i < psi->N) lists[i].push_back(c * L0.size + j);
                }
            std::vector<int> ptr(psi->N + 1, 0), q;
            for (int i = 0; i < psi->N; i++) {
                ptr[i] = static_cast<int>(q.size());
                q.insert(q.end(), lists[i].begin(), lists[i].end());
            }
            ptr[psi->N] = static_cast<int>(q.size());
            if (q.empty()) q.push_back(0);
            RBMG_CK(upload(h.get(), ptr, &d.sptr));
            RBMG_CK(upload(h.get(), q, &d.sq));
        }
        std::vector<float2> f32(psi->final_weights.size());
        std::vector<double2> f64(psi->final_weights.size());
        for (size_t q = 0; q < f32.size(); q++) {
            const cplx z = psi->kind != 2 ? psi->final_weights[q]
                                          : (part == 0 ? cplx(psi->final_weights[q].real(), 0.0)
                                                       : cplx(psi->final_weights[q].imag(), 0.0));
            f32[q] = make_float2(float(z.real()), float(z.imag()));
            f64[q] = make_double2(z.real(), z.imag());
        }
        RBMG_CK(upload(h.get(), f32, &d.fw));
        RBMG_CK(upload(h.get(), f64, &d.fw64));
    }
    if (nets == 1) h->net[1] = h->net[0];
    psi->deep_dev[0] = h->net[0];
    psi->deep_dev[1] = h->net[1];
    psi->deep_host = std::shared_ptr<void>(h.release(), [](void* p) { delete static_cast<DeepHost*>(p); });
    return RBMG_OK;
}

static DeepNetDev net_of(const rbmg_psi* psi, int part) {
    DeepNetDev d = psi->deep_dev[part];
    d.ti = psi->translational_invariance;
    return d;
}

int deep_log_psi(const rbmg_psi* psi, int count, const uint64_t* d_spins, uint64_t enum_base, int enumerate,
                 double2* d_out, cudaStream_t st) {
    if (count <= 0) return RBMG_OK;
    const DeepNetDev n0 = net_of(psi, 0), n1 = net_of(psi, 1);
    // FP64: exact-summation weights and the psi vector are built from these values
    const size_t sm = smem_for(n0, sizeof(double2), false) + sizeof(uint64_t) * kMaxWords;
    RBMG_CK(set_smem(deep_logpsi_kernel<double2>, sm));
    deep_logpsi_kernel<double2><<<count, threads_for(n0), sm, st>>>(n0, n1, psi->kind == 2, count, d_spins, enum_base,
                                                                     enumerate, d_out);
    RBMG_CK(cudaGetLastError());
    return RBMG_OK;
}

int deep_eloc_chunk(const rbmg_psi* psi, const rbmg_operator* op, const Chunk& c, double2* d_eloc, cudaStream_t st) {
    if (c.count <= 0) return RBMG_OK;
    const DeepNetDev n0 = net_of(psi, 0), n1 = net_of(psi, 1);
    const size_t sm = smem_for(n0, sizeof(double2), false) + 2 * sizeof(uint64_t) * kMaxWords;
    RBMG_CK(set_smem(deep_eloc_kernel<double2, false>, sm));
    deep_eloc_kernel<double2, false><<<c.count, threads_for(n0), sm, st>>>(n0, n1, psi->kind == 2, n0, n1, op->dev(),
                                                                           c.count, c.spins, c.enum_base, c.enumerate,
                                                                           d_eloc, nullptr);
    RBMG_CK(cudaGetLastError());
    return RBMG_OK;
}

int deep_hsd64_chunk(const rbmg_psi* psi, const rbmg_psi* pp, const rbmg_operator* op, const Chunk& c,
                     double2* d_eloc, double2* d_dlp, cudaStream_t st) {
    if (c.count <= 0) return RBMG_OK;
    if (pp->width != psi->width || pp->layers.size() != psi->layers.size())
        return fail(RBMG_EUNSUPPORTED, "hsd: psi and psi_prime need the same layer shapes");
    const DeepNetDev n0 = net_of(psi, 0), n1 = net_of(psi, 1), q0 = net_of(pp, 0), q1 = net_of(pp, 1);
    const size_t sm = smem_for(n0, sizeof(double2), false) + 2 * sizeof(uint64_t) * kMaxWords;
    RBMG_CK(set_smem(deep_eloc_kernel<double2, true>, sm));
    deep_eloc_kernel<double2, true><<<c.count, threads_for(n0), sm, st>>>(n0, n1, psi->kind == 2, q0, q1, op->dev(),
                                                                         c.count, c.spins, c.enum_base, c.enumerate,
                                                                         d_eloc, d_dlp);
    RBMG_CK(cudaGetLastError());
    return RBMG_OK;
}

static DevBuf& rows_buf(int which) {
    static thread_local DevBuf b[3];
    return b[which];
}

static int col_reduce(int count, int P, const double2* c, const double2* A, long ld, int conj_a, double2* out,
                      cudaStream_t st) {
    if (count <= 0) return RBMG_OK;
    const int per_split = std::max(64, (count + 63) / 64);
    const int splits = (count + per_split - 1) / per_split;
    DevBuf& part = rows_buf(2);
    RBMG_CK(part.ensure(sizeof(double2) * static_cast<size_t>(splits) * P));
    const dim3 grid((P + 255) / 256, splits);
    col_reduce_kernel<<<grid, 256, 0, st>>>(count, P, c, A, ld, conj_a, part.as<double2>(), per_split);
    col_finish_kernel<<<(P + 255) / 256, 256, 0, st>>>(P, splits, part.as<double2>(), out);
    RBMG_CK(cudaGetLastError());
    return RBMG_OK;
}

// O_k rows (k >= 2N) of `count` configurations into rows [count][ld] (FP64, PsiDeep)
int deep_ok_rows(const rbmg_psi* psi, int count, const uint64_t* d_spins, uint64_t enum_base, int enumerate,
                 double2* rows, long ld, cudaStream_t st) {
    if (psi->kind != 1) return fail(RBMG_EUNSUPPORTED, "O_k rows: PsiDeep only (PsiPair.hpp:73-76 defines none)");
    if (count <= 0) return RBMG_OK;
    const DeepNetDev net = net_of(psi, 0);
    const size_t sm = smem_for(net, sizeof(double2), true);
    RBMG_CK(set_smem(deep_ok_kernel<false>, sm));
    deep_ok_kernel<false><<<count, threads_for(net), sm, st>>>(net, count, d_spins, enum_base, enumerate, rows, ld);
    RBMG_CK(cudaGetLastError());
    return RBMG_OK;
}

int deep_hsd_okreduce(const rbmg_psi* pp, int pair_part, int count, const uint64_t* d_spins, uint64_t enum_base,
                      int enumerate, const double2* d_coef, double2* acc, cudaStream_t st) {
    const DeepNetDev net = net_of(pp, pair_part == 1 ? 1 : 0);
    const int P = net.P - 2 * net.N;
    const int chunk = std::max(1, static_cast<int>((size_t(256) << 20) / (sizeof(double2) * P)));
    DevBuf& rows = rows_buf(0);
    RBMG_CK(rows.ensure(sizeof(double2) * static_cast<size_t>(std::min(chunk, count)) * P));
    const size_t sm = smem_for(net, sizeof(double2), true);
    for (int base = 0; base < count; base += chunk) {
        const int cnt = std::min(chunk, count - base);
        const uint64_t* sp = d_spins ? d_spins + static_cast<size_t>(base) * ((net.N + 63) / 64) : nullptr;
        if (pp->kind == 2) {
            RBMG_CK(set_smem(deep_ok_kernel<true>, sm));
            deep_ok_kernel<true><<<cnt, threads_for(net), sm, st>>>(net, cnt, sp, enum_base + base, enumerate,
                                                                    rows.as<double2>(), P);
        } else {
            RBMG_CK(set_smem(deep_ok_kernel<false>, sm));
            deep_ok_kernel<false><<<cnt, threads_for(net), sm, st>>>(net, cnt, sp, enum_base + base, enumerate,
                                                                     rows.as<double2>(), P);
        }
        RBMG_CK(cudaGetLastError());
        // real O_k (PsiPair) multiply the real or complex coefficient; complex O_k enter conjugated
        const int r = col_reduce(cnt, P, d_coef + base, rows.as<double2>(), P, pp->kind == 2 ? 0 : 1, acc, st);
        if (r != RBMG_OK) return r;
    }
    return RBMG_OK;
}

int deep_ok_vector(const rbmg_psi* psi, const uint64_t* d_spins, double2* d_out, cudaStream_t st) {
    if (psi->kind == 2) return fail(RBMG_EUNSUPPORTED, "psi_O_k_vector: not defined for PsiPair (PsiPair.hpp:73-76)");
    const DeepNetDev net = net_of(psi, 0);
    const int P = net.P - 2 * net.N;
    DevBuf& rows = rows_buf(0);
    RBMG_CK(rows.ensure(sizeof(double2) * P));
    const size_t sm = smem_for(net, sizeof(double2), true);
    RBMG_CK(set_smem(deep_ok_kernel<false>, sm));
    deep_ok_kernel<false><<<1, threads_for(net), sm, st>>>(net, 1, d_spins, 0, 0, rows.as<double2>(), P);
    RBMG_CK(cudaGetLastError());
    RBMG_CK(cudaMemsetAsync(d_out, 0, sizeof(double2) * P, st));
    DevBuf& one = rows_buf(1);
    RBMG_CK(one.ensure(sizeof(double2)));
    const double2 h1 = make_double2(1.0, 0.0);
    RBMG_CK(cudaMemcpyAsync(one.p, &h1, sizeof(double2), cudaMemcpyHostToDevice, st));
    return col_reduce(1, P, one.as<double2>(), rows.as<double2>(), P, 0, d_out, st);
}

int deep_gradient_chunk(const rbmg_psi* psi, const rbmg_operator* op, const Chunk& c, double2 e_shift,
                        double2* d_eloc, double2* acc_O, double2* acc_EO, double2* acc_Ek, double2* coef1,
                        double2* coef2, cudaStream_t st, double2* acc_B, double2* coef3) {
    if (psi->kind == 2) return fail(RBMG_EUNSUPPORTED, "gradient: not instantiated for PsiPair (ExpectationValue.cu:553)");
    const DeepNetDev net = net_of(psi, 0);
    const int P = net.P - 2 * net.N;
    const int chunk = std::max(1, static_cast<int>((size_t(512) << 20) / (2 * sizeof(double2) * P)));
    DevBuf& orows = rows_buf(0);
    DevBuf& erows = rows_buf(1);
    RBMG_CK(orows.ensure(sizeof(double2) * static_cast<size_t>(std::min(chunk, c.count)) * P));
    RBMG_CK(erows.ensure(sizeof(double2) * static_cast<size_t>(std::min(chunk, c.count)) * P));
    const size_t sm = smem_for(net, sizeof(double2), true) + sizeof(uint64_t) * kMaxWords;
    RBMG_CK(set_smem(deep_grad_kernel, sm));
    RBMG_CK(launch_coef(c.count, c.weights, nullptr, 1.0, coef1, st));
    for (int base = 0; base < c.count; base += chunk) {
        const int cnt = std::min(chunk, c.count - base);
        const uint64_t* sp = c.spins ? c.spins + static_cast<size_t>(base) * ((net.N + 63) / 64) : nullptr;
        deep_grad_kernel<<<cnt, threads_for(net), sm, st>>>(net, op->dev(), cnt, sp, c.enum_base + base, c.enumerate,
                                                            e_shift, d_eloc + base, orows.as<double2>(),
                                                            erows.as<double2>(), P);
        RBMG_CK(cudaGetLastError());
        RBMG_CK(launch_coef(cnt, c.weights ? c.weights + base : nullptr, d_eloc + base, 1.0, coef2 + base, st,
                            e_shift));
        int r = col_reduce(cnt, P, coef1 + base, orows.as<double2>(), P, 0, acc_O, st);
        if (r == RBMG_OK) r = col_reduce(cnt, P, coef2 + base, orows.as<double2>(), P, 1, acc_EO, st);
        if (r == RBMG_OK) r = col_reduce(cnt, P, coef1 + base, erows.as<double2>(), P, 0, acc_Ek, st);
        if (r == RBMG_OK && acc_B) {
            // sum w conj(E - E0) (E_k - E0 O_k): the fluctuation gradient's covariance term
            RBMG_CK(launch_coef_conj(cnt, c.weights ? c.weights + base : nullptr, d_eloc + base, e_shift, coef3 + base,
                                     st));
            r = col_reduce(cnt, P, coef3 + base, erows.as<double2>(), P, 0, acc_B, st);
        }
        if (r != RBMG_OK) return r;
    }
    return RBMG_OK;
}

// Adjoint of the local energy over one chunk of samples, accumulated into the dense
// per-layer gradient blocks G (double2): for layer l, G_w[l] [size_l][in_l] (in_0 = N)
// and G_b[l] [size_l], then G_fw [last]; offsets in `goff`.  d_eloc receives E_loc.
int deep_adjoint_chunk(const rbmg_psi* psi, const rbmg_operator* op, const Chunk& c, int score, double2* d_eloc,
                       double2* G, double2* GO, const std::vector<size_t>& goff, cudaStream_t st) {
    const DeepNetDev net = net_of(psi, 0);
    const int nw = (net.N + 63) / 64;
    const int xs = 1 + op->num_offdiag;
    static thread_local DevBuf acts, dlts, alpha, xsp, dltsO, alphaO, partial;
    const size_t per_sample = static_cast<size_t>(xs) * (2 * sizeof(float2) * net.units + sizeof(float2) + 8 * nw) +
                              sizeof(float2) * (net.units + 1);
    const int chunk = std::max(1, static_cast<int>(std::min<size_t>(c.count, (size_t(768) << 20) / per_sample)));
    RBMG_CK(acts.ensure(sizeof(float2) * static_cast<size_t>(chunk) * xs * net.units));
    RBMG_CK(dlts.ensure(sizeof(float2) * static_cast<size_t>(chunk) * xs * net.units));
    RBMG_CK(alpha.ensure(sizeof(float2) * static_cast<size_t>(chunk) * xs));
    RBMG_CK(xsp.ensure(sizeof(uint64_t) * static_cast<size_t>(chunk) * xs * nw));
    RBMG_CK(dltsO.ensure(sizeof(float2) * static_cast<size_t>(chunk) * net.units));
    RBMG_CK(alphaO.ensure(sizeof(float2) * static_cast<size_t>(chunk)));
    const size_t sm = smem_for(net, sizeof(float2), true) + 2 * sizeof(float2) * net.size[0];
    RBMG_CK(set_smem(deep_adjoint_kernel, sm));
    // neighbours per pass of the reverse kernel (RBMG_DEEP_ADJOINT_BATCH = 1, 2, 4 or 8;
    // default 4), the same outputs
    int nbatch = 4;
    if (const char* v = std::getenv("RBMG_DEEP_ADJOINT_BATCH")) nbatch = std::atoi(v);
    if (nbatch != 1 && nbatch != 2 && nbatch != 4 && nbatch != 8)
        return fail(RBMG_EINVAL, "RBMG_DEEP_ADJOINT_BATCH: 1, 2, 4 or 8");
    const size_t smb = deep_adjoint_multi_smem(net, nbatch);
    if (nbatch == 2) RBMG_CK(set_smem(deep_adjoint_multi_kernel<2>, smb));
    if (nbatch == 4) RBMG_CK(set_smem(deep_adjoint_multi_kernel<4>, smb));
    if (nbatch == 8) RBMG_CK(set_smem(deep_adjoint_multi_kernel<8>, smb));
    constexpr int kMaxSplits = 64;
    for (int base = 0; base < c.count; base += chunk) {
        const int cnt = std::min(chunk, c.count - base);
        const uint64_t* sp = c.spins ? c.spins + static_cast<size_t>(base) * nw : nullptr;
        const double* wb = c.weights ? c.weights + base : nullptr;
        if (nbatch == 8)
            deep_adjoint_multi_kernel<8><<<cnt, threads_for(net), smb, st>>>(
                net, op->dev(), cnt, sp, c.enum_base + base, c.enumerate, wb, score, d_eloc + base,
                acts.as<float2>(), dlts.as<float2>(), alpha.as<float2>(), xsp.as<uint64_t>(), xs, dltsO.as<float2>(),
                alphaO.as<float2>());
        else if (nbatch == 4)
            deep_adjoint_multi_kernel<4><<<cnt, threads_for(net), smb, st>>>(
                net, op->dev(), cnt, sp, c.enum_base + base, c.enumerate, wb, score, d_eloc + base,
                acts.as<float2>(), dlts.as<float2>(), alpha.as<float2>(), xsp.as<uint64_t>(), xs, dltsO.as<float2>(),
                alphaO.as<float2>());
        else if (nbatch == 2)
            deep_adjoint_multi_kernel<2><<<cnt, threads_for(net), smb, st>>>(
                net, op->dev(), cnt, sp, c.enum_base + base, c.enumerate, wb, score, d_eloc + base,
                acts.as<float2>(), dlts.as<float2>(), alpha.as<float2>(), xsp.as<uint64_t>(), xs, dltsO.as<float2>(),
                alphaO.as<float2>());
        else
            deep_adjoint_kernel<<<cnt, threads_for(net), sm, st>>>(
                net, op->dev(), cnt, sp, c.enum_base + base, c.enumerate, wb, score, d_eloc + base,
                acts.as<float2>(), dlts.as<float2>(), alpha.as<float2>(), xsp.as<uint64_t>(), xs, dltsO.as<float2>(),
                alphaO.as<float2>());
        RBMG_CK(cudaGetLastError());
        // reduce over K configurations whose rows are `stride` configurations apart
        auto reduce = [&](int K, int amode, int M, int Nn, const float2* D, int ldd, const float2* A, int lda, int xld,
                          double2* out) -> int {
            const int splits = std::min(kMaxSplits, std::max(1, K / 256));
            const int per = (K + splits - 1) / splits;
            RBMG_CK(partial.ensure(sizeof(double2) * static_cast<size_t>(splits) * M * Nn));
            const dim3 grid((M + 31) / 32, (Nn + 31) / 32, splits);
            if (amode == A_ACTS)
                adj_cgemm_kernel<A_ACTS><<<grid, 256, 0, st>>>(K, M, Nn, D, ldd, A, lda, xsp.as<uint64_t>(), xld, per,
                                                                partial.as<double2>());
            else if (amode == A_SPINS)
                adj_cgemm_kernel<A_SPINS><<<grid, 256, 0, st>>>(K, M, Nn, D, ldd, A, lda, xsp.as<uint64_t>(), xld, per,
                                                                 partial.as<double2>());
            else
                adj_cgemm_kernel<A_ONES><<<grid, 256, 0, st>>>(K, M, Nn, D, ldd, A, lda, xsp.as<uint64_t>(), xld, per,
                                                                partial.as<double2>());
            RBMG_CK(cudaGetLastError());
            const long tot = static_cast<long>(M) * Nn;
            adj_split_sum_kernel<<<static_cast<unsigned>((tot + 255) / 256), 256, 0, st>>>(M, Nn, splits,
                                                                                         partial.as<double2>(), out);
            RBMG_CK(cudaGetLastError());
            return RBMG_OK;
        };
        // pass 0: all configurations with alpha-weighted deltas -> G; pass 1 (score): the
        // samples themselves with weight w_s -> GO
        for (int pass = 0; pass < (score ? 2 : 1); pass++) {
            const int K = pass == 0 ? cnt * xs : cnt;
            const int row = pass == 0 ? net.units : xs * net.units;     // activation row stride
            const float2* dl = pass == 0 ? dlts.as<float2>() : dltsO.as<float2>();
            double2* out = pass == 0 ? G : GO;
            for (int l = 0; l < net.L; l++) {
                const int size = net.size[l];
                const int in = l == 0 ? net.N : net.size[l - 1];
                const float2* D = dl + net.begin_angle[l];
                int r = l == 0 ? reduce(K, A_SPINS, size, in, D, net.units, nullptr, 0, pass == 0 ? nw : xs * nw,
                                        out + goff[2 * l])
                               : reduce(K, A_ACTS, size, in, D, net.units, acts.as<float2>() + net.begin_angle[l - 1],
                                        row, 0, out + goff[2 * l]);
                if (r != RBMG_OK) return r;
                r = reduce(K, A_ONES, size, 1, D, net.units, nullptr, 0, 0, out + goff[2 * l + 1]);
                if (r != RBMG_OK) return r;
            }
            const int last = net.size[net.L - 1];
            const int r = reduce(K, A_ACTS, 1, last, pass == 0 ? alpha.as<float2>() : alphaO.as<float2>(), 1,
                                 acts.as<float2>() + net.begin_angle[net.L - 1], row, 0, out + goff[2 * net.L]);
            if (r != RBMG_OK) return r;
        }
    }
    return RBMG_OK;
}

// MonteCarloLoop::foreach for PsiDeep / PsiPair (MonteCarloLoop.hpp:294-339)
int deep_stream(rbmg_ensemble* e, const rbmg_psi* psi, const rbmg_operator* op, bool want_eloc,
                size_t max_chunk_samples, const std::function<int(const Chunk&)>& fn) {
    (void)op;
    (void)want_eloc;
    if (e->total_z) return fail(RBMG_EUNSUPPORTED, "PsiDeep chains: S_z symmetry is not provided");
    const int nw = (psi->N + 63) / 64;
    const int B = static_cast<int>(e->num_chains);
    const int steps = static_cast<int>(e->num_samples / e->num_chains);
    RBMG_CK(e->spins.ensure(sizeof(uint64_t) * nw * B));
    RBMG_CK(cudaMemsetAsync(e->accepts.p, 0, sizeof(unsigned long long) * B, stream()));
    RBMG_CK(cudaMemsetAsync(e->proposals.p, 0, sizeof(unsigned long long) * B, stream()));
    static thread_local DevBuf samples;
    const int rows_per_chunk = static_cast<int>(std::max<size_t>(1, std::min<size_t>(steps, max_chunk_samples / B)));
    RBMG_CK(samples.ensure(sizeof(uint64_t) * nw * B * rows_per_chunk));
    const DeepNetDev n0 = net_of(psi, 0), n1 = net_of(psi, 1);
    // + layer 0's pre-activations of the state and of a proposal
    const size_t sm = smem_for(n0, sizeof(float2), false) + 2 * sizeof(float2) * n0.size[0];
    RBMG_CK(set_smem(deep_mc_kernel, sm));
    // single-flip chains of a complex net: several walkers per CTA (RBMG_DEEP_WALKERS_PER_BLOCK
    // = 1, 2, 4 or 8; default 8, the fastest on the 100-200-100-50 net), the same chains
    int wpc = 8;
    if (const char* v = std::getenv("RBMG_DEEP_WALKERS_PER_BLOCK")) wpc = std::atoi(v);
    if (wpc != 1 && wpc != 2 && wpc != 4 && wpc != 8) return fail(RBMG_EINVAL, "RBMG_DEEP_WALKERS_PER_BLOCK: 1, 2, 4 or 8");
    if (e->fast_sweep_tries != 0 || psi->kind == 2 || n0.ti) wpc = 1;
    const size_t smm = deep_mc_multi_smem(n0, wpc);
    if (wpc == 2) RBMG_CK(set_smem(deep_mc_multi_kernel<2>, smm));
    if (wpc == 4) RBMG_CK(set_smem(deep_mc_multi_kernel<4>, smm));
    if (wpc == 8) RBMG_CK(set_smem(deep_mc_multi_kernel<8>, smm));
    const int blocks = (B + wpc - 1) / wpc;
    bool first = true;
    for (int row0 = 0; row0 < steps; row0 += rows_per_chunk) {
        const int rows = std::min(rows_per_chunk, steps - row0);
        McLaunch L{};
        L.B = B;
        L.seed = e->seed;
        L.spins = e->spins.as<uint64_t>();
        L.rng_index = e->rng_index.as<uint64_t>();
        L.init = first ? 1 : 0;
        L.fast_tries = static_cast<int>(e->fast_sweep_tries);
        L.n_therm = first ? static_cast<int>(e->num_therm) : 0;
        L.n_samples = rows;
        L.sweeps_per_sample = static_cast<int>(e->num_sweeps);
        L.sample_spins = samples.as<uint64_t>();
        L.accepts = e->accepts.as<unsigned long long>();
        L.proposals = e->proposals.as<unsigned long long>();
        if (wpc == 2)
            deep_mc_multi_kernel<2><<<blocks, threads_for(n0), smm, stream()>>>(n0, L);
        else if (wpc == 4)
            deep_mc_multi_kernel<4><<<blocks, threads_for(n0), smm, stream()>>>(n0, L);
        else if (wpc == 8)
            deep_mc_multi_kernel<8><<<blocks, threads_for(n0), smm, stream()>>>(n0, L);
        else
            deep_mc_kernel<<<B, threads_for(n0), sm, stream()>>>(n0, n1, psi->kind == 2, L);
        RBMG_CK(cudaGetLastError());
        first = false;
        Chunk c;
        c.count = rows * B;
        c.spins = samples.as<uint64_t>();
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

}  // namespace rbmg
