// Complex-RBM kernels: Metropolis sampler and per-sample estimator pass.
//
// Layout: one warp per walker (or per configuration).  Lane l owns hidden units
// j = l + 32 k, k < K, and keeps their angles theta_j and Re f(theta_j) in
// registers for the whole chain; W rows are read coalesced (one float2 per lane
// per k) from global memory through L1/L2.  This file is included by the rbm_k*.cu
// translation units, each instantiating one K.
#pragma once

#include "device_math.cuh"
#include "kernels.h"

namespace rbmg {

// angles from scratch: theta_j = b_j, then theta_j +/-= W_ij for i = 0..N-1 in order
// (include/quantum_state/Psi.hpp:43-53)
template <int K, int NW>
__device__ __forceinline__ void rbm_refresh(const RbmDev& P, const Spins<NW>& s, float (&tr)[K], float (&ti)[K],
                                            int lane) {
#pragma unroll
    for (int k = 0; k < K; k++) {
        const float2 b = __ldg(P.b + lane + 32 * k);
        tr[k] = b.x;
        ti[k] = b.y;
    }
    const float2* row = P.W + lane;
    for (int i = 0; i < P.N; i++, row += P.Mpad) {
        const float sg = s.up(i) ? 1.0f : -1.0f;
#pragma unroll
        for (int k = 0; k < K; k++) {
            const float2 w = __ldg(row + 32 * k);
            tr[k] = __fmaf_rn(sg, w.x, tr[k]);   // sg = +-1: the product is exact
            ti[k] = __fmaf_rn(sg, w.y, ti[k]);
        }
    }
}

template <int NW, class Rng>
__device__ __forceinline__ void draw_spins(Rng& rng, int N, Spins<NW>& s) {
#pragma unroll
    for (int k = 0; k < NW; k++) {
        const uint64_t lo = rng.next();
        const uint64_t hi = rng.next();
        s.w[k] = lo | (hi << 32);
    }
    if (N / 64 < NW) s.w[N / 64] &= (1ull << (N % 64)) - 1ull;
}

// include/random.h:60-79 with 64-bit masks (single word, N <= 64)
template <class Rng>
__device__ __forceinline__ uint64_t draw_n_over_k(Rng& rng, unsigned n, unsigned k) {
    const uint64_t mask = n >= 64 ? ~0ull : ((1ull << n) - 1ull);
    uint64_t w = rng.next();
    w |= static_cast<uint64_t>(rng.next()) << 32;
    uint64_t result = w & mask;
    int diff = static_cast<int>(k) - __popcll(result);
    while (diff != 0) {
        uint64_t w2 = rng.next();
        w2 |= static_cast<uint64_t>(rng.next()) << 32;
        unsigned pos = static_cast<unsigned>(w2 % n);
        for (unsigned guard = 0; ((result >> pos) & 1u) == static_cast<uint64_t>(diff > 0) && guard < 64; guard++)
            pos = (pos + 1) % n;
        result ^= 1ull << pos;
        diff += diff > 0 ? -1 : 1;
    }
    return result;
}

// One Metropolis proposal (include/spin_ensembles/MonteCarloLoop.hpp:153-256): flip
// site `u32 % N` (and a partner with the same new spin under S_z symmetry), update the
// angles of the trial state, accept if Delta > 0 or u <= exp(2 Delta), u drawn only
// when Delta <= 0.
template <int K, int NW, class Rng>
__device__ __forceinline__ bool rbm_mh_step(const RbmDev& P, Spins<NW>& s, float (&tr)[K], float (&ti)[K],
                                            float (&re)[K], Rng& rng, int lane, int total_z, uint64_t nmagic) {
    const uint32_t N = static_cast<uint32_t>(P.N);
    int sites[2];
    int ns = 1;
    sites[0] = static_cast<int>(fastmod(rng.next(), nmagic, N));
    if (total_z) {
        const bool first_new = !s.up(sites[0]);
        int sec = sites[0];
        for (int guard = 0; guard < (1 << 20); guard++) {
            const int c = static_cast<int>(fastmod(rng.next(), nmagic, N));
            const bool v = c == sites[0] ? first_new : s.up(c);
            if (v == first_new) { sec = c; break; }
        }
        sites[1] = sec;
        ns = 2;
    }
    // The trial angles are not kept: each is formed, evaluated and dropped, and on the
    // (rare) accept they are formed again -- bit-identical -- to commit.  Only theta and
    // Re f(theta) stay live, which keeps the register footprint low.
    Spins<NW> s2 = s;
    float two_s[2];
    const float2* rows[2];
#pragma unroll
    for (int q = 0; q < 2; q++) {
        if (q >= ns) break;
        const int site = q == 0 ? sites[0] : sites[1];
        s2.flip(site);
        two_s[q] = s2.up(site) ? 2.0f : -2.0f;
        rows[q] = P.W + static_cast<long>(site) * P.Mpad + lane;
    }
    float part = 0.0f;
    if (ns == 1) {
        // single flip: the K loads of the W row are issued together
        float2 w[K];
#pragma unroll
        for (int k = 0; k < K; k++) w[k] = __ldg(rows[0] + 32 * k);
#pragma unroll
        for (int k = 0; k < K; k++) {
            const float nr = __fmaf_rn(two_s[0], w[k].x, tr[k]);
            const float ni = __fmaf_rn(two_s[0], w[k].y, ti[k]);
            part = __fadd_rn(part, __fsub_rn(lc_re(nr, ni), re[k]));
        }
    } else {
#pragma unroll
        for (int k = 0; k < K; k++) {
            float nr = tr[k], ni = ti[k];
            for (int q = 0; q < ns; q++) {
                const float2 w = __ldg(rows[q] + 32 * k);
                nr = __fmaf_rn(two_s[q], w.x, nr);
                ni = __fmaf_rn(two_s[q], w.y, ni);
            }
            part = __fadd_rn(part, __fsub_rn(lc_re(nr, ni), re[k]));
        }
    }
    const float delta = warp_sum_xor(part);
    bool accept = delta > 0.0f;
    if (!accept) accept = rng.uniform() <= expf_det(__fmul_rn(2.0f, delta));
    if (accept) {
        s = s2;
#pragma unroll
        for (int k = 0; k < K; k++) {
            for (int q = 0; q < ns; q++) {
                const float2 w = __ldg(rows[q] + 32 * k);
                tr[k] = __fmaf_rn(two_s[q], w.x, tr[k]);
                ti[k] = __fmaf_rn(two_s[q], w.y, ti[k]);
            }
            re[k] = lc_re(tr[k], ti[k]);
        }
    }
    return accept;
}

// ---------------------------------------------------------------------------
// The sampler's form of the above on packed pairs (device_math.cuh: pair_t, FP32x2):
// pair kk of a lane holds hidden units k = 2 kk and 2 kk + 1; every half is computed with
// the scalar form's operations in its order, so angles, Re f and the decision are the
// scalar ones bit for bit.  KP = ceil(K / 2); for odd K the last pair's second unit is a
// zero row (W and b padded) that enters no sum.
// ---------------------------------------------------------------------------
template <int KP, int NW>
__device__ __forceinline__ void rbm_refresh2(const RbmDev& P, const Spins<NW>& s, pair_t (&tr)[KP],
                                             pair_t (&ti)[KP], int lane) {
#pragma unroll
    for (int kk = 0; kk < KP; kk++) {
        const float4 b = __ldg(P.bq + kk * 32 + lane);
        tr[kk] = pk2(b.x, b.y);
        ti[kk] = pk2(b.z, b.w);
    }
    const float4* row = P.Wq + lane;
    for (int i = 0; i < P.N; i++, row += KP * 32) {
        const pair_t sg = splat2(s.up(i) ? 1.0f : -1.0f);
#pragma unroll
        for (int kk = 0; kk < KP; kk++) {
            const float4 w = __ldg(row + 32 * kk);
            tr[kk] = fma2(sg, pk2(w.x, w.y), tr[kk]);   // sg = +-1: the products are exact
            ti[kk] = fma2(sg, pk2(w.z, w.w), ti[kk]);
        }
    }
}

template <int K, int KP, int NW, class Rng>
__device__ __forceinline__ bool rbm_mh_step2(const RbmDev& P, Spins<NW>& s, pair_t (&tr)[KP], pair_t (&ti)[KP],
                                             pair_t (&re)[KP], Rng& rng, int lane, int total_z, uint64_t nmagic) {
    const uint32_t N = static_cast<uint32_t>(P.N);
    int sites[2];
    int ns = 1;
    sites[0] = static_cast<int>(fastmod(rng.next(), nmagic, N));
    if (total_z) {
        const bool first_new = !s.up(sites[0]);
        int sec = sites[0];
        for (int guard = 0; guard < (1 << 20); guard++) {
            const int c = static_cast<int>(fastmod(rng.next(), nmagic, N));
            const bool v = c == sites[0] ? first_new : s.up(c);
            if (v == first_new) { sec = c; break; }
        }
        sites[1] = sec;
        ns = 2;
    }
    Spins<NW> s2 = s;
    pair_t two_s[2];
    const float4* rows[2];
#pragma unroll
    for (int q = 0; q < 2; q++) {
        if (q >= ns) break;
        const int site = q == 0 ? sites[0] : sites[1];
        s2.flip(site);
        two_s[q] = splat2(s2.up(site) ? 2.0f : -2.0f);
        rows[q] = P.Wq + static_cast<long>(site) * KP * 32 + lane;
    }
    float part = 0.0f;
    pair_t fnew[KP];   // Re f of the proposed angles
    if (ns == 1) {
        // single flip: the KP loads of the paired W row are issued together
        float4 w[KP];
#pragma unroll
        for (int kk = 0; kk < KP; kk++) w[kk] = __ldg(rows[0] + 32 * kk);
#pragma unroll
        for (int kk = 0; kk < KP; kk++) {
            const pair_t nr = fma2(two_s[0], pk2(w[kk].x, w[kk].y), tr[kk]);
            const pair_t ni = fma2(two_s[0], pk2(w[kk].z, w[kk].w), ti[kk]);
            fnew[kk] = lc_re2(nr, ni);
            float d0, d1;
            up2(sub2(fnew[kk], re[kk]), d0, d1);
            part = __fadd_rn(part, d0);
            if (2 * kk + 1 < K) part = __fadd_rn(part, d1);
        }
    } else {
#pragma unroll
        for (int kk = 0; kk < KP; kk++) {
            pair_t nr = tr[kk], ni = ti[kk];
            for (int q = 0; q < ns; q++) {
                const float4 w = __ldg(rows[q] + 32 * kk);
                nr = fma2(two_s[q], pk2(w.x, w.y), nr);
                ni = fma2(two_s[q], pk2(w.z, w.w), ni);
            }
            fnew[kk] = lc_re2(nr, ni);
            float d0, d1;
            up2(sub2(fnew[kk], re[kk]), d0, d1);
            part = __fadd_rn(part, d0);
            if (2 * kk + 1 < K) part = __fadd_rn(part, d1);
        }
    }
    const float delta = warp_sum_xor(part);
    bool accept = delta > 0.0f;
    if (!accept) accept = rng.uniform() <= expf_det(__fmul_rn(2.0f, delta));
    if (accept) {
        s = s2;
#pragma unroll
        for (int kk = 0; kk < KP; kk++) {
            for (int q = 0; q < ns; q++) {
                const float4 w = __ldg(rows[q] + 32 * kk);
                tr[kk] = fma2(two_s[q], pk2(w.x, w.y), tr[kk]);
                ti[kk] = fma2(two_s[q], pk2(w.z, w.w), ti[kk]);
            }
            // lc_re2 of the new angles, formed by the same operations: kept from the proposal
            // where the registers allow (the larger layers take rbm_mc_smem_kernel's buffers)
            re[kk] = K <= 8 ? fnew[kk] : lc_re2(tr[kk], ti[kk]);
        }
    }
    return accept;
}

// The single-flip proposal of rbm_mh_step2 with the walker's angles and Re f in this
// warp's shared-memory slice st [4][KP][32] pairs (theta re, theta im, Re f in two buffers)
// instead of registers: the same operations in the same order, so the same chain bit for
// bit.  It frees ~3 KP registers per lane, which for the large hidden layers lets more warps
// stay resident to hide the dependent chain of each proposal.  Buffer cur holds the walker's
// Re f.  KEEP: the proposal writes its Re f(theta') into the other buffer, and an accepted
// move takes that buffer as is (the values that recomputing from the new angles gives, bit
// for bit) and only advances the angles; otherwise an accepted move recomputes Re f in
// place.  Keeping costs KP stores per proposal and a quarter more shared memory (less L1 for
// the W rows), and saves KP activations per acceptance: measured on N = 100, M = 416 and
// 16384 walkers, 10 sweeps take 12.60 ms kept against 13.26 ms recomputed at an acceptance
// of 0.235 (sigma 0.05 weights), but 12.44 against 11.79 ms at 0.026 (sigma 0.1).  The
// sampler keeps; a per-warp switch on the running acceptance measured worse in both cases.
template <int K, int KP, bool KEEP, int NW>
__device__ __forceinline__ bool rbm_flip_step_s(const RbmDev& P, Spins<NW>& s, pair_t* st, int& cur, WarpRng& rng,
                                                int lane, uint64_t nmagic) {
    const int site = static_cast<int>(fastmod(rng.next(), nmagic, static_cast<uint32_t>(P.N)));
    const pair_t two_s = splat2(s.up(site) ? -2.0f : 2.0f);   // 2 x the new spin
    const float4* row = P.Wq + static_cast<long>(site) * KP * 32 + lane;
    pair_t* re = st + (2 + cur) * KP * 32 + lane;
    pair_t* re_new = st + (3 - cur) * KP * 32 + lane;
    float4 w[KP];
#pragma unroll
    for (int kk = 0; kk < KP; kk++) w[kk] = __ldg(row + 32 * kk);
    float part = 0.0f;
#pragma unroll
    for (int kk = 0; kk < KP; kk++) {
        const pair_t nr = fma2(two_s, pk2(w[kk].x, w[kk].y), st[kk * 32 + lane]);
        const pair_t ni = fma2(two_s, pk2(w[kk].z, w[kk].w), st[(KP + kk) * 32 + lane]);
        const pair_t f = lc_re2(nr, ni);
        if (KEEP) re_new[kk * 32] = f;
        float d0, d1;
        up2(sub2(f, re[kk * 32]), d0, d1);
        part = __fadd_rn(part, d0);
        if (2 * kk + 1 < K) part = __fadd_rn(part, d1);
    }
    const float delta = warp_sum_xor(part);
    bool accept = delta > 0.0f;
    if (!accept) accept = rng.uniform() <= expf_det(__fmul_rn(2.0f, delta));
    if (accept) {
        s.flip(site);
        if (KEEP) cur ^= 1;
#pragma unroll
        for (int kk = 0; kk < KP; kk++) {
            const float4 ww = __ldg(row + 32 * kk);
            const pair_t tr = fma2(two_s, pk2(ww.x, ww.y), st[kk * 32 + lane]);
            const pair_t ti = fma2(two_s, pk2(ww.z, ww.w), st[(KP + kk) * 32 + lane]);
            st[kk * 32 + lane] = tr;
            st[(KP + kk) * 32 + lane] = ti;
            if (!KEEP) re[kk * 32] = lc_re2(tr, ti);
        }
    }
    return accept;
}

// One update of the fast sweep (MonteCarloLoop.hpp:162-171): the proposal flips the spins
// of a mask that is the AND of `tries` random configurations (each spin flips with
// probability 2^-tries; the mask is warp-uniform).  Unlike the reference, whose Psi keeps
// its angles unchanged for these moves, the proposal's angles follow every flipped site in
// increasing order (theta += 2 s'_i W_i), and the move is accepted on the change of
// Re log psi like a single flip.
template <int K, int KP, int NW, class Rng>
__device__ __forceinline__ bool rbm_fast_step2(const RbmDev& P, Spins<NW>& s, pair_t (&tr)[KP], pair_t (&ti)[KP],
                                               pair_t (&re)[KP], Rng& rng, int lane, int tries) {
    Spins<NW> mask;
    draw_spins(rng, P.N, mask);
    for (int t = 1; t < tries; t++) {
        Spins<NW> m2;
        draw_spins(rng, P.N, m2);
#pragma unroll
        for (int k = 0; k < NW; k++) mask.w[k] &= m2.w[k];
    }
    Spins<NW> s2 = s;
    pair_t nr[KP], ni[KP];
#pragma unroll
    for (int kk = 0; kk < KP; kk++) {
        nr[kk] = tr[kk];
        ni[kk] = ti[kk];
    }
#pragma unroll
    for (int k = 0; k < NW; k++) {
        uint64_t m = mask.w[k];
        while (m) {
            const int site = 64 * k + (__ffsll(static_cast<long long>(m)) - 1);
            m &= m - 1;
            s2.flip(site);
            const pair_t two_s = splat2(s2.up(site) ? 2.0f : -2.0f);
            const float4* row = P.Wq + static_cast<long>(site) * KP * 32 + lane;
#pragma unroll
            for (int kk = 0; kk < KP; kk++) {
                const float4 w = __ldg(row + 32 * kk);
                nr[kk] = fma2(two_s, pk2(w.x, w.y), nr[kk]);
                ni[kk] = fma2(two_s, pk2(w.z, w.w), ni[kk]);
            }
        }
    }
    pair_t nre[KP];
    float part = 0.0f;
#pragma unroll
    for (int kk = 0; kk < KP; kk++) {
        nre[kk] = lc_re2(nr[kk], ni[kk]);
        float d0, d1;
        up2(sub2(nre[kk], re[kk]), d0, d1);
        part = __fadd_rn(part, d0);
        if (2 * kk + 1 < K) part = __fadd_rn(part, d1);
    }
    const float delta = warp_sum_xor(part);
    bool accept = delta > 0.0f;
    if (!accept) accept = rng.uniform() <= expf_det(__fmul_rn(2.0f, delta));
    if (accept) {
        s = s2;
#pragma unroll
        for (int kk = 0; kk < KP; kk++) {
            tr[kk] = nr[kk];
            ti[kk] = ni[kk];
            re[kk] = nre[kk];
        }
    }
    return accept;
}

// sign * (-i)^ypow * coef of string n for the current (original) spins, in FP32: the
// local-energy sums run in FP32 with compensated (Kahan) accumulation, since GB300's
// FP64 rate is 1/64 of its FP32 rate and every lane of the warp executes the sum
template <int NW>
__device__ __forceinline__ float2 string_factor(const OpDev& op, int n, const Spins<NW>& s) {
    int parity = 0;
#pragma unroll
    for (int k = 0; k < NW; k++) parity += __popcll(op.zmask[n * kMaxWords + k] & ~s.w[k]);
    const float2 c = op.coef32[n];
    const int yp = op.ypow[n] & 3;
    float2 r;
    if (yp == 0) r = c;
    else if (yp == 1) r = make_float2(c.y, -c.x);
    else if (yp == 2) r = make_float2(-c.x, -c.y);
    else r = make_float2(-c.y, c.x);
    return (parity & 1) ? make_float2(-r.x, -r.y) : r;
}

// compensated FP32 sum (Kahan 1965): the represented value is s - c
struct KahanC {
    float sr = 0.0f, si = 0.0f, cr = 0.0f, ci = 0.0f;
    __device__ __forceinline__ void add(float x, float y) {
        const float yr = __fsub_rn(x, cr), yi = __fsub_rn(y, ci);
        const float tr = __fadd_rn(sr, yr), ti = __fadd_rn(si, yi);
        cr = __fsub_rn(__fsub_rn(tr, sr), yr);
        ci = __fsub_rn(__fsub_rn(ti, si), yi);
        sr = tr;
        si = ti;
    }
    __device__ __forceinline__ double2 value() const {
        return make_double2(static_cast<double>(sr) - static_cast<double>(cr),
                            static_cast<double>(si) - static_cast<double>(ci));
    }
};

// coef * exp(d) for the complex log-ratio d
__device__ __forceinline__ float2 string_term(float2 cf, float2 d) {
    float sn, cs;
    sincosf(d.y, &sn, &cs);
    const float mag = expf(d.x);
    const float xr = mag * cs, xi = mag * sn;
    return make_float2(fmaf(cf.x, xr, -cf.y * xi), fmaf(cf.x, xi, cf.y * xr));
}

// Local energy E_loc(s) = sum_n coef_n phase_n exp(log psi(s'_n) - log psi(s))
// (include/operator/Operator.hpp:90-115).  Diagonal strings contribute coef * phase
// exactly.  With GRAD, also accumulates U_j = sum_n e_n tanh(theta'_nj) (the E_k term,
// Operator.hpp:145-179) and stores X[slot][j] = e_n tanh(theta'_nj) per off-diagonal string.
template <bool GRAD, int K, int NW>
__device__ __forceinline__ double2 rbm_local_energy(const RbmDev& P, const OpDev& op, const Spins<NW>& s,
                                                    const float (&tr)[K], const float (&ti)[K],
                                                    const float2 (&f)[K], const float2 (&T)[K], float2 (&U)[K],
                                                    float2* X, int lane) {
    KahanC acc;
    if (GRAD) {
#pragma unroll
        for (int k = 0; k < K; k++) U[k] = make_float2(0.0f, 0.0f);
    }
    for (int n = 0; n < op.S; n++) {
        const float2 cf = string_factor(op, n, s);
        const int nf = op.nflip[n];
        if (nf == 0) {
            acc.add(cf.x, cf.y);
            if (GRAD) {
                const float ex = cf.x, ey = cf.y;
#pragma unroll
                for (int k = 0; k < K; k++) {
                    U[k].x += ex * T[k].x - ey * T[k].y;
                    U[k].y += ex * T[k].y + ey * T[k].x;
                }
            }
            continue;
        }
        float nr[K], ni[K];
#pragma unroll
        for (int k = 0; k < K; k++) { nr[k] = tr[k]; ni[k] = ti[k]; }
        const int off = op.flip_off[n];
        for (int q = 0; q < nf; q++) {
            const int site = op.flip_sites[off + q];
            const float two_s = s.up(site) ? -2.0f : 2.0f;   // new spin = -old
            const float2* row = P.W + static_cast<long>(site) * P.Mpad + lane;
#pragma unroll
            for (int k = 0; k < K; k++) {
                const float2 w = __ldg(row + 32 * k);
                nr[k] = fmaf(two_s, w.x, nr[k]);
                ni[k] = fmaf(two_s, w.y, ni[k]);
            }
        }
        float2 part = make_float2(0.0f, 0.0f);
        float2 th[GRAD ? K : 1];
#pragma unroll
        for (int k = 0; k < K; k++) {
            float2 g;
            if (GRAD) {
                // f and tanh of the flipped angle from one denominator (lc_tanh_approx)
                lc_tanh_approx(nr[k], ni[k], g, th[k]);
            } else {
                g = lc_c(nr[k], ni[k]);
            }
            part.x += g.x - f[k].x;
            part.y += g.y - f[k].y;
        }
        const float2 e = string_term(cf, warp_sum_xor2(part));
        acc.add(e.x, e.y);
        if (GRAD) {
            const float ex = e.x, ey = e.y;
            float2* xrow = X + static_cast<long>(op.offdiag_slot[n]) * P.Mpad + lane;
#pragma unroll
            for (int k = 0; k < K; k++) {
                const float2 t2 = th[k];
                const float2 v = make_float2(ex * t2.x - ey * t2.y, ex * t2.y + ey * t2.x);
                U[k].x += v.x;
                U[k].y += v.y;
                xrow[32 * k] = v;
            }
        }
    }
    return acc.value();
}

template <int K>
__device__ __forceinline__ double2 warp_log_psi(const float2 (&f)[K]) {
    float2 acc = make_float2(0.0f, 0.0f);
#pragma unroll
    for (int k = 0; k < K; k++) { acc.x += f[k].x; acc.y += f[k].y; }
    acc = warp_sum_xor2(acc);
    return make_double2(acc.x, acc.y);
}

// ---------------------------------------------------------------------------
// Metropolis sampler: one warp per walker for a whole launch
// (include/spin_ensembles/MonteCarloLoop.hpp:55-138).  The angles are recomputed
// from the spins at the start of every sweep.  Measurements (local energies, log psi)
// are a separate pass (rbm_est_kernel) over the recorded configurations, which keeps
// the sampler's register footprint to the walker state.
// ---------------------------------------------------------------------------
template <int K, int NW>
__global__ void __launch_bounds__(32 * kWarpsPerBlock, K > 13 ? 3 : 4) rbm_mc_kernel(RbmDev P, McLaunch L) {
    const int lane = threadIdx.x & 31;
    const int w = blockIdx.x * kWarpsPerBlock + (threadIdx.x >> 5);
    if (w >= L.B) return;
    WarpRng rng;
    rng.init(L.seed, L.walker_base + static_cast<uint32_t>(w), L.rng_index[w], lane);
    const uint64_t nmagic = fastmod_magic(static_cast<uint32_t>(P.N));
    Spins<NW> s;
    if (L.init) {
#pragma unroll
        for (int k = 0; k < NW; k++) s.w[k] = 0;
        if (L.total_z) s.w[0] = draw_n_over_k(rng, P.N, static_cast<unsigned>((L.sector + P.N) / 2));
        else draw_spins(rng, P.N, s);
    } else {
#pragma unroll
        for (int k = 0; k < NW; k++) s.w[k] = L.spins[static_cast<long>(w) * NW + k];
    }
    constexpr int KP = (K + 1) / 2;
    pair_t tr[KP], ti[KP], re[KP];
    unsigned long long acc = 0, props = 0;
    const int total_sweeps = L.n_therm + L.n_samples * L.sweeps_per_sample;
    int sample = 0;
    for (int sw = 0; sw < total_sweeps; sw++) {
        rbm_refresh2(P, s, tr, ti, lane);
#pragma unroll
        for (int kk = 0; kk < KP; kk++) re[kk] = lc_re2(tr[kk], ti[kk]);
        for (int p = 0; p < P.N; p++)
            acc += rbm_mh_step2<K>(P, s, tr, ti, re, rng, lane, L.total_z, nmagic);
        props += P.N;
        const int done = sw + 1 - L.n_therm;
        if (done > 0 && done % L.sweeps_per_sample == 0) {
            const long row = static_cast<long>(L.sample_base + sample) * L.B + w;
            if (L.sample_spins && lane == 0) {
#pragma unroll
                for (int k = 0; k < NW; k++) L.sample_spins[row * NW + k] = s.w[k];
            }
            sample++;
        }
    }
    if (lane == 0) {
#pragma unroll
        for (int k = 0; k < NW; k++) L.spins[static_cast<long>(w) * NW + k] = s.w[k];
        L.rng_index[w] = rng.index;
        L.accepts[w] += acc;
        L.proposals[w] += props;
    }
}

// The sampler for large hidden layers (K >= 13) without the S_z constraint: the walker
// state in shared memory (rbm_flip_step_s), 6 blocks of 4 warps per SM instead of 4 (3).
// Chains, samples and counters are those of rbm_mc_kernel.
template <int K, int NW>
__global__ void __launch_bounds__(32 * kWarpsPerBlock, 6) rbm_mc_smem_kernel(RbmDev P, McLaunch L) {
    const int lane = threadIdx.x & 31;
    const int w = blockIdx.x * kWarpsPerBlock + (threadIdx.x >> 5);
    if (w >= L.B) return;
    constexpr int KP = (K + 1) / 2;
    extern __shared__ pair_t s_state[];
    pair_t* st = s_state + (threadIdx.x >> 5) * 4 * KP * 32;
    int cur = 0;
    WarpRng rng;
    rng.init(L.seed, L.walker_base + static_cast<uint32_t>(w), L.rng_index[w], lane);
    const uint64_t nmagic = fastmod_magic(static_cast<uint32_t>(P.N));
    Spins<NW> s;
    if (L.init) {
#pragma unroll
        for (int k = 0; k < NW; k++) s.w[k] = 0;
        draw_spins(rng, P.N, s);
    } else {
#pragma unroll
        for (int k = 0; k < NW; k++) s.w[k] = L.spins[static_cast<long>(w) * NW + k];
    }
    unsigned long long acc = 0, props = 0;
    const int total_sweeps = L.n_therm + L.n_samples * L.sweeps_per_sample;
    int sample = 0;
    for (int sw = 0; sw < total_sweeps; sw++) {
        {
            pair_t tr[KP], ti[KP];
            rbm_refresh2(P, s, tr, ti, lane);
            cur = 0;
#pragma unroll
            for (int kk = 0; kk < KP; kk++) {
                st[kk * 32 + lane] = tr[kk];
                st[(KP + kk) * 32 + lane] = ti[kk];
                st[(2 * KP + kk) * 32 + lane] = lc_re2(tr[kk], ti[kk]);
            }
        }
        for (int p = 0; p < P.N; p++) acc += rbm_flip_step_s<K, KP, true>(P, s, st, cur, rng, lane, nmagic);
        props += P.N;
        const int done = sw + 1 - L.n_therm;
        if (done > 0 && done % L.sweeps_per_sample == 0) {
            const long row = static_cast<long>(L.sample_base + sample) * L.B + w;
            if (L.sample_spins && lane == 0) {
#pragma unroll
                for (int k = 0; k < NW; k++) L.sample_spins[row * NW + k] = s.w[k];
            }
            sample++;
        }
    }
    if (lane == 0) {
#pragma unroll
        for (int k = 0; k < NW; k++) L.spins[static_cast<long>(w) * NW + k] = s.w[k];
        L.rng_index[w] = rng.index;
        L.accepts[w] += acc;
        L.proposals[w] += props;
    }
}

// Fast-sweep sampler (MonteCarloLoop::set_fast_sweep, MonteCarloLoop.hpp:108-113, 139-151,
// 162-171): a thermalisation sweep is N mask updates, a sampling sweep one.  The angles are
// recomputed from the spins every N updates of the thermalisation and at the start of every
// sample's updates (and every N updates within them).
template <int K, int NW>
__global__ void __launch_bounds__(32 * kWarpsPerBlock, K > 13 ? 3 : 4) rbm_mc_fast_kernel(RbmDev P, McLaunch L) {
    const int lane = threadIdx.x & 31;
    const int w = blockIdx.x * kWarpsPerBlock + (threadIdx.x >> 5);
    if (w >= L.B) return;
    WarpRng rng;
    rng.init(L.seed, L.walker_base + static_cast<uint32_t>(w), L.rng_index[w], lane);
    Spins<NW> s;
    if (L.init) {
#pragma unroll
        for (int k = 0; k < NW; k++) s.w[k] = 0;
        draw_spins(rng, P.N, s);
    } else {
#pragma unroll
        for (int k = 0; k < NW; k++) s.w[k] = L.spins[static_cast<long>(w) * NW + k];
    }
    constexpr int KP = (K + 1) / 2;
    pair_t tr[KP], ti[KP], re[KP];
    unsigned long long acc = 0, props = 0;
    auto refresh = [&]() {
        rbm_refresh2(P, s, tr, ti, lane);
#pragma unroll
        for (int kk = 0; kk < KP; kk++) re[kk] = lc_re2(tr[kk], ti[kk]);
    };
    for (int sw = 0; sw < L.n_therm; sw++) {
        refresh();
        for (int p = 0; p < P.N; p++) acc += rbm_fast_step2<K>(P, s, tr, ti, re, rng, lane, L.fast_tries);
        props += P.N;
    }
    for (int sample = 0; sample < L.n_samples; sample++) {
        for (int u = 0; u < L.sweeps_per_sample; u++) {
            if (u % P.N == 0) refresh();
            acc += rbm_fast_step2<K>(P, s, tr, ti, re, rng, lane, L.fast_tries);
        }
        props += L.sweeps_per_sample;
        const long row = static_cast<long>(L.sample_base + sample) * L.B + w;
        if (L.sample_spins && lane == 0) {
#pragma unroll
            for (int k = 0; k < NW; k++) L.sample_spins[row * NW + k] = s.w[k];
        }
    }
    if (lane == 0) {
#pragma unroll
        for (int k = 0; k < NW; k++) L.spins[static_cast<long>(w) * NW + k] = s.w[k];
        L.rng_index[w] = rng.index;
        L.accepts[w] += acc;
        L.proposals[w] += props;
    }
}

// ---------------------------------------------------------------------------
// Estimator pass over given configurations (one warp each): local energy, log psi,
// the O_k vectors T = tanh(theta), the E_k vectors U and X, and psi' quantities for
// the Hilbert-space distance.
// ---------------------------------------------------------------------------
template <int K, int NW>
__global__ void __launch_bounds__(32 * kWarpsPerBlock) rbm_est_kernel(RbmDev P, OpDev op, int has_op, RbmDev PP,
                                                                       EstLaunch L) {
    const int lane = threadIdx.x & 31;
    const long t = static_cast<long>(blockIdx.x) * kWarpsPerBlock + (threadIdx.x >> 5);
    if (t >= L.count) return;
    Spins<NW> s;
    if (L.flags & EST_ENUMERATE) {
        const uint64_t idx = L.enum_base + static_cast<uint64_t>(t);
        s.w[0] = P.N >= 64 ? idx : (idx & ((1ull << P.N) - 1ull));
#pragma unroll
        for (int k = 1; k < NW; k++) s.w[k] = 0;
    } else {
#pragma unroll
        for (int k = 0; k < NW; k++) s.w[k] = L.spins[t * NW + k];
    }
    if (L.flags & (EST_ELOC | EST_LOGPSI | EST_GRADVEC)) {
        float tr[K], ti[K];
        rbm_refresh(P, s, tr, ti, lane);
        float2 f[K], T[K], U[K];
        const bool grad = (L.flags & EST_GRADVEC) != 0;
#pragma unroll
        for (int k = 0; k < K; k++) {
            // with the O_k vectors: f and tanh from one denominator, the same evaluation as
            // the flipped angles' in rbm_local_energy<true> (so that unchanged units cancel)
            if (grad) lc_tanh_approx(tr[k], ti[k], f[k], T[k]);
            else f[k] = lc_c(tr[k], ti[k]);
        }
        if (L.flags & EST_LOGPSI) {
            const double2 lp = warp_log_psi(f);
            if (lane == 0) L.logpsi[t] = lp;
        }
        if (grad) {
#pragma unroll
            for (int k = 0; k < K; k++) L.T[t * P.Mpad + lane + 32 * k] = T[k];
            const double2 e = rbm_local_energy<true>(P, op, s, tr, ti, f, T, U,
                                                     L.X + t * op.num_offdiag * P.Mpad, lane);
            const float shx = static_cast<float>(L.e_shift.x), shy = static_cast<float>(L.e_shift.y);
#pragma unroll
            for (int k = 0; k < K; k++) {
                U[k].x -= shx * T[k].x - shy * T[k].y;
                U[k].y -= shx * T[k].y + shy * T[k].x;
                L.U[t * P.Mpad + lane + 32 * k] = U[k];
            }
            if (lane == 0 && L.eloc) L.eloc[t] = e;
        } else if ((L.flags & EST_ELOC) && has_op) {
            const double2 e = rbm_local_energy<false>(P, op, s, tr, ti, f, T, U, nullptr, lane);
            if (lane == 0) L.eloc[t] = e;
        }
    }
    if (L.flags & EST_PRIME) {
        float pr[K], pi[K];
        rbm_refresh(PP, s, pr, pi, lane);
        float2 fp[K];
#pragma unroll
        for (int k = 0; k < K; k++) fp[k] = lc_c(pr[k], pi[k]);
        const double2 lp = warp_log_psi(fp);
        if (lane == 0) L.logpsi_prime[t] = lp;
        if (L.Tp) {
#pragma unroll
            for (int k = 0; k < K; k++) L.Tp[t * PP.Mpad + lane + 32 * k] = tanh_c(pr[k], pi[k]);
        }
    }
}

// ---------------------------------------------------------------------------
// Local energies only (the measurement of a chain step, Operator.hpp:90-115), the lanes
// over the strings: one warp per configuration; its angles
// and f(theta) sit in the warp's shared-memory slice, and every lane evaluates the whole
// log-ratio of its own (off-diagonal string, quarter of the hidden units) item: units
// j = q, q + 4, ... two at a time on FP32x2 pairs (j and j + 4), the flipped angles from the
// transposed W (the lanes of a round read neighbouring spins of the same unit rows), the
// differences f(theta'') - f(theta) summed in pairs (104 units a lane at M = 400; the
// reciprocal of the activation's denominator is the hardware's approximation, within an
// ulp).  Two shuffles join a
// string's quarters; one warp reduction per configuration joins the strings.  No
// per-string reduction sits on the critical path, and each lane's loop over units is
// independent work.
// ---------------------------------------------------------------------------
template <int K, int NW>
__global__ void __launch_bounds__(32 * kWarpsPerBlock) rbm_eloc_t_kernel(RbmDev P, OpDev op, EstLaunch L) {
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const long t = static_cast<long>(blockIdx.x) * kWarpsPerBlock + wib;
    if (t >= L.count) return;
    Spins<NW> s;
    if (L.flags & EST_ENUMERATE) {
        const uint64_t idx = L.enum_base + static_cast<uint64_t>(t);
        s.w[0] = P.N >= 64 ? idx : (idx & ((1ull << P.N) - 1ull));
#pragma unroll
        for (int k = 1; k < NW; k++) s.w[k] = 0;
    } else {
#pragma unroll
        for (int k = 0; k < NW; k++) s.w[k] = L.spins[t * NW + k];
    }
    constexpr int KP = (K + 1) / 2;
    constexpr int MP = 32 * K;
    // the angles and f of every unit in the warp's slice, units j and j + 4 side by side
    // (the pairs the loops below evaluate): pair p = 4 (j / 8) + j % 4 holds
    // tA[p] = (theta.re_j, theta.re_j+4, theta.im_j, theta.im_j+4) and
    // tB[p] = (f.re_j, f.re_j+4, f.im_j, f.im_j+4)
    __shared__ float4 tf_sm[kWarpsPerBlock][MP];
    float4* tA = tf_sm[wib];
    float4* tB = tA + MP / 2;
    {
        // a lane's pair kk holds units lane + 64 kk and lane + 64 kk + 32
        pair_t tr[KP], ti[KP];
        rbm_refresh2(P, s, tr, ti, lane);
        float* fa = reinterpret_cast<float*>(tA);
        float* fb = reinterpret_cast<float*>(tB);
        auto put = [&](int j, float a, float b, float r, float i) {
            const int p = 4 * (j >> 3) + (j & 3), h = (j >> 2) & 1;
            fa[4 * p + h] = a;
            fa[4 * p + 2 + h] = b;
            fb[4 * p + h] = r;
            fb[4 * p + 2 + h] = i;
        };
#pragma unroll
        for (int kk = 0; kk < KP; kk++) {
            // f(theta) with the same approximate reciprocal as f(theta'') below
            const Pair2 v = lc_c2_approx(tr[kk], ti[kk]);
            float a0, a1, b0, b1, r0, r1, i0, i1;
            up2(tr[kk], a0, a1);
            up2(ti[kk], b0, b1);
            up2(v.re, r0, r1);
            up2(v.im, i0, i1);
            const int j0 = lane + 64 * kk;
            put(j0, a0, b0, r0, i0);
            if (2 * kk + 1 < K) put(j0 + 32, a1, b1, r1, i1);
        }
    }
    __syncwarp();
    KahanC acc;
    // diagonal strings: the lanes over the strings
    for (int n = lane; n < op.S; n += 32) {
        if (op.nflip[n] == 0) {
            const float2 cf = string_factor(op, n, s);
            acc.add(cf.x, cf.y);
        }
    }
    const int items = 4 * op.num_offdiag;
    const int N = P.N;
    for (int it0 = 0; it0 < items; it0 += 32) {
        const int it = it0 + lane;
        const bool live = it < items;
        const int n = live ? op.offdiag[it >> 2] : 0;
        const int q = it & 3;
        // sums of the real and imaginary differences on pairs (units j, j + 4)
        pair_t sr = splat2(0.0f), si = sr;
        if (live) {
            const int nf = op.nflip[n];
            const int off = op.flip_off[n];
            // pairs p = q, q + 4, ...: units (j, j + 4), j = q, q + 8, ...
            if (nf == 1) {
                const int site = op.flip_sites[off];
                const pair_t two_s = splat2(s.up(site) ? -2.0f : 2.0f);
                const float4* wcol = P.Wt4 + site;
#pragma unroll 2
                for (int p = q; p < MP / 2; p += 4) {
                    const float4 w = __ldg(wcol + static_cast<long>(p) * N);
                    const float4 a = tA[p], f = tB[p];
                    const Pair2 g = lc_c2_approx(fma2(two_s, pk2(w.x, w.y), pk2(a.x, a.y)),
                                                 fma2(two_s, pk2(w.z, w.w), pk2(a.z, a.w)));
                    sr = add2(sr, sub2(g.re, pk2(f.x, f.y)));
                    si = add2(si, sub2(g.im, pk2(f.z, f.w)));
                }
            } else {
                for (int p = q; p < MP / 2; p += 4) {
                    const float4 a = tA[p], f = tB[p];
                    pair_t xr = pk2(a.x, a.y), xi = pk2(a.z, a.w);
                    for (int u = 0; u < nf; u++) {
                        const int site = op.flip_sites[off + u];
                        const pair_t two_s = splat2(s.up(site) ? -2.0f : 2.0f);
                        const float4 w = __ldg(P.Wt4 + static_cast<long>(p) * N + site);
                        xr = fma2(two_s, pk2(w.x, w.y), xr);
                        xi = fma2(two_s, pk2(w.z, w.w), xi);
                    }
                    const Pair2 g = lc_c2_approx(xr, xi);
                    sr = add2(sr, sub2(g.re, pk2(f.x, f.y)));
                    si = add2(si, sub2(g.im, pk2(f.z, f.w)));
                }
            }
        }
        float r0, r1, i0, i1;
        up2(sr, r0, r1);
        up2(si, i0, i1);
        float dx = r0 + r1, dy = i0 + i1;
        // the four quarters of a string are lanes 4m .. 4m + 3
        dx += __shfl_xor_sync(0xffffffffu, dx, 1);
        dy += __shfl_xor_sync(0xffffffffu, dy, 1);
        dx += __shfl_xor_sync(0xffffffffu, dx, 2);
        dy += __shfl_xor_sync(0xffffffffu, dy, 2);
        if (live && q == 0) {
            const float2 e = string_term(string_factor(op, n, s), make_float2(dx, dy));
            acc.add(e.x, e.y);
        }
    }
    double2 v = acc.value();
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1) {
        v.x += __shfl_xor_sync(0xffffffffu, v.x, o);
        v.y += __shfl_xor_sync(0xffffffffu, v.y, o);
    }
    if (lane == 0) L.eloc[t] = v;
}

// ---------------------------------------------------------------------------
// launchers for this K (instantiated by rbm_k<K>.cu)
// ---------------------------------------------------------------------------
template <int K>
cudaError_t rbm_mc_launch_k(const RbmDev& P, const OpDev* op, const McLaunch& L, cudaStream_t st) {
    const int nw = (P.N + 63) / 64;
    const dim3 grid((L.B + kWarpsPerBlock - 1) / kWarpsPerBlock), block(32 * kWarpsPerBlock);
    (void)op;
    if (L.fast_tries > 0) {
        if (L.total_z) return cudaErrorInvalidValue;
        switch (nw) {
            case 1: rbm_mc_fast_kernel<K, 1><<<grid, block, 0, st>>>(P, L); break;
            case 2: rbm_mc_fast_kernel<K, 2><<<grid, block, 0, st>>>(P, L); break;
            case 3: rbm_mc_fast_kernel<K, 3><<<grid, block, 0, st>>>(P, L); break;
            case 4: rbm_mc_fast_kernel<K, 4><<<grid, block, 0, st>>>(P, L); break;
            default: return cudaErrorInvalidValue;
        }
        return cudaGetLastError();
    }
    if (K >= 13 && !L.total_z) {
        constexpr int KP = (K + 1) / 2;
        const size_t sm = sizeof(pair_t) * 4 * KP * 32 * kWarpsPerBlock;
        switch (nw) {
            case 1: rbm_mc_smem_kernel<K, 1><<<grid, block, sm, st>>>(P, L); break;
            case 2: rbm_mc_smem_kernel<K, 2><<<grid, block, sm, st>>>(P, L); break;
            case 3: rbm_mc_smem_kernel<K, 3><<<grid, block, sm, st>>>(P, L); break;
            case 4: rbm_mc_smem_kernel<K, 4><<<grid, block, sm, st>>>(P, L); break;
            default: return cudaErrorInvalidValue;
        }
        return cudaGetLastError();
    }
    switch (nw) {
        case 1: rbm_mc_kernel<K, 1><<<grid, block, 0, st>>>(P, L); break;
        case 2: rbm_mc_kernel<K, 2><<<grid, block, 0, st>>>(P, L); break;
        case 3: rbm_mc_kernel<K, 3><<<grid, block, 0, st>>>(P, L); break;
        case 4: rbm_mc_kernel<K, 4><<<grid, block, 0, st>>>(P, L); break;
        default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

template <int K>
cudaError_t rbm_est_launch_k(const RbmDev& P, const OpDev* op, const RbmDev* PP, const EstLaunch& L,
                             cudaStream_t st) {
    const int nw = (P.N + 63) / 64;
    const dim3 grid((L.count + kWarpsPerBlock - 1) / kWarpsPerBlock), block(32 * kWarpsPerBlock);
    OpDev o = op ? *op : OpDev{};
    const int has = op != nullptr;
    RbmDev pp = PP ? *PP : P;
    if (has && (L.flags & ~(EST_ELOC | EST_ENUMERATE)) == 0) {
        switch (nw) {
            case 1: rbm_eloc_t_kernel<K, 1><<<grid, block, 0, st>>>(P, o, L); break;
            case 2: rbm_eloc_t_kernel<K, 2><<<grid, block, 0, st>>>(P, o, L); break;
            case 3: rbm_eloc_t_kernel<K, 3><<<grid, block, 0, st>>>(P, o, L); break;
            case 4: rbm_eloc_t_kernel<K, 4><<<grid, block, 0, st>>>(P, o, L); break;
            default: return cudaErrorInvalidValue;
        }
        return cudaGetLastError();
    }
    switch (nw) {
        case 1: rbm_est_kernel<K, 1><<<grid, block, 0, st>>>(P, o, has, pp, L); break;
        case 2: rbm_est_kernel<K, 2><<<grid, block, 0, st>>>(P, o, has, pp, L); break;
        case 3: rbm_est_kernel<K, 3><<<grid, block, 0, st>>>(P, o, has, pp, L); break;
        case 4: rbm_est_kernel<K, 4><<<grid, block, 0, st>>>(P, o, has, pp, L); break;
        default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

}  // namespace rbmg
