// Batched serving of many independent complex RBMs of uneven N and M (extension: the
// reference runs one network per call, include/spin_ensembles/MonteCarloLoop.hpp:294-339).
//
// One persistent launch serves the whole batch.  Its warps take tasks from a global
// queue (one atomic counter): first the walker tasks of every instance, longest first
// (sweeps of single-flip Metropolis, then at the final configuration the local energy,
// tanh(theta), the angles, U_j = sum_n e_n tanh(theta''_nj) over every string and the
// terms e_n of the off-diagonal strings), then the reduction tasks,
// each a tile of rows by a chunk of walkers of one instance's sums, which start once that
// instance's walkers are all done (a per-instance counter; the wait is bounded by a
// wall-clock limit after which the kernel raises an error flag and returns).  Each tile
// writes its chunk's partial sums; a second kernel of the graph adds the chunks in a fixed
// order, so every replay gives the same sums bit for bit.  The walker tasks are compiled
// for each hidden-unit count per lane (1, 2, 4, 8, 13, 18: M <= 576) as separate functions
// of the one kernel.  The launch (counter resets + both kernels) is captured once in a
// CUDA graph and replayed; the warps per block, the reduction tile height and a register
// cap come from an autotuner that times the candidates on the batch itself.
//
// Per instance and replay the result is <E_loc> over its walkers and the reference's O_k
// gradient <E O*> + conj<E_k> - 2 <E> <O*> (source/network_functions/ExpectationValue.cu:
// 243-253), with E_k(s) = sum_n e_n O_k(s'_n) (include/operator/Operator.hpp:145-179): for
// W_ij, s_i (U_j - 2 V_ij) with V_ij = sum of e_n tanh(theta''_nj) over the strings n
// flipping site i, recomputed in the tiles from the stored angles (storing these terms
// per walker and string would move O(N^2 M) bytes per walker through HBM).
// The sums run centred on the instance's mean energy E (the same value in every tile):
//   gO = sum conj(O),  gE = sum (E_w - E) conj(O),  gK = sum conj(E_k) - conj(E) conj(O),
//   gradient = (gE + gK) / W + (conj(E) - E) gO / W.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <memory>
#include <vector>

#include "host.h"
#include "rbm_impl.cuh"

namespace rbmg {
namespace {

constexpr int kSK = 18;   // hidden units per lane at most (Mpad <= 576)
constexpr int kSW = 3;    // spin words at most (N <= 192)

struct SInst {
    int N, M, Mpad, K, nw;
    const float2* W;
    const float2* b;
    const float4* Wq;     // W and b with a lane's hidden units k and k + 1 side by side (kernels.h)
    const float4* bq;
    OpDev op;
    int walkers;
    uint64_t seed;
    double2* eloc;        // [walkers]
    float2* T;            // [walkers][Mpad] tanh(theta)
    float2* U;            // [walkers][Mpad] sum over every string of e_n tanh(theta''_n)
    float2* theta;        // [walkers][Mpad] the angles of the final configuration
    float2* en;           // [walkers][num_offdiag] e_n of the off-diagonal strings
    const int* site_ptr;  // [N + 1] off-diagonal slots flipping each site (CSR)
    const int* site_slots;
    uint64_t* spins;      // [walkers][nw]
    uint64_t* rng_index;  // [walkers]
    int chunks;           // walker chunks of kReduceWalkers
    float2* part;         // [chunks][3][N + 1][Mpad] a chunk's gO, gE, gK (row N: the biases)
    double2* g;           // [3][N + 1][Mpad] the sums over all chunks
    double2* emean;       // [1] the mean local energy the sums are centred on
    unsigned int* done;   // walkers finished in this replay
};

struct STask {
    int kind;    // 0 walker, 1 reduction tile
    int inst;
    int index;   // walker within the instance, or first row of the tile
    int w0;      // reduction tile: first walker of its walker chunk
    int general; // reduction tile: 1 if a row's site is not flipped by exactly one string
                 // that flips that site alone
};

constexpr int kReduceWalkers = 256;   // walkers per reduction tile

struct SLaunch {
    const SInst* inst;
    const STask* tasks;
    int ntasks;
    unsigned int* next;
    int therm, sweeps;    // sweeps before this replay's measurement: therm (first replay) + sweeps
    int first;            // 1: draw the walkers' start spins
    int* error;           // 1: a reduction task gave up waiting
    unsigned long long* accepts;   // [1]
    unsigned long long wait_ns;    // wall-clock limit of a reduction task's wait
    unsigned int wait_extra;       // walkers a reduction task waits for beyond the instance's
                                   // (0; a test sets it so that the wait runs out)
};

__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

template <int K, int NW>
__device__ __forceinline__ void s_refresh(const SInst& I, const Spins<NW>& s, float (&tr)[K], float (&ti)[K],
                                          int lane) {
#pragma unroll
    for (int k = 0; k < K; k++) {
        const float2 b = __ldg(I.b + lane + 32 * k);
        tr[k] = b.x;
        ti[k] = b.y;
    }
    const float2* row = I.W + lane;
    for (int i = 0; i < I.N; i++, row += I.Mpad) {
        const float sg = s.up(i) ? 1.0f : -1.0f;
#pragma unroll
        for (int k = 0; k < K; k++) {
            const float2 w = __ldg(row + 32 * k);
            tr[k] = __fmaf_rn(sg, w.x, tr[k]);   // sg = +-1: the product is exact
            ti[k] = __fmaf_rn(sg, w.y, ti[k]);
        }
    }
}

// the sweeps on packed pairs (rbm_refresh2 / rbm_mh_step2 of the single-network sampler,
// same arithmetic and draw order)
template <int KP, int NW>
__device__ __forceinline__ void s_refresh2(const SInst& I, const Spins<NW>& s, pair_t (&tr)[KP], pair_t (&ti)[KP],
                                           int lane) {
#pragma unroll
    for (int kk = 0; kk < KP; kk++) {
        const float4 b = __ldg(I.bq + kk * 32 + lane);
        tr[kk] = pk2(b.x, b.y);
        ti[kk] = pk2(b.z, b.w);
    }
    const float4* row = I.Wq + lane;
    for (int i = 0; i < I.N; i++, row += KP * 32) {
        const pair_t sg = splat2(s.up(i) ? 1.0f : -1.0f);
#pragma unroll
        for (int kk = 0; kk < KP; kk++) {
            const float4 w = __ldg(row + 32 * kk);
            tr[kk] = fma2(sg, pk2(w.x, w.y), tr[kk]);
            ti[kk] = fma2(sg, pk2(w.z, w.w), ti[kk]);
        }
    }
}

template <int K, int KP, int NW>
__device__ __forceinline__ bool s_mh_step2(const SInst& I, Spins<NW>& s, pair_t (&tr)[KP], pair_t (&ti)[KP],
                                           pair_t (&re)[KP], WarpRng& rng, int lane, uint64_t nmagic) {
    const int site = static_cast<int>(fastmod(rng.next(), nmagic, static_cast<uint32_t>(I.N)));
    Spins<NW> s2 = s;
    s2.flip(site);
    const pair_t two_s = splat2(s2.up(site) ? 2.0f : -2.0f);
    const float4* row = I.Wq + static_cast<long>(site) * KP * 32 + lane;
    float4 w[KP];
#pragma unroll
    for (int kk = 0; kk < KP; kk++) w[kk] = __ldg(row + 32 * kk);
    float part = 0.0f;
    pair_t fnew[KP];   // Re f of the proposed angles
#pragma unroll
    for (int kk = 0; kk < KP; kk++) {
        const pair_t nr = fma2(two_s, pk2(w[kk].x, w[kk].y), tr[kk]);
        const pair_t ni = fma2(two_s, pk2(w[kk].z, w[kk].w), ti[kk]);
        fnew[kk] = lc_re2(nr, ni);
        float d0, d1;
        up2(sub2(fnew[kk], re[kk]), d0, d1);
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
            const float4 ww = __ldg(row + 32 * kk);
            tr[kk] = fma2(two_s, pk2(ww.x, ww.y), tr[kk]);
            ti[kk] = fma2(two_s, pk2(ww.z, ww.w), ti[kk]);
            // lc_re2 of the new angles: kept from the proposal where the registers allow
            re[kk] = K <= 8 ? fnew[kk] : lc_re2(tr[kk], ti[kk]);
        }
    }
    return accept;
}

// each task kind is a separate (not inlined) function, so that the register allocation of
// one does not constrain the others
template <int K>
__device__ __noinline__ void walker_task(const SLaunch& L, const SInst& Ig, int w, int lane) {
    constexpr int NW = kSW;
    const SInst I = Ig;   // the descriptor in registers / local memory, not re-read from global
    WarpRng rng;
    rng.init(I.seed, static_cast<uint32_t>(w), I.rng_index[w], lane);
    const uint64_t nmagic = fastmod_magic(static_cast<uint32_t>(I.N));
    Spins<NW> s;
#pragma unroll
    for (int k = 0; k < NW; k++) s.w[k] = 0;
    if (L.first) {
        // the draws of draw_spins for this instance's word count (low then high half)
#pragma unroll
        for (int k = 0; k < NW; k++)
            if (k < I.nw) {
                const uint64_t lo = rng.next();
                const uint64_t hi = rng.next();
                s.w[k] = lo | (hi << 32);
            }
#pragma unroll
        for (int k = 0; k < NW; k++)
            if (k == I.N / 64 && k < I.nw) s.w[k] &= (1ull << (I.N % 64)) - 1ull;
    } else {
#pragma unroll
        for (int k = 0; k < NW; k++)
            if (k < I.nw) s.w[k] = I.spins[static_cast<long>(w) * I.nw + k];
    }
    unsigned long long acc = 0;
    {
        constexpr int KP = (K + 1) / 2;
        pair_t tp[KP], tq[KP], rp[KP];
        const int total = (L.first ? L.therm : 0) + L.sweeps;
        for (int sw = 0; sw < total; sw++) {
            s_refresh2(I, s, tp, tq, lane);
#pragma unroll
            for (int kk = 0; kk < KP; kk++) rp[kk] = lc_re2(tp[kk], tq[kk]);
            for (int p = 0; p < I.N; p++) acc += s_mh_step2<K>(I, s, tp, tq, rp, rng, lane, nmagic);
        }
    }
    // measurement at the final configuration: the local energy, tanh(theta), and for the
    // E_k term the angles, U_j = sum_n e_n tanh(theta''_nj) and the e_n.  Three
    // shared-memory slices [kSK][32] of this warp hold f(theta), the current string's
    // tanh(theta'') and U, keeping the register footprint of the sweeps; f and tanh of an
    // angle come from one evaluation with the approximate reciprocal (lc_tanh_approx; the
    // local-energy differences, as rbm_eloc_t_kernel takes them)
    float tr[K], ti[K];
    s_refresh(I, s, tr, ti, lane);
    extern __shared__ float2 s_f[];
    float2* myf = s_f + (threadIdx.x >> 5) * 3 * kSK * 32 + lane;
    float2* myt = myf + kSK * 32;
    float2* myu = myt + kSK * 32;
    const long row_w = static_cast<long>(w) * I.Mpad + lane;
#pragma unroll
    for (int k = 0; k < K; k++) {
        float2 f, t;
        lc_tanh_approx(tr[k], ti[k], f, t);
        myf[32 * k] = f;
        I.T[row_w + 32 * k] = t;
        I.theta[row_w + 32 * k] = make_float2(tr[k], ti[k]);
        myu[32 * k] = make_float2(0.0f, 0.0f);
    }
    float2 dsum = make_float2(0.0f, 0.0f);   // the diagonal strings' summed coefficient
    KahanC e;
    for (int n = 0; n < I.op.S; n++) {
        const float2 cf = string_factor(I.op, n, s);
        const int nf = I.op.nflip[n];
        if (nf == 0) {
            e.add(cf.x, cf.y);
            dsum.x += cf.x;
            dsum.y += cf.y;
            continue;
        }
        const int off = I.op.flip_off[n];
        float2 part = make_float2(0.0f, 0.0f);
        if (nf == 1) {
            const int site = I.op.flip_sites[off];
            const float two_s = s.up(site) ? -2.0f : 2.0f;
            const float2* row = I.W + static_cast<long>(site) * I.Mpad + lane;
            float2 wv[K];
#pragma unroll
            for (int k = 0; k < K; k++) wv[k] = __ldg(row + 32 * k);
#pragma unroll
            for (int k = 0; k < K; k++) {
                float2 g, h;
                lc_tanh_approx(fmaf(two_s, wv[k].x, tr[k]), fmaf(two_s, wv[k].y, ti[k]), g, h);
                const float2 f0 = myf[32 * k];
                part.x += g.x - f0.x;
                part.y += g.y - f0.y;
                myt[32 * k] = h;
            }
        } else {
#pragma unroll
            for (int k = 0; k < K; k++) {
                float nr = tr[k], ni = ti[k];
                for (int q = 0; q < nf; q++) {
                    const int site = I.op.flip_sites[off + q];
                    const float two_s = s.up(site) ? -2.0f : 2.0f;
                    const float2 wv = __ldg(I.W + static_cast<long>(site) * I.Mpad + lane + 32 * k);
                    nr = fmaf(two_s, wv.x, nr);
                    ni = fmaf(two_s, wv.y, ni);
                }
                float2 g, h;
                lc_tanh_approx(nr, ni, g, h);
                const float2 f0 = myf[32 * k];
                part.x += g.x - f0.x;
                part.y += g.y - f0.y;
                myt[32 * k] = h;
            }
        }
        const float2 t = string_term(cf, warp_sum_xor2(part));
        e.add(t.x, t.y);
        if (lane == 0) I.en[static_cast<long>(w) * I.op.num_offdiag + I.op.offdiag_slot[n]] = t;
#pragma unroll
        for (int k = 0; k < K; k++) {
            const float2 h = myt[32 * k];
            const float2 x = make_float2(t.x * h.x - t.y * h.y, t.x * h.y + t.y * h.x);
            float2 u = myu[32 * k];
            u.x += x.x;
            u.y += x.y;
            myu[32 * k] = u;
        }
    }
#pragma unroll
    for (int k = 0; k < K; k++) {
        const float2 h = I.T[row_w + 32 * k];
        float2 u = myu[32 * k];
        u.x += dsum.x * h.x - dsum.y * h.y;
        u.y += dsum.x * h.y + dsum.y * h.x;
        I.U[row_w + 32 * k] = u;
    }
    if (lane == 0) {
#pragma unroll
        for (int k = 0; k < NW; k++)
            if (k < I.nw) I.spins[static_cast<long>(w) * I.nw + k] = s.w[k];
        I.rng_index[w] = rng.index;
        I.eloc[w] = e.value();
        atomicAdd(L.accepts, acc);
    }
    __syncwarp();
    __threadfence();
    if (lane == 0) atomicAdd(I.done, 1u);
}

// rows [r0, r0 + R) of the instance's sums (row N: the biases), every column, over the
// walkers of chunk [w0, w0 + kReduceWalkers): the chunk's partial sums of gO, gE and gK
// (every partial is written by exactly one tile; serve_finish_kernel adds the chunks)
template <int R, bool GENERAL>
__device__ __noinline__ void reduce_task(const SLaunch& L, const SInst& Ig, int r0, int w0, int lane) {
    const SInst I = Ig;   // the descriptor in registers: loop-invariant, not re-read per walker
    // wait for the instance's walkers (bounded by L.wait_ns of wall clock; a wait that gives
    // up raises the error flag, and every other waiter leaves as soon as it sees the flag)
    if (lane == 0) {
        const unsigned long long t0 = global_ns();
        const unsigned int need = static_cast<unsigned int>(I.walkers) + L.wait_extra;
        while (atomicAdd(I.done, 0u) < need) {
            if (*reinterpret_cast<volatile int*>(L.error)) break;
            if (global_ns() - t0 > L.wait_ns) {
                atomicExch(L.error, 1);
                break;
            }
            __nanosleep(1000);
        }
    }
    __syncwarp();
    if (*reinterpret_cast<volatile int*>(L.error)) return;
    __threadfence();
    // the instance's mean local energy, in a fixed order (the same value in every tile)
    double mx = 0.0, my = 0.0;
    for (int w = lane; w < I.walkers; w += 32) {
        const double2 ed = __ldcg(I.eloc + w);
        mx += ed.x;
        my += ed.y;
    }
#pragma unroll
    for (int off = 16; off >= 1; off >>= 1) {
        mx += __shfl_xor_sync(0xffffffffu, mx, off);
        my += __shfl_xor_sync(0xffffffffu, my, off);
    }
    mx /= I.walkers;
    my /= I.walkers;
    if (r0 == 0 && w0 == 0 && lane == 0) *I.emean = make_double2(mx, my);
    const float Er = static_cast<float>(mx), Ei = static_cast<float>(my);
    const int chunk = w0 / kReduceWalkers;
    const long plane = static_cast<long>(I.N + 1) * I.Mpad;
    float2* part = I.part + static_cast<long>(chunk) * 3 * plane;
    const int w1 = min(I.walkers, w0 + kReduceWalkers);
    // per row, fetched once: the off-diagonal slots flipping its site; in the common case
    // of one slot whose string flips that one site, the slot and the site
    int sb[R], se[R], fslot[R];
#pragma unroll
    for (int r = 0; r < R; r++) {
        const int i = r0 + r;
        sb[r] = i < I.N ? I.site_ptr[i] : 0;
        se[r] = i < I.N ? I.site_ptr[i + 1] : 0;
        fslot[r] = -1;
        if (se[r] - sb[r] == 1) {
            const int slot = I.site_slots[sb[r]];
            const int n = I.op.offdiag[slot];
            if (I.op.nflip[n] == 1) fslot[r] = slot;
        }
    }
    // the e_n of a block of 32 walkers, [R][32], in this warp's shared-memory slice
    extern __shared__ float2 s_f[];
    float2* sen = s_f + (threadIdx.x >> 5) * 3 * kSK * 32;
    const long estride = I.op.num_offdiag;
    const uint64_t* spins = reinterpret_cast<const uint64_t*>(I.spins);
    for (int kc = 0; kc < I.K; kc++) {
        float2 aO[R], aE[R], aK[R];
#pragma unroll
        for (int r = 0; r < R; r++) {
            aO[r] = make_float2(0.0f, 0.0f);
            aE[r] = make_float2(0.0f, 0.0f);
            aK[r] = make_float2(0.0f, 0.0f);
        }
        const int j = lane + 32 * kc;
        float2 wr[R];   // W[i][j] of each row's site (the single-flip case)
#pragma unroll
        for (int r = 0; r < R; r++)
            wr[r] = (r0 + r < I.N) ? __ldg(I.W + static_cast<long>(r0 + r) * I.Mpad + j) : make_float2(0.0f, 0.0f);
        for (int wb = w0; wb < w1; wb += 32) {
            // a block of 32 walkers: lane b fetches walker wb + b's centred energy, the spins
            // of the tile's rows (bit r: row r0 + r up) and the e_n of the rows' single-flip
            // strings, all at once; the walker loop below takes them by shuffles.  L2 loads
            // (__ldcg): the walkers' results were written by other SMs
            const int nb = min(32, w1 - wb);
            float sdx = 0.0f, sdy = 0.0f;
            unsigned int sbits = 0u;
            __syncwarp();   // the previous block's reads of the slice are done
            if (lane < nb) {
                const int ws = wb + lane;
                const double2 ed = __ldcg(I.eloc + ws);
                sdx = static_cast<float>(ed.x - mx);
                sdy = static_cast<float>(ed.y - my);
                // rows r0 .. r0 + R - 1 (R <= 64) lie in at most two spin words
                const int q0 = min(r0, I.N - 1) >> 6, q1 = min(r0 + R - 1, I.N - 1) >> 6;
                const uint64_t lo = __ldcg(spins + static_cast<long>(ws) * I.nw + q0);
                const uint64_t hi = q1 != q0 ? __ldcg(spins + static_cast<long>(ws) * I.nw + q1) : lo;
#pragma unroll
                for (int r = 0; r < R; r++) {
                    const int i = r0 + r;
                    if (i < I.N) {
                        const uint64_t wd = (i >> 6) == q0 ? lo : hi;
                        sbits |= static_cast<unsigned int>((wd >> (i & 63)) & 1ull) << r;
                        if (fslot[r] >= 0) sen[r * 32 + lane] = __ldcg(I.en + ws * estride + fslot[r]);
                    }
                }
            }
            __syncwarp();
            for (int bw = 0; bw < nb; bw++) {
                const int w = wb + bw;
                const long o = static_cast<long>(w) * I.Mpad + j;
                const float2 t = __ldcg(I.T + o);
                const float2 u = __ldcg(I.U + o);
                const float2 th = __ldcg(I.theta + o);
                const float dx = __shfl_sync(0xffffffffu, sdx, bw);
                const float dy = __shfl_sync(0xffffffffu, sdy, bw);
                const unsigned int bits = __shfl_sync(0xffffffffu, sbits, bw);
                // conj(t), (E - <E>) conj(t), and U - <E> t (E_k of the biases, centred)
                const float cx = t.x, cy = -t.y;
                const float ex = dx * cx - dy * cy, ey = dx * cy + dy * cx;
                const float kx = u.x - (Er * t.x - Ei * t.y), ky = u.y - (Er * t.y + Ei * t.x);
                uint64_t sw[kSW];
#pragma unroll
                for (int q = 0; q < kSW; q++)
                    sw[q] = GENERAL && q < I.nw ? __ldcg(spins + static_cast<long>(w) * I.nw + q) : 0ull;
                auto up = [&](int site) {
                    uint64_t wd = sw[0];
#pragma unroll
                    for (int q = 1; q < kSW; q++)
                        if ((site >> 6) == q) wd = sw[q];
                    return ((wd >> (site & 63)) & 1ull) != 0ull;
                };
#pragma unroll
                for (int r = 0; r < R; r++) {
                    const int i = r0 + r;
                    if (i > I.N) continue;
                    float sg = 1.0f;
                    float vx = 0.0f, vy = 0.0f;
                    if (i < I.N) {
                        sg = (bits >> r) & 1u ? 1.0f : -1.0f;
                        // V_ij = sum over the strings n flipping site i of e_n tanh(theta''_nj),
                        // the angles theta'' formed as the walker task formed them
                        if (fslot[r] >= 0) {
                            const float two_s = sg > 0.0f ? -2.0f : 2.0f;
                            float2 g, h;
                            lc_tanh_approx(fmaf(two_s, wr[r].x, th.x), fmaf(two_s, wr[r].y, th.y), g, h);
                            const float2 en = sen[r * 32 + bw];
                            vx = en.x * h.x - en.y * h.y;
                            vy = en.x * h.y + en.y * h.x;
                        } else if (GENERAL) {
                            const float2* enw = I.en + w * estride;
                            for (int q = sb[r]; q < se[r]; q++) {
                                const int slot = I.site_slots[q];
                                const int n = I.op.offdiag[slot];
                                const int nf = I.op.nflip[n], fo = I.op.flip_off[n];
                                float nr = th.x, ni = th.y;
                                for (int f = 0; f < nf; f++) {
                                    const int site = I.op.flip_sites[fo + f];
                                    const float ts = up(site) ? -2.0f : 2.0f;
                                    const float2 wv = __ldg(I.W + static_cast<long>(site) * I.Mpad + j);
                                    nr = fmaf(ts, wv.x, nr);
                                    ni = fmaf(ts, wv.y, ni);
                                }
                                float2 g, h;
                                lc_tanh_approx(nr, ni, g, h);
                                const float2 en = __ldcg(enw + slot);
                                vx += en.x * h.x - en.y * h.y;
                                vy += en.x * h.y + en.y * h.x;
                            }
                        }
                    }
                    aO[r].x += sg * cx;
                    aO[r].y += sg * cy;
                    aE[r].x += sg * ex;
                    aE[r].y += sg * ey;
                    // conj(s_i (U - 2 V) - <E> O) = sg conj(U - <E> t - 2 V)
                    aK[r].x += sg * (kx - 2.0f * vx);
                    aK[r].y -= sg * (ky - 2.0f * vy);
                }
            }
        }
#pragma unroll
        for (int r = 0; r < R; r++) {
            const int i = r0 + r;
            if (i <= I.N) {
                const long e = static_cast<long>(i) * I.Mpad + j;
                part[e] = aO[r];
                part[plane + e] = aE[r];
                part[2 * plane + e] = aK[r];
            }
        }
    }
}

// the sums over the walker chunks, in chunk order (FP64): blockIdx.y is the instance
__global__ void serve_finish_kernel(const SInst* inst) {
    const SInst& I = inst[blockIdx.y];
    const long n = 3L * (I.N + 1) * I.Mpad;
    for (long e = static_cast<long>(blockIdx.x) * blockDim.x + threadIdx.x; e < n;
         e += static_cast<long>(gridDim.x) * blockDim.x) {
        double sx = 0.0, sy = 0.0;
        for (int c = 0; c < I.chunks; c++) {
            const float2 v = I.part[c * n + e];
            sx += v.x;
            sy += v.y;
        }
        I.g[e] = make_double2(sx, sy);
    }
}

// REGS caps the registers per thread (the largest walker task sets the kernel's count, so
// a cap trades its spills against more resident warps for every task); the autotuner picks
template <int R, int REGS>
__global__ void __maxnreg__(REGS) serve_kernel(SLaunch L) {
    const int lane = threadIdx.x & 31;
    for (;;) {
        int t = 0;
        if (lane == 0) t = static_cast<int>(atomicAdd(L.next, 1u));
        t = __shfl_sync(0xffffffffu, t, 0);
        if (t >= L.ntasks) return;
        const STask task = L.tasks[t];
        const SInst& I = L.inst[task.inst];
        if (task.kind == 0) {
            switch (I.K) {   // the hidden-unit counts per lane of rbm_lanes_k
                case 1: walker_task<1>(L, I, task.index, lane); break;
                case 2: walker_task<2>(L, I, task.index, lane); break;
                case 4: walker_task<4>(L, I, task.index, lane); break;
                case 8: walker_task<8>(L, I, task.index, lane); break;
                case 13: walker_task<13>(L, I, task.index, lane); break;
                default: walker_task<18>(L, I, task.index, lane); break;
            }
        } else {
            // rows whose sites are all flipped by one single-flip string each take the
            // specialised tile (task.general: some row is not)
            if (task.general) reduce_task<R, true>(L, I, task.index, task.w0, lane);
            else reduce_task<R, false>(L, I, task.index, task.w0, lane);
        }
    }
}

}  // namespace
}  // namespace rbmg

using namespace rbmg;

struct rbmg_batch {
    int n = 0;
    std::vector<const rbmg_psi*> psis;
    std::vector<const rbmg_operator*> ops;
    std::vector<SInst> host_inst;
    std::vector<std::vector<char>> single_flip;   // [instance][site]: the single-flip tile serves the site
    std::vector<uint32_t> walkers;
    DevBuf d_inst, d_tasks, d_next, d_done, d_error, d_accepts;
    int max_elems = 0;          // largest instance's 3 (N + 1) Mpad (the finish kernel's grid)
    std::vector<std::unique_ptr<DevBuf>> bufs;
    int ntasks_walk = 0, ntasks = 0;
    int rows = 16;              // reduction tile height
    int warps_per_block = 4;
    int regs = 255;             // register cap per thread: 255, 128 or 96
    int blocks = 0;
    bool first = true;
    int therm = 0, sweeps = 1;  // graph parameters
    unsigned long long wait_ns = 20000000000ull;
    unsigned int wait_extra = 0;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    int graph_rows = 0, graph_wpb = 0, graph_regs = 0, graph_first = -1, graph_therm = -1, graph_sweeps = -1;
    unsigned long long graph_wait_ns = 0;
    unsigned int graph_wait_extra = 0;
    double tuned_ms = 0.0;
    ~rbmg_batch() {
        if (exec) cudaGraphExecDestroy(exec);
        if (graph) cudaGraphDestroy(graph);
    }
};

namespace {

int batch_tasks(rbmg_batch* b) {
    // walker tasks, longest first (cost ~ N * Mpad per sweep), then reduction tiles
    std::vector<int> order(b->n);
    for (int i = 0; i < b->n; i++) order[i] = i;
    std::stable_sort(order.begin(), order.end(), [&](int a, int c) {
        return static_cast<long>(b->host_inst[a].N) * b->host_inst[a].Mpad >
               static_cast<long>(b->host_inst[c].N) * b->host_inst[c].Mpad;
    });
    std::vector<STask> tasks;
    for (int i : order)
        for (int w = 0; w < b->host_inst[i].walkers; w++) tasks.push_back(STask{0, i, w, 0, 0});
    b->ntasks_walk = static_cast<int>(tasks.size());
    for (int i : order) {
        const int N = b->host_inst[i].N;
        for (int r0 = 0; r0 <= N; r0 += b->rows) {
            int general = 0;
            for (int r = r0; r < std::min(N, r0 + b->rows); r++) general |= !b->single_flip[i][r];
            for (int w0 = 0; w0 < b->host_inst[i].walkers; w0 += kReduceWalkers)
                tasks.push_back(STask{1, i, r0, w0, general});
        }
    }
    b->ntasks = static_cast<int>(tasks.size());
    RBMG_CK(b->d_tasks.ensure(sizeof(STask) * tasks.size()));
    RBMG_CK(cudaMemcpy(b->d_tasks.p, tasks.data(), sizeof(STask) * tasks.size(), cudaMemcpyHostToDevice));
    return RBMG_OK;
}

size_t serve_smem(int warps_per_block) { return sizeof(float2) * 3 * kSK * 32 * warps_per_block; }

// calls f with the kernel instantiation of (reduction rows, register cap)
template <class F>
void with_serve_kernel(int rows, int regs, F f) {
    if (rows == 8) {
        if (regs == 128) f(serve_kernel<8, 128>);
        else if (regs == 96) f(serve_kernel<8, 96>);
        else f(serve_kernel<8, 255>);
    } else {
        if (regs == 128) f(serve_kernel<16, 128>);
        else if (regs == 96) f(serve_kernel<16, 96>);
        else f(serve_kernel<16, 255>);
    }
}

// the kernel instantiation's dynamic shared-memory limit (above the 48 KB default for 4 and
// 8 warps per block); the attribute belongs to the current device's context
cudaError_t serve_smem_attr(int rows, int regs, size_t sm) {
    cudaError_t e = cudaSuccess;
    with_serve_kernel(rows, regs, [&](auto kern) {
        e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(sm));
    });
    return e;
}

cudaError_t launch_serve(rbmg_batch* b, cudaStream_t st) {
    SLaunch L{};
    L.inst = b->d_inst.as<SInst>();
    L.tasks = b->d_tasks.as<STask>();
    L.ntasks = b->ntasks;
    L.next = b->d_next.as<unsigned int>();
    L.therm = b->therm;
    L.sweeps = b->sweeps;
    L.first = b->first ? 1 : 0;
    L.error = b->d_error.as<int>();
    L.accepts = b->d_accepts.as<unsigned long long>();
    L.wait_ns = b->wait_ns;
    L.wait_extra = b->wait_extra;
    const int threads = 32 * b->warps_per_block;
    const size_t sm = serve_smem(b->warps_per_block);
    const cudaError_t e = serve_smem_attr(b->rows, b->regs, sm);
    if (e != cudaSuccess) return e;
    with_serve_kernel(b->rows, b->regs, [&](auto kern) { kern<<<b->blocks, threads, sm, st>>>(L); });
    return cudaGetLastError();
}

// (re)captures the replay: counter resets and the persistent launch
int batch_capture(rbmg_batch* b) {
    if (b->exec && b->graph_rows == b->rows && b->graph_wpb == b->warps_per_block && b->graph_regs == b->regs &&
        b->graph_first == static_cast<int>(b->first) && b->graph_therm == b->therm && b->graph_sweeps == b->sweeps &&
        b->graph_wait_ns == b->wait_ns && b->graph_wait_extra == b->wait_extra)
        return RBMG_OK;
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    b->exec = nullptr;
    b->graph = nullptr;
    int dev = 0, sms = 0, per_sm = 0;
    RBMG_CK(cudaGetDevice(&dev));
    RBMG_CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const int threads = 32 * b->warps_per_block;
    const size_t sm = serve_smem(b->warps_per_block);
    RBMG_CK(serve_smem_attr(b->rows, b->regs, sm));
    cudaError_t oe = cudaSuccess;
    with_serve_kernel(b->rows, b->regs,
                      [&](auto kern) { oe = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, threads, sm); });
    RBMG_CK(oe);
    b->blocks = std::max(1, sms * std::max(1, per_sm));
    cudaStream_t st = stream();
    RBMG_CK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    cudaMemsetAsync(b->d_next.p, 0, sizeof(unsigned int), st);
    cudaMemsetAsync(b->d_done.p, 0, sizeof(unsigned int) * b->n, st);
    cudaMemsetAsync(b->d_accepts.p, 0, sizeof(unsigned long long), st);
    cudaError_t le = launch_serve(b, st);
    if (le == cudaSuccess) {
        const dim3 grid(std::min(64, (b->max_elems + 255) / 256), b->n);
        serve_finish_kernel<<<grid, 256, 0, st>>>(b->d_inst.as<SInst>());
        le = cudaGetLastError();
    }
    cudaGraph_t g = nullptr;
    const cudaError_t ce = cudaStreamEndCapture(st, &g);
    RBMG_CK(le);
    RBMG_CK(ce);
    b->graph = g;
    RBMG_CK(cudaGraphInstantiate(&b->exec, b->graph, 0));
    b->graph_rows = b->rows;
    b->graph_wpb = b->warps_per_block;
    b->graph_regs = b->regs;
    b->graph_first = static_cast<int>(b->first);
    b->graph_therm = b->therm;
    b->graph_sweeps = b->sweeps;
    b->graph_wait_ns = b->wait_ns;
    b->graph_wait_extra = b->wait_extra;
    return RBMG_OK;
}

int batch_replay(rbmg_batch* b) {
    int r = batch_capture(b);
    if (r != RBMG_OK) return r;
    RBMG_CK(cudaGraphLaunch(b->exec, stream()));
    int err = 0;
    RBMG_CK(cudaMemcpyAsync(&err, b->d_error.p, sizeof(int), cudaMemcpyDeviceToHost, stream()));
    RBMG_CK(cudaStreamSynchronize(stream()));
    if (err) {
        RBMG_CK(cudaMemset(b->d_error.p, 0, sizeof(int)));
        return fail(RBMG_ETIMEOUT, "batch: a reduction task timed out waiting for its walkers");
    }
    b->first = false;
    return RBMG_OK;
}

}  // namespace

extern "C" int rbmg_batch_create(int n, const rbmg_psi* const* psis, const rbmg_operator* const* ops,
                                 const uint32_t* walkers, const uint64_t* seeds, rbmg_batch** out) {
    if (n <= 0 || !psis || !ops || !walkers || !seeds || !out) return fail(RBMG_EINVAL, "batch: bad arguments");
    auto b = std::make_unique<rbmg_batch>();
    b->n = n;
    for (int i = 0; i < n; i++) {
        const rbmg_psi* p = psis[i];
        const rbmg_operator* o = ops[i];
        if (!p || !o || walkers[i] == 0) return fail(RBMG_EINVAL, "batch: null instance or no walkers");
        if (p->kind != 0) return fail(RBMG_EUNSUPPORTED, "batch: complex RBM (Psi) instances only");
        if (p->Mpad / 32 > kSK) return fail(RBMG_EUNSUPPORTED, "batch: M <= 576");
        {
            const int K = p->Mpad / 32;
            if (K != 1 && K != 2 && K != 4 && K != 8 && K != 13 && K != 18)
                return fail(RBMG_EINVAL, "batch: unexpected hidden-unit padding");
        }
        if (p->N > 64 * kSW) return fail(RBMG_EUNSUPPORTED, "batch: N <= 192");
        if (o->max_site >= p->N) return fail(RBMG_EINVAL, "batch: operator acts on a site >= N");
        for (int q = 0; q < i; q++)
            if (ops[q] == o && psis[q]->N != p->N)
                return fail(RBMG_EINVAL, "batch: an operator shared by instances of different N");
        {
            const int r = op_site_lists(const_cast<rbmg_operator*>(o), p->N);
            if (r != RBMG_OK) return r;
        }
        const int nw = nwords_of(p->N);
        SInst I{};
        I.N = p->N;
        I.M = p->M;
        I.Mpad = p->Mpad;
        I.K = p->Mpad / 32;
        I.nw = nw;
        const RbmDev d = p->rbm_dev();
        I.W = d.W;
        I.b = d.b;
        I.Wq = d.Wq;
        I.bq = d.bq;
        I.op = o->dev();
        I.walkers = static_cast<int>(walkers[i]);
        I.seed = seeds[i];
        auto alloc = [&](size_t bytes) -> void* {
            b->bufs.push_back(std::make_unique<DevBuf>());
            if (b->bufs.back()->ensure(std::max<size_t>(bytes, 16)) != cudaSuccess) return nullptr;
            return b->bufs.back()->p;
        };
        const size_t B = walkers[i];
        I.eloc = static_cast<double2*>(alloc(sizeof(double2) * B));
        I.T = static_cast<float2*>(alloc(sizeof(float2) * B * p->Mpad));
        I.U = static_cast<float2*>(alloc(sizeof(float2) * B * p->Mpad));
        I.theta = static_cast<float2*>(alloc(sizeof(float2) * B * p->Mpad));
        I.en = static_cast<float2*>(alloc(sizeof(float2) * B * std::max(1, o->num_offdiag)));
        I.spins = static_cast<uint64_t*>(alloc(sizeof(uint64_t) * B * nw));
        I.rng_index = static_cast<uint64_t*>(alloc(sizeof(uint64_t) * B));
        I.chunks = static_cast<int>((B + kReduceWalkers - 1) / kReduceWalkers);
        const size_t elems = 3 * static_cast<size_t>(p->N + 1) * p->Mpad;
        I.part = static_cast<float2*>(alloc(sizeof(float2) * I.chunks * elems));
        I.g = static_cast<double2*>(alloc(sizeof(double2) * elems));
        I.emean = static_cast<double2*>(alloc(sizeof(double2)));
        // the batch's own copy of the site lists (the operator's are rebuilt when it is used
        // with another N), and per site whether the single-flip tile serves it: exactly one
        // off-diagonal string flips the site and flips it alone (reduce_task's test)
        int* site_ptr = static_cast<int*>(alloc(sizeof(int) * o->site_ptr.size()));
        int* site_slots = static_cast<int*>(alloc(sizeof(int) * o->site_slots.size()));
        if (!site_ptr || !site_slots) return fail(RBMG_ENOMEM, "batch: device allocation failed");
        RBMG_CK(cudaMemcpy(site_ptr, o->site_ptr.data(), sizeof(int) * o->site_ptr.size(), cudaMemcpyHostToDevice));
        RBMG_CK(cudaMemcpy(site_slots, o->site_slots.data(), sizeof(int) * o->site_slots.size(),
                           cudaMemcpyHostToDevice));
        I.site_ptr = site_ptr;
        I.site_slots = site_slots;
        {
            std::vector<int> string_of(std::max(1, o->num_offdiag), 0);
            for (int n = 0; n < o->S; n++)
                if (o->offdiag_slot[n] >= 0) string_of[o->offdiag_slot[n]] = n;
            std::vector<char> single(p->N);
            for (int site = 0; site < p->N; site++) {
                const int sb = o->site_ptr[site], se = o->site_ptr[site + 1];
                single[site] = se - sb == 1 && o->nflip[string_of[o->site_slots[sb]]] == 1;
            }
            b->single_flip.push_back(std::move(single));
        }
        b->max_elems = std::max(b->max_elems, static_cast<int>(elems));
        if (!I.eloc || !I.T || !I.U || !I.theta || !I.en || !I.spins || !I.rng_index || !I.part || !I.g ||
            !I.emean)
            return fail(RBMG_ENOMEM, "batch: device allocation failed");
        RBMG_CK(cudaMemset(I.rng_index, 0, sizeof(uint64_t) * B));
        b->psis.push_back(p);
        b->ops.push_back(o);
        b->walkers.push_back(walkers[i]);
        b->host_inst.push_back(I);
    }
    RBMG_CK(b->d_done.ensure(sizeof(unsigned int) * n));
    for (int i = 0; i < n; i++) b->host_inst[i].done = b->d_done.as<unsigned int>() + i;
    RBMG_CK(b->d_inst.ensure(sizeof(SInst) * n));
    RBMG_CK(cudaMemcpy(b->d_inst.p, b->host_inst.data(), sizeof(SInst) * n, cudaMemcpyHostToDevice));
    RBMG_CK(b->d_next.ensure(sizeof(unsigned int)));
    RBMG_CK(b->d_error.ensure(sizeof(int)));
    RBMG_CK(b->d_accepts.ensure(sizeof(unsigned long long)));
    RBMG_CK(cudaMemset(b->d_error.p, 0, sizeof(int)));
    const int r = batch_tasks(b.get());
    if (r != RBMG_OK) return r;
    *out = b.release();
    return RBMG_OK;
}

extern "C" int rbmg_batch_destroy(rbmg_batch* b) {
    delete b;
    return RBMG_OK;
}

extern "C" int rbmg_batch_set_shape(rbmg_batch* b, int warps_per_block, int rows) {
    if (!b || (warps_per_block != 2 && warps_per_block != 4 && warps_per_block != 8) || (rows != 8 && rows != 16))
        return fail(RBMG_EINVAL, "batch: warps per block in {2, 4, 8}, tile rows in {8, 16}");
    if (rows != b->rows) {
        b->rows = rows;
        const int r = batch_tasks(b);
        if (r != RBMG_OK) return r;
    }
    b->warps_per_block = warps_per_block;
    return RBMG_OK;
}

extern "C" int rbmg_batch_set_wait(rbmg_batch* b, double seconds, uint32_t extra_walkers) {
    if (!b || !(seconds > 0.0) || seconds > 60.0) return fail(RBMG_EINVAL, "batch: wait limit in (0, 60] s");
    b->wait_ns = static_cast<unsigned long long>(seconds * 1e9);
    b->wait_extra = extra_walkers;
    return RBMG_OK;
}

extern "C" int rbmg_batch_set_register_cap(rbmg_batch* b, int regs) {
    if (!b || (regs != 255 && regs != 128 && regs != 96))
        return fail(RBMG_EINVAL, "batch: register cap in {255, 128, 96}");
    b->regs = regs;
    return RBMG_OK;
}

extern "C" int rbmg_batch_get_register_cap(const rbmg_batch* b, int* regs) {
    if (!b || !regs) return fail(RBMG_EINVAL, "batch: null");
    *regs = b->regs;
    return RBMG_OK;
}

extern "C" int rbmg_batch_get_shape(const rbmg_batch* b, int* warps_per_block, int* rows, int* blocks) {
    if (!b) return fail(RBMG_EINVAL, "batch: null");
    if (warps_per_block) *warps_per_block = b->warps_per_block;
    if (rows) *rows = b->rows;
    if (blocks) *blocks = b->blocks;
    return RBMG_OK;
}

extern "C" int rbmg_batch_run(rbmg_batch* b, int therm, int sweeps) {
    if (!b || therm < 0 || sweeps < 0) return fail(RBMG_EINVAL, "batch run: bad arguments");
    b->therm = therm;
    b->sweeps = sweeps;
    return batch_replay(b);
}

// Times every candidate shape on `reps` replays of `sweeps` sweeps (the chains advance),
// keeps the fastest; ms_out [18] receives the candidates' mean milliseconds per replay,
// register caps 255, 128, 96 in turn, each in the order (2,8) (2,16) (4,8) (4,16) (8,8) (8,16).
extern "C" int rbmg_batch_autotune(rbmg_batch* b, int sweeps, int reps, double* ms_out) {
    if (!b || sweeps < 0 || reps <= 0) return fail(RBMG_EINVAL, "batch autotune: bad arguments");
    if (b->first) {   // start the chains outside the timing
        const int r = rbmg_batch_run(b, 0, 0);
        if (r != RBMG_OK) return r;
    }
    const int wpbs[3] = {2, 4, 8}, rowss[2] = {8, 16}, capss[3] = {255, 128, 96};
    double best = 1e300;
    int bw = 4, brows = 16, bregs = 255, c = 0;
    for (int regs : capss)
    for (int wpb : wpbs)
        for (int rows : rowss) {
            int r = rbmg_batch_set_shape(b, wpb, rows);
            if (r == RBMG_OK) r = rbmg_batch_set_register_cap(b, regs);
            if (r != RBMG_OK) return r;
            b->therm = 0;
            b->sweeps = sweeps;
            r = batch_replay(b);   // capture + warm-up
            if (r != RBMG_OK) return r;
            cudaEvent_t e0, e1;
            RBMG_CK(cudaEventCreate(&e0));
            RBMG_CK(cudaEventCreate(&e1));
            RBMG_CK(cudaEventRecord(e0, stream()));
            for (int k = 0; k < reps; k++) RBMG_CK(cudaGraphLaunch(b->exec, stream()));
            RBMG_CK(cudaEventRecord(e1, stream()));
            RBMG_CK(cudaEventSynchronize(e1));
            float ms = 0.0f;
            RBMG_CK(cudaEventElapsedTime(&ms, e0, e1));
            cudaEventDestroy(e0);
            cudaEventDestroy(e1);
            int err = 0;
            RBMG_CK(cudaMemcpy(&err, b->d_error.p, sizeof(int), cudaMemcpyDeviceToHost));
            if (err) return fail(RBMG_ETIMEOUT, "batch autotune: a reduction task timed out");
            const double per = ms / reps;
            if (ms_out) ms_out[c] = per;
            c++;
            if (per < best) {
                best = per;
                bw = wpb;
                brows = rows;
                bregs = regs;
            }
        }
    b->tuned_ms = best;
    const int r = rbmg_batch_set_shape(b, bw, brows);
    return r != RBMG_OK ? r : rbmg_batch_set_register_cap(b, bregs);
}

// results of the last replay for instance i: <E_loc> over its walkers, the reference's O_k
// gradient <E O*> + conj<E_k> - 2 <E> <O*> in the reference's parameter layout [2P] (alpha
// and beta entries 0), optionally the walkers' local energies [2 walkers]
extern "C" int rbmg_batch_result(const rbmg_batch* b, int i, double* energy, double* grad, double* eloc) {
    if (!b || i < 0 || i >= b->n || !energy) return fail(RBMG_EINVAL, "batch result: bad arguments");
    const SInst& I = b->host_inst[i];
    double2 em;
    RBMG_CK(cudaMemcpy(&em, I.emean, sizeof(double2), cudaMemcpyDeviceToHost));
    const cplx E(em.x, em.y);
    energy[0] = E.real();
    energy[1] = E.imag();
    if (eloc) RBMG_CK(cudaMemcpy(eloc, I.eloc, sizeof(double2) * I.walkers, cudaMemcpyDeviceToHost));
    if (grad) {
        const size_t plane = static_cast<size_t>(I.N + 1) * I.Mpad;
        std::vector<double2> g(3 * plane);
        RBMG_CK(cudaMemcpy(g.data(), I.g, sizeof(double2) * 3 * plane, cudaMemcpyDeviceToHost));
        cplx* out = reinterpret_cast<cplx*>(grad);
        const int N = I.N, M = I.M;
        const double inv = 1.0 / I.walkers;
        const cplx shift = std::conj(E) - E;
        for (int k = 0; k < 2 * N; k++) out[k] = 0.0;
        auto val = [&](int row, int j) {
            const size_t e = static_cast<size_t>(row) * I.Mpad + j;
            const cplx gO(g[e].x, g[e].y), gE(g[plane + e].x, g[plane + e].y), gK(g[2 * plane + e].x, g[2 * plane + e].y);
            return (gE + gK) * inv + shift * gO * inv;
        };
        for (int j = 0; j < M; j++) out[2 * N + j] = val(N, j);
        for (int r = 0; r < N; r++)
            for (int j = 0; j < M; j++) out[2 * N + M + static_cast<size_t>(r) * M + j] = val(r, j);
    }
    return RBMG_OK;
}

// the walkers' configurations of instance i after the last replay [walkers][ceil(N/64)]
extern "C" int rbmg_batch_spins(const rbmg_batch* b, int i, uint64_t* spins) {
    if (!b || i < 0 || i >= b->n || !spins) return fail(RBMG_EINVAL, "batch spins: bad arguments");
    const SInst& I = b->host_inst[i];
    RBMG_CK(cudaMemcpy(spins, I.spins, sizeof(uint64_t) * I.walkers * I.nw, cudaMemcpyDeviceToHost));
    return RBMG_OK;
}

extern "C" int rbmg_batch_info(const rbmg_batch* b, int* num_instances, uint64_t* accepts, double* tuned_ms) {
    if (!b) return fail(RBMG_EINVAL, "batch: null");
    if (num_instances) *num_instances = b->n;
    if (accepts) RBMG_CK(cudaMemcpy(accepts, b->d_accepts.p, sizeof(unsigned long long), cudaMemcpyDeviceToHost));
    if (tuned_ms) *tuned_ms = b->tuned_ms;
    return RBMG_OK;
}
