// The S matrix S[k][k'] = < O_k conj(O_k') > over an ensemble (the reference's
// get_S_matrix, source/network_functions/S_matrix.cu:10-53, which adds
// O_k O_k'* for every configuration with a complex global atomic per entry).
//
// Here it is a complex Hermitian rank-n update S += F^T conj(F) of the per-sample O_k
// rows F [n][L] (L = P - 2N), tiled 64 x 64 over the upper triangle of S: each CTA
// stages 16 samples of its row block and its column block in shared memory, every
// thread accumulates a 4 x 4 block of complex products in FP32 registers (its rows and
// columns read with 128-bit shared loads, 64 FFMA per 4 loads), and every
// 1024 samples the CTA adds its partial tile into the FP64 matrix in HBM (plain
// read-modify-write when it owns the tile, FP64 atomics when the samples are split
// across CTAs).  For the complex RBM the rows are never stored: an element of F is
// tanh(theta_j) (k < M) or s_i tanh(theta_j) (k = M + i M + j, Psi.hpp:165-178), formed
// while the tile is loaded from the sample's tanh row and spins.  PsiDeep rows come
// from the FP64 reverse pass.  The lower triangle is mirrored at the end.
#include "host.h"
#include "smatrix.h"
#include "smatrix_rows.cuh"

namespace rbmg {

namespace {

constexpr int kT = 64;          // tile edge
constexpr int kS = 16;          // samples per shared-memory stage
constexpr int kFlush = 1024;    // samples accumulated in FP32 before the FP64 update

__global__ void __launch_bounds__(256) sm_herk_kernel(SmSource a, double2* __restrict__ S, int nt, int slice,
                                                      int atomic) {
    const int tm = blockIdx.x / nt, tn = blockIdx.x - (blockIdx.x / nt) * nt;
    if (tm > tn) return;   // lower triangle: mirrored at the end
    const int s_begin = blockIdx.y * slice;
    const int s_end = min(a.count, s_begin + slice);
    if (s_begin >= s_end) return;
    __shared__ __align__(16) float2 Fa[kS][kT];
    __shared__ __align__(16) float2 Fb[kS][kT];
    const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
    const int m0 = tm * kT, n0 = tn * kT;
    // this thread's four loader columns of each block, sample row ty of the stage
    SmElem ea[4], eb[4];
#pragma unroll
    for (int q = 0; q < 4; q++) {
        ea[q] = sm_elem_of(a, m0 + tx + 16 * q);
        eb[q] = sm_elem_of(a, n0 + tx + 16 * q);
    }
    for (int f0 = s_begin; f0 < s_end; f0 += kFlush) {
        const int f1 = min(s_end, f0 + kFlush);
        float re[4][4], im[4][4];
#pragma unroll
        for (int i = 0; i < 4; i++)
#pragma unroll
            for (int j = 0; j < 4; j++) re[i][j] = im[i][j] = 0.0f;
        float2 pa[4], pb[4];
#pragma unroll
        for (int q = 0; q < 4; q++) {
            pa[q] = f0 + ty < f1 ? sm_load_f(a, ea[q], f0 + ty, m0 + tx + 16 * q) : make_float2(0.0f, 0.0f);
            pb[q] = f0 + ty < f1 ? sm_load_f(a, eb[q], f0 + ty, n0 + tx + 16 * q) : make_float2(0.0f, 0.0f);
        }
        for (int s0 = f0; s0 < f1; s0 += kS) {
            __syncthreads();
#pragma unroll
            for (int q = 0; q < 4; q++) {
                Fa[ty][tx + 16 * q] = pa[q];
                Fb[ty][tx + 16 * q] = pb[q];
            }
            __syncthreads();
            const int sn = s0 + kS + ty;   // next stage's sample of this thread, loaded during the products
#pragma unroll
            for (int q = 0; q < 4; q++) {
                pa[q] = sn < f1 ? sm_load_f(a, ea[q], sn, m0 + tx + 16 * q) : make_float2(0.0f, 0.0f);
                pb[q] = sn < f1 ? sm_load_f(a, eb[q], sn, n0 + tx + 16 * q) : make_float2(0.0f, 0.0f);
            }
#pragma unroll
            for (int s = 0; s < kS; s++) {
                // rows 2 ty, 2 ty + 1, 32 + 2 ty, 33 + 2 ty of the tile (columns alike with tx):
                // two 128-bit loads per block, consecutive threads on consecutive 16 bytes
                const float4 a0 = *reinterpret_cast<const float4*>(&Fa[s][2 * ty]);
                const float4 a1 = *reinterpret_cast<const float4*>(&Fa[s][32 + 2 * ty]);
                const float4 b0 = *reinterpret_cast<const float4*>(&Fb[s][2 * tx]);
                const float4 b1 = *reinterpret_cast<const float4*>(&Fb[s][32 + 2 * tx]);
                const float2 x[4] = {make_float2(a0.x, a0.y), make_float2(a0.z, a0.w), make_float2(a1.x, a1.y),
                                     make_float2(a1.z, a1.w)};
                const float2 y[4] = {make_float2(b0.x, b0.y), make_float2(b0.z, b0.w), make_float2(b1.x, b1.y),
                                     make_float2(b1.z, b1.w)};
#pragma unroll
                for (int i = 0; i < 4; i++)
#pragma unroll
                    for (int j = 0; j < 4; j++) {
                        // x conj(y)
                        re[i][j] = fmaf(x[i].x, y[j].x, fmaf(x[i].y, y[j].y, re[i][j]));
                        im[i][j] = fmaf(x[i].y, y[j].x, fmaf(-x[i].x, y[j].y, im[i][j]));
                    }
            }
        }
#pragma unroll
        for (int i = 0; i < 4; i++) {
            const int r = m0 + (i >> 1) * 32 + 2 * ty + (i & 1);
            if (r >= a.L) continue;
#pragma unroll
            for (int j = 0; j < 4; j++) {
                const int c = n0 + (j >> 1) * 32 + 2 * tx + (j & 1);
                if (c >= a.L) continue;
                double2* p = S + static_cast<long>(r) * a.L + c;
                if (atomic) {
                    atomicAdd(&p->x, static_cast<double>(re[i][j]));
                    atomicAdd(&p->y, static_cast<double>(im[i][j]));
                } else {
                    double2 v = *p;
                    v.x += static_cast<double>(re[i][j]);
                    v.y += static_cast<double>(im[i][j]);
                    *p = v;
                }
            }
        }
    }
}

// mean[k] += sum_s w_s (F[s][k] - shift[k]) (FP64); assign: mean[k] = the sum * scale
__global__ void sm_mean_kernel(SmSource a, double2* mean, int assign, double scale) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= a.L) return;
    SmSource u = a;
    u.weighted = 0;
    const SmElem e = sm_elem_of(u, k);
    double sr = 0.0, si = 0.0;
    for (int s = 0; s < a.count; s++) {
        const float2 v = sm_load_f(u, e, s, k);
        const double c = a.weighted ? a.w[s] : 1.0;
        sr += c * v.x;
        si += c * v.y;
    }
    if (assign) {
        mean[k] = make_double2(sr * scale, si * scale);
    } else {
        mean[k].x += sr;
        mean[k].y += si;
    }
}

// out[off + r][off + c] = S[r][c] / Z with the lower triangle mirrored from the upper and
// a real diagonal (out: ldo columns; rows and columns below off are left to the caller);
// centred: - m m^dagger with m = mean / Z (mean of the shifted rows: the covariance does
// not depend on the shift)
__global__ void sm_finish_kernel(int L, const double2* __restrict__ S, const double2* mean, double inv_z,
                                 int centered, double2* __restrict__ out, long ldo, int off) {
    const long idx = static_cast<long>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (idx >= static_cast<long>(L) * L) return;
    const int r = static_cast<int>(idx / L), c = static_cast<int>(idx - static_cast<long>(r) * L);
    // the upper triangle only (the diagonal tiles' lower halves are rewritten from their
    // upper halves, so that S is Hermitian to the bit); the mirror images are written below
    if (r > c) return;
    double2 v = S[idx];
    if (r == c) v.y = 0.0;
    v.x *= inv_z;
    v.y *= inv_z;
    if (centered) {
        const double2 a = mean[r], b = mean[c];
        const double ar = a.x * inv_z, ai = a.y * inv_z, br = b.x * inv_z, bi = b.y * inv_z;
        v.x -= ar * br + ai * bi;
        v.y -= ai * br - ar * bi;
        if (r == c) v.y = 0.0;
    }
    out[(off + r) * ldo + off + c] = v;
    if (r < c) out[(off + c) * ldo + off + r] = make_double2(v.x, -v.y);
}

}  // namespace

cudaError_t launch_sm_accumulate(const SmSource& a, double2* S, double2* mean, int num_sms, cudaStream_t st) {
    if (a.count <= 0) return cudaSuccess;
    const int nt = (a.L + kT - 1) / kT;
    const int upper = nt * (nt + 1) / 2;
    // split the samples over CTAs only when the triangle alone cannot fill the GPU
    int split = 1;
    const int want = 2 * num_sms;
    if (upper < want) split = std::min((a.count + kFlush - 1) / kFlush, (want + upper - 1) / upper);
    split = std::max(split, 1);
    const int slice = (a.count + split - 1) / split;
    const dim3 grid(nt * nt, split);
    sm_herk_kernel<<<grid, 256, 0, st>>>(a, S, nt, slice, split > 1);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess || !mean) return e;
    return launch_sm_mean(a, mean, st);
}

cudaError_t launch_sm_mean(const SmSource& a, double2* mean, cudaStream_t st) {
    if (a.count <= 0) return cudaSuccess;
    sm_mean_kernel<<<(a.L + 127) / 128, 128, 0, st>>>(a, mean, 0, 1.0);
    return cudaGetLastError();
}

cudaError_t launch_sm_row_mean(const SmSource& a, double2* out, cudaStream_t st) {
    SmSource u = a;
    u.weighted = 0;
    u.shift = nullptr;
    sm_mean_kernel<<<(a.L + 127) / 128, 128, 0, st>>>(u, out, 1, 1.0 / static_cast<double>(a.count));
    return cudaGetLastError();
}

cudaError_t launch_sm_finish(int L, const double2* S, const double2* mean, double inv_z, int centered,
                             double2* out, long ldo, int off, cudaStream_t st) {
    const long n = static_cast<long>(L) * L;
    sm_finish_kernel<<<static_cast<int>((n + 255) / 256), 256, 0, st>>>(L, S, mean, inv_z, centered, out, ldo, off);
    return cudaGetLastError();
}

}  // namespace rbmg
