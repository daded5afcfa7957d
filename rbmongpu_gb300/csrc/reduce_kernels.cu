// Deterministic reductions of per-sample quantities into the estimator sums.
//
// All sums over samples run in a fixed order: FP32 partial sums over chunks of at
// most 32 samples, accumulated in FP64, then per-block partials combined by a
// second kernel in block order.  No floating-point atomics, so results are
// bit-reproducible run to run.
#include "kernels.h"
#include "reduce.h"

namespace rbmg {

namespace {

constexpr int kChunk = 32;

__device__ __forceinline__ float spin_sign(const uint64_t* spins, uint64_t enum_base, int enumerate, long s, int nw,
                                           int i) {
    uint64_t word;
    if (enumerate) {
        const uint64_t idx = enum_base + static_cast<uint64_t>(s);
        word = (i >> 6) == 0 ? idx : 0ull;
    } else {
        word = spins[s * nw + (i >> 6)];
    }
    return ((word >> (i & 63)) & 1ull) ? 1.0f : -1.0f;
}

// grid (ceil(M/32), ceil((1+N)/16), splits), block (32, 8): thread (tx, ty) owns column
// j = 32 bx + tx and rows r = 16 by + 2 ty + {0, 1}.
__global__ void outer_reduce_kernel(int count, int N, int nw, int M, const uint64_t* __restrict__ spins,
                                    uint64_t enum_base, int enumerate, const double2* __restrict__ c,
                                    const float2* __restrict__ A, int lda, int conj_a, double2* __restrict__ partial,
                                    int per_split) {
    __shared__ float2 sA[kChunk][32];
    __shared__ float2 sC[kChunk];
    __shared__ float sSign[kChunk][16];
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int j = blockIdx.x * 32 + tx;
    const int r0 = blockIdx.y * 16 + 2 * ty;
    const long s_begin = static_cast<long>(blockIdx.z) * per_split;
    const long s_end = min(static_cast<long>(count), s_begin + per_split);
    double2 acc[2] = {make_double2(0.0, 0.0), make_double2(0.0, 0.0)};
    const int tid = ty * 32 + tx;
    for (long base = s_begin; base < s_end; base += kChunk) {
        const int n = static_cast<int>(min(static_cast<long>(kChunk), s_end - base));
        __syncthreads();
        for (int q = tid; q < kChunk * 32; q += 256) {
            const int ss = q / 32, jj = q % 32;
            float2 a = make_float2(0.0f, 0.0f);
            if (ss < n && blockIdx.x * 32 + jj < M) {
                a = A[(base + ss) * lda + blockIdx.x * 32 + jj];
                if (conj_a) a.y = -a.y;
            }
            sA[ss][jj] = a;
        }
        for (int q = tid; q < kChunk; q += 256) {
            const double2 cc = q < n ? c[base + q] : make_double2(0.0, 0.0);
            sC[q] = make_float2(static_cast<float>(cc.x), static_cast<float>(cc.y));
        }
        for (int q = tid; q < kChunk * 16; q += 256) {
            const int ss = q / 16, rr = blockIdx.y * 16 + q % 16;
            float sg = 0.0f;
            if (ss < n && rr <= N) sg = rr == 0 ? 1.0f : spin_sign(spins, enum_base, enumerate, base + ss, nw, rr - 1);
            sSign[ss][q % 16] = sg;
        }
        __syncthreads();
        float2 p0 = make_float2(0.0f, 0.0f), p1 = make_float2(0.0f, 0.0f);
        for (int ss = 0; ss < n; ss++) {
            const float2 a = sA[ss][tx], cc = sC[ss];
            const float2 v = make_float2(cc.x * a.x - cc.y * a.y, cc.x * a.y + cc.y * a.x);
            const float g0 = sSign[ss][2 * ty], g1 = sSign[ss][2 * ty + 1];
            p0.x = fmaf(g0, v.x, p0.x);
            p0.y = fmaf(g0, v.y, p0.y);
            p1.x = fmaf(g1, v.x, p1.x);
            p1.y = fmaf(g1, v.y, p1.y);
        }
        acc[0].x += p0.x; acc[0].y += p0.y;
        acc[1].x += p1.x; acc[1].y += p1.y;
    }
    if (j < M) {
        const long plane = static_cast<long>(1 + N) * M;
        for (int q = 0; q < 2; q++) {
            const int r = r0 + q;
            if (r <= N) partial[blockIdx.z * plane + static_cast<long>(r) * M + j] = acc[q];
        }
    }
}

// out[e] += sum_z partial[z][e], in z order
__global__ void finish_splits_kernel(long elems, int splits, const double2* __restrict__ partial, double2* out,
                                     double scale) {
    for (long e = blockIdx.x * static_cast<long>(blockDim.x) + threadIdx.x; e < elems;
         e += static_cast<long>(gridDim.x) * blockDim.x) {
        double2 a = make_double2(0.0, 0.0);
        for (int z = 0; z < splits; z++) {
            const double2 p = partial[z * elems + e];
            a.x += p.x;
            a.y += p.y;
        }
        out[e].x += scale * a.x;
        out[e].y += scale * a.y;
    }
}

// grid (ceil(M/32), N, splits), block 256 = 8 warps; warp w takes samples w, w+8, ...
__global__ void vterm_kernel(int count, int N, int nw, int M, int Mpad, const uint64_t* __restrict__ spins,
                             uint64_t enum_base, int enumerate, const double* __restrict__ w,
                             const double2* __restrict__ cw, const float2* __restrict__ X, int num_offdiag,
                             const int* __restrict__ site_ptr, const int* __restrict__ site_slots,
                             double2* __restrict__ partial, int per_split) {
    __shared__ double2 red[8][32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int j = blockIdx.x * 32 + lane;
    const int i = blockIdx.y;
    const int sb = site_ptr[i], se = site_ptr[i + 1];
    const long s_begin = static_cast<long>(blockIdx.z) * per_split;
    const long s_end = min(static_cast<long>(count), s_begin + per_split);
    double2 acc = make_double2(0.0, 0.0);
    float2 part = make_float2(0.0f, 0.0f);
    int in_chunk = 0;
    if (se > sb && j < Mpad) {
        for (long s = s_begin + warp; s < s_end; s += 8) {
            const float g = spin_sign(spins, enum_base, enumerate, s, nw, i) * (w ? static_cast<float>(w[s]) : 1.0f);
            float2 x = make_float2(0.0f, 0.0f);
            for (int q = sb; q < se; q++) {
                const float2 v = X[(s * num_offdiag + site_slots[q]) * Mpad + j];
                x.x += v.x;
                x.y += v.y;
            }
            if (cw) {   // complex per-sample coefficient
                const float cr = static_cast<float>(cw[s].x), ci = static_cast<float>(cw[s].y);
                x = make_float2(cr * x.x - ci * x.y, cr * x.y + ci * x.x);
            }
            part.x = fmaf(g, x.x, part.x);
            part.y = fmaf(g, x.y, part.y);
            if (++in_chunk == kChunk) {
                acc.x += part.x; acc.y += part.y;
                part = make_float2(0.0f, 0.0f);
                in_chunk = 0;
            }
        }
    }
    acc.x += part.x;
    acc.y += part.y;
    red[warp][lane] = acc;
    __syncthreads();
    if (warp == 0 && j < M) {
        double2 t = make_double2(0.0, 0.0);
        for (int q = 0; q < 8; q++) { t.x += red[q][lane].x; t.y += red[q][lane].y; }
        const long plane = static_cast<long>(1 + N) * M;
        partial[blockIdx.z * plane + static_cast<long>(1 + i) * M + j] = t;
    }
    if (warp == 0 && i == 0 && j < M) {
        const long plane = static_cast<long>(1 + N) * M;
        partial[blockIdx.z * plane + j] = make_double2(0.0, 0.0);   // row 0 carries no V term
    }
}

// ---- weighted sums of complex series -------------------------------------
__global__ void wsum_blocks_kernel(int count, const double* __restrict__ w, SeriesSet set,
                                   double2* __restrict__ block_out) {
    __shared__ double2 red[kMaxSeries][256 / 32];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    double2 acc[kMaxSeries];
    for (int q = 0; q < kMaxSeries; q++) acc[q] = make_double2(0.0, 0.0);
    for (long s = blockIdx.x * 256L + tid; s < count; s += static_cast<long>(gridDim.x) * 256) {
        const double ws = w ? w[s] : 1.0;
        for (int q = 0; q < set.n; q++) {
            const double2 v = set.v[q][s];
            acc[q].x += ws * v.x;
            acc[q].y += ws * v.y;
        }
    }
    for (int q = 0; q < set.n; q++) {
        double x = acc[q].x, y = acc[q].y;
        for (int off = 16; off >= 1; off >>= 1) {
            x += __shfl_down_sync(0xffffffffu, x, off);
            y += __shfl_down_sync(0xffffffffu, y, off);
        }
        if (lane == 0) red[q][warp] = make_double2(x, y);
    }
    __syncthreads();
    if (tid < set.n) {
        double2 t = make_double2(0.0, 0.0);
        for (int q = 0; q < 256 / 32; q++) { t.x += red[tid][q].x; t.y += red[tid][q].y; }
        block_out[blockIdx.x * kMaxSeries + tid] = t;
    }
}

__global__ void wsum_finish_kernel(int blocks, int n, const double2* __restrict__ block_out, double2* sums) {
    const int q = threadIdx.x;
    if (q >= n) return;
    double2 t = make_double2(0.0, 0.0);
    for (int b = 0; b < blocks; b++) { t.x += block_out[b * kMaxSeries + q].x; t.y += block_out[b * kMaxSeries + q].y; }
    sums[q].x += t.x;
    sums[q].y += t.y;
}

// ---- elementwise per-sample coefficients ---------------------------------
__global__ void max_re2_kernel(int count, const double2* __restrict__ lp, double* block_max) {
    __shared__ double red[256];
    double m = -INFINITY;
    for (long s = blockIdx.x * 256L + threadIdx.x; s < count; s += static_cast<long>(gridDim.x) * 256)
        m = fmax(m, 2.0 * lp[s].x);
    red[threadIdx.x] = m;
    __syncthreads();
    for (int h = 128; h >= 1; h >>= 1) {
        if (threadIdx.x < h) red[threadIdx.x] = fmax(red[threadIdx.x], red[threadIdx.x + h]);
        __syncthreads();
    }
    if (threadIdx.x == 0) block_max[blockIdx.x] = red[0];
}

__global__ void exp_weights_kernel(int count, const double2* __restrict__ lp, double shift, double* w) {
    for (long s = blockIdx.x * 256L + threadIdx.x; s < count; s += static_cast<long>(gridDim.x) * 256)
        w[s] = exp(2.0 * lp[s].x - shift);
}

__global__ void coef_kernel(int count, const double* __restrict__ w, const double2* __restrict__ v, double scale,
                            double2 shift, double2* c) {
    for (long s = blockIdx.x * 256L + threadIdx.x; s < count; s += static_cast<long>(gridDim.x) * 256) {
        const double ws = (w ? w[s] : 1.0) * scale;
        c[s] = v ? make_double2(ws * (v[s].x - shift.x), ws * (v[s].y - shift.y)) : make_double2(ws, 0.0);
    }
}

// c[s] = w[s] conj(v[s] - shift)
__global__ void coef_conj_kernel(int count, const double* __restrict__ w, const double2* __restrict__ v,
                                 double2 shift, double2* c) {
    for (long s = blockIdx.x * 256L + threadIdx.x; s < count; s += static_cast<long>(gridDim.x) * 256) {
        const double ws = w ? w[s] : 1.0;
        c[s] = make_double2(ws * (v[s].x - shift.x), -ws * (v[s].y - shift.y));
    }
}

// c[s] = (w[s] (Re v[s] - shift), 0)
__global__ void coef_real_kernel(int count, const double* __restrict__ w, const double2* __restrict__ v, double shift,
                                 double2* c) {
    for (long s = blockIdx.x * 256L + threadIdx.x; s < count; s += static_cast<long>(gridDim.x) * 256)
        c[s] = make_double2((w ? w[s] : 1.0) * (v[s].x - shift), 0.0);
}

// rw[s] = w[s] exp(2 (Re lp[s] - Re lpp[s])) (ExpectationValue.cu:391-395), rwc[s] = (rw[s], 0)
__global__ void ratio_weight_kernel(int count, const double* __restrict__ w, const double2* __restrict__ lp,
                                    const double2* __restrict__ lpp, double* rw, double2* rwc) {
    for (long s = blockIdx.x * 256L + threadIdx.x; s < count; s += static_cast<long>(gridDim.x) * 256) {
        const double r = (w ? w[s] : 1.0) * exp(2.0 * (lp[s].x - lpp[s].x));
        rw[s] = r;
        rwc[s] = make_double2(r, 0.0);
    }
}

// a[s] = exp(2 Im E + Re(E E - E)) (ExpectationValue.cu:106-109)
__global__ void corrected_kernel(int count, const double2* __restrict__ e, double2* a) {
    for (long s = blockIdx.x * 256L + threadIdx.x; s < count; s += static_cast<long>(gridDim.x) * 256) {
        const double2 v = e[s];
        a[s] = make_double2(exp(2.0 * v.y + (v.x * v.x - v.y * v.y - v.x)), 0.0);
    }
}

__global__ void abs2_kernel(int count, const double2* __restrict__ v, double2* out) {
    for (long s = blockIdx.x * 256L + threadIdx.x; s < count; s += static_cast<long>(gridDim.x) * 256)
        out[s] = make_double2(v[s].x * v[s].x + v[s].y * v[s].y, 0.0);
}

// Hilbert-space distance per-sample terms (source/network_functions/HilbertSpaceDistance.cu:83-106)
__global__ void hsd_terms_kernel(int count, const double2* __restrict__ eloc, const double2* __restrict__ lp,
                                 const double2* __restrict__ lpp, int is_unitary, double2* omega, double2* pr,
                                 double2* nn) {
    for (long s = blockIdx.x * 256L + threadIdx.x; s < count; s += static_cast<long>(gridDim.x) * 256) {
        const double2 e = eloc[s];
        const double dr = lpp[s].x - lp[s].x, di = -(lpp[s].y - lp[s].y);   // conj(log psi' - log psi)
        double2 om;
        double n;
        if (is_unitary) {
            const double m = exp(dr);
            const double ar = m * cos(di), ai = m * sin(di);
            om = make_double2(ar * e.x - ai * e.y, ar * e.y + ai * e.x);
            n = e.x * e.x + e.y * e.y;
        } else {
            const double m = exp(e.x + dr);
            om = make_double2(m * cos(e.y + di), m * sin(e.y + di));
            n = exp(2.0 * e.x);
        }
        omega[s] = om;
        pr[s] = make_double2(exp(2.0 * (lpp[s].x - lp[s].x)), 0.0);
        nn[s] = make_double2(n, 0.0);
    }
}

inline int grid_for(long count) { return static_cast<int>(min(1024L, max(1L, (count + 255) / 256))); }

}  // namespace

cudaError_t launch_outer_reduce(int count, int N, int nw, int M, const uint64_t* spins, uint64_t enum_base,
                                int enumerate, const double2* c, const float2* A, int lda, int conj_a, double2* out,
                                double2* partial, int max_splits, cudaStream_t st) {
    if (count <= 0) return cudaSuccess;
    const int per_split = max(kChunk, ((count + max_splits - 1) / max_splits + kChunk - 1) / kChunk * kChunk);
    const int splits = (count + per_split - 1) / per_split;
    const dim3 grid((M + 31) / 32, (N + 1 + 15) / 16, splits), block(32, 8);
    outer_reduce_kernel<<<grid, block, 0, st>>>(count, N, nw, M, spins, enum_base, enumerate, c, A, lda, conj_a,
                                                partial, per_split);
    const long elems = static_cast<long>(1 + N) * M;
    finish_splits_kernel<<<grid_for(elems), 256, 0, st>>>(elems, splits, partial, out, 1.0);
    return cudaGetLastError();
}

cudaError_t launch_vterm_reduce(int count, int N, int nw, int M, int Mpad, const uint64_t* spins, uint64_t enum_base,
                                int enumerate, const double* w, const float2* X, int num_offdiag,
                                const int* site_ptr, const int* site_slots, double2* out, double2* partial,
                                int max_splits, cudaStream_t st, const double2* cw) {
    if (count <= 0 || num_offdiag == 0) return cudaSuccess;
    const int per_split = max(64, (count + max_splits - 1) / max_splits);
    const int splits = (count + per_split - 1) / per_split;
    const dim3 grid((M + 31) / 32, N, splits);
    vterm_kernel<<<grid, 256, 0, st>>>(count, N, nw, M, Mpad, spins, enum_base, enumerate, w, cw, X, num_offdiag,
                                       site_ptr, site_slots, partial, per_split);
    const long elems = static_cast<long>(1 + N) * M;
    finish_splits_kernel<<<grid_for(elems), 256, 0, st>>>(elems, splits, partial, out, -2.0);
    return cudaGetLastError();
}

cudaError_t launch_weighted_sums(int count, const double* w, const SeriesSet& set, double2* block_scratch,
                                 double2* sums, cudaStream_t st) {
    if (count <= 0) return cudaSuccess;
    const int blocks = min(kSumBlocks, max(1, (count + 255) / 256));
    wsum_blocks_kernel<<<blocks, 256, 0, st>>>(count, w, set, block_scratch);
    wsum_finish_kernel<<<1, 32, 0, st>>>(blocks, set.n, block_scratch, sums);
    return cudaGetLastError();
}

cudaError_t launch_max_re2(int count, const double2* lp, double* block_max, int* blocks_out, cudaStream_t st) {
    const int blocks = min(kSumBlocks, max(1, (count + 255) / 256));
    *blocks_out = blocks;
    max_re2_kernel<<<blocks, 256, 0, st>>>(count, lp, block_max);
    return cudaGetLastError();
}

cudaError_t launch_exp_weights(int count, const double2* lp, double shift, double* w, cudaStream_t st) {
    exp_weights_kernel<<<grid_for(count), 256, 0, st>>>(count, lp, shift, w);
    return cudaGetLastError();
}

cudaError_t launch_coef(int count, const double* w, const double2* v, double scale, double2* c, cudaStream_t st,
                        double2 shift) {
    coef_kernel<<<grid_for(count), 256, 0, st>>>(count, w, v, scale, shift, c);
    return cudaGetLastError();
}

cudaError_t launch_coef_conj(int count, const double* w, const double2* v, double2 shift, double2* c,
                             cudaStream_t st) {
    coef_conj_kernel<<<grid_for(count), 256, 0, st>>>(count, w, v, shift, c);
    return cudaGetLastError();
}

cudaError_t launch_coef_real(int count, const double* w, const double2* v, double shift, double2* c,
                             cudaStream_t st) {
    coef_real_kernel<<<grid_for(count), 256, 0, st>>>(count, w, v, shift, c);
    return cudaGetLastError();
}

cudaError_t launch_ratio_weights(int count, const double* w, const double2* lp, const double2* lpp, double* rw,
                                 double2* rwc, cudaStream_t st) {
    ratio_weight_kernel<<<grid_for(count), 256, 0, st>>>(count, w, lp, lpp, rw, rwc);
    return cudaGetLastError();
}

cudaError_t launch_corrected_terms(int count, const double2* e, double2* a, cudaStream_t st) {
    corrected_kernel<<<grid_for(count), 256, 0, st>>>(count, e, a);
    return cudaGetLastError();
}

cudaError_t launch_abs2(int count, const double2* v, double2* out, cudaStream_t st) {
    abs2_kernel<<<grid_for(count), 256, 0, st>>>(count, v, out);
    return cudaGetLastError();
}

cudaError_t launch_hsd_terms(int count, const double2* eloc, const double2* lp, const double2* lpp, int is_unitary,
                             double2* omega, double2* pr, double2* nn, cudaStream_t st) {
    hsd_terms_kernel<<<grid_for(count), 256, 0, st>>>(count, eloc, lp, lpp, is_unitary, omega, pr, nn);
    return cudaGetLastError();
}

}  // namespace rbmg
