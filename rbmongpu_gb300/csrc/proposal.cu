// Learned Metropolis-Hastings proposal for the complex-RBM chain (extension: the
// reference proposes single spin flips only, include/spin_ensembles/MonteCarloLoop.hpp:153-256).
//
// An MLP on the walker's spins, N -> 256 -> 256 (SiLU) -> N + 8 logits, picks a seed site
// i (softmax over the first N logits) and a cluster length l in 1..8 (softmax over the
// last 8); the move flips the contiguous periodic cluster {i, ..., i+l-1}.  For l < N the
// cluster determines (i, l), so q(s'|s) = p_s(i) p_s(l) and the reverse move has
// q(s|s') = p_s'(i) p_s'(l): the acceptance min(1, |psi(s')/psi(s)|^2 q(s|s')/q(s'|s))
// keeps |psi|^2 stationary for any network weights.
//
// The network runs in BF16 operands with FP32 accumulation on the tensor cores
// (mma.sync m16n8k16); forward, backward and Adam are kernels of this file.  It is
// trained online on the chain's own configurations.  The default objective is the
// cross-entropy to the locally balanced proposal (Zanella 2020), p*(i, l | s) propto
// sqrt(|psi(s')|^2 / |psi(s)|^2) over all N x 8 cluster moves, computed exactly for the
// training walkers: it is the proposal whose Metropolis-Hastings acceptance
// Z(s) / Z(s') tends to 1, and the factorised network is fitted to its seed and length
// marginals.  The alternative objective, REINFORCE on the acceptance itself (reward
// min(1, a) * l, batch-mean baseline, entropy bonus), has degenerate optima: a proposal
// that pairs states (s -> s' -> s ...) is accepted almost always and does not mix.
#include <cmath>
#include <cstring>
#include <memory>
#include <vector>

#include <cuda_bf16.h>

#include "host.h"
#include "rbm_impl.cuh"

namespace rbmg {

using bf16 = __nv_bfloat16;

constexpr int kHidden = 256;
constexpr int kLengths = 8;
constexpr float kEntropyBonus = 0.01f;

inline int pad8(int x) { return (x + 7) & ~7; }

// ============================================================================ GEMM
// C[M][N] = A[M][K] B[K][N] with BF16 operands and FP32 accumulation.  A is stored
// [m][k] (A_MK) or [k][m] (A_KM), B is stored [n][k] (B_NK) or [k][n] (B_KN); leading
// dimensions are multiples of 8 elements and 16-byte aligned.  Columns past K inside a
// row's leading dimension must hold zeros (they enter the sums); columns past M or N
// are only read, never stored.
enum : int { A_MK = 0, A_KM = 1 };
enum : int { B_NK = 0, B_KN = 1 };
enum : int {
    EPI_F32 = 0,     // C32 = acc + bias
    EPI_SILU = 1,    // C32 = z = acc + bias, C16 = bf16(silu(z))
    EPI_DSILU = 2,   // C32 = dz = acc * silu'(Z), C16 = bf16(dz)
    EPI_PARTIAL = 3  // C32[split] = acc (split-K partial sums)
};

struct GemmArgs {
    int M, N, K;
    const bf16* A;
    int lda;
    const bf16* B;
    int ldb;
    int k_per_split;     // multiple of kBK
    const float* bias;   // [N] or null
    float* C32;
    int ldc;
    bf16* C16;
    int ldc16;
    const float* Z;
    int ldz;
    long split_stride;   // elements between the partial sums of consecutive splits
};

constexpr int kBM = 128, kBN = 64, kBK = 32, kSK = kBK + 8, kGemmThreads = 256;

// SiLU and its derivative with the hardware exponential and division: the activations
// are rounded to BF16 (8 significant bits) right after, far above their ~1e-6 error
__device__ __forceinline__ float silu_f(float z) { return __fdividef(z, 1.0f + __expf(-z)); }
__device__ __forceinline__ float dsilu_f(float z) {
    const float sg = __fdividef(1.0f, 1.0f + __expf(-z));
    return sg * (1.0f + z * (1.0f - sg));
}

__device__ __forceinline__ void mma_bf16_16816(float (&d)[4], const uint32_t (&a)[4], const uint32_t (&b)[2]) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

template <int LA, int LB, int EPI>
__global__ void __launch_bounds__(kGemmThreads) gemm_bf16_kernel(GemmArgs g) {
    __shared__ __align__(16) bf16 sA[kBM][kSK];
    __shared__ __align__(16) bf16 sB[kBN][kSK];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int wm = warp & 3, wn = warp >> 2;       // 4 x 2 warps, 32 x 32 each
    const int gq = lane >> 2, tq = lane & 3;
    const int m0 = blockIdx.x * kBM, n0 = blockIdx.y * kBN;
    const int kbeg = blockIdx.z * g.k_per_split;
    const int kend = min(g.K, kbeg + g.k_per_split);
    float acc[2][4][4];
#pragma unroll
    for (int i = 0; i < 2; i++)
#pragma unroll
        for (int j = 0; j < 4; j++)
#pragma unroll
            for (int e = 0; e < 4; e++) acc[i][j][e] = 0.0f;
    const uint4 zero = make_uint4(0u, 0u, 0u, 0u);
    for (int k0 = kbeg; k0 < kend; k0 += kBK) {
        // ---- stage A as sA[m][k]
        if (LA == A_MK) {
            for (int c = tid; c < kBM * (kBK / 8); c += kGemmThreads) {
                const int r = c >> 2, kc = (c & 3) * 8;
                const int m = m0 + r, k = k0 + kc;
                uint4 v = zero;
                if (m < g.M && k < kend) v = *reinterpret_cast<const uint4*>(g.A + static_cast<long>(m) * g.lda + k);
                *reinterpret_cast<uint4*>(&sA[r][kc]) = v;
            }
        } else {
            for (int c = tid; c < kBK * (kBM / 8); c += kGemmThreads) {
                const int kk = c / (kBM / 8), mc = (c % (kBM / 8)) * 8;
                const int k = k0 + kk, m = m0 + mc;
                uint4 v = zero;
                if (k < kend && m < g.M) v = *reinterpret_cast<const uint4*>(g.A + static_cast<long>(k) * g.lda + m);
                const bf16* e = reinterpret_cast<const bf16*>(&v);
#pragma unroll
                for (int q = 0; q < 8; q++) sA[mc + q][kk] = e[q];
            }
        }
        // ---- stage B as sB[n][k]
        if (LB == B_NK) {
            for (int c = tid; c < kBN * (kBK / 8); c += kGemmThreads) {
                const int r = c >> 2, kc = (c & 3) * 8;
                const int n = n0 + r, k = k0 + kc;
                uint4 v = zero;
                if (n < g.N && k < kend) v = *reinterpret_cast<const uint4*>(g.B + static_cast<long>(n) * g.ldb + k);
                *reinterpret_cast<uint4*>(&sB[r][kc]) = v;
            }
        } else {
            for (int c = tid; c < kBK * (kBN / 8); c += kGemmThreads) {
                const int kk = c / (kBN / 8), nc = (c % (kBN / 8)) * 8;
                const int k = k0 + kk, n = n0 + nc;
                uint4 v = zero;
                if (k < kend && n < g.N) v = *reinterpret_cast<const uint4*>(g.B + static_cast<long>(k) * g.ldb + n);
                const bf16* e = reinterpret_cast<const bf16*>(&v);
#pragma unroll
                for (int q = 0; q < 8; q++) sB[nc + q][kk] = e[q];
            }
        }
        __syncthreads();
#pragma unroll
        for (int ks = 0; ks < kBK; ks += 16) {
            uint32_t af[2][4], bfr[4][2];
#pragma unroll
            for (int mi = 0; mi < 2; mi++) {
                const int row = wm * 32 + mi * 16 + gq;
                af[mi][0] = *reinterpret_cast<const uint32_t*>(&sA[row][ks + 2 * tq]);
                af[mi][1] = *reinterpret_cast<const uint32_t*>(&sA[row + 8][ks + 2 * tq]);
                af[mi][2] = *reinterpret_cast<const uint32_t*>(&sA[row][ks + 2 * tq + 8]);
                af[mi][3] = *reinterpret_cast<const uint32_t*>(&sA[row + 8][ks + 2 * tq + 8]);
            }
#pragma unroll
            for (int ni = 0; ni < 4; ni++) {
                const int col = wn * 32 + ni * 8 + gq;
                bfr[ni][0] = *reinterpret_cast<const uint32_t*>(&sB[col][ks + 2 * tq]);
                bfr[ni][1] = *reinterpret_cast<const uint32_t*>(&sB[col][ks + 2 * tq + 8]);
            }
#pragma unroll
            for (int mi = 0; mi < 2; mi++)
#pragma unroll
                for (int ni = 0; ni < 4; ni++) mma_bf16_16816(acc[mi][ni], af[mi], bfr[ni]);
        }
        __syncthreads();
    }
    // ---- epilogue: acc[mi][ni][h * 2 + e] is C[row g + 8 h][col 2 t + e] of the tile
#pragma unroll
    for (int mi = 0; mi < 2; mi++)
#pragma unroll
        for (int ni = 0; ni < 4; ni++)
#pragma unroll
            for (int h = 0; h < 2; h++)
#pragma unroll
                for (int e = 0; e < 2; e++) {
                    const int m = m0 + wm * 32 + mi * 16 + gq + 8 * h;
                    const int n = n0 + wn * 32 + ni * 8 + 2 * tq + e;
                    if (m >= g.M || n >= g.N) continue;
                    const float a = acc[mi][ni][h * 2 + e];
                    if (EPI == EPI_F32) {
                        g.C32[static_cast<long>(m) * g.ldc + n] = a + (g.bias ? g.bias[n] : 0.0f);
                    } else if (EPI == EPI_SILU) {
                        const float z = a + g.bias[n];
                        g.C32[static_cast<long>(m) * g.ldc + n] = z;
                        g.C16[static_cast<long>(m) * g.ldc16 + n] = __float2bfloat16_rn(silu_f(z));
                    } else if (EPI == EPI_DSILU) {
                        const float dz = a * dsilu_f(g.Z[static_cast<long>(m) * g.ldz + n]);
                        g.C32[static_cast<long>(m) * g.ldc + n] = dz;
                        g.C16[static_cast<long>(m) * g.ldc16 + n] = __float2bfloat16_rn(dz);
                    } else {
                        g.C32[blockIdx.z * g.split_stride + static_cast<long>(m) * g.ldc + n] = a;
                    }
                }
}

template <int LA, int LB, int EPI>
cudaError_t gemm(const GemmArgs& g, int splits, cudaStream_t st) {
    if (g.M <= 0 || g.N <= 0) return cudaSuccess;
    const dim3 grid((g.M + kBM - 1) / kBM, (g.N + kBN - 1) / kBN, splits);
    gemm_bf16_kernel<LA, LB, EPI><<<grid, kGemmThreads, 0, st>>>(g);
    return cudaGetLastError();
}

// out[m * ldo + n] = sum over splits s (in order) of part[s][m * ldp + n]
__global__ void split_reduce_kernel(const float* part, int splits, long stride, int M, int N, int ldp, float* out,
                                    int ldo) {
    const long t = static_cast<long>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (t >= static_cast<long>(M) * N) return;
    const int m = static_cast<int>(t / N), n = static_cast<int>(t % N);
    float s = 0.0f;
    for (int q = 0; q < splits; q++) s += part[q * stride + static_cast<long>(m) * ldp + n];
    out[static_cast<long>(m) * ldo + n] = s;
}

// column sums of X[rows][ld] (first `cols` columns), two passes in a fixed order
constexpr int kColChunks = 64;
__global__ void colsum_partial_kernel(const float* X, int rows, int cols, int ld, float* part) {
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= cols) return;
    const int per = (rows + kColChunks - 1) / kColChunks;
    const int r0 = blockIdx.y * per, r1 = min(rows, r0 + per);
    float s = 0.0f;
    for (int r = r0; r < r1; r++) s += X[static_cast<long>(r) * ld + n];
    part[blockIdx.y * cols + n] = s;
}

__global__ void colsum_final_kernel(const float* part, int cols, float* out) {
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= cols) return;
    float s = 0.0f;
    for (int q = 0; q < kColChunks; q++) s += part[q * cols + n];
    out[n] = s;
}

// x[b][i] = +-1 (bf16) for i < N, 0 up to the padded width
template <int NW>
__global__ void spins_to_x_kernel(const uint64_t* spins, int count, int N, int Np, bf16* x) {
    const long t = static_cast<long>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (t >= static_cast<long>(count) * Np) return;
    const long b = t / Np;
    const int i = static_cast<int>(t % Np);
    float v = 0.0f;
    if (i < N) v = ((spins[b * NW + (i >> 6)] >> (i & 63)) & 1ull) ? 1.0f : -1.0f;
    x[t] = __float2bfloat16_rn(v);
}

// dl16[b][j] = bf16(dl32[b][j]) for j < O, 0 up to Op
__global__ void to_bf16_padded_kernel(const float* src, int rows, int cols, int ldd, bf16* dst) {
    const long t = static_cast<long>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (t >= static_cast<long>(rows) * ldd) return;
    const long r = t / ldd;
    const int c = static_cast<int>(t % ldd);
    dst[t] = __float2bfloat16_rn(c < cols ? src[r * cols + c] : 0.0f);
}

// Adam (Kingma & Ba 2015) with bias correction bc1 = 1 - beta1^t, bc2 = 1 - beta2^t
__global__ void adam_kernel(float* p, const float* g, float* m, float* v, long n, float lr, float bc1, float bc2) {
    const long t = static_cast<long>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (t >= n) return;
    const float gt = g[t];
    const float mt = 0.9f * m[t] + 0.1f * gt;
    const float vt = 0.999f * v[t] + 0.001f * gt * gt;
    m[t] = mt;
    v[t] = vt;
    p[t] -= lr * (mt / bc1) / (sqrtf(vt / bc2) + 1e-8f);
}

// bf16 copy of a [rows][cols] FP32 matrix into [rows][ldd] (pad columns zero)
__global__ void weights_to_bf16_kernel(const float* w, int rows, int cols, int ldd, bf16* out) {
    const long t = static_cast<long>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (t >= static_cast<long>(rows) * ldd) return;
    const long r = t / ldd;
    const int c = static_cast<int>(t % ldd);
    out[t] = __float2bfloat16_rn(c < cols ? w[r * cols + c] : 0.0f);
}

// out[n][k] = bf16(w[k][n]) for a [rows][cols] FP32 matrix w, out [out_rows][ldo]; zero
// outside (k >= rows or n >= cols)
__global__ void weights_to_bf16_t_kernel(const float* w, int rows, int cols, int out_rows, int ldo, bf16* out) {
    const long t = static_cast<long>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (t >= static_cast<long>(out_rows) * ldo) return;
    const int n = static_cast<int>(t / ldo), k = static_cast<int>(t % ldo);
    out[t] = __float2bfloat16_rn(n < cols && k < rows ? w[static_cast<long>(k) * cols + n] : 0.0f);
}

inline unsigned blocks_for(long n, int threads = 256) { return static_cast<unsigned>((n + threads - 1) / threads); }

}  // namespace rbmg

// ============================================================================ the network
struct rbmg_proposal {
    int N = 0, O = 0, Np = 0, Op = 0;
    float lr = 1e-3f;
    int objective = RBMG_PROPOSAL_LOCALLY_BALANCED;
    long steps = 0;   // Adam steps taken
    int64_t P = 0;
    size_t oW1 = 0, ob1 = 0, oW2 = 0, ob2 = 0, oW3 = 0, ob3 = 0;   // offsets in the FP32 parameter vector
    rbmg::DevBuf master, adam_m, adam_v, grad;
    rbmg::DevBuf w1, w2, w3;            // bf16 [N][H], [H][H], [H][Op]
    // transposed bf16 copies for the fused inference kernel: [H][ldw1], [H][H], [w3_rows][H]
    rbmg::DevBuf w1t, w2t, w3t;
    rbmg::DevBuf tcpack;                // the tensor-core kernel's B operands in its shared-memory layout (O <= 128)
    int ldw1 = 0, w3_rows = 0;
    rbmg::DevBuf tc_error;              // set by the tensor-core kernel when a bounded wait gives up
    int cap = 0;                        // activation rows held
    rbmg::DevBuf x16, z1, h1, z2, h2;   // [cap][Np] bf16, [cap][H] f32 / bf16
    rbmg::DevBuf logits;                // [cap][O] f32 (training forward)
    rbmg::DevBuf dl32, dl16, dz2_32, dz2_16, dz1_32, dz1_16;
    rbmg::DevBuf partial, colpart;
};

namespace rbmg {

int proposal_reserve(rbmg_proposal* p, int rows) {
    if (rows <= p->cap) return RBMG_OK;
    const size_t r = static_cast<size_t>(rows);
    RBMG_CK(p->x16.ensure(sizeof(bf16) * r * p->Np));
    RBMG_CK(p->z1.ensure(sizeof(float) * r * kHidden));
    RBMG_CK(p->h1.ensure(sizeof(bf16) * r * kHidden));
    RBMG_CK(p->z2.ensure(sizeof(float) * r * kHidden));
    RBMG_CK(p->h2.ensure(sizeof(bf16) * r * kHidden));
    RBMG_CK(p->logits.ensure(sizeof(float) * r * p->O));
    RBMG_CK(p->dl32.ensure(sizeof(float) * r * p->O));
    RBMG_CK(p->dl16.ensure(sizeof(bf16) * r * p->Op));
    RBMG_CK(p->dz2_32.ensure(sizeof(float) * r * kHidden));
    RBMG_CK(p->dz2_16.ensure(sizeof(bf16) * r * kHidden));
    RBMG_CK(p->dz1_32.ensure(sizeof(float) * r * kHidden));
    RBMG_CK(p->dz1_16.ensure(sizeof(bf16) * r * kHidden));
    p->cap = rows;
    return RBMG_OK;
}

cudaError_t proposal_refresh_tc(rbmg_proposal* p, cudaStream_t st);

cudaError_t proposal_refresh_bf16(rbmg_proposal* p, cudaStream_t st) {
    const float* w = p->master.as<float>();
    weights_to_bf16_kernel<<<blocks_for(static_cast<long>(p->N) * kHidden), 256, 0, st>>>(w + p->oW1, p->N, kHidden,
                                                                                          kHidden, p->w1.as<bf16>());
    weights_to_bf16_kernel<<<blocks_for(static_cast<long>(kHidden) * kHidden), 256, 0, st>>>(
        w + p->oW2, kHidden, kHidden, kHidden, p->w2.as<bf16>());
    weights_to_bf16_kernel<<<blocks_for(static_cast<long>(kHidden) * p->Op), 256, 0, st>>>(w + p->oW3, kHidden, p->O,
                                                                                         p->Op, p->w3.as<bf16>());
    weights_to_bf16_t_kernel<<<blocks_for(static_cast<long>(kHidden) * p->ldw1), 256, 0, st>>>(
        w + p->oW1, p->N, kHidden, kHidden, p->ldw1, p->w1t.as<bf16>());
    weights_to_bf16_t_kernel<<<blocks_for(static_cast<long>(kHidden) * kHidden), 256, 0, st>>>(
        w + p->oW2, kHidden, kHidden, kHidden, kHidden, p->w2t.as<bf16>());
    weights_to_bf16_t_kernel<<<blocks_for(static_cast<long>(p->w3_rows) * kHidden), 256, 0, st>>>(
        w + p->oW3, kHidden, p->O, p->w3_rows, kHidden, p->w3t.as<bf16>());
    const cudaError_t e = cudaGetLastError();
    return e != cudaSuccess ? e : proposal_refresh_tc(p, st);
}

// logits_out [count][O] of the configurations spins [count][nw] (logits_out null: the
// network's own logits buffer, valid only after the reserve below); activations kept in
// the network's buffers for a following backward pass
int proposal_forward(rbmg_proposal* p, int count, const uint64_t* spins, float* logits_out, cudaStream_t st) {
    if (count <= 0) return RBMG_OK;
    int r = proposal_reserve(p, count);
    if (r != RBMG_OK) return r;
    if (!logits_out) logits_out = p->logits.as<float>();
    const int nw = nwords_of(p->N);
    const long xs = static_cast<long>(count) * p->Np;
    switch (nw) {
        case 1: spins_to_x_kernel<1><<<blocks_for(xs), 256, 0, st>>>(spins, count, p->N, p->Np, p->x16.as<bf16>()); break;
        case 2: spins_to_x_kernel<2><<<blocks_for(xs), 256, 0, st>>>(spins, count, p->N, p->Np, p->x16.as<bf16>()); break;
        case 3: spins_to_x_kernel<3><<<blocks_for(xs), 256, 0, st>>>(spins, count, p->N, p->Np, p->x16.as<bf16>()); break;
        default: spins_to_x_kernel<4><<<blocks_for(xs), 256, 0, st>>>(spins, count, p->N, p->Np, p->x16.as<bf16>()); break;
    }
    RBMG_CK(cudaGetLastError());
    const float* w = p->master.as<float>();
    GemmArgs g{};
    g.M = count;
    g.N = kHidden;
    g.K = p->N;
    g.A = p->x16.as<bf16>();
    g.lda = p->Np;
    g.B = p->w1.as<bf16>();
    g.ldb = kHidden;
    g.k_per_split = (g.K + kBK - 1) / kBK * kBK;
    g.bias = w + p->ob1;
    g.C32 = p->z1.as<float>();
    g.ldc = kHidden;
    g.C16 = p->h1.as<bf16>();
    g.ldc16 = kHidden;
    RBMG_CK((gemm<A_MK, B_KN, EPI_SILU>(g, 1, st)));
    g.K = kHidden;
    g.A = p->h1.as<bf16>();
    g.lda = kHidden;
    g.B = p->w2.as<bf16>();
    g.k_per_split = kHidden;
    g.bias = w + p->ob2;
    g.C32 = p->z2.as<float>();
    g.C16 = p->h2.as<bf16>();
    RBMG_CK((gemm<A_MK, B_KN, EPI_SILU>(g, 1, st)));
    g.N = p->O;
    g.A = p->h2.as<bf16>();
    g.B = p->w3.as<bf16>();
    g.ldb = p->Op;
    g.bias = w + p->ob3;
    g.C32 = logits_out;
    g.ldc = p->O;
    g.C16 = nullptr;
    RBMG_CK((gemm<A_MK, B_KN, EPI_F32>(g, 1, st)));
    return RBMG_OK;
}

// dW = A^T dZ over `count` rows (split-K partials, reduced in a fixed order) into grad
static int weight_grad(rbmg_proposal* p, int count, const bf16* A, int lda, int Mrows, const bf16* dZ, int ldz,
                       int Ncols, float* out, cudaStream_t st) {
    const int tiles = ((Mrows + kBM - 1) / kBM) * ((Ncols + kBN - 1) / kBN);
    const int kchunks = (count + kBK - 1) / kBK;
    int splits = std::max(1, std::min(kchunks, (2 * 152 + tiles - 1) / tiles));
    const int per = (kchunks + splits - 1) / splits * kBK;
    splits = (count + per - 1) / per;
    const long stride = static_cast<long>(Mrows) * Ncols;
    RBMG_CK(p->partial.ensure(sizeof(float) * stride * splits));
    GemmArgs g{};
    g.M = Mrows;
    g.N = Ncols;
    g.K = count;
    g.A = A;
    g.lda = lda;
    g.B = dZ;
    g.ldb = ldz;
    g.k_per_split = per;
    g.C32 = p->partial.as<float>();
    g.ldc = Ncols;
    g.split_stride = stride;
    RBMG_CK((gemm<A_KM, B_KN, EPI_PARTIAL>(g, splits, st)));
    split_reduce_kernel<<<blocks_for(stride), 256, 0, st>>>(p->partial.as<float>(), splits, stride, Mrows, Ncols, Ncols,
                                                            out, Ncols);
    RBMG_CK(cudaGetLastError());
    return RBMG_OK;
}

static int bias_grad(rbmg_proposal* p, const float* X, int rows, int cols, float* out, cudaStream_t st) {
    RBMG_CK(p->colpart.ensure(sizeof(float) * kColChunks * cols));
    colsum_partial_kernel<<<dim3(blocks_for(cols), kColChunks), 256, 0, st>>>(X, rows, cols, cols,
                                                                            p->colpart.as<float>());
    colsum_final_kernel<<<blocks_for(cols), 256, 0, st>>>(p->colpart.as<float>(), cols, out);
    RBMG_CK(cudaGetLastError());
    return RBMG_OK;
}

// gradient of sum_b sum_j dl32[b][j] logits[b][j] with respect to all parameters, for
// the activations of the last proposal_forward over `count` rows -> p->grad
int proposal_backward(rbmg_proposal* p, int count, cudaStream_t st) {
    float* gr = p->grad.as<float>();
    const long n16 = static_cast<long>(count) * p->Op;
    to_bf16_padded_kernel<<<blocks_for(n16), 256, 0, st>>>(p->dl32.as<float>(), count, p->O, p->Op,
                                                           p->dl16.as<bf16>());
    RBMG_CK(cudaGetLastError());
    int r = weight_grad(p, count, p->h2.as<bf16>(), kHidden, kHidden, p->dl16.as<bf16>(), p->Op, p->O, gr + p->oW3, st);
    if (r != RBMG_OK) return r;
    r = bias_grad(p, p->dl32.as<float>(), count, p->O, gr + p->ob3, st);
    if (r != RBMG_OK) return r;
    GemmArgs g{};
    g.M = count;
    g.N = kHidden;
    g.K = p->O;
    g.A = p->dl16.as<bf16>();
    g.lda = p->Op;
    g.B = p->w3.as<bf16>();
    g.ldb = p->Op;
    g.k_per_split = (p->O + kBK - 1) / kBK * kBK;
    g.Z = p->z2.as<float>();
    g.ldz = kHidden;
    g.C32 = p->dz2_32.as<float>();
    g.ldc = kHidden;
    g.C16 = p->dz2_16.as<bf16>();
    g.ldc16 = kHidden;
    RBMG_CK((gemm<A_MK, B_NK, EPI_DSILU>(g, 1, st)));
    r = weight_grad(p, count, p->h1.as<bf16>(), kHidden, kHidden, p->dz2_16.as<bf16>(), kHidden, kHidden, gr + p->oW2,
                    st);
    if (r != RBMG_OK) return r;
    r = bias_grad(p, p->dz2_32.as<float>(), count, kHidden, gr + p->ob2, st);
    if (r != RBMG_OK) return r;
    g.K = kHidden;
    g.A = p->dz2_16.as<bf16>();
    g.lda = kHidden;
    g.B = p->w2.as<bf16>();
    g.ldb = kHidden;
    g.k_per_split = kHidden;
    g.Z = p->z1.as<float>();
    g.C32 = p->dz1_32.as<float>();
    g.C16 = p->dz1_16.as<bf16>();
    RBMG_CK((gemm<A_MK, B_NK, EPI_DSILU>(g, 1, st)));
    r = weight_grad(p, count, p->x16.as<bf16>(), p->Np, p->N, p->dz1_16.as<bf16>(), kHidden, kHidden, gr + p->oW1, st);
    if (r != RBMG_OK) return r;
    return bias_grad(p, p->dz1_32.as<float>(), count, kHidden, gr + p->ob1, st);
}

int proposal_adam(rbmg_proposal* p, cudaStream_t st) {
    p->steps++;
    const double bc1 = 1.0 - std::pow(0.9, static_cast<double>(p->steps));
    const double bc2 = 1.0 - std::pow(0.999, static_cast<double>(p->steps));
    adam_kernel<<<blocks_for(p->P), 256, 0, st>>>(p->master.as<float>(), p->grad.as<float>(), p->adam_m.as<float>(),
                                                  p->adam_v.as<float>(), p->P, p->lr, static_cast<float>(bc1),
                                                  static_cast<float>(bc2));
    RBMG_CK(cudaGetLastError());
    RBMG_CK(proposal_refresh_bf16(p, st));
    return RBMG_OK;
}

// ============================================================================ chain kernels
// log-normalisers of the seed and length softmaxes of one logits row (warp-wide,
// identical in every lane; the same function serves the forward and the reverse
// density, so both see bit-identical values for identical logits).  The softmax
// arithmetic (expf_det, logf_det, explicitly rounded sums in a fixed order) is replayed
// bit for bit by the CPU restatement, so the chain's draws can be checked exactly.
struct LogNorm {
    float seed, len;
};

// one logits row in registers: seed logits j = lane + 32 c (N <= 256), length logit `lane`
struct RowRegs {
    float v[8], vl;
};

__device__ __forceinline__ RowRegs load_row(const float* row, int N, int lane) {
    RowRegs r;
#pragma unroll
    for (int c = 0; c < 8; c++) r.v[c] = lane + 32 * c < N ? row[lane + 32 * c] : -INFINITY;
    r.vl = lane < kLengths ? row[N + lane] : -INFINITY;
    return r;
}

__device__ __forceinline__ LogNorm log_norms_of(const RowRegs& r, int N, int lane) {
    const float* v = r.v;
    const float vl = r.vl;
    float m = v[0];
#pragma unroll
    for (int c = 1; c < 8; c++) m = fmaxf(m, v[c]);
#pragma unroll
    for (int off = 16; off >= 1; off >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, off));
    float s = 0.0f;
#pragma unroll
    for (int c = 0; c < 8; c++)
        if (lane + 32 * c < N) s = __fadd_rn(s, expf_det(__fsub_rn(v[c], m)));
    s = warp_sum_xor(s);
    float m2 = vl;
#pragma unroll
    for (int off = 16; off >= 1; off >>= 1) m2 = fmaxf(m2, __shfl_xor_sync(0xffffffffu, m2, off));
    const float s2 = warp_sum_xor(lane < kLengths ? expf_det(__fsub_rn(vl, m2)) : 0.0f);
    return LogNorm{__fadd_rn(m, logf_det(s)), __fadd_rn(m2, logf_det(s2))};
}

__device__ __forceinline__ LogNorm log_norms(const float* row, int N, int lane) {
    return log_norms_of(load_row(row, N, lane), N, lane);
}

// inverse-CDF draw from softmax(row[0..n)) with u in (0, 1]; entries are visited in
// index order, 32 at a time
__device__ __forceinline__ int draw_index(const float* row, int n, float lse, float u, int lane) {
    const float target = u;
    float base = 0.0f;
    int last = 0;
    for (int c = 0; c < n; c += 32) {
        const int j = c + lane;
        const float e = j < n ? expf_det(__fsub_rn(row[j], lse)) : 0.0f;
        float x = e;
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            const float y = __shfl_up_sync(0xffffffffu, x, off);
            if (lane >= off) x = __fadd_rn(x, y);
        }
        const float cum = __fadd_rn(base, x);
        const unsigned hit = __ballot_sync(0xffffffffu, e > 0.0f && cum >= target);
        if (hit) return c + __ffs(hit) - 1;
        const unsigned pos = __ballot_sync(0xffffffffu, e > 0.0f);
        if (pos) last = c + 31 - __clz(pos);
        base = __fadd_rn(base, __shfl_sync(0xffffffffu, x, 31));
    }
    return last;
}

// log q(i, l) = log softmax_seed(i) + log softmax_len(l) of one logits row
__device__ __forceinline__ float log_q_of(const float* row, int N, int i, int l, const LogNorm& ln) {
    return __fadd_rn(__fsub_rn(row[i], ln.seed), __fsub_rn(row[N + l - 1], ln.len));
}

struct LearnedLaunch {
    int B, N, O;
    uint64_t seed;
    uint64_t* spins;             // [B][NW] chain state
    uint64_t* rng_index;         // [B]
    uint64_t* spins_prop;        // [B][NW]
    uint64_t* spins_pre;         // [B][NW] or null (training copy of the state the move started from)
    int* site;                   // [B]
    int* len;                    // [B]
    float* logq_fwd;             // [B]
    float* logits_cur;           // [B][O] logits at the current state
    const float* logits_prop;    // [B][O] logits at the proposed state
    float4* theta;               // [B][KP][32] angles of a lane's units 2 kk, 2 kk + 1: (re, re, im, im)
    float2* re;                  // [B][KP][32] their Re f(theta)   (KP = ceil(K / 2), kernels.h pairing)
    float* reward;               // [B]
    unsigned long long* accepts;
    unsigned long long* proposals;
    int propose_next;            // accept kernel: also draw the next step's move (frozen network)
    int walker_base;             // walker index of entry 0 (a slice of the chain): keys its Philox streams
};

template <int K, int NW>
__global__ void __launch_bounds__(32 * kWarpsPerBlock) learned_angles_kernel(RbmDev P, LearnedLaunch L) {
    const int lane = threadIdx.x & 31;
    const int w = blockIdx.x * kWarpsPerBlock + (threadIdx.x >> 5);
    if (w >= L.B) return;
    Spins<NW> s;
#pragma unroll
    for (int k = 0; k < NW; k++) s.w[k] = L.spins[static_cast<long>(w) * NW + k];
    constexpr int KP = (K + 1) / 2;
    pair_t tr[KP], ti[KP];
    rbm_refresh2(P, s, tr, ti, lane);
#pragma unroll
    for (int kk = 0; kk < KP; kk++) {
        const long o = (static_cast<long>(w) * KP + kk) * 32 + lane;
        float a0, a1, b0, b1, r0, r1;
        up2(tr[kk], a0, a1);
        up2(ti[kk], b0, b1);
        up2(lc_re2(tr[kk], ti[kk]), r0, r1);
        L.theta[o] = make_float4(a0, a1, b0, b1);
        L.re[o] = make_float2(r0, r1);
    }
}

// the move of every walker drawn from the logits of its current state (warp per walker)
template <int NW>
__global__ void __launch_bounds__(32 * kWarpsPerBlock) learned_draw_kernel(LearnedLaunch L) {
    const int lane = threadIdx.x & 31;
    const int w = blockIdx.x * kWarpsPerBlock + (threadIdx.x >> 5);
    if (w >= L.B) return;
    WalkerRng rng;
    rng.init(L.seed, static_cast<uint32_t>(L.walker_base + w), L.rng_index[w]);
    const float* row = L.logits_cur + static_cast<long>(w) * L.O;
    const LogNorm ln = log_norms(row, L.N, lane);
    const int i = draw_index(row, L.N, ln.seed, rng.uniform(), lane);
    const int l = 1 + draw_index(row + L.N, kLengths, ln.len, rng.uniform(), lane);
    if (lane == 0) {
        Spins<NW> s;
#pragma unroll
        for (int k = 0; k < NW; k++) s.w[k] = L.spins[static_cast<long>(w) * NW + k];
        if (L.spins_pre) {
#pragma unroll
            for (int k = 0; k < NW; k++) L.spins_pre[static_cast<long>(w) * NW + k] = s.w[k];
        }
        for (int q = 0; q < l; q++) {
            int c = i + q;
            if (c >= L.N) c -= L.N;
            s.flip(c);
        }
#pragma unroll
        for (int k = 0; k < NW; k++) L.spins_prop[static_cast<long>(w) * NW + k] = s.w[k];
        L.site[w] = i;
        L.len[w] = l;
        L.logq_fwd[w] = log_q_of(row, L.N, i, l, ln);
        L.rng_index[w] = rng.index;
        L.proposals[w] += 1;
    }
}

cudaError_t launch_draw(const LearnedLaunch& L, cudaStream_t st) {
    const dim3 grid((L.B + kWarpsPerBlock - 1) / kWarpsPerBlock), block(32 * kWarpsPerBlock);
    switch (nwords_of(L.N)) {
        case 1: learned_draw_kernel<1><<<grid, block, 0, st>>>(L); break;
        case 2: learned_draw_kernel<2><<<grid, block, 0, st>>>(L); break;
        case 3: learned_draw_kernel<3><<<grid, block, 0, st>>>(L); break;
        case 4: learned_draw_kernel<4><<<grid, block, 0, st>>>(L); break;
        default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

// Metropolis-Hastings test of the proposed cluster flip:
// log a = 2 (Re log psi(s') - Re log psi(s)) + log q(s|s') - log q(s'|s)
template <int K, int NW>
__global__ void __launch_bounds__(32 * kWarpsPerBlock) learned_accept_kernel(RbmDev P, LearnedLaunch L) {
    const int lane = threadIdx.x & 31;
    const int w = blockIdx.x * kWarpsPerBlock + (threadIdx.x >> 5);
    if (w >= L.B) return;
    // every independent load is issued up front: the move, the spins, the proposed
    // state's logits row, the angles and their Re f
    Spins<NW> s;
#pragma unroll
    for (int k = 0; k < NW; k++) s.w[k] = L.spins[static_cast<long>(w) * NW + k];
    const int i = L.site[w], l = L.len[w];
    const float* rowp = L.logits_prop + static_cast<long>(w) * L.O;
    const RowRegs rr = load_row(rowp, L.N, lane);
    constexpr int KP = (K + 1) / 2;
    const long base = static_cast<long>(w) * KP * 32 + lane;
    pair_t tr[KP], ti[KP], re[KP];
#pragma unroll
    for (int kk = 0; kk < KP; kk++) {
        const float4 t = L.theta[base + 32 * kk];
        const float2 f = L.re[base + 32 * kk];
        tr[kk] = pk2(t.x, t.y);
        ti[kk] = pk2(t.z, t.w);
        re[kk] = pk2(f.x, f.y);
    }
    // trial angles: two_s = 2 * (new spin) for each cluster site, added in cluster order
    // (per unit the scalar sequence), from the paired W rows
    pair_t nr[KP], ni[KP], nre[KP];
#pragma unroll
    for (int kk = 0; kk < KP; kk++) { nr[kk] = tr[kk]; ni[kk] = ti[kk]; }
    for (int q = 0; q < l; q++) {
        int c = i + q;
        if (c >= P.N) c -= P.N;
        const pair_t ts = splat2(s.up(c) ? -2.0f : 2.0f);
        const float4* row = P.Wq + static_cast<long>(c) * KP * 32 + lane;
        float4 wv[KP];
#pragma unroll
        for (int kk = 0; kk < KP; kk++) wv[kk] = __ldg(row + 32 * kk);
#pragma unroll
        for (int kk = 0; kk < KP; kk++) {
            nr[kk] = fma2(ts, pk2(wv[kk].x, wv[kk].y), nr[kk]);
            ni[kk] = fma2(ts, pk2(wv[kk].z, wv[kk].w), ni[kk]);
        }
    }
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
    const LogNorm ln = log_norms_of(rr, L.N, lane);
    const float logq_rev = log_q_of(rowp, L.N, i, l, ln);
    const float log_a = __fsub_rn(__fmaf_rn(2.0f, delta, logq_rev), L.logq_fwd[w]);
    WalkerRng rng;
    rng.init(L.seed, static_cast<uint32_t>(L.walker_base + w), L.rng_index[w]);
    const float a = log_a >= 0.0f ? 1.0f : expf_det(log_a);
    bool accept = log_a >= 0.0f;
    if (!accept) accept = rng.uniform() <= a;
    if (accept) {
#pragma unroll
        for (int kk = 0; kk < KP; kk++) {
            float a0, a1, b0, b1, r0, r1;
            up2(nr[kk], a0, a1);
            up2(ni[kk], b0, b1);
            up2(nre[kk], r0, r1);
            L.theta[base + 32 * kk] = make_float4(a0, a1, b0, b1);
            L.re[base + 32 * kk] = make_float2(r0, r1);
        }
        float* cur = L.logits_cur + static_cast<long>(w) * L.O;
        for (int j = lane; j < L.O; j += 32) cur[j] = rowp[j];
    }
    Spins<NW> cur = s;
    if (accept) {
#pragma unroll
        for (int k = 0; k < NW; k++) cur.w[k] = L.spins_prop[static_cast<long>(w) * NW + k];
    }
    if (lane == 0) {
        if (accept) {
#pragma unroll
            for (int k = 0; k < NW; k++) L.spins[static_cast<long>(w) * NW + k] = cur.w[k];
            L.accepts[w] += 1;
        }
        L.reward[w] = a * static_cast<float>(l);
    }
    if (L.propose_next) {
        // the next step's move, drawn from the logits of the state the walker is now in
        // (the draws a separate proposal pass would make, in the same order)
        const float* row = accept ? rowp : L.logits_cur + static_cast<long>(w) * L.O;
        const LogNorm lnn = accept ? ln : log_norms(row, L.N, lane);
        const int i2 = draw_index(row, L.N, lnn.seed, rng.uniform(), lane);
        const int l2 = 1 + draw_index(row + L.N, kLengths, lnn.len, rng.uniform(), lane);
        if (lane == 0) {
            for (int q = 0; q < l2; q++) {
                int c = i2 + q;
                if (c >= L.N) c -= L.N;
                cur.flip(c);
            }
#pragma unroll
            for (int k = 0; k < NW; k++) L.spins_prop[static_cast<long>(w) * NW + k] = cur.w[k];
            L.site[w] = i2;
            L.len[w] = l2;
            L.logq_fwd[w] = log_q_of(row, L.N, i2, l2, lnn);
            L.proposals[w] += 1;
        }
    }
    if (lane == 0) L.rng_index[w] = rng.index;
}

__device__ __forceinline__ float log_add(float a, float b) {
    const float m = fmaxf(a, b);
    if (m == -INFINITY) return m;
    return m + logf(expf(a - m) + expf(b - m));
}

// Locally balanced target of the first n walkers (warp per walker): Re Delta(i, l) =
// Re log psi(s with {i..i+l-1} flipped) - Re log psi(s) for all N seeds and 8 lengths,
// p*(i, l) propto exp(Re Delta(i, l)); writes dl = (q - p*) / n, the gradient of the mean
// cross-entropy -sum p* log q with respect to the seed and length logits (q factorises
// into the seed and length softmaxes, whose optimum is the marginals of p*).
template <int K, int NW>
__global__ void __launch_bounds__(32 * kWarpsPerBlock) lb_target_kernel(RbmDev P, int n, const uint64_t* spins,
                                                                       const float4* theta, const float2* re_all,
                                                                       const float* logits, int O, float* dl) {
    const int lane = threadIdx.x & 31;
    const int w = blockIdx.x * kWarpsPerBlock + (threadIdx.x >> 5);
    if (w >= n) return;
    Spins<NW> s;
#pragma unroll
    for (int k = 0; k < NW; k++) s.w[k] = spins[static_cast<long>(w) * NW + k];
    constexpr int KP = (K + 1) / 2;
    const long base = static_cast<long>(w) * KP * 32 + lane;
    float tr[K], ti[K], re[K];
#pragma unroll
    for (int kk = 0; kk < KP; kk++) {
        const float4 t = theta[base + 32 * kk];
        const float2 f = re_all[base + 32 * kk];
        tr[2 * kk] = t.x;
        ti[2 * kk] = t.z;
        re[2 * kk] = f.x;
        if (2 * kk + 1 < K) {
            tr[2 * kk + 1] = t.y;
            ti[2 * kk + 1] = t.w;
            re[2 * kk + 1] = f.y;
        }
    }
    constexpr int kSlots = (64 * NW + 31) / 32;   // seeds i = lane + 32 c held by lane
    float ms[kSlots], ml[kLengths];
#pragma unroll
    for (int c = 0; c < kSlots; c++) ms[c] = -INFINITY;
#pragma unroll
    for (int q = 0; q < kLengths; q++) ml[q] = -INFINITY;
    for (int i = 0; i < P.N; i++) {
        float nr[K], ni[K];
#pragma unroll
        for (int k = 0; k < K; k++) { nr[k] = tr[k]; ni[k] = ti[k]; }
        float seed_acc = -INFINITY;
#pragma unroll
        for (int q = 0; q < kLengths; q++) {
            int c = i + q;
            if (c >= P.N) c -= P.N;
            const float two_s = s.up(c) ? -2.0f : 2.0f;
            const float2* row = P.W + static_cast<long>(c) * P.Mpad + lane;
            float part = 0.0f;
#pragma unroll
            for (int k = 0; k < K; k++) {
                const float2 wv = __ldg(row + 32 * k);
                nr[k] = __fmaf_rn(two_s, wv.x, nr[k]);
                ni[k] = __fmaf_rn(two_s, wv.y, ni[k]);
                part += lc_re(nr[k], ni[k]) - re[k];
            }
            const float d = warp_sum_xor(part);
            seed_acc = log_add(seed_acc, d);
            ml[q] = log_add(ml[q], d);
        }
        const int slot = i >> 5;
        if (lane == (i & 31)) {
#pragma unroll
            for (int c = 0; c < kSlots; c++)
                if (c == slot) ms[c] = seed_acc;
        }
    }
    float total = -INFINITY;
#pragma unroll
    for (int q = 0; q < kLengths; q++) total = log_add(total, ml[q]);
    const float* row = logits + static_cast<long>(w) * O;
    const LogNorm ln = log_norms(row, P.N, lane);
    float* out = dl + static_cast<long>(w) * O;
    const float inv = 1.0f / static_cast<float>(n);
#pragma unroll
    for (int c = 0; c < kSlots; c++) {
        const int j = lane + 32 * c;
        if (j < P.N) out[j] = (expf(row[j] - ln.seed) - expf(ms[c] - total)) * inv;
    }
#pragma unroll
    for (int q = 0; q < kLengths; q++)
        if (lane == q) out[P.N + q] = (expf(row[P.N + q] - ln.len) - expf(ml[q] - total)) * inv;
}

// mean reward of the first n walkers (one block, fixed order)
__global__ void reward_mean_kernel(const float* r, int n, float* out) {
    __shared__ float part[256];
    float s = 0.0f;
    for (int i = threadIdx.x; i < n; i += 256) s += r[i];
    part[threadIdx.x] = s;
    __syncthreads();
    for (int h = 128; h >= 1; h >>= 1) {
        if (threadIdx.x < h) part[threadIdx.x] += part[threadIdx.x + h];
        __syncthreads();
    }
    if (threadIdx.x == 0) out[0] = part[0] / static_cast<float>(n);
}

// REINFORCE gradient of the mean over n walkers of
//   -(r - rbar) log q(i, l) - beta (H_seed + H_len)
// with respect to the logits (warp per walker) -> dl [n][O]
__global__ void __launch_bounds__(32 * kWarpsPerBlock) reinforce_kernel(const float* logits, int n, int N, int O,
                                                                       const int* site, const int* len,
                                                                       const float* reward, const float* rbar,
                                                                       float* dl) {
    const int lane = threadIdx.x & 31;
    const int w = blockIdx.x * kWarpsPerBlock + (threadIdx.x >> 5);
    if (w >= n) return;
    const float* row = logits + static_cast<long>(w) * O;
    const LogNorm ln = log_norms(row, N, lane);
    const float adv = (reward[w] - rbar[0]) / static_cast<float>(n);
    const float beta = kEntropyBonus / static_cast<float>(n);
    // entropies H = -sum p log p
    float hs = 0.0f;
    for (int j = lane; j < N; j += 32) {
        const float lp = row[j] - ln.seed;
        hs -= expf(lp) * lp;
    }
    hs = warp_sum_xor(hs);
    const float lpl = lane < kLengths ? row[N + lane] - ln.len : 0.0f;
    const float hl = warp_sum_xor(lane < kLengths ? -expf(lpl) * lpl : 0.0f);
    const int i = site[w], l = len[w];
    float* out = dl + static_cast<long>(w) * O;
    for (int j = lane; j < N; j += 32) {
        const float lp = row[j] - ln.seed, p = expf(lp);
        out[j] = adv * (p - (j == i ? 1.0f : 0.0f)) + beta * p * (lp + hs);
    }
    if (lane < kLengths) {
        const float p = expf(lpl);
        out[N + lane] = adv * (p - (lane == l - 1 ? 1.0f : 0.0f)) + beta * p * (lpl + hl);
    }
}

template <int K>
cudaError_t launch_learned_k(int which, int nw, const RbmDev& P, const LearnedLaunch& L, cudaStream_t st) {
    const dim3 grid((L.B + kWarpsPerBlock - 1) / kWarpsPerBlock), block(32 * kWarpsPerBlock);
#define RBMG_LEARNED_CASE(NWV)                                                             \
    case NWV:                                                                               \
        if (which == 0) learned_angles_kernel<K, NWV><<<grid, block, 0, st>>>(P, L);        \
        else learned_accept_kernel<K, NWV><<<grid, block, 0, st>>>(P, L);                    \
        break;
    switch (nw) {
        RBMG_LEARNED_CASE(1)
        RBMG_LEARNED_CASE(2)
        RBMG_LEARNED_CASE(3)
        RBMG_LEARNED_CASE(4)
        default: return cudaErrorInvalidValue;
    }
#undef RBMG_LEARNED_CASE
    return cudaGetLastError();
}

// which: 0 angles from the spins, 1 accept / reject
cudaError_t launch_learned(int which, const RbmDev& P, const LearnedLaunch& L, cudaStream_t st) {
    const int nw = nwords_of(P.N);
    switch (P.Mpad / 32) {
        case 1: return launch_learned_k<1>(which, nw, P, L, st);
        case 2: return launch_learned_k<2>(which, nw, P, L, st);
        case 4: return launch_learned_k<4>(which, nw, P, L, st);
        case 8: return launch_learned_k<8>(which, nw, P, L, st);
        case 13: return launch_learned_k<13>(which, nw, P, L, st);
        case 18: return launch_learned_k<18>(which, nw, P, L, st);
        default: return cudaErrorInvalidValue;
    }
}

template <int K>
cudaError_t launch_lb_k(int nw, const RbmDev& P, int n, const uint64_t* spins, const float4* theta, const float2* re,
                        const float* logits, int O, float* dl, cudaStream_t st) {
    const dim3 grid((n + kWarpsPerBlock - 1) / kWarpsPerBlock), block(32 * kWarpsPerBlock);
    switch (nw) {
        case 1: lb_target_kernel<K, 1><<<grid, block, 0, st>>>(P, n, spins, theta, re, logits, O, dl); break;
        case 2: lb_target_kernel<K, 2><<<grid, block, 0, st>>>(P, n, spins, theta, re, logits, O, dl); break;
        case 3: lb_target_kernel<K, 3><<<grid, block, 0, st>>>(P, n, spins, theta, re, logits, O, dl); break;
        case 4: lb_target_kernel<K, 4><<<grid, block, 0, st>>>(P, n, spins, theta, re, logits, O, dl); break;
        default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

cudaError_t launch_lb_target(const RbmDev& P, int n, const uint64_t* spins, const float4* theta, const float2* re,
                             const float* logits, int O, float* dl, cudaStream_t st) {
    const int nw = nwords_of(P.N);
    switch (P.Mpad / 32) {
        case 1: return launch_lb_k<1>(nw, P, n, spins, theta, re, logits, O, dl, st);
        case 2: return launch_lb_k<2>(nw, P, n, spins, theta, re, logits, O, dl, st);
        case 4: return launch_lb_k<4>(nw, P, n, spins, theta, re, logits, O, dl, st);
        case 8: return launch_lb_k<8>(nw, P, n, spins, theta, re, logits, O, dl, st);
        case 13: return launch_lb_k<13>(nw, P, n, spins, theta, re, logits, O, dl, st);
        case 18: return launch_lb_k<18>(nw, P, n, spins, theta, re, logits, O, dl, st);
        default: return cudaErrorInvalidValue;
    }
}

// tensor-core (tcgen05) inference, mlp_tc.cu
struct TcNet {
    int N, O, ldw1;
    const bf16* w1t;
    const bf16* w2t;
    const bf16* w3t;
    const float* b1;
    const float* b2;
    const float* b3;
    const bf16* pack;
};
size_t tc_pack_size(int ldw1);
cudaError_t launch_tc_pack(const TcNet& net, bf16* pack, cudaStream_t st);
// the tensor-core kernel's packed B operands from the transposed BF16 copies
cudaError_t proposal_refresh_tc(rbmg_proposal* p, cudaStream_t st) {
    if (p->O > 128) return cudaSuccess;
    const TcNet tn{p->N, p->O, p->ldw1, p->w1t.as<bf16>(), p->w2t.as<bf16>(), p->w3t.as<bf16>(), nullptr, nullptr,
                   nullptr, nullptr};
    return launch_tc_pack(tn, p->tcpack.as<bf16>(), st);
}

cudaError_t launch_mlp_tc(const TcNet& net, int nw, const uint64_t* spins, int count, float* out, int* error,
                          cudaStream_t st);

// ============================================================================ fused inference
// One CTA runs the whole network for 128 configurations with the activations in shared
// memory: x [128][<=256] -> h1 -> h2 -> logits.  The weights stream through a 4-stage
// cp.async pipeline in chunks of 32 input features; the MMA fragments come from shared
// memory by ldmatrix.  The k order, tile arithmetic and epilogues are those of the
// layer-by-layer GEMM path, so the logits agree bit for bit.  With PROPOSE the CTA first
// draws the walkers' moves from their current logits and evaluates the network on the
// proposed configurations.
constexpr int kFRows = 128;                  // configurations per CTA
constexpr int kFThreads = 512;               // 16 warps: 4 (rows) x 4 (columns)
constexpr int kFStages = 4;
constexpr int kFLd = kHidden + 8;            // activation row stride (bf16): 528 bytes
constexpr int kFWLd = 40;                    // weight-chunk row stride (bf16): 80 bytes
constexpr size_t kFSmem = 2 * sizeof(bf16) * kFRows * kFLd + kFStages * sizeof(bf16) * kHidden * kFWLd;

struct FusedNet {
    int N, O, ldw1;
    const bf16* w1t;   // [256][ldw1]
    const bf16* w2t;   // [256][256]
    const bf16* w3t;   // [passes * 128][256]
    const float* b1;
    const float* b2;
    const float* b3;
};

__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
    const unsigned sa = static_cast<unsigned>(__cvta_generic_to_shared(smem));
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(sa), "l"(gmem));
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::); }
template <int NPEND>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(NPEND)); }

// four 8x8 b16 matrices; lanes 8q..8q+7 address the rows of matrix q
__device__ __forceinline__ void ldsm_x4(uint32_t (&r)[4], const bf16* p) {
    const unsigned a = static_cast<unsigned>(__cvta_generic_to_shared(p));
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
                 : "r"(a));
}

// acc = A [128][k] (shared, stride kFLd) x Wt^T, Wt [NT*32][ldw] (global, k contiguous);
// warp (wm, wn) computes rows wm*32 .. +32 and columns wn*NT*8 .. +NT*8
template <int NT>
__device__ __forceinline__ void fused_layer(const bf16* sA, int kchunks, const bf16* Wt, int ldw, bf16* sW,
                                            float (&acc)[2][NT][4]) {
    static_assert(NT % 2 == 0, "B fragments are loaded two n8 tiles at a time");
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int wm = warp & 3, wn = warp >> 2;
    constexpr int kOut = NT * 32;
#pragma unroll
    for (int i = 0; i < 2; i++)
#pragma unroll
        for (int j = 0; j < NT; j++)
#pragma unroll
            for (int e = 0; e < 4; e++) acc[i][j][e] = 0.0f;
    auto issue = [&](int kc, int stage) {
        bf16* dst = sW + stage * (kHidden * kFWLd);
        for (int c = tid; c < kOut * 4; c += kFThreads) {
            const int n = c >> 2, q = (c & 3) * 8;
            cp_async16(dst + n * kFWLd + q, Wt + static_cast<long>(n) * ldw + kc * 32 + q);
        }
        cp_async_commit();
    };
#pragma unroll
    for (int st = 0; st < kFStages - 1; st++) {
        if (st < kchunks) issue(st, st);
        else cp_async_commit();
    }
    // ldmatrix row addresses of this lane: A rows (lane & 15), column half (lane >> 4);
    // B rows (lane & 7) + 8 (lane >> 4), column half (lane >> 3) & 1
    const int a_row = wm * 32 + (lane & 15), a_col = (lane >> 4) * 8;
    const int b_row = wn * NT * 8 + (lane & 7) + ((lane >> 4) << 3), b_col = ((lane >> 3) & 1) * 8;
    for (int kc = 0; kc < kchunks; kc++) {
        cp_async_wait<kFStages - 2>();
        __syncthreads();
        const int nk = kc + kFStages - 1;
        if (nk < kchunks) issue(nk, nk % kFStages);
        else cp_async_commit();
        const bf16* w = sW + (kc % kFStages) * (kHidden * kFWLd);
#pragma unroll
        for (int ks = 0; ks < 32; ks += 16) {
            uint32_t af[2][4], bfr[NT][2];
#pragma unroll
            for (int mi = 0; mi < 2; mi++) ldsm_x4(af[mi], sA + (a_row + mi * 16) * kFLd + kc * 32 + ks + a_col);
#pragma unroll
            for (int ni = 0; ni < NT; ni += 2) {
                uint32_t r[4];
                ldsm_x4(r, w + (b_row + ni * 8) * kFWLd + ks + b_col);
                bfr[ni][0] = r[0];
                bfr[ni][1] = r[1];
                bfr[ni + 1][0] = r[2];
                bfr[ni + 1][1] = r[3];
            }
#pragma unroll
            for (int mi = 0; mi < 2; mi++)
#pragma unroll
                for (int ni = 0; ni < NT; ni++) mma_bf16_16816(acc[mi][ni], af[mi], bfr[ni]);
        }
    }
    cp_async_wait<0>();
    __syncthreads();   // every warp is done with the stages before they are refilled
}

// h = bf16(silu(acc + b)) into dst [128][kFLd]; the thread's 16 bias values are loaded once
__device__ __forceinline__ void fused_silu_store(const float (&acc)[2][8][4], const float* b, bf16* dst) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int wm = warp & 3, wn = warp >> 2, gq = lane >> 2, tq = lane & 3;
    float bias[8][2];
#pragma unroll
    for (int ni = 0; ni < 8; ni++) {
        const float2 v = *reinterpret_cast<const float2*>(b + wn * 64 + ni * 8 + 2 * tq);
        bias[ni][0] = v.x;
        bias[ni][1] = v.y;
    }
#pragma unroll
    for (int mi = 0; mi < 2; mi++)
#pragma unroll
        for (int ni = 0; ni < 8; ni++)
#pragma unroll
            for (int h = 0; h < 2; h++) {
                const int r = wm * 32 + mi * 16 + gq + 8 * h, n = wn * 64 + ni * 8 + 2 * tq;
                __nv_bfloat162 v;
                v.x = __float2bfloat16_rn(silu_f(acc[mi][ni][h * 2] + bias[ni][0]));
                v.y = __float2bfloat16_rn(silu_f(acc[mi][ni][h * 2 + 1] + bias[ni][1]));
                *reinterpret_cast<__nv_bfloat162*>(dst + r * kFLd + n) = v;
            }
}

template <int NW, bool PROPOSE>
__global__ void __launch_bounds__(kFThreads, 1) mlp_fused_kernel(FusedNet net, LearnedLaunch L,
                                                                 const uint64_t* in_spins, int count,
                                                                 float* logits_out) {
    extern __shared__ __align__(16) unsigned char fsm[];
    bf16* sX = reinterpret_cast<bf16*>(fsm);
    bf16* sH = sX + kFRows * kFLd;
    bf16* sW = sH + kFRows * kFLd;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int row0 = blockIdx.x * kFRows;
    // ---- the input configurations (proposed moves with PROPOSE), one warp per row
    for (int r = warp; r < kFRows; r += kFThreads / 32) {
        const int w = row0 + r;
        Spins<NW> s;
#pragma unroll
        for (int k = 0; k < NW; k++) s.w[k] = 0;
        if (w < count) {
            if (PROPOSE) {
                WalkerRng rng;
                rng.init(L.seed, static_cast<uint32_t>(L.walker_base + w), L.rng_index[w]);
                const float* row = L.logits_cur + static_cast<long>(w) * L.O;
                const LogNorm ln = log_norms(row, L.N, lane);
                const int i = draw_index(row, L.N, ln.seed, rng.uniform(), lane);
                const int l = 1 + draw_index(row + L.N, kLengths, ln.len, rng.uniform(), lane);
#pragma unroll
                for (int k = 0; k < NW; k++) s.w[k] = L.spins[static_cast<long>(w) * NW + k];
                if (lane == 0 && L.spins_pre) {
#pragma unroll
                    for (int k = 0; k < NW; k++) L.spins_pre[static_cast<long>(w) * NW + k] = s.w[k];
                }
                for (int q = 0; q < l; q++) {
                    int c = i + q;
                    if (c >= L.N) c -= L.N;
                    s.flip(c);
                }
                if (lane == 0) {
#pragma unroll
                    for (int k = 0; k < NW; k++) L.spins_prop[static_cast<long>(w) * NW + k] = s.w[k];
                    L.site[w] = i;
                    L.len[w] = l;
                    L.logq_fwd[w] = log_q_of(row, L.N, i, l, ln);
                    L.rng_index[w] = rng.index;
                    L.proposals[w] += 1;
                }
            } else {
#pragma unroll
                for (int k = 0; k < NW; k++) s.w[k] = in_spins[static_cast<long>(w) * NW + k];
            }
        }
        for (int i = lane; i < net.ldw1; i += 32) {
            const float v = (w < count && i < net.N) ? (s.up(i) ? 1.0f : -1.0f) : 0.0f;
            sX[r * kFLd + i] = __float2bfloat16_rn(v);
        }
    }
    __syncthreads();
    {
        float acc[2][8][4];
        fused_layer<8>(sX, net.ldw1 / 32, net.w1t, net.ldw1, sW, acc);
        fused_silu_store(acc, net.b1, sH);
        __syncthreads();
        fused_layer<8>(sH, kHidden / 32, net.w2t, kHidden, sW, acc);
        fused_silu_store(acc, net.b2, sX);
        __syncthreads();
    }
    const int wm = warp & 3, wn = warp >> 2, gq = lane >> 2, tq = lane & 3;
    for (int pass = 0; pass * 128 < net.O; pass++) {
        float acc[2][4][4];
        fused_layer<4>(sX, kHidden / 32, net.w3t + static_cast<long>(pass) * 128 * kHidden, kHidden, sW, acc);
#pragma unroll
        for (int mi = 0; mi < 2; mi++)
#pragma unroll
            for (int ni = 0; ni < 4; ni++)
#pragma unroll
                for (int h = 0; h < 2; h++)
#pragma unroll
                    for (int e = 0; e < 2; e++) {
                        const int r = wm * 32 + mi * 16 + gq + 8 * h;
                        const int n = pass * 128 + wn * 32 + ni * 8 + 2 * tq + e;
                        if (row0 + r < count && n < net.O)
                            logits_out[static_cast<long>(row0 + r) * net.O + n] = acc[mi][ni][h * 2 + e] + net.b3[n];
                    }
    }
}

FusedNet fused_net(const rbmg_proposal* p) {
    const float* w = p->master.as<float>();
    return FusedNet{p->N, p->O, p->ldw1, p->w1t.as<bf16>(), p->w2t.as<bf16>(), p->w3t.as<bf16>(),
                    w + p->ob1, w + p->ob2, w + p->ob3};
}

template <int NW, bool PROPOSE>
cudaError_t launch_fused_nw(const FusedNet& net, const LearnedLaunch& L, const uint64_t* in, int count, float* out,
                            cudaStream_t st) {
    // the attribute belongs to the current device's context: set it on every launch
    const cudaError_t e = cudaFuncSetAttribute(mlp_fused_kernel<NW, PROPOSE>,
                                               cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(kFSmem));
    if (e != cudaSuccess) return e;
    mlp_fused_kernel<NW, PROPOSE><<<(count + kFRows - 1) / kFRows, kFThreads, kFSmem, st>>>(net, L, in, count, out);
    return cudaGetLastError();
}

// logits of `count` configurations (PROPOSE = false: in_spins) or of the walkers' proposed
// moves (PROPOSE = true: drawn from L.logits_cur, written to L's move buffers)
template <bool PROPOSE>
cudaError_t launch_fused(const rbmg_proposal* p, const LearnedLaunch& L, const uint64_t* in, int count, float* out,
                         cudaStream_t st) {
    if (count <= 0) return cudaSuccess;
    const FusedNet net = fused_net(p);
    if (!PROPOSE && p->O <= 128) {
        // tcgen05 / TMEM path (one output pass of 128): every logits row of the chain comes from it
        const TcNet tn{net.N, net.O, net.ldw1, net.w1t, net.w2t, net.w3t, net.b1, net.b2, net.b3, p->tcpack.as<bf16>()};
        return launch_mlp_tc(tn, nwords_of(p->N), in, count, out, p->tc_error.as<int>(), st);
    }
    switch (nwords_of(p->N)) {
        case 1: return launch_fused_nw<1, PROPOSE>(net, L, in, count, out, st);
        case 2: return launch_fused_nw<2, PROPOSE>(net, L, in, count, out, st);
        case 3: return launch_fused_nw<3, PROPOSE>(net, L, in, count, out, st);
        case 4: return launch_fused_nw<4, PROPOSE>(net, L, in, count, out, st);
        default: return cudaErrorInvalidValue;
    }
}

// per-chain buffers of the learned steps
// chains of at least 8192 walkers run their frozen steps as 2 slices on 2 streams (4 slices
// measured no faster at 16384 walkers: the network pass is latency-bound inside a CTA)
constexpr int kSplitWalkers = 8192;
constexpr int kMaxSlices = 4;

struct LearnedState {
    int B = 0, Mpad = 0, nw = 0, O = 0;
    DevBuf theta, re, spins_prop, spins_pre, site, len, logq, logits_cur, logits_prop, reward, rbar;
    // extra streams of the frozen steps: slices of the walkers run as independent chains,
    // so that one slice's network pass overlaps another slice's accept pass
    cudaStream_t side[kMaxSlices - 1] = {};
    cudaEvent_t fork = nullptr, join[kMaxSlices - 1] = {};
    LearnedState() = default;
    LearnedState(const LearnedState&) = delete;
    LearnedState& operator=(const LearnedState&) = delete;
    ~LearnedState() {
        if (fork) cudaEventDestroy(fork);
        for (int i = 0; i < kMaxSlices - 1; i++) {
            if (join[i]) cudaEventDestroy(join[i]);
            if (side[i]) cudaStreamDestroy(side[i]);
        }
    }
};

// walkers [base, base + count) of a chain as a chain of their own (same Philox streams)
LearnedLaunch learned_slice(const LearnedLaunch& L, int base, int count, int nw, int Mpad) {
    LearnedLaunch h = L;
    const size_t b = static_cast<size_t>(base);
    h.B = count;
    h.walker_base = L.walker_base + base;
    h.spins = L.spins + b * nw;
    h.rng_index = L.rng_index + b;
    h.spins_prop = L.spins_prop + b * nw;
    h.spins_pre = L.spins_pre ? L.spins_pre + b * nw : nullptr;
    h.site = L.site + b;
    h.len = L.len + b;
    h.logq_fwd = L.logq_fwd + b;
    h.logits_cur = L.logits_cur + b * L.O;
    h.logits_prop = L.logits_prop + b * L.O;
    const size_t per = static_cast<size_t>((Mpad / 32 + 1) / 2) * 32;   // KP * 32 entries per walker
    h.theta = L.theta + b * per;
    h.re = L.re + b * per;
    h.reward = L.reward + b;
    h.accepts = L.accepts + b;
    h.proposals = L.proposals + b;
    return h;
}

}  // namespace rbmg

using namespace rbmg;

// ============================================================================ C ABI
extern "C" int rbmg_proposal_create(int N, uint64_t seed, float lr, rbmg_proposal** out) {
    if (!out) return fail(RBMG_EINVAL, "proposal: null output");
    if (N <= kLengths || N > 64 * kMaxWords)
        return fail(RBMG_EINVAL, "proposal: N must be in 9..256 (clusters of up to 8 sites must not wrap onto themselves)");
    if (!(lr > 0.0f) || !std::isfinite(lr)) return fail(RBMG_EINVAL, "proposal: learning rate must be positive");
    auto p = std::make_unique<rbmg_proposal>();
    p->N = N;
    p->O = N + kLengths;
    p->Np = pad8(N);
    p->Op = pad8(p->O);
    p->lr = lr;
    const int H = kHidden;
    p->oW1 = 0;
    p->ob1 = p->oW1 + static_cast<size_t>(N) * H;
    p->oW2 = p->ob1 + H;
    p->ob2 = p->oW2 + static_cast<size_t>(H) * H;
    p->oW3 = p->ob2 + H;
    p->ob3 = p->oW3 + static_cast<size_t>(H) * p->O;
    p->P = static_cast<int64_t>(p->ob3 + p->O);
    // He-uniform hidden layers (splitmix64 stream of the seed); zero output layer, so
    // the untrained proposal is uniform over seeds and lengths
    std::vector<float> h(static_cast<size_t>(p->P), 0.0f);
    uint64_t z = seed;
    auto uni = [&z]() {
        z += 0x9E3779B97F4A7C15ull;
        uint64_t x = z;
        x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
        x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
        x ^= x >> 31;
        return static_cast<double>(x >> 11) * (1.0 / 9007199254740992.0);
    };
    const double a1 = std::sqrt(6.0 / N), a2 = std::sqrt(6.0 / H);
    for (size_t t = 0; t < static_cast<size_t>(N) * H; t++) h[p->oW1 + t] = static_cast<float>(a1 * (2.0 * uni() - 1.0));
    for (size_t t = 0; t < static_cast<size_t>(H) * H; t++) h[p->oW2 + t] = static_cast<float>(a2 * (2.0 * uni() - 1.0));
    RBMG_CK(p->master.ensure(sizeof(float) * p->P));
    RBMG_CK(p->adam_m.ensure(sizeof(float) * p->P));
    RBMG_CK(p->adam_v.ensure(sizeof(float) * p->P));
    RBMG_CK(p->grad.ensure(sizeof(float) * p->P));
    RBMG_CK(p->w1.ensure(sizeof(bf16) * static_cast<size_t>(N) * H));
    RBMG_CK(p->w2.ensure(sizeof(bf16) * static_cast<size_t>(H) * H));
    RBMG_CK(p->w3.ensure(sizeof(bf16) * static_cast<size_t>(H) * p->Op));
    p->ldw1 = (N + 31) / 32 * 32;
    p->w3_rows = (p->O + 127) / 128 * 128;
    RBMG_CK(p->w1t.ensure(sizeof(bf16) * static_cast<size_t>(H) * p->ldw1));
    RBMG_CK(p->w2t.ensure(sizeof(bf16) * static_cast<size_t>(H) * H));
    RBMG_CK(p->w3t.ensure(sizeof(bf16) * static_cast<size_t>(p->w3_rows) * H));
    if (p->O <= 128) RBMG_CK(p->tcpack.ensure(sizeof(bf16) * tc_pack_size(p->ldw1)));
    RBMG_CK(p->tc_error.ensure(sizeof(int)));
    RBMG_CK(cudaMemset(p->tc_error.p, 0, sizeof(int)));
    RBMG_CK(cudaMemcpy(p->master.p, h.data(), sizeof(float) * p->P, cudaMemcpyHostToDevice));
    RBMG_CK(cudaMemset(p->adam_m.p, 0, sizeof(float) * p->P));
    RBMG_CK(cudaMemset(p->adam_v.p, 0, sizeof(float) * p->P));
    RBMG_CK(cudaMemset(p->grad.p, 0, sizeof(float) * p->P));
    RBMG_CK(proposal_refresh_bf16(p.get(), stream()));
    RBMG_CK(cudaStreamSynchronize(stream()));
    *out = p.release();
    return RBMG_OK;
}

extern "C" int rbmg_proposal_destroy(rbmg_proposal* p) {
    delete p;
    return RBMG_OK;
}

extern "C" int rbmg_proposal_num_params(const rbmg_proposal* p, int64_t* n) {
    if (!p || !n) return fail(RBMG_EINVAL, "proposal: null argument");
    *n = p->P;
    return RBMG_OK;
}

extern "C" int rbmg_proposal_get_params(const rbmg_proposal* p, float* params) {
    if (!p || !params) return fail(RBMG_EINVAL, "proposal: null argument");
    RBMG_CK(cudaStreamSynchronize(stream()));
    RBMG_CK(cudaMemcpy(params, p->master.p, sizeof(float) * p->P, cudaMemcpyDeviceToHost));
    return RBMG_OK;
}

extern "C" int rbmg_proposal_set_params(rbmg_proposal* p, const float* params) {
    if (!p || !params) return fail(RBMG_EINVAL, "proposal: null argument");
    for (int64_t t = 0; t < p->P; t++)
        if (!std::isfinite(params[t])) return fail(RBMG_ENAN, "proposal: non-finite parameter");
    RBMG_CK(cudaStreamSynchronize(stream()));
    RBMG_CK(cudaMemcpy(p->master.p, params, sizeof(float) * p->P, cudaMemcpyHostToDevice));
    RBMG_CK(proposal_refresh_bf16(p, stream()));
    RBMG_CK(cudaStreamSynchronize(stream()));
    return RBMG_OK;
}

extern "C" int rbmg_proposal_status(rbmg_proposal* p) {
    if (!p) return fail(RBMG_EINVAL, "proposal status: null");
    int err = 0;
    RBMG_CK(cudaDeviceSynchronize());
    RBMG_CK(cudaMemcpy(&err, p->tc_error.p, sizeof(int), cudaMemcpyDeviceToHost));
    if (err) {
        RBMG_CK(cudaMemset(p->tc_error.p, 0, sizeof(int)));
        return fail(RBMG_ETIMEOUT, "proposal: a tensor-core pass gave up waiting for its MMAs");
    }
    return RBMG_OK;
}

extern "C" int rbmg_proposal_eval(rbmg_proposal* p, int count, const uint64_t* spins, const float* dlogits,
                                  float* logits, float* grads) {
    if (!p || count <= 0 || !spins || !logits) return fail(RBMG_EINVAL, "proposal eval: bad arguments");
    if (dlogits && !grads) return fail(RBMG_EINVAL, "proposal eval: dlogits needs a gradient output");
    const int nw = nwords_of(p->N);
    cudaStream_t st = stream();
    DevBuf dsp, dlog;
    RBMG_CK(dsp.ensure(sizeof(uint64_t) * nw * count));
    RBMG_CK(dlog.ensure(sizeof(float) * static_cast<size_t>(count) * p->O));
    RBMG_CK(cudaMemcpyAsync(dsp.p, spins, sizeof(uint64_t) * nw * count, cudaMemcpyHostToDevice, st));
    int r = RBMG_OK;
    if (dlogits) {
        r = proposal_forward(p, count, dsp.as<uint64_t>(), dlog.as<float>(), st);
        if (r != RBMG_OK) return r;
    } else {
        RBMG_CK(launch_fused<false>(p, LearnedLaunch{}, dsp.as<uint64_t>(), count, dlog.as<float>(), st));
    }
    r = rbmg_proposal_status(p);
    if (r != RBMG_OK) return r;
    RBMG_CK(cudaMemcpyAsync(logits, dlog.p, sizeof(float) * count * p->O, cudaMemcpyDeviceToHost, st));
    if (dlogits) {
        RBMG_CK(cudaMemcpyAsync(p->dl32.p, dlogits, sizeof(float) * count * p->O, cudaMemcpyHostToDevice, st));
        r = proposal_backward(p, count, st);
        if (r != RBMG_OK) return r;
        RBMG_CK(cudaMemcpyAsync(grads, p->grad.p, sizeof(float) * p->P, cudaMemcpyDeviceToHost, st));
    }
    RBMG_CK(cudaStreamSynchronize(st));
    return RBMG_OK;
}

extern "C" int rbmg_proposal_adam(rbmg_proposal* p, const float* grads) {
    if (!p || !grads) return fail(RBMG_EINVAL, "proposal adam: null argument");
    cudaStream_t st = stream();
    RBMG_CK(cudaMemcpyAsync(p->grad.p, grads, sizeof(float) * p->P, cudaMemcpyHostToDevice, st));
    const int r = proposal_adam(p, st);
    if (r != RBMG_OK) return r;
    RBMG_CK(cudaStreamSynchronize(st));
    return RBMG_OK;
}

// training state: FP32 parameters, Adam moments (each [num_params]) and the Adam step count
extern "C" int rbmg_proposal_get_state(const rbmg_proposal* p, float* params, float* m, float* v, int64_t* steps) {
    if (!p || !params || !m || !v || !steps) return fail(RBMG_EINVAL, "proposal state: null");
    RBMG_CK(cudaDeviceSynchronize());
    RBMG_CK(cudaMemcpy(params, p->master.p, sizeof(float) * p->P, cudaMemcpyDeviceToHost));
    RBMG_CK(cudaMemcpy(m, p->adam_m.p, sizeof(float) * p->P, cudaMemcpyDeviceToHost));
    RBMG_CK(cudaMemcpy(v, p->adam_v.p, sizeof(float) * p->P, cudaMemcpyDeviceToHost));
    *steps = p->steps;
    return RBMG_OK;
}

extern "C" int rbmg_proposal_set_state(rbmg_proposal* p, const float* params, const float* m, const float* v,
                                       int64_t steps) {
    if (!p || !params || !m || !v || steps < 0) return fail(RBMG_EINVAL, "proposal state: bad arguments");
    for (int64_t t = 0; t < p->P; t++)
        if (!std::isfinite(params[t]) || !std::isfinite(m[t]) || !(v[t] >= 0.0f))
            return fail(RBMG_ENAN, "proposal state: non-finite entry or negative second moment");
    RBMG_CK(cudaDeviceSynchronize());
    RBMG_CK(cudaMemcpy(p->master.p, params, sizeof(float) * p->P, cudaMemcpyHostToDevice));
    RBMG_CK(cudaMemcpy(p->adam_m.p, m, sizeof(float) * p->P, cudaMemcpyHostToDevice));
    RBMG_CK(cudaMemcpy(p->adam_v.p, v, sizeof(float) * p->P, cudaMemcpyHostToDevice));
    p->steps = steps;
    RBMG_CK(proposal_refresh_bf16(p, stream()));
    RBMG_CK(cudaStreamSynchronize(stream()));
    return RBMG_OK;
}

extern "C" int rbmg_proposal_set_objective(rbmg_proposal* p, int objective) {
    if (!p) return fail(RBMG_EINVAL, "proposal: null");
    if (objective != RBMG_PROPOSAL_LOCALLY_BALANCED && objective != RBMG_PROPOSAL_REINFORCE)
        return fail(RBMG_EINVAL, "proposal: unknown objective");
    p->objective = objective;
    return RBMG_OK;
}

extern "C" int rbmg_chain_set_learned_streams(rbmg_chain* c, int streams) {
    if (!c || streams < 0 || streams > kMaxSlices)
        return fail(RBMG_EINVAL, "learned streams: 0 (automatic) or 1 to 4");
    c->learned_streams = streams;
    return RBMG_OK;
}

// The chain's learned-step buffers (allocated on first use or when the shapes change), the
// launch record of its walkers, and the angles and logits of the current states: plain
// sweeps or new weights may have changed them since the last call.
static int learned_prepare(rbmg_chain* c, const rbmg_psi* psi, rbmg_proposal* prop, int train, cudaStream_t st,
                           LearnedState** state, LearnedLaunch& L) {
    const RbmDev P = psi->rbm_dev();
    const int B = static_cast<int>(c->walkers);
    if (!c->initialised) {
        // random start spins from the walkers' Philox streams (no sweep)
        McLaunch M{};
        M.B = B;
        M.seed = c->seed;
        M.spins = c->spins.as<uint64_t>();
        M.rng_index = c->rng_index.as<uint64_t>();
        M.init = 1;
        M.sweeps_per_sample = 1;
        M.accepts = c->accepts.as<unsigned long long>();
        M.proposals = c->proposals.as<unsigned long long>();
        RBMG_CK(launch_rbm_mc(P, nullptr, M, st));
        c->initialised = true;
    }
    auto* S = static_cast<LearnedState*>(c->learned.get());
    if (!S || S->Mpad != P.Mpad || S->O != prop->O) {
        c->learned = std::make_shared<LearnedState>();
        S = static_cast<LearnedState*>(c->learned.get());
        S->B = B;
        S->Mpad = P.Mpad;
        S->nw = c->nw;
        S->O = prop->O;
        const size_t b = static_cast<size_t>(B);
        const size_t per = static_cast<size_t>((P.Mpad / 32 + 1) / 2) * 32;
        RBMG_CK(S->theta.ensure(sizeof(float4) * b * per));
        RBMG_CK(S->re.ensure(sizeof(float2) * b * per));
        RBMG_CK(S->spins_prop.ensure(sizeof(uint64_t) * b * c->nw));
        RBMG_CK(S->spins_pre.ensure(sizeof(uint64_t) * b * c->nw));
        RBMG_CK(S->site.ensure(sizeof(int) * b));
        RBMG_CK(S->len.ensure(sizeof(int) * b));
        RBMG_CK(S->logq.ensure(sizeof(float) * b));
        RBMG_CK(S->logits_cur.ensure(sizeof(float) * b * prop->O));
        RBMG_CK(S->logits_prop.ensure(sizeof(float) * b * prop->O));
        RBMG_CK(S->reward.ensure(sizeof(float) * b));
        RBMG_CK(S->rbar.ensure(sizeof(float)));
    }
    L.B = B;
    L.N = c->N;
    L.O = prop->O;
    L.seed = c->seed;
    L.spins = c->spins.as<uint64_t>();
    L.rng_index = c->rng_index.as<uint64_t>();
    L.spins_prop = S->spins_prop.as<uint64_t>();
    L.spins_pre = train > 0 && prop->objective == RBMG_PROPOSAL_REINFORCE ? S->spins_pre.as<uint64_t>() : nullptr;
    L.site = S->site.as<int>();
    L.len = S->len.as<int>();
    L.logq_fwd = S->logq.as<float>();
    L.logits_cur = S->logits_cur.as<float>();
    L.logits_prop = S->logits_prop.as<float>();
    L.theta = S->theta.as<float4>();
    L.re = S->re.as<float2>();
    L.reward = S->reward.as<float>();
    L.accepts = c->accepts.as<unsigned long long>();
    L.proposals = c->proposals.as<unsigned long long>();
    // the angles and logits of the current states (plain sweeps or new weights may
    // have changed them since the last call); the angles from scratch on the tensor cores
    // where the psi carries their operands (its waits report through the proposal's flag)
    if (psi->dWtc.p) {
        RBMG_CK(launch_angles_tc(B, psi->N, psi->Mpad, L.spins, psi->db.as<float2>(), psi->dWtc.as<__nv_bfloat16>(),
                                 L.theta, L.re, nullptr, prop->tc_error.as<int>(), st));
    } else {
        RBMG_CK(launch_learned(0, P, L, st));
    }
    RBMG_CK(launch_fused<false>(prop, L, L.spins, B, L.logits_cur, st));
    *state = S;
    return RBMG_OK;
}

extern "C" int rbmg_chain_learned_async(rbmg_chain* c, const rbmg_psi* psi, const rbmg_operator* op,
                                        rbmg_proposal* prop, int n_steps, int train, int measure_every,
                                        void* d_eloc_out, void* stream_ptr) {
    if (!c || !psi || !prop || n_steps < 0 || train < 0) return fail(RBMG_EINVAL, "learned steps: bad arguments");
    if (psi->kind != 0 || psi->N != c->N) return fail(RBMG_EINVAL, "learned steps: psi does not match the chain");
    if (prop->N != c->N) return fail(RBMG_EINVAL, "learned steps: proposal does not match the chain");
    if (d_eloc_out && (!op || measure_every <= 0)) return fail(RBMG_EINVAL, "learned steps: measurement needs op");
    if (op && op->max_site >= psi->N) return fail(RBMG_EINVAL, "learned steps: operator acts on a site >= N");
    if (n_steps == 0) return RBMG_OK;
    cudaStream_t st = stream_ptr ? static_cast<cudaStream_t>(stream_ptr) : stream();
    const RbmDev P = psi->rbm_dev();
    const int B = static_cast<int>(c->walkers);
    LearnedState* S = nullptr;
    LearnedLaunch L{};
    int r = learned_prepare(c, psi, prop, train, st, &S, L);
    if (r != RBMG_OK) return r;
    const int nt = std::min(train, B);
    OpDev od;
    if (op) od = op->dev();
    double2* out = static_cast<double2*>(d_eloc_out);
    const int lead = d_eloc_out ? n_steps % measure_every : n_steps;
    auto measure = [&](int step, cudaStream_t s) -> cudaError_t {
        EstLaunch E{};
        E.count = B;
        E.spins = L.spins;
        E.flags = EST_ELOC;
        E.eloc = out + static_cast<size_t>((step - lead) / measure_every) * B;
        return launch_rbm_estimate(P, &od, nullptr, E, s);
    };
    auto measured = [&](int step) { return d_eloc_out && step >= lead && (step - lead + 1) % measure_every == 0; };
    int slices = c->learned_streams;
    if (slices == 0) slices = B >= kSplitWalkers ? 2 : 1;
    if (nt == 0 && slices > 1 && B >= 128 * slices) {
        // frozen network, many walkers: slices as independent chains on their own streams
        // (every walker keeps its own Philox stream and arithmetic, so the chains are the
        // ones a single pass would produce)
        if (!S->fork) RBMG_CK(cudaEventCreateWithFlags(&S->fork, cudaEventDisableTiming));
        for (int q = 0; q < slices - 1; q++) {
            if (!S->side[q]) {
                RBMG_CK(cudaStreamCreateWithFlags(&S->side[q], cudaStreamNonBlocking));
                RBMG_CK(cudaEventCreateWithFlags(&S->join[q], cudaEventDisableTiming));
            }
        }
        // slice boundaries at multiples of 128 walkers (whole tensor-core tiles)
        LearnedLaunch Lh[kMaxSlices];
        cudaStream_t sh[kMaxSlices];
        int base = 0;
        for (int q = 0; q < slices; q++) {
            const int end = q + 1 == slices ? B : (B * (q + 1) / slices) / 128 * 128;
            Lh[q] = learned_slice(L, base, end - base, c->nw, P.Mpad);
            sh[q] = q == 0 ? st : S->side[q - 1];
            base = end;
        }
        auto fork_all = [&]() -> cudaError_t {
            cudaError_t e = cudaEventRecord(S->fork, st);
            for (int q = 1; q < slices && e == cudaSuccess; q++) e = cudaStreamWaitEvent(sh[q], S->fork, 0);
            return e;
        };
        auto join_all = [&]() -> cudaError_t {
            cudaError_t e = cudaSuccess;
            for (int q = 1; q < slices && e == cudaSuccess; q++) {
                e = cudaEventRecord(S->join[q - 1], sh[q]);
                if (e == cudaSuccess) e = cudaStreamWaitEvent(st, S->join[q - 1], 0);
            }
            return e;
        };
        RBMG_CK(fork_all());
        for (int step = 0; step < n_steps; step++) {
            for (int h = 0; h < slices; h++) {
                LearnedLaunch& Q = Lh[h];
                if (step > 0) {
                    RBMG_CK(launch_fused<false>(prop, Q, Q.spins_prop, Q.B, const_cast<float*>(Q.logits_prop), sh[h]));
                } else if (prop->O <= 128) {
                    RBMG_CK(launch_draw(Q, sh[h]));
                    RBMG_CK(launch_fused<false>(prop, Q, Q.spins_prop, Q.B, const_cast<float*>(Q.logits_prop), sh[h]));
                } else {
                    RBMG_CK(launch_fused<true>(prop, Q, nullptr, Q.B, const_cast<float*>(Q.logits_prop), sh[h]));
                }
                Q.propose_next = step + 1 < n_steps ? 1 : 0;
                RBMG_CK(launch_learned(1, P, Q, sh[h]));
            }
            if (measured(step)) {
                RBMG_CK(join_all());
                RBMG_CK(measure(step, st));
                RBMG_CK(fork_all());
            }
        }
        RBMG_CK(join_all());
        return RBMG_OK;
    }
    for (int step = 0; step < n_steps; step++) {
        // frozen network: the accept kernel draws the next move, so the later steps only
        // evaluate the network on the proposed configurations; while training, the weights
        // change after every step and each step draws its move from the new logits
        if (nt == 0 && step > 0) {
            RBMG_CK(launch_fused<false>(prop, L, L.spins_prop, B, S->logits_prop.as<float>(), st));
        } else if (prop->O <= 128) {
            // the tensor-core path evaluates every logits row, so the draw is its own pass
            RBMG_CK(launch_draw(L, st));
            RBMG_CK(launch_fused<false>(prop, L, L.spins_prop, B, S->logits_prop.as<float>(), st));
        } else {
            RBMG_CK(launch_fused<true>(prop, L, nullptr, B, S->logits_prop.as<float>(), st));
        }
        L.propose_next = nt == 0 && step + 1 < n_steps ? 1 : 0;
        RBMG_CK(launch_learned(1, P, L, st));
        if (nt > 0 && prop->objective == RBMG_PROPOSAL_LOCALLY_BALANCED) {
            // cross-entropy to the locally balanced proposal at the first nt walkers' states
            r = proposal_forward(prop, nt, L.spins, nullptr, st);
            if (r != RBMG_OK) return r;
            RBMG_CK(launch_lb_target(P, nt, L.spins, L.theta, L.re, prop->logits.as<float>(), prop->O,
                                     prop->dl32.as<float>(), st));
        } else if (nt > 0) {
            // REINFORCE on the moves of the first nt walkers, from the states they started at
            r = proposal_forward(prop, nt, L.spins_pre, nullptr, st);
            if (r != RBMG_OK) return r;
            reward_mean_kernel<<<1, 256, 0, st>>>(L.reward, nt, S->rbar.as<float>());
            reinforce_kernel<<<(nt + kWarpsPerBlock - 1) / kWarpsPerBlock, 32 * kWarpsPerBlock, 0, st>>>(
                prop->logits.as<float>(), nt, c->N, prop->O, L.site, L.len, L.reward, S->rbar.as<float>(),
                prop->dl32.as<float>());
            RBMG_CK(cudaGetLastError());
        }
        if (nt > 0) {
            r = proposal_backward(prop, nt, st);
            if (r != RBMG_OK) return r;
            r = proposal_adam(prop, st);
            if (r != RBMG_OK) return r;
            // the walkers' current logits under the new weights
            RBMG_CK(launch_fused<false>(prop, L, L.spins, B, L.logits_cur, st));
        }
        if (measured(step)) RBMG_CK(measure(step, st));
    }
    return RBMG_OK;
}

// Measurement hook: n_steps frozen learned steps on one stream (the single-stream sequence
// of rbmg_chain_learned_async, train = 0) with CUDA events around every network pass and
// every accept pass; returns their mean durations in milliseconds.
extern "C" int rbmg_chain_learned_kernel_times(rbmg_chain* c, const rbmg_psi* psi, rbmg_proposal* prop, int n_steps,
                                               double* ms_network, double* ms_accept) {
    if (!c || !psi || !prop || n_steps < 1 || !ms_network || !ms_accept)
        return fail(RBMG_EINVAL, "learned kernel times: bad arguments");
    if (psi->kind != 0 || psi->N != c->N || prop->N != c->N)
        return fail(RBMG_EINVAL, "learned kernel times: psi or proposal does not match the chain");
    if (prop->O > 128) return fail(RBMG_EUNSUPPORTED, "learned kernel times: networks with N + 8 <= 128");
    cudaStream_t st = stream();
    const RbmDev P = psi->rbm_dev();
    LearnedState* S = nullptr;
    LearnedLaunch L{};
    int r = learned_prepare(c, psi, prop, 0, st, &S, L);
    if (r != RBMG_OK) return r;
    std::vector<cudaEvent_t> ev(4 * static_cast<size_t>(n_steps));
    for (auto& e : ev) RBMG_CK(cudaEventCreate(&e));
    cudaError_t err = launch_draw(L, st);
    for (int step = 0; step < n_steps && err == cudaSuccess; step++) {
        cudaEvent_t* e = ev.data() + 4 * static_cast<size_t>(step);
        cudaEventRecord(e[0], st);
        err = launch_fused<false>(prop, L, L.spins_prop, static_cast<int>(c->walkers), S->logits_prop.as<float>(), st);
        cudaEventRecord(e[1], st);
        L.propose_next = step + 1 < n_steps ? 1 : 0;
        cudaEventRecord(e[2], st);
        if (err == cudaSuccess) err = launch_learned(1, P, L, st);
        cudaEventRecord(e[3], st);
    }
    if (err == cudaSuccess) err = cudaStreamSynchronize(st);
    double tn = 0.0, ta = 0.0;
    for (int step = 0; step < n_steps && err == cudaSuccess; step++) {
        float a = 0.0f, b = 0.0f;
        cudaEvent_t* e = ev.data() + 4 * static_cast<size_t>(step);
        err = cudaEventElapsedTime(&a, e[0], e[1]);
        if (err == cudaSuccess) err = cudaEventElapsedTime(&b, e[2], e[3]);
        tn += a;
        ta += b;
    }
    for (auto& e : ev) cudaEventDestroy(e);
    if (err != cudaSuccess) return cuda_fail(err, "learned kernel times");
    *ms_network = tn / n_steps;
    *ms_accept = ta / n_steps;
    return RBMG_OK;
}

// Test hook: the locally balanced training target of lb_target_kernel for `count`
// configurations with the given logits [count][N+8]: dl = (q - p*) / count, the angles of
// the configurations from scratch by the scalar angles kernel.
extern "C" int rbmg_proposal_lb_target(rbmg_proposal* prop, const rbmg_psi* psi, int count, const uint64_t* spins,
                                       const float* logits, float* dl) {
    if (!prop || !psi || count < 1 || !spins || !logits || !dl) return fail(RBMG_EINVAL, "lb target: bad arguments");
    if (psi->kind != 0 || psi->N != prop->N) return fail(RBMG_EINVAL, "lb target: psi does not match the proposal");
    cudaStream_t st = stream();
    const RbmDev P = psi->rbm_dev();
    const size_t n = static_cast<size_t>(count), nw = static_cast<size_t>(nwords_of(P.N)),
                 O = static_cast<size_t>(prop->O), per = static_cast<size_t>((P.Mpad / 32 + 1) / 2) * 32;
    DevBuf d_spins, d_theta, d_re, d_logits, d_dl;
    RBMG_CK(d_spins.ensure(sizeof(uint64_t) * n * nw));
    RBMG_CK(d_theta.ensure(sizeof(float4) * n * per));
    RBMG_CK(d_re.ensure(sizeof(float2) * n * per));
    RBMG_CK(d_logits.ensure(sizeof(float) * n * O));
    RBMG_CK(d_dl.ensure(sizeof(float) * n * O));
    RBMG_CK(cudaMemcpyAsync(d_spins.p, spins, sizeof(uint64_t) * n * nw, cudaMemcpyHostToDevice, st));
    RBMG_CK(cudaMemcpyAsync(d_logits.p, logits, sizeof(float) * n * O, cudaMemcpyHostToDevice, st));
    LearnedLaunch L{};
    L.B = count;
    L.N = P.N;
    L.O = prop->O;
    L.spins = d_spins.as<uint64_t>();
    L.theta = d_theta.as<float4>();
    L.re = d_re.as<float2>();
    RBMG_CK(launch_learned(0, P, L, st));
    RBMG_CK(launch_lb_target(P, count, L.spins, L.theta, L.re, d_logits.as<float>(), prop->O, d_dl.as<float>(), st));
    RBMG_CK(cudaMemcpyAsync(dl, d_dl.p, sizeof(float) * n * O, cudaMemcpyDeviceToHost, st));
    RBMG_CK(cudaStreamSynchronize(st));
    return RBMG_OK;
}

// Test hook: n_steps frozen learned steps of every walker (the single-stream sequence of
// rbmg_chain_learned_async with train = 0: the first move drawn by its own pass, the
// network on the proposed states, the accept pass drawing the next move), with the state
// copied to the host around every launch, so that a CPU replay fed the same logits can
// check every draw, acceptance ratio and decision.
extern "C" int rbmg_chain_learned_trace(rbmg_chain* c, const rbmg_psi* psi, rbmg_proposal* prop, int n_steps,
                                        uint64_t* spins0, uint64_t* rng0, float* theta0, float* re0, float* logits0,
                                        float* logits_prop, int* site, int* len, float* logq, uint64_t* spins,
                                        uint64_t* accepts, uint64_t* rng_end) {
    if (!c || !psi || !prop || n_steps < 1 || !spins0 || !rng0 || !theta0 || !re0 || !logits0 || !logits_prop ||
        !site || !len || !logq || !spins || !accepts || !rng_end)
        return fail(RBMG_EINVAL, "learned trace: bad arguments");
    if (psi->kind != 0 || psi->N != c->N || prop->N != c->N)
        return fail(RBMG_EINVAL, "learned trace: psi or proposal does not match the chain");
    if (prop->O > 128) return fail(RBMG_EUNSUPPORTED, "learned trace: networks with N + 8 <= 128");
    cudaStream_t st = stream();
    const RbmDev P = psi->rbm_dev();
    LearnedState* S = nullptr;
    LearnedLaunch L{};
    int r = learned_prepare(c, psi, prop, 0, st, &S, L);
    if (r != RBMG_OK) return r;
    const size_t B = static_cast<size_t>(c->walkers), nw = static_cast<size_t>(c->nw), O = static_cast<size_t>(prop->O);
    const int KP = (P.Mpad / 32 + 1) / 2;
    std::vector<float4> th(B * KP * 32);
    std::vector<float2> rf(B * KP * 32);
    RBMG_CK(cudaMemcpyAsync(spins0, L.spins, sizeof(uint64_t) * B * nw, cudaMemcpyDeviceToHost, st));
    RBMG_CK(cudaMemcpyAsync(rng0, L.rng_index, sizeof(uint64_t) * B, cudaMemcpyDeviceToHost, st));
    RBMG_CK(cudaMemcpyAsync(th.data(), L.theta, sizeof(float4) * th.size(), cudaMemcpyDeviceToHost, st));
    RBMG_CK(cudaMemcpyAsync(rf.data(), L.re, sizeof(float2) * rf.size(), cudaMemcpyDeviceToHost, st));
    RBMG_CK(cudaMemcpyAsync(logits0, L.logits_cur, sizeof(float) * B * O, cudaMemcpyDeviceToHost, st));
    RBMG_CK(cudaStreamSynchronize(st));
    // paired layout -> unit order: lane l, pair kk holds units l + 32 (2 kk) and l + 32 (2 kk + 1)
    for (size_t w = 0; w < B; w++)
        for (int kk = 0; kk < KP; kk++)
            for (int l = 0; l < 32; l++) {
                const float4 t = th[(w * KP + kk) * 32 + l];
                const float2 f = rf[(w * KP + kk) * 32 + l];
                const int j0 = l + 64 * kk, j1 = j0 + 32;
                if (j0 < P.Mpad) {
                    theta0[(w * P.Mpad + j0) * 2] = t.x;
                    theta0[(w * P.Mpad + j0) * 2 + 1] = t.z;
                    re0[w * P.Mpad + j0] = f.x;
                }
                if (j1 < P.Mpad) {
                    theta0[(w * P.Mpad + j1) * 2] = t.y;
                    theta0[(w * P.Mpad + j1) * 2 + 1] = t.w;
                    re0[w * P.Mpad + j1] = f.y;
                }
            }
    for (int step = 0; step < n_steps; step++) {
        if (step == 0) RBMG_CK(launch_draw(L, st));
        RBMG_CK(launch_fused<false>(prop, L, L.spins_prop, static_cast<int>(B), S->logits_prop.as<float>(), st));
        const size_t t = static_cast<size_t>(step);
        RBMG_CK(cudaMemcpyAsync(logits_prop + t * B * O, L.logits_prop, sizeof(float) * B * O, cudaMemcpyDeviceToHost,
                                st));
        RBMG_CK(cudaMemcpyAsync(site + t * B, L.site, sizeof(int) * B, cudaMemcpyDeviceToHost, st));
        RBMG_CK(cudaMemcpyAsync(len + t * B, L.len, sizeof(int) * B, cudaMemcpyDeviceToHost, st));
        RBMG_CK(cudaMemcpyAsync(logq + t * B, L.logq_fwd, sizeof(float) * B, cudaMemcpyDeviceToHost, st));
        L.propose_next = step + 1 < n_steps ? 1 : 0;
        RBMG_CK(launch_learned(1, P, L, st));
        RBMG_CK(cudaMemcpyAsync(spins + t * B * nw, L.spins, sizeof(uint64_t) * B * nw, cudaMemcpyDeviceToHost, st));
        RBMG_CK(cudaMemcpyAsync(accepts + t * B, L.accepts, sizeof(uint64_t) * B, cudaMemcpyDeviceToHost, st));
        RBMG_CK(cudaStreamSynchronize(st));
    }
    RBMG_CK(cudaMemcpyAsync(rng_end, L.rng_index, sizeof(uint64_t) * B, cudaMemcpyDeviceToHost, st));
    RBMG_CK(cudaStreamSynchronize(st));
    return RBMG_OK;
}
