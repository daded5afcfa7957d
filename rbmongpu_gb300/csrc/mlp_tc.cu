// Proposal-network inference on the 5th-generation tensor cores (tcgen05, TMEM).
//
// One CTA (16 warps) evaluates the network N -> 256 -> 256 (SiLU) -> N+8 for 128
// configurations.  Per layer the activations (A, 128 x K) and the layer's transposed
// weights (B, n x K) sit in shared memory in the canonical K-major layout without swizzle
// (8-row x 16-byte core matrices, 128 contiguous bytes each).  The weights are kept in
// global memory already in that layout (tc_pack_kernel, run when the weights change), so
// one thread moves a whole layer with a single bulk copy (cp.async.bulk) that completes
// on an mbarrier.  One elected thread issues K/16 tcgen05.mma (kind::f16, BF16 operands,
// FP32 accumulation, M = 128) into a 256-column TMEM accumulator (of 512 allocated), and
// tcgen05.commit arrives on a second mbarrier when they are done; the next layer's
// weights are then copied into B while the epilogue runs: warp w reads TMEM lanes
// 32 (w % 4) .. +31 (its rows) and a quarter of the columns with tcgen05.ld, adds the
// bias, applies SiLU and writes the BF16 result as the next layer's A operand.  The logits
// are staged in shared memory and written out row-contiguous.  Every wait on an mbarrier is
// bounded: on timeout the kernel raises an error flag, waits (bounded) for its copies and
// MMAs in flight, frees its TMEM and returns.
#include <cuda_bf16.h>

#include "host.h"
#include "rbm_impl.cuh"
#include "tc_common.cuh"

namespace rbmg {

using bf16 = __nv_bfloat16;

namespace {

using namespace tc;

constexpr int kTcRows = 128;               // configurations per CTA (the MMA's M)
constexpr int kTcThreads = 512;            // 16 warps: 4 TMEM lane quarters x 4 column groups
constexpr int kTcHidden = 256;
// TMEM columns allocated: the accumulator uses 256 (FP32, 128 x 256); the whole 512 are
// held (one CTA per SM by its shared memory) so no MMA shape can reach unallocated columns
constexpr int kTcCols = 512;

// shared memory: A [128 x 256] bf16 = 64 KB, B [256 x 256] bf16 = 128 KB (after the last
// MMA it holds the FP32 logits, [128][O + 1]), biases (256 + 256 + 128 floats), barrier + slot
constexpr size_t kTcA = size_t(kTcRows) * kTcHidden * 2;
constexpr size_t kTcB = size_t(kTcHidden) * kTcHidden * 2;
constexpr size_t kTcBias = (2 * kTcHidden + kTcRows) * sizeof(float);
constexpr size_t kTcSmem = kTcA + kTcB + kTcBias + 64;
static_assert(size_t(kTcRows) * (kTcRows + 1) * sizeof(float) <= kTcB, "logit staging fits in B");

__device__ __forceinline__ float tanh_hw(float x) {
    float y;
    asm("tanh.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// SiLU(z) = z sigmoid(z) = h + h tanh(h) with h = z / 2: one hardware tanh per element;
// the result is rounded to BF16, coarser than the tanh's own error
__device__ __forceinline__ float tc_silu(float z) {
    const float h = 0.5f * z;
    return fmaf(h, tanh_hw(h), h);
}


}  // namespace

struct TcNet {
    int N, O, ldw1;
    const bf16* w1t;   // [256][ldw1]
    const bf16* w2t;   // [256][256]
    const bf16* w3t;   // [>= 128][256]
    const float* b1;
    const float* b2;
    const float* b3;
    const bf16* pack;  // the three layers' B operands in the shared-memory layout (tc_pack_size)
};

// elements of the packed operands: W1 [256 x ldw1], W2 [256 x 256], W3 [128 x 256]
size_t tc_pack_size(int ldw1) {
    return static_cast<size_t>(kTcHidden) * ldw1 + static_cast<size_t>(kTcHidden) * kTcHidden +
           static_cast<size_t>(kTcRows) * kTcHidden;
}

namespace {

// out (image of a B operand with n rows and K columns) <- Wt [n][ldw]
__global__ void tc_pack_kernel(const bf16* Wt, int ldw, int n, int K, bf16* out) {
    const long idx = static_cast<long>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (idx >= static_cast<long>(n) * K) return;
    const int row = static_cast<int>(idx / K), col = static_cast<int>(idx - static_cast<long>(row) * K);
    out[kmajor_offset(row, col, n) / 2] = Wt[static_cast<long>(row) * ldw + col];
}

}  // namespace

cudaError_t launch_tc_pack(const TcNet& net, bf16* pack, cudaStream_t st) {
    const long n1 = static_cast<long>(kTcHidden) * net.ldw1, n2 = static_cast<long>(kTcHidden) * kTcHidden,
               n3 = static_cast<long>(kTcRows) * kTcHidden;
    tc_pack_kernel<<<static_cast<int>((n1 + 255) / 256), 256, 0, st>>>(net.w1t, net.ldw1, kTcHidden, net.ldw1, pack);
    tc_pack_kernel<<<static_cast<int>((n2 + 255) / 256), 256, 0, st>>>(net.w2t, kTcHidden, kTcHidden, kTcHidden,
                                                                         pack + n1);
    tc_pack_kernel<<<static_cast<int>((n3 + 255) / 256), 256, 0, st>>>(net.w3t, kTcHidden, kTcRows, kTcHidden,
                                                                         pack + n1 + n2);
    return cudaGetLastError();
}

template <int NW>
__global__ void __launch_bounds__(kTcThreads, 1) mlp_tc_kernel(TcNet net, const uint64_t* spins, int count,
                                                               float* logits_out, int* error) {
    extern __shared__ __align__(1024) unsigned char tsm[];
    unsigned char* sA = tsm;
    unsigned char* sB = tsm + kTcA;
    float* sBias = reinterpret_cast<float*>(tsm + kTcA + kTcB);   // b1 | b2 | b3
    uint64_t* mbar = reinterpret_cast<uint64_t*>(tsm + kTcA + kTcB + kTcBias);        // MMAs done
    uint32_t* tslot = reinterpret_cast<uint32_t*>(tsm + kTcA + kTcB + kTcBias + 16);
    uint64_t* wbar = reinterpret_cast<uint64_t*>(tsm + kTcA + kTcB + kTcBias + 32);   // weights landed
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int quarter = warp & 3, cgroup = warp >> 2;
    const int row0 = blockIdx.x * kTcRows;
    const int rows = min(kTcRows, count - row0);
    const uint32_t aA = saddr_of(sA), aB = saddr_of(sB), aM = saddr_of(mbar), aW = saddr_of(wbar);
    // layer l's packed B operand and its size
    auto w_src = [&](int l) {
        const size_t o1 = static_cast<size_t>(kTcHidden) * net.ldw1;
        return l == 0 ? net.pack : (l == 1 ? net.pack + o1 : net.pack + o1 + static_cast<size_t>(kTcHidden) * kTcHidden);
    };
    auto w_bytes = [&](int l) {
        return static_cast<uint32_t>(l == 0 ? kTcHidden * net.ldw1 * 2 : (l == 1 ? kTcHidden * kTcHidden * 2
                                                                                  : kTcRows * kTcHidden * 2));
    };
    // ---- the mbarriers, and the layer-1 weights streaming in at once (thread 0)
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(aM));
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(aW));
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
        bulk_g2s(aB, w_src(0), w_bytes(0), aW);
    }
    bool w_pending = true;   // a weight copy is in flight (known to every thread)
    // ---- TMEM (warp 0)
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(saddr_of(tslot)),
                     "r"(kTcCols));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::);
    }
    for (int j = tid; j < 2 * kTcHidden + kTcRows; j += kTcThreads) {
        float b = 0.0f;
        if (j < kTcHidden) b = net.b1[j];
        else if (j < 2 * kTcHidden) b = net.b2[j - kTcHidden];
        else if (j - 2 * kTcHidden < net.O) b = net.b3[j - 2 * kTcHidden];
        sBias[j] = b;
    }
    // ---- layer-1 input: row r = configuration row0 + r, +-1 spins, zero beyond N; the
    // 8 columns of a chunk lie in one spin word, loaded once
    {
        const int kc = net.ldw1 / 8;
        for (int c = tid; c < kTcRows * kc; c += kTcThreads) {
            const int r = c % kTcRows, col = (c / kTcRows) * 8;
            const bool live = r < rows;
            const uint64_t word = live ? spins[static_cast<long>(row0 + r) * NW + (col >> 6)] : 0ull;
            uint32_t pk[4];
#pragma unroll
            for (int e = 0; e < 8; e += 2) {
                float x[2];
#pragma unroll
                for (int u = 0; u < 2; u++) {
                    const int i = col + e + u;
                    x[u] = (live && i < net.N) ? (((word >> (i & 63)) & 1ull) ? 1.0f : -1.0f) : 0.0f;
                }
                pk[e / 2] = pack_bf16(x[0], x[1]);
            }
            *reinterpret_cast<uint4*>(sA + kmajor_offset(r, col, kTcRows)) = make_uint4(pk[0], pk[1], pk[2], pk[3]);
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::);
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::);
    const uint32_t tmem = *tslot;
    bool ok = true;
    uint32_t phase = 0, wphase = 0;
    bool mma_pending = false;
    const int r = quarter * 32 + lane;                                  // this thread's row (TMEM lane)
    const uint32_t lane_base = static_cast<uint32_t>(quarter * 32) << 16;
    for (int layer = 0; layer < 3; layer++) {
        const int K = layer == 0 ? net.ldw1 : kTcHidden;
        const int n = layer == 2 ? kTcRows : kTcHidden;
        // the epilogue's generic-proxy writes of A are visible to the tensor cores, and this
        // layer's weights have landed
        asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
        ok = __syncthreads_and(mbar_wait(aW, wphase)) != 0;
        if (!ok) break;
        w_pending = false;
        wphase ^= 1u;
        if (tid == 0) {
            asm volatile("tcgen05.fence::after_thread_sync;\n" ::);
            const uint32_t idesc = instr_desc(kTcRows, n);
            for (int s = 0; s < K / 16; s++) {
                const uint64_t da = smem_desc(aA + s * (kTcRows / 8) * 256, 128, 256);
                const uint64_t db = smem_desc(aB + s * (n / 8) * 256, 128, 256);
                tc_mma(tmem, da, db, idesc, s > 0);
            }
            tc_commit(aM);
        }
        mma_pending = true;
        __syncwarp();
        // every thread has seen the MMAs complete (or the block gives up) before A or B is rewritten
        ok = __syncthreads_and(mbar_wait(aM, phase)) != 0;
        if (!ok) break;
        mma_pending = false;
        phase ^= 1u;
        asm volatile("tcgen05.fence::after_thread_sync;\n" ::);
        // the next layer's weights stream into B during the epilogue
        if (layer < 2) {
            if (tid == 0) bulk_g2s(aB, w_src(layer + 1), w_bytes(layer + 1), aW);
            w_pending = true;
            const float* bias = sBias + layer * kTcHidden;
            for (int c = cgroup * 64; c < cgroup * 64 + 64; c += 32) {
                float v[32];
                tc_ld32(tmem + lane_base + static_cast<uint32_t>(c), v);
#pragma unroll
                for (int g = 0; g < 32; g += 8) {
                    uint32_t pk[4];
#pragma unroll
                    for (int e = 0; e < 8; e += 2)
                        pk[e / 2] = pack_bf16(tc_silu(v[g + e] + bias[c + g + e]),
                                              tc_silu(v[g + e + 1] + bias[c + g + e + 1]));
                    *reinterpret_cast<uint4*>(sA + kmajor_offset(r, c + g, kTcRows)) =
                        make_uint4(pk[0], pk[1], pk[2], pk[3]);
                }
            }
        } else {
            // logits [128][O + 1] (odd stride: lanes = rows hit distinct banks) over B
            float* stage = reinterpret_cast<float*>(sB);
            const int ld = net.O + 1;
            const int c = cgroup * 32;
            float v[32];
            tc_ld32(tmem + lane_base + static_cast<uint32_t>(c), v);
#pragma unroll
            for (int e = 0; e < 32; e++)
                if (c + e < net.O) stage[r * ld + c + e] = v[e] + sBias[2 * kTcHidden + c + e];
            __syncthreads();
            float* out = logits_out + static_cast<long>(row0) * net.O;
            for (int i = tid; i < rows * net.O; i += kTcThreads) {
                const int rr = i / net.O, j = i - rr * net.O;
                out[i] = stage[rr * ld + j];
            }
        }
        asm volatile("tcgen05.fence::before_thread_sync;\n" ::);
    }
    if (!ok) {
        if (tid == 0) atomicExch(error, 1);
        // copies and MMAs still in flight: a bounded second wait before the block leaves
        if (w_pending) mbar_wait(aW, wphase);
        if (mma_pending) mbar_wait(aM, phase);
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::);
    __syncthreads();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(kTcCols));
}

cudaError_t launch_mlp_tc(const TcNet& net, int nw, const uint64_t* spins, int count, float* out, int* error,
                          cudaStream_t st) {
    if (count <= 0) return cudaSuccess;
    const dim3 grid((count + kTcRows - 1) / kTcRows);
#define RBMG_TC_CASE(NWV)                                                                                       \
    case NWV: {                                                                                                 \
        cudaError_t e = cudaFuncSetAttribute(mlp_tc_kernel<NWV>, cudaFuncAttributeMaxDynamicSharedMemorySize,   \
                                             static_cast<int>(kTcSmem));                                        \
        if (e != cudaSuccess) return e;                                                                         \
        mlp_tc_kernel<NWV><<<grid, kTcThreads, kTcSmem, st>>>(net, spins, count, out, error);                   \
        break;                                                                                                  \
    }
    switch (nw) {
        RBMG_TC_CASE(1)
        RBMG_TC_CASE(2)
        RBMG_TC_CASE(3)
        RBMG_TC_CASE(4)
        default: return cudaErrorInvalidValue;
    }
#undef RBMG_TC_CASE
    return cudaGetLastError();
}

}  // namespace rbmg
