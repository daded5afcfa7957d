// Proposal-network inference on the 5th-generation tensor cores (tcgen05, TMEM).
//
// One CTA (4 warps) evaluates the network N -> 256 -> 256 (SiLU) -> N+8 for 128
// configurations.  Per layer the activations (A, 128 x K) and the layer's transposed
// weights (B, n x K) sit in shared memory in the canonical K-major layout without swizzle
// (8-row x 16-byte core matrices, 128 contiguous bytes each); one elected thread issues
// K/16 tcgen05.mma (kind::f16, BF16 operands, FP32 accumulation, M = 128) into a
// 256-column TMEM accumulator (of 512 allocated), and tcgen05.commit arrives on an
// mbarrier when they are done.  Each thread then reads its row of the accumulator with
// tcgen05.ld, adds the bias, applies SiLU and writes the BF16 result as the next layer's A
// operand.  The waits on the mbarrier are bounded: on timeout the kernel raises an error
// flag, waits (bounded) for its MMAs, frees its TMEM and returns.
#include <cuda_bf16.h>

#include "host.h"
#include "rbm_impl.cuh"

namespace rbmg {

using bf16 = __nv_bfloat16;

namespace {

constexpr int kTcRows = 128;               // configurations per CTA (the MMA's M)
constexpr int kTcThreads = 128;            // one thread per row
constexpr int kTcHidden = 256;
// TMEM columns allocated: the accumulator uses 256 (FP32, 128 x 256); the whole 512 are
// held (one CTA per SM by its shared memory) so no MMA shape can reach unallocated columns
constexpr int kTcCols = 512;
constexpr uint32_t kTcSpin = 1u << 24;     // mbarrier polls before giving up

// shared memory: A [128 x 256] bf16 = 64 KB, B [256 x 256] bf16 = 128 KB, barrier + slot
constexpr size_t kTcA = size_t(kTcRows) * kTcHidden * 2;
constexpr size_t kTcB = size_t(kTcHidden) * kTcHidden * 2;
constexpr size_t kTcSmem = kTcA + kTcB + 64;

// byte offset of element (row, col) of a K-major operand with `rows` rows in the canonical
// no-swizzle layout, one block per MMA K step of 16 columns: within the block of step
// col / 16, core matrix (row / 8, (col / 8) & 1) at (row / 8) * 256 + ((col / 8) & 1) * 128.
// A step's descriptor has start = block, leading (K) byte offset 128, stride (M / N) 256;
// every address it can form lies inside its own block.
__device__ __forceinline__ uint32_t kmajor_offset(int row, int col, int rows) {
    return static_cast<uint32_t>((col >> 4) * (rows >> 3) * 256 + (row >> 3) * 256 + ((col >> 3) & 1) * 128 +
                                 (row & 7) * 16 + (col & 7) * 2);
}

// shared-memory matrix descriptor (sm_100 UMMA): start >> 4 [0,14), leading-dimension
// byte offset >> 4 [16,30) (between core matrices adjacent in K), stride-dimension byte
// offset >> 4 [32,46) (between core matrices adjacent in M / N), version 1 [46,48),
// layout 0 = no swizzle [61,64)
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    return static_cast<uint64_t>((saddr & 0x3FFFFu) >> 4) | (static_cast<uint64_t>(lbo >> 4) << 16) |
           (static_cast<uint64_t>(sbo >> 4) << 32) | (1ull << 46);
}

// instruction descriptor, kind::f16: D FP32 [4,6) = 1, A BF16 [7,10) = 1, B BF16 [10,13) = 1,
// both K-major, N >> 3 [17,23), M >> 4 [24,29)
__device__ __forceinline__ uint32_t instr_desc(int n) {
    return (1u << 4) | (1u << 7) | (1u << 10) | (static_cast<uint32_t>(n >> 3) << 17) |
           (static_cast<uint32_t>(kTcRows >> 4) << 24);
}

__device__ __forceinline__ uint32_t saddr_of(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void tc_mma(uint32_t tmem_d, uint64_t da, uint64_t db, uint32_t idesc, int accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem_d),
        "l"(da), "l"(db), "r"(idesc), "r"(accumulate));
}

__device__ __forceinline__ void tc_commit(uint32_t mbar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(mbar)
                 : "memory");
}

// bounded wait for the mbarrier phase `parity`; false on timeout
__device__ __forceinline__ bool mbar_wait(uint32_t mbar, uint32_t parity) {
    for (uint32_t i = 0; i < kTcSpin; i++) {
        uint32_t done = 0;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}\n"
            : "=r"(done)
            : "r"(mbar), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}

__device__ __forceinline__ void tc_ld32(uint32_t taddr, float (&v)[32]) {
    uint32_t r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
        "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];\n"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
          "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
          "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
#pragma unroll
    for (int i = 0; i < 32; i++) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ void cp16(uint32_t saddr, const void* g) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(saddr), "l"(g));
}

// B <- rows [0, n) of Wt [n][ldw] (k contiguous), k < K, in the canonical layout with n rows
__device__ __forceinline__ void load_weights(uint32_t sB, const bf16* Wt, int ldw, int n, int K) {
    const int chunks = n * (K / 8);
    for (int c = threadIdx.x; c < chunks; c += kTcThreads) {
        const int row = c / (K / 8), kb = c % (K / 8);
        cp16(sB + kmajor_offset(row, kb * 8, n), Wt + static_cast<long>(row) * ldw + kb * 8);
    }
    asm volatile("cp.async.commit_group;\n" ::);
}

// the SiLU of the layer-by-layer path: hardware exponential and division, then BF16
__device__ __forceinline__ bf16 tc_silu(float acc, float b) {
    const float z = acc + b;
    return __float2bfloat16_rn(__fdividef(z, 1.0f + __expf(-z)));
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
};

template <int NW>
__global__ void __launch_bounds__(kTcThreads, 1) mlp_tc_kernel(TcNet net, const uint64_t* spins, int count,
                                                               float* logits_out, int* error) {
    extern __shared__ __align__(1024) unsigned char tsm[];
    unsigned char* sA = tsm;
    unsigned char* sB = tsm + kTcA;
    uint64_t* mbar = reinterpret_cast<uint64_t*>(tsm + kTcA + kTcB);
    uint32_t* tslot = reinterpret_cast<uint32_t*>(tsm + kTcA + kTcB + 16);
    const int tid = threadIdx.x, warp = tid >> 5;
    const int row0 = blockIdx.x * kTcRows;
    const uint32_t aA = saddr_of(sA), aB = saddr_of(sB), aM = saddr_of(mbar);
    // ---- TMEM (warp 0) and the mbarrier (thread 0)
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(saddr_of(tslot)),
                     "r"(kTcCols));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::);
    }
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(aM));
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::);
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::);
    const uint32_t tmem = *tslot;
    // ---- layer-1 input: row tid = configuration row0 + tid, +-1 spins, zero beyond N
    {
        const int w = row0 + tid;
        uint64_t s[NW];
#pragma unroll
        for (int k = 0; k < NW; k++) s[k] = w < count ? spins[static_cast<long>(w) * NW + k] : 0ull;
        for (int c = 0; c < net.ldw1; c += 8) {
            __align__(16) bf16 v[8];
#pragma unroll
            for (int e = 0; e < 8; e++) {
                const int i = c + e;
                float x = 0.0f;
                if (w < count && i < net.N) x = ((s[i >> 6] >> (i & 63)) & 1ull) ? 1.0f : -1.0f;
                v[e] = __float2bfloat16_rn(x);
            }
            *reinterpret_cast<uint4*>(sA + kmajor_offset(tid, c, kTcRows)) = *reinterpret_cast<const uint4*>(v);
        }
    }
    bool ok = true;
    uint32_t phase = 0;
    const uint32_t lane_base = static_cast<uint32_t>(warp * 32) << 16;
    for (int layer = 0; layer < 3; layer++) {
        const int K = layer == 0 ? net.ldw1 : kTcHidden;
        const int n = layer == 2 ? 128 : kTcHidden;
        const bf16* Wt = layer == 0 ? net.w1t : (layer == 1 ? net.w2t : net.w3t);
        const int ldw = layer == 0 ? net.ldw1 : kTcHidden;
        load_weights(aB, Wt, ldw, n, K);
        asm volatile("cp.async.wait_group 0;\n" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");   // generic-proxy writes -> async proxy
        __syncthreads();
        if (tid == 0) {
            asm volatile("tcgen05.fence::after_thread_sync;\n" ::);
            const uint32_t idesc = instr_desc(n);
            for (int s = 0; s < K / 16; s++) {
                const uint64_t da = smem_desc(aA + s * (kTcRows / 8) * 256, 128, 256);
                const uint64_t db = smem_desc(aB + s * (n / 8) * 256, 128, 256);
                tc_mma(tmem, da, db, idesc, s > 0);
            }
            tc_commit(aM);
        }
        __syncwarp();
        // every thread has seen the MMAs complete (or the block gives up) before A is rewritten
        ok = __syncthreads_and(mbar_wait(aM, phase)) != 0;
        if (!ok) break;
        phase ^= 1u;
        asm volatile("tcgen05.fence::after_thread_sync;\n" ::);
        // ---- epilogue: this thread's row of the accumulator
        const float* bias = layer == 0 ? net.b1 : (layer == 1 ? net.b2 : net.b3);
        for (int c = 0; c < n; c += 32) {
            float v[32];
            tc_ld32(tmem + lane_base + static_cast<uint32_t>(c), v);
            if (layer < 2) {
#pragma unroll
                for (int g = 0; g < 32; g += 8) {
                    __align__(16) bf16 h[8];
#pragma unroll
                    for (int e = 0; e < 8; e++) h[e] = tc_silu(v[g + e], bias[c + g + e]);
                    *reinterpret_cast<uint4*>(sA + kmajor_offset(tid, c + g, kTcRows)) =
                        *reinterpret_cast<const uint4*>(h);
                }
            } else {
                const int w = row0 + tid;
#pragma unroll
                for (int e = 0; e < 32; e++) {
                    const int j = c + e;
                    if (w < count && j < net.O) logits_out[static_cast<long>(w) * net.O + j] = v[e] + bias[j];
                }
            }
        }
        asm volatile("tcgen05.fence::before_thread_sync;\n" ::);
        __syncthreads();
    }
    if (!ok) {
        if (tid == 0) atomicExch(error, 1);
        // the MMAs of the timed-out layer may still run: give them a bounded second wait
        mbar_wait(aM, phase);
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
