// Hidden angles from scratch on the tensor cores: theta[w][j] = b_j + sum_i s_i(w) W_ij for a
// batch of configurations, the dense (configurations x spins) . (spins x hidden) contraction
// (include/quantum_state/Psi.hpp:43-53 sums it one spin at a time per angle).
//
// The spins are +-1, exact in BF16.  W is split into three BF16 parts per real component,
// W = hi + mid + lo (each the rounded remainder of the previous: 24 significant bits in
// all), so the products are exact and the tensor cores accumulate them in FP32 in TMEM;
// the result differs from the scalar sum only in the order of the FP32 additions.
//
// One CTA (16 warps) takes 128 configurations: their spins form the A operand (128 x Kp,
// Kp = N rounded up to 16) in shared memory.  The hidden units are taken in chunks of at
// most 256; for each chunk the six B operands (hi / mid / lo of Re W and Im W, each n x Kp,
// packed in global memory in the shared-memory layout by rbm_tc_pack_kernel when W
// changes) arrive one after another by bulk copy, and one thread issues Kp / 16
// tcgen05.mma per operand into the chunk's real (TMEM columns 0..255) and imaginary
// (256..511) accumulators.  The epilogue adds the bias and writes theta (and, for the
// learned chain, Re f(theta)) in the paired layout of the sampler, or plain complex64 rows.
// Every mbarrier wait is bounded: on timeout the kernel raises an error flag, waits
// (bounded) for its copy or MMAs in flight, frees its TMEM and returns.
#include "host.h"
#include "rbm_impl.cuh"
#include "tc_common.cuh"

namespace rbmg {

using bf16 = __nv_bfloat16;

namespace {

using namespace tc;

constexpr int kAgRows = 128;        // configurations per CTA (the MMA's M)
constexpr int kAgThreads = 512;     // 16 warps: 4 TMEM lane quarters x 4 column groups
constexpr int kAgChunk = 256;       // hidden units per accumulator chunk
constexpr int kAgCols = 512;        // TMEM columns: real and imaginary accumulators
constexpr size_t kAgMinSmem = 116 * 1024;   // one CTA per SM: it holds the whole TMEM

__host__ __device__ inline int chunks_of(int Mpad) { return (Mpad + kAgChunk - 1) / kAgChunk; }
__host__ __device__ inline int chunk_cols(int Mpad, int c) { return Mpad - c * kAgChunk < kAgChunk ? Mpad - c * kAgChunk : kAgChunk; }

// B operand images of W: for chunk c, split s (hi, mid, lo), part p (re, im): rows = the
// chunk's hidden units, columns = spins, zero beyond N and M
__global__ void rbm_tc_pack_kernel(int N, int M, int Mpad, int Kp, const float2* W, bf16* out) {
    const long idx = static_cast<long>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (idx >= static_cast<long>(Mpad) * Kp) return;
    const int j = static_cast<int>(idx / Kp), i = static_cast<int>(idx - static_cast<long>(j) * Kp);
    const int c = j / kAgChunk, jl = j - c * kAgChunk;
    const int nc = min(kAgChunk, Mpad - c * kAgChunk);
    const size_t image = static_cast<size_t>(nc) * Kp;              // elements of one image
    bf16* base = out + static_cast<size_t>(c) * kAgChunk * Kp * 6;  // chunks before c are full
    const float2 w = (i < N && j < M) ? W[static_cast<long>(i) * Mpad + j] : make_float2(0.0f, 0.0f);
    const uint32_t off = kmajor_offset(jl, i, nc) / 2;
#pragma unroll
    for (int p = 0; p < 2; p++) {
        float x = p == 0 ? w.x : w.y;
#pragma unroll
        for (int sp = 0; sp < 3; sp++) {
            const bf16 h = __float2bfloat16_rn(x);
            base[(static_cast<size_t>(sp) * 2 + p) * image + off] = h;
            x -= __bfloat162float(h);   // exact: the remainder of a rounding to 8 bits
        }
    }
}

struct AgLaunch {
    int count, N, Mpad, Kp, KP;
    const uint64_t* spins;   // [count][NW]
    const float2* b;         // [Mpad]
    const bf16* images;      // rbm_tc_pack_kernel output
    float4* theta;           // paired: [count][KP][32] (re k, re k+1, im k, im k+1), or null
    float2* re;              // paired: [count][KP][32] Re f, or null
    float2* plain;           // [count][Mpad] complex64 angles, or null
    int* error;
};

template <int NW>
__global__ void __launch_bounds__(kAgThreads, 1) angles_tc_kernel(AgLaunch L) {
    extern __shared__ __align__(1024) unsigned char asm_[];
    const size_t a_bytes = static_cast<size_t>(kAgRows) * L.Kp * 2;
    const size_t b_bytes = static_cast<size_t>(kAgChunk) * L.Kp * 2;
    unsigned char* sA = asm_;
    unsigned char* sB = asm_ + a_bytes;
    uint64_t* mbar = reinterpret_cast<uint64_t*>(asm_ + a_bytes + b_bytes);   // MMAs done
    uint64_t* wbar = mbar + 1;                                                // operand landed
    uint32_t* tslot = reinterpret_cast<uint32_t*>(mbar + 2);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int quarter = warp & 3, cgroup = warp >> 2;
    const int row0 = blockIdx.x * kAgRows;
    const int rows = min(kAgRows, L.count - row0);
    const uint32_t aA = saddr_of(sA), aB = saddr_of(sB), aM = saddr_of(mbar), aW = saddr_of(wbar);
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(aM));
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(aW));
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(saddr_of(tslot)),
                     "r"(kAgCols));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::);
    }
    // A: row r = configuration row0 + r, +-1 spins, zero beyond N (a chunk's 8 columns lie
    // in one spin word)
    {
        const int kc = L.Kp / 8;
        for (int c = tid; c < kAgRows * kc; c += kAgThreads) {
            const int r = c % kAgRows, col = (c / kAgRows) * 8;
            const bool live = r < rows;
            const uint64_t word = live ? L.spins[static_cast<long>(row0 + r) * NW + (col >> 6)] : 0ull;
            uint32_t pk[4];
#pragma unroll
            for (int e = 0; e < 8; e += 2) {
                float x[2];
#pragma unroll
                for (int u = 0; u < 2; u++) {
                    const int i = col + e + u;
                    x[u] = (live && i < L.N) ? (((word >> (i & 63)) & 1ull) ? 1.0f : -1.0f) : 0.0f;
                }
                pk[e / 2] = pack_bf16(x[0], x[1]);
            }
            *reinterpret_cast<uint4*>(sA + kmajor_offset(r, col, kAgRows)) = make_uint4(pk[0], pk[1], pk[2], pk[3]);
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::);
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::);
    const uint32_t tmem = *tslot;
    bool ok = true, w_pending = false, m_pending = false;
    uint32_t mphase = 0, wphase = 0;
    const int r = quarter * 32 + lane;   // this thread's configuration (TMEM lane)
    const uint32_t lane_base = static_cast<uint32_t>(quarter * 32) << 16;
    const int nchunks = chunks_of(L.Mpad);
    for (int c = 0; c < nchunks && ok; c++) {
        const int nc = chunk_cols(L.Mpad, c);
        const size_t image_bytes = static_cast<size_t>(nc) * L.Kp * 2;
        const unsigned char* cbase =
            reinterpret_cast<const unsigned char*>(L.images) + static_cast<size_t>(c) * kAgChunk * L.Kp * 2 * 6;
        for (int q = 0; q < 6 && ok; q++) {   // q = 2 split + part
            const int sp = q >> 1, p = q & 1;
            if (tid == 0) bulk_g2s(aB, cbase + static_cast<size_t>(q) * image_bytes, static_cast<uint32_t>(image_bytes), aW);
            w_pending = true;
            // A (first round) is visible to the tensor cores, the operand has landed
            asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
            ok = __syncthreads_and(mbar_wait(aW, wphase)) != 0;
            if (!ok) break;
            w_pending = false;
            wphase ^= 1u;
            if (tid == 0) {
                asm volatile("tcgen05.fence::after_thread_sync;\n" ::);
                const uint32_t idesc = instr_desc(kAgRows, nc);
                for (int s = 0; s < L.Kp / 16; s++) {
                    const uint64_t da = smem_desc(aA + s * (kAgRows / 8) * 256, 128, 256);
                    const uint64_t db = smem_desc(aB + s * (nc / 8) * 256, 128, 256);
                    tc_mma(tmem + static_cast<uint32_t>(p * kAgChunk), da, db, idesc, (sp > 0 || s > 0) ? 1 : 0);
                }
                tc_commit(aM);
            }
            m_pending = true;
            __syncwarp();
            // the MMAs are done before B is overwritten or the accumulators are read
            ok = __syncthreads_and(mbar_wait(aM, mphase)) != 0;
            if (!ok) break;
            m_pending = false;
            mphase ^= 1u;
        }
        if (!ok) break;
        asm volatile("tcgen05.fence::after_thread_sync;\n" ::);
        // epilogue: pair kk = 4 c + cgroup of hidden units (k = 2 kk, 2 kk + 1), columns
        // 64 cgroup .. + 63 of the chunk, eight lanes' units at a time
        const int c0 = cgroup * 64;
        if (c0 < nc) {   // warp-uniform: the TMEM loads are warp-collective
            const int kk = 4 * c + cgroup;
            const long w = row0 + r;
            const bool live = r < rows;
            const bool odd = c0 + 32 < nc;   // the pair's second unit exists in W (else zero padding)
            for (int l0 = 0; l0 < 32; l0 += 8) {
                float re0[8], re1[8], im0[8], im1[8];
                tc_ld8(tmem + lane_base + static_cast<uint32_t>(c0 + l0), re0);
                tc_ld8(tmem + lane_base + static_cast<uint32_t>(kAgChunk + c0 + l0), im0);
                if (odd) {
                    tc_ld8(tmem + lane_base + static_cast<uint32_t>(c0 + 32 + l0), re1);
                    tc_ld8(tmem + lane_base + static_cast<uint32_t>(kAgChunk + c0 + 32 + l0), im1);
                }
                if (!live) continue;
#pragma unroll
                for (int e = 0; e < 8; e++) {
                    const int l = l0 + e;
                    const int j0 = 64 * kk + l, j1 = j0 + 32;
                    const float2 b0 = __ldg(L.b + j0);
                    const float2 b1 = odd ? __ldg(L.b + j1) : make_float2(0.0f, 0.0f);
                    const float tr0 = re0[e] + b0.x, ti0 = im0[e] + b0.y;
                    const float tr1 = odd ? re1[e] + b1.x : 0.0f, ti1 = odd ? im1[e] + b1.y : 0.0f;
                    if (L.theta) {
                        const long o = (w * L.KP + kk) * 32 + l;
                        L.theta[o] = make_float4(tr0, tr1, ti0, ti1);
                        float f0, f1;
                        up2(lc_re2(pk2(tr0, tr1), pk2(ti0, ti1)), f0, f1);
                        L.re[o] = make_float2(f0, f1);
                    }
                    if (L.plain) {
                        L.plain[w * L.Mpad + j0] = make_float2(tr0, ti0);
                        if (odd) L.plain[w * L.Mpad + j1] = make_float2(tr1, ti1);
                    }
                }
            }
        }
        // the accumulators are read before the next chunk's MMAs overwrite them
        asm volatile("tcgen05.fence::before_thread_sync;\n" ::);
        __syncthreads();
    }
    if (!ok) {
        if (tid == 0) atomicExch(L.error, 1);
        if (w_pending) mbar_wait(aW, wphase);
        if (m_pending) mbar_wait(aM, mphase);
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::);
    __syncthreads();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(kAgCols));
}

size_t ag_smem(int Kp) {
    const size_t need = static_cast<size_t>(kAgRows) * Kp * 2 + static_cast<size_t>(kAgChunk) * Kp * 2 + 64;
    return std::max(need, kAgMinSmem);
}

}  // namespace

int rbm_tc_kp(int N) { return (N + 15) / 16 * 16; }

size_t rbm_tc_pack_elems(int Mpad, int Kp) { return static_cast<size_t>(Mpad) * Kp * 6; }

bool rbm_tc_supported(int N, int Mpad) {
    // A and one B operand in shared memory (227 KB), chunks of whole pairs of 32 units
    return ag_smem(rbm_tc_kp(N)) <= 220 * 1024 && Mpad % 32 == 0;
}

cudaError_t launch_rbm_tc_pack(int N, int M, int Mpad, const float2* W, bf16* out, cudaStream_t st) {
    const int Kp = rbm_tc_kp(N);
    const long n = static_cast<long>(Mpad) * Kp;
    rbm_tc_pack_kernel<<<static_cast<int>((n + 255) / 256), 256, 0, st>>>(N, M, Mpad, Kp, W, out);
    return cudaGetLastError();
}

cudaError_t launch_angles_tc(int count, int N, int Mpad, const uint64_t* spins, const float2* b, const bf16* images,
                             float4* theta, float2* re, float2* plain, int* error, cudaStream_t st) {
    if (count <= 0) return cudaSuccess;
    AgLaunch L{};
    L.count = count;
    L.N = N;
    L.Mpad = Mpad;
    L.Kp = rbm_tc_kp(N);
    L.KP = (Mpad / 32 + 1) / 2;
    L.spins = spins;
    L.b = b;
    L.images = images;
    L.theta = theta;
    L.re = re;
    L.plain = plain;
    L.error = error;
    const size_t sm = ag_smem(L.Kp);
    const dim3 grid((count + kAgRows - 1) / kAgRows);
#define RBMG_AG_CASE(NWV)                                                                                      \
    case NWV: {                                                                                                \
        cudaError_t e = cudaFuncSetAttribute(angles_tc_kernel<NWV>, cudaFuncAttributeMaxDynamicSharedMemorySize, \
                                             static_cast<int>(sm));                                            \
        if (e != cudaSuccess) return e;                                                                        \
        angles_tc_kernel<NWV><<<grid, kAgThreads, sm, st>>>(L);                                                \
        break;                                                                                                 \
    }
    switch ((N + 63) / 64) {
        RBMG_AG_CASE(1)
        RBMG_AG_CASE(2)
        RBMG_AG_CASE(3)
        RBMG_AG_CASE(4)
        default: return cudaErrorInvalidValue;
    }
#undef RBMG_AG_CASE
    return cudaGetLastError();
}

}  // namespace rbmg
