// The S matrix on the tensor cores: S += G^T conj(G) for a chunk of per-sample O_k rows
// G [n][L] (smatrix.cu holds the reference's semantics, the FP32 tile kernel, the centring
// mean and the finishing pass; this file replaces the tile kernel's products).
//
// Complex products in real arithmetic: with a = G[s][k], b = G[s][k'],
//   Re S += Re a Re b + Im a Im b,   Im S += Im a Re b - Re a Im b.
// Every real value is split into three BF16 parts (hi, mid, lo: 24 significant bits) and a
// product keeps the six part pairs whose size reaches 2^-16 of it (hi hi, hi mid, mid hi,
// hi lo, lo hi, mid mid), so the FP32 accumulators see the products to about FP32
// accuracy.  The hi-hi products go into "main" accumulators and the five smaller pairs into
// separate "correction" accumulators, so that the large running sums take only two
// tensor-core additions per 16 samples (the accumulation's rounding grows with the number
// of additions into a sum); both are added when the tile leaves TMEM.
//
// Two kernels per window of at most 1024 samples (the depth of the FP32 sums before the FP64
// matrix takes them):
//   sm_tc_prep_kernel   forms sqrt(w) (G - shift) once per element (for the complex RBM from
//                       tanh(theta) and the spins, never stored in FP32) and writes its six
//                       BF16 planes (Re / Im x hi / mid / lo) in the tensor cores' canonical
//                       K-major no-swizzle layout: [stage of 16 samples][group of 8 rows]
//                       [plane][8 rows x 16 samples] (256 B per core-matrix pair), so that
//                       the operand of a 128-row tile for one stage is 24 KB in one piece;
//   sm_tc_kernel        one CTA per 128 x 128 tile of the upper triangle: one thread streams
//                       the tile's row and column operands of each stage into a four-deep
//                       ring of shared-memory buffers with bulk copies and issues 24
//                       tcgen05.mma (kind::f16, M = N = 128, K = 16) per stage into four
//                       TMEM accumulators (main Re / Im, correction Re / Im: 512 columns);
//                       the negated term (- Re a Im b) uses the instruction descriptor's
//                       negate-A bit.  At the end the 16 warps read TMEM, add main and
//                       correction, stage the tile in shared memory and add it into the FP64
//                       matrix with coalesced read-modify-writes (the CTA owns the tile).
// Every mbarrier wait is bounded: on timeout the kernel raises an error flag, waits
// (bounded) for its copies and MMAs in flight, frees its TMEM and returns.
#include "host.h"
#include "smatrix.h"
#include "smatrix_rows.cuh"
#include "tc_common.cuh"

namespace rbmg {

namespace {

using namespace tc;
using bf16 = __nv_bfloat16;

constexpr int kTile = 128;                           // tile edge = MMA M = MMA N
constexpr int kStageSamples = 16;                    // MMA K
constexpr int kPlanes = 6;                           // Re hi / mid / lo, Im hi / mid / lo
constexpr int kGroupBytes = 8 * kStageSamples * 2;   // one core-matrix pair: 256 B
constexpr int kTileGroups = kTile / 8;               // 16 row groups per tile
constexpr int kOpBytes = kTileGroups * kPlanes * kGroupBytes;   // 24 KB: one operand of a stage
constexpr int kRing = 4;                             // stage buffers (A and B each)
constexpr int kWindow = 1024;                        // samples per launch (FP32 depth)
constexpr int kWindowStages = kWindow / kStageSamples;
constexpr int kThreads = 512;
constexpr int kTmemCols = 512;
constexpr int kHeader = 1024;                        // barriers and the TMEM slot
constexpr size_t kSmem = kHeader + static_cast<size_t>(kRing) * 2 * kOpBytes;
constexpr int kEpiPitch = kTile + 1;                 // float2 per row of the staged tile
static_assert(static_cast<size_t>(kTile) * kEpiPitch * sizeof(float2) <= kSmem - kHeader, "epilogue tile");

// hi / mid / lo BF16 parts of x (each the rounded remainder of the previous; the
// remainders are exact in FP32)
__device__ __forceinline__ void split3(float x, bf16 (&p)[3]) {
#pragma unroll
    for (int q = 0; q < 3; q++) {
        p[q] = __float2bfloat16_rn(x);
        x -= __bfloat162float(p[q]);
    }
}

__device__ __forceinline__ uint32_t pair_bits(bf16 lo, bf16 hi) {
    __nv_bfloat162 v;
    v.x = lo;
    v.y = hi;
    return *reinterpret_cast<const uint32_t*>(&v);
}

// planes of samples [s0 + 16 g, s0 + 16 g + 16) for row groups 16 blockIdx.x ..: a thread
// writes the 16-byte core-matrix row (row, half of the stage's samples) of every plane
__global__ void __launch_bounds__(256) sm_tc_prep_kernel(SmSource a, int s0, int cnt, int RG,
                                                         uint4* __restrict__ planes) {
    __shared__ float cw[kStageSamples];
    const int g = blockIdx.y, tid = threadIdx.x;
    if (tid < kStageSamples) {
        const int s = s0 + g * kStageSamples + tid;
        cw[tid] = (a.weighted && s < s0 + cnt) ? static_cast<float>(sqrt(a.w[s])) : 1.0f;
    }
    __syncthreads();
    const int rg = blockIdx.x * kTileGroups + (tid >> 4);
    if (rg >= RG) return;
    const int r7 = (tid >> 1) & 7, half = tid & 1;
    const int k = rg * 8 + r7;
    SmSource u = a;
    u.weighted = 0;   // the weight's root is cw[], taken once per sample
    const SmElem e = sm_elem_of(u, k);
    uint32_t w[kPlanes][4];
#pragma unroll
    for (int q = 0; q < 8; q += 2) {
        const int sl = half * 8 + q;
        const int s = s0 + g * kStageSamples + sl;
        float2 v0 = s < s0 + cnt ? sm_load_f(u, e, s, k) : make_float2(0.0f, 0.0f);
        float2 v1 = s + 1 < s0 + cnt ? sm_load_f(u, e, s + 1, k) : make_float2(0.0f, 0.0f);
        v0.x *= cw[sl];
        v0.y *= cw[sl];
        v1.x *= cw[sl + 1];
        v1.y *= cw[sl + 1];
        bf16 r0[3], i0[3], r1[3], i1[3];
        split3(v0.x, r0);
        split3(v0.y, i0);
        split3(v1.x, r1);
        split3(v1.y, i1);
#pragma unroll
        for (int p = 0; p < 3; p++) {
            w[p][q / 2] = pair_bits(r0[p], r1[p]);
            w[3 + p][q / 2] = pair_bits(i0[p], i1[p]);
        }
    }
    // uint4 units: 16 per core-matrix pair, 8 per K half, 1 per row
    uint4* dst = planes + (static_cast<size_t>(g) * RG + rg) * kPlanes * 16 + half * 8 + r7;
#pragma unroll
    for (int p = 0; p < kPlanes; p++) dst[p * 16] = make_uint4(w[p][0], w[p][1], w[p][2], w[p][3]);
}

__device__ __forceinline__ void expect_tx(uint32_t mbar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(mbar), "r"(bytes) : "memory");
}

__device__ __forceinline__ void bulk_copy(uint32_t dst, const void* src, uint32_t bytes, uint32_t mbar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n" ::"r"(
                     dst),
                 "l"(src), "r"(bytes), "r"(mbar)
                 : "memory");
}

// tile (tm, tn), tm <= tn, of the upper triangle's idx-th tile, column by column
__device__ __forceinline__ void tri_tile(int idx, int& tm, int& tn) {
    int c = static_cast<int>((sqrtf(8.0f * static_cast<float>(idx) + 1.0f) - 1.0f) * 0.5f);
    while (c > 0 && c * (c + 1) / 2 > idx) c--;
    while ((c + 1) * (c + 2) / 2 <= idx) c++;
    tn = c;
    tm = idx - c * (c + 1) / 2;
}

struct TcLaunch {
    const unsigned char* planes;   // [G][RG][6][256 B]
    int G, RG, L;
    double2* S;
    int* error;
};

// the 24 MMAs of one stage; a / b: shared addresses of the row and column operands
__device__ __forceinline__ void stage_mmas(uint32_t tmem, uint32_t a, uint32_t b, bool first) {
    const uint32_t id = instr_desc(kTile, kTile);
    const uint32_t id_neg = id | (1u << 13);   // negate A
    constexpr uint32_t kSbo = kPlanes * kGroupBytes;   // between row groups of one plane
    auto da = [&](int p) { return smem_desc(a + p * kGroupBytes, 128, kSbo); };
    auto db = [&](int p) { return smem_desc(b + p * kGroupBytes, 128, kSbo); };
    const uint32_t main_re = tmem, main_im = tmem + 128, corr_re = tmem + 256, corr_im = tmem + 384;
    const int acc0 = first ? 0 : 1;
    // planes: Re parts 0, 1, 2; Im parts 3, 4, 5
    tc_mma(main_re, da(0), db(0), id, acc0);
    tc_mma(main_re, da(3), db(3), id, 1);
    tc_mma(main_im, da(3), db(0), id, acc0);
    tc_mma(main_im, da(0), db(3), id_neg, 1);
    const int pa[5] = {0, 1, 0, 2, 1}, pb[5] = {1, 0, 2, 0, 1};
#pragma unroll
    for (int q = 0; q < 5; q++) {
        const int acc = (first && q == 0) ? 0 : 1;
        tc_mma(corr_re, da(pa[q]), db(pb[q]), id, acc);
        tc_mma(corr_re, da(3 + pa[q]), db(3 + pb[q]), id, 1);
        tc_mma(corr_im, da(3 + pa[q]), db(pb[q]), id, acc);
        tc_mma(corr_im, da(pa[q]), db(3 + pb[q]), id_neg, 1);
    }
}

__global__ void __launch_bounds__(kThreads, 1) sm_tc_kernel(TcLaunch p) {
    int tm, tn;
    tri_tile(blockIdx.x, tm, tn);
    extern __shared__ __align__(1024) unsigned char smem[];
    uint64_t* full = reinterpret_cast<uint64_t*>(smem);   // [kRing]: a stage's operands arrived
    uint64_t* empty = full + kRing;                       // [kRing]: a stage's MMAs finished
    uint32_t* tslot = reinterpret_cast<uint32_t*>(empty + kRing);
    unsigned char* ring = smem + kHeader;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    if (tid == 0) {
        for (int i = 0; i < kRing; i++) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(saddr_of(full + i)));
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(saddr_of(empty + i)));
        }
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(saddr_of(tslot)),
                     "r"(kTmemCols));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::);
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::);
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::);
    const uint32_t tmem = *tslot;
    const int G = p.G;
    int ok = 1;
    if (warp == 0) {
        if (lane == 0) {
            const bool diag = tm == tn;
            const uint32_t ring0 = saddr_of(ring);
            const size_t stage_bytes = static_cast<size_t>(p.RG) * kPlanes * kGroupBytes;
            auto load = [&](int g) {
                const int b = g % kRing;
                const uint32_t dst = ring0 + b * 2 * kOpBytes;
                const uint32_t bar = saddr_of(full + b);
                const unsigned char* src = p.planes + static_cast<size_t>(g) * stage_bytes;
                expect_tx(bar, diag ? kOpBytes : 2 * kOpBytes);
                bulk_copy(dst, src + static_cast<size_t>(tm) * kOpBytes, kOpBytes, bar);
                if (!diag) bulk_copy(dst + kOpBytes, src + static_cast<size_t>(tn) * kOpBytes, kOpBytes, bar);
            };
            int loaded = 0, consumed = 0, committed = 0;
            for (; loaded < min(kRing, G); loaded++) load(loaded);
            for (int g = 0; g < G; g++) {
                const int b = g % kRing;
                if (!mbar_wait(saddr_of(full + b), (g / kRing) & 1)) {
                    ok = 0;
                    break;
                }
                consumed = g + 1;
                asm volatile("tcgen05.fence::after_thread_sync;\n" ::);
                const uint32_t a_op = ring0 + b * 2 * kOpBytes;
                stage_mmas(tmem, a_op, diag ? a_op : a_op + kOpBytes, g == 0);
                tc_commit(saddr_of(empty + b));
                committed = g + 1;
                // refill the previous stage's buffer once its MMAs are done (this stage's
                // MMAs keep the tensor pipe busy meanwhile)
                if (g >= 1 && g - 1 + kRing < G) {
                    const int bp = (g - 1) % kRing;
                    if (!mbar_wait(saddr_of(empty + bp), ((g - 1) / kRing) & 1)) {
                        ok = 0;
                        break;
                    }
                    load(loaded++);
                }
            }
            // the last commit tracks every MMA issued before it
            if (committed > 0 && !mbar_wait(saddr_of(empty + (committed - 1) % kRing), ((committed - 1) / kRing) & 1))
                ok = 0;
            if (!ok) {
                atomicExch(p.error, 1);
                for (int g = consumed; g < loaded; g++) mbar_wait(saddr_of(full + g % kRing), (g / kRing) & 1);
            }
        }
        __syncwarp();
    }
    ok = __syncthreads_and(ok);
    if (ok && G > 0) {
        asm volatile("tcgen05.fence::after_thread_sync;\n" ::);
        // TMEM -> registers: warp (quarter, column group) holds rows 32 quarter + lane,
        // columns 32 group .. + 31; main + correction; staged as float2 [128][129]
        float2* tile = reinterpret_cast<float2*>(ring);
        const int quarter = warp & 3, cg = warp >> 2;
        const uint32_t t0 = tmem + (static_cast<uint32_t>(quarter * 32) << 16) + static_cast<uint32_t>(cg * 32);
        float re[32], im[32], c[32];
        tc_ld32(t0, re);
        tc_ld32(t0 + 256, c);
#pragma unroll
        for (int e = 0; e < 32; e++) re[e] += c[e];
        tc_ld32(t0 + 128, im);
        tc_ld32(t0 + 384, c);
#pragma unroll
        for (int e = 0; e < 32; e++) im[e] += c[e];
        float2* row = tile + (quarter * 32 + lane) * kEpiPitch + cg * 32;
#pragma unroll
        for (int e = 0; e < 32; e++) row[e] = make_float2(re[e], im[e]);
        __syncthreads();
        const int m0 = tm * kTile, n0 = tn * kTile;
        for (int idx = tid; idx < kTile * kTile; idx += kThreads) {
            const int r = idx / kTile, cc = idx - r * kTile;
            const int gr = m0 + r, gc = n0 + cc;
            if (gr < p.L && gc < p.L && gr <= gc) {
                const float2 v = tile[r * kEpiPitch + cc];
                double2* d = p.S + static_cast<long>(gr) * p.L + gc;
                double2 x = *d;
                x.x += static_cast<double>(v.x);
                x.y += static_cast<double>(v.y);
                *d = x;
            }
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::);
    __syncthreads();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(kTmemCols));
}

int padded_rows(int L) { return (L + kTile - 1) / kTile * kTile; }

}  // namespace

size_t sm_tc_planes_bytes(int L) {
    return static_cast<size_t>(kWindowStages) * (padded_rows(L) / 8) * kPlanes * kGroupBytes;
}

cudaError_t launch_sm_tc_accumulate(const SmSource& a, double2* S, void* planes, int* error, int* launches,
                                    cudaStream_t st) {
    if (a.count <= 0) return cudaSuccess;
    const int Lpad = padded_rows(a.L), RG = Lpad / 8, nt = Lpad / kTile;
    cudaError_t e = cudaFuncSetAttribute(sm_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         static_cast<int>(kSmem));
    if (e != cudaSuccess) return e;
    for (int s0 = 0; s0 < a.count; s0 += kWindow) {
        const int cnt = std::min(kWindow, a.count - s0);
        const int G = (cnt + kStageSamples - 1) / kStageSamples;
        sm_tc_prep_kernel<<<dim3(nt, G), 256, 0, st>>>(a, s0, cnt, RG, static_cast<uint4*>(planes));
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
        TcLaunch p{static_cast<const unsigned char*>(planes), G, RG, a.L, S, error};
        sm_tc_kernel<<<nt * (nt + 1) / 2, kThreads, kSmem, st>>>(p);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
        if (launches) *launches += 2;
    }
    return cudaSuccess;
}

}  // namespace rbmg
