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
// of additions into a sum); both are added when the tile leaves TMEM.  A tile's FP32 sums
// span one window of at most 1024 samples before the FP64 matrix takes them.
//
// Two kernels per chunk of samples:
//   sm_tc_prep_kernel   forms sqrt(w) (G - shift) once per element (for the complex RBM from
//                       tanh(theta) and the spins in FP32, never stored) and writes its six
//                       BF16 planes (Re / Im x hi / mid / lo) in the tensor cores' canonical
//                       K-major no-swizzle layout: [stage of 16 samples][group of 8 rows]
//                       [plane][8 rows x 16 samples] (256 B per core-matrix pair), so that
//                       the operand of a 128-row tile for one stage is 24 KB in one piece;
//   sm_tc_kernel        persistent, one CTA per SM, each owning a fixed set of the 128 x 128
//                       tiles of the upper triangle for every window (so that no two CTAs
//                       update one tile).  Warp 16 streams a tile's row and column operands
//                       of each stage into a three-deep ring of shared-memory buffers with
//                       bulk copies; warp 17 issues 24 tcgen05.mma (kind::f16, M = N = 128,
//                       K = 16) per stage into four TMEM accumulators (main Re / Im,
//                       correction Re / Im: 512 columns; the negated term - Re a Im b uses
//                       the instruction descriptor's negate-A bit); warps 0-15 drain the
//                       accumulators into registers, hand TMEM back, and add the tile into
//                       the FP64 matrix (staged in shared memory, in two halves, for
//                       coalesced read-modify-writes) while the next tile's MMAs run.
// Every mbarrier wait is bounded: a role that gives up raises the CTA's abort flag and the
// error flag, the others leave at their next wait, and the CTA waits (bounded) for its
// copies and MMAs in flight, frees its TMEM and returns.
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
constexpr int kRing = 3;                             // stage buffers (A and B each)
constexpr int kWindowStages = 64;                    // 1024 samples per window (FP32 depth)
constexpr int kEpiWarps = 16;                        // TMEM drain and FP64 update
constexpr int kProducerWarp = kEpiWarps, kMmaWarp = kEpiWarps + 1;
constexpr int kThreads = (kEpiWarps + 2) * 32;
constexpr int kEpiThreads = kEpiWarps * 32;
constexpr int kTmemCols = 512;
constexpr int kHeader = 1024;                        // barriers, flags and the TMEM slot
constexpr int kHalf = kTile / 2;                     // columns per epilogue half
constexpr int kEpiPitch = kHalf + 1;                 // float2 per row of the staged half tile
constexpr size_t kEpiOff = kHeader + static_cast<size_t>(kRing) * 2 * kOpBytes;
constexpr size_t kSmem = kEpiOff + static_cast<size_t>(kTile) * kEpiPitch * sizeof(float2);
static_assert(kSmem <= 232448, "shared memory");

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

// planes of samples [16 g, 16 g + 16) of the chunk for row groups 16 blockIdx.x ..: a thread
// writes the 16-byte core-matrix row (row, half of the stage's samples) of every plane.
// Complex RBM rows are formed in FP32: s_i tanh(theta_j), minus the shift as an FP32 pair
// (hi + lo: within an ulp of the FP64 difference the CUDA-core kernel takes); FP64 rows
// (PsiDeep) are shifted in FP64.
__global__ void __launch_bounds__(256) sm_tc_prep_kernel(SmSource a, int RG, uint4* __restrict__ planes) {
    __shared__ float cw[kStageSamples];
    const int g = blockIdx.y, tid = threadIdx.x;
    if (tid < kStageSamples) {
        const int s = g * kStageSamples + tid;
        cw[tid] = (a.weighted && s < a.count) ? static_cast<float>(sqrt(a.w[s])) : 1.0f;
    }
    __syncthreads();
    const int rg = blockIdx.x * kTileGroups + (tid >> 4);
    if (rg >= RG) return;
    const int r7 = (tid >> 1) & 7, half = tid & 1;
    const int k = rg * 8 + r7;
    SmSource u = a;
    u.weighted = 0;   // the weight's root is cw[], taken once per sample
    const SmElem e = sm_elem_of(u, k);
    float2 sh_hi = make_float2(0.0f, 0.0f), sh_lo = sh_hi;
    if (a.kind == 0 && a.shift && e.live) {
        const double2 d = a.shift[k];
        sh_hi = make_float2(static_cast<float>(d.x), static_cast<float>(d.y));
        sh_lo = make_float2(static_cast<float>(d.x - static_cast<double>(sh_hi.x)),
                            static_cast<float>(d.y - static_cast<double>(sh_hi.y)));
    }
    auto value = [&](int s) -> float2 {
        if (!e.live || s >= a.count) return make_float2(0.0f, 0.0f);
        if (a.kind != 0) return sm_load_f(u, e, s, k);
        float2 t = a.T[static_cast<long>(s) * a.Mpad + e.j];
        if (e.i >= 0) {
            const uint64_t word = a.enumerate ? ((e.i >> 6) == 0 ? a.enum_base + static_cast<uint64_t>(s) : 0ull)
                                              : a.spins[static_cast<long>(s) * a.nw + (e.i >> 6)];
            if (!((word >> (e.i & 63)) & 1ull)) t = make_float2(-t.x, -t.y);
        }
        return make_float2((t.x - sh_hi.x) - sh_lo.x, (t.y - sh_hi.y) - sh_lo.y);
    };
    uint32_t w[kPlanes][4];
#pragma unroll
    for (int q = 0; q < 8; q += 2) {
        const int sl = half * 8 + q;
        const int s = g * kStageSamples + sl;
        float2 v0 = value(s), v1 = value(s + 1);
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

// sixteen consecutive accumulator columns of this warp's 32 TMEM lanes, added into v
__device__ __forceinline__ void tc_add16(uint32_t taddr, float* v) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; i++) v[i] += __uint_as_float(r[i]);
}

__device__ __forceinline__ void mbar_arrive(uint32_t mbar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];\n" ::"r"(mbar) : "memory");
}

// bounded wait for the mbarrier phase `parity` that also gives up once another role of
// the CTA has raised the abort flag
__device__ __forceinline__ bool wait_or_abort(uint32_t mbar, uint32_t parity, const volatile int* abort) {
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
        if ((i & 255u) == 255u && *abort) return false;
    }
    return false;
}

// named barrier of the epilogue warps with an AND over their predicates
__device__ __forceinline__ bool epi_all(bool pred) {
    uint32_t r;
    asm volatile(
        "{\n\t.reg .pred p, q;\n\t"
        "setp.ne.u32 p, %1, 0;\n\t"
        "bar.red.and.pred q, 1, %2, p;\n\t"
        "selp.u32 %0, 1, 0, q;\n\t}\n"
        : "=r"(r)
        : "r"(static_cast<uint32_t>(pred)), "n"(kEpiThreads)
        : "memory");
    return r != 0;
}

__device__ __forceinline__ void epi_sync() { asm volatile("bar.sync 1, %0;\n" ::"n"(kEpiThreads) : "memory"); }

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
    int G, RG, L, ntiles;
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
    extern __shared__ __align__(1024) unsigned char smem[];
    uint64_t* full = reinterpret_cast<uint64_t*>(smem);   // [kRing]: a stage's operands arrived
    uint64_t* empty = full + kRing;                       // [kRing]: a stage's MMAs finished
    uint64_t* tfull = empty + kRing;                      // a tile's accumulators are complete
    uint64_t* tempty = tfull + 1;                         // the epilogue has drained TMEM
    volatile int* abort = reinterpret_cast<volatile int*>(tempty + 1);
    int* consumed_sh = const_cast<int*>(abort) + 1;       // stages the MMA warp took
    uint32_t* tslot = reinterpret_cast<uint32_t*>(consumed_sh + 1);
    unsigned char* ring = smem + kHeader;
    float2* stage_tile = reinterpret_cast<float2*>(smem + kEpiOff);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int windows = (p.G + kWindowStages - 1) / kWindowStages;
    if (tid == 0) {
        for (int i = 0; i < kRing; i++) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(saddr_of(full + i)));
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(saddr_of(empty + i)));
        }
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(saddr_of(tfull)));
        asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(saddr_of(tempty)), "r"(kEpiWarps));
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
        *abort = 0;
        *consumed_sh = 0;
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
    const uint32_t ring0 = saddr_of(ring);
    const size_t stage_bytes = static_cast<size_t>(p.RG) * kPlanes * kGroupBytes;
    int issued = 0;   // producer: stages whose copies were issued

    if (warp == kProducerWarp) {
        if (lane == 0) {
            bool ok = true;
            for (int w = 0; w < windows && ok; w++) {
                const int gw = min(kWindowStages, p.G - w * kWindowStages);
                for (int t = blockIdx.x; t < p.ntiles && ok; t += gridDim.x) {
                    int tm, tn;
                    tri_tile(t, tm, tn);
                    const bool diag = tm == tn;
                    for (int g = 0; g < gw; g++) {
                        const int slot = issued % kRing;
                        if (issued >= kRing &&
                            !wait_or_abort(saddr_of(empty + slot), ((issued / kRing) - 1) & 1, abort)) {
                            ok = false;
                            break;
                        }
                        const uint32_t dst = ring0 + slot * 2 * kOpBytes, bar = saddr_of(full + slot);
                        const unsigned char* src =
                            p.planes + static_cast<size_t>(w * kWindowStages + g) * stage_bytes;
                        expect_tx(bar, diag ? kOpBytes : 2 * kOpBytes);
                        bulk_copy(dst, src + static_cast<size_t>(tm) * kOpBytes, kOpBytes, bar);
                        if (!diag) bulk_copy(dst + kOpBytes, src + static_cast<size_t>(tn) * kOpBytes, kOpBytes, bar);
                        issued++;
                    }
                }
            }
            if (!ok) {
                *abort = 1;
                atomicExch(p.error, 1);
            }
        }
        __syncwarp();
    } else if (warp == kMmaWarp) {
        if (lane == 0) {
            bool ok = true;
            int it = 0, tw = 0;
            for (int w = 0; w < windows && ok; w++) {
                const int gw = min(kWindowStages, p.G - w * kWindowStages);
                for (int t = blockIdx.x; t < p.ntiles && ok; t += gridDim.x) {
                    int tm, tn;
                    tri_tile(t, tm, tn);
                    const bool diag = tm == tn;
                    if (tw > 0) {
                        if (!wait_or_abort(saddr_of(tempty), (tw - 1) & 1, abort)) {
                            ok = false;
                            break;
                        }
                        asm volatile("tcgen05.fence::after_thread_sync;\n" ::);
                    }
                    for (int g = 0; g < gw; g++) {
                        const int slot = it % kRing;
                        if (!wait_or_abort(saddr_of(full + slot), (it / kRing) & 1, abort)) {
                            ok = false;
                            break;
                        }
                        asm volatile("tcgen05.fence::after_thread_sync;\n" ::);
                        const uint32_t a_op = ring0 + slot * 2 * kOpBytes;
                        stage_mmas(tmem, a_op, diag ? a_op : a_op + kOpBytes, g == 0);
                        tc_commit(saddr_of(empty + slot));
                        it++;
                    }
                    if (!ok) break;
                    tc_commit(saddr_of(tfull));
                    tw++;
                }
            }
            *consumed_sh = it;
            if (!ok) {
                *abort = 1;
                atomicExch(p.error, 1);
                // the last commit tracks every MMA issued before it
                if (it > 0) mbar_wait(saddr_of(empty + (it - 1) % kRing), ((it - 1) / kRing) & 1);
            }
        }
        __syncwarp();
    } else {
        // epilogue: warp (quarter, column group) drains rows 32 quarter + lane, columns
        // 32 group .. + 31 of the four accumulators
        const int quarter = warp & 3, cg = warp >> 2;
        const uint32_t t0 = tmem + (static_cast<uint32_t>(quarter * 32) << 16) + static_cast<uint32_t>(cg * 32);
        int tw = 0;
        for (int w = 0; w < windows; w++) {
            bool go = true;
            for (int t = blockIdx.x; t < p.ntiles; t += gridDim.x) {
                int r = 0;
                if (lane == 0) r = wait_or_abort(saddr_of(tfull), tw & 1, abort) ? 1 : 0;
                r = __shfl_sync(0xffffffffu, r, 0);
                if (!epi_all(r != 0)) {
                    go = false;
                    break;
                }
                asm volatile("tcgen05.fence::after_thread_sync;\n" ::);
                float re[32], im[32];
                tc_ld32(t0, re);
                tc_add16(t0 + 256, re);
                tc_add16(t0 + 256 + 16, re + 16);
                tc_ld32(t0 + 128, im);
                tc_add16(t0 + 384, im);
                tc_add16(t0 + 384 + 16, im + 16);
                asm volatile("tcgen05.fence::before_thread_sync;\n" ::);
                __syncwarp();
                if (lane == 0) mbar_arrive(saddr_of(tempty));
                tw++;
                int tm, tn;
                tri_tile(t, tm, tn);
                const int m0 = tm * kTile, n0 = tn * kTile;
#pragma unroll
                for (int h = 0; h < 2; h++) {
                    epi_sync();   // the staged half of the previous pass has been read
                    if ((cg >> 1) == h) {
                        float2* row = stage_tile + (quarter * 32 + lane) * kEpiPitch + (cg & 1) * 32;
#pragma unroll
                        for (int e = 0; e < 32; e++) row[e] = make_float2(re[e], im[e]);
                    }
                    epi_sync();
#pragma unroll 1
                    for (int idx = tid; idx < kTile * kHalf; idx += kEpiThreads) {
                        const int rr = idx / kHalf, cc = idx - rr * kHalf;
                        const int gr = m0 + rr, gc = n0 + h * kHalf + cc;
                        if (gr < p.L && gc < p.L && gr <= gc) {
                            const float2 v = stage_tile[rr * kEpiPitch + cc];
                            double2* d = p.S + static_cast<long>(gr) * p.L + gc;
                            double2 x = *d;
                            x.x += static_cast<double>(v.x);
                            x.y += static_cast<double>(v.y);
                            *d = x;
                        }
                    }
                }
            }
            if (!go) {
                if (tid == 0) {
                    *abort = 1;
                    atomicExch(p.error, 1);
                }
                break;
            }
        }
    }
    __syncthreads();
    if (warp == kProducerWarp && lane == 0 && *abort) {
        // copies in flight: issued by the producer, not taken by the MMA warp
        for (int g = *consumed_sh; g < issued; g++) mbar_wait(saddr_of(full + g % kRing), (g / kRing) & 1);
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::);
    __syncthreads();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(kTmemCols));
}

int padded_rows(int L) { return (L + kTile - 1) / kTile * kTile; }

}  // namespace

size_t sm_tc_planes_bytes(int L, int count) {
    const size_t stages = static_cast<size_t>((count + kStageSamples - 1) / kStageSamples);
    return stages * (padded_rows(L) / 8) * kPlanes * kGroupBytes;
}

cudaError_t launch_sm_tc_accumulate(const SmSource& a, double2* S, void* planes, int* error, int* launches,
                                    int num_sms, cudaStream_t st) {
    if (a.count <= 0) return cudaSuccess;
    const int Lpad = padded_rows(a.L), RG = Lpad / 8, nt = Lpad / kTile;
    const int G = (a.count + kStageSamples - 1) / kStageSamples;
    if (G > 65535) return cudaErrorInvalidValue;
    cudaError_t e = cudaFuncSetAttribute(sm_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         static_cast<int>(kSmem));
    if (e != cudaSuccess) return e;
    sm_tc_prep_kernel<<<dim3(nt, G), 256, 0, st>>>(a, RG, static_cast<uint4*>(planes));
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    const int ntiles = nt * (nt + 1) / 2;
    TcLaunch p{static_cast<const unsigned char*>(planes), G, RG, a.L, ntiles, S, error};
    sm_tc_kernel<<<std::min(ntiles, std::max(1, num_sms)), kThreads, kSmem, st>>>(p);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    if (launches) *launches += 2;
    return cudaSuccess;
}

}  // namespace rbmg
