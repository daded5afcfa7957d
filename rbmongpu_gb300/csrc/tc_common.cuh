// tcgen05 building blocks shared by the tensor-core kernels (mlp_tc.cu, angles_tc.cu):
// the canonical K-major no-swizzle operand layout of BF16 operands, shared-memory and
// instruction descriptors, the MMA / commit / TMEM-load instructions, bounded mbarrier
// waits and bulk copies into shared memory.
#pragma once

#include <cstdint>
#include <cuda_bf16.h>

namespace rbmg {
namespace tc {

constexpr uint32_t kTcSpin = 1u << 24;     // mbarrier polls before giving up

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
__device__ __forceinline__ uint32_t instr_desc(int m, int n) {
    return (1u << 4) | (1u << 7) | (1u << 10) | (static_cast<uint32_t>(n >> 3) << 17) |
           (static_cast<uint32_t>(m >> 4) << 24);
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

// bulk copy of `bytes` (a multiple of 16) from global memory into shared memory,
// completing on the mbarrier (which expects the bytes first)
__device__ __forceinline__ void bulk_g2s(uint32_t dst, const void* src, uint32_t bytes, uint32_t mbar) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(mbar), "r"(bytes) : "memory");
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n" ::"r"(
                     dst),
                 "l"(src), "r"(bytes), "r"(mbar)
                 : "memory");
}

// eight consecutive accumulator columns of this warp's 32 TMEM lanes
__device__ __forceinline__ void tc_ld8(uint32_t taddr, float (&v)[8]) {
    uint32_t r[8];
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];\n"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
                 : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
#pragma unroll
    for (int i = 0; i < 8; i++) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
    const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<const uint32_t*>(&v);
}

}  // namespace tc
}  // namespace rbmg
