// Inline-PTX helpers for the 5th-generation tensor cores (tcgen05): shared-memory
// matrix descriptors for the no-swizzle K-major canonical layout, kind::f16 MMAs with
// BF16 operands and FP32 accumulation in TMEM, commits to an mbarrier, bounded waits,
// TMEM loads and the split of FP32 values into BF16 hi + lo operand rows.
//
// Canonical layout of an R x K BF16 operand (K-major, no swizzle): 8 x 8 core matrices
// of 128 bytes; element (r, k) sits at ((r/8) * (K/8) + k/8) * 64 + (r%8) * 8 + k%8;
// core matrices adjacent in K are LBO = 128 bytes apart, in R SBO = (K/8) * 128 bytes.
#pragma once

#include <cuda_bf16.h>
#include <stdint.h>

namespace nnapgb {
namespace tc {

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ uint64_t make_desc(uint32_t saddr, int K) {
    const uint64_t lbo = 128, sbo = (uint64_t)(K >> 3) * 128;
    uint64_t d = 0;
    d |= (uint64_t)((saddr >> 4) & 0x3FFF);
    d |= (uint64_t)((lbo >> 4) & 0x3FFF) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFF) << 32;
    d |= (uint64_t)1 << 46;  // descriptor version for this architecture
    return d;                // base offset 0, layout type 0 (no swizzle)
}

// kind::f16 instruction descriptor: D = F32, A = B = BF16, both K-major, M = 128.
__device__ __forceinline__ uint32_t make_idesc(int N) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(128 >> 4) << 24);
}

__device__ __forceinline__ void mma_bf16(uint32_t tmem_d, uint64_t da, uint64_t db, uint32_t idesc, uint32_t acc) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem_d),
        "l"(da), "l"(db), "r"(idesc), "r"(acc));
}

__device__ __forceinline__ void mma_commit(uint32_t mbar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar) : "memory");
}

__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// Bounded wait on an mbarrier phase: gives up after ~2 s of device time.
__device__ __forceinline__ bool mbar_wait(uint32_t mbar, uint32_t phase) {
    const long long t0 = clock64();
    for (;;) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}\n"
            : "=r"(done)
            : "r"(mbar), "r"(phase)
            : "memory");
        if (done) return true;
        if (clock64() - t0 > 4000000000LL) return false;
    }
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* v) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int q = 0; q < 16; ++q) v[q] = __uint_as_float(r[q]);
}

// Split 8 FP32 values into BF16 hi/lo and store one 16-byte core-matrix row each.
__device__ __forceinline__ void store_split8(uint8_t* hi_base, uint8_t* lo_base, int row, int k0, int K,
                                             const float* v) {
    uint32_t h[4], l[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const __nv_bfloat16 h0 = __float2bfloat16_rn(v[2 * q]), h1 = __float2bfloat16_rn(v[2 * q + 1]);
        const __nv_bfloat16 l0 = __float2bfloat16_rn(v[2 * q] - __bfloat162float(h0));
        const __nv_bfloat16 l1 = __float2bfloat16_rn(v[2 * q + 1] - __bfloat162float(h1));
        h[q] = (uint32_t)__bfloat16_as_ushort(h0) | ((uint32_t)__bfloat16_as_ushort(h1) << 16);
        l[q] = (uint32_t)__bfloat16_as_ushort(l0) | ((uint32_t)__bfloat16_as_ushort(l1) << 16);
    }
    const size_t off = (((size_t)(row >> 3) * (K >> 3) + (k0 >> 3)) * 64 + (row & 7) * 8) * 2;
    *reinterpret_cast<uint4*>(hi_base + off) = make_uint4(h[0], h[1], h[2], h[3]);
    *reinterpret_cast<uint4*>(lo_base + off) = make_uint4(l[0], l[1], l[2], l[3]);
}

// Issue one split-BF16 GEMM: D[128 x N] (+)= A[128 x K] * B[N x K]^T.
__device__ __forceinline__ void issue_gemm(uint32_t tmem_d, uint32_t a_hi, uint32_t a_lo, uint32_t b_hi, uint32_t b_lo,
                                           int K, int N) {
    const uint32_t idesc = make_idesc(N);
    for (int ks = 0; ks < K / 16; ++ks) {
        const uint32_t step = ks * 256;  // two core matrices along K
        const uint64_t ah = make_desc(a_hi + step, K), al = make_desc(a_lo + step, K);
        const uint64_t bh = make_desc(b_hi + step, K), bl = make_desc(b_lo + step, K);
        mma_bf16(tmem_d, ah, bh, idesc, ks > 0 ? 1u : 0u);
        mma_bf16(tmem_d, al, bh, idesc, 1u);
        mma_bf16(tmem_d, ah, bl, idesc, 1u);
    }
}

}  // namespace tc
}  // namespace nnapgb
