// tcgen05.cuh -- the fifth-generation tensor-core instructions of sm_100/sm_103 (tcgen05.*) as inline
// PTX, for the kernels that put their dense contractions on the tensor cores.
//
// Model: one thread issues tcgen05.mma; its operands A (M x K) and B (N x K) sit in shared memory in
// the canonical K-major layout without swizzle, and its FP32 accumulator D (M x N) lives in tensor
// memory (TMEM: 128 lanes x 512 columns of 32 bits per SM; row i of D in lane i, column j in column
// base + j for M = 128). tcgen05.commit makes an mbarrier track completion of the issued MMAs;
// warps then read D back with tcgen05.ld, each warp from the 32-lane quarter (warp id mod 4) it may
// access.
//
// Canonical K-major layout without swizzle: the operand is tiled into core matrices of 8 rows x 16
// bytes (4 FP32/TF32 values of K), each stored as 128 contiguous bytes (row-major); the descriptor's
// leading-dimension byte offset (LBO) steps between core matrices adjacent in K, the stride-dimension
// byte offset (SBO) between core matrices adjacent in M (or N). The layout used here stores, for each
// group g of 4 consecutive K, all rows contiguously: element (r, k) at byte
//   (k / 4) * rows * 16 + r * 16 + (k % 4) * 4,
// so that LBO = rows * 16 and SBO = 128, and a sub-block of rows starting at a multiple of 8 is the
// same descriptor with its start address moved by 16 bytes per row.
#pragma once

#include <cstdint>

namespace uepm {
namespace tc {

__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// Shared memory matrix descriptor (64 bits): start address >> 4 in bits 0-13, LBO >> 4 in 16-29,
// SBO >> 4 in 32-45, the fixed descriptor version 1 in bits 46-48, base offset 0, swizzle mode 0
// (none) in bits 61-63.
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((saddr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

// Instruction descriptor of kind::tf32 (32 bits): D format F32 (1) in bits 4-5, A and B format TF32
// (2) in bits 7-9 and 10-12, both K-major (bits 15, 16 clear), N >> 3 in bits 17-22, M >> 4 in
// bits 24-28; dense, no negation.
__host__ __device__ constexpr uint32_t idesc_tf32(int M, int N) {
    return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

// Instruction descriptor of kind::f16 with BF16 A and B (format 1) and an F32 accumulator.
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

// TF32 value of x rounded to nearest (ties away), as an FP32 bit pattern with the low 13 bits clear.
__device__ __forceinline__ float to_tf32(float x) {
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
    return __uint_as_float(r);
}

// ---- TMEM allocation (one whole warp executes these) ---------------------------------------------
__device__ __forceinline__ void tmem_alloc(uint32_t* dst_smem, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(dst_smem)),
                 "r"(ncols)
                 : "memory");
}
__device__ __forceinline__ void tmem_relinquish() {
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

// ---- ordering ------------------------------------------------------------------------------------
__device__ __forceinline__ void fence_before_sync() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after_sync() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
// generic-proxy writes to shared memory made visible to the tensor core (async proxy)
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// ---- MMA -----------------------------------------------------------------------------------------
// D (TMEM) = A B^T (+ D when accumulate), cta_group::1, kind::tf32; issued by one thread
__device__ __forceinline__ void mma_tf32(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc, uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
        : "memory");
}
// D (TMEM) = A B^T (+ D when accumulate), cta_group::1, kind::f16 (BF16 operands by the descriptor)
__device__ __forceinline__ void mma_f16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc, uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
        : "memory");
}
// the mbarrier at bar (shared memory) completes a phase when every MMA issued so far by this thread
// has completed
__device__ __forceinline__ void mma_commit(uint64_t* bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_addr(bar))
                 : "memory");
}

// ---- mbarrier ------------------------------------------------------------------------------------
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return done != 0;
}
// waits for the phase of the given parity to complete, at most max_tries polls; false if it gave up
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity, uint32_t max_tries) {
    for (uint32_t t = 0; t < max_tries; ++t)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}

// arrive (release, CTA scope) on the mbarrier at bar
__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
    asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.shared::cta.b64 st, [%0];\n\t}" ::"r"(smem_addr(bar)) : "memory");
}

// ---- TMEM -> registers ---------------------------------------------------------------------------
// 8 consecutive columns of this thread's lane, load and wait in one statement (see tmem_ld16)
__device__ __forceinline__ void tmem_ld8(uint32_t taddr, float (&v)[8]) {
    uint32_t r[8];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];\n\t"
        "tcgen05.wait::ld.sync.aligned;"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
        : "r"(taddr)
        : "memory");
#pragma unroll
    for (int i = 0; i < 8; ++i) v[i] = __uint_as_float(r[i]);
}
// 16 consecutive columns of this thread's lane (32x32b shape: lane = the warp's quarter base + lane
// id). The load and its wait are one asm statement, so no use of the values can be scheduled before
// the wait.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n\t"
        "tcgen05.wait::ld.sync.aligned;"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
          "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr)
        : "memory");
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

// three 8-column loads (at a, b, c) and one wait, in one statement
__device__ __forceinline__ void tmem_ld8x3(uint32_t a, uint32_t b, uint32_t c, float (&va)[8], float (&vb)[8],
                                           float (&vc)[8]) {
    uint32_t r[24];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%24];\n\t"
        "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%8,%9,%10,%11,%12,%13,%14,%15}, [%25];\n\t"
        "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%16,%17,%18,%19,%20,%21,%22,%23}, [%26];\n\t"
        "tcgen05.wait::ld.sync.aligned;"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
          "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]),
          "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23])
        : "r"(a), "r"(b), "r"(c)
        : "memory");
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        va[i] = __uint_as_float(r[i]);
        vb[i] = __uint_as_float(r[8 + i]);
        vc[i] = __uint_as_float(r[16 + i]);
    }
}

}  // namespace tc
}  // namespace uepm
