// nsg_tc.cuh -- fifth-generation tensor core (tcgen05) primitives for sm_103a, in
// inline PTX: tensor-memory allocation, the BF16 MMA with FP32 accumulation in
// tensor memory, its completion through an mbarrier, tensor-memory loads, and the
// shared-memory operand descriptors of the canonical no-swizzle K-major layout.
//
// Operand layout (K-major, no swizzle).  A tile of R rows x K bf16 columns is stored
// as core matrices of 8 rows x 16 bytes (8 elements), each 128 contiguous bytes (row
// j of the core at +16 j).  Core (row group g, column group c) sits at
//     (c * (R / 8) + g) * 128
// so cores adjacent along K are R/8 * 128 bytes apart (the descriptor's leading
// byte offset) and cores adjacent along the rows 128 bytes apart (its stride byte
// offset).  One MMA of kind::f16 consumes K = 16, two column groups; the k-th MMA of
// a chain starts at column group 2k.
#pragma once
#include <cstdint>

#if defined(__CUDACC__)
#define NSG_TC_HD __host__ __device__
#else
#define NSG_TC_HD
#endif

namespace nsg {

// byte offset of element (row, k) in an R-row tile of the layout above
NSG_TC_HD constexpr uint32_t tc_offset(uint32_t R, uint32_t row, uint32_t k)
{
    return ((k / 8) * (R / 8) + row / 8) * 128 + (row % 8) * 16 + (k % 8) * 2;
}

// leading (K) and stride (row) byte offsets of an R-row tile
NSG_TC_HD constexpr uint32_t tc_lbo(uint32_t R) { return (R / 8) * 128; }
constexpr uint32_t kTcSbo = 128;

// Shared-memory matrix descriptor: start address, leading and stride byte offsets
// (all >> 4), descriptor version 1 (bits 46-47), base offset 0, layout type 0 (no
// swizzle, bits 61-63).
NSG_TC_HD constexpr uint64_t tc_smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo)
{
    return (uint64_t)((saddr >> 4) & 0x3fffu) | ((uint64_t)((lbo >> 4) & 0x3fffu) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3fffu) << 32) | (1ull << 46);
}

// Instruction descriptor of kind::f16: D in FP32 (bits 4-5 = 1), A and B in BF16
// (bits 7-9 = 1, 10-12 = 1), both K-major (bits 15, 16 = 0), N >> 3 in bits 17-22,
// M >> 4 in bits 24-28.
NSG_TC_HD constexpr uint32_t tc_idesc_bf16(uint32_t M, uint32_t N)
{
    return (1u << 4) | (1u << 7) | (1u << 10) | ((N >> 3) << 17) | ((M >> 4) << 24);
}

#if defined(__CUDACC__)
__device__ __forceinline__ uint32_t smem_u32(const void *p)
{
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// Tensor memory: ncols columns (a power of two >= 32) for this CTA; the address is
// written to *slot (shared memory).  One full warp calls alloc and, later, dealloc.
__device__ __forceinline__ void tc_alloc(uint32_t slot_saddr, uint32_t ncols)
{
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(slot_saddr), "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tc_dealloc(uint32_t taddr, uint32_t ncols)
{
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
// generic-proxy shared-memory writes made visible to the tensor core's (async) proxy
__device__ __forceinline__ void tc_fence_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// D[tmem] (+)= A[smem] * B[smem]^T, issued by one thread.
__device__ __forceinline__ void tc_mma_bf16(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                            uint32_t accumulate)
{
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem_d),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
        : "memory");
}

// The mbarrier at bar_saddr receives one arrival when every MMA this thread issued
// before has completed.
__device__ __forceinline__ void tc_commit(uint32_t bar_saddr)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar_saddr)
                 : "memory");
}

// Initialises the mbarrier and makes the initialisation visible to the tensor core's
// arrivals (followed by a CTA barrier before first use).
__device__ __forceinline__ void mbar_init(uint32_t bar_saddr, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar_saddr), "r"(count) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint32_t bar_saddr, uint32_t parity)
{
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(ok)
        : "r"(bar_saddr), "r"(parity)
        : "memory");
    return ok != 0u;
}

// Waits for the phase with the given parity to complete, at most `limit` polls;
// returns false if it gave up.
__device__ __forceinline__ bool mbar_wait_bounded(uint32_t bar_saddr, uint32_t parity, uint32_t limit)
{
    for (uint32_t i = 0; i < limit; i++)
        if (mbar_try_wait(bar_saddr, parity)) return true;
    return false;
}

// 16 consecutive FP32 columns of this thread's tensor-memory lane (shape 32x32b:
// thread l of warp w reads lane 32 (w % 4) + l).
__device__ __forceinline__ void tc_ld16(uint32_t taddr, float (&v)[16])
{
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr)
        : "memory");
#pragma unroll
    for (int i = 0; i < 16; i++) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ void tc_ld8(uint32_t taddr, float (&v)[8])
{
    uint32_t r[8];
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
                 : "r"(taddr)
                 : "memory");
#pragma unroll
    for (int i = 0; i < 8; i++) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ void tc_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }
#endif  // __CUDACC__

}  // namespace nsg
