// Fifth-generation tensor-core (tcgen05) building blocks for sm_103a, as inline PTX.
//
// Operands live in shared memory in the K-major, 128-byte-swizzled layout:
//   * a row (one M or N index) holds 64 consecutive K elements of 16 bits = 128 B;
//   * rows are 128 B apart, so 8 rows form a 1024-byte swizzle atom and the atoms
//     of consecutive 8-row groups are 1024 B apart (the descriptor's stride offset);
//   * inside a row, the 16-byte chunk j (K elements 8j .. 8j+7) is stored at chunk
//     position j ^ (row mod 8).
// An operand region must start on a 1024-byte boundary.  One MMA consumes K = 16
// (32 bytes of each row); the K-steps inside the 128-byte row are addressed by
// moving the descriptor's start address by 32 bytes.
//
// Accumulators (FP32) live in tensor memory: row m of a 128-row tile is TMEM lane m,
// column n is TMEM column base + n.  Warp w of a CTA reads lanes 32*(w%4) .. +31.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace msosm {
namespace umma {

__device__ __forceinline__ uint32_t smem_addr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

// Byte offset of K element k (a multiple of 4 for 8-byte stores, of 8 for 16-byte
// stores) of row r inside a K-major 128-byte-swizzled operand.
__host__ __device__ __forceinline__ uint32_t sw128_offset(int r, int k)
{
    return (uint32_t)(r * 128 + ((((k >> 3) ^ (r & 7)) & 7) << 4) + ((k & 7) << 1));
}

// Shared-memory matrix descriptor of a K-major 128-byte-swizzled operand whose
// first row starts at shared address `saddr` (plus a K offset of a multiple of 32 B).
__device__ __forceinline__ uint64_t desc_sw128(uint32_t saddr)
{
    return (uint64_t)((saddr & 0x3FFFFu) >> 4)   // start address, 16-byte units
           | ((uint64_t)1u << 16)                // leading byte offset (unused inside one atom)
           | ((uint64_t)(1024u >> 4) << 32)      // stride byte offset: 8 rows x 128 B
           | ((uint64_t)1u << 46)                // descriptor version of tcgen05
           | ((uint64_t)2u << 61);               // 128-byte swizzle
}

// Instruction descriptor of kind::f16 with FP32 accumulation, both operands
// K-major: A and B both FP16 (bf16 = false) or both BF16 (bf16 = true).
__host__ __device__ constexpr uint32_t idesc_f16(int M, int N, bool bf16)
{
    return (1u << 4)                         // D format: F32
           | ((bf16 ? 1u : 0u) << 7)         // A format
           | ((bf16 ? 1u : 0u) << 10)        // B format
           | ((uint32_t)(N >> 3) << 17)      // N / 8
           | ((uint32_t)(M >> 4) << 24);     // M / 16
}

// D[tmem] (+)= A[smem] x B[smem]^T, issued by one thread.
__device__ __forceinline__ void mma_f16(uint32_t d_tmem, uint64_t a_desc, uint64_t b_desc, uint32_t idesc,
                                        uint32_t accumulate)
{
    asm volatile("{\n\t.reg .pred p;\n\t"
                 "setp.ne.b32 p, %4, 0;\n\t"
                 "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}"
                 :
                 : "r"(d_tmem), "l"(a_desc), "l"(b_desc), "r"(idesc), "r"(accumulate)
                 : "memory");
}

// The mbarrier at `mbar` completes a phase when every tcgen05 operation this
// thread issued before has finished (its shared-memory reads included).
__device__ __forceinline__ void commit(uint64_t *mbar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                     smem_addr(mbar))
                 : "memory");
}

__device__ __forceinline__ void fence_before_sync() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after_sync() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
// Generic-proxy shared-memory writes made visible to the tensor core's (async) reads.
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// Whole warp: allocate `ncols` TMEM columns (a power of two >= 32); the base address
// is written to *dst (shared memory).  Then give up the right to allocate again.
__device__ __forceinline__ void tmem_alloc(uint32_t *dst, uint32_t ncols)
{
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(dst)), "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
// Whole warp (the allocating one).
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols)
{
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

__device__ __forceinline__ void mbar_init(uint64_t *mbar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(mbar)), "r"(count) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// Suspends the thread until the phase completes or about suspend_ns pass.
__device__ __forceinline__ bool mbar_try_wait(uint64_t *mbar, uint32_t parity, uint32_t suspend_ns = 20000)
{
    uint32_t ok;
    asm volatile("{\n\t.reg .pred p;\n\t"
                 "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\t"
                 "selp.u32 %0, 1, 0, p;\n\t}"
                 : "=r"(ok)
                 : "r"(smem_addr(mbar)), "r"(parity), "r"(suspend_ns)
                 : "memory");
    return ok != 0;
}

__device__ __forceinline__ uint64_t globaltimer_ns()
{
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Wait for phase `parity` of the mbarrier to complete, for at most timeout_ns.
__device__ __forceinline__ bool mbar_wait(uint64_t *mbar, uint32_t parity, unsigned long long timeout_ns)
{
    if (mbar_try_wait(mbar, parity))
        return true;
    const uint64_t t0 = globaltimer_ns();
    while (!mbar_try_wait(mbar, parity))
    {
        if (globaltimer_ns() - t0 > timeout_ns)
            return false;
    }
    return true;
}

// 32 lanes x 32 consecutive FP32 columns starting at taddr (lane field = the warp's
// quarter): this thread's lane, columns col .. col+31.  Waits for the load.
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float (&v)[32])
{
    uint32_t r[32];
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x32.b32 "
                 "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, "
                 "%16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];\n\t"
                 "tcgen05.wait::ld.sync.aligned;"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
                   "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]),
                   "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]),
                   "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]),
                   "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
                 : "r"(taddr)
                 : "memory");
#pragma unroll
    for (int i = 0; i < 32; i++)
        v[i] = __uint_as_float(r[i]);
}

// 32 lanes x 16 consecutive FP32 columns.  Waits for the load.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16])
{
    uint32_t r[16];
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 "
                 "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, [%16];\n\t"
                 "tcgen05.wait::ld.sync.aligned;"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
                   "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]),
                   "=r"(r[15])
                 : "r"(taddr)
                 : "memory");
#pragma unroll
    for (int i = 0; i < 16; i++)
        v[i] = __uint_as_float(r[i]);
}

} // namespace umma
} // namespace msosm
