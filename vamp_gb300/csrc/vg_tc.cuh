// 5th-generation tensor core (tcgen05) building blocks for sm_103a: shared-memory operand
// descriptors, the instruction descriptor for BF16 x BF16 -> FP32, TMEM allocation, MMA issue,
// commit to an mbarrier with a bounded wait, and TMEM -> register loads.
//
// Operand layout: no swizzle, K-major.  A tile of R rows x KC columns (bf16) is stored as 8x8
// "core matrices" of 128 bytes (8 rows of 16 bytes); core matrices adjacent in K are 128 bytes
// apart (the descriptor's leading-dimension byte offset) and 8-row groups are KC / 8 * 128 bytes
// apart (its stride byte offset).  Either reading of those two offsets stays inside the tile.
#pragma once

#include <cstdint>

namespace vg::tc
{
    // Byte offset of element (r, k) in a K-major, no-swizzle tile with KC columns.
    __host__ __device__ constexpr uint32_t tile_offset(uint32_t r, uint32_t k, uint32_t KC)
    {
        return ((r >> 3) * (KC >> 3) + (k >> 3)) * 128u + (r & 7u) * 16u + (k & 7u) * 2u;
    }

    // Shared-memory matrix descriptor (sm_100 family): start address, leading-dimension byte
    // offset (between core matrices adjacent in K), stride byte offset (between core matrices
    // adjacent in M/N), descriptor version 1, no swizzle.
    __device__ __forceinline__ uint64_t smem_desc(uint32_t smem_addr, uint32_t lbo, uint32_t sbo)
    {
        uint64_t d = 0;
        d |= static_cast<uint64_t>((smem_addr >> 4) & 0x3fffu);
        d |= static_cast<uint64_t>((lbo >> 4) & 0x3fffu) << 16;
        d |= static_cast<uint64_t>((sbo >> 4) & 0x3fffu) << 32;
        d |= static_cast<uint64_t>(1u) << 46;  // version
        // base offset 0, leading-byte-offset mode 0, layout type 0 (no swizzle)
        return d;
    }

    // Instruction descriptor for tcgen05.mma.kind::f16 with BF16 A and B, FP32 D, both operands
    // K-major, no negation, dense.
    __host__ __device__ constexpr uint32_t idesc_bf16_f32(uint32_t M, uint32_t N)
    {
        return (1u << 4)            // D format: F32
               | (1u << 7)          // A format: BF16
               | (1u << 10)         // B format: BF16
               | ((N >> 3) << 17)   // N / 8
               | ((M >> 4) << 24);  // M / 16
    }

    __device__ __forceinline__ uint32_t smem_u32(const void *p)
    {
        return static_cast<uint32_t>(__cvta_generic_to_shared(p));
    }

    // TMEM allocation of `cols` columns (power of two >= 32) by one whole warp; the address is
    // written to *slot in shared memory.
    __device__ __forceinline__ void tmem_alloc(uint32_t *slot, uint32_t cols)
    {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(slot)), "r"(cols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }

    __device__ __forceinline__ void tmem_free(uint32_t taddr, uint32_t cols)
    {
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(cols) : "memory");
    }

    __device__ __forceinline__ void fence_before_sync()
    {
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    }

    __device__ __forceinline__ void fence_after_sync()
    {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    }

    // Makes this thread's generic-proxy shared-memory writes visible to the tensor core's reads.
    __device__ __forceinline__ void fence_smem_to_async()
    {
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }

    __device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count)
    {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }

    // D (TMEM) [+]= A (smem) * B (smem)^T, one instruction of K = 16; issued by one thread.
    __device__ __forceinline__ void mma_bf16(uint32_t tmem_d, uint64_t a_desc, uint64_t b_desc, uint32_t idesc, bool accumulate)
    {
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "setp.ne.b32 p, %4, 0;\n\t"
            "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem_d),
            "l"(a_desc), "l"(b_desc), "r"(idesc), "r"(accumulate ? 1u : 0u)
            : "memory");
    }

    // Arrives on *bar once every MMA this thread issued before has completed.
    __device__ __forceinline__ void mma_commit(uint64_t *bar)
    {
        asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                     : "memory");
    }

    // Waits for the mbarrier phase `parity` to complete; gives up after `limit` polls and
    // returns false.
    __device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity, uint32_t limit)
    {
        const uint32_t addr = smem_u32(bar);
        for (uint32_t i = 0; i < limit; ++i)
        {
            uint32_t done;
            asm volatile(
                "{\n\t.reg .pred p;\n\t"
                "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                "selp.u32 %0, 1, 0, p;\n\t}"
                : "=r"(done)
                : "r"(addr), "r"(parity)
                : "memory");
            if (done)
            {
                return true;
            }
        }
        return false;
    }

    // 32 consecutive FP32 accumulator columns of this thread's TMEM lane (warp w of the CTA reads
    // lanes 32 (w % 4) .. 32 (w % 4) + 31).
    __device__ __forceinline__ void tmem_load32(uint32_t taddr, float *v)
    {
        uint32_t r[32];
        asm volatile(
            "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
            "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, "
            "%16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
            : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
              "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
              "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
              "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
            : "r"(taddr)
            : "memory");
        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
        for (int i = 0; i < 32; ++i)
        {
            v[i] = __uint_as_float(r[i]);
        }
    }
}  // namespace vg::tc
