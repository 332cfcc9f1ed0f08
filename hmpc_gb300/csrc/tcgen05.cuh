// Inline-PTX wrappers for the Blackwell (sm_100a / sm_103a) tensor-core path:
// tensor-memory allocation, tcgen05.mma of kind::f16 with shared-memory
// operand descriptors, commits to mbarriers, tensor-memory loads, the
// untiled bulk copy (cp.async.bulk) and bounded mbarrier waits.
//
// Shared-memory operands use the no-swizzle K-major canonical layout: a core
// matrix is 8 rows x 16 bytes (8 fp16) stored contiguously; core matrices
// adjacent along M/N are SBO = 128 bytes apart and those adjacent along K are
// LBO bytes apart (LBO = rows / 8 * 128 for a tile stored K-segment-major).
#pragma once

#include <cstdint>

namespace hmpc_gb300::tc
{
    __device__ __forceinline__ uint32_t smem_u32(const void* p)
    {
        return static_cast<uint32_t>(__cvta_generic_to_shared(p));
    }

    // byte offset of (row, k) of a K-major no-swizzle operand with `rows` rows
    __host__ __device__ __forceinline__ uint32_t operand_offset(uint32_t row, uint32_t k, uint32_t rows)
    {
        return (k >> 3) * (rows / 8u * 128u) + (row >> 3) * 128u + (row & 7u) * 16u + (k & 7u) * 2u;
    }

    // 64-bit shared-memory matrix descriptor (no swizzle, descriptor version 1)
    __device__ __forceinline__ uint64_t smem_descriptor(uint32_t addr, uint32_t lbo, uint32_t sbo)
    {
        uint64_t d = static_cast<uint64_t>((addr & 0x3FFFFu) >> 4);
        d |= static_cast<uint64_t>((lbo >> 4) & 0x3FFFu) << 16;
        d |= static_cast<uint64_t>((sbo >> 4) & 0x3FFFu) << 32;
        d |= static_cast<uint64_t>(1) << 46;
        return d;
    }

    // instruction descriptor of kind::f16: fp16 A and B (K-major), f32 D
    __host__ __device__ constexpr uint32_t f16_instr_descriptor(uint32_t m, uint32_t n)
    {
        return (1u << 4) | ((n >> 3) << 17) | ((m >> 4) << 24);
    }

    __device__ __forceinline__ void tmem_alloc(uint32_t* slot, uint32_t columns)
    {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(slot)),
                     "r"(columns)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }

    __device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t columns)
    {
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(columns) : "memory");
    }

    __device__ __forceinline__ void fence_before_sync()
    {
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    }

    __device__ __forceinline__ void fence_after_sync()
    {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    }

    // make generic-proxy shared-memory writes visible to the tensor core / bulk copies
    __device__ __forceinline__ void fence_proxy_async()
    {
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }

    __device__ __forceinline__ void mma_f16(uint32_t d_tmem, uint64_t a_desc, uint64_t b_desc, uint32_t idesc,
                                            bool accumulate)
    {
        asm volatile(
            "{\n .reg .pred p;\n setp.ne.u32 p, %4, 0;\n"
            " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
            "l"(a_desc), "l"(b_desc), "r"(idesc), "r"(accumulate ? 1u : 0u)
            : "memory");
    }

    // arrive on the mbarrier once every previously issued tcgen05.mma of this thread completed
    __device__ __forceinline__ void mma_commit(uint64_t* bar)
    {
        asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                         smem_u32(bar))
                     : "memory");
    }

    __device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count)
    {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
    }

    __device__ __forceinline__ void mbar_init_fence()
    {
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }

    __device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes)
    {
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                     : "memory");
    }

    __device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity)
    {
        uint32_t done;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done)
            : "r"(smem_u32(bar)), "r"(parity)
            : "memory");
        return done != 0;
    }

    // as mbar_try_wait, but a thread whose phase is not complete may sleep up
    // to `ns` nanoseconds (waking when the phase completes) instead of
    // returning at once: waiting warps leave the issue slots to working ones
    __device__ __forceinline__ bool mbar_try_wait_sleep(uint64_t* bar, uint32_t parity, uint32_t ns)
    {
        uint32_t done;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done)
            : "r"(smem_u32(bar)), "r"(parity), "r"(ns)
            : "memory");
        return done != 0;
    }

    // bounded wait for the phase `parity` of an mbarrier; false when the limit ran out
    __device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, uint32_t limit)
    {
        for (uint32_t i = 0; i < limit; ++i)
        {
            if (mbar_try_wait(bar, parity))
            {
                return true;
            }
        }
        return false;
    }

    // bounded wait of at most limit polls of up to ns nanoseconds each
    __device__ __forceinline__ bool mbar_wait_sleep(uint64_t* bar, uint32_t parity, uint32_t limit,
                                                    uint32_t ns = 1000u)
    {
        for (uint32_t i = 0; i < limit; ++i)
        {
            if (mbar_try_wait_sleep(bar, parity, ns))
            {
                return true;
            }
        }
        return false;
    }

    // global -> shared bulk copy completing on an mbarrier (16-byte aligned, size multiple of 16)
    __device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar)
    {
        asm volatile(
            "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                smem_u32(dst)),
            "l"(src), "r"(bytes), "r"(smem_u32(bar))
            : "memory");
    }

    // 32 lanes x 32-bit, N consecutive columns per thread
    template<int N>
    __device__ __forceinline__ void tmem_load(uint32_t taddr, uint32_t (&r)[N]);

    template<>
    __device__ __forceinline__ void tmem_load<32>(uint32_t taddr, uint32_t (&r)[32])
    {
        asm volatile(
            "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
            "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
            : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
              "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
              "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]),
              "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]),
              "=r"(r[30]), "=r"(r[31])
            : "r"(taddr));
    }

    template<>
    __device__ __forceinline__ void tmem_load<16>(uint32_t taddr, uint32_t (&r)[16])
    {
        asm volatile(
            "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
            : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
              "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
            : "r"(taddr));
    }

    template<>
    __device__ __forceinline__ void tmem_load<8>(uint32_t taddr, uint32_t (&r)[8])
    {
        asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                     : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
                       "=r"(r[7])
                     : "r"(taddr));
    }

    template<>
    __device__ __forceinline__ void tmem_load<4>(uint32_t taddr, uint32_t (&r)[4])
    {
        asm volatile("tcgen05.ld.sync.aligned.32x32b.x4.b32 {%0,%1,%2,%3}, [%4];"
                     : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
                     : "r"(taddr));
    }

    __device__ __forceinline__ void tmem_load_wait()
    {
        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
    }
}
