// Negacyclic NTT / INTT of one polynomial per thread-block cluster, the
// polynomial held in the cluster's distributed shared memory from its load
// to its store: one launch per transform for small degrees (2^10..2^14),
// where the tiled passes spend most of their time in launch latency.
//
// The transform is hmpc's stage-per-kernel schedule
// (hmpc/expr/number_theoretic_transform.hpp:90-197): forward stage s pairs
// elements e and e + N/2^(s+1) with twiddle T[2^s + (e >> (log N - s))];
// inverse stage s pairs e and e + 2^s with T[N/2^(s+1) + (e >> (s + 1))], its
// last stage scaling by T[0] and T[1].  With 8 CTAs of N/8 elements each:
//  - the three stages on the top three index bits run where a CTA holds, for
//    a slice of low values l, all eight elements (h << (log N - 3)) | l;
//  - the other log N - 3 stages run where CTA h holds the contiguous block
//    h * N/8 .. (h + 1) * N/8 - 1.
// One all-to-all exchange through distributed shared memory moves every
// element between the two layouts (forward: after the top stages; inverse:
// before them).  Each thread applies up to three consecutive stages to eight
// elements in registers (radix 8), with a CTA barrier between rounds inside
// the block layout.  The values are the fully reduced representatives of the
// reference's transform, bit for bit.
#pragma once

#include <cstdint>

#include <cooperative_groups.h>

#include "limbs.cuh"
#include "ntt.cuh"

namespace hmpc_gb300
{
    constexpr int cl_ctas = 8;  // CTAs per cluster (the portable maximum)

    struct ClusterNttParams
    {
        const uint32_t* in;        // limb-planar, `elements` words per plane
        uint32_t* out;             // may equal in
        const uint32_t* twiddles;  // element-major [N][L]
        uint64_t elements;         // batch * N
        uint32_t log_n;            // 10..14
        uint32_t inverse;
    };

    // shared memory of one CTA: two buffers of N/8 elements (element-major),
    // one per layout, so the exchange never writes a buffer still being read,
    // and the CTA's twiddles (N/8 + 7 entries, loaded once at the start)
    template<int L>
    __host__ __device__ constexpr size_t cl_smem_bytes(uint32_t log_n)
    {
        return (3ull * (1ull << (log_n - 3)) + 8ull) * L * sizeof(uint32_t);
    }

    // Shared-memory slot of the twiddle of stage s for the butterfly whose
    // first element is e.  Slots 0..7 hold T[0..7] (the three stages on the
    // top index bits use only these); the stages inside CTA `rank`'s block
    // use 2^(stage's depth) consecutive entries each, stored after them.
    struct ClTwiddles
    {
        uint32_t log_n, inverse;

        // global table index
        __device__ __forceinline__ uint32_t index(uint32_t s, uint32_t e) const
        {
            return inverse ? (1u << (log_n - s - 1)) + (e >> (s + 1)) : (1u << s) + (e >> (log_n - s));
        }

        // slot: top-bit stages map to their index (0..7); block stages to
        // 8 + (2^d - 1) + (index - first index of the stage in this CTA's
        // block), d the number of bits of the index below the block bits
        __device__ __forceinline__ uint32_t slot(uint32_t s, uint32_t e) const
        {
            const uint32_t kb = log_n - 3;
            const bool block = inverse ? s < kb : s >= 3;
            if (!block)
            {
                return index(s, e);
            }
            const uint32_t d = inverse ? kb - s - 1 : s - 3;  // index bits from the local part of e
            return 8u + (1u << d) - 1u + (index(s, e) & ((1u << d) - 1u));
        }
    };

    template<int L>
    __device__ __forceinline__ void cl_twiddle(uint32_t (&t)[L], const uint32_t* tw, uint32_t slot)
    {
#pragma unroll
        for (int j = 0; j < L; ++j)
        {
            t[j] = tw[slot * L + j];
        }
    }

    template<int L>
    __device__ __forceinline__ void cl_butterfly(uint32_t (&u)[L], uint32_t (&v)[L], const ClusterNttParams& p,
                                                 const Modulus<L>& m, uint32_t s, uint32_t e, const uint32_t* tw)
    {
        const ClTwiddles tws{p.log_n, p.inverse};
        uint32_t t[L], x[L];
        if (!p.inverse)
        {
            cl_twiddle<L>(t, tw, tws.slot(s, e));
            mont_mul<L>(v, v, t, m);
            mod_add<L>(x, u, v, m);
            mod_sub<L>(v, u, v, m);
#pragma unroll
            for (int j = 0; j < L; ++j)
            {
                u[j] = x[j];
            }
        }
        else if (s + 1 < p.log_n)
        {
            cl_twiddle<L>(t, tw, tws.slot(s, e));
            uint32_t d[L];
            mod_add<L>(x, u, v, m);
            mod_sub<L>(d, u, v, m);
            mont_mul<L>(v, d, t, m);
#pragma unroll
            for (int j = 0; j < L; ++j)
            {
                u[j] = x[j];
            }
        }
        else
        {
            uint32_t d[L];
            mod_add<L>(x, u, v, m);
            mod_sub<L>(d, u, v, m);
            cl_twiddle<L>(t, tw, 0);
            mont_mul<L>(u, x, t, m);
            cl_twiddle<L>(t, tw, 1);
            mont_mul<L>(v, d, t, m);
        }
    }

    // stages s0 .. s0 + G - 1 on the 2^G elements x[i] at indices e0 + i * dist
    // (index bit `bit0` upwards in the inverse, downwards in the forward)
    template<int L, int G>
    __device__ __forceinline__ void cl_stages(uint32_t (&x)[1 << G][L], const ClusterNttParams& p,
                                              const Modulus<L>& m, uint32_t s0, uint32_t e0, uint32_t bit0,
                                              const uint32_t* tw)
    {
#pragma unroll
        for (int st = 0; st < G; ++st)
        {
            // forward: the first stage pairs on the highest of the G bits
            const int b = p.inverse ? st : G - 1 - st;
#pragma unroll
            for (int i = 0; i < (1 << G); ++i)
            {
                if (i & (1 << b))
                {
                    continue;
                }
                const uint32_t e = e0 + (static_cast<uint32_t>(i) << bit0);
                cl_butterfly<L>(x[i], x[i | (1 << b)], p, m, s0 + static_cast<uint32_t>(st), e, tw);
            }
        }
    }

    template<int L>
    __device__ __forceinline__ void cl_read(uint32_t (&x)[L], const uint32_t* sm, uint32_t local)
    {
#pragma unroll
        for (int j = 0; j < L; ++j)
        {
            x[j] = sm[local * L + j];
        }
    }

    template<int L>
    __device__ __forceinline__ void cl_write(uint32_t* sm, uint32_t local, const uint32_t (&x)[L])
    {
#pragma unroll
        for (int j = 0; j < L; ++j)
        {
            sm[local * L + j] = x[j];
        }
    }

    // One round of G stages inside the block layout (CTA `rank` holds indices
    // rank * B .. rank * B + B - 1): every thread group of 2^G elements whose
    // local indices differ in bits bit0 .. bit0 + G - 1.  Source and sink are
    // the CTA's block buffer or global memory.
    template<int L, int G, bool FromGlobal, bool ToGlobal>
    __device__ __forceinline__ void cl_block_round(const ClusterNttParams& p, const Modulus<L>& m, uint32_t* blk,
                                                   uint32_t rank, uint64_t base, uint32_t s0, uint32_t bit0,
                                                   const uint32_t* tw)
    {
        const uint32_t kb = p.log_n - 3;
        const uint32_t groups = 1u << (kb - G);
        for (uint32_t g = threadIdx.x; g < groups; g += blockDim.x)
        {
            // local index of element 0 of the group: g with G zero bits inserted at bit0
            const uint32_t low = g & ((1u << bit0) - 1u);
            const uint32_t l0 = ((g >> bit0) << (bit0 + G)) | low;
            const uint32_t e0 = (rank << kb) | l0;
            uint32_t x[1 << G][L];
#pragma unroll
            for (int i = 0; i < (1 << G); ++i)
            {
                const uint32_t l = l0 + (static_cast<uint32_t>(i) << bit0);
                if constexpr (FromGlobal)
                {
#pragma unroll
                    for (int j = 0; j < L; ++j)
                    {
                        x[i][j] = p.in[static_cast<uint64_t>(j) * p.elements + base + (rank << kb) + l];
                    }
                }
                else
                {
                    cl_read<L>(x[i], blk, l);
                }
            }
            cl_stages<L, G>(x, p, m, s0, e0, bit0, tw);
#pragma unroll
            for (int i = 0; i < (1 << G); ++i)
            {
                const uint32_t l = l0 + (static_cast<uint32_t>(i) << bit0);
                if constexpr (ToGlobal)
                {
#pragma unroll
                    for (int j = 0; j < L; ++j)
                    {
                        p.out[static_cast<uint64_t>(j) * p.elements + base + (rank << kb) + l] = x[i][j];
                    }
                }
                else
                {
                    cl_write<L>(blk, l, x[i]);
                }
            }
        }
    }

    template<int L>
    __global__ void __cluster_dims__(cl_ctas, 1, 1) __launch_bounds__(256)
        ntt_cluster_kernel(const ClusterNttParams p, const Modulus<L> m)
    {
        namespace cg = cooperative_groups;
        cg::cluster_group cluster = cg::this_cluster();
        extern __shared__ __align__(16) uint32_t cl_smem[];
        const uint32_t k = p.log_n, kb = k - 3;
        const uint32_t B = 1u << kb;          // elements per CTA
        const uint32_t slice = B >> 3;        // low values per CTA in the top-bit layout
        uint32_t* blk = cl_smem;              // block layout: local index l of element (rank << kb) | l
        uint32_t* top = cl_smem + B * L;      // top-bit layout: element (h << kb) | (rank * slice + g) at g * 8 + h
        uint32_t* tw = cl_smem + 2 * B * L;   // twiddle slots (ClTwiddles::slot)
        const uint32_t rank = cluster.block_rank();
        const uint64_t base = static_cast<uint64_t>(blockIdx.x / cl_ctas) << k;
        // the CTA's twiddles: T[0..7], then per block stage its 2^d entries
        // starting at the index of the block's first butterfly
        {
            const ClTwiddles tws{k, p.inverse};
            const uint32_t slots = B + 7u;
            for (uint32_t i = threadIdx.x; i < slots * L; i += blockDim.x)
            {
                const uint32_t sl = i / L, j = i % L;
                uint32_t index = sl;
                if (sl >= 8)
                {
                    // slot 8 + 2^d - 1 + o: depth d, offset o
                    const uint32_t r = sl - 7u;                  // 2^d + o, o < 2^d
                    const uint32_t d = 31u - __clz(r);
                    const uint32_t o = r - (1u << d);
                    const uint32_t s = p.inverse ? kb - 1u - d : d + 3u;
                    index = tws.index(s, rank << kb) + o;
                }
                tw[i] = p.twiddles[static_cast<uint64_t>(index) * L + j];
            }
            __syncthreads();
        }
        // every CTA of the cluster runs before any writes into its shared memory
        cluster.sync();
        if (!p.inverse)
        {
            // stages 0..2 on the top bits, straight from global memory, then each
            // element to the CTA that holds its block
            for (uint32_t g = threadIdx.x; g < slice; g += blockDim.x)
            {
                const uint32_t l = rank * slice + g;
                uint32_t x[8][L];
#pragma unroll
                for (int h = 0; h < 8; ++h)
                {
#pragma unroll
                    for (int j = 0; j < L; ++j)
                    {
                        x[h][j] = p.in[static_cast<uint64_t>(j) * p.elements + base + (static_cast<uint64_t>(h) << kb) + l];
                    }
                }
                cl_stages<L, 3>(x, p, m, 0, l, kb, tw);
#pragma unroll
                for (int h = 0; h < 8; ++h)
                {
                    cl_write<L>(cluster.map_shared_rank(blk, h), l, x[h]);
                }
            }
            cluster.sync();
            // stages 3 .. k - 1 in the block layout, three per round
            uint32_t s = 3;
            while (k - s > 3)
            {
                cl_block_round<L, 3, false, false>(p, m, blk, rank, base, s, k - s - 3, tw);
                __syncthreads();
                s += 3;
            }
            if (k - s == 3)
            {
                cl_block_round<L, 3, false, true>(p, m, blk, rank, base, s, 0, tw);
            }
            else if (k - s == 2)
            {
                cl_block_round<L, 2, false, true>(p, m, blk, rank, base, s, 0, tw);
            }
            else
            {
                cl_block_round<L, 1, false, true>(p, m, blk, rank, base, s, 0, tw);
            }
        }
        else
        {
            // stages 0 .. kb - 1 in the block layout (low bits first), the first
            // round from global memory
            const uint32_t first = kb % 3 ? kb % 3 : 3;
            if (first == 3)
            {
                cl_block_round<L, 3, true, false>(p, m, blk, rank, base, 0, 0, tw);
            }
            else if (first == 2)
            {
                cl_block_round<L, 2, true, false>(p, m, blk, rank, base, 0, 0, tw);
            }
            else
            {
                cl_block_round<L, 1, true, false>(p, m, blk, rank, base, 0, 0, tw);
            }
            for (uint32_t s = first; s < kb; s += 3)
            {
                __syncthreads();
                cl_block_round<L, 3, false, false>(p, m, blk, rank, base, s, s, tw);
            }
            __syncthreads();
            // each element to the CTA that holds its slice of low values
            for (uint32_t l = threadIdx.x; l < B; l += blockDim.x)
            {
                uint32_t x[L];
                cl_read<L>(x, blk, l);
                const uint32_t c = l / slice;
                cl_write<L>(cluster.map_shared_rank(top, c), (l % slice) * 8 + rank, x);
            }
            cluster.sync();
            // stages kb .. k - 1 on the top bits, the last with the scaling
            for (uint32_t g = threadIdx.x; g < slice; g += blockDim.x)
            {
                const uint32_t l = rank * slice + g;
                uint32_t x[8][L];
#pragma unroll
                for (int h = 0; h < 8; ++h)
                {
                    cl_read<L>(x[h], top, g * 8 + h);
                }
                cl_stages<L, 3>(x, p, m, kb, l, kb, tw);
#pragma unroll
                for (int h = 0; h < 8; ++h)
                {
#pragma unroll
                    for (int j = 0; j < L; ++j)
                    {
                        p.out[static_cast<uint64_t>(j) * p.elements + base + (static_cast<uint64_t>(h) << kb) + l] =
                            x[h][j];
                    }
                }
            }
        }
    }
}
