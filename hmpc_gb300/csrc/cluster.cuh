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
// before them).  Every stage is one radix-2 butterfly per thread on shared
// memory with a CTA barrier after it, so all of a CTA's threads take part
// in every stage; the twiddles a CTA needs are preloaded into shared memory.
// The values are the fully reduced representatives of the reference's
// transform, bit for bit.
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

    // index i with a zero bit inserted at position b
    __device__ __forceinline__ uint32_t cl_spread(uint32_t i, uint32_t b)
    {
        return ((i >> b) << (b + 1)) | (i & ((1u << b) - 1u));
    }

    // One stage on the block layout (CTA `rank` holds elements (rank << kb) | l
    // at local index l): butterflies on local index bit `bit`, one per thread
    // and pass, then a CTA barrier.
    template<int L>
    __device__ __forceinline__ void cl_block_stage(const ClusterNttParams& p, const Modulus<L>& m, uint32_t* blk,
                                                   uint32_t rank, uint32_t s, uint32_t bit, const uint32_t* tw)
    {
        const uint32_t kb = p.log_n - 3;
        for (uint32_t t = threadIdx.x; t < (1u << (kb - 1)); t += blockDim.x)
        {
            const uint32_t lu = cl_spread(t, bit);
            const uint32_t lv = lu | (1u << bit);
            uint32_t u[L], v[L];
            cl_read<L>(u, blk, lu);
            cl_read<L>(v, blk, lv);
            cl_butterfly<L>(u, v, p, m, s, (rank << kb) | lu, tw);
            cl_write<L>(blk, lu, u);
            cl_write<L>(blk, lv, v);
        }
        __syncthreads();
    }

    // One stage on the top-bit layout (element (h << kb) | (rank * slice + g)
    // at local index g * 8 + h): butterflies on bit `hb` of h.
    template<int L>
    __device__ __forceinline__ void cl_top_stage(const ClusterNttParams& p, const Modulus<L>& m, uint32_t* top,
                                                 uint32_t rank, uint32_t s, uint32_t hb, const uint32_t* tw)
    {
        const uint32_t kb = p.log_n - 3;
        const uint32_t slice = 1u << (kb - 3);
        for (uint32_t t = threadIdx.x; t < slice * 4u; t += blockDim.x)
        {
            const uint32_t g = t >> 2;
            const uint32_t hu = cl_spread(t & 3u, hb);
            const uint32_t hv = hu | (1u << hb);
            uint32_t u[L], v[L];
            cl_read<L>(u, top, g * 8u + hu);
            cl_read<L>(v, top, g * 8u + hv);
            cl_butterfly<L>(u, v, p, m, s, (hu << kb) | (rank * slice + g), tw);
            cl_write<L>(top, g * 8u + hu, u);
            cl_write<L>(top, g * 8u + hv, v);
        }
        __syncthreads();
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
        }
        if (!p.inverse)
        {
            // the CTA's slice of every top-bit group, coalesced along g
            for (uint32_t i = threadIdx.x; i < B; i += blockDim.x)
            {
                const uint32_t g = i % slice, h = i / slice;
                const uint64_t e = base + (static_cast<uint64_t>(h) << kb) + rank * slice + g;
#pragma unroll
                for (int j = 0; j < L; ++j)
                {
                    top[(g * 8u + h) * L + j] = p.in[static_cast<uint64_t>(j) * p.elements + e];
                }
            }
            __syncthreads();
            // stages 0..2 on the top bits (bits 2, 1, 0 of h)
            for (uint32_t s = 0; s < 3; ++s)
            {
                cl_top_stage<L>(p, m, top, rank, s, 2u - s, tw);
            }
            // every CTA runs before remote stores reach its shared memory
            cluster.sync();
            for (uint32_t i = threadIdx.x; i < B; i += blockDim.x)
            {
                const uint32_t g = i % slice, h = i / slice;
                uint32_t x[L];
                cl_read<L>(x, top, g * 8u + h);
                cl_write<L>(cluster.map_shared_rank(blk, h), rank * slice + g, x);
            }
            cluster.sync();
            // stages 3 .. k - 1 in the block layout (local bits kb - 1 .. 0)
            for (uint32_t s = 3; s < k; ++s)
            {
                cl_block_stage<L>(p, m, blk, rank, s, k - 1u - s, tw);
            }
            for (uint32_t i = threadIdx.x; i < B; i += blockDim.x)
            {
#pragma unroll
                for (int j = 0; j < L; ++j)
                {
                    p.out[static_cast<uint64_t>(j) * p.elements + base + (rank << kb) + i] = blk[i * L + j];
                }
            }
        }
        else
        {
            for (uint32_t i = threadIdx.x; i < B; i += blockDim.x)
            {
#pragma unroll
                for (int j = 0; j < L; ++j)
                {
                    blk[i * L + j] = p.in[static_cast<uint64_t>(j) * p.elements + base + (rank << kb) + i];
                }
            }
            __syncthreads();
            // stages 0 .. kb - 1 in the block layout (local bits 0 .. kb - 1)
            for (uint32_t s = 0; s < kb; ++s)
            {
                cl_block_stage<L>(p, m, blk, rank, s, s, tw);
            }
            cluster.sync();
            // each element to the CTA that holds its slice of low values
            for (uint32_t l = threadIdx.x; l < B; l += blockDim.x)
            {
                uint32_t x[L];
                cl_read<L>(x, blk, l);
                cl_write<L>(cluster.map_shared_rank(top, l / slice), (l % slice) * 8u + rank, x);
            }
            cluster.sync();
            // stages kb .. k - 1 on the top bits (bits 0, 1, 2 of h), the last with the scaling
            for (uint32_t s = kb; s < k; ++s)
            {
                cl_top_stage<L>(p, m, top, rank, s, s - kb, tw);
            }
            for (uint32_t i = threadIdx.x; i < B; i += blockDim.x)
            {
                const uint32_t g = i % slice, h = i / slice;
                const uint64_t e = base + (static_cast<uint64_t>(h) << kb) + rank * slice + g;
#pragma unroll
                for (int j = 0; j < L; ++j)
                {
                    p.out[static_cast<uint64_t>(j) * p.elements + e] = top[(g * 8u + h) * L + j];
                }
            }
        }
    }
}
