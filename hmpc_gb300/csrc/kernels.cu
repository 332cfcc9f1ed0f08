// Per-limb-count kernel instantiations and launchers.  Compiled once per L
// with -DHMPC_L=<L>; exports kernel_table_<L>().
#include <algorithm>

#include "cast.cuh"
#include "dispatch.hpp"
#include "elementwise.cuh"
#include "linalg.cuh"
#include "ntt.cuh"

#ifndef HMPC_L
#error "compile with -DHMPC_L=<limbs>"
#endif

#define HMPC_CAT2(a, b) a##b
#define HMPC_CAT(a, b) HMPC_CAT2(a, b)

namespace hmpc_gb300
{
    namespace
    {
        constexpr int L = HMPC_L;
        constexpr int R = 3;  // 8 elements per thread in the NTT passes

        Modulus<L> device_modulus(const HostModulus& h)
        {
            Modulus<L> m{};
            for (int j = 0; j < L; ++j)
            {
                m.q[j] = h.q[j];
                m.one[j] = h.one[j];
            }
            m.ninv = h.ninv;
            m.bits = static_cast<uint32_t>(h.bits);
            return m;
        }

        Modulus<L> holder(const uint32_t* words)
        {
            Modulus<L> m{};
            for (int j = 0; j < L; ++j)
            {
                m.one[j] = words[j];
            }
            return m;
        }

        unsigned grid_for(uint64_t work, unsigned block)
        {
            const uint64_t g = (work + block - 1) / block;
            return static_cast<unsigned>(std::max<uint64_t>(1, std::min<uint64_t>(g, 152ull * 64ull)));
        }

        template<int Kind, int NW, int RB>
        cudaError_t launch_pass(const NttPassParams& p, const Modulus<L>& m, unsigned grid, unsigned block,
                                size_t smem, cudaStream_t stream)
        {
            auto kernel = ntt_pass_kernel<L, RB, Kind, NW>;
            static bool configured = false;
            if (!configured)
            {
                cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
                if (e != cudaSuccess)
                {
                    return e;
                }
                configured = true;
            }
            cudaLaunchConfig_t cfg{};
            cfg.gridDim = dim3(grid);
            cfg.blockDim = dim3(block);
            cfg.dynamicSmemBytes = smem;
            cfg.stream = stream;
            cudaLaunchAttribute attr[1];
            attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
            attr[0].val.programmaticStreamSerializationAllowed = 1;
            cfg.attrs = attr;
            cfg.numAttrs = p.dependent ? 1u : 0u;
            return cudaLaunchKernelEx(&cfg, kernel, p, m);
        }

        template<int RB>
        cudaError_t ntt_pass_radix(const NttPassParams& p, int kind, int nw, const Modulus<L>& m, unsigned grid,
                                   unsigned block, size_t smem, cudaStream_t stream)
        {
            if (kind == producer_tensor)
            {
                return launch_pass<producer_tensor, 1, RB>(p, m, grid, block, smem, stream);
            }
            if (kind == producer_cbd)
            {
                switch (nw)
                {
                case 1: return launch_pass<producer_cbd, 1, RB>(p, m, grid, block, smem, stream);
                case 2: return launch_pass<producer_cbd, 2, RB>(p, m, grid, block, smem, stream);
                case 3: return launch_pass<producer_cbd, 3, RB>(p, m, grid, block, smem, stream);
                case 4: return launch_pass<producer_cbd, 4, RB>(p, m, grid, block, smem, stream);
                default: return cudaErrorInvalidValue;
                }
            }
            if (kind == producer_uniform)
            {
                if (nw == L + 2)
                {
                    return launch_pass<producer_uniform, L + 2, RB>(p, m, grid, block, smem, stream);
                }
                if (nw == L + 3)
                {
                    return launch_pass<producer_uniform, L + 3, RB>(p, m, grid, block, smem, stream);
                }
            }
            return cudaErrorInvalidValue;
        }

        cudaError_t ntt_pass(const NttPassParams& p, int kind, int nw, int radix_bits, const HostModulus& h,
                             unsigned grid, unsigned block, size_t smem, cudaStream_t stream)
        {
            const Modulus<L> m = device_modulus(h);
            if (radix_bits == 2)
            {
                return ntt_pass_radix<2>(p, kind, nw, m, grid, block, smem, stream);
            }
            if (radix_bits == 3)
            {
                return ntt_pass_radix<3>(p, kind, nw, m, grid, block, smem, stream);
            }
            return cudaErrorInvalidValue;
        }

        cudaError_t fma(uint32_t* d, const uint32_t* a, const uint32_t* b, const uint32_t* c, uint64_t elements,
                        const HostModulus& h, cudaStream_t stream)
        {
            const uintptr_t align = reinterpret_cast<uintptr_t>(a) | reinterpret_cast<uintptr_t>(b) |
                                    reinterpret_cast<uintptr_t>(c) | reinterpret_cast<uintptr_t>(d);
            const int vectorised = (elements % vec == 0) && (align % 16 == 0);
            const unsigned block = 256;
            unsigned grid;
            if (vectorised)
            {
                grid = static_cast<unsigned>((elements / vec + block - 1) / block);
            }
            else
            {
                grid = grid_for(elements, block);
            }
            if (elements == 0)
            {
                return cudaSuccess;
            }
            fma_kernel<L><<<grid, block, 0, stream>>>(d, a, b, c, elements, vectorised, device_modulus(h));
            return cudaGetLastError();
        }

        cudaError_t binary(uint32_t* out, const uint32_t* a, uint64_t a_elements, const uint32_t* b,
                           uint64_t b_elements, uint64_t elements, int op, const HostModulus& h, cudaStream_t stream)
        {
            if (elements == 0)
            {
                return cudaSuccess;
            }
            binary_kernel<L><<<grid_for(elements, 256), 256, 0, stream>>>(out, a, a_elements, b, b_elements,
                                                                          elements, op, device_modulus(h));
            return cudaGetLastError();
        }

        cudaError_t lhe_combine(uint32_t* out, const uint32_t* k, uint64_t n, const uint32_t* u, const uint32_t* v,
                                const uint32_t* msg, uint64_t elements, const uint32_t* p_mont, const HostModulus& h,
                                cudaStream_t stream)
        {
            if (elements == 0)
            {
                return cudaSuccess;
            }
            lhe_combine_kernel<L><<<grid_for(elements, 256), 256, 0, stream>>>(out, k, n, u, v, msg, elements,
                                                                               device_modulus(h), holder(p_mont));
            return cudaGetLastError();
        }

        cudaError_t uniform(uint32_t* out, uint64_t elements, const RngKey& rng, int words, uint32_t top_mask,
                            const HostModulus& h, cudaStream_t stream)
        {
            if (elements == 0)
            {
                return cudaSuccess;
            }
            const unsigned grid = grid_for(elements, 256);
            if (words == L + 2)
            {
                uniform_kernel<L, L + 2><<<grid, 256, 0, stream>>>(out, elements, rng, top_mask, device_modulus(h));
            }
            else if (words == L + 3)
            {
                uniform_kernel<L, L + 3><<<grid, 256, 0, stream>>>(out, elements, rng, top_mask, device_modulus(h));
            }
            else
            {
                return cudaErrorInvalidValue;
            }
            return cudaGetLastError();
        }

        cudaError_t uniform_pairs(uint32_t* out, uint32_t log_n, uint64_t elements, const RngKey& rng, int words,
                                  uint32_t top_mask, const HostModulus& h, cudaStream_t stream)
        {
            if (elements < 2 || log_n < 1)
            {
                return elements ? cudaErrorInvalidValue : cudaSuccess;
            }
            const unsigned grid = grid_for(elements / 2, 256);
            if (words == L + 2)
            {
                uniform_pairs_kernel<L, L + 2><<<grid, 256, 0, stream>>>(out, log_n, elements, rng, top_mask,
                                                                         device_modulus(h));
            }
            else if (words == L + 3)
            {
                uniform_pairs_kernel<L, L + 3><<<grid, 256, 0, stream>>>(out, log_n, elements, rng, top_mask,
                                                                         device_modulus(h));
            }
            else
            {
                return cudaErrorInvalidValue;
            }
            return cudaGetLastError();
        }

        cudaError_t cbd(uint32_t* out, uint64_t elements, const RngKey& rng, uint32_t vx2, const uint32_t* table,
                        const HostModulus& h, cudaStream_t stream)
        {
            if (elements == 0)
            {
                return cudaSuccess;
            }
            const unsigned grid = grid_for(elements, 256);
            const Modulus<L> m = device_modulus(h);
            switch ((2 * vx2 + 31) / 32)
            {
            case 1: cbd_kernel<L, 1><<<grid, 256, 0, stream>>>(out, elements, rng, vx2, table, m); break;
            case 2: cbd_kernel<L, 2><<<grid, 256, 0, stream>>>(out, elements, rng, vx2, table, m); break;
            case 3: cbd_kernel<L, 3><<<grid, 256, 0, stream>>>(out, elements, rng, vx2, table, m); break;
            case 4: cbd_kernel<L, 4><<<grid, 256, 0, stream>>>(out, elements, rng, vx2, table, m); break;
            default: return cudaErrorInvalidValue;
            }
            return cudaGetLastError();
        }

        cudaError_t to_montgomery(uint32_t* out, const uint32_t* in, uint64_t elements, const HostModulus& h,
                                  cudaStream_t stream)
        {
            if (elements == 0)
            {
                return cudaSuccess;
            }
            to_montgomery_kernel<L><<<grid_for(elements, 256), 256, 0, stream>>>(out, in, elements, holder(h.r2),
                                                                                 device_modulus(h));
            return cudaGetLastError();
        }

        cudaError_t from_montgomery(uint32_t* out, const uint32_t* in, uint64_t elements, const HostModulus& h,
                                    cudaStream_t stream)
        {
            if (elements == 0)
            {
                return cudaSuccess;
            }
            from_montgomery_kernel<L><<<grid_for(elements, 256), 256, 0, stream>>>(out, in, elements,
                                                                                   device_modulus(h));
            return cudaGetLastError();
        }

        cudaError_t cast(uint32_t* out, const uint32_t* in, uint64_t elements, const CastParams& cp,
                         const HostModulus& h, cudaStream_t stream)
        {
            if (elements == 0)
            {
                return cudaSuccess;
            }
            cast_kernel<L><<<grid_for(elements, 256), 256, 0, stream>>>(out, in, elements, cp, device_modulus(h));
            return cudaGetLastError();
        }

        template<int Kind, int NW>
        cudaError_t launch_plain(const PlainStageParams& p, const Modulus<L>& m, cudaStream_t stream)
        {
            plain_stage_kernel<L, Kind, NW><<<grid_for(p.elements / 2, 256), 256, 0, stream>>>(p, m);
            return cudaGetLastError();
        }

        cudaError_t plain_stage(const PlainStageParams& p, int kind, int nw, const HostModulus& h, cudaStream_t stream)
        {
            const Modulus<L> m = device_modulus(h);
            if (kind == producer_tensor || p.stage != 0)
            {
                return launch_plain<producer_tensor, 1>(p, m, stream);
            }
            if (kind == producer_cbd)
            {
                switch (nw)
                {
                case 1: return launch_plain<producer_cbd, 1>(p, m, stream);
                case 2: return launch_plain<producer_cbd, 2>(p, m, stream);
                case 3: return launch_plain<producer_cbd, 3>(p, m, stream);
                case 4: return launch_plain<producer_cbd, 4>(p, m, stream);
                default: return cudaErrorInvalidValue;
                }
            }
            if (kind == producer_uniform)
            {
                if (nw == L + 2)
                {
                    return launch_plain<producer_uniform, L + 2>(p, m, stream);
                }
                if (nw == L + 3)
                {
                    return launch_plain<producer_uniform, L + 3>(p, m, stream);
                }
            }
            return cudaErrorInvalidValue;
        }

        cudaError_t ct_mul(uint32_t* d0, uint32_t* d1, uint32_t* d2, const uint32_t* a0, const uint32_t* a1,
                           const uint32_t* b0, const uint32_t* b1, uint64_t elements, const HostModulus& h,
                           cudaStream_t stream)
        {
            if (elements == 0)
            {
                return cudaSuccess;
            }
            ct_mul_kernel<L><<<grid_for(elements, 256), 256, 0, stream>>>(d0, d1, d2, a0, a1, b0, b1, elements,
                                                                          device_modulus(h));
            return cudaGetLastError();
        }

        cudaError_t dec_combine(uint32_t* x, const uint32_t* s, uint64_t n, const uint32_t* c0, const uint32_t* c1,
                                const uint32_t* c2, uint64_t elements, const HostModulus& h, cudaStream_t stream)
        {
            if (elements == 0)
            {
                return cudaSuccess;
            }
            dec_combine_kernel<L><<<grid_for(elements, 256), 256, 0, stream>>>(x, s, n, c0, c1, c2, elements,
                                                                               device_modulus(h));
            return cudaGetLastError();
        }

        template<int RB>
        cudaError_t launch_batched(const BatchedParams& bp, const Modulus<L>& m, unsigned grid, size_t smem,
                                   cudaStream_t stream)
        {
            // the shared-memory attribute is set by ntt_batched_blocks_per_sm, which
            // the batch planner calls before it captures this launch
            ntt_batched_kernel<L, RB><<<grid, 256, smem, stream>>>(bp, m);
            return cudaGetLastError();
        }

        cudaError_t ntt_batched(const BatchedParams& bp, int radix_bits, const HostModulus& h, unsigned grid,
                                size_t smem, cudaStream_t stream)
        {
            const Modulus<L> m = device_modulus(h);
            if (radix_bits == 2)
            {
                return launch_batched<2>(bp, m, grid, smem, stream);
            }
            if (radix_bits == 3)
            {
                return launch_batched<3>(bp, m, grid, smem, stream);
            }
            return cudaErrorInvalidValue;
        }

        int ntt_batched_blocks_per_sm(int radix_bits, size_t smem)
        {
            int blocks = 0;
            cudaError_t e;
            if (radix_bits == 2)
            {
                cudaFuncSetAttribute(ntt_batched_kernel<L, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
                e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, ntt_batched_kernel<L, 2>, 256, smem);
            }
            else
            {
                cudaFuncSetAttribute(ntt_batched_kernel<L, 3>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
                e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, ntt_batched_kernel<L, 3>, 256, smem);
            }
            return e == cudaSuccess ? blocks : 0;
        }

        cudaError_t lhe_combine_pair(uint32_t* c0, uint32_t* c1, const uint32_t* ka, const uint32_t* kb, uint64_t n,
                                     const uint32_t* stacked, uint64_t elements, const HostModulus& h,
                                     cudaStream_t stream)
        {
            if (elements == 0)
            {
                return cudaSuccess;
            }
            lhe_combine_pair_kernel<L><<<grid_for(elements, 256), 256, 0, stream>>>(c0, c1, ka, kb, n, stacked,
                                                                                   elements, device_modulus(h));
            return cudaGetLastError();
        }

        cudaError_t matvec(uint32_t* z, const uint32_t* mat, const uint32_t* x, const MatvecParams& p,
                           const HostModulus& h, cudaStream_t stream)
        {
            if (p.total == 0)
            {
                return cudaSuccess;
            }
            matvec_kernel<L><<<grid_for(p.total, 256), 256, 0, stream>>>(z, mat, x, p, device_modulus(h));
            return cudaGetLastError();
        }

        cudaError_t matvec_monomial(uint32_t* z, const int64_t* degrees, const uint32_t* x, const MatvecParams& p,
                                    const HostModulus& h, cudaStream_t stream)
        {
            if (p.total == 0)
            {
                return cudaSuccess;
            }
            matvec_monomial_kernel<L><<<grid_for(p.total, 256), 256, 0, stream>>>(z, degrees, x, p,
                                                                                device_modulus(h));
            return cudaGetLastError();
        }

        cudaError_t reduce(uint32_t* out, const uint32_t* in, uint64_t elements, int op, bool mod,
                           uint32_t top_mask, unsigned grid, const HostModulus& h, cudaStream_t stream)
        {
            const bool vectorised = elements % vec == 0 && reinterpret_cast<uintptr_t>(in) % 16 == 0;
            if (mod)
            {
                const Reducer<L, true> red{op, 0xffffffffu, device_modulus(h)};
                reduce_kernel<L, true><<<grid, 256, 0, stream>>>(out, grid, in, elements, vectorised, red);
            }
            else
            {
                const Reducer<L, false> red{op, top_mask, Modulus<L>{}};
                reduce_kernel<L, false><<<grid, 256, 0, stream>>>(out, grid, in, elements, vectorised, red);
            }
            return cudaGetLastError();
        }

        cudaError_t equal(uint32_t* out, const uint32_t* a, const uint32_t* b, uint64_t elements,
                          cudaStream_t stream)
        {
            if (elements == 0)
            {
                return cudaSuccess;
            }
            equal_kernel<L><<<grid_for(elements, 256), 256, 0, stream>>>(out, a, b, elements);
            return cudaGetLastError();
        }

        cudaError_t ntt_cluster(const ClusterNttParams& p, uint64_t batch, const HostModulus& h, cudaStream_t stream)
        {
            if (batch == 0)
            {
                return cudaSuccess;
            }
            if (p.log_n < 10 || p.log_n > 14)
            {
                return cudaErrorInvalidValue;
            }
            const size_t smem = cl_smem_bytes<L>(p.log_n);
            static cudaError_t configured = cudaFuncSetAttribute(
                ntt_cluster_kernel<L>, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(cl_smem_bytes<L>(14)));
            if (configured != cudaSuccess)
            {
                return configured;
            }
            // one butterfly per thread and stage: N/16 per CTA
            const uint32_t work = 1u << (p.log_n - 4);
            const unsigned threads = std::min(256u, std::max(32u, work));
            ntt_cluster_kernel<L><<<static_cast<unsigned>(batch * cl_ctas), threads, smem, stream>>>(p, device_modulus(h));
            return cudaGetLastError();
        }

        const KernelTable table = {ntt_pass, fma, binary, lhe_combine, uniform, cbd, to_montgomery,
                                   from_montgomery, cast, plain_stage, ct_mul, dec_combine, ntt_batched,
                                   ntt_batched_blocks_per_sm, R, lhe_combine_pair, matvec, matvec_monomial,
                                   reduce, equal, ntt_cluster, uniform_pairs};
    }

    const KernelTable* HMPC_CAT(kernel_table_, HMPC_L)()
    {
        return &table;
    }
}
