// Tensor-core transform kernels of one limb count, compiled with
// -DHMPC_L=<2..8>; exports tc_kernels_<L>().  Instantiated group shapes:
// the first group (r = 8) from limbs or from centred binomial samples, the
// middle groups (r = 8) digits to digits, the last group (r = 2, 4 or 8)
// digits to reduced limbs.
#include <mutex>

#include "dispatch.hpp"
#include "tensor_ntt.cuh"

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
        constexpr int DC = 4 * L;
        static_assert(L >= 2 && L <= 8, "tensor-core transform for 2 to 8 limbs");

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

        template<int R, int IN, int OUT, int NS, bool Contig, int Lay>
        cudaError_t launch(const TcGroupParams& p, unsigned grid, cudaStream_t stream)
        {
            using S = TcShape<DC, R, IN, NS>;
            // at least half of an SM's shared memory: one CTA per SM, so a CTA's
            // two accumulators (up to all 512 TMEM columns) are always free
            constexpr uint32_t smem = S::smem > 116u * 1024u ? S::smem : 116u * 1024u;
            static std::once_flag once;
            static cudaError_t configured = cudaSuccess;
            std::call_once(once, [] {
                configured = cudaFuncSetAttribute(tc_group_kernel<DC, R, IN, OUT, NS, Contig, Lay>,
                                                  cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
            });
            if (configured != cudaSuccess)
            {
                return configured;
            }
            cudaLaunchConfig_t cfg{};
            cfg.gridDim = dim3(grid);
            cfg.blockDim = dim3(tc_workers<Contig> + 32);
            cfg.dynamicSmemBytes = smem;
            cfg.stream = stream;
            cudaLaunchAttribute attr[1];
            attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
            attr[0].val.programmaticStreamSerializationAllowed = 1;
            cfg.attrs = attr;
            cfg.numAttrs = p.dependent ? 1u : 0u;
            return cudaLaunchKernelEx(&cfg, tc_group_kernel<DC, R, IN, OUT, NS, Contig, Lay>, p);
        }

        template<int R, int IN, int NS>
        void fill(TcShapeInfo& out)
        {
            using S = TcShape<DC, R, IN, NS>;
            out.smem = S::smem;
            out.a_bytes = S::a_bytes;
            out.b_bytes = S::b_bytes;
            out.k_pad = S::k_pad;
            out.n_mma = S::n_mma;
            out.w_in = S::w_in;
            out.w_out = S::w_out;
            out.d_in = S::d_in;
            out.splits = NS;
        }

        // the instantiated shapes: every (R, input, output, splits, contiguous,
        // record layout) a plan uses; P: the limb input / output in one buffer
        // per polynomial (layout bit 2), for the shapes that read or write limbs
        template<bool P, typename F>
        bool dispatch_shapes(int r, int in_kind, int out_kind, int splits, bool contig, int lay, F& f)
        {
            constexpr int X = P ? 4 : 0;
            if (out_kind == tc_out_digits && r == 8 && !contig && splits == 1)
            {
                if (in_kind == tc_in_limbs) return lay ? f.template run<8, tc_in_limbs, tc_out_digits, 1, false, 2 | X>()
                                                       : f.template run<8, tc_in_limbs, tc_out_digits, 1, false, X>();
                if constexpr (!P)
                {
                    if (in_kind == tc_in_cbd) return lay ? f.template run<8, tc_in_cbd, tc_out_digits, 1, false, 2>()
                                                         : f.template run<8, tc_in_cbd, tc_out_digits, 1, false, 0>();
                    if (in_kind == tc_in_small) return lay ? f.template run<8, tc_in_small, tc_out_digits, 1, false, 2>()
                                                           : f.template run<8, tc_in_small, tc_out_digits, 1, false, 0>();
                    if (in_kind == tc_in_digits) return lay ? f.template run<8, tc_in_digits, tc_out_digits, 1, false, 2>()
                                                            : f.template run<8, tc_in_digits, tc_out_digits, 1, false, 0>();
                }
            }
            if (out_kind == tc_out_digits && r == 8 && contig && in_kind == tc_in_limbs && lay == 0)
            {
                if (splits == 2) return f.template run<8, tc_in_limbs, tc_out_digits, 2, true, X>();
                if (splits == 1) return f.template run<8, tc_in_limbs, tc_out_digits, 1, true, X>();
            }
            if (out_kind == tc_out_limbs && in_kind == tc_in_digits)
            {
                if (lay == 1 && contig && splits == 1)
                {
                    if (r == 8) return f.template run<8, tc_in_digits, tc_out_limbs, 1, true, 1 | X>();
                    if (r == 4) return f.template run<4, tc_in_digits, tc_out_limbs, 1, true, 1 | X>();
                    if (r == 2) return f.template run<2, tc_in_digits, tc_out_limbs, 1, true, 1 | X>();
                }
                if (lay == 0)
                {
                    if (r == 8 && splits == 2 && contig) return f.template run<8, tc_in_digits, tc_out_limbs, 2, true, X>();
                    if (r == 8 && splits == 1) return contig ? f.template run<8, tc_in_digits, tc_out_limbs, 1, true, X>()
                                                             : f.template run<8, tc_in_digits, tc_out_limbs, 1, false, X>();
                    if (r == 4 && splits == 1) return contig ? f.template run<4, tc_in_digits, tc_out_limbs, 1, true, X>()
                                                             : f.template run<4, tc_in_digits, tc_out_limbs, 1, false, X>();
                    if (r == 2 && splits == 1) return contig ? f.template run<2, tc_in_digits, tc_out_limbs, 1, true, X>()
                                                             : f.template run<2, tc_in_digits, tc_out_limbs, 1, false, X>();
                }
            }
            return false;
        }

        template<typename F>
        bool dispatch(int r, int in_kind, int out_kind, int splits, bool contig, int lay, F& f)
        {
            return (lay & 4) ? dispatch_shapes<true>(r, in_kind, out_kind, splits, contig, lay & 3, f)
                             : dispatch_shapes<false>(r, in_kind, out_kind, splits, contig, lay & 3, f);
        }

        struct Launcher
        {
            const TcGroupParams& p;
            unsigned grid;
            cudaStream_t stream;
            cudaError_t e;

            template<int R, int IN, int OUT, int NS, bool Contig, int Lay>
            bool run()
            {
                e = launch<R, IN, OUT, NS, Contig, Lay>(p, grid, stream);
                return true;
            }
        };

        struct Filler
        {
            TcShapeInfo& out;

            template<int R, int IN, int OUT, int NS, bool Contig, int Lay>
            bool run()
            {
                fill<R, IN, NS>(out);
                return true;
            }
        };

        cudaError_t group(const TcGroupParams& p, int r, int in_kind, int out_kind, int splits, int layout,
                          unsigned grid, cudaStream_t stream)
        {
            Launcher f{p, grid, stream, cudaErrorInvalidValue};
            dispatch(r, in_kind, out_kind, splits, p.lo == 0, layout, f);
            return f.e;
        }

        bool shape(int r, int in_kind, int out_kind, int splits, TcShapeInfo& out)
        {
            Filler f{out};
            return dispatch(r, in_kind, out_kind, splits, splits == 2, 0, f) ||
                   dispatch(r, in_kind, out_kind, splits, false, 0, f) ||
                   dispatch(r, in_kind, out_kind, splits, true, 0, f);
        }

        unsigned blocks_for(uint64_t threads)
        {
            return static_cast<unsigned>((threads + 255) / 256);
        }

        cudaError_t gen(const TcGenParams& p, const HostModulus& h, cudaStream_t stream)
        {
            const uint64_t threads = p.blocks << p.g;
            if (threads == 0)
            {
                return cudaSuccess;
            }
            tc_gen_kernel<L><<<blocks_for(threads), 256, 0, stream>>>(p, device_modulus(h));
            return cudaGetLastError();
        }

        cudaError_t expand(const TcExpandParams& p, const HostModulus& h, cudaStream_t stream)
        {
            const uint64_t threads = p.blocks * p.r * p.r * p.d_in;
            if (threads == 0)
            {
                return cudaSuccess;
            }
            tc_expand_kernel<L><<<blocks_for(threads), 256, 0, stream>>>(p, device_modulus(h));
            return cudaGetLastError();
        }

        cudaError_t combine6(const TcCombineParams& p, const HostModulus& h, cudaStream_t stream)
        {
            tc_combine6_kernel<L><<<16, 256, 0, stream>>>(p, device_modulus(h));
            return cudaGetLastError();
        }

        cudaError_t wide(const TcGroupParams& p, unsigned grid, cudaStream_t stream)
        {
            static std::once_flag once;
            static cudaError_t configured = cudaSuccess;
            std::call_once(once, [] {
                configured = cudaFuncSetAttribute(tc_wide_kernel<DC>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                  tc_wide_smem);
            });
            if (configured != cudaSuccess)
            {
                return configured;
            }
            cudaLaunchConfig_t cfg{};
            cfg.gridDim = dim3(grid);
            cfg.blockDim = dim3(512 + 32);
            cfg.dynamicSmemBytes = tc_wide_smem;
            cfg.stream = stream;
            cudaLaunchAttribute attr[1];
            attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
            attr[0].val.programmaticStreamSerializationAllowed = 1;
            cfg.attrs = attr;
            cfg.numAttrs = p.dependent ? 1u : 0u;
            return cudaLaunchKernelEx(&cfg, tc_wide_kernel<DC>, p);
        }

        const TcKernels table = {DC, group, shape, gen, expand, combine6, wide};
    }

    const TcKernels* HMPC_CAT(tc_kernels_, HMPC_L)()
    {
        return &table;
    }
}
