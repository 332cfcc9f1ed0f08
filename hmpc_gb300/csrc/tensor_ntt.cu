// Tensor-core transform kernels of one limb count, compiled with
// -DHMPC_L=<2|4|8>; exports tc_kernels_<L>().  Instantiated group shapes:
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
        static_assert(L == 2 || L == 4 || L == 8, "tensor-core transform for 2, 4 or 8 limbs");

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

        template<int R, int IN, int OUT>
        cudaError_t launch(const TcGroupParams& p, unsigned grid, cudaStream_t stream)
        {
            using S = TcShape<DC, R, IN>;
            // at least half of an SM's shared memory: one CTA per SM, so a CTA's
            // two accumulators (up to all 512 TMEM columns) are always free
            constexpr uint32_t smem = S::smem > 116u * 1024u ? S::smem : 116u * 1024u;
            static std::once_flag once;
            static cudaError_t configured = cudaSuccess;
            std::call_once(once, [] {
                configured = cudaFuncSetAttribute(tc_group_kernel<DC, R, IN, OUT>,
                                                  cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
            });
            if (configured != cudaSuccess)
            {
                return configured;
            }
            tc_group_kernel<DC, R, IN, OUT><<<grid, tc_threads, smem, stream>>>(p);
            return cudaGetLastError();
        }

        template<int R, int IN>
        void fill(TcShapeInfo& out)
        {
            using S = TcShape<DC, R, IN>;
            out.smem = S::smem;
            out.a_bytes = S::a_bytes;
            out.b_bytes = S::b_bytes;
            out.k_pad = S::k_pad;
            out.n_mma = S::n_mma;
            out.w_in = S::w_in;
            out.w_out = S::w_out;
            out.d_in = S::d_in;
        }

        cudaError_t group(const TcGroupParams& p, int r, int in_kind, int out_kind, unsigned grid,
                          cudaStream_t stream)
        {
            if (out_kind == tc_out_digits && r == 8)
            {
                switch (in_kind)
                {
                case tc_in_limbs: return launch<8, tc_in_limbs, tc_out_digits>(p, grid, stream);
                case tc_in_cbd: return launch<8, tc_in_cbd, tc_out_digits>(p, grid, stream);
                case tc_in_digits: return launch<8, tc_in_digits, tc_out_digits>(p, grid, stream);
                default: break;
                }
            }
            if (out_kind == tc_out_limbs && in_kind == tc_in_digits)
            {
                switch (r)
                {
                case 2: return launch<2, tc_in_digits, tc_out_limbs>(p, grid, stream);
                case 4: return launch<4, tc_in_digits, tc_out_limbs>(p, grid, stream);
                case 8: return launch<8, tc_in_digits, tc_out_limbs>(p, grid, stream);
                default: break;
                }
            }
            return cudaErrorInvalidValue;
        }

        bool shape(int r, int in_kind, int out_kind, TcShapeInfo& out)
        {
            if (out_kind == tc_out_digits && r == 8)
            {
                switch (in_kind)
                {
                case tc_in_limbs: fill<8, tc_in_limbs>(out); return true;
                case tc_in_cbd: fill<8, tc_in_cbd>(out); return true;
                case tc_in_digits: fill<8, tc_in_digits>(out); return true;
                default: return false;
                }
            }
            if (out_kind == tc_out_limbs && in_kind == tc_in_digits)
            {
                switch (r)
                {
                case 2: fill<2, tc_in_digits>(out); return true;
                case 4: fill<4, tc_in_digits>(out); return true;
                case 8: fill<8, tc_in_digits>(out); return true;
                default: return false;
                }
            }
            return false;
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

        const TcKernels table = {DC, group, shape, gen, expand};
    }

    const TcKernels* HMPC_CAT(tc_kernels_, HMPC_L)()
    {
        return &table;
    }
}
