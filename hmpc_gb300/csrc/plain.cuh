// The plain transform: one kernel launch per stage, radix-2 butterflies in
// global memory, one thread per butterfly -- the schedule of hmpc's SYCL
// transform (hmpc/expr/number_theoretic_transform.hpp:90-197: a parallel_for
// of N/2 * batch work-items per stage) on this GPU.  It is the comparator the
// tiled passes are measured against, and computes the same values.
#pragma once

#include <cstdint>

#include "chacha.cuh"
#include "limbs.cuh"
#include "ntt.cuh"

namespace hmpc_gb300
{
    struct PlainStageParams
    {
        uint32_t* out;
        const uint32_t* src;        // stage-0 tensor input (nullptr: out)
        const uint32_t* twiddles;   // element-major [N][L]
        const uint32_t* small_table;
        uint64_t elements;
        uint32_t log_n;
        uint32_t stage;
        uint32_t inverse;
        RngKey rng;
        uint32_t vx2;
        uint32_t top_mask;
    };

    template<int L, int Kind, int NW>
    __global__ void __launch_bounds__(256) plain_stage_kernel(const PlainStageParams p, const Modulus<L> m)
    {
        const uint64_t half = 1ull << (p.log_n - 1);
        const uint64_t n = 1ull << p.log_n;
        const uint64_t pairs = p.elements / 2;
        for (uint64_t id = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x; id < pairs;
             id += static_cast<uint64_t>(gridDim.x) * blockDim.x)
        {
            const uint64_t poly = id / half;
            const uint64_t tid = id % half;
            const uint32_t s = p.stage;
            const uint64_t length = p.inverse ? (n >> (s + 1)) : (1ull << s);
            const uint64_t step = p.inverse ? (1ull << s) : (n / length / 2);
            const uint64_t psi_step = tid / step;
            const uint64_t target = psi_step * step * 2 + tid % step;
            const uint64_t eu = poly * n + target;
            const uint64_t ev = eu + step;
            uint32_t u[L], v[L], t[L];
            if (Kind != producer_tensor && s == 0)
            {
                NttPassParams q{};
                q.log_n = p.log_n;
                q.rng = p.rng;
                q.vx2 = p.vx2;
                q.top_mask = p.top_mask;
                q.small_table = p.small_table;
                produce_pair<L, Kind, NW>(q, m, poly, target, target + step, u, v);
            }
            else
            {
                const uint32_t* in = (s == 0 && p.src) ? p.src : p.out;
#pragma unroll
                for (int j = 0; j < L; ++j)
                {
                    u[j] = in[static_cast<uint64_t>(j) * p.elements + eu];
                    v[j] = in[static_cast<uint64_t>(j) * p.elements + ev];
                }
            }
            if (!p.inverse)
            {
                load_twiddle<L>(t, p.twiddles, length + psi_step);
                mont_mul<L>(v, v, t, m);
                uint32_t sum[L];
                mod_add<L>(sum, u, v, m);
                mod_sub<L>(v, u, v, m);
#pragma unroll
                for (int j = 0; j < L; ++j)
                {
                    u[j] = sum[j];
                }
            }
            else if (s + 1 < p.log_n)
            {
                load_twiddle<L>(t, p.twiddles, length + psi_step);
                uint32_t sum[L], diff[L];
                mod_add<L>(sum, u, v, m);
                mod_sub<L>(diff, u, v, m);
                mont_mul<L>(v, diff, t, m);
#pragma unroll
                for (int j = 0; j < L; ++j)
                {
                    u[j] = sum[j];
                }
            }
            else
            {
                uint32_t sum[L], diff[L];
                mod_add<L>(sum, u, v, m);
                mod_sub<L>(diff, u, v, m);
                load_twiddle<L>(t, p.twiddles, 0);
                mont_mul<L>(u, sum, t, m);
                load_twiddle<L>(t, p.twiddles, 1);
                mont_mul<L>(v, diff, t, m);
            }
#pragma unroll
            for (int j = 0; j < L; ++j)
            {
                p.out[static_cast<uint64_t>(j) * p.elements + eu] = u[j];
                p.out[static_cast<uint64_t>(j) * p.elements + ev] = v[j];
            }
        }
    }
}
