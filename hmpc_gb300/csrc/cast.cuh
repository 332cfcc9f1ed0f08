// Centred lift of residues between two moduli (hmpc/ints/mod.hpp:259-307):
// the source's canonical value v is shifted by `offset` when v > src/2 and is
// then converted into the target modulus as an unsigned integer -- directly
// (v*R^2, reduced) when it fits the target, otherwise with one reduction by
// R' = 2^(32 * words) followed by a product with R'*R^2 mod Q (mod.hpp:180-189).
// The source width is a runtime value, so this kernel uses runtime loops; it
// is not on the throughput path (enc fuses the lift into the NTT's producer).
#pragma once

#include <cstdint>

#include "dispatch.hpp"
#include "limbs.cuh"

namespace hmpc_gb300
{
    // word-by-word reduction with runtime sizes (hmpc/core/num/modulo.hpp:30-66)
    __device__ inline void redc_runtime(uint32_t* out, const uint32_t* value, int value_words, int r,
                                        const uint32_t* q, int p, uint32_t ninv)
    {
        uint32_t t[3 * max_device_limbs + 4];
        const int tl = r + p + 1;
        for (int k = 0; k < tl; ++k)
        {
            t[k] = k < value_words ? value[k] : 0u;
        }
        for (int i = 0; i < r; ++i)
        {
            const uint32_t mq = t[i] * ninv;
            uint64_t carry = 0;
            for (int j = 0; j < p; ++j)
            {
                const uint64_t s = static_cast<uint64_t>(mq) * q[j] + t[i + j] + carry;
                t[i + j] = static_cast<uint32_t>(s);
                carry = s >> 32;
            }
            for (int k = i + p; k < tl; ++k)
            {
                const uint64_t s = static_cast<uint64_t>(t[k]) + carry;
                t[k] = static_cast<uint32_t>(s);
                carry = s >> 32;
            }
        }
        // S = t[r .. r+p]; subtract Q when S >= Q
        bool ge = t[r + p] != 0u;
        if (!ge)
        {
            ge = true;
            for (int j = p - 1; j >= 0; --j)
            {
                if (t[r + j] != q[j])
                {
                    ge = t[r + j] > q[j];
                    break;
                }
            }
        }
        uint64_t borrow = 0;
        for (int j = 0; j < p; ++j)
        {
            const uint64_t d = static_cast<uint64_t>(t[r + j]) - (ge ? q[j] : 0u) - borrow;
            out[j] = static_cast<uint32_t>(d);
            borrow = (d >> 63) & 1u;
        }
    }

    template<int L>
    __global__ void __launch_bounds__(256) cast_kernel(uint32_t* out, const uint32_t* in, uint64_t elements,
                                                       const CastParams cp, const Modulus<L> m)
    {
        for (uint64_t e = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x; e < elements;
             e += static_cast<uint64_t>(gridDim.x) * blockDim.x)
        {
            const int ls = static_cast<int>(cp.src_limbs);
            uint32_t x[max_device_limbs];
            for (int j = 0; j < ls; ++j)
            {
                x[j] = in[static_cast<uint64_t>(j) * elements + e];
            }
            uint32_t v[max_device_limbs + 1];
            redc_runtime(v, x, ls, ls, cp.src_q, ls, cp.src_ninv);
            // above = v > src/2
            bool above = false;
            for (int j = ls - 1; j >= 0; --j)
            {
                if (v[j] != cp.src_half[j])
                {
                    above = v[j] > cp.src_half[j];
                    break;
                }
            }
            const int nw = static_cast<int>(cp.norm_words);
            uint32_t norm[max_device_limbs + 1];
            uint64_t carry = 0;
            for (int j = 0; j < nw; ++j)
            {
                const uint64_t s = static_cast<uint64_t>(j < ls ? v[j] : 0u) + (above ? cp.offset[j] : 0u) + carry;
                norm[j] = static_cast<uint32_t>(s);
                carry = s >> 32;
            }
            uint32_t y[L];
            if (cp.direct)
            {
#pragma unroll
                for (int j = 0; j < L; ++j)
                {
                    y[j] = j < nw ? norm[j] : 0u;
                }
            }
            else
            {
                redc_runtime(y, norm, nw, nw, m.q, L, m.ninv);
            }
            uint32_t f[L];
#pragma unroll
            for (int j = 0; j < L; ++j)
            {
                f[j] = cp.factor[j];
            }
            mont_mul<L>(y, y, f, m);
#pragma unroll
            for (int j = 0; j < L; ++j)
            {
                out[static_cast<uint64_t>(j) * elements + e] = y[j];
            }
        }
    }
}
