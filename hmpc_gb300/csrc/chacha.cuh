// ChaCha20 keystream blocks and the samplers that consume them, generated
// per thread in registers so that no noise tensor ever goes through HBM.
//
// State layout and block function follow hmpc's chacha20 = chacha<20,3,1>
// (hmpc/crypto/chacha.hpp:91-166): [constants x4, key x8, counter x1,
// nonce x3]; the output adds the input state back.  A sampler draws one
// 32-bit word per limb in stream order and moves to block counter+1 after
// word 15 (hmpc/random/number_generator.hpp:66-91).  Because every sampler
// here consumes a compile-time number of words, the word positions are
// compile-time constants and the blocks stay in registers.
#pragma once

#include <cstdint>

#include "limbs.cuh"

namespace hmpc_gb300
{
    struct RngKey
    {
        uint32_t key[8];
        uint32_t nonce[3];
    };

    __device__ __forceinline__ void chacha_quarter(uint32_t& a, uint32_t& b, uint32_t& c, uint32_t& d)
    {
        a += b;
        d = __funnelshift_l(d ^ a, d ^ a, 16);
        c += d;
        b = __funnelshift_l(b ^ c, b ^ c, 12);
        a += b;
        d = __funnelshift_l(d ^ a, d ^ a, 8);
        c += d;
        b = __funnelshift_l(b ^ c, b ^ c, 7);
    }

    // The part of a block's first round that every block of one key and
    // nonce shares: the column quarter rounds of columns 1-3 (constants, key
    // words, nonce; the counter is in column 0) and the first addition of
    // column 0.  Computed once, it saves three of the block's eighty quarter
    // rounds for each further block.
    struct ChachaPre
    {
        uint32_t x[16];  // the state after those steps (x[12], the counter, unset)
    };

    __device__ __forceinline__ ChachaPre chacha_pre(const RngKey& k)
    {
        ChachaPre p{{0x61707865u, 0x3320646eu, 0x79622d32u, 0x6b206574u, k.key[0], k.key[1], k.key[2], k.key[3],
                     k.key[4], k.key[5], k.key[6], k.key[7], 0u, k.nonce[0], k.nonce[1], k.nonce[2]}};
        chacha_quarter(p.x[1], p.x[5], p.x[9], p.x[13]);
        chacha_quarter(p.x[2], p.x[6], p.x[10], p.x[14]);
        chacha_quarter(p.x[3], p.x[7], p.x[11], p.x[15]);
        p.x[0] += p.x[4];
        return p;
    }

    __device__ __forceinline__ void chacha20_block(const ChachaPre& pre, const RngKey& k, uint32_t counter,
                                                   uint32_t (&out)[16])
    {
        uint32_t x[16];
#pragma unroll
        for (int i = 0; i < 16; ++i)
        {
            x[i] = pre.x[i];
        }
        // the rest of column 0's first quarter round (a += b is in pre)
        x[12] = __funnelshift_l(counter ^ x[0], counter ^ x[0], 16);
        x[8] += x[12];
        x[4] = __funnelshift_l(x[4] ^ x[8], x[4] ^ x[8], 12);
        x[0] += x[4];
        x[12] = __funnelshift_l(x[12] ^ x[0], x[12] ^ x[0], 8);
        x[8] += x[12];
        x[4] = __funnelshift_l(x[4] ^ x[8], x[4] ^ x[8], 7);
#pragma unroll
        for (int r = 0; r < 10; ++r)
        {
            if (r > 0)
            {
                chacha_quarter(x[0], x[4], x[8], x[12]);
                chacha_quarter(x[1], x[5], x[9], x[13]);
                chacha_quarter(x[2], x[6], x[10], x[14]);
                chacha_quarter(x[3], x[7], x[11], x[15]);
            }
            chacha_quarter(x[0], x[5], x[10], x[15]);
            chacha_quarter(x[1], x[6], x[11], x[12]);
            chacha_quarter(x[2], x[7], x[8], x[13]);
            chacha_quarter(x[3], x[4], x[9], x[14]);
        }
        out[0] = x[0] + 0x61707865u;
        out[1] = x[1] + 0x3320646eu;
        out[2] = x[2] + 0x79622d32u;
        out[3] = x[3] + 0x6b206574u;
#pragma unroll
        for (int i = 0; i < 8; ++i)
        {
            out[4 + i] = x[4 + i] + k.key[i];
        }
        out[12] = x[12] + counter;
        out[13] = x[13] + k.nonce[0];
        out[14] = x[14] + k.nonce[1];
        out[15] = x[15] + k.nonce[2];
    }

    __device__ __forceinline__ void chacha20_block(const RngKey& k, uint32_t counter, uint32_t (&out)[16])
    {
        chacha20_block(chacha_pre(k), k, counter, out);
    }

    // The first `Words` words of the stream that starts at block `counter`
    // (blocks counter, counter+1, ... as the generator refills).
    template<int Words>
    __device__ __forceinline__ void chacha_stream(const ChachaPre& pre, const RngKey& k, uint32_t counter,
                                                  uint32_t (&w)[Words])
    {
        constexpr int blocks = (Words + 15) / 16;
#pragma unroll
        for (int b = 0; b < blocks; ++b)
        {
            uint32_t blk[16];
            chacha20_block(pre, k, counter + static_cast<uint32_t>(b), blk);
#pragma unroll
            for (int i = 0; i < 16; ++i)
            {
                if (b * 16 + i < Words)
                {
                    w[b * 16 + i] = blk[i];
                }
            }
        }
    }

    template<int Words>
    __device__ __forceinline__ void chacha_stream(const RngKey& k, uint32_t counter, uint32_t (&w)[Words])
    {
        chacha_stream<Words>(chacha_pre(k), k, counter, w);
    }

    // Centred binomial value popcount(low 4V bits) - 2V from words
    // [First, First + ceil(4V/32)) (hmpc/random/binomial.hpp:29-86,110-122).
    template<int VarianceX2, int First, int Words>
    __device__ __forceinline__ int cbd_from_words(const uint32_t (&w)[Words])
    {
        constexpr int count = 2 * VarianceX2;
        constexpr int n = (count + 31) / 32;
        int sum = 0;
#pragma unroll
        for (int i = 0; i < n; ++i)
        {
            uint32_t word = w[First + i];
            if (i == n - 1 && (count % 32) != 0)
            {
                word &= (1u << (count % 32)) - 1u;
            }
            sum += __popc(word);
        }
        return sum - VarianceX2;
    }

    template<int VarianceX2>
    struct CbdWords
    {
        static constexpr int value = (2 * VarianceX2 + 31) / 32;
    };

    // Montgomery form of a small signed integer v, |v| <= 64, using a table
    // of the Montgomery forms of 0..64 (hmpc/ints/mod.hpp:219-226 yields
    // (Q + v)*R mod Q for v < 0, i.e. -(|v|*R mod Q)).
    template<int L>
    __device__ __forceinline__ void small_to_mont(uint32_t (&r)[L], int v, const uint32_t* small_table,
                                                  const Modulus<L>& m)
    {
        const int a = v < 0 ? -v : v;
        uint32_t x[L];
#pragma unroll
        for (int j = 0; j < L; ++j)
        {
            x[j] = small_table[a * L + j];
        }
        if (v < 0)
        {
            mod_neg<L>(r, x, m);
        }
        else
        {
#pragma unroll
            for (int j = 0; j < L; ++j)
            {
                r[j] = x[j];
            }
        }
    }

    // uniform<mod<Q>> from words [First, First + W): the top word is masked
    // to (bits + security) mod 32 bits, then one reduction with R' = 2^(32W)
    // (hmpc/random/uniform.hpp:35-47,62-66; hmpc/ints/mod.hpp:210-215).
    template<int L, int W, int First, int Words>
    __device__ __forceinline__ void uniform_from_words(uint32_t (&r)[L], const uint32_t (&w)[Words], uint32_t top_mask,
                                                       const Modulus<L>& m)
    {
        uint32_t v[W];
#pragma unroll
        for (int i = 0; i < W; ++i)
        {
            v[i] = w[First + i];
        }
        v[W - 1] &= top_mask;
        redc_wide<L, W>(r, v, m);
    }
}
