// Negacyclic NTT / INTT on the tensor cores.
//
// The transform is the same linear map as hmpc's stage-per-kernel transform
// (hmpc/expr/number_theoretic_transform.hpp:90-197,262-549); only the
// arithmetic differs.  The log2(N) butterfly stages are cut into groups of
// g <= 3 consecutive stages.  Inside a group, the r = 2^g elements
//   p(m) = (h << (lo + g)) | (m << lo) | c,   m = 0..r-1
// only mix among themselves, through an r x r matrix G_h over Z_q that
// depends on the block h alone (the stages' twiddles are selected by the
// position bits above the group) -- not on the column c or the polynomial.
// So one group over a batch is, per block h, the product of a
// (batch * 2^lo) x r matrix of residues with G_h^T: a GEMM with a shared
// constant operand.
//
// Exact arithmetic on fp16 tensor cores: a residue X in [0, 2^(8D)) is written
// as D base-256 digits; the constant (256^a * G[k][i] mod q), taken as a
// signed value in (-q/2, q/2], is written as DC balanced digits gamma in
// [-128, 128].  Then
//   G[k][i] * X = sum_a x_a * 256^a * G[k][i]
//              == sum_b 256^b * (sum_a x_a * gamma[k][i][a][b])   (mod q)
// and the inner sums over (i, a) are exactly what an fp16 x fp16 -> f32 MMA
// computes: each product is at most 2^15 in magnitude and a sum has at most
// 288 terms, so every partial sum is an integer below 2^24 and exact in f32.
//
// Between groups the data stays in digit form: the f32 column sums are
// carried into DC balanced digits plus two carry digits (the value is then
// congruent to the true residue but not reduced, which the next group's
// constants absorb), stored one byte per digit (biased by 128), 4 digits per
// 32-bit word, digit-word-planar like the limb-planar tensors.  The last group
// carries, packs and reduces into the fully reduced representative in
// [0, q) -- the same bits the reference produces, since the map is linear and
// the reduced representative is unique.  Montgomery form passes through
// unchanged (the map is applied to representatives); a sampler's raw small
// values are scaled by R inside the first group's constants.
//
// One CTA per SM, persistent over a contiguous range of 128-row tiles: the
// constant operand (up to 136 KB) arrives by one bulk copy per block change,
// the 128 x K digit tile is converted to fp16 by all threads, one thread
// issues the MMAs into one of two TMEM accumulators, and while the tensor
// core works on tile t+1 the threads carry tile t out of TMEM; the global
// loads of tile t+2 are in flight meanwhile.
#pragma once

#include <cstdint>
#include <type_traits>

#include <cuda_fp16.h>

#include "chacha.cuh"
#include "limbs.cuh"
#include "tcgen05.cuh"

namespace hmpc_gb300
{
    enum TcInput : int
    {
        tc_in_digits = 0,  // digit words of the previous group
        tc_in_limbs = 1,   // limb-planar residues (unsigned bytes)
        tc_in_cbd = 2,     // centred binomial samples drawn in the loader
        tc_in_small = 3,   // x = p * CBD sample + centred lift of a residue mod p, computed in the loader
    };

    enum TcOutput : int
    {
        tc_out_digits = 0,
        tc_out_limbs = 1,
    };

    constexpr int tc_rows = 128;
    // worker threads of a group kernel: 16 warps, or 8 where a tile row's
    // elements are adjacent (wider output runs per thread)
    template<bool Contig>
    constexpr int tc_workers = Contig ? 256 : 512;
    constexpr int tc_max_threads = 512 + 32;

    struct TcGroupParams
    {
        const uint32_t* in;        // digit or limb planes, `elements` words each
        uint32_t* out;             // digit or limb planes
        const uint8_t* images;     // per (block, N-split): the constant operand in its shared-memory layout
        uint32_t* error;           // set when a bounded wait runs out
        uint64_t elements;         // batch * N
        uint64_t rows;             // rows per block: batch << lo
        uint64_t tiles;            // blocks * NS * tiles_per_block
        uint32_t tiles_per_block;
        uint32_t log_n;
        uint32_t lo;               // column bits below the group's element bits
        uint32_t spin_limit;       // polls of an mbarrier before giving up
        uint32_t test_stall;       // test hook: nonzero -- the MMA thread waits before its first tile on a
                                   // barrier nothing arrives at, so that bounded wait runs out
        RngKey rng;                // CBD loader
        uint32_t vx2;
        uint32_t nw;
        uint32_t q[8];             // final reduction
        float inv_q_top;           // 2^(32(L-1)) / q
        uint32_t block_shift;      // blocked digit planes: log2 of the elements per block
        // small-integer loader: plaintext residues mod p (msg_limbs planes of
        // `elements` words, Montgomery form; nullptr: none) and p's constants
        const uint32_t* msg;
        uint64_t msg_stride;       // plane stride of msg
        uint32_t msg_limbs;
        uint32_t pq[2];
        uint32_t pninv;
        uint32_t phalf[2];
        // polynomials in buffers of their own (limb-planar, N words per plane,
        // 16-byte aligned): the first group reads in_polys[i] instead of `in`
        // and the last group writes out_polys[i] instead of `out` (nullptr: the
        // batch is one buffer of `elements` words per plane)
        const uint32_t* const* in_polys;
        uint32_t* const* out_polys;
        // launch with programmatic dependence on the kernel before it in the
        // stream (another group of the same transform): this launch's CTAs set
        // up while that one drains, and read its output only after it is
        // complete (host side only)
        uint32_t dependent;
    };

    // base-256 digits of the small-integer input (|x| < 2^70 for p < 2^64, 2V <= 64):
    // eight unsigned low bytes and the signed remainder
    constexpr int tc_small_digits = 9;

    // Sizes of one group kernel.  NS splits a block's R output elements over
    // NS constant images (N = R / NS * DC columns each); NBUF constant buffers
    // (two when they fit) let the next block's constants arrive while the
    // current block computes.
    template<int DC, int R, int IN, int NS>
    struct TcShape
    {
        static constexpr int g = R == 8 ? 3 : (R == 4 ? 2 : 1);
        static constexpr int d_in = IN == tc_in_digits ? DC + 2
                                    : (IN == tc_in_limbs ? DC : (IN == tc_in_small ? tc_small_digits : 1));
        static constexpr bool generated = IN == tc_in_cbd || IN == tc_in_small;  // no input planes
        static constexpr int w_in = generated ? 0 : (d_in + 3) / 4;
        // digit slots per element on the K axis (K index of digit a of element m: tc_k_index)
        static constexpr int d_eff = generated ? d_in : (R == 8 ? d_in : (R == 4 ? (d_in + 1) / 2 * 2 : w_in * 4));
        static constexpr int k_real = R * d_eff;
        static constexpr int k_pad = (k_real + 15) / 16 * 16;
        static constexpr int outputs = R / NS;  // output elements per N-split
        static constexpr int n_mma = (outputs * DC + 15) / 16 * 16;
        static constexpr int cols = n_mma <= 32 ? 32 : (n_mma <= 64 ? 64 : (n_mma <= 128 ? 128 : 256));
        static constexpr uint32_t a_bytes = tc_rows * k_pad * 2;
        static constexpr uint32_t b_bytes = n_mma * k_pad * 2;
        static constexpr uint32_t control_bytes = 128;  // 8 mbarriers, the TMEM address, the abort flag
        static constexpr int nbuf = a_bytes + 2 * b_bytes + control_bytes <= 227u * 1024u ? 2 : 1;
        static constexpr uint32_t smem = a_bytes + nbuf * b_bytes + control_bytes;
        static constexpr int w_out = (DC + 2 + 3) / 4;
        static constexpr uint32_t lbo_a = tc_rows / 8 * 128;
        static constexpr uint32_t lbo_b = n_mma / 8 * 128;
    };

    // two bytes (byte t of x0 and of x1) -> fp16x2 of (byte - bias)
    template<int Bias>
    __device__ __forceinline__ uint32_t bytes_to_half2(uint32_t x0, uint32_t x1, uint32_t t)
    {
        uint32_t y = __byte_perm(x0, x1, t | ((t + 4u) << 8));
        y = (y & 0x00FF00FFu) | 0x64006400u;  // fp16 1024 + byte in each half
        __half2 h = *reinterpret_cast<__half2*>(&y);
        const __half2 b = __halves2half2(__float2half(1024.0f + Bias), __float2half(1024.0f + Bias));
        h = __hsub2(h, b);
        return *reinterpret_cast<uint32_t*>(&h);
    }

    // bytes t and t + 1 of one word -> fp16x2 of (byte - bias): one byte
    // permute puts them under the exponent byte of 1024
    template<int Bias>
    __device__ __forceinline__ uint32_t byte_pair_to_half2(uint32_t x, uint32_t t)
    {
        uint32_t y = __byte_perm(x, 0x64646464u, t | (4u << 4) | ((t + 1u) << 8) | (4u << 12));
        __half2 h = *reinterpret_cast<__half2*>(&y);
        const __half2 b = __halves2half2(__float2half(1024.0f + Bias), __float2half(1024.0f + Bias));
        h = __hsub2(h, b);
        return *reinterpret_cast<uint32_t*>(&h);
    }

    // K index of digit a of the group's input element i.  Word-major (r = 8
    // fed by digits or limbs, rows of strided elements): the first DC digits
    // at (a / 4) * 4r + 4i + a % 4,
    // so one 16-byte piece holds the four digits of one word of two elements;
    // otherwise (and for the carry digits past DC) a * r + i
    __host__ __device__ __forceinline__ uint32_t tc_k_index(uint32_t a, uint32_t i, uint32_t r, uint32_t dc,
                                                            bool word_major)
    {
        return word_major && a < dc ? (a / 4u) * 4u * r + 4u * i + a % 4u : a * r + i;
    }

    __device__ __forceinline__ void st_shared_v4(uint8_t* p, uint32_t a, uint32_t b, uint32_t c, uint32_t d)
    {
        asm volatile("st.shared.v4.u32 [%0], {%1, %2, %3, %4};" ::"r"(tc::smem_u32(p)), "r"(a), "r"(b), "r"(c),
                     "r"(d)
                     : "memory");
    }

    __device__ __forceinline__ void st_shared_u32(uint8_t* p, uint32_t a)
    {
        asm volatile("st.shared.u32 [%0], %1;" ::"r"(tc::smem_u32(p)), "r"(a) : "memory");
    }

    // position of a tile in the CTA's contiguous range, advanced without division
    struct TcCursor
    {
        uint64_t hb;   // block * NS + split
        uint32_t mt;   // 128-row tile within the block
        uint32_t jb;   // index of the block in this CTA's range

        __device__ __forceinline__ TcCursor next(uint32_t tiles_per_block) const
        {
            TcCursor c = *this;
            if (++c.mt == tiles_per_block)
            {
                c.mt = 0;
                ++c.hb;
                ++c.jb;
            }
            return c;
        }
    };

    struct TcRow
    {
        bool ok;
        uint64_t base;  // element index of m = 0
        uint64_t poly;
    };

    template<int G>
    __device__ __forceinline__ TcRow tc_row(const TcGroupParams& p, uint64_t h, uint32_t mt, uint32_t row)
    {
        const uint64_t rho = static_cast<uint64_t>(mt) * tc_rows + row;
        TcRow r;
        r.ok = rho < p.rows;
        r.poly = rho >> p.lo;
        r.base = (r.poly << p.log_n) + (h << (p.lo + G)) + (rho & ((1ull << p.lo) - 1ull));
        return r;
    }

    // loader of digit / limb tiles: thread (row, part) owns words part, part +
    // tc_parts, ... of the row's R elements
    // InBlk: the input digit planes are blocked per R adjacent elements (word w
    // of element e at (e - e mod R) * W + w * R + e mod R): a row is one run
    // WordMajor: r = 8 tiles take the word-major K order of tc_k_index
    // Polys: the group's limb input is one buffer per polynomial (in_polys)
    template<int DC, int R, int IN, int NS, int Parts, bool InBlk = false, bool WordMajor = false, bool Polys = false>
    struct TcLoader
    {
        using S = TcShape<DC, R, IN, NS>;
        static constexpr int tc_parts = Parts;
        static constexpr int wh = S::w_in > 0 ? (S::w_in + tc_parts - 1) / tc_parts : 1;
        uint32_t v[wh][R];

        __device__ __forceinline__ void load(const TcGroupParams& p, uint64_t h, uint32_t mt, uint32_t tid)
        {
            const uint32_t row = tid % tc_rows, part = tid / tc_rows;
            const TcRow r = tc_row<S::g>(p, h, mt, row);
            const uint32_t* rp = p.in + r.base;
            uint64_t stride = p.elements;
            if constexpr (Polys && IN == tc_in_limbs)
            {
                // the row's polynomial in its own buffer (read only for rows in range)
                stride = 1ull << p.log_n;
                rp = r.ok ? p.in_polys[r.poly] + (r.base & (stride - 1ull)) : p.in;
            }
            const bool contiguous = p.lo == 0;  // the row's R elements are adjacent: vector loads
#pragma unroll
            for (int wi = 0; wi < wh; ++wi)
            {
                const uint32_t w = part + tc_parts * wi;
                const bool live = r.ok && w < static_cast<uint32_t>(S::w_in);
                const uint32_t* wp = InBlk ? p.in + r.base * S::w_in + w * R : rp + w * stride;
                if (live && contiguous)
                {
                    if constexpr (R == 8)
                    {
                        const uint4 a = __ldg(reinterpret_cast<const uint4*>(wp));
                        const uint4 b = __ldg(reinterpret_cast<const uint4*>(wp) + 1);
                        v[wi][0] = a.x; v[wi][1] = a.y; v[wi][2] = a.z; v[wi][3] = a.w;
                        v[wi][4] = b.x; v[wi][5] = b.y; v[wi][6] = b.z; v[wi][7] = b.w;
                    }
                    else if constexpr (R == 4)
                    {
                        const uint4 a = __ldg(reinterpret_cast<const uint4*>(wp));
                        v[wi][0] = a.x; v[wi][1] = a.y; v[wi][2] = a.z; v[wi][3] = a.w;
                    }
                    else
                    {
                        const uint2 a = __ldg(reinterpret_cast<const uint2*>(wp));
                        v[wi][0] = a.x; v[wi][1] = a.y;
                    }
                }
                else
                {
#pragma unroll
                    for (int m = 0; m < R; ++m)
                    {
                        v[wi][m] = live ? __ldg(wp + (static_cast<uint64_t>(m) << p.lo)) : 0u;
                    }
                }
            }
        }

        __device__ __forceinline__ void store(uint8_t* sa, uint32_t tid) const
        {
            const uint32_t row = tid % tc_rows, part = tid / tc_rows;
            constexpr int bias = IN == tc_in_digits ? 128 : 0;
#pragma unroll
            for (int wi = 0; wi < wh; ++wi)
            {
                const uint32_t w = part + tc_parts * wi;
                if (w >= static_cast<uint32_t>(S::w_in))
                {
                    continue;
                }
                if constexpr (R == 8)
                {
                    if (WordMajor && w < static_cast<uint32_t>(DC / 4))
                    {
                        // word-major K (tc_k_index): elements 2 mp and 2 mp + 1 per piece
#pragma unroll
                        for (uint32_t mp = 0; mp < 4; ++mp)
                        {
                            st_shared_v4(sa + tc::operand_offset(row, 32 * w + 8 * mp, tc_rows),
                                         byte_pair_to_half2<bias>(v[wi][2 * mp], 0),
                                         byte_pair_to_half2<bias>(v[wi][2 * mp], 2),
                                         byte_pair_to_half2<bias>(v[wi][2 * mp + 1], 0),
                                         byte_pair_to_half2<bias>(v[wi][2 * mp + 1], 2));
                        }
                    }
                    else
                    {
                        // K = a * 8 + m (and the carry digits past DC in word-major order)
#pragma unroll
                        for (uint32_t t = 0; t < 4; ++t)
                        {
                            const uint32_t a = 4 * w + t;
                            if (a < static_cast<uint32_t>(S::d_eff))
                            {
                                st_shared_v4(sa + tc::operand_offset(row, a * 8, tc_rows),
                                             bytes_to_half2<bias>(v[wi][0], v[wi][1], t),
                                             bytes_to_half2<bias>(v[wi][2], v[wi][3], t),
                                             bytes_to_half2<bias>(v[wi][4], v[wi][5], t),
                                             bytes_to_half2<bias>(v[wi][6], v[wi][7], t));
                            }
                        }
                    }
                }
                else if constexpr (R == 4)
                {
#pragma unroll
                    for (uint32_t t = 0; t < 4; t += 2)
                    {
                        const uint32_t a = 4 * w + t;
                        if (a < static_cast<uint32_t>(S::d_eff))
                        {
                            st_shared_v4(sa + tc::operand_offset(row, a * 4, tc_rows),
                                         bytes_to_half2<bias>(v[wi][0], v[wi][1], t),
                                         bytes_to_half2<bias>(v[wi][2], v[wi][3], t),
                                         bytes_to_half2<bias>(v[wi][0], v[wi][1], t + 1),
                                         bytes_to_half2<bias>(v[wi][2], v[wi][3], t + 1));
                        }
                    }
                }
                else
                {
                    st_shared_v4(sa + tc::operand_offset(row, 8 * w, tc_rows),
                                 bytes_to_half2<bias>(v[wi][0], v[wi][1], 0),
                                 bytes_to_half2<bias>(v[wi][0], v[wi][1], 1),
                                 bytes_to_half2<bias>(v[wi][0], v[wi][1], 2),
                                 bytes_to_half2<bias>(v[wi][0], v[wi][1], 3));
                }
            }
        }
    };

    __device__ __forceinline__ void st_shared_u16(uint8_t* p, uint16_t a)
    {
        asm volatile("st.shared.u16 [%0], %1;" ::"r"(tc::smem_u32(p)), "h"(a) : "memory");
    }

    __device__ __forceinline__ void st_shared_v2(uint8_t* p, uint32_t a, uint32_t b)
    {
        asm volatile("st.shared.v2.u32 [%0], {%1, %2};" ::"r"(tc::smem_u32(p)), "r"(a), "r"(b) : "memory");
    }

    // The pair of centred binomial values of one stage-0 generator: the first
    // ceil(2V/32) keystream words for the first sample, the next as many for
    // the second, the top word of each masked to 2V mod 32 bits, popcount - V'
    // with V' = 2V / 2 (hmpc/random/binomial.hpp:29-86,110-122).  BGV's two
    // variances (2V = 1 for the secret and u, 2V = 20 for the noise) take
    // compile-time word counts, so only the keystream words they consume are
    // computed and the masks fold away; other variances draw eight words.
    __device__ __forceinline__ void tc_cbd_pair(const TcGroupParams& p, const ChachaPre& pre, uint32_t counter,
                                                int& a, int& b)
    {
        if (p.vx2 == 20)
        {
            uint32_t w[4];
            chacha_stream<4>(pre, p.rng, counter, w);
            a = __popc(w[0]) + __popc(w[1] & 0xffu) - 20;
            b = __popc(w[2]) + __popc(w[3] & 0xffu) - 20;
            return;
        }
        if (p.vx2 == 1)
        {
            uint32_t w[2];
            chacha_stream<2>(pre, p.rng, counter, w);
            a = __popc(w[0] & 3u) - 1;
            b = __popc(w[1] & 3u) - 1;
            return;
        }
        const int count = 2 * static_cast<int>(p.vx2);
        const int nw = static_cast<int>(p.nw);
        uint32_t w[8];
        chacha_stream<8>(pre, p.rng, counter, w);
        a = 0;
        b = 0;
#pragma unroll
        for (int i = 0; i < 8; ++i)
        {
            const int iv = i - nw;  // word of the second sample
            uint32_t mu = 0u, mv = 0u;
            if (i < nw)
            {
                mu = (i == nw - 1 && (count & 31)) ? (1u << (count & 31)) - 1u : 0xffffffffu;
            }
            else if (iv < nw)
            {
                mv = (iv == nw - 1 && (count & 31)) ? (1u << (count & 31)) - 1u : 0xffffffffu;
            }
            a += __popc(w[i] & mu);
            b += __popc(w[i] & mv);
        }
        a -= static_cast<int>(p.vx2);
        b -= static_cast<int>(p.vx2);
    }

    // first forward group fed by centred binomial samples: r = 8, stage-0 pairs
    // (m, m + 4) of a row come from one generator with counter = poly * N +
    // index of the first element, first draw for m, second for m + 4
    // (number_theoretic_transform.hpp:316-329, comp/queue.hpp:191-212); thread
    // (row, part) draws the pair m = part
    __device__ __forceinline__ void tc_store_cbd(const TcGroupParams& p, const ChachaPre& pre, uint8_t* sa,
                                                 uint32_t mt, uint32_t tid)
    {
        // the four threads of a row are adjacent lanes: a warp's stores cover eight whole segment rows
        const uint32_t row = tid >> 2, part = tid & 3u;
        const TcRow r = tc_row<3>(p, 0, mt, row);
        int e_u = 0, e_v = 0;
        if (r.ok)
        {
            const uint64_t idx = r.base + (static_cast<uint64_t>(part) << p.lo);
            tc_cbd_pair(p, pre, static_cast<uint32_t>(idx), e_u, e_v);
        }
        uint8_t* seg = sa + tc::operand_offset(row, 0, tc_rows);
        const __half hu = __int2half_rn(e_u), hv = __int2half_rn(e_v);
        st_shared_u16(seg + 2 * part, *reinterpret_cast<const uint16_t*>(&hu));
        st_shared_u16(seg + 8 + 2 * part, *reinterpret_cast<const uint16_t*>(&hv));
    }

    // canonical value of a residue mod p (one or two limbs, Montgomery form),
    // lifted to the centred integer in (-p/2, p/2] (hmpc/ints/mod.hpp:259-307:
    // the canonical value v becomes v - p when v > floor(p/2))
    // (m: the residue's limbs as loaded)
    __device__ __forceinline__ long long tc_centred_lift(const TcGroupParams& p, const uint32_t (&m)[2])
    {
        // word-by-word Montgomery reduction by 2^(32 lp) (core/num/modulo.hpp:30-66),
        // written out for one and two limbs so no scratch array is indexed
        const bool two = p.msg_limbs > 1;
        const uint64_t q = p.pq[0] | (two ? static_cast<uint64_t>(p.pq[1]) << 32 : 0ull);
        const uint64_t half = p.phalf[0] | (two ? static_cast<uint64_t>(p.phalf[1]) << 32 : 0ull);
        uint64_t v;
        if (two)
        {
            unsigned __int128 t = (static_cast<uint64_t>(m[1]) << 32) | m[0];
            t += static_cast<unsigned __int128>(m[0] * p.pninv) * q;  // low word becomes 0
            t >>= 32;
            t += static_cast<unsigned __int128>(static_cast<uint32_t>(t) * p.pninv) * q;
            t >>= 32;  // < 2q
            v = static_cast<uint64_t>(t);
            if ((t >> 64) != 0 || v >= q)
            {
                v -= q;
            }
        }
        else
        {
            const uint64_t t = (static_cast<uint64_t>(m[0] * p.pninv) * p.pq[0] + m[0]) >> 32;  // <= q
            v = t >= q ? t - q : t;
        }
        return v > half ? static_cast<long long>(v) - static_cast<long long>(q) : static_cast<long long>(v);
    }

    // first forward group fed by x = p * e + lift(m): e drawn as the CBD
    // loader draws it (one generator per stage-0 pair, thread (row, part) draws
    // the pair m = part, m + 4), m the plaintext residue of the same element;
    // x (|x| < 2^70) is written as its 8 low bytes (unsigned digits) and the
    // signed value x >> 64 (K index = a * 8 + m)
    __device__ __forceinline__ void tc_store_small(const TcGroupParams& p, const ChachaPre& pre, uint8_t* sa,
                                                   uint32_t mt, uint32_t tid)
    {
        const uint32_t row = tid >> 2, part = tid & 3u;
        const TcRow r = tc_row<3>(p, 0, mt, row);
        __int128 x[2] = {0, 0};
        if (r.ok)
        {
            const uint64_t idx = r.base + (static_cast<uint64_t>(part) << p.lo);
            // the plaintext loads go out before the keystream is computed, so
            // their latency hides behind it
            uint32_t msg[2][2] = {{0u, 0u}, {0u, 0u}};
            if (p.msg)
            {
#pragma unroll
                for (int j = 0; j < 2; ++j)
                {
                    const uint64_t e = idx + (static_cast<uint64_t>(4 * j) << p.lo);
                    msg[j][0] = __ldcs(p.msg + e);
                    msg[j][1] = p.msg_limbs > 1 ? __ldcs(p.msg + p.msg_stride + e) : 0u;
                }
            }
            int a = 0, b = 0;
            tc_cbd_pair(p, pre, static_cast<uint32_t>(idx), a, b);
            const uint64_t pval = p.pq[0] | (p.msg_limbs > 1 ? static_cast<uint64_t>(p.pq[1]) << 32 : 0ull);
            x[0] = static_cast<__int128>(pval) * a;
            x[1] = static_cast<__int128>(pval) * b;
            if (p.msg)
            {
                x[0] += tc_centred_lift(p, msg[0]);
                x[1] += tc_centred_lift(p, msg[1]);
            }
        }
#pragma unroll
        for (int j = 0; j < 2; ++j)
        {
            const uint64_t lo = static_cast<uint64_t>(x[j]);
            const int hi = static_cast<int>(static_cast<long long>(x[j] >> 64));
#pragma unroll
            for (int d = 0; d < tc_small_digits; ++d)
            {
                const int digit = d < 8 ? static_cast<int>((lo >> (8 * d)) & 255u) : hi;
                const __half h = __int2half_rn(digit);
                st_shared_u16(sa + tc::operand_offset(row, d * 8 + part + 4 * j, tc_rows),
                              *reinterpret_cast<const uint16_t*>(&h));
            }
        }
    }

    __device__ __forceinline__ uint32_t pack_bytes(uint32_t b0, uint32_t b1, uint32_t b2, uint32_t b3)
    {
        return __byte_perm(__byte_perm(b0, b1, 0x0040), __byte_perm(b2, b3, 0x0040), 0x5410);
    }

    // Carry of exact f32 column sums into balanced base-256 digits, in f32.
    // With t = s + carry + 128 the digit is t mod 256 - 128 and the next carry
    // floor(t / 256).  The state x = floor(t / 256) + 2^23 also equals
    // (next carry + 128) + C with C = 2^23 + 2^15, so the next t + C is s + x:
    // four exact operations per digit (every value an integer below 2^24).
    struct DigitCarry
    {
        float x = 8421504.0f;  // carry 0: 128 + C

        __device__ __forceinline__ uint32_t step(float s)
        {
            const float tc = s + x;                        // t + C
            x = __fmaf_rd(tc, 0.00390625f, 8388608.0f);    // floor((t + C) / 256) + 2^23
            const float z = x - 8421376.0f;                // next carry + 128
            return __float_as_uint(__fmaf_rn(-256.0f, z, tc));  // 2^23 + digit + 128
        }

        // the carry out of the last digit
        __device__ __forceinline__ int carry() const
        {
            return static_cast<int>(__float_as_uint(x) - 0x4B000000u) - 32896;
        }
    };

    // The same carry in two operations per digit where |t| < 2^22 - 2^15: with
    // C2 = 2^23 + 2^22 every T = t + C2 lies in [2^23, 2^24), where a float's
    // mantissa is T - 2^23 exactly, so the low byte of T's bits is t mod 256 --
    // the biased digit, read from T itself.  The state x = floor(T / 256) +
    // C2 - C2 / 256 + 128 equals (next carry + 128) + C2, so the next T is s + x.
    // Sums of a group fed by digits (|x| <= 128) stay in range when every
    // constant column's sum of |digit| is at most 32512: checked when the
    // group's constants are built.  Fed by limbs (unsigned bytes) they may not.
    struct DigitCarryByte
    {
        float x = 12583040.0f;  // carry 0: 128 + C2

        __device__ __forceinline__ uint32_t step(float s)
        {
            const float t = s + x;                          // t + C2
            x = __fmaf_rd(t, 0.00390625f, 12533888.0f);     // floor((t + C2) / 256) + C2 - C2 / 256 + 128
            return __float_as_uint(t);
        }

        __device__ __forceinline__ int carry() const
        {
            return static_cast<int>(__float_as_uint(x) - 0x4B000000u) - 4194432;
        }
    };

    // the DC column sums of one output element: one TMEM load of 32, or
    // loads of 16, 8 and 4 consecutive columns that add up to DC (digit counts
    // of 2..8 limbs), completed by one wait
    template<int DC>
    __device__ __forceinline__ void tc_load_sums(uint32_t taddr, uint32_t (&s)[DC])
    {
        static_assert(DC % 4 == 0 && DC >= 8 && DC <= 32, "digit counts of 2 to 8 limbs");
        if constexpr (DC == 32)
        {
            tc::tmem_load<32>(taddr, s);
        }
        else
        {
            constexpr int a16 = DC & 16, a8 = DC & 8, a4 = DC & 4;
            if constexpr (a16 != 0)
            {
                tc::tmem_load<16>(taddr, *reinterpret_cast<uint32_t(*)[16]>(&s[0]));
            }
            if constexpr (a8 != 0)
            {
                tc::tmem_load<8>(taddr + a16, *reinterpret_cast<uint32_t(*)[8]>(&s[a16]));
            }
            if constexpr (a4 != 0)
            {
                tc::tmem_load<4>(taddr + a16 + a8, *reinterpret_cast<uint32_t(*)[4]>(&s[a16 + a8]));
            }
        }
    }

    // the signed value sum_j x_j 2^(32 j) + top 2^(32 L), |value / q| < 2^15,
    // reduced into [0, q).  The quotient estimate reads the value's top word
    // top * 2^32 + x[L-1] as one signed 64-bit integer converted once to f32
    // (relative error 2^-24, so at most 2^-9 in the quotient), then scales by
    // 2^(32(L-1)) / q; the dropped limbs add at most 1 / 32 for a top limb of
    // q >= 32.  The estimate is within one of the quotient: one correction each
    // way.  (Converting x[L-1] to f32 on its own would round a word near 2^32
    // by up to 128 before a negative top cancels it -- 128 / 32 quotient units
    // at the smallest top limb.)
    template<int L>
    __device__ __forceinline__ void tc_reduce(uint32_t (&x)[L], int top, const TcGroupParams& p)
    {
        const long long top_word = static_cast<long long>(top) * 4294967296ll + static_cast<long long>(x[L - 1]);
        const float est = static_cast<float>(top_word) * p.inv_q_top;
        const int t = __float2int_rd(est);
        long long carry = 0;
#pragma unroll
        for (int j = 0; j < L; ++j)
        {
            const long long acc = static_cast<long long>(x[j]) - static_cast<long long>(t) * p.q[j] + carry;
            x[j] = static_cast<uint32_t>(acc);
            carry = acc >> 32;
        }
        int rt = top + static_cast<int>(carry);
        if (rt < 0)
        {
            uint32_t c = 0;
#pragma unroll
            for (int j = 0; j < L; ++j)
            {
                const unsigned long long s = static_cast<unsigned long long>(x[j]) + p.q[j] + c;
                x[j] = static_cast<uint32_t>(s);
                c = static_cast<uint32_t>(s >> 32);
            }
            rt += static_cast<int>(c);
        }
        bool ge = rt > 0;
        if (!ge)
        {
            ge = true;  // x == q counts as >= q
#pragma unroll
            for (int j = L - 1; j >= 0; --j)
            {
                if (x[j] != p.q[j])
                {
                    ge = x[j] > p.q[j];
                    break;
                }
            }
        }
        if (ge)
        {
            uint32_t b = 0;
#pragma unroll
            for (int j = 0; j < L; ++j)
            {
                const unsigned long long s = static_cast<unsigned long long>(x[j]) - p.q[j] - b;
                x[j] = static_cast<uint32_t>(s);
                b = static_cast<uint32_t>(s >> 63);
            }
        }
    }

    template<int Per>
    __device__ __forceinline__ void store_run(uint32_t* p, const uint32_t (&v)[Per])
    {
        if constexpr (Per == 4)
        {
            *reinterpret_cast<uint4*>(p) = make_uint4(v[0], v[1], v[2], v[3]);
        }
        else if constexpr (Per == 2)
        {
            *reinterpret_cast<uint2*>(p) = make_uint2(v[0], v[1]);
        }
        else
        {
            p[0] = v[0];
        }
    }

    // carry the accumulator of one tile out of TMEM: each thread owns one row
    // and `per` consecutive output elements of the block's split; Contig: the
    // row's elements are adjacent (no column bits), stored as vectors;
    // ByteCarry: the two-operation carry (inputs other than limbs)
    template<int DC, int R, int OUT, int NS, bool Contig, bool OutRec, bool ByteCarry, bool Polys>
    __device__ __forceinline__ void tc_epilogue(const TcGroupParams& p, uint32_t tmem, const TcCursor& cur,
                                                uint32_t warp, uint32_t lane)
    {
        constexpr int g = R == 64 ? 6 : (R == 8 ? 3 : (R == 4 ? 2 : 1));
        constexpr int L = DC / 4;
        constexpr int W = (DC + 2 + 3) / 4;
        constexpr int outputs = R / NS;
        constexpr int kgroups = tc_workers<Contig> / tc_rows;  // warps sharing a TMEM lane quadrant
        constexpr int per = outputs >= kgroups ? outputs / kgroups : 1;
        constexpr int words_out = OUT == tc_out_digits ? W : L;
        if ((warp >> 2) * per >= static_cast<uint32_t>(outputs))
        {
            return;  // more warps than output elements (R = 2)
        }
        const uint32_t lg = warp & 3u;
        const uint32_t row = 32u * lg + lane;
        const uint64_t h = cur.hb / NS;
        const uint32_t split = static_cast<uint32_t>(cur.hb % NS);
        const TcRow r = tc_row<g>(p, h, cur.mt, row);
        const uint32_t kl0 = (warp >> 2) * per;      // first local output of this thread
        const uint32_t k0 = split * outputs + kl0;   // its element index in the group
        uint32_t* op = p.out + r.base;
        uint64_t ostride = p.elements;
        if constexpr (Polys && OUT == tc_out_limbs)
        {
            // the row's polynomial in its own buffer (written only for rows in range)
            ostride = 1ull << p.log_n;
            op = r.ok ? p.out_polys[r.poly] + (r.base & (ostride - 1ull)) : p.out;
        }
        uint32_t res[Contig ? words_out : 1][Contig ? per : 1];
#pragma unroll
        for (int kk = 0; kk < per; ++kk)
        {
            uint32_t s[DC];
            tc_load_sums<DC>(tmem + ((32u * lg) << 16) + (kl0 + kk) * DC, s);
            tc::tmem_load_wait();
            std::conditional_t<ByteCarry, DigitCarryByte, DigitCarry> carry;
            uint32_t words[W];
            uint32_t bb[4];
#pragma unroll
            for (int b = 0; b < DC; ++b)
            {
                bb[b & 3] = carry.step(__uint_as_float(s[b]));
                if ((b & 3) == 3)
                {
                    words[b >> 2] = pack_bytes(bb[0], bb[1], bb[2], bb[3]);
                }
            }
            if constexpr (OUT == tc_out_digits)
            {
                const uint32_t c0 = carry.step(0.0f);
                const uint32_t c1 = carry.step(0.0f);
                words[DC / 4] = pack_bytes(c0, c1, 0x80u, 0x80u);
            }
            else
            {
                // value = (packed biased bytes) - 0x8080..80 + carry * 2^(8 DC)
                uint32_t x[L];
                uint32_t borrow = 0;
#pragma unroll
                for (int j = 0; j < L; ++j)
                {
                    const unsigned long long d = static_cast<unsigned long long>(words[j]) - 0x80808080u - borrow;
                    x[j] = static_cast<uint32_t>(d);
                    borrow = static_cast<uint32_t>(d >> 63);
                }
                tc_reduce<L>(x, carry.carry() - static_cast<int>(borrow), p);
#pragma unroll
                for (int j = 0; j < L; ++j)
                {
                    words[j] = x[j];
                }
            }
            if constexpr (Contig)
            {
#pragma unroll
                for (int w = 0; w < words_out; ++w)
                {
                    res[w][kk] = words[w];
                }
            }
            else if (r.ok)
            {
                const uint64_t e = static_cast<uint64_t>(k0 + kk) << p.lo;
                if constexpr (OutRec)
                {
                    // digit planes blocked per 2^block_shift elements, for a next
                    // group whose rows are that many adjacent elements
                    const uint64_t ea = r.base + e;
                    const uint64_t m = ea & ((1ull << p.block_shift) - 1ull);
                    uint32_t* blk = p.out + (ea - m) * W + m;
#pragma unroll
                    for (int w = 0; w < words_out; ++w)
                    {
                        blk[static_cast<uint64_t>(w) << p.block_shift] = words[w];
                    }
                }
                else
                {
#pragma unroll
                    for (int w = 0; w < words_out; ++w)
                    {
                        op[w * ostride + e] = words[w];
                    }
                }
            }
        }
        if constexpr (Contig)
        {
            if (r.ok)
            {
#pragma unroll
                for (int w = 0; w < words_out; ++w)
                {
                    store_run<per>(op + w * ostride + k0, res[w]);
                }
            }
        }
    }

    __device__ __forceinline__ void mbar_arrive(uint64_t* bar)
    {
        asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(tc::smem_u32(bar)) : "memory");
    }

    // One CTA per SM, persistent over a contiguous range of tiles, warp-specialised:
    // warps 0-15 convert each 128-row digit tile into shared memory and carry
    // accumulators out of TMEM; one thread of warp 16 streams the constant
    // operands (bulk copies) and issues the MMAs.  mbarriers hand over the
    // digit tile (full: 512 arrivals; empty: MMA commit), the two TMEM
    // accumulators (full: MMA commit; empty: 512 arrivals) and the constant
    // buffers (transaction count).  Every wait is bounded; a timeout sets the
    // error word and both sides leave their loops.
    // Lay bit 0: the input digit planes are blocked per R adjacent elements;
    // bit 1: the output planes are blocked for the next group; bit 2: limb
    // input or output in one buffer per polynomial (in_polys / out_polys)
    template<int DC, int R, int IN, int OUT, int NS, bool Contig, int Lay>
    __global__ void __launch_bounds__(tc_workers<Contig> + 32, 1) tc_group_kernel(const TcGroupParams p)
    {
        using S = TcShape<DC, R, IN, NS>;
        constexpr int tc_threads = tc_workers<Contig>;
        static_assert(!TcShape<DC, R, IN, NS>::generated || tc_threads / tc_rows == 4,
                      "the sampling loaders draw one pair per thread");
        constexpr int NBUF = S::nbuf;
        extern __shared__ __align__(1024) uint8_t tc_smem[];
        uint8_t* sb = tc_smem;                           // NBUF constant buffers
        uint8_t* sa = tc_smem + NBUF * S::b_bytes;       // the digit tile
        uint64_t* bars = reinterpret_cast<uint64_t*>(sa + S::a_bytes);
        uint64_t* bar_b = bars;           // [2] constants full
        uint64_t* bar_a_full = bars + 2;  // digit tile stored (one arrival per worker)
        uint64_t* bar_a_empty = bars + 3; // MMAs of the tile complete (commit)
        uint64_t* bar_acc_full = bars + 4;   // [2] accumulator ready (commit)
        uint64_t* bar_acc_empty = bars + 6;  // [2] accumulator read out (one arrival per worker)
        uint64_t* bar_k0 = bars + 8;         // MMAs on the first K half complete (commit)
        uint32_t* tslot = reinterpret_cast<uint32_t*>(bars + 9);
        volatile uint32_t* abort_flag = tslot + 1;
        uint64_t* bar_never = bars + 10;     // test hook: no thread arrives here
        static_assert(11 * sizeof(uint64_t) <= S::control_bytes, "control block");

        const uint32_t tid = threadIdx.x;
        const uint32_t warp = tid >> 5, lane = tid & 31u;
        // a dependent launch (the next group) may be scheduled once every CTA
        // of this one is resident; its CTAs land on SMs as these exit
        asm volatile("griddepcontrol.launch_dependents;" ::: "memory");

        const uint64_t t_begin = p.tiles * blockIdx.x / gridDim.x;
        const uint64_t t_end = p.tiles * (blockIdx.x + 1) / gridDim.x;
        const uint64_t count = t_end - t_begin;
        const uint32_t tpb = p.tiles_per_block;
        const uint64_t hb_first = t_begin / tpb;
        const uint64_t hb_last = count ? (t_end - 1) / tpb : hb_first;
        const TcCursor first{hb_first, static_cast<uint32_t>(t_begin - hb_first * tpb), 0};

        // K padding of the A tile stays zero
        constexpr uint32_t pad_units = static_cast<uint32_t>(S::k_pad - S::k_real) / 8 * tc_rows;
        if constexpr (pad_units > 0)
        {
            for (uint32_t u = tid; u < pad_units; u += tc_threads + 32)
            {
                st_shared_v4(sa + tc::operand_offset(u % tc_rows, S::k_real + 8 * (u / tc_rows), tc_rows), 0, 0, 0,
                             0);
            }
        }
        if (tid == 0)
        {
            tc::mbar_init(&bar_b[0], 1);
            tc::mbar_init(&bar_b[1], 1);
            tc::mbar_init(bar_a_full, tc_threads);
            tc::mbar_init(bar_a_empty, 1);
            tc::mbar_init(&bar_acc_full[0], 1);
            tc::mbar_init(&bar_acc_full[1], 1);
            tc::mbar_init(&bar_acc_empty[0], tc_threads);
            tc::mbar_init(&bar_acc_empty[1], tc_threads);
            tc::mbar_init(bar_k0, 1);
            tc::mbar_init(bar_never, 1);
            *abort_flag = 0;
            tc::mbar_init_fence();
        }
        if (warp == 0)
        {
            tc::tmem_alloc(tslot, 2 * S::cols);
        }
        tc::fence_proxy_async();
        tc::fence_before_sync();
        __syncthreads();
        tc::fence_after_sync();
        const uint32_t tmem = *tslot;

        auto give_up = [&](uint32_t code) {
            atomicExch(p.error, code);
            *abort_flag = 1;
        };

        if (warp == tc_threads / 32)
        {
            // ------------------------------------------------ MMA and copies
            // Two constant buffers (NBUF 2): block jb's image goes to buffer jb % 2
            // as soon as block jb - 2's MMAs are complete.  One buffer (NBUF 1): the
            // image arrives in two K halves on their own barriers, the first as
            // soon as the previous block's MMAs on the first half completed, so the
            // next block's constants stream in while the last tile finishes.
            if (lane == 0 && count)
            {
                constexpr uint32_t idesc = tc::f16_instr_descriptor(tc_rows, S::n_mma);
                constexpr int ks_total = S::k_pad / 16;
                constexpr int ks_half = NBUF == 1 ? (ks_total + 1) / 2 : ks_total;
                constexpr uint32_t h0_bytes = NBUF == 1 ? 2u * ks_half * S::lbo_b : S::b_bytes;
                // copies issued and waited for per barrier (scalars: an indexed
                // array would live in local memory on this thread's issue path):
                // on an abort the copies still in flight are waited for
                // (bounded) before the CTA exits
                uint32_t issued0 = 0, issued1 = 0, landed0 = 0, landed1 = 0;
                auto copy = [&](uint32_t jb, uint32_t piece) {
                    // NBUF 2: piece = buffer (whole image); NBUF 1: piece = K half
                    issued0 += piece == 0u ? 1u : 0u;
                    issued1 += piece != 0u ? 1u : 0u;
                    const uint8_t* src = p.images + (hb_first + jb) * S::b_bytes;
                    if constexpr (NBUF == 2)
                    {
                        tc::mbar_arrive_expect_tx(&bar_b[piece], S::b_bytes);
                        tc::bulk_g2s(sb + piece * S::b_bytes, src, S::b_bytes, &bar_b[piece]);
                    }
                    else
                    {
                        const uint32_t off = piece ? h0_bytes : 0u;
                        const uint32_t bytes = piece ? S::b_bytes - h0_bytes : h0_bytes;
                        tc::mbar_arrive_expect_tx(&bar_b[piece], bytes);
                        tc::bulk_g2s(sb + off, src + off, bytes, &bar_b[piece]);
                    }
                };
                copy(0, 0);
                if (NBUF == 1 || hb_first + 1 <= hb_last)
                {
                    copy(NBUF == 1 ? 0u : 1u, 1);
                }
                TcCursor cur = first;
                uint32_t prev_jb = ~0u;
                for (uint64_t i = 0; i < count && !*abort_flag; ++i)
                {
                    const uint32_t acc = static_cast<uint32_t>(i & 1u);
                    const uint32_t prev = static_cast<uint32_t>((i - 1) & 1u);
                    const bool new_block = cur.jb != prev_jb;
                    if (new_block && i > 0)
                    {
                        if constexpr (NBUF == 1)
                        {
                            if (!tc::mbar_wait(bar_k0, prev, p.spin_limit))
                            {
                                give_up(3);
                                break;
                            }
                            copy(cur.jb, 0);
                            if (!tc::mbar_wait(bar_a_empty, prev, p.spin_limit))
                            {
                                give_up(3);
                                break;
                            }
                            copy(cur.jb, 1);
                        }
                        else if (hb_first + prev_jb + 2 <= hb_last)
                        {
                            if (!tc::mbar_wait(bar_a_empty, prev, p.spin_limit))
                            {
                                give_up(3);
                                break;
                            }
                            copy(prev_jb + 2, prev_jb % 2);
                        }
                    }
                    // the longest wait of this thread: sleeping in it leaves the
                    // issue slots of its sub-partition to the workers
                    if (!tc::mbar_wait_sleep(bar_a_full, static_cast<uint32_t>(i & 1u), p.spin_limit, 200u))
                    {
                        give_up(4);
                        break;
                    }
                    if (p.test_stall && i == 0 && !tc::mbar_wait(bar_never, 0u, p.spin_limit))
                    {
                        give_up(8);
                        break;
                    }
                    if (i >= 2 && !tc::mbar_wait(&bar_acc_empty[acc], static_cast<uint32_t>(((i - 2) >> 1) & 1u),
                                                 p.spin_limit))
                    {
                        give_up(5);
                        break;
                    }
                    const uint32_t piece0 = NBUF == 1 ? 0u : cur.jb % 2;
                    const uint32_t parity = NBUF == 1 ? (cur.jb & 1u) : ((cur.jb / 2) & 1u);
                    if (new_block)
                    {
                        if (!tc::mbar_wait(&bar_b[piece0], parity, p.spin_limit))
                        {
                            give_up(1);
                            break;
                        }
                        landed0 += piece0 == 0u ? 1u : 0u;
                        landed1 += piece0 != 0u ? 1u : 0u;
                    }
                    tc::fence_after_sync();
                    const uint32_t a0 = tc::smem_u32(sa);
                    const uint32_t b0 = tc::smem_u32(sb + (NBUF == 1 ? 0u : (cur.jb % 2) * S::b_bytes));
#pragma unroll
                    for (int ks = 0; ks < ks_half; ++ks)
                    {
                        tc::mma_f16(tmem + acc * S::cols, tc::smem_descriptor(a0 + ks * 2 * S::lbo_a, S::lbo_a, 128),
                                    tc::smem_descriptor(b0 + ks * 2 * S::lbo_b, S::lbo_b, 128), idesc, ks > 0);
                    }
                    if constexpr (NBUF == 1)
                    {
                        tc::mma_commit(bar_k0);
                        if (new_block)
                        {
                            if (!tc::mbar_wait(&bar_b[1], parity, p.spin_limit))
                            {
                                give_up(1);
                                break;
                            }
                            ++landed1;
                        }
                        tc::fence_after_sync();
#pragma unroll
                        for (int ks = ks_half; ks < ks_total; ++ks)
                        {
                            tc::mma_f16(tmem + acc * S::cols,
                                        tc::smem_descriptor(a0 + ks * 2 * S::lbo_a, S::lbo_a, 128),
                                        tc::smem_descriptor(b0 + ks * 2 * S::lbo_b, S::lbo_b, 128), idesc, true);
                        }
                    }
                    tc::mma_commit(&bar_acc_full[acc]);
                    tc::mma_commit(bar_a_empty);
                    prev_jb = cur.jb;
                    cur = cur.next(tpb);
                }
                if (*abort_flag)
                {
                    // at most one copy per barrier is in flight (the next one into a
                    // buffer is issued after the previous one was waited for): let
                    // it land before the shared memory is released
                    if (issued0 > landed0)
                    {
                        tc::mbar_wait(&bar_b[0], landed0 & 1u, p.spin_limit);
                    }
                    if (issued1 > landed1)
                    {
                        tc::mbar_wait(&bar_b[1], landed1 & 1u, p.spin_limit);
                    }
                }
            }
        }
        else
        {
            // ------------------------------------------------ workers
            // the kernel before this one in the stream (launched with
            // programmatic dependence: the previous group) is complete and its
            // writes visible before any digit is read or any output written;
            // the constants the MMA thread streams meanwhile were complete
            // before that kernel started
            asm volatile("griddepcontrol.wait;" ::: "memory");
            constexpr bool in_blk = (Lay & 1) != 0;
            static_assert(!in_blk || (IN == tc_in_digits && Contig), "blocked input: adjacent rows");
            // word-major K where rows are columns of strided elements; the
            // contiguous last group measured faster with digit-major K
            TcLoader<DC, R, IN, NS, tc_threads / tc_rows, in_blk, !Contig, (Lay & 4) != 0> loader;
            TcCursor cur = first;
            if constexpr (!S::generated)
            {
                if (count)
                {
                    loader.load(p, cur.hb / NS, cur.mt, tid);
                }
            }
            // the sampling loaders' keystream blocks share one key and nonce
            const ChachaPre pre = S::generated ? chacha_pre(p.rng) : ChachaPre{};
            TcCursor prev = cur;
            for (uint64_t i = 0; i <= count; ++i)
            {
                if (i < count)
                {
                    // the previous tile's MMAs no longer read the digit tile
                    if (i > 0)
                    {
                        uint32_t ok = 1;
                        if (lane == 0)
                        {
                            ok = tc::mbar_wait_sleep(bar_a_empty, static_cast<uint32_t>((i - 1) & 1u),
                                                     p.spin_limit);
                        }
                        if (!__shfl_sync(0xffffffffu, ok, 0))
                        {
                            give_up(6);
                            break;
                        }
                    }
                    if constexpr (IN == tc_in_cbd)
                    {
                        tc_store_cbd(p, pre, sa, cur.mt, tid);
                    }
                    else if constexpr (IN == tc_in_small)
                    {
                        tc_store_small(p, pre, sa, cur.mt, tid);
                    }
                    else
                    {
                        loader.store(sa, tid);
                    }
                    tc::fence_proxy_async();
                    mbar_arrive(bar_a_full);
                    if constexpr (!S::generated)
                    {
                        if (i + 1 < count)
                        {
                            const TcCursor n1 = cur.next(tpb);
                            loader.load(p, n1.hb / NS, n1.mt, tid);
                        }
                    }
                }
                if (i > 0)
                {
                    // carry out the previous tile while the tensor core works on this one
                    const uint32_t acc = static_cast<uint32_t>((i - 1) & 1u);
                    uint32_t ok = 1;
                    if (lane == 0)
                    {
                        ok = tc::mbar_wait_sleep(&bar_acc_full[acc], static_cast<uint32_t>(((i - 1) >> 1) & 1u),
                                           p.spin_limit);
                    }
                    if (!__shfl_sync(0xffffffffu, ok, 0))
                    {
                        give_up(7);
                        break;
                    }
                    tc::fence_after_sync();
                    tc_epilogue<DC, R, OUT, NS, Contig, (Lay & 2) != 0, IN != tc_in_limbs, (Lay & 4) != 0>(
                        p, tmem + acc * S::cols, prev, warp, lane);
                    tc::fence_before_sync();
                    mbar_arrive(&bar_acc_empty[acc]);
                }
                if (*abort_flag)
                {
                    break;
                }
                prev = cur;
                cur = cur.next(tpb);
            }
        }
        __syncthreads();
        if (*abort_flag && tid == 0)
        {
            // give in-flight MMAs a bounded chance to land before the memory is released
            tc::mbar_wait(bar_a_empty, 0, p.spin_limit);
            tc::mbar_wait(bar_a_empty, 1, p.spin_limit);
        }
        __syncthreads();
        tc::fence_after_sync();
        if (warp == 0)
        {
            tc::tmem_dealloc(tmem, 2 * S::cols);
        }
    }

    // ------------------------------------------------------------- wide group
    // The first six forward stages of a transform fed by centred binomial
    // samples, in one group of r = 64: the samples are single digits, so the
    // 64 x 64 constant of the one block (the product of the first two
    // three-stage groups' matrices) streams through shared memory in eight
    // images of eight outputs each (K = 64, N = 256), while each 128-row
    // digit tile -- 8192 elements, one generator per stage-0 pair (m, m + 32)
    // -- is drawn once.  Per row tile: the workers draw and store the tile,
    // then carry out the eight accumulators as the MMA thread fills them
    // (two TMEM buffers of 256 columns, two image buffers).
    constexpr int tc_wide_r = 64;
    constexpr int tc_wide_splits = 8;
    constexpr uint32_t tc_wide_a_bytes = tc_rows * tc_wide_r * 2;       // K = 64 fp16
    constexpr uint32_t tc_wide_b_bytes = tc_wide_r * 256 * 2;           // K = 64, N = 256
    constexpr uint32_t tc_wide_control = 128;
    // at least half of an SM's shared memory: one CTA per SM, so its two
    // accumulators (all 512 TMEM columns) are always free
    constexpr uint32_t tc_wide_smem = 116u * 1024u;
    static_assert(tc_wide_a_bytes + 2 * tc_wide_b_bytes + tc_wide_control <= tc_wide_smem, "wide group smem");

    // the tile's CBD samples: thread (row, part) draws the pairs m = part + 4j
    // (j < 8) of its row: generator counter = index of element m, first
    // draw for m, second for m + 32 (number_theoretic_transform.hpp:316-329)
    __device__ __forceinline__ void tc_store_cbd_wide(const TcGroupParams& p, const ChachaPre& pre, uint8_t* sa,
                                                      uint32_t mt, uint32_t tid)
    {
        const uint32_t row = tid >> 2, part = tid & 3u;
        const TcRow r = tc_row<6>(p, 0, mt, row);
#pragma unroll 2
        for (uint32_t j = 0; j < 8; ++j)
        {
            const uint32_t m = part + 4u * j;
            int e_u = 0, e_v = 0;
            if (r.ok)
            {
                tc_cbd_pair(p, pre, static_cast<uint32_t>(r.base + (static_cast<uint64_t>(m) << p.lo)), e_u, e_v);
            }
            const __half hu = __int2half_rn(e_u), hv = __int2half_rn(e_v);
            st_shared_u16(sa + tc::operand_offset(row, m, tc_rows), *reinterpret_cast<const uint16_t*>(&hu));
            st_shared_u16(sa + tc::operand_offset(row, m + 32u, tc_rows), *reinterpret_cast<const uint16_t*>(&hv));
        }
    }

    // p.images: the eight images of the block (split s at s * tc_wide_b_bytes);
    // p.tiles: the row tiles (rows = batch << lo, lo = log N - 6); the output
    // is digit planes (stride p.elements)
    template<int DC>
    __global__ void __launch_bounds__(512 + 32, 1) tc_wide_kernel(const TcGroupParams p)
    {
        constexpr int tc_threads = 512;
        extern __shared__ __align__(1024) uint8_t tc_smem[];
        uint8_t* sb = tc_smem;                              // two image buffers
        uint8_t* sa = tc_smem + 2 * tc_wide_b_bytes;        // the digit tile
        uint64_t* bars = reinterpret_cast<uint64_t*>(sa + tc_wide_a_bytes);
        uint64_t* bar_b = bars;            // [2] image landed
        uint64_t* bar_bfree = bars + 2;    // [2] MMAs reading the image complete (commit)
        uint64_t* bar_a_full = bars + 4;   // tile stored (one arrival per worker)
        uint64_t* bar_a_empty = bars + 5;  // all eight splits' MMAs of the tile complete (commit)
        uint64_t* bar_acc_full = bars + 6;   // [2]
        uint64_t* bar_acc_empty = bars + 8;  // [2] one arrival per worker
        uint32_t* tslot = reinterpret_cast<uint32_t*>(bars + 10);
        volatile uint32_t* abort_flag = tslot + 1;
        static_assert(11 * sizeof(uint64_t) <= tc_wide_control, "control block");

        const uint32_t tid = threadIdx.x;
        const uint32_t warp = tid >> 5, lane = tid & 31u;
        asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
        const uint64_t t_begin = p.tiles * blockIdx.x / gridDim.x;
        const uint64_t t_end = p.tiles * (blockIdx.x + 1) / gridDim.x;
        const uint64_t count = t_end - t_begin;

        if (tid == 0)
        {
            for (int b = 0; b < 2; ++b)
            {
                tc::mbar_init(&bar_b[b], 1);
                tc::mbar_init(&bar_bfree[b], 1);
                tc::mbar_init(&bar_acc_full[b], 1);
                tc::mbar_init(&bar_acc_empty[b], tc_threads);
            }
            tc::mbar_init(bar_a_full, tc_threads);
            tc::mbar_init(bar_a_empty, 1);
            *abort_flag = 0;
            tc::mbar_init_fence();
        }
        if (warp == 0)
        {
            tc::tmem_alloc(tslot, 512);
        }
        tc::fence_proxy_async();
        tc::fence_before_sync();
        __syncthreads();
        tc::fence_after_sync();
        const uint32_t tmem = *tslot;

        auto give_up = [&](uint32_t code) {
            atomicExch(p.error, code);
            *abort_flag = 1;
        };

        if (warp == tc_threads / 32)
        {
            // ------------------------------------------------ MMA and copies
            if (lane == 0 && count)
            {
                constexpr uint32_t idesc = tc::f16_instr_descriptor(tc_rows, 256);
                constexpr uint32_t lbo_a = tc_rows / 8 * 128;
                constexpr uint32_t lbo_b = 256 / 8 * 128;
                const uint64_t total = count * tc_wide_splits;
                uint32_t issued0 = 0, issued1 = 0, landed0 = 0, landed1 = 0;
                auto copy = [&](uint32_t split) {
                    const uint32_t buf = split & 1u;
                    issued0 += buf == 0u ? 1u : 0u;
                    issued1 += buf != 0u ? 1u : 0u;
                    tc::mbar_arrive_expect_tx(&bar_b[buf], tc_wide_b_bytes);
                    tc::bulk_g2s(sb + buf * tc_wide_b_bytes, p.images + static_cast<uint64_t>(split) * tc_wide_b_bytes,
                                 tc_wide_b_bytes, &bar_b[buf]);
                };
                copy(0);
                copy(1);
                for (uint64_t i = 0; i < count && !*abort_flag; ++i)
                {
                    if (!tc::mbar_wait_sleep(bar_a_full, static_cast<uint32_t>(i & 1u), p.spin_limit, 200u))
                    {
                        give_up(14);
                        break;
                    }
                    for (uint32_t s = 0; s < static_cast<uint32_t>(tc_wide_splits); ++s)
                    {
                        const uint64_t j = i * tc_wide_splits + s;
                        const uint32_t buf = static_cast<uint32_t>(j & 1u);
                        const uint32_t par = static_cast<uint32_t>((j >> 1) & 1u);
                        if (!tc::mbar_wait(&bar_b[buf], par, p.spin_limit))
                        {
                            give_up(11);
                            break;
                        }
                        landed0 += buf == 0u ? 1u : 0u;
                        landed1 += buf != 0u ? 1u : 0u;
                        if (j >= 2 && !tc::mbar_wait(&bar_acc_empty[buf], static_cast<uint32_t>(((j - 2) >> 1) & 1u),
                                                     p.spin_limit))
                        {
                            give_up(15);
                            break;
                        }
                        tc::fence_after_sync();
                        const uint32_t a0 = tc::smem_u32(sa);
                        const uint32_t b0 = tc::smem_u32(sb + buf * tc_wide_b_bytes);
#pragma unroll
                        for (int ks = 0; ks < tc_wide_r / 16; ++ks)
                        {
                            tc::mma_f16(tmem + buf * 256u, tc::smem_descriptor(a0 + ks * 2 * lbo_a, lbo_a, 128),
                                        tc::smem_descriptor(b0 + ks * 2 * lbo_b, lbo_b, 128), idesc, ks > 0);
                        }
                        tc::mma_commit(&bar_acc_full[buf]);
                        tc::mma_commit(&bar_bfree[buf]);
                        if (s + 1 == static_cast<uint32_t>(tc_wide_splits))
                        {
                            tc::mma_commit(bar_a_empty);
                        }
                        if (j + 2 < total)
                        {
                            // the image buffer is free once these MMAs complete
                            if (!tc::mbar_wait(&bar_bfree[buf], par, p.spin_limit))
                            {
                                give_up(12);
                                break;
                            }
                            copy((s + 2u) % static_cast<uint32_t>(tc_wide_splits));
                        }
                    }
                }
                if (*abort_flag)
                {
                    // copies still in flight land before the shared memory is released
                    if (issued0 > landed0)
                    {
                        tc::mbar_wait(&bar_b[0], landed0 & 1u, p.spin_limit);
                    }
                    if (issued1 > landed1)
                    {
                        tc::mbar_wait(&bar_b[1], landed1 & 1u, p.spin_limit);
                    }
                }
            }
        }
        else
        {
            // ------------------------------------------------ workers
            asm volatile("griddepcontrol.wait;" ::: "memory");
            const ChachaPre pre = chacha_pre(p.rng);
            for (uint64_t i = 0; i < count; ++i)
            {
                const uint32_t mt = static_cast<uint32_t>(t_begin + i);
                if (i > 0)
                {
                    // the previous tile's MMAs no longer read the digit tile
                    uint32_t ok = 1;
                    if (lane == 0)
                    {
                        ok = tc::mbar_wait_sleep(bar_a_empty, static_cast<uint32_t>((i - 1) & 1u), p.spin_limit);
                    }
                    if (!__shfl_sync(0xffffffffu, ok, 0))
                    {
                        give_up(16);
                        break;
                    }
                }
                tc_store_cbd_wide(p, pre, sa, mt, tid);
                tc::fence_proxy_async();
                mbar_arrive(bar_a_full);
                bool stop = false;
                for (uint32_t s = 0; s < static_cast<uint32_t>(tc_wide_splits); ++s)
                {
                    const uint64_t j = i * tc_wide_splits + s;
                    const uint32_t buf = static_cast<uint32_t>(j & 1u);
                    uint32_t ok = 1;
                    if (lane == 0)
                    {
                        ok = tc::mbar_wait_sleep(&bar_acc_full[buf], static_cast<uint32_t>((j >> 1) & 1u),
                                                 p.spin_limit);
                    }
                    if (!__shfl_sync(0xffffffffu, ok, 0))
                    {
                        give_up(17);
                        stop = true;
                        break;
                    }
                    tc::fence_after_sync();
                    const TcCursor cur{s, mt, 0};
                    tc_epilogue<DC, tc_wide_r, tc_out_digits, tc_wide_splits, false, false, true, false>(
                        p, tmem + buf * 256u, cur, warp, lane);
                    tc::fence_before_sync();
                    mbar_arrive(&bar_acc_empty[buf]);
                    if (*abort_flag)
                    {
                        stop = true;
                        break;
                    }
                }
                if (stop || *abort_flag)
                {
                    break;
                }
            }
        }
        __syncthreads();
        if (*abort_flag && tid == 0)
        {
            // give in-flight MMAs a bounded chance to land before the memory is released
            tc::mbar_wait(&bar_bfree[0], 0, p.spin_limit);
            tc::mbar_wait(&bar_bfree[0], 1, p.spin_limit);
            tc::mbar_wait(&bar_bfree[1], 0, p.spin_limit);
            tc::mbar_wait(&bar_bfree[1], 1, p.spin_limit);
        }
        __syncthreads();
        tc::fence_after_sync();
        if (warp == 0)
        {
            tc::tmem_dealloc(tmem, 512);
        }
    }

    // ------------------------------------------------------------- constants

    struct TcGenParams
    {
        const uint32_t* twiddles;  // element-major [N][L], Montgomery
        uint32_t* gx;              // [blocks][r][r][L]: G[k][i] (canonical, or Montgomery when montgomery = 1)
        uint64_t blocks;
        uint32_t log_n, inverse, s0, g, lo, montgomery;
    };

    // column i of every block's matrix: the group's butterflies applied to the unit vector e_i
    template<int L>
    __global__ void tc_gen_kernel(const TcGenParams p, const Modulus<L> m)
    {
        const uint32_t r = 1u << p.g;
        const uint64_t id = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
        if (id >= p.blocks * r)
        {
            return;
        }
        const uint64_t h = id / r;
        const uint32_t i = static_cast<uint32_t>(id % r);
        const uint64_t n = 1ull << p.log_n;
        uint32_t v[8][L];
        for (uint32_t k = 0; k < 8; ++k)
        {
            for (int j = 0; j < L; ++j)
            {
                v[k][j] = k == i ? m.one[j] : 0u;
            }
        }
        auto twiddle = [&](uint64_t index, uint32_t (&t)[L]) {
            for (int j = 0; j < L; ++j)
            {
                t[j] = p.twiddles[index * L + j];
            }
        };
        for (uint32_t st = 0; st < p.g; ++st)
        {
            const uint32_t s = p.s0 + st;
            const uint32_t bit = p.inverse ? (1u << st) : (1u << (p.g - 1 - st));
            for (uint32_t mu = 0; mu < r; ++mu)
            {
                if (mu & bit)
                {
                    continue;
                }
                const uint32_t mv = mu | bit;
                const uint64_t pu = (h << (p.lo + p.g)) | (static_cast<uint64_t>(mu) << p.lo);
                uint32_t a[L], b[L], t[L], x[L];
                for (int j = 0; j < L; ++j)
                {
                    a[j] = v[mu][j];
                    b[j] = v[mv][j];
                }
                if (!p.inverse)
                {
                    twiddle((1ull << s) + (pu >> (p.log_n - s)), t);
                    mont_mul<L>(x, b, t, m);
                    mod_add<L>(v[mu], a, x, m);
                    mod_sub<L>(v[mv], a, x, m);
                }
                else if (s + 1 == p.log_n)
                {
                    mod_add<L>(x, a, b, m);
                    twiddle(0, t);
                    mont_mul<L>(v[mu], x, t, m);
                    mod_sub<L>(x, a, b, m);
                    twiddle(1, t);
                    mont_mul<L>(v[mv], x, t, m);
                }
                else
                {
                    mod_add<L>(v[mu], a, b, m);
                    mod_sub<L>(x, a, b, m);
                    twiddle((n >> (s + 1)) + (pu >> (s + 1)), t);
                    mont_mul<L>(v[mv], x, t, m);
                }
            }
        }
        uint32_t unit[L];
        for (int j = 0; j < L; ++j)
        {
            unit[j] = j == 0 ? 1u : 0u;
        }
        for (uint32_t k = 0; k < r; ++k)
        {
            uint32_t out[L];
            if (p.montgomery)
            {
                for (int j = 0; j < L; ++j)
                {
                    out[j] = v[k][j];
                }
            }
            else
            {
                mont_mul<L>(out, v[k], unit, m);
            }
            for (int j = 0; j < L; ++j)
            {
                p.gx[((h * r + k) * r + i) * L + j] = out[j];
            }
        }
    }

    // The wide group's 64 x 64 matrix over Z_q from the first two three-stage
    // groups of the forward transform: the second applies B_kh (block kh =
    // the element's top three bits, already mixed by the first) to the low
    // three bits, the first A to the top three, so G6[(kh, kl)][(ih, il)] =
    // B_kh[kl][il] * A[kh][ih], optionally times a scale (all Montgomery).
    struct TcCombineParams
    {
        const uint32_t* gx_a;   // [1][8][8][L]
        const uint32_t* gx_b;   // [8][8][8][L]
        const uint32_t* scale;  // [L] Montgomery form, or nullptr
        uint32_t* gx;           // [1][64][64][L]
    };

    template<int L>
    __global__ void tc_combine6_kernel(const TcCombineParams p, const Modulus<L> m)
    {
        const uint32_t id = blockIdx.x * blockDim.x + threadIdx.x;
        if (id >= 64u * 64u)
        {
            return;
        }
        const uint32_t k = id / 64u, i = id % 64u;
        const uint32_t kh = k >> 3, kl = k & 7u, ih = i >> 3, il = i & 7u;
        uint32_t a[L], b[L], v[L];
        for (int j = 0; j < L; ++j)
        {
            a[j] = p.gx_a[((kh * 8u) + ih) * L + j];
            b[j] = p.gx_b[((kh * 8u + kl) * 8u + il) * L + j];
        }
        mont_mul<L>(v, b, a, m);
        if (p.scale)
        {
            for (int j = 0; j < L; ++j)
            {
                a[j] = p.scale[j];
            }
            mont_mul<L>(v, v, a, m);
        }
        for (int j = 0; j < L; ++j)
        {
            p.gx[static_cast<uint64_t>(id) * L + j] = v[j];
        }
    }

    struct TcExpandParams
    {
        const uint32_t* gx;      // [blocks][r][r][L]
        const uint32_t* pow256;  // [d_in][L]: 256^a * R mod q
        uint8_t* images;         // blocks * splits images of image_bytes, zero-filled
        uint64_t blocks;
        uint32_t r, dc, d_in, splits, n_mma, image_bytes;
        uint32_t word_major;     // K order of the group's loader (tc_k_index)
        uint32_t half[8];        // floor(q / 2)
    };

    // Constant digits: output k of block h lives in image h * splits + k / (r /
    // splits), row (k mod (r / splits)) * DC + b, column tc_k_index(a, i): balanced
    // digit b in [-128, 127] of the signed value V = (256^a * G[k][i] mod q)
    // in (-q/2, q/2] (V taken in two's complement; the 4L balanced digits of
    // any |V| <= 0x7F7F..7F are exact).
    template<int L>
    __global__ void tc_expand_kernel(const TcExpandParams p, const Modulus<L> m)
    {
        const uint64_t id = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
        const uint64_t per_block = static_cast<uint64_t>(p.r) * p.r * p.d_in;
        if (id >= p.blocks * per_block)
        {
            return;
        }
        const uint64_t h = id / per_block;
        uint32_t rest = static_cast<uint32_t>(id % per_block);
        const uint32_t a = rest % p.d_in;
        rest /= p.d_in;
        const uint32_t i = rest % p.r;
        const uint32_t k = rest / p.r;
        uint32_t gkx[L], pw[L], w[L];
        for (int j = 0; j < L; ++j)
        {
            gkx[j] = p.gx[((h * p.r + k) * p.r + i) * L + j];
            pw[j] = p.pow256[a * L + j];
        }
        mont_mul<L>(w, gkx, pw, m);
        bool neg = false;
        for (int j = L - 1; j >= 0; --j)
        {
            if (w[j] != p.half[j])
            {
                neg = w[j] > p.half[j];
                break;
            }
        }
        if (neg)
        {
            // V = W - q in two's complement over L words
            uint32_t b = 0;
            for (int j = 0; j < L; ++j)
            {
                const unsigned long long s = static_cast<unsigned long long>(w[j]) - m.q[j] - b;
                w[j] = static_cast<uint32_t>(s);
                b = static_cast<uint32_t>(s >> 63);
            }
        }
        const uint32_t outputs = p.r / p.splits;
        uint8_t* img = p.images + (h * p.splits + k / outputs) * p.image_bytes;
        const uint32_t k_local = k % outputs;
        int carry = 0;
        for (uint32_t b = 0; b < p.dc; ++b)
        {
            const int byte = static_cast<int>((w[b / 4] >> (8 * (b % 4))) & 255u) + carry;
            int digit = byte;
            carry = 0;
            if (byte >= 128)
            {
                digit = byte - 256;
                carry = 1;
            }
            *reinterpret_cast<__half*>(img + tc::operand_offset(k_local * p.dc + b,
                                                                 tc_k_index(a, i, p.r, p.dc, p.word_major != 0),
                                                                 p.n_mma)) = __int2half_rn(digit);
        }
    }
}
