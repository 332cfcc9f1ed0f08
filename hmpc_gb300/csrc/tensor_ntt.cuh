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
    };

    enum TcOutput : int
    {
        tc_out_digits = 0,
        tc_out_limbs = 1,
    };

    constexpr int tc_rows = 128;
    constexpr int tc_threads = 256;

    struct TcGroupParams
    {
        const uint32_t* in;        // digit or limb planes, `elements` words each
        uint32_t* out;             // digit or limb planes
        const uint8_t* images;     // per block: the constant operand in its shared-memory layout
        uint32_t* error;           // set when a bounded wait runs out
        uint64_t elements;         // batch * N
        uint64_t rows;             // rows per block: batch << lo
        uint64_t tiles;            // blocks * tiles_per_block
        uint32_t tiles_per_block;
        uint32_t log_n;
        uint32_t lo;               // column bits below the group's element bits
        uint32_t spin_limit;       // polls of an mbarrier before giving up
        RngKey rng;                // CBD loader
        uint32_t vx2;
        uint32_t nw;
        uint32_t q[8];             // final reduction
        float inv_q_top;           // 2^(32(L-1)) / q
    };

    template<int DC, int R, int IN>
    struct TcShape
    {
        static constexpr int g = R == 8 ? 3 : (R == 4 ? 2 : 1);
        static constexpr int d_in = IN == tc_in_digits ? DC + 2 : (IN == tc_in_limbs ? DC : 1);
        static constexpr int w_in = IN == tc_in_cbd ? 0 : (d_in + 3) / 4;
        // digit slots per element on the K axis (K index = a * R + m)
        static constexpr int d_eff = IN == tc_in_cbd ? 1 : (R == 8 ? d_in : (R == 4 ? (d_in + 1) / 2 * 2 : w_in * 4));
        static constexpr int k_real = R * d_eff;
        static constexpr int k_pad = (k_real + 15) / 16 * 16;
        static constexpr int n_mma = (R * DC + 15) / 16 * 16;
        static constexpr int cols = n_mma <= 32 ? 32 : (n_mma <= 64 ? 64 : (n_mma <= 128 ? 128 : 256));
        static constexpr uint32_t a_bytes = tc_rows * k_pad * 2;
        static constexpr uint32_t b_bytes = n_mma * k_pad * 2;
        static constexpr uint32_t smem = a_bytes + b_bytes + 64;
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

    struct TcRow
    {
        bool ok;
        uint64_t base;  // element index of m = 0
        uint64_t poly;
        uint64_t col;
    };

    template<int G>
    __device__ __forceinline__ TcRow tc_row(const TcGroupParams& p, uint64_t tile, uint32_t row)
    {
        const uint64_t h = tile / p.tiles_per_block;
        const uint64_t rho = (tile - h * p.tiles_per_block) * tc_rows + row;
        TcRow r;
        r.ok = rho < p.rows;
        r.poly = rho >> p.lo;
        r.col = rho & ((1ull << p.lo) - 1ull);
        r.base = (r.poly << p.log_n) + (h << (p.lo + G)) + r.col;
        return r;
    }

    // loader of digit / limb tiles: thread (row, half) owns words [half * WH, ...) of the row's R elements
    template<int DC, int R, int IN>
    struct TcLoader
    {
        using S = TcShape<DC, R, IN>;
        static constexpr int wh = S::w_in > 0 ? (S::w_in + 1) / 2 : 1;
        uint32_t v[wh][R];

        __device__ __forceinline__ void load(const TcGroupParams& p, uint64_t tile, uint32_t row, uint32_t half)
        {
            const TcRow r = tc_row<S::g>(p, tile, row);
#pragma unroll
            for (int wi = 0; wi < wh; ++wi)
            {
                const uint32_t w = half * wh + wi;
#pragma unroll
                for (int m = 0; m < R; ++m)
                {
                    v[wi][m] = 0u;
                    if (r.ok && w < static_cast<uint32_t>(S::w_in))
                    {
                        v[wi][m] = __ldg(p.in + w * p.elements + r.base + (static_cast<uint64_t>(m) << p.lo));
                    }
                }
            }
        }

        __device__ __forceinline__ void store(uint8_t* sa, uint32_t row, uint32_t half) const
        {
            constexpr int bias = IN == tc_in_digits ? 128 : 0;
#pragma unroll
            for (int wi = 0; wi < wh; ++wi)
            {
                const uint32_t w = half * wh + wi;
                if (w >= static_cast<uint32_t>(S::w_in))
                {
                    continue;
                }
                if constexpr (R == 8)
                {
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

    // first forward group fed by centred binomial samples: r = 8, stage-0 pairs
    // (m, m + 4) of a row come from one generator with counter = poly * N +
    // index of the first element, first draw for m, second for m + 4
    // (number_theoretic_transform.hpp:316-329, comp/queue.hpp:191-212)
    __device__ __forceinline__ void tc_store_cbd(const TcGroupParams& p, uint8_t* sa, uint64_t tile, uint32_t row,
                                                 uint32_t half)
    {
        const TcRow r = tc_row<3>(p, tile, row);
        int e_u[2] = {0, 0}, e_v[2] = {0, 0};
        if (r.ok)
        {
            const int count = 2 * static_cast<int>(p.vx2);
#pragma unroll
            for (int j = 0; j < 2; ++j)
            {
                const uint64_t idx_u = r.base - (r.poly << p.log_n) + (static_cast<uint64_t>(2 * half + j) << p.lo);
                uint32_t w[8];
                chacha_stream<8>(p.rng, static_cast<uint32_t>((r.poly << p.log_n) + idx_u), w);
                int a = 0, b = 0;
#pragma unroll
                for (int i = 0; i < 8; ++i)
                {
                    const int iu = i;               // word i of the first sample
                    const int iv = i - static_cast<int>(p.nw);  // word of the second sample
                    uint32_t mu = 0u, mv = 0u;
                    if (iu < static_cast<int>(p.nw))
                    {
                        mu = 0xffffffffu;
                        if (iu == static_cast<int>(p.nw) - 1 && (count & 31))
                        {
                            mu = (1u << (count & 31)) - 1u;
                        }
                    }
                    else if (iv < static_cast<int>(p.nw))
                    {
                        mv = 0xffffffffu;
                        if (iv == static_cast<int>(p.nw) - 1 && (count & 31))
                        {
                            mv = (1u << (count & 31)) - 1u;
                        }
                    }
                    a += __popc(w[i] & mu);
                    b += __popc(w[i] & mv);
                }
                e_u[j] = a - static_cast<int>(p.vx2);
                e_v[j] = b - static_cast<int>(p.vx2);
            }
        }
        uint8_t* seg = sa + tc::operand_offset(row, 0, tc_rows);
        __half2 lo = __halves2half2(__int2half_rn(e_u[0]), __int2half_rn(e_u[1]));
        __half2 hi = __halves2half2(__int2half_rn(e_v[0]), __int2half_rn(e_v[1]));
        st_shared_u32(seg + 4 * half, *reinterpret_cast<uint32_t*>(&lo));
        st_shared_u32(seg + 8 + 4 * half, *reinterpret_cast<uint32_t*>(&hi));
    }

    __device__ __forceinline__ uint32_t pack_bytes(uint32_t b0, uint32_t b1, uint32_t b2, uint32_t b3)
    {
        return __byte_perm(__byte_perm(b0, b1, 0x0040), __byte_perm(b2, b3, 0x0040), 0x5410);
    }

    // carry of exact f32 column sums into balanced base-256 digits, all in f32:
    // t = s + carry + 128; c = floor(t / 256); digit + 128 = t - 256 c
    struct DigitCarry
    {
        float cp = 128.0f;  // carry + 128

        __device__ __forceinline__ uint32_t step(float s)
        {
            const float t = s + cp;
            const float x = __fmaf_rd(t, 0.00390625f, 12582912.0f);
            const float c = x - 12582912.0f;
            const float d = __fmaf_rn(-256.0f, c, t);
            cp = c + 128.0f;
            return __float_as_uint(d + 8388608.0f);  // low byte = digit + 128
        }
    };

    template<int DC>
    __device__ __forceinline__ void tc_load_sums(uint32_t taddr, uint32_t (&s)[DC])
    {
        static_assert(DC == 8 || DC == 16 || DC == 32, "digit counts of 2, 4 and 8 limbs");
        tc::tmem_load<DC>(taddr, s);
    }

    // the signed value sum_j x_j 2^(32 j) + top 2^(32 L), |value / q| < 2^17,
    // reduced into [0, q)
    template<int L>
    __device__ __forceinline__ void tc_reduce(uint32_t (&x)[L], int top, const TcGroupParams& p)
    {
        const float est = (static_cast<float>(top) * 4294967296.0f + static_cast<float>(x[L - 1])) * p.inv_q_top;
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

    template<int DC, int R, int OUT>
    __device__ __forceinline__ void tc_epilogue(const TcGroupParams& p, uint32_t tmem, uint64_t tile, uint32_t warp,
                                                uint32_t lane)
    {
        constexpr int g = R == 8 ? 3 : (R == 4 ? 2 : 1);
        constexpr int L = DC / 4;
        constexpr int W = (DC + 2 + 3) / 4;
        const uint32_t lg = warp & 3u;
        const uint32_t row = 32u * lg + lane;
        const TcRow r = tc_row<g>(p, tile, row);
        constexpr int per = R / 2;
        const uint32_t k0 = (warp >> 2) * per;
#pragma unroll 1
        for (int kk = 0; kk < per; ++kk)
        {
            const uint32_t k = k0 + kk;
            uint32_t s[DC];
            tc_load_sums<DC>(tmem + ((32u * lg) << 16) + k * DC, s);
            tc::tmem_load_wait();
            DigitCarry carry;
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
            const uint64_t e = r.base + (static_cast<uint64_t>(k) << p.lo);
            if constexpr (OUT == tc_out_digits)
            {
                const uint32_t c0 = carry.step(0.0f);
                const uint32_t c1 = carry.step(0.0f);
                words[DC / 4] = pack_bytes(c0, c1, 0x80u, 0x80u);
                if (r.ok)
                {
#pragma unroll
                    for (int w = 0; w < W; ++w)
                    {
                        p.out[w * p.elements + e] = words[w];
                    }
                }
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
                const int top = __float2int_rn(carry.cp - 128.0f) - static_cast<int>(borrow);
                tc_reduce<L>(x, top, p);
                if (r.ok)
                {
#pragma unroll
                    for (int j = 0; j < L; ++j)
                    {
                        p.out[j * p.elements + e] = x[j];
                    }
                }
            }
        }
    }

    template<int DC, int R, int IN, int OUT>
    __global__ void __launch_bounds__(tc_threads, 1) tc_group_kernel(const TcGroupParams p)
    {
        using S = TcShape<DC, R, IN>;
        extern __shared__ __align__(1024) uint8_t tc_smem[];
        uint8_t* sb = tc_smem;
        uint8_t* sa = tc_smem + S::b_bytes;
        uint64_t* bars = reinterpret_cast<uint64_t*>(sa + S::a_bytes);  // [0] operand B, [1..2] accumulators
        uint32_t* tslot = reinterpret_cast<uint32_t*>(bars + 3);
        volatile uint32_t* abort_flag = tslot + 1;

        const uint32_t tid = threadIdx.x;
        const uint32_t warp = tid >> 5, lane = tid & 31u;
        const uint32_t row = tid & (tc_rows - 1), half = tid >> 7;

        const uint64_t t_begin = p.tiles * blockIdx.x / gridDim.x;
        const uint64_t t_end = p.tiles * (blockIdx.x + 1) / gridDim.x;

        // K padding of the A tile stays zero
        for (uint32_t u = tid; u < (S::k_pad - S::k_real) / 8 * tc_rows; u += tc_threads)
        {
            st_shared_v4(sa + tc::operand_offset(u % tc_rows, S::k_real + 8 * (u / tc_rows), tc_rows), 0, 0, 0, 0);
        }
        if (tid == 0)
        {
            tc::mbar_init(&bars[0], 1);
            tc::mbar_init(&bars[1], 1);
            tc::mbar_init(&bars[2], 1);
            *abort_flag = 0;
            tc::mbar_init_fence();
        }
        if (warp == 0)
        {
            tc::tmem_alloc(tslot, 2 * S::cols);
        }
        tc::fence_before_sync();
        __syncthreads();
        tc::fence_after_sync();
        const uint32_t tmem = *tslot;
        constexpr uint32_t idesc = tc::f16_instr_descriptor(tc_rows, S::n_mma);

        uint32_t phase_b = 0, phase_acc = 0;  // bit i: parity of accumulator i
        uint64_t cur_block = ~0ull;
        bool failed = false;

        auto issue_b = [&](uint64_t block) {
            tc::mbar_arrive_expect_tx(&bars[0], S::b_bytes);
            tc::bulk_g2s(sb, p.images + block * S::b_bytes, S::b_bytes, &bars[0]);
        };
        auto issue_mma = [&](uint32_t buf, bool wait_b) {
            // thread 0 only
            if (wait_b)
            {
                if (!tc::mbar_wait(&bars[0], phase_b, p.spin_limit))
                {
                    atomicExch(p.error, 1u);
                    *abort_flag = 1;
                }
                phase_b ^= 1u;
            }
            tc::fence_after_sync();
            const uint32_t a0 = tc::smem_u32(sa), b0 = tc::smem_u32(sb);
#pragma unroll
            for (int ks = 0; ks < S::k_pad / 16; ++ks)
            {
                tc::mma_f16(tmem + buf * S::cols, tc::smem_descriptor(a0 + ks * 2 * S::lbo_a, S::lbo_a, 128),
                            tc::smem_descriptor(b0 + ks * 2 * S::lbo_b, S::lbo_b, 128), idesc, ks > 0);
            }
            tc::mma_commit(&bars[1 + buf]);
        };

        TcLoader<DC, R, IN> loader;
        if (t_begin < t_end)
        {
            // prologue: tile t_begin into accumulator 0
            cur_block = t_begin / p.tiles_per_block;
            if (tid == 0)
            {
                issue_b(cur_block);
            }
            if constexpr (IN == tc_in_cbd)
            {
                tc_store_cbd(p, sa, t_begin, row, half);
            }
            else
            {
                loader.load(p, t_begin, row, half);
                loader.store(sa, row, half);
            }
            tc::fence_proxy_async();
            __syncthreads();
            if constexpr (IN != tc_in_cbd)
            {
                if (t_begin + 1 < t_end)
                {
                    loader.load(p, t_begin + 1, row, half);
                }
            }
            if (tid == 0)
            {
                issue_mma(0, true);
            }
        }
        for (uint64_t t = t_begin; t < t_end; ++t)
        {
            const uint32_t buf = static_cast<uint32_t>((t - t_begin) & 1u);
            // accumulator of tile t complete (warp-uniform bounded wait)
            uint32_t ok = 1;
            if (lane == 0)
            {
                ok = tc::mbar_wait(&bars[1 + buf], (phase_acc >> buf) & 1u, p.spin_limit) ? 1u : 0u;
            }
            ok = __shfl_sync(0xffffffffu, ok, 0);
            phase_acc ^= 1u << buf;
            if (!ok)
            {
                atomicExch(p.error, 2u);
                *abort_flag = 1;
            }
            tc::fence_after_sync();
            if (t + 1 < t_end)
            {
                const uint64_t next_block = (t + 1) / p.tiles_per_block;
                const bool new_b = next_block != cur_block;
                if (new_b && tid == 0)
                {
                    issue_b(next_block);  // the MMAs reading the old operand are complete
                }
                cur_block = next_block;
                if constexpr (IN == tc_in_cbd)
                {
                    tc_store_cbd(p, sa, t + 1, row, half);
                }
                else
                {
                    loader.store(sa, row, half);
                }
                tc::fence_proxy_async();
                tc::fence_before_sync();
                __syncthreads();
                if (*abort_flag)
                {
                    failed = true;
                    break;
                }
                if constexpr (IN != tc_in_cbd)
                {
                    if (t + 2 < t_end)
                    {
                        loader.load(p, t + 2, row, half);
                    }
                }
                if (tid == 0)
                {
                    issue_mma(buf ^ 1u, new_b);
                }
            }
            tc_epilogue<DC, R, OUT>(p, tmem + buf * S::cols, t, warp, lane);
            tc::fence_before_sync();
        }
        if (failed && tid == 0)
        {
            // give in-flight copies and MMAs a bounded chance to land before the memory is released
            tc::mbar_wait(&bars[1], phase_acc & 1u, p.spin_limit);
            tc::mbar_wait(&bars[2], (phase_acc >> 1) & 1u, p.spin_limit);
        }
        __syncthreads();
        tc::fence_after_sync();
        if (warp == 0)
        {
            tc::tmem_dealloc(tmem, 2 * S::cols);
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

    struct TcExpandParams
    {
        const uint32_t* gx;      // [blocks][r][r][L]
        const uint32_t* pow256;  // [d_in][L]: 256^a * R mod q
        uint8_t* images;         // blocks * image_bytes, zero-filled
        uint64_t blocks;
        uint32_t r, dc, d_in, n_mma, image_bytes;
        uint32_t half[8];        // floor(q / 2)
    };

    // constant digits: image[h] row (k * DC + b), column (a * r + i) holds digit b
    // of the signed value (256^a * G[k][i] mod q) in (-q/2, q/2]
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
        // signed representative
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
            uint32_t b = 0;
            for (int j = 0; j < L; ++j)
            {
                const unsigned long long s = static_cast<unsigned long long>(m.q[j]) - w[j] - b;
                w[j] = static_cast<uint32_t>(s);
                b = static_cast<uint32_t>(s >> 63);
            }
        }
        uint8_t* img = p.images + h * p.image_bytes;
        int carry = 0;
        for (uint32_t b = 0; b < p.dc; ++b)
        {
            int byte = static_cast<int>((w[b / 4] >> (8 * (b % 4))) & 255u) + carry;
            int digit = byte;
            carry = 0;
            if (byte >= 128)
            {
                digit = byte - 256;
                carry = 1;
            }
            if (neg)
            {
                digit = -digit;
            }
            *reinterpret_cast<__half*>(img + tc::operand_offset(k * p.dc + b, a * p.r + i, p.n_mma)) =
                __int2half_rn(digit);
        }
    }
}
