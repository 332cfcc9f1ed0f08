// Negacyclic NTT / INTT as a sequence of shared-memory tile passes.
//
// Semantics are those of hmpc's stage-per-kernel transform
// (hmpc/expr/number_theoretic_transform.hpp:90-197,262-549):
//   forward stage s: length = 2^s, step = N/2^(s+1), the lower element idx of
//     a pair takes psi = T[2^s + (idx >> (n - s))]; v *= psi; (u+v, u-v)
//   inverse stage s: length = N/2^(s+1), step = 2^s,
//     psi = T[N/2^(s+1) + (idx >> (s+1))]; (u+v, (u-v)*psi); the last stage
//     multiplies u+v by T[0] = N^-1 and u-v by T[1] (pre-multiplied by N^-1)
// The butterflies are the same ones on the same positions, so the output
// (natural order in -> bit-reversed order out for the forward transform) is
// identical; only the schedule differs.
//
// Schedule: the log2(N) stages are split into passes.  A pass covers stages
// [s0, s1); the element-index bits those stages touch are the "row" bits of a
// tile.  One CTA stages T tiles (x 2^c columns for coalescing) in shared
// memory, limb-planar.  Inside a pass, stages are processed in groups of up
// to R: each thread holds 2^R elements in registers, applies the group's
// butterflies there, and writes them back, so shared memory is touched once
// per group instead of once per stage.  The first pass can generate its input
// in registers (ChaCha20 samplers) instead of reading a tensor.
#pragma once

#include <cstdint>

#include "chacha.cuh"
#include "limbs.cuh"

namespace hmpc_gb300
{
    enum ProducerKind : int
    {
        producer_tensor = 0,   // read `src` (or the output buffer when src == nullptr)
        producer_cbd = 1,      // centred binomial, 2V = vx2, NW words per sample
        producer_uniform = 2,  // uniform mod Q, W words per sample
    };

    constexpr int max_groups = 8;

    struct NttGroup
    {
        uint32_t stage;          // first stage of the group
        uint32_t count;          // stages in the group (<= R)
        uint32_t reg_pos[6];     // local bit position of register bit k (k < R)
        uint32_t rest_mask;      // local bits enumerated by the thread's block id
    };

    struct NttPassParams
    {
        uint32_t* out;                 // limb-planar, `elements` entries per limb
        const uint32_t* src;           // tensor producer input (nullptr: read out)
        const uint32_t* twiddles;      // element-major [N][L]
        const uint32_t* small_table;   // Montgomery forms of 0..64, element-major
        uint64_t elements;             // batch * N
        uint64_t tiles;                // batch * tiles per polynomial
        uint32_t log_n;
        uint32_t inverse;
        uint32_t s0, s1;               // stages of this pass
        uint32_t row_shift;            // element bit of the lowest row bit
        uint32_t col_bits;             // c
        uint32_t tile_bits;            // log2 tiles per CTA
        uint32_t local_bits;           // log2 elements per CTA = tile_bits + w + c
        uint32_t num_groups;
        NttGroup groups[max_groups];
        RngKey rng;
        uint32_t vx2;                  // 2V for the CBD producer
        uint32_t top_mask;             // uniform producer: mask of the top word
        // Per-polynomial RNG (batches of independent requests): when set,
        // polynomial i draws with nonce = desc[0..2] + rng_slot * desc[4] * N and
        // counter = desc[3] * N + coefficient, desc = poly_rng + 5 i -- exactly
        // what the request would draw alone with its own nonce.
        const uint32_t* poly_rng;
        uint32_t rng_slot;
        // host side: launch with programmatic dependence on the pass before
        // it in the stream (a pass of the same transform)
        uint32_t dependent;
    };

    __device__ __forceinline__ uint32_t smem_addr(uint32_t local)
    {
        return local + (local >> 5);  // one pad word per 32: spreads strided accesses over banks
    }

    // scatter the low bits of v into the set bits of mask (ascending)
    __device__ __forceinline__ uint32_t deposit_bits(uint32_t v, uint32_t mask)
    {
        uint32_t r = 0;
        while (mask)
        {
            const uint32_t low = mask & (0u - mask);
            if (v & 1u)
            {
                r |= low;
            }
            v >>= 1;
            mask ^= low;
        }
        return r;
    }

    template<int L>
    struct NttTileGeometry
    {
        uint32_t w, c, tile_bits, rs, log_n;
        uint64_t tile0;  // first global tile of this CTA
        uint64_t n;

        // element index inside its polynomial, and the polynomial, of a CTA-local index
        __device__ __forceinline__ uint64_t tile_of(uint32_t local) const
        {
            return tile0 + (local >> (c + w));
        }

        __device__ __forceinline__ void locate(uint32_t local, uint64_t& poly, uint64_t& idx) const
        {
            const uint32_t col = local & ((1u << c) - 1u);
            const uint32_t row = (local >> c) & ((1u << w) - 1u);
            const uint64_t tile = tile_of(local);
            const uint32_t tile_bits_per_poly = log_n - w - c;
            const uint64_t t_in_poly = tile & ((1ull << tile_bits_per_poly) - 1ull);
            poly = tile >> tile_bits_per_poly;
            const uint64_t mid = t_in_poly & ((1ull << (rs - c)) - 1ull);
            const uint64_t top = t_in_poly >> (rs - c);
            idx = (top << (rs + w)) | (static_cast<uint64_t>(row) << rs) | (mid << c) | col;
        }
    };

    // generator key, nonce and counter of the stage-0 pair whose first element
    // is coefficient idx_u of polynomial `poly`
    __device__ __forceinline__ uint32_t pair_generator(const NttPassParams& p, uint64_t poly, uint64_t idx_u,
                                                       RngKey& rng)
    {
        rng = p.rng;
        if (p.poly_rng)
        {
            const uint32_t* d = p.poly_rng + poly * 5;
            const uint64_t add = static_cast<uint64_t>(p.rng_slot) * d[4] << p.log_n;
            uint64_t s = static_cast<uint64_t>(d[0]) + static_cast<uint32_t>(add);
            rng.nonce[0] = static_cast<uint32_t>(s);
            s = static_cast<uint64_t>(d[1]) + static_cast<uint32_t>(add >> 32) + (s >> 32);
            rng.nonce[1] = static_cast<uint32_t>(s);
            rng.nonce[2] = d[2] + static_cast<uint32_t>(s >> 32);
            return static_cast<uint32_t>((static_cast<uint64_t>(d[3]) << p.log_n) + idx_u);
        }
        return static_cast<uint32_t>(poly * (1ull << p.log_n) + idx_u);
    }

    template<int L, int Kind, int NW>
    __device__ __forceinline__ void produce_pair(const NttPassParams& p, const Modulus<L>& m, uint64_t poly,
                                                 uint64_t idx_u, uint64_t idx_v, uint32_t (&u)[L],
                                                 uint32_t (&v)[L])
    {
        if constexpr (Kind == producer_cbd)
        {
            // one generator per pair, counter = low word of the first element's
            // linear index; u draws first, v next (number_theoretic_transform.hpp
            // :316-329, comp/queue.hpp:191-212)
            uint32_t w[2 * NW];
            RngKey rng;
            const uint32_t counter = pair_generator(p, poly, idx_u, rng);
            chacha_stream<2 * NW>(rng, counter, w);
            int a = 0, b = 0;
            const int count = 2 * static_cast<int>(p.vx2);
#pragma unroll
            for (int i = 0; i < NW; ++i)
            {
                uint32_t mask = 0xffffffffu;
                if (i == NW - 1 && (count & 31))
                {
                    mask = (1u << (count & 31)) - 1u;
                }
                a += __popc(w[i] & mask);
                b += __popc(w[NW + i] & mask);
            }
            small_to_mont<L>(u, a - static_cast<int>(p.vx2), p.small_table, m);
            small_to_mont<L>(v, b - static_cast<int>(p.vx2), p.small_table, m);
        }
        else if constexpr (Kind == producer_uniform)
        {
            uint32_t w[2 * NW];
            RngKey rng;
            const uint32_t counter = pair_generator(p, poly, idx_u, rng);
            chacha_stream<2 * NW>(rng, counter, w);
            uniform_from_words<L, NW, 0, 2 * NW>(u, w, p.top_mask, m);
            uniform_from_words<L, NW, NW, 2 * NW>(v, w, p.top_mask, m);
        }
        else
        {
            (void)idx_v;
        }
    }

    template<int L>
    __device__ __forceinline__ void load_twiddle(uint32_t (&t)[L], const uint32_t* table, uint32_t index)
    {
        const uint32_t* ptr = table + static_cast<size_t>(index) * L;
        if constexpr (L % 4 == 0)
        {
#pragma unroll
            for (int j = 0; j < L; j += 4)
            {
                const uint4 v = __ldg(reinterpret_cast<const uint4*>(ptr + j));
                t[j] = v.x;
                t[j + 1] = v.y;
                t[j + 2] = v.z;
                t[j + 3] = v.w;
            }
        }
        else if constexpr (L % 2 == 0)
        {
#pragma unroll
            for (int j = 0; j < L; j += 2)
            {
                const uint2 v = __ldg(reinterpret_cast<const uint2*>(ptr + j));
                t[j] = v.x;
                t[j + 1] = v.y;
            }
        }
        else
        {
#pragma unroll
            for (int j = 0; j < L; ++j)
            {
                t[j] = __ldg(ptr + j);
            }
        }
    }

    // One pass over the tiles of a batch.  R = register bits per thread.
    // The first register group reads its elements straight from global memory
    // (or generates them), the last one writes them straight back; the groups
    // in between exchange data through shared memory.  Register bits always
    // lie inside one tile (the planner keeps c + w >= R), so a register
    // block's element indices are its base index plus fixed offsets.
    template<int L, int R, int Kind, int NW>
    __device__ __forceinline__ void ntt_process(const NttPassParams& p, const Modulus<L>& m, uint64_t tile0,
                                                uint32_t* smem)
    {
        constexpr int regs = 1 << R;
        const uint32_t local_count = 1u << p.local_bits;
        const uint32_t limb_stride = smem_addr(local_count);
        const uint32_t w = p.s1 - p.s0;
        const uint32_t c = p.col_bits;
        const uint32_t log_n = p.log_n;
        const uint64_t n = 1ull << log_n;

        NttTileGeometry<L> geo;
        geo.w = w;
        geo.c = c;
        geo.tile_bits = p.tile_bits;
        geo.rs = p.row_shift;
        geo.log_n = log_n;
        geo.n = n;
        geo.tile0 = tile0;

        const uint32_t* in = p.src ? p.src : p.out;
        const uint32_t blocks = local_count >> R;
        const uint32_t last = p.num_groups - 1;
        for (uint32_t gi = 0; gi < p.num_groups; ++gi)
        {
            const NttGroup& g = p.groups[gi];
            uint32_t off[regs];    // CTA-local offset of register x
            uint32_t eoff[regs];   // offset of register x inside its polynomial
#pragma unroll
            for (int x = 0; x < regs; ++x)
            {
                uint32_t o = 0;
#pragma unroll
                for (int k = 0; k < R; ++k)
                {
                    if (x & (1 << k))
                    {
                        o |= 1u << g.reg_pos[k];
                    }
                }
                off[x] = o;
                eoff[x] = (o & ((1u << c) - 1u)) | ((o >> c) << p.row_shift);
            }
            for (uint32_t b = threadIdx.x; b < blocks; b += blockDim.x)
            {
                const uint32_t base = deposit_bits(b, g.rest_mask);
                if (geo.tile_of(base) >= p.tiles)
                {
                    continue;  // partial last CTA: nothing to load or store
                }
                uint64_t poly, idx64;
                geo.locate(base, poly, idx64);
                const uint32_t idx = static_cast<uint32_t>(idx64);
                const uint64_t ebase = poly * n + idx;
                uint32_t x_reg[regs][L];
                if (gi == 0)
                {
                    if constexpr (Kind != producer_tensor)
                    {
                        // stage 0 pairs register bit 0: (x, x | 1)
#pragma unroll
                        for (int x = 0; x < regs; x += 2)
                        {
                            produce_pair<L, Kind, NW>(p, m, poly, idx + eoff[x], idx + eoff[x | 1], x_reg[x],
                                                      x_reg[x | 1]);
                        }
                    }
                    else
                    {
#pragma unroll
                        for (int x = 0; x < regs; ++x)
                        {
#pragma unroll
                            for (int j = 0; j < L; ++j)
                            {
                                x_reg[x][j] = in[static_cast<uint64_t>(j) * p.elements + ebase + eoff[x]];
                            }
                        }
                    }
                }
                else
                {
#pragma unroll
                    for (int x = 0; x < regs; ++x)
                    {
                        const uint32_t a = smem_addr(base | off[x]);
#pragma unroll
                        for (int j = 0; j < L; ++j)
                        {
                            x_reg[x][j] = smem[j * limb_stride + a];
                        }
                    }
                }
#pragma unroll
                for (int k = 0; k < R; ++k)
                {
                    if (static_cast<uint32_t>(k) < g.count)
                    {
                        const uint32_t s = g.stage + k;
                        const bool last_inverse = p.inverse && s == log_n - 1;
#pragma unroll
                        for (int x = 0; x < regs; ++x)
                        {
                            if ((x & (1 << k)) == 0)
                            {
                                const uint32_t e = idx + eoff[x];  // lower element of the pair
                                uint32_t t[L];
                                if (!p.inverse)
                                {
                                    load_twiddle<L>(t, p.twiddles, (1u << s) + (e >> (log_n - s)));
                                    mont_mul<L>(x_reg[x | (1 << k)], x_reg[x | (1 << k)], t, m);
                                    uint32_t sum[L];
                                    mod_add<L>(sum, x_reg[x], x_reg[x | (1 << k)], m);
                                    mod_sub<L>(x_reg[x | (1 << k)], x_reg[x], x_reg[x | (1 << k)], m);
#pragma unroll
                                    for (int j = 0; j < L; ++j)
                                    {
                                        x_reg[x][j] = sum[j];
                                    }
                                }
                                else if (!last_inverse)
                                {
                                    load_twiddle<L>(t, p.twiddles, static_cast<uint32_t>(n >> (s + 1)) + (e >> (s + 1)));
                                    uint32_t sum[L], diff[L];
                                    mod_add<L>(sum, x_reg[x], x_reg[x | (1 << k)], m);
                                    mod_sub<L>(diff, x_reg[x], x_reg[x | (1 << k)], m);
                                    mont_mul<L>(x_reg[x | (1 << k)], diff, t, m);
#pragma unroll
                                    for (int j = 0; j < L; ++j)
                                    {
                                        x_reg[x][j] = sum[j];
                                    }
                                }
                                else
                                {
                                    uint32_t sum[L], diff[L];
                                    mod_add<L>(sum, x_reg[x], x_reg[x | (1 << k)], m);
                                    mod_sub<L>(diff, x_reg[x], x_reg[x | (1 << k)], m);
                                    load_twiddle<L>(t, p.twiddles, 0u);
                                    mont_mul<L>(x_reg[x], sum, t, m);
                                    load_twiddle<L>(t, p.twiddles, 1u);
                                    mont_mul<L>(x_reg[x | (1 << k)], diff, t, m);
                                }
                            }
                        }
                    }
                }
                if (gi == last)
                {
#pragma unroll
                    for (int x = 0; x < regs; ++x)
                    {
#pragma unroll
                        for (int j = 0; j < L; ++j)
                        {
                            p.out[static_cast<uint64_t>(j) * p.elements + ebase + eoff[x]] = x_reg[x][j];
                        }
                    }
                }
                else
                {
#pragma unroll
                    for (int x = 0; x < regs; ++x)
                    {
                        const uint32_t a = smem_addr(base | off[x]);
#pragma unroll
                        for (int j = 0; j < L; ++j)
                        {
                            smem[j * limb_stride + a] = x_reg[x][j];
                        }
                    }
                }
            }
            if (gi != last)
            {
                __syncthreads();
            }
        }
    }

    // R = 3 (8 elements per thread) fits 2 CTAs of 256 threads per SM at
    // L = 8; R = 2 (4 elements) is bounded to 3 CTAs per SM
    template<int L, int R, int Kind, int NW>
    __global__ void __launch_bounds__(256, (R >= 3 ? 2 : 3)) ntt_pass_kernel(const NttPassParams p,
                                                                            const Modulus<L> m)
    {
        // the next pass may be scheduled once every CTA of this one has
        // started; a pass launched with programmatic dependence on the one
        // before proceeds once that one is complete and its writes visible
        asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
        asm volatile("griddepcontrol.wait;" ::: "memory");
        extern __shared__ uint32_t smem[];
        ntt_process<L, R, Kind, NW>(p, m, static_cast<uint64_t>(blockIdx.x) << p.tile_bits, smem);
    }

    // ----------------------------------------------------------------------
    // Persistent transform over a batch of polynomials of uneven degree.
    // Work items are (pass of one polynomial, CTA tile group) in a list that
    // holds every first-pass item before any later-pass item; CTAs take items
    // in list order from an atomic counter.  An item of pass k of a
    // polynomial waits until all earlier-pass items of that polynomial have
    // signalled.  Every item it waits for was taken earlier by a running CTA
    // that never waits on later items, so the waits end; they are still
    // bounded, and a wait that runs out sets `error` and the kernel returns.
    struct BatchedControl
    {
        uint32_t next;      // work counter
        uint32_t error;     // nonzero: a wait ran out (value = item + 1)
        uint32_t done;      // items finished
        uint32_t pad;
    };

    struct BatchedParams
    {
        const NttPassParams* params;    // one per (polynomial, pass)
        const uint32_t* item_param;     // item -> params index
        const uint32_t* item_tile;      // item -> CTA tile group inside that pass
        const uint32_t* item_wait;      // item -> signals needed before it may start (0: none)
        const uint32_t* item_poly;      // item -> polynomial (counter index)
        const uint32_t* item_signal;    // item -> 1 when it must signal its polynomial
        uint32_t* counters;             // per polynomial
        BatchedControl* control;
        uint32_t items;
        uint32_t spin_limit;            // polls of 64 ns before a wait gives up
    };

    __device__ __forceinline__ uint32_t load_acquire(const uint32_t* ptr)
    {
        uint32_t v;
        asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(ptr) : "memory");
        return v;
    }

    template<int L, int R>
    __global__ void __launch_bounds__(256, (R >= 3 ? 2 : 3)) ntt_batched_kernel(const BatchedParams bp,
                                                                               const Modulus<L> m)
    {
        extern __shared__ uint32_t smem[];
        __shared__ uint32_t item_s;
        __shared__ uint32_t abort_s;
        for (;;)
        {
            if (threadIdx.x == 0)
            {
                uint32_t item = atomicAdd(&bp.control->next, 1u);
                uint32_t abort = 0;
                if (item < bp.items)
                {
                    const uint32_t need = bp.item_wait[item];
                    if (need)
                    {
                        const uint32_t* counter = bp.counters + bp.item_poly[item];
                        uint32_t polls = 0;
                        while (load_acquire(counter) < need)
                        {
                            if (++polls > bp.spin_limit || load_acquire(&bp.control->error))
                            {
                                atomicCAS(&bp.control->error, 0u, item + 1u);
                                abort = 1;
                                break;
                            }
                            __nanosleep(64);
                        }
                    }
                }
                item_s = item;
                abort_s = abort;
            }
            __syncthreads();
            const uint32_t item = item_s;
            const uint32_t abort = abort_s;
            __syncthreads();
            if (item >= bp.items || abort)
            {
                return;
            }
            const NttPassParams& p = bp.params[bp.item_param[item]];
            ntt_process<L, R, producer_tensor, 1>(p, m, static_cast<uint64_t>(bp.item_tile[item]) << p.tile_bits,
                                                  smem);
            __syncthreads();
            if (threadIdx.x == 0)
            {
                if (bp.item_signal[item])
                {
                    __threadfence();
                    atomicAdd(bp.counters + bp.item_poly[item], 1u);
                }
                atomicAdd(&bp.control->done, 1u);
            }
        }
    }
}
