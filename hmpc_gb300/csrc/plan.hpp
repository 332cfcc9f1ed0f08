// Pass planner for the tiled transform (see ntt.cuh): splits the log2(N)
// stages into shared-memory passes and each pass into register groups.
#pragma once

#include <algorithm>
#include <cstdint>
#include <vector>

#include "ntt.cuh"

namespace hmpc_gb300
{
    struct PassPlan
    {
        NttPassParams params;
        unsigned grid = 0;
        unsigned block = 0;
        size_t smem = 0;
    };

    struct PlanOptions
    {
        int max_local_bits = 0;   // 0: derived from the shared-memory budget
        int col_bits = 4;         // preferred coalescing width (2^c consecutive elements)
        int smem_budget = 112 * 1024;
        bool spread_small_batches = true;  // shrink CTA tiles to fill the GPU when the batch is small
    };

    inline uint32_t smem_words(uint32_t local_count)
    {
        return local_count + (local_count >> 5);
    }

    inline int local_bits_for(int limbs, const PlanOptions& o)
    {
        if (o.max_local_bits)
        {
            return o.max_local_bits;
        }
        int b = 13;
        while (b > 4 && static_cast<uint64_t>(limbs) * 4u * smem_words(1u << b) > static_cast<uint64_t>(o.smem_budget))
        {
            --b;
        }
        return b;
    }

    struct BitRange
    {
        int lo, hi, c;
    };

    // Bit ranges in forward-stage order (top bits first).
    inline std::vector<BitRange> plan_ranges(int log_n, int b, int col_pref)
    {
        std::vector<BitRange> r;
        int hi = log_n;
        while (hi > b)
        {
            int w = std::max(1, b - col_pref);
            if (hi - w < 1)
            {
                w = hi - 1;
            }
            // keep the final contiguous pass within the budget: never leave more
            // than b bits below unless another column pass follows
            const int lo = hi - w;
            const int c = std::min(std::min(b - w, lo), 5);
            r.push_back({lo, hi, c});
            hi = lo;
        }
        r.push_back({0, hi, 0});
        return r;
    }

    // every pass must hold at least one full register group inside a tile
    // (c + w >= R); shrink the column pass above a too-narrow final pass
    inline void keep_register_groups(std::vector<BitRange>& r, int R, int b)
    {
        if (r.size() >= 2 && r.back().hi < R)
        {
            BitRange& prev = r[r.size() - 2];
            const int grow = R - r.back().hi;
            prev.lo += grow;
            prev.c = std::min(std::min(b - (prev.hi - prev.lo), prev.lo), 5);
            r.back().hi += grow;
        }
    }

    inline std::vector<PassPlan> plan_transform(int limbs, int log_n, uint64_t batch, bool inverse, int R,
                                                const PlanOptions& o = {})
    {
        const int b = local_bits_for(limbs, o);
        std::vector<BitRange> ranges = plan_ranges(log_n, b, o.col_bits);
        keep_register_groups(ranges, R, b);
        if (inverse)
        {
            std::reverse(ranges.begin(), ranges.end());
        }
        std::vector<PassPlan> out;
        for (const BitRange& rg : ranges)
        {
            PassPlan pp{};
            NttPassParams& p = pp.params;
            const int w = rg.hi - rg.lo;
            const int c = rg.c;
            p.log_n = static_cast<uint32_t>(log_n);
            p.inverse = inverse ? 1u : 0u;
            if (inverse)
            {
                p.s0 = static_cast<uint32_t>(rg.lo);
                p.s1 = static_cast<uint32_t>(rg.hi);
            }
            else
            {
                p.s0 = static_cast<uint32_t>(log_n - rg.hi);
                p.s1 = static_cast<uint32_t>(log_n - rg.lo);
            }
            p.row_shift = static_cast<uint32_t>(rg.lo);
            p.col_bits = static_cast<uint32_t>(c);
            const uint64_t tiles_per_poly = 1ull << (log_n - w - c);
            p.tiles = batch * tiles_per_poly;
            int tile_bits = std::max(0, b - w - c);
            if (!o.spread_small_batches)
            {
                // whole CTA groups inside one polynomial
                tile_bits = std::min(tile_bits, log_n - w - c);
            }
            tile_bits = std::max(tile_bits, R - w - c);
            // keep at least ~2 CTAs per SM when the batch is small, as long as a
            // CTA still holds a full register block per thread
            while (o.spread_small_batches && tile_bits > 0 && tile_bits + w + c > R + 5 &&
                   ((p.tiles + (1ull << tile_bits) - 1) >> tile_bits) < 304)
            {
                --tile_bits;
            }
            p.tile_bits = static_cast<uint32_t>(tile_bits);
            p.local_bits = static_cast<uint32_t>(tile_bits + w + c);
            // register groups
            int g = 0;
            for (int s = static_cast<int>(p.s0); s < static_cast<int>(p.s1); s += R, ++g)
            {
                NttGroup& grp = p.groups[g];
                grp.stage = static_cast<uint32_t>(s);
                grp.count = static_cast<uint32_t>(std::min(R, static_cast<int>(p.s1) - s));
                uint32_t used = 0;
                for (int k = 0; k < static_cast<int>(grp.count); ++k)
                {
                    const int stage = s + k;
                    const int bit = inverse ? stage : (log_n - 1 - stage);
                    const int local = c + (bit - rg.lo);
                    grp.reg_pos[k] = static_cast<uint32_t>(local);
                    used |= 1u << local;
                }
                int next = 0;
                for (int k = static_cast<int>(grp.count); k < R; ++k)
                {
                    while (used & (1u << next))
                    {
                        ++next;
                    }
                    grp.reg_pos[k] = static_cast<uint32_t>(next);
                    used |= 1u << next;
                }
                grp.rest_mask = ((1u << p.local_bits) - 1u) & ~used;
            }
            p.num_groups = static_cast<uint32_t>(g);
            pp.grid = static_cast<unsigned>((p.tiles + (1ull << tile_bits) - 1) >> tile_bits);
            pp.block = static_cast<unsigned>(std::min<uint32_t>(256u, 1u << (p.local_bits - R)));
            pp.smem = static_cast<size_t>(limbs) * 4u * smem_words(1u << p.local_bits);
            out.push_back(pp);
        }
        return out;
    }
}
