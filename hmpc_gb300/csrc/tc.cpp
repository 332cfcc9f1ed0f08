// Host side of the tensor-core transform: group plan, lazily generated
// constant matrices per (modulus, degree, direction), and the launch sequence.
#include <algorithm>
#include <cmath>

#include <cuda_fp16.h>

#include "internal.hpp"
#include "tcgen05.cuh"

using namespace hmpc_gb300;
using namespace hmpc_gb300::detail;

namespace
{
    const TcKernels* kernels_of(const hmpc_modulus* mod)
    {
        return tc_kernels(mod->c.limbs);
    }

    // groups of three stages from the first stage on; the remainder (1-3
    // stages) is the last group, whose constants are the most numerous in the
    // forward direction (one matrix per block above it)
    std::vector<TcGroupPlan> plan_groups(const TcKernels* k, int log_n, bool inverse, int contiguous_splits)
    {
        const int count = (log_n + 2) / 3;
        std::vector<TcGroupPlan> groups;
        for (int j = 0; j < count; ++j)
        {
            TcGroupPlan gp;
            gp.s0 = static_cast<uint32_t>(3 * j);
            gp.g = static_cast<uint32_t>(j + 1 < count ? 3 : log_n - 3 * (count - 1));
            gp.lo = inverse ? gp.s0 : static_cast<uint32_t>(log_n) - gp.s0 - gp.g;
            gp.blocks = 1ull << (static_cast<uint32_t>(log_n) - gp.lo - gp.g);
            gp.in_kind = j == 0 ? tc_in_limbs : tc_in_digits;
            gp.out_kind = j + 1 == count ? tc_out_limbs : tc_out_digits;
            // a group with one block per 2^g contiguous elements (the forward
            // transform's last, the inverse's first) has as many constant
            // matrices as rows per matrix are few: split in two, each image fits
            // twice in shared memory and the next block's streams in meanwhile;
            // unsplit, the digit tile is converted once per block instead of twice
            const int splits = (gp.g == 3 && gp.lo == 0) ? contiguous_splits : 1;
            k->shape(1 << gp.g, gp.in_kind, gp.out_kind, splits, gp.shape);
            groups.push_back(gp);
        }
        // a last group whose rows are adjacent elements reads digit planes
        // blocked per row (one contiguous run per row instead of a short piece
        // per word plane), written so by the group before it
        TcGroupPlan& last = groups.back();
        if (last.lo == 0 && last.shape.splits == 1 && last.in_kind == tc_in_digits && groups.size() >= 2)
        {
            last.layout |= 1;
            groups[groups.size() - 2].layout |= 2;
        }
        return groups;
    }

    // the largest sum of |digit| over one column (output digit) of a group's images
    __global__ void tc_column_bound_kernel(const uint8_t* images, uint64_t columns, uint32_t n_mma,
                                           uint32_t image_bytes, uint32_t k_pad, uint32_t* out)
    {
        const uint64_t id = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
        if (id >= columns)
        {
            return;
        }
        const uint8_t* img = images + (id / n_mma) * image_bytes;
        const uint32_t n = static_cast<uint32_t>(id % n_mma);
        float sum = 0.0f;  // at most 288 * 128: exact
        for (uint32_t k = 0; k < k_pad; ++k)
        {
            sum += fabsf(__half2float(*reinterpret_cast<const __half*>(img + tc::operand_offset(n, k, n_mma))));
        }
        atomicMax(out, static_cast<uint32_t>(sum));
    }

    // the largest column sum of |digit| of a digit-fed group's constants (the
    // group keeps its sums in the two-operation carry's range while it is at
    // most tc_byte_carry_column_bound)
    int column_bound(hmpc_context* ctx, const TcGroupPlan& gp, const uint8_t* images, uint32_t* d_max,
                     uint32_t* out)
    {
        const uint64_t columns = gp.blocks * gp.shape.splits * gp.shape.n_mma;
        HMPC_CUDA(cudaMemsetAsync(d_max, 0, sizeof(uint32_t), ctx->stream), "clearing the column bound");
        tc_column_bound_kernel<<<static_cast<unsigned>((columns + 255) / 256), 256, 0, ctx->stream>>>(
            images, columns, gp.shape.n_mma, gp.shape.b_bytes, gp.shape.k_pad, d_max);
        HMPC_CUDA(cudaGetLastError(), "launching the column bound");
        uint32_t bound = 0;
        HMPC_CUDA(cudaMemcpyAsync(&bound, d_max, sizeof(uint32_t), cudaMemcpyDeviceToHost, ctx->stream),
                  "reading the column bound");
        HMPC_CUDA(cudaStreamSynchronize(ctx->stream), "checking tensor-core constants");
        *out = bound;
        return HMPC_OK;
    }

    // generate and expand one group's constants into `images`
    int build_group(hmpc_context* ctx, hmpc_modulus* mod, const Tables* t, int log_n, bool inverse,
                    const TcGroupPlan& gp, bool montgomery, uint32_t d_in, uint8_t* images, uint32_t* gx,
                    const uint32_t* pow256)
    {
        const TcKernels* k = kernels_of(mod);
        TcGenParams gen{};
        gen.twiddles = inverse ? t->inverse : t->forward;
        gen.gx = gx;
        gen.blocks = gp.blocks;
        gen.log_n = static_cast<uint32_t>(log_n);
        gen.inverse = inverse ? 1u : 0u;
        gen.s0 = gp.s0;
        gen.g = gp.g;
        gen.lo = gp.lo;
        gen.montgomery = montgomery ? 1u : 0u;
        HMPC_CUDA(k->gen(gen, mod->h, ctx->stream), "generating tensor-core constants");
        TcExpandParams ex{};
        ex.gx = gx;
        ex.pow256 = pow256;
        ex.images = images;
        ex.blocks = gp.blocks;
        ex.r = 1u << gp.g;
        ex.dc = static_cast<uint32_t>(k->digits);
        ex.d_in = d_in;
        ex.splits = gp.shape.splits;
        ex.n_mma = gp.shape.n_mma;
        ex.image_bytes = gp.shape.b_bytes;
        // the loaders of r = 8 groups fed by digits or limbs whose rows are
        // strided elements (the kernel's contiguous variant runs where lo = 0)
        // take word-major K
        ex.word_major = ex.r == 8 && d_in >= ex.dc && gp.lo != 0 ? 1u : 0u;
        for (int j = 0; j < mod->c.limbs; ++j)
        {
            ex.half[j] = mod->c.half[static_cast<size_t>(j)];
        }
        HMPC_CUDA(k->expand(ex, mod->h, ctx->stream), "expanding tensor-core constants");
        return HMPC_OK;
    }

    int prepare_tc(hmpc_context* ctx, hmpc_modulus* mod, uint64_t n, bool inverse, int splits, bool need_cbd,
                   bool need_small, TcTables** out)
    {
        Tables* t = nullptr;
        if (int rc = mod->prepare(n, &t))
        {
            return rc;
        }
        const int log_n = __builtin_ctzll(n);
        const TcKernels* k = kernels_of(mod);
        const int L = mod->c.limbs;
        std::lock_guard<std::mutex> lock(mod->tables_mutex);
        auto key = std::make_tuple(log_n, inverse ? 1 : 0, splits);
        auto it = mod->tc_tables.find(key);
        const bool fresh = it == mod->tc_tables.end();
        if (!fresh && !it->second.fit)
        {
            return fail(HMPC_ERROR_UNSUPPORTED,
                        "this modulus's tensor-core constants exceed the carry's range; use a CUDA-core tile shape");
        }
        if (!fresh && (!need_cbd || it->second.first_cbd) && (!need_small || it->second.first_small))
        {
            *out = &it->second;
            return HMPC_OK;
        }
        TcTables tt;
        if (!fresh)
        {
            tt = it->second;
        }
        else
        {
            tt.groups = plan_groups(k, log_n, inverse, splits);
            size_t bytes = 0;
            for (auto& gp : tt.groups)
            {
                gp.offset = bytes;
                bytes += static_cast<size_t>(gp.blocks) * gp.shape.splits * gp.shape.b_bytes;
                bytes = (bytes + 255) & ~static_cast<size_t>(255);
            }
            tt.bytes = bytes;
        }
        // 256^a * R mod q for every digit slot
        const uint32_t slots = static_cast<uint32_t>(k->digits + 2);
        std::vector<uint32_t> pow256(static_cast<size_t>(slots) * L);
        for (uint32_t a = 0; a < slots; ++a)
        {
            host::words v(static_cast<size_t>(a / 4 + 1), 0u);
            v[a / 4] = 1u << (8 * (a % 4));
            const host::words mv = host::to_mont(mod->c, v);
            for (int j = 0; j < L; ++j)
            {
                pow256[static_cast<size_t>(a) * L + j] = mv[static_cast<size_t>(j)];
            }
        }
        uint64_t gx_words = 0;
        for (const auto& gp : tt.groups)
        {
            gx_words = std::max<uint64_t>(gx_words, (gp.blocks << (2 * gp.g)) * static_cast<uint64_t>(L));
        }
        uint32_t* d_pow = nullptr;
        uint32_t* d_gx = nullptr;
        auto cleanup = [&]() {
            cudaStreamSynchronize(ctx->stream);
            cudaFree(d_pow);
            cudaFree(d_gx);
        };
        if (cudaMalloc(&d_pow, (pow256.size() + 1) * sizeof(uint32_t)) != cudaSuccess ||
            cudaMalloc(&d_gx, gx_words * sizeof(uint32_t)) != cudaSuccess)
        {
            cleanup();
            return fail(HMPC_ERROR_OUT_OF_MEMORY, "allocating tensor-core generation scratch");
        }
        if (cudaMemcpyAsync(d_pow, pow256.data(), pow256.size() * sizeof(uint32_t), cudaMemcpyHostToDevice,
                            ctx->stream) != cudaSuccess)
        {
            cleanup();
            return fail(HMPC_ERROR_CUDA, "uploading digit powers");
        }
        if (fresh)
        {
            if (cudaMalloc(&tt.images, tt.bytes) != cudaSuccess)
            {
                cleanup();
                return fail(HMPC_ERROR_OUT_OF_MEMORY, "allocating tensor-core constants");
            }
            cudaMemsetAsync(tt.images, 0, tt.bytes, ctx->stream);
            for (const auto& gp : tt.groups)
            {
                if (int rc = build_group(ctx, mod, t, log_n, inverse, gp, false, gp.shape.d_in, tt.images + gp.offset,
                                         d_gx, d_pow))
                {
                    cleanup();
                    cudaFree(tt.images);
                    return rc;
                }
                // the generation scratch is reused by the next group
                cudaStreamSynchronize(ctx->stream);
                if (gp.in_kind == tc_in_digits)
                {
                    uint32_t bound = 0;
                    if (int rc = column_bound(ctx, gp, tt.images + gp.offset, d_pow + pow256.size(), &bound))
                    {
                        cleanup();
                        cudaFree(tt.images);
                        return rc;
                    }
                    tt.column_max = std::max(tt.column_max, bound);
                }
                if (tt.column_max > ctx->tc_column_bound)
                {
                    cleanup();
                    cudaFree(tt.images);
                    TcTables unfit;
                    unfit.fit = false;
                    unfit.column_max = tt.column_max;
                    mod->tc_tables[key] = unfit;
                    return fail(HMPC_ERROR_UNSUPPORTED, "this modulus's tensor-core constants exceed the carry's "
                                                        "range; use a CUDA-core tile shape");
                }
            }
        }
        if (need_cbd && !tt.first_cbd)
        {
            // first forward group fed by raw samples: constants G * R
            k->shape(8, tc_in_cbd, tc_out_digits, 1, tt.cbd_shape);
            TcGroupPlan gp = tt.groups.front();
            gp.shape = tt.cbd_shape;
            if (cudaMalloc(&tt.first_cbd, tt.cbd_shape.b_bytes) != cudaSuccess)
            {
                cleanup();
                return fail(HMPC_ERROR_OUT_OF_MEMORY, "allocating tensor-core constants");
            }
            cudaMemsetAsync(tt.first_cbd, 0, tt.cbd_shape.b_bytes, ctx->stream);
            if (int rc = build_group(ctx, mod, t, log_n, inverse, gp, true, 1, tt.first_cbd, d_gx, d_pow))
            {
                cleanup();
                return rc;
            }
        }
        if (need_small && !tt.first_small)
        {
            // first forward group fed by x = p * sample + lift(m): constants G * R * 256^a, 9 digit slots
            k->shape(8, tc_in_small, tc_out_digits, 1, tt.small_shape);
            TcGroupPlan gp = tt.groups.front();
            gp.shape = tt.small_shape;
            if (cudaMalloc(&tt.first_small, tt.small_shape.b_bytes) != cudaSuccess)
            {
                cleanup();
                return fail(HMPC_ERROR_OUT_OF_MEMORY, "allocating tensor-core constants");
            }
            cudaMemsetAsync(tt.first_small, 0, tt.small_shape.b_bytes, ctx->stream);
            if (int rc = build_group(ctx, mod, t, log_n, inverse, gp, true, tc_small_digits, tt.first_small, d_gx,
                                     d_pow))
            {
                cleanup();
                return rc;
            }
        }
        cleanup();
        if (cudaGetLastError() != cudaSuccess)
        {
            return fail(HMPC_ERROR_CUDA, "generating tensor-core constants");
        }
        mod->tc_tables[key] = tt;
        *out = &mod->tc_tables[key];
        return HMPC_OK;
    }

    // whether a forward plan starts with two three-stage groups and has at
    // least two more after them (the wide group replaces the first two)
    bool wide_plan(const std::vector<TcGroupPlan>& groups)
    {
        // the second group must write plain planes (not the blocked runs of a
        // group before the last)
        return groups.size() >= 4 && groups[0].g == 3 && groups[1].g == 3 && (groups[1].layout & 2) == 0;
    }

    bool wide_plan(const TcTables* tt)
    {
        return wide_plan(tt->groups);
    }

    // the wide group's images: unscaled, and scaled by p (nullptr: not needed)
    int prepare_wide(hmpc_context* ctx, hmpc_modulus* mod, uint64_t n, TcTables* tt, const hmpc_modulus* p)
    {
        const int L = mod->c.limbs;
        std::vector<uint32_t> pwords;
        if (p)
        {
            pwords.assign(p->c.q.begin(), p->c.q.end());
        }
        Tables* t = nullptr;
        if (int rc = mod->prepare(n, &t))
        {
            return rc;
        }
        std::lock_guard<std::mutex> lock(mod->tables_mutex);
        const bool need_plain = !tt->wide_cbd;
        const bool need_p = p && (!tt->wide_cbd_p || tt->wide_p != pwords);
        if (!need_plain && !need_p)
        {
            return HMPC_OK;
        }
        const TcKernels* k = kernels_of(mod);
        const int log_n = __builtin_ctzll(n);
        const uint32_t image_bytes = tc_wide_b_bytes;
        const size_t images_bytes = static_cast<size_t>(tc_wide_splits) * image_bytes;
        uint32_t *gx_a = nullptr, *gx_b = nullptr, *gx6 = nullptr, *d_pow = nullptr, *d_scale = nullptr;
        auto cleanup = [&]() {
            cudaStreamSynchronize(ctx->stream);
            cudaFree(gx_a);
            cudaFree(gx_b);
            cudaFree(gx6);
            cudaFree(d_pow);
            cudaFree(d_scale);
        };
        if (cudaMalloc(&gx_a, 64u * L * sizeof(uint32_t)) != cudaSuccess ||
            cudaMalloc(&gx_b, 8u * 64u * L * sizeof(uint32_t)) != cudaSuccess ||
            cudaMalloc(&gx6, 64u * 64u * L * sizeof(uint32_t)) != cudaSuccess ||
            cudaMalloc(&d_pow, L * sizeof(uint32_t)) != cudaSuccess ||
            cudaMalloc(&d_scale, L * sizeof(uint32_t)) != cudaSuccess)
        {
            cleanup();
            return fail(HMPC_ERROR_OUT_OF_MEMORY, "allocating tensor-core generation scratch");
        }
        // the first two groups' matrices in Montgomery form
        for (int j = 0; j < 2; ++j)
        {
            const TcGroupPlan& gp = tt->groups[static_cast<size_t>(j)];
            TcGenParams gen{};
            gen.twiddles = t->forward;
            gen.gx = j == 0 ? gx_a : gx_b;
            gen.blocks = gp.blocks;
            gen.log_n = static_cast<uint32_t>(log_n);
            gen.inverse = 0;
            gen.s0 = gp.s0;
            gen.g = gp.g;
            gen.lo = gp.lo;
            gen.montgomery = 1;
            if (cudaError_t e = k->gen(gen, mod->h, ctx->stream))
            {
                cleanup();
                return cuda_fail(e, "generating tensor-core constants");
            }
        }
        // raw samples: one digit slot, 256^0 * R
        const host::words one = host::to_mont(mod->c, host::words{1u});
        cudaMemcpyAsync(d_pow, one.data(), L * sizeof(uint32_t), cudaMemcpyHostToDevice, ctx->stream);
        for (int variant = 0; variant < 2; ++variant)
        {
            if ((variant == 0 && !need_plain) || (variant == 1 && !need_p))
            {
                continue;
            }
            TcCombineParams cp{};
            cp.gx_a = gx_a;
            cp.gx_b = gx_b;
            cp.gx = gx6;
            if (variant == 1)
            {
                const host::words pm = host::to_mont(mod->c, p->c.q);
                cudaMemcpyAsync(d_scale, pm.data(), L * sizeof(uint32_t), cudaMemcpyHostToDevice, ctx->stream);
                cp.scale = d_scale;
            }
            if (cudaError_t e = k->combine6(cp, mod->h, ctx->stream))
            {
                cleanup();
                return cuda_fail(e, "combining tensor-core constants");
            }
            uint8_t*& images = variant == 0 ? tt->wide_cbd : tt->wide_cbd_p;
            if (!images && cudaMalloc(&images, images_bytes) != cudaSuccess)
            {
                cleanup();
                return fail(HMPC_ERROR_OUT_OF_MEMORY, "allocating tensor-core constants");
            }
            cudaMemsetAsync(images, 0, images_bytes, ctx->stream);
            TcExpandParams ex{};
            ex.gx = gx6;
            ex.pow256 = d_pow;
            ex.images = images;
            ex.blocks = 1;
            ex.r = tc_wide_r;
            ex.dc = static_cast<uint32_t>(k->digits);
            ex.d_in = 1;
            ex.splits = tc_wide_splits;
            ex.n_mma = 256;
            ex.image_bytes = image_bytes;
            ex.word_major = 0;
            for (int j = 0; j < L; ++j)
            {
                ex.half[j] = mod->c.half[static_cast<size_t>(j)];
            }
            if (cudaError_t e = k->expand(ex, mod->h, ctx->stream))
            {
                cleanup();
                return cuda_fail(e, "expanding tensor-core constants");
            }
            // gx6 is reused by the next variant
            cudaStreamSynchronize(ctx->stream);
        }
        cleanup();
        if (need_p)
        {
            tt->wide_p = pwords;
        }
        return HMPC_OK;
    }
}

namespace hmpc_gb300::detail
{
    bool tc_supported(const hmpc_modulus* mod)
    {
        const int L = mod->c.limbs;
        if (!tc_kernels(L))
        {
            return false;
        }
        // q / 2 must have 4L balanced base-256 digits: floor(q / 2) <= 0x7F7F...7F
        host::words bound(static_cast<size_t>(L), 0x7F7F7F7Fu);
        if (host::compare(mod->c.half, bound) > 0)
        {
            return false;
        }
        // the quotient estimate of the final reduction reads the top limb
        return mod->c.q[static_cast<size_t>(L - 1)] >= 32u;
    }

    bool tc_applicable(const hmpc_modulus* mod, int log_n, int kind, const uint32_t* poly_rng)
    {
        return log_n >= 4 && !poly_rng && (kind == producer_tensor || kind == producer_cbd || kind == producer_uniform) &&
               tc_supported(mod);
    }

    // launch state shared by the groups of one transform (or one stack of them)
    struct TcLaunch
    {
        hmpc_context* ctx;
        hmpc_modulus* mod;
        const TcKernels* k;
        TcTables* tt;
        uint32_t log_n;
        float inv_q_top;
        cudaStream_t stream = nullptr;
        // polynomials in buffers of their own: the first group's input and
        // the last group's output tables (device arrays of pointers)
        const uint32_t* const* in_polys = nullptr;
        uint32_t* const* out_polys = nullptr;

        int init(hmpc_context* c, hmpc_modulus* m, uint64_t n, TcTables* t)
        {
            ctx = c;
            stream = c->stream;
            mod = m;
            k = kernels_of(m);
            tt = t;
            log_n = static_cast<uint32_t>(__builtin_ctzll(n));
            const int L = m->c.limbs;
            // 2^(32(L-1)) / q from the top two limbs
            const double top = static_cast<double>(m->c.q[static_cast<size_t>(L - 1)]) +
                               static_cast<double>(m->c.q[static_cast<size_t>(L - 2)]) / 4294967296.0;
            inv_q_top = static_cast<float>(1.0 / top);
            if (!ctx->tc_error)
            {
                HMPC_CUDA(cudaMalloc(&ctx->tc_error, sizeof(uint32_t)), "allocating the error word");
                HMPC_CUDA(cudaMemsetAsync(ctx->tc_error, 0, sizeof(uint32_t), ctx->stream), "clearing the error word");
            }
            if (!ctx->sm_count)
            {
                HMPC_CUDA(cudaDeviceGetAttribute(&ctx->sm_count, cudaDevAttrMultiProcessorCount, ctx->device),
                          "querying the SM count");
            }
            return HMPC_OK;
        }

        // group j over `batch` polynomials; stride = plane stride of the digit / limb planes
        // dependent: the kernel before this one in the stream is another group
        // of this call (programmatic dependent launch)
        int group(size_t j, const uint32_t* in, uint32_t* out, uint64_t stride, uint64_t batch, int in_kind,
                  uint32_t vx2, const TcSmallInput* small, uint64_t msg_stride, bool dependent = false)
        {
            const TcGroupPlan& gp = tt->groups[j];
            const bool first_sampled = j == 0 && (in_kind == tc_in_cbd || in_kind == tc_in_small);
            TcGroupParams p{};
            p.in = in;
            p.out = out;
            p.images = first_sampled ? (in_kind == tc_in_small ? tt->first_small : tt->first_cbd)
                                     : tt->images + gp.offset;
            p.error = ctx->tc_error;
            p.elements = stride;
            p.rows = batch << gp.lo;
            p.tiles_per_block = static_cast<uint32_t>((p.rows + tc_rows - 1) / tc_rows);
            p.tiles = gp.blocks * gp.shape.splits * p.tiles_per_block;
            // launches captured into a graph keep ordinary dependences
            cudaStreamCaptureStatus capture = cudaStreamCaptureStatusNone;
            if (dependent && cudaStreamIsCapturing(stream, &capture) == cudaSuccess &&
                capture != cudaStreamCaptureStatusNone)
            {
                dependent = false;
            }
            p.dependent = dependent ? 1u : 0u;
            p.log_n = log_n;
            p.lo = gp.lo;
            p.spin_limit = ctx->tc_spin_limit;
            p.test_stall = ctx->tc_test_stall;
            p.rng = ctx->rng();
            p.vx2 = vx2;
            p.nw = (2 * vx2 + 31) / 32;
            for (int i = 0; i < mod->c.limbs; ++i)
            {
                p.q[i] = mod->c.q[static_cast<size_t>(i)];
            }
            p.inv_q_top = inv_q_top;
            p.block_shift = tt->groups.back().g;  // the last group's elements per row
            if (small)
            {
                const hmpc_modulus* pm = small->p;
                p.msg = small->msg;
                p.msg_stride = msg_stride;
                p.msg_limbs = static_cast<uint32_t>(pm->c.limbs);
                p.pninv = pm->c.ninv;
                for (int i = 0; i < pm->c.limbs; ++i)
                {
                    p.pq[i] = pm->c.q[static_cast<size_t>(i)];
                    p.phalf[i] = pm->c.half[static_cast<size_t>(i)];
                }
            }
            const unsigned grid =
                static_cast<unsigned>(std::min<uint64_t>(p.tiles, static_cast<uint64_t>(ctx->sm_count)));
            const int splits = first_sampled ? 1 : static_cast<int>(gp.shape.splits);
            int layout = gp.layout;
            if (j == 0 && in_polys)
            {
                p.in_polys = in_polys;
                layout |= 4;
            }
            if (j + 1 == tt->groups.size() && out_polys)
            {
                p.out_polys = out_polys;
                layout |= 4;
            }
            cudaError_t e = k->group(p, 1 << gp.g, in_kind, gp.out_kind, splits, layout, grid, stream);
            if (e != cudaSuccess)
            {
                return cuda_fail(e, "launching a tensor-core transform group");
            }
            ++ctx->launches;
            return HMPC_OK;
        }

        // the first six stages of `batch` CBD(vx2)-fed transforms in one wide
        // group (images: the eight images of G6 or G6 * p), written as digit
        // planes of plane stride `stride` at `out`
        int wide(const uint8_t* images, uint32_t* out, uint64_t stride, uint64_t batch, uint32_t vx2)
        {
            TcGroupParams p{};
            p.out = out;
            p.images = images;
            p.error = ctx->tc_error;
            p.elements = stride;
            p.lo = log_n - 6;
            p.rows = batch << p.lo;
            p.tiles_per_block = static_cast<uint32_t>((p.rows + tc_rows - 1) / tc_rows);
            p.tiles = p.tiles_per_block;
            p.log_n = log_n;
            p.spin_limit = ctx->tc_spin_limit;
            p.rng = ctx->rng();
            p.vx2 = vx2;
            p.nw = (2 * vx2 + 31) / 32;
            // dependent launch: its constants were built before this call's
            // first launch, and its workers wait for the kernel before it
            // (ordinary launches while the stream is being captured)
            cudaStreamCaptureStatus capture = cudaStreamCaptureStatusNone;
            p.dependent = cudaStreamIsCapturing(stream, &capture) == cudaSuccess &&
                                  capture == cudaStreamCaptureStatusNone
                              ? 1u
                              : 0u;
            const unsigned grid =
                static_cast<unsigned>(std::min<uint64_t>(p.tiles, static_cast<uint64_t>(ctx->sm_count)));
            cudaError_t e = k->wide(p, grid, stream);
            if (e != cudaSuccess)
            {
                return cuda_fail(e, "launching the wide tensor-core group");
            }
            ++ctx->launches;
            return HMPC_OK;
        }
    };

    int run_tc_transform(hmpc_context* ctx, hmpc_modulus* mod, uint64_t n, uint64_t batch, bool inverse, int kind,
                         uint32_t vx2, const uint32_t* src, uint32_t* out, int splits, const TcSmallInput* small)
    {
        const bool cbd = kind == producer_cbd;
        if (small && (!cbd || inverse || !small->p || small->p->c.limbs > 2))
        {
            return fail(HMPC_ERROR_UNSUPPORTED, "the small-integer first group needs a forward CBD transform and p < 2^64");
        }
        if (cbd && (vx2 < 1 || vx2 > 64))
        {
            return fail(HMPC_ERROR_UNSUPPORTED, "centred binomial needs 1 <= 2V <= 64");
        }
        TcTables* tt = nullptr;
        if (splits != 1 && splits != 2)
        {
            splits = 1;
        }
        if (int rc = prepare_tc(ctx, mod, n, inverse, splits, cbd && !small, small != nullptr, &tt))
        {
            return rc;
        }
        const uint64_t elements = n * batch;
        const uint64_t w = tt->groups.front().shape.w_out;
        const size_t stages = tt->groups.size();
        uint32_t* digits = nullptr;
        if (stages > 1)
        {
            digits = ctx->tc_scratch((stages > 2 ? 2 : 1) * w * elements);
            if (!digits)
            {
                return fail(HMPC_ERROR_OUT_OF_MEMORY, "allocating tensor-core digit buffers");
            }
        }
        TcLaunch run;
        if (int rc = run.init(ctx, mod, n, tt))
        {
            return rc;
        }
        if (cbd && !small && !inverse && wide_plan(tt))
        {
            // the first six stages in one wide group into buffer 1, then the
            // groups from the third on
            if (int rc = prepare_wide(ctx, mod, n, tt, nullptr))
            {
                return rc;
            }
            if (int rc = run.wide(tt->wide_cbd, digits + w * elements, elements, batch, vx2))
            {
                return rc;
            }
            for (size_t j = 2; j < stages; ++j)
            {
                const uint32_t* in = digits + (((j - 1) & 1u) ? w * elements : 0);
                uint32_t* o = j + 1 == stages ? out : digits + ((j & 1u) ? w * elements : 0);
                if (int rc = run.group(j, in, o, elements, batch, tc_in_digits, 0, nullptr, elements, true))
                {
                    return rc;
                }
            }
            nonce_add(ctx->nonce, elements);
            return HMPC_OK;
        }
        const int first_kind = cbd ? (small ? tc_in_small : tc_in_cbd) : tc_in_limbs;
        for (size_t j = 0; j < stages; ++j)
        {
            const uint32_t* in = j == 0 ? src : digits + (((j - 1) & 1u) ? w * elements : 0);
            uint32_t* o = j + 1 == stages ? out : digits + ((j & 1u) ? w * elements : 0);
            if (int rc = run.group(j, in, o, elements, batch, j == 0 ? first_kind : tc_in_digits, vx2,
                                   j == 0 ? small : nullptr, elements, j > 0))
            {
                return rc;
            }
        }
        if (cbd)
        {
            nonce_add(ctx->nonce, elements);
        }
        return HMPC_OK;
    }

    int run_tc_stacked(hmpc_context* ctx, hmpc_modulus* mod, uint64_t n, uint64_t batch, const TcStackPart* parts,
                       int count, uint32_t* out, int splits)
    {
        bool need_cbd = false, need_small = false;
        for (int i = 0; i < count; ++i)
        {
            if (parts[i].vx2 < 1 || parts[i].vx2 > 64)
            {
                return fail(HMPC_ERROR_UNSUPPORTED, "centred binomial needs 1 <= 2V <= 64");
            }
            if (parts[i].small && (!parts[i].small->p || parts[i].small->p->c.limbs > 2))
            {
                return fail(HMPC_ERROR_UNSUPPORTED, "the small-integer first group needs p < 2^64");
            }
            (parts[i].small ? need_small : need_cbd) = true;
        }
        if (splits != 1 && splits != 2)
        {
            splits = 1;
        }
        TcTables* tt = nullptr;
        if (int rc = prepare_tc(ctx, mod, n, false, splits, need_cbd, need_small, &tt))
        {
            return rc;
        }
        const uint64_t elements = n * batch;
        const uint64_t total = elements * static_cast<uint64_t>(count);
        const uint64_t w = tt->groups.front().shape.w_out;
        const size_t stages = tt->groups.size();
        uint32_t* digits = ctx->tc_scratch((stages > 2 ? 2 : 1) * w * total);
        if (!digits)
        {
            return fail(HMPC_ERROR_OUT_OF_MEMORY, "allocating tensor-core digit buffers");
        }
        TcLaunch run;
        if (int rc = run.init(ctx, mod, n, tt))
        {
            return rc;
        }
        // Parts fed by CBD samples alone (or p times them) take the first six
        // stages in one wide group into their slice of buffer 1; the others
        // their first group into buffer 0 and the second from there into
        // buffer 1 -- the shared groups then start at the third.  Launch order
        // (and so nonce order) stays the parts' order.
        const hmpc_modulus* scale_p = nullptr;
        bool any_wide = false;
        for (int i = 0; i < count; ++i)
        {
            if (!parts[i].small)
            {
                any_wide = true;
            }
            else if (!parts[i].small->msg)
            {
                any_wide = true;
                scale_p = parts[i].small->p;
            }
        }
        const bool use_wide = any_wide && wide_plan(tt);
        if (use_wide)
        {
            if (int rc = prepare_wide(ctx, mod, n, tt, scale_p))
            {
                return rc;
            }
            for (int i = 0; i < count; ++i)
            {
                uint32_t* slice0 = digits + static_cast<uint64_t>(i) * elements;
                uint32_t* slice1 = digits + w * total + static_cast<uint64_t>(i) * elements;
                if (!parts[i].small || !parts[i].small->msg)
                {
                    const uint8_t* images = parts[i].small ? tt->wide_cbd_p : tt->wide_cbd;
                    if (int rc = run.wide(images, slice1, total, batch, parts[i].vx2))
                    {
                        return rc;
                    }
                    nonce_add(ctx->nonce, elements);
                    continue;
                }
                if (int rc = run.group(0, nullptr, slice0, total, batch, tc_in_small, parts[i].vx2, parts[i].small,
                                       elements, i > 0))
                {
                    return rc;
                }
                nonce_add(ctx->nonce, elements);
                if (int rc = run.group(1, slice0, slice1, total, batch, tc_in_digits, 0, nullptr, 0, true))
                {
                    return rc;
                }
            }
            for (size_t j = 2; j < stages; ++j)
            {
                const uint32_t* in = digits + (((j - 1) & 1u) ? w * total : 0);
                uint32_t* o = j + 1 == stages ? out : digits + ((j & 1u) ? w * total : 0);
                if (int rc = run.group(j, in, o, total, batch * static_cast<uint64_t>(count), tc_in_digits, 0, nullptr,
                                       0, true))
                {
                    return rc;
                }
            }
            return HMPC_OK;
        }
        // first groups: part i into its slice of buffer 0 (plane-major slices,
        // or whole blocked runs when the next group is the last)
        const bool blocked = (tt->groups.front().layout & 2) != 0;
        for (int i = 0; i < count; ++i)
        {
            uint32_t* slice = digits + static_cast<uint64_t>(i) * elements * (blocked ? w : 1);
            const int kind = parts[i].small ? tc_in_small : tc_in_cbd;
            if (int rc = run.group(0, nullptr, stages == 1 ? out + static_cast<uint64_t>(i) * elements : slice, total,
                                   batch, kind, parts[i].vx2, parts[i].small, elements, i > 0))
            {
                return rc;
            }
            nonce_add(ctx->nonce, elements);
        }
        // the shared groups over the stacked batch
        for (size_t j = 1; j < stages; ++j)
        {
            const uint32_t* in = digits + (((j - 1) & 1u) ? w * total : 0);
            uint32_t* o = j + 1 == stages ? out : digits + ((j & 1u) ? w * total : 0);
            if (int rc = run.group(j, in, o, total, batch * static_cast<uint64_t>(count), tc_in_digits, 0, nullptr, 0,
                                   true))
            {
                return rc;
            }
        }
        return HMPC_OK;
    }

    int tc_prepare_polys(hmpc_context* ctx, hmpc_modulus* mod, uint64_t n, bool inverse, int splits,
                         uint64_t* digit_words_per_element)
    {
        if (!tc_supported(mod) || n < 16 || (splits != 1 && splits != 2))
        {
            return fail(HMPC_ERROR_UNSUPPORTED, "the tensor-core engine does not cover this transform");
        }
        TcTables* tt = nullptr;
        if (int rc = prepare_tc(ctx, mod, n, inverse, splits, false, false, &tt))
        {
            return rc;
        }
        TcLaunch run;
        if (int rc = run.init(ctx, mod, n, tt))
        {
            return rc;
        }
        const uint64_t w = tt->groups.front().shape.w_out;
        *digit_words_per_element = tt->groups.size() > 1 ? (tt->groups.size() > 2 ? 2 : 1) * w : 0;
        return HMPC_OK;
    }

    int run_tc_polys(hmpc_context* ctx, hmpc_modulus* mod, uint64_t n, uint64_t count, bool inverse, int splits,
                     const uint32_t* const* in_polys, uint32_t* const* out_polys, uint32_t* digits,
                     cudaStream_t stream)
    {
        TcTables* tt = nullptr;
        {
            std::lock_guard<std::mutex> lock(mod->tables_mutex);
            auto it = mod->tc_tables.find(std::make_tuple(__builtin_ctzll(n), inverse ? 1 : 0, splits));
            if (it == mod->tc_tables.end() || !it->second.fit || !it->second.images)
            {
                return fail(HMPC_ERROR_INVALID_ARGUMENT, "tensor-core constants not prepared for this degree");
            }
            tt = &it->second;
        }
        const uint64_t elements = n * count;
        const uint64_t w = tt->groups.front().shape.w_out;
        const size_t stages = tt->groups.size();
        TcLaunch run;
        if (int rc = run.init(ctx, mod, n, tt))
        {
            return rc;
        }
        run.stream = stream;
        run.in_polys = in_polys;
        run.out_polys = out_polys;
        for (size_t j = 0; j < stages; ++j)
        {
            const uint32_t* in = j == 0 ? nullptr : digits + (((j - 1) & 1u) ? w * elements : 0);
            uint32_t* o = j + 1 == stages ? nullptr : digits + ((j & 1u) ? w * elements : 0);
            if (int rc = run.group(j, in, o, elements, count, j == 0 ? tc_in_limbs : tc_in_digits, 0, nullptr, 0))
            {
                return rc;
            }
        }
        return HMPC_OK;
    }

    int tc_cost(hmpc_modulus* mod, uint64_t n, uint64_t batch, bool inverse, int kind, int splits, hmpc_tc_cost* out)
    {
        if (!tc_supported(mod) || n < 16 || (kind != producer_tensor && kind != producer_cbd) ||
            (kind == producer_cbd && inverse) || (splits != 1 && splits != 2))
        {
            return fail(HMPC_ERROR_UNSUPPORTED, "the tensor-core engine does not cover this transform");
        }
        const TcKernels* k = kernels_of(mod);
        const int log_n = __builtin_ctzll(n);
        const std::vector<TcGroupPlan> groups = plan_groups(k, log_n, inverse, splits);
        const double elements = static_cast<double>(n) * static_cast<double>(batch);
        const double limb_bytes = 4.0 * mod->c.limbs;
        out->launches = static_cast<uint32_t>(groups.size());
        out->bytes = 0.0;
        out->flops = 0.0;
        size_t first = 0;
        if (kind == producer_cbd && wide_plan(groups))
        {
            // the wide group: digit planes written, eight images read, eight
            // N = 256 products of K = 64 per 128-row tile
            const uint64_t rows = batch << (log_n - 6);
            const double tiles = static_cast<double>((rows + tc_rows - 1) / tc_rows);
            out->launches -= 1;
            out->bytes += elements * 4.0 * groups[1].shape.w_out +
                          static_cast<double>(tc_wide_splits) * tc_wide_b_bytes;
            out->flops += tiles * tc_wide_splits * 2.0 * tc_rows * 256.0 * tc_wide_r;
            first = 2;
        }
        for (size_t j = first; j < groups.size(); ++j)
        {
            TcShapeInfo shape = groups[j].shape;
            const bool cbd = j == 0 && kind == producer_cbd;
            if (cbd)
            {
                k->shape(8, tc_in_cbd, tc_out_digits, 1, shape);
            }
            const double in = j == 0 ? (cbd ? 0.0 : limb_bytes) : 4.0 * shape.w_in;
            const double outb = j + 1 == groups.size() ? limb_bytes : 4.0 * shape.w_out;
            const uint64_t rows = batch << groups[j].lo;
            const double tiles = static_cast<double>(groups[j].blocks * shape.splits) *
                                 static_cast<double>((rows + tc_rows - 1) / tc_rows);
            out->bytes += elements * (in + outb) + static_cast<double>(groups[j].blocks * shape.splits) * shape.b_bytes;
            out->flops += tiles * 2.0 * tc_rows * shape.n_mma * shape.k_pad;
        }
        return HMPC_OK;
    }

    int tc_column_max(hmpc_context* ctx, hmpc_modulus* mod, uint64_t n, bool inverse, int splits, uint32_t* out)
    {
        if (!tc_supported(mod) || n < 16)
        {
            return fail(HMPC_ERROR_UNSUPPORTED, "the tensor-core engine does not cover this transform");
        }
        if (splits != 1 && splits != 2)
        {
            return fail(HMPC_ERROR_INVALID_ARGUMENT, "the contiguous group splits 1 or 2 ways");
        }
        TcTables* tt = nullptr;
        const int rc = prepare_tc(ctx, mod, n, inverse, splits, false, false, &tt);
        if (rc && rc != HMPC_ERROR_UNSUPPORTED)
        {
            return rc;
        }
        std::lock_guard<std::mutex> lock(mod->tables_mutex);
        auto it = mod->tc_tables.find(std::make_tuple(__builtin_ctzll(n), inverse ? 1 : 0, splits));
        if (it == mod->tc_tables.end())
        {
            return rc ? rc : fail(HMPC_ERROR_CUDA, "tensor-core constants missing");
        }
        *out = it->second.column_max;
        return HMPC_OK;
    }

    int tc_plan_splits(hmpc_modulus* mod, uint64_t n, uint64_t batch)
    {
        std::lock_guard<std::mutex> lock(mod->tables_mutex);
        auto it = mod->tile_choices.find(std::make_tuple(__builtin_ctzll(n), 0, batch));
        if (it == mod->tile_choices.end() || it->second.radix_bits != 0)
        {
            return 0;
        }
        return it->second.local_bits == 2 ? 2 : 1;
    }
}

