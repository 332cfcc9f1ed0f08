// C-ABI layer: contexts (device, stream, RNG capability), registered moduli
// with their cached twiddle tables, the NTT pass planner and the launchers.
#include "../../include/hmpc_gb300.h"

#include <algorithm>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "dispatch.hpp"
#include "host_math.hpp"
#include "internal.hpp"
#include "plan.hpp"

using namespace hmpc_gb300;

namespace hmpc_gb300::detail
{
    thread_local std::string last_error;

    int fail(int code, const std::string& message)
    {
        last_error = message;
        return code;
    }

    int cuda_fail(cudaError_t e, const char* what)
    {
        return fail(HMPC_ERROR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
    }

    void nonce_add(uint32_t nonce[3], uint64_t v)
    {
        uint64_t s = static_cast<uint64_t>(nonce[0]) + static_cast<uint32_t>(v);
        nonce[0] = static_cast<uint32_t>(s);
        s = static_cast<uint64_t>(nonce[1]) + static_cast<uint32_t>(v >> 32) + (s >> 32);
        nonce[1] = static_cast<uint32_t>(s);
        nonce[2] += static_cast<uint32_t>(s >> 32);
    }
}

using namespace hmpc_gb300::detail;

namespace
{
    host::words to_words(const uint32_t* p, int n)
    {
        return host::words(p, p + n);
    }
}

namespace hmpc_gb300::detail
{
    int check_degree(uint64_t n)
    {
        if (n < 4 || (n & (n - 1)) != 0 || n > (1ull << 30))
        {
            return fail(HMPC_ERROR_INVALID_ARGUMENT, "ring degree must be a power of two in [4, 2^30]");
        }
        return HMPC_OK;
    }

    int enter(hmpc_context* ctx)
    {
        if (!ctx)
        {
            return fail(HMPC_ERROR_INVALID_ARGUMENT, "null context");
        }
        HMPC_CUDA(cudaSetDevice(ctx->device), "cudaSetDevice");
        return HMPC_OK;
    }

    int run_transform(hmpc_context* ctx, hmpc_modulus* mod, uint64_t n, uint64_t batch, bool inverse, int kind,
                      uint32_t vx2, uint32_t security, const uint32_t* src, uint32_t* out, const uint32_t* poly_rng,
                      uint32_t rng_slot, bool cuda_cores_only)
    {
        if (int rc = enter(ctx))
        {
            return rc;
        }
        if (!mod)
        {
            return fail(HMPC_ERROR_INVALID_ARGUMENT, "null modulus");
        }
        if (int rc = check_degree(n))
        {
            return rc;
        }
        if (batch == 0)
        {
            return HMPC_OK;
        }
        if (!out)
        {
            return fail(HMPC_ERROR_INVALID_ARGUMENT, "null output");
        }
        Tables* t = nullptr;
        if (int rc = mod->prepare(n, &t))
        {
            return rc;
        }
        const int L = mod->c.limbs;
        int nw = 1;
        uint32_t top_mask = 0xffffffffu;
        if (kind == producer_cbd)
        {
            if (vx2 < 1 || vx2 > 64)
            {
                return fail(HMPC_ERROR_UNSUPPORTED, "centred binomial needs 1 <= 2V <= 64");
            }
            nw = static_cast<int>((2 * vx2 + 31) / 32);
        }
        else if (kind == producer_uniform)
        {
            const uint32_t bits = static_cast<uint32_t>(mod->c.bits) + security;
            nw = static_cast<int>((bits + 31) / 32);
            if (nw != L + 2 && nw != L + 3)
            {
                return fail(HMPC_ERROR_UNSUPPORTED, "uniform sampler supports statistical security 80");
            }
            if (bits % 32)
            {
                top_mask = (1u << (bits % 32)) - 1u;
            }
        }
        else if (kind != producer_tensor)
        {
            return fail(HMPC_ERROR_INVALID_ARGUMENT, "unknown producer kind");
        }
        if (kind == producer_tensor && !src)
        {
            return fail(HMPC_ERROR_INVALID_ARGUMENT, "tensor producer without source");
        }
        const int log_n = __builtin_ctzll(n);
        if (log_n < mod->kt->radix_bits && !poly_rng)
        {
            // fewer stages than one register group holds: the per-stage kernel
            return run_plain(ctx, mod, n, batch, inverse, kind, vx2, security, src, out);
        }
        hmpc_modulus::TileChoice choice;
        {
            std::lock_guard<std::mutex> lock(mod->tables_mutex);
            auto it = mod->tile_choices.find(std::make_tuple(log_n, inverse ? 1 : 0, batch));
            if (it != mod->tile_choices.end())
            {
                choice = it->second;
            }
        }
        if (choice.radix_bits == 0)
        {
            // tensor-core engine; calls it does not cover run the default CUDA-core tiles
            if (!cuda_cores_only && tc_applicable(mod, log_n, kind, poly_rng) &&
                (kind != producer_uniform || !inverse))
            {
                if (kind != producer_uniform)
                {
                    return run_tc_transform(ctx, mod, n, batch, inverse, kind, vx2, src, out, choice.local_bits);
                }
                // the engine's first group reads memory: the stage-0 pairs'
                // uniform draws go to `out` first, then the transform runs in place
                cudaError_t e = mod->kt->uniform_pairs(out, static_cast<uint32_t>(log_n), n * batch, ctx->rng(), nw,
                                                       top_mask, mod->h, ctx->stream);
                if (e != cudaSuccess)
                {
                    return cuda_fail(e, "launching the uniform pair sampler");
                }
                ++ctx->launches;
                if (int rc = run_tc_transform(ctx, mod, n, batch, false, producer_tensor, 0, out, out,
                                              choice.local_bits))
                {
                    return rc;
                }
                nonce_add(ctx->nonce, n * batch);
                return HMPC_OK;
            }
            choice = hmpc_modulus::TileChoice{};
        }
        if (choice.radix_bits == 1)
        {
            // one thread-block cluster per polynomial; calls it does not cover
            // run the default CUDA-core tiles
            if (kind == producer_tensor && !poly_rng && log_n >= 10 && log_n <= 14)
            {
                ClusterNttParams cp{};
                cp.in = src;
                cp.out = out;
                cp.twiddles = inverse ? t->inverse : t->forward;
                cp.elements = n * batch;
                cp.log_n = static_cast<uint32_t>(log_n);
                cp.inverse = inverse ? 1u : 0u;
                cudaError_t e = mod->kt->ntt_cluster(cp, batch, mod->h, ctx->stream);
                if (e != cudaSuccess)
                {
                    return cuda_fail(e, "launching the cluster transform");
                }
                ++ctx->launches;
                return HMPC_OK;
            }
            choice = hmpc_modulus::TileChoice{};
        }
        PlanOptions options;
        options.max_local_bits = choice.local_bits;
        options.col_bits = choice.col_bits;
        const std::vector<PassPlan> plan = plan_transform(L, log_n, batch, inverse, choice.radix_bits, options);
        const RngKey rng = ctx->rng();
        // A pass after the first whose grid fills at most a quarter of the SMs
        // (single polynomials: the launch gap is a large share of its time)
        // launches with programmatic dependence on the pass before: 87.5 ->
        // 84.9 us for one polynomial of 2^15 coefficients at 8 limbs, while
        // 16 polynomials measured 2 % slower that way.  Ordinary launches
        // while the stream is being captured.
        cudaStreamCaptureStatus capture = cudaStreamCaptureStatusNone;
        const bool capturing =
            cudaStreamIsCapturing(ctx->stream, &capture) == cudaSuccess && capture != cudaStreamCaptureStatusNone;
        if (!ctx->sm_count)
        {
            HMPC_CUDA(cudaDeviceGetAttribute(&ctx->sm_count, cudaDevAttrMultiProcessorCount, ctx->device),
                      "querying the SM count");
        }
        for (size_t i = 0; i < plan.size(); ++i)
        {
            NttPassParams p = plan[i].params;
            p.dependent = i > 0 && !capturing && 4ull * plan[i].grid <= static_cast<uint64_t>(ctx->sm_count) ? 1u : 0u;
            p.out = out;
            p.src = i == 0 ? src : nullptr;
            p.twiddles = inverse ? t->inverse : t->forward;
            p.small_table = mod->small_table;
            p.elements = n * batch;
            p.rng = rng;
            p.vx2 = vx2;
            p.top_mask = top_mask;
            p.poly_rng = poly_rng;
            p.rng_slot = rng_slot;
            const int k = i == 0 ? kind : producer_tensor;
            cudaError_t e = mod->kt->ntt_pass(p, k, k == producer_tensor ? 1 : nw, choice.radix_bits, mod->h,
                                              plan[i].grid,
                                              plan[i].block, plan[i].smem, ctx->stream);
            if (e != cudaSuccess)
            {
                return cuda_fail(e, "launching NTT pass");
            }
            ++ctx->launches;
        }
        if (kind != producer_tensor && !poly_rng)
        {
            nonce_add(ctx->nonce, n * batch);
        }
        return HMPC_OK;
    }

    CastParams make_cast(const hmpc_modulus* dst, const hmpc_modulus* src)
    {
        CastParams cp{};
        const int ls = src->c.limbs;
        const int ld = dst->c.limbs;
        cp.src_limbs = static_cast<uint32_t>(ls);
        cp.src_ninv = src->c.ninv;
        for (int j = 0; j < ls; ++j)
        {
            cp.src_q[j] = src->c.q[static_cast<size_t>(j)];
            cp.src_half[j] = src->c.half[static_cast<size_t>(j)];
        }
        const int nw = std::max(ls, ld) + 1;
        cp.norm_words = static_cast<uint32_t>(nw);
        host::words offset;
        if (host::compare(dst->c.q, src->c.q) > 0)
        {
            offset = host::sub(dst->c.q, src->c.q, nw);
            cp.direct = 1;
            for (int j = 0; j < ld; ++j)
            {
                cp.factor[j] = dst->c.r2[static_cast<size_t>(j)];
            }
        }
        else
        {
            const host::words rem = host::mod(src->c.q, dst->c.q);
            offset = host::bit_width(rem) == 0 ? host::words(static_cast<size_t>(nw), 0u) : host::sub(dst->c.q, rem, nw);
            cp.direct = 0;
            host::words wide(static_cast<size_t>(nw + ld), 0u);
            for (int j = 0; j < ld; ++j)
            {
                wide[static_cast<size_t>(nw + j)] = dst->c.r2[static_cast<size_t>(j)];
            }
            const host::words f = host::mod(wide, dst->c.q);
            for (int j = 0; j < ld; ++j)
            {
                cp.factor[j] = f[static_cast<size_t>(j)];
            }
        }
        offset = host::resize(offset, nw);
        for (int j = 0; j < nw; ++j)
        {
            cp.offset[j] = offset[static_cast<size_t>(j)];
        }
        return cp;
    }
}

namespace hmpc_gb300::detail
{
    // x = c0 - s*c1 (+ s^2*c2) -> INTT_q -> cast to p (-> NTT_p)
    int decrypt(hmpc_context* ctx, hmpc_modulus* q, hmpc_modulus* p, uint64_t n, uint64_t batch, const uint32_t* s,
                const uint32_t* c0, const uint32_t* c1, const uint32_t* c2, int plaintext_ntt, uint32_t* out)
    {
        if (int rc = enter(ctx))
        {
            return rc;
        }
        if (!q || !p || !s || !c0 || !c1 || !out)
        {
            return fail(HMPC_ERROR_INVALID_ARGUMENT, "null argument");
        }
        if (int rc = check_degree(n))
        {
            return rc;
        }
        if (batch == 0)
        {
            return HMPC_OK;
        }
        const uint64_t elements = n * batch;
        uint32_t* x = ctx->scratch(elements * static_cast<uint64_t>(q->c.limbs));
        if (!x)
        {
            return fail(HMPC_ERROR_OUT_OF_MEMORY, "allocating the decryption workspace");
        }
        cudaError_t e = q->kt->dec_combine(x, s, n, c0, c1, c2, elements, q->h, ctx->stream);
        if (e != cudaSuccess)
        {
            return cuda_fail(e, "launching decryption combine");
        }
        ++ctx->launches;
        int rc = run_transform(ctx, q, n, batch, true, producer_tensor, 0, 0, x, x);
        if (rc)
        {
            return rc;
        }
        e = p->kt->cast(out, x, elements, make_cast(p, q), p->h, ctx->stream);
        if (e != cudaSuccess)
        {
            return cuda_fail(e, "launching cast");
        }
        ++ctx->launches;
        if (plaintext_ntt)
        {
            rc = run_transform(ctx, p, n, batch, false, producer_tensor, 0, 0, out, out);
        }
        return rc;
    }

    // one launch per stage over global memory (plain.cuh)
    int run_plain(hmpc_context* ctx, hmpc_modulus* mod, uint64_t n, uint64_t batch, bool inverse, int kind,
                  uint32_t vx2, uint32_t security, const uint32_t* src, uint32_t* out)
    {
        if (int rc = enter(ctx))
        {
            return rc;
        }
        if (!mod)
        {
            return fail(HMPC_ERROR_INVALID_ARGUMENT, "null modulus");
        }
        if (int rc = check_degree(n))
        {
            return rc;
        }
        if (batch == 0)
        {
            return HMPC_OK;
        }
        if (!out)
        {
            return fail(HMPC_ERROR_INVALID_ARGUMENT, "null output");
        }
        Tables* t = nullptr;
        if (int rc = mod->prepare(n, &t))
        {
            return rc;
        }
        const int L = mod->c.limbs;
        int nw = 1;
        uint32_t top_mask = 0xffffffffu;
        if (kind == producer_cbd)
        {
            if (vx2 < 1 || vx2 > 64)
            {
                return fail(HMPC_ERROR_UNSUPPORTED, "centred binomial needs 1 <= 2V <= 64");
            }
            nw = static_cast<int>((2 * vx2 + 31) / 32);
        }
        else if (kind == producer_uniform)
        {
            const uint32_t bits = static_cast<uint32_t>(mod->c.bits) + security;
            nw = static_cast<int>((bits + 31) / 32);
            if (nw != L + 2 && nw != L + 3)
            {
                return fail(HMPC_ERROR_UNSUPPORTED, "uniform sampler supports statistical security 80");
            }
            if (bits % 32)
            {
                top_mask = (1u << (bits % 32)) - 1u;
            }
        }
        else if (kind != producer_tensor || !src)
        {
            return fail(HMPC_ERROR_INVALID_ARGUMENT, "bad producer");
        }
        PlainStageParams p{};
        p.out = out;
        p.src = src;
        p.twiddles = inverse ? t->inverse : t->forward;
        p.small_table = mod->small_table;
        p.elements = n * batch;
        p.log_n = static_cast<uint32_t>(__builtin_ctzll(n));
        p.inverse = inverse ? 1u : 0u;
        p.rng = ctx->rng();
        p.vx2 = vx2;
        p.top_mask = top_mask;
        for (uint32_t stage = 0; stage < p.log_n; ++stage)
        {
            p.stage = stage;
            cudaError_t e = mod->kt->plain_stage(p, kind, nw, mod->h, ctx->stream);
            if (e != cudaSuccess)
            {
                return cuda_fail(e, "launching plain stage");
            }
            ++ctx->launches;
        }
        if (kind != producer_tensor)
        {
            nonce_add(ctx->nonce, n * batch);
        }
        return HMPC_OK;
    }
}

extern "C" {

const char* hmpc_last_error(void)
{
    return last_error.c_str();
}

int hmpc_version(int* major, int* minor)
{
    if (major)
    {
        *major = 0;
    }
    if (minor)
    {
        *minor = 1;
    }
    return HMPC_OK;
}

int hmpc_context_create(int device, const uint32_t key[8], void* stream, hmpc_context** out)
{
    if (!out)
    {
        return fail(HMPC_ERROR_INVALID_ARGUMENT, "null output");
    }
    int count = 0;
    HMPC_CUDA(cudaGetDeviceCount(&count), "cudaGetDeviceCount");
    if (device < 0 || device >= count)
    {
        return fail(HMPC_ERROR_INVALID_ARGUMENT, "no such CUDA device");
    }
    HMPC_CUDA(cudaSetDevice(device), "cudaSetDevice");
    auto* ctx = new hmpc_context;
    ctx->device = device;
    ctx->stream = static_cast<cudaStream_t>(stream);
    if (key)
    {
        std::memcpy(ctx->key, key, sizeof ctx->key);
    }
    *out = ctx;
    return HMPC_OK;
}

int hmpc_context_destroy(hmpc_context* ctx)
{
    if (!ctx)
    {
        return HMPC_OK;
    }
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    for (auto* m : ctx->moduli)
    {
        delete m;
    }
    cudaFree(ctx->workspace);
    cudaFree(ctx->tc_workspace);
    cudaFree(ctx->tc_error);
    if (ctx->aux_stream)
    {
        cudaStreamSynchronize(ctx->aux_stream);
        cudaStreamDestroy(ctx->aux_stream);
    }
    if (ctx->fork_event)
    {
        cudaEventDestroy(ctx->fork_event);
    }
    if (ctx->join_event)
    {
        cudaEventDestroy(ctx->join_event);
    }
    delete ctx;
    return HMPC_OK;
}

int hmpc_context_set_stream(hmpc_context* ctx, void* stream)
{
    if (!ctx)
    {
        return fail(HMPC_ERROR_INVALID_ARGUMENT, "null context");
    }
    ctx->stream = static_cast<cudaStream_t>(stream);
    return HMPC_OK;
}

int hmpc_context_get_nonce(const hmpc_context* ctx, uint32_t nonce[3])
{
    if (!ctx || !nonce)
    {
        return fail(HMPC_ERROR_INVALID_ARGUMENT, "null argument");
    }
    std::memcpy(nonce, ctx->nonce, sizeof ctx->nonce);
    return HMPC_OK;
}

int hmpc_context_set_nonce(hmpc_context* ctx, const uint32_t nonce[3])
{
    if (!ctx || !nonce)
    {
        return fail(HMPC_ERROR_INVALID_ARGUMENT, "null argument");
    }
    std::memcpy(ctx->nonce, nonce, sizeof ctx->nonce);
    return HMPC_OK;
}

int hmpc_context_launch_count(const hmpc_context* ctx, uint64_t* count)
{
    if (!ctx || !count)
    {
        return fail(HMPC_ERROR_INVALID_ARGUMENT, "null argument");
    }
    *count = ctx->launches;
    return HMPC_OK;
}

int hmpc_context_synchronize(hmpc_context* ctx)
{
    if (int rc = enter(ctx))
    {
        return rc;
    }
    HMPC_CUDA(cudaStreamSynchronize(ctx->stream), "synchronizing");
    if (ctx->tc_error)
    {
        uint32_t code = 0;
        HMPC_CUDA(cudaMemcpy(&code, ctx->tc_error, sizeof code, cudaMemcpyDeviceToHost), "reading the error word");
        if (code)
        {
            HMPC_CUDA(cudaMemset(ctx->tc_error, 0, sizeof code), "clearing the error word");
            return fail(HMPC_ERROR_TIMEOUT, "a tensor-core transform gave up waiting for its tensor core or copy");
        }
    }
    return HMPC_OK;
}

int hmpc_modulus_create(hmpc_context* ctx, const uint32_t* q, int q_words, hmpc_modulus** out)
{
    if (int rc = enter(ctx))
    {
        return rc;
    }
    if (!q || q_words <= 0 || !out)
    {
        return fail(HMPC_ERROR_INVALID_ARGUMENT, "null modulus words");
    }
    auto m = std::make_unique<hmpc_modulus>();
    std::string error;
    if (!host::make_constants(to_words(q, q_words), m->c, error))
    {
        return fail(HMPC_ERROR_INVALID_ARGUMENT, error);
    }
    const int L = m->c.limbs;
    if (L > max_device_limbs)
    {
        return fail(HMPC_ERROR_UNSUPPORTED, "moduli up to 9 limbs (288 bits) are supported on the device");
    }
    m->ctx = ctx;
    m->kt = kernel_table(L);
    m->h.limbs = L;
    m->h.bits = m->c.bits;
    m->h.ninv = m->c.ninv;
    for (int j = 0; j < L; ++j)
    {
        m->h.q[j] = m->c.q[static_cast<size_t>(j)];
        m->h.one[j] = m->c.one[static_cast<size_t>(j)];
        m->h.r2[j] = m->c.r2[static_cast<size_t>(j)];
        m->h.half[j] = m->c.half[static_cast<size_t>(j)];
    }
    std::vector<uint32_t> small(static_cast<size_t>(65 * L));
    for (uint32_t v = 0; v <= 64; ++v)
    {
        const host::words mv = host::to_mont(m->c, host::words{v});
        std::copy(mv.begin(), mv.end(), small.begin() + static_cast<std::ptrdiff_t>(v * static_cast<uint32_t>(L)));
    }
    HMPC_CUDA(cudaMalloc(&m->small_table, small.size() * sizeof(uint32_t)), "allocating constants");
    HMPC_CUDA(cudaMemcpy(m->small_table, small.data(), small.size() * sizeof(uint32_t), cudaMemcpyHostToDevice),
              "uploading constants");
    ctx->moduli.push_back(m.get());
    *out = m.release();
    return HMPC_OK;
}

int hmpc_modulus_destroy(hmpc_modulus* mod)
{
    if (!mod)
    {
        return HMPC_OK;
    }
    auto& list = mod->ctx->moduli;
    list.erase(std::remove(list.begin(), list.end(), mod), list.end());
    cudaSetDevice(mod->ctx->device);
    cudaStreamSynchronize(mod->ctx->stream);
    delete mod;
    return HMPC_OK;
}

int hmpc_modulus_info(const hmpc_modulus* mod, int* limbs, int* bits, uint32_t* one)
{
    if (!mod)
    {
        return fail(HMPC_ERROR_INVALID_ARGUMENT, "null modulus");
    }
    if (limbs)
    {
        *limbs = mod->c.limbs;
    }
    if (bits)
    {
        *bits = mod->c.bits;
    }
    if (one)
    {
        std::copy(mod->c.one.begin(), mod->c.one.end(), one);
    }
    return HMPC_OK;
}

int hmpc_modulus_prepare(hmpc_modulus* mod, uint64_t n)
{
    if (!mod)
    {
        return fail(HMPC_ERROR_INVALID_ARGUMENT, "null modulus");
    }
    if (int rc = check_degree(n))
    {
        return rc;
    }
    return mod->prepare(n, nullptr);
}

int hmpc_modulus_get_plan(hmpc_modulus* mod, uint64_t n, uint64_t batch, int inverse, int* radix_bits,
                          int* local_bits, int* col_bits)
{
    if (!mod || !radix_bits || !local_bits || !col_bits)
    {
        return fail(HMPC_ERROR_INVALID_ARGUMENT, "null argument");
    }
    if (int rc = check_degree(n))
    {
        return rc;
    }
    hmpc_modulus::TileChoice choice;
    {
        std::lock_guard<std::mutex> lock(mod->tables_mutex);
        auto it = mod->tile_choices.find(std::make_tuple(__builtin_ctzll(n), inverse ? 1 : 0, batch));
        if (it != mod->tile_choices.end())
        {
            choice = it->second;
        }
    }
    *radix_bits = choice.radix_bits;
    *local_bits = choice.local_bits;
    *col_bits = choice.col_bits;
    return HMPC_OK;
}

int hmpc_modulus_tc_cost(hmpc_modulus* mod, uint64_t n, uint64_t batch, int inverse, int producer_kind, int splits,
                         hmpc_tc_cost* out)
{
    if (!mod || !out)
    {
        return fail(HMPC_ERROR_INVALID_ARGUMENT, "null argument");
    }
    if (int rc = check_degree(n))
    {
        return rc;
    }
    return tc_cost(mod, n, batch, inverse != 0, producer_kind, splits, out);
}

int hmpc_modulus_tc_column_max(hmpc_modulus* mod, uint64_t n, int inverse, int splits, uint32_t* out)
{
    if (!mod || !out)
    {
        return fail(HMPC_ERROR_INVALID_ARGUMENT, "null argument");
    }
    if (int rc = enter(mod->ctx))
    {
        return rc;
    }
    if (int rc = check_degree(n))
    {
        return rc;
    }
    return tc_column_max(mod->ctx, mod, n, inverse != 0, splits, out);
}

int hmpc_context_set_test_wait(hmpc_context* ctx, uint32_t polls, int stall)
{
    if (!ctx)
    {
        return fail(HMPC_ERROR_INVALID_ARGUMENT, "null context");
    }
    ctx->tc_spin_limit = polls ? polls : tc_default_spin_limit;
    ctx->tc_test_stall = stall ? 1u : 0u;
    return HMPC_OK;
}

int hmpc_context_set_tc_column_bound(hmpc_context* ctx, uint32_t bound)
{
    if (!ctx)
    {
        return fail(HMPC_ERROR_INVALID_ARGUMENT, "null context");
    }
    if (bound > tc_byte_carry_column_bound)
    {
        return fail(HMPC_ERROR_INVALID_ARGUMENT, "the two-operation carry is exact up to a column bound of 32512");
    }
    ctx->tc_column_bound = bound;
    return HMPC_OK;
}

int hmpc_modulus_set_plan(hmpc_modulus* mod, uint64_t n, uint64_t batch, int inverse, int radix_bits,
                          int local_bits, int col_bits)
{
    if (!mod)
    {
        return fail(HMPC_ERROR_INVALID_ARGUMENT, "null modulus");
    }
    if (int rc = check_degree(n))
    {
        return rc;
    }
    if (radix_bits == 0)
    {
        if (local_bits < 0 || local_bits > 2)
        {
            return fail(HMPC_ERROR_INVALID_ARGUMENT, "the tensor-core engine splits its contiguous group 1 or 2 ways");
        }
        if (!tc_supported(mod))
        {
            return fail(HMPC_ERROR_UNSUPPORTED, "the tensor-core transform needs a 2- to 8-limb modulus below "
                                                "0.996 * 2^(32L) whose top limb is at least 32");
        }
    }
    else if (radix_bits == 1)
    {
        // the cluster engine has no tile shape
        local_bits = 0;
        col_bits = 0;
    }
    else if ((radix_bits != 2 && radix_bits != 3) || local_bits < 0 || local_bits > 13 || col_bits < 0 ||
             col_bits > 6 ||
             (local_bits && static_cast<uint64_t>(mod->c.limbs) * 4u * smem_words(1u << local_bits) > 200 * 1024))
    {
        return fail(HMPC_ERROR_INVALID_ARGUMENT, "tile shape out of range");
    }
    std::lock_guard<std::mutex> lock(mod->tables_mutex);
    mod->tile_choices[std::make_tuple(__builtin_ctzll(n), inverse ? 1 : 0, batch)] = {radix_bits, local_bits,
                                                                                      col_bits};
    return HMPC_OK;
}

int hmpc_modulus_tune(hmpc_modulus* mod, uint64_t n, uint64_t batch, int inverse, float* best_ms)
{
    if (!mod)
    {
        return fail(HMPC_ERROR_INVALID_ARGUMENT, "null modulus");
    }
    hmpc_context* ctx = mod->ctx;
    if (int rc = enter(ctx))
    {
        return rc;
    }
    if (int rc = check_degree(n))
    {
        return rc;
    }
    if (batch == 0)
    {
        return fail(HMPC_ERROR_INVALID_ARGUMENT, "empty batch");
    }
    if (int rc = mod->prepare(n, nullptr))
    {
        return rc;
    }
    const int L = mod->c.limbs;
    const uint64_t words = n * batch * static_cast<uint64_t>(L);
    uint32_t* buf = nullptr;
    if (cudaMalloc(&buf, words * sizeof(uint32_t)) != cudaSuccess)
    {
        return fail(HMPC_ERROR_OUT_OF_MEMORY, "allocating tuning scratch");
    }
    cudaMemsetAsync(buf, 0, words * sizeof(uint32_t), ctx->stream);
    cudaEvent_t t0, t1;
    cudaEventCreate(&t0);
    cudaEventCreate(&t1);
    const int log_n = __builtin_ctzll(n);
    const auto key = std::make_tuple(log_n, inverse ? 1 : 0, batch);
    PlanOptions def;
    const int b0 = local_bits_for(L, def);
    float best = 1e30f;
    hmpc_modulus::TileChoice best_choice;
    auto time_choice = [&](const hmpc_modulus::TileChoice& choice) {
        {
            std::lock_guard<std::mutex> lock(mod->tables_mutex);
            mod->tile_choices[key] = choice;
        }
        float sample = 1e30f;
        for (int rep = 0; rep < 4; ++rep)
        {
            cudaEventRecord(t0, ctx->stream);
            if (run_transform(ctx, mod, n, batch, inverse, producer_tensor, 0, 0, buf, buf) != HMPC_OK)
            {
                return 1e30f;
            }
            cudaEventRecord(t1, ctx->stream);
            cudaEventSynchronize(t1);
            float ms = 0.f;
            cudaEventElapsedTime(&ms, t0, t1);
            if (rep)
            {
                sample = std::min(sample, ms);
            }
        }
        return sample;
    };
    if (log_n >= 4 && tc_supported(mod))
    {
        for (int splits : {1, 2})
        {
            hmpc_modulus::TileChoice tensor;
            tensor.radix_bits = 0;
            tensor.local_bits = splits;
            const float sample = time_choice(tensor);
            if (sample < best)
            {
                best = sample;
                best_choice = tensor;
            }
        }
    }
    if (log_n >= 10 && log_n <= 14 && batch <= 64)
    {
        // one thread-block cluster per polynomial
        hmpc_modulus::TileChoice cluster;
        cluster.radix_bits = 1;
        cluster.local_bits = 0;
        cluster.col_bits = 0;
        const float sample = time_choice(cluster);
        if (sample < best)
        {
            best = sample;
            best_choice = cluster;
        }
    }
    for (int R : {3, 2})
    {
        for (int lb = std::max(R + 2, b0 - 5); lb <= std::min(13, b0 + 1); ++lb)
        {
            if (static_cast<uint64_t>(L) * 4u * smem_words(1u << lb) > 200 * 1024)
            {
                continue;
            }
            for (int c : {3, 4, 5})
            {
                const float sample = time_choice({R, lb, c});
                if (sample < best)
                {
                    best = sample;
                    best_choice = {R, lb, c};
                }
            }
        }
    }
    {
        std::lock_guard<std::mutex> lock(mod->tables_mutex);
        mod->tile_choices[key] = best_choice;
    }
    cudaEventDestroy(t0);
    cudaEventDestroy(t1);
    cudaFree(buf);
    if (best_ms)
    {
        *best_ms = best;
    }
    return HMPC_OK;
}

int hmpc_modulus_root(hmpc_modulus* mod, uint64_t n, int inverse, uint32_t* root)
{
    if (!mod || !root)
    {
        return fail(HMPC_ERROR_INVALID_ARGUMENT, "null argument");
    }
    if (int rc = check_degree(n))
    {
        return rc;
    }
    Tables* t = nullptr;
    if (int rc = mod->prepare(n, &t))
    {
        return rc;
    }
    const host::words& r = inverse ? t->inverse_root : t->root;
    std::copy(r.begin(), r.end(), root);
    return HMPC_OK;
}

int hmpc_modulus_twiddles(hmpc_modulus* mod, uint64_t n, int inverse, uint32_t* host_table)
{
    if (!mod || !host_table)
    {
        return fail(HMPC_ERROR_INVALID_ARGUMENT, "null argument");
    }
    Tables* t = nullptr;
    if (int rc = check_degree(n))
    {
        return rc;
    }
    if (int rc = mod->prepare(n, &t))
    {
        return rc;
    }
    HMPC_CUDA(cudaMemcpy(host_table, inverse ? t->inverse : t->forward,
                         n * static_cast<uint64_t>(mod->c.limbs) * sizeof(uint32_t), cudaMemcpyDeviceToHost),
              "downloading twiddles");
    return HMPC_OK;
}

int hmpc_tensor_alloc(hmpc_context* ctx, uint64_t words, uint32_t** out)
{
    if (int rc = enter(ctx))
    {
        return rc;
    }
    if (!out)
    {
        return fail(HMPC_ERROR_INVALID_ARGUMENT, "null output");
    }
    if (cudaMalloc(out, std::max<uint64_t>(words, 1) * sizeof(uint32_t)) != cudaSuccess)
    {
        return fail(HMPC_ERROR_OUT_OF_MEMORY, "cudaMalloc failed");
    }
    return HMPC_OK;
}

int hmpc_tensor_free(hmpc_context* ctx, uint32_t* ptr)
{
    if (int rc = enter(ctx))
    {
        return rc;
    }
    HMPC_CUDA(cudaFree(ptr), "cudaFree");
    return HMPC_OK;
}

int hmpc_tensor_upload(hmpc_context* ctx, uint32_t* dst, const uint32_t* host, uint64_t words)
{
    if (int rc = enter(ctx))
    {
        return rc;
    }
    HMPC_CUDA(cudaMemcpyAsync(dst, host, words * sizeof(uint32_t), cudaMemcpyHostToDevice, ctx->stream), "upload");
    return HMPC_OK;
}

int hmpc_tensor_download(hmpc_context* ctx, uint32_t* host, const uint32_t* src, uint64_t words)
{
    if (int rc = enter(ctx))
    {
        return rc;
    }
    HMPC_CUDA(cudaMemcpyAsync(host, src, words * sizeof(uint32_t), cudaMemcpyDeviceToHost, ctx->stream),
              "download");
    HMPC_CUDA(cudaStreamSynchronize(ctx->stream), "download");
    return HMPC_OK;
}

int hmpc_ntt_forward(hmpc_context* ctx, hmpc_modulus* mod, uint64_t n, uint64_t batch, const hmpc_producer* producer,
                     uint32_t* out)
{
    if (!producer)
    {
        return fail(HMPC_ERROR_INVALID_ARGUMENT, "null producer");
    }
    return run_transform(ctx, mod, n, batch, false, producer->kind, producer->variance_x2, producer->security,
                         producer->src, out);
}

int hmpc_ntt_inverse(hmpc_context* ctx, hmpc_modulus* mod, uint64_t n, uint64_t batch, const uint32_t* in,
                     uint32_t* out)
{
    return run_transform(ctx, mod, n, batch, true, producer_tensor, 0, 0, in, out);
}

int hmpc_fma(hmpc_context* ctx, hmpc_modulus* mod, uint64_t elements, const uint32_t* a, const uint32_t* b,
             const uint32_t* c, uint32_t* d)
{
    if (int rc = enter(ctx))
    {
        return rc;
    }
    if (!mod || (elements && (!a || !b || !c || !d)))
    {
        return fail(HMPC_ERROR_INVALID_ARGUMENT, "null argument");
    }
    cudaError_t e = mod->kt->fma(d, a, b, c, elements, mod->h, ctx->stream);
    ctx->launches += elements ? 1 : 0;
    return e == cudaSuccess ? HMPC_OK : cuda_fail(e, "launching fma");
}

int hmpc_binary(hmpc_context* ctx, hmpc_modulus* mod, int op, uint64_t elements, const uint32_t* a,
                uint64_t a_elements, const uint32_t* b, uint64_t b_elements, uint32_t* out)
{
    if (int rc = enter(ctx))
    {
        return rc;
    }
    if (!mod || op < 0 || op > 2)
    {
        return fail(HMPC_ERROR_INVALID_ARGUMENT, "bad modulus or operation");
    }
    if (elements == 0)
    {
        return HMPC_OK;
    }
    if (!a || !b || !out || a_elements == 0 || b_elements == 0 || elements % a_elements || elements % b_elements)
    {
        return fail(HMPC_ERROR_INVALID_ARGUMENT, "operand sizes must divide the result size");
    }
    cudaError_t e = mod->kt->binary(out, a, a_elements, b, b_elements, elements, op, mod->h, ctx->stream);
    ++ctx->launches;
    return e == cudaSuccess ? HMPC_OK : cuda_fail(e, "launching binary op");
}

int hmpc_sample_uniform(hmpc_context* ctx, hmpc_modulus* mod, uint64_t elements, uint32_t security, uint32_t* out)
{
    if (int rc = enter(ctx))
    {
        return rc;
    }
    if (!mod || (elements && !out))
    {
        return fail(HMPC_ERROR_INVALID_ARGUMENT, "null argument");
    }
    const uint32_t bits = static_cast<uint32_t>(mod->c.bits) + security;
    const int words = static_cast<int>((bits + 31) / 32);
    if (words != mod->c.limbs + 2 && words != mod->c.limbs + 3)
    {
        return fail(HMPC_ERROR_UNSUPPORTED, "uniform sampler supports statistical security 80");
    }
    const uint32_t top_mask = bits % 32 ? (1u << (bits % 32)) - 1u : 0xffffffffu;
    cudaError_t e = mod->kt->uniform(out, elements, ctx->rng(), words, top_mask, mod->h, ctx->stream);
    ctx->launches += elements ? 1 : 0;
    if (e != cudaSuccess)
    {
        return cuda_fail(e, "launching uniform sampler");
    }
    nonce_add(ctx->nonce, elements);
    return HMPC_OK;
}

int hmpc_sample_cbd(hmpc_context* ctx, hmpc_modulus* mod, uint64_t elements, uint32_t variance_x2, uint32_t* out)
{
    if (int rc = enter(ctx))
    {
        return rc;
    }
    if (!mod || (elements && !out))
    {
        return fail(HMPC_ERROR_INVALID_ARGUMENT, "null argument");
    }
    if (variance_x2 < 1 || variance_x2 > 64)
    {
        return fail(HMPC_ERROR_UNSUPPORTED, "centred binomial needs 1 <= 2V <= 64");
    }
    cudaError_t e = mod->kt->cbd(out, elements, ctx->rng(), variance_x2, mod->small_table, mod->h, ctx->stream);
    ctx->launches += elements ? 1 : 0;
    if (e != cudaSuccess)
    {
        return cuda_fail(e, "launching binomial sampler");
    }
    nonce_add(ctx->nonce, elements);
    return HMPC_OK;
}

int hmpc_cast(hmpc_context* ctx, hmpc_modulus* dst, hmpc_modulus* src, uint64_t elements, const uint32_t* in,
              uint32_t* out)
{
    if (int rc = enter(ctx))
    {
        return rc;
    }
    if (!dst || !src || (elements && (!in || !out)))
    {
        return fail(HMPC_ERROR_INVALID_ARGUMENT, "null argument");
    }
    cudaError_t e = dst->kt->cast(out, in, elements, make_cast(dst, src), dst->h, ctx->stream);
    ctx->launches += elements ? 1 : 0;
    return e == cudaSuccess ? HMPC_OK : cuda_fail(e, "launching cast");
}

int hmpc_to_montgomery(hmpc_context* ctx, hmpc_modulus* mod, uint64_t elements, const uint32_t* in, uint32_t* out)
{
    if (int rc = enter(ctx))
    {
        return rc;
    }
    if (!mod)
    {
        return fail(HMPC_ERROR_INVALID_ARGUMENT, "null modulus");
    }
    cudaError_t e = mod->kt->to_montgomery(out, in, elements, mod->h, ctx->stream);
    ctx->launches += elements ? 1 : 0;
    return e == cudaSuccess ? HMPC_OK : cuda_fail(e, "launching conversion");
}

int hmpc_from_montgomery(hmpc_context* ctx, hmpc_modulus* mod, uint64_t elements, const uint32_t* in, uint32_t* out)
{
    if (int rc = enter(ctx))
    {
        return rc;
    }
    if (!mod)
    {
        return fail(HMPC_ERROR_INVALID_ARGUMENT, "null modulus");
    }
    cudaError_t e = mod->kt->from_montgomery(out, in, elements, mod->h, ctx->stream);
    ctx->launches += elements ? 1 : 0;
    return e == cudaSuccess ? HMPC_OK : cuda_fail(e, "launching conversion");
}

int hmpc_lhe_enc(hmpc_context* ctx, hmpc_modulus* q, hmpc_modulus* p, uint64_t n, uint64_t batch,
                 const uint32_t* key_a, const uint32_t* key_b, const uint32_t* plaintext, int plaintext_ntt,
                 uint32_t* c0, uint32_t* c1)
{
    if (int rc = enter(ctx))
    {
        return rc;
    }
    if (!q || !p || !key_a || !key_b || !plaintext || !c0 || !c1)
    {
        return fail(HMPC_ERROR_INVALID_ARGUMENT, "null argument");
    }
    if (int rc = check_degree(n))
    {
        return rc;
    }
    if (batch == 0)
    {
        return HMPC_OK;
    }
    const uint64_t elements = n * batch;
    const uint64_t lq = static_cast<uint64_t>(q->c.limbs);
    const uint64_t lp = static_cast<uint64_t>(p->c.limbs);
    const uint64_t poly_words = elements * lq;
    uint32_t* ws = ctx->scratch(3 * poly_words + (plaintext_ntt ? elements * lp : 0));
    if (!ws)
    {
        return fail(HMPC_ERROR_OUT_OF_MEMORY, "allocating the encryption workspace");
    }
    uint32_t* u = ws;
    uint32_t* v = ws + poly_words;
    uint32_t* msg = ws + 2 * poly_words;
    uint32_t* coeff = ws + 3 * poly_words;
    const int tc_splits = tc_plan_splits(q, n, batch);
    if (tc_splits && n >= 16 && tc_supported(q) && p->c.limbs <= 2)
    {
        // Tensor-core plan for q: the NTT is linear, so p*NTT(v) + NTT(lift(m))
        // is one transform of the small integers p*v + lift(m) drawn and lifted
        // in its first group, and p*NTT(w) one of p*w.  The three transforms
        // (u, p*v + lift(m), p*w) share every constant after their first
        // group, so they run stacked: three first-group launches, then the
        // other groups once over 3 * batch polynomials.  One combine reads u
        // once and writes c0 and c1; every result is the reduced
        // representative, so the ciphertext is the reference's bit for bit.  RNG order as the
        // reference's plan: u, v, w (expr/cache.hpp:226-271).
        int rc = HMPC_OK;
        const uint32_t* coefficients = plaintext;
        if (plaintext_ntt)
        {
            rc = run_transform(ctx, p, n, batch, true, producer_tensor, 0, 0, plaintext, coeff);
            coefficients = coeff;
        }
        const TcSmallInput with_msg{coefficients, p};
        const TcSmallInput no_msg{nullptr, p};
        TcStackPart parts[3];
        parts[0].vx2 = 1;
        parts[1].vx2 = 20;
        parts[1].small = &with_msg;
        parts[2].vx2 = 20;
        parts[2].small = &no_msg;
        uint32_t* stacked = ws;  // [L][3 * elements]: u | p*v + lift(m) | p*w, in NTT form
        if (!rc)
        {
            rc = run_tc_stacked(ctx, q, n, batch, parts, 3, stacked, tc_splits);
        }
        if (!rc)
        {
            cudaError_t e = q->kt->lhe_combine_pair(c0, c1, key_a, key_b, n, stacked, elements, q->h, ctx->stream);
            if (e != cudaSuccess)
            {
                return cuda_fail(e, "launching combine");
            }
            ++ctx->launches;
        }
        return rc;
    }
    // the execution order of the reference's plan: NTT(u), NTT(v),
    // [INTT_p(x)], NTT_q(msg), c0, NTT(w), c1 (expr/cache.hpp:226-271)
    int rc = run_transform(ctx, q, n, batch, false, producer_cbd, 1, 0, nullptr, u);
    if (!rc)
    {
        rc = run_transform(ctx, q, n, batch, false, producer_cbd, 20, 0, nullptr, v);
    }
    const uint32_t* coefficients = plaintext;
    if (!rc && plaintext_ntt)
    {
        rc = run_transform(ctx, p, n, batch, true, producer_tensor, 0, 0, plaintext, coeff);
        coefficients = coeff;
    }
    if (!rc)
    {
        cudaError_t e = q->kt->cast(msg, coefficients, elements, make_cast(q, p), q->h, ctx->stream);
        if (e != cudaSuccess)
        {
            return cuda_fail(e, "launching cast");
        }
        ++ctx->launches;
        rc = run_transform(ctx, q, n, batch, false, producer_tensor, 0, 0, msg, msg);
    }
    const host::words pm = host::to_mont(q->c, p->c.q);
    if (!rc)
    {
        cudaError_t e = q->kt->lhe_combine(c0, key_a, n, u, v, msg, elements, pm.data(), q->h, ctx->stream);
        if (e != cudaSuccess)
        {
            return cuda_fail(e, "launching combine");
        }
        ++ctx->launches;
        rc = run_transform(ctx, q, n, batch, false, producer_cbd, 20, 0, nullptr, v);  // w reuses v's buffer
    }
    if (!rc)
    {
        cudaError_t e = q->kt->lhe_combine(c1, key_b, n, u, v, nullptr, elements, pm.data(), q->h, ctx->stream);
        if (e != cudaSuccess)
        {
            return cuda_fail(e, "launching combine");
        }
        ++ctx->launches;
    }
    return rc;
}

int hmpc_lhe_dec(hmpc_context* ctx, hmpc_modulus* q, hmpc_modulus* p, uint64_t n, uint64_t batch,
                 const uint32_t* s, const uint32_t* c0, const uint32_t* c1, int plaintext_ntt, uint32_t* out)
{
    return decrypt(ctx, q, p, n, batch, s, c0, c1, nullptr, plaintext_ntt, out);
}

int hmpc_lhe_dec2(hmpc_context* ctx, hmpc_modulus* q, hmpc_modulus* p, uint64_t n, uint64_t batch,
                  const uint32_t* s, const uint32_t* c0, const uint32_t* c1, const uint32_t* c2, int plaintext_ntt,
                  uint32_t* out)
{
    if (!c2)
    {
        return fail(HMPC_ERROR_INVALID_ARGUMENT, "null c2");
    }
    return decrypt(ctx, q, p, n, batch, s, c0, c1, c2, plaintext_ntt, out);
}

int hmpc_lhe_ct_mul(hmpc_context* ctx, hmpc_modulus* q, uint64_t elements, const uint32_t* a0, const uint32_t* a1,
                    const uint32_t* b0, const uint32_t* b1, uint32_t* d0, uint32_t* d1, uint32_t* d2)
{
    if (int rc = enter(ctx))
    {
        return rc;
    }
    if (!q || (elements && (!a0 || !a1 || !b0 || !b1 || !d0 || !d1 || !d2)))
    {
        return fail(HMPC_ERROR_INVALID_ARGUMENT, "null argument");
    }
    cudaError_t e = q->kt->ct_mul(d0, d1, d2, a0, a1, b0, b1, elements, q->h, ctx->stream);
    if (e != cudaSuccess)
    {
        return cuda_fail(e, "launching ciphertext product");
    }
    ctx->launches += elements ? 1 : 0;
    return HMPC_OK;
}

int hmpc_ntt_forward_plain(hmpc_context* ctx, hmpc_modulus* mod, uint64_t n, uint64_t batch,
                           const hmpc_producer* producer, uint32_t* out)
{
    if (!producer)
    {
        return fail(HMPC_ERROR_INVALID_ARGUMENT, "null producer");
    }
    return run_plain(ctx, mod, n, batch, false, producer->kind, producer->variance_x2, producer->security,
                     producer->src, out);
}

int hmpc_ntt_inverse_plain(hmpc_context* ctx, hmpc_modulus* mod, uint64_t n, uint64_t batch, const uint32_t* in,
                           uint32_t* out)
{
    return run_plain(ctx, mod, n, batch, true, producer_tensor, 0, 0, in, out);
}

int hmpc_lhe_keygen(hmpc_context* ctx, hmpc_modulus* q, hmpc_modulus* p, uint64_t n, uint32_t* s, uint32_t* a,
                    uint32_t* b)
{
    if (int rc = enter(ctx))
    {
        return rc;
    }
    if (!q || !p || !s || !a || !b)
    {
        return fail(HMPC_ERROR_INVALID_ARGUMENT, "null argument");
    }
    if (int rc = check_degree(n))
    {
        return rc;
    }
    uint32_t* e_poly = ctx->scratch(n * static_cast<uint64_t>(q->c.limbs));
    if (!e_poly)
    {
        return fail(HMPC_ERROR_OUT_OF_MEMORY, "allocating the key workspace");
    }
    int rc = hmpc_sample_uniform(ctx, q, n, 80, b);
    // s and e are independent transforms; on the CUDA-core passes (no shared
    // workspace) e's runs on the context's second stream meanwhile.  The
    // nonces are taken on the host in the reference's order either way.
    bool fork = false;
    if (!rc)
    {
        std::lock_guard<std::mutex> lock(q->tables_mutex);
        auto it = q->tile_choices.find(std::make_tuple(__builtin_ctzll(n), 0, static_cast<uint64_t>(1)));
        const int radix = it == q->tile_choices.end() ? hmpc_modulus::TileChoice{}.radix_bits : it->second.radix_bits;
        fork = radix != 0 && __builtin_ctzll(n) >= q->kt->radix_bits;
    }
    fork = fork && ctx->aux();
    if (fork)
    {
        HMPC_CUDA(cudaEventRecord(ctx->fork_event, ctx->stream), "forking the key generation");
        HMPC_CUDA(cudaStreamWaitEvent(ctx->aux_stream, ctx->fork_event, 0), "forking the key generation");
    }
    if (!rc)
    {
        rc = run_transform(ctx, q, n, 1, false, producer_cbd, 1, 0, nullptr, s);
    }
    if (!rc)
    {
        cudaStream_t main = ctx->stream;
        if (fork)
        {
            ctx->stream = ctx->aux_stream;
        }
        rc = run_transform(ctx, q, n, 1, false, producer_cbd, 20, 0, nullptr, e_poly);
        ctx->stream = main;
    }
    if (fork)
    {
        HMPC_CUDA(cudaEventRecord(ctx->join_event, ctx->aux_stream), "joining the key generation");
        HMPC_CUDA(cudaStreamWaitEvent(ctx->stream, ctx->join_event, 0), "joining the key generation");
    }
    if (!rc)
    {
        const host::words pm = host::to_mont(q->c, p->c.q);
        cudaError_t e = q->kt->lhe_combine(a, b, n, s, e_poly, nullptr, n, pm.data(), q->h, ctx->stream);
        if (e != cudaSuccess)
        {
            return cuda_fail(e, "launching combine");
        }
        ++ctx->launches;
    }
    return rc;
}

}  // extern "C"
