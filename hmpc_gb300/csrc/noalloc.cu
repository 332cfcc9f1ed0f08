// BGV encryption that allocates no device memory.
//
// hmpc_lhe_enc keeps its intermediates (the NTT'd randomness u and v/w and
// the lifted message) in a per-context workspace that grows with cudaMalloc
// and is released with cudaFree.  Some callers cannot allocate: a serving
// process whose device memory is reserved up front by its own pool, or a
// latency-critical loop that must not pay the implicit device-wide
// synchronisation that cudaMalloc and cudaFree can trigger.  For them,
// hmpc_lhe_enc_noalloc takes its intermediates from one fixed array in device
// memory that is part of this library's image.  Its transforms always run on
// the CUDA-core tiles (the tensor-core engine keeps digit buffers and constant
// images of its own, which it allocates), in the reference's four-transform
// order; the ciphertexts are bit-identical to hmpc_lhe_enc's on either engine.
#include <cstdint>
#include <mutex>
#include <string>

#include "internal.hpp"

// 8 Mi words = 32 MiB.  Every GPU that loads this library holds the array
// until the process exits; every call on a device shares it.
static constexpr uint64_t noalloc_scratch_words = 8ull << 20;
static __device__ __align__(256) uint32_t hmpc_noalloc_scratch[noalloc_scratch_words];

namespace
{
    constexpr int max_devices = 64;
    std::mutex setup_mutex;
    uint32_t* scratch_address[max_devices] = {};

    // Device address of the array on the current device.  The name of a
    // __device__ variable in host code is only a host-side stand-in, so the
    // address is looked up once per device (with that device current) and
    // kept.
    int scratch_on_current_device(int device, uint32_t** out)
    {
        using hmpc_gb300::detail::fail;
        if (device < 0 || device >= max_devices)
        {
            return fail(HMPC_ERROR_UNSUPPORTED, "device index beyond the allocation-free entry point's table");
        }
        std::lock_guard<std::mutex> lock(setup_mutex);
        if (!scratch_address[device])
        {
            void* ptr = nullptr;
            const cudaError_t e = cudaGetSymbolAddress(&ptr, hmpc_noalloc_scratch);
            if (e != cudaSuccess)
            {
                return hmpc_gb300::detail::cuda_fail(e, "cudaGetSymbolAddress of the encryption scratch");
            }
            scratch_address[device] = static_cast<uint32_t*>(ptr);
        }
        *out = scratch_address[device];
        return HMPC_OK;
    }
}

extern "C" int hmpc_lhe_enc_noalloc(hmpc_context* ctx, hmpc_modulus* q, hmpc_modulus* p, uint64_t n, uint64_t batch,
                                    const uint32_t* key_a, const uint32_t* key_b, const uint32_t* plaintext,
                                    int plaintext_ntt, uint32_t* c0, uint32_t* c1)
{
    using namespace hmpc_gb300;
    using namespace hmpc_gb300::detail;
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
    // the transforms must not build (and allocate) twiddle tables here
    if (!q->has_tables(n) || (plaintext_ntt && !p->has_tables(n)))
    {
        return fail(HMPC_ERROR_INVALID_ARGUMENT,
                    "twiddle tables for this degree are not built: call hmpc_modulus_prepare(q, n) (and "
                    "hmpc_modulus_prepare(p, n) for NTT-form plaintexts) before the allocation-free encryption");
    }
    // bound the batch before forming n * batch, which could wrap otherwise
    if (batch > noalloc_scratch_words / n)
    {
        return fail(HMPC_ERROR_INVALID_ARGUMENT, "batch too large for the allocation-free encryption");
    }
    const uint64_t elements = n * batch;
    const uint64_t lq = static_cast<uint64_t>(q->c.limbs);
    const uint64_t lp = static_cast<uint64_t>(p->c.limbs);
    if (lq > noalloc_scratch_words / elements)
    {
        return fail(HMPC_ERROR_INVALID_ARGUMENT, "batch too large for the allocation-free encryption");
    }
    const uint64_t poly_words = elements * lq;
    const uint64_t needed = 3 * poly_words + (plaintext_ntt ? elements * lp : 0);
    if (poly_words > noalloc_scratch_words / 3 || needed > noalloc_scratch_words)
    {
        return fail(HMPC_ERROR_INVALID_ARGUMENT,
                    "the allocation-free encryption needs " + std::to_string(needed) +
                        " words of scratch but holds at most " + std::to_string(noalloc_scratch_words) +
                        " (32 MiB): split the batch or use hmpc_lhe_enc");
    }
    uint32_t* scratch = nullptr;
    if (int rc = scratch_on_current_device(ctx->device, &scratch))
    {
        return rc;
    }
    // every scratch word read below is written earlier in the same call, so
    // nothing has to be cleared
    uint32_t* u = scratch;
    uint32_t* v = scratch + poly_words;
    uint32_t* msg = scratch + 2 * poly_words;
    uint32_t* coeff = scratch + 3 * poly_words;
    // the reference's execution order: NTT(u), NTT(v), [INTT_p(x)],
    // NTT_q(msg), c0, NTT(w), c1 (expr/cache.hpp:226-271)
    int rc = run_transform(ctx, q, n, batch, false, producer_cbd, 1, 0, nullptr, u, nullptr, 0, true);
    if (!rc)
    {
        rc = run_transform(ctx, q, n, batch, false, producer_cbd, 20, 0, nullptr, v, nullptr, 0, true);
    }
    const uint32_t* coefficients = plaintext;
    if (!rc && plaintext_ntt)
    {
        rc = run_transform(ctx, p, n, batch, true, producer_tensor, 0, 0, plaintext, coeff, nullptr, 0, true);
        coefficients = coeff;
    }
    if (rc)
    {
        return rc;
    }
    cudaError_t e = q->kt->cast(msg, coefficients, elements, make_cast(q, p), q->h, ctx->stream);
    if (e != cudaSuccess)
    {
        return cuda_fail(e, "launching cast");
    }
    ++ctx->launches;
    if ((rc = run_transform(ctx, q, n, batch, false, producer_tensor, 0, 0, msg, msg, nullptr, 0, true)))
    {
        return rc;
    }
    const host::words pm = host::to_mont(q->c, p->c.q);
    e = q->kt->lhe_combine(c0, key_a, n, u, v, msg, elements, pm.data(), q->h, ctx->stream);
    if (e != cudaSuccess)
    {
        return cuda_fail(e, "launching combine");
    }
    ++ctx->launches;
    if ((rc = run_transform(ctx, q, n, batch, false, producer_cbd, 20, 0, nullptr, v, nullptr, 0, true)))  // w reuses v
    {
        return rc;
    }
    e = q->kt->lhe_combine(c1, key_b, n, u, v, nullptr, elements, pm.data(), q->h, ctx->stream);
    if (e != cudaSuccess)
    {
        return cuda_fail(e, "launching combine");
    }
    ++ctx->launches;
    return HMPC_OK;
}
