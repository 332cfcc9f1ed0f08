// Internal declarations shared by the C-ABI translation units: the opaque
// context and modulus objects and the helpers that launch transforms.
#pragma once

#include <cstdint>
#include <cstring>
#include <map>
#include <mutex>
#include <tuple>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/hmpc_gb300.h"
#include "dispatch.hpp"
#include "host_math.hpp"

namespace hmpc_gb300::detail
{
    int fail(int code, const std::string& message);
    int cuda_fail(cudaError_t e, const char* what);
    void nonce_add(uint32_t nonce[3], uint64_t v);

    struct Tables
    {
        uint32_t* forward = nullptr;
        uint32_t* inverse = nullptr;
        host::words root, inverse_root;
    };

    // one group of the tensor-core transform: stages [s0, s0 + g), element
    // bits below the group `lo`, `blocks` constant matrices of shape.b_bytes
    // each at byte `offset` of the images
    struct TcGroupPlan
    {
        uint32_t s0 = 0, g = 0, lo = 0;
        uint64_t blocks = 0;
        int in_kind = 0, out_kind = 0;
        int layout = 0;  // bit 0: reads digit planes blocked per row, bit 1: writes them
        TcShapeInfo shape;
        size_t offset = 0;
    };

    struct TcTables
    {
        std::vector<TcGroupPlan> groups;
        uint8_t* images = nullptr;     // every group's constants (first group fed by limbs)
        size_t bytes = 0;
        uint8_t* first_cbd = nullptr;  // first group fed by centred binomial samples
        TcShapeInfo cbd_shape;
        uint8_t* first_small = nullptr;  // first group fed by p * sample + lift(plaintext)
        TcShapeInfo small_shape;
        // false: a group's constants exceed the two-operation carry's range and
        // this (modulus, degree, direction) runs on the CUDA cores
        bool fit = true;
        // the largest sum of |digit| over one column of the digit-fed groups' images
        uint32_t column_max = 0;
        // the first six forward stages as one group fed by CBD samples
        // (tc_wide_kernel): constants G6 * R, and G6 * p * R for the p-scaled
        // draws of the encryption (p: the plaintext modulus they were built for)
        uint8_t* wide_cbd = nullptr;
        uint8_t* wide_cbd_p = nullptr;
        std::vector<uint32_t> wide_p;
    };

    // The carry of a group fed by digits takes two operations per digit while
    // every column sum stays within (-2^22 + 2^15, 2^22 - 2^15); with digits
    // |x| <= 128 that holds when each constant column's sum of |digit| is at
    // most this bound (about twice what balanced random digits give)
    constexpr uint32_t tc_byte_carry_column_bound = 32512;
    constexpr uint32_t tc_default_spin_limit = 1u << 20;

    // first group of a forward transform fed by x = p * CBD(V) + lift(m):
    // plaintext residues m mod p (nullptr: none) and the plaintext modulus
    struct TcSmallInput
    {
        const uint32_t* msg = nullptr;
        const hmpc_modulus* p = nullptr;
    };
}

#define HMPC_CUDA(call, what)                                                                                         \
    do                                                                                                                \
    {                                                                                                                 \
        cudaError_t hmpc_e_ = (call);                                                                                 \
        if (hmpc_e_ != cudaSuccess)                                                                                   \
        {                                                                                                             \
            return ::hmpc_gb300::detail::cuda_fail(hmpc_e_, what);                                                    \
        }                                                                                                             \
    } while (0)

struct hmpc_context
{
    int device = 0;
    cudaStream_t stream = nullptr;
    uint32_t key[8] = {};
    uint32_t nonce[3] = {};
    uint32_t* workspace = nullptr;
    uint64_t workspace_words = 0;
    uint64_t launches = 0;  // kernels launched through this context
    std::vector<hmpc_modulus*> moduli;
    // tensor-core transforms: two digit buffers (separate from `workspace`,
    // which callers of a transform may hold), the bounded-wait error word
    // and the SM count that sizes the persistent grid
    uint32_t* tc_workspace = nullptr;
    uint64_t tc_workspace_words = 0;
    uint32_t* tc_error = nullptr;
    int sm_count = 0;
    // column bound the tensor-core engine accepts for constants built through
    // this context (at most tc_byte_carry_column_bound; lowered only by tests
    // of the refusal)
    uint32_t tc_column_bound = hmpc_gb300::detail::tc_byte_carry_column_bound;
    // polls of an mbarrier before a tensor-core group kernel gives up (each
    // poll a try_wait that itself suspends for a bounded time), and the test
    // hook that makes one such wait run out (hmpc_context_set_test_wait)
    uint32_t tc_spin_limit = hmpc_gb300::detail::tc_default_spin_limit;
    uint32_t tc_test_stall = 0;
    // a second stream for independent work of one call (fork / join events)
    cudaStream_t aux_stream = nullptr;
    cudaEvent_t fork_event = nullptr;
    cudaEvent_t join_event = nullptr;

    bool aux()
    {
        if (!aux_stream &&
            (cudaStreamCreateWithFlags(&aux_stream, cudaStreamNonBlocking) != cudaSuccess ||
             cudaEventCreateWithFlags(&fork_event, cudaEventDisableTiming) != cudaSuccess ||
             cudaEventCreateWithFlags(&join_event, cudaEventDisableTiming) != cudaSuccess))
        {
            return false;
        }
        return true;
    }

    // memory lent for the tensor-core digit buffers of the next calls instead
    // of the context's own (a serving lane's share of its server's pool, so
    // admission by memory counts it); nullptr: none
    uint32_t* tc_lent = nullptr;
    uint64_t tc_lent_words = 0;

    uint32_t* tc_scratch(uint64_t words)
    {
        if (tc_lent && words <= tc_lent_words)
        {
            return tc_lent;
        }
        if (words > tc_workspace_words)
        {
            if (tc_workspace)
            {
                cudaStreamSynchronize(stream);
                cudaFree(tc_workspace);
                tc_workspace = nullptr;
                tc_workspace_words = 0;
            }
            if (cudaMalloc(&tc_workspace, words * sizeof(uint32_t)) != cudaSuccess)
            {
                return nullptr;
            }
            tc_workspace_words = words;
        }
        return tc_workspace;
    }

    uint32_t* scratch(uint64_t words)
    {
        if (words > workspace_words)
        {
            if (workspace)
            {
                cudaStreamSynchronize(stream);
                cudaFree(workspace);
                workspace = nullptr;
                workspace_words = 0;
            }
            if (cudaMalloc(&workspace, words * sizeof(uint32_t)) != cudaSuccess)
            {
                return nullptr;
            }
            workspace_words = words;
        }
        return workspace;
    }

    hmpc_gb300::RngKey rng() const
    {
        hmpc_gb300::RngKey k{};
        std::memcpy(k.key, key, sizeof key);
        std::memcpy(k.nonce, nonce, sizeof nonce);
        return k;
    }
};

struct hmpc_modulus
{
    hmpc_context* ctx = nullptr;
    hmpc_gb300::host::ModulusConstants c;
    hmpc_gb300::HostModulus h;
    const hmpc_gb300::KernelTable* kt = nullptr;
    uint32_t* small_table = nullptr;  // Montgomery forms of 0..64, element-major
    std::map<uint64_t, hmpc_gb300::detail::Tables> tables;
    // tensor-core transform constants per (log2 N, inverse, splits of the contiguous group)
    std::map<std::tuple<int, int, int>, hmpc_gb300::detail::TcTables> tc_tables;

    ~hmpc_modulus()
    {
        cudaFree(small_table);
        for (auto& kv : tables)
        {
            cudaFree(kv.second.forward);
            cudaFree(kv.second.inverse);
        }
        for (auto& kv : tc_tables)
        {
            cudaFree(kv.second.images);
            cudaFree(kv.second.first_cbd);
            cudaFree(kv.second.first_small);
            cudaFree(kv.second.wide_cbd);
            cudaFree(kv.second.wide_cbd_p);
        }
    }

    // tile shape per (log2 N, inverse, batch): register radix bits, tile
    // bits, column bits -- set by hmpc_modulus_tune / hmpc_modulus_set_plan.
    // Radix bits 0 selects the tensor-core engine; its local_bits is the output
    // split (1 or 2; 0 = 1) of the group whose rows are contiguous.
    struct TileChoice
    {
        int radix_bits = 3;
        int local_bits = 0;
        int col_bits = 4;
    };
    std::map<std::tuple<int, int, uint64_t>, TileChoice> tile_choices;
    std::mutex tables_mutex;  // the serving thread looks tables up while clients register new degrees

    // whether the twiddle tables of degree n exist (no allocation)
    bool has_tables(uint64_t n)
    {
        std::lock_guard<std::mutex> lock(tables_mutex);
        return tables.find(n) != tables.end();
    }

    int prepare(uint64_t n, hmpc_gb300::detail::Tables** out)
    {
        std::lock_guard<std::mutex> lock(tables_mutex);
        auto it = tables.find(n);
        if (it == tables.end())
        {
            hmpc_gb300::detail::Tables t;
            std::vector<uint32_t> fwd, inv;
            std::string error;
            if (!hmpc_gb300::host::twiddle_table(c, n, false, fwd, t.root, error) ||
                !hmpc_gb300::host::twiddle_table(c, n, true, inv, t.inverse_root, error))
            {
                return hmpc_gb300::detail::fail(HMPC_ERROR_NO_ROOT, error);
            }
            const size_t bytes = fwd.size() * sizeof(uint32_t);
            HMPC_CUDA(cudaSetDevice(ctx->device), "cudaSetDevice");
            HMPC_CUDA(cudaMalloc(&t.forward, bytes), "allocating twiddles");
            if (cudaMalloc(&t.inverse, bytes) != cudaSuccess)
            {
                cudaFree(t.forward);
                return hmpc_gb300::detail::fail(HMPC_ERROR_OUT_OF_MEMORY, "allocating twiddles");
            }
            HMPC_CUDA(cudaMemcpy(t.forward, fwd.data(), bytes, cudaMemcpyHostToDevice), "uploading twiddles");
            HMPC_CUDA(cudaMemcpy(t.inverse, inv.data(), bytes, cudaMemcpyHostToDevice), "uploading twiddles");
            it = tables.emplace(n, t).first;
        }
        if (out)
        {
            *out = &it->second;
        }
        return HMPC_OK;
    }
};

namespace hmpc_gb300::detail
{
    int check_degree(uint64_t n);
    int enter(hmpc_context* ctx);
    // cuda_cores_only: ignore a tensor-core plan (callers that must not allocate)
    int run_transform(hmpc_context* ctx, hmpc_modulus* mod, uint64_t n, uint64_t batch, bool inverse, int kind,
                      uint32_t vx2, uint32_t security, const uint32_t* src, uint32_t* out,
                      const uint32_t* poly_rng = nullptr, uint32_t rng_slot = 0, bool cuda_cores_only = false);
    int run_plain(hmpc_context* ctx, hmpc_modulus* mod, uint64_t n, uint64_t batch, bool inverse, int kind,
                  uint32_t vx2, uint32_t security, const uint32_t* src, uint32_t* out);
    CastParams make_cast(const hmpc_modulus* dst, const hmpc_modulus* src);
    // tensor-core engine: whether the modulus qualifies (2 to 8 limbs, q
    // below 0.996 * 2^(32L), top limb at least 32) and whether a call does
    // (forward from a tensor or CBD(V) samples, or inverse; at least 16
    // coefficients; no per-polynomial RNG)
    bool tc_supported(const hmpc_modulus* mod);
    bool tc_applicable(const hmpc_modulus* mod, int log_n, int kind, const uint32_t* poly_rng);
    // splits: output split of the group whose rows are contiguous (1 or 2)
    int run_tc_transform(hmpc_context* ctx, hmpc_modulus* mod, uint64_t n, uint64_t batch, bool inverse, int kind,
                         uint32_t vx2, const uint32_t* src, uint32_t* out, int splits,
                         const TcSmallInput* small = nullptr);
    // the tensor-core plan of (n, batch, forward) if one is set for the modulus: splits, else 0
    int tc_plan_splits(hmpc_modulus* mod, uint64_t n, uint64_t batch);
    // Forward transforms of `count` batches fed by CBD(V) samples (optionally
    // as p * sample + lift(m)) that share every constant past their first
    // group: one first-group launch per part into its slice of one digit
    // buffer, then the remaining groups once over count * batch polynomials.
    // Part j draws with the context nonce advanced by j * n * batch; out holds
    // the parts' results side by side (plane stride count * n * batch).
    struct TcStackPart
    {
        uint32_t vx2 = 0;
        const TcSmallInput* small = nullptr;  // nullptr: plain CBD(V) input
    };
    int run_tc_stacked(hmpc_context* ctx, hmpc_modulus* mod, uint64_t n, uint64_t batch, const TcStackPart* parts,
                       int count, uint32_t* out, int splits);
    int tc_cost(hmpc_modulus* mod, uint64_t n, uint64_t batch, bool inverse, int kind, int splits, hmpc_tc_cost* out);
    // Polynomials of one degree n in buffers of their own (the batched
    // transform's buckets).  tc_prepare_polys builds the constants of (n,
    // direction, splits) and the launch state outside any stream capture and
    // gives the digit words per element the transform needs in `digits`;
    // run_tc_polys launches the groups on `stream` (capturable): the first
    // group reads in_polys[i], the last writes out_polys[i] (device pointer
    // tables of `count` entries, buffers 16-byte aligned).
    int tc_prepare_polys(hmpc_context* ctx, hmpc_modulus* mod, uint64_t n, bool inverse, int splits,
                         uint64_t* digit_words_per_element);
    int run_tc_polys(hmpc_context* ctx, hmpc_modulus* mod, uint64_t n, uint64_t count, bool inverse, int splits,
                     const uint32_t* const* in_polys, uint32_t* const* out_polys, uint32_t* digits,
                     cudaStream_t stream);
    // builds (once) the constants of the transform (n, direction, splits) and
    // reports their largest column sum of |digit|
    int tc_column_max(hmpc_context* ctx, hmpc_modulus* mod, uint64_t n, bool inverse, int splits, uint32_t* out);
}
