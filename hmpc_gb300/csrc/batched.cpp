// Batched transforms of polynomials of uneven degree: one persistent kernel
// launch per batch, replayed from a captured CUDA graph, with the tile shape
// (register radix, stages per shared-memory pass, coalescing columns) chosen
// by timing candidates on the device.
#include <algorithm>
#include <cstring>
#include <numeric>
#include <string>
#include <vector>

#include "internal.hpp"
#include "plan.hpp"

using namespace hmpc_gb300;
using namespace hmpc_gb300::detail;

struct hmpc_ntt_batch
{
    hmpc_context* ctx = nullptr;
    hmpc_modulus* mod = nullptr;
    bool inverse = false;
    std::vector<uint64_t> degrees;

    // chosen configuration
    int radix_bits = 3;
    int local_bits = 0;
    int col_bits = 4;
    float tuned_ms = 0.f;

    // plan
    std::vector<NttPassParams> params;        // host copy (pointers rebound per run)
    std::vector<uint32_t> param_poly;         // params index -> polynomial
    std::vector<uint32_t> param_pass;         // params index -> pass
    uint32_t items = 0;
    size_t smem = 0;
    unsigned grid = 0;
    std::vector<uint32_t> item_wait_host, item_signal_host;
    // polls of a wait before it gives up, and the test hook's withheld item
    // (1-based, 0: none; hmpc_ntt_batch_set_test_wait)
    uint32_t spin_limit = 1u << 24;  // ~1 s of 64 ns polls
    uint32_t withheld = 0;

    // device state
    NttPassParams* d_params = nullptr;
    uint32_t* d_items = nullptr;               // 5 arrays of `items` words
    uint32_t* d_counters = nullptr;            // one per polynomial + control block
    NttPassParams* h_params = nullptr;         // pinned staging
    cudaStream_t stream = nullptr;
    cudaGraphExec_t exec = nullptr;
    cudaEvent_t start = nullptr, finish = nullptr;
    std::vector<const uint32_t*> bound_in;
    std::vector<uint32_t*> bound_out;

    // tensor-core engine (radix_bits 0): the polynomials bucketed by degree,
    // each bucket one transform whose first group reads and last group writes
    // the polynomials' own buffers through device pointer tables
    struct Bucket
    {
        uint64_t n = 0;
        std::vector<uint32_t> polys;
        size_t table = 0;  // offset of its in-pointers in the tables (out-pointers follow)
        size_t digits = 0; // offset of its digit buffers
    };
    // the buckets run side by side in the graph (one stream each, forked
    // from and joined to the batch stream), each with digit buffers of its own
    std::vector<cudaStream_t> side;
    std::vector<cudaEvent_t> joins;
    cudaEvent_t fork = nullptr;
    bool tc = false;
    std::vector<Bucket> buckets;
    void** d_tables = nullptr;  // device pointer tables
    void** h_tables = nullptr;  // pinned staging
    size_t table_entries = 0;
    uint32_t* d_digits = nullptr;

    void release_plan()
    {
        if (exec)
        {
            cudaGraphExecDestroy(exec);
            exec = nullptr;
        }
        cudaFree(d_params);
        cudaFree(d_items);
        cudaFree(d_counters);
        cudaFreeHost(h_params);
        cudaFree(d_tables);
        cudaFreeHost(h_tables);
        cudaFree(d_digits);
        d_params = nullptr;
        d_items = nullptr;
        d_counters = nullptr;
        h_params = nullptr;
        d_tables = nullptr;
        h_tables = nullptr;
        d_digits = nullptr;
        table_entries = 0;
        tc = false;
        buckets.clear();
        bound_in.clear();
        bound_out.clear();
    }

    ~hmpc_ntt_batch()
    {
        if (stream)
        {
            cudaStreamSynchronize(stream);
        }
        release_plan();
        for (cudaStream_t st : side)
        {
            cudaStreamSynchronize(st);
            cudaStreamDestroy(st);
        }
        for (cudaEvent_t ev : joins)
        {
            cudaEventDestroy(ev);
        }
        if (fork)
        {
            cudaEventDestroy(fork);
        }
        if (start)
        {
            cudaEventDestroy(start);
        }
        if (finish)
        {
            cudaEventDestroy(finish);
        }
        if (stream)
        {
            cudaStreamDestroy(stream);
        }
    }

    BatchedControl* control() const
    {
        return reinterpret_cast<BatchedControl*>(d_counters + degrees.size());
    }

    // whether the tensor-core engine covers every polynomial of the batch
    bool tc_covers() const
    {
        if (!tc_supported(mod))
        {
            return false;
        }
        for (uint64_t n : degrees)
        {
            if (n < 16)
            {
                return false;
            }
        }
        return true;
    }

    // The tensor-core configuration: buckets by degree (largest first), the
    // constants and launch state of each degree built now, then one graph of
    // every bucket's group launches on the batch stream.
    int build_tc(int splits)
    {
        release_plan();
        tc = true;
        radix_bits = 0;
        local_bits = splits;
        col_bits = 0;
        std::vector<uint64_t> sizes(degrees.begin(), degrees.end());
        std::sort(sizes.begin(), sizes.end(), std::greater<uint64_t>());
        sizes.erase(std::unique(sizes.begin(), sizes.end()), sizes.end());
        uint64_t digit_words = 0;
        for (uint64_t n : sizes)
        {
            Bucket bk;
            bk.n = n;
            for (size_t i = 0; i < degrees.size(); ++i)
            {
                if (degrees[i] == n)
                {
                    bk.polys.push_back(static_cast<uint32_t>(i));
                }
            }
            bk.table = table_entries;
            table_entries += 2 * bk.polys.size();
            uint64_t per_element = 0;
            if (int rc = tc_prepare_polys(ctx, mod, n, inverse, splits, &per_element))
            {
                return rc;
            }
            bk.digits = digit_words;
            digit_words += (per_element * n * bk.polys.size() + 63) & ~uint64_t{63};
            buckets.push_back(std::move(bk));
        }
        while (side.size() < buckets.size())
        {
            cudaStream_t st = nullptr;
            cudaEvent_t ev = nullptr;
            HMPC_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking), "creating a bucket stream");
            side.push_back(st);
            HMPC_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming), "creating a bucket event");
            joins.push_back(ev);
        }
        if (!fork)
        {
            HMPC_CUDA(cudaEventCreateWithFlags(&fork, cudaEventDisableTiming), "creating the fork event");
        }
        HMPC_CUDA(cudaMalloc(&d_tables, table_entries * sizeof(void*)), "allocating pointer tables");
        HMPC_CUDA(cudaMallocHost(&h_tables, table_entries * sizeof(void*)), "allocating pointer tables");
        std::memset(h_tables, 0, table_entries * sizeof(void*));
        if (digit_words)
        {
            HMPC_CUDA(cudaMalloc(&d_digits, digit_words * sizeof(uint32_t)), "allocating digit buffers");
        }
        return capture_tc();
    }

    int capture_tc()
    {
        if (exec)
        {
            cudaGraphExecDestroy(exec);
            exec = nullptr;
        }
        // the captured launches are counted per replay, not here
        const uint64_t launches_before = ctx->launches;
        cudaGraph_t graph = nullptr;
        HMPC_CUDA(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal), "capturing batch graph");
        int rc = HMPC_OK;
        cudaError_t ce = cudaEventRecord(fork, stream);
        for (size_t b = 0; b < buckets.size() && !rc && ce == cudaSuccess; ++b)
        {
            const Bucket& bk = buckets[b];
            ce = cudaStreamWaitEvent(side[b], fork, 0);
            if (ce != cudaSuccess)
            {
                break;
            }
            auto** table = d_tables + bk.table;
            rc = run_tc_polys(ctx, mod, bk.n, bk.polys.size(), inverse, local_bits,
                              reinterpret_cast<const uint32_t* const*>(table),
                              reinterpret_cast<uint32_t* const*>(table + bk.polys.size()),
                              d_digits ? d_digits + bk.digits : nullptr, side[b]);
            if (!rc)
            {
                ce = cudaEventRecord(joins[b], side[b]);
            }
            if (!rc && ce == cudaSuccess)
            {
                ce = cudaStreamWaitEvent(stream, joins[b], 0);
            }
        }
        if (!rc && ce != cudaSuccess)
        {
            rc = cuda_fail(ce, "capturing batch graph");
        }
        items = static_cast<uint32_t>(ctx->launches - launches_before);
        ctx->launches = launches_before;
        cudaError_t e = cudaStreamEndCapture(stream, &graph);
        if (rc || e != cudaSuccess)
        {
            if (graph)
            {
                cudaGraphDestroy(graph);
            }
            return rc ? rc : cuda_fail(e, "capturing batch graph");
        }
        e = cudaGraphInstantiate(&exec, graph, 0);
        cudaGraphDestroy(graph);
        if (e != cudaSuccess)
        {
            return cuda_fail(e, "instantiating batch graph");
        }
        return HMPC_OK;
    }

    // Build the work list and device arrays for one configuration.
    int build(int R, int b, int c_pref)
    {
        release_plan();
        radix_bits = R;
        local_bits = b;
        col_bits = c_pref;
        const int L = mod->c.limbs;
        PlanOptions o;
        o.max_local_bits = b;
        o.col_bits = c_pref;
        o.spread_small_batches = false;
        params.clear();
        param_poly.clear();
        param_pass.clear();
        std::vector<std::vector<PassPlan>> plans(degrees.size());
        size_t max_passes = 0;
        smem = 0;
        for (size_t i = 0; i < degrees.size(); ++i)
        {
            Tables* t = nullptr;
            if (int rc = mod->prepare(degrees[i], &t))
            {
                return rc;
            }
            plans[i] = plan_transform(L, __builtin_ctzll(degrees[i]), 1, inverse, R, o);
            max_passes = std::max(max_passes, plans[i].size());
            for (const PassPlan& pp : plans[i])
            {
                smem = std::max(smem, pp.smem);
            }
        }
        if (smem > 200 * 1024)
        {
            return fail(HMPC_ERROR_UNSUPPORTED, "tile configuration exceeds shared memory");
        }
        // params index of (poly, pass); items: every pass-0 item first, larger
        // polynomials first, then pass 1, ...
        std::vector<std::vector<uint32_t>> index(degrees.size());
        for (size_t i = 0; i < degrees.size(); ++i)
        {
            Tables* t = nullptr;
            mod->prepare(degrees[i], &t);
            for (size_t k = 0; k < plans[i].size(); ++k)
            {
                NttPassParams p = plans[i][k].params;
                p.twiddles = inverse ? t->inverse : t->forward;
                p.small_table = mod->small_table;
                p.elements = degrees[i];
                p.out = nullptr;
                p.src = nullptr;
                index[i].push_back(static_cast<uint32_t>(params.size()));
                params.push_back(p);
                param_poly.push_back(static_cast<uint32_t>(i));
                param_pass.push_back(static_cast<uint32_t>(k));
            }
        }
        std::vector<uint32_t> order(degrees.size());
        std::iota(order.begin(), order.end(), 0u);
        std::stable_sort(order.begin(), order.end(), [&](uint32_t a, uint32_t b2) { return degrees[a] > degrees[b2]; });
        std::vector<uint32_t> item_param, item_tile, item_wait, item_poly, item_signal;
        for (size_t k = 0; k < max_passes; ++k)
        {
            for (uint32_t i : order)
            {
                if (k >= plans[i].size())
                {
                    continue;
                }
                uint32_t before = 0;
                for (size_t j = 0; j < k; ++j)
                {
                    before += plans[i][j].grid;
                }
                for (unsigned g = 0; g < plans[i][k].grid; ++g)
                {
                    item_param.push_back(index[i][k]);
                    item_tile.push_back(g);
                    item_wait.push_back(before);
                    item_poly.push_back(i);
                    item_signal.push_back(k + 1 < plans[i].size() ? 1u : 0u);
                }
            }
        }
        items = static_cast<uint32_t>(item_param.size());
        item_wait_host = item_wait;
        item_signal_host = item_signal;
        withheld = 0;
        const size_t pbytes = params.size() * sizeof(NttPassParams);
        HMPC_CUDA(cudaMalloc(&d_params, pbytes), "allocating batch parameters");
        HMPC_CUDA(cudaMallocHost(&h_params, pbytes), "allocating batch parameters");
        std::memcpy(h_params, params.data(), pbytes);
        HMPC_CUDA(cudaMalloc(&d_items, 5ull * items * sizeof(uint32_t)), "allocating work list");
        HMPC_CUDA(cudaMalloc(&d_counters, (degrees.size() + 4) * sizeof(uint32_t)), "allocating counters");
        std::vector<uint32_t> packed;
        for (auto* v : {&item_param, &item_tile, &item_wait, &item_poly, &item_signal})
        {
            packed.insert(packed.end(), v->begin(), v->end());
        }
        HMPC_CUDA(cudaMemcpy(d_items, packed.data(), packed.size() * sizeof(uint32_t), cudaMemcpyHostToDevice),
                  "uploading work list");
        int sms = 0;
        HMPC_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device), "querying SMs");
        const int per_sm = std::max(1, mod->kt->ntt_batched_blocks_per_sm(R, smem));
        grid = static_cast<unsigned>(std::min<uint64_t>(items, static_cast<uint64_t>(sms) * per_sm));
        return capture();
    }

    // graph: reset counters and control, then the persistent kernel
    int capture()
    {
        if (exec)
        {
            cudaGraphExecDestroy(exec);
            exec = nullptr;
        }
        BatchedParams bp{};
        bp.params = d_params;
        bp.item_param = d_items;
        bp.item_tile = d_items + items;
        bp.item_wait = d_items + 2ull * items;
        bp.item_poly = d_items + 3ull * items;
        bp.item_signal = d_items + 4ull * items;
        bp.counters = d_counters;
        bp.control = control();
        bp.items = items;
        bp.spin_limit = spin_limit;
        cudaGraph_t graph = nullptr;
        HMPC_CUDA(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal), "capturing batch graph");
        cudaError_t e = cudaMemsetAsync(d_counters, 0, (degrees.size() + 4) * sizeof(uint32_t), stream);
        if (e == cudaSuccess)
        {
            e = mod->kt->ntt_batched(bp, radix_bits, mod->h, grid, smem, stream);
        }
        cudaError_t e2 = cudaStreamEndCapture(stream, &graph);
        if (e != cudaSuccess || e2 != cudaSuccess)
        {
            if (graph)
            {
                cudaGraphDestroy(graph);
            }
            return cuda_fail(e != cudaSuccess ? e : e2, "capturing batch graph");
        }
        e = cudaGraphInstantiate(&exec, graph, 0);
        cudaGraphDestroy(graph);
        if (e != cudaSuccess)
        {
            return cuda_fail(e, "instantiating batch graph");
        }
        return HMPC_OK;
    }

    // the test hook: item `item` (1-based, 0: none) waits for one signal more
    // than its polynomial's earlier passes give, so its wait runs out after
    // `polls` polls (0: the default limit)
    int set_test_wait(uint32_t polls, uint32_t item)
    {
        if (tc)
        {
            return fail(HMPC_ERROR_UNSUPPORTED, "the tensor-core batch's waits follow hmpc_context_set_test_wait");
        }
        if (item)
        {
            const uint32_t k = item - 1;
            if (k >= items || item_signal_host[k] != 0 || item_wait_host[k] == 0)
            {
                return fail(HMPC_ERROR_INVALID_ARGUMENT,
                            "the withheld item must be a work item of a polynomial's last pass after its first");
            }
        }
        HMPC_CUDA(cudaStreamSynchronize(stream), "waiting for the batch");
        auto put = [&](uint32_t k, uint32_t value) {
            return cudaMemcpy(d_items + 2ull * items + k, &value, sizeof value, cudaMemcpyHostToDevice);
        };
        if (withheld)
        {
            HMPC_CUDA(put(withheld - 1, item_wait_host[withheld - 1]), "restoring the work list");
            withheld = 0;
        }
        if (item)
        {
            HMPC_CUDA(put(item - 1, item_wait_host[item - 1] + 1u), "withholding a signal");
            withheld = item;
        }
        spin_limit = polls ? polls : (1u << 24);
        return capture();
    }

    int bind(const uint32_t* const* in, uint32_t* const* out)
    {
        bool same = bound_in.size() == degrees.size();
        for (size_t i = 0; same && i < degrees.size(); ++i)
        {
            same = bound_in[i] == in[i] && bound_out[i] == out[i];
        }
        if (same)
        {
            return HMPC_OK;
        }
        // the staging buffer may still feed the previous copy
        HMPC_CUDA(cudaStreamSynchronize(stream), "waiting for the previous batch");
        if (tc)
        {
            for (size_t i = 0; i < degrees.size(); ++i)
            {
                if ((reinterpret_cast<uintptr_t>(in[i]) | reinterpret_cast<uintptr_t>(out[i])) & 15u)
                {
                    return fail(HMPC_ERROR_INVALID_ARGUMENT,
                                "the tensor-core batch needs 16-byte aligned polynomial buffers");
                }
            }
            for (const Bucket& bk : buckets)
            {
                for (size_t k = 0; k < bk.polys.size(); ++k)
                {
                    h_tables[bk.table + k] = const_cast<uint32_t*>(in[bk.polys[k]]);
                    h_tables[bk.table + bk.polys.size() + k] = out[bk.polys[k]];
                }
            }
            HMPC_CUDA(cudaMemcpyAsync(d_tables, h_tables, table_entries * sizeof(void*), cudaMemcpyHostToDevice,
                                      stream),
                      "uploading batch pointers");
            bound_in.assign(in, in + degrees.size());
            bound_out.assign(out, out + degrees.size());
            return HMPC_OK;
        }
        for (size_t k = 0; k < params.size(); ++k)
        {
            const uint32_t i = param_poly[k];
            h_params[k].out = out[i];
            h_params[k].src = param_pass[k] == 0 ? in[i] : nullptr;
        }
        HMPC_CUDA(cudaMemcpyAsync(d_params, h_params, params.size() * sizeof(NttPassParams), cudaMemcpyHostToDevice,
                                  stream),
                  "uploading batch pointers");
        bound_in.assign(in, in + degrees.size());
        bound_out.assign(out, out + degrees.size());
        return HMPC_OK;
    }

    int launch(const uint32_t* const* in, uint32_t* const* out)
    {
        HMPC_CUDA(cudaEventRecord(start, ctx->stream), "ordering batch");
        HMPC_CUDA(cudaStreamWaitEvent(stream, start, 0), "ordering batch");
        if (int rc = bind(in, out))
        {
            return rc;
        }
        HMPC_CUDA(cudaGraphLaunch(exec, stream), "launching batch graph");
        HMPC_CUDA(cudaEventRecord(finish, stream), "ordering batch");
        HMPC_CUDA(cudaStreamWaitEvent(ctx->stream, finish, 0), "ordering batch");
        ctx->launches += tc ? items : 1;
        return HMPC_OK;
    }
};

namespace
{
    // time one configuration on scratch buffers (the transform's cost does
    // not depend on the values)
    float time_config(hmpc_ntt_batch* b, const std::vector<const uint32_t*>& in, const std::vector<uint32_t*>& out)
    {
        cudaEvent_t t0, t1;
        cudaEventCreate(&t0);
        cudaEventCreate(&t1);
        float best = 1e30f;
        for (int rep = 0; rep < 5; ++rep)
        {
            cudaEventRecord(t0, b->ctx->stream);
            if (b->launch(in.data(), out.data()) != HMPC_OK)
            {
                best = 1e30f;
                break;
            }
            cudaEventRecord(t1, b->ctx->stream);
            cudaEventSynchronize(t1);
            float ms = 0.f;
            cudaEventElapsedTime(&ms, t0, t1);
            if (rep >= 1)
            {
                best = std::min(best, ms);
            }
        }
        cudaEventDestroy(t0);
        cudaEventDestroy(t1);
        return best;
    }
}

extern "C" {

int hmpc_ntt_batch_create(hmpc_context* ctx, hmpc_modulus* mod, uint64_t count, const uint64_t* degrees, int inverse,
                          int autotune, hmpc_ntt_batch** out)
{
    if (int rc = enter(ctx))
    {
        return rc;
    }
    if (!mod || !degrees || !out || count == 0)
    {
        return fail(HMPC_ERROR_INVALID_ARGUMENT, "empty batch or null argument");
    }
    auto* b = new hmpc_ntt_batch;
    b->ctx = ctx;
    b->mod = mod;
    b->inverse = inverse != 0;
    b->degrees.assign(degrees, degrees + count);
    for (uint64_t n : b->degrees)
    {
        if (int rc = check_degree(n))
        {
            delete b;
            return rc;
        }
        if (__builtin_ctzll(n) < 3)
        {
            delete b;
            return fail(HMPC_ERROR_UNSUPPORTED, "batched transforms need degree >= 8");
        }
    }
    cudaError_t e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess)
    {
        e = cudaEventCreateWithFlags(&b->start, cudaEventDisableTiming);
    }
    if (e == cudaSuccess)
    {
        e = cudaEventCreateWithFlags(&b->finish, cudaEventDisableTiming);
    }
    if (e != cudaSuccess)
    {
        delete b;
        return cuda_fail(e, "creating the batch stream");
    }
    const int L = mod->c.limbs;
    PlanOptions def;
    const int b_default = local_bits_for(L, def);
    int best_r = 3, best_b = b_default, best_c = 4;
    if (autotune == HMPC_BATCH_TENSOR_CORES)
    {
        if (!b->tc_covers())
        {
            delete b;
            return fail(HMPC_ERROR_UNSUPPORTED, "the tensor-core engine does not cover this modulus or a degree below 16");
        }
        best_r = 0;
        best_b = 1;
    }
    else if (autotune)
    {
        // scratch buffers for the trial runs
        std::vector<uint32_t*> bufs;
        std::vector<const uint32_t*> ins;
        bool ok = true;
        for (uint64_t n : b->degrees)
        {
            uint32_t* p = nullptr;
            if (cudaMalloc(&p, n * static_cast<uint64_t>(L) * sizeof(uint32_t)) != cudaSuccess)
            {
                ok = false;
                break;
            }
            cudaMemsetAsync(p, 0, n * static_cast<uint64_t>(L) * sizeof(uint32_t), ctx->stream);
            bufs.push_back(p);
            ins.push_back(p);
        }
        float best = 1e30f;
        if (ok)
        {
            for (int R : {3, 2})
            {
                for (int lb : {b_default - 1, b_default, b_default + 1})
                {
                    for (int c : {3, 4, 5})
                    {
                        if (lb < 8 || static_cast<uint64_t>(L) * 4u * smem_words(1u << lb) > 200 * 1024)
                        {
                            continue;
                        }
                        if (b->build(R, lb, c) != HMPC_OK)
                        {
                            continue;
                        }
                        const float ms = time_config(b, ins, bufs);
                        if (ms < best)
                        {
                            best = ms;
                            best_r = R;
                            best_b = lb;
                            best_c = c;
                        }
                    }
                }
            }
            // the tensor-core engine, one bucket per degree, with either split
            // of the groups whose rows are contiguous elements
            for (int splits : {1, 2})
            {
                if (!b->tc_covers() || b->build_tc(splits) != HMPC_OK)
                {
                    break;
                }
                const float ms = time_config(b, ins, bufs);
                if (ms < best)
                {
                    best = ms;
                    best_r = 0;
                    best_b = splits;
                }
            }
        }
        cudaStreamSynchronize(b->stream);
        for (auto* p : bufs)
        {
            cudaFree(p);
        }
        b->tuned_ms = best < 1e29f ? best : 0.f;
    }
    if (int rc = best_r == 0 ? b->build_tc(best_b) : b->build(best_r, best_b, best_c))
    {
        delete b;
        return rc;
    }
    *out = b;
    return HMPC_OK;
}

int hmpc_ntt_batch_run(hmpc_ntt_batch* batch, const uint32_t* const* in, uint32_t* const* out)
{
    if (!batch || !in || !out)
    {
        return fail(HMPC_ERROR_INVALID_ARGUMENT, "null argument");
    }
    if (int rc = enter(batch->ctx))
    {
        return rc;
    }
    for (size_t i = 0; i < batch->degrees.size(); ++i)
    {
        if (!in[i] || !out[i])
        {
            return fail(HMPC_ERROR_INVALID_ARGUMENT, "null polynomial buffer");
        }
    }
    return batch->launch(in, out);
}

int hmpc_ntt_batch_info(const hmpc_ntt_batch* batch, int* radix_bits, int* local_bits, int* col_bits, uint32_t* items,
                        float* tuned_ms)
{
    if (!batch)
    {
        return fail(HMPC_ERROR_INVALID_ARGUMENT, "null batch");
    }
    if (radix_bits)
    {
        *radix_bits = batch->radix_bits;
    }
    if (local_bits)
    {
        *local_bits = batch->local_bits;
    }
    if (col_bits)
    {
        *col_bits = batch->col_bits;
    }
    if (items)
    {
        *items = batch->items;
    }
    if (tuned_ms)
    {
        *tuned_ms = batch->tuned_ms;
    }
    return HMPC_OK;
}

int hmpc_ntt_batch_status(hmpc_ntt_batch* batch, uint32_t* failed_item)
{
    if (!batch || !failed_item)
    {
        return fail(HMPC_ERROR_INVALID_ARGUMENT, "null argument");
    }
    if (int rc = enter(batch->ctx))
    {
        return rc;
    }
    HMPC_CUDA(cudaStreamSynchronize(batch->stream), "waiting for the batch");
    if (batch->tc)
    {
        // the tensor-core groups report a wait that ran out in the context's error word
        *failed_item = 0;
        hmpc_context* ctx = batch->ctx;
        if (ctx->tc_error)
        {
            uint32_t code = 0;
            HMPC_CUDA(cudaMemcpy(&code, ctx->tc_error, sizeof code, cudaMemcpyDeviceToHost), "reading batch status");
            if (code)
            {
                HMPC_CUDA(cudaMemset(ctx->tc_error, 0, sizeof code), "clearing the error word");
                return fail(HMPC_ERROR_TIMEOUT, "a tensor-core group of the batch gave up a wait; the outputs are "
                                                "incomplete");
            }
        }
        return HMPC_OK;
    }
    BatchedControl control{};
    HMPC_CUDA(cudaMemcpy(&control, batch->control(), sizeof control, cudaMemcpyDeviceToHost), "reading batch status");
    *failed_item = control.error;
    if (control.error || control.done != batch->items)
    {
        return fail(HMPC_ERROR_TIMEOUT, "a batched transform wait ran out; the outputs are incomplete");
    }
    return HMPC_OK;
}

int hmpc_ntt_batch_set_test_wait(hmpc_ntt_batch* batch, uint32_t polls, uint32_t withheld_item)
{
    if (!batch)
    {
        return fail(HMPC_ERROR_INVALID_ARGUMENT, "null batch");
    }
    if (int rc = enter(batch->ctx))
    {
        return rc;
    }
    return batch->set_test_wait(polls, withheld_item);
}

int hmpc_ntt_batch_destroy(hmpc_ntt_batch* batch)
{
    if (batch)
    {
        cudaSetDevice(batch->ctx->device);
        delete batch;
    }
    return HMPC_OK;
}

}  // extern "C"
