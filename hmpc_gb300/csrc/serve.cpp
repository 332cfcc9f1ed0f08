// Serving loop: requests (NTT, BGV encryption, ciphertext x ciphertext) are
// submitted from any host thread and return a ticket; a scheduler thread
// batches compatible pending requests as device lanes (streams) and memory
// free up, so work of requests that arrive while others run overlaps on the
// device (continuous batching).
//
// Admission is by device memory: the server reserves one pool at creation and
// every dispatch takes its scratch from it; a dispatch waits until its
// scratch fits, and a request whose scratch can never fit is rejected.  Keys
// and twiddle tables stay resident.  Every request's result is the result it
// would have alone: transforms and products have no state, and an encryption
// draws its randomness from its own nonce with coefficient indices local to
// the request (per-polynomial RNG descriptors), whatever batch it lands in.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <thread>
#include <tuple>
#include <unordered_map>
#include <vector>

#include "internal.hpp"

using namespace hmpc_gb300;
using namespace hmpc_gb300::detail;

namespace
{
    using clock_type = std::chrono::steady_clock;

    enum state : int
    {
        state_queued = 0,
        state_running = 1,
        state_done = 2,
        state_failed = -2,
    };

    struct Request
    {
        hmpc_request r{};
        uint64_t ticket = 0;
        clock_type::time_point submitted, finished;
        std::atomic<int> st{state_queued};
    };

    struct ResidentKey
    {
        hmpc_modulus* q = nullptr;
        hmpc_modulus* p = nullptr;
        uint64_t n = 0;
        uint32_t* a = nullptr;
        uint32_t* b = nullptr;
    };

    // first-fit allocator over the reserved device pool
    class Pool
    {
    public:
        void reset(uint64_t bytes)
        {
            free_.clear();
            free_[0] = bytes;
            total_ = bytes;
        }
        bool allocate(uint64_t bytes, uint64_t& offset)
        {
            bytes = (bytes + 255) & ~uint64_t{255};
            for (auto it = free_.begin(); it != free_.end(); ++it)
            {
                if (it->second >= bytes)
                {
                    offset = it->first;
                    const uint64_t rest = it->second - bytes;
                    const uint64_t at = it->first + bytes;
                    free_.erase(it);
                    if (rest)
                    {
                        free_[at] = rest;
                    }
                    return true;
                }
            }
            return false;
        }
        void release(uint64_t offset, uint64_t bytes)
        {
            bytes = (bytes + 255) & ~uint64_t{255};
            auto it = free_.emplace(offset, bytes).first;
            auto next = std::next(it);
            if (next != free_.end() && it->first + it->second == next->first)
            {
                it->second += next->second;
                free_.erase(next);
            }
            if (it != free_.begin())
            {
                auto prev = std::prev(it);
                if (prev->first + prev->second == it->first)
                {
                    prev->second += it->second;
                    free_.erase(it);
                }
            }
        }
        uint64_t total() const
        {
            return total_;
        }

    private:
        std::map<uint64_t, uint64_t> free_;
        uint64_t total_ = 0;
    };

    struct Dispatch
    {
        std::vector<Request*> reqs;
        int lane = -1;
        uint64_t offset = 0, bytes = 0;
    };

    using GroupKey = std::tuple<int, const void*, uint64_t, uint32_t>;  // kind, modulus, n, key
}

struct hmpc_server
{
    hmpc_context* ctx = nullptr;
    uint32_t max_batch = 16;
    std::vector<std::unique_ptr<hmpc_context>> lanes;
    std::vector<cudaEvent_t> lane_done;
    std::vector<uint32_t*> lane_desc;        // pinned RNG descriptors per lane
    std::vector<Dispatch> lane_work;
    std::vector<bool> lane_busy;
    uint32_t desc_capacity = 0;              // polynomials per lane descriptor buffer
    uint32_t batch_window_us = 0;            // hold a group that is not full for compatible arrivals
    uint32_t* d_desc = nullptr;              // device descriptors, one region per lane
    uint8_t* pool_base = nullptr;
    Pool pool;
    std::vector<ResidentKey> keys;

    std::mutex mu;
    std::condition_variable cv;
    std::deque<Request*> incoming;
    std::map<GroupKey, std::deque<Request*>> pending;
    std::unordered_map<uint64_t, std::unique_ptr<Request>> requests;
    uint64_t next_ticket = 1;
    std::thread worker;
    std::atomic<bool> stop{false};
    std::atomic<uint64_t> in_system{0};

    // statistics (worker thread; read under mu)
    uint64_t submitted = 0, completed = 0, rejected = 0, failed = 0, dispatches = 0, batched_requests = 0;
    std::vector<double> latencies_us;

    static uint64_t words_of(const hmpc_modulus* m, uint64_t n, uint64_t count)
    {
        return n * count * static_cast<uint64_t>(m->c.limbs);
    }

    // words of tensor-core digit buffers (two buffers of ceil((4L + 2) / 4)
    // words per element) that a forward transform of `polys` polynomials
    // takes when q's plan for that shape is the tensor-core engine, else 0
    static uint64_t tc_words(hmpc_modulus* q, uint64_t n, uint64_t polys)
    {
        if (n < 16 || !tc_applicable(q, __builtin_ctzll(n), producer_tensor, nullptr) ||
            !tc_plan_splits(q, n, polys))
        {
            return 0;
        }
        return 2 * ((4ull * static_cast<uint64_t>(q->c.limbs) + 5) / 4) * n * polys;
    }

    // scratch bytes of a dispatch of the given requests: buffers of its own
    // and, after them, the digit buffers of a tensor-core transform
    uint64_t scratch_bytes(const std::vector<Request*>& rs) const
    {
        const hmpc_request& r0 = rs.front()->r;
        uint64_t polys = 0;
        for (auto* x : rs)
        {
            polys += x->r.count;
        }
        const bool single = rs.size() == 1;
        switch (r0.kind)
        {
        case HMPC_REQUEST_NTT:
            return ((single ? 0 : words_of(r0.q, r0.n, polys)) + tc_words(r0.q, r0.n, polys)) * 4;
        case HMPC_REQUEST_ENCRYPT:
        {
            const ResidentKey& k = keys[r0.key_id];
            return (encrypt_words(k, polys, single) + tc_words(k.q, k.n, polys)) * 4;
        }
        default:
            return 0;
        }
    }

    static uint64_t encrypt_words(const ResidentKey& k, uint64_t polys, bool single)
    {
        uint64_t w = 3 * words_of(k.q, k.n, polys);  // u, v/w, msg
        if (!single)
        {
            w += words_of(k.p, k.n, polys) + 2 * words_of(k.q, k.n, polys);  // plaintext, c0, c1
        }
        return w;
    }

    GroupKey group_of(const hmpc_request& r) const
    {
        return GroupKey{r.kind, r.q, r.n, r.kind == HMPC_REQUEST_ENCRYPT ? r.key_id : 0u};
    }

    // gather / scatter request blocks of a limb-planar batch buffer
    static cudaError_t copy_block(uint32_t* dst, uint64_t dst_pitch_words, const uint32_t* src,
                                  uint64_t src_pitch_words, uint64_t width_words, int limbs, cudaStream_t s)
    {
        return cudaMemcpy2DAsync(dst, dst_pitch_words * 4, src, src_pitch_words * 4, width_words * 4,
                                 static_cast<size_t>(limbs), cudaMemcpyDeviceToDevice, s);
    }

    int issue(Dispatch& d)
    {
        hmpc_context* lane = lanes[static_cast<size_t>(d.lane)].get();
        cudaStream_t s = lane->stream;
        const hmpc_request& r0 = d.reqs.front()->r;
        const bool single = d.reqs.size() == 1;
        uint64_t polys = 0;
        for (auto* x : d.reqs)
        {
            polys += x->r.count;
        }
        uint32_t* scratch = reinterpret_cast<uint32_t*>(pool_base + d.offset);
        // the lane's tensor-core digit buffers come from the dispatch's share
        // of the pool, after its own buffers
        struct Lend
        {
            hmpc_context* ctx;
            ~Lend()
            {
                ctx->tc_lent = nullptr;
                ctx->tc_lent_words = 0;
            }
        } lend{lane};
        if (r0.kind == HMPC_REQUEST_NTT || r0.kind == HMPC_REQUEST_ENCRYPT)
        {
            const bool ntt = r0.kind == HMPC_REQUEST_NTT;
            hmpc_modulus* q = ntt ? r0.q : keys[r0.key_id].q;
            const uint64_t n = ntt ? r0.n : keys[r0.key_id].n;
            const uint64_t own = ntt ? (single ? 0 : words_of(q, n, polys)) : encrypt_words(keys[r0.key_id], polys, single);
            if (const uint64_t tw = tc_words(q, n, polys))
            {
                lane->tc_lent = scratch + own;
                lane->tc_lent_words = tw;
            }
        }
        if (r0.kind == HMPC_REQUEST_NTT)
        {
            hmpc_modulus* q = r0.q;
            const int L = q->c.limbs;
            if (single)
            {
                return run_transform(lane, q, r0.n, r0.count, false, producer_tensor, 0, 0, r0.in0, r0.out0);
            }
            const uint64_t total = r0.n * polys;
            uint64_t at = 0;
            for (auto* x : d.reqs)
            {
                const uint64_t w = x->r.n * x->r.count;
                HMPC_CUDA(copy_block(scratch + at, total, x->r.in0, w, w, L, s), "gathering transform inputs");
                at += w;
            }
            if (int rc = run_transform(lane, q, r0.n, polys, false, producer_tensor, 0, 0, scratch, scratch))
            {
                return rc;
            }
            at = 0;
            for (auto* x : d.reqs)
            {
                const uint64_t w = x->r.n * x->r.count;
                HMPC_CUDA(copy_block(x->r.out0, w, scratch + at, total, w, L, s), "scattering transform outputs");
                at += w;
            }
            return HMPC_OK;
        }
        if (r0.kind == HMPC_REQUEST_CT_MUL)
        {
            for (auto* x : d.reqs)
            {
                const hmpc_request& r = x->r;
                cudaError_t e = r.q->kt->ct_mul(r.out0, r.out1, r.out2, r.in0, r.in1, r.in2, r.in3, r.n * r.count,
                                                r.q->h, s);
                if (e != cudaSuccess)
                {
                    return cuda_fail(e, "launching ciphertext product");
                }
                ++lane->launches;
            }
            return HMPC_OK;
        }
        // encryption: the batch of requests shares the key; polynomial i of
        // the batch draws with its request's nonce and local index
        const ResidentKey& k = keys[r0.key_id];
        const uint64_t n = k.n;
        const int lq = k.q->c.limbs;
        const int lp = k.p->c.limbs;
        const uint64_t total = n * polys;
        const uint64_t qw = total * static_cast<uint64_t>(lq);
        uint32_t* u = scratch;
        uint32_t* v = u + qw;
        uint32_t* msg = v + qw;
        uint32_t* pt = msg + qw;
        uint32_t* c0 = pt + total * static_cast<uint64_t>(lp);
        uint32_t* c1 = c0 + qw;
        uint32_t* host_desc = lane_desc[static_cast<size_t>(d.lane)];
        uint32_t* dev_desc = d_desc + static_cast<uint64_t>(d.lane) * desc_capacity * 5;
        uint64_t poly = 0;
        for (auto* x : d.reqs)
        {
            for (uint64_t j = 0; j < x->r.count; ++j, ++poly)
            {
                uint32_t* desc = host_desc + poly * 5;
                desc[0] = x->r.nonce[0];
                desc[1] = x->r.nonce[1];
                desc[2] = x->r.nonce[2];
                desc[3] = static_cast<uint32_t>(j);
                desc[4] = static_cast<uint32_t>(x->r.count);
            }
        }
        HMPC_CUDA(cudaMemcpyAsync(dev_desc, host_desc, polys * 5 * sizeof(uint32_t), cudaMemcpyHostToDevice, s),
                  "uploading RNG descriptors");
        const uint32_t* plaintext = r0.in0;
        if (!single)
        {
            plaintext = pt;
            uint64_t at = 0;
            for (auto* x : d.reqs)
            {
                const uint64_t w = n * x->r.count;
                HMPC_CUDA(copy_block(pt + at, total, x->r.in0, w, w, lp, s), "gathering plaintexts");
                at += w;
            }
        }
        uint32_t* out0 = single ? r0.out0 : c0;
        uint32_t* out1 = single ? r0.out1 : c1;
        int rc = run_transform(lane, k.q, n, polys, false, producer_cbd, 1, 0, nullptr, u, dev_desc, 0);
        if (!rc)
        {
            rc = run_transform(lane, k.q, n, polys, false, producer_cbd, 20, 0, nullptr, v, dev_desc, 1);
        }
        if (rc)
        {
            return rc;
        }
        cudaError_t e = k.q->kt->cast(msg, plaintext, total, make_cast(k.q, k.p), k.q->h, s);
        if (e != cudaSuccess)
        {
            return cuda_fail(e, "launching cast");
        }
        ++lane->launches;
        if ((rc = run_transform(lane, k.q, n, polys, false, producer_tensor, 0, 0, msg, msg)))
        {
            return rc;
        }
        const host::words pm = host::to_mont(k.q->c, k.p->c.q);
        if ((e = k.q->kt->lhe_combine(out0, k.a, n, u, v, msg, total, pm.data(), k.q->h, s)) != cudaSuccess)
        {
            return cuda_fail(e, "launching combine");
        }
        ++lane->launches;
        if ((rc = run_transform(lane, k.q, n, polys, false, producer_cbd, 20, 0, nullptr, v, dev_desc, 2)))
        {
            return rc;
        }
        if ((e = k.q->kt->lhe_combine(out1, k.b, n, u, v, nullptr, total, pm.data(), k.q->h, s)) != cudaSuccess)
        {
            return cuda_fail(e, "launching combine");
        }
        ++lane->launches;
        if (!single)
        {
            uint64_t at = 0;
            for (auto* x : d.reqs)
            {
                const uint64_t w = n * x->r.count;
                HMPC_CUDA(copy_block(x->r.out0, w, c0 + at, total, w, lq, s), "scattering c0");
                HMPC_CUDA(copy_block(x->r.out1, w, c1 + at, total, w, lq, s), "scattering c1");
                at += w;
            }
        }
        return HMPC_OK;
    }

    void finish(int lane_index, bool ok)
    {
        Dispatch& d = lane_work[static_cast<size_t>(lane_index)];
        const auto now = clock_type::now();
        {
            std::lock_guard<std::mutex> lock(mu);
            for (auto* x : d.reqs)
            {
                x->finished = now;
                x->st.store(ok ? state_done : state_failed);
                if (ok)
                {
                    ++completed;
                    latencies_us.push_back(std::chrono::duration<double, std::micro>(now - x->submitted).count());
                }
                else
                {
                    ++failed;
                }
            }
        }
        in_system.fetch_sub(d.reqs.size());
        if (d.bytes)
        {
            pool.release(d.offset, d.bytes);
        }
        d = Dispatch{};
        lane_busy[static_cast<size_t>(lane_index)] = false;
        cv.notify_all();
    }

    void run()
    {
        cudaSetDevice(ctx->device);
        while (!stop.load())
        {
            bool progress = false;
            {
                std::unique_lock<std::mutex> lock(mu);
                while (!incoming.empty())
                {
                    Request* x = incoming.front();
                    incoming.pop_front();
                    pending[group_of(x->r)].push_back(x);
                    progress = true;
                }
            }
            // completions
            for (size_t i = 0; i < lanes.size(); ++i)
            {
                if (lane_busy[i])
                {
                    const cudaError_t e = cudaEventQuery(lane_done[i]);
                    if (e != cudaErrorNotReady)
                    {
                        finish(static_cast<int>(i), e == cudaSuccess);
                        progress = true;
                    }
                }
            }
            // dispatch: oldest group first, one batch per free lane
            for (;;)
            {
                int lane = -1;
                for (size_t i = 0; i < lanes.size(); ++i)
                {
                    if (!lane_busy[i])
                    {
                        lane = static_cast<int>(i);
                        break;
                    }
                }
                if (lane < 0)
                {
                    break;
                }
                std::deque<Request*>* best = nullptr;
                const auto now = std::chrono::steady_clock::now();
                for (auto& kv : pending)
                {
                    if (kv.second.empty() || (best && kv.second.front()->submitted >= best->front()->submitted))
                    {
                        continue;
                    }
                    // a group that could still grow waits for the window to pass
                    // since its oldest request arrived
                    if (batch_window_us && kv.second.size() < max_batch &&
                        now - kv.second.front()->submitted < std::chrono::microseconds(batch_window_us))
                    {
                        continue;
                    }
                    best = &kv.second;
                }
                if (!best)
                {
                    break;
                }
                Dispatch d;
                d.lane = lane;
                uint64_t polys = 0;
                while (!best->empty() && d.reqs.size() < max_batch &&
                       polys + best->front()->r.count <= desc_capacity)
                {
                    d.reqs.push_back(best->front());
                    const uint64_t need = scratch_bytes(d.reqs);
                    if (need > pool.total())
                    {
                        d.reqs.pop_back();
                        break;
                    }
                    // grow the dispatch's block: give the old one back first
                    if (d.bytes)
                    {
                        pool.release(d.offset, d.bytes);
                    }
                    uint64_t offset = 0;
                    if (need && !pool.allocate(need, offset))
                    {
                        if (d.bytes)
                        {
                            pool.allocate(d.bytes, d.offset);  // the block just released fits again
                        }
                        d.reqs.pop_back();
                        break;
                    }
                    d.offset = offset;
                    d.bytes = need;
                    polys += best->front()->r.count;
                    best->pop_front();
                }
                if (d.reqs.empty())
                {
                    break;  // the oldest group waits for memory
                }
                for (auto* x : d.reqs)
                {
                    x->st.store(state_running);
                }
                lane_work[static_cast<size_t>(lane)] = d;
                lane_busy[static_cast<size_t>(lane)] = true;
                ++dispatches;
                batched_requests += d.reqs.size();
                const int rc = issue(lane_work[static_cast<size_t>(lane)]);
                const cudaError_t e = cudaEventRecord(lane_done[static_cast<size_t>(lane)],
                                                      lanes[static_cast<size_t>(lane)]->stream);
                if (rc != HMPC_OK || e != cudaSuccess)
                {
                    cudaStreamSynchronize(lanes[static_cast<size_t>(lane)]->stream);
                    finish(lane, false);
                }
                progress = true;
            }
            if (!progress)
            {
                std::unique_lock<std::mutex> lock(mu);
                cv.wait_for(lock, std::chrono::microseconds(20), [&] { return !incoming.empty() || stop.load(); });
            }
        }
    }
};

extern "C" {

int hmpc_server_create(hmpc_context* ctx, const hmpc_server_config* config, hmpc_server** out)
{
    if (int rc = enter(ctx))
    {
        return rc;
    }
    if (!config || !out || config->lanes == 0 || config->max_batch == 0)
    {
        return fail(HMPC_ERROR_INVALID_ARGUMENT, "bad server configuration");
    }
    auto srv = std::make_unique<hmpc_server>();
    srv->ctx = ctx;
    srv->max_batch = config->max_batch;
    srv->desc_capacity = config->max_batch_polynomials ? config->max_batch_polynomials : 4096;
    srv->batch_window_us = config->batch_window_us;
    for (uint32_t i = 0; i < config->lanes; ++i)
    {
        auto lane = std::make_unique<hmpc_context>();
        lane->device = ctx->device;
        std::memcpy(lane->key, ctx->key, sizeof lane->key);
        HMPC_CUDA(cudaStreamCreateWithFlags(&lane->stream, cudaStreamNonBlocking), "creating a lane stream");
        cudaEvent_t ev;
        HMPC_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming), "creating a lane event");
        uint32_t* desc = nullptr;
        HMPC_CUDA(cudaMallocHost(&desc, srv->desc_capacity * 5ull * sizeof(uint32_t)), "allocating descriptors");
        srv->lanes.push_back(std::move(lane));
        srv->lane_done.push_back(ev);
        srv->lane_desc.push_back(desc);
    }
    srv->lane_work.resize(config->lanes);
    srv->lane_busy.assign(config->lanes, false);
    HMPC_CUDA(cudaMalloc(&srv->d_desc, srv->desc_capacity * 5ull * config->lanes * sizeof(uint32_t)),
              "allocating descriptors");
    if (config->memory_budget_bytes)
    {
        if (cudaMalloc(&srv->pool_base, config->memory_budget_bytes) != cudaSuccess)
        {
            return fail(HMPC_ERROR_OUT_OF_MEMORY, "reserving the server's memory pool");
        }
    }
    srv->pool.reset(config->memory_budget_bytes);
    hmpc_server* raw = srv.get();
    srv->worker = std::thread([raw] { raw->run(); });
    *out = srv.release();
    return HMPC_OK;
}

int hmpc_server_add_key(hmpc_server* srv, hmpc_modulus* q, hmpc_modulus* p, uint64_t n, const uint32_t* a,
                        const uint32_t* b, uint32_t* key_id)
{
    if (!srv || !q || !p || !a || !b || !key_id)
    {
        return fail(HMPC_ERROR_INVALID_ARGUMENT, "null argument");
    }
    if (int rc = enter(srv->ctx))
    {
        return rc;
    }
    if (int rc = check_degree(n))
    {
        return rc;
    }
    if (int rc = q->prepare(n, nullptr))
    {
        return rc;
    }
    ResidentKey k;
    k.q = q;
    k.p = p;
    k.n = n;
    const uint64_t bytes = n * static_cast<uint64_t>(q->c.limbs) * sizeof(uint32_t);
    HMPC_CUDA(cudaMalloc(&k.a, bytes), "allocating a resident key");
    HMPC_CUDA(cudaMalloc(&k.b, bytes), "allocating a resident key");
    HMPC_CUDA(cudaMemcpy(k.a, a, bytes, cudaMemcpyDeviceToDevice), "copying a resident key");
    HMPC_CUDA(cudaMemcpy(k.b, b, bytes, cudaMemcpyDeviceToDevice), "copying a resident key");
    std::lock_guard<std::mutex> lock(srv->mu);
    *key_id = static_cast<uint32_t>(srv->keys.size());
    srv->keys.push_back(k);
    return HMPC_OK;
}

int hmpc_server_submit(hmpc_server* srv, const hmpc_request* request, uint64_t* ticket)
{
    if (!srv || !request || !ticket)
    {
        return fail(HMPC_ERROR_INVALID_ARGUMENT, "null argument");
    }
    const hmpc_request& r = *request;
    if (r.count == 0 || r.count > srv->desc_capacity)
    {
        return fail(HMPC_ERROR_INVALID_ARGUMENT, "request polynomial count out of range");
    }
    switch (r.kind)
    {
    case HMPC_REQUEST_NTT:
        if (!r.q || !r.in0 || !r.out0)
        {
            return fail(HMPC_ERROR_INVALID_ARGUMENT, "transform request needs q, in0, out0");
        }
        if (int rc = check_degree(r.n))
        {
            return rc;
        }
        if (int rc = r.q->prepare(r.n, nullptr))
        {
            return rc;
        }
        break;
    case HMPC_REQUEST_ENCRYPT:
    {
        std::lock_guard<std::mutex> lock(srv->mu);
        if (r.key_id >= srv->keys.size() || !r.in0 || !r.out0 || !r.out1 || srv->keys[r.key_id].n != r.n)
        {
            return fail(HMPC_ERROR_INVALID_ARGUMENT, "encryption request needs a resident key of its degree");
        }
        break;
    }
    case HMPC_REQUEST_CT_MUL:
        if (!r.q || !r.in0 || !r.in1 || !r.in2 || !r.in3 || !r.out0 || !r.out1 || !r.out2)
        {
            return fail(HMPC_ERROR_INVALID_ARGUMENT, "product request needs two ciphertexts and three outputs");
        }
        break;
    default:
        return fail(HMPC_ERROR_INVALID_ARGUMENT, "unknown request kind");
    }
    auto x = std::make_unique<Request>();
    x->r = r;
    if (r.kind == HMPC_REQUEST_ENCRYPT)
    {
        x->r.q = srv->keys[r.key_id].q;
    }
    x->submitted = clock_type::now();
    {
        std::lock_guard<std::mutex> lock(srv->mu);
        // a request that cannot run even alone is rejected
        std::vector<Request*> alone{x.get()};
        if (srv->scratch_bytes(alone) > srv->pool.total())
        {
            ++srv->rejected;
            return fail(HMPC_ERROR_REJECTED, "request needs more scratch than the server's memory budget");
        }
        x->ticket = srv->next_ticket++;
        *ticket = x->ticket;
        ++srv->submitted;
        srv->incoming.push_back(x.get());
        srv->requests.emplace(x->ticket, std::move(x));
    }
    srv->in_system.fetch_add(1);
    srv->cv.notify_all();
    return HMPC_OK;
}

int hmpc_server_poll(hmpc_server* srv, uint64_t ticket, int* state, double* latency_us)
{
    if (!srv || !state)
    {
        return fail(HMPC_ERROR_INVALID_ARGUMENT, "null argument");
    }
    std::lock_guard<std::mutex> lock(srv->mu);
    auto it = srv->requests.find(ticket);
    if (it == srv->requests.end())
    {
        return fail(HMPC_ERROR_INVALID_ARGUMENT, "unknown ticket");
    }
    *state = it->second->st.load();
    if (latency_us)
    {
        *latency_us = *state == state_done
                          ? std::chrono::duration<double, std::micro>(it->second->finished - it->second->submitted).count()
                          : 0.0;
    }
    return HMPC_OK;
}

int hmpc_server_drain(hmpc_server* srv, uint32_t timeout_ms)
{
    if (!srv)
    {
        return fail(HMPC_ERROR_INVALID_ARGUMENT, "null server");
    }
    std::unique_lock<std::mutex> lock(srv->mu);
    const bool ok = srv->cv.wait_for(lock, std::chrono::milliseconds(timeout_ms),
                                     [&] { return srv->in_system.load() == 0; });
    return ok ? HMPC_OK : fail(HMPC_ERROR_TIMEOUT, "requests still in flight");
}

int hmpc_server_get_stats(hmpc_server* srv, hmpc_server_stats* out)
{
    if (!srv || !out)
    {
        return fail(HMPC_ERROR_INVALID_ARGUMENT, "null argument");
    }
    std::lock_guard<std::mutex> lock(srv->mu);
    *out = hmpc_server_stats{};
    out->submitted = srv->submitted;
    out->completed = srv->completed;
    out->rejected = srv->rejected;
    out->failed = srv->failed;
    out->dispatches = srv->dispatches;
    out->mean_batch = srv->dispatches ? static_cast<double>(srv->batched_requests) / srv->dispatches : 0.0;
    uint64_t launches = 0;
    for (auto& lane : srv->lanes)
    {
        launches += lane->launches;
    }
    out->launches = launches;
    std::vector<double> lat = srv->latencies_us;
    if (!lat.empty())
    {
        std::sort(lat.begin(), lat.end());
        auto at = [&](double f) { return lat[std::min(lat.size() - 1, static_cast<size_t>(f * (lat.size() - 1) + 0.5))]; };
        out->p50_us = at(0.50);
        out->p99_us = at(0.99);
        double sum = 0;
        for (double v : lat)
        {
            sum += v;
        }
        out->mean_us = sum / lat.size();
    }
    return HMPC_OK;
}

int hmpc_server_destroy(hmpc_server* srv)
{
    if (!srv)
    {
        return HMPC_OK;
    }
    srv->stop.store(true);
    srv->cv.notify_all();
    if (srv->worker.joinable())
    {
        srv->worker.join();
    }
    cudaSetDevice(srv->ctx->device);
    for (size_t i = 0; i < srv->lanes.size(); ++i)
    {
        cudaStreamSynchronize(srv->lanes[i]->stream);
        cudaStreamDestroy(srv->lanes[i]->stream);
        cudaEventDestroy(srv->lane_done[i]);
        cudaFreeHost(srv->lane_desc[i]);
        srv->lanes[i]->stream = nullptr;
    }
    for (auto& k : srv->keys)
    {
        cudaFree(k.a);
        cudaFree(k.b);
    }
    cudaFree(srv->d_desc);
    cudaFree(srv->pool_base);
    delete srv;
    return HMPC_OK;
}

}  // extern "C"
