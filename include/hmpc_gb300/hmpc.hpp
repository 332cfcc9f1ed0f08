// hmpc_gb300/hmpc.hpp -- C++ front end over the C ABI (include/hmpc_gb300.h),
// shaped like hmpc's host API so that code written against hmpc::comp::queue
// and hmpc::expr reads the same:
//
//   hmpc::comp::queue queue(key);                          // comp/queue.hpp:229-239
//   auto& q = queue.modulus(q_words);                     // mod<Q>
//   auto x = hmpc::comp::make_tensor(q, {n_polys}, N);    // comp/tensor.hpp:86-90
//   auto y = queue(hmpc::expr::number_theoretic_transform(hmpc::expr::tensor(x)));
//   auto [u, v] = queue(ntt(centered_binomial(q, {n}, N, half)), ntt(centered_binomial(q, {n}, N, ten)));
//   auto ct = queue(hmpc::expr::crypto::lhe::enc(key, tensor(m), randomness(q, {n}, N)));
//
// The reference's degree, modulus and shapes are template parameters; here
// they are run-time values.  Expressions are lazy, and queue(...) evaluates
// them with the reference's execution plan (expr/cache.hpp:226-306): children
// before parents, left to right, every node materialised once, samplers fused
// into the transform that consumes them -- so sampler nodes draw their nonces
// in the reference's order (comp/queue.hpp:241-253).
#pragma once

#include <algorithm>
#include <array>
#include <cstdint>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <tuple>
#include <utility>
#include <vector>

#include "../hmpc_gb300.h"

namespace hmpc
{
    class error : public std::runtime_error
    {
    public:
        error(int code, const std::string& what) : std::runtime_error(what), code(code)
        {
        }
        int code;
    };

    inline void check(int rc)
    {
        if (rc != HMPC_OK)
        {
            throw error(rc, hmpc_last_error());
        }
    }

    namespace comp
    {
        class queue;

        // mod<Q> registered on a queue (ints/mod.hpp:73-193)
        class modulus
        {
        public:
            modulus(hmpc_context* ctx, const std::vector<uint32_t>& q) : words_(q)
            {
                check(hmpc_modulus_create(ctx, q.data(), static_cast<int>(q.size()), &handle_));
                check(hmpc_modulus_info(handle_, &limbs_, &bits_, nullptr));
            }
            modulus(const modulus&) = delete;
            modulus& operator=(const modulus&) = delete;
            ~modulus()
            {
                hmpc_modulus_destroy(handle_);
            }
            int limbs() const
            {
                return limbs_;
            }
            int bits() const
            {
                return bits_;
            }
            const std::vector<uint32_t>& words() const
            {
                return words_;
            }
            hmpc_modulus* handle() const
            {
                return handle_;
            }
            void prepare(uint64_t n)
            {
                check(hmpc_modulus_prepare(handle_, n));
            }

        private:
            hmpc_modulus* handle_ = nullptr;
            std::vector<uint32_t> words_;
            int limbs_ = 0, bits_ = 0;
        };

        // tensor<poly_mod<Q, N>, Dimensions...>: limb-planar device buffer
        // [limbs][prod(shape) * n] (comp/tensor.hpp:21,25-29)
        class tensor
        {
        public:
            tensor() = default;
            tensor(hmpc_context* ctx, modulus* mod, std::vector<uint64_t> shape, uint64_t n)
                : ctx_(ctx), mod_(mod), shape_(std::move(shape)), n_(n)
            {
                uint32_t* p = nullptr;
                check(hmpc_tensor_alloc(ctx, words(), &p));
                data_ = std::shared_ptr<uint32_t>(p, [ctx](uint32_t* q) { hmpc_tensor_free(ctx, q); });
            }
            uint64_t batch() const
            {
                uint64_t b = 1;
                for (uint64_t s : shape_)
                {
                    b *= s;
                }
                return b;
            }
            uint64_t elements() const
            {
                return batch() * n_;
            }
            uint64_t words() const
            {
                return elements() * static_cast<uint64_t>(mod_->limbs());
            }
            uint64_t n() const
            {
                return n_;
            }
            const std::vector<uint64_t>& shape() const
            {
                return shape_;
            }
            modulus& mod() const
            {
                return *mod_;
            }
            uint32_t* data() const
            {
                return data_.get();
            }
            void upload(const std::vector<uint32_t>& host)
            {
                if (host.size() != words())
                {
                    throw error(HMPC_ERROR_INVALID_ARGUMENT, "host buffer size differs from the tensor");
                }
                check(hmpc_tensor_upload(ctx_, data(), host.data(), words()));
            }
            std::vector<uint32_t> download() const
            {
                std::vector<uint32_t> host(words());
                check(hmpc_tensor_download(ctx_, host.data(), data(), words()));
                return host;
            }

        private:
            hmpc_context* ctx_ = nullptr;
            modulus* mod_ = nullptr;
            std::vector<uint64_t> shape_;
            uint64_t n_ = 1;
            std::shared_ptr<uint32_t> data_;
        };
    }

    namespace expr
    {
        enum class kind
        {
            tensor,
            centered_binomial,
            uniform,
            ntt,
            intt,
            add,
            subtract,
            multiply,
            cast,
            lhe_combine,
            matrix_vector_product,
            sum,
            product,
        };

        // A node of the lazy expression DAG.  Nodes are shared; identity
        // (pointer equality) plays the role of the reference's type tags in
        // its cache plan.
        struct node
        {
            kind k;
            comp::modulus* mod = nullptr;
            std::vector<uint64_t> shape;
            uint64_t n = 1;
            comp::tensor value;                      // leaf tensor or materialised result
            uint32_t variance_x2 = 0;                // centered_binomial
            std::vector<std::shared_ptr<node>> children;
            std::vector<uint32_t> constant;          // lhe_combine: p as a residue mod q
        };

        using expression = std::shared_ptr<node>;

        inline uint64_t batch_of(const std::vector<uint64_t>& shape)
        {
            uint64_t b = 1;
            for (uint64_t s : shape)
            {
                b *= s;
            }
            return b;
        }

        // tensor(t) (expr/tensor.hpp:10-49)
        inline expression tensor(const comp::tensor& t)
        {
            auto e = std::make_shared<node>();
            e->k = kind::tensor;
            e->mod = &t.mod();
            e->shape = t.shape();
            e->n = t.n();
            e->value = t;
            return e;
        }

        constexpr uint32_t half = 1;  // 2V for V = 1/2
        constexpr uint32_t ten = 20;  // 2V for V = 10

        // centered_binomial<R>(shape, V) (expr/random/binomial.hpp:176-236), 2V = variance_x2
        inline expression centered_binomial(comp::modulus& mod, std::vector<uint64_t> shape, uint64_t n,
                                            uint32_t variance_x2)
        {
            auto e = std::make_shared<node>();
            e->k = kind::centered_binomial;
            e->mod = &mod;
            e->shape = std::move(shape);
            e->n = n;
            e->variance_x2 = variance_x2;
            return e;
        }

        // uniform<R>(shape) (expr/random/uniform.hpp:10-58)
        inline expression uniform(comp::modulus& mod, std::vector<uint64_t> shape, uint64_t n)
        {
            auto e = std::make_shared<node>();
            e->k = kind::uniform;
            e->mod = &mod;
            e->shape = std::move(shape);
            e->n = n;
            return e;
        }

        inline expression unary(kind k, expression inner)
        {
            auto e = std::make_shared<node>();
            e->k = k;
            e->mod = inner->mod;
            e->shape = inner->shape;
            e->n = inner->n;
            e->children = {std::move(inner)};
            return e;
        }

        // number_theoretic_transform(e) / inverse_...(e)
        // (expr/number_theoretic_transform.hpp:552-592)
        inline expression number_theoretic_transform(expression e)
        {
            return unary(kind::ntt, std::move(e));
        }
        inline expression inverse_number_theoretic_transform(expression e)
        {
            return unary(kind::intt, std::move(e));
        }

        // cast<mod<Q'>>(e): centred lift (expr/cast.hpp:10-53)
        inline expression cast(comp::modulus& target, expression e)
        {
            auto c = unary(kind::cast, std::move(e));
            c->mod = &target;
            return c;
        }

        inline expression binary(kind k, expression a, expression b)
        {
            auto e = std::make_shared<node>();
            e->k = k;
            e->mod = a->mod;
            // broadcasting: the operand with more elements gives the shape
            // (unsqueeze + common_shape, expr/unsqueeze.hpp, shape.hpp:207-239)
            const bool a_big = batch_of(a->shape) >= batch_of(b->shape);
            e->shape = a_big ? a->shape : b->shape;
            e->n = a->n;
            e->children = {std::move(a), std::move(b)};
            return e;
        }

        // matrix_vector_product(m, x) (expr/matrix_vector_product.hpp:125-143):
        // m of shape {batch or 1, rows, cols}, x of shape {batch or 1, cols},
        // both of the same modulus and degree; the result has shape {batch, rows}
        inline expression matrix_vector_product(expression m, expression x)
        {
            if (m->shape.size() != 3 || x->shape.size() != 2 || m->shape[2] != x->shape[1] || m->n != x->n ||
                m->mod != x->mod)
            {
                throw error(HMPC_ERROR_INVALID_ARGUMENT,
                            "matrix_vector_product takes shapes {batch, rows, cols} and {batch, cols}");
            }
            auto e = std::make_shared<node>();
            e->k = kind::matrix_vector_product;
            e->mod = m->mod;
            e->shape = {std::max(m->shape[0], x->shape[0]), m->shape[1]};
            e->n = m->n;
            e->children = {std::move(m), std::move(x)};
            return e;
        }

        // sum(e) / product(e) of every residue (expr/reduce.hpp:257-267): a
        // rank-0 result
        inline expression reduction(kind k, expression inner)
        {
            auto e = std::make_shared<node>();
            e->k = k;
            e->mod = inner->mod;
            e->n = 1;
            e->children = {std::move(inner)};
            return e;
        }
        inline expression sum(expression e)
        {
            return reduction(kind::sum, std::move(e));
        }
        inline expression product(expression e)
        {
            return reduction(kind::product, std::move(e));
        }

        namespace operators
        {
            inline expression operator+(expression a, expression b)
            {
                return binary(kind::add, std::move(a), std::move(b));
            }
            inline expression operator-(expression a, expression b)
            {
                return binary(kind::subtract, std::move(a), std::move(b));
            }
            inline expression operator*(expression a, expression b)
            {
                return binary(kind::multiply, std::move(a), std::move(b));
            }
        }
    }

    namespace comp
    {
        class queue
        {
        public:
            explicit queue(const std::array<uint32_t, 8>& key, int device = 0, void* stream = nullptr)
            {
                check(hmpc_context_create(device, key.data(), stream, &ctx_));
            }
            queue(const queue&) = delete;
            queue& operator=(const queue&) = delete;
            ~queue()
            {
                moduli_.clear();
                hmpc_context_destroy(ctx_);
            }

            hmpc_context* handle() const
            {
                return ctx_;
            }

            comp::modulus& modulus(const std::vector<uint32_t>& q)
            {
                auto it = moduli_.find(q);
                if (it == moduli_.end())
                {
                    it = moduli_.emplace(q, std::make_unique<comp::modulus>(ctx_, q)).first;
                }
                return *it->second;
            }

            void wait()
            {
                check(hmpc_context_synchronize(ctx_));
            }

            std::array<uint32_t, 3> nonce() const
            {
                std::array<uint32_t, 3> n{};
                check(hmpc_context_get_nonce(ctx_, n.data()));
                return n;
            }
            void set_nonce(const std::array<uint32_t, 3>& n)
            {
                check(hmpc_context_set_nonce(ctx_, n.data()));
            }

            // queue(exprs...) (comp/queue.hpp:416-529): evaluate with the
            // reference's plan and return the results
            template<typename... E>
            auto operator()(E... exprs)
            {
                std::vector<expr::expression> plan;
                (collect(exprs, plan), ...);
                for (auto& e : plan)
                {
                    execute(e);
                }
                if constexpr (sizeof...(E) == 1)
                {
                    return (exprs->value, ...);
                }
                else
                {
                    return std::make_tuple(exprs->value...);
                }
            }

        private:
            static bool is_sampler(const expr::expression& e)
            {
                return e->k == expr::kind::centered_binomial || e->k == expr::kind::uniform;
            }

            // post-order, left to right, each node once; a sampler that is the
            // direct input of a forward transform is fused into it
            // (expr/cache.hpp:226-271: complex nodes are always materialised,
            // a once-accessed single-consumer child is fused)
            void collect(const expr::expression& e, std::vector<expr::expression>& plan)
            {
                for (const auto& p : plan)
                {
                    if (p == e)
                    {
                        return;
                    }
                }
                if (e->k == expr::kind::tensor)
                {
                    return;
                }
                const bool fuse_child = e->k == expr::kind::ntt && is_sampler(e->children[0]);
                if (!fuse_child)
                {
                    for (const auto& c : e->children)
                    {
                        collect(c, plan);
                    }
                }
                plan.push_back(e);
            }

            comp::tensor result_of(const expr::expression& e)
            {
                if (!e->value.data())
                {
                    e->value = comp::tensor(ctx_, e->mod, e->shape, e->n);
                }
                return e->value;
            }

            void execute(const expr::expression& e)
            {
                comp::tensor out = result_of(e);
                auto child = [&](size_t i) { return e->children[i]->value; };
                switch (e->k)
                {
                case expr::kind::ntt:
                {
                    const auto& c = e->children[0];
                    hmpc_producer p{HMPC_PRODUCER_TENSOR, nullptr, 0, 0};
                    if (c->k == expr::kind::centered_binomial)
                    {
                        p = {HMPC_PRODUCER_CBD, nullptr, c->variance_x2, 0};
                    }
                    else if (c->k == expr::kind::uniform)
                    {
                        p = {HMPC_PRODUCER_UNIFORM, nullptr, 0, 80};
                    }
                    else
                    {
                        p.src = c->value.data();
                    }
                    check(hmpc_ntt_forward(ctx_, e->mod->handle(), e->n, expr::batch_of(e->shape), &p, out.data()));
                    break;
                }
                case expr::kind::intt:
                    check(hmpc_ntt_inverse(ctx_, e->mod->handle(), e->n, expr::batch_of(e->shape), child(0).data(),
                                           out.data()));
                    break;
                case expr::kind::centered_binomial:
                    check(hmpc_sample_cbd(ctx_, e->mod->handle(), out.elements(), e->variance_x2, out.data()));
                    break;
                case expr::kind::uniform:
                    check(hmpc_sample_uniform(ctx_, e->mod->handle(), out.elements(), 80, out.data()));
                    break;
                case expr::kind::cast:
                    check(hmpc_cast(ctx_, e->mod->handle(), e->children[0]->mod->handle(), out.elements(),
                                    child(0).data(), out.data()));
                    break;
                case expr::kind::add:
                case expr::kind::subtract:
                case expr::kind::multiply:
                {
                    const int op = e->k == expr::kind::add ? HMPC_OP_ADD
                                   : e->k == expr::kind::subtract ? HMPC_OP_SUB : HMPC_OP_MUL;
                    const comp::tensor a = child(0), b = child(1);
                    check(hmpc_binary(ctx_, e->mod->handle(), op, out.elements(), a.data(), a.elements(), b.data(),
                                      b.elements(), out.data()));
                    break;
                }
                case expr::kind::matrix_vector_product:
                {
                    const auto& m = e->children[0];
                    const auto& x = e->children[1];
                    check(hmpc_matvec(ctx_, e->mod->handle(), e->shape[0], m->shape[1], m->shape[2], e->n,
                                      child(0).data(), m->shape[0], child(1).data(), x->shape[0], out.data()));
                    break;
                }
                case expr::kind::sum:
                case expr::kind::product:
                    check(hmpc_reduce(ctx_, e->mod->handle(),
                                      e->k == expr::kind::sum ? HMPC_REDUCE_ADD : HMPC_REDUCE_MULTIPLY,
                                      child(0).elements(), child(0).data(), out.data()));
                    break;
                default:
                    throw error(HMPC_ERROR_UNSUPPORTED, "expression node not supported by this front end");
                }
            }

            hmpc_context* ctx_ = nullptr;
            std::map<std::vector<uint32_t>, std::unique_ptr<comp::modulus>> moduli_;
        };

        inline tensor make_tensor(queue& q, modulus& mod, std::vector<uint64_t> shape, uint64_t n = 1)
        {
            return tensor(q.handle(), &mod, std::move(shape), n);
        }
    }

    namespace crypto::lhe
    {
        // comp::crypto::lhe::key{a, b} (comp/crypto/lhe/key.hpp:7-12)
        struct key
        {
            comp::tensor a, b;
        };

        // comp::crypto::lhe::ciphertext{c0, c1} (comp/crypto/lhe/ciphertext.hpp:8-32)
        struct ciphertext
        {
            comp::tensor c0, c1;
        };

        // (s, key) with a = b*s + p*e; no counterpart in the reference
        inline std::pair<comp::tensor, key> keygen(comp::queue& queue, comp::modulus& q, comp::modulus& p, uint64_t n)
        {
            comp::tensor s = comp::make_tensor(queue, q, {}, n);
            key k{comp::make_tensor(queue, q, {}, n), comp::make_tensor(queue, q, {}, n)};
            check(hmpc_lhe_keygen(queue.handle(), q.handle(), p.handle(), n, s.data(), k.a.data(), k.b.data()));
            return {s, k};
        }

        // enc(key, plaintext, randomness<Rq>(shape)) (expr/crypto/lhe/enc.hpp:19-69)
        inline ciphertext enc(comp::queue& queue, const key& k, const comp::tensor& plaintext, comp::modulus& q,
                              bool plaintext_ntt = false)
        {
            ciphertext ct{comp::make_tensor(queue, q, plaintext.shape(), plaintext.n()),
                          comp::make_tensor(queue, q, plaintext.shape(), plaintext.n())};
            check(hmpc_lhe_enc(queue.handle(), q.handle(), plaintext.mod().handle(), plaintext.n(),
                               plaintext.elements() / plaintext.n(), k.a.data(), k.b.data(), plaintext.data(),
                               plaintext_ntt ? 1 : 0, ct.c0.data(), ct.c1.data()));
            return ct;
        }

        // dec<Plaintext>(s, ct) (expr/crypto/lhe/dec.hpp:13-45)
        inline comp::tensor dec(comp::queue& queue, const comp::tensor& s, const ciphertext& ct, comp::modulus& p,
                                bool plaintext_ntt = false)
        {
            comp::tensor out = comp::make_tensor(queue, p, ct.c0.shape(), ct.c0.n());
            check(hmpc_lhe_dec(queue.handle(), ct.c0.mod().handle(), p.handle(), ct.c0.n(),
                               ct.c0.elements() / ct.c0.n(), s.data(), ct.c0.data(), ct.c1.data(),
                               plaintext_ntt ? 1 : 0, out.data()));
            return out;
        }
    }
}
