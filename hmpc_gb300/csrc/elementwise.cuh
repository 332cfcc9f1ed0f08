// Elementwise kernels over limb-planar tensors (limb j of element e at
// [j * elements + e], hmpc/comp/tensor.hpp:21,25-29).
//
// Every thread handles V = 4 consecutive elements so that each limb plane is
// read and written with 128-bit accesses; HBM traffic is the algorithmic
// minimum (each operand limb read once, each result limb written once).
#pragma once

#include <cstdint>

#include "chacha.cuh"
#include "limbs.cuh"

namespace hmpc_gb300
{
    constexpr int vec = 4;

    template<int L>
    __device__ __forceinline__ void load4(uint32_t (&x)[vec][L], const uint32_t* t, uint64_t elements, uint64_t e)
    {
#pragma unroll
        for (int j = 0; j < L; ++j)
        {
            const uint4 v = __ldcs(reinterpret_cast<const uint4*>(t + static_cast<uint64_t>(j) * elements + e));
            x[0][j] = v.x;
            x[1][j] = v.y;
            x[2][j] = v.z;
            x[3][j] = v.w;
        }
    }

    template<int L>
    __device__ __forceinline__ void store4(uint32_t* t, uint64_t elements, uint64_t e, const uint32_t (&x)[vec][L])
    {
#pragma unroll
        for (int j = 0; j < L; ++j)
        {
            const uint4 v = make_uint4(x[0][j], x[1][j], x[2][j], x[3][j]);
            __stcs(reinterpret_cast<uint4*>(t + static_cast<uint64_t>(j) * elements + e), v);
        }
    }

    template<int L>
    __device__ __forceinline__ void load1(uint32_t (&x)[L], const uint32_t* t, uint64_t elements, uint64_t e)
    {
#pragma unroll
        for (int j = 0; j < L; ++j)
        {
            x[j] = t[static_cast<uint64_t>(j) * elements + e];
        }
    }

    template<int L>
    __device__ __forceinline__ void store1(uint32_t* t, uint64_t elements, uint64_t e, const uint32_t (&x)[L])
    {
#pragma unroll
        for (int j = 0; j < L; ++j)
        {
            t[static_cast<uint64_t>(j) * elements + e] = x[j];
        }
    }

    // d = a*b + c (examples/fma.cpp:56-67).  vectorised path: elements % 4 == 0
    // and 16-byte aligned planes; the scalar path covers everything else.
    template<int L>
    __global__ void __launch_bounds__(256) fma_kernel(uint32_t* d, const uint32_t* a, const uint32_t* b,
                                                      const uint32_t* c, uint64_t elements, int vectorised,
                                                      const Modulus<L> m)
    {
        const uint64_t tid = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
        if (vectorised)
        {
            const uint64_t e = tid * vec;
            if (e >= elements)
            {
                return;
            }
            uint32_t x[vec][L], y[vec][L], z[vec][L];
            load4<L>(x, a, elements, e);
            load4<L>(y, b, elements, e);
            load4<L>(z, c, elements, e);
#pragma unroll
            for (int k = 0; k < vec; ++k)
            {
                mont_mul<L>(x[k], x[k], y[k], m);
                mod_add<L>(x[k], x[k], z[k], m);
            }
            store4<L>(d, elements, e, x);
        }
        else
        {
            for (uint64_t e = tid; e < elements; e += static_cast<uint64_t>(gridDim.x) * blockDim.x)
            {
                uint32_t x[L], y[L], z[L];
                load1<L>(x, a, elements, e);
                load1<L>(y, b, elements, e);
                load1<L>(z, c, elements, e);
                mont_mul<L>(x, x, y, m);
                mod_add<L>(x, x, z, m);
                store1<L>(d, elements, e, x);
            }
        }
    }

    enum BinaryOp : int
    {
        op_add = 0,
        op_sub = 1,
        op_mul = 2,
    };

    // out[e] = a[e mod a_elements] OP b[e mod b_elements]: broadcasting of a
    // single polynomial (or scalar) over a batch, as unsqueeze + the binary
    // expressions evaluate it (hmpc/expr/binary_expression.hpp:118-136,
    // hmpc/expr/unsqueeze.hpp:9-61).
    template<int L>
    __global__ void __launch_bounds__(256) binary_kernel(uint32_t* out, const uint32_t* a, uint64_t a_elements,
                                                         const uint32_t* b, uint64_t b_elements, uint64_t elements,
                                                         int op, const Modulus<L> m)
    {
        for (uint64_t e = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x; e < elements;
             e += static_cast<uint64_t>(gridDim.x) * blockDim.x)
        {
            uint32_t x[L], y[L], r[L];
            load1<L>(x, a, a_elements, a_elements == elements ? e : e % a_elements);
            load1<L>(y, b, b_elements, b_elements == elements ? e : e % b_elements);
            if (op == op_add)
            {
                mod_add<L>(r, x, y, m);
            }
            else if (op == op_sub)
            {
                mod_sub<L>(r, x, y, m);
            }
            else
            {
                mont_mul<L>(r, x, y, m);
            }
            store1<L>(out, elements, e, r);
        }
    }

    // out[e] = k[e mod n]*u[e] + v[e]*pc + (msg ? msg[e] : 0), the fused
    // elementwise node of BGV encryption (expr/crypto/lhe/enc.hpp:65-68,
    // examples/bgv.cpp:88-91): c0 with msg, c1 without.
    template<int L>
    __global__ void __launch_bounds__(256) lhe_combine_kernel(uint32_t* out, const uint32_t* k, uint64_t n,
                                                              const uint32_t* u, const uint32_t* v,
                                                              const uint32_t* msg, uint64_t elements,
                                                              const Modulus<L> m, const Modulus<L> pc_holder)
    {
        for (uint64_t e = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x; e < elements;
             e += static_cast<uint64_t>(gridDim.x) * blockDim.x)
        {
            uint32_t x[L], y[L], r[L];
            load1<L>(x, k, n, e % n);
            load1<L>(y, u, elements, e);
            mont_mul<L>(r, x, y, m);
            load1<L>(x, v, elements, e);
            mont_mul<L>(x, x, pc_holder.one, m);
            mod_add<L>(r, r, x, m);
            if (msg)
            {
                load1<L>(x, msg, elements, e);
                mod_add<L>(r, r, x, m);
            }
            store1<L>(out, elements, e, r);
        }
    }

    // c0 = a * u + x and c1 = b * u + w with the key polynomials a, b broadcast
    // over the batch: the BGV combine when p * v (+ the lifted plaintext) and
    // p * w already went through the transform as inputs of their own
    // (linearity of the NTT).  u, x, w are the three parts of one stacked
    // transform output, [L][3 * elements]; u is read once for both products.
    // One element per thread (about 50 registers at L = 8): enough resident
    // warps to cover the loads' latency with the products' arithmetic.
    // n is a power of two.
    template<int L>
    __global__ void __launch_bounds__(256) lhe_combine_pair_kernel(uint32_t* c0, uint32_t* c1, const uint32_t* ka,
                                                                   const uint32_t* kb, uint64_t n,
                                                                   const uint32_t* stacked, uint64_t elements,
                                                                   const Modulus<L> m)
    {
        const uint64_t stride = 3 * elements;
        const uint64_t mask = n - 1;
        for (uint64_t e = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x; e < elements;
             e += static_cast<uint64_t>(gridDim.x) * blockDim.x)
        {
            uint32_t u[L], k[L], x[L];
            load1<L>(u, stacked, stride, e);
            load1<L>(k, ka, n, e & mask);
            load1<L>(x, stacked + elements, stride, e);
            mont_mul<L>(k, k, u, m);
            mod_add<L>(x, x, k, m);
            store1<L>(c0, elements, e, x);
            load1<L>(k, kb, n, e & mask);
            load1<L>(x, stacked + 2 * elements, stride, e);
            mont_mul<L>(k, k, u, m);
            mod_add<L>(x, x, k, m);
            store1<L>(c1, elements, e, x);
        }
    }

    // ciphertext x ciphertext in NTT form: the tensor product
    // (d0, d1, d2) = (a0*b0, a0*b1 + a1*b0, a1*b1).  No counterpart in the
    // reference, whose ciphertexts only support linear operations
    // (expr/crypto/lhe/ciphertext.hpp:49-81).
    template<int L>
    __global__ void __launch_bounds__(256) ct_mul_kernel(uint32_t* d0, uint32_t* d1, uint32_t* d2,
                                                         const uint32_t* a0, const uint32_t* a1, const uint32_t* b0,
                                                         const uint32_t* b1, uint64_t elements, const Modulus<L> m)
    {
        for (uint64_t e = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x; e < elements;
             e += static_cast<uint64_t>(gridDim.x) * blockDim.x)
        {
            uint32_t x0[L], x1[L], y0[L], y1[L], r[L], t[L];
            load1<L>(x0, a0, elements, e);
            load1<L>(x1, a1, elements, e);
            load1<L>(y0, b0, elements, e);
            load1<L>(y1, b1, elements, e);
            mont_mul<L>(r, x0, y0, m);
            store1<L>(d0, elements, e, r);
            mont_mul<L>(r, x0, y1, m);
            mont_mul<L>(t, x1, y0, m);
            mod_add<L>(r, r, t, m);
            store1<L>(d1, elements, e, r);
            mont_mul<L>(r, x1, y1, m);
            store1<L>(d2, elements, e, r);
        }
    }

    // x = c0 - s*c1 (+ s^2*c2 for a product ciphertext), s broadcast over the
    // batch: the first node of dec (expr/crypto/lhe/dec.hpp:29), extended to
    // degree-2 ciphertexts by Horner's rule c0 - s*(c1 - s*c2).
    template<int L>
    __global__ void __launch_bounds__(256) dec_combine_kernel(uint32_t* x, const uint32_t* s, uint64_t n,
                                                              const uint32_t* c0, const uint32_t* c1,
                                                              const uint32_t* c2, uint64_t elements,
                                                              const Modulus<L> m)
    {
        for (uint64_t e = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x; e < elements;
             e += static_cast<uint64_t>(gridDim.x) * blockDim.x)
        {
            uint32_t sk[L], a[L], b[L];
            load1<L>(sk, s, n, e % n);
            load1<L>(b, c1, elements, e);
            if (c2)
            {
                load1<L>(a, c2, elements, e);
                mont_mul<L>(a, sk, a, m);
                mod_sub<L>(b, b, a, m);
            }
            mont_mul<L>(b, sk, b, m);
            load1<L>(a, c0, elements, e);
            mod_sub<L>(a, a, b, m);
            store1<L>(x, elements, e, a);
        }
    }

    // elementwise samplers: element e uses the generator (key, nonce,
    // counter = e) and draws one value (expr/random/uniform.hpp:41-45,
    // expr/random/binomial.hpp:207-211, comp/queue.hpp:386-412)
    template<int L, int W>
    __global__ void __launch_bounds__(256) uniform_kernel(uint32_t* out, uint64_t elements, const RngKey rng,
                                                          uint32_t top_mask, const Modulus<L> m)
    {
        for (uint64_t e = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x; e < elements;
             e += static_cast<uint64_t>(gridDim.x) * blockDim.x)
        {
            uint32_t w[W];
            chacha_stream<W>(rng, static_cast<uint32_t>(e), w);
            uint32_t r[L];
            uniform_from_words<L, W, 0, W>(r, w, top_mask, m);
            store1<L>(out, elements, e, r);
        }
    }

    // The uniform draws of a forward transform's stage-0 pairs, written as the
    // transform's input: pair (j, j + n/2) of polynomial i uses the generator
    // (key, nonce, counter = i * n + j) and draws element j's value, then
    // element j + n/2's -- the values the sampler fused into the transform's
    // first stage draws (expr/number_theoretic_transform.hpp:316-329), for a
    // transform engine that reads its input from memory.  W words per value.
    template<int L, int W>
    __global__ void __launch_bounds__(256) uniform_pairs_kernel(uint32_t* out, uint32_t log_n, uint64_t elements,
                                                                const RngKey rng, uint32_t top_mask,
                                                                const Modulus<L> m)
    {
        const uint64_t half = 1ull << (log_n - 1);
        for (uint64_t t = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x; t < elements / 2;
             t += static_cast<uint64_t>(gridDim.x) * blockDim.x)
        {
            const uint64_t e = ((t >> (log_n - 1)) << log_n) + (t & (half - 1));
            uint32_t w[2 * W];
            chacha_stream<2 * W>(rng, static_cast<uint32_t>(e), w);
            uint32_t u[L], v[L];
            uniform_from_words<L, W, 0, 2 * W>(u, w, top_mask, m);
            uniform_from_words<L, W, W, 2 * W>(v, w, top_mask, m);
            store1<L>(out, elements, e, u);
            store1<L>(out, elements, e + half, v);
        }
    }

    template<int L, int NW>
    __global__ void __launch_bounds__(256) cbd_kernel(uint32_t* out, uint64_t elements, const RngKey rng,
                                                      uint32_t vx2, const uint32_t* small_table, const Modulus<L> m)
    {
        for (uint64_t e = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x; e < elements;
             e += static_cast<uint64_t>(gridDim.x) * blockDim.x)
        {
            uint32_t w[NW];
            chacha_stream<NW>(rng, static_cast<uint32_t>(e), w);
            const int count = 2 * static_cast<int>(vx2);
            int a = 0;
#pragma unroll
            for (int i = 0; i < NW; ++i)
            {
                uint32_t mask = 0xffffffffu;
                if (i == NW - 1 && (count & 31))
                {
                    mask = (1u << (count & 31)) - 1u;
                }
                a += __popc(w[i] & mask);
            }
            uint32_t r[L];
            small_to_mont<L>(r, a - static_cast<int>(vx2), small_table, m);
            store1<L>(out, elements, e, r);
        }
    }

    // canonical integers (< Q) -> Montgomery form: mont_mul(x, R^2)
    template<int L>
    __global__ void __launch_bounds__(256) to_montgomery_kernel(uint32_t* out, const uint32_t* in, uint64_t elements,
                                                                const Modulus<L> r2_holder, const Modulus<L> m)
    {
        for (uint64_t e = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x; e < elements;
             e += static_cast<uint64_t>(gridDim.x) * blockDim.x)
        {
            uint32_t x[L];
            load1<L>(x, in, elements, e);
            mont_mul<L>(x, x, r2_holder.one, m);
            store1<L>(out, elements, e, x);
        }
    }

    // Montgomery form -> canonical integer: mont_mul(x, 1) (mod.hpp:356-361)
    template<int L>
    __global__ void __launch_bounds__(256) from_montgomery_kernel(uint32_t* out, const uint32_t* in,
                                                                  uint64_t elements, const Modulus<L> m)
    {
        for (uint64_t e = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x; e < elements;
             e += static_cast<uint64_t>(gridDim.x) * blockDim.x)
        {
            uint32_t x[L], o[L];
            load1<L>(x, in, elements, e);
            set_zero<L>(o);
            o[0] = 1u;
            mont_mul<L>(x, x, o, m);
            store1<L>(out, elements, e, x);
        }
    }
}
