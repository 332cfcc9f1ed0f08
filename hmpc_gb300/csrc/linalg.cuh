// Matrix-vector products and reductions over limb-planar tensors: the
// consumers of NTT-form data after the transform (hmpc/expr/
// matrix_vector_product.hpp, hmpc/expr/bit_monomial.hpp, hmpc/expr/reduce.hpp).
//
// Every kernel is exact modular (or wrapping unsigned) arithmetic on fully
// reduced representatives, so any evaluation order gives the reference's bits.
#pragma once

#include <cstdint>

#include "elementwise.cuh"
#include "limbs.cuh"

namespace hmpc_gb300
{
    // z[b][i][c] over `total` = batch * rows * coeffs output elements, row-major;
    // the matrix and vector batches advance by their strides (0: broadcast)
    struct MatvecParams
    {
        uint64_t total;
        uint64_t rows, cols, coeffs;
        int coeff_shift;             // log2(coeffs) when a power of two, else -1
        uint64_t m_bstride, x_bstride;  // elements between batches of m (or degrees) and of x
        uint64_t m_elements, x_elements;
    };

    struct MatvecIndex
    {
        uint64_t b, i, c, r;  // r = b * rows + i
    };

    __device__ __forceinline__ MatvecIndex matvec_index(const MatvecParams& p, uint64_t e)
    {
        MatvecIndex ix;
        ix.r = p.coeff_shift >= 0 ? e >> p.coeff_shift : e / p.coeffs;
        ix.c = e - ix.r * p.coeffs;
        ix.b = ix.r / p.rows;
        ix.i = ix.r - ix.b * p.rows;
        return ix;
    }

    // z[b][i][c] = sum_k m[b][i][k][c] * x[b][k][c] mod Q: the fold of
    // expr/matrix_vector_product.hpp:88-140 with mod<Q>'s product and sum.  One
    // thread per output element; consecutive threads take consecutive
    // coefficients, so every matrix and vector plane is read coalesced (the
    // vector rows are shared by all `rows` outputs of a batch through L2).
    template<int L>
    __global__ void __launch_bounds__(256) matvec_kernel(uint32_t* z, const uint32_t* mat, const uint32_t* x,
                                                         const MatvecParams p, const Modulus<L> m)
    {
        for (uint64_t e = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x; e < p.total;
             e += static_cast<uint64_t>(gridDim.x) * blockDim.x)
        {
            const MatvecIndex ix = matvec_index(p, e);
            const uint64_t mb = ix.b * p.m_bstride + ix.i * p.cols * p.coeffs + ix.c;
            const uint64_t xb = ix.b * p.x_bstride + ix.c;
            uint32_t acc[L], a[L], v[L];
            set_zero<L>(acc);
            for (uint64_t k = 0; k < p.cols; ++k)
            {
                load1<L>(a, mat, p.m_elements, mb + k * p.coeffs);
                load1<L>(v, x, p.x_elements, xb + k * p.coeffs);
                mont_mul<L>(a, a, v, m);
                mod_add<L>(acc, acc, a, m);
            }
            store1<L>(z, p.total, e, acc);
        }
    }

    // The same fold with a matrix of bit monomials (expr/bit_monomial.hpp:
    // 28-104): coefficient c of X^d * x is x[(c - d) mod n], negated when the
    // unsigned difference c - d has bit log2(n) set; a negative degree is
    // std::nullopt and contributes zero.  Here coeffs = n and coeff_shift =
    // log2(n) always.  The degree of (b, i, k) is uniform across a warp's
    // consecutive coefficients, so its load is a broadcast.
    template<int L>
    __global__ void __launch_bounds__(256) matvec_monomial_kernel(uint32_t* z, const int64_t* degrees,
                                                                  const uint32_t* x, const MatvecParams p,
                                                                  const Modulus<L> m)
    {
        const uint64_t mask = p.coeffs - 1;
        for (uint64_t e = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x; e < p.total;
             e += static_cast<uint64_t>(gridDim.x) * blockDim.x)
        {
            const MatvecIndex ix = matvec_index(p, e);
            const int64_t* dp = degrees + ix.b * p.m_bstride + ix.i * p.cols;
            const uint64_t xb = ix.b * p.x_bstride;
            uint32_t acc[L], v[L];
            set_zero<L>(acc);
            for (uint64_t k = 0; k < p.cols; ++k)
            {
                const int64_t d = __ldg(dp + k);
                if (d < 0)
                {
                    continue;
                }
                const uint64_t difference = ix.c - static_cast<uint64_t>(d);
                load1<L>(v, x, p.x_elements, xb + k * p.coeffs + (difference & mask));
                if ((difference >> p.coeff_shift) & 1u)
                {
                    mod_neg<L>(v, v, m);
                }
                mod_add<L>(acc, acc, v, m);
            }
            store1<L>(z, p.total, e, acc);
        }
    }

    enum ReduceOp : int
    {
        reduce_add = 0,
        reduce_multiply = 1,
        reduce_bit_and = 2,
        reduce_bit_or = 3,
        reduce_bit_xor = 4,
        reduce_min = 5,
        reduce_max = 6,
    };

    // low L limbs of a * b (uint<bits> keeps the low bits of its products)
    template<int L>
    __device__ __forceinline__ void mul_low(uint32_t (&r)[L], const uint32_t (&a)[L], const uint32_t (&b)[L])
    {
        uint32_t t[L];
        set_zero<L>(t);
#pragma unroll
        for (int i = 0; i < L; ++i)
        {
            uint32_t carry = 0;
#pragma unroll
            for (int j = 0; j + i < L; ++j)
            {
                const uint64_t s = static_cast<uint64_t>(a[j]) * b[i] + t[i + j] + carry;
                t[i + j] = static_cast<uint32_t>(s);
                carry = static_cast<uint32_t>(s >> 32);
            }
        }
#pragma unroll
        for (int j = 0; j < L; ++j)
        {
            r[j] = t[j];
        }
    }

    // -1, 0, 1 as a <, ==, > b
    template<int L>
    __device__ __forceinline__ int compare(const uint32_t (&a)[L], const uint32_t (&b)[L])
    {
        int c = 0;
#pragma unroll
        for (int j = 0; j < L; ++j)
        {
            c = a[j] != b[j] ? (a[j] > b[j] ? 1 : -1) : c;
        }
        return c;
    }

    // The reduction's operation and identity (expr/reduce.hpp:14-48, 167-200):
    // mod<Q> sums and Montgomery products (identity R mod Q,
    // ints/integer_traits.hpp:75-76), or uint<bits> operations wrapping modulo
    // 2^bits (identities ints/integer_traits.hpp:39-46).  top_mask keeps the
    // low bits of the top limb of a uint<bits>.
    template<int L, bool Mod>
    struct Reducer
    {
        int op;
        uint32_t top_mask;
        Modulus<L> m;

        __device__ __forceinline__ void identity(uint32_t (&acc)[L]) const
        {
            const bool ones = !Mod && (op == reduce_bit_and || op == reduce_min);
#pragma unroll
            for (int j = 0; j < L; ++j)
            {
                acc[j] = ones ? 0xffffffffu : 0u;
            }
            acc[L - 1] &= Mod ? 0xffffffffu : top_mask;
            if (op == reduce_multiply)
            {
                if constexpr (Mod)
                {
#pragma unroll
                    for (int j = 0; j < L; ++j)
                    {
                        acc[j] = m.one[j];
                    }
                }
                else
                {
                    acc[0] = 1u;
                }
            }
        }

        __device__ __forceinline__ void combine(uint32_t (&acc)[L], const uint32_t (&v)[L]) const
        {
            if constexpr (Mod)
            {
                if (op == reduce_add)
                {
                    mod_add<L>(acc, acc, v, m);
                }
                else
                {
                    mont_mul<L>(acc, acc, v, m);
                }
            }
            else
            {
                switch (op)
                {
                case reduce_add:
                {
                    uint32_t carry = 0;
#pragma unroll
                    for (int j = 0; j < L; ++j)
                    {
                        const uint64_t s = static_cast<uint64_t>(acc[j]) + v[j] + carry;
                        acc[j] = static_cast<uint32_t>(s);
                        carry = static_cast<uint32_t>(s >> 32);
                    }
                    break;
                }
                case reduce_multiply:
                    mul_low<L>(acc, acc, v);
                    break;
                case reduce_bit_and:
#pragma unroll
                    for (int j = 0; j < L; ++j)
                    {
                        acc[j] &= v[j];
                    }
                    break;
                case reduce_bit_or:
#pragma unroll
                    for (int j = 0; j < L; ++j)
                    {
                        acc[j] |= v[j];
                    }
                    break;
                case reduce_bit_xor:
#pragma unroll
                    for (int j = 0; j < L; ++j)
                    {
                        acc[j] ^= v[j];
                    }
                    break;
                default:
                {
                    const int c = compare<L>(v, acc);
                    if (op == reduce_min ? c < 0 : c > 0)
                    {
#pragma unroll
                        for (int j = 0; j < L; ++j)
                        {
                            acc[j] = v[j];
                        }
                    }
                    break;
                }
                }
                acc[L - 1] &= top_mask;
            }
        }
    };

    // One level of a two-level reduction: each thread folds a grid-strided
    // share of the elements in registers (four consecutive elements per
    // 128-bit load of each limb plane when `vectorised`: elements % 4 == 0 and
    // 16-byte aligned planes), then the block folds across its warps by
    // shuffles and shared memory and block j writes its value to element j of
    // `out` (limb-planar, out_elements = the number of blocks).  The second
    // level is this kernel on the block values with one block.  The operations
    // are associative and commutative on exact values, so the grouping does
    // not change the result.
    template<int L, bool Mod>
    __global__ void __launch_bounds__(256) reduce_kernel(uint32_t* out, uint64_t out_elements, const uint32_t* in,
                                                         uint64_t elements, bool vectorised,
                                                         const Reducer<L, Mod> red)
    {
        __shared__ uint32_t part[L][8];
        const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
        const uint64_t tid = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
        const uint64_t threads = static_cast<uint64_t>(gridDim.x) * blockDim.x;
        uint32_t acc[L], v[L];
        red.identity(acc);
        if (vectorised)
        {
            for (uint64_t e = tid * vec; e < elements; e += threads * vec)
            {
                uint32_t x[vec][L];
                load4<L>(x, in, elements, e);
#pragma unroll
                for (int k = 0; k < vec; ++k)
                {
                    if constexpr (!Mod)
                    {
                        x[k][L - 1] &= red.top_mask;
                    }
                    red.combine(acc, x[k]);
                }
            }
        }
        else
        {
            for (uint64_t e = tid; e < elements; e += threads)
            {
                load1<L>(v, in, elements, e);
                if constexpr (!Mod)
                {
                    v[L - 1] &= red.top_mask;
                }
                red.combine(acc, v);
            }
        }
#pragma unroll
        for (int off = 16; off > 0; off >>= 1)
        {
#pragma unroll
            for (int j = 0; j < L; ++j)
            {
                v[j] = __shfl_xor_sync(0xffffffffu, acc[j], off);
            }
            red.combine(acc, v);
        }
        if (lane == 0)
        {
#pragma unroll
            for (int j = 0; j < L; ++j)
            {
                part[j][warp] = acc[j];
            }
        }
        __syncthreads();
        if (warp == 0)
        {
            const uint32_t warps = blockDim.x >> 5;
            if (lane < warps)
            {
#pragma unroll
                for (int j = 0; j < L; ++j)
                {
                    acc[j] = part[j][lane];
                }
            }
            else
            {
                red.identity(acc);
            }
#pragma unroll
            for (int off = 4; off > 0; off >>= 1)
            {
#pragma unroll
                for (int j = 0; j < L; ++j)
                {
                    v[j] = __shfl_xor_sync(0xffffffffu, acc[j], off);
                }
                red.combine(acc, v);
            }
            if (lane == 0)
            {
                store1<L>(out, out_elements, blockIdx.x, acc);
            }
        }
    }

    // out[e] = 1 if every limb of a[e] and b[e] agrees, else 0: the hmpc::bit
    // of x == y (expr/binary_expression.hpp with core/equal_to.hpp)
    template<int L>
    __global__ void __launch_bounds__(256) equal_kernel(uint32_t* out, const uint32_t* a, const uint32_t* b,
                                                        uint64_t elements)
    {
        for (uint64_t e = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x; e < elements;
             e += static_cast<uint64_t>(gridDim.x) * blockDim.x)
        {
            uint32_t eq = 1u;
#pragma unroll
            for (int j = 0; j < L; ++j)
            {
                eq &= a[static_cast<uint64_t>(j) * elements + e] == b[static_cast<uint64_t>(j) * elements + e];
            }
            out[e] = eq;
        }
    }
}
