// C-ABI entry points of the matrix-vector products and reductions
// (kernels in linalg.cuh, launched through the per-limb-count tables).
#include "../../include/hmpc_gb300.h"

#include <algorithm>
#include <cstdint>

#include <cuda_runtime.h>

#include "dispatch.hpp"
#include "internal.hpp"

using namespace hmpc_gb300;
using namespace hmpc_gb300::detail;

namespace
{
    // blocks of the first reduction level: enough to fill the GPU several times
    // over, few enough that one block folds their values in the second level
    constexpr uint64_t reduce_blocks = 1024;

    bool mul_overflows(uint64_t a, uint64_t b, uint64_t& out)
    {
        return __builtin_mul_overflow(a, b, &out);
    }

    int shift_of(uint64_t v)
    {
        return v && (v & (v - 1)) == 0 ? __builtin_ctzll(v) : -1;
    }

    // Two launches: `grid` block values into the context's scratch, then one
    // block folds them into out (limb-planar with one element = L words).
    int run_reduce(hmpc_context* ctx, const KernelTable* kt, int limbs, int op, bool mod, uint32_t top_mask,
                   uint64_t elements, const uint32_t* in, uint32_t* out, const HostModulus& h)
    {
        const uint64_t grid = std::max<uint64_t>(1, std::min<uint64_t>(reduce_blocks, (elements + 255) / 256));
        cudaError_t e;
        if (grid == 1)
        {
            e = kt->reduce(out, in, elements, op, mod, top_mask, 1, h, ctx->stream);
            ++ctx->launches;
        }
        else
        {
            uint32_t* part = ctx->scratch(grid * static_cast<uint64_t>(limbs));
            if (!part)
            {
                return fail(HMPC_ERROR_OUT_OF_MEMORY, "allocating the reduction workspace");
            }
            e = kt->reduce(part, in, elements, op, mod, top_mask, static_cast<unsigned>(grid), h, ctx->stream);
            if (e == cudaSuccess)
            {
                e = kt->reduce(out, part, grid, op, mod, top_mask, 1, h, ctx->stream);
            }
            ctx->launches += 2;
        }
        return e == cudaSuccess ? HMPC_OK : cuda_fail(e, "launching reduction");
    }
}

int hmpc_matvec(hmpc_context* ctx, hmpc_modulus* mod, uint64_t batch, uint64_t rows, uint64_t cols, uint64_t coeffs,
                const uint32_t* m, uint64_t m_batch, const uint32_t* x, uint64_t x_batch, uint32_t* z)
{
    if (int rc = enter(ctx))
    {
        return rc;
    }
    if (!mod)
    {
        return fail(HMPC_ERROR_INVALID_ARGUMENT, "null modulus");
    }
    if ((m_batch != batch && m_batch != 1) || (x_batch != batch && x_batch != 1))
    {
        return fail(HMPC_ERROR_INVALID_ARGUMENT, "matrix and vector batches must be the output batch or 1");
    }
    MatvecParams p{};
    uint64_t row_elements, cells, m_per, x_per;
    if (mul_overflows(batch, rows, row_elements) || mul_overflows(row_elements, coeffs, p.total) ||
        mul_overflows(rows, cols, cells) || mul_overflows(cells, coeffs, m_per) ||
        mul_overflows(cols, coeffs, x_per) || mul_overflows(m_per, m_batch, p.m_elements) ||
        mul_overflows(x_per, x_batch, p.x_elements))
    {
        return fail(HMPC_ERROR_INVALID_ARGUMENT, "matrix-vector sizes overflow");
    }
    if (p.total == 0)
    {
        return HMPC_OK;
    }
    if (!z || (cols && (!m || !x)))
    {
        return fail(HMPC_ERROR_INVALID_ARGUMENT, "null tensor");
    }
    p.rows = rows;
    p.cols = cols;
    p.coeffs = coeffs;
    p.coeff_shift = shift_of(coeffs);
    p.m_bstride = m_batch == 1 ? 0 : m_per;
    p.x_bstride = x_batch == 1 ? 0 : x_per;
    cudaError_t e = mod->kt->matvec(z, m, x, p, mod->h, ctx->stream);
    ++ctx->launches;
    return e == cudaSuccess ? HMPC_OK : cuda_fail(e, "launching matrix-vector product");
}

int hmpc_matvec_monomial(hmpc_context* ctx, hmpc_modulus* mod, uint64_t n, uint64_t batch, uint64_t rows,
                         uint64_t cols, const int64_t* degrees, uint64_t d_batch, const uint32_t* x,
                         uint64_t x_batch, uint32_t* z)
{
    if (int rc = enter(ctx))
    {
        return rc;
    }
    if (!mod)
    {
        return fail(HMPC_ERROR_INVALID_ARGUMENT, "null modulus");
    }
    if (shift_of(n) < 0)
    {
        return fail(HMPC_ERROR_INVALID_ARGUMENT, "the degree of a bit monomial's ring must be a power of two");
    }
    if ((d_batch != batch && d_batch != 1) || (x_batch != batch && x_batch != 1))
    {
        return fail(HMPC_ERROR_INVALID_ARGUMENT, "degree and vector batches must be the output batch or 1");
    }
    MatvecParams p{};
    uint64_t row_elements, d_per, x_per;
    if (mul_overflows(batch, rows, row_elements) || mul_overflows(row_elements, n, p.total) ||
        mul_overflows(rows, cols, d_per) || mul_overflows(cols, n, x_per) ||
        mul_overflows(x_per, x_batch, p.x_elements) || mul_overflows(d_per, d_batch, p.m_elements))
    {
        return fail(HMPC_ERROR_INVALID_ARGUMENT, "matrix-vector sizes overflow");
    }
    if (p.total == 0)
    {
        return HMPC_OK;
    }
    if (!z || (cols && (!degrees || !x)))
    {
        return fail(HMPC_ERROR_INVALID_ARGUMENT, "null tensor");
    }
    p.rows = rows;
    p.cols = cols;
    p.coeffs = n;
    p.coeff_shift = shift_of(n);
    p.m_bstride = d_batch == 1 ? 0 : d_per;
    p.x_bstride = x_batch == 1 ? 0 : x_per;
    cudaError_t e = mod->kt->matvec_monomial(z, degrees, x, p, mod->h, ctx->stream);
    ++ctx->launches;
    return e == cudaSuccess ? HMPC_OK : cuda_fail(e, "launching bit-monomial matrix-vector product");
}

int hmpc_reduce(hmpc_context* ctx, hmpc_modulus* mod, int op, uint64_t elements, const uint32_t* in, uint32_t* out)
{
    if (int rc = enter(ctx))
    {
        return rc;
    }
    if (!mod || !out || (elements && !in))
    {
        return fail(HMPC_ERROR_INVALID_ARGUMENT, "null argument");
    }
    if (op != HMPC_REDUCE_ADD && op != HMPC_REDUCE_MULTIPLY)
    {
        return fail(HMPC_ERROR_INVALID_ARGUMENT, "residues reduce by HMPC_REDUCE_ADD or HMPC_REDUCE_MULTIPLY");
    }
    return run_reduce(ctx, mod->kt, mod->c.limbs, op, true, 0xffffffffu, elements, in, out, mod->h);
}

int hmpc_reduce_uint(hmpc_context* ctx, int op, int bits, uint64_t elements, const uint32_t* in, uint32_t* out)
{
    if (int rc = enter(ctx))
    {
        return rc;
    }
    if (!out || (elements && !in))
    {
        return fail(HMPC_ERROR_INVALID_ARGUMENT, "null argument");
    }
    if (op < HMPC_REDUCE_ADD || op > HMPC_REDUCE_MAX)
    {
        return fail(HMPC_ERROR_INVALID_ARGUMENT, "unknown reduction");
    }
    const int limbs = (bits + 31) / 32;
    const KernelTable* kt = bits >= 1 ? kernel_table(limbs) : nullptr;
    if (!kt)
    {
        return fail(HMPC_ERROR_UNSUPPORTED, "uint reductions take 1 to 288 bits");
    }
    const uint32_t top_mask = bits % 32 ? (1u << (bits % 32)) - 1u : 0xffffffffu;
    return run_reduce(ctx, kt, limbs, op, false, top_mask, elements, in, out, HostModulus{});
}

int hmpc_equal(hmpc_context* ctx, int limbs, uint64_t elements, const uint32_t* a, const uint32_t* b, uint32_t* out)
{
    if (int rc = enter(ctx))
    {
        return rc;
    }
    const KernelTable* kt = kernel_table(limbs);
    if (!kt)
    {
        return fail(HMPC_ERROR_UNSUPPORTED, "comparisons take 1 to 9 limbs");
    }
    if (elements == 0)
    {
        return HMPC_OK;
    }
    if (!a || !b || !out)
    {
        return fail(HMPC_ERROR_INVALID_ARGUMENT, "null tensor");
    }
    cudaError_t e = kt->equal(out, a, b, elements, ctx->stream);
    ++ctx->launches;
    return e == cudaSuccess ? HMPC_OK : cuda_fail(e, "launching comparison");
}
