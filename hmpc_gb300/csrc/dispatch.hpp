// Kernel launch table, one per limb count L (1..9).  Each table is compiled
// in its own translation unit (kernels.cu with -DHMPC_L=<L>) so the builds
// run in parallel; the C-ABI layer picks the table by the modulus' L.
#pragma once

#include <cstdint>

#include <cuda_runtime.h>

#include "chacha.cuh"
#include "cluster.cuh"
#include "linalg.cuh"
#include "ntt.cuh"
#include "plain.cuh"
#include "tensor_ntt.cuh"

namespace hmpc_gb300
{
    constexpr int max_device_limbs = 9;
    constexpr int max_wide_words = 2 * max_device_limbs + 2;

    struct HostModulus
    {
        int limbs = 0;
        int bits = 0;
        uint32_t ninv = 0;
        uint32_t q[16] = {};
        uint32_t one[16] = {};
        uint32_t r2[16] = {};
        uint32_t half[16] = {};
    };

    // constants of a centred lift from a source modulus into the target one
    // (hmpc/ints/mod.hpp:259-307)
    struct CastParams
    {
        uint32_t src_limbs;
        uint32_t src_ninv;
        uint32_t src_q[max_device_limbs];
        uint32_t src_half[max_device_limbs];
        uint32_t offset[max_device_limbs + 1];  // added when the value exceeds src/2
        uint32_t norm_words;                      // words of value + offset
        uint32_t direct;                          // 1: value + offset < target Q
        uint32_t factor[max_device_limbs];        // R^2 (direct) or R'*R^2 mod Q
    };

    struct KernelTable
    {
        cudaError_t (*ntt_pass)(const NttPassParams& p, int kind, int nw, int radix_bits, const HostModulus& m,
                                unsigned grid, unsigned block, size_t smem, cudaStream_t stream);
        cudaError_t (*fma)(uint32_t* d, const uint32_t* a, const uint32_t* b, const uint32_t* c, uint64_t elements,
                           const HostModulus& m, cudaStream_t stream);
        cudaError_t (*binary)(uint32_t* out, const uint32_t* a, uint64_t a_elements, const uint32_t* b,
                              uint64_t b_elements, uint64_t elements, int op, const HostModulus& m,
                              cudaStream_t stream);
        cudaError_t (*lhe_combine)(uint32_t* out, const uint32_t* k, uint64_t n, const uint32_t* u,
                                   const uint32_t* v, const uint32_t* msg, uint64_t elements,
                                   const uint32_t* p_mont, const HostModulus& m, cudaStream_t stream);
        cudaError_t (*uniform)(uint32_t* out, uint64_t elements, const RngKey& rng, int words, uint32_t top_mask,
                               const HostModulus& m, cudaStream_t stream);
        cudaError_t (*cbd)(uint32_t* out, uint64_t elements, const RngKey& rng, uint32_t vx2,
                           const uint32_t* small_table, const HostModulus& m, cudaStream_t stream);
        cudaError_t (*to_montgomery)(uint32_t* out, const uint32_t* in, uint64_t elements, const HostModulus& m,
                                     cudaStream_t stream);
        cudaError_t (*from_montgomery)(uint32_t* out, const uint32_t* in, uint64_t elements, const HostModulus& m,
                                       cudaStream_t stream);
        cudaError_t (*cast)(uint32_t* out, const uint32_t* in, uint64_t elements, const CastParams& cp,
                            const HostModulus& m, cudaStream_t stream);
        cudaError_t (*plain_stage)(const PlainStageParams& p, int kind, int nw, const HostModulus& m,
                                   cudaStream_t stream);
        cudaError_t (*ct_mul)(uint32_t* d0, uint32_t* d1, uint32_t* d2, const uint32_t* a0, const uint32_t* a1,
                              const uint32_t* b0, const uint32_t* b1, uint64_t elements, const HostModulus& m,
                              cudaStream_t stream);
        cudaError_t (*dec_combine)(uint32_t* x, const uint32_t* s, uint64_t n, const uint32_t* c0,
                                   const uint32_t* c1, const uint32_t* c2, uint64_t elements, const HostModulus& m,
                                   cudaStream_t stream);
        // persistent batched transform with R = radix_bits register bits (2 or 3)
        cudaError_t (*ntt_batched)(const BatchedParams& bp, int radix_bits, const HostModulus& m, unsigned grid,
                                   size_t smem, cudaStream_t stream);
        int (*ntt_batched_blocks_per_sm)(int radix_bits, size_t smem);
        int radix_bits;
        cudaError_t (*lhe_combine_pair)(uint32_t* c0, uint32_t* c1, const uint32_t* ka, const uint32_t* kb,
                                        uint64_t n, const uint32_t* stacked, uint64_t elements,
                                        const HostModulus& m, cudaStream_t stream);
        // matrix-vector products (linalg.cuh)
        cudaError_t (*matvec)(uint32_t* z, const uint32_t* mat, const uint32_t* x, const MatvecParams& p,
                              const HostModulus& m, cudaStream_t stream);
        cudaError_t (*matvec_monomial)(uint32_t* z, const int64_t* degrees, const uint32_t* x,
                                       const MatvecParams& p, const HostModulus& m, cudaStream_t stream);
        // one level of a reduction into `grid` values (mod: mod<Q> with m, else uint with top_mask)
        cudaError_t (*reduce)(uint32_t* out, const uint32_t* in, uint64_t elements, int op, bool mod,
                              uint32_t top_mask, unsigned grid, const HostModulus& m, cudaStream_t stream);
        cudaError_t (*equal)(uint32_t* out, const uint32_t* a, const uint32_t* b, uint64_t elements,
                             cudaStream_t stream);
        // one thread-block cluster per polynomial (cluster.cuh), degrees 2^10..2^14
        cudaError_t (*ntt_cluster)(const ClusterNttParams& p, uint64_t batch, const HostModulus& m,
                                   cudaStream_t stream);
        // the uniform draws of a forward transform's stage-0 pairs as its input
        // (for the tensor-core engine, whose first group reads memory)
        cudaError_t (*uniform_pairs)(uint32_t* out, uint32_t log_n, uint64_t elements, const RngKey& rng,
                                     int words, uint32_t top_mask, const HostModulus& m, cudaStream_t stream);
    };

    // sizes of one tensor-core group kernel instantiation (TcShape)
    struct TcShapeInfo
    {
        uint32_t smem = 0, a_bytes = 0, b_bytes = 0, k_pad = 0, n_mma = 0, w_in = 0, w_out = 0, d_in = 0;
        uint32_t splits = 1;  // constant images per block (output elements split over them)
    };

    // tensor-core transform kernels of one limb count (2 to 8 limbs: 4L digits
    // per residue)
    struct TcKernels
    {
        int digits;
        // layout bit 0: the input digit planes are blocked per row, bit 1: the output
        // planes; bit 2: limb input / output through per-polynomial pointer tables
        cudaError_t (*group)(const TcGroupParams& p, int r, int in_kind, int out_kind, int splits, int layout,
                             unsigned grid, cudaStream_t stream);
        bool (*shape)(int r, int in_kind, int out_kind, int splits, TcShapeInfo& out);
        cudaError_t (*gen)(const TcGenParams& p, const HostModulus& m, cudaStream_t stream);
        cudaError_t (*expand)(const TcExpandParams& p, const HostModulus& m, cudaStream_t stream);
        // the first six forward stages of CBD-fed transforms as one group (tc_wide_kernel)
        cudaError_t (*combine6)(const TcCombineParams& p, const HostModulus& m, cudaStream_t stream);
        cudaError_t (*wide)(const TcGroupParams& p, unsigned grid, cudaStream_t stream);
    };

    const TcKernels* tc_kernels_2();
    const TcKernels* tc_kernels_3();
    const TcKernels* tc_kernels_4();
    const TcKernels* tc_kernels_5();
    const TcKernels* tc_kernels_6();
    const TcKernels* tc_kernels_7();
    const TcKernels* tc_kernels_8();

    inline const TcKernels* tc_kernels(int limbs)
    {
        switch (limbs)
        {
        case 2: return tc_kernels_2();
        case 3: return tc_kernels_3();
        case 4: return tc_kernels_4();
        case 5: return tc_kernels_5();
        case 6: return tc_kernels_6();
        case 7: return tc_kernels_7();
        case 8: return tc_kernels_8();
        default: return nullptr;
        }
    }

    const KernelTable* kernel_table_1();
    const KernelTable* kernel_table_2();
    const KernelTable* kernel_table_3();
    const KernelTable* kernel_table_4();
    const KernelTable* kernel_table_5();
    const KernelTable* kernel_table_6();
    const KernelTable* kernel_table_7();
    const KernelTable* kernel_table_8();
    const KernelTable* kernel_table_9();

    inline const KernelTable* kernel_table(int limbs)
    {
        switch (limbs)
        {
        case 1: return kernel_table_1();
        case 2: return kernel_table_2();
        case 3: return kernel_table_3();
        case 4: return kernel_table_4();
        case 5: return kernel_table_5();
        case 6: return kernel_table_6();
        case 7: return kernel_table_7();
        case 8: return kernel_table_8();
        case 9: return kernel_table_9();
        default: return nullptr;
        }
    }
}
