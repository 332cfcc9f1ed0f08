// ChaCha20 stream cipher over tensors (hmpc/expr/crypto/cipher.hpp:59-319,
// hmpc/crypto/cipher.hpp:29-44): element i's limbs are XORed with keystream
// words i*L .. i*L+L-1 of ChaCha20(key, nonce, counter from 0) -- the
// reference cuts the words into batches of lcm(16, L), starting batch b's
// generator at counter b * lcm(16, L) / 16, which is the same as word w using
// word w % 16 of block w / 16.  Encryption reads a limb-planar tensor and
// writes element-major words (the reference's [elements..., L] limb tensor);
// decryption is the reverse.  One thread per keystream block; the block stays
// in registers.
#include <cstdint>

#include "chacha.cuh"
#include "internal.hpp"

namespace
{
    using hmpc_gb300::RngKey;

    __global__ void __launch_bounds__(256) cipher_kernel(const RngKey rng, uint64_t elements, uint32_t limbs,
                                                         const uint32_t* in, uint32_t* out, int decrypt)
    {
        const uint64_t words = elements * limbs;
        const uint64_t blocks = (words + 15) / 16;
        for (uint64_t k = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x; k < blocks;
             k += static_cast<uint64_t>(gridDim.x) * blockDim.x)
        {
            uint32_t ks[16];
            hmpc_gb300::chacha20_block(rng, static_cast<uint32_t>(k), ks);
            uint64_t w = k * 16;
            uint64_t i = w / limbs;
            uint32_t j = static_cast<uint32_t>(w - i * limbs);
#pragma unroll
            for (int t = 0; t < 16; ++t)
            {
                if (w + t < words)
                {
                    if (!decrypt)
                    {
                        out[w + t] = in[static_cast<uint64_t>(j) * elements + i] ^ ks[t];
                    }
                    else
                    {
                        out[static_cast<uint64_t>(j) * elements + i] = in[w + t] ^ ks[t];
                    }
                }
                if (++j == limbs)
                {
                    j = 0;
                    ++i;
                }
            }
        }
    }

    int run_cipher(hmpc_context* ctx, const uint32_t key[8], const uint32_t nonce[3], uint64_t elements,
                   int limbs, const uint32_t* in, uint32_t* out, int decrypt)
    {
        using namespace hmpc_gb300::detail;
        if (int rc = enter(ctx))
        {
            return rc;
        }
        if (!key || !nonce || limbs <= 0 || (elements && (!in || !out)))
        {
            return fail(HMPC_ERROR_INVALID_ARGUMENT, "null argument or no limbs");
        }
        if (elements == 0)
        {
            return HMPC_OK;
        }
        const uint64_t blocks = (elements * static_cast<uint64_t>(limbs) + 15) / 16;
        if (blocks > (1ull << 32))
        {
            return fail(HMPC_ERROR_UNSUPPORTED, "more keystream blocks than the 32-bit block counter holds");
        }
        RngKey rng{};
        for (int i = 0; i < 8; ++i)
        {
            rng.key[i] = key[i];
        }
        for (int i = 0; i < 3; ++i)
        {
            rng.nonce[i] = nonce[i];
        }
        const uint64_t grid = (blocks + 255) / 256;
        cipher_kernel<<<static_cast<unsigned>(grid < 152ull * 64 ? grid : 152ull * 64), 256, 0, ctx->stream>>>(
            rng, elements, static_cast<uint32_t>(limbs), in, out, decrypt);
        const cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess)
        {
            return cuda_fail(e, "launching the cipher");
        }
        ++ctx->launches;
        return HMPC_OK;
    }
}

extern "C" {

int hmpc_cipher_enc(hmpc_context* ctx, const uint32_t key[8], const uint32_t nonce[3], uint64_t elements, int limbs,
                    const uint32_t* planar_in, uint32_t* flat_out)
{
    return run_cipher(ctx, key, nonce, elements, limbs, planar_in, flat_out, 0);
}

int hmpc_cipher_dec(hmpc_context* ctx, const uint32_t key[8], const uint32_t nonce[3], uint64_t elements, int limbs,
                    const uint32_t* flat_in, uint32_t* planar_out)
{
    return run_cipher(ctx, key, nonce, elements, limbs, flat_in, planar_out, 1);
}

}  // extern "C"
