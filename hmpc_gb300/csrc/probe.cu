// Rate probes of the benchmark: the integer-multiply throughput and the
// ChaCha20 block rate of the device, the denominators of the integer-pipe and
// integer-ALU rooflines (no vendor figure exists for 32-bit mad.lo / mad.hi or
// for the keystream on this part).  Built into libhmpc_gb300_probes.so, a
// measurement library beside the product library, not part of its C ABI.
#include <cstdint>

#include <cuda_runtime.h>

#include "chacha.cuh"

namespace hmpc_gb300
{
    namespace
    {
        constexpr int chains = 8;
        constexpr int iterations = 4096;

        // independent mad.lo / mad.hi chains: every instruction is a 32-bit
        // multiply-add, the mix the Montgomery products issue
        __global__ void __launch_bounds__(256) imad_kernel(uint32_t seed, uint32_t* sink)
        {
            uint32_t lo[chains], hi[chains];
            const uint32_t b = seed | 1u;
#pragma unroll
            for (int k = 0; k < chains; ++k)
            {
                lo[k] = threadIdx.x + k;
                hi[k] = blockIdx.x + 3u * k;
            }
            for (int i = 0; i < iterations; ++i)
            {
#pragma unroll
                for (int k = 0; k < chains; ++k)
                {
                    asm volatile("mad.lo.u32 %0, %0, %1, %2;" : "+r"(lo[k]) : "r"(b), "r"(hi[k]));
                    asm volatile("mad.hi.u32 %0, %0, %1, %2;" : "+r"(hi[k]) : "r"(b), "r"(lo[k]));
                }
            }
            uint32_t acc = 0;
#pragma unroll
            for (int k = 0; k < chains; ++k)
            {
                acc ^= lo[k] ^ hi[k];
            }
            if (acc == 0x12345678u)
            {
                sink[threadIdx.x] = acc;
            }
        }
    }

    namespace
    {
        constexpr int chacha_blocks_per_thread = 64;

        // ChaCha20 blocks as the samplers compute them: one block per
        // (key, nonce, counter), the first four output words consumed (a
        // stage-0 pair of CBD(10) draws).  The nonce changes every iteration so
        // that no quarter round of the first column round is loop-invariant
        // (a sampler thread computes one block, where none can be hoisted).
        __global__ void __launch_bounds__(256) chacha_kernel(RngKey k, uint32_t* sink)
        {
            const uint32_t counter0 = (blockIdx.x * blockDim.x + threadIdx.x) * chacha_blocks_per_thread;
            uint32_t acc = 0;
            for (int i = 0; i < chacha_blocks_per_thread; ++i)
            {
                RngKey ki = k;
                ki.nonce[0] += static_cast<uint32_t>(i);
                ki.nonce[1] ^= static_cast<uint32_t>(i) * 0x9e3779b9u;
                ki.nonce[2] += static_cast<uint32_t>(i) << 7;
                uint32_t out[16];
                chacha20_block(ki, counter0 + static_cast<uint32_t>(i), out);
                acc ^= out[0] ^ out[1] ^ out[2] ^ out[3];
            }
            if (acc == 0x12345678u)
            {
                sink[threadIdx.x] = acc;
            }
        }
    }

    cudaError_t probe_chacha_rate(cudaStream_t stream, double* blocks_per_second)
    {
        int device = 0, sms = 0;
        cudaError_t e = cudaGetDevice(&device);
        if (e == cudaSuccess)
        {
            e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
        }
        if (e != cudaSuccess)
        {
            return e;
        }
        uint32_t* sink = nullptr;
        if ((e = cudaMalloc(&sink, 256 * sizeof(uint32_t))) != cudaSuccess)
        {
            return e;
        }
        RngKey k{};
        for (int i = 0; i < 8; ++i)
        {
            k.key[i] = 0x01234567u * static_cast<uint32_t>(i + 1);
        }
        const unsigned blocks = static_cast<unsigned>(sms) * 8u;
        cudaEvent_t start, stop;
        cudaEventCreate(&start);
        cudaEventCreate(&stop);
        float best = 1e30f;
        for (int rep = 0; rep < 6; ++rep)
        {
            k.nonce[0] = static_cast<uint32_t>(rep);
            cudaEventRecord(start, stream);
            chacha_kernel<<<blocks, 256, 0, stream>>>(k, sink);
            cudaEventRecord(stop, stream);
            e = cudaEventSynchronize(stop);
            if (e != cudaSuccess)
            {
                break;
            }
            float ms = 0.f;
            cudaEventElapsedTime(&ms, start, stop);
            if (rep > 0 && ms < best)
            {
                best = ms;
            }
        }
        cudaEventDestroy(start);
        cudaEventDestroy(stop);
        cudaFree(sink);
        if (e != cudaSuccess)
        {
            return e;
        }
        const double count = static_cast<double>(blocks) * 256.0 * chacha_blocks_per_thread;
        *blocks_per_second = count / (static_cast<double>(best) * 1e-3);
        return cudaSuccess;
    }

    cudaError_t probe_int_multiply_rate(cudaStream_t stream, double* ops_per_second)
    {
        int device = 0, sms = 0;
        cudaError_t e = cudaGetDevice(&device);
        if (e == cudaSuccess)
        {
            e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
        }
        if (e != cudaSuccess)
        {
            return e;
        }
        uint32_t* sink = nullptr;
        if ((e = cudaMalloc(&sink, 256 * sizeof(uint32_t))) != cudaSuccess)
        {
            return e;
        }
        const unsigned blocks = static_cast<unsigned>(sms) * 8u;
        cudaEvent_t start, stop;
        cudaEventCreate(&start);
        cudaEventCreate(&stop);
        float best = 1e30f;
        for (int rep = 0; rep < 6; ++rep)
        {
            cudaEventRecord(start, stream);
            imad_kernel<<<blocks, 256, 0, stream>>>(0x9e3779b9u + rep, sink);
            cudaEventRecord(stop, stream);
            e = cudaEventSynchronize(stop);
            if (e != cudaSuccess)
            {
                break;
            }
            float ms = 0.f;
            cudaEventElapsedTime(&ms, start, stop);
            if (rep > 0 && ms < best)
            {
                best = ms;
            }
        }
        cudaEventDestroy(start);
        cudaEventDestroy(stop);
        cudaFree(sink);
        if (e != cudaSuccess)
        {
            return e;
        }
        const double ops = static_cast<double>(blocks) * 256.0 * iterations * chains * 2.0;
        *ops_per_second = ops / (static_cast<double>(best) * 1e-3);
        return cudaSuccess;
    }
}

// 32-bit multiply operations (mad.lo and mad.hi each count one) per second on
// the current device, timed on `stream`; 0 or the CUDA error code
extern "C" int hmpc_bench_int_multiply_rate(void* stream, double* ops_per_second)
{
    return static_cast<int>(hmpc_gb300::probe_int_multiply_rate(static_cast<cudaStream_t>(stream), ops_per_second));
}

// ChaCha20 blocks per second (20 rounds, four output words used) on the
// current device, timed on `stream`; 0 or the CUDA error code
extern "C" int hmpc_bench_chacha_rate(void* stream, double* blocks_per_second)
{
    return static_cast<int>(hmpc_gb300::probe_chacha_rate(static_cast<cudaStream_t>(stream), blocks_per_second));
}
