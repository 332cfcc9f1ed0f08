// Measured integer-multiply throughput of the device: the denominator of the
// integer-pipe roofline for the multi-limb kernels (no vendor figure exists
// for 32-bit mad.lo/mad.hi on this part).
#pragma once

#include <cuda_runtime.h>

namespace hmpc_gb300
{
    // 32-bit multiply operations (mad.lo and mad.hi each count one) per second
    cudaError_t probe_int_multiply_rate(cudaStream_t stream, double* ops_per_second);
    // ChaCha20 blocks per second (20 rounds, four output words used): the
    // denominator of the integer-ALU roofline of the fused samplers
    cudaError_t probe_chacha_rate(cudaStream_t stream, double* blocks_per_second);
}
