// kmc_common.cuh -- shared device helpers of the sm_103a hop-loop kernels.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/kmc_dn_gb300.h"

namespace kmc {

// ---------------------------------------------------------------------------
// Counter-based generator: Philox4x32-10 (Salmon, Moraes, Dror, Shaw,
// "Parallel random numbers: as easy as 1, 2, 3", SC'11).  Own restatement of
// the published round function; the multipliers and Weyl constants are the
// paper's.  Counter = (hop lo, hop hi, stream lo, stream hi), key = seed, so a
// chain's stream depends only on (seed, stream id, hop index) and not on where
// or in which launch the chain runs.
// ---------------------------------------------------------------------------
struct u32x4 { uint32_t x, y, z, w; };

__device__ __forceinline__ u32x4 philox4x32_10(u32x4 c, uint32_t k0, uint32_t k1)
{
    constexpr uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u;
    constexpr uint32_t W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        const uint32_t hi0 = __umulhi(M0, c.x), lo0 = M0 * c.x;
        const uint32_t hi1 = __umulhi(M1, c.z), lo1 = M1 * c.z;
        c = u32x4{hi1 ^ c.y ^ k0, lo1, hi0 ^ c.w ^ k1, lo0};
        k0 += W0;
        k1 += W1;
    }
    return c;
}

// Uniform in (0,1) from the top 23 bits: (k + 1/2) 2^-23, exact in FP32,
// so never 0 and at most 1 - 2^-24.
__device__ __forceinline__ float u01_from32(uint32_t x)
{
    return (static_cast<float>(x >> 9) + 0.5f) * (1.0f / 8388608.0f);
}

// Uniform in (0,1] for the clock's exponential variate: (x + 1/2) 2^-32
// rounded to FP32.  Near 0, where -log u is large, FP32 keeps every one of
// the 32 bits, so -log u reaches ln(2^33) = 22.9 and the exponential tail
// beyond it (mean weight e^-22.9 = 1e-10) is all that is cut.
__device__ __forceinline__ float u01_tail32(uint32_t x)
{
    return fmaf(static_cast<float>(x), 0x1.0p-32f, 0x1.0p-33f);
}

// Uniform in (0,1) with 53 random bits from two words.
__device__ __forceinline__ double u01_from64(uint32_t hi, uint32_t lo)
{
    const uint64_t v = ((static_cast<uint64_t>(hi) << 32) | lo) >> 11;
    return (static_cast<double>(v) + 0.5) * 0x1.0p-53;
}

// ---------------------------------------------------------------------------
// Batched-engine launch description (device pointers).  Mirrors struct
// kmc_batch of the C ABI; kept as the same layout.
// ---------------------------------------------------------------------------
using Batch = kmc_batch;

__device__ __forceinline__ bool finite_pos(double x) { return x > 0.0 && x < 1.0e300; }

}  // namespace kmc
