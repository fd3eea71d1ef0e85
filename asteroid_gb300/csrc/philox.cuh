// philox.cuh -- Philox4x32-10 counter-based generator (Salmon, Moraes, Dror, Shaw, "Parallel
// random numbers: as easy as 1, 2, 3", SC'11).  Chains draw their random start from
// (seed, chain, stage, draw index) alone, so a chain's result does not depend on which
// thread, launch or batch ran it.  The reference draws from per-thread cuRAND XORWOW states
// instead (cuda.c:1462,1519,1523, setup_kernel cuda.c:2039); start points are therefore
// distributed the same way but not identical draw for draw.
#pragma once
#include <stdint.h>

#ifndef AST_HD
#define AST_HD __host__ __device__ __forceinline__
#endif

namespace ast {

AST_HD void mulhilo32(uint32_t a, uint32_t b, uint32_t& hi, uint32_t& lo)
{
#ifdef __CUDA_ARCH__
    lo = a * b;
    hi = __umulhi(a, b);
#else
    uint64_t p = (uint64_t)a * (uint64_t)b;
    hi = (uint32_t)(p >> 32);
    lo = (uint32_t)p;
#endif
}

// Ten rounds with the published multipliers and Weyl key increments.
AST_HD void philox4x32_10(uint32_t c[4], uint32_t k0, uint32_t k1)
{
#pragma unroll
    for (int r = 0; r < 10; r++) {
        uint32_t hi0, lo0, hi1, lo1;
        mulhilo32(0xD2511F53u, c[0], hi0, lo0);
        mulhilo32(0xCD9E8D57u, c[2], hi1, lo1);
        uint32_t n0 = hi1 ^ c[1] ^ k0, n2 = hi0 ^ c[3] ^ k1;
        c[0] = n0; c[1] = lo1; c[2] = n2; c[3] = lo0;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
}

// Draw k of stream (seed, chain, stage): uniform float in (0,1), ((u >> 8) + 0.5) * 2^-24,
// exact in float, so host and device agree bit for bit.
AST_HD float uniform01(uint64_t seed, uint64_t chain, uint32_t stage, uint32_t k)
{
    uint32_t c[4] = {k >> 2, stage, (uint32_t)chain, (uint32_t)(chain >> 32)};
    philox4x32_10(c, (uint32_t)seed, (uint32_t)(seed >> 32));
    uint32_t u = c[k & 3];
    return ((float)(u >> 8) + 0.5f) * (1.0f / 16777216.0f);
}

// Four standard normals from one Philox block (counter ctr of stream (seed, domain, stream)):
// the Box-Muller transform (Box & Muller 1958) of the block's two pairs of uniforms, in float
// as curand_normal is.  Host and device use their own logf / sin / cos, so the two agree to a
// few float ulps, not bit for bit.
AST_HD void normal4(uint64_t seed, uint64_t stream, uint32_t domain, uint32_t ctr, float z[4])
{
    uint32_t c[4] = {ctr, domain, (uint32_t)stream, (uint32_t)(stream >> 32)};
    philox4x32_10(c, (uint32_t)seed, (uint32_t)(seed >> 32));
#pragma unroll
    for (int p = 0; p < 2; p++) {
        const float u1 = ((float)(c[2 * p] >> 8) + 0.5f) * (1.0f / 16777216.0f);
        const float u2 = ((float)(c[2 * p + 1] >> 8) + 0.5f) * (1.0f / 16777216.0f);
        const float r = sqrtf(-2.0f * logf(u1));
        float s, co;
#ifdef __CUDA_ARCH__
        sincospif(2.0f * u2, &s, &co);
#else
        s = sinf(6.2831853071795865f * u2);
        co = cosf(6.2831853071795865f * u2);
#endif
        z[2 * p] = r * co;
        z[2 * p + 1] = r * s;
    }
}

}  // namespace ast
