// Test program: the packed FP32x2 RK4 step of the mixed path (rk4_step_df2, ode_*_df2, df2_sincos
// in the product's headers) against a scalar restatement of the same step on random states, on the
// GPU, bit for bit.  Each lane of a packed operation must perform exactly the scalar operation:
// the compiler may not fuse a packed product into the next packed add (ptxas does so for a
// single-use product even when both are .rn PTX), so this check catches such a contraction, or a
// lane mix-up, anywhere in the step.  Usage: packed_step_check [states per configuration]; prints
// one line per configuration and exits 1 on any mismatch.
#include <cstdio>
#include <cstdlib>
#include <cuda_runtime.h>
#include "engine.cuh"
#include "mixed.cuh"

using namespace ast;

namespace {

// ---- the scalar step: the same operations on unpacked double-floats (one angle at a time)

__device__ void s_sincos2(df a0, df a1, const float4* tab, df* s0, df* c0, df* s1, df* c1)
{
    df_sincos(a0, tab, s0, c0);
    df_sincos(a1, tab, s1, c1);
}

__device__ void s_torque(const df* y, df* f, const df* mu, const float4* tab)
{
    df s5, c5, s4, c4;
    s_sincos2(y[5], y[4], tab, &s5, &c5, &s4, &c4);
    f[0] = df_add_fast(df_mul_fast(df_mul_fast(mu[0], y[1]), y[2]), mu[3]);
    f[1] = df_add_fast(df_mul_fast(df_mul_fast(mu[1], y[2]), y[0]), mu[4]);
    f[2] = df_add_fast(df_mul_fast(df_mul_fast(mu[2], y[0]), y[1]), mu[5]);
    f[3] = df_div_fast(df_add_fast(df_mul_fast(y[0], s5), df_mul_fast(y[1], c5)), s4);
    f[4] = df_sub_fast(df_mul_fast(y[0], c5), df_mul_fast(y[1], s5));
    f[5] = df_sub_fast(y[2], df_mul_fast(f[3], c4));
}

__device__ void s_free(const df* y, df* f, const df* mu, const float4* tab)
{
    df s2, c2, s1, c1;
    s_sincos2(df{DF_MUL(2.0f, y[2].hi), DF_MUL(2.0f, y[2].lo)}, y[1], tab, &s2, &c2, &s1, &c1);
    f[0] = df_mul_fast(mu[0], df_sub_fast(mu[1], df_mul_fast(mu[2], c2)));
    f[1] = df_mul_fast(df_mul_fast(df_mul_fast(mu[0], mu[2]), s1), s2);
    f[2] = df_mul_fast(c1, df_sub_fast(mu[0], f[0]));
}

template <int NODE>
__device__ void s_step(df* y, float4 hq, float4 hw, const df* mu, const float4* tab)
{
    df f[NODE], K[NODE], acc[NODE];
    for (int j = 0; j < NODE; j++) {
        f[j] = y[j];
        acc[j] = df{0.0f, 0.0f};
    }
    for (int st = 0; st < 4; st++) {
        if (NODE == 6) s_torque(f, K, mu, tab); else s_free(f, K, mu, tab);
        const float w = (st == 1 || st == 2) ? 2.0f : 1.0f;
        for (int j = 0; j < NODE; j++) acc[j] = df_add_fast(acc[j], df{DF_MUL(w, K[j].hi), DF_MUL(w, K[j].lo)});
        if (st < 3) {
            const df c = st < 2 ? df{hq.z, hq.w} : df{hq.x, hq.y};
            for (int j = 0; j < NODE; j++) f[j] = df_mad(y[j], c, K[j]);
        }
    }
    const df h6{hw.x, hw.y};
    for (int j = 0; j < NODE; j++) y[j] = df_mad(y[j], h6, acc[j]);
}

// ---- random states

__device__ uint32_t mix(uint32_t x)
{
    x ^= x >> 16; x *= 0x7feb352du; x ^= x >> 15; x *= 0x846ca68bu; x ^= x >> 16;
    return x;
}
__device__ float unit(uint32_t h) { return (float)(mix(h) >> 8) * (1.0f / 16777216.0f); }
// A double-float of random sign with |value| log-uniform in [2^lo, 2^hi] and a random low word.
__device__ df random_df(uint32_t h, float lo, float hi)
{
    const float m = exp2f(lo + (hi - lo) * unit(h));
    const float v = (mix(h + 9u) & 1u) ? -m : m;
    return fast_two_sum(v, DF_MUL(v, DF_MUL(2.9802322e-8f, unit(h + 3u) - 0.5f)));
}
__device__ bool differ(df a, df b)
{
    return __float_as_uint(a.hi) != __float_as_uint(b.hi) || __float_as_uint(a.lo) != __float_as_uint(b.lo);
}

// bad[0] sin/cos, [1] torque right-hand side, [2] torque step, [3] free right-hand side, [4] free step.
__global__ void check(unsigned long long* bad, int n, float angle_exp, float rate_exp, uint32_t seed)
{
    __shared__ float4 tab[kTrigTable];
    trig_table_fill(tab);
    __syncthreads();
    const df H = df_from_double(0.01), H2 = df_from_double(0.005), H6 = df_from_double(0.01 / 6),
             H3 = df_from_double(0.01 / 3);
    const float4 hq = make_float4(H.hi, H.lo, H2.hi, H2.lo), hw = make_float4(H6.hi, H6.lo, H3.hi, H3.lo);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint32_t s = mix((uint32_t)i * 2654435761u ^ seed);
        df y[6], mu[6];
        for (int j = 0; j < 3; j++) y[j] = random_df(s + 17u * j, -4.0f, rate_exp);
        for (int j = 3; j < 6; j++) y[j] = random_df(s + 17u * j, -6.0f, angle_exp);
        for (int j = 0; j < 3; j++) mu[j] = random_df(s + 101u + 13u * j, -3.0f, 0.0f);
        for (int j = 3; j < 6; j++) mu[j] = random_df(s + 101u + 13u * j, -3.0f, 3.3f);
        {
            df s5, c5, s4, c4;
            s_sincos2(y[5], y[4], tab, &s5, &c5, &s4, &c4);
            df2 S, C;
            df2_sincos(df2_pack(y[5], y[4]), tab, &S, &C);
            if (differ(s5, df2_x(S)) || differ(s4, df2_y(S)) || differ(c5, df2_x(C)) || differ(c4, df2_y(C)))
                atomicAdd(&bad[0], 1ull);
        }
        {
            df f[6];
            s_torque(y, f, mu, tab);
            df2 Y[3] = {df2_pack(y[0], y[1]), df2_pack(y[2], y[3]), df2_pack(y[5], y[4])}, F[3];
            ode_torque_df2(Y, F, mu, tab);
            if (differ(f[0], df2_x(F[0])) || differ(f[1], df2_y(F[0])) || differ(f[2], df2_x(F[1])) ||
                differ(f[3], df2_y(F[1])) || differ(f[5], df2_x(F[2])) || differ(f[4], df2_y(F[2])))
                atomicAdd(&bad[1], 1ull);
            df z[6];
            for (int j = 0; j < 6; j++) z[j] = y[j];
            s_step<6>(z, hq, hw, mu, tab);
            rk4_step_df2<6>(Y, hq, hw, mu, tab);
            if (differ(z[0], df2_x(Y[0])) || differ(z[1], df2_y(Y[0])) || differ(z[2], df2_x(Y[1])) ||
                differ(z[3], df2_y(Y[1])) || differ(z[5], df2_x(Y[2])) || differ(z[4], df2_y(Y[2])))
                atomicAdd(&bad[2], 1ull);
        }
        {
            df w[3] = {y[3], y[4], y[5]}, f[3];  // (phi, theta, psi)
            s_free(w, f, mu, tab);
            df2 Y[2] = {df2_pack(w[2], w[1]), df2_pack(w[0], df{0.0f, 0.0f})}, F[2];
            ode_free_df2(Y, F, mu, tab);
            if (differ(f[2], df2_x(F[0])) || differ(f[1], df2_y(F[0])) || differ(f[0], df2_x(F[1])))
                atomicAdd(&bad[3], 1ull);
            s_step<3>(w, hq, hw, mu, tab);
            rk4_step_df2<3>(Y, hq, hw, mu, tab);
            if (differ(w[2], df2_x(Y[0])) || differ(w[1], df2_y(Y[0])) || differ(w[0], df2_x(Y[1])))
                atomicAdd(&bad[4], 1ull);
        }
    }
}

}  // namespace

int main(int argc, char** argv)
{
    const int n = argc > 1 ? atoi(argv[1]) : (1 << 20);
    int sms = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, 0) != cudaSuccess) return 2;
    unsigned long long* bad = nullptr;
    if (cudaMalloc(&bad, 5 * sizeof(unsigned long long)) != cudaSuccess) return 2;
    const char* what[5] = {"sincos", "torque_rhs", "torque_step", "free_rhs", "free_step"};
    unsigned long long total = 0;
    const float angles[3] = {2.0f, 12.0f, 20.0f}, rates[3] = {4.0f, 10.0f, 17.0f};
    for (float ae : angles)
        for (float re : rates) {
            cudaMemset(bad, 0, 5 * sizeof(unsigned long long));
            check<<<sms * 4, 128>>>(bad, n, ae, re, 0x5eedu ^ (uint32_t)(ae * 131.0f + re));
            unsigned long long h[5];
            if (cudaMemcpy(h, bad, sizeof h, cudaMemcpyDeviceToHost) != cudaSuccess) return 2;
            printf("angles <= 2^%g rad, rates <= 2^%g rad/day, %d states:", ae, re, n);
            for (int j = 0; j < 5; j++) {
                printf(" %s %llu", what[j], h[j]);
                total += h[j];
            }
            printf("\n");
        }
    cudaFree(bad);
    if (cudaGetLastError() != cudaSuccess) return 2;
    return total ? 1 : 0;
}
