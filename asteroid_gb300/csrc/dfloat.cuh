// dfloat.cuh -- double-float ("double-FP32") arithmetic for the mixed-precision path.
//
// A value is an unevaluated sum hi + lo of two floats with |lo| <= ulp(hi)/2, about 48 bits of
// significand.  Every operation is a short sequence of FP32 instructions, so it runs on the FP32
// pipe (64x the FP64 rate on GB300).  Building blocks are the published error-free transforms:
// TwoSum (Knuth, TAOCP vol. 2), Fast2Sum (Dekker 1971), TwoProd through a fused multiply-add,
// and the double-word algorithms of Joldes, Muller and Popescu, "Tight and rigorous error bounds
// for basic building blocks of double-word arithmetic", ACM TOMS 44 (2017): add (their
// Algorithm 6 "AccurateDWPlusDW" and the cheaper Algorithm 4 where operands cannot cancel),
// multiply (Algorithm 12, DWTimesDW3) and divide (a Newton correction of the FP32 quotient).
//
// sincos of a double-float angle: Cody-Waite reduction by 2*pi/TABLE with a three-float
// constant, a TABLE-point table of sin/cos of k*2*pi/TABLE held as double-floats in shared
// memory, and short series for the remainder |e| <= pi/TABLE, in which only the leading terms
// are carried as double-floats.  Absolute error ~1e-14 for angles up to ~1e5 rad.
#pragma once
#include <math.h>
#include <stdint.h>

namespace ast {

struct df {
    float hi, lo;
};

__device__ __forceinline__ df df_make(float hi, float lo) { return df{hi, lo}; }
__host__ __device__ __forceinline__ df df_from_double(double d)
{
    const float hi = (float)d;
    return df{hi, (float)(d - (double)hi)};
}
__device__ __forceinline__ double df_to_double(df a) { return (double)a.hi + (double)a.lo; }

// Knuth TwoSum: s + e == a + b exactly.
__device__ __forceinline__ df two_sum(float a, float b)
{
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    return df{s, e};
}
// Dekker Fast2Sum, |a| >= |b|.
__device__ __forceinline__ df fast_two_sum(float a, float b)
{
    const float s = __fadd_rn(a, b);
    return df{s, __fsub_rn(b, __fsub_rn(s, a))};
}
// TwoProd with an FMA: p + e == a * b exactly.
__device__ __forceinline__ df two_prod(float a, float b)
{
    const float p = __fmul_rn(a, b);
    return df{p, __fmaf_rn(a, b, -p)};
}

// AccurateDWPlusDW (Joldes et al. 2017, Alg. 6): relative error <= 3u^2 for any operands.
__device__ __forceinline__ df df_add(df x, df y)
{
    df s = two_sum(x.hi, y.hi);
    const df t = two_sum(x.lo, y.lo);
    float c = __fadd_rn(s.lo, t.hi);
    df v = fast_two_sum(s.hi, c);
    const float w = __fadd_rn(t.lo, v.lo);
    return fast_two_sum(v.hi, w);
}
__device__ __forceinline__ df df_neg(df x) { return df{-x.hi, -x.lo}; }
__device__ __forceinline__ df df_sub(df x, df y) { return df_add(x, df_neg(y)); }

// SloppyDWPlusDW (Alg. 4): accurate unless x and y nearly cancel; for same-sign sums.
__device__ __forceinline__ df df_add_fast(df x, df y)
{
    const df s = two_sum(x.hi, y.hi);
    const float v = __fadd_rn(x.lo, __fadd_rn(y.lo, s.lo));
    return fast_two_sum(s.hi, v);
}

// DW + float (Alg. 4 of Joldes et al., DWPlusFP).
__device__ __forceinline__ df df_add_f(df x, float y)
{
    const df s = two_sum(x.hi, y);
    const float v = __fadd_rn(x.lo, s.lo);
    return fast_two_sum(s.hi, v);
}

// DWTimesDW3 (Alg. 12): relative error <= 4u^2.
__device__ __forceinline__ df df_mul(df x, df y)
{
    const df c = two_prod(x.hi, y.hi);
    float t = __fmul_rn(x.lo, y.lo);
    t = __fmaf_rn(x.hi, y.lo, t);
    t = __fmaf_rn(x.lo, y.hi, t);
    const float cl = __fadd_rn(c.lo, t);
    return fast_two_sum(c.hi, cl);
}

// DW times FP (DWTimesFP3 style).
__device__ __forceinline__ df df_mul_f(df x, float y)
{
    const df c = two_prod(x.hi, y);
    const float cl = __fmaf_rn(x.lo, y, c.lo);
    return fast_two_sum(c.hi, cl);
}

// x / y: FP32 quotient corrected once with the double-float residual.
__device__ __forceinline__ df df_div(df x, df y)
{
    const float inv = __frcp_rn(y.hi);
    const float q1 = __fmul_rn(x.hi, inv);
    const df r = df_sub(x, df_mul_f(y, q1));
    const float q2 = __fmul_rn(r.hi, inv);
    df q = fast_two_sum(q1, q2);
    // one more correction keeps ~46 bits when y.hi's reciprocal is rounded
    const df r2 = df_sub(x, df_mul(y, q));
    return df_add_f(q, __fmul_rn(r2.hi, inv));
}

// y + a * x for df y, x and df scalar a (the RK4 stage combination).
__device__ __forceinline__ df df_fma(df a, df x, df y) { return df_add(y, df_mul(a, x)); }

// ---------------------------------------------------------------- sincos

constexpr int kTrigTable = 256;  // table points over one turn

// The table lives in shared memory: float4 (sin_hi, sin_lo, cos_hi, cos_lo) per point.
struct TrigTable {
    const float4* t;
};

// Fill the table (call from every thread of the CTA, then __syncthreads()).  Values are the
// FP64 sin/cos of k * 2*pi / kTrigTable split into double-floats.
__device__ __forceinline__ void trig_table_fill(float4* t)
{
    for (int k = threadIdx.x; k < kTrigTable; k += blockDim.x) {
        double s, c;
        sincospi(2.0 * k / kTrigTable, &s, &c);
        const df S = df_from_double(s), Cc = df_from_double(c);
        t[k] = make_float4(S.hi, S.lo, Cc.hi, Cc.lo);
    }
}

// a - 2*pi*round(a / 2*pi) for |a| < 2^22 * 2*pi, with a three-float 2*pi.
__device__ __forceinline__ df df_reduce_2pi(df a)
{
    const float magic = 12582912.0f;
    const float k = __fsub_rn(__fadd_rn(__fmul_rn(a.hi, 0.159154943091895335768883763373f), magic), magic);
    df e = df_sub(a, two_prod(k, 6.2831854820251465f));
    e = df_sub(e, two_prod(k, -1.7484555314695172e-07f));
    return df_add_f(e, -__fmul_rn(k, -6.8604980400235275e-15f));
}

// sin and cos of the double-float angle a (absolute error < 1e-13 for |a| < 2e7).
__device__ __forceinline__ void df_sincos(df a, const float4* __restrict__ table, df* s_out, df* c_out)
{
    // Very long phases are first brought into [-pi, pi] so that k below stays under 2^22.
    if (fabsf(a.hi) > 65536.0f) a = df_reduce_2pi(a);
    // k = round(a * TABLE / 2pi) with the 1.5*2^23 trick (exact for |k| < 2^22); the low
    // mantissa bits of the biased sum are k mod 2^22, so k mod TABLE is a mask.
    const float inv_step = (float)(kTrigTable / (2.0 * 3.14159265358979323846));
    const float magic = 12582912.0f;
    const float kb = __fadd_rn(__fmul_rn(a.hi, inv_step), magic);
    const float k = __fsub_rn(kb, magic);
    const int idx = __float_as_int(kb) & (kTrigTable - 1);
    // e = a - k * (2pi/TABLE), 2pi/TABLE = C1 + C2 + C3 as three floats.
    const float C1 = 0.02454369328916073f;      // float(2pi/256)
    const float C2 = -6.829904419802801e-10f;   // float(2pi/256 - C1)
    const float C3 = -2.6798820468841904e-17f;  // float(2pi/256 - C1 - C2)
    df e = df_sub(a, two_prod(k, C1));
    e = df_sub(e, two_prod(k, C2));
    e = df_add_f(e, -__fmul_rn(k, C3));
    // sin e = e - e^3/6 (1 - e^2/20 + e^4/840), cos e = 1 - d with d = e^2/2 - e^4/24 (1 - e^2/30).
    const float e1 = e.hi;
    const float e2 = __fmul_rn(e1, e1);
    const float q = __fmul_rn(__fmul_rn(e2, 1.0f / 6.0f), __fmaf_rn(e2, __fmaf_rn(e2, 1.0f / 840.0f, -1.0f / 20.0f), 1.0f));
    // e^3/6 ~ e1^3/6 + e1^2 e.lo / 2: the second term keeps the low word of e in sin e.
    const df sig = df_add_f(e, -__fmaf_rn(0.5f * e2, e.lo, __fmul_rn(e1, q)));  // sin e
    df h2 = two_prod(e1, e1);                                        // e^2 as a double-float
    h2.lo = __fmaf_rn(2.0f * e1, e.lo, h2.lo);
    h2 = fast_two_sum(h2.hi, h2.lo);
    const float e4 = __fmul_rn(e2, e2);
    const float tail = __fmul_rn(__fmul_rn(e4, 1.0f / 24.0f), __fmaf_rn(e2, -1.0f / 30.0f, 1.0f));
    const df d = df_add_f(df{0.5f * h2.hi, 0.5f * h2.lo}, -tail);  // 1 - cos e
    const float4 T = table[idx];
    const df S{T.x, T.y}, Cc{T.z, T.w};
    // sin a = S - S d + C sin e ; cos a = C - C d - S sin e
    *s_out = df_add_fast(df_sub(S, df_mul(S, d)), df_mul(Cc, sig));
    *c_out = df_sub(df_sub(Cc, df_mul(Cc, d)), df_mul(S, sig));
}

// Angle reduced to [-pi, pi] as a float (for FP32 sin/cos in the brightness model).
__device__ __forceinline__ float df_reduce_f(df a)
{
    const float inv_2pi = 0.159154943091895335768883763373f;
    const float magic = 12582912.0f;
    const float k = __fsub_rn(__fadd_rn(__fmul_rn(a.hi, inv_2pi), magic), magic);
    const float C1 = 6.28318548202514648437500000000f;   // float(2pi)
    const float C2 = -1.74845553146951604103613980208e-07f;
    df e = df_sub(a, two_prod(k, C1));
    e = df_sub(e, two_prod(k, C2));
    return __fadd_rn(e.hi, e.lo);
}

}  // namespace ast
