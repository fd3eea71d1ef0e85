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
// are carried as double-floats.  Absolute error < 1e-13 for angles up to ~2e7 rad.
//
// The same code compiles for the host (used to test the arithmetic against FP64): there the
// operations map to IEEE round-to-nearest float arithmetic (compile with -ffp-contract=off).
#pragma once
#include <math.h>
#include <stdint.h>
#include <string.h>

#ifndef AST_HD
#define AST_HD __host__ __device__ __forceinline__
#endif

#ifdef __CUDA_ARCH__
#define DF_ADD(a, b) __fadd_rn(a, b)
#define DF_SUB(a, b) __fsub_rn(a, b)
#define DF_MUL(a, b) __fmul_rn(a, b)
#define DF_FMA(a, b, c) __fmaf_rn(a, b, c)
#define DF_RCP(a) __frcp_rn(a)
#define DF_BITS(a) __float_as_int(a)
#else
static inline float df_h_add(float a, float b) { volatile float r = a + b; return r; }
static inline float df_h_sub(float a, float b) { volatile float r = a - b; return r; }
static inline float df_h_mul(float a, float b) { volatile float r = a * b; return r; }
static inline float df_h_rcp(float a) { volatile float r = 1.0f / a; return r; }
static inline int df_h_bits(float a) { int i; memcpy(&i, &a, 4); return i; }
#define DF_ADD(a, b) df_h_add(a, b)
#define DF_SUB(a, b) df_h_sub(a, b)
#define DF_MUL(a, b) df_h_mul(a, b)
#define DF_FMA(a, b, c) fmaf(a, b, c)
#define DF_RCP(a) df_h_rcp(a)
#define DF_BITS(a) df_h_bits(a)
#endif

namespace ast {

struct df {
    float hi, lo;
};

AST_HD df df_from_double(double d)
{
    const float hi = (float)d;
    return df{hi, (float)(d - (double)hi)};
}
AST_HD double df_to_double(df a) { return (double)a.hi + (double)a.lo; }

// Knuth TwoSum: s + e == a + b exactly.
AST_HD df two_sum(float a, float b)
{
    const float s = DF_ADD(a, b);
    const float bb = DF_SUB(s, a);
    const float e = DF_ADD(DF_SUB(a, DF_SUB(s, bb)), DF_SUB(b, bb));
    return df{s, e};
}
// Dekker Fast2Sum, |a| >= |b|.
AST_HD df fast_two_sum(float a, float b)
{
    const float s = DF_ADD(a, b);
    return df{s, DF_SUB(b, DF_SUB(s, a))};
}
// TwoProd with an FMA: p + e == a * b exactly.
AST_HD df two_prod(float a, float b)
{
    const float p = DF_MUL(a, b);
    return df{p, DF_FMA(a, b, -p)};
}

// AccurateDWPlusDW (Joldes et al. 2017, Alg. 6): relative error <= 3u^2 for any operands.
AST_HD df df_add(df x, df y)
{
    const df s = two_sum(x.hi, y.hi);
    const df t = two_sum(x.lo, y.lo);
    const float c = DF_ADD(s.lo, t.hi);
    const df v = fast_two_sum(s.hi, c);
    const float w = DF_ADD(t.lo, v.lo);
    return fast_two_sum(v.hi, w);
}
AST_HD df df_neg(df x) { return df{-x.hi, -x.lo}; }
AST_HD df df_sub(df x, df y) { return df_add(x, df_neg(y)); }

// SloppyDWPlusDW (Alg. 4): accurate unless x and y nearly cancel; for same-sign sums.
AST_HD df df_add_fast(df x, df y)
{
    const df s = two_sum(x.hi, y.hi);
    const float v = DF_ADD(x.lo, DF_ADD(y.lo, s.lo));
    return fast_two_sum(s.hi, v);
}

// DW + float (DWPlusFP).
AST_HD df df_add_f(df x, float y)
{
    const df s = two_sum(x.hi, y);
    const float v = DF_ADD(x.lo, s.lo);
    return fast_two_sum(s.hi, v);
}

// DWTimesDW3 (Alg. 12): relative error <= 4u^2.
AST_HD df df_mul(df x, df y)
{
    const df c = two_prod(x.hi, y.hi);
    float t = DF_MUL(x.lo, y.lo);
    t = DF_FMA(x.hi, y.lo, t);
    t = DF_FMA(x.lo, y.hi, t);
    const float cl = DF_ADD(c.lo, t);
    return fast_two_sum(c.hi, cl);
}

// DW times FP.
AST_HD df df_mul_f(df x, float y)
{
    const df c = two_prod(x.hi, y);
    const float cl = DF_FMA(x.lo, y, c.lo);
    return fast_two_sum(c.hi, cl);
}

// x / y: FP32 quotient corrected twice with double-float residuals.
AST_HD df df_div(df x, df y)
{
    const float inv = DF_RCP(y.hi);
    const float q1 = DF_MUL(x.hi, inv);
    const df r = df_sub(x, df_mul_f(y, q1));
    const float q2 = DF_MUL(r.hi, inv);
    const df q = fast_two_sum(q1, q2);
    const df r2 = df_sub(x, df_mul(y, q));
    return df_add_f(q, DF_MUL(r2.hi, inv));
}

// ---------------------------------------------------------------- sincos

constexpr int kTrigTable = 256;  // table points over one turn

// Table entry k: (sin_hi, sin_lo, cos_hi, cos_lo) of k * 2*pi / kTrigTable.
AST_HD float4 trig_table_entry(int k)
{
    double s, c;
#ifdef __CUDA_ARCH__
    sincospi(2.0 * k / kTrigTable, &s, &c);
#else
    s = sin(2.0 * 3.14159265358979323846 * k / kTrigTable);
    c = cos(2.0 * 3.14159265358979323846 * k / kTrigTable);
#endif
    const df S = df_from_double(s), C = df_from_double(c);
    float4 v;
    v.x = S.hi; v.y = S.lo; v.z = C.hi; v.w = C.lo;
    return v;
}

#ifdef __CUDACC__
// Fill the shared-memory table from every thread of the CTA (then __syncthreads()).
__device__ __forceinline__ void trig_table_fill(float4* t)
{
    for (int k = threadIdx.x; k < kTrigTable; k += blockDim.x) t[k] = trig_table_entry(k);
}
#endif

// a - 2*pi*round(a / 2*pi) for |a| < 2^22 * 2*pi, with a three-float 2*pi.
AST_HD df df_reduce_2pi(df a)
{
    const float magic = 12582912.0f;
    const float k = DF_SUB(DF_ADD(DF_MUL(a.hi, 0.159154943091895335768883763373f), magic), magic);
    df e = df_sub(a, two_prod(k, 6.2831854820251465f));
    e = df_sub(e, two_prod(k, -1.7484555314695172e-07f));
    return df_add_f(e, -DF_MUL(k, -6.8604980400235275e-15f));
}

// sin and cos of the double-float angle a.
AST_HD void df_sincos(df a, const float4* __restrict__ table, df* s_out, df* c_out)
{
    // Very long phases are first brought into [-pi, pi] so that k below stays under 2^22.
    if (fabsf(a.hi) > 65536.0f) a = df_reduce_2pi(a);
    // k = round(a * TABLE / 2pi) with the 1.5*2^23 trick (exact for |k| < 2^22); the low
    // mantissa bits of the biased sum are k mod 2^22, so k mod TABLE is a mask.
    const float inv_step = (float)(kTrigTable / (2.0 * 3.14159265358979323846));
    const float magic = 12582912.0f;
    const float kb = DF_ADD(DF_MUL(a.hi, inv_step), magic);
    const float k = DF_SUB(kb, magic);
    const int idx = DF_BITS(kb) & (kTrigTable - 1);
    // e = a - k * (2pi/TABLE), 2pi/TABLE = C1 + C2 + C3 as three floats.
    const float C1 = 0.02454369328916073f;      // float(2pi/256)
    const float C2 = -6.829904419802801e-10f;   // float(2pi/256 - C1)
    const float C3 = -2.6798820468841904e-17f;  // float(2pi/256 - C1 - C2)
    df e = df_sub(a, two_prod(k, C1));
    e = df_sub(e, two_prod(k, C2));
    e = df_add_f(e, -DF_MUL(k, C3));
    // sin e = e - e^3/6 (1 - e^2/20 + e^4/840), cos e = 1 - d with d = e^2/2 - e^4/24 (1 - e^2/30).
    const float e1 = e.hi;
    const float e2 = DF_MUL(e1, e1);
    const float q = DF_MUL(DF_MUL(e2, 1.0f / 6.0f), DF_FMA(e2, DF_FMA(e2, 1.0f / 840.0f, -1.0f / 20.0f), 1.0f));
    // e^3/6 ~ e1^3/6 + e1^2 e.lo / 2: the second term keeps the low word of e in sin e.
    const df sig = df_add_f(e, -DF_FMA(0.5f * e2, e.lo, DF_MUL(e1, q)));  // sin e
    df h2 = two_prod(e1, e1);                                            // e^2 as a double-float
    h2.lo = DF_FMA(2.0f * e1, e.lo, h2.lo);
    h2 = fast_two_sum(h2.hi, h2.lo);
    const float e4 = DF_MUL(e2, e2);
    const float tail = DF_MUL(DF_MUL(e4, 1.0f / 24.0f), DF_FMA(e2, -1.0f / 30.0f, 1.0f));
    const df d = df_add_f(df{0.5f * h2.hi, 0.5f * h2.lo}, -tail);  // 1 - cos e
    const float4 T = table[idx];
    const df S{T.x, T.y}, C{T.z, T.w};
    // sin a = S - S d + C sin e ; cos a = C - C d - S sin e
    *s_out = df_add_fast(df_sub(S, df_mul(S, d)), df_mul(C, sig));
    *c_out = df_sub(df_sub(C, df_mul(C, d)), df_mul(S, sig));
}

// Angle reduced to [-pi, pi] as a float (for FP32 sin/cos in the brightness model).
AST_HD float df_reduce_f(df a)
{
    const df e = df_reduce_2pi(a);
    return DF_ADD(e.hi, e.lo);
}

}  // namespace ast
