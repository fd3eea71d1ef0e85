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
// are carried as double-floats.  Absolute error ~1e-13 (the e^3/6 term of sin e in FP32).
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
#define DF_DIV(a, b) __fdiv_rn(a, b)
#define DF_BITS(a) __float_as_int(a)
__device__ __forceinline__ float df_rcp_approx(float a)
{
    float r;
    asm("rcp.approx.f32 %0, %1;" : "=f"(r) : "f"(a));
    return r;
}
#define DF_RCP_APPROX(a) df_rcp_approx(a)
#define DD_ADD(a, b) __dadd_rn(a, b)
#define DD_SUB(a, b) __dsub_rn(a, b)
#define DD_MUL(a, b) __dmul_rn(a, b)
#define DD_FMA(a, b, c) __fma_rn(a, b, c)
#else
static inline float df_h_add(float a, float b) { volatile float r = a + b; return r; }
static inline float df_h_sub(float a, float b) { volatile float r = a - b; return r; }
static inline float df_h_mul(float a, float b) { volatile float r = a * b; return r; }
static inline float df_h_rcp(float a) { volatile float r = 1.0f / a; return r; }
static inline float df_h_div(float a, float b) { volatile float r = a / b; return r; }
static inline int df_h_bits(float a) { int i; memcpy(&i, &a, 4); return i; }
#define DF_ADD(a, b) df_h_add(a, b)
#define DF_SUB(a, b) df_h_sub(a, b)
#define DF_MUL(a, b) df_h_mul(a, b)
#define DF_FMA(a, b, c) fmaf(a, b, c)
#define DF_RCP(a) df_h_rcp(a)
#define DF_DIV(a, b) df_h_div(a, b)
#define DF_RCP_APPROX(a) df_h_rcp(a)
static inline double dd_h_add(double a, double b) { volatile double r = a + b; return r; }
static inline double dd_h_sub(double a, double b) { volatile double r = a - b; return r; }
static inline double dd_h_mul(double a, double b) { volatile double r = a * b; return r; }
#define DD_ADD(a, b) dd_h_add(a, b)
#define DD_SUB(a, b) dd_h_sub(a, b)
#define DD_MUL(a, b) dd_h_mul(a, b)
#define DD_FMA(a, b, c) fma(a, b, c)
#define DF_BITS(a) df_h_bits(a)
#endif

namespace ast {

// Single operations with their rounding spelled out.  Code built from these gives the same bits
// wherever the compiler inlines it: a free expression such as a*b + c*d may be fused into a
// multiply-add on either product, and which one can depend on the surrounding kernel.
AST_HD float f_dot2(float a, float b, float c, float d) { return DF_FMA(a, b, DF_MUL(c, d)); }   // ab + cd
AST_HD float f_dif2(float a, float b, float c, float d) { return DF_FMA(a, b, -DF_MUL(c, d)); }  // ab - cd
AST_HD float f_dot3(float a, float b, float c, float d, float e, float f)
{
    return DF_FMA(a, b, DF_FMA(c, d, DF_MUL(e, f)));
}
AST_HD double d_dot2(double a, double b, double c, double d) { return DD_FMA(a, b, DD_MUL(c, d)); }
AST_HD double d_dif2(double a, double b, double c, double d) { return DD_FMA(a, b, -DD_MUL(c, d)); }

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

// ------------------------------------------------ cheaper forms for the integrator
//
// The right-hand side and the Runge-Kutta stage updates need an absolute error of a few u^2
// (u = 2^-24) of their operands' magnitudes, not a relative error of the result, so they use
// the sloppy sum (absolute error <= 2u^2 (|x| + |y|), Joldes et al. Alg. 4 analysis), a product
// without the lo*lo term, and a quotient with a single Newton correction (relative error ~4u^2).

AST_HD df df_sub_fast(df x, df y) { return df_add_fast(x, df_neg(y)); }

// x*y without the lo*lo term (DWTimesDW1 of Joldes et al.).
AST_HD df df_mul_fast(df x, df y)
{
    const df c = two_prod(x.hi, y.hi);
    const float t = DF_FMA(x.lo, y.hi, DF_FMA(x.hi, y.lo, c.lo));
    return fast_two_sum(c.hi, t);
}

// y + c*k in one pass: the exact product of the high words, the cross terms folded into its
// error, then a sloppy sum.
AST_HD df df_mad(df y, df c, df k)
{
    const float p = DF_MUL(c.hi, k.hi);
    const float pe = DF_FMA(c.lo, k.hi, DF_FMA(c.hi, k.lo, DF_FMA(c.hi, k.hi, -p)));
    const df s = two_sum(y.hi, p);
    const float v = DF_ADD(DF_ADD(y.lo, pe), s.lo);
    return fast_two_sum(s.hi, v);
}

// x / y with one Newton correction of the FP32 quotient.  The reciprocal may be the hardware
// approximation (relative error ~2^-23): the correction removes its error to first order.
AST_HD df df_div_fast(df x, df y)
{
    const float inv = DF_RCP_APPROX(y.hi);
    const float q1 = DF_MUL(x.hi, inv);
    // r = x - y*q1: the high part is exact (fma), the rest carries the low words.
    const float rh = DF_FMA(-y.hi, q1, x.hi);
    const float r = DF_FMA(-y.lo, q1, DF_ADD(rh, x.lo));
    return fast_two_sum(q1, DF_MUL(r, inv));
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
    // e = a - k * (2pi/TABLE), 2pi/TABLE = C1 + C2 + C3 as three floats.  a.hi - k*C1 is exact
    // in one fma (Cody-Waite with a fused multiply-add): both are multiples of ulp(C1) = 2^-29
    // and |a.hi - k*C1| < 2^-5 for |a.hi| <= 65536, so the difference has at most 24 bits.
    const float C1 = 0.02454369328916073f;      // float(2pi/256)
    const float C2 = -6.829904419802801e-10f;   // float(2pi/256 - C1)
    const float C3 = -2.6798820468841904e-17f;  // float(2pi/256 - C1 - C2)
    const float e0 = DF_FMA(-k, C1, a.hi);
    df e = two_sum(e0, a.lo);
    e = df_sub_fast(e, two_prod(k, C2));
    e = df_add_f(e, -DF_MUL(k, C3));
    // sin e = e - e^3/6 (1 - e^2/20 + e^4/840), cos e = 1 - d with d = e^2/2 - e^4/24 (1 - e^2/30).
    const float e1 = e.hi;
    const float e2 = DF_MUL(e1, e1);
    const float q = DF_MUL(DF_MUL(e2, 1.0f / 6.0f), DF_FMA(e2, DF_FMA(e2, 1.0f / 840.0f, -1.0f / 20.0f), 1.0f));
    // e^3/6 ~ e1^3/6 + e1^2 e.lo / 2: the second term keeps the low word of e in sin e.
    const df sig = df_add_f(e, -DF_FMA(0.5f * e2, e.lo, DF_MUL(e1, q)));  // sin e
    // cos e = 1 - e^2/2 + tail as a double-float: 1 - h with h exact to ~u^2.
    const float h2 = DF_MUL(e1, e1);
    const float h2l = DF_FMA(2.0f * e1, e.lo, DF_FMA(e1, e1, -h2));
    const float e4 = DF_MUL(e2, e2);
    const float tail = DF_MUL(DF_MUL(e4, 1.0f / 24.0f), DF_FMA(e2, -1.0f / 30.0f, 1.0f));
    const df c0 = fast_two_sum(1.0f, -0.5f * h2);  // exact: |h2/2| < 2^-10
    const df ce = fast_two_sum(c0.hi, DF_ADD(c0.lo, DF_FMA(-0.5f, h2l, tail)));  // cos e
    const float4 T = table[idx];
    const df S{T.x, T.y}, C{T.z, T.w};
    // sin a = S cos e + C sin e ; cos a = C cos e - S sin e
    *s_out = df_add_fast(df_mul_fast(S, ce), df_mul_fast(C, sig));
    *c_out = df_sub_fast(df_mul_fast(C, ce), df_mul_fast(S, sig));
}

// ------------------------------------------------ packed pairs
//
// df2 holds two double-floats side by side, (hi.x + lo.x) and (hi.y + lo.y).  Each operation
// below is its scalar namesake applied to both lanes, with the same roundings in the same order,
// so a lane's result is bit for bit the scalar one.  On the device a pair is one packed FP32x2
// instruction (add/mul/fma .rn.f32x2 of sm_100 and later, the __fadd2_rn family): one issue slot
// for two lanes of arithmetic, where the FP32 pipe itself processes the same number of lanes
// either way.  A negated operand folds into the packed instruction.  Every packed product below
// either is exact or has a second use, except the sincos table index, which is scalar (see
// df2_sincos).  On the host the lanes are computed one after the other.
struct df2 {
    float2 hi, lo;
};

AST_HD float2 f2(float a) { return make_float2(a, a); }
AST_HD float2 f2_neg(float2 a) { return make_float2(-a.x, -a.y); }
AST_HD float2 f2_add(float2 a, float2 b)
{
#if defined(__CUDA_ARCH__) && __CUDA_ARCH__ >= 1000
    return __fadd2_rn(a, b);
#else
    return make_float2(DF_ADD(a.x, b.x), DF_ADD(a.y, b.y));
#endif
}
AST_HD float2 f2_sub(float2 a, float2 b) { return f2_add(a, f2_neg(b)); }
AST_HD float2 f2_mul(float2 a, float2 b)
{
#if defined(__CUDA_ARCH__) && __CUDA_ARCH__ >= 1000
    return __fmul2_rn(a, b);
#else
    return make_float2(DF_MUL(a.x, b.x), DF_MUL(a.y, b.y));
#endif
}
AST_HD float2 f2_fma(float2 a, float2 b, float2 c)
{
#if defined(__CUDA_ARCH__) && __CUDA_ARCH__ >= 1000
    return __ffma2_rn(a, b, c);
#else
    return make_float2(DF_FMA(a.x, b.x, c.x), DF_FMA(a.y, b.y, c.y));
#endif
}

AST_HD df2 df2_pack(df a, df b) { return df2{make_float2(a.hi, b.hi), make_float2(a.lo, b.lo)}; }
AST_HD df df2_x(df2 a) { return df{a.hi.x, a.lo.x}; }
AST_HD df df2_y(df2 a) { return df{a.hi.y, a.lo.y}; }
AST_HD df2 df2_neg(df2 a) { return df2{f2_neg(a.hi), f2_neg(a.lo)}; }

AST_HD df2 two_sum2(float2 a, float2 b)
{
    const float2 s = f2_add(a, b);
    const float2 bb = f2_sub(s, a);
    return df2{s, f2_add(f2_sub(a, f2_sub(s, bb)), f2_sub(b, bb))};
}
AST_HD df2 fast_two_sum2(float2 a, float2 b)
{
    const float2 s = f2_add(a, b);
    return df2{s, f2_sub(b, f2_sub(s, a))};
}
AST_HD df2 two_prod2(float2 a, float2 b)
{
    const float2 p = f2_mul(a, b);
    return df2{p, f2_fma(a, b, f2_neg(p))};
}
AST_HD df2 df2_add_fast(df2 x, df2 y)
{
    const df2 s = two_sum2(x.hi, y.hi);
    return fast_two_sum2(s.hi, f2_add(x.lo, f2_add(y.lo, s.lo)));
}
AST_HD df2 df2_sub_fast(df2 x, df2 y) { return df2_add_fast(x, df2_neg(y)); }
AST_HD df2 df2_add_f(df2 x, float2 y)
{
    const df2 s = two_sum2(x.hi, y);
    return fast_two_sum2(s.hi, f2_add(x.lo, s.lo));
}
AST_HD df2 df2_mul_fast(df2 x, df2 y)
{
    const df2 c = two_prod2(x.hi, y.hi);
    return fast_two_sum2(c.hi, f2_fma(x.lo, y.hi, f2_fma(x.hi, y.lo, c.lo)));
}
AST_HD df2 df2_mad(df2 y, df2 c, df2 k)
{
    const float2 p = f2_mul(c.hi, k.hi);
    const float2 pe = f2_fma(c.lo, k.hi, f2_fma(c.hi, k.lo, f2_fma(c.hi, k.hi, f2_neg(p))));
    const df2 s = two_sum2(y.hi, p);
    return fast_two_sum2(s.hi, f2_add(f2_add(y.lo, pe), s.lo));
}

// sin and cos of two double-float angles at once: df_sincos lane by lane.
AST_HD void df2_sincos(df2 a, const float4* __restrict__ table, df2* s_out, df2* c_out)
{
    if (fabsf(a.hi.x) > 65536.0f || fabsf(a.hi.y) > 65536.0f) {
        const df ax = fabsf(a.hi.x) > 65536.0f ? df_reduce_2pi(df2_x(a)) : df2_x(a);
        const df ay = fabsf(a.hi.y) > 65536.0f ? df_reduce_2pi(df2_y(a)) : df2_y(a);
        a = df2_pack(ax, ay);
    }
    const float inv_step = (float)(kTrigTable / (2.0 * 3.14159265358979323846));
    const float magic = 12582912.0f;
    // The table index in scalar operations: the compiler contracts a packed product whose only use
    // is a packed add into one fused multiply-add, even written as mul.rn.f32x2 and add.rn.f32x2
    // (measured on sm_103a), and the fused round(a*c + m) picks the neighbouring table point
    // where a*c lies within its rounding error of a half-integer.  Scalar .rn operations are
    // never merged, so k is the scalar df_sincos's.
    const float2 kb = make_float2(DF_ADD(DF_MUL(a.hi.x, inv_step), magic), DF_ADD(DF_MUL(a.hi.y, inv_step), magic));
    const float2 k = f2_sub(kb, f2(magic));
    const float4 T0 = table[DF_BITS(kb.x) & (kTrigTable - 1)];
    const float4 T1 = table[DF_BITS(kb.y) & (kTrigTable - 1)];
    const float2 e0 = f2_fma(f2_neg(k), f2(0.02454369328916073f), a.hi);
    df2 e = two_sum2(e0, a.lo);
    e = df2_sub_fast(e, two_prod2(k, f2(-6.829904419802801e-10f)));
    e = df2_add_f(e, f2_neg(f2_mul(k, f2(-2.6798820468841904e-17f))));
    const float2 e1 = e.hi;
    const float2 e2 = f2_mul(e1, e1);
    const float2 q = f2_mul(f2_mul(e2, f2(1.0f / 6.0f)),
                            f2_fma(e2, f2_fma(e2, f2(1.0f / 840.0f), f2(-1.0f / 20.0f)), f2(1.0f)));
    const df2 sig = df2_add_f(e, f2_neg(f2_fma(f2_mul(f2(0.5f), e2), e.lo, f2_mul(e1, q))));
    const float2 h2l = f2_fma(f2_mul(f2(2.0f), e1), e.lo, f2_fma(e1, e1, f2_neg(e2)));
    const float2 e4 = f2_mul(e2, e2);
    const float2 tail = f2_mul(f2_mul(e4, f2(1.0f / 24.0f)), f2_fma(e2, f2(-1.0f / 30.0f), f2(1.0f)));
    const df2 c0 = fast_two_sum2(f2(1.0f), f2_mul(f2(-0.5f), e2));
    const df2 ce = fast_two_sum2(c0.hi, f2_add(c0.lo, f2_fma(f2(-0.5f), h2l, tail)));
    const df2 S{make_float2(T0.x, T1.x), make_float2(T0.y, T1.y)};
    const df2 C{make_float2(T0.z, T1.z), make_float2(T0.w, T1.w)};
    *s_out = df2_add_fast(df2_mul_fast(S, ce), df2_mul_fast(C, sig));
    *c_out = df2_sub_fast(df2_mul_fast(C, ce), df2_mul_fast(S, sig));
}

// ------------------------------------------------ sqrt, atan2, log

// sqrt(x), x >= 0: the FP32 root corrected once with the double-float residual.
AST_HD df df_sqrt(df x)
{
    if (!(x.hi > 0.0f)) return df{x.hi == 0.0f ? 0.0f : sqrtf(x.hi), 0.0f};
    const float s0 = sqrtf(x.hi);
    const df p = two_prod(s0, s0);
    const float d = DF_ADD(DF_SUB(DF_SUB(x.hi, p.hi), p.lo), x.lo);
    return fast_two_sum(s0, DF_MUL(d, DF_MUL(0.5f, DF_RCP_APPROX(s0))));
}

// atan2(y, x): the FP32 angle t0 corrected by delta = atan((y cos t0 - x sin t0) / (x cos t0 +
// y sin t0)) ~ the quotient itself (|delta| ~ 1e-7, so the cubic term is far below u^2).
AST_HD df df_atan2(df y, df x, const float4* __restrict__ table)
{
    const float t0 = atan2f(y.hi, x.hi);
    df s, c;
    df_sincos(df{t0, 0.0f}, table, &s, &c);
    const df num = df_sub(df_mul(y, c), df_mul(x, s));
    const df den = df_add(df_mul(x, c), df_mul(y, s));
    const float delta = den.hi != 0.0f ? num.hi / den.hi : 0.0f;
    return two_sum(t0, delta);
}

// Natural logarithm, x > 0: x = 2^e m with m in [1/sqrt2, sqrt2), log m = 2 atanh(r),
// r = (m - 1) / (m + 1), |r| <= 0.1716; the series 2r (1 + z/3 + z^2/5 + z^3 p(z)), z = r^2,
// carries its first three terms as double-floats and the tail p in FP32 (absolute error of the
// result ~1e-14).
AST_HD df df_log(df x)
{
    int e;
    float m = frexpf(x.hi, &e);
    if (m < 0.70710678f) {
        m = 2.0f * m;
        e = e - 1;
    }
    const float mlo = ldexpf(x.lo, -e);
    const df num = two_sum(DF_SUB(m, 1.0f), mlo);  // m - 1 is exact for m in [0.5, 2]
    const df den = df_add_f(df{m, mlo}, 1.0f);
    const df r = df_div(num, den);
    const df z = df_mul(r, r);
    const float zf = z.hi;
    const float p = DF_FMA(zf, DF_FMA(zf, DF_FMA(zf, DF_FMA(zf, DF_FMA(zf, DF_FMA(zf, 1.0f / 19.0f, 1.0f / 17.0f),
                                                                         1.0f / 15.0f), 1.0f / 13.0f), 1.0f / 11.0f),
                                      1.0f / 9.0f), 1.0f / 7.0f);
    const df C5{0.2f, -2.9802323e-09f};       // 1/5
    const df C3{0.33333334f, -9.934108e-09f};  // 1/3
    df w = df_add_f(C5, DF_MUL(zf, p));
    w = df_add(C3, df_mul(z, w));
    w = df_add_f(df_mul(z, w), 1.0f);
    const df lm = df_mul(df{2.0f * r.hi, 2.0f * r.lo}, w);
    const df LN2{0.6931472f, -1.9046542e-09f};
    return df_add(df_mul_f(LN2, (float)e), lm);
}

}  // namespace ast
