// mixed.cuh -- the mixed-precision chi^2.
//
// GB300 executes FP32 FMAs at 64x its FP64 rate, so the plain path (cuda.c's arithmetic, all
// FP64) is bound by the FP64 pipe.  Here the fixed-step RK4 of the Euler equations and Euler
// angles (cuda.c:13-77, 319-372) runs entirely on the FP32 pipe: the state, the stage
// combinations and the right-hand side (including sin/cos of the Euler angles) are double-float
// values (dfloat.cuh), ~48-bit significands, which keeps the integrated rotation phase (up to
// ~1e5 rad over a long light curve) accurate to ~1e-10 rad.  The brightness model at each
// observation (cuda.c:432-689) is evaluated in plain FP32 from the double-float angles reduced
// to [-pi, pi].  FP64 is left for the per-evaluation set-up (initial angles and angular
// velocity, cuda.c:195-252), the parameter-independent ephemeris interpolation (hoisted per
// object) and the per-filter sums and chi^2 (cuda.c:707-714, 887-910).
#pragma once
#include <math.h>
#include "dfloat.cuh"
#include "model.cuh"

namespace ast {

// f(t) = t - (1 - t^2) atanh(t) for 0 <= t < 1, without cancellation: for t < 1/2 the series
// sum_k 2 t^(2k+1) / ((2k-1)(2k+1)), else the closed form (cancellation at most 6x there).
AST_HD float ls_f(float t)
{
    const float t2 = DF_MUL(t, t);
    if (t < 0.5f) {
        float p = 2.0f / 575.0f;  // k = 12
        p = fmaf(p, t2, 2.0f / 483.0f);
        p = fmaf(p, t2, 2.0f / 399.0f);
        p = fmaf(p, t2, 2.0f / 323.0f);
        p = fmaf(p, t2, 2.0f / 255.0f);
        p = fmaf(p, t2, 2.0f / 195.0f);
        p = fmaf(p, t2, 2.0f / 143.0f);
        p = fmaf(p, t2, 2.0f / 99.0f);
        p = fmaf(p, t2, 2.0f / 63.0f);
        p = fmaf(p, t2, 2.0f / 35.0f);
        p = fmaf(p, t2, 2.0f / 15.0f);
        p = fmaf(p, t2, 2.0f / 3.0f);
        return DF_MUL(DF_MUL(p, t2), t);
    }
    const float om = DF_SUB(1.0f, t);
    return DF_SUB(t, DF_MUL(DF_MUL(DF_SUB(1.0f, t2), 0.5f), log1pf(DF_MUL(2.0f, t) / om)));
}

// Lommel-Seeliger ellipsoid magnitude, Muinonen & Lumme (2015) eqs. 10-14 as in cuda.c:664-689,
// rearranged for FP32.  Sp, Ep: unit Sun and Earth vectors in the body frame (b, c, a);
// ib = 1/b, ic = 1/c; bc = b*c.  Exact identities replace the two cancellations of the
// reference's form, which amplify FP32 rounding by up to ~(1/c)^2 for flattened bodies:
//  * scalar = |S' + E'| of the scaled vectors S' = (Sb/b, Sc/c, Sa), E' likewise, computed from
//    the body-frame half vector S + E instead of sqrt(sS^2 + sE^2 + 2 sS sE cos alpha');
//  * with mu = lambda', nu = alpha' - lambda' (each from atan2 of a cross and a dot product),
//    cos(lambda'-alpha') + cos lambda' + sin lambda' sin(lambda'-alpha') ln(cot(mu/2) cot(nu/2))
//    = 2 D^2 f(s/D), D = cos((mu - nu)/2), s = cos((mu + nu)/2), f as in ls_f.
AST_HD float ls_magnitude_f(float Sb, float Sc, float Sa, float Eb, float Ec, float Ea, float ib, float ic, float bc)
{
    const float sx = DF_MUL(Sb, ib), sy = DF_MUL(Sc, ic), sz = Sa;
    const float ex = DF_MUL(Eb, ib), ey = DF_MUL(Ec, ic), ez = Ea;
    const float hx = DF_MUL(DF_ADD(Sb, Eb), ib), hy = DF_MUL(DF_ADD(Sc, Ec), ic), hz = DF_ADD(Sa, Ea);
    const float sS = sqrtf(f_dot3(sx, sx, sy, sy, sz, sz));
    const float sE = sqrtf(f_dot3(ex, ex, ey, ey, ez, ez));
    const float scalar = sqrtf(f_dot3(hx, hx, hy, hy, hz, hz));
    const float cx = f_dif2(sy, ez, sz, ey), cy = f_dif2(sz, ex, sx, ez), cz = f_dif2(sx, ey, sy, ex);
    const float cn = sqrtf(f_dot3(cx, cx, cy, cy, cz, cz));  // |S' x E'| = |S' x H'| = |H' x E'|
    const float mu = atan2f(cn, f_dot3(sx, hx, sy, hy, sz, hz));
    const float nu = atan2f(cn, f_dot3(hx, ex, hy, ey, hz, ez));
    const float D = cosf(DF_MUL(0.5f, DF_SUB(mu, nu)));
    // s = cos(alpha'/2) = sin(eps/2) with eps = pi - alpha' taken directly from the vectors.
    const float s = sinf(DF_MUL(0.5f, atan2f(cn, -f_dot3(sx, ex, sy, ey, sz, ez))));
    const float B = DF_MUL(DF_MUL(DF_MUL(2.0f, D), D), ls_f(s / D));
    return DF_MUL(-2.5f, log10f(DF_MUL(DF_MUL(DF_MUL(bc, sS), sE) / scalar, B)));
}

// The rotation ODEs (cuda.c:13-77) in double-float, on the state in packed pairs (df2): the
// sin and cos of the two angles the right-hand side needs are one df2_sincos, its products and
// quotient are the scalar double-float operations on the pairs' halves.  Pair layout, torque:
// (y0, y1), (y2, phi), (psi, theta), where y0..y2 are the body-frame angular velocities of
// cuda.c:46-58; free rotation (cuda.c:69-75): (psi, theta), (phi, unused 0).  mu: torque
// ((Is-1)/Ii, (1-Ii)/Is, Ii-Is, Ti, Ts, Tl); free (L, Ip, Im).
AST_HD void ode_torque_df2(const df2* y, df2* f, const df* mu, const float4* tab)
{
    df2 s, c;
    df2_sincos(y[2], tab, &s, &c);  // (sin psi, sin theta), (cos psi, cos theta)
    const df y0 = df2_x(y[0]), y1 = df2_y(y[0]), y2 = df2_x(y[1]);
    const df s5 = df2_x(s), s4 = df2_y(s), c5 = df2_x(c), c4 = df2_y(c);
    const df f0 = df_add_fast(df_mul_fast(df_mul_fast(mu[0], y1), y2), mu[3]);
    const df f1 = df_add_fast(df_mul_fast(df_mul_fast(mu[1], y2), y0), mu[4]);
    const df f2 = df_add_fast(df_mul_fast(df_mul_fast(mu[2], y0), y1), mu[5]);
    const df f3 = df_div_fast(df_add_fast(df_mul_fast(y0, s5), df_mul_fast(y1, c5)), s4);
    const df f4 = df_sub_fast(df_mul_fast(y0, c5), df_mul_fast(y1, s5));
    const df f5 = df_sub_fast(y2, df_mul_fast(f3, c4));
    f[0] = df2_pack(f0, f1);
    f[1] = df2_pack(f2, f3);
    f[2] = df2_pack(f5, f4);
}

AST_HD void ode_free_df2(const df2* y, df2* f, const df* mu, const float4* tab)
{
    df2 s, c;  // of (2 psi, theta): doubling is exact
    df2_sincos(df2{f2_mul(y[0].hi, make_float2(2.0f, 1.0f)), f2_mul(y[0].lo, make_float2(2.0f, 1.0f))}, tab, &s, &c);
    const df s2 = df2_x(s), c2 = df2_x(c), s1 = df2_y(s), c1 = df2_y(c);
    const df dphi = df_mul_fast(mu[0], df_sub_fast(mu[1], df_mul_fast(mu[2], c2)));
    const df dtheta = df_mul_fast(df_mul_fast(df_mul_fast(mu[0], mu[2]), s1), s2);
    const df dpsi = df_mul_fast(c1, df_sub_fast(mu[0], dphi));
    f[0] = df2_pack(dpsi, dtheta);
    f[1] = df2_pack(dphi, df{0.0f, 0.0f});
}

// One RK4 step, y <- y + h/6 (K1 + 2 K2 + 2 K3 + K4) with K1..K4 at y, y + h/2 K1, y + h/2 K2,
// y + h K3 (cuda.c:319-372, the same combination), on the packed pairs of the ODE's layout
// (NODE = 6 torque, 3 free).  hq = (h, h/2), hw = (h/6, h/3) as double-floats.  The four stages
// run through a single right-hand-side call site (a rolled loop) and the stage derivatives are
// summed as they come (doubling is exact), so the hot loop is one copy of the right-hand side --
// small enough for the instruction cache -- and only one stage derivative is live at a time; the
// last stage needs no next-stage point.  Sums and products are the integrator forms of
// dfloat.cuh (absolute error a few u^2 of the operands), two components per instruction.
template <int NODE>
AST_HD void rk4_step_df2(df2* y, float4 hq, float4 hw, const df* mu, const float4* tab)
{
    constexpr int P = (NODE + 1) / 2;
    df2 f[P], K[P], acc[P];
#pragma unroll
    for (int j = 0; j < P; j++) {
        f[j] = y[j];
        acc[j] = df2{f2(0.0f), f2(0.0f)};
    }
#pragma unroll 1
    for (int st = 0; st < 4; st++) {
        if (NODE == 6) ode_torque_df2(f, K, mu, tab); else ode_free_df2(f, K, mu, tab);
        const float2 w = f2((st == 1 || st == 2) ? 2.0f : 1.0f);  // K1 + 2 K2 + 2 K3 + K4
#pragma unroll
        for (int j = 0; j < P; j++) acc[j] = df2_add_fast(acc[j], df2{f2_mul(w, K[j].hi), f2_mul(w, K[j].lo)});
        if (st < 3) {
            const df2 c = st < 2 ? df2{f2(hq.z), f2(hq.w)} : df2{f2(hq.x), f2(hq.y)};  // h/2, h/2, h
#pragma unroll
            for (int j = 0; j < P; j++) f[j] = df2_mad(y[j], c, K[j]);
        }
    }
    const df2 h6{f2(hw.x), f2(hw.y)};
#pragma unroll
    for (int j = 0; j < P; j++) y[j] = df2_mad(y[j], h6, acc[j]);
}

// ---------------------------------------------------------------- FP32 right-hand side
//
// AST_PREC_MIXED_RHS32: the right-hand side of the rotation ODEs (cuda.c:26-75) in FP32 from the
// double-float state rounded to float, the four stage derivatives K1..K4 in FP32, and the state
// advanced in double-float, y + h/6 K1 + h/3 K2 + h/3 K3 + h/6 K4, so that the rounding of the
// accumulated phase stays at u^2 while each step's increment carries the FP32 error of its
// derivatives (relative ~u of h*K per step).

// sin and cos of a float angle |a| <~ 4 from the shared-memory table: a = k 2pi/256 + e with
// |e| <= pi/256, sin e = e (1 - e^2/6), cos e = 1 - e^2/2 (truncation < 2e-10).
AST_HD void f_sincos_tab(float a, const float4* __restrict__ tab, float* s, float* c)
{
    const float inv_step = (float)(kTrigTable / (2.0 * 3.14159265358979323846));
    const float magic = 12582912.0f;
    const float kb = DF_ADD(DF_MUL(a, inv_step), magic);
    const float k = DF_SUB(kb, magic);
    const int idx = DF_BITS(kb) & (kTrigTable - 1);
    const float e = DF_FMA(-k, -6.829904419802801e-10f, DF_FMA(-k, 0.02454369328916073f, a));
    const float e2 = DF_MUL(e, e);
    const float se = DF_MUL(e, DF_FMA(e2, -1.0f / 6.0f, 1.0f));  // sin e
    const float hc = DF_MUL(0.5f, e2);                           // 1 - cos e
    const float4 T = tab[idx];
    *s = DF_FMA(T.z, se, DF_FMA(-T.x, hc, T.x));  // S cos e + C sin e
    *c = DF_FMA(-T.x, se, DF_FMA(-T.z, hc, T.z)); // C cos e - S sin e
}

// cuda.c:46-58 in FP32.  mu as in ode_torque_df2.
AST_HD void ode_torque_f32(const float* y, float* f, const float* mu, const float4* tab)
{
    float s5, c5, s4, c4;
    f_sincos_tab(y[5], tab, &s5, &c5);
    f_sincos_tab(y[4], tab, &s4, &c4);
    f[0] = DF_FMA(DF_MUL(mu[0], y[1]), y[2], mu[3]);
    f[1] = DF_FMA(DF_MUL(mu[1], y[2]), y[0], mu[4]);
    f[2] = DF_FMA(DF_MUL(mu[2], y[0]), y[1], mu[5]);
    f[3] = DF_DIV(f_dot2(y[0], s5, y[1], c5), s4);
    f[4] = f_dif2(y[0], c5, y[1], s5);
    f[5] = DF_FMA(-f[3], c4, y[2]);
}

// cuda.c:69-75 in FP32: mu = (L, Ip, Im, 1 - Ip); dpsi/dt = cos(theta) L (1 - Ip + Im cos 2psi)
// without the cancellation of L - dphi/dt.
AST_HD void ode_free_f32(const float* y, float* f, const float* mu, const float4* tab)
{
    float s2, c2, s1, c1;
    f_sincos_tab(DF_MUL(2.0f, y[2]), tab, &s2, &c2);
    f_sincos_tab(y[1], tab, &s1, &c1);
    f[0] = DF_MUL(mu[0], DF_FMA(-mu[2], c2, mu[1]));
    f[1] = DF_MUL(DF_MUL(DF_MUL(mu[0], mu[2]), s1), s2);
    f[2] = DF_MUL(DF_MUL(c1, mu[0]), DF_FMA(mu[2], c2, mu[3]));
}

// y + c*k, c a double-float, k a float (df_mad with a zero low word).
AST_HD df df_mad_f(df y, df c, float k)
{
    const float p = DF_MUL(c.hi, k);
    const float pe = DF_FMA(c.lo, k, DF_FMA(c.hi, k, -p));
    const df s = two_sum(y.hi, p);
    const float v = DF_ADD(DF_ADD(y.lo, pe), s.lo);
    return fast_two_sum(s.hi, v);
}

// One RK4 step with the FP32 right-hand side.  The angle psi is brought into [-pi, pi] first so
// that its float value (the argument of sin and cos) is accurate to u of pi; theta is bounded and
// phi does not enter the right-hand side.
template <int NODE>
AST_HD void rk4_step_f32(df* y, float4 hq, float4 hw, const float* mu, const float4* tab)
{
    constexpr int PSI = NODE == 6 ? 5 : 2;
    y[PSI] = df_reduce_2pi(y[PSI]);
    float f[NODE], K[NODE];
    df yn[NODE];
#pragma unroll
    for (int j = 0; j < NODE; j++) f[j] = DF_ADD(y[j].hi, y[j].lo);
#pragma unroll 1
    for (int st = 0; st < 4; st++) {
        if (NODE == 6) ode_torque_f32(f, K, mu, tab); else ode_free_f32(f, K, mu, tab);
        const float c = st < 2 ? hq.z : hq.x;                                      // h/2, h/2, h, h
        const df wgt = (st == 1 || st == 2) ? df{hw.z, hw.w} : df{hw.x, hw.y};   // h/6, h/3, h/3, h/6
#pragma unroll
        for (int j = 0; j < NODE; j++) {
            yn[j] = df_mad_f(st == 0 ? y[j] : yn[j], wgt, K[j]);
            f[j] = DF_ADD(y[j].hi, DF_FMA(c, K[j], y[j].lo));
        }
    }
#pragma unroll
    for (int j = 0; j < NODE; j++) y[j] = yn[j];
}

// ---------------------------------------------------------------- double-float magnitudes
//
// The NUDGE minimum candidates need model magnitudes far more accurate than FP32 (their
// parabola turns magnitude differences of ~1e-3 mag into the minimum's time).  They are
// evaluated here in double-float arithmetic on the FP32 pipe, ~1e-13 mag, rather than in FP64,
// which on GB300 runs at 1/64 of the FP32 rate.

AST_HD df df_dot3(const df* a, const df* b)
{
    return df_add(df_add(df_mul(a[0], b[0]), df_mul(a[1], b[1])), df_mul(a[2], b[2]));
}
AST_HD void df_cross3(const df* a, const df* b, df* c)
{
    c[0] = df_sub(df_mul(a[1], b[2]), df_mul(a[2], b[1]));
    c[1] = df_sub(df_mul(a[2], b[0]), df_mul(a[0], b[2]));
    c[2] = df_sub(df_mul(a[0], b[1]), df_mul(a[1], b[0]));
}

// f(t) = t - (1 - t^2) atanh(t), 0 <= t < 1 (ls_f in double-float): the series
// t^3 sum_{k>=1} 2 t^(2k-2) / ((2k-1)(2k+1)) below 1/4, the closed form above.
AST_HD df ls_f_df(df t)
{
    const df z = df_mul(t, t);
    if (t.hi < 0.25f) {
        const float zf = z.hi;
        float p = 2.0f / 899.0f;  // k = 15: 2 / (29 * 31)
        p = DF_FMA(p, zf, 2.0f / 783.0f);
        p = DF_FMA(p, zf, 2.0f / 675.0f);
        p = DF_FMA(p, zf, 2.0f / 575.0f);
        p = DF_FMA(p, zf, 2.0f / 483.0f);
        p = DF_FMA(p, zf, 2.0f / 399.0f);
        p = DF_FMA(p, zf, 2.0f / 323.0f);
        p = DF_FMA(p, zf, 2.0f / 255.0f);
        p = DF_FMA(p, zf, 2.0f / 195.0f);
        p = DF_FMA(p, zf, 2.0f / 143.0f);
        p = DF_FMA(p, zf, 2.0f / 99.0f);
        p = DF_FMA(p, zf, 2.0f / 63.0f);  // k = 4
        const df C2{0.057142857f, -3.193106e-10f};  // 2/35
        const df C1{0.13333334f, -6.9538753e-09f};  // 2/15
        const df C0{0.6666667f, -1.9868216e-08f};   // 2/3
        df w = df_add_f(C2, DF_MUL(zf, p));
        w = df_add(C1, df_mul(z, w));
        w = df_add(C0, df_mul(z, w));
        return df_mul(df_mul(z, t), w);
    }
    // atanh t = log((1 + t) / (1 - t)) / 2
    const df at = df_log(df_div(df_add_f(t, 1.0f), df_add_f(df_neg(t), 1.0f)));
    const df one_m_z = df_add_f(df_neg(z), 1.0f);
    return df_sub(t, df_mul(one_m_z, df{0.5f * at.hi, 0.5f * at.lo}));
}

// ls_magnitude_f in double-float: the same cancellation-free Lommel-Seeliger form.
AST_HD df ls_magnitude_df(const df* Sp, const df* Ep, df ib, df ic, df bc, const float4* tab)
{
    const df sv[3] = {df_mul(Sp[0], ib), df_mul(Sp[1], ic), Sp[2]};
    const df ev[3] = {df_mul(Ep[0], ib), df_mul(Ep[1], ic), Ep[2]};
    const df hv[3] = {df_mul(df_add(Sp[0], Ep[0]), ib), df_mul(df_add(Sp[1], Ep[1]), ic), df_add(Sp[2], Ep[2])};
    const df sS = df_sqrt(df_dot3(sv, sv));
    const df sE = df_sqrt(df_dot3(ev, ev));
    const df scalar = df_sqrt(df_dot3(hv, hv));
    df cr[3];
    df_cross3(sv, ev, cr);
    const df cn = df_sqrt(df_dot3(cr, cr));
    const df mu = df_atan2(cn, df_dot3(sv, hv), tab);
    const df nu = df_atan2(cn, df_dot3(hv, ev), tab);
    const df eps = df_atan2(cn, df_neg(df_dot3(sv, ev)), tab);
    df sd, D, s, cd;
    const df hmn = df_sub(mu, nu);
    df_sincos(df{0.5f * hmn.hi, 0.5f * hmn.lo}, tab, &sd, &D);
    df_sincos(df{0.5f * eps.hi, 0.5f * eps.lo}, tab, &s, &cd);
    const df B = df_mul(df_mul(df{2.0f * D.hi, 2.0f * D.lo}, D), ls_f_df(df_div(s, D)));
    const df arg = df_mul(df_div(df_mul(df_mul(bc, sS), sE), scalar), B);
    const df INV_LN10{0.4342945f, -1.010305e-08f};
    return df_mul_f(df_mul(df_log(arg), INV_LN10), -2.5f);
}

// Per-evaluation constants of the double-float magnitude: the spin-axis frame (cuda.c:195-217)
// and the shape or BW_BALL parameters.
struct DfFrame {
    df M[3], XM_x, XM_z, YM[3];
    df ib, ic, bc;
    df cR, sR, cT, sT, kappa;
};

// The per-evaluation constants of vmod_df for parameter vector params (cuda.c:195-217, 568-574).
AST_HD DfFrame make_df_frame(const DevModel& M, const double* params)
{
    const ast_type_ids& T = M.t;
#define AST_Q(tt) params[M.idx[T.tt]]
    const double th_M = AST_Q(theta_M), ph_M = AST_Q(phi_M);
    const double Mx = DD_MUL(sin(th_M), cos(ph_M)), My = DD_MUL(sin(th_M), sin(ph_M)), Mz = cos(th_M);
    const double XM = sqrt(d_dot2(Mz, Mz, Mx, Mx));
    const double XMx = Mz / XM, XMz = -Mx / XM;
    DfFrame F;
    F.M[0] = df_from_double(Mx);
    F.M[1] = df_from_double(My);
    F.M[2] = df_from_double(Mz);
    F.XM_x = df_from_double(XMx);
    F.XM_z = df_from_double(XMz);
    F.YM[0] = df_from_double(DD_MUL(My, XMz));
    F.YM[1] = df_from_double(d_dif2(Mz, XMx, Mx, XMz));
    F.YM[2] = df_from_double(-DD_MUL(My, XMx));
    if (M.flags & AST_BW_BALL) {
        F.kappa = df_from_double(AST_Q(kappa));
        F.cR = df_from_double(cos(AST_Q(phi_R)));
        F.sR = df_from_double(sin(AST_Q(phi_R)));
        F.cT = df_from_double(cos(AST_Q(theta_R)));
        F.sT = df_from_double(sin(AST_Q(theta_R)));
    } else {
        const double b = (M.flags & AST_BC) ? AST_Q(b) : AST_Q(b_tumb);
        const double c = (M.flags & AST_BC) ? AST_Q(c) : AST_Q(c_tumb);
        F.ib = df_from_double(1.0 / b);
        F.ic = df_from_double(1.0 / c);
        F.bc = df_from_double(DD_MUL(b, c));
    }
#undef AST_Q
    return F;
}

// Model magnitude at observation i for the double-float Euler angles ang = (phi, theta, psi):
// the body frame as in cuda.c:432-473, then ls_magnitude_df or the BW_BALL law (cuda.c:568-580).
AST_HD double vmod_df(const DevModel& M, const ObsView& o, const DfFrame& F, const df* ang, int i, const float4* tab)
{
    df sph, cph, sth, cth, sps, cps;
    df_sincos(ang[0], tab, &sph, &cph);
    df_sincos(ang[1], tab, &sth, &cth);
    df_sincos(ang[2], tab, &sps, &cps);
    const df N[3] = {df_add(df_mul(F.XM_x, cph), df_mul(F.YM[0], sph)), df_mul(F.YM[1], sph),
                     df_add(df_mul(F.XM_z, cph), df_mul(F.YM[2], sph))};
    df p[3];
    df_cross3(N, F.M, p);
    df a[3], w[3], b[3], c[3];
    for (int k = 0; k < 3; k++) a[k] = df_add(df_mul(F.M[k], cth), df_mul(p[k], sth));
    df_cross3(a, N, w);
    for (int k = 0; k < 3; k++) b[k] = df_add(df_mul(N[k], cps), df_mul(w[k], sps));
    df_cross3(a, b, c);
    const df E[3] = {df_from_double(o.ex[i]), df_from_double(o.ey[i]), df_from_double(o.ez[i])};
    if (M.flags & AST_BW_BALL) {
        df Nb[3], pb[3];
        for (int k = 0; k < 3; k++) Nb[k] = df_add(df_mul(b[k], F.cR), df_mul(c[k], F.sR));
        df_cross3(Nb, a, pb);
        for (int k = 0; k < 3; k++) a[k] = df_add(df_mul(a[k], F.cT), df_mul(pb[k], F.sT));
        const df cz = df_dot3(a, E);
        const df one_p = df_add_f(cz, 1.0f), one_m = df_add_f(df_neg(cz), 1.0f);
        const df arg = df_add(df_mul(F.kappa, one_p), df{0.5f * one_m.hi, 0.5f * one_m.lo});
        const df l10 = df_mul(df_log(df{0.5f * arg.hi, 0.5f * arg.lo}), df{0.4342945f, -1.010305e-08f});
        return -2.5 * df_to_double(l10);
    }
    const df S[3] = {df_from_double(o.sx[i]), df_from_double(o.sy[i]), df_from_double(o.sz[i])};
    const df Sp[3] = {df_dot3(b, S), df_dot3(c, S), df_dot3(a, S)};
    const df Ep[3] = {df_dot3(b, E), df_dot3(c, E), df_dot3(a, E)};
    return df_to_double(ls_magnitude_df(Sp, Ep, F.ib, F.ic, F.bc, tab));
}

// NUDGE minimum candidates of the mixed path: observation i and the Euler angles at i-2, i-1, i.
// They are re-evaluated with double-float magnitudes in queue order after the last observation
// (or when the queue fills).  Deferring them lets the lanes of a warp evaluate their candidates
// side by side (each lane has its own, at different observations) instead of one observation
// after another; the queue is long enough (more than the AST_M_MAX minima a model may have)
// that a flush in the middle of the light curve, which the lanes would take one at a time, is
// rare.
constexpr int kNudgeQueue = 32;
struct NudgeCand {
    int i;
    df a[3][3];
};

// The reference's test and parabola (cuda.c:716-760) on each queued triple, with double-float
// magnitudes.  Returns false as soon as more than AST_M_MAX minima are found (the model is then
// rejected exactly as the reference rejects it, only after a few more observations).
// Not inlined: the magnitude code is cold and large, and one copy serves both call sites.
static __host__ __device__ __noinline__ bool nudge_flush(const DevModel& M, const ObsView& o, const DfFrame& F,
                                                         const float4* tab, NudgeCand* cand, int* n_cand, int* Mmin,
                                                         float* t_mod, float* V_mod)
{
    for (int q = 0; q < *n_cand; q++) {
        const int ic = cand[q].i;
        const float f0 = (float)vmod_df(M, o, F, cand[q].a[0], ic - 2, tab);
        const float f1 = (float)vmod_df(M, o, F, cand[q].a[1], ic - 1, tab);
        const double v2 = vmod_df(M, o, F, cand[q].a[2], ic, tab);
        if (f1 > f0 && f1 >= v2) {
            if (++*Mmin > AST_M_MAX) return false;
            const float t0 = (float)o.t[ic - 2], t1 = (float)o.t[ic - 1];
            const double ti = o.t[ic];
            const double a = ((v2 - f1) / (ti - t1) - (f1 - f0) / (t1 - t0)) / (ti - t0);
            const double b = DD_SUB((f1 - f0) / (t1 - t0), DD_MUL(a, (double)DF_ADD(t1, t0)));
            const double c = DD_SUB(DD_SUB(f1, DD_MUL(DD_MUL(a, t1), t1)), DD_MUL(b, t1));
            const int m = *Mmin - 1;
            t_mod[m] = (float)(-b / 2.0 / a);
            const double tm = t_mod[m];
            V_mod[m] = (float)DD_ADD(DD_ADD(DD_MUL(DD_MUL(a, tm), tm), DD_MUL(b, tm)), c);
        }
    }
    *n_cand = 0;
    return true;
}

// Per-evaluation constants of the FP32 magnitude: the spin-axis frame (cuda.c:195-217) and the
// photometric shape (cuda.c:568-574) or the BW_BALL parameters.
struct MixedFrame {
    float M_x, M_y, M_z, XM_x, XM_z, YM_x, YM_y, YM_z;
    float ib, ic, bc;
    float kappa, cos_phR, sin_phR, cos_thR, sin_thR;
};
constexpr int kMixedFrameFloats = 16;

// The integrated state of one evaluation of the mixed path: y and the ODE constants mu as
// double-floats (and in FP32 for the FP32 right-hand side), the magnitude frame.
struct MixedState {
    df y[6];
    df mu[6];
    float muf[6];
    bool torque, bw;
    MixedFrame F;
};

// Per-evaluation set-up in FP64 (cuda.c:195-252): initial Euler angles and angular velocity, the
// ODE constants, the magnitude frame.  Every rounding explicit (DD_*, DF_*, f_*, d_*), with float
// and double operands as in the reference's expressions: the same bits in every kernel.
AST_HD void mixed_setup(const DevModel& M, const double* params, MixedState& S)
{
    const int flags = M.flags;
    const ast_type_ids& T = M.t;
#define AST_P(tt) params[M.idx[T.tt]]
    const double th_M = AST_P(theta_M), ph_M = AST_P(phi_M);
    const double M_xd = DD_MUL(sin(th_M), cos(ph_M)), M_yd = DD_MUL(sin(th_M), sin(ph_M)), M_zd = cos(th_M);
    const double XMd = sqrt(d_dot2(M_zd, M_zd, M_xd, M_xd));
    MixedFrame& F = S.F;
    F.M_x = (float)M_xd;
    F.M_y = (float)M_yd;
    F.M_z = (float)M_zd;
    F.XM_x = (float)(M_zd / XMd);
    F.XM_z = (float)(-M_xd / XMd);
    F.YM_x = DF_MUL(F.M_y, F.XM_z);
    F.YM_y = f_dif2(F.M_z, F.XM_x, F.M_x, F.XM_z);
    F.YM_z = -DF_MUL(F.M_y, F.XM_x);
    const double bt = AST_P(b_tumb), ct = AST_P(c_tumb);
    const double bt2 = DD_MUL(bt, bt), ct2 = DD_MUL(ct, ct);
    const double Is = DD_ADD(1.0, bt2) / DD_ADD(bt2, ct2);
    const double Ii = DD_ADD(1.0, ct2) / DD_ADD(bt2, ct2);
    const double Is_inv = 1.0 / Is, Ii_inv = 1.0 / Ii;
    const double psi0 = AST_P(psi_0);
    S.torque = (flags & AST_TORQUE) != 0;
    {
        const double sp = sin(psi0);
        const double den = DD_SUB(DD_ADD(DD_MUL(DD_MUL(sp, sp), DD_SUB(Ii_inv, Is_inv)), Is_inv), 1.0);
        const double theta = asin(sqrt(DD_SUB(AST_P(Es), 1.0) / den));
        if (S.torque) {
            S.mu[0] = df_from_double(DD_MUL(DD_SUB(Is, 1.0), Ii_inv));
            S.mu[1] = df_from_double(DD_MUL(DD_SUB(1.0, Ii), Is_inv));
            S.mu[2] = df_from_double(DD_SUB(Ii, Is));
            S.mu[3] = df_from_double(AST_P(Ti));
            S.mu[4] = df_from_double(AST_P(Ts));
            S.mu[5] = df_from_double(AST_P(Tl));
            const double L = AST_P(L);
            S.y[0] = df_from_double(DD_MUL(DD_MUL(DD_MUL(L, Ii_inv), sin(theta)), sp));
            S.y[1] = df_from_double(DD_MUL(DD_MUL(DD_MUL(L, Is_inv), sin(theta)), cos(psi0)));
            S.y[2] = df_from_double(DD_MUL(L, cos(theta)));
            S.y[3] = df_from_double(AST_P(phi_0));
            S.y[4] = df_from_double(theta);
            S.y[5] = df_from_double(psi0);
            for (int k = 0; k < 6; k++) S.muf[k] = DF_ADD(S.mu[k].hi, S.mu[k].lo);
        } else {
            S.mu[0] = df_from_double(AST_P(L));
            const double Ip = DD_MUL(0.5, DD_ADD(Ii_inv, Is_inv));
            S.mu[1] = df_from_double(Ip);
            S.mu[2] = df_from_double(DD_MUL(0.5, DD_SUB(Ii_inv, Is_inv)));
            S.y[0] = df_from_double(AST_P(phi_0));
            S.y[1] = df_from_double(theta);
            S.y[2] = df_from_double(psi0);
            for (int k = 0; k < 3; k++) S.muf[k] = DF_ADD(S.mu[k].hi, S.mu[k].lo);
            S.muf[3] = (float)DD_SUB(1.0, Ip);
        }
    }
    S.bw = (flags & AST_BW_BALL) != 0;
    float b_ph = 1, c_ph = 1;
    F.kappa = F.cos_phR = F.sin_phR = F.cos_thR = F.sin_thR = 0;
    if (S.bw) {
        F.kappa = (float)AST_P(kappa);
        sincosf((float)AST_P(phi_R), &F.sin_phR, &F.cos_phR);
        sincosf((float)AST_P(theta_R), &F.sin_thR, &F.cos_thR);
    } else {
        b_ph = (float)((flags & AST_BC) ? AST_P(b) : bt);
        c_ph = (float)((flags & AST_BC) ? AST_P(c) : ct);
    }
    F.ib = 1.0f / b_ph;
    F.ic = 1.0f / c_ph;
    F.bc = DF_MUL(b_ph, c_ph);
#undef AST_P
}

// Integrate from observation i-1 to i (cuda.c:319-372; nothing for i = 0) and return the Euler
// angles (phi, theta, psi) reduced to [-pi, pi].  They enter the right-hand side and the
// brightness only through sin and cos, so the state itself is kept reduced: the double-float then
// resolves the phase to ~1e-14 rad instead of u^2 of the accumulated angle.  RHS32: the FP32
// right-hand side (AST_PREC_MIXED_RHS32), a separate instantiation so that the double-float
// kernels carry none of its code.
template <bool RHS32>
AST_HD void mixed_advance(MixedState& S, const ObsView& o, int i, const float4* tab, df* ang)
{
    if (i > 0) {
        const int N_steps = o.nst[i];
        const float4 hq = o.hq[i], hw = o.hw[i];
        // Not unrolled: one copy of the step keeps the hot loop inside the instruction cache.
        if (RHS32) {
            if (S.torque) {
#pragma unroll 1
                for (int l = 0; l < N_steps; l++) rk4_step_f32<6>(S.y, hq, hw, S.muf, tab);
            } else {
#pragma unroll 1
                for (int l = 0; l < N_steps; l++) rk4_step_f32<3>(S.y, hq, hw, S.muf, tab);
            }
        } else if (S.torque) {
            df2 Y[3] = {df2_pack(S.y[0], S.y[1]), df2_pack(S.y[2], S.y[3]), df2_pack(S.y[5], S.y[4])};
#pragma unroll 1
            for (int l = 0; l < N_steps; l++) rk4_step_df2<6>(Y, hq, hw, S.mu, tab);
            S.y[0] = df2_x(Y[0]);
            S.y[1] = df2_y(Y[0]);
            S.y[2] = df2_x(Y[1]);
            S.y[3] = df2_y(Y[1]);
            S.y[5] = df2_x(Y[2]);
            S.y[4] = df2_y(Y[2]);
        } else {
            df2 Y[2] = {df2_pack(S.y[2], S.y[1]), df2_pack(S.y[0], df{0.0f, 0.0f})};
#pragma unroll 1
            for (int l = 0; l < N_steps; l++) rk4_step_df2<3>(Y, hq, hw, S.mu, tab);
            S.y[2] = df2_x(Y[0]);
            S.y[1] = df2_y(Y[0]);
            S.y[0] = df2_x(Y[1]);
        }
    }
    // (Constant indices only: an index computed at run time would move y to local memory.)
    if (S.torque) {
        S.y[3] = df_reduce_2pi(S.y[3]);
        S.y[4] = df_reduce_2pi(S.y[4]);
        S.y[5] = df_reduce_2pi(S.y[5]);
        ang[0] = S.y[3];
        ang[1] = S.y[4];
        ang[2] = S.y[5];
    } else {
        S.y[0] = df_reduce_2pi(S.y[0]);
        S.y[1] = df_reduce_2pi(S.y[1]);
        S.y[2] = df_reduce_2pi(S.y[2]);
        ang[0] = S.y[0];
        ang[1] = S.y[1];
        ang[2] = S.y[2];
    }
}

// FP32 model magnitude at observation i for the Euler angles (phi, theta, psi): the body frame
// as in cuda.c:432-473, then the cancellation-free Lommel-Seeliger form (ls_magnitude_f) or the
// BW_BALL law (cuda.c:475-497, 603-607).
AST_HD float mixed_vmod(const MixedFrame& F, bool bw, float phi, float theta, float psi, const ObsView& o, int i)
{
    float sin_phi, cos_phi, sin_theta, cos_theta, sin_psi, cos_psi;
    sincosf(phi, &sin_phi, &cos_phi);
    sincosf(theta, &sin_theta, &cos_theta);
    sincosf(psi, &sin_psi, &cos_psi);
    float N_x = f_dot2(F.XM_x, cos_phi, F.YM_x, sin_phi);
    float N_y = DF_MUL(F.YM_y, sin_phi);
    float N_z = f_dot2(F.XM_z, cos_phi, F.YM_z, sin_phi);
    float p_x = f_dif2(N_y, F.M_z, N_z, F.M_y);
    float p_y = f_dif2(N_z, F.M_x, N_x, F.M_z);
    float p_z = f_dif2(N_x, F.M_y, N_y, F.M_x);
    float a_x = f_dot2(F.M_x, cos_theta, p_x, sin_theta);
    float a_y = f_dot2(F.M_y, cos_theta, p_y, sin_theta);
    float a_z = f_dot2(F.M_z, cos_theta, p_z, sin_theta);
    const float w_x = f_dif2(a_y, N_z, a_z, N_y);
    const float w_y = f_dif2(a_z, N_x, a_x, N_z);
    const float w_z = f_dif2(a_x, N_y, a_y, N_x);
    const float b_x = f_dot2(N_x, cos_psi, w_x, sin_psi);
    const float b_y = f_dot2(N_y, cos_psi, w_y, sin_psi);
    const float b_z = f_dot2(N_z, cos_psi, w_z, sin_psi);
    const float c_x = f_dif2(a_y, b_z, a_z, b_y);
    const float c_y = f_dif2(a_z, b_x, a_x, b_z);
    const float c_z = f_dif2(a_x, b_y, a_y, b_x);
    const float E_x1 = o.efx[i], E_y1 = o.efy[i], E_z1 = o.efz[i];
    const float S_x1 = o.sfx[i], S_y1 = o.sfy[i], S_z1 = o.sfz[i];
    if (bw) {
        N_x = f_dot2(b_x, F.cos_phR, c_x, F.sin_phR);
        N_y = f_dot2(b_y, F.cos_phR, c_y, F.sin_phR);
        N_z = f_dot2(b_z, F.cos_phR, c_z, F.sin_phR);
        p_x = f_dif2(N_y, a_z, N_z, a_y);
        p_y = f_dif2(N_z, a_x, N_x, a_z);
        p_z = f_dif2(N_x, a_y, N_y, a_x);
        a_x = f_dot2(a_x, F.cos_thR, p_x, F.sin_thR);
        a_y = f_dot2(a_y, F.cos_thR, p_y, F.sin_thR);
        a_z = f_dot2(a_z, F.cos_thR, p_z, F.sin_thR);
        const float cos_zeta = f_dot3(a_x, E_x1, a_y, E_y1, a_z, E_z1);
        const float arg = f_dot2(F.kappa, DF_ADD(1.0f, cos_zeta), 0.5f, DF_SUB(1.0f, cos_zeta));
        return DF_MUL(-2.5f, log10f(DF_MUL(0.5f, arg)));
    }
    const float Ep_b = f_dot3(b_x, E_x1, b_y, E_y1, b_z, E_z1);
    const float Ep_c = f_dot3(c_x, E_x1, c_y, E_y1, c_z, E_z1);
    const float Ep_a = f_dot3(a_x, E_x1, a_y, E_y1, a_z, E_z1);
    const float Sp_b = f_dot3(b_x, S_x1, b_y, S_y1, b_z, S_z1);
    const float Sp_c = f_dot3(c_x, S_x1, c_y, S_y1, c_z, S_z1);
    const float Sp_a = f_dot3(a_x, S_x1, a_y, S_y1, a_z, S_z1);
    return ls_magnitude_f(Sp_b, Sp_c, Sp_a, Ep_b, Ep_c, Ep_a, F.ib, F.ic, F.bc);
}

// Per-filter delta_V and chi^2 from the double-float residual sums (cuda.c:887-910): the
// combination in FP64, the sum of the filters' chi^2 over the degrees of freedom (or the RMSD).
template <class CF>
AST_HD CF mixed_combine(const DevModel& M, const ObsView& o, const df* sum_y, const df* sum_y2, CF* dv)
{
    const int N_filters = M.n_filters;
    CF chi2m, chi2a = 0.0, SUM_w = 0.0;
    for (int m = 0; m < N_filters; m++) {
        const double sy = df_to_double(sum_y[m]), sy2 = df_to_double(sum_y2[m]), sw = o.sum_w[m];
        chi2m = (CF)DD_SUB(sy2, DD_MUL(sy, sy) / sw);
        chi2a = chi2a + chi2m;
        dv[m] = (CF)(sy / sw);
        SUM_w = (CF)DD_ADD((double)SUM_w, sw);
    }
    if (M.flags & AST_RMSD)
        chi2a = sqrt(chi2a / SUM_w);
    else
        chi2a = chi2a / (CF)(M.n_data - M.n_params - N_filters);
    return chi2a;
}

// Same contract as chi2_fp64 (model.cuh); tab is the shared-memory sin/cos table; ang_out, when
// non-null, receives the Euler angles at every observation (reduced to [-pi, pi]).  RHS32 selects
// the FP32 right-hand side of AST_PREC_MIXED_RHS32.
template <class CF, bool RHS32 = false>
__host__ __device__ CF chi2_mixed(const DevModel& M, const ObsView& o, const double* params, CF* delta_V, const float4* tab,
                                  double* ang_out = nullptr)
{
    const int flags = M.flags;
    const int N_data = M.n_data, N_filters = M.n_filters;
    df sum_y2[AST_MAX_FILTERS], sum_y[AST_MAX_FILTERS];
    for (int m = 0; m < N_filters; m++) { sum_y2[m] = df{0.0f, 0.0f}; sum_y[m] = df{0.0f, 0.0f}; }
    int Mmin = 0;
    float t_mod[AST_M_MAX], V_mod[AST_M_MAX];
    float t_old[2] = {0.f, 0.f}, V_old[2] = {0.f, 0.f};
    df ang_old[2][3] = {};
    NudgeCand cand[kNudgeQueue];
    int n_cand = 0;
    MixedState S;
    mixed_setup(M, params, S);
    DfFrame F;
    if (flags & AST_NUDGE) F = make_df_frame(M, params);
    for (int i = 0; i < N_data; i++) {
        df ang[3];
        mixed_advance<RHS32>(S, o, i, tab, ang);
        if (ang_out)
            for (int k = 0; k < 3; k++) ang_out[3 * i + k] = df_to_double(ang[k]);
        const float Vmod = mixed_vmod(S.F, S.bw, DF_ADD(ang[0].hi, ang[0].lo), DF_ADD(ang[1].hi, ang[1].lo),
                                      DF_ADD(ang[2].hi, ang[2].lo), o, i);
        {
            // Residual and weighted sums as double-floats: v - Vmod exactly (TwoSum), products
            // to ~u^2, sums with the sloppy double-float add (absolute error ~u^2 of the sum).
            const int m = o.f[i];
            const df yv = two_sum(o.v[i], -Vmod);
            const df wy = df_mul_f(yv, o.w[i]);
            sum_y[m] = df_add_fast(sum_y[m], wy);
            sum_y2[m] = df_add_fast(sum_y2[m], df_mul_fast(wy, yv));
        }
        if (flags & AST_NUDGE) {
            // Model minima near observed minima (cuda.c:716-760).  The detection and the parabola
            // are discontinuous in the magnitudes (the reference even rounds them to float), so an
            // FP32 magnitude is used only to rule a triple out with a margin far above its error;
            // a candidate triple is queued with its double-float angles and re-evaluated with
            // double-float magnitudes (nudge_flush), in order, exactly as the reference tests it.
            const df ang_i[3] = {ang[0], ang[1], ang[2]};
            if (i >= 2) {
                bool local = false;
                for (int ii = 0; ii < M.n_min; ii++)
                    if (fabsf(t_old[1] - M.t_min[ii]) < AST_DT_MAX2) local = true;
                const float margin = 1e-4f;
                if (local && V_old[1] > V_old[0] - margin && V_old[1] >= Vmod - margin) {
                    NudgeCand& q = cand[n_cand];
                    q.i = i;
                    for (int k = 0; k < 3; k++) {
                        q.a[0][k] = ang_old[0][k];
                        q.a[1][k] = ang_old[1][k];
                        q.a[2][k] = ang_i[k];
                    }
                    if (++n_cand == kNudgeQueue && !nudge_flush(M, o, F, tab, cand, &n_cand, &Mmin, t_mod, V_mod))
                        return (CF)kHuge;
                }
            }
            const int slot = i < 2 ? i : 1;
            if (i >= 2) {
                t_old[0] = t_old[1];
                V_old[0] = V_old[1];
                for (int k = 0; k < 3; k++) ang_old[0][k] = ang_old[1][k];
            }
            t_old[slot] = (float)o.t[i];
            V_old[slot] = Vmod;
            for (int k = 0; k < 3; k++) ang_old[slot][k] = ang_i[k];
        }
    }
    if ((flags & AST_NUDGE) && !nudge_flush(M, o, F, tab, cand, &n_cand, &Mmin, t_mod, V_mod)) return (CF)kHuge;
    CF dv[AST_MAX_FILTERS];
    CF chi2a = mixed_combine<CF>(M, o, sum_y, sum_y2, dv);
    if (flags & AST_NUDGE) {
        float S_M = 0.0f, P_tot = 1.0f;
        for (int imod = 0; imod < Mmin; imod++) {
            for (int iobs = 0; iobs < M.n_min; iobs++) {
                const float dt = fabsf(t_mod[imod] - M.t_min[iobs]);
                if (dt < AST_DT_MAX2) {
                    if (dt > AST_DT_MAX) {
                        const float x = (AST_DT_MAX2 - dt) / (AST_DT_MAX2 - AST_DT_MAX);
                        S_M = (float)DD_ADD(S_M, DD_MUL((double)DF_MUL(x, x), DD_ADD(DD_MUL(-2.0, (double)x), 3.0)));
                    } else {
                        S_M = (float)(S_M + 1.0);
                        const float dV = (float)(V_mod[imod] + dv[0] - M.v_min[iobs]);
                        const float x = sqrtf(DF_ADD(DF_MUL(dt, dt) / AST_DT_MAX / AST_DT_MAX,
                                                     DF_MUL(dV, dV) / AST_DV_MAX / AST_DV_MAX));
                        if (x < 1.0f) {
                            const float P_i = DF_MUL(DF_MUL(AST_L_A, x), x) / DF_ADD(DF_MUL(x, x), AST_L_RC2);
                            P_tot = (float)DD_MUL(P_tot, DD_MUL(AST_P_MIN, DD_ADD(1.0, (double)DF_MUL(AST_P_MIN2, P_i))));
                        }
                    }
                }
            }
        }
        P_tot = powf(P_tot, (float)(1.0 / M.n_min));
        if (P_tot < AST_P_MIN) P_tot = AST_P_MIN;
        if (chi2a > AST_CHI2_1)
            P_tot = 1.0f;
        else if (chi2a > AST_CHI2_0) {
            const float x = (float)((AST_CHI2_1 - chi2a) / (AST_CHI2_1 - AST_CHI2_0));
            const float beta = DF_MUL(DF_MUL(x, x), DF_ADD(DF_MUL(-2.0f, x), 3.0f));
            P_tot = powf(P_tot, beta);
        }
        float P_M;
        if (S_M < AST_M_MAX2)
            P_M = 1.0f;
        else if (S_M < AST_M_MAX) {
            const float x = (S_M - AST_M_MAX2) / (AST_M_MAX - AST_M_MAX2);
            P_M = (float)DD_ADD(1.0, (double)DF_MUL(DF_MUL(DF_MUL(3.0f, x), x), DF_ADD(DF_MUL(-2.0f, x), 3.0f)));
        } else
            P_M = 4.0f;
        chi2a = chi2a * P_tot * P_M;
    }
    for (int m = 0; m < N_filters; m++) delta_V[m] = dv[m];
    return chi2a;
}

// ---------------------------------------------------------------- warp-tiled evaluation
//
// Warp per model with observation tiles: the 32 lanes of a warp evaluate 32 parameter vectors of
// one object together.  Each lane integrates its own vector through a tile of T observations and
// leaves the Euler angles in shared memory; the warp then computes the tile's magnitudes
// transposed -- the 32 x T (vector, observation) pairs spread over the lanes, consecutive lanes
// on consecutive observations of one vector -- and each lane sums its own vector's residuals in
// observation order.  The arithmetic is that of chi2_mixed, term for term, so the result is the
// same bit for bit; what changes is which lane computes a magnitude.  The residual sums need no
// cross-lane reduction: the transposed residuals go back to their vector's lane through shared
// memory, which keeps the summation order, and the bits, of the thread path.  No NUDGE (its
// minimum search runs along one vector's curve); ast_batch_tune weighs this mapping and T
// against the thread-per-model kernels.

// Shared-memory bytes of one warp: the 32 vectors' magnitude frames, their angles over a tile
// and the tile's residuals (double-floats).
__host__ __device__ constexpr int tile_warp_bytes(int T)
{
    return 4 * (kMixedFrameFloats * 32 + 3 * 32 * (T + 1)) + 8 * 32 * (T + 1);
}

__device__ __forceinline__ void frame_store(float* fr, int lane, const MixedFrame& F)
{
    const float* f = &F.M_x;
#pragma unroll
    for (int k = 0; k < kMixedFrameFloats; k++) fr[k * 32 + lane] = f[k];
}

__device__ __forceinline__ MixedFrame frame_load(const float* fr, int lane)
{
    MixedFrame F;
    float* f = &F.M_x;
#pragma unroll
    for (int k = 0; k < kMixedFrameFloats; k++) f[k] = fr[k * 32 + lane];
    return F;
}

// Called by all 32 lanes of a warp at once (uniform control flow), each with its own params;
// `active` lanes get their chi^2 and delta_V, the others only take part.  wsm: the warp's
// tile_warp_bytes(T) of shared memory.
template <class CF, int T>
__device__ CF chi2_mixed_tile(const DevModel& M, const ObsView& o, const double* params, bool active, CF* delta_V,
                              const float4* tab, unsigned char* wsm)
{
    static_assert(sizeof(MixedFrame) == 4 * kMixedFrameFloats, "MixedFrame is kMixedFrameFloats floats");
    const int lane = threadIdx.x & 31;
    const int N_data = M.n_data, N_filters = M.n_filters;
    float* fr = (float*)wsm;                          // [kMixedFrameFloats][32]
    float* ang = fr + kMixedFrameFloats * 32;         // [3][32][T + 1]
    float2* res = (float2*)(ang + 3 * 32 * (T + 1));  // [32][T + 1]
    df sum_y2[AST_MAX_FILTERS], sum_y[AST_MAX_FILTERS];
    for (int m = 0; m < N_filters; m++) { sum_y2[m] = df{0.0f, 0.0f}; sum_y[m] = df{0.0f, 0.0f}; }
    MixedState S;
    mixed_setup(M, params, S);
    frame_store(fr, lane, S.F);
    const bool bw = S.bw;
    for (int i0 = 0; i0 < N_data; i0 += T) {
        const int n = min(T, N_data - i0);
        // Integrate this lane's vector through the tile.
        for (int j = 0; j < n; j++) {
            df a[3];
            mixed_advance<false>(S, o, i0 + j, tab, a);
#pragma unroll
            for (int c = 0; c < 3; c++) ang[(c * 32 + lane) * (T + 1) + j] = DF_ADD(a[c].hi, a[c].lo);
        }
        __syncwarp();
        // The tile's 32 x n magnitudes, consecutive lanes on consecutive observations.
        for (int q = lane; q < 32 * n; q += 32) {
            const int v = q / n, j = q - v * n, i = i0 + j;
            const MixedFrame F = frame_load(fr, v);
            const float Vmod = mixed_vmod(F, bw, ang[(0 * 32 + v) * (T + 1) + j], ang[(1 * 32 + v) * (T + 1) + j],
                                          ang[(2 * 32 + v) * (T + 1) + j], o, i);
            const df yv = two_sum(o.v[i], -Vmod);
            res[v * (T + 1) + j] = make_float2(yv.hi, yv.lo);
        }
        __syncwarp();
        // This lane's residuals in observation order (the sums of chi2_mixed).
        for (int j = 0; j < n; j++) {
            const int i = i0 + j;
            const float2 r = res[lane * (T + 1) + j];
            const df yv{r.x, r.y};
            const int m = o.f[i];
            const df wy = df_mul_f(yv, o.w[i]);
            sum_y[m] = df_add_fast(sum_y[m], wy);
            sum_y2[m] = df_add_fast(sum_y2[m], df_mul_fast(wy, yv));
        }
        __syncwarp();
    }
    CF dv[AST_MAX_FILTERS];
    const CF chi2a = mixed_combine<CF>(M, o, sum_y, sum_y2, dv);
    if (active)
        for (int m = 0; m < N_filters; m++) delta_V[m] = dv[m];
    return chi2a;
}

}  // namespace ast
