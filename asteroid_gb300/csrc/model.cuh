// model.cuh -- the light-curve model in FP64: device tables, the x <-> params maps, the ODE
// right-hand sides and the chi^2 of one parameter vector.
//
// The plain path must agree with the reference kernel to 1e-12 relative chi^2, so every
// expression below keeps the operand order and the float/double types of the reference's
// chi2one (cuda.c:81-1011), x2params (cuda.c:1120-1319) and params2x (cuda.c:1016-1115);
// nvcc then makes the same multiply-add contractions in both.  What differs is the data
// flow: quantities that do not depend on the parameters (per-interval RK4 step count and
// size, the ephemeris interpolation of E and S) are computed once per object by
// prep_obs_kernel with the same expressions, instead of once per evaluation.
#pragma once
#include <math.h>
#include <stdint.h>
#include "asteroid_gb300.h"

#ifndef AST_HD
#define AST_HD __host__ __device__ __forceinline__
#endif

namespace ast {

constexpr double kPi = 3.141592653589793238;
constexpr double kHuge = 1e30;


// Tables of one variant, by value in kernel parameters (the reference's dProperty, dTypes,
// dLimits, d_x2_params, d_chi2_params symbols, asteroid.h:460,509-513,533).
struct DevModel {
    int32_t flags;
    int32_t n_params;
    int32_t n_filters;
    int32_t n_data;
    double time_step;
    int8_t ptype[AST_MAX_PARAMS];     // Property[i][P_type]
    int8_t indep[AST_MAX_PARAMS];     // Property[i][P_independent]
    int8_t frozen[AST_MAX_PARAMS];    // Property[i][P_frozen]
    int8_t periodic[AST_MAX_PARAMS];  // Property[i][P_periodic]
    int8_t idx[AST_MAX_TYPES];        // Types[type][0]: parameter index of a type, -1 if absent
    ast_type_ids t;                   // type ids of this variant
    double lim0[AST_MAX_TYPES], lim1[AST_MAX_TYPES];  // Limits (rounded to float unless ACC)
    float ppsi1, ppsi2;               // x2_struct
    int32_t n_min;                    // chi2_struct (NUDGE)
    float t_min[AST_NOBS_MAX], v_min[AST_NOBS_MAX];
    double eph_e[3][3], eph_s[3][3], eph_mjd0[3];
};

// Launch shape of the persistent evaluation kernels by precision.  The double-float path runs
// fastest with three CTAs of 128 threads per SM (a 170-register budget, a few registers spilled:
// 12 warps per SM instead of 8 issue-bound warps); the FP64 path is bound by its pipe and keeps
// one CTA of 256 threads with the full register file.
template <int PREC>
struct KernShape {
    static constexpr int tpb = PREC != AST_PREC_FP64 ? 128 : 256;
    static constexpr int min_ctas = PREC != AST_PREC_FP64 ? 3 : 1;
};

// SoA observations of one object (one device buffer; also the shared-memory image).
//   t[n]  asteroid time - hMJD0       h[n]  RK4 step of interval (i-1,i)   nst[n] its steps
//   v[n], w[n] (float)                f[n] filter                           e{x,y,z}[n], s{x,y,z}[n]
struct ObsView {
    const double* t;
    const double* h;
    const int32_t* nst;
    const float* v;
    const float* w;
    const int32_t* f;
    const double* ex;
    const double* ey;
    const double* ez;
    const double* sx;
    const double* sy;
    const double* sz;
    // Derived for the mixed-precision path (prep_obs_point): step sizes as double-floats,
    // unit vectors rounded to float, per-filter weight sums.
    const float4* hq;      // (h, h/2)
    const float4* hw;      // (h/6, h/3)
    const float* efx;
    const float* efy;
    const float* efz;
    const float* sfx;
    const float* sfy;
    const float* sfz;
    const double* sum_w;   // [AST_MAX_FILTERS]
};

// Byte layout of the SoA buffer for n observations: every array starts on a 16-byte boundary
// and the total is a multiple of 16, as the bulk copies into shared memory require.
struct ObsLayout {
    int64_t off_t, off_h, off_nst, off_v, off_w, off_f, off_e, off_s, off_hq, off_hw, off_ef, off_sf, off_sw, bytes;
    AST_HD static int64_t up16(int64_t x) { return (x + 15) & ~(int64_t)15; }
    AST_HD static ObsLayout make(int64_t n)
    {
        ObsLayout L;
        int64_t o = 0;
        L.off_t = o;   o = up16(o + 8 * n);
        L.off_h = o;   o = up16(o + 8 * n);
        L.off_e = o;   o = up16(o + 3 * 8 * n);
        L.off_s = o;   o = up16(o + 3 * 8 * n);
        L.off_hq = o;  o = up16(o + 16 * n);
        L.off_hw = o;  o = up16(o + 16 * n);
        L.off_sw = o;  o = up16(o + 8 * AST_MAX_FILTERS);
        L.off_ef = o;  o = up16(o + 3 * 4 * n);
        L.off_sf = o;  o = up16(o + 3 * 4 * n);
        L.off_nst = o; o = up16(o + 4 * n);
        L.off_v = o;   o = up16(o + 4 * n);
        L.off_w = o;   o = up16(o + 4 * n);
        L.off_f = o;   o = up16(o + 4 * n);
        L.bytes = o;
        return L;
    }
    AST_HD ObsView view(const void* base, int64_t n) const
    {
        const char* b = (const char*)base;
        ObsView o;
        o.t = (const double*)(b + off_t);
        o.h = (const double*)(b + off_h);
        o.ex = (const double*)(b + off_e);
        o.ey = o.ex + n;
        o.ez = o.ey + n;
        o.sx = (const double*)(b + off_s);
        o.sy = o.sx + n;
        o.sz = o.sy + n;
        o.nst = (const int32_t*)(b + off_nst);
        o.v = (const float*)(b + off_v);
        o.w = (const float*)(b + off_w);
        o.f = (const int32_t*)(b + off_f);
        o.hq = (const float4*)(b + off_hq);
        o.hw = (const float4*)(b + off_hw);
        o.efx = (const float*)(b + off_ef);
        o.efy = o.efx + n;
        o.efz = o.efy + n;
        o.sfx = (const float*)(b + off_sf);
        o.sfy = o.sfx + n;
        o.sfz = o.sfy + n;
        o.sum_w = (const double*)(b + off_sw);
        return o;
    }
};

// NUDGE constants (asteroid.h:216-231) with the reference's float rounding.
#define AST_M_MAX2 20.0f
#define AST_DT_MAX 0.12f
#define AST_DV_MAX 24.0f
#define AST_DT_MAX2 ((float)(1.5 * 0.12f))
#define AST_P_MIN 0.01f
#define AST_CHI2_0 10.0f
#define AST_CHI2_1 30.0f
#define AST_L_RC2 (0.05f * 0.05f)
#define AST_L_A ((float)(1.0 / (1.0 - AST_L_RC2 / (1.0 + AST_L_RC2))))
#define AST_P_MIN2 ((float)(1 / 0.01f - 1))
#define AST_BC_DEV_MAX 100.0f

// ------------------------------------------------------------------ x <-> params

// x2params (cuda.c:1120-1319); CF is CHI_FLOAT.  Returns 1 when x leaves a hard limit or a
// BC shape strays more than BC_DEV_MAX from the tumbling shape.
template <class CF>
AST_HD int x2params(const DevModel& M, int reopt, const CF* x, double* params)
{
    const ast_type_ids& T = M.t;
    const int N = M.n_params;
    int LAM = 0;
    for (int i = 0; i < N; i++) {
        const int per = M.periodic[i];
        if (M.ptype[i] == T.Es) LAM = x[i] >= 0.5;
        if ((x[i] < 0.0 && (per == AST_HARD_BOTH || per == AST_HARD_LEFT || (LAM == 0 && per == AST_PERIODIC_LAM))) ||
            (x[i] > 1.0 && (per == AST_HARD_BOTH || per == AST_HARD_RIGHT || (LAM == 0 && per == AST_PERIODIC_LAM))))
            return 1;
    }
    double log_c_tumb = 0, log_b_tumb = 0, Is = 0, Ii = 0, psi_min = 0, psi_max = 0, log_c = 0;
    const bool p_psi = (M.flags & AST_P_PSI) != 0;
    for (int i = 0; i < N; i++) {
        const int pt = M.ptype[i];
        const CF L0 = (CF)M.lim0[pt], L1 = (CF)M.lim1[pt];
        if (pt == T.b_tumb) {
            log_b_tumb = log_c_tumb * (CF)(x[i] * (L1 - L0) + L0);
            params[i] = exp(log_b_tumb);
            const double b_tumb = params[i];
            const double c_tumb = params[M.idx[T.c_tumb]];
            Is = (1.0 + b_tumb * b_tumb) / (b_tumb * b_tumb + c_tumb * c_tumb);
            Ii = (1.0 + c_tumb * c_tumb) / (b_tumb * b_tumb + c_tumb * c_tumb);
        } else if (pt == T.Es) {
            if (LAM) {
                params[i] = 2.0 * (x[i] - 0.5) * (1.0 - 1.0 / Ii) + 1.0 / Ii;
                psi_min = 0.0;
                psi_max = 2.0 * kPi;
            } else {
                params[i] = 2.0 * x[i] * (1.0 / Ii - 1.0 / Is) + 1.0 / Is;
                psi_max = atan(sqrt(Ii * (Is - 1.0 / params[i]) / Is / (1.0 / params[i] - Ii)));
                psi_min = -psi_max;
            }
        } else if (pt == T.psi_0) {
            params[i] = x[i] * (psi_max - psi_min) + psi_min;
        } else if ((M.flags & AST_BC) && pt == T.b) {
            const double log_b = log_c * (CF)(x[i] * (L1 - L0) + L0);
            if (fabs(log_b - log_b_tumb) > AST_BC_DEV_MAX) return 1;
            params[i] = exp(log_b);
        } else if (M.periodic[i] == AST_PERIODIC) {
            params[i] = x[i] * 2.0 * kPi;
        } else if (M.indep[i] == 1) {
            if (!p_psi || pt != T.L || reopt) params[i] = (CF)(x[i] * (L1 - L0) + L0);
            if (pt == T.c_tumb) {
                log_c_tumb = params[i];
                params[i] = exp(log_c_tumb);
            } else if ((M.flags & AST_BC) && pt == T.c) {
                log_c = params[i];
                if (fabs(log_c - log_c_tumb) > AST_BC_DEV_MAX) return 1;
                params[i] = exp(log_c);
            } else if ((M.flags & AST_BW_BALL) && pt == T.kappa) {
                params[i] = exp(params[i]);
            } else if (pt == T.L && !reopt && p_psi) {
                // 1/Ppsi -> L via K(k^2) from five arithmetic-geometric-mean steps.
                params[i] = x[i] * (CF)(M.ppsi2 - M.ppsi1) + M.ppsi1;
                const double Es = params[M.idx[T.Es]];
                const double Einv = 1.0 / Es;
                double k2;
                if (LAM)
                    k2 = (Is - Ii) * (Einv - 1.0) / ((Ii - 1.0) * (Is - Einv));
                else
                    k2 = (Ii - 1.0) * (Is - Einv) / ((Is - Ii) * (Einv - 1.0));
                double a = 1.0, g = sqrt(1.0 - k2), a1, g1;
                for (int ii = 0; ii < 5; ii++) {
                    a1 = 0.5 * (a + g);
                    g1 = sqrt(a * g);
                    a = a1;
                    g = g1;
                }
                if (LAM)
                    params[i] = 4.0 * params[i] * kPi / (a + g) * sqrt(Ii * Is / (Es * (Ii - 1.0) * (Is - Einv)));
                else
                    params[i] = 4.0 * params[i] * kPi / (a + g) * sqrt(Ii * Is / (Es * (Is - Ii) * (Einv - 1.0)));
            }
        }
    }
    return 0;
}

template <class CF>
AST_HD CF cf_floor(CF v);
template <>
AST_HD float cf_floor<float>(float v) { return floorf(v); }
template <>
AST_HD double cf_floor<double>(double v) { return floor(v); }

// params2x (cuda.c:1016-1115).
template <class CF>
AST_HD void params2x(const DevModel& M, const double* params, CF* x)
{
    const ast_type_ids& T = M.t;
    const int N = M.n_params;
    const double b_tumb = params[M.idx[T.b_tumb]];
    const double c_tumb = params[M.idx[T.c_tumb]];
    const double Is = (1.0 + b_tumb * b_tumb) / (b_tumb * b_tumb + c_tumb * c_tumb);
    const double Ii = (1.0 + c_tumb * c_tumb) / (b_tumb * b_tumb + c_tumb * c_tumb);
    int LAM = 0, i_Es = M.idx[T.Es];
    for (int i = 0; i < N; i++) {
        const int pt = M.ptype[i];
        const CF L0 = (CF)M.lim0[pt], L1 = (CF)M.lim1[pt];
        if (M.frozen[i] != 0) { x[i] = 0; continue; }
        if (M.indep[i] == 1) {
            double par = params[i];
            if (M.periodic[i] == 1) {
                x[i] = (CF)(par / (2 * kPi));
                x[i] = x[i] - cf_floor<CF>(x[i]);
            } else {
                if ((M.flags & AST_BC) && pt == T.c) {
                    const CF C0 = (CF)M.lim0[T.c_tumb], C1 = (CF)M.lim1[T.c_tumb];
                    x[i] = (CF)((log(params[i]) - C0) / (CF)(C1 - C0));
                    continue;
                }
                if (pt == T.c_tumb) par = log(par);
                if ((M.flags & AST_BW_BALL) && pt == T.kappa) par = log(par);
                x[i] = (CF)((par - L0) / (CF)(L1 - L0));
            }
        } else {
            if (pt == T.b_tumb) {
                const double par = log(b_tumb) / log(c_tumb);
                x[i] = (CF)((par - L0) / (CF)(L1 - L0));
            } else if (pt == T.Es) {
                i_Es = i;
                LAM = params[i] > 1.0 / Ii;
                if (LAM)
                    x[i] = (CF)(0.5 * ((params[i] - 1.0 / Ii) / (1.0 - 1.0 / Ii) + 1.0));
                else
                    x[i] = (CF)(0.5 * (params[i] - 1.0 / Is) / (1.0 / Ii - 1.0 / Is));
            } else if (pt == T.psi_0) {
                double psi_min, psi_max;
                if (LAM) {
                    psi_min = 0.0;
                    psi_max = 2.0 * kPi;
                } else {
                    psi_max = atan(sqrt(Ii * (Is - 1.0 / params[i_Es]) / Is / (1.0 / params[i_Es] - Ii)));
                    psi_min = -psi_max;
                }
                x[i] = (CF)((params[i] - psi_min) / (psi_max - psi_min));
            } else if ((M.flags & AST_BC) && pt == T.b) {
                const double par = log(params[i]) / log(params[M.idx[T.c]]);
                x[i] = (CF)((par - L0) / (CF)(L1 - L0));
            }
        }
    }
}

// ------------------------------------------------------------------ ODE right-hand sides

// Euler equations with constant body-frame torque + Euler-angle kinematics (cuda.c:44-58).
// y = (Omega_i, Omega_s, Omega_l, phi, theta, psi); mu = ((Is-Il)/Ii, (Il-Ii)/Is, (Ii-Is)/Il,
// Ki/Ii, Ks/Is, Kl/Il) with Il = 1.
__device__ __forceinline__ void ode_torque(const double* y, double* f, const double* mu)
{
    double s5, c5, s4, c4;
    sincos(y[5], &s5, &c5);
    sincos(y[4], &s4, &c4);
    f[0] = mu[0] * y[1] * y[2] + mu[3];
    f[1] = mu[1] * y[2] * y[0] + mu[4];
    f[2] = mu[2] * y[0] * y[1] + mu[5];
    f[3] = (y[0] * s5 + y[1] * c5) / s4;
    f[4] = y[0] * c5 - y[1] * s5;
    f[5] = y[2] - f[3] * c4;
}

// Torque-free Euler angles (cuda.c:68-75): y = (phi, theta, psi), mu = (L, Ip, Im).
__device__ __forceinline__ void ode_free(const double* y, double* f, const double* mu)
{
    double s2, c2, s1, c1;
    sincos(2.0 * y[2], &s2, &c2);
    sincos(y[1], &s1, &c1);
    f[0] = mu[0] * (mu[1] - mu[2] * c2);
    f[1] = mu[0] * mu[2] * s1 * s2;
    f[2] = c1 * (mu[0] - f[0]);
}

// One classic RK4 step of size h (cuda.c:348-372), in the reference's operation order.
template <int NODE>
__device__ __forceinline__ void rk4_step(double* y, double h, const double* mu)
{
    double f[NODE], K1[NODE], K2[NODE], K3[NODE], K4[NODE];
    if (NODE == 6) ode_torque(y, K1, mu); else ode_free(y, K1, mu);
#pragma unroll
    for (int j = 0; j < NODE; j++) f[j] = y[j] + 0.5 * h * K1[j];
    if (NODE == 6) ode_torque(f, K2, mu); else ode_free(f, K2, mu);
#pragma unroll
    for (int j = 0; j < NODE; j++) f[j] = y[j] + 0.5 * h * K2[j];
    if (NODE == 6) ode_torque(f, K3, mu); else ode_free(f, K3, mu);
#pragma unroll
    for (int j = 0; j < NODE; j++) f[j] = y[j] + h * K3[j];
    if (NODE == 6) ode_torque(f, K4, mu); else ode_free(f, K4, mu);
#pragma unroll
    for (int j = 0; j < NODE; j++) y[j] = y[j] + 1 / 6.0 * h * (K1[j] + 2 * K2[j] + 2 * K3[j] + K4[j]);
}

// ------------------------------------------------------------------ chi^2, FP64

// Per-observation brightness from body axes (a, b, c), unit E and S (cuda.c:475-689).
struct Geometry {
    double M_x, M_y, M_z, XM_x, XM_z, YM_x, YM_y, YM_z;
};

// chi2one (cuda.c:81-1011) for one parameter vector over the object's observations.
// Returns CHI_FLOAT; delta_V is written only when the evaluation runs to the end (the NUDGE
// "more than M_MAX minima" exit returns 1e30 and leaves it, as the reference does).
// vmod_out, when non-null, receives the model magnitude of every observation (the reference's
// Nplot > 0 mode, cuda.c:699-704, without the delta_V shift); ang_out the Euler angles
// (phi, theta, psi) at every observation; geo_out the kAstGeo inputs of the ANIMATE renderer
// at every observation (compute_rgb's arguments, cuda.c:576-586).
constexpr int kAstGeo = 20;

__device__ __forceinline__ void write_geo(double* g, double b, double c, double Ex, double Ey, double Ez, double Epb,
                                          double Epc, double Epa, double Spb, double Spc, double Spa, double bx,
                                          double by, double bz, double cx, double cy, double cz, double ax, double ay,
                                          double az)
{
    g[0] = b; g[1] = c;
    g[2] = Ex; g[3] = Ey; g[4] = Ez;
    g[5] = Epb; g[6] = Epc; g[7] = Epa;
    g[8] = Spb; g[9] = Spc; g[10] = Spa;
    g[11] = bx; g[12] = by; g[13] = bz;
    g[14] = cx; g[15] = cy; g[16] = cz;
    g[17] = ax; g[18] = ay; g[19] = az;
}

template <class CF>
__device__ CF chi2_fp64(const DevModel& M, const ObsView& o, const double* params, CF* delta_V,
                        double* vmod_out = nullptr, double* ang_out = nullptr, double* geo_out = nullptr)
{
    const int flags = M.flags;
    const ast_type_ids& T = M.t;
    const int N_data = M.n_data, N_filters = M.n_filters;
    double sum_y2[AST_MAX_FILTERS], sum_y[AST_MAX_FILTERS], sum_w[AST_MAX_FILTERS];
    for (int m = 0; m < N_filters; m++) { sum_y2[m] = 0.0; sum_y[m] = 0.0; sum_w[m] = 0.0; }
    int Mmin = 0;
    float t_mod[AST_M_MAX], V_mod[AST_M_MAX];
    float t_old[2] = {0.f, 0.f}, V_old[2] = {0.f, 0.f};

#define AST_P(tt) params[M.idx[T.tt]]
    const double th_M = AST_P(theta_M), ph_M = AST_P(phi_M);
    const double M_x = sin(th_M) * cos(ph_M);
    const double M_y = sin(th_M) * sin(ph_M);
    const double M_z = cos(th_M);
    const double XM = sqrt(M_z * M_z + M_x * M_x);
    const double XM_x = M_z / XM;
    const double XM_z = -M_x / XM;
    const double YM_x = M_y * XM_z;
    const double YM_y = M_z * XM_x - M_x * XM_z;
    const double YM_z = -M_y * XM_x;
    const double bt = AST_P(b_tumb), ct = AST_P(c_tumb);
    const double Is = (1.0 + bt * bt) / (bt * bt + ct * ct);
    const double Ii = (1.0 + ct * ct) / (bt * bt + ct * ct);
    const double Is_inv = 1.0 / Is;
    const double Ii_inv = 1.0 / Ii;
    const double psi0 = AST_P(psi_0);
    double y[6];
    double mu[6];
    const bool torque = (flags & AST_TORQUE) != 0;
    {
        const double phi = AST_P(phi_0);
        const double theta = asin(sqrt((AST_P(Es) - 1.0) / (sin(psi0) * sin(psi0) * (Ii_inv - Is_inv) + Is_inv - 1.0)));
        const double psi = psi0;
        if (torque) {
            mu[0] = (Is - 1.0) * Ii_inv;
            mu[1] = (1.0 - Ii) * Is_inv;
            mu[2] = Ii - Is;
            mu[3] = AST_P(Ti);
            mu[4] = AST_P(Ts);
            mu[5] = AST_P(Tl);
            const double L = AST_P(L);
            y[0] = L * Ii_inv * sin(theta) * sin(psi);
            y[1] = L * Is_inv * sin(theta) * cos(psi);
            y[2] = L * cos(theta);
            y[3] = phi;
            y[4] = theta;
            y[5] = psi;
        } else {
            const double Ip = 0.5 * (Ii_inv + Is_inv);
            const double Im = 0.5 * (Ii_inv - Is_inv);
            mu[0] = AST_P(L);
            mu[1] = Ip;
            mu[2] = Im;
            y[0] = phi;
            y[1] = theta;
            y[2] = psi;
        }
    }
    double b_ph = 0, c_ph = 0, kappa = 0, cos_phR = 0, sin_phR = 0, cos_thR = 0, sin_thR = 0;
    const bool bw = (flags & AST_BW_BALL) != 0;
    if (bw) {
        kappa = AST_P(kappa);
    } else {
        b_ph = (flags & AST_BC) ? AST_P(b) : bt;
        c_ph = (flags & AST_BC) ? AST_P(c) : ct;
    }

    for (int i = 0; i < N_data; i++) {
        if (i > 0) {
            const int N_steps = o.nst[i];
            const double h = o.h[i];
            if (torque) {
#pragma unroll 1
                for (int l = 0; l < N_steps; l++) rk4_step<6>(y, h, mu);
            } else {
#pragma unroll 1
                for (int l = 0; l < N_steps; l++) rk4_step<3>(y, h, mu);
            }
        }
        const double phi = torque ? y[3] : y[0];
        const double theta = torque ? y[4] : y[1];
        const double psi = torque ? y[5] : y[2];
        if (ang_out) {
            ang_out[3 * i] = phi;
            ang_out[3 * i + 1] = theta;
            ang_out[3 * i + 2] = psi;
        }

        double cos_phi, sin_phi;
        sincos(phi, &sin_phi, &cos_phi);
        double N_x = XM_x * cos_phi + YM_x * sin_phi;
        double N_y = YM_y * sin_phi;
        double N_z = XM_z * cos_phi + YM_z * sin_phi;
        double p_x = N_y * M_z - N_z * M_y;
        double p_y = N_z * M_x - N_x * M_z;
        double p_z = N_x * M_y - N_y * M_x;
        double cos_theta, sin_theta;
        sincos(theta, &sin_theta, &cos_theta);
        double a_x = M_x * cos_theta + p_x * sin_theta;
        double a_y = M_y * cos_theta + p_y * sin_theta;
        double a_z = M_z * cos_theta + p_z * sin_theta;
        const double w_x = a_y * N_z - a_z * N_y;
        const double w_y = a_z * N_x - a_x * N_z;
        const double w_z = a_x * N_y - a_y * N_x;
        double sin_psi, cos_psi;
        sincos(psi, &sin_psi, &cos_psi);
        const double b_x = N_x * cos_psi + w_x * sin_psi;
        const double b_y = N_y * cos_psi + w_y * sin_psi;
        const double b_z = N_z * cos_psi + w_z * sin_psi;
        const double c_x = a_y * b_z - a_z * b_y;
        const double c_y = a_z * b_x - a_x * b_z;
        const double c_z = a_x * b_y - a_y * b_x;

        const double E_x1 = o.ex[i], E_y1 = o.ey[i], E_z1 = o.ez[i];
        const double S_x1 = o.sx[i], S_y1 = o.sy[i], S_z1 = o.sz[i];
        double Vmod;
        if (bw) {
            // Brightness frame rotated by theta_R, phi_R (cuda.c:475-497), then the
            // black-and-white ball (cuda.c:596-607).
            sincos(AST_P(phi_R), &sin_phR, &cos_phR);
            sincos(AST_P(theta_R), &sin_thR, &cos_thR);
            N_x = b_x * cos_phR + c_x * sin_phR;
            N_y = b_y * cos_phR + c_y * sin_phR;
            N_z = b_z * cos_phR + c_z * sin_phR;
            p_x = N_y * a_z - N_z * a_y;
            p_y = N_z * a_x - N_x * a_z;
            p_z = N_x * a_y - N_y * a_x;
            a_x = a_x * cos_thR + p_x * sin_thR;
            a_y = a_y * cos_thR + p_y * sin_thR;
            a_z = a_z * cos_thR + p_z * sin_thR;
            const double Ep_a = a_x * E_x1 + a_y * E_y1 + a_z * E_z1;
            if (geo_out)
                write_geo(geo_out + (int64_t)kAstGeo * i, bt, ct, E_x1, E_y1, E_z1, b_x * E_x1 + b_y * E_y1 + b_z * E_z1,
                          c_x * E_x1 + c_y * E_y1 + c_z * E_z1, Ep_a, b_x * S_x1 + b_y * S_y1 + b_z * S_z1,
                          c_x * S_x1 + c_y * S_y1 + c_z * S_z1, a_x * S_x1 + a_y * S_y1 + a_z * S_z1, b_x, b_y, b_z,
                          c_x, c_y, c_z, a_x, a_y, a_z);
            const double cos_zeta = Ep_a;
            Vmod = -2.5 * log10(0.5 * (kappa * (1 + cos_zeta) + 0.5 * (1 - cos_zeta)));
        } else {
            const double Ep_b = b_x * E_x1 + b_y * E_y1 + b_z * E_z1;
            const double Ep_c = c_x * E_x1 + c_y * E_y1 + c_z * E_z1;
            const double Ep_a = a_x * E_x1 + a_y * E_y1 + a_z * E_z1;
            const double Sp_b = b_x * S_x1 + b_y * S_y1 + b_z * S_z1;
            const double Sp_c = c_x * S_x1 + c_y * S_y1 + c_z * S_z1;
            const double Sp_a = a_x * S_x1 + a_y * S_y1 + a_z * S_z1;
            // Lommel-Seeliger ellipsoid, Muinonen & Lumme (2015) eqs. 10-14 (cuda.c:664-689).
            const double b = b_ph, c = c_ph;
            if (geo_out)
                write_geo(geo_out + (int64_t)kAstGeo * i, b, c, E_x1, E_y1, E_z1, Ep_b, Ep_c, Ep_a, Sp_b, Sp_c, Sp_a,
                          b_x, b_y, b_z, c_x, c_y, c_z, a_x, a_y, a_z);
            const double scalar_Sun = sqrt(Sp_b * Sp_b / (b * b) + Sp_c * Sp_c / (c * c) + Sp_a * Sp_a);
            const double scalar_Earth = sqrt(Ep_b * Ep_b / (b * b) + Ep_c * Ep_c / (c * c) + Ep_a * Ep_a);
            const double cos_alpha_p = (Sp_b * Ep_b / (b * b) + Sp_c * Ep_c / (c * c) + Sp_a * Ep_a) / (scalar_Sun * scalar_Earth);
            const double sin_alpha_p = sqrt(1.0 - cos_alpha_p * cos_alpha_p);
            const double alpha_p = atan2(sin_alpha_p, cos_alpha_p);
            const double scalar = sqrt(scalar_Sun * scalar_Sun + scalar_Earth * scalar_Earth + 2 * scalar_Sun * scalar_Earth * cos_alpha_p);
            const double cos_lambda_p = (scalar_Sun + scalar_Earth * cos_alpha_p) / scalar;
            const double sin_lambda_p = scalar_Earth * sin_alpha_p / scalar;
            const double lambda_p = atan2(sin_lambda_p, cos_lambda_p);
            Vmod = -2.5 * log10(b * c * scalar_Sun * scalar_Earth / scalar *
                                (cos(lambda_p - alpha_p) + cos_lambda_p +
                                 sin_lambda_p * sin(lambda_p - alpha_p) * log(1.0 / tan(0.5 * lambda_p) / tan(0.5 * (alpha_p - lambda_p)))));
        }
        if (vmod_out) vmod_out[i] = Vmod;

        {   // Per-filter sums (cuda.c:707-714).
            const int m = o.f[i];
            const double yv = o.v[i] - Vmod;
            const float wi = o.w[i];
            sum_y2[m] = sum_y2[m] + yv * yv * wi;
            sum_y[m] = sum_y[m] + yv * wi;
            sum_w[m] = sum_w[m] + wi;
        }

        if (flags & AST_NUDGE) {
            // Model minima (V maxima) near the observed ones (cuda.c:716-760).
            if (i < 2) {
                t_old[i] = (float)o.t[i];
                V_old[i] = (float)Vmod;
            } else {
                if (V_old[1] > V_old[0] && V_old[1] >= Vmod) {
                    bool local = false;
                    for (int ii = 0; ii < M.n_min; ii++)
                        if (fabsf(t_old[1] - M.t_min[ii]) < AST_DT_MAX2) local = true;
                    if (local) {
                        Mmin++;
                        if (Mmin > AST_M_MAX) return (CF)kHuge;
                        const double ti = o.t[i];
                        const double a = ((Vmod - V_old[1]) / (ti - t_old[1]) - (V_old[1] - V_old[0]) / (t_old[1] - t_old[0])) / (ti - t_old[0]);
                        const double b = (V_old[1] - V_old[0]) / (t_old[1] - t_old[0]) - a * (t_old[1] + t_old[0]);
                        const double c = V_old[1] - a * t_old[1] * t_old[1] - b * t_old[1];
                        t_mod[Mmin - 1] = (float)(-b / 2.0 / a);
                        V_mod[Mmin - 1] = (float)(a * t_mod[Mmin - 1] * t_mod[Mmin - 1] + b * t_mod[Mmin - 1] + c);
                    }
                }
                t_old[0] = t_old[1];
                V_old[0] = V_old[1];
                t_old[1] = (float)o.t[i];
                V_old[1] = (float)Vmod;
            }
        }
    }
#undef AST_P

    // Per-filter chi^2 and delta_V (cuda.c:887-910); under RMSD the root of the summed chi^2 over
    // the summed weights (cuda.c:890,901-908).
    CF chi2m, chi2a = 0.0, SUM_w = 0.0;
    CF dv[AST_MAX_FILTERS];
    for (int m = 0; m < N_filters; m++) {
        chi2m = (CF)(sum_y2[m] - sum_y[m] * sum_y[m] / sum_w[m]);
        chi2a = chi2a + chi2m;
        dv[m] = (CF)(sum_y[m] / sum_w[m]);
        SUM_w = (CF)((double)SUM_w + sum_w[m]);
    }
    if (flags & AST_RMSD)
        chi2a = sqrt(chi2a / SUM_w);
    else
        chi2a = chi2a / (CF)(N_data - M.n_params - N_filters);

    if (flags & AST_NUDGE) {
        // Reward and punishment factors (cuda.c:912-993).
        float S_M = 0.0f;
        float P_tot = 1.0f;
        for (int imod = 0; imod < Mmin; imod++) {
            for (int iobs = 0; iobs < M.n_min; iobs++) {
                const float dt = fabsf(t_mod[imod] - M.t_min[iobs]);
                if (dt < AST_DT_MAX2) {
                    if (dt > AST_DT_MAX) {
                        const float x = (AST_DT_MAX2 - dt) / (AST_DT_MAX2 - AST_DT_MAX);
                        S_M = (float)(S_M + x * x * (-2.0 * x + 3.0));
                    } else {
                        S_M = (float)(S_M + 1.0);
                        const float dV = (float)(V_mod[imod] + dv[0] - M.v_min[iobs]);
                        const float x = sqrtf(dt * dt / AST_DT_MAX / AST_DT_MAX + dV * dV / AST_DV_MAX / AST_DV_MAX);
                        if (x < 1.0f) {
                            const float P_i = AST_L_A * x * x / (x * x + AST_L_RC2);
                            P_tot = (float)(P_tot * (AST_P_MIN * (1.0 + AST_P_MIN2 * P_i)));
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
            const float beta = x * x * (-2 * x + 3);
            P_tot = powf(P_tot, beta);
        }
        float P_M;
        if (S_M < AST_M_MAX2)
            P_M = 1.0f;
        else if (S_M < AST_M_MAX) {
            const float x = (S_M - AST_M_MAX2) / (AST_M_MAX - AST_M_MAX2);
            P_M = (float)(1.0 + 3 * x * x * (-2 * x + 3));
        } else
            P_M = 4.0f;
        chi2a = chi2a * P_tot * P_M;
    }
    for (int m = 0; m < N_filters; m++) delta_V[m] = dv[m];
    return chi2a;
}

}  // namespace ast
