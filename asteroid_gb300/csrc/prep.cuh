// prep.cuh -- per-object preparation of the observation block, once per ast_prepare.
//
// Everything here depends on the observations only, never on the parameters, so it is hoisted
// out of the chi^2 evaluation: the RK4 step count and size of each interval (cuda.c:414-420),
// the INTERP ephemeris at each observation (cuda.c:522-545 with misc.c:20-35), and the
// derived arrays the mixed-precision path reads (step sizes as double-floats, unit vectors in
// float, per-filter weight sums).  The functions are __host__ __device__ so that a host build
// can prepare a block the same way.
#pragma once
#include "dfloat.cuh"
#include "model.cuh"

namespace ast {

// Observation i of n: h, nst, INTERP E/S, and the mixed-path copies.  E and S must already
// hold the unit vectors (uploaded) unless the model interpolates them.
AST_HD void prep_obs_point(const DevModel& M, char* base, const ObsLayout& L, int64_t n, int64_t i)
{
    double* t = (double*)(base + L.off_t);
    double* h = (double*)(base + L.off_h);
    int32_t* nst = (int32_t*)(base + L.off_nst);
    double hi = 0.0;
    if (i == 0) {
        h[0] = 0.0;
        nst[0] = 0;
    } else {
        const double t1 = t[i - 1], t2 = t[i];
        const int N_steps = (int)((t2 - t1) / M.time_step + 1);
        hi = (t2 - t1) / N_steps;
        h[i] = hi;
        nst[i] = N_steps;
    }
    double* ex = (double*)(base + L.off_e);
    double* sx = (double*)(base + L.off_s);
    if (M.flags & AST_INTERP) {
        const double* M0 = M.eph_mjd0;
        const double ti = t[i];
        double rr[3];
        rr[0] = (ti - M0[1]) * (ti - M0[2]) / (M0[0] - M0[1]) / (M0[0] - M0[2]);
        rr[1] = (ti - M0[0]) * (ti - M0[2]) / (M0[1] - M0[0]) / (M0[1] - M0[2]);
        rr[2] = (ti - M0[0]) * (ti - M0[1]) / (M0[2] - M0[0]) / (M0[2] - M0[1]);
        double E_x1 = M.eph_e[0][0] * rr[0] + M.eph_e[0][1] * rr[1] + M.eph_e[0][2] * rr[2];
        double E_y1 = M.eph_e[1][0] * rr[0] + M.eph_e[1][1] * rr[1] + M.eph_e[1][2] * rr[2];
        double E_z1 = M.eph_e[2][0] * rr[0] + M.eph_e[2][1] * rr[1] + M.eph_e[2][2] * rr[2];
        double S_x1 = M.eph_s[0][0] * rr[0] + M.eph_s[0][1] * rr[1] + M.eph_s[0][2] * rr[2];
        double S_y1 = M.eph_s[1][0] * rr[0] + M.eph_s[1][1] * rr[1] + M.eph_s[1][2] * rr[2];
        double S_z1 = M.eph_s[2][0] * rr[0] + M.eph_s[2][1] * rr[1] + M.eph_s[2][2] * rr[2];
        const double E = sqrt(E_x1 * E_x1 + E_y1 * E_y1 + E_z1 * E_z1);
        E_x1 = E_x1 / E; E_y1 = E_y1 / E; E_z1 = E_z1 / E;
        const double S = sqrt(S_x1 * S_x1 + S_y1 * S_y1 + S_z1 * S_z1);
        S_x1 = S_x1 / S; S_y1 = S_y1 / S; S_z1 = S_z1 / S;
        ex[i] = E_x1; ex[n + i] = E_y1; ex[2 * n + i] = E_z1;
        sx[i] = S_x1; sx[n + i] = S_y1; sx[2 * n + i] = S_z1;
    }
    float* ef = (float*)(base + L.off_ef);
    float* sf = (float*)(base + L.off_sf);
    for (int k = 0; k < 3; k++) {
        ef[k * n + i] = (float)ex[k * n + i];
        sf[k * n + i] = (float)sx[k * n + i];
    }
    const df H = df_from_double(hi), HH = df_from_double(0.5 * hi);
    const df H6 = df_from_double(hi / 6.0), H3 = df_from_double(hi / 3.0);
    float4* hq = (float4*)(base + L.off_hq);
    float4* hw = (float4*)(base + L.off_hw);
    hq[i] = float4{H.hi, H.lo, HH.hi, HH.lo};
    hw[i] = float4{H6.hi, H6.lo, H3.hi, H3.lo};
}

// Per-filter sums of the weights, in observation order (the sum_w of cuda.c:707-714, which
// does not depend on the parameters).
AST_HD void prep_obs_sums(const DevModel& M, char* base, const ObsLayout& L, int64_t n)
{
    double* sw = (double*)(base + L.off_sw);
    const float* w = (const float*)(base + L.off_w);
    const int32_t* f = (const int32_t*)(base + L.off_f);
    for (int m = 0; m < AST_MAX_FILTERS; m++) sw[m] = 0.0;
    for (int64_t i = 0; i < n; i++) sw[f[i]] = sw[f[i]] + (double)w[i];
}

}  // namespace ast
