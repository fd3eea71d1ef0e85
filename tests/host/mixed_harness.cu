// Host build of the mixed-precision code (double-float arithmetic, the double-float magnitude and
// chi2_mixed) for the CPU tests: the product's headers compiled for the host, where the
// double-float operations map to IEEE float arithmetic (-ffp-contract=off keeps every rounding).
// vmod_fp64 below restates the reference's FP64 magnitude (cuda.c:195-217, 432-689) as the
// yardstick of vmod_df.
#include <string.h>
#include <vector>
#include "engine.cuh"
#include "mixed.cuh"
#include "prep.cuh"

using namespace ast;

namespace {

double vmod_fp64(const DevModel& M, const ObsView& o, const double* params, const double* ang, int i)
{
    const ast_type_ids& T = M.t;
#define AST_Q(tt) params[M.idx[T.tt]]
    const double th_M = AST_Q(theta_M), ph_M = AST_Q(phi_M);
    const double M_x = sin(th_M) * cos(ph_M), M_y = sin(th_M) * sin(ph_M), M_z = cos(th_M);
    const double XM = sqrt(M_z * M_z + M_x * M_x);
    const double XM_x = M_z / XM, XM_z = -M_x / XM;
    const double YM_x = M_y * XM_z, YM_y = M_z * XM_x - M_x * XM_z, YM_z = -M_y * XM_x;
    const double cos_phi = cos(ang[0]), sin_phi = sin(ang[0]);
    const double N_x = XM_x * cos_phi + YM_x * sin_phi, N_y = YM_y * sin_phi, N_z = XM_z * cos_phi + YM_z * sin_phi;
    const double p_x = N_y * M_z - N_z * M_y, p_y = N_z * M_x - N_x * M_z, p_z = N_x * M_y - N_y * M_x;
    const double cos_theta = cos(ang[1]), sin_theta = sin(ang[1]);
    double a_x = M_x * cos_theta + p_x * sin_theta, a_y = M_y * cos_theta + p_y * sin_theta,
           a_z = M_z * cos_theta + p_z * sin_theta;
    const double w_x = a_y * N_z - a_z * N_y, w_y = a_z * N_x - a_x * N_z, w_z = a_x * N_y - a_y * N_x;
    const double sin_psi = sin(ang[2]), cos_psi = cos(ang[2]);
    const double b_x = N_x * cos_psi + w_x * sin_psi, b_y = N_y * cos_psi + w_y * sin_psi,
                 b_z = N_z * cos_psi + w_z * sin_psi;
    const double c_x = a_y * b_z - a_z * b_y, c_y = a_z * b_x - a_x * b_z, c_z = a_x * b_y - a_y * b_x;
    const double E_x1 = o.ex[i], E_y1 = o.ey[i], E_z1 = o.ez[i], S_x1 = o.sx[i], S_y1 = o.sy[i], S_z1 = o.sz[i];
    if (M.flags & AST_BW_BALL) {
        const double cR = cos(AST_Q(phi_R)), sR = sin(AST_Q(phi_R)), cT = cos(AST_Q(theta_R)), sT = sin(AST_Q(theta_R));
        const double Nx = b_x * cR + c_x * sR, Ny = b_y * cR + c_y * sR, Nz = b_z * cR + c_z * sR;
        const double px = Ny * a_z - Nz * a_y, py = Nz * a_x - Nx * a_z, pz = Nx * a_y - Ny * a_x;
        a_x = a_x * cT + px * sT;
        a_y = a_y * cT + py * sT;
        a_z = a_z * cT + pz * sT;
        const double cos_zeta = a_x * E_x1 + a_y * E_y1 + a_z * E_z1;
        return -2.5 * log10(0.5 * (AST_Q(kappa) * (1 + cos_zeta) + 0.5 * (1 - cos_zeta)));
    }
    const double Ep_b = b_x * E_x1 + b_y * E_y1 + b_z * E_z1, Ep_c = c_x * E_x1 + c_y * E_y1 + c_z * E_z1,
                 Ep_a = a_x * E_x1 + a_y * E_y1 + a_z * E_z1;
    const double Sp_b = b_x * S_x1 + b_y * S_y1 + b_z * S_z1, Sp_c = c_x * S_x1 + c_y * S_y1 + c_z * S_z1,
                 Sp_a = a_x * S_x1 + a_y * S_y1 + a_z * S_z1;
    const double b = (M.flags & AST_BC) ? AST_Q(b) : AST_Q(b_tumb);
    const double c = (M.flags & AST_BC) ? AST_Q(c) : AST_Q(c_tumb);
#undef AST_Q
    const double sS = sqrt(Sp_b * Sp_b / (b * b) + Sp_c * Sp_c / (c * c) + Sp_a * Sp_a);
    const double sE = sqrt(Ep_b * Ep_b / (b * b) + Ep_c * Ep_c / (c * c) + Ep_a * Ep_a);
    const double cos_alpha_p = (Sp_b * Ep_b / (b * b) + Sp_c * Ep_c / (c * c) + Sp_a * Ep_a) / (sS * sE);
    const double sin_alpha_p = sqrt(1.0 - cos_alpha_p * cos_alpha_p);
    const double alpha_p = atan2(sin_alpha_p, cos_alpha_p);
    const double scalar = sqrt(sS * sS + sE * sE + 2 * sS * sE * cos_alpha_p);
    const double cos_lambda_p = (sS + sE * cos_alpha_p) / scalar;
    const double sin_lambda_p = sE * sin_alpha_p / scalar;
    const double lambda_p = atan2(sin_lambda_p, cos_lambda_p);
    return -2.5 * log10(b * c * sS * sE / scalar *
                        (cos(lambda_p - alpha_p) + cos_lambda_p +
                         sin_lambda_p * sin(lambda_p - alpha_p) * log(1.0 / tan(0.5 * lambda_p) / tan(0.5 * (alpha_p - lambda_p)))));
}

struct Block {
    DevModel dm;
    ObsLayout L;
    std::vector<unsigned char> img;
    ObsView o;
};

Block prepare(const ast_model* m, const ast_obs_set* obs)
{
    Block B;
    build_dev_model(m, obs, &B.dm);
    const int64_t n = obs->n_data;
    B.L = ObsLayout::make(n);
    obs_image(m, obs, B.L, B.img);
    char* b = (char*)B.img.data();
    for (int64_t i = 0; i < n; i++) prep_obs_point(B.dm, b, B.L, n, i);
    prep_obs_sums(B.dm, b, B.L, n);
    B.o = B.L.view(B.img.data(), n);
    return B;
}

std::vector<float4> table()
{
    std::vector<float4> t(kTrigTable);
    for (int k = 0; k < kTrigTable; k++) t[k] = trig_table_entry(k);
    return t;
}

}  // namespace

extern "C" {

// Double-float operations on n operand pairs (hi, lo interleaved): 0 add, 1 sloppy add, 2 mul,
// 3 mul without lo*lo, 4 div, 5 one-step div, 6 sqrt, 7 log, 8 atan2(x, y), 9 sin, 10 cos.
void h_df_op(int op, int n, const double* x, const double* y, double* out)
{
    const std::vector<float4> tab = table();
    for (int i = 0; i < n; i++) {
        const df a{(float)x[2 * i], (float)x[2 * i + 1]}, b{(float)y[2 * i], (float)y[2 * i + 1]};
        df r{0.f, 0.f}, s, c;
        switch (op) {
            case 0: r = df_add(a, b); break;
            case 1: r = df_add_fast(a, b); break;
            case 2: r = df_mul(a, b); break;
            case 3: r = df_mul_fast(a, b); break;
            case 4: r = df_div(a, b); break;
            case 5: r = df_div_fast(a, b); break;
            case 6: r = df_sqrt(a); break;
            case 7: r = df_log(a); break;
            case 8: r = df_atan2(a, b, tab.data()); break;
            case 9: df_sincos(a, tab.data(), &s, &c); r = s; break;
            default: df_sincos(a, tab.data(), &s, &c); r = c; break;
        }
        out[2 * i] = r.hi;
        out[2 * i + 1] = r.lo;
    }
}

// |vmod_df - vmod_fp64| at every observation for n_ang angle triples; returns the largest.
double h_vmod_diff(const ast_model* m, const ast_obs_set* obs, const double* params, const double* angs, int n_ang)
{
    Block B = prepare(m, obs);
    const std::vector<float4> tab = table();
    const DfFrame F = make_df_frame(B.dm, params);
    double mx = 0;
    for (int k = 0; k < n_ang; k++) {
        const df ad[3] = {df_from_double(angs[3 * k]), df_from_double(angs[3 * k + 1]), df_from_double(angs[3 * k + 2])};
        const double a2[3] = {df_to_double(ad[0]), df_to_double(ad[1]), df_to_double(ad[2])};
        for (int i = 0; i < obs->n_data; i++) {
            const double d = fabs(vmod_df(B.dm, B.o, F, ad, i, tab.data()) - vmod_fp64(B.dm, B.o, params, a2, i));
            if (!(d <= mx)) mx = d;
        }
    }
    return mx;
}

// chi2_mixed of one parameter vector on the host; rhs32 selects the FP32 right-hand side.
double h_chi2_mixed_rhs(const ast_model* m, const ast_obs_set* obs, const double* params, double* dv, int rhs32)
{
    Block B = prepare(m, obs);
    const std::vector<float4> tab = table();
    double d[AST_MAX_FILTERS];
    const double r = rhs32 ? chi2_mixed<double, true>(B.dm, B.o, params, d, tab.data())
                           : chi2_mixed<double, false>(B.dm, B.o, params, d, tab.data());
    for (int k = 0; k < obs->n_filters; k++) dv[k] = d[k];
    return r;
}

// chi2_mixed of one parameter vector on the host.
double h_chi2_mixed(const ast_model* m, const ast_obs_set* obs, const double* params, double* dv)
{
    Block B = prepare(m, obs);
    const std::vector<float4> tab = table();
    double d[AST_MAX_FILTERS];
    const double r = chi2_mixed<double>(B.dm, B.o, params, d, tab.data());
    for (int k = 0; k < obs->n_filters; k++) dv[k] = d[k];
    return r;
}

}  // extern "C"
