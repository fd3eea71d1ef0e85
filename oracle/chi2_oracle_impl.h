/*
 * chi2_oracle_impl.h -- TEST INFRASTRUCTURE ONLY (the oracle).  Included twice by
 * chi2_oracle.c: once with ORC_CF = double (the reference built with -DACC) and once with
 * ORC_CF = float (the default build), because CHI_FLOAT changes the rounding of the
 * simplex coordinates, of the limits and of the returned chi^2 (asteroid.h:24-28).
 *
 * A CPU restatement, in plain C, of the reference's chi^2 model and parameter maps:
 *   ode_func    cuda.c:13-77     Euler equations with torque / torque-free Euler angles
 *   chi2one     cuda.c:81-1011   RK4 + geometry + LS/BC/BW_BALL brightness + per-filter
 *                                delta_V and chi^2 + NUDGE merit
 *   x2params    cuda.c:1120-1319 dimensionless x -> physical parameters (hard limits, LAM/SAM,
 *                                P_PSI period -> L through the AGM elliptic integral)
 *   params2x    cuda.c:1016-1115 physical parameters -> x
 * Every expression keeps the reference's operand order and types (float where the reference
 * has float, C++ overload semantics for float math calls), so on the same machine it matches
 * a host build of the reference bit for bit; the pin is tests/test_oracle_pin.py.
 */

#define ORC_CAT2(a, b) a##_##b
#define ORC_CAT(a, b) ORC_CAT2(a, b)
#define ORC_FN(name) ORC_CAT(name, ORC_SUFFIX)

/* chi2one (cuda.c:81-1011).  Returns chi^2 (1e30 on the NUDGE "too many minima" exit, in
 * which case delta_V is left untouched, as in the reference). */
ORC_CF ORC_FN(orc_chi2one)(const ast_model* md, const ast_obs_set* o, const double* params,
                           ORC_CF* delta_V, double* vmod_out)
{
    const int flags = md->flags;
    const ast_type_ids* T = &md->ids;
    const int N_data = o->n_data, N_filters = o->n_filters;
    double sum_y2[AST_MAX_FILTERS], sum_y[AST_MAX_FILTERS], sum_w[AST_MAX_FILTERS];
    for (int m = 0; m < N_filters; m++) { sum_y2[m] = 0.0; sum_y[m] = 0.0; sum_w[m] = 0.0; }

    int M = 0;
    float t_mod[AST_M_MAX], V_mod[AST_M_MAX];
    float t_old[2] = {0, 0}, V_old[2] = {0, 0};

#define P(t) params[md->types[T->t]]
    double M_x = sin(P(theta_M)) * cos(P(phi_M));
    double M_y = sin(P(theta_M)) * sin(P(phi_M));
    double M_z = cos(P(theta_M));
    double XM = sqrt(M_z * M_z + M_x * M_x);
    double XM_x = M_z / XM;
    double XM_z = -M_x / XM;
    double YM_x = M_y * XM_z;
    double YM_y = M_z * XM_x - M_x * XM_z;
    double YM_z = -M_y * XM_x;
    double bt = P(b_tumb), ct = P(c_tumb);
    double Is = (1.0 + bt * bt) / (bt * bt + ct * ct);
    double Ii = (1.0 + ct * ct) / (bt * bt + ct * ct);
    double Is_inv = 1.0 / Is;
    double Ii_inv = 1.0 / Ii;
    double phi = P(phi_0);
    double theta = asin(sqrt((P(Es) - 1.0) / (sin(P(psi_0)) * sin(P(psi_0)) * (Ii_inv - Is_inv) + Is_inv - 1.0)));
    double psi = P(psi_0);
    double mu[6];
    double Omega_i = 0, Omega_s = 0, Omega_l = 0;
    const int torque = (flags & AST_TORQUE) != 0;
    if (torque) {
        mu[0] = (Is - 1.0) * Ii_inv;
        mu[1] = (1.0 - Ii) * Is_inv;
        mu[2] = Ii - Is;
        mu[3] = P(Ti);
        mu[4] = P(Ts);
        mu[5] = P(Tl);
        Omega_i = P(L) * Ii_inv * sin(theta) * sin(psi);
        Omega_s = P(L) * Is_inv * sin(theta) * cos(psi);
        Omega_l = P(L) * cos(theta);
    } else {
        double Ip = 0.5 * (Ii_inv + Is_inv);
        double Im = 0.5 * (Ii_inv - Is_inv);
        mu[0] = P(L);
        mu[1] = Ip;
        mu[2] = Im;
    }
    const double TIME_STEP = md->time_step;

    for (int i = 0; i < N_data; i++) {
        if (i > 0) {
            double t1 = o->mjd[i - 1], t2 = o->mjd[i];
            int N_steps = (int)((t2 - t1) / TIME_STEP + 1);
            double h = (t2 - t1) / N_steps;
            if (torque) {
                double y[6] = {Omega_i, Omega_s, Omega_l, phi, theta, psi};
                for (int l = 0; l < N_steps; l++) {
                    double f[6], K1[6], K2[6], K3[6], K4[6];
                    orc_ode_torque(y, K1, mu);
                    for (int j = 0; j < 6; j++) f[j] = y[j] + 0.5 * h * K1[j];
                    orc_ode_torque(f, K2, mu);
                    for (int j = 0; j < 6; j++) f[j] = y[j] + 0.5 * h * K2[j];
                    orc_ode_torque(f, K3, mu);
                    for (int j = 0; j < 6; j++) f[j] = y[j] + h * K3[j];
                    orc_ode_torque(f, K4, mu);
                    for (int j = 0; j < 6; j++) y[j] = y[j] + 1 / 6.0 * h * (K1[j] + 2 * K2[j] + 2 * K3[j] + K4[j]);
                }
                Omega_i = y[0]; Omega_s = y[1]; Omega_l = y[2];
                phi = y[3]; theta = y[4]; psi = y[5];
            } else {
                double y[3] = {phi, theta, psi};
                for (int l = 0; l < N_steps; l++) {
                    double f[3], K1[3], K2[3], K3[3], K4[3];
                    orc_ode_free(y, K1, mu);
                    for (int j = 0; j < 3; j++) f[j] = y[j] + 0.5 * h * K1[j];
                    orc_ode_free(f, K2, mu);
                    for (int j = 0; j < 3; j++) f[j] = y[j] + 0.5 * h * K2[j];
                    orc_ode_free(f, K3, mu);
                    for (int j = 0; j < 3; j++) f[j] = y[j] + h * K3[j];
                    orc_ode_free(f, K4, mu);
                    for (int j = 0; j < 3; j++) y[j] = y[j] + 1 / 6.0 * h * (K1[j] + 2 * K2[j] + 2 * K3[j] + K4[j]);
                }
                phi = y[0]; theta = y[1]; psi = y[2];
            }
        }

        /* Body axes from the Euler angles (cuda.c:432-473). */
        double cos_phi = cos(phi);
        double sin_phi = sin(phi);
        double N_x = XM_x * cos_phi + YM_x * sin_phi;
        double N_y = YM_y * sin_phi;
        double N_z = XM_z * cos_phi + YM_z * sin_phi;
        double p_x = N_y * M_z - N_z * M_y;
        double p_y = N_z * M_x - N_x * M_z;
        double p_z = N_x * M_y - N_y * M_x;
        double cos_theta = cos(theta);
        double sin_theta = sin(theta);
        double a_x = M_x * cos_theta + p_x * sin_theta;
        double a_y = M_y * cos_theta + p_y * sin_theta;
        double a_z = M_z * cos_theta + p_z * sin_theta;
        double w_x = a_y * N_z - a_z * N_y;
        double w_y = a_z * N_x - a_x * N_z;
        double w_z = a_x * N_y - a_y * N_x;
        double sin_psi = sin(psi);
        double cos_psi = cos(psi);
        double b_x = N_x * cos_psi + w_x * sin_psi;
        double b_y = N_y * cos_psi + w_y * sin_psi;
        double b_z = N_z * cos_psi + w_z * sin_psi;
        double c_x = a_y * b_z - a_z * b_y;
        double c_y = a_z * b_x - a_x * b_z;
        double c_z = a_x * b_y - a_y * b_x;

        if (flags & AST_BW_BALL) {
            /* Brightness frame rotation by theta_R, phi_R (cuda.c:475-497). */
            cos_phi = cos(P(phi_R));
            sin_phi = sin(P(phi_R));
            N_x = b_x * cos_phi + c_x * sin_phi;
            N_y = b_y * cos_phi + c_y * sin_phi;
            N_z = b_z * cos_phi + c_z * sin_phi;
            p_x = N_y * a_z - N_z * a_y;
            p_y = N_z * a_x - N_x * a_z;
            p_z = N_x * a_y - N_y * a_x;
            cos_theta = cos(P(theta_R));
            sin_theta = sin(P(theta_R));
            a_x = a_x * cos_theta + p_x * sin_theta;
            a_y = a_y * cos_theta + p_y * sin_theta;
            a_z = a_z * cos_theta + p_z * sin_theta;
        }

        double E_x1, E_y1, E_z1, S_x1, S_y1, S_z1;
        if (flags & AST_INTERP) {
            /* In-kernel 3-point interpolation at asteroid time (cuda.c:522-545). */
            const double* M0 = o->eph_mjd0;
            double t = o->mjd[i];
            double rr[3];
            rr[0] = (t - M0[1]) * (t - M0[2]) / (M0[0] - M0[1]) / (M0[0] - M0[2]);
            rr[1] = (t - M0[0]) * (t - M0[2]) / (M0[1] - M0[0]) / (M0[1] - M0[2]);
            rr[2] = (t - M0[0]) * (t - M0[1]) / (M0[2] - M0[0]) / (M0[2] - M0[1]);
            E_x1 = o->eph_e[0][0] * rr[0] + o->eph_e[0][1] * rr[1] + o->eph_e[0][2] * rr[2];
            E_y1 = o->eph_e[1][0] * rr[0] + o->eph_e[1][1] * rr[1] + o->eph_e[1][2] * rr[2];
            E_z1 = o->eph_e[2][0] * rr[0] + o->eph_e[2][1] * rr[1] + o->eph_e[2][2] * rr[2];
            S_x1 = o->eph_s[0][0] * rr[0] + o->eph_s[0][1] * rr[1] + o->eph_s[0][2] * rr[2];
            S_y1 = o->eph_s[1][0] * rr[0] + o->eph_s[1][1] * rr[1] + o->eph_s[1][2] * rr[2];
            S_z1 = o->eph_s[2][0] * rr[0] + o->eph_s[2][1] * rr[1] + o->eph_s[2][2] * rr[2];
            double E = sqrt(E_x1 * E_x1 + E_y1 * E_y1 + E_z1 * E_z1);
            E_x1 = E_x1 / E; E_y1 = E_y1 / E; E_z1 = E_z1 / E;
            double S = sqrt(S_x1 * S_x1 + S_y1 * S_y1 + S_z1 * S_z1);
            S_x1 = S_x1 / S; S_y1 = S_y1 / S; S_z1 = S_z1 / S;
        } else {
            E_x1 = o->e_unit[3 * i]; E_y1 = o->e_unit[3 * i + 1]; E_z1 = o->e_unit[3 * i + 2];
            S_x1 = o->s_unit[3 * i]; S_y1 = o->s_unit[3 * i + 1]; S_z1 = o->s_unit[3 * i + 2];
        }

        double Ep_b = b_x * E_x1 + b_y * E_y1 + b_z * E_z1;
        double Ep_c = c_x * E_x1 + c_y * E_y1 + c_z * E_z1;
        double Ep_a = a_x * E_x1 + a_y * E_y1 + a_z * E_z1;
        double Sp_b = b_x * S_x1 + b_y * S_y1 + b_z * S_z1;
        double Sp_c = c_x * S_x1 + c_y * S_y1 + c_z * S_z1;
        double Sp_a = a_x * S_x1 + a_y * S_y1 + a_z * S_z1;
        if (orc_geo_out) {
            /* compute_rgb's inputs at this point (cuda.c:576-586). */
            double* g = orc_geo_out + 20 * (int64_t)i;
            g[0] = (flags & AST_BC) ? P(b) : P(b_tumb);
            g[1] = (flags & AST_BC) ? P(c) : P(c_tumb);
            g[2] = E_x1; g[3] = E_y1; g[4] = E_z1;
            g[5] = Ep_b; g[6] = Ep_c; g[7] = Ep_a;
            g[8] = Sp_b; g[9] = Sp_c; g[10] = Sp_a;
            g[11] = b_x; g[12] = b_y; g[13] = b_z;
            g[14] = c_x; g[15] = c_y; g[16] = c_z;
            g[17] = a_x; g[18] = a_y; g[19] = a_z;
        }

        double Vmod;
        if (flags & AST_BW_BALL) {
            /* Black-and-white ball (cuda.c:596-607). */
            double cos_zeta = Ep_a;
            Vmod = -2.5 * log10(0.5 * (P(kappa) * (1 + cos_zeta) + 0.5 * (1 - cos_zeta)));
        } else {
            /* Lommel-Seeliger ellipsoid, Muinonen & Lumme 2015 eqs. 10-14 (cuda.c:664-689). */
            double b = (flags & AST_BC) ? P(b) : P(b_tumb);
            double c = (flags & AST_BC) ? P(c) : P(c_tumb);
            double scalar_Sun = sqrt(Sp_b * Sp_b / (b * b) + Sp_c * Sp_c / (c * c) + Sp_a * Sp_a);
            double scalar_Earth = sqrt(Ep_b * Ep_b / (b * b) + Ep_c * Ep_c / (c * c) + Ep_a * Ep_a);
            double cos_alpha_p = (Sp_b * Ep_b / (b * b) + Sp_c * Ep_c / (c * c) + Sp_a * Ep_a) / (scalar_Sun * scalar_Earth);
            double sin_alpha_p = sqrt(1.0 - cos_alpha_p * cos_alpha_p);
            double alpha_p = atan2(sin_alpha_p, cos_alpha_p);
            double scalar = sqrt(scalar_Sun * scalar_Sun + scalar_Earth * scalar_Earth + 2 * scalar_Sun * scalar_Earth * cos_alpha_p);
            double cos_lambda_p = (scalar_Sun + scalar_Earth * cos_alpha_p) / scalar;
            double sin_lambda_p = scalar_Earth * sin_alpha_p / scalar;
            double lambda_p = atan2(sin_lambda_p, cos_lambda_p);
            Vmod = -2.5 * log10(b * c * scalar_Sun * scalar_Earth / scalar *
                                (cos(lambda_p - alpha_p) + cos_lambda_p +
                                 sin_lambda_p * sin(lambda_p - alpha_p) * log(1.0 / tan(0.5 * lambda_p) / tan(0.5 * (alpha_p - lambda_p)))));
        }

        if (vmod_out) vmod_out[i] = Vmod;
        {   /* Per-filter sums (cuda.c:707-714). */
            int m = o->filter[i];
            double y = o->v[i] - Vmod;
            sum_y2[m] = sum_y2[m] + y * y * o->w[i];
            sum_y[m] = sum_y[m] + y * o->w[i];
            sum_w[m] = sum_w[m] + o->w[i];
        }

        if (flags & AST_NUDGE) {
            /* Model minima (V maxima) near observed minima (cuda.c:716-760). */
            if (i < 2) {
                t_old[i] = (float)o->mjd[i];
                V_old[i] = (float)Vmod;
            } else {
                if (V_old[1] > V_old[0] && V_old[1] >= Vmod) {
                    int local = 0;
                    for (int ii = 0; ii < o->n_minima; ii++)
                        if (fabsf(t_old[1] - o->t_min[ii]) < ORC_DT_MAX2) local = 1;
                    if (local) {
                        M++;
                        if (M > AST_M_MAX) return (ORC_CF)1e30;
                        double t = o->mjd[i];
                        double a = ((Vmod - V_old[1]) / (t - t_old[1]) - (V_old[1] - V_old[0]) / (t_old[1] - t_old[0])) / (t - t_old[0]);
                        double b = (V_old[1] - V_old[0]) / (t_old[1] - t_old[0]) - a * (t_old[1] + t_old[0]);
                        double c = V_old[1] - a * t_old[1] * t_old[1] - b * t_old[1];
                        t_mod[M - 1] = (float)(-b / 2.0 / a);
                        V_mod[M - 1] = (float)(a * t_mod[M - 1] * t_mod[M - 1] + b * t_mod[M - 1] + c);
                    }
                }
                t_old[0] = t_old[1];
                V_old[0] = V_old[1];
                t_old[1] = (float)o->mjd[i];
                V_old[1] = (float)Vmod;
            }
        }
    }

    /* chi^2 per filter and delta_V (cuda.c:887-910); under RMSD the root of the summed chi^2 over
     * the summed weights, SUM_w in CHI_FLOAT (cuda.c:890,901-908). */
    ORC_CF chi2m, chi2a = 0.0, SUM_w = 0.0;
    for (int m = 0; m < N_filters; m++) {
        chi2m = (ORC_CF)(sum_y2[m] - sum_y[m] * sum_y[m] / sum_w[m]);
        chi2a = chi2a + chi2m;
        delta_V[m] = (ORC_CF)(sum_y[m] / sum_w[m]);
        SUM_w = SUM_w + sum_w[m];
    }
    if (flags & AST_RMSD)
        chi2a = sqrt(chi2a / SUM_w);
    else
        chi2a = chi2a / (ORC_CF)(N_data - md->n_params - N_filters);

    if (flags & AST_NUDGE) {
        /* Reward / punishment factors (cuda.c:912-993). */
        float S_M = 0.0f;
        float P_tot = 1.0f;
        for (int imod = 0; imod < M; imod++) {
            for (int iobs = 0; iobs < o->n_minima; iobs++) {
                float dt = fabsf(t_mod[imod] - o->t_min[iobs]);
                if (dt < ORC_DT_MAX2) {
                    if (dt > ORC_DT_MAX) {
                        float x = (ORC_DT_MAX2 - dt) / (ORC_DT_MAX2 - ORC_DT_MAX);
                        S_M = (float)(S_M + x * x * (-2.0 * x + 3.0));
                    } else {
                        S_M = (float)(S_M + 1.0);
                        float dV = (float)(V_mod[imod] + delta_V[0] - o->v_min[iobs]);
                        float x = sqrtf(dt * dt / ORC_DT_MAX / ORC_DT_MAX + dV * dV / ORC_DV_MAX / ORC_DV_MAX);
                        if (x < 1.0f) {
                            float P_i = ORC_L_A * x * x / (x * x + ORC_L_RC2);
                            P_tot = (float)(P_tot * (ORC_P_MIN * (1.0 + ORC_P_MIN2 * P_i)));
                        }
                    }
                }
            }
        }
        P_tot = powf(P_tot, (float)(1.0 / o->n_minima));
        if (P_tot < ORC_P_MIN) P_tot = ORC_P_MIN;
        if (chi2a > ORC_CHI2_1)
            P_tot = 1.0f;
        else if (chi2a > ORC_CHI2_0) {
            float x = (float)((ORC_CHI2_1 - chi2a) / (ORC_CHI2_1 - ORC_CHI2_0));
            float beta = x * x * (-2 * x + 3);
            P_tot = powf(P_tot, beta);
        }
        float P_M;
        if (S_M < ORC_M_MAX2)
            P_M = 1.0f;
        else if (S_M < AST_M_MAX) {
            float x = (S_M - ORC_M_MAX2) / (AST_M_MAX - ORC_M_MAX2);
            P_M = (float)(1.0 + 3 * x * x * (-2 * x + 3));
        } else
            P_M = 4.0f;
        chi2a = chi2a * P_tot * P_M;
    }
    return chi2a;
#undef P
}

/* x2params (cuda.c:1120-1319).  Returns nonzero when x is outside a hard limit or a BC
 * shape deviates by more than BC_DEV_MAX. */
int ORC_FN(orc_x2params)(const ast_model* md, int reopt, const ORC_CF* x, double* params)
{
    const ast_type_ids* T = &md->ids;
    const int N = md->n_params;
    int LAM = 0;
    for (int i = 0; i < N; i++) {
        int per = md->property[i][AST_P_PERIODIC];
        if (md->property[i][AST_P_TYPE] == T->Es) LAM = x[i] >= 0.5;
        if ((x[i] < 0.0 && (per == AST_HARD_BOTH || per == AST_HARD_LEFT || (LAM == 0 && per == AST_PERIODIC_LAM))) ||
            (x[i] > 1.0 && (per == AST_HARD_BOTH || per == AST_HARD_RIGHT || (LAM == 0 && per == AST_PERIODIC_LAM))))
            return 1;
    }
    double log_c_tumb = 0, log_b_tumb = 0, Is = 0, Ii = 0, psi_min = 0, psi_max = 0, log_c = 0;
    const int p_psi = (md->flags & AST_P_PSI) != 0;
    for (int i = 0; i < N; i++) {
        int pt = md->property[i][AST_P_TYPE];
        ORC_CF L0 = (ORC_CF)md->limits[0][pt], L1 = (ORC_CF)md->limits[1][pt];
        if (pt == T->b_tumb) {
            log_b_tumb = log_c_tumb * (ORC_CF)(x[i] * (L1 - L0) + L0);
            params[i] = exp(log_b_tumb);
            double b_tumb = params[i];
            double c_tumb = params[md->types[T->c_tumb]];
            Is = (1.0 + b_tumb * b_tumb) / (b_tumb * b_tumb + c_tumb * c_tumb);
            Ii = (1.0 + c_tumb * c_tumb) / (b_tumb * b_tumb + c_tumb * c_tumb);
        } else if (pt == T->Es) {
            if (LAM) {
                params[i] = 2.0 * (x[i] - 0.5) * (1.0 - 1.0 / Ii) + 1.0 / Ii;
                psi_min = 0.0;
                psi_max = 2.0 * ORC_PI;
            } else {
                params[i] = 2.0 * x[i] * (1.0 / Ii - 1.0 / Is) + 1.0 / Is;
                psi_max = atan(sqrt(Ii * (Is - 1.0 / params[i]) / Is / (1.0 / params[i] - Ii)));
                psi_min = -psi_max;
            }
        } else if (pt == T->psi_0) {
            params[i] = x[i] * (psi_max - psi_min) + psi_min;
        } else if ((md->flags & AST_BC) && pt == T->b) {
            double log_b = log_c * (ORC_CF)(x[i] * (L1 - L0) + L0);
            if (fabs(log_b - log_b_tumb) > ORC_BC_DEV_MAX) return 1;
            params[i] = exp(log_b);
        } else if (md->property[i][AST_P_PERIODIC] == AST_PERIODIC) {
            params[i] = x[i] * 2.0 * ORC_PI;
        } else if (md->property[i][AST_P_INDEPENDENT] == 1) {
            if (!p_psi || pt != T->L || reopt) params[i] = (ORC_CF)(x[i] * (L1 - L0) + L0);
            if (pt == T->c_tumb) {
                log_c_tumb = params[i];
                params[i] = exp(log_c_tumb);
            } else if ((md->flags & AST_BC) && pt == T->c) {
                log_c = params[i];
                if (fabs(log_c - log_c_tumb) > ORC_BC_DEV_MAX) return 1;
                params[i] = exp(log_c);
            } else if ((md->flags & AST_BW_BALL) && pt == T->kappa) {
                params[i] = exp(params[i]);
            } else if (pt == T->L && !reopt && p_psi) {
                /* 1/Ppsi -> L through the complete elliptic integral K(k^2) (cuda.c:1260-1285). */
                params[i] = x[i] * (ORC_CF)(md->ppsi2 - md->ppsi1) + md->ppsi1;
                double Es = params[md->types[T->Es]];
                double Einv = 1.0 / Es;
                double k2;
                if (LAM)
                    k2 = (Is - Ii) * (Einv - 1.0) / ((Ii - 1.0) * (Is - Einv));
                else
                    k2 = (Ii - 1.0) * (Is - Einv) / ((Is - Ii) * (Einv - 1.0));
                double a = 1.0, g = sqrt(1.0 - k2), a1, g1;
                for (int ii = 0; ii < 5; ii++) {
                    a1 = 0.5 * (a + g);
                    g1 = sqrt(a * g);
                    a = a1; g = g1;
                }
                if (LAM)
                    params[i] = 4.0 * params[i] * ORC_PI / (a + g) * sqrt(Ii * Is / (Es * (Ii - 1.0) * (Is - Einv)));
                else
                    params[i] = 4.0 * params[i] * ORC_PI / (a + g) * sqrt(Ii * Is / (Es * (Is - Ii) * (Einv - 1.0)));
            }
        }
    }
    return 0;
}

/* params2x (cuda.c:1016-1115). */
void ORC_FN(orc_params2x)(const ast_model* md, const double* params, ORC_CF* x)
{
    const ast_type_ids* T = &md->ids;
    const int N = md->n_params;
    double b_tumb = params[md->types[T->b_tumb]];
    double c_tumb = params[md->types[T->c_tumb]];
    double Is = (1.0 + b_tumb * b_tumb) / (b_tumb * b_tumb + c_tumb * c_tumb);
    double Ii = (1.0 + c_tumb * c_tumb) / (b_tumb * b_tumb + c_tumb * c_tumb);
    int LAM = 0, i_Es = md->types[T->Es];
    for (int i = 0; i < N; i++) {
        int pt = md->property[i][AST_P_TYPE];
        ORC_CF L0 = (ORC_CF)md->limits[0][pt], L1 = (ORC_CF)md->limits[1][pt];
        if (md->property[i][AST_P_FROZEN] != 0) { x[i] = 0; continue; }
        if (md->property[i][AST_P_INDEPENDENT] == 1) {
            double par = params[i];
            if (md->property[i][AST_P_PERIODIC] == 1) {
                x[i] = (ORC_CF)(par / (2 * ORC_PI));
                x[i] = x[i] - ORC_FLOOR(x[i]);
            } else {
                if ((md->flags & AST_BC) && pt == T->c) {
                    ORC_CF C0 = (ORC_CF)md->limits[0][T->c_tumb], C1 = (ORC_CF)md->limits[1][T->c_tumb];
                    x[i] = (ORC_CF)((log(params[i]) - C0) / (ORC_CF)(C1 - C0));
                    continue;
                }
                if (pt == T->c_tumb) par = log(par);
                if ((md->flags & AST_BW_BALL) && pt == T->kappa) par = log(par);
                x[i] = (ORC_CF)((par - L0) / (ORC_CF)(L1 - L0));
            }
        } else {
            if (pt == T->b_tumb) {
                double par = log(b_tumb) / log(c_tumb);
                x[i] = (ORC_CF)((par - L0) / (ORC_CF)(L1 - L0));
            } else if (pt == T->Es) {
                i_Es = i;
                LAM = params[i] > 1.0 / Ii;
                if (LAM)
                    x[i] = (ORC_CF)(0.5 * ((params[i] - 1.0 / Ii) / (1.0 - 1.0 / Ii) + 1.0));
                else
                    x[i] = (ORC_CF)(0.5 * (params[i] - 1.0 / Is) / (1.0 / Ii - 1.0 / Is));
            } else if (pt == T->psi_0) {
                double psi_min, psi_max;
                if (LAM) {
                    psi_min = 0.0;
                    psi_max = 2.0 * ORC_PI;
                } else {
                    psi_max = atan(sqrt(Ii * (Is - 1.0 / params[i_Es]) / Is / (1.0 / params[i_Es] - Ii)));
                    psi_min = -psi_max;
                }
                x[i] = (ORC_CF)((params[i] - psi_min) / (psi_max - psi_min));
            } else if ((md->flags & AST_BC) && pt == T->b) {
                double par = log(params[i]) / log(params[md->types[T->c]]);
                x[i] = (ORC_CF)((par - L0) / (ORC_CF)(L1 - L0));
            }
        }
    }
}

#undef ORC_FN
#undef ORC_CAT
#undef ORC_CAT2
