/*
 * ref_harness_host.cu -- TEST INFRASTRUCTURE ONLY.  Host-side entry points around the
 * reference's own chi2one / x2params / params2x (cuda.c:81,1016,1120), for pinning the oracle.
 *
 * oracle/build_ref.sh compiles this file as the tail of one translation unit whose head is the
 * reference's asteroid.h and cuda.c, read in place under the reference checkout and streamed
 * to nvcc with the four device functions re-qualified __host__ __device__ and the per-build
 * constants (N_FILTERS, TIME_STEP) set.  Nothing of the reference is written to disk; the
 * result, oracle/_ref/libref_<variant>.so, is git-ignored.
 *
 * The functions take the engine's own table and observation layouts and convert them to the
 * reference's (Property[N_PARAMS][N_COLUMNS], Types[N_TYPES][N_SEG], CHI_FLOAT
 * Limits[2][N_TYPES], AoS struct obs_data, struct chi2_struct, struct x2_struct).
 */
#include <stdlib.h>
#include <string.h>

static int h_prop[N_PARAMS][N_COLUMNS];
static int h_types[N_TYPES][N_SEG];
static CHI_FLOAT h_limits[2][N_TYPES];

static int refh_load_tables(const int* property, int n_params, const int* types, int n_types,
                            const double* limits /* [2][max_types] */, int max_types)
{
    if (n_params != N_PARAMS || n_types != N_TYPES) return -1;
    for (int i = 0; i < N_PARAMS; i++)
        for (int j = 0; j < N_COLUMNS; j++) h_prop[i][j] = property[i * N_COLUMNS + j];
    for (int t = 0; t < N_TYPES; t++) {
        h_types[t][0] = types[t];
        h_limits[0][t] = (CHI_FLOAT)limits[t];
        h_limits[1][t] = (CHI_FLOAT)limits[max_types + t];
    }
    return 0;
}

extern "C" int refh_n_params(void) { return N_PARAMS; }
extern "C" int refh_n_types(void) { return N_TYPES; }
extern "C" int refh_chi_float_bytes(void) { return (int)sizeof(CHI_FLOAT); }
extern "C" double refh_time_step(void) { return TIME_STEP; }
extern "C" int refh_max_filters(void) { return N_FILTERS; }

/* chi2one on one parameter vector. */
extern "C" int refh_chi2(const int* property, int n_params, const int* types, int n_types,
                         const double* limits, int max_types,
                         int n_data, int n_filters, const double* mjd, const float* v, const float* w,
                         const int* filt, const double* e_unit, const double* s_unit,
                         const double* eph_e /* [3][3] */, const double* eph_s, const double* eph_mjd0,
                         int n_min, const float* t_min, const float* v_min,
                         const double* params, double* chi2_out, double* dv_out)
{
    if (refh_load_tables(property, n_params, types, n_types, limits, max_types)) return -1;
    if (n_filters > N_FILTERS) return -2;
    struct obs_data* data = (struct obs_data*)calloc((size_t)n_data, sizeof(struct obs_data));
    for (int i = 0; i < n_data; i++) {
        data[i].V = v[i];
        data[i].w = w[i];
        data[i].MJD = mjd[i];
        data[i].Filter = filt[i];
#ifndef INTERP
        data[i].E_x = e_unit[3 * i]; data[i].E_y = e_unit[3 * i + 1]; data[i].E_z = e_unit[3 * i + 2];
        data[i].S_x = s_unit[3 * i]; data[i].S_y = s_unit[3 * i + 1]; data[i].S_z = s_unit[3 * i + 2];
#endif
    }
    struct chi2_struct sp;
    memset(&sp, 0, sizeof(sp));
#ifdef INTERP
    for (int k = 0; k < 3; k++) {
        sp.E_x0[k] = eph_e[0 * 3 + k]; sp.E_y0[k] = eph_e[1 * 3 + k]; sp.E_z0[k] = eph_e[2 * 3 + k];
        sp.S_x0[k] = eph_s[0 * 3 + k]; sp.S_y0[k] = eph_s[1 * 3 + k]; sp.S_z0[k] = eph_s[2 * 3 + k];
        sp.MJD0[k] = eph_mjd0[k];
    }
#endif
#ifdef NUDGE
    sp.N_obs = n_min;
    for (int k = 0; k < n_min; k++) { sp.t_obs[k] = t_min[k]; sp.V_obs[k] = v_min[k]; }
#endif
    double p[N_PARAMS];
    for (int i = 0; i < N_PARAMS; i++) p[i] = params[i];
    CHI_FLOAT dv[N_FILTERS];
    for (int m = 0; m < N_FILTERS; m++) dv[m] = 0;
    CHI_FLOAT r = chi2one(p, data, n_data, n_filters, dv, 0, &sp, h_types);
    *chi2_out = (double)r;
    for (int m = 0; m < n_filters; m++) dv_out[m] = (double)dv[m];
    free(data);
    return 0;
}

extern "C" int refh_x2params(const int* property, int n_params, const int* types, int n_types,
                             const double* limits, int max_types, float ppsi1, float ppsi2, int reopt,
                             const double* x, double* params)
{
    if (refh_load_tables(property, n_params, types, n_types, limits, max_types)) return -1;
    struct x2_struct x2;
    memset(&x2, 0, sizeof(x2));
    x2.reopt = reopt;
#ifdef P_PSI
    x2.Ppsi1 = ppsi1;
    x2.Ppsi2 = ppsi2;
#endif
    CHI_FLOAT xc[N_PARAMS];
    for (int i = 0; i < N_PARAMS; i++) xc[i] = (CHI_FLOAT)x[i];
    int rc = x2params(xc, params, h_limits, &x2, h_prop, h_types);
    return rc;
}

extern "C" int refh_params2x(const int* property, int n_params, const int* types, int n_types,
                             const double* limits, int max_types, const double* params, double* x)
{
    if (refh_load_tables(property, n_params, types, n_types, limits, max_types)) return -1;
    struct x2_struct x2;
    memset(&x2, 0, sizeof(x2));
    CHI_FLOAT xc[N_PARAMS];
    double p[N_PARAMS];
    for (int i = 0; i < N_PARAMS; i++) p[i] = params[i];
    params2x(xc, p, h_limits, h_prop, h_types, &x2);
    for (int i = 0; i < N_PARAMS; i++) x[i] = (double)xc[i];
    return 0;
}

/* chi2one with Nplot > 0 on one parameter vector (the model-curve branch that chi2_plot calls,
 * cuda.c:699-704, cuda.c:1945): the reference writes Vmod + delta_V[0] into d_Vmod, whose host
 * copy this build reads back; with delta_V[0] = 0 that is the model magnitude itself.  Not for
 * -DNUDGE builds (the reference's NUDGE code does not support the plot branch, cuda.c:1937). */
extern "C" int refh_model_curve(const int* property, int n_params, const int* types, int n_types,
                                const double* limits, int max_types,
                                int n_data, int n_filters, const double* mjd, const float* v, const float* w,
                                const int* filt, const double* e_unit, const double* s_unit,
                                const double* eph_e /* [3][3] */, const double* eph_s, const double* eph_mjd0,
                                const double* params, double* vmod)
{
#ifdef NUDGE
    return -4;
#endif
    if (refh_load_tables(property, n_params, types, n_types, limits, max_types)) return -1;
    if (n_filters > N_FILTERS) return -2;
    if (n_data > NPLOT) return -3;
    struct obs_data* data = (struct obs_data*)calloc((size_t)n_data, sizeof(struct obs_data));
    for (int i = 0; i < n_data; i++) {
        data[i].V = v[i];
        data[i].w = w[i];
        data[i].MJD = mjd[i];
        data[i].Filter = filt[i];
#ifndef INTERP
        data[i].E_x = e_unit[3 * i]; data[i].E_y = e_unit[3 * i + 1]; data[i].E_z = e_unit[3 * i + 2];
        data[i].S_x = s_unit[3 * i]; data[i].S_y = s_unit[3 * i + 1]; data[i].S_z = s_unit[3 * i + 2];
#endif
    }
    struct chi2_struct sp;
    memset(&sp, 0, sizeof(sp));
#ifdef INTERP
    for (int k = 0; k < 3; k++) {
        sp.E_x0[k] = eph_e[0 * 3 + k]; sp.E_y0[k] = eph_e[1 * 3 + k]; sp.E_z0[k] = eph_e[2 * 3 + k];
        sp.S_x0[k] = eph_s[0 * 3 + k]; sp.S_y0[k] = eph_s[1 * 3 + k]; sp.S_z0[k] = eph_s[2 * 3 + k];
        sp.MJD0[k] = eph_mjd0[k];
    }
#endif
    double p[N_PARAMS];
    for (int i = 0; i < N_PARAMS; i++) p[i] = params[i];
    CHI_FLOAT dv[N_FILTERS];
    for (int m = 0; m < N_FILTERS; m++) dv[m] = 0;
    chi2one(p, data, n_data, n_filters, dv, n_data, &sp, h_types);
    for (int i = 0; i < n_data; i++) vmod[i] = d_Vmod[i];
    free(data);
    return 0;
}
