/*
 * misc.c -- host helpers that keep the roles of the reference's misc.c:
 *   ast_quadratic_interpolation  quadratic_interpolation (misc.c:20-35)
 *   ast_read_minima              prepare_chi2_params (misc.c:279-323), observed.min for NUDGE
 *   ast_format_result            the output line of asteroid.c:798-811
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include "asteroid_gb300.h"
#include "host_internal.h"

#define AST_LINE 1024

void ast_quadratic_interpolation(const double mjd0[3], const double e[3][3], const double s[3][3],
                                 double t, double out_e[3], double out_s[3])
{
    /* Lagrange basis on the three window times, in the reference's operation order
     * (misc.c:24-32) so the host and device interpolations agree bit for bit. */
    double rr[3];
    rr[0] = (t - mjd0[1]) * (t - mjd0[2]) / (mjd0[0] - mjd0[1]) / (mjd0[0] - mjd0[2]);
    rr[1] = (t - mjd0[0]) * (t - mjd0[2]) / (mjd0[1] - mjd0[0]) / (mjd0[1] - mjd0[2]);
    rr[2] = (t - mjd0[0]) * (t - mjd0[1]) / (mjd0[2] - mjd0[0]) / (mjd0[2] - mjd0[1]);
    for (int k = 0; k < 3; k++) {
        out_e[k] = e[k][0] * rr[0] + e[k][1] * rr[1] + e[k][2] * rr[2];
        out_s[k] = s[k][0] * rr[0] + s[k][1] * rr[1] + s[k][2] * rr[2];
    }
}

int ast_plot_grid(const ast_host_data* d, int32_t interp, int32_t n_plot, double* t, double* e_unit, double* s_unit)
{
    if (!d || !t || !e_unit || !s_unit || n_plot < 2)
        return ast_set_error(AST_E_INVALID, "ast_plot_grid: bad argument");
    const int64_t n = d->obs.n_data;
    /* The ephemeris times of the grid are relative to hMJD0 in both modes (read_data.c:317-320). */
    double mjd0[3];
    for (int k = 0; k < 3; k++) mjd0[k] = interp ? d->obs.eph_mjd0[k] : d->obs.eph_mjd0[k] - d->hmjd0;
    const double h = d->mjd[n - 1] / (n_plot - 1);
    for (int32_t i = 0; i < n_plot; i++) {
        double* ev = &e_unit[3 * i];
        double* sv = &s_unit[3 * i];
        if (i == 0 || i == n_plot - 1) {
            /* The two ends are the first and the last observation (read_data.c:326-341). */
            const int64_t j = i == 0 ? 0 : n - 1;
            t[i] = d->mjd[j];
            for (int k = 0; k < 3; k++) { ev[k] = d->e_unit[3 * j + k]; sv[k] = d->s_unit[3 * j + k]; }
            continue;
        }
        t[i] = i * h;
        ast_quadratic_interpolation(mjd0, d->obs.eph_e, d->obs.eph_s, t[i], ev, sv);
        const double E = sqrt(ev[0] * ev[0] + ev[1] * ev[1] + ev[2] * ev[2]);
        const double S = sqrt(sv[0] * sv[0] + sv[1] * sv[1] + sv[2] * sv[2]);
        for (int k = 0; k < 3; k++) { ev[k] = ev[k] / E; sv[k] = sv[k] / S; }
    }
    return AST_OK;
}

int ast_read_minima(const char* path, ast_host_data* d)
{
    if (!path || !d) return ast_set_error(AST_E_INVALID, "ast_read_minima: NULL argument");
    FILE* f1 = fopen(path, "r");
    if (!f1) return ast_set_error(AST_E_IO, "%s does not exist!", path);
    char line[AST_LINE];
    int i = -1;
    const double small = 0.05;
    double t_last = d->mjd[d->obs.n_data - 1] + d->hmjd0;
    while (fgets(line, sizeof(line), f1)) {
        float t_obs, v_obs;
        if (sscanf(line, "%f %f", &t_obs, &v_obs) != 2) continue;
        if (t_obs >= d->hmjd0 - small && t_obs <= t_last + small) {
            i++;
            if (i >= AST_NOBS_MAX) {
                fclose(f1);
                return ast_set_error(AST_E_TOO_LARGE, "Too many lines in observed.min file! (>NOBS_MAX)!");
            }
            d->obs.t_min[i] = (float)(t_obs - d->hmjd0);
            d->obs.v_min[i] = v_obs;
        }
    }
    fclose(f1);
    d->obs.n_minima = i + 1;
    if (d->obs.n_minima < 1) return ast_set_error(AST_E_IO, "No local minima in the data range!");
    return AST_OK;
}

int ast_format_result(char* buf, int64_t cap, double chi2, const double* dv, int32_t n_filters,
                      const double* params, int32_t n_params)
{
    if (!buf || cap <= 0) return ast_set_error(AST_E_INVALID, "ast_format_result: no buffer");
    int64_t k = 0;
    k += snprintf(buf + k, (size_t)(cap - k), "%13.6e ", chi2);
    for (int m = 0; m < n_filters && k < cap; m++) k += snprintf(buf + k, (size_t)(cap - k), "%13.6e ", dv[m]);
    for (int j = 0; j < n_params && k < cap; j++) k += snprintf(buf + k, (size_t)(cap - k), "%15.11f ", params[j]);
    if (k < cap) k += snprintf(buf + k, (size_t)(cap - k), "\n");
    if (k >= cap) return ast_set_error(AST_E_TOO_LARGE, "ast_format_result: buffer too small");
    return (int)k;
}
