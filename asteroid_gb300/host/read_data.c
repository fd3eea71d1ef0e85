/*
 * read_data.c -- light-curve and ephemeris readers (host, C).
 *
 * Keeps the role of the reference's read_data.c: it reads the reference's own file formats
 * and applies the same conversions, so a light curve fitted here is the light curve the
 * reference fits.
 *
 *   light curve:  one observation per line, "filter MJD V sgm aux" (README.md:11-24);
 *                 MJD strictly increasing (read_data.c:81-85); w = 1/sgm^2 (read_data.c:87);
 *                 filters numbered in order of first appearance (read_data.c:88-114).
 *   ephemerides:  asteroid.eph, earth.eph, sun.eph, HORIZONS "VECTORS" output: data between
 *                 "$$SOE" and "$$EOE", alternating a JD line and an "X Y Z" line
 *                 (read_data.c:127-232).  A 3-point window slides along the file; each
 *                 observation time t with MJD0[0] <= t < MJD0[2] takes E and S from
 *                 second-order interpolation in the window that first brackets it.
 *   conversion:   for filters other than 'W', V += 5 log10(1/E * 1/S) (read_data.c:259-260);
 *                 for filters other than 'W' and 'D', asteroid time = MJD - E/c
 *                 (read_data.c:265-270); all times minus the first one (hMJD0); E, S unit.
 *                 Under INTERP the window times are shifted by hMJD0 (read_data.c:298-302).
 *   observed.min: "MJD_min V_min" read as floats, kept within 0.05 d of the data range,
 *                 at most 10 (misc.c:279-323).
 *
 * Deviations, all on inputs the reference mishandles: a last line without a newline is
 * read (the reference counts newline characters only), blank lines are skipped, and an
 * observation no ephemeris window brackets is an error instead of uninitialised memory.
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include "asteroid_gb300.h"
#include "host_internal.h"

#define AST_LIGHT_SPEED 173.144632674 /* au/day, asteroid.h:287 */
#define AST_LINE 1024

static int is_blank(const char* line)
{
    for (; *line; line++)
        if (*line != ' ' && *line != '\t' && *line != '\r' && *line != '\n') return 0;
    return 1;
}

static FILE* open_in(const char* dir, const char* name, char* path, size_t cap)
{
    snprintf(path, cap, "%s/%s", (dir && dir[0]) ? dir : ".", name);
    return fopen(path, "r");
}

/* Advance to the line after "$$SOE". */
static int seek_soe(FILE* fp)
{
    char line[AST_LINE];
    while (fgets(line, sizeof(line), fp))
        if (strncmp(line, "$$SOE", 5) == 0) return 1;
    return 0;
}

void ast_free_host_data(ast_host_data* d)
{
    if (!d) return;
    free(d->mjd); free(d->v); free(d->w); free(d->filter);
    free(d->e_unit); free(d->s_unit); free(d->mjd_obs);
    free(d);
}

int ast_read_data(const char* lc_path, const char* eph_dir, int32_t interp,
                  int32_t max_filters, ast_host_data** out)
{
    if (!lc_path || !out) return ast_set_error(AST_E_INVALID, "ast_read_data: NULL argument");
    if (max_filters <= 0 || max_filters > AST_MAX_FILTERS) max_filters = AST_MAX_FILTERS;
    *out = NULL;
    FILE* fp = fopen(lc_path, "r");
    if (!fp) return ast_set_error(AST_E_IO, "Input file %s does not exist!", lc_path);

    /* Pass 1: count observation lines. */
    char line[AST_LINE];
    int64_t n = 0;
    while (fgets(line, sizeof(line), fp))
        if (!is_blank(line)) n++;
    if (n == 0) { fclose(fp); return ast_set_error(AST_E_IO, "%s: no observations", lc_path); }
    if (n > AST_MAX_DATA) {
        fclose(fp);
        return ast_set_error(AST_E_TOO_LARGE, "Error: N_data (%lld) > MAX_DATA!", (long long)n);
    }

    ast_host_data* d = (ast_host_data*)calloc(1, sizeof(ast_host_data));
    if (!d) { fclose(fp); return ast_set_error(AST_E_NOMEM, "ast_read_data: out of host memory"); }
    d->mjd = (double*)calloc((size_t)n, sizeof(double));
    d->v = (float*)calloc((size_t)n, sizeof(float));
    d->w = (float*)calloc((size_t)n, sizeof(float));
    d->filter = (int32_t*)calloc((size_t)n, sizeof(int32_t));
    d->e_unit = (double*)calloc((size_t)n * 3, sizeof(double));
    d->s_unit = (double*)calloc((size_t)n * 3, sizeof(double));
    d->mjd_obs = (double*)calloc((size_t)n, sizeof(double));
    if (!d->mjd || !d->v || !d->w || !d->filter || !d->e_unit || !d->s_unit || !d->mjd_obs) {
        fclose(fp); ast_free_host_data(d);
        return ast_set_error(AST_E_NOMEM, "ast_read_data: out of host memory");
    }

    /* Pass 2: parse (read_data.c:74-116). */
    rewind(fp);
    int64_t i = 0;
    int32_t nf = 0, w_filter = -1, d_filter = -1;
    while (fgets(line, sizeof(line), fp)) {
        if (is_blank(line)) continue;
        char filt;
        double mjd1, v1, sgm;
        const char* p = line;
        while (*p == ' ' || *p == '\t') p++;
        if (sscanf(p, "%c %lf %lf %lf", &filt, &mjd1, &v1, &sgm) != 4) {
            fclose(fp); ast_free_host_data(d);
            return ast_set_error(AST_E_IO, "%s:%lld: expected 'filter MJD V sgm aux'", lc_path, (long long)(i + 1));
        }
        d->mjd_obs[i] = mjd1;
        if (i > 0 && d->mjd_obs[i] <= d->mjd_obs[i - 1]) {
            fclose(fp); ast_free_host_data(d);
            return ast_set_error(AST_E_IO, "Error: the data have to be sorted chronologically!");
        }
        d->v[i] = (float)v1;
        d->w[i] = (float)(1.0 / (sgm * sgm));
        int32_t k, found = -1;
        for (k = 0; k < nf; k++)
            if (d->filters[k] == filt) { found = k; break; }
        if (found < 0) {
            if (nf >= max_filters) {
                fclose(fp); ast_free_host_data(d);
                return ast_set_error(AST_E_TOO_LARGE, "Too many filters - increase N_FILTERS parameter! %d", nf + 1);
            }
            d->filters[nf] = filt;
            if (filt == 'W') w_filter = nf;
            if (filt == 'D') d_filter = nf;
            found = nf++;
        }
        d->filter[i] = found;
        i++;
    }
    fclose(fp);

    /* Ephemerides (read_data.c:127-235). */
    char pa[1024], pe[1024], ps[1024];
    FILE* fa = open_in(eph_dir, "asteroid.eph", pa, sizeof(pa));
    FILE* fe = open_in(eph_dir, "earth.eph", pe, sizeof(pe));
    FILE* fs = open_in(eph_dir, "sun.eph", ps, sizeof(ps));
    if (!fa || !fe || !fs) {
        if (fa) fclose(fa);
        if (fe) fclose(fe);
        if (fs) fclose(fs);
        ast_free_host_data(d);
        return ast_set_error(AST_E_IO, "ephemeris files asteroid.eph/earth.eph/sun.eph missing in %s",
                             eph_dir ? eph_dir : ".");
    }
    if (!seek_soe(fa) || !seek_soe(fe) || !seek_soe(fs)) {
        fclose(fa); fclose(fe); fclose(fs); ast_free_host_data(d);
        return ast_set_error(AST_E_IO, "ephemeris file without $$SOE marker");
    }
    double e0[3][3] = {{0}}, s0[3][3] = {{0}}, mjd0[3] = {0};
    char la[AST_LINE], le[AST_LINE], ls[AST_LINE];
    int64_t j = -1, iobs = 0;
    int l = 0;
    double jd = 0;
    while (fgets(la, sizeof(la), fa)) {
        if (strncmp(la, "$$EOE", 5) == 0) break;
        j++;
        if (!fgets(le, sizeof(le), fe) || !fgets(ls, sizeof(ls), fs)) break;
        if (j % 2 == 0) {
            sscanf(la, "%lf", &jd);
        } else {
            if (l > 2) {
                for (int m = 0; m < 2; m++) {
                    for (int k = 0; k < 3; k++) { e0[k][m] = e0[k][m + 1]; s0[k][m] = s0[k][m + 1]; }
                    mjd0[m] = mjd0[m + 1];
                }
                l = 2;
            }
            double xa, ya, za, xe, ye, ze, xs, ys, zs;
            if (sscanf(la, "%lE %lE %lE", &xa, &ya, &za) != 3 || sscanf(le, "%lE %lE %lE", &xe, &ye, &ze) != 3 ||
                sscanf(ls, "%lE %lE %lE", &xs, &ys, &zs) != 3) {
                fclose(fa); fclose(fe); fclose(fs); ast_free_host_data(d);
                return ast_set_error(AST_E_IO, "ephemeris: malformed X Y Z line");
            }
            e0[0][l] = xe - xa; e0[1][l] = ye - ya; e0[2][l] = ze - za;
            s0[0][l] = xs - xa; s0[1][l] = ys - ya; s0[2][l] = zs - za;
            mjd0[l] = jd - 2400000.5;
            l++;
            if (l > 2) {
                while (iobs < n && d->mjd_obs[iobs] >= mjd0[0] && d->mjd_obs[iobs] < mjd0[2]) {
                    ast_quadratic_interpolation(mjd0, (const double(*)[3])e0, (const double(*)[3])s0,
                                                d->mjd_obs[iobs], &d->e_unit[3 * iobs], &d->s_unit[3 * iobs]);
                    iobs++;
                }
            }
        }
        if (iobs >= n) break;
    }
    fclose(fa); fclose(fe); fclose(fs);
    if (iobs < n) {
        ast_free_host_data(d);
        return ast_set_error(AST_E_IO, "ephemerides do not bracket observation %lld (MJD %.6f)",
                             (long long)iobs, iobs < n ? d->mjd_obs[iobs] : 0.0);
    }

    /* Conversion (read_data.c:243-285). */
    for (i = 0; i < n; i++) {
        double* ev = &d->e_unit[3 * i];
        double* sv = &d->s_unit[3 * i];
        double E = sqrt(ev[0] * ev[0] + ev[1] * ev[1] + ev[2] * ev[2]);
        double S = sqrt(sv[0] * sv[0] + sv[1] * sv[1] + sv[2] * sv[2]);
        if (d->filter[i] != w_filter)
            d->v[i] = (float)(d->v[i] + 5.0 * log10(1.0 / E * 1.0 / S));
        double delay = E / AST_LIGHT_SPEED;
        d->mjd[i] = d->mjd_obs[i];
        if (d->filter[i] != w_filter && d->filter[i] != d_filter) d->mjd[i] = d->mjd[i] - delay;
        if (i == 0) d->hmjd0 = d->mjd[i];
        d->mjd[i] = d->mjd[i] - d->hmjd0;
        for (int k = 0; k < 3; k++) { ev[k] = ev[k] / E; sv[k] = sv[k] / S; }
    }
    for (int k = 0; k < 3; k++) {
        for (int m = 0; m < 3; m++) { d->obs.eph_e[k][m] = e0[k][m]; d->obs.eph_s[k][m] = s0[k][m]; }
        d->obs.eph_mjd0[k] = interp ? mjd0[k] - d->hmjd0 : mjd0[k];
    }
    d->obs.n_data = (int32_t)n;
    d->obs.n_filters = nf;
    d->obs.mjd = d->mjd; d->obs.v = d->v; d->obs.w = d->w; d->obs.filter = d->filter;
    d->obs.e_unit = d->e_unit; d->obs.s_unit = d->s_unit;
    d->obs.n_minima = 0;
    *out = d;
    return AST_OK;
}
