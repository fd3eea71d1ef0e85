/*
 * tables.c -- model-variant tables of the fitting engine (host, C).
 *
 * Builds, for one combination of the variant flags, the three tables the reference keeps in
 * __device__ symbols: the Property table (asteroid.c:86-125), the Types map
 * (asteroid.c:152-169) and the hLimits table (asteroid.c:473-564), plus the P_PSI period
 * range of x2_struct (asteroid.c:598-601).  The parameter order and the type numbering have to
 * be the reference's: they fix the order of the parameters on the output line and the integer
 * ids the -f and -l switches take.
 */
#include <math.h>
#include <string.h>
#include "asteroid_gb300.h"
#include "host_internal.h"

#define AST_PI 3.141592653589793238
#define AST_RAD (180.0 / AST_PI)

/* hLimits is CHI_FLOAT in the reference (asteroid.c:474): float unless ACC. */
static double chi_float(const ast_model* m, double v)
{
    return (m->flags & AST_ACC) ? v : (double)(float)v;
}

/* Type ids in the reference's __COUNTER__ order (asteroid.h:137-178); ROTATE, TREND and
 * TORQUE2 are not among the supported variants. */
static void make_type_ids(int32_t flags, ast_type_ids* t)
{
    int32_t k = 0;
    t->theta_M = k++;
    t->phi_M = k++;
    t->phi_0 = k++;
    t->L = k++;
    t->Ti = t->Ts = t->Tl = -1;
    if (flags & AST_TORQUE) { t->Ti = k++; t->Ts = k++; t->Tl = k++; }
    t->c_tumb = k++;
    t->b_tumb = k++;
    t->Es = k++;
    t->psi_0 = k++;
    t->c = t->b = -1;
    if (flags & AST_BC) { t->c = k++; t->b = k++; }
    t->theta_R = t->phi_R = t->kappa = -1;
    if (flags & AST_BW_BALL) { t->theta_R = k++; t->phi_R = k++; t->kappa = k++; }
    t->n_types = k;
}

static void add_row(ast_model* m, int32_t type, int32_t independent, int32_t multi, int32_t periodic)
{
    int32_t i = m->n_params++;
    m->property[i][AST_P_TYPE] = type;
    m->property[i][AST_P_INDEPENDENT] = independent;
    m->property[i][AST_P_FROZEN] = 0;
    m->property[i][AST_P_ISEG] = 0;
    m->property[i][AST_P_MULTI_SEGMENT] = multi;
    m->property[i][AST_P_PERIODIC] = periodic;
}

int ast_model_init(ast_model* m, int32_t flags, double time_step,
                   double ppsi_min_hours, double ppsi_max_hours)
{
    if (!m) return ast_set_error(AST_E_INVALID, "ast_model_init: NULL model");
    if (flags & ~(AST_TORQUE | AST_BC | AST_BW_BALL | AST_P_PSI | AST_INTERP | AST_ACC | AST_NUDGE | AST_RMSD))
        return ast_set_error(AST_E_INVALID, "ast_model_init: unknown flag bits 0x%x", flags);
    if (!(time_step > 0.0))
        return ast_set_error(AST_E_INVALID, "ast_model_init: time_step must be > 0");
    if ((flags & AST_P_PSI) && !(ppsi_min_hours > 0.0 && ppsi_max_hours > 0.0))
        return ast_set_error(AST_E_INVALID, "ast_model_init: P_PSI needs -Ppsi min max > 0");
    memset(m, 0, sizeof(*m));
    m->flags = flags;
    m->time_step = time_step;
    make_type_ids(flags, &m->ids);
    const ast_type_ids* t = &m->ids;
    m->n_types = t->n_types;

    /* Property rows in output order (asteroid.c:86-125). */
    add_row(m, t->theta_M, 1, 0, AST_HARD_BOTH);
    add_row(m, t->phi_M, 1, 0, AST_PERIODIC);
    add_row(m, t->phi_0, 1, 0, AST_PERIODIC);
    if (flags & AST_TORQUE) {
        add_row(m, t->Ti, 1, 0, AST_SOFT_BOTH);
        add_row(m, t->Ts, 1, 0, AST_SOFT_BOTH);
        add_row(m, t->Tl, 1, 0, AST_SOFT_BOTH);
    }
    add_row(m, t->c_tumb, 1, 1, AST_HARD_RIGHT);
    add_row(m, t->b_tumb, 0, 1, AST_HARD_BOTH);
    add_row(m, t->Es, 0, 0, AST_HARD_BOTH);
    add_row(m, t->L, 1, 0, AST_HARD_LEFT);
    add_row(m, t->psi_0, 0, 0, AST_PERIODIC_LAM);
    if (flags & AST_BC) {
        add_row(m, t->c, 1, 1, AST_HARD_RIGHT);
        add_row(m, t->b, 0, 1, AST_HARD_BOTH);
    }
    if (flags & AST_BW_BALL) {
        add_row(m, t->theta_R, 1, 1, AST_HARD_BOTH);
        add_row(m, t->phi_R, 1, 1, AST_PERIODIC);
        add_row(m, t->kappa, 1, 1, AST_SOFT_BOTH);
    }

    /* Types map (asteroid.c:152-169): one segment, so every type maps to its row. */
    for (int j = 0; j < AST_MAX_TYPES; j++) m->types[j] = -1;
    for (int i = 0; i < m->n_params; i++) m->types[m->property[i][AST_P_TYPE]] = i;

    /* hLimits (asteroid.c:473-564); Es and psi_0 have none (their x maps are special). */
    m->limits[0][t->theta_M] = chi_float(m, 0.001 / AST_RAD);
    m->limits[1][t->theta_M] = chi_float(m, 179.999 / AST_RAD);
    m->limits[0][t->L] = chi_float(m, 48.0 * AST_PI / 10);
    m->limits[1][t->L] = chi_float(m, 48.0 * AST_PI / 0.1);
    if (flags & AST_TORQUE) {
        const double tmax = 10.0;
        m->limits[0][t->Ti] = chi_float(m, -tmax); m->limits[1][t->Ti] = chi_float(m, tmax);
        m->limits[0][t->Ts] = chi_float(m, -tmax); m->limits[1][t->Ts] = chi_float(m, tmax);
        m->limits[0][t->Tl] = chi_float(m, -tmax); m->limits[1][t->Tl] = chi_float(m, tmax);
    }
    m->limits[0][t->c_tumb] = chi_float(m, log(0.01));
    m->limits[1][t->c_tumb] = chi_float(m, log(1.0));
    m->limits[0][t->b_tumb] = 0;
    m->limits[1][t->b_tumb] = 1;
    if (flags & AST_BC) {
        m->limits[0][t->c] = m->limits[0][t->c_tumb];
        m->limits[1][t->c] = m->limits[1][t->c_tumb];
        m->limits[0][t->b] = 0;
        m->limits[1][t->b] = 1;
    }
    if (flags & AST_BW_BALL) {
        m->limits[0][t->theta_R] = chi_float(m, 0.001 / AST_RAD);
        m->limits[1][t->theta_R] = chi_float(m, 179.999 / AST_RAD);
        m->limits[0][t->kappa] = chi_float(m, log(0.01));
        m->limits[1][t->kappa] = chi_float(m, log(0.1));
    }
    /* x2_struct.Ppsi1/2 are floats holding 1/Ppsi in 1/day (asteroid.c:598-601). */
    if (flags & AST_P_PSI) {
        m->ppsi1 = (float)(24.0 / ppsi_max_hours);
        m->ppsi2 = (float)(24.0 / ppsi_min_hours);
    }
    return AST_OK;
}

int ast_model_freeze(ast_model* m, int32_t type, double value)
{
    if (!m || type < 0 || type >= m->n_types)
        return ast_set_error(AST_E_INVALID, "ast_model_freeze: bad type id %d", type);
    for (int i = 0; i < m->n_params; i++)
        if (m->property[i][AST_P_TYPE] == type) {
            m->property[i][AST_P_FROZEN] = 1;
            m->limits[0][type] = chi_float(m, value);
            m->limits[1][type] = chi_float(m, value);
        }
    return AST_OK;
}

int ast_model_set_limits(ast_model* m, int32_t type, double l0, double l1)
{
    if (!m || type < 0 || type >= m->n_types)
        return ast_set_error(AST_E_INVALID, "ast_model_set_limits: bad type id %d", type);
    m->limits[0][type] = chi_float(m, l0);
    m->limits[1][type] = chi_float(m, l1);
    return AST_OK;
}

int ast_model_set_free_random(ast_model* m, int32_t param_index)
{
    if (!m || param_index < 0 || param_index >= m->n_params)
        return ast_set_error(AST_E_INVALID, "ast_model_set_free_random: bad index %d", param_index);
    m->property[param_index][AST_P_FROZEN] = -1;
    return AST_OK;
}

const char* ast_param_name(const ast_model* m, int32_t i)
{
    if (!m || i < 0 || i >= m->n_params) return "?";
    int32_t type = m->property[i][AST_P_TYPE];
    const ast_type_ids* t = &m->ids;
    if (type == t->theta_M) return "theta_M";
    if (type == t->phi_M) return "phi_M";
    if (type == t->phi_0) return "phi_0";
    if (type == t->L) return "L";
    if (type == t->Ti) return "Ti";
    if (type == t->Ts) return "Ts";
    if (type == t->Tl) return "Tl";
    if (type == t->c_tumb) return "c_tumb";
    if (type == t->b_tumb) return "b_tumb";
    if (type == t->Es) return "Es";
    if (type == t->psi_0) return "psi_0";
    if (type == t->c) return "c";
    if (type == t->b) return "b";
    if (type == t->theta_R) return "theta_R";
    if (type == t->phi_R) return "phi_R";
    if (type == t->kappa) return "kappa";
    return "?";
}
