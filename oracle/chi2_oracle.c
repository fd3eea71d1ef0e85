/*
 * chi2_oracle.c -- THE ORACLE.  TEST INFRASTRUCTURE ONLY.
 *
 * Only tests/, __graft_entry__.smoke() and bench.py's cpu_baseline leg / --impl reference arm
 * load this library, and only as the checker or as the timed CPU baseline.  The product
 * (asteroid_gb300, its CUDA kernels and its C-ABI) never links or calls it.
 *
 * Contents (all plain C, compiled with -ffp-contract=off so that no multiply-add is fused):
 *   - chi2_oracle_impl.h, twice: chi2one / x2params / params2x for CHI_FLOAT = double
 *     ("_acc", the -DACC build) and CHI_FLOAT = float ("_sp", the default build);
 *   - the two ODE right-hand sides of cuda.c:13-77;
 *   - Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11), the engine's counter-based RNG;
 *   - one downhill-simplex chain with the reference's semantics (cuda.c:1424-1742) and the
 *     group / stage driver around it (cuda.c:1424-1823), for small cases;
 *   - an OpenMP batch evaluator, the timed CPU baseline;
 *   - minima_oracle.h: the periodogram of model minima of -plot mode (misc.c:65-276);
 *   - rmsd_oracle.h: the RMSD confidence intervals of chi2_gpu_rms (cuda.c:2148-2389);
 *   - animate_oracle.h: the ANIMATE frames of compute_rgb (cuda.c:2394-2540), and
 *     orc_model_geometry, their per-snapshot inputs.
 * Parity status: pinned bit-for-bit against a host build of the reference's own chi2one,
 * x2params and params2x compiled from its sources (oracle/build_ref.sh, tests/golden/).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif
#include "asteroid_gb300.h"

#define ORC_PI 3.141592653589793238

/* NUDGE constants (asteroid.h:216-231), with the reference's float rounding. */
static const float ORC_M_MAX2 = 20;
static const float ORC_DT_MAX = 0.12f;
static const float ORC_DV_MAX = 24;
#define ORC_DT_MAX2 ((float)(1.5 * 0.12f))
static const float ORC_P_MIN = 0.01f;
static const float ORC_CHI2_0 = 10;
static const float ORC_CHI2_1 = 30;
#define ORC_L_RC2 (0.05f * 0.05f)
#define ORC_L_A ((float)(1.0 / (1.0 - ORC_L_RC2 / (1.0 + ORC_L_RC2))))
#define ORC_P_MIN2 ((float)(1 / 0.01f - 1))
static const float ORC_BC_DEV_MAX = 100;

/* ODE right-hand side with torque (cuda.c:44-58): y = (Omega_i, Omega_s, Omega_l, phi, theta, psi). */
static void orc_ode_torque(const double* y, double* f, const double* mu)
{
    f[0] = mu[0] * y[1] * y[2] + mu[3];
    f[1] = mu[1] * y[2] * y[0] + mu[4];
    f[2] = mu[2] * y[0] * y[1] + mu[5];
    f[3] = (y[0] * sin(y[5]) + y[1] * cos(y[5])) / sin(y[4]);
    f[4] = y[0] * cos(y[5]) - y[1] * sin(y[5]);
    f[5] = y[2] - f[3] * cos(y[4]);
}

/* Torque-free Euler angles (cuda.c:68-75): y = (phi, theta, psi), mu = (L, Ip, Im). */
static void orc_ode_free(const double* y, double* f, const double* mu)
{
    f[0] = mu[0] * (mu[1] - mu[2] * cos(2.0 * y[2]));
    f[1] = mu[0] * mu[2] * sin(y[1]) * sin(2.0 * y[2]);
    f[2] = cos(y[1]) * (mu[0] - f[0]);
}

/* When set, chi2one also writes compute_rgb's 20 inputs of every point here (orc_model_geometry;
 * not thread-safe, test use only). */
static double* orc_geo_out = NULL;

#define ORC_CF double
#define ORC_SUFFIX acc
#define ORC_FLOOR floor
#include "chi2_oracle_impl.h"
#undef ORC_CF
#undef ORC_SUFFIX
#undef ORC_FLOOR

#define ORC_CF float
#define ORC_SUFFIX sp
#define ORC_FLOOR floorf
#include "chi2_oracle_impl.h"
#undef ORC_CF
#undef ORC_SUFFIX
#undef ORC_FLOOR

/* ------------------------------------------------------------------ exported, double I/O */

/* One chi2one call; chi2 and delta_v returned as double whatever CHI_FLOAT is. */
double orc_chi2(const ast_model* md, const ast_obs_set* o, const double* params, double* delta_v)
{
    if (md->flags & AST_ACC) {
        double dv[AST_MAX_FILTERS] = {0};
        double r = orc_chi2one_acc(md, o, params, dv, NULL);
        if (delta_v) for (int m = 0; m < o->n_filters; m++) delta_v[m] = dv[m];
        return r;
    } else {
        float dv[AST_MAX_FILTERS] = {0};
        float r = orc_chi2one_sp(md, o, params, dv, NULL);
        if (delta_v) for (int m = 0; m < o->n_filters; m++) delta_v[m] = dv[m];
        return r;
    }
}

/* Model magnitude at every observation (the true-model hook of the test data generator). */
void orc_model_curve(const ast_model* md, const ast_obs_set* o, const double* params, double* vmod)
{
    ast_model m2 = *md;
    m2.flags &= ~AST_NUDGE;
    double dv[AST_MAX_FILTERS];
    orc_chi2one_acc(&m2, o, params, dv, vmod);
}

/* compute_rgb's inputs (b, c, E, E', S', body axes b, c, a) at every observation of o. */
void orc_model_geometry(const ast_model* md, const ast_obs_set* o, const double* params, double* geo)
{
    ast_model m2 = *md;
    m2.flags &= ~AST_NUDGE;
    double dv[AST_MAX_FILTERS];
    orc_geo_out = geo;
    orc_chi2one_acc(&m2, o, params, dv, NULL);
    orc_geo_out = NULL;
}

/* Batch of n evaluations over `threads` OpenMP threads (0 = all); the CPU baseline. */
void orc_chi2_batch(const ast_model* md, const ast_obs_set* o, const double* params, int64_t n,
                    double* chi2, double* delta_v, int threads)
{
#ifdef _OPENMP
    if (threads <= 0) threads = omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 4) num_threads(threads)
#endif
    for (int64_t k = 0; k < n; k++)
        chi2[k] = orc_chi2(md, o, params + k * md->n_params, delta_v ? delta_v + k * o->n_filters : NULL);
    (void)threads;
}

int orc_max_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* x2params with x given as double (rounded to CHI_FLOAT first). */
int orc_x2params(const ast_model* md, int reopt, const double* x, double* params)
{
    if (md->flags & AST_ACC) return orc_x2params_acc(md, reopt, x, params);
    float xf[AST_MAX_PARAMS];
    for (int i = 0; i < md->n_params; i++) xf[i] = (float)x[i];
    return orc_x2params_sp(md, reopt, xf, params);
}

void orc_params2x(const ast_model* md, const double* params, double* x)
{
    if (md->flags & AST_ACC) { orc_params2x_acc(md, params, x); return; }
    float xf[AST_MAX_PARAMS];
    orc_params2x_sp(md, params, xf);
    for (int i = 0; i < md->n_params; i++) x[i] = xf[i];
}

/* ------------------------------------------------------------------ Philox4x32-10 */

static inline void orc_mulhilo(uint32_t a, uint32_t b, uint32_t* hi, uint32_t* lo)
{
    uint64_t p = (uint64_t)a * (uint64_t)b;
    *hi = (uint32_t)(p >> 32);
    *lo = (uint32_t)p;
}

/* Philox4x32 with 10 rounds: multipliers 0xD2511F53, 0xCD9E8D57 and Weyl key increments
 * 0x9E3779B9, 0xBB67AE85, as published by Salmon et al. (2011). */
void orc_philox4x32_10(const uint32_t ctr_in[4], const uint32_t key_in[2], uint32_t out[4])
{
    uint32_t c0 = ctr_in[0], c1 = ctr_in[1], c2 = ctr_in[2], c3 = ctr_in[3];
    uint32_t k0 = key_in[0], k1 = key_in[1];
    for (int r = 0; r < 10; r++) {
        uint32_t hi0, lo0, hi1, lo1;
        orc_mulhilo(0xD2511F53u, c0, &hi0, &lo0);
        orc_mulhilo(0xCD9E8D57u, c2, &hi1, &lo1);
        uint32_t n0 = hi1 ^ c1 ^ k0, n1 = lo1, n2 = hi0 ^ c3 ^ k1, n3 = lo0;
        c0 = n0; c1 = n1; c2 = n2; c3 = n3;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

/* Draw k of (seed, chain, stage) as a float uniform in (0,1): ((u >> 8) + 0.5) * 2^-24. */
float orc_uniform(uint64_t seed, uint64_t chain, uint32_t stage, uint32_t k)
{
    uint32_t ctr[4] = {k >> 2, stage, (uint32_t)chain, (uint32_t)(chain >> 32)};
    uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
    uint32_t out[4];
    orc_philox4x32_10(ctr, key, out);
    return ((float)(out[k & 3] >> 8) + 0.5f) * (1.0f / 16777216.0f);
}

/* ------------------------------------------------------------------ simplex chains */

#include "nm_oracle_impl.h"

#include "minima_oracle.h"
#include "rmsd_oracle.h"
#include "animate_oracle.h"
