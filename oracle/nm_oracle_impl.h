/*
 * nm_oracle_impl.h -- TEST INFRASTRUCTURE ONLY (the oracle).  Downhill-simplex chains with
 * the semantics of the reference's chi2_gpu (cuda.c:1424-1823), one chain at a time, for
 * small cases.  Included once for each CHI_FLOAT (double "_acc", float "_sp").
 *
 * Deliberate, documented differences from the reference (all on draws or on reads the
 * reference leaves undefined):
 *   - random numbers come from Philox4x32-10 keyed by (seed, chain, stage), not cuRAND XORWOW;
 *   - trial coordinates of frozen parameters are set to the centroid (the reference leaves
 *     them uninitialised, cuda.c:1638,1663,1696);
 *   - the sort permutation starts as the identity (the reference reads it uninitialised when
 *     every f is NaN, cuda.c:1592-1598);
 *   - evals_cap adds an evaluation budget next to the N_STEPS iteration cap (cuda.c:1630).
 */

typedef struct orc_chain_out {
    double f;                       /* best chi^2, 1e30 if the chain failed */
    double x_best[AST_MAX_PARAMS];  /* best vertex (dimensionless) */
    double dv_last[AST_MAX_FILTERS];/* delta_V of the chain's last completed chi2one */
    int64_t evals;                  /* chi2one calls */
    int32_t iters;                  /* simplex iterations (l) */
    int32_t failed;
} orc_chain_out;

#define ORC_SMALL 1e-8

#define NM_CAT2(a, b) a##_##b
#define NM_CAT(a, b) NM_CAT2(a, b)

#define NM_CF double
#define NM_SFX acc
#define NM_EXP exp
#include "nm_oracle_body.h"
#undef NM_CF
#undef NM_SFX
#undef NM_EXP

#define NM_CF float
#define NM_SFX sp
#define NM_EXP expf
#include "nm_oracle_body.h"
#undef NM_CF
#undef NM_SFX
#undef NM_EXP

/* One chain (stage `stage`) with the chi^2 objective.  x_start: the stage start point
 * (params2x of the -m model, or the group best of the previous stage), NULL when reopt == 0. */
void orc_nm_chain(const ast_model* md, const ast_obs_set* o, int reopt, const double* x_start,
                  uint64_t seed, uint64_t chain, uint32_t stage, int64_t evals_cap, int32_t steps_cap,
                  orc_chain_out* out)
{
    if (md->flags & AST_ACC)
        orc_nm_chain_acc(md, o, reopt, x_start, seed, chain, stage, evals_cap, steps_cap, out);
    else
        orc_nm_chain_sp(md, o, reopt, x_start, seed, chain, stage, evals_cap, steps_cap, out);
}

/* Group/stage driver (cuda.c:1424-1823): chains [0, n_chains) in groups of group_size; every
 * stage after the first restarts each group's chains from its previous-stage best with
 * reopt = 1.  Outputs per group: best f (lowest f, lowest chain on ties), its physical
 * parameters (x2params with the final reopt), and that chain's last delta_V. */
void orc_fit(const ast_model* md, const ast_obs_set* o, uint64_t seed, int64_t n_chains, int32_t group_size,
             int32_t n_stages, int32_t reopt0, const double* params0, int64_t evals_cap, int32_t steps_cap,
             double* best_f, double* best_params, double* best_dv, double* chain_f, int64_t* n_evals)
{
    const int N = md->n_params;
    const int64_t n_groups = n_chains / group_size;
    orc_chain_out* res = (orc_chain_out*)calloc((size_t)n_chains, sizeof(orc_chain_out));
    double* start = (double*)calloc((size_t)n_groups * N, sizeof(double));
    int* reopt_g = (int*)calloc((size_t)n_groups, sizeof(int));
    int64_t ev = 0;
    for (int64_t g = 0; g < n_groups; g++) {
        reopt_g[g] = reopt0;
        if (reopt0) orc_params2x(md, params0, start + g * N);
    }
    for (int32_t s = 0; s < n_stages; s++) {
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 1) reduction(+ : ev)
#endif
        for (int64_t c = 0; c < n_chains; c++) {
            int64_t g = c / group_size;
            /* res[c].dv_last carries over: it is overwritten only by completed chi2one calls. */
            orc_nm_chain(md, o, reopt_g[g], reopt_g[g] ? start + g * N : NULL, seed, (uint64_t)c, (uint32_t)s,
                         evals_cap, steps_cap, &res[c]);
            ev += res[c].evals;
        }
        for (int64_t g = 0; g < n_groups; g++) {
            int64_t cmin = g * group_size;
            double fmin = 1e30;
            for (int64_t c = g * group_size; c < (g + 1) * group_size; c++)
                if (res[c].f < fmin) { fmin = res[c].f; cmin = c; }
            if (s < n_stages - 1) {
                double* xs = start + g * N;
                for (int i = 0; i < N; i++) xs[i] = res[cmin].x_best[i];
                if ((md->flags & AST_P_PSI) && reopt_g[g] == 0) {
                    double p[AST_MAX_PARAMS];
                    orc_x2params(md, 0, xs, p);
                    orc_params2x(md, p, xs);
                }
                reopt_g[g] = 1;
            } else {
                if (best_f) best_f[g] = fmin;
                if (best_params) {
                    double p[AST_MAX_PARAMS] = {0};
                    if (fmin < 1e30) orc_x2params(md, reopt_g[g], res[cmin].x_best, p);
                    for (int i = 0; i < N; i++) best_params[g * N + i] = p[i];
                }
                if (best_dv)
                    for (int m = 0; m < o->n_filters; m++) best_dv[g * o->n_filters + m] = fmin < 1e30 ? res[cmin].dv_last[m] : 0.0;
            }
        }
    }
    if (chain_f)
        for (int64_t c = 0; c < n_chains; c++) chain_f[c] = res[c].f;
    if (n_evals) *n_evals = ev;
    free(res);
    free(start);
    free(reopt_g);
}
