/*
 * nm_oracle_body.h -- TEST INFRASTRUCTURE ONLY (the oracle).  One downhill-simplex chain
 * (cuda.c:1424-1742) for CHI_FLOAT = NM_CF.  Included by nm_oracle_impl.h.
 */
#define NM_FN(name) NM_CAT(name, NM_SFX)

/* chi^2 of a dimensionless point: 1 if x2params rejects it, else 0 with *f set.  dv_last is
 * updated only when chi2one runs to completion (the NUDGE 1e30 exit leaves it). */
static int NM_FN(nm_eval)(const ast_model* md, const ast_obs_set* o, int reopt, const NM_CF* x, NM_CF* f,
                          double* dv_last, int64_t* evals)
{
    double params[AST_MAX_PARAMS];
    if (NM_FN(orc_x2params)(md, reopt, x, params)) return 1;
    NM_CF dv[AST_MAX_FILTERS];
    for (int m = 0; m < o->n_filters; m++) dv[m] = (NM_CF)dv_last[m];
    *f = NM_FN(orc_chi2one)(md, o, params, dv, NULL);
    for (int m = 0; m < o->n_filters; m++) dv_last[m] = dv[m];
    (*evals)++;
    return 0;
}

static int NM_FN(nm_hard)(int per, int LAM, int left)
{
    if (per == AST_HARD_BOTH) return 1;
    if (left && per == AST_HARD_LEFT) return 1;
    if (!left && per == AST_HARD_RIGHT) return 1;
    return LAM == 0 && per == AST_PERIODIC_LAM;
}

static void NM_FN(orc_nm_chain)(const ast_model* md, const ast_obs_set* o, int reopt, const double* x_start,
                                uint64_t seed, uint64_t chain, uint32_t stage, int64_t evals_cap, int32_t steps_cap,
                                orc_chain_out* out)
{
    const ast_type_ids* T = &md->ids;
    const int N = md->n_params;
    const NM_CF DX_INI = (NM_CF)0.001, D2X_INI = (NM_CF)-1.2, DX_RAND = (NM_CF)0.0001;
    const NM_CF SIZE2_MIN = (md->flags & AST_ACC) ? (NM_CF)(1e-10 * 1e-10) : (NM_CF)((float)1e-5 * (float)1e-5);
    const NM_CF ALPHA = 1.0, GAMMA = 2.0, RHO = 0.5, SIGMA = 0.5;
    if (steps_cap <= 0) steps_cap = 5000;
    NM_CF x[AST_MAX_PARAMS + 1][AST_MAX_PARAMS], f[AST_MAX_PARAMS + 1];
    int ind[AST_MAX_PARAMS + 1];
    uint32_t k = 0;
    int64_t evals = 0;
    out->evals = 0;
    out->iters = 0;
    out->failed = 0;
    for (int j = 0; j <= N; j++) ind[j] = j;
    if (x_start)
        for (int i = 0; i < N; i++) x[0][i] = (NM_CF)x_start[i];
    else
        for (int i = 0; i < N; i++) x[0][i] = 0;

    /* Random start (cuda.c:1459-1508). */
    int LAM = 0;
    for (int i = 0; i < N; i++) {
        float r = orc_uniform(seed, chain, stage, k++);
        int pt = md->property[i][AST_P_TYPE];
        int per = md->property[i][AST_P_PERIODIC];
        if ((md->flags & AST_BC) && !reopt) {
            if (pt == T->c) { x[0][i] = x[0][md->types[T->c_tumb]]; continue; }
            if (pt == T->b) { x[0][i] = x[0][md->types[T->b_tumb]]; continue; }
        }
        if (!reopt || md->property[i][AST_P_FROZEN] == -1) {
            x[0][i] = (NM_CF)(DX_INI + ORC_SMALL + r * (1.0 - 2 * (ORC_SMALL + DX_INI)));
        } else {
            NM_CF xmin = x[0][i] - DX_RAND;
            NM_CF xmax = x[0][i] + DX_RAND;
            if (xmin < ORC_SMALL && NM_FN(nm_hard)(per, LAM, 1)) xmin = (NM_CF)ORC_SMALL;
            if (xmax > 1.0 - ORC_SMALL && NM_FN(nm_hard)(per, LAM, 0)) xmax = (NM_CF)(1.0 - ORC_SMALL);
            x[0][i] = xmin + r * (xmax - xmin);
        }
        if (pt == T->Es) LAM = x[0][i] >= 0.5;
    }

    /* Initial simplex (cuda.c:1512-1545). */
    for (int j = 1; j <= N; j++) {
        for (int i = 0; i < N; i++) {
            if (i == j - 1) {
                int per = md->property[i][AST_P_PERIODIC];
                float d2x = orc_uniform(seed, chain, stage, k++);
                NM_CF dx = DX_INI * NM_EXP(D2X_INI * d2x);
                if (orc_uniform(seed, chain, stage, k++) < 0.5) {
                    dx = -dx;
                    if (x[0][i] + dx < ORC_SMALL && NM_FN(nm_hard)(per, LAM, 1)) dx = -dx;
                } else {
                    if (x[0][i] + dx > 1.0 - ORC_SMALL && NM_FN(nm_hard)(per, LAM, 0)) dx = -dx;
                }
                x[j][i] = x[0][i] + dx;
            } else {
                x[j][i] = x[0][i];
            }
        }
    }

    /* Initial values (cuda.c:1549-1559). */
    int failed = 0;
    for (int j = 0; j <= N; j++) {
        if (NM_FN(nm_eval)(md, o, reopt, x[j], &f[j], out->dv_last, &evals)) { failed = 1; break; }
    }

    int l = 0;
    while (!failed) {
        l++;
        /* Selection sort, ties -> last index (cuda.c:1575-1601). */
        int taken[AST_MAX_PARAMS + 1];
        for (int j = 0; j <= N; j++) taken[j] = 0;
        for (int j = 0; j <= N; j++) {
            NM_CF fmin = (NM_CF)1e30;
            int jmin = -1;
            for (int j2 = 0; j2 <= N; j2++)
                if (!taken[j2] && f[j2] <= fmin) { fmin = f[j2]; jmin = j2; }
            if (jmin < 0) { ind[0] = 0; f[ind[0]] = (NM_CF)1e30; break; }
            ind[j] = jmin;
            taken[jmin] = 1;
        }
        /* Centroid over all N+1 vertices, worst included (cuda.c:1604-1611). */
        NM_CF x0[AST_MAX_PARAMS];
        for (int i = 0; i < N; i++) {
            NM_CF sum = 0.0;
            for (int j = 0; j <= N; j++) sum = sum + x[j][i];
            x0[i] = sum / (NM_CF)(N + 1);
        }
        NM_CF size2 = 0.0;
        for (int j = 0; j <= N; j++) {
            NM_CF sum = 0.0;
            for (int i = 0; i < N; i++) {
                NM_CF dx = x[j][i] - x0[i];
                sum = sum + dx * dx;
            }
            size2 = size2 + sum;
        }
        size2 = size2 / (NM_CF)N;
        if (size2 < SIZE2_MIN) break;
        if (l > steps_cap) break;
        if (evals_cap > 0 && evals >= evals_cap) break;

        const int w = ind[N];
        NM_CF x_r[AST_MAX_PARAMS], f_r;
        for (int i = 0; i < N; i++)
            x_r[i] = (md->property[i][AST_P_FROZEN] != 1) ? x0[i] + ALPHA * (x0[i] - x[w][i]) : x0[i];
        if (NM_FN(nm_eval)(md, o, reopt, x_r, &f_r, out->dv_last, &evals)) f_r = (NM_CF)1e30;
        if (f_r >= f[ind[0]] && f_r < f[ind[N - 1]]) {
            for (int i = 0; i < N; i++) x[w][i] = x_r[i];
            f[w] = f_r;
            continue;
        }
        if (f_r < f[ind[0]]) {
            NM_CF x_e[AST_MAX_PARAMS], f_e;
            for (int i = 0; i < N; i++)
                x_e[i] = (md->property[i][AST_P_FROZEN] != 1) ? x0[i] + GAMMA * (x_r[i] - x0[i]) : x0[i];
            if (NM_FN(nm_eval)(md, o, reopt, x_e, &f_e, out->dv_last, &evals)) f_e = (NM_CF)1e30;
            if (f_e < f_r) {
                for (int i = 0; i < N; i++) x[w][i] = x_e[i];
                f[w] = f_e;
            } else {
                for (int i = 0; i < N; i++) x[w][i] = x_r[i];
                f[w] = f_r;
            }
            continue;
        }
        for (int i = 0; i < N; i++)
            x_r[i] = (md->property[i][AST_P_FROZEN] != 1) ? x0[i] + RHO * (x[w][i] - x0[i]) : x0[i];
        if (NM_FN(nm_eval)(md, o, reopt, x_r, &f_r, out->dv_last, &evals)) f_r = (NM_CF)1e30;
        if (f_r < f[w]) {
            for (int i = 0; i < N; i++) x[w][i] = x_r[i];
            f[w] = f_r;
            continue;
        }
        int bad = 0;
        for (int j = 1; j <= N; j++) {
            const int v = ind[j], b = ind[0];
            for (int i = 0; i < N; i++)
                if (md->property[i][AST_P_FROZEN] != 1) x[v][i] = x[b][i] + SIGMA * (x[v][i] - x[b][i]);
            if (NM_FN(nm_eval)(md, o, reopt, x[v], &f[v], out->dv_last, &evals)) bad = 1;
        }
        if (bad) { failed = 1; break; }
    }

    out->failed = failed;
    out->f = failed ? 1e30 : (double)f[ind[0]];
    for (int i = 0; i < N; i++) out->x_best[i] = failed ? (double)x[0][i] : (double)x[ind[0]][i];
    out->evals = evals;
    out->iters = l;
}

#undef NM_FN
