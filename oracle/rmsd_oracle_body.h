/*
 * rmsd_oracle_body.h -- TEST INFRASTRUCTURE ONLY (the oracle).  chi2_gpu_rms for CHI_FLOAT =
 * RM_CF (cuda.c:2148-2389).  Included by rmsd_oracle.h.
 */
static int RM_FN(orc_rmsd)(const ast_model* md, const ast_obs_set* o, const double* params0, uint64_t seed,
                           uint32_t call, int64_t n_streams, int32_t samples, float dx, int reopt, int spherical,
                           const double* x_in, const double* f_in, double* f01, int64_t* counts, double* pmin,
                           double* pmax, double* trace_x, double* trace_f)
{
    const double PI_ = 3.141592653589793238;
    const ast_type_ids* T = &md->ids;
    const int N = md->n_params;
    const int nq = (N + 3) / 4;
    RM_CF x0[AST_MAX_PARAMS], dv[AST_MAX_FILTERS];
    double p0[AST_MAX_PARAMS];
    for (int i = 0; i < N; i++) p0[i] = params0[i];
    RM_FN(orc_params2x)(md, p0, x0);
    const RM_CF f0 = RM_FN(orc_chi2one)(md, o, p0, dv, NULL);
    const RM_CF f1 = f0 + f0 / sqrt((RM_CF)(o->n_data - N - o->n_filters));
    f01[0] = f0;
    f01[1] = f1;
    spherical = spherical && (md->flags & AST_TORQUE);
    const int iM = md->types[T->phi_M], i0 = md->types[T->phi_0];
    const double phi_M0 = p0[iM], phi_00 = p0[i0];
    int iTi = -1, iTs = -1, iTl = -1, ib = md->types[T->b_tumb], ic = md->types[T->c_tumb];
    double phiK0 = 0;
    if (spherical) {
        iTi = md->types[T->Ti]; iTs = md->types[T->Ts]; iTl = md->types[T->Tl];
        const double b = p0[ib], c = p0[ic];
        const double Is = (1.0 + b * b) / (b * b + c * c), Ii = (1.0 + c * c) / (b * b + c * c);
        phiK0 = atan2(Is * p0[iTs], Ii * p0[iTi]);
    }
    for (int i = 0; i < N; i++) { pmin[i] = 1e30; pmax[i] = -1e30; }
    int64_t n_tot = 0, n_bad = 0;
    for (int64_t st = 0; st < n_streams; st++)
        for (int k = 0; k < samples; k++) {
            const int64_t row = st * samples + k;
            RM_CF x1[AST_MAX_PARAMS];
            if (x_in) {
                if (x_in[row * N] != x_in[row * N]) continue;
                for (int i = 0; i < N; i++) x1[i] = (RM_CF)x_in[row * N + i];
            } else {
                int LAM = 0;
                for (int q = 0; q < nq; q++) {
                    float z[4];
                    orc_normal4(seed, (uint64_t)st, 0x80000000u | call, (uint32_t)k * (uint32_t)nq + (uint32_t)q, z);
                    for (int r = 0; r < 4 && 4 * q + r < N; r++) {
                        const int i = 4 * q + r;
                        RM_CF xx = x0[i] + (RM_CF)(dx * z[r]);
                        const int per = md->property[i][AST_P_PERIODIC];
                        const int soft_lam = LAM == 0 && per == AST_PERIODIC_LAM;
                        if (xx < ORC_SMALL && (per == AST_HARD_BOTH || per == AST_HARD_LEFT || soft_lam))
                            xx = (RM_CF)ORC_SMALL;
                        else if (xx > 1.0 - ORC_SMALL && (per == AST_HARD_BOTH || per == AST_HARD_RIGHT || soft_lam))
                            xx = (RM_CF)(1.0 - ORC_SMALL);
                        x1[i] = xx;
                        if (md->property[i][AST_P_TYPE] == T->Es) LAM = x1[i] >= 0.5;
                    }
                }
            }
            if (trace_x)
                for (int i = 0; i < N; i++) trace_x[row * N + i] = x1[i];
            double p[AST_MAX_PARAMS];
            if (RM_FN(orc_x2params)(md, reopt, x1, p)) {
                if (trace_f) trace_f[row] = NAN;
                continue;
            }
            const RM_CF f = f_in ? (RM_CF)f_in[row] : RM_FN(orc_chi2one)(md, o, p, dv, NULL);
            if (trace_f) trace_f[row] = f;
            n_tot++;
            if (!(f < f1)) {
                n_bad++;
                continue;
            }
            if (p[iM] > phi_M0 + PI_) p[iM] = phi_M0 - 2 * PI_;
            if (p[iM] < phi_M0 - PI_) p[iM] = phi_M0 + 2 * PI_;
            if (p[i0] > phi_00 + PI_) p[i0] = phi_00 - 2 * PI_;
            if (p[i0] < phi_00 - PI_) p[i0] = phi_00 + 2 * PI_;
            if (spherical) {
                const double b = p[ib], c = p[ic];
                const double Is = (1.0 + b * b) / (b * b + c * c), Ii = (1.0 + c * c) / (b * b + c * c);
                const double Ki = Ii * p[iTi], Ks = Is * p[iTs], Kl = p[iTl];
                p[iTi] = sqrt(Ki * Ki + Ks * Ks + Kl * Kl);
                p[iTs] = acos(Kl / p[iTi]);
                double phi = atan2(Ks, Ki);
                if (phi > phiK0 + PI_) phi = phi - 2 * PI_;
                if (phi < phiK0 - PI_) phi = phi + 2 * PI_;
                p[iTl] = phi;
            }
            for (int i = 0; i < N; i++) {
                if (p[i] < pmin[i]) pmin[i] = p[i];
                if (p[i] > pmax[i]) pmax[i] = p[i];
            }
        }
    counts[0] = n_tot;
    counts[1] = n_bad;
    return 0;
}
