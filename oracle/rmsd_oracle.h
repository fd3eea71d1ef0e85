/*
 * rmsd_oracle.h -- THE ORACLE for the RMSD confidence intervals.  TEST INFRASTRUCTURE ONLY.
 * Included by chi2_oracle.c after the Philox generator and the chi2one / x2params / params2x
 * restatements, once per CHI_FLOAT.
 *
 * A plain CPU restatement of chi2_gpu_rms (cuda.c:2148-2389) for one call: f0 = RMSD of the -m
 * model and f1 = f0 + f0/sqrt(N_data - N - Nf) (cuda.c:2224-2227); per stream, `samples` draws
 * x = x0 + dx * N(0,1) with the SMALL clamps inside hard limits and psi_0's periodicity set by
 * the drawn Es (cuda.c:2260-2290); a draw x2params rejects is skipped (cuda.c:2292-2295); the
 * others are evaluated (Ntot), and a model with RMSD < f1 widens every parameter's range after
 * the phi_M / phi_0 replacement and the optional spherical torque (cuda.c:2300-2345), else it
 * counts in Nbad.  The normals are the engine's: Philox4x32-10 keyed by (seed, stream, call,
 * draw) and Box-Muller in float, with the C library's logf / sinf / cosf (the device uses its
 * own, so drawn points agree to a few float ulps).  x_in, when given, replaces the draws
 * ([n_streams*samples][N], NaN rows skipped as rejected), so a test can evaluate exactly the
 * points the device drew; f_in, when given, replaces the RMSDs as well, so the bookkeeping can be
 * checked on the device's own figures.
 */
/* Four Box-Muller normals of Philox block ctr of stream (seed, domain, stream). */
void orc_normal4(uint64_t seed, uint64_t stream, uint32_t domain, uint32_t ctr, float z[4])
{
    uint32_t c[4] = {ctr, domain, (uint32_t)stream, (uint32_t)(stream >> 32)};
    uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
    uint32_t u[4];
    orc_philox4x32_10(c, key, u);
    for (int p = 0; p < 2; p++) {
        const float u1 = ((float)(u[2 * p] >> 8) + 0.5f) * (1.0f / 16777216.0f);
        const float u2 = ((float)(u[2 * p + 1] >> 8) + 0.5f) * (1.0f / 16777216.0f);
        const float r = sqrtf(-2.0f * logf(u1));
        z[2 * p] = r * cosf(6.2831853071795865f * u2);
        z[2 * p + 1] = r * sinf(6.2831853071795865f * u2);
    }
}

#define RM_FN(name) NM_CAT(name, RM_SFX)

#define RM_CF double
#define RM_SFX acc
#include "rmsd_oracle_body.h"
#undef RM_CF
#undef RM_SFX

#define RM_CF float
#define RM_SFX sp
#include "rmsd_oracle_body.h"
#undef RM_CF
#undef RM_SFX

/* Returns 0; ranges as double (the device reports them rounded to float). */
int orc_rmsd(const ast_model* md, const ast_obs_set* o, const double* params0, uint64_t seed, uint32_t call,
             int64_t n_streams, int32_t samples, float dx, int reopt, int spherical, const double* x_in,
             const double* f_in, double* f01, int64_t* counts, double* pmin, double* pmax, double* trace_x,
             double* trace_f)
{
    if (md->flags & AST_ACC)
        return orc_rmsd_acc(md, o, params0, seed, call, n_streams, samples, dx, reopt, spherical, x_in, f_in, f01,
                            counts, pmin, pmax, trace_x, trace_f);
    return orc_rmsd_sp(md, o, params0, seed, call, n_streams, samples, dx, reopt, spherical, x_in, f_in, f01, counts,
                       pmin, pmax, trace_x, trace_f);
}
