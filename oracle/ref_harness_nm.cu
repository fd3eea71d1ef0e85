/*
 * ref_harness_nm.cu -- TEST INFRASTRUCTURE ONLY.  Appended by oracle/build_ref.sh (after
 * ref_harness_kernel.cu) to the reference's asteroid.h + cuda.c for the simplex builds
 * ref_nm_<variant>.cubin.  oracle/ref_gpu_loader.cpp (refn_fit) calls:
 *   refn_setup   one thread: the __device__ tables and parameters the reference's host uploads
 *                with cudaMemcpyToSymbol before a fit (asteroid.c:603-606,637; misc.c:296;
 *                gpu_prepare.c:38-46), from plain arrays, plus the instrumentation pointers
 *   refn_sizes   sizeof(curandState) and sizeof(struct obs_data) of this build
 * and then the reference's own setup_kernel and chi2_gpu, unmodified but for the hooks of
 * ref_harness_nm_pre.cuh.
 */
extern "C" __global__ void refn_sizes(int* out)
{
    out[0] = (int)sizeof(curandState);
    out[1] = (int)sizeof(struct obs_data);
    out[2] = (int)sizeof(CHI_FLOAT);
    out[3] = N_PARAMS;
    out[4] = N_TYPES;
}

extern "C" __global__ void refn_setup(const int* property /* [N_PARAMS][N_COLUMNS] */, const int* types,
                                      const double* limits /* [2][max_types] */, int max_types, float ppsi1,
                                      float ppsi2, const double* params0, const double* eph /* E[3][3],S[3][3],MJD0[3] */,
                                      int n_min, const float* t_min, const float* v_min, unsigned int n_steps,
                                      double* chain_f, int* chain_l, unsigned int* evals, int threads)
{
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    for (int i = 0; i < N_PARAMS; i++)
        for (int j = 0; j < N_COLUMNS; j++) dProperty[i][j] = property[i * N_COLUMNS + j];
    for (int t = 0; t < N_TYPES; t++) {
        dTypes[t][0] = types[t];
        dLimits[0][t] = (CHI_FLOAT)limits[t];
        dLimits[1][t] = (CHI_FLOAT)limits[max_types + t];
    }
    d_x2_params.reopt = 0;
#ifdef P_PSI
    d_x2_params.Ppsi1 = ppsi1;
    d_x2_params.Ppsi2 = ppsi2;
#endif
    for (int i = 0; i < N_PARAMS; i++) d_params0[i] = params0 ? params0[i] : 0.0;
#ifdef INTERP
    for (int k = 0; k < 3; k++) {
        dE_x0[k] = eph[0 + k]; dE_y0[k] = eph[3 + k]; dE_z0[k] = eph[6 + k];
        dS_x0[k] = eph[9 + k]; dS_y0[k] = eph[12 + k]; dS_z0[k] = eph[15 + k];
        dMJD0[k] = eph[18 + k];
    }
#endif
#ifdef NUDGE
    d_chi2_params.N_obs = n_min;
    for (int k = 0; k < n_min; k++) {
        d_chi2_params.t_obs[k] = t_min[k];
        d_chi2_params.V_obs[k] = v_min[k];
    }
#endif
    refk_n_steps = n_steps;
    refk_chain_f = chain_f;
    refk_chain_l = chain_l;
    refk_evals = evals;
    refk_threads = threads;
}
