/*
 * ref_harness_kernel.cu -- TEST INFRASTRUCTURE ONLY.  Device entry points around the
 * reference's own chi2one (cuda.c:81), appended by oracle/build_ref.sh to the reference's
 * asteroid.h + cuda.c (streamed from the reference checkout, never written to disk) and compiled
 * to oracle/_ref/ref_<variant>.cubin for sm_100.  oracle/ref_gpu_loader.cpp loads the cubin on
 * the GPU and calls:
 *   refk_pack  SoA observations -> the reference's AoS struct obs_data (asteroid.h:355-368)
 *   refk_eval  one thread per parameter vector: chi2one(params, obs, N_data, N_filters, dV, 0,
 *              &sp, sTypes), with sp (struct chi2_struct) and sTypes built from plain arrays.
 */
extern "C" __global__ void refk_pack(const double* mjd, const float* v, const float* w, const int* filt,
                                     const double* e_unit, const double* s_unit, int n, struct obs_data* out)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    out[i].V = v[i];
    out[i].w = w[i];
    out[i].MJD = mjd[i];
    out[i].Filter = filt[i];
#ifndef INTERP
    out[i].E_x = e_unit[3 * i];
    out[i].E_y = e_unit[3 * i + 1];
    out[i].E_z = e_unit[3 * i + 2];
    out[i].S_x = s_unit[3 * i];
    out[i].S_y = s_unit[3 * i + 1];
    out[i].S_z = s_unit[3 * i + 2];
#endif
}

extern "C" __global__ void refk_eval(const double* params, int n, const int* types, struct obs_data* data,
                                     int n_data, int n_filters, const double* eph /* E[3][3], S[3][3], MJD0[3] */,
                                     int n_min, const float* t_min, const float* v_min, double* chi2_out,
                                     double* dv_out)
{
    __shared__ int sTypes[N_TYPES][N_SEG];
    __shared__ struct chi2_struct sp;
    if (threadIdx.x == 0) {
        for (int t = 0; t < N_TYPES; t++) sTypes[t][0] = types[t];
#ifdef INTERP
        for (int k = 0; k < 3; k++) {
            sp.E_x0[k] = eph[0 + k]; sp.E_y0[k] = eph[3 + k]; sp.E_z0[k] = eph[6 + k];
            sp.S_x0[k] = eph[9 + k]; sp.S_y0[k] = eph[12 + k]; sp.S_z0[k] = eph[15 + k];
            sp.MJD0[k] = eph[18 + k];
        }
#endif
#ifdef NUDGE
        sp.N_obs = n_min;
        for (int k = 0; k < n_min; k++) { sp.t_obs[k] = t_min[k]; sp.V_obs[k] = v_min[k]; }
#endif
    }
    __syncthreads();
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    double p[N_PARAMS];
    for (int i = 0; i < N_PARAMS; i++) p[i] = params[k * N_PARAMS + i];
    CHI_FLOAT dv[N_FILTERS];
    for (int m = 0; m < N_FILTERS; m++) dv[m] = 0;
    CHI_FLOAT r = chi2one(p, data, n_data, n_filters, dv, 0, &sp, sTypes);
    chi2_out[k] = (double)r;
    for (int m = 0; m < n_filters; m++) dv_out[k * n_filters + m] = (double)dv[m];
}
