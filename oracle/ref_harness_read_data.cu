/*
 * ref_harness_read_data.cu -- TEST INFRASTRUCTURE ONLY.  Runs the reference's own host readers on
 * the CPU: read_data() (read_data.c:6-377: the light curve, the three HORIZONS ephemerides, the
 * magnitude and light-time conversions, the -plot grid) and, in -DNUDGE builds,
 * prepare_chi2_params() (misc.c:279-323: observed.min), so that the engine's C reader
 * (host/read_data.c, host/misc.c) can be pinned to them bit for bit.
 *
 * oracle/build_ref.sh streams into one translation unit: the reference's asteroid.h, this file's
 * head (below, up to the reference sources), the reference's read_data.c and misc.c read in
 * place with their #include "asteroid.h" removed, and this file's tail.  The head replaces the two
 * CUDA runtime calls the readers make with host equivalents: cudaMallocHost is malloc and
 * cudaMemcpyToSymbol copies into the host copy of the __device__ symbol, which the tail reads.
 * Nothing of the reference is written to disk.
 */
#ifndef REFR_TAIL
#include <stdlib.h>
#include <string.h>
#include <unistd.h>

#define cudaMallocHost(pp, n) ((*(void**)(pp) = malloc(n)) ? cudaSuccess : cudaErrorMemoryAllocation)
#define cudaMemcpyToSymbol(sym, src, n, off, kind) (memcpy((char*)&(sym) + (off), (src), (n)), cudaSuccess)

#else  /* the tail, after read_data.c and misc.c */

#undef cudaMallocHost
#undef cudaMemcpyToSymbol

/* read_data() (and prepare_chi2_params() under NUDGE) in directory `dir`, as the reference's
 * main() calls them (asteroid.c:436-441), then everything they computed.  Arrays are sized by the
 * caller: n_max points, nplot plot points.  E/S unit vectors exist only without INTERP (with it
 * the reference interpolates them on the GPU and frees its host copies). */
extern "C" int refr_read(const char* dir, const char* lc_file, int n_max, int nplot, int* n_data, int* n_filters,
                         char* filters, double* mjd, float* v, float* w, int* filt, double* e_unit, double* s_unit,
                         double* hmjd0, double* eph /* E_x0,E_y0,E_z0,S_x0,S_y0,S_z0,MJD0 [7][3] */,
                         double* plot_t, double* plot_e, double* plot_s, int* n_min, float* t_min, float* v_min)
{
    char cwd[4096];
    if (!getcwd(cwd, sizeof cwd) || chdir(dir) != 0) return -1;
    int N_data = 0, N_filters = 0;
    const int rc = read_data((char*)lc_file, &N_data, &N_filters, nplot);
#ifdef NUDGE
    if (rc == 0) prepare_chi2_params(&N_data);
#endif
    if (chdir(cwd) != 0 || rc != 0) return -2;
    if (N_data > n_max) return -3;
    *n_data = N_data;
    *n_filters = N_filters;
    for (int k = 0; k < N_filters; k++) filters[k] = all_filters[k];
    for (int i = 0; i < N_data; i++) {
        mjd[i] = hData[i].MJD;
        v[i] = hData[i].V;
        w[i] = hData[i].w;
        filt[i] = hData[i].Filter;
#ifndef INTERP
        e_unit[3 * i] = hData[i].E_x; e_unit[3 * i + 1] = hData[i].E_y; e_unit[3 * i + 2] = hData[i].E_z;
        s_unit[3 * i] = hData[i].S_x; s_unit[3 * i + 1] = hData[i].S_y; s_unit[3 * i + 2] = hData[i].S_z;
#endif
    }
    *hmjd0 = hMJD0;
    const double* src[7] = {E_x0, E_y0, E_z0, S_x0, S_y0, S_z0, MJD0};
    for (int r = 0; r < 7; r++)
        for (int k = 0; k < 3; k++) eph[3 * r + k] = src[r][k];
    for (int i = 0; i < nplot; i++) {
        plot_t[i] = hPlot[i].MJD;
#ifndef INTERP
        plot_e[3 * i] = hPlot[i].E_x; plot_e[3 * i + 1] = hPlot[i].E_y; plot_e[3 * i + 2] = hPlot[i].E_z;
        plot_s[3 * i] = hPlot[i].S_x; plot_s[3 * i + 1] = hPlot[i].S_y; plot_s[3 * i + 2] = hPlot[i].S_z;
#endif
    }
#ifdef NUDGE
    *n_min = d_chi2_params.N_obs;
    for (int k = 0; k < d_chi2_params.N_obs; k++) {
        t_min[k] = d_chi2_params.t_obs[k];
        v_min[k] = d_chi2_params.V_obs[k];
    }
#else
    *n_min = 0;
    (void)t_min;
    (void)v_min;
#endif
    free(hData);
    free(MJD_obs);
    if (nplot > 0) free(hPlot);
    hData = NULL;
    hPlot = NULL;
    MJD_obs = NULL;
    return 0;
}

#endif
