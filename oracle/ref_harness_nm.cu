/*
 * ref_harness_nm.cu -- TEST INFRASTRUCTURE ONLY.  Tail of the translation unit that runs the
 * reference's chi2_gpu (cuda.c:1326-1833) or, in -DRMSD builds, chi2_gpu_rms (cuda.c:2148-2389)
 * on the host (see ref_nm_shim.h for the head): undoes the shim's macros and provides the entry
 * point, which does what the reference's host does around one launch (asteroid.c:603-606,
 * 628-637,673-675,687-723,728-730): upload the tables, the observations and the start point or
 * model, run the blocks of BSIZE threads, and return each block's best chi^2, parameters and
 * delta_V (chi2_gpu) or the RMSD f0, f1, sample counts and parameter ranges reduced over the
 * blocks (chi2_gpu_rms).  Build: oracle/build_ref.sh (libref_nm_<variant>.so, git-ignored).
 */
#undef __global__
#undef __shared__
#pragma pop_macro("__shared__")
#pragma pop_macro("__global__")
#undef threadIdx
#undef blockIdx
#undef blockDim
#undef __syncthreads
#undef curandState
#undef curand_uniform
#undef curand_normal
#undef atomicAdd
#undef chi2_gpu
#undef chi2_gpu_rms
#undef d_Ntot
#undef d_Nbad
#undef d_f0
#undef d_f1
#undef dLimits
#undef dTypes
#undef dProperty
#undef d_x2_params
#undef d_chi2_params
#undef d_params0
#undef dE_x0
#undef dE_y0
#undef dE_z0
#undef dS_x0
#undef dS_y0
#undef dS_z0
#undef dMJD0

#include <stdlib.h>
#include <string.h>
#include <thread>
#include <vector>

extern "C" int refnm_block_size(void) { return BSIZE; }
extern "C" int refnm_n_params(void) { return N_PARAMS; }
extern "C" unsigned refnm_n_steps(void) { return N_STEPS; }

/* The reference host's uploads (asteroid.c:603-606 and the observation copy), into the host
 * copies of the __device__ variables; the observations as an AoS obs_data array. */
static int refnm_upload(const int* property, int n_params, const int* types, int n_types, const double* limits,
                        int max_types, float ppsi1, float ppsi2, int n_data, int n_filters, const double* mjd,
                        const float* v, const float* w, const int* filt, const double* e_unit, const double* s_unit,
                        const double* eph_e, const double* eph_s, const double* eph_mjd0, int n_min,
                        const float* t_min, const float* v_min, const double* params0, std::vector<struct obs_data>& data)
{
    if (n_params != N_PARAMS || n_types != N_TYPES || n_filters > N_FILTERS || n_data > MAX_DATA) return -1;
    (void)ppsi1;
    (void)ppsi2;
    for (int i = 0; i < N_PARAMS; i++)
        for (int j = 0; j < N_COLUMNS; j++) refnm_dProperty[i][j] = property[i * N_COLUMNS + j];
    for (int t = 0; t < N_TYPES; t++) {
        refnm_dTypes[t][0] = types[t];
        refnm_dLimits[0][t] = (CHI_FLOAT)limits[t];
        refnm_dLimits[1][t] = (CHI_FLOAT)limits[max_types + t];
    }
    memset(&refnm_d_x2_params, 0, sizeof(refnm_d_x2_params));
#ifdef P_PSI
    refnm_d_x2_params.Ppsi1 = ppsi1;
    refnm_d_x2_params.Ppsi2 = ppsi2;
#endif
    memset(&refnm_d_chi2_params, 0, sizeof(refnm_d_chi2_params));
#ifdef NUDGE
    refnm_d_chi2_params.N_obs = n_min;
    for (int k = 0; k < n_min; k++) {
        refnm_d_chi2_params.t_obs[k] = t_min[k];
        refnm_d_chi2_params.V_obs[k] = v_min[k];
    }
#else
    (void)n_min;
    (void)t_min;
    (void)v_min;
#endif
#ifdef INTERP
    for (int k = 0; k < 3; k++) {
        refnm_dE_x0[k] = eph_e[k]; refnm_dE_y0[k] = eph_e[3 + k]; refnm_dE_z0[k] = eph_e[6 + k];
        refnm_dS_x0[k] = eph_s[k]; refnm_dS_y0[k] = eph_s[3 + k]; refnm_dS_z0[k] = eph_s[6 + k];
        refnm_dMJD0[k] = eph_mjd0[k];
    }
#else
    (void)eph_e;
    (void)eph_s;
    (void)eph_mjd0;
#endif
    for (int i = 0; i < N_PARAMS; i++) refnm_d_params0[i] = params0 ? params0[i] : 0.0;
    data.assign((size_t)n_data, obs_data());
    memset(data.data(), 0, sizeof(struct obs_data) * (size_t)n_data);
    for (int i = 0; i < n_data; i++) {
        data[i].V = v[i];
        data[i].w = w[i];
        data[i].MJD = mjd[i];
        data[i].Filter = filt[i];
#ifndef INTERP
        data[i].E_x = e_unit[3 * i]; data[i].E_y = e_unit[3 * i + 1]; data[i].E_z = e_unit[3 * i + 2];
        data[i].S_x = s_unit[3 * i]; data[i].S_y = s_unit[3 * i + 1]; data[i].S_z = s_unit[3 * i + 2];
#else
        (void)e_unit;
        (void)s_unit;
#endif
    }
    return 0;
}

/* n_blocks blocks of BSIZE host threads, one block after the other. */
template <class F>
static void refnm_launch(int n_blocks, F kernel)
{
    refnm::bdim = refnm::dim3h{(unsigned)BSIZE, 1u, 1u};
    refnm::barrier.n = BSIZE;
    for (int b = 0; b < n_blocks; b++) {
        std::vector<std::thread> th;
        th.reserve(BSIZE);
        for (int t = 0; t < BSIZE; t++)
            th.emplace_back([&kernel, b, t] {
                refnm::tid = refnm::dim3h{(unsigned)t, 0u, 0u};
                refnm::bid = refnm::dim3h{(unsigned)b, 0u, 0u};
                kernel();
            });
        for (auto& x : th) x.join();
    }
}

#ifndef RMSD
/* One chi2_gpu launch of n_blocks blocks on the host.  Tables and observations as in
 * ref_harness_host.cu (the engine's layouts); outputs per block. */
extern "C" int refnm_fit(const int* property, int n_params, const int* types, int n_types, const double* limits,
                         int max_types, float ppsi1, float ppsi2, int n_data, int n_filters, const double* mjd,
                         const float* v, const float* w, const int* filt, const double* e_unit, const double* s_unit,
                         const double* eph_e, const double* eph_s, const double* eph_mjd0, int n_min,
                         const float* t_min, const float* v_min, int reopt, const double* params0, int n_blocks,
                         int n_stages, unsigned long long seed, double* best_f, double* best_params, double* best_dv)
{
    std::vector<struct obs_data> data;
    if (refnm_upload(property, n_params, types, n_types, limits, max_types, ppsi1, ppsi2, n_data, n_filters, mjd, v,
                     w, filt, e_unit, s_unit, eph_e, eph_s, eph_mjd0, n_min, t_min, v_min, params0, data))
        return -1;
    std::vector<CHI_FLOAT> d_f((size_t)n_blocks, (CHI_FLOAT)HUGE);
    std::vector<double> d_params((size_t)n_blocks * N_PARAMS, 0.0), d_dV((size_t)n_blocks * N_FILTERS, 0.0);
    std::vector<refnm::Rng> states((size_t)n_blocks * BSIZE);
    for (size_t id = 0; id < states.size(); id++) states[id] = refnm::Rng{seed, (uint64_t)id, 0u, 3 * N_PARAMS, 0u};
    refnm_launch(n_blocks, [&] {
        refnm_chi2_gpu(data.data(), n_data, n_filters, reopt, n_stages, states.data(), d_f.data(), d_params.data(),
                       d_dV.data());
    });
    for (int b = 0; b < n_blocks; b++) {
        best_f[b] = (double)d_f[(size_t)b];
        for (int i = 0; i < N_PARAMS; i++) best_params[b * N_PARAMS + i] = d_params[(size_t)b * N_PARAMS + i];
        for (int m = 0; m < n_filters; m++) best_dv[b * n_filters + m] = d_dV[(size_t)b * N_FILTERS + m];
    }
    return 0;
}

#else

/* One chi2_gpu_rms launch (call index `call` of the host loop) of n_blocks blocks, `samples`
 * random points per thread around the model params0 with step dx_rand.  Outputs f0, f1 (d_f0,
 * d_f1), the counts of evaluated and rejected points (d_Ntot, d_Nbad) and the parameter ranges
 * reduced over the blocks as the reference's host does (asteroid.c:705-716), in float. */
extern "C" int refnm_rmsd(const int* property, int n_params, const int* types, int n_types, const double* limits,
                          int max_types, int n_data, int n_filters, const double* mjd, const float* v, const float* w,
                          const int* filt, const double* e_unit, const double* s_unit, const double* eph_e,
                          const double* eph_s, const double* eph_mjd0, int reopt, const double* params0, int n_blocks,
                          int samples, float dx_rand, unsigned long long seed, unsigned call, double* f01,
                          long long* counts, float* par_min, float* par_max)
{
    std::vector<struct obs_data> data;
    if (refnm_upload(property, n_params, types, n_types, limits, max_types, 0.0f, 0.0f, n_data, n_filters, mjd, v, w,
                     filt, e_unit, s_unit, eph_e, eph_s, eph_mjd0, 0, nullptr, nullptr, params0, data))
        return -1;
    refnm_d_Ntot = refnm_d_Nbad = 0;
    std::vector<CHI_FLOAT> d_f((size_t)n_blocks, (CHI_FLOAT)HUGE);
    std::vector<double> d_params((size_t)n_blocks * N_PARAMS, 0.0), d_dV((size_t)n_blocks * N_FILTERS, 0.0);
    std::vector<float> dpar_min((size_t)n_blocks * N_PARAMS), dpar_max((size_t)n_blocks * N_PARAMS);
    std::vector<refnm::Rng> states((size_t)n_blocks * BSIZE);
    for (size_t id = 0; id < states.size(); id++) states[id] = refnm::Rng{seed, (uint64_t)id, 0u, N_PARAMS, call};
    refnm_launch(n_blocks, [&] {
        refnm_chi2_gpu_rms(data.data(), n_data, n_filters, reopt, samples, states.data(), d_f.data(), d_params.data(),
                           d_dV.data(), dx_rand, dpar_min.data(), dpar_max.data());
    });
    f01[0] = refnm_d_f0;
    f01[1] = refnm_d_f1;
    counts[0] = refnm_d_Ntot;
    counts[1] = refnm_d_Nbad;
    for (int j = 0; j < N_PARAMS; j++) {
        par_min[j] = 1e30f;
        par_max[j] = -1e30f;
        for (int i = 0; i < n_blocks; i++) {
            const int k = i * N_PARAMS + j;
            if (dpar_min[(size_t)k] < par_min[j]) par_min[j] = dpar_min[(size_t)k];
            if (dpar_max[(size_t)k] > par_max[j]) par_max[j] = dpar_max[(size_t)k];
        }
    }
    return 0;
}

#endif
