/*
 * ref_gpu_loader.cpp -- TEST INFRASTRUCTURE ONLY.  Runs the reference's own chi2one on the GPU:
 * loads oracle/_ref/ref_<variant>.cubin (built from the reference sources by build_ref.sh) with
 * the CUDA driver API and launches its refk_pack / refk_eval harness kernels
 * (ref_harness_kernel.cu).  Used by tests/test_ref_kernel.py to hold the engine's FP64 path to
 * 1e-12 relative chi^2 against the reference kernel, and by tests/golden/ fixture generation on
 * the GPU; refn_fit runs the reference's setup_kernel + chi2_gpu (ref_nm_<variant>.cubin) for
 * tests/test_ref_simplex.py.  Built on the GPU machine by asteroid_gb300.build.build_oracle().
 */
#include <cuda.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>

#include <initializer_list>

static char g_err[512];

extern "C" const char* refk_last_error(void) { return g_err; }

#define CK(x)                                                                             \
    do {                                                                                  \
        CUresult r_ = (x);                                                                \
        if (r_ != CUDA_SUCCESS) {                                                         \
            const char* s_ = nullptr;                                                     \
            cuGetErrorString(r_, &s_);                                                    \
            snprintf(g_err, sizeof(g_err), "%s: %s", #x, s_ ? s_ : "?");                  \
            rc = -1;                                                                      \
            goto done;                                                                    \
        }                                                                                 \
    } while (0)

/* obs_bytes: sizeof(struct obs_data) of the build (24 with INTERP, 72 without). */
extern "C" int refk_eval_batch(const char* cubin, int obs_bytes, int n_params, const double* params, int n,
                               const int* types, int n_types, int n_data, int n_filters, const double* mjd,
                               const float* v, const float* w, const int* filt, const double* e_unit,
                               const double* s_unit, const double* eph21, int n_min, const float* t_min,
                               const float* v_min, double* chi2_out, double* dv_out, double* kernel_ms)
{
    int rc = 0;
    CUdevice dev;
    CUcontext ctx = nullptr;
    CUmodule mod = nullptr;
    CUfunction fpack, feval;
    CUdeviceptr d_p = 0, d_types = 0, d_mjd = 0, d_v = 0, d_w = 0, d_f = 0, d_e = 0, d_s = 0, d_eph = 0, d_tmin = 0,
                d_vmin = 0, d_obs = 0, d_chi2 = 0, d_dv = 0;
    const int nn = n_data;
    CK(cuInit(0));
    CK(cuDeviceGet(&dev, 0));
    CK(cuDevicePrimaryCtxRetain(&ctx, dev));
    CK(cuCtxPushCurrent(ctx));
    CK(cuModuleLoad(&mod, cubin));
    CK(cuModuleGetFunction(&fpack, mod, "refk_pack"));
    CK(cuModuleGetFunction(&feval, mod, "refk_eval"));
    CK(cuMemAlloc(&d_p, sizeof(double) * (size_t)n * n_params));
    CK(cuMemAlloc(&d_types, sizeof(int) * (size_t)n_types));
    CK(cuMemAlloc(&d_mjd, sizeof(double) * nn));
    CK(cuMemAlloc(&d_v, sizeof(float) * nn));
    CK(cuMemAlloc(&d_w, sizeof(float) * nn));
    CK(cuMemAlloc(&d_f, sizeof(int) * nn));
    CK(cuMemAlloc(&d_e, sizeof(double) * 3 * nn));
    CK(cuMemAlloc(&d_s, sizeof(double) * 3 * nn));
    CK(cuMemAlloc(&d_eph, sizeof(double) * 21));
    CK(cuMemAlloc(&d_tmin, sizeof(float) * 16));
    CK(cuMemAlloc(&d_vmin, sizeof(float) * 16));
    CK(cuMemAlloc(&d_obs, (size_t)obs_bytes * nn));
    CK(cuMemAlloc(&d_chi2, sizeof(double) * n));
    CK(cuMemAlloc(&d_dv, sizeof(double) * (size_t)n * n_filters));
    CK(cuMemcpyHtoD(d_p, params, sizeof(double) * (size_t)n * n_params));
    CK(cuMemcpyHtoD(d_types, types, sizeof(int) * (size_t)n_types));
    CK(cuMemcpyHtoD(d_mjd, mjd, sizeof(double) * nn));
    CK(cuMemcpyHtoD(d_v, v, sizeof(float) * nn));
    CK(cuMemcpyHtoD(d_w, w, sizeof(float) * nn));
    CK(cuMemcpyHtoD(d_f, filt, sizeof(int) * nn));
    CK(cuMemcpyHtoD(d_e, e_unit, sizeof(double) * 3 * nn));
    CK(cuMemcpyHtoD(d_s, s_unit, sizeof(double) * 3 * nn));
    CK(cuMemcpyHtoD(d_eph, eph21, sizeof(double) * 21));
    if (n_min > 0) {
        CK(cuMemcpyHtoD(d_tmin, t_min, sizeof(float) * n_min));
        CK(cuMemcpyHtoD(d_vmin, v_min, sizeof(float) * n_min));
    }
    {
        void* args[] = {&d_mjd, &d_v, &d_w, &d_f, &d_e, &d_s, (void*)&nn, &d_obs};
        CK(cuLaunchKernel(fpack, (nn + 127) / 128, 1, 1, 128, 1, 1, 0, nullptr, args, nullptr));
    }
    {
        int nv = n, nd = n_data, nf = n_filters, nm = n_min;
        void* args[] = {&d_p, &nv, &d_types, &d_obs, &nd, &nf, &d_eph, &nm, &d_tmin, &d_vmin, &d_chi2, &d_dv};
        CUevent e0 = nullptr, e1 = nullptr;
        CK(cuEventCreate(&e0, CU_EVENT_DEFAULT));
        CK(cuEventCreate(&e1, CU_EVENT_DEFAULT));
        CK(cuEventRecord(e0, nullptr));
        CK(cuLaunchKernel(feval, (n + 63) / 64, 1, 1, 64, 1, 1, 0, nullptr, args, nullptr));
        CK(cuEventRecord(e1, nullptr));
        CK(cuEventSynchronize(e1));
        float ms = 0;
        CK(cuEventElapsedTime(&ms, e0, e1));
        if (kernel_ms) *kernel_ms = ms;
        cuEventDestroy(e0);
        cuEventDestroy(e1);
    }
    CK(cuCtxSynchronize());
    CK(cuMemcpyDtoH(chi2_out, d_chi2, sizeof(double) * n));
    CK(cuMemcpyDtoH(dv_out, d_dv, sizeof(double) * (size_t)n * n_filters));
done:
    for (CUdeviceptr p : {d_p, d_types, d_mjd, d_v, d_w, d_f, d_e, d_s, d_eph, d_tmin, d_vmin, d_obs, d_chi2, d_dv})
        if (p) cuMemFree(p);
    if (mod) cuModuleUnload(mod);
    if (ctx) {
        cuCtxPopCurrent(nullptr);
        cuDevicePrimaryCtxRelease(dev);
    }
    return rc;
}

/* The reference's own setup_kernel + chi2_gpu (cuda.c:2039,1326) from ref_nm_<variant>.cubin:
 * one fitting pass of n_blocks x block chains as asteroid.c:626-688 launches it, with the
 * tables and parameters set by refn_setup (ref_harness_nm.cu).  Outputs: the reference's
 * per-block results (d_f, d_params, d_dV with its N_FILTERS stride dv_stride), and from the
 * instrumentation hooks every chain's final chi^2 and iteration count per stage
 * ([n_stages][threads]) and chi2one calls per thread.  *kernel_ms = chi2_gpu's device time. */
static CUfunction find_function(CUmodule mod, const char* prefix)
{
    unsigned int n = 0;
    if (cuModuleGetFunctionCount(&n, mod) != CUDA_SUCCESS || n == 0 || n > 4096) return nullptr;
    CUfunction fs[4096];
    if (cuModuleEnumerateFunctions(fs, n, mod) != CUDA_SUCCESS) return nullptr;
    for (unsigned int i = 0; i < n; i++) {
        const char* name = nullptr;
        if (cuFuncGetName(&name, fs[i]) == CUDA_SUCCESS && name && strncmp(name, prefix, strlen(prefix)) == 0)
            return fs[i];
    }
    return nullptr;
}

extern "C" int refn_fit(const char* cubin, const int* property, const int* types, const double* limits,
                        int max_types, float ppsi1, float ppsi2, int n_data, int n_filters, const double* mjd,
                        const float* v, const float* w, const int* filt, const double* e_unit, const double* s_unit,
                        const double* eph21, int n_min, const float* t_min, const float* v_min, uint64_t seed,
                        int n_blocks, int block, int n_stages, int reopt, const double* params0,
                        unsigned int n_steps, int* sizes_out /* [5] */, double* block_f, double* block_params,
                        double* block_dv, int dv_stride, double* chain_f, int* chain_l, unsigned int* evals,
                        double* kernel_ms)
{
    int rc = 0;
    CUdevice dev;
    CUcontext ctx = nullptr;
    CUmodule mod = nullptr;
    CUfunction fsizes, fsetup, fpack, frng = nullptr, ffit = nullptr;
    CUdeviceptr d_sizes = 0, d_prop = 0, d_types = 0, d_lim = 0, d_p0 = 0, d_eph = 0, d_tmin = 0, d_vmin = 0,
                d_mjd = 0, d_v = 0, d_w = 0, d_f = 0, d_e = 0, d_s = 0, d_obs = 0, d_state = 0, d_bf = 0, d_bp = 0,
                d_bdv = 0, d_cf = 0, d_cl = 0, d_ev = 0;
    CUevent e0 = nullptr, e1 = nullptr;
    int sz[5] = {0, 0, 0, 0, 0};
    const int threads = n_blocks * block, nn = n_data;
    CK(cuInit(0));
    CK(cuDeviceGet(&dev, 0));
    CK(cuDevicePrimaryCtxRetain(&ctx, dev));
    CK(cuCtxPushCurrent(ctx));
    CK(cuModuleLoad(&mod, cubin));
    CK(cuModuleGetFunction(&fsizes, mod, "refn_sizes"));
    CK(cuModuleGetFunction(&fsetup, mod, "refn_setup"));
    CK(cuModuleGetFunction(&fpack, mod, "refk_pack"));
    frng = find_function(mod, "_Z12setup_kernel");
    ffit = find_function(mod, "_Z8chi2_gpu");
    if (!frng || !ffit) {
        snprintf(g_err, sizeof(g_err), "setup_kernel / chi2_gpu not found in %s", cubin);
        rc = -1;
        goto done;
    }
    CK(cuMemAlloc(&d_sizes, sizeof(sz)));
    {
        void* args[] = {&d_sizes};
        CK(cuLaunchKernel(fsizes, 1, 1, 1, 1, 1, 1, 0, nullptr, args, nullptr));
    }
    CK(cuMemcpyDtoH(sz, d_sizes, sizeof(sz)));
    if (sizes_out) memcpy(sizes_out, sz, sizeof(sz));
    if (sz[3] <= 0 || sz[4] <= 0 || sz[4] > max_types || n_filters > dv_stride) {
        snprintf(g_err, sizeof(g_err), "tables do not match the build (N_PARAMS %d, N_TYPES %d)", sz[3], sz[4]);
        rc = -2;
        goto done;
    }
    CK(cuMemAlloc(&d_prop, sizeof(int) * 6 * sz[3]));
    CK(cuMemAlloc(&d_types, sizeof(int) * (size_t)max_types));
    CK(cuMemAlloc(&d_lim, sizeof(double) * 2 * (size_t)max_types));
    CK(cuMemAlloc(&d_p0, sizeof(double) * sz[3]));
    CK(cuMemAlloc(&d_eph, sizeof(double) * 21));
    CK(cuMemAlloc(&d_tmin, sizeof(float) * 16));
    CK(cuMemAlloc(&d_vmin, sizeof(float) * 16));
    CK(cuMemAlloc(&d_mjd, sizeof(double) * nn));
    CK(cuMemAlloc(&d_v, sizeof(float) * nn));
    CK(cuMemAlloc(&d_w, sizeof(float) * nn));
    CK(cuMemAlloc(&d_f, sizeof(int) * nn));
    CK(cuMemAlloc(&d_e, sizeof(double) * 3 * nn));
    CK(cuMemAlloc(&d_s, sizeof(double) * 3 * nn));
    CK(cuMemAlloc(&d_obs, (size_t)sz[1] * nn));
    CK(cuMemAlloc(&d_state, (size_t)sz[0] * threads));
    CK(cuMemAlloc(&d_bf, (size_t)sz[2] * n_blocks));
    CK(cuMemAlloc(&d_bp, sizeof(double) * sz[3] * (size_t)n_blocks));
    CK(cuMemAlloc(&d_bdv, sizeof(double) * dv_stride * (size_t)n_blocks));
    CK(cuMemAlloc(&d_cf, sizeof(double) * (size_t)n_stages * threads));
    CK(cuMemAlloc(&d_cl, sizeof(int) * (size_t)n_stages * threads));
    CK(cuMemAlloc(&d_ev, sizeof(unsigned int) * (size_t)threads));
    CK(cuMemsetD8(d_bp, 0, sizeof(double) * sz[3] * (size_t)n_blocks));
    CK(cuMemsetD8(d_bdv, 0, sizeof(double) * dv_stride * (size_t)n_blocks));
    CK(cuMemsetD8(d_cf, 0, sizeof(double) * (size_t)n_stages * threads));
    CK(cuMemsetD8(d_cl, 0, sizeof(int) * (size_t)n_stages * threads));
    CK(cuMemsetD8(d_ev, 0, sizeof(unsigned int) * (size_t)threads));
    CK(cuMemcpyHtoD(d_prop, property, sizeof(int) * 6 * sz[3]));
    CK(cuMemcpyHtoD(d_types, types, sizeof(int) * (size_t)max_types));
    CK(cuMemcpyHtoD(d_lim, limits, sizeof(double) * 2 * (size_t)max_types));
    CK(cuMemsetD8(d_p0, 0, sizeof(double) * sz[3]));
    if (params0) CK(cuMemcpyHtoD(d_p0, params0, sizeof(double) * sz[3]));
    CK(cuMemcpyHtoD(d_eph, eph21, sizeof(double) * 21));
    if (n_min > 0) {
        CK(cuMemcpyHtoD(d_tmin, t_min, sizeof(float) * n_min));
        CK(cuMemcpyHtoD(d_vmin, v_min, sizeof(float) * n_min));
    }
    CK(cuMemcpyHtoD(d_mjd, mjd, sizeof(double) * nn));
    CK(cuMemcpyHtoD(d_v, v, sizeof(float) * nn));
    CK(cuMemcpyHtoD(d_w, w, sizeof(float) * nn));
    CK(cuMemcpyHtoD(d_f, filt, sizeof(int) * nn));
    CK(cuMemcpyHtoD(d_e, e_unit, sizeof(double) * 3 * nn));
    CK(cuMemcpyHtoD(d_s, s_unit, sizeof(double) * 3 * nn));
    {
        void* args[] = {&d_mjd, &d_v, &d_w, &d_f, &d_e, &d_s, (void*)&nn, &d_obs};
        CK(cuLaunchKernel(fpack, (nn + 127) / 128, 1, 1, 128, 1, 1, 0, nullptr, args, nullptr));
    }
    {
        int mt = max_types, nm = n_min, th = threads;
        unsigned int ns = n_steps;
        float p1 = ppsi1, p2 = ppsi2;
        const bool with_p0 = params0 != nullptr;
        CUdeviceptr p0 = with_p0 ? d_p0 : 0;
        void* args[] = {&d_prop, &d_types, &d_lim, &mt, &p1, &p2, &p0, &d_eph, &nm, &d_tmin, &d_vmin, &ns,
                        &d_cf, &d_cl, &d_ev, &th};
        CK(cuLaunchKernel(fsetup, 1, 1, 1, 1, 1, 1, 0, nullptr, args, nullptr));
    }
    {
        unsigned long sd = (unsigned long)seed;
        int gen = 1;
        void* args[] = {&d_state, &sd, &d_bf, &gen};
        CK(cuLaunchKernel(frng, n_blocks, 1, 1, block, 1, 1, 0, nullptr, args, nullptr));
    }
    {
        int nd = n_data, nf = n_filters, ro = reopt, ns = n_stages;
        void* args[] = {&d_obs, &nd, &nf, &ro, &ns, &d_state, &d_bf, &d_bp, &d_bdv};
        CK(cuEventCreate(&e0, CU_EVENT_DEFAULT));
        CK(cuEventCreate(&e1, CU_EVENT_DEFAULT));
        CK(cuEventRecord(e0, nullptr));
        CK(cuLaunchKernel(ffit, n_blocks, 1, 1, block, 1, 1, 0, nullptr, args, nullptr));
        CK(cuEventRecord(e1, nullptr));
        CK(cuEventSynchronize(e1));
        float ms = 0;
        CK(cuEventElapsedTime(&ms, e0, e1));
        if (kernel_ms) *kernel_ms = ms;
    }
    CK(cuCtxSynchronize());
    if (sz[2] == 8) {
        CK(cuMemcpyDtoH(block_f, d_bf, sizeof(double) * n_blocks));
    } else {
        float tmp[1024];
        for (int b0 = 0; b0 < n_blocks; b0 += 1024) {
            const int nb = n_blocks - b0 < 1024 ? n_blocks - b0 : 1024;
            CK(cuMemcpyDtoH(tmp, d_bf + sizeof(float) * b0, sizeof(float) * nb));
            for (int b = 0; b < nb; b++) block_f[b0 + b] = tmp[b];
        }
    }
    CK(cuMemcpyDtoH(block_params, d_bp, sizeof(double) * sz[3] * (size_t)n_blocks));
    CK(cuMemcpyDtoH(block_dv, d_bdv, sizeof(double) * dv_stride * (size_t)n_blocks));
    CK(cuMemcpyDtoH(chain_f, d_cf, sizeof(double) * (size_t)n_stages * threads));
    CK(cuMemcpyDtoH(chain_l, d_cl, sizeof(int) * (size_t)n_stages * threads));
    CK(cuMemcpyDtoH(evals, d_ev, sizeof(unsigned int) * (size_t)threads));
done:
    if (e0) cuEventDestroy(e0);
    if (e1) cuEventDestroy(e1);
    for (CUdeviceptr p : {d_sizes, d_prop, d_types, d_lim, d_p0, d_eph, d_tmin, d_vmin, d_mjd, d_v, d_w, d_f, d_e, d_s,
                          d_obs, d_state, d_bf, d_bp, d_bdv, d_cf, d_cl, d_ev})
        if (p) cuMemFree(p);
    if (mod) cuModuleUnload(mod);
    if (ctx) {
        cuCtxPopCurrent(nullptr);
        cuDevicePrimaryCtxRelease(dev);
    }
    return rc;
}

/* The reference's compute_rgb (ref_animate.cubin, harness refa_render) for n_frames snapshots
 * of 1080 x 1080 pixels: rgb receives n_frames * 1080 * 1080 * 3 bytes in its d_rgb layout. */
extern "C" int refk_render(const char* cubin, const double* geo, int n_frames, unsigned char* rgb)
{
    int rc = 0;
    CUdevice dev;
    CUcontext ctx = nullptr;
    CUmodule mod = nullptr;
    CUfunction fr;
    CUdeviceptr d_geo = 0, d_rgb = 0;
    const size_t frame = (size_t)1080 * 1080 * 3;
    CK(cuInit(0));
    CK(cuDeviceGet(&dev, 0));
    CK(cuDevicePrimaryCtxRetain(&ctx, dev));
    CK(cuCtxPushCurrent(ctx));
    CK(cuModuleLoad(&mod, cubin));
    CK(cuModuleGetFunction(&fr, mod, "refa_render"));
    CK(cuMemAlloc(&d_geo, sizeof(double) * 20 * (size_t)n_frames));
    CK(cuMemAlloc(&d_rgb, frame * (size_t)n_frames));
    CK(cuMemcpyHtoD(d_geo, geo, sizeof(double) * 20 * (size_t)n_frames));
    for (int f = 0; f < n_frames; f++) {
        int ff = f;
        void* args[] = {&d_rgb, &d_geo, &ff};
        /* 1080^2 = 2025 x 576: every thread reaches compute_rgb's __syncthreads. */
        CK(cuLaunchKernel(fr, 2025, 1, 1, 576, 1, 1, 0, nullptr, args, nullptr));
    }
    CK(cuCtxSynchronize());
    CK(cuMemcpyDtoH(rgb, d_rgb, frame * (size_t)n_frames));
done:
    if (d_geo) cuMemFree(d_geo);
    if (d_rgb) cuMemFree(d_rgb);
    if (mod) cuModuleUnload(mod);
    if (ctx) {
        cuCtxPopCurrent(nullptr);
        cuDevicePrimaryCtxRelease(dev);
    }
    return rc;
}
