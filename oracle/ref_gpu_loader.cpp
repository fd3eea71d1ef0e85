/*
 * ref_gpu_loader.cpp -- TEST INFRASTRUCTURE ONLY.  Runs the reference's own chi2one on the GPU:
 * loads oracle/_ref/ref_<variant>.cubin (built from the reference sources by build_ref.sh) with
 * the CUDA driver API and launches its refk_pack / refk_eval harness kernels
 * (ref_harness_kernel.cu).  Used by tests/test_ref_kernel.py to hold the engine's FP64 path to
 * 1e-12 relative chi^2 against the reference kernel, and by tests/golden/ fixture generation on
 * the GPU.  Built on the GPU machine by asteroid_gb300.build.build_oracle().
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
