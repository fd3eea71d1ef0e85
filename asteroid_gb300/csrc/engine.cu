// engine.cu -- context, observation packing, chi^2 batch evaluation and model curves.
//
// Replaces the reference's gpu_prepare.c (pinned AoS obs_data read zero-copy, thread 0 of
// every block copying it serially into shared memory, cuda.c:1350-1354) with an SoA device
// buffer that each CTA stages into shared memory with one bulk copy, and chi2one calls from
// inside the simplex kernel with a batch entry point (one thread per parameter vector).
#include <cuda_runtime.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <vector>

#include "asteroid_gb300.h"
#include "engine.cuh"
#include "mixed.cuh"
#include "model.cuh"
#include "prep.cuh"
#include "staging.cuh"

namespace ast {

int build_dev_model(const ast_model* m, const ast_obs_set* obs, DevModel* dm)
{
    memset(dm, 0, sizeof(*dm));
    if (m->n_params <= 0 || m->n_params > AST_MAX_PARAMS || m->n_types <= 0 || m->n_types > AST_MAX_TYPES)
        return ast_set_error(AST_E_INVALID, "model: n_params %d / n_types %d out of range", m->n_params, m->n_types);
    dm->flags = m->flags;
    dm->n_params = m->n_params;
    dm->n_filters = obs ? obs->n_filters : 1;
    dm->n_data = obs ? obs->n_data : 0;
    dm->time_step = m->time_step;
    for (int i = 0; i < m->n_params; i++) {
        dm->ptype[i] = (int8_t)m->property[i][AST_P_TYPE];
        dm->indep[i] = (int8_t)m->property[i][AST_P_INDEPENDENT];
        dm->frozen[i] = (int8_t)m->property[i][AST_P_FROZEN];
        dm->periodic[i] = (int8_t)m->property[i][AST_P_PERIODIC];
        if (dm->ptype[i] < 0 || dm->ptype[i] >= m->n_types)
            return ast_set_error(AST_E_INVALID, "model: parameter %d has type %d", i, dm->ptype[i]);
    }
    for (int t = 0; t < AST_MAX_TYPES; t++) {
        dm->idx[t] = (int8_t)(t < m->n_types ? m->types[t] : -1);
        dm->lim0[t] = m->limits[0][t];
        dm->lim1[t] = m->limits[1][t];
    }
    dm->t = m->ids;
    const ast_type_ids& T = m->ids;
    const int need[] = {T.theta_M, T.phi_M, T.phi_0, T.L, T.c_tumb, T.b_tumb, T.Es, T.psi_0};
    for (int k = 0; k < 8; k++)
        if (need[k] < 0 || need[k] >= m->n_types || m->types[need[k]] < 0)
            return ast_set_error(AST_E_INVALID, "model: type table incomplete");
    if ((m->flags & AST_TORQUE) && (T.Ti < 0 || T.Ts < 0 || T.Tl < 0))
        return ast_set_error(AST_E_INVALID, "model: TORQUE without torque types");
    if ((m->flags & AST_BC) && (T.c < 0 || T.b < 0)) return ast_set_error(AST_E_INVALID, "model: BC without c, b");
    if ((m->flags & AST_BW_BALL) && (T.theta_R < 0 || T.phi_R < 0 || T.kappa < 0))
        return ast_set_error(AST_E_INVALID, "model: BW_BALL without theta_R, phi_R, kappa");
    dm->ppsi1 = m->ppsi1;
    dm->ppsi2 = m->ppsi2;
    if (obs) {
        dm->n_min = obs->n_minima;
        for (int k = 0; k < AST_NOBS_MAX; k++) { dm->t_min[k] = obs->t_min[k]; dm->v_min[k] = obs->v_min[k]; }
        memcpy(dm->eph_e, obs->eph_e, sizeof(dm->eph_e));
        memcpy(dm->eph_s, obs->eph_s, sizeof(dm->eph_s));
        memcpy(dm->eph_mjd0, obs->eph_mjd0, sizeof(dm->eph_mjd0));
    }
    return AST_OK;
}

// Parameter-independent per-observation quantities, once per object, in the reference's
// expressions: the RK4 step count and size of interval (i-1, i) (cuda.c:321-323) and, under
// INTERP, the interpolated unit E and S at the asteroid time (cuda.c:528-545).
__global__ void prep_obs_kernel(DevModel M, char* base, ObsLayout L, int64_t n)
{
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n) prep_obs_point(M, base, L, n, i);
}

__global__ void prep_sums_kernel(DevModel M, char* base, ObsLayout L, int64_t n)
{
    if (blockIdx.x == 0 && threadIdx.x == 0) prep_obs_sums(M, base, L, n);
}

// Host image of an object's SoA block: t, V, w, filter and (without INTERP) the unit E and S
// vectors; h, nst, the INTERP vectors and the mixed-path arrays are filled on the device.
void obs_image(const ast_model* model, const ast_obs_set* obs, const ObsLayout& L, std::vector<unsigned char>& img)
{
    const int64_t n = obs->n_data;
    img.assign((size_t)L.bytes, 0);
    unsigned char* b = img.data();
    memcpy(b + L.off_t, obs->mjd, 8 * n);
    memcpy(b + L.off_v, obs->v, 4 * n);
    memcpy(b + L.off_w, obs->w, 4 * n);
    memcpy(b + L.off_f, obs->filter, 4 * n);
    if (!(model->flags & AST_INTERP)) {
        double* ex = (double*)(b + L.off_e);
        double* sx = (double*)(b + L.off_s);
        for (int64_t i = 0; i < n; i++)
            for (int k = 0; k < 3; k++) {
                ex[k * n + i] = obs->e_unit[3 * i + k];
                sx[k * n + i] = obs->s_unit[3 * i + k];
            }
    }
}

// The parameter-independent preparation of an uploaded block (prep.cuh), stream-ordered.
int launch_prep(const DevModel& dm, char* d_block, const ObsLayout& L, int64_t n, cudaStream_t s)
{
    prep_obs_kernel<<<(unsigned)((n + 127) / 128), 128, 0, s>>>(dm, d_block, L, n);
    AST_CUDA(cudaGetLastError());
    prep_sums_kernel<<<1, 32, 0, s>>>(dm, d_block, L, n);
    AST_CUDA(cudaGetLastError());
    return AST_OK;
}

// One thread per parameter vector; the block's observations are staged into shared memory.
template <class CF, int PREC>
__global__ void __launch_bounds__(128) eval_kernel(DevModel M, const void* g_obs, ObsLayout L, int use_smem,
                                                   const double* __restrict__ params, int64_t n,
                                                   double* __restrict__ chi2, double* __restrict__ dv,
                                                   unsigned long long* err)
{
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ uint64_t bar;
    __shared__ float4 trig[PREC != AST_PREC_FP64 ? kTrigTable : 1];
    if (PREC != AST_PREC_FP64) {
        trig_table_fill(trig);
        __syncthreads();
    }
    const bool staged = use_smem ? bulk_stage(smem, g_obs, (uint32_t)L.bytes, &bar, err) : false;
    const ObsView o = L.view(staged ? (const void*)smem : g_obs, M.n_data);
    const int N = M.n_params;
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
        double p[AST_MAX_PARAMS];
        for (int i = 0; i < N; i++) p[i] = params[k * N + i];
        CF d[AST_MAX_FILTERS];
        for (int m = 0; m < M.n_filters; m++) d[m] = 0;
        CF r;
        if (PREC == AST_PREC_FP64)
            r = chi2_fp64<CF>(M, o, p, d);
        else
            r = chi2_mixed<CF, PREC == AST_PREC_MIXED_RHS32>(M, o, p, d, trig);
        chi2[k] = (double)r;
        if (dv)
            for (int m = 0; m < M.n_filters; m++) dv[k * M.n_filters + m] = (double)d[m];
    }
    bulk_drain(&bar, staged || !use_smem);
}

// Model magnitudes (and, with geo, the renderer's geometry) of one parameter vector at every
// observation (single thread: the RK4 recursion is sequential in time).
__global__ void model_curve_kernel(DevModel M, const void* g_obs, ObsLayout L, const double* params, double* vmod,
                                   double* geo = nullptr)
{
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    const ObsView o = L.view(g_obs, M.n_data);
    double p[AST_MAX_PARAMS];
    for (int i = 0; i < M.n_params; i++) p[i] = params[i];
    double d[AST_MAX_FILTERS];
    DevModel M2 = M;
    M2.flags &= ~AST_NUDGE;  // the curve is the brightness model alone
    chi2_fp64<double>(M2, o, p, d, vmod, nullptr, geo);
}

// Euler angles at every observation along the FP64 or the mixed-precision integration.
template <int PREC>
__global__ void model_angles_kernel(DevModel M, const void* g_obs, ObsLayout L, const double* params, double* ang)
{
    __shared__ float4 trig[kTrigTable];
    trig_table_fill(trig);
    __syncthreads();
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    const ObsView o = L.view(g_obs, M.n_data);
    double p[AST_MAX_PARAMS];
    for (int i = 0; i < M.n_params; i++) p[i] = params[i];
    double d[AST_MAX_FILTERS];
    DevModel M2 = M;
    M2.flags &= ~AST_NUDGE;
    if (PREC == AST_PREC_FP64) chi2_fp64<double>(M2, o, p, d, nullptr, ang);
    else chi2_mixed<double, PREC == AST_PREC_MIXED_RHS32>(M2, o, p, d, trig, ang);
}

// FMA throughput probe (roofline denominators for CUDA-core bound kernels).
template <class T>
__global__ void fma_probe_kernel(T* out, int iters, T a, T b)
{
    T x0 = (T)(threadIdx.x * 1e-3), x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6,
      x7 = x0 + 7;
    for (int i = 0; i < iters; ++i) {
        x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
        x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
    }
    out[blockIdx.x * (int64_t)blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}

int set_device(int device)
{
    int cur = 0;
    AST_CUDA(cudaGetDevice(&cur));
    if (device >= 0 && device != cur) AST_CUDA(cudaSetDevice(device));
    return AST_OK;
}

}  // namespace ast

using namespace ast;

static int validate_obs(const ast_model* m, const ast_obs_set* o)
{
    if (!o) return ast_set_error(AST_E_INVALID, "ast_prepare: NULL observations");
    if (o->n_data <= 0 || o->n_data > AST_MAX_DATA)
        return ast_set_error(AST_E_TOO_LARGE, "ast_prepare: n_data %d outside 1..%d", o->n_data, AST_MAX_DATA);
    if (o->n_filters <= 0 || o->n_filters > AST_MAX_FILTERS)
        return ast_set_error(AST_E_TOO_LARGE, "ast_prepare: n_filters %d outside 1..%d", o->n_filters, AST_MAX_FILTERS);
    if (o->n_data <= m->n_params + o->n_filters)
        return ast_set_error(AST_E_INVALID, "ast_prepare: %d observations leave no degrees of freedom for %d parameters",
                             o->n_data, m->n_params);
    if (!o->mjd || !o->v || !o->w || !o->filter) return ast_set_error(AST_E_INVALID, "ast_prepare: NULL array");
    if (!(m->flags & AST_INTERP) && (!o->e_unit || !o->s_unit))
        return ast_set_error(AST_E_INVALID, "ast_prepare: E/S unit vectors needed without AST_INTERP");
    for (int i = 0; i < o->n_data; i++) {
        if (o->filter[i] < 0 || o->filter[i] >= o->n_filters)
            return ast_set_error(AST_E_INVALID, "ast_prepare: observation %d has filter %d", i, o->filter[i]);
        if (i > 0 && !(o->mjd[i] > o->mjd[i - 1]))
            return ast_set_error(AST_E_INVALID, "ast_prepare: times must increase strictly (observation %d)", i);
    }
    if ((m->flags & AST_NUDGE) && (o->n_minima < 1 || o->n_minima > AST_NOBS_MAX))
        return ast_set_error(AST_E_INVALID, "ast_prepare: NUDGE needs 1..%d observed minima", AST_NOBS_MAX);
    if (!(m->time_step > 0.0)) return ast_set_error(AST_E_INVALID, "ast_prepare: time_step must be > 0");
    return AST_OK;
}

extern "C" int ast_prepare(const ast_model* model, const ast_obs_set* obs, int32_t device, ast_ctx** out)
{
    if (!model || !out) return ast_set_error(AST_E_INVALID, "ast_prepare: NULL argument");
    *out = nullptr;
    int rc = validate_obs(model, obs);
    if (rc) return rc;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return ast_set_error(AST_E_NODEVICE, "ast_prepare: no CUDA device");
    }
    if ((rc = set_device(device))) return rc;
    ast_ctx* c = new ast_ctx();
    AST_CUDA(cudaGetDevice(&c->device));
    AST_CUDA(cudaDeviceGetAttribute(&c->sm_count, cudaDevAttrMultiProcessorCount, c->device));
    int optin = 0;
    AST_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, c->device));
    c->smem_optin = (size_t)optin;
    AST_CUDA(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
    AST_CUDA(cudaEventCreate(&c->ev0));
    AST_CUDA(cudaEventCreate(&c->ev1));
    c->model = *model;
    if ((rc = build_dev_model(model, obs, &c->dm))) { ast_destroy(c); return rc; }
    c->n_data = obs->n_data;
    c->n_filters = obs->n_filters;
    const int64_t n = obs->n_data;
    c->layout = ObsLayout::make(n);
    std::vector<unsigned char> img;
    obs_image(model, obs, c->layout, img);
    if (cudaMalloc(&c->d_obs, (size_t)c->layout.bytes) != cudaSuccess) {
        cudaGetLastError();
        ast_destroy(c);
        return ast_set_error(AST_E_NOMEM, "ast_prepare: cudaMalloc(%lld) failed", (long long)c->layout.bytes);
    }
    AST_CUDA(cudaMemcpyAsync(c->d_obs, img.data(), (size_t)c->layout.bytes, cudaMemcpyHostToDevice, c->stream));
    if ((rc = launch_prep(c->dm, (char*)c->d_obs, c->layout, n, c->stream))) { ast_destroy(c); return rc; }
    AST_CUDA(cudaStreamSynchronize(c->stream));
    *out = c;
    return AST_OK;
}

extern "C" int ast_set_tables(ast_ctx* c, const ast_model* model)
{
    if (!c || !model) return ast_set_error(AST_E_INVALID, "ast_set_tables: NULL argument");
    if (model->flags != c->model.flags || model->n_params != c->model.n_params)
        return ast_set_error(AST_E_INVALID, "ast_set_tables: variant or parameter count differs from ast_prepare");
    DevModel dm;
    int rc = build_dev_model(model, nullptr, &dm);
    if (rc) return rc;
    dm.n_filters = c->dm.n_filters;
    dm.n_data = c->dm.n_data;
    dm.n_min = c->dm.n_min;
    memcpy(dm.t_min, c->dm.t_min, sizeof(dm.t_min));
    memcpy(dm.v_min, c->dm.v_min, sizeof(dm.v_min));
    memcpy(dm.eph_e, c->dm.eph_e, sizeof(dm.eph_e));
    memcpy(dm.eph_s, c->dm.eph_s, sizeof(dm.eph_s));
    memcpy(dm.eph_mjd0, c->dm.eph_mjd0, sizeof(dm.eph_mjd0));
    c->dm = dm;
    c->model = *model;
    return AST_OK;
}

extern "C" void ast_fit_free(ast_ctx* c);

extern "C" void ast_destroy(ast_ctx* c)
{
    if (!c) return;
    ast_fit_free(c);
    if (c->d_obs) cudaFree(c->d_obs);
    if (c->d_params) cudaFree(c->d_params);
    if (c->d_chi2) cudaFree(c->d_chi2);
    if (c->d_dv) cudaFree(c->d_dv);
    if (c->ev0) cudaEventDestroy(c->ev0);
    if (c->ev1) cudaEventDestroy(c->ev1);
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
}

extern "C" void* ast_stream(ast_ctx* c) { return c ? (void*)c->stream : nullptr; }

template <class CF, int PREC>
static int launch_eval(ast_ctx* c, const DevModel& dm, const double* d_params, int64_t n, double* d_chi2, double* d_dv,
                       cudaStream_t s, unsigned long long* d_err)
{
    auto kern = eval_kernel<CF, PREC>;
    size_t smem = 0;
    int rc = obs_smem_for(kern, (size_t)c->layout.bytes, c->smem_optin, &smem);
    if (rc) return rc;
    const int tpb = 128;
    int per_sm = 1;
    AST_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, tpb, smem));
    if (per_sm < 1) per_sm = 1;
    int64_t blocks = (n + tpb - 1) / tpb;
    const int64_t cap = (int64_t)c->sm_count * per_sm;
    if (blocks > cap) blocks = cap;
    if (blocks < 1) blocks = 1;
    kern<<<(unsigned)blocks, tpb, smem, s>>>(dm, c->d_obs, c->layout, smem ? 1 : 0, d_params, n, d_chi2, d_dv, d_err);
    AST_CUDA(cudaGetLastError());
    return AST_OK;
}

static int eval_dispatch(ast_ctx* c, int32_t precision, const double* d_params, int64_t n, double* d_chi2,
                         double* d_dv, cudaStream_t s)
{
    if (precision != AST_PREC_FP64 && precision != AST_PREC_MIXED && precision != AST_PREC_MIXED_RHS32)
        return ast_set_error(AST_E_INVALID, "precision must be AST_PREC_FP64, AST_PREC_MIXED or AST_PREC_MIXED_RHS32");
    const bool acc = (c->model.flags & AST_ACC) != 0;
    const DevModel& dm = c->dm;
    if (precision == AST_PREC_FP64)
        return acc ? launch_eval<double, AST_PREC_FP64>(c, dm, d_params, n, d_chi2, d_dv, s, nullptr)
                   : launch_eval<float, AST_PREC_FP64>(c, dm, d_params, n, d_chi2, d_dv, s, nullptr);
    if (precision == AST_PREC_MIXED_RHS32)
        return acc ? launch_eval<double, AST_PREC_MIXED_RHS32>(c, dm, d_params, n, d_chi2, d_dv, s, nullptr)
                   : launch_eval<float, AST_PREC_MIXED_RHS32>(c, dm, d_params, n, d_chi2, d_dv, s, nullptr);
    return acc ? launch_eval<double, AST_PREC_MIXED>(c, dm, d_params, n, d_chi2, d_dv, s, nullptr)
               : launch_eval<float, AST_PREC_MIXED>(c, dm, d_params, n, d_chi2, d_dv, s, nullptr);
}

extern "C" int ast_eval_batch_device(ast_ctx* c, int32_t precision, const double* d_params, int64_t n,
                                     double* d_chi2, double* d_delta_v, void* stream)
{
    if (!c || !d_params || !d_chi2 || n < 0) return ast_set_error(AST_E_INVALID, "ast_eval_batch_device: bad argument");
    if (n == 0) return AST_OK;
    int rc = set_device(c->device);
    if (rc) return rc;
    return eval_dispatch(c, precision, d_params, n, d_chi2, d_delta_v, (cudaStream_t)stream);
}

extern "C" int ast_eval_batch(ast_ctx* c, int32_t precision, const double* params, int64_t n, double* chi2,
                              double* delta_v)
{
    if (!c || !params || !chi2 || n < 0) return ast_set_error(AST_E_INVALID, "ast_eval_batch: bad argument");
    if (n == 0) return AST_OK;
    int rc = set_device(c->device);
    if (rc) return rc;
    const int N = c->model.n_params, NF = c->n_filters;
    if (n > c->eval_cap) {
        if (c->d_params) cudaFree(c->d_params);
        if (c->d_chi2) cudaFree(c->d_chi2);
        if (c->d_dv) cudaFree(c->d_dv);
        c->d_params = c->d_chi2 = c->d_dv = nullptr;
        c->eval_cap = 0;
        if (cudaMalloc(&c->d_params, sizeof(double) * n * N) != cudaSuccess ||
            cudaMalloc(&c->d_chi2, sizeof(double) * n) != cudaSuccess ||
            cudaMalloc(&c->d_dv, sizeof(double) * n * NF) != cudaSuccess) {
            cudaGetLastError();
            return ast_set_error(AST_E_NOMEM, "ast_eval_batch: cudaMalloc for %lld vectors failed", (long long)n);
        }
        c->eval_cap = n;
    }
    AST_CUDA(cudaMemcpyAsync(c->d_params, params, sizeof(double) * n * N, cudaMemcpyHostToDevice, c->stream));
    if ((rc = eval_dispatch(c, precision, c->d_params, n, c->d_chi2, c->d_dv, c->stream))) return rc;
    AST_CUDA(cudaMemcpyAsync(chi2, c->d_chi2, sizeof(double) * n, cudaMemcpyDeviceToHost, c->stream));
    if (delta_v)
        AST_CUDA(cudaMemcpyAsync(delta_v, c->d_dv, sizeof(double) * n * NF, cudaMemcpyDeviceToHost, c->stream));
    AST_CUDA(cudaStreamSynchronize(c->stream));
    return AST_OK;
}

extern "C" int ast_model_curve(ast_ctx* c, const double* params, double* vmod)
{
    if (!c || !params || !vmod) return ast_set_error(AST_E_INVALID, "ast_model_curve: NULL argument");
    int rc = set_device(c->device);
    if (rc) return rc;
    const int N = c->model.n_params;
    double *dp = nullptr, *dv = nullptr;
    if (cudaMalloc(&dp, sizeof(double) * N) != cudaSuccess || cudaMalloc(&dv, sizeof(double) * c->n_data) != cudaSuccess) {
        cudaGetLastError();
        if (dp) cudaFree(dp);
        return ast_set_error(AST_E_NOMEM, "ast_model_curve: cudaMalloc failed");
    }
    AST_CUDA(cudaMemcpyAsync(dp, params, sizeof(double) * N, cudaMemcpyHostToDevice, c->stream));
    model_curve_kernel<<<1, 32, 0, c->stream>>>(c->dm, c->d_obs, c->layout, dp, dv);
    AST_CUDA(cudaGetLastError());
    AST_CUDA(cudaMemcpyAsync(vmod, dv, sizeof(double) * c->n_data, cudaMemcpyDeviceToHost, c->stream));
    AST_CUDA(cudaStreamSynchronize(c->stream));
    cudaFree(dp);
    cudaFree(dv);
    return AST_OK;
}

// The model at n other times: magnitudes (vmod) and / or the renderer's geometry (geo).
static int curve_at(ast_ctx* c, const double* params, int32_t n, const double* t, const double* e_unit,
                    const double* s_unit, double* vmod, double* geo)
{
    if (!c || !params || !t || (!vmod && !geo) || n < 2) return ast_set_error(AST_E_INVALID, "ast_model_curve_at: bad argument");
    const bool interp = (c->model.flags & AST_INTERP) != 0;
    if (!interp && (!e_unit || !s_unit)) return ast_set_error(AST_E_INVALID, "ast_model_curve_at: E and S needed");
    for (int32_t i = 1; i < n; i++)
        if (!(t[i] > t[i - 1])) return ast_set_error(AST_E_INVALID, "ast_model_curve_at: times must increase");
    int rc = set_device(c->device);
    if (rc) return rc;
    // A block of n points with the context's model: magnitudes are not used, one filter.
    std::vector<float> v((size_t)n, 0.0f), w((size_t)n, 1.0f);
    std::vector<int32_t> f((size_t)n, 0);
    ast_obs_set o;
    memset(&o, 0, sizeof(o));
    o.n_data = n;
    o.n_filters = 1;
    o.mjd = t;
    o.v = v.data();
    o.w = w.data();
    o.filter = f.data();
    o.e_unit = e_unit;
    o.s_unit = s_unit;
    DevModel dm = c->dm;
    dm.n_data = n;
    dm.n_filters = 1;
    dm.flags &= ~AST_NUDGE;
    const ObsLayout L = ObsLayout::make(n);
    std::vector<unsigned char> img;
    obs_image(&c->model, &o, L, img);
    // Device scratch for this call, freed on every return.
    struct Scratch {
        void* blk = nullptr;
        double* p = nullptr;
        double* v = nullptr;
        double* g = nullptr;
        ~Scratch() { cudaFree(blk); cudaFree(p); cudaFree(v); cudaFree(g); }
    } d;
    if (cudaMalloc(&d.blk, (size_t)L.bytes) != cudaSuccess || cudaMalloc(&d.p, sizeof(double) * AST_MAX_PARAMS) != cudaSuccess ||
        cudaMalloc(&d.v, sizeof(double) * n) != cudaSuccess ||
        (geo && cudaMalloc(&d.g, sizeof(double) * kAstGeo * n) != cudaSuccess)) {
        cudaGetLastError();
        return ast_set_error(AST_E_NOMEM, "ast_model_curve_at: cudaMalloc failed");
    }
    AST_CUDA(cudaMemcpyAsync(d.blk, img.data(), img.size(), cudaMemcpyHostToDevice, c->stream));
    AST_CUDA(cudaMemcpyAsync(d.p, params, sizeof(double) * c->model.n_params, cudaMemcpyHostToDevice, c->stream));
    if ((rc = launch_prep(dm, (char*)d.blk, L, n, c->stream))) return rc;
    model_curve_kernel<<<1, 32, 0, c->stream>>>(dm, d.blk, L, d.p, d.v, d.g);
    AST_CUDA(cudaGetLastError());
    if (vmod) AST_CUDA(cudaMemcpyAsync(vmod, d.v, sizeof(double) * n, cudaMemcpyDeviceToHost, c->stream));
    if (geo) AST_CUDA(cudaMemcpyAsync(geo, d.g, sizeof(double) * kAstGeo * n, cudaMemcpyDeviceToHost, c->stream));
    AST_CUDA(cudaStreamSynchronize(c->stream));
    return AST_OK;
}

extern "C" int ast_model_curve_at(ast_ctx* c, const double* params, int32_t n, const double* t,
                                  const double* e_unit, const double* s_unit, double* vmod)
{
    if (!vmod) return ast_set_error(AST_E_INVALID, "ast_model_curve_at: NULL vmod");
    return curve_at(c, params, n, t, e_unit, s_unit, vmod, nullptr);
}

extern "C" int ast_model_geometry(ast_ctx* c, const double* params, int32_t n, const double* t,
                                  const double* e_unit, const double* s_unit, double* geo)
{
    if (!geo) return ast_set_error(AST_E_INVALID, "ast_model_geometry: NULL geo");
    return curve_at(c, params, n, t, e_unit, s_unit, nullptr, geo);
}

extern "C" int ast_model_angles(ast_ctx* c, int32_t precision, const double* params, double* angles)
{
    if (!c || !params || !angles) return ast_set_error(AST_E_INVALID, "ast_model_angles: NULL argument");
    if (precision != AST_PREC_FP64 && precision != AST_PREC_MIXED && precision != AST_PREC_MIXED_RHS32)
        return ast_set_error(AST_E_INVALID, "ast_model_angles: bad precision");
    int rc = set_device(c->device);
    if (rc) return rc;
    double *dp = nullptr, *da = nullptr;
    if (cudaMalloc(&dp, sizeof(double) * AST_MAX_PARAMS) != cudaSuccess ||
        cudaMalloc(&da, sizeof(double) * 3 * c->n_data) != cudaSuccess) {
        cudaGetLastError();
        cudaFree(dp);
        return ast_set_error(AST_E_NOMEM, "ast_model_angles: cudaMalloc failed");
    }
    AST_CUDA(cudaMemcpyAsync(dp, params, sizeof(double) * c->model.n_params, cudaMemcpyHostToDevice, c->stream));
    if (precision == AST_PREC_FP64)
        model_angles_kernel<AST_PREC_FP64><<<1, 32, 0, c->stream>>>(c->dm, c->d_obs, c->layout, dp, da);
    else if (precision == AST_PREC_MIXED_RHS32)
        model_angles_kernel<AST_PREC_MIXED_RHS32><<<1, 32, 0, c->stream>>>(c->dm, c->d_obs, c->layout, dp, da);
    else
        model_angles_kernel<AST_PREC_MIXED><<<1, 32, 0, c->stream>>>(c->dm, c->d_obs, c->layout, dp, da);
    AST_CUDA(cudaGetLastError());
    AST_CUDA(cudaMemcpyAsync(angles, da, sizeof(double) * 3 * c->n_data, cudaMemcpyDeviceToHost, c->stream));
    AST_CUDA(cudaStreamSynchronize(c->stream));
    cudaFree(dp);
    cudaFree(da);
    return AST_OK;
}

extern "C" int ast_x2params(const ast_model* m, int32_t reopt, const double* x, double* params)
{
    if (!m || !x || !params) return ast_set_error(AST_E_INVALID, "ast_x2params: NULL argument");
    DevModel dm;
    int rc = build_dev_model(m, nullptr, &dm);
    if (rc) return rc;
    if (m->flags & AST_ACC) return x2params<double>(dm, reopt, x, params);
    float xf[AST_MAX_PARAMS];
    for (int i = 0; i < m->n_params; i++) xf[i] = (float)x[i];
    return x2params<float>(dm, reopt, xf, params);
}

extern "C" int ast_params2x(const ast_model* m, const double* params, double* x)
{
    if (!m || !x || !params) return ast_set_error(AST_E_INVALID, "ast_params2x: NULL argument");
    DevModel dm;
    int rc = build_dev_model(m, nullptr, &dm);
    if (rc) return rc;
    if (m->flags & AST_ACC) {
        params2x<double>(dm, params, x);
        return AST_OK;
    }
    float xf[AST_MAX_PARAMS];
    params2x<float>(dm, params, xf);
    for (int i = 0; i < m->n_params; i++) x[i] = xf[i];
    return AST_OK;
}

extern "C" int ast_probe_peak(int32_t device, int32_t kind, double* gflops)
{
    if (!gflops) return ast_set_error(AST_E_INVALID, "ast_probe_peak: NULL output");
    int rc = set_device(device);
    if (rc) return rc;
    int dev = 0, sms = 0;
    AST_CUDA(cudaGetDevice(&dev));
    AST_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const int blocks = sms * 8, tpb = 256;
    void* out = nullptr;
    AST_CUDA(cudaMalloc(&out, (size_t)blocks * tpb * 8));
    cudaEvent_t e0, e1;
    AST_CUDA(cudaEventCreate(&e0));
    AST_CUDA(cudaEventCreate(&e1));
    const int iters = kind == 0 ? 4000 : 100000;
    float best = 1e30f;
    for (int rep = 0; rep < 3; rep++) {
        AST_CUDA(cudaEventRecord(e0));
        if (kind == 0)
            fma_probe_kernel<double><<<blocks, tpb>>>((double*)out, iters, 0.999999, 1e-7);
        else
            fma_probe_kernel<float><<<blocks, tpb>>>((float*)out, iters, 0.999999f, 1e-7f);
        AST_CUDA(cudaEventRecord(e1));
        AST_CUDA(cudaEventSynchronize(e1));
        float ms = 0;
        AST_CUDA(cudaEventElapsedTime(&ms, e0, e1));
        if (ms < best) best = ms;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    *gflops = 2.0 * 8.0 * iters * (double)blocks * tpb / (best * 1e-3) / 1e9;
    return AST_OK;
}
