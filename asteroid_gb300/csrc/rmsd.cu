// rmsd.cu -- unconstrained RMSD confidence intervals of a model (chi2_gpu_rms, cuda.c:2148-2389,
// driven by asteroid.c:690-725 of the reference).
//
// The reference runs one random stream per thread of chi2_gpu_rms<<<N_BLOCKS, BSIZE>>>: each
// stream draws Nstages models around the -m model, evaluates their RMSD and keeps, per
// parameter, the range over the models whose RMSD is below f1; a serial reduction per block
// and a host loop over blocks give the interval.  Here:
//
//   * rmsd_setup_kernel evaluates f0 = RMSD(-m model), f1 and x0 = params2x(-m model) once
//     (the reference repeats them in every thread);
//   * rmsd_kernel is persistent: each thread takes streams s, s + G, ... and, within a stream,
//     draws until x2params accepts a model (a rejected draw costs no evaluation), so the lanes
//     of a warp evaluate together instead of idling behind a rejected lane; the evaluation is
//     the fit's (FP64 or mixed), with the observations staged in shared memory by one bulk copy;
//   * a stream's draws are Philox4x32-10 keyed by (seed, call, stream, draw), so the result does
//     not depend on the launch geometry;
//   * ranges live per thread in HBM ([param][thread], coalesced) and touched only by good
//     models; rmsd_reduce_kernel takes the min / max over threads, one CTA per parameter.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>
#include <string.h>
#include <algorithm>
#include <vector>

#include "asteroid_gb300.h"
#include "engine.cuh"
#include "mixed.cuh"
#include "model.cuh"
#include "philox.cuh"
#include "simplex.cuh"
#include "staging.cuh"


namespace ast {
namespace {

constexpr double kPi = 3.141592653589793238;  // PI (asteroid.h:16)
constexpr double kSmall = 1e-8;                // SMALL (cuda.c:2258)
constexpr uint32_t kRmsdDomain = 0x80000000u;  // Philox counter word 1 of RMSD draws (fit stages are below it)

template <class CF>
struct RmsdView {
    int64_t n_streams;
    int32_t samples;
    int32_t reopt;
    float dx;
    int32_t spherical;
    uint64_t seed;
    uint32_t call;
    const CF* x0;             // [N] params2x of the -m model
    const double* p0;         // [N] the -m model
    const CF* f01;            // [2] f0, f1
    double* pmin;             // [N][threads]
    double* pmax;
    int64_t threads;
    unsigned long long* ctr;  // [0] n_tot, [1] n_bad, [4] staging error
    double* trace_x;          // optional [n_streams*samples][N]
    double* trace_f;          // optional [n_streams*samples]
};

// f0 = RMSD of the -m model, f1 = f0 + f0/sqrt(N_data - N - Nf) (cuda.c:2224-2227), and x0.
template <class CF, int PREC>
__global__ void rmsd_setup_kernel(DevModel M, const void* g_obs, ObsLayout L, const double* p0, CF* x0, CF* f01)
{
    __shared__ float4 trig[PREC == AST_PREC_MIXED ? kTrigTable : 1];
    if (PREC == AST_PREC_MIXED) {
        trig_table_fill(trig);
        __syncthreads();
    }
    if (threadIdx.x != 0) return;
    const ObsView o = L.view(g_obs, M.n_data);
    double p[AST_MAX_PARAMS];
    for (int i = 0; i < M.n_params; i++) p[i] = p0[i];
    params2x<CF>(M, p, x0);
    CF dv[AST_MAX_FILTERS];
    const CF f0 = eval_point<CF, PREC>(M, o, p, dv, trig);
    f01[0] = f0;
    f01[1] = f0 + f0 / sqrt((CF)(M.n_data - M.n_params - M.n_filters));
}

// Draw k of stream st: x = x0 + dx * N(0,1) per parameter, clamped SMALL inside hard limits,
// with psi_0's periodicity following the drawn Es (cuda.c:2260-2290).
template <class CF>
__device__ __forceinline__ void rmsd_draw(const DevModel& M, const RmsdView<CF>& V, int64_t st, int k, CF* x1)
{
    const int N = M.n_params;
    const int nq = (N + 3) >> 2;
    int LAM = 0;
    for (int q = 0; q < nq; q++) {
        float z[4];
        normal4(V.seed, (uint64_t)st, kRmsdDomain | V.call, (uint32_t)k * (uint32_t)nq + (uint32_t)q, z);
#pragma unroll
        for (int r = 0; r < 4; r++) {
            const int i = 4 * q + r;
            if (i >= N) break;
            CF xx = V.x0[i] + (CF)(V.dx * z[r]);
            const int per = M.periodic[i];
            if (xx < kSmall && hard_side(per, LAM, true))
                xx = (CF)kSmall;
            else if (xx > 1.0 - kSmall && hard_side(per, LAM, false))
                xx = (CF)(1.0 - kSmall);
            x1[i] = xx;
            if (M.ptype[i] == M.t.Es) LAM = x1[i] >= 0.5;
        }
    }
}

// The reference's bookkeeping of a good model before its range update (cuda.c:2302-2332).
__device__ __forceinline__ void rmsd_good_params(const DevModel& M, bool spherical, double phi_M0, double phi_00,
                                                 double phiK0, double* p)
{
    const int iM = M.idx[M.t.phi_M], i0 = M.idx[M.t.phi_0];
    // As the reference writes it: the replacement value is the -m model's angle -/+ 2 pi, and
    // the second test then sees that value.
    if (p[iM] > phi_M0 + kPi) p[iM] = phi_M0 - 2 * kPi;
    if (p[iM] < phi_M0 - kPi) p[iM] = phi_M0 + 2 * kPi;
    if (p[i0] > phi_00 + kPi) p[i0] = phi_00 - 2 * kPi;
    if (p[i0] < phi_00 - kPi) p[i0] = phi_00 + 2 * kPi;
    if (spherical) {
        const int iTi = M.idx[M.t.Ti], iTs = M.idx[M.t.Ts], iTl = M.idx[M.t.Tl];
        const double b = p[M.idx[M.t.b_tumb]], c = p[M.idx[M.t.c_tumb]];
        const double Is = (1.0 + b * b) / (b * b + c * c);
        const double Ii = (1.0 + c * c) / (b * b + c * c);
        const double Ki = Ii * p[iTi], Ks = Is * p[iTs], Kl = p[iTl];
        p[iTi] = sqrt(Ki * Ki + Ks * Ks + Kl * Kl);
        p[iTs] = acos(Kl / p[iTi]);
        double phi = atan2(Ks, Ki);
        if (phi > phiK0 + kPi) phi = phi - 2 * kPi;
        if (phi < phiK0 - kPi) phi = phi + 2 * kPi;
        p[iTl] = phi;
    }
}

__device__ __forceinline__ double torque_phi(const DevModel& M, const double* p)
{
    const double b = p[M.idx[M.t.b_tumb]], c = p[M.idx[M.t.c_tumb]];
    const double Is = (1.0 + b * b) / (b * b + c * c);
    const double Ii = (1.0 + c * c) / (b * b + c * c);
    return atan2(Is * p[M.idx[M.t.Ts]], Ii * p[M.idx[M.t.Ti]]);
}

template <class CF, int PREC>
__global__ void __launch_bounds__(KernShape<PREC>::tpb, KernShape<PREC>::min_ctas) rmsd_kernel(DevModel M, const void* g_obs, ObsLayout L, int use_smem,
                                                           RmsdView<CF> V)
{
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ uint64_t bar;
    __shared__ float4 trig[PREC == AST_PREC_MIXED ? kTrigTable : 1];
    if (PREC == AST_PREC_MIXED) {
        trig_table_fill(trig);
        __syncthreads();
    }
    const bool staged = use_smem ? bulk_stage(smem, g_obs, (uint32_t)L.bytes, &bar, &V.ctr[4]) : false;
    const ObsView o = L.view(staged ? (const void*)smem : g_obs, M.n_data);
    const int N = M.n_params;
    const int64_t tid = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int64_t G = (int64_t)gridDim.x * blockDim.x;
    const CF f1 = V.f01[1];
    const bool spherical = V.spherical && (M.flags & AST_TORQUE);
    const double phi_M0 = V.p0[M.idx[M.t.phi_M]], phi_00 = V.p0[M.idx[M.t.phi_0]];
    const double phiK0 = spherical ? torque_phi(M, V.p0) : 0.0;
    unsigned long long n_tot = 0, n_bad = 0;
    for (int64_t st = tid; st < V.n_streams; st += G) {
        int k = 0;
        while (true) {
            CF x1[AST_MAX_PARAMS];
            double p[AST_MAX_PARAMS];
            bool ok = false;
            for (; k < V.samples && !ok; k++) {
                rmsd_draw<CF>(M, V, st, k, x1);
                ok = x2params<CF>(M, V.reopt, x1, p) == 0;
                if (V.trace_x) {
                    const int64_t row = st * V.samples + k;
                    for (int i = 0; i < N; i++) V.trace_x[row * N + i] = (double)x1[i];
                    if (!ok) V.trace_f[row] = __longlong_as_double(0x7ff8000000000000ll);
                }
            }
            if (!ok) break;
            CF dv[AST_MAX_FILTERS];
            const CF f = eval_point<CF, PREC>(M, o, p, dv, trig);
            if (V.trace_f) V.trace_f[st * V.samples + (k - 1)] = (double)f;
            n_tot++;
            if (f < f1) {
                rmsd_good_params(M, spherical, phi_M0, phi_00, phiK0, p);
                for (int i = 0; i < N; i++) {
                    double* a = &V.pmin[(int64_t)i * V.threads + tid];
                    double* b = &V.pmax[(int64_t)i * V.threads + tid];
                    if (p[i] < *a) *a = p[i];
                    if (p[i] > *b) *b = p[i];
                }
            } else {
                n_bad++;
            }
        }
    }
    if (n_tot) atomicAdd(&V.ctr[0], n_tot);
    if (n_bad) atomicAdd(&V.ctr[1], n_bad);
    bulk_drain(&bar, staged || !use_smem);
}

__global__ void rmsd_init_kernel(double* pmin, double* pmax, int64_t n)
{
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
        pmin[k] = 1e30;
        pmax[k] = -1e30;
    }
}

// out[i] = min / max over threads of parameter i: one CTA per parameter.
__global__ void __launch_bounds__(256) rmsd_reduce_kernel(const double* pmin, const double* pmax, int64_t threads,
                                                          double* out_min, double* out_max)
{
    __shared__ double smin[8], smax[8];
    const int i = blockIdx.x;
    double a = 1e30, b = -1e30;
    for (int64_t t = threadIdx.x; t < threads; t += blockDim.x) {
        a = fmin(a, pmin[(int64_t)i * threads + t]);
        b = fmax(b, pmax[(int64_t)i * threads + t]);
    }
    for (int off = 16; off; off >>= 1) {
        a = fmin(a, __shfl_xor_sync(0xffffffffu, a, off));
        b = fmax(b, __shfl_xor_sync(0xffffffffu, b, off));
    }
    if ((threadIdx.x & 31) == 0) {
        smin[threadIdx.x >> 5] = a;
        smax[threadIdx.x >> 5] = b;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < (int)(blockDim.x >> 5); w++) {
            a = fmin(a, smin[w]);
            b = fmax(b, smax[w]);
        }
        out_min[i] = a;
        out_max[i] = b;
    }
}

// Device buffers of one call, freed on every return.
struct RmsdScratch {
    void* x0 = nullptr;
    void* f01 = nullptr;
    double* p0 = nullptr;
    double* pmin = nullptr;
    double* pmax = nullptr;
    double* red = nullptr;
    unsigned long long* ctr = nullptr;
    double* tx = nullptr;
    double* tf = nullptr;
    ~RmsdScratch()
    {
        cudaFree(x0); cudaFree(f01); cudaFree(p0); cudaFree(pmin); cudaFree(pmax); cudaFree(red); cudaFree(ctr);
        cudaFree(tx); cudaFree(tf);
    }
};

template <class CF, int PREC>
int rmsd_run(ast_ctx* c, const ast_rmsd_cfg* cfg, ast_rmsd_out* out)
{
    const int N = c->model.n_params;
    auto kern = rmsd_kernel<CF, PREC>;
    constexpr int kRmsdTpb = KernShape<PREC>::tpb;
    size_t smem_obs = 0;
    if (int rc = obs_smem_for(kern, (size_t)c->layout.bytes, c->smem_optin, &smem_obs)) return rc;
    int occ_s = 0, occ_g = 0;
    AST_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_g, kern, kRmsdTpb, 0));
    if (smem_obs) AST_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_s, kern, kRmsdTpb, smem_obs));
    const bool stage = smem_obs != 0 && occ_s >= occ_g;
    const int occ = stage ? occ_s : occ_g;
    if (occ < 1) return ast_set_error(AST_E_TOO_LARGE, "ast_rmsd: kernel does not fit on an SM");
    int64_t ctas = std::min<int64_t>((int64_t)c->sm_count * occ, (cfg->n_streams + kRmsdTpb - 1) / kRmsdTpb);
    ctas = std::max<int64_t>(ctas, 1);
    const int64_t threads = ctas * kRmsdTpb;
    const int64_t rows = cfg->n_streams * (int64_t)cfg->samples;
    const bool trace = cfg->trace_x && cfg->trace_f;
    RmsdScratch d;
    if (cudaMalloc(&d.x0, sizeof(double) * AST_MAX_PARAMS) != cudaSuccess || cudaMalloc(&d.f01, 16) != cudaSuccess ||
        cudaMalloc(&d.p0, sizeof(double) * AST_MAX_PARAMS) != cudaSuccess ||
        cudaMalloc(&d.pmin, sizeof(double) * N * threads) != cudaSuccess ||
        cudaMalloc(&d.pmax, sizeof(double) * N * threads) != cudaSuccess ||
        cudaMalloc(&d.red, sizeof(double) * 2 * AST_MAX_PARAMS) != cudaSuccess ||
        cudaMalloc(&d.ctr, 8 * sizeof(unsigned long long)) != cudaSuccess ||
        (trace && (cudaMalloc(&d.tx, sizeof(double) * rows * N) != cudaSuccess ||
                   cudaMalloc(&d.tf, sizeof(double) * rows) != cudaSuccess))) {
        cudaGetLastError();
        return ast_set_error(AST_E_NOMEM, "ast_rmsd: cudaMalloc failed");
    }
    cudaStream_t s = c->stream;
    AST_CUDA(cudaMemcpyAsync(d.p0, cfg->params0, sizeof(double) * N, cudaMemcpyHostToDevice, s));
    AST_CUDA(cudaMemsetAsync(d.ctr, 0, 8 * sizeof(unsigned long long), s));
    rmsd_setup_kernel<CF, PREC><<<1, 128, 0, s>>>(c->dm, c->d_obs, c->layout, d.p0, (CF*)d.x0, (CF*)d.f01);
    AST_CUDA(cudaGetLastError());
    rmsd_init_kernel<<<(unsigned)std::min<int64_t>((N * threads + 255) / 256, 4096), 256, 0, s>>>(d.pmin, d.pmax,
                                                                                                  N * threads);
    AST_CUDA(cudaGetLastError());
    RmsdView<CF> V;
    V.n_streams = cfg->n_streams;
    V.samples = cfg->samples;
    V.reopt = cfg->reopt ? 1 : 0;
    V.dx = (float)cfg->dx;
    V.spherical = cfg->spherical_k ? 1 : 0;
    V.seed = cfg->seed;
    V.call = cfg->call & 0x7fffffffu;
    V.x0 = (const CF*)d.x0;
    V.p0 = d.p0;
    V.f01 = (const CF*)d.f01;
    V.pmin = d.pmin;
    V.pmax = d.pmax;
    V.threads = threads;
    V.ctr = d.ctr;
    V.trace_x = trace ? d.tx : nullptr;
    V.trace_f = trace ? d.tf : nullptr;
    AST_CUDA(cudaEventRecord(c->ev0, s));
    kern<<<(unsigned)ctas, kRmsdTpb, stage ? smem_obs : 0, s>>>(c->dm, c->d_obs, c->layout, stage ? 1 : 0, V);
    AST_CUDA(cudaGetLastError());
    AST_CUDA(cudaEventRecord(c->ev1, s));
    rmsd_reduce_kernel<<<N, 256, 0, s>>>(d.pmin, d.pmax, threads, d.red, d.red + AST_MAX_PARAMS);
    AST_CUDA(cudaGetLastError());
    CF f01[2];
    unsigned long long ctr[8];
    double red[2 * AST_MAX_PARAMS];
    AST_CUDA(cudaMemcpyAsync(f01, d.f01, sizeof(f01), cudaMemcpyDeviceToHost, s));
    AST_CUDA(cudaMemcpyAsync(ctr, d.ctr, sizeof(ctr), cudaMemcpyDeviceToHost, s));
    AST_CUDA(cudaMemcpyAsync(red, d.red, sizeof(red), cudaMemcpyDeviceToHost, s));
    if (trace) {
        AST_CUDA(cudaMemcpyAsync(cfg->trace_x, d.tx, sizeof(double) * rows * N, cudaMemcpyDeviceToHost, s));
        AST_CUDA(cudaMemcpyAsync(cfg->trace_f, d.tf, sizeof(double) * rows, cudaMemcpyDeviceToHost, s));
    }
    AST_CUDA(cudaStreamSynchronize(s));
    if (ctr[4]) return ast_set_error(AST_E_TIMEOUT, "ast_rmsd: observation staging wait ran out");
    float ms = 0;
    AST_CUDA(cudaEventElapsedTime(&ms, c->ev0, c->ev1));
    memset(out, 0, sizeof(*out));
    out->f0 = (double)f01[0];
    out->f1 = (double)f01[1];
    out->n_tot = (int64_t)ctr[0];
    out->n_bad = (int64_t)ctr[1];
    // The reference reduces the ranges in float (cuda.c:2356-2376, asteroid.c:703-717).
    for (int i = 0; i < AST_MAX_PARAMS; i++) {
        out->par_min[i] = i < N ? (double)(float)red[i] : 0.0;
        out->par_max[i] = i < N ? (double)(float)red[AST_MAX_PARAMS + i] : 0.0;
    }
    out->kernel_ms = ms;
    return AST_OK;
}

}  // namespace
}  // namespace ast

using namespace ast;

extern "C" int ast_rmsd(ast_ctx* c, const ast_rmsd_cfg* cfg, ast_rmsd_out* out)
{
    if (!c || !cfg || !out || !cfg->params0) return ast_set_error(AST_E_INVALID, "ast_rmsd: NULL argument");
    if (!(c->model.flags & AST_RMSD))
        return ast_set_error(AST_E_INVALID, "ast_rmsd: the model must carry AST_RMSD (chi2_gpu_rms exists only under -DRMSD)");
    if (cfg->n_streams <= 0 || cfg->samples <= 0) return ast_set_error(AST_E_INVALID, "ast_rmsd: n_streams and samples must be positive");
    if (cfg->precision != AST_PREC_FP64 && cfg->precision != AST_PREC_MIXED)
        return ast_set_error(AST_E_INVALID, "ast_rmsd: bad precision");
    if (!(cfg->dx >= 0) || !(cfg->dx < 1e30)) return ast_set_error(AST_E_INVALID, "ast_rmsd: dx must be finite and >= 0");
    if ((cfg->trace_x != nullptr) != (cfg->trace_f != nullptr))
        return ast_set_error(AST_E_INVALID, "ast_rmsd: trace_x and trace_f go together");
    if (cfg->spherical_k && !(c->model.flags & AST_TORQUE))
        return ast_set_error(AST_E_INVALID, "ast_rmsd: spherical_k needs a TORQUE model");
    if ((int64_t)cfg->samples * (int64_t)((c->model.n_params + 3) / 4) >= (int64_t)1 << 32)
        return ast_set_error(AST_E_TOO_LARGE, "ast_rmsd: too many samples per stream");
    int rc = set_device(c->device);
    if (rc) return rc;
    const bool acc = (c->model.flags & AST_ACC) != 0;
    if (acc)
        return cfg->precision == AST_PREC_FP64 ? rmsd_run<double, AST_PREC_FP64>(c, cfg, out)
                                               : rmsd_run<double, AST_PREC_MIXED>(c, cfg, out);
    return cfg->precision == AST_PREC_FP64 ? rmsd_run<float, AST_PREC_FP64>(c, cfg, out)
                                           : rmsd_run<float, AST_PREC_MIXED>(c, cfg, out);
}
