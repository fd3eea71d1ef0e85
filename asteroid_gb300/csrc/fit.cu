// fit.cu -- the downhill-simplex / random-search driver as a persistent device loop.
//
// The reference runs one Nelder-Mead chain per thread of chi2_gpu<<<N_BLOCKS, BSIZE>>>
// (cuda.c:1326-1833), keeps each simplex in local memory (255 registers plus spills on
// sm_103a), and lets a thread whose chain converged idle until its block finishes.  Here:
//
//   * every thread is a persistent "slot" that pulls chains from a device-wide pool with an
//     atomic counter, so a chain that converges early is replaced at once;
//   * the simplex of each slot lives in HBM as structure-of-arrays indexed [k][slot], so a
//     warp's 32 slots touch 32 consecutive words (coalesced), and registers stay with chi^2;
//   * the chain is a state machine (INIT j, REFLECT, EXPAND, CONTRACT, SHRINK j) in which every
//     loop iteration performs exactly one chi^2 evaluation: all lanes of a warp evaluate
//     together, and the RK4 trip counts are the same for every lane (they depend on the
//     observation times only), so the hot loop does not diverge;
//   * a launch runs until every slot has spent its evaluation budget or the pool is empty and
//     saves its state, so a fit can be advanced in bounded steps (bench, serving);
//   * stages (-Nstages) are separate pools; between them group_best_kernel takes each group's
//     best chain (the reference's per-block argmin and hand-off, cuda.c:1769-1805).
// The chain semantics (random start, initial simplex, sort with ties to the last index,
// centroid over all N+1 vertices, reflect/expand/contract/shrink tests, failure rules,
// iteration cap) are those of cuda.c:1424-1742; the restatement in oracle/nm_oracle_body.h
// follows the same steps on the CPU.
#include <cuda_runtime.h>
#include <stdio.h>
#include <string.h>
#include <vector>

#include "asteroid_gb300.h"
#include "engine.cuh"
#include "mixed.cuh"
#include "model.cuh"
#include "philox.cuh"
#include "simplex.cuh"
#include "staging.cuh"

namespace ast {

// MINB: CTAs that must fit on one SM -- 1 (CTAs of up to 256) lets the compiler use up to 255
// registers per thread, 2 caps it at 128 (twice the warps per SM, some spilled registers), 3 (CTAs
// of up to 128) at 170: 12 warps per SM, the double-float path's best.
//
// Persistent slots: each slot pulls chains of the fit from an atomic pool and performs `budget`
// evaluations (or runs until the pool is empty).  Every loop iteration is exactly one chi^2
// evaluation per slot, so the lanes of a warp integrate in lockstep.
template <class CF, int PREC, int MINB>
__global__ void __launch_bounds__(MINB == 3 ? 128 : 256, MINB) fit_kernel(DevModel M, const void* g_obs, ObsLayout L, int use_smem,
                                                        FitView<CF> V, int64_t budget)
{
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ uint64_t bar;
    __shared__ float4 trig[PREC != AST_PREC_FP64 ? kTrigTable : 1];
    if (PREC != AST_PREC_FP64) {
        trig_table_fill(trig);
        __syncthreads();
    }
    const bool staged = use_smem ? bulk_stage(smem, g_obs, (uint32_t)L.bytes, &bar, &V.ctr[4], V.stage_wait) : false;
    const ObsView o = L.view(staged ? (const void*)smem : g_obs, M.n_data);
    const int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int NF = M.n_filters;
    const int64_t S = V.S;
    if (s < V.n_slots) {
        SlotState<CF> R;
        R.chain = V.chain[s];
        R.st = V.st[s];
        R.l = V.it[s];
        R.ev = V.ev[s];
        for (int m = 0; m < NF; m++) R.dvl[m] = (CF)V.dv[(int64_t)m * S + s];
        int64_t used = 0;
        unsigned long long n_ev = 0, n_fit = 0, n_done = 0;
        while (true) {
            if (R.chain < 0) {
                const unsigned long long c = atomicAdd(&V.ctr[0], 1ull);
                if (c >= (unsigned long long)V.n_chains) break;
                R.chain = (int64_t)c;
                start_chain<CF>(M, V, s, R.chain);
                R.st = PH_INIT;
                R.l = 0;
                R.ev = 0;
                for (int m = 0; m < NF; m++) R.dvl[m] = V.stage > 0 ? (CF)V.chain_dv[R.chain * NF + m] : (CF)0;
            }
            if (slot_iterate<CF, PREC>(M, o, V, s, R, trig, n_ev, n_fit)) {
                n_done++;
                R.chain = -1;
            }
            if (++used >= budget) break;
        }
        V.chain[s] = R.chain;
        V.st[s] = R.st;
        V.it[s] = R.l;
        V.ev[s] = R.ev;
        for (int m = 0; m < NF; m++) V.dv[(int64_t)m * S + s] = (double)R.dvl[m];
        if (n_done) atomicAdd(&V.ctr[1], n_done);
        if (n_ev) atomicAdd(&V.ctr[2], n_ev);
        if (n_fit) atomicAdd(&V.ctr[3], n_fit);
    }
    bulk_drain(&bar, staged || !use_smem);
}
// Per-group argmin over the chains' results (lowest chi^2, lowest chain on ties, as the serial
// loop of cuda.c:1770-1782) and the stage hand-off or the final output (cuda.c:1785-1823).
template <class CF>
__global__ void group_best_kernel(DevModel M, FitView<CF> V, double* out_f, double* out_p, double* out_dv,
                                  const void* g_obs, ObsLayout L, int fp64_result)
{
    const ObsView o = L.view(g_obs, M.n_data);
    group_best_body<CF>(M, V, blockIdx.x, out_f, out_p, out_dv, fp64_result ? &o : nullptr);
}

__global__ void reset_slots_kernel(int64_t* chain, int32_t* st, int32_t* it, int32_t* ev, double* dv, int64_t S, int NF)
{
    const int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (s >= S) return;
    chain[s] = -1;
    st[s] = 0;
    it[s] = 0;
    ev[s] = 0;
    for (int m = 0; m < NF; m++) dv[(int64_t)m * S + s] = 0.0;
}

}  // namespace ast

using namespace ast;

template <class CF>
static FitView<CF> make_view(ast_ctx* c)
{
    FitBuffers& b = c->fb;
    FitView<CF> V;
    V.x = (CF*)b.x; V.f = (CF*)b.f; V.ind = b.ind; V.x0 = (CF*)b.x0; V.xr = (CF*)b.xr; V.fr = (CF*)b.fr;
    V.st = b.st; V.it = b.it; V.ev = b.ev; V.chain = b.chain; V.dv = b.dv;
    V.chain_f = b.chain_f; V.chain_x = (CF*)b.chain_x; V.chain_dv = b.chain_dv; V.group_x = (CF*)b.group_x;
    V.ctr = b.ctr;
    V.S = b.slots_pad;
    V.n_slots = b.slots;
    V.n_chains = c->run.cfg.n_chains;
    V.group_size = c->run.cfg.group_size;
    V.stage = c->run.stage;
    V.reopt = c->run.reopt;
    V.last_stage = c->run.stage == c->run.cfg.n_stages - 1;
    V.seed = c->run.cfg.seed;
    V.evals_cap = c->run.cfg.evals_cap;
    V.steps_cap = c->run.cfg.steps_cap > 0 ? c->run.cfg.steps_cap : 5000;
    V.stage_wait = c->stage_wait;
    return V;
}

extern "C" void ast_fit_free(ast_ctx* c)
{
    if (c && c->fb.base) cudaFree(c->fb.base);
    if (c) c->fb = FitBuffers();
}

static int fit_alloc(ast_ctx* c, int64_t slots, int64_t chains, int64_t groups, int cf_bytes)
{
    const int N = c->model.n_params, NF = c->n_filters;
    FitBuffers& b = c->fb;
    const int64_t S = (slots + 31) / 32 * 32;
    if (b.base && b.slots_pad >= S && b.chains >= chains && b.groups >= groups && b.n_params == N &&
        b.n_filters == NF && b.cf_bytes == cf_bytes) {
        b.slots = slots;
        return AST_OK;
    }
    ast_fit_free(c);
    auto al = [](int64_t v) { return (v + 255) / 256 * 256; };
    int64_t o = 0;
    const int64_t o_x = o; o += al(S * (N + 1) * N * cf_bytes);
    const int64_t o_f = o; o += al(S * (N + 1) * cf_bytes);
    const int64_t o_ind = o; o += al(S * (N + 1));
    const int64_t o_x0 = o; o += al(S * N * cf_bytes);
    const int64_t o_xr = o; o += al(S * N * cf_bytes);
    const int64_t o_fr = o; o += al(S * cf_bytes);
    const int64_t o_st = o; o += al(S * 4);
    const int64_t o_it = o; o += al(S * 4);
    const int64_t o_ev = o; o += al(S * 4);
    const int64_t o_ch = o; o += al(S * 8);
    const int64_t o_dv = o; o += al(S * NF * 8);
    const int64_t o_cf = o; o += al(chains * 8);
    const int64_t o_cx = o; o += al(chains * N * cf_bytes);
    const int64_t o_cdv = o; o += al(chains * NF * 8);
    const int64_t o_gx = o; o += al(groups * N * cf_bytes);
    const int64_t o_of = o; o += al(groups * 8);
    const int64_t o_op = o; o += al(groups * N * 8);
    const int64_t o_odv = o; o += al(groups * NF * 8);
    const int64_t o_ctr = o; o += al(8 * 8);
    void* base = nullptr;
    if (cudaMalloc(&base, (size_t)o) != cudaSuccess) {
        cudaGetLastError();
        return ast_set_error(AST_E_NOMEM, "fit: cudaMalloc(%lld bytes) for %lld slots / %lld chains failed",
                             (long long)o, (long long)slots, (long long)chains);
    }
    char* p = (char*)base;
    b.base = base;
    b.bytes = (size_t)o;
    b.x = p + o_x; b.f = p + o_f; b.ind = (uint8_t*)(p + o_ind); b.x0 = p + o_x0; b.xr = p + o_xr; b.fr = p + o_fr;
    b.st = (int32_t*)(p + o_st); b.it = (int32_t*)(p + o_it); b.ev = (int32_t*)(p + o_ev);
    b.chain = (int64_t*)(p + o_ch); b.dv = (double*)(p + o_dv);
    b.chain_f = (double*)(p + o_cf); b.chain_x = p + o_cx; b.chain_dv = (double*)(p + o_cdv);
    b.group_x = p + o_gx; b.out_f = (double*)(p + o_of); b.out_p = (double*)(p + o_op); b.out_dv = (double*)(p + o_odv);
    b.ctr = (unsigned long long*)(p + o_ctr);
    b.slots = slots; b.slots_pad = S; b.chains = chains; b.groups = groups;
    b.n_params = N; b.n_filters = NF; b.cf_bytes = cf_bytes;
    return AST_OK;
}

template <class CF, int PREC>
static decltype(&fit_kernel<CF, PREC, 1>) fit_kernel_ptr(int minb)
{
    return minb >= 3 ? fit_kernel<CF, PREC, 3> : minb == 2 ? fit_kernel<CF, PREC, 2> : fit_kernel<CF, PREC, 1>;
}

// Launch geometry: CTA size (tpb), register budget (minb) and whether the CTA stages the
// observations in shared memory.  Staging is dropped when the block would lower the number of
// CTAs an SM holds (observations are read once per observation, not per RK4 step, so global
// reads through L1 cost little, while warps per SM decide how well latency is hidden).
// `obs_bytes` is the observation block's size, `optin` the device's per-CTA shared-memory limit.
template <class CF, int PREC>
static int fit_launch_core(int sm_count, size_t obs_bytes, size_t optin, int tpb_req, int minb_req, int stage_req,
                           int64_t n_chains, FitRun* r)
{
    // Register budget: 1 (255 registers, CTAs of up to 256), 2 (128), 3 (170, CTAs of up to 128).
    // Unset, the kernel's own shape (KernShape) when the chains fill it -- 3 for the double-float
    // path -- and the full register file when they do not: with fewer chains than three CTAs of
    // 128 per SM hold, the extra warps would not exist and the spills would remain.
    int minb = minb_req >= 3 ? 3 : minb_req == 2 ? 2 : minb_req == 1 ? 1 : KernShape<PREC>::min_ctas;
    if (minb_req <= 0 && minb == 3 &&
        n_chains < (int64_t)sm_count * KernShape<PREC>::tpb * KernShape<PREC>::min_ctas)
        minb = 1;
    if (minb == 3 && tpb_req > 128) {
        if (minb_req >= 3) return ast_set_error(AST_E_INVALID, "fit: min_ctas_per_sm 3 needs tpb <= 128");
        minb = 1;
    }
    auto kern = fit_kernel_ptr<CF, PREC>(minb);
    size_t smem_obs = 0;
    if (int rc = obs_smem_for(kern, obs_bytes, optin, &smem_obs)) return rc;
    int tpb = tpb_req;
    if (tpb <= 0) {
        // Enough CTAs to cover every SM before growing the CTA (small chain counts).
        int64_t per_sm = n_chains / (sm_count > 0 ? sm_count : 1);
        const int tpb_max = minb == 3 ? 128 : 256;
        tpb = 32;
        while (tpb < tpb_max && tpb * 2 <= per_sm) tpb *= 2;
    }
    if (tpb < 32 || tpb > 256 || (tpb & 31)) return ast_set_error(AST_E_INVALID, "fit: tpb must be 32..256, multiple of 32");
    int occ_smem = 0, occ_gmem = 0;
    AST_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_gmem, kern, tpb, 0));
    if (smem_obs) AST_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_smem, kern, tpb, smem_obs));
    bool stage = smem_obs != 0 && (stage_req > 0 || (stage_req == 0 && occ_smem >= occ_gmem));
    if (stage && occ_smem < 1) stage = false;
    const int occ = stage ? occ_smem : occ_gmem;
    if (occ < 1) return ast_set_error(AST_E_TOO_LARGE, "fit: kernel does not fit on an SM");
    int64_t ctas = (int64_t)sm_count * occ;
    const int64_t need = (n_chains + tpb - 1) / tpb;
    if (ctas > need) ctas = need;
    if (ctas < 1) ctas = 1;
    r->tpb = tpb;
    r->ctas = (int)ctas;
    r->smem = stage ? smem_obs : 0;
    r->minb = minb;
    return AST_OK;
}

template <class CF, int PREC>
static int fit_launch_cfg(ast_ctx* c, int tpb_req, int minb_req, int stage_req, int64_t n_chains, FitRun* r)
{
    return fit_launch_core<CF, PREC>(c->sm_count, (size_t)c->layout.bytes, c->smem_optin, tpb_req, minb_req, stage_req,
                                     n_chains, r);
}

extern "C" int ast_fit_begin(ast_ctx* c, const ast_fit_cfg* cfg)
{
    if (!c || !cfg) return ast_set_error(AST_E_INVALID, "ast_fit_begin: NULL argument");
    if (cfg->n_chains <= 0 || cfg->group_size <= 0 || cfg->n_chains % cfg->group_size)
        return ast_set_error(AST_E_INVALID, "ast_fit_begin: n_chains must be a positive multiple of group_size");
    if (cfg->n_stages <= 0) return ast_set_error(AST_E_INVALID, "ast_fit_begin: n_stages must be >= 1");
    if (cfg->precision != AST_PREC_FP64 && cfg->precision != AST_PREC_MIXED && cfg->precision != AST_PREC_MIXED_RHS32)
        return ast_set_error(AST_E_INVALID, "ast_fit_begin: bad precision");
    if (cfg->reopt && !cfg->params0) return ast_set_error(AST_E_INVALID, "ast_fit_begin: reopt needs params0");
    if (cfg->n_stages > 1 && cfg->n_stages > 1000000) return ast_set_error(AST_E_INVALID, "ast_fit_begin: n_stages too large");
    int rc = set_device(c->device);
    if (rc) return rc;
    FitRun& r = c->run;
    r = FitRun();
    r.cfg = *cfg;
    r.cfg.params0 = nullptr;
    r.stage = 0;
    r.reopt = cfg->reopt ? 1 : 0;
    const bool acc = (c->model.flags & AST_ACC) != 0;
    const int cfb = acc ? 8 : 4;
    const int mb = cfg->min_ctas_per_sm, so = cfg->stage_obs;
    const int32_t pr = cfg->precision;
    if (acc)
        rc = pr == AST_PREC_FP64        ? fit_launch_cfg<double, AST_PREC_FP64>(c, cfg->tpb, mb, so, cfg->n_chains, &r)
             : pr == AST_PREC_MIXED_RHS32 ? fit_launch_cfg<double, AST_PREC_MIXED_RHS32>(c, cfg->tpb, mb, so, cfg->n_chains, &r)
                                        : fit_launch_cfg<double, AST_PREC_MIXED>(c, cfg->tpb, mb, so, cfg->n_chains, &r);
    else
        rc = pr == AST_PREC_FP64        ? fit_launch_cfg<float, AST_PREC_FP64>(c, cfg->tpb, mb, so, cfg->n_chains, &r)
             : pr == AST_PREC_MIXED_RHS32 ? fit_launch_cfg<float, AST_PREC_MIXED_RHS32>(c, cfg->tpb, mb, so, cfg->n_chains, &r)
                                        : fit_launch_cfg<float, AST_PREC_MIXED>(c, cfg->tpb, mb, so, cfg->n_chains, &r);
    if (rc) return rc;
    const int64_t slots = (int64_t)r.tpb * r.ctas;
    const int64_t groups = cfg->n_chains / cfg->group_size;
    if ((rc = fit_alloc(c, slots, cfg->n_chains, groups, cfb))) return rc;
    FitBuffers& b = c->fb;
    AST_CUDA(cudaMemsetAsync(b.ctr, 0, 8 * 8, c->stream));
    reset_slots_kernel<<<(unsigned)((b.slots_pad + 255) / 256), 256, 0, c->stream>>>(b.chain, b.st, b.it, b.ev, b.dv,
                                                                                      b.slots_pad, c->n_filters);
    AST_CUDA(cudaGetLastError());
    AST_CUDA(cudaMemsetAsync(b.chain_dv, 0, sizeof(double) * cfg->n_chains * c->n_filters, c->stream));
    if (cfg->reopt) {
        // Stage-0 start of every group: params2x of the -m model (cuda.c:1409-1416).
        const int N = c->model.n_params;
        std::vector<double> x(N);
        if ((rc = ast_params2x(&c->model, cfg->params0, x.data()))) return rc;
        std::vector<unsigned char> gx((size_t)groups * N * cfb);
        for (int64_t g = 0; g < groups; g++)
            for (int i = 0; i < N; i++) {
                if (acc) ((double*)gx.data())[g * N + i] = x[i];
                else ((float*)gx.data())[g * N + i] = (float)x[i];
            }
        AST_CUDA(cudaMemcpyAsync(b.group_x, gx.data(), gx.size(), cudaMemcpyHostToDevice, c->stream));
        AST_CUDA(cudaStreamSynchronize(c->stream));
    }
    r.active = true;
    return AST_OK;
}

template <class CF, int PREC>
static int fit_step_t(ast_ctx* c, int64_t budget, int32_t* done, cudaStream_t s)
{
    FitRun& r = c->run;
    FitBuffers& b = c->fb;
    FitView<CF> V = make_view<CF>(c);
    AST_CUDA(cudaEventRecord(c->ev0, s));
    fit_kernel_ptr<CF, PREC>(r.minb)<<<r.ctas, r.tpb, r.smem, s>>>(c->dm, c->d_obs, c->layout, r.smem ? 1 : 0, V, budget);
    AST_CUDA(cudaGetLastError());
    AST_CUDA(cudaEventRecord(c->ev1, s));
    unsigned long long h[8];
    AST_CUDA(cudaMemcpyAsync(h, b.ctr, sizeof(h), cudaMemcpyDeviceToHost, s));
    AST_CUDA(cudaStreamSynchronize(s));
    float ms = 0;
    AST_CUDA(cudaEventElapsedTime(&ms, c->ev0, c->ev1));
    r.kernel_ms += ms;
    // A staging wait that ran out is reported, not fatal: the CTAs concerned read the observations
    // from global memory (same results) and drained their copies before exiting.  The error word
    // is cleared for the next launch and the step completes normally (*done is valid).
    int status = AST_OK;
    if (h[4]) {
        status = ast_set_error(AST_E_TIMEOUT, "fit: a CTA's shared-memory staging wait ran out (error word %llu)", h[4]);
        AST_CUDA(cudaMemsetAsync(&b.ctr[4], 0, sizeof(unsigned long long), s));
    }
    if (h[1] < (unsigned long long)r.cfg.n_chains) {
        *done = 0;
        if (status) AST_CUDA(cudaStreamSynchronize(s));
        return status;
    }
    // Stage finished: group argmin, hand-off or output.
    const int fp64_result = (PREC != AST_PREC_FP64 && r.cfg.fp64_result) ? 1 : 0;
    group_best_kernel<CF><<<(unsigned)b.groups, 256, 0, s>>>(c->dm, V, b.out_f, b.out_p, b.out_dv, c->d_obs,
                                                               c->layout, fp64_result);
    AST_CUDA(cudaGetLastError());
    if (r.stage == r.cfg.n_stages - 1) {
        *done = 1;
        r.n_evals = (int64_t)h[2];
        r.n_fits = (int64_t)h[3];
        AST_CUDA(cudaStreamSynchronize(s));
        return status;
    }
    r.stage++;
    r.reopt = 1;
    unsigned long long z[2] = {0, 0};
    AST_CUDA(cudaMemcpyAsync(b.ctr, z, sizeof(z), cudaMemcpyHostToDevice, s));
    AST_CUDA(cudaStreamSynchronize(s));
    *done = 0;
    return status;
}

extern "C" int ast_fit_step(ast_ctx* c, int64_t evals_per_slot, int32_t* done, void* stream)
{
    if (!c || !done) return ast_set_error(AST_E_INVALID, "ast_fit_step: NULL argument");
    if (!c->run.active) return ast_set_error(AST_E_INVALID, "ast_fit_step: no fit begun");
    if (evals_per_slot <= 0) evals_per_slot = INT64_MAX;
    int rc = set_device(c->device);
    if (rc) return rc;
    cudaStream_t s = stream ? (cudaStream_t)stream : c->stream;
    const bool acc = (c->model.flags & AST_ACC) != 0;
    if (c->run.cfg.precision == AST_PREC_FP64)
        return acc ? fit_step_t<double, AST_PREC_FP64>(c, evals_per_slot, done, s)
                   : fit_step_t<float, AST_PREC_FP64>(c, evals_per_slot, done, s);
    if (c->run.cfg.precision == AST_PREC_MIXED_RHS32)
        return acc ? fit_step_t<double, AST_PREC_MIXED_RHS32>(c, evals_per_slot, done, s)
                   : fit_step_t<float, AST_PREC_MIXED_RHS32>(c, evals_per_slot, done, s);
    return acc ? fit_step_t<double, AST_PREC_MIXED>(c, evals_per_slot, done, s)
               : fit_step_t<float, AST_PREC_MIXED>(c, evals_per_slot, done, s);
}

extern "C" int ast_fit_counters(ast_ctx* c, int64_t* n_evals, int64_t* n_fits)
{
    if (!c || !c->fb.ctr) return ast_set_error(AST_E_INVALID, "ast_fit_counters: no fit");
    unsigned long long h[8];
    AST_CUDA(cudaMemcpyAsync(h, c->fb.ctr, sizeof(h), cudaMemcpyDeviceToHost, c->stream));
    AST_CUDA(cudaStreamSynchronize(c->stream));
    if (n_evals) *n_evals = (int64_t)h[2];
    if (n_fits) *n_fits = (int64_t)h[3];
    return AST_OK;
}

extern "C" int64_t ast_fit_slots(ast_ctx* c) { return c ? c->fb.slots : 0; }

extern "C" int ast_set_stage_wait(ast_ctx* c, int32_t polls)
{
    if (!c || polls < 0) return ast_set_error(AST_E_INVALID, "ast_set_stage_wait: bad argument");
    c->stage_wait = polls;
    return AST_OK;
}

extern "C" int ast_fit_launch(ast_ctx* c, int32_t* tpb, int32_t* ctas, int32_t* minb, int32_t* smem)
{
    if (!c || !c->fb.ctr) return ast_set_error(AST_E_INVALID, "ast_fit_launch: no fit");
    if (tpb) *tpb = c->run.tpb;
    if (ctas) *ctas = c->run.ctas;
    if (minb) *minb = c->run.minb;
    if (smem) *smem = (int32_t)c->run.smem;
    return AST_OK;
}

extern "C" int ast_fit_end(ast_ctx* c, ast_fit_out* out)
{
    if (!c || !out) return ast_set_error(AST_E_INVALID, "ast_fit_end: NULL argument");
    if (!c->run.active) return ast_set_error(AST_E_INVALID, "ast_fit_end: no fit begun");
    int rc = set_device(c->device);
    if (rc) return rc;
    FitBuffers& b = c->fb;
    const int N = c->model.n_params, NF = c->n_filters;
    const int64_t G = c->run.cfg.n_chains / c->run.cfg.group_size;
    unsigned long long h[8];
    AST_CUDA(cudaMemcpyAsync(h, b.ctr, sizeof(h), cudaMemcpyDeviceToHost, c->stream));
    if (out->best_f) AST_CUDA(cudaMemcpyAsync(out->best_f, b.out_f, sizeof(double) * G, cudaMemcpyDeviceToHost, c->stream));
    if (out->best_params)
        AST_CUDA(cudaMemcpyAsync(out->best_params, b.out_p, sizeof(double) * G * N, cudaMemcpyDeviceToHost, c->stream));
    if (out->best_dv)
        AST_CUDA(cudaMemcpyAsync(out->best_dv, b.out_dv, sizeof(double) * G * NF, cudaMemcpyDeviceToHost, c->stream));
    if (out->chain_f)
        AST_CUDA(cudaMemcpyAsync(out->chain_f, b.chain_f, sizeof(double) * c->run.cfg.n_chains, cudaMemcpyDeviceToHost,
                                 c->stream));
    AST_CUDA(cudaStreamSynchronize(c->stream));
    out->n_evals = c->run.n_evals ? c->run.n_evals : (int64_t)h[2];
    out->n_fits = c->run.n_fits ? c->run.n_fits : (int64_t)h[3];
    out->kernel_ms = c->run.kernel_ms;
    c->run.active = false;
    return AST_OK;
}

extern "C" int ast_fit(ast_ctx* c, const ast_fit_cfg* cfg, ast_fit_out* out)
{
    int rc = ast_fit_begin(c, cfg);
    if (rc) return rc;
    int32_t done = 0;
    bool stage_timeout = false;
    for (int guard = 0; !done; guard++) {
        rc = ast_fit_step(c, 0, &done, nullptr);
        if (rc == AST_E_TIMEOUT) stage_timeout = true;  // reported at the end; results unaffected
        else if (rc) return rc;
        if (guard > 4 * cfg->n_stages + 16)
            return ast_set_error(AST_E_TIMEOUT, "ast_fit: stages did not complete");
    }
    if ((rc = ast_fit_end(c, out))) return rc;
    return stage_timeout ? ast_set_error(AST_E_TIMEOUT, "ast_fit: a shared-memory staging wait ran out (results "
                                                        "read the observations from global memory)")
                         : AST_OK;
}

// ==================================================================================== no-alloc fit
//
// ast_fit_noalloc: the same simplex search for callers that cannot allocate device memory --
// code running inside a host framework that owns every allocation through its own pool, or a
// process whose memory is reserved up front and must not grow.  Inputs and outputs are the
// caller's device buffers; everything else the search needs (the observation block, the chain
// state, per-chain and per-group results, counters) lives in one file-scope device array of
// AST_NOALLOC_SCRATCH_BYTES, which every GPU that loads this library holds until the process
// exits.  Nothing here calls cudaMalloc, cudaFree or an allocating library routine.
//
// The array is shared by all calls and keeps the last call's contents; each call re-initialises
// what must start at zero.  Calls whose work overlaps on a GPU (two streams, two threads) race on
// the array.  The first call on a device looks up the array's device address with
// cudaGetSymbolAddress with that device current; make that first call before any stream capture.

static __device__ __align__(256) unsigned char g_noalloc_scratch[AST_NOALLOC_SCRATCH_BYTES];

namespace ast {
__global__ void prep_obs_kernel(DevModel M, char* base, ObsLayout L, int64_t n);
__global__ void prep_sums_kernel(DevModel M, char* base, ObsLayout L, int64_t n);

template <class CF>
struct StartPoint {
    CF x[AST_MAX_PARAMS];
};

// Every group's stage-0 start point (the -m model, as x) written by value.
template <class CF>
__global__ void noalloc_fill_groups_kernel(CF* group_x, int64_t groups, int N, StartPoint<CF> p)
{
    const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (k < groups * N) group_x[k] = p.x[k % N];
}

// Copy the caller's observation arrays into the SoA block in scratch (E, S only without INTERP).
__global__ void noalloc_pack_kernel(char* base, ObsLayout L, int64_t n, const double* mjd, const float* v,
                                    const float* w, const int32_t* filt, const double* e_unit, const double* s_unit)
{
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    ((double*)(base + L.off_t))[i] = mjd[i];
    ((float*)(base + L.off_v))[i] = v[i];
    ((float*)(base + L.off_w))[i] = w[i];
    ((int32_t*)(base + L.off_f))[i] = filt[i];
    if (e_unit && s_unit) {
        double* ex = (double*)(base + L.off_e);
        double* sx = (double*)(base + L.off_s);
        for (int k = 0; k < 3; k++) {
            ex[k * n + i] = e_unit[3 * i + k];
            sx[k * n + i] = s_unit[3 * i + k];
        }
    }
}
}  // namespace ast

static void* g_noalloc_ptr[64];

// Bytes of scratch a call needs (the layout of fit_alloc, with the call's own sizes).
static int64_t noalloc_layout(int64_t S, int64_t C, int64_t G, int N, int NF, int cfb, int64_t obs_bytes,
                              int64_t* off /* [20] */)
{
    auto al = [](int64_t v) { return (v + 255) / 256 * 256; };
    int64_t o = 0, k = 0;
    off[k++] = o; o += al(obs_bytes);
    off[k++] = o; o += al(S * (N + 1) * N * cfb);   // x
    off[k++] = o; o += al(S * (N + 1) * cfb);       // f
    off[k++] = o; o += al(S * (N + 1));             // ind
    off[k++] = o; o += al(S * N * cfb);             // x0
    off[k++] = o; o += al(S * N * cfb);             // xr
    off[k++] = o; o += al(S * cfb);                 // fr
    off[k++] = o; o += al(S * 4);                   // st
    off[k++] = o; o += al(S * 4);                   // it
    off[k++] = o; o += al(S * 4);                   // ev
    off[k++] = o; o += al(S * 8);                   // chain
    off[k++] = o; o += al(S * NF * 8);              // dv
    off[k++] = o; o += al(C * 8);                   // chain_f
    off[k++] = o; o += al(C * N * cfb);             // chain_x
    off[k++] = o; o += al(C * NF * 8);              // chain_dv
    off[k++] = o; o += al(G * N * cfb);             // group_x
    off[k++] = o; o += al(8 * 8);                   // counters
    return o;
}

template <class CF, int PREC>
static int noalloc_run(const DevModel& dm, char* base, const int64_t* off, const ObsLayout& L, const ast_fit_cfg* cfg,
                       int64_t S, const FitRun& r, double* d_best_f, double* d_best_params, double* d_best_dv,
                       cudaStream_t s)
{
    const int64_t slots = (int64_t)r.tpb * r.ctas;
    const int N = dm.n_params, NF = dm.n_filters;
    const int64_t C = cfg->n_chains, G = C / cfg->group_size;
    FitView<CF> V;
    V.x = (CF*)(base + off[1]); V.f = (CF*)(base + off[2]); V.ind = (uint8_t*)(base + off[3]);
    V.x0 = (CF*)(base + off[4]); V.xr = (CF*)(base + off[5]); V.fr = (CF*)(base + off[6]);
    V.st = (int32_t*)(base + off[7]); V.it = (int32_t*)(base + off[8]); V.ev = (int32_t*)(base + off[9]);
    V.chain = (int64_t*)(base + off[10]); V.dv = (double*)(base + off[11]);
    V.chain_f = (double*)(base + off[12]); V.chain_x = (CF*)(base + off[13]); V.chain_dv = (double*)(base + off[14]);
    V.group_x = (CF*)(base + off[15]); V.ctr = (unsigned long long*)(base + off[16]);
    V.S = S; V.n_slots = slots; V.n_chains = C; V.group_size = cfg->group_size;
    V.seed = cfg->seed; V.evals_cap = cfg->evals_cap; V.steps_cap = cfg->steps_cap > 0 ? cfg->steps_cap : 5000;
    V.reopt = cfg->reopt ? 1 : 0;
    // What must start at zero: counters, slot state, the chains' last delta_V.
    AST_CUDA(cudaMemsetAsync(V.ctr, 0, 8 * 8, s));
    reset_slots_kernel<<<(unsigned)((S + 255) / 256), 256, 0, s>>>(V.chain, V.st, V.it, V.ev, V.dv, S, NF);
    AST_CUDA(cudaGetLastError());
    AST_CUDA(cudaMemsetAsync(V.chain_dv, 0, sizeof(double) * C * NF, s));
    if (cfg->reopt) {
        // Every group starts from params2x of the -m model (cuda.c:1409-1416).
        StartPoint<CF> p;
        params2x<CF>(dm, cfg->params0, p.x);
        noalloc_fill_groups_kernel<CF><<<(unsigned)((G * N + 255) / 256), 256, 0, s>>>(V.group_x, G, N, p);
        AST_CUDA(cudaGetLastError());
    }
    for (int32_t stage = 0; stage < cfg->n_stages; stage++) {
        V.stage = stage;
        V.last_stage = stage == cfg->n_stages - 1;
        fit_kernel_ptr<CF, PREC>(r.minb)<<<r.ctas, r.tpb, r.smem, s>>>(dm, base + off[0], L, r.smem ? 1 : 0, V,
                                                                       INT64_MAX);
        AST_CUDA(cudaGetLastError());
        unsigned long long h[8];
        AST_CUDA(cudaMemcpyAsync(h, V.ctr, sizeof(h), cudaMemcpyDeviceToHost, s));
        AST_CUDA(cudaStreamSynchronize(s));
        if (h[4]) return ast_set_error(AST_E_TIMEOUT, "ast_fit_noalloc: a CTA's shared-memory staging wait ran out");
        if (h[1] != (unsigned long long)C)
            return ast_set_error(AST_E_TIMEOUT, "ast_fit_noalloc: stage %d finished %llu of %lld chains", stage, h[1],
                                 (long long)C);
        // As in ast_fit: with fp64_result a mixed search reports each group's FP64 chi^2.
        const int fp64_result = (PREC == AST_PREC_MIXED && cfg->fp64_result) ? 1 : 0;
        group_best_kernel<CF><<<(unsigned)G, 256, 0, s>>>(dm, V, d_best_f, d_best_params, d_best_dv, base + off[0], L,
                                                          fp64_result);
        AST_CUDA(cudaGetLastError());
        V.reopt = 1;
        unsigned long long z[2] = {0, 0};
        AST_CUDA(cudaMemcpyAsync(V.ctr, z, sizeof(z), cudaMemcpyHostToDevice, s));
    }
    AST_CUDA(cudaStreamSynchronize(s));
    return AST_OK;
}

extern "C" int ast_fit_noalloc(const ast_model* model, const ast_obs_set* obs, const double* d_mjd, const float* d_v,
                               const float* d_w, const int32_t* d_filter, const double* d_e_unit,
                               const double* d_s_unit, const ast_fit_cfg* cfg, double* d_best_f,
                               double* d_best_params, double* d_best_dv, void* stream)
{
    if (!model || !obs || !cfg || !d_mjd || !d_v || !d_w || !d_filter || !d_best_f || !d_best_params || !d_best_dv)
        return ast_set_error(AST_E_INVALID, "ast_fit_noalloc: NULL argument");
    const bool interp = (model->flags & AST_INTERP) != 0;
    if (!interp && (!d_e_unit || !d_s_unit))
        return ast_set_error(AST_E_INVALID, "ast_fit_noalloc: E/S unit vectors needed without AST_INTERP");
    if (obs->n_data <= model->n_params + obs->n_filters || obs->n_data > AST_NOALLOC_MAX_DATA)
        return ast_set_error(AST_E_TOO_LARGE, "ast_fit_noalloc: n_data %d outside %d..%d", obs->n_data,
                             model->n_params + obs->n_filters + 1, AST_NOALLOC_MAX_DATA);
    if (obs->n_filters < 1 || obs->n_filters > AST_MAX_FILTERS)
        return ast_set_error(AST_E_INVALID, "ast_fit_noalloc: n_filters %d outside 1..%d", obs->n_filters, AST_MAX_FILTERS);
    if (cfg->n_chains <= 0 || cfg->n_chains > AST_NOALLOC_MAX_CHAINS)
        return ast_set_error(AST_E_TOO_LARGE, "ast_fit_noalloc: n_chains %lld outside 1..%d (the fixed scratch size)",
                             (long long)cfg->n_chains, AST_NOALLOC_MAX_CHAINS);
    if (cfg->group_size <= 0 || cfg->n_chains % cfg->group_size || cfg->n_stages <= 0 ||
        (cfg->precision != AST_PREC_FP64 && cfg->precision != AST_PREC_MIXED) || (cfg->reopt && !cfg->params0))
        return ast_set_error(AST_E_INVALID, "ast_fit_noalloc: bad configuration");
    if ((model->flags & AST_NUDGE) && (obs->n_minima < 1 || obs->n_minima > AST_NOBS_MAX))
        return ast_set_error(AST_E_INVALID, "ast_fit_noalloc: NUDGE needs 1..%d observed minima", AST_NOBS_MAX);
    DevModel dm;
    int rc = build_dev_model(model, obs, &dm);
    if (rc) return rc;
    int dev = 0;
    AST_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) return ast_set_error(AST_E_INVALID, "ast_fit_noalloc: device %d", dev);
    if (!g_noalloc_ptr[dev]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p)
            return ast_set_error(AST_E_CUDA, "ast_fit_noalloc: cudaGetSymbolAddress: %s", cudaGetErrorString(e));
        g_noalloc_ptr[dev] = p;
    }
    char* base = (char*)g_noalloc_ptr[dev];
    cudaStream_t s = (cudaStream_t)stream;
    const int N = model->n_params, NF = obs->n_filters;
    const bool acc = (model->flags & AST_ACC) != 0;
    const int cfb = acc ? 8 : 4;
    const ObsLayout L = ObsLayout::make(obs->n_data);
    // Launch geometry as ast_fit_begin chooses it (CTA size, register budget, staging of the
    // observations in shared memory, CTAs); the slots are the launch's threads.
    int sms = 0, optin = 0;
    AST_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    AST_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    FitRun r;
    if (acc)
        rc = cfg->precision == AST_PREC_FP64
                 ? fit_launch_core<double, AST_PREC_FP64>(sms, L.bytes, optin, cfg->tpb, cfg->min_ctas_per_sm, cfg->stage_obs, cfg->n_chains, &r)
                 : fit_launch_core<double, AST_PREC_MIXED>(sms, L.bytes, optin, cfg->tpb, cfg->min_ctas_per_sm, cfg->stage_obs, cfg->n_chains, &r);
    else
        rc = cfg->precision == AST_PREC_FP64
                 ? fit_launch_core<float, AST_PREC_FP64>(sms, L.bytes, optin, cfg->tpb, cfg->min_ctas_per_sm, cfg->stage_obs, cfg->n_chains, &r)
                 : fit_launch_core<float, AST_PREC_MIXED>(sms, L.bytes, optin, cfg->tpb, cfg->min_ctas_per_sm, cfg->stage_obs, cfg->n_chains, &r);
    if (rc) return rc;
    const int64_t slots = (int64_t)r.tpb * r.ctas, S = (slots + 31) / 32 * 32;
    int64_t off[20];
    const int64_t bytes = noalloc_layout(S, cfg->n_chains, cfg->n_chains / cfg->group_size, N, NF, cfb, L.bytes, off);
    if (bytes > (int64_t)AST_NOALLOC_SCRATCH_BYTES)
        return ast_set_error(AST_E_TOO_LARGE, "ast_fit_noalloc: needs %lld scratch bytes, the library holds %lld",
                             (long long)bytes, (long long)AST_NOALLOC_SCRATCH_BYTES);
    // Observations: pack into scratch, then the per-interval RK4 steps and INTERP E, S.
    const int64_t n = obs->n_data;
    noalloc_pack_kernel<<<(unsigned)((n + 127) / 128), 128, 0, s>>>(base + off[0], L, n, d_mjd, d_v, d_w, d_filter,
                                                                    interp ? nullptr : d_e_unit, interp ? nullptr : d_s_unit);
    AST_CUDA(cudaGetLastError());
    prep_obs_kernel<<<(unsigned)((n + 127) / 128), 128, 0, s>>>(dm, base + off[0], L, n);
    AST_CUDA(cudaGetLastError());
    prep_sums_kernel<<<1, 32, 0, s>>>(dm, base + off[0], L, n);
    AST_CUDA(cudaGetLastError());
    if (acc)
        return cfg->precision == AST_PREC_FP64
                   ? noalloc_run<double, AST_PREC_FP64>(dm, base, off, L, cfg, S, r, d_best_f, d_best_params, d_best_dv, s)
                   : noalloc_run<double, AST_PREC_MIXED>(dm, base, off, L, cfg, S, r, d_best_f, d_best_params, d_best_dv, s);
    return cfg->precision == AST_PREC_FP64
               ? noalloc_run<float, AST_PREC_FP64>(dm, base, off, L, cfg, S, r, d_best_f, d_best_params, d_best_dv, s)
               : noalloc_run<float, AST_PREC_MIXED>(dm, base, off, L, cfg, S, r, d_best_f, d_best_params, d_best_dv, s);
}
