// simplex.cuh -- the downhill-simplex chain as a per-slot state machine (device code shared by
// the single-object fit, the multi-object batch and the serving loop).
//
// Slot state lives in HBM as structure-of-arrays indexed [k][slot] (FitView); every call of
// slot_iterate performs exactly one chi^2 evaluation of the slot's chain and the simplex move it
// completes.  The chain semantics (random start, initial simplex, sort with ties to the last
// index, centroid over all N+1 vertices, reflect/expand/contract/shrink tests, failure rules,
// iteration cap) are those of cuda.c:1424-1742.
#pragma once
#include <stdint.h>
#include "asteroid_gb300.h"
#include "mixed.cuh"
#include "model.cuh"
#include "philox.cuh"

namespace ast {

enum : int32_t { PH_INIT = 0, PH_REFLECT = 1, PH_EXPAND = 2, PH_CONTRACT = 3, PH_SHRINK = 4 };

template <class CF>
struct FitView {
    CF* x;
    CF* f;
    uint8_t* ind;
    CF* x0;
    CF* xr;
    CF* fr;
    int32_t* st;
    int32_t* it;
    int32_t* ev;
    int64_t* chain;
    double* dv;
    double* chain_f;
    CF* chain_x;
    double* chain_dv;
    CF* group_x;
    unsigned long long* ctr;
    int64_t S;          // slot stride (padded slot count)
    int64_t n_slots;
    int64_t n_chains;
    int32_t group_size;
    int32_t stage;
    int32_t reopt;
    int32_t last_stage;
    uint64_t seed;
    int64_t evals_cap;
    int32_t steps_cap;
    int32_t stage_wait = 1 << 22;  // polls of the shared-memory staging wait (bulk_stage)
};

template <class CF>
struct NMConst;
template <>
struct NMConst<double> {
    static constexpr double DX_INI = 0.001, D2X_INI = -1.2, DX_RAND = 0.0001;
    __device__ static double size2_min() { return 1e-10 * 1e-10; }
};
template <>
struct NMConst<float> {
    static constexpr float DX_INI = 0.001f, D2X_INI = -1.2f, DX_RAND = 0.0001f;
    __device__ static float size2_min() { return 1e-5f * 1e-5f; }
};
__device__ __forceinline__ double cf_exp(double v) { return exp(v); }
__device__ __forceinline__ float cf_exp(float v) { return expf(v); }

__device__ __forceinline__ bool hard_side(int per, int LAM, bool left)
{
    if (per == AST_HARD_BOTH) return true;
    if (left && per == AST_HARD_LEFT) return true;
    if (!left && per == AST_HARD_RIGHT) return true;
    return LAM == 0 && per == AST_PERIODIC_LAM;
}

#define XV(v, i) V.x[((int64_t)(v) * N + (i)) * S + s]
#define FV(v) V.f[(int64_t)(v) * S + s]
#define IND(v) V.ind[(int64_t)(v) * S + s]
#define X0V(i) V.x0[(int64_t)(i) * S + s]
#define XRV(i) V.xr[(int64_t)(i) * S + s]

// Random start point and initial simplex of chain c (cuda.c:1459-1545).
template <class CF>
__device__ void start_chain(const DevModel& M, const FitView<CF>& V, int64_t s, int64_t c)
{
    const int N = M.n_params;
    const int64_t S = V.S;
    const ast_type_ids& T = M.t;
    const int reopt = V.reopt;
    const double SMALL = 1e-8;
    const CF DX_INI = NMConst<CF>::DX_INI, D2X_INI = NMConst<CF>::D2X_INI, DX_RAND = NMConst<CF>::DX_RAND;
    CF x0[AST_MAX_PARAMS];
    const int64_t g = c / V.group_size;
    for (int i = 0; i < N; i++) x0[i] = reopt ? V.group_x[g * N + i] : (CF)0;
    uint32_t k = 0;
    int LAM = 0;
    for (int i = 0; i < N; i++) {
        const float r = uniform01(V.seed, (uint64_t)c, (uint32_t)V.stage, k++);
        const int pt = M.ptype[i], per = M.periodic[i];
        if ((M.flags & AST_BC) && !reopt) {
            if (pt == T.c) { x0[i] = x0[M.idx[T.c_tumb]]; continue; }
            if (pt == T.b) { x0[i] = x0[M.idx[T.b_tumb]]; continue; }
        }
        if (!reopt || M.frozen[i] == -1) {
            x0[i] = (CF)(DX_INI + SMALL + r * (1.0 - 2 * (SMALL + DX_INI)));
        } else {
            CF xmin = x0[i] - DX_RAND;
            CF xmax = x0[i] + DX_RAND;
            if (xmin < SMALL && hard_side(per, LAM, true)) xmin = (CF)SMALL;
            if (xmax > 1.0 - SMALL && hard_side(per, LAM, false)) xmax = (CF)(1.0 - SMALL);
            x0[i] = xmin + r * (xmax - xmin);
        }
        if (pt == T.Es) LAM = x0[i] >= 0.5;
    }
    for (int i = 0; i < N; i++) XV(0, i) = x0[i];
    for (int j = 1; j <= N; j++) {
        for (int i = 0; i < N; i++) {
            CF xv = x0[i];
            if (i == j - 1) {
                const int per = M.periodic[i];
                const float d2x = uniform01(V.seed, (uint64_t)c, (uint32_t)V.stage, k++);
                CF dx = DX_INI * cf_exp(D2X_INI * d2x);
                if (uniform01(V.seed, (uint64_t)c, (uint32_t)V.stage, k++) < 0.5) {
                    dx = -dx;
                    if (x0[i] + dx < SMALL && hard_side(per, LAM, true)) dx = -dx;
                } else {
                    if (x0[i] + dx > 1.0 - SMALL && hard_side(per, LAM, false)) dx = -dx;
                }
                xv = x0[i] + dx;
            }
            XV(j, i) = xv;
        }
    }
    for (int j = 0; j <= N; j++) IND(j) = (uint8_t)j;
}

template <class CF, int PREC>
__device__ __forceinline__ CF eval_point(const DevModel& M, const ObsView& o, const double* params, CF* dv,
                                         const float4* trig)
{
    if (PREC == AST_PREC_FP64) return chi2_fp64<CF>(M, o, params, dv);
    return chi2_mixed<CF, PREC == AST_PREC_MIXED_RHS32>(M, o, params, dv, trig);
}

// Register state of a slot between evaluations.
template <class CF>
struct SlotState {
    int64_t chain;  // chain index within its object, -1 = idle
    int32_t st, l, ev;
    CF dvl[AST_MAX_FILTERS];
};

// End of a simplex iteration (cuda.c:1575-1640): selection sort with ties to the last index
// (an all-NaN simplex keeps ind[0] = 0 with f = 1e30), centroid of all N+1 vertices, the size,
// iteration and evaluation caps, and the next reflection point.  Returns true if the chain ends.
template <class CF>
__device__ __forceinline__ bool nm_iter_top(const DevModel& M, const FitView<CF>& V, int64_t s, SlotState<CF>& R,
                                            int32_t& st)
{
    const int N = M.n_params;
    const int64_t S = V.S;
    const CF HUGEV = (CF)kHuge;
    const CF size2_min = NMConst<CF>::size2_min();
    bool finish = false;
    R.l++;
    // Selection sort, ties to the last index; an all-NaN simplex keeps ind[0] = 0
    // with f = 1e30 (cuda.c:1575-1601).
    uint32_t taken = 0;
    for (int jj = 0; jj <= N; jj++) {
        CF fmin = HUGEV;
        int jmin = -1;
        for (int j2 = 0; j2 <= N; j2++) {
            const CF fj = FV(j2);
            if (!(taken >> j2 & 1u) && fj <= fmin) { fmin = fj; jmin = j2; }
        }
        if (jmin < 0) {
            IND(0) = 0;
            FV(0) = HUGEV;
            break;
        }
        IND(jj) = (uint8_t)jmin;
        taken |= 1u << jmin;
    }
    // Centroid of all N+1 vertices and the size test (cuda.c:1604-1632).
    CF size2 = 0;
    for (int i = 0; i < N; i++) {
        CF sum = 0;
        for (int v = 0; v <= N; v++) sum = sum + XV(v, i);
        X0V(i) = sum / (CF)(N + 1);
    }
    for (int v = 0; v <= N; v++) {
        CF sum = 0;
        for (int i = 0; i < N; i++) {
            const CF dx = XV(v, i) - X0V(i);
            sum = sum + dx * dx;
        }
        size2 = size2 + sum;
    }
    size2 = size2 / (CF)N;
    if (size2 < size2_min || R.l > V.steps_cap || (V.evals_cap > 0 && R.ev >= V.evals_cap)) {
        finish = true;
    } else {
        const int w = IND(N);
        for (int i = 0; i < N; i++) {
            const CF c0 = X0V(i);
            XRV(i) = (M.frozen[i] != 1) ? c0 + (CF)1.0 * (c0 - XV(w, i)) : c0;
        }
        st = PH_REFLECT;
    }
    return finish;
}

// A finished chain's result: its best vertex and value (vertex 0 and 1e30 if it failed) and the
// delta_V of its last evaluation (cuda.c:1760-1821).
template <class CF>
__device__ __forceinline__ void nm_finish(const DevModel& M, const FitView<CF>& V, int64_t s, const SlotState<CF>& R,
                                          bool failed, unsigned long long& n_fit)
{
    const int N = M.n_params, NF = M.n_filters;
    const int64_t S = V.S;
    const int64_t chain = R.chain;
    const int b = failed ? 0 : IND(0);
    V.chain_f[chain] = failed ? kHuge : (double)FV(b);
    for (int i = 0; i < N; i++) V.chain_x[chain * N + i] = XV(b, i);
    for (int m = 0; m < NF; m++) V.chain_dv[chain * NF + m] = (double)R.dvl[m];
    n_fit += V.last_stage ? 1 : 0;
}

// The point the slot's chain evaluates next, in x (cuda.c:1512-1545 start vertices, 1635-1640
// reflection, 1660-1663 expansion, 1694-1698 contraction, 1716-1722 shrink).
template <class CF>
__device__ __forceinline__ void slot_point(const DevModel& M, const FitView<CF>& V, int64_t s, const SlotState<CF>& R,
                                           CF* p)
{
    const int N = M.n_params;
    const int64_t S = V.S;
    const int phase = R.st & 0xff;
    const int j = (R.st >> 8) & 0xff;
    if (phase == PH_INIT) {
        for (int i = 0; i < N; i++) p[i] = XV(j, i);
    } else if (phase == PH_REFLECT || phase == PH_CONTRACT) {
        for (int i = 0; i < N; i++) p[i] = XRV(i);
    } else if (phase == PH_EXPAND) {
        for (int i = 0; i < N; i++) {
            const CF c0 = X0V(i);
            p[i] = (M.frozen[i] != 1) ? c0 + (CF)2.0 * (XRV(i) - c0) : c0;
        }
    } else {
        const int v = IND(j);
        for (int i = 0; i < N; i++) p[i] = XV(v, i);
    }
}

// The simplex move an evaluation completes (cuda.c:1546-1760), as a state machine: INIT
// evaluates the N+1 start vertices, then REFLECT / EXPAND / CONTRACT / SHRINK.  p is the point
// slot_point gave, rej whether x2params rejected it, fv its chi^2 (counted in R.ev by the
// caller).  Returns true when the chain has finished (its result is written).
template <class CF>
__device__ __forceinline__ bool slot_apply(const DevModel& M, const FitView<CF>& V, int64_t s, SlotState<CF>& R,
                                           const CF* p, int rej, CF fv, unsigned long long& n_fit)
{
    const int N = M.n_params;
    const int64_t S = V.S;
    const CF HUGEV = (CF)kHuge;
    int32_t st = R.st;
    const int phase = st & 0xff;
    int j = (st >> 8) & 0xff;
    int bad = (st >> 16) & 1;
    bool iter_top = false, finish = false, failed = false;
    if (phase == PH_INIT) {
        if (rej) {
            finish = failed = true;
        } else {
            FV(j) = fv;
            j++;
            if (j > N) iter_top = true;
            else st = PH_INIT | (j << 8);
        }
    } else if (phase == PH_REFLECT) {
        const CF f_r = rej ? HUGEV : fv;
        const int b = IND(0), sw = IND(N - 1), w = IND(N);
        if (f_r >= FV(b) && f_r < FV(sw)) {
            for (int i = 0; i < N; i++) XV(w, i) = p[i];
            FV(w) = f_r;
            iter_top = true;
        } else if (f_r < FV(b)) {
            V.fr[s] = f_r;
            st = PH_EXPAND;
        } else {
            for (int i = 0; i < N; i++) {
                const CF c0 = X0V(i);
                XRV(i) = (M.frozen[i] != 1) ? c0 + (CF)0.5 * (XV(w, i) - c0) : c0;
            }
            st = PH_CONTRACT;
        }
    } else if (phase == PH_EXPAND) {
        const CF f_e = rej ? HUGEV : fv;
        const CF f_r = V.fr[s];
        const int w = IND(N);
        if (f_e < f_r) {
            for (int i = 0; i < N; i++) XV(w, i) = p[i];
            FV(w) = f_e;
        } else {
            for (int i = 0; i < N; i++) XV(w, i) = XRV(i);
            FV(w) = f_r;
        }
        iter_top = true;
    } else if (phase == PH_CONTRACT) {
        const CF f_c = rej ? HUGEV : fv;
        const int w = IND(N);
        if (f_c < FV(w)) {
            for (int i = 0; i < N; i++) XV(w, i) = p[i];
            FV(w) = f_c;
            iter_top = true;
        } else {
            // Shrink every vertex but the best towards it (cuda.c:1716-1727).
            const int b = IND(0), v = IND(1);
            for (int i = 0; i < N; i++)
                if (M.frozen[i] != 1) XV(v, i) = XV(b, i) + (CF)0.5 * (XV(v, i) - XV(b, i));
            st = PH_SHRINK | (1 << 8);
        }
    } else {  // PH_SHRINK
        if (rej) bad = 1;
        else FV(IND(j)) = fv;
        j++;
        if (j <= N) {
            const int b = IND(0), v = IND(j);
            for (int i = 0; i < N; i++)
                if (M.frozen[i] != 1) XV(v, i) = XV(b, i) + (CF)0.5 * (XV(v, i) - XV(b, i));
            st = PH_SHRINK | (j << 8) | (bad << 16);
        } else if (bad) {
            finish = failed = true;
        } else {
            iter_top = true;
        }
    }
    if (iter_top && nm_iter_top<CF>(M, V, s, R, st)) finish = true;
    R.st = st;
    if (finish) nm_finish<CF>(M, V, s, R, failed, n_fit);
    return finish;
}

// One evaluation of the slot's chain and the simplex move it completes.  V carries the slot
// buffers and the chain-level settings of the chain's object.  Returns true when the chain has
// finished (its result is written).
template <class CF, int PREC>
__device__ __forceinline__ bool slot_iterate(const DevModel& M, const ObsView& o, const FitView<CF>& V, int64_t s,
                                             SlotState<CF>& R, const float4* trig, unsigned long long& n_ev,
                                             unsigned long long& n_fit)
{
    CF p[AST_MAX_PARAMS];
    slot_point<CF>(M, V, s, R, p);
    // One evaluation: x -> params (hard limits), then chi^2.
    double params[AST_MAX_PARAMS];
    const int rej = x2params<CF>(M, V.reopt, p, params);
    CF fv = (CF)kHuge;
    if (!rej) {
        fv = eval_point<CF, PREC>(M, o, params, R.dvl, trig);
        R.ev++;
        n_ev++;
    }
    return slot_apply<CF>(M, V, s, R, p, rej, fv, n_fit);
}


// Argmin over group g of V's chains (lowest chi^2, lowest chain on ties, as the serial loop of
// cuda.c:1770-1782) and the stage hand-off or the final output (cuda.c:1785-1823).  One CTA per
// group.  With fp64_obs (a mixed-precision fit asked for FP64 results), the reported chi^2 of the
// group is the plain FP64 path's chi^2 at its best parameters.
template <class CF>
__device__ void group_best_body(const DevModel& M, const FitView<CF>& V, int64_t g, double* out_f, double* out_p,
                                double* out_dv, const ObsView* fp64_obs = nullptr)
{
    const int N = M.n_params, NF = M.n_filters;
    double best = kHuge;
    int64_t bi = INT64_MAX;
    for (int64_t c = g * V.group_size + threadIdx.x; c < (g + 1) * V.group_size; c += blockDim.x) {
        const double f = V.chain_f[c];
        if (f < best || (f == best && c < bi)) { best = f; bi = c; }
    }
    for (int off = 16; off > 0; off >>= 1) {
        const double of = __shfl_down_sync(0xffffffffu, best, off);
        const long long oi = __shfl_down_sync(0xffffffffu, (long long)bi, off);
        if (of < best || (of == best && oi < bi)) { best = of; bi = oi; }
    }
    __shared__ double sf[32];
    __shared__ long long si[32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) { sf[warp] = best; si[warp] = bi; }
    __syncthreads();
    if (threadIdx.x != 0) return;
    for (int w = 1; w < (int)(blockDim.x + 31) / 32; w++)
        if (sf[w] < best || (sf[w] == best && si[w] < bi)) { best = sf[w]; bi = si[w]; }
    // Strictly below 1e30, else the group's first chain (the reference's thread_min = 0).
    const int64_t cb = (best < kHuge) ? bi : g * V.group_size;
    CF xb[AST_MAX_PARAMS];
    for (int i = 0; i < N; i++) xb[i] = V.chain_x[cb * N + i];
    if (!V.last_stage) {
        if ((M.flags & AST_P_PSI) && V.reopt == 0) {
            // P_PSI hand-off: x of L changes meaning from 1/Ppsi to L (cuda.c:1788-1799).
            double p[AST_MAX_PARAMS];
            x2params<CF>(M, 0, xb, p);
            params2x<CF>(M, p, xb);
        }
        for (int i = 0; i < N; i++) V.group_x[g * N + i] = xb[i];
    } else {
        out_f[g] = best < kHuge ? best : kHuge;
        double p[AST_MAX_PARAMS];
        for (int i = 0; i < N; i++) p[i] = 0;
        if (best < kHuge) x2params<CF>(M, V.reopt, xb, p);
        if (fp64_obs && best < kHuge) {
            double d[AST_MAX_FILTERS];
            out_f[g] = (double)chi2_fp64<double>(M, *fp64_obs, p, d);
        }
        for (int i = 0; i < N; i++) out_p[g * N + i] = p[i];
        for (int m = 0; m < NF; m++) out_dv[g * NF + m] = best < kHuge ? V.chain_dv[cb * NF + m] : 0.0;
    }
}


#undef XV
#undef FV
#undef IND
#undef X0V
#undef XRV

}  // namespace ast
