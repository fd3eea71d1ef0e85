// batch.cu -- many objects fitted by one persistent launch, and the serving loop built on it.
//
// The reference fits one object per process: chi2_gpu<<<N_BLOCKS, BSIZE>>> over one light curve
// held in shared memory (cuda.c:1326-1354).  Here a device table of objects (BatchObj) sits
// beside one pool of persistent slots (the slot buffers of simplex.cuh, sized for the largest
// parameter and filter counts).  Chains of all objects share one global chain index space: an
// object owns [chain0, chain0 + n_chains), a slot that needs work takes the next index from an
// atomic counter and finds its object by binary search.  Every object keeps its own model
// variant, light curve, filter count, parameter count, seed and caps, and its results are the
// same as a single-object fit with the same settings (the chain's random draws are keyed by the
// object's seed and the chain's index within the object).
//
// Two refill mappings:
//   REFILL 1   thread per chain: a slot takes a new chain as soon as its own has finished;
//   REFILL 32  warp per object: a warp takes 32 consecutive chains at once when all its lanes
//              are idle, so the lanes of a warp always integrate the same light curve (no
//              divergence between objects of different lengths, at the cost of idle lanes
//              while the warp's last chain finishes).
// ast_batch_tune times both, with several CTA sizes, on the caller's batch.
//
// Batch (ast_batch_*): all objects are added, then one CUDA graph -- slot reset, the persistent
// kernel run to completion, the per-group argmin of every object -- is captured once and
// replayed by ast_batch_run.
//
// Serving (ast_server_*, ast_submit, ast_poll): requests are admitted while their device
// footprint fits an HBM budget; each ast_server_step launches the same kernel for a bounded
// number of evaluations per slot, retires the objects whose chains have all finished (argmin,
// results to the host, memory freed) and admits queued requests in arrival order, whose chains
// the slots pick up as soon as the chains before them are taken.
#include <cuda_runtime.h>
#include <stdio.h>
#include <string.h>
#include <algorithm>
#include <type_traits>
#include <chrono>
#include <deque>
#include <vector>

#include "asteroid_gb300.h"
#include "engine.cuh"
#include "simplex.cuh"

namespace ast {

template <class CF>
struct BatchObj {
    DevModel M;
    const void* obs;
    ObsLayout L;
    int64_t chain0, n_chains;
    int32_t group_size, reopt, steps_cap, fp64_result;
    int32_t cancelled;         // ast_cancel: slots drop the object's chains (counted as finished)
    uint64_t seed;
    int64_t evals_cap;
    CF* x_start;               // [G][N] start points under reopt, else unused
    double* chain_f;           // [n_chains]
    CF* chain_x;               // [n_chains][N]
    double* chain_dv;          // [n_chains][NF]
    double* out_f;             // [G]
    double* out_p;             // [G][N]
    double* out_dv;            // [G][NF]
    unsigned long long* done;  // finished chains
};

// Last object whose chain0 <= c (the table is sorted by chain0).
template <class CF>
__device__ __forceinline__ int find_obj(const BatchObj<CF>* objs, int n, int64_t c)
{
    int lo = 0, hi = n - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (objs[mid].chain0 <= c) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// The slot buffers of V with the chain-level settings and outputs of object B.
template <class CF>
__device__ __forceinline__ FitView<CF> obj_view(const FitView<CF>& V, const BatchObj<CF>& B)
{
    FitView<CF> W = V;
    W.n_chains = B.n_chains;
    W.group_size = B.group_size;
    W.stage = 0;
    W.reopt = B.reopt;
    W.last_stage = 1;
    W.seed = B.seed;
    W.evals_cap = B.evals_cap;
    W.steps_cap = B.steps_cap;
    W.group_x = B.x_start;
    W.chain_f = B.chain_f;
    W.chain_x = B.chain_x;
    W.chain_dv = B.chain_dv;
    return W;
}

template <class CF>
__device__ __forceinline__ void batch_start(const BatchObj<CF>* objs, int n_objs, const FitView<CF>& V, int64_t s,
                                            int64_t gchain, int& k, SlotState<CF>& R)
{
    k = find_obj(objs, n_objs, gchain);
    const BatchObj<CF>& B = objs[k];
    R.chain = gchain - B.chain0;
    start_chain<CF>(B.M, obj_view(V, B), s, R.chain);
    R.st = PH_INIT;
    R.l = 0;
    R.ev = 0;
    for (int m = 0; m < AST_MAX_FILTERS; m++) R.dvl[m] = (CF)0;
}

// V.chain[s] holds the slot's global chain index; V.n_chains is the end of the chain space.
template <class CF, int PREC, int REFILL>
__global__ void __launch_bounds__(KernShape<PREC>::tpb, KernShape<PREC>::min_ctas) batch_kernel(const BatchObj<CF>* objs, int n_objs, FitView<CF> V,
                                                       int64_t budget)
{
    __shared__ float4 trig[PREC == AST_PREC_MIXED ? kTrigTable : 1];
    if (PREC == AST_PREC_MIXED) {
        trig_table_fill(trig);
        __syncthreads();
    }
    const int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (s >= V.n_slots) return;  // n_slots is a multiple of 32: whole warps leave
    const int64_t S = V.S;
    int64_t gchain = V.chain[s];
    int k = 0;
    SlotState<CF> R;
    R.chain = -1;
    R.st = V.st[s];
    R.l = V.it[s];
    R.ev = V.ev[s];
    for (int m = 0; m < AST_MAX_FILTERS; m++) R.dvl[m] = (CF)0;
    if (gchain >= 0) {
        k = find_obj(objs, n_objs, gchain);
        R.chain = gchain - objs[k].chain0;
        for (int m = 0; m < objs[k].M.n_filters; m++) R.dvl[m] = (CF)V.dv[(int64_t)m * S + s];
    }
    int64_t used = 0;
    unsigned long long n_ev = 0, n_fit = 0, n_done = 0;
    const unsigned lane = threadIdx.x & 31u;
    while (true) {
        if (REFILL == 1) {
            if (gchain < 0) {
                const unsigned long long c = atomicAdd(&V.ctr[0], 1ull);
                if (c >= (unsigned long long)V.n_chains) break;
                gchain = (int64_t)c;
                batch_start<CF>(objs, n_objs, V, s, gchain, k, R);
            }
        } else {
            const unsigned idle = __ballot_sync(0xffffffffu, gchain < 0);
            if (idle == 0xffffffffu) {
                unsigned long long base = 0;
                if (lane == 0) base = atomicAdd(&V.ctr[0], 32ull);
                base = __shfl_sync(0xffffffffu, base, 0);
                if (base >= (unsigned long long)V.n_chains) break;
                const unsigned long long c = base + lane;
                if (c < (unsigned long long)V.n_chains) {
                    gchain = (int64_t)c;
                    batch_start<CF>(objs, n_objs, V, s, gchain, k, R);
                }
            }
        }
        if (gchain >= 0) {
            const BatchObj<CF>& B = objs[k];
            const ObsView o = B.L.view(B.obs, B.M.n_data);
            if (B.cancelled || slot_iterate<CF, PREC>(B.M, o, obj_view(V, B), s, R, trig, n_ev, n_fit)) {
                atomicAdd(B.done, 1ull);
                n_done++;
                gchain = -1;
                R.chain = -1;
            }
        }
        if (++used >= budget) break;
    }
    V.chain[s] = gchain;
    V.st[s] = R.st;
    V.it[s] = R.l;
    V.ev[s] = R.ev;
    if (gchain >= 0)
        for (int m = 0; m < objs[k].M.n_filters; m++) V.dv[(int64_t)m * S + s] = (double)R.dvl[m];
    if (n_done) atomicAdd(&V.ctr[1], n_done);
    if (n_ev) atomicAdd(&V.ctr[2], n_ev);
    if (n_fit) atomicAdd(&V.ctr[3], n_fit);
}

// ---------------------------------------------------------------- warp-tiled mapping
//
// REFILL 32 (a warp takes 32 chains of one object at once) with the warp-tiled evaluation
// (chi2_mixed_tile): the warp's 32 chains are evaluated together, the magnitudes of each tile of
// T observations spread over the lanes.  Lanes whose chain is idle or whose point x2params
// rejects take part without a result.  A warp whose chains belong to different objects, or to a
// NUDGE object, evaluates lane by lane as batch_kernel does.  Results are those of batch_kernel
// bit for bit.
template <class CF, int T>
__global__ void __launch_bounds__(KernShape<AST_PREC_MIXED>::tpb, KernShape<AST_PREC_MIXED>::min_ctas)
    batch_tile_kernel(const BatchObj<CF>* objs, int n_objs, FitView<CF> V, int64_t budget)
{
    __shared__ float4 trig[kTrigTable];
    extern __shared__ __align__(16) unsigned char tile_smem[];
    trig_table_fill(trig);
    __syncthreads();
    const int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (s >= V.n_slots) return;  // n_slots is a multiple of 32: whole warps leave
    unsigned char* wsm = tile_smem + (size_t)(threadIdx.x >> 5) * tile_warp_bytes(T);
    const int64_t S = V.S;
    int64_t gchain = V.chain[s];
    int k = 0;
    SlotState<CF> R;
    R.chain = -1;
    R.st = V.st[s];
    R.l = V.it[s];
    R.ev = V.ev[s];
    for (int m = 0; m < AST_MAX_FILTERS; m++) R.dvl[m] = (CF)0;
    if (gchain >= 0) {
        k = find_obj(objs, n_objs, gchain);
        R.chain = gchain - objs[k].chain0;
        for (int m = 0; m < objs[k].M.n_filters; m++) R.dvl[m] = (CF)V.dv[(int64_t)m * S + s];
    }
    int64_t used = 0;
    unsigned long long n_ev = 0, n_fit = 0, n_done = 0;
    const unsigned lane = threadIdx.x & 31u;
    while (true) {
        const unsigned idle = __ballot_sync(0xffffffffu, gchain < 0);
        if (idle == 0xffffffffu) {
            unsigned long long base = 0;
            if (lane == 0) base = atomicAdd(&V.ctr[0], 32ull);
            base = __shfl_sync(0xffffffffu, base, 0);
            if (base >= (unsigned long long)V.n_chains) break;
            const unsigned long long c = base + lane;
            if (c < (unsigned long long)V.n_chains) {
                gchain = (int64_t)c;
                batch_start<CF>(objs, n_objs, V, s, gchain, k, R);
            }
        }
        const bool has = gchain >= 0;
        // Cancelled objects drop their chains (counted as finished) without an evaluation.
        const bool drop = has && objs[k].cancelled;
        if (drop) {
            atomicAdd(objs[k].done, 1ull);
            n_done++;
            gchain = -1;
            R.chain = -1;
        }
        const bool live = has && !drop;
        CF p[AST_MAX_PARAMS];
        double params[AST_MAX_PARAMS];
        int rej = 1;
        if (live) {
            const BatchObj<CF>& B = objs[k];
            slot_point<CF>(B.M, obj_view(V, B), s, R, p);
            rej = x2params<CF>(B.M, B.reopt, p, params);
        } else {
            for (int i = 0; i < AST_MAX_PARAMS; i++) params[i] = 0.5;
        }
        // One object for every live lane of the warp, and no NUDGE: the tiled evaluation.
        const unsigned live_mask = __ballot_sync(0xffffffffu, live);
        const int k0 = __shfl_sync(0xffffffffu, k, live_mask ? __ffs(live_mask) - 1 : 0);
        const bool same = __all_sync(0xffffffffu, !live || k == k0);
        CF fv = (CF)kHuge;
        if (live_mask && same && !(objs[k0].M.flags & AST_NUDGE)) {
            const BatchObj<CF>& B = objs[k0];
            const ObsView o = B.L.view(B.obs, B.M.n_data);
            fv = chi2_mixed_tile<CF, T>(B.M, o, params, live && !rej, R.dvl, trig, wsm);
        } else if (live && !rej) {
            const BatchObj<CF>& B = objs[k];
            const ObsView o = B.L.view(B.obs, B.M.n_data);
            fv = eval_point<CF, AST_PREC_MIXED>(B.M, o, params, R.dvl, trig);
        }
        if (live) {
            const BatchObj<CF>& B = objs[k];
            if (!rej) {
                R.ev++;
                n_ev++;
            }
            if (slot_apply<CF>(B.M, obj_view(V, B), s, R, p, rej, rej ? (CF)kHuge : fv, n_fit)) {
                atomicAdd(B.done, 1ull);
                n_done++;
                gchain = -1;
                R.chain = -1;
            }
        }
        if (++used >= budget) break;
    }
    V.chain[s] = gchain;
    V.st[s] = R.st;
    V.it[s] = R.l;
    V.ev[s] = R.ev;
    if (gchain >= 0)
        for (int m = 0; m < objs[k].M.n_filters; m++) V.dv[(int64_t)m * S + s] = (double)R.dvl[m];
    if (n_done) atomicAdd(&V.ctr[1], n_done);
    if (n_ev) atomicAdd(&V.ctr[2], n_ev);
    if (n_fit) atomicAdd(&V.ctr[3], n_fit);
}

// ---------------------------------------------------------------- cooperative chains
//
// For a lightly loaded server (few chains in flight, each 5000 sequential evaluations), a chain
// can use G lanes instead of one.  Each round the group's leader lane lists the points the
// sequential chain may evaluate next -- the N+1 start vertices (G at a time), the reflection,
// expansion and inside contraction of an iteration (all three at once), the shrunk vertices (G
// at a time) -- the G lanes evaluate them side by side, and the leader applies the results in
// the sequential order, counting only the evaluations the one-lane chain makes.  The chain's
// path, counters and result are those of slot_iterate, bit for bit; an iteration costs one
// round instead of one to two evaluations in a row, and INIT and SHRINK G times fewer.

constexpr int kCoopLanes = 4;

// The slot-buffer accessors of simplex.cuh (vertex v's coordinate i, its value, the sort index,
// the centroid, the trial point), for slot s of a view V with stride S and N parameters.
#define XV(v, i) V.x[((int64_t)(v) * N + (i)) * S + s]
#define FV(v) V.f[(int64_t)(v) * S + s]
#define IND(v) V.ind[(int64_t)(v) * S + s]
#define X0V(i) V.x0[(int64_t)(i) * S + s]
#define XRV(i) V.xr[(int64_t)(i) * S + s]

template <class CF>
struct CoopXchg {  // one group's exchange area in shared memory
    CF pts[kCoopLanes][AST_MAX_PARAMS];
    CF f[kCoopLanes];
    CF dv[kCoopLanes][AST_MAX_FILTERS];
    int32_t rej[kCoopLanes];
    int32_t dv_set[kCoopLanes];
};

// The points of the next round into X; returns how many.
template <class CF>
__device__ int coop_plan(const DevModel& M, const FitView<CF>& V, int64_t s, const SlotState<CF>& R, CoopXchg<CF>& X)
{
    const int N = M.n_params;
    const int64_t S = V.S;
    const int phase = R.st & 0xff, j = (R.st >> 8) & 0xff;
    if (phase == PH_REFLECT) {
        const int w = IND(N);
        for (int i = 0; i < N; i++) {
            const CF c0 = X0V(i), xr = XRV(i);
            X.pts[0][i] = xr;
            X.pts[1][i] = (M.frozen[i] != 1) ? c0 + (CF)2.0 * (xr - c0) : c0;         // expansion
            X.pts[2][i] = (M.frozen[i] != 1) ? c0 + (CF)0.5 * (XV(w, i) - c0) : c0;   // contraction
        }
        return 3;
    }
    const int n = min(kCoopLanes, N + 1 - j);
    for (int k = 0; k < n; k++) {
        const int v = phase == PH_INIT ? j + k : IND(j + k);
        for (int i = 0; i < N; i++) X.pts[k][i] = XV(v, i);
    }
    return n;
}

// The round's results in the sequential order (cuda.c:1546-1742): returns true when the chain
// ends; *failed as slot_iterate.
template <class CF>
__device__ bool coop_apply(const DevModel& M, const FitView<CF>& V, int64_t s, SlotState<CF>& R, const CoopXchg<CF>& X,
                           int n, unsigned long long& n_ev, bool* failed)
{
    const int N = M.n_params, NF = M.n_filters;
    const int64_t S = V.S;
    const CF HUGEV = (CF)kHuge;
    int32_t st = R.st;
    const int phase = st & 0xff;
    int j = (st >> 8) & 0xff;
    int bad = (st >> 16) & 1;
    *failed = false;
    // An evaluation the one-lane chain makes: counted, and its delta_V kept when it wrote one.
    auto use = [&](int k) -> CF {
        R.ev++;
        n_ev++;
        if (X.dv_set[k])
            for (int m = 0; m < NF; m++) R.dvl[m] = X.dv[k][m];
        return X.f[k];
    };
    bool iter_top = false;
    if (phase == PH_INIT) {
        for (int k = 0; k < n; k++) {
            if (X.rej[k]) {
                *failed = true;
                return true;
            }
            FV(j) = use(k);
            j++;
        }
        if (j > N) iter_top = true;
        else st = PH_INIT | (j << 8);
    } else if (phase == PH_REFLECT) {
        const CF f_r = X.rej[0] ? HUGEV : use(0);
        const int b = IND(0), sw = IND(N - 1), w = IND(N);
        if (f_r >= FV(b) && f_r < FV(sw)) {
            for (int i = 0; i < N; i++) XV(w, i) = X.pts[0][i];
            FV(w) = f_r;
        } else if (f_r < FV(b)) {
            const CF f_e = X.rej[1] ? HUGEV : use(1);
            const int from = f_e < f_r ? 1 : 0;
            for (int i = 0; i < N; i++) XV(w, i) = X.pts[from][i];
            FV(w) = from ? f_e : f_r;
        } else {
            for (int i = 0; i < N; i++) XRV(i) = X.pts[2][i];
            const CF f_c = X.rej[2] ? HUGEV : use(2);
            if (f_c < FV(w)) {
                for (int i = 0; i < N; i++) XV(w, i) = X.pts[2][i];
                FV(w) = f_c;
            } else {
                // Shrink every vertex but the best towards it (cuda.c:1716-1727); the best does
                // not move, so all of them can be shrunk before they are evaluated.
                for (int jj = 1; jj <= N; jj++) {
                    const int v = IND(jj);
                    for (int i = 0; i < N; i++)
                        if (M.frozen[i] != 1) XV(v, i) = XV(b, i) + (CF)0.5 * (XV(v, i) - XV(b, i));
                }
                R.st = PH_SHRINK | (1 << 8);
                return false;
            }
        }
        iter_top = true;
    } else {  // PH_SHRINK
        for (int k = 0; k < n; k++, j++) {
            if (X.rej[k]) bad = 1;
            else FV(IND(j)) = use(k);
        }
        if (j <= N) {
            st = PH_SHRINK | (j << 8) | (bad << 16);
        } else if (bad) {
            *failed = true;
            return true;
        } else {
            iter_top = true;
        }
    }
    bool finish = false;
    if (iter_top && nm_iter_top<CF>(M, V, s, R, st)) finish = true;
    R.st = st;
    return finish;
}

#undef XV
#undef FV
#undef IND
#undef X0V
#undef XRV

// G = kCoopLanes lanes per slot; V.n_slots counts groups.  Dynamic shared memory: one CoopXchg
// per group.
// Servers use cooperative chains for latency, not throughput: with the slot pool far from full a
// chain's evaluation runs fastest with the full register file (255 registers, no spills), so this
// kernel keeps the one-CTA-of-256 budget that the throughput kernels trade for occupancy.
template <class CF, int PREC>
__global__ void __launch_bounds__(256, 1) coop_kernel(const BatchObj<CF>* objs, int n_objs, FitView<CF> V,
                                                      int64_t budget)
{
    constexpr int G = kCoopLanes;
    __shared__ float4 trig[PREC == AST_PREC_MIXED ? kTrigTable : 1];
    extern __shared__ __align__(16) unsigned char coop_smem[];
    if (PREC == AST_PREC_MIXED) {
        trig_table_fill(trig);
        __syncthreads();
    }
    const int r = threadIdx.x % G;
    const int64_t s = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) / G;
    if (s >= V.n_slots) return;  // whole groups leave
    CoopXchg<CF>& X = ((CoopXchg<CF>*)coop_smem)[threadIdx.x / G];
    const unsigned mask = ((1u << G) - 1u) << ((threadIdx.x & 31u) & ~(unsigned)(G - 1));
    const int leader = (int)((threadIdx.x & 31u) & ~(unsigned)(G - 1));
    const int64_t S = V.S;
    int64_t gchain = -1;
    int k = 0;
    SlotState<CF> R;
    R.chain = -1;
    unsigned long long n_ev = 0, n_fit = 0, n_done = 0;
    if (r == 0) {
        gchain = V.chain[s];
        R.st = V.st[s];
        R.l = V.it[s];
        R.ev = V.ev[s];
        for (int m = 0; m < AST_MAX_FILTERS; m++) R.dvl[m] = (CF)0;
        if (gchain >= 0) {
            k = find_obj(objs, n_objs, gchain);
            R.chain = gchain - objs[k].chain0;
            for (int m = 0; m < objs[k].M.n_filters; m++) R.dvl[m] = (CF)V.dv[(int64_t)m * S + s];
        }
    }
    for (int64_t used = 0; used < budget; used++) {
        int n = 0, stop = 0;
        if (r == 0) {
            if (gchain < 0) {
                const unsigned long long c = atomicAdd(&V.ctr[0], 1ull);
                if (c >= (unsigned long long)V.n_chains) stop = 1;
                else {
                    gchain = (int64_t)c;
                    batch_start<CF>(objs, n_objs, V, s, gchain, k, R);
                }
            }
            if (!stop && objs[k].cancelled) {
                // A cancelled request's chain is dropped (counted as finished) without a round.
                atomicAdd(objs[k].done, 1ull);
                n_done++;
                gchain = -1;
                R.chain = -1;
            } else if (!stop) {
                n = coop_plan<CF>(objs[k].M, obj_view(V, objs[k]), s, R, X);
            }
        }
        stop = __shfl_sync(mask, stop, leader);
        if (stop) break;
        n = __shfl_sync(mask, n, leader);
        const int kk = __shfl_sync(mask, k, leader);
        __syncwarp(mask);
        if (r < n) {
            const BatchObj<CF>& B = objs[kk];
            const ObsView o = B.L.view(B.obs, B.M.n_data);
            CF p[AST_MAX_PARAMS];
            for (int i = 0; i < B.M.n_params; i++) p[i] = X.pts[r][i];
            double params[AST_MAX_PARAMS];
            const int rej = x2params<CF>(B.M, B.reopt, p, params);
            const CF unset = (CF)-7.5e37f;  // no chi^2 writes this delta_V: tells an early exit apart
            CF dvl[AST_MAX_FILTERS];
            for (int m = 0; m < AST_MAX_FILTERS; m++) dvl[m] = unset;
            CF fv = (CF)kHuge;
            if (!rej) fv = eval_point<CF, PREC>(B.M, o, params, dvl, trig);
            X.f[r] = fv;
            X.rej[r] = rej;
            X.dv_set[r] = !rej && dvl[0] != unset;
            for (int m = 0; m < AST_MAX_FILTERS; m++) X.dv[r][m] = dvl[m];
        }
        __syncwarp(mask);
        if (r == 0 && gchain >= 0) {
            const BatchObj<CF>& B = objs[k];
            const FitView<CF> W = obj_view(V, B);
            bool failed = false;
            if (coop_apply<CF>(B.M, W, s, R, X, n, n_ev, &failed)) {
                nm_finish<CF>(B.M, W, s, R, failed, n_fit);
                atomicAdd(B.done, 1ull);
                n_done++;
                gchain = -1;
                R.chain = -1;
            }
        }
        __syncwarp(mask);
    }
    if (r == 0) {
        V.chain[s] = gchain;
        V.st[s] = R.st;
        V.it[s] = R.l;
        V.ev[s] = R.ev;
        if (gchain >= 0)
            for (int m = 0; m < objs[k].M.n_filters; m++) V.dv[(int64_t)m * S + s] = (double)R.dvl[m];
        if (n_done) atomicAdd(&V.ctr[1], n_done);
        if (n_ev) atomicAdd(&V.ctr[2], n_ev);
        if (n_fit) atomicAdd(&V.ctr[3], n_fit);
    }
}

// One CTA per (object, group) of gmap.
template <class CF>
__global__ void batch_group_best_kernel(const BatchObj<CF>* objs, const int2* gmap, FitView<CF> V)
{
    const int2 kg = gmap[blockIdx.x];
    const BatchObj<CF>& B = objs[kg.x];
    const ObsView o = B.L.view(B.obs, B.M.n_data);
    group_best_body<CF>(B.M, obj_view(V, B), kg.y, B.out_f, B.out_p, B.out_dv, B.fp64_result ? &o : nullptr);
}

__global__ void batch_reset_kernel(int64_t* chain, int32_t* st, int32_t* it, int32_t* ev, int64_t S)
{
    const int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (s >= S) return;
    chain[s] = -1;
    st[s] = 0;
    it[s] = 0;
    ev[s] = 0;
}

}  // namespace ast

using namespace ast;

namespace {

double now_s()
{
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

// One object of a batch, or one request of a server.
struct Entry {
    int64_t id = 0;
    ast_model model{};
    DevModel dm{};
    ObsLayout L{};
    int32_t N = 0, NF = 0;
    int64_t n_chains = 0, groups = 0;
    int32_t group_size = 0, reopt = 0, steps_cap = 0, fp64_result = 0;
    uint64_t seed = 0;
    int64_t evals_cap = 0;
    std::vector<unsigned char> img;  // host image of the observation block
    std::vector<double> x_start;     // [G][N] (reopt)
    void* dev = nullptr;
    size_t bytes = 0;
    int64_t off_obs = 0, off_xs = 0, off_cf = 0, off_cx = 0, off_cdv = 0, off_of = 0, off_op = 0, off_odv = 0;
    int64_t chain0 = -1;
    int state = 0;  // 0 queued, 1 running, 2 done, 3 cancelled
    bool cancel = false;  // ast_cancel on a running request: its chains are being dropped
    int done_slot = -1;
    std::vector<double> res_f, res_p, res_dv;
    double t_submit = 0, t_admit = 0, t_done = 0;
    double cost = 0;  // RK4 steps plus observations of one evaluation (ordering of a batch)
};

size_t entry_bytes(Entry& e, int cfb)
{
    auto al = [](int64_t v) { return (v + 255) / 256 * 256; };
    int64_t o = 0;
    e.off_obs = o; o += al(e.L.bytes);
    e.off_xs = o;  o += al(e.groups * e.N * cfb);
    e.off_cf = o;  o += al(e.n_chains * 8);
    e.off_cx = o;  o += al(e.n_chains * e.N * cfb);
    e.off_cdv = o; o += al(e.n_chains * e.NF * 8);
    e.off_of = o;  o += al(e.groups * 8);
    e.off_op = o;  o += al(e.groups * e.N * 8);
    e.off_odv = o; o += al(e.groups * e.NF * 8);
    return (size_t)o;
}

}  // namespace

// The engine shared by ast_batch and ast_server: the slot pool, the device object table and
// the entries.
struct ast_pool {
    int device = 0, sm_count = 0, precision = 0;
    bool acc = false;
    int cfb = 8;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    // slots
    int64_t n_slots = 0, S = 0;
    void* slot_base = nullptr;
    void *x = nullptr, *f = nullptr, *x0 = nullptr, *xr = nullptr, *fr = nullptr;
    uint8_t* ind = nullptr;
    int32_t *st = nullptr, *it = nullptr, *ev = nullptr;
    int64_t* chain = nullptr;
    double* dv = nullptr;
    unsigned long long* ctr = nullptr;          // [0] next chain, [1] finished, [2] evals, [3] fits
    unsigned long long* done = nullptr;         // per-entry finished chains [cap]
    void* d_objs = nullptr;                     // BatchObj<CF>[cap]
    int2* d_gmap = nullptr;                     // [gcap]
    int cap = 0, gcap = 0;
    std::vector<int> free_done;
    // launch geometry
    int tpb = 256, refill = 1, ctas = 0;
    int tile = 0;       // warp-tiled evaluation with tiles of this many observations (0: none)
    int lanes = 1;      // lanes per chain: 1, or kCoopLanes (cooperative chains, servers only)
    size_t smem = 0;    // dynamic shared memory of the launch
    // entries
    std::vector<Entry*> all;                    // by id
    std::vector<Entry*> active;                 // running, by chain0
    std::deque<Entry*> queued;
    int64_t chain_end = 0;
    size_t hbm_budget = 0, hbm_used = 0;
    bool table_dirty = true;
    double kernel_ms = 0;
    unsigned long long evals = 0, fits = 0;
};

struct ast_batch {
    ast_pool P;
    cudaGraphExec_t graph = nullptr;
    int g_tpb = 0, g_refill = 0, g_ctas = 0, g_tile = 0;
    bool ordered = false;
    bool ran = false;
};

struct ast_server {
    ast_pool P;
};

static int pool_init(ast_pool& P, int32_t device, int32_t precision, int32_t acc, int64_t n_slots, int cap)
{
    if (precision != AST_PREC_FP64 && precision != AST_PREC_MIXED)
        return ast_set_error(AST_E_INVALID, "pool: bad precision");
    int rc = set_device(device);
    if (rc) return rc;
    AST_CUDA(cudaGetDevice(&P.device));
    AST_CUDA(cudaDeviceGetAttribute(&P.sm_count, cudaDevAttrMultiProcessorCount, P.device));
    P.precision = precision;
    P.acc = acc != 0;
    P.cfb = P.acc ? 8 : 4;
    AST_CUDA(cudaStreamCreateWithFlags(&P.stream, cudaStreamNonBlocking));
    AST_CUDA(cudaEventCreate(&P.ev0));
    AST_CUDA(cudaEventCreate(&P.ev1));
    // Default: every thread the kernel keeps resident (KernShape: 3 x 128 per SM for the
    // double-float path, 256 for FP64).
    if (n_slots <= 0)
        n_slots = (int64_t)P.sm_count * (precision == AST_PREC_MIXED ? KernShape<AST_PREC_MIXED>::tpb * KernShape<AST_PREC_MIXED>::min_ctas
                                                                     : KernShape<AST_PREC_FP64>::tpb * KernShape<AST_PREC_FP64>::min_ctas);
    P.n_slots = (n_slots + 31) / 32 * 32;
    P.S = P.n_slots;
    const int64_t S = P.S;
    const int N = AST_MAX_PARAMS, NF = AST_MAX_FILTERS, cfb = P.cfb;
    auto al = [](int64_t v) { return (v + 255) / 256 * 256; };
    int64_t o = 0;
    const int64_t o_x = o; o += al(S * (N + 1) * N * cfb);
    const int64_t o_f = o; o += al(S * (N + 1) * cfb);
    const int64_t o_ind = o; o += al(S * (N + 1));
    const int64_t o_x0 = o; o += al(S * N * cfb);
    const int64_t o_xr = o; o += al(S * N * cfb);
    const int64_t o_fr = o; o += al(S * cfb);
    const int64_t o_st = o; o += al(S * 4);
    const int64_t o_it = o; o += al(S * 4);
    const int64_t o_ev = o; o += al(S * 4);
    const int64_t o_ch = o; o += al(S * 8);
    const int64_t o_dv = o; o += al(S * NF * 8);
    const int64_t o_ctr = o; o += al(8 * 8);
    const int64_t o_done = o; o += al((int64_t)cap * 8);
    const int64_t o_objs = o; o += al((int64_t)cap * (P.acc ? sizeof(BatchObj<double>) : sizeof(BatchObj<float>)));
    P.gcap = 4 * cap;
    const int64_t o_gmap = o; o += al((int64_t)P.gcap * sizeof(int2));
    if (cudaMalloc(&P.slot_base, (size_t)o) != cudaSuccess) {
        cudaGetLastError();
        return ast_set_error(AST_E_NOMEM, "pool: cudaMalloc(%lld) for %lld slots failed", (long long)o, (long long)S);
    }
    char* b = (char*)P.slot_base;
    P.x = b + o_x; P.f = b + o_f; P.ind = (uint8_t*)(b + o_ind); P.x0 = b + o_x0; P.xr = b + o_xr; P.fr = b + o_fr;
    P.st = (int32_t*)(b + o_st); P.it = (int32_t*)(b + o_it); P.ev = (int32_t*)(b + o_ev);
    P.chain = (int64_t*)(b + o_ch); P.dv = (double*)(b + o_dv); P.ctr = (unsigned long long*)(b + o_ctr);
    P.done = (unsigned long long*)(b + o_done); P.d_objs = b + o_objs; P.d_gmap = (int2*)(b + o_gmap);
    P.cap = cap;
    for (int i = cap - 1; i >= 0; i--) P.free_done.push_back(i);
    AST_CUDA(cudaMemsetAsync(P.ctr, 0, 64, P.stream));
    AST_CUDA(cudaMemsetAsync(P.done, 0, (size_t)cap * 8, P.stream));
    batch_reset_kernel<<<(unsigned)((S + 255) / 256), 256, 0, P.stream>>>(P.chain, P.st, P.it, P.ev, S);
    AST_CUDA(cudaGetLastError());
    AST_CUDA(cudaStreamSynchronize(P.stream));
    return AST_OK;
}

static void pool_free(ast_pool& P)
{
    if (P.stream) cudaStreamSynchronize(P.stream);
    for (Entry* e : P.all) {
        if (e->dev) cudaFree(e->dev);
        delete e;
    }
    P.all.clear();
    P.active.clear();
    P.queued.clear();
    if (P.slot_base) cudaFree(P.slot_base);
    if (P.ev0) cudaEventDestroy(P.ev0);
    if (P.ev1) cudaEventDestroy(P.ev1);
    if (P.stream) cudaStreamDestroy(P.stream);
    P.slot_base = nullptr;
    P.stream = nullptr;
}

// Validate and record a new object (host side only; no device memory yet).
static int pool_new_entry(ast_pool& P, const ast_model* model, const ast_obs_set* obs, const ast_fit_cfg* cfg,
                          Entry** out)
{
    if (!model || !obs || !cfg || !out) return ast_set_error(AST_E_INVALID, "batch: NULL argument");
    if (((model->flags & AST_ACC) != 0) != P.acc)
        return ast_set_error(AST_E_INVALID, "batch: every object of a batch or server must %s ACC", P.acc ? "have" : "not have");
    if (cfg->precision != P.precision) return ast_set_error(AST_E_INVALID, "batch: precision differs from the pool's");
    if (cfg->n_stages != 1) return ast_set_error(AST_E_INVALID, "batch: one stage per object (n_stages = 1)");
    if (cfg->n_chains <= 0 || cfg->group_size <= 0 || cfg->n_chains % cfg->group_size)
        return ast_set_error(AST_E_INVALID, "batch: n_chains must be a positive multiple of group_size");
    if (cfg->reopt && !cfg->params0) return ast_set_error(AST_E_INVALID, "batch: reopt needs params0");
    if (model->n_params > AST_MAX_PARAMS || obs->n_filters > AST_MAX_FILTERS || obs->n_data < 3)
        return ast_set_error(AST_E_INVALID, "batch: object sizes out of range");
    Entry* e = new Entry();
    int rc = build_dev_model(model, obs, &e->dm);
    if (rc) { delete e; return rc; }
    e->model = *model;
    e->N = model->n_params;
    e->NF = obs->n_filters;
    e->n_chains = cfg->n_chains;
    e->group_size = cfg->group_size;
    e->groups = cfg->n_chains / cfg->group_size;
    e->reopt = cfg->reopt ? 1 : 0;
    e->steps_cap = cfg->steps_cap > 0 ? cfg->steps_cap : 5000;
    e->fp64_result = (cfg->precision == AST_PREC_MIXED && cfg->fp64_result) ? 1 : 0;
    e->seed = cfg->seed;
    e->evals_cap = cfg->evals_cap;
    e->L = ObsLayout::make(obs->n_data);
    obs_image(model, obs, e->L, e->img);
    if (e->reopt) {
        // Every group starts from params0 as x (asteroid.c:640-660 with reopt).
        double x[AST_MAX_PARAMS];
        params2x<double>(e->dm, cfg->params0, x);
        e->x_start.resize((size_t)e->groups * e->N);
        for (int64_t g = 0; g < e->groups; g++)
            for (int i = 0; i < e->N; i++) e->x_start[g * e->N + i] = x[i];
    }
    e->bytes = entry_bytes(*e, P.cfb);
    // Work of one evaluation: the RK4 steps between consecutive observations (cuda.c:321) and a
    // magnitude per observation.
    e->cost = (double)obs->n_data;
    for (int i = 1; i < obs->n_data; i++)
        e->cost += (double)(int)((obs->mjd[i] - obs->mjd[i - 1]) / model->time_step) + 1.0;
    e->id = (int64_t)P.all.size();
    e->t_submit = now_s();
    P.all.push_back(e);
    *out = e;
    return AST_OK;
}

// Device memory, upload, preparation; the entry's chains start at the end of the chain space.
static int pool_admit(ast_pool& P, Entry* e)
{
    if (P.free_done.empty() || P.active.size() >= (size_t)P.cap)
        return ast_set_error(AST_E_TOO_LARGE, "batch: more than %d objects in flight", P.cap);
    if (cudaMalloc(&e->dev, e->bytes) != cudaSuccess) {
        cudaGetLastError();
        e->dev = nullptr;
        return ast_set_error(AST_E_NOMEM, "batch: cudaMalloc(%lld) for an object failed", (long long)e->bytes);
    }
    char* b = (char*)e->dev;
    AST_CUDA(cudaMemcpyAsync(b + e->off_obs, e->img.data(), e->img.size(), cudaMemcpyHostToDevice, P.stream));
    if (e->reopt) {
        if (P.acc) {
            AST_CUDA(cudaMemcpyAsync(b + e->off_xs, e->x_start.data(), e->x_start.size() * 8, cudaMemcpyHostToDevice,
                                     P.stream));
        } else {
            std::vector<float> xf(e->x_start.begin(), e->x_start.end());
            AST_CUDA(cudaMemcpyAsync(b + e->off_xs, xf.data(), xf.size() * 4, cudaMemcpyHostToDevice, P.stream));
            AST_CUDA(cudaStreamSynchronize(P.stream));
        }
    }
    int rc = launch_prep(e->dm, b + e->off_obs, e->L, e->dm.n_data, P.stream);
    if (rc) return rc;
    e->done_slot = P.free_done.back();
    P.free_done.pop_back();
    AST_CUDA(cudaMemsetAsync(P.done + e->done_slot, 0, 8, P.stream));
    e->chain0 = P.chain_end;
    P.chain_end += e->n_chains;
    e->state = 1;
    e->t_admit = now_s();
    P.hbm_used += e->bytes;
    P.active.push_back(e);
    P.table_dirty = true;
    return AST_OK;
}

template <class CF>
static BatchObj<CF> make_obj(const ast_pool& P, const Entry* e)
{
    BatchObj<CF> o;
    memset(&o, 0, sizeof(o));
    char* b = (char*)e->dev;
    o.M = e->dm;
    o.obs = b + e->off_obs;
    o.L = e->L;
    o.chain0 = e->chain0;
    o.n_chains = e->n_chains;
    o.group_size = e->group_size;
    o.reopt = e->reopt;
    o.steps_cap = e->steps_cap;
    o.fp64_result = e->fp64_result;
    o.cancelled = e->cancel ? 1 : 0;
    o.seed = e->seed;
    o.evals_cap = e->evals_cap;
    o.x_start = (CF*)(b + e->off_xs);
    o.chain_f = (double*)(b + e->off_cf);
    o.chain_x = (CF*)(b + e->off_cx);
    o.chain_dv = (double*)(b + e->off_cdv);
    o.out_f = (double*)(b + e->off_of);
    o.out_p = (double*)(b + e->off_op);
    o.out_dv = (double*)(b + e->off_odv);
    o.done = P.done + e->done_slot;
    return o;
}

template <class CF>
static int upload_table(ast_pool& P)
{
    if (!P.table_dirty) return AST_OK;
    std::vector<BatchObj<CF>> t;
    t.reserve(P.active.size());
    for (const Entry* e : P.active) t.push_back(make_obj<CF>(P, e));
    if (!t.empty())
        AST_CUDA(cudaMemcpyAsync(P.d_objs, t.data(), t.size() * sizeof(BatchObj<CF>), cudaMemcpyHostToDevice, P.stream));
    AST_CUDA(cudaStreamSynchronize(P.stream));  // t is a host temporary
    P.table_dirty = false;
    return AST_OK;
}

template <class CF>
static FitView<CF> pool_view(const ast_pool& P)
{
    FitView<CF> V;
    memset(&V, 0, sizeof(V));
    V.x = (CF*)P.x; V.f = (CF*)P.f; V.ind = P.ind; V.x0 = (CF*)P.x0; V.xr = (CF*)P.xr; V.fr = (CF*)P.fr;
    V.st = P.st; V.it = P.it; V.ev = P.ev; V.chain = P.chain; V.dv = P.dv; V.ctr = P.ctr;
    V.S = P.S;
    V.n_slots = (int64_t)P.ctas * P.tpb / P.lanes;
    V.n_chains = P.chain_end;
    V.last_stage = 1;
    return V;
}

template <class CF, int PREC>
static decltype(&batch_kernel<CF, PREC, 1>) batch_kernel_ptr(int refill)
{
    return refill == 32 ? batch_kernel<CF, PREC, 32> : batch_kernel<CF, PREC, 1>;
}

// Cooperative chains: CTA size -> CTAs (full occupancy, groups capped by the slot pool).
template <class CF, int PREC>
static int coop_geometry(ast_pool& P, int tpb)
{
    const size_t smem = (size_t)(tpb / kCoopLanes) * sizeof(CoopXchg<CF>);
    auto kern = coop_kernel<CF, PREC>;
    AST_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int occ = 0;
    AST_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, tpb, smem));
    if (occ < 1) return ast_set_error(AST_E_TOO_LARGE, "server: cooperative kernel does not fit on an SM");
    int64_t ctas = (int64_t)P.sm_count * occ;
    if (ctas * tpb > P.n_slots * kCoopLanes) ctas = P.n_slots * kCoopLanes / tpb;
    if (ctas < 1) return ast_set_error(AST_E_INVALID, "server: slot pool smaller than one CTA");
    P.tpb = tpb;
    P.refill = 1;
    P.ctas = (int)ctas;
    P.smem = smem;
    return AST_OK;
}

// The warp-tiled kernel for tiles of T observations (double-float state; ACC pools).
static decltype(&batch_tile_kernel<double, 16>) batch_tile_ptr(int T)
{
    return T == 8 ? batch_tile_kernel<double, 8> : T == 32 ? batch_tile_kernel<double, 32> : batch_tile_kernel<double, 16>;
}

// CTA size and refill mapping (and, tile > 0, the warp-tiled evaluation with tiles of that many
// observations) -> CTAs (full occupancy, capped by the slot pool).
template <class CF, int PREC>
static int pool_geometry(ast_pool& P, int tpb, int refill, int tile = 0)
{
    if (P.lanes > 1) return coop_geometry<CF, PREC>(P, 128);
    if (tpb < 32 || tpb > 256 || (tpb & 31)) return ast_set_error(AST_E_INVALID, "batch: tpb must be 32..256, x32");
    tpb = std::min(tpb, KernShape<PREC>::tpb);  // the kernel's launch bounds
    if (refill != 1 && refill != 32) return ast_set_error(AST_E_INVALID, "batch: refill must be 1 or 32");
    if (tile && tile != 8 && tile != 16 && tile != 32)
        return ast_set_error(AST_E_INVALID, "batch: tile must be 0, 8, 16 or 32");
    if (tile && (PREC != AST_PREC_MIXED || !P.acc))
        return ast_set_error(AST_E_INVALID, "batch: the warp-tiled evaluation is built for mixed-precision ACC pools");
    int occ = 0;
    size_t smem = 0;
    if (tile) {
        refill = 32;
        smem = (size_t)(tpb / 32) * tile_warp_bytes(tile);
        auto kern = batch_tile_ptr(tile);
        // Always raised to the request: without it, dynamic and static shared memory together stay
        // within 48 KB (the sin/cos table takes 4 KB of that).
        AST_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        AST_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, tpb, smem));
    } else {
        AST_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, batch_kernel_ptr<CF, PREC>(refill), tpb, 0));
    }
    if (occ < 1) return ast_set_error(AST_E_TOO_LARGE, "batch: kernel does not fit on an SM");
    int64_t ctas = (int64_t)P.sm_count * occ;
    if (ctas * tpb > P.n_slots) ctas = P.n_slots / tpb;
    if (ctas < 1) return ast_set_error(AST_E_INVALID, "batch: slot pool smaller than one CTA");
    P.tpb = tpb;
    P.refill = refill;
    P.tile = tile;
    P.smem = smem;
    P.ctas = (int)ctas;
    return AST_OK;
}

// One launch of the pool's kernel (thread per chain or warp per object, or the warp-tiled
// evaluation) on its stream.
template <class CF, int PREC>
static void launch_pool(ast_pool& P, const FitView<CF>& V, int64_t budget)
{
    if constexpr (std::is_same<CF, double>::value && PREC == AST_PREC_MIXED) {
        if (P.tile) {  // pool_geometry allows tiles for mixed-precision ACC pools only
            batch_tile_ptr(P.tile)<<<P.ctas, P.tpb, P.smem, P.stream>>>((const BatchObj<double>*)P.d_objs,
                                                                       (int)P.active.size(), V, budget);
            return;
        }
    }
    batch_kernel_ptr<CF, PREC>(P.refill)<<<P.ctas, P.tpb, 0, P.stream>>>((const BatchObj<CF>*)P.d_objs,
                                                                           (int)P.active.size(), V, budget);
}

// Per-(object, group) map of the given entries.
static int fill_gmap(ast_pool& P, const std::vector<std::pair<int, Entry*>>& which, int* n_blocks)
{
    std::vector<int2> g;
    for (const auto& kv : which)
        for (int64_t gi = 0; gi < kv.second->groups; gi++) g.push_back(int2{kv.first, (int)gi});
    if ((int)g.size() > P.gcap) return ast_set_error(AST_E_TOO_LARGE, "batch: more than %d result groups", P.gcap);
    if (!g.empty()) AST_CUDA(cudaMemcpyAsync(P.d_gmap, g.data(), g.size() * sizeof(int2), cudaMemcpyHostToDevice, P.stream));
    AST_CUDA(cudaStreamSynchronize(P.stream));
    *n_blocks = (int)g.size();
    return AST_OK;
}

static int fetch_results(ast_pool& P, Entry* e)
{
    char* b = (char*)e->dev;
    e->res_f.resize((size_t)e->groups);
    e->res_p.resize((size_t)e->groups * e->N);
    e->res_dv.resize((size_t)e->groups * e->NF);
    AST_CUDA(cudaMemcpyAsync(e->res_f.data(), b + e->off_of, e->res_f.size() * 8, cudaMemcpyDeviceToHost, P.stream));
    AST_CUDA(cudaMemcpyAsync(e->res_p.data(), b + e->off_op, e->res_p.size() * 8, cudaMemcpyDeviceToHost, P.stream));
    AST_CUDA(cudaMemcpyAsync(e->res_dv.data(), b + e->off_odv, e->res_dv.size() * 8, cudaMemcpyDeviceToHost, P.stream));
    AST_CUDA(cudaStreamSynchronize(P.stream));
    return AST_OK;
}

static int copy_out(const Entry* e, ast_fit_out* out)
{
    if (out->best_f) memcpy(out->best_f, e->res_f.data(), e->res_f.size() * 8);
    if (out->best_params) memcpy(out->best_params, e->res_p.data(), e->res_p.size() * 8);
    if (out->best_dv) memcpy(out->best_dv, e->res_dv.data(), e->res_dv.size() * 8);
    out->n_evals = 0;
    out->n_fits = e->n_chains;
    out->kernel_ms = 0;
    return AST_OK;
}

// ---------------------------------------------------------------- batch

// Before a batch's first launch: its objects take the chain index space longest evaluation
// first, so the chains that run longest start first and the launch does not end on a tail of a
// few long chains (longest-processing-time-first order).  A chain's index within its object --
// its random draws and its result -- does not change.
static void batch_order(ast_batch* B)
{
    if (B->ordered) return;
    ast_pool& P = B->P;
    std::stable_sort(P.active.begin(), P.active.end(), [](const Entry* a, const Entry* b) { return a->cost > b->cost; });
    int64_t c = 0;
    for (Entry* e : P.active) {
        e->chain0 = c;
        c += e->n_chains;
    }
    P.table_dirty = true;
    B->ordered = true;
}

template <class CF, int PREC>
static int batch_capture(ast_batch* B)
{
    ast_pool& P = B->P;
    if (B->graph && B->g_tpb == P.tpb && B->g_refill == P.refill && B->g_ctas == P.ctas && B->g_tile == P.tile)
        return AST_OK;
    if (B->graph) { cudaGraphExecDestroy(B->graph); B->graph = nullptr; }
    std::vector<std::pair<int, Entry*>> all;
    for (size_t k = 0; k < P.active.size(); k++) all.push_back({(int)k, P.active[k]});
    int n_blocks = 0;
    int rc = fill_gmap(P, all, &n_blocks);
    if (rc) return rc;
    if ((rc = upload_table<CF>(P))) return rc;
    const FitView<CF> V = pool_view<CF>(P);
    cudaGraph_t g = nullptr;
    AST_CUDA(cudaStreamBeginCapture(P.stream, cudaStreamCaptureModeThreadLocal));
    batch_reset_kernel<<<(unsigned)((P.S + 255) / 256), 256, 0, P.stream>>>(P.chain, P.st, P.it, P.ev, P.S);
    cudaMemsetAsync(P.ctr, 0, 64, P.stream);
    cudaMemsetAsync(P.done, 0, (size_t)P.cap * 8, P.stream);
    launch_pool<CF, PREC>(P, V, INT64_MAX);
    batch_group_best_kernel<CF><<<(unsigned)n_blocks, 256, 0, P.stream>>>((const BatchObj<CF>*)P.d_objs, P.d_gmap, V);
    const cudaError_t ec = cudaStreamEndCapture(P.stream, &g);
    if (ec != cudaSuccess) return ast_set_error(AST_E_CUDA, "batch: graph capture: %s", cudaGetErrorString(ec));
    const cudaError_t ei = cudaGraphInstantiate(&B->graph, g, 0);
    cudaGraphDestroy(g);
    if (ei != cudaSuccess) return ast_set_error(AST_E_CUDA, "batch: graph instantiate: %s", cudaGetErrorString(ei));
    B->g_tpb = P.tpb;
    B->g_refill = P.refill;
    B->g_ctas = P.ctas;
    B->g_tile = P.tile;
    return AST_OK;
}

template <class CF, int PREC>
static int batch_run_t(ast_batch* B, const ast_batch_launch* tune, double* kernel_ms)
{
    ast_pool& P = B->P;
    batch_order(B);
    int rc;
    if (tune) {
        if ((rc = pool_geometry<CF, PREC>(P, tune->tpb, tune->refill, tune->tile))) return rc;
    } else if (!P.ctas) {
        if ((rc = pool_geometry<CF, PREC>(P, 256, 1))) return rc;
    }
    if ((rc = batch_capture<CF, PREC>(B))) return rc;
    AST_CUDA(cudaEventRecord(P.ev0, P.stream));
    AST_CUDA(cudaGraphLaunch(B->graph, P.stream));
    AST_CUDA(cudaEventRecord(P.ev1, P.stream));
    unsigned long long h[8];
    AST_CUDA(cudaMemcpyAsync(h, P.ctr, sizeof(h), cudaMemcpyDeviceToHost, P.stream));
    AST_CUDA(cudaStreamSynchronize(P.stream));
    float ms = 0;
    AST_CUDA(cudaEventElapsedTime(&ms, P.ev0, P.ev1));
    P.kernel_ms = ms;
    P.evals = h[2];
    P.fits = h[3];
    if (kernel_ms) *kernel_ms = ms;
    if (h[1] < (unsigned long long)P.chain_end)
        return ast_set_error(AST_E_CUDA, "batch: %llu of %lld chains finished", h[1], (long long)P.chain_end);
    for (Entry* e : P.active) {
        if ((rc = fetch_results(P, e))) return rc;
        e->state = 2;
    }
    B->ran = true;
    return AST_OK;
}

// One bounded launch from a fresh slot state: evaluations per second of this geometry.
template <class CF, int PREC>
static int batch_probe(ast_batch* B, int tpb, int refill, int tile, int64_t evals_per_slot, double* rate)
{
    ast_pool& P = B->P;
    int rc = pool_geometry<CF, PREC>(P, tpb, refill, tile);
    if (rc) return rc;
    if ((rc = upload_table<CF>(P))) return rc;
    const FitView<CF> V = pool_view<CF>(P);
    batch_reset_kernel<<<(unsigned)((P.S + 255) / 256), 256, 0, P.stream>>>(P.chain, P.st, P.it, P.ev, P.S);
    AST_CUDA(cudaMemsetAsync(P.ctr, 0, 64, P.stream));
    AST_CUDA(cudaMemsetAsync(P.done, 0, (size_t)P.cap * 8, P.stream));
    // A first launch takes every slot through its start-up; the second is timed.
    launch_pool<CF, PREC>(P, V, evals_per_slot);
    unsigned long long h0[8], h1[8];
    AST_CUDA(cudaMemcpyAsync(h0, P.ctr, sizeof(h0), cudaMemcpyDeviceToHost, P.stream));
    AST_CUDA(cudaEventRecord(P.ev0, P.stream));
    launch_pool<CF, PREC>(P, V, evals_per_slot);
    AST_CUDA(cudaGetLastError());
    AST_CUDA(cudaEventRecord(P.ev1, P.stream));
    AST_CUDA(cudaMemcpyAsync(h1, P.ctr, sizeof(h1), cudaMemcpyDeviceToHost, P.stream));
    AST_CUDA(cudaStreamSynchronize(P.stream));
    float ms = 0;
    AST_CUDA(cudaEventElapsedTime(&ms, P.ev0, P.ev1));
    *rate = ms > 0 ? (double)(h1[2] - h0[2]) / (ms * 1e-3) : 0.0;
    return AST_OK;
}

template <class CF, int PREC>
static int batch_tune_t(ast_batch* B, int64_t evals_per_slot, ast_batch_launch* best)
{
    batch_order(B);
    const int tpbs[3] = {64, 128, 256};
    const int refills[2] = {1, 32};
    const int tiles[3] = {8, 16, 32};
    double best_rate = -1;
    ast_batch_launch bt{256, 1, 0, 0.0, 0};
    auto probe = [&](int t, int r, int tile) -> int {
        double rate = 0;
        int rc = batch_probe<CF, PREC>(B, t, r, tile, evals_per_slot, &rate);
        if (rc) return rc;
        if (rate > best_rate) {
            best_rate = rate;
            bt.tpb = t;
            bt.refill = r;
            bt.tile = tile;
        }
        return AST_OK;
    };
    // Thread per model (refill 1) and warp per object (refill 32), each lane its own chain's
    // whole light curve; then, for mixed-precision ACC pools, the warp-tiled evaluation.
    for (int r : refills)
        for (int t : tpbs) {
            if (t > KernShape<PREC>::tpb) continue;
            if (int rc = probe(t, r, 0)) return rc;
        }
    if (PREC == AST_PREC_MIXED && B->P.acc)
        for (int tile : tiles)
            for (int t : tpbs) {
                if (t > KernShape<PREC>::tpb) continue;
                if (int rc = probe(t, 32, tile)) return rc;
            }
    int rc = pool_geometry<CF, PREC>(B->P, bt.tpb, bt.refill, bt.tile);
    if (rc) return rc;
    // Back to the untouched state: the probes ran chains that the batch will run again.
    ast_pool& P = B->P;
    batch_reset_kernel<<<(unsigned)((P.S + 255) / 256), 256, 0, P.stream>>>(P.chain, P.st, P.it, P.ev, P.S);
    AST_CUDA(cudaMemsetAsync(P.ctr, 0, 64, P.stream));
    AST_CUDA(cudaMemsetAsync(P.done, 0, (size_t)P.cap * 8, P.stream));
    AST_CUDA(cudaStreamSynchronize(P.stream));
    bt.ctas = B->P.ctas;
    bt.evals_per_s = best_rate;
    if (best) *best = bt;
    return AST_OK;
}

// One bounded launch from the batch's current state (no graph): every slot performs at most
// evals_per_slot evaluations; when the last chain has finished, the group argmins run and the
// results come back.
template <class CF, int PREC>
static int batch_step_t(ast_batch* B, int64_t evals_per_slot, int32_t* done, double* kernel_ms)
{
    ast_pool& P = B->P;
    batch_order(B);
    int rc;
    if (!P.ctas && (rc = pool_geometry<CF, PREC>(P, 256, 1))) return rc;
    if ((rc = upload_table<CF>(P))) return rc;
    const FitView<CF> V = pool_view<CF>(P);
    AST_CUDA(cudaEventRecord(P.ev0, P.stream));
    launch_pool<CF, PREC>(P, V, evals_per_slot);
    AST_CUDA(cudaGetLastError());
    AST_CUDA(cudaEventRecord(P.ev1, P.stream));
    unsigned long long h[8];
    AST_CUDA(cudaMemcpyAsync(h, P.ctr, sizeof(h), cudaMemcpyDeviceToHost, P.stream));
    AST_CUDA(cudaStreamSynchronize(P.stream));
    float ms = 0;
    AST_CUDA(cudaEventElapsedTime(&ms, P.ev0, P.ev1));
    P.kernel_ms += ms;
    P.evals = h[2];
    P.fits = h[3];
    if (kernel_ms) *kernel_ms = ms;
    *done = h[1] >= (unsigned long long)P.chain_end;
    if (*done) {
        std::vector<std::pair<int, Entry*>> all;
        for (size_t k = 0; k < P.active.size(); k++) all.push_back({(int)k, P.active[k]});
        int n_blocks = 0;
        if ((rc = fill_gmap(P, all, &n_blocks))) return rc;
        batch_group_best_kernel<CF><<<(unsigned)n_blocks, 256, 0, P.stream>>>((const BatchObj<CF>*)P.d_objs, P.d_gmap, V);
        AST_CUDA(cudaGetLastError());
        for (Entry* e : P.active) {
            if ((rc = fetch_results(P, e))) return rc;
            e->state = 2;
        }
        B->ran = true;
    }
    return AST_OK;
}

#define AST_DISPATCH(P, fn, ...)                                                              \
    ((P).acc ? ((P).precision == AST_PREC_FP64 ? fn<double, AST_PREC_FP64>(__VA_ARGS__)       \
                                               : fn<double, AST_PREC_MIXED>(__VA_ARGS__))     \
             : ((P).precision == AST_PREC_FP64 ? fn<float, AST_PREC_FP64>(__VA_ARGS__)        \
                                               : fn<float, AST_PREC_MIXED>(__VA_ARGS__)))

extern "C" int ast_batch_create(int32_t device, int32_t precision, int32_t acc, int64_t n_slots, ast_batch** out)
{
    if (!out) return ast_set_error(AST_E_INVALID, "ast_batch_create: NULL argument");
    *out = nullptr;
    ast_batch* B = new ast_batch();
    int rc = pool_init(B->P, device, precision, acc, n_slots, 4096);
    if (rc) { pool_free(B->P); delete B; return rc; }
    *out = B;
    return AST_OK;
}

extern "C" int ast_batch_add(ast_batch* B, const ast_model* model, const ast_obs_set* obs, const ast_fit_cfg* cfg,
                             int32_t* index)
{
    if (!B) return ast_set_error(AST_E_INVALID, "ast_batch_add: NULL batch");
    if (B->ran || B->graph) return ast_set_error(AST_E_INVALID, "ast_batch_add: the batch has already run");
    int rc = set_device(B->P.device);
    if (rc) return rc;
    Entry* e = nullptr;
    if ((rc = pool_new_entry(B->P, model, obs, cfg, &e))) return rc;
    if ((rc = pool_admit(B->P, e))) return rc;
    AST_CUDA(cudaStreamSynchronize(B->P.stream));
    if (index) *index = (int32_t)e->id;
    return AST_OK;
}

extern "C" int ast_batch_tune(ast_batch* B, int64_t evals_per_slot, ast_batch_launch* best)
{
    if (!B || B->P.active.empty()) return ast_set_error(AST_E_INVALID, "ast_batch_tune: empty batch");
    if (B->ran) return ast_set_error(AST_E_INVALID, "ast_batch_tune: the batch has finished");
    int rc = set_device(B->P.device);
    if (rc) return rc;
    if (evals_per_slot <= 0) evals_per_slot = 4;
    return AST_DISPATCH(B->P, batch_tune_t, B, evals_per_slot, best);
}

extern "C" int ast_batch_run(ast_batch* B, const ast_batch_launch* tune, double* kernel_ms)
{
    if (!B || B->P.active.empty()) return ast_set_error(AST_E_INVALID, "ast_batch_run: empty batch");
    int rc = set_device(B->P.device);
    if (rc) return rc;
    return AST_DISPATCH(B->P, batch_run_t, B, tune, kernel_ms);
}

extern "C" int ast_batch_step(ast_batch* B, int64_t evals_per_slot, int32_t* done, double* kernel_ms)
{
    if (!B || !done || B->P.active.empty()) return ast_set_error(AST_E_INVALID, "ast_batch_step: bad argument");
    if (B->ran) return ast_set_error(AST_E_INVALID, "ast_batch_step: the batch has finished");
    int rc = set_device(B->P.device);
    if (rc) return rc;
    if (evals_per_slot <= 0) evals_per_slot = INT64_MAX;
    return AST_DISPATCH(B->P, batch_step_t, B, evals_per_slot, done, kernel_ms);
}

extern "C" int ast_batch_result(ast_batch* B, int32_t index, ast_fit_out* out)
{
    if (!B || !out || index < 0 || index >= (int32_t)B->P.all.size())
        return ast_set_error(AST_E_INVALID, "ast_batch_result: bad argument");
    const Entry* e = B->P.all[(size_t)index];
    if (e->state != 2) return ast_set_error(AST_E_INVALID, "ast_batch_result: the batch has not run");
    return copy_out(e, out);
}

template <class CF, int PREC>
static int batch_set_geometry_t(ast_batch* B, const ast_batch_launch* g)
{
    return pool_geometry<CF, PREC>(B->P, g->tpb, g->refill, g->tile);
}

extern "C" int ast_batch_set_geometry(ast_batch* B, const ast_batch_launch* g)
{
    if (!B || !g) return ast_set_error(AST_E_INVALID, "ast_batch_set_geometry: NULL argument");
    if (B->ran) return ast_set_error(AST_E_INVALID, "ast_batch_set_geometry: the batch has finished");
    int rc = set_device(B->P.device);
    if (rc) return rc;
    return AST_DISPATCH(B->P, batch_set_geometry_t, B, g);
}

extern "C" int ast_batch_geometry(ast_batch* B, ast_batch_launch* out)
{
    if (!B || !out) return ast_set_error(AST_E_INVALID, "ast_batch_geometry: NULL argument");
    out->tpb = B->P.tpb;
    out->refill = B->P.refill;
    out->ctas = B->P.ctas;
    out->tile = B->P.tile;
    out->evals_per_s = 0;
    return AST_OK;
}

extern "C" int ast_batch_counters(ast_batch* B, int64_t* n_evals, int64_t* n_fits, int32_t* tpb, int32_t* refill,
                                  int32_t* ctas)
{
    if (!B) return ast_set_error(AST_E_INVALID, "ast_batch_counters: NULL batch");
    if (n_evals) *n_evals = (int64_t)B->P.evals;
    if (n_fits) *n_fits = (int64_t)B->P.fits;
    if (tpb) *tpb = B->P.tpb;
    if (refill) *refill = B->P.refill;
    if (ctas) *ctas = B->P.ctas;
    return AST_OK;
}

extern "C" void ast_batch_destroy(ast_batch* B)
{
    if (!B) return;
    set_device(B->P.device);
    if (B->graph) cudaGraphExecDestroy(B->graph);
    pool_free(B->P);
    delete B;
}

// ---------------------------------------------------------------- serving

extern "C" int ast_server_create(int32_t device, int32_t precision, int32_t acc, int64_t n_slots,
                                 int64_t hbm_budget_bytes, ast_server** out)
{
    if (!out) return ast_set_error(AST_E_INVALID, "ast_server_create: NULL argument");
    *out = nullptr;
    ast_server* V = new ast_server();
    int rc = pool_init(V->P, device, precision, acc, n_slots, 4096);
    if (rc) { pool_free(V->P); delete V; return rc; }
    V->P.hbm_budget = hbm_budget_bytes > 0 ? (size_t)hbm_budget_bytes : (size_t)150 << 30;
    *out = V;
    return AST_OK;
}

extern "C" int ast_server_set_lanes(ast_server* V, int32_t lanes_per_chain)
{
    if (!V) return ast_set_error(AST_E_INVALID, "ast_server_set_lanes: NULL server");
    if (lanes_per_chain != 1 && lanes_per_chain != kCoopLanes)
        return ast_set_error(AST_E_INVALID, "ast_server_set_lanes: lanes per chain must be 1 or %d", kCoopLanes);
    if (!V->P.active.empty() || V->P.evals)
        return ast_set_error(AST_E_INVALID, "ast_server_set_lanes: the server has already run requests");
    V->P.lanes = lanes_per_chain;
    V->P.ctas = 0;  // the geometry is chosen again at the next step
    return AST_OK;
}

extern "C" int ast_submit(ast_server* V, const ast_model* model, const ast_obs_set* obs, const ast_fit_cfg* cfg,
                          int64_t* request)
{
    if (!V) return ast_set_error(AST_E_INVALID, "ast_submit: NULL server");
    Entry* e = nullptr;
    int rc = pool_new_entry(V->P, model, obs, cfg, &e);
    if (rc) return rc;
    if (e->bytes > V->P.hbm_budget)
        return ast_set_error(AST_E_TOO_LARGE, "ast_submit: the request needs %lld bytes, the budget is %lld",
                             (long long)e->bytes, (long long)V->P.hbm_budget);
    V->P.queued.push_back(e);
    if (request) *request = e->id;
    return AST_OK;
}

template <class CF, int PREC>
static int server_step_t(ast_server* V, int64_t evals_per_slot, int32_t* n_running, int32_t* n_queued)
{
    ast_pool& P = V->P;
    int rc;
    // Admission in arrival order while the HBM budget (and the object table) allow.
    while (!P.queued.empty()) {
        Entry* e = P.queued.front();
        if (P.hbm_used + e->bytes > P.hbm_budget || P.free_done.empty()) break;
        if ((rc = pool_admit(P, e))) return rc;
        P.queued.pop_front();
    }
    if (!P.ctas && (rc = pool_geometry<CF, PREC>(P, 256, 1))) return rc;
    if (!P.active.empty()) {
        if ((rc = upload_table<CF>(P))) return rc;
        const FitView<CF> W = pool_view<CF>(P);
        AST_CUDA(cudaEventRecord(P.ev0, P.stream));
        if (P.lanes > 1)
            coop_kernel<CF, PREC><<<P.ctas, P.tpb, P.smem, P.stream>>>((const BatchObj<CF>*)P.d_objs,
                                                                       (int)P.active.size(), W, evals_per_slot);
        else
            batch_kernel_ptr<CF, PREC>(P.refill)<<<P.ctas, P.tpb, 0, P.stream>>>(
                (const BatchObj<CF>*)P.d_objs, (int)P.active.size(), W, evals_per_slot);
        AST_CUDA(cudaGetLastError());
        AST_CUDA(cudaEventRecord(P.ev1, P.stream));
        unsigned long long h[8];
        std::vector<unsigned long long> dn((size_t)P.cap);
        AST_CUDA(cudaMemcpyAsync(h, P.ctr, sizeof(h), cudaMemcpyDeviceToHost, P.stream));
        AST_CUDA(cudaMemcpyAsync(dn.data(), P.done, dn.size() * 8, cudaMemcpyDeviceToHost, P.stream));
        AST_CUDA(cudaStreamSynchronize(P.stream));
        float ms = 0;
        AST_CUDA(cudaEventElapsedTime(&ms, P.ev0, P.ev1));
        P.kernel_ms += ms;
        P.evals = h[2];
        P.fits = h[3];
        // Pulls past the end of the chain space are void: the next admitted object starts there.
        if (h[0] > (unsigned long long)P.chain_end) {
            const unsigned long long e0 = (unsigned long long)P.chain_end;
            AST_CUDA(cudaMemcpyAsync(P.ctr, &e0, 8, cudaMemcpyHostToDevice, P.stream));
            AST_CUDA(cudaStreamSynchronize(P.stream));
        }
        // Retire the objects whose chains have all finished (or, cancelled, have all been dropped).
        std::vector<std::pair<int, Entry*>> fin, gone;
        for (size_t k = 0; k < P.active.size(); k++) {
            Entry* e = P.active[k];
            if (dn[(size_t)e->done_slot] >= (unsigned long long)e->n_chains) (e->cancel ? gone : fin).push_back({(int)k, e});
        }
        if (!fin.empty() || !gone.empty()) {
            int n_blocks = 0;
            if ((rc = fill_gmap(P, fin, &n_blocks))) return rc;
            if (n_blocks) {
                batch_group_best_kernel<CF><<<(unsigned)n_blocks, 256, 0, P.stream>>>((const BatchObj<CF>*)P.d_objs,
                                                                                     P.d_gmap, W);
                AST_CUDA(cudaGetLastError());
            }
            for (auto& kv : fin)
                if ((rc = fetch_results(P, kv.second))) return rc;
            AST_CUDA(cudaStreamSynchronize(P.stream));
            for (auto* list : {&fin, &gone})
                for (auto& kv : *list) {
                    Entry* e = kv.second;
                    cudaFree(e->dev);
                    e->dev = nullptr;
                    P.hbm_used -= e->bytes;
                    P.free_done.push_back(e->done_slot);
                    e->state = e->cancel ? 3 : 2;
                    e->t_done = now_s();
                }
            std::vector<Entry*> keep;
            for (Entry* e : P.active)
                if (e->state == 1) keep.push_back(e);
            P.active.swap(keep);
            P.table_dirty = true;
            // Admit into the memory just freed.
            while (!P.queued.empty()) {
                Entry* e = P.queued.front();
                if (P.hbm_used + e->bytes > P.hbm_budget || P.free_done.empty()) break;
                if ((rc = pool_admit(P, e))) return rc;
                P.queued.pop_front();
            }
        }
    }
    if (n_running) *n_running = (int32_t)P.active.size();
    if (n_queued) *n_queued = (int32_t)P.queued.size();
    return AST_OK;
}

extern "C" int ast_server_step(ast_server* V, int64_t evals_per_slot, int32_t* n_running, int32_t* n_queued)
{
    if (!V) return ast_set_error(AST_E_INVALID, "ast_server_step: NULL server");
    int rc = set_device(V->P.device);
    if (rc) return rc;
    if (evals_per_slot <= 0) evals_per_slot = 16;
    return AST_DISPATCH(V->P, server_step_t, V, evals_per_slot, n_running, n_queued);
}

extern "C" int ast_cancel(ast_server* V, int64_t request)
{
    if (!V || request < 0 || request >= (int64_t)V->P.all.size())
        return ast_set_error(AST_E_INVALID, "ast_cancel: bad request");
    Entry* e = V->P.all[(size_t)request];
    if (e->state == 2) return 1;                         // finished: the result stays available
    if (e->state == 3 || e->cancel) return AST_OK;       // already cancelled
    if (e->state == 0) {                                 // queued: no device memory yet
        auto& q = V->P.queued;
        q.erase(std::remove(q.begin(), q.end(), e), q.end());
        e->state = 3;
        e->t_done = now_s();
        return AST_OK;
    }
    // Running: the next ast_server_step drops its chains; once every chain is accounted for, the
    // request retires without results and its memory returns to the budget.
    e->cancel = true;
    V->P.table_dirty = true;
    return AST_OK;
}

extern "C" int ast_poll(ast_server* V, int64_t request, ast_fit_out* out, double* latency_s)
{
    if (!V || request < 0 || request >= (int64_t)V->P.all.size())
        return ast_set_error(AST_E_INVALID, "ast_poll: bad request");
    const Entry* e = V->P.all[(size_t)request];
    if (e->state == 3) return ast_set_error(AST_E_CANCELLED, "ast_poll: request %lld was cancelled", (long long)request);
    if (e->state != 2) return 0;
    if (out) copy_out(e, out);
    if (latency_s) *latency_s = e->t_done - e->t_submit;
    return 1;
}

extern "C" int ast_server_stats(ast_server* V, int64_t* n_evals, double* kernel_ms, int64_t* hbm_used,
                                int64_t* hbm_budget)
{
    if (!V) return ast_set_error(AST_E_INVALID, "ast_server_stats: NULL server");
    if (n_evals) *n_evals = (int64_t)V->P.evals;
    if (kernel_ms) *kernel_ms = V->P.kernel_ms;
    if (hbm_used) *hbm_used = (int64_t)V->P.hbm_used;
    if (hbm_budget) *hbm_budget = (int64_t)V->P.hbm_budget;
    return AST_OK;
}

extern "C" int64_t ast_request_bytes(ast_server* V, int64_t request)
{
    if (!V || request < 0 || request >= (int64_t)V->P.all.size()) return -1;
    return (int64_t)V->P.all[(size_t)request]->bytes;
}

extern "C" void ast_server_destroy(ast_server* V)
{
    if (!V) return;
    set_device(V->P.device);
    pool_free(V->P);
    delete V;
}
