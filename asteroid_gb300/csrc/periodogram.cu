// periodogram.cu -- the periodogram of model minima printed by -plot mode (minima(),
// misc.c:65-276 of the reference, default build: no PARABOLIC_MAX, no MINIMA_SPLINE).
//
// The reference takes the brightness minima of the model curve on the plot grid, forms the
// N(N-1)/2 intervals dt between every two of them, and for each of NN = 10000 trial frequencies
// fr counts the intervals with |dt/(1/fr) - int(dt/(1/fr) + 0.5)| < 0.1 (misc.c:140-166).  That
// count is the whole cost: NN x N(N-1)/2 tests, 1.2e9 for 500 minima and up to 5e11 at the
// reference's cap of 10000 minima, run there on one host core.
//
// The intervals are first reduced to their distinct values with multiplicities (pair_hash_kernel,
// compact_kernel): a count depends on an interval's value only, and the minima of a curve on the
// evenly spaced plot grid are separated by few distinct intervals.  Each distinct interval is
// tested once and counted with its multiplicity.
//
// The count is one kernel on the FP32 pipe.  Each thread holds kFreqs frequencies as
// double-float pairs; the intervals stream through shared memory, also as double-float pairs;
// each test forms x = dt * fr as a double-float product (relative error ~2^-45), rounds its
// high word to the nearest integer with the 1.5*2^23 addition, and takes the distance
// |x_hi - r + x_lo| (x_hi - r is exact).  That distance is within kMarginBase + 1e-13 x of the
// reference's, so every test farther than that from the 0.1 threshold is decided in float;
// the few closer ones (a fraction of about 4e-7) are redone in FP64 exactly as the reference
// writes them (dt / dt1 and int(x + 0.5) with dt1 = 1/fr), so every count is the reference's
// bit for bit.  Counts are integers: the order in which threads add them is immaterial.  The
// normalisation by mean and standard deviation and the cluster search stay on the host, in the
// reference's order of operations (compiled without floating-point contraction).
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>
#include <string.h>
#include <algorithm>
#include <vector>

#include "asteroid_gb300.h"
#include "engine.cuh"

namespace ast {
namespace {

constexpr int kBins = AST_MINIMA_BINS;
constexpr int kPeriodTpb = 256;
constexpr int kFreqs = 8;                       // frequencies per thread
constexpr int kFreqTile = kPeriodTpb * kFreqs;  // frequencies per CTA
constexpr int kChunk = 2048;                    // intervals per shared-memory pass (16 KB)
constexpr float kMarginBase = 1e-7f;            // rounding of x_hi - r + x_lo (<= 2^-25) and 0.1f vs 0.1
// Periodogram constants of misc.c:131-135.
constexpr double kSgm = 0.1, kDt0 = 1.0 / 24.0, kDt2 = 80.0 / 24.0, kS0 = 3;

// Intervals between every two minima (misc.c:106-121) go straight into a hash table of distinct
// values with their multiplicities: a count depends on an interval's value only, and on a plot
// grid the N(N-1)/2 intervals take far fewer distinct values (71 093 of 11 560 836 for 4 809
// minima on 20 000 points).  Open addressing with linear probing over a power-of-two table of at
// least twice the intervals; the key is the double's bit pattern (intervals are positive, so a
// key is never 0, the empty mark); a slot's key changes once, from 0, so a plain read that finds
// the key needs no compare-and-swap.  The mixer is splitmix64's finaliser (Steele, Lea and Flood,
// OOPSLA 2014).
__device__ __forceinline__ uint64_t mix64(uint64_t z)
{
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
}

// One CTA per first minimum i: the intervals tm[j] - tm[i], j > i, into the table.
__global__ void pair_hash_kernel(const double* __restrict__ tm, int n, unsigned long long* keys,
                                 unsigned int* mult, uint64_t mask, unsigned int* err)
{
    const int i = blockIdx.x;
    if (i >= n - 1) return;
    const double ti = tm[i];
    for (int j = i + 1 + threadIdx.x; j < n; j += blockDim.x) {
        const unsigned long long key = (unsigned long long)__double_as_longlong(tm[j] - ti);
        uint64_t h = mix64(key) & mask;
        bool done = false;
        for (uint64_t probe = 0; probe <= mask; probe++) {
            unsigned long long cur = __ldcg(&keys[h]);
            if (cur == 0) cur = atomicCAS(&keys[h], 0ull, key);
            if (cur == 0 || cur == key) {
                atomicAdd(&mult[h], 1u);
                done = true;
                break;
            }
            h = (h + 1) & mask;
        }
        if (!done) atomicExch(err, 1u);  // a full table: impossible at twice the intervals
    }
}

// The distinct intervals and their multiplicities, packed (in no particular order).
__global__ void compact_kernel(const unsigned long long* __restrict__ keys, const unsigned int* __restrict__ mult,
                               uint64_t size, double* __restrict__ udt, unsigned int* __restrict__ uw,
                               unsigned int* n_unique)
{
    const unsigned lane = threadIdx.x & 31;
    for (uint64_t base = (uint64_t)blockIdx.x * blockDim.x; base < size; base += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t k = base + threadIdx.x;
        const unsigned long long key = k < size ? keys[k] : 0ull;
        const unsigned ballot = __ballot_sync(0xffffffffu, key != 0ull);
        if (!ballot) continue;
        unsigned first = 0;
        if (lane == 0) first = atomicAdd(n_unique, (unsigned)__popc(ballot));
        first = __shfl_sync(0xffffffffu, first, 0);
        if (key != 0ull) {
            const unsigned idx = first + __popc(ballot & ((1u << lane) - 1u));
            udt[idx] = __longlong_as_double((long long)key);
            uw[idx] = mult[k];
        }
    }
}

__device__ __forceinline__ float2 split_df(double v)
{
    const float hi = __double2float_rn(v);
    return make_float2(hi, __double2float_rn(v - (double)hi));
}

constexpr float kRound = 12582912.0f;  // 1.5 * 2^23: x + kRound - kRound is x rounded to an integer

// The decision for one interval and frequency when the fast test is too close to call:
// the double-float distance (error < kMarginBase + 1e-13 x), and where even that is too close,
// the reference's own FP64 test (misc.c:145).  Returns 1 if the interval counts.
__device__ __noinline__ unsigned int precise_test(float dth, float dtl, float fh, float fl, double dt, double dt1,
                                                  float margin)
{
    const float xh = __fmul_rn(dth, fh);
    float xl = __fmaf_rn(dth, fh, -xh);
    xl = __fmaf_rn(dth, fl, xl);
    xl = __fmaf_rn(dtl, fh, xl);
    const float r = __fadd_rn(__fadd_rn(xh, kRound), -kRound);
    const float dd = fabsf(__fadd_rn(__fadd_rn(xh, -r), xl));
    if (fabsf(__fadd_rn(dd, -0.1f)) > margin) return dd < 0.1f ? 1u : 0u;
    const double x = dt / dt1;
    const double dv = fabs(x - (double)(int)(x + 0.5));
    return dv < kSgm ? 1u : 0u;
}

// counts[f] += number of intervals in this CTA's slice within sgm of a whole number of periods.
// grid: (frequency tiles, interval slices).
//
// Fast test of interval dt_h against frequency f_h, four FP32 instructions: y = fma(dt_h, f_h,
// 1.5*2^23) rounds the exact product p to the nearest integer r; d = fma(dt_h, f_h, -r) is p - r
// with one rounding; a = |d| - 0.1.  The interval counts when a < 0 (its sign bit is added).  The
// error of a against the reference's |x - int(x + 0.5)| - 0.1 is below 1.2e-7 x + 3.2e-8 (the
// float rounding of dt and fr, then two roundings of at most 2^-26); each interval's bound
// dt_h * (2.4e-7 max f_h) + 1e-7 covers twice that.  The smallest |a| of the thread's frequencies is
// kept, and only when it is within the bound does the warp take the precise test, for the
// frequencies that need it, correcting the count by the difference of the two decisions.
__device__ __forceinline__ void test_interval(float dth, int w, int j, const float* s_dtl, int64_t base,
                                              const double* __restrict__ dt, const double* __restrict__ dt1, int f0,
                                              int nn, const float (&fh)[kFreqs], const float (&fl)[kFreqs], float thr,
                                              float margin, int (&cnt)[kFreqs])
{
    float a[kFreqs];
    float amin = 1.0f;
#pragma unroll
    for (int k = 0; k < kFreqs; k++) {
        const float y = __fmaf_rn(dth, fh[k], kRound);
        const float r = __fadd_rn(y, -kRound);
        const float d = __fmaf_rn(dth, fh[k], -r);
        a[k] = __fadd_rn(fabsf(d), -0.1f);
        cnt[k] += (int)(__float_as_uint(a[k]) >> 31) * w;
        amin = fminf(amin, fabsf(a[k]));
    }
    const float bound = __fmaf_rn(dth, thr, kMarginBase);
    if (amin <= bound) {
        const float dtl = s_dtl[j];
        const double dtd = dt[base + j];
#pragma unroll
        for (int k = 0; k < kFreqs; k++)
            if (fabsf(a[k]) <= bound && f0 + k < nn) {
                const int fast = (int)(__float_as_uint(a[k]) >> 31);
                cnt[k] += ((int)precise_test(dth, dtl, fh[k], fl[k], dtd, dt1[f0 + k], margin) - fast) * w;
            }
    }
}

__global__ void __launch_bounds__(kPeriodTpb) interval_count_kernel(const double* __restrict__ dt,
                                                                     const unsigned int* __restrict__ wt, int64_t m,
                                                                     int64_t per_slice, const double* __restrict__ fr,
                                                                     const double* __restrict__ dt1, int nn,
                                                                     float margin, unsigned int* __restrict__ counts)
{
    __shared__ __align__(16) float s_dth[kChunk];
    __shared__ float s_dtl[kChunk];
    __shared__ __align__(16) int s_w[kChunk];
    const int f0 = blockIdx.x * kFreqTile + threadIdx.x * kFreqs;
    float fh[kFreqs], fl[kFreqs];
    int cnt[kFreqs];
    float fmax = 0.0f;
#pragma unroll
    for (int k = 0; k < kFreqs; k++) {
        const float2 f = f0 + k < nn ? split_df(fr[f0 + k]) : make_float2(0.f, 0.f);
        fh[k] = f.x;
        fl[k] = f.y;
        cnt[k] = 0;
        fmax = fmaxf(fmax, f.x);
    }
    const float thr = fmax * 2.4e-7f;
    const int64_t p0 = (int64_t)blockIdx.y * per_slice;
    const int64_t p1 = min(m, p0 + per_slice);
    for (int64_t base = p0; base < p1; base += kChunk) {
        const int n = (int)min((int64_t)kChunk, p1 - base);
        __syncthreads();
        for (int j = threadIdx.x; j < n; j += kPeriodTpb) {
            const float2 d = split_df(dt[base + j]);
            s_dth[j] = d.x;
            s_dtl[j] = d.y;
            s_w[j] = (int)wt[base + j];
        }
        __syncthreads();
        const int n4 = n & ~3;
        for (int j = 0; j < n4; j += 4) {
            const float4 d4 = *reinterpret_cast<const float4*>(&s_dth[j]);
            const int4 w4 = *reinterpret_cast<const int4*>(&s_w[j]);
            test_interval(d4.x, w4.x, j, s_dtl, base, dt, dt1, f0, nn, fh, fl, thr, margin, cnt);
            test_interval(d4.y, w4.y, j + 1, s_dtl, base, dt, dt1, f0, nn, fh, fl, thr, margin, cnt);
            test_interval(d4.z, w4.z, j + 2, s_dtl, base, dt, dt1, f0, nn, fh, fl, thr, margin, cnt);
            test_interval(d4.w, w4.w, j + 3, s_dtl, base, dt, dt1, f0, nn, fh, fl, thr, margin, cnt);
        }
        for (int j = n4; j < n; j++)
            test_interval(s_dth[j], s_w[j], j, s_dtl, base, dt, dt1, f0, nn, fh, fl, thr, margin, cnt);
    }
#pragma unroll
    for (int k = 0; k < kFreqs; k++)
        if (f0 + k < nn && cnt[k]) atomicAdd(&counts[f0 + k], (unsigned int)cnt[k]);
}

// Device buffers of one call, freed on every return.
struct PeriodScratch {
    double* tm = nullptr;
    unsigned long long* keys = nullptr;  // hash table of distinct intervals
    unsigned int* mult = nullptr;        // their multiplicities
    double* dt = nullptr;                // distinct intervals, packed
    unsigned int* wt = nullptr;          // their multiplicities, packed
    unsigned int* misc = nullptr;        // [0] distinct intervals, [1] table full
    double* fr = nullptr;
    double* dt1 = nullptr;
    unsigned int* counts = nullptr;
    cudaStream_t s = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr, em = nullptr;
    ~PeriodScratch()
    {
        cudaFree(tm); cudaFree(keys); cudaFree(mult); cudaFree(dt); cudaFree(wt); cudaFree(misc);
        cudaFree(fr); cudaFree(dt1); cudaFree(counts);
        if (e0) cudaEventDestroy(e0);
        if (e1) cudaEventDestroy(e1);
        if (em) cudaEventDestroy(em);
        if (s) cudaStreamDestroy(s);
    }
};

}  // namespace
}  // namespace ast

using namespace ast;

extern "C" int ast_minima(int32_t device, int32_t n_plot, const double* t, const double* vm, ast_periodogram* out,
                          int32_t* counts_out)
{
    if (!t || !vm || !out || n_plot < 0) return ast_set_error(AST_E_INVALID, "ast_minima: bad argument");
    for (int32_t i = 1; i < n_plot; i++)
        if (!(t[i] > t[i - 1])) return ast_set_error(AST_E_INVALID, "ast_minima: times must increase");
    memset(out, 0, sizeof(*out));
    // Minima of the curve at their grid times (misc.c:73-96).
    std::vector<double> tm;
    for (int32_t i = 1; i <= n_plot - 2; i++)
        if (vm[i] > vm[i - 1] && vm[i] >= vm[i + 1]) {
            if ((int)tm.size() >= AST_MINIMA_MAX)
                return ast_set_error(AST_E_TOO_LARGE, "ast_minima: N>NMIN_MAX! (more than %d minima)", AST_MINIMA_MAX);
            tm.push_back(t[i]);
        }
    const int n = (int)tm.size();
    const int64_t m = (int64_t)n * (n - 1) / 2;
    out->n_minima = n;
    out->n_intervals = m;
    // Trial frequencies (misc.c:137-144).
    const double fr0 = 1 / kDt0, fr2 = 1 / kDt2;
    std::vector<double> fr(kBins), dt1(kBins);
    for (int i = 0; i < kBins; i++) {
        fr[i] = fr2 + (double)i / (double)(kBins - 1) * (fr0 - fr2);
        dt1[i] = 1 / fr[i];
    }
    std::vector<unsigned int> cnt(kBins, 0);
    if (m > 0) {
        // x = dt * fr must stay below 2^21 for the rounding of the count kernel.
        const double x_max = (tm[n - 1] - tm[0]) * fr[kBins - 1];
        if (!(x_max < 2097152.0))
            return ast_set_error(AST_E_TOO_LARGE, "ast_minima: minima span %.6g days is too long", tm[n - 1] - tm[0]);
        int rc = set_device(device);
        if (rc) return rc;
        PeriodScratch d;
        uint64_t table = 1024;
        while (table < 2 * (uint64_t)m) table <<= 1;
        if (cudaMalloc(&d.tm, sizeof(double) * n) != cudaSuccess ||
            cudaMalloc(&d.keys, sizeof(unsigned long long) * table) != cudaSuccess ||
            cudaMalloc(&d.mult, sizeof(unsigned int) * table) != cudaSuccess ||
            cudaMalloc(&d.dt, sizeof(double) * m) != cudaSuccess || cudaMalloc(&d.wt, sizeof(unsigned int) * m) != cudaSuccess ||
            cudaMalloc(&d.misc, sizeof(unsigned int) * 2) != cudaSuccess ||
            cudaMalloc(&d.fr, sizeof(double) * kBins) != cudaSuccess ||
            cudaMalloc(&d.dt1, sizeof(double) * kBins) != cudaSuccess ||
            cudaMalloc(&d.counts, sizeof(unsigned int) * kBins) != cudaSuccess) {
            cudaGetLastError();
            return ast_set_error(AST_E_NOMEM, "ast_minima: cudaMalloc failed (%lld intervals)", (long long)m);
        }
        AST_CUDA(cudaStreamCreateWithFlags(&d.s, cudaStreamNonBlocking));
        AST_CUDA(cudaEventCreate(&d.e0));
        AST_CUDA(cudaEventCreate(&d.e1));
        AST_CUDA(cudaEventCreate(&d.em));
        AST_CUDA(cudaMemcpyAsync(d.tm, tm.data(), sizeof(double) * n, cudaMemcpyHostToDevice, d.s));
        AST_CUDA(cudaMemcpyAsync(d.fr, fr.data(), sizeof(double) * kBins, cudaMemcpyHostToDevice, d.s));
        AST_CUDA(cudaMemcpyAsync(d.dt1, dt1.data(), sizeof(double) * kBins, cudaMemcpyHostToDevice, d.s));
        AST_CUDA(cudaMemsetAsync(d.counts, 0, sizeof(unsigned int) * kBins, d.s));
        AST_CUDA(cudaMemsetAsync(d.keys, 0, sizeof(unsigned long long) * table, d.s));
        AST_CUDA(cudaMemsetAsync(d.mult, 0, sizeof(unsigned int) * table, d.s));
        AST_CUDA(cudaMemsetAsync(d.misc, 0, sizeof(unsigned int) * 2, d.s));
        int cur = 0, sms = 0;
        AST_CUDA(cudaGetDevice(&cur));
        AST_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, cur));
        AST_CUDA(cudaEventRecord(d.e0, d.s));
        pair_hash_kernel<<<n - 1, 256, 0, d.s>>>(d.tm, n, d.keys, d.mult, table - 1, d.misc + 1);
        AST_CUDA(cudaGetLastError());
        compact_kernel<<<(unsigned)std::min<uint64_t>((table + 255) / 256, (uint64_t)sms * 8), 256, 0, d.s>>>(
            d.keys, d.mult, table, d.dt, d.wt, d.misc);
        AST_CUDA(cudaGetLastError());
        unsigned int misc[2] = {0, 0};
        AST_CUDA(cudaMemcpyAsync(misc, d.misc, sizeof(misc), cudaMemcpyDeviceToHost, d.s));
        AST_CUDA(cudaStreamSynchronize(d.s));
        if (misc[1]) return ast_set_error(AST_E_INVALID, "ast_minima: interval table full");
        const int64_t mu = misc[0];  // distinct intervals
        out->n_distinct = mu;
        const int tiles = (kBins + kFreqTile - 1) / kFreqTile;
        // One wave: as many (tile, slice) CTAs as are resident at once, all with the same work
        // (each slice at least 512 intervals).
        int occ = 0;
        AST_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, interval_count_kernel, kPeriodTpb, 0));
        int64_t slices = std::max<int64_t>(1, (int64_t)sms * std::max(occ, 1) / tiles);
        slices = std::max<int64_t>(1, std::min<int64_t>(slices, (mu + 511) / 512));
        const int64_t per_slice = (mu + slices - 1) / slices;
        slices = (mu + per_slice - 1) / per_slice;
        const float margin = kMarginBase + (float)(1e-13 * x_max);
        AST_CUDA(cudaEventRecord(d.em, d.s));
        interval_count_kernel<<<dim3(tiles, (unsigned)slices), kPeriodTpb, 0, d.s>>>(d.dt, d.wt, mu, per_slice, d.fr,
                                                                                     d.dt1, kBins, margin, d.counts);
        AST_CUDA(cudaGetLastError());
        AST_CUDA(cudaEventRecord(d.e1, d.s));
        AST_CUDA(cudaMemcpyAsync(cnt.data(), d.counts, sizeof(unsigned int) * kBins, cudaMemcpyDeviceToHost, d.s));
        AST_CUDA(cudaStreamSynchronize(d.s));
        float ms = 0, cms = 0;
        AST_CUDA(cudaEventElapsedTime(&ms, d.e0, d.e1));
        AST_CUDA(cudaEventElapsedTime(&cms, d.em, d.e1));
        out->kernel_ms = ms;
        out->count_ms = cms;
    }
    // Normalisation and clusters (misc.c:170-268), in the reference's order.
    std::vector<double> H(kBins);
    std::vector<int> marked(kBins, 0);
    double mean = 0.0;
    for (int i = 0; i < kBins; i++) {
        H[i] = (double)cnt[i];
        mean = mean + H[i];
        if (counts_out) counts_out[i] = (int32_t)cnt[i];
    }
    mean = mean / kBins;
    double s = 0;
    for (int i = 0; i < kBins; i++) {
        const double dev = H[i] - mean;
        s = s + dev * dev;
    }
    s = sqrt(s / (kBins - 1));
    for (int i = 0; i < kBins; i++) H[i] = (H[i] - mean) / s;
    int ncl = 0;
    for (int j = 0; j < AST_NCL_MAX; j++) {
        double top = -100;
        int imax = -1;
        out->cl_fr[j] = -1.0;
        for (int i = 0; i < kBins; i++)
            if (marked[i] == 0 && H[i] > top) {
                top = H[i];
                imax = i;
            }
        if (imax > -1 && H[imax] >= kS0) {
            out->cl_fr[ncl] = fr[imax];
            out->cl_H[ncl] = H[imax];
            ncl++;
            // The cluster extends both ways while the normalised count stays above s0.  (The
            // reference's leftward walk from imax = 0 reads one element before the array; here
            // it stops at the first bin.)
            for (int i = imax; i < kBins && H[i] > kS0; i++) marked[i] = 1;
            for (int i = imax - 1; i >= 0 && H[i] > kS0; i--) marked[i] = 1;
        }
    }
    out->n_clusters = ncl;
    return AST_OK;
}
