/*
 * ref_nm_shim.h -- TEST INFRASTRUCTURE ONLY.  Lets the text of the reference's chi2_gpu kernel
 * (cuda.c:1326-1833, the downhill-simplex driver) or chi2_gpu_rms kernel (cuda.c:2148-2389, the
 * RMSD confidence-interval sampler) compile and run as host code, so that the oracle's
 * restatements of them (nm_oracle_*.h, rmsd_oracle*.h) can be pinned to the reference's own
 * code on the CPU.
 *
 * oracle/build_ref.sh streams, into one translation unit: the reference's asteroid.h and cuda.c
 * (as for libref_<variant>.so, chi2one / x2params / params2x re-qualified __host__ __device__),
 * this header, the kernel cut from cuda.c, and ref_harness_nm.cu, which undoes the macros below
 * and provides the entry point.  Nothing of the reference is written to disk.
 *
 * The CUDA execution model of one block, on the host:
 *   - a block's BSIZE threads are BSIZE host threads; __syncthreads() is a barrier among them;
 *   - __shared__ variables become function-static, i.e. one copy shared by the block's threads
 *     (blocks run one after the other); atomicAdd is a locked host add;
 *   - threadIdx / blockIdx / blockDim are per-thread (thread_local) values;
 *   - the __device__ variables the kernels read or write (dLimits, dTypes, dProperty, d_x2_params,
 *     d_chi2_params, d_params0, the INTERP ephemeris, d_Ntot, d_Nbad, d_f0, d_f1) are host
 *     variables that the entry point fills and reads;
 *   - curandState / curand_uniform / curand_normal is the engine's Philox stream (philox.cuh):
 *     chi2_gpu draws exactly 3 N_PARAMS uniforms per stage (N_PARAMS for the start point, two
 *     for each further vertex, cuda.c:1462,1519,1523), so draw k of stage s of thread c is
 *     uniform01(seed, c, s, k); chi2_gpu_rms draws exactly N_PARAMS normals per sample
 *     (cuda.c:2277), so normal i of sample k of thread c is element i mod 4 of
 *     normal4(seed, c, 0x80000000 | call, k ceil(N_PARAMS / 4) + i / 4).  Both follow from the
 *     running count of draws.
 * With the reference's own cuRAND XORWOW states replaced by these draws, the kernels take the
 * same random points as the oracle and the engine, and every other step is the reference's.
 */
#include <stdint.h>
#include <condition_variable>
#include <mutex>
#include "philox.cuh"

namespace refnm {

struct dim3h {
    unsigned x, y, z;
};
static thread_local dim3h tid;
static thread_local dim3h bid;
static dim3h bdim;

/* Generation-counting barrier for the threads of one block. */
struct Barrier {
    std::mutex m;
    std::condition_variable cv;
    int n = 0, waiting = 0;
    uint64_t gen = 0;
    void wait()
    {
        std::unique_lock<std::mutex> lk(m);
        const uint64_t g = gen;
        if (++waiting == n) {
            waiting = 0;
            ++gen;
            cv.notify_all();
        } else {
            cv.wait(lk, [&] { return gen != g; });
        }
    }
};
static Barrier barrier;

struct Rng {
    uint64_t seed, chain;
    uint32_t count;    /* draws so far */
    int per_stage;     /* chi2_gpu: 3 N_PARAMS uniforms per stage; chi2_gpu_rms: N_PARAMS normals per sample */
    uint32_t call;     /* chi2_gpu_rms: the launch's index in the host loop */
};

static inline float uniform(Rng* s)
{
    const uint32_t stage = s->count / (uint32_t)s->per_stage, k = s->count % (uint32_t)s->per_stage;
    s->count++;
    return ast::uniform01(s->seed, s->chain, stage, k);
}

static inline float normal(Rng* s)
{
    const uint32_t k = s->count / (uint32_t)s->per_stage, i = s->count % (uint32_t)s->per_stage;
    const uint32_t nq = ((uint32_t)s->per_stage + 3u) / 4u;
    s->count++;
    float z[4];
    ast::normal4(s->seed, s->chain, 0x80000000u | s->call, k * nq + i / 4u, z);
    return z[i % 4u];
}

static std::mutex atomic_lock;
static inline int atomic_add(int* p, int v)
{
    std::lock_guard<std::mutex> g(atomic_lock);
    const int old = *p;
    *p = old + v;
    return old;
}

}  // namespace refnm

/* Host copies of the __device__ tables the kernel reads. */
static CHI_FLOAT refnm_dLimits[2][N_TYPES];
static int refnm_dTypes[N_TYPES][N_SEG];
static int refnm_dProperty[N_PARAMS][N_COLUMNS];
static struct x2_struct refnm_d_x2_params;
static struct chi2_struct refnm_d_chi2_params;
static double refnm_d_params0[N_PARAMS];
static double refnm_dE_x0[3], refnm_dE_y0[3], refnm_dE_z0[3], refnm_dS_x0[3], refnm_dS_y0[3], refnm_dS_z0[3],
    refnm_dMJD0[3];
static int refnm_d_Ntot, refnm_d_Nbad;
static float refnm_d_f0, refnm_d_f1;

#pragma push_macro("__global__")
#pragma push_macro("__shared__")
#undef __global__
#undef __shared__
#define __global__ static
#define __shared__ static
#define threadIdx refnm::tid
#define blockIdx refnm::bid
#define blockDim refnm::bdim
#define __syncthreads() refnm::barrier.wait()
#define curandState refnm::Rng
#define curand_uniform(s) refnm::uniform(s)
#define curand_normal(s) refnm::normal(s)
#define atomicAdd refnm::atomic_add
#define chi2_gpu refnm_chi2_gpu
#define chi2_gpu_rms refnm_chi2_gpu_rms
#define d_Ntot refnm_d_Ntot
#define d_Nbad refnm_d_Nbad
#define d_f0 refnm_d_f0
#define d_f1 refnm_d_f1
#define dLimits refnm_dLimits
#define dTypes refnm_dTypes
#define dProperty refnm_dProperty
#define d_x2_params refnm_d_x2_params
#define d_chi2_params refnm_d_chi2_params
#define d_params0 refnm_d_params0
#define dE_x0 refnm_dE_x0
#define dE_y0 refnm_dE_y0
#define dE_z0 refnm_dE_z0
#define dS_x0 refnm_dS_x0
#define dS_y0 refnm_dS_y0
#define dS_z0 refnm_dS_z0
#define dMJD0 refnm_dMJD0
