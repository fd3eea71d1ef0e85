/*
 * ref_nm_shim.h -- TEST INFRASTRUCTURE ONLY.  Lets the text of the reference's chi2_gpu kernel
 * (cuda.c:1326-1833, the downhill-simplex driver) compile and run as host code, so that the
 * oracle's restatement of it (nm_oracle_body.h, nm_oracle_impl.h) can be pinned to the
 * reference's own code on the CPU.
 *
 * oracle/build_ref.sh streams, into one translation unit: the reference's asteroid.h and cuda.c
 * (as for libref_<variant>.so, chi2one / x2params / params2x re-qualified __host__ __device__),
 * this header, the chi2_gpu function cut from cuda.c, and ref_harness_nm.cu, which undoes the
 * macros below and provides the entry point.  Nothing of the reference is written to disk.
 *
 * The CUDA execution model of one block, on the host:
 *   - a block's BSIZE threads are BSIZE host threads; __syncthreads() is a barrier among them;
 *   - __shared__ variables become function-static, i.e. one copy shared by the block's threads
 *     (blocks run one after the other);
 *   - threadIdx / blockIdx / blockDim are per-thread (thread_local) values;
 *   - the __device__ tables the kernel reads (dLimits, dTypes, dProperty, d_x2_params,
 *     d_chi2_params, d_params0, the INTERP ephemeris) are host arrays that the entry point fills;
 *   - curandState / curand_uniform is the engine's Philox stream: draw k of stage s of chain c is
 *     uniform01(seed, c, s, k) (philox.cuh).  The kernel draws exactly 3 N_PARAMS numbers per
 *     stage (N_PARAMS for the start point, two for each further vertex, cuda.c:1462,1519,1523),
 *     so the stage and the draw index follow from the running count of draws.
 * With the reference's own cuRAND XORWOW states replaced by these draws, the kernel's chains take
 * the same start points as the oracle's and the engine's, and every later step is the reference's.
 */
#include <stdint.h>
#include <condition_variable>
#include <mutex>

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

/* Philox4x32-10 (Salmon et al., SC'11), as in philox.cuh. */
static inline void philox(uint32_t c[4], uint32_t k0, uint32_t k1)
{
    for (int r = 0; r < 10; r++) {
        const uint64_t p0 = (uint64_t)0xD2511F53u * c[0], p1 = (uint64_t)0xCD9E8D57u * c[2];
        const uint32_t n0 = (uint32_t)(p1 >> 32) ^ c[1] ^ k0, n2 = (uint32_t)(p0 >> 32) ^ c[3] ^ k1;
        c[0] = n0;
        c[1] = (uint32_t)p1;
        c[2] = n2;
        c[3] = (uint32_t)p0;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
}

struct Rng {
    uint64_t seed, chain;
    uint32_t count;  /* draws so far */
    int per_stage;   /* 3 N_PARAMS */
};

static inline float uniform(Rng* s)
{
    const uint32_t stage = s->count / (uint32_t)s->per_stage, k = s->count % (uint32_t)s->per_stage;
    s->count++;
    uint32_t c[4] = {k >> 2, stage, (uint32_t)s->chain, (uint32_t)(s->chain >> 32)};
    philox(c, (uint32_t)s->seed, (uint32_t)(s->seed >> 32));
    const uint32_t u = c[k & 3];
    return ((float)(u >> 8) + 0.5f) * (1.0f / 16777216.0f);
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
#define chi2_gpu refnm_chi2_gpu
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
