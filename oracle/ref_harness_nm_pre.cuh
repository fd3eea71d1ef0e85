/*
 * ref_harness_nm_pre.cuh -- TEST INFRASTRUCTURE ONLY.  Streamed by oracle/build_ref.sh between
 * the reference's asteroid.h and cuda.c for the simplex builds (ref_nm_<variant>.cubin), which
 * run the reference's own setup_kernel + chi2_gpu (cuda.c:2039, cuda.c:1326) on the GPU.
 *
 * The reference reports only each block's best (d_f, d_params, d_dV) and caps simplex
 * iterations (N_STEPS, asteroid.h:213), not evaluations.  Three hooks make the run comparable
 * with ast_fit chain by chain; build_ref.sh inserts the calls with sed, in the stream only:
 *   N_STEPS            becomes the device variable refk_n_steps (set per run by refn_setup)
 *   refk_count_eval()  first statement of chi2one (cuda.c:81): per-thread evaluation count
 *   refk_record_chain  in place of the comment line after the per-stage s_f assignment
 *                      (cuda.c:1739-1745): every chain's final chi^2 and iteration count l
 * Nothing else of the reference's code changes.
 */
__device__ unsigned int refk_n_steps = 5000;
__device__ double* refk_chain_f;    /* [Nstages][threads] final chi^2 of each chain and stage */
__device__ int* refk_chain_l;       /* [Nstages][threads] its simplex iterations l */
__device__ unsigned int* refk_evals; /* [threads] chi2one calls */
__device__ int refk_threads;

__device__ __forceinline__ void refk_count_eval(void)
{
    if (refk_evals) refk_evals[blockIdx.x * blockDim.x + threadIdx.x]++;
}

__device__ __forceinline__ void refk_record_chain(int id, int istage, double f, int l)
{
    if (refk_chain_f) {
        refk_chain_f[(size_t)istage * refk_threads + id] = f;
        refk_chain_l[(size_t)istage * refk_threads + id] = l;
    }
}
