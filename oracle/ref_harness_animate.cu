/*
 * ref_harness_animate.cu -- TEST INFRASTRUCTURE ONLY.  A kernel around the reference's own
 * compute_rgb (cuda.c:2394-2540, the -DANIMATE build), so the frames of the CUDA renderer can be
 * held to the reference's pixels on the same geometry.
 *
 * oracle/build_ref.sh compiles this file as the tail of one translation unit whose head is the
 * reference's asteroid.h (its png.h include dropped) and cuda.c with -DANIMATE, streamed to nvcc;
 * nothing of the reference is written to disk.  The cubin, oracle/_ref/ref_animate.cubin, is
 * git-ignored.  Launched with 576 threads per block (1080^2 = 2025 x 576), so no thread leaves
 * compute_rgb before its __syncthreads.
 */
extern "C" __global__ void refa_render(unsigned char* rgb, const double* geo, int frame)
{
    const double* g = geo + 20 * (long)frame;
    compute_rgb(rgb, g[0], g[1], g[2], g[3], g[4], g[5], g[6], g[7], g[8], g[9], g[10], g[11], g[12], g[13], g[14],
                g[15], g[16], g[17], g[18], g[19], frame, 0);
}
