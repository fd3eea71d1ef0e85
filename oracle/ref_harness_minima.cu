/*
 * ref_harness_minima.cu -- TEST INFRASTRUCTURE ONLY.  A host entry point around the reference's
 * own minima() (misc.c:65-276), for pinning the periodogram oracle.
 *
 * oracle/build_ref.sh compiles this file as the tail of one translation unit whose head is the
 * reference's asteroid.h and misc.c (default macros), read in place under the reference checkout
 * and streamed to nvcc; nothing of the reference is written to disk.  The result,
 * oracle/_ref/libref_minima.so, is git-ignored.
 *
 * minima() reads the plot-grid times from struct obs_data and writes the globals cl_fr and cl_H;
 * cl_H is zeroed before each call, as at the start of the reference's program.  More than
 * NMIN_MAX minima make the reference exit, so the harness refuses those inputs itself.
 */
#include <stdlib.h>

extern "C" int refm_minima(const double* t, const double* vm, int nplot, double* fr_out, double* h_out)
{
    int n = 0;
    for (int i = 1; i <= nplot - 2; i++)
        if (vm[i] > vm[i - 1] && vm[i] >= vm[i + 1]) n++;
    if (n > 10000) return -1;
    struct obs_data* p = (struct obs_data*)calloc(nplot, sizeof(struct obs_data));
    double* v = (double*)malloc(sizeof(double) * (nplot > 0 ? nplot : 1));
    for (int i = 0; i < nplot; i++) {
        p[i].MJD = t[i];
        v[i] = vm[i];
    }
    for (int j = 0; j < NCL_MAX; j++) {
        cl_fr[j] = 0.0;
        cl_H[j] = 0.0;
    }
    minima(p, v, nplot);
    for (int j = 0; j < NCL_MAX; j++) {
        fr_out[j] = cl_fr[j];
        h_out[j] = cl_H[j];
    }
    free(p);
    free(v);
    return n;
}
