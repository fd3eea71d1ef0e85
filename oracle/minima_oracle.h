/*
 * minima_oracle.h -- THE ORACLE for the periodogram of model minima.  TEST INFRASTRUCTURE ONLY.
 * Included by chi2_oracle.c (compiled with -ffp-contract=off).
 *
 * A plain CPU restatement of minima() of the reference (misc.c:65-276, default build: minima at
 * grid times, step-function histogram).  Step by step:
 *   misc.c:73-96    minima: V[i] > V[i-1] && V[i] >= V[i+1] for 1 <= i <= Nplot-2, time t[i];
 *                   more than 10000 (NMIN_MAX) is an error (the reference exits);
 *   misc.c:106-121  every interval t[j] - t[i], i < j;
 *   misc.c:131-168  NN = 10000 frequencies fr[i] = fr2 + i/(NN-1) (fr0 - fr2), fr0 = 1/(1/24),
 *                   fr2 = 1/(80/24); H[i] = number of intervals with
 *                   |dt/dt1 - int(dt/dt1 + 0.5)| < 0.1, dt1 = 1/fr[i];
 *                   (the reference sorts the intervals first, misc.c:128; a count does not
 *                   depend on their order, so the sort is left out);
 *   misc.c:172-197  mean m = sum H / NN, s = sqrt(sum (H-m)^2 / (NN-1)), H = (H - m) / s;
 *   misc.c:210-268  NCL_MAX = 5 times: the highest unmarked H at or above s0 = 3 is a cluster
 *                   (cl_fr, cl_H); the bins around it with H > s0 are marked.  (The reference's
 *                   leftward walk from the first bin reads H[-1]; here it stops at the first bin.)
 * threads > 0 runs the frequency loop on that many OpenMP threads (counts are integers, so
 * the result does not depend on it).
 */

int orc_minima(const double* t, const double* vm, int n_plot, int threads, double* cl_fr, double* cl_H,
               int32_t* counts, int32_t* n_minima)
{
    enum { NN = 10000, NCL = 5, NMAX = 10000 };
    const double sgm = 0.1, dt0 = 1.0 / 24.0, dt2 = 80.0 / 24.0, s0 = 3;
    double* tm = (double*)malloc(sizeof(double) * NMAX);
    int n = 0;
    for (int i = 1; i <= n_plot - 2; i++)
        if (vm[i] > vm[i - 1] && vm[i] >= vm[i + 1]) {
            if (n == NMAX) {
                free(tm);
                return -1;
            }
            tm[n++] = t[i];
        }
    *n_minima = n;
    const int64_t m = (int64_t)n * (n - 1) / 2;
    double* dt = (double*)malloc(sizeof(double) * (m > 0 ? m : 1));
    int64_t k = 0;
    for (int i = 0; i < n - 1; i++)
        for (int j = i + 1; j < n; j++) dt[k++] = tm[j] - tm[i];
    const double fr0 = 1 / dt0, fr2 = 1 / dt2;
    double* fr = (double*)malloc(sizeof(double) * NN);
    double* H = (double*)malloc(sizeof(double) * NN);
    int* marked = (int*)calloc(NN, sizeof(int));
    for (int i = 0; i < NN; i++) fr[i] = fr2 + (double)i / (double)(NN - 1) * (fr0 - fr2);
#ifdef _OPENMP
    if (threads <= 0) threads = 1;
#pragma omp parallel for num_threads(threads) schedule(dynamic, 16)
#endif
    for (int i = 0; i < NN; i++) {
        const double dt1 = 1 / fr[i];
        int64_t c = 0;
        for (int64_t j = 0; j < m; j++) {
            const double x = dt[j] / dt1;
            const double dv = fabs(x - (double)(int)(x + 0.5));
            if (dv < sgm) c++;
        }
        counts[i] = (int32_t)c;
    }
    double mean = 0.0;
    for (int i = 0; i < NN; i++) {
        H[i] = (double)counts[i];
        mean = mean + H[i];
    }
    mean = mean / NN;
    double s = 0;
    for (int i = 0; i < NN; i++) {
        const double dev = H[i] - mean;
        s = s + dev * dev;
    }
    s = sqrt(s / (NN - 1));
    for (int i = 0; i < NN; i++) H[i] = (H[i] - mean) / s;
    int ncl = 0;
    for (int j = 0; j < NCL; j++) cl_H[j] = 0.0;
    for (int j = 0; j < NCL; j++) {
        double top = -100;
        int imax = -1;
        cl_fr[j] = -1.0;
        for (int i = 0; i < NN; i++)
            if (!marked[i] && H[i] > top) {
                top = H[i];
                imax = i;
            }
        if (imax < 0 || !(H[imax] >= s0)) continue;
        cl_fr[ncl] = fr[imax];
        cl_H[ncl] = H[imax];
        ncl++;
        int i = imax;
        while (i < NN && H[i] > s0) marked[i++] = 1;
        i = imax - 1;
        while (i >= 0 && H[i] > s0) marked[i--] = 1;
    }
    free(tm); free(dt); free(fr); free(H); free(marked);
    return ncl;
}
