/*
 * asteroid.c -- command-line driver (host, C), the drop-in for the reference's asteroid
 * binary on its fitting path (asteroid.c:18-831 of the reference) and its -plot mode
 * (asteroid.c:834-1060).
 *
 * Same switches and meanings: -i -o -m -t -reopt -keep -best -seed -N -Nstages -f -l -Ppsi
 * -plot (asteroid.c:173-431), same output line ("%13.6e " chi^2, "%13.6e " per-filter delta_V,
 * "%15.11f " parameters in Property order, asteroid.c:798-811), same stdout best line
 * (asteroid.c:770-779), same keep/best/travel semantics (asteroid.c:741-818).  Periodic
 * parameters are printed unwrapped, as the reference does (its wrap loop never runs, see
 * asteroid.c:753).
 *
 * The reference fixes the model variant, N_BLOCKS, BSIZE and TIME_STEP at compile time; here
 * the compile-time macros (-DTORQUE -DBC -DBW_BALL -DP_PSI -DACC -DNUDGE -DINTERP, -DN_BLOCKS,
 * -DBSIZE, -DTIME_STEP) give the defaults and these extra switches override them at run time:
 *   -variant TORQUE,P_PSI,...   -Nblocks n   -bsize n   -time_step h   -mixed   -evals n
 *   -eph dir (directory of asteroid.eph / earth.eph / sun.eph, default ".")
 *   -Nplot n (points of the -plot model curve, default NPLOT = 20000)
 *   -spherical_k (the -DSPHERICAL_K torque output of RMSD runs)
 *   -animate (the -DANIMATE build: -plot renders image_%05d.png frames, with -i1 / -i2, NPLOT 15440)
 *   -size_pix n (frame size, default SIZE_PIX = 1080)
 * With the RMSD variant (-variant ...,RMSD, or -DRMSD) the program computes the RMSD confidence
 * intervals of the -m model instead of fitting (asteroid.c:643-725), with -dx and -Nstages.
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#include "asteroid_gb300.h"

#ifndef N_BLOCKS
#define N_BLOCKS 152
#endif
#ifndef BSIZE
#define BSIZE 256
#endif
#ifndef TIME_STEP
#define TIME_STEP 1e-2
#endif

static int default_flags(void)
{
    int f = 0;
#ifdef TORQUE
    f |= AST_TORQUE;
#endif
#ifdef BC
    f |= AST_BC;
#endif
#ifdef BW_BALL
    f |= AST_BW_BALL;
#endif
#ifdef P_PSI
    f |= AST_P_PSI;
#endif
#ifdef INTERP
    f |= AST_INTERP;
#endif
#ifdef ACC
    f |= AST_ACC;
#endif
#ifdef NUDGE
    f |= AST_NUDGE;
#endif
#ifdef RMSD
    f |= AST_RMSD;
#endif
    if (f == 0) f = AST_TORQUE | AST_P_PSI; /* the README's fiducial model */
    return f;
}

static int parse_variant(const char* s)
{
    static const struct { const char* n; int f; } names[] = {
        {"TORQUE", AST_TORQUE}, {"BC", AST_BC}, {"BW_BALL", AST_BW_BALL}, {"P_PSI", AST_P_PSI},
        {"INTERP", AST_INTERP}, {"ACC", AST_ACC}, {"NUDGE", AST_NUDGE}, {"RMSD", AST_RMSD}, {"LS", 0}};
    int f = 0;
    char buf[256];
    snprintf(buf, sizeof(buf), "%s", s);
    for (char* tok = strtok(buf, ",+ "); tok; tok = strtok(NULL, ",+ ")) {
        if (tok[0] == '-' && tok[1] == 'D') tok += 2;
        int found = 0;
        for (size_t k = 0; k < sizeof(names) / sizeof(names[0]); k++)
            if (strcmp(tok, names[k].n) == 0) { f |= names[k].f; found = 1; }
        if (!found) { fprintf(stderr, "Unknown variant %s\n", tok); exit(1); }
    }
    return f;
}

static void usage(void)
{
    printf("\n Command line arguments:\n\n");
    printf("-best : only keep the best result\n");
    printf("-f type_constant value: forces the parameter with the type_constant to be frozen during optimization at \"value\" \n");
    printf("-i name : input (data) file name\n");
    printf("-i1 index : index of the first snapshot  [-animate]\n");
    printf("-i2 index : index of the last snapshot minus one  [-animate]\n");
    printf("-keep : keep all intermediate results, not just the best ones\n");
    printf("-l type_constant limit1 limit2 : specify range for the parameter type_constant\n");
    printf("-m param1 param2 ... paramN : input model parameters, for plotting and re-optimization\n");
    printf("     If one of the parameters has a special value of \"v\", it is allowed to vary randomly within its full range.\n");
    printf("-N number : exit after \"number\" cycles\n");
    printf("-Nstages number : each initial optimization stage is followed by \"number-1\" reoptimization stages\n");
    printf("-o name : output (results) file name\n");
    printf("-plot : plotting (only makes sense when -m is also used)\n");
    printf("-dx value : maximum shift for parameters in scale-free units (0...1)  [RMSD variant]\n");
    printf("-Ppsi min max : minimum and maximum values for Ppsi period, in hours\n");
    printf("-reopt : reoptimize the model provided with -m switch\n");
    printf("-seed SEED : use the SEED number to initialize the random number generator\n");
    printf("-t : travelling reoptimization\n");
    printf("\n GB300 engine switches: -variant TORQUE,P_PSI,... -Nblocks n -bsize n -time_step h -mixed -evals n -eph dir -Nplot n -spherical_k\n"
           "   -animate -size_pix n\n\n");
}

/* -plot mode (asteroid.c:834-1060, the default build): the chi^2 and delta_V of the -m model on
 * the data, the model curve on an evenly spaced grid of n_plot times shifted by delta_V of the
 * first filter, the periodogram of that curve's minima (cluster frequencies and heights), and
 * the files delta_V, model_params.dat, model.dat and data.dat in the reference's formats.  The model curve is the brightness model alone: NUDGE bookkeeping,
 * which in the reference can end the curve early after M_MAX minima, plays no part. */
static int run_plot(const ast_model* m, const ast_host_data* hd, ast_ctx* ctx, const double* params, int interp,
                    int n_plot)
{
    printf("\n*** Plotting ***\n\n");
    const int N = m->n_params, NF = hd->obs.n_filters;
    double chi2 = 0, dv[AST_MAX_FILTERS];
    if (ast_eval_batch(ctx, AST_PREC_FP64, params, 1, &chi2, dv)) { printf("%s\n", ast_last_error()); return 1; }
    FILE* fp = fopen("delta_V", "w");
    if (!fp) { printf("Cannot write delta_V\n"); return 1; }
    for (int k = 0; k < NF; k++) fprintf(fp, "%8.4f\n", dv[k]);
    fclose(fp);
    /* The initial model state without the torque, BC and BW_BALL parameters (asteroid.c:913-941). */
    fp = fopen("model_params.dat", "w");
    if (!fp) { printf("Cannot write model_params.dat\n"); return 1; }
    const ast_type_ids* T = &m->ids;
    for (int j = 0; j < N; j++) {
        const int ty = m->property[j][AST_P_TYPE];
        if ((m->flags & AST_TORQUE) && (ty == T->Ti || ty == T->Ts || ty == T->Tl)) continue;
        if ((m->flags & AST_BC) && (ty == T->c || ty == T->b)) continue;
        if ((m->flags & AST_BW_BALL) && (ty == T->theta_R || ty == T->phi_R || ty == T->kappa)) continue;
        fprintf(fp, "%15.11f ", params[j]);
    }
    fprintf(fp, "\n");
    fclose(fp);
    double* t = (double*)malloc(sizeof(double) * n_plot);
    double* e = (double*)malloc(sizeof(double) * 3 * n_plot);
    double* sv = (double*)malloc(sizeof(double) * 3 * n_plot);
    double* vm = (double*)malloc(sizeof(double) * n_plot);
    int rc = (!t || !e || !sv || !vm) ? 1 : 0;
    if (!rc && (ast_plot_grid(hd, interp, n_plot, t, e, sv) || ast_model_curve_at(ctx, params, n_plot, t, e, sv, vm))) {
        printf("%s\n", ast_last_error());
        rc = 1;
    }
    if (!rc) {
        /* The curve as the reference keeps it, shifted to the first filter (cuda.c:764). */
        for (int i = 0; i < n_plot; i++) vm[i] = vm[i] + dv[0];
        /* Periodogram of the model minima (asteroid.c:972-980). */
        ast_periodogram pg;
        if (ast_minima(-1, n_plot, t, vm, &pg, NULL)) {
            printf("%s\n", ast_last_error());
            rc = 1;
        } else {
            for (int j = 0; j < AST_NCL_MAX; j++) printf("%f ", pg.cl_fr[j]);
            for (int j = 0; j < AST_NCL_MAX; j++) printf("%f ", pg.cl_H[j]);
            printf("\n");
        }
    }
    if (!rc) {
        /* "lsq" bins per-point values the default build never computes (asteroid.c:987-1025, on a
         * freshly allocated, zero-filled array): 0 when all six time bins hold data, else nan. */
        double cnt[6] = {0}, sum = 0, sw = 0;
        for (int i = 0; i < hd->obs.n_data; i++) {
            const double tt = hd->mjd[i];
            cnt[tt < 0.5 ? 0 : tt < 1.5 ? 1 : tt < 2.7 ? 2 : tt < 3.7 ? 3 : tt < 4.5 ? 4 : 5] += 1;
        }
        for (int k = 0; k < 6; k++) {
            const double W = (k == 2 || k == 3) ? 2 : 1;
            sum = sum + W * (0.0 / cnt[k]);
            sw = sw + W;
        }
        printf("chi2_plot = %13.6e, lsq = %13.6e\n", chi2, sqrt(sum / sw));
        fp = fopen("model.dat", "w");
        if (!fp) rc = 1;
        else {
            for (int i = 0; i < n_plot; i++) fprintf(fp, "%13.7f %13.6e\n", hd->hmjd0 + t[i], vm[i]);
            fclose(fp);
        }
        fp = rc ? NULL : fopen("data.dat", "w");
        if (!fp) rc = 1;
        else {
            /* V converted to the first filter (asteroid.c:1039-1045). */
            for (int i = 0; i < hd->obs.n_data; i++)
                fprintf(fp, "%13.7f %13.6e %13.6e w\n", hd->hmjd0 + hd->mjd[i], hd->v[i] - dv[hd->filter[i]] + dv[0],
                        1 / sqrt(hd->w[i]));
            fclose(fp);
        }
    }
    free(t); free(e); free(sv); free(vm);
    return rc;
}

/* -plot under ANIMATE (asteroid.c:863-878): the frames of snapshots i1 .. i2-1 in steps of
 * dNPLOT = 1500, each step ending at min(start + 1500, NPLOT) as the reference's loop does, written
 * as image_%05d.png (misc.c:372-460).  Rendered in groups of at most 64 frames. */
static int run_animate(const ast_host_data* hd, ast_ctx* ctx, const double* params, int interp, int n_plot, int i1,
                       int i2, int size_pix)
{
    printf("\n*** Plotting ***\n\n");
    if (i1 < 0 || i2 > n_plot || i1 >= i2) { printf("Bad arguments!\n"); return 1; }
    double* t = (double*)malloc(sizeof(double) * n_plot);
    double* e = (double*)malloc(sizeof(double) * 3 * n_plot);
    double* sv = (double*)malloc(sizeof(double) * 3 * n_plot);
    double* geo = (double*)malloc(sizeof(double) * AST_GEO * n_plot);
    const int group = 64;
    uint8_t* rgb = (uint8_t*)malloc((size_t)3 * size_pix * size_pix * group);
    int rc = (!t || !e || !sv || !geo || !rgb) ? 1 : 0;
    if (!rc && (ast_plot_grid(hd, interp, n_plot, t, e, sv) || ast_model_geometry(ctx, params, n_plot, t, e, sv, geo))) {
        printf("%s\n", ast_last_error());
        rc = 1;
    }
    for (int h_i1 = i1; !rc && h_i1 < i2; h_i1 += 1500) {
        const int h_i2 = h_i1 + 1500 > n_plot ? n_plot : h_i1 + 1500;
        for (int f0 = h_i1; !rc && f0 < h_i2; f0 += group) {
            const int nf = h_i2 - f0 < group ? h_i2 - f0 : group;
            if (ast_render_frames(-1, geo + (size_t)AST_GEO * f0, nf, size_pix, rgb, NULL)) {
                printf("%s\n", ast_last_error());
                rc = 1;
                break;
            }
            for (int k = 0; k < nf && !rc; k++) {
                char name[64];
                snprintf(name, sizeof(name), "image_%05d.png", f0 + k);
                if (ast_write_png(name, rgb + (size_t)3 * size_pix * size_pix * k, size_pix, size_pix)) {
                    fprintf(stderr, "%s\n", ast_last_error());
                    rc = 1;
                }
            }
        }
    }
    free(t); free(e); free(sv); free(geo); free(rgb);
    return rc;
}

/* -DRMSD runs (asteroid.c:643-725): repeated chi2_gpu_rms calls, each followed by one line with
 * the fraction of bad models so far and every parameter's cumulative [min max] (stdout), and the
 * ranges alone in the output file. */
static int run_rmsd(ast_ctx* ctx, int N, const char* outp, const double* params, unsigned long seed, long long n_streams,
                    int samples, float dx, int reopt, int spherical, int precision, int Ncases)
{
    float PAR_min[AST_MAX_PARAMS], PAR_max[AST_MAX_PARAMS];
    for (int j = 0; j < N; j++) { PAR_min[j] = 1e30f; PAR_max[j] = -1e30f; }
    printf("\n");
    FILE* fp = fopen(outp, "w");
    if (!fp) { printf("Bad output file name!\n"); return 1; }
    long long n_tot = 0, n_bad = 0;
    for (int loop_counter = 1;; loop_counter++) {
        ast_rmsd_cfg cfg;
        memset(&cfg, 0, sizeof(cfg));
        cfg.seed = (unsigned long long)seed;
        cfg.n_streams = n_streams;
        cfg.samples = samples;
        cfg.precision = precision;
        cfg.dx = dx;
        cfg.reopt = reopt;
        cfg.spherical_k = spherical;
        cfg.call = (uint32_t)(loop_counter - 1);
        cfg.params0 = params;
        ast_rmsd_out ro;
        if (ast_rmsd(ctx, &cfg, &ro)) { printf("%s\n", ast_last_error()); fclose(fp); return 1; }
        /* d_Ntot and d_Nbad accumulate over the calls (cuda.c:2348-2349). */
        n_tot += ro.n_tot;
        n_bad += ro.n_bad;
        if (loop_counter == 1) printf("f0=%f, f1=%f\n\n", (double)(float)ro.f0, (double)(float)ro.f1);
        printf("%e ", n_bad / (double)n_tot);
        for (int j = 0; j < N; j++) {
            if ((float)ro.par_min[j] < PAR_min[j]) PAR_min[j] = (float)ro.par_min[j];
            if ((float)ro.par_max[j] > PAR_max[j]) PAR_max[j] = (float)ro.par_max[j];
            printf("%13.6e %13.6e ; ", PAR_min[j], PAR_max[j]);
            fprintf(fp, "%13.6e %13.6e ; ", PAR_min[j], PAR_max[j]);
        }
        printf("\n");
        fflush(stdout);
        fprintf(fp, "\n");
        fflush(fp);
        if (loop_counter == Ncases) break;
    }
    fclose(fp);
    return 0;
}

int main(int argc, char** argv)
{
    if (argc == 1) { usage(); return 0; }
    int flags = default_flags();
    int n_blocks = N_BLOCKS, bsize = BSIZE, precision = AST_PREC_FP64;
    double time_step = TIME_STEP, ppsi1 = 2.0, ppsi2 = 4800.0;
    long long evals_cap = 0;
    const char *in = NULL, *outp = NULL, *eph = ".";
    int travel = 0, keep = 0, best = 0, reopt = 0, model_given = 0, plot = 0, Ncases = -1, Nstages = 1;
    int n_plot = 20000; /* NPLOT (asteroid.h:266) */
    float dx_rand = 0.0001f; /* DX_RAND (asteroid.h:209) */
#ifdef ANIMATE
    int animate = 1;
#else
    int animate = 0;
#endif
    int i1_input = 0, i2_input = -1, size_pix = AST_SIZE_PIX, nplot_given = 0;
#ifdef SPHERICAL_K
    int spherical = 1;
#else
    int spherical = 0;
#endif
    unsigned long seed = 0;
    int n_frozen = 0, n_limits = 0;
    int Fi[64], Li[64];
    double Fv[64], L0[64], L1[64];
    char* mtok[AST_MAX_PARAMS + 2] = {0};
    int mtok_n = 0;

    for (int j = 1; j < argc;) {
        const char* a = argv[j];
        if (a[0] != '-') { printf("Bad arguments!\n"); return 1; }
#define NEED(k) do { if (j + (k) >= argc) { printf("Bad arguments!\n"); return 1; } } while (0)
        if (!strcmp(a, "-i")) { NEED(1); in = argv[j + 1]; j += 2; }
        else if (!strcmp(a, "-o")) { NEED(1); outp = argv[j + 1]; j += 2; }
        else if (!strcmp(a, "-Ppsi")) { NEED(2); ppsi1 = atof(argv[j + 1]); ppsi2 = atof(argv[j + 2]); j += 3; }
        else if (!strcmp(a, "-m")) {
            /* The parameter count depends on the variant, which may come later: keep the tokens. */
            j++;
            while (j < argc && mtok_n < AST_MAX_PARAMS && (argv[j][0] != '-' || (argv[j][1] >= '0' && argv[j][1] <= '9') || argv[j][1] == '.'))
                mtok[mtok_n++] = argv[j++];
            model_given = 1;
        }
        else if (!strcmp(a, "-plot")) { plot = 1; j++; }
        else if (!strcmp(a, "-Nplot")) { NEED(1); n_plot = atoi(argv[j + 1]); nplot_given = 1; j += 2; }
        else if (!strcmp(a, "-animate")) { animate = 1; j++; }
        else if (!strcmp(a, "-i1")) { NEED(1); i1_input = atoi(argv[j + 1]); j += 2; }
        else if (!strcmp(a, "-i2")) { NEED(1); i2_input = atoi(argv[j + 1]); j += 2; }
        else if (!strcmp(a, "-size_pix")) { NEED(1); size_pix = atoi(argv[j + 1]); j += 2; }
        else if (!strcmp(a, "-dx")) { NEED(1); dx_rand = (float)atof(argv[j + 1]); j += 2; }
        else if (!strcmp(a, "-spherical_k")) { spherical = 1; j++; }
        else if (!strcmp(a, "-t")) { travel = 1; j++; }
        else if (!strcmp(a, "-reopt")) { reopt = 1; j++; }
        else if (!strcmp(a, "-keep")) { keep = 1; j++; }
        else if (!strcmp(a, "-best")) { best = 1; j++; }
        else if (!strcmp(a, "-seed")) { NEED(1); seed = strtoul(argv[j + 1], NULL, 10); j += 2; }
        else if (!strcmp(a, "-N")) { NEED(1); Ncases = atoi(argv[j + 1]); j += 2; }
        else if (!strcmp(a, "-Nstages")) { NEED(1); Nstages = atoi(argv[j + 1]); j += 2; }
        else if (!strcmp(a, "-f")) { NEED(2); if (n_frozen < 64) { Fi[n_frozen] = atoi(argv[j + 1]); Fv[n_frozen++] = atof(argv[j + 2]); } j += 3; }
        else if (!strcmp(a, "-l")) { NEED(3); if (n_limits < 64) { Li[n_limits] = atoi(argv[j + 1]); L0[n_limits] = atof(argv[j + 2]); L1[n_limits++] = atof(argv[j + 3]); } j += 4; }
        else if (!strcmp(a, "-variant")) { NEED(1); flags = parse_variant(argv[j + 1]); j += 2; }
        else if (!strcmp(a, "-Nblocks")) { NEED(1); n_blocks = atoi(argv[j + 1]); j += 2; }
        else if (!strcmp(a, "-bsize")) { NEED(1); bsize = atoi(argv[j + 1]); j += 2; }
        else if (!strcmp(a, "-time_step")) { NEED(1); time_step = atof(argv[j + 1]); j += 2; }
        else if (!strcmp(a, "-mixed")) { precision = AST_PREC_MIXED; j++; }
        else if (!strcmp(a, "-evals")) { NEED(1); evals_cap = atoll(argv[j + 1]); j += 2; }
        else if (!strcmp(a, "-eph")) { NEED(1); eph = argv[j + 1]; j += 2; }
        else { printf("Bad arguments!\n"); return 1; }
#undef NEED
    }
    if (!in) { printf("-i parameter is missing!\n"); return 1; }
    if ((reopt || plot) && !model_given) { printf("-reopt and -plot switches require -m switch!\n"); return 1; }
    if (!reopt && !plot && model_given) { printf("-m can only be used together with -reopt or -plot switches!\n"); return 1; }
    if (animate && !nplot_given) n_plot = AST_NPLOT_ANIMATE;
    if (i2_input < 0) i2_input = n_plot;
    if (plot && n_plot < 2) { printf("Bad arguments!\n"); return 1; }

    ast_model model;
    if (ast_model_init(&model, flags, time_step, ppsi1, ppsi2)) { fprintf(stderr, "%s\n", ast_last_error()); return 1; }
    const int N = model.n_params;
    double params[AST_MAX_PARAMS] = {0};
    if (model_given) {
        if (mtok_n < N) { printf("Not enough of model parameters in -m switch!\n"); return 1; }
        for (int k = 0; k < N; k++) {
            if (mtok[k][0] == 'v') { ast_model_set_free_random(&model, k); params[k] = 0; }
            else params[k] = atof(mtok[k]);
        }
    }
    for (int k = 0; k < n_frozen; k++)
        if (ast_model_freeze(&model, Fi[k], Fv[k])) { fprintf(stderr, "%s\n", ast_last_error()); return 1; }
    for (int k = 0; k < n_limits; k++)
        if (ast_model_set_limits(&model, Li[k], L0[k], L1[k])) { fprintf(stderr, "%s\n", ast_last_error()); return 1; }

    ast_host_data* hd = NULL;
    if (ast_read_data(in, eph, (flags & AST_INTERP) != 0, AST_MAX_FILTERS, &hd)) { printf("%s\n", ast_last_error()); return 1; }
    printf("Filters:\n");
    for (int k = 0; k < hd->obs.n_filters; k++) printf("%d: %c\n", k + 1, hd->filters[k]);
    if (flags & AST_NUDGE) {
        if (ast_read_minima("observed.min", hd)) { printf("%s\n", ast_last_error()); return 1; }
        printf("%d minima in observed.min\n", hd->obs.n_minima);
    }
    ast_ctx* ctx = NULL;
    if (ast_prepare(&model, &hd->obs, -1, &ctx)) { printf("%s\n", ast_last_error()); return 1; }
    if (plot && animate) {
        const int rc = run_animate(hd, ctx, params, (flags & AST_INTERP) != 0, n_plot, i1_input, i2_input, size_pix);
        ast_destroy(ctx);
        ast_free_host_data(hd);
        return rc;
    }
    if (plot) {
        const int rc = run_plot(&model, hd, ctx, params, (flags & AST_INTERP) != 0, n_plot);
        ast_destroy(ctx);
        ast_free_host_data(hd);
        return rc;
    }
    if (!outp) { printf("Bad output file name!\n"); return 1; }
    const int NF = hd->obs.n_filters;
    const long long n_chains = (long long)n_blocks * bsize;
    printf("\n*** Simplex optimization ***\n\n");
    printf("  N_threads = %lld\n", n_chains);
    if (seed == 0) seed = (unsigned long)time(NULL);
    if (flags & AST_RMSD) {
        /* chi2_gpu_rms reads the -m model only where -reopt uploaded it (asteroid.c:637). */
        if (!model_given) { printf("-reopt and -plot switches require -m switch!\n"); return 1; }
        const int rc = run_rmsd(ctx, N, outp, params, seed, n_chains, Nstages, dx_rand, reopt, spherical, precision,
                                Ncases);
        ast_destroy(ctx);
        ast_free_host_data(hd);
        return rc;
    }

    double* h_f = (double*)malloc(sizeof(double) * n_blocks);
    double* h_p = (double*)malloc(sizeof(double) * n_blocks * N);
    double* h_dv = (double*)malloc(sizeof(double) * n_blocks * NF);
    double* c_f = (double*)malloc(sizeof(double) * n_blocks);
    double* c_p = (double*)malloc(sizeof(double) * n_blocks * N);
    double* c_dv = (double*)malloc(sizeof(double) * n_blocks * NF);
    for (int b = 0; b < n_blocks; b++) h_f[b] = 1e30;
    int loop_counter = 0;
    while (1) {
        loop_counter++;
        ast_fit_cfg cfg;
        memset(&cfg, 0, sizeof(cfg));
        /* The reference's cuRAND states advance across loops; here every loop has its own key. */
        cfg.seed = (unsigned long long)seed + 0x9E3779B97F4A7C15ull * (unsigned long long)(loop_counter - 1);
        cfg.n_chains = n_chains;
        cfg.group_size = bsize;
        cfg.n_stages = Nstages;
        cfg.reopt = reopt;
        cfg.precision = precision;
        cfg.evals_cap = evals_cap;
        cfg.params0 = params;
        ast_fit_out out;
        memset(&out, 0, sizeof(out));
        out.best_f = c_f;
        out.best_params = c_p;
        out.best_dv = c_dv;
        if (ast_fit(ctx, &cfg, &out)) { printf("%s\n", ast_last_error()); return 1; }
        /* d_f keeps each block's best across loops unless -keep resets it (asteroid.c:816-818). */
        for (int b = 0; b < n_blocks; b++)
            if (c_f[b] < h_f[b]) {
                h_f[b] = c_f[b];
                memcpy(h_p + (size_t)b * N, c_p + (size_t)b * N, sizeof(double) * N);
                memcpy(h_dv + (size_t)b * NF, c_dv + (size_t)b * NF, sizeof(double) * NF);
            }
        int i_best = 0;
        double chi2_tot = 1e32;
        for (int b = 0; b < n_blocks; b++)
            if (h_f[b] < chi2_tot) { chi2_tot = h_f[b]; i_best = b; }
        if (reopt && travel) memcpy(params, h_p + (size_t)i_best * N, sizeof(double) * N);
        printf("%13.6e ", h_f[i_best]);
        for (int k = 0; k < N; k++) printf("%15.11f ", h_p[(size_t)i_best * N + k]);
        printf("\n");
        fflush(stdout);
        FILE* fp = fopen(outp, keep ? "a" : "w");
        if (!fp) { printf("Bad output file name!\n"); return 1; }
        int i1 = best ? i_best : 0, i2 = best ? i_best + 1 : n_blocks;
        char line[8192];
        for (int b = i1; b < i2; b++) {
            ast_format_result(line, sizeof(line), h_f[b], h_dv + (size_t)b * NF, NF, h_p + (size_t)b * N, N);
            fputs(line, fp);
        }
        fclose(fp);
        if (keep)
            for (int b = 0; b < n_blocks; b++) h_f[b] = 1e30;
        if (loop_counter == Ncases) break;
    }
    ast_destroy(ctx);
    ast_free_host_data(hd);
    free(h_f); free(h_p); free(h_dv); free(c_f); free(c_p); free(c_dv);
    return 0;
}
