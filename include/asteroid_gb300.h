/*
 * asteroid_gb300.h -- C ABI of the GB300 (sm_103a) light-curve fitting engine.
 *
 * The engine evaluates the chi^2 of a tumbling, optionally torqued asteroid model against a
 * photometric light curve, and runs downhill-simplex (Nelder-Mead) chains with random starts
 * on the device.  It is a drop-in for the fitting path of pulsar123/Asteroid:
 *
 *   reference interface (file:line in the Asteroid sources)      replaced here by
 *   --------------------------------------------------------      ----------------------------
 *   gpu_prepare(N_data,N_filters,N_threads,Nplot)  gpu_prepare.c:2  ast_prepare()
 *   cudaMemcpyToSymbol(dProperty,dTypes,dLimits,d_x2_params)
 *                                              asteroid.c:603-606  ast_set_tables()
 *   prepare_chi2_params() (observed.min upload)   misc.c:279-323  ast_obs_set.n_minima/t_min/v_min
 *   chi2one(params,sData,...)  (one chi^2 evaluation) cuda.c:81    ast_eval_batch()
 *   setup_kernel + chi2_gpu<<<N_BLOCKS,BSIZE>>>  cuda.c:2039,1326   ast_fit() / ast_fit_begin/step/end
 *   cudaMemcpy D2H of d_params,d_dV,d_f           asteroid.c:728-730 ast_fit_out (caller buffers)
 *   ERR() -> gpuAssert -> exit                     cuda_errors.h:4-14 int status + ast_last_error()
 *   read_data()                                    read_data.c:6     ast_read_data()
 *   quadratic_interpolation()                      misc.c:20         ast_quadratic_interpolation()
 *   Property/Types/hLimits tables                  asteroid.c:86-169,473-601  ast_model_init()
 *
 * All entry points take plain pointers and sizes.  Every function returns 0 on success or a
 * negative AST_E_* status; ast_last_error() gives a message for the calling thread.
 * A context is single-threaded: calls on one ast_ctx must not overlap.  All calls block until
 * their results are in the caller's buffers, except the *_device variants, which are
 * stream-ordered on the stream passed in.
 */
#ifndef ASTEROID_GB300_H
#define ASTEROID_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------- sizes */
#define AST_MAX_PARAMS   16   /* N_PARAMS of every supported variant is <= 14 */
#define AST_MAX_TYPES    16
#define AST_MAX_FILTERS  8    /* N_FILTERS (asteroid.h:191) is a runtime value here */
#define AST_NOBS_MAX     10   /* observed minima, asteroid.h:219 */
#define AST_M_MAX        30   /* model minima, asteroid.h:217 */
#define AST_N_COLUMNS    6
#define AST_MAX_DATA     16384 /* observations per object (MAX_DATA, asteroid.h; a run-time limit here) */

/* ---------------------------------------------------------------- status codes */
#define AST_OK             0
#define AST_E_INVALID     -1   /* bad argument / inconsistent input */
#define AST_E_NOMEM       -2   /* device or host allocation failed */
#define AST_E_CUDA        -3   /* CUDA runtime error (message in ast_last_error) */
#define AST_E_IO          -4   /* file missing or malformed */
#define AST_E_TOO_LARGE   -5   /* size beyond a documented maximum */
#define AST_E_BUDGET      -6   /* request does not fit the admission budget */
#define AST_E_TIMEOUT     -7   /* a device wait gave up after its iteration limit */
#define AST_E_NOT_READY   -8   /* result not available yet */
#define AST_E_NODEVICE    -9   /* no CUDA device */
#define AST_E_CANCELLED  -10   /* the request was cancelled (ast_cancel) */

/* ---------------------------------------------------------------- model variants
 * The reference selects these with compile-time macros (makefile:1-36); here they are
 * runtime flags of an ast_model.  Parameter order and type numbering follow the reference
 * for every combination (asteroid.c:86-125, asteroid.h:137-178). */
#define AST_TORQUE   0x01  /* -DTORQUE : constant body-frame torque, 3 extra parameters */
#define AST_BC       0x02  /* -DBC     : photometric c, b independent of c_tumb, b_tumb */
#define AST_BW_BALL  0x04  /* -DBW_BALL: black-and-white ball brightness, theta_R phi_R kappa */
#define AST_P_PSI    0x08  /* -DP_PSI  : L is generated from the Ppsi period range */
#define AST_INTERP   0x10  /* -DINTERP : E,S from the 3-point ephemeris at asteroid time */
#define AST_ACC      0x20  /* -DACC    : CHI_FLOAT = double, SIZE_MIN = 1e-10 */
#define AST_NUDGE    0x40  /* -DNUDGE  : reward for model minima near observed minima */
#define AST_RMSD     0x80  /* -DRMSD   : chi2one returns sqrt(sum chi2_m / sum w), the RMSD */

/* Property table columns (asteroid.h:115-123) */
#define AST_P_TYPE          0
#define AST_P_INDEPENDENT   1
#define AST_P_FROZEN        2
#define AST_P_ISEG          3
#define AST_P_MULTI_SEGMENT 4
#define AST_P_PERIODIC      5
/* P_periodic values (asteroid.h:126-131) */
#define AST_PERIODIC       1
#define AST_PERIODIC_LAM   0
#define AST_SOFT_BOTH     -1
#define AST_HARD_LEFT     -2
#define AST_HARD_RIGHT    -3
#define AST_HARD_BOTH     -4

/* Parameter type ids of one variant: the reference numbers types with __COUNTER__ in the
 * order theta_M, phi_M, phi_0, L, [Ti Ts Tl], c_tumb, b_tumb, Es, psi_0, [c b],
 * [theta_R phi_R], [kappa] (asteroid.h:137-178).  Absent types are -1.  These ids are
 * what the -f and -l command-line switches take. */
typedef struct ast_type_ids {
    int32_t theta_M, phi_M, phi_0, L, Ti, Ts, Tl, c_tumb, b_tumb, Es, psi_0, c, b,
            theta_R, phi_R, kappa;
    int32_t n_types;
} ast_type_ids;

/* One model variant with its tables; the device copy of the reference's dProperty,
 * dTypes, dLimits and d_x2_params symbols (asteroid.h:460,509-510,533). */
typedef struct ast_model {
    int32_t flags;                                   /* AST_TORQUE | ... */
    int32_t n_params;                                /* N_PARAMS (asteroid.h:110) */
    int32_t n_types;                                 /* N_TYPES  (asteroid.h:178) */
    int32_t property[AST_MAX_PARAMS][AST_N_COLUMNS]; /* Property (asteroid.c:86-125) */
    int32_t types[AST_MAX_TYPES];                    /* Types[type][0]: parameter index or -1 */
    double  limits[2][AST_MAX_TYPES];                /* hLimits; float-rounded unless AST_ACC */
    float   ppsi1, ppsi2;                            /* x2_struct.Ppsi1/2 = 24/Ppsi_max, 24/Ppsi_min */
    double  time_step;                               /* TIME_STEP, days (asteroid.h:202) */
    ast_type_ids ids;
} ast_model;

/* One object's light curve after the reference's host conversion (read_data.c:243-302):
 * times are asteroid times minus the first one (hMJD0), magnitudes are geometry corrected,
 * E and S are unit asteroid->Earth and asteroid->Sun vectors. */
typedef struct ast_obs_set {
    int32_t n_data;                 /* observations, >= n_params + n_filters + 1 */
    int32_t n_filters;              /* distinct filters, <= AST_MAX_FILTERS */
    const double*  mjd;             /* [n_data] days, strictly increasing */
    const float*   v;               /* [n_data] magnitude (obs_data.V is float) */
    const float*   w;               /* [n_data] 1/sgm^2    (obs_data.w is float) */
    const int32_t* filter;          /* [n_data] 0..n_filters-1 */
    const double*  e_unit;          /* [n_data*3] (x,y,z) per point; unused under AST_INTERP */
    const double*  s_unit;          /* [n_data*3] */
    double eph_e[3][3];             /* AST_INTERP: E_x0[3],E_y0[3],E_z0[3] (read_data.c:189-191) */
    double eph_s[3][3];             /*             S_x0[3],S_y0[3],S_z0[3] */
    double eph_mjd0[3];             /*             MJD0[3] minus hMJD0 (read_data.c:298-302) */
    int32_t n_minima;               /* AST_NUDGE: observed minima (misc.c:279-323) */
    float   t_min[AST_NOBS_MAX];    /*   minimum time minus hMJD0 */
    float   v_min[AST_NOBS_MAX];    /*   minimum magnitude */
} ast_obs_set;

/* ---------------------------------------------------------------- tables (host, C) */

/* Fill the Property/Types/hLimits tables of a variant exactly as asteroid.c:86-169 and
 * :473-564 do, and the P_PSI range as asteroid.c:598-601 (ppsi_* in hours; ignored unless
 * AST_P_PSI).  Replaces the table set-up at the top of the reference's main(). */
int ast_model_init(ast_model* m, int32_t flags, double time_step,
                   double ppsi_min_hours, double ppsi_max_hours);
/* -f type value: freeze every parameter of that type at value (asteroid.c:566-581). */
int ast_model_freeze(ast_model* m, int32_t type, double value);
/* -l type l0 l1: custom limits for a type (asteroid.c:583-589). */
int ast_model_set_limits(ast_model* m, int32_t type, double l0, double l1);
/* -m ... "v": parameter randomly varied over its full range under -reopt (asteroid.c:310-315). */
int ast_model_set_free_random(ast_model* m, int32_t param_index);
/* Name of parameter i in output order (README.md:110-115 order), e.g. "theta_M". */
const char* ast_param_name(const ast_model* m, int32_t i);

/* x2params (cuda.c:1120-1319) on the host, with the model's CHI_FLOAT rounding of x:
 * returns 0, 1 when x leaves a hard limit (the reference's failure), or a negative status.
 * reopt selects the meaning of the L coordinate under P_PSI (cuda.c:1219,1244). */
int ast_x2params(const ast_model* m, int32_t reopt, const double* x, double* params);
/* params2x (cuda.c:1016-1115) on the host. */
int ast_params2x(const ast_model* m, const double* params, double* x);

/* ---------------------------------------------------------------- host I/O (C) */

/* Host copy of a light curve read from the reference's files. */
typedef struct ast_host_data {
    ast_obs_set obs;          /* pointers into the arrays below */
    double* mjd; float* v; float* w; int32_t* filter; double* e_unit; double* s_unit;
    double* mjd_obs;          /* observer times as read (MJD_obs) */
    double  hmjd0;            /* first asteroid time (read_data.c:274-276) */
    char    filters[AST_MAX_FILTERS]; /* filter characters in order of appearance */
} ast_host_data;

/* read_data.c:6-302: read "filter MJD V sgm aux" lines from lc_path and the HORIZONS
 * vector files asteroid.eph, earth.eph, sun.eph from eph_dir; apply the geometry and
 * light-time corrections, normalise E and S.  interp selects the INTERP time shift of
 * the ephemeris points.  Rejects unsorted times and more than max_filters filters. */
int ast_read_data(const char* lc_path, const char* eph_dir, int32_t interp,
                  int32_t max_filters, ast_host_data** out);
/* misc.c:279-323: read observed.min lines "MJD_min V_min" from path, keep those within
 * 0.05 d of the data range, at most AST_NOBS_MAX, into d->obs.n_minima/t_min/v_min. */
int ast_read_minima(const char* path, ast_host_data* d);
void ast_free_host_data(ast_host_data* d);

/* misc.c:20-35: second-order Lagrange interpolation of E and S at time t. */
void ast_quadratic_interpolation(const double mjd0[3], const double e[3][3], const double s[3][3],
                                 double t, double out_e[3], double out_s[3]);

/* read_data.c:309-370: the plot grid of -plot mode: n_plot times evenly spaced from the first to
 * the last observation (relative to hMJD0), the two ends being those observations with their
 * E and S, the interior E and S interpolated from the three ephemeris points and normalised.
 * interp: the light curve was read with AST_INTERP. */
int ast_plot_grid(const ast_host_data* d, int32_t interp, int32_t n_plot, double* t, double* e_unit,
                  double* s_unit);

/* asteroid.c:798-811: one result line "chi2 dV_1..dV_Nf p_1..p_N\n" with the reference's
 * "%13.6e " / "%15.11f " formats.  Returns the number of characters written. */
int ast_format_result(char* buf, int64_t cap, double chi2, const double* dv, int32_t n_filters,
                      const double* params, int32_t n_params);

/* ---------------------------------------------------------------- device engine */

typedef struct ast_ctx ast_ctx;

#define AST_PREC_FP64   0   /* plain path: the reference's double arithmetic */
#define AST_PREC_MIXED  1   /* double-FP32 state and right-hand side, FP32 brightness */
#define AST_PREC_MIXED_RHS32 2 /* AST_PREC_MIXED with the ODE right-hand side in FP32 (the state
                                  still double-FP32): faster, but outside 1e-6 relative chi^2 on
                                  about 5-10% of vectors; single-object evaluation and fits only */

/* gpu_prepare.c:2-56 + asteroid.c:603-606: pack one object's observations into SoA device
 * buffers (16-byte aligned segments staged into shared memory by bulk copies), hoist the
 * parameter-independent ephemeris interpolation, upload the tables.  device < 0 means the
 * current device. */
int ast_prepare(const ast_model* model, const ast_obs_set* obs, int32_t device, ast_ctx** out);
/* Replace the tables after ast_prepare (same variant flags and n_params). */
int ast_set_tables(ast_ctx* ctx, const ast_model* model);
void ast_destroy(ast_ctx* ctx);
const char* ast_last_error(void);

/* chi2one (cuda.c:81-1011) on n physical parameter vectors params[n][n_params], host
 * buffers.  chi2[n] receives the value chi2one returns (1e30 for the NUDGE failure),
 * delta_v[n][n_filters] (may be NULL) the per-filter offsets.  Results follow CHI_FLOAT:
 * rounded to float unless the model has AST_ACC. */
int ast_eval_batch(ast_ctx* ctx, int32_t precision, const double* params, int64_t n,
                   double* chi2, double* delta_v);
/* Same with device pointers, stream-ordered on `stream` (a cudaStream_t; NULL = legacy). */
int ast_eval_batch_device(ast_ctx* ctx, int32_t precision, const double* d_params, int64_t n,
                          double* d_chi2, double* d_delta_v, void* stream);

/* Model magnitude at every observation of the context's object for one parameter vector
 * (the reference's chi2one with Nplot > 0, cuda.c:699-704, without the delta_V shift):
 * the model-curve path of the plot mode and of the synthetic-data generator. */
int ast_model_curve(ast_ctx* ctx, const double* params, double* vmod);

/* The same model magnitudes at n other times t (relative to hMJD0, increasing, n >= 2) with
 * unit E and S vectors e_unit, s_unit (ignored under AST_INTERP, where they are interpolated
 * from the ephemeris as for the data): the model curve of -plot mode on its fine grid
 * (chi2one with Nplot > 0 on dPlot, cuda.c:1949-1950), without the delta_V shift. */
int ast_model_curve_at(ast_ctx* ctx, const double* params, int32_t n, const double* t, const double* e_unit,
                       const double* s_unit, double* vmod);

/* ---------------------------------------------------------------- ANIMATE frames
 * The -DANIMATE build renders the asteroid as seen from Earth at every plot-grid time
 * (chi2one's compute_rgb call, cuda.c:576-586; compute_rgb cuda.c:2394-2540) and writes
 * image_%05d.png files (write_PNGs, misc.c:372-460).  Here that is three calls: the geometry of
 * every snapshot, the frames, and a PNG writer. */
#define AST_GEO       20    /* doubles per snapshot, see ast_model_geometry */
#define AST_SIZE_PIX  1080  /* SIZE_PIX (asteroid.h:259) */
#define AST_NPLOT_ANIMATE 15440 /* NPLOT of the ANIMATE build (asteroid.h:264) */

/* Geometry at n increasing times (as ast_model_curve_at), geo[AST_GEO*i + k]: b, c (the
 * brightness ellipsoid's axes), E (unit, inertial), E and S in the body frame (b, c, a
 * components), and the body axes b, c, a in inertial coordinates. */
int ast_model_geometry(ast_ctx* ctx, const double* params, int32_t n, const double* t, const double* e_unit,
                       const double* s_unit, double* geo);

/* compute_rgb for n_frames snapshots on CUDA device `device` (-1: current): rgb receives
 * n_frames x size_pix x size_pix x 3 bytes, rgb[ic + 3*(x + size_pix*(y + size_pix*f))], the
 * reference's d_rgb layout (row y = the image's z1 axis).  size_pix even, <= 8192.  kernel_ms
 * (optional) receives the device time of the rendering. */
int ast_render_frames(int32_t device, const double* geo, int32_t n_frames, int32_t size_pix, uint8_t* rgb,
                      double* kernel_ms);

/* One 8-bit RGB PNG (write_PNGs' per-snapshot file; colour type 2, no interlace). */
int ast_write_png(const char* path, const uint8_t* rgb, int32_t width, int32_t height);

/* Euler angles (phi, theta, psi) at every observation, angles[3*i + k], as integrated by the
 * FP64 path or by the mixed path (double-float state, reduced to [-pi, pi] at each
 * observation): the phase drift of the mixed path.  No reference counterpart. */
int ast_model_angles(ast_ctx* ctx, int32_t precision, const double* params, double* angles);

/* The periodogram of model minima printed by -plot mode: minima() (misc.c:65-276, default
 * build).  The brightness minima of a model curve (V[i] > V[i-1] && V[i] >= V[i+1]) are taken at
 * their grid times; every interval between two of them is tested against AST_MINIMA_BINS trial
 * frequencies fr evenly spaced from 24/80 to 24 per day: it counts for fr when it lies within
 * 0.1 of a whole number of periods 1/fr.  The counts, normalised by their mean and standard
 * deviation, give the AST_NCL_MAX highest clusters at or above 3 (cl_fr, cl_H; -1 and 0 where
 * there are fewer), which asteroid.c:974-980 prints.  At most AST_MINIMA_MAX minima
 * (NMIN_MAX; more is AST_E_TOO_LARGE, where the reference exits). */
#define AST_MINIMA_BINS 10000 /* NN, misc.c:131 */
#define AST_NCL_MAX     5     /* NCL_MAX, asteroid.h:277 */
#define AST_MINIMA_MAX  10000 /* NMIN_MAX, misc.c:69 */

typedef struct ast_periodogram {
    int32_t n_minima;          /* minima found on the curve */
    int32_t n_clusters;        /* clusters found (<= AST_NCL_MAX) */
    int64_t n_intervals;       /* n_minima (n_minima - 1) / 2 */
    int64_t n_distinct;        /* distinct interval values among them (each tested once, weighted) */
    double  cl_fr[AST_NCL_MAX];  /* cluster frequency (1/day), -1 where none */
    double  cl_H[AST_NCL_MAX];   /* normalised count at that frequency, 0 where none */
    double  kernel_ms;         /* device time of the interval reduction and test */
    double  count_ms;          /* of which the test of the distinct intervals */
} ast_periodogram;

/* Curve vm at n_plot increasing times t (days) on CUDA device `device` (-1: current).  counts
 * (optional, AST_MINIMA_BINS entries) receives the raw count of each frequency bin. */
int ast_minima(int32_t device, int32_t n_plot, const double* t, const double* vm, ast_periodogram* out,
               int32_t* counts);

typedef struct ast_fit_cfg {
    uint64_t seed;          /* -seed; chains draw from Philox4x32-10 keyed by (seed, chain) */
    int64_t  n_chains;      /* N_BLOCKS*BSIZE in the reference */
    int32_t  group_size;    /* chains per result group (BSIZE); n_chains % group_size == 0 */
    int32_t  n_stages;      /* -Nstages */
    int32_t  reopt;         /* -reopt: start from params0 */
    int32_t  precision;     /* AST_PREC_* */
    int64_t  evals_cap;     /* per chain and stage, checked where N_STEPS is; 0 = none */
    int32_t  steps_cap;     /* N_STEPS (asteroid.h:213); 0 = 5000 */
    int32_t  tpb;           /* threads per CTA; 0 = autotuned */
    const double* params0;  /* [n_params] start model for reopt (d_params0) */
    int32_t  min_ctas_per_sm; /* register budget: 1 (or 0) = up to 255 registers/thread, 2 = 128 */
    int32_t  stage_obs;     /* observations in shared memory: 1 = always when they fit, -1 = never,
                                 0 = only when it does not lower the CTAs per SM */
    int32_t  fp64_result;   /* AST_PREC_MIXED only: report each group's chi^2 as the plain FP64
                                 path's chi^2 at its best parameters (one FP64 evaluation per group
                                 at the end); the search itself stays mixed.  0 = the mixed chi^2 */
} ast_fit_cfg;

typedef struct ast_fit_out {
    double*  best_f;        /* [n_groups]            d_f          (may be NULL) */
    double*  best_params;   /* [n_groups][n_params]  d_params     (may be NULL) */
    double*  best_dv;       /* [n_groups][n_filters] d_dV         (may be NULL) */
    double*  chain_f;       /* [n_chains] final best of every chain (may be NULL) */
    int64_t  n_evals;       /* chi^2 evaluations performed */
    int64_t  n_fits;        /* chains finished (all stages) */
    double   kernel_ms;     /* device time of the simplex launches */
} ast_fit_out;

/* One full fitting pass: setup_kernel + chi2_gpu + the host argmin inputs
 * (asteroid.c:626-759).  Group g's best follows the reference's block best: lowest chi^2,
 * lowest chain index on ties; its delta_V is that chain's last evaluation's (cuda.c:1816-1821). */
int ast_fit(ast_ctx* ctx, const ast_fit_cfg* cfg, ast_fit_out* out);

/* ---------------------------------------------------------------- RMSD confidence intervals
 * chi2_gpu_rms<<<N_BLOCKS, BSIZE>>> (cuda.c:2148-2389) with the host loop of asteroid.c:690-725:
 * unconstrained confidence intervals of the -m model (Bartczak & Dudzinski 2019).  Every one of
 * n_streams random streams draws `samples` models x = x0 + dx * N(0,1) per parameter (clamped
 * 1e-8 inside hard limits, cuda.c:2276-2287), maps them with x2params (a rejected draw is not
 * counted), and evaluates the RMSD; a model with RMSD below f1 = f0 + f0/sqrt(N_data - N - Nf),
 * f0 the RMSD of the -m model, widens the [min, max] range of every parameter.  The ctx model
 * must carry AST_RMSD.  Draws are Philox4x32-10 keyed by (seed, call, stream, draw) with
 * Box-Muller normals: the same distribution as the reference's curand_normal, not the same
 * numbers.  Kept from the reference: phi_M / phi_0 of a good model more than pi from the -m
 * model's value are replaced by that value -/+ 2 pi (cuda.c:2304-2311), and under spherical_k the
 * torque is reported as (K, theta_K, phi_K) (cuda.c:2312-2331). */
typedef struct ast_rmsd_cfg {
    uint64_t seed;          /* -seed */
    int64_t  n_streams;     /* N_BLOCKS*BSIZE threads of chi2_gpu_rms */
    int32_t  samples;       /* -Nstages: draws per stream per call */
    int32_t  precision;     /* AST_PREC_FP64 or AST_PREC_MIXED */
    double   dx;            /* -dx: shift scale in dimensionless units (a float in the reference) */
    int32_t  reopt;         /* -reopt: the reopt flag x2params sees */
    int32_t  spherical_k;   /* -DSPHERICAL_K (TORQUE models): torque as K, theta_K, phi_K */
    uint32_t call;          /* index of this call in a sequence (each call draws new models) */
    int32_t  reserved;
    const double* params0;  /* the -m model [n_params] */
    double*  trace_x;       /* optional [n_streams*samples][n_params]: every drawn point */
    double*  trace_f;       /* optional [n_streams*samples]: its RMSD, NaN where x2params rejected it */
} ast_rmsd_cfg;

typedef struct ast_rmsd_out {
    double  f0, f1;                     /* RMSD of the -m model and the bound (cuda.c:2225-2227) */
    int64_t n_tot;                      /* models evaluated (d_Ntot) */
    int64_t n_bad;                      /* of those, RMSD >= f1 or NaN (d_Nbad) */
    double  par_min[AST_MAX_PARAMS];    /* per parameter over the good models, as float; 1e30 if none */
    double  par_max[AST_MAX_PARAMS];    /* -1e30 if none */
    double  kernel_ms;                  /* device time of the sampling launch */
} ast_rmsd_out;

/* One chi2_gpu_rms launch (asteroid.c:673): this call's counts and ranges (the caller
 * accumulates them over calls as asteroid.c:698-718 does). */
int ast_rmsd(ast_ctx* ctx, const ast_rmsd_cfg* cfg, ast_rmsd_out* out);

/* The same pass split into resumable launches: chain state stays resident on the device
 * between ast_fit_step calls.  Each step lets every chain slot perform at most
 * evals_per_slot evaluations; *done becomes 1 when all stages of all chains finished.
 * AST_E_TIMEOUT from ast_fit_step (or ast_fit) means a CTA's shared-memory staging wait ran
 * out and it read the observations from global memory instead: the step is complete, *done is
 * valid and the results are unaffected; the fit may continue. */
int ast_fit_begin(ast_ctx* ctx, const ast_fit_cfg* cfg);
int ast_fit_step(ast_ctx* ctx, int64_t evals_per_slot, int32_t* done, void* stream);
int ast_fit_end(ast_ctx* ctx, ast_fit_out* out);

/* A fit that allocates nothing (no counterpart in the reference).  For callers that cannot
 * call cudaMalloc -- code embedded in a host framework that owns every device allocation through
 * its own pool, or a service whose device memory is reserved at start-up and must not grow.
 * Inputs are the caller's device arrays (d_mjd, d_v, d_w, d_filter as in ast_obs_set; d_e_unit,
 * d_s_unit [n_data*3], ignored under AST_INTERP) plus the host struct obs for n_data, n_filters,
 * the INTERP ephemeris and the NUDGE minima (its array pointers are not read).  Outputs are the
 * caller's device arrays d_best_f[groups], d_best_params[groups*n_params],
 * d_best_dv[groups*n_filters], with ast_fit's meaning.  All other state lives in one
 * file-scope device array of AST_NOALLOC_SCRATCH_BYTES (14 MiB) that every GPU loading the
 * library holds until the process exits; sizes above AST_NOALLOC_MAX_CHAINS chains or
 * AST_NOALLOC_MAX_DATA observations are rejected with AST_E_TOO_LARGE.  Stream-ordered on
 * `stream` (NULL = legacy default stream); returns when the fit is complete.  Every call shares
 * the array: calls that overlap on a GPU race.  The first call on a device looks up the array's
 * address (cudaGetSymbolAddress) with that device current; make it before any stream capture. */
#define AST_NOALLOC_MAX_CHAINS 4096
#define AST_NOALLOC_MAX_DATA 4096
#define AST_NOALLOC_SCRATCH_BYTES (14u << 20)
int ast_fit_noalloc(const ast_model* model, const ast_obs_set* obs, const double* d_mjd, const float* d_v,
                    const float* d_w, const int32_t* d_filter, const double* d_e_unit, const double* d_s_unit,
                    const ast_fit_cfg* cfg, double* d_best_f, double* d_best_params, double* d_best_dv,
                    void* stream);

/* How many times each thread of the fit kernel polls the barrier of the shared-memory staging
 * copy before it gives up (default 4194304; no reference counterpart).  A CTA whose wait runs out
 * reads the observations from global memory instead (the results do not change), waits for its
 * copy before it exits, and the step returns AST_E_TIMEOUT.  0 takes that path at once: the
 * device-side failure path can be exercised without a fault. */
int ast_set_stage_wait(ast_ctx* ctx, int32_t polls);

/* Number of chain slots (persistent threads) the fit kernel of this context runs. */
int64_t ast_fit_slots(ast_ctx* ctx);

/* Launch geometry ast_fit_begin chose: threads per CTA, CTAs, register budget (CTAs of 256
 * threads per SM the kernel was compiled for) and dynamic shared memory bytes.  Any pointer may
 * be NULL.  No reference counterpart (the reference's geometry is the compile-time
 * N_BLOCKS x BSIZE, asteroid.h:38-48). */
int ast_fit_launch(ast_ctx* ctx, int32_t* tpb, int32_t* ctas, int32_t* min_ctas_per_sm, int32_t* smem_bytes);

/* Device-side evaluation and fit counters since ast_fit_begin. */
int ast_fit_counters(ast_ctx* ctx, int64_t* n_evals, int64_t* n_fits);

/* The CUDA stream the context launches on (a cudaStream_t). */
void* ast_stream(ast_ctx* ctx);

/* Peak-rate probe: times an FP64 (kind 0) or FP32 (kind 1) FMA loop over every SM and
 * returns GFLOP/s in *gflops.  Used as the roofline denominator for CUDA-core bound kernels. */
int ast_probe_peak(int32_t device, int32_t kind, double* gflops);

/* ---------------------------------------------------------------- batched fits
 * Many objects -- each with its own model variant, light curve, filter and parameter counts,
 * seed and caps -- fitted by one persistent launch over a shared pool of chain slots, captured
 * once as a CUDA graph and replayed by ast_batch_run.  No reference counterpart: the reference
 * fits one object per process (asteroid.c:main).  Each object's results are those ast_fit gives
 * for the same model, observations and configuration (one stage: cfg->n_stages must be 1).  All
 * objects of a batch share the precision and the ACC flag given at creation. */
typedef struct ast_batch ast_batch;

typedef struct ast_batch_launch {
    int32_t tpb;          /* threads per CTA (32..256, multiple of 32) */
    int32_t refill;       /* 1: a slot takes a new chain as soon as its own finishes (thread per
                             chain); 32: a warp takes 32 chains of one object at once (warp per
                             object, no divergence between light curves) */
    int32_t ctas;         /* CTAs of the launch (output) */
    double evals_per_s;   /* rate measured by ast_batch_tune (output) */
    int32_t tile;         /* 0: every lane integrates and evaluates its own chain's whole light
                             curve; 8, 16 or 32 (refill 32, mixed-precision ACC batches): warp per
                             model with observation tiles -- the warp's 32 chains are integrated
                             one per lane through a tile of this many observations, then the
                             tile's 32 x T magnitudes are spread over the lanes (same results) */
} ast_batch_launch;

/* n_slots: persistent chain slots (0 = 256 per SM). */
int ast_batch_create(int32_t device, int32_t precision, int32_t acc, int64_t n_slots, ast_batch** out);
/* Upload one object; *index numbers objects from 0 in the order added. */
int ast_batch_add(ast_batch* batch, const ast_model* model, const ast_obs_set* obs, const ast_fit_cfg* cfg,
                  int32_t* index);
/* Autotuner: times every (tpb, refill, tile) candidate on this batch with bounded launches of
 * evals_per_slot evaluations per slot, keeps the fastest for ast_batch_run / ast_batch_step and
 * returns it.  Call it before those: it leaves the batch in its initial state. */
int ast_batch_tune(ast_batch* batch, int64_t evals_per_slot, ast_batch_launch* best);
/* Run every chain of every object to completion (tune NULL: the tuned or default geometry). */
int ast_batch_run(ast_batch* batch, const ast_batch_launch* tune, double* kernel_ms);
/* Alternatively, advance the batch in bounded launches of evals_per_slot evaluations per slot
 * (no graph; *done = 1 once every chain has finished and the results are in).  The batch runs
 * once: either ast_batch_run or ast_batch_step to completion. */
int ast_batch_step(ast_batch* batch, int64_t evals_per_slot, int32_t* done, double* kernel_ms);
/* Results of object index, laid out as ast_fit_out of ast_fit (n_evals not filled). */
int ast_batch_result(ast_batch* batch, int32_t index, ast_fit_out* out);
int ast_batch_counters(ast_batch* batch, int64_t* n_evals, int64_t* n_fits, int32_t* tpb, int32_t* refill,
                       int32_t* ctas);
/* The launch geometry the batch runs with (tpb, refill, ctas, tile); evals_per_s is 0. */
int ast_batch_geometry(ast_batch* batch, ast_batch_launch* out);
/* Set the geometry (tpb, refill, tile of *geometry) for the following ast_batch_step calls,
 * instead of the tuned or default one. */
int ast_batch_set_geometry(ast_batch* batch, const ast_batch_launch* geometry);
void ast_batch_destroy(ast_batch* batch);

/* ---------------------------------------------------------------- serving
 * Continuous batching of fit requests: ast_submit queues a request (an object and its fit
 * configuration, n_stages = 1); each ast_server_step admits queued requests in arrival order
 * while their device footprint (observations, start points, chain and group results) fits the
 * HBM budget, runs the shared slot pool for evals_per_slot evaluations per slot, and retires the
 * requests whose chains have all finished (results to the host, memory freed).  A request's
 * chains start as soon as the chains submitted before it are taken, while those still run;
 * its result does not depend on what else is in flight.  No reference counterpart. */
typedef struct ast_server ast_server;

/* hbm_budget_bytes <= 0: 150 GiB. */
int ast_server_create(int32_t device, int32_t precision, int32_t acc, int64_t n_slots, int64_t hbm_budget_bytes,
                      ast_server** out);
/* Lanes per chain, 1 (default) or 4, set before the first ast_server_step.  With 4, the lanes
 * of a chain evaluate the points its next simplex move may need side by side (the reflection,
 * expansion and contraction of an iteration; the start and shrunk vertices four at a time), and
 * its leader keeps the sequential order: the same results, about half the sequential rounds per
 * chain -- lower latency while few requests are in flight, a quarter of the chains per slot. */
int ast_server_set_lanes(ast_server* server, int32_t lanes_per_chain);
int ast_submit(ast_server* server, const ast_model* model, const ast_obs_set* obs, const ast_fit_cfg* cfg,
               int64_t* request);
int ast_server_step(ast_server* server, int64_t evals_per_slot, int32_t* n_running, int32_t* n_queued);
/* 1 and the result (and the seconds from ast_submit to retirement) once the request is done,
 * 0 while it is queued or running, AST_E_CANCELLED after ast_cancel, < 0 on other errors. */
int ast_poll(ast_server* server, int64_t request, ast_fit_out* out, double* latency_s);
/* Cancel a request (no reference counterpart: the reference runs one fit per process).  A queued
 * request leaves the queue at once.  A running one is dropped by the next ast_server_step: its
 * slots abandon its chains and take other work, and once every chain is accounted for, the
 * request retires without results and its device memory returns to the HBM budget; the other
 * requests' results do not change.  Returns 0, or 1 when the request had already finished (its
 * result stays available). */
int ast_cancel(ast_server* server, int64_t request);
int ast_server_stats(ast_server* server, int64_t* n_evals, double* kernel_ms, int64_t* hbm_used,
                     int64_t* hbm_budget);
/* Device bytes the request holds while admitted (what admission counts against the budget). */
int64_t ast_request_bytes(ast_server* server, int64_t request);
void ast_server_destroy(ast_server* server);

/* Library version string. */
const char* ast_version(void);

#ifdef __cplusplus
}
#endif
#endif /* ASTEROID_GB300_H */
