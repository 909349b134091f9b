/*
 * rsd_capi.h -- C-ABI of the GB300 (sm_103a) hydrodynamic step of
 * regularized Stokesian dynamics.
 *
 * Every entry point replaces one subroutine of the Fortran reference
 * (sherlockyzd/Regularized-Stokesian-Dynamics); the comment above each one
 * names the routine and its file:line.  Conventions follow the Fortran side:
 *   - all host arrays are column-major, leading dimension = row count, no
 *     padding; p_pos is (3, nn), so particle a sits at p_pos[3a .. 3a+2];
 *   - outputs are fully overwritten; inputs are not modified except where an
 *     entry says "in place" (rsd_matrev, like MATREV);
 *   - return 0 on success, a positive LAPACK-style INFO (leading minor k is
 *     not positive definite) from the factorisations, or a negative RSD_E*
 *     code; rsd_ctx_last_error() then holds a one-line message;
 *   - one host thread per context; calls are synchronous with respect to the
 *     host arrays they take (the caller may read outputs on return).
 * Entry points ending in _dev take device pointers (cudaMalloc'ed, on the
 * context's device) and run asynchronously on the context's stream; they
 * return after enqueueing, except where an INFO must be read back.
 */
#ifndef RSD_CAPI_H
#define RSD_CAPI_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define RSD_OK 0
#define RSD_EARG (-1)     /* invalid argument (size, null pointer, lattice) */
#define RSD_ECUDA (-2)    /* CUDA runtime error */
#define RSD_ENAN (-3)     /* non-finite input or result */
#define RSD_ETIMEOUT (-4) /* a bounded device wait ran out */
#define RSD_ENOMEM (-5)   /* device allocation failed */
#define RSD_EIO (-6)      /* lubrication table files unreadable */
#define RSD_EUNSUP (-7)   /* option of the reference not built here */
#define RSD_ELIMIT (-8)   /* request beyond the static scratch of the allocation-free entry point */
#define RSD_ENOCONV (-9)  /* mixed form: the FP64 refinement (stationary, then flexible GMRES) did not reach
                             100 x its tolerance; the outputs hold the last iterate */

typedef struct rsd_ctx rsd_ctx;
typedef struct rsd_lubtab rsd_lubtab;

/* Module LATTICE_BASE (src/mymodules.f90:33-42): the Lees-Edwards lattice
 * LR (3x3, column-major), its inverse LI, the cell volume LV, and the Ewald
 * parameters that CALC_LATTICE_INVERSE derives from them. */
typedef struct rsd_lattice {
  double LR[9];
  double LI[9];
  double LV;
  double lammda; /* Ewald splitting parameter, sqrt(pi)/LV^(1/3) */
  double sig;
  double logerr;
  double phi; /* volume fraction sum(4/3 pi a^3)/LV */
  int32_t NR; /* real-space images in [-NR,NR]^3 */
  int32_t NI; /* reciprocal vectors in [-NI,NI]^3 \ {0} */
} rsd_lattice;

/* ---------------------------------------------------------------- context */
/* Creates a context on CUDA device `device` (one stream, grow-only device
 * buffers reused across calls). */
int rsd_ctx_create(rsd_ctx** ctx, int device);
int rsd_ctx_destroy(rsd_ctx* ctx);
const char* rsd_ctx_last_error(const rsd_ctx* ctx);
/* The context's CUDA stream (a cudaStream_t), for callers that want to order
 * their own work after _dev calls. */
void* rsd_ctx_stream(rsd_ctx* ctx);
/* Device-time of the last step's phases in milliseconds: assembly, lub,
 * solve (including the update), and the refinement part of the solve (mixed
 * form; 0 otherwise), measured with CUDA events on the context stream. */
int rsd_ctx_phase_ms(const rsd_ctx* ctx, double ms[4]);
/* Diagnostic (no counterpart in the reference): kernel launches issued by
 * this library since it was loaded, over all contexts. */
long long rsd_launch_count(void);
/* Tensor cores in the FP32 factorisations of the mixed-precision form:
 * 1 (the default) = tcgen05 kernels wherever the layout allows (16-byte
 * aligned blocks, leading dimension a multiple of 4), TF32 for the factor of
 * the grand mobility and the inverse of its Schur factor, 3xTF32 (close to
 * FP32) for the factor of RPP; 3 = 3xTF32 for all three (at most one
 * refinement iteration fewer); 0 = FP32 SIMT kernels only.  The FP64 form
 * is unaffected. */
int rsd_ctx_set_tensor_cores(rsd_ctx* ctx, int mode);
/* Precision split of the mixed-precision Ewald assembly: real-space images
 * with lammda*r < lam_r_cut (at most 6) and reciprocal vectors with
 * k^2/(4 lammda^2) <= 3 pi kshell^2 (on a cubic cell at the reference's
 * lammda: max|n_i| <= kshell) are summed in double-single (~1e-14), the
 * rest in FP32.  Defaults 4.5 and 1. */
int rsd_ctx_set_mixed_split(rsd_ctx* ctx, double lam_r_cut, int32_t kshell);
/* Truncation of the mixed-precision Ewald sums inside the reference's image
 * cubes: real-space images with lammda*r >= lam_r_max and reciprocal vectors
 * with k^2/(4 lammda^2) >= k2_over_4lam2_max are dropped.  Defaults 6.0 and
 * 10 pi: each changes a mobility block by less than ~1e-12 of its largest
 * entry (the reference's cubes reach lammda*r ~ 10 and k^2/(4 lammda^2) ~
 * 85 at zero strain).  The FP64 form always sums the whole cubes. */
int rsd_ctx_set_mixed_truncation(rsd_ctx* ctx, double lam_r_max, double k2_over_4lam2_max);
/* Ewald splitting parameter of the mixed-precision assembly relative to the
 * reference's lammda = sqrt(pi)/LV^(1/3).  The Ewald sum does not depend on
 * it; a larger value moves work from the real-space images to the cheaper
 * reciprocal vectors, and the image cubes are widened to hold the
 * truncation spheres.  1 keeps the reference's lammda, NR and NI; the
 * default is 1.75.  The FP64 form always uses the reference's values. */
int rsd_ctx_set_mixed_lambda_scale(rsd_ctx* ctx, double scale);
/* Equal radii, mixed-precision assembly: the double-single near images are
 * summed in `passes` passes (1 to 4), each over one part of the moments
 * (fewer live accumulators and a shorter loop per pass; r, erfc and exp are
 * evaluated once per pass).  A performance setting; the sums are the same. */
int rsd_ctx_set_mixed_real_passes(rsd_ctx* ctx, int32_t passes);
/* Overlap corrections in the fused step (rsd_stepper_stokesian): the
 * correction_method of per_GRPY_YZD.f90:98-116 (0 none, the default; 1
 * Yamakawa; 2 regularized), added to the grand mobility of either precision
 * form for the pairs whose minimum image overlaps. */
int rsd_ctx_set_correction_method(rsd_ctx* ctx, int32_t method);

/* Refinement of the mixed-precision form (no counterpart in the reference,
 * which solves in FP64 directly): mode 0 (the default) = the stationary
 * iteration x += P (b - A x), P the correction that the FP32 factors give,
 * FP64 residuals; it stops at the step's relative residual tolerance, or
 * within 100 times it once an iteration no longer halves the residual (the
 * floor of the residual arithmetic on stiff systems).  When it diverges
 * (its residual grows 1000 times above its best) or ends above 100 times the
 * tolerance, flexible GMRES finishes the solve from zero
 * (rsd_step_info.fallback = 1).  Mode 1 = flexible GMRES alone, with the
 * same preconditioner and FP64 residuals, restarted every `restart`
 * iterations (1..30, 0: 30).  A solve that ends above 100 times the
 * tolerance returns RSD_ENOCONV. */
int rsd_ctx_set_refinement(rsd_ctx* ctx, int32_t mode, int32_t restart);
/* Bounds of the device-side waits of the mixed form's FP32 kernels (no
 * counterpart in the reference): every mbarrier wait of the tensor-core
 * GEMMs gives up after tc_wait_ns nanoseconds (0: the default, 0.5 s), and
 * every wait of the refinement's dataflow triangular sweeps after
 * tri_spin_polls polls of at least 64 ns (0: the default, 2^21).  A wait
 * that gives up ends its kernel without a fault: the kernel drains the
 * copies and MMAs it issued, frees its tensor memory, skips its stores and
 * raises an error word; the call returns RSD_ETIMEOUT and the context stays
 * usable.  Values far below the defaults only serve to exercise that path. */
int rsd_ctx_set_wait_limits(rsd_ctx* ctx, int64_t tc_wait_ns, int64_t tri_spin_polls);
/* Schedule of the mixed form's FP32 Cholesky factorisations on tensor
 * cores: 1 (default) keeps only the next diagonal tile on the chain of
 * diagonal blocks and runs the wide row-panel work on a second stream beside
 * the next block's factor; 0 runs each 128-wide step's panel work in order
 * before the next factor.  Both give the same factor up to the order of
 * FP32 sums. */
int rsd_ctx_set_factor_schedule(rsd_ctx* ctx, int32_t schedule);

/* ---------------------------------------------------------------- lattice */
/* SET_LATTICE_SKEW (src/csd_post.f90:105-136) with MAT_INV3
 * (src/tensors.f90:704-726): fills lat->LR, LI, LV for strain time T. */
int rsd_set_lattice_skew(double T, const double LB[3], double gamma, int32_t oscillation, double gamma_alpha,
                         double frequency, rsd_lattice* lat);
/* CALC_LATTICE_INVERSE (src/csd_post.f90:158-183): lammda, sig, logerr, NR,
 * NI and phi from LR, LV, EWS_ERR and the radii (module side effects that
 * yetamu_solve later reads). */
int rsd_calc_lattice_inverse(rsd_lattice* lat, double ews_err, int32_t nn, const double* radii);

/* ------------------------------------------------- kernel 1: grand mobility */
/* PER_GRPERY_INV_FRI (src/per_GRPY_YZD.f90:13-200): Ewald-summed periodic
 * grand mobility, scaled by 1/(pi mu_f), split into APP (6nn x 6nn),
 * APQ (6nn x 5nn), AQQ (5nn x 5nn).  Calls CALC_LATTICE_INVERSE first and
 * leaves its results in *lat.  correction_method (per_GRPY_YZD.f90:98-116)
 * acts on pairs whose minimum image overlaps or touches (r <= a_i + a_j):
 * 0 none; 1 adds Yamakawa's overlapping-sphere blocks minus the free-space
 * pair (overlap_Yamakawa_CORRECTION_IJ, GRPY_YZD.f90:789-811); 2 adds the
 * regularized pair blocks of Regularization.f90 minus the free-space pair
 * (overlap_Regular_CORRECTION_IJ, 813-836; NaN for a pair at exact contact,
 * as in the reference); other values return RSD_EARG. */
int rsd_per_grpery_inv_fri(rsd_ctx* ctx, int32_t nn, const double* p_pos, const double* radii, rsd_lattice* lat,
                           double ews_err, double mu_f, int32_t correction_method, double* APP, double* APQ,
                           double* AQQ);
/* Same on device: writes the whole grmobmx (11nn x 11nn, leading dimension
 * ldm >= 11nn) in the reference's row/column order. */
int rsd_per_grpery_inv_fri_dev(rsd_ctx* ctx, int32_t nn, const double* d_pos, const double* d_radii,
                               rsd_lattice* lat, double ews_err, double mu_f, int32_t correction_method,
                               double* d_grmobmx, int64_t ldm);

/* Allocation-free variant of rsd_per_grpery_inv_fri_dev.  No counterpart in
 * the reference: it serves callers that cannot call cudaMalloc -- programs
 * that give all device memory to their own fixed pool at start, and
 * time-step loops that cannot afford the device-wide synchronisation
 * cudaMalloc/cudaFree imply.  It takes no context, allocates nothing and runs
 * on `stream` (a cudaStream_t, NULL for the default stream) on the current
 * device; the caller passes the inputs and the output, as in the _dev entry
 * point.  Its one scratch buffer, the reciprocal-vector weight table, is a
 * static device array of about 1.6 MB that every GPU loading the library
 * holds until exit; it fits at most 2456 reciprocal vectors in the half space
 * (NI <= 8: EWS_ERR above about 5e-88 in a cubic box), and a larger request
 * returns RSD_ELIMIT before any kernel that writes the output runs.  All
 * calls on a device share that array and it keeps the last call's contents:
 * calls that overlap on the GPU race and must be serialised by the caller.
 * The first call on each device looks the array's address up with that
 * device current.  The call synchronises `stream` once, to read the radii's
 * cube sum back for NR, NI and phi, and returns once the rest is enqueued. */
int rsd_per_grpery_inv_fri_static(int32_t nn, const double* d_pos, const double* d_radii, rsd_lattice* lat,
                                  double ews_err, double mu_f, double* d_grmobmx, int64_t ldm, void* stream);

/* ------------------------------------------- kernel 2: lubrication R_lub-R_2B */
/* The three tables lubtabcalc reads once (src/hydro_lub.f90:529-596):
 * r2babc.dat (39 rows x 11), r2bgh.dat (47 x 7), r2bm.dat (47 x 4), each
 * with one header line, from directory `dir` (the reference opens
 * lubdat/ relative to its working directory). */
int rsd_lubtab_load(rsd_lubtab** tab, const char* dir);
/* Same tables from memory, rows in file order (row-major per row). */
int rsd_lubtab_create(rsd_lubtab** tab, int32_t nabc, const double* abc, int32_t ngh, const double* gh, int32_t nm,
                      const double* m);
int rsd_lubtab_destroy(rsd_lubtab* tab);
/* lubmxcalc (src/hydro_lub.f90:22-308): dense rfu (6nn x 6nn),
 * rfe (6nn x 5nn), rse (5nn x 5nn).  Pairs with s = r/a_avg <= 2 are
 * mirrored to 4.00001 - s like the reference; *n_contact (may be NULL)
 * returns how many.  nb trailing boundary particles are skipped. */
int rsd_lubmxcalc(rsd_ctx* ctx, const rsd_lubtab* tab, int32_t nn, int32_t nb, int32_t is_period,
                  const double* p_pos, const double* radii, const rsd_lattice* lat, double mu_f, double* rfu,
                  double* rfe, double* rse, int32_t* n_contact);
/* Same on device, written into the grand layout L = [rfu rfe; rfe^T rse]
 * (11nn x 11nn, leading dimension ldl).  accumulate != 0 adds L into d_L
 * (arrangResist, src/matrices.f90:218-228) instead of overwriting it. */
int rsd_lubmxcalc_dev(rsd_ctx* ctx, const rsd_lubtab* tab, int32_t nn, int32_t nb, int32_t is_period,
                      const double* d_pos, const double* d_radii, const rsd_lattice* lat, double mu_f, double* d_L,
                      int64_t ldl, int32_t accumulate, int32_t* n_contact);

/* --------------------------------------------- kernel 3: grand resistance */
/* MATREV (src/matrices.f90:4-34): SPD inverse in place (upper Cholesky,
 * inverse, upper triangle mirrored).  *info > 0 as DPOTRF's INFO; the
 * reference prints and continues, so A then holds an undefined result. */
int rsd_matrev(rsd_ctx* ctx, int32_t n, double* A, int32_t* info);
int rsd_matrev_dev(rsd_ctx* ctx, int32_t n, double* d_A, int64_t lda, int32_t* info);
/* CHOLESKY (src/matrices.f90:126-157): lower factor, strict upper part
 * zeroed.  Returns the positive INFO when not SPD (the reference stops). */
int rsd_cholesky(rsd_ctx* ctx, int32_t n, double* B, int32_t* info);
/* MobToResist_FTS (src/matrices.f90:393-416): RPP, RPQ, RQQ blocks of the
 * inverse of [APP APQ; APQ^T AQQ]. */
int rsd_mob_to_resist_fts(rsd_ctx* ctx, int32_t nn, const double* APP, const double* APQ, const double* AQQ,
                          double* RPP, double* RPQ, double* RQQ, int32_t* info);
/* arrangement (src/matrices.f90:432-445): mu = RPQ^T RPP^-1 RPQ - RQQ. */
int rsd_arrangement(rsd_ctx* ctx, int32_t nn, const double* RPP, const double* RPQ, const double* RQQ, double* mu,
                    int32_t* info);
/* STEPPER_NOGmres (src/stepper.f90:348-410) for the FTS path, with
 * MobToResist_FTS, arrangResist, arrangement and Rheology (412-447):
 * U_par = RPP^-1 (Fe + RPQ EIN), SijN_hyd = mu EIN,
 * SijN_FP = RPQ^T RPP^-1 Fe_inter + sym(x (x) F) in Y2,
 * SijN_B = RPQ^T UB.  On return RPP holds the inverse of RPP0 + rfu, as the
 * reference's Rheology leaves it.  u_brown (3nn) may be NULL (zero). */
int rsd_stepper_nogmres(rsd_ctx* ctx, int32_t nn, const double* APP, const double* APQ, const double* AQQ,
                        const double* rfu, const double* rfe, const double* rse, const double* Fe, const double* EIN,
                        const double* Fe_inter, const double* conf, const double* u_brown, double* U_par,
                        double* SijN_hyd, double* SijN_FP, double* SijN_B, double* RPP, int32_t* info);

/* DMDX_CAL (src/stepper.f90:664-688): the Brownian drift term
 * DMDX = (A1 - A2) Z / deta, A1 and A2 the translational blocks
 * APP(1:3nn, 1:3nn) of the grand mobility (PER_GRPERY_INV_FRI with lat,
 * ews_err = LINERR, mu_f, correction_method) at conf +- deta Z / 2, with
 * deta the REAL*8 value of the default-real literal 0.001 (1.0000000474974513e-3).
 * conf and Z as the reference's CONF(3, nn) and Z(3 nn). */
int rsd_dmdx_cal(rsd_ctx* ctx, int32_t nn, const double* conf, const double* radii, rsd_lattice* lat, double ews_err,
                 double mu_f, int32_t correction_method, const double* Z, double* DMDX);
/* The Brownian velocity of STEPPER_Stokesian with BROWN (src/stepper.f90:
 * 72-86): CHOLESKY of A = APP(1:3nn, 1:3nn) (APP the caller's 6nn x 6nn
 * mobility block at conf), VB = sqrt(2 kBT) L Z / dt, and
 * u_brown = VB + kBT DMDX_CAL(Z).  Z (3nn) are the standard normal numbers
 * that the reference draws with GAUSS (the caller draws them).  info is
 * CHOLESKY's (positive: A not SPD, nothing written; the reference stops). */
int rsd_brownian_velocity(rsd_ctx* ctx, int32_t nn, const double* APP, const double* conf, const double* radii,
                          rsd_lattice* lat, double ews_err, double mu_f, int32_t correction_method, const double* Z,
                          double kBT, double dt, double* u_brown, int32_t* info);
/* hydro_SD_FTS (src/stepper.f90:476-546), the FTS solve of the GMRES
 * variant (useGMRESmethod).  The reference alternates two GMRES(2) solves,
 * a mobility one and a lubrication one, until the FTS residual is below
 * LINERR 1e-2; its inner tolerance (1e-12 relative) can hold the residual
 * above that, after which it returns the last velocity iterate and leaves
 * SijN unassigned.  This returns the solution that the iteration
 * approaches, solved directly: U_par = RPP^-1 (Fe + RPQ EIN) and
 * SijN = RPQ^T U_par - RQQ EIN (R = MobToResist_FTS(A) + [rfu rfe; . rse]).
 * info as MATREV's (mobility, then RPP); on info != 0 the outputs are not
 * written. */
int rsd_hydro_sd_fts(rsd_ctx* ctx, int32_t nn, const double* APP, const double* APQ, const double* AQQ,
                     const double* rfu, const double* rfe, const double* rse, const double* Fe, const double* EIN,
                     double* U_par, double* SijN, int32_t* info);

/* ------------------------------------------------------------ fused step */
#define RSD_PREC_FP64 0  /* plain: every kernel in FP64 */
#define RSD_PREC_MIXED 1 /* FP32 bulk + FP64 near terms and refinement */

typedef struct rsd_step_params {
  int32_t nn;        /* particles */
  int32_t nb;        /* trailing boundary particles (skipped by lub) */
  double LB[3];      /* box edges */
  double T;          /* time at the start of the step (strain = gamma T) */
  double dt;         /* time step */
  double gamma;      /* shear rate */
  double mu_f;       /* dimensionless viscosity (1/pi for the reference's units) */
  double ews_err;    /* Ewald tolerance EWS_ERR = LINERR */
  int32_t use_lub;   /* uselub */
  int32_t precision; /* RSD_PREC_FP64 or RSD_PREC_MIXED */
  double tol;        /* mixed: relative residual target of the refinement (0: 1e-12) */
  int32_t max_iter;  /* mixed: refinement iteration cap (0: 50) */
} rsd_step_params;

typedef struct rsd_step_info {
  int32_t info;       /* positive: leading minor not SPD (plain path) */
  int32_t n_contact;  /* lub pairs with s <= 2 */
  int32_t NR, NI;     /* Ewald images used */
  int32_t iterations; /* mixed: refinement iterations */
  double residual;    /* mixed: final relative residual */
  double phi;         /* volume fraction */
  double LV;          /* cell volume */
  int32_t rpp_iterations; /* FP64 form with a PCG RPP solver: its iterations
                             (negative: not converged, factorised instead) */
  int32_t fallback;   /* mixed: 1 when the stationary refinement diverged or
                         stalled and flexible GMRES finished the solve */
} rsd_step_info;

/* One STEPPER_Stokesian step (src/stepper.f90:33-156) on the periodic FTS
 * path with lubrication: SET_LATTICE_SKEW, PER_GRPERY_INV_FRI, lubmxcalc,
 * STEPPER_NOGmres, INIT_uo_bg/calc_uo_bg (src/csd_post.f90:442-522),
 * STEPPER_conf with PERIOD_CORRECTION (src/stepper.f90:160-227,
 * src/csd_post.f90:65-102) and yetamu_solve (src/csd_post.f90:313-367).
 * conf (3 x nn) is advanced in place; U_pos (6nn), SijN (5nn, the hydrodynamic
 * stresslet SijN_hyd) and yeta_mu[5] are written.  Fe (6nn) may be NULL. */
int rsd_stepper_stokesian(rsd_ctx* ctx, const rsd_lubtab* tab, const rsd_step_params* p, double* conf,
                          const double* radii, const double* Fe, double* U_pos, double* SijN, double yeta_mu[5],
                          rsd_step_info* info);
/* Same with device-resident arrays (no host copies). */
int rsd_stepper_stokesian_dev(rsd_ctx* ctx, const rsd_lubtab* tab, const rsd_step_params* p, double* d_conf,
                              const double* d_radii, const double* d_Fe, double* d_U_pos, double* d_SijN,
                              double yeta_mu[5], rsd_step_info* info);

/* --------------------------------- learned preconditioner of the RPP solve */
/* The resistance solve of STEPPER_NOGmres (src/stepper.f90:370-393,
 * MATREV(RPP)) by preconditioned conjugate gradients in FP64 instead of a
 * dense Cholesky factorisation.  The reference has no counterpart: it always
 * factors RPP (LAPACK DPOTRF/DPOTRI).  The preconditioner is a block-sparse
 * approximate inverse G = D^-1/2 Z^T Z D^-1/2 of RPP (D its diagonal, Z
 * block lower triangular with 6 x 6 blocks on each particle and on each pair
 * of particles closer than 3 a_avg, b < a), either exact (the factorised
 * sparse approximate inverse, from one local dense solve per particle) or
 * learned: a 3-layer message-passing network (hidden width 64, BF16 weights
 * and activations, FP32 accumulation) over those pairs, whose inputs are the
 * Jacobi-scaled blocks of RPP and the pair gaps, emits the direction
 * W_ab = Z_aa^-1 Z_ab of every pair block, and each row block of Z is
 * normalised from the local matrix so that (Z A Z^T)_aa = I (G is SPD
 * whatever the network emits). */
#define RSD_PC_NONE 0
#define RSD_PC_JACOBI 1
#define RSD_PC_BLOCK_JACOBI 2
#define RSD_PC_FSAI 3
#define RSD_PC_LEARNED 4
typedef struct rsd_lp rsd_lp;
/* Number of network parameters (FP32). */
int64_t rsd_lp_param_count(void);
/* A network on CUDA device `device`: from `params` (rsd_lp_param_count()
 * FP32 values, e.g. trained weights) or, when NULL, initialised from `seed`. */
int rsd_lp_create(rsd_lp** net, int device, const float* params, uint64_t seed);
int rsd_lp_destroy(rsd_lp* net);
/* Current parameters and/or last gradient to host arrays (either may be NULL). */
int rsd_lp_get_params(rsd_lp* net, float* params, float* grad);
/* The near-neighbour graph of a configuration: edges (a <- b), b != a, with
 * minimum-image centre distance below 3 (a_a + a_b)/2, in CSR by a (h_off,
 * nn + 1), sources ascending (h_src), surface gaps (h_gap); any of the host
 * arrays may be NULL (n_edges alone sizes them). */
int rsd_lp_graph_dev(rsd_ctx* ctx, int32_t nn, const double* d_pos, const double* d_radii, const rsd_lattice* lat,
                     int32_t* n_edges, int32_t* h_off, int32_t* h_src, float* h_gap);
/* The network alone on a given graph (CSR d_off, edges d_src -> d_dst) and
 * FP32 inputs d_xn (nn x 36) and d_xe (ne x 40): outputs the blocks d_zd
 * (nn x 36) and d_ze (ne x 36); when d_dzd and d_dze are given, also the
 * gradient of the parameters for those output gradients (read it with
 * rsd_lp_get_params). */
int rsd_lp_forward_dev(rsd_ctx* ctx, rsd_lp* net, int32_t nn, int32_t ne, const int32_t* d_off, const int32_t* d_src,
                       const int32_t* d_dst, const float* d_xn, const float* d_xe, const float* d_dzd,
                       const float* d_dze, float* d_zd, float* d_ze);
/* One Adam step (beta 0.9, 0.999, eps 1e-8) on the stored gradient, scaled
 * to norm clip_norm when it is larger (rsd_lp_set_training); a gradient
 * whose norm is not finite makes no update. */
int rsd_lp_adam_step(rsd_lp* net, float lr);
/* Training guards: clip_norm > 0 clips the gradient to that global norm;
 * max_loss > 0 makes a train step whose loss is larger (or not finite) make
 * no update.  0 switches either off (the default). */
int rsd_lp_set_training(rsd_lp* net, float clip_norm, double max_loss);
/* The norm of the last gradient, the train steps that made no update and the
 * Adam steps taken; any pointer may be NULL. */
int rsd_lp_training_stats(rsd_lp* net, double* last_grad_norm, int64_t* skipped, int64_t* steps);
/* One training step on one resistance matrix: d_rpp (6nn x 6nn, grand
 * layout, ld, FP32 if fp32 != 0 else FP64, full symmetric storage) of the
 * configuration d_pos/d_radii on lattice lat; the targets are the
 * directions W of its exact FSAI; loss returns their mean squared error
 * before the step (a loss above the max_loss of rsd_lp_set_training, or not
 * finite, makes no update). */
int rsd_lp_train_step(rsd_ctx* ctx, rsd_lp* net, int32_t nn, const double* d_pos, const double* d_radii,
                      const rsd_lattice* lat, int32_t fp32, const void* d_rpp, int64_t ld, float lr, double* loss);
/* The blocks of Z for mode RSD_PC_BLOCK_JACOBI, RSD_PC_FSAI or
 * RSD_PC_LEARNED to host arrays (h_zd nn x 36, h_ze n_edges x 36 in the
 * graph's edge order; entries of edges (a <- b) with b >= a are not used). */
int rsd_lp_blocks_dev(rsd_ctx* ctx, rsd_lp* net, int32_t mode, int32_t nn, const double* d_pos, const double* d_radii,
                      const rsd_lattice* lat, int32_t fp32, const void* d_rpp, int64_t ld, float* h_zd, float* h_ze,
                      int32_t* n_edges);
/* RPP x = b by PCG in FP64 (d_rpp FP64, full symmetric storage in the grand
 * layout, ld; d_b, d_x: nrhs columns of 6nn) with preconditioner `mode`
 * (net only for RSD_PC_LEARNED), to relative residual tol or maxit
 * iterations; iters and resid return the largest over the columns. */
int rsd_lp_pcg_dev(rsd_ctx* ctx, rsd_lp* net, int32_t mode, int32_t nn, const double* d_pos, const double* d_radii,
                   const rsd_lattice* lat, const double* d_rpp, int64_t ld, int32_t nrhs, const double* d_b,
                   double* d_x, double tol, int32_t maxit, int32_t* iters, double* resid);
/* RPP = (M^-1)_PP + rfu of one configuration (the matrix STEPPER_NOGmres
 * factors), into d_rpp (6nn x 6nn, ld): FP64 through the plain FP64 path
 * (precision RSD_PREC_FP64) or FP32 through the mixed form's factors
 * (RSD_PREC_MIXED, about 1e-4 relative).  p->T sets the strain; lat returns
 * the lattice. */
int rsd_resistance_pp_dev(rsd_ctx* ctx, const rsd_lubtab* tab, const rsd_step_params* p, const double* d_conf,
                          const double* d_radii, void* d_rpp, int64_t ld, rsd_lattice* lat);
/* The RPP solve of the plain FP64 fused step: mode RSD_PC_NONE keeps the
 * Cholesky factorisation (the default); RSD_PC_JACOBI, RSD_PC_BLOCK_JACOBI,
 * RSD_PC_FSAI or RSD_PC_LEARNED (with `net`) use PCG to relative residual
 * tol (0: 1e-12) within maxit iterations (0: 1000), falling back to the
 * Cholesky factorisation when it does not converge.  rsd_step_info reports
 * the iterations. */
int rsd_ctx_set_rpp_solver(rsd_ctx* ctx, int32_t mode, rsd_lp* net, double tol, int32_t maxit);

/* ------------------------------------------ FP32 blocks of the mixed form */
/* The reference solves in FP64 only (LAPACK DPOTRF/DPOTRI); these are the
 * single-precision building blocks that the mixed form's refinement uses as a
 * preconditioner, exported for testing and for callers that build their own
 * refinement.  Device pointers, column-major.  prec selects the product
 * arithmetic: 0 = FP32 SIMT, 1 = TF32 tensor cores, 3 = 3xTF32 tensor cores
 * (head/tail split, close to FP32); the tensor-core forms need 16-byte
 * aligned pointers and leading dimensions that are multiples of 4, and fall
 * back to SIMT otherwise. */
/* C (n x n, the 128 x 128 tiles on and above the diagonal) -= P^T P with P
 * k x n (ld ldp); k <= 128 for the tensor-core path. */
int rsd_syrk_f32_dev(rsd_ctx* ctx, int32_t n, int32_t k, const float* d_P, int64_t ldp, float* d_C, int64_t ldc,
                     int32_t prec);
/* Upper Cholesky factor in place (lower triangle left as scratch); info as
 * DPOTRF. */
int rsd_potrf_f32_dev(rsd_ctx* ctx, int32_t n, float* d_A, int64_t lda, int32_t prec, int32_t* info);
/* A <- A^-1 (upper triangle; the lower triangle is scratch) from the upper
 * factor in A, as DPOTRI. */
int rsd_potri_f32_dev(rsd_ctx* ctx, int32_t n, float* d_A, int64_t lda, int32_t prec);

#ifdef __cplusplus
}
#endif
#endif /* RSD_CAPI_H */
