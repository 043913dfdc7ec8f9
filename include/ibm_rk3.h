/*
 * ibm_rk3.h -- C ABI of the GB300-native immersed-boundary RK3 substep.
 *
 * This is the drop-in boundary for the InterPartS hot path (one RK3 substep
 * of a particle-resolved channel DNS: momentum predictor, multidirect IBM
 * forcing, FFT/tridiagonal pressure projection, sphere integrals, soft-sphere
 * collisions with lubrication, Newton-Euler update).  A single-rank Fortran
 * main program binds these entry points through ISO_C_BINDING; every call
 * replaces one reference subroutine (or one block of the reference driver),
 * cited beside it as file:line within the reference project.
 *
 * Conventions
 *   - Plain C types only: pointers, sizes, doubles, ints.
 *   - Every entry point returns an int status: IBM_OK (0) or a negative code;
 *     ibm_last_error() gives a message for the last failing call.
 *   - Host field arrays use the reference layout exactly: Fortran order
 *     (i fastest) with one ghost layer, shape (0:itot+1, 0:jtot+1, 0:ktot+1),
 *     i.e. (itot+2)*(jtot+2)*(ktot+2) doubles (mod_common, common.f90:4-8).
 *   - All state lives on the GPU between calls; set/get copy it.
 *   - One host thread per context; all work is ordered on the context stream.
 *   - No MPI: the 2-D pencil decomposition of the reference collapses to one
 *     rank with dims=(1,1); halos become periodic index wrap in x and y.
 */
#ifndef IBM_RK3_H
#define IBM_RK3_H

#ifdef __cplusplus
extern "C" {
#endif

#define IBM_ABI_VERSION 3

/* status codes */
#define IBM_OK                 0
#define IBM_E_INVALID        (-1)  /* bad argument or size                        */
#define IBM_E_CUDA           (-2)  /* CUDA runtime error                          */
#define IBM_E_NOMEM          (-3)  /* device allocation failed                    */
#define IBM_E_CONTACT_OVERFLOW (-4)/* a particle exceeded nqmax contacts          */
#define IBM_E_NOT_CONVERGED  (-5)  /* bounded iteration gave up                   */
#define IBM_E_DIVERGENCE     (-6)  /* chkdiv total divergence above 1e-3          */
#define IBM_E_STATE          (-7)  /* call out of order (e.g. no fields set yet)  */

/* boundary condition types for the z walls (param.f90:33-34, bound.f90:17-65) */
#define IBM_BC_NOSLIP   0
#define IBM_BC_FREESLIP 1
/* Periodic z (no counterpart in the reference, whose z boundaries are
 * always walls): set for both bc_top and bc_bot.  The plain FP64 form only,
 * at most one particle (the collision pass has no images across z); no
 * scalar transport, no plane statistics.  Ghost planes are periodic copies,
 * the Poisson solve in z is cyclic (Sherman-Morrison around the Thomas
 * sweep, the zero mode pinned at its last plane), the IBM stencils and the
 * sphere integrals wrap in z, and the particle position wraps in z. */
#define IBM_BC_PERIODIC 2

/* arithmetic forms of the step */
#define IBM_MODE_PLAIN_FP64    0   /* drop-in: FP64 everywhere                    */
#define IBM_MODE_MIXED         1   /* FP32 bulk passes, FP64 where required       */
#define IBM_MODE_MIXED_LEARNED 2   /* MIXED + learned forcing correction          */

/*
 * Run parameters: mod_gridsize (gridsize.f90:6-26), the &parameters namelist
 * (param.f90:66-86) and the Lagrangian force-point table read by coordsfp
 * (coordsfp.f90:21-29).  Derived constants (init.f90:74-243) are computed
 * inside ibm_create exactly as derived_parameters does.
 */
typedef struct ibm_params {
  int    itot, jtot, ktot;     /* grid cells                                   */
  double lx, ly, lz;           /* domain size                                  */
  double visc;                 /* kinematic viscosity                          */
  double radius;               /* sphere radius                                */
  double ratiorho;             /* particle/fluid density ratio                 */
  int    bc_top, bc_bot;       /* IBM_BC_*                                     */
  int    particle_rotation;    /* 0/1 (param.f90:52)                           */
  int    np;                   /* number of spheres (gridsize.f90 np)          */
  int    nl;                   /* Lagrangian points per sphere (must equal the
                                  value derived_parameters computes, main.f90:118-132) */
  const double *thetarc;       /* [nl] polar angle of each point               */
  const double *phirc;         /* [nl] azimuth of each point                   */
  double radfp;                /* radius of the force-point shell              */
  int    nb_copies;            /* 9: single-rank reference collision loop over the
                                  self-neighbour copies nb=0..8 (intgr_nwtn_eulr.f90:358);
                                  1: only nb=0                                 */
  int    mode;                 /* IBM_MODE_*                                   */
  const double *radii;         /* NULL: every sphere has `radius`.  Otherwise
                                  [np] radii (polydisperse, a variant the
                                  reference cannot express: it has one radius
                                  and one nl, param.f90:48, init.f90:129).
                                  Sphere p then has nl_p = nint(pi/3*(12*((r_p-
                                  retrac)*dxi)^2+1)) force points on the shell
                                  r_p - retrac (retrac = 0.3/dxi); thetarc and
                                  phirc hold the nl_p-point tables of the
                                  spheres one after the other (sum of nl_p
                                  entries), nl must equal the largest nl_p
                                  (the capacity of every sphere's Lagrangian
                                  arrays), and radius and radfp are ignored.
                                  Pairs: contact at r_p + r_q; the spring and
                                  dashpot of the effective mass and the
                                  lubrication of the equivalent radius
                                  2 r_p r_q / (r_p + r_q).  The plane
                                  statistics reject it. */
} ibm_params;

/*
 * Particle state, structure of arrays, host pointers.  Mirrors the reference
 * derived type `particle` (common.f90:35-71) plus the RK accumulators `rkp`
 * (common.f90:97-105).  Per-particle arrays have np entries; contact arrays
 * have np*nqmax entries (particle-major: [p*nqmax + q]); nb has np*9 entries
 * ([p*9 + nb], the neighbour flags ap(p)%nb(0:8)); rkp has np*19 entries in
 * the field order of particle_sumrk.  nqmax = min(np+2, 15) (param.f90:100).
 * Lagrangian arrays (np*nl, [p*nl + l]) are optional on set (may be NULL:
 * they are then regenerated from the centres as coordsfp does).  nb may be
 * NULL on set: the flags are then derived from the centres as a warm start
 * does (loadd.f90:362-397); rkp may be NULL (zero).  On get, any member may
 * be NULL (not returned).
 */
typedef struct ibm_particles {
  double *x, *y, *z, *theta, *phi;
  double *u, *v, *w, *omx, *omy, *omz, *omtheta;
  double *intu, *intv, *intw, *intomx, *intomy, *intomz;
  double *colfx, *colfy, *colfz, *coltx, *colty, *coltz;
  double *fxltot, *fyltot, *fzltot, *torqxltot, *torqyltot, *torqzltot, *torqtheta;
  int    *qmax;                /* [np]                                         */
  int    *firstc;              /* [np*nqmax] partner ids (np+1, np+2 = walls)  */
  double *cdx, *cdy, *cdz, *cdxt, *cdyt, *cdzt, *cdut, *cdvt, *cdwt, *cpsi; /* [np*nqmax] */
  int    *nb;                  /* [np*9]                                       */
  int    *mslv;                /* [np] master id (= particle id 1..np)         */
  double *rkp;                 /* [np*19]                                      */
  double *xfp, *yfp, *zfp, *ul, *vl, *wl, *fxl, *fyl, *fzl; /* [np*nl]         */
} ibm_particles;

typedef struct ibm_ctx ibm_ctx;

/* --- context ------------------------------------------------------------ */

/* Creates a context on the current CUDA device and computes the derived
 * parameters (init.f90:74-243) and the solver tables (initsolver,
 * initsolver.f90:10-66).  Replaces the set-up part of program interpt
 * (main.f90:95-195) for one rank.  Returns NULL on failure (see
 * ibm_last_error(NULL)). */
ibm_ctx *ibm_create(const ibm_params *params);
int      ibm_destroy(ibm_ctx *ctx);
const char *ibm_last_error(const ibm_ctx *ctx);
int      ibm_abi_version(void);
/* nqmax and nl as used by the context (param.f90:100, init.f90:129). */
int      ibm_sizes(const ibm_ctx *ctx, int *nqmax, int *nl, int *ncells);

/* --- state transfer ------------------------------------------------------ */

/* Fields u,v,w,p (unew..pnew) and the RK right-hand side kept between stages
 * (durkold.., main.f90:49), reference layout (0:i1,0:j1,0:k1).  Any of durk,
 * dvrk, dwrk may be NULL (taken as zero, as main.f90:218-220 does). */
int ibm_set_fields(ibm_ctx *ctx, const double *u, const double *v, const double *w,
                   const double *p, const double *durk, const double *dvrk,
                   const double *dwrk);
int ibm_get_fields(ibm_ctx *ctx, double *u, double *v, double *w, double *p,
                   double *durk, double *dvrk, double *dwrk);
/* Forced intermediate velocity dudt/dvdt/dwdt after the IBM loop (the input
 * of fillps, main.f90:356-357). */
int ibm_get_intermediate(ibm_ctx *ctx, double *dudt, double *dvdt, double *dwdt);

int ibm_set_particles(ibm_ctx *ctx, const ibm_particles *ps);
int ibm_get_particles(ibm_ctx *ctx, ibm_particles *ps);

/* coordsfp (coordsfp.f90:10-124) followed by intgr_over_sphere(1..3)
 * (main.f90:202-206): Lagrangian points, dVlagr/dVeul and the initial
 * sphere integrals.  vol_calc (may be NULL) receives the type-1 volume of
 * particle 1 (intgr_over_sphere.f90:607-622). */
int ibm_init_particles(ibm_ctx *ctx, double *vol_calc);

/* --- one reference subroutine per call ---------------------------------- */

/* rk1/rk2/rk3 (rk3.f90:13-329) incl. momxp..momzad (mom.f90:8-231):
 * predictor dudt and the stored RHS.  rkiter in 1..3. */
int ibm_rk_predict(ibm_ctx *ctx, int rkiter, double dt);

/* IBM block of the driver (main.f90:286-338): dudtf=dudt, then for
 * ibmiter=0..nl_iter-1: eulr2lagr, complagrforces/updtlagrforces,
 * lagr2eulr, updtintermediatevel; dudt=dudtf.  nl_iter = 3 in the reference. */
int ibm_forcing_loop(ibm_ctx *ctx, double dt, int nl_iter);

/* bounduvw(dudt), fillps, solver2d, boundp, correc, bounduvw(unew),
 * pnew+=p, boundp(pnew)  (main.f90:356-372). */
int ibm_project(ibm_ctx *ctx, int rkiter, double dt);

/* intgr_nwtn_eulr (intgr_nwtn_eulr.f90:12-1514) on one rank. */
int ibm_newton_euler(ibm_ctx *ctx, int rkiter, double dt);

/* One full RK3 time step: rkiter=1..3 of the above (main.f90:268-413). */
int ibm_rk3_step(ibm_ctx *ctx, double dt);
/* nsteps consecutive RK3 steps with a fixed dt. */
int ibm_run(ibm_ctx *ctx, double dt, int nsteps);

/* nsteps RK3 steps with the reference's time-step control (main.f90:425-441):
 * every ioutchk steps chkdiv (IBM_E_DIVERGENCE above a total of 1e-3, as the
 * reference aborts) and chkdt, then dt = 0.75*dtmax.  dt (in: first step's,
 * out: current) and time (may be NULL) are updated in place. */
int ibm_run_adaptive(ibm_ctx *ctx, int nsteps, int ioutchk, double *dt, double *time);

/* Mixed forms: FP32 Poisson solves per projection.  1 (default): one solve
 * of fillps(u*) (double-float Thomas sweep), one correction into the FP32
 * velocity and the double-float pnew; 2: that solve plus one defect-
 * correction solve driven by the double-float divergence residual of the
 * corrected state.  Both end with the divergence at the FP32 rounding level
 * of the velocity state.  The FP64 form always solves once in FP64 (only 1
 * is accepted there). */
int ibm_set_projection_solves(ibm_ctx *ctx, int solves);

/* Kernel of the FP32 momentum predictor of the mixed forms (rk1..rk3 +
 * mom.f90; no counterpart in the reference, which has one CPU loop nest).
 * Each stages the planes of u, v, w, p in shared memory tile by tile:
 * IBM_PREDICTOR_AUTO (default): 16-byte loads through registers, where the
 * rows are a multiple of 4 cells; otherwise, and with IBM_PREDICTOR_PAIRS,
 * 4-byte loads; IBM_PREDICTOR_TMA: tensor-memory-accelerator copies (rows a
 * multiple of 4 cells).  These three share their arithmetic: identical
 * results.  IBM_PREDICTOR_CELLS: one cell per thread (FP32 terms grouped
 * differently, results within FP32 rounding).  The FP64 form has one kernel
 * and ignores this.  IBM_E_INVALID for any other value. */
#define IBM_PREDICTOR_AUTO  0
#define IBM_PREDICTOR_PAIRS 1
#define IBM_PREDICTOR_CELLS 2
#define IBM_PREDICTOR_TMA   3
int ibm_set_predictor_kernel(ibm_ctx *ctx, int kind);
/* CUDA graphs of the RK stages in ibm_rk3_step / ibm_run (default on): each
 * stage (predictor, forcing loop, projection, Newton-Euler) is captured the
 * second time it runs with a given dt and forcing kind, and replayed after;
 * settings that change a stage's launches drop the graphs.  Not used for
 * timed steps, while probing, harvesting or perturbing the forcing, or with
 * scalar transport.  enable = 0: every launch issued directly. */
int ibm_set_step_graphs(ibm_ctx *ctx, int enable);
/* Captures now, without launching them, the stage graphs that steps with
 * this dt and the current settings will replay (both forcing kinds of the
 * learned form), so that no capture falls inside later steps.  Needs one
 * step run before (launch settings initialised outside a capture). */
int ibm_prepare_step_graphs(ibm_ctx *ctx, double dt);

/* --- diagnostics ----------------------------------------------------------- */

/* chkdiv (chkdiv.f90:7-61): total and max |div| of (unew,vnew,wnew) and the
 * 1-based (i,j,k) of the maximum.  Returns IBM_E_DIVERGENCE when tot > 1e-3
 * (the reference aborts there) after filling the outputs. */
int ibm_chkdiv(ibm_ctx *ctx, double *divtot, double *divmax, int ijk[3]);
/* chkdt (chkdt.f90:6-273): stability limit dtmax. */
int ibm_chkdt(ibm_ctx *ctx, double *dtmax);
/* Lagrangian no-slip residual |U_l - u~_l| after the last forcing pass:
 * max and rms over all points. */
int ibm_slip_residual(ibm_ctx *ctx, double *maxres, double *rmsres);
/* wallshearnew/wallshearold (rk3.f90:88-103) and the IBM mean-force
 * diagnostics of updtintermediatevel (forcing.f90:445-463) of the last pass. */
int ibm_diagnostics(ibm_ctx *ctx, double *wallshearnew, double *wallshearold,
                    double forcetot[3]);

/* --- scalar field (runmodes 1001-1003) --------------------------------------- */

#define IBM_BC_C_DIRICHLET 0        /* 'BC_DIRICHLET' (bound.f90:113-122)           */
#define IBM_BC_C_NEUMANN   1        /* 'BC_NEUMANN'   (bound.f90:124-132)           */

typedef struct ibm_scalar_params {
  double pran;                      /* Prandtl number: kappa = visc/Pran (init.f90:94) */
  double beta;                      /* expansion coefficient (param.f90:47)        */
  double bc_c_top_val, bc_c_bot_val;/* wall values (param.f90:41-42)               */
  int    bc_c_top_type, bc_c_bot_type; /* IBM_BC_C_* (param.f90:39-40)             */
} ibm_scalar_params;

/* Scalar field cnew and its stored right-hand side dcrkold (main.f90:49),
 * reference layout (0:i1,0:j1,0:k1), and the scalar parameters.  The set
 * applies boundscal (bound.f90:109-171) as the driver does after loading
 * (main.f90:198); dcrk may be NULL (zero).  Once set, every RK substep
 * transports the scalar (scalad, scal.f90:11-58, in rk1..rk3, rk3.f90:13-329;
 * cnew = dcdt and boundscal after the projection, main.f90:374-376) and adds
 * the buoyancy momzbuoy (mom.f90:233-259) to the w right-hand side.  Without
 * a call the scalar is zero and stays zero, as it does in the reference with
 * zero wall values. */
int ibm_set_scalar(ibm_ctx *ctx, const ibm_scalar_params *sp, const double *c, const double *dcrk);
int ibm_get_scalar(ibm_ctx *ctx, double *c, double *dcrk);

/* --- plane statistics (post1d, output.f90:13-917) ------------------------------ */

/* phase_indicator (phase_indicator.f90:11-559) on one rank: fluid fractions
 * gamu..gamp of the u, v, w and pressure cells (1 = fluid) and the rigid-body
 * velocity of the particle occupying each cell, reference layout
 * (0:i1,0:j1,0:k1) with the reference's halos and wall ghost planes.
 * itype 1: translation + rotation on the velocity cells; itype 0: angular
 * velocity on the pressure cells.  Any output pointer may be NULL.  The
 * fractions are bit-identical to the reference's arithmetic. */
int ibm_phase_indicator(ibm_ctx *ctx, int itype, double *gamu, double *gamv, double *gamw,
                        double *gamp, double *upart, double *vpart, double *wpart);

/* Profiles of post1d, each ktot+2 values k = 0..k1, quantity-major:
 * profiles[IBM_STAT_x*(ktot+2) + k].  Entries the reference leaves unset
 * (gwm(0), gpm/cm/c2/wc/cdflx ghost planes, ss/ssp(k1)) are 0. */
#define IBM_STAT_UM    0   /* phase-averaged mean velocity and pressure       */
#define IBM_STAT_VM    1
#define IBM_STAT_WM    2
#define IBM_STAT_PM    3
#define IBM_STAT_U2    4   /* rms                                              */
#define IBM_STAT_V2    5
#define IBM_STAT_W2    6
#define IBM_STAT_P2    7
#define IBM_STAT_UV    8   /* plane sums of the fluid-weighted products        */
#define IBM_STAT_UW    9
#define IBM_STAT_VW    10  /* Reynolds stress v'w'                             */
#define IBM_STAT_UPM   11  /* solid-phase rigid-body velocity                  */
#define IBM_STAT_VPM   12
#define IBM_STAT_WPM   13
#define IBM_STAT_UP2   14
#define IBM_STAT_VP2   15
#define IBM_STAT_WP2   16
#define IBM_STAT_UPVP  17
#define IBM_STAT_UPWP  18
#define IBM_STAT_VPWP  19
#define IBM_STAT_GUM   20  /* plane sums of the fluid fractions                */
#define IBM_STAT_GVM   21
#define IBM_STAT_GWM   22
#define IBM_STAT_GPM   23
#define IBM_STAT_GP2   24
#define IBM_STAT_GUV   25
#define IBM_STAT_GUW   26
#define IBM_STAT_GVW   27
#define IBM_STAT_SS    28  /* viscous shear stress, fluid and particle phase   */
#define IBM_STAT_SSP   29
#define IBM_STAT_CM    30  /* scalar mean, rms, convective and diffusive flux  */
#define IBM_STAT_C2    31
#define IBM_STAT_WC    32
#define IBM_STAT_CDFLX 33
#define IBM_NSTAT      34
/* scalars[]: Re_tau, u_tau, Nu, Re_RBC, grad_k_wall (output.f90:465-477) */
#define IBM_NSTAT_SCALAR 5

/* post1d (output.f90:13-917) without its file output: phase_indicator(itype
 * 1) when np > 0, the plane sums of output.f90:88-364 as device reductions,
 * then the reference's ghost values, normalisations and derived scalars.
 * profiles: IBM_NSTAT*(ktot+2) doubles; scalars: IBM_NSTAT_SCALAR doubles
 * (either may be NULL). */
int ibm_post1d(ibm_ctx *ctx, double *profiles, double *scalars);

/* --- streams and timing ------------------------------------------------------ */

/* Runs all further work of the context on the given cudaStream_t (NULL:
 * back to a private stream).  Lets a host program time the library with
 * its own CUDA events on the launching stream. */
int ibm_set_stream(ibm_ctx *ctx, void *cuda_stream);
/* ibm_rk3_step with CUDA events around the four phases (see
 * ibm_phase_times); synchronises once per substep. */
int ibm_timed_step(ibm_ctx *ctx, double dt);

/* Milliseconds of the last ibm_rk3_step/ibm_run per phase (fluid predictor,
 * IBM loop, projection, Newton-Euler), measured with CUDA events on the
 * context stream, like the per-phase MPI_WTIME report (main.f90:396-410).
 * ms must hold 4 doubles. */
int ibm_phase_times(ibm_ctx *ctx, double ms[4]);
/* Number of kernels the library launched since the context was created. */
long long ibm_launch_count(const ibm_ctx *ctx);
/* Device synchronisation of the context stream. */
int ibm_sync(ibm_ctx *ctx);

/* --- learned forcing (IBM_MODE_MIXED_LEARNED; no counterpart in the reference) -
 *
 * A per-Lagrangian-point network 96 -> 128 -> 128 -> 3 (GELU) collapses the
 * multidirect passes of ibm_forcing_loop to one sweep plus one inference: the
 * first pass's interpolation and point forces F0, the network's prediction
 * of the correction the remaining passes would add, one spreading of
 * F0 + correction; the plain passes 2..nl_iter run as fallback whenever the
 * rms no-slip residual exceeds fallback_ratio x the plain method's.
 * Features per point, from the field the first pass interpolates: u/v/w at
 * the 27 stencil taps relative to the body velocity, slip, rigid-body
 * velocity, outward normal, F0*dt, centre delta weights.  Target:
 * (F_final - F0) * dt of the plain passes. */
#define IBM_NN_IN     96
#define IBM_NN_HIDDEN 128
#define IBM_NN_OUT    3
#define IBM_NN_NPARAM 29315   /* W1[128][96] b1[128] W2[128][128] b2[128] W3[3][128] b3[3] */
#define IBM_NN_NNORM  198     /* feature mean[96], 1/sigma[96]; target mean[3], sigma[3] */

/* Start harvesting (features, target) pairs from the plain passes of the
 * following forcing loops: every stride-th point, up to capacity samples kept
 * on the device (previous samples are discarded).  While harvesting, each
 * loop runs max(nl_iter, passes) plain passes (passes > nl_iter harvests a
 * more converged correction) and records the plain residual after nl_iter
 * passes as the reference for the fallback test.  capacity = 0 stops
 * harvesting and keeps the samples. */
int ibm_harvest(ibm_ctx *ctx, int capacity, int stride, int passes);
/* The harvested training set to host arrays: the first min(cap, *n) samples'
 * features [cap][IBM_NN_IN] and targets [cap][IBM_NN_OUT] (either may be
 * NULL); *n = the number of samples kept. */
int ibm_harvest_read(ibm_ctx *ctx, float *feat, float *targ, int cap, int *n);
/* nsteps Adam steps (lr, betas 0.9/0.999) on batches of `batch` samples drawn
 * with replacement from the harvest, on the GPU (forward, backward and weight
 * gradients on the tcgen05 tensor cores with BF16 operands, FP32 master
 * weights).  On the first call, or with reinit, the standardisation is
 * computed from the samples (FP64 column statistics on the device) and the
 * weights start afresh from `seed`.  *loss = mean squared error of the last
 * batch (standardised units).  Enables the learned correction and resets the
 * fallback gate's calibration.  IBM_E_NOT_CONVERGED: a tensor-core wait
 * timed out. */
int ibm_train_forcing_model(ibm_ctx *ctx, int nsteps, int batch, double lr, unsigned seed, int reinit,
                            double *loss);
/* Model transfer: params[IBM_NN_NPARAM], norm[IBM_NN_NNORM].  set enables it. */
int ibm_set_forcing_model(ibm_ctx *ctx, const float *params, const float *norm);
int ibm_get_forcing_model(ibm_ctx *ctx, float *params, float *norm);
/* enable (needs a model), fallback_ratio (default 1.5), plain_rms_ref > 0
 * fixes the plain residual reference; 0 (the default) uses the live one:
 * the learned loop's residual R is held to fallback_ratio x c_s x R0, R0 its
 * own first-pass slip (rms |U - u~| before any forcing) and c_s the factor
 * by which the plain passes reduced the first-pass slip on the latest plain
 * loop measured at the same RK stage s (a calibration loop below, or before
 * any, a harvested loop).  The stage is that of the last ibm_rk_predict. */
int ibm_learned_config(ibm_ctx *ctx, int enable, double fallback_ratio, double plain_rms_ref);
/* Calibration loops: with the network on, a forcing loop at RK stage s runs
 * the plain passes instead and measures c_s on the current state when s has
 * none measured since the model was trained or set, and then after 1, 2, 4,
 * 8 ... learned loops of s, at most period - 1 (default 10: one loop in ten
 * per stage once settled; 0: the first only). */
int ibm_learned_calibration(ibm_ctx *ctx, int period);
/* stats[6]: rms residual of the last learned loop, the reference its gate
 * used (before any learned loop: the last plain residual measured), fallback
 * ratio, fallbacks taken, learned loops run, harvested samples. */
int ibm_learned_stats(ibm_ctx *ctx, double stats[6]);
/* g[6]: first-pass slip R0 of the last learned loop, the reduction factor
 * c_s its gate used, plain loops measured, the last gate's reference
 * c_s x R0, R0 and residual of the last plain loop measured. */
int ibm_learned_gate_state(ibm_ctx *ctx, double g[6]);
/* Error-budget experiment for the learned form (mixed forms, plain passes):
 * after the plain passes of every following forcing loop, each point's
 * F*dt gets independent normal noise of rms sigma[c] per component
 * (velocity units; seeded), spread into the forced field as an increment
 * and included in the force sums.  All zero switches it off. */
int ibm_forcing_perturbation(ibm_ctx *ctx, const double sigma[3], unsigned seed);
/* The training kernels on a caller batch (features x[nb][96] already
 * standardised, targets t[nb][3]) with a scratch copy of params: loss,
 * gradient[IBM_NN_NPARAM] and outputs y[nb][3] (any may be NULL).  Loss =
 * mean over rows of the squared error summed over the 3 outputs. */
int ibm_mlp_gradient(ibm_ctx *ctx, const float *params, const float *x, const float *t, int nb, float *grad,
                     float *loss, float *y);
/* The inference kernel of the forcing loop on a caller batch: y[nb][3]. */
int ibm_mlp_infer(ibm_ctx *ctx, const float *params, const float *x, int nb, float *y);
/* The same on the tcgen05 (TMEM-accumulator) inference kernel. */
int ibm_mlp_infer_tc(ibm_ctx *ctx, const float *params, const float *x, int nb, float *y);
/* nsteps full-batch Adam steps from params_in with fresh moments:
 * params_out[IBM_NN_NPARAM], losses[nsteps] (loss before each update). */
int ibm_mlp_fit(ibm_ctx *ctx, const float *params_in, const float *x, const float *t, int nb, int nsteps,
                double lr, float *params_out, float *losses);

/* --- per-kernel timing ------------------------------------------------------- */

/* Kernel classes of the step for ibm_probe (bit i of the mask = class i). */
#define IBM_PROBE_PREDICT     0   /* k_predict                                   */
#define IBM_PROBE_STENCIL     1   /* IBM stencil cache                           */
#define IBM_PROBE_INTERP      2   /* interpolation + point forces (+ force sums) */
#define IBM_PROBE_SPREAD      3   /* spreading                                   */
#define IBM_PROBE_FILLPS_FFTX 4   /* fillps fused with the x FFT                 */
#define IBM_PROBE_FFTY        5   /* y FFT (forward and inverse)                 */
#define IBM_PROBE_THOMAS      6   /* Thomas sweep in z                           */
#define IBM_PROBE_IFFTX       7   /* inverse x FFT                               */
#define IBM_PROBE_CORREC      8   /* correc + pnew update                        */
#define IBM_PROBE_SPHERE      9   /* sphere integrals                            */
#define IBM_PROBE_FEATURES    10  /* learned forcing: features                   */
#define IBM_PROBE_MLP         11  /* learned forcing: network inference         */
#define IBM_PROBE_PHASE       12  /* statistics: phase indicator (both passes)   */
#define IBM_PROBE_STATS       13  /* statistics: plane sums of post1d            */
#define IBM_PROBE_GATED       14  /* learned loop: plain passes 2..Nl, gated     */
#define IBM_PROBE_N           15
/* Records CUDA events on the context stream around every launch of the
 * selected classes from now on (a profiler-free per-kernel timer; the events
 * add no GPU work).  ibm_probe_result synchronises, returns per class the
 * summed milliseconds and the number of launches timed, and stops probing. */
int ibm_probe(ibm_ctx *ctx, unsigned mask);
int ibm_probe_result(ibm_ctx *ctx, double ms[IBM_PROBE_N], int launches[IBM_PROBE_N]);

/* --- calibration (no counterpart in the reference) --------------------------- */

/* FP64 fused multiply-add rate of the current device in TFLOP/s, measured with
 * independent FMA chains on all SMs: the roofline denominator of the kernels
 * whose bound is the FP64 pipe (GB300 issues FP64 at 1/64 of the FP32 rate). */
int ibm_fp64_peak(double *tflops);

/* --- allocation-free variant ------------------------------------------------ */

/* chkdiv for callers that cannot allocate device memory (no counterpart in the
 * reference).  A host program whose fields already live on the GPU under its
 * own memory manager, that runs under a fixed device-memory budget, or that is
 * at a point where cudaMalloc is not allowed passes its own device arrays u, v,
 * w in the reference layout (0:itot+1, 0:jtot+1, 0:ktot+1), the inverse grid
 * spacings, and a device output of 5 doubles {total divergence, max |div|,
 * i, j, k of the maximum (1-based)}.  Work is queued on cuda_stream (NULL =
 * default stream) and not synchronised.  The call allocates nothing: its
 * per-plane partial sums live in a static device array of 4096 records
 * (96 KiB, held by every GPU that loads the library), so ktot > 4096 returns
 * IBM_E_INVALID.  All calls share that array: calls that overlap on the GPU
 * race.  The first call on each device looks the array up with
 * cudaGetSymbolAddress; make it before any stream capture. */
int ibm_chkdiv_noalloc(const double *u, const double *v, const double *w,
                       int itot, int jtot, int ktot, double dxi, double dyi, double dzi,
                       double *out5, void *cuda_stream);

#ifdef __cplusplus
}
#endif
#endif /* IBM_RK3_H */
