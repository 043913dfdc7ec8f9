/*
 * ibm_oracle.h -- TEST INFRASTRUCTURE ONLY.
 *
 * CPU FP64 restatement of the reference's IBM RK3 substep (InterPartS,
 * single rank, dims=(1,1)).  It is the checker the GPU library is compared
 * against; only tests/, __graft_entry__.smoke() and bench.py's cpu_baseline
 * leg may load it.  The product (libibm_rk3.so) never links or calls it.
 *
 * Parity status: the reference is Fortran + MPI + 2DECOMP and cannot be
 * compiled here (no gfortran, no MPI), and its own tests hold no golden
 * vectors for this path.  The restatement is pinned instead by the
 * reference's built-in invariants (kerneltest, sphere volume check, chkdiv,
 * VFFTPACK forward/backward identity, nl/nlmax values of the shipped case) --
 * see tests/test_oracle_pins.py.  Against the reference itself: parity
 * unpinned.
 *
 * The entry points mirror include/ibm_rk3.h one for one with an orc_ prefix,
 * so the same driver code runs both.
 */
#ifndef IBM_ORACLE_H
#define IBM_ORACLE_H
#include "../include/ibm_rk3.h"
#ifdef __cplusplus
extern "C" {
#endif
typedef struct orc_ctx orc_ctx;
orc_ctx *orc_create(const ibm_params *params);
int orc_destroy(orc_ctx *c);
const char *orc_last_error(const orc_ctx *c);
int orc_sizes(const orc_ctx *c, int *nqmax, int *nl, int *ncells);
int orc_set_fields(orc_ctx *c, const double *u, const double *v, const double *w,
                   const double *p, const double *durk, const double *dvrk, const double *dwrk);
int orc_get_fields(orc_ctx *c, double *u, double *v, double *w, double *p,
                   double *durk, double *dvrk, double *dwrk);
int orc_get_intermediate(orc_ctx *c, double *dudt, double *dvdt, double *dwdt);
int orc_set_particles(orc_ctx *c, const ibm_particles *ps);
int orc_get_particles(orc_ctx *c, ibm_particles *ps);
int orc_init_particles(orc_ctx *c, double *vol_calc);
int orc_rk_predict(orc_ctx *c, int rkiter, double dt);
int orc_forcing_loop(orc_ctx *c, double dt, int nl_iter);
int orc_project(orc_ctx *c, int rkiter, double dt);
int orc_newton_euler(orc_ctx *c, int rkiter, double dt);
int orc_rk3_step(orc_ctx *c, double dt);
int orc_run(orc_ctx *c, double dt, int nsteps);
int orc_chkdiv(orc_ctx *c, double *divtot, double *divmax, int ijk[3]);
int orc_chkdt(orc_ctx *c, double *dtmax);
int orc_slip_residual(orc_ctx *c, double *maxres, double *rmsres);
int orc_diagnostics(orc_ctx *c, double *wallshearnew, double *wallshearold, double forcetot[3]);
int orc_set_scalar(orc_ctx *c, const ibm_scalar_params *sp, const double *cf, const double *dcrk);
int orc_get_scalar(orc_ctx *c, double *cf, double *dcrk);
int orc_phase_indicator(orc_ctx *c, int itype, double *gamu, double *gamv, double *gamw, double *gamp,
                        double *upart, double *vpart, double *wpart);
int orc_post1d(orc_ctx *c, double *profiles, double *scalars);
/* pins */
double orc_kernel(double r);
double orc_kerneltest(void);
/* VFFTPACK-semantics real transforms of one sequence (in place, length n):
 * dir=+1 forward (vrfftf), dir=-1 backward (vrfftb). */
int orc_vrfft(double *r, int n, int dir);
/* derived nl for a radius/grid (init.f90:127-129) */
int orc_nl(double radius, double dxi);
int orc_set_threads(int n);
#ifdef __cplusplus
}
#endif
#endif
