/*
 * layout_check.c -- the reference host layout through the C ABI, with every
 * array built by hand from the index arithmetic of the reference
 * declarations (no Python structure mirror involved):
 *   fields (0:i1,0:j1,0:k1), Fortran order: element (i,j,k) at
 *     i + (itot+2)*(j + (jtot+2)*k)                  (common.f90:4-8)
 *   particle members one array each, Lagrangian arrays [p*nl + l]
 *                                                    (common.f90:35-71)
 * Built against include/ibm_rk3.h with PFX = ibm_ (the CUDA library) or
 * orc_ (the CPU oracle), it checks:
 *   1. set_fields/get_fields return every interior value unchanged;
 *   2. chkdiv (chkdiv.f90:7-61) finds a divergence planted in one cell of
 *      u, of v and of w at that cell's 1-based (i,j,k), with value dxi, dyi
 *      or dzi times the planted jump;
 *   3. set_particles/init_particles/get_particles keep each particle's
 *      centre, and the Lagrangian points of particle p lie on the shell of
 *      radius radfp about centre p (coordsfp.f90:44-89).
 * Prints "layout ok" and exits 0 on success.
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "ibm_rk3.h"

#ifndef PFX
#define PFX ibm_
#endif
#define CAT2(a, b) a##b
#define CAT(a, b) CAT2(a, b)
#define F(name) CAT(PFX, name)

/* the entry points under PFX (the oracle exports the same signatures) */
ibm_ctx *F(create)(const ibm_params *);
int F(destroy)(ibm_ctx *);
const char *F(last_error)(const ibm_ctx *);
int F(sizes)(const ibm_ctx *, int *, int *, int *);
int F(set_fields)(ibm_ctx *, const double *, const double *, const double *, const double *, const double *,
                  const double *, const double *);
int F(get_fields)(ibm_ctx *, double *, double *, double *, double *, double *, double *, double *);
int F(set_particles)(ibm_ctx *, const ibm_particles *);
int F(get_particles)(ibm_ctx *, ibm_particles *);
int F(init_particles)(ibm_ctx *, double *);
int F(chkdiv)(ibm_ctx *, double *, double *, int[3]);

enum { IT = 16, JT = 12, KT = 10, NP = 2 };
#define I1 (IT + 2)
#define J1 (JT + 2)
#define K1 (KT + 2)
#define AT(i, j, k) ((size_t)(i) + (size_t)I1 * ((size_t)(j) + (size_t)J1 * (size_t)(k)))

static int fail(const char *what, ibm_ctx *c) {
  fprintf(stderr, "layout check failed: %s (%s)\n", what, c ? F(last_error)(c) : "");
  return 1;
}

static int planted_div(ibm_ctx *c, double *f[4], int comp, int i0, int j0, int k0, double di) {
  const size_t n = (size_t)I1 * J1 * K1;
  for (int q = 0; q < 4; ++q) memset(f[q], 0, n * sizeof(double));
  /* one face value 1 and its neighbour 0.5 along the component's axis: the
   * divergence is +d at (i0,j0,k0) and -d/2 at the next two cells */
  const int si = comp == 0, sj = comp == 1, sk = comp == 2;
  f[comp][AT(i0, j0, k0)] = 1.0;
  f[comp][AT(i0 + si, j0 + sj, k0 + sk)] = 0.5;
  if (F(set_fields)(c, f[0], f[1], f[2], f[3], NULL, NULL, NULL)) return fail("set_fields (planted)", c);
  double tot = 0, mx = 0;
  int ijk[3] = {0, 0, 0};
  int st = F(chkdiv)(c, &tot, &mx, ijk);
  if (st != IBM_OK && st != IBM_E_DIVERGENCE) return fail("chkdiv", c);
  if (ijk[0] != i0 || ijk[1] != j0 || ijk[2] != k0) {
    fprintf(stderr, "component %d: max at (%d,%d,%d), planted at (%d,%d,%d)\n", comp, ijk[0], ijk[1], ijk[2], i0,
            j0, k0);
    return fail("chkdiv location", c);
  }
  if (fabs(mx - di) > 1e-12 * di) return fail("chkdiv maximum", c);
  return 0;
}

int main(void) {
  const double PI = 3.141592653589793;
  const double lx = 1.0, ly = 0.75, lz = 0.625;
  const double dxi = IT / lx, dyi = JT / ly, dzi = KT / lz;
  const double radius = 3.0 / dxi;
  const int nl = (int)lround((PI / 3.) * (12. * pow((radius - 0.3 / dxi) * dxi, 2) + 1.));
  double *theta = malloc(nl * sizeof(double)), *phi = malloc(nl * sizeof(double));
  for (int l = 0; l < nl; ++l) { /* a spiral over the unit sphere */
    theta[l] = acos(1.0 - (2.0 * l + 1.0) / nl);
    phi[l] = fmod(l * 2.399963229728653, 2 * PI);
  }
  ibm_params P;
  memset(&P, 0, sizeof P);
  P.itot = IT; P.jtot = JT; P.ktot = KT;
  P.lx = lx; P.ly = ly; P.lz = lz;
  P.visc = 1e-3; P.radius = radius; P.ratiorho = 1.0;
  P.bc_top = IBM_BC_NOSLIP; P.bc_bot = IBM_BC_NOSLIP;
  P.np = NP; P.nl = nl; P.thetarc = theta; P.phirc = phi;
  P.radfp = radius - 0.3 / dxi;
  P.nb_copies = 9;
  P.mode = IBM_MODE_PLAIN_FP64;
  ibm_ctx *c = F(create)(&P);
  if (!c) return fail("create", NULL);
  int nq = 0, nlc = 0, ncells = 0;
  if (F(sizes)(c, &nq, &nlc, &ncells) || nlc != nl || ncells != I1 * J1 * K1) return fail("sizes", c);

  /* 1. interior round trip of values that encode their own indices */
  const size_t n = (size_t)I1 * J1 * K1;
  double *f[4], *g[4];
  for (int q = 0; q < 4; ++q) {
    f[q] = calloc(n, sizeof(double));
    g[q] = calloc(n, sizeof(double));
  }
  for (int k = 0; k < K1; ++k)
    for (int j = 0; j < J1; ++j)
      for (int i = 0; i < I1; ++i)
        for (int q = 0; q < 4; ++q) f[q][AT(i, j, k)] = 1e-3 * (q + 1) * (i + 100 * j + 10000 * k);
  if (F(set_fields)(c, f[0], f[1], f[2], f[3], NULL, NULL, NULL)) return fail("set_fields", c);
  if (F(get_fields)(c, g[0], g[1], g[2], g[3], NULL, NULL, NULL)) return fail("get_fields", c);
  for (int k = 1; k <= KT; ++k)
    for (int j = 1; j <= JT; ++j)
      for (int i = 1; i <= IT; ++i)
        for (int q = 0; q < 4; ++q)
          if (g[q][AT(i, j, k)] != f[q][AT(i, j, k)]) {
            fprintf(stderr, "field %d differs at (%d,%d,%d)\n", q, i, j, k);
            return fail("field round trip", c);
          }

  /* 2. one planted divergence per component, away from the walls and the
   *    periodic edges */
  if (planted_div(c, f, 0, 5, 7, 4, dxi)) return 1;
  if (planted_div(c, f, 1, 9, 3, 6, dyi)) return 1;
  if (planted_div(c, f, 2, 12, 10, 3, dzi)) return 1;

  /* 3. particles: every member its own array */
  const double cx[NP] = {0.31, 0.62}, cy[NP] = {0.27, 0.49}, cz[NP] = {0.30, 0.33};
  double *pd[31];
  for (int q = 0; q < 31; ++q) pd[q] = calloc(NP, sizeof(double));
  double *cd[10];
  for (int q = 0; q < 10; ++q) cd[q] = calloc((size_t)NP * nq, sizeof(double));
  int *qmax = calloc(NP, sizeof(int)), *firstc = calloc((size_t)NP * nq, sizeof(int));
  int *nb = calloc(NP * 9, sizeof(int)), *mslv = calloc(NP, sizeof(int));
  double *rkp = calloc(NP * 19, sizeof(double));
  ibm_particles S;
  memset(&S, 0, sizeof S);
  double **sc[31] = {&S.x, &S.y, &S.z, &S.theta, &S.phi, &S.u, &S.v, &S.w, &S.omx, &S.omy, &S.omz, &S.omtheta,
                     &S.intu, &S.intv, &S.intw, &S.intomx, &S.intomy, &S.intomz, &S.colfx, &S.colfy, &S.colfz,
                     &S.coltx, &S.colty, &S.coltz, &S.fxltot, &S.fyltot, &S.fzltot, &S.torqxltot, &S.torqyltot,
                     &S.torqzltot, &S.torqtheta};
  for (int q = 0; q < 31; ++q) *sc[q] = pd[q];
  double **cc[10] = {&S.cdx, &S.cdy, &S.cdz, &S.cdxt, &S.cdyt, &S.cdzt, &S.cdut, &S.cdvt, &S.cdwt, &S.cpsi};
  for (int q = 0; q < 10; ++q) *cc[q] = cd[q];
  for (int p = 0; p < NP; ++p) {
    S.x[p] = cx[p]; S.y[p] = cy[p]; S.z[p] = cz[p];
    mslv[p] = p + 1;
  }
  S.qmax = qmax; S.firstc = firstc; S.nb = nb; S.mslv = mslv; S.rkp = rkp;
  for (int q = 0; q < 4; ++q) memset(f[q], 0, n * sizeof(double));
  if (F(set_fields)(c, f[0], f[1], f[2], f[3], NULL, NULL, NULL)) return fail("set_fields (rest)", c);
  if (F(set_particles)(c, &S)) return fail("set_particles", c);
  double vol = 0;
  if (F(init_particles)(c, &vol)) return fail("init_particles", c);
  const double vexact = 4. / 3. * PI * radius * radius * radius;
  if (!(fabs(vol - vexact) < 0.05 * vexact)) return fail("sphere volume", c);
  ibm_particles T;
  memset(&T, 0, sizeof T);
  double *tx = calloc(NP, sizeof(double)), *ty = calloc(NP, sizeof(double)), *tz = calloc(NP, sizeof(double));
  double *xfp = calloc((size_t)NP * nl, sizeof(double)), *yfp = calloc((size_t)NP * nl, sizeof(double)),
         *zfp = calloc((size_t)NP * nl, sizeof(double));
  T.x = tx; T.y = ty; T.z = tz; T.xfp = xfp; T.yfp = yfp; T.zfp = zfp;
  if (F(get_particles)(c, &T)) return fail("get_particles", c);
  for (int p = 0; p < NP; ++p) {
    if (tx[p] != cx[p] || ty[p] != cy[p] || tz[p] != cz[p]) return fail("particle centre round trip", c);
    double mx = 0, my = 0, mz = 0;
    for (int l = 0; l < nl; ++l) {
      const size_t t = (size_t)p * nl + l;
      double dx = xfp[t] - cx[p], dy = yfp[t] - cy[p], dz = zfp[t] - cz[p];
      const double r = sqrt(dx * dx + dy * dy + dz * dz);
      if (fabs(r - P.radfp) > 1e-12) {
        fprintf(stderr, "particle %d point %d at distance %.15g from its centre, shell radius %.15g\n", p, l, r,
                P.radfp);
        return fail("Lagrangian point layout", c);
      }
      mx += dx; my += dy; mz += dz;
    }
    if (fabs(mx) + fabs(my) + fabs(mz) > 0.05 * nl * P.radfp) return fail("Lagrangian shell centre", c);
  }
  F(destroy)(c);
  printf("layout ok\n");
  return 0;
}
