// ibm_oracle.cpp -- TEST INFRASTRUCTURE ONLY (the checker, never the product).
//
// A CPU FP64 restatement of the reference InterPartS IBM RK3 substep on one
// MPI rank (dims=(1,1)), written to follow the reference subroutines line by
// line: loop orders, expression orders and quirks are kept so that the GPU
// library can be compared against it.  Each function cites the reference file
// and lines it restates (paths relative to the reference project).
//
// Single-rank reductions of the MPI machinery, all exact:
//   * updthalos (bound.f90:173-221): SENDRECV to self = periodic plane copy.
//   * updthalos_ibm (bound.f90:223-309): 2-wide periodic copy (case 1) and
//     reverse accumulation of the 2-wide halos (case 2).
//   * 2DECOMP transposes in solver2d: identity.
//   * master/slave exchanges: every particle is its own master (mslv = id > 0),
//     neighbour(1..8) = myid, so the neighbour copies are the same particles
//     shifted by +-lx/+-ly exactly as the reference computes them.
//   * MPI_ALLREDUCE of scalars: the local value.
//
// Parity status against the reference build itself: unpinned (no Fortran or
// MPI toolchain is available); pinned by the reference's own invariants in
// tests/test_oracle_pins.py.
#include "ibm_oracle.h"

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

const double PI = std::acos(-1.0);

// 3-D array with Fortran (i fastest) layout and a common lower bound.
struct Arr3 {
  std::vector<double> d;
  int lo = 0, ni = 0, nj = 0, nk = 0;
  long sj = 0, sk = 0;
  void init(int lo_, int ni_, int nj_, int nk_) {
    lo = lo_; ni = ni_; nj = nj_; nk = nk_;
    sj = ni; sk = (long)ni * nj;
    d.assign((size_t)ni * nj * nk, 0.0);
  }
  inline double &operator()(int i, int j, int k) {
    return d[(size_t)(i - lo) + sj * (j - lo) + sk * (k - lo)];
  }
  inline double operator()(int i, int j, int k) const {
    return d[(size_t)(i - lo) + sj * (j - lo) + sk * (k - lo)];
  }
};

// particle (common.f90:35-71), old particle (common.f90:75-92), rkp (:97-105)
struct Part {
  double x, y, z, theta, phi, u, v, w, omx, omy, omz, omtheta;
  double intu, intv, intw, intomx, intomy, intomz;
  double colfx, colfy, colfz, coltx, colty, coltz;
  std::vector<double> dx, dy, dz, dxt, dyt, dzt, dut, dvt, dwt, psi;
  int qmax;
  std::vector<int> firstc;
  double fxltot, fyltot, fzltot, torqxltot, torqyltot, torqzltot, torqtheta;
  std::vector<double> xfp, yfp, zfp, ul, vl, wl, dudtl, dvdtl, dwdtl, fxl, fyl, fzl;
  double vol, mominert, ratiorho;
  int mslv;
  int nb[9];
};
struct OldPart {
  double x, y, z, theta, phi, u, v, w, omx, omy, omz, omtheta;
  double intu, intv, intw, intomx, intomy, intomz;
  double colfx, colfy, colfz, coltx, colty, coltz;
  std::vector<double> dx, dy, dz, dxt, dyt, dzt, dut, dvt, dwt, psi;
  int qmax;
  std::vector<int> firstc;
};
enum { RK_FX, RK_FY, RK_FZ, RK_TX, RK_TY, RK_TZ, RK_TT, RK_CFX, RK_CFY, RK_CFZ,
       RK_CTX, RK_CTY, RK_CTZ, RK_DUDT, RK_DVDT, RK_DWDT, RK_DOMX, RK_DOMY, RK_DOMZ, RK_N };

// Roma-Peskin 3-point regularised delta times h (kernel.f90:7-25)
inline double kernel(double r) {
  double k;
  if (std::fabs(r) > 1.5) {
    k = 0.;
  } else {
    if (std::fabs(r) > 0.5) {
      k = (1. / 6.) * (5. - 3. * std::fabs(r) - std::sqrt(-3. * ((1. - std::fabs(r)) * (1. - std::fabs(r))) + 1.));
    } else {
      k = (1. / 3.) * (1. + std::sqrt(-3. * (r * r) + 1.));
    }
  }
  return k;
}

inline int nint(double x) { return (int)std::lround(x); }  // Fortran NINT: half away from zero
inline int ffloor(double x) { return (int)std::floor(x); }

// ---------------------------------------------------------------------------
// Real FFT with VFFTPACK semantics (fft.f:693-760 forward, fft.f:1-80
// backward): half-complex storage R(1)=Re F0, R(2k)=Re Fk, R(2k+1)=Im Fk,
// R(N)=Re F(N/2) for even N, both directions scaled by sqrt(1/N), so that
// backward(forward(x)) = x.  Restated with an own mixed-radix complex FFT.
// ---------------------------------------------------------------------------
void cfft(std::complex<double> *a, int n, int sign, std::vector<std::complex<double>> &tmp) {
  if (n == 1) return;
  int r = 0;
  for (int f : {4, 2, 3, 5}) if (n % f == 0) { r = f; break; }
  if (r == 0) {  // plain DFT for other prime factors
    tmp.assign(a, a + n);
    for (int k = 0; k < n; ++k) {
      std::complex<double> s = 0;
      for (int j = 0; j < n; ++j) {
        double ang = sign * 2.0 * PI * (double)((long)j * k % n) / n;
        s += tmp[j] * std::complex<double>(std::cos(ang), std::sin(ang));
      }
      a[k] = s;
    }
    return;
  }
  int m = n / r;
  std::vector<std::complex<double>> sub((size_t)n);
  for (int q = 0; q < r; ++q)
    for (int j = 0; j < m; ++j) sub[(size_t)q * m + j] = a[(size_t)j * r + q];
  for (int q = 0; q < r; ++q) cfft(&sub[(size_t)q * m], m, sign, tmp);
  for (int k = 0; k < m; ++k) {
    for (int s = 0; s < r; ++s) {
      std::complex<double> acc = 0;
      int kk = k + s * m;
      for (int q = 0; q < r; ++q) {
        double ang = sign * 2.0 * PI * (double)((long)q * kk % n) / n;
        acc += sub[(size_t)q * m + k] * std::complex<double>(std::cos(ang), std::sin(ang));
      }
      a[kk] = acc;
    }
  }
}

void vrfft(double *r, int n, int dir) {
  std::vector<std::complex<double>> c((size_t)n), tmp;
  const double sc = std::sqrt(1.0 / n);
  if (dir > 0) {
    for (int j = 0; j < n; ++j) c[j] = r[j];
    cfft(c.data(), n, -1, tmp);
    r[0] = c[0].real() * sc;
    for (int k = 1; 2 * k < n; ++k) {
      r[2 * k - 1] = c[k].real() * sc;
      r[2 * k] = c[k].imag() * sc;
    }
    if (n % 2 == 0) r[n - 1] = c[n / 2].real() * sc;
  } else {
    c[0] = r[0];
    for (int k = 1; 2 * k < n; ++k) {
      c[k] = std::complex<double>(r[2 * k - 1], r[2 * k]);
      c[n - k] = std::conj(c[k]);
    }
    if (n % 2 == 0) c[n / 2] = r[n - 1];
    cfft(c.data(), n, +1, tmp);
    for (int j = 0; j < n; ++j) r[j] = c[j].real() * sc;
  }
}

}  // namespace

struct orc_ctx {
  std::string err;
  // grid (param.f90:91-94) -- dims=(1,1)
  int itot, jtot, ktot, imax, jmax, kmax, i1, j1, k1;
  double lx, ly, lz, visc, radius, ratiorho;
  int bc_top, bc_bot, particle_rotation, np, nl, nqmax, npmax, nb_copies;
  // periodic in z (bc_top = bc_bot = IBM_BC_PERIODIC): a variant the
  // reference cannot express (its z boundaries are always walls, bound.f90:
  // 17-65, initsolver.f90:26-30); see the functions marked "periodic z"
  bool zper = false;
  // polydisperse (ibm_params.radii set): per-particle radius, force-point
  // shell radius, point count, offset into the concatenated point table and
  // Lagrangian volume; another variant the reference cannot express (one
  // radius and one nl, param.f90:48, init.f90:129).  Pair constants: see
  // pair_consts.
  bool poly = false;
  std::vector<double> prad, pradfp, pdvl;
  std::vector<int> pnl, ptoff;
  // derived (init.f90:74-243)
  double dxi, dyi, dzi, dx, dy, dz, offset, volp, mominert, retrac;
  double rkcoeffab[3];
  double gaccx, gaccy, gaccz;
  double meffn_ss, mefft_ss, kn_ss, kt_ss, etan_ss, etat_ss, muc_ss, psi_crit_ss;
  double meffn_sw, mefft_sw, kn_sw, kt_sw, etan_sw, etat_sw, muc_sw, psi_crit_sw, colthr_pw;
  double coeff_f, coeff_t;
  double a11_ini_pp, a11a_ini_pp, a11b_ini_pp, a11_sat_pp, a11a_sat_pp, a11b_sat_pp;
  double a11_ini_pw, a11_sat_pw;
  // fields (common.f90:4-8)
  Arr3 unew, vnew, wnew, pnew, dudt, dvdt, dwdt, dudtold, dvdtold, dwdtold, p;
  Arr3 durk, dvrk, dwrk;
  // scalar (param.f90:39-47, init.f90:94); zero and not transported unless
  // set (cnew = 0 with zero wall values stays 0 exactly in the reference)
  Arr3 cnew, dcdt, dcrk;
  bool have_scalar = false;
  double kappa = 0., beta = 0., bc_c_top_val = 0., bc_c_bot_val = 0.;
  int bc_c_top_type = IBM_BC_C_DIRICHLET, bc_c_bot_type = IBM_BC_C_DIRICHLET;
  Arr3 dudtf, dvdtf, dwdtf;
  // solver (initsolver.f90)
  std::vector<double> a, b, c, xyrt;
  // particles
  std::vector<Part> ap;
  std::vector<OldPart> op;
  std::vector<double> rkp;  // [npmax*RK_N]
  std::vector<int> nla;
  std::vector<double> thetarc, phirc;
  double radfp, dVlagr, dVeul;
  int pmax;
  bool have_fields = false, have_particles = false;
  // diagnostics
  double wallshearnew = 0, wallshearold = 0, forcetot[3] = {0, 0, 0};
  double forceytot = 0;
};

namespace {

int fail(orc_ctx *c, int code, const char *msg) {
  c->err = msg;
  return code;
}

// Polydisperse pair constants: the contact spring/dashpot of init.f90:137-
// 241 with the effective mass ratiorho vp vq / (vp + vq) of the pair (vq = 0:
// a wall, ratiorho vp), and the lubrication prefactor 6 pi nu Re with the
// equivalent radius Re = 2 Rp Rq / (Rp + Rq) (Rp for a wall), so that the
// leading squeeze term 6 pi nu Re^2 / (4 gap) is the unequal-sphere one;
// both reduce to the equal-sphere constants.
struct PairC {
  double kn, kt, etan, etat, muc, coeff_f;
};
PairC pair_consts(const orc_ctx *c, double vp, double vq, double re);

// derived_parameters (init.f90:74-243), single rank
void derived_parameters(orc_ctx *c) {
  c->dxi = c->itot / c->lx; c->dyi = c->jtot / c->ly; c->dzi = c->ktot / c->lz;
  c->dx = 1. / c->dxi; c->dy = 1. / c->dyi; c->dz = 1. / c->dzi;
  c->offset = (std::sqrt(3. * (1.5 * 1.5))) / c->dxi + 0.01 / c->dxi;
  c->volp = (4. / 3.) * PI * std::pow(c->radius, 3.);
  c->mominert = (2. / 5.) * c->volp * std::pow(c->radius, 2.);
  c->retrac = 0.3 / c->dxi;
  // rkcoeff (param.f90:110-112): rkcoeffab = rkcoeff(:,1)+rkcoeff(:,2)
  c->rkcoeffab[0] = 32. / 60. + 0.;
  c->rkcoeffab[1] = 25. / 60. + (-17. / 60.);
  c->rkcoeffab[2] = 45. / 60. + (-25. / 60.);
  const double gacc = -9.81;  // param.f90:102-104
  c->gaccx = gacc * std::cos(PI / 2.);
  c->gaccy = gacc * std::cos(PI / 2.);
  c->gaccz = gacc * std::sin(PI / 2.);
  const double Nstretch = 8, dt_estim = 0.05, en = 0.97, et = 0.10, muc = 0.;
  c->meffn_ss = c->ratiorho * c->volp / 2.;
  c->mefft_ss = 2. / 7. * c->meffn_ss;
  c->kn_ss = (PI * PI + std::pow(std::fabs(std::log(en)), 2.)) * c->meffn_ss / std::pow(Nstretch * dt_estim, 2.);
  c->kt_ss = (PI * PI + std::pow(std::fabs(std::log(et)), 2.)) * c->mefft_ss / std::pow(Nstretch * dt_estim, 2.);
  c->etan_ss = -2. * (std::log(en)) * c->meffn_ss / (Nstretch * dt_estim);
  c->etat_ss = -2. * (std::log(et)) * c->mefft_ss / (Nstretch * dt_estim);
  c->muc_ss = muc;
  c->psi_crit_ss = 7. / 2. * (1. + en) / (1. + et) * c->muc_ss;
  c->colthr_pw = 0.001 * c->radius;
  c->meffn_sw = c->ratiorho * c->volp;
  c->mefft_sw = 2. / 7. * c->meffn_sw;
  c->kn_sw = (PI * PI + std::pow(std::fabs(std::log(en)), 2.)) * c->meffn_sw / std::pow(Nstretch * dt_estim, 2.);
  c->kt_sw = (PI * PI + std::pow(std::fabs(std::log(et)), 2.)) * c->mefft_sw / std::pow(Nstretch * dt_estim, 2.);
  c->etan_sw = -2. * (std::log(en)) * c->meffn_sw / (Nstretch * dt_estim);
  c->etat_sw = -2. * (std::log(et)) * c->mefft_sw / (Nstretch * dt_estim);
  c->muc_sw = muc;
  c->psi_crit_sw = 7. / 2. * (1. + en) / (1. + et) * c->muc_sw;
  c->coeff_f = 6. * PI * c->visc * c->radius;
  c->coeff_t = 8. * PI * c->visc * std::pow(c->radius, 2.);
  const double eps_ini_pp = 0.025, eps_sat_pp = 0.001, eps_ini_pw = 0.075, eps_sat_pw = 0.001;
  c->a11_ini_pp = -(1. / 4. * std::pow(eps_ini_pp, -1.)) + 9. / 40. * std::log(eps_ini_pp) +
                  3. / 112. * eps_ini_pp * std::log(eps_ini_pp);
  c->a11a_ini_pp = c->a11_ini_pp - .995;
  c->a11b_ini_pp = -c->a11_ini_pp + .350;
  c->a11_sat_pp = -(1. / 4. * std::pow(eps_sat_pp, -1.)) + 9. / 40. * std::log(eps_sat_pp) +
                  3. / 112. * eps_sat_pp * std::log(eps_sat_pp);
  c->a11a_sat_pp = c->a11_sat_pp - .995;
  c->a11b_sat_pp = -c->a11_sat_pp + .350;
  c->a11_ini_pw = -(1. / eps_ini_pw) + 1. / 5. * std::log(eps_ini_pw) + 1. / 21. * eps_ini_pw * std::log(eps_ini_pw) - .9713;
  c->a11_sat_pw = -(1. / eps_sat_pw) + 1. / 5. * std::log(eps_sat_pw) + 1. / 21. * eps_sat_pw * std::log(eps_sat_pw) - .9713;
}

PairC pair_consts(const orc_ctx *c, double vp, double vq, double re) {
  const double Nstretch = 8, dt_estim = 0.05, en = 0.97, et = 0.10;
  const double me = vq > 0. ? c->ratiorho * vp * vq / (vp + vq) : c->ratiorho * vp, mt = 2. / 7. * me;
  PairC k;
  k.kn = (PI * PI + std::pow(std::fabs(std::log(en)), 2.)) * me / std::pow(Nstretch * dt_estim, 2.);
  k.kt = (PI * PI + std::pow(std::fabs(std::log(et)), 2.)) * mt / std::pow(Nstretch * dt_estim, 2.);
  k.etan = -2. * (std::log(en)) * me / (Nstretch * dt_estim);
  k.etat = -2. * (std::log(et)) * mt / (Nstretch * dt_estim);
  k.muc = 0.;
  k.coeff_f = 6. * PI * c->visc * re;
  return k;
}
double prad(const orc_ctx *c, int p) { return c->poly ? c->prad[p] : c->radius; }
double pdvl(const orc_ctx *c, int p) { return c->poly ? c->pdvl[p] : c->dVlagr; }

// ---- boundary conditions (bound.f90) ---------------------------------------
// updthalos (bound.f90:173-221) on one rank: periodic copy of one plane.
void updthalos(orc_ctx *c, Arr3 &v, int dir) {
  if (dir == 1) {
    for (int k = 0; k <= c->k1; ++k)
      for (int j = 0; j <= c->j1; ++j) {
        v(c->i1, j, k) = v(1, j, k);
        v(0, j, k) = v(c->imax, j, k);
      }
  } else {
    for (int k = 0; k <= c->k1; ++k)
      for (int i = 0; i <= c->i1; ++i) {
        v(i, c->j1, k) = v(i, 1, k);
        v(i, 0, k) = v(i, c->jmax, k);
      }
  }
}

// bounduvw (bound.f90:11-80)
void bounduvw(orc_ctx *c, Arr3 &u, Arr3 &v, Arr3 &w) {
  if (c->zper) {  // periodic z: ghost planes are copies, w(kmax) is an unknown
    for (int j = 0; j <= c->j1; ++j)
      for (int i = 0; i <= c->i1; ++i)
        for (Arr3 *f : {&u, &v, &w}) {
          (*f)(i, j, c->k1) = (*f)(i, j, 1);
          (*f)(i, j, 0) = (*f)(i, j, c->kmax);
        }
    updthalos(c, u, 1); updthalos(c, v, 1); updthalos(c, w, 1);
    updthalos(c, u, 2); updthalos(c, v, 2); updthalos(c, w, 2);
    return;
  }
  for (int j = 0; j <= c->j1; ++j)
    for (int i = 0; i <= c->i1; ++i) {
      if (c->bc_top == IBM_BC_NOSLIP) {
        u(i, j, c->k1) = -u(i, j, c->kmax);
        v(i, j, c->k1) = -v(i, j, c->kmax);
      } else {
        u(i, j, c->k1) = u(i, j, c->kmax);
        v(i, j, c->k1) = v(i, j, c->kmax);
      }
      w(i, j, c->kmax) = 0.;
    }
  for (int j = 0; j <= c->j1; ++j)
    for (int i = 0; i <= c->i1; ++i) {
      if (c->bc_bot == IBM_BC_NOSLIP) {
        u(i, j, 0) = -u(i, j, 1);
        v(i, j, 0) = -v(i, j, 1);
      } else {
        u(i, j, 0) = u(i, j, 1);
        v(i, j, 0) = v(i, j, 1);
      }
      w(i, j, 0) = 0.;
    }
  updthalos(c, u, 1); updthalos(c, v, 1); updthalos(c, w, 1);
  updthalos(c, u, 2); updthalos(c, v, 2); updthalos(c, w, 2);
}

// boundp (bound.f90:82-107)
void boundp(orc_ctx *c, Arr3 &p) {
  for (int j = 0; j <= c->j1; ++j)
    for (int i = 0; i <= c->i1; ++i) {
      if (c->zper) {  // periodic z
        p(i, j, 0) = p(i, j, c->kmax);
        p(i, j, c->k1) = p(i, j, 1);
      } else {
        p(i, j, 0) = p(i, j, 1);
        p(i, j, c->k1) = p(i, j, c->kmax);
      }
    }
  updthalos(c, p, 1);
  updthalos(c, p, 2);
}

// updthalos_ibm (bound.f90:223-309) on one rank.
// icase 1: 2-wide periodic copy; icase 2: reverse accumulation of the halos.
void updthalos_ibm(orc_ctx *c, Arr3 &v, int dir, int icase) {
  const int imax = c->imax, jmax = c->jmax, i1 = c->i1, j1 = c->j1, k1 = c->k1;
  if (dir == 3) {  // periodic z: the x and y patterns along k, over the full x/y halo range
    const int kmax = c->kmax;
    for (int j = -1; j <= j1 + 1; ++j)
      for (int i = -1; i <= i1 + 1; ++i) {
        if (icase == 1) {
          v(i, j, k1) = v(i, j, 1); v(i, j, k1 + 1) = v(i, j, 2);
          v(i, j, -1) = v(i, j, kmax - 1); v(i, j, 0) = v(i, j, kmax);
        } else {
          v(i, j, 1) += v(i, j, k1); v(i, j, 2) += v(i, j, k1 + 1);
          v(i, j, kmax - 1) += v(i, j, -1); v(i, j, kmax) += v(i, j, 0);
        }
      }
    return;
  }
  if (icase == 1) {
    if (dir == 1) {
      for (int k = -1; k <= k1 + 1; ++k)
        for (int j = -1; j <= j1 + 1; ++j) {
          v(i1, j, k) = v(1, j, k); v(i1 + 1, j, k) = v(2, j, k);
          v(-1, j, k) = v(imax - 1, j, k); v(0, j, k) = v(imax, j, k);
        }
    } else {
      for (int k = -1; k <= k1 + 1; ++k)
        for (int i = -1; i <= i1 + 1; ++i) {
          v(i, j1, k) = v(i, 1, k); v(i, j1 + 1, k) = v(i, 2, k);
          v(i, -1, k) = v(i, jmax - 1, k); v(i, 0, k) = v(i, jmax, k);
        }
    }
  } else {
    if (dir == 1) {
      // xhm <- var(i1:i1+1) from left (= self); var(1:2) += xhm
      for (int k = -1; k <= k1 + 1; ++k)
        for (int j = -1; j <= j1 + 1; ++j) {
          v(1, j, k) += v(i1, j, k);
          v(2, j, k) += v(i1 + 1, j, k);
        }
      for (int k = -1; k <= k1 + 1; ++k)
        for (int j = -1; j <= j1 + 1; ++j) {
          v(imax - 1, j, k) += v(-1, j, k);
          v(imax, j, k) += v(0, j, k);
        }
    } else {
      for (int k = -1; k <= k1 + 1; ++k)
        for (int i = -1; i <= i1 + 1; ++i) {
          v(i, 1, k) += v(i, j1, k);
          v(i, 2, k) += v(i, j1 + 1, k);
        }
      for (int k = -1; k <= k1 + 1; ++k)
        for (int i = -1; i <= i1 + 1; ++i) {
          v(i, jmax - 1, k) += v(i, -1, k);
          v(i, jmax, k) += v(i, 0, k);
        }
    }
  }
}

// ---- momentum (mom.f90) ------------------------------------------------------
// momxad (mom.f90:8-54)
void momxad(orc_ctx *c, Arr3 &dudt, const Arr3 &U, const Arr3 &V, const Arr3 &W) {
  const double dxi = c->dxi, dyi = c->dyi, dzi = c->dzi, visc = c->visc;
#pragma omp parallel for schedule(static)
  for (int k = 1; k <= c->kmax; ++k)
    for (int j = 1; j <= c->jmax; ++j)
      for (int i = 1; i <= c->imax; ++i) {
        int ip = i + 1, jp = j + 1, kp = k + 1, im = i - 1, jm = j - 1, km = k - 1;
        double uuip = 0.25 * (U(ip, j, k) + U(i, j, k)) * (U(ip, j, k) + U(i, j, k));
        double uuim = 0.25 * (U(im, j, k) + U(i, j, k)) * (U(im, j, k) + U(i, j, k));
        double uvjp = 0.25 * (U(i, jp, k) + U(i, j, k)) * (V(ip, j, k) + V(i, j, k));
        double uvjm = 0.25 * (U(i, jm, k) + U(i, j, k)) * (V(ip, jm, k) + V(i, jm, k));
        double uwkp = 0.25 * (U(i, j, kp) + U(i, j, k)) * (W(ip, j, k) + W(i, j, k));
        double uwkm = 0.25 * (U(i, j, km) + U(i, j, k)) * (W(ip, j, km) + W(i, j, km));
        double dudxp = (U(ip, j, k) - U(i, j, k)) * dxi;
        double dudxm = (U(i, j, k) - U(im, j, k)) * dxi;
        double dudyp = (U(i, jp, k) - U(i, j, k)) * dyi;
        double dudym = (U(i, j, k) - U(i, jm, k)) * dyi;
        double dudzp = (U(i, j, kp) - U(i, j, k)) * dzi;
        double dudzm = (U(i, j, k) - U(i, j, km)) * dzi;
        dudt(i, j, k) = dxi * (-uuip + uuim) + visc * (dudxp - dudxm) * dxi +
                        dyi * (-uvjp + uvjm) + visc * (dudyp - dudym) * dyi +
                        dzi * (-uwkp + uwkm) + visc * (dudzp - dudzm) * dzi;
      }
}
// momyad (mom.f90:81-127)
void momyad(orc_ctx *c, Arr3 &dvdt, const Arr3 &U, const Arr3 &V, const Arr3 &W) {
  const double dxi = c->dxi, dyi = c->dyi, dzi = c->dzi, visc = c->visc;
#pragma omp parallel for schedule(static)
  for (int k = 1; k <= c->kmax; ++k)
    for (int j = 1; j <= c->jmax; ++j)
      for (int i = 1; i <= c->imax; ++i) {
        int ip = i + 1, jp = j + 1, kp = k + 1, im = i - 1, jm = j - 1, km = k - 1;
        double uvip = 0.25 * (U(i, j, k) + U(i, jp, k)) * (V(i, j, k) + V(ip, j, k));
        double uvim = 0.25 * (U(im, j, k) + U(im, jp, k)) * (V(i, j, k) + V(im, j, k));
        double vvjp = 0.25 * (V(i, j, k) + V(i, jp, k)) * (V(i, j, k) + V(i, jp, k));
        double vvjm = 0.25 * (V(i, j, k) + V(i, jm, k)) * (V(i, j, k) + V(i, jm, k));
        double wvkp = 0.25 * (W(i, j, k) + W(i, jp, k)) * (V(i, j, kp) + V(i, j, k));
        double wvkm = 0.25 * (W(i, j, km) + W(i, jp, km)) * (V(i, j, km) + V(i, j, k));
        double dvdxp = (V(ip, j, k) - V(i, j, k)) * dxi;
        double dvdxm = (V(i, j, k) - V(im, j, k)) * dxi;
        double dvdyp = (V(i, jp, k) - V(i, j, k)) * dyi;
        double dvdym = (V(i, j, k) - V(i, jm, k)) * dyi;
        double dvdzp = (V(i, j, kp) - V(i, j, k)) * dzi;
        double dvdzm = (V(i, j, k) - V(i, j, km)) * dzi;
        dvdt(i, j, k) = dxi * (-uvip + uvim) + visc * (dvdxp - dvdxm) * dxi +
                        dyi * (-vvjp + vvjm) + visc * (dvdyp - dvdym) * dyi +
                        dzi * (-wvkp + wvkm) + visc * (dvdzp - dvdzm) * dzi;
      }
}
// momzad (mom.f90:157-203)
void momzad(orc_ctx *c, Arr3 &dwdt, const Arr3 &U, const Arr3 &V, const Arr3 &W) {
  const double dxi = c->dxi, dyi = c->dyi, dzi = c->dzi, visc = c->visc;
#pragma omp parallel for schedule(static)
  for (int k = 1; k <= c->kmax; ++k)
    for (int j = 1; j <= c->jmax; ++j)
      for (int i = 1; i <= c->imax; ++i) {
        int ip = i + 1, jp = j + 1, kp = k + 1, im = i - 1, jm = j - 1, km = k - 1;
        double uwip = 0.25 * (W(i, j, k) + W(ip, j, k)) * (U(i, j, k) + U(i, j, kp));
        double uwim = 0.25 * (W(i, j, k) + W(im, j, k)) * (U(im, j, k) + U(im, j, kp));
        double vwjp = 0.25 * (W(i, j, k) + W(i, jp, k)) * (V(i, j, k) + V(i, j, kp));
        double vwjm = 0.25 * (W(i, j, k) + W(i, jm, k)) * (V(i, jm, k) + V(i, jm, kp));
        double wwkp = 0.25 * (W(i, j, k) + W(i, j, kp)) * (W(i, j, k) + W(i, j, kp));
        double wwkm = 0.25 * (W(i, j, k) + W(i, j, km)) * (W(i, j, k) + W(i, j, km));
        double dwdxp = (W(ip, j, k) - W(i, j, k)) * dxi;
        double dwdxm = (W(i, j, k) - W(im, j, k)) * dxi;
        double dwdyp = (W(i, jp, k) - W(i, j, k)) * dyi;
        double dwdym = (W(i, j, k) - W(i, jm, k)) * dyi;
        double dwdzp = (W(i, j, kp) - W(i, j, k)) * dzi;
        double dwdzm = (W(i, j, k) - W(i, j, km)) * dzi;
        dwdt(i, j, k) = dxi * (-uwip + uwim) + visc * (dwdxp - dwdxm) * dxi +
                        dyi * (-vwjp + vwjm) + visc * (dwdyp - dwdym) * dyi +
                        dzi * (-wwkp + wwkm) + visc * (dwdzp - dwdzm) * dzi;
      }
}
// momxp/momyp/momzp (mom.f90:56-79,129-155,205-231)
void momp(orc_ctx *c, Arr3 &du, Arr3 &dv, Arr3 &dw, const Arr3 &p) {
#pragma omp parallel for schedule(static)
  for (int k = 1; k <= c->kmax; ++k)
    for (int j = 1; j <= c->jmax; ++j)
      for (int i = 1; i <= c->imax; ++i) {
        du(i, j, k) = -c->dxi * (p(i + 1, j, k) - p(i, j, k));
        dv(i, j, k) = -c->dyi * (p(i, j + 1, k) - p(i, j, k));
        dw(i, j, k) = -c->dzi * (p(i, j, k + 1) - p(i, j, k));
      }
}

// wall shear part of rk1/rk2/rk3 (rk3.f90:80-103, 195-217, 305-325)
double wallshear_sum(orc_ctx *c) {
  double s = 0.;
  for (int j = 1; j <= c->jmax; ++j)
    for (int i = 1; i <= c->imax; ++i)
      s = s + c->visc * (c->vnew(i, j, c->kmax + 1) - c->vnew(i, j, c->kmax)) * c->dzi * (1. / c->dxi) * (1. / c->dyi)
            - c->visc * (c->vnew(i, j, 1) - c->vnew(i, j, 0)) * c->dzi * (1. / c->dxi) * (1. / c->dyi);
  return s;
}

// scalad (scal.f90:11-58): advection-diffusion of the scalar
void scalad(orc_ctx *c, Arr3 &dcdt, const Arr3 &U, const Arr3 &V, const Arr3 &W, const Arr3 &C) {
  const double dxi = c->dxi, dyi = c->dyi, dzi = c->dzi, kappa = c->kappa;
#pragma omp parallel for schedule(static)
  for (int k = 1; k <= c->kmax; ++k)
    for (int j = 1; j <= c->jmax; ++j)
      for (int i = 1; i <= c->imax; ++i) {
        const int ip = i + 1, jp = j + 1, kp = k + 1, im = i - 1, jm = j - 1, km = k - 1;
        const double ucip = 0.5 * U(i, j, k) * (C(ip, j, k) + C(i, j, k));
        const double ucim = 0.5 * U(im, j, k) * (C(i, j, k) + C(im, j, k));
        const double vcjp = 0.5 * V(i, j, k) * (C(i, jp, k) + C(i, j, k));
        const double vcjm = 0.5 * V(i, jm, k) * (C(i, j, k) + C(i, jm, k));
        const double wckp = 0.5 * W(i, j, k) * (C(i, j, kp) + C(i, j, k));
        const double wckm = 0.5 * W(i, j, km) * (C(i, j, k) + C(i, j, km));
        const double dcdxp = (C(ip, j, k) - C(i, j, k)) * dxi, dcdxm = (C(i, j, k) - C(im, j, k)) * dxi;
        const double dcdyp = (C(i, jp, k) - C(i, j, k)) * dyi, dcdym = (C(i, j, k) - C(i, jm, k)) * dyi;
        const double dcdzp = (C(i, j, kp) - C(i, j, k)) * dzi, dcdzm = (C(i, j, k) - C(i, j, km)) * dzi;
        dcdt(i, j, k) = dxi * (-ucip + ucim) + kappa * (dcdxp - dcdxm) * dxi + dyi * (-vcjp + vcjm) +
                        kappa * (dcdyp - dcdym) * dyi + dzi * (-wckp + wckm) + kappa * (dcdzp - dcdzm) * dzi;
      }
}

// momzbuoy (mom.f90:233-259) added to the advective w right-hand side the
// way rk1..rk3 combine them (rk3.f90:56-58): dw = B + dw
void add_buoyancy(orc_ctx *c, Arr3 &dw, const Arr3 &C) {
#pragma omp parallel for schedule(static)
  for (int k = 1; k <= c->kmax; ++k)
    for (int j = 1; j <= c->jmax; ++j)
      for (int i = 1; i <= c->imax; ++i)
        dw(i, j, k) = 0.5 * c->beta * 9.81 * (C(i, j, k) + C(i, j, k + 1)) + dw(i, j, k);
}

// boundscal (bound.f90:109-171)
void boundscal(orc_ctx *c, Arr3 &C) {
  const int k1 = c->k1, kmax = c->kmax;
  for (int j = 0; j <= c->j1; ++j)
    for (int i = 0; i <= c->i1; ++i) {
      if (c->bc_c_top_type == IBM_BC_C_DIRICHLET) C(i, j, k1) = 2 * c->bc_c_top_val - C(i, j, kmax);
      else C(i, j, k1) = C(i, j, kmax);
    }
  for (int j = 0; j <= c->j1; ++j)
    for (int i = 0; i <= c->i1; ++i) {
      if (c->bc_c_bot_type == IBM_BC_C_DIRICHLET) C(i, j, 0) = 2 * c->bc_c_bot_val - C(i, j, 1);
      else C(i, j, 0) = C(i, j, 1);
    }
  updthalos(c, C, 1);
  updthalos(c, C, 2);
}

// rk1/rk2/rk3 (rk3.f90:13-329), with the scalar (dcdt, scalad) and the
// buoyancy term (momzbuoy) once a scalar is set; without one they add
// exactly +0 to the momentum (c = 0).
void rk_stage(orc_ctx *c, int rkiter, double dt) {
  Arr3 &du = c->durk, &dv = c->dvrk, &dw = c->dwrk;
  const double dVeul = (1. / c->dxi) * (1. / c->dyi) * (1. / c->dzi);
  const double ntot = (double)c->itot * c->jtot * c->kmax;
  if (rkiter == 1) {
    const double factor = dt * (32. / 60.);
    momp(c, du, dv, dw, c->pnew);
#pragma omp parallel for schedule(static)
    for (int k = 1; k <= c->kmax; ++k)
      for (int j = 1; j <= c->jmax; ++j)
        for (int i = 1; i <= c->imax; ++i) {
          c->dudt(i, j, k) = c->unew(i, j, k) + factor * du(i, j, k);
          c->dvdt(i, j, k) = c->vnew(i, j, k) + factor * dv(i, j, k);
          c->dwdt(i, j, k) = c->wnew(i, j, k) + factor * dw(i, j, k);
        }
    momxad(c, du, c->unew, c->vnew, c->wnew);
    momyad(c, dv, c->unew, c->vnew, c->wnew);
    momzad(c, dw, c->unew, c->vnew, c->wnew);
    if (c->have_scalar) {
      add_buoyancy(c, dw, c->cnew);
      scalad(c, c->dcrk, c->unew, c->vnew, c->wnew, c->cnew);
    }
#pragma omp parallel for schedule(static)
    for (int k = 1; k <= c->kmax; ++k)
      for (int j = 1; j <= c->jmax; ++j)
        for (int i = 1; i <= c->imax; ++i) {
          c->dudt(i, j, k) = c->dudt(i, j, k) + factor * du(i, j, k);
          c->dvdt(i, j, k) = c->dvdt(i, j, k) + factor * dv(i, j, k);
          c->dwdt(i, j, k) = c->dwdt(i, j, k) + factor * dw(i, j, k);
          if (c->have_scalar) c->dcdt(i, j, k) = c->cnew(i, j, k) + factor * c->dcrk(i, j, k);
        }
    double all = wallshear_sum(c);
    c->wallshearnew = (factor / dt) * all / (dVeul * ntot);
    c->wallshearold = all / (dVeul * ntot);
  } else {
    const double factor1 = dt * ((rkiter == 2 ? 8. : 20.) / 60.);
    const double factor2 = dt * ((rkiter == 2 ? 25. : 45.) / 60.);
    const double factor3 = dt * ((rkiter == 2 ? 17. : 25.) / 60.);
    Arr3 dnu = c->unew, dnv = c->vnew, dnw = c->wnew;  // dummy arrays (shape only)
    momp(c, dnu, dnv, dnw, c->pnew);
#pragma omp parallel for schedule(static)
    for (int k = 1; k <= c->kmax; ++k)
      for (int j = 1; j <= c->jmax; ++j)
        for (int i = 1; i <= c->imax; ++i) {
          c->dudt(i, j, k) = c->unew(i, j, k) + factor1 * dnu(i, j, k);
          c->dvdt(i, j, k) = c->vnew(i, j, k) + factor1 * dnv(i, j, k);
          c->dwdt(i, j, k) = c->wnew(i, j, k) + factor1 * dnw(i, j, k);
        }
    momxad(c, dnu, c->unew, c->vnew, c->wnew);
    momyad(c, dnv, c->unew, c->vnew, c->wnew);
    momzad(c, dnw, c->unew, c->vnew, c->wnew);
    Arr3 dnc;
    if (c->have_scalar) {
      dnc = c->cnew;  // dummy array (shape only)
      add_buoyancy(c, dnw, c->cnew);
      scalad(c, dnc, c->unew, c->vnew, c->wnew, c->cnew);
    }
#pragma omp parallel for schedule(static)
    for (int k = 1; k <= c->kmax; ++k)
      for (int j = 1; j <= c->jmax; ++j)
        for (int i = 1; i <= c->imax; ++i) {
          c->dudt(i, j, k) = c->dudt(i, j, k) + (factor2 * dnu(i, j, k) - factor3 * du(i, j, k));
          c->dvdt(i, j, k) = c->dvdt(i, j, k) + (factor2 * dnv(i, j, k) - factor3 * dv(i, j, k));
          c->dwdt(i, j, k) = c->dwdt(i, j, k) + (factor2 * dnw(i, j, k) - factor3 * dw(i, j, k));
          if (c->have_scalar)
            c->dcdt(i, j, k) = c->cnew(i, j, k) + (factor2 * dnc(i, j, k) - factor3 * c->dcrk(i, j, k));
          if (rkiter == 2) {
            du(i, j, k) = dnu(i, j, k);
            dv(i, j, k) = dnv(i, j, k);
            dw(i, j, k) = dnw(i, j, k);
            if (c->have_scalar) c->dcrk(i, j, k) = dnc(i, j, k);
          }
        }
    double all = wallshear_sum(c);
    c->wallshearnew = (factor2 / dt) * all / (dVeul * ntot) - (factor3 / dt) * c->wallshearold;
    if (rkiter == 2) c->wallshearold = all / (dVeul * ntot);
  }
}

// ---- IBM (interp_spread.f90, forcing.f90) --------------------------------------
struct Stencil {
  int ilow, jlow, klow, ilows, jlows, klows;
  double phix[3], phiy[3], phiz[3], phixh[3], phiyh[3], phizh[3];
};
// stencil set-up shared by eulr2lagr and lagr2eulr (interp_spread.f90:76-130, 277-327)
inline void stencil(const orc_ctx *c, double xfp, double yfp, double zfp, Stencil &s) {
  const double coorxfp = xfp * c->dxi - std::floor((xfp - 0.5 * c->dx) / c->lx) * (c->itot) - (1 - 1);
  const double cooryfp = yfp * c->dyi - std::floor((yfp - 0.5 * c->dy) / c->ly) * (c->jtot) - (1 - 1);
  const int val_k_min = 1, val_k_max = c->kmax;
  s.ilows = nint(coorxfp) - 1;
  s.jlows = nint(cooryfp) - 1;
  s.ilow = ffloor(coorxfp);
  s.jlow = ffloor(cooryfp);
  double coorzfp;
  if (c->zper) {  // periodic z: the x/y image rule along z, no wall clamps
    coorzfp = zfp * c->dzi - std::floor((zfp - 0.5 * c->dz) / c->lz) * (c->ktot);
    s.klows = nint(coorzfp) - 1;
    s.klow = ffloor(coorzfp);
  } else {
    coorzfp = zfp * c->dzi;
    s.klows = std::max(nint(coorzfp) - 1, val_k_min);
    s.klow = std::max(std::min(ffloor(coorzfp), val_k_max - 2), val_k_min);
  }
  for (int m = 0; m < 3; ++m) {
    s.phix[m] = kernel(1. * s.ilows + m - coorxfp);
    s.phiy[m] = kernel(1. * s.jlows + m - cooryfp);
    s.phiz[m] = kernel(1. * s.klows + m - coorzfp);
    s.phixh[m] = kernel(1. * s.ilow + m - .5 - coorxfp);
    s.phiyh[m] = kernel(1. * s.jlow + m - .5 - cooryfp);
    s.phizh[m] = kernel(1. * s.klow + m - .5 - coorzfp);
  }
}

// eulr2lagr (interp_spread.f90:12-228)
void eulr2lagr(orc_ctx *c) {
  for (int p = 0; p < c->pmax; ++p)
    for (int l = 0; l < c->nl; ++l) {
      c->ap[p].dudtl[l] = 0.; c->ap[p].dvdtl[l] = 0.; c->ap[p].dwdtl[l] = 0.;
    }
  updthalos_ibm(c, c->dudtf, 1, 1); updthalos_ibm(c, c->dvdtf, 1, 1); updthalos_ibm(c, c->dwdtf, 1, 1);
  updthalos_ibm(c, c->dudtf, 2, 1); updthalos_ibm(c, c->dvdtf, 2, 1); updthalos_ibm(c, c->dwdtf, 2, 1);
  if (c->zper) { updthalos_ibm(c, c->dudtf, 3, 1); updthalos_ibm(c, c->dvdtf, 3, 1); updthalos_ibm(c, c->dwdtf, 3, 1); }
#pragma omp parallel for schedule(static)
  for (int p = 0; p < c->pmax; ++p) {
    Part &P = c->ap[p];
    if (P.mslv == 0) continue;
    for (int l = 0; l < c->nla[p]; ++l) {
      Stencil s;
      stencil(c, P.xfp[l], P.yfp[l], P.zfp[l], s);
      for (int k = 0; k < 3; ++k) for (int j = 0; j < 3; ++j) for (int i = 0; i < 3; ++i)
        P.dudtl[l] = P.dudtl[l] + c->dudtf(s.ilows + i, s.jlow + j, s.klow + k) * s.phix[i] * s.phiyh[j] * s.phizh[k];
      for (int k = 0; k < 3; ++k) for (int j = 0; j < 3; ++j) for (int i = 0; i < 3; ++i)
        P.dvdtl[l] = P.dvdtl[l] + c->dvdtf(s.ilow + i, s.jlows + j, s.klow + k) * s.phixh[i] * s.phiy[j] * s.phizh[k];
      for (int k = 0; k < 3; ++k) for (int j = 0; j < 3; ++j) for (int i = 0; i < 3; ++i)
        P.dwdtl[l] = P.dwdtl[l] + c->dwdtf(s.ilow + i, s.jlow + j, s.klows + k) * s.phixh[i] * s.phiyh[j] * s.phiz[k];
    }
  }
}

// complagrforces (forcing.f90:9-187) / updtlagrforces (forcing.f90:189-391)
void lagrforces(orc_ctx *c, double dt, bool first) {
  const double dti = 1. / dt;
#pragma omp parallel for schedule(static)
  for (int p = 0; p < c->pmax; ++p) {
    Part &P = c->ap[p];
    if (P.mslv == 0) continue;
    P.fxltot = 0.; P.fyltot = 0.; P.fzltot = 0.;
    P.torqxltot = 0.; P.torqyltot = 0.; P.torqzltot = 0.;
    for (int l = 0; l < c->nla[p]; ++l) {
      if (first) {
        P.fxl[l] = (P.ul[l] - P.dudtl[l]) * dti;
        P.fyl[l] = (P.vl[l] - P.dvdtl[l]) * dti;
        P.fzl[l] = (P.wl[l] - P.dwdtl[l]) * dti;
      } else {
        P.fxl[l] = P.fxl[l] + (P.ul[l] - P.dudtl[l]) * dti;
        P.fyl[l] = P.fyl[l] + (P.vl[l] - P.dvdtl[l]) * dti;
        P.fzl[l] = P.fzl[l] + (P.wl[l] - P.dwdtl[l]) * dti;
      }
      P.fxltot = P.fxltot + P.fxl[l];
      P.fyltot = P.fyltot + P.fyl[l];
      P.fzltot = P.fzltot + P.fzl[l];
      P.torqxltot = P.torqxltot + (P.yfp[l] - P.y) * P.fzl[l] - (P.zfp[l] - P.z) * P.fyl[l];
      P.torqyltot = P.torqyltot + (P.zfp[l] - P.z) * P.fxl[l] - (P.xfp[l] - P.x) * P.fzl[l];
      P.torqzltot = P.torqzltot + (P.xfp[l] - P.x) * P.fyl[l] - (P.yfp[l] - P.y) * P.fxl[l];
    }
    const double dVl = pdvl(c, p);
    P.fxltot = P.fxltot * dVl;
    P.fyltot = P.fyltot * dVl;
    P.fzltot = P.fzltot * dVl;
    P.torqxltot = P.torqxltot * dVl;
    P.torqyltot = P.torqyltot * dVl;
    P.torqzltot = P.torqzltot * dVl;
    P.torqtheta = (P.torqyltot * std::cos(P.phi)) - (P.torqxltot * std::sin(P.phi));
  }
  // master/slave exchange: on one rank anb(1..8)=0 and the sum over nb=0..8
  // returns the same totals (0 + ... exact).
}

// lagr2eulr (interp_spread.f90:230-474)
void lagr2eulr(orc_ctx *c, double dt) {
  double dVlagrdVeuli = c->dVlagr / c->dVeul;
  std::fill(c->dudtf.d.begin(), c->dudtf.d.end(), 0.);
  std::fill(c->dvdtf.d.begin(), c->dvdtf.d.end(), 0.);
  std::fill(c->dwdtf.d.begin(), c->dwdtf.d.end(), 0.);
  double coeffx0 = dVlagrdVeuli * dt, coeffy0 = dVlagrdVeuli * dt, coeffz0 = dVlagrdVeuli * dt;
  c->forceytot = 0.;
  for (int p = 0; p < c->pmax; ++p) {  // serial: the atomic-add order of the reference loop
    Part &P = c->ap[p];
    if (P.mslv == 0) continue;
    if (c->poly) {  // the particle's own Lagrangian volume
      dVlagrdVeuli = c->pdvl[p] / c->dVeul;
      coeffx0 = coeffy0 = coeffz0 = dVlagrdVeuli * dt;
    }
    for (int l = 0; l < c->nla[p]; ++l) {
      Stencil s;
      stencil(c, P.xfp[l], P.yfp[l], P.zfp[l], s);
      for (int k = 0; k < 3; ++k) for (int j = 0; j < 3; ++j) for (int i = 0; i < 3; ++i)
        c->dudtf(s.ilows + i, s.jlow + j, s.klow + k) += P.fxl[l] * coeffx0 * s.phix[i] * s.phiyh[j] * s.phizh[k];
      for (int k = 0; k < 3; ++k) for (int j = 0; j < 3; ++j) for (int i = 0; i < 3; ++i) {
        c->dvdtf(s.ilow + i, s.jlows + j, s.klow + k) += P.fyl[l] * coeffy0 * s.phixh[i] * s.phiy[j] * s.phizh[k];
        c->forceytot = c->forceytot + P.fyl[l] * coeffy0 * s.phixh[i] * s.phiy[j] * s.phizh[k];
      }
      for (int k = 0; k < 3; ++k) for (int j = 0; j < 3; ++j) for (int i = 0; i < 3; ++i)
        c->dwdtf(s.ilow + i, s.jlow + j, s.klows + k) += P.fzl[l] * coeffz0 * s.phixh[i] * s.phiyh[j] * s.phiz[k];
    }
  }
  updthalos_ibm(c, c->dudtf, 1, 2); updthalos_ibm(c, c->dvdtf, 1, 2); updthalos_ibm(c, c->dwdtf, 1, 2);
  updthalos_ibm(c, c->dudtf, 2, 2); updthalos_ibm(c, c->dvdtf, 2, 2); updthalos_ibm(c, c->dwdtf, 2, 2);
  if (c->zper) { updthalos_ibm(c, c->dudtf, 3, 2); updthalos_ibm(c, c->dvdtf, 3, 2); updthalos_ibm(c, c->dwdtf, 3, 2); }
  c->forceytot = c->forceytot / dt / (1. * c->itot * c->jtot * c->ktot) + c->wallshearnew;
  // iniu .ne. 'COU' always holds (lower-case values are used): add dudtold
#pragma omp parallel for schedule(static)
  for (int k = 1; k <= c->kmax; ++k)
    for (int j = 1; j <= c->jmax; ++j)
      for (int i = 1; i <= c->imax; ++i) {
        c->dudtf(i, j, k) = c->dudtf(i, j, k) + c->dudtold(i, j, k);
        c->dvdtf(i, j, k) = c->dvdtf(i, j, k) + c->dvdtold(i, j, k);
        c->dwdtf(i, j, k) = c->dwdtf(i, j, k) + c->dwdtold(i, j, k);
      }
}

// updtintermediatevel (forcing.f90:393-513) without its file appends:
// forcex/forcey/forcez are never written, so the mean forcing is zero; the
// particle force sums are kept as diagnostics.
void updtintermediatevel(orc_ctx *c) {
  double fx = 0, fy = 0, fz = 0;
  for (int p = 0; p < c->pmax; ++p)
    if (c->ap[p].mslv > 0) { fx += c->ap[p].fxltot; fy += c->ap[p].fyltot; fz += c->ap[p].fzltot; }
  c->forcetot[0] = fx; c->forcetot[1] = fy; c->forcetot[2] = fz;
}

// ---- projection -------------------------------------------------------------------
// fillps (fillps.f90:8-53)
void fillps(orc_ctx *c, int rkiter, double dt) {
  const double dti = 1. / (c->rkcoeffab[rkiter - 1] * dt);
  const double dtidxi = dti * c->dxi, dtidyi = dti * c->dyi, dtidzi = dti * c->dzi;
#pragma omp parallel for schedule(static)
  for (int k = 1; k <= c->kmax; ++k)
    for (int j = 1; j <= c->jmax; ++j)
      for (int i = 1; i <= c->imax; ++i)
        c->p(i, j, k) = ((c->dwdt(i, j, k) - c->dwdt(i, j, k - 1)) * dtidzi +
                         (c->dvdt(i, j, k) - c->dvdt(i, j - 1, k)) * dtidyi +
                         (c->dudt(i, j, k) - c->dudt(i - 1, j, k)) * dtidxi);
}

// initsolver (initsolver.f90:10-66)
void initsolver(orc_ctx *c) {
  const int kmax = c->kmax, itot = c->itot, jtot = c->jtot;
  c->a.assign(kmax + 1, 0.); c->b.assign(kmax + 1, 0.); c->c.assign(kmax + 1, 0.);
  for (int k = 1; k <= kmax; ++k) {
    c->a[k] = c->dzi * c->dzi;
    c->c[k] = c->dzi * c->dzi;
    c->b[k] = -(c->a[k] + c->c[k]);
  }
  if (!c->zper) {  // Neumann walls; periodic z keeps the cyclic corners a(1), c(kmax)
    c->b[1] = c->b[1] + c->a[1];
    c->b[kmax] = c->b[kmax] + c->c[kmax];
    c->a[1] = 0.;
    c->c[kmax] = 0.;
  }
  std::vector<double> xrt(itot + 1), yrt(jtot + 1);
  for (int i = 3; i <= itot; i += 2) {
    xrt[i - 1] = -4. * c->dxi * c->dxi * std::pow(std::sin(double(i - 1) * PI / (2. * itot)), 2);
    xrt[i] = xrt[i - 1];
  }
  xrt[1] = 0.;
  xrt[itot] = -4. * c->dxi * c->dxi;
  for (int j = 3; j <= jtot; j += 2) {
    yrt[j - 1] = -4. * c->dyi * c->dyi * std::pow(std::sin(double(j - 1) * PI / (2. * jtot)), 2);
    yrt[j] = yrt[j - 1];
  }
  yrt[1] = 0.;
  yrt[jtot] = -4. * c->dyi * c->dyi;
  c->xyrt.assign((size_t)c->imax * c->jmax, 0.);
  for (int j = 1; j <= c->jmax; ++j)
    for (int i = 1; i <= c->imax; ++i) c->xyrt[(size_t)(i - 1) + (size_t)c->imax * (j - 1)] = xrt[i] + yrt[j];
}

// Periodic z: the cyclic tridiagonal system of one (kx, ky) mode, diagonal
// -2 a2 + xy, off-diagonals and corners a2 (n unknowns, in place in r).
// Sherman-Morrison around the tridiagonal part with gamma = -b: x = y -
// f z, T y = r, T z = (gamma, 0.., 0, a2), f = (y_0 + a2 y_{n-1}/gamma) /
// (1 + z_0 + a2 z_{n-1}/gamma), where T has b - gamma and b - a2^2/gamma in
// its first and last diagonal entries.  The zero mode (xy = 0) is singular:
// its last unknown is pinned to 0 and rows 0..n-2 are solved (the
// counterpart of the reference's zero-mode guard, solver.f90:119-123).
// w1, w2: work arrays of n.
void tri_solve(double *r, int n, double a2, double b0, double b, double bn, double *cp) {
  double den = b0;
  cp[0] = a2 / den;
  r[0] = r[0] / den;
  for (int k = 1; k < n; ++k) {
    const double bk = k == n - 1 ? bn : b;
    den = bk - a2 * cp[k - 1];
    cp[k] = a2 / den;
    r[k] = (r[k] - a2 * r[k - 1]) / den;
  }
  for (int k = n - 2; k >= 0; --k) r[k] = r[k] - cp[k] * r[k + 1];
}
void cyclic_solve(double *r, int n, double a2, double xy, double *w1, double *w2) {
  const double b = -2. * a2 + xy;
  if (xy == 0.) {
    tri_solve(r, n - 1, a2, b, b, b, w1);
    r[n - 1] = 0.;
    return;
  }
  const double gamma = -b;
  const double b0 = b - gamma, bn = b - a2 * a2 / gamma;
  tri_solve(r, n, a2, b0, b, bn, w1);
  for (int k = 0; k < n; ++k) w2[k] = 0.;
  w2[0] = gamma;
  w2[n - 1] = a2;
  tri_solve(w2, n, a2, b0, b, bn, w1);
  const double f = (r[0] + a2 * r[n - 1] / gamma) / (1. + w2[0] + a2 * w2[n - 1] / gamma);
  for (int k = 0; k < n; ++k) r[k] = r[k] - f * w2[k];
}

// solver2d (solver.f90:43-172): x-FFT, y-FFT, Thomas in k, inverse y, inverse x.
void solver2d(orc_ctx *c) {
  const int imax = c->imax, jmax = c->jmax, kmax = c->kmax;
  Arr3 &pz = c->p;  // pz => p(1:imax,1:jmax,1:kmax)
#pragma omp parallel for schedule(static)
  for (int k = 1; k <= kmax; ++k) {
    std::vector<double> row(imax);
    for (int j = 1; j <= jmax; ++j) {
      for (int i = 0; i < imax; ++i) row[i] = pz(i + 1, j, k);
      vrfft(row.data(), imax, +1);
      for (int i = 0; i < imax; ++i) pz(i + 1, j, k) = row[i];
    }
    std::vector<double> col(jmax);
    for (int i = 1; i <= imax; ++i) {
      for (int j = 0; j < jmax; ++j) col[j] = pz(i, j + 1, k);
      vrfft(col.data(), jmax, +1);
      for (int j = 0; j < jmax; ++j) pz(i, j + 1, k) = col[j];
    }
  }
  if (c->zper) {
#pragma omp parallel for schedule(static)
    for (int j = 1; j <= jmax; ++j) {
      std::vector<double> col(kmax), w1(kmax), w2(kmax);
      for (int i = 1; i <= imax; ++i) {
        for (int k = 0; k < kmax; ++k) col[k] = pz(i, j, k + 1);
        cyclic_solve(col.data(), kmax, c->dzi * c->dzi, c->xyrt[(size_t)(i - 1) + (size_t)imax * (j - 1)],
                     w1.data(), w2.data());
        for (int k = 0; k < kmax; ++k) pz(i, j, k + 1) = col[k];
      }
    }
  } else {
  // Thomas algorithm with the zero-mode guard (solver.f90:94-134)
#pragma omp parallel for schedule(static)
  for (int j = 1; j <= jmax; ++j) {
    std::vector<double> d(kmax + 1);
    for (int i = 1; i <= imax; ++i) {
      const double xy = c->xyrt[(size_t)(i - 1) + (size_t)imax * (j - 1)];
      double z = 1. / (c->b[1] + xy);
      d[1] = c->c[1] * z;
      pz(i, j, 1) = pz(i, j, 1) * z;
      for (int k = 2; k <= kmax - 1; ++k) {
        double bb = c->b[k] + xy;
        z = 1. / (bb - c->a[k] * d[k - 1]);
        d[k] = c->c[k] * z;
        pz(i, j, k) = (pz(i, j, k) - c->a[k] * pz(i, j, k - 1)) * z;
      }
      double bb = c->b[kmax] + xy;
      z = bb - c->a[kmax] * d[kmax - 1];
      if (z != 0.)
        pz(i, j, kmax) = (pz(i, j, kmax) - c->a[kmax] * pz(i, j, kmax - 1)) / z;
      else
        pz(i, j, kmax) = 0.;
      for (int k = kmax - 1; k >= 1; --k) pz(i, j, k) = pz(i, j, k) - d[k] * pz(i, j, k + 1);
    }
  }
  }
#pragma omp parallel for schedule(static)
  for (int k = 1; k <= kmax; ++k) {
    std::vector<double> col(jmax);
    for (int i = 1; i <= imax; ++i) {
      for (int j = 0; j < jmax; ++j) col[j] = pz(i, j + 1, k);
      vrfft(col.data(), jmax, -1);
      for (int j = 0; j < jmax; ++j) pz(i, j + 1, k) = col[j];
    }
    std::vector<double> row(imax);
    for (int j = 1; j <= jmax; ++j) {
      for (int i = 0; i < imax; ++i) row[i] = pz(i + 1, j, k);
      vrfft(row.data(), imax, -1);
      for (int i = 0; i < imax; ++i) pz(i + 1, j, k) = row[i];
    }
  }
}

// correc (correc.f90:11-42)
void correc(orc_ctx *c, int rkiter, double dt) {
  const double factor = c->rkcoeffab[rkiter - 1] * dt;
  const double factori = factor * c->dxi, factorj = factor * c->dyi, factork = factor * c->dzi;
#pragma omp parallel for schedule(static)
  for (int k = 1; k <= c->kmax; ++k)
    for (int j = 1; j <= c->jmax; ++j)
      for (int i = 1; i <= c->imax; ++i) {
        c->unew(i, j, k) = c->dudt(i, j, k) - factori * (c->p(i + 1, j, k) - c->p(i, j, k));
        c->vnew(i, j, k) = c->dvdt(i, j, k) - factorj * (c->p(i, j + 1, k) - c->p(i, j, k));
        c->wnew(i, j, k) = c->dwdt(i, j, k) - factork * (c->p(i, j, k + 1) - c->p(i, j, k));
      }
}

// ---- particles ------------------------------------------------------------------------
// Lagrangian points and their rigid-body velocity (coordsfp.f90:44-79 and
// intgr_nwtn_eulr.f90:1438-1485; rotation of the point set ignored: theta*0.)
void lagrangian_points(orc_ctx *c) {
  for (int p = 0; p < c->pmax; ++p) {
    Part &P = c->ap[p];
    c->nla[p] = 0;
    if (P.mslv == 0) continue;
    int ll = 0;
    const int nlp = c->poly ? c->pnl[p] : c->nl, to = c->poly ? c->ptoff[p] : 0;
    const double radfp = c->poly ? c->pradfp[p] : c->radfp;
    for (int l = 0; l < nlp; ++l) {
      const double th = c->thetarc[to + l], ph = c->phirc[to + l];
      double xfploc = P.x + radfp * std::sin(P.theta * 0. + th) * std::cos(P.phi * 0. + ph);
      double yfploc = P.y + radfp * std::sin(P.theta * 0. + th) * std::sin(P.phi * 0. + ph);
      double zfploc = P.z + radfp * std::cos(P.theta * 0. + th);
      double isperiodx = 0., isperiody = 0.;
      if (xfploc < 0. + 0.5 * c->dx) isperiodx = 1.;
      if (xfploc >= c->lx + 0.5 * c->dx) isperiodx = -1.;
      if (yfploc < 0. + 0.5 * c->dy) isperiody = 1.;
      if (yfploc >= c->ly + 0.5 * c->dy) isperiody = -1.;
      bool isout = false;
      double coorxfp = (xfploc + isperiodx * c->lx - 0.) * c->dxi;
      if (nint(coorxfp) < 1 || nint(coorxfp) > c->imax) isout = true;
      double cooryfp = (yfploc + isperiody * c->ly - 0.) * c->dyi;
      if (nint(cooryfp) < 1 || nint(cooryfp) > c->jmax) isout = true;
      if (!isout) {
        P.xfp[ll] = xfploc; P.yfp[ll] = yfploc; P.zfp[ll] = zfploc;
        P.ul[ll] = P.u + P.omy * (P.zfp[ll] - P.z) - P.omz * (P.yfp[ll] - P.y);
        P.vl[ll] = P.v + P.omz * (P.xfp[ll] - P.x) - P.omx * (P.zfp[ll] - P.z);
        P.wl[ll] = P.w + P.omx * (P.yfp[ll] - P.y) - P.omy * (P.xfp[ll] - P.x);
        ++ll;
      }
    }
    c->nla[p] = ll;
  }
}

// nb flags of a master on one rank (intgr_nwtn_eulr.f90:1051-1090, bounds 0..lx, 0..ly)
void nb_flags(const orc_ctx *c, Part &P) {
  const double ro = (c->poly ? c->prad[&P - c->ap.data()] : c->radius) + c->offset;
  const double leftb = 0. * c->lx / 1., rightb = 1. * c->lx / 1., frontb = 0. * c->ly / 1., backb = 1. * c->ly / 1.;
  for (int n = 0; n < 9; ++n) P.nb[n] = 0;
  double dist;
  if (P.x > (rightb - ro)) P.nb[1] = 1;
  dist = std::sqrt((rightb - P.x) * (rightb - P.x) + (frontb - P.y) * (frontb - P.y));
  if (std::fabs(dist) < ro) P.nb[2] = 1;
  if (P.y < (frontb + ro)) P.nb[3] = 1;
  dist = std::sqrt((leftb - P.x) * (leftb - P.x) + (frontb - P.y) * (frontb - P.y));
  if (std::fabs(dist) < ro) P.nb[4] = 1;
  if (P.x < (leftb + ro)) P.nb[5] = 1;
  dist = std::sqrt((leftb - P.x) * (leftb - P.x) + (backb - P.y) * (backb - P.y));
  if (std::fabs(dist) < ro) P.nb[6] = 1;
  if (P.y > (backb - ro)) P.nb[7] = 1;
  dist = std::sqrt((rightb - P.x) * (rightb - P.x) + (backb - P.y) * (backb - P.y));
  if (std::fabs(dist) < ro) P.nb[8] = 1;
}

// position of the self-neighbour copy nb of a particle on one rank
// (intgr_over_sphere.f90:84-112 for a master that is also its own slave)
inline void copy_shift_sphere(const orc_ctx *c, int nbrecv, double &x, double &y) {
  switch (nbrecv) {
    case 1: x = x + c->lx; break;
    case 2: x = x + c->lx; y = y - c->ly; break;
    case 3: y = y - c->ly; break;
    case 4: x = x - c->lx; y = y - c->ly; break;
    case 5: x = x - c->lx; break;
    case 6: x = x - c->lx; y = y + c->ly; break;
    case 7: y = y + c->ly; break;
    case 8: x = x + c->lx; y = y + c->ly; break;
    default: break;
  }
}

// intgr_over_sphere (intgr_over_sphere.f90:12-625) on one rank.  Types 2 and
// 3 read the current (unew,vnew,wnew).
void intgr_over_sphere(orc_ctx *c, int type) {
  const double dx = 1. / c->dxi, dy = 1. / c->dyi, dz = 1. / c->dzi;
  const double dVeul = c->dVeul;
#pragma omp parallel for schedule(dynamic)
  for (int p = 0; p < c->pmax; ++p) {
    const double radius = prad(c, p);  // polydisperse: the particle's own
    const double radin = radius - 2. * dx;
    const double radin2 = radin * radin;
    Part &P = c->ap[p];
    double ax[9], ay[9], az[9], iu[9], iv[9], iw[9];
    for (int n = 0; n < 9; ++n) { ax[n] = 0; ay[n] = 0; az[n] = 0; iu[n] = 0; iv[n] = 0; iw[n] = 0; }
    ax[0] = P.x; ay[0] = P.y; az[0] = P.z;
    for (int nb = 1; nb <= 8; ++nb) {
      int nbrecv = nb + 4; if (nbrecv > 8) nbrecv -= 8;
      if (P.mslv > 0 && P.nb[nb] == 1) {
        ax[nbrecv] = ax[0]; ay[nbrecv] = ay[0]; az[nbrecv] = az[0];
        copy_shift_sphere(c, nbrecv, ax[nbrecv], ay[nbrecv]);
      }
    }
    if (P.mslv == 0) continue;
    for (int nb = 0; nb <= 8; ++nb) {
      bool go = (nb == 0 && P.mslv > 0) || (nb > 0 && P.mslv > 0 && P.nb[nb] == 1);
      if (!go) continue;
      int nbrecv = nb;
      if (nb > 0 && P.mslv > 0) { nbrecv = nb + 4; if (nbrecv > 8) nbrecv -= 8; }
      // periodic z: the images at z -+ lz as well (clipped to the grid like
      // the x/y copies), summed into the same copy
      for (int zs = 0; zs < (c->zper ? 3 : 1); ++zs) {
      const double cx = ax[nbrecv], cy = ay[nbrecv], cz = az[nbrecv] + (zs == 1 ? -c->lz : (zs == 2 ? c->lz : 0.));
      const double coorxc = cx - 0., cooryc = cy - 0., coorzc = cz;
      int ilow = nint((coorxc - radius) * c->dxi - 2.);
      int ihigh = nint((coorxc + radius) * c->dxi + 2.);
      int jlow = nint((cooryc - radius) * c->dyi - 2.);
      int jhigh = nint((cooryc + radius) * c->dyi + 2.);
      int klow = nint((coorzc - radius) * c->dzi - 2.);
      int khigh = nint((coorzc + radius) * c->dzi + 2.);
      if (ilow < 1) ilow = 1;
      if (jlow < 1) jlow = 1;
      if (klow < 1) klow = 1;
      if (ihigh > c->imax) ihigh = c->imax;
      if (jhigh > c->jmax) jhigh = c->jmax;
      if (khigh > c->kmax) khigh = c->kmax;
      for (int comp = 0; comp < 3; ++comp) {
        const Arr3 &F = comp == 0 ? c->unew : (comp == 1 ? c->vnew : c->wnew);
        for (int k = klow; k <= khigh; ++k) {
          double coorzmin, coorzplus;
          if (comp < 2) { coorzmin = (k - 1) * dz; coorzplus = k * dz; }
          else { coorzmin = (k - 0.5) * dz; coorzplus = (k + 0.5) * dz; }
          const double dzp2 = (coorzplus - cz) * (coorzplus - cz);
          for (int j = jlow; j <= jhigh; ++j) {
            double coorymin, cooryplus;
            if (comp == 1) { coorymin = 0. + (j - 0.5) * dy; cooryplus = 0. + (j + 0.5) * dy; }
            else { coorymin = 0. + (j - 1) * dy; cooryplus = 0. + j * dy; }
            const double dyp2 = (cooryplus - cy) * (cooryplus - cy);
            for (int i = ilow; i <= ihigh; ++i) {
              double coorxmin, coorxplus;
              if (comp == 0) { coorxmin = 0. + (i - 0.5) * dx; coorxplus = 0. + (i + 0.5) * dx; }
              else { coorxmin = 0. + (i - 1) * dx; coorxplus = 0. + i * dx; }
              const double dxp2 = (coorxplus - cx) * (coorxplus - cx);
              const double dist2 = dxp2 + dyp2 + dzp2;
              double frac = 1.;
              bool full = dist2 < radin2;
              if (!full) {
                const double dxm2 = (coorxmin - cx) * (coorxmin - cx);
                const double dym2 = (coorymin - cy) * (coorymin - cy);
                const double dzm2 = (coorzmin - cz) * (coorzmin - cz);
                double sg[8];
                sg[0] = radius - std::sqrt(dxm2 + dym2 + dzm2);
                sg[1] = radius - std::sqrt(dxm2 + dyp2 + dzm2);
                sg[2] = radius - std::sqrt(dxp2 + dyp2 + dzm2);
                sg[3] = radius - std::sqrt(dxp2 + dym2 + dzm2);
                sg[4] = radius - std::sqrt(dxm2 + dym2 + dzp2);
                sg[5] = radius - std::sqrt(dxm2 + dyp2 + dzp2);
                sg[6] = radius - std::sqrt(dxp2 + dyp2 + dzp2);
                sg[7] = radius - std::sqrt(dxp2 + dym2 + dzp2);
                double sum1 = 0., sum2 = 0.;
                for (int cp = 0; cp < 8; ++cp) {
                  if (sg[cp] > 0.) sum1 = sum1 + sg[cp];
                  sum2 = sum2 + std::fabs(sg[cp]);
                }
                frac = sum1 / sum2;
              }
              const double f = F(i, j, k);
              if (type == 1) {
                double add = full ? dVeul : (frac)*dVeul;
                if (comp == 0) iu[nbrecv] += add; else if (comp == 1) iv[nbrecv] += add; else iw[nbrecv] += add;
              } else if (type == 2) {
                double add = full ? f * dVeul : f * (frac)*dVeul;
                if (comp == 0) iu[nbrecv] += add; else if (comp == 1) iv[nbrecv] += add; else iw[nbrecv] += add;
              } else {
                const double rx = 0. + (i - 0.5) * dx - cx;
                const double ry = 0. + (j - 0.5) * dy - cy;
                const double rz = (k - 0.5) * dz - cz;
                if (comp == 0) {
                  if (full) { iv[nbrecv] = iv[nbrecv] + rz * f * dVeul; iw[nbrecv] = iw[nbrecv] - ry * f * dVeul; }
                  else { iv[nbrecv] = iv[nbrecv] + rz * f * (frac)*dVeul; iw[nbrecv] = iw[nbrecv] - ry * f * (frac)*dVeul; }
                } else if (comp == 1) {
                  if (full) { iu[nbrecv] = iu[nbrecv] - rz * f * dVeul; iw[nbrecv] = iw[nbrecv] + rx * f * dVeul; }
                  else { iu[nbrecv] = iu[nbrecv] - rz * f * (frac)*dVeul; iw[nbrecv] = iw[nbrecv] + rx * f * (frac)*dVeul; }
                } else {
                  if (full) { iu[nbrecv] = iu[nbrecv] + ry * f * dVeul; iv[nbrecv] = iv[nbrecv] - rx * f * dVeul; }
                  else { iu[nbrecv] = iu[nbrecv] + ry * f * (frac)*dVeul; iv[nbrecv] = iv[nbrecv] - rx * f * (frac)*dVeul; }
                }
              }
            }
          }
        }
      }
      }
    }
    double su = 0., sv = 0., sw = 0.;
    for (int nb = 0; nb <= 8; ++nb) { su = su + iu[nb]; sv = sv + iv[nb]; sw = sw + iw[nb]; }
    if (type <= 2) { P.intu = su; P.intv = sv; P.intw = sw; }
    else { P.intomx = su; P.intomy = sv; P.intomz = sw; }
  }
}

// lubrication (collisions.f90:222-438): only the normal (squeeze) force is
// applied (collisions.f90:430-432), so only f1 is evaluated.
void lubrication(orc_ctx *c, Part &P, int idq, double nx, double ny, double nz, double eps,
                 double u_nb, double v_nb, double w_nb, double coeff_f) {
  const double u1a = P.u * nx + P.v * ny + P.w * nz;
  const double u1b = u_nb * nx + v_nb * ny + w_nb * nz;
  double f1;
  if (idq > c->np) {
    double a11;
    if (eps < 0.001) a11 = c->a11_sat_pw;
    else a11 = -(1. / eps) + 1. / 5. * std::log(eps) + 1. / 21. * eps * std::log(eps) - .9713;
    f1 = (a11 * u1a);
    f1 = coeff_f * (f1 - (c->a11_ini_pw * u1a));
  } else {
    double a11a, a11b;
    if (eps < 0.001) { a11a = c->a11a_sat_pp; a11b = c->a11b_sat_pp; }
    else {
      double a11 = -(1. / 4. * std::pow(eps, -1.)) + 9. / 40. * std::log(eps) + 3. / 112. * eps * std::log(eps);
      a11a = a11 - .995;
      a11b = -a11 + .350;
    }
    f1 = (a11a * u1a + a11b * u1b);
    f1 = coeff_f * (f1 - (c->a11a_ini_pp * u1a + c->a11b_ini_pp * u1b));
  }
  P.colfx = P.colfx + f1 * nx;
  P.colfy = P.colfy + f1 * ny;
  P.colfz = P.colfz + f1 * nz;
}

// collisions (collisions.f90:10-220)
void collisions(orc_ctx *c, int p, int qq, int idq, double dist, double deltax, double deltay,
                double deltaz, double u_nb, double v_nb, double w_nb, double omx_nb, double omy_nb,
                double omz_nb, double dtsub, int rkiter) {
  Part &P = c->ap[p];
  OldPart &O = c->op[p];
  const double radius = prad(c, p);
  // polydisperse: the partner's radius in its own rotation term (a wall: 0)
  const double rq = c->poly ? (idq <= c->np ? c->prad[idq - 1] : 0.) : radius;
  const double nx = deltax / dist, ny = deltay / dist, nz = deltaz / dist;
  double deltan, kn, etan, kt, etat, muc;
  if (c->poly) {
    const bool wall = idq > c->np;
    const PairC k = pair_consts(c, P.vol, wall ? 0. : c->ap[idq - 1].vol, radius);
    deltan = (wall ? radius : radius + rq) - dist;
    kn = k.kn; kt = k.kt; etan = k.etan; etat = k.etat; muc = k.muc;
  } else if (idq <= c->np) {
    deltan = 2 * radius - dist; kn = c->kn_ss; kt = c->kt_ss; etan = c->etan_ss; etat = c->etat_ss; muc = c->muc_ss;
  } else {
    deltan = radius - dist; kn = c->kn_sw; kt = c->kt_sw; etan = c->etan_sw; etat = c->etat_sw; muc = c->muc_sw;
  }
  const double dun = (P.u + (P.omy * radius * nz) - (P.omz * radius * ny)) -
                     (u_nb + (omy_nb * rq * (-nz)) - (omz_nb * rq * (-ny)));
  const double dvn = (P.v - (P.omx * radius * nz) + (P.omz * radius * nx)) -
                     (v_nb - (omx_nb * rq * (-nz)) + (omz_nb * rq * (-nx)));
  const double dwn = (P.w + (P.omx * radius * ny) - (P.omy * radius * nx)) -
                     (w_nb + (omx_nb * rq * (-ny)) - (omy_nb * rq * (-nx)));
  const double vabs = dun * nx + dvn * ny + dwn * nz;
  const double fxn = -(kn * (deltan * nx)) - etan * (vabs * nx);
  const double fyn = -(kn * (deltan * ny)) - etan * (vabs * ny);
  const double fzn = -(kn * (deltan * nz)) - etan * (vabs * nz);
  const double dut = dun - vabs * nx, dvt = dvn - vabs * ny, dwt = dwn - vabs * nz;
  const double vtabs = std::sqrt(dut * dut + dvt * dvt + dwt * dwt);
  const int q = qq - 1;
  const double distold = std::sqrt(O.dx[q] * O.dx[q] + O.dy[q] * O.dy[q] + O.dz[q] * O.dz[q]);
  double nxold, nyold, nzold;
  if (distold == 0) { nxold = nx; nyold = ny; nzold = nz; }
  else { nxold = O.dx[q] / distold; nyold = O.dy[q] / distold; nzold = O.dz[q] / distold; }
  double dxt, dyt, dzt;
  const double rkab = c->rkcoeffab[rkiter - 1];
  if (P.firstc[q] == idq) {
    double hx = ny * nzold - nyold * nz;
    double hy = nz * nxold - nzold * nx;
    double hz = nx * nyold - nxold * ny;
    const double aa = std::sqrt(hx * hx + hy * hy + hz * hz);
    const double cc = std::cos(std::asin(aa));
    const double bb = 1. - cc;
    if (aa == 0.) { hx = 0.; hy = 0.; hz = 0.; }
    else { hx = hx / aa; hy = hy / aa; hz = hz / aa; }
    const double h11 = bb * (hx * hx) + cc, h12 = bb * hx * hy - aa * hz, h13 = bb * hx * hz + aa * hy;
    const double h21 = bb * hx * hy + aa * hz, h22 = bb * (hy * hy) + cc, h23 = bb * hy * hz - aa * hx;
    const double h31 = bb * hx * hz - aa * hy, h32 = bb * hy * hz + aa * hx, h33 = bb * (hz * hz) + cc;
    dxt = O.dxt[q] * h11 + O.dyt[q] * h21 + O.dzt[q] * h31 +
          0.5 * dtsub * rkab * (dut + O.dut[q] * h11 + O.dvt[q] * h21 + O.dwt[q] * h31);
    dyt = O.dxt[q] * h12 + O.dyt[q] * h22 + O.dzt[q] * h32 +
          0.5 * dtsub * rkab * (dvt + O.dut[q] * h12 + O.dvt[q] * h22 + O.dwt[q] * h32);
    dzt = O.dxt[q] * h13 + O.dyt[q] * h23 + O.dzt[q] * h33 +
          0.5 * dtsub * rkab * (dwt + O.dut[q] * h13 + O.dvt[q] * h23 + O.dwt[q] * h33);
  } else {
    P.psi[q] = vtabs / std::fabs(vabs);
    dxt = 0.; dyt = 0.; dzt = 0.;
  }
  double fxt = -(kt * dxt) - (etat * dut);
  double fyt = -(kt * dyt) - (etat * dvt);
  double fzt = -(kt * dzt) - (etat * dwt);
  const double fnabs = std::sqrt(fxn * fxn + fyn * fyn + fzn * fzn);
  double ftabs = std::sqrt(fxt * fxt + fyt * fyt + fzt * fzt);
  const double tx = -fxt / ftabs, ty = -fyt / ftabs, tz = -fzt / ftabs;
  if (ftabs <= muc * fnabs) {
    // sticking
  } else {
    dxt = muc * fnabs * tx / kt;
    dyt = muc * fnabs * ty / kt;
    dzt = muc * fnabs * tz / kt;
    fxt = -(kt * dxt) - (etat * dut);
    fyt = -(kt * dyt) - (etat * dvt);
    fzt = -(kt * dzt) - (etat * dwt);
    ftabs = std::sqrt(fxt * fxt + fyt * fyt + fzt * fzt);
    if (!(ftabs <= muc * fnabs)) {
      fxt = -muc * fnabs * tx; fyt = -muc * fnabs * ty; fzt = -muc * fnabs * tz;
    }
  }
  (void)fxt; (void)fyt; (void)fzt;  // tangential force and torque are not applied
  P.colfx = P.colfx + fxn;
  P.colfy = P.colfy + fyn;
  P.colfz = P.colfz + fzn;
  P.dx[q] = deltax; P.dy[q] = deltay; P.dz[q] = deltaz;
  P.dxt[q] = dxt; P.dyt[q] = dyt; P.dzt[q] = dzt;
  P.dut[q] = dut; P.dvt[q] = dvt; P.dwt[q] = dwt;
}

// removal of contact i (1-based) by moving the last entry into it
// (intgr_nwtn_eulr.f90:416-457)
void remove_contact(Part &P, OldPart &O, int i, int &qlast) {
  const int a = i - 1, l = qlast - 1;
  if (qlast > 1) {
    P.firstc[a] = P.firstc[l]; P.dxt[a] = P.dxt[l]; P.dyt[a] = P.dyt[l]; P.dzt[a] = P.dzt[l];
    P.dut[a] = P.dut[l]; P.dvt[a] = P.dvt[l]; P.dwt[a] = P.dwt[l];
    O.firstc[a] = O.firstc[l]; O.dxt[a] = O.dxt[l]; O.dyt[a] = O.dyt[l]; O.dzt[a] = O.dzt[l];
    O.dut[a] = O.dut[l]; O.dvt[a] = O.dvt[l]; O.dwt[a] = O.dwt[l];
  }
  P.firstc[l] = 0; P.dx[l] = 0.; P.dy[l] = 0.; P.dz[l] = 0.; P.dxt[l] = 0.; P.dyt[l] = 0.; P.dzt[l] = 0.;
  P.dut[l] = 0.; P.dvt[l] = 0.; P.dwt[l] = 0.;
  O.firstc[l] = 0; O.dx[l] = 0.; O.dy[l] = 0.; O.dz[l] = 0.; O.dxt[l] = 0.; O.dyt[l] = 0.; O.dzt[l] = 0.;
  O.dut[l] = 0.; O.dvt[l] = 0.; O.dwt[l] = 0.;
  qlast = qlast - 1;
}
// initialisation of a new contact slot (intgr_nwtn_eulr.f90:461-479)
void new_contact(Part &P, OldPart &O, int slot) {
  const int s = slot - 1;
  P.dx[s] = 0.; P.dy[s] = 0.; P.dz[s] = 0.; P.dxt[s] = 0.; P.dyt[s] = 0.; P.dzt[s] = 0.;
  P.dut[s] = 0.; P.dvt[s] = 0.; P.dwt[s] = 0.;
  O.dx[s] = 0.; O.dy[s] = 0.; O.dz[s] = 0.; O.dxt[s] = 0.; O.dyt[s] = 0.; O.dzt[s] = 0.;
  O.dut[s] = 0.; O.dvt[s] = 0.; O.dwt[s] = 0.;
}

// position of particle copy nb as seen in the collision loop on one rank
// (intgr_nwtn_eulr.f90:223-322 with coords=(0,0), dims=(1,1))
inline void copy_shift_coll(const orc_ctx *c, int nb, double &x, double &y) {
  const double boundleftnb = (0 + 1) * c->lx / (1. * 1), boundrightnb = (0) * c->lx / (1. * 1);
  const double boundbacknb = (0) * c->ly / (1. * 1), boundfrontnb = (0 + 1) * c->ly / (1. * 1);
  switch (nb) {
    case 1: if (x < boundleftnb) x = x + c->lx; break;
    case 2: if (x < boundleftnb) x = x + c->lx; if (y > boundbacknb) y = y - c->ly; break;
    case 3: if (y > boundbacknb) y = y - c->ly; break;
    case 4: if (x > boundrightnb) x = x - c->lx; if (y > boundbacknb) y = y - c->ly; break;
    case 5: if (x > boundrightnb) x = x - c->lx; break;
    case 6: if (x > boundrightnb) x = x - c->lx; if (y < boundfrontnb) y = y + c->ly; break;
    case 7: if (y < boundfrontnb) y = y + c->ly; break;
    case 8: if (x < boundleftnb) x = x + c->lx; if (y < boundfrontnb) y = y + c->ly; break;
    default: break;
  }
}

inline int minloc_abs3(const double a[3]) {
  int m = 0;
  for (int t = 1; t < 3; ++t) if (std::fabs(a[t]) < std::fabs(a[m])) m = t;
  return m;
}

// sumrk3 (intgr_nwtn_eulr.f90:1586-1669)
void sumrk3(orc_ctx *c, int rkiter, double dt) {
  const double dpdy_new = 0.;  // never assigned in the reference (module default 0)
  for (int p = 0; p < c->pmax; ++p) {
    Part &P = c->ap[p];
    OldPart &O = c->op[p];
    double *r = &c->rkp[(size_t)p * RK_N];
    if (rkiter == 1 && P.mslv > 0)
      for (int t = 0; t < RK_N; ++t) r[t] = 0.;
    if (P.mslv > 0) {
      const double ab = c->rkcoeffab[rkiter - 1];
      r[RK_FX] = r[RK_FX] + (-1.) * P.fxltot + (P.intu - O.intu) / dt;
      r[RK_FY] = r[RK_FY] + (-1.) * P.fyltot + (P.intv - O.intv) / dt;
      r[RK_FZ] = r[RK_FZ] + (-1.) * P.fzltot + (P.intw - O.intw) / dt;
      r[RK_TX] = r[RK_TX] + (-1.) * P.torqxltot + (P.intomx - O.intomx) / dt;
      r[RK_TY] = r[RK_TY] + (-1.) * P.torqyltot + (P.intomy - O.intomy) / dt;
      r[RK_TZ] = r[RK_TZ] + (-1.) * P.torqzltot + (P.intomz - O.intomz) / dt;
      r[RK_TT] = r[RK_TT] + (-1.) * (-dpdy_new * c->dVlagr);
      r[RK_CFX] = r[RK_CFX] + 0.5 * ab * (P.colfx + O.colfx);
      r[RK_CFY] = r[RK_CFY] + 0.5 * ab * (P.colfy + O.colfy);
      r[RK_CFZ] = r[RK_CFZ] + 0.5 * ab * (P.colfz + O.colfz);
      r[RK_CTX] = r[RK_CTX] + 0.5 * ab * (P.coltx + O.coltx);
      r[RK_CTY] = r[RK_CTY] + 0.5 * ab * (P.colty + O.colty);
      r[RK_CTZ] = r[RK_CTZ] + 0.5 * ab * (P.coltz + O.coltz);
      r[RK_DUDT] = r[RK_DUDT] + (P.u - O.u) / dt;
      r[RK_DVDT] = r[RK_DVDT] + (P.v - O.v) / dt;
      r[RK_DWDT] = r[RK_DWDT] + (P.w - O.w) / dt;
    }
  }
}

// intgr_nwtn_eulr (intgr_nwtn_eulr.f90:12-1514) on one rank
int intgr_nwtn_eulr(orc_ctx *c, int rkiter, double dt) {
  const int np = c->np, pmax = c->pmax;
  const double radius = c->radius;
  // new -> old (:77-118)
  for (int p = 0; p < pmax; ++p) {
    Part &P = c->ap[p];
    OldPart &O = c->op[p];
    if (P.mslv > 0) {
      O.x = P.x; O.y = P.y; O.z = P.z; O.theta = P.theta; O.phi = P.phi;
      O.u = P.u; O.v = P.v; O.w = P.w; O.omx = P.omx; O.omy = P.omy; O.omz = P.omz; O.omtheta = P.omtheta;
      O.intu = P.intu; O.intv = P.intv; O.intw = P.intw;
      O.intomx = P.intomx; O.intomy = P.intomy; O.intomz = P.intomz;
      O.colfx = P.colfx; O.colfy = P.colfy; O.colfz = P.colfz;
      O.coltx = P.coltx; O.colty = P.colty; O.coltz = P.coltz;
      O.dx = P.dx; O.dy = P.dy; O.dz = P.dz; O.dxt = P.dxt; O.dyt = P.dyt; O.dzt = P.dzt;
      O.dut = P.dut; O.dvt = P.dvt; O.dwt = P.dwt;
    }
  }
  intgr_over_sphere(c, 2);
  intgr_over_sphere(c, 3);
  const int itermax = 1;
  std::vector<double> sx(pmax), sy(pmax), sz(pmax), su(pmax), sv(pmax), sw(pmax), sox(pmax), soy(pmax), soz(pmax);
  std::vector<int> smslv(pmax);
  int status = IBM_OK;
  for (int iter = 0; iter <= itermax; ++iter) {
    for (int p = 0; p < pmax; ++p) {
      const Part &P = c->ap[p];
      smslv[p] = P.mslv;
      if (P.mslv > 0) {
        sx[p] = P.x; sy[p] = P.y; sz[p] = P.z; su[p] = P.u; sv[p] = P.v; sw[p] = P.w;
        sox[p] = P.omx; soy[p] = P.omy; soz[p] = P.omz;
      } else {
        sx[p] = sy[p] = sz[p] = su[p] = sv[p] = sw[p] = sox[p] = soy[p] = soz[p] = 0.;
      }
    }
    const int botw = np + 1, topw = np + 2;
#pragma omp parallel for schedule(dynamic)
    for (int p = 0; p < pmax; ++p) {
      Part &P = c->ap[p];
      OldPart &O = c->op[p];
      int qlast = P.qmax;
      if (P.mslv <= 0) continue;
      const int idp = P.mslv;
      qlast = P.qmax;
      P.colfx = 0.; P.colfy = 0.; P.colfz = 0.; P.coltx = 0.; P.colty = 0.; P.coltz = 0.;
      for (int nb = 0; nb < c->nb_copies; ++nb) {
        for (int q = 0; q < pmax; ++q) {
          if (idp == smslv[q]) continue;
          if (!(smslv[q] > 0)) continue;
          const int idq = smslv[q];
          double qx = sx[q], qy = sy[q];
          copy_shift_coll(c, nb, qx, qy);
          const double deltaz = sz[q] - P.z;
          double adx[3] = {qx - P.x, qx - c->lx - P.x, qx + c->lx - P.x};
          const double deltax = adx[minloc_abs3(adx)];
          double ady[3] = {qy - P.y, qy - c->ly - P.y, qy + c->ly - P.y};
          const double deltay = ady[minloc_abs3(ady)];
          const double dist = std::sqrt(deltax * deltax + deltay * deltay + deltaz * deltaz);
          const double nx = deltax / dist, ny = deltay / dist, nz = deltaz / dist;
          // polydisperse: contact at the sum of the radii, eps and the
          // lubrication prefactor with the equivalent radius (pair_consts)
          const double rp = prad(c, p), rqq = prad(c, q);
          const double rsum = c->poly ? rp + rqq : 2. * radius;
          const double re = c->poly ? 2. * rp * rqq / (rp + rqq) : radius;
          const double cfl = c->poly ? 6. * PI * c->visc * re : c->coeff_f;
          const double eps = (dist - rsum) / re;
          if ((eps < 0.025) && (eps > 0.)) lubrication(c, P, idq, nx, ny, nz, eps, su[q], sv[q], sw[q], cfl);
          int qq = 0;
          for (int i = 1; i <= P.qmax; ++i) {
            if (idq == P.firstc[i - 1]) {
              if (dist < rsum) {
                qq = i;
                collisions(c, p, qq, idq, dist, deltax, deltay, deltaz, su[q], sv[q], sw[q], sox[q], soy[q], soz[q], dt, rkiter);
              } else if (iter == itermax) {
                remove_contact(P, O, i, qlast);
              }
            }
          }
          if (qq == 0 && dist < rsum) {
            qlast = qlast + 1;
            if (qlast > c->nqmax) { status = IBM_E_CONTACT_OVERFLOW; qlast = c->nqmax; continue; }
            qq = qlast;
            new_contact(P, O, qq);
            collisions(c, p, qq, idq, dist, deltax, deltay, deltaz, su[q], sv[q], sw[q], sox[q], soy[q], soz[q], dt, rkiter);
            P.firstc[qlast - 1] = idq;
            O.firstc[qlast - 1] = idq;
          }
          P.qmax = qlast;
        }
      }
      // walls (:503-603); none with periodic z
      for (int q = botw; q <= (c->zper ? botw - 1 : topw); ++q) {
        const int idq = q;
        const double rp = prad(c, p);
        const double deltax = 0., deltay = 0., deltaz = (q - botw) * c->lz - P.z;
        const double dist = std::sqrt(deltax * deltax + deltay * deltay + deltaz * deltaz);
        const double deltan = rp - dist;
        const double nx = deltax / dist, ny = deltay / dist, nz = deltaz / dist;
        int qq = 0;
        const double eps = -deltan / rp;
        const double cfl = c->poly ? 6. * PI * c->visc * rp : c->coeff_f;
        if ((eps < 0.075) && (eps > 0.)) lubrication(c, P, idq, nx, ny, nz, eps, 0., 0., 0., cfl);
        for (int i = 1; i <= P.qmax; ++i) {
          if (idq == P.firstc[i - 1]) {
            qq = i;
            if (dist < rp) {
              collisions(c, p, qq, idq, dist, deltax, deltay, deltaz, 0., 0., 0., 0., 0., 0., dt, rkiter);
            } else if (iter == itermax) {
              remove_contact(P, O, i, qlast);
            }
          }
        }
        if ((qq == 0) && (dist < rp)) {
          qlast = qlast + 1;
          if (qlast > c->nqmax) { status = IBM_E_CONTACT_OVERFLOW; qlast = c->nqmax; continue; }
          qq = qlast;
          new_contact(P, O, qq);
          collisions(c, p, qq, idq, dist, deltax, deltay, deltaz, 0., 0., 0., 0., 0., 0., dt, rkiter);
          P.firstc[qlast - 1] = idq;
          O.firstc[qlast - 1] = idq;
        }
      }
      P.qmax = qlast;
    }
    // new particle positions (:607-667), colflg reset to 0 before use
    const double ab = c->rkcoeffab[rkiter - 1];
    for (int p = 0; p < pmax; ++p) {
      Part &P = c->ap[p];
      OldPart &O = c->op[p];
      if (P.mslv <= 0) continue;
      const double colflgx = 0., colflgy = 0., colflgz = 0.;
      const double vr = P.vol * P.ratiorho;
      P.u = O.u + (1 - colflgx) * ((-1.) * dt * (P.fxltot) / vr + (P.intu - O.intu) / vr) +
            ab * dt * c->gaccx * (1. - (1. / P.ratiorho)) + ab * 0.5 * dt * (P.colfx + O.colfx) / vr;
      P.x = O.x + ab * 0.5 * dt * (P.u + O.u);
      P.v = O.v + (1 - colflgy) * ((-1.) * dt * (P.fyltot) / vr + (P.intv - O.intv) / vr) +
            ab * dt * c->gaccy * (1. - (1. / P.ratiorho)) + ab * 0.5 * dt * (P.colfy + O.colfy) / vr;
      P.y = O.y + ab * 0.5 * dt * (P.v + O.v);
      P.w = O.w + (1 - colflgz) * ((-1.) * dt * (P.fzltot) / vr + (P.intw - O.intw) / vr) +
            ab * dt * c->gaccz * (1. - (1. / P.ratiorho)) + ab * 0.5 * dt * (P.colfz + O.colfz) / vr;
      P.z = O.z + ab * 0.5 * dt * (P.w + O.w);
      if (c->particle_rotation) {
        const double mr = P.mominert * P.ratiorho;
        P.omx = O.omx + (-1.) * dt * P.torqxltot / mr + (P.intomx - O.intomx) / mr + ab * 0.5 * dt * (P.coltx + O.coltx) / mr;
        P.omy = O.omy + (-1.) * dt * P.torqyltot / mr + (P.intomy - O.intomy) / mr + ab * 0.5 * dt * (P.colty + O.colty) / mr;
        P.omz = O.omz + (-1.) * dt * P.torqzltot / mr + (P.intomz - O.intomz) / mr + ab * 0.5 * dt * (P.coltz + O.coltz) / mr;
      } else {
        P.omx = 0.0; P.omy = 0.0; P.omz = 0.0;
      }
      P.phi = O.phi + 0.5 * ab * dt * (P.omz + O.omz);
      P.omtheta = (P.omy * std::cos(P.phi)) - (P.omx * std::sin(P.phi));
      P.theta = O.theta + ab * 0.5 * dt * (P.omtheta + O.omtheta);
    }
    sumrk3(c, rkiter, dt);
  }
  // periodic correction (:702-714)
  for (int p = 0; p < pmax; ++p) {
    Part &P = c->ap[p];
    if (P.mslv > 0) {
      if (P.x > c->lx) P.x = P.x - c->lx;
      if (P.x < 0.) P.x = P.x + c->lx;
      if (P.y > c->ly) P.y = P.y - c->ly;
      if (P.y < 0.) P.y = P.y + c->ly;
      if (c->zper) {  // periodic z: the same correction along z
        if (P.z > c->lz) P.z = P.z - c->lz;
        if (P.z < 0.) P.z = P.z + c->lz;
      }
    }
  }
  // re-ordering of masters (:716-1396): on one rank every particle stays
  // master and keeps its slot; the neighbour flags are recomputed and the
  // rkp accumulators are carried over except domx/y/zdt, which transfer
  // does not copy back (:1698-1718).
  for (int p = 0; p < pmax; ++p) {
    nb_flags(c, c->ap[p]);
    double *r = &c->rkp[(size_t)p * RK_N];
    r[RK_DOMX] = 0.; r[RK_DOMY] = 0.; r[RK_DOMZ] = 0.;
  }
  lagrangian_points(c);
  return status;
}

void alloc(orc_ctx *c) {
  const int ni = c->i1 + 1, nj = c->j1 + 1, nk = c->k1 + 1;
  for (Arr3 *a : {&c->unew, &c->vnew, &c->wnew, &c->pnew, &c->dudt, &c->dvdt, &c->dwdt,
                  &c->dudtold, &c->dvdtold, &c->dwdtold, &c->p, &c->durk, &c->dvrk, &c->dwrk, &c->cnew,
                  &c->dcdt, &c->dcrk})
    a->init(0, ni, nj, nk);
  for (Arr3 *a : {&c->dudtf, &c->dvdtf, &c->dwdtf}) a->init(-1, c->i1 + 3, c->j1 + 3, c->k1 + 3);
  c->ap.assign(c->npmax, Part());      // value-initialised: scalars zero
  c->op.assign(c->npmax, OldPart());
  for (auto &P : c->ap) {
    for (auto *v : {&P.dx, &P.dy, &P.dz, &P.dxt, &P.dyt, &P.dzt, &P.dut, &P.dvt, &P.dwt, &P.psi})
      v->assign(c->nqmax, 0.);
    P.firstc.assign(c->nqmax, 0);
    P.qmax = 0;
    P.fxltot = P.fyltot = P.fzltot = P.torqxltot = P.torqyltot = P.torqzltot = P.torqtheta = 0.;
    for (auto *v : {&P.xfp, &P.yfp, &P.zfp, &P.ul, &P.vl, &P.wl, &P.dudtl, &P.dvdtl, &P.dwdtl,
                    &P.fxl, &P.fyl, &P.fzl})
      v->assign(c->nl, 0.);
    P.vol = c->volp; P.mominert = c->mominert; P.ratiorho = c->ratiorho;
    P.mslv = 0;
    for (int n = 0; n < 9; ++n) P.nb[n] = 0;
  }
  for (auto &O : c->op) {
    for (auto *v : {&O.dx, &O.dy, &O.dz, &O.dxt, &O.dyt, &O.dzt, &O.dut, &O.dvt, &O.dwt, &O.psi})
      v->assign(c->nqmax, 0.);
    O.firstc.assign(c->nqmax, 0);
    O.qmax = 0;
  }
  c->rkp.assign((size_t)c->npmax * RK_N, 0.);
  c->nla.assign(c->npmax, 0);
}

// per-particle volume and moment of inertia (coordsfp.f90:96-102), with the
// particle's own radius when polydisperse
void set_sizes(orc_ctx *c) {
  for (size_t p = 0; p < c->ap.size(); ++p) {
    Part &P = c->ap[p];
    P.ratiorho = c->ratiorho;
    if (c->poly) {
      P.vol = (4. / 3.) * PI * std::pow(c->prad[p], 3.);
      P.mominert = (2. / 5.) * P.vol * std::pow(c->prad[p], 2.);
    } else {
      P.vol = c->volp;
      P.mominert = c->mominert;
    }
  }
}

// the IBM block of the driver (main.f90:286-338)
void forcing_loop(orc_ctx *c, double dt, int nl_iter) {
  c->dudtold.d = c->dudt.d;
  c->dvdtold.d = c->dvdt.d;
  c->dwdtold.d = c->dwdt.d;
  for (int k = 1; k <= c->kmax; ++k)
    for (int j = 1; j <= c->jmax; ++j)
      for (int i = 1; i <= c->imax; ++i) {
        c->dudtf(i, j, k) = c->dudt(i, j, k);
        c->dvdtf(i, j, k) = c->dvdt(i, j, k);
        c->dwdtf(i, j, k) = c->dwdt(i, j, k);
      }
  for (int ibmiter = 0; ibmiter < nl_iter; ++ibmiter) {
    eulr2lagr(c);
    lagrforces(c, dt, ibmiter == 0);
    lagr2eulr(c, dt);
    updtintermediatevel(c);
  }
  for (int k = 1; k <= c->kmax; ++k)
    for (int j = 1; j <= c->jmax; ++j)
      for (int i = 1; i <= c->imax; ++i) {
        c->dudt(i, j, k) = c->dudtf(i, j, k);
        c->dvdt(i, j, k) = c->dvdtf(i, j, k);
        c->dwdt(i, j, k) = c->dwdtf(i, j, k);
      }
}

// projection block of the driver (main.f90:356-372)
void project(orc_ctx *c, int rkiter, double dt) {
  bounduvw(c, c->dudt, c->dvdt, c->dwdt);
  fillps(c, rkiter, dt);
  solver2d(c);
  boundp(c, c->p);
  correc(c, rkiter, dt);
  bounduvw(c, c->unew, c->vnew, c->wnew);
  for (size_t n = 0; n < c->pnew.d.size(); ++n) c->pnew.d[n] = c->pnew.d[n] + c->p.d[n];
  boundp(c, c->pnew);
  if (c->have_scalar) {  // main.f90:374-376
    c->cnew.d = c->dcdt.d;
    boundscal(c, c->cnew);
  }
}

// phase_indicator (phase_indicator.f90:11-559) on one rank.  Every particle
// is its own master; its self-neighbour copies nbrecv = nb+4 (mod 8) for the
// flagged nb carry the shifted position only: the reference copies x, y, z
// into anb(nbrecv) (:83-119) and leaves u..omz at their zero initialisation
// (:68-78), so cells won by a copy get a zero rigid-body velocity.
void phase_indicator(orc_ctx *c, int itype, Arr3 &gamu, Arr3 &gamv, Arr3 &gamw, Arr3 &gamp, Arr3 &upart,
                     Arr3 &vpart, Arr3 &wpart) {
  struct Anb { double x, y, z, u, v, w, omx, omy, omz; };
  const double dx = 1. / c->dxi, dy = 1. / c->dyi, dz = 1. / c->dzi;
  const double radius = c->radius;
  const double radin = radius - 2. * dx;
  const double radin2 = radin * radin;
  const double bl = 0., bf = 0.;  // boundleftmyid, boundfrontmyid
  for (Arr3 *a : {&gamu, &gamv, &gamw, &gamp, &upart, &vpart, &wpart}) std::fill(a->d.begin(), a->d.end(), 0.);
  for (int p = 0; p < c->pmax; ++p) {
    const Part &P = c->ap[p];
    if (P.mslv == 0) continue;
    Anb anb[9];
    for (auto &a : anb) a = Anb{0, 0, 0, 0, 0, 0, 0, 0, 0};
    anb[0] = Anb{P.x, P.y, P.z, P.u, P.v, P.w, P.omx, P.omy, P.omz};
    for (int nb = 1; nb <= 8; ++nb) {
      int nbrecv = nb + 4; if (nbrecv > 8) nbrecv -= 8;
      if (P.mslv > 0 && P.nb[nb] == 1) {
        anb[nbrecv].x = anb[0].x; anb[nbrecv].y = anb[0].y; anb[nbrecv].z = anb[0].z;
        copy_shift_sphere(c, nbrecv, anb[nbrecv].x, anb[nbrecv].y);
      }
    }
    for (int nb = 0; nb <= 8; ++nb) {
      if (!((nb == 0 && P.mslv > 0) || (nb > 0 && P.mslv > 0 && P.nb[nb] == 1))) continue;
      int nbrecv = nb;
      if (nb > 0) { nbrecv = nb + 4; if (nbrecv > 8) nbrecv -= 8; }
      const Anb &A = anb[nbrecv];
      const double coorxc = A.x - bl, cooryc = A.y - bf, coorzc = A.z;
      int ilow = nint((coorxc - radius) * c->dxi - 2.), ihigh = nint((coorxc + radius) * c->dxi + 2.);
      int jlow = nint((cooryc - radius) * c->dyi - 2.), jhigh = nint((cooryc + radius) * c->dyi + 2.);
      int klow = nint((coorzc - radius) * c->dzi - 2.), khigh = nint((coorzc + radius) * c->dzi + 2.);
      if (ilow < 1) ilow = 1;
      if (jlow < 1) jlow = 1;
      if (klow < 1) klow = 1;
      if (ihigh > c->imax) ihigh = c->imax;
      if (jhigh > c->jmax) jhigh = c->jmax;
      if (khigh > c->kmax) khigh = c->kmax;
      // the eight corner distances in the reference's corner order
      auto frac = [&](double dxm2, double dxp2, double dym2, double dyp2, double dzm2, double dzp2) {
        double sg[8];
        sg[0] = radius - std::sqrt(dxm2 + dym2 + dzm2);
        sg[1] = radius - std::sqrt(dxm2 + dyp2 + dzm2);
        sg[2] = radius - std::sqrt(dxp2 + dyp2 + dzm2);
        sg[3] = radius - std::sqrt(dxp2 + dym2 + dzm2);
        sg[4] = radius - std::sqrt(dxm2 + dym2 + dzp2);
        sg[5] = radius - std::sqrt(dxm2 + dyp2 + dzp2);
        sg[6] = radius - std::sqrt(dxp2 + dyp2 + dzp2);
        sg[7] = radius - std::sqrt(dxp2 + dym2 + dzp2);
        double sum1 = 0., sum2 = 0.;
        for (int cp = 0; cp < 8; ++cp) {
          if (sg[cp] > 0.) sum1 = sum1 + sg[cp];
          sum2 = sum2 + std::fabs(sg[cp]);
        }
        return sum1 / sum2;
      };
      // u cells (:266-309)
      for (int k = klow; k <= khigh; ++k) {
        const double zmn = (k - 1) * dz, zpl = k * dz;
        const double dzp2 = (zpl - A.z) * (zpl - A.z);
        for (int j = jlow; j <= jhigh; ++j) {
          const double ymn = bf + (j - 1) * dy, ypl = bf + j * dy;
          const double dyp2 = (ypl - A.y) * (ypl - A.y);
          for (int i = ilow; i <= ihigh; ++i) {
            const double xmn = bl + (i - 0.5) * dx, xpl = bl + (i + 0.5) * dx;
            const double dxp2 = (xpl - A.x) * (xpl - A.x);
            const double dist2 = dxp2 + dyp2 + dzp2;
            const double vel = A.u + A.omy * ((k - 0.5) * dz - A.z) - A.omz * ((j - 0.5) * dy - A.y + bf);
            if (dist2 < radin2 && itype == 1) {
              gamu(i, j, k) = 1.;
              upart(i, j, k) = vel;
            } else {
              const double f = frac((xmn - A.x) * (xmn - A.x), dxp2, (ymn - A.y) * (ymn - A.y), dyp2,
                                    (zmn - A.z) * (zmn - A.z), dzp2);
              if (f > gamu(i, j, k) && itype == 1) { gamu(i, j, k) = f; upart(i, j, k) = vel; }
            }
          }
        }
      }
      // v cells (:313-356)
      for (int k = klow; k <= khigh; ++k) {
        const double zmn = (k - 1) * dz, zpl = k * dz;
        const double dzp2 = (zpl - A.z) * (zpl - A.z);
        for (int j = jlow; j <= jhigh; ++j) {
          const double ymn = bf + (j - 0.5) * dy, ypl = bf + (j + 0.5) * dy;
          const double dyp2 = (ypl - A.y) * (ypl - A.y);
          for (int i = ilow; i <= ihigh; ++i) {
            const double xmn = bl + (i - 1) * dx, xpl = bl + i * dx;
            const double dxp2 = (xpl - A.x) * (xpl - A.x);
            const double dist2 = dxp2 + dyp2 + dzp2;
            const double vel = A.v + A.omz * ((i - 0.5) * dx - A.x + bl) - A.omx * ((k - 0.5) * dz - A.z);
            if (dist2 < radin2 && itype == 1) {
              gamv(i, j, k) = 1.;
              vpart(i, j, k) = vel;
            } else {
              const double f = frac((xmn - A.x) * (xmn - A.x), dxp2, (ymn - A.y) * (ymn - A.y), dyp2,
                                    (zmn - A.z) * (zmn - A.z), dzp2);
              if (f > gamv(i, j, k) && itype == 1) { gamv(i, j, k) = f; vpart(i, j, k) = vel; }
            }
          }
        }
      }
      // w cells (:360-403)
      for (int k = klow; k <= khigh; ++k) {
        const double zmn = (k - 0.5) * dz, zpl = (k + 0.5) * dz;
        const double dzp2 = (zpl - A.z) * (zpl - A.z);
        for (int j = jlow; j <= jhigh; ++j) {
          const double ymn = bf + (j - 1) * dy, ypl = bf + j * dy;
          const double dyp2 = (ypl - A.y) * (ypl - A.y);
          for (int i = ilow; i <= ihigh; ++i) {
            const double xmn = bl + (i - 1) * dx, xpl = bl + i * dx;
            const double dxp2 = (xpl - A.x) * (xpl - A.x);
            const double dist2 = dxp2 + dyp2 + dzp2;
            const double vel = A.w + A.omx * ((j - 0.5) * dy - A.y + bf) - A.omy * ((i - 0.5) * dx - A.x + bl);
            if (dist2 < radin2 && itype == 1) {
              gamw(i, j, k) = 1.;
              wpart(i, j, k) = vel;
            } else {
              const double f = frac((xmn - A.x) * (xmn - A.x), dxp2, (ymn - A.y) * (ymn - A.y), dyp2,
                                    (zmn - A.z) * (zmn - A.z), dzp2);
              if (f > gamw(i, j, k) && itype == 1) { gamw(i, j, k) = f; wpart(i, j, k) = vel; }
            }
          }
        }
      }
      // pressure cells (:407-476)
      for (int k = klow; k <= khigh; ++k) {
        const double zmn = (k - 1) * dz, zpl = k * dz;
        const double dzp2 = (zpl - A.z) * (zpl - A.z);
        for (int j = jlow; j <= jhigh; ++j) {
          const double ymn = bf + (j - 1) * dy, ypl = bf + j * dy;
          const double dyp2 = (ypl - A.y) * (ypl - A.y);
          for (int i = ilow; i <= ihigh; ++i) {
            const double xmn = bl + (i - 1) * dx, xpl = bl + i * dx;
            const double dxp2 = (xpl - A.x) * (xpl - A.x);
            const double dist2 = dxp2 + dyp2 + dzp2;
            const double dxm2 = (xmn - A.x) * (xmn - A.x), dym2 = (ymn - A.y) * (ymn - A.y),
                         dzm2 = (zmn - A.z) * (zmn - A.z);
            if (dist2 < radin2 && itype == 1) {
              gamp(i, j, k) = 1.;
            } else {
              const double f = frac(dxm2, dxp2, dym2, dyp2, dzm2, dzp2);
              if (itype == 1) gamp(i, j, k) = std::max(f, gamp(i, j, k));
            }
            if (dist2 < radin2 && itype == 0) {
              gamp(i, j, k) = 1.;
              upart(i, j, k) = A.omx; vpart(i, j, k) = A.omy; wpart(i, j, k) = A.omz;
            } else {
              const double f = frac(dxm2, dxp2, dym2, dyp2, dzm2, dzp2);
              if (f > gamp(i, j, k) && itype == 0) {
                gamp(i, j, k) = f;
                upart(i, j, k) = A.omx; vpart(i, j, k) = A.omy; wpart(i, j, k) = A.omz;
              }
            }
          }
        }
      }
    }
  }
  // (:480-530)
  for (Arr3 *a : {&gamp, &gamu, &gamv, &gamw})
    for (auto &x : a->d) x = 1. - x;
  for (Arr3 *a : {&gamp, &gamu, &gamv, &gamw}) updthalos(c, *a, 1);
  for (Arr3 *a : {&gamp, &gamu, &gamv, &gamw}) updthalos(c, *a, 2);
  for (Arr3 *a : {&upart, &vpart, &wpart}) updthalos(c, *a, 1);
  for (Arr3 *a : {&upart, &vpart, &wpart}) updthalos(c, *a, 2);
  const int k1 = c->k1, kmax = c->kmax;
  for (int j = 0; j <= c->j1; ++j)
    for (int i = 0; i <= c->i1; ++i)
      for (Arr3 *a : {&gamu, &gamv, &gamw, &gamp}) {
        (*a)(i, j, 0) = (*a)(i, j, 1);
        (*a)(i, j, k1) = (*a)(i, j, kmax);
      }
  for (int j = 0; j <= c->j1; ++j)
    for (int i = 0; i <= c->i1; ++i) {
      upart(i, j, 0) = -upart(i, j, 1);
      vpart(i, j, 0) = -vpart(i, j, 1);
      wpart(i, j, 0) = 0.;
      upart(i, j, k1) = -upart(i, j, kmax);
      vpart(i, j, k1) = -vpart(i, j, kmax);
      wpart(i, j, kmax) = 0.;
      wpart(i, j, k1) = wpart(i, j, kmax - 1);
    }
}

// post1d (output.f90:13-917) without its file output: the plane sums
// (:88-364), ghost values, normalisations and derived scalars (:178-566).
// prof[q*(k1+1) + k] in the IBM_STAT_* order; entries the reference leaves
// unset are 0.  The quadrant analysis after the routine's `return` (:585) is
// dead code and not restated.
void post1d(orc_ctx *c, double *prof, double *scal) {
  const int kmax = c->kmax, k1 = c->k1, imax = c->imax, jmax = c->jmax;
  const int nk = k1 + 1;
  Arr3 gamu, gamv, gamw, gamp, upar, vpar, wpar;
  for (Arr3 *a : {&gamu, &gamv, &gamw, &gamp, &upar, &vpar, &wpar}) a->init(0, c->i1 + 1, c->j1 + 1, k1 + 1);
  if (c->np > 0) phase_indicator(c, 1, gamu, gamv, gamw, gamp, upar, vpar, wpar);
  const Arr3 &U = c->unew, &V = c->vnew, &W = c->wnew, &P = c->pnew, &C = c->cnew;
  std::vector<std::vector<double>> q(IBM_NSTAT, std::vector<double>(nk, 0.));
  auto &um = q[IBM_STAT_UM], &vm = q[IBM_STAT_VM], &wm = q[IBM_STAT_WM], &pm = q[IBM_STAT_PM];
  auto &u2 = q[IBM_STAT_U2], &v2 = q[IBM_STAT_V2], &w2 = q[IBM_STAT_W2], &p2 = q[IBM_STAT_P2];
  auto &uv = q[IBM_STAT_UV], &uw = q[IBM_STAT_UW], &vw = q[IBM_STAT_VW];
  auto &upm = q[IBM_STAT_UPM], &vpm = q[IBM_STAT_VPM], &wpm = q[IBM_STAT_WPM];
  auto &up2 = q[IBM_STAT_UP2], &vp2 = q[IBM_STAT_VP2], &wp2 = q[IBM_STAT_WP2];
  auto &upvp = q[IBM_STAT_UPVP], &upwp = q[IBM_STAT_UPWP], &vpwp = q[IBM_STAT_VPWP];
  auto &gum = q[IBM_STAT_GUM], &gvm = q[IBM_STAT_GVM], &gwm = q[IBM_STAT_GWM], &gpm = q[IBM_STAT_GPM];
  auto &gp2 = q[IBM_STAT_GP2], &guv = q[IBM_STAT_GUV], &guw = q[IBM_STAT_GUW], &gvw = q[IBM_STAT_GVW];
  auto &ss = q[IBM_STAT_SS], &ssp = q[IBM_STAT_SSP];
  auto &cm = q[IBM_STAT_CM], &c2 = q[IBM_STAT_C2], &wc = q[IBM_STAT_WC], &cdflx = q[IBM_STAT_CDFLX];
  const bool parts = c->np > 0;
  // first moments (:88-127); one thread per plane, as the reference's omp do
#pragma omp parallel for schedule(static)
  for (int k = 1; k <= kmax; ++k)
    for (int j = 1; j <= jmax; ++j)
      for (int i = 1; i <= imax; ++i) {
        if (parts) {
          um[k] = um[k] + U(i, j, k) * gamu(i, j, k);
          vm[k] = vm[k] + V(i, j, k) * gamv(i, j, k);
          wm[k] = wm[k] + W(i, j, k) * gamw(i, j, k);
          pm[k] = pm[k] + P(i, j, k) * gamp(i, j, k);
          cm[k] = cm[k] + C(i, j, k) * gamp(i, j, k);
        } else {
          um[k] = um[k] + U(i, j, k) * (1. - gamu(i, j, k));
          vm[k] = vm[k] + V(i, j, k) * (1. - gamv(i, j, k));
          wm[k] = wm[k] + W(i, j, k) * (1. - gamw(i, j, k));
          pm[k] = pm[k] + P(i, j, k) * (1. - gamp(i, j, k));
          cm[k] = cm[k] + C(i, j, k) * (1. - gamp(i, j, k));
        }
        upm[k] = upm[k] + upar(i, j, k) * (1. - gamu(i, j, k));
        vpm[k] = vpm[k] + vpar(i, j, k) * (1. - gamv(i, j, k));
        wpm[k] = wpm[k] + wpar(i, j, k) * (1. - gamw(i, j, k));
        gum[k] = gum[k] + gamu(i, j, k);
        gvm[k] = gvm[k] + gamv(i, j, k);
        gwm[k] = gwm[k] + gamw(i, j, k);
        gpm[k] = gpm[k] + gamp(i, j, k);
      }
  // (:178-200)
  um[0] = -um[1]; um[k1] = -um[kmax];
  vm[0] = -vm[1]; vm[k1] = -vm[kmax];
  wm[0] = 0.; wm[kmax] = 0.; wm[k1] = wm[kmax - 1];
  pm[0] = pm[1]; pm[k1] = pm[kmax];
  upm[0] = -upm[1]; upm[k1] = -upm[kmax];
  vpm[0] = -vpm[1]; vpm[k1] = -vpm[kmax];
  wpm[0] = 0.; wpm[kmax] = 0.; wpm[k1] = wm[kmax - 1];
  gum[0] = gum[1]; gum[k1] = gum[kmax];
  gvm[0] = gvm[1]; gvm[k1] = gvm[kmax];
  gwm[k1] = gwm[kmax - 1];
  // second moments (:207-238); x**2. is x*x
#pragma omp parallel for schedule(static)
  for (int k = 1; k <= kmax; ++k)
    for (int j = 1; j <= jmax; ++j)
      for (int i = 1; i <= imax; ++i) {
        const double uu = U(i, j, k), vv = V(i, j, k), ww = W(i, j, k), pp = P(i, j, k), cc = C(i, j, k);
        if (parts) {
          u2[k] = u2[k] + uu * uu * gamu(i, j, k);
          v2[k] = v2[k] + vv * vv * gamv(i, j, k);
          w2[k] = w2[k] + ww * ww * gamw(i, j, k);
          p2[k] = p2[k] + pp * pp * gamp(i, j, k);
          c2[k] = c2[k] + cc * cc * gamp(i, j, k);
        } else {
          u2[k] = u2[k] + uu * uu * (1. - gamu(i, j, k));
          v2[k] = v2[k] + vv * vv * (1. - gamv(i, j, k));
          w2[k] = w2[k] + ww * ww * (1. - gamw(i, j, k));
          p2[k] = p2[k] + pp * pp * (1. - gamp(i, j, k));
          c2[k] = c2[k] + cc * cc * (1. - gamp(i, j, k));
        }
        up2[k] = up2[k] + upar(i, j, k) * upar(i, j, k) * (1. - gamu(i, j, k));
        vp2[k] = vp2[k] + vpar(i, j, k) * vpar(i, j, k) * (1. - gamv(i, j, k));
        wp2[k] = wp2[k] + wpar(i, j, k) * wpar(i, j, k) * (1. - gamw(i, j, k));
        gp2[k] = gp2[k] + gamp(i, j, k) * gamp(i, j, k);
      }
  // (:276-294)
  u2[0] = -u2[1]; u2[k1] = -u2[kmax];
  v2[0] = -v2[1]; v2[k1] = -v2[kmax];
  w2[0] = 0.; w2[kmax] = 0.; w2[k1] = w2[kmax - 1];
  p2[0] = p2[1]; p2[k1] = p2[kmax];
  up2[0] = -up2[1]; up2[k1] = -up2[kmax];
  vp2[0] = -vp2[1]; vp2[k1] = -vp2[kmax];
  wp2[0] = 0.; wp2[kmax] = 0.; wp2[k1] = w2[kmax - 1];
  gp2[0] = gp2[1]; gp2[k1] = gp2[kmax];
  // products and fluxes (:301-355)
  const double kappa = c->kappa, dzi = c->dzi;
#pragma omp parallel for schedule(static)
  for (int k = 1; k <= kmax; ++k)
    for (int j = 1; j <= jmax; ++j)
      for (int i = 1; i <= imax; ++i) {
        uv[k] = uv[k] + 0.25 * (U(i, j + 1, k) + U(i, j, k)) * (V(i + 1, j, k) + V(i, j, k)) *
                            (0.25 * (gamu(i, j + 1, k) + gamu(i, j, k) + gamv(i + 1, j, k) + gamv(i, j, k)));
        uw[k] = uw[k] + 0.25 * (U(i, j, k + 1) + U(i, j, k)) * (W(i + 1, j, k) + W(i, j, k)) *
                            (0.25 * (gamu(i, j, k + 1) + gamu(i, j, k) + gamw(i + 1, j, k) + gamw(i, j, k)));
        vw[k] = vw[k] + 0.25 * (V(i, j, k + 1) + V(i, j, k)) * (W(i, j + 1, k) + W(i, j, k)) *
                            (0.25 * (gamv(i, j, k + 1) + gamv(i, j, k) + gamw(i, j + 1, k) + gamw(i, j, k)));
        wc[k] = wc[k] + 0.5 * (C(i, j, k + 1) + C(i, j, k)) * W(i, j, k) * (1 - gamw(i, j, k));
        cdflx[k] = cdflx[k] - kappa * (C(i, j, k + 1) - C(i, j, k)) * dzi;
        upvp[k] = upvp[k] + 0.25 * (upar(i, j + 1, k) + upar(i, j, k)) * (vpar(i + 1, j, k) + vpar(i, j, k)) *
                                (0.25 * (2. - gamu(i, j + 1, k) - gamu(i, j, k) + 2. - gamv(i + 1, j, k) -
                                         gamv(i, j, k)));
        upwp[k] = upwp[k] + 0.25 * (upar(i, j, k + 1) + upar(i, j, k)) * (wpar(i + 1, j, k) + wpar(i, j, k)) *
                                (0.25 * (2. - gamu(i, j, k + 1) - gamu(i, j, k) + 2. - gamw(i + 1, j, k) -
                                         gamw(i, j, k)));
        vpwp[k] = vpwp[k] + 0.25 * (vpar(i, j, k + 1) + vpar(i, j, k)) * (wpar(i, j + 1, k) + wpar(i, j, k)) *
                                (0.25 * (2. - gamv(i, j, k + 1) - gamv(i, j, k) + 2. - gamw(i, j + 1, k) -
                                         gamw(i, j, k)));
        guv[k] = guv[k] + 0.25 * (gamu(i, j + 1, k) + gamu(i, j, k) + (gamv(i + 1, j, k) + gamv(i, j, k)));
        guw[k] = guw[k] + 0.25 * (gamu(i, j, k + 1) + gamu(i, j, k) + (gamw(i + 1, j, k) + gamw(i, j, k)));
        gvw[k] = gvw[k] + 0.25 * (gamv(i, j, k + 1) + gamv(i, j, k) + (gamw(i, j + 1, k) + gamw(i, j, k)));
      }
  // (:401-422)
  uv[0] = -uv[1]; uv[k1] = -uv[kmax];
  uw[0] = 0.; uw[kmax] = 0.; uw[k1] = uw[kmax - 1];
  vw[0] = 0.; vw[k1] = vw[kmax - 1]; vw[kmax] = 0.;
  upvp[0] = -upvp[1]; upvp[k1] = -upvp[kmax];
  upwp[0] = 0.; upwp[kmax] = 0.; upwp[k1] = upwp[kmax - 1];
  vpwp[0] = 0.; vpwp[k1] = vpwp[kmax - 1]; vpwp[kmax] = 0.;
  guv[0] = guv[1]; guv[k1] = guv[kmax];
  guw[0] = guw[1]; guw[k1] = guw[kmax];
  gvw[0] = gvw[1]; gvw[k1] = gvw[kmax];
  // normalisation (:426-455); whole-array assignments read the old right-hand side
  const double N = 1. * c->itot * c->jtot;
  std::vector<double> vw_new(nk);
  for (int k = 1; k <= kmax; ++k) {
    const double du = parts ? gum[k] : N - gum[k], dv = parts ? gvm[k] : N - gvm[k];
    const double dw = parts ? gwm[k] : N - gwm[k], dp = parts ? gpm[k] : N - gpm[k];
    um[k] = um[k] / du; vm[k] = vm[k] / dv; wm[k] = wm[k] / dw;
    cm[k] = cm[k] / dp; pm[k] = pm[k] / dp;
  }
  for (int k = 1; k <= kmax; ++k) {
    const double du = parts ? gum[k] : N - gum[k], dv = parts ? gvm[k] : N - gvm[k];
    const double dw = parts ? gwm[k] : N - gwm[k], dp = parts ? gpm[k] : N - gpm[k];
    u2[k] = std::sqrt(u2[k] / du - um[k] * um[k]);
    v2[k] = std::sqrt(v2[k] / dv - vm[k] * vm[k]);
    w2[k] = std::sqrt(w2[k] / dw - wm[k] * wm[k]);
    p2[k] = std::sqrt(p2[k] / dp - pm[k] * pm[k]);
    c2[k] = std::sqrt(c2[k] / dp - cm[k] * cm[k]);
  }
  for (int k = 1; k <= kmax; ++k) {
    const double dvw = parts ? gvw[k] : N - gvw[k];
    vw_new[k] = vw[k] / dvw - 0.5 * (vm[k] + vm[k + 1]) * wm[k];
  }
  for (int k = 1; k <= kmax; ++k) vw[k] = vw_new[k];
  vw[0] = 0.;
  // (:457-477)
  double umax = u2[0];
  for (int k = 1; k <= k1; ++k) umax = std::max(umax, u2[k]);
  const double re_rbc = umax * c->lz / c->visc;
  for (int k = 1; k <= kmax; ++k) {
    wc[k] = wc[k] / (N - gwm[k]);
    cdflx[k] = cdflx[k] / (N - gwm[k]);
  }
  const double visc = c->visc;
  vm[0] = -vm[1]; vm[k1] = -vm[kmax];
  for (int k = 1; k <= kmax; ++k) ss[k] = (vm[k + 1] - vm[k]) * dzi * visc;
  ss[0] = (vm[1] - vm[0]) * dzi * visc;
  um[0] = -um[1]; um[k1] = -um[kmax];
  for (int k = 1; k <= kmax; ++k) {
    const double t = (um[k + 1] - um[k]) * dzi * visc;
    ss[k] = std::sqrt(ss[k] * ss[k] + t * t);
  }
  {
    const double t = (um[1] - um[0]) * dzi * visc;
    ss[0] = std::sqrt(ss[0] * ss[0] + t * t);
  }
  const double grad_k_wall = dzi * (std::sqrt(0.5 * (u2[1] * u2[1] + v2[1] * v2[1] + w2[1] * w2[1])) -
                                    std::sqrt(0.5 * (u2[0] * u2[0] + v2[0] * v2[0] + w2[0] * w2[0])));
  const double u_tau = std::sqrt(visc * grad_k_wall);
  const double re_tau = u_tau * c->lz / visc;
  double wcs = 0., cds = 0.;
  for (int k = 1; k <= kmax; ++k) wcs = wcs + wc[k];
  for (int k = 1; k <= kmax; ++k) cds = cds + cdflx[k];
  const double wc_avg = wcs / kmax, cdflx_avg = cds / kmax;
  const double nu = c->lz / (kappa * (c->bc_c_bot_val - c->bc_c_top_val)) * (wc_avg + cdflx_avg);
  // particle phase (:549-566)
  std::vector<double> vpwp_new(nk);
  for (int k = 1; k <= kmax; ++k) {
    upm[k] = upm[k] / (N - gum[k]);
    vpm[k] = vpm[k] / (N - gvm[k]);
    wpm[k] = wpm[k] / (N - gwm[k]);
  }
  for (int k = 1; k <= kmax; ++k) {
    up2[k] = std::sqrt(up2[k] / (N - gum[k]) - upm[k] * upm[k]);
    vp2[k] = std::sqrt(vp2[k] / (N - gvm[k]) - vpm[k] * vpm[k]);
    wp2[k] = std::sqrt(wp2[k] / (N - gwm[k]) - wpm[k] * wpm[k]);
  }
  for (int k = 1; k <= kmax; ++k) vpwp_new[k] = vpwp[k] / (N - gvw[k]) - 0.5 * (vpm[k] + vpm[k + 1]) * wpm[k];
  for (int k = 1; k <= kmax; ++k) vpwp[k] = vpwp_new[k];
  vpwp[0] = 0.;
  vpm[0] = -vpm[1]; vpm[k1] = -vpm[kmax];
  for (int k = 1; k <= kmax; ++k) ssp[k] = (vpm[k + 1] - vpm[k]) * dzi * visc;
  ssp[0] = (vpm[1] - vpm[0]) * dzi * visc;
  if (prof)
    for (int n = 0; n < IBM_NSTAT; ++n) std::memcpy(prof + (size_t)n * nk, q[n].data(), nk * sizeof(double));
  if (scal) { scal[0] = re_tau; scal[1] = u_tau; scal[2] = nu; scal[3] = re_rbc; scal[4] = grad_k_wall; }
}

void copy_in(orc_ctx *c, Arr3 &a, const double *src) {
  if (src) std::memcpy(a.d.data(), src, a.d.size() * sizeof(double));
  else std::fill(a.d.begin(), a.d.end(), 0.);
}
void copy_out(const Arr3 &a, double *dst) {
  if (dst) std::memcpy(dst, a.d.data(), a.d.size() * sizeof(double));
}

}  // namespace

extern "C" {

orc_ctx *orc_create(const ibm_params *prm) {
  if (!prm || prm->itot < 4 || prm->jtot < 4 || prm->ktot < 4 || prm->np < 0) return nullptr;
  orc_ctx *c = new orc_ctx();
  c->itot = prm->itot; c->jtot = prm->jtot; c->ktot = prm->ktot;
  c->imax = c->itot; c->jmax = c->jtot; c->kmax = c->ktot;
  c->i1 = c->imax + 1; c->j1 = c->jmax + 1; c->k1 = c->kmax + 1;
  c->lx = prm->lx; c->ly = prm->ly; c->lz = prm->lz; c->visc = prm->visc;
  c->radius = prm->radius; c->ratiorho = prm->ratiorho;
  c->bc_top = prm->bc_top; c->bc_bot = prm->bc_bot; c->particle_rotation = prm->particle_rotation;
  c->np = prm->np; c->nl = prm->nl;
  // periodic z: both boundaries, at most one particle (no particle images
  // across z in the collision pass)
  if ((prm->bc_top == IBM_BC_PERIODIC) != (prm->bc_bot == IBM_BC_PERIODIC) ||
      (prm->bc_top == IBM_BC_PERIODIC && prm->np > 1)) {
    delete c;
    return nullptr;
  }
  c->zper = prm->bc_top == IBM_BC_PERIODIC;
  c->nqmax = std::min(c->np + 2, 15);
  c->npmax = c->np;
  c->nb_copies = prm->nb_copies == 1 ? 1 : 9;
  derived_parameters(c);
  c->radfp = prm->radfp;
  if (prm->radii && c->np > 0) {
    // polydisperse: per-sphere point counts (the nl formula of init.f90:
    // 127-129 with the sphere's radius), shells and Lagrangian volumes
    // (coordsfp.f90:84-90); tables concatenated in particle order
    c->poly = true;
    const double retrac = 0.3 / c->dxi;
    int off = 0, nlmax = 0;
    for (int p = 0; p < c->np; ++p) {
      const double r = prm->radii[p];
      const int nlp = (int)std::lround((PI / 3.) * (12. * std::pow((r - retrac) * c->dxi, 2) + 1.));
      if (!(r > retrac) || nlp < 1) { delete c; return nullptr; }
      const double rfp = r - retrac;
      c->prad.push_back(r);
      c->pradfp.push_back(rfp);
      c->pnl.push_back(nlp);
      c->ptoff.push_back(off);
      c->pdvl.push_back(((4. / 3.) * PI * std::pow(rfp + 0.5 / c->dxi, 3.) -
                         (4. / 3.) * PI * std::pow(rfp - 0.5 / c->dxi, 3.)) / (1. * nlp));
      off += nlp;
      nlmax = std::max(nlmax, nlp);
    }
    if (nlmax != c->nl) { delete c; return nullptr; }
    c->thetarc.assign(prm->thetarc, prm->thetarc + off);
    c->phirc.assign(prm->phirc, prm->phirc + off);
  } else if (c->np > 0 && c->nl > 0) {
    c->thetarc.assign(prm->thetarc, prm->thetarc + c->nl);
    c->phirc.assign(prm->phirc, prm->phirc + c->nl);
  }
  alloc(c);
  initsolver(c);
  c->pmax = c->np;
  return c;
}

int orc_destroy(orc_ctx *c) { delete c; return IBM_OK; }
const char *orc_last_error(const orc_ctx *c) { return c ? c->err.c_str() : "null context"; }
int orc_sizes(const orc_ctx *c, int *nqmax, int *nl, int *ncells) {
  if (nqmax) *nqmax = c->nqmax;
  if (nl) *nl = c->nl;
  if (ncells) *ncells = (c->i1 + 1) * (c->j1 + 1) * (c->k1 + 1);
  return IBM_OK;
}

int orc_set_fields(orc_ctx *c, const double *u, const double *v, const double *w, const double *p,
                   const double *durk, const double *dvrk, const double *dwrk) {
  if (!u || !v || !w || !p) return fail(c, IBM_E_INVALID, "u, v, w and p are required");
  copy_in(c, c->unew, u); copy_in(c, c->vnew, v); copy_in(c, c->wnew, w); copy_in(c, c->pnew, p);
  copy_in(c, c->durk, durk); copy_in(c, c->dvrk, dvrk); copy_in(c, c->dwrk, dwrk);
  c->have_fields = true;
  return IBM_OK;
}
int orc_get_fields(orc_ctx *c, double *u, double *v, double *w, double *p, double *durk, double *dvrk, double *dwrk) {
  copy_out(c->unew, u); copy_out(c->vnew, v); copy_out(c->wnew, w); copy_out(c->pnew, p);
  copy_out(c->durk, durk); copy_out(c->dvrk, dvrk); copy_out(c->dwrk, dwrk);
  return IBM_OK;
}
int orc_get_intermediate(orc_ctx *c, double *du, double *dv, double *dw) {
  copy_out(c->dudt, du); copy_out(c->dvdt, dv); copy_out(c->dwdt, dw);
  return IBM_OK;
}

int orc_set_particles(orc_ctx *c, const ibm_particles *s) {
  const int nq = c->nqmax;
  for (int p = 0; p < c->np; ++p) {
    Part &P = c->ap[p];
    P.x = s->x[p]; P.y = s->y[p]; P.z = s->z[p]; P.theta = s->theta[p]; P.phi = s->phi[p];
    P.u = s->u[p]; P.v = s->v[p]; P.w = s->w[p]; P.omx = s->omx[p]; P.omy = s->omy[p]; P.omz = s->omz[p];
    P.omtheta = s->omtheta[p];
    P.intu = s->intu[p]; P.intv = s->intv[p]; P.intw = s->intw[p];
    P.intomx = s->intomx[p]; P.intomy = s->intomy[p]; P.intomz = s->intomz[p];
    P.colfx = s->colfx[p]; P.colfy = s->colfy[p]; P.colfz = s->colfz[p];
    P.coltx = s->coltx[p]; P.colty = s->colty[p]; P.coltz = s->coltz[p];
    P.fxltot = s->fxltot[p]; P.fyltot = s->fyltot[p]; P.fzltot = s->fzltot[p];
    P.torqxltot = s->torqxltot[p]; P.torqyltot = s->torqyltot[p]; P.torqzltot = s->torqzltot[p];
    P.torqtheta = s->torqtheta[p];
    P.qmax = s->qmax[p];
    for (int q = 0; q < nq; ++q) {
      const size_t o = (size_t)p * nq + q;
      P.firstc[q] = s->firstc[o];
      P.dx[q] = s->cdx[o]; P.dy[q] = s->cdy[o]; P.dz[q] = s->cdz[o];
      P.dxt[q] = s->cdxt[o]; P.dyt[q] = s->cdyt[o]; P.dzt[q] = s->cdzt[o];
      P.dut[q] = s->cdut[o]; P.dvt[q] = s->cdvt[o]; P.dwt[q] = s->cdwt[o]; P.psi[q] = s->cpsi[o];
    }
    P.mslv = s->mslv[p];
    // nb NULL: the flags from the centre, as a warm start sets them
    // (loadd.f90:362-397); rkp NULL: zero
    if (s->nb) for (int n = 0; n < 9; ++n) P.nb[n] = s->nb[(size_t)p * 9 + n];
    else nb_flags(c, P);
    for (int t = 0; t < RK_N; ++t) c->rkp[(size_t)p * RK_N + t] = s->rkp ? s->rkp[(size_t)p * RK_N + t] : 0.;
    c->op[p].firstc = P.firstc;
  }
  c->pmax = c->np;
  if (s->xfp) {
    for (int p = 0; p < c->np; ++p) {
      Part &P = c->ap[p];
      for (int l = 0; l < c->nl; ++l) {
        const size_t o = (size_t)p * c->nl + l;
        P.xfp[l] = s->xfp[o]; P.yfp[l] = s->yfp[o]; P.zfp[l] = s->zfp[o];
        P.ul[l] = s->ul[o]; P.vl[l] = s->vl[o]; P.wl[l] = s->wl[o];
        if (s->fxl) { P.fxl[l] = s->fxl[o]; P.fyl[l] = s->fyl[o]; P.fzl[l] = s->fzl[o]; }
      }
      c->nla[p] = c->poly ? c->pnl[p] : c->nl;
    }
  } else {
    lagrangian_points(c);
  }
  // dVlagr of the outer shell and dVeul (coordsfp.f90:84-90), and the
  // per-particle constants of initparticles: a warm start (main.f90:166-201)
  // runs coordsfp without intgr_over_sphere
  c->dVlagr = ((4. / 3.) * PI * std::pow(c->radfp + 0.5 / c->dxi, 3.) -
               (4. / 3.) * PI * std::pow(c->radfp - 0.5 / c->dxi, 3.)) / (1. * c->nl);
  c->dVeul = 1. / (c->dxi * c->dyi * c->dzi);
  set_sizes(c);
  c->have_particles = true;
  return IBM_OK;
}

int orc_get_particles(orc_ctx *c, ibm_particles *s) {
  // any member pointer may be NULL (not returned), as in the library
  const int nq = c->nqmax;
#define PUT(arr, idx, val) \
  do {                     \
    if (arr) (arr)[idx] = (val); \
  } while (0)
  for (int p = 0; p < c->np; ++p) {
    const Part &P = c->ap[p];
    PUT(s->x, p, P.x); PUT(s->y, p, P.y); PUT(s->z, p, P.z); PUT(s->theta, p, P.theta); PUT(s->phi, p, P.phi);
    PUT(s->u, p, P.u); PUT(s->v, p, P.v); PUT(s->w, p, P.w); PUT(s->omx, p, P.omx); PUT(s->omy, p, P.omy);
    PUT(s->omz, p, P.omz); PUT(s->omtheta, p, P.omtheta);
    PUT(s->intu, p, P.intu); PUT(s->intv, p, P.intv); PUT(s->intw, p, P.intw);
    PUT(s->intomx, p, P.intomx); PUT(s->intomy, p, P.intomy); PUT(s->intomz, p, P.intomz);
    PUT(s->colfx, p, P.colfx); PUT(s->colfy, p, P.colfy); PUT(s->colfz, p, P.colfz);
    PUT(s->coltx, p, P.coltx); PUT(s->colty, p, P.colty); PUT(s->coltz, p, P.coltz);
    PUT(s->fxltot, p, P.fxltot); PUT(s->fyltot, p, P.fyltot); PUT(s->fzltot, p, P.fzltot);
    PUT(s->torqxltot, p, P.torqxltot); PUT(s->torqyltot, p, P.torqyltot); PUT(s->torqzltot, p, P.torqzltot);
    PUT(s->torqtheta, p, P.torqtheta);
    PUT(s->qmax, p, P.qmax);
    for (int q = 0; q < nq; ++q) {
      const size_t o = (size_t)p * nq + q;
      PUT(s->firstc, o, P.firstc[q]);
      PUT(s->cdx, o, P.dx[q]); PUT(s->cdy, o, P.dy[q]); PUT(s->cdz, o, P.dz[q]);
      PUT(s->cdxt, o, P.dxt[q]); PUT(s->cdyt, o, P.dyt[q]); PUT(s->cdzt, o, P.dzt[q]);
      PUT(s->cdut, o, P.dut[q]); PUT(s->cdvt, o, P.dvt[q]); PUT(s->cdwt, o, P.dwt[q]); PUT(s->cpsi, o, P.psi[q]);
    }
    for (int n = 0; n < 9; ++n) PUT(s->nb, (size_t)p * 9 + n, P.nb[n]);
    PUT(s->mslv, p, P.mslv);
    for (int t = 0; t < RK_N; ++t) PUT(s->rkp, (size_t)p * RK_N + t, c->rkp[(size_t)p * RK_N + t]);
    for (int l = 0; l < c->nl; ++l) {
      const size_t o = (size_t)p * c->nl + l;
      PUT(s->xfp, o, P.xfp[l]); PUT(s->yfp, o, P.yfp[l]); PUT(s->zfp, o, P.zfp[l]);
      PUT(s->ul, o, P.ul[l]); PUT(s->vl, o, P.vl[l]); PUT(s->wl, o, P.wl[l]);
      PUT(s->fxl, o, P.fxl[l]); PUT(s->fyl, o, P.fyl[l]); PUT(s->fzl, o, P.fzl[l]);
    }
  }
#undef PUT
  return IBM_OK;
}

int orc_init_particles(orc_ctx *c, double *vol_calc) {
  // neighbour flags of each master as initparticles sets them
  // (initparticles.f90:206-242, one rank: bounds 0..lx, 0..ly)
  for (int p = 0; p < c->pmax; ++p) {
    c->ap[p].mslv = p + 1;
    nb_flags(c, c->ap[p]);
  }
  lagrangian_points(c);
  // dVlagr of the outer shell and dVeul (coordsfp.f90:84-90)
  c->dVlagr = ((4. / 3.) * PI * std::pow(c->radfp + 0.5 / c->dxi, 3.) -
               (4. / 3.) * PI * std::pow(c->radfp - 0.5 / c->dxi, 3.)) / (1. * c->nl);
  c->dVeul = 1. / (c->dxi * c->dyi * c->dzi);
  set_sizes(c);
  intgr_over_sphere(c, 1);
  if (vol_calc) *vol_calc = c->np > 0 ? c->ap[0].intu : 0.;
  intgr_over_sphere(c, 2);
  intgr_over_sphere(c, 3);
  return IBM_OK;
}

int orc_rk_predict(orc_ctx *c, int rkiter, double dt) {
  if (rkiter < 1 || rkiter > 3) return fail(c, IBM_E_INVALID, "rkiter must be 1..3");
  rk_stage(c, rkiter, dt);
  return IBM_OK;
}
int orc_forcing_loop(orc_ctx *c, double dt, int nl_iter) {
  if (c->np > 0) forcing_loop(c, dt, nl_iter);
  return IBM_OK;
}
int orc_project(orc_ctx *c, int rkiter, double dt) {
  if (rkiter < 1 || rkiter > 3) return fail(c, IBM_E_INVALID, "rkiter must be 1..3");
  project(c, rkiter, dt);
  return IBM_OK;
}
int orc_newton_euler(orc_ctx *c, int rkiter, double dt) {
  if (c->np == 0) return IBM_OK;
  int st = intgr_nwtn_eulr(c, rkiter, dt);
  if (st != IBM_OK) return fail(c, st, "contact list overflow (nqmax)");
  return IBM_OK;
}
int orc_rk3_step(orc_ctx *c, double dt) {
  for (int rkiter = 1; rkiter <= 3; ++rkiter) {
    int st;
    if ((st = orc_rk_predict(c, rkiter, dt))) return st;
    if ((st = orc_forcing_loop(c, dt, 3))) return st;
    if ((st = orc_project(c, rkiter, dt))) return st;
    if ((st = orc_newton_euler(c, rkiter, dt))) return st;
  }
  return IBM_OK;
}
int orc_run(orc_ctx *c, double dt, int nsteps) {
  for (int s = 0; s < nsteps; ++s) {
    int st = orc_rk3_step(c, dt);
    if (st) return st;
  }
  return IBM_OK;
}

// chkdiv (chkdiv.f90:7-61)
int orc_chkdiv(orc_ctx *c, double *divtot, double *divmax, int ijk[3]) {
  double dmax = 0., dtot = 0.;
  int im = 0, jm = 0, km = 0;
  for (int k = 1; k <= c->kmax; ++k)
    for (int j = 1; j <= c->jmax; ++j)
      for (int i = 1; i <= c->imax; ++i) {
        double div = (c->wnew(i, j, k) - c->wnew(i, j, k - 1)) * c->dzi +
                     (c->vnew(i, j, k) - c->vnew(i, j - 1, k)) * c->dyi +
                     (c->unew(i, j, k) - c->unew(i - 1, j, k)) * c->dxi;
        dtot = dtot + div;
        div = std::fabs(div);
        if (div > dmax) { dmax = div; im = i; jm = j; km = k; }
      }
  if (divtot) *divtot = dtot;
  if (divmax) *divmax = dmax;
  if (ijk) { ijk[0] = im; ijk[1] = jm; ijk[2] = km; }
  if (dtot > 1.e-3) return fail(c, IBM_E_DIVERGENCE, "total divergence > 1e-3");
  return IBM_OK;
}

// chkdt (chkdt.f90:6-273)
int orc_chkdt(orc_ctx *c, double *dtmax) {
  const double dxi = c->dxi, dyi = c->dyi, dzi = c->dzi;
  double best[3];
  for (int comp = 0; comp < 3; ++comp) {
    double m = 899999.;
    for (int k = 1; k <= c->kmax; ++k)
      for (int j = 1; j <= c->jmax; ++j)
        for (int i = 1; i <= c->imax; ++i) {
          const double dxi2 = dxi * dxi + dyi * dyi + dzi * dzi;
          const double dt1 = 1.65 / (4. * c->visc * dxi2);
          double u2, v2, w2;
          const Arr3 &U = c->unew, &V = c->vnew, &W = c->wnew;
          if (comp == 0) {
            u2 = U(i, j, k) * U(i, j, k);
            double t = 0.25 * (V(i, j, k) + V(i, j - 1, k) + V(i + 1, j, k) + V(i + 1, j - 1, k)); v2 = t * t;
            t = 0.25 * (W(i, j, k) + W(i, j, k - 1) + W(i + 1, j, k) + W(i + 1, j, k - 1)); w2 = t * t;
          } else if (comp == 1) {
            double t = 0.25 * (U(i, j, k) + U(i, j + 1, k) + U(i - 1, j + 1, k) + U(i - 1, j, k)); u2 = t * t;
            v2 = V(i, j, k) * V(i, j, k);
            t = 0.25 * (W(i, j, k) + W(i, j + 1, k) + W(i, j + 1, k - 1) + W(i, j, k - 1)); w2 = t * t;
          } else {
            double t = 0.25 * (U(i, j, k) + U(i - 1, j, k) + U(i - 1, j, k + 1) + U(i, j, k + 1)); u2 = t * t;
            t = 0.25 * (V(i, j, k) + V(i, j - 1, k) + V(i, j - 1, k + 1) + V(i, j, k + 1)); v2 = t * t;
            w2 = W(i, j, k) * W(i, j, k);
          }
          const double velo = std::sqrt(u2 + v2 + w2);
          double dt2;
          if (std::fabs(1. * velo) > 1.e-12)
            dt2 = std::sqrt(3.) / (std::sqrt(u2) * dxi + std::sqrt(v2) * dyi + std::sqrt(w2) * dzi);
          else
            dt2 = 99999.;
          m = std::min(m, std::min(dt1, dt2));
        }
    best[comp] = m;
  }
  *dtmax = std::min(best[0], std::min(best[1], best[2]));
  return IBM_OK;
}

int orc_slip_residual(orc_ctx *c, double *maxres, double *rmsres) {
  double mx = 0., s = 0.;
  long n = 0;
  for (int p = 0; p < c->pmax; ++p) {
    const Part &P = c->ap[p];
    for (int l = 0; l < c->nla[p]; ++l) {
      double ex = P.ul[l] - P.dudtl[l], ey = P.vl[l] - P.dvdtl[l], ez = P.wl[l] - P.dwdtl[l];
      double r = std::sqrt(ex * ex + ey * ey + ez * ez);
      mx = std::max(mx, r);
      s += r * r;
      ++n;
    }
  }
  if (maxres) *maxres = mx;
  if (rmsres) *rmsres = n ? std::sqrt(s / n) : 0.;
  return IBM_OK;
}

int orc_diagnostics(orc_ctx *c, double *wsn, double *wso, double ft[3]) {
  if (wsn) *wsn = c->wallshearnew;
  if (wso) *wso = c->wallshearold;
  if (ft) { ft[0] = c->forcetot[0]; ft[1] = c->forcetot[1]; ft[2] = c->forcetot[2]; }
  return IBM_OK;
}

int orc_set_scalar(orc_ctx *c, const ibm_scalar_params *sp, const double *cf, const double *dcrk) {
  if (!sp || !(sp->pran > 0.)) return fail(c, IBM_E_INVALID, "scalar parameters need pran > 0");
  if (c->zper) return fail(c, IBM_E_STATE, "no scalar transport with periodic z");
  c->kappa = c->visc / sp->pran;  // init.f90:94
  c->beta = sp->beta;
  c->bc_c_top_val = sp->bc_c_top_val; c->bc_c_bot_val = sp->bc_c_bot_val;
  c->bc_c_top_type = sp->bc_c_top_type; c->bc_c_bot_type = sp->bc_c_bot_type;
  copy_in(c, c->cnew, cf);
  copy_in(c, c->dcrk, dcrk);
  boundscal(c, c->cnew);  // as the driver does after loading (main.f90:198)
  c->have_scalar = true;
  return IBM_OK;
}
int orc_get_scalar(orc_ctx *c, double *cf, double *dcrk) {
  copy_out(c->cnew, cf);
  copy_out(c->dcrk, dcrk);
  return IBM_OK;
}
int orc_phase_indicator(orc_ctx *c, int itype, double *gamu, double *gamv, double *gamw, double *gamp,
                        double *upart, double *vpart, double *wpart) {
  if (itype != 0 && itype != 1) return fail(c, IBM_E_INVALID, "itype must be 0 or 1");
  if (c->zper || c->poly) return fail(c, IBM_E_STATE, "no plane statistics with periodic z or polydisperse spheres");
  Arr3 a[7];
  for (auto &x : a) x.init(0, c->i1 + 1, c->j1 + 1, c->k1 + 1);
  phase_indicator(c, itype, a[0], a[1], a[2], a[3], a[4], a[5], a[6]);
  double *out[7] = {gamu, gamv, gamw, gamp, upart, vpart, wpart};
  for (int n = 0; n < 7; ++n) copy_out(a[n], out[n]);
  return IBM_OK;
}
int orc_post1d(orc_ctx *c, double *profiles, double *scalars) {
  if (!c->have_fields) return fail(c, IBM_E_STATE, "no fields set");
  if (c->zper || c->poly) return fail(c, IBM_E_STATE, "no plane statistics with periodic z or polydisperse spheres");
  post1d(c, profiles, scalars);
  return IBM_OK;
}

double orc_kernel(double r) { return kernel(r); }

// kerneltest (kernel.f90:43-63)
double orc_kerneltest(void) {
  double sum = 0.;
  for (int k = -25; k <= 25; ++k) {
    double coorz = k / 12.;
    for (int j = -25; j <= 25; ++j) {
      double coory = j / 12.;
      for (int i = -25; i <= 25; ++i) {
        double coorx = i / 12.;
        sum = sum + (1. / 12.) * (1. / 12.) * (1. / 12.) * kernel(coorx) * kernel(coory) * kernel(coorz);
      }
    }
  }
  return sum;
}

int orc_vrfft(double *r, int n, int dir) {
  if (!r || n < 1) return IBM_E_INVALID;
  vrfft(r, n, dir);
  return IBM_OK;
}

// nl (init.f90:127-129)
int orc_nl(double radius, double dxi) {
  const double retrac = 0.3 / dxi;
  return nint((PI / 3.) * (12. * std::pow((radius - retrac) * dxi, 2) + 1.));
}

int orc_set_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
  return omp_get_max_threads();
#else
  (void)n;
  return 1;
#endif
}

}  // extern "C"
