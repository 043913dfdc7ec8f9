// ibm_common.cuh -- device data layout and helpers shared by the kernels.
//
// HBM layout (one rank, periodic x/y, walls in z):
//   cell fields   F[(k*J + j)*I + i], i in [0,I), j in [0,J), k in [0,K+1]
//                 -> reference F(i+1, j+1, k); the x/y ghosts of the
//                 reference are replaced by periodic index wrap, the z ghost
//                 planes k=0 and k=K+1 are stored.
//   spectra       S[(k*J + ky)*MX + kx], complex, kx in [0, I/2], MX = I/2+1,
//                 k in [0,K) (reference k-1).
//   particles     scalar state pf[f*np + p] (field-major), contact arrays
//                 [p*nq + q], Lagrangian arrays [p*nl + l].
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/ibm_rk3.h"

#define IBM_PI 3.141592653589793238462643383279502884

// particle scalar fields (order of the reference type `particle`, then the
// force totals, then the old-state copy `op`)
enum PField {
  PF_X, PF_Y, PF_Z, PF_THETA, PF_PHI, PF_U, PF_V, PF_W, PF_OMX, PF_OMY, PF_OMZ, PF_OMTHETA,
  PF_INTU, PF_INTV, PF_INTW, PF_INTOMX, PF_INTOMY, PF_INTOMZ,
  PF_COLFX, PF_COLFY, PF_COLFZ, PF_COLTX, PF_COLTY, PF_COLTZ,
  PF_FXLTOT, PF_FYLTOT, PF_FZLTOT, PF_TQX, PF_TQY, PF_TQZ, PF_TQTHETA,
  // old state (op), same order as the first 24 fields
  PF_OX, PF_OY, PF_OZ, PF_OTHETA, PF_OPHI, PF_OU, PF_OV, PF_OW, PF_OOMX, PF_OOMY, PF_OOMZ, PF_OOMTHETA,
  PF_OINTU, PF_OINTV, PF_OINTW, PF_OINTOMX, PF_OINTOMY, PF_OINTOMZ,
  PF_OCOLFX, PF_OCOLFY, PF_OCOLFZ, PF_OCOLTX, PF_OCOLTY, PF_OCOLTZ,
  // snapshot of the collision pass (anb(:,0)): x,y,z,u,v,w,omx,omy,omz
  PF_SX, PF_SY, PF_SZ, PF_SU, PF_SV, PF_SW, PF_SOMX, PF_SOMY, PF_SOMZ,
  PF_N
};
// contact arrays: current and old
enum CField { CF_DX, CF_DY, CF_DZ, CF_DXT, CF_DYT, CF_DZT, CF_DUT, CF_DVT, CF_DWT, CF_PSI,
              CF_ODX, CF_ODY, CF_ODZ, CF_ODXT, CF_ODYT, CF_ODZT, CF_ODUT, CF_ODVT, CF_ODWT, CF_N };
// rkp accumulators (particle_sumrk, common.f90:97-105)
enum RKField { RK_FX, RK_FY, RK_FZ, RK_TX, RK_TY, RK_TZ, RK_TT, RK_CFX, RK_CFY, RK_CFZ,
               RK_CTX, RK_CTY, RK_CTZ, RK_DUDT, RK_DVDT, RK_DWDT, RK_DOMX, RK_DOMY, RK_DOMZ, RK_N };

// Per-point stencil of the 3-point delta (interp_spread.f90:76-130), cached
// once per substep because the points do not move during the forcing loop.
struct PointStencil {
  int ilow, jlow, klow, ilows, jlows, klows;  // reference indices
  double phix[3], phiy[3], phiz[3], phixh[3], phiyh[3], phizh[3];
};

// Mixed form: one velocity component of one Lagrangian point: index of tap
// (0,0,0) of the 3x3x3 block (x, y unwrapped) and the component's FP32 delta
// weights wx[3], wy[3], wz[3], formed in registers from the point's record
// (make_cs)
struct __align__(16) CompStencil {
  int b[3];
  float w[9];
};

// Mixed form: one Lagrangian point in 16 bytes, written once per substep:
// the fractions of its grid coordinates x dxi, y dyi, z dzi (FP32, exact
// from FP64 floors) and the floors themselves as 10-bit offsets (+512) from
// its particle's reference floor (the floors of the centre's coordinates).
// Every pass recomputes a component's stencil from it (make_cs).
struct __align__(16) PointRec {
  float fx, fy, fz;
  unsigned rel;  // (nx - refx + 512) | (ny - refy + 512) << 10 | (nz - refz + 512) << 20
};
__device__ __forceinline__ int rec_dx(unsigned r) { return (int)(r & 1023u) - 512; }
__device__ __forceinline__ int rec_dy(unsigned r) { return (int)((r >> 10) & 1023u) - 512; }
__device__ __forceinline__ int rec_dz(unsigned r) { return (int)((r >> 20) & 1023u) - 512; }

// Constants of one context, passed by value to the kernels.
struct Geo {
  int I, J, K, MX;            // grid, MX = I/2+1
  long plane, nfield;         // I*J, (K+2)*I*J
  double lx, ly, lz, dxi, dyi, dzi, dx, dy, dz, visc;
  int bc_top, bc_bot;
  int zper;  // periodic z (IBM_BC_PERIODIC): ghost planes are copies, no walls
};

struct PartGeo {
  int np, nl, nq, nb_copies, rotation;
  double radius, radfp, offset, dVlagr, dVeul, lx, ly, lz, dxi, dyi, dzi, dx, dy, dz;
  double gacc[3], rkab[3], volp, ratiorho, mominert, rthr;
  double kn_ss, etan_ss, kt_ss, etat_ss, muc_ss, kn_sw, etan_sw, kt_sw, etat_sw, muc_sw;
  double coeff_f, a11a_ini_pp, a11b_ini_pp, a11a_sat_pp, a11b_sat_pp, a11_ini_pw, a11_sat_pw;
  int I, J, K;
  int zper;  // periodic z: stencils and sphere boxes wrap in z, no walls
  // polydisperse (poly = 1): per-sphere radius, force-point shell radius,
  // Lagrangian volume, volume, moment of inertia, sphere-integral threshold
  // (smallest double whose square root is >= the radius), point count and
  // offset into the point table; rmax the largest radius
  int poly;
  double visc;
  // host-formed factors of the pair constants: kn = (pc_an me) / pc_b,
  // kt = (pc_at mt) / pc_b, etan = (pc_en me) / pc_ndt, etat = (pc_et mt) / pc_ndt
  double pc_an, pc_at, pc_b, pc_en, pc_et, pc_ndt;
  const double *prad, *pradfp, *pdvl, *pvol, *pmi, *prthr;
  const int *pnl, *ptoff;
  double rmax;
  int ntab;     // entries of each of the four point tables (sum of the point counts)
  int box_cap;  // mixed form: cells of the shared-memory box of one (particle, component)
  // uniform cell list of the collision candidate search: cells at least
  // 1.01 x the FP32 filter distance 2.1 R wide (ncx, ncy >= 3, else the
  // search scans all particles)
  int ncx, ncy, ncz;
  float cix, ciy, ciz;  // cells per unit length
};

// per-sphere sizes: the particle's own when polydisperse, else the scalars
__device__ __forceinline__ double p_rad(const PartGeo &pg, int p) { return pg.poly ? pg.prad[p] : pg.radius; }
__device__ __forceinline__ double p_radfp(const PartGeo &pg, int p) { return pg.poly ? pg.pradfp[p] : pg.radfp; }
__device__ __forceinline__ double p_dvl(const PartGeo &pg, int p) { return pg.poly ? pg.pdvl[p] : pg.dVlagr; }
__device__ __forceinline__ double p_vol(const PartGeo &pg, int p) { return pg.poly ? pg.pvol[p] : pg.volp; }
__device__ __forceinline__ double p_mi(const PartGeo &pg, int p) { return pg.poly ? pg.pmi[p] : pg.mominert; }
__device__ __forceinline__ double p_rthr(const PartGeo &pg, int p) { return pg.poly ? pg.prthr[p] : pg.rthr; }
__device__ __forceinline__ int p_nl(const PartGeo &pg, int p) { return pg.poly ? pg.pnl[p] : pg.nl; }
__device__ __forceinline__ int p_toff(const PartGeo &pg, int p) { return pg.poly ? pg.ptoff[p] : 0; }

__host__ __device__ inline long fidx(const Geo &g, int i, int j, int k) {
  return ((long)k * g.J + j) * g.I + i;
}
__device__ __forceinline__ int wrapm(int i, int n) {  // i in [-n, 2n)
  return i < 0 ? i + n : (i >= n ? i - n : i);
}
// z plane of a stencil tap: as given with walls (ghost planes stored);
// periodic z maps planes 0, K+1, K+2 onto K, 1, 2
__device__ __forceinline__ int zwrap(const Geo &g, int k) {
  return g.zper ? (k < 1 ? k + g.K : (k > g.K ? k - g.K : k)) : k;
}

// Roma-Peskin 3-point regularised delta times h (kernel.f90:7-25)
__device__ __forceinline__ double delta3(double r) {
  const double ar = fabs(r);
  if (ar > 1.5) return 0.;
  if (ar > 0.5) return (1. / 6.) * (5. - 3. * ar - sqrt(-3. * ((1. - ar) * (1. - ar)) + 1.));
  return (1. / 3.) * (1. + sqrt(-3. * (r * r) + 1.));
}
__device__ __forceinline__ float delta3f(float r) {
  const float ar = fabsf(r);
  if (ar > 1.5f) return 0.f;
  if (ar > 0.5f) return (1.f / 6.f) * (5.f - 3.f * ar - sqrtf(-3.f * ((1.f - ar) * (1.f - ar)) + 1.f));
  return (1.f / 3.f) * (1.f + sqrtf(-3.f * (r * r) + 1.f));
}
// Square root, approximate (relative error about 2^-22; the mixed form's
// delta weights are FP32 approximations of the FP64 ones anyway).
__device__ __forceinline__ float sqrt_apx(float x) {
  float y;
  asm("sqrt.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
// FP32 delta weights at three consecutive nodes m = 0, 1, 2 of a point whose
// signed distance from node 1 is r1 = x_1 - x_point (in cells).  For r1 in
// (-0.5, 0.5] node 1 takes the inner branch of kernel.f90:7-25 and nodes 0
// and 2 (distances 1 - r1 and 1 + r1) the outer one, and all three share
// sqrt(1 - 3 r1^2): w1 = (1 + s)/3, w0 = (2 + 3 r1 - s)/6,
// w2 = (2 - 3 r1 - s)/6 (they sum to one).  Any other r1 (a wall-clamped
// origin in z) takes the general form node by node.
__device__ __forceinline__ void delta3w(float r1, float *w) {
  if (r1 > -0.5f && r1 <= 0.5f) {
    const float s = sqrt_apx(fmaf(-3.f * r1, r1, 1.f));
    w[1] = (1.f + s) * (1.f / 3.f);
    w[0] = (fmaf(3.f, r1, 2.f) - s) * (1.f / 6.f);
    w[2] = (fmaf(-3.f, r1, 2.f) - s) * (1.f / 6.f);
  } else {
    w[0] = delta3f(r1 - 1.f);
    w[1] = delta3f(r1);
    w[2] = delta3f(r1 + 1.f);
  }
}
// Stencil of velocity component c (0 u, 1 v, 2 w) of a point, as eulr2lagr
// forms it (interp_spread.f90:60-131): tap (0,0,0) of the 3x3x3 block
// relative to the particle's reference floor in x and y and absolute in z
// (refz: the reference floor in z), and the component's FP32 delta weights.
// Along the component's own axis the staggered origin (ilows, jlows, klows:
// the nearest face, max(.,1) in z) and offsets; along the other axes the
// cell-centred origin (ilow, jlow, klow clamped to [1, K-2], quirk Q5).
// The delta argument of node m is m - o with o the point's offset from the
// origin (own axis) or m - 1/2 - o (cell-centred axes); delta3w takes the
// distance r1 of node 1.
__device__ __forceinline__ CompStencil make_cs(const PointRec &r, int c, int refz, int K) {
  const int dx = rec_dx(r.rel), dy = rec_dy(r.rel), nz = refz + rec_dz(r.rel);
  CompStencil s;
  if (c == 0) {
    const int ux = r.fx >= 0.5f;
    s.b[0] = dx + ux - 2;
    delta3w((float)ux - r.fx, s.w);  // 1 - (fx + 1 - ux)
  } else {
    s.b[0] = dx - 1;
    delta3w(0.5f - r.fx, s.w);
  }
  if (c == 1) {
    const int uy = r.fy >= 0.5f;
    s.b[1] = dy + uy - 2;
    delta3w((float)uy - r.fy, s.w + 3);
  } else {
    s.b[1] = dy - 1;
    delta3w(0.5f - r.fy, s.w + 3);
  }
  if (c == 2) {
    const int uz = r.fz > 0.5f || (r.fz == 0.5f && nz >= 0);
    const int klows = max(nz + uz - 1, 1);
    s.b[2] = klows;
    delta3w(1.f - (r.fz + (float)(nz - klows)), s.w + 6);
  } else {
    const int klow = max(min(nz, K - 2), 1);
    s.b[2] = klow;
    delta3w(0.5f - (r.fz + (float)(nz - klow)), s.w + 6);
  }
  return s;
}
// Offset of a point from its particle's centre along one axis, FP32: the
// point's floor offset d from the particle's reference floor plus its
// fraction fr, minus the centre's position cf relative to the same floor
// (all in cells), times the cell size h.
__device__ __forceinline__ float rec_armf(int d, float fr, float cf, float h) {
  return (((float)d - cf) + fr) * h;
}
// Error-free FP32 transformations (Knuth two-sum, FMA two-product) for
// double-float arithmetic: a value is carried as hi + lo (about 48 bits) on the
// FP32 pipes, which GB300 runs 64x faster than FP64.
__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e) {
  s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}
__device__ __forceinline__ void two_prod(float a, float b, float &p, float &e) {
  p = __fmul_rn(a, b);
  e = fmaf(a, b, -p);
}
// (ah + al) * (bh + bl) -> (ph + pl)
__device__ __forceinline__ void df_mul(float ah, float al, float bh, float bl, float &ph, float &pl) {
  float p, e;
  two_prod(ah, bh, p, e);
  e = fmaf(ah, bl, fmaf(al, bh, e));
  ph = __fadd_rn(p, e);
  pl = __fsub_rn(e, __fsub_rn(ph, p));
}
// (ah + al) + (bh + bl) -> (sh + sl)
__device__ __forceinline__ void df_add(float ah, float al, float bh, float bl, float &sh, float &sl) {
  float s, e;
  two_sum(ah, bh, s, e);
  e = __fadd_rn(e, __fadd_rn(al, bl));
  sh = __fadd_rn(s, e);
  sl = __fsub_rn(e, __fsub_rn(sh, s));
}

// Sums of three per-thread double-float values (h[q] + l[q]) over the block
// (blockDim a multiple of 32, at most 1024) with error-free TwoSum steps on
// the FP32 pipes, about 48 significant bits, widened to FP64 by three
// threads at the end: no FP64 instruction per warp (this GPU issues FP64 at
// 1/64 of the FP32 rate).  st: 192 floats of shared memory; res[0..2] valid
// for every thread after the call.
__device__ __forceinline__ void block_sum3_df2(float h[3], float l[3], float *st, double *res) {
#pragma unroll
  for (int d = 16; d > 0; d >>= 1)
#pragma unroll
    for (int q = 0; q < 3; ++q) {
      const float oh = __shfl_xor_sync(0xffffffffu, h[q], d), ol = __shfl_xor_sync(0xffffffffu, l[q], d);
      df_add(h[q], l[q], oh, ol, h[q], l[q]);
    }
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  if (lane == 0)
#pragma unroll
    for (int q = 0; q < 3; ++q) {
      st[(2 * q) * 32 + w] = h[q];
      st[(2 * q + 1) * 32 + w] = l[q];
    }
  __syncthreads();
  if (threadIdx.x < 3) {
    const int q = threadIdx.x;
    float sh = 0.f, sl = 0.f;
    for (int k = 0; k < nw; ++k) df_add(sh, sl, st[(2 * q) * 32 + k], st[(2 * q + 1) * 32 + k], sh, sl);
    res[q] = (double)sh + (double)sl;
  }
  __syncthreads();
}
// the same for three per-thread FP32 values
__device__ __forceinline__ void block_sum3_df(float a, float b, float c, float *st, double *res) {
  float h[3] = {a, b, c}, l[3] = {0.f, 0.f, 0.f};
  block_sum3_df2(h, l, st, res);
}

// Fortran NINT (half away from zero)
__device__ __forceinline__ int fnint(double x) { return (int)round(x); }

// launch helpers (the host side counts every launch)
#define IBM_CHECK_LAUNCH() cudaGetLastError()
