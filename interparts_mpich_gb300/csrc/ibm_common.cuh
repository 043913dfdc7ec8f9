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
// weights wx[3], wy[3], wz[3] (48 bytes, read as three float4)
struct __align__(16) CompStencil {
  int b[3];
  float w[9];
};
// one 48-byte record as three 16-byte loads
__device__ __forceinline__ CompStencil load_cs(const CompStencil *p) {
  const float4 *q = reinterpret_cast<const float4 *>(p);
  const float4 a = q[0], bb = q[1], c = q[2];
  CompStencil s;
  s.b[0] = __float_as_int(a.x); s.b[1] = __float_as_int(a.y); s.b[2] = __float_as_int(a.z);
  s.w[0] = a.w; s.w[1] = bb.x; s.w[2] = bb.y; s.w[3] = bb.z; s.w[4] = bb.w;
  s.w[5] = c.x; s.w[6] = c.y; s.w[7] = c.z; s.w[8] = c.w;
  return s;
}

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
};

struct PartGeo {
  int np, nl, nq, nb_copies, rotation;
  double radius, radfp, offset, dVlagr, dVeul, lx, ly, lz, dxi, dyi, dzi, dx, dy, dz;
  double gacc[3], rkab[3], volp, ratiorho, mominert, rthr;
  double kn_ss, etan_ss, kt_ss, etat_ss, muc_ss, kn_sw, etan_sw, kt_sw, etat_sw, muc_sw;
  double coeff_f, a11a_ini_pp, a11b_ini_pp, a11a_sat_pp, a11b_sat_pp, a11_ini_pw, a11_sat_pw;
  int I, J, K;
  // uniform cell list of the collision candidate search: cells at least
  // 1.01 x the FP32 filter distance 2.1 R wide (ncx, ncy >= 3, else the
  // search scans all particles)
  int ncx, ncy, ncz;
  float cix, ciy, ciz;  // cells per unit length
};

__host__ __device__ inline long fidx(const Geo &g, int i, int j, int k) {
  return ((long)k * g.J + j) * g.I + i;
}
__device__ __forceinline__ int wrapm(int i, int n) {  // i in [-n, 2n)
  return i < 0 ? i + n : (i >= n ? i - n : i);
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
// Stencil of velocity component c (0 u, 1 v, 2 w) of a point, as eulr2lagr
// forms it (interp_spread.f90:60-131): tap (0,0,0) of the 3x3x3 block
// relative to the particle's reference floor in x and y and absolute in z
// (refz: the reference floor in z), and the component's FP32 delta weights.
// Along the component's own axis the staggered origin (ilows, jlows, klows:
// the nearest face, max(.,1) in z) and offsets; along the other axes the
// cell-centred origin (ilow, jlow, klow clamped to [1, K-2], quirk Q5).
__device__ __forceinline__ CompStencil make_cs(const PointRec &r, int c, int refz, int K) {
  const int dx = rec_dx(r.rel), dy = rec_dy(r.rel), nz = refz + rec_dz(r.rel);
  CompStencil s;
  float o;
  if (c == 0) {
    const int ux = r.fx >= 0.5f;
    s.b[0] = dx + ux - 2;
    o = r.fx + (float)(1 - ux);
#pragma unroll
    for (int m = 0; m < 3; ++m) s.w[m] = delta3f((float)m - o);
  } else {
    s.b[0] = dx - 1;
#pragma unroll
    for (int m = 0; m < 3; ++m) s.w[m] = delta3f(((float)m - 0.5f) - r.fx);
  }
  if (c == 1) {
    const int uy = r.fy >= 0.5f;
    s.b[1] = dy + uy - 2;
    o = r.fy + (float)(1 - uy);
#pragma unroll
    for (int m = 0; m < 3; ++m) s.w[3 + m] = delta3f((float)m - o);
  } else {
    s.b[1] = dy - 1;
#pragma unroll
    for (int m = 0; m < 3; ++m) s.w[3 + m] = delta3f(((float)m - 0.5f) - r.fy);
  }
  if (c == 2) {
    const int uz = r.fz > 0.5f || (r.fz == 0.5f && nz >= 0);
    const int klows = max(nz + uz - 1, 1);
    s.b[2] = klows;
    o = r.fz + (float)(nz - klows);
#pragma unroll
    for (int m = 0; m < 3; ++m) s.w[6 + m] = delta3f((float)m - o);
  } else {
    const int klow = max(min(nz, K - 2), 1);
    s.b[2] = klow;
    o = r.fz + (float)(nz - klow);
#pragma unroll
    for (int m = 0; m < 3; ++m) s.w[6 + m] = delta3f(((float)m - 0.5f) - o);
  }
  return s;
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

// Fortran NINT (half away from zero)
__device__ __forceinline__ int fnint(double x) { return (int)round(x); }

// launch helpers (the host side counts every launch)
#define IBM_CHECK_LAUNCH() cudaGetLastError()
