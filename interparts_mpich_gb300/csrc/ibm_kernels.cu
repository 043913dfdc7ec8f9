// ibm_kernels.cu -- multidirect immersed-boundary forcing on the Lagrangian
// points: eulr2lagr (interp_spread.f90:12-228), complagrforces /
// updtlagrforces (forcing.f90:9-391) and lagr2eulr (interp_spread.f90:230-474).
//
// Compiled without FMA contraction so the stencil indices, delta weights and
// point forces follow the reference roundings.
//
// Spreading is incremental: lagr2eulr rebuilds dudtf = dudtold + S(F) with
// the cumulative point force F every pass (zeroing and re-adding the whole
// field).  By linearity of S, dudtf after pass n equals the pass n-1 field
// plus S(F_n - F_{n-1}); the GPU adds only S(dF) over the points' footprint,
// so no full-field pass is needed.  The one plane that the reference never
// refreshes from dwdt, dwdtf(:,:,k1), is zeroed before the first spread of
// a substep so it carries S(F) exactly as in the reference.
#include <cuda_bf16.h>

#include "kernels.cuh"

namespace ibmk {

// stencil of one point (interp_spread.f90:76-130): same arithmetic as the
// reference, single rank (zstart = 1)
__global__ void __launch_bounds__(256) k_ibm_stencil(Geo g, PartGeo pg, IbmBuffers b) {
  const int n = pg.np * pg.nl;  // < 2^31 points (checked at create)
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
    const int p = t / pg.nl, l = t - p * pg.nl;
    if (l >= b.nla[p]) continue;
    const double xfp = b.xfp[t], yfp = b.yfp[t], zfp = b.zfp[t];
    double coorxfp = xfp * g.dxi - (double)((long)floor((xfp - 0.5 * g.dx) / g.lx) * g.I) - (1 - 1);
    double cooryfp = yfp * g.dyi - (double)((long)floor((yfp - 0.5 * g.dy) / g.ly) * g.J) - (1 - 1);
    double coorzfp = zfp * g.dzi;
    // Guard: a point outside the grid (or a non-finite position) would index
    // outside the arrays; flag it and park the point at a safe location.
    if (!(coorxfp >= 0. && coorxfp <= g.I + 1.) || !(cooryfp >= 0. && cooryfp <= g.J + 1.) ||
        !(coorzfp >= -1. && coorzfp <= g.K + 0.49)) {
      atomicExch(&b.err[2], 1);
      coorxfp = 1.; cooryfp = 1.; coorzfp = 1.5;
    }
    PointStencil s;
    s.ilows = fnint(coorxfp) - 1;
    s.jlows = fnint(cooryfp) - 1;
    s.klows = max(fnint(coorzfp) - 1, 1);
    s.ilow = (int)floor(coorxfp);
    s.jlow = (int)floor(cooryfp);
    s.klow = max(min((int)floor(coorzfp), g.K - 2), 1);
    for (int m = 0; m < 3; ++m) {
      s.phix[m] = delta3(1. * s.ilows + m - coorxfp);
      s.phiy[m] = delta3(1. * s.jlows + m - cooryfp);
      s.phiz[m] = delta3(1. * s.klows + m - coorzfp);
      s.phixh[m] = delta3(1. * s.ilow + m - .5 - coorxfp);
      s.phiyh[m] = delta3(1. * s.jlow + m - .5 - cooryfp);
      s.phizh[m] = delta3(1. * s.klow + m - .5 - coorzfp);
    }
    b.st[t] = s;
  }
}

template <typename T>
void launch_ibm_stencil(cudaStream_t s, const Geo &g, const PartGeo &pg, IbmBuffers b) {
  k_ibm_stencil<<<1216, 256, 0, s>>>(g, pg, b);
}
template void launch_ibm_stencil<double>(cudaStream_t, const Geo &, const PartGeo &, IbmBuffers);
template void launch_ibm_stencil<float>(cudaStream_t, const Geo &, const PartGeo &, IbmBuffers);

// interpolation of the three staggered components at point t
template <typename T>
__device__ __forceinline__ void interp_point(const Geo &g, const PointStencil &s, const T *__restrict__ fu,
                                             const T *__restrict__ fv, const T *__restrict__ fw, double &ou,
                                             double &ov, double &ow) {
  double au = 0., av = 0., aw = 0.;
  int ix[3], ixh[3], jy[3], jyh[3];
  for (int m = 0; m < 3; ++m) {
    ix[m] = wrapm(s.ilows + m - 1, g.I);
    ixh[m] = wrapm(s.ilow + m - 1, g.I);
    jy[m] = wrapm(s.jlows + m - 1, g.J);
    jyh[m] = wrapm(s.jlow + m - 1, g.J);
  }
  // separable form of the 27-tap sums of interp_spread.f90:132-154:
  // sum_k phiz_k sum_j phiy_j sum_i phix_i f_ijk (same terms, fewer FP64 ops)
  for (int k = 0; k < 3; ++k) {
    double su = 0., sv = 0., sw = 0.;
    for (int j = 0; j < 3; ++j) {
      double ru = 0., rv = 0., rw = 0.;
      for (int i = 0; i < 3; ++i) {
        ru += (double)fu[fidx(g, ix[i], jyh[j], s.klow + k)] * s.phix[i];
        rv += (double)fv[fidx(g, ixh[i], jy[j], s.klow + k)] * s.phixh[i];
        rw += (double)fw[fidx(g, ixh[i], jyh[j], s.klows + k)] * s.phixh[i];
      }
      su += ru * s.phiyh[j];
      sv += rv * s.phiy[j];
      sw += rw * s.phiyh[j];
    }
    au += su * s.phizh[k];
    av += sv * s.phizh[k];
    aw += sw * s.phiz[k];
  }
  ou = au; ov = av; ow = aw;
}

// eulr2lagr + complagrforces/updtlagrforces for one particle per block:
// interpolation, point force update and the per-particle force/torque sums.
template <typename T>
__global__ void __launch_bounds__(256) k_ibm_interp_force(Geo g, PartGeo pg, IbmBuffers b, const T *__restrict__ fu,
                                                          const T *__restrict__ fv, const T *__restrict__ fw,
                                                          double dti, int first) {
  const int p = blockIdx.x;
  const int nla = b.nla[p];
  const double *pf = b.pf;
  const double px = pf[PF_X * pg.np + p], py = pf[PF_Y * pg.np + p], pz = pf[PF_Z * pg.np + p];
  double sfx = 0, sfy = 0, sfz = 0, stx = 0, sty = 0, stz = 0;
  for (int l = threadIdx.x; l < nla; l += blockDim.x) {
    const long t = (long)p * pg.nl + l;
    const PointStencil s = b.st[t];
    double iu, iv, iw;
    interp_point<T>(g, s, fu, fv, fw, iu, iv, iw);
    b.dudtl[t] = iu; b.dvdtl[t] = iv; b.dwdtl[t] = iw;
    if (first < 0) continue;  // interpolation only (slip residual)
    double fx, fy, fz;
    if (first) {
      fx = (b.ul[t] - iu) * dti;
      fy = (b.vl[t] - iv) * dti;
      fz = (b.wl[t] - iw) * dti;
    } else {
      fx = b.fxl[t] + (b.ul[t] - iu) * dti;
      fy = b.fyl[t] + (b.vl[t] - iv) * dti;
      fz = b.fzl[t] + (b.wl[t] - iw) * dti;
    }
    b.fxl[t] = fx; b.fyl[t] = fy; b.fzl[t] = fz;
    const double rx = b.xfp[t] - px, ry = b.yfp[t] - py, rz = b.zfp[t] - pz;
    sfx += fx; sfy += fy; sfz += fz;
    stx = stx + ry * fz - rz * fy;
    sty = sty + rz * fx - rx * fz;
    stz = stz + rx * fy - ry * fx;
  }
  __shared__ double red[6][256];
  red[0][threadIdx.x] = sfx; red[1][threadIdx.x] = sfy; red[2][threadIdx.x] = sfz;
  red[3][threadIdx.x] = stx; red[4][threadIdx.x] = sty; red[5][threadIdx.x] = stz;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o)
      for (int q = 0; q < 6; ++q) red[q][threadIdx.x] += red[q][threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0 && first >= 0) {
    double *pw = b.pf;
    const double dV = pg.dVlagr;
    const double tx = red[3][0] * dV, ty = red[4][0] * dV, tz = red[5][0] * dV;
    pw[PF_FXLTOT * pg.np + p] = red[0][0] * dV;
    pw[PF_FYLTOT * pg.np + p] = red[1][0] * dV;
    pw[PF_FZLTOT * pg.np + p] = red[2][0] * dV;
    pw[PF_TQX * pg.np + p] = tx;
    pw[PF_TQY * pg.np + p] = ty;
    pw[PF_TQZ * pg.np + p] = tz;
    const double phi = pw[PF_PHI * pg.np + p];
    pw[PF_TQTHETA * pg.np + p] = (ty * cos(phi)) - (tx * sin(phi));
  }
}

template <typename T>
void launch_ibm_interp_force(cudaStream_t s, const Geo &g, const PartGeo &pg, IbmBuffers b, const T *fu, const T *fv,
                             const T *fw, double dt, int first) {
  if (pg.np == 0) return;
  k_ibm_interp_force<T><<<pg.np, 256, 0, s>>>(g, pg, b, fu, fv, fw, 1. / dt, first);
}
template void launch_ibm_interp_force<double>(cudaStream_t, const Geo &, const PartGeo &, IbmBuffers, const double *,
                                              const double *, const double *, double, int);
template void launch_ibm_interp_force<float>(cudaStream_t, const Geo &, const PartGeo &, IbmBuffers, const float *,
                                             const float *, const float *, double, int);

// lagr2eulr spreading: see k_ibm_spread_box below

template <typename T>
__global__ void k_zero_plane(Geo g, T *f, int k) {
  for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < g.plane; t += (long)gridDim.x * blockDim.x)
    f[(long)k * g.plane + t] = (T)0;
}
template <typename T>
void launch_zero_plane(cudaStream_t s, const Geo &g, T *f, int k) {
  k_zero_plane<T><<<152, 256, 0, s>>>(g, f, k);
}
template void launch_zero_plane<double>(cudaStream_t, const Geo &, double *, int);
template void launch_zero_plane<float>(cudaStream_t, const Geo &, float *, int);

// |U_l - u~_l| statistics (max, sum of squares, count) over all points,
// using the interpolation stored by the last pass.
__global__ void k_slip_residual(PartGeo pg, IbmBuffers b, double *out) {
  __shared__ double smax[256], ssum[256];
  double mx = 0., sm = 0.;
  const int n = pg.np * pg.nl;
  for (int t = threadIdx.x; t < n; t += blockDim.x) {
    const int p = t / pg.nl, l = t - p * pg.nl;
    if (l >= b.nla[p]) continue;
    const double ex = b.ul[t] - b.dudtl[t], ey = b.vl[t] - b.dvdtl[t], ez = b.wl[t] - b.dwdtl[t];
    const double r2 = ex * ex + ey * ey + ez * ez;
    mx = fmax(mx, sqrt(r2));
    sm += r2;
  }
  smax[threadIdx.x] = mx; ssum[threadIdx.x] = sm;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if (threadIdx.x < o) {
      smax[threadIdx.x] = fmax(smax[threadIdx.x], smax[threadIdx.x + o]);
      ssum[threadIdx.x] += ssum[threadIdx.x + o];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) { out[0] = smax[0]; out[1] = ssum[0]; }
}
void launch_slip_residual(cudaStream_t s, const PartGeo &pg, IbmBuffers b, double *out) {
  k_slip_residual<<<1, 256, 0, s>>>(pg, b, out);
}

// ---------------------------------------------------------------------------
// Mixed form.  Stencil origins come from the same FP64 coordinates; the
// delta weights, the 27-tap interpolation sums and the spreading run in FP32.
// The point forces F_l and the per-particle force/torque sums stay FP64.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_ibm_stencil_f(Geo g, PartGeo pg, IbmBuffers b) {
  const int n = pg.np * pg.nl;  // < 2^31 points (checked at create)
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
    const int p = t / pg.nl, l = t - p * pg.nl;
    if (l >= b.nla[p]) continue;
    const double xfp = b.xfp[t], yfp = b.yfp[t], zfp = b.zfp[t];
    double coorxfp = xfp * g.dxi - (double)((long)floor((xfp - 0.5 * g.dx) / g.lx) * g.I);
    double cooryfp = yfp * g.dyi - (double)((long)floor((yfp - 0.5 * g.dy) / g.ly) * g.J);
    double coorzfp = zfp * g.dzi;
    if (!(coorxfp >= 0. && coorxfp <= g.I + 1.) || !(cooryfp >= 0. && cooryfp <= g.J + 1.) ||
        !(coorzfp >= -1. && coorzfp <= g.K + 0.49)) {
      atomicExch(&b.err[2], 1);
      coorxfp = 1.; cooryfp = 1.; coorzfp = 1.5;
    }
    PointStencilF s;
    s.ilows = fnint(coorxfp) - 1;
    s.jlows = fnint(cooryfp) - 1;
    s.klows = max(fnint(coorzfp) - 1, 1);
    s.ilow = (int)floor(coorxfp);
    s.jlow = (int)floor(cooryfp);
    s.klow = max(min((int)floor(coorzfp), g.K - 2), 1);
    for (int m = 0; m < 3; ++m) {
      s.phix[m] = delta3f((float)(1. * s.ilows + m - coorxfp));
      s.phiy[m] = delta3f((float)(1. * s.jlows + m - cooryfp));
      s.phiz[m] = delta3f((float)(1. * s.klows + m - coorzfp));
      s.phixh[m] = delta3f((float)(1. * s.ilow + m - .5 - coorxfp));
      s.phiyh[m] = delta3f((float)(1. * s.jlow + m - .5 - cooryfp));
      s.phizh[m] = delta3f((float)(1. * s.klow + m - .5 - coorzfp));
    }
    b.st32[t] = s;
  }
}
void launch_ibm_stencil_f(cudaStream_t s, const Geo &g, const PartGeo &pg, IbmBuffers b) {
  k_ibm_stencil_f<<<1216, 256, 0, s>>>(g, pg, b);
}

__device__ __forceinline__ void interp_point_f(const Geo &g, const PointStencilF &s, const float *__restrict__ fu,
                                               const float *__restrict__ fv, const float *__restrict__ fw, float &ou,
                                               float &ov, float &ow) {
  float au = 0.f, av = 0.f, aw = 0.f;
  int ix[3], ixh[3], jy[3], jyh[3];
  for (int m = 0; m < 3; ++m) {
    ix[m] = wrapm(s.ilows + m - 1, g.I);
    ixh[m] = wrapm(s.ilow + m - 1, g.I);
    jy[m] = wrapm(s.jlows + m - 1, g.J);
    jyh[m] = wrapm(s.jlow + m - 1, g.J);
  }
  for (int k = 0; k < 3; ++k)
    for (int j = 0; j < 3; ++j) {
      const float wyz = s.phiyh[j] * s.phizh[k];
      const float wyz2 = s.phiy[j] * s.phizh[k];
      const float wyz3 = s.phiyh[j] * s.phiz[k];
      for (int i = 0; i < 3; ++i) {
        au += __ldg(&fu[fidx(g, ix[i], jyh[j], s.klow + k)]) * (s.phix[i] * wyz);
        av += __ldg(&fv[fidx(g, ixh[i], jy[j], s.klow + k)]) * (s.phixh[i] * wyz2);
        aw += __ldg(&fw[fidx(g, ixh[i], jyh[j], s.klows + k)]) * (s.phixh[i] * wyz3);
      }
    }
  ou = au; ov = av; ow = aw;
}

__global__ void __launch_bounds__(256) k_ibm_interp_force_f(Geo g, PartGeo pg, IbmBuffers b,
                                                            const float *__restrict__ fu, const float *__restrict__ fv,
                                                            const float *__restrict__ fw, double dti, int first,
                                                            const int *__restrict__ gate) {
  if (gate && *gate == 0) return;  // learned form: plain pass not needed
  const int p = blockIdx.x;
  const int nla = b.nla[p];
  const double *pf = b.pf;
  const double px = pf[PF_X * pg.np + p], py = pf[PF_Y * pg.np + p], pz = pf[PF_Z * pg.np + p];
  double sfx = 0, sfy = 0, sfz = 0, stx = 0, sty = 0, stz = 0;
  for (int l = threadIdx.x; l < nla; l += blockDim.x) {
    const long t = (long)p * pg.nl + l;
    const PointStencilF s = b.st32[t];
    float iu, iv, iw;
    interp_point_f(g, s, fu, fv, fw, iu, iv, iw);
    b.dudtl[t] = iu; b.dvdtl[t] = iv; b.dwdtl[t] = iw;
    if (first < 0) continue;
    double fx, fy, fz;
    if (first) {
      fx = (b.ul[t] - iu) * dti; fy = (b.vl[t] - iv) * dti; fz = (b.wl[t] - iw) * dti;
    } else {
      fx = b.fxl[t] + (b.ul[t] - iu) * dti; fy = b.fyl[t] + (b.vl[t] - iv) * dti; fz = b.fzl[t] + (b.wl[t] - iw) * dti;
    }
    b.fxl[t] = fx; b.fyl[t] = fy; b.fzl[t] = fz;
    const double rx = b.xfp[t] - px, ry = b.yfp[t] - py, rz = b.zfp[t] - pz;
    sfx += fx; sfy += fy; sfz += fz;
    stx = stx + ry * fz - rz * fy;
    sty = sty + rz * fx - rx * fz;
    stz = stz + rx * fy - ry * fx;
  }
  __shared__ double red[6][256];
  red[0][threadIdx.x] = sfx; red[1][threadIdx.x] = sfy; red[2][threadIdx.x] = sfz;
  red[3][threadIdx.x] = stx; red[4][threadIdx.x] = sty; red[5][threadIdx.x] = stz;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o)
      for (int q = 0; q < 6; ++q) red[q][threadIdx.x] += red[q][threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0 && first >= 0) {
    double *pw = b.pf;
    const double dV = pg.dVlagr;
    const double tx = red[3][0] * dV, ty = red[4][0] * dV, tz = red[5][0] * dV;
    pw[PF_FXLTOT * pg.np + p] = red[0][0] * dV;
    pw[PF_FYLTOT * pg.np + p] = red[1][0] * dV;
    pw[PF_FZLTOT * pg.np + p] = red[2][0] * dV;
    pw[PF_TQX * pg.np + p] = tx;
    pw[PF_TQY * pg.np + p] = ty;
    pw[PF_TQZ * pg.np + p] = tz;
    const double phi = pw[PF_PHI * pg.np + p];
    pw[PF_TQTHETA * pg.np + p] = (ty * cos(phi)) - (tx * sin(phi));
  }
}
void launch_ibm_interp_force_f(cudaStream_t s, const Geo &g, const PartGeo &pg, IbmBuffers b, const float *fu,
                               const float *fv, const float *fw, double dt, int first, const int *gate) {
  if (pg.np == 0) return;
  k_ibm_interp_force_f<<<pg.np, 256, 0, s>>>(g, pg, b, fu, fv, fw, 1. / dt, first, gate);
}

// ---------------------------------------------------------------------------
// lagr2eulr spreading of dF = (U_l - u~_l)/dt (or a given increment) with
// the terms of interp_spread.f90:329-355, F*coeff0*phix*phiy*phiz.  Block
// (particle, component): the particle's contributions are accumulated in a
// shared-memory box over the cells its stencils touch, then every touched
// cell is flushed to HBM with one atomic add (instead of one per tap).  In
// FP32 the box accumulation is compensated: the rounding error of each
// shared atomic add is recovered exactly by TwoSum from the value the atomic
// returned and accumulated in a second box, so the flushed hi+lo carries the
// particle's sum to about FP64 accuracy.  A box larger than SPREAD_BOX cells
// (spheres beyond ~D = 16 dx) falls back to direct atomics per tap.
// ---------------------------------------------------------------------------
constexpr int SPREAD_BOX = 8192;

template <typename T>
__device__ __forceinline__ void box_add(T *hi, T *lo, int c, T v) {
  if constexpr (sizeof(T) == 8) {
    atomicAdd(&hi[c], v);
    (void)lo;
  } else {
    const float old = atomicAdd(&hi[c], v);
    const float s = __fadd_rn(old, v);
    const float bb = __fsub_rn(s, old);
    const float e = __fadd_rn(__fsub_rn(old, __fsub_rn(s, bb)), __fsub_rn(v, bb));
    if (e != 0.f) atomicAdd(&lo[c], e);
  }
}

template <typename T, typename ST, typename W>
__global__ void __launch_bounds__(256) k_ibm_spread_box(Geo g, PartGeo pg, IbmBuffers b, const ST *__restrict__ st,
                                                        T *__restrict__ fu, T *__restrict__ fv, T *__restrict__ fw,
                                                        double dti, double coeff0, const float *__restrict__ dfin,
                                                        const int *__restrict__ gate) {
  if (gate && *gate == 0) return;  // learned form: plain pass not needed
  const int p = blockIdx.x, comp = blockIdx.y;
  const int nla = b.nla[p];
  if (nla <= 0) return;
  T *F = comp == 0 ? fu : (comp == 1 ? fv : fw);
  extern __shared__ __align__(16) unsigned char spread_sm[];
  T *hi = reinterpret_cast<T *>(spread_sm);
  T *lo = hi + SPREAD_BOX;  // FP32 only
  __shared__ int bmin[3], bmax[3];
  const long t0 = (long)p * pg.nl;
  const int refx = comp == 0 ? st[t0].ilows : st[t0].ilow;
  const int refy = comp == 1 ? st[t0].jlows : st[t0].jlow;
  const int hI = g.I / 2, hJ = g.J / 2;
  if (threadIdx.x < 3) { bmin[threadIdx.x] = 0x7fffffff; bmax[threadIdx.x] = -0x7fffffff; }
  __syncthreads();
  // box of the stencil origins, x/y relative to the first point (periodic)
  for (int l = threadIdx.x; l < nla; l += blockDim.x) {
    const ST &s = st[t0 + l];
    int rx = (comp == 0 ? s.ilows : s.ilow) - refx;
    int ry = (comp == 1 ? s.jlows : s.jlow) - refy;
    const int rz = comp == 2 ? s.klows : s.klow;
    rx = rx >= hI ? rx - g.I : (rx < -hI ? rx + g.I : rx);
    ry = ry >= hJ ? ry - g.J : (ry < -hJ ? ry + g.J : ry);
    atomicMin(&bmin[0], rx); atomicMax(&bmax[0], rx);
    atomicMin(&bmin[1], ry); atomicMax(&bmax[1], ry);
    atomicMin(&bmin[2], rz); atomicMax(&bmax[2], rz);
  }
  __syncthreads();
  const int nbx = bmax[0] - bmin[0] + 3, nby = bmax[1] - bmin[1] + 3, nbz = bmax[2] - bmin[2] + 3;
  const long nbox = (long)nbx * nby * nbz;
  const bool boxed = nbox <= SPREAD_BOX && nbx < hI && nby < hJ;
  if (boxed) {
    for (int c = threadIdx.x; c < nbox; c += blockDim.x) {
      hi[c] = (T)0;
      if constexpr (sizeof(T) == 4) lo[c] = 0.f;
    }
  }
  __syncthreads();
  for (int l = threadIdx.x; l < nla; l += blockDim.x) {
    const long t = t0 + l;
    const ST s = st[t];
    int bx, by, bz;
    W wx[3], wy[3], wz[3];
    double ucomp, icomp;
    if (comp == 0) {
      bx = s.ilows; by = s.jlow; bz = s.klow;
      for (int m = 0; m < 3; ++m) { wx[m] = s.phix[m]; wy[m] = s.phiyh[m]; wz[m] = s.phizh[m]; }
      ucomp = b.ul[t]; icomp = b.dudtl[t];
    } else if (comp == 1) {
      bx = s.ilow; by = s.jlows; bz = s.klow;
      for (int m = 0; m < 3; ++m) { wx[m] = s.phixh[m]; wy[m] = s.phiy[m]; wz[m] = s.phizh[m]; }
      ucomp = b.vl[t]; icomp = b.dvdtl[t];
    } else {
      bx = s.ilow; by = s.jlow; bz = s.klows;
      for (int m = 0; m < 3; ++m) { wx[m] = s.phixh[m]; wy[m] = s.phiyh[m]; wz[m] = s.phiz[m]; }
      ucomp = b.wl[t]; icomp = b.dwdtl[t];
    }
    // the (j,k) factor first, then the x weight (the reference's product order)
    T pre;
    if constexpr (sizeof(T) == 8) pre = (ucomp - icomp) * dti * coeff0;
    else pre = dfin ? (float)(dfin[3 * t + comp] * coeff0) : (float)((ucomp - icomp) * dti * coeff0);
    if (boxed) {
      int rx = bx - refx, ry = by - refy;
      rx = rx >= hI ? rx - g.I : (rx < -hI ? rx + g.I : rx);
      ry = ry >= hJ ? ry - g.J : (ry < -hJ ? ry + g.J : ry);
      const int cx = rx - bmin[0], cy = ry - bmin[1], cz = bz - bmin[2];
      for (int k = 0; k < 3; ++k)
        for (int j = 0; j < 3; ++j) {
          const T a = pre * wy[j] * wz[k];
          const int row = ((cz + k) * nby + (cy + j)) * nbx + cx;
          for (int i = 0; i < 3; ++i) box_add<T>(hi, lo, row + i, (T)(a * wx[i]));
        }
    } else {
      for (int k = 0; k < 3; ++k)
        for (int j = 0; j < 3; ++j) {
          const T a = pre * wy[j] * wz[k];
          const int y = wrapm(by + j - 1, g.J);
          for (int i = 0; i < 3; ++i) atomicAdd(&F[fidx(g, wrapm(bx + i - 1, g.I), y, bz + k)], (T)(a * wx[i]));
        }
    }
  }
  if (!boxed) return;
  __syncthreads();
  for (int c = threadIdx.x; c < nbox; c += blockDim.x) {
    T v = hi[c];
    if constexpr (sizeof(T) == 4) v += lo[c];
    if (v != (T)0) {
      const int cx = c % nbx, cy = (c / nbx) % nby, cz = c / (nbx * nby);
      const int x = wrapm(refx + bmin[0] - 1 + cx, g.I), y = wrapm(refy + bmin[1] - 1 + cy, g.J);
      atomicAdd(&F[fidx(g, x, y, bmin[2] + cz)], v);
    }
  }
}

template <typename T>
void launch_ibm_spread(cudaStream_t s, const Geo &g, const PartGeo &pg, IbmBuffers b, T *fu, T *fv, T *fw, double dt,
                       int first) {
  (void)first;
  if (pg.np == 0) return;
  const double coeff0 = (pg.dVlagr / pg.dVeul) * dt;
  k_ibm_spread_box<double, PointStencil, double><<<dim3(pg.np, 3), 256, SPREAD_BOX * sizeof(double), s>>>(
      g, pg, b, b.st, fu, fv, fw, 1. / dt, coeff0, nullptr, nullptr);
}
template void launch_ibm_spread<double>(cudaStream_t, const Geo &, const PartGeo &, IbmBuffers, double *, double *,
                                        double *, double, int);

void launch_ibm_spread_f(cudaStream_t s, const Geo &g, const PartGeo &pg, IbmBuffers b, float *fu, float *fv,
                         float *fw, double dt, const float *dfin, const int *gate) {
  if (pg.np == 0) return;
  const double coeff0 = (pg.dVlagr / pg.dVeul) * dt;
  k_ibm_spread_box<float, PointStencilF, float><<<dim3(pg.np, 3), 256, 2 * SPREAD_BOX * sizeof(float), s>>>(
      g, pg, b, b.st32, fu, fv, fw, 1. / dt, coeff0, dfin, gate);
}

int ibm_set_smem_limits() {
  cudaError_t e1 = cudaFuncSetAttribute(k_ibm_spread_box<double, PointStencil, double>,
                                        cudaFuncAttributeMaxDynamicSharedMemorySize, SPREAD_BOX * (int)sizeof(double));
  cudaError_t e2 = cudaFuncSetAttribute(k_ibm_spread_box<float, PointStencilF, float>,
                                        cudaFuncAttributeMaxDynamicSharedMemorySize, 2 * SPREAD_BOX * (int)sizeof(float));
  return (e1 == cudaSuccess && e2 == cudaSuccess) ? 0 : -1;
}

// ---------------------------------------------------------------------------
// Learned forcing (mixed form).  Features of each point after the first
// forcing pass:
//   [0:3]   slip U - u~ after pass 0      [3:6]  rigid-body velocity U
//   [6:9]   outward unit normal           [9:90] u, v, w at the 3x27 stencil
//                                                taps minus U (k,j,i order)
//   [90:93] pass-0 correction F0*dt       [93:96] centre delta weights
// X receives them standardised with (mu, isig) and rounded to BF16 for the
// network; a harvest selects every stride-th point and stores the raw FP32
// features with the point index, for the target written after the plain
// passes.  The interpolated velocity is stored in dudtl as eulr2lagr would.
// ---------------------------------------------------------------------------

__global__ void __launch_bounds__(256) k_ibm_features_f(Geo g, PartGeo pg, IbmBuffers b, const float *__restrict__ fu,
                                                        const float *__restrict__ fv, const float *__restrict__ fw,
                                                        double dt, const float *__restrict__ mu,
                                                        const float *__restrict__ isig,
                                                        __nv_bfloat16 *__restrict__ X, HarvestArgs H) {
  const int n = pg.np * pg.nl;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
    const int p = t / pg.nl, l = t - p * pg.nl;
    if (l >= b.nla[p]) {
      if (X)
        for (int q = 0; q < 96; q += 2)
          *reinterpret_cast<__nv_bfloat162 *>(&X[(long)t * 96 + q]) = __floats2bfloat162_rn(0.f, 0.f);
      continue;
    }
    const PointStencilF s = b.st32[t];
    int ix[3], ixh[3], jy[3], jyh[3];
    for (int m = 0; m < 3; ++m) {
      ix[m] = wrapm(s.ilows + m - 1, g.I);
      ixh[m] = wrapm(s.ilow + m - 1, g.I);
      jy[m] = wrapm(s.jlows + m - 1, g.J);
      jyh[m] = wrapm(s.jlow + m - 1, g.J);
    }
    const float Ux = (float)b.ul[t], Uy = (float)b.vl[t], Uz = (float)b.wl[t];
    float f[96];
    float au = 0.f, av = 0.f, aw = 0.f;
    int q = 0;
#pragma unroll
    for (int k = 0; k < 3; ++k)
#pragma unroll
      for (int j = 0; j < 3; ++j)
#pragma unroll
        for (int i = 0; i < 3; ++i, ++q) {
          const float tu = __ldg(&fu[fidx(g, ix[i], jyh[j], s.klow + k)]);
          const float tv = __ldg(&fv[fidx(g, ixh[i], jy[j], s.klow + k)]);
          const float tw = __ldg(&fw[fidx(g, ixh[i], jyh[j], s.klows + k)]);
          au += tu * (s.phix[i] * (s.phiyh[j] * s.phizh[k]));
          av += tv * (s.phixh[i] * (s.phiy[j] * s.phizh[k]));
          aw += tw * (s.phixh[i] * (s.phiyh[j] * s.phiz[k]));
          f[9 + q] = tu - Ux;
          f[36 + q] = tv - Uy;
          f[63 + q] = tw - Uz;
        }
    b.dudtl[t] = au; b.dvdtl[t] = av; b.dwdtl[t] = aw;
    const double px = b.pf[PF_X * pg.np + p], py = b.pf[PF_Y * pg.np + p], pz = b.pf[PF_Z * pg.np + p];
    const float inv_r = (float)(1. / pg.radfp);
    f[0] = Ux - au; f[1] = Uy - av; f[2] = Uz - aw;
    f[3] = Ux; f[4] = Uy; f[5] = Uz;
    f[6] = (float)(b.xfp[t] - px) * inv_r; f[7] = (float)(b.yfp[t] - py) * inv_r; f[8] = (float)(b.zfp[t] - pz) * inv_r;
    f[90] = (float)(b.fxl[t] * dt); f[91] = (float)(b.fyl[t] * dt); f[92] = (float)(b.fzl[t] * dt);
    f[93] = s.phix[1]; f[94] = s.phiy[1]; f[95] = s.phiz[1];
    if (X) {
#pragma unroll
      for (int c = 0; c < 96; c += 2)
        *reinterpret_cast<__nv_bfloat162 *>(&X[(long)t * 96 + c]) =
            __floats2bfloat162_rn((f[c] - mu[c]) * isig[c], (f[c + 1] - mu[c + 1]) * isig[c + 1]);
    }
    if (H.feat && (t + H.phase) % H.stride == 0) {
      const int h = atomicAdd(&H.count[0], 1);
      if (h < H.cap) {
#pragma unroll
        for (int c = 0; c < 96; ++c) H.feat[(long)h * 96 + c] = f[c];
        H.pidx[h] = t;
      }
    }
  }
}
void launch_ibm_features_f(cudaStream_t s, const Geo &g, const PartGeo &pg, IbmBuffers b, const float *fu,
                           const float *fv, const float *fw, double dt, const float *mu, const float *isig,
                           __nv_bfloat16 *X, const HarvestArgs &H) {
  if (pg.np == 0) return;
  k_ibm_features_f<<<1216, 256, 0, s>>>(g, pg, b, fu, fv, fw, dt, mu, isig, X, H);
}

// targets of the slots reserved since the last call: (F_final - F0) * dt, the
// correction the plain passes 1.. added after pass 0
__global__ void k_ibm_harvest_targets(IbmBuffers b, HarvestArgs H, double dt) {
  const int lo = H.count[1], hi = min(H.count[0], H.cap);
  for (int h = lo + blockIdx.x * blockDim.x + threadIdx.x; h < hi; h += gridDim.x * blockDim.x) {
    const int t = H.pidx[h];
    H.targ[3 * (long)h] = (float)(b.fxl[t] * dt) - H.feat[(long)h * 96 + 90];
    H.targ[3 * (long)h + 1] = (float)(b.fyl[t] * dt) - H.feat[(long)h * 96 + 91];
    H.targ[3 * (long)h + 2] = (float)(b.fzl[t] * dt) - H.feat[(long)h * 96 + 92];
  }
}
__global__ void k_ibm_harvest_close(HarvestArgs H) {
  if (threadIdx.x == 0 && blockIdx.x == 0) H.count[1] = min(H.count[0], H.cap);
}
void launch_ibm_harvest_targets(cudaStream_t s, IbmBuffers b, const HarvestArgs &H, double dt) {
  k_ibm_harvest_targets<<<152, 256, 0, s>>>(b, H, dt);
  k_ibm_harvest_close<<<1, 32, 0, s>>>(H);
}

// learned update: dF = Y/dt per point, F += dF, and the per-particle force and
// torque sums of the updated F (as updtlagrforces computes them)
__global__ void __launch_bounds__(256) k_ibm_learned_apply(PartGeo pg, IbmBuffers b, const float *__restrict__ Y,
                                                           const float *__restrict__ tmu,
                                                           const float *__restrict__ tsig, double dti,
                                                           float *__restrict__ dF) {
  const int p = blockIdx.x;
  const int nla = b.nla[p];
  const double px = b.pf[PF_X * pg.np + p], py = b.pf[PF_Y * pg.np + p], pz = b.pf[PF_Z * pg.np + p];
  double sfx = 0, sfy = 0, sfz = 0, stx = 0, sty = 0, stz = 0;
  for (int l = threadIdx.x; l < nla; l += blockDim.x) {
    const long t = (long)p * pg.nl + l;
    const double dx = (double)(Y[3 * t] * tsig[0] + tmu[0]) * dti;
    const double dy = (double)(Y[3 * t + 1] * tsig[1] + tmu[1]) * dti;
    const double dz = (double)(Y[3 * t + 2] * tsig[2] + tmu[2]) * dti;
    dF[3 * t] = (float)dx; dF[3 * t + 1] = (float)dy; dF[3 * t + 2] = (float)dz;
    const double fx = b.fxl[t] + dx, fy = b.fyl[t] + dy, fz = b.fzl[t] + dz;
    b.fxl[t] = fx; b.fyl[t] = fy; b.fzl[t] = fz;
    const double rx = b.xfp[t] - px, ry = b.yfp[t] - py, rz = b.zfp[t] - pz;
    sfx += fx; sfy += fy; sfz += fz;
    stx = stx + ry * fz - rz * fy;
    sty = sty + rz * fx - rx * fz;
    stz = stz + rx * fy - ry * fx;
  }
  __shared__ double red[6][256];
  red[0][threadIdx.x] = sfx; red[1][threadIdx.x] = sfy; red[2][threadIdx.x] = sfz;
  red[3][threadIdx.x] = stx; red[4][threadIdx.x] = sty; red[5][threadIdx.x] = stz;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o)
      for (int q = 0; q < 6; ++q) red[q][threadIdx.x] += red[q][threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    double *pw = b.pf;
    const double dV = pg.dVlagr;
    const double tx = red[3][0] * dV, ty = red[4][0] * dV, tz = red[5][0] * dV;
    pw[PF_FXLTOT * pg.np + p] = red[0][0] * dV;
    pw[PF_FYLTOT * pg.np + p] = red[1][0] * dV;
    pw[PF_FZLTOT * pg.np + p] = red[2][0] * dV;
    pw[PF_TQX * pg.np + p] = tx;
    pw[PF_TQY * pg.np + p] = ty;
    pw[PF_TQZ * pg.np + p] = tz;
    const double phi = pw[PF_PHI * pg.np + p];
    pw[PF_TQTHETA * pg.np + p] = (ty * cos(phi)) - (tx * sin(phi));
  }
}
void launch_ibm_learned_apply(cudaStream_t s, const PartGeo &pg, IbmBuffers b, const float *Y, const float *tmu,
                              const float *tsig, double dt, float *dF) {
  if (pg.np == 0) return;
  k_ibm_learned_apply<<<pg.np, 256, 0, s>>>(pg, b, Y, tmu, tsig, 1. / dt, dF);
}

// residual gate: sum of |U - u~|^2 over the points (block partials), then
// gate = (rms > threshold); counts fallbacks
__global__ void k_ibm_res_partial(PartGeo pg, IbmBuffers b, double *__restrict__ part) {
  __shared__ double sm[256];
  double acc = 0.;
  const int n = pg.np * pg.nl;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
    const int p = t / pg.nl, l = t - p * pg.nl;
    if (l >= b.nla[p]) continue;
    const double ex = b.ul[t] - b.dudtl[t], ey = b.vl[t] - b.dvdtl[t], ez = b.wl[t] - b.dwdtl[t];
    acc += ex * ex + ey * ey + ez * ez;
  }
  sm[threadIdx.x] = acc;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if (threadIdx.x < o) sm[threadIdx.x] += sm[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = sm[0];
}
// LearnState (device): [0] rms of the last learned substep, [1] sum and
// [2] count of the plain passes' rms, [3] fallback ratio, [4] fallbacks,
// [5] learned substeps; gate = 1 runs the plain passes after the inference
__global__ void k_ibm_res_gate(int nb, const double *__restrict__ part, long npts, double *ls, int *gate, int plain) {
  if (threadIdx.x != 0) return;
  double s = 0.;
  for (int q = 0; q < nb; ++q) s += part[q];
  const double rms = npts ? sqrt(s / (double)npts) : 0.;
  if (plain) {  // residual of the plain passes: the reference the learned one is held to
    ls[1] += rms;
    ls[2] += 1.;
    return;
  }
  ls[0] = rms;
  ls[5] += 1.;
  const double ref = ls[2] > 0. ? ls[1] / ls[2] : 0.;
  const int g = (!(rms <= ls[3] * ref)) ? 1 : 0;  // NaN falls back too
  *gate = g;
  if (g) ls[4] += 1.;
}
void launch_ibm_residual_gate(cudaStream_t s, const PartGeo &pg, IbmBuffers b, double *scratch, long npts,
                              double *ls, int *gate, int plain) {
  const int nb = 152;
  k_ibm_res_partial<<<nb, 256, 0, s>>>(pg, b, scratch);
  k_ibm_res_gate<<<1, 32, 0, s>>>(nb, scratch, npts, ls, gate, plain);
}


}  // namespace ibmk
