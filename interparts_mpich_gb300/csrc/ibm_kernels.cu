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


// ---------------------------------------------------------------------------
// Shared-memory field boxes of one particle.  Per component the box covers
// the cells of the 27-tap stencils of the particle's points, x/y indices
// relative to the first point (periodic wrap), z absolute; box cell
// (cx, cy, cz) <-> tap (bx - 1 + i, by - 1 + j, bz + k) of a point with
// relative origin (rx, ry, bz) at cx = rx - b0 + i, cy = ry - b1 + j,
// cz = bz - b2 + k.  bg[c] = {refx, refy, b0, b1, b2, nbx, nby, nbz}.
// ---------------------------------------------------------------------------
__device__ __forceinline__ int relwrap(int d, int n) {
  const int h = n / 2;
  return d >= h ? d - n : (d < -h ? d + n : d);
}
template <typename ST>
__device__ __forceinline__ void comp_origin(const ST &s, int c, int &bx, int &by, int &bz) {
  bx = c == 0 ? s.ilows : s.ilow;
  by = c == 1 ? s.jlows : s.jlow;
  bz = c == 2 ? s.klows : s.klow;
}
// block-wide; returns the same value in every thread: true when all three
// boxes fit `cap` cells (and are not wider than half the periodic domain)
template <typename T, typename ST>
__device__ bool build_boxes(const Geo &g, const ST *__restrict__ st, long t0, int nla, const T *__restrict__ fu,
                            const T *__restrict__ fv, const T *__restrict__ fw, T *box, int cap, int (*bg)[8],
                            int (*bmax)[3]) {
  if (threadIdx.x < 3) {
    const int c = threadIdx.x;
    int bx, by, bz;
    comp_origin(st[t0], c, bx, by, bz);
    bg[c][0] = bx; bg[c][1] = by;
    bg[c][2] = bg[c][3] = bg[c][4] = 0x7fffffff;
    bmax[c][0] = bmax[c][1] = bmax[c][2] = -0x7fffffff;
  }
  __syncthreads();
  // per-thread extremes, then one shared atomic per warp and bound
  int lo[3][3], hi[3][3];
  for (int c = 0; c < 3; ++c)
    for (int d = 0; d < 3; ++d) { lo[c][d] = 0x7fffffff; hi[c][d] = -0x7fffffff; }
  for (int l = threadIdx.x; l < nla; l += blockDim.x) {
    const ST &s = st[t0 + l];
    for (int c = 0; c < 3; ++c) {
      int bx, by, bz;
      comp_origin(s, c, bx, by, bz);
      const int r[3] = {relwrap(bx - bg[c][0], g.I), relwrap(by - bg[c][1], g.J), bz};
      for (int d = 0; d < 3; ++d) { lo[c][d] = min(lo[c][d], r[d]); hi[c][d] = max(hi[c][d], r[d]); }
    }
  }
  for (int c = 0; c < 3; ++c)
    for (int d = 0; d < 3; ++d) {
      const int wl = __reduce_min_sync(0xffffffffu, lo[c][d]), wh = __reduce_max_sync(0xffffffffu, hi[c][d]);
      if ((threadIdx.x & 31) == 0) { atomicMin(&bg[c][2 + d], wl); atomicMax(&bmax[c][d], wh); }
    }
  __syncthreads();
  if (threadIdx.x < 3) {
    const int c = threadIdx.x;
    bg[c][5] = bmax[c][0] - bg[c][2] + 3;
    bg[c][6] = bmax[c][1] - bg[c][3] + 3;
    bg[c][7] = bmax[c][2] - bg[c][4] + 3;
  }
  __syncthreads();
  bool ok = true;
  for (int c = 0; c < 3; ++c)
    ok = ok && (long)bg[c][5] * bg[c][6] * bg[c][7] <= cap && bg[c][5] < g.I / 2 && bg[c][6] < g.J / 2;
  if (!ok) return false;
  for (int c = 0; c < 3; ++c) {
    const T *F = c == 0 ? fu : (c == 1 ? fv : fw);
    const int nbx = bg[c][5], nby = bg[c][6], nxy = nbx * nby, nbox = nxy * bg[c][7];
    const int x0 = bg[c][0] + bg[c][2] - 1, y0 = bg[c][1] + bg[c][3] - 1, z0 = bg[c][4];
    for (int q = threadIdx.x; q < nbox; q += blockDim.x) {
      const int cz = q / nxy, r = q - cz * nxy, cy = r / nbx, cx = r - cy * nbx;
      box[c * cap + q] = __ldg(&F[fidx(g, wrapm(x0 + cx, g.I), wrapm(y0 + cy, g.J), z0 + cz)]);
    }
  }
  __syncthreads();
  return true;
}
// offset of tap (0,0,0) of component c for a point, and the box strides
template <typename ST>
__device__ __forceinline__ int box_origin(const Geo &g, const ST &s, int c, const int (*bg)[8]) {
  int bx, by, bz;
  comp_origin(s, c, bx, by, bz);
  const int cx = relwrap(bx - bg[c][0], g.I) - bg[c][2], cy = relwrap(by - bg[c][1], g.J) - bg[c][3];
  return ((bz - bg[c][4]) * bg[c][6] + cy) * bg[c][5] + cx;
}
constexpr int INTERP_BOX = 8192;  // cells per component box

// interpolation of the three staggered components at point t
// separable form of the 27-tap sums of interp_spread.f90:132-154:
// sum_k phiz_k sum_j phiy_j sum_i phix_i f_ijk (same terms, fewer FP64 ops)
template <typename FU, typename FV, typename FW>
__device__ __forceinline__ void interp_sep(const PointStencil &s, FU U, FV V, FW W, double &ou, double &ov,
                                           double &ow) {
  double au = 0., av = 0., aw = 0.;
  for (int k = 0; k < 3; ++k) {
    double su = 0., sv = 0., sw = 0.;
    for (int j = 0; j < 3; ++j) {
      double ru = 0., rv = 0., rw = 0.;
      for (int i = 0; i < 3; ++i) {
        ru += U(i, j, k) * s.phix[i];
        rv += V(i, j, k) * s.phixh[i];
        rw += W(i, j, k) * s.phixh[i];
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

template <typename T>
__device__ __forceinline__ void interp_point(const Geo &g, const PointStencil &s, const T *__restrict__ fu,
                                             const T *__restrict__ fv, const T *__restrict__ fw, double &ou,
                                             double &ov, double &ow) {
  int ix[3], ixh[3], jy[3], jyh[3];
  for (int m = 0; m < 3; ++m) {
    ix[m] = wrapm(s.ilows + m - 1, g.I);
    ixh[m] = wrapm(s.ilow + m - 1, g.I);
    jy[m] = wrapm(s.jlows + m - 1, g.J);
    jyh[m] = wrapm(s.jlow + m - 1, g.J);
  }
  interp_sep(s, [&](int i, int j, int k) { return (double)fu[fidx(g, ix[i], jyh[j], s.klow + k)]; },
             [&](int i, int j, int k) { return (double)fv[fidx(g, ixh[i], jy[j], s.klow + k)]; },
             [&](int i, int j, int k) { return (double)fw[fidx(g, ixh[i], jyh[j], s.klows + k)]; }, ou, ov, ow);
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

// lagr2eulr increment: spread dF = (U_l - u~_l)/dt with the terms of
// interp_spread.f90:329-355, F*coeff0*phix*phiy*phiz, the (j,k) factor
// formed once per row of three taps
template <typename T>
__global__ void __launch_bounds__(256) k_ibm_spread(Geo g, PartGeo pg, IbmBuffers b, T *__restrict__ fu,
                                                    T *__restrict__ fv, T *__restrict__ fw, double dti,
                                                    double coeff0) {
  const int n = pg.np * pg.nl;  // < 2^31 points (checked at create)
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
    const int p = t / pg.nl, l = t - p * pg.nl;
    if (l >= b.nla[p]) continue;
    const PointStencil s = b.st[t];
    const double dfx = (b.ul[t] - b.dudtl[t]) * dti;
    const double dfy = (b.vl[t] - b.dvdtl[t]) * dti;
    const double dfz = (b.wl[t] - b.dwdtl[t]) * dti;
    int ix[3], ixh[3], jy[3], jyh[3];
    for (int m = 0; m < 3; ++m) {
      ix[m] = wrapm(s.ilows + m - 1, g.I);
      ixh[m] = wrapm(s.ilow + m - 1, g.I);
      jy[m] = wrapm(s.jlows + m - 1, g.J);
      jyh[m] = wrapm(s.jlow + m - 1, g.J);
    }
    for (int k = 0; k < 3; ++k)
      for (int j = 0; j < 3; ++j) {
        const double a = dfx * coeff0 * s.phiyh[j] * s.phizh[k];
        const double bb = dfy * coeff0 * s.phiy[j] * s.phizh[k];
        const double cc = dfz * coeff0 * s.phiyh[j] * s.phiz[k];
        for (int i = 0; i < 3; ++i) {
          atomicAdd(&fu[fidx(g, ix[i], jyh[j], s.klow + k)], (T)(a * s.phix[i]));
          atomicAdd(&fv[fidx(g, ixh[i], jy[j], s.klow + k)], (T)(bb * s.phixh[i]));
          atomicAdd(&fw[fidx(g, ixh[i], jyh[j], s.klows + k)], (T)(cc * s.phixh[i]));
        }
      }
  }
}


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
    // periodic image by a multiply: any image whose coordinate stays in
    // [0, I+1] addresses the same (wrapped) cells with the same weights
    const double inv_lx = 1. / g.lx, inv_ly = 1. / g.ly;
    double coorxfp = xfp * g.dxi - (double)((long)floor((xfp - 0.5 * g.dx) * inv_lx) * g.I);
    double cooryfp = yfp * g.dyi - (double)((long)floor((yfp - 0.5 * g.dy) * inv_ly) * g.J);
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
    // offsets of the point from the stencil origins (FP64, exact integer
    // parts), the 3-tap arguments then in FP32
    const float ox = (float)(coorxfp - s.ilows), oy = (float)(cooryfp - s.jlows), oz = (float)(coorzfp - s.klows);
    const float hx = (float)(coorxfp - s.ilow), hy = (float)(cooryfp - s.jlow), hz = (float)(coorzfp - s.klow);
    for (int m = 0; m < 3; ++m) {
      s.phix[m] = delta3f((float)m - ox);
      s.phiy[m] = delta3f((float)m - oy);
      s.phiz[m] = delta3f((float)m - oz);
      s.phixh[m] = delta3f(((float)m - 0.5f) - hx);
      s.phiyh[m] = delta3f(((float)m - 0.5f) - hy);
      s.phizh[m] = delta3f(((float)m - 0.5f) - hz);
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

// eulr2lagr + complagrforces/updtlagrforces, mixed form.  Block (particle,
// component): the component's field box in shared memory (32 KB), the 27-tap
// interpolation of that component for every point (FP32, the same terms in
// the same order as interp_point_f), the FP64 point-force update of that
// component and its partial sums: sum F_c and the two lever-arm moments of
// F_c that enter the torque.  k_ibm_force_sums combines the three components.
__device__ bool build_box1(const Geo &g, const PointStencilF *__restrict__ st, long t0, int nla, int c,
                           const float *__restrict__ F, float *box, int cap, int *bg, int *bmx) {
  if (threadIdx.x == 0) {
    int bx, by, bz;
    comp_origin(st[t0], c, bx, by, bz);
    bg[0] = bx; bg[1] = by;
    bg[2] = bg[3] = bg[4] = 0x7fffffff;
    bmx[0] = bmx[1] = bmx[2] = -0x7fffffff;
  }
  __syncthreads();
  int lo[3] = {0x7fffffff, 0x7fffffff, 0x7fffffff}, hi[3] = {-0x7fffffff, -0x7fffffff, -0x7fffffff};
  for (int l = threadIdx.x; l < nla; l += blockDim.x) {
    int bx, by, bz;
    comp_origin(st[t0 + l], c, bx, by, bz);
    const int r[3] = {relwrap(bx - bg[0], g.I), relwrap(by - bg[1], g.J), bz};
    for (int d = 0; d < 3; ++d) { lo[d] = min(lo[d], r[d]); hi[d] = max(hi[d], r[d]); }
  }
  for (int d = 0; d < 3; ++d) {
    const int wl = __reduce_min_sync(0xffffffffu, lo[d]), wh = __reduce_max_sync(0xffffffffu, hi[d]);
    if ((threadIdx.x & 31) == 0) { atomicMin(&bg[2 + d], wl); atomicMax(&bmx[d], wh); }
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    bg[5] = bmx[0] - bg[2] + 3;
    bg[6] = bmx[1] - bg[3] + 3;
    bg[7] = bmx[2] - bg[4] + 3;
  }
  __syncthreads();
  const bool ok = (long)bg[5] * bg[6] * bg[7] <= cap && bg[5] < g.I / 2 && bg[6] < g.J / 2;
  if (!ok) return false;
  const int nbx = bg[5], nby = bg[6], nxy = nbx * nby, nbox = nxy * bg[7];
  const int x0 = bg[0] + bg[2] - 1, y0 = bg[1] + bg[3] - 1, z0 = bg[4];
  for (int q = threadIdx.x; q < nbox; q += blockDim.x) {
    const int cz = q / nxy, r = q - cz * nxy, cy = r / nbx, cx = r - cy * nbx;
    box[q] = __ldg(&F[fidx(g, wrapm(x0 + cx, g.I), wrapm(y0 + cy, g.J), z0 + cz)]);
  }
  __syncthreads();
  return true;
}

__global__ void __launch_bounds__(256) k_ibm_interp_comp_f(Geo g, PartGeo pg, IbmBuffers b,
                                                           const float *__restrict__ fu, const float *__restrict__ fv,
                                                           const float *__restrict__ fw, double dti, int first,
                                                           const int *__restrict__ gate) {
  if (gate && *gate == 0) return;  // learned form: plain pass not needed
  const int p = blockIdx.x, c = blockIdx.y;
  const int nla = b.nla[p];
  const long t0 = (long)p * pg.nl;
  const float *F = c == 0 ? fu : (c == 1 ? fv : fw);
  extern __shared__ __align__(16) unsigned char ibox_sm[];
  float *box = reinterpret_cast<float *>(ibox_sm);
  __shared__ int bg[8], bmx[3];
  const bool boxed = nla > 0 && build_box1(g, b.st32, t0, nla, c, F, box, INTERP_BOX, bg, bmx);
  double *dud = c == 0 ? b.dudtl : (c == 1 ? b.dvdtl : b.dwdtl);
  const double *U = c == 0 ? b.ul : (c == 1 ? b.vl : b.wl);
  double *Fl = c == 0 ? b.fxl : (c == 1 ? b.fyl : b.fzl);
  const double *pf = b.pf;
  const double px = pf[PF_X * pg.np + p], py = pf[PF_Y * pg.np + p], pz = pf[PF_Z * pg.np + p];
  double sF = 0., sa = 0., sb = 0.;
  for (int l = threadIdx.x; l < nla; l += blockDim.x) {
    const long t = t0 + l;
    const PointStencilF s = b.st32[t];
    float wx[3], wy[3], wz[3];
    if (c == 0) { for (int m = 0; m < 3; ++m) { wx[m] = s.phix[m]; wy[m] = s.phiyh[m]; wz[m] = s.phizh[m]; } }
    else if (c == 1) { for (int m = 0; m < 3; ++m) { wx[m] = s.phixh[m]; wy[m] = s.phiy[m]; wz[m] = s.phizh[m]; } }
    else { for (int m = 0; m < 3; ++m) { wx[m] = s.phixh[m]; wy[m] = s.phiyh[m]; wz[m] = s.phiz[m]; } }
    float acc = 0.f;
    if (boxed) {
      int bx, by, bz;
      comp_origin(s, c, bx, by, bz);
      const float *B = box + ((bz - bg[4]) * bg[6] + relwrap(by - bg[1], g.J) - bg[3]) * bg[5] +
                       (relwrap(bx - bg[0], g.I) - bg[2]);
      const int ys = bg[5], zs = bg[5] * bg[6];
#pragma unroll
      for (int k = 0; k < 3; ++k)
#pragma unroll
        for (int j = 0; j < 3; ++j) {
          const float wyz = wy[j] * wz[k];
#pragma unroll
          for (int i = 0; i < 3; ++i) acc += B[i + j * ys + k * zs] * (wx[i] * wyz);
        }
    } else {
      int bx, by, bz;
      comp_origin(s, c, bx, by, bz);
      for (int k = 0; k < 3; ++k)
        for (int j = 0; j < 3; ++j) {
          const float wyz = wy[j] * wz[k];
          const int y = wrapm(by + j - 1, g.J);
          for (int i = 0; i < 3; ++i) acc += __ldg(&F[fidx(g, wrapm(bx + i - 1, g.I), y, bz + k)]) * (wx[i] * wyz);
        }
    }
    dud[t] = acc;
    if (first < 0) continue;  // interpolation only (slip residual)
    const double f = first ? (U[t] - acc) * dti : Fl[t] + (U[t] - acc) * dti;
    Fl[t] = f;
    // lever arms of the torque terms of this component:
    // c=0: (rz, ry), c=1: (rz, rx), c=2: (ry, rx)
    const double la = c == 2 ? b.yfp[t] - py : b.zfp[t] - pz;
    const double lb = c == 0 ? b.yfp[t] - py : b.xfp[t] - px;
    sF += f;
    sa += la * f;
    sb += lb * f;
  }
  if (first < 0) return;
  __shared__ double red[3][256];
  red[0][threadIdx.x] = sF; red[1][threadIdx.x] = sa; red[2][threadIdx.x] = sb;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o)
      for (int q = 0; q < 3; ++q) red[q][threadIdx.x] += red[q][threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x < 3) b.psum[((long)p * 3 + c) * 3 + threadIdx.x] = red[threadIdx.x][0];
}
// per-particle force and torque of updtlagrforces from the component sums
__global__ void k_ibm_force_sums(PartGeo pg, IbmBuffers b, const int *__restrict__ gate) {
  if (gate && *gate == 0) return;
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= pg.np) return;
  const double *s = b.psum + (long)p * 9;
  const double dV = pg.dVlagr;
  double *pw = b.pf;
  const double tx = (s[7] - s[4]) * dV, ty = (s[1] - s[8]) * dV, tz = (s[5] - s[2]) * dV;
  pw[PF_FXLTOT * pg.np + p] = s[0] * dV;
  pw[PF_FYLTOT * pg.np + p] = s[3] * dV;
  pw[PF_FZLTOT * pg.np + p] = s[6] * dV;
  pw[PF_TQX * pg.np + p] = tx;
  pw[PF_TQY * pg.np + p] = ty;
  pw[PF_TQZ * pg.np + p] = tz;
  const double phi = pw[PF_PHI * pg.np + p];
  pw[PF_TQTHETA * pg.np + p] = (ty * cos(phi)) - (tx * sin(phi));
}
int launch_ibm_interp_force_f(cudaStream_t s, const Geo &g, const PartGeo &pg, IbmBuffers b, const float *fu,
                              const float *fv, const float *fw, double dt, int first, const int *gate) {
  if (pg.np == 0) return 0;
  k_ibm_interp_comp_f<<<dim3(pg.np, 3), 256, INTERP_BOX * sizeof(float), s>>>(g, pg, b, fu, fv, fw, 1. / dt, first,
                                                                              gate);
  if (first < 0) return 1;
  k_ibm_force_sums<<<(pg.np + 127) / 128, 128, 0, s>>>(pg, b, gate);
  return 2;
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
__global__ void __launch_bounds__(384) k_ibm_spread_box(Geo g, PartGeo pg, IbmBuffers b, const ST *__restrict__ st,
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
  int elo[3] = {0x7fffffff, 0x7fffffff, 0x7fffffff}, ehi[3] = {-0x7fffffff, -0x7fffffff, -0x7fffffff};
  for (int l = threadIdx.x; l < nla; l += blockDim.x) {
    const ST &s = st[t0 + l];
    int rx = (comp == 0 ? s.ilows : s.ilow) - refx;
    int ry = (comp == 1 ? s.jlows : s.jlow) - refy;
    const int rz = comp == 2 ? s.klows : s.klow;
    rx = rx >= hI ? rx - g.I : (rx < -hI ? rx + g.I : rx);
    ry = ry >= hJ ? ry - g.J : (ry < -hJ ? ry + g.J : ry);
    elo[0] = min(elo[0], rx); ehi[0] = max(ehi[0], rx);
    elo[1] = min(elo[1], ry); ehi[1] = max(ehi[1], ry);
    elo[2] = min(elo[2], rz); ehi[2] = max(ehi[2], rz);
  }
  for (int d = 0; d < 3; ++d) {
    const int wl = __reduce_min_sync(0xffffffffu, elo[d]), wh = __reduce_max_sync(0xffffffffu, ehi[d]);
    if ((threadIdx.x & 31) == 0) { atomicMin(&bmin[d], wl); atomicMax(&bmax[d], wh); }
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
  // FP64: per-tap atomics (a 64 KB FP64 box per block leaves too few
  // blocks per SM for the FP64-bound arithmetic)
  k_ibm_spread<T><<<1216, 256, 0, s>>>(g, pg, b, fu, fv, fw, 1. / dt, coeff0);
}
template void launch_ibm_spread<double>(cudaStream_t, const Geo &, const PartGeo &, IbmBuffers, double *, double *,
                                        double *, double, int);

void launch_ibm_spread_f(cudaStream_t s, const Geo &g, const PartGeo &pg, IbmBuffers b, float *fu, float *fv,
                         float *fw, double dt, const float *dfin, const int *gate) {
  if (pg.np == 0) return;
  const double coeff0 = (pg.dVlagr / pg.dVeul) * dt;
  k_ibm_spread_box<float, PointStencilF, float><<<dim3(pg.np, 3), 384, 2 * SPREAD_BOX * sizeof(float), s>>>(
      g, pg, b, b.st32, fu, fv, fw, 1. / dt, coeff0, dfin, gate);
}


// ---------------------------------------------------------------------------
// Learned forcing (mixed form).  Features of each point after the first
// forcing pass, in the order they are produced:
//   [3q + c], q = (k*3 + j)*3 + i = 0..26, c = u, v, w : the velocity
//            component c at stencil tap q minus the body velocity U_c
//   [81:84] slip U - u~ after pass 1     [84:87] rigid-body velocity U
//   [87:90] outward unit normal          [90:93] pass-1 correction F0*dt
//   [93:96] centre delta weights (x, y, z)
// X receives them standardised with (mu, isig) and rounded to BF16 for the
// network, written in 16-byte groups as they are produced (no 96-float
// register array); a harvest stores every stride-th point's raw FP32
// features and index, for the target written after the plain passes.  The
// interpolated velocity goes to dudtl as eulr2lagr would.
// ---------------------------------------------------------------------------
struct FeatSink {
  __nv_bfloat16 *x;  // row of the standardised features (or null)
  float *raw;        // row of the raw features (or null)
  const float *mu, *isig;
  float buf[8];
  int n;  // features produced so far
  __device__ __forceinline__ void put(float v) {
    buf[n & 7] = v;
    ++n;
    if ((n & 7) == 0) flush(n - 8);
  }
  __device__ __forceinline__ void flush(int c0) {
    if (x) {
      __nv_bfloat162 h[4];
#pragma unroll
      for (int e = 0; e < 4; ++e)
        h[e] = __floats2bfloat162_rn((buf[2 * e] - mu[c0 + 2 * e]) * isig[c0 + 2 * e],
                                     (buf[2 * e + 1] - mu[c0 + 2 * e + 1]) * isig[c0 + 2 * e + 1]);
      *reinterpret_cast<uint4 *>(x + c0) = *reinterpret_cast<const uint4 *>(h);
    }
    if (raw) {
      *reinterpret_cast<float4 *>(raw + c0) = make_float4(buf[0], buf[1], buf[2], buf[3]);
      *reinterpret_cast<float4 *>(raw + c0 + 4) = make_float4(buf[4], buf[5], buf[6], buf[7]);
    }
  }
};

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
        for (int q = 0; q < 96; q += 8) *reinterpret_cast<uint4 *>(&X[(long)t * 96 + q]) = make_uint4(0, 0, 0, 0);
      continue;
    }
    FeatSink snk;
    snk.x = X ? X + (long)t * 96 : nullptr;
    snk.raw = nullptr;
    snk.mu = mu;
    snk.isig = isig;
    snk.n = 0;
    int h = -1;
    if (H.feat && (t + H.phase) % H.stride == 0) {
      h = atomicAdd(&H.count[0], 1);
      if (h < H.cap) {
        snk.raw = H.feat + (long)h * 96;
        H.pidx[h] = t;
      }
    }
    if (!snk.x && !snk.raw) {
      // nothing to write for this point: interpolation only
      float iu, iv, iw;
      interp_point_f(g, b.st32[t], fu, fv, fw, iu, iv, iw);
      b.dudtl[t] = iu; b.dvdtl[t] = iv; b.dwdtl[t] = iw;
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
    float au = 0.f, av = 0.f, aw = 0.f;
#pragma unroll
    for (int k = 0; k < 3; ++k)
#pragma unroll
      for (int j = 0; j < 3; ++j) {
        const float wyz = s.phiyh[j] * s.phizh[k];
        const float wyz2 = s.phiy[j] * s.phizh[k];
        const float wyz3 = s.phiyh[j] * s.phiz[k];
#pragma unroll
        for (int i = 0; i < 3; ++i) {
          const float tu = __ldg(&fu[fidx(g, ix[i], jyh[j], s.klow + k)]);
          const float tv = __ldg(&fv[fidx(g, ixh[i], jy[j], s.klow + k)]);
          const float tw = __ldg(&fw[fidx(g, ixh[i], jyh[j], s.klows + k)]);
          au += tu * (s.phix[i] * wyz);
          av += tv * (s.phixh[i] * wyz2);
          aw += tw * (s.phixh[i] * wyz3);
          snk.put(tu - Ux);
          snk.put(tv - Uy);
          snk.put(tw - Uz);
        }
      }
    b.dudtl[t] = au; b.dvdtl[t] = av; b.dwdtl[t] = aw;
    const double px = b.pf[PF_X * pg.np + p], py = b.pf[PF_Y * pg.np + p], pz = b.pf[PF_Z * pg.np + p];
    const float inv_r = (float)(1. / pg.radfp);
    snk.put(Ux - au); snk.put(Uy - av); snk.put(Uz - aw);
    snk.put(Ux); snk.put(Uy); snk.put(Uz);
    snk.put((float)(b.xfp[t] - px) * inv_r);
    snk.put((float)(b.yfp[t] - py) * inv_r);
    snk.put((float)(b.zfp[t] - pz) * inv_r);
    snk.put((float)(b.fxl[t] * dt)); snk.put((float)(b.fyl[t] * dt)); snk.put((float)(b.fzl[t] * dt));
    snk.put(s.phix[1]); snk.put(s.phiy[1]); snk.put(s.phiz[1]);
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


int ibm_set_smem_limits() {
  const cudaError_t e1 = cudaSuccess;
  cudaError_t e2 = cudaFuncSetAttribute(k_ibm_spread_box<float, PointStencilF, float>,
                                        cudaFuncAttributeMaxDynamicSharedMemorySize, 2 * SPREAD_BOX * (int)sizeof(float));
  const cudaError_t e3 = cudaSuccess;
  cudaError_t e4 = cudaFuncSetAttribute(k_ibm_interp_comp_f, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        INTERP_BOX * (int)sizeof(float));
  const cudaError_t e5 = cudaSuccess;
  return (e1 == cudaSuccess && e2 == cudaSuccess && e3 == cudaSuccess && e4 == cudaSuccess && e5 == cudaSuccess)
             ? 0
             : -1;
}

}  // namespace ibmk
