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
    // periodic z: the image rule of x and y along z (no wall clamps below)
    double coorzfp = g.zper ? zfp * g.dzi - (double)((long)floor((zfp - 0.5 * g.dz) / g.lz) * g.K) : zfp * g.dzi;
    // Guard: a point outside the grid (or a non-finite position) would index
    // outside the arrays; flag it and park the point at a safe location.
    if (!(coorxfp >= 0. && coorxfp <= g.I + 1.) || !(cooryfp >= 0. && cooryfp <= g.J + 1.) ||
        !(g.zper ? (coorzfp >= 0. && coorzfp <= g.K + 1.) : (coorzfp >= -1. && coorzfp <= g.K + 0.49))) {
      atomicExch(&b.err[2], 1);
      coorxfp = 1.; cooryfp = 1.; coorzfp = 1.5;
    }
    PointStencil s;
    s.ilows = fnint(coorxfp) - 1;
    s.jlows = fnint(cooryfp) - 1;
    s.klows = g.zper ? fnint(coorzfp) - 1 : max(fnint(coorzfp) - 1, 1);
    s.ilow = (int)floor(coorxfp);
    s.jlow = (int)floor(cooryfp);
    s.klow = g.zper ? (int)floor(coorzfp) : max(min((int)floor(coorzfp), g.K - 2), 1);
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
  int kz[3], kzs[3];
  for (int m = 0; m < 3; ++m) {
    kz[m] = zwrap(g, s.klow + m);
    kzs[m] = zwrap(g, s.klows + m);
  }
  interp_sep(s, [&](int i, int j, int k) { return (double)fu[fidx(g, ix[i], jyh[j], kz[k])]; },
             [&](int i, int j, int k) { return (double)fv[fidx(g, ixh[i], jy[j], kz[k])]; },
             [&](int i, int j, int k) { return (double)fw[fidx(g, ixh[i], jyh[j], kzs[k])]; }, ou, ov, ow);
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
    const double dV = p_dvl(pg, p);
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
                                                    double coeff0_, double dt) {
  const int n = pg.np * pg.nl;  // < 2^31 points (checked at create)
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
    const int p = t / pg.nl, l = t - p * pg.nl;
    if (l >= b.nla[p]) continue;
    const PointStencil s = b.st[t];
    // the particle's own Lagrangian volume when polydisperse
    const double coeff0 = pg.poly ? (pg.pdvl[p] / pg.dVeul) * dt : coeff0_;
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
    for (int k = 0; k < 3; ++k) {
      const int kz = zwrap(g, s.klow + k), kzs = zwrap(g, s.klows + k);
      for (int j = 0; j < 3; ++j) {
        const double a = dfx * coeff0 * s.phiyh[j] * s.phizh[k];
        const double bb = dfy * coeff0 * s.phiy[j] * s.phizh[k];
        const double cc = dfz * coeff0 * s.phiyh[j] * s.phiz[k];
        for (int i = 0; i < 3; ++i) {
          atomicAdd(&fu[fidx(g, ix[i], jyh[j], kz)], (T)(a * s.phix[i]));
          atomicAdd(&fv[fidx(g, ixh[i], jy[j], kz)], (T)(bb * s.phixh[i]));
          atomicAdd(&fw[fidx(g, ixh[i], jyh[j], kzs)], (T)(cc * s.phixh[i]));
        }
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

template <typename T>
void launch_ibm_spread(cudaStream_t s, const Geo &g, const PartGeo &pg, IbmBuffers b, T *fu, T *fv, T *fw, double dt,
                       int first) {
  (void)first;
  if (pg.np == 0) return;
  const double coeff0 = (pg.dVlagr / pg.dVeul) * dt;
  k_ibm_spread<T><<<1216, 256, 0, s>>>(g, pg, b, fu, fv, fw, 1. / dt, coeff0, dt);
}
template void launch_ibm_spread<double>(cudaStream_t, const Geo &, const PartGeo &, IbmBuffers, double *, double *,
                                        double *, double, int);

// targets of the slots reserved since the last call: (F_final - F0) * dt, the
// correction the plain passes 1.. added after pass 0
__global__ void k_ibm_harvest_targets(IbmBuffers b, HarvestArgs H, double dt) {
  const int lo = H.count[1], hi = min(H.count[0], H.cap);
  for (int h = lo + blockIdx.x * blockDim.x + threadIdx.x; h < hi; h += gridDim.x * blockDim.x) {
    const int t = H.pidx[h];
    const float *f = H.feat + (long)h * 96 + FEAT_F0;
    H.targ[3 * (long)h] = b.fxs[t] * (float)dt - f[0];
    H.targ[3 * (long)h + 1] = b.fys[t] * (float)dt - f[FEAT_PER_COMP];
    H.targ[3 * (long)h + 2] = b.fzs[t] * (float)dt - f[2 * FEAT_PER_COMP];
  }
}
__global__ void k_ibm_harvest_close(HarvestArgs H) {
  if (threadIdx.x == 0 && blockIdx.x == 0) H.count[1] = min(H.count[0], H.cap);
}
void launch_ibm_harvest_targets(cudaStream_t s, IbmBuffers b, const HarvestArgs &H, double dt) {
  k_ibm_harvest_targets<<<152, 256, 0, s>>>(b, H, dt);
  k_ibm_harvest_close<<<1, 32, 0, s>>>(H);
}
// Residual gate.  R = rms |U - u~| over all points after the loop (from the
// per-(particle, component) sums psum[p][c][0]) and R0 = rms of the first
// pass's slip (from rsum).  A plain loop's R/R0 measures how far its Nl
// passes reduce the slip on the current state, per RK stage (the predicted
// field, and with it the slip's pattern, differs between the stages); the
// learned loop of stage s is held to fallback ratio x (that stage's ratio x
// its own R0), i.e. to what the plain passes would reach from the same
// first-pass slip.  Learn state ls (device):
//   [0] R of the last learned loop      [1] plain R/R0 of stage 1 (the last measured)
//   [2] plain loops measured            [3] fallback ratio
//   [4] fallbacks taken                 [5] learned loops
//   [6] R0 of the last learned loop     [7] reference of the last gate
//   [8] fixed reference (> 0 replaces ratio x R0)
//   [9] R0 and [10] R of the last plain loop measured
//   [11], [12] plain R/R0 of stages 2 and 3; [13..15] plain loops measured per stage
// gate = 1 runs the plain passes 2..Nl after the learned correction.
__global__ void __launch_bounds__(1024) k_ibm_res_gate(int n, const double *__restrict__ psum,
                                                       const float *__restrict__ rsum, long npts, double *ls,
                                                       int *gate, int plain, int stage) {
  // per-(particle, component) sums are FP32 accurate (formed in FP32): their
  // totals in FP32 with warp shuffles, FP64 only for the gate's arithmetic
  __shared__ float sm[2][32];
  float acc = 0.f, acc0 = 0.f;
  for (int q = threadIdx.x; q < n; q += blockDim.x) {
    acc += (float)psum[3 * (long)q];
    acc0 += rsum[q];
  }
#pragma unroll
  for (int d = 16; d > 0; d >>= 1) {
    acc += __shfl_xor_sync(0xffffffffu, acc, d);
    acc0 += __shfl_xor_sync(0xffffffffu, acc0, d);
  }
  if ((threadIdx.x & 31) == 0) { sm[0][threadIdx.x >> 5] = acc; sm[1][threadIdx.x >> 5] = acc0; }
  __syncthreads();
  if (threadIdx.x != 0) return;
  double tot = 0., tot0 = 0.;
  for (int w = 0; w < (int)(blockDim.x >> 5); ++w) { tot += sm[0][w]; tot0 += sm[1][w]; }
  const double R = npts ? sqrt(tot / (double)npts) : 0., R0 = npts ? sqrt(tot0 / (double)npts) : 0.;
  const int cs = stage == 0 ? 1 : 10 + stage, ns = 13 + stage;
  if (plain) {  // the plain passes' reduction of the slip on the current state
    // the latest measurement alone: the reduction drifts as the flow (and
    // the learned forcing's imprint on it) develops, an average lags it
    ls[cs] = R0 > 0. ? R / R0 : 0.;
    ls[ns] += 1.;
    ls[2] += 1.;
    ls[9] = R0;
    ls[10] = R;
    return;
  }
  const double ref = ls[8] > 0. ? ls[8] : (ls[ns] > 0. ? ls[cs] * R0 : 0.);
  ls[0] = R;
  ls[5] += 1.;
  ls[6] = R0;
  ls[7] = ref;
  const int g = (!(R <= ls[3] * ref)) ? 1 : 0;  // NaN falls back too
  *gate = g;
  if (g) ls[4] += 1.;
}
void launch_ibm_residual_gate(cudaStream_t s, const PartGeo &pg, IbmBuffers b, long npts, double *ls, int *gate,
                              int plain, int stage) {
  k_ibm_res_gate<<<1, 1024, 0, s>>>(3 * pg.np, b.psum, b.rsum, npts, ls, gate, plain, stage);
}

__device__ __forceinline__ unsigned long long mix64(unsigned long long z) {  // splitmix64 finaliser
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}
__global__ void k_normal_fill(float *__restrict__ y, long n, unsigned seed, unsigned counter) {
  const unsigned long long key = ((unsigned long long)seed << 32) ^ counter;
  for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < n; q += (long)gridDim.x * blockDim.x) {
    const unsigned long long h = mix64(mix64(key * 0x9E3779B97F4A7C15ULL + (unsigned long long)q));
    // two 24-bit uniforms in (0, 1), Box-Muller (one deviate kept)
    const float u1 = ((float)(h & 0xFFFFFF) + 0.5f) * (1.f / 16777216.f);
    const float u2 = ((float)((h >> 24) & 0xFFFFFF) + 0.5f) * (1.f / 16777216.f);
    y[q] = sqrtf(-2.f * logf(u1)) * cospif(2.f * u2);
  }
}
void launch_normal_fill(cudaStream_t s, float *y, long n, unsigned seed, unsigned counter) {
  if (n <= 0) return;
  k_normal_fill<<<1216, 256, 0, s>>>(y, n, seed, counter);
}

}  // namespace ibmk
