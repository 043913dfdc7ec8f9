// particle_kernels.cu -- rigid-sphere side of the substep on one rank:
// intgr_over_sphere (intgr_over_sphere.f90:12-625), the collision /
// lubrication pass with its integer contact lists (intgr_nwtn_eulr.f90:326-605,
// collisions.f90:10-438), the Newton-Euler update (:607-667), sumrk3
// (:1586-1669), the periodic wrap and neighbour flags (:702-714, :1051-1090)
// and the new Lagrangian points (:1438-1485).
//
// Compiled without FMA contraction: these are few, sequential-per-particle
// operations whose roundings are kept equal to the reference so that the
// integer contact lists (firstc/qmax) come out identical.
#include "kernels.cuh"

namespace ibmk {

#define PF(f) b.pf[(long)(f) * np + p]
#define CFA(f, q) b.cf[((long)(f) * np + p) * nq + (q)]

// ---------------------------------------------------------------------------
// new -> old (intgr_nwtn_eulr.f90:77-118)
// ---------------------------------------------------------------------------
__global__ void k_save_old(PartGeo pg, PartBuffers b) {
  // one element per thread: the scalar fields x..coltz and the contact
  // fields dx..dwt of every master particle into their "old" copies
  const int np = pg.np, nq = pg.nq;
  const long nps = (long)(PF_COLTZ - PF_X + 1) * np;
  const long ncf = (long)(CF_DWT - CF_DX + 1) * np * nq;
  for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < nps + ncf; e += (long)gridDim.x * blockDim.x) {
    if (e < nps) {
      const int f = PF_X + (int)(e / np), p = (int)(e % np);
      if (b.mslv[p] > 0) b.pf[(long)(f + (PF_OX - PF_X)) * np + p] = b.pf[(long)f * np + p];
    } else {
      const long r = e - nps;
      const int f = CF_DX + (int)(r / ((long)np * nq));
      const long pq = r % ((long)np * nq);
      const int p = (int)(pq / nq);
      if (b.mslv[p] > 0) b.cf[(long)(f + (CF_ODX - CF_DX)) * np * nq + pq] = b.cf[(long)f * np * nq + pq];
    }
  }
}
void launch_save_old(cudaStream_t s, const PartGeo &pg, PartBuffers b) {
  if (pg.np == 0) return;
  k_save_old<<<304, 256, 0, s>>>(pg, b);
}

// ---------------------------------------------------------------------------
// intgr_over_sphere.  One block per particle; the self-neighbour copies of a
// particle near the periodic edges integrate the wrapped part of the box
// (intgr_over_sphere.f90:84-112 and :298-313).  type 1 = volume, type 2 =
// integral of u (intu..), type 3 = integral of r x u (intomx..), type 23 =
// types 2 and 3 in one sweep (they read the same fields).
// ---------------------------------------------------------------------------
__device__ __forceinline__ void copy_shift_sphere(int nbrecv, double lx, double ly, double &x, double &y) {
  switch (nbrecv) {
    case 1: x = x + lx; break;
    case 2: x = x + lx; y = y - ly; break;
    case 3: y = y - ly; break;
    case 4: x = x - lx; y = y - ly; break;
    case 5: x = x - lx; break;
    case 6: x = x - lx; y = y + ly; break;
    case 7: y = y + ly; break;
    case 8: x = x + lx; y = y + ly; break;
    default: break;
  }
}

// corner signed-distance fraction of a cell cut by the sphere surface
// (intgr_over_sphere.f90:357-374): sum of the positive signed distances over
// the sum of their magnitudes, corners in the reference's order
__device__ __forceinline__ double corner_fraction(double radius, double dxm2, double dxp2, double dym2, double dyp2,
                                                  double dzm2, double dzp2) {
  double sg[8];
  sg[0] = radius - sqrt(dxm2 + dym2 + dzm2);
  sg[1] = radius - sqrt(dxm2 + dyp2 + dzm2);
  sg[2] = radius - sqrt(dxp2 + dyp2 + dzm2);
  sg[3] = radius - sqrt(dxp2 + dym2 + dzm2);
  sg[4] = radius - sqrt(dxm2 + dym2 + dzp2);
  sg[5] = radius - sqrt(dxm2 + dyp2 + dzp2);
  sg[6] = radius - sqrt(dxp2 + dyp2 + dzp2);
  sg[7] = radius - sqrt(dxp2 + dym2 + dzp2);
  double sum1 = 0., sum2 = 0.;
  for (int cp = 0; cp < 8; ++cp) {
    if (sg[cp] > 0.) sum1 = sum1 + sg[cp];
    sum2 = sum2 + fabs(sg[cp]);
  }
  return sum1 / sum2;
}

// FP32 corner fraction (mixed form): the same expression in single
// precision, with the hardware's approximate square root and reciprocal
// (relative errors of a few 1e-7, below the FP32 rounding of the squared
// distances they act on); its decisions at the surface are continuous in
// the distances
__device__ __forceinline__ float sqrt_approx(float x) {
  float y;
  asm("sqrt.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
__device__ __forceinline__ float corner_fraction_f(float radius, float dxm2, float dxp2, float dym2, float dyp2,
                                                  float dzm2, float dzp2) {
  float sg[8];
  sg[0] = radius - sqrt_approx(dxm2 + dym2 + dzm2);
  sg[1] = radius - sqrt_approx(dxm2 + dyp2 + dzm2);
  sg[2] = radius - sqrt_approx(dxp2 + dyp2 + dzm2);
  sg[3] = radius - sqrt_approx(dxp2 + dym2 + dzm2);
  sg[4] = radius - sqrt_approx(dxm2 + dym2 + dzp2);
  sg[5] = radius - sqrt_approx(dxm2 + dyp2 + dzp2);
  sg[6] = radius - sqrt_approx(dxp2 + dyp2 + dzp2);
  sg[7] = radius - sqrt_approx(dxp2 + dym2 + dzp2);
  float sum1 = 0.f, sum2 = 0.f;
#pragma unroll
  for (int cp = 0; cp < 8; ++cp) {
    sum1 += fmaxf(sg[cp], 0.f);
    sum2 += fabsf(sg[cp]);
  }
  return __fdividef(sum1, sum2);
}

// Sums of one velocity component over the cells of the sphere's box.  Block
// (p, comp); a thread owns whole i-lines (fixed j, k), so the lever arms ry,
// rz of the torque are constant along its line and only
//   S0 = sum f*w,  Sx = sum rx*f*w
// accumulate per cell (FP64).  w = 1 for cells inside radin or with all
// corners inside, 0 with all corners outside, else the corner fraction.
// Classification: FP32 screening of the squared corner distances with a
// relative margin (1e-5) far above its rounding; in the plain form every
// cell the screen cannot decide goes to a shared-memory queue that all
// threads then run through the reference's FP64 tests (full warps for the
// FP64 work).  The mixed form (GEO32) evaluates the cut cells in FP32.
// Output: b.red[np + (p*3 + comp)*3 + {0,1,2}] = {S0, torque_a, torque_b}
// without the dVeul factor (k_sphere_final).
template <typename T, bool GEO32>
__global__ void __launch_bounds__(256) k_sphere_int(Geo g, PartGeo pg, PartBuffers b, const T *__restrict__ u,
                                                    const T *__restrict__ v, const T *__restrict__ w) {
  constexpr int AX = 128, QCAP = 2048;
  const int np = pg.np;
  const int p = blockIdx.x, comp = blockIdx.y;
  const int ms = b.mslv[p];
  if (ms <= 0) return;
  // Block-uniform FP64 set-up (thresholds, the box of each periodic copy)
  // is computed by one thread and read from shared memory: FP64 issues at a
  // small fraction of the FP32 rate, and every thread repeating it cost more
  // than the line sums themselves.
  __shared__ double s_radin2, s_cx, s_cy, s_cz, s_rad, s_rthr;
  __shared__ float s_thr[7];
  __shared__ int s_box[6];  // ilow, ni, jlow, nj, klow, nk
  if (threadIdx.x == 0) {
    const double rad = p_rad(pg, p), rth = p_rthr(pg, p);  // the particle's own when polydisperse
    const double radin = rad - 2. * g.dx;
    const double radin2 = radin * radin;
    s_radin2 = radin2;
    s_rad = rad;
    s_rthr = rth;
    // sqrt(d2) >= radius  <=>  d2 >= rthr (rthr: smallest double whose
    // correctly rounded square root is >= radius)
    s_thr[0] = (float)(radin2 * (1. - 1e-5));
    s_thr[1] = (float)(radin2 * (1. + 1e-5));
    s_thr[2] = (float)(rth * (1. - 1e-5));
    s_thr[3] = (float)(rth * (1. + 1e-5));
    s_thr[4] = (float)radin2;
    s_thr[5] = (float)rth;
    s_thr[6] = (float)rad;
  }
  __syncthreads();
  const double radius = s_rad, dx = g.dx, dy = g.dy, dz = g.dz;
  const double radin2 = s_radin2, rthr = s_rthr;
  const float radin2_lo = s_thr[0], radin2_hi = s_thr[1], rthr_lo = s_thr[2], rthr_hi = s_thr[3];
  const float radin2f = s_thr[4], rthrf = s_thr[5], radiusf = s_thr[6];
  __shared__ double sxm[AX], sxp[AX], srx[AX], sym[AX], syp[AX], sry[AX], szm[AX], szp[AX], srz[AX];
  __shared__ float fxm[AX], fxp[AX], fym[AX], fyp[AX], fzm[AX], fzp[AX];
  // rx, ry, rz as double-float pairs (mixed form)
  __shared__ float frxh[GEO32 ? AX : 1], frxl[GEO32 ? AX : 1], fryh[GEO32 ? AX : 1], fryl[GEO32 ? AX : 1];
  __shared__ float frzh[GEO32 ? AX : 1], frzl[GEO32 ? AX : 1];
  __shared__ int queue[GEO32 ? 1 : QCAP];
  __shared__ int qn;
  __shared__ double red[3][256];
  const T *F = comp == 0 ? u : (comp == 1 ? v : w);
  const int *nbf = b.nb + (long)p * 9;
  double a0 = 0., ta = 0., tb = 0.;
  // mixed form: the same three sums in double-float across the lines
  float A0h = 0.f, A0l = 0.f, TAh = 0.f, TAl = 0.f, TBh = 0.f, TBl = 0.f;
  // lever arms per component: ta += la * f*w, tb += lb * f*w with
  // comp 0: (rz, -ry), comp 1: (-rz, rx), comp 2: (ry, -rx)
  // copies nb = 0..8 (x/y images); with periodic z each also at z -+ lz
  const int nzs = pg.zper ? 3 : 1;
  for (int nbz = 0; nbz < 9 * nzs; ++nbz) {
    const int nb = nbz / nzs, zs = nbz - nb * nzs;
    if (nb > 0 && nbf[nb] != 1) continue;
    __syncthreads();  // previous copy done with the tables and the box
    if (threadIdx.x == 0) {
      int nbrecv = nb;
      if (nb > 0) { nbrecv = nb + 4; if (nbrecv > 8) nbrecv -= 8; }
      double cx = PF(PF_X), cy = PF(PF_Y);
      const double cz = PF(PF_Z) + (zs == 1 ? -pg.lz : (zs == 2 ? pg.lz : 0.));
      if (nb > 0) copy_shift_sphere(nbrecv, g.lx, g.ly, cx, cy);
      int ilow = fnint((cx - radius) * g.dxi - 2.), ihigh = fnint((cx + radius) * g.dxi + 2.);
      int jlow = fnint((cy - radius) * g.dyi - 2.), jhigh = fnint((cy + radius) * g.dyi + 2.);
      int klow = fnint((cz - radius) * g.dzi - 2.), khigh = fnint((cz + radius) * g.dzi + 2.);
      if (ilow < 1) ilow = 1;
      if (jlow < 1) jlow = 1;
      if (klow < 1) klow = 1;
      if (ihigh > g.I) ihigh = g.I;
      if (jhigh > g.J) jhigh = g.J;
      if (khigh > g.K) khigh = g.K;
      s_cx = cx; s_cy = cy; s_cz = cz;
      s_box[0] = ilow; s_box[1] = ihigh - ilow + 1;
      s_box[2] = jlow; s_box[3] = jhigh - jlow + 1;
      s_box[4] = klow; s_box[5] = khigh - klow + 1;
    }
    __syncthreads();
    const double cx = s_cx, cy = s_cy, cz = s_cz;
    const int ilow = s_box[0], ni = s_box[1], jlow = s_box[2], nj = s_box[3], klow = s_box[4], nk = s_box[5];
    if (ni <= 0 || nj <= 0 || nk <= 0) continue;
    if (ni > AX || nj > AX || nk > AX) {  // sphere wider than the axis tables: flag, skip
      if (threadIdx.x == 0) atomicExch(&b.err[3], 1);
      continue;
    }
    // per-axis corner distances and cell-centre offsets, in the reference's
    // expressions (intgr_over_sphere.f90:335-508)
    for (int t = threadIdx.x; t < AX; t += blockDim.x) {
      if (t < ni) {
        const int i = ilow + t;
        double mn, pl;
        if (comp == 0) { mn = 0. + (i - 0.5) * dx; pl = 0. + (i + 0.5) * dx; }
        else { mn = 0. + (i - 1) * dx; pl = 0. + i * dx; }
        sxm[t] = (mn - cx) * (mn - cx); sxp[t] = (pl - cx) * (pl - cx);
        fxm[t] = (float)sxm[t]; fxp[t] = (float)sxp[t];
        srx[t] = 0. + (i - 0.5) * dx - cx;
        if constexpr (GEO32) {
          frxh[t] = (float)srx[t];
          frxl[t] = (float)(srx[t] - (double)frxh[t]);
        }
      }
      if (t < nj) {
        const int j = jlow + t;
        double mn, pl;
        if (comp == 1) { mn = 0. + (j - 0.5) * dy; pl = 0. + (j + 0.5) * dy; }
        else { mn = 0. + (j - 1) * dy; pl = 0. + j * dy; }
        sym[t] = (mn - cy) * (mn - cy); syp[t] = (pl - cy) * (pl - cy);
        fym[t] = (float)sym[t]; fyp[t] = (float)syp[t];
        sry[t] = 0. + (j - 0.5) * dy - cy;
        if constexpr (GEO32) {
          fryh[t] = (float)sry[t];
          fryl[t] = (float)(sry[t] - (double)fryh[t]);
        }
      }
      if (t < nk) {
        const int k = klow + t;
        double mn, pl;
        if (comp < 2) { mn = (k - 1) * dz; pl = k * dz; }
        else { mn = (k - 0.5) * dz; pl = (k + 0.5) * dz; }
        szm[t] = (mn - cz) * (mn - cz); szp[t] = (pl - cz) * (pl - cz);
        fzm[t] = (float)szm[t]; fzp[t] = (float)szp[t];
        srz[t] = (k - 0.5) * dz - cz;
        if constexpr (GEO32) {
          frzh[t] = (float)srz[t];
          frzl[t] = (float)(srz[t] - (double)frzh[t]);
        }
      }
    }
    if (threadIdx.x == 0) qn = 0;
    __syncthreads();
    const int nlines = nj * nk;
    const long row0 = fidx(g, ilow - 1, 0, 0);
    for (int base = 0; base < nlines; base += blockDim.x) {
      const int L = base + threadIdx.x;
      if (L < nlines) {
        const int tj = L % nj, tk = L / nj;
        const float yzp = fyp[tj] + fzp[tk];
        const float ymin = fminf(fym[tj], fyp[tj]) + fminf(fzm[tk], fzp[tk]);
        const float ymax = fmaxf(fym[tj], fyp[tj]) + fmaxf(fzm[tk], fzp[tk]);
        const long lo = row0 + fidx(g, 0, jlow + tj - 1, klow + tk);
        double s0 = 0., sx = 0.;
        float s0h = 0.f, s0l = 0.f, sxh = 0.f, sxl = 0.f;  // mixed form: double-float line sums
        for (int ti = 0; ti < ni; ++ti) {
          const float dxp2f = fxp[ti], dxm2f = fxm[ti];
          const float dist2f = dxp2f + yzp;
          const float mind2f = fminf(dxm2f, dxp2f) + ymin;
          if (GEO32) {
            if (!(dist2f < radin2f) && mind2f >= rthrf) continue;  // outside
          } else {
            if (!(dist2f < radin2_lo) && !(dist2f <= radin2_hi) && mind2f > rthr_hi) continue;
          }
          if constexpr (GEO32) {
            // FP32 velocity times FP32 weight, summed along the line in
            // double-float (error-free products and sums on the FP32 pipes)
            const float ff = F ? (float)F[lo + ti] : 1.f;
            float wgt = 1.f;
            if (!(dist2f < radin2f)) {
              const float maxd2f = fmaxf(dxm2f, dxp2f) + ymax;
              if (!(maxd2f < rthrf))
                wgt = corner_fraction_f(radiusf, dxm2f, dxp2f, fym[tj], fyp[tj], fzm[tk], fzp[tk]);
            }
            float ph = ff, pe = 0.f;
            if (wgt != 1.f) two_prod(ff, wgt, ph, pe);
            df_add(s0h, s0l, ph, pe, s0h, s0l);
            if (comp != 0) {
              float qh, ql;
              df_mul(ph, pe, frxh[ti], frxl[ti], qh, ql);
              df_add(sxh, sxl, qh, ql, sxh, sxl);
            }
            continue;
          }
          const double f = F ? (double)F[lo + ti] : 1.;
          double fw;
          {
            bool sure = dist2f < radin2_lo;  // surely inside radin
            if (!sure && dist2f > radin2_hi) {
              const float maxd2f = fmaxf(dxm2f, dxp2f) + ymax;
              sure = maxd2f < rthr_lo;  // surely all corners inside
            }
            if (!sure) {  // the reference's FP64 test decides
              const int q = atomicAdd(&qn, 1);
              if (q < QCAP) {
                queue[q] = ti | (tj << 8) | (tk << 16);
                continue;
              }
              // queue full: decide here
              const double dxp2 = sxp[ti], dyp2 = syp[tj], dzp2 = szp[tk];
              double frac = 1.;
              if (!(dxp2 + dyp2 + dzp2 < radin2)) {
                const double dxm2 = sxm[ti], dym2 = sym[tj], dzm2 = szm[tk];
                const double mind2 = fmin(dxm2, dxp2) + fmin(dym2, dyp2) + fmin(dzm2, dzp2);
                if (mind2 >= rthr) continue;
                const double maxd2 = fmax(dxm2, dxp2) + fmax(dym2, dyp2) + fmax(dzm2, dzp2);
                if (!(maxd2 < rthr)) frac = corner_fraction(radius, dxm2, dxp2, dym2, dyp2, dzm2, dzp2);
              }
              fw = f * frac;
            } else {
              fw = f;
            }
          }
          s0 += fw;
          sx = fma(srx[ti], fw, sx);
        }
        if constexpr (GEO32) {
          // the line sums into the thread's double-float totals (no FP64
          // per line)
          float qh, ql;
          df_add(A0h, A0l, s0h, s0l, A0h, A0l);
          if (comp == 0) {
            df_mul(s0h, s0l, frzh[tk], frzl[tk], qh, ql);
            df_add(TAh, TAl, qh, ql, TAh, TAl);
            df_mul(s0h, s0l, fryh[tj], fryl[tj], qh, ql);
            df_add(TBh, TBl, -qh, -ql, TBh, TBl);
          } else if (comp == 1) {
            df_mul(s0h, s0l, frzh[tk], frzl[tk], qh, ql);
            df_add(TAh, TAl, -qh, -ql, TAh, TAl);
            df_add(TBh, TBl, sxh, sxl, TBh, TBl);
          } else {
            df_mul(s0h, s0l, fryh[tj], fryl[tj], qh, ql);
            df_add(TAh, TAl, qh, ql, TAh, TAl);
            df_add(TBh, TBl, -sxh, -sxl, TBh, TBl);
          }
        } else {
          const double ry = sry[tj], rz = srz[tk];
          a0 += s0;
          if (comp == 0) { ta = fma(rz, s0, ta); tb = fma(-ry, s0, tb); }
          else if (comp == 1) { ta = fma(-rz, s0, ta); tb += sx; }
          else { ta = fma(ry, s0, ta); tb -= sx; }
        }
      }
      if (!GEO32) {
        __syncthreads();
        const int nq = min(qn, QCAP);
        for (int q = threadIdx.x; q < nq; q += blockDim.x) {
          const int e = queue[q];
          const int ti = e & 0xff, tj = (e >> 8) & 0xff, tk = e >> 16;
          const double dxp2 = sxp[ti], dyp2 = syp[tj], dzp2 = szp[tk];
          double frac = 1.;
          if (!(dxp2 + dyp2 + dzp2 < radin2)) {
            const double dxm2 = sxm[ti], dym2 = sym[tj], dzm2 = szm[tk];
            const double mind2 = fmin(dxm2, dxp2) + fmin(dym2, dyp2) + fmin(dzm2, dzp2);
            if (mind2 >= rthr) continue;
            const double maxd2 = fmax(dxm2, dxp2) + fmax(dym2, dyp2) + fmax(dzm2, dzp2);
            if (!(maxd2 < rthr)) frac = corner_fraction(radius, dxm2, dxp2, dym2, dyp2, dzm2, dzp2);
          }
          const double fw = (F ? (double)F[row0 + fidx(g, ti, jlow + tj - 1, klow + tk)] : 1.) * frac;
          const double rx = srx[ti], ry = sry[tj], rz = srz[tk];
          a0 += fw;
          if (comp == 0) { ta = fma(rz, fw, ta); tb = fma(-ry, fw, tb); }
          else if (comp == 1) { ta = fma(-rz, fw, ta); tb = fma(rx, fw, tb); }
          else { ta = fma(ry, fw, ta); tb = fma(-rx, fw, tb); }
        }
        __syncthreads();
        if (threadIdx.x == 0) qn = 0;
        __syncthreads();
      }
    }
  }
  if constexpr (GEO32) {
    a0 += (double)A0h + (double)A0l;
    ta += (double)TAh + (double)TAl;
    tb += (double)TBh + (double)TBl;
  }
  // block sums: three warps, each over one of the staged partials
  red[0][threadIdx.x] = a0;
  red[1][threadIdx.x] = ta;
  red[2][threadIdx.x] = tb;
  __syncthreads();
  const int wq = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (wq < 3) {
    double x = 0.;
    for (int q = lane; q < (int)blockDim.x; q += 32) x += red[wq][q];
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) x += __shfl_down_sync(0xffffffffu, x, d);
    if (lane == 0) b.red[np + ((long)p * 3 + comp) * 3 + wq] = x;
  }
}

// unit field for the volume sums (type 1)
__device__ __forceinline__ void snapshot_particle(const PartGeo &pg, PartBuffers &b, int p);
// snap: also take the collision iteration's snapshot of this particle (the
// positions and velocities the integrals leave unchanged), saving its launch
template <typename T>
__global__ void k_sphere_final(PartGeo pg, PartBuffers b, int type, int snap) {
  const int np = pg.np;
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= np) return;
  if (snap) snapshot_particle(pg, b, p);
  const int ms = b.mslv[p];
  if (ms == 0) return;
  const double dV = pg.dVeul;
  double A[3] = {0, 0, 0}, tq[3] = {0, 0, 0};
  if (ms > 0) {
    const double *s = b.red + np + (long)p * 9;  // [comp][S0, ta, tb]
    for (int c = 0; c < 3; ++c) A[c] = s[3 * c] * dV;
    tq[0] = (s[3 * 1 + 1] + s[3 * 2 + 1]) * dV;
    tq[1] = (s[3 * 0 + 1] + s[3 * 2 + 2]) * dV;
    tq[2] = (s[3 * 0 + 2] + s[3 * 1 + 2]) * dV;
  }
  if (type == 1) b.red[p] = A[0];  // volume of the u-cells (intgr_over_sphere.f90:607-622)
  if (type == 1 || type == 2 || type == 23) { PF(PF_INTU) = A[0]; PF(PF_INTV) = A[1]; PF(PF_INTW) = A[2]; }
  if (type == 3 || type == 23) { PF(PF_INTOMX) = tq[0]; PF(PF_INTOMY) = tq[1]; PF(PF_INTOMZ) = tq[2]; }
}

template <typename T>
void launch_sphere_integrals(cudaStream_t s, const Geo &g, const PartGeo &pg, PartBuffers b, const T *u, const T *v,
                             const T *w, int type, bool snapshot) {
  if (pg.np == 0) return;
  const dim3 grid(pg.np, 3);
  const bool unit = type == 1;  // volume: integrate w = 1 (F == nullptr)
  if constexpr (sizeof(T) == 4)
    k_sphere_int<T, true><<<grid, 256, 0, s>>>(g, pg, b, unit ? nullptr : u, unit ? nullptr : v, unit ? nullptr : w);
  else
    k_sphere_int<T, false><<<grid, 256, 0, s>>>(g, pg, b, unit ? nullptr : u, unit ? nullptr : v, unit ? nullptr : w);
  k_sphere_final<T><<<(pg.np + 127) / 128, 128, 0, s>>>(pg, b, type, snapshot ? 1 : 0);
}
template void launch_sphere_integrals<double>(cudaStream_t, const Geo &, const PartGeo &, PartBuffers,
                                              const double *, const double *, const double *, int, bool);
template void launch_sphere_integrals<float>(cudaStream_t, const Geo &, const PartGeo &, PartBuffers, const float *,
                                             const float *, const float *, int, bool);

// ---------------------------------------------------------------------------
// collisions / lubrication (collisions.f90).  Only the normal contact force
// and the normal lubrication force are applied (collisions.f90:199-205,
// 430-432); the tangential history is still evolved and stored.
// ---------------------------------------------------------------------------
// the scalar normal lubrication force f1 of lubrication (collisions.f90:222-438)
__device__ double d_lub_f1(const PartGeo &pg, double pu, double pv, double pw, int idq, double nx, double ny,
                           double nz, double eps, double u_nb, double v_nb, double w_nb, double coeff_f) {
  const double u1a = pu * nx + pv * ny + pw * nz;
  const double u1b = u_nb * nx + v_nb * ny + w_nb * nz;
  double f1;
  if (idq > pg.np) {
    double a11;
    if (eps < 0.001) a11 = pg.a11_sat_pw;
    else a11 = -(1. / eps) + 1. / 5. * log(eps) + 1. / 21. * eps * log(eps) - .9713;
    f1 = (a11 * u1a);
    f1 = coeff_f * (f1 - (pg.a11_ini_pw * u1a));
  } else {
    double a11a, a11b;
    if (eps < 0.001) { a11a = pg.a11a_sat_pp; a11b = pg.a11b_sat_pp; }
    else {
      const double a11 = -(1. / 4. * pow(eps, -1.)) + 9. / 40. * log(eps) + 3. / 112. * eps * log(eps);
      a11a = a11 - .995;
      a11b = -a11 + .350;
    }
    f1 = (a11a * u1a + a11b * u1b);
    f1 = coeff_f * (f1 - (pg.a11a_ini_pp * u1a + pg.a11b_ini_pp * u1b));
  }
  return f1;
}
__device__ void d_lubrication(const PartGeo &pg, double pu, double pv, double pw, int idq, double nx, double ny,
                              double nz, double eps, double u_nb, double v_nb, double w_nb, double coeff_f,
                              double &cfx, double &cfy, double &cfz) {
  const double f1 = d_lub_f1(pg, pu, pv, pw, idq, nx, ny, nz, eps, u_nb, v_nb, w_nb, coeff_f);
  cfx = cfx + f1 * nx;
  cfy = cfy + f1 * ny;
  cfz = cfz + f1 * nz;
}

// Polydisperse pair constants (init.f90:137-241 with the pair's effective
// mass ratiorho vp vq / (vp + vq), or ratiorho vp for a wall, and the
// lubrication prefactor 6 pi nu Re of the equivalent radius Re), as the
// oracle's pair_consts forms them
struct PairC {
  double kn, kt, etan, etat, muc, coeff_f;
};
__device__ PairC pair_consts(const PartGeo &pg, double vp, double vq, double re) {
  const double me = vq > 0. ? pg.ratiorho * vp * vq / (vp + vq) : pg.ratiorho * vp, mt = 2. / 7. * me;
  PairC k;
  k.kn = pg.pc_an * me / pg.pc_b;
  k.kt = pg.pc_at * mt / pg.pc_b;
  k.etan = pg.pc_en * me / pg.pc_ndt;
  k.etat = pg.pc_et * mt / pg.pc_ndt;
  k.muc = 0.;
  k.coeff_f = 6. * IBM_PI * pg.visc * re;
  return k;
}

struct PState {  // the particle's own state held in registers by the collision thread
  double u, v, w, omx, omy, omz, colfx, colfy, colfz;
};

__device__ void d_collisions(const PartGeo &pg, PartBuffers &b, int p, PState &S, int qq, int idq, double dist,
                             double deltax, double deltay, double deltaz, double u_nb, double v_nb, double w_nb,
                             double omx_nb, double omy_nb, double omz_nb, double dtsub, double rkab) {
  const int np = pg.np, nq = pg.nq;
  const double radius = p_rad(pg, p);
  // polydisperse: the partner's radius in its own rotation term (a wall: 0)
  const double rq = pg.poly ? (idq <= np ? pg.prad[idq - 1] : 0.) : radius;
  const double nx = deltax / dist, ny = deltay / dist, nz = deltaz / dist;
  double deltan, kn, etan, kt, etat, muc;
  if (pg.poly) {
    const bool wall = idq > np;
    const PairC k = pair_consts(pg, pg.pvol[p], wall ? 0. : pg.pvol[idq - 1], radius);
    deltan = (wall ? radius : radius + rq) - dist;
    kn = k.kn; kt = k.kt; etan = k.etan; etat = k.etat; muc = k.muc;
  } else if (idq <= np) {
    deltan = 2 * radius - dist; kn = pg.kn_ss; kt = pg.kt_ss; etan = pg.etan_ss; etat = pg.etat_ss; muc = pg.muc_ss;
  } else {
    deltan = radius - dist; kn = pg.kn_sw; kt = pg.kt_sw; etan = pg.etan_sw; etat = pg.etat_sw; muc = pg.muc_sw;
  }
  const double dun = (S.u + (S.omy * radius * nz) - (S.omz * radius * ny)) -
                     (u_nb + (omy_nb * rq * (-nz)) - (omz_nb * rq * (-ny)));
  const double dvn = (S.v - (S.omx * radius * nz) + (S.omz * radius * nx)) -
                     (v_nb - (omx_nb * rq * (-nz)) + (omz_nb * rq * (-nx)));
  const double dwn = (S.w + (S.omx * radius * ny) - (S.omy * radius * nx)) -
                     (w_nb + (omx_nb * rq * (-ny)) - (omy_nb * rq * (-nx)));
  const double vabs = dun * nx + dvn * ny + dwn * nz;
  const double fxn = -(kn * (deltan * nx)) - etan * (vabs * nx);
  const double fyn = -(kn * (deltan * ny)) - etan * (vabs * ny);
  const double fzn = -(kn * (deltan * nz)) - etan * (vabs * nz);
  const double dut = dun - vabs * nx, dvt = dvn - vabs * ny, dwt = dwn - vabs * nz;
  const double vtabs = sqrt(dut * dut + dvt * dvt + dwt * dwt);
  const int q = qq - 1;
  const double odx = CFA(CF_ODX, q), ody = CFA(CF_ODY, q), odz = CFA(CF_ODZ, q);
  const double distold = sqrt(odx * odx + ody * ody + odz * odz);
  double nxold, nyold, nzold;
  if (distold == 0) { nxold = nx; nyold = ny; nzold = nz; }
  else { nxold = odx / distold; nyold = ody / distold; nzold = odz / distold; }
  double dxt, dyt, dzt;
  if (b.firstc[(long)p * nq + q] == idq) {
    double hx = ny * nzold - nyold * nz;
    double hy = nz * nxold - nzold * nx;
    double hz = nx * nyold - nxold * ny;
    const double aa = sqrt(hx * hx + hy * hy + hz * hz);
    const double cc = cos(asin(aa));
    const double bb = 1. - cc;
    if (aa == 0.) { hx = 0.; hy = 0.; hz = 0.; }
    else { hx = hx / aa; hy = hy / aa; hz = hz / aa; }
    const double h11 = bb * (hx * hx) + cc, h12 = bb * hx * hy - aa * hz, h13 = bb * hx * hz + aa * hy;
    const double h21 = bb * hx * hy + aa * hz, h22 = bb * (hy * hy) + cc, h23 = bb * hy * hz - aa * hx;
    const double h31 = bb * hx * hz - aa * hy, h32 = bb * hy * hz + aa * hx, h33 = bb * (hz * hz) + cc;
    const double oxt = CFA(CF_ODXT, q), oyt = CFA(CF_ODYT, q), ozt = CFA(CF_ODZT, q);
    const double out_ = CFA(CF_ODUT, q), ovt = CFA(CF_ODVT, q), owt = CFA(CF_ODWT, q);
    dxt = oxt * h11 + oyt * h21 + ozt * h31 + 0.5 * dtsub * rkab * (dut + out_ * h11 + ovt * h21 + owt * h31);
    dyt = oxt * h12 + oyt * h22 + ozt * h32 + 0.5 * dtsub * rkab * (dvt + out_ * h12 + ovt * h22 + owt * h32);
    dzt = oxt * h13 + oyt * h23 + ozt * h33 + 0.5 * dtsub * rkab * (dwt + out_ * h13 + ovt * h23 + owt * h33);
  } else {
    CFA(CF_PSI, q) = vtabs / fabs(vabs);
    dxt = 0.; dyt = 0.; dzt = 0.;
  }
  double fxt = -(kt * dxt) - (etat * dut);
  double fyt = -(kt * dyt) - (etat * dvt);
  double fzt = -(kt * dzt) - (etat * dwt);
  const double fnabs = sqrt(fxn * fxn + fyn * fyn + fzn * fzn);
  double ftabs = sqrt(fxt * fxt + fyt * fyt + fzt * fzt);
  const double tx = -fxt / ftabs, ty = -fyt / ftabs, tz = -fzt / ftabs;
  if (!(ftabs <= muc * fnabs)) {
    dxt = muc * fnabs * tx / kt;
    dyt = muc * fnabs * ty / kt;
    dzt = muc * fnabs * tz / kt;
  }
  S.colfx = S.colfx + fxn;
  S.colfy = S.colfy + fyn;
  S.colfz = S.colfz + fzn;
  CFA(CF_DX, q) = deltax; CFA(CF_DY, q) = deltay; CFA(CF_DZ, q) = deltaz;
  CFA(CF_DXT, q) = dxt; CFA(CF_DYT, q) = dyt; CFA(CF_DZT, q) = dzt;
  CFA(CF_DUT, q) = dut; CFA(CF_DVT, q) = dvt; CFA(CF_DWT, q) = dwt;
}

__device__ void d_remove_contact(const PartGeo &pg, PartBuffers &b, int p, int i, int &qlast) {
  const int np = pg.np, nq = pg.nq;
  const int a = i - 1, l = qlast - 1;
  int *fc = b.firstc + (long)p * nq, *ofc = b.ofirstc + (long)p * nq;
  if (qlast > 1) {
    fc[a] = fc[l];
    for (int f : {CF_DXT, CF_DYT, CF_DZT, CF_DUT, CF_DVT, CF_DWT}) CFA(f, a) = CFA(f, l);
    ofc[a] = ofc[l];
    for (int f : {CF_ODXT, CF_ODYT, CF_ODZT, CF_ODUT, CF_ODVT, CF_ODWT}) CFA(f, a) = CFA(f, l);
  }
  fc[l] = 0;
  ofc[l] = 0;
  for (int f = CF_DX; f <= CF_DWT; ++f) CFA(f, l) = 0.;
  for (int f = CF_ODX; f <= CF_ODWT; ++f) CFA(f, l) = 0.;
  qlast = qlast - 1;
}
__device__ void d_new_contact(const PartGeo &pg, PartBuffers &b, int p, int slot) {
  const int np = pg.np, nq = pg.nq;
  const int s = slot - 1;
  for (int f = CF_DX; f <= CF_DWT; ++f) CFA(f, s) = 0.;
  for (int f = CF_ODX; f <= CF_ODWT; ++f) CFA(f, s) = 0.;
}

// position of particle copy nb in the collision loop on one rank
// (intgr_nwtn_eulr.f90:223-322, coords=(0,0), dims=(1,1))
__device__ __forceinline__ void copy_shift_coll(int nb, double lx, double ly, double &x, double &y) {
  const double boundleftnb = lx, boundrightnb = 0., boundbacknb = 0., boundfrontnb = ly;
  switch (nb) {
    case 1: if (x < boundleftnb) x = x + lx; break;
    case 2: if (x < boundleftnb) x = x + lx; if (y > boundbacknb) y = y - ly; break;
    case 3: if (y > boundbacknb) y = y - ly; break;
    case 4: if (x > boundrightnb) x = x - lx; if (y > boundbacknb) y = y - ly; break;
    case 5: if (x > boundrightnb) x = x - lx; break;
    case 6: if (x > boundrightnb) x = x - lx; if (y < boundfrontnb) y = y + ly; break;
    case 7: if (y < boundfrontnb) y = y + ly; break;
    case 8: if (x < boundleftnb) x = x + lx; if (y < boundfrontnb) y = y + ly; break;
    default: break;
  }
}
__device__ __forceinline__ double minimg(double a0, double a1, double a2) {
  double m = a0;
  if (fabs(a1) < fabs(m)) m = a1;
  if (fabs(a2) < fabs(m)) m = a2;
  return m;
}

#define COLL_WARPS 4
#define COLL_CAP 64

// snapshot of the collision iteration (anb(:,0), intgr_nwtn_eulr.f90:153-206)
__device__ __forceinline__ void snapshot_particle(const PartGeo &pg, PartBuffers &b, int p) {
  const int np = pg.np;
  const bool m = b.mslv[p] > 0;
  PF(PF_SX) = m ? PF(PF_X) : 0.; PF(PF_SY) = m ? PF(PF_Y) : 0.; PF(PF_SZ) = m ? PF(PF_Z) : 0.;
  PF(PF_SU) = m ? PF(PF_U) : 0.; PF(PF_SV) = m ? PF(PF_V) : 0.; PF(PF_SW) = m ? PF(PF_W) : 0.;
  PF(PF_SOMX) = m ? PF(PF_OMX) : 0.; PF(PF_SOMY) = m ? PF(PF_OMY) : 0.; PF(PF_SOMZ) = m ? PF(PF_OMZ) : 0.;
  // FP32 copy of the snapshot positions for the candidate filter (w: master flag)
  b.pos4[p] = make_float4((float)PF(PF_SX), (float)PF(PF_SY), (float)PF(PF_SZ), m ? 1.f : 0.f);
}
__global__ void k_snapshot(PartGeo pg, PartBuffers b) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p < pg.np) snapshot_particle(pg, b, p);
}

// Uniform cell list of the snapshot positions (one block): cell of every
// particle, counts, exclusive scan, scatter, then every cell's items sorted
// ascending.  Cells are at least 1.01 x the filter distance wide, so every
// partner the FP32 filter accepts lies in the 27 cells around the particle's
// own (periodic in x and y, clamped in z).
__device__ __forceinline__ int coll_cell(const PartGeo &pg, float4 x) {
  int cx = (int)floorf(x.x * pg.cix), cy = (int)floorf(x.y * pg.ciy), cz = (int)floorf(x.z * pg.ciz);
  cx = ((cx % pg.ncx) + pg.ncx) % pg.ncx;
  cy = ((cy % pg.ncy) + pg.ncy) % pg.ncy;
  cz = min(max(cz, 0), pg.ncz - 1);
  return (cz * pg.ncy + cy) * pg.ncx + cx;
}
__global__ void __launch_bounds__(1024) k_cell_build(PartGeo pg, PartBuffers b) {
  const int np = pg.np, ncell = pg.ncx * pg.ncy * pg.ncz, tid = threadIdx.x;
  __shared__ int part[1024];
  for (int q = tid; q < ncell; q += 1024) b.cfill[q] = 0;
  __syncthreads();
  for (int p = tid; p < np; p += 1024) {
    const int c = coll_cell(pg, b.pos4[p]);
    b.ccell[p] = c;
    atomicAdd(&b.cfill[c], 1);
  }
  __syncthreads();
  const int per = (ncell + 1023) / 1024, lo = min(tid * per, ncell), hi = min(lo + per, ncell);
  int sum = 0;
  for (int q = lo; q < hi; ++q) sum += b.cfill[q];
  part[tid] = sum;
  __syncthreads();
  for (int off = 1; off < 1024; off <<= 1) {
    const int v = tid >= off ? part[tid - off] : 0;
    __syncthreads();
    part[tid] += v;
    __syncthreads();
  }
  int run = tid ? part[tid - 1] : 0;
  for (int q = lo; q < hi; ++q) {
    const int n = b.cfill[q];
    b.cstart[q] = run;
    b.cfill[q] = run;
    run += n;
  }
  if (tid == 1023) b.cstart[ncell] = part[1023];
  __syncthreads();
  for (int p = tid; p < np; p += 1024) b.citem[atomicAdd(&b.cfill[b.ccell[p]], 1)] = p;
  __syncthreads();
  for (int q = tid; q < ncell; q += 1024) {  // ascending within the cell
    const int e0 = b.cstart[q], e1 = b.cstart[q + 1];
    for (int i = e0 + 1; i < e1; ++i) {
      const int v = b.citem[i];
      int j = i - 1;
      while (j >= e0 && b.citem[j] > v) { b.citem[j + 1] = b.citem[j]; --j; }
      b.citem[j + 1] = v;
    }
  }
}

// the FP32 periodic-distance filter of the candidate search
__device__ __forceinline__ bool coll_near(float4 q, float pxf, float pyf, float pzf, float lxf, float lyf, float thr2) {
  float dxf = fabsf(q.x - pxf);
  float dyf = fabsf(q.y - pyf);
  const float dzf = q.z - pzf;
  dxf = fminf(dxf, fabsf(lxf - dxf));
  dyf = fminf(dyf, fabsf(lyf - dyf));
  return dxf * dxf + dyf * dyf + dzf * dzf < thr2;
}

// One warp per particle: a coarse FP32 periodic-distance filter selects the
// partners that can interact (lubrication range, contact, or listed in
// firstc), from the 27 cells of the cell list around the particle (or from
// all particles when the grid is narrower than three cells), in ascending
// particle order; lane 0 then walks them in the reference (nb, q) order,
// handles the walls, integrates Newton-Euler and accumulates sumrk3.
__global__ void __launch_bounds__(32 * COLL_WARPS) k_collide_update(PartGeo pg, PartBuffers b, int iter, int rkiter,
                                                                   double dt) {
  __shared__ int cand[COLL_WARPS][COLL_CAP];
  __shared__ int ncand[COLL_WARPS];
  __shared__ int fcs[COLL_WARPS][16];  // the particle's first contact partners (nq <= 15 here)
  const int np = pg.np, nq = pg.nq;
  const int wid = threadIdx.x / 32, lane = threadIdx.x % 32;
  const int p = blockIdx.x * COLL_WARPS + wid;
  if (p >= np) return;
  if (lane == 0) ncand[wid] = 0;
  const double radius = p_rad(pg, p);
  const int qmax0 = b.qmax[p];
  const int *fc = b.firstc + (long)p * nq;
  if (lane < qmax0 && lane < 16) fcs[wid][lane] = fc[lane];
  __syncwarp();
  // FP32 filter distance: 2.1 R (polydisperse: 1.05 (R + Rmax), a superset
  // of every pair's 1.05 (Rp + Rq))
  const float thr = pg.poly ? 1.05f * (float)(radius + pg.rmax) : 2.1f * (float)radius;
  const float thr2 = thr * thr;
  const float lxf = (float)pg.lx, lyf = (float)pg.ly;
  const float4 pp = b.pos4[p];
  const float pxf = pp.x, pyf = pp.y, pzf = pp.z;
  if (pg.ncx >= 3 && pg.ncy >= 3) {
    // cell list: lane t < 27 scans neighbouring cell t; partners in firstc
    // beyond the filter distance are added by the lane of their slot; then
    // the list is sorted ascending (as the full scan produces it)
    if (lane < 27) {
      const int c0 = b.ccell[p];
      const int cx = c0 % pg.ncx, cy = (c0 / pg.ncx) % pg.ncy, cz = c0 / (pg.ncx * pg.ncy);
      const int x = (cx + lane % 3 - 1 + pg.ncx) % pg.ncx, y = (cy + (lane / 3) % 3 - 1 + pg.ncy) % pg.ncy;
      const int z = cz + lane / 9 - 1;
      if (z >= 0 && z < pg.ncz) {
        const int c = (z * pg.ncy + y) * pg.ncx + x;
        for (int t = b.cstart[c]; t < b.cstart[c + 1]; ++t) {
          const int q = b.citem[t];
          const float4 qp = b.pos4[q];
          if (q != p && qp.w != 0.f && coll_near(qp, pxf, pyf, pzf, lxf, lyf, thr2)) {
            const int pos = atomicAdd(&ncand[wid], 1);
            if (pos < COLL_CAP) cand[wid][pos] = q;
          }
        }
      }
    }
    if (lane < qmax0) {
      const int id = fc[lane];
      if (id >= 1 && id <= np) {
        const int q = id - 1;
        const float4 qp = b.pos4[q];
        if (q != p && qp.w != 0.f && b.mslv[q] == id && !coll_near(qp, pxf, pyf, pzf, lxf, lyf, thr2)) {
          const int pos = atomicAdd(&ncand[wid], 1);
          if (pos < COLL_CAP) cand[wid][pos] = q;
        }
      }
    }
    __syncwarp();
    const int n = min(ncand[wid], COLL_CAP);
    const int v0 = lane < n ? cand[wid][lane] : 0, v1 = lane + 32 < n ? cand[wid][lane + 32] : 0;
    int r0 = 0, r1 = 0;
    for (int i = 0; i < n; ++i) {
      const int w = cand[wid][i];
      r0 += w < v0;
      r1 += w < v1;
    }
    __syncwarp();
    if (lane < n) cand[wid][r0] = v0;
    if (lane + 32 < n) cand[wid][r1] = v1;
    __syncwarp();
  } else {
  // candidates in ascending q: within the collision distance or already in
  // contact; four slices of 32 per round, loads issued together
  constexpr int SL = 4;
  for (int base = 0; base < np; base += 32 * SL) {
    float4 qp[SL];
    int qms[SL];
#pragma unroll
    for (int u = 0; u < SL; ++u) {
      const int q = base + 32 * u + lane;
      qp[u] = q < np ? b.pos4[q] : make_float4(0.f, 0.f, 0.f, 0.f);  // w: 1 for masters
      qms[u] = q < np ? b.mslv[q] : 0;
    }
#pragma unroll
    for (int u = 0; u < SL; ++u) {
      const int q = base + 32 * u + lane;
      bool c = false;
      if (q < np && q != p && qp[u].w != 0.f) {
        c = coll_near(qp[u], pxf, pyf, pzf, lxf, lyf, thr2);
        for (int i = 0; i < qmax0 && !c; ++i) c = ((i < 16 ? fcs[wid][i] : fc[i]) == qms[u]);
      }
      const unsigned m = __ballot_sync(0xffffffffu, c);
      if (c) {
        const int pos = ncand[wid] + __popc(m & ((1u << lane) - 1u));
        if (pos < COLL_CAP) cand[wid][pos] = q;
      }
      __syncwarp();
      if (lane == 0) ncand[wid] += __popc(m);
      __syncwarp();
    }
  }
  }
  int nc = ncand[wid];
  if (nc > COLL_CAP) { if (lane == 0) atomicExch(&b.err[0], 1); nc = COLL_CAP; }
  if (b.mslv[p] <= 0) return;
  const int idp = b.mslv[p];
  const double rkab = pg.rkab[rkiter - 1];
  const int itermax = 1;
  PState S;
  S.u = PF(PF_U); S.v = PF(PF_V); S.w = PF(PF_W); S.omx = PF(PF_OMX); S.omy = PF(PF_OMY); S.omz = PF(PF_OMZ);
  S.colfx = 0.; S.colfy = 0.; S.colfz = 0.;
  const double px = PF(PF_X), py = PF(PF_Y), pz = PF(PF_Z);
  int qlast = b.qmax[p];
  int *fcw = b.firstc + (long)p * nq, *ofcw = b.ofirstc + (long)p * nq;
  // (i) other particles, nb-outer / q-inner as in the reference.  The 32
  // lanes evaluate the geometry and the lubrication force f1 of 32 (copy,
  // candidate) pairs at a time; lane 0 then takes them in the reference's
  // order for the force sums, the contact bookkeeping and the collision
  // forces, with the same arithmetic as a sequential pass.
  const int npair = pg.nb_copies * nc;
  for (int base = 0; base < npair; base += 32) {
    const int k = base + lane;
    int q = 0, idq = 0, use = 0, lub = 0;
    double dist = 0., deltax = 0., deltay = 0., deltaz = 0., nx = 0., ny = 0., nz = 0., f1 = 0.;
    double qu = 0., qv = 0., qw = 0.;
    if (k < npair) {
      const int nb = k / nc, ci = k - nb * nc;
      q = cand[wid][ci];
      use = idp != b.mslv[q] && b.mslv[q] > 0;
      if (use) {
        idq = b.mslv[q];
        double qx = b.pf[(long)PF_SX * np + q], qy = b.pf[(long)PF_SY * np + q];
        const double qz = b.pf[(long)PF_SZ * np + q];
        copy_shift_coll(nb, pg.lx, pg.ly, qx, qy);
        deltaz = qz - pz;
        deltax = minimg(qx - px, qx - pg.lx - px, qx + pg.lx - px);
        deltay = minimg(qy - py, qy - pg.ly - py, qy + pg.ly - py);
        dist = sqrt(deltax * deltax + deltay * deltay + deltaz * deltaz);
        nx = deltax / dist; ny = deltay / dist; nz = deltaz / dist;
        // polydisperse: contact at the sum of the radii, eps and the
        // lubrication prefactor with the equivalent radius (pair_consts)
        const double rqq = p_rad(pg, q);
        const double rsum = pg.poly ? radius + rqq : 2. * radius;
        const double re = pg.poly ? 2. * radius * rqq / (radius + rqq) : radius;
        const double eps = (dist - rsum) / re;
        qu = b.pf[(long)PF_SU * np + q]; qv = b.pf[(long)PF_SV * np + q]; qw = b.pf[(long)PF_SW * np + q];
        if ((eps < 0.025) && (eps > 0.)) {
          lub = 1;
          f1 = d_lub_f1(pg, S.u, S.v, S.w, idq, nx, ny, nz, eps, qu, qv, qw,
                        pg.poly ? 6. * IBM_PI * pg.visc * re : pg.coeff_f);
        }
      }
    }
    const int cnt = min(32, npair - base);
    for (int j = 0; j < cnt; ++j) {
      const int juse = __shfl_sync(0xffffffffu, use, j);
      if (!juse) continue;  // uniform across the warp
      const int jq = __shfl_sync(0xffffffffu, q, j), jidq = __shfl_sync(0xffffffffu, idq, j);
      const int jlub = __shfl_sync(0xffffffffu, lub, j);
      const double jdist = __shfl_sync(0xffffffffu, dist, j);
      const double jdx = __shfl_sync(0xffffffffu, deltax, j), jdy = __shfl_sync(0xffffffffu, deltay, j),
                   jdz = __shfl_sync(0xffffffffu, deltaz, j);
      const double jnx = __shfl_sync(0xffffffffu, nx, j), jny = __shfl_sync(0xffffffffu, ny, j),
                   jnz = __shfl_sync(0xffffffffu, nz, j);
      const double jf1 = __shfl_sync(0xffffffffu, f1, j);
      const double jqu = __shfl_sync(0xffffffffu, qu, j), jqv = __shfl_sync(0xffffffffu, qv, j),
                   jqw = __shfl_sync(0xffffffffu, qw, j);
      if (lane != 0) continue;
      if (jlub) {
        S.colfx = S.colfx + jf1 * jnx;
        S.colfy = S.colfy + jf1 * jny;
        S.colfz = S.colfz + jf1 * jnz;
      }
      int qq = 0;
      const int qm = b.qmax[p];
      const double jrsum = pg.poly ? radius + pg.prad[jq] : 2. * radius;
      for (int i = 1; i <= qm; ++i) {
        if (jidq == fcw[i - 1]) {
          if (jdist < jrsum) {
            qq = i;
            d_collisions(pg, b, p, S, qq, jidq, jdist, jdx, jdy, jdz, jqu, jqv, jqw,
                         b.pf[(long)PF_SOMX * np + jq], b.pf[(long)PF_SOMY * np + jq], b.pf[(long)PF_SOMZ * np + jq],
                         dt, rkab);
          } else if (iter == itermax) {
            d_remove_contact(pg, b, p, i, qlast);
          }
        }
      }
      if (qq == 0 && jdist < jrsum) {
        qlast = qlast + 1;
        if (qlast > nq) {  // overflow: flagged, the pair's update skipped
          atomicExch(&b.err[1], 1);
          qlast = nq;
          continue;
        }
        qq = qlast;
        d_new_contact(pg, b, p, qq);
        d_collisions(pg, b, p, S, qq, jidq, jdist, jdx, jdy, jdz, jqu, jqv, jqw,
                     b.pf[(long)PF_SOMX * np + jq], b.pf[(long)PF_SOMY * np + jq], b.pf[(long)PF_SOMZ * np + jq],
                     dt, rkab);
        fcw[qlast - 1] = jidq;
        ofcw[qlast - 1] = jidq;
      }
      b.qmax[p] = qlast;
    }
  }
  if (lane != 0) return;
  // (ii) walls (intgr_nwtn_eulr.f90:503-603)
  const int botw = np + 1, topw = np + 2;
  const int qm_w = b.qmax[p];
  for (int qw_ = botw; qw_ <= topw; ++qw_) {
    const int idq = qw_;
    if (pg.zper) break;  // periodic z: no walls
    const double deltax = 0., deltay = 0., deltaz = (qw_ - botw) * pg.lz - pz;
    const double dist = sqrt(deltax * deltax + deltay * deltay + deltaz * deltaz);
    const double deltan = radius - dist;
    const double nx = deltax / dist, ny = deltay / dist, nz = deltaz / dist;
    int qq = 0;
    const double eps = -deltan / radius;
    if ((eps < 0.075) && (eps > 0.))
      d_lubrication(pg, S.u, S.v, S.w, idq, nx, ny, nz, eps, 0., 0., 0.,
                    pg.poly ? 6. * IBM_PI * pg.visc * radius : pg.coeff_f, S.colfx, S.colfy, S.colfz);
    for (int i = 1; i <= qm_w; ++i) {
      if (idq == fcw[i - 1]) {
        qq = i;
        if (dist < radius) {
          d_collisions(pg, b, p, S, qq, idq, dist, deltax, deltay, deltaz, 0., 0., 0., 0., 0., 0., dt, rkab);
        } else if (iter == itermax) {
          d_remove_contact(pg, b, p, i, qlast);
        }
      }
    }
    if ((qq == 0) && (dist < radius)) {
      qlast = qlast + 1;
      if (qlast > nq) { atomicExch(&b.err[1], 1); qlast = nq; continue; }
      qq = qlast;
      d_new_contact(pg, b, p, qq);
      d_collisions(pg, b, p, S, qq, idq, dist, deltax, deltay, deltaz, 0., 0., 0., 0., 0., 0., dt, rkab);
      fcw[qlast - 1] = idq;
      ofcw[qlast - 1] = idq;
    }
  }
  b.qmax[p] = qlast;
  // Newton-Euler (intgr_nwtn_eulr.f90:611-667); colflg is reset to 0 first
  const double colflgx = 0., colflgy = 0., colflgz = 0.;
  const double vol = p_vol(pg, p), rr = pg.ratiorho;  // ap%vol, ap%ratiorho (coordsfp.f90:96-102)
  const double vr = vol * rr;
  const double ou = PF(PF_OU), ov = PF(PF_OV), ow = PF(PF_OW);
  double nu = ou + (1 - colflgx) * ((-1.) * dt * (PF(PF_FXLTOT)) / vr + (PF(PF_INTU) - PF(PF_OINTU)) / vr) +
              rkab * dt * pg.gacc[0] * (1. - (1. / rr)) + rkab * 0.5 * dt * (S.colfx + PF(PF_OCOLFX)) / vr;
  PF(PF_X) = PF(PF_OX) + rkab * 0.5 * dt * (nu + ou);
  double nv = ov + (1 - colflgy) * ((-1.) * dt * (PF(PF_FYLTOT)) / vr + (PF(PF_INTV) - PF(PF_OINTV)) / vr) +
              rkab * dt * pg.gacc[1] * (1. - (1. / rr)) + rkab * 0.5 * dt * (S.colfy + PF(PF_OCOLFY)) / vr;
  PF(PF_Y) = PF(PF_OY) + rkab * 0.5 * dt * (nv + ov);
  double nw = ow + (1 - colflgz) * ((-1.) * dt * (PF(PF_FZLTOT)) / vr + (PF(PF_INTW) - PF(PF_OINTW)) / vr) +
              rkab * dt * pg.gacc[2] * (1. - (1. / rr)) + rkab * 0.5 * dt * (S.colfz + PF(PF_OCOLFZ)) / vr;
  PF(PF_Z) = PF(PF_OZ) + rkab * 0.5 * dt * (nw + ow);
  PF(PF_U) = nu; PF(PF_V) = nv; PF(PF_W) = nw;
  PF(PF_COLFX) = S.colfx; PF(PF_COLFY) = S.colfy; PF(PF_COLFZ) = S.colfz;
  PF(PF_COLTX) = 0.; PF(PF_COLTY) = 0.; PF(PF_COLTZ) = 0.;
  double omx, omy, omz;
  if (pg.rotation) {
    const double mr = p_mi(pg, p) * rr;
    omx = PF(PF_OOMX) + (-1.) * dt * PF(PF_TQX) / mr + (PF(PF_INTOMX) - PF(PF_OINTOMX)) / mr +
          rkab * 0.5 * dt * (PF(PF_COLTX) + PF(PF_OCOLTX)) / mr;
    omy = PF(PF_OOMY) + (-1.) * dt * PF(PF_TQY) / mr + (PF(PF_INTOMY) - PF(PF_OINTOMY)) / mr +
          rkab * 0.5 * dt * (PF(PF_COLTY) + PF(PF_OCOLTY)) / mr;
    omz = PF(PF_OOMZ) + (-1.) * dt * PF(PF_TQZ) / mr + (PF(PF_INTOMZ) - PF(PF_OINTOMZ)) / mr +
          rkab * 0.5 * dt * (PF(PF_COLTZ) + PF(PF_OCOLTZ)) / mr;
  } else {
    omx = 0.0; omy = 0.0; omz = 0.0;
  }
  PF(PF_OMX) = omx; PF(PF_OMY) = omy; PF(PF_OMZ) = omz;
  const double phi = PF(PF_OPHI) + 0.5 * rkab * dt * (omz + PF(PF_OOMZ));
  PF(PF_PHI) = phi;
  const double omtheta = (omy * cos(phi)) - (omx * sin(phi));
  PF(PF_OMTHETA) = omtheta;
  PF(PF_THETA) = PF(PF_OTHETA) + rkab * 0.5 * dt * (omtheta + PF(PF_OOMTHETA));
  // sumrk3 (intgr_nwtn_eulr.f90:1586-1669)
  double *r = b.rkp + (long)p * RK_N;
  if (rkiter == 1)
    for (int t = 0; t < RK_N; ++t) r[t] = 0.;
  const double dpdy_new = 0.;
  r[RK_FX] = r[RK_FX] + (-1.) * PF(PF_FXLTOT) + (PF(PF_INTU) - PF(PF_OINTU)) / dt;
  r[RK_FY] = r[RK_FY] + (-1.) * PF(PF_FYLTOT) + (PF(PF_INTV) - PF(PF_OINTV)) / dt;
  r[RK_FZ] = r[RK_FZ] + (-1.) * PF(PF_FZLTOT) + (PF(PF_INTW) - PF(PF_OINTW)) / dt;
  r[RK_TX] = r[RK_TX] + (-1.) * PF(PF_TQX) + (PF(PF_INTOMX) - PF(PF_OINTOMX)) / dt;
  r[RK_TY] = r[RK_TY] + (-1.) * PF(PF_TQY) + (PF(PF_INTOMY) - PF(PF_OINTOMY)) / dt;
  r[RK_TZ] = r[RK_TZ] + (-1.) * PF(PF_TQZ) + (PF(PF_INTOMZ) - PF(PF_OINTOMZ)) / dt;
  r[RK_TT] = r[RK_TT] + (-1.) * (-dpdy_new * p_dvl(pg, p));
  r[RK_CFX] = r[RK_CFX] + 0.5 * rkab * (S.colfx + PF(PF_OCOLFX));
  r[RK_CFY] = r[RK_CFY] + 0.5 * rkab * (S.colfy + PF(PF_OCOLFY));
  r[RK_CFZ] = r[RK_CFZ] + 0.5 * rkab * (S.colfz + PF(PF_OCOLFZ));
  r[RK_CTX] = r[RK_CTX] + 0.5 * rkab * (PF(PF_COLTX) + PF(PF_OCOLTX));
  r[RK_CTY] = r[RK_CTY] + 0.5 * rkab * (PF(PF_COLTY) + PF(PF_OCOLTY));
  r[RK_CTZ] = r[RK_CTZ] + 0.5 * rkab * (PF(PF_COLTZ) + PF(PF_OCOLTZ));
  r[RK_DUDT] = r[RK_DUDT] + (nu - ou) / dt;
  r[RK_DVDT] = r[RK_DVDT] + (nv - ov) / dt;
  r[RK_DWDT] = r[RK_DWDT] + (nw - ow) / dt;
}

int launch_collide_update(cudaStream_t s, const PartGeo &pg, PartBuffers b, int iter, int rkiter, double dt,
                          bool snapshot) {
  if (pg.np == 0) return 0;
  int n = 1;
  if (snapshot) { k_snapshot<<<(pg.np + 127) / 128, 128, 0, s>>>(pg, b); ++n; }
  if (pg.ncx >= 3 && pg.ncy >= 3) { k_cell_build<<<1, 1024, 0, s>>>(pg, b); ++n; }
  k_collide_update<<<(pg.np + COLL_WARPS - 1) / COLL_WARPS, 32 * COLL_WARPS, 0, s>>>(pg, b, iter, rkiter, dt);
  return n;
}

// ---------------------------------------------------------------------------
// periodic correction (:702-714), neighbour flags (:1051-1090, one rank) and
// new Lagrangian points with their rigid-body velocity (:1438-1485).
// One block per particle; the compaction of points flagged `isout` keeps the
// reference order.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_ne_finalize(PartGeo pg, PartBuffers b, IbmBuffers ib, int init) {
  const int np = pg.np;
  const int p = blockIdx.x;
  __shared__ double sx, sy, sz, su, sv, sw, somx, somy, somz;
  __shared__ int wcount[32];
  __shared__ int base;
  // init: 0 = after Newton-Euler, 1 = initial set-up (initparticles +
  // coordsfp), 2 = Lagrangian points only (restart with given flags)
  if (threadIdx.x == 0) {
    if (init == 1) b.mslv[p] = p + 1;
    double x = PF(PF_X), y = PF(PF_Y);
    if (b.mslv[p] > 0 && init == 0) {
      if (x > pg.lx) x = x - pg.lx;
      if (x < 0.) x = x + pg.lx;
      if (y > pg.ly) y = y - pg.ly;
      if (y < 0.) y = y + pg.ly;
      PF(PF_X) = x; PF(PF_Y) = y;
      if (pg.zper) {  // periodic z: the same correction along z
        double z = PF(PF_Z);
        if (z > pg.lz) z = z - pg.lz;
        if (z < 0.) z = z + pg.lz;
        PF(PF_Z) = z;
      }
    }
    const double ro = p_rad(pg, p) + pg.offset;
    const double leftb = 0., rightb = pg.lx, frontb = 0., backb = pg.ly;
    int *nbf = b.nb + (long)p * 9;
    if (init != 2) {
    for (int n = 0; n < 9; ++n) nbf[n] = 0;
    double dist;
    if (x > (rightb - ro)) nbf[1] = 1;
    dist = sqrt((rightb - x) * (rightb - x) + (frontb - y) * (frontb - y));
    if (fabs(dist) < ro) nbf[2] = 1;
    if (y < (frontb + ro)) nbf[3] = 1;
    dist = sqrt((leftb - x) * (leftb - x) + (frontb - y) * (frontb - y));
    if (fabs(dist) < ro) nbf[4] = 1;
    if (x < (leftb + ro)) nbf[5] = 1;
    dist = sqrt((leftb - x) * (leftb - x) + (backb - y) * (backb - y));
    if (fabs(dist) < ro) nbf[6] = 1;
    if (y > (backb - ro)) nbf[7] = 1;
    dist = sqrt((rightb - x) * (rightb - x) + (backb - y) * (backb - y));
    if (fabs(dist) < ro) nbf[8] = 1;
    }
    if (init == 0) {
      double *r = b.rkp + (long)p * RK_N;
      r[RK_DOMX] = 0.; r[RK_DOMY] = 0.; r[RK_DOMZ] = 0.;
    }
    sx = x; sy = y; sz = PF(PF_Z); su = PF(PF_U); sv = PF(PF_V); sw = PF(PF_W);
    somx = PF(PF_OMX); somy = PF(PF_OMY); somz = PF(PF_OMZ);
    base = 0;
  }
  __syncthreads();
  // nl: the per-particle capacity of the Lagrangian arrays; the sphere's
  // own point count, table offset and shell radius when polydisperse
  const int nl = pg.nl, nlp = p_nl(pg, p), nt = pg.ntab;
  const double radfp = p_radfp(pg, p);
  const double *sct = b.sincos + p_toff(pg, p);
  const int wid = threadIdx.x / 32, lane = threadIdx.x % 32;
  const float lxf = (float)pg.lx, lyf = (float)pg.ly;
  for (int l0 = 0; l0 < nlp; l0 += blockDim.x) {
    const int l = l0 + threadIdx.x;
    bool keep = false;
    double xfploc = 0, yfploc = 0, zfploc = 0, rx = 0, ry = 0, rz = 0;
    if (l < nlp && b.mslv[p] != 0) {
      const double st = sct[l], ct = sct[nt + l], sp = sct[2 * nt + l], cp = sct[3 * nt + l];
      // offsets from the centre, radfp*st*cp etc. with the reference's
      // rounding; they also serve as (xfp - xc) in the point velocities
      const double rst = radfp * st;
      rx = rst * cp;
      ry = rst * sp;
      rz = radfp * ct;
      xfploc = sx + rx;
      yfploc = sy + ry;
      zfploc = sz + rz;
      // isout (periodic image outside 1..I, 1..J) is impossible for points
      // within half a domain of it: an FP32 screen decides those, the
      // reference's FP64 test the rest
      const float xf = (float)xfploc, yf = (float)yfploc;
      bool isout = false;
      if (!(xf > -0.4f * lxf && xf < 1.4f * lxf && yf > -0.4f * lyf && yf < 1.4f * lyf)) {
        double isperiodx = 0., isperiody = 0.;
        if (xfploc < 0. + 0.5 * pg.dx) isperiodx = 1.;
        if (xfploc >= pg.lx + 0.5 * pg.dx) isperiodx = -1.;
        if (yfploc < 0. + 0.5 * pg.dy) isperiody = 1.;
        if (yfploc >= pg.ly + 0.5 * pg.dy) isperiody = -1.;
        const double coorxfp = (xfploc + isperiodx * pg.lx - 0.) * pg.dxi;
        if (fnint(coorxfp) < 1 || fnint(coorxfp) > pg.I) isout = true;
        const double cooryfp = (yfploc + isperiody * pg.ly - 0.) * pg.dyi;
        if (fnint(cooryfp) < 1 || fnint(cooryfp) > pg.J) isout = true;
      }
      keep = !isout;
    }
    const unsigned m = __ballot_sync(0xffffffffu, keep);
    if (lane == 0) wcount[wid] = __popc(m);
    __syncthreads();
    int off = base;
    for (int q = 0; q < wid; ++q) off += wcount[q];
    off += __popc(m & ((1u << lane) - 1u));
    if (keep) {
      const long t = (long)p * nl + off;
      ib.xfp[t] = xfploc; ib.yfp[t] = yfploc; ib.zfp[t] = zfploc;
      ib.ul[t] = su + somy * rz - somz * ry;
      ib.vl[t] = sv + somz * rx - somx * rz;
      ib.wl[t] = sw + somx * ry - somy * rx;
    }
    __syncthreads();
    if (threadIdx.x == 0) for (int q = 0; q < (int)(blockDim.x / 32); ++q) base += wcount[q];
    __syncthreads();
  }
  if (threadIdx.x == 0) ib.nla[p] = b.mslv[p] != 0 ? base : 0;
}

void launch_ne_finalize(cudaStream_t s, const PartGeo &pg, PartBuffers b, IbmBuffers ib, int init) {
  if (pg.np == 0) return;
  k_ne_finalize<<<pg.np, 256, 0, s>>>(pg, b, ib, init);
}

}  // namespace ibmk
