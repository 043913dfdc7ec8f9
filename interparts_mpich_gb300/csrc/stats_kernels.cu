// stats_kernels.cu -- plane statistics of post1d (output.f90:13-917) and the
// phase indicator it calls (phase_indicator.f90:11-559), one rank.
//
// Phase indicator.  The reference loops over particles p, their copies
// nb = 0..8 and the cells of each copy's box, keeping per cell the largest
// solid fraction and the rigid-body velocity of the candidate that set it
// last.  Here every (particle, grid) pair is one block and the sequential
// "last writer" is recovered from two order-independent maxima:
//   pass 0: G[cell] = max over candidates of the key (inner cell: +inf bits,
//           otherwise the fraction's bits; positive doubles order as their
//           bit patterns);
//   pass 1: W[cell] = max over the candidates whose key equals G[cell] of
//           q+1 for inner candidates (the reference overwrites: the last
//           one, the largest q = 9p + nb, wins) or 9np+1-q for fractions
//           (strict ">": the first one wins).
// The fraction is 1 - the decoded G; the velocity is evaluated from the
// winner when it is read.  The corner fractions use the reference's
// operation order without FMA contraction (this file is compiled with
// -fmad=false), so they are bit-identical; cells whose eight corners all lie
// outside (inside) the sphere are decided from the nearest (farthest) corner
// alone, which gives the same 0 (1) exactly.
//
// Plane sums.  One block per (plane, slice of the plane) accumulates the 32
// sums of output.f90:88-355 in FP64 and writes them to a partials array; the
// host adds the slices in a fixed order and applies the ghost values and
// normalisations (O(ktot)).
#include "kernels.cuh"

namespace ibmk {

struct PhaseCell {
  double xmn, xpl, ymn, ypl, zmn, zpl;
};
// corner planes of cell (i,j,k) (1-based) of grid c = u, v, w, p
// (phase_indicator.f90:268-274, 315-321, 362-368, 409-415)
__device__ __forceinline__ PhaseCell phase_cell(int c, int i, int j, int k, double dx, double dy, double dz) {
  PhaseCell r;
  if (c == 0) { r.xmn = (i - 0.5) * dx; r.xpl = (i + 0.5) * dx; }
  else { r.xmn = (i - 1) * dx; r.xpl = i * dx; }
  if (c == 1) { r.ymn = (j - 0.5) * dy; r.ypl = (j + 0.5) * dy; }
  else { r.ymn = (j - 1) * dy; r.ypl = j * dy; }
  if (c == 2) { r.zmn = (k - 0.5) * dz; r.zpl = (k + 0.5) * dz; }
  else { r.zmn = (k - 1) * dz; r.zpl = k * dz; }
  return r;
}

// key of one candidate (0: no candidate): inner cells of the reference's
// dist2 < radin2 test, else the corner fraction sum1/sum2 when positive
__device__ __forceinline__ unsigned long long phase_key(const PhaseCell &e, double cx, double cy, double cz,
                                                        double radius, double radin2, double rthr) {
  const double dxp2 = (e.xpl - cx) * (e.xpl - cx), dyp2 = (e.ypl - cy) * (e.ypl - cy),
               dzp2 = (e.zpl - cz) * (e.zpl - cz);
  const double dist2 = dxp2 + dyp2 + dzp2;
  if (dist2 < radin2) return PH_INNER;
  const double dxm2 = (e.xmn - cx) * (e.xmn - cx), dym2 = (e.ymn - cy) * (e.ymn - cy),
               dzm2 = (e.zmn - cz) * (e.zmn - cz);
  // nearest corner at or beyond the sphere: every signed distance <= 0
  if (fmin(dxm2, dxp2) + fmin(dym2, dyp2) + fmin(dzm2, dzp2) >= rthr) return 0ull;
  // farthest corner inside: every signed distance > 0, sum1 == sum2
  if (fmax(dxm2, dxp2) + fmax(dym2, dyp2) + fmax(dzm2, dzp2) < rthr) return (unsigned long long)__double_as_longlong(1.0);
  double sg[8];
  sg[0] = radius - sqrt(dxm2 + dym2 + dzm2);
  sg[1] = radius - sqrt(dxm2 + dyp2 + dzm2);
  sg[2] = radius - sqrt(dxp2 + dyp2 + dzm2);
  sg[3] = radius - sqrt(dxp2 + dym2 + dzm2);
  sg[4] = radius - sqrt(dxm2 + dym2 + dzp2);
  sg[5] = radius - sqrt(dxm2 + dyp2 + dzp2);
  sg[6] = radius - sqrt(dxp2 + dyp2 + dzp2);
  sg[7] = radius - sqrt(dxp2 + dym2 + dzp2);
  double s1 = 0., s2 = 0.;
#pragma unroll
  for (int q = 0; q < 8; ++q) {
    if (sg[q] > 0.) s1 = s1 + sg[q];
    s2 = s2 + fabs(sg[q]);
  }
  const double f = s1 / s2;
  return f > 0. ? (unsigned long long)__double_as_longlong(f) : 0ull;
}

// shift of self-neighbour copy nbrecv (phase_indicator.f90:90-118)
__device__ __forceinline__ void phase_copy_shift(int nbrecv, double lx, double ly, double &x, double &y) {
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

template <int PASS>
__global__ void __launch_bounds__(256) k_phase_mark(Geo g, PartGeo pg, PartBuffers b, PhaseBuffers ph, int itype) {
  const int np = pg.np, p = blockIdx.x, c = blockIdx.y;
  if (b.mslv[p] <= 0) return;
  // itype 0 updates only the pressure cells; itype 1 needs no winner there
  if (itype == 0 && c < 3) return;
  if (PASS == 1 && itype == 1 && c == 3) return;
  const double dx = 1. / g.dxi, dy = 1. / g.dyi, dz = 1. / g.dzi;
  const double radius = pg.radius, radin = radius - 2. * dx, radin2 = radin * radin;
  const long plane = (long)g.I * g.J, nc = plane * g.K;
  unsigned long long *G = ph.G + c * nc;
  int *W = ph.W + c * nc;
  const int bigq = 9 * np + 1;
  for (int nb = 0; nb <= 8; ++nb) {
    if (nb > 0 && b.nb[(long)p * 9 + nb] != 1) continue;
    int nbrecv = nb;
    if (nb > 0) { nbrecv = nb + 4; if (nbrecv > 8) nbrecv -= 8; }
    double cx = b.pf[(long)PF_X * np + p], cy = b.pf[(long)PF_Y * np + p];
    const double cz = b.pf[(long)PF_Z * np + p];
    phase_copy_shift(nbrecv, g.lx, g.ly, cx, cy);
    int ilow = fnint((cx - radius) * g.dxi - 2.), ihigh = fnint((cx + radius) * g.dxi + 2.);
    int jlow = fnint((cy - radius) * g.dyi - 2.), jhigh = fnint((cy + radius) * g.dyi + 2.);
    int klow = fnint((cz - radius) * g.dzi - 2.), khigh = fnint((cz + radius) * g.dzi + 2.);
    if (ilow < 1) ilow = 1;
    if (jlow < 1) jlow = 1;
    if (klow < 1) klow = 1;
    if (ihigh > g.I) ihigh = g.I;
    if (jhigh > g.J) jhigh = g.J;
    if (khigh > g.K) khigh = g.K;
    const int ni = ihigh - ilow + 1, nj = jhigh - jlow + 1, nk = khigh - klow + 1;
    if (ni <= 0 || nj <= 0 || nk <= 0) continue;
    const int ncell = ni * nj * nk;
    const int qid = p * 9 + nb;
    for (int e = threadIdx.x; e < ncell; e += blockDim.x) {
      const int kk = e / (ni * nj), r = e - kk * ni * nj, jj = r / ni, ii = r - jj * ni;
      const int i = ilow + ii, j = jlow + jj, k = klow + kk;
      const unsigned long long key = phase_key(phase_cell(c, i, j, k, dx, dy, dz), cx, cy, cz, radius, radin2, pg.rthr);
      if (key == 0ull) continue;
      const long cell = (long)(k - 1) * plane + (long)(j - 1) * g.I + (i - 1);
      if (PASS == 0) {
        atomicMax(&G[cell], key);
      } else if (key == G[cell]) {
        atomicMax(&W[cell], key == PH_INNER ? qid + 1 : bigq - qid);
      }
    }
  }
}

void launch_phase_indicator(cudaStream_t s, const Geo &g, const PartGeo &pg, PartBuffers b, PhaseBuffers ph,
                            int itype) {
  const long nc = (long)g.I * g.J * g.K;
  cudaMemsetAsync(ph.G, 0, 4 * nc * sizeof(unsigned long long), s);
  cudaMemsetAsync(ph.W, 0, 4 * nc * sizeof(int), s);
  if (pg.np == 0) return;
  k_phase_mark<0><<<dim3(pg.np, 4), 256, 0, s>>>(g, pg, b, ph, itype);
  k_phase_mark<1><<<dim3(pg.np, 4), 256, 0, s>>>(g, pg, b, ph, itype);
}

// one phase field (f = gamu, gamv, gamw, gamp, upart, vpart, wpart) in the
// reference layout (0:i1,0:j1,0:k1)
__global__ void k_phase_export(PhaseView v, int f, double *__restrict__ out) {
  const long ni = v.I + 2, nj = v.J + 2, n = ni * nj * (v.K + 2);
  for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < n; e += (long)gridDim.x * blockDim.x) {
    const int k = (int)(e / (ni * nj));
    const long r = e - k * ni * nj;
    const int j = (int)(r / ni), i = (int)(r - j * ni);
    const int iw = i == 0 ? v.I : (i == v.I + 1 ? 1 : i);
    const int jw = j == 0 ? v.J : (j == v.J + 1 ? 1 : j);
    out[e] = f < 4 ? v.gam(f, iw, jw, k) : v.part(f - 4, iw, jw, k);
  }
}
void launch_phase_export(cudaStream_t s, const PhaseView &v, int f, double *out) {
  k_phase_export<<<1216, 256, 0, s>>>(v, f, out);
}

// ---------------------------------------------------------------------------
// plane sums of post1d
// ---------------------------------------------------------------------------
template <typename T>
struct StatFields {
  const T *u, *v, *w;
  const double *p;                     // FP64 pressure, or
  const float *phi, *plo;              // double-float pressure (mixed form)
  const double *c;                     // scalar, or null (zero)
  __device__ __forceinline__ double pr(long o) const {
    return p ? p[o] : (double)phi[o] + (double)plo[o];
  }
};

template <typename T>
__global__ void __launch_bounds__(256) k_post1d_sums(Geo g, PhaseView ph, StatFields<T> F, double kappa,
                                                     double *__restrict__ part, int slices) {
  const int k = blockIdx.x + 1, sl = blockIdx.y;
  const int I = g.I, J = g.J;
  const long nxy = (long)I * J;
  const long per = (nxy + slices - 1) / slices;
  const long e0 = sl * per, e1 = min(nxy, e0 + per);
  double s[POST1D_NSUM];
#pragma unroll
  for (int q = 0; q < POST1D_NSUM; ++q) s[q] = 0.;
  const bool parts = ph.parts;
  const double dzi = g.dzi;
  for (long e = e0 + threadIdx.x; e < e1; e += blockDim.x) {
    const int j0 = (int)(e / I), i0 = (int)(e - (long)j0 * I);
    const int i = i0 + 1, j = j0 + 1;
    const int ip = i == I ? 1 : i + 1, jp = j == J ? 1 : j + 1;
    const long o = fidx(g, i0, j0, k), oi = fidx(g, ip - 1, j0, k), oj = fidx(g, i0, jp - 1, k),
               ok = fidx(g, i0, j0, k + 1);
    const double u = F.u[o], v = F.v[o], w = F.w[o], pp = F.pr(o);
    const double cc = F.c ? F.c[o] : 0., ck = F.c ? F.c[ok] : 0.;
    const double gu = ph.gam(0, i, j, k), gv = ph.gam(1, i, j, k), gw = ph.gam(2, i, j, k), gp = ph.gam(3, i, j, k);
    const double pu = ph.part(0, i, j, k), pv = ph.part(1, i, j, k), pw = ph.part(2, i, j, k);
    // output.f90:103-123
    if (parts) {
      s[0] += u * gu; s[1] += v * gv; s[2] += w * gw; s[3] += pp * gp; s[4] += cc * gp;
    } else {
      s[0] += u * (1. - gu); s[1] += v * (1. - gv); s[2] += w * (1. - gw); s[3] += pp * (1. - gp);
      s[4] += cc * (1. - gp);
    }
    s[5] += pu * (1. - gu); s[6] += pv * (1. - gv); s[7] += pw * (1. - gw);
    s[8] += gu; s[9] += gv; s[10] += gw; s[11] += gp;
    // output.f90:218-235
    if (parts) {
      s[12] += u * u * gu; s[13] += v * v * gv; s[14] += w * w * gw; s[15] += pp * pp * gp;
      s[16] += cc * cc * gp;
    } else {
      s[12] += u * u * (1. - gu); s[13] += v * v * (1. - gv); s[14] += w * w * (1. - gw);
      s[15] += pp * pp * (1. - gp); s[16] += cc * cc * (1. - gp);
    }
    s[17] += pu * pu * (1. - gu); s[18] += pv * pv * (1. - gv); s[19] += pw * pw * (1. - gw);
    s[20] += gp * gp;
    // output.f90:316-352
    const double uj = F.u[oj], uk = F.u[ok], vi = F.v[oi], vk = F.v[ok], wi = F.w[oi], wj = F.w[oj];
    const double guj = ph.gam(0, i, jp, k), guk = ph.gam(0, i, j, k + 1), gvi = ph.gam(1, ip, j, k),
                 gvk = ph.gam(1, i, j, k + 1), gwi = ph.gam(2, ip, j, k), gwj = ph.gam(2, i, jp, k);
    s[21] += 0.25 * (uj + u) * (vi + v) * (0.25 * (guj + gu + gvi + gv));
    s[22] += 0.25 * (uk + u) * (wi + w) * (0.25 * (guk + gu + gwi + gw));
    s[23] += 0.25 * (vk + v) * (wj + w) * (0.25 * (gvk + gv + gwj + gw));
    s[24] += 0.5 * (ck + cc) * w * (1 - gw);
    s[25] -= kappa * (ck - cc) * dzi;
    const double puj = ph.part(0, i, jp, k), puk = ph.part(0, i, j, k + 1), pvi = ph.part(1, ip, j, k),
                 pvk = ph.part(1, i, j, k + 1), pwi = ph.part(2, ip, j, k), pwj = ph.part(2, i, jp, k);
    s[26] += 0.25 * (puj + pu) * (pvi + pv) * (0.25 * (2. - guj - gu + 2. - gvi - gv));
    s[27] += 0.25 * (puk + pu) * (pwi + pw) * (0.25 * (2. - guk - gu + 2. - gwi - gw));
    s[28] += 0.25 * (pvk + pv) * (pwj + pw) * (0.25 * (2. - gvk - gv + 2. - gwj - gw));
    s[29] += 0.25 * (guj + gu + (gvi + gv));
    s[30] += 0.25 * (guk + gu + (gwi + gw));
    s[31] += 0.25 * (gvk + gv + (gwj + gw));
  }
  __shared__ double red[8][POST1D_NSUM];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int q = 0; q < POST1D_NSUM; ++q) {
    double x = s[q];
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) x += __shfl_down_sync(0xffffffffu, x, d);
    if (lane == 0) red[wid][q] = x;
  }
  __syncthreads();
  if (threadIdx.x < POST1D_NSUM) {
    double x = 0.;
    for (int w8 = 0; w8 < (int)(blockDim.x >> 5); ++w8) x += red[w8][threadIdx.x];
    part[((long)blockIdx.x * slices + sl) * POST1D_NSUM + threadIdx.x] = x;
  }
}

template <typename T>
void launch_post1d_sums(cudaStream_t s, const Geo &g, const PhaseView &ph, const T *u, const T *v, const T *w,
                        const double *p, const float *phi, const float *plo, const double *c, double kappa,
                        double *part, int slices) {
  StatFields<T> F{u, v, w, p, phi, plo, c};
  k_post1d_sums<T><<<dim3(g.K, slices), 256, 0, s>>>(g, ph, F, kappa, part, slices);
}
template void launch_post1d_sums<double>(cudaStream_t, const Geo &, const PhaseView &, const double *, const double *,
                                         const double *, const double *, const float *, const float *,
                                         const double *, double, double *, int);
template void launch_post1d_sums<float>(cudaStream_t, const Geo &, const PhaseView &, const float *, const float *,
                                        const float *, const double *, const float *, const float *, const double *,
                                        double, double *, int);

}  // namespace ibmk
