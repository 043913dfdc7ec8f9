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

// box of copy nb of particle p (phase_indicator.f90:255-273); false when
// the copy is not processed or its clipped box is empty
struct PhaseBox {
  double cx, cy, cz;
  int ilow, jlow, klow, ni, nj, nk;
};
__device__ __forceinline__ bool phase_box(const Geo &g, const PartGeo &pg, const PartBuffers &b, int p, int nb,
                                          PhaseBox &x) {
  const int np = pg.np;
  if (nb > 0 && b.nb[(long)p * 9 + nb] != 1) return false;
  int nbrecv = nb;
  if (nb > 0) { nbrecv = nb + 4; if (nbrecv > 8) nbrecv -= 8; }
  x.cx = b.pf[(long)PF_X * np + p];
  x.cy = b.pf[(long)PF_Y * np + p];
  x.cz = b.pf[(long)PF_Z * np + p];
  phase_copy_shift(nbrecv, g.lx, g.ly, x.cx, x.cy);
  const double radius = pg.radius;
  int ilow = fnint((x.cx - radius) * g.dxi - 2.), ihigh = fnint((x.cx + radius) * g.dxi + 2.);
  int jlow = fnint((x.cy - radius) * g.dyi - 2.), jhigh = fnint((x.cy + radius) * g.dyi + 2.);
  int klow = fnint((x.cz - radius) * g.dzi - 2.), khigh = fnint((x.cz + radius) * g.dzi + 2.);
  if (ilow < 1) ilow = 1;
  if (jlow < 1) jlow = 1;
  if (klow < 1) klow = 1;
  if (ihigh > g.I) ihigh = g.I;
  if (jhigh > g.J) jhigh = g.J;
  if (khigh > g.K) khigh = g.K;
  x.ilow = ilow; x.jlow = jlow; x.klow = klow;
  x.ni = ihigh - ilow + 1; x.nj = jhigh - jlow + 1; x.nk = khigh - klow + 1;
  return x.ni > 0 && x.nj > 0 && x.nk > 0;
}

// lower corner coordinate of cell n (1-based) on grid c along axis d
// (x: 0, y: 1, z: 2); the upper corner of cell n is the lower one of n+1
__device__ __forceinline__ double phase_lo(int c, int d, int n, double h) {
  return c == d ? (n - 0.5) * h : (n - 1) * h;
}

constexpr int PH_AX = 192;  // cells per box axis held in the tables

// Pass 0.  The box is swept plane by plane in z over its corner lattice:
// each lattice point's squared distance (dxm2 + dym2) + dzm2 is formed once
// from per-axis tables, and its signed distance radius - sqrt(d2) once, for
// points within a cell diagonal of the surface (the only corners of cells
// that are partly inside).  Every cell then reads its eight corners in the
// reference's order.  Key per cell: +inf bits for the inner test, else the
// fraction; atomicMax into G, and (1 << 32) + code added into W0 (count in
// the high word and, for a single candidate, its code in the low word).
__global__ void __launch_bounds__(256) k_phase_mark(Geo g, PartGeo pg, PartBuffers b, PhaseBuffers ph, int itype,
                                                    int plmax) {
  const int np = pg.np, p = blockIdx.x, c = blockIdx.y;
  if (b.mslv[p] <= 0) return;
  if (itype == 0 && c < 3) return;  // itype 0 updates only the pressure cells
  extern __shared__ __align__(16) unsigned char ph_sm[];
  double *sg = reinterpret_cast<double *>(ph_sm);                   // [2][plmax] signed distances
  unsigned char *inside = reinterpret_cast<unsigned char *>(sg + 2 * plmax);  // [2][plmax]
  __shared__ double tx[PH_AX + 1], ty[PH_AX + 1], tz[PH_AX + 1];
  const double dx = 1. / g.dxi, dy = 1. / g.dyi, dz = 1. / g.dzi;
  const double radius = pg.radius, radin = radius - 2. * dx, radin2 = radin * radin, rthr = pg.rthr;
  // band of lattice points that can be corners of a cut cell
  const double diag = 1.05 * sqrt(dx * dx + dy * dy + dz * dz);
  const double blo = radius > diag ? (radius - diag) * (radius - diag) : 0., bhi = (radius + diag) * (radius + diag);
  const long plane = (long)g.I * g.J, nc = plane * g.K;
  unsigned long long *G = ph.G + c * nc;
  unsigned long long *W0 = ph.W0 + c * nc;
  int *W1 = ph.W1 + c * nc;
  const int bigq = 9 * np + 1;
  for (int nb = 0; nb <= 8; ++nb) {
    PhaseBox x;
    if (!phase_box(g, pg, b, p, nb, x)) continue;
    const int ni = x.ni, nj = x.nj, nk = x.nk, li = ni + 1, lp = li * (nj + 1);
    if (ni > PH_AX || nj > PH_AX || nk > PH_AX || lp > plmax) {
      if (threadIdx.x == 0) atomicExch(ph.err, 1);
      continue;
    }
    __syncthreads();  // the previous copy is done with the tables
    for (int t = threadIdx.x; t <= PH_AX; t += blockDim.x) {
      if (t <= ni) { const double v = phase_lo(c, 0, x.ilow + t, dx) - x.cx; tx[t] = v * v; }
      if (t <= nj) { const double v = phase_lo(c, 1, x.jlow + t, dy) - x.cy; ty[t] = v * v; }
      if (t <= nk) { const double v = phase_lo(c, 2, x.klow + t, dz) - x.cz; tz[t] = v * v; }
    }
    __syncthreads();
    const int qid = p * 9 + nb;
    for (int l = 0; l <= nk; ++l) {
      // lattice plane l
      double *sgl = sg + (l & 1) * plmax;
      unsigned char *inl = inside + (l & 1) * plmax;
      for (int e = threadIdx.x; e < lp; e += blockDim.x) {
        const int bb = e / li, a = e - bb * li;
        const double d2 = tx[a] + ty[bb] + tz[l];
        inl[e] = d2 < rthr;
        sgl[e] = (d2 >= blo && d2 <= bhi) ? radius - sqrt(d2) : __longlong_as_double(0x7FF8000000000000ll);
      }
      __syncthreads();
      if (l > 0) {  // cells of layer k = klow + l - 1, between lattice planes l-1 and l
        const double *s0 = sg + ((l - 1) & 1) * plmax, *s1 = sgl;
        const unsigned char *f0 = inside + ((l - 1) & 1) * plmax, *f1 = inl;
        const int k = x.klow + l - 1;
        for (int e = threadIdx.x; e < ni * nj; e += blockDim.x) {
          const int jj = e / ni, ii = e - jj * ni;
          const int o00 = jj * li + ii, o01 = o00 + li;  // (a, b) and (a, b+1)
          unsigned long long key;
          if (tx[ii + 1] + ty[jj + 1] + tz[l] < radin2) {
            key = PH_INNER;
          } else {
            const int nin = f0[o00] + f0[o01] + f0[o01 + 1] + f0[o00 + 1] + f1[o00] + f1[o01] + f1[o01 + 1] +
                            f1[o00 + 1];
            if (nin == 0) continue;
            if (nin == 8) {
              key = (unsigned long long)__double_as_longlong(1.0);
            } else {
              // reference corner order: (m,m,m) (m,p,m) (p,p,m) (p,m,m), then the same at z+
              const double q[8] = {s0[o00], s0[o01], s0[o01 + 1], s0[o00 + 1],
                                   s1[o00], s1[o01], s1[o01 + 1], s1[o00 + 1]};
              double s1s = 0., s2s = 0.;
              bool miss = false;
#pragma unroll
              for (int r = 0; r < 8; ++r) {
                miss |= isnan(q[r]);
                if (q[r] > 0.) s1s = s1s + q[r];
                s2s = s2s + fabs(q[r]);
              }
              if (miss) { atomicExch(ph.err, 2); continue; }
              const double f = s1s / s2s;
              if (!(f > 0.)) continue;
              key = (unsigned long long)__double_as_longlong(f);
            }
          }
          const long cell = (long)(k - 1) * plane + (long)(x.jlow + jj - 1) * g.I + (x.ilow + ii - 1);
          atomicMax(&G[cell], key);
          const unsigned long long code = key == PH_INNER ? qid + 1 : bigq - qid;
          const unsigned long long old = atomicAdd(&W0[cell], (1ull << 32) + code);
          if ((old >> 32) == 1) W1[cell] = 0;  // a second candidate: the resolving pass decides
        }
      }
      __syncthreads();  // plane l-1's buffers are rewritten next
    }
  }
}

// Pass 1.  Cells with several candidates: each candidate whose key equals
// the maximum takes part in atomicMax(W1, code).  The key is recomputed
// directly from its eight corners (same values as pass 0).
__global__ void __launch_bounds__(256) k_phase_resolve(Geo g, PartGeo pg, PartBuffers b, PhaseBuffers ph, int itype) {
  const int np = pg.np, p = blockIdx.x, c = blockIdx.y;
  if (b.mslv[p] <= 0) return;
  if (itype == 0 ? c < 3 : c == 3) return;  // winners are read on these grids only
  const double dx = 1. / g.dxi, dy = 1. / g.dyi, dz = 1. / g.dzi;
  const double radius = pg.radius, radin = radius - 2. * dx, radin2 = radin * radin;
  const long plane = (long)g.I * g.J, nc = plane * g.K;
  const unsigned long long *G = ph.G + c * nc;
  const unsigned long long *W0 = ph.W0 + c * nc;
  int *W1 = ph.W1 + c * nc;
  const int bigq = 9 * np + 1;
  for (int nb = 0; nb <= 8; ++nb) {
    PhaseBox x;
    if (!phase_box(g, pg, b, p, nb, x)) continue;
    const int qid = p * 9 + nb, ncell = x.ni * x.nj * x.nk;
    for (int e = threadIdx.x; e < ncell; e += blockDim.x) {
      const int kk = e / (x.ni * x.nj), r = e - kk * x.ni * x.nj, jj = r / x.ni, ii = r - jj * x.ni;
      const int i = x.ilow + ii, j = x.jlow + jj, k = x.klow + kk;
      const long cell = (long)(k - 1) * plane + (long)(j - 1) * g.I + (i - 1);
      if ((W0[cell] >> 32) < 2) continue;
      const unsigned long long key =
          phase_key(phase_cell(c, i, j, k, dx, dy, dz), x.cx, x.cy, x.cz, radius, radin2, pg.rthr);
      if (key != 0ull && key == G[cell]) atomicMax(&W1[cell], key == PH_INNER ? qid + 1 : bigq - qid);
    }
  }
}

size_t phase_smem_bytes(int nx, int ny) { return (size_t)2 * (nx + 1) * (ny + 1) * (sizeof(double) + 1); }
int phase_set_smem(size_t bytes) {
  return cudaFuncSetAttribute(k_phase_mark, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes) == cudaSuccess
             ? 0
             : -1;
}

void launch_phase_indicator(cudaStream_t s, const Geo &g, const PartGeo &pg, PartBuffers b, PhaseBuffers ph,
                            int itype, int nxmax, int nymax) {
  const long nc = (long)g.I * g.J * g.K;
  cudaMemsetAsync(ph.G, 0, 4 * nc * sizeof(unsigned long long), s);
  cudaMemsetAsync(ph.W0, 0, 4 * nc * sizeof(unsigned long long), s);
  if (pg.np == 0) return;
  const int plmax = (nxmax + 1) * (nymax + 1);
  k_phase_mark<<<dim3(pg.np, 4), 256, phase_smem_bytes(nxmax, nymax), s>>>(g, pg, b, ph, itype, plmax);
  k_phase_resolve<<<dim3(pg.np, 4), 256, 0, s>>>(g, pg, b, ph, itype);
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

// Plane sums of one cell.  Three paths with the reference's per-cell terms:
// np = 0 (all fractions 0), a cell whose ten phase keys are all empty (all
// fractions 1, all particle velocities 0: the terms weighted by 1 - gam
// vanish and the weights of the others are exactly 1), and the general one.
// Sums of exactly 1.0 are counted as integers.  Cells of the general path
// are queued in shared memory and evaluated together, so that the warps stay
// converged on both paths.
template <typename T>
struct CellStats {
  const Geo &g;
  const PhaseView &ph;
  const StatFields<T> &F;
  double kappa;
  int k;
  // neighbours of interior cell e of plane k
  struct Nb {
    int i, j, ip, jp;
    long o, oi, oj, ok;
  };
  __device__ __forceinline__ Nb nb(int e) const {
    Nb n;
    const int j0 = e / g.I, i0 = e - j0 * g.I;
    n.i = i0 + 1; n.j = j0 + 1;
    n.ip = n.i == g.I ? 1 : n.i + 1; n.jp = n.j == g.J ? 1 : n.j + 1;
    n.o = fidx(g, i0, j0, k); n.oi = fidx(g, n.ip - 1, j0, k); n.oj = fidx(g, i0, n.jp - 1, k);
    n.ok = n.o + g.plane;
    return n;
  }
  // fast paths; false when the cell needs the general path
  __device__ __forceinline__ bool fast(int e, double *s, int &nfluid) const {
    const Nb n = nb(e);
    const double u = F.u[n.o], v = F.v[n.o], w = F.w[n.o], pp = F.pr(n.o);
    const double cc = F.c ? F.c[n.o] : 0., ck = F.c ? F.c[n.ok] : 0.;
    if (!ph.parts) {  // post1d without particles: every fraction is 0 (output.f90:41-49)
      s[0] += u; s[1] += v; s[2] += w; s[3] += pp; s[4] += cc;
      s[12] += u * u; s[13] += v * v; s[14] += w * w; s[15] += pp * pp; s[16] += cc * cc;
      s[24] += 0.5 * (ck + cc) * w;
      s[25] -= kappa * (ck - cc) * g.dzi;
      return true;
    }
    const long gc = ph.grid_off(1), nxy = g.plane;
    const long c0 = ph.cell(n.i, n.j, k), ci = ph.cell(n.ip, n.j, k), cj = ph.cell(n.i, n.jp, k);
    const long ck1 = k < g.K ? c0 + nxy : c0;
    const unsigned long long any = ph.G[c0] | ph.G[cj] | ph.G[ck1] | ph.G[gc + c0] | ph.G[gc + ci] |
                                   ph.G[gc + ck1] | ph.G[2 * gc + c0] | ph.G[2 * gc + ci] | ph.G[2 * gc + cj] |
                                   ph.G[3 * gc + c0];
    if (any) return false;
    const double uj = F.u[n.oj], uk = F.u[n.ok], vi = F.v[n.oi], vk = F.v[n.ok], wi = F.w[n.oi], wj = F.w[n.oj];
    ++nfluid;
    s[0] += u; s[1] += v; s[2] += w; s[3] += pp; s[4] += cc;
    s[12] += u * u; s[13] += v * v; s[14] += w * w; s[15] += pp * pp; s[16] += cc * cc;
    s[21] += 0.25 * (uj + u) * (vi + v);
    s[22] += 0.25 * (uk + u) * (wi + w);
    s[23] += 0.25 * (vk + v) * (wj + w);
    s[25] -= kappa * (ck - cc) * g.dzi;
    return true;
  }
  // phase keys: u at (i,j,k) (i,j+1,k) (i,j,k+1); v at (i,j,k) (i+1,j,k)
  // (i,j,k+1); w at (i,j,k) (i+1,j,k) (i,j+1,k); p at (i,j,k).  Above the
  // top plane the fraction repeats plane K and the velocity mirrors it.
  __device__ void general(int e, double *s) const {
    const Nb n = nb(e);
    const int i = n.i, j = n.j, ip = n.ip, jp = n.jp, K = g.K;
    const double u = F.u[n.o], v = F.v[n.o], w = F.w[n.o], pp = F.pr(n.o);
    const double cc = F.c ? F.c[n.o] : 0., ck = F.c ? F.c[n.ok] : 0.;
    const double uj = F.u[n.oj], uk = F.u[n.ok], vi = F.v[n.oi], vk = F.v[n.ok], wi = F.w[n.oi], wj = F.w[n.oj];
    const long gc = ph.grid_off(1), nxy = g.plane;
    const long c0 = ph.cell(i, j, k), ci = ph.cell(ip, j, k), cj = ph.cell(i, jp, k);
    const long ck1 = k < K ? c0 + nxy : c0;
    const unsigned long long ku = ph.G[c0], kuj = ph.G[cj], kuk = ph.G[ck1];
    const unsigned long long kv = ph.G[gc + c0], kvi = ph.G[gc + ci], kvk = ph.G[gc + ck1];
    const unsigned long long kw = ph.G[2 * gc + c0], kwi = ph.G[2 * gc + ci], kwj = ph.G[2 * gc + cj];
    const unsigned long long kp = ph.G[3 * gc + c0];
    const double gu = 1. - PhaseView::solid(ku), gv = 1. - PhaseView::solid(kv), gw = 1. - PhaseView::solid(kw),
                 gp = 1. - PhaseView::solid(kp);
    const double guj = 1. - PhaseView::solid(kuj), guk = 1. - PhaseView::solid(kuk),
                 gvi = 1. - PhaseView::solid(kvi), gvk = 1. - PhaseView::solid(kvk),
                 gwi = 1. - PhaseView::solid(kwi), gwj = 1. - PhaseView::solid(kwj);
    const double pu = ph.part_key(0, ku, c0, i, j, k), pv = ph.part_key(1, kv, gc + c0, i, j, k);
    const double pw = k == K ? 0. : ph.part_key(2, kw, 2 * gc + c0, i, j, k);
    const double puj = ph.part_key(0, kuj, cj, i, jp, k), pvi = ph.part_key(1, kvi, gc + ci, ip, j, k);
    const double puk = k < K ? ph.part_key(0, kuk, ck1, i, j, k + 1) : -pu;
    const double pvk = k < K ? ph.part_key(1, kvk, gc + ck1, i, j, k + 1) : -pv;
    const double pwi = k == K ? 0. : ph.part_key(2, kwi, 2 * gc + ci, ip, j, k);
    const double pwj = k == K ? 0. : ph.part_key(2, kwj, 2 * gc + cj, i, jp, k);
    // output.f90:103-123
    s[0] += u * gu; s[1] += v * gv; s[2] += w * gw; s[3] += pp * gp; s[4] += cc * gp;
    s[5] += pu * (1. - gu); s[6] += pv * (1. - gv); s[7] += pw * (1. - gw);
    s[8] += gu; s[9] += gv; s[10] += gw; s[11] += gp;
    // output.f90:218-235
    s[12] += u * u * gu; s[13] += v * v * gv; s[14] += w * w * gw; s[15] += pp * pp * gp; s[16] += cc * cc * gp;
    s[17] += pu * pu * (1. - gu); s[18] += pv * pv * (1. - gv); s[19] += pw * pw * (1. - gw);
    s[20] += gp * gp;
    // output.f90:316-352
    s[21] += 0.25 * (uj + u) * (vi + v) * (0.25 * (guj + gu + gvi + gv));
    s[22] += 0.25 * (uk + u) * (wi + w) * (0.25 * (guk + gu + gwi + gw));
    s[23] += 0.25 * (vk + v) * (wj + w) * (0.25 * (gvk + gv + gwj + gw));
    s[24] += 0.5 * (ck + cc) * w * (1 - gw);
    s[25] -= kappa * (ck - cc) * g.dzi;
    s[26] += 0.25 * (puj + pu) * (pvi + pv) * (0.25 * (2. - guj - gu + 2. - gvi - gv));
    s[27] += 0.25 * (puk + pu) * (pwi + pw) * (0.25 * (2. - guk - gu + 2. - gwi - gw));
    s[28] += 0.25 * (pvk + pv) * (pwj + pw) * (0.25 * (2. - gvk - gv + 2. - gwj - gw));
    s[29] += 0.25 * (guj + gu + (gvi + gv));
    s[30] += 0.25 * (guk + gu + (gwi + gw));
    s[31] += 0.25 * (gvk + gv + (gwj + gw));
  }
};

constexpr int STAT_BLOCK = 128, STAT_QCAP = 4 * STAT_BLOCK;

template <typename T>
__global__ void __launch_bounds__(STAT_BLOCK, 3) k_post1d_sums(Geo g, PhaseView ph, StatFields<T> F, double kappa,
                                                               double *__restrict__ part, int slices) {
  const int k = blockIdx.x + 1, sl = blockIdx.y;
  const int nxy = g.I * g.J;  // a plane has fewer than 2^31 cells
  const int per = (nxy + slices - 1) / slices;
  const int e0 = sl * per, e1 = min(nxy, e0 + per);
  double s[POST1D_NSUM];
#pragma unroll
  for (int q = 0; q < POST1D_NSUM; ++q) s[q] = 0.;
  int nfluid = 0;  // cells of the fast path with particles: +1 to gum..gpm, gp2, guv..gvw
  const CellStats<T> cs{g, ph, F, kappa, k};
  __shared__ int queue[STAT_QCAP];
  __shared__ int qn;
  if (threadIdx.x == 0) qn = 0;
  __syncthreads();
  for (int base = e0; base < e1; base += STAT_BLOCK) {
    const int e = base + threadIdx.x;
    if (e < e1 && !cs.fast(e, s, nfluid)) queue[atomicAdd(&qn, 1)] = e;
    __syncthreads();
    const int nq = qn;
    if (nq > STAT_QCAP - STAT_BLOCK || base + STAT_BLOCK >= e1) {
      for (int q = threadIdx.x; q < nq; q += STAT_BLOCK) cs.general(queue[q], s);
      __syncthreads();
      if (threadIdx.x == 0) qn = 0;
      __syncthreads();
    }
  }
  if (nfluid) {
    const double n1 = (double)nfluid;
    s[8] += n1; s[9] += n1; s[10] += n1; s[11] += n1; s[20] += n1; s[29] += n1; s[30] += n1; s[31] += n1;
  }
  __shared__ double red[STAT_BLOCK / 32][POST1D_NSUM];
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
    for (int w8 = 0; w8 < STAT_BLOCK / 32; ++w8) x += red[w8][threadIdx.x];
    part[((long)blockIdx.x * slices + sl) * POST1D_NSUM + threadIdx.x] = x;
  }
}

template <typename T>
void launch_post1d_sums(cudaStream_t s, const Geo &g, const PhaseView &ph, const T *u, const T *v, const T *w,
                        const double *p, const float *phi, const float *plo, const double *c, double kappa,
                        double *part, int slices) {
  StatFields<T> F{u, v, w, p, phi, plo, c};
  k_post1d_sums<T><<<dim3(g.K, slices), STAT_BLOCK, 0, s>>>(g, ph, F, kappa, part, slices);
}
template void launch_post1d_sums<double>(cudaStream_t, const Geo &, const PhaseView &, const double *, const double *,
                                         const double *, const double *, const float *, const float *,
                                         const double *, double, double *, int);
template void launch_post1d_sums<float>(cudaStream_t, const Geo &, const PhaseView &, const float *, const float *,
                                        const float *, const double *, const float *, const float *, const double *,
                                        double, double *, int);

}  // namespace ibmk
