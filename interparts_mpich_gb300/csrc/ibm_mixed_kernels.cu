// ibm_mixed_kernels.cu -- the multidirect IBM loop of the mixed form
// (interp_spread.f90, forcing.f90 restated for FP32 fields).
//
// Per Lagrangian point and velocity component a 48-byte stencil record
// (origin of the 3x3x3 tap block and the component's 9 delta weights) is
// built once per substep; the per-particle, per-component box of cells the
// stencils touch is computed once as well.  Interpolation and spreading then
// run one block per (particle, component) on a shared-memory copy of that
// box: interpolation reads it with coalesced rows, spreading accumulates into
// it and flushes each touched cell to HBM once.
//
// Origins come from the FP64 point coordinates exactly as the FP64 form
// computes them; delta weights, interpolation sums and spreading are FP32;
// point forces F_l and the per-particle force/torque sums stay FP64.
#include <cuda_bf16.h>

#include "kernels.cuh"

namespace ibmk {


// ---------------------------------------------------------------------------
// Point records (16 bytes, PointRec): the fractions of the grid coordinates
// and the floors relative to the particle's reference floor; make_cs turns
// one into a component's stencil (origin of the 3x3x3 tap block and the
// component's 9 delta weights, interp_spread.f90:60-131) whenever a pass
// needs it, instead of reading 3 x 48-byte records per point and pass.
// ---------------------------------------------------------------------------
// The rigid-body velocity of a point as an FP32 pair hi + lo (the slip
// U - u~ = (hi - u~) + lo keeps the FP64 velocity's bits that FP32 u~ resolves)
__device__ __forceinline__ float2 split_u(double U) {
  const float hi = (float)U;
  return make_float2(hi, (float)(U - (double)hi));
}
// Reference floors of the particles (the floors of the centres' grid
// coordinates), the centres' offsets from them in cells and the velocities
// as FP32 pairs, FP64 once per particle.
__global__ void k_ibm_pref(Geo g, PartGeo pg, IbmBuffers b) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= pg.np) return;
  const double x = b.pf[PF_X * pg.np + p] * g.dxi, y = b.pf[PF_Y * pg.np + p] * g.dyi,
               z = b.pf[PF_Z * pg.np + p] * g.dzi;
  const int4 ref = make_int4(__double2int_rd(x), __double2int_rd(y), __double2int_rd(z), 0);
  b.pref[p] = ref;
  b.pcen[p] = make_float4((float)(x - (double)ref.x), (float)(y - (double)ref.y), (float)(z - (double)ref.z), 0.f);
  const float2 u = split_u(b.pf[PF_U * pg.np + p]), v = split_u(b.pf[PF_V * pg.np + p]),
               w = split_u(b.pf[PF_W * pg.np + p]);
  b.pvh[p] = make_float4(u.x, v.x, w.x, 0.f);
  b.pvl[p] = make_float4(u.y, v.y, w.y, 0.f);
}
// Point records: the point's position relative to its particle's reference
// floor in cells, from its FP64 offset from the centre (exact to the FP32
// rounding of an offset of at most the radius) plus the centre's offset;
// the floor and the fraction of that FP32 position.  A point whose
// absolute z lies beyond the walls' reach (or is not finite) is flagged and
// parked at the centre, as in the FP64 form.
__global__ void __launch_bounds__(256) k_ibm_points(Geo g, PartGeo pg, IbmBuffers b) {
  const int n = pg.np * pg.nl;  // < 2^31 points (checked at create)
  const float dxi = (float)g.dxi, dyi = (float)g.dyi, dzi = (float)g.dzi;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
    const int p = t / pg.nl, l = t - p * pg.nl;
    if (l >= b.nla[p]) continue;
    const int4 ref = b.pref[p];
    const float4 cf = b.pcen[p];
    const float cx = fmaf((float)(b.xfp[t] - b.pf[PF_X * pg.np + p]), dxi, cf.x);
    const float cy = fmaf((float)(b.yfp[t] - b.pf[PF_Y * pg.np + p]), dyi, cf.y);
    const float cz = fmaf((float)(b.zfp[t] - b.pf[PF_Z * pg.np + p]), dzi, cf.z);
    float fx = floorf(cx), fy = floorf(cy), fz = floorf(cz);
    int dx = (int)fx, dy = (int)fy, dz = (int)fz;
    float frx = cx - fx, fry = cy - fy, frz = cz - fz;
    const float zabs = (float)ref.z + cz;
    if (!(fabsf(cx) < 510.f && fabsf(cy) < 510.f && fabsf(cz) < 510.f) ||
        !(zabs >= -1.f && zabs <= (float)g.K + 0.49f)) {  // also NaN
      atomicExch(&b.err[2], 1);
      dx = 0; dy = 0; dz = max(min(ref.z, g.K - 1), 1) - ref.z; frx = 0.f; fry = 0.f; frz = 0.5f;
    }
    PointRec r;
    r.fx = frx;
    r.fy = fry;
    r.fz = frz;
    r.rel = (unsigned)(dx + 512) | ((unsigned)(dy + 512) << 10) | ((unsigned)(dz + 512) << 20);
    b.rec[t] = r;
  }
}

// Box of the cells the stencils of particle p, component c touch:
// bgeo[(p*3 + c)*8 + ] = {refx, refy, bmin_x, bmin_y, bmin_z, nbx, nby, nbz};
// x, y relative to the particle's reference floor, box cell (cx,cy,cz) =
// tap (refx + bmin_x + cx, refy + bmin_y + cy, bmin_z + cz).  With at most
// IBM_BOX_ROWS rows and at most 32 cells in x, rowm[(p*3 + c)*IBM_BOX_ROWS +
// cz*nby + cy] = the cells the stencils touch in that row (bit cx): a
// sphere's shell touches about 40 % of its box, and a row through the
// sphere only its two ends.
__global__ void __launch_bounds__(256) k_ibm_box_geom(PartGeo pg, IbmBuffers b, int K) {
  const int p = blockIdx.x, c = blockIdx.y;
  const int nla = b.nla[p];
  const PointRec *rp = b.rec + (long)p * pg.nl;
  __shared__ int mn[3], mx[3];
  __shared__ unsigned rm[IBM_BOX_ROWS];
  if (threadIdx.x < 3) { mn[threadIdx.x] = 0x7fffffff; mx[threadIdx.x] = -0x7fffffff; }
  for (int q = threadIdx.x; q < IBM_BOX_ROWS; q += blockDim.x) rm[q] = 0u;
  __syncthreads();
  const int4 ref = b.pref[p];
  int lo[3] = {0x7fffffff, 0x7fffffff, 0x7fffffff}, hi[3] = {-0x7fffffff, -0x7fffffff, -0x7fffffff};
  for (int l = threadIdx.x; l < nla; l += blockDim.x) {
    const CompStencil s = make_cs(rp[l], c, ref.z, K);
    for (int d = 0; d < 3; ++d) { lo[d] = min(lo[d], s.b[d]); hi[d] = max(hi[d], s.b[d]); }
  }
  for (int d = 0; d < 3; ++d) {
    const int wl = __reduce_min_sync(0xffffffffu, lo[d]), wh = __reduce_max_sync(0xffffffffu, hi[d]);
    if ((threadIdx.x & 31) == 0) { atomicMin(&mn[d], wl); atomicMax(&mx[d], wh); }
  }
  __syncthreads();
  const int nbx = mx[0] - mn[0] + 3, nby = mx[1] - mn[1] + 3, nbz = mx[2] - mn[2] + 3;
  if (nla > 0 && nby * nbz <= IBM_BOX_ROWS && nbx <= 32) {
    for (int l = threadIdx.x; l < nla; l += blockDim.x) {
      const CompStencil s = make_cs(rp[l], c, ref.z, K);
      const int x0 = s.b[0] - mn[0], y0 = s.b[1] - mn[1], z0 = s.b[2] - mn[2];
      const unsigned bits = 7u << x0;  // cells x0 .. x0 + 2 (x0 + 2 < nbx <= 32)
#pragma unroll
      for (int k = 0; k < 3; ++k)
#pragma unroll
        for (int j = 0; j < 3; ++j) atomicOr(&rm[(z0 + k) * nby + y0 + j], bits);
    }
    __syncthreads();
    unsigned *rx = b.rowm + ((long)p * 3 + c) * IBM_BOX_ROWS;
    for (int q = threadIdx.x; q < nby * nbz; q += blockDim.x) rx[q] = rm[q];
  }
  if (threadIdx.x == 0) {
    int *o = b.bgeo + ((long)p * 3 + c) * 8;
    o[0] = ref.x; o[1] = ref.y;
    if (nla > 0) {
      o[2] = mn[0]; o[3] = mn[1]; o[4] = mn[2];
      o[5] = mx[0] - mn[0] + 3; o[6] = nby; o[7] = nbz;
    } else {
      o[2] = o[3] = o[4] = o[5] = o[6] = o[7] = 0;
    }
  }
}

void launch_ibm_stencil_f(cudaStream_t s, const Geo &g, const PartGeo &pg, IbmBuffers b) {
  if (pg.np == 0) return;
  k_ibm_pref<<<(pg.np + 127) / 128, 128, 0, s>>>(g, pg, b);
  k_ibm_points<<<1216, 256, 0, s>>>(g, pg, b);
  k_ibm_box_geom<<<dim3(pg.np, 3), 256, 0, s>>>(pg, b, g.K);
}

// box usable in shared memory: fits cap and narrower than half the periodic
// domain (so relative indices are unambiguous)
__device__ __forceinline__ bool box_ok(const int *bg, int cap, int I, int J) {
  return bg[5] > 0 && (long)bg[5] * bg[6] * bg[7] <= cap && bg[5] < I / 2 && bg[6] < J / 2;
}
// offset of tap (0,0,0) of a point (make_cs origin, relative in x and y) in
// its particle's box
__device__ __forceinline__ int box_off(const CompStencil &s, const int *bg) {
  return ((s.b[2] - bg[4]) * bg[6] + (s.b[1] - bg[3])) * bg[5] + (s.b[0] - bg[2]);
}
__device__ __forceinline__ void load_box(const Geo &g, const float *__restrict__ F, const int *bg, float *box,
                                         const unsigned *__restrict__ rowm) {
  const int nbx = bg[5], nby = bg[6], nxy = nbx * nby, nbox = nxy * bg[7];
  const int x0 = bg[0] + bg[2], y0 = bg[1] + bg[3], z0 = bg[4];
  if ((g.I & 3) == 0) {
    // rows read as 16-byte quads of x-cells (aligned: I is a multiple of 4,
    // so a quad never straddles the periodic wrap); cells outside the row
    // are dropped, and so are quads holding none of the cells the stencils
    // read (the row masks of k_ibm_box_geom, for boxes up to 32 cells wide)
    const int a0 = x0 - (((x0 % 4) + 4) % 4);
    const int nq = (x0 + nbx - a0 + 3) >> 2, nrow = nby * bg[7];
    const bool masked = nrow <= IBM_BOX_ROWS && nbx <= 32;
    for (int e = threadIdx.x; e < nrow * nq; e += blockDim.x) {
      const int row = e / nq, t = e - row * nq;
      const int cz = row / nby, cy = row - cz * nby, gx = a0 + 4 * t;
      if (masked) {
        const unsigned m = rowm[row];
        const int sh = gx - x0;  // first cell of the quad, -3 .. nbx - 1
        if (((sh >= 0 ? m >> sh : m << -sh) & 0xFu) == 0u) continue;
      }
      const float4 v =
          __ldg(reinterpret_cast<const float4 *>(&F[fidx(g, wrapm(gx, g.I), wrapm(y0 + cy, g.J), z0 + cz)]));
      const float vv[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
      for (int d = 0; d < 4; ++d) {
        const int cx = gx + d - x0;
        if (cx >= 0 && cx < nbx) box[row * nbx + cx] = vv[d];
      }
    }
    return;
  }
  for (int q = threadIdx.x; q < nbox; q += blockDim.x) {
    const int cz = q / nxy, r = q - cz * nxy, cy = r / nbx, cx = r - cy * nbx;
    box[q] = __ldg(&F[fidx(g, wrapm(x0 + cx, g.I), wrapm(y0 + cy, g.J), z0 + cz)]);
  }
}
// Lever arms of the torque terms of component c (c=0: (rz, ry), c=1:
// (rz, rx), c=2: (ry, rx)), FP32 from the point record and the centre
// offsets cf (cells from the reference floor)
__device__ __forceinline__ void lever_arms(const PointRec &rr, const float4 &cf, int c, float hx, float hy, float hz,
                                           float &la, float &lb) {
  const float ry = rec_armf(rec_dy(rr.rel), rr.fy, cf.y, hy);
  la = c == 2 ? ry : rec_armf(rec_dz(rr.rel), rr.fz, cf.z, hz);
  lb = c == 0 ? ry : rec_armf(rec_dx(rr.rel), rr.fx, cf.x, hx);
}
// rigid-body velocity component of point t: the particle's, or with rotation
// on the per-point value (u + omega x r, updated with the points)
__device__ __forceinline__ double point_u(const PartGeo &pg, const double *Ua, double Up, long t) {
  return pg.rotation ? Ua[t] : Up;
}

// 27-tap interpolation of one component, k outer, j, i inner, each term
// f * (wx_i * (wy_j * wz_k))
template <typename TAP>
__device__ __forceinline__ float interp27(const CompStencil &s, TAP tap) {
  float acc = 0.f;
#pragma unroll
  for (int k = 0; k < 3; ++k)
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      const float wyz = s.w[3 + j] * s.w[6 + k];
#pragma unroll
      for (int i = 0; i < 3; ++i) acc += tap(i, j, k) * (s.w[i] * wyz);
    }
  return acc;
}

// ---------------------------------------------------------------------------
// eulr2lagr + complagrforces/updtlagrforces: block (particle, component).
// Interpolated component to dudtl/dvdtl/dwdtl; with first >= 0 the FP64
// point-force update of the component and its partial sums (sum F_c and the
// two lever-arm moments of F_c in the torque) to psum; k_ibm_force_sums
// combines the components.  first == -1: the residual sum of (U - u~)^2 only
// (FP32: it feeds the learned loop's gate), dudtl left as it was; first ==
// -2: the interpolation to dudtl only (the slip-residual diagnostic).
// ---------------------------------------------------------------------------
// box capacity: pg.box_cap cells (8192 = 32 KB for spheres up to about
// D = 16 dx; polydisperse runs size it for the largest sphere)
constexpr int INTERP_THREADS = 256;

// FP32 sum over the block (blockDim a multiple of 32, at most 1024), to every thread
__device__ __forceinline__ float block_sum_all(float a) {
  __shared__ float part[32];
#pragma unroll
  for (int d = 16; d > 0; d >>= 1) a += __shfl_xor_sync(0xffffffffu, a, d);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  if (lane == 0) part[w] = a;
  __syncthreads();
  float t = 0.f;
  for (int q = 0; q < nw; ++q) t += part[q];
  return t;
}

// FIRST (the pass kind) and ROT (per-point rigid-body velocities) are
// template parameters: FP64 instructions of an if-converted branch issue
// under a false predicate and still occupy the FP64 pipe, which this GPU
// runs at 1/64 of the FP32 rate.
template <int FIRST, bool ROT>
__global__ void __launch_bounds__(INTERP_THREADS, 4) k_ibm_interp_comp_f(Geo g, PartGeo pg, IbmBuffers b,
                                                           const float *__restrict__ fu, const float *__restrict__ fv,
                                                           const float *__restrict__ fw, double dti,
                                                           const int *__restrict__ gate) {
  constexpr int first = FIRST;
  if (gate && *gate == 0) return;  // learned form: plain pass not needed
  const int p = blockIdx.x, c = blockIdx.y;
  const int nla = b.nla[p];
  const long npl = (long)pg.np * pg.nl, t0 = (long)p * pg.nl;
  const float *F = c == 0 ? fu : (c == 1 ? fv : fw);
  extern __shared__ __align__(16) unsigned char ibox_sm[];
  float *box = reinterpret_cast<float *>(ibox_sm);
  __shared__ int bg[8];
  __shared__ float kc[4];  // FP32 1/dt and grid spacings, converted once per block
  if (threadIdx.x < 8) bg[threadIdx.x] = b.bgeo[((long)p * 3 + c) * 8 + threadIdx.x];
  if (threadIdx.x == 32) {
    kc[0] = (float)dti;
    kc[1] = (float)g.dx;
    kc[2] = (float)g.dy;
    kc[3] = (float)g.dz;
  }
  __syncthreads();
  const bool boxed = box_ok(bg, pg.box_cap, g.I, g.J);
  if (boxed) {
    load_box(g, F, bg, box, b.rowm + ((long)p * 3 + c) * IBM_BOX_ROWS);
    __syncthreads();
  }
  double *dud = c == 0 ? b.dudtl : (c == 1 ? b.dvdtl : b.dwdtl);
  const double *Ua = c == 0 ? b.ul : (c == 1 ? b.vl : b.wl);
  float *Fl = c == 0 ? b.fxs : (c == 1 ? b.fys : b.fzs);
  float *slip = b.slip + c * npl;
  const float4 vh = b.pvh[p], vl = b.pvl[p];
  const float2 Us = c == 0 ? make_float2(vh.x, vl.x) : (c == 1 ? make_float2(vh.y, vl.y) : make_float2(vh.z, vl.z));
  const int4 ref = b.pref[p];
  const float4 cf = b.pcen[p];
  const float hx = kc[1], hy = kc[2], hz = kc[3];
  const float dtif = kc[0];
  const PointRec *rp = b.rec + t0;
  const int ys = bg[5], zs = bg[5] * bg[6];
  // per-thread force and lever-arm sums in FP32 (a few points per thread),
  // the block's sums in FP64
  float sF = 0.f, sa = 0.f, sb = 0.f;
  float r2 = 0.f, r0 = 0.f;
  for (int l = threadIdx.x; l < nla; l += blockDim.x) {
    const long t = t0 + l;
    const PointRec rr = rp[l];
    const CompStencil s = make_cs(rr, c, ref.z, g.K);
    float acc;
    if (boxed) {
      const float *B = box + box_off(s, bg);
      acc = interp27(s, [&](int i, int j, int k) { return B[i + j * ys + k * zs]; });
    } else {
      acc = interp27(s, [&](int i, int j, int k) {
        return __ldg(&F[fidx(g, wrapm(ref.x + s.b[0] + i, g.I), wrapm(ref.y + s.b[1] + j, g.J), s.b[2] + k)]);
      });
    }
    float2 U = Us;
    if constexpr (ROT) U = split_u(Ua[t]);
    const float sd = (U.x - acc) + U.y;  // slip U - u~
    if constexpr (FIRST == -1) {  // residual only: sum of (U - u~)^2 of the component
      r2 = fmaf(sd, sd, r2);
      continue;
    }
    if constexpr (FIRST < 0) {  // the interpolation only (diagnostics)
      dud[t] = acc;
      continue;
    }
    slip[t] = sd;  // the spreading's increment (U - u~)/dt, FP32
    if constexpr (FIRST == 1) r0 = fmaf(sd, sd, r0);  // first-pass slip, for the learned loop's gate reference
    float ff;  // the point force, FP32 (its sums below, FP64 across the block)
    if constexpr (FIRST == 1) ff = sd * dtif;
    else ff = fmaf(sd, dtif, Fl[t]);
    Fl[t] = ff;
    float la, lb;
    lever_arms(rr, cf, c, hx, hy, hz, la, lb);
    sF += ff;
    sa = fmaf(la, ff, sa);
    sb = fmaf(lb, ff, sb);
  }
  // psum[p][c]: force and lever-arm sums, or (first < 0) the residual sum in
  // slot 0 for k_ibm_res_gate
  if (first == -1) {
    const float tot = block_sum_all(r2);
    if (threadIdx.x == 0) b.psum[((long)p * 3 + c) * 3] = tot;
    return;
  }
  if (first < 0) return;
  if (first) {
    const float tot = block_sum_all(r0);
    if (threadIdx.x == 0) b.rsum[(long)p * 3 + c] = tot;
  }
  __syncthreads();  // the box is dead: its first words hold the partial sums
  float *st = reinterpret_cast<float *>(ibox_sm);
  __shared__ double res[3];
  block_sum3_df(sF, sa, sb, st, res);
  if (threadIdx.x < 3) b.psum[((long)p * 3 + c) * 3 + threadIdx.x] = res[threadIdx.x];
}
// per-particle force and torque of updtlagrforces from the component sums
__global__ void k_ibm_force_sums(PartGeo pg, IbmBuffers b, const int *__restrict__ gate) {
  if (gate && *gate == 0) return;
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= pg.np) return;
  const double *s = b.psum + (long)p * 9;
  const double dV = p_dvl(pg, p);
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
  const dim3 grd(pg.np, 3);
  const size_t sm = pg.box_cap * sizeof(float);
  auto go = [&](auto kern) { kern<<<grd, INTERP_THREADS, sm, s>>>(g, pg, b, fu, fv, fw, 1. / dt, gate); };
  const bool rot = pg.rotation != 0;
  if (first == 1) rot ? go(k_ibm_interp_comp_f<1, true>) : go(k_ibm_interp_comp_f<1, false>);
  else if (first == 0) rot ? go(k_ibm_interp_comp_f<0, true>) : go(k_ibm_interp_comp_f<0, false>);
  else if (first == -1) rot ? go(k_ibm_interp_comp_f<-1, true>) : go(k_ibm_interp_comp_f<-1, false>);
  else rot ? go(k_ibm_interp_comp_f<-2, true>) : go(k_ibm_interp_comp_f<-2, false>);
  if (first < 0) return 1;
  k_ibm_force_sums<<<(pg.np + 127) / 128, 128, 0, s>>>(pg, b, gate);
  return 2;
}

// ---------------------------------------------------------------------------
// lagr2eulr spreading of dF = (U_l - u~_l)/dt (or a given increment) with
// the terms of interp_spread.f90:329-355, F*coeff0*phix*phiy*phiz.  Block
// (particle, component): contributions accumulate in the particle's box in
// shared memory, and each touched cell is flushed to HBM with one atomic add.
// The box holds 32-bit fixed-point sums: a first pass computes every point's
// prefactor F*coeff0 into shared memory and their absolute sum B, which
// bounds every cell's sum (the 27 delta weights of a point are non-negative
// and sum to one); with the scale 2^s, B * 2^s < 2^29, each tap adds
// rint(2^s * prefactor * weight) with a native integer shared-memory add
// (no compare-and-swap loop, no wait on its result), and the sums are exact
// and independent of the order of the adds.  The resolution, at most
// B / 2^28 per tap, is of the order of the FP32 rounding of the cell sums
// it replaces (B is a few hundred times the largest prefactor).  Particles with
// more than SPREAD_PRE points, or a bound that is zero or not finite, add
// FP32 values into the box instead; boxes beyond pg.box_cap cells add per
// tap to the field.
// ---------------------------------------------------------------------------
constexpr int SPREAD_PRE = 2048;
constexpr int SPREAD_THREADS = 384;

// the 27 taps of one point into the box: FP32 adds, or fixed-point adds of
// rint(pre * w) (pre already scaled)
template <bool FIXED>
__device__ __forceinline__ void spread27_box(float *box, const CompStencil &s, int o, int nbx, int nby, float pre) {
#pragma unroll
  for (int k = 0; k < 3; ++k)
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      const float a = pre * s.w[3 + j] * s.w[6 + k];  // the (j,k) factor, then the x weight
      const int row = o + (k * nby + j) * nbx;
#pragma unroll
      for (int i = 0; i < 3; ++i) {
        if constexpr (FIXED) atomicAdd(reinterpret_cast<int *>(box) + row + i, __float2int_rn(a * s.w[i]));
        else atomicAdd(&box[row + i], a * s.w[i]);
      }
    }
}

// LY: a learned (or perturbation) force is given (lf.Y), as a template
// parameter so that the plain passes issue none of its FP64 work
template <bool LY>
__global__ void __launch_bounds__(SPREAD_THREADS, 3) k_ibm_spread_f(Geo g, PartGeo pg, IbmBuffers b, float *__restrict__ fu,
                                                      float *__restrict__ fv, float *__restrict__ fw, double dti,
                                                      double coeff0_, LearnedForce lf,
                                                      const int *__restrict__ gate, double dt) {
  if (gate && *gate == 0) return;  // learned form: plain pass not needed
  const int p = blockIdx.x, c = blockIdx.y;
  const int nla = b.nla[p];
  if (nla <= 0) {
    if (LY && threadIdx.x < 3) b.psum[((long)p * 3 + c) * 3 + threadIdx.x] = 0.;
    if (LY && !lf.incr && threadIdx.x == 0) b.rsum[(long)p * 3 + c] = 0.f;
    return;
  }
  const long npl = (long)pg.np * pg.nl, t0 = (long)p * pg.nl;
  float *F = c == 0 ? fu : (c == 1 ? fv : fw);
  extern __shared__ __align__(16) unsigned char spread_sm[];
  float *box = reinterpret_cast<float *>(spread_sm);
  int *ibox = reinterpret_cast<int *>(spread_sm);
  __shared__ int bg[8];
  __shared__ float spre[SPREAD_PRE];  // prefactors of the staged points
  // the block's FP32 constants, formed once by one thread (FP64 arithmetic
  // in every thread, or issued under a false predicate, would occupy the
  // 1/64-rate FP64 pipe): prefactors F coeff0 (F given) and (U - u~) dti
  // coeff0 (coeff0 with the particle's own Lagrangian volume when
  // polydisperse), 1/dt and dt of the learned force
  __shared__ float kc[7];
  if (threadIdx.x < 8) bg[threadIdx.x] = b.bgeo[((long)p * 3 + c) * 8 + threadIdx.x];
  if (threadIdx.x == 32) {
    const double coeff0 = pg.poly ? (pg.pdvl[p] / pg.dVeul) * dt : coeff0_;
    kc[0] = (float)coeff0;
    kc[1] = (float)(dti * coeff0);
    kc[2] = LY ? (float)lf.dti : 0.f;
    kc[3] = LY ? (float)(1. / lf.dti) : 0.f;
    kc[4] = (float)g.dx;
    kc[5] = (float)g.dy;
    kc[6] = (float)g.dz;
  }
  __syncthreads();
  const bool boxed = box_ok(bg, pg.box_cap, g.I, g.J);
  const bool staged = boxed && nla <= SPREAD_PRE;
  const int nbx = bg[5], nby = bg[6], nbox = nbx * nby * bg[7];
  if (boxed) {
    for (int q = threadIdx.x; q < nbox; q += blockDim.x) box[q] = 0.f;
    __syncthreads();
  }
  const float *slip = b.slip + c * npl;
  float *Fl = c == 0 ? b.fxs : (c == 1 ? b.fys : b.fzs);
  const int4 ref = b.pref[p];
  const PointRec *rp = b.rec + t0;
  // per-thread force and lever-arm sums in FP32, the block's sums in FP64
  float sF = 0.f, sa = 0.f, sb = 0.f;
  float4 cf = make_float4(0.f, 0.f, 0.f, 0.f);
  float ysig = 0.f, ymu = 0.f, dtif = 0.f, dtf = 0.f;
  const float hx = kc[4], hy = kc[5], hz = kc[6];
  if constexpr (LY) {
    cf = b.pcen[p];
    ysig = lf.tsig[c]; ymu = lf.tmu[c];
    dtif = kc[2]; dtf = kc[3];
  }
  const float pcoef = kc[0], ucoef = kc[1];
  // Taps into the box: points in transposed order, the 32 lanes of a warp
  // taking points nq apart in the particle's list (neighbouring points have
  // overlapping stencils, and shared-memory adds to one address in one
  // instruction serialise).  Prefactors of staged points: natural order
  // (coalesced loads of the point arrays).
  const int nq = (nla + 31) >> 5;
  float asum = 0.f, r0 = 0.f;
  for (int m = threadIdx.x; m < 32 * nq; m += blockDim.x) {
    const int l = staged ? m : (m & 31) * nq + (m >> 5);
    if (l >= nla) continue;
    const long t = t0 + l;
    float pre;
    if constexpr (LY) {
      // total point force F0 + the network's correction, its sums
      // (updtlagrforces), spread once
      const float f0 = Fl[t];
      const float d = fmaf(lf.Y[3 * t + c], ysig, ymu) * dtif;
      const float ff = f0 + d;
      Fl[t] = ff;
      const float e0 = f0 * dtf;  // the first pass's slip U - u~
      r0 = fmaf(e0, e0, r0);
      float la, lb;
      lever_arms(rp[l], cf, c, hx, hy, hz, la, lb);
      sF += ff;
      sa = fmaf(la, ff, sa);
      sb = fmaf(lb, ff, sb);
      pre = (lf.incr ? d : ff) * pcoef;
    } else {
      pre = slip[t] * ucoef;
    }
    if (staged) {
      spre[l] = pre;
      asum += fabsf(pre);
      continue;
    }
    const CompStencil s = make_cs(rp[l], c, ref.z, g.K);
    if (boxed) {
      spread27_box<false>(box, s, box_off(s, bg), nbx, nby, pre);
    } else {
      for (int k = 0; k < 3; ++k)
        for (int j = 0; j < 3; ++j) {
          const float a = pre * s.w[3 + j] * s.w[6 + k];
          const int y = wrapm(ref.y + s.b[1] + j, g.J);
          for (int i = 0; i < 3; ++i)
            atomicAdd(&F[fidx(g, wrapm(ref.x + s.b[0] + i, g.I), y, s.b[2] + k)], a * s.w[i]);
        }
    }
  }
  if constexpr (LY) {  // psum[p][c] for k_ibm_force_sums; rsum for the gate
    __shared__ float sred[192];
    __shared__ double res[3];
    block_sum3_df(sF, sa, sb, sred, res);
    if (threadIdx.x < 3) b.psum[((long)p * 3 + c) * 3 + threadIdx.x] = res[threadIdx.x];
    if (!lf.incr) {
      const float tot = block_sum_all(r0);
      if (threadIdx.x == 0) b.rsum[(long)p * 3 + c] = tot;
      __syncthreads();  // block_sum_all's partials are read again below
    }
  }
  if (!boxed) return;
  // fixed point: scale 2^(29 - e) with bound < 2^e, so that bound * scale < 2^30
  float scale = 0.f;
  if (staged) {
    const float bound = block_sum_all(asum);  // also orders spre before its reads
    int e = 0;
    if (bound > 0.f && bound <= 3.0e38f) {
      frexpf(bound, &e);
      scale = ldexpf(1.f, min(29 - e, 126));
    }
    for (int m = threadIdx.x; m < 32 * nq; m += blockDim.x) {
      const int l = (m & 31) * nq + (m >> 5);
      if (l >= nla) continue;
      const CompStencil s = make_cs(rp[l], c, ref.z, g.K);
      const int o = box_off(s, bg);
      if (scale > 0.f) spread27_box<true>(box, s, o, nbx, nby, spre[l] * scale);
      else spread27_box<false>(box, s, o, nbx, nby, spre[l]);
    }
  }
  __syncthreads();
  const bool fixed = scale > 0.f;
  const float iscale = fixed ? 1.f / scale : 0.f;  // a power of two: exact
  auto cell = [&](int q) { return fixed ? (float)ibox[q] * iscale : box[q]; };
  const int nxy = nbx * nby, x0 = bg[0] + bg[2], y0 = bg[1] + bg[3], z0 = bg[4];
  if ((g.I & 3) == 0) {
    // flush by 16-byte quads of x-cells (rows padded with zeros to the
    // aligned quads that cover them; with I a multiple of 4 a quad never
    // straddles the periodic wrap): one vector atomic per nonzero quad
    const int a0 = x0 - (((x0 % 4) + 4) % 4);
    const int nqd = (x0 + nbx - a0 + 3) >> 2, nrow = nby * bg[7];
    for (int e = threadIdx.x; e < nrow * nqd; e += blockDim.x) {
      const int row = e / nqd, t = e - row * nqd;
      const int cz = row / nby, cy = row - cz * nby, gx = a0 + 4 * t;
      float v[4];
#pragma unroll
      for (int d = 0; d < 4; ++d) {
        const int cx = gx + d - x0;
        v[d] = (cx >= 0 && cx < nbx) ? cell(row * nbx + cx) : 0.f;
      }
      if (v[0] == 0.f && v[1] == 0.f && v[2] == 0.f && v[3] == 0.f) continue;
      float4 *dst = reinterpret_cast<float4 *>(&F[fidx(g, wrapm(gx, g.I), wrapm(y0 + cy, g.J), z0 + cz)]);
      atomicAdd(dst, make_float4(v[0], v[1], v[2], v[3]));
    }
    return;
  }
  for (int q = threadIdx.x; q < nbox; q += blockDim.x) {
    const float v = cell(q);
    if (v != 0.f) {
      const int cz = q / nxy, r = q - cz * nxy, cy = r / nbx, cx = r - cy * nbx;
      atomicAdd(&F[fidx(g, wrapm(x0 + cx, g.I), wrapm(y0 + cy, g.J), z0 + cz)], v);
    }
  }
}
void launch_ibm_spread_f(cudaStream_t s, const Geo &g, const PartGeo &pg, IbmBuffers b, float *fu, float *fv,
                         float *fw, double dt, const LearnedForce &lf, const int *gate) {
  if (pg.np == 0) return;
  const double coeff0 = (pg.dVlagr / pg.dVeul) * dt;
  auto go = [&](auto kern) {
    kern<<<dim3(pg.np, 3), SPREAD_THREADS, pg.box_cap * sizeof(float), s>>>(g, pg, b, fu, fv, fw, 1. / dt, coeff0, lf,
                                                                          gate, dt);
  };
  if (lf.Y) go(k_ibm_spread_f<true>);
  else go(k_ibm_spread_f<false>);
}
void launch_ibm_force_sums(cudaStream_t s, const PartGeo &pg, IbmBuffers b) {
  if (pg.np == 0) return;
  k_ibm_force_sums<<<(pg.np + 127) / 128, 128, 0, s>>>(pg, b, nullptr);
}

// ---------------------------------------------------------------------------
// Learned forcing.  Features of each point from the field before the
// forcing of the substep (the state the first pass interpolates), 32 per
// velocity component c = u, v, w at [32c + k]:
//   k = 0..26   the component at stencil tap q = (kz*3 + jy)*3 + ix minus U_c
//   k = 27      slip U_c - u~_c            k = 28  rigid-body velocity U_c
//   k = 29      outward unit normal (c)    k = 30  first-pass force F0_c*dt
//   k = 31      centre delta weight of the component's own axis
// X receives them standardised with (mu, isig) and rounded to BF16 for the
// network.  The interpolated velocity goes to dudtl as eulr2lagr would;
// with first_force the first pass's point force F0 = (U - u~)/dt as well
// (complagrforces), so the feature kernel is that pass's interpolation.
// k_ibm_features_f (one thread per point, all components) serves the
// harvest, which also stores every stride-th point's raw FP32 features and
// index for the target written after the plain passes; the learned loop
// forms the same features inside the tensor-core inference kernel.
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

__global__ void __launch_bounds__(256, 2) k_ibm_features_f(Geo g, PartGeo pg, IbmBuffers b, const float *__restrict__ fu,
                                                        const float *__restrict__ fv, const float *__restrict__ fw,
                                                        double dt, double dti, float inv_r,
                                                        const float *__restrict__ mu,
                                                        const float *__restrict__ isig,
                                                        __nv_bfloat16 *__restrict__ X, HarvestArgs H,
                                                        int first_force) {
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
    if (H.feat && (t + H.phase) % H.stride == 0) {
      const int h = atomicAdd(&H.count[0], 1);
      if (h < H.cap) {
        snk.raw = H.feat + (long)h * 96;
        H.pidx[h] = t;
      }
    }
    const int4 ref = b.pref[p];
    const PointRec rr = b.rec[t];
    auto tap = [&](const float *F, const CompStencil &s, int i, int j, int k) {
      return __ldg(&F[fidx(g, wrapm(ref.x + s.b[0] + i, g.I), wrapm(ref.y + s.b[1] + j, g.J), s.b[2] + k)]);
    };
    const double *pf = b.pf;
    const double Up[3] = {pf[PF_U * pg.np + p], pf[PF_V * pg.np + p], pf[PF_W * pg.np + p]};
    const double *Ua[3] = {b.ul, b.vl, b.wl};
    if (!snk.x && !snk.raw) {  // interpolation (and the first-pass force) only
      for (int c = 0; c < 3; ++c) {
        const CompStencil s = make_cs(rr, c, ref.z, g.K);
        const float a = interp27(s, [&](int i, int j, int k) { return tap(c == 0 ? fu : (c == 1 ? fv : fw), s, i, j, k); });
        (c == 0 ? b.dudtl : (c == 1 ? b.dvdtl : b.dwdtl))[t] = a;
        if (first_force)
          (c == 0 ? b.fxs : (c == 1 ? b.fys : b.fzs))[t] = (float)((point_u(pg, Ua[c], Up[c], t) - a) * dti);
      }
      continue;
    }
    const float4 cf = b.pcen[p];
    const float ir = pg.poly ? (float)(1. / pg.pradfp[p]) : inv_r;  // the sphere's own shell when polydisperse
    const float nrm[3] = {rec_armf(rec_dx(rr.rel), rr.fx, cf.x, (float)g.dx) * ir,
                          rec_armf(rec_dy(rr.rel), rr.fy, cf.y, (float)g.dy) * ir,
                          rec_armf(rec_dz(rr.rel), rr.fz, cf.z, (float)g.dz) * ir};
    const float *F3[3] = {fu, fv, fw};
    double *D3[3] = {b.dudtl, b.dvdtl, b.dwdtl};
    float *Fl3[3] = {b.fxs, b.fys, b.fzs};
#pragma unroll 1
    for (int c = 0; c < 3; ++c) {
      const CompStencil s = make_cs(rr, c, ref.z, g.K);
      const double Ud = point_u(pg, Ua[c], Up[c], t);
      const float Uc = (float)Ud;
      float acc = 0.f;
#pragma unroll
      for (int k = 0; k < 3; ++k)
#pragma unroll
        for (int j = 0; j < 3; ++j) {
          const float wyz = s.w[3 + j] * s.w[6 + k];
#pragma unroll
          for (int i = 0; i < 3; ++i) {
            const float tv = tap(F3[c], s, i, j, k);
            acc += tv * (s.w[i] * wyz);
            snk.put(tv - Uc);
          }
        }
      D3[c][t] = acc;
      if (first_force) Fl3[c][t] = (float)((Ud - acc) * dti);
      snk.put(Uc - acc);
      snk.put(Uc);
      snk.put(nrm[c]);
      snk.put(Fl3[c][t] * (float)dt);
      snk.put(s.w[3 * c + 1]);
    }
  }
}
void launch_ibm_features_f(cudaStream_t s, const Geo &g, const PartGeo &pg, IbmBuffers b, const float *fu,
                           const float *fv, const float *fw, double dt, const float *mu, const float *isig,
                           __nv_bfloat16 *X, const HarvestArgs &H, int first_force) {
  if (pg.np == 0) return;
  // reciprocals on the host: an FP64 division in every thread costs more
  // than the kernel's per-point FP64 work
  k_ibm_features_f<<<1216, 256, 0, s>>>(g, pg, b, fu, fv, fw, dt, 1. / dt, (float)(1. / pg.radfp), mu, isig, X, H,
                                        first_force);
}

// the box kernels' dynamic shared memory, raised (never lowered: other
// contexts may use larger boxes) to box_cap cells
int ibm_set_smem_limits(int box_cap) {
  static int cur = 0;
  if (box_cap <= cur) return 0;
  cudaError_t e1 = cudaFuncSetAttribute(k_ibm_spread_f<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        box_cap * (int)sizeof(float));
  if (e1 == cudaSuccess)
    e1 = cudaFuncSetAttribute(k_ibm_spread_f<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              box_cap * (int)sizeof(float));
  cudaError_t e2 = cudaSuccess;
  for (auto k : {k_ibm_interp_comp_f<1, false>, k_ibm_interp_comp_f<0, false>, k_ibm_interp_comp_f<-1, false>,
                 k_ibm_interp_comp_f<-2, false>, k_ibm_interp_comp_f<1, true>, k_ibm_interp_comp_f<0, true>,
                 k_ibm_interp_comp_f<-1, true>, k_ibm_interp_comp_f<-2, true>})
    if (e2 == cudaSuccess)
      e2 = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, box_cap * (int)sizeof(float));
  if (e1 != cudaSuccess || e2 != cudaSuccess) return -1;
  cur = box_cap;
  return 0;
}

}  // namespace ibmk
