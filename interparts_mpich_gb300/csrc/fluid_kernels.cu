// fluid_kernels.cu -- momentum predictor, velocity correction, boundary
// conditions, layout conversion and the chkdiv/chkdt reductions.
//
// One thread per interior cell; x/y neighbours by periodic wrap, z ghosts
// stored.  All arithmetic follows the reference expression order; FP64
// fused multiply-add contraction is allowed (differences at 1 ulp level).
#include <cuda.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstdint>

#include "kernels.cuh"

namespace ibmk {

// ---------------------------------------------------------------------------
// Momentum predictor: rk1/rk2/rk3 (rk3.f90:13-329) fused with momxp..momzad
// (mom.f90:8-231).  STAGE 1: dudt = u + f1*gradp; dudt += f1*RHS; rhs_old=RHS
// STAGE 2/3: dudt = u + f1*gradp; dudt += (f2*RHS - f3*rhs_old); stage 2
// stores rhs_old = RHS.  The output goes straight into the forcing buffer
// (dudtf == dudt on entry of the IBM loop, main.f90:288-306).
// ---------------------------------------------------------------------------
template <typename TU, typename T, int STAGE>
__global__ void __launch_bounds__(256) k_predict(Geo g, const TU *__restrict__ u, const TU *__restrict__ v,
                                                 const TU *__restrict__ w, const TU *__restrict__ p,
                                                 T *__restrict__ ru, T *__restrict__ rv, T *__restrict__ rw,
                                                 T *__restrict__ fu, T *__restrict__ fv, T *__restrict__ fw,
                                                 T f1, T f2, T f3, const double *__restrict__ cb, double bcoef) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int k = blockIdx.z + 1;
  if (i >= g.I || j >= g.J) return;
  // neighbours as 32-bit offsets from one 64-bit cell address (periodic
  // wrap in x and y folded into the offsets)
  const int dip = i + 1 == g.I ? 1 - g.I : 1, dim = i == 0 ? g.I - 1 : -1;
  const int djp = (j + 1 == g.J ? 1 - g.J : 1) * g.I, djm = (j == 0 ? g.J - 1 : -1) * g.I;
  const int PL = g.I * g.J;
  const long c = fidx(g, i, j, k);
  const int ip = dip, im = dim, jp = djp, jm = djm;
  auto at = [&](int di, int dj, int dk) -> long { return c + (di + dj + dk); };
  const int j0 = 0, i0 = 0;
  const int kp = PL, km = -PL;
  const T dxi = (T)g.dxi, dyi = (T)g.dyi, dzi = (T)g.dzi, visc = (T)g.visc;
  const T q = (T)0.25;
  // u-neighbourhood
  const T U0 = (T)u[c], Uip = (T)u[at(ip, j0, 0)], Uim = (T)u[at(im, j0, 0)], Ujp = (T)u[at(i0, jp, 0)],
          Ujm = (T)u[at(i0, jm, 0)];
  const T Ukp = (T)u[c + PL], Ukm = (T)u[c - PL];
  const T V0 = (T)v[c], Vip = (T)v[at(ip, j0, 0)], Vim = (T)v[at(im, j0, 0)], Vjp = (T)v[at(i0, jp, 0)],
          Vjm = (T)v[at(i0, jm, 0)];
  const T Vkp = (T)v[c + PL], Vkm = (T)v[c - PL];
  const T W0 = (T)w[c], Wip = (T)w[at(ip, j0, 0)], Wim = (T)w[at(im, j0, 0)], Wjp = (T)w[at(i0, jp, 0)],
          Wjm = (T)w[at(i0, jm, 0)];
  const T Wkp = (T)w[c + PL], Wkm = (T)w[c - PL];
  // diagonal neighbours
  const T Vipjm = (T)v[at(ip, jm, 0)], Wipkm = (T)w[at(ip, j0, km)];
  const T Uimjp = (T)u[at(im, jp, 0)], Wjpkm = (T)w[at(i0, jp, km)];
  const T Uimkp = (T)u[at(im, j0, kp)], Vjmkp = (T)v[at(i0, jm, kp)];
  // momxad (mom.f90:21-50)
  T ru_new;
  {
    const T uuip = q * (Uip + U0) * (Uip + U0);
    const T uuim = q * (Uim + U0) * (Uim + U0);
    const T uvjp = q * (Ujp + U0) * (Vip + V0);
    const T uvjm = q * (Ujm + U0) * (Vipjm + Vjm);
    const T uwkp = q * (Ukp + U0) * (Wip + W0);
    const T uwkm = q * (Ukm + U0) * (Wipkm + Wkm);
    const T dudxp = (Uip - U0) * dxi, dudxm = (U0 - Uim) * dxi;
    const T dudyp = (Ujp - U0) * dyi, dudym = (U0 - Ujm) * dyi;
    const T dudzp = (Ukp - U0) * dzi, dudzm = (U0 - Ukm) * dzi;
    ru_new = dxi * (-uuip + uuim) + visc * (dudxp - dudxm) * dxi + dyi * (-uvjp + uvjm) +
             visc * (dudyp - dudym) * dyi + dzi * (-uwkp + uwkm) + visc * (dudzp - dudzm) * dzi;
  }
  T rv_new;
  {  // momyad (mom.f90:94-123)
    const T uvip = q * (U0 + Ujp) * (V0 + Vip);
    const T uvim = q * (Uim + Uimjp) * (V0 + Vim);
    const T vvjp = q * (V0 + Vjp) * (V0 + Vjp);
    const T vvjm = q * (V0 + Vjm) * (V0 + Vjm);
    const T wvkp = q * (W0 + Wjp) * (Vkp + V0);
    const T wvkm = q * (Wkm + Wjpkm) * (Vkm + V0);
    const T dvdxp = (Vip - V0) * dxi, dvdxm = (V0 - Vim) * dxi;
    const T dvdyp = (Vjp - V0) * dyi, dvdym = (V0 - Vjm) * dyi;
    const T dvdzp = (Vkp - V0) * dzi, dvdzm = (V0 - Vkm) * dzi;
    rv_new = dxi * (-uvip + uvim) + visc * (dvdxp - dvdxm) * dxi + dyi * (-vvjp + vvjm) +
             visc * (dvdyp - dvdym) * dyi + dzi * (-wvkp + wvkm) + visc * (dvdzp - dvdzm) * dzi;
  }
  T rw_new;
  {  // momzad (mom.f90:170-199)
    const T uwip = q * (W0 + Wip) * (U0 + Ukp);
    const T uwim = q * (W0 + Wim) * (Uim + Uimkp);
    const T vwjp = q * (W0 + Wjp) * (V0 + Vkp);
    const T vwjm = q * (W0 + Wjm) * (Vjm + Vjmkp);
    const T wwkp = q * (W0 + Wkp) * (W0 + Wkp);
    const T wwkm = q * (W0 + Wkm) * (W0 + Wkm);
    const T dwdxp = (Wip - W0) * dxi, dwdxm = (W0 - Wim) * dxi;
    const T dwdyp = (Wjp - W0) * dyi, dwdym = (W0 - Wjm) * dyi;
    const T dwdzp = (Wkp - W0) * dzi, dwdzm = (W0 - Wkm) * dzi;
    rw_new = dxi * (-uwip + uwim) + visc * (dwdxp - dwdxm) * dxi + dyi * (-vwjp + vwjm) +
             visc * (dwdyp - dwdym) * dyi + dzi * (-wwkp + wwkm) + visc * (dwdzp - dwdzm) * dzi;
  }
  // momzbuoy (mom.f90:251), added as rk1..rk3 do (rk3.f90:56-58)
  if (cb) rw_new = (T)(bcoef * (cb[c] + cb[c + PL])) + rw_new;
  // pressure gradient (momxp/momyp/momzp)
  const T P0 = (T)p[c];
  const T gx = -dxi * ((T)p[at(ip, j0, 0)] - P0);
  const T gy = -dyi * ((T)p[at(i0, jp, 0)] - P0);
  const T gz = -dzi * ((T)p[c + PL] - P0);
  T du = U0 + f1 * gx, dv = V0 + f1 * gy, dw = W0 + f1 * gz;
  if (STAGE == 1) {
    du = du + f1 * ru_new;
    dv = dv + f1 * rv_new;
    dw = dw + f1 * rw_new;
  } else {
    du = du + (f2 * ru_new - f3 * ru[c]);
    dv = dv + (f2 * rv_new - f3 * rv[c]);
    dw = dw + (f2 * rw_new - f3 * rw[c]);
  }
  fu[c] = du;
  fv[c] = dv;
  fw[c] = dw;
  if (STAGE != 3) {
    ru[c] = ru_new;
    rv[c] = rv_new;
    rw[c] = rw_new;
  }
}

// FP32 predictor with 2.5D blocking: a 32 x 8 column tile marches along z
// through a chunk of planes, keeping the planes k-1, k, k+1 of u, v, w and
// k, k+1 of p (with a one-cell x/y halo, periodic) in shared memory, so each
// field is read from HBM about once.  The terms of k_predict, regrouped (below).
constexpr int PTX = 32, PTY = 8, PHX = PTX + 2, PHY = PTY + 2, PKC = 32;
// BUOY: momzbuoy from the scalar field cb (FP64).  A separate instantiation
// keeps the FP64 buoyancy instructions out of the kernel without a scalar:
// issued under a false predicate they still take FP64 issue slots, which on
// this GPU run at 1/64 of the FP32 rate.
template <int STAGE, bool BUOY>
__global__ void __launch_bounds__(PTX *PTY) k_predict_tiled(Geo g, const float *__restrict__ u,
                                                            const float *__restrict__ v,
                                                            const float *__restrict__ w,
                                                            const float *__restrict__ p, float *__restrict__ ru,
                                                            float *__restrict__ rv, float *__restrict__ rw,
                                                            float *__restrict__ fu, float *__restrict__ fv,
                                                            float *__restrict__ fw, float f1, float f2, float f3,
                                                            const double *__restrict__ cb, double bcoef) {
  __shared__ float su[3][PHY][PHX], sv[3][PHY][PHX], sw[3][PHY][PHX], sp[2][PHY][PHX];
  const int tx = threadIdx.x % PTX, ty = threadIdx.x / PTX;
  const int i0 = blockIdx.x * PTX, j0 = blockIdx.y * PTY;
  const int k0 = 1 + blockIdx.z * PKC, k1 = min(g.K, k0 + PKC - 1);
  const int i = i0 + tx, j = j0 + ty;
  const bool in = i < g.I && j < g.J;
  const int PL = g.I * g.J;  // 32-bit offsets: launched only for fields < 2^31 cells
  // this thread's halo elements (at most two of the PHY*PHX) and their
  // in-plane offsets, periodic in x and y (full wrap: tiles wider than the
  // grid reach beyond one period)
  constexpr int NH = PHY * PHX, NT = PTX * PTY;
  int hoff[2], hyx[2];
  bool has[2];
  for (int q = 0; q < 2; ++q) {
    const int e = threadIdx.x + q * NT;
    has[q] = e < NH;
    const int hy = has[q] ? e / PHX : 0, hx = has[q] ? e - hy * PHX : 0;
    int gi = (i0 - 1 + hx) % g.I, gj = (j0 - 1 + hy) % g.J;
    if (gi < 0) gi += g.I;
    if (gj < 0) gj += g.J;
    hoff[q] = gj * g.I + gi;
    hyx[q] = hy * PHX + hx;
  }
  // next plane in registers (u, v, w, p for each halo element)
  float nu[2], nv[2], nw[2], np_[2];
  auto fetch = [&](int kk) {
    for (int q = 0; q < 2; ++q)
      if (has[q]) {
        const int o = kk * PL + hoff[q];
        nu[q] = u[o]; nv[q] = v[o]; nw[q] = w[o]; np_[q] = p[o];
      }
  };
  auto commit = [&](int kk) {
    for (int q = 0; q < 2; ++q)
      if (has[q]) {
        (&su[kk % 3][0][0])[hyx[q]] = nu[q];
        (&sv[kk % 3][0][0])[hyx[q]] = nv[q];
        (&sw[kk % 3][0][0])[hyx[q]] = nw[q];
        (&sp[kk % 2][0][0])[hyx[q]] = np_[q];
      }
  };
  fetch(k0 - 1);
  commit(k0 - 1);
  fetch(k0);
  commit(k0);
  fetch(k0 + 1);
  const float dxi = (float)g.dxi, dyi = (float)g.dyi, dzi = (float)g.dzi, visc = (float)g.visc;
  const float qdxi = 0.25f * dxi, qdyi = 0.25f * dyi, qdzi = 0.25f * dzi;
  const float vdx2 = visc * dxi * dxi, vdy2 = visc * dyi * dyi, vdz2 = visc * dzi * dzi;
  for (int k = k0; k <= k1; ++k) {
    commit(k + 1);  // slots of k-2 (u, v, w) and k-1 (p) are free
    __syncthreads();
    if (k + 1 <= k1) fetch(k + 2);  // in flight while plane k is computed
    if (in) {
      const int cm = (k - 1) % 3, c0 = k % 3, cp = (k + 1) % 3;
      const int x = tx + 1, y = ty + 1;
      const float U0 = su[c0][y][x], Uip = su[c0][y][x + 1], Uim = su[c0][y][x - 1], Ujp = su[c0][y + 1][x],
                  Ujm = su[c0][y - 1][x], Ukp = su[cp][y][x], Ukm = su[cm][y][x];
      const float V0 = sv[c0][y][x], Vip = sv[c0][y][x + 1], Vim = sv[c0][y][x - 1], Vjp = sv[c0][y + 1][x],
                  Vjm = sv[c0][y - 1][x], Vkp = sv[cp][y][x], Vkm = sv[cm][y][x];
      const float W0 = sw[c0][y][x], Wip = sw[c0][y][x + 1], Wim = sw[c0][y][x - 1], Wjp = sw[c0][y + 1][x],
                  Wjm = sw[c0][y - 1][x], Wkp = sw[cp][y][x], Wkm = sw[cm][y][x];
      const float Vipjm = sv[c0][y - 1][x + 1], Wipkm = sw[cm][y][x + 1];
      const float Uimjp = su[c0][y + 1][x - 1], Wjpkm = sw[cm][y + 1][x];
      const float Uimkp = su[cp][y][x - 1], Vjmkp = sv[cp][y - 1][x];
      // momxad, momyad, momzad (mom.f90:21-50, 94-123, 170-199), the same
      // terms regrouped for the FP32 pipes: each of the three mixed products
      // that two equations share is formed once; q (a + b)^2 - q (c + d)^2
      // as one FMA; the diffusion from neighbour differences, which are
      // exact for neighbouring values within a factor of two.
      const float Puv = (Ujp + U0) * (Vip + V0);  // momx uvjp, momy uvip
      const float Puw = (Ukp + U0) * (Wip + W0);  // momx uwkp, momz uwip
      const float Pvw = (Wjp + W0) * (Vkp + V0);  // momy wvkp, momz vwjp
      float ru_new, rv_new, rw_new;
      {
        const float sp_ = Uip + U0, sm_ = Uim + U0;
        ru_new = qdxi * fmaf(sm_, sm_, -(sp_ * sp_)) + qdyi * ((Ujm + U0) * (Vipjm + Vjm) - Puv) +
                 qdzi * ((Ukm + U0) * (Wipkm + Wkm) - Puw) + vdx2 * ((Uip - U0) - (U0 - Uim)) +
                 vdy2 * ((Ujp - U0) - (U0 - Ujm)) + vdz2 * ((Ukp - U0) - (U0 - Ukm));
      }
      {
        const float sp_ = V0 + Vjp, sm_ = V0 + Vjm;
        rv_new = qdxi * ((Uim + Uimjp) * (V0 + Vim) - Puv) + qdyi * fmaf(sm_, sm_, -(sp_ * sp_)) +
                 qdzi * ((Wkm + Wjpkm) * (Vkm + V0) - Pvw) + vdx2 * ((Vip - V0) - (V0 - Vim)) +
                 vdy2 * ((Vjp - V0) - (V0 - Vjm)) + vdz2 * ((Vkp - V0) - (V0 - Vkm));
      }
      {
        const float sp_ = W0 + Wkp, sm_ = W0 + Wkm;
        rw_new = qdxi * ((W0 + Wim) * (Uim + Uimkp) - Puw) + qdyi * ((W0 + Wjm) * (Vjm + Vjmkp) - Pvw) +
                 qdzi * fmaf(sm_, sm_, -(sp_ * sp_)) + vdx2 * ((Wip - W0) - (W0 - Wim)) +
                 vdy2 * ((Wjp - W0) - (W0 - Wjm)) + vdz2 * ((Wkp - W0) - (W0 - Wkm));
      }
      // pressure gradient (momxp/momyp/momzp)
      const float P0 = sp[k % 2][y][x];
      const float gx = -dxi * (sp[k % 2][y][x + 1] - P0);
      const float gy = -dyi * (sp[k % 2][y + 1][x] - P0);
      const float gz = -dzi * (sp[(k + 1) % 2][y][x] - P0);
      const int c = k * PL + j * g.I + i;
      if constexpr (BUOY) rw_new = (float)(bcoef * (cb[c] + cb[c + PL])) + rw_new;  // momzbuoy
      float du = U0 + f1 * gx, dv = V0 + f1 * gy, dw = W0 + f1 * gz;
      if (STAGE == 1) {
        du = du + f1 * ru_new;
        dv = dv + f1 * rv_new;
        dw = dw + f1 * rw_new;
      } else {
        du = du + (f2 * ru_new - f3 * ru[c]);
        dv = dv + (f2 * rv_new - f3 * rv[c]);
        dw = dw + (f2 * rw_new - f3 * rw[c]);
      }
      fu[c] = du;
      fv[c] = dv;
      fw[c] = dw;
      if (STAGE != 3) {
        ru[c] = ru_new;
        rv[c] = rv_new;
        rw[c] = rw_new;
      }
    }
    __syncthreads();  // slot (k-1) % 3 is reloaded next
  }
}

// The same stage with two x-neighbouring cells per thread in packed FP32x2
// arithmetic (one instruction for both cells; the x neighbours of the pair
// come from three aligned 8-byte shared loads instead of six): 64 x 8 cells
// per block.  Three kernels stage the planes differently and share the
// arithmetic (pair_cells), so that they agree bit for bit:
//   k_predict_quad  rows of 72 cells from x = i0 - 4, loaded as 16-byte
//                   quads through registers one plane ahead (the default);
//   k_predict_pair  rows of 66 cells, one 4-byte load per cell;
//   k_predict_tma   the k_predict_quad rows, copied by the tensor-memory
//                   accelerator into a ring of four planes per field.
constexpr int QTX = 64, QTY = 8, QHY = QTY + 2, QROW = QTX + 4;
constexpr int TBX = QTX + 8, TBY = QTY + 2;  // quad / TMA rows: 72 cells from x = i0 - 4, 10 rows from y = j0 - 1
__device__ __forceinline__ float2 f2(float a) { return make_float2(a, a); }
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 sub2(float2 a, float2 b) { return __fadd2_rn(a, make_float2(-b.x, -b.y)); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 ld2(const float *row, int idx) { return *reinterpret_cast<const float2 *>(row + idx); }
__device__ __forceinline__ float2 mid(float2 a, float2 b) { return make_float2(a.y, b.x); }

struct PairCoef {
  float2 qdxi, qdyi, qdzi, vdx2, vdy2, vdz2, mdxi, mdyi, mdzi, F1, F2, mF3;
  __device__ PairCoef(const Geo &g, float f1, float f2_, float f3) {
    const float dxi = (float)g.dxi, dyi = (float)g.dyi, dzi = (float)g.dzi, visc = (float)g.visc;
    qdxi = f2(0.25f * dxi); qdyi = f2(0.25f * dyi); qdzi = f2(0.25f * dzi);
    vdx2 = f2(visc * dxi * dxi); vdy2 = f2(visc * dyi * dyi); vdz2 = f2(visc * dzi * dzi);
    mdxi = f2(-dxi); mdyi = f2(-dyi); mdzi = f2(-dzi);
    F1 = f2(f1); F2 = f2(f2_); mF3 = f2(-f3);
  }
};
// Planes k-1 (m), k (0), k+1 (p) of u, v, w and k, k+1 of p in shared
// memory, rows of RS cells; the pair's first cell at column x of row y.
struct PairPlanes {
  const float *um, *u0, *up, *vm, *v0, *vp, *wm, *w0, *wp, *p0, *pp;
};
// momxad, momyad, momzad (mom.f90:21-50, 94-123, 170-199), momxp..momzp and
// the rk1..rk3 update of two cells (global index c, c + 1; 32-bit: the
// tiled kernels run on fields of fewer than 2^31 cells)
template <int STAGE, bool BUOY, int RS>
__device__ __forceinline__ void pair_cells(const PairPlanes &P, int x, int y, int c, int PL, const PairCoef &q,
                                           float *__restrict__ ru, float *__restrict__ rv, float *__restrict__ rw,
                                           float *__restrict__ fu, float *__restrict__ fv, float *__restrict__ fw,
                                           const double *__restrict__ cb, double bcoef) {
  auto row = [&](const float *f, int yy) { return f + yy * RS; };
  // u
  const float *ur = row(P.u0, y);
  const float2 U0 = ld2(ur, x), UL = ld2(ur, x - 2), UR = ld2(ur, x + 2);
  const float2 Uip = mid(U0, UR), Uim = mid(UL, U0);
  const float2 Ujp = ld2(row(P.u0, y + 1), x), Ujm = ld2(row(P.u0, y - 1), x);
  const float2 Ukp = ld2(row(P.up, y), x), Ukm = ld2(row(P.um, y), x);
  const float2 Uimjp = mid(ld2(row(P.u0, y + 1), x - 2), Ujp), Uimkp = mid(ld2(row(P.up, y), x - 2), Ukp);
  // v
  const float *vr = row(P.v0, y);
  const float2 V0 = ld2(vr, x), VL = ld2(vr, x - 2), VR = ld2(vr, x + 2);
  const float2 Vip = mid(V0, VR), Vim = mid(VL, V0);
  const float2 Vjp = ld2(row(P.v0, y + 1), x), Vjm = ld2(row(P.v0, y - 1), x);
  const float2 Vkp = ld2(row(P.vp, y), x), Vkm = ld2(row(P.vm, y), x);
  const float2 Vipjm = mid(Vjm, ld2(row(P.v0, y - 1), x + 2)), Vjmkp = ld2(row(P.vp, y - 1), x);
  // w
  const float *wr = row(P.w0, y);
  const float2 W0 = ld2(wr, x), WL = ld2(wr, x - 2), WR = ld2(wr, x + 2);
  const float2 Wip = mid(W0, WR), Wim = mid(WL, W0);
  const float2 Wjp = ld2(row(P.w0, y + 1), x), Wjm = ld2(row(P.w0, y - 1), x);
  const float2 Wkp = ld2(row(P.wp, y), x), Wkm = ld2(row(P.wm, y), x);
  const float2 Wipkm = mid(Wkm, ld2(row(P.wm, y), x + 2)), Wjpkm = ld2(row(P.wm, y + 1), x);
  // the terms of k_predict_tiled in packed arithmetic
  const float2 Puv = mul2(add2(Ujp, U0), add2(Vip, V0));
  const float2 Puw = mul2(add2(Ukp, U0), add2(Wip, W0));
  const float2 Pvw = mul2(add2(Wjp, W0), add2(Vkp, V0));
  auto lap = [&](float2 cc, float2 xp, float2 xm, float2 yp, float2 ym, float2 zp, float2 zm) {
    const float2 dx_ = sub2(sub2(xp, cc), sub2(cc, xm)), dy_ = sub2(sub2(yp, cc), sub2(cc, ym)),
                 dz_ = sub2(sub2(zp, cc), sub2(cc, zm));
    return fma2(q.vdx2, dx_, fma2(q.vdy2, dy_, mul2(q.vdz2, dz_)));
  };
  auto sqd = [&](float2 a, float2 b) { return fma2(a, a, mul2(f2(-1.f), mul2(b, b))); };  // a^2 - b^2
  float2 ru_new, rv_new, rw_new;
  {
    const float2 sp_ = add2(Uip, U0), sm_ = add2(Uim, U0);
    ru_new = fma2(q.qdxi, sqd(sm_, sp_),
                  fma2(q.qdyi, sub2(mul2(add2(Ujm, U0), add2(Vipjm, Vjm)), Puv),
                       fma2(q.qdzi, sub2(mul2(add2(Ukm, U0), add2(Wipkm, Wkm)), Puw),
                            lap(U0, Uip, Uim, Ujp, Ujm, Ukp, Ukm))));
  }
  {
    const float2 sp_ = add2(V0, Vjp), sm_ = add2(V0, Vjm);
    rv_new = fma2(q.qdxi, sub2(mul2(add2(Uim, Uimjp), add2(V0, Vim)), Puv),
                  fma2(q.qdyi, sqd(sm_, sp_),
                       fma2(q.qdzi, sub2(mul2(add2(Wkm, Wjpkm), add2(Vkm, V0)), Pvw),
                            lap(V0, Vip, Vim, Vjp, Vjm, Vkp, Vkm))));
  }
  {
    const float2 sp_ = add2(W0, Wkp), sm_ = add2(W0, Wkm);
    rw_new = fma2(q.qdxi, sub2(mul2(add2(W0, Wim), add2(Uim, Uimkp)), Puw),
                  fma2(q.qdyi, sub2(mul2(add2(W0, Wjm), add2(Vjm, Vjmkp)), Pvw),
                       fma2(q.qdzi, sqd(sm_, sp_), lap(W0, Wip, Wim, Wjp, Wjm, Wkp, Wkm))));
  }
  // pressure gradient (momxp/momyp/momzp)
  const float *pr = row(P.p0, y);
  const float2 P0 = ld2(pr, x);
  const float2 gx = mul2(q.mdxi, sub2(mid(P0, ld2(pr, x + 2)), P0));
  const float2 gy = mul2(q.mdyi, sub2(ld2(row(P.p0, y + 1), x), P0));
  const float2 gz = mul2(q.mdzi, sub2(ld2(row(P.pp, y), x), P0));
  if constexpr (BUOY) {
    rw_new.x = (float)(bcoef * (cb[c] + cb[c + PL])) + rw_new.x;  // momzbuoy
    rw_new.y = (float)(bcoef * (cb[c + 1] + cb[c + 1 + PL])) + rw_new.y;
  }
  float2 du = fma2(q.F1, gx, U0), dv = fma2(q.F1, gy, V0), dw = fma2(q.F1, gz, W0);
  if (STAGE == 1) {
    du = fma2(q.F1, ru_new, du);
    dv = fma2(q.F1, rv_new, dv);
    dw = fma2(q.F1, rw_new, dw);
  } else {
    const float2 ou = *reinterpret_cast<const float2 *>(ru + c), ov = *reinterpret_cast<const float2 *>(rv + c),
                 ow = *reinterpret_cast<const float2 *>(rw + c);
    du = add2(du, fma2(q.F2, ru_new, mul2(q.mF3, ou)));
    dv = add2(dv, fma2(q.F2, rv_new, mul2(q.mF3, ov)));
    dw = add2(dw, fma2(q.F2, rw_new, mul2(q.mF3, ow)));
  }
  *reinterpret_cast<float2 *>(fu + c) = du;
  *reinterpret_cast<float2 *>(fv + c) = dv;
  *reinterpret_cast<float2 *>(fw + c) = dw;
  if (STAGE != 3) {
    *reinterpret_cast<float2 *>(ru + c) = ru_new;
    *reinterpret_cast<float2 *>(rv + c) = rv_new;
    *reinterpret_cast<float2 *>(rw + c) = rw_new;
  }
}

#define PREDICT_ARGS                                                                                          \
  Geo g, const float *__restrict__ u, const float *__restrict__ v, const float *__restrict__ w,               \
      const float *__restrict__ p, float *__restrict__ ru, float *__restrict__ rv, float *__restrict__ rw,    \
      float *__restrict__ fu, float *__restrict__ fv, float *__restrict__ fw, float f1, float f2_, float f3,  \
      const double *__restrict__ cb, double bcoef, int kc

template <int STAGE, bool BUOY>
__global__ void __launch_bounds__(QTX / 2 * QTY, 3) k_predict_pair(PREDICT_ARGS) {
  // row layout: [pad, x = i0 - 1, x = i0 .. i0 + 63, x = i0 + 64, pad]
  __shared__ __align__(16) float su[3][QHY][QROW], sv[3][QHY][QROW], sw[3][QHY][QROW], sp[2][QHY][QROW];
  constexpr int NT = QTX / 2 * QTY, NH = QHY * (QTX + 2), HQ = (NH + NT - 1) / NT;
  const int tx = threadIdx.x % (QTX / 2), ty = threadIdx.x / (QTX / 2);
  const int i0 = blockIdx.x * QTX, j0 = blockIdx.y * QTY;
  const int k0 = 1 + blockIdx.z * kc, k1 = min(g.K, k0 + kc - 1);
  const int i = i0 + 2 * tx, j = j0 + ty;
  const bool in = i < g.I && j < g.J;  // I even: i + 1 < I as well
  const int PL = g.I * g.J;  // 32-bit offsets: launched only for fields < 2^31 cells
  int hoff[HQ], hyx[HQ];
  bool has[HQ];
#pragma unroll
  for (int q = 0; q < HQ; ++q) {
    const int e = threadIdx.x + q * NT;
    has[q] = e < NH;
    const int hy = has[q] ? e / (QTX + 2) : 0, hx = has[q] ? e - hy * (QTX + 2) : 0;
    int gi = (i0 - 1 + hx) % g.I, gj = (j0 - 1 + hy) % g.J;
    if (gi < 0) gi += g.I;
    if (gj < 0) gj += g.J;
    hoff[q] = gj * g.I + gi;
    hyx[q] = hy * QROW + hx + 1;
  }
  float nu[HQ], nv[HQ], nw[HQ], np_[HQ];
  auto fetch = [&](int kk) {
#pragma unroll
    for (int q = 0; q < HQ; ++q)
      if (has[q]) {
        const int o = kk * PL + hoff[q];
        nu[q] = u[o]; nv[q] = v[o]; nw[q] = w[o]; np_[q] = p[o];
      }
  };
  auto commit = [&](int kk) {
#pragma unroll
    for (int q = 0; q < HQ; ++q)
      if (has[q]) {
        (&su[kk % 3][0][0])[hyx[q]] = nu[q];
        (&sv[kk % 3][0][0])[hyx[q]] = nv[q];
        (&sw[kk % 3][0][0])[hyx[q]] = nw[q];
        (&sp[kk % 2][0][0])[hyx[q]] = np_[q];
      }
  };
  fetch(k0 - 1);
  commit(k0 - 1);
  fetch(k0);
  commit(k0);
  fetch(k0 + 1);
  const PairCoef cf(g, f1, f2_, f3);
  for (int k = k0; k <= k1; ++k) {
    commit(k + 1);
    __syncthreads();
    if (k + 1 <= k1) fetch(k + 2);
    if (in) {
      const int cm = (k - 1) % 3, c0 = k % 3, cp = (k + 1) % 3;
      const PairPlanes P{&su[cm][0][0], &su[c0][0][0], &su[cp][0][0], &sv[cm][0][0], &sv[c0][0][0],
                         &sv[cp][0][0], &sw[cm][0][0], &sw[c0][0][0], &sw[cp][0][0], &sp[k % 2][0][0],
                         &sp[(k + 1) % 2][0][0]};
      pair_cells<STAGE, BUOY, QROW>(P, 2 * tx + 2, ty + 1, k * PL + j * g.I + i, PL, cf, ru, rv, rw, fu,
                                    fv, fw, cb, bcoef);
    }
    __syncthreads();
  }
}

// Quads: the block's 18 x 10 quads of a plane (16-byte aligned with I a
// multiple of 4, so that a quad never straddles the periodic wrap, which is
// applied to whole quads) are read by its first 180 threads, one quad of
// each field per thread, into registers one plane ahead.
constexpr int QQX = TBX / 4, NQUAD = QQX * TBY;
template <int STAGE, bool BUOY>
__global__ void __launch_bounds__(QTX / 2 * QTY, 3) k_predict_quad(PREDICT_ARGS) {
  __shared__ __align__(16) float su[3][TBY][TBX], sv[3][TBY][TBX], sw[3][TBY][TBX], sp[2][TBY][TBX];
  const int tx = threadIdx.x % (QTX / 2), ty = threadIdx.x / (QTX / 2);
  const int i0 = blockIdx.x * QTX, j0 = blockIdx.y * QTY;
  const int k0 = 1 + blockIdx.z * kc, k1 = min(g.K, k0 + kc - 1);
  const int i = i0 + 2 * tx, j = j0 + ty;
  const bool in = i < g.I && j < g.J;
  const int PL = g.I * g.J;  // 32-bit offsets: launched only for fields < 2^31 cells
  const bool has = threadIdx.x < NQUAD;
  const int qy = threadIdx.x / QQX, qx = threadIdx.x - qy * QQX;
  const int gx = (((i0 - 4 + 4 * qx) % g.I) + g.I) % g.I, gy = (((j0 - 1 + qy) % g.J) + g.J) % g.J;
  const int qoff = gy * g.I + gx, qsm = qy * TBX + 4 * qx;
  float4 nu, nv, nw, np_;
  auto fetch = [&](int kk) {
    if (has) {
      const int o = kk * PL + qoff;
      nu = __ldg(reinterpret_cast<const float4 *>(u + o));
      nv = __ldg(reinterpret_cast<const float4 *>(v + o));
      nw = __ldg(reinterpret_cast<const float4 *>(w + o));
      np_ = __ldg(reinterpret_cast<const float4 *>(p + o));
    }
  };
  auto commit = [&](int kk) {
    if (has) {
      *reinterpret_cast<float4 *>(&su[kk % 3][0][0] + qsm) = nu;
      *reinterpret_cast<float4 *>(&sv[kk % 3][0][0] + qsm) = nv;
      *reinterpret_cast<float4 *>(&sw[kk % 3][0][0] + qsm) = nw;
      *reinterpret_cast<float4 *>(&sp[kk % 2][0][0] + qsm) = np_;
    }
  };
  fetch(k0 - 1);
  commit(k0 - 1);
  fetch(k0);
  commit(k0);
  fetch(k0 + 1);
  const PairCoef cf(g, f1, f2_, f3);
  for (int k = k0; k <= k1; ++k) {
    commit(k + 1);
    __syncthreads();
    if (k + 1 <= k1) fetch(k + 2);
    if (in) {
      const int cm = (k - 1) % 3, c0 = k % 3, cp = (k + 1) % 3;
      const PairPlanes P{&su[cm][0][0], &su[c0][0][0], &su[cp][0][0], &sv[cm][0][0], &sv[c0][0][0],
                         &sv[cp][0][0], &sw[cm][0][0], &sw[c0][0][0], &sw[cp][0][0], &sp[k % 2][0][0],
                         &sp[(k + 1) % 2][0][0]};
      pair_cells<STAGE, BUOY, TBX>(P, 2 * tx + 4, ty + 1, k * PL + j * g.I + i, PL, cf, ru, rv, rw, fu,
                                   fv, fw, cb, bcoef);
    }
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------
// The quad rows staged by the tensor-memory accelerator: one
// cp.async.bulk.tensor load per field and plane brings the block's 72 x 10
// box (x from i0 - 4, 16-byte aligned) from HBM into shared memory,
// completing on the slot's mbarrier.  Four slots per field hold the planes
// k-1, k, k+1 being read and k+2 in flight; the next load is issued into the
// slot of k-1 once the block has finished reading it.  Box cells outside the
// domain (filled with zeros by the copy) are patched with their periodic
// images by plain loads, fetched one plane ahead into registers.  Measured
// at 256^3 this stages no faster than the quads through registers (the
// waits for the copies stay on the critical path at every prefetch depth
// tried), so it is selectable (IBM_PREDICTOR_TMA), not the default.
// ---------------------------------------------------------------------------
constexpr int TSLOT = ((TBX * TBY * 4 + 127) / 128) * 128 / 4;     // floats per field slot (128-byte aligned)
constexpr int TNS = 4;                                             // slots per field
constexpr int TPATCH = (QTX + 2) * TBY;                            // cells of the box the stencils read
constexpr int TPQ = (TPATCH + QTX / 2 * QTY - 1) / (QTX / 2 * QTY);  // patch cells per thread
constexpr size_t TMA_SMEM = (size_t)TNS * 4 * TSLOT * 4 + 128;
struct TmaFields {
  CUtensorMap u, v, w, p;
};
namespace {
__device__ __forceinline__ uint32_t sm_addr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }
__device__ __forceinline__ bool tma_wait(uint64_t *bar, uint32_t parity) {
  for (long it = 0; it < (1L << 22); ++it) {
    uint32_t ok;
    asm volatile(
        "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(sm_addr(bar)), "r"(parity)
        : "memory");
    if (ok) return true;
  }
  return false;
}
__device__ __forceinline__ void tma_load_plane(const TmaFields &tm, float *slot, uint64_t *bar, int x, int y, int z) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(sm_addr(bar)), "r"(4 * TBX * TBY * 4)
               : "memory");
  const CUtensorMap *m[4] = {&tm.u, &tm.v, &tm.w, &tm.p};
#pragma unroll
  for (int f = 0; f < 4; ++f)
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
        "[%5];" ::"r"(sm_addr(slot + f * TSLOT)),
        "l"(reinterpret_cast<uint64_t>(m[f])), "r"(x), "r"(y), "r"(z), "r"(sm_addr(bar))
        : "memory");
}
}  // namespace

template <int STAGE, bool BUOY>
__global__ void __launch_bounds__(QTX / 2 * QTY, 3) k_predict_tma(PREDICT_ARGS, const __grid_constant__ TmaFields tm,
                                                                 int *__restrict__ err) {
  extern __shared__ __align__(128) unsigned char tma_sm[];
  float *sbase = reinterpret_cast<float *>((reinterpret_cast<uintptr_t>(tma_sm) + 127) & ~uintptr_t(127));
  __shared__ __align__(8) uint64_t bar[TNS];
  constexpr int NT = QTX / 2 * QTY;
  const int tx = threadIdx.x % (QTX / 2), ty = threadIdx.x / (QTX / 2);
  const int i0 = blockIdx.x * QTX, j0 = blockIdx.y * QTY;
  const int k0 = 1 + blockIdx.z * kc, k1 = min(g.K, k0 + kc - 1);
  const int pfirst = k0 - 1, plast = k1 + 1;  // planes this block reads
  const int i = i0 + 2 * tx, j = j0 + ty;
  const bool in = i < g.I && j < g.J;  // I even: i + 1 < I as well
  const int PL = g.I * g.J;  // 32-bit offsets: launched only for fields < 2^31 cells
  auto sidx = [&](int P) { return (P - pfirst) & (TNS - 1); };
  auto slot_of = [&](int P) { return sbase + sidx(P) * 4 * TSLOT; };
  auto parity_of = [&](int P) { return (uint32_t)(((P - pfirst) / TNS) & 1); };
  if (threadIdx.x == 0) {
    for (int q = 0; q < TNS; ++q) asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(sm_addr(&bar[q])));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  if (threadIdx.x == 0)
    for (int P = pfirst; P <= min(plast, pfirst + TNS - 1); ++P)
      tma_load_plane(tm, slot_of(P), &bar[sidx(P)], i0 - 4, j0 - 1, P);
  // box cells outside the domain that the stencils read: their periodic
  // images by plain loads (none in tiles away from the domain's edges).
  // Thread cell q is e = tid + q NT of the (QTX + 2) x TBY region from x =
  // i0 - 1; bit q of pmask marks the ones outside.
  auto patch_cell = [&](int q, int &hyx, int &off) {
    const int e = threadIdx.x + q * NT;
    const int hy = e / (QTX + 2), hx = e - hy * (QTX + 2) + 3;
    const int gx = i0 - 4 + hx, gy = j0 - 1 + hy;
    hyx = hy * TBX + hx;
    off = (((gy % g.J) + g.J) % g.J) * g.I + ((gx % g.I) + g.I) % g.I;
    return e < TPATCH && (gx < 0 || gx >= g.I || gy < 0 || gy >= g.J);
  };
  unsigned pmask = 0;
#pragma unroll
  for (int q = 0; q < TPQ; ++q) {
    int a, b;
    if (patch_cell(q, a, b)) pmask |= 1u << q;
  }
  const bool edge = __syncthreads_or(pmask != 0) != 0;  // the block patches cells
  float nu[TPQ], nv[TPQ], nw[TPQ], np_[TPQ];
  auto fetch = [&](int P) {
#pragma unroll
    for (int q = 0; q < TPQ; ++q)
      if (pmask & (1u << q)) {
        int a, b;
        patch_cell(q, a, b);
        const int o = P * PL + b;
        nu[q] = u[o]; nv[q] = v[o]; nw[q] = w[o]; np_[q] = p[o];
      }
  };
  auto commit = [&](int P) {
    float *sl = slot_of(P);
#pragma unroll
    for (int q = 0; q < TPQ; ++q)
      if (pmask & (1u << q)) {
        int a, b;
        patch_cell(q, a, b);
        sl[a] = nu[q];
        sl[TSLOT + a] = nv[q];
        sl[2 * TSLOT + a] = nw[q];
        sl[3 * TSLOT + a] = np_[q];
      }
  };
  // bounded wait on plane P, the same outcome in every thread
  bool failed = false;
  auto wait_plane = [&](int P) {
    const bool ok = tma_wait(&bar[sidx(P)], parity_of(P));
    failed = __syncthreads_or(!ok) != 0;
  };
  int issued = min(plast, pfirst + TNS - 1);  // last plane whose load is issued
  int waited = pfirst - 1;                    // last plane waited for
  fetch(pfirst);
  wait_plane(pfirst);
  waited = pfirst;
  if (!failed) {
    commit(pfirst);
    fetch(pfirst + 1);
    wait_plane(pfirst + 1);
    waited = pfirst + 1;
  }
  if (!failed) {
    commit(pfirst + 1);
    fetch(pfirst + 2);
  }
  const PairCoef cf(g, f1, f2_, f3);
  for (int k = k0; k <= k1 && !failed; ++k) {
    wait_plane(k + 1);
    if (failed) break;
    waited = k + 1;
    if (edge) {
      commit(k + 1);
      if (k + 2 <= plast) fetch(k + 2);
      __syncthreads();
    }
    if (in) {
      const float *Sm = slot_of(k - 1), *S0 = slot_of(k), *Sp = slot_of(k + 1);
      const PairPlanes P{Sm, S0, Sp, Sm + TSLOT, S0 + TSLOT, Sp + TSLOT, Sm + 2 * TSLOT, S0 + 2 * TSLOT,
                         Sp + 2 * TSLOT, S0 + 3 * TSLOT, Sp + 3 * TSLOT};
      pair_cells<STAGE, BUOY, TBX>(P, 2 * tx + 4, ty + 1, k * PL + j * g.I + i, PL, cf, ru, rv, rw, fu,
                                   fv, fw, cb, bcoef);
    }
    // the slot of plane k - 1 is free once every thread is past this point;
    // the patches written into it are ordered before the next copy into it
    if (pmask) asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();
    if (threadIdx.x == 0 && issued < plast) {
      ++issued;
      tma_load_plane(tm, slot_of(issued), &bar[sidx(issued)], i0 - 4, j0 - 1, issued);
    }
  }
  if (failed && threadIdx.x == 0) {
    // a copy did not complete within the limit: flag it, and give the copies
    // still in flight a bounded time to land before the block exits
    atomicExch(err, 1);
    for (int P = waited + 1; P <= issued; ++P) tma_wait(&bar[sidx(P)], parity_of(P));
  }
}

namespace {
PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = [] {
    void *f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      f = nullptr;
    return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(f);
  }();
  return fn;
}
// 3-D map of one FP32 cell field (I, J, K + 2), box 72 x 10 x 1
bool encode_field_map(CUtensorMap *m, const Geo &g, const float *f) {
  auto enc = tensor_map_encoder();
  if (!enc || (reinterpret_cast<uintptr_t>(f) & 15)) return false;
  const cuuint64_t dims[3] = {(cuuint64_t)g.I, (cuuint64_t)g.J, (cuuint64_t)(g.K + 2)};
  const cuuint64_t strides[2] = {(cuuint64_t)g.I * 4, (cuuint64_t)g.I * g.J * 4};
  const cuuint32_t box[3] = {(cuuint32_t)TBX, (cuuint32_t)TBY, 1};
  const cuuint32_t estr[3] = {1, 1, 1};
  return enc(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<float *>(f), dims, strides, box, estr,
             CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_NONE,
             CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}
// z chunks of a 2.5D predictor launch with nbs resident blocks per SM: the
// split that keeps the block waves fullest, net of the two halo planes each
// chunk reads in addition, chunks of at most maxkc planes
int predict_zchunk(const Geo &g, int nbs, int maxkc) {
  static int nsm = [] {
    int dev = 0, n = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    return n;
  }();
  const int tiles = ((g.I + QTX - 1) / QTX) * ((g.J + QTY - 1) / QTY), slots = std::max(1, nsm * nbs);
  int kc = g.K;
  double best = -1.;
  for (int nz = 1; nz <= std::min(g.K, 64); ++nz) {
    const int kcz = (g.K + nz - 1) / nz, nb = tiles * ((g.K + kcz - 1) / kcz);
    if (kcz > maxkc && nz < std::min(g.K, 64)) continue;
    const double waves = (double)nb / slots, eff = waves / std::ceil(waves) * kcz / (kcz + 2.);
    if (eff > best + 1e-9) { best = eff; kc = kcz; }
  }
  return kc;
}
int quad_blocks_per_sm() {
  static int n = [] {
    int nb = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_predict_quad<2, false>, QTX / 2 * QTY, 0) != cudaSuccess)
      return 3;
    return nb > 0 ? nb : 3;
  }();
  return n;
}
int tma_blocks_per_sm() {
  static int n = [] {
    int nb = 0;
    for (auto k : {k_predict_tma<1, false>, k_predict_tma<2, false>, k_predict_tma<3, false>,
                   k_predict_tma<1, true>, k_predict_tma<2, true>, k_predict_tma<3, true>})
      if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)TMA_SMEM) != cudaSuccess) return 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_predict_tma<2, false>, QTX / 2 * QTY, TMA_SMEM) !=
        cudaSuccess)
      return 0;
    return nb;
  }();
  return n;
}
}  // namespace

// The TMA-staged stage: false when it does not apply (rows not a multiple of
// 4 cells, no tensor-map encoder).
bool launch_predict_tma(cudaStream_t s, const Geo &g, int stage, const float *u, const float *v, const float *w,
                        const float *p, float *ru, float *rv, float *rw, float *fu, float *fv, float *fw, float a,
                        float b, float c, const double *cb, double bcoef, int *err) {
  if (!err || g.I % 4 != 0 || g.nfield >= (1L << 31)) return false;
  const int nbs = tma_blocks_per_sm();
  if (nbs <= 0) return false;
  TmaFields tm;
  if (!encode_field_map(&tm.u, g, u) || !encode_field_map(&tm.v, g, v) || !encode_field_map(&tm.w, g, w) ||
      !encode_field_map(&tm.p, g, p))
    return false;
  // at most 24 planes a chunk (measured fastest at 256^3)
  const int kc = predict_zchunk(g, nbs, 24);
  dim3 grd((g.I + QTX - 1) / QTX, (g.J + QTY - 1) / QTY, (g.K + kc - 1) / kc);
  auto go = [&](auto kern) {
    kern<<<grd, QTX / 2 * QTY, TMA_SMEM, s>>>(g, u, v, w, p, ru, rv, rw, fu, fv, fw, a, b, c, cb, bcoef, kc, tm, err);
  };
  if (cb) {
    if (stage == 1) go(k_predict_tma<1, true>);
    else if (stage == 2) go(k_predict_tma<2, true>);
    else go(k_predict_tma<3, true>);
  } else {
    if (stage == 1) go(k_predict_tma<1, false>);
    else if (stage == 2) go(k_predict_tma<2, false>);
    else go(k_predict_tma<3, false>);
  }
  return true;
}

template <typename TU, typename T>
void launch_predict(cudaStream_t s, const Geo &g, int stage, const TU *u, const TU *v, const TU *w, const TU *p,
                    T *ru, T *rv, T *rw, T *fu, T *fv, T *fw, double f1, double f2, double f3, const double *cb,
                    double bcoef, int kind, int *err) {
  if constexpr (sizeof(T) == 4 && sizeof(TU) == 4) {
    if (g.nfield < (1L << 31)) {
    const float a = (float)f1, b = (float)f2, c = (float)f3;
    if (kind == IBM_PREDICTOR_TMA &&
        launch_predict_tma(s, g, stage, u, v, w, p, ru, rv, rw, fu, fv, fw, a, b, c, cb, bcoef, err))
      return;
    const int kc = predict_zchunk(g, quad_blocks_per_sm(), 64);
    dim3 gq((g.I + QTX - 1) / QTX, (g.J + QTY - 1) / QTY, (g.K + kc - 1) / kc);
    auto goq = [&](auto kern) {
      kern<<<gq, QTX / 2 * QTY, 0, s>>>(g, u, v, w, p, ru, rv, rw, fu, fv, fw, a, b, c, cb, bcoef, kc);
    };
    if (g.I % 4 == 0 && (kind == IBM_PREDICTOR_AUTO || kind == IBM_PREDICTOR_TMA)) {
      if (cb) {
        if (stage == 1) goq(k_predict_quad<1, true>);
        else if (stage == 2) goq(k_predict_quad<2, true>);
        else goq(k_predict_quad<3, true>);
      } else {
        if (stage == 1) goq(k_predict_quad<1, false>);
        else if (stage == 2) goq(k_predict_quad<2, false>);
        else goq(k_predict_quad<3, false>);
      }
      return;
    }
    if (g.I % 2 == 0 && kind != IBM_PREDICTOR_CELLS) {
      if (cb) {
        if (stage == 1) goq(k_predict_pair<1, true>);
        else if (stage == 2) goq(k_predict_pair<2, true>);
        else goq(k_predict_pair<3, true>);
      } else {
        if (stage == 1) goq(k_predict_pair<1, false>);
        else if (stage == 2) goq(k_predict_pair<2, false>);
        else goq(k_predict_pair<3, false>);
      }
      return;
    }
    dim3 grd((g.I + PTX - 1) / PTX, (g.J + PTY - 1) / PTY, (g.K + PKC - 1) / PKC);
    auto go = [&](auto kern) { kern<<<grd, PTX * PTY, 0, s>>>(g, u, v, w, p, ru, rv, rw, fu, fv, fw, a, b, c, cb, bcoef); };
    if (cb) {
      if (stage == 1) go(k_predict_tiled<1, true>);
      else if (stage == 2) go(k_predict_tiled<2, true>);
      else go(k_predict_tiled<3, true>);
    } else {
      if (stage == 1) go(k_predict_tiled<1, false>);
      else if (stage == 2) go(k_predict_tiled<2, false>);
      else go(k_predict_tiled<3, false>);
    }
    return;
    }
  }
  dim3 blk(64, 4, 1);
  dim3 grd((g.I + 63) / 64, (g.J + 3) / 4, g.K);
  if (stage == 1)
    k_predict<TU, T, 1><<<grd, blk, 0, s>>>(g, u, v, w, p, ru, rv, rw, fu, fv, fw, (T)f1, (T)f2, (T)f3, cb, bcoef);
  else if (stage == 2)
    k_predict<TU, T, 2><<<grd, blk, 0, s>>>(g, u, v, w, p, ru, rv, rw, fu, fv, fw, (T)f1, (T)f2, (T)f3, cb, bcoef);
  else
    k_predict<TU, T, 3><<<grd, blk, 0, s>>>(g, u, v, w, p, ru, rv, rw, fu, fv, fw, (T)f1, (T)f2, (T)f3, cb, bcoef);
}
template void launch_predict<double, double>(cudaStream_t, const Geo &, int, const double *, const double *,
                                             const double *, const double *, double *, double *, double *,
                                             double *, double *, double *, double, double, double, const double *,
                                             double, int, int *);
template void launch_predict<float, float>(cudaStream_t, const Geo &, int, const float *, const float *,
                                           const float *, const float *, float *, float *, float *, float *,
                                           float *, float *, double, double, double, const double *, double, int,
                                           int *);

// ---------------------------------------------------------------------------
// Scalar: scalad (scal.f90:11-58) fused with the dcdt update of rk1..rk3
// (rk3.f90:48,78 / 151,188 / 266,300).  STAGE 1: cnext = c + f1*RHS,
// rhs_old = RHS; STAGE 2/3: cnext = c + (f2*RHS - f3*rhs_old), stage 2 stores
// rhs_old = RHS.  cnext becomes cnew after the projection (main.f90:374-376).
// ---------------------------------------------------------------------------
template <typename TU, int STAGE>
__global__ void __launch_bounds__(256) k_scalar_stage(Geo g, const TU *__restrict__ u, const TU *__restrict__ v,
                                                      const TU *__restrict__ w, const double *__restrict__ cf,
                                                      double *__restrict__ rc, double *__restrict__ cnext,
                                                      double kappa, double f1, double f2, double f3) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int k = blockIdx.z + 1;
  if (i >= g.I || j >= g.J) return;
  const long c = fidx(g, i, j, k);
  const long cip = fidx(g, i + 1 == g.I ? 0 : i + 1, j, k), cim = fidx(g, i == 0 ? g.I - 1 : i - 1, j, k);
  const long cjp = fidx(g, i, j + 1 == g.J ? 0 : j + 1, k), cjm = fidx(g, i, j == 0 ? g.J - 1 : j - 1, k);
  const long ckp = c + g.plane, ckm = c - g.plane;
  const double dxi = g.dxi, dyi = g.dyi, dzi = g.dzi;
  const double C0 = cf[c], Cip = cf[cip], Cim = cf[cim], Cjp = cf[cjp], Cjm = cf[cjm], Ckp = cf[ckp], Ckm = cf[ckm];
  const double ucip = 0.5 * (double)u[c] * (Cip + C0);
  const double ucim = 0.5 * (double)u[cim] * (C0 + Cim);
  const double vcjp = 0.5 * (double)v[c] * (Cjp + C0);
  const double vcjm = 0.5 * (double)v[cjm] * (C0 + Cjm);
  const double wckp = 0.5 * (double)w[c] * (Ckp + C0);
  const double wckm = 0.5 * (double)w[ckm] * (C0 + Ckm);
  const double dcdxp = (Cip - C0) * dxi, dcdxm = (C0 - Cim) * dxi;
  const double dcdyp = (Cjp - C0) * dyi, dcdym = (C0 - Cjm) * dyi;
  const double dcdzp = (Ckp - C0) * dzi, dcdzm = (C0 - Ckm) * dzi;
  const double rhs = dxi * (-ucip + ucim) + kappa * (dcdxp - dcdxm) * dxi + dyi * (-vcjp + vcjm) +
                     kappa * (dcdyp - dcdym) * dyi + dzi * (-wckp + wckm) + kappa * (dcdzp - dcdzm) * dzi;
  if (STAGE == 1) cnext[c] = C0 + f1 * rhs;
  else cnext[c] = C0 + (f2 * rhs - f3 * rc[c]);
  if (STAGE != 3) rc[c] = rhs;
}
template <typename TU>
void launch_scalar_stage(cudaStream_t s, const Geo &g, int stage, const TU *u, const TU *v, const TU *w,
                         const double *cf, double *rc, double *cnext, double kappa, double f1, double f2, double f3) {
  dim3 blk(64, 4, 1);
  dim3 grd((g.I + 63) / 64, (g.J + 3) / 4, g.K);
  if (stage == 1) k_scalar_stage<TU, 1><<<grd, blk, 0, s>>>(g, u, v, w, cf, rc, cnext, kappa, f1, f2, f3);
  else if (stage == 2) k_scalar_stage<TU, 2><<<grd, blk, 0, s>>>(g, u, v, w, cf, rc, cnext, kappa, f1, f2, f3);
  else k_scalar_stage<TU, 3><<<grd, blk, 0, s>>>(g, u, v, w, cf, rc, cnext, kappa, f1, f2, f3);
}
template void launch_scalar_stage<double>(cudaStream_t, const Geo &, int, const double *, const double *,
                                          const double *, const double *, double *, double *, double, double,
                                          double, double);
template void launch_scalar_stage<float>(cudaStream_t, const Geo &, int, const float *, const float *, const float *,
                                         const double *, double *, double *, double, double, double, double);

// boundscal (bound.f90:109-171): wall ghost planes of the scalar
__global__ void k_boundscal(Geo g, double *__restrict__ cf, int top_dirichlet, double top, int bot_dirichlet,
                            double bot) {
  for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < g.plane; e += (long)gridDim.x * blockDim.x) {
    const long t = (long)(g.K + 1) * g.plane + e, n = (long)g.K * g.plane + e;
    cf[t] = top_dirichlet ? 2 * top - cf[n] : cf[n];
    cf[e] = bot_dirichlet ? 2 * bot - cf[g.plane + e] : cf[g.plane + e];
  }
}
void launch_boundscal(cudaStream_t s, const Geo &g, double *cf, int top_dirichlet, double top, int bot_dirichlet,
                      double bot) {
  k_boundscal<<<(int)std::min<long>(1216, (g.plane + 255) / 256), 256, 0, s>>>(g, cf, top_dirichlet, top,
                                                                               bot_dirichlet, bot);
}

// ---------------------------------------------------------------------------
// correc (correc.f90:11-42) + pnew += p (main.f90:369-371) + bounduvw(unew)
// and boundp(pnew) z-ghosts (bound.f90:11-107).  phi holds the Poisson
// solution on planes 1..K; its Neumann ghost p(k1)=p(kmax) is implied.
// ---------------------------------------------------------------------------
template <typename TF, typename TPh, typename TU>
__global__ void __launch_bounds__(256) k_correc(Geo g, const TF *fu, const TF *fv, const TF *fw,
                                                const TPh *__restrict__ phi, TU *u, TU *v, TU *w,
                                                double *__restrict__ pn, float *__restrict__ pn32, double fi_,
                                                double fj_, double fk_) {
  // fu may alias u (the defect correction updates the state in place: each
  // thread reads and writes only its own cell of u/v/w)
  typedef TU T;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int k = blockIdx.z + 1;
  if (i >= g.I || j >= g.J) return;
  const int ip = i + 1 == g.I ? 0 : i + 1;
  const int jp = j + 1 == g.J ? 0 : j + 1;
  const long PL = g.plane;
  const long c = fidx(g, i, j, k);
  const T fi = (T)fi_, fj = (T)fj_, fk = (T)fk_;
  const T P0 = (T)phi[c];
  const T Pip = (T)phi[fidx(g, ip, j, k)];
  const T Pjp = (T)phi[fidx(g, i, jp, k)];
  if (g.zper) {  // periodic z: p(k1) = p(1); w(kmax) is an unknown; ghost planes are copies
    const T Pkp = (k == g.K) ? (T)phi[c - (long)(g.K - 1) * PL] : (T)phi[c + PL];
    const T un = (T)fu[c] - fi * (Pip - P0);
    const T vn = (T)fv[c] - fj * (Pjp - P0);
    const T wn = (T)fw[c] - fk * (Pkp - P0);
    u[c] = un;
    v[c] = vn;
    w[c] = wn;
    const double pnn = pn[c] + (double)phi[c];
    pn[c] = pnn;
    if (pn32) pn32[c] = (float)pnn;
    const long gh = k == 1 ? c + (long)g.K * PL : (k == g.K ? c - (long)g.K * PL : -1);
    if (gh >= 0) {  // plane 1 -> ghost k1, plane K -> ghost 0
      u[gh] = un;
      v[gh] = vn;
      w[gh] = wn;
      pn[gh] = pnn;
      if (pn32) pn32[gh] = (float)pnn;
    }
    return;
  }
  const T Pkp = (k == g.K) ? P0 : (T)phi[c + PL];
  const T un = (T)fu[c] - fi * (Pip - P0);
  const T vn = (T)fv[c] - fj * (Pjp - P0);
  const T wn = (k == g.K) ? (T)0 : (T)fw[c] - fk * (Pkp - P0);
  u[c] = un;
  v[c] = vn;
  w[c] = wn;
  const double pnn = pn[c] + (double)phi[c];
  pn[c] = pnn;
  if (pn32) pn32[c] = (float)pnn;
  if (k == g.K) {
    const T sg = g.bc_top == IBM_BC_NOSLIP ? (T)-1 : (T)1;
    u[c + PL] = sg * un;
    v[c + PL] = sg * vn;
    pn[c + PL] = pnn;
    if (pn32) pn32[c + PL] = (float)pnn;
  }
  if (k == 1) {
    const T sg = g.bc_bot == IBM_BC_NOSLIP ? (T)-1 : (T)1;
    u[c - PL] = sg * un;
    v[c - PL] = sg * vn;
    w[c - PL] = (T)0;
    pn[c - PL] = pnn;
    if (pn32) pn32[c - PL] = (float)pnn;
  }
}

template <typename TF, typename TPh, typename TU>
void launch_correc(cudaStream_t s, const Geo &g, const TF *fu, const TF *fv, const TF *fw, const TPh *phi, TU *u,
                   TU *v, TU *w, double *pn, float *pn32, double fi, double fj, double fk) {
  dim3 blk(64, 4, 1);
  dim3 grd((g.I + 63) / 64, (g.J + 3) / 4, g.K);
  k_correc<TF, TPh, TU><<<grd, blk, 0, s>>>(g, fu, fv, fw, phi, u, v, w, pn, pn32, fi, fj, fk);
}
template void launch_correc<double, double, double>(cudaStream_t, const Geo &, const double *, const double *,
                                                    const double *, const double *, double *, double *, double *,
                                                    double *, float *, double, double, double);
template void launch_correc<float, float, float>(cudaStream_t, const Geo &, const float *, const float *,
                                                 const float *, const float *, float *, float *, float *, double *,
                                                 float *, double, double, double);

// Mixed form of the same update: FP32 velocity; pnew carried as the
// double-float pair (ph, pl), ph doubling as the FP32 pressure that the
// predictor reads.  fu may alias u (defect correction in place).
__global__ void __launch_bounds__(256) k_correc_mixed(Geo g, const float *fu, const float *fv, const float *fw,
                                                      const float *__restrict__ phi, float *u, float *v, float *w,
                                                      float *__restrict__ ph, float *__restrict__ pl, float fi,
                                                      float fj, float fk) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int k = blockIdx.z + 1;
  if (i >= g.I || j >= g.J) return;
  const int ip = i + 1 == g.I ? 0 : i + 1;
  const int jp = j + 1 == g.J ? 0 : j + 1;
  const long PL = g.plane;
  const long c = fidx(g, i, j, k);
  const float P0 = phi[c];
  const float Pip = phi[fidx(g, ip, j, k)];
  const float Pjp = phi[fidx(g, i, jp, k)];
  const float Pkp = (k == g.K) ? P0 : phi[c + PL];
  const float un = fu[c] - fi * (Pip - P0);
  const float vn = fv[c] - fj * (Pjp - P0);
  const float wn = (k == g.K) ? 0.f : fw[c] - fk * (Pkp - P0);
  u[c] = un;
  v[c] = vn;
  w[c] = wn;
  float sh, sl;
  df_add(ph[c], pl[c], P0, 0.f, sh, sl);
  ph[c] = sh;
  pl[c] = sl;
  if (k == g.K) {
    const float sg = g.bc_top == IBM_BC_NOSLIP ? -1.f : 1.f;
    u[c + PL] = sg * un;
    v[c + PL] = sg * vn;
    ph[c + PL] = sh;
    pl[c + PL] = sl;
  }
  if (k == 1) {
    const float sg = g.bc_bot == IBM_BC_NOSLIP ? -1.f : 1.f;
    u[c - PL] = sg * un;
    v[c - PL] = sg * vn;
    w[c - PL] = 0.f;
    ph[c - PL] = sh;
    pl[c - PL] = sl;
  }
}
// correc with the defect correction folded in: u = u* - f grad(phi1 + phi2)
// and pnew += phi1 + phi2 (double-float), one pass over the fields
__global__ void __launch_bounds__(256) k_correc_mixed2(Geo g, const float *__restrict__ fu,
                                                       const float *__restrict__ fv, const float *__restrict__ fw,
                                                       const float *__restrict__ phi1,
                                                       const float *__restrict__ phi2, float *__restrict__ u,
                                                       float *__restrict__ v, float *__restrict__ w,
                                                       float *__restrict__ ph, float *__restrict__ pl, float fi,
                                                       float fj, float fk) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int k = blockIdx.z + 1;
  if (i >= g.I || j >= g.J) return;
  const int dip = i + 1 == g.I ? 1 - g.I : 1;
  const int djp = (j + 1 == g.J ? 1 - g.J : 1) * g.I;
  const long PL = g.plane;
  const long c = fidx(g, i, j, k);
  const float a0 = phi1[c], b0 = phi2[c];
  const float P0 = a0 + b0;
  const float Pip = phi1[c + dip] + phi2[c + dip];
  const float Pjp = phi1[c + djp] + phi2[c + djp];
  const float Pkp = (k == g.K) ? P0 : phi1[c + PL] + phi2[c + PL];
  const float un = fu[c] - fi * (Pip - P0);
  const float vn = fv[c] - fj * (Pjp - P0);
  const float wn = (k == g.K) ? 0.f : fw[c] - fk * (Pkp - P0);
  u[c] = un;
  v[c] = vn;
  w[c] = wn;
  float sh, sl;
  df_add(ph[c], pl[c], a0, 0.f, sh, sl);
  df_add(sh, sl, b0, 0.f, sh, sl);
  ph[c] = sh;
  pl[c] = sl;
  if (k == g.K) {
    const float sg = g.bc_top == IBM_BC_NOSLIP ? -1.f : 1.f;
    u[c + PL] = sg * un;
    v[c + PL] = sg * vn;
    ph[c + PL] = sh;
    pl[c + PL] = sl;
  }
  if (k == 1) {
    const float sg = g.bc_bot == IBM_BC_NOSLIP ? -1.f : 1.f;
    u[c - PL] = sg * un;
    v[c - PL] = sg * vn;
    w[c - PL] = 0.f;
    ph[c - PL] = sh;
    pl[c - PL] = sl;
  }
}
void launch_correc_mixed2(cudaStream_t s, const Geo &g, const float *fu, const float *fv, const float *fw,
                          const float *phi1, const float *phi2, float *u, float *v, float *w, float *ph, float *pl,
                          double fi, double fj, double fk) {
  dim3 blk(64, 4, 1);
  dim3 grd((g.I + 63) / 64, (g.J + 3) / 4, g.K);
  k_correc_mixed2<<<grd, blk, 0, s>>>(g, fu, fv, fw, phi1, phi2, u, v, w, ph, pl, (float)fi, (float)fj, (float)fk);
}

// The same update four x-cells per thread with 16-byte loads and stores
// (I a multiple of 4): identical arithmetic per cell, a quarter of the
// memory instructions.
__device__ __forceinline__ float4 ld4(const float *p) { return *reinterpret_cast<const float4 *>(p); }
__device__ __forceinline__ void st4(float *p, float4 v) { *reinterpret_cast<float4 *>(p) = v; }
__global__ void __launch_bounds__(256) k_correc_mixed4(Geo g, const float *fu, const float *fv, const float *fw,
                                                       const float *__restrict__ phi, float *u, float *v, float *w,
                                                       float *__restrict__ ph, float *__restrict__ pl, float fi,
                                                       float fj, float fk) {
  const int i0 = 4 * (blockIdx.x * blockDim.x + threadIdx.x);
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int k = blockIdx.z + 1;
  if (i0 >= g.I || j >= g.J) return;
  const int jp = j + 1 == g.J ? 0 : j + 1;
  const long PL = g.plane;
  const long c = fidx(g, i0, j, k);
  const float4 P0 = ld4(phi + c);
  const float P4 = phi[fidx(g, i0 + 4 == g.I ? 0 : i0 + 4, j, k)];
  const float4 Pjp = ld4(phi + fidx(g, i0, jp, k));
  const float4 Pkp = (k == g.K) ? P0 : ld4(phi + c + PL);
  const float4 FU = ld4(fu + c), FV = ld4(fv + c);
  const float4 FW = (k == g.K) ? make_float4(0.f, 0.f, 0.f, 0.f) : ld4(fw + c);
  const float p0[4] = {P0.x, P0.y, P0.z, P0.w}, pip[4] = {P0.y, P0.z, P0.w, P4};
  const float pjp[4] = {Pjp.x, Pjp.y, Pjp.z, Pjp.w}, pkp[4] = {Pkp.x, Pkp.y, Pkp.z, Pkp.w};
  const float fu4[4] = {FU.x, FU.y, FU.z, FU.w}, fv4[4] = {FV.x, FV.y, FV.z, FV.w}, fw4[4] = {FW.x, FW.y, FW.z, FW.w};
  const float4 H = ld4(ph + c), Lo = ld4(pl + c);
  const float h4[4] = {H.x, H.y, H.z, H.w}, l4[4] = {Lo.x, Lo.y, Lo.z, Lo.w};
  float un[4], vn[4], wn[4], sh[4], sl[4];
#pragma unroll
  for (int e = 0; e < 4; ++e) {
    un[e] = fu4[e] - fi * (pip[e] - p0[e]);
    vn[e] = fv4[e] - fj * (pjp[e] - p0[e]);
    wn[e] = (k == g.K) ? 0.f : fw4[e] - fk * (pkp[e] - p0[e]);
    df_add(h4[e], l4[e], p0[e], 0.f, sh[e], sl[e]);
  }
  const float4 U = make_float4(un[0], un[1], un[2], un[3]), V = make_float4(vn[0], vn[1], vn[2], vn[3]);
  const float4 W = make_float4(wn[0], wn[1], wn[2], wn[3]);
  const float4 SH = make_float4(sh[0], sh[1], sh[2], sh[3]), SL = make_float4(sl[0], sl[1], sl[2], sl[3]);
  st4(u + c, U);
  st4(v + c, V);
  st4(w + c, W);
  st4(ph + c, SH);
  st4(pl + c, SL);
  if (k == g.K) {
    const float sg = g.bc_top == IBM_BC_NOSLIP ? -1.f : 1.f;
    st4(u + c + PL, make_float4(sg * un[0], sg * un[1], sg * un[2], sg * un[3]));
    st4(v + c + PL, make_float4(sg * vn[0], sg * vn[1], sg * vn[2], sg * vn[3]));
    st4(ph + c + PL, SH);
    st4(pl + c + PL, SL);
  }
  if (k == 1) {
    const float sg = g.bc_bot == IBM_BC_NOSLIP ? -1.f : 1.f;
    st4(u + c - PL, make_float4(sg * un[0], sg * un[1], sg * un[2], sg * un[3]));
    st4(v + c - PL, make_float4(sg * vn[0], sg * vn[1], sg * vn[2], sg * vn[3]));
    st4(w + c - PL, make_float4(0.f, 0.f, 0.f, 0.f));
    st4(ph + c - PL, SH);
    st4(pl + c - PL, SL);
  }
}

void launch_correc_mixed(cudaStream_t s, const Geo &g, const float *fu, const float *fv, const float *fw,
                         const float *phi, float *u, float *v, float *w, float *ph, float *pl, double fi, double fj,
                         double fk) {
  if ((g.I & 3) == 0) {
    dim3 blk(64, 4, 1);
    dim3 grd((g.I / 4 + 63) / 64, (g.J + 3) / 4, g.K);
    k_correc_mixed4<<<grd, blk, 0, s>>>(g, fu, fv, fw, phi, u, v, w, ph, pl, (float)fi, (float)fj, (float)fk);
    return;
  }
  dim3 blk(64, 4, 1);
  dim3 grd((g.I + 63) / 64, (g.J + 3) / 4, g.K);
  k_correc_mixed<<<grd, blk, 0, s>>>(g, fu, fv, fw, phi, u, v, w, ph, pl, (float)fi, (float)fj, (float)fk);
}

// double-float pair <-> FP64 array
__global__ void k_df_to_d(long n, const float *__restrict__ h, const float *__restrict__ l, double *__restrict__ d) {
  for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < n; t += (long)gridDim.x * blockDim.x)
    d[t] = (double)h[t] + (double)l[t];
}
__global__ void k_d_to_df(long n, const double *__restrict__ d, float *__restrict__ h, float *__restrict__ l) {
  for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < n; t += (long)gridDim.x * blockDim.x) {
    const float hh = (float)d[t];
    h[t] = hh;
    l[t] = (float)(d[t] - (double)hh);
  }
}
void launch_df_to_d(cudaStream_t s, long n, const float *h, const float *l, double *d) {
  k_df_to_d<<<1216, 256, 0, s>>>(n, h, l, d);
}
void launch_d_to_df(cudaStream_t s, long n, const double *d, float *h, float *l) {
  k_d_to_df<<<1216, 256, 0, s>>>(n, d, h, l);
}

// ---------------------------------------------------------------------------
// Layout conversion between the reference host layout (0:i1,0:j1,0:k1) and
// the device layout.  to_dev: dev(i,j,k) = ref(i+1,j+1,k).  to_ref fills the
// x/y ghosts with the periodic values, as bounduvw/boundp leave them.
// ---------------------------------------------------------------------------
template <typename T>
__global__ void k_ref_to_dev(Geo g, const double *__restrict__ ref, T *__restrict__ dev) {
  const long n = g.nfield;
  for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < n; t += (long)gridDim.x * blockDim.x) {
    const int i = (int)(t % g.I);
    const int j = (int)((t / g.I) % g.J);
    const int k = (int)(t / g.plane);
    const long r = (long)(i + 1) + (long)(g.I + 2) * ((j + 1) + (long)(g.J + 2) * k);
    dev[t] = (T)ref[r];
  }
}
template <typename T>
__global__ void k_dev_to_ref(Geo g, const T *__restrict__ dev, double *__restrict__ ref) {
  const long n = (long)(g.I + 2) * (g.J + 2) * (g.K + 2);
  for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < n; t += (long)gridDim.x * blockDim.x) {
    const int i = (int)(t % (g.I + 2));
    const int j = (int)((t / (g.I + 2)) % (g.J + 2));
    const int k = (int)(t / ((long)(g.I + 2) * (g.J + 2)));
    const int id = wrapm(i - 1, g.I), jd = wrapm(j - 1, g.J);
    ref[t] = (double)dev[fidx(g, id, jd, k)];
  }
}
template <typename T>
void launch_ref_to_dev(cudaStream_t s, const Geo &g, const double *ref, T *dev) {
  k_ref_to_dev<T><<<1216, 256, 0, s>>>(g, ref, dev);
}
template <typename T>
void launch_dev_to_ref(cudaStream_t s, const Geo &g, const T *dev, double *ref) {
  k_dev_to_ref<T><<<1216, 256, 0, s>>>(g, dev, ref);
}
template void launch_ref_to_dev<double>(cudaStream_t, const Geo &, const double *, double *);
template void launch_ref_to_dev<float>(cudaStream_t, const Geo &, const double *, float *);
template void launch_dev_to_ref<double>(cudaStream_t, const Geo &, const double *, double *);
template void launch_dev_to_ref<float>(cudaStream_t, const Geo &, const float *, double *);

// ---------------------------------------------------------------------------
// chkdiv (chkdiv.f90:7-61): block partials of sum(div) and (max|div|, first
// linear index), combined in a fixed order by a single block.
// ---------------------------------------------------------------------------
template <typename T>
__global__ void __launch_bounds__(256) k_div_partial(Geo g, const T *__restrict__ u,
                                                     const T *__restrict__ v, const T *__restrict__ w,
                                                     double *__restrict__ psum, double *__restrict__ pmax,
                                                     long long *__restrict__ ploc) {
  const long n = (long)g.I * g.J * g.K;
  double s = 0., m = -1.;
  long long loc = -1;
  for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < n; t += (long)gridDim.x * blockDim.x) {
    const int i = (int)(t % g.I), j = (int)((t / g.I) % g.J), k = (int)(t / g.plane) + 1;
    const long c = fidx(g, i, j, k);
    const double div = ((double)w[c] - (double)w[c - g.plane]) * g.dzi +
                       ((double)v[c] - (double)v[fidx(g, i, wrapm(j - 1, g.J), k)]) * g.dyi +
                       ((double)u[c] - (double)u[fidx(g, wrapm(i - 1, g.I), j, k)]) * g.dxi;
    s += div;
    const double a = fabs(div);
    if (a > m) { m = a; loc = t; }
  }
  __shared__ double ss[256], sm[256];
  __shared__ long long sl[256];
  ss[threadIdx.x] = s; sm[threadIdx.x] = m; sl[threadIdx.x] = loc;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if (threadIdx.x < o) {
      ss[threadIdx.x] += ss[threadIdx.x + o];
      const double m2 = sm[threadIdx.x + o];
      const long long l2 = sl[threadIdx.x + o];
      if (m2 > sm[threadIdx.x] || (m2 == sm[threadIdx.x] && l2 >= 0 && (sl[threadIdx.x] < 0 || l2 < sl[threadIdx.x]))) {
        sm[threadIdx.x] = m2; sl[threadIdx.x] = l2;
      }
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) { psum[blockIdx.x] = ss[0]; pmax[blockIdx.x] = sm[0]; ploc[blockIdx.x] = sl[0]; }
}
__global__ void k_div_final(int nb, const double *psum, const double *pmax, const long long *ploc, double *out) {
  if (threadIdx.x != 0) return;
  double s = 0., m = -1.;
  long long l = -1;
  for (int b = 0; b < nb; ++b) {
    s += psum[b];
    if (pmax[b] > m || (pmax[b] == m && ploc[b] >= 0 && (l < 0 || ploc[b] < l))) { m = pmax[b]; l = ploc[b]; }
  }
  out[0] = s; out[1] = m; out[2] = (double)l;
}
template <typename T>
void launch_chkdiv(cudaStream_t s, const Geo &g, const T *u, const T *v, const T *w, double *scratch, double *out) {
  const int nb = 608;
  double *psum = scratch, *pmax = scratch + nb;
  long long *ploc = (long long *)(scratch + 2 * nb);
  k_div_partial<T><<<nb, 256, 0, s>>>(g, u, v, w, psum, pmax, ploc);
  k_div_final<<<1, 32, 0, s>>>(nb, psum, pmax, ploc, out);
}
template void launch_chkdiv<double>(cudaStream_t, const Geo &, const double *, const double *, const double *,
                                    double *, double *);
template void launch_chkdiv<float>(cudaStream_t, const Geo &, const float *, const float *, const float *, double *,
                                   double *);

// chkdt (chkdt.f90:6-273): min over the three staggered components.
template <typename T>
__global__ void __launch_bounds__(256) k_dt_partial(Geo g, const T *__restrict__ u,
                                                    const T *__restrict__ v, const T *__restrict__ w,
                                                    double *__restrict__ pmin) {
  const long n = (long)g.I * g.J * g.K;
  double m = 899999.;
  const double dxi = g.dxi, dyi = g.dyi, dzi = g.dzi;
  for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < n; t += (long)gridDim.x * blockDim.x) {
    const int i = (int)(t % g.I), j = (int)((t / g.I) % g.J), k = (int)(t / g.plane) + 1;
    const int ip = wrapm(i + 1, g.I), im = wrapm(i - 1, g.I), jp = wrapm(j + 1, g.J), jm = wrapm(j - 1, g.J);
    auto U = [&](int a, int b, int c) { return (double)u[fidx(g, a, b, c)]; };
    auto V = [&](int a, int b, int c) { return (double)v[fidx(g, a, b, c)]; };
    auto W = [&](int a, int b, int c) { return (double)w[fidx(g, a, b, c)]; };
    const double dxi2 = dxi * dxi + dyi * dyi + dzi * dzi;
    const double dt1 = 1.65 / (4. * g.visc * dxi2);
    for (int comp = 0; comp < 3; ++comp) {
      double u2, v2, w2, tt;
      if (comp == 0) {
        u2 = U(i, j, k) * U(i, j, k);
        tt = 0.25 * (V(i, j, k) + V(i, jm, k) + V(ip, j, k) + V(ip, jm, k)); v2 = tt * tt;
        tt = 0.25 * (W(i, j, k) + W(i, j, k - 1) + W(ip, j, k) + W(ip, j, k - 1)); w2 = tt * tt;
      } else if (comp == 1) {
        tt = 0.25 * (U(i, j, k) + U(i, jp, k) + U(im, jp, k) + U(im, j, k)); u2 = tt * tt;
        v2 = V(i, j, k) * V(i, j, k);
        tt = 0.25 * (W(i, j, k) + W(i, jp, k) + W(i, jp, k - 1) + W(i, j, k - 1)); w2 = tt * tt;
      } else {
        tt = 0.25 * (U(i, j, k) + U(im, j, k) + U(im, j, k + 1) + U(i, j, k + 1)); u2 = tt * tt;
        tt = 0.25 * (V(i, j, k) + V(i, jm, k) + V(i, jm, k + 1) + V(i, j, k + 1)); v2 = tt * tt;
        w2 = W(i, j, k) * W(i, j, k);
      }
      const double velo = sqrt(u2 + v2 + w2);
      double dt2;
      if (fabs(velo) > 1.e-12) dt2 = sqrt(3.) / (sqrt(u2) * dxi + sqrt(v2) * dyi + sqrt(w2) * dzi);
      else dt2 = 99999.;
      m = fmin(m, fmin(dt1, dt2));
    }
  }
  __shared__ double sm[256];
  sm[threadIdx.x] = m;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if (threadIdx.x < o) sm[threadIdx.x] = fmin(sm[threadIdx.x], sm[threadIdx.x + o]);
    __syncthreads();
  }
  if (threadIdx.x == 0) pmin[blockIdx.x] = sm[0];
}
__global__ void k_min_final(int nb, const double *p, double *out) {
  if (threadIdx.x != 0) return;
  double m = 899999.;
  for (int b = 0; b < nb; ++b) m = fmin(m, p[b]);
  out[0] = m;
}
template <typename T>
void launch_chkdt(cudaStream_t s, const Geo &g, const T *u, const T *v, const T *w, double *scratch, double *out) {
  const int nb = 608;
  k_dt_partial<T><<<nb, 256, 0, s>>>(g, u, v, w, scratch);
  k_min_final<<<1, 32, 0, s>>>(nb, scratch, out);
}
template void launch_chkdt<double>(cudaStream_t, const Geo &, const double *, const double *, const double *,
                                   double *, double *);
template void launch_chkdt<float>(cudaStream_t, const Geo &, const float *, const float *, const float *, double *,
                                  double *);

// wall shear of rk1/rk2/rk3 (rk3.f90:80-103): sum over the wall planes,
// block partials combined in a fixed order.
template <typename T>
__global__ void __launch_bounds__(256) k_wallshear_partial(Geo g, const T *__restrict__ v, double *__restrict__ part) {
  __shared__ double sm[256];
  double s = 0.;
  const long PL = g.plane;
  for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < PL; t += (long)gridDim.x * blockDim.x) {
    const long top = (long)g.K * PL + t, bot = PL + t;
    s = s + g.visc * ((double)v[top + PL] - (double)v[top]) * g.dzi * (1. / g.dxi) * (1. / g.dyi) -
        g.visc * ((double)v[bot] - (double)v[bot - PL]) * g.dzi * (1. / g.dxi) * (1. / g.dyi);
  }
  sm[threadIdx.x] = s;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) sm[threadIdx.x] += sm[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = sm[0];
}
__global__ void k_sum_final(int nb, const double *__restrict__ part, double *out) {
  if (threadIdx.x != 0) return;
  double s = 0.;
  for (int b = 0; b < nb; ++b) s += part[b];
  out[0] = s;
}
template <typename T>
void launch_wallshear(cudaStream_t s, const Geo &g, const T *v, double *scratch, double *out) {
  const int nb = 64;
  k_wallshear_partial<T><<<nb, 256, 0, s>>>(g, v, scratch);
  k_sum_final<<<1, 32, 0, s>>>(nb, scratch, out);
}
template void launch_wallshear<double>(cudaStream_t, const Geo &, const double *, double *, double *);
template void launch_wallshear<float>(cudaStream_t, const Geo &, const float *, double *, double *);

// convert / copy helpers for the mixed form
__global__ void k_d2f(long n, const double *__restrict__ a, float *__restrict__ b) {
  for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < n; t += (long)gridDim.x * blockDim.x)
    b[t] = (float)a[t];
}
__global__ void k_f2d(long n, const float *__restrict__ a, double *__restrict__ b) {
  for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < n; t += (long)gridDim.x * blockDim.x)
    b[t] = (double)a[t];
}
void launch_d2f(cudaStream_t s, long n, const double *a, float *b) { k_d2f<<<1216, 256, 0, s>>>(n, a, b); }
void launch_f2d(cudaStream_t s, long n, const float *a, double *b) { k_f2d<<<1216, 256, 0, s>>>(n, a, b); }

}  // namespace ibmk
