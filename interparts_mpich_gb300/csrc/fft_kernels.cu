// fft_kernels.cu -- pressure Poisson solve of solver2d (solver.f90:43-172):
// real FFT along x fused with fillps (fillps.f90:8-53), complex FFT along y,
// batched Thomas sweep along z with the zero-mode guard, inverse y, inverse x.
//
// The reference transforms with VFFTPACK in half-complex storage; the solve
// is storage independent (each Fourier mode decouples with eigenvalue
// xrt+yrt, initsolver.f90:42-64), so the GPU keeps an ordinary complex
// spectrum S[k][ky][kx], kx = 0..I/2, built from a half-length complex FFT.
//
// FFTs run in shared memory with a Stockham autosort formulation of radix
// 2/3/4 stages (Govindaraju et al., SC'08); twiddles come from a host-built
// table W_M^t = exp(-2*pi*i*t/M).
#include "kernels.cuh"

namespace ibmk {

template <typename T> struct cpx;
template <> struct cpx<double> { typedef double2 t; };
template <> struct cpx<float> { typedef float2 t; };

template <typename C> __device__ __forceinline__ C cmk(decltype(C().x) a, decltype(C().x) b) { C r; r.x = a; r.y = b; return r; }
template <typename C> __device__ __forceinline__ C cadd(C a, C b) { return cmk<C>(a.x + b.x, a.y + b.y); }
template <typename C> __device__ __forceinline__ C csub(C a, C b) { return cmk<C>(a.x - b.x, a.y - b.y); }
template <typename C> __device__ __forceinline__ C cmul(C a, C b) { return cmk<C>(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); }
template <typename C> __device__ __forceinline__ C cconj(C a) { return cmk<C>(a.x, -a.y); }
template <typename C> __device__ __forceinline__ C cscale(C a, decltype(C().x) s) { return cmk<C>(a.x * s, a.y * s); }
// multiply by -i (forward) or +i (inverse)
template <typename C> __device__ __forceinline__ C cmi(C a, int inv) { return inv ? cmk<C>(-a.y, a.x) : cmk<C>(a.y, -a.x); }

// small DFTs, forward e^{-2 pi i qr/R} (inverse: conjugate kernel)
template <typename C> __device__ __forceinline__ void dft2(C *v) {
  C a = v[0], b = v[1];
  v[0] = cadd(a, b); v[1] = csub(a, b);
}
template <typename C> __device__ __forceinline__ void dft4(C *v, int inv) {
  C t0 = cadd(v[0], v[2]), t1 = csub(v[0], v[2]);
  C t2 = cadd(v[1], v[3]), t3 = cmi(csub(v[1], v[3]), inv);
  v[0] = cadd(t0, t2); v[2] = csub(t0, t2);
  v[1] = cadd(t1, t3); v[3] = csub(t1, t3);
}
template <typename C> __device__ __forceinline__ void dft3(C *v, int inv) {
  typedef decltype(C().x) R;
  const R h = (R)0.5, s3 = (R)0.86602540378443864676372317075294;
  C t1 = cadd(v[1], v[2]);
  C t2 = csub(v[0], cscale(t1, h));
  C t3 = cscale(cmi(csub(v[1], v[2]), inv), s3);
  v[0] = cadd(v[0], t1);
  v[1] = cadd(t2, t3);
  v[2] = csub(t2, t3);
}

// In-place (ping-pong) shared-memory FFT of nseq sequences of length M.
// element m of sequence s lives at buf[s*ss + m*es].  Returns the buffer
// holding the result (a or b).
template <typename C>
__device__ C *fft_smem(C *a, C *b, int M, int nseq, int es, int ss, const FftPlan &pl, const C *__restrict__ tw,
                       int inv) {
  int Ns = 1;
  for (int st = 0; st < pl.nst; ++st) {
    const int R = pl.rad[st];
    const int nb = M / R;
    const int twst = M / (Ns * R);
    for (int t = threadIdx.x; t < nb * nseq; t += blockDim.x) {
      const int sq = t / nb, jb = t - sq * nb;
      const C *src = a + (long)sq * ss;
      C *dst = b + (long)sq * ss;
      const int kk = jb % Ns;
      C v[4];
      for (int r = 0; r < R; ++r) {
        C x = src[(jb + r * nb) * es];
        if (r > 0 && kk > 0) {
          C wt = tw[kk * twst * r];
          if (inv) wt = cconj(wt);
          x = cmul(x, wt);
        }
        v[r] = x;
      }
      if (R == 2) dft2(v);
      else if (R == 4) dft4(v, inv);
      else dft3(v, inv);
      const int idxD = (jb / Ns) * Ns * R + kk;
      for (int r = 0; r < R; ++r) dst[(idxD + r * Ns) * es] = v[r];
    }
    __syncthreads();
    C *t = a; a = b; b = t;
    Ns *= R;
  }
  return a;
}

// Compile-time specialisation of the same Stockham stages for the lengths
// used by the configurations: the index arithmetic (divisions by the
// butterfly count and the sub-transform size) becomes shifts and constant
// multiplies.  Radix order as in the runtime plan: 4s, then 2, then 3.
template <int M, int Ns, typename C>
__device__ __forceinline__ C *fft_stages_ct(C *a, C *b, int nseq, int ss, const C *__restrict__ tw, int inv) {
  if constexpr (Ns >= M) {
    return a;
  } else {
    constexpr int rem = M / Ns;
    constexpr int R = (rem % 4 == 0) ? 4 : ((rem % 2 == 0) ? 2 : 3);
    constexpr int nb = M / R;
    constexpr int twst = M / (Ns * R);
    for (int t = threadIdx.x; t < nb * nseq; t += blockDim.x) {
      const int sq = t / nb, jb = t - sq * nb;
      const C *src = a + (long)sq * ss;
      C *dst = b + (long)sq * ss;
      const int kk = jb % Ns;
      C v[R];
#pragma unroll
      for (int r = 0; r < R; ++r) {
        C x = src[jb + r * nb];
        if (r > 0 && kk > 0) {
          C wt = tw[kk * twst * r];
          if (inv) wt = cconj(wt);
          x = cmul(x, wt);
        }
        v[r] = x;
      }
      if constexpr (R == 2) dft2(v);
      else if constexpr (R == 4) dft4(v, inv);
      else dft3(v, inv);
      const int idxD = (jb / Ns) * Ns * R + kk;
#pragma unroll
      for (int r = 0; r < R; ++r) dst[idxD + r * Ns] = v[r];
    }
    __syncthreads();
    return fft_stages_ct<M, Ns * R, C>(b, a, nseq, ss, tw, inv);
  }
}

// unit-stride sequences (es = 1); lengths without a specialisation use the
// runtime plan
template <typename C>
__device__ C *fft_smem1(C *a, C *b, int M, int nseq, int ss, const FftPlan &pl, const C *__restrict__ tw, int inv) {
  switch (M) {
    case 16: return fft_stages_ct<16, 1, C>(a, b, nseq, ss, tw, inv);
    case 24: return fft_stages_ct<24, 1, C>(a, b, nseq, ss, tw, inv);
    case 32: return fft_stages_ct<32, 1, C>(a, b, nseq, ss, tw, inv);
    case 48: return fft_stages_ct<48, 1, C>(a, b, nseq, ss, tw, inv);
    case 64: return fft_stages_ct<64, 1, C>(a, b, nseq, ss, tw, inv);
    case 96: return fft_stages_ct<96, 1, C>(a, b, nseq, ss, tw, inv);
    case 128: return fft_stages_ct<128, 1, C>(a, b, nseq, ss, tw, inv);
    case 192: return fft_stages_ct<192, 1, C>(a, b, nseq, ss, tw, inv);
    case 256: return fft_stages_ct<256, 1, C>(a, b, nseq, ss, tw, inv);
    case 384: return fft_stages_ct<384, 1, C>(a, b, nseq, ss, tw, inv);
    case 512: return fft_stages_ct<512, 1, C>(a, b, nseq, ss, tw, inv);
    case 768: return fft_stages_ct<768, 1, C>(a, b, nseq, ss, tw, inv);
    default: return fft_smem<C>(a, b, M, nseq, 1, ss, pl, tw, inv);
  }
}

// ---------------------------------------------------------------------------
// Register four-step FFT (FP32 path).  N = N1*N2 with N1 = N2 or 2*N2 and
// N1 <= 16: a group of N2 threads holds a sequence, thread t the elements
// x[t + N2*n1]; an N1-point DFT in registers, the twiddle W_N^(t*k1), one
// exchange through a padded shared buffer (group-private, __syncwarp only),
// then N2-point DFTs in registers (N1/N2 per thread), written back in
// natural order.  Same DFT as the Stockham stages, other summation order.
// ---------------------------------------------------------------------------
// multiply by exp(-+2 pi i m/den) given cos, sin of 2 pi m/den
template <typename C>
__device__ __forceinline__ C cmulcs(C x, float c, float s, int inv) {
  return inv ? cmk<C>(x.x * c - x.y * s, x.y * c + x.x * s) : cmk<C>(x.x * c + x.y * s, x.y * c - x.x * s);
}
// cos, sin of 2 pi m / 16, m = 0..9
__device__ __forceinline__ void w16(int m, float &c, float &s) {
  const float C1 = 0.92387953251128675613f, S1 = 0.38268343236508977173f, R2 = 0.70710678118654752440f;
  const float cs[10] = {1.f, C1, R2, S1, 0.f, -S1, -R2, -C1, -1.f, -C1};
  const float sn[10] = {0.f, S1, R2, C1, 1.f, C1, R2, S1, 0.f, -S1};
  c = cs[m]; s = sn[m];
}
template <int N, typename C> __device__ __forceinline__ void dft_reg(C *v, int inv);
template <> __device__ __forceinline__ void dft_reg<2, float2>(float2 *v, int) { dft2(v); }
template <> __device__ __forceinline__ void dft_reg<4, float2>(float2 *v, int inv) { dft4(v, inv); }
template <> __device__ __forceinline__ void dft_reg<8, float2>(float2 *v, int inv) {
  // n = n2 + 2 n1, k = k1 + 4 k2
  float2 a0[4] = {v[0], v[2], v[4], v[6]}, a1[4] = {v[1], v[3], v[5], v[7]};
  dft4(a0, inv);
  dft4(a1, inv);
  float c, s;
  w16(2, c, s); a1[1] = cmulcs(a1[1], c, s, inv);
  a1[2] = cmi(a1[2], inv);
  w16(6, c, s); a1[3] = cmulcs(a1[3], c, s, inv);
#pragma unroll
  for (int k1 = 0; k1 < 4; ++k1) { v[k1] = cadd(a0[k1], a1[k1]); v[k1 + 4] = csub(a0[k1], a1[k1]); }
}
template <> __device__ __forceinline__ void dft_reg<16, float2>(float2 *v, int inv) {
  // n = n2 + 4 n1, k = k1 + 4 k2
  float2 a[4][4];
#pragma unroll
  for (int n2 = 0; n2 < 4; ++n2) {
#pragma unroll
    for (int n1 = 0; n1 < 4; ++n1) a[n2][n1] = v[n2 + 4 * n1];
    dft4(a[n2], inv);
  }
#pragma unroll
  for (int n2 = 1; n2 < 4; ++n2)
#pragma unroll
    for (int k1 = 1; k1 < 4; ++k1) {
      float c, s;
      w16(n2 * k1, c, s);
      a[n2][k1] = cmulcs(a[n2][k1], c, s, inv);
    }
#pragma unroll
  for (int k1 = 0; k1 < 4; ++k1) {
    float2 b[4] = {a[0][k1], a[1][k1], a[2][k1], a[3][k1]};
    dft4(b, inv);
#pragma unroll
    for (int k2 = 0; k2 < 4; ++k2) v[k1 + 4 * k2] = b[k2];
  }
}
// one sequence in shared memory (unit stride) per group of N2 threads;
// ex: group-private exchange buffer of N1*(N2+1) elements.  Every thread of
// the warp must call it (it synchronises the warp).
template <int N1, int N2>
__device__ __forceinline__ void fft_group(float2 *row, float2 *ex, int t, const float2 *__restrict__ tw, int inv,
                                          bool active) {
  constexpr int N = N1 * N2;
  float2 v[N1];
  if (active) {
#pragma unroll
    for (int r = 0; r < N1; ++r) v[r] = row[t + N2 * r];
    dft_reg<N1, float2>(v, inv);
#pragma unroll
    for (int k1 = 1; k1 < N1; ++k1) {
      if (t > 0) {
        float2 w = __ldg(&tw[(t * k1) % N]);
        if (inv) w.y = -w.y;
        v[k1] = cmul(v[k1], w);
      }
    }
#pragma unroll
    for (int k1 = 0; k1 < N1; ++k1) ex[k1 * (N2 + 1) + t] = v[k1];
  }
  __syncwarp();
  if (active) {
#pragma unroll
    for (int q = 0; q < N1 / N2; ++q) {
      const int k1 = t + q * N2;
      float2 w[N2];
#pragma unroll
      for (int n2 = 0; n2 < N2; ++n2) w[n2] = ex[k1 * (N2 + 1) + n2];
      dft_reg<N2, float2>(w, inv);
#pragma unroll
      for (int k2 = 0; k2 < N2; ++k2) row[k1 + N1 * k2] = w[k2];
    }
  }
  __syncwarp();
}
// (N1, N2) of the supported lengths; 0 = use the Stockham stages
__host__ __device__ inline int reg_n2(int N) {
  return N == 16 ? 4 : N == 32 ? 4 : N == 64 ? 8 : N == 128 ? 8 : N == 256 ? 16 : 0;
}

// divergence factors dt/dx, dt/dy, dt/dz as double-float pairs (hi, lo)
struct DivScale {
  float xh, xl, yh, yl, zh, zl;
};

// With phi1 (defect correction, DF): the right-hand side is the divergence
// residual of the corrected velocity u* - f grad(phi1) (correc's FP32
// expressions), formed on the fly instead of read from a stored state.
template <int N1, int N2, bool DF>
__global__ void __launch_bounds__(128) k_fillps_fftx_r(Geo g, const float *__restrict__ fu,
                                                       const float *__restrict__ fv, float *__restrict__ fw,
                                                       float2 *__restrict__ S, const float2 *__restrict__ twM,
                                                       const float2 *__restrict__ twN, DivScale ds,
                                                       const float *__restrict__ phi1, float cfi, float cfj,
                                                       float cfk) {
  constexpr int M = N1 * N2, ROWS = 128 / N2;
  // group strides padded by 8 elements (64 B): groups sharing a warp start
  // half a bank row apart
  constexpr int RS = M + 8, ES = N1 * (N2 + 1) + 8;
  __shared__ __align__(16) float2 A[ROWS * RS];
  __shared__ float2 EX[ROWS * ES];
  const int row0 = blockIdx.x * ROWS;
  const int nrow = g.J * g.K;
  const float fx_hi = ds.xh, fx_lo = ds.xl, fy_hi = ds.yh, fy_lo = ds.yl, fz_hi = ds.zh, fz_lo = ds.zl;
  const float fxs = ds.xh, fys = ds.yh, fzs = ds.zh;
  const int PL = g.I * g.J;
  // 1. right-hand side, packed z_m = x_{2m} + i x_{2m+1}; four consecutive
  // i per thread with 128-bit loads (I % 4 == 0 on this path)
  constexpr int Q = 2 * M / 4;  // float4 per row
#pragma unroll 4
  for (int q = threadIdx.x; q < ROWS * Q; q += blockDim.x) {
    const int r = q / Q, i0 = (q - r * Q) * 4;
    const int row = row0 + r;
    float val[4] = {0.f, 0.f, 0.f, 0.f};
    if (row < nrow) {
      const int j = row % g.J, k = row / g.J + 1;
      const long c = fidx(g, i0, j, k);
      const float4 w4 = (k == g.K) ? make_float4(0.f, 0.f, 0.f, 0.f) : *reinterpret_cast<const float4 *>(fw + c);
      const float4 wm4 = *reinterpret_cast<const float4 *>(fw + c - PL);  // plane 0 holds w(0)=0
      if (k == g.K) *reinterpret_cast<float4 *>(fw + c) = make_float4(0.f, 0.f, 0.f, 0.f);
      const long cjm = c + (j == 0 ? (g.J - 1) * g.I : -g.I);
      const float4 v4 = *reinterpret_cast<const float4 *>(fv + c);
      const float4 vm4 = *reinterpret_cast<const float4 *>(fv + cjm);
      const float4 u4 = *reinterpret_cast<const float4 *>(fu + c);
      const long cim = c + (i0 == 0 ? g.I - 1 : -1);
      const float um1 = fu[cim];
      float wk[4] = {w4.x, w4.y, w4.z, w4.w}, wkm[4] = {wm4.x, wm4.y, wm4.z, wm4.w};
      float vv[4] = {v4.x, v4.y, v4.z, v4.w}, vjm[4] = {vm4.x, vm4.y, vm4.z, vm4.w};
      float uu[4] = {u4.x, u4.y, u4.z, u4.w}, uim[4] = {um1, u4.x, u4.y, u4.z};
      if (DF && phi1) {
        // u - fi (phi(i+1) - phi(i)) etc. as correc stores them (w = 0 on
        // the walls k = K and 0)
        const float4 p4 = *reinterpret_cast<const float4 *>(phi1 + c);
        const float pim = phi1[cim];
        const float pip = phi1[c + (i0 + 4 == g.I ? 4 - g.I : 4)];
        const float4 pjp4 = *reinterpret_cast<const float4 *>(phi1 + c + (j + 1 == g.J ? (1 - g.J) * g.I : g.I));
        const float4 pjm4 = *reinterpret_cast<const float4 *>(phi1 + cjm);
        const float4 pkp4 = (k == g.K) ? p4 : *reinterpret_cast<const float4 *>(phi1 + c + PL);
        const float4 pkm4 = *reinterpret_cast<const float4 *>(phi1 + c - PL);
        const float P[6] = {pim, p4.x, p4.y, p4.z, p4.w, pip};
        const float Pjp[4] = {pjp4.x, pjp4.y, pjp4.z, pjp4.w}, Pjm[4] = {pjm4.x, pjm4.y, pjm4.z, pjm4.w};
        const float Pkp[4] = {pkp4.x, pkp4.y, pkp4.z, pkp4.w}, Pkm[4] = {pkm4.x, pkm4.y, pkm4.z, pkm4.w};
        for (int e = 0; e < 4; ++e) {
          const float P0 = P[e + 1];
          const float un = uu[e] - cfi * (P[e + 2] - P0);
          const float unm = uim[e] - cfi * (P0 - P[e]);
          const float vn = vv[e] - cfj * (Pjp[e] - P0);
          const float vnm = vjm[e] - cfj * (P0 - Pjm[e]);
          const float wn = (k == g.K) ? 0.f : wk[e] - cfk * (Pkp[e] - P0);
          const float wnm = (k == 1) ? 0.f : wkm[e] - cfk * (P0 - Pkm[e]);
          uu[e] = un; uim[e] = unm; vv[e] = vn; vjm[e] = vnm; wk[e] = wn; wkm[e] = wnm;
        }
      }
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        if constexpr (DF) {
          // divergence residual in double-float arithmetic: exact differences
          // of the FP32 velocities, products with the split FP64 factors
          float dh, dl, th, tl, sh, sl;
          two_sum(wk[e], -wkm[e], dh, dl);
          df_mul(dh, dl, fz_hi, fz_lo, sh, sl);
          two_sum(vv[e], -vjm[e], dh, dl);
          df_mul(dh, dl, fy_hi, fy_lo, th, tl);
          df_add(sh, sl, th, tl, sh, sl);
          two_sum(uu[e], -uim[e], dh, dl);
          df_mul(dh, dl, fx_hi, fx_lo, th, tl);
          df_add(sh, sl, th, tl, sh, sl);
          val[e] = sh + sl;
        } else {
          val[e] = (wk[e] - wkm[e]) * fzs + (vv[e] - vjm[e]) * fys + (uu[e] - uim[e]) * fxs;
        }
      }
    }
    *reinterpret_cast<float4 *>(reinterpret_cast<float *>(A + r * RS) + i0) = make_float4(val[0], val[1], val[2], val[3]);
  }
  __syncthreads();
  const int grp = threadIdx.x / N2, t = threadIdx.x - grp * N2;
  fft_group<N1, N2>(A + grp * RS, EX + grp * ES, t, twM, 0, true);
  __syncthreads();
  // 2. unpack to X_k, k = 0..M  (X_k = E_k + W_N^k O_k)
  for (int q = threadIdx.x; q < ROWS * (M + 1); q += blockDim.x) {
    const int r = q / (M + 1), kx = q - r * (M + 1);
    const int row = row0 + r;
    if (row >= nrow) continue;
    const float2 Zk = A[r * RS + (kx == M ? 0 : kx)];
    const float2 Zc = cconj(A[r * RS + (kx == 0 ? 0 : M - kx)]);
    const float2 E = cscale(cadd(Zk, Zc), 0.5f);
    const float2 D = csub(Zk, Zc);
    const float2 O = cmk<float2>(D.y * 0.5f, -D.x * 0.5f);  // D/(2i)
    S[(long)row * g.MX + kx] = cadd(E, cmul(__ldg(&twN[kx]), O));
  }
}

// complex FFT along y; a group of N2 threads per kx-column, 256 threads
template <int N1, int N2>
__global__ void __launch_bounds__(256) k_ffty_r(Geo g, float2 *__restrict__ S, const float2 *__restrict__ twJ, int inv) {
  constexpr int J = N1 * N2, COLS = 256 / N2, LD = J + 1;
  extern __shared__ __align__(16) unsigned char smr[];
  float2 *A = reinterpret_cast<float2 *>(smr);  // [COLS][LD]
  float2 *EX = A + COLS * LD;                   // [COLS][N1*(N2+1)]
  const int kx0 = blockIdx.x * COLS;
  float2 *plane = S + (long)blockIdx.y * J * g.MX;
  // the block's columns straight into shared memory by asynchronous 8-byte
  // copies (all of a thread's loads in flight together; zero fill beyond MX)
  for (int q = threadIdx.x; q < J * COLS; q += blockDim.x) {
    const int jy = q / COLS, cx = q - jy * COLS;
    const int kx = kx0 + cx;
    const bool ok = kx < g.MX;
    const uint32_t dst = (uint32_t)__cvta_generic_to_shared(&A[cx * LD + jy]);
    const float2 *src = ok ? &plane[(long)jy * g.MX + kx] : plane;
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;\n" ::"r"(dst), "l"(src), "r"(ok ? 8 : 0));
  }
  asm volatile("cp.async.wait_all;\n" ::: "memory");
  __syncthreads();
  const int grp = threadIdx.x / N2, t = threadIdx.x - grp * N2;
  fft_group<N1, N2>(A + grp * LD, EX + grp * N1 * (N2 + 1), t, twJ, inv, kx0 + grp < g.MX);
  __syncthreads();
  for (int q = threadIdx.x; q < J * COLS; q += blockDim.x) {
    const int jy = q / COLS, cx = q - jy * COLS;
    const int kx = kx0 + cx;
    if (kx < g.MX) plane[(long)jy * g.MX + kx] = A[cx * LD + jy];
  }
}

// inverse real FFT along x: spectrum row -> phi(i,j,k), k = 1..K
template <int N1, int N2>
__global__ void __launch_bounds__(128) k_ifftx_r(Geo g, const float2 *__restrict__ S, float *__restrict__ phi,
                                                 const float2 *__restrict__ twM, const float2 *__restrict__ twN) {
  constexpr int M = N1 * N2, ROWS = 128 / N2;
  constexpr int RS = M + 8, ES = N1 * (N2 + 1) + 8;  // padded group strides
  __shared__ __align__(16) float2 A[ROWS * RS];
  __shared__ float2 EX[ROWS * ES];
  const int row0 = blockIdx.x * ROWS;
  const int nrow = g.J * g.K;
  // pack X_k and conj(X_{M-k}) straight from the (L2-resident) spectrum
  for (int q = threadIdx.x; q < ROWS * M; q += blockDim.x) {
    const int r = q / M, kx = q - r * M;
    const int row = row0 + r;
    float2 Xk = make_float2(0.f, 0.f), Xc = Xk;
    if (row < nrow) {
      Xk = S[(long)row * g.MX + kx];
      Xc = cconj(S[(long)row * g.MX + (M - kx)]);
    }
    const float2 E = cscale(cadd(Xk, Xc), 0.5f);
    const float2 O = cmul(cscale(csub(Xk, Xc), 0.5f), cconj(__ldg(&twN[kx])));
    A[r * RS + kx] = cadd(E, cmk<float2>(-O.y, O.x));  // E + i O
  }
  __syncthreads();
  const int grp = threadIdx.x / N2, t = threadIdx.x - grp * N2;
  fft_group<N1, N2>(A + grp * RS, EX + grp * ES, t, twM, 1, true);
  __syncthreads();
  constexpr int Q = 2 * M / 4;
  for (int q = threadIdx.x; q < ROWS * Q; q += blockDim.x) {
    const int r = q / Q, i0 = (q - r * Q) * 4;
    const int row = row0 + r;
    if (row >= nrow) continue;
    const int j = row % g.J, k = row / g.J + 1;
    *reinterpret_cast<float4 *>(phi + fidx(g, i0, j, k)) =
        *reinterpret_cast<const float4 *>(reinterpret_cast<const float *>(A + r * RS) + i0);
  }
}

// dispatch of the register FFT kernels for one length pair (M = I/2, J)
template <int M1, int M2>
bool launch_fftx_r(cudaStream_t s, const Geo &g, const float *fu, const float *fv, float *fw, float2 *S,
                   const float2 *twM, const float2 *twN, double a, double b, double c, bool df, bool inv, float *phi,
                   const PoissonResid &rs) {
  const int nrow = g.J * g.K;
  constexpr int ROWS = 128 / M2;
  const int grid = (nrow + ROWS - 1) / ROWS;
  // the divergence factors as double-float pairs, split here once rather
  // than in every thread (FP64 issues at a small fraction of the FP32 rate)
  DivScale ds;
  ds.xh = (float)a; ds.xl = (float)(a - (double)ds.xh);
  ds.yh = (float)b; ds.yl = (float)(b - (double)ds.yh);
  ds.zh = (float)c; ds.zl = (float)(c - (double)ds.zh);
  if (inv) k_ifftx_r<M1, M2><<<grid, 128, 0, s>>>(g, S, phi, twM, twN);
  else if (df)
    k_fillps_fftx_r<M1, M2, true><<<grid, 128, 0, s>>>(g, fu, fv, fw, S, twM, twN, ds, rs.phi1, rs.fi, rs.fj, rs.fk);
  else
    k_fillps_fftx_r<M1, M2, false><<<grid, 128, 0, s>>>(g, fu, fv, fw, S, twM, twN, ds, nullptr, 0.f, 0.f, 0.f);
  return true;
}
bool fftx_r(cudaStream_t s, const Geo &g, const float *fu, const float *fv, float *fw, float2 *S, const float2 *twM,
            const float2 *twN, double a, double b, double c, bool df, bool inv, float *phi, const PoissonResid &rs) {
  switch (g.I / 2) {
    case 16: return launch_fftx_r<4, 4>(s, g, fu, fv, fw, S, twM, twN, a, b, c, df, inv, phi, rs);
    case 32: return launch_fftx_r<8, 4>(s, g, fu, fv, fw, S, twM, twN, a, b, c, df, inv, phi, rs);
    case 64: return launch_fftx_r<8, 8>(s, g, fu, fv, fw, S, twM, twN, a, b, c, df, inv, phi, rs);
    case 128: return launch_fftx_r<16, 8>(s, g, fu, fv, fw, S, twM, twN, a, b, c, df, inv, phi, rs);
    case 256: return launch_fftx_r<16, 16>(s, g, fu, fv, fw, S, twM, twN, a, b, c, df, inv, phi, rs);
    default: return false;
  }
}
bool poisson_fused_residual_ok(const Geo &g) { return reg_n2(g.I / 2) && reg_n2(g.J) && g.I % 4 == 0; }
template <int N1, int N2>
size_t ffty_r_smem() { return (size_t)(256 / N2) * ((N1 * N2 + 1) + N1 * (N2 + 1)) * sizeof(float2); }
template <int N1, int N2>
void launch_ffty_r1(cudaStream_t s, const Geo &g, float2 *S, const float2 *twJ, int inv) {
  constexpr int COLS = 256 / N2;
  dim3 grid((g.MX + COLS - 1) / COLS, g.K);
  k_ffty_r<N1, N2><<<grid, 256, ffty_r_smem<N1, N2>(), s>>>(g, S, twJ, inv);
}
bool ffty_r(cudaStream_t s, const Geo &g, float2 *S, const float2 *twJ, int inv) {
  switch (g.J) {
    case 16: launch_ffty_r1<4, 4>(s, g, S, twJ, inv); return true;
    case 32: launch_ffty_r1<8, 4>(s, g, S, twJ, inv); return true;
    case 64: launch_ffty_r1<8, 8>(s, g, S, twJ, inv); return true;
    case 128: launch_ffty_r1<16, 8>(s, g, S, twJ, inv); return true;
    case 256: launch_ffty_r1<16, 16>(s, g, S, twJ, inv); return true;
    default: return false;
  }
}
int ffty_r_set_smem_limits() {
  cudaError_t e[5] = {
      cudaFuncSetAttribute(k_ffty_r<4, 4>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ffty_r_smem<4, 4>()),
      cudaFuncSetAttribute(k_ffty_r<8, 4>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ffty_r_smem<8, 4>()),
      cudaFuncSetAttribute(k_ffty_r<8, 8>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ffty_r_smem<8, 8>()),
      cudaFuncSetAttribute(k_ffty_r<16, 8>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ffty_r_smem<16, 8>()),
      cudaFuncSetAttribute(k_ffty_r<16, 16>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ffty_r_smem<16, 16>())};
  for (cudaError_t x : e)
    if (x != cudaSuccess) return -1;
  return 0;
}

// ---------------------------------------------------------------------------
// fillps + forward real FFT along x.  One CTA handles ROWS rows (j,k).
// Reads the forced predictor (fu,fv,fw) with the bounduvw(dudt) wall values
// w(0)=w(kmax)=0 applied (and stored back into fw plane K).
// ---------------------------------------------------------------------------
template <typename TIn, typename T, typename TA, bool DF = false>
__global__ void __launch_bounds__(128) k_fillps_fftx(Geo g, FftPlan plx, const TIn *__restrict__ fu,
                                                     const TIn *__restrict__ fv, TIn *__restrict__ fw,
                                                     typename cpx<T>::t *__restrict__ S,
                                                     const typename cpx<T>::t *__restrict__ twM,
                                                     const typename cpx<T>::t *__restrict__ twN, double dtidxi,
                                                     double dtidyi, double dtidzi, int rows) {
  typedef typename cpx<T>::t C;
  extern __shared__ unsigned char smraw[];
  C *A = reinterpret_cast<C *>(smraw);
  const int M = g.I / 2;
  C *B = A + rows * M;
  const int row0 = blockIdx.x * rows;
  const int nrow = g.J * g.K;
  const float fx_hi = (float)dtidxi, fx_lo = (float)(dtidxi - (double)fx_hi);
  const float fy_hi = (float)dtidyi, fy_lo = (float)(dtidyi - (double)fy_hi);
  const float fz_hi = (float)dtidzi, fz_lo = (float)(dtidzi - (double)fz_hi);
  (void)fx_lo; (void)fy_lo; (void)fz_lo;
  // 1. right-hand side, packed z_m = x_{2m} + i x_{2m+1}
  for (int t = threadIdx.x; t < rows * g.I; t += blockDim.x) {
    const int r = t / g.I, i = t - r * g.I;
    const int row = row0 + r;
    T val = 0;
    if (row < nrow) {
      const int j = row % g.J, k = row / g.J + 1;
      const long c = fidx(g, i, j, k);
      if constexpr (DF) {
        // divergence residual in double-float arithmetic: exact differences
        // of the FP32 velocities, products with the split FP64 factors
        const float wk = (k == g.K) ? 0.f : (float)fw[c];
        const float wkm = (float)fw[c - g.plane];
        if (k == g.K) fw[c] = (TIn)0;
        const float vjm = (float)fv[fidx(g, i, j == 0 ? g.J - 1 : j - 1, k)];
        const float uim = (float)fu[fidx(g, i == 0 ? g.I - 1 : i - 1, j, k)];
        float dh, dl, th, tl, sh, sl;
        two_sum(wk, -wkm, dh, dl);
        df_mul(dh, dl, fz_hi, fz_lo, sh, sl);
        two_sum((float)fv[c], -vjm, dh, dl);
        df_mul(dh, dl, fy_hi, fy_lo, th, tl);
        df_add(sh, sl, th, tl, sh, sl);
        two_sum((float)fu[c], -uim, dh, dl);
        df_mul(dh, dl, fx_hi, fx_lo, th, tl);
        df_add(sh, sl, th, tl, sh, sl);
        val = (T)(sh + sl);
      } else {
        // walls: w(kmax) = 0 (bounduvw on dudt), plane 0 holds w(0) = 0;
        // periodic z: w(kmax) is an unknown and w(0) = w(kmax)
        const TA wk = (k == g.K && !g.zper) ? (TA)0 : (TA)fw[c];
        const TA wkm = (TA)fw[(k == 1 && g.zper) ? c + (long)(g.K - 1) * g.plane : c - g.plane];
        if (k == g.K && !g.zper) fw[c] = (TIn)0;
        const TA vjm = (TA)fv[fidx(g, i, j == 0 ? g.J - 1 : j - 1, k)];
        const TA uim = (TA)fu[fidx(g, i == 0 ? g.I - 1 : i - 1, j, k)];
        val = (T)((wk - wkm) * (TA)dtidzi + ((TA)fv[c] - vjm) * (TA)dtidyi + ((TA)fu[c] - uim) * (TA)dtidxi);
      }
    }
    T *Ar = reinterpret_cast<T *>(A + r * M);
    Ar[i] = val;
  }
  __syncthreads();
  C *Z = fft_smem1<C>(A, B, M, rows, M, plx, twM, 0);
  // 2. unpack to X_k, k = 0..M  (X_k = E_k + W_N^k O_k)
  for (int t = threadIdx.x; t < rows * (M + 1); t += blockDim.x) {
    const int r = t / (M + 1), kx = t - r * (M + 1);
    const int row = row0 + r;
    if (row >= nrow) continue;
    const C Zk = Z[r * M + (kx == M ? 0 : kx)];
    const C Zc = cconj(Z[r * M + (kx == 0 ? 0 : M - kx)]);
    const C E = cscale(cadd(Zk, Zc), (T)0.5);
    const C D = csub(Zk, Zc);
    const C O = cmk<C>(D.y * (T)0.5, -D.x * (T)0.5);  // D/(2i)
    const C X = cadd(E, cmul(twN[kx], O));
    S[(long)row * g.MX + kx] = X;
  }
}

// complex FFT along y for a tile of COLS kx-columns of one k-plane, in place.
template <typename T>
__global__ void __launch_bounds__(256) k_ffty(Geo g, FftPlan ply, typename cpx<T>::t *__restrict__ S,
                                              const typename cpx<T>::t *__restrict__ twJ, int cols, int inv) {
  typedef typename cpx<T>::t C;
  extern __shared__ unsigned char smraw[];
  // each column is stored contiguously (row length J+1 to spread the banks),
  // so the Stockham stages access shared memory with unit stride
  const int LD = g.J + 1;
  C *A = reinterpret_cast<C *>(smraw);
  C *B = A + LD * cols;
  const int kx0 = blockIdx.x * cols;
  const int k = blockIdx.y;
  C *plane = S + (long)k * g.J * g.MX;
  for (int t = threadIdx.x; t < g.J * cols; t += blockDim.x) {
    const int jy = t / cols, cx = t - jy * cols;
    const int kx = kx0 + cx;
    A[cx * LD + jy] = (kx < g.MX) ? plane[(long)jy * g.MX + kx] : cmk<C>((T)0, (T)0);
  }
  __syncthreads();
  C *Y = fft_smem1<C>(A, B, g.J, cols, LD, ply, twJ, inv);
  for (int t = threadIdx.x; t < g.J * cols; t += blockDim.x) {
    const int jy = t / cols, cx = t - jy * cols;
    const int kx = kx0 + cx;
    if (kx < g.MX) plane[(long)jy * g.MX + kx] = Y[cx * LD + jy];
  }
}

// Thomas sweep along z for every (kx,ky) (solver.f90:94-134), FP64, with
// the precomputed pivots zt (pivot reciprocal for k<K, denominator for k=K).
template <typename T>
__global__ void __launch_bounds__(128) k_thomas(Geo g, typename cpx<T>::t *__restrict__ S,
                                                const double *__restrict__ zt, double a2, double scale) {
  typedef typename cpx<T>::t C;
  const long t = blockIdx.x * (long)blockDim.x + threadIdx.x;
  const long ncol = (long)g.MX * g.J;
  if (t >= ncol) return;
  const int kx = (int)(t % g.MX), ky = (int)(t / g.MX);
  const int kyy = ky <= g.J / 2 ? ky : g.J - ky;
  const long zstride = (long)(g.J / 2 + 1) * g.MX;
  const double *z = zt + (long)kyy * g.MX + kx;
  const long sstride = (long)g.J * g.MX;
  C *s = S + t;
  // The recurrence is a dependent chain over k; loads of the next planes
  // are issued in groups of PF so that several are in flight at once.
  constexpr int PF = 8;
  auto ld = [&](int k) -> double2 {
    const C v = s[k * sstride];
    return make_double2((double)v.x * scale, (double)v.y * scale);
  };
  auto st = [&](int k, double2 v) { C o; o.x = (decltype(o.x))v.x; o.y = (decltype(o.y))v.y; s[k * sstride] = o; };
  const int K = g.K;
  double2 prev = make_double2(0., 0.);
  for (int k0 = 0; k0 < K; k0 += PF) {
    double2 buf[PF];
    double zb[PF];
#pragma unroll
    for (int q = 0; q < PF; ++q) {
      const int k = k0 + q;
      if (k < K) { buf[q] = ld(k); zb[q] = z[(long)k * zstride]; }
    }
#pragma unroll
    for (int q = 0; q < PF; ++q) {
      const int k = k0 + q;
      if (k >= K) break;
      double2 cur = buf[q];
      if (k == 0) {
        cur = make_double2(cur.x * zb[q], cur.y * zb[q]);
      } else if (k < K - 1) {
        cur = make_double2((cur.x - a2 * prev.x) * zb[q], (cur.y - a2 * prev.y) * zb[q]);
      } else {
        const double den = zb[q];
        if (den != 0.) cur = make_double2((cur.x - a2 * prev.x) / den, (cur.y - a2 * prev.y) / den);
        else cur = make_double2(0., 0.);
      }
      buf[q] = cur;
      prev = cur;
    }
#pragma unroll
    for (int q = 0; q < PF; ++q)
      if (k0 + q < K) st(k0 + q, buf[q]);
  }
  // back substitution, d(k) = c(k)*z(k) with c(k) = dzi^2 for k < kmax
  for (int k1 = K - 2; k1 >= 0; k1 -= PF) {
    double2 buf[PF];
    double zb[PF];
#pragma unroll
    for (int q = 0; q < PF; ++q) {
      const int k = k1 - q;
      if (k >= 0) {
        const C v = s[k * sstride];
        buf[q] = make_double2((double)v.x, (double)v.y);
        zb[q] = z[(long)k * zstride];
      }
    }
#pragma unroll
    for (int q = 0; q < PF; ++q) {
      const int k = k1 - q;
      if (k < 0) break;
      const double d = a2 * zb[q];
      const double2 cur = make_double2(buf[q].x - d * prev.x, buf[q].y - d * prev.y);
      buf[q] = cur;
      prev = cur;
    }
#pragma unroll
    for (int q = 0; q < PF; ++q)
      if (k1 - q >= 0) st(k1 - q, buf[q]);
  }
}

// Periodic z: the cyclic tridiagonal solve of every (kx, ky) mode in FP64,
// one thread per column: Sherman-Morrison around the Thomas sweep (diagonal
// -2 a2 + xy, off-diagonals and corners a2; gamma = -b), the zero mode
// (xy = 0) pinned at its last plane.  The same operation order as the
// oracle's cyclic_solve; the two right-hand sides (the spectrum and the
// Sherman-Morrison vector) are swept together.  xy = xrt(kx) + yrt(ky) from
// the host tables.
__global__ void __launch_bounds__(128) k_thomas_cyclic(Geo g, double2 *__restrict__ S, const double *__restrict__ xrt,
                                                       const double *__restrict__ yrt, double a2, double scale,
                                                       double *__restrict__ work) {
  const long t = blockIdx.x * (long)blockDim.x + threadIdx.x;
  const long ncol = (long)g.MX * g.J;
  if (t >= ncol) return;
  const int kx = (int)(t % g.MX), ky = (int)(t / g.MX);
  const long sstride = (long)g.J * g.MX;
  double2 *s = S + t;
  double *cp = work + t, *zz = work + ncol * g.K + t;  // [K][ncol] each
  const double xy = xrt[kx] + yrt[ky];
  const double b = -2. * a2 + xy;
  const int K = g.K;
  auto rd = [&](int k) { const double2 v = s[k * sstride]; return make_double2(v.x * scale, v.y * scale); };
  if (xy == 0.) {  // rows 0..K-2 with the last unknown pinned to 0
    const int n = K - 1;
    double den = b;
    cp[0] = a2 / den;
    double2 r = rd(0);
    r = make_double2(r.x / den, r.y / den);
    s[0] = r;
    for (int k = 1; k < n; ++k) {
      den = b - a2 * cp[(long)(k - 1) * ncol];
      cp[(long)k * ncol] = a2 / den;
      const double2 v = rd(k);
      r = make_double2((v.x - a2 * r.x) / den, (v.y - a2 * r.y) / den);
      s[k * sstride] = r;
    }
    for (int k = n - 2; k >= 0; --k) {
      const double2 v = s[k * sstride];
      const double c = cp[(long)k * ncol];
      r = make_double2(v.x - c * r.x, v.y - c * r.y);
      s[k * sstride] = r;
    }
    s[(long)(K - 1) * sstride] = make_double2(0., 0.);
    return;
  }
  const double gamma = -b;
  const double b0 = b - gamma, bn = b - a2 * a2 / gamma;
  // forward sweep of both right-hand sides: the spectrum r and u = (gamma, 0.., 0, a2)
  double den = b0;
  cp[0] = a2 / den;
  double2 r = rd(0);
  r = make_double2(r.x / den, r.y / den);
  s[0] = r;
  double z = gamma / den;
  zz[0] = z;
  for (int k = 1; k < K; ++k) {
    const double bk = k == K - 1 ? bn : b;
    den = bk - a2 * cp[(long)(k - 1) * ncol];
    cp[(long)k * ncol] = a2 / den;
    const double2 v = rd(k);
    r = make_double2((v.x - a2 * r.x) / den, (v.y - a2 * r.y) / den);
    s[k * sstride] = r;
    const double uk = k == K - 1 ? a2 : 0.;
    z = (uk - a2 * z) / den;
    zz[(long)k * ncol] = z;
  }
  // back substitution of both
  for (int k = K - 2; k >= 0; --k) {
    const double2 v = s[k * sstride];
    const double c = cp[(long)k * ncol];
    r = make_double2(v.x - c * r.x, v.y - c * r.y);
    s[k * sstride] = r;
    z = zz[(long)k * ncol] - c * z;
    zz[(long)k * ncol] = z;
  }
  // r, z hold row 0; rows K-1 from memory
  const double2 rl = s[(long)(K - 1) * sstride];
  const double zl = zz[(long)(K - 1) * ncol];
  const double fdn = 1. + z + a2 * zl / gamma;
  const double fx = (r.x + a2 * rl.x / gamma) / fdn, fy = (r.y + a2 * rl.y / gamma) / fdn;
  for (int k = 0; k < K; ++k) {
    const double2 v = s[k * sstride];
    const double zk = zz[(long)k * ncol];
    s[k * sstride] = make_double2(v.x - fx * zk, v.y - fy * zk);
  }
}

// Thomas sweep of the mixed form in double-float arithmetic (pairs of FP32
// with error-free products and sums, ~48 significant bits) on the FP32
// pipes; GB300 issues FP64 at 1/64 of the FP32 rate.  Tables (built on the
// host in FP64, split hi + lo): zt[k] for k < K-1 and 1/den for k = K-1 (0
// for the zero mode), azt[k] = dzi^2 * zt[k] for the back substitution.  The
// recurrence carries its value in double-float from plane to plane; the
// forward intermediate between the sweeps is kept in the FP32 spectrum, and
// the 1/(M*J) FFT scale is applied at the final FP32 store.
__global__ void __launch_bounds__(128) k_thomas_df(Geo g, float2 *__restrict__ S, const float2 *__restrict__ zt,
                                                   const float2 *__restrict__ azt, float a2h, float a2l,
                                                   float fscale) {
  const long t = blockIdx.x * (long)blockDim.x + threadIdx.x;
  const long ncol = (long)g.MX * g.J;
  if (t >= ncol) return;
  const int kx = (int)(t % g.MX), ky = (int)(t / g.MX);
  const int kyy = ky <= g.J / 2 ? ky : g.J - ky;
  const long zstride = (long)(g.J / 2 + 1) * g.MX;
  const float2 *z = zt + (long)kyy * g.MX + kx;
  const float2 *az = azt + (long)kyy * g.MX + kx;
  const long sstride = (long)g.J * g.MX;
  float2 *s = S + t;
  const int K = g.K;
  constexpr int PF = 16;
  // previous plane's value, real and imaginary parts, double-float
  float prh = 0.f, prl = 0.f, pih = 0.f, pil = 0.f;
  // Both sweeps run over chunks of PF planes with the next chunk's loads
  // issued before the current chunk is computed (two buffers), so that the
  // HBM latency of a chunk overlaps the dependent double-float chain of the
  // previous one.
  float2 buf[2][PF], cb[2][PF];
  auto load_fwd = [&](int slot, int k0) {
#pragma unroll
    for (int q = 0; q < PF; ++q) {
      const int k = k0 + q;
      if (k < K) { buf[slot][q] = s[k * sstride]; cb[slot][q] = z[(long)k * zstride]; }
    }
  };
  auto fwd = [&](int slot, int k0) {
#pragma unroll
    for (int q = 0; q < PF; ++q) {
      const int k = k0 + q;
      if (k >= K) break;
      float rh = buf[slot][q].x, rl = 0.f, ih = buf[slot][q].y, il = 0.f;
      if (k > 0) {  // d - dzi^2 * prev
        float qh, ql;
        df_mul(a2h, a2l, prh, prl, qh, ql);
        df_add(rh, rl, -qh, -ql, rh, rl);
        df_mul(a2h, a2l, pih, pil, qh, ql);
        df_add(ih, il, -qh, -ql, ih, il);
      }
      // times the pivot reciprocal (k < K-1) or 1/den (k = K-1)
      df_mul(rh, rl, cb[slot][q].x, cb[slot][q].y, prh, prl);
      df_mul(ih, il, cb[slot][q].x, cb[slot][q].y, pih, pil);
      const float2 o = make_float2(__fadd_rn(prh, prl), __fadd_rn(pih, pil));
      if (k < K - 1) s[k * sstride] = o;
      else s[k * sstride] = make_float2(o.x * fscale, o.y * fscale);
    }
  };
  load_fwd(0, 0);
  for (int k0 = 0; k0 < K; k0 += 2 * PF) {
    if (k0 + PF < K) load_fwd(1, k0 + PF);
    fwd(0, k0);
    if (k0 + PF >= K) break;
    if (k0 + 2 * PF < K) load_fwd(0, k0 + 2 * PF);
    fwd(1, k0 + PF);
  }
  // back substitution x_k = x'_k - dzi^2 z_k x_{k+1}
  auto load_bwd = [&](int slot, int k1) {
#pragma unroll
    for (int q = 0; q < PF; ++q) {
      const int k = k1 - q;
      if (k >= 0) { buf[slot][q] = s[k * sstride]; cb[slot][q] = az[(long)k * zstride]; }
    }
  };
  auto bwd = [&](int slot, int k1) {
#pragma unroll
    for (int q = 0; q < PF; ++q) {
      const int k = k1 - q;
      if (k < 0) break;
      float qh, ql;
      df_mul(cb[slot][q].x, cb[slot][q].y, prh, prl, qh, ql);
      df_add(buf[slot][q].x, 0.f, -qh, -ql, prh, prl);
      df_mul(cb[slot][q].x, cb[slot][q].y, pih, pil, qh, ql);
      df_add(buf[slot][q].y, 0.f, -qh, -ql, pih, pil);
      s[k * sstride] = make_float2(__fadd_rn(prh, prl) * fscale, __fadd_rn(pih, pil) * fscale);
    }
  };
  if (K >= 2) load_bwd(0, K - 2);
  for (int k1 = K - 2; k1 >= 0; k1 -= 2 * PF) {
    if (k1 - PF >= 0) load_bwd(1, k1 - PF);
    bwd(0, k1);
    if (k1 - PF < 0) break;
    if (k1 - 2 * PF >= 0) load_bwd(0, k1 - 2 * PF);
    bwd(1, k1 - PF);
  }
}

// inverse real FFT along x: spectrum row -> phi(i,j,k), k = 1..K
template <typename T>
__global__ void __launch_bounds__(128) k_ifftx(Geo g, FftPlan plx, const typename cpx<T>::t *__restrict__ S,
                                               T *__restrict__ phi, const typename cpx<T>::t *__restrict__ twM,
                                               const typename cpx<T>::t *__restrict__ twN, int rows) {
  typedef typename cpx<T>::t C;
  extern __shared__ unsigned char smraw[];
  C *A = reinterpret_cast<C *>(smraw);
  const int M = g.I / 2;
  C *B = A + rows * M;
  C *X = B + rows * M;  // rows*(M+1) spectrum staging
  const int row0 = blockIdx.x * rows;
  const int nrow = g.J * g.K;
  for (int t = threadIdx.x; t < rows * (M + 1); t += blockDim.x) {
    const int r = t / (M + 1), kx = t - r * (M + 1);
    const int row = row0 + r;
    X[t] = row < nrow ? S[(long)row * g.MX + kx] : cmk<C>((T)0, (T)0);
  }
  __syncthreads();
  for (int t = threadIdx.x; t < rows * M; t += blockDim.x) {
    const int r = t / M, kx = t - r * M;
    const C Xk = X[r * (M + 1) + kx];
    const C Xc = cconj(X[r * (M + 1) + (M - kx)]);
    const C E = cscale(cadd(Xk, Xc), (T)0.5);
    const C O = cmul(cscale(csub(Xk, Xc), (T)0.5), cconj(twN[kx]));
    A[r * M + kx] = cadd(E, cmk<C>(-O.y, O.x));  // E + i O
  }
  __syncthreads();
  C *Z = fft_smem1<C>(A, B, M, rows, M, plx, twM, 1);
  for (int t = threadIdx.x; t < rows * g.I; t += blockDim.x) {
    const int r = t / g.I, i = t - r * g.I;
    const int row = row0 + r;
    if (row >= nrow) continue;
    const int j = row % g.J, k = row / g.J + 1;
    const T *Zr = reinterpret_cast<const T *>(Z + r * M);
    phi[fidx(g, i, j, k)] = Zr[i];
  }
}

template <typename TIn, typename T>
void launch_poisson(cudaStream_t s, const Geo &g, const FftPlan &plx, const FftPlan &ply, const TIn *fu,
                    const TIn *fv, TIn *fw, void *spec, T *phi, const void *twM, const void *twN, const void *twJ,
                    const double *zt, double dtidxi, double dtidyi, double dtidzi, int *launches, bool res64,
                    const float2 *thomas_df, PoissonHook hook, PoissonResid resid) {
  typedef typename cpx<T>::t C;
  C *S = reinterpret_cast<C *>(spec);
  const int M = g.I / 2;
  const int rows = g.I <= 256 ? 4 : 2;
  const int nrow = g.J * g.K;
  size_t smx = (size_t)2 * rows * M * sizeof(C);
  if constexpr (sizeof(T) == 4 && sizeof(TIn) == 4) {
    // register four-step FFTs for the supported lengths
    if (reg_n2(M) && reg_n2(g.J)) {
      float2 *Sf = reinterpret_cast<float2 *>(spec);
      const float2 *tM = (const float2 *)twM, *tN = (const float2 *)twN, *tJ = (const float2 *)twJ;
      hook(0, 1);
      fftx_r(s, g, (const float *)fu, (const float *)fv, (float *)fw, Sf, tM, tN, dtidxi, dtidyi, dtidzi, res64, false,
             nullptr, resid);
      hook(0, 0);
      hook(1, 1);
      ffty_r(s, g, Sf, tJ, 0);
      hook(1, 0);
      const long ncol = (long)g.MX * g.J;
      const double scale = 1.0 / ((double)M * g.J);
      hook(2, 1);
      const double a2 = g.dzi * g.dzi;
      const float a2h = (float)a2, a2l = (float)(a2 - (double)a2h);
      k_thomas_df<<<(unsigned)((ncol + 127) / 128), 128, 0, s>>>(
          g, Sf, thomas_df, thomas_df + (long)g.K * (g.J / 2 + 1) * g.MX, a2h, a2l, (float)scale);
      hook(2, 0);
      hook(3, 1);
      ffty_r(s, g, Sf, tJ, 1);
      hook(3, 0);
      hook(4, 1);
      fftx_r(s, g, nullptr, nullptr, nullptr, Sf, tM, tN, 0., 0., 0., false, true, (float *)phi, PoissonResid{});
      hook(4, 0);
      if (launches) *launches += 5;
      return;
    }
  }
  hook(0, 1);
  if (res64 && sizeof(TIn) == 4)
    k_fillps_fftx<TIn, T, float, true><<<(nrow + rows - 1) / rows, 128, smx, s>>>(
        g, plx, fu, fv, fw, S, (const C *)twM, (const C *)twN, dtidxi, dtidyi, dtidzi, rows);
  else if (res64)
    k_fillps_fftx<TIn, T, double><<<(nrow + rows - 1) / rows, 128, smx, s>>>(g, plx, fu, fv, fw, S, (const C *)twM,
                                                                            (const C *)twN, dtidxi, dtidyi, dtidzi,
                                                                            rows);
  else
    k_fillps_fftx<TIn, T, TIn><<<(nrow + rows - 1) / rows, 128, smx, s>>>(g, plx, fu, fv, fw, S, (const C *)twM,
                                                                         (const C *)twN, dtidxi, dtidyi, dtidzi,
                                                                         rows);
  hook(0, 0);
  const int cols = 8;
  size_t smy = (size_t)2 * (g.J + 1) * cols * sizeof(C);
  dim3 gy((g.MX + cols - 1) / cols, g.K);
  hook(1, 1);
  k_ffty<T><<<gy, 256, smy, s>>>(g, ply, S, (const C *)twJ, cols, 0);
  hook(1, 0);
  const long ncol = (long)g.MX * g.J;
  const double scale = 1.0 / ((double)M * g.J);
  hook(2, 1);
  if constexpr (sizeof(T) == 4) {
    const double a2 = g.dzi * g.dzi;
    const float a2h = (float)a2, a2l = (float)(a2 - (double)a2h);
    k_thomas_df<<<(unsigned)((ncol + 127) / 128), 128, 0, s>>>(
        g, reinterpret_cast<float2 *>(S), thomas_df, thomas_df + (long)g.K * (g.J / 2 + 1) * g.MX, a2h, a2l,
        (float)scale);
  } else if (g.zper) {
    k_thomas_cyclic<<<(unsigned)((ncol + 127) / 128), 128, 0, s>>>(g, reinterpret_cast<double2 *>(S), zt, zt + g.MX,
                                                                    g.dzi * g.dzi, scale,
                                                                    const_cast<double *>(zt) + g.MX + g.J);
  } else {
    k_thomas<T><<<(unsigned)((ncol + 127) / 128), 128, 0, s>>>(g, S, zt, g.dzi * g.dzi, scale);
  }
  hook(2, 0);
  hook(3, 1);
  k_ffty<T><<<gy, 256, smy, s>>>(g, ply, S, (const C *)twJ, cols, 1);
  hook(3, 0);
  size_t smi = (size_t)(2 * rows * M + rows * (M + 1)) * sizeof(C);
  hook(4, 1);
  k_ifftx<T><<<(nrow + rows - 1) / rows, 128, smi, s>>>(g, plx, S, phi, (const C *)twM, (const C *)twN, rows);
  hook(4, 0);
  if (launches) *launches += 5;
}

template <typename T>
int poisson_set_smem_limits() {
  if (sizeof(T) == 4 && ffty_r_set_smem_limits() != 0) return -1;
  cudaError_t e[4];
  e[0] = cudaFuncSetAttribute(k_fillps_fftx<T, T, double>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
  if (sizeof(T) == 4)
    if (cudaFuncSetAttribute(k_fillps_fftx<T, T, float, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             200 * 1024) != cudaSuccess)
      return -1;
  e[1] = cudaFuncSetAttribute(k_fillps_fftx<T, T, T>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
  e[2] = cudaFuncSetAttribute(k_ffty<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
  e[3] = cudaFuncSetAttribute(k_ifftx<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
  for (cudaError_t x : e)
    if (x != cudaSuccess) return -1;
  return 0;
}

template void launch_poisson<double, double>(cudaStream_t, const Geo &, const FftPlan &, const FftPlan &,
                                             const double *, const double *, double *, void *, double *,
                                             const void *, const void *, const void *, const double *, double, double,
                                             double, int *, bool, const float2 *, PoissonHook, PoissonResid);
template void launch_poisson<float, float>(cudaStream_t, const Geo &, const FftPlan &, const FftPlan &,
                                           const float *, const float *, float *, void *, float *, const void *,
                                           const void *, const void *, const double *, double, double, double, int *,
                                           bool, const float2 *, PoissonHook, PoissonResid);
template int poisson_set_smem_limits<double>();
template int poisson_set_smem_limits<float>();

}  // namespace ibmk
