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

// ---------------------------------------------------------------------------
// fillps + forward real FFT along x.  One CTA handles ROWS rows (j,k).
// Reads the forced predictor (fu,fv,fw) with the bounduvw(dudt) wall values
// w(0)=w(kmax)=0 applied (and stored back into fw plane K).
// ---------------------------------------------------------------------------
template <typename T>
__global__ void __launch_bounds__(128) k_fillps_fftx(Geo g, FftPlan plx, const T *__restrict__ fu,
                                                     const T *__restrict__ fv, T *__restrict__ fw,
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
  // 1. right-hand side, packed z_m = x_{2m} + i x_{2m+1}
  for (int t = threadIdx.x; t < rows * g.I; t += blockDim.x) {
    const int r = t / g.I, i = t - r * g.I;
    const int row = row0 + r;
    T val = 0;
    if (row < nrow) {
      const int j = row % g.J, k = row / g.J + 1;
      const long c = fidx(g, i, j, k);
      const T wk = (k == g.K) ? (T)0 : fw[c];
      const T wkm = fw[c - g.plane];  // plane 0 holds w(0)=0
      if (k == g.K) fw[c] = (T)0;
      const T vjm = fv[fidx(g, i, j == 0 ? g.J - 1 : j - 1, k)];
      const T uim = fu[fidx(g, i == 0 ? g.I - 1 : i - 1, j, k)];
      val = ((wk - wkm) * (T)dtidzi + (fv[c] - vjm) * (T)dtidyi + (fu[c] - uim) * (T)dtidxi);
    }
    T *Ar = reinterpret_cast<T *>(A + r * M);
    Ar[i] = val;
  }
  __syncthreads();
  C *Z = fft_smem<C>(A, B, M, rows, 1, M, plx, twM, 0);
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
  C *A = reinterpret_cast<C *>(smraw);
  C *B = A + g.J * cols;
  const int kx0 = blockIdx.x * cols;
  const int k = blockIdx.y;
  C *plane = S + (long)k * g.J * g.MX;
  for (int t = threadIdx.x; t < g.J * cols; t += blockDim.x) {
    const int jy = t / cols, cx = t - jy * cols;
    const int kx = kx0 + cx;
    A[jy * cols + cx] = (kx < g.MX) ? plane[(long)jy * g.MX + kx] : cmk<C>((T)0, (T)0);
  }
  __syncthreads();
  C *Y = fft_smem<C>(A, B, g.J, cols, cols, 1, ply, twJ, inv);
  for (int t = threadIdx.x; t < g.J * cols; t += blockDim.x) {
    const int jy = t / cols, cx = t - jy * cols;
    const int kx = kx0 + cx;
    if (kx < g.MX) plane[(long)jy * g.MX + kx] = Y[jy * cols + cx];
  }
}

// Thomas sweep along z for every (kx,ky) (solver.f90:94-134), with the
// precomputed pivots zt (pivot reciprocal for k<K, denominator for k=K).
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
  const T A2 = (T)a2;
  // forward elimination
  C prev = cscale(s[0], (T)scale);
  {
    const T z0 = (T)z[0];
    prev = cscale(prev, z0);
    s[0] = prev;
  }
  for (int k = 1; k < g.K - 1; ++k) {
    const T zk = (T)z[k * zstride];
    C cur = cscale(s[k * sstride], (T)scale);
    cur = cscale(csub(cur, cscale(prev, A2)), zk);
    s[k * sstride] = cur;
    prev = cur;
  }
  {
    const int k = g.K - 1;
    const T den = (T)z[k * zstride];
    C cur = cscale(s[k * sstride], (T)scale);
    if (den != (T)0) {
      cur = csub(cur, cscale(prev, A2));
      cur = cmk<C>(cur.x / den, cur.y / den);
    } else {
      cur = cmk<C>((T)0, (T)0);
    }
    s[k * sstride] = cur;
    prev = cur;
  }
  // back substitution, d(k) = c(k)*z(k) with c(k) = dzi^2 for k < kmax
  for (int k = g.K - 2; k >= 0; --k) {
    const T d = A2 * (T)z[k * zstride];
    C cur = csub(s[k * sstride], cscale(prev, d));
    s[k * sstride] = cur;
    prev = cur;
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
  C *Z = fft_smem<C>(A, B, M, rows, 1, M, plx, twM, 1);
  for (int t = threadIdx.x; t < rows * g.I; t += blockDim.x) {
    const int r = t / g.I, i = t - r * g.I;
    const int row = row0 + r;
    if (row >= nrow) continue;
    const int j = row % g.J, k = row / g.J + 1;
    const T *Zr = reinterpret_cast<const T *>(Z + r * M);
    phi[fidx(g, i, j, k)] = Zr[i];
  }
}

template <typename T>
void launch_poisson(cudaStream_t s, const Geo &g, const FftPlan &plx, const FftPlan &ply, const T *fu, const T *fv,
                    T *fw, void *spec, T *phi, const void *twM, const void *twN, const void *twJ,
                    const double *zt, double dtidxi, double dtidyi, double dtidzi, int *launches) {
  typedef typename cpx<T>::t C;
  C *S = reinterpret_cast<C *>(spec);
  const int M = g.I / 2;
  const int rows = g.I <= 256 ? 4 : 2;
  const int nrow = g.J * g.K;
  size_t smx = (size_t)2 * rows * M * sizeof(C);
  k_fillps_fftx<T><<<(nrow + rows - 1) / rows, 128, smx, s>>>(g, plx, fu, fv, fw, S, (const C *)twM,
                                                               (const C *)twN, dtidxi, dtidyi, dtidzi, rows);
  const int cols = 8;
  size_t smy = (size_t)2 * g.J * cols * sizeof(C);
  dim3 gy((g.MX + cols - 1) / cols, g.K);
  k_ffty<T><<<gy, 256, smy, s>>>(g, ply, S, (const C *)twJ, cols, 0);
  const long ncol = (long)g.MX * g.J;
  const double scale = 1.0 / ((double)M * g.J);
  k_thomas<T><<<(unsigned)((ncol + 127) / 128), 128, 0, s>>>(g, S, zt, g.dzi * g.dzi, scale);
  k_ffty<T><<<gy, 256, smy, s>>>(g, ply, S, (const C *)twJ, cols, 1);
  size_t smi = (size_t)(2 * rows * M + rows * (M + 1)) * sizeof(C);
  k_ifftx<T><<<(nrow + rows - 1) / rows, 128, smi, s>>>(g, plx, S, phi, (const C *)twM, (const C *)twN, rows);
  if (launches) *launches += 5;
}

template <typename T>
int poisson_set_smem_limits() {
  typedef typename cpx<T>::t C;
  (void)sizeof(C);
  cudaError_t e1 = cudaFuncSetAttribute(k_fillps_fftx<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
  cudaError_t e2 = cudaFuncSetAttribute(k_ffty<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
  cudaError_t e3 = cudaFuncSetAttribute(k_ifftx<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
  return (e1 == cudaSuccess && e2 == cudaSuccess && e3 == cudaSuccess) ? 0 : -1;
}

template void launch_poisson<double>(cudaStream_t, const Geo &, const FftPlan &, const FftPlan &, const double *,
                                     const double *, double *, void *, double *, const void *, const void *,
                                     const void *, const double *, double, double, double, int *);
template void launch_poisson<float>(cudaStream_t, const Geo &, const FftPlan &, const FftPlan &, const float *,
                                    const float *, float *, void *, float *, const void *, const void *,
                                    const void *, const double *, double, double, double, int *);
template int poisson_set_smem_limits<double>();
template int poisson_set_smem_limits<float>();

}  // namespace ibmk
