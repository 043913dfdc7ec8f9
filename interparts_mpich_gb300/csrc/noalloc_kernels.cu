// noalloc_kernels.cu -- chkdiv for callers that cannot allocate device memory.
//
// Some callers of this library own every byte of device memory themselves: a
// Fortran/OpenACC or CUDA Fortran main program whose velocity arrays already
// live on the GPU under its own memory manager, a solver running under a
// fixed device-memory budget, or code that must not call cudaMalloc at a given
// point (a real-time loop, a region being recorded into a CUDA graph).  They
// can still check the divergence of their fields with ibm_chkdiv_noalloc:
// it reads the caller's device arrays, writes the caller's device output and
// keeps its per-plane partial results in the fixed array below instead of
// allocating.
//
// Limits and sharing rules:
//   * the array holds one (sum, max, location) record per k-plane, so ktot is
//     limited to IBM_NOALLOC_MAX_PLANES (4096, 96 KiB); larger grids are
//     rejected with IBM_E_INVALID;
//   * every GPU that loads the library holds the array until the process exits;
//   * all calls share it and it keeps the last call's contents; each call
//     rewrites every record it reads, so nothing has to be cleared, but calls
//     that overlap on the GPU (for example on two streams at once) race;
//   * the first call on a device looks up the array's device address with
//     cudaGetSymbolAddress (with that device current) and caches it; make that
//     first call before any stream capture.  The cached address belongs to
//     the device's primary context: after cudaDeviceReset a new context may
//     load the array elsewhere, so a process that resets a device must not
//     call this function on that device again;
//   * each launch reports its own status (cudaLaunchKernel), so an error
//     pending from the caller's earlier work is neither returned here nor
//     cleared.
#include <mutex>

#include "kernels.cuh"

#define IBM_NOALLOC_MAX_PLANES 4096
#define IBM_NOALLOC_MAX_DEVICES 64

// per-plane partial records: [0,P) sums, [P,2P) maxima, [2P,3P) locations
static __device__ __align__(256) double g_noalloc_scratch[3 * IBM_NOALLOC_MAX_PLANES];

namespace {

std::mutex g_noalloc_mutex;
double *g_noalloc_ptr[IBM_NOALLOC_MAX_DEVICES] = {nullptr};

// One block per k-plane: divergence of (u,v,w) given in the reference layout
// (0:itot+1, 0:jtot+1, 0:ktot+1), i fastest, as chkdiv.f90:21-38 computes it.
__global__ void __launch_bounds__(256) k_div_planes_ref(const double *__restrict__ u, const double *__restrict__ v,
                                                        const double *__restrict__ w, int I, int J, double dxi,
                                                        double dyi, double dzi, double *__restrict__ rec, int K) {
  const int k = blockIdx.x + 1;
  const long si = 1, sj = I + 2, sk = (long)(I + 2) * (J + 2);
  double s = 0., m = -1.;
  long long loc = -1;
  const long n = (long)I * J;
  for (long t = threadIdx.x; t < n; t += blockDim.x) {
    const int i = (int)(t % I) + 1, j = (int)(t / I) + 1;
    const long c = i * si + j * sj + k * sk;
    const double div = (w[c] - w[c - sk]) * dzi + (v[c] - v[c - sj]) * dyi + (u[c] - u[c - si]) * dxi;
    s += div;
    const double a = fabs(div);
    if (a > m) { m = a; loc = (long long)(k - 1) * n + t; }
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
  if (threadIdx.x == 0) {
    rec[blockIdx.x] = ss[0];
    rec[K + blockIdx.x] = sm[0];
    rec[2 * K + blockIdx.x] = (double)sl[0];
  }
}

// combines the plane records in k order; out = {tot, max, i, j, k} (1-based)
__global__ void k_div_planes_final(const double *__restrict__ rec, int K, int I, int J, double *__restrict__ out) {
  if (threadIdx.x != 0) return;
  double s = 0., m = -1.;
  long long l = -1;
  for (int k = 0; k < K; ++k) {
    s += rec[k];
    const double mk = rec[K + k];
    const long long lk = (long long)rec[2 * K + k];
    if (mk > m || (mk == m && lk >= 0 && (l < 0 || lk < l))) { m = mk; l = lk; }
  }
  out[0] = s;
  out[1] = m;
  if (l >= 0) {
    const long long n = (long long)I * J;
    out[2] = (double)(l % I + 1);
    out[3] = (double)((l % n) / I + 1);
    out[4] = (double)(l / n + 1);
  } else {
    out[2] = out[3] = out[4] = 0.;
  }
}

}  // namespace

extern "C" int ibm_chkdiv_noalloc(const double *u, const double *v, const double *w, int itot, int jtot, int ktot,
                                  double dxi, double dyi, double dzi, double *out5, void *cuda_stream) {
  if (!u || !v || !w || !out5 || itot < 1 || jtot < 1 || ktot < 1) return IBM_E_INVALID;
  if (ktot > IBM_NOALLOC_MAX_PLANES) return IBM_E_INVALID;  // the fixed array holds 4096 plane records
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= IBM_NOALLOC_MAX_DEVICES) return IBM_E_CUDA;
  double *rec = nullptr;
  {
    std::lock_guard<std::mutex> lk(g_noalloc_mutex);
    if (!g_noalloc_ptr[dev]) {
      double *p = nullptr;
      if (cudaGetSymbolAddress((void **)&p, g_noalloc_scratch) != cudaSuccess || !p) return IBM_E_CUDA;
      g_noalloc_ptr[dev] = p;
    }
    rec = g_noalloc_ptr[dev];
  }
  cudaStream_t s = (cudaStream_t)cuda_stream;
  int I = itot, J = jtot, K = ktot;
  void *a1[] = {(void *)&u, (void *)&v, (void *)&w, &I, &J, &dxi, &dyi, &dzi, &rec, &K};
  if (cudaLaunchKernel((const void *)k_div_planes_ref, dim3(ktot), dim3(256), a1, 0, s) != cudaSuccess)
    return IBM_E_CUDA;
  const double *crec = rec;
  void *a2[] = {(void *)&crec, &K, &I, &J, &out5};
  if (cudaLaunchKernel((const void *)k_div_planes_final, dim3(1), dim3(32), a2, 0, s) != cudaSuccess)
    return IBM_E_CUDA;
  return IBM_OK;
}
