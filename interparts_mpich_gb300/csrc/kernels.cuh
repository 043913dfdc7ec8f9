// kernels.cuh -- launcher declarations shared by the C ABI and the kernels.
#pragma once
#include "ibm_common.cuh"

struct FftPlan {
  int nst;       // number of Stockham stages
  int rad[16];   // radix of each stage (2, 3 or 4)
};

namespace ibmk {

// fluid_kernels.cu
template <typename T>
void launch_predict(cudaStream_t s, const Geo &g, int stage, const T *u, const T *v, const T *w, const T *p, T *ru,
                    T *rv, T *rw, T *fu, T *fv, T *fw, double f1, double f2, double f3);
template <typename T, typename TP>
void launch_correc(cudaStream_t s, const Geo &g, const T *fu, const T *fv, const T *fw, const T *phi, T *u, T *v,
                   T *w, TP *pn, double fi, double fj, double fk);
template <typename T> void launch_ref_to_dev(cudaStream_t s, const Geo &g, const double *ref, T *dev);
template <typename T> void launch_dev_to_ref(cudaStream_t s, const Geo &g, const T *dev, double *ref);
void launch_chkdiv(cudaStream_t s, const Geo &g, const double *u, const double *v, const double *w,
                   double *scratch, double *out);
void launch_chkdt(cudaStream_t s, const Geo &g, const double *u, const double *v, const double *w,
                  double *scratch, double *out);
void launch_wallshear(cudaStream_t s, const Geo &g, const double *v, double *out);
void launch_d2f(cudaStream_t s, long n, const double *a, float *b);
void launch_f2d(cudaStream_t s, long n, const float *a, double *b);

// fft_kernels.cu
template <typename T>
void launch_poisson(cudaStream_t s, const Geo &g, const FftPlan &plx, const FftPlan &ply, const T *fu, const T *fv,
                    T *fw, void *spec, T *phi, const void *twM, const void *twN, const void *twJ,
                    const double *zt, double dtidxi, double dtidyi, double dtidzi, int *launches);
template <typename T> int poisson_set_smem_limits();

// ibm_kernels.cu
struct IbmBuffers {
  // per-point arrays [np*nl]
  double *xfp, *yfp, *zfp, *ul, *vl, *wl, *dudtl, *dvdtl, *dwdtl, *fxl, *fyl, *fzl;
  PointStencil *st;
  int *nla;          // [np]
  double *pf;        // particle scalar fields [PF_N*np]
  double *diag;      // [8] force totals etc.
  int *err;          // shared with PartBuffers::err ([2]: point outside the grid)
};
template <typename T>
void launch_ibm_stencil(cudaStream_t s, const Geo &g, const PartGeo &pg, IbmBuffers b);
template <typename T>
void launch_ibm_interp_force(cudaStream_t s, const Geo &g, const PartGeo &pg, IbmBuffers b, const T *fu,
                             const T *fv, const T *fw, double dt, int first);
template <typename T>
void launch_ibm_spread(cudaStream_t s, const Geo &g, const PartGeo &pg, IbmBuffers b, T *fu, T *fv, T *fw,
                       double dt, int first);
template <typename T>
void launch_zero_plane(cudaStream_t s, const Geo &g, T *f, int k);
void launch_slip_residual(cudaStream_t s, const PartGeo &pg, IbmBuffers b, double *out);

// particle_kernels.cu
struct PartBuffers {
  double *pf;     // [PF_N*np]
  double *cf;     // [CF_N*np*nq]
  int *qmax;      // [np]
  int *firstc;    // [np*nq]
  int *ofirstc;   // [np*nq]
  int *nb;        // [np*9]
  int *mslv;      // [np]
  double *rkp;    // [RK_N*np]
  double *sincos; // [4*nl]: sin(theta), cos(theta), sin(phi), cos(phi)
  int *err;       // [4] error flags
  double *red;    // [np*9*6] sphere-integral partials
};
template <typename T>
void launch_sphere_integrals(cudaStream_t s, const Geo &g, const PartGeo &pg, PartBuffers b, const T *u, const T *v,
                             const T *w, int type);
void launch_save_old(cudaStream_t s, const PartGeo &pg, PartBuffers b);
void launch_collide_update(cudaStream_t s, const PartGeo &pg, PartBuffers b, int iter, int rkiter, double dt);
void launch_ne_finalize(cudaStream_t s, const PartGeo &pg, PartBuffers b, IbmBuffers ib, int init_flags);

}  // namespace ibmk
