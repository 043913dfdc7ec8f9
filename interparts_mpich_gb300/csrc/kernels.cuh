// kernels.cuh -- launcher declarations shared by the C ABI and the kernels.
#pragma once
#include <cuda_bf16.h>

#include "ibm_common.cuh"

struct FftPlan {
  int nst;       // number of Stockham stages
  int rad[16];   // radix of each stage (2, 3 or 4)
};

namespace ibmk {

// fluid_kernels.cu
template <typename TU, typename T>
void launch_predict(cudaStream_t s, const Geo &g, int stage, const TU *u, const TU *v, const TU *w, const TU *p,
                    T *ru, T *rv, T *rw, T *fu, T *fv, T *fw, double f1, double f2, double f3,
                    const double *cb = nullptr, double bcoef = 0., int kind = IBM_PREDICTOR_AUTO,
                    int *err = nullptr);
template <typename TU>
void launch_scalar_stage(cudaStream_t s, const Geo &g, int stage, const TU *u, const TU *v, const TU *w,
                         const double *cf, double *rc, double *cnext, double kappa, double f1, double f2, double f3);
void launch_boundscal(cudaStream_t s, const Geo &g, double *cf, int top_dirichlet, double top, int bot_dirichlet,
                      double bot);
template <typename TF, typename TPh, typename TU>
void launch_correc(cudaStream_t s, const Geo &g, const TF *fu, const TF *fv, const TF *fw, const TPh *phi, TU *u,
                   TU *v, TU *w, double *pn, float *pn32, double fi, double fj, double fk);
void launch_correc_mixed2(cudaStream_t s, const Geo &g, const float *fu, const float *fv, const float *fw,
                          const float *phi1, const float *phi2, float *u, float *v, float *w, float *ph, float *pl,
                          double fi, double fj, double fk);
void launch_correc_mixed(cudaStream_t s, const Geo &g, const float *fu, const float *fv, const float *fw,
                         const float *phi, float *u, float *v, float *w, float *ph, float *pl, double fi, double fj,
                         double fk);
void launch_df_to_d(cudaStream_t s, long n, const float *h, const float *l, double *d);
void launch_d_to_df(cudaStream_t s, long n, const double *d, float *h, float *l);
template <typename T> void launch_ref_to_dev(cudaStream_t s, const Geo &g, const double *ref, T *dev);
template <typename T> void launch_dev_to_ref(cudaStream_t s, const Geo &g, const T *dev, double *ref);
template <typename T>
void launch_chkdiv(cudaStream_t s, const Geo &g, const T *u, const T *v, const T *w, double *scratch, double *out);
template <typename T>
void launch_chkdt(cudaStream_t s, const Geo &g, const T *u, const T *v, const T *w, double *scratch, double *out);
template <typename T>
void launch_wallshear(cudaStream_t s, const Geo &g, const T *v, double *scratch, double *out);
void launch_d2f(cudaStream_t s, long n, const double *a, float *b);
void launch_f2d(cudaStream_t s, long n, const float *a, double *b);

// fft_kernels.cu
// TIn: type of the velocity read by fillps (the forced predictor, or the
// corrected state for the defect-correction residual); T: FFT type;
// Optional callback around each of the five kernels of a solve (stage 0
// fillps + x FFT, 1 y FFT, 2 Thomas, 3 inverse y FFT, 4 inverse x FFT;
// begin = 1 before the launch, 0 after), for per-kernel event timing.
struct PoissonHook {
  void (*fn)(void *arg, int stage, int begin);
  void *arg;
  void operator()(int stage, int begin) const {
    if (fn) fn(arg, stage, begin);
  }
};
// Defect-correction right-hand side without a stored corrected state: with
// phi1 the FP32 register-FFT path forms the divergence residual of
// u - (fi, fj, fk) grad(phi1) on the fly (poisson_fused_residual_ok).
struct PoissonResid {
  const float *phi1 = nullptr;
  float fi = 0.f, fj = 0.f, fk = 0.f;
};
bool poisson_fused_residual_ok(const Geo &g);
// res64: evaluate the divergence in FP64 arithmetic.
template <typename TIn, typename T>
void launch_poisson(cudaStream_t s, const Geo &g, const FftPlan &plx, const FftPlan &ply, const TIn *fu,
                    const TIn *fv, TIn *fw, void *spec, T *phi, const void *twM, const void *twN, const void *twJ,
                    const double *zt, double dtidxi, double dtidyi, double dtidzi, int *launches, bool res64 = false,
                    const float2 *thomas_df = nullptr,  // FP32 spectrum: double-float pivot tables
                    PoissonHook hook = PoissonHook{nullptr, nullptr}, PoissonResid resid = PoissonResid{});
template <typename T> int poisson_set_smem_limits();

// ibm_kernels.cu
// rows (y, z) of a particle's box with a recorded x extent; boxes with more
// rows are read whole
constexpr int IBM_BOX_ROWS = 1024;
struct IbmBuffers {
  // per-point arrays [np*nl]
  double *xfp, *yfp, *zfp, *ul, *vl, *wl, *dudtl, *dvdtl, *dwdtl, *fxl, *fyl, *fzl;
  PointStencil *st;
  PointRec *rec;     // mixed form: [np*nl] compact point records (make_cs)
  float *fxs, *fys, *fzs;  // mixed forms: [np*nl] point forces F_l (FP32; fxl.. hold FP64 copies at the boundary)
  float4 *pvh, *pvl;       // mixed forms: [np] particle velocity u, v, w as FP32 pairs hi + lo
  int4 *pref;        // mixed form: [np] reference floors (refx, refy, refz) of the particles
  float4 *pcen;      // mixed form: [np] centre position in cells relative to the reference floor (FP32)
  float *slip;       // mixed form: [3][np*nl] slip U - u~ of the last pass (FP32)
  int *bgeo;         // mixed form: [np][3][8] per-particle stencil boxes
  unsigned *rowm;    // mixed form: [np][3][IBM_BOX_ROWS] the cells of every box row the stencils touch (bit cx)
  int *nla;          // [np]
  double *pf;        // particle scalar fields [PF_N*np]
  double *diag;      // [8] force totals etc.
  int *err;          // shared with PartBuffers::err ([2]: point outside the grid)
  double *psum;      // [np*9] mixed form: per-component force and lever-arm sums
  float *rsum;       // [np*3] mixed form: per-component sums of the first-pass slip (U - u~)^2
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
// mixed form: FP32 fields, FP32 weights and interpolation sums, FP64 point
// forces and per-particle sums
void launch_ibm_stencil_f(cudaStream_t s, const Geo &g, const PartGeo &pg, IbmBuffers b);
int launch_ibm_interp_force_f(cudaStream_t s, const Geo &g, const PartGeo &pg, IbmBuffers b, const float *fu,
                              const float *fv, const float *fw, double dt, int first, const int *gate = nullptr);
// learned form: the network's output Y, its target de-standardisation
// (mean, sigma) and 1/dt; Y == nullptr: the plain pass
// Point-force increment spread by k_ibm_spread_f: per point and component
// d = (Y*tsig + tmu)*dti is added to F; incr = 0 spreads the total F (the
// learned loop: F0 + the network's correction, the field holding no part of
// F yet), incr = 1 only d (a perturbation of an already spread F).
struct LearnedForce {
  const float *Y, *tmu, *tsig;
  double dti;
  int incr;
};
void launch_ibm_spread_f(cudaStream_t s, const Geo &g, const PartGeo &pg, IbmBuffers b, float *fu, float *fv,
                         float *fw, double dt, const LearnedForce &lf = LearnedForce{}, const int *gate = nullptr);
void launch_ibm_force_sums(cudaStream_t s, const PartGeo &pg, IbmBuffers b);
// feature row of a Lagrangian point: 32 per velocity component c at
// [FEAT_PER_COMP*c + k]; k = FEAT_F0 holds the first-pass force F0_c*dt
constexpr int FEAT_PER_COMP = 32, FEAT_F0 = 30;
struct HarvestArgs {
  float *feat;   // [cap][96] raw features
  int *pidx;     // [cap] point index
  float *targ;   // [cap][3] (F_final - F0) * dt
  int *count;    // [2]: reserved slots, slots with targets
  int cap, stride, phase;
};
void launch_ibm_features_f(cudaStream_t s, const Geo &g, const PartGeo &pg, IbmBuffers b, const float *fu,
                           const float *fv, const float *fw, double dt, const float *mu, const float *isig,
                           __nv_bfloat16 *X, const HarvestArgs &H, int first_force = 0);
void launch_ibm_harvest_targets(cudaStream_t s, IbmBuffers b, const HarvestArgs &H, double dt);
// Residual gate from the per-(particle, component) sums of (U - u~)^2 that
// the interpolation with first < 0 leaves in psum[p][c][0] and the sums of
// the first-pass slip in rsum.  Learn state ls[IBM_LS_N], see k_ibm_res_gate.
constexpr int IBM_LS_N = 16;
void launch_ibm_residual_gate(cudaStream_t s, const PartGeo &pg, IbmBuffers b, long npts, double *ls, int *gate,
                              int plain, int stage);
// y[3*npts] standard normal deviates from (seed, counter, index): a
// counter-based hash and the Box-Muller transform
void launch_normal_fill(cudaStream_t s, float *y, long n, unsigned seed, unsigned counter);

// mlp_kernels.cu (learned forcing model)
struct MlpTrainBuffers {
  float *params, *m, *v, *grad, *loss;       // FP32 masters, Adam moments, gradient, loss
  __nv_bfloat16 *w1b, *w2b;                  // BF16 copies of W1, W2
  __nv_bfloat16 *x;                           // [nb][96] batch features (test hooks)
  float *t, *y;                               // targets, outputs [nb][3] (test hooks)
  float *part;                                // per-tile gradients and losses [mlp_part_floats(nb)]
  int *err;                                   // MMA wait timed out
};
int mlp_nparam();
size_t mlp_part_floats(int nb);
int ibm_set_smem_limits(int box_cap);
int mlp_set_smem_limits();
void launch_mlp_refresh(cudaStream_t s, const float *params, __nv_bfloat16 *w1b, __nv_bfloat16 *w2b);
void launch_mlp_infer(cudaStream_t s, const __nv_bfloat16 *x, int n, const __nv_bfloat16 *w1b,
                      const __nv_bfloat16 *w2b, const float *params, float *y);
int launch_mlp_infer_tc(cudaStream_t s, const __nv_bfloat16 *x, int n, const __nv_bfloat16 *w1b,
                        const __nv_bfloat16 *w2b, const float *params, float *y, int *err);
// Inputs of the fused feature + inference kernel of the learned loop: the
// first pass's interpolation (to dudtl), point forces F0 (to fxl) and the 96
// standardised features of every point are formed in the tile's operand
// region, the same values the feature kernel writes to HBM.
struct FeatIn {
  Geo g;
  int np, nl;
  const int *nla;
  const PointRec *rec;
  const int4 *pref;
  const float4 *pcen;
  const float4 *pvh, *pvl;  // particle velocity as FP32 pairs (without rotation)
  int rotation;        // 0: U is the particle velocity; 1: read U[] (with the rotation term)
  const float *F[3];   // u, v, w (FP32 fields)
  const double *U[3];  // rigid-body velocity at the points (read with rotation on)
  const double *pf;    // particle scalar fields (centres, velocities)
  float *Fl[3];      // point forces (FP32)
  double dt, dti;
  float dtf, dtif, hx, hy, hz;  // FP32 copies of dt, 1/dt and the grid spacings
  float inv_r;
  const double *pradfp;  // polydisperse: per-sphere shell radius (the normal's scale), else null
  const float *mu, *isig;  // feature standardisation
};
int launch_mlp_features_tc(cudaStream_t s, const FeatIn &fi, const __nv_bfloat16 *w1b, const float *params,
                           float *y, int *err);
// one Adam step (adam = 1) or the gradient alone on nb rows drawn from X, T
// (n rows) by the (seed, step, row) hash (gather = 1) or rows 0..nb-1;
// outputs to y when not null.  Returns the launches.
int launch_mlp_train_step(cudaStream_t s, const MlpTrainBuffers &B, const __nv_bfloat16 *X, const float *T, int n,
                          int nb, unsigned seed, int gather, int step, float lr, int adam, float *y);
void launch_mlp_stage(cudaStream_t s, int n, const float *feat, const float *targ, const float *mu, const float *isig,
                      const float *tmu, const float *tsig, __nv_bfloat16 *X, float *T);
void launch_f2bf(cudaStream_t s, long n, const float *a, __nv_bfloat16 *b);
// standardisation of n harvested samples into norm[198] (mu, 1/sd of the
// features; mu, sd of the targets); scratch of mlp_norm_scratch() doubles
size_t mlp_norm_scratch();
int launch_mlp_norm(cudaStream_t s, int n, const float *feat, const float *targ, double *scratch, float *norm);

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
  int *err;       // [8] error flags ([4]: learned-forcing MMA wait timeout)
  double *red;    // [10*np]: volume [np], sphere-integral partials [np][3][3]
  float4 *pos4;   // [np] FP32 snapshot positions (w: master flag) for the collision filter
  int *cstart;    // [ncell+1] cell list of the snapshot positions: first item of each cell
  int *cfill;     // [ncell] scatter cursors
  int *citem;     // [np] particle indices by cell, ascending within a cell
  int *ccell;     // [np] cell of each particle
};
template <typename T>
void launch_sphere_integrals(cudaStream_t s, const Geo &g, const PartGeo &pg, PartBuffers b, const T *u, const T *v,
                             const T *w, int type, bool snapshot = false);
void launch_save_old(cudaStream_t s, const PartGeo &pg, PartBuffers b);
// snapshot: take the iteration's snapshot first (false when the sphere
// integrals' final kernel took it)
// returns the number of kernels launched
int launch_collide_update(cudaStream_t s, const PartGeo &pg, PartBuffers b, int iter, int rkiter, double dt,
                          bool snapshot = true);
void launch_ne_finalize(cudaStream_t s, const PartGeo &pg, PartBuffers b, IbmBuffers ib, int init_flags);


// ---------------------------------------------------------------------------
// plane statistics (stats_kernels.cu)
// ---------------------------------------------------------------------------
constexpr unsigned long long PH_INNER = 0x7FF0000000000000ull;  // +inf bits: above every fraction
constexpr int POST1D_NSUM = 32;  // plane sums of output.f90:88-355
struct PhaseBuffers {
  unsigned long long *G;  // [4][K*I*J] largest candidate key per cell (grids u, v, w, p)
  unsigned long long *W0; // [4][K*I*J] sum over candidates of (1 << 32) + code: count and, if one, its code
  int *W1;                // [4][K*I*J] winner code of cells with several candidates
  int *err;               // error flag (a box wider than the plane tables)
};
// shared memory of the marking pass for boxes of up to nx x ny cells
size_t phase_smem_bytes(int nx, int ny);
int phase_set_smem(size_t bytes);
void launch_phase_indicator(cudaStream_t s, const Geo &g, const PartGeo &pg, PartBuffers b, PhaseBuffers ph,
                            int itype, int nxmax, int nymax);
// Reads of the phase fields at reference indices i, j in 1..I/J (periodic
// halos wrapped by the caller) and k in 0..K+1 with the wall ghost rules of
// phase_indicator.f90:497-530.
struct PhaseView {
  const unsigned long long *G;
  const unsigned long long *W0;
  const int *W1;
  const double *pf;
  int np, I, J, K, itype;
  bool parts;  // false: np = 0, post1d's zero fields (output.f90:41-49)
  double dx, dy, dz;

  __device__ __forceinline__ long cell(int i, int j, int k) const {
    return (long)(k - 1) * I * J + (long)(j - 1) * I + (i - 1);
  }
  __device__ __forceinline__ long grid_off(int c) const { return (long)c * I * J * K; }
  // solid fraction encoded by a key
  __device__ __forceinline__ static double solid(unsigned long long key) {
    return key == 0ull ? 0. : (key == PH_INNER ? 1. : __longlong_as_double((long long)key));
  }
  // fluid fraction of grid c (0..3)
  __device__ __forceinline__ double gam(int c, int i, int j, int k) const {
    if (!parts) return 0.;
    if (k < 1) k = 1;
    if (k > K) k = K;
    return 1. - solid(G[grid_off(c) + cell(i, j, k)]);
  }
  // rigid-body velocity component c (0..2) at an interior cell whose key on
  // the velocity's grid is `key` (element `off` of that grid's arrays)
  __device__ double part_key(int c, unsigned long long key, long off, int i, int j, int k) const {
    if (key == 0ull) return 0.;
    const unsigned long long w0 = W0[off];
    const int w = (w0 >> 32) == 1 ? (int)(w0 & 0xFFFFFFFFull) : W1[off];
    if (w <= 0) return 0.;  // no winner recorded (not reached: the resolving pass repeats the keys)
    const int q = key == PH_INNER ? w - 1 : 9 * np + 1 - w;
    const int p = q / 9, nb = q - 9 * p;
    if (nb > 0) return 0.;  // the copies carry no velocity (phase_indicator.f90:68-78, 83-87)
    if (itype == 0) return pf[(long)(PF_OMX + c) * np + p];
    const double x = pf[(long)PF_X * np + p], y = pf[(long)PF_Y * np + p], z = pf[(long)PF_Z * np + p];
    const double omx = pf[(long)PF_OMX * np + p], omy = pf[(long)PF_OMY * np + p], omz = pf[(long)PF_OMZ * np + p];
    if (c == 0) return pf[(long)PF_U * np + p] + omy * ((k - 0.5) * dz - z) - omz * ((j - 0.5) * dy - y);
    if (c == 1) return pf[(long)PF_V * np + p] + omz * ((i - 0.5) * dx - x) - omx * ((k - 0.5) * dz - z);
    return pf[(long)PF_W * np + p] + omx * ((j - 0.5) * dy - y) - omy * ((i - 0.5) * dx - x);
  }
  __device__ double part_in(int c, int i, int j, int k) const {
    const long off = grid_off(itype == 1 ? c : 3) + cell(i, j, k);
    return part_key(c, G[off], off, i, j, k);
  }
  __device__ double part(int c, int i, int j, int k) const {
    if (!parts) return 0.;
    if (c < 2) {
      if (k == 0) return -part_in(c, i, j, 1);
      if (k == K + 1) return -part_in(c, i, j, K);
      return part_in(c, i, j, k);
    }
    if (k == 0 || k == K) return 0.;
    if (k == K + 1) return K - 1 >= 1 ? part_in(2, i, j, K - 1) : 0.;
    return part_in(2, i, j, k);
  }
};

void launch_phase_export(cudaStream_t s, const PhaseView &v, int f, double *out);
template <typename T>
void launch_post1d_sums(cudaStream_t s, const Geo &g, const PhaseView &ph, const T *u, const T *v, const T *w,
                        const double *p, const float *phi, const float *plo, const double *c, double kappa,
                        double *part, int slices);

}  // namespace ibmk
