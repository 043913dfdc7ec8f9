// ibm_capi.cu -- the C ABI of include/ibm_rk3.h: context set-up (derived
// parameters, solver tables), state transfer and the per-subroutine entry
// points that sequence the kernels on the context stream.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <utility>
#include <vector>

#include "kernels.cuh"

using namespace ibmk;

namespace {
thread_local std::string g_create_error;
const double PI = 3.141592653589793238462643383279502884;

bool make_plan(int n, FftPlan &pl) {
  pl.nst = 0;
  while (n % 4 == 0 && n > 1) { pl.rad[pl.nst++] = 4; n /= 4; if (pl.nst >= 16) return false; }
  while (n % 2 == 0 && n > 1) { pl.rad[pl.nst++] = 2; n /= 2; if (pl.nst >= 16) return false; }
  while (n % 3 == 0 && n > 1) { pl.rad[pl.nst++] = 3; n /= 3; if (pl.nst >= 16) return false; }
  return n == 1;
}
}  // namespace

struct ibm_ctx {
  std::string err;
  int device = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  ibm_params prm{};
  std::vector<double> thetarc, phirc;
  Geo g{};
  PartGeo pg{};
  int mode = IBM_MODE_PLAIN_FP64;
  int nq = 0;
  // derived (init.f90:74-243)
  double offset = 0, volp = 0, mominert = 0, rkab[3] = {0, 0, 0};
  // FP64 fields
  double *u = nullptr, *v = nullptr, *w = nullptr, *p = nullptr;
  double *ru = nullptr, *rv = nullptr, *rw = nullptr;
  double *fu = nullptr, *fv = nullptr, *fw = nullptr, *phi = nullptr;
  void *spec = nullptr;
  // mixed form: FP32 predictor, RHS, Poisson work arrays
  bool mixed = false;
  float *u32 = nullptr, *v32 = nullptr, *w32 = nullptr, *p32 = nullptr;  // FP32 state
  float *plo32 = nullptr;  // pnew = p32 + plo32 (double-float); p is the FP64 staging copy
  float *ru32 = nullptr, *rv32 = nullptr, *rw32 = nullptr;
  float *fu32 = nullptr, *fv32 = nullptr, *fw32 = nullptr, *phi32 = nullptr;
  float *phi32b = nullptr;  // second (defect-correction) Poisson solution
  void *spec32 = nullptr, *twM32 = nullptr, *twN32 = nullptr, *twJ32 = nullptr;
  float2 *thomas_df = nullptr;  // mixed form: double-float pivot tables of the Thomas sweep
  double *zt = nullptr;
  void *twM = nullptr, *twN = nullptr, *twJ = nullptr;
  FftPlan plx{}, ply{};
  // particles
  IbmBuffers ib{};
  PartBuffers pb{};
  // misc
  double *scratch = nullptr;   // reduction partials
  double *dout = nullptr;      // small device results
  double *href = nullptr;      // device staging buffer in the reference layout
  double *hpin = nullptr;      // pinned host results
  // learned forcing (IBM_MODE_MIXED_LEARNED)
  MlpTrainBuffers mt{};        // model (params, Adam moments, BF16 copies) + training batch buffers
  int mt_cap = 0;              // batch capacity of mt
  float *norm = nullptr;       // [198]: feature mean, 1/sigma; target mean, sigma
  float *ly = nullptr;         // [np*nl][3] network output
  double *ls = nullptr;        // learn state, see k_ibm_res_gate
  double *nscr = nullptr;      // standardisation scratch
  int *gate = nullptr;
  HarvestArgs hv{};
  int hv_passes = 0;
  bool harvesting = false, learn_on = false, model_ready = false, stats_ready = false;
  // live plain reference of the fallback gate: a loop with the network on
  // at RK stage s runs the plain passes instead and measures their
  // reduction of the first-pass slip when s has no plain loop measured
  // since the model was set, and then after 1, 2, 4, 8 ... learned loops of
  // s (the learned forcing's imprint on the flow changes the reduction over
  // the first steps), at most calib_period - 1; period 0: the first only
  int calib_period = 10;
  // CUDA graphs of whole RK stages (predictor, forcing loop, projection,
  // Newton-Euler), one per (stage, forcing kind): a stage runs directly the
  // first time with a given dt and is captured the second, then replayed
  bool use_graphs = true;
  cudaGraphExec_t gexec[3][3] = {};
  double gdt[3][3] = {};
  long long glaunch[3][3] = {};
  int gseen[3][3] = {};
  int ncal[3] = {0, 0, 0};               // plain loops measured per stage since the model was set
  long long since[3] = {0, 0, 0};        // learned loops per stage since its last plain loop
  int stage = 0;  // RK stage of the last predictor call (0..2)
  // forcing perturbation (a test of the learned form's error budget): point
  // noise of rms noise_sigma (velocity units) after the plain passes
  double noise_sigma[3] = {0, 0, 0};
  unsigned noise_seed = 0, noise_counter = 0;
  float *noise_y = nullptr;    // [np*nl*3] deviates
  float *noise_par = nullptr;  // [6]: sigma (3), mean 0 (3)
  __nv_bfloat16 *tx = nullptr; // staged training set
  float *tt = nullptr;
  int tcap = 0, train_step = 0;
  // per-kernel event probe (ibm_probe): events around every launch of the
  // selected kernel classes, on the context stream
  unsigned probe_mask = 0;
  std::vector<cudaEvent_t> probe_ev[IBM_PROBE_N];
  int probe_used[IBM_PROBE_N] = {};
  bool have_fields = false, have_particles = false, particles_ready = false;
  long long launches = 0;
  cudaEvent_t ev[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
  double phase_ms[4] = {0, 0, 0, 0};
  double wall_raw[3] = {0, 0, 0};
  double dt_last = 0;
  // plane statistics and the scalar field
  PhaseBuffers ph{};
  double *stat_part = nullptr;  // [ktot][slices][POST1D_NSUM] plane partial sums
  size_t stat_cap = 0;
  double *cfield = nullptr;     // scalar cnew, device layout; null until ibm_set_scalar
  double *cnext = nullptr;      // dcdt of the substep: cnew after the projection
  double *crk = nullptr;        // dcrkold, the scalar's stored right-hand side
  bool c_pending = false;       // cnext holds this substep's scalar
  // polydisperse sizes (host copies; device arrays in pg)
  std::vector<double> prad_h, pradfp_h, pdvl_h, pvol_h, pmi_h, prthr_h;
  std::vector<int> pnl_h, ptoff_h;
  double *psize = nullptr;      // device [6][np]: radius, shell radius, dVlagr, volume, moment of inertia, rthr
  int *pcount = nullptr;        // device [2][np]: point count, table offset
  int pred_kind = IBM_PREDICTOR_AUTO;  // mixed forms: predictor kernel (ibm_set_predictor_kernel)
  int *ferr = nullptr;          // [4] fluid kernels' flags: [0] a staged-plane copy did not complete
  int proj_solves = 1;          // mixed forms: FP32 Poisson solves per projection (2: defect correction)
  ibm_scalar_params sp{};
  double kappa = 0.;
};

namespace {

int set_err(ibm_ctx *c, int code, const std::string &msg) {
  if (c) c->err = msg;
  return code;
}
int cuda_err(ibm_ctx *c, cudaError_t e, const char *where) {
  if (e == cudaSuccess) return IBM_OK;
  return set_err(c, e == cudaErrorMemoryAllocation ? IBM_E_NOMEM : IBM_E_CUDA,
                 std::string(where) + ": " + cudaGetErrorString(e));
}
#define CK(call)                                          \
  do {                                                    \
    cudaError_t e_ = (call);                              \
    if (e_ != cudaSuccess) return cuda_err(c, e_, #call); \
  } while (0)
#define LAUNCHED(n)                                                     \
  do {                                                                  \
    c->launches += (n);                                                 \
    cudaError_t e_ = cudaGetLastError();                                \
    if (e_ != cudaSuccess) return cuda_err(c, e_, "kernel launch");     \
  } while (0)

void probe_mark(ibm_ctx *c, int id) {
  if (!(c->probe_mask & (1u << id))) return;
  std::vector<cudaEvent_t> &ev = c->probe_ev[id];
  if (c->probe_used[id] == (int)ev.size()) {
    cudaEvent_t e;
    if (cudaEventCreate(&e) != cudaSuccess) { c->probe_mask &= ~(1u << id); return; }
    ev.push_back(e);
  }
  cudaEventRecord(ev[c->probe_used[id]++], c->stream);
}
// Poisson stages -> probe ids
void poisson_probe(void *arg, int stage, int begin) {
  (void)begin;
  static const int ids[5] = {IBM_PROBE_FILLPS_FFTX, IBM_PROBE_FFTY, IBM_PROBE_THOMAS, IBM_PROBE_FFTY, IBM_PROBE_IFFTX};
  probe_mark(reinterpret_cast<ibm_ctx *>(arg), ids[stage]);
}
#define PROBED(id, ...) \
  do {                  \
    probe_mark(c, id);  \
    __VA_ARGS__;        \
    probe_mark(c, id);  \
  } while (0)

template <typename T>
int dalloc(ibm_ctx *c, T **ptr, size_t n) {
  cudaError_t e = cudaMalloc((void **)ptr, n * sizeof(T) + 256);
  if (e != cudaSuccess) return cuda_err(c, e, "cudaMalloc");
  e = cudaMemsetAsync(*ptr, 0, n * sizeof(T) + 256, c->stream);
  return cuda_err(c, e, "cudaMemset");
}

void free_mlp_batch(MlpTrainBuffers &B) {
  void *q[] = {B.x, B.t, B.y, B.part, B.err};
  for (void *p : q)
    if (p) cudaFree(p);
  B.x = nullptr; B.t = B.y = B.part = nullptr; B.err = nullptr;
}
// training batch buffers for nb rows: the per-tile gradients, the error
// flag, and a batch of features, targets and outputs for the test hooks
int alloc_mlp_batch(ibm_ctx *c, MlpTrainBuffers &B, int nb) {
  const size_t n = ((size_t)nb + 127) / 128 * 128;
  int st;
  if ((st = dalloc(c, &B.x, n * 96))) return st;
  for (float **f : {&B.t, &B.y})
    if ((st = dalloc(c, f, n * 3))) return st;
  if ((st = dalloc(c, &B.part, mlp_part_floats(nb)))) return st;
  if ((st = dalloc(c, &B.err, 1))) return st;
  CK(cudaMemsetAsync(B.err, 0, sizeof(int), c->stream));
  return IBM_OK;
}
// model buffers (params, moments, gradient, BF16 copies) of a scratch model
int alloc_mlp_model(ibm_ctx *c, MlpTrainBuffers &B) {
  int st;
  for (float **f : {&B.params, &B.m, &B.v, &B.grad})
    if ((st = dalloc(c, f, mlp_nparam()))) return st;
  if ((st = dalloc(c, &B.loss, 4))) return st;
  for (__nv_bfloat16 **f : {&B.w1b, &B.w2b})
    if ((st = dalloc(c, f, 128 * 128))) return st;
  return IBM_OK;
}
void free_mlp_model(MlpTrainBuffers &B) {
  void *q[] = {B.params, B.m, B.v, B.grad, B.loss, B.w1b, B.w2b};
  for (void *p : q)
    if (p) cudaFree(p);
}

// He-style initial weights (deterministic counter-based normal deviates)
void init_mlp_params(std::vector<float> &w, unsigned seed) {
  const int sizes[6] = {128 * 96, 128, 128 * 128, 128, 3 * 128, 3};
  const double scale[6] = {std::sqrt(2. / 96.), 0., std::sqrt(2. / 128.), 0., 0.1 * std::sqrt(1. / 128.), 0.};
  uint64_t x = 0x9E3779B97F4A7C15ULL ^ ((uint64_t)seed << 17);
  auto next = [&x]() {  // splitmix64
    uint64_t z = (x += 0x9E3779B97F4A7C15ULL);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
  };
  w.clear();
  for (int b = 0; b < 6; ++b)
    for (int q = 0; q < sizes[b]; ++q) {
      const double u1 = ((next() >> 11) + 0.5) * (1.0 / 9007199254740992.0);
      const double u2 = ((next() >> 11) + 0.5) * (1.0 / 9007199254740992.0);
      const double nrm = std::sqrt(-2. * std::log(u1)) * std::cos(2. * PI * u2);  // Box-Muller
      w.push_back((float)(scale[b] * nrm));
    }
}

// smallest double x with sqrt(x) >= r (sqrt is correctly rounded and
// monotone on host and device alike)
double sqrt_threshold(double r) {
  double t = r * r;
  if (std::sqrt(t) >= r) {
    while (t > 0 && std::sqrt(std::nextafter(t, 0.)) >= r) t = std::nextafter(t, 0.);
  } else {
    while (!(std::sqrt(t) >= r)) t = std::nextafter(t, 1e300);
  }
  return t;
}

void derived(ibm_ctx *c) {
  const ibm_params &P = c->prm;
  Geo &g = c->g;
  g.I = P.itot; g.J = P.jtot; g.K = P.ktot; g.MX = P.itot / 2 + 1;
  g.plane = (long)g.I * g.J;
  g.nfield = (long)(g.K + 2) * g.plane;
  g.lx = P.lx; g.ly = P.ly; g.lz = P.lz;
  g.dxi = P.itot / P.lx; g.dyi = P.jtot / P.ly; g.dzi = P.ktot / P.lz;
  g.dx = 1. / g.dxi; g.dy = 1. / g.dyi; g.dz = 1. / g.dzi;
  g.visc = P.visc;
  g.bc_top = P.bc_top; g.bc_bot = P.bc_bot;
  g.zper = P.bc_top == IBM_BC_PERIODIC ? 1 : 0;
  c->offset = (std::sqrt(3. * (1.5 * 1.5))) / g.dxi + 0.01 / g.dxi;
  c->volp = (4. / 3.) * PI * std::pow(P.radius, 3.);
  c->mominert = (2. / 5.) * c->volp * std::pow(P.radius, 2.);
  c->rkab[0] = 32. / 60. + 0.;
  c->rkab[1] = 25. / 60. + (-17. / 60.);
  c->rkab[2] = 45. / 60. + (-25. / 60.);
  c->nq = std::min(P.np + 2, 15);
  PartGeo &pg = c->pg;
  pg.np = P.np; pg.nl = P.nl; pg.nq = c->nq;
  pg.nb_copies = P.nb_copies == 1 ? 1 : 9;
  pg.rotation = P.particle_rotation;
  pg.radius = P.radius; pg.radfp = P.radfp; pg.offset = c->offset;
  // dVlagr of the outer shell and dVeul (coordsfp.f90:84-90)
  pg.dVlagr = ((4. / 3.) * PI * std::pow(P.radfp + 0.5 / g.dxi, 3.) -
               (4. / 3.) * PI * std::pow(P.radfp - 0.5 / g.dxi, 3.)) / (1. * P.nl);
  pg.dVeul = 1. / (g.dxi * g.dyi * g.dzi);
  pg.lx = g.lx; pg.ly = g.ly; pg.lz = g.lz;
  pg.dxi = g.dxi; pg.dyi = g.dyi; pg.dzi = g.dzi; pg.dx = g.dx; pg.dy = g.dy; pg.dz = g.dz;
  const double gacc = -9.81;  // param.f90:102-104
  pg.gacc[0] = gacc * std::cos(PI / 2.);
  pg.gacc[1] = gacc * std::cos(PI / 2.);
  pg.gacc[2] = gacc * std::sin(PI / 2.);
  for (int r = 0; r < 3; ++r) pg.rkab[r] = c->rkab[r];
  pg.volp = c->volp; pg.ratiorho = P.ratiorho; pg.mominert = c->mominert;
  // collision / lubrication constants (init.f90:137-241, param.f90:114-120)
  const double Nstretch = 8, dt_estim = 0.05, en = 0.97, et = 0.10, muc = 0.;
  const double meffn_ss = P.ratiorho * c->volp / 2., mefft_ss = 2. / 7. * meffn_ss;
  const double meffn_sw = P.ratiorho * c->volp, mefft_sw = 2. / 7. * meffn_sw;
  pg.kn_ss = (PI * PI + std::pow(std::fabs(std::log(en)), 2.)) * meffn_ss / std::pow(Nstretch * dt_estim, 2.);
  pg.kt_ss = (PI * PI + std::pow(std::fabs(std::log(et)), 2.)) * mefft_ss / std::pow(Nstretch * dt_estim, 2.);
  pg.etan_ss = -2. * (std::log(en)) * meffn_ss / (Nstretch * dt_estim);
  pg.etat_ss = -2. * (std::log(et)) * mefft_ss / (Nstretch * dt_estim);
  pg.muc_ss = muc;
  pg.kn_sw = (PI * PI + std::pow(std::fabs(std::log(en)), 2.)) * meffn_sw / std::pow(Nstretch * dt_estim, 2.);
  pg.kt_sw = (PI * PI + std::pow(std::fabs(std::log(et)), 2.)) * mefft_sw / std::pow(Nstretch * dt_estim, 2.);
  pg.etan_sw = -2. * (std::log(en)) * meffn_sw / (Nstretch * dt_estim);
  pg.etat_sw = -2. * (std::log(et)) * mefft_sw / (Nstretch * dt_estim);
  pg.muc_sw = muc;
  pg.coeff_f = 6. * PI * P.visc * P.radius;
  const double eps_ini_pp = 0.025, eps_sat_pp = 0.001, eps_ini_pw = 0.075, eps_sat_pw = 0.001;
  const double a11_ini_pp = -(1. / 4. * std::pow(eps_ini_pp, -1.)) + 9. / 40. * std::log(eps_ini_pp) +
                            3. / 112. * eps_ini_pp * std::log(eps_ini_pp);
  const double a11_sat_pp = -(1. / 4. * std::pow(eps_sat_pp, -1.)) + 9. / 40. * std::log(eps_sat_pp) +
                            3. / 112. * eps_sat_pp * std::log(eps_sat_pp);
  pg.a11a_ini_pp = a11_ini_pp - .995;
  pg.a11b_ini_pp = -a11_ini_pp + .350;
  pg.a11a_sat_pp = a11_sat_pp - .995;
  pg.a11b_sat_pp = -a11_sat_pp + .350;
  pg.a11_ini_pw = -(1. / eps_ini_pw) + 1. / 5. * std::log(eps_ini_pw) + 1. / 21. * eps_ini_pw * std::log(eps_ini_pw) - .9713;
  pg.a11_sat_pw = -(1. / eps_sat_pw) + 1. / 5. * std::log(eps_sat_pw) + 1. / 21. * eps_sat_pw * std::log(eps_sat_pw) - .9713;
  pg.I = g.I; pg.J = g.J; pg.K = g.K;
  pg.zper = g.zper;
  {  // collision cell list: cells >= 1.01 x 2.1 R wide
    const double w = 1.01 * 2.1 * P.radius;
    pg.ncx = std::max(1, (int)std::floor(P.lx / w));
    pg.ncy = std::max(1, (int)std::floor(P.ly / w));
    pg.ncz = std::max(1, (int)std::floor(P.lz / w));
    pg.cix = (float)(pg.ncx / P.lx);
    pg.ciy = (float)(pg.ncy / P.ly);
    pg.ciz = (float)(pg.ncz / P.lz);
  }
  pg.rthr = sqrt_threshold(P.radius);
  pg.visc = P.visc;
  pg.pc_an = PI * PI + std::pow(std::fabs(std::log(en)), 2.);
  pg.pc_at = PI * PI + std::pow(std::fabs(std::log(et)), 2.);
  pg.pc_b = std::pow(Nstretch * dt_estim, 2.);
  pg.pc_en = -2. * (std::log(en));
  pg.pc_et = -2. * (std::log(et));
  pg.pc_ndt = Nstretch * dt_estim;
  pg.poly = 0;
  pg.ntab = P.nl;
  pg.rmax = P.radius;
  pg.box_cap = 8192;
  if (!c->prad_h.empty()) {
    // polydisperse: per-sphere point counts, shells, Lagrangian volumes
    // (coordsfp.f90:84-90), volumes and moments of inertia (coordsfp.f90:
    // 96-102) from each radius, in the oracle's expressions
    pg.poly = 1;
    const double retrac = 0.3 / g.dxi;
    int off = 0;
    double rmax = 0.;
    c->pradfp_h.clear(); c->pdvl_h.clear(); c->pvol_h.clear(); c->pmi_h.clear(); c->prthr_h.clear();
    c->pnl_h.clear(); c->ptoff_h.clear();
    for (int p = 0; p < P.np; ++p) {
      const double r = c->prad_h[p];
      const int nlp = (int)std::lround((PI / 3.) * (12. * std::pow((r - retrac) * g.dxi, 2) + 1.));
      const double rfp = r - retrac;
      const double vol = (4. / 3.) * PI * std::pow(r, 3.);
      c->pradfp_h.push_back(rfp);
      c->pdvl_h.push_back(((4. / 3.) * PI * std::pow(rfp + 0.5 / g.dxi, 3.) -
                           (4. / 3.) * PI * std::pow(rfp - 0.5 / g.dxi, 3.)) / (1. * nlp));
      c->pvol_h.push_back(vol);
      c->pmi_h.push_back((2. / 5.) * vol * std::pow(r, 2.));
      c->prthr_h.push_back(sqrt_threshold(r));
      c->pnl_h.push_back(nlp);
      c->ptoff_h.push_back(off);
      off += nlp;
      rmax = std::max(rmax, r);
    }
    pg.ntab = off;
    pg.rmax = rmax;
    // the largest (particle, component) box of the mixed form: the shell's
    // extent plus the 3-point stencils, per axis
    const int ext = (int)std::ceil(2. * (rmax - retrac) * g.dxi + 6.);
    pg.box_cap = std::min(40960, std::max(8192, ext * ext * ext));
    // collision cell list: cells >= 1.01 x 2.1 Rmax wide
    const double w = 1.01 * 2.1 * rmax;
    pg.ncx = std::max(1, (int)std::floor(P.lx / w));
    pg.ncy = std::max(1, (int)std::floor(P.ly / w));
    pg.ncz = std::max(1, (int)std::floor(P.lz / w));
    pg.cix = (float)(pg.ncx / P.lx);
    pg.ciy = (float)(pg.ncy / P.ly);
    pg.ciz = (float)(pg.ncz / P.lz);
  }
}

// twiddles and the Thomas pivots (initsolver.f90:10-66)
int build_solver_tables(ibm_ctx *c) {
  const Geo &g = c->g;
  const int I = g.I, J = g.J, K = g.K, M = I / 2, MX = g.MX;
  std::vector<double2> twM(M), twN(M + 1), twJ(J);
  for (int t = 0; t < M; ++t) twM[t] = make_double2(std::cos(2. * PI * t / M), -std::sin(2. * PI * t / M));
  for (int t = 0; t <= M; ++t) twN[t] = make_double2(std::cos(2. * PI * t / I), -std::sin(2. * PI * t / I));
  for (int t = 0; t < J; ++t) twJ[t] = make_double2(std::cos(2. * PI * t / J), -std::sin(2. * PI * t / J));
  int st;
  if ((st = dalloc(c, (double2 **)&c->twM, M))) return st;
  if ((st = dalloc(c, (double2 **)&c->twN, M + 1))) return st;
  if ((st = dalloc(c, (double2 **)&c->twJ, J))) return st;
  CK(cudaMemcpyAsync(c->twM, twM.data(), M * sizeof(double2), cudaMemcpyHostToDevice, c->stream));
  CK(cudaMemcpyAsync(c->twN, twN.data(), (M + 1) * sizeof(double2), cudaMemcpyHostToDevice, c->stream));
  CK(cudaMemcpyAsync(c->twJ, twJ.data(), J * sizeof(double2), cudaMemcpyHostToDevice, c->stream));
  if (c->mixed) {
    std::vector<float2> fM(M), fN(M + 1), fJ(J);
    for (int t = 0; t < M; ++t) fM[t] = make_float2((float)twM[t].x, (float)twM[t].y);
    for (int t = 0; t <= M; ++t) fN[t] = make_float2((float)twN[t].x, (float)twN[t].y);
    for (int t = 0; t < J; ++t) fJ[t] = make_float2((float)twJ[t].x, (float)twJ[t].y);
    if ((st = dalloc(c, (float2 **)&c->twM32, M))) return st;
    if ((st = dalloc(c, (float2 **)&c->twN32, M + 1))) return st;
    if ((st = dalloc(c, (float2 **)&c->twJ32, J))) return st;
    CK(cudaMemcpyAsync(c->twM32, fM.data(), M * sizeof(float2), cudaMemcpyHostToDevice, c->stream));
    CK(cudaMemcpyAsync(c->twN32, fN.data(), (M + 1) * sizeof(float2), cudaMemcpyHostToDevice, c->stream));
    CK(cudaMemcpyAsync(c->twJ32, fJ.data(), J * sizeof(float2), cudaMemcpyHostToDevice, c->stream));
    CK(cudaStreamSynchronize(c->stream));
  }
  // tridiagonal matrix with Neumann rows
  std::vector<double> a(K + 1), b(K + 1), cc(K + 1);
  for (int k = 1; k <= K; ++k) { a[k] = g.dzi * g.dzi; cc[k] = g.dzi * g.dzi; b[k] = -(a[k] + cc[k]); }
  b[1] = b[1] + a[1]; b[K] = b[K] + cc[K]; a[1] = 0.; cc[K] = 0.;
  // eigenvalues in the reference's expression order
  std::vector<double> xrt(MX), yrt(J / 2 + 1);
  xrt[0] = 0.;
  for (int k = 1; k < MX; ++k) {
    const double s = std::sin(double(2 * k) * PI / (2. * I));
    xrt[k] = -4. * g.dxi * g.dxi * (s * s);
  }
  if (I % 2 == 0) xrt[M] = -4. * g.dxi * g.dxi;
  yrt[0] = 0.;
  for (int k = 1; k <= J / 2; ++k) {
    const double s = std::sin(double(2 * k) * PI / (2. * J));
    yrt[k] = -4. * g.dyi * g.dyi * (s * s);
  }
  if (J % 2 == 0) yrt[J / 2] = -4. * g.dyi * g.dyi;
  if (g.zper) {
    // periodic z: the cyclic solve forms its pivots itself; tables xrt[MX],
    // yrt[J] (both signs of ky) and its work space (2 K ncol)
    const long ncol = (long)MX * J;
    std::vector<double> tb((size_t)(MX + J), 0.);
    for (int kx = 0; kx < MX; ++kx) tb[kx] = xrt[kx];
    for (int ky = 0; ky < J; ++ky) tb[MX + ky] = yrt[ky <= J / 2 ? ky : J - ky];
    if ((st = dalloc(c, &c->zt, tb.size() + (size_t)2 * K * ncol))) return st;
    CK(cudaMemcpyAsync(c->zt, tb.data(), tb.size() * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    return IBM_OK;
  }
  const long zst = (long)(J / 2 + 1) * MX;
  std::vector<double> z((size_t)zst * K);
  for (int ky = 0; ky <= J / 2; ++ky)
    for (int kx = 0; kx < MX; ++kx) {
      const double xy = xrt[kx] + yrt[ky];
      double zz = 1. / (b[1] + xy);
      double d = cc[1] * zz;
      z[(size_t)ky * MX + kx] = zz;
      for (int k = 2; k <= K - 1; ++k) {
        const double bb = b[k] + xy;
        zz = 1. / (bb - a[k] * d);
        d = cc[k] * zz;
        z[(size_t)(k - 1) * zst + (size_t)ky * MX + kx] = zz;
      }
      const double bb = b[K] + xy;
      z[(size_t)(K - 1) * zst + (size_t)ky * MX + kx] = bb - a[K] * d;
    }
  if ((st = dalloc(c, &c->zt, z.size()))) return st;
  CK(cudaMemcpyAsync(c->zt, z.data(), z.size() * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  if (c->mixed) {
    // double-float tables of the mixed form: pivots with 1/den in the last
    // plane (0 for the zero mode, den == 0), and dzi^2 * pivot
    std::vector<float2> t(2 * z.size());
    const double a2 = g.dzi * g.dzi;
    auto split = [](double v) {
      const float h = (float)v;
      return make_float2(h, (float)(v - (double)h));
    };
    for (size_t q = 0; q < z.size(); ++q) {
      const bool last = q >= (size_t)(K - 1) * zst;
      t[q] = split(last ? (z[q] != 0. ? 1. / z[q] : 0.) : z[q]);
      t[z.size() + q] = split(a2 * z[q]);
    }
    if ((st = dalloc(c, &c->thomas_df, t.size()))) return st;
    CK(cudaMemcpyAsync(c->thomas_df, t.data(), t.size() * sizeof(float2), cudaMemcpyHostToDevice, c->stream));
  }
  CK(cudaStreamSynchronize(c->stream));
  return IBM_OK;
}

int alloc_all(ibm_ctx *c) {
  const Geo &g = c->g;
  const size_t nf = (size_t)g.nfield;
  int st;
  if ((st = dalloc(c, &c->p, nf))) return st;
  if (!c->mixed) {
    for (double **f : {&c->u, &c->v, &c->w})
      if ((st = dalloc(c, f, nf))) return st;
    for (double **f : {&c->ru, &c->rv, &c->rw, &c->fu, &c->fv, &c->fw, &c->phi})
      if ((st = dalloc(c, f, nf))) return st;
    if ((st = dalloc(c, (double2 **)&c->spec, (size_t)g.K * g.J * g.MX))) return st;
  } else {
    for (float **f : {&c->u32, &c->v32, &c->w32, &c->p32, &c->plo32, &c->ru32, &c->rv32, &c->rw32, &c->fu32, &c->fv32,
                      &c->fw32, &c->phi32, &c->phi32b})
      if ((st = dalloc(c, f, nf))) return st;
    if ((st = dalloc(c, (float2 **)&c->spec32, (size_t)g.K * g.J * g.MX))) return st;
  }
  if ((st = dalloc(c, &c->scratch, 4096))) return st;
  if ((st = dalloc(c, &c->dout, 64))) return st;
  if ((st = dalloc(c, &c->ferr, 4))) return st;
  CK(cudaMallocHost((void **)&c->hpin, 64 * sizeof(double)));
  const int np = c->pg.np, nl = c->pg.nl, nq = c->nq;
  if (np > 0) {
    const size_t npl = (size_t)np * nl;
    for (double **f : {&c->ib.xfp, &c->ib.yfp, &c->ib.zfp, &c->ib.ul, &c->ib.vl, &c->ib.wl, &c->ib.dudtl,
                       &c->ib.dvdtl, &c->ib.dwdtl, &c->ib.fxl, &c->ib.fyl, &c->ib.fzl})
      if ((st = dalloc(c, f, npl))) return st;
    if (c->mixed) {
      if ((st = dalloc(c, &c->ib.rec, npl))) return st;
      if ((st = dalloc(c, &c->ib.pref, (size_t)np))) return st;
      if ((st = dalloc(c, &c->ib.pcen, (size_t)np))) return st;
      for (float **f : {&c->ib.fxs, &c->ib.fys, &c->ib.fzs})
        if ((st = dalloc(c, f, npl))) return st;
      if ((st = dalloc(c, &c->ib.pvh, (size_t)np))) return st;
      if ((st = dalloc(c, &c->ib.pvl, (size_t)np))) return st;
      if ((st = dalloc(c, &c->ib.slip, 3 * npl))) return st;
      if ((st = dalloc(c, &c->ib.bgeo, (size_t)24 * np))) return st;
      if ((st = dalloc(c, &c->ib.rowm, (size_t)3 * IBM_BOX_ROWS * np))) return st;
      if ((st = dalloc(c, &c->ib.psum, (size_t)9 * np))) return st;
      if ((st = dalloc(c, &c->ib.rsum, (size_t)3 * np))) return st;
    } else {
      if ((st = dalloc(c, &c->ib.st, npl))) return st;
    }
    if ((st = dalloc(c, &c->ib.nla, np))) return st;
    if ((st = dalloc(c, &c->pb.pf, (size_t)PF_N * np))) return st;
    if ((st = dalloc(c, &c->pb.cf, (size_t)CF_N * np * nq))) return st;
    if ((st = dalloc(c, &c->pb.qmax, np))) return st;
    if ((st = dalloc(c, &c->pb.firstc, (size_t)np * nq))) return st;
    if ((st = dalloc(c, &c->pb.ofirstc, (size_t)np * nq))) return st;
    if ((st = dalloc(c, &c->pb.nb, (size_t)np * 9))) return st;
    if ((st = dalloc(c, &c->pb.mslv, np))) return st;
    if ((st = dalloc(c, &c->pb.rkp, (size_t)RK_N * np))) return st;
    const int nt = c->pg.ntab;  // entries of each point table (nl, or the sum of the point counts)
    if ((st = dalloc(c, &c->pb.sincos, (size_t)4 * nt))) return st;
    if ((st = dalloc(c, &c->pb.err, 8))) return st;
    if ((st = dalloc(c, &c->pb.red, (size_t)10 * np))) return st;
    if ((st = dalloc(c, &c->pb.pos4, (size_t)np))) return st;
    const size_t ncell = (size_t)c->pg.ncx * c->pg.ncy * c->pg.ncz;
    if ((st = dalloc(c, &c->pb.cstart, ncell + 1))) return st;
    if ((st = dalloc(c, &c->pb.cfill, ncell))) return st;
    if ((st = dalloc(c, &c->pb.citem, (size_t)np))) return st;
    if ((st = dalloc(c, &c->pb.ccell, (size_t)np))) return st;
    if ((st = dalloc(c, &c->ib.diag, 8))) return st;
    c->ib.pf = c->pb.pf;
    c->ib.err = c->pb.err;
    std::vector<double> sc((size_t)4 * nt);
    for (int l = 0; l < nt; ++l) {
      sc[l] = std::sin(c->thetarc[l]);
      sc[nt + l] = std::cos(c->thetarc[l]);
      sc[2 * nt + l] = std::sin(c->phirc[l]);
      sc[3 * nt + l] = std::cos(c->phirc[l]);
    }
    CK(cudaMemcpyAsync(c->pb.sincos, sc.data(), sc.size() * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    if (c->pg.poly) {  // per-sphere sizes on the device
      if ((st = dalloc(c, &c->psize, (size_t)6 * np))) return st;
      if ((st = dalloc(c, &c->pcount, (size_t)2 * np))) return st;
      std::vector<double> ps((size_t)6 * np);
      std::vector<int> pc((size_t)2 * np);
      for (int p = 0; p < np; ++p) {
        ps[p] = c->prad_h[p]; ps[np + p] = c->pradfp_h[p]; ps[2 * np + p] = c->pdvl_h[p];
        ps[3 * np + p] = c->pvol_h[p]; ps[4 * np + p] = c->pmi_h[p]; ps[5 * np + p] = c->prthr_h[p];
        pc[p] = c->pnl_h[p]; pc[np + p] = c->ptoff_h[p];
      }
      CK(cudaMemcpyAsync(c->psize, ps.data(), ps.size() * sizeof(double), cudaMemcpyHostToDevice, c->stream));
      CK(cudaMemcpyAsync(c->pcount, pc.data(), pc.size() * sizeof(int), cudaMemcpyHostToDevice, c->stream));
      CK(cudaStreamSynchronize(c->stream));
      c->pg.prad = c->psize; c->pg.pradfp = c->psize + np; c->pg.pdvl = c->psize + 2 * np;
      c->pg.pvol = c->psize + 3 * np; c->pg.pmi = c->psize + 4 * np; c->pg.prthr = c->psize + 5 * np;
      c->pg.pnl = c->pcount; c->pg.ptoff = c->pcount + np;
    }
  }
  if (c->mode == IBM_MODE_MIXED_LEARNED) {
    const int npar = mlp_nparam();
    for (float **f : {&c->mt.params, &c->mt.m, &c->mt.v, &c->mt.grad})
      if ((st = dalloc(c, f, npar))) return st;
    if ((st = dalloc(c, &c->mt.loss, 4))) return st;
    for (__nv_bfloat16 **f : {&c->mt.w1b, &c->mt.w2b})
      if ((st = dalloc(c, f, 128 * 128))) return st;
    if ((st = dalloc(c, &c->norm, 198))) return st;
    if ((st = dalloc(c, &c->ls, IBM_LS_N))) return st;
    if ((st = dalloc(c, &c->gate, 4))) return st;
    double ls0[IBM_LS_N] = {};
    ls0[3] = 1.5;
    CK(cudaMemcpyAsync(c->ls, ls0, sizeof(ls0), cudaMemcpyHostToDevice, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    if (np > 0) {
      const size_t npl = (size_t)np * nl;
      if ((st = dalloc(c, &c->ly, npl * 3))) return st;
    }
  }
  return IBM_OK;
}

int check_flags(ibm_ctx *c) {
  if (c->ferr) {
    int f = 0;
    CK(cudaMemcpyAsync(&f, c->ferr, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    if (f) return set_err(c, IBM_E_NOT_CONVERGED, "a staged-plane copy of the predictor did not complete in time");
  }
  if (c->pg.np == 0) return IBM_OK;
  int h[5];
  CK(cudaMemcpyAsync(h, c->pb.err, 5 * sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  if (h[4]) return set_err(c, IBM_E_NOT_CONVERGED, "a tensor-core MMA wait of the learned forcing timed out");
  if (h[2]) return set_err(c, IBM_E_INVALID, "a Lagrangian point left the grid (non-finite or beyond the walls)");
  if (h[3]) return set_err(c, IBM_E_INVALID, "sphere integration box wider than 128 cells");
  if (h[1]) return set_err(c, IBM_E_CONTACT_OVERFLOW, "a particle exceeded nqmax contacts (param.f90:100)");
  if (h[0]) return set_err(c, IBM_E_CONTACT_OVERFLOW, "more than 64 interaction candidates for one particle");
  return IBM_OK;
}

int predict(ibm_ctx *c, int rkiter, double dt) {
  const Geo &g = c->g;
  c->stage = rkiter - 1;
  if (c->mixed) launch_wallshear<float>(c->stream, g, c->v32, c->scratch, c->dout + 8 + (rkiter - 1));
  else launch_wallshear<double>(c->stream, g, c->v, c->scratch, c->dout + 8 + (rkiter - 1));
  LAUNCHED(2);
  double f1, f2 = 0, f3 = 0;
  if (rkiter == 1) f1 = dt * (32. / 60.);
  else if (rkiter == 2) { f1 = dt * (8. / 60.); f2 = dt * (25. / 60.); f3 = dt * (17. / 60.); }
  else { f1 = dt * (20. / 60.); f2 = dt * (45. / 60.); f3 = dt * (25. / 60.); }
  // buoyancy 0.5*beta*9.81*(c + c(k+1)) of momzbuoy (mom.f90:251) once a scalar is set
  const double *cb = c->cfield;
  const double bcoef = 0.5 * c->sp.beta * 9.81;
  if (c->mixed)
    PROBED(IBM_PROBE_PREDICT, launch_predict<float, float>(c->stream, g, rkiter, c->u32, c->v32, c->w32, c->p32, c->ru32, c->rv32, c->rw32,
                                 c->fu32, c->fv32, c->fw32, f1, f2, f3, cb, bcoef, c->pred_kind, c->ferr));
  else
    PROBED(IBM_PROBE_PREDICT, launch_predict<double, double>(c->stream, g, rkiter, c->u, c->v, c->w, c->p, c->ru, c->rv, c->rw, c->fu, c->fv,
                                   c->fw, f1, f2, f3, cb, bcoef));
  LAUNCHED(1);
  if (c->cfield) {  // scalad and dcdt of rk1..rk3
    if (c->mixed)
      launch_scalar_stage<float>(c->stream, g, rkiter, c->u32, c->v32, c->w32, c->cfield, c->crk, c->cnext, c->kappa,
                                 f1, f2, f3);
    else
      launch_scalar_stage<double>(c->stream, g, rkiter, c->u, c->v, c->w, c->cfield, c->crk, c->cnext, c->kappa, f1,
                                  f2, f3);
    LAUNCHED(1);
    c->c_pending = true;
  }
  return IBM_OK;
}

int forcing_learned(ibm_ctx *c, double dt, int nl_iter) {
  // one sweep plus one inference: the first pass's interpolation, the point
  // forces F0 and the network features formed in the inference kernel's
  // operand tiles, the network's correction (one kernel); one spreading of
  // F0 + correction; then the plain passes 2..Nl only where the no-slip
  // residual exceeds fallback_ratio x the plain method's
  const Geo &g = c->g;
  const long npts = (long)c->pg.np * c->pg.nl;
  PROBED(IBM_PROBE_STENCIL, launch_ibm_stencil_f(c->stream, g, c->pg, c->ib));
  LAUNCHED(3);  // reference floors, point records, boxes
  FeatIn fi;
  fi.g = g;
  fi.np = c->pg.np;
  fi.nl = c->pg.nl;
  fi.nla = c->ib.nla;
  fi.rec = c->ib.rec;
  fi.pref = c->ib.pref;
  fi.pcen = c->ib.pcen;
  fi.pvh = c->ib.pvh;
  fi.pvl = c->ib.pvl;
  fi.rotation = c->pg.rotation;
  fi.F[0] = c->fu32; fi.F[1] = c->fv32; fi.F[2] = c->fw32;
  fi.U[0] = c->ib.ul; fi.U[1] = c->ib.vl; fi.U[2] = c->ib.wl;
  fi.pf = c->pb.pf;
  fi.Fl[0] = c->ib.fxs; fi.Fl[1] = c->ib.fys; fi.Fl[2] = c->ib.fzs;
  fi.dt = dt;
  fi.dti = 1. / dt;
  fi.dtf = (float)dt;
  fi.dtif = (float)(1. / dt);
  fi.hx = (float)g.dx;
  fi.hy = (float)g.dy;
  fi.hz = (float)g.dz;
  fi.inv_r = (float)(1. / c->pg.radfp);
  fi.pradfp = c->pg.poly ? c->pg.pradfp : nullptr;
  fi.mu = c->norm;
  fi.isig = c->norm + 96;
  PROBED(IBM_PROBE_MLP, c->launches += launch_mlp_features_tc(c->stream, fi, c->mt.w1b, c->mt.params, c->ly,
                                                              c->pb.err + 4));
  // the top plane of fw carries only the spread force (read above by the
  // w features, zeroed before the spreading)
  launch_zero_plane<float>(c->stream, g, c->fw32, g.K + 1);
  LAUNCHED(1);
  // F = F0 + the network's correction per point, its force and torque sums,
  // one spreading
  const LearnedForce lf{c->ly, c->norm + 192, c->norm + 195, 1. / dt, 0};
  PROBED(IBM_PROBE_SPREAD, launch_ibm_spread_f(c->stream, g, c->pg, c->ib, c->fu32, c->fv32, c->fw32, dt, lf));
  launch_ibm_force_sums(c->stream, c->pg, c->ib);
  PROBED(IBM_PROBE_INTERP, c->launches += -1 + launch_ibm_interp_force_f(c->stream, g, c->pg, c->ib, c->fu32,
                                                                         c->fv32, c->fw32, dt, -1));
  launch_ibm_residual_gate(c->stream, c->pg, c->ib, npts, c->ls, c->gate, 0, c->stage);
  LAUNCHED(4);  // spreading, force sums, residual interpolation, gate
  // (their own probe class: they return at once unless the gate fell back)
  for (int it = 1; it < nl_iter; ++it) {
    PROBED(IBM_PROBE_GATED, c->launches += -1 + launch_ibm_interp_force_f(c->stream, g, c->pg, c->ib, c->fu32,
                                                                          c->fv32, c->fw32, dt, 0, c->gate));
    PROBED(IBM_PROBE_GATED,
           launch_ibm_spread_f(c->stream, g, c->pg, c->ib, c->fu32, c->fv32, c->fw32, dt, LearnedForce{}, c->gate));
    LAUNCHED(2);
  }
  return IBM_OK;
}

int perturb_forces(ibm_ctx *c, double dt) {
  // point noise of rms noise_sigma (velocity units) added to F*dt of every
  // point and spread as an increment; the force sums follow
  const long npts = (long)c->pg.np * c->pg.nl;
  int st;
  if (!c->noise_y) {
    if ((st = dalloc(c, &c->noise_y, (size_t)3 * npts))) return st;
    if ((st = dalloc(c, &c->noise_par, 6))) return st;
  }
  const float par[6] = {(float)c->noise_sigma[0], (float)c->noise_sigma[1], (float)c->noise_sigma[2], 0.f, 0.f, 0.f};
  CK(cudaMemcpyAsync(c->noise_par, par, sizeof(par), cudaMemcpyHostToDevice, c->stream));
  launch_normal_fill(c->stream, c->noise_y, 3 * npts, c->noise_seed, c->noise_counter++);
  const LearnedForce lf{c->noise_y, c->noise_par + 3, c->noise_par, 1. / dt, 1};
  launch_ibm_spread_f(c->stream, c->g, c->pg, c->ib, c->fu32, c->fv32, c->fw32, dt, lf);
  launch_ibm_force_sums(c->stream, c->pg, c->ib);
  LAUNCHED(3);
  CK(cudaStreamSynchronize(c->stream));  // par is a host array
  return IBM_OK;
}

// The forcing loop's kind at the current RK stage, decided on the host (and
// the calibration schedule's counters advanced): FORCING_PLAIN, the plain
// passes (and a calibration measurement, FORCING_CALIB), or FORCING_LEARNED.
enum { FORCING_PLAIN = 0, FORCING_CALIB = 1, FORCING_LEARNED = 2 };
int forcing_kind(ibm_ctx *c, int nl_iter) {
  if (!c->mixed || !c->learn_on || c->harvesting || nl_iter < 2 || c->pg.np == 0) return FORCING_PLAIN;
  const int s = c->stage;
  const long long gap = std::min<long long>(1LL << std::min(std::max(c->ncal[s] - 1, 0), 30), c->calib_period - 1);
  if (c->ncal[s] == 0 || (c->calib_period > 0 && c->since[s] >= gap)) {
    ++c->ncal[s];
    c->since[s] = 0;
    return FORCING_CALIB;
  }
  ++c->since[s];
  return FORCING_LEARNED;
}

// the launches of one forcing loop of the given kind (no host decision)
int forcing_run(ibm_ctx *c, double dt, int nl_iter, int kind) {
  if (c->pg.np == 0 || nl_iter <= 0) return IBM_OK;
  const Geo &g = c->g;
  if (c->mixed) {
    if (kind == FORCING_LEARNED) return forcing_learned(c, dt, nl_iter);
    const bool measure = c->harvesting || kind == FORCING_CALIB;
    const long npts = (long)c->pg.np * c->pg.nl;
    const int npass = c->harvesting ? std::max(nl_iter, c->hv_passes) : nl_iter;
    PROBED(IBM_PROBE_STENCIL, launch_ibm_stencil_f(c->stream, g, c->pg, c->ib));
    LAUNCHED(3);  // reference floors, point records, boxes
    for (int it = 0; it < npass; ++it) {
      PROBED(IBM_PROBE_INTERP, c->launches += -1 + launch_ibm_interp_force_f(c->stream, g, c->pg, c->ib, c->fu32,
                                                                             c->fv32, c->fw32, dt, it == 0 ? 1 : 0));
      LAUNCHED(1);
      if (c->harvesting && it == 0) {
        // features from the field the first pass interpolated (before any
        // spreading), as the learned loop computes them
        c->hv.phase = (c->hv.phase + 1) % c->hv.stride;
        PROBED(IBM_PROBE_FEATURES, launch_ibm_features_f(c->stream, g, c->pg, c->ib, c->fu32, c->fv32, c->fw32, dt,
                                                         nullptr, nullptr, nullptr, c->hv, 0));
        LAUNCHED(1);
      }
      if (it == 0) {
        launch_zero_plane<float>(c->stream, g, c->fw32, g.K + 1);
        LAUNCHED(1);
      }
      PROBED(IBM_PROBE_SPREAD, launch_ibm_spread_f(c->stream, g, c->pg, c->ib, c->fu32, c->fv32, c->fw32, dt));
      LAUNCHED(1);
      if (measure && c->ls && it == nl_iter - 1) {
        // the plain method's residual at its own number of passes, against
        // its first-pass slip: the reference of the learned loop's gate
        PROBED(IBM_PROBE_INTERP, c->launches += -1 + launch_ibm_interp_force_f(c->stream, g, c->pg, c->ib, c->fu32, c->fv32, c->fw32, dt, -1));
        launch_ibm_residual_gate(c->stream, c->pg, c->ib, npts, c->ls, c->gate, 1, c->stage);
        LAUNCHED(2);
      }
    }
    if (c->harvesting) {
      launch_ibm_harvest_targets(c->stream, c->ib, c->hv, dt);
      LAUNCHED(2);
    } else if (c->noise_sigma[0] > 0 || c->noise_sigma[1] > 0 || c->noise_sigma[2] > 0) {
      return perturb_forces(c, dt);
    }
    return IBM_OK;
  }
  PROBED(IBM_PROBE_STENCIL, launch_ibm_stencil<double>(c->stream, g, c->pg, c->ib));
  LAUNCHED(1);
  for (int it = 0; it < nl_iter; ++it) {
    PROBED(IBM_PROBE_INTERP,
           launch_ibm_interp_force<double>(c->stream, g, c->pg, c->ib, c->fu, c->fv, c->fw, dt, it == 0 ? 1 : 0));
    LAUNCHED(1);
    if (it == 0 && !g.zper) {  // dwdtf(:,:,k1) carries only S(F) (interp_spread.f90:267-269)
      launch_zero_plane<double>(c->stream, g, c->fw, g.K + 1);
      LAUNCHED(1);
    }
    PROBED(IBM_PROBE_SPREAD, launch_ibm_spread<double>(c->stream, g, c->pg, c->ib, c->fu, c->fv, c->fw, dt, it == 0));
    LAUNCHED(1);
  }
  return IBM_OK;
}

int forcing(ibm_ctx *c, double dt, int nl_iter) { return forcing_run(c, dt, nl_iter, forcing_kind(c, nl_iter)); }

int project_fluid(ibm_ctx *c, int rkiter, double dt) {
  const Geo &g = c->g;
  const double dti = 1. / (c->rkab[rkiter - 1] * dt);
  int nl = 0;
  const double factor = c->rkab[rkiter - 1] * dt;
  if (c->mixed && c->proj_solves == 1) {
    // one FP32 solve of fillps(u*) and one correction into the FP32 state
    // and the double-float pnew
    launch_poisson<float, float>(c->stream, g, c->plx, c->ply, c->fu32, c->fv32, c->fw32, c->spec32, c->phi32,
                                 c->twM32, c->twN32, c->twJ32, c->zt, dti * g.dxi, dti * g.dyi, dti * g.dzi, &nl,
                                 false, c->thomas_df, PoissonHook{poisson_probe, c});
    LAUNCHED(nl);
    PROBED(IBM_PROBE_CORREC, launch_correc_mixed(c->stream, g, c->fu32, c->fv32, c->fw32, c->phi32, c->u32, c->v32,
                                                 c->w32, c->p32, c->plo32, factor * g.dxi, factor * g.dyi,
                                                 factor * g.dzi));
    LAUNCHED(1);
    return IBM_OK;
  }
  if (c->mixed && poisson_fused_residual_ok(g)) {
    // FP32 solve of fillps(u*) -> phi1; one defect correction: the divergence
    // residual of u* - f grad(phi1), evaluated in double-float, drives a
    // second solve -> phi2; then one correction u = u* - f grad(phi1 + phi2),
    // pnew += phi1 + phi2
    launch_poisson<float, float>(c->stream, g, c->plx, c->ply, c->fu32, c->fv32, c->fw32, c->spec32, c->phi32,
                                 c->twM32, c->twN32, c->twJ32, c->zt, dti * g.dxi, dti * g.dyi, dti * g.dzi, &nl,
                                 false, c->thomas_df, PoissonHook{poisson_probe, c});
    LAUNCHED(nl);
    nl = 0;
    PoissonResid rs;
    rs.phi1 = c->phi32;
    rs.fi = (float)(factor * g.dxi); rs.fj = (float)(factor * g.dyi); rs.fk = (float)(factor * g.dzi);
    launch_poisson<float, float>(c->stream, g, c->plx, c->ply, c->fu32, c->fv32, c->fw32, c->spec32, c->phi32b,
                                 c->twM32, c->twN32, c->twJ32, c->zt, dti * g.dxi, dti * g.dyi, dti * g.dzi, &nl,
                                 true, c->thomas_df, PoissonHook{poisson_probe, c}, rs);
    LAUNCHED(nl);
    PROBED(IBM_PROBE_CORREC, launch_correc_mixed2(c->stream, g, c->fu32, c->fv32, c->fw32, c->phi32, c->phi32b,
                                                  c->u32, c->v32, c->w32, c->p32, c->plo32, factor * g.dxi,
                                                  factor * g.dyi, factor * g.dzi));
    LAUNCHED(1);
    return IBM_OK;
  }
  if (c->mixed) {
    // FP32 solve of fillps(u*), FP64 Thomas; correction into the FP64 state
    launch_poisson<float, float>(c->stream, g, c->plx, c->ply, c->fu32, c->fv32, c->fw32, c->spec32, c->phi32,
                                 c->twM32, c->twN32, c->twJ32, c->zt, dti * g.dxi, dti * g.dyi, dti * g.dzi, &nl,
                                 false, c->thomas_df, PoissonHook{poisson_probe, c});
    LAUNCHED(nl);
    PROBED(IBM_PROBE_CORREC, launch_correc_mixed(c->stream, g, c->fu32, c->fv32, c->fw32, c->phi32, c->u32, c->v32, c->w32, c->p32, c->plo32,
                        factor * g.dxi, factor * g.dyi, factor * g.dzi));
    LAUNCHED(1);
    // one defect correction: the divergence residual of the corrected state,
    // evaluated in FP64, drives a second solve; its pressure is accumulated
    // into the FP64 pnew
    nl = 0;
    launch_poisson<float, float>(c->stream, g, c->plx, c->ply, c->u32, c->v32, c->w32, c->spec32, c->phi32, c->twM32,
                                 c->twN32, c->twJ32, c->zt, dti * g.dxi, dti * g.dyi, dti * g.dzi, &nl, true,
                                 c->thomas_df, PoissonHook{poisson_probe, c});
    LAUNCHED(nl);
    PROBED(IBM_PROBE_CORREC, launch_correc_mixed(c->stream, g, c->u32, c->v32, c->w32, c->phi32, c->u32, c->v32, c->w32, c->p32, c->plo32,
                        factor * g.dxi, factor * g.dyi, factor * g.dzi));
    LAUNCHED(1);
    return IBM_OK;
  }
  launch_poisson<double, double>(c->stream, g, c->plx, c->ply, c->fu, c->fv, c->fw, c->spec, c->phi, c->twM, c->twN,
                                 c->twJ, c->zt, dti * g.dxi, dti * g.dyi, dti * g.dzi, &nl, false, nullptr, PoissonHook{poisson_probe, c});
  LAUNCHED(nl);
  PROBED(IBM_PROBE_CORREC, launch_correc<double, double, double>(c->stream, g, c->fu, c->fv, c->fw, c->phi, c->u, c->v, c->w, c->p, nullptr,
                                        factor * g.dxi, factor * g.dyi, factor * g.dzi));
  LAUNCHED(1);
  return IBM_OK;
}

int project(ibm_ctx *c, int rkiter, double dt) {
  int st;
  if ((st = project_fluid(c, rkiter, dt))) return st;
  if (c->c_pending) {  // cnew = dcdt; boundscal (main.f90:374-376)
    std::swap(c->cfield, c->cnext);
    launch_boundscal(c->stream, c->g, c->cfield, c->sp.bc_c_top_type == IBM_BC_C_DIRICHLET, c->sp.bc_c_top_val,
                     c->sp.bc_c_bot_type == IBM_BC_C_DIRICHLET, c->sp.bc_c_bot_val);
    LAUNCHED(1);
    c->c_pending = false;
  }
  return IBM_OK;
}

int newton_euler(ibm_ctx *c, int rkiter, double dt) {
  if (c->pg.np == 0) return IBM_OK;
  launch_save_old(c->stream, c->pg, c->pb);
  LAUNCHED(1);
  probe_mark(c, IBM_PROBE_SPHERE);
  // the sphere integrals' final kernel also takes the first collision
  // iteration's snapshot
  if (c->mixed) launch_sphere_integrals<float>(c->stream, c->g, c->pg, c->pb, c->u32, c->v32, c->w32, 23, true);
  else launch_sphere_integrals<double>(c->stream, c->g, c->pg, c->pb, c->u, c->v, c->w, 23, true);
  probe_mark(c, IBM_PROBE_SPHERE);
  LAUNCHED(1);
  for (int iter = 0; iter <= 1; ++iter) {
    c->launches += launch_collide_update(c->stream, c->pg, c->pb, iter, rkiter, dt, iter > 0);
    LAUNCHED(0);
  }
  launch_ne_finalize(c->stream, c->pg, c->pb, c->ib, 0);
  LAUNCHED(1);
  return IBM_OK;
}

void drop_graphs(ibm_ctx *c) {
  for (auto &r : c->gexec)
    for (auto &e : r)
      if (e) {
        cudaGraphExecDestroy(e);
        e = nullptr;
      }
  for (auto &r : c->gseen)
    for (int &n : r) n = 0;
}

int stage_direct(ibm_ctx *c, int rkiter, double dt, int kind) {
  int st;
  if ((st = predict(c, rkiter, dt))) return st;
  if ((st = forcing_run(c, dt, 3, kind))) return st;
  if ((st = project(c, rkiter, dt))) return st;
  return newton_euler(c, rkiter, dt);
}

// a stage's launches depend on host state only through what the graph keys
// hold (stage, forcing kind, dt) and the settings whose setters drop the
// graphs; these conditions change the launch sequence from step to step
// (scalar transport swaps its buffers every stage) or add host work
bool graphs_apply(const ibm_ctx *c) {
  return c->use_graphs && c->probe_mask == 0 && !c->harvesting && !c->cfield &&
         !(c->noise_sigma[0] > 0 || c->noise_sigma[1] > 0 || c->noise_sigma[2] > 0);
}

// Captures the stage into its graph (which it replaces) and, with launch,
// launches it; without, the stage's host state is left as it was.  A failed
// capture turns the graphs off and (with launch) runs the stage directly.
int stage_capture(ibm_ctx *c, int rkiter, double dt, int kind, bool launch) {
  const int s = rkiter - 1;
  cudaGraphExec_t &ex = c->gexec[s][kind];
  if (ex) cudaGraphExecDestroy(ex);
  ex = nullptr;
  const long long l0 = c->launches;
  const int stage0 = c->stage;
  if (cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeRelaxed) != cudaSuccess) {
    cudaGetLastError();
    c->use_graphs = false;
    return launch ? stage_direct(c, rkiter, dt, kind) : IBM_OK;
  }
  const int st = stage_direct(c, rkiter, dt, kind);
  const long long ncap = c->launches - l0;  // the stage's launches, counted again at every replay
  cudaGraph_t gr = nullptr;
  const cudaError_t e1 = cudaStreamEndCapture(c->stream, &gr);
  cudaGraphExec_t ne = nullptr;
  const cudaError_t e2 = (st == IBM_OK && e1 == cudaSuccess) ? cudaGraphInstantiate(&ne, gr, 0) : cudaErrorUnknown;
  if (gr) cudaGraphDestroy(gr);
  c->launches = l0;
  if (st != IBM_OK || e1 != cudaSuccess || e2 != cudaSuccess) {
    // the stage was only recorded
    cudaGetLastError();
    if (ne) cudaGraphExecDestroy(ne);
    c->use_graphs = false;
    c->stage = stage0;
    if (st != IBM_OK) return st;
    return launch ? stage_direct(c, rkiter, dt, kind) : IBM_OK;
  }
  ex = ne;
  c->gdt[s][kind] = dt;
  c->gseen[s][kind] = 2;
  c->glaunch[s][kind] = ncap;
  if (!launch) {
    c->stage = stage0;
    return IBM_OK;
  }
  CK(cudaGraphLaunch(ex, c->stream));
  c->launches += c->glaunch[s][kind];
  return IBM_OK;
}

int stage_graph(ibm_ctx *c, int rkiter, double dt, int kind) {
  const int s = rkiter - 1;
  cudaGraphExec_t &ex = c->gexec[s][kind];
  if (c->gdt[s][kind] != dt) {
    if (ex) cudaGraphExecDestroy(ex);
    ex = nullptr;
    c->gdt[s][kind] = dt;
    c->gseen[s][kind] = 0;
  }
  if (ex) {
    CK(cudaGraphLaunch(ex, c->stream));
    c->launches += c->glaunch[s][kind];
    c->stage = s;
    return IBM_OK;
  }
  // first time: directly (lazily initialised launch settings are set up
  // outside a capture); second time: captured, then launched
  if (c->gseen[s][kind]++ == 0) return stage_direct(c, rkiter, dt, kind);
  return stage_capture(c, rkiter, dt, kind, true);
}

int ready(ibm_ctx *c) {
  if (!c) return IBM_E_INVALID;
  if (!c->have_fields) return set_err(c, IBM_E_STATE, "ibm_set_fields has not been called");
  if (c->pg.np > 0 && !c->particles_ready)
    return set_err(c, IBM_E_STATE, "particles not initialised (ibm_set_particles + ibm_init_particles)");
  return IBM_OK;
}

}  // namespace

extern "C" {

int ibm_abi_version(void) { return IBM_ABI_VERSION; }

const char *ibm_last_error(const ibm_ctx *c) { return c ? c->err.c_str() : g_create_error.c_str(); }

ibm_ctx *ibm_create(const ibm_params *P) {
  g_create_error.clear();
  if (!P) { g_create_error = "null params"; return nullptr; }
  if (P->itot < 4 || P->jtot < 4 || P->ktot < 3 || P->itot % 2) {
    g_create_error = "grid must have even itot >= 4, jtot >= 4, ktot >= 3";
    return nullptr;
  }
  if (!(P->lx > 0 && P->ly > 0 && P->lz > 0 && P->visc > 0)) { g_create_error = "lx, ly, lz, visc must be > 0"; return nullptr; }
  if (P->np < 0 || (P->np > 0 && (P->nl <= 0 || !P->thetarc || !P->phirc || !(P->radius > 0)))) {
    g_create_error = "np > 0 requires nl > 0, thetarc, phirc and radius > 0";
    return nullptr;
  }
  if (P->mode != IBM_MODE_PLAIN_FP64 && P->mode != IBM_MODE_MIXED && P->mode != IBM_MODE_MIXED_LEARNED) {
    g_create_error = "mode must be IBM_MODE_PLAIN_FP64, IBM_MODE_MIXED or IBM_MODE_MIXED_LEARNED";
    return nullptr;
  }
  if ((P->bc_top == IBM_BC_PERIODIC) != (P->bc_bot == IBM_BC_PERIODIC) ||
      (P->bc_top == IBM_BC_PERIODIC && (P->mode != IBM_MODE_PLAIN_FP64 || P->np > 1))) {
    g_create_error = "periodic z needs bc_top = bc_bot = IBM_BC_PERIODIC, the plain FP64 form and at most one particle";
    return nullptr;
  }
  long ntab = P->nl;  // entries of the point tables
  if (P->np > 0 && P->radii) {
    // polydisperse: every sphere's point count from its radius; nl is their
    // maximum, the tables hold them one after the other
    const double dxi = P->itot / P->lx, retrac = 0.3 / dxi;
    int nlmax = 0;
    ntab = 0;
    for (int p = 0; p < P->np; ++p) {
      const double r = P->radii[p];
      const int nlp = r > retrac ? (int)std::lround((PI / 3.) * (12. * std::pow((r - retrac) * dxi, 2) + 1.)) : 0;
      if (!(r > retrac) || nlp < 1) {
        g_create_error = "radii must exceed 0.3 dx (the force-point shell r - 0.3 dx)";
        return nullptr;
      }
      nlmax = std::max(nlmax, nlp);
      ntab += nlp;
    }
    if (nlmax != P->nl) {
      g_create_error = "nl = " + std::to_string(P->nl) + " must equal the largest sphere's point count " +
                       std::to_string(nlmax);
      return nullptr;
    }
    if (!P->thetarc || !P->phirc) { g_create_error = "polydisperse spheres need thetarc and phirc"; return nullptr; }
  } else if (P->np > 0) {
    // nl must equal nint(pi/3*(12*((radius-retrac)*dxi)^2+1)) (main.f90:118-132)
    const double dxi = P->itot / P->lx, retrac = 0.3 / dxi;
    const int nl = (int)std::lround((PI / 3.) * (12. * std::pow((P->radius - retrac) * dxi, 2) + 1.));
    if (nl != P->nl) {
      g_create_error = "nl = " + std::to_string(P->nl) + " does not match the derived value " + std::to_string(nl) +
                       " (main.f90:118-132)";
      return nullptr;
    }
  }
  if ((long long)P->np * P->nl >= (1LL << 31) || (long long)(P->itot + 2) * (P->jtot + 2) * (P->ktot + 2) >= (1LL << 40)) {
    g_create_error = "problem too large (np*nl must be < 2^31)";
    return nullptr;
  }
  ibm_ctx *c = new ibm_ctx();
  c->prm = *P;
  if (P->np > 0) {
    c->thetarc.assign(P->thetarc, P->thetarc + ntab);
    c->phirc.assign(P->phirc, P->phirc + ntab);
  }
  if (P->np > 0 && P->radii) c->prad_h.assign(P->radii, P->radii + P->np);
  c->prm.thetarc = nullptr;
  c->prm.phirc = nullptr;
  c->prm.radii = nullptr;
  c->mode = P->mode;
  c->mixed = P->mode != IBM_MODE_PLAIN_FP64;
  derived(c);
  if (!make_plan(c->g.I / 2, c->plx) || !make_plan(c->g.J, c->ply)) {
    g_create_error = "itot/2 and jtot must be products of 2 and 3";
    delete c;
    return nullptr;
  }
  cudaGetDevice(&c->device);
  if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) {
    g_create_error = "cudaStreamCreate failed (no CUDA device?)";
    delete c;
    return nullptr;
  }
  c->own_stream = true;
  for (auto &e : c->ev) cudaEventCreate(&e);
  int st = alloc_all(c);
  if (st == IBM_OK) st = build_solver_tables(c);
  if (st == IBM_OK && (poisson_set_smem_limits<double>() != 0 || poisson_set_smem_limits<float>() != 0 ||
                       mlp_set_smem_limits() != 0 || ibm_set_smem_limits(c->pg.box_cap) != 0))
    st = set_err(c, IBM_E_CUDA, "cudaFuncSetAttribute failed");
  if (st == IBM_OK) st = cuda_err(c, cudaStreamSynchronize(c->stream), "create");
  if (st != IBM_OK) {
    g_create_error = c->err;
    ibm_destroy(c);
    return nullptr;
  }
  return c;
}

int ibm_destroy(ibm_ctx *c) {
  if (!c) return IBM_OK;
  if (c->stream) cudaStreamSynchronize(c->stream);
  drop_graphs(c);
  void *ptrs[] = {c->u, c->v, c->w, c->p, c->ru, c->rv, c->rw, c->fu, c->fv, c->fw, c->phi, c->spec, c->zt, c->twM,
                  c->twN, c->twJ, c->scratch, c->dout, c->href, c->ib.xfp, c->ib.yfp, c->ib.zfp, c->ib.ul, c->ib.vl,
                  c->ib.wl, c->ib.dudtl, c->ib.dvdtl, c->ib.dwdtl, c->ib.fxl, c->ib.fyl, c->ib.fzl, c->ib.st,
                  c->ib.nla, c->ib.diag, c->pb.pf, c->pb.cf, c->pb.qmax, c->pb.firstc, c->pb.ofirstc, c->pb.nb,
                  c->pb.mslv, c->pb.rkp, c->pb.sincos, c->pb.err, c->pb.red, c->pb.pos4, c->pb.cstart, c->pb.cfill, c->pb.citem, c->pb.ccell, c->ru32, c->rv32, c->rw32, c->fu32,
                  c->fv32, c->fw32, c->phi32, c->phi32b, c->spec32, c->twM32, c->twN32, c->twJ32, c->ib.rec, c->ib.pref, c->ib.pcen, c->ib.fxs, c->ib.fys, c->ib.fzs, c->ib.pvh, c->ib.pvl, c->ib.slip, c->ib.bgeo, c->ib.rowm, c->u32, c->v32,
                  c->w32, c->p32, c->plo32, c->thomas_df, c->ib.psum, c->ib.rsum, c->noise_y, c->noise_par, c->ph.G, c->ph.W0, c->ph.W1, c->stat_part,
                  c->cfield, c->cnext, c->crk, c->ferr, c->psize, c->pcount};
  for (void *q : ptrs)
    if (q) cudaFree(q);
  void *lptrs[] = {c->mt.params, c->mt.m, c->mt.v, c->mt.grad, c->mt.loss, c->mt.w1b, c->mt.w2b,
                   c->norm, c->ls, c->gate, c->ly, c->hv.feat, c->hv.pidx, c->hv.targ,
                   c->hv.count, c->tx, c->tt, c->nscr};
  for (void *q : lptrs)
    if (q) cudaFree(q);
  free_mlp_batch(c->mt);
  for (auto &v : c->probe_ev)
    for (cudaEvent_t e : v) cudaEventDestroy(e);
  if (c->hpin) cudaFreeHost(c->hpin);
  for (auto &e : c->ev)
    if (e) cudaEventDestroy(e);
  if (c->own_stream && c->stream) cudaStreamDestroy(c->stream);
  delete c;
  return IBM_OK;
}

int ibm_sizes(const ibm_ctx *c, int *nqmax, int *nl, int *ncells) {
  if (!c) return IBM_E_INVALID;
  if (nqmax) *nqmax = c->nq;
  if (nl) *nl = c->pg.nl;
  if (ncells) *ncells = (c->g.I + 2) * (c->g.J + 2) * (c->g.K + 2);
  return IBM_OK;
}

int ibm_set_stream(ibm_ctx *c, void *stream) {
  if (!c) return IBM_E_INVALID;
  CK(cudaStreamSynchronize(c->stream));
  if (c->own_stream) cudaStreamDestroy(c->stream);
  c->own_stream = stream == nullptr;
  if (stream) c->stream = (cudaStream_t)stream;
  else CK(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
  return IBM_OK;
}

static int ensure_href(ibm_ctx *c) {
  if (c->href) return IBM_OK;
  const size_t n = (size_t)(c->g.I + 2) * (c->g.J + 2) * (c->g.K + 2);
  CK(cudaMalloc((void **)&c->href, n * sizeof(double)));
  return IBM_OK;
}

// A device-side alias of a caller's array: page-locked host memory is mapped
// into the device's address space (unified addressing), so the layout
// conversion kernels can read and write it directly over the host link, with
// no staging copy; device and managed memory are used as they are.  nullptr
// for pageable memory, which takes the staging buffer and cudaMemcpy.
static const void *device_view(const void *h) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, h) != cudaSuccess) return nullptr;
  if (a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged) return a.devicePointer ? a.devicePointer : h;
  if (a.type == cudaMemoryTypeHost && a.devicePointer) return a.devicePointer;
  return nullptr;
}

static int upload_field(ibm_ctx *c, const double *h, double *d) {
  const size_t n = (size_t)(c->g.I + 2) * (c->g.J + 2) * (c->g.K + 2);
  if (!h) {
    CK(cudaMemsetAsync(d, 0, (size_t)c->g.nfield * sizeof(double), c->stream));
    return IBM_OK;
  }
  if (const double *dv = static_cast<const double *>(device_view(h))) {
    launch_ref_to_dev<double>(c->stream, c->g, dv, d);
    LAUNCHED(1);
    return IBM_OK;
  }
  CK(cudaMemcpyAsync(c->href, h, n * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  launch_ref_to_dev<double>(c->stream, c->g, c->href, d);
  LAUNCHED(1);
  return IBM_OK;
}
// the reference-layout copy of one device field into h (synchronised by the
// caller)
extern "C++" {
template <typename T>
static int download_any(ibm_ctx *c, const T *d, double *h) {
  if (!h) return IBM_OK;
  const size_t n = (size_t)(c->g.I + 2) * (c->g.J + 2) * (c->g.K + 2);
  if (double *dv = static_cast<double *>(const_cast<void *>(device_view(h)))) {
    launch_dev_to_ref<T>(c->stream, c->g, d, dv);
    LAUNCHED(1);
    return IBM_OK;
  }
  launch_dev_to_ref<T>(c->stream, c->g, d, c->href);
  LAUNCHED(1);
  CK(cudaMemcpyAsync(h, c->href, n * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));  // href is reused by the next field
  return IBM_OK;
}
}  // extern "C++"
static int download_field(ibm_ctx *c, const double *d, double *h) { return download_any<double>(c, d, h); }
static int download_field32(ibm_ctx *c, const float *d, double *h) { return download_any<float>(c, d, h); }

int ibm_set_fields(ibm_ctx *c, const double *u, const double *v, const double *w, const double *p, const double *durk,
                   const double *dvrk, const double *dwrk) {
  if (!c) return IBM_E_INVALID;
  if (!u || !v || !w || !p) return set_err(c, IBM_E_INVALID, "u, v, w and p are required");
  int st;
  if ((st = ensure_href(c))) return st;
  const double *hs[7] = {u, v, w, p, durk, dvrk, dwrk};
  double *ds[7] = {c->u, c->v, c->w, c->p, c->ru, c->rv, c->rw};
  if (!c->mixed) {
    for (int f = 0; f < 7; ++f)
      if ((st = upload_field(c, hs[f], ds[f]))) return st;
  } else {
    if ((st = upload_field(c, p, c->p))) return st;
    launch_d_to_df(c->stream, c->g.nfield, c->p, c->p32, c->plo32);
    LAUNCHED(1);
  }
  if (c->mixed) {
    float *d32[6] = {c->u32, c->v32, c->w32, c->ru32, c->rv32, c->rw32};
    const double *h32[6] = {u, v, w, durk, dvrk, dwrk};
    for (int f = 0; f < 6; ++f) {
      if (h32[f]) {
        const size_t n = (size_t)(c->g.I + 2) * (c->g.J + 2) * (c->g.K + 2);
        const double *src = static_cast<const double *>(device_view(h32[f]));
        if (!src) {
          CK(cudaMemcpyAsync(c->href, h32[f], n * sizeof(double), cudaMemcpyHostToDevice, c->stream));
          src = c->href;
        }
        launch_ref_to_dev<float>(c->stream, c->g, src, d32[f]);
        LAUNCHED(1);
      } else {
        CK(cudaMemsetAsync(d32[f], 0, (size_t)c->g.nfield * sizeof(float), c->stream));
      }
    }
    for (float *f : {c->fu32, c->fv32, c->fw32}) CK(cudaMemsetAsync(f, 0, (size_t)c->g.nfield * sizeof(float), c->stream));
  } else {
    // dudtf starts from zero (module storage), in particular its k1 plane
    for (double *f : {c->fu, c->fv, c->fw}) CK(cudaMemsetAsync(f, 0, (size_t)c->g.nfield * sizeof(double), c->stream));
  }
  CK(cudaStreamSynchronize(c->stream));
  c->have_fields = true;
  return IBM_OK;
}

int ibm_get_fields(ibm_ctx *c, double *u, double *v, double *w, double *p, double *durk, double *dvrk, double *dwrk) {
  if (!c) return IBM_E_INVALID;
  int st;
  if ((st = ensure_href(c))) return st;
  const double *ds[7] = {c->u, c->v, c->w, c->p, c->ru, c->rv, c->rw};
  double *hs[7] = {u, v, w, p, durk, dvrk, dwrk};
  if (!c->mixed) {
    for (int f = 0; f < 7; ++f)
      if ((st = download_field(c, ds[f], hs[f]))) return st;
    CK(cudaStreamSynchronize(c->stream));
    return IBM_OK;
  }
  if (p) {
    launch_df_to_d(c->stream, c->g.nfield, c->p32, c->plo32, c->p);
    LAUNCHED(1);
  }
  if ((st = download_field(c, c->p, p))) return st;
  const float *d32[6] = {c->u32, c->v32, c->w32, c->ru32, c->rv32, c->rw32};
  double *h32[6] = {u, v, w, durk, dvrk, dwrk};
  for (int f = 0; f < 6; ++f)
    if ((st = download_field32(c, d32[f], h32[f]))) return st;
  CK(cudaStreamSynchronize(c->stream));
  return IBM_OK;
}

int ibm_get_intermediate(ibm_ctx *c, double *du, double *dv, double *dw) {
  if (!c) return IBM_E_INVALID;
  int st;
  if ((st = ensure_href(c))) return st;
  if (c->mixed) {
    if ((st = download_field32(c, c->fu32, du))) return st;
    if ((st = download_field32(c, c->fv32, dv))) return st;
    return download_field32(c, c->fw32, dw);
  }
  if ((st = download_field(c, c->fu, du))) return st;
  if ((st = download_field(c, c->fv, dv))) return st;
  return download_field(c, c->fw, dw);
}

static const double *const *pf_host_ptrs(const ibm_particles *s, const double **arr) {
  const double *a[31] = {s->x, s->y, s->z, s->theta, s->phi, s->u, s->v, s->w, s->omx, s->omy, s->omz, s->omtheta,
                         s->intu, s->intv, s->intw, s->intomx, s->intomy, s->intomz, s->colfx, s->colfy, s->colfz,
                         s->coltx, s->colty, s->coltz, s->fxltot, s->fyltot, s->fzltot, s->torqxltot, s->torqyltot,
                         s->torqzltot, s->torqtheta};
  for (int f = 0; f < 31; ++f) arr[f] = a[f];
  return arr;
}

int ibm_set_particles(ibm_ctx *c, const ibm_particles *s) {
  if (!c || !s) return IBM_E_INVALID;
  const int np = c->pg.np, nq = c->nq, nl = c->pg.nl;
  if (np == 0) { c->have_particles = true; c->particles_ready = true; return IBM_OK; }
  const double *arr[31];
  pf_host_ptrs(s, arr);
  std::vector<double> pf((size_t)PF_N * np, 0.);
  for (int f = 0; f < 31; ++f) {
    if (!arr[f]) return set_err(c, IBM_E_INVALID, "particle array missing");
    std::memcpy(&pf[(size_t)f * np], arr[f], np * sizeof(double));
  }
  CK(cudaMemcpyAsync(c->pb.pf, pf.data(), pf.size() * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  std::vector<double> cf((size_t)CF_N * np * nq, 0.);
  const double *carr[10] = {s->cdx, s->cdy, s->cdz, s->cdxt, s->cdyt, s->cdzt, s->cdut, s->cdvt, s->cdwt, s->cpsi};
  for (int f = 0; f < 10; ++f)
    if (carr[f]) std::memcpy(&cf[(size_t)f * np * nq], carr[f], (size_t)np * nq * sizeof(double));
  CK(cudaMemcpyAsync(c->pb.cf, cf.data(), cf.size() * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  if (!s->qmax || !s->firstc || !s->mslv)
    return set_err(c, IBM_E_INVALID, "qmax, firstc and mslv are required");
  for (int p = 0; p < np; ++p) {
    if (s->qmax[p] < 0 || s->qmax[p] > nq) return set_err(c, IBM_E_INVALID, "qmax outside 0..nqmax");
    if (s->mslv[p] != p + 1) return set_err(c, IBM_E_INVALID, "mslv must be the particle id p+1 on one rank");
    if (s->nb)
      for (int n = 0; n < 9; ++n)
        if (s->nb[(size_t)p * 9 + n] != 0 && s->nb[(size_t)p * 9 + n] != 1) return set_err(c, IBM_E_INVALID, "nb flags must be 0/1");
  }
  // without nb: the flags of the self-neighbour copies from the centres, as a
  // warm start sets them (loadd.f90:362-397, one rank: bounds 0..lx, 0..ly)
  std::vector<int> nbh((size_t)np * 9, 0);
  if (s->nb) {
    std::memcpy(nbh.data(), s->nb, nbh.size() * sizeof(int));
  } else {
    const double ro = c->prm.radius + c->offset, rightb = c->prm.lx, backb = c->prm.ly, leftb = 0., frontb = 0.;
    for (int p = 0; p < np; ++p) {
      const double x = s->x[p], y = s->y[p];
      int *f = &nbh[(size_t)p * 9];
      double dist;
      if (x > (rightb - ro)) f[1] = 1;
      dist = std::sqrt((rightb - x) * (rightb - x) + (frontb - y) * (frontb - y));
      if (std::fabs(dist) < ro) f[2] = 1;
      if (y < (frontb + ro)) f[3] = 1;
      dist = std::sqrt((leftb - x) * (leftb - x) + (frontb - y) * (frontb - y));
      if (std::fabs(dist) < ro) f[4] = 1;
      if (x < (leftb + ro)) f[5] = 1;
      dist = std::sqrt((leftb - x) * (leftb - x) + (backb - y) * (backb - y));
      if (std::fabs(dist) < ro) f[6] = 1;
      if (y > (backb - ro)) f[7] = 1;
      dist = std::sqrt((rightb - x) * (rightb - x) + (backb - y) * (backb - y));
      if (std::fabs(dist) < ro) f[8] = 1;
    }
  }
  CK(cudaMemcpyAsync(c->pb.qmax, s->qmax, np * sizeof(int), cudaMemcpyHostToDevice, c->stream));
  CK(cudaMemcpyAsync(c->pb.firstc, s->firstc, (size_t)np * nq * sizeof(int), cudaMemcpyHostToDevice, c->stream));
  CK(cudaMemcpyAsync(c->pb.ofirstc, s->firstc, (size_t)np * nq * sizeof(int), cudaMemcpyHostToDevice, c->stream));
  CK(cudaMemcpyAsync(c->pb.nb, nbh.data(), (size_t)np * 9 * sizeof(int), cudaMemcpyHostToDevice, c->stream));
  CK(cudaMemcpyAsync(c->pb.mslv, s->mslv, np * sizeof(int), cudaMemcpyHostToDevice, c->stream));
  std::vector<double> rk((size_t)RK_N * np, 0.);  // rkp may be NULL (zero)
  if (s->rkp)
    for (int p = 0; p < np; ++p)
      for (int t = 0; t < RK_N; ++t) rk[(size_t)p * RK_N + t] = s->rkp[(size_t)p * RK_N + t];
  CK(cudaMemcpyAsync(c->pb.rkp, rk.data(), rk.size() * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  CK(cudaMemsetAsync(c->pb.err, 0, 8 * sizeof(int), c->stream));
  if (s->xfp && s->yfp && s->zfp && s->ul && s->vl && s->wl) {
    const size_t npl = (size_t)np * nl;
    const double *la[6] = {s->xfp, s->yfp, s->zfp, s->ul, s->vl, s->wl};
    double *ld[6] = {c->ib.xfp, c->ib.yfp, c->ib.zfp, c->ib.ul, c->ib.vl, c->ib.wl};
    for (int f = 0; f < 6; ++f) CK(cudaMemcpyAsync(ld[f], la[f], npl * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    if (s->fxl && s->fyl && s->fzl) {
      CK(cudaMemcpyAsync(c->ib.fxl, s->fxl, npl * sizeof(double), cudaMemcpyHostToDevice, c->stream));
      CK(cudaMemcpyAsync(c->ib.fyl, s->fyl, npl * sizeof(double), cudaMemcpyHostToDevice, c->stream));
      CK(cudaMemcpyAsync(c->ib.fzl, s->fzl, npl * sizeof(double), cudaMemcpyHostToDevice, c->stream));
      if (c->mixed) {  // the mixed forms carry the point forces in FP32
        launch_d2f(c->stream, (long)npl, c->ib.fxl, c->ib.fxs);
        launch_d2f(c->stream, (long)npl, c->ib.fyl, c->ib.fys);
        launch_d2f(c->stream, (long)npl, c->ib.fzl, c->ib.fzs);
        LAUNCHED(3);
      }
    }
    std::vector<int> nla(np, nl);
    if (c->pg.poly) nla = c->pnl_h;  // each sphere's own point count (the arrays' capacity is nl)
    CK(cudaMemcpyAsync(c->ib.nla, nla.data(), np * sizeof(int), cudaMemcpyHostToDevice, c->stream));
    c->particles_ready = true;
  } else {
    launch_ne_finalize(c->stream, c->pg, c->pb, c->ib, 2);
    LAUNCHED(1);
    c->particles_ready = true;
  }
  CK(cudaStreamSynchronize(c->stream));
  c->have_particles = true;
  return IBM_OK;
}

int ibm_get_particles(ibm_ctx *c, ibm_particles *s) {
  if (!c || !s) return IBM_E_INVALID;
  const int np = c->pg.np, nq = c->nq, nl = c->pg.nl;
  if (np == 0) return IBM_OK;
  std::vector<double> pf((size_t)PF_N * np);
  CK(cudaMemcpyAsync(pf.data(), c->pb.pf, pf.size() * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  std::vector<double> cf((size_t)CF_N * np * nq);
  CK(cudaMemcpyAsync(cf.data(), c->pb.cf, cf.size() * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  std::vector<double> rk((size_t)RK_N * np);
  CK(cudaMemcpyAsync(rk.data(), c->pb.rkp, rk.size() * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  if (s->qmax) CK(cudaMemcpyAsync(s->qmax, c->pb.qmax, np * sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  if (s->firstc) CK(cudaMemcpyAsync(s->firstc, c->pb.firstc, (size_t)np * nq * sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  if (s->nb) CK(cudaMemcpyAsync(s->nb, c->pb.nb, (size_t)np * 9 * sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  if (s->mslv) CK(cudaMemcpyAsync(s->mslv, c->pb.mslv, np * sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  const size_t npl = (size_t)np * nl;
  if (c->mixed && (s->fxl || s->fyl || s->fzl)) {  // the mixed forms' FP32 point forces, widened
    launch_f2d(c->stream, (long)npl, c->ib.fxs, c->ib.fxl);
    launch_f2d(c->stream, (long)npl, c->ib.fys, c->ib.fyl);
    launch_f2d(c->stream, (long)npl, c->ib.fzs, c->ib.fzl);
    LAUNCHED(3);
  }
  const double *ls[9] = {c->ib.xfp, c->ib.yfp, c->ib.zfp, c->ib.ul, c->ib.vl, c->ib.wl, c->ib.fxl, c->ib.fyl, c->ib.fzl};
  double *lh[9] = {s->xfp, s->yfp, s->zfp, s->ul, s->vl, s->wl, s->fxl, s->fyl, s->fzl};
  for (int f = 0; f < 9; ++f)
    if (lh[f]) CK(cudaMemcpyAsync(lh[f], ls[f], npl * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  double *arr[31] = {s->x, s->y, s->z, s->theta, s->phi, s->u, s->v, s->w, s->omx, s->omy, s->omz, s->omtheta,
                     s->intu, s->intv, s->intw, s->intomx, s->intomy, s->intomz, s->colfx, s->colfy, s->colfz,
                     s->coltx, s->colty, s->coltz, s->fxltot, s->fyltot, s->fzltot, s->torqxltot, s->torqyltot,
                     s->torqzltot, s->torqtheta};
  for (int f = 0; f < 31; ++f)
    if (arr[f]) std::memcpy(arr[f], &pf[(size_t)f * np], np * sizeof(double));
  double *carr[10] = {s->cdx, s->cdy, s->cdz, s->cdxt, s->cdyt, s->cdzt, s->cdut, s->cdvt, s->cdwt, s->cpsi};
  for (int f = 0; f < 10; ++f)
    if (carr[f]) std::memcpy(carr[f], &cf[(size_t)f * np * nq], (size_t)np * nq * sizeof(double));
  if (s->rkp) std::memcpy(s->rkp, rk.data(), rk.size() * sizeof(double));
  return check_flags(c);
}

int ibm_init_particles(ibm_ctx *c, double *vol_calc) {
  if (!c) return IBM_E_INVALID;
  drop_graphs(c);  // the captured stages may depend on what this changes
  if (!c->have_fields) return set_err(c, IBM_E_STATE, "ibm_set_fields has not been called");
  if (c->pg.np == 0) { c->particles_ready = true; if (vol_calc) *vol_calc = 0.; return IBM_OK; }
  if (!c->have_particles) return set_err(c, IBM_E_STATE, "ibm_set_particles has not been called");
  launch_ne_finalize(c->stream, c->pg, c->pb, c->ib, 1);
  LAUNCHED(1);
  if (c->mixed) launch_sphere_integrals<float>(c->stream, c->g, c->pg, c->pb, c->u32, c->v32, c->w32, 1);
  else launch_sphere_integrals<double>(c->stream, c->g, c->pg, c->pb, c->u, c->v, c->w, 1);
  LAUNCHED(1);
  double vol = 0.;
  CK(cudaMemcpyAsync(&vol, c->pb.red, sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  if (c->mixed) launch_sphere_integrals<float>(c->stream, c->g, c->pg, c->pb, c->u32, c->v32, c->w32, 23);
  else launch_sphere_integrals<double>(c->stream, c->g, c->pg, c->pb, c->u, c->v, c->w, 23);
  LAUNCHED(1);
  CK(cudaStreamSynchronize(c->stream));
  if (vol_calc) *vol_calc = vol;
  c->particles_ready = true;
  return IBM_OK;
}

int ibm_rk_predict(ibm_ctx *c, int rkiter, double dt) {
  int st;
  if ((st = ready(c))) return st;
  if (rkiter < 1 || rkiter > 3) return set_err(c, IBM_E_INVALID, "rkiter must be 1..3");
  c->dt_last = dt;
  return predict(c, rkiter, dt);
}
int ibm_forcing_loop(ibm_ctx *c, double dt, int nl_iter) {
  int st;
  if ((st = ready(c))) return st;
  return forcing(c, dt, nl_iter);
}
int ibm_project(ibm_ctx *c, int rkiter, double dt) {
  int st;
  if ((st = ready(c))) return st;
  if (rkiter < 1 || rkiter > 3) return set_err(c, IBM_E_INVALID, "rkiter must be 1..3");
  return project(c, rkiter, dt);
}
int ibm_newton_euler(ibm_ctx *c, int rkiter, double dt) {
  int st;
  if ((st = ready(c))) return st;
  if (rkiter < 1 || rkiter > 3) return set_err(c, IBM_E_INVALID, "rkiter must be 1..3");
  return newton_euler(c, rkiter, dt);
}

static int step_once(ibm_ctx *c, double dt, bool timed) {
  int st;
  float ms[4] = {0, 0, 0, 0};
  for (int rkiter = 1; rkiter <= 3; ++rkiter) {
    if (!timed) {
      c->stage = rkiter - 1;
      const int kind = forcing_kind(c, 3);
      if ((st = graphs_apply(c) ? stage_graph(c, rkiter, dt, kind) : stage_direct(c, rkiter, dt, kind))) return st;
      continue;
    }
    // timed: directly, with events between the phases
    CK(cudaEventRecord(c->ev[0], c->stream));
    if ((st = predict(c, rkiter, dt))) return st;
    CK(cudaEventRecord(c->ev[1], c->stream));
    if ((st = forcing(c, dt, 3))) return st;
    CK(cudaEventRecord(c->ev[2], c->stream));
    if ((st = project(c, rkiter, dt))) return st;
    CK(cudaEventRecord(c->ev[3], c->stream));
    if ((st = newton_euler(c, rkiter, dt))) return st;
    CK(cudaEventRecord(c->ev[4], c->stream));
    CK(cudaEventSynchronize(c->ev[4]));
    for (int q = 0; q < 4; ++q) {
      float t = 0;
      cudaEventElapsedTime(&t, c->ev[q], c->ev[q + 1]);
      ms[q] += t;
    }
  }
  if (timed)
    for (int q = 0; q < 4; ++q) c->phase_ms[q] = ms[q];
  c->dt_last = dt;
  return IBM_OK;
}

int ibm_rk3_step(ibm_ctx *c, double dt) {
  int st;
  if ((st = ready(c))) return st;
  return step_once(c, dt, false);
}

int ibm_run(ibm_ctx *c, double dt, int nsteps) {
  int st;
  if ((st = ready(c))) return st;
  for (int s = 0; s < nsteps; ++s)
    if ((st = step_once(c, dt, false))) return st;
  return IBM_OK;
}

int ibm_timed_step(ibm_ctx *c, double dt) {
  int st;
  if ((st = ready(c))) return st;
  return step_once(c, dt, true);
}

int ibm_chkdiv(ibm_ctx *c, double *divtot, double *divmax, int ijk[3]) {
  if (!c) return IBM_E_INVALID;
  if (c->mixed) launch_chkdiv<float>(c->stream, c->g, c->u32, c->v32, c->w32, c->scratch, c->dout);
  else launch_chkdiv<double>(c->stream, c->g, c->u, c->v, c->w, c->scratch, c->dout);
  LAUNCHED(2);
  CK(cudaMemcpyAsync(c->hpin, c->dout, 3 * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  const double tot = c->hpin[0], mx = c->hpin[1];
  const long long loc = (long long)c->hpin[2];
  if (divtot) *divtot = tot;
  if (divmax) *divmax = mx;
  if (ijk) {
    if (loc >= 0) {
      ijk[0] = (int)(loc % c->g.I) + 1;
      ijk[1] = (int)((loc / c->g.I) % c->g.J) + 1;
      ijk[2] = (int)(loc / c->g.plane) + 1;
    } else {
      ijk[0] = ijk[1] = ijk[2] = 0;
    }
  }
  if (tot > 1.e-3) return set_err(c, IBM_E_DIVERGENCE, "total divergence > 1e-3 (chkdiv.f90:51-58)");
  return IBM_OK;
}

int ibm_chkdt(ibm_ctx *c, double *dtmax) {
  if (!c || !dtmax) return IBM_E_INVALID;
  if (c->mixed) launch_chkdt<float>(c->stream, c->g, c->u32, c->v32, c->w32, c->scratch, c->dout);
  else launch_chkdt<double>(c->stream, c->g, c->u, c->v, c->w, c->scratch, c->dout);
  LAUNCHED(2);
  CK(cudaMemcpyAsync(c->hpin, c->dout, sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  *dtmax = c->hpin[0];
  return IBM_OK;
}

int ibm_run_adaptive(ibm_ctx *c, int nsteps, int ioutchk, double *dt, double *time) {
  // main.f90:268-441: RK3 steps; every ioutchk steps chkdiv (abort above a
  // total divergence of 1e-3) and chkdt, then dt = 0.75*dtmax
  if (!c || !dt || nsteps < 0 || ioutchk < 1 || !(*dt > 0)) return IBM_E_INVALID;
  int st;
  if ((st = ready(c))) return st;
  for (int istep = 1; istep <= nsteps; ++istep) {
    if ((st = step_once(c, *dt, false))) return st;
    if (time) *time += *dt;
    if (istep % ioutchk == 0) {
      double tot, mx, dtmax;
      int ijk[3];
      if ((st = ibm_chkdiv(c, &tot, &mx, ijk))) return st;
      if ((st = ibm_chkdt(c, &dtmax))) return st;
      *dt = 0.75 * dtmax;
    }
  }
  return check_flags(c);
}


// ---------------------------------------------------------------------------
// scalar field and plane statistics (post1d, output.f90:13-917)
// ---------------------------------------------------------------------------
int ibm_set_scalar(ibm_ctx *c, const ibm_scalar_params *sp, const double *cf, const double *dcrk) {
  if (!c) return IBM_E_INVALID;
  drop_graphs(c);  // the captured stages may depend on what this changes
  if (!sp || !(sp->pran > 0.)) return set_err(c, IBM_E_INVALID, "scalar parameters need pran > 0");
  if (c->g.zper) return set_err(c, IBM_E_STATE, "no scalar transport with periodic z");
  if ((sp->bc_c_top_type != IBM_BC_C_DIRICHLET && sp->bc_c_top_type != IBM_BC_C_NEUMANN) ||
      (sp->bc_c_bot_type != IBM_BC_C_DIRICHLET && sp->bc_c_bot_type != IBM_BC_C_NEUMANN))
    return set_err(c, IBM_E_INVALID, "scalar boundary types must be IBM_BC_C_DIRICHLET or IBM_BC_C_NEUMANN");
  int st;
  if ((st = ensure_href(c))) return st;
  for (double **f : {&c->cfield, &c->cnext, &c->crk})
    if (!*f) CK(cudaMalloc((void **)f, (size_t)c->g.nfield * sizeof(double)));
  c->sp = *sp;
  c->kappa = c->prm.visc / sp->pran;  // init.f90:94
  c->c_pending = false;
  if ((st = upload_field(c, cf, c->cfield))) return st;
  if ((st = upload_field(c, dcrk, c->crk))) return st;
  // boundscal as the driver applies it after loading (main.f90:198)
  launch_boundscal(c->stream, c->g, c->cfield, sp->bc_c_top_type == IBM_BC_C_DIRICHLET, sp->bc_c_top_val,
                   sp->bc_c_bot_type == IBM_BC_C_DIRICHLET, sp->bc_c_bot_val);
  LAUNCHED(1);
  // cells of cnext that the stage kernel does not write (ghost planes) start
  // from cnew
  CK(cudaMemcpyAsync(c->cnext, c->cfield, (size_t)c->g.nfield * sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  return IBM_OK;
}

int ibm_get_scalar(ibm_ctx *c, double *cf, double *dcrk) {
  if (!c) return IBM_E_INVALID;
  const size_t n = (size_t)(c->g.I + 2) * (c->g.J + 2) * (c->g.K + 2);
  if (!c->cfield) {
    if (cf) std::memset(cf, 0, n * sizeof(double));
    if (dcrk) std::memset(dcrk, 0, n * sizeof(double));
    return IBM_OK;
  }
  int st;
  if ((st = ensure_href(c))) return st;
  if ((st = download_field(c, c->cfield, cf))) return st;
  return download_field(c, c->crk, dcrk);
}

static int run_phase_indicator(ibm_ctx *c, int itype) {
  if (c->pg.np >= (1 << 20)) return set_err(c, IBM_E_INVALID, "phase indicator: more than 2^20 particles");
  // widest box (phase_indicator.f90:255-273): 2 r/dx + 4 cells plus rounding
  const int nx = (int)std::ceil(2. * c->prm.radius * c->g.dxi) + 6, ny = (int)std::ceil(2. * c->prm.radius * c->g.dyi) + 6;
  const size_t smem = phase_smem_bytes(nx, ny);
  if (smem > 227 * 1024) return set_err(c, IBM_E_INVALID, "phase indicator: sphere too wide for the plane tables");
  if (!c->ph.G) {
    const size_t nc = (size_t)c->g.I * c->g.J * c->g.K;
    CK(cudaMalloc((void **)&c->ph.G, 4 * nc * sizeof(unsigned long long)));
    CK(cudaMalloc((void **)&c->ph.W0, 4 * nc * sizeof(unsigned long long)));
    CK(cudaMalloc((void **)&c->ph.W1, 4 * nc * sizeof(int)));
    if (smem > 48 * 1024 && phase_set_smem(smem)) return set_err(c, IBM_E_CUDA, "phase indicator: shared memory");
  }
  c->ph.err = c->pb.err + 5;
  PROBED(IBM_PROBE_PHASE, launch_phase_indicator(c->stream, c->g, c->pg, c->pb, c->ph, itype, nx, ny));
  LAUNCHED(c->pg.np > 0 ? 2 : 0);
  return IBM_OK;
}

static int phase_check(ibm_ctx *c) {
  if (c->pg.np == 0) return IBM_OK;
  int h = 0;
  CK(cudaMemcpyAsync(&h, c->pb.err + 5, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  if (h) return set_err(c, IBM_E_INVALID, "phase indicator: a box exceeded its tables");
  return IBM_OK;
}

static PhaseView phase_view(const ibm_ctx *c, int itype, bool parts) {
  PhaseView v;
  v.G = c->ph.G;
  v.W0 = c->ph.W0;
  v.W1 = c->ph.W1;
  v.pf = c->pb.pf;
  v.np = c->pg.np;
  v.I = c->g.I; v.J = c->g.J; v.K = c->g.K;
  v.itype = itype;
  v.parts = parts;
  v.dx = 1. / c->g.dxi; v.dy = 1. / c->g.dyi; v.dz = 1. / c->g.dzi;
  return v;
}

int ibm_phase_indicator(ibm_ctx *c, int itype, double *gamu, double *gamv, double *gamw, double *gamp,
                        double *upart, double *vpart, double *wpart) {
  if (!c) return IBM_E_INVALID;
  if (itype != 0 && itype != 1) return set_err(c, IBM_E_INVALID, "itype must be 0 or 1");
  if (c->g.zper || c->pg.poly) return set_err(c, IBM_E_STATE, "no plane statistics with periodic z or polydisperse spheres");
  if (c->pg.np > 0 && !c->have_particles) return set_err(c, IBM_E_STATE, "no particles set");
  int st;
  if ((st = ensure_href(c))) return st;
  if ((st = run_phase_indicator(c, itype))) return st;
  const PhaseView v = phase_view(c, itype, true);
  double *out[7] = {gamu, gamv, gamw, gamp, upart, vpart, wpart};
  const size_t n = (size_t)(c->g.I + 2) * (c->g.J + 2) * (c->g.K + 2);
  for (int f = 0; f < 7; ++f) {
    if (!out[f]) continue;
    launch_phase_export(c->stream, v, f, c->href);
    LAUNCHED(1);
    CK(cudaMemcpyAsync(out[f], c->href, n * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
  }
  return phase_check(c);
}

// Ghost values, normalisations and derived scalars of post1d
// (output.f90:178-200, 276-294, 401-477, 549-566) from the plane sums
// S[k-1][POST1D_NSUM], k = 1..ktot.  Whole-array Fortran assignments read
// their right-hand sides before writing, hence the two-loop forms.
static void post1d_finish(const ibm_ctx *c, const std::vector<double> &S, bool parts, double *prof, double *scal) {
  const int K = c->g.K, k1 = K + 1, nk = K + 2;
  std::vector<std::vector<double>> q(IBM_NSTAT, std::vector<double>(nk, 0.));
  // plane sum index -> profile
  static const int src[POST1D_NSUM] = {
      IBM_STAT_UM,  IBM_STAT_VM,  IBM_STAT_WM,  IBM_STAT_PM,   IBM_STAT_CM,   IBM_STAT_UPM,  IBM_STAT_VPM, IBM_STAT_WPM,
      IBM_STAT_GUM, IBM_STAT_GVM, IBM_STAT_GWM, IBM_STAT_GPM,  IBM_STAT_U2,   IBM_STAT_V2,   IBM_STAT_W2,  IBM_STAT_P2,
      IBM_STAT_C2,  IBM_STAT_UP2, IBM_STAT_VP2, IBM_STAT_WP2,  IBM_STAT_GP2,  IBM_STAT_UV,   IBM_STAT_UW,  IBM_STAT_VW,
      IBM_STAT_WC,  IBM_STAT_CDFLX, IBM_STAT_UPVP, IBM_STAT_UPWP, IBM_STAT_VPWP, IBM_STAT_GUV, IBM_STAT_GUW, IBM_STAT_GVW};
  for (int k = 1; k <= K; ++k)
    for (int n = 0; n < POST1D_NSUM; ++n) q[src[n]][k] = S[(size_t)(k - 1) * POST1D_NSUM + n];
  auto &um = q[IBM_STAT_UM], &vm = q[IBM_STAT_VM], &wm = q[IBM_STAT_WM], &pm = q[IBM_STAT_PM];
  auto &u2 = q[IBM_STAT_U2], &v2 = q[IBM_STAT_V2], &w2 = q[IBM_STAT_W2], &p2 = q[IBM_STAT_P2];
  auto &uv = q[IBM_STAT_UV], &uw = q[IBM_STAT_UW], &vw = q[IBM_STAT_VW];
  auto &upm = q[IBM_STAT_UPM], &vpm = q[IBM_STAT_VPM], &wpm = q[IBM_STAT_WPM];
  auto &up2 = q[IBM_STAT_UP2], &vp2 = q[IBM_STAT_VP2], &wp2 = q[IBM_STAT_WP2];
  auto &upvp = q[IBM_STAT_UPVP], &upwp = q[IBM_STAT_UPWP], &vpwp = q[IBM_STAT_VPWP];
  auto &gum = q[IBM_STAT_GUM], &gvm = q[IBM_STAT_GVM], &gwm = q[IBM_STAT_GWM], &gpm = q[IBM_STAT_GPM];
  auto &gp2 = q[IBM_STAT_GP2], &guv = q[IBM_STAT_GUV], &guw = q[IBM_STAT_GUW], &gvw = q[IBM_STAT_GVW];
  auto &ss = q[IBM_STAT_SS], &ssp = q[IBM_STAT_SSP];
  auto &cm = q[IBM_STAT_CM], &c2 = q[IBM_STAT_C2], &wc = q[IBM_STAT_WC], &cdflx = q[IBM_STAT_CDFLX];
  // ghost planes of the raw sums; w-type quantities are zero on the top wall
  um[0] = -um[1]; um[k1] = -um[K];
  vm[0] = -vm[1]; vm[k1] = -vm[K];
  wm[0] = 0.; wm[K] = 0.; wm[k1] = wm[K - 1];
  pm[0] = pm[1]; pm[k1] = pm[K];
  upm[0] = -upm[1]; upm[k1] = -upm[K];
  vpm[0] = -vpm[1]; vpm[k1] = -vpm[K];
  wpm[0] = 0.; wpm[K] = 0.; wpm[k1] = wm[K - 1];  // wm, as the reference writes it
  gum[0] = gum[1]; gum[k1] = gum[K];
  gvm[0] = gvm[1]; gvm[k1] = gvm[K];
  gwm[k1] = gwm[K - 1];
  u2[0] = -u2[1]; u2[k1] = -u2[K];
  v2[0] = -v2[1]; v2[k1] = -v2[K];
  w2[0] = 0.; w2[K] = 0.; w2[k1] = w2[K - 1];
  p2[0] = p2[1]; p2[k1] = p2[K];
  up2[0] = -up2[1]; up2[k1] = -up2[K];
  vp2[0] = -vp2[1]; vp2[k1] = -vp2[K];
  wp2[0] = 0.; wp2[K] = 0.; wp2[k1] = w2[K - 1];  // w2, as the reference writes it
  gp2[0] = gp2[1]; gp2[k1] = gp2[K];
  uv[0] = -uv[1]; uv[k1] = -uv[K];
  uw[0] = 0.; uw[K] = 0.; uw[k1] = uw[K - 1];
  vw[0] = 0.; vw[k1] = vw[K - 1]; vw[K] = 0.;
  upvp[0] = -upvp[1]; upvp[k1] = -upvp[K];
  upwp[0] = 0.; upwp[K] = 0.; upwp[k1] = upwp[K - 1];
  vpwp[0] = 0.; vpwp[k1] = vpwp[K - 1]; vpwp[K] = 0.;
  guv[0] = guv[1]; guv[k1] = guv[K];
  guw[0] = guw[1]; guw[k1] = guw[K];
  gvw[0] = gvw[1]; gvw[k1] = gvw[K];
  // means and rms of the fluid (np > 0: weighted by the fluid fraction)
  const double N = 1. * c->prm.itot * c->prm.jtot;
  auto den = [&](const std::vector<double> &g, int k) { return parts ? g[k] : N - g[k]; };
  for (int k = 1; k <= K; ++k) {
    um[k] = um[k] / den(gum, k); vm[k] = vm[k] / den(gvm, k); wm[k] = wm[k] / den(gwm, k);
    cm[k] = cm[k] / den(gpm, k); pm[k] = pm[k] / den(gpm, k);
  }
  for (int k = 1; k <= K; ++k) {
    u2[k] = std::sqrt(u2[k] / den(gum, k) - um[k] * um[k]);
    v2[k] = std::sqrt(v2[k] / den(gvm, k) - vm[k] * vm[k]);
    w2[k] = std::sqrt(w2[k] / den(gwm, k) - wm[k] * wm[k]);
    p2[k] = std::sqrt(p2[k] / den(gpm, k) - pm[k] * pm[k]);
    c2[k] = std::sqrt(c2[k] / den(gpm, k) - cm[k] * cm[k]);
  }
  std::vector<double> t(nk);
  for (int k = 1; k <= K; ++k) t[k] = vw[k] / den(gvw, k) - 0.5 * (vm[k] + vm[k + 1]) * wm[k];
  for (int k = 1; k <= K; ++k) vw[k] = t[k];
  vw[0] = 0.;
  double umax = u2[0];
  for (int k = 1; k <= k1; ++k) umax = std::max(umax, u2[k]);
  const double visc = c->prm.visc, lz = c->prm.lz, dzi = c->g.dzi;
  const double re_rbc = umax * lz / visc;
  for (int k = 1; k <= K; ++k) {
    wc[k] = wc[k] / (N - gwm[k]);
    cdflx[k] = cdflx[k] / (N - gwm[k]);
  }
  // wall shear stress and friction velocity
  vm[0] = -vm[1]; vm[k1] = -vm[K];
  for (int k = 1; k <= K; ++k) ss[k] = (vm[k + 1] - vm[k]) * dzi * visc;
  ss[0] = (vm[1] - vm[0]) * dzi * visc;
  um[0] = -um[1]; um[k1] = -um[K];
  for (int k = 1; k <= K; ++k) {
    const double d = (um[k + 1] - um[k]) * dzi * visc;
    ss[k] = std::sqrt(ss[k] * ss[k] + d * d);
  }
  const double d0 = (um[1] - um[0]) * dzi * visc;
  ss[0] = std::sqrt(ss[0] * ss[0] + d0 * d0);
  const double grad_k_wall = dzi * (std::sqrt(0.5 * (u2[1] * u2[1] + v2[1] * v2[1] + w2[1] * w2[1])) -
                                    std::sqrt(0.5 * (u2[0] * u2[0] + v2[0] * v2[0] + w2[0] * w2[0])));
  const double u_tau = std::sqrt(visc * grad_k_wall);
  const double re_tau = u_tau * lz / visc;
  // Nusselt number
  double swc = 0., scd = 0.;
  for (int k = 1; k <= K; ++k) swc = swc + wc[k];
  for (int k = 1; k <= K; ++k) scd = scd + cdflx[k];
  const double nu = lz / (c->kappa * (c->sp.bc_c_bot_val - c->sp.bc_c_top_val)) * (swc / K + scd / K);
  // particle phase
  for (int k = 1; k <= K; ++k) {
    upm[k] = upm[k] / (N - gum[k]);
    vpm[k] = vpm[k] / (N - gvm[k]);
    wpm[k] = wpm[k] / (N - gwm[k]);
  }
  for (int k = 1; k <= K; ++k) {
    up2[k] = std::sqrt(up2[k] / (N - gum[k]) - upm[k] * upm[k]);
    vp2[k] = std::sqrt(vp2[k] / (N - gvm[k]) - vpm[k] * vpm[k]);
    wp2[k] = std::sqrt(wp2[k] / (N - gwm[k]) - wpm[k] * wpm[k]);
  }
  for (int k = 1; k <= K; ++k) t[k] = vpwp[k] / (N - gvw[k]) - 0.5 * (vpm[k] + vpm[k + 1]) * wpm[k];
  for (int k = 1; k <= K; ++k) vpwp[k] = t[k];
  vpwp[0] = 0.;
  vpm[0] = -vpm[1]; vpm[k1] = -vpm[K];
  for (int k = 1; k <= K; ++k) ssp[k] = (vpm[k + 1] - vpm[k]) * dzi * visc;
  ssp[0] = (vpm[1] - vpm[0]) * dzi * visc;
  if (prof)
    for (int n = 0; n < IBM_NSTAT; ++n) std::memcpy(prof + (size_t)n * nk, q[n].data(), nk * sizeof(double));
  if (scal) { scal[0] = re_tau; scal[1] = u_tau; scal[2] = nu; scal[3] = re_rbc; scal[4] = grad_k_wall; }
}

int ibm_post1d(ibm_ctx *c, double *prof, double *scal) {
  if (!c) return IBM_E_INVALID;
  if (!c->have_fields) return set_err(c, IBM_E_STATE, "no fields set");
  if (c->g.zper || c->pg.poly) return set_err(c, IBM_E_STATE, "no plane statistics with periodic z or polydisperse spheres");
  const bool parts = c->pg.np > 0;
  if (parts && !c->have_particles) return set_err(c, IBM_E_STATE, "no particles set");
  int st;
  if (parts && (st = run_phase_indicator(c, 1))) return st;
  const int K = c->g.K;
  // slices per plane: about four waves of three 128-thread blocks per SM
  const int slices = std::max(1, std::min(64, (1824 + K - 1) / K));
  const size_t np = (size_t)K * slices * POST1D_NSUM;
  if (c->stat_cap < np) {
    if (c->stat_part) cudaFree(c->stat_part);
    c->stat_part = nullptr;
    c->stat_cap = 0;
    CK(cudaMalloc((void **)&c->stat_part, np * sizeof(double)));
    c->stat_cap = np;
  }
  const PhaseView v = phase_view(c, 1, parts);
  if (c->mixed)
    PROBED(IBM_PROBE_STATS, launch_post1d_sums<float>(c->stream, c->g, v, c->u32, c->v32, c->w32, nullptr, c->p32,
                                                      c->plo32, c->cfield, c->kappa, c->stat_part, slices));
  else
    PROBED(IBM_PROBE_STATS, launch_post1d_sums<double>(c->stream, c->g, v, c->u, c->v, c->w, c->p, nullptr, nullptr,
                                                       c->cfield, c->kappa, c->stat_part, slices));
  LAUNCHED(1);
  std::vector<double> part(np), S((size_t)K * POST1D_NSUM, 0.);
  CK(cudaMemcpyAsync(part.data(), c->stat_part, np * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  if (parts && (st = phase_check(c))) return st;
  for (int k = 0; k < K; ++k)
    for (int s = 0; s < slices; ++s)
      for (int n = 0; n < POST1D_NSUM; ++n)
        S[(size_t)k * POST1D_NSUM + n] += part[((size_t)k * slices + s) * POST1D_NSUM + n];
  post1d_finish(c, S, parts, prof, scal);
  return IBM_OK;
}

int ibm_set_projection_solves(ibm_ctx *c, int solves) {
  if (!c) return IBM_E_INVALID;
  drop_graphs(c);  // the captured stages may depend on what this changes
  if (solves != 1 && solves != 2) return set_err(c, IBM_E_INVALID, "projection solves must be 1 or 2");
  if (!c->mixed) return solves == 1 ? IBM_OK : set_err(c, IBM_E_STATE, "the FP64 form solves once");
  c->proj_solves = solves;
  return IBM_OK;
}

int ibm_set_predictor_kernel(ibm_ctx *c, int kind) {
  if (!c) return IBM_E_INVALID;
  drop_graphs(c);  // the captured stages may depend on what this changes
  if (kind != IBM_PREDICTOR_AUTO && kind != IBM_PREDICTOR_PAIRS && kind != IBM_PREDICTOR_CELLS &&
      kind != IBM_PREDICTOR_TMA)
    return set_err(c, IBM_E_INVALID, "predictor kernel must be IBM_PREDICTOR_AUTO, _PAIRS, _CELLS or _TMA");
  c->pred_kind = kind;
  return IBM_OK;
}

int ibm_set_step_graphs(ibm_ctx *c, int enable) {
  if (!c) return IBM_E_INVALID;
  CK(cudaStreamSynchronize(c->stream));
  drop_graphs(c);
  c->use_graphs = enable != 0;
  return IBM_OK;
}

int ibm_prepare_step_graphs(ibm_ctx *c, double dt) {
  int st;
  if ((st = ready(c))) return st;
  if (!(dt > 0)) return set_err(c, IBM_E_INVALID, "dt must be > 0");
  // lazily initialised launch settings are set up by a direct step first
  if (!graphs_apply(c) || !(c->dt_last > 0)) return IBM_OK;
  CK(cudaStreamSynchronize(c->stream));
  const bool learned = c->mixed && c->learn_on && c->pg.np > 0;
  for (int rkiter = 1; rkiter <= 3; ++rkiter)
    for (int kind = FORCING_PLAIN; kind <= FORCING_LEARNED; ++kind) {
      if (learned ? kind == FORCING_PLAIN : kind != FORCING_PLAIN) continue;
      if ((st = stage_capture(c, rkiter, dt, kind, false))) return st;
      if (!c->use_graphs) return IBM_OK;
    }
  return IBM_OK;
}

int ibm_slip_residual(ibm_ctx *c, double *maxres, double *rmsres) {
  if (!c) return IBM_E_INVALID;
  if (c->pg.np == 0) { if (maxres) *maxres = 0; if (rmsres) *rmsres = 0; return IBM_OK; }
  // re-interpolate the forced field (valid between ibm_forcing_loop and ibm_project)
  if (c->mixed) c->launches += -1 + launch_ibm_interp_force_f(c->stream, c->g, c->pg, c->ib, c->fu32, c->fv32, c->fw32,
                                                             1., -2);
  else launch_ibm_interp_force<double>(c->stream, c->g, c->pg, c->ib, c->fu, c->fv, c->fw, 1., -1);
  LAUNCHED(1);
  launch_slip_residual(c->stream, c->pg, c->ib, c->dout + 16);
  LAUNCHED(1);
  CK(cudaMemcpyAsync(c->hpin, c->dout + 16, 2 * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  std::vector<int> nla(c->pg.np);
  CK(cudaMemcpy(nla.data(), c->ib.nla, c->pg.np * sizeof(int), cudaMemcpyDeviceToHost));
  long n = 0;
  for (int q : nla) n += q;
  if (maxres) *maxres = c->hpin[0];
  if (rmsres) *rmsres = n ? std::sqrt(c->hpin[1] / n) : 0.;
  return IBM_OK;
}

int ibm_diagnostics(ibm_ctx *c, double *wsn, double *wso, double ft[3]) {
  if (!c) return IBM_E_INVALID;
  double raw[3];
  CK(cudaMemcpyAsync(raw, c->dout + 8, 3 * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  // rk3.f90:99-103, 213-217, 321-325 for the last completed stage sequence
  const double dt = c->dt_last;
  const double dVeul = (1. / c->g.dxi) * (1. / c->g.dyi) * (1. / c->g.dzi);
  const double nt = (double)c->g.I * c->g.J * c->g.K;
  const double old1 = raw[0] / (dVeul * nt);
  const double old2 = raw[1] / (dVeul * nt);
  const double new3 = ((dt * (45. / 60.)) / dt) * raw[2] / (dVeul * nt) - ((dt * (25. / 60.)) / dt) * old2;
  (void)old1;
  if (wsn) *wsn = new3;
  if (wso) *wso = old2;
  if (ft) {
    ft[0] = ft[1] = ft[2] = 0.;
    const int np = c->pg.np;
    if (np > 0) {
      std::vector<double> f((size_t)3 * np);
      CK(cudaMemcpy(f.data(), c->pb.pf + (size_t)PF_FXLTOT * np, 3 * np * sizeof(double), cudaMemcpyDeviceToHost));
      for (int q = 0; q < 3; ++q)
        for (int p = 0; p < np; ++p) ft[q] += f[(size_t)q * np + p];
    }
  }
  return IBM_OK;
}

int ibm_phase_times(ibm_ctx *c, double ms[4]) {
  if (!c || !ms) return IBM_E_INVALID;
  for (int q = 0; q < 4; ++q) ms[q] = c->phase_ms[q];
  return IBM_OK;
}

long long ibm_launch_count(const ibm_ctx *c) { return c ? c->launches : 0; }

int ibm_sync(ibm_ctx *c) {
  if (!c) return IBM_E_INVALID;
  CK(cudaStreamSynchronize(c->stream));
  return check_flags(c);
}

/* --- learned forcing -------------------------------------------------------- */

int ibm_harvest_read(ibm_ctx *c, float *feat, float *targ, int cap, int *n) {
  if (!c || !n || cap < 0) return IBM_E_INVALID;
  *n = 0;
  if (!c->hv.count) return IBM_OK;
  int cnt[2];
  CK(cudaMemcpyAsync(cnt, c->hv.count, sizeof(cnt), cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  *n = cnt[1];
  const size_t m = (size_t)std::min(cap, cnt[1]);
  if (feat && m) CK(cudaMemcpyAsync(feat, c->hv.feat, m * 96 * sizeof(float), cudaMemcpyDeviceToHost, c->stream));
  if (targ && m) CK(cudaMemcpyAsync(targ, c->hv.targ, m * 3 * sizeof(float), cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  return IBM_OK;
}

int ibm_harvest(ibm_ctx *c, int capacity, int stride, int passes) {
  if (!c) return IBM_E_INVALID;
  drop_graphs(c);  // the captured stages may depend on what this changes
  if (c->mode != IBM_MODE_MIXED_LEARNED) return set_err(c, IBM_E_STATE, "harvesting needs IBM_MODE_MIXED_LEARNED");
  if (capacity < 0 || (capacity > 0 && (stride < 1 || passes < 0))) return set_err(c, IBM_E_INVALID, "bad harvest arguments");
  if (capacity == 0) {
    c->harvesting = false;
    return IBM_OK;
  }
  CK(cudaStreamSynchronize(c->stream));
  void *old[] = {c->hv.feat, c->hv.pidx, c->hv.targ, c->hv.count};
  for (void *q : old)
    if (q) cudaFree(q);
  c->hv = HarvestArgs{};
  int st;
  if ((st = dalloc(c, &c->hv.feat, (size_t)capacity * 96))) return st;
  if ((st = dalloc(c, &c->hv.pidx, (size_t)capacity))) return st;
  if ((st = dalloc(c, &c->hv.targ, (size_t)capacity * 3))) return st;
  if ((st = dalloc(c, &c->hv.count, 2))) return st;
  c->hv.cap = capacity;
  c->hv.stride = stride;
  c->hv.phase = 0;
  c->hv_passes = passes;
  c->harvesting = true;
  CK(cudaStreamSynchronize(c->stream));
  return IBM_OK;
}

// a new model: the live gate's plain reduction factors are measured afresh
// per RK stage (those of the harvest come from an earlier flow)
static int reset_gate_factors(ibm_ctx *c) {
  for (int s = 0; s < 3; ++s) c->ncal[s] = 0, c->since[s] = 0;
  if (!c->ls) return IBM_OK;
  double h[IBM_LS_N];
  CK(cudaMemcpyAsync(h, c->ls, sizeof(h), cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  h[1] = h[11] = h[12] = 0.;
  h[13] = h[14] = h[15] = 0.;
  CK(cudaMemcpyAsync(c->ls, h, sizeof(h), cudaMemcpyHostToDevice, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  return IBM_OK;
}

int ibm_train_forcing_model(ibm_ctx *c, int nsteps, int batch, double lr, unsigned seed, int reinit, double *loss) {
  if (!c) return IBM_E_INVALID;
  drop_graphs(c);  // the captured stages may depend on what this changes
  if (c->mode != IBM_MODE_MIXED_LEARNED) return set_err(c, IBM_E_STATE, "training needs IBM_MODE_MIXED_LEARNED");
  if (nsteps < 0 || batch < 1 || !(lr > 0)) return set_err(c, IBM_E_INVALID, "bad training arguments");
  if (!c->hv.count) return set_err(c, IBM_E_STATE, "no harvested samples (ibm_harvest)");
  int cnt[2];
  CK(cudaMemcpyAsync(cnt, c->hv.count, sizeof(cnt), cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  const int n = cnt[1];
  if (n < 1) return set_err(c, IBM_E_STATE, "no harvested samples (ibm_harvest)");
  if (reinit || !c->stats_ready) {
    // standardisation from the samples (device reductions), fresh weights
    // and moments
    int st;
    if (!c->nscr && (st = dalloc(c, &c->nscr, mlp_norm_scratch()))) return st;
    c->launches += launch_mlp_norm(c->stream, n, c->hv.feat, c->hv.targ, c->nscr, c->norm);
    std::vector<float> w;
    init_mlp_params(w, seed);
    CK(cudaMemcpy(c->mt.params, w.data(), w.size() * sizeof(float), cudaMemcpyHostToDevice));
    CK(cudaMemsetAsync(c->mt.m, 0, w.size() * sizeof(float), c->stream));
    CK(cudaMemsetAsync(c->mt.v, 0, w.size() * sizeof(float), c->stream));
    launch_mlp_refresh(c->stream, c->mt.params, c->mt.w1b, c->mt.w2b);
    LAUNCHED(1);
    c->train_step = 0;
    c->stats_ready = true;
  }
  if (c->tcap < n) {
    if (c->tx) cudaFree(c->tx);
    if (c->tt) cudaFree(c->tt);
    c->tx = nullptr; c->tt = nullptr; c->tcap = 0;
    int st;
    if ((st = dalloc(c, &c->tx, (size_t)n * 96))) return st;
    if ((st = dalloc(c, &c->tt, (size_t)n * 3))) return st;
    c->tcap = n;
  }
  launch_mlp_stage(c->stream, n, c->hv.feat, c->hv.targ, c->norm, c->norm + 96, c->norm + 192, c->norm + 195, c->tx,
                   c->tt);
  LAUNCHED(1);
  if (c->mt_cap < batch) {
    CK(cudaStreamSynchronize(c->stream));
    free_mlp_batch(c->mt);
    c->mt_cap = 0;
    int st;
    if ((st = alloc_mlp_batch(c, c->mt, batch))) return st;
    c->mt_cap = batch;
  }
  for (int q = 0; q < nsteps; ++q) {
    ++c->train_step;
    c->launches += launch_mlp_train_step(c->stream, c->mt, c->tx, c->tt, n, batch, seed, 1, c->train_step, (float)lr,
                                         1, nullptr);
  }
  float l = 0.f;
  int herr = 0;
  CK(cudaMemcpyAsync(&l, c->mt.loss, sizeof(float), cudaMemcpyDeviceToHost, c->stream));
  CK(cudaMemcpyAsync(&herr, c->mt.err, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  if (herr) return set_err(c, IBM_E_NOT_CONVERGED, "tensor-core MMA wait timed out in training");
  if (loss) *loss = l;
  c->model_ready = true;
  c->learn_on = true;
  return reset_gate_factors(c);
}

int ibm_set_forcing_model(ibm_ctx *c, const float *params, const float *norm) {
  if (!c || !params || !norm) return IBM_E_INVALID;
  drop_graphs(c);  // the captured stages may depend on what this changes
  if (c->mode != IBM_MODE_MIXED_LEARNED) return set_err(c, IBM_E_STATE, "a model needs IBM_MODE_MIXED_LEARNED");
  CK(cudaMemcpyAsync(c->mt.params, params, mlp_nparam() * sizeof(float), cudaMemcpyHostToDevice, c->stream));
  CK(cudaMemcpyAsync(c->norm, norm, 198 * sizeof(float), cudaMemcpyHostToDevice, c->stream));
  CK(cudaMemsetAsync(c->mt.m, 0, mlp_nparam() * sizeof(float), c->stream));
  CK(cudaMemsetAsync(c->mt.v, 0, mlp_nparam() * sizeof(float), c->stream));
  launch_mlp_refresh(c->stream, c->mt.params, c->mt.w1b, c->mt.w2b);
  LAUNCHED(1);
  CK(cudaStreamSynchronize(c->stream));
  c->train_step = 0;
  c->stats_ready = c->model_ready = c->learn_on = true;
  return reset_gate_factors(c);
}

int ibm_get_forcing_model(ibm_ctx *c, float *params, float *norm) {
  if (!c) return IBM_E_INVALID;
  if (!c->model_ready) return set_err(c, IBM_E_STATE, "no model (ibm_train_forcing_model or ibm_set_forcing_model)");
  if (params) CK(cudaMemcpyAsync(params, c->mt.params, mlp_nparam() * sizeof(float), cudaMemcpyDeviceToHost, c->stream));
  if (norm) CK(cudaMemcpyAsync(norm, c->norm, 198 * sizeof(float), cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  return IBM_OK;
}

int ibm_learned_config(ibm_ctx *c, int enable, double fallback_ratio, double plain_rms_ref) {
  if (!c) return IBM_E_INVALID;
  drop_graphs(c);  // the captured stages may depend on what this changes
  if (c->mode != IBM_MODE_MIXED_LEARNED) return set_err(c, IBM_E_STATE, "needs IBM_MODE_MIXED_LEARNED");
  if (enable && !c->model_ready) return set_err(c, IBM_E_STATE, "no model to enable");
  if (!(fallback_ratio > 0) || plain_rms_ref < 0) return set_err(c, IBM_E_INVALID, "bad learned-forcing settings");
  double h[IBM_LS_N];
  CK(cudaMemcpyAsync(h, c->ls, sizeof(h), cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  h[3] = fallback_ratio;
  h[8] = plain_rms_ref;  // > 0: a fixed reference; 0: the live one
  CK(cudaMemcpyAsync(c->ls, h, sizeof(h), cudaMemcpyHostToDevice, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  c->learn_on = enable != 0;
  return IBM_OK;
}

int ibm_learned_stats(ibm_ctx *c, double stats[6]) {
  if (!c || !stats) return IBM_E_INVALID;
  for (int q = 0; q < 6; ++q) stats[q] = 0.;
  if (c->mode != IBM_MODE_MIXED_LEARNED) return IBM_OK;
  double h[IBM_LS_N];
  int cnt[2] = {0, 0};
  CK(cudaMemcpyAsync(h, c->ls, sizeof(h), cudaMemcpyDeviceToHost, c->stream));
  if (c->hv.count) CK(cudaMemcpyAsync(cnt, c->hv.count, sizeof(cnt), cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  stats[0] = h[0];
  stats[1] = h[5] > 0 ? h[7] : h[10];  // the last gate's reference (before any: the last plain residual)
  stats[2] = h[3];
  stats[3] = h[4];
  stats[4] = h[5];
  stats[5] = cnt[1];
  return IBM_OK;
}

int ibm_learned_calibration(ibm_ctx *c, int period) {
  if (!c) return IBM_E_INVALID;
  if (c->mode != IBM_MODE_MIXED_LEARNED) return set_err(c, IBM_E_STATE, "needs IBM_MODE_MIXED_LEARNED");
  if (period < 0) return set_err(c, IBM_E_INVALID, "period must be >= 0");
  c->calib_period = period;
  for (long long &n : c->since) n = 0;
  return IBM_OK;
}

int ibm_learned_gate_state(ibm_ctx *c, double g[6]) {
  if (!c || !g) return IBM_E_INVALID;
  for (int q = 0; q < 6; ++q) g[q] = 0.;
  if (c->mode != IBM_MODE_MIXED_LEARNED) return IBM_OK;
  double h[IBM_LS_N];
  CK(cudaMemcpyAsync(h, c->ls, sizeof(h), cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  g[0] = h[6]; g[1] = h[6] > 0 ? h[7] / h[6] : 0.; g[2] = h[2]; g[3] = h[7]; g[4] = h[9]; g[5] = h[10];
  return IBM_OK;
}

int ibm_forcing_perturbation(ibm_ctx *c, const double sigma[3], unsigned seed) {
  if (!c || !sigma) return IBM_E_INVALID;
  if (!c->mixed) return set_err(c, IBM_E_STATE, "the forcing perturbation needs a mixed form");
  for (int q = 0; q < 3; ++q)
    if (!(sigma[q] >= 0.)) return set_err(c, IBM_E_INVALID, "sigma must be >= 0");
  for (int q = 0; q < 3; ++q) c->noise_sigma[q] = sigma[q];
  c->noise_seed = seed;
  c->noise_counter = 0;
  return IBM_OK;
}

// test hooks on a scratch model: the library's forward/backward kernels on a
// caller batch, for the check against a CPU reference
static int mlp_scratch(ibm_ctx *c, const float *params, const float *x, const float *t, int nb, MlpTrainBuffers &B) {
  int st;
  if ((st = alloc_mlp_model(c, B))) return st;
  if ((st = alloc_mlp_batch(c, B, nb))) return st;
  std::vector<float> tmp;
  CK(cudaMemcpyAsync(B.params, params, mlp_nparam() * sizeof(float), cudaMemcpyHostToDevice, c->stream));
  float *xf = nullptr;
  if ((st = dalloc(c, &xf, (size_t)nb * 96))) return st;
  CK(cudaMemcpyAsync(xf, x, (size_t)nb * 96 * sizeof(float), cudaMemcpyHostToDevice, c->stream));
  launch_f2bf(c->stream, (long)nb * 96, xf, B.x);
  CK(cudaMemcpyAsync(B.t, t, (size_t)nb * 3 * sizeof(float), cudaMemcpyHostToDevice, c->stream));
  launch_mlp_refresh(c->stream, B.params, B.w1b, B.w2b);
  LAUNCHED(2);
  CK(cudaStreamSynchronize(c->stream));
  cudaFree(xf);
  return IBM_OK;
}

int ibm_mlp_gradient(ibm_ctx *c, const float *params, const float *x, const float *t, int nb, float *grad,
                     float *loss, float *y) {
  if (!c || !params || !x || !t || nb < 1) return IBM_E_INVALID;
  MlpTrainBuffers B{};
  int st = mlp_scratch(c, params, x, t, nb, B);
  if (st == IBM_OK) {
    c->launches += launch_mlp_train_step(c->stream, B, B.x, B.t, nb, nb, 0u, 0, 1, 0.f, 0, B.y);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess && grad)
      e = cudaMemcpyAsync(grad, B.grad, mlp_nparam() * sizeof(float), cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess && loss) e = cudaMemcpyAsync(loss, B.loss, sizeof(float), cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess && y)
      e = cudaMemcpyAsync(y, B.y, (size_t)nb * 3 * sizeof(float), cudaMemcpyDeviceToHost, c->stream);
    int herr = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&herr, B.err, sizeof(int), cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    st = cuda_err(c, e, "ibm_mlp_gradient");
    if (st == IBM_OK && herr) st = set_err(c, IBM_E_NOT_CONVERGED, "tensor-core MMA wait timed out");
  }
  cudaStreamSynchronize(c->stream);
  free_mlp_batch(B);
  free_mlp_model(B);
  return st;
}

int ibm_mlp_infer(ibm_ctx *c, const float *params, const float *x, int nb, float *y) {
  if (!c || !params || !x || !y || nb < 1) return IBM_E_INVALID;
  MlpTrainBuffers B{};
  std::vector<float> t((size_t)nb * 3, 0.f);
  int st = mlp_scratch(c, params, x, t.data(), nb, B);
  if (st == IBM_OK) {
    launch_mlp_infer(c->stream, B.x, nb, B.w1b, B.w2b, B.params, B.y);
    c->launches += 1;
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(y, B.y, (size_t)nb * 3 * sizeof(float), cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    st = cuda_err(c, e, "ibm_mlp_infer");
  }
  cudaStreamSynchronize(c->stream);
  free_mlp_batch(B);
  free_mlp_model(B);
  return st;
}

int ibm_mlp_infer_tc(ibm_ctx *c, const float *params, const float *x, int nb, float *y) {
  if (!c || !params || !x || !y || nb < 1) return IBM_E_INVALID;
  MlpTrainBuffers B{};
  std::vector<float> t((size_t)nb * 3, 0.f);
  int st = mlp_scratch(c, params, x, t.data(), nb, B);
  int *derr = nullptr;
  if (st == IBM_OK) st = dalloc(c, &derr, 1);
  if (st == IBM_OK) {
    c->launches += launch_mlp_infer_tc(c->stream, B.x, nb, B.w1b, B.w2b, B.params, B.y, derr);
    int herr = 0;
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(y, B.y, (size_t)nb * 3 * sizeof(float), cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&herr, derr, sizeof(int), cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    st = cuda_err(c, e, "ibm_mlp_infer_tc");
    if (st == IBM_OK && herr) st = set_err(c, IBM_E_NOT_CONVERGED, "tensor-core MMA wait timed out");
  }
  cudaStreamSynchronize(c->stream);
  if (derr) cudaFree(derr);
  free_mlp_batch(B);
  free_mlp_model(B);
  return st;
}

int ibm_mlp_fit(ibm_ctx *c, const float *params_in, const float *x, const float *t, int nb, int nsteps, double lr,
                float *params_out, float *losses) {
  if (!c || !params_in || !x || !t || nb < 1 || nsteps < 0 || !(lr > 0)) return IBM_E_INVALID;
  MlpTrainBuffers B{};
  int st = mlp_scratch(c, params_in, x, t, nb, B);
  cudaError_t e = cudaSuccess;
  for (int q = 0; st == IBM_OK && e == cudaSuccess && q < nsteps; ++q) {
    c->launches += launch_mlp_train_step(c->stream, B, B.x, B.t, nb, nb, 0u, 0, q + 1, (float)lr, 1, nullptr);
    e = cudaGetLastError();
    if (e == cudaSuccess && losses) e = cudaMemcpyAsync(losses + q, B.loss, sizeof(float), cudaMemcpyDeviceToHost, c->stream);
  }
  if (st == IBM_OK && e == cudaSuccess && params_out)
    e = cudaMemcpyAsync(params_out, B.params, mlp_nparam() * sizeof(float), cudaMemcpyDeviceToHost, c->stream);
  int herr = 0;
  if (st == IBM_OK && e == cudaSuccess) e = cudaMemcpyAsync(&herr, B.err, sizeof(int), cudaMemcpyDeviceToHost, c->stream);
  if (st == IBM_OK && e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  if (st == IBM_OK) st = cuda_err(c, e, "ibm_mlp_fit");
  if (st == IBM_OK && herr) st = set_err(c, IBM_E_NOT_CONVERGED, "tensor-core MMA wait timed out");
  cudaStreamSynchronize(c->stream);
  free_mlp_batch(B);
  free_mlp_model(B);
  return st;
}

/* --- per-kernel event probe --------------------------------------------------- */

int ibm_probe(ibm_ctx *c, unsigned mask) {
  if (!c) return IBM_E_INVALID;
  CK(cudaStreamSynchronize(c->stream));
  c->probe_mask = mask & ((1u << IBM_PROBE_N) - 1);
  for (int q = 0; q < IBM_PROBE_N; ++q) c->probe_used[q] = 0;
  return IBM_OK;
}

int ibm_probe_result(ibm_ctx *c, double ms[IBM_PROBE_N], int launches[IBM_PROBE_N]) {
  if (!c) return IBM_E_INVALID;
  CK(cudaStreamSynchronize(c->stream));
  for (int q = 0; q < IBM_PROBE_N; ++q) {
    double tot = 0.;
    const int n = c->probe_used[q] / 2;
    for (int k = 0; k < n; ++k) {
      float t = 0.f;
      CK(cudaEventElapsedTime(&t, c->probe_ev[q][2 * k], c->probe_ev[q][2 * k + 1]));
      tot += t;
    }
    if (ms) ms[q] = tot;
    if (launches) launches[q] = n;
    c->probe_used[q] = 0;
  }
  c->probe_mask = 0;
  return IBM_OK;
}


}  // extern "C"
