// C ABI of the GB300 GetHI path (include/gethi_gpu.h): context lifecycle,
// device memory plan and the stage sequence of src/main_gh.c:34-74.
//
// Device memory per context (N = n_grid, m = N/2):
//   main  N^3 floats  : delta_k (split half spectrum) -> delta(x) -> HI mass
//   nyq   N^2 complex : kx = N/2 plane of delta_k
//   A, B, C N^3 floats (+ N^2 complex Nyquist planes each): phi after the Z
//         pass, i kz phi, and v_x after the Y pass (spectral velocity); only A
//         for the finite-difference velocity, none without RSD
//   vr    N^3 floats  : radial velocity -> dz_rsd
//   maps  n_nu 12 nside^2 floats
//   plus FP64/FP32 tables, twiddles, per-block partial sums.
#include <cmath>
#include <cstdio>
#include <chrono>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/gethi_gpu.h"
#include "common.cuh"
#include "fft.h"
#include "host.h"

using namespace gethi;

struct gethi_ctx {
  Setup s;
  int device = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  float2 *main = nullptr, *nyq = nullptr, *modes = nullptr;
  float2 *bA = nullptr, *bAn = nullptr, *bB = nullptr, *bBn = nullptr, *bC = nullptr, *bCn = nullptr;
  float *vr = nullptr, *maps = nullptr;
  float2 *twN = nullptr, *twM = nullptr;
  double2 *partials = nullptr;
  double *stats = nullptr;
  float *pk_f = nullptr, *logk_f = nullptr, *tab_f = nullptr, *prefac = nullptr, *edges_f = nullptr;
  double *tab_d = nullptr, *edges_d = nullptr;
  int *counters = nullptr;
  long npartials = 0;
  DevCfg cfg;
  int stage = 0;  // 0: init, 1: fields (delta, v_r), 2: mass and dz
  cudaEvent_t ev[8] = {};
  float times[7] = {};
  int nev = 0;
  // per-kernel-class device time (profiling on): events around each launch
  int prof = 0;
  cudaEvent_t kev[2 * 64] = {};
  int kcls[64] = {};
  int nk = 0;
  double ktime[GETHI_NKCLASS] = {};
  long kcount[GETHI_NKCLASS] = {};
  long launches = 0;
  void *staging = nullptr;  // pinned host copy of the per-realisation inputs
  void *fq = nullptr;       // queue of samples whose FP32 key is uncertain
  long fq_cap = 0;
  float2 *pg = nullptr, *pgn = nullptr;  // Gaussianised spectrum (gaussianise=1)
  // point sources (do_psources=1): per-pixel sums, channel maps, tables, source count
  float *ps_acc = nullptr, *maps_ps = nullptr, *ps_nz = nullptr, *ps_icdf = nullptr, *ps_chan = nullptr;
  unsigned long long *ps_total = nullptr;
  PsConst psc{};
  float2 *tab_df = nullptr, *edges_df = nullptr;  // double-float tables for the key refinement
  // pipelined realisations (gethi_gpu_run_async): two device map buffers, a copy stream, events
  float *maps_b[2] = {nullptr, nullptr};
  cudaStream_t copy_stream = nullptr;
  cudaEvent_t ev_done[2] = {nullptr, nullptr}, ev_copied[2] = {nullptr, nullptr};
  bool copied_pending[2] = {false, false};
  int cur_buf = 0;
  uint4 *tc_bmat = nullptr;                // fft_precision=tc_split tables and error flag
  float2 *tc_tw = nullptr;
  int *tc_err = nullptr;
};

namespace {

// FP32 tables, NZ entries each: z(r), density growth, velocity growth, and the
// projection's line table (slope, deviation bound)
constexpr int kTabF = 5;

void line_table(const Setup &s, float *out)
{
  const double dx = s.d.l_box / s.p.n_grid, rho = subsample_radius(s.xs, s.ys, s.zs, dx);
  for (int i = 0; i < NZ; i++) {
    const float2 v = shell_line_entry(s.z_r2z.data(), s.d.glob_idr, dx, rho, i);
    out[i] = v.x;
    out[NZ + i] = v.y;
  }
}

int cuda_fail(cudaError_t e, const char *what)
{
  set_error(std::string(what) + ": " + cudaGetErrorString(e));
  return GETHI_E_CUDA;
}

#define CK(call)                                           \
  do {                                                     \
    cudaError_t e_ = (call);                               \
    if (e_ != cudaSuccess) return cuda_fail(e_, #call);    \
  } while (0)

template <class T>
int dalloc(T **p, size_t count)
{
  cudaError_t e = cudaMalloc((void **)p, count * sizeof(T) + 256);
  if (e != cudaSuccess) {
    *p = nullptr;
    set_error(std::string("cudaMalloc of ") + std::to_string(count * sizeof(T)) + " bytes: " + cudaGetErrorString(e));
    return GETHI_E_NOMEM;
  }
  return GETHI_OK;
}

void twiddles(std::vector<float2> &t, int L)
{
  t.resize(L);
  for (int k = 0; k < L; k++) {
    double a = 2 * M_PI * (double)k / L;
    t[k] = make_float2((float)std::cos(a), (float)std::sin(a));
  }
}

void fill_cfg(gethi_ctx *c)
{
  const Setup &s = c->s;
  DevCfg &g = c->cfg;
  std::memset(&g, 0, sizeof(g));
  g.n = s.p.n_grid;
  g.m = s.p.n_grid / 2;
  g.l_box = s.d.l_box;
  g.dx = s.d.l_box / s.p.n_grid;  // src/pixelize.c:175
  g.pos_obs = s.d.pos_obs;
  g.dxf = (float)g.dx;
  g.pos_obsf = (float)g.pos_obs;
  g.logk_f = c->logk_f;
  g.pk_f = c->pk_f;
  g.numk = s.d.numk;
  g.logkmin = (float)s.d.logkmin;
  g.logkmax = (float)s.d.logkmax;
  g.idlogk = (float)s.d.idlogk;
  g.n_scal = (float)s.n_scal;
  double dk = 2 * M_PI / s.d.l_box;
  g.dk = (float)dk;
  g.idk3 = (float)(1. / (dk * dk * dk));
  g.r2_smooth = (float)s.d.r2_smooth;
  g.do_smoothing = s.d.do_smoothing;
  g.norm = (float)std::pow(std::sqrt(2 * M_PI) / s.d.l_box, 3);
  g.vfac = (float)(s.d.fgrowth_0 * s.d.hubble_0);
  g.seed = s.p.seed;
  g.z_r2z = c->tab_d;
  g.r_r2z = c->tab_d + NZ;
  g.gd = c->tab_d + 2 * NZ;
  g.gv = c->tab_d + 3 * NZ;
  g.z_r2z_f = c->tab_f;
  g.gd_f = c->tab_f + NZ;
  g.gv_f = c->tab_f + 2 * NZ;
  g.z_lin_g = c->tab_f + 3 * NZ;
  g.z_lin_e = c->tab_f + 4 * NZ;
  g.glob_idr = s.d.glob_idr;
  g.glob_idr_f = (float)s.d.glob_idr;
  g.r_tab_max = s.r_r2z[NZ - 1];
  g.r_tab_max_f = (float)g.r_tab_max;
  g.n_nu = s.p.n_nu;
  g.regular_nu = s.d.regular_nu;
  g.nside = s.p.n_side;
  g.npix = 12 * s.p.n_side * s.p.n_side;
  g.nu_min = s.p.nu_min;
  g.nu_max = s.p.nu_max;
  g.inv_dnu = s.p.n_nu / (s.p.nu_max - s.p.nu_min);  // src/pixelize.c:177
  g.nu_edges = c->edges_d;
  g.nu_edges_f = c->edges_f;
  g.prefac = c->prefac;
  for (int i = 0; i < NSUB; i++) {
    g.xs[i] = s.xs[i];
    g.ys[i] = s.ys[i];
    g.zs[i] = s.zs[i];
  }
  g.bias_const = s.p.bias_model;
  g.b_HI = (float)s.p.b_HI;
  g.do_rsd = s.p.do_rsd;
  g.mass_prefac = (float)(g.dx * g.dx * g.dx);  // src/grid_tools.c:122
  g.tc_bmat = c->tc_bmat;
  g.tc_tw = c->tc_tw;
  g.tc_err = c->tc_err;
  if (c->tab_df) {
    auto split = [](double v) { const float h = (float)v; return make_float2(h, (float)(v - (double)h)); };
    g.z_r2z_df = c->tab_df;
    g.r_r2z_df = c->tab_df + NZ;
    g.nu_edges_df = c->edges_df;
    g.dx_df = split(g.dx);
    g.pos_obs_df = split(g.pos_obs);
    g.glob_idr_df = split(g.glob_idr);
    g.inv_dnu_df = split(g.inv_dnu);
    g.nu_min_df = split(g.nu_min);
    for (int i = 0; i < NSUB; i++) {
      g.xs_df[i] = split(g.xs[i]);
      g.ys_df[i] = split(g.ys[i]);
      g.zs_df[i] = split(g.zs[i]);
    }
  }
}

ColGeom geom(float2 *base, long cpp, long pstride, long cstride, long estride, long ncols)
{
  ColGeom g;
  g.base = base;
  g.cpp = cpp;
  g.pstride = pstride;
  g.cstride = cstride;
  g.estride = estride;
  g.ncols = ncols;
  return g;
}

void record(gethi_ctx *c)
{
  if (c->nev < 8) cudaEventRecord(c->ev[c->nev++], c->stream);
}

// bracket one kernel launch of class `cls` (KC_*) with events when profiling
struct KTimer {
  gethi_ctx *c;
  int slot = -1;
  KTimer(gethi_ctx *c_, int cls) : c(c_)
  {
    c->launches++;
    if (c->prof && c->nk < 64) {
      slot = c->nk++;
      c->kcls[slot] = cls;
      cudaEventRecord(c->kev[2 * slot], c->stream);
    }
  }
  ~KTimer()
  {
    if (slot >= 0) cudaEventRecord(c->kev[2 * slot + 1], c->stream);
  }
};

void collect_kernel_times(gethi_ctx *c)
{
  for (int i = 0; i < c->nk; i++) {
    float ms = 0;
    if (cudaEventElapsedTime(&ms, c->kev[2 * i], c->kev[2 * i + 1]) == cudaSuccess) {
      c->ktime[c->kcls[i]] += ms;
      c->kcount[c->kcls[i]]++;
    }
  }
  c->nk = 0;
}

// One field: Z pass (modes generated on the fly), Y pass, X pass with epilogue.

// Geometries of the column sets (main block and Nyquist plane, Z and Y axes).
struct Geoms {
  ColGeom zm, zn, ym, yn;
};
Geoms geoms(float2 *main, float2 *nyq, long n, long m)
{
  return {geom(main, n * m, 0, 1, n * m, n * m), geom(nyq, n, 0, 1, n, n), geom(main, m, n * m, 1, m, n * m),
          geom(nyq, n, 0, n, 1, n)};
}

int plain_c2r(gethi_ctx *c, float2 *main, float2 *nyq, float scale)
{
  DevCfg g = c->cfg;
  g.tc_bmat = nullptr;  // FP32 passes: P_G spans many decades and is shared by both FFT precisions
  const long n = g.n, m = g.m;
  cudaStream_t st = c->stream;
  Geoms d = geoms(main, nyq, n, m);
  CK(col_pass(g, d.zm, 0, 0, 0, nullptr, c->twN, nullptr, nullptr, st));
  CK(col_pass(g, d.zn, 1, 0, 0, nullptr, c->twN, nullptr, nullptr, st));
  CK(col_pass(g, d.ym, 0, 0, 0, nullptr, c->twN, nullptr, nullptr, st));
  CK(col_pass(g, d.yn, 1, 0, 0, nullptr, c->twN, nullptr, nullptr, st));
  RowIn in = {{main, nullptr, nullptr}, {nyq, nullptr, nullptr}};
  CK(row_pass(g, in, c->twN, c->twM, scale, 3, nullptr, nullptr, st));
  c->launches += 5;
  return GETHI_OK;
}

// Gaussianised spectrum P_G on the grid, once per context (pg holds N^3 floats,
// main/nyq serve as scratch for xi).  src/fourier.c has no counterpart: the
// reference draws the modes from P(k) itself.
int make_pg(gethi_ctx *c)
{
  const DevCfg &g = c->cfg;
  const long n = g.n;
  const double vol = c->s.d.l_box * c->s.d.l_box * c->s.d.l_box;
  cudaStream_t st = c->stream;
  CK(pack_pk(g, c->main, c->nyq, (float)(1.0 / vol), st));
  int rc = plain_c2r(c, c->main, c->nyq, 1.f);  // xi(x), compact N^3 in main
  if (rc) return rc;
  CK(log_xi(g, reinterpret_cast<const float *>(c->main), c->pg, c->pgn, st));
  rc = plain_c2r(c, c->pg, c->pgn, (float)(vol / ((double)n * n * n)));  // P_G(k) on the full grid
  if (rc) return rc;
  c->launches += 2;
  c->cfg.pg = reinterpret_cast<const float *>(c->pg);
  return GETHI_OK;
}

// P_G for drawing the modes when gaussianise=1 (built on first use)
int ensure_pg(gethi_ctx *c)
{
  if (!c->s.p.gaussianise || c->cfg.pg) return GETHI_OK;
  const size_t n = c->s.p.n_grid;
  if (!c->pg) {
    int rc = dalloc(&c->pg, n * n * n / 2);
    if (!rc) rc = dalloc(&c->pgn, n * n);
    if (rc) return rc;
  }
  return make_pg(c);
}

// point sources of the current (Gaussian) fields into maps_ps; cat != nullptr
// also records the sources
int enqueue_psources(gethi_ctx *c, cudaStream_t st, const PsCatalogue *cat)
{
  PsCatalogue none{};
  CK(cudaMemsetAsync(c->ps_total, 0, sizeof(unsigned long long), st));
  KTimer t(c, KC_PSOURCES);
  CK(psources(c->cfg, c->psc, c->stats, reinterpret_cast<const float *>(c->main), c->vr, c->ps_acc, c->maps_ps,
              c->ps_chan, c->ps_total, cat ? *cat : none, st));
  c->launches += 1;
  return GETHI_OK;
}

// All Fourier-space work of one realisation: one Z pass drawing the modes and
// transforming delta (+ phi, + i kz phi), Y passes, X passes.
int fields_fft(gethi_ctx *c, const float2 *src)
{
  const DevCfg &g = c->cfg;
  const Setup &s = c->s;
  const long n = g.n, m = g.m;
  cudaStream_t st = c->stream;
  const int nout = s.p.do_rsd ? (s.p.velocity_mode == 1 ? 3 : 2) : 1;
  Geoms d = geoms(c->main, c->nyq, n, m), A = geoms(c->bA, c->bAn, n, m), B = geoms(c->bB, c->bBn, n, m),
        C = geoms(c->bC, c->bCn, n, m);
  {
    KTimer t(c, KC_ZPASS);
    CK(col_pass(g, d.zm, 0, 1, nout, src, c->twN, c->bA, c->bB, st));
  }
  {
    KTimer t(c, KC_NYQ);
    CK(col_pass(g, d.zn, 1, 1, nout, src, c->twN, c->bAn, c->bBn, st));
  }
  // density
  {
    KTimer t(c, KC_YPASS);
    CK(col_pass(g, d.ym, 0, 0, 0, nullptr, c->twN, nullptr, nullptr, st));
  }
  {
    KTimer t(c, KC_NYQ);
    CK(col_pass(g, d.yn, 1, 0, 0, nullptr, c->twN, nullptr, nullptr, st));
  }
  RowIn in = {{c->main, nullptr, nullptr}, {c->nyq, nullptr, nullptr}};
  {
    KTimer t(c, KC_XPASS);
    CK(row_pass(g, in, c->twN, c->twM, g.norm, 0, nullptr, c->partials, st));
  }
  {
    KTimer t(c, KC_SIGMA);
    CK(finish_sigma(c->partials, (int)c->npartials, (double)n * n * n, c->stats, st));
  }
  if (!s.p.do_rsd) {
    CK(cudaMemsetAsync(c->vr, 0, sizeof(float) * n * n * n, st));
    return GETHI_OK;
  }
  if (s.p.velocity_mode == 1) {
    // v_x = Y(i kx phi) -> C; v_y = Y(i ky phi) -> A; v_z = Y(i kz phi) in B
    {
      KTimer t(c, KC_YPASS);
      CK(col_pass(g, A.ym, 0, 4, 0, nullptr, c->twN, c->bC, nullptr, st));
    }
    {
      KTimer t(c, KC_NYQ);
      CK(col_pass(g, A.yn, 1, 4, 0, nullptr, c->twN, c->bCn, nullptr, st));
    }
    {
      KTimer t(c, KC_YPASS);
      CK(col_pass(g, A.ym, 0, 5, 0, nullptr, c->twN, nullptr, nullptr, st));
    }
    {
      KTimer t(c, KC_NYQ);
      CK(col_pass(g, A.yn, 1, 5, 0, nullptr, c->twN, nullptr, nullptr, st));
    }
    {
      KTimer t(c, KC_YPASS);
      CK(col_pass(g, B.ym, 0, 0, 0, nullptr, c->twN, nullptr, nullptr, st));
    }
    {
      KTimer t(c, KC_NYQ);
      CK(col_pass(g, B.yn, 1, 0, 0, nullptr, c->twN, nullptr, nullptr, st));
    }
    RowIn v = {{c->bC, c->bA, c->bB}, {c->bCn, c->bAn, c->bBn}};
    KTimer t(c, KC_XPASS_VEL);
    CK(row_pass(g, v, c->twN, c->twM, g.norm, 2, c->vr, nullptr, st));
  } else {
    {
      KTimer t(c, KC_YPASS);
      CK(col_pass(g, A.ym, 0, 0, 0, nullptr, c->twN, nullptr, nullptr, st));
    }
    {
      KTimer t(c, KC_NYQ);
      CK(col_pass(g, A.yn, 1, 0, 0, nullptr, c->twN, nullptr, nullptr, st));
    }
    RowIn v = {{c->bA, nullptr, nullptr}, {c->bAn, nullptr, nullptr}};
    {
      KTimer t(c, KC_XPASS);
      CK(row_pass(g, v, c->twN, c->twM, g.norm, 3, nullptr, nullptr, st));
    }
    KTimer t(c, KC_FDVEL);
    CK(radial_velocity_fd(g, reinterpret_cast<const float *>(c->bA), c->vr, st));
  }
  return GETHI_OK;
}

}  // namespace

extern "C" int gethi_gpu_init(const gethi_params *p, int device, gethi_ctx **out)
{
  if (!p || !out) return GETHI_E_ARG;
  *out = nullptr;
  if (!fft_supported(p->n_grid)) {
    set_error("n_grid " + std::to_string(p->n_grid) + " not supported (16,24,32,64,128,256,384,512,1024,2048)");
    return GETHI_E_ARG;
  }
  gethi_ctx *c = new gethi_ctx();
  std::string err;
  int rc = setup_build(*p, c->s, err);
  if (rc) {
    set_error(err);
    delete c;
    return rc;
  }
  c->device = device;
  cudaError_t e = cudaSetDevice(device);
  if (e != cudaSuccess) {
    delete c;
    return cuda_fail(e, "cudaSetDevice");
  }
  const Setup &s = c->s;
  const long n = s.p.n_grid, m = n / 2;
  const size_t ncell = (size_t)n * n * n;
  const long npix = 12 * s.p.n_side * s.p.n_side;
  c->npartials = row_pass_blocks((int)n);
  const bool va = s.p.do_rsd, vbc = s.p.do_rsd && s.p.velocity_mode == 1;
  if ((rc = dalloc(&c->main, ncell / 2)) || (rc = dalloc(&c->nyq, (size_t)n * n)) ||
      (va && ((rc = dalloc(&c->bA, ncell / 2)) || (rc = dalloc(&c->bAn, (size_t)n * n)))) ||
      (vbc && ((rc = dalloc(&c->bB, ncell / 2)) || (rc = dalloc(&c->bBn, (size_t)n * n)) ||
               (rc = dalloc(&c->bC, ncell / 2)) || (rc = dalloc(&c->bCn, (size_t)n * n)))) ||
      (rc = dalloc(&c->vr, ncell)) || (rc = dalloc(&c->maps, (size_t)npix * s.p.n_nu)) ||
      (rc = dalloc(&c->twN, (size_t)n)) || (rc = dalloc(&c->twM, (size_t)m)) ||
      (rc = dalloc(&c->partials, (size_t)c->npartials)) || (rc = dalloc(&c->stats, 4)) ||
      (rc = dalloc(&c->pk_f, (size_t)s.d.numk)) || (rc = dalloc(&c->logk_f, (size_t)s.d.numk)) ||
      (rc = dalloc(&c->tab_f, (size_t)kTabF * NZ)) || (rc = dalloc(&c->tab_d, (size_t)4 * NZ)) ||
      (rc = dalloc(&c->prefac, (size_t)s.p.n_nu)) || (rc = dalloc(&c->edges_f, (size_t)s.p.n_nu + 1)) ||
      (rc = dalloc(&c->edges_d, (size_t)s.p.n_nu + 1)) || (rc = dalloc(&c->counters, 16))) {
    gethi_gpu_free(c);
    return rc;
  }
  {  // double-float copies of the FP64 tables the key refinement reads
    if ((rc = dalloc(&c->tab_df, (size_t)2 * NZ)) || (rc = dalloc(&c->edges_df, (size_t)s.p.n_nu + 1))) {
      gethi_gpu_free(c);
      return rc;
    }
    auto split = [](double v) { const float h = (float)v; return make_float2(h, (float)(v - (double)h)); };
    std::vector<float2> t2(2 * NZ);
    for (int i = 0; i < NZ; i++) {
      t2[i] = split(s.z_r2z[i]);
      t2[NZ + i] = split(s.r_r2z[i]);
    }
    cudaMemcpy(c->tab_df, t2.data(), sizeof(float2) * t2.size(), cudaMemcpyHostToDevice);
    std::vector<float2> e2(s.p.n_nu + 1);
    for (int i = 0; i < s.p.n_nu; i++) e2[i] = split(s.nu0[i]);
    e2[s.p.n_nu] = split(s.nuf[s.p.n_nu - 1]);
    cudaMemcpy(c->edges_df, e2.data(), sizeof(float2) * e2.size(), cudaMemcpyHostToDevice);
  }
  if (s.p.do_psources) {
    const int ni = PS_NICDF;
    if ((rc = dalloc(&c->ps_acc, (size_t)2 * npix)) || (rc = dalloc(&c->maps_ps, (size_t)npix * s.p.n_nu)) ||
        (rc = dalloc(&c->ps_nz, (size_t)PS_NZ)) || (rc = dalloc(&c->ps_icdf, (size_t)ni + 1)) ||
        (rc = dalloc(&c->ps_chan, (size_t)2 * s.p.n_nu)) || (rc = dalloc(&c->ps_total, 1))) {
      gethi_gpu_free(c);
      return rc;
    }
    std::vector<float> v(s.ps_nz.begin(), s.ps_nz.end());
    cudaMemcpy(c->ps_nz, v.data(), sizeof(float) * v.size(), cudaMemcpyHostToDevice);
    v.assign(s.ps_icdf.begin(), s.ps_icdf.end());
    cudaMemcpy(c->ps_icdf, v.data(), sizeof(float) * v.size(), cudaMemcpyHostToDevice);
    v.assign(s.ps_chan.begin(), s.ps_chan.end());
    cudaMemcpy(c->ps_chan, v.data(), sizeof(float) * v.size(), cudaMemcpyHostToDevice);
    const double dx = s.d.l_box / n;
    c->psc.nz = c->ps_nz;
    c->psc.icdf = c->ps_icdf;
    c->psc.inv_dz = (float)(1.0 / s.ps_glob_dz);
    c->psc.z_max = (float)s.d.z_max;
    c->psc.cell_vol = (float)(dx * dx * dx);
    c->psc.nicdf = ni;
  }
  if (s.p.fft_precision == 1) {
    std::vector<uint16_t> bm;
    std::vector<float2> tw;
    if (!tc_tables((int)n, bm, tw)) {
      set_error("fft_precision=tc_split needs n_grid=1024");
      gethi_gpu_free(c);
      return GETHI_E_ARG;
    }
    if ((rc = dalloc(&c->tc_bmat, tc_table_bytes() / sizeof(uint4))) || (rc = dalloc(&c->tc_tw, tw.size()))) {
      gethi_gpu_free(c);
      return rc;
    }
    cudaMemcpy(c->tc_bmat, bm.data(), tc_table_bytes(), cudaMemcpyHostToDevice);
    cudaMemcpy(c->tc_tw, tw.data(), sizeof(float2) * tw.size(), cudaMemcpyHostToDevice);
  }
  // error flag of the bounded device-side waits (tensor-core passes, wait self-test)
  if ((rc = dalloc(&c->tc_err, 1))) {
    gethi_gpu_free(c);
    return rc;
  }
  cudaMemset(c->tc_err, 0, sizeof(int));
  // tables
  std::vector<float2> t;
  twiddles(t, (int)n);
  cudaMemcpy(c->twN, t.data(), sizeof(float2) * n, cudaMemcpyHostToDevice);
  twiddles(t, (int)m);
  cudaMemcpy(c->twM, t.data(), sizeof(float2) * m, cudaMemcpyHostToDevice);
  std::vector<float> f(s.d.numk);
  for (int i = 0; i < s.d.numk; i++) f[i] = (float)s.pk[i];
  cudaMemcpy(c->pk_f, f.data(), sizeof(float) * s.d.numk, cudaMemcpyHostToDevice);
  for (int i = 0; i < s.d.numk; i++) f[i] = (float)s.logk[i];
  cudaMemcpy(c->logk_f, f.data(), sizeof(float) * s.d.numk, cudaMemcpyHostToDevice);
  std::vector<double> td(4 * NZ);
  std::vector<float> tf(kTabF * NZ);
  for (int i = 0; i < NZ; i++) {
    td[i] = s.z_r2z[i];
    td[NZ + i] = s.r_r2z[i];
    td[2 * NZ + i] = s.gd[i];
    td[3 * NZ + i] = s.gv[i];
    tf[i] = (float)s.z_r2z[i];
    tf[NZ + i] = (float)s.gd[i];
    tf[2 * NZ + i] = (float)s.gv[i];
  }
  line_table(s, tf.data() + 3 * NZ);
  cudaMemcpy(c->tab_d, td.data(), sizeof(double) * 4 * NZ, cudaMemcpyHostToDevice);
  cudaMemcpy(c->tab_f, tf.data(), sizeof(float) * kTabF * NZ, cudaMemcpyHostToDevice);
  std::vector<double> ed(s.p.n_nu + 1);
  std::vector<float> ef(s.p.n_nu + 1), pf(s.p.n_nu);
  for (int i = 0; i < s.p.n_nu; i++) {
    ed[i] = s.nu0[i];
    pf[i] = (float)s.prefac[i];
  }
  ed[s.p.n_nu] = s.nuf[s.p.n_nu - 1];
  for (int i = 0; i <= s.p.n_nu; i++) ef[i] = (float)ed[i];
  cudaMemcpy(c->edges_d, ed.data(), sizeof(double) * (s.p.n_nu + 1), cudaMemcpyHostToDevice);
  cudaMemcpy(c->edges_f, ef.data(), sizeof(float) * (s.p.n_nu + 1), cudaMemcpyHostToDevice);
  cudaMemcpy(c->prefac, pf.data(), sizeof(float) * s.p.n_nu, cudaMemcpyHostToDevice);
  if ((e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking)) != cudaSuccess) {
    gethi_gpu_free(c);
    return cuda_fail(e, "cudaStreamCreate");
  }
  c->own_stream = true;
  for (int i = 0; i < 8; i++) cudaEventCreate(&c->ev[i]);
  for (int i = 0; i < 128; i++) cudaEventCreate(&c->kev[i]);
  fill_cfg(c);
  if ((e = cudaGetLastError()) != cudaSuccess) {
    gethi_gpu_free(c);
    return cuda_fail(e, "gethi_gpu_init");
  }
  *out = c;
  return GETHI_OK;
}

extern "C" void gethi_gpu_free(gethi_ctx *c)
{
  if (!c) return;
  cudaSetDevice(c->device);
  if (c->stream) cudaStreamSynchronize(c->stream);
  if (c->copy_stream) {
    cudaStreamSynchronize(c->copy_stream);
    cudaStreamDestroy(c->copy_stream);
  }
  for (int b = 0; b < 2; b++) {
    if (c->ev_done[b]) cudaEventDestroy(c->ev_done[b]);
    if (c->ev_copied[b]) cudaEventDestroy(c->ev_copied[b]);
  }
  void *bufs[] = {c->main, c->nyq, c->bA, c->bAn, c->bB, c->bBn, c->bC, c->bCn, c->modes, c->vr, c->pg, c->pgn,
                  c->tc_bmat, c->tc_tw, c->tc_err, c->tab_df, c->edges_df, c->maps_b[1], c->ps_acc, c->maps_ps, c->ps_nz, c->ps_icdf, c->ps_chan,
                  c->ps_total, c->maps, c->twN, c->twM, c->partials,
                  c->stats, c->pk_f, c->logk_f, c->tab_f, c->tab_d, c->prefac, c->edges_f, c->edges_d, c->counters};
  for (void *b : bufs)
    if (b) cudaFree(b);
  for (auto &ev : c->ev)
    if (ev) cudaEventDestroy(ev);
  for (auto &ev : c->kev)
    if (ev) cudaEventDestroy(ev);
  if (c->own_stream && c->stream) cudaStreamDestroy(c->stream);
  if (c->staging) cudaFreeHost(c->staging);
  if (c->fq) cudaFree(c->fq);
  delete c;
}

extern "C" int gethi_gpu_set_stream(gethi_ctx *c, void *stream)
{
  if (!c) return GETHI_E_ARG;
  if (c->own_stream && c->stream) {
    cudaStreamSynchronize(c->stream);
    cudaStreamDestroy(c->stream);
  }
  if (stream) {
    c->stream = (cudaStream_t)stream;
    c->own_stream = false;
  } else {
    CK(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
    c->own_stream = true;
  }
  return GETHI_OK;
}

extern "C" int gethi_gpu_get_derived(const gethi_ctx *c, gethi_derived *out)
{
  if (!c || !out) return GETHI_E_ARG;
  *out = c->s.d;
  if (c->stage >= 1) {
    double st[2];
    if (cudaMemcpy(st, c->stats, sizeof(st), cudaMemcpyDeviceToHost) == cudaSuccess) {
      out->mean_gauss = st[0];
      out->sigma2_gauss = st[1];
    }
  }
  return GETHI_OK;
}

extern "C" int gethi_gpu_make_fields(gethi_ctx *c, const float *modes_k)
{
  if (!c) return GETHI_E_ARG;
  CK(cudaSetDevice(c->device));
  const Setup &s = c->s;
  const long n = s.p.n_grid, h = n / 2 + 1;
  const float2 *src = nullptr;
  std::vector<float> host_modes;
  if (!modes_k && s.p.rng == 1) {  // mt_validation: the reference's own draws, made on the host
    host_modes.resize((size_t)2 * n * n * h);
    modes_mt(s, s.p.omp_threads_for_modes, host_modes.data());
    modes_k = host_modes.data();
  }
  if (modes_k) {
    if (!c->modes) {
      int rc = dalloc(&c->modes, (size_t)n * n * h);
      if (rc) return rc;
    }
    CK(cudaMemcpyAsync(c->modes, modes_k, sizeof(float2) * n * n * h, cudaMemcpyHostToDevice, c->stream));
    src = c->modes;
  }
  c->nev = 0;
  if (!src) {
    int rc = ensure_pg(c);
    if (rc) return rc;
  }
  record(c);
  int rc = fields_fft(c, src);
  if (rc) return rc;
  if (s.p.do_psources) {  // src/main_gh.c:55-58: on the Gaussian field, before get_HI
    rc = enqueue_psources(c, c->stream, nullptr);
    if (rc) return rc;
  }
  record(c);
  c->stage = 1;
  return GETHI_OK;
}

extern "C" int gethi_gpu_get_hi(gethi_ctx *c)
{
  if (!c) return GETHI_E_ARG;
  if (c->stage != 1) {
    set_error("get_hi needs the fields of gethi_gpu_make_fields");
    return GETHI_E_STATE;
  }
  CK(cudaSetDevice(c->device));
  {
    KTimer t(c, KC_GETHI);
    CK(get_hi(c->cfg, c->stats, reinterpret_cast<float *>(c->main), c->vr, c->stream));
  }
  c->stage = 2;
  return GETHI_OK;
}

// queue of the samples whose FP32 key needs the FP64 decision (first projection)
static int ensure_fq(gethi_ctx *c)
{
  if (c->fq) return GETHI_OK;
  const long cap = fallback_queue_capacity((int)c->s.p.n_grid);
  int rc = dalloc(reinterpret_cast<char **>(&c->fq), (size_t)cap * fallback_entry_bytes());
  if (rc) return rc;
  c->fq_cap = cap;
  return GETHI_OK;
}

// the tensor-core passes record an expired wait in tc_err (read after a
// synchronize); the flag is reported once, by the call whose work expired, and
// cleared, so the context serves the next call
static int check_tc(const gethi_ctx *c)
{
  if (!c->tc_err) return GETHI_OK;
  int flag = 0;
  CK(cudaMemcpy(&flag, c->tc_err, sizeof(int), cudaMemcpyDeviceToHost));
  if (flag) {
    CK(cudaMemset(c->tc_err, 0, sizeof(int)));
    set_error("a bounded device wait expired (tensor-core MMA completion or wait self-test)");
    return GETHI_E_CUDA;
  }
  return GETHI_OK;
}

extern "C" int gethi_gpu_wait_selftest(gethi_ctx *c, long limit_us)
{
  if (!c || limit_us < 1 || limit_us > 10000000) return GETHI_E_ARG;
  CK(cudaSetDevice(c->device));
  CK(wait_selftest(c->tc_err, (uint64_t)limit_us * 1000ull, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  return check_tc(c);
}

static int maps_common(gethi_ctx *c, float *maps_out, int fused)
{
  const Setup &s = c->s;
  const long npix = 12 * s.p.n_side * s.p.n_side;
  CK(cudaMemsetAsync(c->maps, 0, sizeof(float) * npix * s.p.n_nu, c->stream));
  CK(cudaMemsetAsync(c->counters, 0, sizeof(int) * 16, c->stream));
  int rq = ensure_fq(c);
  if (rq) return rq;
  {
    KTimer t(c, KC_PROJECT);
    CK(project(c->cfg, c->stats, reinterpret_cast<const float *>(c->main), c->vr, fused, c->maps, c->counters,
               c->fq, c->fq_cap, c->stream));
  }
  {
    KTimer t(c, KC_FIXUP);
    CK(fixup(c->cfg, c->fq, c->counters, c->fq_cap, c->maps, c->stream));
  }
  {
    KTimer t(c, KC_SCALE);
    CK(scale_maps(c->cfg, c->maps, c->stream));
  }
  record(c);
  if (maps_out) {
    CK(cudaMemcpyAsync(maps_out, c->maps, sizeof(float) * npix * s.p.n_nu, cudaMemcpyDeviceToHost, c->stream));
    record(c);
  }
  CK(cudaStreamSynchronize(c->stream));
  int rc = check_tc(c);
  if (rc) return rc;
  for (int i = 0; i + 1 < c->nev && i < 7; i++) cudaEventElapsedTime(&c->times[i], c->ev[i], c->ev[i + 1]);
  collect_kernel_times(c);
  return GETHI_OK;
}

extern "C" int gethi_gpu_make_maps(gethi_ctx *c, float *maps_out)
{
  if (!c) return GETHI_E_ARG;
  if (c->stage != 2) {
    set_error("make_maps needs the HI grids of gethi_gpu_get_hi");
    return GETHI_E_STATE;
  }
  CK(cudaSetDevice(c->device));
  if (c->nev == 0) record(c);
  return maps_common(c, maps_out, 0);
}

extern "C" int gethi_gpu_device_maps(const gethi_ctx *c, const float **maps, const float **maps_ps)
{
  if (!c || !maps) return GETHI_E_ARG;
  *maps = c->maps;
  if (maps_ps) *maps_ps = c->s.p.do_psources ? c->maps_ps : nullptr;
  return GETHI_OK;
}

extern "C" int gethi_gpu_run(gethi_ctx *c, float *maps_out)
{
  if (!c) return GETHI_E_ARG;
  int rc = gethi_gpu_make_fields(c, nullptr);
  if (rc) return rc;
  rc = maps_common(c, maps_out, 1);
  if (rc) return rc;
  c->stage = 3;  // mass is not materialised by the fused path
  if (c->s.p.write_maps && maps_out) return gethi_gpu_write_maps(c, maps_out);
  return GETHI_OK;
}

// ---------------------------------------------------------------------------
// Batches of realisations: enqueue-only realisations (no host synchronisation,
// no allocation), captured into one CUDA graph
// ---------------------------------------------------------------------------

// every lazily allocated buffer and the per-configuration set-up, so that a
// realisation only enqueues work
static int prepare(gethi_ctx *c)
{
  CK(cudaSetDevice(c->device));
  int rc = ensure_fq(c);
  if (!rc) rc = ensure_pg(c);
  if (!rc) CK(cudaStreamSynchronize(c->stream));
  return rc;
}

// one Philox realisation on stream st (fields, fused get_HI + projection, FP64
// key fix-up, channel scaling) and, maps_out != NULL, the maps copied to
// maps_out (device or page-locked host memory)
static int enqueue_realisation(gethi_ctx *c, unsigned int seed, float *maps_out, cudaStream_t st)
{
  const Setup &s = c->s;
  const size_t bytes = sizeof(float) * 12 * (size_t)s.p.n_side * s.p.n_side * s.p.n_nu;
  const cudaStream_t s0 = c->stream;
  const int prof = c->prof;
  const unsigned int seed0 = c->cfg.seed;
  c->stream = st;
  c->prof = 0;
  c->cfg.seed = seed;
  int rc = fields_fft(c, nullptr);
  auto step = [&](cudaError_t e, const char *what) {
    if (!rc && e != cudaSuccess) rc = cuda_fail(e, what);
  };
  step(cudaMemsetAsync(c->maps, 0, bytes, st), "memset maps");
  step(cudaMemsetAsync(c->counters, 0, sizeof(int) * 16, st), "memset counters");
  if (!rc)
    step(project(c->cfg, c->stats, reinterpret_cast<const float *>(c->main), c->vr, 1, c->maps, c->counters, c->fq,
                 c->fq_cap, st),
         "project");
  if (!rc) step(fixup(c->cfg, c->fq, c->counters, c->fq_cap, c->maps, st), "fixup");
  if (!rc) step(scale_maps(c->cfg, c->maps, st), "scale_maps");
  if (!rc && maps_out) step(cudaMemcpyAsync(maps_out, c->maps, bytes, cudaMemcpyDefault, st), "maps copy");
  c->launches += 3;
  c->stream = s0;
  c->prof = prof;
  c->cfg.seed = seed0;
  return rc;
}

extern "C" int gethi_gpu_run_batch(gethi_ctx *const *ctxs, int nctx, const int *job_ctx, const unsigned int *seeds,
                                   int njobs, float *const *maps_out, int use_graph, double *stats)
{
  if (!ctxs || nctx < 1 || !job_ctx || !seeds || njobs < 0) return GETHI_E_ARG;
  for (int k = 0; k < nctx; k++)
    if (!ctxs[k] || ctxs[k]->device != ctxs[0]->device || ctxs[k]->s.p.rng != 0 || ctxs[k]->s.p.do_psources) {
      set_error("run_batch: contexts must be valid, on one device, with rng=philox and no point sources");
      return GETHI_E_ARG;
    }
  for (int i = 0; i < njobs; i++)
    if (job_ctx[i] < 0 || job_ctx[i] >= nctx) {
      set_error("run_batch: job_ctx out of range");
      return GETHI_E_ARG;
    }
  CK(cudaSetDevice(ctxs[0]->device));
  for (int k = 0; k < nctx; k++) {
    int rc = prepare(ctxs[k]);
    if (rc) return rc;
  }
  // page-lock pageable host outputs for the duration of the call
  std::vector<void *> registered;
  if (maps_out)
    for (int i = 0; i < njobs; i++) {
      if (!maps_out[i]) continue;
      cudaPointerAttributes at;
      if (cudaPointerGetAttributes(&at, maps_out[i]) == cudaSuccess && at.type != cudaMemoryTypeUnregistered) continue;
      cudaGetLastError();
      const Setup &s = ctxs[job_ctx[i]]->s;
      const size_t bytes = sizeof(float) * 12 * (size_t)s.p.n_side * s.p.n_side * s.p.n_nu;
      if (cudaHostRegister(maps_out[i], bytes, cudaHostRegisterDefault) == cudaSuccess)
        registered.push_back(maps_out[i]);
      else
        cudaGetLastError();  // already page-locked
    }
  auto unregister = [&]() {
    for (void *p : registered) cudaHostUnregister(p);
  };
  long launches0 = 0;
  for (int k = 0; k < nctx; k++) launches0 += ctxs[k]->launches;

  cudaStream_t origin = nullptr;
  cudaEvent_t fork = nullptr, t0 = nullptr, t1 = nullptr;
  std::vector<cudaEvent_t> joins(nctx, nullptr);
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  int rc = GETHI_OK;
  auto cu = [&](cudaError_t e, const char *what) {
    if (!rc && e != cudaSuccess) rc = cuda_fail(e, what);
  };
  cu(cudaStreamCreateWithFlags(&origin, cudaStreamNonBlocking), "stream");
  cu(cudaEventCreateWithFlags(&fork, cudaEventDisableTiming), "event");
  cu(cudaEventCreate(&t0), "event");
  cu(cudaEventCreate(&t1), "event");
  for (int k = 0; k < nctx; k++) cu(cudaEventCreateWithFlags(&joins[k], cudaEventDisableTiming), "event");
  const auto c0 = std::chrono::steady_clock::now();
  double capture_ms = 0, nodes = 0;
  if (!rc) {
    if (use_graph) cu(cudaStreamBeginCapture(origin, cudaStreamCaptureModeThreadLocal), "begin capture");
    else cu(cudaEventRecord(t0, origin), "event");
    cu(cudaEventRecord(fork, origin), "fork");
    for (int k = 0; k < nctx; k++) cu(cudaStreamWaitEvent(ctxs[k]->stream, fork, 0), "fork wait");
    for (int i = 0; i < njobs && !rc; i++) {
      gethi_ctx *c = ctxs[job_ctx[i]];
      rc = enqueue_realisation(c, seeds[i], maps_out ? maps_out[i] : nullptr, c->stream);
    }
    for (int k = 0; k < nctx; k++) {
      cu(cudaEventRecord(joins[k], ctxs[k]->stream), "join");
      cu(cudaStreamWaitEvent(origin, joins[k], 0), "join wait");
    }
    if (use_graph) {
      cudaError_t e = cudaStreamEndCapture(origin, &graph);
      if (!rc && e != cudaSuccess) rc = cuda_fail(e, "end capture");
      if (!rc) cu(cudaGraphInstantiate(&exec, graph, 0), "instantiate");
      size_t nn = 0;
      if (!rc && cudaGraphGetNodes(graph, nullptr, &nn) == cudaSuccess) nodes = (double)nn;
      capture_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - c0).count();
      cu(cudaEventRecord(t0, origin), "event");
      if (!rc) cu(cudaGraphLaunch(exec, origin), "graph launch");
    }
    cu(cudaEventRecord(t1, origin), "event");
    cu(cudaStreamSynchronize(origin), "synchronize");
  }
  float run_ms = 0;
  if (!rc) cudaEventElapsedTime(&run_ms, t0, t1);
  for (int k = 0; k < nctx && !rc; k++) rc = check_tc(ctxs[k]);
  long launches1 = 0;
  for (int k = 0; k < nctx; k++) launches1 += ctxs[k]->launches;
  if (stats) {
    stats[0] = capture_ms;
    stats[1] = run_ms;
    stats[2] = nodes;
    stats[3] = (double)(launches1 - launches0);
  }
  if (exec) cudaGraphExecDestroy(exec);
  if (graph) cudaGraphDestroy(graph);
  for (cudaEvent_t e : joins)
    if (e) cudaEventDestroy(e);
  if (fork) cudaEventDestroy(fork);
  if (t0) cudaEventDestroy(t0);
  if (t1) cudaEventDestroy(t1);
  if (origin) cudaStreamDestroy(origin);
  unregister();
  for (int k = 0; k < nctx; k++) ctxs[k]->stage = 3;
  return rc;
}

// Pipelined realisations: the maps of realisation i go to the host on a copy
// stream while realisation i+1 computes into the other device buffer.
extern "C" int gethi_gpu_run_async(gethi_ctx *c, float *maps_out)
{
  if (!c) return GETHI_E_ARG;
  if (c->s.p.rng != 0) {
    set_error("run_async: needs rng=philox");
    return GETHI_E_ARG;
  }
  CK(cudaSetDevice(c->device));
  if (!c->copy_stream) {
    int rc = prepare(c);
    if (rc) return rc;
    const size_t nm = 12 * (size_t)c->s.p.n_side * c->s.p.n_side * c->s.p.n_nu;
    c->maps_b[0] = c->maps;
    if ((rc = dalloc(&c->maps_b[1], nm))) return rc;
    CK(cudaStreamCreateWithFlags(&c->copy_stream, cudaStreamNonBlocking));
    for (int b = 0; b < 2; b++) {
      CK(cudaEventCreateWithFlags(&c->ev_done[b], cudaEventDisableTiming));
      CK(cudaEventCreateWithFlags(&c->ev_copied[b], cudaEventDisableTiming));
    }
  }
  const int b = c->cur_buf;
  const size_t bytes = sizeof(float) * 12 * (size_t)c->s.p.n_side * c->s.p.n_side * c->s.p.n_nu;
  if (c->copied_pending[b]) CK(cudaStreamWaitEvent(c->stream, c->ev_copied[b], 0));  // buffer b is free again
  float *const keep = c->maps;
  c->maps = c->maps_b[b];
  int rc = enqueue_realisation(c, c->cfg.seed, nullptr, c->stream);
  if (!rc && c->s.p.do_psources) rc = enqueue_psources(c, c->stream, nullptr);
  c->maps = keep;
  if (rc) return rc;
  CK(cudaEventRecord(c->ev_done[b], c->stream));
  if (maps_out) {
    CK(cudaStreamWaitEvent(c->copy_stream, c->ev_done[b], 0));
    CK(cudaMemcpyAsync(maps_out, c->maps_b[b], bytes, cudaMemcpyDefault, c->copy_stream));
    CK(cudaEventRecord(c->ev_copied[b], c->copy_stream));
    c->copied_pending[b] = true;
  }
  c->cur_buf ^= 1;
  c->stage = 3;
  return GETHI_OK;
}

extern "C" int gethi_gpu_wait(gethi_ctx *c)
{
  if (!c) return GETHI_E_ARG;
  CK(cudaSetDevice(c->device));
  CK(cudaStreamSynchronize(c->stream));
  if (c->copy_stream) CK(cudaStreamSynchronize(c->copy_stream));
  c->copied_pending[0] = c->copied_pending[1] = false;
  return check_tc(c);
}

// Launch-shape autotuner: times each candidate (projection tile depth, column
// tile width) on this context's own workload and keeps the fastest.
extern "C" int gethi_gpu_autotune(gethi_ctx *c, int *choice, float *ms_out)
{
  if (!c) return GETHI_E_ARG;
  if (c->s.p.rng != 0) {
    set_error("autotune: needs rng=philox");
    return GETHI_E_ARG;
  }
  int rc = prepare(c);
  if (rc) return rc;
  const int n = c->s.p.n_grid;
  std::vector<std::pair<int, int>> cand;
  for (int zs : {4, 2, 1})
    if (n % (4 * zs) == 0 && n % 8 == 0)
      for (int cv : {0, 1})
        if (cv == 0 || n == 128 || n == 256 || n == 384) cand.push_back({zs, cv});
  if (cand.empty()) return GETHI_OK;
  cudaEvent_t a, b;
  CK(cudaEventCreate(&a));
  CK(cudaEventCreate(&b));
  const int zs0 = c->cfg.proj_zsteps, cv0 = c->cfg.col_variant;
  float best = 1e30f;
  std::pair<int, int> pick = cand[0];
  const int reps = n >= 768 ? 1 : 3;
  for (auto &cd : cand) {
    c->cfg.proj_zsteps = cd.first;
    c->cfg.col_variant = cd.second;
    rc = enqueue_realisation(c, c->cfg.seed, nullptr, c->stream);  // warm-up
    if (!rc) CK(cudaEventRecord(a, c->stream));
    for (int r = 0; r < reps && !rc; r++) rc = enqueue_realisation(c, c->cfg.seed + 1 + r, nullptr, c->stream);
    if (!rc) CK(cudaEventRecord(b, c->stream));
    if (!rc) CK(cudaEventSynchronize(b));
    if (rc) break;
    float ms = 0;
    cudaEventElapsedTime(&ms, a, b);
    ms /= reps;
    if (ms < best) {
      best = ms;
      pick = cd;
    }
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  if (rc) {
    c->cfg.proj_zsteps = zs0;
    c->cfg.col_variant = cv0;
    return rc;
  }
  c->cfg.proj_zsteps = pick.first;
  c->cfg.col_variant = pick.second;
  if (choice) {
    choice[0] = pick.first;
    choice[1] = pick.second;
  }
  if (ms_out) *ms_out = best;
  return check_tc(c);
}

extern "C" int gethi_gpu_set_launch(gethi_ctx *c, int proj_zsteps, int col_variant)
{
  if (!c || proj_zsteps < 0 || proj_zsteps > 4 || col_variant < 0 || col_variant > 2) return GETHI_E_ARG;
  c->cfg.proj_zsteps = proj_zsteps;
  c->cfg.col_variant = col_variant;
  return GETHI_OK;
}

extern "C" int gethi_gpu_write_maps(const gethi_ctx *c, const float *maps)
{
  if (!c || !maps) return GETHI_E_ARG;
  const Setup &s = c->s;
  const long npix = 12 * s.p.n_side * s.p.n_side;
  for (int i = 0; i < s.p.n_nu; i++) {
    char fn[600];
    std::snprintf(fn, sizeof(fn), "%s_%03d.fits", s.p.prefix_out, i + 1);  // src/io_gh.c:75
    if (write_fits_map(fn, maps + (size_t)i * npix, s.p.n_side)) {
      set_error(std::string("cannot write ") + fn);
      return GETHI_E_IO;
    }
  }
  if (s.p.do_psources) {  // <prefix>_ps_%03d.fits (src/io_gh.c:122-128)
    std::vector<float> ps((size_t)npix * s.p.n_nu);
    CK(cudaStreamSynchronize(c->stream));
    CK(cudaMemcpy(ps.data(), c->maps_ps, sizeof(float) * ps.size(), cudaMemcpyDeviceToHost));
    for (int i = 0; i < s.p.n_nu; i++) {
      char fn[600];
      std::snprintf(fn, sizeof(fn), "%s_ps_%03d.fits", s.p.prefix_out, i + 1);
      if (write_fits_map(fn, ps.data() + (size_t)i * npix, s.p.n_side)) {
        set_error(std::string("cannot write ") + fn);
        return GETHI_E_IO;
      }
    }
  }
  return GETHI_OK;
}

extern "C" int gethi_gpu_psources_maps(gethi_ctx *c, float *maps_out, long *nsources)
{
  if (!c) return GETHI_E_ARG;
  if (!c->s.p.do_psources) {
    set_error("psources_maps: do_psources=0");
    return GETHI_E_STATE;
  }
  if (c->stage < 1) {
    set_error("psources_maps needs the fields of gethi_gpu_make_fields");
    return GETHI_E_STATE;
  }
  CK(cudaSetDevice(c->device));
  CK(cudaStreamSynchronize(c->stream));
  const size_t bytes = sizeof(float) * 12 * (size_t)c->s.p.n_side * c->s.p.n_side * c->s.p.n_nu;
  if (maps_out) CK(cudaMemcpy(maps_out, c->maps_ps, bytes, cudaMemcpyDeviceToHost));
  if (nsources) {
    unsigned long long t = 0;
    CK(cudaMemcpy(&t, c->ps_total, sizeof(t), cudaMemcpyDeviceToHost));
    *nsources = (long)t;
  }
  return GETHI_OK;
}

extern "C" int gethi_gpu_psources_catalogue(gethi_ctx *c, long cap, long *cell, float *u_l, float *dz, int *pix,
                                            long *count)
{
  if (!c || cap < 0 || (cap > 0 && (!cell || !u_l || !dz || !pix))) return GETHI_E_ARG;
  if (!c->s.p.do_psources || (c->stage != 1 && c->stage != 3)) {
    set_error("psources_catalogue: needs do_psources=1 and the Gaussian fields (before get_HI)");
    return GETHI_E_STATE;
  }
  CK(cudaSetDevice(c->device));
  PsCatalogue cat{};
  const size_t m = cap > 0 ? (size_t)cap : 1;
  int rc = dalloc(&cat.count, 1);
  if (!rc) rc = dalloc(&cat.cell, m);
  if (!rc) rc = dalloc(&cat.u, m);
  if (!rc) rc = dalloc(&cat.dz, m);
  if (!rc) rc = dalloc(&cat.pix, m);
  cat.cap = cap;
  unsigned long long k = 0;
  if (!rc && cudaMemsetAsync(cat.count, 0, sizeof(unsigned long long), c->stream) != cudaSuccess) rc = GETHI_E_CUDA;
  if (!rc) rc = enqueue_psources(c, c->stream, &cat);
  if (!rc && cudaStreamSynchronize(c->stream) != cudaSuccess) rc = cuda_fail(cudaGetLastError(), "catalogue");
  if (!rc && cudaMemcpy(&k, cat.count, sizeof(k), cudaMemcpyDeviceToHost) != cudaSuccess) rc = GETHI_E_CUDA;
  const size_t got = (size_t)std::min<unsigned long long>(k, (unsigned long long)cap);
  if (!rc && got) {
    if (cudaMemcpy(cell, cat.cell, sizeof(long) * got, cudaMemcpyDeviceToHost) != cudaSuccess ||
        cudaMemcpy(u_l, cat.u, sizeof(float4) * got, cudaMemcpyDeviceToHost) != cudaSuccess ||
        cudaMemcpy(dz, cat.dz, sizeof(float) * got, cudaMemcpyDeviceToHost) != cudaSuccess ||
        cudaMemcpy(pix, cat.pix, sizeof(int) * got, cudaMemcpyDeviceToHost) != cudaSuccess)
      rc = GETHI_E_CUDA;
  }
  cudaFree(cat.count);
  cudaFree(cat.cell);
  cudaFree(cat.u);
  cudaFree(cat.dz);
  cudaFree(cat.pix);
  if (count) *count = (long)k;
  return rc;
}

extern "C" int gethi_gpu_download_grids(const gethi_ctx *c, float *dens, float *rvel)
{
  if (!c) return GETHI_E_ARG;
  const long n = c->s.p.n_grid;
  CK(cudaStreamSynchronize(c->stream));
  int rc = check_tc(c);
  if (rc) return rc;
  if (dens) CK(cudaMemcpy(dens, c->main, sizeof(float) * n * n * n, cudaMemcpyDeviceToHost));
  if (rvel) CK(cudaMemcpy(rvel, c->vr, sizeof(float) * n * n * n, cudaMemcpyDeviceToHost));
  return GETHI_OK;
}

extern "C" int gethi_gpu_upload_grids(gethi_ctx *c, const float *dens, const float *rvel, int stage)
{
  if (!c || stage < 1 || stage > 2) return GETHI_E_ARG;
  const long n = c->s.p.n_grid;
  CK(cudaStreamSynchronize(c->stream));
  if (dens) CK(cudaMemcpy(c->main, dens, sizeof(float) * n * n * n, cudaMemcpyHostToDevice));
  if (rvel) CK(cudaMemcpy(c->vr, rvel, sizeof(float) * n * n * n, cudaMemcpyHostToDevice));
  c->stage = stage;
  return GETHI_OK;
}

extern "C" int gethi_gpu_sample_keys(gethi_ctx *c, uint32_t *keys, int exact_fp64)
{
  if (!c || !keys) return GETHI_E_ARG;
  const long n = c->s.p.n_grid;
  uint32_t *dk = nullptr;
  int rc = dalloc(&dk, (size_t)n * n * n * NSUB);
  if (rc) return rc;
  cudaError_t e = cudaMemsetAsync(c->counters, 0, sizeof(int) * 16, c->stream);
  if (e == cudaSuccess) e = sample_keys(c->cfg, c->vr, dk, exact_fp64, c->counters, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  if (e == cudaSuccess) e = cudaMemcpy(keys, dk, sizeof(uint32_t) * n * n * n * NSUB, cudaMemcpyDeviceToHost);
  cudaFree(dk);
  if (e != cudaSuccess) return cuda_fail(e, "sample_keys");
  return GETHI_OK;
}

extern "C" int gethi_gpu_download_modes(gethi_ctx *c, float *modes_k)
{
  if (!c || !modes_k) return GETHI_E_ARG;
  const long n = c->s.p.n_grid, h = n / 2 + 1;
  int rc = ensure_pg(c);
  if (rc) return rc;
  float2 *d = nullptr;
  rc = dalloc(&d, (size_t)n * n * h);
  if (rc) return rc;
  cudaError_t e = gen_modes(c->cfg, d, FIELD_DENS, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  if (e == cudaSuccess) e = cudaMemcpy(modes_k, d, sizeof(float2) * n * n * h, cudaMemcpyDeviceToHost);
  cudaFree(d);
  if (e != cudaSuccess) return cuda_fail(e, "download_modes");
  return GETHI_OK;
}

extern "C" int gethi_gpu_stage_times(const gethi_ctx *c, float *ms, int n)
{
  if (!c || !ms) return GETHI_E_ARG;
  int k = c->nev > 0 ? c->nev - 1 : 0;
  for (int i = 0; i < n; i++) ms[i] = i < k ? c->times[i] : 0.f;
  return k;
}

extern "C" int gethi_gpu_profile(gethi_ctx *c, int on)
{
  if (!c) return GETHI_E_ARG;
  c->prof = on;
  c->nk = 0;
  for (int i = 0; i < GETHI_NKCLASS; i++) {
    c->ktime[i] = 0;
    c->kcount[i] = 0;
  }
  return GETHI_OK;
}

extern "C" int gethi_gpu_kernel_times(const gethi_ctx *c, double *ms, long *count, long *launches)
{
  if (!c) return GETHI_E_ARG;
  for (int i = 0; i < GETHI_NKCLASS; i++) {
    if (ms) ms[i] = c->ktime[i];
    if (count) count[i] = c->kcount[i];
  }
  if (launches) *launches = c->launches;
  return GETHI_NKCLASS;
}

extern "C" int gethi_gpu_fallback_count(const gethi_ctx *c, long *n)
{
  if (!c || !n) return GETHI_E_ARG;
  int v = 0;
  CK(cudaMemcpy(&v, c->counters, sizeof(int), cudaMemcpyDeviceToHost));
  *n = v;
  return GETHI_OK;
}

extern "C" int gethi_gpu_set_seed(gethi_ctx *c, unsigned int seed)
{
  if (!c) return GETHI_E_ARG;
  c->s.p.seed = seed;
  c->cfg.seed = seed;
  return GETHI_OK;
}

// Host inputs of one realisation (P(k), distance/growth tables, shell edges,
// channel factors) copied again from the host-side setup, through pinned
// staging, on the context's stream.  Returns the number of bytes copied.
extern "C" long gethi_gpu_upload_inputs(gethi_ctx *c)
{
  if (!c) return GETHI_E_ARG;
  const Setup &s = c->s;
  const int nk = s.d.numk, nn = s.p.n_nu;
  size_t bytes = sizeof(float) * (2 * nk + kTabF * NZ + nn + nn + 1) + sizeof(double) * (4 * NZ + nn + 1);
  if (!c->staging) {
    if (cudaHostAlloc(&c->staging, bytes, cudaHostAllocDefault) != cudaSuccess) {
      c->staging = nullptr;
      set_error("cudaHostAlloc of the input staging buffer failed");
      return GETHI_E_NOMEM;
    }
    char *p = (char *)c->staging;
    double *td = (double *)p;
    for (int i = 0; i < NZ; i++) {
      td[i] = s.z_r2z[i];
      td[NZ + i] = s.r_r2z[i];
      td[2 * NZ + i] = s.gd[i];
      td[3 * NZ + i] = s.gv[i];
    }
    double *ed = td + 4 * NZ;
    for (int i = 0; i < nn; i++) ed[i] = s.nu0[i];
    ed[nn] = s.nuf[nn - 1];
    float *f = (float *)(ed + nn + 1);
    for (int i = 0; i < nk; i++) f[i] = (float)s.pk[i];
    for (int i = 0; i < nk; i++) f[nk + i] = (float)s.logk[i];
    float *tf = f + 2 * nk;
    for (int i = 0; i < NZ; i++) {
      tf[i] = (float)s.z_r2z[i];
      tf[NZ + i] = (float)s.gd[i];
      tf[2 * NZ + i] = (float)s.gv[i];
    }
    line_table(s, tf + 3 * NZ);
    float *pf = tf + kTabF * NZ;
    for (int i = 0; i < nn; i++) pf[i] = (float)s.prefac[i];
    float *ef = pf + nn;
    for (int i = 0; i <= nn; i++) ef[i] = (float)ed[i];
  }
  cudaStream_t st = c->stream;
  char *p = (char *)c->staging;
  double *td = (double *)p, *ed = td + 4 * NZ;
  float *f = (float *)(ed + nn + 1), *tf = f + 2 * nk, *pf = tf + kTabF * NZ, *ef = pf + nn;
  CK(cudaMemcpyAsync(c->tab_d, td, sizeof(double) * 4 * NZ, cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(c->edges_d, ed, sizeof(double) * (nn + 1), cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(c->pk_f, f, sizeof(float) * nk, cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(c->logk_f, f + nk, sizeof(float) * nk, cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(c->tab_f, tf, sizeof(float) * kTabF * NZ, cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(c->prefac, pf, sizeof(float) * nn, cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(c->edges_f, ef, sizeof(float) * (nn + 1), cudaMemcpyHostToDevice, st));
  return (long)bytes;
}
