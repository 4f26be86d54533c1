// Host-side FP64 setup for the GB300 GetHI path.  See host.h.
#include "host.h"

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>

namespace gethi {

// --------------------------------------------------------------------------
// parameters
// --------------------------------------------------------------------------
}  // namespace gethi

extern "C" int gethi_params_default(gethi_params *p)
{
  if (!p) return GETHI_E_ARG;
  std::memset(p, 0, sizeof(*p));
  // src/io_gh.c:133-186
  std::snprintf(p->prefix_out, sizeof(p->prefix_out), "default");
  std::snprintf(p->pk_filename, sizeof(p->pk_filename), "default");
  std::snprintf(p->frequencies_filename, sizeof(p->frequencies_filename), "default");
  p->omega_M = 0.3;
  p->omega_L = 0.7;
  p->omega_B = 0.05;
  p->h = 0.7;
  p->w = -1.;
  p->ns = 0.96;
  p->sigma_8 = 0.83;
  p->r_smooth = 2.0;
  p->seed = 1234;
  p->n_side = 128;
  p->nu_max = 1050.;
  p->nu_min = 350.;
  p->n_nu = 150;
  p->n_grid = 512;
  p->do_psources = 0;
  // new keys: reference behaviour by default
  p->l_box = -1;
  p->bias_model = 0;
  p->b_HI = 1;
  p->do_rsd = 1;
  p->velocity_mode = 0;
  p->gaussianise = 0;
  p->fft_precision = 0;
  p->rng = 0;
  p->omp_threads_for_modes = 1;
  p->write_maps = 0;
  return GETHI_OK;
}

static bool parse_choice(const char *v, const char *a, const char *b, int *out)
{
  if (!std::strcmp(v, a) || !std::strcmp(v, "0")) { *out = 0; return true; }
  if (!std::strcmp(v, b) || !std::strcmp(v, "1")) { *out = 1; return true; }
  return false;
}

extern "C" int gethi_read_params(const char *ini_path, gethi_params *p)
{
  if (!ini_path || !p) return GETHI_E_ARG;
  gethi_params_default(p);
  FILE *fi = std::fopen(ini_path, "r");
  if (!fi) {
    gethi::set_error(std::string("Couldn't open file ") + ini_path);
    return GETHI_E_IO;
  }
  char s0[512];
  int line = 0;
  while (std::fgets(s0, sizeof(s0), fi)) {
    line++;
    if (s0[0] == '#' || s0[0] == '\n') continue;
    char s1[64], s2[256];
    if (std::sscanf(s0, "%63s %255s", s1, s2) != 2) {
      std::fclose(fi);
      gethi::set_error(std::string("Error reading file ") + ini_path + ", line " + std::to_string(line));
      return GETHI_E_IO;
    }
    // keys of src/io_gh.c:211-249
    if (!std::strcmp(s1, "prefix_out=")) std::snprintf(p->prefix_out, 256, "%s", s2);
    else if (!std::strcmp(s1, "pk_filename=")) std::snprintf(p->pk_filename, 256, "%s", s2);
    else if (!std::strcmp(s1, "omega_M=")) p->omega_M = std::atof(s2);
    else if (!std::strcmp(s1, "omega_L=")) p->omega_L = std::atof(s2);
    else if (!std::strcmp(s1, "omega_B=")) p->omega_B = std::atof(s2);
    else if (!std::strcmp(s1, "h=")) p->h = std::atof(s2);
    else if (!std::strcmp(s1, "w=")) p->w = std::atof(s2);
    else if (!std::strcmp(s1, "ns=")) p->ns = std::atof(s2);
    else if (!std::strcmp(s1, "sigma_8=")) p->sigma_8 = std::atof(s2);
    else if (!std::strcmp(s1, "r_smooth=")) p->r_smooth = std::atof(s2);
    else if (!std::strcmp(s1, "frequencies_filename=")) std::snprintf(p->frequencies_filename, 256, "%s", s2);
    else if (!std::strcmp(s1, "nu_min=")) p->nu_min = std::atof(s2);
    else if (!std::strcmp(s1, "nu_max=")) p->nu_max = std::atof(s2);
    else if (!std::strcmp(s1, "n_nu=")) p->n_nu = std::atoi(s2);
    else if (!std::strcmp(s1, "n_grid=")) p->n_grid = std::atoi(s2);
    else if (!std::strcmp(s1, "n_side=")) p->n_side = std::atoi(s2);
    else if (!std::strcmp(s1, "seed=")) p->seed = (unsigned)std::atoi(s2);
    else if (!std::strcmp(s1, "do_psources=")) p->do_psources = std::atoi(s2);
    // new keys
    else if (!std::strcmp(s1, "l_box=")) p->l_box = std::atof(s2);
    else if (!std::strcmp(s1, "b_HI=")) p->b_HI = std::atof(s2);
    else if (!std::strcmp(s1, "do_rsd=")) p->do_rsd = std::atoi(s2);
    else if (!std::strcmp(s1, "gaussianise=")) p->gaussianise = std::atoi(s2);
    else if (!std::strcmp(s1, "omp_threads_for_modes=")) p->omp_threads_for_modes = std::atoi(s2);
    else if (!std::strcmp(s1, "write_maps=")) p->write_maps = std::atoi(s2);
    else if (!std::strcmp(s1, "bias_model=") || !std::strcmp(s1, "velocity_mode=") ||
             !std::strcmp(s1, "fft_precision=") || !std::strcmp(s1, "rng=")) {
      int v = 0;
      bool ok = !std::strcmp(s1, "bias_model=")      ? parse_choice(s2, "fit", "const", &v)
                : !std::strcmp(s1, "velocity_mode=") ? parse_choice(s2, "fd", "spectral", &v)
                : !std::strcmp(s1, "fft_precision=") ? parse_choice(s2, "fp32", "tc_split", &v)
                                                     : parse_choice(s2, "philox", "mt_validation", &v);
      if (!ok) {
        std::fclose(fi);
        gethi::set_error(std::string("Bad value for ") + s1 + " " + s2);
        return GETHI_E_ARG;
      }
      if (!std::strcmp(s1, "bias_model=")) p->bias_model = v;
      else if (!std::strcmp(s1, "velocity_mode=")) p->velocity_mode = v;
      else if (!std::strcmp(s1, "fft_precision=")) p->fft_precision = v;
      else p->rng = v;
    } else
      std::fprintf(stderr, "CRIME: Unknown parameter %s\n", s1);  // io_gh.c:251
  }
  std::fclose(fi);
  return GETHI_OK;
}

namespace gethi {

// --------------------------------------------------------------------------
// quadrature: adaptive Gauss-Legendre, 20 nodes, to 1e-13 relative with an
// absolute floor of 1e-16 of the whole integral
// --------------------------------------------------------------------------
namespace {
struct GL {
  double x[20], w[20];
  GL()
  {
    const int n = 20;
    for (int i = 0; i < n; i++) {
      double xx = std::cos(M_PI * (i + 0.75) / (n + 0.5)), dp = 0;
      for (int it = 0; it < 100; it++) {
        double p0 = 1, p1 = xx;
        for (int k = 2; k <= n; k++) {
          double p2 = ((2 * k - 1) * xx * p1 - (k - 1) * p0) / k;
          p0 = p1;
          p1 = p2;
        }
        dp = n * (xx * p1 - p0) / (xx * xx - 1);
        double dx = p1 / dp;
        xx -= dx;
        if (std::fabs(dx) < 1e-16) break;
      }
      x[i] = xx;
      w[i] = 2 / ((1 - xx * xx) * dp * dp);
    }
  }
};
const GL &gl()
{
  static GL g;
  return g;
}

template <class F>
double panel(const F &f, double a, double b)
{
  const GL &g = gl();
  double h = 0.5 * (b - a), m = 0.5 * (b + a), s = 0;
  for (int i = 0; i < 20; i++) s += g.w[i] * f(m + h * g.x[i]);
  return s * h;
}

template <class F>
double adapt(const F &f, double a, double b, double whole, double epsabs, int depth)
{
  double m = 0.5 * (a + b);
  double l = panel(f, a, m), r = panel(f, m, b), s = l + r;
  if (depth >= 48 || std::fabs(s - whole) <= 1e-13 * std::fabs(s) + epsabs) return s;
  return adapt(f, a, m, l, epsabs, depth + 1) + adapt(f, m, b, r, epsabs, depth + 1);
}

template <class F>
double integrate(const F &f, double a, double b)
{
  double coarse = 0;
  for (int i = 0; i < 8; i++) coarse += panel(f, a + (b - a) * i / 8, a + (b - a) * (i + 1) / 8);
  return adapt(f, a, b, panel(f, a, b), 1e-16 * std::fabs(coarse), 0);
}

// integral over (-inf, b] with x = b - (1-t)/t
template <class F>
double integrate_lower_inf(const F &f, double b)
{
  auto g = [&](double t) { return f(b - (1 - t) / t) / (t * t); };
  const int NSEG = 64;
  double lo[NSEG + 1], hi[NSEG + 1], coarse = 0, acc = 0;
  lo[0] = 1e-12;
  hi[0] = 1e-3;
  for (int i = 0; i < NSEG; i++) {
    lo[i + 1] = 1e-3 + (1 - 1e-3) * i / NSEG;
    hi[i + 1] = 1e-3 + (1 - 1e-3) * (i + 1) / NSEG;
  }
  for (int i = 0; i <= NSEG; i++) coarse += panel(g, lo[i], hi[i]);
  for (int i = 0; i <= NSEG; i++) acc += adapt(g, lo[i], hi[i], panel(g, lo[i], hi[i]), 1e-16 * std::fabs(coarse), 0);
  return acc;
}

// --------------------------------------------------------------------------
// background cosmology (src/cosmo_mad.c:160-507)
// --------------------------------------------------------------------------
struct Background {
  double OM, OL, OK, w0;
  int ksign, normalDE, constantw;
  double a_eq, phorizon;

  double e2a3(double a) const
  {
    if (normalDE) return OM + OL * a * a * a + OK * a;
    return OM + OL * std::pow(a, -3 * w0) + OK * a;
  }
  double naHm1(double a) const { return std::sqrt(a / e2a3(a)); }
  double na2Hm1(double a) const { return 1 / std::sqrt(a * e2a3(a)); }
  double naHm3(double a) const
  {
    double d = std::sqrt(a / e2a3(a));
    return d * d * d;
  }
  double parthor(double aa) const  // cosmo_mad.c:260-289
  {
    double alim = 0.01 * a_eq;
    if (aa <= alim) return 2 * std::sqrt(aa / OM) * HMPC;
    double int0 = 2 * std::sqrt(alim / OM);
    return (int0 + integrate([this](double a) { return na2Hm1(a); }, alim, aa)) * HMPC;
  }
  double growth(double aa) const  // cosmo_mad.c:291-319
  {
    double alim = 0.01 * a_eq;
    double int0 = 0.4 * std::sqrt(alim * alim * alim * alim * alim / (OM * OM * OM));
    if (aa <= alim) return aa;
    double integral = integrate([this](double a) { return naHm3(a); }, alim, aa);
    return (int0 + integral) * 2.5 * OM / (aa * naHm1(aa));
  }
  double hubble(double aa) const { return std::sqrt(e2a3(aa) / (aa * aa * aa)) / HMPC; }
  double fgrowth(double aa) const  // cosmo_mad.c:385-409
  {
    double apow, coeff, Da = growth(aa);
    if (normalDE) {
      coeff = 0;
      apow = aa * aa * aa;
    } else {
      coeff = 1 + w0;
      apow = std::pow(aa, -3 * w0);
    }
    return 0.5 * (5 * OM * aa / Da - (3 * OM + 3 * coeff * OL * apow + 2 * OK * aa)) / (OM + OL * apow + OK * aa);
  }
  double chi(double aa) const { return phorizon - parthor(aa); }

  int set(double om, double ol, double ob, double w)  // cosmo_mad.c:411-507
  {
    OM = om;
    OL = ol;
    w0 = w;
    OK = 1 - OM - OL;
    constantw = 1;
    normalDE = std::fabs(w0 + 1) < 1e-6 ? 1 : 0;
    ksign = std::fabs(OK) < 1e-6 ? 0 : (OK > 0 ? -1 : 1);
    if (OM <= 0 || OM < ob || w0 > -0.333333) return -1;
    double aeqK = 1, aeqL = 1;
    if (ksign != 0) aeqK = OM / std::fabs(OK);
    if (OL != 0) aeqL = normalDE ? std::pow(OM / OL, 0.333) : std::pow(OM / OL, -1 / (3 * w0));
    a_eq = aeqK < aeqL ? aeqK : aeqL;
    phorizon = parthor(1);
    return 0;
  }
};

double wind_tophat(double x)  // src/cosmo.c:127-151
{
  if (x < 0.1)
    return 1. - 0.1 * x * x + 0.003571429 * x * x * x * x - 6.61376E-5 * x * x * x * x * x * x +
           7.51563E-7 * x * x * x * x * x * x * x * x;
  return 3 * (std::sin(x) - x * std::cos(x)) / (x * x * x);
}

bool load_table(const char *fn, std::vector<double> &a, std::vector<double> &b, int ncol)
{
  std::ifstream f(fn);
  if (!f) return false;
  std::string line;
  while (std::getline(f, line)) {
    std::istringstream is(line);
    double x, y;
    if (!(is >> x)) continue;
    if (ncol == 2) {
      if (!(is >> y)) return false;
      b.push_back(y);
    }
    a.push_back(x);
  }
  return !a.empty();
}

// Eisenstein & Hu (1998, ApJ 496:605) no-wiggle transfer function times k^ns.
void eh_nowiggle_table(const gethi_params &p, std::vector<double> &k, std::vector<double> &pk)
{
  const int nk = 1000;
  const double tcmb = 2.7255, theta = tcmb / 2.7;
  double om = p.omega_M, ob = p.omega_B, h = p.h;
  double omh2 = om * h * h, obh2 = ob * h * h, fb = ob / om;
  double s = 44.5 * std::log(9.83 / omh2) / std::sqrt(1 + 10 * std::pow(obh2, 0.75));
  double alpha = 1 - 0.328 * std::log(431 * omh2) * fb + 0.38 * std::log(22.3 * omh2) * fb * fb;
  k.resize(nk);
  pk.resize(nk);
  for (int i = 0; i < nk; i++) {
    double kk = std::pow(10.0, -4.0 + 5.0 * i / (nk - 1));
    double gamma = om * h * (alpha + (1 - alpha) / (1 + std::pow(0.43 * kk * h * s, 4)));
    double q = kk * theta * theta / gamma;
    double l0 = std::log(2 * M_E + 1.8 * q), c0 = 14.2 + 731.0 / (1 + 62.5 * q);
    double t = l0 / (l0 + c0 * q * q);
    k[i] = kk;
    pk[i] = std::pow(kk, p.ns) * t * t * 2e4;
  }
}
}  // namespace

thread_local std::string g_err;
void set_error(const std::string &e) { g_err = e; }

MT19937::MT19937(uint32_t seed)
{
  if (seed == 0) seed = 4357;
  mt[0] = seed;
  for (int i = 1; i < 624; i++) mt[i] = 1812433253u * (mt[i - 1] ^ (mt[i - 1] >> 30)) + (uint32_t)i;
  mti = 624;
}

uint32_t MT19937::next()
{
  if (mti >= 624) {
    for (int k = 0; k < 624; k++) {
      uint32_t y = (mt[k] & 0x80000000u) | (mt[(k + 1) % 624] & 0x7fffffffu);
      mt[k] = mt[(k + 397) % 624] ^ (y >> 1) ^ ((y & 1u) ? 0x9908b0dfu : 0u);
    }
    mti = 0;
  }
  uint32_t y = mt[mti++];
  y ^= y >> 11;
  y ^= (y << 7) & 0x9d2c5680u;
  y ^= (y << 15) & 0xefc60000u;
  y ^= y >> 18;
  return y;
}

double r_of_z(const Setup &s, double z)
{
  if (z <= 0) return 0;
  if (z >= s.z_z2r[NZ - 1]) return s.r_z2r[NZ - 1];
  int iz = (int)(z / DZ);
  return s.r_z2r[iz] + (s.r_z2r[iz + 1] - s.r_z2r[iz]) * (z - s.z_z2r[iz]) / DZ;
}

double z_of_r(const Setup &s, double r)
{
  if (r <= 0) return 0;
  if (r >= s.r_r2z[NZ - 1]) return s.z_r2z[NZ - 1];
  int ir = (int)(r * s.d.glob_idr);
  return s.z_r2z[ir] + (s.z_r2z[ir + 1] - s.z_r2z[ir]) * (r - s.r_r2z[ir]) * s.d.glob_idr;
}

double pk_linear0(const Setup &s, double lgk)
{
  int ik = (int)((lgk - s.d.logkmin) * s.d.idlogk);
  if (ik < 0) return s.pk[0] * std::pow(10, s.n_scal * (lgk - s.d.logkmin));
  if (ik < s.d.numk - 1) return s.pk[ik] + (lgk - s.logk[ik]) * (s.pk[ik + 1] - s.pk[ik]) * s.d.idlogk;
  // the reference reads one past the table for ik == numk-1 (src/cosmo.c:164-165);
  // the k^-3 tail is used instead
  return s.pk[s.d.numk - 1] * std::pow(10, -3 * (lgk - s.d.logkmax));
}

static double z_of_r_provisional(const Setup &s, double r)  // src/cosmo.c:27-38
{
  if (r <= 0) return 0;
  if (r >= s.r_z2r[NZ - 1]) return s.z_z2r[NZ - 1];
  int iz = 0;
  while (r >= s.r_z2r[iz]) iz++;
  return s.z_z2r[iz - 1] + (s.z_z2r[iz] - s.z_z2r[iz - 1]) * (r - s.r_z2r[iz - 1]) / (s.r_z2r[iz] - s.r_z2r[iz - 1]);
}

int setup_build(const gethi_params &p, Setup &s, std::string &err)
{
  s.p = p;
  std::memset(&s.d, 0, sizeof(s.d));
  if (p.n_grid < 4 || (p.n_grid & 1)) { err = "n_grid must be even and >= 4"; return GETHI_E_ARG; }
  if (p.n_side < 1 || p.n_side > 8192) { err = "n_side out of range"; return GETHI_E_ARG; }
  if (p.fft_precision == 1 && p.n_grid != 1024) {
    err = "fft_precision=tc_split: the tensor-core column transform is built for n_grid=1024";
    return GETHI_E_ARG;
  }
  if (p.gaussianise && p.rng != 0) {
    err = "gaussianise=1 draws its modes with rng=philox (the validation draws follow P(k) as the reference does)";
    return GETHI_E_ARG;
  }

  // frequency shells (src/io_gh.c:29-57); a file takes precedence as in the
  // reference's default build (-D_IRREGULAR_NUTABLE)
  s.nu0.clear();
  s.nuf.clear();
  bool regular = !p.frequencies_filename[0] || !std::strcmp(p.frequencies_filename, "default");
  if (!regular) {
    std::vector<double> e, dummy;
    if (!load_table(p.frequencies_filename, e, dummy, 1) || e.size() < 2) {
      err = std::string("Couldn't open file ") + p.frequencies_filename;
      return GETHI_E_IO;
    }
    for (size_t i = 0; i + 1 < e.size(); i++) {
      s.nu0.push_back(e[i]);
      s.nuf.push_back(e[i + 1]);
      if (e[i + 1] <= e[i]) { err = "Frequency bins don't make sense"; return GETHI_E_ARG; }
    }
    s.p.nu_min = s.nu0.front();
    s.p.nu_max = s.nuf.back();
    s.p.n_nu = (int)s.nu0.size();
  } else {
    if (p.n_nu < 1 || !(p.nu_max > p.nu_min)) { err = "bad regular frequency table"; return GETHI_E_ARG; }
    for (int i = 0; i < p.n_nu; i++) {
      s.nu0.push_back(p.nu_min + (p.nu_max - p.nu_min) * (i + 0.0) / p.n_nu);
      s.nuf.push_back(p.nu_min + (p.nu_max - p.nu_min) * (i + 1.0) / p.n_nu);
    }
  }
  if ((double)s.p.n_nu * 12.0 * p.n_side * p.n_side >= 4294967295.0) {
    err = "n_nu*12*n_side^2 must fit in 32 bits";
    return GETHI_E_ARG;
  }
  s.d.n_nu = s.p.n_nu;
  s.d.regular_nu = regular ? 1 : 0;

  // cosmo_set (src/cosmo.c:341-394)
  Background b;
  if (b.set(p.omega_M, p.omega_L, p.omega_B, p.w)) { err = "cosmological parameters rejected"; return GETHI_E_COSMO; }
  s.d.fgrowth_0 = b.fgrowth(1);
  s.d.hubble_0 = b.hubble(1);
  s.d.z_min = NU21 / s.p.nu_max - 1;
  s.d.z_max = NU21 / s.p.nu_min - 1;
  s.d.r_min = b.chi(1 / (1 + s.d.z_min));
  s.d.r_max = b.chi(1 / (1 + s.d.z_max));
  s.d.l_box = 2 * s.d.r_max * (1 + 2. / p.n_grid);
  if (p.l_box > 0) s.d.l_box = p.l_box;
  s.d.pos_obs = 0.5 * s.d.l_box;

  s.z_z2r.assign(NZ, 0);
  s.r_z2r.assign(NZ, 0);
  s.z_r2z.assign(NZ, 0);
  s.r_r2z.assign(NZ, 0);
  s.gd.assign(NZ, 0);
  s.gv.assign(NZ, 0);
  for (int ii = 0; ii < NZ; ii++) {
    double z = ((double)ii) * DZ;
    s.z_z2r[ii] = z;
    s.r_z2r[ii] = b.chi(1 / (1 + z));
  }
  if (s.z_z2r[NZ - 1] <= s.d.z_max || s.r_z2r[NZ - 1] <= s.d.r_max) { err = "OMG! (z range beyond tables)"; return GETHI_E_COSMO; }
  double growth0 = b.growth(1);
  s.d.glob_idr = (NZ - 1) / (s.r_z2r[NZ - 1] - s.r_z2r[0]);
  for (int ii = 0; ii < NZ; ii++) {
    double r = ii / s.d.glob_idr;
    double z = z_of_r_provisional(s, r);
    double a = 1 / (1 + z);
    s.z_r2z[ii] = z;
    s.r_r2z[ii] = r;
    double gz = b.growth(a) / growth0;
    double fz = b.fgrowth(a);
    double hz = b.hubble(a);
    s.gd[ii] = gz;
    s.gv[ii] = (gz * hz * fz) / (s.d.fgrowth_0 * s.d.hubble_0);
  }
  if (s.z_r2z[NZ - 1] <= s.d.z_max || s.r_r2z[NZ - 1] <= s.d.r_max) { err = "OMG! (r range beyond tables)"; return GETHI_E_COSMO; }

  // smoothing (src/io_gh.c:255-260)
  if (p.r_smooth > 0) {
    s.d.r2_smooth = std::pow(p.r_smooth, 2);
    s.d.do_smoothing = 1;
  } else {
    s.d.r2_smooth = p.r_smooth;
    s.d.do_smoothing = 0;
  }

  // P(k) (src/cosmo.c:306-339)
  std::vector<double> kk, pp;
  if (!std::strcmp(p.pk_filename, "EH")) eh_nowiggle_table(p, kk, pp);
  else if (!load_table(p.pk_filename, kk, pp, 2)) {
    err = std::string("Couldn't open file ") + p.pk_filename;
    return GETHI_E_IO;
  }
  s.d.numk = (int)kk.size();
  if (s.d.numk < 2) { err = "P(k) table too short"; return GETHI_E_IO; }
  s.logk.resize(kk.size());
  s.pk = pp;
  for (size_t i = 0; i < kk.size(); i++) s.logk[i] = std::log10(kk[i]);
  s.n_scal = p.ns;
  s.d.logkmin = s.logk[0];
  s.d.logkmax = s.logk[s.d.numk - 1];
  s.d.idlogk = (s.d.numk - 1) / (s.logk[s.d.numk - 1] - s.logk[0]);
  const double TWOPIPIINVLOGTEN = 0.1166503235296796;  // src/common_gh.h:31
  auto integrand = [&](double lgk) {
    double k = std::pow(10, lgk);
    double w = wind_tophat(k * 8);
    return TWOPIPIINVLOGTEN * pk_linear0(s, lgk) * k * k * k * w * w;
  };
  double s2 = integrate_lower_inf(integrand, s.d.logkmax);
  s.d.sigma8_in = std::sqrt(s2);
  s.d.pk_norm = p.sigma_8 * p.sigma_8 / s2;
  for (auto &v : s.pk) v *= s.d.pk_norm;

  // sub-sample offsets (src/pixelize.c:157-164)
  {
    MT19937 rng(p.seed);
    double lcell = s.d.l_box / p.n_grid;
    for (int i = 0; i < NSUB; i++) {
      s.xs[i] = lcell * (rng.uniform() - 0.5);
      s.ys[i] = lcell * (rng.uniform() - 0.5);
      s.zs[i] = lcell * (rng.uniform() - 0.5);
    }
  }

  // channel factors (src/pixelize.c:155, 246-261)
  double M2T = 90.057156 * p.omega_B * p.h * (12.0 * p.n_side * p.n_side) / (4 * M_PI);
  s.prefac.resize(s.p.n_nu);
  for (int inu = 0; inu < s.p.n_nu; inu++) {
    double dnu, nu;
    if (regular) {
      dnu = (s.p.nu_max - s.p.nu_min) / s.p.n_nu;
      nu = s.p.nu_min + (inu + 0.5) * dnu;
    } else {
      dnu = s.nuf[inu] - s.nu0[inu];
      nu = (s.nuf[inu] + s.nu0[inu]) * 0.5;
    }
    double r = r_of_z(s, NU21 / nu - 1);
    s.prefac[inu] = M2T / (r * r * dnu);
  }

  if (p.do_psources) setup_psources(s);

  // fraction of the shell volume [r_min, r_max] inside the box (for reporting)
  {
    const int ns = 64;
    double in = 0, tot = 0, half = 0.5 * s.d.l_box;
    for (int ir = 0; ir < ns; ir++) {
      double r = s.d.r_min + (s.d.r_max - s.d.r_min) * (ir + 0.5) / ns;
      for (int it = 0; it < ns; it++) {
        double ct = -1 + 2 * (it + 0.5) / ns, st = std::sqrt(1 - ct * ct);
        for (int ip = 0; ip < ns; ip++) {
          double ph = 2 * M_PI * (ip + 0.5) / ns;
          double x = r * st * std::cos(ph), y = r * st * std::sin(ph), z = r * ct;
          double wgt = r * r;
          tot += wgt;
          if (std::fabs(x) < half && std::fabs(y) < half && std::fabs(z) < half) in += wgt;
        }
      }
    }
    s.d.filled_fraction = in / tot;
  }
  return GETHI_OK;
}

// --------------------------------------------------------------------------
// validation modes (src/fourier.c:234-305, drawn as the reference draws them)
// --------------------------------------------------------------------------
void modes_mt(const Setup &s, int nthreads, float *dens_k)
{
  const int n = s.p.n_grid, h = n / 2 + 1;
  const double dk = 2 * M_PI / s.d.l_box, idk3 = 1. / (dk * dk * dk);
  if (nthreads < 1) nthreads = 1;
  auto kval = [&](int i) { return (2 * i <= n) ? i * dk : -(n - i) * dk; };
  for (int t = 0; t < nthreads; t++) {
    // libgomp static schedule: contiguous blocks, the first n%T threads get one more plane
    int q = n / nthreads, r = n % nthreads, i0;
    if (t < r) {
      q++;
      i0 = q * t;
    } else
      i0 = q * t + r;
    MT19937 rng(s.p.seed + (unsigned)t);
    for (int ii = i0; ii < i0 + q; ii++) {
      double kz = kval(ii);
      for (int jj = 0; jj < n; jj++) {
        double ky = kval(jj);
        for (int kk = 0; kk <= n / 2; kk++) {
          double kx = kval(kk);
          size_t idx = kk + (size_t)h * (jj + (size_t)n * ii);
          double k2 = kx * kx + ky * ky + kz * kz;
          if (k2 <= 0) {
            dens_k[2 * idx] = dens_k[2 * idx + 1] = 0;
            continue;
          }
          double lgk = 0.5 * std::log10(k2);
          double sigma2 = pk_linear0(s, lgk) * idk3;
          if (s.d.do_smoothing) sigma2 *= std::exp(-s.d.r2_smooth * k2);
          double phase = 2 * M_PI * rng.uniform();
          double u = rng.uniform();
          double mod = std::sqrt(-sigma2 * std::log(1 - u));
          dens_k[2 * idx] = (float)(mod * std::cos(phase));
          dens_k[2 * idx + 1] = (float)(mod * std::sin(phase));
        }
      }
    }
  }
}

// --------------------------------------------------------------------------
// FITS output (src/io_gh.c:69-82, src/healpix_extra.c:132-164): one binary
// table HDU, column T (1E, mK), PIXTYPE=HEALPIX ORDERING=RING NSIDE COORDSYS=G
// --------------------------------------------------------------------------
namespace {
void card(std::string &h, const char *key, const std::string &val, const char *comment)
{
  char buf[81];
  if (val.empty())
    std::snprintf(buf, sizeof(buf), "%-80s", key);
  else if (comment && *comment)
    std::snprintf(buf, sizeof(buf), "%-8s= %20s / %-47s", key, val.c_str(), comment);
  else
    std::snprintf(buf, sizeof(buf), "%-8s= %20s", key, val.c_str());
  std::string c(buf);
  c.resize(80, ' ');
  h += c;
}
std::string sq(const char *s)
{
  std::string v = std::string("'") + s;
  while (v.size() < 9) v += ' ';
  return v + "'";
}
std::string sql(const char *s)  // left-justified string value
{
  std::string v = sq(s);
  while (v.size() < 20) v += ' ';
  return v;
}
void pad_block(std::string &h, char fill)
{
  while (h.size() % 2880) h += fill;
}
}  // namespace

int write_fits_map(const char *fname, const float *map, long nside)
{
  long npix = 12 * nside * nside;
  std::string h0;
  card(h0, "SIMPLE", "T", "conforms to FITS standard");
  card(h0, "BITPIX", "8", "array data type");
  card(h0, "NAXIS", "0", "number of array dimensions");
  card(h0, "EXTEND", "T", "");
  card(h0, "END", "", nullptr);
  pad_block(h0, ' ');
  std::string h1;
  card(h1, "XTENSION", sql("BINTABLE"), "binary table extension");
  card(h1, "BITPIX", "8", "8-bit bytes");
  card(h1, "NAXIS", "2", "2-dimensional binary table");
  card(h1, "NAXIS1", "4", "width of table in bytes");
  card(h1, "NAXIS2", std::to_string(npix), "number of rows in table");
  card(h1, "PCOUNT", "0", "size of special data area");
  card(h1, "GCOUNT", "1", "one data group (required keyword)");
  card(h1, "TFIELDS", "1", "number of fields in each row");
  card(h1, "TTYPE1", sql("T"), "label for field   1");
  card(h1, "TFORM1", sql("1E"), "data format of field: 4-byte REAL");
  card(h1, "TUNIT1", sql("mK"), "physical unit of field");
  card(h1, "EXTNAME", sql("BINTABLE"), "name of this binary table extension");
  card(h1, "PIXTYPE", sql("HEALPIX"), "HEALPIX Pixelisation");
  card(h1, "ORDERING", sql("RING"), "Pixel ordering scheme, either RING or NESTED");
  card(h1, "NSIDE", std::to_string(nside), "Resolution parameter for HEALPIX");
  card(h1, "COORDSYS", sql("G"), "Pixelisation coordinate system");
  {
    char buf[81];
    std::snprintf(buf, sizeof(buf), "COMMENT G = Galactic, E = ecliptic, C = celestial = equatorial");
    std::string c(buf);
    c.resize(80, ' ');
    h1 += c;
  }
  card(h1, "END", "", nullptr);
  pad_block(h1, ' ');
  std::string data(npix * 4, '\0');
  for (long i = 0; i < npix; i++) {
    uint32_t u;
    std::memcpy(&u, &map[i], 4);
    data[4 * i + 0] = (char)(u >> 24);
    data[4 * i + 1] = (char)(u >> 16);
    data[4 * i + 2] = (char)(u >> 8);
    data[4 * i + 3] = (char)u;
  }
  pad_block(data, '\0');
  FILE *f = std::fopen(fname, "wb");
  if (!f) return GETHI_E_IO;
  bool ok = std::fwrite(h0.data(), 1, h0.size(), f) == h0.size() && std::fwrite(h1.data(), 1, h1.size(), f) == h1.size() &&
            std::fwrite(data.data(), 1, data.size(), f) == data.size();
  ok = (std::fclose(f) == 0) && ok;
  return ok ? GETHI_OK : GETHI_E_IO;
}

// ---- point sources ----
namespace {
constexpr double kLLogMin = -5., kLLogMax = 6.;                 // src/psources.c:25-26
constexpr double kLX = 2.11, kAlpha = -0.633, kRho = 3.2E-4;    // src/psources.c:33-35
constexpr double kSedNorm = 0.114461;                           // src/psources.c:54
constexpr double kFlux2Temp = 3.2548291E-2, kLum2Flux = 8.35774E7;  // src/psources.c:154-155

// dn(z, L)/dlog10(L), L in 1e22 W/Hz (src/psources.c:39-52)
double l_z_function(double L, double z)
{
  double rho_l = 2.5 * M_LN10 * kRho * std::pow(L / kLX, kAlpha + 1) * std::exp(-L / kLX);
  double fz = z < 1.5 ? std::pow(1 + z, 3.1) : 17.124;
  return fz * rho_l;
}
}  // namespace

void setup_psources(Setup &s)
{
  // n(z) on NZ_PSOURCES bins of z_max / 256 and the rejection bound (src/psources.c:98-124)
  const int NL = 256;
  const double dlogL = (kLLogMax - kLLogMin) / NL;
  s.ps_glob_dz = s.d.z_max / PS_NZ;
  s.ps_nz.assign(PS_NZ, 0.0);
  s.ps_maxpdf.assign(PS_NZ, 0.0);
  for (int ii = 0; ii < PS_NZ; ii++) {
    double z = ii * s.ps_glob_dz, max_dist = -1;
    for (int jj = 0; jj < NL; jj++) {
      double lfunc = l_z_function(std::pow(10., kLLogMin + (jj + 0.5) * dlogL), z);
      if (lfunc >= max_dist) max_dist = lfunc;
      s.ps_nz[ii] += dlogL * lfunc;
    }
    s.ps_maxpdf[ii] = s.ps_nz[ii] > 0 ? 1.1 * max_dist / s.ps_nz[ii] : 0;
  }
  // The reference draws log10 L by rejection with density proportional to
  // l_z_function(L, z) on [-5, 6] (src/psources.c:126-152).  Its z factor cancels,
  // so one inverse CDF serves every redshift: CDF by the trapezoid rule on a fine
  // grid, inverted at PS_NICDF + 1 equally spaced probabilities.
  const int M = 1 << 18;
  std::vector<double> cdf(M + 1, 0.0);
  double prev = l_z_function(std::pow(10., kLLogMin), 0.0);
  for (int i = 1; i <= M; i++) {
    double f = l_z_function(std::pow(10., kLLogMin + (kLLogMax - kLLogMin) * i / M), 0.0);
    cdf[i] = cdf[i - 1] + 0.5 * (prev + f);
    prev = f;
  }
  s.ps_icdf.assign(PS_NICDF + 1, 0.0);
  int j = 0;
  for (int q = 0; q <= PS_NICDF; q++) {
    double target = cdf[M] * q / PS_NICDF;
    while (j < M && cdf[j + 1] < target) j++;
    double t = (j < M && cdf[j + 1] > cdf[j]) ? (target - cdf[j]) / (cdf[j + 1] - cdf[j]) : 0.0;
    if (t > 1) t = 1;
    s.ps_icdf[q] = kLLogMin + (kLLogMax - kLLogMin) * (j + t) / M;
  }
  s.ps_icdf[0] = kLLogMin;
  s.ps_icdf[PS_NICDF] = kLLogMax;
  // temp_of_l (src/psources.c:158-167) with spec_ed (src/psources.c:55-63) is
  //   T = K L0 [(1+z)^-0.1 nu_GHz^-0.1 + 10 (1+z)^-0.75 nu_GHz^-0.75] / (r^2 (1+z) nu^2),
  //   K = FLUX2TEMP LUM2FLUX 4 pi SED_NORM h^2 / dOmega,
  // so per pixel S1 = sum L0 (1+z)^-1.1 / r^2 and S2 = sum 10 L0 (1+z)^-1.75 / r^2
  // give every channel: T(nu) = a(nu) S1 + b(nu) S2.  Channel centres as in
  // src/pixelize.c:64-71.
  const double npix = 12.0 * s.p.n_side * s.p.n_side, dOmega = 4 * M_PI / npix;
  const double K = kFlux2Temp * kLum2Flux * 4 * M_PI * kSedNorm * s.p.h * s.p.h / dOmega;
  const bool regular = s.d.regular_nu != 0;
  s.ps_chan.assign(2 * (size_t)s.p.n_nu, 0.0);
  for (int inu = 0; inu < s.p.n_nu; inu++) {
    double nu = regular ? s.p.nu_min + (s.p.nu_max - s.p.nu_min) * (inu + 0.5) / s.p.n_nu
                        : (s.nu0[inu] + s.nuf[inu]) * 0.5;
    double ng = nu * 0.001;
    s.ps_chan[2 * inu] = K * std::pow(ng, -0.1) / (nu * nu);
    s.ps_chan[2 * inu + 1] = K * std::pow(ng, -0.75) / (nu * nu);
  }
}

}  // namespace gethi

extern "C" int gethi_host_psources(const gethi_params *p, double *nz_arr, double *maxpdf, double *glob_dz,
                                   double *logl_icdf)
{
  if (!p) return GETHI_E_ARG;
  gethi_params q = *p;
  q.do_psources = 1;
  gethi::Setup s;
  std::string err;
  int rc = gethi::setup_build(q, s, err);
  if (rc) {
    gethi::set_error(err);
    return rc;
  }
  if (nz_arr) std::memcpy(nz_arr, s.ps_nz.data(), sizeof(double) * gethi::PS_NZ);
  if (maxpdf) std::memcpy(maxpdf, s.ps_maxpdf.data(), sizeof(double) * gethi::PS_NZ);
  if (glob_dz) *glob_dz = s.ps_glob_dz;
  if (logl_icdf) std::memcpy(logl_icdf, s.ps_icdf.data(), sizeof(double) * (gethi::PS_NICDF + 1));
  return GETHI_OK;
}

extern "C" const char *gethi_last_error(void) { return gethi::g_err.c_str(); }

extern "C" int gethi_host_setup(const gethi_params *p, gethi_derived *d, double *tables, double *logk, double *pk,
                                double *offsets, double *prefac)
{
  if (!p) return GETHI_E_ARG;
  gethi::Setup s;
  std::string err;
  int rc = gethi::setup_build(*p, s, err);
  if (rc) {
    gethi::set_error(err);
    return rc;
  }
  if (d) *d = s.d;
  const int NZ = gethi::NZ;
  if (tables) {
    const std::vector<double> *t[6] = {&s.z_z2r, &s.r_z2r, &s.z_r2z, &s.r_r2z, &s.gd, &s.gv};
    for (int k = 0; k < 6; k++) std::memcpy(tables + k * NZ, t[k]->data(), sizeof(double) * NZ);
  }
  if (logk) std::memcpy(logk, s.logk.data(), sizeof(double) * s.logk.size());
  if (pk) std::memcpy(pk, s.pk.data(), sizeof(double) * s.pk.size());
  if (offsets)
    for (int i = 0; i < gethi::NSUB; i++) {
      offsets[3 * i] = s.xs[i];
      offsets[3 * i + 1] = s.ys[i];
      offsets[3 * i + 2] = s.zs[i];
    }
  if (prefac) std::memcpy(prefac, s.prefac.data(), sizeof(double) * s.prefac.size());
  return GETHI_OK;
}

extern "C" int gethi_host_modes_mt(const gethi_params *p, int nthreads, float *out)
{
  if (!p || !out) return GETHI_E_ARG;
  gethi::Setup s;
  std::string err;
  int rc = gethi::setup_build(*p, s, err);
  if (rc) {
    gethi::set_error(err);
    return rc;
  }
  gethi::modes_mt(s, nthreads, out);
  return GETHI_OK;
}
