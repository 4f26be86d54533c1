// Host side of JoinT: the param_JoinT .ini (src/io_jt.c:86-186), the frequency
// table (src/io_jt.c:215-241), HEALPix FITS maps in and out
// (src/healpix_extra.c:132-224, src/io_jt.c:25-80), the instrument table
// (src/main_jt.c:28-72) and the whole run (src/main_jt.c:326-389) over the
// joint_gpu_* stages.
#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <ctime>
#include <string>
#include <vector>

#include "../../include/joint_gpu.h"
#include "healpix.h"
#include "host.h"

using namespace gethi;

namespace {

constexpr double kPrefacFwhm = 1030610.55;  // src/main_jt.c:26
constexpr double kPrefacTnu = 3.6e9;        // src/main_jt.c:25

// ---- FITS (binary table of E/D columns) ----
struct Cards {
  std::vector<std::string> c;
  const char *get(const char *key) const
  {
    const size_t kl = std::strlen(key);
    for (const auto &s : c)
      if (s.compare(0, kl, key) == 0 && (s.size() <= kl || s[kl] == ' ' || s[kl] == '=') && s.size() > 9 &&
          s[8] == '=')
        return s.c_str() + 10;
    return nullptr;
  }
  long num(const char *key, long dflt) const
  {
    const char *v = get(key);
    return v ? std::atol(v) : dflt;
  }
  std::string str(const char *key) const
  {
    const char *v = get(key);
    if (!v) return "";
    const char *a = std::strchr(v, '\'');
    if (!a) return "";
    const char *b = std::strchr(a + 1, '\'');
    if (!b) return "";
    std::string s(a + 1, b);
    while (!s.empty() && s.back() == ' ') s.pop_back();
    return s;
  }
};

bool read_header(FILE *f, Cards &h)
{
  char block[2880];
  for (;;) {
    if (std::fread(block, 1, 2880, f) != 2880) return false;
    for (int i = 0; i < 36; i++) {
      std::string card(block + 80 * i, 80);
      if (card.compare(0, 8, "END     ") == 0) return true;
      h.c.push_back(card);
    }
  }
}

double be_read(const unsigned char *p, char type)
{
  if (type == 'D') {
    uint64_t u = 0;
    for (int i = 0; i < 8; i++) u = (u << 8) | p[i];
    double d;
    std::memcpy(&d, &u, 8);
    return d;
  }
  uint32_t u = 0;
  for (int i = 0; i < 4; i++) u = (u << 8) | p[i];
  float x;
  std::memcpy(&x, &u, 4);
  return x;
}

int io_error(const std::string &m)
{
  set_error(m);
  return GETHI_E_IO;
}

}  // namespace

extern "C" int joint_host_read_map(const char *path, int column, long *nside, float *out)
{
  if (!path || !nside || column < 0) return GETHI_E_ARG;
  FILE *f = std::fopen(path, "rb");
  if (!f) return io_error(std::string("Couldn't open file ") + path);
  Cards h0, h1;
  if (!read_header(f, h0)) {
    std::fclose(f);
    return io_error(std::string("not a FITS file: ") + path);
  }
  long skip = 0;  // primary data, if any
  const long nax0 = h0.num("NAXIS", 0);
  if (nax0 > 0) {
    skip = std::labs(h0.num("BITPIX", 8)) / 8;
    for (long i = 1; i <= nax0; i++) skip *= h0.num(("NAXIS" + std::to_string(i)).c_str(), 0);
    skip = (skip + 2879) / 2880 * 2880;
  }
  if (skip) std::fseek(f, skip, SEEK_CUR);
  if (!read_header(f, h1)) {
    std::fclose(f);
    return io_error(std::string("no table extension in ") + path);
  }
  const long row_bytes = h1.num("NAXIS1", 0), nrows = h1.num("NAXIS2", 0), ncols = h1.num("TFIELDS", 0);
  *nside = h1.num("NSIDE", 0);
  const long npix = 12 * (*nside) * (*nside);
  if (*nside < 1 || ncols < 1 || nrows < 1 || npix % nrows != 0) {  // src/healpix_extra.c:183-186
    std::fclose(f);
    return io_error(std::string("not a HEALPix map table: ") + path);
  }
  if (column >= ncols) {
    std::fclose(f);
    return io_error(std::string("column ") + std::to_string(column + 1) + " missing in " + path);
  }
  long off = 0, rep = 0;
  char type = 0;
  for (long c = 0; c <= column; c++) {
    const std::string tf = h1.str(("TFORM" + std::to_string(c + 1)).c_str());
    long r = 1;
    size_t k = 0;
    if (!tf.empty() && std::isdigit((unsigned char)tf[0])) {
      r = std::atol(tf.c_str());
      while (k < tf.size() && std::isdigit((unsigned char)tf[k])) k++;
    }
    const char t = k < tf.size() ? tf[k] : 'E';
    const long sz = t == 'D' ? 8 : t == 'E' ? 4 : (t == 'J' ? 4 : (t == 'K' ? 8 : (t == 'I' ? 2 : 1)));
    if (c == column) {
      rep = r;
      type = t;
    } else {
      off += r * sz;
    }
  }
  if (type != 'E' && type != 'D') {
    std::fclose(f);
    return io_error(std::string("column type ") + type + " of " + path + " is not E or D");
  }
  if (rep * nrows != npix) {
    std::fclose(f);
    return io_error(std::string("column size does not match NSIDE in ") + path);
  }
  if (!out) {
    std::fclose(f);
    return GETHI_OK;
  }
  std::vector<unsigned char> data((size_t)row_bytes * nrows);
  if (std::fread(data.data(), 1, data.size(), f) != data.size()) {
    std::fclose(f);
    return io_error(std::string("truncated table in ") + path);
  }
  std::fclose(f);
  const int sz = type == 'D' ? 8 : 4;
  const bool nested = h1.str("ORDERING").compare(0, 4, "NEST") == 0;
  for (long row = 0, e = 0; row < nrows; row++)
    for (long k = 0; k < rep; k++, e++) {
      const float v = (float)be_read(data.data() + row * row_bytes + off + k * sz, type);
      if (nested) out[hpx::nest2ring(*nside, e)] = v;  // src/healpix_extra.c:209-219
      else out[e] = v;
    }
  return GETHI_OK;
}

extern "C" int joint_host_read_ini(const char *path, joint_ini *o)
{
  if (!path || !o) return GETHI_E_ARG;
  std::memset(o, 0, sizeof(*o));
  // defaults of src/common_jt.c:27-51
  for (char *s : {o->prefix_cosmo, o->prefix_synchrotron, o->prefix_galactic_freefree,
                  o->prefix_extragalactic_freefree, o->prefix_point_sources, o->prefix_out, o->fname_nutable,
                  o->fname_mask})
    std::snprintf(s, 256, "default");
  std::snprintf(o->prefix_custom, 256, "custom");
  o->seed_signed = -1;
  o->nside = -1;
  o->polarization_leakage = -1;
  o->dish_diameter = -1;
  o->n_dish = -1;
  o->tsys = -1;
  o->time_tot = -1;
  o->rng = JOINT_RNG_PHILOX;
  o->omp_threads_for_noise = 1;
  FILE *f = std::fopen(path, "r");
  if (!f) return io_error(std::string("Couldn't open file ") + path);
  char line[512];
  int ln = 0;
  while (std::fgets(line, sizeof(line), f)) {
    ln++;
    if (line[0] == '#' || line[0] == '\n') continue;
    char s1[64], s2[256];
    if (std::sscanf(line, "%63s %255s", s1, s2) != 2) {
      std::fclose(f);
      return io_error(std::string("Error reading file ") + path + ", line " + std::to_string(ln));
    }
    const std::string k(s1);
    auto str = [&](char *dst) { std::snprintf(dst, 256, "%s", s2); };
    if (k == "fname_nutable=") str(o->fname_nutable);
    else if (k == "fname_mask=") str(o->fname_mask);
    else if (k == "prefix_cosmo=") str(o->prefix_cosmo);
    else if (k == "prefix_synchrotron=") str(o->prefix_synchrotron);
    else if (k == "prefix_galactic_freefree=") str(o->prefix_galactic_freefree);
    else if (k == "prefix_extragalactic_freefree=") str(o->prefix_extragalactic_freefree);
    else if (k == "prefix_point_sources=") str(o->prefix_point_sources);
    else if (k == "prefix_custom=") str(o->prefix_custom);
    else if (k == "prefix_out=") str(o->prefix_out);
    else if (k == "nside=") o->nside = std::atoi(s2);
    else if (k == "seed=") o->seed_signed = std::atoi(s2);
    else if (k == "do_polarization=") o->do_polarization = std::atoi(s2);
    else if (k == "polarization_leakage=") o->polarization_leakage = std::atof(s2);
    else if (k == "dish_diameter=") o->dish_diameter = std::atof(s2);
    else if (k == "n_dishes=") o->n_dish = std::atoi(s2);
    else if (k == "t_system=") o->tsys = std::atof(s2);
    else if (k == "time_total=") o->time_tot = std::atof(s2);
    else if (k == "rng=") {
      if (!std::strcmp(s2, "philox")) o->rng = JOINT_RNG_PHILOX;
      else if (!std::strcmp(s2, "mt_validation")) o->rng = JOINT_RNG_MT_VALIDATION;
      else {
        std::fclose(f);
        set_error(std::string("Bad value for rng= ") + s2);
        return GETHI_E_ARG;
      }
    } else if (k == "omp_threads_for_noise=") o->omp_threads_for_noise = std::atoi(s2);
    else std::fprintf(stderr, "CRIME: unknown param %s in line %d\n", s1, ln);  // src/io_jt.c:165-168
  }
  std::fclose(f);
  if (o->do_polarization != 1) o->do_polarization = 0;
  if (o->do_polarization && (o->polarization_leakage < 0 || o->polarization_leakage > 1)) {
    set_error("wrong polarization leakage " + std::to_string(o->polarization_leakage));  // src/io_jt.c:172-177
    return GETHI_E_ARG;
  }
  if (o->nside <= 0) {
    set_error("Wrong nside = " + std::to_string(o->nside));
    return GETHI_E_ARG;
  }
  return GETHI_OK;
}

extern "C" int joint_host_read_nutable(const char *path, int *n_nu, double *nu0, double *nuf)
{
  if (!path || !n_nu) return GETHI_E_ARG;
  FILE *f = std::fopen(path, "r");
  if (!f) return io_error(std::string("Couldn't open file ") + path);
  int n = 0;
  char line[1000];
  while (std::fgets(line, sizeof(line), f)) n++;  // linecount, src/common.c:65-75
  std::rewind(f);
  for (int i = 0; i < n; i++) {
    int inu;
    double a, b, d1, d2;
    if (std::fscanf(f, "%d %lf %lf %lf %lf\n", &inu, &a, &b, &d1, &d2) != 5) {
      std::fclose(f);
      return io_error(std::string("Error reading file ") + path + ", line " + std::to_string(i + 1));
    }
    if (nu0) nu0[i] = a;
    if (nuf) nuf[i] = b;
  }
  std::fclose(f);
  *n_nu = n;
  if (n <= 0) {
    set_error("Wrong n_nu = " + std::to_string(n));
    return GETHI_E_ARG;
  }
  return GETHI_OK;
}

extern "C" int joint_host_write_maps(const char *prefix, long nside, int n_nu, const float *maps)
{
  const long npix = 12 * nside * nside;
  for (int i = 0; i < n_nu; i++) {
    char fn[600];
    std::snprintf(fn, sizeof(fn), "%s_%03d.fits", prefix, i + 1);
    int rc = write_fits_map(fn, maps + (long)i * npix, nside);
    if (rc) return rc;
  }
  return GETHI_OK;
}

extern "C" int joint_host_write_instrument(const char *prefix, const joint_params *p, double fsky)
{
  char fn[600];
  std::snprintf(fn, sizeof(fn), "%s_instrument.dat", prefix);
  FILE *f = std::fopen(fn, "w");
  if (!f) return io_error(std::string("Couldn't open file ") + fn);
  const double npix = 12.0 * p->nside * p->nside;
  for (int i = 0; i < p->n_nu; i++) {
    const double nu = 0.5 * (p->nu0[i] + p->nuf[i]), dnu = p->nuf[i] - p->nu0[i];
    const double n_pixels = fsky * npix;
    double fwhm_rad = 0, n_point;
    if (p->dish_diameter > 0) {
      fwhm_rad = kPrefacFwhm / (nu * p->dish_diameter) * M_PI / (180 * 60);
      n_point = fsky * 4 * M_PI / (1.1330900354567985 * fwhm_rad * fwhm_rad);
    } else {
      n_point = fsky * npix;
    }
    double s2p = 0, s2x = 0;
    if (p->tsys > 0) {
      s2p = n_point * (p->tsys * p->tsys) / (kPrefacTnu * dnu * p->time_tot * p->n_dish);
      s2x = n_pixels * (p->tsys * p->tsys) / (kPrefacTnu * dnu * p->time_tot * p->n_dish);
    }
    std::fprintf(f, "%lE %lE %lE %lE\n", nu, 180 * fwhm_rad / M_PI, std::sqrt(s2p), std::sqrt(s2x));
  }
  std::fclose(f);
  return GETHI_OK;
}

namespace {

int read_component(const char *prefix, int n_nu, int column, long &nside_in, std::vector<float> &buf)
{
  for (int i = 0; i < n_nu; i++) {
    char fn[600];
    std::snprintf(fn, sizeof(fn), "%s_%03d.fits", prefix, i + 1);
    long ns = 0;
    int rc = joint_host_read_map(fn, column, &ns, nullptr);
    if (rc) return rc;
    if (nside_in == 0) nside_in = ns;
    if (ns != nside_in) {
      set_error("read nside is not the same as provided : " + std::to_string(nside_in) + " != " +
                std::to_string(ns));  // src/main_jt.c:74-81
      return GETHI_E_ARG;
    }
    const long npix = 12 * ns * ns;
    if (buf.size() != (size_t)npix * n_nu) buf.assign((size_t)npix * n_nu, 0.f);
    if ((rc = joint_host_read_map(fn, column, &ns, buf.data() + (size_t)i * npix))) return rc;
  }
  return GETHI_OK;
}

}  // namespace

extern "C" int joint_host_run(const char *ini_path, int device)
{
  joint_ini ini;
  int rc = joint_host_read_ini(ini_path, &ini);
  if (rc) return rc;
  int n_nu = 0;
  if ((rc = joint_host_read_nutable(ini.fname_nutable, &n_nu, nullptr, nullptr))) return rc;
  std::vector<double> nu0(n_nu), nuf(n_nu);
  if ((rc = joint_host_read_nutable(ini.fname_nutable, &n_nu, nu0.data(), nuf.data()))) return rc;
  const long npix = 12L * ini.nside * ini.nside;
  std::vector<int> mask;
  if (std::strcmp(ini.fname_mask, "default") && std::strcmp(ini.fname_mask, "none")) {  // src/io_jt.c:44-80
    long ns = 0;
    std::vector<float> m(npix);
    if ((rc = joint_host_read_map(ini.fname_mask, 0, &ns, nullptr))) return rc;
    if (ns != ini.nside) {
      set_error("read n_side is not the same as provided: " + std::to_string(ns) + " != " +
                std::to_string(ini.nside) + " in file " + ini.fname_mask);
      return GETHI_E_ARG;
    }
    if ((rc = joint_host_read_map(ini.fname_mask, 0, &ns, m.data()))) return rc;
    mask.resize(npix);
    for (long i = 0; i < npix; i++) {
      const float v = m[i];
      if (v < -0.01f || (v > 0.01f && v < 0.99f) || v > 1.01f) {
        set_error("Mask must be 0 or 1 : " + std::to_string(v));
        return GETHI_E_ARG;
      }
      mask[i] = v > 0.99f ? 1 : 0;
    }
  }
  joint_params p;
  std::memset(&p, 0, sizeof(p));
  p.nside = ini.nside;
  p.n_nu = n_nu;
  p.nu0 = nu0.data();
  p.nuf = nuf.data();
  p.seed = ini.seed_signed <= 0 ? (unsigned)std::time(nullptr) : (unsigned)ini.seed_signed;  // src/io_jt.c:179-180
  p.dish_diameter = ini.dish_diameter;
  p.n_dish = ini.n_dish;
  p.tsys = ini.tsys;
  p.time_tot = ini.time_tot;
  p.mask = mask.empty() ? nullptr : mask.data();
  p.rng = ini.rng;
  p.omp_threads_for_noise = ini.omp_threads_for_noise;
  joint_ctx *c = nullptr;
  if ((rc = joint_gpu_init(&p, device, &c))) return rc;
  // merge_maps order (src/main_jt.c:98-200)
  const char *prefixes[6] = {ini.prefix_cosmo, ini.prefix_extragalactic_freefree, ini.prefix_galactic_freefree,
                             ini.prefix_point_sources, ini.prefix_synchrotron, ini.prefix_custom};
  long nside_in = 0;
  std::vector<float> buf;
  for (int k = 0; k < 6 && !rc; k++) {
    if (!std::strcmp(prefixes[k], "none")) continue;
    if (k == 4 && ini.do_polarization && ini.polarization_leakage > 0) {
      if (!(rc = read_component(prefixes[k], n_nu, 1, nside_in, buf)))
        rc = joint_gpu_add_maps(c, buf.data(), nside_in, ini.polarization_leakage);
    }
    if (!rc && !(rc = read_component(prefixes[k], n_nu, 0, nside_in, buf)))
      rc = joint_gpu_add_maps(c, buf.data(), nside_in, 1.0);
  }
  std::vector<float> out((size_t)npix * n_nu);
  if (!rc) rc = joint_gpu_run(c, out.data());
  const double fsky = joint_gpu_fsky(c);
  joint_gpu_free(c);
  if (!rc) rc = joint_host_write_maps(ini.prefix_out, ini.nside, n_nu, out.data());
  if (!rc) rc = joint_host_write_instrument(ini.prefix_out, &p, fsky);
  return rc;
}
