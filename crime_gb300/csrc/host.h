// Host-side FP64 setup of a GetHI run: parameters, cosmology tables, P(k),
// frequency shells, sub-sample offsets, channel normalisation, reference-
// compatible MT19937 draws and the FITS writer.  Runs once per configuration.
#pragma once
#include <cstdint>
#include <string>
#include <vector>

#include "../../include/gethi_gpu.h"

namespace gethi {

constexpr int NZ = GETHI_NZ;        // src/common_gh.h:34
constexpr double DZ = 0.001;        // src/common_gh.h:33
constexpr double NU21 = 1420.40575177;  // src/common.h:38
constexpr double HMPC = 2997.92458; // src/cosmo_mad.h:35
constexpr int NSUB = 10;            // src/pixelize.c:25

struct Setup {
  gethi_params p;
  gethi_derived d;
  // distance/growth tables (src/cosmo.c:366-392)
  std::vector<double> z_z2r, r_z2r, z_r2z, r_r2z, gd, gv;
  // P(k) table: log10 k and normalised P (src/cosmo.c:306-339)
  std::vector<double> logk, pk;
  // frequency shells: bin edges nu0[i] <= nu < nuf[i] (src/io_gh.c:29-57)
  std::vector<double> nu0, nuf;
  // sub-sample offsets (src/pixelize.c:157-164)
  double xs[NSUB], ys[NSUB], zs[NSUB];
  // per-channel temperature factor M2T/(r^2 dnu) (src/pixelize.c:246-261)
  std::vector<double> prefac;
  double n_scal;
  // point sources (do_psources=1): n(z) and rejection bounds (src/psources.c:98-124),
  // inverse CDF of log10 L, and per channel the factors a, b of
  // T = a S1 + b S2 (S1, S2: the per-pixel sums of the sources)
  std::vector<double> ps_nz, ps_maxpdf, ps_icdf, ps_chan;
  double ps_glob_dz = 0;
};

// src/common.c:133-164 draw through GSL's mt19937; this is the published
// MT19937 with the 2002 seeding that GSL uses (seed 0 -> 4357).
struct MT19937 {
  uint32_t mt[624];
  int mti;
  explicit MT19937(uint32_t seed);
  uint32_t next();
  double uniform() { return next() / 4294967296.0; }
};

int setup_build(const gethi_params &p, Setup &s, std::string &err);
constexpr int PS_NZ = 256;      // src/common_gh.h:35 (NZ_PSOURCES)
constexpr int PS_NICDF = 4096;  // intervals of the log10 L inverse CDF
void setup_psources(Setup &s);
double z_of_r(const Setup &s, double r);  // src/cosmo.c:52-62
double r_of_z(const Setup &s, double z);  // src/cosmo.c:40-50
double pk_linear0(const Setup &s, double lgk);  // src/cosmo.c:153-170

// Reference modes (src/fourier.c:234-305) with the draws of `nthreads`
// OpenMP threads under libgomp's static schedule; layout [kz][ky][N/2+1].
void modes_mt(const Setup &s, int nthreads, float *dens_k);

int write_fits_map(const char *fname, const float *map, long nside);

void set_error(const std::string &e);

}  // namespace gethi
