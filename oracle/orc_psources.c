/*
 * Oracle: point sources -- TEST INFRASTRUCTURE ONLY.
 *
 * Restates src/psources.c (luminosity function, n(z) table, rejection-sampled
 * luminosities, flux -> temperature), get_point_sources (src/grid_tools.c:24-101:
 * a Poisson number of sources per cell from the lognormal density) and
 * mk_psources_maps (src/pixelize.c:58-148: each source at a uniform position in
 * its cell, its temperature added to every channel of its pixel).
 *
 * Random numbers follow the reference: per OpenMP thread t an MT19937 seeded
 * with seed + t over libgomp's static partition of the z planes, fresh for the
 * sampling and again for the maps (src/grid_tools.c:50, src/pixelize.c:80).
 * Poisson draws restate GSL's gsl_ran_poisson for means <= 10, Knuth's
 * multiplication method (TAOCP vol. 2, 3.4.1): multiply uniforms until the
 * product drops to e^{-mu}; larger means return an error (not restated).
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "orc.h"

#define LLOGMIN -5.    /* psources.c:25-26 */
#define LLOGMAX 6.
#define LX_TOY 2.11    /* psources.c:33-35 */
#define ALPHA_TOY -0.633
#define RHO_TOY 3.2E-4
#define SED_NORM 0.114461           /* psources.c:54 */
#define FLUX2TEMP 3.2548291E-2      /* psources.c:154 */
#define LUM2FLUX 8.35774E7          /* psources.c:155 */

/* dn(z, L)/dlog10(L), L in 1e22 W/Hz (psources.c:39-52) */
static double l_z_function(double L, double z)
{
  double rho_l = 2.5 * M_LN10 * RHO_TOY * pow(L / LX_TOY, ALPHA_TOY + 1) * exp(-L / LX_TOY);
  double fz = z < 1.5 ? pow(1 + z, 3.1) : 17.124;
  return fz * rho_l;
}

/* SED normalised at 1420 MHz (psources.c:55-63) */
static double spec_ed(double nu)
{
  double nu_GHz = nu * 0.001;
  return SED_NORM * (pow(nu_GHz, -0.1) + 10 * pow(nu_GHz, -0.75));
}

/* setup_psources (psources.c:98-124) */
void orc_setup_psources(double z_max, double *nz_arr, double *maxpdf, double *glob_dz)
{
  double dlogL = (LLOGMAX - LLOGMIN) / ORC_NL_PS;
  *glob_dz = z_max / ORC_NZ_PS;
  for (int ii = 0; ii < ORC_NZ_PS; ii++) {
    double z = ii * *glob_dz, max_dist = -1;
    nz_arr[ii] = 0;
    for (int jj = 0; jj < ORC_NL_PS; jj++) {
      double logL = LLOGMIN + (jj + 0.5) * dlogL;
      double lfunc = l_z_function(pow(10., logL), z);
      if (lfunc >= max_dist) max_dist = lfunc;
      nz_arr[ii] += dlogL * lfunc;
    }
    maxpdf[ii] = nz_arr[ii] > 0 ? 1.1 * max_dist / nz_arr[ii] : 0;
  }
}

/* n_of_z_psources (psources.c:74-90) */
double orc_n_of_z_psources(const double *nz_arr, double glob_dz, double z)
{
  double inv = 1. / glob_dz;
  int iz = (int)(z * inv);
  if (iz >= ORC_NZ_PS || iz < 0) return -1;
  if (iz == ORC_NZ_PS - 1) return nz_arr[ORC_NZ_PS - 1];
  double zi = iz * glob_dz;
  return nz_arr[iz] + (nz_arr[iz + 1] - nz_arr[iz]) * (z - zi) * inv;
}

/* gsl_ran_poisson for mu <= 10 (see the header); -1 beyond */
long orc_poisson_small(orc_mt *r, double mu)
{
  if (mu > 10) return -1;
  double emu = exp(-mu), prod = 1.0;
  long k = 0;
  do {
    prod *= orc_mt_uniform(r);
    k++;
  } while (prod > emu);
  return k - 1;
}

/* draw_luminosity (psources.c:126-152) */
static double draw_luminosity(const double *nz_arr, const double *maxpdf, double glob_dz, double z_max,
                              double z, orc_mt *rng)
{
  if (z >= z_max) return 0;
  int iz = (int)(z * (1. / glob_dz));
  double mp = maxpdf[iz];
  for (;;) {
    double u = orc_mt_uniform(rng);
    double logL = LLOGMIN + (LLOGMAX - LLOGMIN) * orc_mt_uniform(rng);
    double L = pow(10., logL);
    if (u * mp < l_z_function(L, z) / orc_n_of_z_psources(nz_arr, glob_dz, z)) return L;
  }
}

/* temp_of_l (psources.c:158-167), L in 1e22 W/Hz/sr */
double orc_temp_of_l(double hhub, double L0, double nu_obs, double z, double r, double dOmega)
{
  double s_nu = LUM2FLUX * 4 * M_PI * L0 * spec_ed((1 + z) * nu_obs) * hhub * hhub / (r * r * (1 + z));
  return FLUX2TEMP * s_nu / (dOmega * nu_obs * nu_obs);
}

/* libgomp's static partition of n iterations over nt threads */
static void static_block(int n, int nt, int t, int *i0, int *i1)
{
  int q = n / nt, rem = n % nt;
  if (t < rem) {
    q++;
    rem = 0;
  }
  *i0 = q * t + rem;
  *i1 = *i0 + q;
}

/* get_point_sources (grid_tools.c:24-101).  dens: the Gaussian field, padded
 * [z][y][2(N/2+1)]; nsources: same layout (ints).  Returns the total, or -1 if
 * a cell's mean exceeds the restated Poisson range. */
long orc_point_sources(const orc_config *c, const orc_derived *d, const double *nz_arr, double glob_dz,
                       const float *dens, double sigma2, int nthreads, int *nsources)
{
  int n = c->n_grid, ngx = 2 * (n / 2 + 1);
  double dx = d->l_box / n, cell_vol = dx * dx * dx;
  long total = 0;
  int bad = 0;
  if (nthreads < 1) nthreads = 1;
  memset(nsources, 0, sizeof(int) * (size_t)ngx * n * n);
#pragma omp parallel for schedule(dynamic, 1) reduction(+ : total, bad)
  for (int t = 0; t < nthreads; t++) {
    int i0, i1;
    static_block(n, nthreads, t, &i0, &i1);
    orc_mt rng;
    orc_mt_seed(&rng, c->seed + (unsigned int)t);
    for (int iz = i0; iz < i1; iz++) {
      double z0 = (iz + 0.5) * dx - d->pos_obs[2];
      for (int iy = 0; iy < n; iy++) {
        double y0 = (iy + 0.5) * dx - d->pos_obs[1];
        for (int ix = 0; ix < n; ix++) {
          long index = ix + (long)ngx * (iy + (long)n * iz);
          double x0 = (ix + 0.5) * dx - d->pos_obs[1];  /* grid_tools.c:72 uses pos_obs[1] for x */
          double r = sqrt(x0 * x0 + y0 * y0 + z0 * z0);
          double redshift = orc_z_of_r(d, r);
          double ndens = orc_n_of_z_psources(nz_arr, glob_dz, redshift);
          long npp = 0;
          if (ndens > 0) {
            double gfb = orc_dgrowth_of_r(d, r) * 1.0;  /* bias_psources = 1 (psources.c:65-68) */
            double lambda = ndens * cell_vol * exp(gfb * (dens[index] - 0.5 * gfb * sigma2));
            npp = orc_poisson_small(&rng, lambda);
            if (npp < 0) {
              bad++;
              npp = 0;
            }
          }
          nsources[index] = (int)npp;
          total += npp;
        }
      }
    }
  }
  return bad ? -1 : total;
}

/* Poisson means of get_point_sources (grid_tools.c:67-84), 0 where n(z) <= 0; lam:
 * compact [z][y][x] doubles, dens padded */
void orc_ps_lambda(const orc_config *c, const orc_derived *d, const double *nz_arr, double glob_dz,
                   const float *dens, double sigma2, double *lam)
{
  int n = c->n_grid, ngx = 2 * (n / 2 + 1);
  double dx = d->l_box / n, cell_vol = dx * dx * dx;
  for (int iz = 0; iz < n; iz++)
    for (int iy = 0; iy < n; iy++)
      for (int ix = 0; ix < n; ix++) {
        double x0 = (ix + 0.5) * dx - d->pos_obs[0], y0 = (iy + 0.5) * dx - d->pos_obs[1],
               z0 = (iz + 0.5) * dx - d->pos_obs[2];
        double r = sqrt(x0 * x0 + y0 * y0 + z0 * z0);
        double ndens = orc_n_of_z_psources(nz_arr, glob_dz, orc_z_of_r(d, r));
        double gfb = orc_dgrowth_of_r(d, r);
        long index = ix + (long)ngx * (iy + (long)n * iz);
        lam[ix + (long)n * (iy + (long)n * iz)] =
            ndens > 0 ? ndens * cell_vol * exp(gfb * (dens[index] - 0.5 * gfb * sigma2)) : 0.0;
      }
}

/* mk_psources_maps (pixelize.c:58-148).  dz: dz_rsd after get_HI, padded; maps_ps
 * [n_nu][12 n_side^2], accumulated as the reference does (float += double). */
void orc_psources_maps(const orc_config *c, const orc_derived *d, const double *nu0, const double *nuf,
                       const double *nz_arr, const double *maxpdf, double glob_dz, const int *nsources,
                       const float *dz, int nthreads, float *maps_ps)
{
  int n = c->n_grid, ngx = 2 * (n / 2 + 1), nn = c->n_nu;
  long nside = c->n_side, npix = 12 * nside * nside;
  double dx = d->l_box / n, dOmega = 4 * M_PI / npix;
  double *nu_arr = (double *)malloc(sizeof(double) * nn);
  for (int i = 0; i < nn; i++)
    nu_arr[i] = c->regular_nu ? c->nu_min + (c->nu_max - c->nu_min) * (i + 0.5) / nn : (nu0[i] + nuf[i]) * 0.5;
  memset(maps_ps, 0, sizeof(float) * npix * nn);
  if (nthreads < 1) nthreads = 1;
#pragma omp parallel for schedule(dynamic, 1)
  for (int t = 0; t < nthreads; t++) {
    int i0, i1;
    static_block(n, nthreads, t, &i0, &i1);
    orc_mt rng;
    orc_mt_seed(&rng, c->seed + (unsigned int)t);
    for (int iz = i0; iz < i1; iz++) {
      double z0 = dx * iz - d->pos_obs[2];
      for (int iy = 0; iy < n; iy++) {
        double y0 = dx * iy - d->pos_obs[1];
        for (int ix = 0; ix < n; ix++) {
          long index = ix + (long)ngx * (iy + (long)n * iz);
          double x0 = dx * ix - d->pos_obs[0];
          int np = nsources[index];
          double dz_rsd = (double)dz[index];
          for (int ip = 0; ip < np; ip++) {
            double pos[3];
            pos[0] = x0 + dx * orc_mt_uniform(&rng);
            pos[1] = y0 + dx * orc_mt_uniform(&rng);
            pos[2] = z0 + dx * orc_mt_uniform(&rng);
            double r = sqrt(pos[0] * pos[0] + pos[1] * pos[1] + pos[2] * pos[2]);
            double red_cosmo = orc_z_of_r(d, r), red_true = red_cosmo + dz_rsd;
            long ipix = orc_vec2pix_ring(nside, pos);
            double l0 = draw_luminosity(nz_arr, maxpdf, glob_dz, d->z_max, red_cosmo, &rng);
            for (int inu = 0; inu < nn; inu++) {
              double temperature = orc_temp_of_l(c->hhub, l0, nu_arr[inu], red_true, r, dOmega);
              if (temperature > 0) {
#pragma omp atomic
                maps_ps[ipix + npix * inu] += temperature;
              }
            }
          }
        }
      }
    }
  }
  free(nu_arr);
}

/* Point-source maps of a given catalogue, FP64 accumulation (checker of the GPU
 * path, whose draws are counter-based): source s sits in cell cell[s] = ix +
 * n (iy + n iz) at corner + dx u[3s..3s+2], with luminosity L0[s] and the cell's
 * dz_rsd dz[s]; its pixel goes to pix[s]. */
void orc_psources_maps_catalogue(const orc_config *c, const orc_derived *d, const double *nu0, const double *nuf,
                                 long ns, const int64_t *cell, const double *u, const double *L0,
                                 const double *dzs, double *maps_ps, int64_t *pix)
{
  int n = c->n_grid, nn = c->n_nu;
  long nside = c->n_side, npix = 12 * nside * nside;
  double dx = d->l_box / n, dOmega = 4 * M_PI / npix;
  memset(maps_ps, 0, sizeof(double) * npix * nn);
  for (long s = 0; s < ns; s++) {
    long ix = cell[s] % n, iy = (cell[s] / n) % n, iz = cell[s] / ((long)n * n);
    double pos[3] = {dx * ix - d->pos_obs[0] + dx * u[3 * s], dx * iy - d->pos_obs[1] + dx * u[3 * s + 1],
                     dx * iz - d->pos_obs[2] + dx * u[3 * s + 2]};
    double r = sqrt(pos[0] * pos[0] + pos[1] * pos[1] + pos[2] * pos[2]);
    double red_true = orc_z_of_r(d, r) + dzs[s];
    long ipix = orc_vec2pix_ring(nside, pos);
    pix[s] = ipix;
    for (int inu = 0; inu < nn; inu++) {
      double nu = c->regular_nu ? c->nu_min + (c->nu_max - c->nu_min) * (inu + 0.5) / nn : (nu0[inu] + nuf[inu]) * 0.5;
      double t = orc_temp_of_l(c->hhub, L0[s], nu, red_true, r, dOmega);
      if (t > 0) maps_ps[ipix + npix * inu] += t;
    }
  }
}
