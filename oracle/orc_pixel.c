/*
 * Oracle (test infrastructure only): projection of the HI mass grid onto
 * HEALPix maps, one per frequency shell.  Restates src/pixelize.c:28-56
 * (get_inu) and :150-286 (mk_T_maps).
 *
 * vec2pix_ring/pix2ang_ring are restated from the RING-scheme formulas of
 * Gorski et al. 2005 (ApJ 622:759, section 4), not from chealpix, which is
 * absent here: parity with chealpix is unpinned.  For |cos(theta)| > 0.99 the
 * polar-cap radius uses sin(theta)/sqrt((1+|z|)/3), the cancellation-free form
 * of sqrt(3(1-|z|)).
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include "orc.h"

#define TWOTHIRD (2.0 / 3.0)
#define INV_HALFPI 0.63661977236758134308 /* 2/pi */

static long imodl(long a, long m) { long r = a % m; return r < 0 ? r + m : r; }

static long loc2pix_ring(long nside, double z, double s, double phi)
{
  double za = fabs(z);
  double tt = phi * INV_HALFPI;
  if (tt < 0) tt += 4.0;
  long npix = 12 * nside * nside;
  long ncap = 2 * nside * (nside - 1);
  if (za <= TWOTHIRD) {
    double t1 = nside * (0.5 + tt);
    double t2 = nside * z * 0.75;
    long jp = (long)(t1 - t2);
    long jm = (long)(t1 + t2);
    long ir = nside + 1 + jp - jm;
    long kshift = 1 - (ir & 1);
    long ip = (jp + jm - nside + kshift + 1) / 2;
    ip = imodl(ip, 4 * nside);
    return ncap + (ir - 1) * 4 * nside + ip;
  }
  double tp = tt - (long)tt;
  double tmp = (s > -2) ? nside * s / sqrt((1 + za) / 3) : nside * sqrt(3 * (1 - za));
  long jp = (long)(tp * tmp);
  long jm = (long)((1 - tp) * tmp);
  long ir = jp + jm + 1;
  long ip = (long)(tt * ir);
  ip = imodl(ip, 4 * ir);
  return (z > 0) ? 2 * ir * (ir - 1) + ip : npix - 2 * ir * (ir + 1) + ip;
}

long orc_vec2pix_ring(long nside, const double *v)
{
  double xy2 = v[0] * v[0] + v[1] * v[1];
  double vlen = sqrt(xy2 + v[2] * v[2]);
  double cth = v[2] / vlen;
  double sth = (fabs(cth) > 0.99) ? sqrt(xy2) / vlen : -5;
  return loc2pix_ring(nside, cth, sth, atan2(v[1], v[0]));
}

void orc_pix2ang_ring(long nside, long ipix, double *theta, double *phi)
{
  long npix = 12 * nside * nside, ncap = 2 * nside * (nside - 1);
  double z;
  if (ipix < ncap) {
    long iring = (long)(0.5 * (1 + sqrt(1 + 2.0 * ipix)));
    while (2 * iring * (iring - 1) > ipix) iring--;
    while (2 * (iring + 1) * iring <= ipix) iring++;
    long iphi = ipix - 2 * iring * (iring - 1) + 1;
    z = 1 - (double)(iring * iring) / (3.0 * nside * nside);
    *phi = (iphi - 0.5) * M_PI / (2.0 * iring);
  } else if (ipix < npix - ncap) {
    long ip = ipix - ncap;
    long iring = ip / (4 * nside) + nside;
    long iphi = ip % (4 * nside) + 1;
    double fodd = ((iring + nside) & 1) ? 1 : 0.5;
    z = (2 * nside - iring) * 2.0 / (3.0 * nside);
    *phi = (iphi - fodd) * M_PI / (2.0 * nside);
  } else {
    long ip = npix - ipix;
    long iring = (long)(0.5 * (1 + sqrt(2.0 * ip - 1)));
    while (2 * iring * (iring - 1) >= ip) iring--;
    while (2 * (iring + 1) * iring < ip) iring++;
    long iphi = 4 * iring + 1 - (ip - 2 * iring * (iring - 1));
    z = -1 + (double)(iring * iring) / (3.0 * nside * nside);
    *phi = (iphi - 0.5) * M_PI / (2.0 * iring);
  }
  *theta = acos(z);
}

/* src/pixelize.c:28-56: walk from the previous bin to nu0 <= nu < nuf. */
int orc_get_inu(const double *nu0, const double *nuf, int n_nu, double nu, int inu_start)
{
  int inu0 = inu_start < 0 ? 0 : (inu_start >= n_nu ? n_nu - 1 : inu_start);
  for (;;) {
    if (inu0 == -1 || inu0 == n_nu) return inu0;
    if (nu < nu0[inu0]) inu0--;
    else if (nu >= nuf[inu0]) inu0++;
    else return inu0;
  }
}

/* src/pixelize.c:157-164: 10 offsets from one MT19937(seed) stream, x,y,z per sub-sample */
void orc_subsample_offsets(unsigned int seed, double lcell, double *xs, double *ys, double *zs)
{
  orc_mt rng;
  orc_mt_seed(&rng, seed);
  for (int i = 0; i < ORC_NSUB; i++) {
    xs[i] = lcell * (orc_mt_uniform(&rng) - 0.5);
    ys[i] = lcell * (orc_mt_uniform(&rng) - 0.5);
    zs[i] = lcell * (orc_mt_uniform(&rng) - 0.5);
  }
}

/* src/pixelize.c:246-261 */
void orc_channel_prefactors(const orc_config *c, const orc_derived *d, const double *nu0,
                            const double *nuf, double *prefac)
{
  double M2T = 90.057156 * c->OmegaB * c->hhub * (12.0 * c->n_side * c->n_side) / (4 * M_PI);
  for (int inu = 0; inu < c->n_nu; inu++) {
    double dnu, nu;
    if (c->regular_nu) {
      dnu = (c->nu_max - c->nu_min) / c->n_nu;
      nu = c->nu_min + (inu + 0.5) * dnu;
    } else {
      dnu = nuf[inu] - nu0[inu];
      nu = (nuf[inu] + nu0[inu]) * 0.5;
    }
    double r = orc_r_of_z(d, ORC_NU21 / nu - 1);
    prefac[inu] = M2T / (r * r * dnu);
  }
}

void orc_mk_T_maps(const orc_config *c, const orc_derived *d, const double *nu0,
                   const double *nuf, const float *mass, const float *dz, float *maps,
                   uint32_t *keys)
{
  int n = c->n_grid;
  long nside = c->n_side;
  long npix = 12 * nside * nside;
  double dx = d->l_box / n;
  double xs[ORC_NSUB], ys[ORC_NSUB], zs[ORC_NSUB];
  orc_subsample_offsets(c->seed, dx, xs, ys, zs);
  double inv_dnu = c->n_nu / (c->nu_max - c->nu_min);
  long ngx = 2 * (n / 2 + 1);
  memset(maps, 0, sizeof(float) * npix * c->n_nu);
#pragma omp parallel for schedule(static)
  for (int iz = 0; iz < n; iz++) {
    int inu = 0;
    double z0 = dx * (iz + 0.5) - d->pos_obs[2];
    for (int iy = 0; iy < n; iy++) {
      double y0 = dx * (iy + 0.5) - d->pos_obs[1];
      for (int ix = 0; ix < n; ix++) {
        long index = ix + iy * ngx + iz * ngx * n;
        long cell = ix + (long)n * (iy + (long)n * iz);
        double x0 = dx * (ix + 0.5) - d->pos_obs[0];
        float mass_sub = mass[index] / ORC_NSUB;
        double dz_rsd = (double)dz[index];
        for (int is = 0; is < ORC_NSUB; is++) {
          double x = x0 + xs[is], y = y0 + ys[is], z = z0 + zs[is];
          double r = sqrt(x * x + y * y + z * z);
          double redshift = orc_z_of_r(d, r) + dz_rsd;
          double nu = ORC_NU21 / (1 + redshift);
          if (c->regular_nu) inu = (int)(inv_dnu * (nu - c->nu_min));
          else inu = orc_get_inu(nu0, nuf, c->n_nu, nu, inu);
          uint32_t key = 0xFFFFFFFFu;
          if (inu >= 0 && inu < c->n_nu) {
            double pos[3] = {x, y, z};
            long ipix = orc_vec2pix_ring(nside, pos);
#pragma omp atomic
            maps[ipix + npix * inu] += mass_sub;
            key = (uint32_t)(ipix + npix * inu);
          }
          if (keys) keys[cell * ORC_NSUB + is] = key;
        }
      }
    }
  }
  double *prefac = (double *)malloc(sizeof(double) * c->n_nu);
  orc_channel_prefactors(c, d, nu0, nuf, prefac);
  for (int inu = 0; inu < c->n_nu; inu++)
    for (long ip = 0; ip < npix; ip++) maps[ip + npix * inu] *= prefac[inu];
  free(prefac);
}

#ifdef _OPENMP
#include <omp.h>
int orc_num_threads(void) { return omp_get_max_threads(); }
void orc_set_threads(int t) { omp_set_num_threads(t); }
#else
int orc_num_threads(void) { return 1; }
void orc_set_threads(int t) { (void)t; }
#endif
