/*
 * Oracle (test infrastructure only): Fourier modes and the real-space stages
 * of GetHI.  Restates src/fourier.c:24-76 (sigma), :234-305 (modes),
 * :307-373 (radial velocity) and src/grid_tools.c:103-153 (get_HI), with the
 * user model of src/user_defined.c:27-35.
 */
#include <complex.h>
#include <math.h>
#include <stdlib.h>
#include "orc.h"

static double fraction_HI(double z) { return 0.008 * pow(1 + z, 0.6); }            /* user_defined.c:27-30 */
static double bias_HI_fit(double z) { return 0.904 + 0.135 * pow(1 + z, 1.696); } /* user_defined.c:32-35 */

static double kval(int i, int n, double dk) { return (2 * i <= n) ? i * dk : -(n - i) * dk; } /* fourier.c:264-283 */

/* libgomp's static schedule: thread t of T gets a contiguous block, the first
 * (n % T) threads one iteration more. */
static void static_block(int n, int T, int t, int *s, int *e)
{
  int q = n / T, r = n % T;
  if (t < r) { q++; r = 0; }
  *s = q * t + r;
  *e = *s + q;
}

void orc_modes_mt(const orc_config *c, const orc_derived *d, const double *logk,
                  const double *pk, int nthreads, float *dens_k, float *vpot_k)
{
  int n = c->n_grid, h = n / 2 + 1;
  double dk = 2 * M_PI / d->l_box;
  double idk3 = 1. / (dk * dk * dk);
  double factor = d->fgrowth_0 * d->hubble_0;
  if (nthreads < 1) nthreads = 1;
#pragma omp parallel for schedule(dynamic, 1)
  for (int t = 0; t < nthreads; t++) {
    int i0, i1;
    static_block(n, nthreads, t, &i0, &i1);
    orc_mt rng;
    orc_mt_seed(&rng, c->seed + (unsigned int)t);
    for (int ii = i0; ii < i1; ii++) {
      double kz = kval(ii, n, dk);
      for (int jj = 0; jj < n; jj++) {
        double ky = kval(jj, n, dk);
        for (int kk = 0; kk <= n / 2; kk++) {
          double kx = kval(kk, n, dk);
          long index = kk + (long)h * (jj + (long)n * ii);
          double k_mod2 = kx * kx + ky * ky + kz * kz;
          if (k_mod2 <= 0) {
            dens_k[2 * index] = dens_k[2 * index + 1] = 0;
            if (vpot_k) vpot_k[2 * index] = vpot_k[2 * index + 1] = 0;
            continue;
          }
          double lgk = 0.5 * log10(k_mod2);
          double sigma2 = orc_pk_linear0(d, logk, pk, lgk) * idk3;
          if (d->do_smoothing) sigma2 *= exp(-d->r2_smooth * k_mod2);
          /* rng_delta_gauss, common.c:154-164: phase first, then modulus */
          double phase = 2 * M_PI * orc_mt_uniform(&rng);
          double u = orc_mt_uniform(&rng);
          double mod = sqrt(-sigma2 * log(1 - u));
          float complex dkc = mod * cexp(I * phase);
          dens_k[2 * index] = crealf(dkc);
          dens_k[2 * index + 1] = cimagf(dkc);
          if (vpot_k) {
            float complex vk = dkc * factor / k_mod2;
            vpot_k[2 * index] = crealf(vk);
            vpot_k[2 * index + 1] = cimagf(vk);
          }
        }
      }
    }
  }
}

/* Production modes: the same amplitude law with counter-based draws.
 * One Philox4x32-10 call serves the modes kz and kz + N/2 (same ky, kx):
 * ctr = (id lo, id hi, 0, 0), id = kx + (N/2+1)(ky + N (kz mod N/2)),
 * key = (seed, 0x4352494D); the lower mode uses words 0,1, the upper 2,3.
 * Phase = 2 pi w0/2^32; modulus w = (2^32 - w1)/2^32 = 1 - u. */
void orc_modes_philox(const orc_config *c, const orc_derived *d, const double *logk,
                      const double *pk, float *dens_k)
{
  orc_modes_philox_pg(c, d, logk, pk, NULL, dens_k);
}

/* Smoothed P(k) of every grid mode, [kz][ky][kx] over the full n^3 grid, zero at k=0
 * (the amplitude law of src/fourier.c:288-296 without the 1/dk^3 factor). */
void orc_pk_grid(const orc_config *c, const orc_derived *d, const double *logk, const double *pk,
                 double *out)
{
  int n = c->n_grid;
  double dk = 2 * M_PI / d->l_box;
  for (int ii = 0; ii < n; ii++)
    for (int jj = 0; jj < n; jj++)
      for (int kk = 0; kk < n; kk++) {
        double kz = kval(ii, n, dk), ky = kval(jj, n, dk), kx = kval(kk, n, dk);
        double k2 = kx * kx + ky * ky + kz * kz, p = 0;
        if (k2 > 0) {
          p = orc_pk_linear0(d, logk, pk, 0.5 * log10(k2));
          if (d->do_smoothing) p *= exp(-d->r2_smooth * k2);
        }
        out[((long)ii * n + jj) * n + kk] = p;
      }
}

/* Production modes; pg (full n^3 grid [kz][ky][kx], or NULL) replaces the smoothed
 * table P(k) by a Gaussianised spectrum, negative values clipped to zero. */
void orc_modes_philox_pg(const orc_config *c, const orc_derived *d, const double *logk,
                         const double *pk, const double *pg, float *dens_k)
{
  int n = c->n_grid, h = n / 2 + 1;
  double dk = 2 * M_PI / d->l_box;
  double idk3 = 1. / (dk * dk * dk);
#pragma omp parallel for schedule(static)
  for (int ii = 0; ii < n; ii++) {
    double kz = kval(ii, n, dk);
    int half = 2 * ii >= n, ii0 = ii - half * (n / 2);
    for (int jj = 0; jj < n; jj++) {
      double ky = kval(jj, n, dk);
      for (int kk = 0; kk <= n / 2; kk++) {
        double kx = kval(kk, n, dk);
        long index = kk + (long)h * (jj + (long)n * ii);
        double k_mod2 = kx * kx + ky * ky + kz * kz;
        if (k_mod2 <= 0) { dens_k[2 * index] = dens_k[2 * index + 1] = 0; continue; }
        double sigma2;
        if (pg) {
          double p = pg[((long)ii * n + jj) * n + kk];
          sigma2 = (p > 0 ? p : 0) * idk3;
        } else {
          double lgk = 0.5 * log10(k_mod2);
          sigma2 = orc_pk_linear0(d, logk, pk, lgk) * idk3;
          if (d->do_smoothing) sigma2 *= exp(-d->r2_smooth * k_mod2);
        }
        uint64_t id = (uint64_t)kk + (uint64_t)h * ((uint64_t)jj + (uint64_t)n * ii0);
        uint32_t ctr[4] = {(uint32_t)id, (uint32_t)(id >> 32), 0, 0};
        uint32_t key[2] = {c->seed, 0x4352494Du}, o[4];
        orc_philox4x32_10(ctr, key, o);
        uint32_t w0 = half ? o[2] : o[0], w1 = half ? o[3] : o[1];
        double phase = 2 * M_PI * (w0 * (1.0 / 4294967296.0));
        double w = (4294967296.0 - (double)w1) * (1.0 / 4294967296.0);
        double mod = sqrt(-sigma2 * log(w));
        dens_k[2 * index] = (float)(mod * cos(phase));
        dens_k[2 * index + 1] = (float)(mod * sin(phase));
      }
    }
  }
}

void orc_radial_velocity_fd(const orc_config *c, const orc_derived *d, const float *vpot,
                            float *rvel)
{
  int n = c->n_grid;
  double dx = d->l_box / n, idx = 1. / dx;
  long ngx = 2 * (n / 2 + 1);
#pragma omp parallel for schedule(static)
  for (int iz = 0; iz < n; iz++) {
    long iz_hi = iz + 1, iz_lo = iz - 1, iz_0 = iz;
    double z = dx * (iz + 0.5) - d->pos_obs[2];
    if (iz == 0) iz_lo = n - 1;
    if (iz == n - 1) iz_hi = 0;
    iz_hi *= ngx * n; iz_lo *= ngx * n; iz_0 *= ngx * n;
    for (int iy = 0; iy < n; iy++) {
      long iy_hi = iy + 1, iy_lo = iy - 1, iy_0 = iy;
      double y = dx * (iy + 0.5) - d->pos_obs[1];
      if (iy == 0) iy_lo = n - 1;
      if (iy == n - 1) iy_hi = 0;
      iy_hi *= ngx; iy_lo *= ngx; iy_0 *= ngx;
      for (int ix = 0; ix < n; ix++) {
        long ix_hi = ix + 1, ix_lo = ix - 1, ix_0 = ix;
        double x = dx * (ix + 0.5) - d->pos_obs[0];
        double irr = 1. / sqrt(x * x + y * y + z * z);
        if (ix == 0) ix_lo = n - 1;
        if (ix == n - 1) ix_hi = 0;
        double ur0 = x * irr, ur1 = y * irr, ur2 = z * irr;
        /* float differences, as in fourier.c:359-366 */
        float dvx = vpot[ix_hi + iy_0 + iz_0] - vpot[ix_lo + iy_0 + iz_0];
        float dvy = vpot[ix_0 + iy_hi + iz_0] - vpot[ix_0 + iy_lo + iz_0];
        float dvz = vpot[ix_0 + iy_0 + iz_hi] - vpot[ix_0 + iy_0 + iz_lo];
        double v0 = 0.5 * idx * dvx, v1 = 0.5 * idx * dvy, v2 = 0.5 * idx * dvz;
        rvel[ix_0 + iy_0 + iz_0] = v0 * ur0 + v1 * ur1 + v2 * ur2;
      }
    }
  }
}

void orc_sigma_dens(int n, const float *dens, double *mean, double *sigma2)
{
  long ngx = 2 * (n / 2 + 1);
  long ng_tot = (long)n * n * n;
  double s2 = 0, m = 0;
  for (int iz = 0; iz < n; iz++)
    for (int iy = 0; iy < n; iy++)
      for (int ix = 0; ix < n; ix++) {
        float v = dens[ix + iy * ngx + iz * ngx * n];
        s2 += v * v; /* float product, fourier.c:51 */
        m += v;
      }
  *mean = m / ng_tot;
  *sigma2 = s2 / ng_tot - (*mean) * (*mean);
}

void orc_get_hi(const orc_config *c, const orc_derived *d, double sigma2, float *dens, float *rvel)
{
  int n = c->n_grid;
  double dx = d->l_box / n;
  long ngx = 2 * (n / 2 + 1);
  double mass_prefac = dx * dx * dx;
#pragma omp parallel for schedule(static)
  for (int iz = 0; iz < n; iz++) {
    double z = dx * (iz + 0.5) - d->pos_obs[2];
    long iz0 = iz * (ngx * n);
    for (int iy = 0; iy < n; iy++) {
      double y = dx * (iy + 0.5) - d->pos_obs[1];
      long iy0 = iy * ngx;
      for (int ix = 0; ix < n; ix++) {
        long index = iz0 + iy0 + ix;
        double x = dx * (ix + 0.5) - d->pos_obs[0];
        double r = sqrt(x * x + y * y + z * z);
        double redshift = orc_z_of_r(d, r);
        double bias = c->bias_const ? c->b_HI : bias_HI_fit(redshift);
        double gfd = orc_dgrowth_of_r(d, r) * bias;
        double delta_gauss = dens[index];
        double dz_rsd = c->do_rsd ? rvel[index] * orc_vgrowth_of_r(d, r) : 0;
        double dens_LN = exp(gfd * (delta_gauss - 0.5 * gfd * sigma2));
        double mass_HI = mass_prefac * fraction_HI(redshift) * dens_LN;
        dens[index] = mass_HI;
        rvel[index] = dz_rsd;
      }
    }
  }
}

/* Spectral radial velocity (velocity_mode=spectral, not in the reference):
 * v_j(x) = c2r(i k_j phi_k) with phi_k = delta_k f0 H0 / k^2 (src/fourier.c:298)
 * and the derivative of a Nyquist component set to zero, normalised like
 * src/fourier.c:403 and projected on the unit vector from the observer.
 * FP64 throughout; rvel is the padded [z][y][2(N/2+1)] float grid. */
void orc_radial_velocity_spectral(const orc_config *c, const orc_derived *d, const float *dens_k, float *rvel)
{
  int n = c->n_grid, h = n / 2 + 1;
  size_t nh = (size_t)n * n * h, n3 = (size_t)n * n * n;
  double dk = 2 * M_PI / d->l_box, factor = d->fgrowth_0 * d->hubble_0;
  double norm = pow(sqrt(2 * M_PI) / d->l_box, 3), dx = d->l_box / n;
  float *spec = (float *)malloc(sizeof(float) * 2 * nh);
  double *comp = (double *)malloc(sizeof(double) * n3), *acc = (double *)calloc(n3, sizeof(double));
  for (int j = 0; j < 3; j++) {
    /* the c2r helper reads float input: keep i k_j phi_k in double until the
     * final rounding by splitting into hi + lo float parts */
    float *lo = (float *)malloc(sizeof(float) * 2 * nh);
    for (int ii = 0; ii < n; ii++)
      for (int jj = 0; jj < n; jj++)
        for (int kk = 0; kk < h; kk++) {
          size_t idx = kk + (size_t)h * (jj + (size_t)n * ii);
          double kx = kval(kk, n, dk), ky = kval(jj, n, dk), kz = kval(ii, n, dk);
          double k2 = kx * kx + ky * ky + kz * kz;
          double kj = j == 0 ? (2 * kk == n ? 0 : kx) : j == 1 ? (2 * jj == n ? 0 : ky) : (2 * ii == n ? 0 : kz);
          double re = 0, im = 0;
          if (k2 > 0) {
            double f = factor / k2 * kj;
            re = -dens_k[2 * idx + 1] * f;
            im = dens_k[2 * idx] * f;
          }
          spec[2 * idx] = (float)re;
          spec[2 * idx + 1] = (float)im;
          lo[2 * idx] = (float)(re - (double)spec[2 * idx]);
          lo[2 * idx + 1] = (float)(im - (double)spec[2 * idx + 1]);
        }
    orc_c2r_to_double(n, spec, comp);
    double *c2 = (double *)malloc(sizeof(double) * n3);
    orc_c2r_to_double(n, lo, c2);
    for (int iz = 0; iz < n; iz++)
      for (int iy = 0; iy < n; iy++)
        for (int ix = 0; ix < n; ix++) {
          size_t q = ix + (size_t)n * (iy + (size_t)n * iz);
          double x = dx * (ix + 0.5) - d->pos_obs[0], y = dx * (iy + 0.5) - d->pos_obs[1], z = dx * (iz + 0.5) - d->pos_obs[2];
          double u = (j == 0 ? x : j == 1 ? y : z) / sqrt(x * x + y * y + z * z);
          acc[q] += (comp[q] + c2[q]) * norm * u;
        }
    free(c2);
    free(lo);
  }
  for (int iz = 0; iz < n; iz++)
    for (int iy = 0; iy < n; iy++)
      for (int ix = 0; ix < n; ix++)
        rvel[ix + 2 * (size_t)h * (iy + (size_t)n * iz)] = (float)acc[ix + (size_t)n * (iy + (size_t)n * iz)];
  free(spec);
  free(comp);
  free(acc);
}
