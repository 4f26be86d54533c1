/*
 * Oracle (test infrastructure only): the JoinT map combination of
 * src/main_jt.c:98-321 -- merge + ud_grade, Gaussian beam through a spherical
 * harmonic transform, white noise, mask -- and the HEALPix helpers it uses
 * (src/healpix_extra.c:31-43, 318-421).
 *
 * RING <-> NESTED conversion and the ring geometry are restated from the
 * HEALPix scheme of Gorski et al. 2005 (ApJ 622:759, sections 4-5); chealpix is
 * absent here, so parity with it is unpinned (the tests check the round trip
 * and the nesting geometry instead).  The spherical harmonic transform restates
 * what src/healpix_extra.c:44-130 asks of libsharp (absent here; unpinned):
 * triangular a_lm with lmax = mmax, HEALPix ring geometry with the uniform
 * quadrature weight 4 pi / npix on every pixel, no iteration, FP64 throughout:
 *   map2alm: a_lm = 4pi/npix sum_rings lambda_lm(theta) sum_j map_j e^{-i m phi_j}
 *   alm2map: map_j = sum_m (2 - delta_m0) Re(e^{i m phi_j} sum_l a_lm lambda_lm(theta))
 * with lambda_lm the orthonormal associated Legendre functions including the
 * Condon-Shortley phase (-1)^m, evaluated by the standard three-term recursion
 * in l with an explicit power-of-two exponent so that sin^m(theta) cannot
 * underflow before the recursion brings it back into range.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include "orc.h"

static long spread_bits(long v)
{
  long r = 0;
  for (int b = 0; b < 31; b++) r |= ((v >> b) & 1L) << (2 * b);
  return r;
}
static long compress_bits(long v)
{
  long r = 0;
  for (int b = 0; b < 31; b++) r |= ((v >> (2 * b)) & 1L) << b;
  return r;
}
static long isqrt_l(long v)
{
  long r = (long)sqrt((double)v + 0.5);
  while (r * r > v) r--;
  while ((r + 1) * (r + 1) <= v) r++;
  return r;
}
/* base-pixel ring row (in units of nside) and longitude offset of the 12 faces */
static const int kFaceRow[12] = {2, 2, 2, 2, 3, 3, 3, 3, 4, 4, 4, 4};
static const int kFaceLon[12] = {1, 3, 5, 7, 0, 2, 4, 6, 1, 3, 5, 7};

long orc_nest2ring(long nside, long ipnest)
{
  const long npface = nside * nside, npix = 12 * npface, ncap = 2 * nside * (nside - 1);
  const long face = ipnest / npface, ipf = ipnest % npface;
  const long ix = compress_bits(ipf), iy = compress_bits(ipf >> 1);
  const long jr = kFaceRow[face] * nside - (ix + iy) - 1; /* ring number, 1-based */
  long nr, first, shift;
  if (jr < nside) {
    nr = jr;
    first = 2 * nr * (nr - 1);
    shift = 0;
  } else if (jr > 3 * nside) {
    nr = 4 * nside - jr;
    first = npix - 2 * (nr + 1) * nr;
    shift = 0;
  } else {
    nr = nside;
    first = ncap + (jr - nside) * 4 * nside;
    shift = (jr - nside) & 1;
  }
  long jp = (kFaceLon[face] * nr + (ix - iy) + 1 + shift) / 2;
  if (jp > 4 * nr) jp -= 4 * nr;
  if (jp < 1) jp += 4 * nr;
  return first + jp - 1;
}

long orc_ring2nest(long nside, long ipring)
{
  const long npface = nside * nside, npix = 12 * npface, ncap = 2 * nside * (nside - 1);
  long iring, iphi, shift, nr, face;
  if (ipring < ncap) {
    iring = (1 + isqrt_l(1 + 2 * ipring)) >> 1;
    iphi = ipring + 1 - 2 * iring * (iring - 1);
    shift = 0;
    nr = iring;
    face = (iphi - 1) / nr;
  } else if (ipring < npix - ncap) {
    const long ip = ipring - ncap, t = ip / (4 * nside);
    iring = t + nside;
    iphi = ip - t * 4 * nside + 1;
    shift = (iring + nside) & 1;
    nr = nside;
    const long ire = t + 1, irm = 2 * nside + 2 - ire;
    const long fm = (iphi - ire / 2 + nside - 1) / nside, fp = (iphi - irm / 2 + nside - 1) / nside;
    face = (fp == fm) ? (fp | 4) : (fp < fm ? fp : fm + 8);
  } else {
    const long ip = npix - ipring;
    iring = (1 + isqrt_l(2 * ip - 1)) >> 1;
    iphi = 4 * iring + 1 - (ip - 2 * iring * (iring - 1));
    shift = 0;
    nr = iring;
    iring = 4 * nside - iring;
    face = 8 + (iphi - 1) / nr;
  }
  const long irt = iring - kFaceRow[face] * nside + 1;
  long ipt = 2 * iphi - kFaceLon[face] * nr - shift - 1;
  if (ipt >= 2 * nside) ipt -= 8 * nside;
  const long ix = (ipt - irt) >> 1, iy = (-(ipt + irt)) >> 1;
  return face * npface + spread_bits(ix) + 2 * spread_bits(iy);
}

/* Ring `ring` (0-based, 0 .. 4 nside - 2): first pixel, pixels in the ring,
 * cos(theta), sin(theta) and the longitude of its first pixel. */
void orc_ring_info(long nside, long ring, long *first, long *nph, double *z, double *sth, double *phi0)
{
  const long npix = 12 * nside * nside, ncap = 2 * nside * (nside - 1);
  const long ir = ring + 1, north = ir > 2 * nside ? 4 * nside - ir : ir;
  double cz, sz;
  if (north < nside) {
    const double a = (double)north * north / (3.0 * nside * nside); /* 1 - cos(theta), exact form */
    cz = 1.0 - a;
    sz = sqrt(a * (2.0 - a));
    *nph = 4 * north;
    *phi0 = M_PI / (double)(*nph);
    *first = 2 * north * (north - 1);
  } else {
    cz = (double)(2 * nside - north) * (2.0 / (3.0 * nside));
    sz = sqrt((1.0 - cz) * (1.0 + cz));
    *nph = 4 * nside;
    *phi0 = ((north - nside) & 1) ? 0.0 : M_PI / (double)(*nph);
    *first = ncap + (north - nside) * (*nph);
  }
  if (north != ir) {
    cz = -cz;
    *first = npix - *nph - *first;
  }
  *z = cz;
  *sth = sz;
}

long orc_nalms(int lmax) { return ((long)(lmax + 1) * (lmax + 2)) / 2; }
long orc_indexlm(int l, int m, int lmax) { return m > 0 ? l + (long)m * lmax - ((long)m * (m - 1)) / 2 : l; }

/* lambda_lm(theta) for l = m .. lmax into out[l - m] */
void orc_lambda_m(int lmax, int m, double z, double sth, double *out)
{
  double lg = 0.5 * log2((2.0 * m + 1.0) / (4.0 * M_PI));
  for (int k = 1; k <= m; k++) lg += 0.5 * log2((2.0 * k - 1.0) / (2.0 * k));
  if (m > 0) lg += m * log2(sth);
  int e = (int)floor(lg);
  double p1 = exp2(lg - e), p2 = 0.0;
  if (m & 1) p1 = -p1;
  out[0] = ldexp(p1, e);
  for (int l = m + 1; l <= lmax; l++) {
    const double a = sqrt((4.0 * l * l - 1.0) / ((double)(l - m) * (l + m)));
    const double b = sqrt(((double)(l - 1) * (l - 1) - (double)m * m) / (4.0 * (l - 1) * (l - 1) - 1.0));
    const double p = a * (z * p1 - b * p2);
    p2 = p1;
    p1 = p;
    if (fabs(p1) > 0x1p300) {
      p1 *= 0x1p-300;
      p2 *= 0x1p-300;
      e += 300;
    }
    out[l - m] = ldexp(p1, e);
  }
}

/* e^{-i m phi_j} sums of one ring for m = 0 .. lmax (f: 2 (lmax+1) doubles) */
static void ring_analysis(const double *px, long nph, double phi0, int lmax, double *f)
{
  for (int m = 0; m <= lmax; m++) {
    double re = 0, im = 0;
    long idx = 0;
    const long step = m % nph;
    for (long j = 0; j < nph; j++) {
      const double ang = 2.0 * M_PI * (double)idx / (double)nph;
      re += px[j] * cos(ang);
      im -= px[j] * sin(ang);
      idx += step;
      if (idx >= nph) idx -= nph;
    }
    const double a0 = M_PI * (double)(m % (2 * nph)) / (double)nph * (phi0 > 0 ? 1.0 : 0.0);
    const double c = cos(a0), s = sin(a0);
    f[2 * m] = re * c + im * s; /* (re + i im) e^{-i m phi0} */
    f[2 * m + 1] = im * c - re * s;
  }
}

void orc_map2alm(long nside, int lmax, const double *map, double *alm)
{
  const long npix = 12 * nside * nside;
  const double w = 4.0 * M_PI / (double)npix;
  memset(alm, 0, sizeof(double) * 2 * orc_nalms(lmax));
  double *f = malloc(sizeof(double) * 2 * (lmax + 1));
  double *lam = malloc(sizeof(double) * (lmax + 1));
  for (long r = 0; r < 4 * nside - 1; r++) {
    long first, nph;
    double z, sth, phi0;
    orc_ring_info(nside, r, &first, &nph, &z, &sth, &phi0);
    ring_analysis(map + first, nph, phi0, lmax, f);
    for (int m = 0; m <= lmax; m++) {
      orc_lambda_m(lmax, m, z, sth, lam);
      for (int l = m; l <= lmax; l++) {
        const long i = orc_indexlm(l, m, lmax);
        alm[2 * i] += w * lam[l - m] * f[2 * m];
        alm[2 * i + 1] += w * lam[l - m] * f[2 * m + 1];
      }
    }
  }
  free(f);
  free(lam);
}

void orc_alm2map(long nside, int lmax, const double *alm, double *map)
{
  double *g = malloc(sizeof(double) * 2 * (lmax + 1));
  double *lam = malloc(sizeof(double) * (lmax + 1));
  for (long r = 0; r < 4 * nside - 1; r++) {
    long first, nph;
    double z, sth, phi0;
    orc_ring_info(nside, r, &first, &nph, &z, &sth, &phi0);
    for (int m = 0; m <= lmax; m++) {
      orc_lambda_m(lmax, m, z, sth, lam);
      double re = 0, im = 0;
      for (int l = m; l <= lmax; l++) {
        const long i = orc_indexlm(l, m, lmax);
        re += lam[l - m] * alm[2 * i];
        im += lam[l - m] * alm[2 * i + 1];
      }
      g[2 * m] = re;
      g[2 * m + 1] = im;
    }
    for (long j = 0; j < nph; j++) {
      double v = 0;
      for (int m = 0; m <= lmax; m++) {
        /* angle m (phi0 + 2 pi j / nph), reduced exactly: phi0 is 0 or pi/nph */
        const long k = (phi0 > 0 ? 1 : 0) + 2 * j;
        const long t = (long)(((long long)m * k) % (2 * nph));
        const double ang = M_PI * (double)t / (double)nph;
        const double c = cos(ang), s = sin(ang);
        v += (m == 0 ? 1.0 : 2.0) * (g[2 * m] * c - g[2 * m + 1] * s);
      }
      map[first + j] = v;
    }
  }
  free(g);
  free(lam);
}

/* src/healpix_extra.c:318-388 with nest = 0 (RING in and out) */
void orc_udgrade(const float *map_in, long nside_in, float *map_out, long nside_out)
{
  const long npix_in = 12 * nside_in * nside_in, npix_out = 12 * nside_out * nside_out;
  if (nside_in == nside_out) {
    memcpy(map_out, map_in, sizeof(float) * npix_out);
  } else if (nside_in > nside_out) {
    const long ratio = npix_in / npix_out;
    const double inv = 1.0 / (double)ratio;
    for (long i = 0; i < npix_out; i++) {
      const long nest_out = orc_ring2nest(nside_out, i);
      double tot = 0;
      for (long j = 0; j < ratio; j++) tot += map_in[orc_nest2ring(nside_in, j + ratio * nest_out)];
      map_out[i] = (float)(tot * inv);
    }
  } else {
    const long ratio = npix_out / npix_in;
    for (long i = 0; i < npix_in; i++) {
      const long nest_in = orc_ring2nest(nside_in, i);
      const float v = map_in[i];
      for (long j = 0; j < ratio; j++) map_out[orc_nest2ring(nside_out, j + nest_in * ratio)] = v;
    }
  }
}

/* src/healpix_extra.c:390-400: FWHM (arcmin) -> exp(-l(l+1) sigma^2 / 2) */
#define ORC_FWHM2SIGMA 0.00012352884853326381
void orc_beam_window(int lmax, double fwhm_amin, double *beam)
{
  const double sigma = ORC_FWHM2SIGMA * fwhm_amin;
  for (long l = 0; l <= lmax; l++) beam[l] = exp(-0.5 * l * (l + 1) * sigma * sigma);
}

/* src/main_jt.c:202-238 with single-precision maps and a_lm (the reference's
 * _SPREC build): each map is transformed in FP64, its a_lm rounded to float,
 * scaled by the beam (float * double -> float, src/healpix_extra.c:402-421),
 * synthesised in FP64 and rounded to float.  lmax = 3 nside - 1. */
void orc_apply_beam(long nside, int n_maps, const double *fwhm_amin, float *maps)
{
  const int lmax = (int)(3 * nside - 1);
  const long npix = 12 * nside * nside, nalm = orc_nalms(lmax);
  double *md = malloc(sizeof(double) * npix), *ad = malloc(sizeof(double) * 2 * nalm);
  double *beam = malloc(sizeof(double) * (lmax + 1));
  for (int c = 0; c < n_maps; c++) {
    float *mp = maps + (long)c * npix;
    for (long i = 0; i < npix; i++) md[i] = mp[i];
    orc_map2alm(nside, lmax, md, ad);
    orc_beam_window(lmax, fwhm_amin[c], beam);
    for (int m = 0; m <= lmax; m++)
      for (int l = m; l <= lmax; l++) {
        const long i = orc_indexlm(l, m, lmax);
        ad[2 * i] = (double)(float)((double)(float)ad[2 * i] * beam[l]);
        ad[2 * i + 1] = (double)(float)((double)(float)ad[2 * i + 1] * beam[l]);
      }
    orc_alm2map(nside, lmax, ad, md);
    for (long i = 0; i < npix; i++) mp[i] = (float)md[i];
  }
  free(md);
  free(ad);
  free(beam);
}

#define ORC_PREFAC_TNU 3.6E9 /* src/main_jt.c:25 */

/* src/main_jt.c:263-317: per emulated OpenMP thread t an MT19937 seeded
 * seed + t draws the channels of t's static block, pixel by pixel:
 * phase = 2 pi u1, modulus = sqrt(-sigma2 log(1 - u2)), noise = modulus cos(phase). */
void orc_add_noise(long nside, int n_nu, const double *nu0, const double *nuf, double fsky, double tsys,
                   double time_tot, int n_dish, unsigned int seed, int nthreads, float *maps)
{
  const long npix = 12 * nside * nside;
  if (nthreads < 1) nthreads = 1;
  for (int t = 0; t < nthreads; t++) {
    int q = n_nu / nthreads, r = n_nu % nthreads, i0;
    if (t < r) {
      q++;
      i0 = q * t;
    } else
      i0 = q * t + r;
    orc_mt rng;
    orc_mt_seed(&rng, seed + (unsigned)t);
    for (int inu = i0; inu < i0 + q; inu++) {
      const double dnu = nuf[inu] - nu0[inu];
      const double n_el = fsky * npix;
      const double s2 = n_el * tsys * tsys / (ORC_PREFAC_TNU * dnu * time_tot * n_dish);
      float *mp = maps + (long)inu * npix;
      for (long i = 0; i < npix; i++) {
        const double phase = 2 * M_PI * orc_mt_uniform(&rng);
        const double u = orc_mt_uniform(&rng);
        const double mod = sqrt(-s2 * log(1 - u));
        mp[i] = (float)((double)mp[i] + mod * cos(phase));
      }
    }
  }
}
