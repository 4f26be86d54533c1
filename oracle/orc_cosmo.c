/*
 * Oracle (test infrastructure only): background cosmology, distance/growth
 * tables and P(k) normalisation.  Restates src/cosmo.c:27-413 and
 * src/cosmo_mad.c:160-507 of the reference.  The GSL quadratures used there
 * (qng, qagil) are replaced by an adaptive Gauss-Legendre rule converged to
 * ~1e-13 relative, i.e. the value GSL approximates to its requested tolerance.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include "orc.h"

#define TWOPIPIINVLOGTEN 0.1166503235296796 /* src/common_gh.h:31 */

/* ------------------------------------------------------------------ */
/* adaptive Gauss-Legendre quadrature                                  */
/* ------------------------------------------------------------------ */
#define GL_N 20
static double gl_x[GL_N], gl_w[GL_N];
static int gl_ready = 0;

static void gl_setup(void)
{
  if (gl_ready) return;
  for (int i = 0; i < GL_N; i++) {
    double x = cos(M_PI * (i + 0.75) / (GL_N + 0.5)), dp = 0;
    for (int it = 0; it < 100; it++) {
      double p0 = 1, p1 = x;
      for (int k = 2; k <= GL_N; k++) {
        double p2 = ((2 * k - 1) * x * p1 - (k - 1) * p0) / k;
        p0 = p1; p1 = p2;
      }
      dp = GL_N * (x * p1 - p0) / (x * x - 1);
      double dx = p1 / dp;
      x -= dx;
      if (fabs(dx) < 1e-16) break;
    }
    gl_x[i] = x;
    gl_w[i] = 2 / ((1 - x * x) * dp * dp);
  }
  gl_ready = 1;
}

typedef double (*orc_fn)(double, void *);

static double gl_panel(orc_fn f, void *p, double a, double b)
{
  double h = 0.5 * (b - a), m = 0.5 * (b + a), s = 0;
  for (int i = 0; i < GL_N; i++) s += gl_w[i] * f(m + h * gl_x[i], p);
  return s * h;
}

/* Bisect until the two halves agree with the whole panel to 1e-13 relative or
 * to epsabs (1e-16 of the whole integral), which bounds the work where the
 * integrand underflows or jumps. */
static double gl_adapt(orc_fn f, void *p, double a, double b, double whole, double epsabs, int depth)
{
  double m = 0.5 * (a + b);
  double l = gl_panel(f, p, a, m), r = gl_panel(f, p, m, b);
  double s = l + r;
  if (depth >= 48 || fabs(s - whole) <= 1e-13 * fabs(s) + epsabs) return s;
  return gl_adapt(f, p, a, m, l, epsabs, depth + 1) + gl_adapt(f, p, m, b, r, epsabs, depth + 1);
}

static double integrate_eps(orc_fn f, void *p, double a, double b, double epsabs)
{
  gl_setup();
  return gl_adapt(f, p, a, b, gl_panel(f, p, a, b), epsabs, 0);
}

static double integrate(orc_fn f, void *p, double a, double b)
{
  gl_setup();
  double coarse = 0;
  for (int i = 0; i < 8; i++) coarse += gl_panel(f, p, a + (b - a) * i / 8, a + (b - a) * (i + 1) / 8);
  return integrate_eps(f, p, a, b, 1e-16 * fabs(coarse));
}

double orc_integrate(double (*f)(double, void *), void *p, double a, double b)
{
  return integrate(f, p, a, b);
}

/* integral over (-inf, b] through x = b - (1-t)/t, t in (0,1] (the map GSL's
 * qagil uses), split into fixed panels before adaptive refinement */
typedef struct { double (*f)(double, void *); void *p; double b; } lowinf_t;
static double lowinf_integrand(double t, void *q)
{
  lowinf_t *s = (lowinf_t *)q;
  return s->f(s->b - (1 - t) / t, s->p) / (t * t);
}

double orc_integrate_lower_inf(double (*f)(double, void *), void *p, double b)
{
  lowinf_t s = {f, p, b};
  enum { NSEG = 64 };
  double lo[NSEG + 1], hi[NSEG + 1], coarse = 0, acc = 0;
  gl_setup();
  lo[0] = 1e-12; hi[0] = 1e-3;
  for (int i = 0; i < NSEG; i++) {
    lo[i + 1] = 1e-3 + (1 - 1e-3) * i / NSEG;
    hi[i + 1] = 1e-3 + (1 - 1e-3) * (i + 1) / NSEG;
  }
  for (int i = 0; i <= NSEG; i++) coarse += gl_panel(lowinf_integrand, &s, lo[i], hi[i]);
  for (int i = 0; i <= NSEG; i++) acc += integrate_eps(lowinf_integrand, &s, lo[i], hi[i], 1e-16 * fabs(coarse));
  return acc;
}

/* ------------------------------------------------------------------ */
/* background (src/cosmo_mad.c)                                       */
/* ------------------------------------------------------------------ */
typedef struct {
  double OM, OL, OK, w0, wa;
  int ksign, normalDE, constantw;
  double a_equality, phorizon;
} bg_t;

static double e2a3(const bg_t *b, double a) /* OM + OL*a^(-3w)... + OK*a */
{
  if (b->normalDE) return b->OM + b->OL * a * a * a + b->OK * a;
  if (b->constantw) return b->OM + b->OL * pow(a, -3 * b->w0) + b->OK * a;
  return b->OM + b->OL * pow(a, -3 * (b->w0 + b->wa)) * exp(3 * (a - 1) * b->wa) + b->OK * a;
}

static double naHm1(double a, void *p) { return sqrt(a / e2a3((bg_t *)p, a)); }      /* cosmo_mad.c:199-217 */
static double na2Hm1(double a, void *p) { return 1 / sqrt(a * e2a3((bg_t *)p, a)); } /* cosmo_mad.c:219-237 */
static double naHm3(double a, void *p)                                              /* cosmo_mad.c:239-258 */
{
  double d = sqrt(a / e2a3((bg_t *)p, a));
  return d * d * d;
}

static double parthor(const bg_t *b, double aa) /* cosmo_mad.c:260-289 */
{
  double alim = 0.01 * b->a_equality;
  if (aa <= alim) return 2 * sqrt(aa / b->OM) * ORC_HMPC;
  double int0 = 2 * sqrt(alim / b->OM);
  return (int0 + integrate(na2Hm1, (void *)b, alim, aa)) * ORC_HMPC;
}

static double gfac(const bg_t *b, double aa) /* cosmo_mad.c:291-319 */
{
  double alim = 0.01 * b->a_equality;
  double int0 = 0.4 * sqrt(alim * alim * alim * alim * alim / (b->OM * b->OM * b->OM));
  if (aa <= alim) return aa;
  double integral = integrate(naHm3, (void *)b, alim, aa);
  return (int0 + integral) * 2.5 * b->OM / (aa * naHm1(aa, (void *)b));
}

static double hubble(const bg_t *b, double aa) /* cosmo_mad.c:321-337 */
{
  return sqrt(e2a3(b, aa) / (aa * aa * aa)) / ORC_HMPC;
}

static double f_growth(const bg_t *b, double aa) /* cosmo_mad.c:385-409 */
{
  double apow, coeff, Da = gfac(b, aa);
  if (b->normalDE) { coeff = 0; apow = aa * aa * aa; }
  else if (b->constantw) { coeff = 1 + b->w0; apow = pow(aa, -3 * b->w0); }
  else {
    coeff = 1 + b->w0 + b->wa * (1 - aa);
    apow = pow(aa, -3 * (b->w0 + b->wa)) * exp(3 * b->wa * (aa - 1));
  }
  return 0.5 * (5 * b->OM * aa / Da - (3 * b->OM + 3 * coeff * b->OL * apow + 2 * b->OK * aa)) /
         (b->OM + b->OL * apow + b->OK * aa);
}

static double chi(const bg_t *b, double aa) { return b->phorizon - parthor(b, aa); } /* cosmo_mad.c:349-357 */

static int bg_set(bg_t *b, double OM, double OL, double w0) /* cosmo_mad.c:411-507 */
{
  memset(b, 0, sizeof(*b));
  b->OM = OM; b->OL = OL; b->w0 = w0; b->wa = 0; b->OK = 1 - OM - OL;
  if (fabs(b->w0 + 1) < 1e-6) { b->constantw = 1; b->normalDE = 1; }
  else { b->constantw = 1; b->normalDE = 0; }
  if (fabs(b->OK) < 1e-6) b->ksign = 0;
  else if (b->OK > 0) b->ksign = -1;
  else b->ksign = 1;
  if (b->OM <= 0 || b->w0 > -0.333333) return -1;
  /* aeqmin, cosmo_mad.c:160-179 */
  double aeqK = 1, aeqL = 1;
  if (b->ksign != 0) aeqK = b->OM / fabs(b->OK);
  if (b->OL != 0) aeqL = b->normalDE ? pow(b->OM / b->OL, 0.333) : pow(b->OM / b->OL, -1 / (3 * b->w0));
  b->a_equality = aeqK < aeqL ? aeqK : aeqL;
  b->phorizon = parthor(b, 1);
  return 0;
}

/* ------------------------------------------------------------------ */
/* table lookups (src/cosmo.c:27-86)                                  */
/* ------------------------------------------------------------------ */
static double z_of_r_provisional(const orc_derived *d, double r)
{
  if (r <= 0) return 0;
  if (r >= d->r_z2r[ORC_NZ - 1]) return d->z_z2r[ORC_NZ - 1];
  int iz = 0;
  while (r >= d->r_z2r[iz]) iz++;
  return d->z_z2r[iz - 1] + (d->z_z2r[iz] - d->z_z2r[iz - 1]) * (r - d->r_z2r[iz - 1]) /
                                (d->r_z2r[iz] - d->r_z2r[iz - 1]);
}

double orc_r_of_z(const orc_derived *d, double z)
{
  if (z <= 0) return 0;
  if (z >= d->z_z2r[ORC_NZ - 1]) return d->r_z2r[ORC_NZ - 1];
  int iz = (int)(z / ORC_DZ);
  return d->r_z2r[iz] + (d->r_z2r[iz + 1] - d->r_z2r[iz]) * (z - d->z_z2r[iz]) / ORC_DZ;
}

double orc_z_of_r(const orc_derived *d, double r)
{
  if (r <= 0) return 0;
  if (r >= d->r_r2z[ORC_NZ - 1]) return d->z_r2z[ORC_NZ - 1];
  int ir = (int)(r * d->glob_idr);
  return d->z_r2z[ir] + (d->z_r2z[ir + 1] - d->z_r2z[ir]) * (r - d->r_r2z[ir]) * d->glob_idr;
}

double orc_dgrowth_of_r(const orc_derived *d, double r)
{
  if (r <= 0) return 1;
  if (r >= d->r_r2z[ORC_NZ - 1]) return d->gd[ORC_NZ - 1];
  int ir = (int)(r * d->glob_idr);
  return d->gd[ir] + (d->gd[ir + 1] - d->gd[ir]) * (r - d->r_r2z[ir]) * d->glob_idr;
}

double orc_vgrowth_of_r(const orc_derived *d, double r)
{
  if (r <= 0) return 1;
  if (r >= d->r_r2z[ORC_NZ - 1]) return d->gv[ORC_NZ - 1];
  int ir = (int)(r * d->glob_idr);
  return d->gv[ir] + (d->gv[ir + 1] - d->gv[ir]) * (r - d->r_r2z[ir]) * d->glob_idr;
}

/* P(k) lookup, src/cosmo.c:153-170.  The reference reads pkarr[numk] when
 * ik == numk-1; that case takes the k^-3 tail here (documented deviation). */
double orc_pk_linear0(const orc_derived *d, const double *logk, const double *pk, double lgk)
{
  int ik = (int)((lgk - d->logkmin) * d->idlogk);
  if (ik < 0) return pk[0] * pow(10, d->n_scal * (lgk - d->logkmin));
  if (ik < d->numk - 1)
    return pk[ik] + (lgk - logk[ik]) * (pk[ik + 1] - pk[ik]) * d->idlogk;
  return pk[d->numk - 1] * pow(10, -3 * (lgk - d->logkmax));
}

/* ------------------------------------------------------------------ */
/* sigma_8 normalisation (src/cosmo.c:127-339)                        */
/* ------------------------------------------------------------------ */
static double wind_tophat(double x) /* cosmo.c:127-151, setwf=0 */
{
  if (x < 0.1)
    return 1. - 0.1 * x * x + 0.003571429 * x * x * x * x - 6.61376E-5 * x * x * x * x * x * x +
           7.51563E-7 * x * x * x * x * x * x * x * x;
  return 3 * (sin(x) - x * cos(x)) / (x * x * x);
}

typedef struct {
  const orc_derived *d;
  const double *logk, *pk;
  double R;
} sig_t;

/* integxiL_NO at r=0 (cosmo.c:212-230; j_bessel_0(0) = 1) */
static double sig_integrand(double lgk, void *p)
{
  sig_t *s = (sig_t *)p;
  double kk = pow(10, lgk);
  double w = wind_tophat(kk * s->R);
  return TWOPIPIINVLOGTEN * orc_pk_linear0(s->d, s->logk, s->pk, lgk) * kk * kk * kk * w * w;
}

/* sigL2(R,R,TopHat,TopHat) = xi2p_L at r=0, which takes the qagil branch (cosmo.c:271-276) */
static double sigL2_tophat(const orc_derived *d, const double *logk, const double *pk, double R)
{
  sig_t s = {d, logk, pk, R};
  return orc_integrate_lower_inf(sig_integrand, &s, d->logkmax);
}

int orc_cosmo_set(const orc_config *c, int numk, const double *k_in, const double *pk_in,
                  double *logk_out, double *pk_out, orc_derived *d)
{
  bg_t b;
  memset(d, 0, sizeof(*d));
  if (bg_set(&b, c->OmegaM, c->OmegaL, c->weos)) return -1;
  if (c->OmegaM < c->OmegaB) return -1;

  d->fgrowth_0 = f_growth(&b, 1);
  d->hubble_0 = hubble(&b, 1);
  d->z_min = ORC_NU21 / c->nu_max - 1;
  d->z_max = ORC_NU21 / c->nu_min - 1;
  d->r_min = chi(&b, 1 / (1 + d->z_min));
  d->r_max = chi(&b, 1 / (1 + d->z_max));
  d->l_box = 2 * d->r_max * (1 + 2. / c->n_grid);
  if (c->l_box_override > 0) d->l_box = c->l_box_override;
  d->pos_obs[0] = d->pos_obs[1] = d->pos_obs[2] = 0.5 * d->l_box;

  for (int ii = 0; ii < ORC_NZ; ii++) {
    double z = ((double)ii) * ORC_DZ;
    d->z_z2r[ii] = z;
    d->r_z2r[ii] = chi(&b, 1 / (1 + z));
  }
  if (d->z_z2r[ORC_NZ - 1] <= d->z_max || d->r_z2r[ORC_NZ - 1] <= d->r_max) return -2;

  double growth0 = gfac(&b, 1);
  d->glob_idr = (ORC_NZ - 1) / (d->r_z2r[ORC_NZ - 1] - d->r_z2r[0]);
  for (int ii = 0; ii < ORC_NZ; ii++) {
    double r = ii / d->glob_idr;
    double z = z_of_r_provisional(d, r);
    double a = 1 / (1 + z);
    d->z_r2z[ii] = z;
    d->r_r2z[ii] = r;
    double gz = gfac(&b, a) / growth0;
    double fz = f_growth(&b, a);
    double hz = hubble(&b, a);
    d->gd[ii] = gz;
    d->gv[ii] = (gz * hz * fz) / (d->fgrowth_0 * d->hubble_0);
  }
  if (d->z_r2z[ORC_NZ - 1] <= d->z_max || d->r_r2z[ORC_NZ - 1] <= d->r_max) return -2;

  /* io_gh.c:255-260 */
  if (c->r_smooth > 0) { d->r2_smooth = c->r_smooth * c->r_smooth; d->do_smoothing = 1; }
  else { d->r2_smooth = c->r_smooth; d->do_smoothing = 0; }

  /* pk_linear_set, cosmo.c:306-339 */
  d->numk = numk;
  d->n_scal = c->n_scal;
  for (int i = 0; i < numk; i++) { pk_out[i] = pk_in[i]; logk_out[i] = log10(k_in[i]); }
  d->logkmin = logk_out[0];
  d->logkmax = logk_out[numk - 1];
  d->idlogk = (numk - 1) / (logk_out[numk - 1] - logk_out[0]);
  double s2 = sigL2_tophat(d, logk_out, pk_out, 8);
  d->sigma8_in = sqrt(s2);
  d->pk_norm = c->sig8 * c->sig8 / s2;
  for (int i = 0; i < numk; i++) pk_out[i] *= d->pk_norm;
  return 0;
}
