/*
 * Test-infrastructure shim implementations that let the reference's GetHI
 * sources (src/common.c, common_gh.c, cosmo.c, cosmo_mad.c, fourier.c,
 * grid_tools.c, pixelize.c, io_gh.c, user_defined.c) build and run here.
 * GSL RNG -> oracle MT19937; GSL quadrature -> oracle Gauss-Legendre; FFTW
 * c2r -> oracle FP64 FFT (rounded to float on output); chealpix -> oracle
 * RING restatement.  Each FFT input is also copied aside so the driver can
 * dump the Fourier-space modes before the in-place transform destroys them.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include "common_gh.h"
#include <gsl/gsl_integration.h>
#include <gsl/gsl_errno.h>
#include <gsl/gsl_randist.h>
#include <chealpix.h>
#include "orc.h"

/* ---- GSL RNG ---- */
struct gsl_rng { orc_mt mt; };
static const gsl_rng_type mt_type = {"mt19937"};
const gsl_rng_type *gsl_rng_mt19937 = &mt_type;
gsl_rng *gsl_rng_alloc(const gsl_rng_type *T) { (void)T; return (gsl_rng *)calloc(1, sizeof(gsl_rng)); }
void gsl_rng_set(const gsl_rng *r, unsigned long int s) { orc_mt_seed((orc_mt *)&r->mt, (uint32_t)s); }
double gsl_rng_uniform(const gsl_rng *r) { return orc_mt_uniform((orc_mt *)&r->mt); }
void gsl_rng_free(gsl_rng *r) { free(r); }
/* GSL's gsl_ran_poisson for mu <= 10 (Knuth's multiplication method, restated in
 * orc_psources.c); the golden cases keep every cell's mean below 10 */
unsigned int gsl_ran_poisson(const gsl_rng *r, double mu)
{
  long k = orc_poisson_small((orc_mt *)&r->mt, mu);
  if (k < 0) {
    fprintf(stderr, "shim: gsl_ran_poisson with mu = %g > 10 is not restated\n", mu);
    abort();
  }
  return (unsigned int)k;
}

/* ---- GSL errors / quadrature ---- */
gsl_error_handler_t *gsl_set_error_handler_off(void) { return NULL; }
struct gsl_integration_workspace { int dummy; };
struct gsl_integration_qawo_table { int dummy; };
gsl_integration_workspace *gsl_integration_workspace_alloc(size_t n) { (void)n; return calloc(1, sizeof(gsl_integration_workspace)); }
void gsl_integration_workspace_free(gsl_integration_workspace *w) { free(w); }
gsl_integration_qawo_table *gsl_integration_qawo_table_alloc(double omega, double L,
                                                             enum gsl_integration_qawo_enum s, size_t n)
{ (void)omega; (void)L; (void)s; (void)n; return calloc(1, sizeof(gsl_integration_qawo_table)); }
void gsl_integration_qawo_table_free(gsl_integration_qawo_table *t) { free(t); }
int gsl_integration_qng(const gsl_function *f, double a, double b, double epsabs, double epsrel,
                        double *result, double *abserr, size_t *neval)
{
  (void)epsabs; (void)epsrel;
  *result = orc_integrate(f->function, f->params, a, b);
  *abserr = 0; *neval = 0;
  return 0;
}
int gsl_integration_qagil(gsl_function *f, double b, double epsabs, double epsrel, size_t limit,
                          gsl_integration_workspace *w, double *result, double *abserr)
{
  (void)epsabs; (void)epsrel; (void)limit; (void)w;
  *result = orc_integrate_lower_inf(f->function, f->params, b);
  *abserr = 0;
  return 0;
}
int gsl_integration_qawf(gsl_function *f, const double a, const double epsabs, const size_t limit,
                         gsl_integration_workspace *w, gsl_integration_workspace *cw,
                         gsl_integration_qawo_table *wf, double *result, double *abserr)
{
  (void)f; (void)a; (void)epsabs; (void)limit; (void)w; (void)cw; (void)wf; (void)result; (void)abserr;
  fprintf(stderr, "shim: qawf is not on the GetHI path\n");
  abort();
}

/* ---- FFTW ---- */
struct shim_fftwf_plan_s { int n; fftwf_complex *in; float *out; };
float *shim_captured[8];
int shim_ncaptured = 0;
fftwf_plan fftwf_plan_dft_c2r_3d(int n0, int n1, int n2, fftwf_complex *in, float *out, unsigned flags)
{
  (void)flags;
  if (n0 != n1 || n1 != n2) abort();
  fftwf_plan p = (fftwf_plan)malloc(sizeof(*p));
  p->n = n0; p->in = in; p->out = out;
  return p;
}
void fftwf_execute(const fftwf_plan p)
{
  int n = p->n;
  size_t nf = (size_t)n * n * (n / 2 + 1) * 2;
  if (shim_ncaptured < 8) {
    shim_captured[shim_ncaptured] = (float *)malloc(nf * sizeof(float));
    memcpy(shim_captured[shim_ncaptured], p->in, nf * sizeof(float));
    shim_ncaptured++;
  }
  if ((void *)p->in != (void *)p->out) abort(); /* the reference transforms in place */
  orc_c2r_inplace(n, (float *)p->in);
}
void fftwf_destroy_plan(fftwf_plan p) { free(p); }
fftwf_complex *fftwf_alloc_complex(size_t n) { return (fftwf_complex *)malloc(n * sizeof(fftwf_complex)); }
void fftwf_free(void *p) { free(p); }
int fftwf_init_threads(void) { return 1; }
void fftwf_plan_with_nthreads(int nthreads) { (void)nthreads; }
void fftwf_cleanup_threads(void) {}

/* ---- chealpix ---- */
void vec2pix_ring(long nside, const double *vec, long *ipix) { *ipix = orc_vec2pix_ring(nside, vec); }
long nside2npix(long nside) { return 12 * nside * nside; }

/* ---- healpix_extra.c entry point (FITS output is not on the tested path) ---- */
void he_write_healpix_map(float **tmap, int nfields, long nside, char *fname)
{ (void)tmap; (void)nfields; (void)nside; (void)fname; }
