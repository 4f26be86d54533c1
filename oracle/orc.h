/*
 * Oracle for the GetHI realisation path -- TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C restatement of the reference algorithm (damonge/CRIME, GetHI) used
 * as the checker for the GPU path.  Only tests/, __graft_entry__.smoke() and
 * bench.py's CPU-baseline leg may load it; the product library never links it.
 *
 * Parity pin: the restatement is checked against golden vectors produced by the
 * reference's own C sources (src/fourier.c, grid_tools.c, pixelize.c, cosmo.c,
 * cosmo_mad.c, io_gh.c, common.c) compiled here against project-written shims
 * for GSL, FFTW, chealpix and cfitsio (oracle/Makefile, target `ref`).  The
 * third-party algorithms behind those shims (MT19937 seeding of GSL, GSL
 * quadrature, FFTW's c2r, chealpix's vec2pix_ring) are restated from their
 * published descriptions; parity with the real libraries is unpinned.
 *
 * Grid layout used here is the reference's: real grids are [z][y][2(N/2+1)]
 * floats (FFTW in-place padding, src/fourier.c:169-192), half spectra are
 * [kz][ky][N/2+1] complex floats.
 */
#ifndef ORC_H
#define ORC_H
#include <stdint.h>

#define ORC_NZ 5001          /* src/common_gh.h:34 */
#define ORC_DZ 0.001         /* src/common_gh.h:33 */
#define ORC_NU21 1420.40575177 /* src/common.h:38 */
#define ORC_NSUB 10          /* src/pixelize.c:25 */
#define ORC_HMPC 2997.92458  /* src/cosmo_mad.h:35 */
#define ORC_NZ_PS 256        /* src/common_gh.h:35 */
#define ORC_NL_PS 256        /* src/psources.c:24 */

#ifdef __cplusplus
extern "C" {
#endif

/* Run configuration (the .ini keys of src/io_gh.c:211-249 plus the new keys). */
typedef struct {
  double OmegaM, OmegaL, OmegaB, hhub, weos, n_scal, sig8;
  double r_smooth;        /* as written in the ini; squared when > 0 (io_gh.c:255-260) */
  double nu_min, nu_max;  /* regular table bounds; overwritten from the edges otherwise */
  double l_box_override;  /* > 0: use this box side instead of 2 r_max (1+2/N) */
  double b_HI;            /* bias when bias_const != 0 */
  long n_side;
  int n_grid;
  int n_nu;
  unsigned int seed;
  int regular_nu;         /* 1: (int)(inv_dnu (nu-nu_min)) binning (pixelize.c:216) */
  int bias_const;         /* 0: bias_HI(z) of src/user_defined.c:32-35 */
  int do_rsd;             /* 0: dz_rsd forced to 0 */
  int pad_;
} orc_config;

/* Derived quantities (the derived members of ParamGetHI, src/common_gh.h:67-116). */
typedef struct {
  double fgrowth_0, hubble_0, z_min, z_max, r_min, r_max, l_box;
  double pos_obs[3];
  double r2_smooth;
  double glob_idr;
  double logkmin, logkmax, idlogk, n_scal;
  double sigma8_in;      /* sigma_8 of the table before renormalisation */
  double pk_norm;         /* factor applied to the table */
  int do_smoothing;
  int numk;
  double z_z2r[ORC_NZ], r_z2r[ORC_NZ];
  double z_r2z[ORC_NZ], r_r2z[ORC_NZ];
  double gd[ORC_NZ], gv[ORC_NZ];
} orc_derived;

/* ---- cosmology (src/cosmo.c, src/cosmo_mad.c) ---- */
int orc_cosmo_set(const orc_config *c, int numk, const double *k_in, const double *pk_in,
                  double *logk_out, double *pk_out, orc_derived *d);
double orc_z_of_r(const orc_derived *d, double r);
double orc_r_of_z(const orc_derived *d, double z);
double orc_dgrowth_of_r(const orc_derived *d, double r);
double orc_vgrowth_of_r(const orc_derived *d, double r);
double orc_pk_linear0(const orc_derived *d, const double *logk, const double *pk, double lgk);
double orc_integrate(double (*f)(double, void *), void *p, double a, double b);
double orc_integrate_lower_inf(double (*f)(double, void *), void *p, double b);

/* ---- random numbers ---- */
typedef struct { uint32_t mt[624]; int mti; } orc_mt;
void orc_mt_seed(orc_mt *s, uint32_t seed);
uint32_t orc_mt_next(orc_mt *s);
double orc_mt_uniform(orc_mt *s);
void orc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);

/* ---- Fourier-space fields ---- */
/* Reference modes (src/fourier.c:234-305) with the MT19937 draws of `nthreads`
 * emulated OpenMP threads (libgomp static partition of the kz planes). */
void orc_modes_mt(const orc_config *c, const orc_derived *d, const double *logk,
                  const double *pk, int nthreads, float *dens_k, float *vpot_k);
/* Counter-based production modes (same amplitude law, Philox4x32-10 draws). */
void orc_pk_grid(const orc_config *c, const orc_derived *d, const double *logk, const double *pk,
                 double *out);
void orc_modes_philox_pg(const orc_config *c, const orc_derived *d, const double *logk,
                         const double *pk, const double *pg, float *dens_k);
void orc_modes_philox(const orc_config *c, const orc_derived *d, const double *logk,
                      const double *pk, float *dens_k);

/* ---- FFT (FP64 internally) ---- */
void orc_c2r_inplace(int n, float *data);                     /* padded in-place c2r */
void orc_c2r_to_double(int n, const float *spec, double *out); /* out: N^3 compact */
void orc_normalize(int n, double l_box, float *data);          /* fourier.c:397-412 */

/* ---- real-space stages ---- */
void orc_radial_velocity_fd(const orc_config *c, const orc_derived *d, const float *vpot,
                            float *rvel);                       /* fourier.c:307-373 */
void orc_radial_velocity_spectral(const orc_config *c, const orc_derived *d, const float *dens_k,
                                  float *rvel);
void orc_sigma_dens(int n, const float *dens, double *mean, double *sigma2); /* fourier.c:24-76 */
void orc_get_hi(const orc_config *c, const orc_derived *d, double sigma2, float *dens,
                float *rvel);                                   /* grid_tools.c:103-153 */

/* ---- projection (src/pixelize.c:150-286) ---- */
void orc_subsample_offsets(unsigned int seed, double lcell, double *xs, double *ys, double *zs);
long orc_vec2pix_ring(long nside, const double *v);
void orc_pix2ang_ring(long nside, long ipix, double *theta, double *phi);
int orc_get_inu(const double *nu0, const double *nuf, int n_nu, double nu, int inu_start);
/* keys (optional, N^3*10 entries, 0xFFFFFFFF = dropped) are bin*npix+pix. */
void orc_mk_T_maps(const orc_config *c, const orc_derived *d, const double *nu0,
                   const double *nuf, const float *mass, const float *dz, float *maps,
                   uint32_t *keys);
void orc_channel_prefactors(const orc_config *c, const orc_derived *d, const double *nu0,
                            const double *nuf, double *prefac);

/* ---- whole realisation (CPU baseline) ---- */
int orc_num_threads(void);
void orc_set_threads(int t);

/* Point sources (src/psources.c, grid_tools.c:24-101, pixelize.c:58-148); orc_psources.c */
void orc_setup_psources(double z_max, double *nz_arr, double *maxpdf, double *glob_dz);
double orc_n_of_z_psources(const double *nz_arr, double glob_dz, double z);
long orc_poisson_small(orc_mt *r, double mu);
double orc_temp_of_l(double hhub, double L0, double nu_obs, double z, double r, double dOmega);
long orc_point_sources(const orc_config *c, const orc_derived *d, const double *nz_arr, double glob_dz,
                       const float *dens, double sigma2, int nthreads, int *nsources);
void orc_ps_lambda(const orc_config *c, const orc_derived *d, const double *nz_arr, double glob_dz,
                   const float *dens, double sigma2, double *lam);
void orc_psources_maps(const orc_config *c, const orc_derived *d, const double *nu0, const double *nuf,
                       const double *nz_arr, const double *maxpdf, double glob_dz, const int *nsources,
                       const float *dz, int nthreads, float *maps_ps);
void orc_psources_maps_catalogue(const orc_config *c, const orc_derived *d, const double *nu0, const double *nuf,
                                 long ns, const int64_t *cell, const double *u, const double *L0,
                                 const double *dzs, double *maps_ps, int64_t *pix);

/* JoinT map combination (src/main_jt.c:98-321, src/healpix_extra.c:31-43,318-421); orc_joint.c */
long orc_nest2ring(long nside, long ipnest);
long orc_ring2nest(long nside, long ipring);
void orc_ring_info(long nside, long ring, long *first, long *nph, double *z, double *sth, double *phi0);
long orc_nalms(int lmax);
long orc_indexlm(int l, int m, int lmax);
void orc_lambda_m(int lmax, int m, double z, double sth, double *out);
void orc_map2alm(long nside, int lmax, const double *map, double *alm);
void orc_alm2map(long nside, int lmax, const double *alm, double *map);
void orc_udgrade(const float *map_in, long nside_in, float *map_out, long nside_out);
void orc_beam_window(int lmax, double fwhm_amin, double *beam);
void orc_apply_beam(long nside, int n_maps, const double *fwhm_amin, float *maps);
void orc_add_noise(long nside, int n_nu, const double *nu0, const double *nuf, double fsky, double tsys,
                   double time_tot, int n_dish, unsigned int seed, int nthreads, float *maps);

#ifdef __cplusplus
}
#endif
#endif
