/*
 * Test-infrastructure driver: runs the reference's GetHI stages
 * (src/main_gh.c:24-80 minus FITS output) and dumps every
 * stage's buffers as raw files, so the fixture script can turn them into
 * golden vectors.  Usage: gethi_ref <param.ini> <outdir>
 * With outdir "-" nothing is written and the wall time of each stage is
 * printed instead (the CPU baseline timing of oracle/time_ref.py).
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include "common_gh.h"
#include <omp.h>

extern float *shim_captured[8];
extern int shim_ncaptured;

static int timing;  /* outdir "-": no files, per-stage wall times on stdout */
static double t_last;

static void lap(const char *stage)
{
  const double t = omp_get_wtime();
  if (timing) printf("stage %s %.6f\n", stage, t - t_last);
  t_last = omp_get_wtime();
}

static void dump(const char *dir, const char *name, const void *p, size_t bytes)
{
  if (timing) return;
  char fn[1024];
  snprintf(fn, sizeof(fn), "%s/%s", dir, name);
  FILE *f = fopen(fn, "wb");
  if (!f) { perror(fn); exit(2); }
  fwrite(p, 1, bytes, f);
  fclose(f);
}

int main(int argc, char **argv)
{
  if (argc != 3) { fprintf(stderr, "usage: %s param.ini outdir\n", argv[0]); return 1; }
  mpi_init(&argc, &argv);
  timing = !strcmp(argv[2], "-");
  t_last = omp_get_wtime();
  ParamGetHI *par = read_run_params(argv[1]);
  lap("setup");
  const char *od = argv[2];
  int n = par->n_grid;
  size_t ngrid = (size_t)2 * (n / 2 + 1) * n * n;

  char fn[1024];
  snprintf(fn, sizeof(fn), "%s/params.txt", od);
  FILE *f = fopen(timing ? "/dev/null" : fn, "w");
  fprintf(f, "fgrowth_0 %.17g\nhubble_0 %.17g\nz_min %.17g\nz_max %.17g\nr_min %.17g\nr_max %.17g\n",
          par->fgrowth_0, par->hubble_0, par->z_min, par->z_max, par->r_min, par->r_max);
  fprintf(f, "l_box %.17g\npos_obs %.17g\nglob_idr %.17g\nr2_smooth %.17g\ndo_smoothing %d\n",
          par->l_box, par->pos_obs[0], par->glob_idr, par->r2_smooth, par->do_smoothing);
  fprintf(f, "numk %d\nlogkmin %.17g\nlogkmax %.17g\nidlogk %.17g\nn_nu %d\nnu_min %.17g\nnu_max %.17g\n",
          par->numk, par->logkmin, par->logkmax, par->idlogk, par->n_nu, par->nu_min, par->nu_max);
  fprintf(f, "n_grid %d\nn_side %ld\nseed %u\n", par->n_grid, par->n_side, par->seed_rng);
  double tabs[6 * NZ];
  memcpy(tabs + 0 * NZ, par->z_arr_z2r, sizeof(double) * NZ);
  memcpy(tabs + 1 * NZ, par->r_arr_z2r, sizeof(double) * NZ);
  memcpy(tabs + 2 * NZ, par->z_arr_r2z, sizeof(double) * NZ);
  memcpy(tabs + 3 * NZ, par->r_arr_r2z, sizeof(double) * NZ);
  memcpy(tabs + 4 * NZ, par->growth_d_arr, sizeof(double) * NZ);
  memcpy(tabs + 5 * NZ, par->growth_v_arr, sizeof(double) * NZ);
  dump(od, "tables.f64", tabs, sizeof(tabs));
  dump(od, "logk.f64", par->logkarr, sizeof(double) * par->numk);
  dump(od, "pk.f64", par->pkarr, sizeof(double) * par->numk);
#ifdef _IRREGULAR_NUTABLE
  dump(od, "nu0.f64", par->nu0_arr, sizeof(double) * par->n_nu);
  dump(od, "nuf.f64", par->nuf_arr, sizeof(double) * par->n_nu);
#endif

  lap("dumps");
  create_d_and_vr_fields(par);
  lap("create_d_and_vr_fields");
  fprintf(f, "sigma2_gauss %.17g\n", par->sigma2_gauss);
  if (par->do_psources) {  /* src/main_gh.c:55-58 */
    setup_psources(par);
    get_point_sources(par);
    fprintf(f, "glob_dz %.17g\n", par->glob_dz);
    dump(od, "ps_nz.f64", par->nz_psources_arr, sizeof(double) * NZ_PSOURCES);
    dump(od, "ps_maxpdf.f64", par->max_Lpdf_arr, sizeof(double) * NZ_PSOURCES);
    dump(od, "nsources.i32", par->nsources, ngrid * sizeof(int));
  }
  fclose(f);
  size_t nspec = (size_t)n * n * (n / 2 + 1) * 2 * sizeof(float);
  dump(od, "dens_k.f32", shim_captured[0], nspec);
  dump(od, "vpot_k.f32", shim_captured[1], nspec);
  dump(od, "dens_real.f32", par->grid_dens, ngrid * sizeof(float));
  dump(od, "vpot_real.f32", par->grid_vpot, ngrid * sizeof(float));
  dump(od, "rvel.f32", par->grid_rvel, ngrid * sizeof(float));

  lap("dumps");
  get_HI(par);
  lap("get_HI");
  dump(od, "mass.f32", par->grid_dens, ngrid * sizeof(float));
  dump(od, "dz.f32", par->grid_rvel, ngrid * sizeof(float));

  lap("dumps");
  mk_T_maps(par);
  lap("mk_T_maps");
  dump(od, "maps.f32", par->maps_HI, sizeof(float) * par->n_nu * 12 * par->n_side * par->n_side);
  if (par->do_psources) {  /* src/main_gh.c:63-64 */
    mk_psources_maps(par);
    dump(od, "maps_ps.f32", par->maps_PS, sizeof(float) * par->n_nu * 12 * par->n_side * par->n_side);
  }
  return 0;
}
