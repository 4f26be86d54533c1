/*
 * GetHI_gpu: command-line drop-in for the reference's `./GetHI param.ini`
 * (src/main_gh.c:24-80).  Reads the same .ini, runs the realisation on the
 * GPU and writes <prefix_out>_%03d.fits, one RING map per frequency shell.
 */
#include <stdio.h>
#include <stdlib.h>

#include "gethi_gpu.h"

int main(int argc, char **argv)
{
  if (argc != 2) {
    fprintf(stderr, "Usage: %s file_name\n", argv[0]);
    return 0;
  }
  gethi_params p;
  if (gethi_read_params(argv[1], &p) != GETHI_OK) {
    fprintf(stderr, "CRIME: %s\n", gethi_last_error());
    return 1;
  }
  gethi_ctx *ctx = NULL;
  if (gethi_gpu_init(&p, 0, &ctx) != GETHI_OK) {
    fprintf(stderr, "CRIME: %s\n", gethi_last_error());
    return 1;
  }
  gethi_derived d;
  gethi_gpu_get_derived(ctx, &d);
  printf("Run parameters:\n  %.3lf < nu/MHz < %.3lf\n  %.3lf < z < %.3lf\n  %.3lf < r/(Mpc/h) < %.3lf\n",
         p.nu_min, p.nu_max, d.z_min, d.z_max, d.r_min, d.r_max);
  printf("  L_box = %.3lf Mpc/h, N_grid = %d, n_nu = %d, n_side = %ld\n", d.l_box, p.n_grid, d.n_nu, p.n_side);
  size_t npix = 12 * (size_t)p.n_side * p.n_side;
  float *maps = (float *)malloc(sizeof(float) * npix * d.n_nu);
  int rc = maps ? gethi_gpu_run(ctx, maps) : GETHI_E_NOMEM;
  if (rc == GETHI_OK) {
    float t[8];
    int k = gethi_gpu_stage_times(ctx, t, 8);
    for (int i = 0; i < k; i++) printf(">    Stage %d: %.1f ms\n", i, t[i]);
    printf("*** Writing files %s_###.fits\n", p.prefix_out);
    rc = gethi_gpu_write_maps(ctx, maps);
  }
  if (rc != GETHI_OK) fprintf(stderr, "CRIME: %s\n", gethi_last_error());
  free(maps);
  gethi_gpu_free(ctx);
  return rc == GETHI_OK ? 0 : 1;
}
