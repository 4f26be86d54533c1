/*
 * joint_gpu.h -- C ABI of the GB300 JoinT map combination.
 *
 * Drop-in for the stages of damonge/CRIME's JoinT (src/main_jt.c:98-372),
 * which turn the per-channel HEALPix maps of GetHI (and of foreground codes)
 * into mock observations: merge_maps (sum of the components, then he_udgrade
 * to the output resolution), apply_beam (Gaussian beam of a single dish through
 * a spherical harmonic transform, lmax = 3 nside - 1), add_noise (white noise
 * of the system temperature), apply_mask.  The reference has no plugin API;
 * its stages are `void f(ParamsJoinT *, flouble **maps)` functions.
 *
 * Conventions as in gethi_gpu.h: every entry point returns GETHI_OK or a
 * negative GETHI_E* code (the reference calls exit()), with the message in
 * gethi_last_error(); maps are float32 [channel][12 nside^2] in RING order;
 * no torch or CUDA types in the signatures.  One context is used by one host
 * thread at a time; its stages run in order on the context's stream.
 */
#ifndef JOINT_GPU_H
#define JOINT_GPU_H
#include "gethi_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

#define JOINT_RNG_PHILOX 0        /* noise drawn on the device (Philox4x32-10) */
#define JOINT_RNG_MT_VALIDATION 1 /* the reference's MT19937 draws, made on the host */

/* Run parameters: the numeric keys of the reference's param_JoinT .ini
 * (src/io_jt.c:86-186) with the frequency table and the mask already read. */
typedef struct {
  int nside;                 /* nside= : output resolution */
  int n_nu;                  /* channels: rows of fname_nutable= */
  const double *nu0, *nuf;   /* channel edges in MHz (src/io_jt.c:215-241); copied at init */
  unsigned int seed;         /* seed= */
  double dish_diameter;      /* dish_diameter= (m); <= 0: no beam */
  int n_dish;                /* n_dishes= */
  double tsys;               /* t_system= (mK); <= 0: no noise */
  double time_tot;           /* time_total= (h) */
  const int *mask;           /* fname_mask= as 0/1 per pixel [12 nside^2], or NULL (all 1); copied */
  int rng;                   /* JOINT_RNG_* */
  int omp_threads_for_noise; /* JOINT_RNG_MT_VALIDATION: OpenMP threads of the emulated reference run */
  int sht_chunk;             /* channels per spherical-harmonic batch; 0: automatic (every channel, up to
                                256, on the tensor cores; 64 on the CUDA cores); the tensor cores need a
                                multiple of 64 */
  int sht_precision;         /* Legendre sums: 0 = tensor cores (3xTF32) where their tables fit (nside <= 512),
                                else FP32 CUDA cores; 1 = FP32 CUDA cores */
} joint_params;

typedef struct joint_ctx joint_ctx;

/* Allocate a context on `device`: output maps, mask, channel tables.  The
 * spherical-harmonic tables (orthonormal Legendre functions of every ring,
 * FP64-evaluated, stored FP32: 4.8 GB at nside 512) are built at the first
 * beam or transform and kept. */
int joint_gpu_init(const joint_params *p, int device, joint_ctx **out);
void joint_gpu_free(joint_ctx *c);
int joint_gpu_set_stream(joint_ctx *c, void *stream);

/* merge_maps (src/main_jt.c:98-200): add one component, [n_nu][12 nside_in^2]
 * host maps (pageable or pinned), each value first scaled as
 * (float)(value * factor) when factor != 1 (the polarisation leakage of
 * src/main_jt.c:175-183).  All components of a run share nside_in; they are
 * added in call order in FP32, as the reference adds them. */
int joint_gpu_add_maps(joint_ctx *c, const float *maps, long nside_in, double factor);
/* The same from device memory of this context's device, e.g. the maps a GetHI
 * context left there (gethi_gpu_device_maps); no host round trip.  The sum is
 * deferred: the memory must stay valid and unchanged until joint_gpu_merge (or
 * joint_gpu_run) has returned, and, for a repeated run of the same combination,
 * until then too.  Consecutive device components are summed in one pass (at the
 * output resolution straight into the maps). */
int joint_gpu_add_maps_device(joint_ctx *c, const float *dmaps, long nside_in, double factor);
/* he_udgrade of the sum to the output nside (src/healpix_extra.c:318-388,
 * RING in and out, degrading by the FP64 mean of the NESTED children). */
int joint_gpu_merge(joint_ctx *c);
/* apply_beam (src/main_jt.c:202-238): map2alm, a_lm *= exp(-l(l+1) sigma^2/2)
 * with FWHM = 1030610.55 / (nu dish) arcmin, alm2map.  FP32 on the device. */
int joint_gpu_apply_beam(joint_ctx *c);
/* add_noise (src/main_jt.c:263-317): noise = sqrt(-s2 log(1-u2)) cos(2 pi u1),
 * s2 = fsky npix tsys^2 / (3.6e9 dnu time_tot n_dish). */
int joint_gpu_add_noise(joint_ctx *c);
/* apply_mask (src/main_jt.c:240-261) */
int joint_gpu_apply_mask(joint_ctx *c);
/* copy the current maps [n_nu][12 nside^2] to host memory (synchronises) */
int joint_gpu_get_maps(joint_ctx *c, float *maps_out);
/* device pointer of the current maps (valid until the next stage or free) */
int joint_gpu_device_maps(const joint_ctx *c, const float **dmaps);
/* merge, beam (dish_diameter > 0), noise (tsys > 0), mask, copy out: the order
 * of src/main_jt.c:343-372.  maps_out may be NULL (maps stay on the device). */
int joint_gpu_run(joint_ctx *c, float *maps_out);
/* sky fraction of the mask (src/io_jt.c:44-80) */
double joint_gpu_fsky(const joint_ctx *c);

/* he_map2alm / he_alm2map (src/healpix_extra.c:44-130) at the context's nside,
 * lmax = 3 nside - 1, for n_maps host maps.  a_lm are complex float pairs in
 * HEALPix order (index l + m lmax - m(m-1)/2, src/healpix_extra.c:36-42),
 * ((lmax+1)(lmax+2)/2) per map. */
int joint_gpu_map2alm(joint_ctx *c, const float *maps, int n_maps, float *alms);
int joint_gpu_alm2map(joint_ctx *c, const float *alms, int n_maps, float *maps);

/* 1 when the context's Legendre sums run on the tensor cores (known after the first transform) */
int joint_gpu_uses_tensor_cores(const joint_ctx *c);
/* device time of the last joint_gpu_run per stage (ms): merge, beam, noise, mask (with device noise
 * and a mask the two run as one pass, timed as noise) */
int joint_gpu_stage_times(const joint_ctx *c, float *ms4);
/* Per-kernel-class device times of the beam, accumulated while profiling is on
 * (events around each class; off by default): ring analysis (FFT + Bluestein),
 * Legendre analysis (including the E/O pack of the tensor-core path), Legendre
 * synthesis, ring synthesis, E/O pack alone.  Turning profiling on or off resets
 * the sums.  No counterpart in the reference. */
int joint_gpu_profile(joint_ctx *c, int on);
int joint_gpu_kernel_times(joint_ctx *c, double *ms5, long *launches5);

/* ---- host helpers (no GPU) ---- */

/* The param_JoinT .ini (src/io_jt.c:86-186): keys, defaults and checks of the
 * reference, strings included.  Unknown keys warn, as in the reference. */
typedef struct {
  char prefix_cosmo[256], prefix_synchrotron[256], prefix_galactic_freefree[256];
  char prefix_extragalactic_freefree[256], prefix_point_sources[256], prefix_custom[256];
  char prefix_out[256], fname_nutable[256], fname_mask[256];
  int seed_signed;           /* seed= as written; <= 0 means "time(NULL)" in the reference */
  int nside, do_polarization;
  double polarization_leakage, dish_diameter, tsys, time_tot;
  int n_dish;
  int rng, omp_threads_for_noise; /* new keys: rng= philox|mt_validation, omp_threads_for_noise= */
} joint_ini;
int joint_host_read_ini(const char *path, joint_ini *out);
/* the frequency table (src/io_jt.c:215-241): n_nu rows "i nu0 nuf z0 zf";
 * call with nu0 = nuf = NULL to get the count */
int joint_host_read_nutable(const char *path, int *n_nu, double *nu0, double *nuf);
/* one column (0-based) of a HEALPix FITS map (src/healpix_extra.c:166-224):
 * binary table of E or D columns of any repeat; NESTED files are returned in
 * RING order.  Call with out = NULL to get nside. */
int joint_host_read_map(const char *path, int column, long *nside, float *out);
/* write_maps (src/io_jt.c:25-42): <prefix>_%03d.fits, one RING table per channel */
int joint_host_write_maps(const char *prefix, long nside, int n_nu, const float *maps);
/* write_arrays (src/main_jt.c:28-72): <prefix>_instrument.dat */
int joint_host_write_instrument(const char *prefix, const joint_params *p, double fsky);
/* The whole JoinT run of an .ini on `device` (src/main_jt.c:326-389). */
int joint_host_run(const char *ini_path, int device);

#ifdef __cplusplus
}
#endif
#endif
