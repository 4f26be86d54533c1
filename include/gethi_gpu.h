/*
 * gethi_gpu.h -- C ABI of the GB300 GetHI realisation path.
 *
 * Drop-in for the stage functions of damonge/CRIME's GetHI (the reference has
 * no plugin API; its path is `void f(ParamGetHI*)` stages driven by
 * src/main_gh.c).  Every entry point returns 0 on success and a negative
 * GETHI_E* code on failure (the reference calls exit(); here the caller
 * decides), with a message available from gethi_last_error().  No torch or
 * CUDA types appear in the signatures; the only CUDA object that can be passed
 * in is a stream, as an opaque pointer.
 *
 * Threading: one context is used by one host thread at a time; stages of a
 * context run in order on the context's stream.
 */
#ifndef GETHI_GPU_H
#define GETHI_GPU_H
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GETHI_OK 0
#define GETHI_E_ARG (-1)     /* invalid argument or parameter combination */
#define GETHI_E_IO (-2)      /* file missing or unreadable / unwritable */
#define GETHI_E_COSMO (-3)   /* cosmology rejected (src/cosmo_mad.c:455-473, "OMG!" checks) */
#define GETHI_E_CUDA (-4)    /* CUDA runtime error */
#define GETHI_E_NOMEM (-5)   /* device or host allocation failed */
#define GETHI_E_STATE (-6)   /* stage called out of order */
#define GETHI_E_DEVICE (-7)  /* a device-side check failed (bounded wait expired, bad index) */

#define GETHI_NZ 5001        /* table length, src/common_gh.h:34 */

/* Run parameters: every key of the reference's param_GetHI .ini
 * (src/io_gh.c:211-249, defaults src/io_gh.c:133-186) plus new keys. */
typedef struct {
  char prefix_out[256];           /* prefix_out= */
  char pk_filename[256];          /* pk_filename= ; "EH" selects the built-in no-wiggle fit */
  char frequencies_filename[256]; /* frequencies_filename= ; "" or "default" -> regular table */
  double omega_M, omega_L, omega_B, h, w, ns, sigma_8;
  double r_smooth;                /* r_smooth= ; <= 0 disables the k-space smoothing */
  double nu_min, nu_max;          /* nu_min= nu_max= (regular table) */
  int n_nu;                       /* n_nu= */
  int n_grid;                     /* n_grid= */
  long n_side;                    /* n_side= */
  unsigned int seed;              /* seed= */
  int do_psources;                /* do_psources= (point sources: must be 0) */
  /* ---- new keys (the reference parser only warns on unknown keys) ---- */
  double l_box;                   /* l_box= ; > 0 overrides the derived 2 r_max (1+2/N) */
  int bias_model;                 /* bias_model= fit|const  (0|1) */
  double b_HI;                    /* b_HI= (bias_model=const) */
  int do_rsd;                     /* do_rsd= 0|1 */
  int velocity_mode;              /* velocity_mode= fd|spectral (0|1) */
  int gaussianise;                /* gaussianise= 0|1 : use P_G with xi_G = ln(1+xi) */
  int fft_precision;              /* fft_precision= fp32|tc_split (0|1) */
  int rng;                        /* rng= philox|mt_validation (0|1) */
  int omp_threads_for_modes;      /* omp_threads_for_modes= (mt_validation thread emulation) */
  int write_maps;                 /* write_maps= 0|1 (FITS output in gethi_gpu_run) */
} gethi_params;

/* Derived quantities, the derived members of ParamGetHI (src/common_gh.h:67-116). */
typedef struct {
  double fgrowth_0, hubble_0, z_min, z_max, r_min, r_max, l_box, pos_obs;
  double r2_smooth, glob_idr, logkmin, logkmax, idlogk, pk_norm, sigma8_in;
  double sigma2_gauss, mean_gauss; /* set by gethi_gpu_make_fields */
  int do_smoothing, numk, n_nu, regular_nu;
  double filled_fraction;          /* fraction of shell volume inside the box */
} gethi_derived;

/* ---- host-side parameter handling ---- */
/* Reference defaults, src/io_gh.c:133-186 (param_gethi_new). */
int gethi_params_default(gethi_params *p);
/* .ini parser, src/io_gh.c:188-253 (read_run_params, file part): `key= value`
 * lines, '#' and blank lines skipped, unknown keys warned about on stderr. */
int gethi_read_params(const char *ini_path, gethi_params *p);

/* Host-only FP64 setup (no GPU needed): the derived quantities of
 * read_run_params/cosmo_set (src/io_gh.c:255-266, src/cosmo.c:341-413).
 * Optional outputs: tables[6*GETHI_NZ] = z_z2r, r_z2r, z_r2z, r_r2z, growth_d,
 * growth_v; logk[numk], pk[numk] (normalised); offsets[30] = the sub-sample
 * offsets x0,y0,z0,x1,... (src/pixelize.c:159-163); prefac[n_nu]. */
int gethi_host_setup(const gethi_params *p, gethi_derived *d, double *tables, double *logk, double *pk,
                     double *offsets, double *prefac);
/* Host draw of the reference's modes (src/fourier.c:234-305) as `nthreads`
 * OpenMP threads would make them; out: [kz][ky][N/2+1] complex float. */
int gethi_host_modes_mt(const gethi_params *p, int nthreads, float *out);

/* ---- context lifecycle ---- */
typedef struct gethi_ctx gethi_ctx;
/* Replaces the tail of read_run_params (src/io_gh.c:255-266: cosmo_set,
 * init_fftw, allocate_maps) and init_fftw (src/fourier.c:101-199): FP64 host
 * setup, device tables, device buffers.  `device` selects the CUDA device. */
int gethi_gpu_init(const gethi_params *p, int device, gethi_ctx **out);
/* Replaces param_gethi_free + end_fftw (src/io_gh.c:298-324, src/fourier.c:201-232). */
void gethi_gpu_free(gethi_ctx *ctx);
/* Run the context's work on this stream (cudaStream_t passed as void*; NULL = own stream). */
int gethi_gpu_set_stream(gethi_ctx *ctx, void *stream);
int gethi_gpu_get_derived(const gethi_ctx *ctx, gethi_derived *out);
const char *gethi_last_error(void);

/* ---- stages (same order and meaning as src/main_gh.c:34-74) ---- */
/* create_d_and_vr_fields (src/fourier.c:375-438): Gaussian modes, c2r FFTs,
 * normalisation, radial velocity, sigma^2.  modes_k == NULL: modes are drawn
 * on the device (rng=philox) or by the host MT19937 emulation of the
 * reference (rng=mt_validation).  modes_k != NULL: a host half spectrum in the
 * reference layout [kz][ky][N/2+1] complex float (interleaved), used as delta_k. */
int gethi_gpu_make_fields(gethi_ctx *ctx, const float *modes_k);
/* get_HI (src/grid_tools.c:103-153): lognormal HI mass and dz_rsd, in place. */
int gethi_gpu_get_hi(gethi_ctx *ctx);
/* mk_T_maps (src/pixelize.c:150-286): maps[n_nu][12 n_side^2] in mK.
 * maps_out may be NULL (maps stay on the device). */
int gethi_gpu_make_maps(gethi_ctx *ctx, float *maps_out);
/* Device pointers of the maps the last make_maps / run left on the context's
 * device ([n_nu][12 n_side^2] float32; maps_ps NULL without point sources),
 * valid until the next realisation or free.  No counterpart in the reference,
 * whose JoinT reads the maps back from FITS files (src/main_jt.c:98-200); this
 * hands them to joint_gpu_add_maps_device without a host round trip. */
int gethi_gpu_device_maps(const gethi_ctx *ctx, const float **maps, const float **maps_ps);
/* write_maps (src/io_gh.c:109-131): <prefix>_%03d.fits, RING, column T [mK]. */
int gethi_gpu_write_maps(const gethi_ctx *ctx, const float *maps);
/* All stages; get_HI is fused into the projection (no separate HBM pass). */
int gethi_gpu_run(gethi_ctx *ctx, float *maps_out);
/* Pipelined form of gethi_gpu_run (no counterpart in the reference): enqueues
 * one realisation and the copy of its maps to maps_out (page-locked host or
 * device memory; NULL: no copy) and returns without waiting.  Consecutive calls
 * alternate between two device map buffers, and the copies run on a second
 * stream, so a realisation computes while the previous one's maps travel.
 * maps_out must stay valid until gethi_gpu_wait, and the host may read it
 * only after that; it may be passed again as the destination of the call after
 * next (the GPU orders the two copies).  The point-source maps stay on the
 * device. */
int gethi_gpu_run_async(gethi_ctx *ctx, float *maps_out);
/* Waits for every realisation and copy enqueued by gethi_gpu_run_async. */
int gethi_gpu_wait(gethi_ctx *ctx);
/* Seed of the next realisation (src/io_gh.c:246, seed=). */
int gethi_gpu_set_seed(gethi_ctx *ctx, unsigned int seed);
/* Copy the realisation's host inputs (P(k), distance/growth tables, shell
 * edges, channel factors) to the device again from pinned memory; returns the
 * byte count (>= 0) or an error code. */
long gethi_gpu_upload_inputs(gethi_ctx *ctx);

/* ---- point sources (do_psources=1) ----
 * get_point_sources (src/grid_tools.c:24-101) and mk_psources_maps
 * (src/pixelize.c:58-148) run inside gethi_gpu_make_fields, on the Gaussian
 * density: per cell a Poisson number of sources with mean n(z) dx^3
 * exp(D (delta - D sigma^2/2)), each at a uniform position in its cell with a
 * luminosity from the reference's luminosity function (src/psources.c), its
 * temperature added to every channel of its pixel.  Draws are counter-based
 * (Philox4x32-10), so they follow the reference's distributions, not its GSL
 * stream.  maps_out: [n_nu][12 n_side^2] in mK (may be NULL); nsources: the
 * number of sources of the last realisation (may be NULL). */
int gethi_gpu_psources_maps(gethi_ctx *ctx, float *maps_out, long *nsources);
/* The sources of the current fields (after gethi_gpu_make_fields or
 * gethi_gpu_run, before gethi_gpu_get_hi), drawn again with the same counters:
 * up to cap entries of cell index ix + n (iy + n iz), (ux, uy, uz, L0) (position
 * dx (i + u) - x_obs, luminosity in 1e22 W/Hz), the cell's dz_rsd and the RING
 * pixel; *count = the number of sources (may exceed cap). */
int gethi_gpu_psources_catalogue(gethi_ctx *ctx, long cap, long *cell, float *u_l, float *dz, int *pix, long *count);
/* Host side of the point sources (src/psources.c:98-124): n(z) and rejection
 * bounds on 256 bins of z_max/256, and the inverse CDF of log10 L that replaces
 * the rejection loop (4097 entries); any pointer may be NULL. */
int gethi_host_psources(const gethi_params *p, double *nz_arr, double *maxpdf, double *glob_dz, double *logl_icdf);

/* ---- ensembles ----
 * The reference runs one realisation per process (src/main_gh.c:24-80); an
 * ensemble is many runs of GetHI with different seed= values.  This runs a
 * batch of Philox realisations in one call: job i uses context ctx[job_ctx[i]]
 * (one configuration: grid, box, shells) with seed seeds[i] and, maps_out !=
 * NULL and maps_out[i] != NULL, copies its maps [n_nu][12 n_side^2] (mK) to
 * maps_out[i] (device memory, page-locked host memory, or pageable host memory,
 * which is page-locked for the duration of the call).  Jobs of one context run
 * in order on its stream; different contexts run concurrently.  use_graph != 0:
 * the whole batch is captured into one CUDA graph and launched once.
 * stats (may be NULL) receives {capture + instantiate ms, device ms of the
 * batch, graph nodes, kernel launches}.  Contexts must be on one device with
 * rng=philox. */
int gethi_gpu_run_batch(gethi_ctx *const *ctx, int nctx, const int *job_ctx, const unsigned int *seeds, int njobs,
                        float *const *maps_out, int use_graph, double *stats);
/* Launch-shape autotuner (no counterpart in the reference): times each
 * candidate projection tile depth (8 x 8 x {16, 8, 4} cells) and, for n_grid
 * 128/256/384, the half-width column tile of the FP32 passes on this context's
 * own realisations, and keeps the fastest for the context's later work.
 * choice (may be NULL) = {tile depth / 4, column variant}; ms = best time per
 * realisation. */
int gethi_gpu_autotune(gethi_ctx *ctx, int *choice, float *ms);
/* Launch shapes by hand (no counterpart in the reference; gethi_gpu_autotune
 * picks them by timing): proj_zsteps = projection tile depth / 4 cells (1..4,
 * 0 = built-in), col_variant = FP32 column passes: 0 = built-in (Y passes of
 * 512- and 1024-point columns from TMA-staged tiles), 1 = half-width tiles
 * (128/256/384 points), 2 = tiles loaded through registers.  All choices give
 * the same fields to FP32 rounding. */
int gethi_gpu_set_launch(gethi_ctx *ctx, int proj_zsteps, int col_variant);

/* ---- validation / inspection (compact [z][y][x] float grids, N^3) ---- */
int gethi_gpu_download_grids(const gethi_ctx *ctx, float *dens, float *rvel);
int gethi_gpu_upload_grids(gethi_ctx *ctx, const float *dens, const float *rvel, int stage);
/* per-sample (bin*npix+pixel) keys of the current mass/dz grids; 0xFFFFFFFF = outside the shells */
int gethi_gpu_sample_keys(gethi_ctx *ctx, uint32_t *keys, int exact_fp64);
/* on-device Philox modes of the current config, reference layout */
int gethi_gpu_download_modes(gethi_ctx *ctx, float *modes_k);
/* per-stage device times of the last run, in ms (up to n entries) */
int gethi_gpu_stage_times(const gethi_ctx *ctx, float *ms, int n);

/* ---- projection without device allocation ----
 * No counterpart in the reference.  mk_T_maps (src/pixelize.c:150-286) for
 * callers that cannot let a library call cudaMalloc: they own all device
 * memory through their own allocator or arena, or may not allocate once a run
 * has started.  mass and dz are the caller's device grids (N^3 floats,
 * [z][y][x], the HI mass and dz_rsd of get_HI); maps is the caller's device
 * output [n_nu][12 n_side^2] (overwritten).  d, tables, offsets and prefac are
 * the outputs of gethi_host_setup for the same parameters; nu_edges holds the
 * n_nu+1 shell edges of a frequency file (NULL for a regular table).  stream is
 * a cudaStream_t (NULL: default stream); the work is enqueued on it.  The host
 * arrays are copied through the call's own stack buffers before it returns,
 * so the caller may change or free them once it has returned.
 * The call allocates nothing: its scratch (a 16 MiB queue of samples whose
 * FP32 key needs the FP64 check, counters, distance tables and shell edges,
 * about 16.4 MiB in all) is a set of file-scope device arrays that every GPU
 * loading the library holds until the process exits.  Limits: n_nu <= 4096,
 * n_grid one of the supported sizes; larger requests return GETHI_E_ARG.  The
 * first call on a device looks the arrays' addresses up (cudaGetSymbolAddress
 * with that device current), so make that first call before any stream
 * capture.  All calls share the arrays; the counters are cleared at the start
 * of every call, and calls that overlap on the GPU (other streams, other host
 * threads) race on them. */
int gethi_project_noalloc(const gethi_params *p, const gethi_derived *d, const double *tables,
                          const double *offsets, const double *prefac, const double *nu_edges,
                          const float *mass, const float *dz, float *maps, void *stream);

/* ---- measurement ---- */
/* kernel classes timed when profiling is on (events around each launch) */
#define GETHI_KC_ZPASS 0      /* Z pass drawing the modes on the fly (main block) */
#define GETHI_KC_YPASS 1      /* Y pass (main block) */
#define GETHI_KC_XPASS 2      /* X pass, real field written in place (+ sigma partial sums) */
#define GETHI_KC_XPASS_VEL 3  /* X pass accumulating the radial velocity */
#define GETHI_KC_NYQ 4        /* Z and Y passes of the kx = N/2 plane */
#define GETHI_KC_SIGMA 5
#define GETHI_KC_FDVEL 6
#define GETHI_KC_GETHI 7
#define GETHI_KC_PROJECT 8
#define GETHI_KC_SCALE 9
#define GETHI_KC_ZPASS_RAW 10 /* Z pass of a velocity field from the stored modes */
#define GETHI_KC_FIXUP 11     /* FP64 keys of the samples the FP32 path left uncertain */
#define GETHI_KC_PSOURCES 12  /* point sources: Poisson draws, positions, luminosities, maps */
#define GETHI_NKCLASS 13
int gethi_gpu_profile(gethi_ctx *ctx, int on);
/* accumulated ms and launch counts per class since profiling was switched on,
 * and the total number of kernels this context has launched */
int gethi_gpu_kernel_times(const gethi_ctx *ctx, double *ms, long *count, long *launches);
/* samples of the last projection that needed the FP64 key */
int gethi_gpu_fallback_count(const gethi_ctx *ctx, long *n);
/* Failure detection (the reference has none on this path: every error calls
 * exit(), src/common_gh.c:104-120).  Every device-side wait of this library
 * (mbarrier waits of the tensor-core passes) is bounded by time; on expiry the
 * kernel raises the context's error flag and returns, and the next synchronizing
 * call reports GETHI_E_CUDA once and clears it.  This call runs that path on
 * purpose: one warp waits limit_us (1 us .. 10 s) on an mbarrier nothing arrives
 * on, with no copy or MMA in flight.  Returns GETHI_E_CUDA when the wait
 * expired (always, unless the GPU misbehaves); the context stays usable. */
int gethi_gpu_wait_selftest(gethi_ctx *ctx, long limit_us);

#ifdef __cplusplus
}
#endif
#endif
