// Launchers of the GetHI FFT passes and realisation-stage kernels.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <vector>

#include "common.cuh"

namespace gethi {

enum KernelClass {
  KC_ZPASS = 0, KC_YPASS, KC_XPASS, KC_XPASS_VEL, KC_NYQ, KC_SIGMA, KC_FDVEL, KC_GETHI, KC_PROJECT, KC_SCALE,
  KC_ZPASS_RAW, KC_FIXUP, KC_PSOURCES
};

enum FieldKind { FIELD_DENS = 0, FIELD_VPOT = 1, FIELD_VX = 2, FIELD_VY = 3, FIELD_VZ = 4 };

struct ColGeom {
  float2 *base;
  long cpp, pstride, cstride, estride, ncols;
};

bool fft_supported(int n);
long row_pass_blocks(int n);
struct RowIn {
  float2 *main[3];
  const float2 *nyq[3];
};
// mode 0: out1 (or in place) = FFT(g.base); 1: draw delta_k (Philox or src) and
// write FFT(delta) to g.base, FFT(phi) to out1 (nout >= 2), FFT(i kz phi) to
// out2 (nout == 3); 4: out = FFT(i kx in); 5: out = FFT(i ky in)
cudaError_t col_pass(const DevCfg &c, const ColGeom &g, int nyq, int mode, int nout, const float2 *src,
                     const float2 *tw, float2 *out1, float2 *out2, cudaStream_t st);
// epi 0: real row in place + sigma partials; 3: real row in place; 2: v_r from three rows
cudaError_t row_pass(const DevCfg &c, const RowIn &in, const float2 *twN, const float2 *twM, float scale, int epi,
                     float *vr, double2 *partials, cudaStream_t st);
cudaError_t finish_sigma(const double2 *partials, int np, double ncells, double *stats, cudaStream_t st);
cudaError_t gen_modes(const DevCfg &c, float2 *out, int kind, cudaStream_t st);
cudaError_t pack_pk(const DevCfg &c, float2 *main, float2 *nyq, float inv_vol, cudaStream_t st);
cudaError_t log_xi(const DevCfg &c, const float *xi, float2 *main, float2 *nyq, cudaStream_t st);

// tcfft.cu: split-precision tensor-core column passes (n = 1024, main block)
bool tc_col_supported(const DevCfg &c, const ColGeom &g, int nyq);
cudaError_t tc_col_pass(const DevCfg &c, const ColGeom &g, int mode, int nout, const float2 *src, float2 *out1,
                        float2 *out2, cudaStream_t st);
bool tc_tables(int n, std::vector<uint16_t> &bmat, std::vector<float2> &tw);
size_t tc_table_bytes();
// a bounded wait on an mbarrier nothing arrives on: sets *err after limit_ns
cudaError_t wait_selftest(int *err, uint64_t limit_ns, cudaStream_t st);

// point sources (stages.cu)
constexpr int kPsNZ = 256;                  // src/common_gh.h:35 (NZ_PSOURCES)
constexpr uint32_t kPsKey = 0x50535243u;    // second Philox key word of the point-source draws
struct PsConst {
  const float *nz;    // n(z) at z = i * glob_dz, kPsNZ entries
  const float *icdf;  // log10 L at probabilities q / nicdf, nicdf + 1 entries
  float inv_dz, z_max, cell_vol;
  int nicdf;
};
// sources captured for inspection (count == nullptr: none): cell index, (ux, uy, uz, L0), dz_rsd, pixel
struct PsCatalogue {
  unsigned long long *count;
  long cap;
  long *cell;
  float4 *u;
  float *dz;
  int *pix;
};
cudaError_t psources(const DevCfg &c, const PsConst &p, const double *stats, const float *dens, const float *vr,
                     float *acc, float *maps_ps, const float *chan, unsigned long long *total, const PsCatalogue &cat,
                     cudaStream_t st);

// stages.cu
cudaError_t radial_velocity_fd(const DevCfg &c, const float *vpot, float *rvel, cudaStream_t st);
cudaError_t get_hi(const DevCfg &c, const double *stats, float *dens, float *rvel, cudaStream_t st);
// counters: [0] uncertain samples, [1] sample_keys fallbacks, [2..3] 64-bit fallback-queue length
cudaError_t project(const DevCfg &c, const double *stats, const float *a, const float *b, int fused, float *maps,
                    int *counters, void *fq, long fq_cap, cudaStream_t st);
cudaError_t fixup(const DevCfg &c, const void *fq, const int *counters, long fq_cap, float *maps, cudaStream_t st);
long fallback_queue_capacity(int n);
// largest distance of a sub-sample from its cell centre, in cells
double subsample_radius(const double *xs, const double *ys, const double *zs, double dx);
// entry i of DevCfg::z_lin_g / z_lin_e for the FP64 redshift table z_r2z[kNZ],
// cell size dx and sub-sample radius rho (cells)
float2 shell_line_entry(const double *z_r2z, double glob_idr, double dx, double rho, int i);
size_t fallback_entry_bytes();
cudaError_t scale_maps(const DevCfg &c, float *maps, cudaStream_t st);
cudaError_t sample_keys(const DevCfg &c, const float *dz, uint32_t *keys, int exact, int *counters,
                        cudaStream_t st);

}  // namespace gethi
