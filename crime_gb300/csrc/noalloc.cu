// Projection entry point that allocates nothing (gethi_project_noalloc).
//
// For callers that cannot let a library call cudaMalloc: applications that
// own every byte of device memory through their own arena or pool (an
// ensemble driver that sizes HBM for its grids up front), or that may not
// allocate once their run has started.  The caller passes the HI mass and
// dz_rsd grids and the map array as device pointers plus the host-side setup
// arrays of gethi_host_setup; the projection's scratch -- the queue of samples
// whose FP32 key needs the FP64 check, its counters, and the distance tables
// and shell edges the kernels read -- lives in the file-scope device arrays
// below, which every GPU that loads the library keeps until the process exits.
#include <cstring>
#include <mutex>
#include <string>

#include "../../include/gethi_gpu.h"
#include "common.cuh"
#include "fft.h"
#include "host.h"

namespace gethi {
namespace {

constexpr int kMaxNu = 4096;                  // shells accepted by the entry point
constexpr long kQueueEntries = 1L << 20;      // 16 MiB of queue (16 B per entry)
constexpr int kMaxDevices = 64;

// Scratch shared by every call (one set per device).  Calls that overlap on
// the GPU race on it.
static __device__ __align__(256) unsigned char g_queue[kQueueEntries * 16];
static __device__ __align__(256) int g_counters[16];
static __device__ __align__(256) double g_tab_d[4 * kNZ];
static __device__ __align__(256) float g_tab_f[5 * kNZ];  // z, growth d, growth v, line slope, line bound
static __device__ __align__(256) double g_edges_d[kMaxNu + 1];
static __device__ __align__(256) float g_edges_f[kMaxNu + 1];
static __device__ __align__(256) float g_prefac[kMaxNu];

struct Scratch {
  bool ready = false;
  unsigned char *queue = nullptr;
  int *counters = nullptr;
  double *tab_d = nullptr, *edges_d = nullptr;
  float *tab_f = nullptr, *edges_f = nullptr, *prefac = nullptr;
};
Scratch g_scratch[kMaxDevices];
std::mutex g_scratch_mutex;  // first calls from several host threads look the addresses up once

int fail(const std::string &m, int code)
{
  set_error(m);
  return code;
}

// Device addresses of the arrays above, looked up once per device with that
// device current (host code cannot use the symbols themselves as addresses).
int scratch_for(int dev, Scratch **out)
{
  if (dev < 0 || dev >= kMaxDevices) return fail("device index out of range", GETHI_E_ARG);
  std::lock_guard<std::mutex> lock(g_scratch_mutex);
  Scratch &s = g_scratch[dev];
  if (!s.ready) {
    cudaError_t e = cudaSuccess;
    if (e == cudaSuccess) e = cudaGetSymbolAddress((void **)&s.queue, g_queue);
    if (e == cudaSuccess) e = cudaGetSymbolAddress((void **)&s.counters, g_counters);
    if (e == cudaSuccess) e = cudaGetSymbolAddress((void **)&s.tab_d, g_tab_d);
    if (e == cudaSuccess) e = cudaGetSymbolAddress((void **)&s.tab_f, g_tab_f);
    if (e == cudaSuccess) e = cudaGetSymbolAddress((void **)&s.edges_d, g_edges_d);
    if (e == cudaSuccess) e = cudaGetSymbolAddress((void **)&s.edges_f, g_edges_f);
    if (e == cudaSuccess) e = cudaGetSymbolAddress((void **)&s.prefac, g_prefac);
    if (e != cudaSuccess) return fail(std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e), GETHI_E_CUDA);
    s.ready = true;
  }
  *out = &s;
  return GETHI_OK;
}

#define NA_CK(call)                                                                            \
  do {                                                                                         \
    cudaError_t e_ = (call);                                                                   \
    if (e_ != cudaSuccess) return fail(std::string(#call ": ") + cudaGetErrorString(e_), GETHI_E_CUDA); \
  } while (0)

}  // namespace
}  // namespace gethi

using namespace gethi;

extern "C" int gethi_project_noalloc(const gethi_params *p, const gethi_derived *d, const double *tables,
                                     const double *offsets, const double *prefac, const double *nu_edges,
                                     const float *mass, const float *dz, float *maps, void *stream)
{
  if (!p || !d || !tables || !offsets || !prefac || !mass || !dz || !maps)
    return fail("gethi_project_noalloc: null argument", GETHI_E_ARG);
  const int n = p->n_grid, n_nu = d->n_nu;
  if (!fft_supported(n)) return fail("gethi_project_noalloc: n_grid not supported", GETHI_E_ARG);
  if (n_nu < 1 || n_nu > kMaxNu)
    return fail("gethi_project_noalloc: n_nu " + std::to_string(n_nu) + " is above the maximum of " +
                    std::to_string(kMaxNu) + " shells",
                GETHI_E_ARG);
  if (p->n_side < 1 || (double)n_nu * 12.0 * p->n_side * p->n_side >= 4294967295.0)
    return fail("gethi_project_noalloc: n_nu*12*n_side^2 must fit in 32 bits", GETHI_E_ARG);
  if (!d->regular_nu && !nu_edges) return fail("gethi_project_noalloc: nu_edges needed for a frequency file", GETHI_E_ARG);
  int dev = 0;
  NA_CK(cudaGetDevice(&dev));
  Scratch *sc = nullptr;
  int rc = scratch_for(dev, &sc);
  if (rc) return rc;
  cudaStream_t st = (cudaStream_t)stream;

  // host setup values into the device arrays: stream-ordered copies from
  // pageable stack buffers (each cudaMemcpyAsync returns once its source has
  // been staged, so the buffers can be refilled and the caller's arrays may
  // change as soon as the call returns), up to 8 KB per copy, no allocation
  constexpr int kChunk = 1024;
  double db[kChunk];
  float fb[kChunk];
  // FP64 copy of src[0..cnt); src may be db itself (one chunk)
  auto put_d = [&](double *dst, const double *src, int cnt) -> cudaError_t {
    for (int base = 0; base < cnt; base += kChunk) {
      const int k = cnt - base < kChunk ? cnt - base : kChunk;
      if (src != db) std::memcpy(db, src + base, sizeof(double) * k);
      cudaError_t e = cudaMemcpyAsync(dst + base, db, sizeof(double) * k, cudaMemcpyHostToDevice, st);
      if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
  };
  // FP32 copy of src[0..cnt)
  auto put_f = [&](float *dst, const double *src, int cnt) -> cudaError_t {
    for (int base = 0; base < cnt; base += kChunk) {
      const int k = cnt - base < kChunk ? cnt - base : kChunk;
      for (int i = 0; i < k; i++) fb[i] = (float)src[base + i];
      cudaError_t e = cudaMemcpyAsync(dst + base, fb, sizeof(float) * k, cudaMemcpyHostToDevice, st);
      if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
  };
  NA_CK(put_d(sc->tab_d, tables + 2 * NZ, NZ));               // z(r)
  NA_CK(put_d(sc->tab_d + NZ, tables + 3 * NZ, NZ));          // r
  NA_CK(put_d(sc->tab_d + 2 * NZ, tables + 4 * NZ, 2 * NZ));  // growth of density and velocity
  NA_CK(put_f(sc->tab_f, tables + 2 * NZ, NZ));
  NA_CK(put_f(sc->tab_f + NZ, tables + 4 * NZ, NZ));
  NA_CK(put_f(sc->tab_f + 2 * NZ, tables + 5 * NZ, NZ));
  {  // the projection's line table: slopes, then deviation bounds
    double ox[NSUB], oy[NSUB], oz[NSUB];
    for (int i = 0; i < NSUB; i++) {
      ox[i] = offsets[3 * i];
      oy[i] = offsets[3 * i + 1];
      oz[i] = offsets[3 * i + 2];
    }
    const double dxl = d->l_box / n, rho = subsample_radius(ox, oy, oz, dxl);
    for (int half = 0; half < 2; half++)
      for (int base = 0; base < NZ; base += kChunk) {
        const int k = NZ - base < kChunk ? NZ - base : kChunk;
        for (int i = 0; i < k; i++) {
          const float2 v = shell_line_entry(tables + 2 * NZ, d->glob_idr, dxl, rho, base + i);
          fb[i] = half ? v.y : v.x;
        }
        NA_CK(cudaMemcpyAsync(sc->tab_f + (3 + half) * NZ + base, fb, sizeof(float) * k, cudaMemcpyHostToDevice, st));
      }
  }
  for (int base = 0; base <= n_nu; base += kChunk) {  // shell edges, FP64 and FP32
    const int k = n_nu + 1 - base < kChunk ? n_nu + 1 - base : kChunk;
    for (int i = 0; i < k; i++)
      db[i] = d->regular_nu ? p->nu_min + (p->nu_max - p->nu_min) * (double)(base + i) / n_nu : nu_edges[base + i];
    NA_CK(put_f(sc->edges_f + base, db, k));
    NA_CK(put_d(sc->edges_d + base, db, k));
  }
  NA_CK(put_f(sc->prefac, prefac, n_nu));

  DevCfg g;
  std::memset(&g, 0, sizeof(g));
  g.n = n;
  g.m = n / 2;
  g.l_box = d->l_box;
  g.dx = d->l_box / n;  // src/pixelize.c:175
  g.pos_obs = d->pos_obs;
  g.dxf = (float)g.dx;
  g.pos_obsf = (float)g.pos_obs;
  g.z_r2z = sc->tab_d;
  g.r_r2z = sc->tab_d + NZ;
  g.gd = sc->tab_d + 2 * NZ;
  g.gv = sc->tab_d + 3 * NZ;
  g.z_r2z_f = sc->tab_f;
  g.gd_f = sc->tab_f + NZ;
  g.gv_f = sc->tab_f + 2 * NZ;
  g.z_lin_g = sc->tab_f + 3 * NZ;
  g.z_lin_e = sc->tab_f + 4 * NZ;
  g.glob_idr = d->glob_idr;
  g.glob_idr_f = (float)d->glob_idr;
  g.r_tab_max = tables[3 * NZ + NZ - 1];
  g.r_tab_max_f = (float)g.r_tab_max;
  g.n_nu = n_nu;
  g.regular_nu = d->regular_nu;
  g.nside = p->n_side;
  g.npix = 12 * p->n_side * p->n_side;
  g.nu_min = d->regular_nu ? p->nu_min : nu_edges[0];
  g.nu_max = d->regular_nu ? p->nu_max : nu_edges[n_nu];
  g.inv_dnu = n_nu / (g.nu_max - g.nu_min);  // src/pixelize.c:177
  g.nu_edges = sc->edges_d;
  g.nu_edges_f = sc->edges_f;
  g.prefac = sc->prefac;
  for (int i = 0; i < NSUB; i++) {
    g.xs[i] = offsets[3 * i];
    g.ys[i] = offsets[3 * i + 1];
    g.zs[i] = offsets[3 * i + 2];
  }

  // the counters (queue length) start at zero on every call; the maps are summed into
  NA_CK(cudaMemsetAsync(sc->counters, 0, sizeof(int) * 16, st));
  NA_CK(cudaMemsetAsync(maps, 0, sizeof(float) * g.npix * n_nu, st));
  NA_CK(project(g, nullptr, mass, dz, 0, maps, sc->counters, sc->queue, kQueueEntries, st));
  NA_CK(fixup(g, sc->queue, sc->counters, kQueueEntries, maps, st));
  NA_CK(scale_maps(g, maps, st));
  return GETHI_OK;
}
