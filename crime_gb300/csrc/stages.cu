// Real-space stages of the GetHI realisation on GB300: radial velocity by
// finite differences, the lognormal HI transform and the projection of cells
// onto (HEALPix pixel, frequency shell) maps.
#include <cstdio>

#include "common.cuh"
#include "fft.h"

namespace gethi {

// ---------------------------------------------------------------------------
// radial velocity from the potential, src/fourier.c:307-373 (periodic wrap in
// x, y and z; one GPU holds the whole grid, so no halo exchange)
// ---------------------------------------------------------------------------
__global__ void fd_vel_kernel(DevCfg c, const float *__restrict__ phi, float *__restrict__ vr)
{
  const int n = c.n;
  const long total = (long)n * n * n;
  const float hidx = 0.5f / c.dxf;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < total; i += (long)gridDim.x * blockDim.x) {
    int ix = (int)(i % n);
    long rest = i / n;
    int iy = (int)(rest % n), iz = (int)(rest / n);
    int xh = ix == n - 1 ? 0 : ix + 1, xl = ix == 0 ? n - 1 : ix - 1;
    int yh = iy == n - 1 ? 0 : iy + 1, yl = iy == 0 ? n - 1 : iy - 1;
    int zh = iz == n - 1 ? 0 : iz + 1, zl = iz == 0 ? n - 1 : iz - 1;
    long rowb = ((long)iz * n + iy) * n;
    float dvx = __ldg(&phi[rowb + xh]) - __ldg(&phi[rowb + xl]);
    float dvy = __ldg(&phi[((long)iz * n + yh) * n + ix]) - __ldg(&phi[((long)iz * n + yl) * n + ix]);
    float dvz = __ldg(&phi[((long)zh * n + iy) * n + ix]) - __ldg(&phi[((long)zl * n + iy) * n + ix]);
    float x = c.dxf * (ix + 0.5f) - c.pos_obsf, y = c.dxf * (iy + 0.5f) - c.pos_obsf, z = c.dxf * (iz + 0.5f) - c.pos_obsf;
    float irr = rsqrtf(x * x + y * y + z * z);
    vr[i] = hidx * (dvx * x + dvy * y + dvz * z) * irr;
  }
}

// ---------------------------------------------------------------------------
// lognormal HI mass and RSD displacement, src/grid_tools.c:103-153, FP32
// ---------------------------------------------------------------------------
struct CellHI {
  float mass, dz;
};

__device__ __forceinline__ CellHI cell_hi(const DevCfg &c, float sigma2, int ix, int iy, int iz, float delta, float vr)
{
  float x = c.dxf * (ix + 0.5f) - c.pos_obsf, y = c.dxf * (iy + 0.5f) - c.pos_obsf, z = c.dxf * (iz + 0.5f) - c.pos_obsf;
  float r = sqrtf(x * x + y * y + z * z);
  float tr = fminf(r * c.glob_idr_f, (float)(kNZ - 2));
  int ir = (int)tr;
  float fr = tr - ir;
  float z0 = __ldg(&c.z_r2z_f[ir]), z1 = __ldg(&c.z_r2z_f[ir + 1]);
  float g0 = __ldg(&c.gd_f[ir]), g1 = __ldg(&c.gd_f[ir + 1]);
  float redshift = z0 + (z1 - z0) * fr;
  float lz = log2f(1.f + redshift);
  float bias = c.bias_const ? c.b_HI : 0.904f + 0.135f * exp2f(1.696f * lz);  // src/user_defined.c:32-35
  float gfd = (g0 + (g1 - g0) * fr) * bias;
  float dens_ln = expf(gfd * (delta - 0.5f * gfd * sigma2));
  CellHI o;
  o.mass = c.mass_prefac * (0.008f * exp2f(0.6f * lz)) * dens_ln;  // src/user_defined.c:27-30
  if (c.do_rsd) {
    float v0 = __ldg(&c.gv_f[ir]), v1 = __ldg(&c.gv_f[ir + 1]);
    o.dz = vr * (v0 + (v1 - v0) * fr);
  } else
    o.dz = 0.f;
  return o;
}

__global__ void get_hi_kernel(DevCfg c, const double *__restrict__ stats, float *__restrict__ dens,
                              float *__restrict__ rvel)
{
  const int n = c.n;
  const long total = (long)n * n * n;
  const float sigma2 = (float)stats[1];
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < total; i += (long)gridDim.x * blockDim.x) {
    int ix = (int)(i % n);
    long rest = i / n;
    CellHI h = cell_hi(c, sigma2, ix, (int)(rest % n), (int)(rest / n), dens[i], rvel[i]);
    dens[i] = h.mass;
    rvel[i] = h.dz;
  }
}

// ---------------------------------------------------------------------------
// exact (FP64) sample key: the reference's operation sequence
// (src/pixelize.c:346-379, src/cosmo.c:52-62) with every rounding explicit, so
// no multiply-add is contracted; vec2pix_ring is the RING scheme of Gorski et
// al. (2005) in the same form as the oracle.
// ---------------------------------------------------------------------------
#define INV_HALFPI_D 0.63661977236758134308

__device__ __forceinline__ double z_of_r_exact(const DevCfg &c, double r)
{
  if (r <= 0) return 0;
  if (r >= c.r_tab_max) return __ldg(&c.z_r2z[kNZ - 1]);
  int ir = (int)__dmul_rn(r, c.glob_idr);
  double z0 = __ldg(&c.z_r2z[ir]), z1 = __ldg(&c.z_r2z[ir + 1]), r0 = __ldg(&c.r_r2z[ir]);
  return __dadd_rn(z0, __dmul_rn(__dmul_rn(__dsub_rn(z1, z0), __dsub_rn(r, r0)), c.glob_idr));
}

__device__ __forceinline__ int bin_exact(const DevCfg &c, double nu)
{
  if (c.regular_nu) return (int)__dmul_rn(c.inv_dnu, __dsub_rn(nu, c.nu_min));  // src/pixelize.c:369
  // src/pixelize.c:28-56: the walk ends in the unique bin nu0 <= nu < nuf of the contiguous table
  const double *e = c.nu_edges;
  if (!(nu >= __ldg(&e[0]))) return -1;
  if (nu >= __ldg(&e[c.n_nu])) return c.n_nu;
  int lo = 0, hi = c.n_nu;
  while (hi - lo > 1) {
    int mid = (lo + hi) >> 1;
    if (nu >= __ldg(&e[mid])) lo = mid;
    else hi = mid;
  }
  return lo;
}

__device__ __forceinline__ long loc2pix_exact(long nside, double z, double s, double phi)
{
  const double dn = (double)nside;
  double za = fabs(z);
  double tt = __dmul_rn(phi, INV_HALFPI_D);
  if (tt < 0) tt = __dadd_rn(tt, 4.0);
  if (za <= 2.0 / 3.0) {
    double t1 = __dmul_rn(dn, __dadd_rn(0.5, tt));
    double t2 = __dmul_rn(__dmul_rn(dn, z), 0.75);
    long jp = (long)__dsub_rn(t1, t2), jm = (long)__dadd_rn(t1, t2);
    long ir = nside + 1 + jp - jm;
    long kshift = 1 - (ir & 1);
    long ip = (jp + jm - nside + kshift + 1) / 2;
    ip %= 4 * nside;
    if (ip < 0) ip += 4 * nside;
    return 2 * nside * (nside - 1) + (ir - 1) * 4 * nside + ip;
  }
  double tp = __dsub_rn(tt, (double)(long)tt);
  double tmp = (s > -2) ? __ddiv_rn(__dmul_rn(dn, s), __dsqrt_rn(__ddiv_rn(__dadd_rn(1.0, za), 3.0)))
                        : __dmul_rn(dn, __dsqrt_rn(__dmul_rn(3.0, __dsub_rn(1.0, za))));
  long jp = (long)__dmul_rn(tp, tmp), jm = (long)__dmul_rn(__dsub_rn(1.0, tp), tmp);
  long ir = jp + jm + 1;
  long ip = (long)__dmul_rn(tt, (double)ir);
  ip %= 4 * ir;
  if (ip < 0) ip += 4 * ir;
  return (z > 0) ? 2 * ir * (ir - 1) + ip : 12 * nside * nside - 2 * ir * (ir + 1) + ip;
}

__device__ __noinline__ uint32_t key_exact(const DevCfg &c, int ix, int iy, int iz, int is, float dzf)
{
  double x = __dadd_rn(__dsub_rn(__dmul_rn(c.dx, (double)ix + 0.5), c.pos_obs), c.xs[is]);
  double y = __dadd_rn(__dsub_rn(__dmul_rn(c.dx, (double)iy + 0.5), c.pos_obs), c.ys[is]);
  double z = __dadd_rn(__dsub_rn(__dmul_rn(c.dx, (double)iz + 0.5), c.pos_obs), c.zs[is]);
  double xy2 = __dadd_rn(__dmul_rn(x, x), __dmul_rn(y, y));
  double r = __dsqrt_rn(__dadd_rn(xy2, __dmul_rn(z, z)));
  double red = __dadd_rn(z_of_r_exact(c, r), (double)dzf);
  double nu = __ddiv_rn(kNU21, __dadd_rn(1.0, red));
  int inu = bin_exact(c, nu);
  if (inu < 0 || inu >= c.n_nu) return 0xFFFFFFFFu;
  double cth = __ddiv_rn(z, r);
  double sth = fabs(cth) > 0.99 ? __ddiv_rn(__dsqrt_rn(xy2), r) : -5.0;
  long ipix = loc2pix_exact(c.nside, cth, sth, atan2(y, x));
  return (uint32_t)ipix + (uint32_t)c.npix * (uint32_t)inu;
}

// ---------------------------------------------------------------------------
// FP32 fast key with error margins.  Returns false when a floor or comparison
// of the exact computation lies within the FP32 error bound of a boundary; the
// caller then uses key_exact.  Bounds (5x safety on the estimated error):
//   shells: relative error of nu < 6e-7       -> margin 3e-6 nu
//   pixels: error of the floor arguments < nside (0.64 dtt + 0.75 dcos) + 2 ulp
// ---------------------------------------------------------------------------
struct FastConst {
  float xsf[kNSUB], ysf[kNSUB], zsf[kNSUB];
};

__device__ __forceinline__ bool near_int(float u, float m) { return fabsf(u - rintf(u)) < m; }

__device__ __forceinline__ bool key_fast(const DevCfg &c, const float *__restrict__ ef, float x, float y, float z,
                                         float dz, float epos, uint32_t &key)
{
  float rho2 = x * x + y * y;
  float r = sqrtf(rho2 + z * z);
  float tr = r * c.glob_idr_f;
  if (!(tr < (float)(kNZ - 2))) return false;
  int ir = (int)tr;
  float fr = tr - ir;
  float z0 = __ldg(&c.z_r2z_f[ir]), z1 = __ldg(&c.z_r2z_f[ir + 1]);
  float red = (z0 + (z1 - z0) * fr) + dz;
  float nu = 1420.40575177f / (1.f + red);
  float mnu = 3e-6f * nu;
  int inu;
  if (c.regular_nu) {
    float t = (nu - (float)c.nu_min) * (float)c.inv_dnu;
    if (near_int(t, mnu * (float)c.inv_dnu + 1e-6f * fabsf(t))) return false;
    inu = (int)t;
  } else {
    const int nn = c.n_nu;
    float e0 = __ldg(&ef[0]), en = __ldg(&ef[nn]);
    if (nu < e0) {
      if (e0 - nu < mnu) return false;
      inu = -1;
    } else if (nu >= en) {
      if (nu - en < mnu) return false;
      inu = nn;
    } else {
      int lo = 0, hi = nn;
      while (hi - lo > 1) {
        int mid = (lo + hi) >> 1;
        if (nu >= __ldg(&ef[mid])) lo = mid;
        else hi = mid;
      }
      if (nu - __ldg(&ef[lo]) < mnu || __ldg(&ef[lo + 1]) - nu < mnu) return false;
      inu = lo;
    }
  }
  if (inu < 0 || inu >= c.n_nu) {
    key = 0xFFFFFFFFu;
    return true;
  }
  // pixel
  const float fn = (float)c.nside;
  float ir_ = 1.f / r;
  float cth = z * ir_;
  float za = fabsf(cth);
  float rho = sqrtf(rho2);
  float dcos = 2.5e-7f + epos * ir_;
  if (fabsf(za - 0.6666667f) < 4.f * dcos + 1e-6f) return false;
  float phi = atan2f(y, x);
  float dtt = 0.6366198f * (4.8e-7f + 2.4e-7f * fabsf(phi) + epos / fmaxf(rho, 1e-30f));
  float tt = phi * 0.63661977f;
  if (tt < 0.f) tt += 4.f;
  const int npix = (int)c.npix;
  int pix;
  if (za <= 0.6666667f) {
    float t1 = fn * (0.5f + tt), t2 = fn * cth * 0.75f;
    float u1 = t1 - t2, u2 = t1 + t2;
    float mu = 5.f * (fn * (dtt + 0.75f * dcos) + 2.4e-7f * (fabsf(t1) + fabsf(t2)) + 1e-6f);
    if (near_int(u1, mu) || near_int(u2, mu)) return false;
    int jp = (int)u1, jm = (int)u2;
    int nside = (int)c.nside;
    int ring = nside + 1 + jp - jm;
    int kshift = 1 - (ring & 1);
    int ip = (jp + jm - nside + kshift + 1) / 2;
    ip %= 4 * nside;
    if (ip < 0) ip += 4 * nside;
    pix = 2 * nside * (nside - 1) + (ring - 1) * 4 * nside + ip;
  } else {
    float ft = floorf(tt);
    float tp = tt - ft;
    // nside sqrt(3(1-|z|)) in the cancellation-free form nside (rho/r) / sqrt((1+|z|)/3)
    float tmp = fn * (rho * ir_) * rsqrtf((1.f + za) * (1.f / 3.f));
    float dtmp = tmp * (1e-6f + epos / fmaxf(rho, 1e-30f));
    float u3 = tp * tmp, u4 = (1.f - tp) * tmp;
    float mu = 5.f * (tmp * dtt + dtmp + 2.4e-7f * tmp + 1e-6f);
    if (near_int(u3, mu) || near_int(u4, mu) || near_int(tp, 5.f * dtt + 1e-6f)) return false;
    int jp = (int)u3, jm = (int)u4;
    int ring = jp + jm + 1;
    float u5 = tt * ring;
    if (near_int(u5, 5.f * (ring * dtt + 4.8e-7f * u5 + 1e-6f))) return false;
    int ip = (int)u5;
    ip %= 4 * ring;
    if (ip < 0) ip += 4 * ring;
    pix = (cth > 0) ? 2 * ring * (ring - 1) + ip : npix - 2 * ring * (ring + 1) + ip;
  }
  key = (uint32_t)pix + (uint32_t)npix * (uint32_t)inu;
  return true;
}

// ---------------------------------------------------------------------------
// projection: 10 sub-samples per cell -> maps[bin][pix] += mass/10
// (src/pixelize.c:343-384).  Each block works through a contiguous chunk of
// cells; samples whose FP32 key is not certain are queued in shared memory and
// resolved with the exact FP64 key at the end of the chunk, so the FP64 units
// run on full warps.
// ---------------------------------------------------------------------------
constexpr int kProjThreads = 256;
constexpr int kQueueCap = 2048;

template <bool FUSED>
__global__ void __launch_bounds__(kProjThreads) project_kernel(DevCfg c, FastConst fc, const double *__restrict__ stats,
                                                               const float *__restrict__ a, const float *__restrict__ b,
                                                               float *__restrict__ maps, long cells_per_block,
                                                               int *__restrict__ counters)
{
  __shared__ uint32_t q_cell[kQueueCap];
  __shared__ float q_val[kQueueCap], q_dz[kQueueCap];
  __shared__ uint8_t q_sub[kQueueCap];
  __shared__ int q_n;
  __shared__ float sef[260];
  if (threadIdx.x == 0) q_n = 0;
  if (!c.regular_nu)
    for (int i = threadIdx.x; i <= c.n_nu && i < 260; i += blockDim.x) sef[i] = (float)c.nu_edges[i];
  __syncthreads();
  const float *ef = c.n_nu < 260 ? sef : c.nu_edges_f;
  const int n = c.n;
  const long total = (long)n * n * n;
  const float sigma2 = FUSED ? (float)stats[1] : 0.f;
  const float epos = 4.f * 6e-8f * (0.5f * (float)c.l_box) * 1.7320508f;
  const long c0 = blockIdx.x * cells_per_block;
  const long c1 = min(total, c0 + cells_per_block);
  int nfall = 0;
  for (long i = c0 + threadIdx.x; i < c1; i += blockDim.x) {
    const int ix = (int)(i % n);
    const long rest = i / n;
    const int iy = (int)(rest % n), iz = (int)(rest / n);
    float mass, dz;
    if (FUSED) {
      CellHI h = cell_hi(c, sigma2, ix, iy, iz, a[i], b[i]);
      mass = h.mass;
      dz = h.dz;
    } else {
      mass = a[i];
      dz = b[i];
    }
    const float msub = mass / 10.f;  // src/pixelize.c:356
    const float x0 = c.dxf * (ix + 0.5f) - c.pos_obsf, y0 = c.dxf * (iy + 0.5f) - c.pos_obsf,
                z0 = c.dxf * (iz + 0.5f) - c.pos_obsf;
#pragma unroll 2
    for (int is = 0; is < kNSUB; is++) {
      uint32_t key;
      bool ok = key_fast(c, ef, x0 + fc.xsf[is], y0 + fc.ysf[is], z0 + fc.zsf[is], dz, epos, key);
      if (ok) {
        if (key != 0xFFFFFFFFu) atomicAdd(&maps[key], msub);
      } else {
        int slot = atomicAdd(&q_n, 1);
        if (slot < kQueueCap) {
          q_cell[slot] = (uint32_t)(i - c0);
          q_sub[slot] = (uint8_t)is;
          q_val[slot] = msub;
          q_dz[slot] = dz;
        } else {
          key = key_exact(c, ix, iy, iz, is, dz);
          if (key != 0xFFFFFFFFu) atomicAdd(&maps[key], msub);
        }
        nfall++;
      }
    }
  }
  __syncthreads();
  const int qn = min(q_n, kQueueCap);
  for (int k = threadIdx.x; k < qn; k += blockDim.x) {
    long i = c0 + q_cell[k];
    const int ix = (int)(i % n);
    const long rest = i / n;
    uint32_t key = key_exact(c, ix, (int)(rest % n), (int)(rest / n), q_sub[k], q_dz[k]);
    if (key != 0xFFFFFFFFu) atomicAdd(&maps[key], q_val[k]);
  }
  if (counters) {
    for (int o = 16; o > 0; o >>= 1) nfall += __shfl_xor_sync(0xffffffffu, nfall, o);
    if ((threadIdx.x & 31) == 0 && nfall) atomicAdd(&counters[0], nfall);
  }
}

// maps *= M2T / (r(nu_c)^2 dnu) per channel, src/pixelize.c:399-414
__global__ void scale_maps_kernel(DevCfg c, float *maps)
{
  const long total = c.npix * (long)c.n_nu;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < total; i += (long)gridDim.x * blockDim.x)
    maps[i] *= __ldg(&c.prefac[i / c.npix]);
}

// per-sample keys (validation): exact FP64, or fast FP32 with FP64 fallback
__global__ void sample_keys_kernel(DevCfg c, FastConst fc, const float *__restrict__ dzg, uint32_t *keys, int exact)
{
  const int n = c.n;
  const long total = (long)n * n * n;
  const float epos = 4.f * 6e-8f * (0.5f * (float)c.l_box) * 1.7320508f;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < total; i += (long)gridDim.x * blockDim.x) {
    const int ix = (int)(i % n);
    const long rest = i / n;
    const int iy = (int)(rest % n), iz = (int)(rest / n);
    const float dz = dzg[i];
    const float x0 = c.dxf * (ix + 0.5f) - c.pos_obsf, y0 = c.dxf * (iy + 0.5f) - c.pos_obsf,
                z0 = c.dxf * (iz + 0.5f) - c.pos_obsf;
    for (int is = 0; is < kNSUB; is++) {
      uint32_t key;
      bool ok = false;
      if (!exact)
        ok = key_fast(c, c.nu_edges_f, x0 + fc.xsf[is], y0 + fc.ysf[is], z0 + fc.zsf[is], dz, epos, key);
      if (!ok) key = key_exact(c, ix, iy, iz, is, dz);
      keys[i * kNSUB + is] = key;
    }
  }
}

// ---------------------------------------------------------------------------
static int grid_for(long total, int threads)
{
  long b = (total + threads - 1) / threads;
  return (int)(b < 152L * 32 ? (b < 1 ? 1 : b) : 152L * 32);
}

cudaError_t radial_velocity_fd(const DevCfg &c, const float *vpot, float *rvel, cudaStream_t st)
{
  long total = (long)c.n * c.n * c.n;
  fd_vel_kernel<<<grid_for(total, 256), 256, 0, st>>>(c, vpot, rvel);
  return cudaGetLastError();
}

cudaError_t get_hi(const DevCfg &c, const double *stats, float *dens, float *rvel, cudaStream_t st)
{
  long total = (long)c.n * c.n * c.n;
  get_hi_kernel<<<grid_for(total, 256), 256, 0, st>>>(c, stats, dens, rvel);
  return cudaGetLastError();
}

static FastConst fast_const(const DevCfg &c)
{
  FastConst f;
  for (int i = 0; i < kNSUB; i++) {
    f.xsf[i] = (float)c.xs[i];
    f.ysf[i] = (float)c.ys[i];
    f.zsf[i] = (float)c.zs[i];
  }
  return f;
}

cudaError_t project(const DevCfg &c, const double *stats, const float *a, const float *b, int fused, float *maps,
                    int *counters, cudaStream_t st)
{
  long total = (long)c.n * c.n * c.n;
  long cpb = 4096;
  long blocks = (total + cpb - 1) / cpb;
  FastConst fc = fast_const(c);
  if (fused) project_kernel<true><<<(unsigned)blocks, kProjThreads, 0, st>>>(c, fc, stats, a, b, maps, cpb, counters);
  else project_kernel<false><<<(unsigned)blocks, kProjThreads, 0, st>>>(c, fc, stats, a, b, maps, cpb, counters);
  return cudaGetLastError();
}

cudaError_t scale_maps(const DevCfg &c, float *maps, cudaStream_t st)
{
  scale_maps_kernel<<<grid_for(c.npix * (long)c.n_nu, 256), 256, 0, st>>>(c, maps);
  return cudaGetLastError();
}

cudaError_t sample_keys(const DevCfg &c, const float *dz, uint32_t *keys, int exact, cudaStream_t st)
{
  long total = (long)c.n * c.n * c.n;
  sample_keys_kernel<<<grid_for(total, 128), 128, 0, st>>>(c, fast_const(c), dz, keys, exact);
  return cudaGetLastError();
}

}  // namespace gethi
