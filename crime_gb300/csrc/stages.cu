// Real-space stages of the GetHI realisation on GB300: radial velocity by
// finite differences, the lognormal HI transform and the projection of cells
// onto (HEALPix pixel, frequency shell) maps.
#include <cstdio>

#include <cmath>

#include "common.cuh"
#include "dfloat.cuh"
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
// (src/pixelize.c:206-222, src/cosmo.c:52-62) with every rounding explicit, so
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
  if (c.regular_nu) return (int)__dmul_rn(c.inv_dnu, __dsub_rn(nu, c.nu_min));  // src/pixelize.c:216
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
// Refinement of a key the FP32 path left uncertain, in double-float arithmetic
// (about 48 bits; dfloat.cuh).  The operation sequence is key_exact's, the
// angle comes from a double-float atan2, and every floor and comparison must
// clear a margin of 1e-9 of its operands' scale, far above the errors of both
// this arithmetic (< 1e-12) and the FP64 reference (< 1e-15), so a certain
// result is the FP64 key.  unc = true hands the sample to key_exact.
// ---------------------------------------------------------------------------
__device__ __noinline__ uint32_t key_refine(const DevCfg &c, int ix, int iy, int iz, int is, float dzf, bool &unc)
{
  unc = false;
  constexpr float kM = 1e-9f;
  const df dx = df_of(c.dx_df), po = df_of(c.pos_obs_df);
  const df x = df_add(df_sub(df_mul_f(dx, (float)ix + 0.5f), po), df_of(c.xs_df[is]));
  const df y = df_add(df_sub(df_mul_f(dx, (float)iy + 0.5f), po), df_of(c.ys_df[is]));
  const df z = df_add(df_sub(df_mul_f(dx, (float)iz + 0.5f), po), df_of(c.zs_df[is]));
  const df xy2 = df_add(df_mul(x, x), df_mul(y, y));
  const df r2 = df_add(xy2, df_mul(z, z));
  if (!(r2.hi > 0.f) || !(xy2.hi > 0.f)) {
    unc = true;
    return 0;
  }
  const df r = df_sqrt(r2);
  // z(r), src/cosmo.c:52-62 (piecewise linear: continuous, so the segment index needs no margin)
  df red;
  if (r.hi >= c.r_tab_max_f) {
    red = df_of(c.z_r2z_df[kNZ - 1]);
  } else {
    const df tr = df_mul(r, df_of(c.glob_idr_df));
    const int ir = min(max((int)floorf(tr.hi), 0), kNZ - 2);
    const df z0 = df_of(c.z_r2z_df[ir]), z1 = df_of(c.z_r2z_df[ir + 1]), r0 = df_of(c.r_r2z_df[ir]);
    red = df_add(z0, df_mul(df_mul(df_sub(z1, z0), df_sub(r, r0)), df_of(c.glob_idr_df)));
  }
  red = df_add(red, df_f(dzf));
  constexpr df kNu21 = df_const(1420.40575177);
  const df nu = df_div(kNu21, df_add(df_f(1.f), red));
  int inu;
  if (c.regular_nu) {  // (int) truncation, src/pixelize.c:216
    const df t = df_mul(df_of(c.inv_dnu_df), df_sub(nu, df_of(c.nu_min_df)));
    const float m = kM * (fabsf(t.hi) + fabsf(c.inv_dnu_df.x * nu.hi) + 1.f);
    const int f = df_floor(t, m, unc);
    inu = (t.hi < 0.f) ? f + 1 : f;
  } else {  // the bin nu0 <= nu < nuf of the contiguous table (src/pixelize.c:28-56)
    const int nn = c.n_nu;
    int lo = -1, hi = nn + 1;  // e[lo] <= nu < e[hi] over edges 0..nn, with -1 / nn+1 as sentinels
    while (hi - lo > 1) {
      const int mid = (lo + hi) >> 1;
      if (df_ge(nu, df_of(c.nu_edges_df[mid]))) lo = mid;
      else hi = mid;
    }
    const float m = kM * nu.hi;
    if (lo >= 0 && fabsf(df_sub(nu, df_of(c.nu_edges_df[lo])).hi) < m) unc = true;
    if (hi <= nn && fabsf(df_sub(nu, df_of(c.nu_edges_df[hi])).hi) < m) unc = true;
    inu = lo < 0 ? -1 : (lo >= nn ? nn : lo);
  }
  if (unc) return 0;
  if (inu < 0 || inu >= c.n_nu) return 0xFFFFFFFFu;  // outside the shells
  // pixel (loc2pix_exact)
  const long nside = c.nside;
  const float dn = (float)nside;
  const df cth = df_div(z, r);
  const df za = df_abs(cth);
  constexpr df kTwoThirds = df_const(2.0 / 3.0), kInvHalfPi = df_const(0.63661977236758134308);
  if (fabsf(df_sub(za, kTwoThirds).hi) < kM) {
    unc = true;
    return 0;
  }
  df tt = df_mul(df_atan2(y, x), kInvHalfPi);
  if (tt.hi < 0.f) tt = df_add(tt, df_f(4.f));
  const float m = kM * (5.f * dn + 1.f);
  long pix;
  if (df_ge(kTwoThirds, za)) {
    const df t1 = df_mul_f(df_add(df_f(0.5f), tt), dn);
    const df t2 = df_mul_f(df_mul_f(cth, dn), 0.75f);
    const long jp = df_floor(df_sub(t1, t2), m, unc), jm = df_floor(df_add(t1, t2), m, unc);
    const long ir = nside + 1 + jp - jm;
    const long kshift = 1 - (ir & 1);
    long ip = (jp + jm - nside + kshift + 1) / 2;
    ip %= 4 * nside;
    if (ip < 0) ip += 4 * nside;
    pix = 2 * nside * (nside - 1) + (ir - 1) * 4 * nside + ip;
  } else {
    const int ftt = df_floor(tt, 5.f * kM, unc);
    const df tp = df_sub(tt, df_f((float)ftt));
    const df sth = df_div(df_sqrt(xy2), r);
    const df tmp = df_div(df_mul_f(sth, dn), df_sqrt(df_mul(df_add(df_f(1.f), za), df_const(1.0 / 3.0))));
    const float mt = kM * (tmp.hi + 1.f);
    const long jp = df_floor(df_mul(tp, tmp), mt, unc);
    const long jm = df_floor(df_mul(df_sub(df_f(1.f), tp), tmp), mt, unc);
    const long ir = jp + jm + 1;
    long ip = df_floor(df_mul_f(tt, (float)ir), kM * (4.f * (float)ir + 1.f), unc);
    ip %= 4 * ir;
    if (ip < 0) ip += 4 * ir;
    pix = (cth.hi > 0.f) ? 2 * ir * (ir - 1) + ip : 12 * nside * nside - 2 * ir * (ir + 1) + ip;
  }
  if (unc) return 0;
  return (uint32_t)pix + (uint32_t)c.npix * (uint32_t)inu;
}

// the key of an uncertain sample: double-float refinement, FP64 when that is not decisive
__device__ __forceinline__ uint32_t key_resolve(const DevCfg &c, int ix, int iy, int iz, int is, float dzf)
{
  if (c.z_r2z_df) {
    bool unc;
    const uint32_t k = key_refine(c, ix, iy, iz, is, dzf, unc);
    if (!unc) return k;
  }
  return key_exact(c, ix, iy, iz, is, dzf);
}

// ---------------------------------------------------------------------------
// FP32 fast key with certified margins.  Geometry is in cell units relative to
// the observer: X = (ix - n/2) + (0.5 + xs/dx), which FP32 holds to half an
// ulp of |X|.  Every floor and comparison of the exact computation is made on
// an FP32 value whose worst-case error is bounded below; if the value lies
// within twice that bound of the decision boundary the sample is "uncertain"
// and key_exact decides it.  Error budget (relative unless stated):
//   position 6e-8; R = sqrt(R^2) 3.6e-7; table redshift abs 1e-6 + 3e-7 (1+z);
//   nu 6e-7 -> shell margin 1.2e-6 nu.
//   angle: the octant angle a = atan2f(min,max) in [0, pi/4] has <= 3 ulp
//   (1.8e-7) + 6e-8 from the position; cos(theta) = Z/R <= 2.5e-7 abs.
//   floor arguments are split into an exact integer/half-integer part and a
//   remainder of magnitude <= nside + 1, so their rounding is <= 2 ulp(nside+1).
// ---------------------------------------------------------------------------
struct FastConst {
  float xsp[kNSUB], ysp[kNSUB], zsp[kNSUB];  // 0.5 + offset/dx
  float idr_cell;                             // glob_idr * dx
  float rho, rho_idr;                         // sub-sample distance bound from the cell centre (cells), * idr_cell
  float half_n;                               // n/2
  float nu_min, inv_dnu;                      // regular table
  // the projection visits the sub-samples along a short path through the cell
  // (consecutive samples then share a key more often, so a cell's runs of equal
  // keys are longer): tour[j] is the j-th sample's index, txsp.. its offsets
  int tour[kNSUB];
  float txsp[kNSUB], tysp[kNSUB], tzsp[kNSUB];
  // key_lin: the j-th sample's offset from the cell centre and its monomials
  float tox[kNSUB], toy[kNSUB], toz[kNSUB], toxx[kNSUB], toyy[kNSUB], tozz[kNSUB];
  float toxy[kNSUB], toxz[kNSUB], toyz[kNSUB], tdxy[kNSUB];
};

__device__ __forceinline__ bool near_int(float u, float m) { return fabsf(u - rintf(u)) < m; }

// atan(t) for t in [0,1] as t P(t^2), P of degree 8 (coefficients from a
// weighted least-squares fit toward minimax); evaluated in FP32 with FMAs the
// error stays below 8.6e-8 (checked on 2e6 points against FP64 atan).
__device__ __forceinline__ float atan01(float t)
{
  const float s = t * t;
  float p = 0.0024567206855863333f;
  p = fmaf(p, s, -0.014401344582438469f);
  p = fmaf(p, s, 0.03978120908141136f);
  p = fmaf(p, s, -0.07234856486320496f);
  p = fmaf(p, s, 0.10498946160078049f);
  p = fmaf(p, s, -0.14161229133605957f);
  p = fmaf(p, s, 0.19985906779766083f);
  p = fmaf(p, s, -0.33332598209381104f);
  p = fmaf(p, s, 0.9999998807907104f);
  return p * t;
}

// Error bounds used below (absolute unless noted), with a factor 2 on top:
//   position X,Y,Z: 6e-8 relative; R^2 (3 FMAs): 2.4e-7 rel; rsqrt.approx: 1.3e-7 rel
//   R = R^2 rsqrt(R^2): 3.1e-7 rel; cos(theta) = Z rsqrt(R^2): 3.7e-7
//   1+z from the FP32 table: |z1-z0| tr 3.7e-7 + 4 ulp(1+z); nu (approximate division): +2.7e-7 rel
//   octant angle: atan01 8.6e-8 + ratio (2 ulp) 9e-8; w = 2a/pi or 1-2a/pi: 2.05e-7
//   floor arguments: nside (dw + 6e-8 + 0.75 dcos) + 4 half-ulps at 1.5 nside
constexpr uint32_t kKeyInvalid = 0xFFFFFFFFu;    // outside the shells
constexpr uint32_t kKeyUncertain = 0xFFFFFFFEu;  // FP32 cannot decide: use key_exact
// (valid keys are < n_nu * 12 nside^2 <= 2^32 - 2, checked at set-up)

__device__ __forceinline__ uint32_t pixel_fast(const DevCfg &c, float X, float Y, float Z, float rho2, float iR);

// frequency-file edges ef[0..nn] (FP32, increasing): the last index lo in -1..nn
// with ef[lo] <= nu, branch-free over the steps 2^log2nn .. 1
__device__ __forceinline__ int edge_search(const float *ef, int nn, int log2nn, float nu)
{
  int lo = -1;
#pragma unroll 1
  for (int step = 1 << log2nn; step > 0; step >>= 1) {
    const int cand = lo + step;
    lo = (cand <= nn && nu >= ef[min(cand, nn)]) ? cand : lo;
  }
  return lo;
}

// The shell coordinate of a cell's sub-samples, linear in their radius.
//
// Within one cell the redshift shift dz is fixed and the sub-samples lie within
// rho cells of the centre, so the shell coordinate u (the channel coordinate
// t = (nu - nu_min)/dnu of a regular table, the frequency nu itself for a
// frequency file) is set once per cell as
//     u(R) = u_c + s (R - Rc),   |u(R) - u_exact(R)| < m,
// and each sub-sample spends one subtraction and one FMA on it (key_fast), or
// three FMAs on its offset o with R - Rc = r_hat.o (key_lin, bound ml).  u_exact is the
// FP64 key's value: u of 1 + z(R) + dz, z the piecewise-linear FP64 table
// (src/cosmo.c:52-62).  s = du/dz g, with g the slope of the table interval
// the centre falls in; z(R) stays within e of that interval's line for every R
// a sub-sample of the cell can have (z_lin_g / z_lin_e, from the FP64 table).
// The bound m is the per-sample budget above taken at the centre (whose radius
// is correctly rounded: 1.8e-7), plus (each term x 1.5):
//   radius rounding of the sub-sample and the centre: |s| (3.7e-7 (Rc + rho) + 1.8e-7 Rc)
//     (R - Rc is exact: both lie within a factor 2 of each other);
//   the table: |du/dz| e;
//   the FP32 slope and the products forming s: 2e-6 |s| rho;
//   curvature of u in z: |d2u/dz2| dZ^2/2 <= A sc dZ^2 / (1 + z + dz - dZ)^3,
//     dZ = |g| rho + e the largest change of z over the cell;
//   rounding of the FMAs: 2e-7 (|u_c| + |s| rho) (up to three).
// Cells closer than 2 rho + 2 cells to the observer, or reaching the last table
// interval, get m = inf: their sub-samples all go to the exact path.
//
// A frequency file also keeps the bins around the centre: bin lo of u_c and
// the edges ef[lo-1] .. ef[lo+2] (-inf / +inf beyond 0..nn).  A sub-sample
// within one bin of the centre's is binned with four compares; the search is
// left to samples two or more bins away.
struct CellShell {
  float u, s, Rc, m;
  float gx, gy, gz, ml;  // key_lin: du/do = s r_hat and its bound
  int lo;
  float e0, e1, e2, e3;
};

__device__ __forceinline__ CellShell cell_shell(const DevCfg &c, const FastConst &f, const float *ef, int log2nn,
                                                float Xc, float Yc, float Zc, float dz)
{
  constexpr float A = 1420.40575177f;
  CellShell o;
  // the centre: quarter-integer squares, so R2 is exact below 2^22 and rounded
  // once above; sqrtf is correctly rounded (1.8e-7 covers both)
  const float X = Xc + 0.5f, Y = Yc + 0.5f, Z = Zc + 0.5f;
  const float R2 = fmaf(Z, Z, fmaf(Y, Y, X * X));
  const float Rc = sqrtf(R2);
  const float tr = Rc * f.idr_cell;
  bool ok = tr + f.rho_idr < (float)(kNZ - 3) && Rc > 2.f * f.rho + 2.f;
  const float trs = ok ? tr : 0.f;
  const int ir = (int)trs;
  const float z0 = __ldg(&c.z_r2z_f[ir]), z1 = __ldg(&c.z_r2z_f[ir + 1]);
  const float g = __ldg(&c.z_lin_g[ir]), e = __ldg(&c.z_lin_e[ir]);  // slope per cell, line bound
  const float dzt = z1 - z0;
  const float zz = 1.f + (fmaf(dzt, trs - (float)ir, z0) + dz);
  const float izz = __fdividef(1.f, zz);
  const float nu = A * izz;
  const float sc = c.regular_nu ? f.inv_dnu : 1.f;
  const float u = c.regular_nu ? (nu - f.nu_min) * sc : nu;
  const float mnu = 2.f * nu * (fabsf(dzt) * trs * 1.8e-7f * izz + 4.8e-7f + 2.7e-7f);
  const float mc = c.regular_nu ? (mnu + 1.2e-7f * nu) * sc + 4e-7f * fabsf(u) + 1e-6f : mnu;
  const float d1 = A * sc * izz * izz;  // |du/dz| at the centre
  const float s = -d1 * g;
  const float dZ = fabsf(g) * f.rho + e;  // largest |z(R) - z(Rc)| over the cell
  const float zlo = zz - dZ;
  ok = ok && zlo > 0.25f;
  const float izlo = __fdividef(1.f, zlo);
  const float common = d1 * e + 2e-6f * fabsf(s) * f.rho + A * sc * dZ * dZ * izlo * izlo * izlo +
                       2e-7f * (fabsf(u) + fabsf(s) * f.rho);
  const float lin = fabsf(s) * (3.7e-7f * (Rc + f.rho) + 1.8e-7f * Rc) + common;
  // key_lin: R - Rc = r_hat.o + h, 0 <= h <= rho^2 / (2 (Rc - rho)) (|P| is convex; its
  // Hessian is below 1/|P|); r_hat = C/Rc to 3e-7; FP32 offsets within 1e-7 cells
  const float linq = fabsf(s) * (__fdividef(f.rho * f.rho, 2.f * (Rc - f.rho)) + 3e-7f * f.rho + 1e-7f) + common;
  const float inf = __int_as_float(0x7f800000);
  o.u = ok ? u : 0.5f;
  o.s = ok ? s : 0.f;
  o.Rc = Rc;
  o.m = ok ? mc + 1.5f * lin : inf;
  o.ml = ok ? mc + 1.5f * linq : inf;
  const float sr = o.s * __fdividef(1.f, Rc);
  o.gx = sr * X;
  o.gy = sr * Y;
  o.gz = sr * Z;
  o.lo = 0;
  o.e0 = o.e1 = o.e2 = o.e3 = 0.f;
  if (!c.regular_nu) {
    const int nn = c.n_nu;
    o.lo = edge_search(ef, nn, log2nn, o.u);
    o.e0 = o.lo - 1 >= 0 ? ef[o.lo - 1] : -inf;
    o.e1 = o.lo >= 0 ? ef[o.lo] : -inf;
    o.e2 = o.lo + 1 <= nn ? ef[o.lo + 1] : inf;
    o.e3 = o.lo + 2 <= nn ? ef[min(o.lo + 2, nn)] : inf;
  }
  return o;
}

// shell bin inu of the coordinate u, unc when u lies within m of a bin edge
__device__ __forceinline__ void shell_bin(const DevCfg &c, const float *ef, int log2nn, const CellShell &cs, float u,
                                          float m, int &inu, bool &unc)
{
  if (c.regular_nu) {
    unc = near_int(u, m);
    inu = (int)u;  // truncation, src/pixelize.c:216
  } else {
    // bin inu: ef[inu] <= nu < ef[inu + 1] (-1 below ef[0], nn at or above ef[nn])
    const float nu = u;
    inu = cs.lo + (nu >= cs.e2 ? 1 : 0) - (nu < cs.e1 ? 1 : 0);
    unc = fabsf(nu - cs.e0) < m || fabsf(nu - cs.e1) < m || fabsf(nu - cs.e2) < m || fabsf(nu - cs.e3) < m;
    if (nu < cs.e0 || nu >= cs.e3) {  // two or more bins from the cell centre's (rare)
      const int nn = c.n_nu;
      const int lo = edge_search(ef, nn, log2nn, nu);
      inu = lo;
      const float below = lo >= 0 ? nu - ef[max(lo, 0)] : 1e30f;
      const float above = lo < nn ? ef[min(lo + 1, nn)] - nu : 1e30f;
      unc = below < m || above < m;
    }
  }
}

// every sub-sample of the cell certainly outside the shells (then all its keys are
// kKeyInvalid): the exact coordinate of each lies within max(m, ml) of the cell's
// line, which moves by at most |s| rho over the cell
__device__ __forceinline__ bool cell_outside(const DevCfg &c, const FastConst &f, const float *ef, const CellShell &cs)
{
  const float span = fabsf(cs.s) * f.rho * 1.000001f + fmaxf(cs.m, cs.ml) + 1e-6f * fabsf(cs.u) + 1e-6f;
  const float hi = cs.u + span, lo = cs.u - span;
  return c.regular_nu ? (hi <= -1.f || lo >= (float)c.n_nu) : (hi < ef[0] || lo >= ef[c.n_nu]);
}

__device__ __forceinline__ uint32_t key_fast(const DevCfg &c, const float *ef, int log2nn, const CellShell &cs,
                                             float X, float Y, float Z)
{
  const float rho2 = fmaf(Y, Y, X * X);
  const float R2 = fmaf(Z, Z, rho2);
  const float iR = rsqrtf(R2);
  int inu;
  bool unc;
  shell_bin(c, ef, log2nn, cs, fmaf(cs.s, R2 * iR - cs.Rc, cs.u), cs.m, inu, unc);
  // selected at the end, like key_lin (the pixel of a sample outside the shells is unused)
  const uint32_t pix = pixel_fast(c, X, Y, Z, rho2, iR);
  const bool out = (uint32_t)inu >= (uint32_t)c.n_nu;
  const uint32_t key = pix + (uint32_t)c.npix * (uint32_t)inu;
  return (!(rho2 > 0.f) | unc) ? kKeyUncertain : (out ? kKeyInvalid : (pix == kKeyUncertain ? kKeyUncertain : key));
}

// octant decomposition of the azimuth: a = atan(min/max) in [0, pi/4];
// tt = 2 phi/pi = q + w, q in 0..3, w in [0, 1) within 2.05e-7 of the exact value
__device__ __forceinline__ void azimuth(float X, float Y, int &q, float &w)
{
  const float ax = fabsf(X), ay = fabsf(Y);
  const bool swap = ay > ax;
  const float a2 = atan01(__fdividef(fminf(ax, ay), fmaxf(ax, ay))) * 0.63661977f;  // in [0, 0.5]
  const bool upper = Y >= 0.f, right = X >= 0.f;
  q = upper ? (right ? 0 : 1) : (right ? 3 : 2);
  // w = a2 when the octant runs counter-clockwise from the quadrant start, else 1 - a2
  const bool ccw = ((q & 1) == 0) ? !swap : swap;
  w = ccw ? a2 : 1.f - a2;
  const bool wrap = w >= 1.f;
  w = wrap ? w - 1.f : w;
  q = wrap ? ((q + 1) & 3) : q;
}

// RING pixel of (X, Y, Z) (cell units, |error| <= 6e-8 relative), rho2 = X^2 + Y^2,
// iR = 1/|.|; kKeyUncertain when a floor or comparison is within its margin
__device__ __forceinline__ uint32_t pixel_fast(const DevCfg &c, float X, float Y, float Z, float rho2, float iR)
{
  const int nside = (int)c.nside;
  const float fn = (float)nside;
  const float cth = Z * iR;
  const float za = fabsf(cth);
  const float dcos = 3.7e-7f;
  int q;
  float w;
  azimuth(X, Y, q, w);
  const float dw = 2.05e-7f;
  const int npix = (int)c.npix;
  bool unc = fabsf(za - 0.6666667f) < 2.f * dcos + 6e-8f;
  int pix;
  if (za <= 0.6666667f) {
    const float t2 = fn * cth * 0.75f;
    const float v = fn * (0.5f + w);
    const float v1 = v - t2, v2 = v + t2;
    const float mu = 2.f * (fn * (dw + 6e-8f + 0.75f * dcos) + 2.f * 1.2e-7f * (1.5f * fn + 1.f));
    unc |= near_int(v1, mu) | near_int(v2, mu);
    const int f1 = (int)floorf(v1), f2 = (int)floorf(v2);
    const int ring = nside + 1 + f1 - f2;  // jp - jm: the q nside terms cancel
    const int num = f1 + f2 + (2 * q - 1) * nside + (1 - (ring & 1)) + 1;  // jp + jm - nside + kshift + 1 >= -1
    int ip = (num + (num < 0)) >> 1;                                        // C division by 2
    ip = ip >= 4 * nside ? ip - 4 * nside : ip;
    pix = 2 * nside * (nside - 1) + (ring - 1) * 4 * nside + ip;
  } else {
    // polar caps: nside sqrt(3(1-|z|)) = nside (rho/R) / sqrt((1+|z|)/3)
    const float st = rho2 * rsqrtf(rho2) * iR;
    const float tmp = fn * st * rsqrtf((1.f + za) * (1.f / 3.f));
    const float u3 = w * tmp, u4 = (1.f - w) * tmp;
    const float mu = 2.f * (tmp * (dw + 1e-6f) + 2.f * 1.2e-7f * (tmp + 1.f));
    const int jp = (int)u3, jm = (int)u4;
    const int ring = jp + jm + 1;
    const float u5 = w * (float)ring;
    unc |= near_int(u3, mu) | near_int(u4, mu) | (w < 2.f * dw) | (1.f - w < 2.f * dw) |
           near_int(u5, 2.f * ((float)ring * dw + 2.4e-7f * (u5 + 1.f)));
    const int ip = q * ring + (int)u5;  // floor(tt ring) < 4 ring
    pix = (cth > 0) ? 2 * ring * (ring - 1) + ip : npix - 2 * ring * (ring + 1) + ip;
  }
  // no early returns (as in key_lin); a pixel outside the map only comes from an uncertain sample
  return (unc | ((uint32_t)pix >= (uint32_t)npix)) ? kKeyUncertain : (uint32_t)pix;
}

// ---------------------------------------------------------------------------
// Equatorial cells: the RING floor arguments as quadratics in the sub-sample offset.
//
// In the equatorial zone (|cos theta| <= 2/3) the pixel of a point is fixed by
// floor(V1), floor(V2), V1,2 = n (0.5 + tt) -/+ 0.75 n cos(theta) - n q, with
// tt = 2 phi/pi = q + w (src/pixelize.c:216-218; the RING scheme of Gorski et
// al. 2005).  For a cell C whose sub-samples C + o all lie in that zone, on one
// side of phi = 0, this takes per cell
//     V(C + o) = V(C) + grad V . o + o.H.o/2 + r3,
// phi and cos theta expanded to second order at C:
//   phi: grad = (-y, x, 0)/rxy^2; o.H.o/2 = (xy (ox^2 - oy^2) + (y^2 - x^2) ox oy)/rxy^4;
//        |r3| <= |o|^3/(3 rxy_min^3) (the k-th derivative of Im log(x + iy) is (k-1)!/|x + iy|^k);
//   cos theta = z/r: grad = (-xz, -yz, x^2 + y^2)/r^3;
//        H = -(z P P^T 3/r^2 ... ): H_xx = z (3x^2/r^2 - 1)/r^3, H_yy = z (3y^2/r^2 - 1)/r^3,
//        H_zz = 3z (z^2/r^2 - 1)/r^3, H_xy = 3xyz/r^5, H_xz = x (3z^2/r^2 - 1)/r^3,
//        H_yz = y (3z^2/r^2 - 1)/r^3; |r3| <= |o|^3/(2 r_min^3) (third derivative of z/r below
//        3/r^3 over the sphere), taken twice over.
// The offsets' monomials are per-sample constants, so a sub-sample costs 13 FMAs for
// both arguments.  The bound mu (x2 like every fast-path margin) holds the
// centre's azimuth (2.05e-7) and cos theta (2.4e-7 of |cos|), the rounding of
// V(C) (3e-7 n) and of the final sum (1.2e-7 n), 1e-6 of the expansion's size
// for its FP32 coefficients, 1e-7 cells per offset and the third-order terms.
// ---------------------------------------------------------------------------
struct CellPix {
  float v1, v2, mu;
  int qterm;                                       // (2q - 1) nside
  float a1, a2, a3, a4;                            // n dtt on ox, oy, ox^2 - oy^2, ox oy
  float b1, b2, b3, b4, b5, b6, b7, b8, b9;        // 0.75 n dcos on ox, oy, oz, ox^2, oy^2, oz^2, ox oy, ox oz, oy oz
  bool lin;
};

__device__ __forceinline__ CellPix cell_pix(const DevCfg &c, const FastConst &f, float X, float Y, float Z, float Rc)
{
  CellPix p;
  const float fn = (float)c.nside, K = fn * 0.63661977f, L = 0.75f * fn, rho = f.rho;
  const float rxy2 = fmaf(Y, Y, X * X);
  const float rxy = sqrtf(rxy2);
  const float cth = __fdiv_rn(Z, Rc);
  int q;
  float w;
  azimuth(X, Y, q, w);
  const float rmin = Rc - rho, rxymin = rxy - rho;
  const float i1 = __fdividef(rho, rxymin), i2 = __fdividef(rho, rmin);
  const float dT = 0.63661977f * i1 + 1e-5f;
  p.lin = rxymin > 1.f && fabsf(cth) + i2 + 1e-5f < 0.66666f && !((q == 0 && w < dT) || (q == 3 && w > 1.f - dT));
  const float irxy2 = __fdividef(1.f, rxy2), iR = __fdividef(1.f, Rc);
  const float Kr = K * irxy2, Kr2 = Kr * irxy2;
  p.a1 = -Kr * Y;
  p.a2 = Kr * X;
  p.a3 = Kr2 * (X * Y);
  p.a4 = Kr2 * (Y * Y - X * X);
  const float Lr3 = L * iR * iR * iR, h = 0.5f * Lr3;
  const float sx = X * iR, sy = Y * iR, c2 = cth * cth, t3 = 3.f * c2 - 1.f;
  p.b1 = -Lr3 * (X * Z);
  p.b2 = -Lr3 * (Y * Z);
  p.b3 = Lr3 * rxy2;
  p.b4 = h * Z * (3.f * sx * sx - 1.f);
  p.b5 = h * Z * (3.f * sy * sy - 1.f);
  p.b6 = 3.f * h * Z * (c2 - 1.f);
  p.b7 = 3.f * Lr3 * Z * sx * sy;
  p.b8 = Lr3 * X * t3;
  p.b9 = Lr3 * Y * t3;
  const float base = fn * (0.5f + w), Lc = L * cth;
  p.v1 = base - Lc;
  p.v2 = base + Lc;
  p.qterm = (2 * q - 1) * (int)c.nside;
  const float sa = fabsf(p.a1) + fabsf(p.a2) + fabsf(p.b1) + fabsf(p.b2) + fabsf(p.b3);
  const float sq = fabsf(p.a3) + fabsf(p.a4) + fabsf(p.b4) + fabsf(p.b5) + fabsf(p.b6) + fabsf(p.b7) +
                   fabsf(p.b8) + fabsf(p.b9);
  const float third = K * i1 * i1 * i1 * (1.f / 3.f) + L * i2 * i2 * i2;
  p.mu = 2.f * (fn * (2.05e-7f + 3e-7f + 1.2e-7f) + L * 2.4e-7f + 1e-6f * (sa * rho + sq * rho * rho) + 1e-7f * sa +
                third);
  return p;
}

// key of sub-sample j (tour order) of a cell with cp.lin: shell from u = u_c + s r_hat.o,
// pixel from the quadratics (same integer steps as pixel_fast's equatorial branch).
// Everything is evaluated and the key selected at the end: early returns cost
// more in branches and convergence barriers than the arithmetic they skip.  A
// pixel outside the equatorial rings (impossible for a certified sample) goes to
// the exact key, so no key can leave the maps.
__device__ __forceinline__ uint32_t key_lin(const DevCfg &c, const FastConst &f, const float *ef, int log2nn,
                                            const CellShell &cs, const CellPix &p, int j)
{
  const float ox = f.tox[j], oy = f.toy[j], oz = f.toz[j];
  int inu;
  bool unc;
  shell_bin(c, ef, log2nn, cs, fmaf(cs.gz, oz, fmaf(cs.gy, oy, fmaf(cs.gx, ox, cs.u))), cs.ml, inu, unc);
  const float dP = fmaf(p.a4, f.toxy[j], fmaf(p.a3, f.tdxy[j], fmaf(p.a2, oy, p.a1 * ox)));
  const float dQ = fmaf(p.b9, f.toyz[j], fmaf(p.b8, f.toxz[j], fmaf(p.b7, f.toxy[j], fmaf(p.b6, f.tozz[j],
                   fmaf(p.b5, f.toyy[j], fmaf(p.b4, f.toxx[j], fmaf(p.b3, oz, fmaf(p.b2, oy, p.b1 * ox))))))));
  const float v1 = p.v1 + (dP - dQ), v2 = p.v2 + (dP + dQ);
  const bool pu = near_int(v1, p.mu) | near_int(v2, p.mu);
  const int nside = (int)c.nside;
  const int f1 = (int)floorf(v1), f2 = (int)floorf(v2);
  const int ring = nside + 1 + f1 - f2;
  const int num = f1 + f2 + p.qterm + (1 - (ring & 1)) + 1;
  int ip = (num + (num < 0)) >> 1;
  ip = ip >= 4 * nside ? ip - 4 * nside : ip;
  const int pix = 2 * nside * (nside - 1) + (ring - 1) * 4 * nside + ip;
  const bool out = (uint32_t)inu >= (uint32_t)c.n_nu;
  const bool bad = pu | ((uint32_t)pix >= (uint32_t)c.npix);
  const uint32_t key = (uint32_t)pix + (uint32_t)c.npix * (uint32_t)inu;
  return unc ? kKeyUncertain : (out ? kKeyInvalid : (bad ? kKeyUncertain : key));
}

// ---------------------------------------------------------------------------
// projection: 10 sub-samples per cell -> maps[bin][pix] += mass/10
// (src/pixelize.c:190-231).  One block per 8x8x(4 zsteps) tile of cells.  Each
// thread merges runs of equal keys among its cell's sub-samples (visited along
// a short path through the cell) and adds each run to the map with one L2
// reduction (red.global.add.f32, no return value).  Samples whose FP32 key is
// uncertain are queued and resolved with the FP64 key at the end of the tile
// (or by fixup_kernel).  A shared-memory table that first summed the tile's
// runs per distinct key cost more than it saved: 83 ms against 66 ms for the
// direct reductions at 1024^3, Nside 512 x 150 shells.
// ---------------------------------------------------------------------------
constexpr int kProjThreads = 256;
constexpr int kTile = 8;  // tiles are 8 x 8 x (4 zsteps) cells: 256 threads cover 8 x 8 x 4 cells per step
// projection tile = 8 x 8 x (4 zsteps) cells; zsteps from the autotuner when it divides the grid
__host__ __device__ inline int tile_zsteps(const DevCfg &c)
{
  if (c.proj_zsteps >= 1 && c.proj_zsteps <= 4 && c.n % (4 * c.proj_zsteps) == 0) return c.proj_zsteps;
  return c.n % 16 == 0 ? 4 : 2;
}
constexpr int kQueueCap = 1024;
constexpr int kEdgesSmem = 516;
#ifndef PROJ_UNROLL
#define PROJ_UNROLL 2
#endif
constexpr int kProjUnroll = PROJ_UNROLL;  // sub-samples per loop iteration

// one run of a cell's sub-samples into the map: an L2 reduction whose result is not returned
__device__ __forceinline__ void map_add(float *maps, uint32_t key, float val) { atomicAdd(&maps[key], val); }

// one uncertain sample: tile, (local cell << 4 | sub-sample), mass/10, dz
struct FallbackEntry {
  uint32_t tile, sub;
  float msub, dz;
};

template <bool FUSED>
__global__ void __launch_bounds__(kProjThreads, 4) project_kernel(DevCfg c, FastConst f, const double *__restrict__ stats,
                                                               const float *__restrict__ a, const float *__restrict__ b,
                                                               float *__restrict__ maps, int *__restrict__ counters,
                                                               FallbackEntry *__restrict__ fq, long fq_cap)
{
  __shared__ uint32_t q_cell[kQueueCap];
  __shared__ float q_val[kQueueCap], q_dz[kQueueCap];
  __shared__ uint8_t q_sub[kQueueCap];
  __shared__ float sef[kEdgesSmem];
  __shared__ int q_n;
  const int tid = threadIdx.x;
  const bool smem_edges = !c.regular_nu && c.n_nu < kEdgesSmem;
  if (smem_edges)
    for (int i = tid; i <= c.n_nu; i += kProjThreads) sef[i] = c.nu_edges_f[i];
  if (tid == 0) q_n = 0;
  __syncthreads();
  const float *ef = smem_edges ? sef : c.nu_edges_f;
  int log2nn = 0;
  while ((1 << (log2nn + 1)) - 2 < c.n_nu) log2nn++;  // steps 2^L..1 from -1 reach index n_nu
  const int n = c.n, nt = n / kTile, zsteps = tile_zsteps(c);
  const int bx = blockIdx.x % nt, by = (blockIdx.x / nt) % nt, bz = blockIdx.x / (nt * nt);
  const float sigma2 = FUSED ? (float)stats[1] : 0.f;
  int nfall = 0;
  // all of this thread's cells are loaded up front (up to 4 load pairs in flight)
  const int ix = bx * kTile + (tid & 7), iy = by * kTile + ((tid >> 3) & 7), iz0 = bz * 4 * zsteps + (tid >> 6);
  float va[4], vb[4];
#pragma unroll
  for (int k = 0; k < 4; k++) {
    const long i = ((long)(iz0 + 4 * k) * n + iy) * n + ix;
    va[k] = k < zsteps ? a[i] : 0.f;
    vb[k] = k < zsteps ? b[i] : 0.f;
  }
#pragma unroll 1
  for (int k = 0; k < zsteps; k++) {
    const int iz = iz0 + 4 * k;
    const float ak = k == 0 ? va[0] : k == 1 ? va[1] : k == 2 ? va[2] : va[3];
    const float bk = k == 0 ? vb[0] : k == 1 ? vb[1] : k == 2 ? vb[2] : vb[3];
    float mass, dz;
    if (FUSED) {
      CellHI h = cell_hi(c, sigma2, ix, iy, iz, ak, bk);
      mass = h.mass;
      dz = h.dz;
    } else {
      mass = ak;
      dz = bk;
    }
    const float msub = mass / 10.f;  // src/pixelize.c:203
    const float Xc = (float)ix - f.half_n, Yc = (float)iy - f.half_n, Zc = (float)iz - f.half_n;
    const CellShell cs = cell_shell(c, f, ef, log2nn, Xc, Yc, Zc, dz);
    if (cell_outside(c, f, ef, cs)) continue;  // inside the first shell or beyond the last: no keys
    const CellPix cp = cell_pix(c, f, Xc + 0.5f, Yc + 0.5f, Zc + 0.5f, cs.Rc);
    uint32_t cur = 0xFFFFFFFFu, umask = 0;
    float acc = 0.f;
    // a key inside the shells extends the run of cur or ends it (one reduction);
    // written without branches: the reduction is the only predicated step
    auto take = [&](uint32_t key, int j) {
      umask |= (key == kKeyUncertain ? 1u : 0u) << j;
      const bool valid = key < kKeyUncertain;
      const bool flush = valid & (key != cur) & (cur != 0xFFFFFFFFu);
      if (flush) map_add(maps, cur, acc);
      acc = valid ? (key == cur ? acc + msub : msub) : acc;
      cur = valid ? key : cur;
    };
    if (cp.lin) {
#pragma unroll
      for (int j = 0; j < kNSUB; j++) take(key_lin(c, f, ef, log2nn, cs, cp, j), j);
    } else {
#pragma unroll kProjUnroll
      for (int j = 0; j < kNSUB; j++)
        take(key_fast(c, ef, log2nn, cs, Xc + f.txsp[j], Yc + f.tysp[j], Zc + f.tzsp[j]), j);
    }
    if (cur != 0xFFFFFFFFu) map_add(maps, cur, acc);
    // uncertain samples of the cell: to the tile queue (when it is full, decided here)
#pragma unroll 1
    while (umask) {
      const int is = f.tour[__ffs(umask) - 1];
      umask &= umask - 1;
      nfall++;
      const int slot = atomicAdd(&q_n, 1);
      if (slot < kQueueCap) {
        q_cell[slot] = (uint32_t)(tid + kProjThreads * k);
        q_sub[slot] = (uint8_t)is;
        q_val[slot] = msub;
        q_dz[slot] = dz;
      } else {
        const uint32_t ke = key_exact(c, ix, iy, iz, is, dz);
        if (ke != 0xFFFFFFFFu) map_add(maps, ke, msub);
      }
    }
  }
  __syncthreads();
  // hand the uncertain samples to the global queue (resolved by fixup_kernel on
  // full warps); whatever does not fit is resolved here
  __shared__ long q_base;
  const int qn = min(q_n, kQueueCap);
  if (tid == 0) q_base = qn ? (long)atomicAdd((unsigned long long *)&counters[2], (unsigned long long)qn) : 0;
  __syncthreads();
  for (int j = tid; j < qn; j += kProjThreads) {
    const long g = q_base + j;
    if (g < fq_cap) {
      FallbackEntry e;
      e.tile = blockIdx.x;
      e.sub = (q_cell[j] << 4) | q_sub[j];
      e.msub = q_val[j];
      e.dz = q_dz[j];
      fq[g] = e;
      continue;
    }
    const int lc = (int)q_cell[j], k = lc / kProjThreads, t = lc % kProjThreads;
    const int ix = bx * kTile + (t & 7), iy = by * kTile + ((t >> 3) & 7), iz = bz * 4 * zsteps + (t >> 6) + 4 * k;
    const uint32_t key = key_exact(c, ix, iy, iz, q_sub[j], q_dz[j]);  // global queue full (rare)
    if (key != 0xFFFFFFFFu) map_add(maps, key, q_val[j]);
  }
  if (counters) {
    for (int o = 16; o > 0; o >>= 1) nfall += __shfl_xor_sync(0xffffffffu, nfall, o);
    if ((tid & 31) == 0 && nfall) atomicAdd(&counters[0], nfall);
  }
}

// FP64 keys of the queued uncertain samples (full warps on the FP64 pipe)
__global__ void fixup_kernel(DevCfg c, const FallbackEntry *__restrict__ fq, const int *__restrict__ counters,
                             long fq_cap, float *__restrict__ maps)
{
  const long cnt = min((long)*reinterpret_cast<const unsigned long long *>(&counters[2]), fq_cap);
  const int nt = c.n / kTile, zsteps = tile_zsteps(c);
  for (long j = blockIdx.x * (long)blockDim.x + threadIdx.x; j < cnt; j += (long)gridDim.x * blockDim.x) {
    const FallbackEntry e = fq[j];
    const int bx = e.tile % nt, by = (e.tile / nt) % nt, bz = e.tile / (nt * nt);
    const int lc = (int)(e.sub >> 4), is = (int)(e.sub & 15), k = lc / kProjThreads, t = lc % kProjThreads;
    const int ix = bx * kTile + (t & 7), iy = by * kTile + ((t >> 3) & 7), iz = bz * 4 * zsteps + (t >> 6) + 4 * k;
    const uint32_t key = key_resolve(c, ix, iy, iz, is, e.dz);
    if (key != 0xFFFFFFFFu) atomicAdd(&maps[key], e.msub);
  }
}

// maps *= M2T / (r(nu_c)^2 dnu) per channel, src/pixelize.c:246-261
// blockIdx.y = channel; VEC: four pixels per thread (npix = 12 nside^2 is a multiple
// of 4; maps 16-byte aligned), else one
template <bool VEC>
__global__ void scale_maps_kernel(DevCfg c, float *maps)
{
  const long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  const float f = __ldg(&c.prefac[blockIdx.y]);
  float *mc = maps + (long)blockIdx.y * c.npix;
  if (VEC) {
    if (i >= c.npix / 4) return;
    float4 *m = reinterpret_cast<float4 *>(mc) + i;
    float4 v = *m;
    v.x *= f;
    v.y *= f;
    v.z *= f;
    v.w *= f;
    *m = v;
  } else if (i < c.npix) {
    mc[i] *= f;
  }
}

// per-sample keys (validation): exact FP64, or fast FP32 with FP64 fallback
__global__ void sample_keys_kernel(DevCfg c, FastConst f, const float *__restrict__ dzg, uint32_t *keys, int exact,
                                   int *counters)
{
  const int n = c.n;
  const long total = (long)n * n * n;
  int nfall = 0;
  int log2nn = 0;
  while ((1 << (log2nn + 1)) - 2 < c.n_nu) log2nn++;  // steps 2^L..1 from -1 reach index n_nu
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < total; i += (long)gridDim.x * blockDim.x) {
    const int ix = (int)(i % n);
    const long rest = i / n;
    const int iy = (int)(rest % n), iz = (int)(rest / n);
    const float dz = dzg[i];
    const float Xc = (float)ix - f.half_n, Yc = (float)iy - f.half_n, Zc = (float)iz - f.half_n;
    const CellShell cs = cell_shell(c, f, c.nu_edges_f, log2nn, Xc, Yc, Zc, dz);
    if (!exact && cell_outside(c, f, c.nu_edges_f, cs)) {
      for (int is = 0; is < kNSUB; is++) keys[i * kNSUB + is] = kKeyInvalid;
      continue;
    }
    const CellPix cp = cell_pix(c, f, Xc + 0.5f, Yc + 0.5f, Zc + 0.5f, cs.Rc);
    for (int j = 0; j < kNSUB; j++) {
      const int is = f.tour[j];
      uint32_t key = kKeyUncertain;
      if (!exact)
        key = cp.lin ? key_lin(c, f, c.nu_edges_f, log2nn, cs, cp, j)
                     : key_fast(c, c.nu_edges_f, log2nn, cs, Xc + f.txsp[j], Yc + f.tysp[j], Zc + f.tzsp[j]);
      if (key == kKeyUncertain) {
        key = exact ? key_exact(c, ix, iy, iz, is, dz) : key_resolve(c, ix, iy, iz, is, dz);
        nfall++;
      }
      keys[i * kNSUB + is] = key;
    }
  }
  if (counters) atomicAdd(&counters[1], nfall);
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

double subsample_radius(const double *xs, const double *ys, const double *zs, double dx)
{
  double r = 0;
  for (int i = 0; i < kNSUB; i++) r = std::fmax(r, std::sqrt(xs[i] * xs[i] + ys[i] * ys[i] + zs[i] * zs[i]) / dx);
  return r;
}

// Interval i of the table spans R in [a, a + h) cells (h = 1/(glob_idr dx); the
// nodes sit at r = k/glob_idr).  Its line is z_i + g (R - a).  A cell whose FP32
// centre falls in interval i has its sub-samples within rho of the centre and
// the centre within eps of the interval, so the deviation bound e is the
// largest |z(R) - line| over R in [a - rho - eps, a + h + rho + eps]: z is
// piecewise linear, so the largest value sits at a node or at an end.
float2 shell_line_entry(const double *z, double glob_idr, double dx, double rho, int i)
{
  if (i < 0 || i + 1 >= kNZ) return make_float2(0.f, 0.f);
  const double h = 1.0 / (glob_idr * dx), a = i * h, b = a + h, top = (kNZ - 1) * h;
  const double g = (z[i + 1] - z[i]) * glob_idr * dx;
  const double eps = 1e-3 + 1e-6 * b;  // FP32 centre radius and interval index
  const double lo = std::fmax(0.0, a - rho - eps), hi = std::fmin(top, b + rho + eps);
  auto line_dev = [&](double R) {
    const int k = std::min((int)(R / h), kNZ - 2);
    return std::fabs(z[k] + (z[k + 1] - z[k]) * (R / h - k) - z[i] - g * (R - a));
  };
  double e = std::fmax(line_dev(lo), line_dev(hi));
  for (int k = (int)(lo / h) + 1; k < kNZ && k * h < hi; k++) e = std::fmax(e, std::fabs(z[k] - z[i] - g * (k * h - a)));
  return make_float2((float)g, (float)(e * (1 + 1e-5) + 1e-12));
}

static FastConst fast_const(const DevCfg &c)
{
  FastConst f;
  for (int i = 0; i < kNSUB; i++) {
    f.xsp[i] = (float)(0.5 + c.xs[i] / c.dx);
    f.ysp[i] = (float)(0.5 + c.ys[i] / c.dx);
    f.zsp[i] = (float)(0.5 + c.zs[i] / c.dx);
  }
  f.idr_cell = (float)(c.glob_idr * c.dx);
  f.rho = (float)(subsample_radius(c.xs, c.ys, c.zs, c.dx) * (1 + 1e-5) + 1e-6);
  f.rho_idr = f.rho * f.idr_cell * 1.0001f;
  f.half_n = (float)(c.n / 2);
  f.nu_min = (float)c.nu_min;
  f.inv_dnu = (float)c.inv_dnu;
  // shortest open path through the 10 offsets: nearest-neighbour tours from every
  // start, each improved by 2-opt reversals, the shortest kept
  auto dist = [&](int a, int b) {
    const double dx = c.xs[a] - c.xs[b], dy = c.ys[a] - c.ys[b], dz = c.zs[a] - c.zs[b];
    return std::sqrt(dx * dx + dy * dy + dz * dz);
  };
  auto length = [&](const int *o) {
    double l = 0;
    for (int i = 0; i + 1 < kNSUB; i++) l += dist(o[i], o[i + 1]);
    return l;
  };
  double best = 1e300;
  for (int start = 0; start < kNSUB; start++) {
    int o[kNSUB];
    bool used[kNSUB] = {};
    o[0] = start;
    used[start] = true;
    for (int i = 1; i < kNSUB; i++) {
      int nx = -1;
      for (int j = 0; j < kNSUB; j++)
        if (!used[j] && (nx < 0 || dist(o[i - 1], j) < dist(o[i - 1], nx))) nx = j;
      o[i] = nx;
      used[nx] = true;
    }
    for (bool improved = true; improved;) {
      improved = false;
      for (int i = 1; i + 1 < kNSUB; i++)
        for (int j = i + 1; j < kNSUB; j++) {
          int t[kNSUB];
          for (int k = 0; k < kNSUB; k++) t[k] = (k >= i && k <= j) ? o[i + j - k] : o[k];
          if (length(t) < length(o) - 1e-12) {
            for (int k = 0; k < kNSUB; k++) o[k] = t[k];
            improved = true;
          }
        }
    }
    if (length(o) < best) {
      best = length(o);
      for (int k = 0; k < kNSUB; k++) f.tour[k] = o[k];
    }
  }
  for (int k = 0; k < kNSUB; k++) {
    f.txsp[k] = f.xsp[f.tour[k]];
    f.tysp[k] = f.ysp[f.tour[k]];
    f.tzsp[k] = f.zsp[f.tour[k]];
    // within 4.5e-8 cells of xs/dx: xsp rounds once, the subtraction at most once more
    const float ox = f.txsp[k] - 0.5f, oy = f.tysp[k] - 0.5f, oz = f.tzsp[k] - 0.5f;
    f.tox[k] = ox;
    f.toy[k] = oy;
    f.toz[k] = oz;
    f.toxx[k] = ox * ox;
    f.toyy[k] = oy * oy;
    f.tozz[k] = oz * oz;
    f.toxy[k] = ox * oy;
    f.toxz[k] = ox * oz;
    f.toyz[k] = oy * oz;
    f.tdxy[k] = ox * ox - oy * oy;
  }
  return f;
}

long fallback_queue_capacity(int n)
{
  long cap = (long)n * n * n * kNSUB / 128;
  return cap < (1L << 20) ? (1L << 20) : cap;
}
size_t fallback_entry_bytes() { return sizeof(FallbackEntry); }

cudaError_t project(const DevCfg &c, const double *stats, const float *a, const float *b, int fused, float *maps,
                    int *counters, void *fq, long fq_cap, cudaStream_t st)
{
  const int tz = 4 * tile_zsteps(c);
  if (c.n % kTile || c.n % tz) return cudaErrorInvalidValue;
  const long nt = c.n / kTile;
  const unsigned blocks = (unsigned)(nt * nt * (c.n / tz));
  FastConst f = fast_const(c);
  FallbackEntry *q = reinterpret_cast<FallbackEntry *>(fq);
  if (fused) project_kernel<true><<<blocks, kProjThreads, 0, st>>>(c, f, stats, a, b, maps, counters, q, fq_cap);
  else project_kernel<false><<<blocks, kProjThreads, 0, st>>>(c, f, stats, a, b, maps, counters, q, fq_cap);
  return cudaGetLastError();
}

cudaError_t fixup(const DevCfg &c, const void *fq, const int *counters, long fq_cap, float *maps, cudaStream_t st)
{
  fixup_kernel<<<152 * 8, 256, 0, st>>>(c, reinterpret_cast<const FallbackEntry *>(fq), counters, fq_cap, maps);
  return cudaGetLastError();
}

cudaError_t scale_maps(const DevCfg &c, float *maps, cudaStream_t st)
{
  if ((reinterpret_cast<uintptr_t>(maps) & 15) == 0)
    scale_maps_kernel<true><<<dim3((unsigned)((c.npix / 4 + 255) / 256), c.n_nu), 256, 0, st>>>(c, maps);
  else
    scale_maps_kernel<false><<<dim3((unsigned)((c.npix + 255) / 256), c.n_nu), 256, 0, st>>>(c, maps);
  return cudaGetLastError();
}

cudaError_t sample_keys(const DevCfg &c, const float *dz, uint32_t *keys, int exact, int *counters, cudaStream_t st)
{
  long total = (long)c.n * c.n * c.n;
  sample_keys_kernel<<<grid_for(total, 128), 128, 0, st>>>(c, fast_const(c), dz, keys, exact, counters);
  return cudaGetLastError();
}


// ---------------------------------------------------------------------------
// point sources: get_point_sources (src/grid_tools.c:24-101) and
// mk_psources_maps (src/pixelize.c:58-148) fused, one thread per cell.
// Counter-based draws: Philox4x32-10 with key (seed, 0x50535243) and counter
// (cell lo, cell hi, stream, block): stream 0 feeds the Poisson count, stream
// 1 + s the position (3 uniforms) and luminosity (1 uniform) of source s.
// Each source adds L0 (1+z)^-1.1 / r^2 and 10 L0 (1+z)^-1.75 / r^2 to its pixel's
// two sums, from which every channel follows (ps_expand_kernel).
// ---------------------------------------------------------------------------
__device__ __forceinline__ float u01(uint32_t w) { return ((float)(w >> 8) + 0.5f) * (1.f / 16777216.f); }

// n_of_z_psources (src/psources.c:74-90)
__device__ __forceinline__ float ps_n_of_z(const PsConst &p, float z)
{
  const float t = z * p.inv_dz;
  if (!(t > -1.f) || t >= (float)kPsNZ) return -1.f;  // (int) truncation: iz in [0, 256)
  const int iz = (int)t;
  if (iz == kPsNZ - 1) return __ldg(&p.nz[kPsNZ - 1]);
  const float a = __ldg(&p.nz[iz]), b = __ldg(&p.nz[iz + 1]);
  return a + (b - a) * (t - (float)iz);
}

// table value at r (Mpc/h) by linear interpolation in r (src/cosmo.c:52-86)
__device__ __forceinline__ float table_at_r(const DevCfg &c, const float *tab, float r)
{
  const float tr = fminf(fmaxf(r * c.glob_idr_f, 0.f), (float)(kNZ - 2));
  const int ir = (int)tr;
  const float a = __ldg(&tab[ir]), b = __ldg(&tab[ir + 1]);
  return a + (b - a) * (tr - (float)ir);
}

// Poisson count: Knuth's multiplication method below 12, else the transformed
// rejection PTRS of Hormann (1993, Insurance: Math. Econ. 12, 39)
__device__ int ps_poisson(uint32_t lo, uint32_t hi, uint32_t seed, float lam)
{
  const uint2 key = make_uint2(seed, kPsKey);
  if (lam < 12.f) {
    const float emu = expf(-lam);
    float prod = 1.f;
    int k = 0;
#pragma unroll 1
    for (uint32_t j = 0; j < 64; j++) {
      const uint4 w = philox4x32_10(make_uint4(lo, hi, 0u, j), key);
      const uint32_t ws[4] = {w.x, w.y, w.z, w.w};
#pragma unroll
      for (int q = 0; q < 4; q++) {
        prod *= u01(ws[q]);
        k++;
        if (prod <= emu) return k - 1;
      }
    }
    return k;
  }
  const double mu = lam, smu = sqrt(mu), b = 0.931 + 2.53 * smu, a = -0.059 + 0.02483 * b;
  const double inv_alpha = 1.1239 + 1.1328 / (b - 3.4), vr = 0.9277 - 3.6224 / (b - 2);
  const double lmu = log(mu);
#pragma unroll 1
  for (uint32_t j = 0; j < 256; j++) {
    const uint4 w = philox4x32_10(make_uint4(lo, hi, 0u, j), key);
    const uint32_t ws[4] = {w.x, w.y, w.z, w.w};
#pragma unroll
    for (int q = 0; q < 4; q += 2) {
      const double U = (double)u01(ws[q]) - 0.5, V = (double)u01(ws[q + 1]);
      const double us = 0.5 - fabs(U);
      const double kd = floor((2 * a / us + b) * U + mu + 0.43);
      if (us >= 0.07 && V <= vr) return (int)kd;
      if (kd < 0 || (us < 0.013 && V > us)) continue;
      if (log(V) + log(inv_alpha) - log(a / (us * us) + b) <= -mu + kd * lmu - lgamma(kd + 1)) return (int)kd;
    }
  }
  return (int)rint(mu);
}

// RING pixel of a source at (dx ix - pos_obs) + dx u, FP64 with the reference's
// rounding (src/pixelize.c:112-121)
__device__ __noinline__ uint32_t ps_pixel_exact(const DevCfg &c, int ix, int iy, int iz, float ux, float uy, float uz)
{
  const double x = __dadd_rn(__dsub_rn(__dmul_rn(c.dx, (double)ix), c.pos_obs), __dmul_rn(c.dx, (double)ux));
  const double y = __dadd_rn(__dsub_rn(__dmul_rn(c.dx, (double)iy), c.pos_obs), __dmul_rn(c.dx, (double)uy));
  const double z = __dadd_rn(__dsub_rn(__dmul_rn(c.dx, (double)iz), c.pos_obs), __dmul_rn(c.dx, (double)uz));
  const double xy2 = __dadd_rn(__dmul_rn(x, x), __dmul_rn(y, y));
  const double r = __dsqrt_rn(__dadd_rn(xy2, __dmul_rn(z, z)));
  const double cth = __ddiv_rn(z, r);
  const double sth = fabs(cth) > 0.99 ? __ddiv_rn(__dsqrt_rn(xy2), r) : -5.0;
  return (uint32_t)loc2pix_exact(c.nside, cth, sth, atan2(y, x));
}

__global__ void __launch_bounds__(256) psources_kernel(DevCfg c, PsConst p, const double *__restrict__ stats,
                                                       const float *__restrict__ dens,
                                                       const float *__restrict__ vr, float *__restrict__ acc,
                                                       unsigned long long *__restrict__ total, PsCatalogue cat)
{
  const int n = c.n;
  const long ncell = (long)n * n * n;
  const float sigma2 = (float)stats[1];
  const float half_n = 0.5f * (float)n;
  unsigned long long count = 0;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < ncell; i += (long)gridDim.x * blockDim.x) {
    const int ix = (int)(i % n), iy = (int)((i / n) % n), iz = (int)(i / ((long)n * n));
    // Poisson mean at the cell centre (src/grid_tools.c:67-84)
    const float xc = c.dxf * (ix + 0.5f) - c.pos_obsf, yc = c.dxf * (iy + 0.5f) - c.pos_obsf,
                zc = c.dxf * (iz + 0.5f) - c.pos_obsf;
    const float rc = sqrtf(xc * xc + yc * yc + zc * zc);
    const float ndens = ps_n_of_z(p, table_at_r(c, c.z_r2z_f, rc));
    if (!(ndens > 0.f)) continue;
    const float gfb = table_at_r(c, c.gd_f, rc);  // bias_psources = 1 (src/psources.c:65-68)
    const float delta = dens[i];
    const float lam = ndens * p.cell_vol * expf(gfb * (delta - 0.5f * gfb * sigma2));
    const int np = ps_poisson((uint32_t)i, (uint32_t)(i >> 32), c.seed, lam);
    if (np <= 0) continue;
    count += (unsigned long long)np;
    const float dz = cell_hi(c, sigma2, ix, iy, iz, delta, vr[i]).dz;  // dz_rsd of the cell
    for (int s = 0; s < np; s++) {
      const uint4 w = philox4x32_10(make_uint4((uint32_t)i, (uint32_t)(i >> 32), 1u + (uint32_t)s, 0u),
                                    make_uint2(c.seed, kPsKey));
      const float ux = u01(w.x), uy = u01(w.y), uz = u01(w.z), uL = u01(w.w);
      const float X = ((float)ix - half_n) + ux, Y = ((float)iy - half_n) + uy, Z = ((float)iz - half_n) + uz;
      const float rho2 = fmaf(Y, Y, X * X), R2 = fmaf(Z, Z, rho2), iR = rsqrtf(R2);
      const float r = R2 * iR * c.dxf;
      const float zcos = table_at_r(c, c.z_r2z_f, r);
      if (zcos >= p.z_max) continue;  // draw_luminosity returns 0 (src/psources.c:130)
      uint32_t pix = rho2 > 0.f ? pixel_fast(c, X, Y, Z, rho2, iR) : kKeyUncertain;
      if (pix == kKeyUncertain) pix = ps_pixel_exact(c, ix, iy, iz, ux, uy, uz);
      const float t = uL * (float)p.nicdf;
      const int j = min((int)t, p.nicdf - 1);
      const float l0 = __ldg(&p.icdf[j]), l1 = __ldg(&p.icdf[j + 1]);
      const float L = exp10f(l0 + (l1 - l0) * (t - (float)j));
      const float opz = 1.f + zcos + dz;
      const float wgt = L / (r * r * opz);
      atomicAdd(&acc[pix], wgt * exp2f(-0.1f * log2f(opz)));
      atomicAdd(&acc[c.npix + pix], 10.f * wgt * exp2f(-0.75f * log2f(opz)));
      if (cat.count) {
        const unsigned long long k = atomicAdd(cat.count, 1ull);
        if (k < (unsigned long long)cat.cap) {
          cat.cell[k] = i;
          cat.u[k] = make_float4(ux, uy, uz, L);
          cat.dz[k] = dz;
          cat.pix[k] = (int)pix;
        }
      }
    }
  }
  for (int o = 16; o > 0; o >>= 1) count += __shfl_xor_sync(0xffffffffu, count, o);
  if ((threadIdx.x & 31) == 0 && count) atomicAdd(total, count);
}

// maps_ps[inu][pix] = a[inu] S1[pix] + b[inu] S2[pix]
__global__ void ps_expand_kernel(DevCfg c, const float *__restrict__ acc, const float *__restrict__ chan,
                                 float *__restrict__ maps_ps)
{
  const long npix = c.npix, total = npix * c.n_nu;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < total; i += (long)gridDim.x * blockDim.x) {
    const long inu = i / npix, pix = i - inu * npix;
    maps_ps[i] = __ldg(&chan[2 * inu]) * acc[pix] + __ldg(&chan[2 * inu + 1]) * acc[npix + pix];
  }
}

cudaError_t psources(const DevCfg &c, const PsConst &p, const double *stats, const float *dens, const float *vr,
                     float *acc, float *maps_ps, const float *chan, unsigned long long *total, const PsCatalogue &cat,
                     cudaStream_t st)
{
  cudaError_t e = cudaMemsetAsync(acc, 0, sizeof(float) * 2 * c.npix, st);
  if (e != cudaSuccess) return e;
  psources_kernel<<<152 * 16, 256, 0, st>>>(c, p, stats, dens, vr, acc, total, cat);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  ps_expand_kernel<<<152 * 16, 256, 0, st>>>(c, acc, chan, maps_ps);
  return cudaGetLastError();
}

}  // namespace gethi
