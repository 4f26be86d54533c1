// Mode draw shared by the FP32 and tensor-core column passes: P(k) lookup,
// Philox4x32-10 production draws, uploaded spectra, and the phi = delta f0 H0/k^2
// factor of the velocity potential.
#pragma once
#include "common.cuh"
#include "fft.h"

namespace gethi {

// ---------------------------------------------------------------------------
// Fourier modes
// ---------------------------------------------------------------------------
__device__ __forceinline__ float pk_lookup(const DevCfg &c, float lgk)  // src/cosmo.c:153-170
{
  int ik = (int)floorf((lgk - c.logkmin) * c.idlogk);
  if (lgk - c.logkmin < 0) ik = -1;
  if (ik < 0) return __ldg(&c.pk_f[0]) * exp10f(c.n_scal * (lgk - c.logkmin));
  if (ik < c.numk - 1) {
    float p0 = __ldg(&c.pk_f[ik]), p1 = __ldg(&c.pk_f[ik + 1]);
    return p0 + (lgk - __ldg(&c.logk_f[ik])) * (p1 - p0) * c.idlogk;
  }
  return __ldg(&c.pk_f[c.numk - 1]) * exp10f(-3.f * (lgk - c.logkmax));
}

// Production draw: amplitude law of src/fourier.c:292-298 with Philox4x32-10.
// One Philox call serves the modes kz and kz + N/2 (same ky, kx):
// ctr = (id lo, id hi, 0, 0) with id = kx + (N/2+1)(ky + N (kz mod N/2)),
// key = (seed, 0x4352494D); the lower mode uses words (x, y), the upper (z, w).
// Phase = 2 pi word0/2^32; modulus from ln(1 - word1/2^32).
__device__ __forceinline__ uint4 philox_for_pair(const DevCfg &c, int ii0, int jj, int kk)
{
  uint64_t id = (uint64_t)kk + (uint64_t)(c.m + 1) * ((uint64_t)jj + (uint64_t)c.n * ii0);
  return philox4x32_10(make_uint4((uint32_t)id, (uint32_t)(id >> 32), 0u, 0u), make_uint2(c.seed, 0x4352494Du));
}

__device__ __forceinline__ float2 mode_from_words(const DevCfg &c, int ii, int jj, int kk, uint32_t wph, uint32_t wmod)
{
  const int n = c.n;
  float kz = kval(ii, n, c.dk), ky = kval(jj, n, c.dk), kx = kval(kk, n, c.dk);
  float k2 = kx * kx + ky * ky + kz * kz;
  if (k2 <= 0.f) return make_float2(0.f, 0.f);
  float sigma2;
  if (c.pg) {
    sigma2 = fmaxf(__ldg(&c.pg[((size_t)ii * n + jj) * n + kk]), 0.f) * c.idk3;
  } else {
    float lgk = 0.5f * log10f(k2);
    sigma2 = pk_lookup(c, lgk) * c.idk3;
    if (c.do_smoothing) sigma2 *= expf(-c.r2_smooth * k2);
  }
  float u = (float)wph * 2.3283064365386963e-10f;
  // ln(1 - u2): log1p keeps the relative accuracy for small u2, the direct log of
  // the exact remainder 2^32 - word for u2 >= 1/2
  float lnw = wmod < 0x80000000u ? log1pf(-(float)wmod * 2.3283064365386963e-10f)
                                 : logf((float)(0u - wmod) * 2.3283064365386963e-10f);
  float amp = sqrtf(-sigma2 * lnw);
  float s, co;
  sincospif(2.f * u, &s, &co);
  return make_float2(amp * co, amp * s);
}

// delta_k of mode (kz index ii, ky index jj, kx index kk); src != nullptr: a
// host spectrum in the reference layout [kz][ky][N/2+1]
__device__ __forceinline__ float2 mode_value(const DevCfg &c, int ii, int jj, int kk, int kind,
                                             const float2 *__restrict__ src)
{
  (void)kind;
  const int n = c.n;
  if (src) {
    float kz = kval(ii, n, c.dk), ky = kval(jj, n, c.dk), kx = kval(kk, n, c.dk);
    if (kx * kx + ky * ky + kz * kz <= 0.f) return make_float2(0.f, 0.f);
    return __ldg(&src[((size_t)ii * n + jj) * (size_t)(c.m + 1) + kk]);
  }
  const int half = 2 * ii >= n ? 1 : 0;
  const uint4 o = philox_for_pair(c, ii - half * (n / 2), jj, kk);
  return half ? mode_from_words(c, ii, jj, kk, o.z, o.w) : mode_from_words(c, ii, jj, kk, o.x, o.y);
}

__device__ __forceinline__ float vfac_over_k2(const DevCfg &c, int ii, int jj, int kk)
{
  const int n = c.n;
  float kz = kval(ii, n, c.dk), ky = kval(jj, n, c.dk), kx = kval(kk, n, c.dk);
  float k2 = kx * kx + ky * ky + kz * kz;
  return k2 > 0.f ? __fdividef(c.vfac, k2) : 0.f;  // phi_k = delta_k f0 H0 / k^2, src/fourier.c:298
}

}  // namespace gethi
