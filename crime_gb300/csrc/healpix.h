// HEALPix RING <-> NESTED pixel numbering and the RING-scheme ring geometry,
// from the definitions of Gorski et al. 2005 (ApJ 622:759, sections 4-5),
// for nside <= 8192.  Host and device: the JoinT ud_grade kernels and the
// host-side FITS reader (NESTED files) share it.
#pragma once
#include <cmath>
#include <cstdint>

#ifdef __CUDACC__
#define HPX_HD __host__ __device__ __forceinline__
#else
#define HPX_HD inline
#endif

namespace gethi {
namespace hpx {

HPX_HD uint32_t spread_bits(uint32_t x)  // bit b -> bit 2b, 16 bits in
{
  x &= 0xFFFFu;
  x = (x | (x << 8)) & 0x00FF00FFu;
  x = (x | (x << 4)) & 0x0F0F0F0Fu;
  x = (x | (x << 2)) & 0x33333333u;
  x = (x | (x << 1)) & 0x55555555u;
  return x;
}
HPX_HD uint32_t compress_bits(uint32_t x)  // bit 2b -> bit b
{
  x &= 0x55555555u;
  x = (x | (x >> 1)) & 0x33333333u;
  x = (x | (x >> 2)) & 0x0F0F0F0Fu;
  x = (x | (x >> 4)) & 0x00FF00FFu;
  x = (x | (x >> 8)) & 0x0000FFFFu;
  return x;
}
HPX_HD long long isqrt(long long v)  // floor(sqrt(v)), v < 2^31
{
  long long r = (long long)sqrtf((float)v);
  while (r * r > v) r--;
  while ((r + 1) * (r + 1) <= v) r++;
  return r;
}
// ring row of each base pixel's centre (in units of nside) and its longitude offset
HPX_HD int face_row(int f) { return 2 + (f >> 2); }
HPX_HD int face_lon(int f) { return (f < 4 || f >= 8) ? 2 * (f & 3) + 1 : 2 * (f & 3); }

HPX_HD long long nest2ring(long long nside, long long ipnest)
{
  const long long npface = nside * nside, npix = 12 * npface, ncap = 2 * nside * (nside - 1);
  const int face = (int)(ipnest / npface);
  const uint32_t ipf = (uint32_t)(ipnest % npface);
  const long long ix = compress_bits(ipf), iy = compress_bits(ipf >> 1);
  const long long jr = face_row(face) * nside - (ix + iy) - 1;  // ring number, 1-based
  long long nr, first, shift;
  if (jr < nside) {
    nr = jr;
    first = 2 * nr * (nr - 1);
    shift = 0;
  } else if (jr > 3 * nside) {
    nr = 4 * nside - jr;
    first = npix - 2 * (nr + 1) * nr;
    shift = 0;
  } else {
    nr = nside;
    first = ncap + (jr - nside) * 4 * nside;
    shift = (jr - nside) & 1;
  }
  long long jp = (face_lon(face) * nr + (ix - iy) + 1 + shift) / 2;
  if (jp > 4 * nr) jp -= 4 * nr;
  if (jp < 1) jp += 4 * nr;
  return first + jp - 1;
}

HPX_HD long long ring2nest(long long nside, long long ipring)
{
  const long long npface = nside * nside, npix = 12 * npface, ncap = 2 * nside * (nside - 1);
  long long iring, iphi, shift, nr;
  int face;
  if (ipring < ncap) {
    iring = (1 + isqrt(1 + 2 * ipring)) >> 1;
    iphi = ipring + 1 - 2 * iring * (iring - 1);
    shift = 0;
    nr = iring;
    face = (int)((iphi - 1) / nr);
  } else if (ipring < npix - ncap) {
    const long long ip = ipring - ncap, t = ip / (4 * nside);
    iring = t + nside;
    iphi = ip - t * 4 * nside + 1;
    shift = (iring + nside) & 1;
    nr = nside;
    const long long ire = t + 1, irm = 2 * nside + 2 - ire;
    const long long fm = (iphi - ire / 2 + nside - 1) / nside, fp = (iphi - irm / 2 + nside - 1) / nside;
    face = (int)((fp == fm) ? (fp | 4) : (fp < fm ? fp : fm + 8));
  } else {
    const long long ip = npix - ipring;
    iring = (1 + isqrt(2 * ip - 1)) >> 1;
    iphi = 4 * iring + 1 - (ip - 2 * iring * (iring - 1));
    shift = 0;
    nr = iring;
    iring = 4 * nside - iring;
    face = 8 + (int)((iphi - 1) / nr);
  }
  const long long irt = iring - face_row(face) * nside + 1;
  long long ipt = 2 * iphi - face_lon(face) * nr - shift - 1;
  if (ipt >= 2 * nside) ipt -= 8 * nside;
  const long long ix = (ipt - irt) >> 1, iy = (-(ipt + irt)) >> 1;
  return face * npface + spread_bits((uint32_t)ix) + 2 * (long long)spread_bits((uint32_t)iy);
}

}  // namespace hpx
}  // namespace gethi
