// JoinT on the GPU: merge + ud_grade, Gaussian beam through a HEALPix spherical
// harmonic transform, white noise, mask (src/main_jt.c:98-372,
// src/healpix_extra.c:31-130, 318-421).
//
// Data layout in HBM (nside N, lmax = 3N - 1, R = 2N ring pairs: the north
// rings 1 .. 2N-1 with their south mirrors, and the equator ring alone):
//   maps    [channel][12 N^2] float, RING order, as the reference's maps_out
//   acc     [channel][12 N_in^2] float, the merge sum at the input resolution
//   lam     orthonormal Legendre functions lambda_lm(theta_q) of the north
//           rings, FP64-evaluated and stored FP32, per m two blocks (l - m even,
//           l - m odd) of [l'][q] with l = m + 2 l' + parity: 4.8 GB at N = 512,
//           built once per context and kept (memory traded for FP64 work,
//           which GB300 runs at 1/64 of FP32)
//   E, O    per m, [q][2 c] float: the ring Fourier sums of the north ring plus
//           (E) or minus (O) those of its south mirror, for the channels c of one
//           batch; the same buffers then hold the synthesised north and south
//           ring sums
//   alm     per m, [parity][l'][2 c] float
//   LA, LS, EOp, almp: the same tables and sums packed for the tensor cores
//           (128-row tiles of TF32 hi and lo parts), per 64-channel column tile
// A transform is, per batch of channels: ring DFTs (one launch over a task list
// of (ring pair, channels): the 2 nside + 1 equatorial rings, 4 nside pixels
// each, by a register-resident radix-16 Stockham FFT of north + i south; the
// polar rings, 4 i pixels, by Bluestein's DFT over the same FFTs), the Legendre
// sums per (m, parity) as 3xTF32 tcgen05 GEMMs (nside <= 512) or FP32 GEMMs on
// the CUDA cores (the beam factor exp(-l(l+1) sigma_c^2 / 2) and the quadrature
// weight 4 pi / npix applied in the epilogue), the transposed GEMMs back, and
// the inverse ring transforms.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <ctime>
#include <string>
#include <vector>

#include "../../include/joint_gpu.h"
#include "common.cuh"
#include "healpix.h"
#include "host.h"
#include "stockham.cuh"
#include "tc.cuh"

using namespace gethi;
using namespace stockham;

namespace {

constexpr double kPrefacFwhm = 1030610.55;               // src/main_jt.c:26
constexpr double kPrefacTnu = 3.6e9;                     // src/main_jt.c:25
constexpr double kFwhm2Sigma = 0.00012352884853326381;  // src/healpix_extra.c:388
constexpr int kThreads = 256;
constexpr int kRingThreads = 512;  // ring transforms: threads per block (16 points each)
// shared-memory row pitch (float2) of one ring sequence of n points: padded, odd
__host__ __device__ constexpr int ring_pitch(int n) { return stockham::padded_len(n) | 1; }

struct RingPair {
  long long first_n, first_s;  // first pixel of the north ring and of its south mirror
  int nph;                     // pixels per ring
  int shifted;                 // first pixel at longitude pi / nph (else 0)
  long long tw_off;            // equatorial rings: offset of the twiddles e^{2 pi i t/nph} in the power-of-two
                               // table; polar rings: offset of the chirps e^{-i pi j^2/nph} in the chirp table
  int bm;                      // polar rings: Bluestein FFT size, the power of two >= 2 nph - 1
  int pad_;
  long long b_off;             // polar rings: offset of the chirp spectrum in the Bluestein table
};

// ---------------------------------------------------------------------------
// merge, ud_grade, noise, mask
// ---------------------------------------------------------------------------
// out = (((prev or 0) + s_0) + s_1) + ... element by element in FP32, the order in
// which src/main_jt.c:94 adds the components to its calloc'ed sum; a source with
// a factor is first scaled as (float)(value * factor) (src/main_jt.c:181)
constexpr int kMaxSum = 8;
struct SumSources {
  const float *p[kMaxSum];
  double f[kMaxSum];
  unsigned scaled;  // bit k: source k has a factor
};
// NS sources, one float4 (VEC) or one float per thread, the source loop unrolled.
// The FP64 scaling is compiled in only when some source has a factor (SCALED):
// FP64 instructions left in the loop, even predicated off, occupy GB300's slow
// FP64 pipe and cut this kernel from 7.3 to 1.1 TB/s.
template <int NS, bool VEC, bool SCALED>
__global__ void sum_kernel(float *__restrict__ out, const float *__restrict__ prev, SumSources s, long long n)
{
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (VEC) {
    if (i >= n / 4) return;
    float4 a = prev ? reinterpret_cast<const float4 *>(prev)[i] : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
    for (int k = 0; k < NS; k++) {
      float4 v = reinterpret_cast<const float4 *>(s.p[k])[i];
      if (SCALED && (s.scaled & (1u << k))) {
        v.x = (float)((double)v.x * s.f[k]);
        v.y = (float)((double)v.y * s.f[k]);
        v.z = (float)((double)v.z * s.f[k]);
        v.w = (float)((double)v.w * s.f[k]);
      }
      a.x = __fadd_rn(a.x, v.x);
      a.y = __fadd_rn(a.y, v.y);
      a.z = __fadd_rn(a.z, v.z);
      a.w = __fadd_rn(a.w, v.w);
    }
    reinterpret_cast<float4 *>(out)[i] = a;
  } else {
    if (i >= n) return;
    float a = prev ? prev[i] : 0.f;
#pragma unroll
    for (int k = 0; k < NS; k++) {
      float v = s.p[k][i];
      if (SCALED && (s.scaled & (1u << k))) v = (float)((double)v * s.f[k]);
      a = __fadd_rn(a, v);
    }
    out[i] = a;
  }
}

template <bool VEC, bool SCALED>
void launch_sum_t(float *out, const float *prev, const SumSources &s, int ns, long long n, cudaStream_t st)
{
  const long long items = VEC ? n / 4 : n;
  const unsigned blocks = (unsigned)((items + kThreads - 1) / kThreads);
  switch (ns) {
    case 1: sum_kernel<1, VEC, SCALED><<<blocks, kThreads, 0, st>>>(out, prev, s, n); break;
    case 2: sum_kernel<2, VEC, SCALED><<<blocks, kThreads, 0, st>>>(out, prev, s, n); break;
    case 3: sum_kernel<3, VEC, SCALED><<<blocks, kThreads, 0, st>>>(out, prev, s, n); break;
    case 4: sum_kernel<4, VEC, SCALED><<<blocks, kThreads, 0, st>>>(out, prev, s, n); break;
    case 5: sum_kernel<5, VEC, SCALED><<<blocks, kThreads, 0, st>>>(out, prev, s, n); break;
    case 6: sum_kernel<6, VEC, SCALED><<<blocks, kThreads, 0, st>>>(out, prev, s, n); break;
    case 7: sum_kernel<7, VEC, SCALED><<<blocks, kThreads, 0, st>>>(out, prev, s, n); break;
    default: sum_kernel<8, VEC, SCALED><<<blocks, kThreads, 0, st>>>(out, prev, s, n); break;
  }
}
template <bool VEC>
void launch_sum(float *out, const float *prev, const SumSources &s, int ns, long long n, cudaStream_t st)
{
  if (s.scaled) launch_sum_t<VEC, true>(out, prev, s, ns, n, st);
  else launch_sum_t<VEC, false>(out, prev, s, ns, n, st);
}

// he_udgrade, nside_in > nside_out: FP64 sum of the NESTED children in order, times 1/ratio
__global__ void degrade_kernel(const float *__restrict__ in, long long nside_in, float *__restrict__ out,
                               long long nside_out, int nmaps)
{
  const long long npix_out = 12 * nside_out * nside_out, npix_in = 12 * nside_in * nside_in;
  const long long ratio = npix_in / npix_out;
  const double inv = 1.0 / (double)ratio;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < npix_out * nmaps;
       t += (long long)gridDim.x * blockDim.x) {
    const long long c = t / npix_out, i = t - c * npix_out;
    const long long nest = hpx::ring2nest(nside_out, i);
    const float *m = in + c * npix_in;
    double tot = 0;
    for (long long j = 0; j < ratio; j++) tot = __dadd_rn(tot, (double)m[hpx::nest2ring(nside_in, j + ratio * nest)]);
    out[t] = (float)__dmul_rn(tot, inv);
  }
}

// he_udgrade, nside_in < nside_out: every NESTED child takes the parent's value
__global__ void upgrade_kernel(const float *__restrict__ in, long long nside_in, float *__restrict__ out,
                               long long nside_out, int nmaps)
{
  const long long npix_out = 12 * nside_out * nside_out, npix_in = 12 * nside_in * nside_in;
  const long long ratio = npix_out / npix_in;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < npix_out * nmaps;
       t += (long long)gridDim.x * blockDim.x) {
    const long long c = t / npix_out, i = t - c * npix_out;
    const long long nest = hpx::ring2nest(nside_out, i);
    out[t] = in[c * npix_in + hpx::nest2ring(nside_in, nest / ratio)];
  }
}

// blockIdx.y = channel; four pixels per thread (npix = 12 nside^2 is a multiple of 4)
__global__ void mask_kernel(float *__restrict__ maps, const int *__restrict__ mask, long long npix)
{
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= npix / 4) return;
  const int4 mk = reinterpret_cast<const int4 *>(mask)[i];
  if (mk.x && mk.y && mk.z && mk.w) return;
  float4 *m = reinterpret_cast<float4 *>(maps + (long long)blockIdx.y * npix) + i;
  float4 v = *m;
  if (!mk.x) v.x = 0.f;
  if (!mk.y) v.y = 0.f;
  if (!mk.z) v.z = 0.f;
  if (!mk.w) v.w = 0.f;
  *m = v;
}

// white noise with Philox4x32-10 draws, key (seed, "JOIN"), counter (pixel pair, channel):
// one call serves pixels 2j (words x, y) and 2j + 1 (z, w);
// noise = sqrt(-s2 ln(1 - u2)) cos(2 pi u1), the law of src/main_jt.c:304-311
__device__ __forceinline__ float noise_of(uint32_t w1, uint32_t w2, float s2)
{
  const float u1 = (float)(w1 >> 8) * (1.f / 16777216.f), u2 = (float)(w2 >> 8) * (1.f / 16777216.f);
  return sqrtf(-s2 * log1pf(-u2)) * cospif(2.f * u1);
}
// MASK: the mask applied in the same pass (noise, then mask, as the reference's
// stages: masked pixels end at 0 whatever their noise; the draws are counter-based,
// so skipping those of masked pixels changes no other pixel)
template <bool MASK>
__global__ void noise_philox_kernel(float *__restrict__ maps, const float *__restrict__ s2, long long npix,
                                    uint32_t seed, const int *__restrict__ mask)
{
  const long long j = blockIdx.x * (long long)blockDim.x + threadIdx.x;  // pixel pair
  if (j >= npix / 2) return;
  const int c = blockIdx.y;
  float2 *m = reinterpret_cast<float2 *>(maps + (long long)c * npix) + j;
  int2 mk = make_int2(1, 1);
  if (MASK) {
    mk = reinterpret_cast<const int2 *>(mask)[j];
    if (!mk.x && !mk.y) {
      *m = make_float2(0.f, 0.f);
      return;
    }
  }
  const uint4 r = philox4x32_10(make_uint4((uint32_t)j, (uint32_t)(j >> 32), (uint32_t)c, 0u), make_uint2(seed, 0x4A4F494Eu));
  const float sc = s2[c];
  float2 v = *m;
  v.x = __fadd_rn(v.x, noise_of(r.x, r.y, sc));
  v.y = __fadd_rn(v.y, noise_of(r.z, r.w, sc));
  if (!mk.x) v.x = 0.f;
  if (!mk.y) v.y = 0.f;
  *m = v;
}

// the reference's MT19937 noise (drawn on the host in FP64) added as it adds it:
// float = (float)((double)float + noise)
__global__ void noise_add_kernel(float *__restrict__ map, const double *__restrict__ noise, long long n)
{
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    map[i] = (float)__dadd_rn((double)map[i], noise[i]);
}

// ---------------------------------------------------------------------------
// spherical harmonic transform
// ---------------------------------------------------------------------------
__host__ __device__ inline long long m_offset(int m, int lmax)  // sum of (lmax - m' + 1), m' < m
{
  return (long long)m * (lmax + 1) - (long long)m * (m - 1) / 2;
}

// lambda_lm(theta_q), l = m .. lmax, for one m per blockIdx.y and one ring pair per
// thread: three-term recursion in l in FP64 with a power-of-two exponent kept
// apart (sin^m theta alone underflows FP64 for large m near the poles)
__global__ void lambda_kernel(const double *__restrict__ ring_z, const double *__restrict__ ring_log2sin,
                              const double *__restrict__ lmm0, int lmax, int R, float *__restrict__ lam)
{
  extern __shared__ double coef[];  // a_l at [l - m], b_l at [lmax + 1 + l - m]
  const int m = blockIdx.y, nl = lmax - m + 1;
  for (int i = threadIdx.x; i < nl; i += blockDim.x) {
    const int l = m + i;
    double a = 0, b = 0;
    if (i >= 1) a = sqrt((4.0 * l * l - 1.0) / ((double)(l - m) * (l + m)));
    if (i >= 2) b = sqrt(((double)(l - 1) * (l - 1) - (double)m * m) / (4.0 * (l - 1) * (l - 1) - 1.0));
    coef[i] = a;
    coef[lmax + 1 + i] = b;
  }
  __syncthreads();
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= R) return;
  const int ne = (lmax - m) / 2 + 1;
  const long long off = m_offset(m, lmax);
  float *Le = lam + off * R + q, *Lo = lam + (off + ne) * R + q;
  const double z = ring_z[q];
  const double lg = lmm0[m] + (m ? m * ring_log2sin[q] : 0.0);
  int e = (int)floor(lg);
  double p1 = exp2(lg - e), p2 = 0.0;
  if (m & 1) p1 = -p1;
  double sc = exp2((double)e);  // 0 when e < -1074: such values are far below FP32 range
  Le[0] = (float)(p1 * sc);
  for (int i = 1; i < nl; i++) {
    const double p = coef[i] * (z * p1 - coef[lmax + 1 + i] * p2);
    p2 = p1;
    p1 = p;
    if (fabs(p1) > 0x1p300) {
      p1 *= 0x1p-300;
      p2 *= 0x1p-300;
      e += 300;
      sc = exp2((double)e);
    }
    const float v = (float)(p1 * sc);
    if (i & 1) Lo[(long long)(i >> 1) * R] = v;
    else Le[(long long)(i >> 1) * R] = v;
  }
}

// ---- ring transforms --------------------------------------------------------
// One launch per direction covers every ring pair of a channel batch through a
// task list: task (q, c0, S) is ring pair q with the channels c0 .. c0 + S - 1,
// S = threads / max(1, M/16) sequences of M points (M = the ring length for the
// equatorial rings, the Bluestein size for the polar rings; a power of two, held
// as log2 in the task's w), so that every ring size fills the block.  Tasks are ordered by decreasing work.  The sequences'
// shared-memory rows have an odd pitch (in float2), so that threads of
// consecutive channels at the same frequency fall in different banks.

struct SeqLayout {
  int n, L, TS, PL, b, t;
  bool active;
};
__device__ __forceinline__ SeqLayout seq_layout(int n, int S)
{
  SeqLayout sl;
  sl.n = n;
  sl.L = __ffs(n) - 1;
  sl.TS = n >= 16 ? n >> 4 : 1;
  sl.PL = ring_pitch(n);
  sl.b = threadIdx.x / sl.TS;
  sl.t = threadIdx.x - sl.b * sl.TS;
  sl.active = sl.b < S;
  return sl;
}

// Folded sums Q_k (0 <= k <= n/2) of the north (Gn) and south (Gs) ring of pair q,
// channel c: the alias sum over m = +-k (mod n), m <= lmax, of c_m G_m e^{i m phi0},
// with c_m = 2 for m > 0 (real map) and the negative frequencies as conjugates.
// For a ring whose first pixel sits at phi0 = pi/n, e^{i m pi/n} =
// e^{i pi k/n} (-1)^j for m = k + j n, so the alternating sums are taken first
// and the phase ph = e^{i pi k/n} applied once.  Both rings share the m loop.
__device__ __forceinline__ void fold_pair(const float *__restrict__ Gn, const float *__restrict__ Gs,
                                          long long mstride, int k, int n, int lmax, bool shifted, float2 ph,
                                          float2 &qn, float2 &qs)
{
  const float flip = shifted ? -1.f : 1.f;
  float4 A = make_float4(0.f, 0.f, 0.f, 0.f), B = A;  // (north, south) of +k and of -k
  float sg = k ? 2.f : 1.f;                            // c_0 = 1
  for (int m = k; m <= lmax; m += n) {
    const float2 gn = *reinterpret_cast<const float2 *>(Gn + m * mstride);
    const float2 gs = *reinterpret_cast<const float2 *>(Gs + m * mstride);
    A.x += sg * gn.x;
    A.y += sg * gn.y;
    A.z += sg * gs.x;
    A.w += sg * gs.y;
    sg = (m ? sg : 2.f) * flip;
  }
  if (k != 0 && 2 * k != n) {
    sg = 2.f;
    for (int m = n - k; m <= lmax; m += n) {
      const float2 gn = *reinterpret_cast<const float2 *>(Gn + m * mstride);
      const float2 gs = *reinterpret_cast<const float2 *>(Gs + m * mstride);
      B.x += sg * gn.x;
      B.y += sg * gn.y;
      B.z += sg * gs.x;
      B.w += sg * gs.y;
      sg *= flip;
    }
  }
  if (shifted) {  // ph (A - conj B)
    qn = cmul(ph, make_float2(A.x - B.x, A.y + B.y));
    qs = cmul(ph, make_float2(A.z - B.z, A.w + B.w));
  } else {        // A + conj B
    qn = make_float2(A.x + B.x, A.y - B.y);
    qs = make_float2(A.z + B.z, A.w - B.w);
  }
}

// fold_pair for two adjacent channels (16-byte loads: G 16-byte aligned at the pair)
__device__ __forceinline__ void fold_pair2(const float *__restrict__ Gn, const float *__restrict__ Gs,
                                           long long mstride, int k, int n, int lmax, bool shifted, float2 ph,
                                           float2 (&qn)[2], float2 (&qs)[2])
{
  const float flip = shifted ? -1.f : 1.f;
  float4 An = make_float4(0.f, 0.f, 0.f, 0.f), As = An, Bn = An, Bs = An;
  float sg = k ? 2.f : 1.f;  // c_0 = 1
  for (int m = k; m <= lmax; m += n) {
    const float4 gn = *reinterpret_cast<const float4 *>(Gn + m * mstride);
    const float4 gs = *reinterpret_cast<const float4 *>(Gs + m * mstride);
    An.x += sg * gn.x; An.y += sg * gn.y; An.z += sg * gn.z; An.w += sg * gn.w;
    As.x += sg * gs.x; As.y += sg * gs.y; As.z += sg * gs.z; As.w += sg * gs.w;
    sg = (m ? sg : 2.f) * flip;
  }
  if (k != 0 && 2 * k != n) {
    sg = 2.f;
    for (int m = n - k; m <= lmax; m += n) {
      const float4 gn = *reinterpret_cast<const float4 *>(Gn + m * mstride);
      const float4 gs = *reinterpret_cast<const float4 *>(Gs + m * mstride);
      Bn.x += sg * gn.x; Bn.y += sg * gn.y; Bn.z += sg * gn.z; Bn.w += sg * gn.w;
      Bs.x += sg * gs.x; Bs.y += sg * gs.y; Bs.z += sg * gs.z; Bs.w += sg * gs.w;
      sg *= flip;
    }
  }
  if (shifted) {  // ph (A - conj B)
    qn[0] = cmul(ph, make_float2(An.x - Bn.x, An.y + Bn.y));
    qn[1] = cmul(ph, make_float2(An.z - Bn.z, An.w + Bn.w));
    qs[0] = cmul(ph, make_float2(As.x - Bs.x, As.y + Bs.y));
    qs[1] = cmul(ph, make_float2(As.z - Bs.z, As.w + Bs.w));
  } else {        // A + conj B
    qn[0] = make_float2(An.x + Bn.x, An.y - Bn.y);
    qn[1] = make_float2(An.z + Bn.z, An.w - Bn.w);
    qs[0] = make_float2(As.x + Bs.x, As.y - Bs.y);
    qs[1] = make_float2(As.z + Bs.z, As.w - Bs.w);
  }
}

// the Hermitian-packed values of frequencies kk and n - kk of one channel row from its
// folded sums: H_k = Q_k / 2, H_{n-k} = conj Q_k / 2 (0 < k < n/2), H_0, H_{n/2} = Re Q;
// value north + i south (Bluestein: conjugated, times the chirp)
__device__ __forceinline__ void put_spectrum(float2 *zb, int kk, int n, float2 hn, float2 hs, bool blue,
                                             const float2 *__restrict__ ch)
{
  const bool edge = kk == 0 || 2 * kk == n;
  const float f = edge ? 1.f : 0.5f;
  float2 v = edge ? make_float2(hn.x, hs.x) : make_float2(f * (hn.x - hs.y), f * (hn.y + hs.x));
  if (blue) v = cmul(make_float2(v.x, -v.y), __ldg(ch + kk));
  zb[spad(kk)] = v;
  if (!edge) {
    float2 v2 = make_float2(f * (hn.x + hs.y), f * (hs.x - hn.y));
    if (blue) v2 = cmul(make_float2(v2.x, -v2.y), __ldg(ch + (n - kk)));
    zb[spad(n - kk)] = v2;
  }
}

// E and O of pair q for m = 0 .. lmax from the DFTs Z of z_j = north_j + i south_j
// of S channels (z[b * PL + spad(k)], k < n): D_north,k = (Z_k + conj Z_{n-k}) / 2,
// D_south,k = (Z_k - conj Z_{n-k}) / 2i, F_m = e^{-i m phi0} D_{m mod n} with
// D_{n-k} = conj D_k, E = F_north + F_south, O = F_north - F_south.  One item per
// (m, channel), channels fastest: consecutive threads store consecutive channels.
// S = 2^lS divides the block; a thread keeps its channel and steps m, with
// (j, k) = divmod(m, n) kept up to date without divisions.
// E + i O contributions of one channel row (b) at folded frequency k: (E, O) of m
__device__ __forceinline__ void eo_of(const float2 *z, int PL, int b, int k, int n, bool eq, bool cj, float2 ph,
                                      float2 &e, float2 &o)
{
  const float2 zk = z[b * PL + spad(k)], zm = z[b * PL + spad(k ? n - k : 0)];
  float2 dn = make_float2(0.5f * (zk.x + zm.x), 0.5f * (zk.y - zm.y));
  float2 ds = eq ? make_float2(0.f, 0.f) : make_float2(0.5f * (zk.y + zm.y), -0.5f * (zk.x - zm.x));
  if (cj) {
    dn.y = -dn.y;
    ds.y = -ds.y;
  }
  e = cmul(make_float2(dn.x + ds.x, dn.y + ds.y), ph);
  o = cmul(make_float2(dn.x - ds.x, dn.y - ds.y), ph);
}

__device__ __forceinline__ void write_eo(const float2 *z, int PL, const RingPair &rp, const float2 *__restrict__ phtab,
                                         int q, bool eq, int lmax, int R, int N2, int nch, int c0, int lS,
                                         float *__restrict__ E, float *__restrict__ O)
{
  // items of two adjacent channels when the block holds two or more and the rows keep
  // 16-byte alignment (N2 a multiple of 4; c0 and b even): one 16-byte store each to E, O
  const bool pairs = lS > 0 && (N2 & 3) == 0;
  const int lP = pairs ? lS - 1 : lS, w = pairs ? 2 : 1;
  const int n = rp.nph, half = n / 2, b = (threadIdx.x & ((1 << lP) - 1)) * w, c = c0 + b;
  if (c >= nch) return;
  const bool pair = pairs && c + 1 < nch;
  const int mstep = blockDim.x >> lP, jstep = mstep / n, kstep = mstep - jstep * n;
  int m = threadIdx.x >> lP, j = m / n, kj = m - j * n;
  for (; m <= lmax; m += mstep, kj += kstep, j += jstep) {
    if (kj >= n) {
      kj -= n;
      j++;
    }
    int k = kj;
    float2 ph = make_float2(1.f, 0.f);
    if (rp.shifted) {  // e^{-i pi m/n} = conj(e^{i pi k/n}) (-1)^j
      const float2 t = __ldg(phtab + rp.first_n + k);
      ph = (j & 1) ? make_float2(-t.x, t.y) : make_float2(t.x, -t.y);
    }
    const bool cj = k > half;
    if (cj) k = n - k;
    const long long base = ((long long)m * R + q) * N2 + 2 * c;
    float2 e0, o0;
    eo_of(z, PL, b, k, n, eq, cj, ph, e0, o0);
    if (pair) {
      float2 e1, o1;
      eo_of(z, PL, b + 1, k, n, eq, cj, ph, e1, o1);
      *reinterpret_cast<float4 *>(E + base) = make_float4(e0.x, e0.y, e1.x, e1.y);
      *reinterpret_cast<float4 *>(O + base) = make_float4(o0.x, o0.y, o1.x, o1.y);
    } else {
      *reinterpret_cast<float2 *>(E + base) = e0;
      *reinterpret_cast<float2 *>(O + base) = o0;
    }
  }
}

// Ring analysis of one task.  Equatorial ring pairs (q >= nside - 1, n = 4 nside):
// one FFT per channel of z_j = north_j + i south_j, loaded from global memory
// straight into the first pass's registers.  Polar ring pairs (q < nside - 1,
// n = 4 (q + 1)): Bluestein's DFT, Z_k = c_k sum_j (z_j c_j) b_{k-j} with the chirp
// c_j = e^{-i pi j^2/n} (table ch, FP64-evaluated on the host) and b = conj(c),
// the convolution as a forward FFT of M >= 2n - 1 points, the product with the
// spectrum of b (table Bt) and an inverse FFT that takes the forward one's output
// in registers.  Then E and O of every m.
__global__ __launch_bounds__(kRingThreads, 2) void ring_analysis_kernel(
    const float *__restrict__ maps, long long npix, int nch, const RingPair *__restrict__ rings,
    const int4 *__restrict__ tasks, const float2 *__restrict__ tw2, const float2 *__restrict__ btab,
    const float2 *__restrict__ chirps, const float2 *__restrict__ phtab, int lmax, int R, int N2,
    float *__restrict__ E, float *__restrict__ O)
{
  extern __shared__ __align__(16) float2 z[];  // [S][pitch]
  const int4 tk = tasks[blockIdx.x];
  const int q = tk.x, c0 = tk.y, S = tk.z;
  if (c0 >= nch) return;  // a task of channels beyond this batch (block-uniform)
  const RingPair rp = rings[q];
  const int n = rp.nph;
  const bool blue = rp.bm > 0, eq = (q == R - 1);
  const SeqLayout sl = seq_layout(blue ? rp.bm : n, S);
  const int c = c0 + sl.b;
  const bool live = sl.active && c < nch;
  const float2 *ch = chirps + rp.tw_off, *Bt = btab + rp.b_off;
  float2 *s = z + (sl.active ? sl.b : 0) * sl.PL;
  float2 u[16];
  if (sl.active) {
    const float *mn = maps + (long long)(live ? c : 0) * npix + rp.first_n;
    const float *ms = maps + (long long)(live ? c : 0) * npix + rp.first_s;
#pragma unroll
    for (int i = 0; i < 16; i++) {
      const int j = sl.t + sl.TS * i;
      float2 v = make_float2(0.f, 0.f);
      if (live && j < n) {
        v.x = __ldg(mn + j);
        if (!eq) v.y = __ldg(ms + j);
        if (blue) v = cmul(v, __ldg(ch + j));
      }
      u[i] = v;
    }
  }
  fft_any<-1, false>(u, s, tw2, sl.n, sl.L, sl.t, sl.TS, sl.active);
  if (blue) {
    if (sl.active) {
#pragma unroll
      for (int i = 0; i < 16; i++) {
        const int j = sl.t + sl.TS * i;
        if (j < sl.n) u[i] = cmul(u[i], __ldg(Bt + j));
      }
    }
    fft_any<1, true>(u, s, tw2, sl.n, sl.L, sl.t, sl.TS, sl.active);
  }
  __syncthreads();  // every read of the last pass is done
  if (sl.active) {
    const float inv = 1.f / (float)sl.n;
#pragma unroll
    for (int i = 0; i < 16; i++) {
      const int k = sl.t + sl.TS * i;
      if (k >= n) continue;
      float2 v = u[i];
      if (blue) {
        v = cmul(v, __ldg(ch + k));
        v = make_float2(v.x * inv, v.y * inv);
      }
      s[spad(k)] = v;
    }
  }
  __syncthreads();
  write_eo(z, sl.PL, rp, phtab, q, eq, lmax, R, N2, nch, c0, tk.w, E, O);
}

// Ring synthesis of one task: the packed spectra (one item per (k, channel),
// channels fastest, into shared memory), then for the equatorial ring pairs one
// complex inverse FFT whose real and imaginary parts are the north and south
// rings' pixels, for the polar ring pairs conj(DFT(conj(.))) by Bluestein's DFT;
// the pixels are stored from the registers of the last pass.
__global__ __launch_bounds__(kRingThreads, 2) void ring_synthesis_kernel(
    const float *__restrict__ Gn, const float *__restrict__ Gs, const RingPair *__restrict__ rings,
    const int4 *__restrict__ tasks, const float2 *__restrict__ tw2, const float2 *__restrict__ btab,
    const float2 *__restrict__ chirps, const float2 *__restrict__ phtab, int lmax, int R, int N2, int nch,
    float *__restrict__ maps, long long npix)
{
  extern __shared__ __align__(16) float2 z[];  // [S][pitch]
  const int4 tk = tasks[blockIdx.x];
  const int q = tk.x, c0 = tk.y, S = tk.z;
  if (c0 >= nch) return;
  const RingPair rp = rings[q];
  const int n = rp.nph;
  const bool blue = rp.bm > 0, eq = (q == R - 1);
  const SeqLayout sl = seq_layout(blue ? rp.bm : n, S);
  const float2 *ch = chirps + rp.tw_off, *Bt = btab + rp.b_off;
  {  // one item per (kk <= n/2, channel or pair of adjacent channels), channels fastest
     // (S = 2^lS divides the block): the fold Q_kk serves both H_kk and H_{n-kk};
     // Bluestein's padding n .. M-1 is zero.  Pairs (16-byte loads) where the rows keep
     // 16-byte alignment (N2 a multiple of 4; c0 and b even)
    const bool pairs = tk.w > 0 && (N2 & 3) == 0;
    const int lP = pairs ? tk.w - 1 : tk.w, w = pairs ? 2 : 1;
    const int b = (threadIdx.x & ((1 << lP) - 1)) * w, c = c0 + b, kstep = blockDim.x >> lP, half = n / 2;
    float2 *zb = z + b * sl.PL;
    for (int k = n + (threadIdx.x >> lP); k < sl.n; k += kstep) {
      zb[spad(k)] = make_float2(0.f, 0.f);
      if (pairs) zb[sl.PL + spad(k)] = make_float2(0.f, 0.f);
    }
    const long long mstride = (long long)R * N2, off = (long long)q * N2 + 2 * c;
    for (int kk = threadIdx.x >> lP; kk <= half; kk += kstep) {
      const float2 ph = rp.shifted ? __ldg(phtab + rp.first_n + kk) : make_float2(1.f, 0.f);
      if (pairs) {
        float2 hn[2] = {}, hs[2] = {};
        if (c < nch) {  // the second channel may lie beyond the batch (its spectrum is not used)
          fold_pair2(Gn + off, Gs + off, mstride, kk, n, lmax, rp.shifted, ph, hn, hs);
          if (eq) hs[0] = hs[1] = make_float2(0.f, 0.f);
        }
        put_spectrum(zb, kk, n, hn[0], hs[0], blue, ch);
        put_spectrum(zb + sl.PL, kk, n, hn[1], hs[1], blue, ch);
      } else {
        float2 hn = make_float2(0.f, 0.f), hs = hn;
        if (c < nch) {
          fold_pair(Gn + off, Gs + off, mstride, kk, n, lmax, rp.shifted, ph, hn, hs);
          if (eq) hs = make_float2(0.f, 0.f);
        }
        put_spectrum(zb, kk, n, hn, hs, blue, ch);
      }
    }
  }
  __syncthreads();
  const int c = c0 + sl.b;
  float2 *s = z + (sl.active ? sl.b : 0) * sl.PL;
  float2 u[16];
  slots_load(u, s, sl.n, sl.t, sl.TS);  // all threads (idle ones read row 0): keeps u in registers
  if (blue) {  // the forward FFT of Bluestein's convolution and the product with Bt
    fft_any<-1, false>(u, s, tw2, sl.n, sl.L, sl.t, sl.TS, sl.active);
    if (sl.active) {
#pragma unroll
      for (int i = 0; i < 16; i++) {
        const int j = sl.t + sl.TS * i;
        if (j < sl.n) u[i] = cmul(u[i], __ldg(Bt + j));
      }
    }
  }
  // the inverse FFT: the equatorial rings' transform, or the end of the convolution
  // (the reversed plan, whose first pass takes the forward FFT's last in registers)
  fft_any<1, true>(u, s, tw2, sl.n, sl.L, sl.t, sl.TS, sl.active);
  if (sl.active && c < nch) {
    float *mn = maps + (long long)c * npix + rp.first_n, *msr = maps + (long long)c * npix + rp.first_s;
    const float inv = 1.f / (float)sl.n;
#pragma unroll
    for (int i = 0; i < 16; i++) {
      const int j = sl.t + sl.TS * i;
      if (j >= n) continue;
      if (blue) {
        const float2 v = cmul(u[i], __ldg(ch + j));  // conj of the pixel pair (north + i south), times M
        mn[j] = v.x * inv;
        msr[j] = -v.y * inv;
      } else {
        mn[j] = u[i].x;
        if (!eq) msr[j] = u[i].y;
      }
    }
  }
}

// e^{i pi k/n} of every ring pair q at tab[first_n + k], k < n (FP64-evaluated)
__global__ void ring_phase_kernel(const RingPair *__restrict__ rings, float2 *__restrict__ tab)
{
  const RingPair rp = rings[blockIdx.x];
  for (int k = threadIdx.x; k < rp.nph; k += blockDim.x) {
    double sn, cs;
    sincospi((double)k / (double)rp.nph, &sn, &cs);
    tab[rp.first_n + k] = make_float2((float)cs, (float)sn);
  }
}

constexpr int BM = 64, BN = 128, BK = 16;

// Tiles of the Legendre GEMMs, staged through registers into two shared-memory
// buffers (one barrier per k step): A as As[k][row] (rows padded by 4 floats),
// B as Bs[k][col].  A thread owns rows ty*4 .. ty*4+3 and the column groups
// tx*4 .. tx*4+3 and 64 + tx*4 .. 64 + tx*4+3.
struct GemmSmem {
  float As[2][BK][BM + 4];
  float Bs[2][BK][BN];
};

// 4 consecutive floats of a row (zero-filled beyond `len`)
__device__ __forceinline__ float4 load4(const float *__restrict__ row, int i, int len, bool vec)
{
  if (vec && i + 3 < len) return *reinterpret_cast<const float4 *>(row + i);
  float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
  if (i < len) v.x = row[i];
  if (i + 1 < len) v.y = row[i + 1];
  if (i + 2 < len) v.z = row[i + 2];
  if (i + 3 < len) v.w = row[i + 3];
  return v;
}

__device__ __forceinline__ void mma_tile(const GemmSmem &sm, int buf, int tx, int ty, float (&acc)[4][8])
{
#pragma unroll
  for (int k = 0; k < BK; k++) {
    const float4 a = *reinterpret_cast<const float4 *>(&sm.As[buf][k][ty * 4]);
    const float4 b0 = *reinterpret_cast<const float4 *>(&sm.Bs[buf][k][tx * 4]);
    const float4 b1 = *reinterpret_cast<const float4 *>(&sm.Bs[buf][k][64 + tx * 4]);
    const float av[4] = {a.x, a.y, a.z, a.w}, bv[8] = {b0.x, b0.y, b0.z, b0.w, b1.x, b1.y, b1.z, b1.w};
#pragma unroll
    for (int i = 0; i < 4; i++)
#pragma unroll
      for (int j = 0; j < 8; j++) acc[i][j] = fmaf(av[i], bv[j], acc[i][j]);
  }
}

// acc += A[row0.., 0..K) B[0..K), col0..) with A row-major [rows][K] (TRANS_A
// false, lda = K) or stored transposed as [K][lda] (TRANS_A true), B [K][N2]
template <bool TRANS_A>
__device__ __forceinline__ void gemm_tile(GemmSmem &sm, const float *__restrict__ A, int lda, int rows,
                                          const float *__restrict__ B, int N2, int K, int row0, int col0,
                                          float (&acc)[4][8])
{
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  const bool vec = (lda % 4 == 0) && (N2 % 4 == 0);
  const int nk = (K + BK - 1) / BK;
  float4 ra, rb0, rb1;
  auto load = [&](int k0) {
    if (!TRANS_A) {  // 64 rows x 16 k: row tid/4, k (tid%4)*4
      const int r = row0 + (tid >> 2), k = (tid & 3) * 4;
      ra = r < rows ? load4(A + (long long)r * lda + k0, k, K - k0, vec) : make_float4(0.f, 0.f, 0.f, 0.f);
    } else {         // 16 k x 64 rows: k tid/16, rows (tid%16)*4
      const int k = tid >> 4, r = (tid & 15) * 4;
      ra = k0 + k < K ? load4(A + (long long)(k0 + k) * lda + row0, r, rows - row0, vec)
                      : make_float4(0.f, 0.f, 0.f, 0.f);
    }
    const int kb = tid >> 5, c = (tid & 31) * 4;  // B: k rows kb and kb + 8, columns c .. c+3
    rb0 = k0 + kb < K ? load4(B + (long long)(k0 + kb) * N2 + col0, c, N2 - col0, vec) : make_float4(0.f, 0.f, 0.f, 0.f);
    rb1 = k0 + kb + 8 < K ? load4(B + (long long)(k0 + kb + 8) * N2 + col0, c, N2 - col0, vec)
                          : make_float4(0.f, 0.f, 0.f, 0.f);
  };
  auto store = [&](int buf) {
    if (!TRANS_A) {
      const int r = tid >> 2, k = (tid & 3) * 4;
      sm.As[buf][k][r] = ra.x;
      sm.As[buf][k + 1][r] = ra.y;
      sm.As[buf][k + 2][r] = ra.z;
      sm.As[buf][k + 3][r] = ra.w;
    } else {
      *reinterpret_cast<float4 *>(&sm.As[buf][tid >> 4][(tid & 15) * 4]) = ra;
    }
    const int kb = tid >> 5, c = (tid & 31) * 4;
    *reinterpret_cast<float4 *>(&sm.Bs[buf][kb][c]) = rb0;
    *reinterpret_cast<float4 *>(&sm.Bs[buf][kb + 8][c]) = rb1;
  };
  if (nk == 0) return;
  load(0);
  store(0);
  __syncthreads();
  for (int kt = 0; kt < nk; kt++) {
    const int buf = kt & 1;
    if (kt + 1 < nk) load((kt + 1) * BK);
    mma_tile(sm, buf, tx, ty, acc);
    if (kt + 1 < nk) store(buf ^ 1);
    __syncthreads();
  }
}

// Legendre analysis, one 64 x 128 tile of one (m, parity) per CTA:
// alm[l'][col] = scale(l, col) sum_q lam[l'][q] EO[q][col]
__global__ __launch_bounds__(kThreads, 2) void legendre_analysis_kernel(const float *__restrict__ lam,
                                                                        const float *__restrict__ E,
                                                                        const float *__restrict__ O,
                                                                        float *__restrict__ alm,
                                                                        const int4 *__restrict__ tasks, int R,
                                                                        int lmax, int N2, float w,
                                                                        const float *__restrict__ sig2)
{
  __shared__ __align__(16) GemmSmem sm;
  const int4 t = tasks[blockIdx.x];
  const int m = t.x, p = t.y, row0 = t.z * BM, col0 = t.w * BN;
  const int ne = (lmax - m) / 2 + 1, no = (lmax - m + 1) / 2, M = p ? no : ne;
  const long long off = m_offset(m, lmax) + (p ? ne : 0);
  float acc[4][8] = {};
  gemm_tile<false>(sm, lam + off * R, R, M, (p ? O : E) + (long long)m * R * N2, N2, R, row0, col0, acc);
  float *C = alm + off * N2;
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
#pragma unroll
  for (int i = 0; i < 4; i++) {
    const int r = row0 + ty * 4 + i;
    if (r >= M) continue;
    const float l = (float)(m + 2 * r + p);
#pragma unroll
    for (int j = 0; j < 8; j++) {
      const int col = col0 + (j < 4 ? tx * 4 + j : 64 + tx * 4 + j - 4);
      if (col >= N2) continue;
      float s = w;
      if (sig2) s *= expf(-0.5f * l * (l + 1.f) * sig2[col >> 1]);
      C[(long long)r * N2 + col] = acc[i][j] * s;
    }
  }
}

// Legendre synthesis, one 64 x 128 tile (ring pairs x columns) of one m per CTA:
// G_e[q][col] = sum_l' lam_e[l'][q] alm_e[l'][col] and the same for l - m odd;
// north ring sums G_e + G_o, south G_e - G_o (lambda_lm(-z) = (-1)^{l+m} lambda_lm(z))
__global__ __launch_bounds__(kThreads, 2) void legendre_synthesis_kernel(const float *__restrict__ lam,
                                                                         const float *__restrict__ alm,
                                                                         float *__restrict__ Gn,
                                                                         float *__restrict__ Gs,
                                                                         const int4 *__restrict__ tasks, int R,
                                                                         int lmax, int N2)
{
  __shared__ __align__(16) GemmSmem sm;
  const int4 t = tasks[blockIdx.x];
  const int m = t.x, row0 = t.z * BM, col0 = t.w * BN;
  const int ne = (lmax - m) / 2 + 1, no = (lmax - m + 1) / 2;
  const long long off = m_offset(m, lmax);
  float ae[4][8] = {}, ao[4][8] = {};
  gemm_tile<true>(sm, lam + off * R, R, R, alm + off * N2, N2, ne, row0, col0, ae);
  gemm_tile<true>(sm, lam + (off + ne) * R, R, R, alm + (off + ne) * N2, N2, no, row0, col0, ao);
  float *gn = Gn + (long long)m * R * N2, *gs = Gs + (long long)m * R * N2;
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
#pragma unroll
  for (int i = 0; i < 4; i++) {
    const int r = row0 + ty * 4 + i;
    if (r >= R) continue;
#pragma unroll
    for (int j = 0; j < 8; j++) {
      const int col = col0 + (j < 4 ? tx * 4 + j : 64 + tx * 4 + j - 4);
      if (col >= N2) continue;
      gn[(long long)r * N2 + col] = ae[i][j] + ao[i][j];
      gs[(long long)r * N2 + col] = ae[i][j] - ao[i][j];
    }
  }
}


// ---------------------------------------------------------------------------
// Legendre transforms on the tensor cores (3xTF32 on tcgen05)
//
// Operands live in HBM already packed as the MMA reads them: tiles of 128 rows
// x 32 K elements (128 B per row) in the no-swizzle K-major layout (8-row x 16 B
// core matrices, K-adjacent ones 128 B apart, 8-row groups 1 KB apart), hi
// tile (16 KB) then lo tile (16 KB), hi = x rounded to TF32, lo = x - hi.  The
// products hi*hi, hi*lo and lo*hi accumulate in two FP32 TMEM chains (error
// about 2^-22 per element).  Analysis: D[l'][col] = lambda[l'][q] EO[col][q]
// (A = the lambda table packed by rows l', B = E or O packed by channel
// columns).  Synthesis: D[q][col] = lambda[l'][q] alm[col][l'] over both
// parities (A = the lambda table packed by rows q, B = the a_lm the analysis
// epilogue packs).  A CTA stages its tiles with 16-byte cp.async copies through
// three shared-memory stages; one thread issues the MMAs and commits each stage
// to an mbarrier; every wait is bounded (1 s of the global timer) and sets an
// error flag the host reads.
// ---------------------------------------------------------------------------
namespace tcl {
// operand tiles: 128 rows x KK elements of K, hi then lo; KK for the analysis
// operands (lambda by l' rows, E/O) and for the synthesis operands (lambda by ring
// rows, the packed a_lm).  Both 16: 32 KB stages, two CTAs per SM (32-element
// tiles with one CTA per SM measured slower in both directions)
constexpr int kRows = 128, kKA = 16, kKS = 16;
template <int KK>
struct Geo {
  static constexpr uint32_t kHalf = kRows * KK * 4;  // the hi or the lo tile
  static constexpr uint32_t kTile = 2 * kHalf;
  static constexpr uint32_t kStage = 2 * kTile;      // A and B of one K step
  static constexpr uint32_t kSBO = 8 * KK * 4;       // stride of the 8-row core-matrix groups
};
// stages in flight per CTA (two CTAs of 256 TMEM columns per SM)
constexpr int kStagesA = 3, kStagesS = 3;
constexpr size_t kSmemA = kStagesA * Geo<kKA>::kStage, kSmemS = kStagesS * Geo<kKS>::kStage;
constexpr uint32_t kLBO = 128;  // K-adjacent core matrices
constexpr int kThreads = 128;
constexpr uint64_t kWaitNs = 1000000000ull;
}  // namespace tcl

template <int KK>
__host__ __device__ inline uint32_t tile_off(int r, int k)
{
  return (uint32_t)((r >> 3) * tcl::Geo<KK>::kSBO + (k >> 2) * 128 + (r & 7) * 16 + (k & 3) * 4);
}

__device__ __forceinline__ void split_tf32(float x, float &hi, float &lo)
{
  uint32_t h;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(h) : "f"(x));
  hi = __uint_as_float(h);
  lo = x - hi;
}


// Pack one 128 x KK tile: thread r writes row r (KK values of get(r, k)), hi and lo
template <int KK, class Get>
__device__ __forceinline__ void pack_tile(float *tile, Get get)
{
  const int r = threadIdx.x;
#pragma unroll
  for (int g = 0; g < KK / 4; g++) {
    float4 h, l;
    split_tf32(get(r, 4 * g + 0), h.x, l.x);
    split_tf32(get(r, 4 * g + 1), h.y, l.y);
    split_tf32(get(r, 4 * g + 2), h.z, l.z);
    split_tf32(get(r, 4 * g + 3), h.w, l.w);
    const uint32_t o = tile_off<KK>(r, 4 * g) / 4;
    *reinterpret_cast<float4 *>(tile + o) = h;
    *reinterpret_cast<float4 *>(tile + tcl::Geo<KK>::kHalf / 4 + o) = l;
  }
}

// lambda tables packed for the analysis (rows l', K = ring pairs; task = (m, p, l' tile,
// K tile)) and for the synthesis (rows = ring pairs, K = l'; task = (m, p, q tile, K tile))
template <int KK>
__global__ void __launch_bounds__(tcl::kThreads) pack_lambda_kernel(const float *__restrict__ lam,
                                                                    const int4 *__restrict__ tasks,
                                                                    const long long *__restrict__ off, int R, int lmax,
                                                                    int by_ring, float *__restrict__ out)
{
  const int4 t = tasks[blockIdx.x];
  const int m = t.x, p = t.y;
  const int ne = (lmax - m) / 2 + 1, M = p ? (lmax - m + 1) / 2 : ne;
  const float *L = lam + (m_offset(m, lmax) + (p ? ne : 0)) * (long long)R;
  const int nkq = (R + KK - 1) / KK, nkl = (M + KK - 1) / KK;
  float *tile = out + (off[2 * m + p] + (long long)t.z * (by_ring ? nkl : nkq) + t.w) * (tcl::Geo<KK>::kTile / 4);
  if (!by_ring) {
    const int l0 = t.z * tcl::kRows, q0 = t.w * KK;
    pack_tile<KK>(tile, [&](int r, int k) {
      return (l0 + r < M && q0 + k < R) ? L[(long long)(l0 + r) * R + q0 + k] : 0.f;
    });
  } else {
    const int qq = t.z * tcl::kRows, l0 = t.w * KK;
    pack_tile<KK>(tile, [&](int r, int k) {
      return (qq + r < R && l0 + k < M) ? L[(long long)(l0 + k) * R + qq + r] : 0.f;
    });
  }
}

// E and O packed by channel columns (rows = 128 columns of column tile ct, K = ring
// pairs); one CTA per (m, parity, column tile, K tile), tile index
// ((2 m + parity) NT + ct) nkq + kt.  Rows of columns beyond the batch (n2 = 2 x
// its channels) are left as they are: each MMA output column depends on its own B
// row only, and those outputs are never read.
__global__ void __launch_bounds__(tcl::kThreads) pack_eo_kernel(const float *__restrict__ E,
                                                                const float *__restrict__ O, int R, int N2, int n2,
                                                                float *__restrict__ out)
{
  constexpr int KK = tcl::kKA;
  const int nkq = (R + KK - 1) / KK, NT = N2 / tcl::kRows;
  const int kt = blockIdx.x % nkq, rest = blockIdx.x / nkq, ct = rest % NT, mp = rest / NT, m = mp >> 1, p = mp & 1;
  const float *src = (p ? O : E) + (long long)m * R * N2 + ct * tcl::kRows;
  const int q0 = kt * KK;
  if (ct * tcl::kRows + (int)threadIdx.x >= n2) return;  // this thread's row: a column beyond the batch
  float *tile = out + (long long)blockIdx.x * (tcl::Geo<KK>::kTile / 4);
  pack_tile<KK>(tile, [&](int r, int k) { return q0 + k < R ? src[(long long)(q0 + k) * N2 + r] : 0.f; });
}

// the three MMAs of one K step (KK / 8 instructions of K = 8 each per tile)
template <int KK>
__device__ __forceinline__ void mma3(uint32_t acc0, uint32_t acc1, uint32_t a, uint32_t b, bool first, uint32_t idesc)
{
  constexpr uint32_t sbo = tcl::Geo<KK>::kSBO, half = tcl::Geo<KK>::kHalf;
#pragma unroll
  for (int kk = 0; kk < KK / 8; kk++) {
    const uint64_t ah = tc::smem_desc(a + 256 * kk, tcl::kLBO, sbo);
    const uint64_t al = tc::smem_desc(a + half + 256 * kk, tcl::kLBO, sbo);
    const uint64_t bh = tc::smem_desc(b + 256 * kk, tcl::kLBO, sbo);
    const uint64_t bl = tc::smem_desc(b + half + 256 * kk, tcl::kLBO, sbo);
    const uint32_t acc = (first && kk == 0) ? 0u : 1u;
    tc::mma_tf32(acc0, ah, bh, idesc, acc);
    tc::mma_tf32(acc1, ah, bl, idesc, acc1 == acc0 ? 1u : acc);  // one accumulator: add to hi*hi
    tc::mma_tf32(acc1, al, bh, idesc, 1u);
  }
}

// The K loop shared by both transforms: tiles kt = 0 .. nk-1, A and B of tile kt
// (Geo<KK>::kTile bytes each, contiguous in global memory) at srcA(kt), srcB(kt);
// chain(kt) selects the accumulator pair and first(kt) whether the tile starts it;
// S stages.  Only the first nb rows of B (a multiple of 16: the batch's columns
// in this column tile) are copied and multiplied (MMA N = nb).  One thread drives it: each stage is filled by two bulk copies
// completing on full[s] and released by the commit of its MMAs to empty[s]; the
// stage of tile kt - 1 is refilled once its MMAs are done, while those of tile kt
// are queued.  Every wait is bounded; on an expired wait the copies and MMAs in
// flight are waited for (bounded again) and false is returned.
template <int S, int KK, class SrcA, class SrcB, class Chain>
__device__ bool tc_k_loop(unsigned char *sm, uint64_t *full, uint64_t *empty, int nk, int nb, SrcA srcA, SrcB srcB,
                          Chain chain, int *fail)
{
  using G = tcl::Geo<KK>;
  const uint32_t bpart = (uint32_t)(nb / 8) * G::kSBO;  // rows 0 .. nb-1 of one half of a B tile
  const uint32_t idesc = tc::idesc_tf32_f32(128, nb);
  if (threadIdx.x == 0) {
    auto load = [&](int kt) {
      const int s = kt % S;
      unsigned char *dst = sm + s * G::kStage;
      const unsigned char *b = srcB(kt);
      tc::mbar_arrive_expect_tx(&full[s], G::kTile + 2 * bpart);
      tc::bulk_g2s(dst, srcA(kt), G::kTile, &full[s]);
      tc::bulk_g2s(dst + G::kTile, b, bpart, &full[s]);
      tc::bulk_g2s(dst + G::kTile + G::kHalf, b + G::kHalf, bpart, &full[s]);
    };
    int issued = 0, done = 0;  // tiles whose copies were issued / consumed by MMAs
    bool ok = true;
    for (; issued < nk && issued < S; issued++) load(issued);
    for (int kt = 0; kt < nk; kt++) {
      const int s = kt % S;
      if (!tc::mbar_wait(&full[s], (kt / S) & 1, tcl::kWaitNs)) {
        ok = false;
        break;
      }
      tc::fence_after_sync();
      const uint32_t a = tc::smem_addr(sm + s * G::kStage), b = a + G::kTile;
      uint32_t acc0, acc1;
      bool first;
      chain(kt, acc0, acc1, first);
      mma3<KK>(acc0, acc1, a, b, first, idesc);
      tc::mma_commit(&empty[s]);
      done = kt + 1;
      if (kt >= 1 && issued < nk) {  // refill the stage of tile kt - 1 with tile kt - 1 + S
        const int sp = (kt - 1) % S;
        if (!tc::mbar_wait(&empty[sp], ((kt - 1) / S) & 1, tcl::kWaitNs)) {
          ok = false;
          break;
        }
        load(issued++);
      }
    }
    if (ok) {
      ok = tc::mbar_wait(&empty[(nk - 1) % S], ((nk - 1) / S) & 1, tcl::kWaitNs);
    } else {  // drain: copies of unconsumed tiles, then the last committed MMAs (bounded)
      for (int kt = done; kt < issued; kt++) tc::mbar_wait(&full[kt % S], (kt / S) & 1, tcl::kWaitNs);
      if (done > 0) tc::mbar_wait(&empty[(done - 1) % S], ((done - 1) / S) & 1, tcl::kWaitNs);
    }
    if (!ok) *fail = 1;
  }
  __syncthreads();
  tc::fence_after_sync();
  return *fail == 0;
}

// analysis, one CTA per (m, parity, 128-row l' tile, column tile ct): a_lm of the 128
// channel columns of ct, weight and beam applied, written packed for the synthesis
// (tile (alm_off + l'/32) NT + ct).  The column tiles of one l' tile are consecutive
// tasks, so that the CTAs streaming the same lambda tiles run together and share
// them through L2.
__global__ void __launch_bounds__(tcl::kThreads, 2)
    tc_legendre_analysis_kernel(const float *__restrict__ LA, const long long *__restrict__ la_off,
                                const float *__restrict__ EOp, float *__restrict__ almp,
                                const long long *__restrict__ alm_off, const int4 *__restrict__ tasks, int R, int lmax,
                                int NT, int n2, float w, const float *__restrict__ sig2, int *err)
{
  extern __shared__ __align__(1024) unsigned char sm[];
  __shared__ uint64_t full[tcl::kStagesA], empty[tcl::kStagesA];
  __shared__ uint32_t tslot;
  __shared__ int fail;
  const int4 t = tasks[blockIdx.x];
  const int m = t.x, p = t.y, mt = t.z, ct = t.w;
  const int ne = (lmax - m) / 2 + 1, M = p ? (lmax - m + 1) / 2 : ne;
  using GA = tcl::Geo<tcl::kKA>;
  using GS = tcl::Geo<tcl::kKS>;
  const int nkq = (R + tcl::kKA - 1) / tcl::kKA;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  __shared__ int skip;  // an earlier CTA's MMA wait expired: no new work (decided once for the CTA)
  if (tid == 0) skip = *(volatile int *)err;
  __syncthreads();
  const int neff = min(tcl::kRows, ((n2 - ct * tcl::kRows) + 15) & ~15);  // MMA N: this tile's batch columns
  if (skip || neff <= 0) return;
  if (warp == 0) tc::tmem_alloc(&tslot, 256);
  if (tid == 0) {
    for (int i = 0; i < tcl::kStagesA; i++) {
      tc::mbar_init(&full[i], 1);
      tc::mbar_init(&empty[i], 1);
    }
    fail = 0;
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tm = tslot;
  const unsigned char *A0 = reinterpret_cast<const unsigned char *>(LA) + (la_off[2 * m + p] + (long long)mt * nkq) * GA::kTile;
  const unsigned char *B0 =
      reinterpret_cast<const unsigned char *>(EOp) + ((long long)(2 * m + p) * NT + ct) * nkq * GA::kTile;
  const bool ok = tc_k_loop<tcl::kStagesA, tcl::kKA>(
      sm, full, empty, nkq, neff, [&](int kt) { return A0 + (long long)kt * GA::kTile; },
      [&](int kt) { return B0 + (long long)kt * GA::kTile; },
      [&](int kt, uint32_t &a0, uint32_t &a1, bool &first) {
        a0 = tm;
        a1 = tm + 128;
        first = kt == 0;
      },
      &fail);
  if (ok) {
    const int lp = mt * tcl::kRows + 32 * warp + lane;  // this thread's TMEM lane = row l'
    const bool valid = lp < M;
    const float l = (float)(m + 2 * lp + p);
    // the a_lm in the synthesis' B geometry (rows = columns, K = l' in tiles of kKS)
    float *tile = almp + ((alm_off[2 * m + p] + lp / tcl::kKS) * NT + ct) * (GS::kTile / 4);
    const uint32_t trow = tm + ((uint32_t)(32 * warp) << 16);
#pragma unroll 1
    for (int cb = 0; cb < neff; cb += 32) {
      float v0[32], v1[32];
      tc::tmem_ld32(trow + cb, v0);
      tc::tmem_ld32(trow + 128 + cb, v1);
      if (valid) {
#pragma unroll
        for (int j = 0; j < 32; j++) {
          const int col = cb + j;
          float sc = w;
          if (sig2) sc *= expf(-0.5f * l * (l + 1.f) * sig2[(ct * tcl::kRows + col) >> 1]);
          float hi, lo;
          split_tf32((v0[j] + v1[j]) * sc, hi, lo);
          const uint32_t o = tile_off<tcl::kKS>(col, lp & (tcl::kKS - 1)) / 4;
          tile[o] = hi;
          tile[GS::kHalf / 4 + o] = lo;
        }
      }
    }
  } else if (tid == 0) {
    atomicExch(err, 1);  // the K loop has drained its copies and MMAs
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(tm, 256);
}

// synthesis, one CTA per (m, 128 ring pairs, column tile ct): G_e and G_o over the
// packed a_lm of both parities, each in one TMEM accumulator (hi*hi and the hi*lo,
// lo*hi corrections together: 256 columns, two CTAs per SM); north = G_e + G_o,
// south = G_e - G_o, FP32 [m][q][col]
__global__ void __launch_bounds__(tcl::kThreads, 2)
    tc_legendre_synthesis_kernel(const float *__restrict__ LS, const long long *__restrict__ ls_off,
                                 const float *__restrict__ almp, const long long *__restrict__ alm_off,
                                 const int4 *__restrict__ tasks, int R, int lmax, int N2, int n2, float *__restrict__ Gn,
                                 float *__restrict__ Gs, int *err)
{
  extern __shared__ __align__(1024) unsigned char sm[];
  __shared__ uint64_t full[tcl::kStagesS], empty[tcl::kStagesS];
  __shared__ uint32_t tslot;
  __shared__ int fail;
  const int4 t = tasks[blockIdx.x];
  const int m = t.x, qt = t.z, ct = t.w, NT = N2 / tcl::kRows;
  const int ne = (lmax - m) / 2 + 1, no = (lmax - m + 1) / 2;
  using GS = tcl::Geo<tcl::kKS>;
  const int nke = (ne + tcl::kKS - 1) / tcl::kKS, nko = (no + tcl::kKS - 1) / tcl::kKS;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  __shared__ int skip;  // an earlier CTA's MMA wait expired: no new work (decided once for the CTA)
  if (tid == 0) skip = *(volatile int *)err;
  __syncthreads();
  const int neff = min(tcl::kRows, ((n2 - ct * tcl::kRows) + 15) & ~15);  // MMA N: this tile's batch columns
  if (skip || neff <= 0) return;
  if (warp == 0) tc::tmem_alloc(&tslot, 256);
  if (tid == 0) {
    for (int i = 0; i < tcl::kStagesS; i++) {
      tc::mbar_init(&full[i], 1);
      tc::mbar_init(&empty[i], 1);
    }
    fail = 0;
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tm = tslot;
  const unsigned char *LSb = reinterpret_cast<const unsigned char *>(LS);
  const unsigned char *Ab = reinterpret_cast<const unsigned char *>(almp);
  const bool ok = tc_k_loop<tcl::kStagesS, tcl::kKS>(
      sm, full, empty, nke + nko, neff,
      [&](int kt) {
        const int p = kt >= nke, k = p ? kt - nke : kt, nk = p ? nko : nke;
        return LSb + (ls_off[2 * m + p] + (long long)qt * nk + k) * GS::kTile;
      },
      [&](int kt) {
        const int p = kt >= nke, k = p ? kt - nke : kt;
        return Ab + ((alm_off[2 * m + p] + k) * NT + ct) * GS::kTile;
      },
      [&](int kt, uint32_t &a0, uint32_t &a1, bool &first) {
        const int p = kt >= nke;
        a0 = tm + 128 * p;  // hi*hi and the corrections in one accumulator per parity
        a1 = a0;
        first = kt == 0 || kt == nke;
      },
      &fail);
  if (ok) {
    const int q = qt * tcl::kRows + 32 * warp + lane;
    const uint32_t trow = tm + ((uint32_t)(32 * warp) << 16);
    float *gn = Gn + ((long long)m * R + q) * N2 + ct * tcl::kRows, *gs = Gs + ((long long)m * R + q) * N2 + ct * tcl::kRows;
#pragma unroll 1
    for (int cb = 0; cb < neff; cb += 32) {
      float e0[32], o0[32];
      tc::tmem_ld32(trow + cb, e0);
      tc::tmem_ld32(trow + 128 + cb, o0);
      if (q < R) {
#pragma unroll
        for (int j = 0; j < 32; j += 4) {
          float4 vn, vs;
          float ev[4], ov[4];
#pragma unroll
          for (int i = 0; i < 4; i++) {
            ev[i] = e0[j + i];
            ov[i] = nko ? o0[j + i] : 0.f;
          }
          vn = make_float4(ev[0] + ov[0], ev[1] + ov[1], ev[2] + ov[2], ev[3] + ov[3]);
          vs = make_float4(ev[0] - ov[0], ev[1] - ov[1], ev[2] - ov[2], ev[3] - ov[3]);
          *reinterpret_cast<float4 *>(gn + cb + j) = vn;
          *reinterpret_cast<float4 *>(gs + cb + j) = vs;
        }
      }
    }
  } else if (tid == 0) {
    atomicExch(err, 1);  // the K loop has drained its copies and MMAs
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(tm, 256);
}

// internal a_lm [m][parity][l'][2c] <-> HEALPix order [c][l + m lmax - m(m-1)/2] (complex)
__global__ void alm_to_healpix_kernel(const float *__restrict__ alm, float2 *__restrict__ out, int lmax, int N2,
                                      int nch, long long nalm)
{
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < nalm * nch;
       t += (long long)gridDim.x * blockDim.x) {
    const long long c = t / nalm, i = t - c * nalm;
    // i = m_offset(m) + (l - m): find m
    const float b2 = 2.f * lmax + 3.f;
    int m = max(0, min(lmax, (int)((b2 - sqrtf(fmaxf(b2 * b2 - 8.f * (float)i, 0.f))) * 0.5f)));
    while (m > 0 && m_offset(m, lmax) > i) m--;
    while (m < lmax && m_offset(m + 1, lmax) <= i) m++;
    const int l = m + (int)(i - m_offset(m, lmax)), ne = (lmax - m) / 2 + 1, p = (l - m) & 1;
    const long long row = m_offset(m, lmax) + (p ? ne : 0) + ((l - m) >> 1);
    out[t] = *reinterpret_cast<const float2 *>(alm + row * N2 + 2 * c);
  }
}

__global__ void alm_from_healpix_kernel(const float2 *__restrict__ in, float *__restrict__ alm, int lmax, int N2,
                                        int nch, long long nalm)
{
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < nalm * nch;
       t += (long long)gridDim.x * blockDim.x) {
    const long long c = t / nalm, i = t - c * nalm;
    const float b2 = 2.f * lmax + 3.f;
    int m = max(0, min(lmax, (int)((b2 - sqrtf(fmaxf(b2 * b2 - 8.f * (float)i, 0.f))) * 0.5f)));
    while (m > 0 && m_offset(m, lmax) > i) m--;
    while (m < lmax && m_offset(m + 1, lmax) <= i) m++;
    const int l = m + (int)(i - m_offset(m, lmax)), ne = (lmax - m) / 2 + 1, p = (l - m) & 1;
    const long long row = m_offset(m, lmax) + (p ? ne : 0) + ((l - m) >> 1);
    *reinterpret_cast<float2 *>(alm + row * N2 + 2 * c) = in[t];
  }
}

int grid_for(long long n)
{
  long long b = (n + kThreads - 1) / kThreads;
  return (int)std::max(1LL, std::min(b, 152LL * 16));
}

}  // namespace

// ---------------------------------------------------------------------------
// context
// ---------------------------------------------------------------------------
struct joint_ctx {
  joint_params p{};
  std::vector<double> nu0, nuf;
  std::vector<int> mask;  // empty: no mask
  double fsky = 1.0;
  int device = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  long long npix = 0;
  int lmax = 0, R = 0;
  float *maps = nullptr;   // [n_nu][npix]
  float *acc = nullptr;    // merge sum at nside_in
  long long nside_in = 0, acc_cap = 0;
  float *stage_buf = nullptr;  // host components staged on the device
  long long stage_cap = 0;
  int *dmask = nullptr;
  float *s2 = nullptr;     // per channel noise variance (Philox path)
  int stage = 0;           // 0 nothing added, 1 adding components, 2 merged (maps valid)
  bool have_acc = false;   // a component was added since the combination began
  bool acc_valid = false;  // acc holds the sum of the components before those still pending
  std::vector<std::pair<const float *, double>> pend;  // device components not summed yet, in order
  // spherical harmonic transform
  RingPair *rings = nullptr;
  float2 *tw2 = nullptr;   // e^{2 pi i t/M} at [M + t] for every power of two M
  float2 *btab = nullptr;  // polar rings: spectra of the conjugate Bluestein chirps (natural order)
  float2 *chirps = nullptr;  // polar rings: the chirps e^{-i pi j^2/n}, at 2 i (i - 1) for n = 4 i
  float *lam = nullptr;
  int chunk = 0, N2 = 0;
  float *E = nullptr, *O = nullptr, *alm = nullptr, *sig2 = nullptr, *tmp_maps = nullptr;
  float2 *alm_hp = nullptr;
  int4 *tasks_a = nullptr, *tasks_s = nullptr;
  int ntasks_a = 0, ntasks_s = 0;
  double *noise_h = nullptr, *noise_d = nullptr;  // mt_validation staging (pinned host, device)
  // tensor-core Legendre sums: packed tables, offsets (in operand tiles per (m, parity)), task lists
  bool use_tc = false;
  float *LA = nullptr, *LS = nullptr, *EOp = nullptr, *almp = nullptr;
  long long *la_off = nullptr, *ls_off = nullptr, *alm_off = nullptr;
  int4 *tasks_ta = nullptr, *tasks_ts = nullptr;
  int ntasks_ta = 0, ntasks_ts = 0;
  int *tc_err = nullptr;
  cudaEvent_t ev[5] = {};
  float times[4] = {};
  // ring-transform tasks (q, c0, S) in decreasing work, e^{i pi k/n} per ring, block shared memory
  int4 *rtasks = nullptr;
  int nrtasks = 0;
  float2 *phtab = nullptr;
  size_t ring_smem = 0;
  // optional per-kernel-class device times of the beam (joint_gpu_profile):
  // ring analysis, Legendre analysis, Legendre synthesis, ring synthesis, E/O pack
  int prof = 0;
  std::vector<cudaEvent_t> kev;
  std::vector<int> kcls;
  double ktime[5] = {};
  long kcount[5] = {};
};

namespace {

int jfail(cudaError_t e, const char *what)
{
  set_error(std::string(what) + ": " + cudaGetErrorString(e));
  return GETHI_E_CUDA;
}
#define JCK(call)                                       \
  do {                                                  \
    cudaError_t e_ = (call);                            \
    if (e_ != cudaSuccess) return jfail(e_, #call);     \
  } while (0)

template <class T>
int jalloc(T **p, size_t count)
{
  cudaError_t e = cudaMalloc((void **)p, std::max<size_t>(count, 1) * sizeof(T));
  if (e != cudaSuccess) {
    *p = nullptr;
    set_error(std::string("cudaMalloc of ") + std::to_string(count * sizeof(T)) + " bytes: " + cudaGetErrorString(e));
    return GETHI_E_NOMEM;
  }
  return GETHI_OK;
}

int bluestein_size(int n)  // the power of two >= 2n - 1
{
  int M = 1;
  while (M < 2 * n - 1) M <<= 1;
  return M;
}

// forward DFT (e^{-2 pi i jk/M}) of a power-of-two length in FP64 on the host
void host_fft(std::vector<double> &re, std::vector<double> &im)
{
  const size_t n = re.size();
  for (size_t i = 1, j = 0; i < n; i++) {
    size_t bit = n >> 1;
    for (; j & bit; bit >>= 1) j ^= bit;
    j ^= bit;
    if (i < j) {
      std::swap(re[i], re[j]);
      std::swap(im[i], im[j]);
    }
  }
  std::vector<double> wr(n / 2), wi(n / 2);
  for (size_t k = 0; k < n / 2; k++) {
    wr[k] = std::cos(2 * M_PI * (double)k / (double)n);
    wi[k] = -std::sin(2 * M_PI * (double)k / (double)n);
  }
  for (size_t len = 2; len <= n; len <<= 1) {
    const size_t st = n / len;
    for (size_t i = 0; i < n; i += len)
      for (size_t k = 0; k < len / 2; k++) {
        const double cr = wr[k * st], ci = wi[k * st];
        const size_t a = i + k, b = a + len / 2;
        const double vr = re[b] * cr - im[b] * ci, vi = re[b] * ci + im[b] * cr;
        re[b] = re[a] - vr;
        im[b] = im[a] - vi;
        re[a] += vr;
        im[a] += vi;
      }
  }
}


// packed lambda tables, offsets and task lists of the tensor-core Legendre sums
int ensure_tc_tables(joint_ctx *c)
{
  const int R = c->R, lmax = c->lmax, NT = c->N2 / tcl::kRows;
  const int nkq = (R + tcl::kKA - 1) / tcl::kKA, nqt = (R + tcl::kRows - 1) / tcl::kRows;
  std::vector<long long> la(2 * (lmax + 1)), ls(2 * (lmax + 1)), al(2 * (lmax + 1));
  std::vector<int4> pa, ps, ta, ts;
  long long na = 0, ns = 0, nl = 0;
  for (int m = 0; m <= lmax; m++) {
    for (int p = 0; p < 2; p++) {
      const int M = p ? (lmax - m + 1) / 2 : (lmax - m) / 2 + 1;
      const int nmt = (M + tcl::kRows - 1) / tcl::kRows, nkl = (M + tcl::kKS - 1) / tcl::kKS;
      la[2 * m + p] = na;
      ls[2 * m + p] = ns;
      al[2 * m + p] = nl;
      for (int mt = 0; mt < nmt; mt++) {
        for (int ct = 0; ct < NT; ct++) ta.push_back(make_int4(m, p, mt, ct));
        for (int kt = 0; kt < nkq; kt++) pa.push_back(make_int4(m, p, mt, kt));
      }
      for (int qt = 0; qt < nqt; qt++)
        for (int kt = 0; kt < nkl; kt++) ps.push_back(make_int4(m, p, qt, kt));
      na += (long long)nmt * nkq;
      ns += (long long)nqt * nkl;
      nl += nkl;
    }
    for (int qt = 0; qt < nqt; qt++)
      for (int ct = 0; ct < NT; ct++) ts.push_back(make_int4(m, 0, qt, ct));
  }
  const size_t twa = tcl::Geo<tcl::kKA>::kTile / 4, tws = tcl::Geo<tcl::kKS>::kTile / 4;
  int rc;
  int4 *dpa = nullptr, *dps = nullptr;
  if ((rc = jalloc(&c->LA, (size_t)na * twa)) || (rc = jalloc(&c->LS, (size_t)ns * tws)) ||
      (rc = jalloc(&c->EOp, (size_t)2 * (lmax + 1) * NT * nkq * twa)) ||
      (rc = jalloc(&c->almp, (size_t)nl * NT * tws)) ||
      (rc = jalloc(&c->la_off, la.size())) || (rc = jalloc(&c->ls_off, ls.size())) ||
      (rc = jalloc(&c->alm_off, al.size())) || (rc = jalloc(&c->tasks_ta, ta.size())) ||
      (rc = jalloc(&c->tasks_ts, ts.size())) || (rc = jalloc(&c->tc_err, 1)) || (rc = jalloc(&dpa, pa.size())) ||
      (rc = jalloc(&dps, ps.size()))) {
    cudaFree(dpa);
    for (void **ptr : {(void **)&c->LA, (void **)&c->LS, (void **)&c->EOp, (void **)&c->almp, (void **)&c->la_off,
                       (void **)&c->ls_off, (void **)&c->alm_off, (void **)&c->tasks_ta, (void **)&c->tasks_ts,
                       (void **)&c->tc_err}) {
      cudaFree(*ptr);
      *ptr = nullptr;
    }
    return rc;
  }
  c->ntasks_ta = (int)ta.size();
  c->ntasks_ts = (int)ts.size();
  JCK(cudaMemcpyAsync(c->la_off, la.data(), sizeof(long long) * la.size(), cudaMemcpyHostToDevice, c->stream));
  JCK(cudaMemcpyAsync(c->ls_off, ls.data(), sizeof(long long) * ls.size(), cudaMemcpyHostToDevice, c->stream));
  JCK(cudaMemcpyAsync(c->alm_off, al.data(), sizeof(long long) * al.size(), cudaMemcpyHostToDevice, c->stream));
  JCK(cudaMemcpyAsync(c->tasks_ta, ta.data(), sizeof(int4) * ta.size(), cudaMemcpyHostToDevice, c->stream));
  JCK(cudaMemcpyAsync(c->tasks_ts, ts.data(), sizeof(int4) * ts.size(), cudaMemcpyHostToDevice, c->stream));
  JCK(cudaMemcpyAsync(dpa, pa.data(), sizeof(int4) * pa.size(), cudaMemcpyHostToDevice, c->stream));
  JCK(cudaMemcpyAsync(dps, ps.data(), sizeof(int4) * ps.size(), cudaMemcpyHostToDevice, c->stream));
  JCK(cudaMemsetAsync(c->almp, 0, sizeof(float) * nl * NT * tws, c->stream));  // l' padding stays zero
  JCK(cudaMemsetAsync(c->EOp, 0, sizeof(float) * 2 * (lmax + 1) * NT * nkq * twa, c->stream));  // padded columns
  JCK(cudaMemsetAsync(c->tc_err, 0, sizeof(int), c->stream));
  pack_lambda_kernel<tcl::kKA><<<(unsigned)pa.size(), tcl::kThreads, 0, c->stream>>>(c->lam, dpa, c->la_off, R, lmax,
                                                                                   0, c->LA);
  JCK(cudaGetLastError());
  pack_lambda_kernel<tcl::kKS><<<(unsigned)ps.size(), tcl::kThreads, 0, c->stream>>>(c->lam, dps, c->ls_off, R, lmax,
                                                                                   1, c->LS);
  JCK(cudaGetLastError());
  JCK(cudaFuncSetAttribute(tc_legendre_analysis_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tcl::kSmemA));
  JCK(cudaFuncSetAttribute(tc_legendre_synthesis_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tcl::kSmemS));
  JCK(cudaStreamSynchronize(c->stream));
  cudaFree(dpa);
  cudaFree(dps);
  c->use_tc = true;
  return GETHI_OK;
}

// ring pairs, twiddles and the Legendre table of the context's nside (first transform)
int ensure_sht(joint_ctx *c)
{
  if (c->lam) return GETHI_OK;
  const long long N = c->p.nside;
  if (N > 1024) {
    set_error("spherical harmonic transforms support nside <= 1024");
    return GETHI_E_ARG;
  }
  const int R = (int)(2 * N), lmax = (int)(3 * N - 1);
  c->R = R;
  c->lmax = lmax;
  std::vector<RingPair> rp(R);
  std::vector<double> z(R), lsin(R), lmm0(lmax + 1);
  const long long npix = 12 * N * N, ncap = 2 * N * (N - 1);
  for (int q = 0; q < R; q++) {
    const long long i = q + 1;  // north ring number (q = R - 1: the equator)
    double cz, sz;
    RingPair r;
    if (i < N) {
      const double a = (double)i * i / (3.0 * N * N);
      cz = 1.0 - a;
      sz = std::sqrt(a * (2.0 - a));
      r.nph = (int)(4 * i);
      r.shifted = 1;
      r.first_n = 2 * i * (i - 1);
    } else {
      cz = (double)(2 * N - i) * (2.0 / (3.0 * N));
      sz = std::sqrt((1.0 - cz) * (1.0 + cz));
      r.nph = (int)(4 * N);
      r.shifted = ((i - N) & 1) ? 0 : 1;
      r.first_n = ncap + (i - N) * 4 * N;
    }
    r.first_s = npix - r.nph - r.first_n;
    r.tw_off = i < N ? 2 * i * (i - 1) : r.nph;  // polar: chirp table offset; equatorial: tw2[nph + t]
    r.bm = i < N ? bluestein_size(r.nph) : 0;
    r.pad_ = 0;
    r.b_off = 0;
    rp[q] = r;
    z[q] = cz;
    lsin[q] = std::log2(sz);
  }
  double acc = 0;
  for (int m = 0; m <= lmax; m++) {
    if (m > 0) acc += 0.5 * std::log2((2.0 * m - 1.0) / (2.0 * m));
    lmm0[m] = 0.5 * std::log2((2.0 * m + 1.0) / (4.0 * M_PI)) + acc;
  }
  // power-of-two twiddles, and per polar ring the spectrum of its conjugate chirp
  // b_t = e^{i pi t^2 / n} (t = -(n-1) .. n-1, wrapped modulo M) for Bluestein's DFT
  int Mmax = (int)(4 * N);
  for (int q = 0; q < N - 1; q++) Mmax = std::max(Mmax, rp[q].bm);
  std::vector<float2> tw2(2 * (size_t)Mmax);
  for (int M = 1; M <= Mmax; M <<= 1)
    for (int t = 0; t < M; t++) {
      const double a = 2.0 * M_PI * (double)t / (double)M;
      tw2[M + t] = make_float2((float)std::cos(a), (float)std::sin(a));
    }
  std::vector<float2> chirps(std::max<long long>(2 * N * (N - 1), 1));
  for (int q = 0; q < N - 1; q++) {
    const int n = rp[q].nph;
    for (int j = 0; j < n; j++) {
      const double a = M_PI * (double)(((long long)j * j) % (2 * n)) / (double)n;
      chirps[rp[q].tw_off + j] = make_float2((float)std::cos(a), (float)-std::sin(a));
    }
  }
  std::vector<float2> btab;
  for (int q = 0; q < N - 1; q++) {
    const int n = rp[q].nph, M = rp[q].bm;
    std::vector<double> re(M, 0.0), im(M, 0.0);
    for (int t = 0; t < n; t++) {
      const double a = M_PI * (double)(((long long)t * t) % (2 * n)) / (double)n;
      re[t] = std::cos(a);
      im[t] = std::sin(a);
      if (t) {
        re[M - t] = re[t];
        im[M - t] = im[t];
      }
    }
    host_fft(re, im);
    rp[q].b_off = (long long)btab.size();
    btab.resize(btab.size() + M);
    for (int t = 0; t < M; t++) btab[rp[q].b_off + t] = make_float2((float)re[t], (float)im[t]);
  }
  int rc;
  const size_t lam_elems = (size_t)m_offset(lmax + 1, lmax) * R;
  if ((rc = jalloc(&c->rings, R)) || (rc = jalloc(&c->tw2, tw2.size())) || (rc = jalloc(&c->btab, btab.size())) ||
      (rc = jalloc(&c->chirps, chirps.size())) ||
      (rc = jalloc(&c->lam, lam_elems)))
    return rc;
  double *dz = nullptr, *dl = nullptr, *dm = nullptr;
  if ((rc = jalloc(&dz, R)) || (rc = jalloc(&dl, R)) || (rc = jalloc(&dm, lmax + 1))) {
    cudaFree(dz);
    cudaFree(dl);
    return rc;
  }
  JCK(cudaMemcpyAsync(c->rings, rp.data(), sizeof(RingPair) * R, cudaMemcpyHostToDevice, c->stream));
  JCK(cudaMemcpyAsync(c->tw2, tw2.data(), sizeof(float2) * tw2.size(), cudaMemcpyHostToDevice, c->stream));
  if (!btab.empty())
    JCK(cudaMemcpyAsync(c->btab, btab.data(), sizeof(float2) * btab.size(), cudaMemcpyHostToDevice, c->stream));
  JCK(cudaMemcpyAsync(c->chirps, chirps.data(), sizeof(float2) * chirps.size(), cudaMemcpyHostToDevice, c->stream));
  JCK(cudaMemcpyAsync(dz, z.data(), sizeof(double) * R, cudaMemcpyHostToDevice, c->stream));
  JCK(cudaMemcpyAsync(dl, lsin.data(), sizeof(double) * R, cudaMemcpyHostToDevice, c->stream));
  JCK(cudaMemcpyAsync(dm, lmm0.data(), sizeof(double) * (lmax + 1), cudaMemcpyHostToDevice, c->stream));
  const size_t smem = sizeof(double) * 2 * (lmax + 1);
  JCK(cudaFuncSetAttribute(lambda_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  lambda_kernel<<<dim3((R + 127) / 128, lmax + 1), 128, smem, c->stream>>>(dz, dl, dm, lmax, R, c->lam);
  JCK(cudaGetLastError());
  JCK(cudaStreamSynchronize(c->stream));
  cudaFree(dz);
  cudaFree(dl);
  cudaFree(dm);
  // channel batches and the GEMM tile lists
  // channels per batch: the tensor-core path reads the whole Legendre table once per
  // batch and direction, so it takes every channel at once (columns in tiles of 64
  // channels, up to 256); the CUDA-core path batches 64
  const bool tc_ok = c->p.sht_precision == 0 && N <= 512;
  c->chunk = c->p.sht_chunk > 0 ? c->p.sht_chunk
             : tc_ok            ? std::min(256, 64 * ((c->p.n_nu + 63) / 64))
                                : 64;
  c->N2 = 2 * c->chunk;
  const int tcol = (c->N2 + BN - 1) / BN;
  std::vector<int4> ta, ts;
  for (int m = 0; m <= lmax; m++) {
    const int ne = (lmax - m) / 2 + 1, no = (lmax - m + 1) / 2;
    for (int p = 0; p < 2; p++) {
      const int M = p ? no : ne;
      for (int tr = 0; tr < (M + BM - 1) / BM; tr++)
        for (int tc = 0; tc < tcol; tc++) ta.push_back(make_int4(m, p, tr, tc));
    }
    for (int tr = 0; tr < (R + BM - 1) / BM; tr++)
      for (int tc = 0; tc < tcol; tc++) ts.push_back(make_int4(m, 0, tr, tc));
  }
  c->ntasks_a = (int)ta.size();
  c->ntasks_s = (int)ts.size();
  const size_t eo = (size_t)(lmax + 1) * R * c->N2;
  if ((rc = jalloc(&c->tasks_a, ta.size())) || (rc = jalloc(&c->tasks_s, ts.size())) || (rc = jalloc(&c->E, eo)) ||
      (rc = jalloc(&c->O, eo)) || (rc = jalloc(&c->alm, (size_t)m_offset(lmax + 1, lmax) * c->N2)) ||
      (rc = jalloc(&c->sig2, c->chunk)))
    return rc;
  // columns of channels beyond a batch are never written by the ring transforms: zero
  JCK(cudaMemsetAsync(c->E, 0, sizeof(float) * eo, c->stream));
  JCK(cudaMemsetAsync(c->O, 0, sizeof(float) * eo, c->stream));
  JCK(cudaMemcpyAsync(c->tasks_a, ta.data(), sizeof(int4) * ta.size(), cudaMemcpyHostToDevice, c->stream));
  JCK(cudaMemcpyAsync(c->tasks_s, ts.data(), sizeof(int4) * ts.size(), cudaMemcpyHostToDevice, c->stream));
  // ring-transform tasks: per ring pair, blocks of S = threads / max(1, M/16) channels
  // (M: ring length, or Bluestein size for the polar rings), largest work first
  {
    struct T {
      int4 t;
      double w;
    };
    std::vector<T> tl;
    size_t smem = 0;
    for (int q = 0; q < R; q++) {
      const int M = rp[q].bm > 0 ? rp[q].bm : rp[q].nph, TS = std::max(1, M / 16);
      int S = kRingThreads / TS;
      while (S > c->chunk && S > 1) S >>= 1;  // a power of two, at most the batch (or 1)
      smem = std::max(smem, (size_t)S * ring_pitch(M) * sizeof(float2));
      const double w = (rp[q].bm > 0 ? 2.0 : 1.0) * S * M * std::max(1, __builtin_ctz((unsigned)M));
      for (int c0 = 0; c0 < c->chunk; c0 += S) tl.push_back({make_int4(q, c0, S, __builtin_ctz((unsigned)S)), w});
    }
    std::stable_sort(tl.begin(), tl.end(), [](const T &x, const T &y) { return x.w > y.w; });
    std::vector<int4> tv(tl.size());
    for (size_t i = 0; i < tl.size(); i++) tv[i] = tl[i].t;
    c->nrtasks = (int)tv.size();
    c->ring_smem = smem;
    const size_t nph = (size_t)(rp[R - 1].first_n + rp[R - 1].nph);
    if ((rc = jalloc(&c->rtasks, tv.size())) || (rc = jalloc(&c->phtab, nph))) return rc;
    JCK(cudaMemcpyAsync(c->rtasks, tv.data(), sizeof(int4) * tv.size(), cudaMemcpyHostToDevice, c->stream));
    ring_phase_kernel<<<R, 256, 0, c->stream>>>(c->rings, c->phtab);
    JCK(cudaGetLastError());
    JCK(cudaFuncSetAttribute(ring_analysis_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    JCK(cudaFuncSetAttribute(ring_synthesis_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  }
  if (tc_ok && c->N2 % tcl::kRows == 0) {
    int rt = ensure_tc_tables(c);
    if (rt == GETHI_E_NOMEM) {  // the packed tables do not fit: FP32 CUDA cores
      cudaGetLastError();
      rt = GETHI_OK;
    }
    if (rt) return rt;
  }
  JCK(cudaStreamSynchronize(c->stream));
  return GETHI_OK;
}

// events around one kernel class when profiling (joint_gpu_profile)
struct KSpan {
  joint_ctx *c;
  int cls;
  KSpan(joint_ctx *c_, int cls_) : c(c_), cls(cls_) { mark(); }
  ~KSpan() { mark(); }
  void mark()
  {
    if (!c->prof) return;
    cudaEvent_t e;
    cudaEventCreate(&e);
    cudaEventRecord(e, c->stream);
    c->kev.push_back(e);
    c->kcls.push_back(cls);
  }
};

void collect_kernel_times(joint_ctx *c)  // after a synchronize; spans may nest
{
  std::vector<size_t> open;
  for (size_t i = 0; i < c->kev.size(); i++) {
    if (!open.empty() && c->kcls[open.back()] == c->kcls[i]) {
      float ms = 0;
      cudaEventElapsedTime(&ms, c->kev[open.back()], c->kev[i]);
      c->ktime[c->kcls[i]] += ms;
      c->kcount[c->kcls[i]]++;
      open.pop_back();
    } else {
      open.push_back(i);
    }
  }
  for (cudaEvent_t e : c->kev) cudaEventDestroy(e);
  c->kev.clear();
  c->kcls.clear();
}

int sht_analysis(joint_ctx *c, const float *dmaps, int nch, const float *sig2, bool tc)
{
  {
    KSpan k(c, 0);
    ring_analysis_kernel<<<c->nrtasks, kRingThreads, c->ring_smem, c->stream>>>(
        dmaps, c->npix, nch, c->rings, c->rtasks, c->tw2, c->btab, c->chirps, c->phtab, c->lmax, c->R, c->N2, c->E,
        c->O);
  }
  JCK(cudaGetLastError());
  const float w = (float)(4.0 * M_PI / (double)c->npix);
  {
    KSpan k(c, 1);  // the pack's own span (class 4) nests inside: class 1 = pack + GEMM
    if (tc) {
      const int nkq = (c->R + tcl::kKA - 1) / tcl::kKA;
      {
        KSpan kp(c, 4);
        pack_eo_kernel<<<2 * (c->lmax + 1) * (c->N2 / tcl::kRows) * nkq, tcl::kThreads, 0, c->stream>>>(
            c->E, c->O, c->R, c->N2, 2 * nch, c->EOp);
      }
      tc_legendre_analysis_kernel<<<c->ntasks_ta, tcl::kThreads, tcl::kSmemA, c->stream>>>(
          c->LA, c->la_off, c->EOp, c->almp, c->alm_off, c->tasks_ta, c->R, c->lmax, c->N2 / tcl::kRows, 2 * nch, w,
          sig2, c->tc_err);
    } else {
      legendre_analysis_kernel<<<c->ntasks_a, kThreads, 0, c->stream>>>(c->lam, c->E, c->O, c->alm, c->tasks_a,
                                                                        c->R, c->lmax, c->N2, w, sig2);
    }
  }
  JCK(cudaGetLastError());
  return GETHI_OK;
}

// alm2map of c->alm into nch device maps
int sht_synthesis(joint_ctx *c, float *dmaps, int nch, bool tc)
{
  {
    KSpan k(c, 2);
    if (tc)
      tc_legendre_synthesis_kernel<<<c->ntasks_ts, tcl::kThreads, tcl::kSmemS, c->stream>>>(
          c->LS, c->ls_off, c->almp, c->alm_off, c->tasks_ts, c->R, c->lmax, c->N2, 2 * nch, c->E, c->O, c->tc_err);
    else
      legendre_synthesis_kernel<<<c->ntasks_s, kThreads, 0, c->stream>>>(c->lam, c->alm, c->E, c->O, c->tasks_s,
                                                                         c->R, c->lmax, c->N2);
  }
  JCK(cudaGetLastError());
  {
    KSpan k(c, 3);
    ring_synthesis_kernel<<<c->nrtasks, kRingThreads, c->ring_smem, c->stream>>>(
        c->E, c->O, c->rings, c->rtasks, c->tw2, c->btab, c->chirps, c->phtab, c->lmax, c->R, c->N2, nch, dmaps,
        c->npix);
  }
  JCK(cudaGetLastError());
  return GETHI_OK;
}

void record(joint_ctx *c, int i) { cudaEventRecord(c->ev[i], c->stream); }

}  // namespace

extern "C" int joint_gpu_init(const joint_params *p, int device, joint_ctx **out)
{
  if (!p || !out) return GETHI_E_ARG;
  *out = nullptr;
  if (p->nside < 1 || p->nside > 8192 || (p->nside & (p->nside - 1))) {
    set_error("nside must be a power of two between 1 and 8192");
    return GETHI_E_ARG;
  }
  if (p->n_nu < 1 || !p->nu0 || !p->nuf) {
    set_error("JoinT needs a frequency table (n_nu >= 1)");
    return GETHI_E_ARG;
  }
  if (p->rng != JOINT_RNG_PHILOX && p->rng != JOINT_RNG_MT_VALIDATION) {
    set_error("rng must be philox or mt_validation");
    return GETHI_E_ARG;
  }
  if (p->tsys > 0 && (p->time_tot <= 0 || p->n_dish <= 0)) {
    set_error("noise needs time_total > 0 and n_dishes > 0");
    return GETHI_E_ARG;
  }
  JCK(cudaSetDevice(device));
  joint_ctx *c = new joint_ctx;
  c->p = *p;
  c->device = device;
  c->nu0.assign(p->nu0, p->nu0 + p->n_nu);
  c->nuf.assign(p->nuf, p->nuf + p->n_nu);
  c->p.nu0 = c->nu0.data();
  c->p.nuf = c->nuf.data();
  c->npix = 12LL * p->nside * p->nside;
  if (p->mask) {
    c->mask.assign(p->mask, p->mask + c->npix);
    long long on = 0;
    for (int v : c->mask) on += v != 0;
    c->fsky = (double)on / (double)c->npix;  // src/io_jt.c:76
  }
  c->p.mask = c->mask.empty() ? nullptr : c->mask.data();
  int rc;
  if ((rc = jalloc(&c->maps, (size_t)c->npix * p->n_nu)) || (rc = jalloc(&c->s2, p->n_nu)) ||
      (!c->mask.empty() && (rc = jalloc(&c->dmask, c->npix)))) {
    joint_gpu_free(c);
    return rc;
  }
  cudaError_t e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    joint_gpu_free(c);
    return jfail(e, "cudaStreamCreate");
  }
  c->own_stream = true;
  for (auto &ev : c->ev) cudaEventCreate(&ev);
  if (!c->mask.empty())
    cudaMemcpyAsync(c->dmask, c->mask.data(), sizeof(int) * c->npix, cudaMemcpyHostToDevice, c->stream);
  std::vector<float> s2(p->n_nu);
  for (int i = 0; i < p->n_nu; i++) {
    const double dnu = c->nuf[i] - c->nu0[i];
    s2[i] = (float)(c->fsky * c->npix * p->tsys * p->tsys / (kPrefacTnu * dnu * p->time_tot * p->n_dish));
  }
  cudaMemcpyAsync(c->s2, s2.data(), sizeof(float) * p->n_nu, cudaMemcpyHostToDevice, c->stream);
  e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) {
    joint_gpu_free(c);
    return jfail(e, "joint_gpu_init");
  }
  *out = c;
  return GETHI_OK;
}

extern "C" void joint_gpu_free(joint_ctx *c)
{
  if (!c) return;
  cudaSetDevice(c->device);
  if (c->stream) cudaStreamSynchronize(c->stream);
  for (void *ptr : {(void *)c->maps, (void *)c->acc, (void *)c->stage_buf, (void *)c->dmask, (void *)c->s2,
                    (void *)c->rings, (void *)c->tw2, (void *)c->btab, (void *)c->chirps, (void *)c->lam, (void *)c->E, (void *)c->O, (void *)c->alm,
                    (void *)c->sig2, (void *)c->tmp_maps, (void *)c->alm_hp, (void *)c->tasks_a, (void *)c->tasks_s,
                    (void *)c->noise_d, (void *)c->LA, (void *)c->LS, (void *)c->EOp, (void *)c->almp,
                    (void *)c->la_off, (void *)c->ls_off, (void *)c->alm_off, (void *)c->tasks_ta,
                    (void *)c->tasks_ts, (void *)c->tc_err, (void *)c->rtasks, (void *)c->phtab})
    cudaFree(ptr);
  if (c->noise_h) cudaFreeHost(c->noise_h);
  for (cudaEvent_t e : c->kev) cudaEventDestroy(e);
  for (auto &ev : c->ev)
    if (ev) cudaEventDestroy(ev);
  if (c->own_stream && c->stream) cudaStreamDestroy(c->stream);
  delete c;
}

extern "C" int joint_gpu_set_stream(joint_ctx *c, void *stream)
{
  if (!c) return GETHI_E_ARG;
  JCK(cudaStreamSynchronize(c->stream));
  if (c->own_stream) cudaStreamDestroy(c->stream);
  c->stream = (cudaStream_t)stream;
  c->own_stream = false;
  return GETHI_OK;
}

extern "C" double joint_gpu_fsky(const joint_ctx *c) { return c ? c->fsky : -1.0; }

// launch sums of `prev` and up to kMaxSum pending components at a time into out
static int sum_into(joint_ctx *c, float *out, const float *prev, const std::pair<const float *, double> *src, int ns,
                    long long n)
{
  do {
    SumSources ss;
    const int k_n = std::min(ns, kMaxSum);
    uintptr_t al = reinterpret_cast<uintptr_t>(out) | reinterpret_cast<uintptr_t>(prev);
    ss.scaled = 0;
    for (int k = 0; k < kMaxSum; k++) {
      ss.p[k] = k < k_n ? src[k].first : nullptr;
      ss.f[k] = k < k_n ? src[k].second : 1.0;
      if (k < k_n) {
        al |= reinterpret_cast<uintptr_t>(src[k].first);
        if (src[k].second != 1.0) ss.scaled |= 1u << k;
      }
    }
    if ((al & 15) == 0 && n % 4 == 0) launch_sum<true>(out, prev, ss, k_n, n, c->stream);
    else launch_sum<false>(out, prev, ss, k_n, n, c->stream);
    JCK(cudaGetLastError());
    prev = out;
    src += k_n;
    ns -= k_n;
  } while (ns > 0);
  return GETHI_OK;
}

// the components still pending -> acc (in order after what acc already holds)
static int flush_pending(joint_ctx *c)
{
  if (c->pend.empty()) return GETHI_OK;
  const long long n = 12LL * c->nside_in * c->nside_in * c->p.n_nu;
  if (n > c->acc_cap) {
    JCK(cudaStreamSynchronize(c->stream));
    cudaFree(c->acc);
    c->acc = nullptr;
    int rc = jalloc(&c->acc, n);
    if (rc) return rc;
    c->acc_cap = n;
  }
  int rc = sum_into(c, c->acc, c->acc_valid ? c->acc : nullptr, c->pend.data(), (int)c->pend.size(), n);
  if (rc) return rc;
  c->acc_valid = true;
  c->pend.clear();
  return GETHI_OK;
}

// record one component (device memory valid until the merge); a new combination
// starts with the first component after a merge
static int add_common(joint_ctx *c, const float *dsrc, long nside_in, double factor)
{
  if (c->stage == 1 && nside_in != c->nside_in) {
    set_error("read nside is not the same as provided : " + std::to_string(c->nside_in) +
              " != " + std::to_string(nside_in));  // src/main_jt.c:74-81
    return GETHI_E_ARG;
  }
  if (c->stage != 1) {
    c->nside_in = nside_in;
    c->stage = 1;
    c->have_acc = true;
    c->acc_valid = false;
    c->pend.clear();
  }
  c->pend.push_back({dsrc, factor});
  return GETHI_OK;
}

static bool valid_nside(long ns) { return ns >= 1 && ns <= 8192 && !(ns & (ns - 1)); }

extern "C" int joint_gpu_add_maps(joint_ctx *c, const float *maps, long nside_in, double factor)
{
  if (!c || !maps || !valid_nside(nside_in)) return GETHI_E_ARG;
  JCK(cudaSetDevice(c->device));
  const long long n = 12LL * nside_in * nside_in * c->p.n_nu;
  if (n > c->stage_cap) {
    JCK(cudaStreamSynchronize(c->stream));
    cudaFree(c->stage_buf);
    c->stage_buf = nullptr;
    int rc = jalloc(&c->stage_buf, n);
    if (rc) return rc;
    c->stage_cap = n;
  }
  JCK(cudaMemcpyAsync(c->stage_buf, maps, sizeof(float) * n, cudaMemcpyHostToDevice, c->stream));
  int rc = add_common(c, c->stage_buf, nside_in, factor);
  if (rc) return rc;
  if ((rc = flush_pending(c))) return rc;  // the staging buffer is reused by the next host component
  JCK(cudaStreamSynchronize(c->stream));   // the caller may reuse `maps`
  return GETHI_OK;
}

extern "C" int joint_gpu_add_maps_device(joint_ctx *c, const float *dmaps, long nside_in, double factor)
{
  if (!c || !dmaps || !valid_nside(nside_in)) return GETHI_E_ARG;
  JCK(cudaSetDevice(c->device));
  return add_common(c, dmaps, nside_in, factor);
}

extern "C" int joint_gpu_merge(joint_ctx *c)
{
  if (!c) return GETHI_E_ARG;
  JCK(cudaSetDevice(c->device));
  const long long N = c->p.nside, n = c->npix * c->p.n_nu;
  if (!c->have_acc) {  // no component: the reference leaves the calloc'ed maps at zero
    JCK(cudaMemsetAsync(c->maps, 0, sizeof(float) * n, c->stream));
  } else if (c->nside_in == N && !c->pend.empty()) {
    // same resolution: the pending components are summed straight into the maps (the
    // list is kept, so a repeated run sums them again)
    int rc = sum_into(c, c->maps, c->acc_valid ? c->acc : nullptr, c->pend.data(), (int)c->pend.size(), n);
    if (rc) return rc;
  } else {  // (again) from the sum, so a repeated run starts from the merged components
    int rc = flush_pending(c);
    if (rc) return rc;
    if (c->nside_in == N)
      JCK(cudaMemcpyAsync(c->maps, c->acc, sizeof(float) * n, cudaMemcpyDeviceToDevice, c->stream));
    else if (c->nside_in > N)
      degrade_kernel<<<grid_for(n), kThreads, 0, c->stream>>>(c->acc, c->nside_in, c->maps, N, c->p.n_nu);
    else
      upgrade_kernel<<<grid_for(n), kThreads, 0, c->stream>>>(c->acc, c->nside_in, c->maps, N, c->p.n_nu);
    JCK(cudaGetLastError());
  }
  c->stage = 2;
  return GETHI_OK;
}

static int need_maps(joint_ctx *c)
{
  if (c->stage != 2) {
    set_error("the maps are not merged yet (joint_gpu_merge)");
    return GETHI_E_STATE;
  }
  return GETHI_OK;
}

extern "C" int joint_gpu_apply_beam(joint_ctx *c)
{
  if (!c) return GETHI_E_ARG;
  int rc = need_maps(c);
  if (rc) return rc;
  JCK(cudaSetDevice(c->device));
  if (c->p.dish_diameter <= 0) {
    set_error("apply_beam needs dish_diameter > 0");
    return GETHI_E_ARG;
  }
  if ((rc = ensure_sht(c))) return rc;
  for (int c0 = 0; c0 < c->p.n_nu; c0 += c->chunk) {
    const int nch = std::min(c->chunk, c->p.n_nu - c0);
    std::vector<float> sg(c->chunk, 0.f);
    for (int i = 0; i < nch; i++) {  // src/main_jt.c:224-226, src/healpix_extra.c:390-400
      const double nu = 0.5 * (c->nu0[c0 + i] + c->nuf[c0 + i]);
      const double fwhm = kPrefacFwhm / (nu * c->p.dish_diameter);
      const double sigma = kFwhm2Sigma * fwhm;
      sg[i] = (float)(sigma * sigma);
    }
    JCK(cudaMemcpyAsync(c->sig2, sg.data(), sizeof(float) * c->chunk, cudaMemcpyHostToDevice, c->stream));
    float *m = c->maps + (long long)c0 * c->npix;
    if ((rc = sht_analysis(c, m, nch, c->sig2, c->use_tc))) return rc;
    if ((rc = sht_synthesis(c, m, nch, c->use_tc))) return rc;
  }
  return GETHI_OK;
}

extern "C" int joint_gpu_add_noise(joint_ctx *c)
{
  if (!c) return GETHI_E_ARG;
  int rc = need_maps(c);
  if (rc) return rc;
  JCK(cudaSetDevice(c->device));
  if (c->p.tsys <= 0) {
    set_error("add_noise needs t_system > 0");
    return GETHI_E_ARG;
  }
  const long long npix = c->npix;
  if (c->p.rng == JOINT_RNG_PHILOX) {
    noise_philox_kernel<false><<<dim3((unsigned)((npix / 2 + kThreads - 1) / kThreads), c->p.n_nu), kThreads, 0,
                                 c->stream>>>(c->maps, c->s2, npix, c->p.seed, nullptr);
    JCK(cudaGetLastError());
    return GETHI_OK;
  }
  // mt_validation: the draws of src/main_jt.c:284-313, per emulated OpenMP thread t an
  // MT19937 seeded seed + t over t's static block of channels
  if (!c->noise_h) {
    JCK(cudaMallocHost((void **)&c->noise_h, sizeof(double) * npix));
    if ((rc = jalloc(&c->noise_d, npix))) return rc;
  }
  const int T = std::max(1, c->p.omp_threads_for_noise), n_nu = c->p.n_nu;
  for (int t = 0; t < T; t++) {
    int q = n_nu / T, r = n_nu % T, i0;
    if (t < r) {
      q++;
      i0 = q * t;
    } else
      i0 = q * t + r;
    MT19937 rng(c->p.seed + (unsigned)t);
    for (int inu = i0; inu < i0 + q; inu++) {
      const double dnu = c->nuf[inu] - c->nu0[inu];
      const double s2 = c->fsky * npix * c->p.tsys * c->p.tsys / (kPrefacTnu * dnu * c->p.time_tot * c->p.n_dish);
      JCK(cudaStreamSynchronize(c->stream));  // the staging buffer of the previous channel is free
      for (long long i = 0; i < npix; i++) {
        const double phase = 2 * M_PI * rng.uniform();
        const double u = rng.uniform();
        c->noise_h[i] = std::sqrt(-s2 * std::log(1 - u)) * std::cos(phase);
      }
      JCK(cudaMemcpyAsync(c->noise_d, c->noise_h, sizeof(double) * npix, cudaMemcpyHostToDevice, c->stream));
      noise_add_kernel<<<grid_for(npix), kThreads, 0, c->stream>>>(c->maps + (long long)inu * npix, c->noise_d, npix);
      JCK(cudaGetLastError());
    }
  }
  JCK(cudaStreamSynchronize(c->stream));
  return GETHI_OK;
}

extern "C" int joint_gpu_apply_mask(joint_ctx *c)
{
  if (!c) return GETHI_E_ARG;
  int rc = need_maps(c);
  if (rc) return rc;
  JCK(cudaSetDevice(c->device));
  if (!c->dmask) return GETHI_OK;  // "none"/"default": every pixel kept
  mask_kernel<<<dim3((unsigned)((c->npix / 4 + kThreads - 1) / kThreads), c->p.n_nu), kThreads, 0, c->stream>>>(
      c->maps, c->dmask, c->npix);
  JCK(cudaGetLastError());
  return GETHI_OK;
}

// an expired MMA wait in the tensor-core Legendre sums (read after a synchronize)
static int check_tc(joint_ctx *c)
{
  if (!c->tc_err) return GETHI_OK;
  int e = 0;
  JCK(cudaMemcpy(&e, c->tc_err, sizeof(int), cudaMemcpyDeviceToHost));
  if (e) {
    cudaMemset(c->tc_err, 0, sizeof(int));
    set_error("tensor-core Legendre sums: an MMA completion wait expired");
    return GETHI_E_DEVICE;
  }
  return GETHI_OK;
}

extern "C" int joint_gpu_get_maps(joint_ctx *c, float *maps_out)
{
  if (!c || !maps_out) return GETHI_E_ARG;
  int rc = need_maps(c);
  if (rc) return rc;
  JCK(cudaSetDevice(c->device));
  JCK(cudaMemcpyAsync(maps_out, c->maps, sizeof(float) * c->npix * c->p.n_nu, cudaMemcpyDeviceToHost, c->stream));
  JCK(cudaStreamSynchronize(c->stream));
  return check_tc(c);
}

extern "C" int joint_gpu_device_maps(const joint_ctx *c, const float **dmaps)
{
  if (!c || !dmaps) return GETHI_E_ARG;
  *dmaps = c->maps;
  return GETHI_OK;
}

extern "C" int joint_gpu_run(joint_ctx *c, float *maps_out)
{
  if (!c) return GETHI_E_ARG;
  JCK(cudaSetDevice(c->device));
  int rc;
  record(c, 0);
  if ((rc = joint_gpu_merge(c))) return rc;
  record(c, 1);
  if (c->p.dish_diameter > 0 && (rc = joint_gpu_apply_beam(c))) return rc;
  record(c, 2);
  const bool fuse = c->p.tsys > 0 && c->p.rng == JOINT_RNG_PHILOX && c->dmask;
  if (fuse) {  // noise and mask in one pass (its time is the noise stage's; the mask stage reads 0)
    if ((rc = need_maps(c))) return rc;
    noise_philox_kernel<true><<<dim3((unsigned)((c->npix / 2 + kThreads - 1) / kThreads), c->p.n_nu), kThreads, 0,
                                c->stream>>>(c->maps, c->s2, c->npix, c->p.seed, c->dmask);
    JCK(cudaGetLastError());
    record(c, 3);
  } else {
    if (c->p.tsys > 0 && (rc = joint_gpu_add_noise(c))) return rc;
    record(c, 3);
    if ((rc = joint_gpu_apply_mask(c))) return rc;
  }
  record(c, 4);
  if (maps_out) {
    if ((rc = joint_gpu_get_maps(c, maps_out))) return rc;
  } else {
    JCK(cudaStreamSynchronize(c->stream));
  }
  for (int i = 0; i < 4; i++) cudaEventElapsedTime(&c->times[i], c->ev[i], c->ev[i + 1]);
  collect_kernel_times(c);
  return check_tc(c);
}

extern "C" int joint_gpu_uses_tensor_cores(const joint_ctx *c) { return c && c->use_tc ? 1 : 0; }

extern "C" int joint_gpu_profile(joint_ctx *c, int on)
{
  if (!c) return GETHI_E_ARG;
  JCK(cudaStreamSynchronize(c->stream));
  collect_kernel_times(c);
  c->prof = on ? 1 : 0;
  for (int i = 0; i < 5; i++) {
    c->ktime[i] = 0;
    c->kcount[i] = 0;
  }
  return GETHI_OK;
}

extern "C" int joint_gpu_kernel_times(joint_ctx *c, double *ms5, long *launches5)
{
  if (!c || !ms5) return GETHI_E_ARG;
  JCK(cudaStreamSynchronize(c->stream));
  collect_kernel_times(c);
  for (int i = 0; i < 5; i++) {
    ms5[i] = c->ktime[i];
    if (launches5) launches5[i] = c->kcount[i];
  }
  return GETHI_OK;
}

extern "C" int joint_gpu_stage_times(const joint_ctx *c, float *ms4)
{
  if (!c || !ms4) return GETHI_E_ARG;
  for (int i = 0; i < 4; i++) ms4[i] = c->times[i];
  return GETHI_OK;
}

static int sht_api(joint_ctx *c, const float *in, int n_maps, float *out, bool analysis)
{
  if (!c || !in || !out || n_maps < 1) return GETHI_E_ARG;
  JCK(cudaSetDevice(c->device));
  int rc = ensure_sht(c);
  if (rc) return rc;
  const long long nalm = m_offset(c->lmax + 1, c->lmax);
  if (!c->tmp_maps) {
    if ((rc = jalloc(&c->tmp_maps, (size_t)c->chunk * c->npix)) || (rc = jalloc(&c->alm_hp, (size_t)c->chunk * nalm)))
      return rc;
  }
  for (int c0 = 0; c0 < n_maps; c0 += c->chunk) {
    const int nch = std::min(c->chunk, n_maps - c0);
    if (analysis) {
      JCK(cudaMemcpyAsync(c->tmp_maps, in + (long long)c0 * c->npix, sizeof(float) * nch * c->npix,
                          cudaMemcpyHostToDevice, c->stream));
      if ((rc = sht_analysis(c, c->tmp_maps, nch, nullptr, false))) return rc;  // a_lm in the FP32 layout
      alm_to_healpix_kernel<<<grid_for(nalm * nch), kThreads, 0, c->stream>>>(c->alm, c->alm_hp, c->lmax, c->N2, nch,
                                                                              nalm);
      JCK(cudaGetLastError());
      JCK(cudaMemcpyAsync(out + 2 * (long long)c0 * nalm, c->alm_hp, sizeof(float2) * nch * nalm,
                          cudaMemcpyDeviceToHost, c->stream));
    } else {
      JCK(cudaMemcpyAsync(c->alm_hp, in + 2 * (long long)c0 * nalm, sizeof(float2) * nch * nalm,
                          cudaMemcpyHostToDevice, c->stream));
      alm_from_healpix_kernel<<<grid_for(nalm * nch), kThreads, 0, c->stream>>>(c->alm_hp, c->alm, c->lmax, c->N2,
                                                                                nch, nalm);
      JCK(cudaGetLastError());
      if ((rc = sht_synthesis(c, c->tmp_maps, nch, false))) return rc;
      JCK(cudaMemcpyAsync(out + (long long)c0 * c->npix, c->tmp_maps, sizeof(float) * nch * c->npix,
                          cudaMemcpyDeviceToHost, c->stream));
    }
    JCK(cudaStreamSynchronize(c->stream));
  }
  return GETHI_OK;
}

extern "C" int joint_gpu_map2alm(joint_ctx *c, const float *maps, int n_maps, float *alms)
{
  return sht_api(c, maps, n_maps, alms, true);
}

extern "C" int joint_gpu_alm2map(joint_ctx *c, const float *alms, int n_maps, float *maps)
{
  return sht_api(c, alms, n_maps, maps, false);
}
