// stockham.cuh -- register-resident power-of-two FFTs for thread groups of a block
#pragma once
#include <utility>

#include "common.cuh"

namespace stockham {

// Power-of-two complex FFTs in the self-sorting (Stockham) form of Govindaraju
// et al., "High performance discrete Fourier transforms on graphics processors"
// (SC08): pass p of radix R, with Ns the product of the radices before it,
// takes butterfly j's inputs x[j + r n/R], multiplies them by
// e^{sign 2 pi i r (j mod Ns)/(Ns R)}, does an R-point DFT in registers and
// stores V[s] at (j / Ns) Ns R + (j mod Ns) + s Ns: natural order in and out.
// A sequence of n points is held by TS = max(1, n/16) threads with 16 points
// each (n when n < 16).  Thread t's slot i is point t + TS i at the input of the
// first pass and at the output of the last, so loads from and stores to global
// memory are coalesced, and two FFTs whose adjoining passes have the same radix
// hand over in registers (Bluestein's forward and inverse transforms).  The
// radices are 16 but for one pass of 2^(log2 n mod 4): the first pass of the
// forward plan, the last of the reversed plan.  Between passes the points go
// through shared memory at index i + i/16 (one float2 of padding per 16 points),
// which keeps the 8-byte accesses of every pass free of bank conflicts.  The
// twiddles come from tw2, which holds e^{+2 pi i x/L} at tw2[L + x] (x < L) for
// every power of two L up to n; the inverse sign conjugates them.

using gethi::cadd;
using gethi::cmul;
using gethi::csub;
__device__ __forceinline__ int spad(int i) { return i + (i >> 4); }
__host__ __device__ constexpr int padded_len(int n) { return n + (n >> 4); }
__host__ __device__ constexpr int brev_bits(int v, int bits)
{
  int r = 0;
  for (int b = 0; b < bits; b++) r |= ((v >> b) & 1) << (bits - 1 - b);
  return r;
}

// v e^{SIGN 2 pi i k/16}, k in [0, 8) (a constant once the callers' loops are unrolled)
template <int SIGN>
__device__ __forceinline__ float2 rot16(float2 v, int k)
{
  constexpr float c1 = 0.92387953251128674f, s1 = 0.38268343236508977f, h = 0.70710678118654752f;
  if (k == 0) return v;
  if (k == 4) return SIGN > 0 ? make_float2(-v.y, v.x) : make_float2(v.y, -v.x);
  float c, s;
  switch (k) {
    case 1: c = c1; s = s1; break;
    case 2: c = h; s = h; break;
    case 3: c = s1; s = c1; break;
    case 5: c = -s1; s = c1; break;
    case 6: c = -h; s = h; break;
    default: c = -c1; s = s1; break;
  }
  if (SIGN < 0) s = -s;
  return make_float2(v.x * c - v.y * s, v.x * s + v.y * c);
}

template <int V, int BITS>
constexpr int kBrev = brev_bits(V, BITS);
// a[s] = a[bit-reverse(s)], every index a compile-time constant
template <int R, int... S>
__device__ __forceinline__ void bit_reverse_regs(float2 (&a)[R], std::integer_sequence<int, S...>)
{
  constexpr int LR = R == 2 ? 1 : R == 4 ? 2 : R == 8 ? 3 : 4;
  const float2 o[R] = {a[kBrev<S, LR>]...};
#pragma unroll
  for (int s = 0; s < R; s++) a[s] = o[s];
}

// R-point DFT in registers, V[s] = sum_r a[r] e^{SIGN 2 pi i r s/R}: radix-2
// decimation in frequency, then the bit-reversal as a renaming of registers
template <int R, int SIGN>
__device__ __forceinline__ void dft_reg(float2 (&a)[R])
{
  constexpr int LR = R == 2 ? 1 : R == 4 ? 2 : R == 8 ? 3 : 4;
#pragma unroll
  for (int lh = LR - 1; lh >= 0; lh--) {
    const int H = 1 << lh;
#pragma unroll
    for (int b = 0; b < R; b += 2 * H)
#pragma unroll
      for (int i = 0; i < H; i++) {
        const float2 x = a[b + i], y = a[b + i + H];
        a[b + i] = cadd(x, y);
        a[b + i + H] = rot16<SIGN>(csub(x, y), i * (8 >> lh));  // e^{SIGN 2 pi i i/(2H)}
      }
  }
  bit_reverse_regs(a, std::make_integer_sequence<int, R>{});
}

// the twiddles and DFTs of one pass for the G = (points per thread)/R butterflies
// j = t + g TS of this thread, in place in the slots g + r G
template <int R, int G, int SIGN>
__device__ __forceinline__ void stockham_pass(float2 (&u)[16], int t, int TS, int Ns, const float2 *__restrict__ tw2)
{
#pragma unroll
  for (int g = 0; g < G; g++) {
    const int j = t + g * TS, k = j & (Ns - 1);
    float2 a[R];
#pragma unroll
    for (int r = 0; r < R; r++) a[r] = u[g + r * G];
    if (Ns > 1) {  // w[r] = e^{SIGN 2 pi i r k/(Ns R)}: powers of two from the table, the rest as products
      const float2 *tw = tw2 + Ns * R;
      float2 w[R];
#pragma unroll
      for (int r = 1; r < R; r++) {
        if ((r & (r - 1)) == 0) {
          const float2 v = __ldg(tw + r * k);
          w[r] = make_float2(v.x, SIGN > 0 ? v.y : -v.y);
        } else {
          w[r] = cmul(w[r - (r & -r)], w[r & -r]);
        }
        a[r] = cmul(a[r], w[r]);
      }
    }
    dft_reg<R, SIGN>(a);
#pragma unroll
    for (int s = 0; s < R; s++) u[g + s * G] = a[s];
  }
}

// the outputs of a pass that is not the last into shared memory
template <int R, int G>
__device__ __forceinline__ void stockham_store(const float2 (&u)[16], float2 *s, int t, int TS, int Ns)
{
#pragma unroll
  for (int g = 0; g < G; g++) {
    const int j = t + g * TS, base = (j & ~(Ns - 1)) * R + (j & (Ns - 1));
#pragma unroll
    for (int r = 0; r < R; r++) s[spad(base + r * Ns)] = u[g + r * G];
  }
}

// a sequence's points from shared memory into slot order (points beyond n: zero)
__device__ __forceinline__ void slots_load(float2 (&u)[16], const float2 *s, int n, int t, int TS)
{
#pragma unroll
  for (int i = 0; i < 16; i++) {
    const int k = t + TS * i;
    u[i] = k < n ? s[spad(k)] : make_float2(0.f, 0.f);
  }
}

// FFT of the n = 2^L points of one sequence (s: its shared-memory rows) held by
// TS threads, input and output in u in slot order.  Every thread of the block
// calls this (barriers inside); `active` marks the threads that hold a sequence.
template <int SIGN, bool REV>
__device__ __forceinline__ void fft_run(float2 (&u)[16], float2 *s, const float2 *__restrict__ tw2, int n, int L,
                                        int t, int TS, bool active)
{
  if (L <= 4) {  // one pass of radix n, one thread per sequence
    if (!active) return;
    switch (L) {
      case 1: stockham_pass<2, 1, SIGN>(u, t, 1, 1, tw2); break;
      case 2: stockham_pass<4, 1, SIGN>(u, t, 1, 1, tw2); break;
      case 3: stockham_pass<8, 1, SIGN>(u, t, 1, 1, tw2); break;
      case 4: stockham_pass<16, 1, SIGN>(u, t, 1, 1, tw2); break;
      default: break;
    }
    return;
  }
  const int P = (L + 3) >> 2, r0 = L - 4 * (P - 1);
  int Ns = 1;
  for (int p = 0; p < P; p++) {
    const int lr = (REV ? p == P - 1 : p == 0) ? r0 : 4;
    if (active && p > 0) {
#pragma unroll
      for (int i = 0; i < 16; i++) u[i] = s[spad(t + TS * i)];
    }
    if (active) {
      switch (lr) {
        case 1: stockham_pass<2, 8, SIGN>(u, t, TS, Ns, tw2); break;
        case 2: stockham_pass<4, 4, SIGN>(u, t, TS, Ns, tw2); break;
        case 3: stockham_pass<8, 2, SIGN>(u, t, TS, Ns, tw2); break;
        default: stockham_pass<16, 1, SIGN>(u, t, TS, Ns, tw2); break;
      }
    }
    if (p < P - 1) {
      __syncthreads();  // every read of this pass is done
      if (active) {
        switch (lr) {
          case 1: stockham_store<2, 8>(u, s, t, TS, Ns); break;
          case 2: stockham_store<4, 4>(u, s, t, TS, Ns); break;
          case 3: stockham_store<8, 2>(u, s, t, TS, Ns); break;
          default: stockham_store<16, 1>(u, s, t, TS, Ns); break;
        }
      }
      __syncthreads();
    }
    Ns <<= lr;
  }
}

// log2 of the radix of pass p in the plan for 2^L points (L > 4), and the product
// Ns of the radices before it
__host__ __device__ constexpr int plan_lr(int L, int p, bool rev)
{
  return (rev ? p == (L + 3) / 4 - 1 : p == 0) ? L - 4 * ((L + 3) / 4 - 1) : 4;
}
__host__ __device__ constexpr int plan_ns(int L, int p, bool rev)
{
  int ns = 1;
  for (int i = 0; i < p; i++) ns <<= plan_lr(L, i, rev);
  return ns;
}

// pass P0 and the following ones of fft_fixed
template <int L, int SIGN, bool REV, int P0>
__device__ __forceinline__ void fixed_passes(float2 (&u)[16], float2 *s, const float2 *__restrict__ tw2, int t,
                                             bool active)
{
  constexpr int P = (L + 3) / 4, TS = 1 << (L - 4);
  if constexpr (P0 < P) {
    constexpr int lr = plan_lr(L, P0, REV), R = 1 << lr, G = 16 / R, Ns = plan_ns(L, P0, REV);
    if (active && P0 > 0) {
#pragma unroll
      for (int i = 0; i < 16; i++) u[i] = s[spad(t + TS * i)];
    }
    if (active) stockham_pass<R, G, SIGN>(u, t, TS, Ns, tw2);
    if constexpr (P0 < P - 1) {
      __syncthreads();
      if (active) stockham_store<R, G>(u, s, t, TS, Ns);
      __syncthreads();
    }
    fixed_passes<L, SIGN, REV, P0 + 1>(u, s, tw2, t, active);
  }
}

// fft_run for a compile-time size 2^L (L > 4): the plan's radices, Ns and the
// threads per sequence are constants, so the shared-memory and twiddle addresses
// reduce to per-thread bases plus immediate offsets
template <int L, int SIGN, bool REV>
__device__ __forceinline__ void fft_fixed(float2 (&u)[16], float2 *s, const float2 *__restrict__ tw2, int t,
                                          bool active)
{
  static_assert(L > 4 && L <= 13, "fft_fixed: 32 .. 8192 points");
  fixed_passes<L, SIGN, REV, 0>(u, s, tw2, t, active);
}

// fft_run with the sizes 2^9 .. 2^13 (the equatorial rings and the larger
// Bluestein convolutions) dispatched to fft_fixed
template <int SIGN, bool REV>
__device__ __forceinline__ void fft_any(float2 (&u)[16], float2 *s, const float2 *__restrict__ tw2, int n, int L, int t,
                                        int TS, bool active)
{
  switch (L) {
    case 9: fft_fixed<9, SIGN, REV>(u, s, tw2, t, active); break;
    case 10: fft_fixed<10, SIGN, REV>(u, s, tw2, t, active); break;
    case 11: fft_fixed<11, SIGN, REV>(u, s, tw2, t, active); break;
    case 12: fft_fixed<12, SIGN, REV>(u, s, tw2, t, active); break;
    case 13: fft_fixed<13, SIGN, REV>(u, s, tw2, t, active); break;
    default: fft_run<SIGN, REV>(u, s, tw2, n, L, t, TS, active); break;
  }
}

}  // namespace stockham
