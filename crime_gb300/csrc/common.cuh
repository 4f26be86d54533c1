// Device-side building blocks shared by the GetHI kernels: complex helpers,
// compile-time twiddles, register-resident small DFTs, the Stockham stage
// driver used by every FFT pass, Philox4x32-10 and the kernel configuration.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include <type_traits>

namespace gethi {

constexpr int kNZ = 5001;
constexpr int kNSUB = 10;
constexpr double kNU21 = 1420.40575177;

// ---------------------------------------------------------------------------
// complex helpers
// ---------------------------------------------------------------------------
__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ float2 cmul(float2 a, float2 b)
{
  return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ float2 cscale(float2 a, float s) { return make_float2(a.x * s, a.y * s); }
__device__ __forceinline__ float2 cmul_i(float2 a) { return make_float2(-a.y, a.x); }  // i*a
__device__ __forceinline__ float2 conjf2(float2 a) { return make_float2(a.x, -a.y); }

// ---------------------------------------------------------------------------
// compile-time twiddles exp(+2 pi i K/N); quarter turns exact
// ---------------------------------------------------------------------------
constexpr double ce_pi = 3.14159265358979323846;
constexpr double ce_sin(double x)  // |x| <= pi
{
  double term = x, sum = x;
  for (int n = 1; n < 30; n++) {
    term *= -x * x / ((2.0 * n) * (2.0 * n + 1));
    sum += term;
  }
  return sum;
}
constexpr double ce_cos(double x)
{
  double term = 1, sum = 1;
  for (int n = 1; n < 30; n++) {
    term *= -x * x / ((2.0 * n - 1) * (2.0 * n));
    sum += term;
  }
  return sum;
}
template <int K, int N>
struct Tw {
  static constexpr int k = ((K % N) + N) % N;
  static constexpr bool quarter = (4 * k) % N == 0;
  static constexpr int q = quarter ? (4 * k) / N : 0;
  static constexpr double ang = 2 * ce_pi * (2 * k > N ? k - N : k) / N;
  static constexpr float re = quarter ? (q == 0 ? 1.f : (q == 2 ? -1.f : 0.f)) : (float)ce_cos(ang);
  static constexpr float im = quarter ? (q == 1 ? 1.f : (q == 3 ? -1.f : 0.f)) : (float)ce_sin(ang);
};

template <class W>
__device__ __forceinline__ float2 cmul_tw(float2 v)
{
  if constexpr (W::quarter) {
    if constexpr (W::q == 0) return v;
    else if constexpr (W::q == 1) return make_float2(-v.y, v.x);
    else if constexpr (W::q == 2) return make_float2(-v.x, -v.y);
    else return make_float2(v.y, -v.x);
  } else {
    return make_float2(v.x * W::re - v.y * W::im, v.x * W::im + v.y * W::re);
  }
}

template <int B, int E, class F>
__device__ __forceinline__ void static_for(F &&f)
{
  if constexpr (B < E) {
    f(std::integral_constant<int, B>{});
    static_for<B + 1, E>(f);
  }
}

// ---------------------------------------------------------------------------
// inverse (sign +1) DFTs on registers, natural order in and out
// ---------------------------------------------------------------------------
template <int R>
__device__ __forceinline__ void idft(float2 *x);

template <int A, int B>
__device__ __forceinline__ void idft_ct(float2 *x)
{
  // n = a + A b, k = k1 + B k2:  X[k] = sum_a w_A^{a k2} w_N^{a k1} sum_b w_B^{b k1} x[a + A b]
  constexpr int N = A * B;
  float2 y[N];
  static_for<0, A>([&](auto ai) {
    constexpr int a = decltype(ai)::value;
    float2 t[B];
    static_for<0, B>([&](auto bi) { t[decltype(bi)::value] = x[a + A * decltype(bi)::value]; });
    idft<B>(t);
    static_for<0, B>([&](auto ki) {
      constexpr int k1 = decltype(ki)::value;
      y[a * B + k1] = cmul_tw<Tw<a * k1, N>>(t[k1]);
    });
  });
  static_for<0, B>([&](auto ki) {
    constexpr int k1 = decltype(ki)::value;
    float2 t[A];
    static_for<0, A>([&](auto ai) { t[decltype(ai)::value] = y[decltype(ai)::value * B + k1]; });
    idft<A>(t);
    static_for<0, A>([&](auto ai) { x[k1 + B * decltype(ai)::value] = t[decltype(ai)::value]; });
  });
}

template <int R>
__device__ __forceinline__ void idft(float2 *x)
{
  if constexpr (R == 1) {
  } else if constexpr (R == 2) {
    float2 a = x[0], b = x[1];
    x[0] = cadd(a, b);
    x[1] = csub(a, b);
  } else if constexpr (R == 3) {
    const float s3 = 0.86602540378443864676f;
    float2 s = cadd(x[1], x[2]), d = csub(x[1], x[2]);
    float2 m = make_float2(x[0].x - 0.5f * s.x, x[0].y - 0.5f * s.y);
    float2 id = make_float2(-s3 * d.y, s3 * d.x);
    x[0] = cadd(x[0], s);
    x[1] = cadd(m, id);
    x[2] = csub(m, id);
  } else if constexpr (R == 4) {
    float2 a0 = cadd(x[0], x[2]), a1 = csub(x[0], x[2]);
    float2 b0 = cadd(x[1], x[3]), b1 = csub(x[1], x[3]);
    x[0] = cadd(a0, b0);
    x[2] = csub(a0, b0);
    x[1] = cadd(a1, cmul_i(b1));
    x[3] = csub(a1, cmul_i(b1));
  } else if constexpr (R == 6) {
    idft_ct<2, 3>(x);
  } else if constexpr (R == 8) {
    idft_ct<2, 4>(x);
  } else if constexpr (R == 12) {
    idft_ct<4, 3>(x);
  } else if constexpr (R == 16) {
    idft_ct<4, 4>(x);
  } else if constexpr (R == 24) {
    idft_ct<8, 3>(x);
  } else if constexpr (R == 32) {
    idft_ct<4, 8>(x);
  } else {
    static_assert(R == 0, "unsupported radix");
  }
}

// ---------------------------------------------------------------------------
// Stockham autosort stages.  A length-L transform is held by T = L/P threads,
// P points each.  Stage s (radix R, Ns = product of the earlier radices) lets
// thread t run butterflies b = t + T j (j < P/R) on elements b + (L/R) r and
// writes them to (b/Ns) Ns R + b%Ns + r Ns.  On entry v[j R0 + r] must hold
// x[t + T j + (L/R0) r]; on exit v[j Rl + r] holds X[t + T j + (L/Rl) r].
// Between stages the points go through shared memory: element n lives at
// sm[n * ss].  tw is the table exp(+2 pi i m / L), m < L.
// ---------------------------------------------------------------------------
template <int... R>
struct Radices {};

template <int First, int... Rest>
constexpr int first_radix() { return First; }

// shared-memory slot of element n: n*ss, plus one skew slot per 16 elements
// when SKEW (row transforms, ss = 1) so that the stride-R writes of the first
// stage fall in different banks
template <bool SKEW>
__device__ __forceinline__ int sm_slot(int n, int ss) { return SKEW ? n + (n >> 4) : n * ss; }

template <int L, int P, bool SKEW, int Ns, int R, int... Rest>
__device__ __forceinline__ void stockham(float2 *v, float2 *sm, int ss, int t, const float2 *__restrict__ tw)
{
  constexpr int T = L / P;
  constexpr int NB = P / R;
  static_assert(P % R == 0, "radix must divide the points per thread");
#pragma unroll
  for (int j = 0; j < NB; j++) {
    if constexpr (Ns > 1) {
      const int b = t + T * j;
      const int k = b % Ns;
#pragma unroll
      for (int r = 1; r < R; r++) v[j * R + r] = cmul(v[j * R + r], __ldg(&tw[r * k * (L / (Ns * R))]));
    }
    idft<R>(&v[j * R]);
  }
  if constexpr (sizeof...(Rest) > 0) {
    constexpr int R2 = first_radix<Rest...>();
    __syncthreads();
#pragma unroll
    for (int j = 0; j < NB; j++) {
      const int b = t + T * j;
      const int base = (b / Ns) * Ns * R + (b % Ns);
#pragma unroll
      for (int r = 0; r < R; r++) sm[sm_slot<SKEW>(base + r * Ns, ss)] = v[j * R + r];
    }
    __syncthreads();
#pragma unroll
    for (int j = 0; j < P / R2; j++)
#pragma unroll
      for (int r = 0; r < R2; r++) v[j * R2 + r] = sm[sm_slot<SKEW>(t + T * j + (L / R2) * r, ss)];
    stockham<L, P, SKEW, Ns * R, Rest...>(v, sm, ss, t, tw);
  }
}

template <int L, int P, bool SKEW = false, int... R>
__device__ __forceinline__ void stockham_run(float2 *v, float2 *sm, int ss, int t, const float2 *__restrict__ tw,
                                             Radices<R...>)
{
  stockham<L, P, SKEW, 1, R...>(v, sm, ss, t, tw);
}

// shared-memory slots one transform of length L occupies
template <int L, bool SKEW>
constexpr int sm_len() { return SKEW ? L + L / 16 : L; }

template <int... R>
constexpr int radix_first(Radices<R...>) { return first_radix<R...>(); }
template <int... R>
constexpr int radix_last(Radices<R...>)
{
  int v[] = {R...};
  return v[sizeof...(R) - 1];
}

// ---------------------------------------------------------------------------
// Philox4x32-10 (Salmon et al., SC'11)
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint4 philox4x32_10(uint4 c, uint2 k)
{
#pragma unroll
  for (int r = 0; r < 10; r++) {
    uint32_t hi0 = __umulhi(0xD2511F53u, c.x), lo0 = 0xD2511F53u * c.x;
    uint32_t hi1 = __umulhi(0xCD9E8D57u, c.z), lo1 = 0xCD9E8D57u * c.z;
    c = make_uint4(hi1 ^ c.y ^ k.x, lo1, hi0 ^ c.w ^ k.y, lo0);
    k.x += 0x9E3779B9u;
    k.y += 0xBB67AE85u;
  }
  return c;
}

// ---------------------------------------------------------------------------
// kernel configuration (passed by value)
// ---------------------------------------------------------------------------
struct DevCfg {
  int n;           // n_grid
  int m;           // n/2: complex row length of the split half spectrum
  double l_box, dx, pos_obs;
  float dxf, pos_obsf;
  // P(k)
  const float *logk_f, *pk_f;
  int numk;
  float logkmin, logkmax, idlogk, n_scal;
  float dk, idk3, r2_smooth;
  int do_smoothing;
  float norm;      // (sqrt(2 pi)/L)^3, src/fourier.c:403
  float vfac;      // f0 * H0, src/fourier.c:255
  uint32_t seed;
  // distance / growth tables, FP64 and FP32 copies
  const double *z_r2z, *r_r2z, *gd, *gv;
  const float *z_r2z_f, *gd_f, *gv_f;
  double glob_idr, r_tab_max;
  float glob_idr_f, r_tab_max_f;
  // per table interval i (shell_line_entry): the slope dz/dR per cell and the
  // largest distance of z(R) from that interval's line within a sub-sample
  // radius of the interval
  const float *z_lin_g, *z_lin_e;
  // shells and pixels
  int n_nu, regular_nu;
  long nside, npix;
  double nu_min, nu_max, inv_dnu;
  const double *nu_edges;  // n_nu + 1 edges
  const float *nu_edges_f; // FP32 copy for the fast path
  const float *prefac;     // n_nu
  // sub-samples (src/pixelize.c:157-164)
  double xs[kNSUB], ys[kNSUB], zs[kNSUB];
  // model switches
  int bias_const, do_rsd;
  float b_HI;
  float sigma2;    // Gaussian variance (after the density FFT)
  float mass_prefac;
  // Gaussianised spectrum on the grid (gaussianise=1): P_G of mode (kz,ky,kx)
  // at pg[(kz n + ky) n + kx], smoothing included; nullptr = table lookup
  const float *pg;
  // tensor-core split-precision column passes (fft_precision=tc_split): DFT
  // operand tables, twiddles, error flag; tc_bmat == nullptr selects FP32
  const uint4 *tc_bmat;
  const float2 *tc_tw;
  int *tc_err;
  // launch shapes chosen by the autotuner (0 = built-in choice): cells per
  // projection tile along z / 4, and the half-width column tile of the FP32 passes
  int proj_zsteps;
  int col_variant;
  // double-float (hi, lo) copies for the refinement of uncertain keys
  // (z_r2z_df == nullptr: uncertain keys go straight to FP64)
  const float2 *z_r2z_df, *r_r2z_df, *nu_edges_df;
  float2 dx_df, pos_obs_df, glob_idr_df, inv_dnu_df, nu_min_df;
  float2 xs_df[10], ys_df[10], zs_df[10];
};

// wave number of grid index i (src/fourier.c:264-283): Nyquist is +n/2
__device__ __forceinline__ float kval(int i, int n, float dk) { return (2 * i <= n) ? i * dk : -(n - i) * dk; }

}  // namespace gethi
