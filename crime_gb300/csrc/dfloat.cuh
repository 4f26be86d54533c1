// Double-float arithmetic: a value is hi + lo with two FP32 numbers (|lo| <=
// ulp(hi)/2), about 48 significant bits.  Built on the error-free transforms
// TwoSum (Knuth), FastTwoSum (Dekker) and the FMA-based TwoProd, as in
// Dekker (1971) and the QD library of Hida, Li & Bailey (2001).  Every step is
// an explicitly rounded intrinsic, so the compiler cannot contract or reorder
// it.  GB300 issues FP32 at 64x its FP64 rate; these ~10-instruction operations
// stand in for FP64 where 48 bits suffice.
#pragma once

namespace gethi {

struct df {
  float hi, lo;
};

__host__ __device__ constexpr df df_const(double v) { return {(float)v, (float)(v - (double)(float)v)}; }
__device__ __forceinline__ df df_f(float a) { return {a, 0.f}; }
__device__ __forceinline__ df df_of(float2 v) { return {v.x, v.y}; }

__device__ __forceinline__ df two_sum(float a, float b)
{
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  return {s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb))};
}
__device__ __forceinline__ df fast_two_sum(float a, float b)  // |a| >= |b|
{
  const float s = __fadd_rn(a, b);
  return {s, __fsub_rn(b, __fsub_rn(s, a))};
}
__device__ __forceinline__ df two_prod(float a, float b)
{
  const float p = __fmul_rn(a, b);
  return {p, __fmaf_rn(a, b, -p)};
}
__device__ __forceinline__ df df_neg(df a) { return {-a.hi, -a.lo}; }
__device__ __forceinline__ df df_abs(df a) { return a.hi < 0.f ? df_neg(a) : a; }
__device__ __forceinline__ df df_add(df a, df b)
{
  const df s = two_sum(a.hi, b.hi), t = two_sum(a.lo, b.lo);
  const df v = fast_two_sum(s.hi, __fadd_rn(s.lo, t.hi));
  return fast_two_sum(v.hi, __fadd_rn(t.lo, v.lo));
}
__device__ __forceinline__ df df_sub(df a, df b) { return df_add(a, df_neg(b)); }
__device__ __forceinline__ df df_mul(df a, df b)
{
  const df p = two_prod(a.hi, b.hi);
  return fast_two_sum(p.hi, __fadd_rn(p.lo, __fmaf_rn(a.hi, b.lo, __fmul_rn(a.lo, b.hi))));
}
__device__ __forceinline__ df df_mul_f(df a, float b)
{
  const df p = two_prod(a.hi, b);
  return fast_two_sum(p.hi, __fmaf_rn(a.lo, b, p.lo));
}
__device__ __forceinline__ df df_div(df a, df b)
{
  const float q1 = __fdiv_rn(a.hi, b.hi);
  df r = df_sub(a, df_mul_f(b, q1));
  const float q2 = __fdiv_rn(r.hi, b.hi);
  r = df_sub(r, df_mul_f(b, q2));
  const float q3 = __fdiv_rn(r.hi, b.hi);
  return df_add(fast_two_sum(q1, q2), df_f(q3));
}
__device__ __forceinline__ df df_sqrt(df a)  // a > 0
{
  const float s = __fsqrt_rn(a.hi);
  const df r = df_sub(a, two_prod(s, s));
  return fast_two_sum(s, __fdiv_rn(r.hi, __fmul_rn(2.f, s)));
}

// a >= b on the full values (the high words alone can tie when the values differ)
__device__ __forceinline__ bool df_ge(df a, df b) { return a.hi > b.hi || (a.hi == b.hi && a.lo >= b.lo); }

// floor of v for |v| < 2^23; unc is set when v lies within m of an integer
__device__ __forceinline__ int df_floor(df v, float m, bool &unc)
{
  float f = floorf(v.hi);
  float d = __fadd_rn(__fsub_rn(v.hi, f), v.lo);  // v - f; v.hi - f is exact
  if (d < 0.f) {
    f -= 1.f;
    d += 1.f;
  } else if (d >= 1.f) {
    f += 1.f;
    d -= 1.f;
  }
  if (d < m || 1.f - d < m) unc = true;
  return (int)f;
}

// atan(t), t in [0, 1]: atan(c) + atan((t - c)/(1 + t c)) with c = j/8 nearest
// to t, the second term by its Taylor series (|s| <= 1/16, 8 terms: remainder
// below 1e-21)
__device__ __forceinline__ df df_atan01(df t)
{
  constexpr df kA[9] = {df_const(0.0), df_const(0.12435499454676144), df_const(0.24497866312686414),
                        df_const(0.35877067027057225), df_const(0.4636476090008061), df_const(0.5585993153435624),
                        df_const(0.6435011087932844), df_const(0.7188299996216245), df_const(0.7853981633974483)};
  constexpr df c15 = df_const(-1.0 / 15), c13 = df_const(1.0 / 13), c11 = df_const(-1.0 / 11),
               c9 = df_const(1.0 / 9), c7 = df_const(-1.0 / 7), c5 = df_const(1.0 / 5), c3 = df_const(-1.0 / 3);
  const int j = min(max((int)rintf(8.f * t.hi), 0), 8);
  const float cj = 0.125f * (float)j;  // exact
  const df s = df_div(df_sub(t, df_f(cj)), df_add(df_f(1.f), df_mul_f(t, cj)));
  const df u = df_mul(s, s);
  df p = c15;
  p = df_add(c13, df_mul(u, p));
  p = df_add(c11, df_mul(u, p));
  p = df_add(c9, df_mul(u, p));
  p = df_add(c7, df_mul(u, p));
  p = df_add(c5, df_mul(u, p));
  p = df_add(c3, df_mul(u, p));
  p = df_add(df_f(1.f), df_mul(u, p));
  df a = kA[0];
#pragma unroll
  for (int k = 1; k < 9; k++)
    if (k == j) a = kA[k];
  return df_add(a, df_mul(s, p));
}

// atan2(y, x) in (-pi, pi]
__device__ __forceinline__ df df_atan2(df y, df x)
{
  const df ax = df_abs(x), ay = df_abs(y);
  const bool swap = ay.hi > ax.hi || (ay.hi == ax.hi && ay.lo > ax.lo);
  df a = (ax.hi == 0.f && ay.hi == 0.f) ? df_f(0.f) : df_atan01(swap ? df_div(ax, ay) : df_div(ay, ax));
  constexpr df kHalfPi = df_const(1.5707963267948966), kPi = df_const(3.141592653589793);
  if (swap) a = df_sub(kHalfPi, a);
  if (x.hi < 0.f) a = df_sub(kPi, a);
  if (y.hi < 0.f) a = df_neg(a);
  return a;
}

}  // namespace gethi
