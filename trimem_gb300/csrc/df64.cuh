// Double-float ("double-word") arithmetic on the FP32 pipe.
//
// A value is the unevaluated sum hi + lo of two floats with |lo| <= ulp(hi)/2,
// about 48 significant bits.  The operations are the error-free
// transformations TwoSum / Fast2Sum / TwoProd (with FMA) and the double-word
// algorithms of Joldes, Muller & Popescu, "Tight and rigorous error bounds
// for basic building blocks of double-word arithmetic", ACM TOMS 44 (2017):
// AccurateDWPlusDW (relative error <= 3u^2), DWTimesDW with FMA (<= 5u^2),
// DWDivDW and a Newton step for the square root; u = 2^-24.  Every float
// operation uses an explicitly rounded intrinsic so no FMA contraction can
// change the error-free transformations.
#pragma once

#include <cuda_runtime.h>

namespace tmg {

struct df {
  float hi, lo;
};

__device__ __forceinline__ df df_make(float h) { return {h, 0.0f}; }
__device__ __forceinline__ df df_from(double x) {
  float h = (float)x;
  return {h, (float)(x - (double)h)};
}
__device__ __forceinline__ double df_to(df a) { return (double)a.hi + (double)a.lo; }

__device__ __forceinline__ df two_sum(float a, float b) {
  float s = __fadd_rn(a, b);
  float bb = __fsub_rn(s, a);
  float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return {s, e};
}
__device__ __forceinline__ df fast_two_sum(float a, float b) {  // |a| >= |b|
  float s = __fadd_rn(a, b);
  return {s, __fsub_rn(b, __fsub_rn(s, a))};
}
__device__ __forceinline__ df two_prod(float a, float b) {
  float p = __fmul_rn(a, b);
  return {p, __fmaf_rn(a, b, -p)};
}

__device__ __forceinline__ df operator+(df x, df y) {
  df s = two_sum(x.hi, y.hi);
  df t = two_sum(x.lo, y.lo);
  float c = __fadd_rn(s.lo, t.hi);
  df v = fast_two_sum(s.hi, c);
  float w = __fadd_rn(t.lo, v.lo);
  return fast_two_sum(v.hi, w);
}
__device__ __forceinline__ df operator-(df x) { return {-x.hi, -x.lo}; }
__device__ __forceinline__ df operator-(df x, df y) { return x + (-y); }
__device__ __forceinline__ df operator*(df x, df y) {
  df c = two_prod(x.hi, y.hi);
  float t = __fmul_rn(x.lo, y.lo);
  t = __fmaf_rn(x.hi, y.lo, t);
  t = __fmaf_rn(x.lo, y.hi, t);
  return fast_two_sum(c.hi, __fadd_rn(c.lo, t));
}
__device__ __forceinline__ df operator*(df x, float b) {
  df c = two_prod(x.hi, b);
  return fast_two_sum(c.hi, __fmaf_rn(x.lo, b, c.lo));
}
__device__ __forceinline__ df operator*(float b, df x) { return x * b; }
__device__ __forceinline__ df& operator+=(df& a, df b) { return a = a + b; }
__device__ __forceinline__ df& operator-=(df& a, df b) { return a = a - b; }
// exact scaling by a power of two
__device__ __forceinline__ df ldexp2(df a, float p2) { return {a.hi * p2, a.lo * p2}; }

__device__ __forceinline__ df operator/(df x, df y) {
  float th = __fdiv_rn(x.hi, y.hi);
  df r = y * th;
  df p = x - r;
  float d = __fdiv_rn(p.hi, y.hi);
  return fast_two_sum(th, d);
}
__device__ __forceinline__ df df_sqrt(df x) {
  if (x.hi <= 0.0f) return {0.0f, 0.0f};
  float s = __fsqrt_rn(x.hi);
  df ss = two_prod(s, s);
  float d = __fdiv_rn(__fadd_rn(__fsub_rn(__fsub_rn(x.hi, ss.hi), ss.lo), x.lo), __fmul_rn(2.0f, s));
  return fast_two_sum(s, d);
}
__device__ __forceinline__ bool df_lt0(df a) { return a.hi < 0.0f || (a.hi == 0.0f && a.lo < 0.0f); }

struct df3 {
  df x, y, z;
};
__device__ __forceinline__ df3 operator+(const df3& a, const df3& b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ df3 operator-(const df3& a, const df3& b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ df3 operator*(df s, const df3& a) { return {s * a.x, s * a.y, s * a.z}; }
__device__ __forceinline__ df3& operator+=(df3& a, const df3& b) {
  a.x += b.x;
  a.y += b.y;
  a.z += b.z;
  return a;
}
__device__ __forceinline__ df ddot(const df3& a, const df3& b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ df3 dcross(const df3& a, const df3& b) {
  return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}

// sin and cos of a float angle |t| <= 0.8 to double-word accuracy (Taylor,
// terms to t^19 / t^18)
__device__ __forceinline__ void df_sincos_small(float t, df* s, df* c) {
  df x = df_make(t);
  df x2 = two_prod(t, t);
  // Horner in x^2; coefficients (-1)^k/(2k+1)! and (-1)^k/(2k)! as
  // double-words (hi = float(c), lo = float(c - hi))
  const df sc[10] = {{1.000000000e+00f, 0.000000000e+00f}, {-1.666666716e-01f, 4.967053879e-09f}, {8.333333768e-03f, -4.346172033e-10f}, {-1.984127011e-04f, 2.725596875e-12f}, {2.755731884e-06f, 3.793571224e-14f}, {-2.505210794e-08f, -4.417623045e-16f}, {1.605904437e-10f, -5.352526512e-18f}, {-7.647163610e-13f, -1.220071047e-20f}, {2.811457359e-15f, -1.046208474e-22f}, {-8.220635078e-18f, -1.681478097e-25f}};
  const df cc[10] = {{1.000000000e+00f, 0.000000000e+00f}, {-5.000000000e-01f, 0.000000000e+00f}, {4.166666791e-02f, -1.241763470e-09f}, {-1.388888923e-03f, 3.363109444e-11f}, {2.480158764e-05f, -3.406996094e-13f}, {-2.755731998e-07f, 7.575112209e-15f}, {2.087675588e-09f, 1.108283981e-16f}, {-1.147074536e-11f, -2.372207689e-19f}, {4.779477256e-14f, 7.625444044e-22f}, {-1.561920681e-16f, -1.540447147e-24f}};
  df ps = sc[9], pc = cc[9];
#pragma unroll
  for (int k = 8; k >= 0; --k) {
    ps = ps * x2 + sc[k];
    pc = pc * x2 + cc[k];
  }
  *s = ps * x;
  *c = pc;
}

// e^x for x <= 0 to double-word accuracy (0 below -80, where e^x < 2e-35):
// x = k ln2 + r with a three-part Cody-Waite split of ln2 (the first part
// has 16 significant bits, so k * part is exact), e^r = (e^(r/16))^16 with
// e^(r/16) from its Taylor polynomial of degree 8 (|r/16| < 0.022,
// truncation < 3e-21), then the exact scaling by 2^k.
__device__ __forceinline__ df df_exp_nonpos(df x) {
  if (!(x.hi >= -80.0f)) return df_make(0.0f);
  const float L2H = 0.693145751953125f, L2M = 1.428606765e-06f, L2L = 5.497923148e-14f;
  const float k = rintf(__fmul_rn(x.hi, 1.44269504f));
  df r = x + df_make(__fmul_rn(-k, L2H));
  r = r - two_prod(k, L2M);
  r = r - df_make(__fmul_rn(k, L2L));
  r = ldexp2(r, 0.0625f);
  const df c[9] = {{1.000000000e+00f, 0.000000000e+00f}, {1.000000000e+00f, 0.000000000e+00f},
                   {5.000000000e-01f, 0.000000000e+00f}, {1.666666716e-01f, -4.967053879e-09f},
                   {4.166666791e-02f, -1.241763470e-09f}, {8.333333768e-03f, -4.346172033e-10f},
                   {1.388888923e-03f, -3.363109444e-11f}, {1.984127011e-04f, -2.725596875e-12f},
                   {2.480158764e-05f, -3.406996094e-13f}};
  df p = c[8];
#pragma unroll
  for (int n = 7; n >= 0; --n) p = p * r + c[n];
#pragma unroll
  for (int q = 0; q < 4; ++q) p = p * p;
  const float s = __int_as_float((127 + (int)k) << 23);  // 2^k, -116 <= k <= 0
  return {p.hi * s, p.lo * s};
}

// atan2(y, x) for y >= 0 (so the result is in [0, pi]) to double-word
// accuracy: a float estimate t0 refined by one step
// t = t0 + (y cos t0 - x sin t0) / (x cos t0 + y sin t0); valid while
// |t0| <= 0.8, otherwise the caller falls back to FP64.
__device__ __forceinline__ bool df_atan2_pos(df y, df x, df* out) {
  float t0 = atan2f(y.hi, x.hi);
  if (t0 > 0.8f) return false;
  df s, c;
  df_sincos_small(t0, &s, &c);
  df num = y * c - x * s;
  df den = x * c + y * s;
  *out = df_make(t0) + num / den;
  return true;
}

// ---- lighter forms for the stencils ---------------------------------------
// The positions enter as double-words of about 48 bits, so every quantity of
// the stencils carries an absolute error of a few u^2 times the magnitudes it
// is built from.  These forms keep to that absolute error and skip the work
// that only buys relative accuracy under cancellation:
//   add_s   SloppyDWPlusDW (Joldes, Muller & Popescu 2017, Algorithm 5),
//           error a few u^2 (|x| + |y|), 11 operations instead of 20;
//   mul_s   DWTimesDW without the lo*lo term (below u^2 relative);
//   dot3 / cross_c   sums of exact products (TwoProd with FMA) in the style
//           of Ogita, Rump & Oishi's Dot2, one TwoSum per addition and all
//           error terms collected in one float;
//   dacc    a running sum whose float lo part gathers the TwoSum errors
//           (Sum2 of the same paper), renormalised once at the end;
//   rsqrt_dw / rcp_dw   one Newton step from the float estimate (relative
//           error about 2^-46).
__device__ __forceinline__ df add_s(df x, df y) {
  df s = two_sum(x.hi, y.hi);
  float c = __fadd_rn(s.lo, __fadd_rn(x.lo, y.lo));
  return fast_two_sum(s.hi, c);
}
__device__ __forceinline__ df sub_s(df x, df y) { return add_s(x, df{-y.hi, -y.lo}); }
__device__ __forceinline__ df mul_s(df x, df y) {
  df c = two_prod(x.hi, y.hi);
  float t = __fmaf_rn(x.hi, y.lo, __fmul_rn(x.lo, y.hi));
  return fast_two_sum(c.hi, __fadd_rn(c.lo, t));
}
__device__ __forceinline__ df neg(df x) { return {-x.hi, -x.lo}; }
__device__ __forceinline__ df half(df x) { return {0.5f * x.hi, 0.5f * x.lo}; }
// x >= 0 test and |x| on the leading part (hi carries the sign)
__device__ __forceinline__ df dabs(df x) { return x.hi < 0.0f ? neg(x) : x; }

__device__ __forceinline__ df3 sub3(const df3& a, const df3& b) {
  return {sub_s(a.x, b.x), sub_s(a.y, b.y), sub_s(a.z, b.z)};
}
__device__ __forceinline__ df3 scale3(df s, const df3& a) { return {mul_s(s, a.x), mul_s(s, a.y), mul_s(s, a.z)}; }

// a . b
__device__ __forceinline__ df dot3(const df3& a, const df3& b) {
  df p0 = two_prod(a.x.hi, b.x.hi), p1 = two_prod(a.y.hi, b.y.hi), p2 = two_prod(a.z.hi, b.z.hi);
  df s = two_sum(p0.hi, p1.hi);
  df t = two_sum(s.hi, p2.hi);
  float lo = __fadd_rn(__fadd_rn(p0.lo, p1.lo), __fadd_rn(p2.lo, __fadd_rn(s.lo, t.lo)));
  lo = __fmaf_rn(a.x.hi, b.x.lo, lo);
  lo = __fmaf_rn(a.x.lo, b.x.hi, lo);
  lo = __fmaf_rn(a.y.hi, b.y.lo, lo);
  lo = __fmaf_rn(a.y.lo, b.y.hi, lo);
  lo = __fmaf_rn(a.z.hi, b.z.lo, lo);
  lo = __fmaf_rn(a.z.lo, b.z.hi, lo);
  return two_sum(t.hi, lo);
}
// a1 b2 - a2 b1 (one component of a cross product)
__device__ __forceinline__ df cross_c(df a1, df b2, df a2, df b1) {
  df p = two_prod(a1.hi, b2.hi), q = two_prod(a2.hi, b1.hi);
  df s = two_sum(p.hi, -q.hi);
  float lo = __fadd_rn(__fsub_rn(p.lo, q.lo), s.lo);
  lo = __fmaf_rn(a1.hi, b2.lo, lo);
  lo = __fmaf_rn(a1.lo, b2.hi, lo);
  lo = __fmaf_rn(-a2.hi, b1.lo, lo);
  lo = __fmaf_rn(-a2.lo, b1.hi, lo);
  return two_sum(s.hi, lo);
}
__device__ __forceinline__ df3 cross3(const df3& a, const df3& b) {
  return {cross_c(a.y, b.z, a.z, b.y), cross_c(a.z, b.x, a.x, b.z), cross_c(a.x, b.y, a.y, b.x)};
}

struct dacc {
  float hi, lo;
};
__device__ __forceinline__ void acc_add(dacc& a, df x) {
  df s = two_sum(a.hi, x.hi);
  a.hi = s.hi;
  a.lo = __fadd_rn(a.lo, __fadd_rn(s.lo, x.lo));
}
__device__ __forceinline__ df acc_val(const dacc& a) { return two_sum(a.hi, a.lo); }
struct dacc3 {
  dacc x, y, z;
};
__device__ __forceinline__ void acc_add3(dacc3& a, const df3& v) {
  acc_add(a.x, v.x);
  acc_add(a.y, v.y);
  acc_add(a.z, v.z);
}
__device__ __forceinline__ df3 acc_val3(const dacc3& a) { return {acc_val(a.x), acc_val(a.y), acc_val(a.z)}; }

// 1 / sqrt(q), q > 0: with q r0^2 = 1 - e (r0 the float estimate, |e| of
// order 2^-22), 1/sqrt(q) = r0 (1 + e/2 + 3e^2/8 + O(e^3))
__device__ __forceinline__ df rsqrt_dw(df q) {
  const float r0 = rsqrtf(q.hi);
  const df y = mul_s(q, two_prod(r0, r0));
  const float e = __fsub_rn(__fsub_rn(1.0f, y.hi), y.lo);
  const float c = __fmul_rn(__fmul_rn(r0, e), __fmaf_rn(0.375f, e, 0.5f));
  return fast_two_sum(r0, c);
}
// 1 / x, x != 0: with x r0 = 1 - e (r0 = 1/x_hi rounded, |e| <= 2^-24 plus
// x_lo's share), 1/x = r0 (1 + e + e^2 + O(e^3))
__device__ __forceinline__ df rcp_dw(df x) {
  const float r0 = __frcp_rn(x.hi);
  const df p = two_prod(x.hi, r0);
  const float e = __fsub_rn(__fsub_rn(__fsub_rn(1.0f, p.hi), p.lo), __fmul_rn(x.lo, r0));
  return fast_two_sum(r0, __fmul_rn(__fmul_rn(r0, e), __fadd_rn(1.0f, e)));
}

}  // namespace tmg
