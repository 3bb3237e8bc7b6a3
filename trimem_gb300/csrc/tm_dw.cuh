// Double-word helpers shared by the double-word stencils (energy_df.cu) and
// the flip sweep's property changes (flips.cu): positions split into float
// hi / lo parts, constants, the dihedral angle from its sine and cosine.
#pragma once

#include "df64.cuh"
#include "tm_internal.h"

namespace tmg {

// double-float constants 1/3 and 1/6 (hi = float(c), lo = float(c - hi))
__device__ __forceinline__ df third() { return {3.333333433e-01f, -9.934107481e-09f}; }
__device__ __forceinline__ df sixth() { return {1.666666716e-01f, -4.967053740e-09f}; }

// positions as double-words: hi parts p[v] = (x, y, z, 0), lo parts p[nv + v]
struct PosDW {
  const float4* __restrict__ p;
  int nv;
  __device__ __forceinline__ df3 at(int v) const {
    const float4 h = __ldg(p + v), l = __ldg(p + nv + v);
    return {{h.x, l.x}, {h.y, l.y}, {h.z, l.z}};
  }
};

// double-word parameters (hi / lo from the host)
struct EPD {
  df kb, kt, kr, kb23, a0, inv_a0, inv_tdiv, lc0, lc1, br1, br2;
};
__device__ __forceinline__ bool df_less(df a, df b) { return a.hi < b.hi || (a.hi == b.hi && a.lo < b.lo); }
__device__ __forceinline__ df ipow_dw(df x, int n) {
  df r = df_make(1.0f);
  for (int k = 0; k < n; ++k) r = mul_s(r, x);
  return r;
}
__device__ __forceinline__ df lo_hi(float h, float l) { return {h, l}; }

// Signed dihedral angle from s = sin(theta) (signed) and c = cos(theta):
// theta0 = k/128 nearest to a float atan2(|s|, c), whose sine and cosine the
// table holds as double-words, then |theta| = theta0 + asin(x) with
// x = |s| cos theta0 - c sin theta0 = sin(|theta| - theta0), |x| < 1/250:
// asin(x) = x + x^3/6 + 3x^5/40 + O(x^7), the cubic and quintic terms in
// float (they are below 1e-8 relative).  Small angles keep full relative
// accuracy (k = 0 gives theta = asin(s)).
__device__ __forceinline__ df angle_dw(df s, df c, const float4* __restrict__ sct) {
  const bool neg_s = s.hi < 0.0f;
  const df sa = neg_s ? neg(s) : s;
  const float tf = atan2f(sa.hi, c.hi);
  int k = __float2int_rn(tf * 128.0f);
  k = min(max(k, 0), TM_SCT_N - 1);
  const float4 g = __ldg(sct + k);  // (sin hi, sin lo, cos hi, cos lo) of k/128
  const df x = cross_c(sa, lo_hi(g.z, g.w), c, lo_hi(g.x, g.y));
  const float x2 = x.hi * x.hi;
  const float q = x.hi * x2 * fmaf(x2, 3.0f / 40.0f, 1.0f / 6.0f);
  const float t0 = (float)k * (1.0f / 128.0f);
  const df r = two_sum(t0, x.hi);
  const df th = fast_two_sum(r.hi, __fadd_rn(r.lo, __fadd_rn(x.lo, q)));
  return neg_s ? neg(th) : th;
}

// x = hi + lo with hi = x rounded to 24 significant bits and lo = x - hi
// rounded to a float, from the bits of x with integer operations only:
// GB300's double-to-float conversions run on the scarce FP64 pipe.  The
// rounding of the magnitude's bit pattern carries into the exponent when it
// must, and the pattern difference a - ar counts units of 2^(e - 1075) on
// both sides of that carry.  |x| below the normal float range gives a signed
// zero hi, lo below 2^-126 is dropped (an absolute error below 2^-126);
// infinities and NaN keep their class in hi.
__device__ __forceinline__ void split_bits(double x, float* hi, float* lo) {
  const long long b = __double_as_longlong(x);
  const int sign = (int)(((unsigned long long)b >> 63) << 31);
  const long long a = b & 0x7fffffffffffffffLL;
  const int e = (int)(a >> 52);
  *lo = 0.0f;
  if (e == 0x7ff) {
    *hi = __int_as_float(sign | 0x7f800000 | ((a & 0xfffffffffffffLL) ? 0x400000 : 0));
    return;
  }
  if (e < 1023 - 126) {
    *hi = __int_as_float(sign);
    return;
  }
  const long long ar = (a + (1LL << 28)) & ~((1LL << 29) - 1);
  const int ef = (int)(ar >> 52) - 1023 + 127;
  if (ef > 254) {
    *hi = __int_as_float(sign | 0x7f800000);
    return;
  }
  *hi = __int_as_float(sign | (ef << 23) | (int)((ar >> 29) & 0x7fffff));
  const int el = e - 1075 + 127;
  if (el >= 1) {
    const float r = __int2float_rn((int)(a - ar)) * __int_as_float(el << 23);
    *lo = sign ? -r : r;
  }
}

struct EP;
// double-word copies of the energy parameters (energy_df.cu)
EPD make_epd(const EP& ep);
// positions split into double-words (hi parts [nv], lo parts [nv] of
// e->posdw) and the float copy e->pos32, on stream s; returns e->posdw
const float4* split_positions_dw(tm_energy* e, int nv, const double* P, cudaStream_t s);

}  // namespace tmg
