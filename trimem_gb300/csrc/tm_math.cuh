// Small vector helpers for device code.
#pragma once

#include <cuda_runtime.h>

namespace tmg {

struct d3 {
  double x, y, z;
};
__device__ __forceinline__ d3 mk(double x, double y, double z) { return {x, y, z}; }
__device__ __forceinline__ d3 operator+(d3 a, d3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ d3 operator-(d3 a, d3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ d3 operator-(d3 a) { return {-a.x, -a.y, -a.z}; }
__device__ __forceinline__ d3 operator*(double s, d3 a) { return {s * a.x, s * a.y, s * a.z}; }
__device__ __forceinline__ d3 operator*(d3 a, double s) { return {s * a.x, s * a.y, s * a.z}; }
__device__ __forceinline__ d3& operator+=(d3& a, d3 b) {
  a.x += b.x;
  a.y += b.y;
  a.z += b.z;
  return a;
}
__device__ __forceinline__ double dot(d3 a, d3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ d3 cross(d3 a, d3 b) {
  return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
__device__ __forceinline__ double norm(d3 a) { return sqrt(dot(a, a)); }

__device__ __forceinline__ d3 ld3(const double* p, int i) {
  return {__ldg(p + 3 * i), __ldg(p + 3 * i + 1), __ldg(p + 3 * i + 2)};
}
__device__ __forceinline__ void st3(double* p, int i, d3 v) {
  p[3 * i] = v.x;
  p[3 * i + 1] = v.y;
  p[3 * i + 2] = v.z;
}

// |a - b| rounded exactly like sqrt((dx*dx + dy*dy) + dz*dz) with every
// operation rounded separately (no FMA contraction), so comparisons against
// a cut-off decide exactly like the sequential CPU code.
__device__ __forceinline__ double exact_dist(d3 a, d3 b) {
  double dx = __dsub_rn(a.x, b.x), dy = __dsub_rn(a.y, b.y), dz = __dsub_rn(a.z, b.z);
  double s = __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
  return __dsqrt_rn(s);
}
__device__ __forceinline__ d3 exact_diff(d3 a, d3 b) {
  return {__dsub_rn(a.x, b.x), __dsub_rn(a.y, b.y), __dsub_rn(a.z, b.z)};
}

// integer power (the potentials' exponents are small integers)
__device__ __forceinline__ double ipow(double x, int n) {
  int a = n < 0 ? -n : n;
  double r = 1.0;
  for (int k = 0; k < a; ++k) r *= x;
  return n < 0 ? 1.0 / r : r;
}

}  // namespace tmg
