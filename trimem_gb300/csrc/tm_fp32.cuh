// FP32 element records and float helpers shared by the FP32-stencil
// evaluation and the surrogate force model.
#pragma once
#include "tm_internal.h"

namespace tmg {

struct __align__(16) FaceF {
  float nx, ny, nz, A, V, c0, c1, c2;
};
struct __align__(16) EdgeF {
  float l, th, db, flag;
};

namespace fp32 {

struct f3 {
  float x, y, z;
};
__device__ __forceinline__ f3 operator+(f3 a, f3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ f3 operator-(f3 a, f3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ f3 operator*(float s, f3 a) { return {s * a.x, s * a.y, s * a.z}; }
__device__ __forceinline__ f3& operator+=(f3& a, f3 b) {
  a.x += b.x;
  a.y += b.y;
  a.z += b.z;
  return a;
}
__device__ __forceinline__ float fdot(f3 a, f3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ f3 fcross(f3 a, f3 b) {
  return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
__device__ __forceinline__ float fnorm(f3 a) { return sqrtf(fdot(a, a)); }
__device__ __forceinline__ float fipow(float x, int n) {
  int a = n < 0 ? -n : n;
  float r = 1.0f;
  for (int k = 0; k < a; ++k) r *= x;
  return n < 0 ? 1.0f / r : r;
}

struct Split {
  const float* hi;
  const float* lo;
  __device__ f3 h(int v) const { return {hi[3 * v], hi[3 * v + 1], hi[3 * v + 2]}; }
  // x_b - x_a with FP32 relative accuracy
  __device__ f3 diff(int b, int a) const {
    return {(hi[3 * b] - hi[3 * a]) + (lo[3 * b] - lo[3 * a]), (hi[3 * b + 1] - hi[3 * a + 1]) + (lo[3 * b + 1] - lo[3 * a + 1]),
            (hi[3 * b + 2] - hi[3 * a + 2]) + (lo[3 * b + 2] - lo[3 * a + 2])};
  }
};

}  // namespace fp32
}  // namespace tmg
