#include <algorithm>
// Error plumbing and deterministic scan / reduction helpers.
#include <cmath>
#include <cstdio>
#include <string>

#include "tm_internal.h"

namespace tmg {

static thread_local std::string g_last_error;

void set_last_error(const std::string& m) { g_last_error = m; }

void fail(int code, const std::string& m) { throw Error(code, m); }

void cuda_check(cudaError_t e, const char* what, const char* file, int line) {
  if (e == cudaSuccess) return;
  cudaGetLastError();
  char buf[512];
  snprintf(buf, sizeof(buf), "CUDA error %s (%s) at %s:%d in %s", cudaGetErrorName(e), cudaGetErrorString(e), file,
           line, what);
  fail(TM_ERR_CUDA, buf);
}

double sq_threshold(double d) {
  if (!(d > 0)) return d != d ? d : 0.0;
  if (std::isinf(d)) return d;
  double s = d * d;
  if (std::sqrt(s) >= d) {
    while (s > 0 && std::sqrt(std::nextafter(s, 0.0)) >= d) s = std::nextafter(s, 0.0);
  } else {
    while (std::sqrt(s) < d) s = std::nextafter(s, INFINITY);
  }
  return s;
}

// ---- exclusive scan of int counts (three phases, 1024 items per block) ----
static constexpr int SCAN_B = 1024;

__global__ void k_scan_blocks(const int* in, int* out, int n, int* bsum) {
  __shared__ int s[SCAN_B];
  int i = blockIdx.x * SCAN_B + threadIdx.x;
  int v = i < n ? in[i] : 0;
  s[threadIdx.x] = v;
  __syncthreads();
  for (int off = 1; off < SCAN_B; off <<= 1) {
    int t = threadIdx.x >= off ? s[threadIdx.x - off] : 0;
    __syncthreads();
    s[threadIdx.x] += t;
    __syncthreads();
  }
  if (i < n) out[i] = s[threadIdx.x] - v;
  if (threadIdx.x == SCAN_B - 1) bsum[blockIdx.x] = s[threadIdx.x];
}

__global__ void k_scan_sums(int* bsum, int nb, int* total) {
  // one block; sequential over chunks of SCAN_B
  __shared__ int s[SCAN_B];
  __shared__ int carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (int base = 0; base < nb; base += SCAN_B) {
    int i = base + threadIdx.x;
    int v = i < nb ? bsum[i] : 0;
    s[threadIdx.x] = v;
    __syncthreads();
    for (int off = 1; off < SCAN_B; off <<= 1) {
      int t = threadIdx.x >= off ? s[threadIdx.x - off] : 0;
      __syncthreads();
      s[threadIdx.x] += t;
      __syncthreads();
    }
    if (i < nb) bsum[i] = carry + s[threadIdx.x] - v;
    __syncthreads();
    if (threadIdx.x == SCAN_B - 1) carry += s[threadIdx.x];
    __syncthreads();
  }
  if (threadIdx.x == 0) *total = carry;
}

__global__ void k_scan_add(int* out, int n, const int* bsum) {
  int i = blockIdx.x * SCAN_B + threadIdx.x;
  if (i < n) out[i] += bsum[blockIdx.x];
}

void exclusive_scan_int(const int* in, int* out, int n, int* total_host, DevBuf<int>& tmp, cudaStream_t s) {
  int nb = (n + SCAN_B - 1) / SCAN_B;
  if (nb < 1) nb = 1;
  tmp.ensure(nb + 1);
  k_scan_blocks<<<nb, SCAN_B, 0, s>>>(in, out, n, tmp.get());
  TM_LAUNCH();
  k_scan_sums<<<1, SCAN_B, 0, s>>>(tmp.get(), nb, tmp.get() + nb);
  TM_LAUNCH();
  k_scan_add<<<nb, SCAN_B, 0, s>>>(out, n, tmp.get());
  TM_LAUNCH();
  if (total_host) {
    TM_CUDA(cudaMemcpyAsync(total_host, tmp.get() + nb, sizeof(int), cudaMemcpyDeviceToHost, s));
    TM_CUDA(cudaStreamSynchronize(s));
  }
}

}  // namespace tmg

extern "C" const char* tm_last_error(void) { return tmg::g_last_error.c_str(); }

extern "C" int tm_device_name(char* buf, int len) {
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) {
    cudaGetLastError();
    tmg::set_last_error("no CUDA device");
    return TM_ERR_CUDA;
  }
  cudaDeviceProp p;
  if (cudaGetDeviceProperties(&p, 0) != cudaSuccess) {
    tmg::set_last_error("cudaGetDeviceProperties failed");
    return TM_ERR_CUDA;
  }
  snprintf(buf, len, "%s", p.name);
  return TM_OK;
}

extern "C" int tm_host_alloc(int64_t bytes, void** out) {
  if (!out || bytes < 0) {
    tmg::set_last_error("invalid argument");
    return TM_ERR_ARG;
  }
  *out = nullptr;
  if (cudaMallocHost(out, (size_t)std::max<int64_t>(bytes, 1)) != cudaSuccess) {
    cudaGetLastError();
    *out = nullptr;
    tmg::set_last_error("page-locked allocation failed");
    return TM_ERR_NOMEM;
  }
  return TM_OK;
}

extern "C" int tm_host_free(void* p) {
  if (p) cudaFreeHost(p);
  return TM_OK;
}
