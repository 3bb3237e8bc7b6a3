// Energy minimisation on device-resident positions: limited-memory BFGS
// (Nocedal, "Updating quasi-Newton matrices with limited storage", Math.
// Comp. 35, 1980; two-loop recursion) with a backtracking line search on
// the Armijo condition.  The reference's minimisation path
// (src/trimem/mc/util.py:240-306) runs scipy's L-BFGS-B over the energy and
// gradient with the neighbour list refreshed at every evaluation; here the
// iterate, the gradient and the correction pairs stay in device memory, each
// evaluation refreshes the cell list and evaluates on the device, and only
// scalars (dot products, energies) come back to the host.
#include <algorithm>
#include <cmath>
#include <vector>

#include "tm_energy.cuh"
#include "tm_internal.h"

using namespace tmg;

#define TM_API_BEGIN try {
#define TM_API_END                  \
  }                                 \
  catch (const tmg::Error& e) {     \
    tmg::set_last_error(e.what());  \
    return e.code;                  \
  }                                 \
  catch (const std::exception& e) { \
    tmg::set_last_error(e.what());  \
    return TM_ERR_ARG;              \
  }                                 \
  return TM_OK;

namespace {

constexpr int DB = 256, DG = 296;  // dot-product blocks: 2 per SM

// fixed-order dot products: per-block partials, then one block
__global__ void k_dot_blocks(int n, const double* __restrict__ a, const double* __restrict__ b,
                             double* __restrict__ part) {
  __shared__ double s[DB];
  double acc = 0.0;
  for (int i = blockIdx.x * DB + threadIdx.x; i < n; i += gridDim.x * DB) acc += a[i] * b[i];
  s[threadIdx.x] = acc;
  __syncthreads();
  for (int o = DB / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) s[threadIdx.x] += s[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = s[0];
}
__global__ void k_dot_sum(int nb, const double* __restrict__ part, double* __restrict__ out) {
  __shared__ double s[DB];
  double acc = 0.0;
  for (int i = threadIdx.x; i < nb; i += DB) acc += part[i];
  s[threadIdx.x] = acc;
  __syncthreads();
  for (int o = DB / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) s[threadIdx.x] += s[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = s[0];
}
// max |g_i|
__global__ void k_amax_blocks(int n, const double* __restrict__ a, double* __restrict__ part) {
  __shared__ double s[DB];
  double m = 0.0;
  for (int i = blockIdx.x * DB + threadIdx.x; i < n; i += gridDim.x * DB) m = fmax(m, fabs(a[i]));
  s[threadIdx.x] = m;
  __syncthreads();
  for (int o = DB / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) s[threadIdx.x] = fmax(s[threadIdx.x], s[threadIdx.x + o]);
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = s[0];
}
__global__ void k_axpy(int n, double a, const double* __restrict__ x, double* __restrict__ y) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) y[i] += a * x[i];
}
__global__ void k_scale_copy(int n, double a, const double* __restrict__ x, double* __restrict__ y) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) y[i] = a * x[i];
}
// y = x + a d
__global__ void k_step(int n, double a, const double* __restrict__ x, const double* __restrict__ d,
                       double* __restrict__ y) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) y[i] = x[i] + a * d[i];
}
__global__ void k_sub(int n, const double* __restrict__ a, const double* __restrict__ b, double* __restrict__ out) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = a[i] - b[i];
}

inline int nblk(long n, int b) { return (int)((n + b - 1) / b); }

struct Lbfgs {
  tm_energy* e;
  tm_mesh* m;
  cudaStream_t s;
  int n;
  DevBuf<double> part, scal;
  double dot(const double* a, const double* b) {
    k_dot_blocks<<<DG, DB, 0, s>>>(n, a, b, part.get());
    k_dot_sum<<<1, DB, 0, s>>>(DG, part.get(), scal.get());
    TM_LAUNCH();
    double r;
    TM_CUDA(cudaMemcpyAsync(&r, scal.get(), sizeof(double), cudaMemcpyDeviceToHost, s));
    TM_CUDA(cudaStreamSynchronize(s));
    return r;
  }
  double amax(const double* a) {
    k_amax_blocks<<<DG, DB, 0, s>>>(n, a, part.get());
    TM_LAUNCH();
    std::vector<double> h(DG);
    TM_CUDA(cudaMemcpyAsync(h.data(), part.get(), sizeof(double) * DG, cudaMemcpyDeviceToHost, s));
    TM_CUDA(cudaStreamSynchronize(s));
    return *std::max_element(h.begin(), h.end());
  }
  // energy and gradient at x, neighbour list refreshed first
  double eval(const double* x, double* g) {
    nlist_make(&e->nl, m, e->prm, x, s);
    energy_eval(e, m, x, true, false, g, s);
    double E;
    TM_CUDA(cudaMemcpyAsync(&E, &e->glob.get()->comps[6], sizeof(double), cudaMemcpyDeviceToHost, s));
    TM_CUDA(cudaStreamSynchronize(s));
    return E;
  }
};

}  // namespace

extern "C" int tm_minimize_device(tm_energy* e, tm_mesh* m, double* d_x, int maxiter, int history, double gtol,
                                  double ftol, int32_t* iterations, double* energy, void* stream) {
  TM_API_BEGIN
  if (!e || !m || !d_x) fail(TM_ERR_ARG, "NULL argument");
  if (maxiter < 0 || history < 1 || history > 64) fail(TM_ERR_ARG, "invalid L-BFGS settings");
  cudaStream_t s = stream ? (cudaStream_t)stream : e->stream;
  const int n = 3 * m->nv;
  Lbfgs L{e, m, s, n};
  L.part.ensure(DG);
  L.scal.ensure(1);
  DevBuf<double> g, d, xn, gn, S, Y;
  g.ensure(n);
  d.ensure(n);
  xn.ensure(n);
  gn.ensure(n);
  S.ensure((size_t)history * n);
  Y.ensure((size_t)history * n);
  std::vector<double> rho(history), alpha(history);
  const int b = 256;
  double f = L.eval(d_x, g.get());
  int k = 0, stored = 0, head = 0;
  double gamma = 1.0;
  for (; k < maxiter; ++k) {
    if (L.amax(g.get()) <= gtol) break;
    // two-loop recursion: d = -H g
    k_scale_copy<<<nblk(n, b), b, 0, s>>>(n, -1.0, g.get(), d.get());
    TM_LAUNCH();
    for (int i = 0; i < stored; ++i) {
      int j = (head - 1 - i + history) % history;
      alpha[j] = rho[j] * L.dot(S.get() + (size_t)j * n, d.get());
      k_axpy<<<nblk(n, b), b, 0, s>>>(n, -alpha[j], Y.get() + (size_t)j * n, d.get());
    }
    k_scale_copy<<<nblk(n, b), b, 0, s>>>(n, gamma, d.get(), d.get());
    for (int i = stored - 1; i >= 0; --i) {
      int j = (head - 1 - i + history) % history;
      double beta = rho[j] * L.dot(Y.get() + (size_t)j * n, d.get());
      k_axpy<<<nblk(n, b), b, 0, s>>>(n, alpha[j] - beta, S.get() + (size_t)j * n, d.get());
    }
    TM_LAUNCH();
    double gd = L.dot(g.get(), d.get());
    if (!(gd < 0.0)) {  // not a descent direction: restart from steepest descent
      k_scale_copy<<<nblk(n, b), b, 0, s>>>(n, -1.0, g.get(), d.get());
      TM_LAUNCH();
      stored = 0;
      gamma = 1.0;
      gd = L.dot(g.get(), d.get());
    }
    // first step of a restart: unit step along -g scaled to a max move of
    // 1e-3 of the largest gradient component
    double a = 1.0;
    if (stored == 0) a = std::min(1.0, 1e-3 / std::max(L.amax(g.get()), 1e-300));
    double fn = 0.0;
    bool ok = false;
    for (int ls = 0; ls < 40; ++ls) {
      k_step<<<nblk(n, b), b, 0, s>>>(n, a, d_x, d.get(), xn.get());
      TM_LAUNCH();
      fn = L.eval(xn.get(), gn.get());
      if (std::isfinite(fn) && fn <= f + 1e-4 * a * gd) {
        ok = true;
        break;
      }
      a *= 0.5;
    }
    if (!ok) break;  // no decrease along d
    // correction pair s = x_new - x, y = g_new - g
    double* sk = S.get() + (size_t)head * n;
    double* yk = Y.get() + (size_t)head * n;
    k_sub<<<nblk(n, b), b, 0, s>>>(n, xn.get(), d_x, sk);
    k_sub<<<nblk(n, b), b, 0, s>>>(n, gn.get(), g.get(), yk);
    TM_LAUNCH();
    double sy = L.dot(sk, yk);
    TM_CUDA(cudaMemcpyAsync(d_x, xn.get(), sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
    TM_CUDA(cudaMemcpyAsync(g.get(), gn.get(), sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
    double fprev = f;
    f = fn;
    if (sy > 1e-300) {
      double yy = L.dot(yk, yk);
      rho[head] = 1.0 / sy;
      gamma = sy / yy;
      head = (head + 1) % history;
      stored = std::min(stored + 1, history);
    }
    if ((fprev - f) <= ftol * std::max({std::fabs(fprev), std::fabs(f), 1.0})) {
      ++k;
      break;
    }
  }
  TM_CUDA(cudaStreamSynchronize(s));
  if (iterations) *iterations = k;
  if (energy) *energy = f;
  TM_API_END
}
