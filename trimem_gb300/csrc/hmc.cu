// Device-resident Hamiltonian Monte Carlo step (src/trimem/mc/hmc.py:14-26,
// 129-158): momenta p ~ N(0, m T), n_steps velocity-Verlet steps
//   x <- x + (p dt + 0.5 a dt^2) / m,  a' = -grad E(x),  p <- p + 0.5 (a + a') dt
// and a Metropolis test on dH = (H(x', p') - H(x, p)) / T with
// H = E + 0.5 p.p / m.  Positions, momenta and forces never leave the device;
// the energy of the end point is the one computed with its last force.
// Momenta come from SplitMix64 over (seed, step, coordinate) and Box-Muller.
#include <algorithm>
#include <cmath>

#include "tm_energy.cuh"
#include "tm_internal.h"
#include "tm_math.cuh"

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

__device__ __forceinline__ unsigned long long smix(unsigned long long z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

__global__ void k_momenta(int n3, unsigned long long seed, unsigned long long step, double sd, double* p) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  int pair = i;  // one Box-Muller pair per two coordinates
  if (2 * pair >= n3) return;
  unsigned long long k = smix(smix(seed) ^ smix(step + 0x632BE59BD9B4E019ull)) ^ (unsigned long long)pair;
  unsigned long long a = smix(k), b = smix(a);
  double u1 = ((double)(a >> 11) + 1.0) * 0x1.0p-53;  // (0, 1]
  double u2 = (double)(b >> 11) * 0x1.0p-53;
  double r = sqrt(-2.0 * log(u1));
  double s, c;
  sincospi(2.0 * u2, &s, &c);
  p[2 * pair] = sd * r * c;
  if (2 * pair + 1 < n3) p[2 * pair + 1] = sd * r * s;
}

__global__ void k_copy(int n, const double* a, double* b) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) b[i] = a[i];
}

// x += (p dt + 0.5 a dt^2) / m with a = -g
// im = 1/m: an FP64 division per element would dominate the pass (FP64 is
// GB300's scarce pipe); for the usual m = 1 both forms are exact
__global__ void k_drift(int n3, double dt, double im, const double* p, const double* g, double* x) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n3) {
    double a = -g[i];
    x[i] = x[i] + (p[i] * dt + 0.5 * a * (dt * dt)) * im;
  }
}
// p += 0.5 (a + a') dt
__global__ void k_kick(int n3, double dt, const double* g0, const double* g1, double* p) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n3) p[i] = p[i] + 0.5 * ((-g0[i]) + (-g1[i])) * dt;
}

// k_kick followed by the next step's k_drift (the kick's new momentum and
// the same force), the same arithmetic per element in one pass
__global__ void k_kick_drift(int n3, double dt, double im, const double* g0, const double* g1, double* p,
                             double* x) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n3) {
    const double pn = p[i] + 0.5 * ((-g0[i]) + (-g1[i])) * dt;
    p[i] = pn;
    const double a = -g1[i];
    x[i] = x[i] + (pn * dt + 0.5 * a * (dt * dt)) * im;
  }
}

// fixed-order dot product p.p into out[slot]
__global__ void k_dot_partial(int n, const double* p, double* part) {
  __shared__ double s[256];
  double acc = 0.0;
  for (int i = blockIdx.x * 256 + threadIdx.x; i < n; i += gridDim.x * 256) acc += p[i] * p[i];
  s[threadIdx.x] = acc;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if (threadIdx.x < o) s[threadIdx.x] += s[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = s[0];
}
__global__ void k_dot_final(int nb, const double* part, double* out) {
  __shared__ double s[256];
  double acc = 0.0;
  for (int i = threadIdx.x; i < nb; i += 256) acc += part[i];
  s[threadIdx.x] = acc;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if (threadIdx.x < o) s[threadIdx.x] += s[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = s[0];
}

// out4 = {accepted, H0, H1, E(returned)}; sc = {E0, pp0, E1, pp1};
// props: 8 properties at the start, 8 at the end, 8 of the returned state
__global__ void k_accept(const double* sc, double m, double T, double u, double* out4, int* flag, double* props) {
  if (threadIdx.x || blockIdx.x) return;
  double H0 = sc[0] + 0.5 * sc[1] / m;
  double H1 = sc[2] + 0.5 * sc[3] / m;
  double dh = (H1 - H0) / T;
  double a = dh <= 0.0 ? 1.0 : exp(-dh);
  int acc = u <= a ? 1 : 0;
  out4[0] = acc;
  out4[1] = H0;
  out4[2] = H1;
  out4[3] = acc ? sc[2] : sc[0];
  *flag = acc;
  for (int k = 0; k < 8; ++k) props[16 + k] = acc ? props[8 + k] : props[k];
}
__global__ void k_copy_if(int n, const int* flag, const double* a, double* b) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n && *flag) b[i] = a[i];
}

inline int nblk(long n, int b) { return (int)((n + b - 1) / b); }

}  // namespace

// One HMC step; the leapfrog forces come from the energy manager (exact,
// at its stencil precision) or, when sg is given, from the surrogate, in
// which case the start and end energies are separate exact evaluations.
static void hmc_step(tm_surrogate* sg, tm_energy* e, tm_mesh* m, double* d_x, double mass, double dt, int n_steps,
                     double temperature, uint64_t seed, uint64_t step, double u, double* out4, double* props6,
                     cudaStream_t s) {
  if (!d_x || !out4) fail(TM_ERR_ARG, "NULL argument");
  if (n_steps < 0 || !(mass > 0) || !(temperature > 0)) fail(TM_ERR_ARG, "invalid HMC parameters");
  int n3 = 3 * m->nv;
  // work: x, p, g0, g1, partials, scalars
  int nb = std::max(1, std::min(1024, nblk(n3, 256)));
  e->work.ensure(4 * (size_t)n3 + nb + 16 + 8 + 24);
  double* x = e->work.get();
  double* p = x + n3;
  double* g0 = p + n3;
  double* g1 = g0 + n3;
  double* part = g1 + n3;
  double* sc = part + nb;  // 4 scalars
  double* o4 = sc + 8;
  int* flag = reinterpret_cast<int*>(o4 + 4);
  double* props = o4 + 8;  // 24: start, end, returned
  const Globals* G = e->glob.get();
  int b = 256;
  k_copy<<<nblk(n3, b), b, 0, s>>>(n3, d_x, x);
  TM_LAUNCH();
  k_momenta<<<nblk((n3 + 1) / 2, b), b, 0, s>>>(n3, seed, step, sqrt(mass * temperature), p);
  TM_LAUNCH();
  k_dot_partial<<<nb, 256, 0, s>>>(n3, p, part);
  k_dot_final<<<1, 256, 0, s>>>(nb, part, sc + 1);
  TM_LAUNCH();
  auto force = [&](double* g) {
    if (sg)
      surrogate_grad(sg, e, m, x, g, s);
    else
      energy_eval(e, m, x, true, false, g, s);
  };
  auto record = [&](double* E, double* pr) {
    TM_CUDA(cudaMemcpyAsync(E, &G->comps[6], sizeof(double), cudaMemcpyDeviceToDevice, s));
    TM_CUDA(cudaMemcpyAsync(pr, G->props, sizeof(double) * 8, cudaMemcpyDeviceToDevice, s));
  };
  if (sg) {
    energy_eval(e, m, x, false, false, nullptr, s);
    record(sc + 0, props);
    force(g0);
  } else {
    force(g0);
    record(sc + 0, props);
  }
  // velocity Verlet; each kick is fused with the following drift
  if (n_steps > 0) {
    k_drift<<<nblk(n3, b), b, 0, s>>>(n3, dt, 1.0 / mass, p, g0, x);
    TM_LAUNCH();
  }
  for (int i = 0; i < n_steps; ++i) {
    force(g1);
    if (i + 1 < n_steps)
      k_kick_drift<<<nblk(n3, b), b, 0, s>>>(n3, dt, 1.0 / mass, g0, g1, p, x);
    else
      k_kick<<<nblk(n3, b), b, 0, s>>>(n3, dt, g0, g1, p);
    TM_LAUNCH();
    std::swap(g0, g1);
  }
  if (sg) energy_eval(e, m, x, false, false, nullptr, s);
  record(sc + 2, props + 8);
  k_dot_partial<<<nb, 256, 0, s>>>(n3, p, part);
  k_dot_final<<<1, 256, 0, s>>>(nb, part, sc + 3);
  TM_LAUNCH();
  k_accept<<<1, 1, 0, s>>>(sc, mass, temperature, u, o4, flag, props);
  TM_LAUNCH();
  k_copy_if<<<nblk(n3, b), b, 0, s>>>(n3, flag, x, d_x);
  TM_LAUNCH();
  TM_CUDA(cudaMemcpyAsync(out4, o4, sizeof(double) * 4, cudaMemcpyDeviceToHost, s));
  if (props6) TM_CUDA(cudaMemcpyAsync(props6, props + 16, sizeof(double) * 6, cudaMemcpyDeviceToHost, s));
  TM_CUDA(cudaStreamSynchronize(s));
}

extern "C" int tm_hmc_step_device(tm_energy* e, tm_mesh* m, double* d_x, double mass, double dt, int n_steps,
                                  double temperature, uint64_t seed, uint64_t step, double u, double* out4,
                                  double* props6, void* stream) {
  TM_API_BEGIN
  if (!e || !m) fail(TM_ERR_ARG, "NULL argument");
  cudaStream_t s = stream ? (cudaStream_t)stream : e->stream;
  hmc_step(nullptr, e, m, d_x, mass, dt, n_steps, temperature, seed, step, u, out4, props6, s);
  TM_API_END
}

extern "C" int tm_surrogate_hmc_step_device(tm_surrogate* sg, tm_energy* e, tm_mesh* m, double* d_x, double mass,
                                            double dt, int n_steps, double temperature, uint64_t seed, uint64_t step,
                                            double u, double* out4, double* props6, void* stream) {
  TM_API_BEGIN
  if (!sg || !e || !m) fail(TM_ERR_ARG, "NULL argument");
  cudaStream_t s = stream ? (cudaStream_t)stream : e->stream;
  hmc_step(sg, e, m, d_x, mass, dt, n_steps, temperature, seed, step, u, out4, props6, s);
  TM_API_END
}
