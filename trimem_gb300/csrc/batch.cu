// Batches of independent membrane replicas of uneven sizes and parameters.
//
// The replicas are one disjoint-union mesh: replica r owns the vertex range
// [voff[r], voff[r] + nv_r), padded with isolated vertices to a multiple of
// 256 so that no 256-vertex block straddles two replicas.  Per-replica parameters,
// global sums (a ticket per replica picks the block that finishes the
// replica's reduction) and neighbour-list cells (keys tagged with the replica)
// are looked up through vrep (vertex -> replica, -1 for padding).  Stencils are
// FP32 and the global sums FP64.
//
// An HMC step (momenta, L velocity-Verlet steps, per-replica Metropolis on the
// exact energies) runs entirely on the device; random numbers come from a
// device-side step counter, so one step can be captured once into a CUDA graph
// and replayed.
//
// Replicas fall into size classes (runs of consecutive replicas whose
// vertex counts share a power of two).  The element kernels (position
// split, faces, edges, gradient) run per class, side by side on the
// classes' streams inside the captured step, each with the block size the
// autotuner picked for that class when the batch was created; the
// repulsion and the vertex stage (with the per-replica reductions) run once
// for all replicas.  Each replica keeps its own exclusion level; the
// replicas share the kind of neighbour list (cells, or Verlet rows built
// from the replica-tagged cells at each replica's cut-off).
#include <algorithm>
#include <climits>
#include <cmath>
#include <cstring>
#include <memory>
#include <numeric>
#include <vector>

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

struct tm_batch {
  int R = 0;
  int nv = 0;  // padded union size
  std::vector<int> voff, nreal;
  std::vector<tm_params> prm;
  std::vector<double> initial;  // 6 per replica
  std::unique_ptr<tm_mesh> mesh;
  std::unique_ptr<tm_energy> en;
  DevBuf<int> vrep, rexcl;  // vertex -> replica, replica -> exclusion level
  DevBuf<int2> rblocks;
  DevBuf<EP> eps;
  DevBuf<Globals> gs;
  DevBuf<double> rlist;
  // HMC state
  DevBuf<double> x, xs, p, g0, g1, part, sc;  // sc: 4 scalars per replica (E0, K0, E1, K1)
  DevBuf<int> flag, acc;
  DevBuf<unsigned long long> counter;
  // size classes (runs of consecutive replicas of similar size) with their
  // element ranges and tuned block sizes, and their side streams
  std::vector<BatchClass> cls;
  BatchStreams bs{};
  bool have_side = false;
  cudaStream_t stream = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t gexec = nullptr;
  int g_L = -1;
  double g_dt = 0, g_m = 0, g_T = 0;
  unsigned long long g_seed = 0;
  NLView g_view{};  // the neighbour-list view baked into the graph's launches
  // neighbour list rebuilt after every refresh-th HMC step (0: never), like
  // the evaluator callback of the reference's HMC
  int refresh = 1;
  long long steps_done = 0;
  ~tm_batch() {
    if (gexec) cudaGraphExecDestroy(gexec);
    if (graph) cudaGraphDestroy(graph);
    if (have_side) {
      for (size_t c = 0; c < cls.size(); ++c) {
        cudaStreamDestroy(bs.cs[c]);
        cudaEventDestroy(bs.join[c]);
      }
      cudaEventDestroy(bs.fork[0]);
      cudaEventDestroy(bs.fork[1]);
    }
    if (stream) cudaStreamDestroy(stream);
  }
};

namespace {

constexpr int B = 256;
inline int nblk(long n, int b) { return (int)((n + b - 1) / b); }

__device__ __forceinline__ unsigned long long smix(unsigned long long z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

// momenta ~ N(0, m T) from (seed, step counter, coordinate); padding stays 0
__global__ void k_momenta_b(int n3, unsigned long long seed, const unsigned long long* counter, double sd,
                            const int* vrep, double* p) {
  int pair = blockIdx.x * blockDim.x + threadIdx.x;
  if (2 * pair >= n3) return;
  unsigned long long k = smix(smix(seed) ^ smix(*counter + 0x632BE59BD9B4E019ull)) ^ (unsigned long long)pair;
  unsigned long long a = smix(k), b = smix(a);
  double u1 = ((double)(a >> 11) + 1.0) * 0x1.0p-53;
  double u2 = (double)(b >> 11) * 0x1.0p-53;
  double r = sqrt(-2.0 * log(u1));
  double s, c;
  sincospi(2.0 * u2, &s, &c);
  int i0 = 2 * pair, i1 = 2 * pair + 1;
  p[i0] = vrep[i0 / 3] >= 0 ? sd * r * c : 0.0;
  if (i1 < n3) p[i1] = vrep[i1 / 3] >= 0 ? sd * r * s : 0.0;
}
__global__ void k_copy_b(int n, const double* a, double* b) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) b[i] = a[i];
}
// im = 1/m (no FP64 division per element)
__global__ void k_drift_b(int n3, double dt, double im, const double* p, const double* g, double* x) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n3) x[i] = x[i] + (p[i] * dt + 0.5 * (-g[i]) * (dt * dt)) * im;
}
__global__ void k_kick_b(int n3, double dt, const double* g0, const double* g1, double* p) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n3) p[i] = p[i] + 0.5 * ((-g0[i]) + (-g1[i])) * dt;
}
// a kick and the following drift in one pass (same arithmetic)
__global__ void k_kick_drift_b(int n3, double dt, double im, const double* g0, const double* g1, double* p,
                               double* x) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n3) {
    const double pn = p[i] + 0.5 * ((-g0[i]) + (-g1[i])) * dt;
    p[i] = pn;
    x[i] = x[i] + (pn * dt + 0.5 * (-g1[i]) * (dt * dt)) * im;
  }
}
// p.p per 256-vertex block (blocks never straddle replicas)
__global__ void k_kin_blocks(int nv, const double* p, double* part) {
  __shared__ double s[B];
  double acc = 0.0;
  int v = blockIdx.x * B + threadIdx.x;
  if (v < nv)
    for (int k = 0; k < 3; ++k) acc += p[3 * v + k] * p[3 * v + k];
  s[threadIdx.x] = acc;
  __syncthreads();
  for (int o = B / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) s[threadIdx.x] += s[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = s[0];
}
// per replica: energy from its Globals and p.p from its blocks, in order
__global__ void k_collect(int R, const int2* rblocks, const double* part, const Globals* gs, double* sc, int slot) {
  int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= R) return;
  double k = 0.0;
  for (int b = rblocks[r].x; b < rblocks[r].y; ++b) k += part[b];
  sc[4 * r + slot] = gs[r].comps[6];
  sc[4 * r + slot + 1] = k;
}
// Metropolis per replica (src/trimem/mc/hmc.py:147-155)
__global__ void k_accept_b(int R, unsigned long long seed, unsigned long long* counter, double m, double T,
                           const double* sc, int* flag, int* acc) {
  int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r < R) {
    double H0 = sc[4 * r] + 0.5 * sc[4 * r + 1] / m;
    double H1 = sc[4 * r + 2] + 0.5 * sc[4 * r + 3] / m;
    double dh = (H1 - H0) / T;
    double a = dh <= 0.0 ? 1.0 : exp(-dh);
    unsigned long long z = smix(smix(seed ^ 0xA5A5A5A5ull) ^ smix(*counter * 131ull + (unsigned long long)r));
    double u = (double)(z >> 11) * 0x1.0p-53;
    int ok = u <= a ? 1 : 0;
    flag[r] = ok;
    acc[r] += ok;
  }
}
__global__ void k_finish_b(int n3, const int* vrep, const int* flag, double* x, const double* xs) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n3) return;
  int r = vrep[i / 3];
  if (r >= 0 && !flag[r]) x[i] = xs[i];
}
__global__ void k_tick(unsigned long long* counter) {
  if (threadIdx.x == 0 && blockIdx.x == 0) *counter += 1;
}

}  // namespace

static void batch_eval(tm_batch* b, const double* x, double* g, cudaStream_t s) {
  energy_eval_batch32(b->en.get(), b->mesh.get(), x, g, b->eps.get(), b->vrep.get(), b->rblocks.get(), b->gs.get(),
                      b->cls.data(), (int)b->cls.size(), b->have_side ? &b->bs : nullptr, s);
}

static void batch_hmc_step(tm_batch* b, int L, double dt, double m, double T, unsigned long long seed,
                           cudaStream_t s) {
  int n3 = 3 * b->nv;
  int nb = b->nv / B;
  k_copy_b<<<nblk(n3, B), B, 0, s>>>(n3, b->x.get(), b->xs.get());
  k_momenta_b<<<nblk((n3 + 1) / 2, B), B, 0, s>>>(n3, seed, b->counter.get(), sqrt(m * T), b->vrep.get(), b->p.get());
  k_kin_blocks<<<nb, B, 0, s>>>(b->nv, b->p.get(), b->part.get());
  double* g0 = b->g0.get();
  double* g1 = b->g1.get();
  batch_eval(b, b->x.get(), g0, s);
  k_collect<<<nblk(b->R, 64), 64, 0, s>>>(b->R, b->rblocks.get(), b->part.get(), b->gs.get(), b->sc.get(), 0);
  if (L > 0) k_drift_b<<<nblk(n3, B), B, 0, s>>>(n3, dt, 1.0 / m, b->p.get(), g0, b->x.get());
  for (int i = 0; i < L; ++i) {
    batch_eval(b, b->x.get(), g1, s);
    if (i + 1 < L)
      k_kick_drift_b<<<nblk(n3, B), B, 0, s>>>(n3, dt, 1.0 / m, g0, g1, b->p.get(), b->x.get());
    else
      k_kick_b<<<nblk(n3, B), B, 0, s>>>(n3, dt, g0, g1, b->p.get());
    std::swap(g0, g1);
  }
  k_kin_blocks<<<nb, B, 0, s>>>(b->nv, b->p.get(), b->part.get());
  k_collect<<<nblk(b->R, 64), 64, 0, s>>>(b->R, b->rblocks.get(), b->part.get(), b->gs.get(), b->sc.get(), 2);
  k_accept_b<<<nblk(b->R, 64), 64, 0, s>>>(b->R, seed, b->counter.get(), m, T, b->sc.get(), b->flag.get(),
                                           b->acc.get());
  k_finish_b<<<nblk(n3, B), B, 0, s>>>(n3, b->vrep.get(), b->flag.get(), b->x.get(), b->xs.get());
  k_tick<<<1, 32, 0, s>>>(b->counter.get());
  TM_LAUNCH();
}

static void upload_eps(tm_batch* b) {
  std::vector<EP> eps(b->R);
  for (int r = 0; r < b->R; ++r) {
    tm_energy tmp;  // parameters only
    tmp.prm = b->prm[r];
    std::memcpy(tmp.initial, &b->initial[6 * r], sizeof(double) * 6);
    eps[r] = make_ep(&tmp);
  }
  TM_CUDA(cudaMemcpyAsync(b->eps.get(), eps.data(), sizeof(EP) * b->R, cudaMemcpyHostToDevice, b->stream));
  TM_CUDA(cudaStreamSynchronize(b->stream));
}

// near_rows: also (re)build the near rows (their build only runs when some
// vertex has moved half a cut-off).  The rebuilds between HMC steps skip
// them: members that move that far within a step leave the rows stale at
// once, and the cells' candidate rows, rebuilt every time, serve instead
// (the rows never depend on the cells, and stale rows are never used).
static void rebuild_nlist(tm_batch* b, bool near_rows = true) {
  const bool verlet = b->prm[0].n_search == 1;
  // near rows (cell lists) when every replica's cells are at least its
  // repulsion cut-off
  bool near = near_rows && !verlet;
  for (const tm_params& p : b->prm) near = near && p.rep_lc1 > 0 && p.rlist >= p.rep_lc1;
  int excl = 0;
  for (const tm_params& p : b->prm) excl = std::max(excl, (int)p.exclusion_level);
  nlist_make_batch(&b->en->nl, b->mesh.get(), b->R, b->vrep.get(), b->rblocks.get(), b->rlist.get(), excl,
                   b->rexcl.get(), b->x.get(), b->stream, b->eps.get(), near, verlet);
}

// Size classes: runs of consecutive replicas whose vertex counts have the
// same power of two (the 642 / 2,562 / 10,242 / 40,962-vertex levels of the
// benchmark batch are one class each), with their vertex, face and edge
// ranges in the union mesh (a replica's faces and edges are consecutive:
// the union is built replica by replica).  More than TM_MAX_CLASSES runs,
// or ranges that are not consecutive, give one class for the whole batch.
static int log2_floor(int n) {
  int k = -1;
  for (unsigned u = (unsigned)std::max(n, 1); u; u >>= 1) ++k;
  return k;
}
static void make_classes(tm_batch* b) {
  tm_mesh* m = b->mesh.get();
  std::vector<int> rcls(b->R, 0);
  std::vector<std::pair<int, int>> runs;  // replica ranges
  for (int r = 0; r < b->R; ++r) {
    if (r == 0 || log2_floor(b->nreal[r]) != log2_floor(b->nreal[r - 1]))
      runs.push_back({r, r + 1});
    else
      runs.back().second = r + 1;
    rcls[r] = (int)runs.size() - 1;
  }
  std::vector<int> vrep(std::max(m->nv, 1));
  TM_CUDA(cudaMemcpy(vrep.data(), b->vrep.get(), sizeof(int) * m->nv, cudaMemcpyDeviceToHost));
  std::vector<int> fv(3 * (size_t)std::max(m->nf, 1));
  std::vector<int4> ed(std::max(m->ne, 1));
  if (m->nf) TM_CUDA(cudaMemcpy(fv.data(), m->d_fv.get(), sizeof(int) * 3 * m->nf, cudaMemcpyDeviceToHost));
  if (m->ne) TM_CUDA(cudaMemcpy(ed.data(), m->d_edge.get(), sizeof(int4) * m->ne, cudaMemcpyDeviceToHost));
  const int nc = (int)runs.size();
  std::vector<BatchClass> cls(nc);
  bool ok = nc <= TM_MAX_CLASSES;
  for (int c = 0; c < nc && ok; ++c) {
    cls[c].v0 = b->voff[runs[c].first];
    cls[c].v1 = b->voff[runs[c].second];
    cls[c].f0 = cls[c].e0 = INT_MAX;
    cls[c].f1 = cls[c].e1 = -1;
  }
  std::vector<int> fcount(nc, 0), ecount(nc, 0);
  for (int f = 0; f < m->nf && ok; ++f) {
    const int c = rcls[vrep[fv[3 * (size_t)f]]];
    cls[c].f0 = std::min(cls[c].f0, f);
    cls[c].f1 = std::max(cls[c].f1, f + 1);
    ++fcount[c];
  }
  for (int e = 0; e < m->ne && ok; ++e) {
    const int c = rcls[vrep[ed[e].x]];
    cls[c].e0 = std::min(cls[c].e0, e);
    cls[c].e1 = std::max(cls[c].e1, e + 1);
    ++ecount[c];
  }
  for (int c = 0; c < nc && ok; ++c)
    ok = cls[c].f1 - cls[c].f0 == fcount[c] && cls[c].e1 - cls[c].e0 == ecount[c];
  if (!ok) cls.assign(1, BatchClass{0, m->nv, 0, m->nf, 0, m->ne, {256, 256, 256, 256}});
  for (BatchClass& c : cls)
    for (int k = 0; k < 4; ++k) c.blk[k] = 256;
  b->cls = cls;
  if (cls.size() > 1) {
    for (size_t c = 0; c < cls.size(); ++c) {
      TM_CUDA(cudaStreamCreateWithFlags(&b->bs.cs[c], cudaStreamNonBlocking));
      TM_CUDA(cudaEventCreateWithFlags(&b->bs.join[c], cudaEventDisableTiming));
    }
    TM_CUDA(cudaEventCreateWithFlags(&b->bs.fork[0], cudaEventDisableTiming));
    TM_CUDA(cudaEventCreateWithFlags(&b->bs.fork[1], cudaEventDisableTiming));
    b->have_side = true;
  }
}

// The autotuner: for every size class and element kernel (split, face,
// edge, gradient), the block size among 64 .. 512 (the gradient kernel is
// built for at most 256) with the shortest median of five timed launches
// of that class's kernel alone, after a full evaluation has filled its
// inputs.
static void autotune(tm_batch* b) {
  const int cand[4] = {64, 128, 256, 512};
  cudaEvent_t e0, e1;
  TM_CUDA(cudaEventCreate(&e0));
  TM_CUDA(cudaEventCreate(&e1));
  cudaStream_t s = b->stream;
  batch_eval(b, b->x.get(), b->g0.get(), s);
  for (BatchClass& c : b->cls) {
    for (int k = 0; k < 4; ++k) {
      float best = 1e30f;
      int bestb = 256;
      for (int bsz : cand) {
        if (k == 3 && bsz > 256) continue;
        batch32_class_kernel(k, c, bsz, b->en.get(), b->mesh.get(), b->x.get(), b->g0.get(), b->eps.get(),
                             b->vrep.get(), b->gs.get(), s);  // warm
        std::vector<float> t;
        for (int rep = 0; rep < 5; ++rep) {
          TM_CUDA(cudaEventRecord(e0, s));
          batch32_class_kernel(k, c, bsz, b->en.get(), b->mesh.get(), b->x.get(), b->g0.get(), b->eps.get(),
                               b->vrep.get(), b->gs.get(), s);
          TM_CUDA(cudaEventRecord(e1, s));
          TM_CUDA(cudaEventSynchronize(e1));
          float ms = 0;
          TM_CUDA(cudaEventElapsedTime(&ms, e0, e1));
          t.push_back(ms);
        }
        std::sort(t.begin(), t.end());
        if (t[2] < best) {
          best = t[2];
          bestb = bsz;
        }
      }
      c.blk[k] = bestb;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
}

extern "C" {

int tm_batch_create(int n_rep, const double* const* points, const int64_t* n_points, const int32_t* const* faces,
                    const int64_t* n_faces, const tm_params* params, tm_batch** out) {
  TM_API_BEGIN
  if (!out || n_rep < 1 || !points || !n_points || !faces || !n_faces || !params) fail(TM_ERR_ARG, "NULL argument");
  *out = nullptr;
  std::unique_ptr<tm_batch> b(new tm_batch());
  b->R = n_rep;
  for (int r = 0; r < n_rep; ++r) {
    if (params[r].n_search != 0 && params[r].n_search != 1) fail(TM_ERR_ARG, "Unknown neighbour search algorithm.");
    if (params[r].n_search != params[0].n_search)
      fail(TM_ERR_ARG, "the replicas of a batch use one neighbour search (cell list or Verlet list)");
    if (params[r].bond_type != 0 && params[r].bond_type != 1) fail(TM_ERR_ARG, "Unknown bond potential");
    if (params[r].exclusion_level < 0 || params[r].exclusion_level > 2) fail(TM_ERR_ARG, "Unsupported exclusion level");
    b->prm.push_back(params[r]);
  }
  // union layout: replica ranges padded to multiples of 256 vertices
  b->voff.assign(n_rep + 1, 0);
  for (int r = 0; r < n_rep; ++r) {
    if (n_points[r] < 3) fail(TM_ERR_ARG, "replica with fewer than three vertices");
    b->nreal.push_back((int)n_points[r]);
    b->voff[r + 1] = b->voff[r] + (int)((n_points[r] + B - 1) / B) * B;
  }
  int nv = b->voff[n_rep];
  b->nv = nv;
  std::vector<double> P(3 * (size_t)nv, 0.0);
  std::vector<int32_t> F;
  std::vector<int> vrep(nv, -1);
  std::vector<int2> rb(n_rep);
  for (int r = 0; r < n_rep; ++r) {
    std::memcpy(&P[3 * (size_t)b->voff[r]], points[r], sizeof(double) * 3 * n_points[r]);
    for (int64_t f = 0; f < 3 * n_faces[r]; ++f) {
      int x = faces[r][f];
      F.push_back(x >= 0 && x < n_points[r] ? x + b->voff[r] : -1);
    }
    for (int v = 0; v < n_points[r]; ++v) vrep[b->voff[r] + v] = r;
    rb[r] = make_int2(b->voff[r] / B, b->voff[r + 1] / B);
  }
  TM_CUDA(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking));
  tm_mesh* mraw = nullptr;
  int rc = tm_mesh_create(P.data(), nv, F.data(), (int64_t)F.size() / 3, &mraw);
  if (rc) return rc;
  b->mesh.reset(mraw);
  b->en.reset(new tm_energy());
  b->en->prm = params[0];
  b->en->stream = nullptr;
  b->vrep.ensure(nv);
  b->rblocks.ensure(n_rep);
  b->eps.ensure(n_rep);
  b->gs.ensure(n_rep);
  b->rlist.ensure(n_rep);
  b->x.ensure(3 * (size_t)nv);
  b->xs.ensure(3 * (size_t)nv);
  b->p.ensure(3 * (size_t)nv);
  b->g0.ensure(3 * (size_t)nv);
  b->g1.ensure(3 * (size_t)nv);
  b->part.ensure(nv / B + 1);
  b->sc.ensure(4 * (size_t)n_rep);
  b->flag.ensure(n_rep);
  b->acc.ensure(n_rep);
  b->counter.ensure(1);
  std::vector<double> rl(n_rep);
  std::vector<int> rx(n_rep);
  for (int r = 0; r < n_rep; ++r) {
    rl[r] = params[r].rlist;
    rx[r] = params[r].exclusion_level;
  }
  b->rexcl.ensure(n_rep);
  cudaStream_t s = b->stream;
  TM_CUDA(cudaMemcpyAsync(b->vrep.get(), vrep.data(), sizeof(int) * nv, cudaMemcpyHostToDevice, s));
  TM_CUDA(cudaMemcpyAsync(b->rblocks.get(), rb.data(), sizeof(int2) * n_rep, cudaMemcpyHostToDevice, s));
  TM_CUDA(cudaMemcpyAsync(b->rlist.get(), rl.data(), sizeof(double) * n_rep, cudaMemcpyHostToDevice, s));
  TM_CUDA(cudaMemcpyAsync(b->rexcl.get(), rx.data(), sizeof(int) * n_rep, cudaMemcpyHostToDevice, s));
  TM_CUDA(cudaMemcpyAsync(b->x.get(), P.data(), sizeof(double) * 3 * nv, cudaMemcpyHostToDevice, s));
  TM_CUDA(cudaMemsetAsync(b->gs.get(), 0, sizeof(Globals) * n_rep, s));
  TM_CUDA(cudaMemsetAsync(b->acc.get(), 0, sizeof(int) * n_rep, s));
  TM_CUDA(cudaMemsetAsync(b->counter.get(), 0, sizeof(unsigned long long), s));
  // initial properties per replica (the reference state of the penalties):
  // an FP64 evaluation of each replica on its own, as an energy manager of
  // that mesh computes them at construction (src/energy.cpp:13-28)
  b->initial.assign(6 * (size_t)n_rep, 0.0);
  for (int r = 0; r < n_rep; ++r) {
    tm_mesh* mr = nullptr;
    tm_energy* er = nullptr;
    rc = tm_mesh_create(points[r], n_points[r], faces[r], n_faces[r], &mr);
    if (rc) return rc;
    std::unique_ptr<tm_mesh> hold_m(mr);
    rc = tm_energy_create(mr, &params[r], &er);
    if (rc) return rc;
    std::unique_ptr<tm_energy> hold_e(er);
    std::memcpy(&b->initial[6 * r], er->initial, sizeof(double) * 6);
  }
  upload_eps(b.get());
  rebuild_nlist(b.get());
  make_classes(b.get());
  autotune(b.get());
  *out = b.release();
  TM_API_END
}

int tm_batch_tuning(tm_batch* b, int32_t* n_classes, int32_t* info) {
  TM_API_BEGIN
  if (!b || !n_classes) fail(TM_ERR_ARG, "NULL argument");
  *n_classes = (int32_t)b->cls.size();
  if (info)
    for (size_t c = 0; c < b->cls.size(); ++c) {
      const BatchClass& k = b->cls[c];
      const int32_t row[6] = {k.v0, k.v1, k.blk[0], k.blk[1], k.blk[2], k.blk[3]};
      std::memcpy(info + 6 * c, row, sizeof row);
    }
  TM_API_END
}

int tm_batch_destroy(tm_batch* b) {
  delete b;
  return TM_OK;
}

int tm_batch_layout(tm_batch* b, int64_t* n_total, int64_t* offsets) {
  if (!b) return TM_ERR_ARG;
  if (n_total) *n_total = b->nv;
  if (offsets)
    for (int r = 0; r <= b->R; ++r) offsets[r] = b->voff[r];
  return TM_OK;
}

int tm_batch_positions(tm_batch* b, double* host_x, int direction) {
  TM_API_BEGIN
  if (!b || !host_x) fail(TM_ERR_ARG, "NULL argument");
  size_t bytes = sizeof(double) * 3 * b->nv;
  if (direction == 0)
    TM_CUDA(cudaMemcpyAsync(host_x, b->x.get(), bytes, cudaMemcpyDeviceToHost, b->stream));
  else
    TM_CUDA(cudaMemcpyAsync(b->x.get(), host_x, bytes, cudaMemcpyHostToDevice, b->stream));
  TM_CUDA(cudaStreamSynchronize(b->stream));
  TM_API_END
}

int tm_batch_energy(tm_batch* b, double* energies, double* grad) {
  TM_API_BEGIN
  if (!b || !energies) fail(TM_ERR_ARG, "NULL argument");
  batch_eval(b, b->x.get(), b->g0.get(), b->stream);
  std::vector<Globals> g(b->R);
  TM_CUDA(cudaMemcpyAsync(g.data(), b->gs.get(), sizeof(Globals) * b->R, cudaMemcpyDeviceToHost, b->stream));
  if (grad)
    TM_CUDA(cudaMemcpyAsync(grad, b->g0.get(), sizeof(double) * 3 * b->nv, cudaMemcpyDeviceToHost, b->stream));
  TM_CUDA(cudaStreamSynchronize(b->stream));
  for (int r = 0; r < b->R; ++r) energies[r] = g[r].comps[6];
  TM_API_END
}

int tm_batch_update_repulsion(tm_batch* b) {
  TM_API_BEGIN
  if (!b) fail(TM_ERR_ARG, "NULL argument");
  rebuild_nlist(b);
  TM_CUDA(cudaStreamSynchronize(b->stream));
  TM_API_END
}

int tm_batch_set_refresh(tm_batch* b, int every) {
  TM_API_BEGIN
  if (!b || every < 0) fail(TM_ERR_ARG, "invalid argument");
  b->refresh = every;
  TM_API_END
}

int tm_batch_hmc(tm_batch* b, int n_steps, int n_leapfrog, double dt, double mass, double temperature,
                 uint64_t seed, int use_graph, int32_t* accepted) {
  TM_API_BEGIN
  if (!b || n_steps < 0 || n_leapfrog < 0 || !(mass > 0) || !(temperature > 0)) fail(TM_ERR_ARG, "invalid argument");
  cudaStream_t s = b->stream;
  TM_CUDA(cudaMemsetAsync(b->acc.get(), 0, sizeof(int) * b->R, s));
  for (int k = 0; k < n_steps; ++k) {
    if (use_graph) {
      // the graph holds one step with the current neighbour-list view; a
      // rebuild that moved or resized a buffer invalidates it
      const NLView& v = b->en->nl.view;
      bool same = b->gexec && b->g_L == n_leapfrog && b->g_dt == dt && b->g_m == mass &&
                  b->g_T == temperature && b->g_seed == seed && std::memcmp(&b->g_view, &v, sizeof(NLView)) == 0;
      if (same) {
        TM_CUDA(cudaGraphLaunch(b->gexec, s));
      } else {
        if (b->gexec) cudaGraphExecDestroy(b->gexec);
        if (b->graph) cudaGraphDestroy(b->graph);
        b->gexec = nullptr;
        b->graph = nullptr;
        batch_hmc_step(b, n_leapfrog, dt, mass, temperature, seed, s);  // allocations happen outside capture
        TM_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
        batch_hmc_step(b, n_leapfrog, dt, mass, temperature, seed, s);
        TM_CUDA(cudaStreamEndCapture(s, &b->graph));
        TM_CUDA(cudaGraphInstantiate(&b->gexec, b->graph, 0));
        b->g_L = n_leapfrog;
        b->g_dt = dt;
        b->g_m = mass;
        b->g_T = temperature;
        b->g_seed = seed;
        std::memcpy(&b->g_view, &v, sizeof(NLView));
      }
    } else {
      batch_hmc_step(b, n_leapfrog, dt, mass, temperature, seed, s);
    }
    ++b->steps_done;
    if (b->refresh > 0 && b->steps_done % b->refresh == 0) rebuild_nlist(b, false);
  }
  if (accepted)
    TM_CUDA(cudaMemcpyAsync(accepted, b->acc.get(), sizeof(int) * b->R, cudaMemcpyDeviceToHost, s));
  TM_CUDA(cudaStreamSynchronize(s));
  TM_API_END
}

}  // extern "C"
