// Surface repulsion stage of an evaluation (src/mesh_repulsion.h:28-79 over
// the neighbour list): per vertex the flat-bottom pair potential
// sum_j exp(l/(l - lc1)) / l^r over the neighbours closer than lc1 and, for a
// gradient, 2 sum_j phi'(l) (x_i - x_j) / l.
//
// While no vertex has moved lc1/2 since the near rows were built (k_moved
// decides this for the whole mesh before the pass) every vertex walks its
// near row in k_rep_fast.  Otherwise a vertex whose current position still
// lies in its build-time cell walks the precomputed candidate row of that
// cell; the few that moved
// to another cell are queued and walk the 27 cells through the cell table in
// a second kernel (k_rep_slow), so the long table walk never holds a warp of
// fast vertices.  Both produce the per-vertex values in the reference's pair
// order; the queue order does not matter because each vertex is written by
// one thread.
#include <algorithm>

#include "tm_energy.cuh"
#include "tm_internal.h"
#include "tm_math.cuh"

namespace tmg {
namespace {

struct RepAcc {
  double lc1;
  int rr;
  double pot;
  d3 gr;
  bool grad;
  __device__ void operator()(int, double l, d3 dvec) {
    double lmc = l - lc1;
    double ex = exp(l / lmc);
    pot += ex / ipow(l, rr);
    if (grad) {
      double fac = -(lc1 / (lmc * lmc) + rr / l);
      fac /= ipow(l, rr + 1);
      fac *= ex;
      gr += fac * dvec;
    }
  }
};

template <bool GRAD>
__global__ void __launch_bounds__(256) k_rep_fast(Topo t, const double* __restrict__ P, NLView nl, EP ep,
                                                 double* __restrict__ pot, double* __restrict__ repg,
                                                 int* __restrict__ slow, int* __restrict__ nslow,
                                                 const EP* __restrict__ eps, int use_near) {
  int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= t.nv) return;
  if (nl.vrep) {  // batch: per-replica cut-off, padding vertices have none
    int r = nl.vrep[v];
    if (r < 0) {
      pot[v] = 0.0;
      if (GRAD) st3(repg, v, mk(0, 0, 0));
      return;
    }
    ep = eps[r];
  }
  // near rows usable: built, no vertex moved lc1/2 since (flags written by
  // the previous kernels); mode 1 while the topology is the rows' one
  int near_mode = 0;
  if (use_near && nl.nflag[0] == 0 && nl.nflag[1] == 0) near_mode = nl.nflag[2] == *nl.dtopo ? 1 : 2;
  d3 p = ld3(P, v);
  PairTest pt = make_pair_test(nl, v, ep.rlc1, ep.rT);
  RepAcc acc{ep.rlc1, ep.rr, 0.0, mk(0, 0, 0), GRAD};
  TableExcl x{t, nl.excl, &nl};
  if (nl.kind == 0) {
    int co[3];
    bool fast = in_build_cell(nl, v, p, co);
    if (near_mode) fast = visit_near(pt, nl, P, v, p, near_mode, co, x, acc);
    warp_append(!fast, v, slow, nslow);
    if (!fast) return;
    if (!near_mode) visit_candidates(pt, nl, P, v, p, x, acc);
  } else {
    visit_verlet(pt, nl, P, v, p, x, acc);
  }
  pot[v] = acc.pot;
  if (GRAD) st3(repg, v, 2.0 * acc.gr);
}

// One warp per queued vertex: lane l < 27 scans neighbour cell l (the
// reference's x-outer / z-inner order), then the lanes' sums are combined by
// a fixed shuffle tree, so the result does not depend on timing.
template <bool GRAD>
__global__ void __launch_bounds__(256) k_rep_slow(Topo t, const double* __restrict__ P, NLView nl, EP ep0,
                                                 double* __restrict__ pot, double* __restrict__ repg,
                                                 const int* __restrict__ slow, const int* __restrict__ nslow,
                                                 const EP* __restrict__ eps) {
  int n = *nslow;
  int lane = threadIdx.x & 31;
  int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  int nwarps = (gridDim.x * blockDim.x) >> 5;
  TableExcl x{t, nl.excl, &nl};
  for (int i = warp; i < n; i += nwarps) {
    int v = slow[i];
    const NLGeom& G = geom_of(nl, v);
    const int rep = rep_of(nl, v);
    const EP& ep = nl.vrep ? eps[rep] : ep0;
    d3 p = ld3(P, v);
    PairTest pt = make_pair_test(nl, v, ep.rlc1, ep.rT);
    RepAcc acc{ep.rlc1, ep.rr, 0.0, mk(0, 0, 0), GRAD};
    int co[3];
    in_build_cell(nl, v, p, co);
    if (lane < 27) {
      int ii = co[0] + lane / 9 - 1, jj = co[1] + (lane / 3) % 3 - 1, kk = co[2] + lane % 3 - 1;
      if (ii >= 0 && ii < G.shape[0] && jj >= 0 && jj < G.shape[1] && kk >= 0 && kk < G.shape[2]) {
        long long cid = ii * G.stride[0] + jj * G.stride[1] + kk * G.stride[2];
        int st = 0;
        int cnt = cell_find(nl, cell_key(cid, rep), &st);
        for (int q = 0; q < cnt; ++q) {
          int j = nl.cell_verts[st + q];
          if (j != v) visit_pair(pt, nl, P, v, p, j, x, acc);
        }
      }
    }
    double s = acc.pot, gx = acc.gr.x, gy = acc.gr.y, gz = acc.gr.z;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      s += __shfl_down_sync(0xffffffffu, s, o);
      if (GRAD) {
        gx += __shfl_down_sync(0xffffffffu, gx, o);
        gy += __shfl_down_sync(0xffffffffu, gy, o);
        gz += __shfl_down_sync(0xffffffffu, gz, o);
      }
    }
    if (lane == 0) {
      pot[v] = s;
      if (GRAD) st3(repg, v, 2.0 * mk(gx, gy, gz));
    }
  }
}

// flag = 1 when some vertex is lc1/2 or farther from where the near rows
// were built (squared threshold thr2, rounded down); NaN counts as moved
__global__ void k_moved(int nv, const double* __restrict__ P, const double* __restrict__ xb, double thr2,
                        int* flag, const int* __restrict__ vrep, const EP* __restrict__ eps) {
  int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= nv) return;
  if (vrep) {  // batch: the replica's skin, padding vertices never move
    int r = vrep[v];
    if (r < 0) return;
    thr2 = 0.25 * eps[r].rlc1 * eps[r].rlc1 * (1.0 - 1e-12);
  }
  double dx = P[3 * v] - xb[3 * v], dy = P[3 * v + 1] - xb[3 * v + 1], dz = P[3 * v + 2] - xb[3 * v + 2];
  if (!(dx * dx + dy * dy + dz * dz < thr2)) atomicOr(flag, 1);
}

inline int nblk(long n, int b) { return (int)((n + b - 1) / b); }

}  // namespace

void repulsion_eval(tm_energy* e, tm_mesh* m, const double* P, const float* pos32, bool want_grad,
                    double* pot, double* repg, int* slow, int* nslow, cudaStream_t s, const EP* eps) {
  int nv = m->nv;
  if (nv == 0) return;
  EP ep = make_ep(e);
  if (!eps && !(ep.rlc1 > 0)) {  // no pair can be closer than a non-positive cut-off
    TM_CUDA(cudaMemsetAsync(pot, 0, sizeof(double) * nv, s));
    if (want_grad) TM_CUDA(cudaMemsetAsync(repg, 0, sizeof(double) * 3 * nv, s));
    return;
  }
  Topo t = m->topo();
  NLView nlv = e->nl.view;
  nlv.pos32 = pos32;
  TM_CUDA(cudaMemsetAsync(nslow, 0, sizeof(int), s));
  int use_near = 0;
  if (nlv.kind == 0 && nlv.nent && e->nl.near_nv == nv && (eps || e->nl.near_lc1 == ep.rlc1)) {
    use_near = 1;
    int* flag = e->nl.nflag.get();
    TM_CUDA(cudaMemsetAsync(flag, 0, sizeof(int), s));
    k_moved<<<nblk(nv, 256), 256, 0, s>>>(nv, P, e->nl.xb.get(), e->nl.near_move2, flag, nlv.vrep, eps);
    TM_LAUNCH();
  }
  if (want_grad)
    k_rep_fast<true><<<nblk(nv, 256), 256, 0, s>>>(t, P, nlv, ep, pot, repg, slow, nslow, eps, use_near);
  else
    k_rep_fast<false><<<nblk(nv, 256), 256, 0, s>>>(t, P, nlv, ep, pot, repg, slow, nslow, eps, use_near);
  TM_LAUNCH();
  if (nlv.kind == 0) {
    int grid = 8 * 152;  // 8 warps per block, one warp per queued vertex (all of them when the near rows are stale)
    if (want_grad)
      k_rep_slow<true><<<grid, 256, 0, s>>>(t, P, nlv, ep, pot, repg, slow, nslow, eps);
    else
      k_rep_slow<false><<<grid, 256, 0, s>>>(t, P, nlv, ep, pot, repg, slow, nslow, eps);
    TM_LAUNCH();
  }
}

void fork_repulsion(tm_energy* e, tm_mesh* m, const double* P, bool want_grad, cudaStream_t s, bool concurrent) {
  const int n1 = std::max(m->nv, 1);
  if (!concurrent || !e->aux) {
    repulsion_eval(e, m, P, e->pos32.get(), want_grad, e->reppot.get(), e->repg.get(), e->slow.get(),
                   e->slow.get() + n1, s);
    return;
  }
  TM_CUDA(cudaEventRecord(e->ev_fork, s));
  TM_CUDA(cudaStreamWaitEvent(e->aux, e->ev_fork, 0));
  repulsion_eval(e, m, P, e->pos32.get(), want_grad, e->reppot.get(), e->repg.get(), e->slow.get(),
                 e->slow.get() + n1, e->aux);
  TM_CUDA(cudaEventRecord(e->ev_join, e->aux));
}

void join_repulsion(tm_energy* e, cudaStream_t s, bool concurrent) {
  if (concurrent && e->aux) TM_CUDA(cudaStreamWaitEvent(s, e->ev_join, 0));
}

}  // namespace tmg
