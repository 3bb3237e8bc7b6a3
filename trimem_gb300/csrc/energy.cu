// Energy manager: vertex properties, penalty assembly and gradient.
//
// The reference evaluates, per vertex, every incident face and edge again
// (src/mesh_properties.cpp:12-148), i.e. each face three times and each edge
// two to four times per pass, with acos/tan per call.  On GB300 (FP64 issue
// rate ~1/58 of FP32) the kernels instead compute each face and each edge once
// per evaluation and gather them per vertex:
//
//   k_face   (one thread per face)  unit normal, area, signed volume and the
//            cotangents of the three corners (u.v / |u x v|, no acos/tan)
//   k_edge   (one thread per edge)  length, signed dihedral angle, tether
//            bond value and derivative
//   k_vertex (one thread per vertex) area/volume/curvature/tether sums of
//            the ring, bending 2c^2/a, repulsion (and its gradient), a
//            fixed-order block reduction of the six global sums; the last
//            block reduces the block partials in fixed order and assembles
//            energy and the penalty gradient factors on the device
//   k_grad   (one thread per vertex) gather of dE/dx_i over the ring
//
// No atomics touch floating-point data, so every result is bit-reproducible.
// With w_e = gC/2 + kb (rho_i + rho_j) (rho = curvature/area per vertex) the
// gradient is
//   sum_f [gA - 2/3 kb (rho_a^2+rho_b^2+rho_c^2) (+ kt dpen)] dA_f
//   + gV dV_f + sum_e (w_e theta_e + kt dbond_e) dl_e + w_e l_e dtheta_e
//   + kr drep,
// which is the reference's gather (src/mesh_properties.cpp:51-148 with
// src/kernel.h:124-137) regrouped per face and edge.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <memory>
#include <vector>

#include "tm_internal.h"
#include "tm_math.cuh"
#include "tm_energy.cuh"

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

namespace tmg {

// ---- per-face and per-edge quantities ------------------------------------
// Sign tests and absolute values as integer operations on the bits (no
// FP64 compare or absolute value: FP64 is GB300's scarce pipe).  The sign
// bit of an edge's il is its boundary flag; for non-negative doubles the
// bit patterns order like the values, so a length l >= 0 is compared with
// a threshold by its bits (NaN lengths compare as above every threshold).
__device__ __forceinline__ bool interior_edge(double il) { return __double_as_longlong(il) >= 0; }
__device__ __forceinline__ double abs_bits(double x) {
  return __longlong_as_double(__double_as_longlong(x) & 0x7fffffffffffffffLL);
}
__device__ __forceinline__ bool len_below(double l, double c) {
  return __double_as_longlong(l) < __double_as_longlong(c);
}
__device__ __forceinline__ bool len_above(double l, double c) {
  return __double_as_longlong(l) > __double_as_longlong(c);
}
// fav: (area, volume) of each face again, compact, for k_vertex's gathers
__global__ void k_face(Topo t, const double* __restrict__ P, FaceD* __restrict__ fd, float* __restrict__ P32,
                       double2* __restrict__ fav) {
  int f = blockIdx.x * blockDim.x + threadIdx.x;
  // the float copy of the positions used by the neighbour prefilter
  for (int v = f; v < t.nv; v += gridDim.x * blockDim.x) {
    P32[3 * v] = (float)P[3 * v];
    P32[3 * v + 1] = (float)P[3 * v + 1];
    P32[3 * v + 2] = (float)P[3 * v + 2];
  }
  if (f >= t.nf) return;
  int a = t.fv[3 * f], b = t.fv[3 * f + 1], c = t.fv[3 * f + 2];
  d3 pa = ld3(P, a), pb = ld3(P, b), pc = ld3(P, c);
  d3 eab = pb - pa, eac = pc - pa, ebc = pc - pb;
  d3 N = cross(eab, eac);
  double n2 = dot(N, N);
  double inv = rsqrt(n2);
  double nn = n2 * inv;
  FaceD F;
  F.nx = N.x * inv;
  F.ny = N.y * inv;
  F.nz = N.z * inv;
  F.A = 0.5 * nn;
  // (p_a x p_b) . p_c = p_a . ((p_b - p_a) x (p_c - p_a)) = p_a . N
  F.V = dot(pa, N) * (1.0 / 6.0);
  F.c0 = dot(eab, eac) * inv;
  F.c1 = -dot(eab, ebc) * inv;
  F.c2 = dot(eac, ebc) * inv;
  fd[f] = F;
  fav[f] = make_double2(F.A, F.V);
}

// elt: (l theta, bond value) of each edge, compact, for k_vertex's gathers
// (the bond value of short edges is filled in by k_bond_short)
__global__ void k_edge(Topo t, const double* __restrict__ P, const FaceD* __restrict__ fd, EdgeD* __restrict__ ed,
                       double2* __restrict__ elt, EP ep, int* __restrict__ blist, int* __restrict__ bcnt,
                       const double2* __restrict__ sct) {
  int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= t.ne) return;
  int4 E = t.edge[e];
  d3 pi = ld3(P, E.x), pj = ld3(P, E.y);
  d3 ev = pj - pi;
  double l2 = dot(ev, ev);
  double il = rsqrt(l2);
  double l = l2 * il;
  EdgeD o;
  o.l = l;
  o.th = 0.0;
  o.il = -il;
  if (E.z >= 0 && E.w >= 0) {
    FaceD F0 = fd[E.z], F1 = fd[E.w];
    d3 n0 = mk(F0.nx, F0.ny, F0.nz), n1 = mk(F1.nx, F1.ny, F1.nz);
    // both normals are perpendicular to the shared edge, so n0 x n1 lies
    // along it: its projection on the unit edge is the signed sine, whose
    // sign is the reference's sign test (n0 x n1) . e >= 0
    double sd = dot(cross(n0, n1), ev) * il;
    double a = angle_sc(abs_bits(sd), dot(n0, n1), sct);
    o.th = sd >= 0.0 ? a : -a;
    o.il = il;
  }
  // flat-bottom edge penalty: above the flat bottom inline (products only,
  // edge_bond's l > lc0 branch); edges below it (exp and a division in
  // FP64) go to a list handled by k_bond_short so that whole warps do not
  // wait on a few lanes
  double val = 0.0, fac = 0.0;
  const bool shortb = ep.btype == 0 && len_below(l, ep.lc1);
  if (ep.btype == 0 && !shortb && len_above(l, ep.lc0)) {
    const double d = l - ep.lc0;
    val = ep.br1 * ipow(d, ep.r);
    fac = ep.br2 * ipow(d, ep.r - 1);
  }
  warp_append(shortb, e, blist, bcnt);
  o.db = fac;
  ed[e] = o;
  elt[e] = make_double2(o.l * o.th, val);
}

__global__ void k_bond_short(const double* __restrict__ P, Topo t, EdgeD* __restrict__ ed,
                             double2* __restrict__ elt, EP ep, const int* __restrict__ blist,
                             const int* __restrict__ bcnt) {
  int n = *bcnt;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    int e = blist[i];
    double val, fac;
    const EdgeD E = ed[e];
    edge_bond(ep, E.l, fabs(E.il), &val, &fac);
    ed[e].db = fac;
    elt[e].y = val;
  }
}

constexpr int VG = 6;  // ring slots loaded together by k_vertex
template <bool VPROPS>
__global__ void __launch_bounds__(VB) k_vertex(Topo t, const double2* __restrict__ fav,
                                              const double2* __restrict__ elt, const double* __restrict__ reppot,
                                              EP ep, double2* __restrict__ rk, double* __restrict__ vprops,
                                              double* __restrict__ partial, Globals* g) {
  __shared__ double red[6][VB];
  __shared__ bool last;
  int v = blockIdx.x * VB + threadIdx.x;
  double pr[6] = {0, 0, 0, 0, 0, 0};
  if (v < t.nv) {
    int d = t.val[v];
    double A = 0, V = 0, LT = 0, T = 0;
    // slots in groups of six (one group at the usual valence): all loads of
    // a group are issued before the sums, which keep the slot order
    for (int m0 = 0; m0 < d; m0 += VG) {
      int4 s[VG];
#pragma unroll
      for (int k = 0; k < VG; ++k) s[k] = m0 + k < d ? t.slot[(size_t)(m0 + k) * t.nv + v] : make_int4(0, -1, 0, 0);
      double fa[VG], fv[VG], lt[VG], tb[VG];
#pragma unroll
      for (int k = 0; k < VG; ++k) {
        int f = slot_face(s[k].y);
        fa[k] = fv[k] = lt[k] = tb[k] = 0.0;
        if (f >= 0) {
          const double2 av = fav[f], lb = elt[s[k].z];
          fa[k] = av.x;
          fv[k] = av.y;
          lt[k] = lb.x;
          if (ep.btype == 0) tb[k] = lb.y;
        }
      }
#pragma unroll
      for (int k = 0; k < VG; ++k) {
        if (slot_face(s[k].y) < 0) continue;
        A += fa[k];
        V += fv[k];
        LT += lt[k];
        if (ep.btype == 0) {
          T += tb[k];
        } else {
          double q = fa[k] / ep.a0 - 1.0;
          T += q * q;
        }
      }
    }
    double a = A * (1.0 / 3.0), c = 0.25 * LT;
    double ia = 1.0 / a;
    pr[0] = a;
    pr[1] = V * (1.0 / 3.0);
    pr[2] = c;
    pr[3] = 2 * c * c * ia;
    pr[4] = T * ep.itdiv;
    pr[5] = reppot[v];
    const double rho = c * ia;
    rk[v] = make_double2(ep.kb * rho, (ep.kb * (2.0 / 3.0)) * (rho * rho));
    if (VPROPS)
      for (int k = 0; k < 6; ++k) vprops[6 * (size_t)v + k] = pr[k];
  }
  for (int k = 0; k < 6; ++k) red[k][threadIdx.x] = pr[k];
  __syncthreads();
  for (int o = VB / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o)
      for (int k = 0; k < 6; ++k) red[k][threadIdx.x] += red[k][threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    for (int k = 0; k < 6; ++k) partial[8 * (size_t)blockIdx.x + k] = red[k][0];
    __threadfence();
    unsigned int tk = atomicAdd(&g->ticket, 1u);
    last = (tk == gridDim.x - 1);
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  // last block: fixed-order reduction of the block partials
  double acc[6] = {0, 0, 0, 0, 0, 0};
  for (int b = threadIdx.x; b < (int)gridDim.x; b += VB)
    for (int k = 0; k < 6; ++k) acc[k] += ((volatile double*)partial)[8 * (size_t)b + k];
  for (int k = 0; k < 6; ++k) red[k][threadIdx.x] = acc[k];
  __syncthreads();
  for (int o = VB / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o)
      for (int k = 0; k < 6; ++k) red[k][threadIdx.x] += red[k][threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    for (int k = 0; k < 6; ++k) g->props[k] = red[k][0];
    assemble(ep, g);
    g->ticket = 0;
  }
}

__global__ void k_assemble_props(EP ep, const double* props6, Globals* g) {
  if (threadIdx.x || blockIdx.x) return;
  for (int k = 0; k < 6; ++k) g->props[k] = props6[k];
  assemble(ep, g);
}

// ---- gradient gather ------------------------------------------------------
// rk[v] = (kb rho_v, 2/3 kb rho_v^2), written by k_vertex
__global__ void __launch_bounds__(256) k_grad(Topo t, const double* __restrict__ P, const FaceD* __restrict__ fd,
                                             const EdgeD* __restrict__ ed, const double2* __restrict__ rk,
                                             const double* __restrict__ repg, const Globals* __restrict__ g, EP ep,
                                             double* __restrict__ grad) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= t.nv) return;
  const double gA = g->gA, gV = g->gV, gC = g->gC;
  const double hgC = 0.5 * gC;
  d3 xi = ld3(P, i);
  const double2 qi = rk[i];
  const double ai = gA - qi.y;   // alpha = gA - 2/3 kb (rho_i^2 + rho_j^2 + rho_k^2)
  const double wi = hgC + qi.x;  // w = gC/2 + kb (rho_i + rho_j)
  d3 acc = ep.kr * ld3(repg, i);
  int d = t.val[i];
  if (d > 0) {
    const size_t nv = t.nv;
    int4 sp = t.slot[(size_t)(d - 1) * nv + i];
    d3 xk = ld3(P, sp.x);
    double2 qk = rk[sp.x];
    int4 sc = t.slot[i];
    d3 xj = ld3(P, sc.x);
    double2 qj = rk[sc.x];
    FaceD Fc;
    int fcur = slot_face(sc.y);
    if (fcur >= 0) Fc = fd[fcur];
    const double gV6 = gV * (1.0 / 6.0);
    // scalar multiples of face normals are summed per face: the dihedral
    // term of edge (i, j) reaches the normal of the next face, so its part
    // is carried to the next slot (the last one wraps to the first face)
    double carry = 0.0;
    d3 n0 = mk(0, 0, 0);
    // length terms s_j (x_j - x_i): sum s_j x_j here, - (sum s_j) x_i at the end
    double ssum = 0.0;
    for (int m = 0; m < d; ++m) {
      int4 sn = t.slot[(size_t)((m + 1) == d ? 0 : m + 1) * nv + i];
      int fnx = slot_face(sn.y);
      FaceD Fn;
      if (fnx >= 0) Fn = fd[fnx];
      double carry_next = 0.0;
      if (fcur >= 0) {
        int ci = slot_corner(sc.y);
        double cj = cot_at(Fc, ci == 2 ? 0 : ci + 1);
        double ck = cot_at(Fc, ci == 0 ? 2 : ci - 1);
        d3 n = mk(Fc.nx, Fc.ny, Fc.nz);
        if (m == 0) n0 = n;
        // face (i, j, k): area and volume terms, (alpha/2) n x (x_k - x_j)
        // + (gV/6) x_j x x_k = ((alpha/2) n + (gV/6) x_j) x (x_k - x_j)
        double alpha = (ai - qj.y) - qk.y;
        if (ep.btype == 1) alpha += ep.kt * 2.0 * (Fc.A / ep.a0 - 1.0) / ep.a0;
        d3 u = (0.5 * alpha) * n + gV6 * xj;
        d3 e = xk - xj;
        acc.x = fma(u.y, e.z, fma(-u.z, e.y, acc.x));
        acc.y = fma(u.z, e.x, fma(-u.x, e.z, acc.y));
        acc.z = fma(u.x, e.y, fma(-u.y, e.x, acc.z));
        // edge (i, j): length and dihedral terms
        EdgeD E = ed[sc.z];
        double w = wi + qj.x;
        double cl = w * E.th + (ep.btype == 0 ? ep.kt * E.db : 0.0);
        const double sj = -cl * abs_bits(E.il);
        ssum += sj;
        acc.x = fma(sj, xj.x, acc.x);
        acc.y = fma(sj, xj.y, acc.y);
        acc.z = fma(sj, xj.z, acc.z);
        double cn = carry;
        if (interior_edge(E.il)) {
          int cin = slot_corner(sn.y);
          cn += w * cj;
          carry_next = w * cot_at(Fn, cin == 0 ? 2 : cin - 1);
        }
        // edge (j, k) opposite i: dihedral term
        if (interior_edge(ed[sc.w].il)) cn -= ((hgC + qj.x) + qk.x) * (cj + ck);
        acc += cn * n;
      }
      carry = carry_next;
      xk = xj;
      qk = qj;
      sc = sn;
      fcur = fnx;
      Fc = Fn;
      xj = ld3(P, sn.x);
      qj = rk[sn.x];
    }
    acc += carry * n0;  // the last edge's part on the first face
    acc.x = fma(-ssum, xi.x, acc.x);
    acc.y = fma(-ssum, xi.y, acc.y);
    acc.z = fma(-ssum, xi.z, acc.z);
  }
  st3(grad, i, acc);
}

inline int nblk(long n, int b) { return (int)((n + b - 1) / b); }
// the FP64 path's per-vertex curvature weights (kb rho, 2/3 kb rho^2)
inline double2* rk2(tm_energy* e) { return reinterpret_cast<double2*>(e->rho.get()); }
// the FP64 path's compact (area, volume) per face and (l theta, bond) per edge
inline double2* fav2(tm_energy* e) { return reinterpret_cast<double2*>(e->fav.get()); }
inline double2* elt2(tm_energy* e) { return reinterpret_cast<double2*>(e->ebond.get()); }

EP make_ep(const tm_energy* e) {
  const tm_params& p = e->prm;
  EP ep;
  std::memset(&ep, 0, sizeof ep);  // padding too: evaluation graphs compare EP bytes
  ep.kb = p.kappa_b;
  ep.ka = p.kappa_a;
  ep.kv = p.kappa_v;
  ep.kc = p.kappa_c;
  ep.kt = p.kappa_t;
  ep.kr = p.kappa_r;
  double lam = p.cont_lambda;
  ep.refA = (1.0 - lam * (1.0 - p.area_frac)) * e->initial[0];
  ep.refV = (1.0 - lam * (1.0 - p.volume_frac)) * e->initial[1];
  ep.refC = (1.0 - lam * (1.0 - p.curvature_frac)) * e->initial[2];
  ep.lc0 = p.bond_lc0;
  ep.lc1 = p.bond_lc1;
  ep.a0 = p.bond_a0;
  ep.r = p.bond_r;
  ep.btype = p.bond_type;
  ep.rlc1 = p.rep_lc1;
  ep.rT = sq_threshold(p.rep_lc1);
  ep.rr = p.rep_r;
  ep.tdiv = p.bond_type == 0 ? 2.0 : 3.0;
  ep.itdiv = 1.0 / ep.tdiv;
  auto ipow_h = [](double x, int n) {  // the device's ipow, on the host
    double r = 1.0;
    for (int k = 0; k < std::abs(n); ++k) r *= x;
    return n < 0 ? 1.0 / r : r;
  };
  ep.br1 = ipow_h((double)p.bond_r, p.bond_r + 1);
  ep.br2 = ipow_h((double)p.bond_r, p.bond_r + 2);
  return ep;
}

void energy_eval(tm_energy* e, tm_mesh* m, const double* P, bool want_grad, bool want_vprops, double* d_grad,
                 cudaStream_t s) {
  energy_eval_marked(e, m, P, want_grad, want_vprops, d_grad, s, nullptr);
}

static void eval_fp64_launches(tm_energy* e, tm_mesh* m, const double* P, bool want_grad, bool want_vprops,
                               double* d_grad, cudaStream_t s, cudaEvent_t* ev);

// the launches of one evaluation in the energy's stencil precision
static void eval_launches(tm_energy* e, tm_mesh* m, const double* P, bool want_grad, double* d_grad,
                          cudaStream_t s) {
  if (e->stencil == 1)
    energy_eval32(e, m, P, want_grad, false, d_grad, s, nullptr);
  else if (e->stencil == 2)
    energy_eval_df(e, m, P, want_grad, d_grad, s, nullptr);
  else
    eval_fp64_launches(e, m, P, want_grad, false, d_grad, s, nullptr);
}

// What the launches of an evaluation depend on besides device memory:
// arguments, stencil precision, buffers, parameters and the neighbour-list
// view.  Equal keys mean a captured graph replays the same launches.
static std::vector<unsigned char> eval_key(tm_energy* e, tm_mesh* m, const double* P, bool want_grad,
                                           double* d_grad) {
  std::vector<unsigned char> k;
  auto add = [&k](const void* p, size_t n) {
    const unsigned char* b = static_cast<const unsigned char*>(p);
    k.insert(k.end(), b, b + n);
  };
  // (the launch stream is not part of the key: a graph replays on any stream)
  const void* ptrs[] = {P, d_grad, e->face.get(), e->edge.get(), e->ebond.get(), e->fav.get(), e->rho.get(),
                        e->repg.get(), e->reppot.get(), e->slow.get(), e->pos32.get(), e->poslo.get(), e->partials.get(),
                        e->glob.get(), e->sct.get(), e->aux, e->ev_fork, e->ev_join, e->nl.xb.get(),
                        e->posdw.get(), e->sctf.get()};
  add(ptrs, sizeof ptrs);
  const Topo t = m->topo();
  const int sizes[] = {t.nv, t.ne, t.nf, want_grad ? 1 : 0, e->stencil, e->nl.near_nv};
  add(sizes, sizeof sizes);
  const void* tp[] = {t.to, t.next, t.face, t.vout, t.fhe, t.slot, t.nbr, t.val, t.fv, t.edge};
  add(tp, sizeof tp);
  const double nd[] = {e->nl.near_lc1, e->nl.near_move2};
  add(nd, sizeof nd);
  const EP ep = make_ep(e);
  add(&ep, sizeof ep);
  add(&e->nl.view, sizeof(NLView));
  return k;
}

// Evaluation replayed from a CUDA graph: the launch sequence (about a dozen
// kernels, memsets and the fork/join of the repulsion stream) is captured
// per key and then issued as one graph launch, which removes the gaps
// between the short kernels.  On a miss the launches run directly first
// (any allocation they make happens outside a capture), then they are
// captured for the next call.  A few graphs are kept (with and without the
// gradient, several buffers), the least recently used is replaced.
static void eval_graph(tm_energy* e, tm_mesh* m, const double* P, bool want_grad, double* d_grad, cudaStream_t s) {
  constexpr size_t MAX_GRAPHS = 4;
  std::vector<unsigned char> key = eval_key(e, m, P, want_grad, d_grad);
  for (auto& g : e->eval_graphs)
    if (g.exec && g.key == key) {
      g.used = ++e->eval_tick;
      TM_CUDA(cudaGraphLaunch(g.exec, s));
      return;
    }
  eval_launches(e, m, P, want_grad, d_grad, s);
  key = eval_key(e, m, P, want_grad, d_grad);
  cudaGraph_t g = nullptr;
  TM_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
  try {
    eval_launches(e, m, P, want_grad, d_grad, s);
  } catch (...) {
    cudaStreamEndCapture(s, &g);  // leave capture mode before reporting
    if (g) cudaGraphDestroy(g);
    cudaGetLastError();
    throw;
  }
  TM_CUDA(cudaStreamEndCapture(s, &g));
  cudaGraphExec_t exec = nullptr;
  cudaError_t rc = cudaGraphInstantiate(&exec, g, 0);
  cudaGraphDestroy(g);
  TM_CUDA(rc);
  tm_energy::EvalGraph* slot = nullptr;
  if (e->eval_graphs.size() < MAX_GRAPHS) {
    e->eval_graphs.emplace_back();
    slot = &e->eval_graphs.back();
  } else {
    slot = &e->eval_graphs[0];
    for (auto& c : e->eval_graphs)
      if (c.used < slot->used) slot = &c;
    cudaGraphExecDestroy(slot->exec);
  }
  slot->exec = exec;
  slot->key.swap(key);
  slot->used = ++e->eval_tick;
}

void energy_eval_marked(tm_energy* e, tm_mesh* m, const double* P, bool want_grad, bool want_vprops, double* d_grad,
                        cudaStream_t s, cudaEvent_t* ev) {
  // graphs need a capturable stream (not the legacy default stream)
  if (!ev && !want_vprops && s != nullptr && e->use_graphs) {
    eval_graph(e, m, P, want_grad, d_grad, s);
    return;
  }
  if (e->stencil == 1 && !want_vprops) {
    energy_eval32(e, m, P, want_grad, want_vprops, d_grad, s, ev);
    return;
  }
  if (e->stencil == 2 && !want_vprops) {
    energy_eval_df(e, m, P, want_grad, d_grad, s, ev);
    return;
  }
  eval_fp64_launches(e, m, P, want_grad, want_vprops, d_grad, s, ev);
}

static void eval_fp64_launches(tm_energy* e, tm_mesh* m, const double* P, bool want_grad, bool want_vprops,
                               double* d_grad, cudaStream_t s, cudaEvent_t* ev) {
  if (ev) TM_CUDA(cudaEventRecord(ev[0], s));
  e->ensure(m->nv, m->ne, m->nf);
  Topo t = m->topo();
  EP ep = make_ep(e);
  FaceD* fd = reinterpret_cast<FaceD*>(e->face.get());
  EdgeD* ed = reinterpret_cast<EdgeD*>(e->edge.get());
  NLView nlv = e->nl.view;
  nlv.pos32 = e->pos32.get();
  int nfb = std::max(nblk(std::max(t.nf, t.nv), 256), 1);
  k_face<<<nfb, 256, 0, s>>>(t, P, fd, e->pos32.get(), fav2(e));
  TM_LAUNCH();
  if (ev) TM_CUDA(cudaEventRecord(ev[1], s));
  // the repulsion pass needs only the positions: it overlaps the edge kernels
  // (in sequence when the stages are timed)
  const bool conc = ev == nullptr;
  if (conc) fork_repulsion(e, m, P, want_grad, s, true);
  int* blist = e->slow.get() + std::max(m->nv, 1) + 1;
  int* bcnt = blist + std::max(m->ne, 1);
  TM_CUDA(cudaMemsetAsync(bcnt, 0, sizeof(int), s));
  if (t.ne) k_edge<<<nblk(t.ne, 256), 256, 0, s>>>(t, P, fd, ed, elt2(e), ep, blist, bcnt, e->sct.get());
  TM_LAUNCH();
  if (t.ne) k_bond_short<<<std::min(nblk(t.ne, 256), 4 * 152), 256, 0, s>>>(P, t, ed, elt2(e), ep, blist, bcnt);
  TM_LAUNCH();
  if (ev) TM_CUDA(cudaEventRecord(ev[2], s));
  if (conc)
    join_repulsion(e, s, true);
  else
    fork_repulsion(e, m, P, want_grad, s, false);
  int nb = std::max(1, nblk(t.nv, VB));
  if (want_vprops)
    k_vertex<true><<<nb, VB, 0, s>>>(t, fav2(e), elt2(e), e->reppot.get(), ep, rk2(e),
                                     e->vprops.get(), e->partials.get(), e->glob.get());
  else
    k_vertex<false><<<nb, VB, 0, s>>>(t, fav2(e), elt2(e), e->reppot.get(), ep, rk2(e), nullptr,
                                      e->partials.get(), e->glob.get());
  TM_LAUNCH();
  if (ev) TM_CUDA(cudaEventRecord(ev[3], s));
  if (want_grad && t.nv)
    k_grad<<<nblk(t.nv, 256), 256, 0, s>>>(t, P, fd, ed, rk2(e), e->repg.get(), e->glob.get(), ep, d_grad);
  TM_LAUNCH();
  if (ev) TM_CUDA(cudaEventRecord(ev[4], s));
}

void energy_from_props_device(tm_energy* e, const double* d_props6, double* /*unused*/, cudaStream_t s) {
  EP ep = make_ep(e);
  k_assemble_props<<<1, 1, 0, s>>>(ep, d_props6, e->glob.get());
  TM_LAUNCH();
}

}  // namespace tmg

void tm_energy::ensure(int nv_, int ne_, int nf_) {
  if (nv_ == nv && ne_ == ne && nf_ == nf && glob.get()) return;
  nv = nv_;
  ne = ne_;
  nf = nf_;
  face.ensure(8 * (size_t)std::max(nf, 1));
  edge.ensure(4 * (size_t)std::max(ne, 1));
  ebond.ensure(2 * (size_t)std::max(ne, 1));  // FP64 path: (l theta, bond value) per edge
  fav.ensure(2 * (size_t)std::max(nf, 1));    // FP64 path: (area, volume) per face
  rho.ensure(2 * (size_t)std::max(nv, 1));  // FP64 path: (kb rho, 2/3 kb rho^2) per vertex
  repg.ensure(3 * (size_t)std::max(nv, 1));
  reppot.ensure(std::max(nv, 1));
  // repulsion slow list (nv + 1) and short-bond edge list (ne + 1)
  slow.ensure((size_t)std::max(nv, 1) + 1 + (size_t)std::max(ne, 1) + 1);
  vprops.ensure(6 * (size_t)std::max(nv, 1));
  pos32.ensure(3 * (size_t)std::max(nv, 1));
  int nb = std::max(1, (nv + tmg::VB - 1) / tmg::VB);
  partials.ensure(8 * (size_t)nb);
  grad.ensure(3 * (size_t)std::max(nv, 1));
  work.ensure(64);
  glob.ensure(1);
  TM_CUDA(cudaMemsetAsync(glob.get(), 0, sizeof(tmg::Globals), stream));
}

void tm_energy::to_host(double* dst, const double* src, size_t n) {
  // direct copy: for pageable destinations the driver's own staged copy beat
  // a page-locked staging buffer plus memcpy (the destination is a fresh
  // array whose pages are touched for the first time either way)
  if (n) TM_CUDA(cudaMemcpyAsync(dst, src, sizeof(double) * n, cudaMemcpyDeviceToHost, stream));
  TM_CUDA(cudaStreamSynchronize(stream));
}

tm_energy::~tm_energy() {
  for (auto& g : eval_graphs)
    if (g.exec) cudaGraphExecDestroy(g.exec);
  if (flip_graph.exec) cudaGraphExecDestroy(flip_graph.exec);
  if (ev_fork) cudaEventDestroy(ev_fork);
  if (ev_join) cudaEventDestroy(ev_join);
  if (aux) cudaStreamDestroy(aux);
  if (stream) cudaStreamDestroy(stream);
}

// --------------------------------------------------------------------------
// C ABI
// --------------------------------------------------------------------------
static void check_params(const tm_params& p) {
  if (p.bond_type != 0 && p.bond_type != 1) fail(TM_ERR_ARG, "Unknown bond potential");
  if (p.n_search != 0 && p.n_search != 1) fail(TM_ERR_ARG, "Unknown neighbour search algorithm.");
  if (p.exclusion_level < 0 || p.exclusion_level > 2) fail(TM_ERR_ARG, "Unsupported exclusion level");
}

static void fetch_globals(tm_energy* e, tmg::Globals* g) {
  TM_CUDA(cudaMemcpyAsync(g, e->glob.get(), sizeof(tmg::Globals), cudaMemcpyDeviceToHost, e->stream));
  TM_CUDA(cudaStreamSynchronize(e->stream));
}

static void eval_host(tm_energy* e, tm_mesh* m, bool grad, bool vprops) {
  if (!e || !m) fail(TM_ERR_ARG, "NULL handle");
  m->upload_points(e->stream);
  tmg::energy_eval(e, m, m->d_pts.get(), grad, vprops, e->grad.get(), e->stream);
}

extern "C" {

int tm_energy_create(tm_mesh* m, const tm_params* p, tm_energy** out) {
  TM_API_BEGIN
  if (!m || !p || !out) fail(TM_ERR_ARG, "NULL argument");
  *out = nullptr;
  check_params(*p);
  std::unique_ptr<tm_energy> e(new tm_energy());
  e->prm = *p;
  TM_CUDA(cudaStreamCreateWithFlags(&e->stream, cudaStreamNonBlocking));
  TM_CUDA(cudaStreamCreateWithFlags(&e->aux, cudaStreamNonBlocking));
  TM_CUDA(cudaEventCreateWithFlags(&e->ev_fork, cudaEventDisableTiming));
  TM_CUDA(cudaEventCreateWithFlags(&e->ev_join, cudaEventDisableTiming));
  {
    std::vector<double2> sc(tmg::TM_SCT_N);
    std::vector<float4> scf(tmg::TM_SCT_N);
    auto split = [](double x, float* h, float* l) {
      *h = (float)x;
      *l = (float)(x - (double)*h);
    };
    for (int k = 0; k < tmg::TM_SCT_N; ++k) {
      sc[k] = make_double2(std::sin(k / 128.0), std::cos(k / 128.0));
      split(sc[k].x, &scf[k].x, &scf[k].y);
      split(sc[k].y, &scf[k].z, &scf[k].w);
    }
    e->sct.ensure(tmg::TM_SCT_N);
    e->sctf.ensure(tmg::TM_SCT_N);
    TM_CUDA(cudaMemcpyAsync(e->sct.get(), sc.data(), sizeof(double2) * tmg::TM_SCT_N, cudaMemcpyHostToDevice,
                            e->stream));
    TM_CUDA(cudaMemcpyAsync(e->sctf.get(), scf.data(), sizeof(float4) * tmg::TM_SCT_N, cudaMemcpyHostToDevice,
                            e->stream));
    TM_CUDA(cudaStreamSynchronize(e->stream));
  }
  m->upload_points(e->stream);
  tmg::nlist_make(&e->nl, m, e->prm, m->d_pts.get(), e->stream);
  // initial properties: the reference properties are still unset (zero) and
  // only the sums matter here; taken with the FP64 stencil whatever the
  // handle's stencil precision
  const int stencil = e->stencil;
  e->stencil = 0;
  tmg::energy_eval(e.get(), m, m->d_pts.get(), false, false, nullptr, e->stream);
  e->stencil = stencil;
  tmg::Globals g;
  fetch_globals(e.get(), &g);
  for (int k = 0; k < 6; ++k) e->initial[k] = g.props[k];
  *out = e.release();
  TM_API_END
}

int tm_energy_destroy(tm_energy* e) {
  delete e;
  return TM_OK;
}

int tm_energy_get_params(tm_energy* e, tm_params* out) {
  if (!e || !out) return TM_ERR_ARG;
  *out = e->prm;
  return TM_OK;
}

int tm_energy_initial_props(tm_energy* e, double* out6) {
  if (!e || !out6) return TM_ERR_ARG;
  std::memcpy(out6, e->initial, sizeof(double) * 6);
  return TM_OK;
}

int tm_energy_set_initial_props(tm_energy* e, const double* in6) {
  TM_API_BEGIN
  if (!e || !in6) fail(TM_ERR_ARG, "NULL argument");
  std::memcpy(e->initial, in6, sizeof(double) * 6);
  TM_API_END
}

int tm_energy_properties(tm_energy* e, tm_mesh* m, double* out6) {
  TM_API_BEGIN
  if (!out6) fail(TM_ERR_ARG, "NULL output");
  eval_host(e, m, false, false);
  tmg::Globals g;
  fetch_globals(e, &g);
  std::memcpy(out6, g.props, sizeof(double) * 6);
  TM_API_END
}

int tm_energy_vertex_properties(tm_energy* e, tm_mesh* m, double* out6v) {
  TM_API_BEGIN
  if (!out6v) fail(TM_ERR_ARG, "NULL output");
  eval_host(e, m, false, true);
  TM_CUDA(cudaMemcpyAsync(out6v, e->vprops.get(), sizeof(double) * 6 * m->nv, cudaMemcpyDeviceToHost, e->stream));
  TM_CUDA(cudaStreamSynchronize(e->stream));
  TM_API_END
}

int tm_energy_energy(tm_energy* e, tm_mesh* m, double* energy) {
  TM_API_BEGIN
  if (!energy) fail(TM_ERR_ARG, "NULL output");
  eval_host(e, m, false, false);
  tmg::Globals g;
  fetch_globals(e, &g);
  *energy = g.comps[6];
  TM_API_END
}

int tm_energy_energy_props(tm_energy* e, const double* props6, double* energy) {
  TM_API_BEGIN
  if (!e || !props6 || !energy) fail(TM_ERR_ARG, "NULL argument");
  e->ensure(std::max(e->nv, 1), std::max(e->ne, 1), std::max(e->nf, 1));
  TM_CUDA(cudaMemcpyAsync(e->work.get(), props6, sizeof(double) * 6, cudaMemcpyHostToDevice, e->stream));
  tmg::energy_from_props_device(e, e->work.get(), nullptr, e->stream);
  tmg::Globals g;
  fetch_globals(e, &g);
  *energy = g.comps[6];
  TM_API_END
}

int tm_energy_components(tm_energy* e, tm_mesh* m, double* out7) {
  TM_API_BEGIN
  if (!out7) fail(TM_ERR_ARG, "NULL output");
  eval_host(e, m, false, false);
  tmg::Globals g;
  fetch_globals(e, &g);
  std::memcpy(out7, g.comps, sizeof(double) * 7);
  TM_API_END
}

int tm_energy_gradient(tm_energy* e, tm_mesh* m, double* grad, double* energy) {
  TM_API_BEGIN
  if (!grad) fail(TM_ERR_ARG, "NULL output");
  eval_host(e, m, true, false);
  if (energy)
    TM_CUDA(cudaMemcpyAsync(energy, &e->glob.get()->comps[6], sizeof(double), cudaMemcpyDeviceToHost, e->stream));
  e->to_host(grad, e->grad.get(), 3 * (size_t)m->nv);
  TM_API_END
}

int tm_energy_update_reference_properties(tm_energy* e) {
  if (!e) return TM_ERR_ARG;
  if (e->prm.cont_lambda < 1.0) e->prm.cont_lambda += e->prm.cont_delta;
  return TM_OK;
}

int tm_energy_update_repulsion(tm_energy* e, tm_mesh* m) {
  TM_API_BEGIN
  if (!e || !m) fail(TM_ERR_ARG, "NULL handle");
  m->upload_points(e->stream);
  tmg::nlist_make(&e->nl, m, e->prm, m->d_pts.get(), e->stream);
  TM_CUDA(cudaStreamSynchronize(e->stream));
  TM_API_END
}

int tm_energy_set_stencil_precision(tm_energy* e, int mode) {
  TM_API_BEGIN
  if (!e) fail(TM_ERR_ARG, "NULL handle");
  if (mode < 0 || mode > 2) fail(TM_ERR_ARG, "mode must be 0 (FP64), 1 (FP32) or 2 (double-float)");
  e->stencil = mode;
  TM_API_END
}

int tm_energy_eval_device(tm_energy* e, tm_mesh* m, const double* d_points, double* d_grad, double* d_energy,
                          void* stream) {
  TM_API_BEGIN
  if (!e || !m || !d_points) fail(TM_ERR_ARG, "NULL argument");
  cudaStream_t s = stream ? (cudaStream_t)stream : e->stream;
  tmg::energy_eval(e, m, d_points, d_grad != nullptr, false, d_grad, s);
  if (d_energy)
    TM_CUDA(cudaMemcpyAsync(d_energy, &e->glob.get()->comps[6], sizeof(double), cudaMemcpyDeviceToDevice, s));
  TM_API_END
}

int tm_energy_eval_timed(tm_energy* e, tm_mesh* m, const double* d_points, double* d_grad, float* ms5,
                         void* stream) {
  TM_API_BEGIN
  if (!e || !m || !d_points || !ms5) fail(TM_ERR_ARG, "NULL argument");
  cudaStream_t s = stream ? (cudaStream_t)stream : e->stream;
  cudaEvent_t ev[5];
  for (int k = 0; k < 5; ++k) TM_CUDA(cudaEventCreate(&ev[k]));
  tmg::energy_eval_marked(e, m, d_points, d_grad != nullptr, false, d_grad, s, ev);
  TM_CUDA(cudaEventSynchronize(ev[4]));
  for (int k = 0; k < 4; ++k) TM_CUDA(cudaEventElapsedTime(&ms5[k], ev[k], ev[k + 1]));
  TM_CUDA(cudaEventElapsedTime(&ms5[4], ev[0], ev[4]));
  for (int k = 0; k < 5; ++k) cudaEventDestroy(ev[k]);
  TM_API_END
}

int tm_energy_update_repulsion_device(tm_energy* e, tm_mesh* m, const double* d_points, void* stream) {
  TM_API_BEGIN
  if (!e || !m || !d_points) fail(TM_ERR_ARG, "NULL argument");
  cudaStream_t s = stream ? (cudaStream_t)stream : e->stream;
  tmg::nlist_make(&e->nl, m, e->prm, d_points, s);
  TM_API_END
}

int tm_fd_gradient(tm_mesh* m, tm_energy* e, double eps, double* grad) {
  TM_API_BEGIN
  if (!m || !e || !grad) fail(TM_ERR_ARG, "NULL argument");
  double e0 = 0;
  int rc = tm_energy_energy(e, m, &e0);
  if (rc) return rc;
  for (int i = 0; i < m->nv; ++i)
    for (int k = 0; k < 3; ++k) {
      double* x = m->h_pts + 3 * (size_t)i + k;
      *x += eps;
      double en = 0;
      rc = tm_energy_energy(e, m, &en);
      *x -= eps;
      if (rc) return rc;
      grad[3 * (size_t)i + k] = (en - e0) / eps;
    }
  TM_API_END
}

}  // extern "C"

// --------------------------------------------------------------------------
// Evaluation without allocation.
//
// Some callers cannot call cudaMalloc while they evaluate the energy: a host
// that runs under a strict device-memory budget owned by someone else (an
// embedding application or a pool allocator that forbids side allocations),
// or code that must not enter the CUDA allocator while other streams of the
// process are busy.  tm_energy_eval_device_noalloc evaluates the FP64 energy
// and gradient of a mesh whose scratch (face and edge records, per-vertex
// intermediates, block partials and the reduction state) fits into one
// file-scope device array of TM_NOALLOC_SCRATCH_BYTES, instead of the energy
// manager's own buffers.  It allocates nothing and frees nothing.
//
// The array's host-side name is only a stand-in for the device symbol, so its
// device address is looked up with cudaGetSymbolAddress once per device, on
// the first call made with that device current; make that first call before
// any stream capture.  All calls share the array and it keeps the last call's
// contents: each call clears the reduction state it needs at zero, and calls
// whose executions overlap on the GPU (other streams, other threads) race on
// the shared scratch and must be serialised by the caller.
// --------------------------------------------------------------------------
#include <mutex>

namespace {
static __device__ __align__(256) unsigned char g_noalloc_scratch[TM_NOALLOC_SCRATCH_BYTES];

constexpr int kMaxDevices = 64;
std::mutex g_noalloc_mutex;
unsigned char* g_noalloc_ptr[kMaxDevices] = {nullptr};

unsigned char* noalloc_scratch_for_current_device() {
  int dev = 0;
  TM_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) fail(TM_ERR_ARG, "device index out of range for the no-alloc scratch");
  std::lock_guard<std::mutex> lock(g_noalloc_mutex);
  if (!g_noalloc_ptr[dev]) {
    void* p = nullptr;
    TM_CUDA(cudaGetSymbolAddress(&p, g_noalloc_scratch));
    g_noalloc_ptr[dev] = static_cast<unsigned char*>(p);
  }
  return g_noalloc_ptr[dev];
}

inline size_t align256(size_t x) { return (x + 255) & ~size_t(255); }
}  // namespace

extern "C" int tm_energy_eval_device_noalloc(tm_energy* e, tm_mesh* m, const double* d_points, double* d_grad,
                                             double* d_energy, void* stream) {
  TM_API_BEGIN
  if (!e || !m || !d_points || !d_grad) fail(TM_ERR_ARG, "NULL argument");
  const size_t nv = std::max(m->nv, 1), ne = std::max(m->ne, 1), nf = std::max(m->nf, 1);
  const int nb = std::max(1, (m->nv + VB - 1) / VB);
  // scratch layout, 256-byte aligned pieces
  size_t off_face = 0;
  size_t off_edge = off_face + align256(sizeof(FaceD) * nf);
  size_t off_ebond = off_edge + align256(sizeof(EdgeD) * ne);
  size_t off_fav = off_ebond + align256(sizeof(double2) * ne);
  size_t off_rho = off_fav + align256(sizeof(double2) * nf);
  size_t off_repg = off_rho + align256(sizeof(double2) * nv);
  size_t off_pos32 = off_repg + align256(3 * sizeof(double) * nv);
  size_t off_pot = off_pos32 + align256(3 * sizeof(float) * nv);
  size_t off_slow = off_pot + align256(sizeof(double) * nv);
  size_t off_blist = off_slow + align256(sizeof(int) * (nv + 1));
  size_t off_part = off_blist + align256(sizeof(int) * (ne + 1));
  size_t off_glob = off_part + align256(8 * sizeof(double) * nb);
  size_t need = off_glob + align256(sizeof(Globals));
  if (need > (size_t)TM_NOALLOC_SCRATCH_BYTES)
    fail(TM_ERR_ARG, "mesh needs " + std::to_string(need) + " bytes of scratch, more than the " +
                         std::to_string((size_t)TM_NOALLOC_SCRATCH_BYTES) +
                         " bytes of tm_energy_eval_device_noalloc (about 44,000 vertices)");
  unsigned char* base = noalloc_scratch_for_current_device();
  cudaStream_t s = stream ? (cudaStream_t)stream : e->stream;
  FaceD* fd = reinterpret_cast<FaceD*>(base + off_face);
  EdgeD* ed = reinterpret_cast<EdgeD*>(base + off_edge);
  double2* ebond = reinterpret_cast<double2*>(base + off_ebond);
  double2* fav = reinterpret_cast<double2*>(base + off_fav);
  double2* rho = reinterpret_cast<double2*>(base + off_rho);
  double* repg = reinterpret_cast<double*>(base + off_repg);
  float* pos32 = reinterpret_cast<float*>(base + off_pos32);
  double* reppot = reinterpret_cast<double*>(base + off_pot);
  int* slow = reinterpret_cast<int*>(base + off_slow);
  int* blist = reinterpret_cast<int*>(base + off_blist);
  int* bcnt = blist + ne;
  double* part = reinterpret_cast<double*>(base + off_part);
  Globals* g = reinterpret_cast<Globals*>(base + off_glob);
  // the block ticket of the reduction must start at zero
  TM_CUDA(cudaMemsetAsync(g, 0, sizeof(Globals), s));
  Topo t = m->topo();
  EP ep = make_ep(e);
  NLView nlv = e->nl.view;
  nlv.pos32 = pos32;
  int nfb = std::max(nblk(std::max(t.nf, t.nv), 256), 1);
  k_face<<<nfb, 256, 0, s>>>(t, d_points, fd, pos32, fav);
  TM_LAUNCH();
  TM_CUDA(cudaMemsetAsync(bcnt, 0, sizeof(int), s));
  if (t.ne) k_edge<<<nblk(t.ne, 256), 256, 0, s>>>(t, d_points, fd, ed, ebond, ep, blist, bcnt, e->sct.get());
  TM_LAUNCH();
  if (t.ne) k_bond_short<<<std::min(nblk(t.ne, 256), 4 * 152), 256, 0, s>>>(d_points, t, ed, ebond, ep, blist, bcnt);
  TM_LAUNCH();
  repulsion_eval(e, m, d_points, pos32, true, reppot, repg, slow, slow + nv, s);
  k_vertex<false><<<nb, VB, 0, s>>>(t, fav, ebond, reppot, ep, rho, nullptr, part, g);
  TM_LAUNCH();
  if (t.nv) k_grad<<<nblk(t.nv, 256), 256, 0, s>>>(t, d_points, fd, ed, rho, repg, g, ep, d_grad);
  TM_LAUNCH();
  if (d_energy) TM_CUDA(cudaMemcpyAsync(d_energy, &g->comps[6], sizeof(double), cudaMemcpyDeviceToDevice, s));
  TM_API_END
}
