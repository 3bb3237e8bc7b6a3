// Device helpers shared by the energy, flip and HMC kernels: parameters,
// penalty assembly, the repulsion neighbour walk and the exclusion test.
#pragma once

#include "tm_internal.h"
#include "tm_math.cuh"

namespace tmg {

struct EP {
  double kb, ka, kv, kc, kt, kr;
  double refA, refV, refC;
  double lc0, lc1, a0;
  int r, btype;  // btype 0 edge bonds, 1 area bonds
  double rlc1, rT;  // repulsion cut-off and its exact squared threshold
  int rr;
  double tdiv;
  double itdiv;  // 1 / tdiv, correctly rounded (what a device division gives)
  double br1, br2;  // r^(r+1) and r^(r+2) of the flat-bottom bond above lc0
};

struct __align__(16) FaceD {
  double nx, ny, nz, A, V, c0, c1, c2;
};
// il: 1/l on interior edges, -1/l on boundary edges (the sign is the
// interior flag; the gradient multiplies by |il| instead of dividing by l)
struct __align__(16) EdgeD {
  double l, th, db, il;
};

constexpr int VB = 256;  // threads per block of k_vertex (fixed: it sets the reduction order)

__device__ __forceinline__ double cot_at(const FaceD& F, int c) { return c == 0 ? F.c0 : (c == 1 ? F.c1 : F.c2); }

// Unsigned angle theta in [0, pi] from s = sin(theta) >= 0 and
// c = cos(theta) of two unit vectors: a float atan2 estimate rounded to the
// grid t0 = k/128, whose sine and cosine sct holds (sct[k] = {sin, cos}),
// then theta = t0 + asin(x) with x = s cos t0 - c sin t0 = sin(theta - t0).
// |x| <= 1/256 plus the float error, so asin(x) = x + x^3/6 + 3 x^5/40 is
// exact to below 1e-18; s^2 + c^2 = 1 within rounding enters x only at
// that order.  Unlike acos(c) it keeps full relative accuracy for small
// angles.  NaN inputs give NaN (the grid index is clamped).
__device__ __forceinline__ double angle_sc(double s, double c, const double2* __restrict__ sct) {
  float tf = atan2f((float)s, (float)c);
  int k = __float2int_rn(tf * 128.0f);
  k = min(max(k, 0), TM_SCT_N - 1);
  double2 g = __ldg(sct + k);
  double x = s * g.y - c * g.x;
  double x2 = x * x;
  double p = x2 * fma(x2, 3.0 / 40.0, 1.0 / 6.0);
  return fma(x, p, x) + k * (1.0 / 128.0);
}

// ---- repulsion (src/mesh_repulsion.h:28-79 over the neighbour list) -------
__device__ __forceinline__ unsigned long long cell_hash(long long key) {
  unsigned long long z = (unsigned long long)key + 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
__device__ __forceinline__ int cell_find(const NLView& nl, long long key, int* start) {
  unsigned long long h = cell_hash(key) & nl.tmask;
  for (unsigned long long p = 0; p <= nl.tmask; ++p) {
    CellEntry c = nl.table[h];
    if (c.key == key) {
      *start = c.start;
      return c.count;
    }
    if (c.key == -1) return 0;
    h = (h + 1) & nl.tmask;
  }
  return 0;
}

// j within the 1-ring (level 1) or 2-ring (level 2) of v
__device__ __forceinline__ bool excluded(const Topo& t, int excl, int v, int j) {
  if (excl <= 0) return false;
  int d = t.val[v];
  for (int m = 0; m < d; ++m) {
    int w = t.nbr[(size_t)m * t.nv + v];
    if (w == j) return true;
    if (excl > 1) {
      int dw = t.val[w];
      for (int q = 0; q < dw; ++q)
        if (t.nbr[(size_t)q * t.nv + w] == j) return true;
    }
  }
  return false;
}

struct TableExcl {  // exclusion on the current topology tables
  const Topo& t;
  int excl;
  const NLView* nl = nullptr;  // per-replica levels of a batch, when given
  __device__ bool operator()(int v, int j) const { return excluded(t, nl ? excl_of(*nl, v) : excl, v, j); }
};

// Cell coordinate int((p - bmin) / rl) with C truncation
// (src/nlists/cell_list.h:141), decided without the FP64 division unless
// the quotient is within 1e-9 of an integer, where the exact quotient is used.
__device__ __forceinline__ int cell_coord(double p, const NLGeom& G, int k) {
  double q = __dsub_rn(p, G.bmin[k]);
  double t = __dmul_rn(q, G.inv_rl[k]);
  double ti = trunc(t);
  double fr = fabs(t - ti);
  if (fr > 1e-9 && fr < 1.0 - 1e-9 && fabs(t) < 1.0e9) return (int)ti;
  return (int)__ddiv_rn(q, G.rl[k]);
}

// Distance test of candidate j against the query point p of vertex v:
// an FP32 prefilter (skips only candidates that are certainly outside,
// margin from the float rounding of both points) and the exact test
// sqrt(s) < dmax  <=>  s < T with s rounded operation by operation.
struct PairTest {
  double T;     // exact squared threshold of dmax
  float bound;  // prefilter bound on the float squared distance
  float3 p32;
  bool pre;
};
__device__ __forceinline__ PairTest make_pair_test(const NLView& nl, int v, double dmax, double T) {
  PairTest t;
  t.T = T;
  t.pre = nl.pos32 != nullptr;
  if (t.pre) {
    t.p32 = make_float3(nl.pos32[3 * v], nl.pos32[3 * v + 1], nl.pos32[3 * v + 2]);
    float pinf = fmaxf(fabsf(t.p32.x), fmaxf(fabsf(t.p32.y), fabsf(t.p32.z)));
    float dm = (float)dmax;
    float eps = 1.7320508f * (2.0f * pinf + 2.0f * dm) * 1.1920929e-07f;  // 2 ulp(1) per unit
    float r = dm + eps;
    t.bound = r * r * (1.0f + 9.5367431e-07f);
  }
  return t;
}
// returns true (and s, the exact squared distance) when |p - x_j| < dmax
__device__ __forceinline__ bool pair_within(const PairTest& t, const NLView& nl, const double* P, d3 p, int j,
                                            d3* pj_out, double* s_out) {
  if (t.pre) {
    float dx = nl.pos32[3 * j] - t.p32.x, dy = nl.pos32[3 * j + 1] - t.p32.y, dz = nl.pos32[3 * j + 2] - t.p32.z;
    float s32 = dx * dx + dy * dy + dz * dz;
    if (s32 > t.bound) return false;
  }
  d3 pj = ld3(P, j);
  double dx = __dsub_rn(p.x, pj.x), dy = __dsub_rn(p.y, pj.y), dz = __dsub_rn(p.z, pj.z);
  double s = __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
  *pj_out = pj;
  *s_out = s;
  return s < t.T;
}

// The three ways to enumerate the neighbours of vertex v (at p): the
// candidate row of its build cell, the 27-cell scan through the cell table,
// and the Verlet row.  Each calls fn(j, |p - x_j|, p - x_j) for the
// neighbours closer than the cut-off, in the reference's order (cells x
// outer / z inner, members ascending).
template <class F, class X>
__device__ __forceinline__ void visit_pair(const PairTest& pt, const NLView& nl, const double* P, int v, d3 p, int j,
                                           const X& is_excluded, F& fn) {
  d3 pj;
  double s;
  if (!pair_within(pt, nl, P, p, j, &pj, &s)) return;
  if (nl.excl > 0 && is_excluded(v, j)) return;
  fn(j, __dsqrt_rn(s), exact_diff(p, pj));
}
// Cell coordinate from the float copy of the position when the float
// quotient is clearly away from an integer: its error is bounded by
// 2^-23 (|p| + |bmin| + |p - bmin|) / rl + 2^-23 |t| (four times the
// rounding bound); otherwise the exact FP64 coordinate.
__device__ __forceinline__ int cell_coord_f(float pf, double p, const NLGeom& G, int k) {
  float q = pf - G.bminf[k];
  float t = q * G.inv_rlf[k];
  float ti = truncf(t);
  float fr = fabsf(t - ti);
  float margin = 1.1920929e-07f * ((fabsf(pf) + fabsf(G.bminf[k]) + fabsf(q)) * G.inv_rlf[k] + fabsf(t) + 1.0f);
  if (fr > margin && fr < 1.0f - margin && fabsf(t) < 1.0e6f) return (int)ti;
  return cell_coord(p, G, k);
}
__device__ __forceinline__ bool in_build_cell(const NLView& nl, int v, d3 p, int* co) {
  const NLGeom& G = geom_of(nl, v);
  const double* pp = &p.x;
  if (nl.pos32) {
    for (int k = 0; k < 3; ++k) co[k] = cell_coord_f(nl.pos32[3 * v + k], pp[k], G, k);
  } else {
    for (int k = 0; k < 3; ++k) co[k] = cell_coord(pp[k], G, k);
  }
  return nl.crow && co[0] == nl.bcoord[3 * v] && co[1] == nl.bcoord[3 * v + 1] && co[2] == nl.bcoord[3 * v + 2];
}
template <class F, class X>
__device__ __forceinline__ void visit_candidates(const PairTest& pt, const NLView& nl, const double* P, int v, d3 p,
                                                 const X& is_excluded, F& fn) {
  int lo = nl.crow[v], hi = nl.crow[v + 1];
  for (int q = lo; q < hi; ++q) visit_pair(pt, nl, P, v, p, nl.ccol[q], is_excluded, fn);
}
// The neighbours of v closer than the cut-off from its near row: those whose
// build-time cell (of the current cell list) is among the 27 cells around
// v's current cell co are the reference's candidates.  They are visited in
// the reference's order (cell offset x outer / z inner, then ascending
// index): the accepted pairs, usually none or one, are sorted in registers.
// mode 1: topology unchanged since the rows were built, entries flagged
// excluded are skipped without a test; mode 2: exclusion tested on the
// current topology.  Returns false (nothing visited) when more than
// NEAR_HITS pairs are accepted; the caller then takes the cell walk.
constexpr int NEAR_HITS = 8;
template <class F, class X>
__device__ __forceinline__ bool visit_near(const PairTest& pt, const NLView& nl, const double* P, int v, d3 p,
                                           int mode, const int* co, const X& is_excluded, F& fn) {
  const int* row = nl.nent + (size_t)v * TM_NEAR_CAP;
  const int n = nl.ncnt[v];
  long long key[NEAR_HITS];
  double dist[NEAR_HITS];
  d3 dif[NEAR_HITS];
  int hits = 0;
  for (int q = 0; q < n; ++q) {
    int c = row[q];
    if (mode == 1 && c < 0) continue;
    int j = c & 0x7fffffff;
    d3 pj;
    double s;
    if (!pair_within(pt, nl, P, p, j, &pj, &s)) continue;
    int ox = nl.bcoord[3 * j] - co[0], oy = nl.bcoord[3 * j + 1] - co[1], oz = nl.bcoord[3 * j + 2] - co[2];
    if (ox < -1 || ox > 1 || oy < -1 || oy > 1 || oz < -1 || oz > 1) continue;
    if (mode == 2 && nl.excl > 0 && is_excluded(v, j)) continue;
    if (hits == NEAR_HITS) return false;
    long long k = ((long long)((ox + 1) * 9 + (oy + 1) * 3 + (oz + 1)) << 32) | (long long)j;
    int h = hits++;
    while (h > 0 && key[h - 1] > k) {
      key[h] = key[h - 1];
      dist[h] = dist[h - 1];
      dif[h] = dif[h - 1];
      --h;
    }
    key[h] = k;
    dist[h] = __dsqrt_rn(s);
    dif[h] = exact_diff(p, pj);
  }
  for (int h = 0; h < hits; ++h) fn((int)(key[h] & 0xffffffff), dist[h], dif[h]);
  return true;
}
template <class F, class X>
__device__ __forceinline__ void visit_cells(const PairTest& pt, const NLView& nl, const double* P, int v, d3 p,
                                            const int* co, const X& is_excluded, F& fn) {
  const NLGeom& G = geom_of(nl, v);
  const int rep = rep_of(nl, v);
  for (int a = -1; a < 2; ++a) {
    int ii = co[0] + a;
    if (ii < 0 || ii >= G.shape[0]) continue;
    for (int b = -1; b < 2; ++b) {
      int jj = co[1] + b;
      if (jj < 0 || jj >= G.shape[1]) continue;
      for (int c = -1; c < 2; ++c) {
        int kk = co[2] + c;
        if (kk < 0 || kk >= G.shape[2]) continue;
        long long cid = ii * G.stride[0] + jj * G.stride[1] + kk * G.stride[2];
        int st = 0;
        int cnt = cell_find(nl, cell_key(cid, rep), &st);
        for (int q = 0; q < cnt; ++q) {
          int j = nl.cell_verts[st + q];
          if (j != v) visit_pair(pt, nl, P, v, p, j, is_excluded, fn);
        }
      }
    }
  }
}
template <class F, class X>
__device__ __forceinline__ void visit_verlet(const PairTest& pt, const NLView& nl, const double* P, int v, d3 p,
                                             const X& is_excluded, F& fn) {
  int lo = nl.vrow[v], hi = nl.vrow[v + 1];
  for (int q = lo; q < hi; ++q) visit_pair(pt, nl, P, v, p, nl.vcol[q], is_excluded, fn);
}

// All neighbours of v closer than dmax (T = sq_threshold(dmax)).
template <class F, class X>
__device__ __forceinline__ void for_each_neighbour_x(const NLView& nl, const double* P, int v, d3 p, double dmax,
                                                     double T, const X& is_excluded, F&& fn) {
  PairTest pt = make_pair_test(nl, v, dmax, T);
  if (nl.kind == 0) {
    int co[3];
    if (in_build_cell(nl, v, p, co))
      visit_candidates(pt, nl, P, v, p, is_excluded, fn);
    else
      visit_cells(pt, nl, P, v, p, co, is_excluded, fn);
  } else {
    visit_verlet(pt, nl, P, v, p, is_excluded, fn);
  }
}

template <class F>
__device__ __forceinline__ void for_each_neighbour(const NLView& nl, const Topo& t, const double* P, int v, d3 p,
                                                   double dmax, double T, F&& fn) {
  TableExcl x{t, nl.excl, &nl};
  for_each_neighbour_x(nl, P, v, p, dmax, T, x, fn);
}

// ---- per-vertex properties + block reduction + device-side assembly -------
__device__ __forceinline__ void assemble(const EP& ep, Globals* g) {
  const double* p = g->props;
  double da = p[0] / ep.refA - 1.0, dv = p[1] / ep.refV - 1.0, dc = p[2] / ep.refC - 1.0;
  double cA = ep.ka * da * da, cV = ep.kv * dv * dv, cC = ep.kc * dc * dc;
  double cB = ep.kb * p[3], cT = ep.kt * p[4], cR = ep.kr * p[5];
  double tot = 0.0;
  tot += cA;
  tot += cV;
  tot += cC;
  tot += cT;
  tot += cR;
  tot += cB;
  g->comps[0] = cA;
  g->comps[1] = cV;
  g->comps[2] = cC;
  g->comps[3] = cB;
  g->comps[4] = cT;
  g->comps[5] = cR;
  g->comps[6] = tot;
  g->gA = 2.0 * ep.ka / ep.refA * da;
  g->gV = 2.0 * ep.kv / ep.refV * dv;
  g->gC = 2.0 * ep.kc / ep.refC * dc;
  const double gg[3] = {g->gA, g->gV, g->gC};
  for (int k = 0; k < 3; ++k) {
    float h = (float)gg[k];
    g->gdf[2 * k] = h;
    g->gdf[2 * k + 1] = (float)(gg[k] - (double)h);
  }
}


// Energy of a set of global properties (src/kernel.h:110-122, summation
// order area, volume, area-difference, tether, repulsion, bending).
__device__ __forceinline__ double energy_of(const EP& ep, const double* p) {
  double da = p[0] / ep.refA - 1.0, dv = p[1] / ep.refV - 1.0, dc = p[2] / ep.refC - 1.0;
  double tot = 0.0;
  tot += ep.ka * da * da;
  tot += ep.kv * dv * dv;
  tot += ep.kc * dc * dc;
  tot += ep.kt * p[4];
  tot += ep.kr * p[5];
  tot += ep.kb * p[3];
  return tot;
}

EP make_ep(const tm_energy* e);

// Appends idx to list (count in *cnt) with one atomic per warp.
__device__ __forceinline__ void warp_append(bool need, int idx, int* list, int* cnt) {
  unsigned mask = __ballot_sync(__activemask(), need);
  if (!need) return;
  int lane = threadIdx.x & 31;
  int leader = __ffs(mask) - 1;
  int base = 0;
  if (lane == leader) base = atomicAdd(cnt, __popc(mask));
  base = __shfl_sync(mask, base, leader);
  list[base + __popc(mask & ((1u << lane) - 1u))] = idx;
}

// Flat-bottom edge penalty and its derivative dB/dl
// (src/mesh_tether.h:29-85) for an edge of length l.
// il = 1/l; below the flat bottom one division (1/(l - lc1)) and powers of
// il replace the four divisions of the textbook form
__device__ __forceinline__ void edge_bond(const EP& ep, double l, double il, double* val, double* fac) {
  int r = ep.r;
  double v = 0.0, f = 0.0;
  if (l > ep.lc0) {
    v = ep.br1 * ipow(l - ep.lc0, r);
    f = ep.br2 * ipow(l - ep.lc0, r - 1);
  }
  if (l < ep.lc1) {
    double ilm = 1.0 / (l - ep.lc1);
    double ex = exp(l * ilm);
    double ilr = ipow(il, r);
    if (!(l > ep.lc0)) v = ex * ilr;
    f -= ep.lc1 * (ilm * ilm) + r * il;
    f *= ilr;
    f *= ex;
  }
  *val = v;
  *fac = f;
}

}  // namespace tmg
