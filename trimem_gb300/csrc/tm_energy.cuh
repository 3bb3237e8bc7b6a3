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
  double rlc1;
  int rr;
  double tdiv;
};

struct __align__(16) FaceD {
  double nx, ny, nz, A, V, c0, c1, c2;
};
struct __align__(16) EdgeD {
  double l, th, db, flag;
};

constexpr int VB = 256;  // threads per block of k_vertex (fixed: it sets the reduction order)

__device__ __forceinline__ double cot_at(const FaceD& F, int c) { return c == 0 ? F.c0 : (c == 1 ? F.c1 : F.c2); }

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
  __device__ bool operator()(int v, int j) const { return excluded(t, excl, v, j); }
};

// Calls fn(j, |p - x_j|, p - x_j) for every neighbour j of vertex v (at p)
// closer than dmax, in the reference's order: the 27 cells (x outer, z
// inner), each cell's members in ascending order; or the Verlet row.
template <class F, class X>
__device__ __forceinline__ void for_each_neighbour_x(const NLView& nl, const double* P, int v, d3 p, double dmax,
                                                     const X& is_excluded, F&& fn) {
  if (nl.kind == 0) {
    int co[3];
    const double* pp = &p.x;
    for (int k = 0; k < 3; ++k) co[k] = (int)__ddiv_rn(__dsub_rn(pp[k], nl.bmin[k]), nl.rl[k]);
    for (int a = -1; a < 2; ++a) {
      int ii = co[0] + a;
      if (ii < 0 || ii >= nl.shape[0]) continue;
      for (int b = -1; b < 2; ++b) {
        int jj = co[1] + b;
        if (jj < 0 || jj >= nl.shape[1]) continue;
        for (int c = -1; c < 2; ++c) {
          int kk = co[2] + c;
          if (kk < 0 || kk >= nl.shape[2]) continue;
          long long cid = ii * nl.stride[0] + jj * nl.stride[1] + kk * nl.stride[2];
          int st = 0;
          int cnt = cell_find(nl, cid, &st);
          for (int q = 0; q < cnt; ++q) {
            int j = nl.cell_verts[st + q];
            if (j == v) continue;
            d3 pj = ld3(P, j);
            double l = exact_dist(p, pj);
            if (!(l < dmax)) continue;
            if (nl.excl > 0 && is_excluded(v, j)) continue;
            fn(j, l, exact_diff(p, pj));
          }
        }
      }
    }
  } else {
    int lo = nl.vrow[v], hi = nl.vrow[v + 1];
    for (int q = lo; q < hi; ++q) {
      int j = nl.vcol[q];
      d3 pj = ld3(P, j);
      double l = exact_dist(p, pj);
      if (l < dmax) fn(j, l, exact_diff(p, pj));
    }
  }
}

template <class F>
__device__ __forceinline__ void for_each_neighbour(const NLView& nl, const Topo& t, const double* P, int v, d3 p,
                                                   double dmax, F&& fn) {
  TableExcl x{t, nl.excl};
  for_each_neighbour_x(nl, P, v, p, dmax, x, fn);
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

}  // namespace tmg
