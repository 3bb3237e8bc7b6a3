// Device helpers that (re)derive the flat tables from the half-edge arrays.
#pragma once

#include "tm_internal.h"

namespace tmg {

struct TopoW {  // writable view of the half-edge arrays and derived tables
  int nv, ne, nf;
  int* to;
  int* next;
  int* face;
  int* vout;
  int* fhe;
  int4* slot;
  int* nbr;
  int* val;
  int* fv;
  int4* edge;
};

__device__ __forceinline__ void face_row(const TopoW& t, int f) {
  int h = t.fhe[f];
  int h1 = t.next[h];
  t.fv[3 * f] = t.to[h];
  t.fv[3 * f + 1] = t.to[h1];
  t.fv[3 * f + 2] = t.to[t.next[h1]];
}

__device__ __forceinline__ void edge_row(const TopoW& t, int e) {
  t.edge[e] = make_int4(t.to[2 * e + 1], t.to[2 * e], t.face[2 * e], t.face[2 * e + 1]);
}

// Ring slots of v by the rotation h -> next(opposite(h)); returns false when
// the valence exceeds TM_MAXVAL.
__device__ __forceinline__ bool ring_row(const TopoW& t, int v) {
  int h0 = t.vout[v];
  if (h0 < 0) {
    t.val[v] = 0;
    return true;
  }
  int h = h0, m = 0;
  do {
    if (m >= TM_MAXVAL) {
      t.val[v] = m;
      return false;
    }
    int f = t.face[h];
    int y = -1;
    if (f >= 0) {
      int c = t.fv[3 * f] == v ? 0 : (t.fv[3 * f + 1] == v ? 1 : 2);
      y = f | (c << 30);
    }
    t.slot[(size_t)m * t.nv + v] = make_int4(t.to[h], y, h >> 1, t.next[h] >> 1);
    t.nbr[(size_t)m * t.nv + v] = t.to[h];
    ++m;
    h = t.next[h ^ 1];
  } while (h != h0);
  t.val[v] = m;
  return true;
}

}  // namespace tmg
