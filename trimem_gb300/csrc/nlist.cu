// Neighbour lists: cell list and Verlet list (src/nlists/cell_list.h,
// verlet_list.h, nlist.cpp).
//
// Cell list build (every rebuild, all on the device except the box):
//   1. bounding box by a fixed-order min/max reduction, with the reference's
//      initial values {DBL_MAX,0,0} / {-1,0,0} (cell_list.h:46-47), copied
//      to the host, which derives r_list/shape/strides exactly like
//      cell_list.h:56-65
//   2. cell id per vertex with C truncation (cell_list.h:71-78), inserted
//      into an open-addressing hash table of the non-empty cells
//      (2x the vertex count, power of two) -> per-cell counts
//   3. exclusive scan of the counts -> cell start offsets
//   4. scatter of the vertex ids, then each cell sorted by vertex id, so a
//      cell lists its vertices in ascending order like the reference's
//      std::map<int, std::vector<int>>
// Queries bin the query point with its CURRENT position but look up the
// cells' build-time members, as the reference does (cell_list.h:131-219).
// Distances are rounded operation by operation (no FMA), so pair sets match
// the sequential CPU code bit for bit.
// The Verlet list is a CSR built from the cell list with cut-off rlist
// (verlet_list.h:18-35); its queries apply `< dmax`.
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstring>
#include <memory>

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

namespace tmg {

__device__ __forceinline__ unsigned long long cell_hash2(long long key) {
  unsigned long long z = (unsigned long long)key + 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

__device__ int cell_lookup(const NLView& nl, long long key, int* start) {
  unsigned long long h = cell_hash2(key) & nl.tmask;
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

__device__ bool nl_excluded(const Topo& t, int excl, int v, int j) {
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

namespace {

constexpr int BB = 256;

__global__ void k_bbox(int nv, const double* P, double* part) {
  __shared__ double s[6][BB];
  double lo[3] = {DBL_MAX, 0.0, 0.0}, hi[3] = {-1.0, 0.0, 0.0};
  for (int i = blockIdx.x * BB + threadIdx.x; i < nv; i += gridDim.x * BB)
    for (int k = 0; k < 3; ++k) {
      double x = P[3 * i + k];
      if (x < lo[k]) lo[k] = x;
      if (x > hi[k]) hi[k] = x;
    }
  for (int k = 0; k < 3; ++k) {
    s[k][threadIdx.x] = lo[k];
    s[3 + k][threadIdx.x] = hi[k];
  }
  __syncthreads();
  for (int o = BB / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o)
      for (int k = 0; k < 3; ++k) {
        double a = s[k][threadIdx.x + o];
        if (a < s[k][threadIdx.x]) s[k][threadIdx.x] = a;
        double b = s[3 + k][threadIdx.x + o];
        if (b > s[3 + k][threadIdx.x]) s[3 + k][threadIdx.x] = b;
      }
    __syncthreads();
  }
  if (threadIdx.x == 0)
    for (int k = 0; k < 6; ++k) part[6 * blockIdx.x + k] = s[k][0];
}

// Bounding box with the reference's initial values, then r_list, shape and
// strides exactly like src/nlists/cell_list.h:56-65.  One block reduces the
// block partials (min/max are exact, so the order does not matter).
__device__ void k_bbox_final_body(int nb, const double* part, double rlist, NLGeom* G);
__global__ void k_bbox_final(int nb, const double* part, double rlist, NLGeom* G) {
  k_bbox_final_body(nb, part, rlist, G);
}
__device__ void k_bbox_final_body(int nb, const double* part, double rlist, NLGeom* G) {
  __shared__ double s[6][BB];
  double lo[3] = {DBL_MAX, 0.0, 0.0}, hi[3] = {-1.0, 0.0, 0.0};
  for (int b = threadIdx.x; b < nb; b += BB)
    for (int k = 0; k < 3; ++k) {
      double a = part[6 * b + k], c = part[6 * b + 3 + k];
      if (a < lo[k]) lo[k] = a;
      if (c > hi[k]) hi[k] = c;
    }
  for (int k = 0; k < 3; ++k) {
    s[k][threadIdx.x] = lo[k];
    s[3 + k][threadIdx.x] = hi[k];
  }
  __syncthreads();
  for (int o = BB / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o)
      for (int k = 0; k < 3; ++k) {
        double a = s[k][threadIdx.x + o];
        if (a < s[k][threadIdx.x]) s[k][threadIdx.x] = a;
        double c = s[3 + k][threadIdx.x + o];
        if (c > s[3 + k][threadIdx.x]) s[3 + k][threadIdx.x] = c;
      }
    __syncthreads();
  }
  if (threadIdx.x) return;
  const double box_eps = 1.0e-6;
  for (int k = 0; k < 3; ++k) {
    double dim = __dadd_rn(__dsub_rn(s[3 + k][0], s[k][0]), box_eps);
    int nk = (int)__ddiv_rn(dim, rlist);
    G->rl[k] = nk > 0 ? __ddiv_rn(dim, (double)nk) : dim;
    G->inv_rl[k] = 1.0 / G->rl[k];
    G->inv_rlf[k] = (float)G->inv_rl[k];
    G->bminf[k] = (float)s[k][0];
    G->shape[k] = nk > 0 ? nk : 1;
    G->bmin[k] = s[k][0];
  }
  G->stride[0] = 1;
  G->stride[1] = G->shape[0];
  G->stride[2] = (long long)G->shape[0] * G->shape[1];
}

// batch: one partial box per 256-vertex block (blocks never straddle
// replicas), then one block per replica reduces its blocks
__global__ void k_bbox_blocks(int nv, const double* P, const int* vrep, double* part) {
  __shared__ double s[6][BB];
  double lo[3] = {DBL_MAX, 0.0, 0.0}, hi[3] = {-1.0, 0.0, 0.0};
  int i = blockIdx.x * BB + threadIdx.x;
  if (i < nv && vrep[i] >= 0)
    for (int k = 0; k < 3; ++k) {
      double x = P[3 * i + k];
      if (x < lo[k]) lo[k] = x;
      if (x > hi[k]) hi[k] = x;
    }
  for (int k = 0; k < 3; ++k) {
    s[k][threadIdx.x] = lo[k];
    s[3 + k][threadIdx.x] = hi[k];
  }
  __syncthreads();
  for (int o = BB / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o)
      for (int k = 0; k < 3; ++k) {
        double a = s[k][threadIdx.x + o];
        if (a < s[k][threadIdx.x]) s[k][threadIdx.x] = a;
        double b = s[3 + k][threadIdx.x + o];
        if (b > s[3 + k][threadIdx.x]) s[3 + k][threadIdx.x] = b;
      }
    __syncthreads();
  }
  if (threadIdx.x == 0)
    for (int k = 0; k < 6; ++k) part[6 * blockIdx.x + k] = s[k][0];
}

__global__ void k_bbox_final_batch(const int2* rblocks, const double* part, const double* rlist, NLGeom* geoms) {
  int r = blockIdx.x;
  int2 rb = rblocks[r];
  k_bbox_final_body(rb.y - rb.x, part + 6 * rb.x, rlist[r], geoms + r);
}

__global__ void k_table_init(CellEntry* T, size_t n) {
  size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i < n) {
    T[i].key = -1;
    T[i].start = 0;
    T[i].count = 0;
  }
}

__global__ void k_cell_insert(int nv, const double* P, NLView nl, CellEntry* T, long long* vcid, int* vcoord,
                              int* vslot, int* status) {
  int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= nv) return;
  int rep = rep_of(nl, v);
  if (rep < 0) {  // padding vertex of a batch: in no cell
    vslot[v] = -1;
    vcid[v] = -1;
    vcoord[3 * v] = vcoord[3 * v + 1] = vcoord[3 * v + 2] = -1000000;
    return;
  }
  const NLGeom& G = nl.geom[rep];
  long long id = 0;
  for (int k = 0; k < 3; ++k) {
    int c = (int)__ddiv_rn(__dsub_rn(P[3 * v + k], G.bmin[k]), G.rl[k]);
    vcoord[3 * v + k] = c;
    id += (long long)c * G.stride[k];
  }
  vcid[v] = id;
  id = cell_key(id, rep);
  unsigned long long h = cell_hash2(id) & nl.tmask;
  int slot = -1;
  for (unsigned long long p = 0; p <= nl.tmask; ++p) {
    unsigned long long prev =
        atomicCAS(reinterpret_cast<unsigned long long*>(&T[h].key), (unsigned long long)(-1LL), (unsigned long long)id);
    if (prev == (unsigned long long)(-1LL) || prev == (unsigned long long)id) {
      slot = (int)h;
      break;
    }
    h = (h + 1) & nl.tmask;
  }
  if (slot < 0) {
    atomicExch(status, 1);
    vslot[v] = 0;
    return;
  }
  vslot[v] = slot;
  atomicAdd(&T[slot].count, 1);
}

__global__ void k_counts(const CellEntry* T, int n, int* cnt) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) cnt[i] = T[i].count;
}
__global__ void k_set_start(CellEntry* T, int n, const int* start) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) T[i].start = start[i];
}
__global__ void k_scatter(int nv, const int* vslot, const CellEntry* T, int* fill, int* cell_verts) {
  int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= nv) return;
  int s = vslot[v];
  if (s < 0) return;
  int pos = T[s].start + atomicAdd(&fill[s], 1);
  cell_verts[pos] = v;
}
// sort each cell's members ascending and record each vertex's rank in its cell
__global__ void k_sort_cells(const CellEntry* T, int n, int* cell_verts, int* vrank) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  int c = T[i].count;
  if (c < 1) return;
  int* a = cell_verts + T[i].start;
  for (int x = 1; x < c; ++x) {
    int key = a[x];
    int y = x - 1;
    while (y >= 0 && a[y] > key) {
      a[y + 1] = a[y];
      --y;
    }
    a[y + 1] = key;
  }
  for (int x = 0; x < c; ++x) vrank[a[x]] = x;
}

// Position of the pair {v, u} in the reference's distance_matrix traversal
// (cell pairs in ascending first-cell id, neighbour offsets x-outer/z-inner,
// then the rank of the first-cell vertex, then of the second).
struct PairKey {
  long long icell;
  int off, ra, rb;
};
__device__ __forceinline__ PairKey pair_key(int v, int u, const long long* vcid, const int* vcoord,
                                            const int* vrank) {
  long long cv = vcid[v], cu = vcid[u];
  int a = v, b = u;
  if (cu < cv || (cu == cv && u < v)) {
    a = u;
    b = v;
  }
  PairKey k;
  k.icell = vcid[a];
  int dx = vcoord[3 * b] - vcoord[3 * a], dy = vcoord[3 * b + 1] - vcoord[3 * a + 1];
  int dz = vcoord[3 * b + 2] - vcoord[3 * a + 2];
  k.off = (dx + 1) * 9 + (dy + 1) * 3 + (dz + 1);
  k.ra = vrank[a];
  k.rb = vrank[b];
  return k;
}
__device__ __forceinline__ bool key_less(const PairKey& x, const PairKey& y) {
  if (x.icell != y.icell) return x.icell < y.icell;
  if (x.off != y.off) return x.off < y.off;
  if (x.ra != y.ra) return x.ra < y.ra;
  return x.rb < y.rb;
}

// order each Verlet row like the reference's push_back sequence
// (src/nlists/verlet_list.h:26-34)
__global__ void k_verlet_sort(int nv, const int* vrow, int* vcol, double* vd, const long long* vcid,
                              const int* vcoord, const int* vrank) {
  int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= nv) return;
  int lo = vrow[v], hi = vrow[v + 1];
  for (int x = lo + 1; x < hi; ++x) {
    int u = vcol[x];
    double du = vd[x];
    PairKey ku = pair_key(v, u, vcid, vcoord, vrank);
    int y = x - 1;
    while (y >= lo && key_less(ku, pair_key(v, vcol[y], vcid, vcoord, vrank))) {
      vcol[y + 1] = vcol[y];
      vd[y + 1] = vd[y];
      --y;
    }
    vcol[y + 1] = u;
    vd[y + 1] = du;
  }
}

// Pairs of the build-time cell neighbourhood of vertex a:
//   mode 0: Verlet build, all b != a, d <= rd        (both orders)
//   mode 1: distance_matrix of the cell list, each pair once with
//           (cid_b > cid_a) or (same cell and b > a), d <= rd
// pass 0 counts, pass 1 writes (d, i, j) at row offsets.
__global__ void k_cell_pairs(int nv, const double* P, NLView nl, Topo t, const int* vcoord, const long long* vcid,
                             double rd, int mode, int pass, int* cnt, const int* off, double* od, int* oi, int* oj) {
  int a = blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= nv) return;
  d3 pa = ld3(P, a);
  long long ca = vcid[a];
  const NLGeom& G = *nl.geom;
  int n = 0;
  int base = pass ? off[a] : 0;
  for (int x = -1; x < 2; ++x) {
    int ii = vcoord[3 * a] + x;
    if (ii < 0 || ii >= G.shape[0]) continue;
    for (int y = -1; y < 2; ++y) {
      int jj = vcoord[3 * a + 1] + y;
      if (jj < 0 || jj >= G.shape[1]) continue;
      for (int z = -1; z < 2; ++z) {
        int kk = vcoord[3 * a + 2] + z;
        if (kk < 0 || kk >= G.shape[2]) continue;
        long long cid = ii * G.stride[0] + jj * G.stride[1] + kk * G.stride[2];
        if (mode == 1 && cid < ca) continue;
        int st = 0;
        int cnt_c = cell_lookup(nl, cid, &st);
        for (int q = 0; q < cnt_c; ++q) {
          int b = nl.cell_verts[st + q];
          if (b == a) continue;
          if (mode == 1 && cid == ca && b < a) continue;
          double dd = exact_dist(pa, ld3(P, b));
          if (!(dd <= rd)) continue;
          if (nl_excluded(t, nl.excl, a, b)) continue;
          if (pass) {
            od[base + n] = dd;
            if (mode == 0) {
              oj[base + n] = b;
            } else {
              oi[base + n] = a < b ? a : b;
              oj[base + n] = a < b ? b : a;
            }
          }
          ++n;
        }
      }
    }
  }
  if (!pass) cnt[a] = n;
}

// Verlet rows of a batch of replicas (src/nlists/verlet_list.h:18-35): the
// members of the 27 build-time neighbour cells of vertex a in its own
// replica's grid (replica-tagged cell keys) closer than that replica's
// cut-off rlist[rep], not excluded at that replica's level; padding
// vertices have empty rows.  pass 0 counts, pass 1 writes (then ordered by
// k_verlet_sort like the single-mesh rows).
__global__ void k_verlet_batch(int nv, const double* P, NLView nl, Topo t, const int* vcoord,
                               const double* __restrict__ rlist, int pass, int* cnt, const int* off, double* od,
                               int* oj) {
  int a = blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= nv) return;
  const int rep = rep_of(nl, a);
  if (rep < 0) {
    if (!pass) cnt[a] = 0;
    return;
  }
  const NLGeom& G = nl.geom[rep];
  const double rd = rlist[rep];
  const int excl = excl_of(nl, a);
  const d3 pa = ld3(P, a);
  int n = 0;
  int base = pass ? off[a] : 0;
  for (int x = -1; x < 2; ++x) {
    int ii = vcoord[3 * a] + x;
    if (ii < 0 || ii >= G.shape[0]) continue;
    for (int y = -1; y < 2; ++y) {
      int jj = vcoord[3 * a + 1] + y;
      if (jj < 0 || jj >= G.shape[1]) continue;
      for (int z = -1; z < 2; ++z) {
        int kk = vcoord[3 * a + 2] + z;
        if (kk < 0 || kk >= G.shape[2]) continue;
        long long cid = ii * G.stride[0] + jj * G.stride[1] + kk * G.stride[2];
        int st = 0;
        int c = cell_lookup(nl, cell_key(cid, rep), &st);
        for (int q = 0; q < c; ++q) {
          int b = nl.cell_verts[st + q];
          if (b == a) continue;
          double dd = exact_dist(pa, ld3(P, b));
          if (!(dd <= rd)) continue;
          if (nl_excluded(t, excl, a, b)) continue;
          if (pass) {
            od[base + n] = dd;
            oj[base + n] = b;
          }
          ++n;
        }
      }
    }
  }
  if (!pass) cnt[a] = n;
}

// candidate rows: members of the 27 build-time neighbour cells of vertex a in
// the reference's scan order (x outer, z inner; members ascending), self
// excluded.  pass 0 counts, pass 1 writes.
__global__ void k_cand(int nv, NLView nl, const int* vcoord, int pass, int* cnt, const int* off, int* out) {
  int a = blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= nv) return;
  int rep = rep_of(nl, a);
  if (rep < 0) {
    if (!pass) cnt[a] = 0;
    return;
  }
  const NLGeom& G = nl.geom[rep];
  int n = 0;
  int base = pass ? off[a] : 0;
  for (int x = -1; x < 2; ++x) {
    int ii = vcoord[3 * a] + x;
    if (ii < 0 || ii >= G.shape[0]) continue;
    for (int y = -1; y < 2; ++y) {
      int jj = vcoord[3 * a + 1] + y;
      if (jj < 0 || jj >= G.shape[1]) continue;
      for (int z = -1; z < 2; ++z) {
        int kk = vcoord[3 * a + 2] + z;
        if (kk < 0 || kk >= G.shape[2]) continue;
        long long cid = ii * G.stride[0] + jj * G.stride[1] + kk * G.stride[2];
        int st = 0;
        int c = cell_lookup(nl, cell_key(cid, rep), &st);
        for (int q = 0; q < c; ++q) {
          int b = nl.cell_verts[st + q];
          if (b == a) continue;
          if (pass) out[base + n] = b;
          ++n;
        }
      }
    }
  }
  if (!pass) cnt[a] = n;
}

// Near rows (rebuilt only when flagged stale): the vertices closer than rn
// to each vertex (squared threshold rn2, rounded up), found through the cell
// table (the cells that meet the ball of radius rn), with a flag for pairs
// excluded on the current topology.  A row longer than TM_NEAR_CAP marks the
// rows unusable (flag[3]).
constexpr int NB = 128;  // threads per block of k_near
__global__ void __launch_bounds__(NB) k_near(int nv, const double* P, NLView nl, Topo t, int excl, double rn,
                                             double rn2, int* flag, int* ncnt, int* nent, double* xb,
                                             const EP* eps) {
  // the row of each thread, staged in shared memory (stride 49: no bank
  // conflicts) while the exclusion flags are set
  __shared__ int srow[NB][TM_NEAR_CAP + 1];
  if (flag[1] == 0) return;  // rows still valid
  int a = blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= nv) return;
  const int rep = rep_of(nl, a);
  if (rep < 0) {  // padding vertex of a batch
    ncnt[a] = 0;
    return;
  }
  if (eps) {  // batch: the replica's cut-off
    rn = 2.0 * eps[rep].rlc1;
    rn2 = rn * rn * (1.0 + 1e-12);
  }
  const NLGeom& G = nl.geom[rep];
  d3 pa = ld3(P, a);
  const double* pp = &pa.x;
  int lo[3], hi[3];
  // position in cell units (float) for the box-distance pruning; a cell is
  // skipped only when it is farther than rn after every axis distance is
  // shortened by 1e-3 cell widths plus 8 float ulps of the coordinate, far
  // above the float rounding of the cell coordinate
  float u[3], rlf[3], mg[3];
  for (int k = 0; k < 3; ++k) {
    lo[k] = max(0, (int)floor((pp[k] - rn - G.bmin[k]) * G.inv_rl[k]) - 1);
    hi[k] = min(G.shape[k] - 1, (int)floor((pp[k] + rn - G.bmin[k]) * G.inv_rl[k]) + 1);
    u[k] = (float)((pp[k] - G.bmin[k]) * G.inv_rl[k]);
    rlf[k] = (float)G.rl[k];
    mg[k] = 1e-3f + 9.6e-7f * fabsf(u[k]);
  }
  const float rnf2 = (float)rn2 * 1.0001f;
  int* row = srow[threadIdx.x];
  int n = 0;
  for (int ii = lo[0]; ii <= hi[0]; ++ii) {
    float dx = fmaxf(fmaxf((float)ii - u[0], u[0] - (float)(ii + 1)) - mg[0], 0.0f) * rlf[0];
    for (int jj = lo[1]; jj <= hi[1]; ++jj) {
      float dy = fmaxf(fmaxf((float)jj - u[1], u[1] - (float)(jj + 1)) - mg[1], 0.0f) * rlf[1];
      float gxy = dx * dx + dy * dy;
      if (gxy > rnf2) continue;
      for (int kk = lo[2]; kk <= hi[2]; ++kk) {
        float dz = fmaxf(fmaxf((float)kk - u[2], u[2] - (float)(kk + 1)) - mg[2], 0.0f) * rlf[2];
        if (gxy + dz * dz > rnf2) continue;
        long long cid = ii * G.stride[0] + jj * G.stride[1] + kk * G.stride[2];
        int st = 0;
        int c = cell_lookup(nl, cell_key(cid, rep), &st);
        for (int q = 0; q < c; ++q) {
          int b = nl.cell_verts[st + q];
          if (b == a) continue;
          d3 pb = ld3(P, b);
          double ex = pa.x - pb.x, ey = pa.y - pb.y, ez = pa.z - pb.z;
          if (ex * ex + ey * ey + ez * ez >= rn2) continue;
          if (n < TM_NEAR_CAP) row[n] = b;
          ++n;
        }
      }
    }
  }
  if (n > TM_NEAR_CAP) atomicOr(&flag[3], 1);
  n = min(n, TM_NEAR_CAP);
  // exclusion flags (nl_excluded): an entry is excluded when it is in the
  // ring of a or, at level 2, in the ring of a ring vertex of a; the rings
  // are walked once and their vertices looked up in the row
  if (nl.rexcl) excl = nl.rexcl[rep];  // batch: the replica's level
  if (excl > 0 && n > 0) {
    const int d = t.val[a];
    for (int m = 0; m < d; ++m) {
      const int w = t.nbr[(size_t)m * t.nv + a];
      for (int e = 0; e < n; ++e)
        if (row[e] == w) row[e] |= (int)0x80000000u;
      if (excl > 1) {
        const int dw = t.val[w];
        for (int q = 0; q < dw; ++q) {
          const int x = t.nbr[(size_t)q * t.nv + w];
          for (int e = 0; e < n; ++e)
            if ((row[e] & 0x7fffffff) == x) row[e] |= (int)0x80000000u;
        }
      }
    }
  }
  int* out = nent + (size_t)a * TM_NEAR_CAP;
  for (int e = 0; e < n; ++e) out[e] = row[e];
  ncnt[a] = n;
  xb[3 * a] = pa.x;
  xb[3 * a + 1] = pa.y;
  xb[3 * a + 2] = pa.z;
}
// after a build: usable unless a row overflowed; record the topology version
__global__ void k_near_done(int* flag, const int* dtopo) {
  if (threadIdx.x || blockIdx.x) return;
  if (flag[1] == 0) return;
  flag[1] = flag[3];
  flag[2] = *dtopo;
  flag[3] = 0;
}
// before a cell-list rebuild: the rows go stale once some vertex has moved
// lc1/2 or more from where they were built (thr2 rounded down; NaN moves)
__global__ void k_near_check(int nv, const double* __restrict__ P, const double* __restrict__ xb, double thr2,
                             int* flag, const int* __restrict__ vrep, const EP* __restrict__ eps) {
  int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= nv || flag[1]) return;
  if (vrep) {  // batch: the replica's skin, padding vertices never move
    int r = vrep[v];
    if (r < 0) return;
    thr2 = 0.25 * eps[r].rlc1 * eps[r].rlc1 * (1.0 - 1e-12);
  }
  double dx = P[3 * v] - xb[3 * v], dy = P[3 * v + 1] - xb[3 * v + 1], dz = P[3 * v + 2] - xb[3 * v + 2];
  if (!(dx * dx + dy * dy + dz * dz < thr2)) flag[1] = 1;
}

// distance_matrix of the Verlet list: rows in vertex order, d < rd
__global__ void k_verlet_dm(int nv, const double* P, const int* vrow, const int* vcol, double rd, int pass, int* cnt,
                            const int* off, double* od, int* oi, int* oj) {
  int a = blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= nv) return;
  d3 pa = ld3(P, a);
  int n = 0;
  int base = pass ? off[a] : 0;
  for (int q = vrow[a]; q < vrow[a + 1]; ++q) {
    int b = vcol[q];
    double dd = exact_dist(pa, ld3(P, b));
    if (dd < rd) {
      if (pass) {
        od[base + n] = dd;
        oi[base + n] = a;
        oj[base + n] = b;
      }
      ++n;
    }
  }
  if (!pass) cnt[a] = n;
}

// point_distances for one vertex (single thread; API use only)
__global__ void k_point(int pid, const double* P, NLView nl, Topo t, double rd, int pass, int* count, double* od,
                        int* oj) {
  if (threadIdx.x || blockIdx.x) return;
  d3 p = ld3(P, pid);
  int n = 0;
  if (nl.kind == 0) {
    const NLGeom& G = *nl.geom;
    int co[3];
    const double* pp = &p.x;
    for (int k = 0; k < 3; ++k) co[k] = (int)__ddiv_rn(__dsub_rn(pp[k], G.bmin[k]), G.rl[k]);
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
          int cc = cell_lookup(nl, cid, &st);
          for (int q = 0; q < cc; ++q) {
            int j = nl.cell_verts[st + q];
            if (j == pid) continue;
            if (nl_excluded(t, nl.excl, pid, j)) continue;
            d3 pj = ld3(P, j);
            if (exact_dist(p, pj) < rd) {
              if (pass) {
                st3(od, n, exact_diff(p, pj));
                oj[n] = j;
              }
              ++n;
            }
          }
        }
      }
    }
  } else {
    for (int q = nl.vrow[pid]; q < nl.vrow[pid + 1]; ++q) {
      int j = nl.vcol[q];
      d3 pj = ld3(P, j);
      if (exact_dist(p, pj) < rd) {
        if (pass) {
          st3(od, n, exact_diff(p, pj));
          oj[n] = j;
        }
        ++n;
      }
    }
  }
  if (!pass) *count = n;
}

inline int nblk(long n, int b) { return (int)((n + b - 1) / b); }

}  // namespace

// Steps 2-4 of the cell-list build and the candidate rows (shared by single
// meshes and batches; V.geom and V.vrep are set by the caller).
static void build_cells(tm_nlist* nl, NLView& V, int nv, const double* P, cudaStream_t s, bool candidates) {
  // 2. hash table of the non-empty cells: 2x the vertex count, power of two
  size_t tsize = 64;
  while (tsize < 2 * (size_t)std::max(nv, 1)) tsize <<= 1;
  nl->table.ensure(tsize);
  V.tmask = tsize - 1;
  nl->vcid.ensure(std::max(nv, 1));
  nl->vcoord.ensure(3 * (size_t)std::max(nv, 1));
  nl->vslot.ensure(std::max(nv, 1));
  nl->vrank.ensure(std::max(nv, 1));
  nl->cnt.ensure(tsize + 1);
  nl->fill.ensure(tsize);
  nl->cell_verts.ensure(std::max(nv, 1));
  nl->d_count.ensure(4);
  k_table_init<<<nblk((long)tsize, 256), 256, 0, s>>>(nl->table.get(), tsize);
  TM_LAUNCH();
  V.table = nl->table.get();
  V.cell_verts = nl->cell_verts.get();
  V.bcoord = nl->vcoord.get();  // build-time cell of every vertex
  if (nv > 0) {
    k_cell_insert<<<nblk(nv, 256), 256, 0, s>>>(nv, P, V, nl->table.get(), nl->vcid.get(), nl->vcoord.get(),
                                                nl->vslot.get(), nl->d_count.get());
    TM_LAUNCH();
    // 3. offsets
    k_counts<<<nblk((long)tsize, 256), 256, 0, s>>>(nl->table.get(), (int)tsize, nl->cnt.get());
    TM_LAUNCH();
    exclusive_scan_int(nl->cnt.get(), nl->fill.get(), (int)tsize, nullptr, nl->tmp, s);
    k_set_start<<<nblk((long)tsize, 256), 256, 0, s>>>(nl->table.get(), (int)tsize, nl->fill.get());
    TM_LAUNCH();
    // 4. scatter + per-cell sort (members ascending, rank of each vertex)
    TM_CUDA(cudaMemsetAsync(nl->fill.get(), 0, sizeof(int) * tsize, s));
    k_scatter<<<nblk(nv, 256), 256, 0, s>>>(nv, nl->vslot.get(), nl->table.get(), nl->fill.get(),
                                            nl->cell_verts.get());
    TM_LAUNCH();
    k_sort_cells<<<nblk((long)tsize, 256), 256, 0, s>>>(nl->table.get(), (int)tsize, nl->cell_verts.get(),
                                                        nl->vrank.get());
    TM_LAUNCH();
  }
  if (candidates && nv > 0) {
    // candidate rows for the queries of points that stay in their build cell
    nl->crow.ensure((size_t)nv + 1);
    nl->cnt.ensure((size_t)nv + 1);
    k_cand<<<nblk(nv, 256), 256, 0, s>>>(nv, V, nl->vcoord.get(), 0, nl->cnt.get(), nullptr, nullptr);
    TM_LAUNCH();
    TM_CUDA(cudaMemsetAsync(nl->cnt.get() + nv, 0, sizeof(int), s));
    int total = 0;
    exclusive_scan_int(nl->cnt.get(), nl->crow.get(), nv + 1, &total, nl->tmp, s);
    // rows are only kept while they stay small (coarse grids fall back to the
    // cell table)
    if ((long long)total <= 64LL * nv) {
      nl->ccol.ensure(std::max(total, 1));
      k_cand<<<nblk(nv, 256), 256, 0, s>>>(nv, V, nl->vcoord.get(), 1, nullptr, nl->crow.get(), nl->ccol.get());
      TM_LAUNCH();
      V.crow = nl->crow.get();
      V.ccol = nl->ccol.get();
    }
  }
}

// Near rows for repulsion queries at cut-off lc1 (skin lc1/2).  A pair
// closer than lc1 at query time whose vertices both moved less than lc1/2
// since the rows were built was closer than 2 lc1 then, so the row holds
// every neighbour the query can accept; the query keeps the ones whose
// build-time cell of the current cell list is among the 27 around its own
// current cell and visits them in the reference's order.  The rows do not
// depend on the cell list, so a cell-list rebuild rebuilds them only when a
// vertex has moved lc1/2 since they were built (decided on the device).
static void refresh_near(tm_nlist* nl, tm_mesh* m, NLView& V, const double* P, double lc1, cudaStream_t s,
                         const EP* eps = nullptr) {
  int nv = nl->nv;
  Topo t = m->topo();
  double rn = 2.0 * lc1;
  if (nl->near_nv != nv || nl->near_lc1 != lc1) {
    nl->nent.ensure((size_t)nv * TM_NEAR_CAP);
    nl->ncnt.ensure(nv);
    nl->xb.ensure(3 * (size_t)nv);
    nl->nflag.ensure(4);
    int init[4] = {0, 1, 0, 0};  // stale until built
    TM_CUDA(cudaMemcpyAsync(nl->nflag.get(), init, sizeof(init), cudaMemcpyHostToDevice, s));
    TM_CUDA(cudaStreamSynchronize(s));
    nl->near_nv = nv;
    nl->near_lc1 = lc1;
    nl->near_move2 = 0.25 * lc1 * lc1 * (1.0 - 1e-12);
  }
  int* flag = nl->nflag.get();
  k_near_check<<<nblk(nv, 256), 256, 0, s>>>(nv, P, nl->xb.get(), nl->near_move2, flag, V.vrep, eps);
  TM_LAUNCH();
  k_near<<<nblk(nv, NB), NB, 0, s>>>(nv, P, V, t, V.excl, rn, rn * rn * (1.0 + 1e-12), flag, nl->ncnt.get(),
                                       nl->nent.get(), nl->xb.get(), eps);
  TM_LAUNCH();
  k_near_done<<<1, 32, 0, s>>>(flag, m->d_topo_ver.get());
  TM_LAUNCH();
  V.nent = nl->nent.get();
  V.ncnt = nl->ncnt.get();
  V.nflag = flag;
  V.dtopo = m->d_topo_ver.get();
}

void nlist_make(tm_nlist* nl, tm_mesh* m, const tm_params& p, const double* P, cudaStream_t s) {
  if (p.n_search != 0 && p.n_search != 1) fail(TM_ERR_ARG, "Unknown neighbour search algorithm.");
  if (p.exclusion_level < 0 || p.exclusion_level > 2) fail(TM_ERR_ARG, "Unsupported exclusion level");
  nl->prm = p;
  int nv = m->nv;
  nl->nv = nv;
  NLView& V = nl->view;
  V = NLView{};
  V.kind = 0;
  V.excl = p.exclusion_level;
  // 1. box and cell geometry (device only, no host round trip)
  int nb = std::max(1, std::min(1024, nblk(nv, BB)));
  nl->bbox.ensure(6 * (size_t)nb + 6);
  nl->geom.ensure(1);
  V.geom = nl->geom.get();
  if (nv > 0) {
    k_bbox<<<nb, BB, 0, s>>>(nv, P, nl->bbox.get());
    TM_LAUNCH();
  }
  k_bbox_final<<<1, BB, 0, s>>>(nv > 0 ? nb : 0, nl->bbox.get(), p.rlist, nl->geom.get());
  TM_LAUNCH();
  // with near rows the candidate rows are not needed: the rare fallback
  // (a vertex moved lc1/2 since the rows were built) takes the cell walk
  const bool near = p.n_search == 0 && p.rep_lc1 > 0 && p.rlist >= p.rep_lc1 && nv > 0;
  build_cells(nl, V, nv, P, s, p.n_search == 0 && !near);
  if (near) refresh_near(nl, m, V, P, p.rep_lc1, s);
  if (p.n_search == 1) {
    // Verlet CSR from the cell list at cut-off rlist, rows in the reference's
    // insertion order
    nl->vrow.ensure((size_t)nv + 1);
    Topo t = m->topo();
    int total = 0;
    if (nv > 0) {
      nl->cnt.ensure((size_t)nv + 1);
      k_cell_pairs<<<nblk(nv, 256), 256, 0, s>>>(nv, P, V, t, nl->vcoord.get(), nl->vcid.get(), p.rlist, 0, 0,
                                                 nl->cnt.get(), nullptr, nullptr, nullptr, nullptr);
      TM_LAUNCH();
      TM_CUDA(cudaMemsetAsync(nl->cnt.get() + nv, 0, sizeof(int), s));
      exclusive_scan_int(nl->cnt.get(), nl->vrow.get(), nv + 1, &total, nl->tmp, s);
      nl->vcol.ensure(std::max(total, 1));
      nl->d_res.ensure(std::max(total, 1));
      k_cell_pairs<<<nblk(nv, 256), 256, 0, s>>>(nv, P, V, t, nl->vcoord.get(), nl->vcid.get(), p.rlist, 0, 1,
                                                 nullptr, nl->vrow.get(), nl->d_res.get(), nullptr, nl->vcol.get());
      TM_LAUNCH();
      k_verlet_sort<<<nblk(nv, 128), 128, 0, s>>>(nv, nl->vrow.get(), nl->vcol.get(), nl->d_res.get(),
                                                  nl->vcid.get(), nl->vcoord.get(), nl->vrank.get());
      TM_LAUNCH();
    } else {
      TM_CUDA(cudaMemsetAsync(nl->vrow.get(), 0, sizeof(int), s));
      nl->vcol.ensure(1);
    }
    V.kind = 1;
    V.vrow = nl->vrow.get();
    V.vcol = nl->vcol.get();
  }
}

void nlist_make_batch(tm_nlist* nl, tm_mesh* m, int R, const int* d_vrep, const int2* d_rblocks,
                      const double* d_rlist, int excl, const int* d_rexcl, const double* P, cudaStream_t s,
                      const EP* d_eps, bool near, bool verlet) {
  if (excl < 0 || excl > 2) fail(TM_ERR_ARG, "Unsupported exclusion level");
  int nv = m->nv;
  nl->nv = nv;
  nl->prm.n_search = verlet ? 1 : 0;
  nl->prm.exclusion_level = excl;
  NLView& V = nl->view;
  V = NLView{};
  V.kind = 0;
  V.excl = excl;
  V.rexcl = d_rexcl;
  V.vrep = d_vrep;
  int nb = std::max(1, nblk(nv, BB));
  nl->bbox.ensure(6 * (size_t)nb);
  nl->geom.ensure(R);
  V.geom = nl->geom.get();
  if (nv > 0) {
    k_bbox_blocks<<<nb, BB, 0, s>>>(nv, P, d_vrep, nl->bbox.get());
    TM_LAUNCH();
  }
  k_bbox_final_batch<<<R, BB, 0, s>>>(d_rblocks, nl->bbox.get(), d_rlist, nl->geom.get());
  TM_LAUNCH();
  if (verlet) {
    // Verlet rows at each replica's cut-off, ordered like the single-mesh
    // rows (the reference's insertion order)
    build_cells(nl, V, nv, P, s, false);
    nl->vrow.ensure((size_t)nv + 1);
    Topo t = m->topo();
    int total = 0;
    if (nv > 0) {
      nl->cnt.ensure((size_t)nv + 1);
      k_verlet_batch<<<nblk(nv, 256), 256, 0, s>>>(nv, P, V, t, nl->vcoord.get(), d_rlist, 0, nl->cnt.get(),
                                                   nullptr, nullptr, nullptr);
      TM_LAUNCH();
      TM_CUDA(cudaMemsetAsync(nl->cnt.get() + nv, 0, sizeof(int), s));
      exclusive_scan_int(nl->cnt.get(), nl->vrow.get(), nv + 1, &total, nl->tmp, s);
      nl->vcol.ensure(std::max(total, 1));
      nl->d_res.ensure(std::max(total, 1));
      k_verlet_batch<<<nblk(nv, 256), 256, 0, s>>>(nv, P, V, t, nl->vcoord.get(), d_rlist, 1, nullptr,
                                                   nl->vrow.get(), nl->d_res.get(), nl->vcol.get());
      TM_LAUNCH();
      k_verlet_sort<<<nblk(nv, 128), 128, 0, s>>>(nv, nl->vrow.get(), nl->vcol.get(), nl->d_res.get(),
                                                  nl->vcid.get(), nl->vcoord.get(), nl->vrank.get());
      TM_LAUNCH();
    } else {
      TM_CUDA(cudaMemsetAsync(nl->vrow.get(), 0, sizeof(int), s));
      nl->vcol.ensure(1);
    }
    V.kind = 1;
    V.vrow = nl->vrow.get();
    V.vcol = nl->vcol.get();
    return;
  }
  // candidate rows as well: unrelaxed replicas can move a skin's width
  // within a few steps, and then the candidate rows keep most vertices off
  // the cell walk
  build_cells(nl, V, nv, P, s, true);
  // near rows with each replica's cut-off (the lc1 argument only tags the
  // rows: any positive value)
  if (near && nv > 0) refresh_near(nl, m, V, P, 1.0, s, d_eps);
}

int64_t nlist_distance_matrix(tm_nlist* nl, tm_mesh* m, const double* P, double rd, cudaStream_t s) {
  int nv = m->nv;
  nl->res_d.clear();
  nl->res_i.clear();
  nl->res_j.clear();
  if (nv == 0) return 0;
  if (nv != nl->nv) fail(TM_ERR_ARG, "mesh does not match the neighbour list");
  nl->cnt.ensure((size_t)nv + 1);
  nl->fill.ensure((size_t)nv + 1);
  Topo t = m->topo();
  int total = 0;
  if (nl->view.kind == 0)
    k_cell_pairs<<<nblk(nv, 256), 256, 0, s>>>(nv, P, nl->view, t, nl->vcoord.get(), nl->vcid.get(), rd, 1, 0,
                                               nl->cnt.get(), nullptr, nullptr, nullptr, nullptr);
  else
    k_verlet_dm<<<nblk(nv, 256), 256, 0, s>>>(nv, P, nl->vrow.get(), nl->vcol.get(), rd, 0, nl->cnt.get(), nullptr,
                                              nullptr, nullptr, nullptr);
  TM_LAUNCH();
  TM_CUDA(cudaMemsetAsync(nl->cnt.get() + nv, 0, sizeof(int), s));
  exclusive_scan_int(nl->cnt.get(), nl->fill.get(), nv + 1, &total, nl->tmp, s);
  nl->d_res.ensure(std::max(total, 1));
  nl->d_resi.ensure(std::max(total, 1));
  nl->d_resj.ensure(std::max(total, 1));
  if (nl->view.kind == 0)
    k_cell_pairs<<<nblk(nv, 256), 256, 0, s>>>(nv, P, nl->view, t, nl->vcoord.get(), nl->vcid.get(), rd, 1, 1,
                                               nullptr, nl->fill.get(), nl->d_res.get(), nl->d_resi.get(),
                                               nl->d_resj.get());
  else
    k_verlet_dm<<<nblk(nv, 256), 256, 0, s>>>(nv, P, nl->vrow.get(), nl->vcol.get(), rd, 1, nullptr, nl->fill.get(),
                                              nl->d_res.get(), nl->d_resi.get(), nl->d_resj.get());
  TM_LAUNCH();
  nl->res_d.resize(total);
  nl->res_i.resize(total);
  nl->res_j.resize(total);
  if (total) {
    TM_CUDA(cudaMemcpyAsync(nl->res_d.data(), nl->d_res.get(), sizeof(double) * total, cudaMemcpyDeviceToHost, s));
    TM_CUDA(cudaMemcpyAsync(nl->res_i.data(), nl->d_resi.get(), sizeof(int) * total, cudaMemcpyDeviceToHost, s));
    TM_CUDA(cudaMemcpyAsync(nl->res_j.data(), nl->d_resj.get(), sizeof(int) * total, cudaMemcpyDeviceToHost, s));
  }
  TM_CUDA(cudaStreamSynchronize(s));
  return total;
}

int64_t nlist_point_distances(tm_nlist* nl, tm_mesh* m, const double* P, int pid, double rd, cudaStream_t s) {
  nl->res_d.clear();
  nl->res_i.clear();
  nl->res_j.clear();
  if (pid < 0 || pid >= m->nv) fail(TM_ERR_ARG, "pid out of range");
  if (m->nv != nl->nv) fail(TM_ERR_ARG, "mesh does not match the neighbour list");
  Topo t = m->topo();
  nl->d_count.ensure(4);
  k_point<<<1, 1, 0, s>>>(pid, P, nl->view, t, rd, 0, nl->d_count.get(), nullptr, nullptr);
  TM_LAUNCH();
  int n = 0;
  TM_CUDA(cudaMemcpyAsync(&n, nl->d_count.get(), sizeof(int), cudaMemcpyDeviceToHost, s));
  TM_CUDA(cudaStreamSynchronize(s));
  nl->d_res.ensure(3 * (size_t)std::max(n, 1));
  nl->d_resj.ensure(std::max(n, 1));
  k_point<<<1, 1, 0, s>>>(pid, P, nl->view, t, rd, 1, nullptr, nl->d_res.get(), nl->d_resj.get());
  TM_LAUNCH();
  nl->res_d.resize(3 * (size_t)n);
  nl->res_j.resize(n);
  if (n) {
    TM_CUDA(cudaMemcpyAsync(nl->res_d.data(), nl->d_res.get(), sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, s));
    TM_CUDA(cudaMemcpyAsync(nl->res_j.data(), nl->d_resj.get(), sizeof(int) * n, cudaMemcpyDeviceToHost, s));
  }
  TM_CUDA(cudaStreamSynchronize(s));
  return n;
}

}  // namespace tmg

// --------------------------------------------------------------------------
// C ABI
// --------------------------------------------------------------------------


extern "C" {

int tm_nlist_create(tm_mesh* m, const tm_params* p, tm_nlist** out) {
  TM_API_BEGIN
  if (!m || !p || !out) fail(TM_ERR_ARG, "NULL argument");
  *out = nullptr;
  std::unique_ptr<tm_nlist> nl(new tm_nlist());
  m->upload_points(m->stream);
  tmg::nlist_make(nl.get(), m, *p, m->d_pts.get(), m->stream);
  TM_CUDA(cudaStreamSynchronize(m->stream));
  *out = nl.release();
  TM_API_END
}

int tm_nlist_destroy(tm_nlist* nl) {
  delete nl;
  return TM_OK;
}

int tm_nlist_distance_matrix(tm_nlist* nl, tm_mesh* m, double rdist, int64_t* count) {
  TM_API_BEGIN
  if (!nl || !m || !count) fail(TM_ERR_ARG, "NULL argument");
  m->upload_points(m->stream);
  *count = tmg::nlist_distance_matrix(nl, m, m->d_pts.get(), rdist, m->stream);
  TM_API_END
}

int tm_nlist_point_distances(tm_nlist* nl, tm_mesh* m, int64_t pid, double rdist, int64_t* count) {
  TM_API_BEGIN
  if (!nl || !m || !count) fail(TM_ERR_ARG, "NULL argument");
  m->upload_points(m->stream);
  *count = tmg::nlist_point_distances(nl, m, m->d_pts.get(), (int)pid, rdist, m->stream);
  TM_API_END
}

int tm_nlist_fetch(tm_nlist* nl, double* d, int32_t* i, int32_t* j) {
  if (!nl) return TM_ERR_ARG;
  if (d && !nl->res_d.empty()) std::memcpy(d, nl->res_d.data(), sizeof(double) * nl->res_d.size());
  if (i && !nl->res_i.empty()) std::memcpy(i, nl->res_i.data(), sizeof(int) * nl->res_i.size());
  if (j && !nl->res_j.empty()) std::memcpy(j, nl->res_j.data(), sizeof(int) * nl->res_j.size());
  return TM_OK;
}

}  // extern "C"
