// Metropolis edge-flip sweep (src/flips.cpp:22-165, src/flip_utils.cpp:19-114).
//
// The reference draws random edges and either flips them one by one
// (flip_serial) or lets OpenMP threads lock the edge patches of their
// proposals and serialises the acceptance in a critical section
// (flip_parallel_batches).  Here a sweep is a sequence of windows of
// proposals, every step on the device (windows are queued eight at a time;
// their size lives in device memory, so no window waits for the host):
//   k_fill    window = deferred proposals (in order) + new proposals
//   k_claim   each proposal claims the vertices of its patch (the quad's
//             four vertices and their ring neighbours) with atomicMax of a
//             (window, slot) tag that the lowest slot of the current window
//             wins
//   k_winner  a proposal that owns its quad's four vertices is a winner: no
//             lower slot's quad lies within one edge of its quad, which is
//             what makes the property change of every winner exact on the
//             window's starting topology while the lower winners flip (a
//             flip changes the rings of its quad's vertices only, and the
//             change of a proposal reads the rings of its quad's vertices and
//             of their neighbours); in serial mode the window is cut at the
//             first loser, so proposals are decided in proposal order
//             (k_claim_win does the three in one cooperative launch with a
//             grid barrier when it fits).  The reference locks a larger
//             patch, the edges of the faces around the quad's vertices
//             (flip_utils.cpp:43-68); the vertex patch suffices for the
//             exactness above and lets more proposals of a window win.
//   k_delta   one block per winner evaluates the vertex properties of the
//             four quad vertices before and after a virtual flip (the mesh is
//             not touched), including the repulsion with the post-flip
//             exclusion rings, and reduces them to the property change of
//             the flip (stencils in double-word arithmetic on the FP32 pipe)
//   k_metro   Metropolis with T = 1 in slot order (flips.cpp:142-160): one
//             block decides every slot whose float-filtered decision cannot
//             be changed by earlier acceptances and walks the rest, with the
//             robustly accepted ones, in order with the FP64 test of the
//             energy change (written without cancellation); when the filter
//             decides every slot, the state moves by one warp's reduction of
//             the accepted changes instead; losers are queued for the next
//             window
//   k_commit  accepted flips rewrite their six halfedges, two faces, five
//             edge rows and four ring rows (one block per flip); patches are
//             disjoint, so commits never touch the same entries
// Proposals come from a counter-based SplitMix64 stream of (seed, index), so
// a sweep is reproducible and matches the CPU port of this algorithm.  The
// seed lives in the sweep state in device memory, so the 32 launches of a
// group of eight windows are captured once as a CUDA graph and replayed.
// A flip is also refused when it would raise a valence above TM_MAXVAL.
#include <cooperative_groups.h>

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstring>
#include <vector>

#include "tm_energy.cuh"
#include "tm_internal.h"
#include "tm_math.cuh"
#include "tm_topo.cuh"
#include "tm_dw.cuh"

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
namespace {

constexpr int MAXB = 4096;  // largest window

__host__ __device__ __forceinline__ unsigned long long splitmix64(unsigned long long z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
__device__ __forceinline__ unsigned long long flip_key(unsigned long long seed, long long p, int stream) {
  return splitmix64(splitmix64(seed) ^ (unsigned long long)(2 * p + stream));
}
__device__ __forceinline__ int flip_edge_of(unsigned long long seed, long long p, int ne) {
  return (int)(((flip_key(seed, p, 0) >> 32) * (unsigned long long)ne) >> 32);
}
__device__ __forceinline__ double flip_u_of(unsigned long long seed, long long p) {
  return (double)(flip_key(seed, p, 1) >> 11) * 0x1.0p-53;
}

// Sweep state in device memory.  A window's size W and number wid are set
// by the window fill (k_claim_win, or k_fill) from the state the previous
// window left, so windows follow each other without the host; W = 0 once
// every proposal is decided.
struct FlipState {
  double props[8];
  unsigned long long seed;  // proposal stream of the sweep
  int nacc_win;             // accepted slots of the current window (listed in order)
  float sq[3];  // the filter's d0 of area, volume, curvature (filter_state)
  long long next_new;  // first proposal not yet in a window
  long long nn_next;   // next_new after the current window (committed by k_metro)
  long long nflips;
  int acc;
  int limit;
  int npend;
  int status;
  int W;
  int wid;
};

struct Quad {
  int va0, va1, vb0, vb1;
};
__device__ __forceinline__ Quad quad_of(const TopoW& t, int e) {
  Quad q;
  int a0 = 2 * e, b0 = 2 * e + 1;
  q.va0 = t.to[a0];
  q.va1 = t.to[t.next[a0]];
  q.vb0 = t.to[b0];
  q.vb1 = t.to[t.next[b0]];
  return q;
}


__device__ bool flip_ok(const TopoW& t, int e) {
  if (t.face[2 * e] < 0 || t.face[2 * e + 1] < 0) return false;
  int c = t.to[t.next[2 * e]], d = t.to[t.next[2 * e + 1]];
  if (c == d) return false;
  int dc = t.val[c];
  for (int m = 0; m < dc; ++m)
    if (t.nbr[(size_t)m * t.nv + c] == d) return false;
  if (t.val[c] >= TM_MAXVAL || t.val[d] >= TM_MAXVAL) return false;
  return true;
}

// ---- vertex properties from an explicit ring ------------------------------
struct Ring {
  int n;
  int r[TM_MAXVAL + 1];
  bool f[TM_MAXVAL + 1];  // face (v, r_m, r_{m-1}) exists
};

__device__ void load_ring(const TopoW& t, int v, Ring& R) {
  R.n = t.val[v];
  for (int m = 0; m < R.n; ++m) {
    int4 s = t.slot[(size_t)m * t.nv + v];
    R.r[m] = s.x;
    R.f[m] = s.y != -1;
  }
}
__device__ void ring_remove(Ring& R, int x) {
  int p = 0;
  while (p < R.n && R.r[p] != x) ++p;
  for (int m = p; m + 1 < R.n; ++m) {
    R.r[m] = R.r[m + 1];
    R.f[m] = R.f[m + 1];
  }
  if (p < R.n) R.n -= 1;
}
// insert y right before x
__device__ void ring_insert_before(Ring& R, int x, int y) {
  int p = 0;
  while (p < R.n && R.r[p] != x) ++p;
  for (int m = R.n; m > p; --m) {
    R.r[m] = R.r[m - 1];
    R.f[m] = R.f[m - 1];
  }
  R.r[p] = y;
  R.f[p] = true;
  R.n += 1;
}

// rings after the virtual flip of the quad
__device__ void ring_after(const TopoW& t, const Quad& q, int v, Ring& R) {
  load_ring(t, v, R);
  if (v == q.va0) ring_remove(R, q.vb0);
  else if (v == q.vb0) ring_remove(R, q.va0);
  else if (v == q.va1) ring_insert_before(R, q.vb0, q.vb1);
  else if (v == q.vb1) ring_insert_before(R, q.va0, q.va1);
}

struct OverlayExcl {  // exclusion on the topology after the virtual flip
  const TopoW& t;
  const Quad& q;
  int excl;
  __device__ bool adjacent_after(int a, int b) const {
    if ((a == q.va0 && b == q.vb0) || (a == q.vb0 && b == q.va0)) return false;
    if ((a == q.va1 && b == q.vb1) || (a == q.vb1 && b == q.va1)) return true;
    int d = t.val[a];
    for (int m = 0; m < d; ++m)
      if (t.nbr[(size_t)m * t.nv + a] == b) return true;
    return false;
  }
  __device__ bool operator()(int v, int j) const {
    Ring R;
    ring_after(t, q, v, R);
    for (int m = 0; m < R.n; ++m) {
      int w = R.r[m];
      if (w == j) return true;
      if (excl > 1 && adjacent_after(w, j)) return true;
    }
    return false;
  }
};
struct TableExclW {
  const TopoW& t;
  int excl;
  __device__ bool operator()(int v, int j) const {
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
};


// ---- window kernels --------------------------------------------------------
// The Metropolis test's energy change E(props - dp) - E(props) for the
// penalty energy of src/kernel.h:110-122, with the reciprocals of the
// reference properties (rounded once on the host) in place of divisions,
// written without cancellation: the quadratic penalties as k t (t - 2 d0)
// with d0 = props/ref - 1 of the current state and t = dp/ref, the linear
// terms as -k dp.  Equal to the difference of the two energies in exact
// arithmetic; in FP64 its rounding is relative to the change's own terms,
// while the difference of two totals carries the totals' rounding (an
// unrelaxed membrane's energy reaches 1e12, whose last bit is 1e-4).  The
// CPU port of the sweep evaluates the same expression.
struct FlipE {
  double irA, irV, irC, ka, kv, kc, kt, kr, kb;
};
__device__ __forceinline__ double flip_delta(const FlipE& f, const double* p, const double* dp) {
  const double da = p[0] * f.irA - 1.0, dv = p[1] * f.irV - 1.0, dc = p[2] * f.irC - 1.0;
  const double ta = dp[0] * f.irA, tv = dp[1] * f.irV, tc = dp[2] * f.irC;
  double de = 0.0;
  de += f.ka * ta * (ta - 2.0 * da);
  de += f.kv * tv * (tv - 2.0 * dv);
  de += f.kc * tc * (tc - 2.0 * dc);
  de -= f.kt * dp[4];
  de -= f.kr * dp[5];
  de -= f.kb * dp[3];
  return de;
}

// Float filter of the same test (k_metro), from float copies of dp and of
// the state's d0
struct FlipEF {
  float irA, irV, irC, ka, kv, kc, kt, kr, kb;
};
// per-state constants of the filter: d0 of area, volume and curvature
__device__ __forceinline__ void filter_state(const FlipE& f, const double* p, float* q) {
  q[0] = (float)(p[0] * f.irA - 1.0);
  q[1] = (float)(p[1] * f.irV - 1.0);
  q[2] = (float)(p[2] * f.irC - 1.0);
}

__global__ void k_flip_init(FlipE fe, const Globals* g, long long nflips, unsigned long long seed, FlipState* st) {
  if (threadIdx.x || blockIdx.x) return;
  st->seed = seed;
  for (int k = 0; k < 6; ++k) st->props[k] = g->props[k];
  filter_state(fe, st->props, st->sq);
  st->next_new = 0;
  st->nn_next = 0;
  st->nflips = nflips;
  st->W = 0;
  st->wid = 0;
  st->acc = 0;
  st->npend = 0;
  st->status = 0;
}

__global__ void k_fill(int B, const long long* pend, FlipState* st, long long* win, int* limit) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  const int np = st->npend;
  const long long nn = st->next_new;
  const int W = (int)min((long long)B, (long long)np + (st->nflips - nn));
  if (s == 0) {
    *limit = W;
    st->W = W;
    st->wid += W > 0 ? 1 : 0;
    st->nn_next = nn + (W - np);
  }
  if (s < W) win[s] = s < np ? pend[s] : nn + (s - np);
}

// Patch ownership without a release pass: owner[x] (per vertex) holds the
// largest tag (window << 12) | (4095 - slot) claimed so far in this sweep,
// so within a window the lowest slot wins and tags of earlier windows lose.
// Four threads per slot, one per quad vertex: each claims its vertex and the
// vertex's ring neighbours, then tests that it owns its vertex.
__device__ __forceinline__ int owner_tag(int wid, int s) { return (wid << 12) | (4095 - s); }
__device__ __forceinline__ int quad_vertex(const Quad& q, int k) {
  return k == 0 ? q.va0 : (k == 1 ? q.va1 : (k == 2 ? q.vb0 : q.vb1));
}
__device__ __forceinline__ void claim_closure(const TopoW& t, int v, int tag, int* owner) {
  atomicMax(&owner[v], tag);
  const int d = t.val[v];
  for (int m = 0; m < d; ++m) atomicMax(&owner[t.nbr[(size_t)m * t.nv + v]], tag);
}

__global__ void k_claim(TopoW t, const FlipState* st, const long long* win, int* owner) {
  const unsigned long long seed = st->seed;
  int g = blockIdx.x * blockDim.x + threadIdx.x;
  int s = g >> 2, k = g & 3;
  const int W = st->W, wid = st->wid;
  if (s >= W) return;
  Quad q = quad_of(t, flip_edge_of(seed, win[s], t.ne));
  claim_closure(t, quad_vertex(q, k), owner_tag(wid, s), owner);
}

__global__ void k_winner(TopoW t, const FlipState* st, int mode, const long long* win, const int* owner,
                         unsigned char* winner, int* limit) {
  const unsigned long long seed = st->seed;
  int g = blockIdx.x * blockDim.x + threadIdx.x;
  int s = g >> 2, k = g & 3;
  const int W = st->W, wid = st->wid;
  if (s >= W) return;
  Quad q = quad_of(t, flip_edge_of(seed, win[s], t.ne));
  const int tag = owner_tag(wid, s);
  bool ok = owner[quad_vertex(q, k)] == tag;
  const unsigned gmask = 0xfu << (threadIdx.x & 28);  // the four threads of this slot
  ok = __all_sync(gmask, ok);
  if (k == 0) {
    winner[s] = ok ? 1 : 0;
    if (!ok && mode == 0) atomicMin(limit, s);
  }
}

// k_fill, k_claim and k_winner in one cooperative launch: every thread takes
// its slot's proposal from the previous window's state (deferred proposals
// first, then new ones, as k_fill), the claims, a grid-wide barrier, then
// the window's state is advanced and the ownership test runs on the same
// vertices (read past L1)
__global__ void __launch_bounds__(64) k_claim_win(TopoW t, FlipState* st, int B, int mode, const long long* pend,
                                                 long long* win, int* owner, unsigned char* winner, int* limit) {
  const unsigned long long seed = st->seed;
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  const int s = g >> 2, k = g & 3;
  const int np = st->npend;
  const long long nn = st->next_new;
  const int W = (int)min((long long)B, (long long)np + (st->nflips - nn));
  const int wid = st->wid + (W > 0 ? 1 : 0);
  const bool act = s < W;  // the four threads of a slot agree
  int v = 0, tag = 0;
  if (g == 0) *limit = W;
  if (act) {
    const long long p = s < np ? pend[s] : nn + (s - np);
    if (k == 0) win[s] = p;
    const Quad q = quad_of(t, flip_edge_of(seed, p, t.ne));
    tag = owner_tag(wid, s);
    v = quad_vertex(q, k);
    claim_closure(t, v, tag, owner);
  }
  cooperative_groups::this_grid().sync();  // every thread has read the state and claimed
  if (g == 0) {
    st->W = W;
    st->wid = wid;
    st->nn_next = nn + (W - np);
  }
  if (act) {
    bool ok = __ldcg(&owner[v]) == tag;
    const unsigned gmask = 0xfu << (threadIdx.x & 28);
    ok = __all_sync(gmask, ok);
    if (k == 0) {
      winner[s] = ok ? 1 : 0;
      if (!ok && mode == 0) atomicMin(limit, s);
    }
  }
}

// repulsion value of vertex v at xv (mesh_repulsion.h:28-79): the near rows
// when usable (exclusion tested with the given rules), else the candidate
// row / cell walk; both visit in the reference's order
template <class X>
__device__ double repulsion_of(int v, d3 xv, const double* P, const EP& ep, const NLView& nl, const X& excl) {
  double pot = 0.0;
  const double lc1 = ep.rlc1;
  const int rr = ep.rr;
  auto add = [&](int, double l, d3) { pot += exp(l / (l - lc1)) / ipow(l, rr); };
  bool done = false;
  if (nl.kind == 0 && nl.nent && nl.nflag[0] == 0 && nl.nflag[1] == 0) {
    PairTest pt = make_pair_test(nl, v, lc1, ep.rT);
    int co[3];
    in_build_cell(nl, v, xv, co);
    done = visit_near(pt, nl, P, v, xv, 2, co, excl, add);
  }
  if (!done) for_each_neighbour_x(nl, P, v, xv, lc1, ep.rT, excl, add);
  return pot;
}

// Repulsion value of vertex v at xv from its near row, computed by the 8
// lanes w8 of one variant (gmask: those lanes): each lane tests every 8th
// entry (distance, build cell, exclusion on the given rules) and the
// accepted pairs go to shared memory (key: the reference's visiting order,
// as in visit_near); each lane evaluates the pair of its rank and lane 0
// adds the values in rank order: the same sum, bit for bit, as the
// sequential walk of visit_near.  Returns false (on every lane) when the
// rows are stale or hold more than NEAR_HITS accepted pairs.
template <class X>
__device__ bool repulsion_near8(int v, d3 xv, const double* P, const EP& ep, const NLView& nl, const X& excl,
                                int w8, unsigned gmask, long long* skey, double* sval, double* sterm,
                                double* pot) {
  if (!(nl.kind == 0 && nl.nent && nl.nflag[0] == 0 && nl.nflag[1] == 0)) return false;
  const double lc1 = ep.rlc1;
  PairTest pt = make_pair_test(nl, v, lc1, ep.rT);
  int co[3];
  in_build_cell(nl, v, xv, co);
  const int* row = nl.nent + (size_t)v * TM_NEAR_CAP;
  const int n = nl.ncnt[v];
  const unsigned below = (1u << (threadIdx.x & 31)) - 1u;
  int total = 0;
  for (int q0 = 0; q0 < n; q0 += 8) {
    const int q = q0 + w8;
    bool acc = false;
    long long key = 0;
    double sq = 0.0;
    if (q < n) {
      int j = row[q] & 0x7fffffff;
      d3 pj;
      if (pair_within(pt, nl, P, xv, j, &pj, &sq)) {
        int ox = nl.bcoord[3 * j] - co[0], oy = nl.bcoord[3 * j + 1] - co[1], oz = nl.bcoord[3 * j + 2] - co[2];
        acc = ox >= -1 && ox <= 1 && oy >= -1 && oy <= 1 && oz >= -1 && oz <= 1 && !(nl.excl > 0 && excl(v, j));
        key = ((long long)((ox + 1) * 9 + (oy + 1) * 3 + (oz + 1)) << 32) | (long long)j;
      }
    }
    const unsigned b = __ballot_sync(gmask, acc);
    const int pos = total + __popc(b & below);
    if (acc && pos < NEAR_HITS) {
      skey[pos] = key;
      sval[pos] = sq;
    }
    total += __popc(b);
  }
  if (total > NEAR_HITS) return false;
  __syncwarp(gmask);
  if (w8 < total) {
    const long long k = skey[w8];
    int rank = 0;
    for (int h = 0; h < total; ++h) rank += skey[h] < k ? 1 : 0;
    const double l = __dsqrt_rn(sval[w8]);
    sterm[rank] = exp(l / (l - lc1)) / ipow(l, ep.rr);
  }
  __syncwarp(gmask);
  if (w8 == 0) {
    double acc = 0.0;
    for (int h = 0; h < total; ++h) acc += sterm[h];
    *pot = acc;
  }
  return true;
}

// The sign of the dihedral angle of edge (v, j) between the faces (v, j, k)
// and (v, l, j) as an FP64 evaluation of the stencil decides it (the test of
// the CPU port: the sign of (N0 x N1) . e, from the same operations).  A
// fold (angle near +-pi) is where the angle's value jumps from pi to -pi,
// and there the sign must be the FP64 one.
__device__ __noinline__ bool fold_sign_fp64(const double* P, int v, int j, int k, int l) {
  const d3 xv = ld3(P, v), xj = ld3(P, j), xk = ld3(P, k), xl = ld3(P, l);
  const d3 ev = xj - xv;
  const double il = rsqrt(dot(ev, ev));
  const d3 N0 = cross(ev, xk - xv);
  const double r0 = rsqrt(dot(N0, N0));
  const d3 N1 = cross(xl - xv, ev);
  const double r1 = rsqrt(dot(N1, N1));
  const double inv = r0 * r1;
  const double sd = dot(cross(N0, N1), ev) * (inv * il);
  return sd >= 0.0;
}

// Per ring position m of vertex v (face (v, r_m, r_m-1), edge (v, r_m)):
// half edge length x dihedral angle, face area, face volume, bond, in
// double-words on the FP32 pipe with positions relative to x_v (the face
// normal N0 = (x_j - x_v) x (x_k - x_v), the volume term x_v . N0 / 6 =
// (x_j x x_k) . x_v / 6, the dihedral angle by angle_dw); summed over the
// ring by a butterfly over the variant's 8 lanes (every lane ends with the
// same sums) and written by lane 0 as the vertex's area, volume, curvature,
// bending and tether values o[0..4].  With n <= 8 every lane holds one
// position and the normal of the next face comes from the next lane (the
// same cross product: (x_r(m+1) - x_v) x (x_r(m) - x_v)); lanes past the
// ring and positions without a face compute nothing, and the next face's
// normal is used only where that face exists, so its lane has computed it.
// The results differ from FP64 ones by rounding (about 1e-14 of the terms);
// at a fold (cosine < 0, |sine| < 1e-6: the double-word sine is good to
// about 1e-14, so its sign could differ from the FP64 one only far inside
// that band) the sign comes from fold_sign_fp64.
__device__ void ring_terms_dw(const PosDW& X, const double* P, const EP& ep, const EPD& epd,
                              const float4* __restrict__ sctf, int v, const int* sr, const unsigned char* sf, int n,
                              int w8, int gbase, unsigned gmask, float2* o) {
  const df3 xw = X.at(v);
  const df zero = df_make(0.0f);
  const df3 zero3 = {zero, zero, zero};
  df sc = zero, sa = zero, sv = zero, stt = zero;
  // m: ring position of the edge (v, r_m) between faces (v, r_m, r_m-1) and
  // (v, r_m+1, r_m)
  auto terms = [&](int m, int mn, const df3& ev, const df& el, const df& il, const df& n0s, const df& r0,
                   const df3& N0, bool have1, const df3& N1, const df& n1s, const df& r1) {
    df th = zero;
    if (have1 && n0s.hi != 0.0f && n1s.hi != 0.0f) {
      const df inv = mul_s(r0, r1);
      const df sd = mul_s(dot3(cross3(N0, N1), ev), mul_s(inv, il));
      const df c = mul_s(dot3(N0, N1), inv);
      if (c.hi < 0.0f && fabsf(sd.hi) < 1e-6f) {
        const df a = angle_dw(dabs(sd), c, sctf);
        th = fold_sign_fp64(P, v, sr[m], sr[m == 0 ? n - 1 : m - 1], sr[mn]) ? a : neg(a);
      } else {
        th = angle_dw(sd, c, sctf);
      }
    }
    const df fa = half(mul_s(n0s, r0));
    df tt = zero;
    if (ep.btype == 0) {
      if (ep.r >= 1) {
        if (df_less(epd.lc0, el))
          tt = mul_s(epd.br1, ipow_dw(sub_s(el, epd.lc0), ep.r));
        else if (df_less(el, epd.lc1))
          tt = mul_s(df_exp_nonpos(mul_s(el, rcp_dw(sub_s(el, epd.lc1)))), ipow_dw(il, ep.r));
      } else {  // non-positive exponents: FP64
        const double eld = df_to(el), ild = df_to(il);
        double t64 = 0.0;
        if (eld > ep.lc0) t64 = ep.br1 * ipow(eld - ep.lc0, ep.r);
        else if (eld < ep.lc1) t64 = exp(eld * (1.0 / (eld - ep.lc1))) * ipow(ild, ep.r);
        tt = df_from(t64);
      }
    } else {
      const df qa = sub_s(mul_s(fa, epd.inv_a0), df_make(1.0f));
      tt = mul_s(qa, qa);
    }
    sc = add_s(sc, half(mul_s(el, th)));
    sa = add_s(sa, fa);
    sv = add_s(sv, mul_s(dot3(xw, N0), sixth()));
    stt = add_s(stt, tt);
  };
  if (n <= 8) {
    const int m = w8 < n ? w8 : 0;
    const int mn = m + 1 == n ? 0 : m + 1;
    const bool act = w8 < n && sf[m];
    df3 ev = zero3, N0 = zero3;
    df il = zero, el = zero, n0s = zero, r0 = zero;
    if (act) {
      const df3 xj = X.at(sr[m]), xk = X.at(sr[m == 0 ? n - 1 : m - 1]);
      ev = sub3(xj, xw);
      const df l2 = dot3(ev, ev);
      il = rsqrt_dw(l2);
      el = mul_s(l2, il);
      N0 = cross3(ev, sub3(xk, xw));
      n0s = dot3(N0, N0);
      r0 = rsqrt_dw(n0s);
    }
    const int src = gbase + mn;
    auto shf = [&](const df& x) { return df{__shfl_sync(gmask, x.hi, src), __shfl_sync(gmask, x.lo, src)}; };
    const df3 N1 = {shf(N0.x), shf(N0.y), shf(N0.z)};
    const df n1s = shf(n0s), r1 = shf(r0);
    if (act) terms(m, mn, ev, el, il, n0s, r0, N0, sf[mn] != 0, N1, n1s, r1);
  } else {
    for (int m = w8; m < n; m += 8) {
      if (!sf[m]) continue;
      const int mn = m + 1 == n ? 0 : m + 1;
      const df3 xj = X.at(sr[m]), xk = X.at(sr[m == 0 ? n - 1 : m - 1]);
      const df3 ev = sub3(xj, xw);
      const df l2 = dot3(ev, ev);
      const df il = rsqrt_dw(l2), el = mul_s(l2, il);
      const df3 N0 = cross3(ev, sub3(xk, xw));
      const df n0s = dot3(N0, N0), r0 = rsqrt_dw(n0s);
      df3 N1 = zero3;
      df n1s = zero, r1 = zero;
      const bool have1 = sf[mn] != 0;
      if (have1) {
        N1 = cross3(sub3(X.at(sr[mn]), xw), ev);
        n1s = dot3(N1, N1);
        r1 = rsqrt_dw(n1s);
      }
      terms(m, mn, ev, el, il, n0s, r0, N0, have1, N1, n1s, r1);
    }
  }
#pragma unroll
  for (int q = 4; q > 0; q >>= 1) {
    auto bfly = [&](df& x) {
      const df y = {__shfl_xor_sync(gmask, x.hi, q), __shfl_xor_sync(gmask, x.lo, q)};
      x = add_s(x, y);
    };
    bfly(sc);
    bfly(sa);
    bfly(sv);
    bfly(stt);
  }
  if (w8 == 0) {
    const df A = mul_s(sa, third()), C = half(sc);
    const df Vv = mul_s(sv, third()), B = ldexp2(mul_s(mul_s(C, C), rcp_dw(A)), 2.0f);
    const df T = mul_s(stt, epd.inv_tdiv);
    o[0] = make_float2(A.hi, A.lo);
    o[1] = make_float2(Vv.hi, Vv.lo);
    o[2] = make_float2(C.hi, C.lo);
    o[3] = make_float2(B.hi, B.lo);
    o[4] = make_float2(T.hi, T.lo);
  }
}

// Property changes of a window's proposals (k_delta): one block of 64
// threads per slot of the window (winners with a valid flip do work): 8
// variants (quad vertex sub & 3, before the flip for sub < 4, after it
// otherwise) x 8 workers.  The ring of each variant goes to shared memory,
// the workers compute the per-position terms of vertex_properties
// (src/mesh_properties.cpp:12-49) in double-word arithmetic on the FP32 pipe
// (GB300's FP64 pipe is a small fraction of the FP32 rate) and sum them by a
// butterfly, and the repulsion comes from the variant's near row in FP64.
// The change is written in FP64 (the ordered walk's values) and as floats
// (the filter's).  It differs from an FP64 evaluation of the same stencils
// by rounding, about 1e-14 of the terms, as the FP64 evaluation differs from
// the CPU port's by its summation orders: a Metropolis decision could
// differ only where E(trial) - E lies within that rounding of -log(u).
struct DeltaShared {
  float2 part[64];  // per variant, as double-words: area, volume, curvature, bending, tether, repulsion
  int sr[8][TM_MAXVAL + 1];
  unsigned char sf[8][TM_MAXVAL + 1];
  int sn[8];
  long long rkey[8][NEAR_HITS];
  double rval[8][NEAR_HITS], rterm[8][NEAR_HITS];
};

__device__ __forceinline__ void delta_slot(int s, DeltaShared& sh, const TopoW& t, const FlipState* st,
                                           const long long* win, const double* P, const EP& ep, const EPD& epd,
                                           const PosDW& X, const NLView& nl, double* dpn, float* dpf,
                                           const float4* __restrict__ sctf) {
  const unsigned long long seed = st->seed;
  const int sub = threadIdx.x >> 3, w8 = threadIdx.x & 7;
  const int gbase = threadIdx.x & 24;            // warp lane of the variant's lane 0
  const unsigned gmask = 0xffu << gbase;         // the variant's 8 lanes
  const int e = flip_edge_of(seed, win[s], t.ne);
  if (!flip_ok(t, e)) {
    if (threadIdx.x == 0) dpf[8 * (size_t)s + 7] = 0.0f;
    return;
  }
  const Quad q = quad_of(t, e);
  const int v = quad_vertex(q, sub & 3);
  // ring of the variant, loaded by its 8 lanes (slot m by lane m mod 8);
  // after the virtual flip (ring_after): va0 / vb0 lose vb0 / va0, va1 / vb1
  // gain vb1 / va1 right before vb0 / va0
  {
    const int n0 = t.val[v];
    int x = -1, y = -1;
    if (sub >= 4) {
      if (v == q.va0) x = q.vb0;
      else if (v == q.vb0) x = q.va0;
      else if (v == q.va1) x = q.vb0, y = q.vb1;
      else x = q.va0, y = q.va1;
    }
    int rr[4];
    bool ff[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const int m = w8 + 8 * i;
      rr[i] = -1;
      ff[i] = false;
      if (m < n0) {
        int4 sl = t.slot[(size_t)m * t.nv + v];
        rr[i] = sl.x;
        ff[i] = sl.y != -1;
      }
    }
    int p = n0;  // position of x (n0: absent)
    if (x >= 0) {
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        const unsigned b = __ballot_sync(gmask, rr[i] == x && w8 + 8 * i < n0) >> gbase;
        if (b && p == n0) p = 8 * i + __ffs(b) - 1;
      }
    }
    const bool ins = y >= 0;
    const int n = x < 0 ? n0 : (ins ? n0 + 1 : (p < n0 ? n0 - 1 : n0));
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const int m = w8 + 8 * i;
      if (m >= n0) continue;
      int dst = m;
      if (x >= 0 && m >= p) {
        if (ins) dst = m + 1;
        else if (m == p) continue;
        else dst = m - 1;
      }
      sh.sr[sub][dst] = rr[i];
      sh.sf[sub][dst] = ff[i] ? 1 : 0;
    }
    if (w8 == 0) {
      if (ins) {
        sh.sr[sub][p] = y;
        sh.sf[sub][p] = 1;
      }
      sh.sn[sub] = n;
    }
  }
  __syncthreads();
  const int n = sh.sn[sub];
  float2* o = sh.part + 8 * sub;
  ring_terms_dw(X, P, ep, epd, sctf, v, sh.sr[sub], sh.sf[sub], n, w8, gbase, gmask, o);
  // repulsion: the near row shared by the variant's 8 lanes, else one lane
  // walks the cell list
  {
    const d3 xv = ld3(P, v);
    double pot = 0.0;
    bool near;
    if (sub < 4) {
      TableExclW x{t, nl.excl};
      near = repulsion_near8(v, xv, P, ep, nl, x, w8, gmask, sh.rkey[sub], sh.rval[sub], sh.rterm[sub], &pot);
      if (!near && w8 == 0) pot = repulsion_of(v, xv, P, ep, nl, x);
    } else {
      OverlayExcl x{t, q, nl.excl};
      near = repulsion_near8(v, xv, P, ep, nl, x, w8, gmask, sh.rkey[sub], sh.rval[sub], sh.rterm[sub], &pot);
      if (!near && w8 == 0) pot = repulsion_of(v, xv, P, ep, nl, x);
    }
    if (w8 == 0) {
      float ph, pl;
      split_bits(pot, &ph, &pl);
      o[5] = make_float2(ph, pl);
    }
  }
  __syncthreads();
  // the property change of the flip (before - after, in the summation orders
  // of edge_vertex_properties before (va0, va1, vb0, vb1) and after the flip
  // (va1, vb0, vb1, va0)): lane k of warp 0 takes property k
  if (threadIdx.x < 32) {
    const float2* op = sh.part;
    if (threadIdx.x < 6) {
      const int k = threadIdx.x;
      auto at = [&](int q) { return df{op[q].x, op[q].y}; };
      const df before = add_s(add_s(add_s(at(k), at(8 + k)), at(16 + k)), at(24 + k));
      const df after = add_s(add_s(add_s(at(40 + k), at(48 + k)), at(56 + k)), at(32 + k));
      const df dk = sub_s(before, after);
      dpn[8 * (size_t)s + k] = df_to(dk);
      dpf[8 * (size_t)s + k] = __fadd_rn(dk.hi, dk.lo);
    }
    if (threadIdx.x == 0) {
      // -log(u) in float for the filter (NaN below float range: the FP64
      // test decides; k_metro computes -log(u) in FP64 for the slots it
      // walks) and the eligibility flag
      const float uf = (float)flip_u_of(seed, win[s]);
      dpf[8 * (size_t)s + 6] = uf > 1e-30f ? -logf(uf) : __int_as_float(0x7fc00000);
      dpf[8 * (size_t)s + 7] = 1.0f;
    }
  }
}

__global__ void __launch_bounds__(64, 12) k_delta(TopoW t, const FlipState* st, const long long* win,
                                              const unsigned char* winner, const int* limit, const double* P, EP ep,
                                              EPD epd, PosDW X, NLView nl, double* dpn, float* dpf,
                                              const float4* __restrict__ sctf) {
  __shared__ DeltaShared sh;
  const int s = blockIdx.x;
  if (s >= st->W) return;
  if (s >= *limit || !winner[s]) {
    if (threadIdx.x == 0) dpf[8 * (size_t)s + 7] = 0.0f;
    return;
  }
  delta_slot(s, sh, t, st, win, P, ep, epd, X, nl, dpn, dpf, sctf);
}

// Metropolis with T = 1 in slot order (flips.cpp:142-160): slot s is tried on
// the state left by the accepted slots before it, trial = props - dp, and is
// accepted when E(trial) - E <= -log(u).  The state moves only by the dp of
// accepted slots, and the energy change of slot s depends on the state only
// through the area, volume and curvature penalties, linearly in the state's
// normalised deviations d0: D = k t (t - 2 d0) + ... .  So the first phase
// bounds, for every slot at once, how far any set of earlier acceptances can
// move its D (2 k |t| times the sum of |dp|/ref over the window's eligible
// slots) and decides it by the float filter against the window's starting
// state when the decision survives that shift: robustly accepted or
// rejected.  The second phase walks, in slot order, only the robustly
// accepted slots (state update) and the undecided ones (the FP64 test on the
// current state, then the update when accepted): the same decisions and the
// same FP64 state updates as a walk over every slot.  Then the deferred
// proposals are compacted in order for the next window.
constexpr int MB = 1024, MS = MAXB / MB;  // threads, slots per thread (consecutive)

// exclusive scan of two counters over the block (1,024 threads); returns the
// totals
__device__ __forceinline__ int2 block_scan2(int a, int b, int* ea, int* eb, int2* wsum) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  int ia = a, ib = b;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int ta = __shfl_up_sync(0xffffffffu, ia, o), tb = __shfl_up_sync(0xffffffffu, ib, o);
    if (lane >= o) {
      ia += ta;
      ib += tb;
    }
  }
  if (lane == 31) wsum[w] = make_int2(ia, ib);
  __syncthreads();
  if (w == 0) {
    int2 v = wsum[lane];
    int xa = v.x, xb = v.y;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      int ta = __shfl_up_sync(0xffffffffu, xa, o), tb = __shfl_up_sync(0xffffffffu, xb, o);
      if (lane >= o) {
        xa += ta;
        xb += tb;
      }
    }
    wsum[lane] = make_int2(xa, xb);  // inclusive over warps
  }
  __syncthreads();
  const int2 before = w ? wsum[w - 1] : make_int2(0, 0);
  *ea = before.x + ia - a;
  *eb = before.y + ib - b;
  return wsum[31];
}

constexpr int PREF = 256;  // walked slots whose data is prefetched into shared memory
__global__ void __launch_bounds__(MB) k_metro(const long long* win, const unsigned char* winner, const double* dpn,
                                             const float* dpf, FlipE fe, FlipEF fg, FlipState* st, const int* limit,
                                             int* accl, long long* pend) {
  constexpr unsigned char SKIP = 0, REJECT = 1, ACCEPT = 2, OPEN = 3;
  __shared__ int lst[MAXB];
  __shared__ double sdp[PREF][7];  // dp of the walked slots, and -log(u) of the open ones
  __shared__ int2 wsum[32];
  __shared__ float sb[3][32];
  const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
  const int W = st->W;
  const unsigned long long seed = st->seed;
  float q[3];
  for (int k = 0; k < 3; ++k) q[k] = st->sq[k];
  // this thread's slots' float records (two 16-byte loads each; the
  // eligibility flag 0 for slots past the window)
  float4 fa[MS], fb[MS];
  for (int k = 0; k < MS; ++k) {
    const int s = tid * MS + k;
    fa[k] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    fb[k] = fa[k];
    if (s < W) {
      const float4* r = reinterpret_cast<const float4*>(dpf + 8 * (size_t)s);
      fa[k] = r[0];
      fb[k] = r[1];
    }
  }
  // window-wide bound of the state's movement: sum of |dp|/ref of the
  // eligible slots (area, volume, curvature)
  float ba = 0.0f, bv = 0.0f, bc = 0.0f;
  for (int k = 0; k < MS; ++k) {
    if (fb[k].w == 0.0f) continue;
    ba += fabsf(fa[k].x * fg.irA);
    bv += fabsf(fa[k].y * fg.irV);
    bc += fabsf(fa[k].z * fg.irC);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    ba += __shfl_xor_sync(0xffffffffu, ba, o);
    bv += __shfl_xor_sync(0xffffffffu, bv, o);
    bc += __shfl_xor_sync(0xffffffffu, bc, o);
  }
  if (lane == 0) {
    sb[0][w] = ba;
    sb[1][w] = bv;
    sb[2][w] = bc;
  }
  __syncthreads();  // also: every thread has read W before thread 0 may write the state
  ba = bv = bc = 0.0f;
  for (int k = 0; k < 32; ++k) {  // same order in every thread
    ba += sb[0][k];
    bv += sb[1][k];
    bc += sb[2][k];
  }
  ba *= 1.001f;  // float rounding of the sums
  bv *= 1.001f;
  bc *= 1.001f;
  // phase 1: classify this thread's slots
  unsigned char cls[MS];
  int nopen = 0;
  for (int k = 0; k < MS; ++k) {
    cls[k] = SKIP;
    if (fb[k].w == 0.0f) continue;
    const float f8[8] = {fa[k].x, fa[k].y, fa[k].z, fa[k].w, fb[k].x, fb[k].y, fb[k].z, fb[k].w};
    const float ta = f8[0] * fg.irA, tv = f8[1] * fg.irV, tc = f8[2] * fg.irC;
    const float xa = fg.ka * ta * (ta - 2.0f * q[0]);
    const float xv = fg.kv * tv * (tv - 2.0f * q[1]);
    const float xc = fg.kc * tc * (tc - 2.0f * q[2]);
    const float xl = fg.kt * f8[4] + fg.kr * f8[5] + fg.kb * f8[3];
    const float S = fabsf(fg.ka * ta) * (fabsf(ta) + 2.0f * fabsf(q[0])) +
                    fabsf(fg.kv * tv) * (fabsf(tv) + 2.0f * fabsf(q[1])) +
                    fabsf(fg.kc * tc) * (fabsf(tc) + 2.0f * fabsf(q[2])) + fabsf(fg.kt * f8[4]) +
                    fabsf(fg.kr * f8[5]) + fabsf(fg.kb * f8[3]);
    const float shift = 2.0f * (fabsf(fg.ka * ta) * ba + fabsf(fg.kv * tv) * bv + fabsf(fg.kc * tc) * bc);
    const float m = 1e-4f * S + 1e-6f * fabsf(f8[6]) + 2e-7f + 1.01f * shift;
    const float d = ((xa + xv) + xc - xl) - f8[6];
    cls[k] = d < -m ? ACCEPT : (d > m ? REJECT : OPEN);  // NaN or overflow: OPEN
    if (cls[k] >= ACCEPT) ++nopen;
  }
  // slots to walk (robustly accepted or open) and deferred proposals, both
  // in slot order
  const int lim = *limit;
  int ndef = 0;
  for (int k = 0; k < MS; ++k) {
    const int s = tid * MS + k;
    if (s < W && (s >= lim || !winner[s])) ++ndef;
  }
  int ew = 0, ed = 0;
  const int2 tot = block_scan2(nopen, ndef, &ew, &ed, wsum);
  bool mine_open = false;
  for (int k = 0; k < MS; ++k) {
    const int s = tid * MS + k;
    if (s >= W) break;
    if (cls[k] >= ACCEPT) lst[ew++] = cls[k] == ACCEPT ? s : -1 - s;
    if (s >= lim || !winner[s]) pend[ed++] = win[s];
    mine_open = mine_open || cls[k] == OPEN;
  }
  if (!__syncthreads_or(mine_open)) {
    // every listed slot is a robust acceptance (the common case: the float
    // filter leaves a slot undecided only within about 1e-4 of its terms of
    // the threshold): the state moves by the sum of their changes, taken by
    // a fixed-order warp reduction instead of one thread's chain of FP64
    // subtractions (the FP64 pipe's latency makes that chain the window's
    // longest wait); one warp, since a window accepts tens of flips and
    // FP64 work of more warps would only queue on this SM's FP64 pipe.  The
    // state differs from the ordered walk's by rounding (1e-16 relative),
    // which an FP64 test of a later window could feel only for
    // |E(trial) - E + log u| of that order.
    if (w == 0) {
      double a[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
      for (int i = lane; i < tot.x; i += 32) {
        const int c = lst[i];
        for (int k = 0; k < 6; ++k) a[k] += dpn[8 * (size_t)c + k];
        accl[i] = c;
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1)
        for (int k = 0; k < 6; ++k) a[k] += __shfl_xor_sync(0xffffffffu, a[k], o);
      if (lane == 0) {
        double sP[6];
        for (int k = 0; k < 6; ++k) sP[k] = st->props[k] - a[k];
        if (tot.x > 0) {
          for (int k = 0; k < 6; ++k) st->props[k] = sP[k];
          filter_state(fe, sP, st->sq);
        }
        st->nacc_win = tot.x;
        st->acc += tot.x;
        st->npend = tot.y;
        st->next_new = st->nn_next;
      }
    }
    return;
  }
  // the walk's data (dp, and -log(u) in FP64 for the open slots) fetched and
  // computed in parallel
  if (tid < PREF && tid < tot.x) {
    const int c = lst[tid];
    const int s = c >= 0 ? c : -1 - c;
    for (int k = 0; k < 6; ++k) sdp[tid][k] = dpn[8 * (size_t)s + k];
    sdp[tid][6] = c >= 0 ? 0.0 : -log(flip_u_of(seed, win[s]));
  }
  __syncthreads();
  // phase 2: one thread walks the listed slots in order on the FP64 state:
  // the robustly accepted ones move it, the undecided ones are tested first
  if (tid == 0) {
    double sP[6];
    for (int k = 0; k < 6; ++k) sP[k] = st->props[k];
    int sacc = st->acc, nacc = 0;
    for (int i = 0; i < tot.x; ++i) {
      const int c = lst[i];
      const bool robust = c >= 0;
      const int s = robust ? c : -1 - c;
      double o8[7];
      if (i < PREF) {
        for (int k = 0; k < 7; ++k) o8[k] = sdp[i][k];
      } else {
        for (int k = 0; k < 6; ++k) o8[k] = dpn[8 * (size_t)s + k];
        o8[6] = robust ? 0.0 : -log(flip_u_of(seed, win[s]));
      }
      if (robust || flip_delta(fe, sP, o8) <= o8[6]) {
        for (int k = 0; k < 6; ++k) sP[k] = sP[k] - o8[k];
        sacc += 1;
        accl[nacc++] = s;
      }
    }
    st->nacc_win = nacc;
    for (int k = 0; k < 6; ++k) st->props[k] = sP[k];
    filter_state(fe, sP, st->sq);
    st->acc = sacc;
    st->npend = tot.y;
    st->next_new = st->nn_next;
  }
}

// one block of 32 threads per slot (accepted slots only do work): the
// half-edge rewiring, then the two face rows and five edge rows, then the
// four ring rows, each stage in parallel
// the flip of proposal p's edge: one warp rewires six half-edges, two face
// rows, five edge rows and four ring rows (patches of a window's accepted
// flips are disjoint, so commits never touch the same entries)
__device__ void commit_one(const TopoW& t, long long p, FlipState* st) {
  const int tid = threadIdx.x;
  const int e = flip_edge_of(st->seed, p, t.ne);
  const int a0 = 2 * e, b0 = 2 * e + 1;
  const int a1 = t.next[a0], a2 = t.next[a1], b1 = t.next[b0], b2 = t.next[b1];
  const int va0 = t.to[a0], va1 = t.to[a1], vb0 = t.to[b0], vb1 = t.to[b1];
  const int fa = t.face[a0], fb = t.face[b0];
  __syncwarp();  // every lane has read the old wiring
  if (tid == 0) {
    t.to[a0] = va1;
    t.to[b0] = vb1;
    t.next[a0] = a2;
    t.next[a2] = b1;
    t.next[b1] = a0;
    t.next[b0] = b2;
    t.next[b2] = a1;
    t.next[a1] = b0;
    t.face[a1] = fb;
    t.face[b1] = fa;
    t.fhe[fa] = a0;
    t.fhe[fb] = b0;
    if (t.vout[va0] == b0) t.vout[va0] = a1;
    if (t.vout[vb0] == a0) t.vout[vb0] = b1;
  }
  __syncwarp();
  if (tid == 0) face_row(t, fa);
  if (tid == 1) face_row(t, fb);
  if (tid == 2) edge_row(t, e);
  if (tid == 3) edge_row(t, a1 >> 1);
  if (tid == 4) edge_row(t, a2 >> 1);
  if (tid == 5) edge_row(t, b1 >> 1);
  if (tid == 6) edge_row(t, b2 >> 1);
  __syncwarp();
  if (tid < 4) {
    const int v = tid == 0 ? va0 : (tid == 1 ? va1 : (tid == 2 ? vb0 : vb1));
    if (!ring_row(t, v)) atomicExch(&st->status, TM_ERR_TOPOLOGY);
  }
  __syncwarp();
}

// the window's accepted flips (listed by k_metro), every CB-th per block
constexpr int CB = 152;
__global__ void __launch_bounds__(32) k_commit(TopoW t, const long long* win, const int* accl, FlipState* st) {
  const int nacc = st->nacc_win;
  for (int i = blockIdx.x; i < nacc; i += gridDim.x) commit_one(t, win[accl[i]], st);
}

__global__ void k_set_int(int* p, int v) {
  if (threadIdx.x == 0 && blockIdx.x == 0) *p = v;
}

__global__ void k_owner_init(int* owner, int n) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) owner[i] = 0;  // below every window's tags
}

inline int nblk(long n, int b) { return (int)((n + b - 1) / b); }

}  // namespace
}  // namespace tmg

static int flip_sweep(tm_mesh* m, tm_energy* e, const double* P, double ratio, uint64_t seed, int mode, int batch,
                      cudaStream_t s) {
  if (mode != 0 && mode != 1) fail(TM_ERR_ARG, "mode must be 0 (serial order) or 1 (batched)");
  if (mode == 1 && ratio > 1.0) fail(TM_ERR_RANGE, "flip_ratio must be <= 1.0");
  if (batch < 1 || batch > MAXB) fail(TM_ERR_ARG, "batch must be in [1, 4096]");
  int ne = m->ne;
  long long nflips = (long long)(ne * ratio);
  if (ne == 0 || nflips <= 0) return 0;
  // the sweep's starting properties with the FP64 stencil (the Metropolis
  // test then sees the same global sums as the FP64 CPU port of the sweep)
  {
    const int stencil = e->stencil;
    e->stencil = 0;
    energy_eval(e, m, P, false, false, nullptr, s);
    e->stencil = stencil;
  }
  EP ep = make_ep(e);
  const EPD epd = make_epd(ep);
  // the positions as double-words for the filter pass of the property
  // changes, and the float copy read by the repulsion prefilter
  const PosDW X{split_positions_dw(e, m->nv, P, s), std::max(m->nv, 1)};
  NLView nlv = e->nl.view;
  nlv.pos32 = e->pos32.get();
  TopoW t = m->topo_w();
  // workspace of the energy handle: no allocation per sweep
  DevBuf<int>& owner = e->fw_owner;
  DevBuf<int>& limit = e->fw_limit;
  DevBuf<long long>& win = e->fw_win;
  DevBuf<long long>& pend = e->fw_pend;
  DevBuf<unsigned char>& winner = e->fw_winner;
  DevBuf<int>& accl = e->fw_accl;
  DevBuf<double>& dpn = e->fw_dpn;
  DevBuf<float>& dpf = e->fw_dpf;
  owner.ensure(std::max(m->nv, 1));
  win.ensure(MAXB);
  pend.ensure(MAXB);
  winner.ensure(MAXB);
  accl.ensure(MAXB);
  dpn.ensure(8 * (size_t)MAXB);
  dpf.ensure(8 * (size_t)MAXB);
  e->fw_state.ensure(sizeof(FlipState));
  limit.ensure(1);
  FlipState* st = reinterpret_cast<FlipState*>(e->fw_state.get());
  k_owner_init<<<nblk(std::max(m->nv, 1), 256), 256, 0, s>>>(owner.get(), m->nv);
  TM_LAUNCH();
  FlipE fe{1.0 / ep.refA, 1.0 / ep.refV, 1.0 / ep.refC, ep.ka, ep.kv, ep.kc, ep.kt, ep.kr, ep.kb};
  FlipEF fg{(float)fe.irA, (float)fe.irV, (float)fe.irC, (float)fe.ka, (float)fe.kv,
            (float)fe.kc, (float)fe.kt, (float)fe.kr, (float)fe.kb};
  k_flip_init<<<1, 1, 0, s>>>(fe, e->glob.get(), nflips, seed, st);
  TM_LAUNCH();
  // windows are queued in groups without host round trips; W and the window
  // number live on the device, and a window after the last one is empty
  // (W = 0: every kernel returns at once).  A group's 40 launches do not
  // depend on the sweep (the seed is in the device state), so they are
  // captured once as a CUDA graph per launch key and replayed.
  const int B = batch;
  constexpr int GROUP = 8;
  // claim + winner as one cooperative launch when all its blocks fit on the
  // GPU at once (else, or when the launch is refused, two kernels)
  const int ncw = nblk(4L * B, 64);
  if (e->flip_coop == 0) {
    int per_sm = 0, nsm = 0, dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_claim_win, 64, 0);
    e->flip_coop = per_sm * nsm >= (MAXB * 4 + 63) / 64 ? 1 : -1;
    cudaGetLastError();
  }
  auto claim_win = [&](bool coop) {
    if (coop) {
      cudaLaunchConfig_t cfg = {};
      cfg.gridDim = dim3(ncw);
      cfg.blockDim = dim3(64);
      cfg.stream = s;
      cudaLaunchAttribute attr[1];
      attr[0].id = cudaLaunchAttributeCooperative;
      attr[0].val.cooperative = 1;
      cfg.attrs = attr;
      cfg.numAttrs = 1;
      TM_CUDA(cudaLaunchKernelEx(&cfg, k_claim_win, t, st, B, mode, (const long long*)pend.get(), win.get(),
                                 owner.get(), winner.get(), limit.get()));
    } else {
      k_fill<<<nblk(B, 256), 256, 0, s>>>(B, pend.get(), st, win.get(), limit.get());
      TM_LAUNCH();
      k_claim<<<ncw, 64, 0, s>>>(t, st, win.get(), owner.get());
      TM_LAUNCH();
      k_winner<<<ncw, 64, 0, s>>>(t, st, mode, win.get(), owner.get(), winner.get(), limit.get());
      TM_LAUNCH();
    }
  };
  auto launch_group = [&](bool coop) {
    for (int k = 0; k < GROUP; ++k) {
      claim_win(coop);
      k_delta<<<B, 64, 0, s>>>(t, st, win.get(), winner.get(), limit.get(), P, ep, epd, X, nlv, dpn.get(),
                               dpf.get(), e->sctf.get());
      TM_LAUNCH();
      k_metro<<<1, MB, 0, s>>>(win.get(), winner.get(), dpn.get(), dpf.get(), fe, fg, st, limit.get(), accl.get(),
                               pend.get());
      TM_LAUNCH();
      k_commit<<<CB, 32, 0, s>>>(t, win.get(), accl.get(), st);
      TM_LAUNCH();
    }
  };
  cudaGraphExec_t group = nullptr;
  if (s != nullptr && e->use_graphs) {
    std::vector<unsigned char> key;
    auto add = [&key](const void* p, size_t n) {
      const unsigned char* b = static_cast<const unsigned char*>(p);
      key.insert(key.end(), b, b + n);
    };
    const void* ptrs[] = {P, st, win.get(), pend.get(), limit.get(), owner.get(), winner.get(),
                          dpn.get(), dpf.get(), accl.get(), e->sctf.get(), X.p, m->d_to.get(),
                          m->d_next.get(), m->d_face.get(), m->d_vout.get(), m->d_fhe.get(), m->d_slot.get(),
                          m->d_nbr.get(), m->d_val.get(), m->d_fv.get(), m->d_edge.get()};
    add(ptrs, sizeof ptrs);
    const int ints[] = {B, mode, m->nv, m->ne, m->nf};
    add(ints, sizeof ints);
    add(&ep, sizeof ep);
    add(&nlv, sizeof nlv);
    add(&fe, sizeof fe);
    add(&fg, sizeof fg);
    add(&epd, sizeof epd);
    if (!e->flip_graph.exec || e->flip_graph.key != key) {
      if (e->flip_graph.exec) cudaGraphExecDestroy(e->flip_graph.exec);
      e->flip_graph.exec = nullptr;
      e->flip_graph.key.clear();
      cudaGraph_t g = nullptr;
      for (int attempt = 0;; ++attempt) {
        const bool coop = e->flip_coop > 0;
        TM_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
        bool failed = false;
        try {
          launch_group(coop);
        } catch (...) {
          if (!coop || attempt > 0) {
            cudaStreamEndCapture(s, &g);  // leave capture mode before reporting
            if (g) cudaGraphDestroy(g);
            cudaGetLastError();
            throw;
          }
          failed = true;
        }
        cudaError_t ec = cudaStreamEndCapture(s, &g);
        if (!failed && ec == cudaSuccess) break;
        // a cooperative launch that cannot be captured: two kernels instead
        if (g) cudaGraphDestroy(g);
        g = nullptr;
        cudaGetLastError();
        if (!coop || attempt > 0) TM_CUDA(ec);
        e->flip_coop = -1;
      }
      cudaError_t rc = cudaGraphInstantiate(&e->flip_graph.exec, g, 0);
      cudaGraphDestroy(g);
      if (rc != cudaSuccess) e->flip_graph.exec = nullptr;
      TM_CUDA(rc);
      e->flip_graph.key.swap(key);
    }
    group = e->flip_graph.exec;
  }
  FlipState hs;
  for (;;) {
    if (group)
      TM_CUDA(cudaGraphLaunch(group, s));
    else
      launch_group(e->flip_coop > 0);
    TM_CUDA(cudaMemcpyAsync(&hs, st, sizeof(FlipState), cudaMemcpyDeviceToHost, s));
    TM_CUDA(cudaStreamSynchronize(s));
    if (hs.status) fail(TM_ERR_TOPOLOGY, "flip produced a valence above TM_MAXVAL");
    // slot 0 of a window always owns its patch, so every window decides at
    // least one proposal and the sweep ends
    if (hs.npend == 0 && hs.next_new >= nflips) break;
    if (hs.wid >= (1 << 19) - GROUP) fail(TM_ERR_ARG, "too many windows in one sweep");
  }
  m->host_topo_stale = true;
  if (hs.acc > 0) {
    ++m->topo_version;
    k_set_int<<<1, 1, 0, s>>>(m->d_topo_ver.get(), (int)(m->topo_version & 0x7fffffff));
    TM_LAUNCH();
  }
  return hs.acc;
}

extern "C" int tm_flip(tm_mesh* m, tm_energy* e, double ratio, uint64_t seed, int mode, int batch,
                       int32_t* accepted) {
  TM_API_BEGIN
  if (!m || !e || !accepted) fail(TM_ERR_ARG, "NULL argument");
  *accepted = 0;
  m->upload_points(e->stream);
  *accepted = flip_sweep(m, e, m->d_pts.get(), ratio, seed, mode, batch, e->stream);
  TM_API_END
}

extern "C" int tm_flip_device(tm_mesh* m, tm_energy* e, const double* d_points, double ratio, uint64_t seed,
                              int mode, int batch, int32_t* accepted, void* stream) {
  TM_API_BEGIN
  if (!m || !e || !d_points || !accepted) fail(TM_ERR_ARG, "NULL argument");
  *accepted = 0;
  cudaStream_t s = stream ? (cudaStream_t)stream : e->stream;
  *accepted = flip_sweep(m, e, d_points, ratio, seed, mode, batch, s);
  TM_API_END
}
