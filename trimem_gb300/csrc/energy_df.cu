// Double-float stencil variant of the energy / gradient evaluation
// (tm_energy_set_stencil_precision(e, 2)).
//
// GB300's FP64 pipe retires a small fraction of the FP32 rate, and the FP64
// kernels of energy.cu keep it ~85% busy.  These kernels compute the same
// quantities with double-word numbers (df64.cuh: pairs of floats, ~48-bit
// significands) on the FP32 pipe:
//   * positions are split once per evaluation into float hi / lo parts
//     (one float4 each per vertex); edge vectors are double-word differences,
//     so |x| >> |x_b - x_a| costs no accuracy;
//   * products are exact TwoProds, sums collect their rounding errors in one
//     float (Dot2 / Sum2 style) and are renormalised once, normalisations
//     and reciprocals are a float estimate plus one Newton step;
//   * the dihedral angle is refined from a float atan2 estimate on the grid
//     t0 = k/128 (double-word sine and cosine table), theta = t0 + asin(x)
//     with x = sin(theta - t0) from the sine and cosine of the face normals;
//   * FP64 stays for the flat-bottom potentials below lc1 with non-positive
//     exponents, the repulsion pairs (exact pair decisions), the global sums
//     and the penalty assembly.
// The results agree with the FP64 oracle to ~1e-13 relative (the parity
// tests hold them to 1e-10); they are not bitwise equal to the FP64 kernels.
#include <algorithm>
#include <cmath>

#include "df64.cuh"
#include "tm_dw.cuh"
#include "tm_energy.cuh"
#include "tm_internal.h"
#include "tm_math.cuh"

namespace tmg {

namespace {

// Face record, four float4 per face:
//   [0] (nx, ny)  [1] (nz, A)  [2] (V, cot a)  [3] (cot b, cot c)
// with n the unit normal, A the area, V the signed volume about the origin
// and the cotangents of the corners in the face's stored vertex order.
// Edge record, two float4 per edge:
//   [0] (l, theta)  [1] (dB/dl, s/l)
// with s = +1 on interior edges and -1 on boundary edges.
// Every entry is a double-word (hi, lo).

__global__ void k_split_dw(int nv, const double* __restrict__ P, float4* __restrict__ X, float* __restrict__ P32) {
  int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= nv) return;
  float hx, hy, hz, lx, ly, lz;
  split_bits(P[3 * v], &hx, &lx);
  split_bits(P[3 * v + 1], &hy, &ly);
  split_bits(P[3 * v + 2], &hz, &lz);
  X[v] = make_float4(hx, hy, hz, 0.0f);
  X[nv + v] = make_float4(lx, ly, lz, 0.0f);
  // the float copy of the positions read by the repulsion prefilter
  P32[3 * v] = hx;
  P32[3 * v + 1] = hy;
  P32[3 * v + 2] = hz;
}

// fav: (area, volume) again as (hi, lo, hi, lo), compact for k_vertex_dw
__global__ void __launch_bounds__(256) k_face_dw(Topo t, PosDW X, float4* __restrict__ fd, float4* __restrict__ fav) {
  int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= t.nf) return;
  const int a = t.fv[3 * f], b = t.fv[3 * f + 1], c = t.fv[3 * f + 2];
  const df3 pa = X.at(a), pb = X.at(b), pc = X.at(c);
  const df3 eab = sub3(pb, pa), eac = sub3(pc, pa), ebc = sub3(pc, pb);
  const df3 N = cross3(eab, eac);
  const df n2 = dot3(N, N);
  const df r = rsqrt_dw(n2);  // 1 / |N|
  const df A = half(mul_s(n2, r));
  // (p_a x p_b) . p_c = p_a . ((p_b - p_a) x (p_c - p_a)) = p_a . N
  const df V = mul_s(dot3(pa, N), sixth());
  const df nx = mul_s(N.x, r), ny = mul_s(N.y, r), nz = mul_s(N.z, r);
  const df c0 = mul_s(dot3(eab, eac), r);
  const df c1 = neg(mul_s(dot3(eab, ebc), r));
  const df c2 = mul_s(dot3(eac, ebc), r);
  float4* o = fd + 4 * (size_t)f;
  o[0] = make_float4(nx.hi, nx.lo, ny.hi, ny.lo);
  o[1] = make_float4(nz.hi, nz.lo, A.hi, A.lo);
  o[2] = make_float4(V.hi, V.lo, c0.hi, c0.lo);
  o[3] = make_float4(c1.hi, c1.lo, c2.hi, c2.lo);
  fav[f] = make_float4(A.hi, A.lo, V.hi, V.lo);
}

// Flat-bottom bond of an edge shorter than lc1 (src/mesh_tether.h:29-85)
// in double-word arithmetic: value e^(l/(l-lc1)) / l^r, derivative
// -(lc1/(l-lc1)^2 + r/l) e^(l/(l-lc1)) / l^r (plus the l > lc0 branch when
// lc1 > lc0).
__device__ __forceinline__ void edge_bond_short_dw(const EP& ep, const EPD& epd, df l, df* val, df* fac) {
  const int r = ep.r;
  df v = df_make(0.0f), f = df_make(0.0f);
  const bool above = df_less(epd.lc0, l);
  if (above) {
    const df d = sub_s(l, epd.lc0);
    v = mul_s(epd.br1, ipow_dw(d, r));
    f = mul_s(epd.br2, ipow_dw(d, r - 1));
  }
  const df ilmc = rcp_dw(sub_s(l, epd.lc1)), il = rcp_dw(l);
  const df ex = df_exp_nonpos(mul_s(l, ilmc));
  const df ilr = ipow_dw(il, r);
  if (!above) v = mul_s(ex, ilr);
  f = sub_s(f, add_s(mul_s(epd.lc1, mul_s(ilmc, ilmc)), mul_s(il, df_make((float)r))));
  *val = v;
  *fac = mul_s(mul_s(f, ilr), ex);
}

// elt: (l theta, bond value) as (hi, lo, hi, lo), compact for k_vertex_dw
__global__ void __launch_bounds__(256) k_edge_dw(Topo t, PosDW X, const float4* __restrict__ fd,
                                                float4* __restrict__ ed, float4* __restrict__ elt, EP ep, EPD epd,
                                                const float4* __restrict__ sct) {
  int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= t.ne) return;
  const int4 E = t.edge[e];
  const df3 ev = sub3(X.at(E.y), X.at(E.x));
  const df l2 = dot3(ev, ev);
  const df il = rsqrt_dw(l2);
  const df l = mul_s(l2, il);
  df th = df_make(0.0f);
  const bool interior = E.z >= 0 && E.w >= 0;
  if (interior) {
    const float4 a0 = __ldg(fd + 4 * (size_t)E.z), a1 = __ldg(fd + 4 * (size_t)E.z + 1);
    const float4 b0 = __ldg(fd + 4 * (size_t)E.w), b1 = __ldg(fd + 4 * (size_t)E.w + 1);
    const df3 n0 = {{a0.x, a0.y}, {a0.z, a0.w}, {a1.x, a1.y}};
    const df3 n1 = {{b0.x, b0.y}, {b0.z, b0.w}, {b1.x, b1.y}};
    // n0 x n1 lies along the shared edge: its projection on the unit edge
    // is the signed sine, with the sign of the reference's test
    // (n0 x n1) . e >= 0
    const df sd = mul_s(dot3(cross3(n0, n1), ev), il);
    th = angle_dw(sd, dot3(n0, n1), sct);
  }
  // flat-bottom edge penalty: above the flat bottom products only, below it
  // the exponential (a warp with any short edge takes that branch; on the
  // jittered benchmark membrane nearly every warp has one, which costs less
  // than a list of short edges and a kernel of their own)
  df val = df_make(0.0f), db = df_make(0.0f);
  const bool shortb = ep.btype == 0 && df_less(l, epd.lc1);
  if (ep.btype == 0 && !shortb && df_less(epd.lc0, l) && ep.r >= 1) {
    const df d = sub_s(l, epd.lc0);
    const df dr1 = ipow_dw(d, ep.r - 1);
    val = mul_s(epd.br1, mul_s(dr1, d));
    db = mul_s(epd.br2, dr1);
  }
  if (shortb) {
    if (ep.r >= 1) {
      edge_bond_short_dw(ep, epd, l, &val, &db);
    } else {  // non-positive exponents: FP64
      double v, f;
      const double ld = df_to(l);
      edge_bond(ep, ld, 1.0 / ld, &v, &f);
      val = df_from(v);
      db = df_from(f);
    }
  }
  const df ils = interior ? il : neg(il);
  ed[2 * (size_t)e] = make_float4(l.hi, l.lo, th.hi, th.lo);
  ed[2 * (size_t)e + 1] = make_float4(db.hi, db.lo, ils.hi, ils.lo);
  const df lt = mul_s(l, th);
  elt[e] = make_float4(lt.hi, lt.lo, val.hi, val.lo);
}

// Per-vertex ring sums, the six properties, the curvature weights
// (kb rho, 2/3 kb rho^2) for the gradient, and the global sums: a
// double-word shuffle tree per warp, FP64 over the warps of a block in warp
// order, and the last block (atomic ticket) reduces the block partials in
// block order and assembles energy and the penalty factors.  Fixed order
// throughout: results are bit-reproducible.
__global__ void __launch_bounds__(VB, 4) k_vertex_dw(Topo t, const float4* __restrict__ fav,
                                                 const float4* __restrict__ elt, const double* __restrict__ reppot,
                                                 EP ep, EPD epd, float4* __restrict__ rk, double* __restrict__ partial,
                                                 Globals* g) {
  constexpr int NW = VB / 32;
  __shared__ float2 wsum[6][NW];
  __shared__ double redd[6];
  __shared__ bool last;
  const int v = blockIdx.x * VB + threadIdx.x;
  df pr[6];
  for (int k = 0; k < 6; ++k) pr[k] = df_make(0.0f);
  if (v < t.nv) {
    const int d = t.val[v];
    dacc A = {0.0f, 0.0f}, Vo = A, LT = A, T = A;
    // slots in groups of six (one group at the usual valence): all loads of
    // a group are issued before the sums, which keep the slot order
    constexpr int G = 6;
    for (int m0 = 0; m0 < d; m0 += G) {
      int4 s[G];
#pragma unroll
      for (int k = 0; k < G; ++k) s[k] = m0 + k < d ? t.slot[(size_t)(m0 + k) * t.nv + v] : make_int4(0, -1, 0, 0);
      float4 av[G], lb[G];
#pragma unroll
      for (int k = 0; k < G; ++k) {
        const int f = slot_face(s[k].y);
        av[k] = lb[k] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        if (f >= 0) {
          av[k] = __ldg(fav + f);
          lb[k] = __ldg(elt + s[k].z);
        }
      }
#pragma unroll
      for (int k = 0; k < G; ++k) {
        if (slot_face(s[k].y) < 0) continue;
        acc_add(A, lo_hi(av[k].x, av[k].y));
        acc_add(Vo, lo_hi(av[k].z, av[k].w));
        acc_add(LT, lo_hi(lb[k].x, lb[k].y));
        if (ep.btype == 0) {
          acc_add(T, lo_hi(lb[k].z, lb[k].w));
        } else {
          const df q = sub_s(mul_s(lo_hi(av[k].x, av[k].y), epd.inv_a0), df_make(1.0f));
          acc_add(T, mul_s(q, q));
        }
      }
    }
    const df a = mul_s(acc_val(A), third());
    const df c = ldexp2(acc_val(LT), 0.25f);
    const df ia = rcp_dw(a);
    const df rho = mul_s(c, ia);
    pr[0] = a;
    pr[1] = mul_s(acc_val(Vo), third());
    pr[2] = c;
    pr[3] = ldexp2(mul_s(c, rho), 2.0f);  // 2 c^2 / a
    pr[4] = mul_s(acc_val(T), epd.inv_tdiv);
    split_bits(reppot[v], &pr[5].hi, &pr[5].lo);  // integer operations, no FP64
    const df kr = mul_s(epd.kb, rho), kq = mul_s(epd.kb23, mul_s(rho, rho));
    rk[v] = make_float4(kr.hi, kr.lo, kq.hi, kq.lo);
  }
  // warp tree (lane 0 ends with the warp's sum), then FP64 over the warps
#pragma unroll
  for (int off = 16; off > 0; off >>= 1)
#pragma unroll
    for (int k = 0; k < 6; ++k) {
      const df o = {__shfl_down_sync(0xffffffffu, pr[k].hi, off), __shfl_down_sync(0xffffffffu, pr[k].lo, off)};
      pr[k] = add_s(pr[k], o);
    }
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0)
    for (int k = 0; k < 6; ++k) wsum[k][w] = make_float2(pr[k].hi, pr[k].lo);
  __syncthreads();
  // property k of the block: thread k sums the warps in warp order (one
  // FP64 conversion per block: GB300's FP64 pipe is the scarce one)
  if (threadIdx.x < 6) {
    df s = df_make(0.0f);
    for (int q = 0; q < NW; ++q) s = add_s(s, lo_hi(wsum[threadIdx.x][q].x, wsum[threadIdx.x][q].y));
    partial[8 * (size_t)blockIdx.x + threadIdx.x] = df_to(s);
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    const unsigned int tk = atomicAdd(&g->ticket, 1u);
    last = (tk == gridDim.x - 1);
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  // last block: warp k reduces property k over the block partials (lane l
  // takes blocks l, l + 32, ... in order, then a fixed shuffle tree)
  if (w < 6) {
    double acc = 0.0;
    for (int b = lane; b < (int)gridDim.x; b += 32) acc += ((volatile double*)partial)[8 * (size_t)b + w];
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, off);
    if (lane == 0) redd[w] = acc;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int k = 0; k < 6; ++k) g->props[k] = redd[k];
    assemble(ep, g);
    g->ticket = 0;
  }
}

// Gradient gather per vertex i over its ring (slot m: face (i, j = r_m,
// k = r_{m-1})), the reference's gather (src/mesh_properties.cpp:51-148 with
// src/kernel.h:124-137) regrouped per face and edge, with alpha =
// gA - 2/3 kb (rho_i^2 + rho_j^2 + rho_k^2) and w = gC/2 + kb (rho_i + rho_j):
//   area       (alpha / 2) n x (x_k - x_j)
//   volume     (gV / 6) x_j x x_k, summed as d_j x d_k with d = x - x_i
//              (the x_i x (d_k - d_j) parts cancel around a closed fan)
//   length     -(w theta + kt dB/dl) / l (x_j - x_i) for edge (i, j)
//   dihedral   along n: w_ij cot_j + w_ik cot_k - w_jk (cot_j + cot_k)
// Positions enter relative to x_i, so the sums stay near the size of the
// result.
__device__ __forceinline__ df cot_of(const float4& F2, const float4& F3, int c) {
  return c == 0 ? lo_hi(F2.z, F2.w) : (c == 1 ? lo_hi(F3.x, F3.y) : lo_hi(F3.z, F3.w));
}

template <bool CLOSED>
__global__ void __launch_bounds__(128, 5) k_grad_dw(Topo t, PosDW X, const float4* __restrict__ fd,
                                                const float4* __restrict__ ed, const float4* __restrict__ rk,
                                                const double* __restrict__ repg, const Globals* __restrict__ g,
                                                EP ep, EPD epd, double* __restrict__ grad) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= t.nv) return;
  const df gA = {g->gdf[0], g->gdf[1]}, gV = {g->gdf[2], g->gdf[3]}, gC = {g->gdf[4], g->gdf[5]};
  const df hgC = half(gC);
  const df3 xi = X.at(i);
  const float4 q4 = __ldg(rk + i);
  const df ai = sub_s(gA, lo_hi(q4.z, q4.w));
  const df wi = add_s(hgC, lo_hi(q4.x, q4.y));
  dacc3 acc = {{0.0f, 0.0f}, {0.0f, 0.0f}, {0.0f, 0.0f}};
  dacc3 vcr = acc, vtel = acc;
  const int d = t.val[i];
  if (d > 0) {
    const size_t nv = t.nv;
    const int4 sp = t.slot[(size_t)(d - 1) * nv + i];
    df3 dk = sub3(X.at(sp.x), xi);
    float4 qk = __ldg(rk + sp.x);
    df wprev = df_make(0.0f);  // w of edge (i, k) and whether it is interior
    bool prev_int = false;
    for (int m = 0; m < d; ++m) {
      const int4 sc = t.slot[(size_t)m * nv + i];
      const df3 dj = sub3(X.at(sc.x), xi);
      const float4 qj = __ldg(rk + sc.x);
      const int f = slot_face(sc.y);
      const float4 e0 = __ldg(ed + 2 * (size_t)sc.z), e1 = __ldg(ed + 2 * (size_t)sc.z + 1);
      const bool int_ij = e1.z > 0.0f;
      const df w = add_s(wi, lo_hi(qj.x, qj.y));
      if (f >= 0) {
        const float4 F0 = __ldg(fd + 4 * (size_t)f), F1 = __ldg(fd + 4 * (size_t)f + 1);
        const float4 F2 = __ldg(fd + 4 * (size_t)f + 2), F3 = __ldg(fd + 4 * (size_t)f + 3);
        const float4 ejk = __ldg(ed + 2 * (size_t)sc.w + 1);
        const df3 n = {{F0.x, F0.y}, {F0.z, F0.w}, {F1.x, F1.y}};
        const int ci = slot_corner(sc.y);
        const int cjx = ci == 2 ? 0 : ci + 1, ckx = ci == 0 ? 2 : ci - 1;
        const df cj = cot_of(F2, F3, cjx), ck = cot_of(F2, F3, ckx);
        // face (i, j, k): area and volume terms
        df alpha = sub_s(sub_s(ai, lo_hi(qj.z, qj.w)), lo_hi(qk.z, qk.w));
        if (ep.btype == 1) {
          const df q = sub_s(mul_s(lo_hi(F1.z, F1.w), epd.inv_a0), df_make(1.0f));
          alpha = add_s(alpha, ldexp2(mul_s(mul_s(epd.kt, q), epd.inv_a0), 2.0f));
        }
        const df3 dkj = sub3(dk, dj);
        acc_add3(acc, scale3(half(alpha), cross3(n, dkj)));
        acc_add3(vcr, cross3(dj, dk));
        if (!CLOSED) acc_add3(vtel, dkj);
        // edge (i, j): length term
        df cl = mul_s(w, lo_hi(e0.z, e0.w));
        if (ep.btype == 0) cl = add_s(cl, mul_s(epd.kt, lo_hi(e1.x, e1.y)));
        acc_add3(acc, scale3(neg(mul_s(cl, dabs(lo_hi(e1.z, e1.w)))), dj));
        // dihedral terms of edges (i, j), (i, k) and (j, k) along n
        df cn = df_make(0.0f);
        if (int_ij) cn = mul_s(w, cj);
        if (prev_int && m > 0) cn = add_s(cn, mul_s(wprev, ck));
        if (ejk.z > 0.0f)
          cn = sub_s(cn, mul_s(add_s(add_s(hgC, lo_hi(qj.x, qj.y)), lo_hi(qk.x, qk.y)), add_s(cj, ck)));
        acc_add3(acc, scale3(cn, n));
      }
      wprev = w;
      prev_int = int_ij && f >= 0;
      dk = dj;
      qk = qj;
    }
    // the last edge (i, r_{d-1}) is edge (i, k) of the first face (whose
    // record is read again rather than kept in registers through the loop)
    const int4 s0 = t.slot[i];
    const int f0 = slot_face(s0.y);
    if (prev_int && f0 >= 0) {
      const float4 F0 = __ldg(fd + 4 * (size_t)f0), F1 = __ldg(fd + 4 * (size_t)f0 + 1);
      const float4 F2 = __ldg(fd + 4 * (size_t)f0 + 2), F3 = __ldg(fd + 4 * (size_t)f0 + 3);
      const int ci = slot_corner(s0.y);
      const df ck0 = cot_of(F2, F3, ci == 0 ? 2 : ci - 1);
      const df3 n0 = {{F0.x, F0.y}, {F0.z, F0.w}, {F1.x, F1.y}};
      acc_add3(acc, scale3(mul_s(wprev, ck0), n0));
    }
  }
  df3 vol = acc_val3(vcr);
  if (!CLOSED) {
    const df3 tx = cross3(xi, acc_val3(vtel));
    vol = {add_s(vol.x, tx.x), add_s(vol.y, tx.y), add_s(vol.z, tx.z)};
  }
  const df gV6 = mul_s(gV, sixth());
  acc_add3(acc, scale3(gV6, vol));
  const df3 r = acc_val3(acc);
  const d3 rg = ld3(repg, i);
  grad[3 * i] = df_to(r.x) + ep.kr * rg.x;
  grad[3 * i + 1] = df_to(r.y) + ep.kr * rg.y;
  grad[3 * i + 2] = df_to(r.z) + ep.kr * rg.z;
}

inline int nblk(long n, int b) { return (int)((n + b - 1) / b); }

df host_df(double x) {
  float h = (float)x;
  return {h, (float)(x - (double)h)};
}

}  // namespace

EPD make_epd(const EP& ep) {
  EPD epd;
  epd.kb = host_df(ep.kb);
  epd.kt = host_df(ep.kt);
  epd.kr = host_df(ep.kr);
  epd.kb23 = host_df(ep.kb * (2.0 / 3.0));
  epd.a0 = host_df(ep.a0);
  epd.inv_a0 = host_df(1.0 / ep.a0);
  epd.inv_tdiv = host_df(1.0 / ep.tdiv);
  epd.lc0 = host_df(ep.lc0);
  epd.lc1 = host_df(ep.lc1);
  epd.br1 = host_df(ep.br1);
  epd.br2 = host_df(ep.br2);
  return epd;
}

const float4* split_positions_dw(tm_energy* e, int nv, const double* P, cudaStream_t s) {
  const size_t n = std::max(nv, 1);
  e->pos32.ensure(3 * n);
  e->posdw.ensure(2 * n);
  if (nv) k_split_dw<<<nblk(nv, 256), 256, 0, s>>>(nv, P, e->posdw.get(), e->pos32.get());
  TM_LAUNCH();
  return e->posdw.get();
}

void energy_eval_df(tm_energy* e, tm_mesh* m, const double* P, bool want_grad, double* d_grad, cudaStream_t s,
                    cudaEvent_t* ev) {
  e->ensure(m->nv, m->ne, m->nf);
  const size_t nv = std::max(m->nv, 1);
  e->pos32.ensure(3 * nv);
  e->posdw.ensure(2 * nv);
  Topo t = m->topo();
  EP ep = make_ep(e);
  const EPD epd = make_epd(ep);
  PosDW X{e->posdw.get(), (int)nv};
  float4* fd = reinterpret_cast<float4*>(e->face.get());   // 64 bytes per face
  float4* ed = reinterpret_cast<float4*>(e->edge.get());   // 32 bytes per edge
  float4* eb = reinterpret_cast<float4*>(e->ebond.get());  // (l theta, bond) per edge, 16 bytes
  float4* fav = reinterpret_cast<float4*>(e->fav.get());   // (area, volume) per face, 16 bytes
  float4* rho = reinterpret_cast<float4*>(e->rho.get());   // (kb rho, 2/3 kb rho^2) per vertex
  if (ev) TM_CUDA(cudaEventRecord(ev[0], s));
  if (m->nv) k_split_dw<<<nblk(m->nv, 256), 256, 0, s>>>(m->nv, P, e->posdw.get(), e->pos32.get());
  TM_LAUNCH();
  const bool conc = ev == nullptr;  // repulsion overlaps the face and edge kernels
  if (conc) fork_repulsion(e, m, P, want_grad, s, true);
  if (t.nf) k_face_dw<<<nblk(t.nf, 256), 256, 0, s>>>(t, X, fd, fav);
  TM_LAUNCH();
  if (ev) TM_CUDA(cudaEventRecord(ev[1], s));
  if (t.ne) k_edge_dw<<<nblk(t.ne, 256), 256, 0, s>>>(t, X, fd, ed, eb, ep, epd, e->sctf.get());
  TM_LAUNCH();
  if (ev) TM_CUDA(cudaEventRecord(ev[2], s));
  if (conc)
    join_repulsion(e, s, true);
  else
    fork_repulsion(e, m, P, want_grad, s, false);
  int nb = std::max(1, nblk(t.nv, VB));
  k_vertex_dw<<<nb, VB, 0, s>>>(t, fav, eb, e->reppot.get(), ep, epd, rho, e->partials.get(), e->glob.get());
  TM_LAUNCH();
  if (ev) TM_CUDA(cudaEventRecord(ev[3], s));
  if (want_grad && t.nv) {
    if (m->closed)
      k_grad_dw<true><<<nblk(t.nv, 128), 128, 0, s>>>(t, X, fd, ed, rho, e->repg.get(), e->glob.get(), ep, epd,
                                                      d_grad);
    else
      k_grad_dw<false><<<nblk(t.nv, 128), 128, 0, s>>>(t, X, fd, ed, rho, e->repg.get(), e->glob.get(), ep, epd,
                                                       d_grad);
  }
  TM_LAUNCH();
  if (ev) TM_CUDA(cudaEventRecord(ev[4], s));
}

}  // namespace tmg
