// Double-float stencil variant of the energy / gradient evaluation
// (tm_energy_set_stencil_precision(e, 2)).
//
// The FP64 kernels of energy.cu run the FP64 pipe at ~87% (measured), and on
// GB300 that pipe retires 1/58 of the FP32 rate.  These kernels compute the
// same quantities with double-float numbers (df64.cuh: pairs of floats,
// ~48-bit significands, error-free transformations on the FP32 pipe):
//   * positions are split once per evaluation into float hi/lo parts; edge
//     vectors are double-float differences, so |x| >> |x_b - x_a| costs no
//     accuracy;
//   * face records, edge records, vertex sums and the gradient gather are
//     double-float; the dihedral angle is atan2(|n0 x n1|, n0 . n1) refined
//     from a float estimate (FP64 atan2 only above 0.8 rad);
//   * FP64 stays for the flat-bottom potentials outside the flat bottom,
//     the repulsion pairs (exact pair decisions), the global sums and the
//     penalty assembly.
// The results agree with the FP64 oracle to ~1e-13 relative (the 1e-10 bound
// of the parity tests); they are not bitwise equal to the FP64 kernels.
#include <algorithm>
#include <cmath>

#include "df64.cuh"
#include "tm_energy.cuh"
#include "tm_internal.h"
#include "tm_math.cuh"

namespace tmg {

struct __align__(16) FaceDF {
  df nx, ny, nz, A, V, c0, c1, c2;
};
// il: 1/l on interior edges, -1/l on boundary edges (sign = interior flag)
struct __align__(16) EdgeDF {
  df l, th, db, il;
};

namespace {

// double-float constants 1/3 and 1/6 (hi = float(c), lo = float(c - hi))
__device__ __forceinline__ df third() { return {3.333333433e-01f, -9.934107481e-09f}; }
__device__ __forceinline__ df sixth() { return {1.666666716e-01f, -4.967053740e-09f}; }

struct PosDF {
  const float* hi;
  const float* lo;
  __device__ __forceinline__ df3 at(int v) const {
    return {{hi[3 * v], lo[3 * v]}, {hi[3 * v + 1], lo[3 * v + 1]}, {hi[3 * v + 2], lo[3 * v + 2]}};
  }
};

// double-float parameters (hi/lo from the host)
struct EPD {
  df kb, kt, kr, kb23, a0, inv_a0, inv_tdiv, lc0, lc1;
};
__device__ __forceinline__ bool df_less(df a, df b) { return a.hi < b.hi || (a.hi == b.hi && a.lo < b.lo); }
__device__ __forceinline__ df df_ipow(df x, int n) {
  df r = df_make(1.0f);
  for (int k = 0; k < n; ++k) r = r * x;
  return r;
}

__global__ void k_split_df(int n3, const double* __restrict__ P, float* __restrict__ hi, float* __restrict__ lo) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n3) return;
  double x = P[i];
  float h = (float)x;
  hi[i] = h;
  lo[i] = (float)(x - (double)h);
}

// fav: (area, volume) again as (hi, lo, hi, lo), compact for k_vertex_df
__global__ void __launch_bounds__(256) k_face_df(Topo t, PosDF X, FaceDF* __restrict__ fd, float4* __restrict__ fav) {
  int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= t.nf) return;
  int a = t.fv[3 * f], b = t.fv[3 * f + 1], c = t.fv[3 * f + 2];
  df3 pa = X.at(a), pb = X.at(b), pc = X.at(c);
  df3 eab = pb - pa, eac = pc - pa, ebc = pc - pb;
  df3 N = dcross(eab, eac);
  df nn = df_sqrt(ddot(N, N));
  df inv = df_make(1.0f) / nn;
  FaceDF F;
  F.nx = inv * N.x;
  F.ny = inv * N.y;
  F.nz = inv * N.z;
  F.A = ldexp2(nn, 0.5f);
  F.V = ddot(pa, N) * sixth();
  F.c0 = ddot(eab, eac) * inv;
  F.c1 = -(ddot(eab, ebc) * inv);
  F.c2 = ddot(eac, ebc) * inv;
  fd[f] = F;
  fav[f] = make_float4(F.A.hi, F.A.lo, F.V.hi, F.V.lo);
}

// elt: (l theta, bond value) as (hi, lo, hi, lo), compact for k_vertex_df
// (the bond value of short edges is filled in by k_bond_short_df)
__global__ void __launch_bounds__(256) k_edge_df(Topo t, PosDF X, const FaceDF* __restrict__ fd,
                                                EdgeDF* __restrict__ ed, float4* __restrict__ elt, EP ep, EPD epd,
                                                int* __restrict__ blist, int* __restrict__ bcnt) {
  int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= t.ne) return;
  int4 E = t.edge[e];
  df3 ev = X.at(E.y) - X.at(E.x);
  df l = df_sqrt(ddot(ev, ev));
  EdgeDF o;
  o.l = l;
  o.th = df_make(0.0f);
  o.il = -(df_make(1.0f) / l);
  if (E.z >= 0 && E.w >= 0) {
    const FaceDF& F0 = fd[E.z];
    const FaceDF& F1 = fd[E.w];
    df3 n0 = {F0.nx, F0.ny, F0.nz}, n1 = {F1.nx, F1.ny, F1.nz};
    df3 cr = dcross(n0, n1);
    df c = ddot(n0, n1);
    df sn = df_sqrt(ddot(cr, cr));
    df th;
    if (!df_atan2_pos(sn, c, &th)) th = df_from(atan2(df_to(sn), df_to(c)));
    o.th = df_lt0(ddot(cr, ev)) ? -th : th;
    o.il = -o.il;
  }
  // flat-bottom edge penalty: above the flat bottom inline in double-float
  // (products only), below it (exp, FP64) through the short-edge list
  df val = df_make(0.0f);
  o.db = df_make(0.0f);
  bool shortb = ep.btype == 0 && df_less(l, epd.lc1);
  if (ep.btype == 0 && !shortb && df_less(epd.lc0, l) && ep.r >= 1) {
    int r = ep.r;
    df d = l - epd.lc0;
    df dr1 = df_ipow(d, r - 1);
    float rr = (float)r;
    val = df_ipow(df_make(rr), r + 1) * (dr1 * d);
    o.db = df_ipow(df_make(rr), r + 2) * dr1;
  }
  warp_append(shortb, e, blist, bcnt);
  ed[e] = o;
  const df lt = o.l * o.th;
  elt[e] = make_float4(lt.hi, lt.lo, val.hi, val.lo);
}

// Flat-bottom bond of an edge shorter than lc1 (src/mesh_tether.h:29-85)
// in double-word arithmetic: value e^(l/(l-lc1)) / l^r, derivative
// -(lc1/(l-lc1)^2 + r/l) e^(l/(l-lc1)) / l^r (plus the l > lc0 branch when
// lc1 > lc0).
__device__ __forceinline__ void edge_bond_short_df(const EP& ep, const EPD& epd, df l, df* val, df* fac) {
  const int r = ep.r;
  df v = df_make(0.0f), f = df_make(0.0f);
  const bool above = df_less(epd.lc0, l);
  if (above) {
    const df fr = df_make((float)r), d = l - epd.lc0;
    v = df_ipow(fr, r + 1) * df_ipow(d, r);
    f = df_ipow(fr, r + 2) * df_ipow(d, r - 1);
  }
  const df lmc = l - epd.lc1;
  const df ilmc = df_make(1.0f) / lmc, il = df_make(1.0f) / l;
  const df ex = df_exp_nonpos(l * ilmc);
  const df ilr = df_ipow(il, r);
  if (!above) v = ex * ilr;
  f = f - (epd.lc1 * ilmc * ilmc + il * (float)r);
  *val = v;
  *fac = (f * ilr) * ex;
}

__global__ void k_bond_short_df(EdgeDF* __restrict__ ed, float4* __restrict__ elt, EP ep, EPD epd,
                                const int* __restrict__ blist, const int* __restrict__ bcnt) {
  int n = *bcnt;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    int e = blist[i];
    if (ep.r >= 1) {
      df val, fac;
      edge_bond_short_df(ep, epd, ed[e].l, &val, &fac);
      ed[e].db = fac;
      elt[e].z = val.hi;
      elt[e].w = val.lo;
    } else {  // non-positive exponents: FP64
      double val, fac;
      const double l = df_to(ed[e].l);
      edge_bond(ep, l, 1.0 / l, &val, &fac);
      ed[e].db = df_from(fac);
      const df v = df_from(val);
      elt[e].z = v.hi;
      elt[e].w = v.lo;
    }
  }
}

__global__ void __launch_bounds__(VB) k_vertex_df(Topo t, const float4* __restrict__ fav,
                                                 const float4* __restrict__ elt,
                                                 const double* __restrict__ reppot, EP ep, EPD epd,
                                                 float4* __restrict__ rk, double* __restrict__ partial, Globals* g) {
  __shared__ float2 red[6][VB];
  __shared__ double redd[6][VB];
  __shared__ bool last;
  int v = blockIdx.x * VB + threadIdx.x;
  df pr[6];
  for (int k = 0; k < 6; ++k) pr[k] = df_make(0.0f);
  if (v < t.nv) {
    int d = t.val[v];
    df A = df_make(0.0f), V = df_make(0.0f), LT = df_make(0.0f), T = df_make(0.0f);
    // slots in groups of six (one group at the usual valence): all loads of
    // a group (16-byte compact records) are issued before the sums, which
    // keep the slot order
    constexpr int G = 6;
    for (int m0 = 0; m0 < d; m0 += G) {
      int4 s[G];
#pragma unroll
      for (int k = 0; k < G; ++k) s[k] = m0 + k < d ? t.slot[(size_t)(m0 + k) * t.nv + v] : make_int4(0, -1, 0, 0);
      float4 av[G], lb[G];
#pragma unroll
      for (int k = 0; k < G; ++k) {
        int f = slot_face(s[k].y);
        av[k] = lb[k] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        if (f >= 0) {
          av[k] = fav[f];
          lb[k] = elt[s[k].z];
        }
      }
#pragma unroll
      for (int k = 0; k < G; ++k) {
        if (slot_face(s[k].y) < 0) continue;
        const df fa = {av[k].x, av[k].y}, fv = {av[k].z, av[k].w}, lt = {lb[k].x, lb[k].y}, tb = {lb[k].z, lb[k].w};
        A += fa;
        V += fv;
        LT += lt;
        if (ep.btype == 0) {
          T += tb;
        } else {
          df q = fa * epd.inv_a0 - df_make(1.0f);
          T += q * q;
        }
      }
    }
    df a = A * third(), c = ldexp2(LT, 0.25f);
    pr[0] = a;
    pr[1] = V * third();
    pr[2] = c;
    pr[3] = ldexp2(c * c, 2.0f) / a;
    pr[4] = T * epd.inv_tdiv;
    double pot = reppot[v];
    pr[5] = pot == 0.0 ? df_make(0.0f) : df_from(pot);
    const df rho = c / a;
    const df kr = epd.kb * rho, kq = epd.kb23 * (rho * rho);
    rk[v] = make_float4(kr.hi, kr.lo, kq.hi, kq.lo);  // (kb rho, 2/3 kb rho^2)
  }
  // fixed-order double-float tree over the block, FP64 across blocks
  for (int k = 0; k < 6; ++k) red[k][threadIdx.x] = make_float2(pr[k].hi, pr[k].lo);
  __syncthreads();
  for (int o = VB / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o)
      for (int k = 0; k < 6; ++k) {
        float2 x = red[k][threadIdx.x], y = red[k][threadIdx.x + o];
        df z = df{x.x, x.y} + df{y.x, y.y};
        red[k][threadIdx.x] = make_float2(z.hi, z.lo);
      }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    for (int k = 0; k < 6; ++k) partial[8 * (size_t)blockIdx.x + k] = df_to(df{red[k][0].x, red[k][0].y});
    __threadfence();
    unsigned int tk = atomicAdd(&g->ticket, 1u);
    last = (tk == gridDim.x - 1);
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  double acc[6] = {0, 0, 0, 0, 0, 0};
  for (int b = threadIdx.x; b < (int)gridDim.x; b += VB)
    for (int k = 0; k < 6; ++k) acc[k] += ((volatile double*)partial)[8 * (size_t)b + k];
  for (int k = 0; k < 6; ++k) redd[k][threadIdx.x] = acc[k];
  __syncthreads();
  for (int o = VB / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o)
      for (int k = 0; k < 6; ++k) redd[k][threadIdx.x] += redd[k][threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    for (int k = 0; k < 6; ++k) g->props[k] = redd[k][0];
    assemble(ep, g);
    g->ticket = 0;
  }
}

__device__ __forceinline__ df cot_df(const FaceDF& F, int c) { return c == 0 ? F.c0 : (c == 1 ? F.c1 : F.c2); }

struct df4 {  // two double-float values
  df a, b;
};
__global__ void __launch_bounds__(256) k_grad_df(Topo t, PosDF X, const FaceDF* __restrict__ fd,
                                                const EdgeDF* __restrict__ ed, const float4* __restrict__ rk,
                                                const double* __restrict__ repg, const Globals* __restrict__ g,
                                                EP ep, EPD epd, double* __restrict__ grad) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= t.nv) return;
  const df gA = {g->gdf[0], g->gdf[1]}, gV = {g->gdf[2], g->gdf[3]}, gC = {g->gdf[4], g->gdf[5]};
  const df hgC = ldexp2(gC, 0.5f);
  const df gV6 = gV * sixth();
  df3 xi = X.at(i);
  // per-vertex weights (kb rho, 2/3 kb rho^2) from k_vertex_df:
  // alpha = gA - 2/3 kb (rho_i^2 + rho_j^2 + rho_k^2), w = gC/2 + kb (rho_i + rho_j)
  auto q_of = [&](int v) {
    const float4 q = rk[v];
    return df4{df{q.x, q.y}, df{q.z, q.w}};
  };
  const df4 qi = q_of(i);
  const df ai = gA - qi.b, wi = hgC + qi.a;
  df3 acc = {df_make(0.0f), df_make(0.0f), df_make(0.0f)};
  // volume term sum_f (x_j x x_k)/6 with x = x_i + d: the x_i x (d_k - d_j)
  // parts telescope around the fan, so only sum d_j x d_k and, for open
  // fans, x_i x sum (d_k - d_j) remain
  df3 vcr = acc, vtel = acc;
  int d = t.val[i];
  if (d > 0) {
    const size_t nv = t.nv;
    int4 sp = t.slot[(size_t)(d - 1) * nv + i];
    df3 dk = X.at(sp.x) - xi;  // x_k - x_i
    df4 qk = q_of(sp.x);
    int4 sc = t.slot[i];
    df3 dj = X.at(sc.x) - xi;
    df4 qj = q_of(sc.x);
    int fcur = slot_face(sc.y);
    // scalar multiples of face normals are summed per face: the dihedral
    // term of edge (i, j) reaches the normal of the next face, so its part
    // is carried to the next slot (the last one wraps to the first face)
    df carry = df_make(0.0f);
    df3 n0 = acc;
    for (int m = 0; m < d; ++m) {
      int4 sn = t.slot[(size_t)((m + 1) == d ? 0 : m + 1) * nv + i];
      int fnx = slot_face(sn.y);
      df carry_next = df_make(0.0f);
      if (fcur >= 0) {
        const FaceDF& Fc = fd[fcur];
        int ci = slot_corner(sc.y);
        df cj = cot_df(Fc, ci == 2 ? 0 : ci + 1);
        df ck = cot_df(Fc, ci == 0 ? 2 : ci - 1);
        df3 n = {Fc.nx, Fc.ny, Fc.nz};
        if (m == 0) n0 = n;
        // face (i, j, k): area and volume terms
        df alpha = (ai - qj.b) - qk.b;
        if (ep.btype == 1) alpha += ldexp2(epd.kt * (Fc.A * epd.inv_a0 - df_make(1.0f)) * epd.inv_a0, 2.0f);
        df3 dkj = dk - dj;
        acc += ldexp2(alpha, 0.5f) * dcross(n, dkj);
        vcr += dcross(dj, dk);
        vtel += dkj;
        // edge (i, j): length and dihedral terms
        const EdgeDF& E = ed[sc.z];
        df w = wi + qj.a;
        df cl = w * E.th;
        if (ep.btype == 0) cl += epd.kt * E.db;
        const df il = E.il.hi < 0.0f ? -E.il : E.il;
        acc += (-(cl * il)) * dj;
        df cn = carry;
        if (E.il.hi > 0.0f) {
          int cin = slot_corner(sn.y);
          cn += w * cj;
          carry_next = w * cot_df(fd[fnx], cin == 0 ? 2 : cin - 1);
        }
        // edge (j, k) opposite i: dihedral term
        if (ed[sc.w].il.hi > 0.0f) cn -= ((hgC + qj.a) + qk.a) * (cj + ck);
        acc += cn * n;
      }
      carry = carry_next;
      dk = dj;
      qk = qj;
      sc = sn;
      fcur = fnx;
      dj = X.at(sn.x) - xi;
      qj = q_of(sn.x);
    }
    acc += carry * n0;  // the last edge's part on the first face
  }
  if (d > 0) acc += gV6 * (vcr + dcross(xi, vtel));
  d3 r = ld3(repg, i);
  grad[3 * i] = df_to(acc.x) + ep.kr * r.x;
  grad[3 * i + 1] = df_to(acc.y) + ep.kr * r.y;
  grad[3 * i + 2] = df_to(acc.z) + ep.kr * r.z;
}

inline int nblk(long n, int b) { return (int)((n + b - 1) / b); }

df host_df(double x) {
  float h = (float)x;
  return {h, (float)(x - (double)h)};
}

}  // namespace

void energy_eval_df(tm_energy* e, tm_mesh* m, const double* P, bool want_grad, double* d_grad, cudaStream_t s,
                    cudaEvent_t* ev) {
  e->ensure(m->nv, m->ne, m->nf);
  size_t nv = std::max(m->nv, 1);
  e->pos32.ensure(3 * nv);
  e->poslo.ensure(3 * nv);
  Topo t = m->topo();
  EP ep = make_ep(e);
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
  PosDF X{e->pos32.get(), e->poslo.get()};
  FaceDF* fd = reinterpret_cast<FaceDF*>(e->face.get());
  EdgeDF* ed = reinterpret_cast<EdgeDF*>(e->edge.get());
  float4* eb = reinterpret_cast<float4*>(e->ebond.get());  // (l theta, bond) per edge, 16 bytes
  float4* fav = reinterpret_cast<float4*>(e->fav.get());    // (area, volume) per face, 16 bytes
  float4* rho = reinterpret_cast<float4*>(e->rho.get());  // (kb rho, 2/3 kb rho^2) per vertex
  if (ev) TM_CUDA(cudaEventRecord(ev[0], s));
  if (m->nv) k_split_df<<<nblk(3L * m->nv, 256), 256, 0, s>>>(3 * m->nv, P, e->pos32.get(), e->poslo.get());
  TM_LAUNCH();
  const bool conc = ev == nullptr;  // repulsion overlaps the face and edge kernels
  if (conc) fork_repulsion(e, m, P, want_grad, s, true);
  if (t.nf) k_face_df<<<nblk(t.nf, 256), 256, 0, s>>>(t, X, fd, fav);
  TM_LAUNCH();
  if (ev) TM_CUDA(cudaEventRecord(ev[1], s));
  int* blist = e->slow.get() + std::max(m->nv, 1) + 1;
  int* bcnt = blist + std::max(m->ne, 1);
  TM_CUDA(cudaMemsetAsync(bcnt, 0, sizeof(int), s));
  if (t.ne) k_edge_df<<<nblk(t.ne, 256), 256, 0, s>>>(t, X, fd, ed, eb, ep, epd, blist, bcnt);
  TM_LAUNCH();
  if (t.ne) k_bond_short_df<<<std::min(nblk(t.ne, 256), 4 * 152), 256, 0, s>>>(ed, eb, ep, epd, blist, bcnt);
  TM_LAUNCH();
  if (ev) TM_CUDA(cudaEventRecord(ev[2], s));
  if (conc)
    join_repulsion(e, s, true);
  else
    fork_repulsion(e, m, P, want_grad, s, false);
  int nb = std::max(1, nblk(t.nv, VB));
  k_vertex_df<<<nb, VB, 0, s>>>(t, fav, eb, e->reppot.get(), ep, epd, rho, e->partials.get(), e->glob.get());
  TM_LAUNCH();
  if (ev) TM_CUDA(cudaEventRecord(ev[3], s));
  if (want_grad && t.nv)
    k_grad_df<<<nblk(t.nv, 256), 256, 0, s>>>(t, X, fd, ed, rho, e->repg.get(), e->glob.get(), ep, epd, d_grad);
  TM_LAUNCH();
  if (ev) TM_CUDA(cudaEventRecord(ev[4], s));
}

}  // namespace tmg
