// FP32-stencil variant of the energy / gradient evaluation
// (tm_energy_set_stencil_precision(e, 1)).
//
// Positions stay FP64 in memory.  Each evaluation splits them into float
// hi + lo parts, so an edge vector (x_b - x_a) = (hi_b - hi_a) + (lo_b - lo_a)
// keeps FP32 relative accuracy even though |x| >> |x_b - x_a|; everything
// local (normals, areas, cotangents, dihedral angles, potentials, the
// gradient gather) is then FP32.  Face volumes use x_a . N_f / 6 (N_f from the
// accurate edge vectors), not the triple product of absolute positions.  The
// dihedral angle is atan2(|n0 x n1|, n0 . n1), accurate for the small angles
// of fine meshes where acosf is not.  The global sums, the penalty assembly
// and the neighbour-pair decisions (exact FP64 threshold) stay FP64, so the
// pair set is the same as in FP64.
#include <algorithm>
#include <cmath>

#include "tm_energy.cuh"
#include "tm_internal.h"
#include "tm_math.cuh"
#include "tm_fp32.cuh"

namespace tmg {

namespace {

using namespace fp32;

// elements [i0, i1) of the 3 n coordinates
__global__ void k_split(int i0, int i1, const double* __restrict__ P, float* __restrict__ hi, float* __restrict__ lo) {
  int i = i0 + blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= i1) return;
  double x = P[i];
  float h = (float)x;
  hi[i] = h;
  lo[i] = (float)(x - (double)h);
}

// faces [f0, f1)
__global__ void k_face32(int f0, int f1, Topo t, Split S, FaceF* __restrict__ fd) {
  int f = f0 + blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= f1) return;
  int a = t.fv[3 * f], b = t.fv[3 * f + 1], c = t.fv[3 * f + 2];
  f3 eab = S.diff(b, a), eac = S.diff(c, a), ebc = S.diff(c, b);
  f3 N = fcross(eab, eac);
  float nn = fnorm(N);
  float inv = 1.0f / nn;
  FaceF F;
  F.nx = N.x * inv;
  F.ny = N.y * inv;
  F.nz = N.z * inv;
  F.A = 0.5f * nn;
  F.V = fdot(S.h(a), N) * (1.0f / 6.0f);
  F.c0 = fdot(eab, eac) * inv;
  F.c1 = -fdot(eab, ebc) * inv;
  F.c2 = fdot(eac, ebc) * inv;
  fd[f] = F;
}

__global__ void k_edge32(Topo t, Split S, const FaceF* __restrict__ fd, EdgeF* __restrict__ ed,
                         float* __restrict__ ebond, EP ep) {
  int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= t.ne) return;
  int4 E = t.edge[e];
  f3 ev = S.diff(E.y, E.x);
  float l = fnorm(ev);
  EdgeF o;
  o.l = l;
  o.th = 0.0f;
  o.flag = 0.0f;
  if (E.z >= 0 && E.w >= 0) {
    FaceF F0 = fd[E.z], F1 = fd[E.w];
    f3 n0 = {F0.nx, F0.ny, F0.nz}, n1 = {F1.nx, F1.ny, F1.nz};
    f3 cr = fcross(n0, n1);
    float a = atan2f(fnorm(cr), fdot(n0, n1));
    o.th = fdot(cr, ev) >= 0.0f ? a : -a;
    o.flag = 1.0f;
  }
  float val = 0.0f, fac = 0.0f;
  if (ep.btype == 0) {
    int r = ep.r;
    float lc0 = (float)ep.lc0, lc1 = (float)ep.lc1;
    if (l > lc0) {
      val = fipow((float)r, r + 1) * fipow(l - lc0, r);
      fac = fipow((float)r, r + 2) * fipow(l - lc0, r - 1);
    } else if (l < lc1) {
      val = expf(l / (l - lc1)) / fipow(l, r);
    }
    if (l < lc1) {
      float lmc = l - lc1;
      fac -= lc1 / (lmc * lmc) + r / l;
      fac /= fipow(l, r);
      fac *= expf(l / lmc);
    }
  }
  o.db = fac;
  ed[e] = o;
  ebond[e] = val;
}

__global__ void __launch_bounds__(VB) k_vertex32(Topo t, const FaceF* __restrict__ fd, const EdgeF* __restrict__ ed,
                                                const float* __restrict__ ebond, const double* __restrict__ reppot,
                                                EP ep, float* __restrict__ rho, double* __restrict__ partial,
                                                Globals* g) {
  __shared__ double red[6][VB];
  __shared__ bool last;
  int v = blockIdx.x * VB + threadIdx.x;
  double pr[6] = {0, 0, 0, 0, 0, 0};
  if (v < t.nv) {
    int d = t.val[v];
    float A = 0, V = 0, LT = 0, T = 0;
    for (int m = 0; m < d; ++m) {
      int4 s = t.slot[(size_t)m * t.nv + v];
      int f = slot_face(s.y);
      if (f < 0) continue;
      float fa = fd[f].A;
      A += fa;
      V += fd[f].V;
      EdgeF E = ed[s.z];
      LT += E.l * E.th;
      if (ep.btype == 0) {
        T += ebond[s.z];
      } else {
        float q = fa / (float)ep.a0 - 1.0f;
        T += q * q;
      }
    }
    float a = A / 3, c = 0.25f * LT;
    pr[0] = a;
    pr[1] = V / 3;
    pr[2] = c;
    pr[3] = 2 * c * c / a;
    pr[4] = T / (float)ep.tdiv;
    pr[5] = reppot[v];
    rho[v] = c / a;
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

__device__ __forceinline__ float cotf_at(const FaceF& F, int c) { return c == 0 ? F.c0 : (c == 1 ? F.c1 : F.c2); }

__global__ void __launch_bounds__(256) k_grad32(Topo t, Split S, const FaceF* __restrict__ fd,
                                               const EdgeF* __restrict__ ed, const float* __restrict__ rho,
                                               const double* __restrict__ repg, const Globals* __restrict__ g, EP ep,
                                               double* __restrict__ grad) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= t.nv) return;
  const float gA = (float)g->gA, gV = (float)g->gV, gC = (float)g->gC;
  const float kb = (float)ep.kb, kt = (float)ep.kt, a0 = (float)ep.a0;
  const float hgC = 0.5f * gC;
  const float kb23 = kb * (2.0f / 3.0f);
  float ri = rho[i];
  f3 acc = (float)ep.kr * f3{(float)repg[3 * i], (float)repg[3 * i + 1], (float)repg[3 * i + 2]};
  int d = t.val[i];
  if (d > 0) {
    const size_t nv = t.nv;
    // neighbour positions relative to x_i (accurate small vectors)
    int4 sp = t.slot[(size_t)(d - 1) * nv + i];
    f3 xk = S.diff(sp.x, i);
    float rk = rho[sp.x];
    int4 sc = t.slot[i];
    f3 xj = S.diff(sc.x, i);
    float rj = rho[sc.x];
    FaceF Fc;
    int fcur = slot_face(sc.y);
    if (fcur >= 0) Fc = fd[fcur];
    f3 xi_abs = S.h(i);
    // normal multiples summed per face; the dihedral part of edge (i, j) on
    // the next face is carried to the next slot
    float carry = 0.0f;
    f3 n0 = {0.0f, 0.0f, 0.0f};
    for (int m = 0; m < d; ++m) {
      int4 sn = t.slot[(size_t)((m + 1) == d ? 0 : m + 1) * nv + i];
      int fnx = slot_face(sn.y);
      FaceF Fn;
      if (fnx >= 0) Fn = fd[fnx];
      float carry_next = 0.0f;
      if (fcur >= 0) {
        int ci = slot_corner(sc.y);
        float cj = cotf_at(Fc, ci == 2 ? 0 : ci + 1);
        float ck = cotf_at(Fc, ci == 0 ? 2 : ci - 1);
        f3 n = {Fc.nx, Fc.ny, Fc.nz};
        if (m == 0) n0 = n;
        float alpha = gA - kb23 * (ri * ri + rj * rj + rk * rk);
        if (ep.btype == 1) alpha += kt * 2.0f * (Fc.A / a0 - 1.0f) / a0;
        acc += (0.5f * alpha) * fcross(n, xk - xj);
        // (x_j x x_k)/6 with x = x_i + d: x_i x (d_k - d_j) + d_j x d_k
        f3 vj = fcross(xi_abs, xk - xj) + fcross(xj, xk);
        acc += (gV * (1.0f / 6.0f)) * vj;
        EdgeF E = ed[sc.z];
        float w = hgC + kb * (ri + rj);
        float cl = w * E.th + (ep.btype == 0 ? kt * E.db : 0.0f);
        acc += (-cl / E.l) * xj;
        float cn = carry;
        if (E.flag != 0.0f) {
          int cin = slot_corner(sn.y);
          cn += w * cj;
          carry_next = w * cotf_at(Fn, cin == 0 ? 2 : cin - 1);
        }
        if (ed[sc.w].flag != 0.0f) cn -= (hgC + kb * (rj + rk)) * (cj + ck);
        acc += cn * n;
      }
      carry = carry_next;
      xk = xj;
      rk = rj;
      sc = sn;
      fcur = fnx;
      Fc = Fn;
      xj = S.diff(sn.x, i);
      rj = rho[sn.x];
    }
    acc += carry * n0;
  }
  grad[3 * i] = acc.x;
  grad[3 * i + 1] = acc.y;
  grad[3 * i + 2] = acc.z;
}

// ---- batch of replicas (disjoint-union mesh, replica-aligned blocks) -----
// Same arithmetic as the single-mesh FP32 kernels; the parameters and the
// global sums are per replica (vrep: vertex -> replica, -1 for padding).

// edges [e0, e1)
__global__ void k_edge32b(int e0, int e1, Topo t, Split S, const FaceF* __restrict__ fd, EdgeF* __restrict__ ed,
                          float* __restrict__ ebond, const EP* __restrict__ eps, const int* __restrict__ vrep) {
  int e = e0 + blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= e1) return;
  int4 E = t.edge[e];
  const EP& ep = eps[vrep[E.x]];
  f3 ev = S.diff(E.y, E.x);
  float l = fnorm(ev);
  EdgeF o;
  o.l = l;
  o.th = 0.0f;
  o.flag = 0.0f;
  if (E.z >= 0 && E.w >= 0) {
    FaceF F0 = fd[E.z], F1 = fd[E.w];
    f3 n0 = {F0.nx, F0.ny, F0.nz}, n1 = {F1.nx, F1.ny, F1.nz};
    f3 cr = fcross(n0, n1);
    float a = atan2f(fnorm(cr), fdot(n0, n1));
    o.th = fdot(cr, ev) >= 0.0f ? a : -a;
    o.flag = 1.0f;
  }
  float val = 0.0f, fac = 0.0f;
  if (ep.btype == 0) {
    int r = ep.r;
    float lc0 = (float)ep.lc0, lc1 = (float)ep.lc1;
    if (l > lc0) {
      val = fipow((float)r, r + 1) * fipow(l - lc0, r);
      fac = fipow((float)r, r + 2) * fipow(l - lc0, r - 1);
    } else if (l < lc1) {
      val = expf(l / (l - lc1)) / fipow(l, r);
    }
    if (l < lc1) {
      float lmc = l - lc1;
      fac -= lc1 / (lmc * lmc) + r / l;
      fac /= fipow(l, r);
      fac *= expf(l / lmc);
    }
  }
  o.db = fac;
  ed[e] = o;
  ebond[e] = val;
}

__global__ void __launch_bounds__(VB) k_vertex32b(Topo t, const FaceF* __restrict__ fd, const EdgeF* __restrict__ ed,
                                                 const float* __restrict__ ebond, const double* __restrict__ reppot,
                                                 const EP* __restrict__ eps, const int* __restrict__ vrep,
                                                 const int2* __restrict__ rblocks, float* __restrict__ rho,
                                                 double* __restrict__ partial, Globals* gs) {
  __shared__ double red[6][VB];
  __shared__ bool last;
  const int rep = vrep[blockIdx.x * VB];  // blocks never straddle replicas
  const EP& ep = eps[rep];
  int v = blockIdx.x * VB + threadIdx.x;
  double pr[6] = {0, 0, 0, 0, 0, 0};
  if (v < t.nv && vrep[v] >= 0) {
    int d = t.val[v];
    float A = 0, V = 0, LT = 0, T = 0;
    for (int m = 0; m < d; ++m) {
      int4 s = t.slot[(size_t)m * t.nv + v];
      int f = slot_face(s.y);
      if (f < 0) continue;
      float fa = fd[f].A;
      A += fa;
      V += fd[f].V;
      EdgeF E = ed[s.z];
      LT += E.l * E.th;
      if (ep.btype == 0) {
        T += ebond[s.z];
      } else {
        float q = fa / (float)ep.a0 - 1.0f;
        T += q * q;
      }
    }
    float a = A / 3, c = 0.25f * LT;
    pr[0] = a;
    pr[1] = V / 3;
    pr[2] = c;
    pr[3] = 2 * c * c / a;
    pr[4] = T / (float)ep.tdiv;
    pr[5] = reppot[v];
    rho[v] = c / a;
  }
  for (int k = 0; k < 6; ++k) red[k][threadIdx.x] = pr[k];
  __syncthreads();
  for (int o = VB / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o)
      for (int k = 0; k < 6; ++k) red[k][threadIdx.x] += red[k][threadIdx.x + o];
    __syncthreads();
  }
  Globals* g = gs + rep;
  const int2 rb = rblocks[rep];
  if (threadIdx.x == 0) {
    for (int k = 0; k < 6; ++k) partial[8 * (size_t)blockIdx.x + k] = red[k][0];
    __threadfence();
    unsigned int tk = atomicAdd(&g->ticket, 1u);
    last = (tk == (unsigned)(rb.y - rb.x - 1));
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  double acc[6] = {0, 0, 0, 0, 0, 0};
  for (int b = rb.x + threadIdx.x; b < rb.y; b += VB)
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

// vertices [v0, v1)
__global__ void __launch_bounds__(256) k_grad32b(int v0, int v1, Topo t, Split S, const FaceF* __restrict__ fd,
                                                const EdgeF* __restrict__ ed, const float* __restrict__ rho,
                                                const double* __restrict__ repg, const Globals* __restrict__ gs,
                                                const EP* __restrict__ eps, const int* __restrict__ vrep,
                                                double* __restrict__ grad) {
  int i = v0 + blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= v1) return;
  int rep = vrep[i];
  if (rep < 0) {
    grad[3 * i] = grad[3 * i + 1] = grad[3 * i + 2] = 0.0;
    return;
  }
  const EP& ep = eps[rep];
  const Globals* g = gs + rep;
  const float gA = (float)g->gA, gV = (float)g->gV, gC = (float)g->gC;
  const float kb = (float)ep.kb, kt = (float)ep.kt, a0 = (float)ep.a0;
  const float hgC = 0.5f * gC;
  const float kb23 = kb * (2.0f / 3.0f);
  float ri = rho[i];
  f3 acc = (float)ep.kr * f3{(float)repg[3 * i], (float)repg[3 * i + 1], (float)repg[3 * i + 2]};
  int d = t.val[i];
  if (d > 0) {
    const size_t nv = t.nv;
    int4 sp = t.slot[(size_t)(d - 1) * nv + i];
    f3 xk = S.diff(sp.x, i);
    float rk = rho[sp.x];
    int4 sc = t.slot[i];
    f3 xj = S.diff(sc.x, i);
    float rj = rho[sc.x];
    FaceF Fc;
    int fcur = slot_face(sc.y);
    if (fcur >= 0) Fc = fd[fcur];
    f3 xi_abs = S.h(i);
    // normal multiples summed per face; the dihedral part of edge (i, j) on
    // the next face is carried to the next slot
    float carry = 0.0f;
    f3 n0 = {0.0f, 0.0f, 0.0f};
    for (int m = 0; m < d; ++m) {
      int4 sn = t.slot[(size_t)((m + 1) == d ? 0 : m + 1) * nv + i];
      int fnx = slot_face(sn.y);
      FaceF Fn;
      if (fnx >= 0) Fn = fd[fnx];
      float carry_next = 0.0f;
      if (fcur >= 0) {
        int ci = slot_corner(sc.y);
        float cj = cotf_at(Fc, ci == 2 ? 0 : ci + 1);
        float ck = cotf_at(Fc, ci == 0 ? 2 : ci - 1);
        f3 n = {Fc.nx, Fc.ny, Fc.nz};
        if (m == 0) n0 = n;
        float alpha = gA - kb23 * (ri * ri + rj * rj + rk * rk);
        if (ep.btype == 1) alpha += kt * 2.0f * (Fc.A / a0 - 1.0f) / a0;
        acc += (0.5f * alpha) * fcross(n, xk - xj);
        f3 vj = fcross(xi_abs, xk - xj) + fcross(xj, xk);
        acc += (gV * (1.0f / 6.0f)) * vj;
        EdgeF E = ed[sc.z];
        float w = hgC + kb * (ri + rj);
        float cl = w * E.th + (ep.btype == 0 ? kt * E.db : 0.0f);
        acc += (-cl / E.l) * xj;
        float cn = carry;
        if (E.flag != 0.0f) {
          int cin = slot_corner(sn.y);
          cn += w * cj;
          carry_next = w * cotf_at(Fn, cin == 0 ? 2 : cin - 1);
        }
        if (ed[sc.w].flag != 0.0f) cn -= (hgC + kb * (rj + rk)) * (cj + ck);
        acc += cn * n;
      }
      carry = carry_next;
      xk = xj;
      rk = rj;
      sc = sn;
      fcur = fnx;
      Fc = Fn;
      xj = S.diff(sn.x, i);
      rj = rho[sn.x];
    }
    acc += carry * n0;
  }
  grad[3 * i] = acc.x;
  grad[3 * i + 1] = acc.y;
  grad[3 * i + 2] = acc.z;
}

inline int nblk(long n, int b) { return (int)((n + b - 1) / b); }

}  // namespace

void energy_eval32(tm_energy* e, tm_mesh* m, const double* P, bool want_grad, bool want_vprops, double* d_grad,
                   cudaStream_t s, cudaEvent_t* ev) {
  e->ensure(m->nv, m->ne, m->nf);
  size_t nv = std::max(m->nv, 1), ne = std::max(m->ne, 1), nf = std::max(m->nf, 1);
  // FP32 records live in the FP64 buffers (they are smaller)
  Topo t = m->topo();
  EP ep = make_ep(e);
  e->pos32.ensure(3 * nv);
  float* lo = reinterpret_cast<float*>(e->vprops.get());  // 6*nv doubles >= 3*nv floats
  Split S{e->pos32.get(), lo};
  FaceF* fd = reinterpret_cast<FaceF*>(e->face.get());
  EdgeF* ed = reinterpret_cast<EdgeF*>(e->edge.get());
  float* eb = reinterpret_cast<float*>(e->ebond.get());
  float* rho = reinterpret_cast<float*>(e->rho.get());
  double* repg = e->repg.get();
  (void)nf;
  (void)ne;
  if (ev) TM_CUDA(cudaEventRecord(ev[0], s));
  if (m->nv) k_split<<<nblk(3L * m->nv, 256), 256, 0, s>>>(0, 3 * m->nv, P, e->pos32.get(), lo);
  TM_LAUNCH();
  const bool conc = ev == nullptr;  // repulsion overlaps the face and edge kernels
  if (conc) fork_repulsion(e, m, P, want_grad, s, true);
  if (t.nf) k_face32<<<nblk(t.nf, 256), 256, 0, s>>>(0, t.nf, t, S, fd);
  TM_LAUNCH();
  if (ev) TM_CUDA(cudaEventRecord(ev[1], s));
  if (t.ne) k_edge32<<<nblk(t.ne, 256), 256, 0, s>>>(t, S, fd, ed, eb, ep);
  TM_LAUNCH();
  if (ev) TM_CUDA(cudaEventRecord(ev[2], s));
  if (conc)
    join_repulsion(e, s, true);
  else
    fork_repulsion(e, m, P, want_grad, s, false);
  (void)repg;
  int nb = std::max(1, nblk(t.nv, VB));
  (void)want_vprops;
  k_vertex32<<<nb, VB, 0, s>>>(t, fd, ed, eb, e->reppot.get(), ep, rho, e->partials.get(), e->glob.get());
  TM_LAUNCH();
  if (ev) TM_CUDA(cudaEventRecord(ev[3], s));
  if (want_grad && t.nv) k_grad32<<<nblk(t.nv, 256), 256, 0, s>>>(t, S, fd, ed, rho, repg, e->glob.get(), ep, d_grad);
  TM_LAUNCH();
  if (ev) TM_CUDA(cudaEventRecord(ev[4], s));
}

// The local terms of the energy only (bending and repulsion weights set to
// zero, no neighbour pass) with FP32 stencils: the exact part of the
// surrogate force.  Leaves the FP32 face / edge records, rho = c/a per vertex
// and the split positions (e->pos32, e->poslo) filled for the caller.
void energy_eval32_local(tm_energy* e, tm_mesh* m, const double* P, double* d_grad, cudaStream_t s) {
  e->ensure(m->nv, m->ne, m->nf);
  size_t nv = std::max(m->nv, 1);
  Topo t = m->topo();
  EP ep = make_ep(e);
  ep.kb = 0.0;
  ep.kr = 0.0;
  e->pos32.ensure(3 * nv);
  e->poslo.ensure(3 * nv);
  Split S{e->pos32.get(), e->poslo.get()};
  FaceF* fd = reinterpret_cast<FaceF*>(e->face.get());
  EdgeF* ed = reinterpret_cast<EdgeF*>(e->edge.get());
  float* eb = reinterpret_cast<float*>(e->ebond.get());
  float* rho = reinterpret_cast<float*>(e->rho.get());
  TM_CUDA(cudaMemsetAsync(e->reppot.get(), 0, sizeof(double) * nv, s));
  TM_CUDA(cudaMemsetAsync(e->repg.get(), 0, sizeof(double) * 3 * nv, s));
  if (m->nv) k_split<<<nblk(3L * m->nv, 256), 256, 0, s>>>(0, 3 * m->nv, P, e->pos32.get(), e->poslo.get());
  TM_LAUNCH();
  if (t.nf) k_face32<<<nblk(t.nf, 256), 256, 0, s>>>(0, t.nf, t, S, fd);
  TM_LAUNCH();
  if (t.ne) k_edge32<<<nblk(t.ne, 256), 256, 0, s>>>(t, S, fd, ed, eb, ep);
  TM_LAUNCH();
  int nb = std::max(1, nblk(t.nv, VB));
  k_vertex32<<<nb, VB, 0, s>>>(t, fd, ed, eb, e->reppot.get(), ep, rho, e->partials.get(), e->glob.get());
  TM_LAUNCH();
  if (t.nv) k_grad32<<<nblk(t.nv, 256), 256, 0, s>>>(t, S, fd, ed, rho, e->repg.get(), e->glob.get(), ep, d_grad);
  TM_LAUNCH();
}

// One element kernel of one size class of a batch: which 0 split, 1 face,
// 2 edge, 3 gradient, with block size blk, on stream s.
void batch32_class_kernel(int which, const BatchClass& c, int blk, tm_energy* e, tm_mesh* m, const double* P,
                          double* d_grad, const EP* eps, const int* vrep, const Globals* gs, cudaStream_t s) {
  Topo t = m->topo();
  Split S{e->pos32.get(), e->poslo.get()};
  FaceF* fd = reinterpret_cast<FaceF*>(e->face.get());
  EdgeF* ed = reinterpret_cast<EdgeF*>(e->edge.get());
  float* eb = reinterpret_cast<float*>(e->ebond.get());
  float* rho = reinterpret_cast<float*>(e->rho.get());
  if (which == 0 && c.v1 > c.v0)
    k_split<<<nblk(3L * (c.v1 - c.v0), blk), blk, 0, s>>>(3 * c.v0, 3 * c.v1, P, e->pos32.get(), e->poslo.get());
  if (which == 1 && c.f1 > c.f0) k_face32<<<nblk(c.f1 - c.f0, blk), blk, 0, s>>>(c.f0, c.f1, t, S, fd);
  if (which == 2 && c.e1 > c.e0)
    k_edge32b<<<nblk(c.e1 - c.e0, blk), blk, 0, s>>>(c.e0, c.e1, t, S, fd, ed, eb, eps, vrep);
  if (which == 3 && c.v1 > c.v0)
    k_grad32b<<<nblk(c.v1 - c.v0, blk), blk, 0, s>>>(c.v0, c.v1, t, S, fd, ed, rho, e->repg.get(), gs, eps, vrep,
                                                      d_grad);
  TM_LAUNCH();
}

// The batch's evaluation: per size class (consecutive replicas of similar
// size, each with its own tuned block sizes) the split, face and edge
// kernels, then the repulsion and the vertex stage for all replicas, then
// the gradient per class.  With side streams the classes' kernels run
// side by side (fork and join events), so the small replicas' launches fill
// the SMs the large ones leave idle.
void energy_eval_batch32(tm_energy* e, tm_mesh* m, const double* P, double* d_grad, const EP* eps,
                         const int* vrep, const int2* rblocks, Globals* gs, const BatchClass* cls, int ncls,
                         const BatchStreams* bs, cudaStream_t s) {
  e->ensure(m->nv, m->ne, m->nf);
  size_t nv = std::max(m->nv, 1);
  Topo t = m->topo();
  e->pos32.ensure(3 * nv);
  e->poslo.ensure(3 * nv);
  FaceF* fd = reinterpret_cast<FaceF*>(e->face.get());
  EdgeF* ed = reinterpret_cast<EdgeF*>(e->edge.get());
  float* eb = reinterpret_cast<float*>(e->ebond.get());
  float* rho = reinterpret_cast<float*>(e->rho.get());
  const bool side = bs && ncls > 1;
  auto stream_of = [&](int c) { return side ? bs->cs[c] : s; };
  auto fork = [&](int k) {
    if (!side) return;
    TM_CUDA(cudaEventRecord(bs->fork[k], s));
    for (int c = 0; c < ncls; ++c) TM_CUDA(cudaStreamWaitEvent(bs->cs[c], bs->fork[k], 0));
  };
  auto join = [&]() {
    if (!side) return;
    for (int c = 0; c < ncls; ++c) {
      TM_CUDA(cudaEventRecord(bs->join[c], bs->cs[c]));
      TM_CUDA(cudaStreamWaitEvent(s, bs->join[c], 0));
    }
  };
  fork(0);
  for (int c = 0; c < ncls; ++c)
    for (int k = 0; k < 3; ++k)
      batch32_class_kernel(k, cls[c], cls[c].blk[k], e, m, P, d_grad, eps, vrep, gs, stream_of(c));
  join();
  repulsion_eval(e, m, P, e->pos32.get(), true, e->reppot.get(), e->repg.get(), e->slow.get(),
                 e->slow.get() + std::max(m->nv, 1), s, eps);
  int nb = std::max(1, nblk(t.nv, VB));
  k_vertex32b<<<nb, VB, 0, s>>>(t, fd, ed, eb, e->reppot.get(), eps, vrep, rblocks, rho, e->partials.get(), gs);
  TM_LAUNCH();
  fork(1);
  for (int c = 0; c < ncls; ++c)
    batch32_class_kernel(3, cls[c], cls[c].blk[3], e, m, P, d_grad, eps, vrep, gs, stream_of(c));
  join();
}

}  // namespace tmg
