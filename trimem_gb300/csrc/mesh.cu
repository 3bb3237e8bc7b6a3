// Mesh handle: half-edge construction on the host, flat device tables, the
// geometry primitives and the mesh utilities.
//
// Device layout (all int32 / float64, structure-of-arrays):
//   positions      nv x 3 (x,y,z interleaved)
//   halfedges      to / next / face per halfedge, edge e owns 2e and 2e+1
//   faces          fv (3 per face, starting at to(fhe[f]))
//   edges          (from, to, face of 2e, face of 2e+1)
//   vertex rings   slot-major [TM_MAXVAL][nv] int4 slots + neighbour ids
// Flips edit the halfedge arrays; the face/edge/ring tables are rebuilt
// from them afterwards.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <unordered_map>

#include "tm_internal.h"
#include "tm_math.cuh"
#include "tm_topo.cuh"
#include <memory>

using namespace tmg;

#define TM_API_BEGIN try {
#define TM_API_END                              \
  }                                             \
  catch (const tmg::Error& e) {                 \
    tmg::set_last_error(e.what());              \
    return e.code;                              \
  }                                             \
  catch (const std::exception& e) {             \
    tmg::set_last_error(e.what());              \
    return TM_ERR_ARG;                          \
  }                                             \
  return TM_OK;

namespace {

__global__ void k_faces(int nf, const int* to, const int* next, const int* fhe, int* fv) {
  int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= nf) return;
  int h = fhe[f];
  int h1 = next[h];
  fv[3 * f] = to[h];
  fv[3 * f + 1] = to[h1];
  fv[3 * f + 2] = to[next[h1]];
}

__global__ void k_edges(int ne, const int* to, const int* face, int4* edge) {
  int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= ne) return;
  edge[e] = make_int4(to[2 * e + 1], to[2 * e], face[2 * e], face[2 * e + 1]);
}

__global__ void k_rings(TopoW t, int* status) {
  int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= t.nv) return;
  if (!ring_row(t, v)) atomicExch(status, TM_ERR_TOPOLOGY);
}

// ---- geometry primitives, following src/mesh_util.h term by term ---------
struct HE {
  const int* to;
  const int* next;
  const int* face;
  const double* P;
  int nh;
  __device__ int from(int h) const { return to[h ^ 1]; }
  __device__ int prev(int h) const {
    int g = h;
    for (int k = 0; k < nh && next[g] != h; ++k) g = next[g];
    return g;
  }
  __device__ d3 pt(int v) const { return ld3(P, v); }
  __device__ d3 ev(int h) const { return pt(to[h]) - pt(from(h)); }
  __device__ d3 sector_normal(int h) const { return cross(ev(next[h]), ev(h ^ 1)); }
  __device__ double sector_angle(int h) const {
    d3 a = ev(next[h]), b = ev(h ^ 1);
    double den = norm(a) * norm(b);
    if (den == 0.0) return 0.0;
    double c = fmin(1.0, fmax(-1.0, dot(a, b) / den));
    return acos(c);
  }
  __device__ double dihedral(int h) const {
    if (face[h] < 0 || face[h ^ 1] < 0) return 0.0;
    d3 n0 = sector_normal(h), n1 = sector_normal(h ^ 1);
    double den = norm(n0) * norm(n1);
    if (den == 0.0) return 0.0;
    double c = fmin(1.0, fmax(-1.0, dot(n0, n1) / den));
    double a = acos(c);
    return dot(cross(n0, n1), ev(h)) >= 0.0 ? a : -a;
  }
};

// out layout: [0] l, [1..6] dl (2x3), [7] A, [8..16] dA, [17] V, [18..26] dV,
// [27] theta, [28..39] dtheta (4x3)
__global__ void k_prims(HE m, int h, double* out) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  d3 e = m.ev(h);
  double l = norm(e);
  d3 u = (1.0 / l) * e;
  out[0] = l;
  st3(out + 1, 0, -u);
  st3(out + 1, 1, u);
  d3 n = m.sector_normal(h);
  out[7] = norm(n) / 2;
  d3 nh = (1.0 / norm(n)) * n;
  nh = (1.0 / norm(nh)) * nh;
  int hp = m.prev(h);
  st3(out + 8, 0, 0.5 * cross(nh, m.ev(m.next[h])));
  st3(out + 8, 1, 0.5 * cross(nh, m.ev(hp)));
  st3(out + 8, 2, 0.5 * cross(nh, m.ev(h)));
  d3 p0 = m.pt(m.from(h)), p1 = m.pt(m.to[h]), p2 = m.pt(m.to[m.next[h]]);
  out[17] = dot(cross(p1, p2), p0) / 6;
  st3(out + 18, 0, (1.0 / 6) * cross(p1, p2));
  st3(out + 18, 1, (1.0 / 6) * cross(p2, p0));
  st3(out + 18, 2, (1.0 / 6) * cross(p0, p1));
  out[27] = m.dihedral(h);
  if (m.face[h] < 0 || m.face[h ^ 1] < 0) {
    for (int k = 0; k < 12; ++k) out[28 + k] = 0.0;
    return;
  }
  d3 n0 = m.sector_normal(h), n1 = m.sector_normal(h ^ 1);
  n0 = (1.0 / norm(n0)) * n0;
  n1 = (1.0 / norm(n1)) * n1;
  double a01 = m.sector_angle(m.prev(h));
  double a03 = m.sector_angle(h);
  double a02 = m.sector_angle(h ^ 1);
  double a04 = m.sector_angle(m.prev(h ^ 1));
  double c1 = 1.0 / tan(a01), c2 = 1.0 / tan(a02), c3 = 1.0 / tan(a03), c4 = 1.0 / tan(a04);
  st3(out + 28, 0, (1.0 / l) * (c3 * n0 + c4 * n1));
  st3(out + 28, 1, (1.0 / l) * (c1 * n0 + c2 * n1));
  st3(out + 28, 2, (-(c1 + c3) / l) * n0);
  st3(out + 28, 3, (-(c2 + c4) / l) * n1);
}

// ---- invariants ----------------------------------------------------------
__global__ void k_check(Topo t, int* status) {
  int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= t.nv) return;
  int d = t.val[v];
  if (d > 0 && d < 3) atomicMin(status, -7);
  for (int m = 0; m < d; ++m) {
    int4 s = t.slot[(size_t)m * t.nv + v];
    if (s.y == -1) atomicMin(status, -9);  // open fan
    if (t.to[2 * s.z] != s.x && t.to[2 * s.z + 1] != s.x) atomicMin(status, -5);
    for (int k = m + 1; k < d; ++k)
      if (t.nbr[(size_t)k * t.nv + v] == s.x) atomicMin(status, -4);  // double edge
  }
}
__global__ void k_check_faces(Topo t, int* status) {
  int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= t.nf) return;
  int h = t.fhe[f];
  if (t.face[h] != f || t.next[t.next[t.next[h]]] != h) atomicMin(status, -2);
  int a = t.fv[3 * f], b = t.fv[3 * f + 1], c = t.fv[3 * f + 2];
  if (a == b || b == c || a == c) atomicMin(status, -1);
}

// ---- utilities (src/util.cpp) with a fixed-order reduction ---------------
__global__ void k_sum_terms(int n, int what, Topo t, const double* P, double* partial) {
  __shared__ double s[256];
  double acc = 0.0;
  int per = (n + gridDim.x - 1) / gridDim.x;
  int lo = blockIdx.x * per, hi = min(n, lo + per);
  for (int i = lo + threadIdx.x; i < hi; i += blockDim.x) {
    if (what == 0) {  // face area
      int a = t.fv[3 * i], b = t.fv[3 * i + 1], c = t.fv[3 * i + 2];
      d3 pa = ld3(P, a), pb = ld3(P, b), pc = ld3(P, c);
      acc += norm(cross(pc - pb, pa - pb)) / 2;
    } else {  // edge length
      int4 e = t.edge[i];
      acc += norm(ld3(P, e.y) - ld3(P, e.x));
    }
  }
  s[threadIdx.x] = acc;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) s[threadIdx.x] += s[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) partial[blockIdx.x] = s[0];
}
__global__ void k_sum_final(int nb, const double* partial, double* out) {
  __shared__ double s[256];
  double acc = 0.0;
  for (int i = threadIdx.x; i < nb; i += blockDim.x) acc += partial[i];
  s[threadIdx.x] = acc;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) s[threadIdx.x] += s[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = s[0];
}

inline int nblk(long n, int b) { return (int)((n + b - 1) / b); }

}  // namespace

// --------------------------------------------------------------------------
// tm_mesh methods
// --------------------------------------------------------------------------
Topo tm_mesh::topo() const {
  Topo t;
  t.nv = nv;
  t.ne = ne;
  t.nf = nf;
  t.to = d_to.get();
  t.next = d_next.get();
  t.face = d_face.get();
  t.vout = d_vout.get();
  t.fhe = d_fhe.get();
  t.slot = d_slot.get();
  t.nbr = d_nbr.get();
  t.val = d_val.get();
  t.fv = d_fv.get();
  t.edge = d_edge.get();
  return t;
}

TopoW tm_mesh::topo_w() {
  TopoW t;
  t.nv = nv;
  t.ne = ne;
  t.nf = nf;
  t.to = d_to.get();
  t.next = d_next.get();
  t.face = d_face.get();
  t.vout = d_vout.get();
  t.fhe = d_fhe.get();
  t.slot = d_slot.get();
  t.nbr = d_nbr.get();
  t.val = d_val.get();
  t.fv = d_fv.get();
  t.edge = d_edge.get();
  return t;
}

void tm_mesh::rebuild_tables(cudaStream_t s) {
  if (nf > 0) k_faces<<<nblk(nf, 256), 256, 0, s>>>(nf, d_to.get(), d_next.get(), d_fhe.get(), d_fv.get());
  TM_LAUNCH();
  if (ne > 0) k_edges<<<nblk(ne, 256), 256, 0, s>>>(ne, d_to.get(), d_face.get(), d_edge.get());
  TM_LAUNCH();
  TM_CUDA(cudaMemsetAsync(d_status.get(), 0, sizeof(int), s));
  if (nv > 0) k_rings<<<nblk(nv, 256), 256, 0, s>>>(topo_w(), d_status.get());
  TM_LAUNCH();
  int st = 0;
  TM_CUDA(cudaMemcpyAsync(&st, d_status.get(), sizeof(int), cudaMemcpyDeviceToHost, s));
  TM_CUDA(cudaStreamSynchronize(s));
  if (st != 0) fail(TM_ERR_TOPOLOGY, "vertex valence exceeds TM_MAXVAL (" + std::to_string(TM_MAXVAL) + ")");
}

void tm_mesh::upload_points(cudaStream_t s) {
  if (nv > 0) TM_CUDA(cudaMemcpyAsync(d_pts.get(), h_pts, sizeof(double) * 3 * nv, cudaMemcpyHostToDevice, s));
}

void tm_mesh::sync_host_topology() {
  if (!host_topo_stale) return;
  int nh = 2 * ne;
  TM_CUDA(cudaStreamSynchronize(stream));
  TM_CUDA(cudaMemcpy(h_to.data(), d_to.get(), sizeof(int) * nh, cudaMemcpyDeviceToHost));
  TM_CUDA(cudaMemcpy(h_next.data(), d_next.get(), sizeof(int) * nh, cudaMemcpyDeviceToHost));
  TM_CUDA(cudaMemcpy(h_face.data(), d_face.get(), sizeof(int) * nh, cudaMemcpyDeviceToHost));
  TM_CUDA(cudaMemcpy(h_vout.data(), d_vout.get(), sizeof(int) * nv, cudaMemcpyDeviceToHost));
  TM_CUDA(cudaMemcpy(h_fhe.data(), d_fhe.get(), sizeof(int) * nf, cudaMemcpyDeviceToHost));
  host_topo_stale = false;
}

tm_mesh::~tm_mesh() {
  if (h_pts) cudaFreeHost(h_pts);
  if (stream) cudaStreamDestroy(stream);
}

// Half-edge construction with the add_face semantics of the reference's mesh
// (src/mesh_py.cpp:12-70): new edges are numbered in order of first
// appearance, halfedge 2e points along that appearance, a face keeps its
// v2->v0 halfedge (so fv_indices returns the input order), and a face whose
// directed edge is already taken is skipped.  Boundary halfedges are linked
// into boundary loops; each vertex's outgoing halfedges must form one fan.
static void build_halfedges(tm_mesh* m, const double* pts, int64_t nv, const int32_t* faces, int64_t nf) {
  m->nv = (int)nv;
  m->h_vout.assign(nv, -1);
  if (nv < 3) {
    m->ne = m->nf = 0;
    return;
  }
  std::unordered_map<uint64_t, int> emap;
  emap.reserve((size_t)nf * 2);
  auto key = [](int a, int b) {
    return ((uint64_t)(uint32_t)std::min(a, b) << 32) | (uint32_t)std::max(a, b);
  };
  auto& to = m->h_to;
  auto& nx = m->h_next;
  auto& fc = m->h_face;
  for (int64_t f = 0; f < nf; ++f) {
    int v[3], n = 0;
    for (int k = 0; k < 3; ++k) {
      int x = faces[3 * f + k];
      if (x >= 0 && x < nv) v[n++] = x;
    }
    if (n < 3 || v[0] == v[1] || v[1] == v[2] || v[0] == v[2]) continue;
    int hs[3];
    bool taken = false;
    for (int k = 0; k < 3; ++k) {
      auto it = emap.find(key(v[k], v[(k + 1) % 3]));
      hs[k] = -1;
      if (it != emap.end()) {
        int h = 2 * it->second;
        hs[k] = to[h] == v[(k + 1) % 3] ? h : h + 1;
        if (fc[hs[k]] >= 0) taken = true;
      }
    }
    if (taken) continue;
    for (int k = 0; k < 3; ++k)
      if (hs[k] < 0) {
        int e = (int)(to.size() / 2);
        emap[key(v[k], v[(k + 1) % 3])] = e;
        to.push_back(v[(k + 1) % 3]);
        to.push_back(v[k]);
        nx.push_back(-1);
        nx.push_back(-1);
        fc.push_back(-1);
        fc.push_back(-1);
        hs[k] = 2 * e;
      }
    int fid = (int)m->h_fhe.size();
    for (int k = 0; k < 3; ++k) {
      nx[hs[k]] = hs[(k + 1) % 3];
      fc[hs[k]] = fid;
    }
    m->h_fhe.push_back(hs[2]);
  }
  int nh = (int)to.size();
  m->ne = nh / 2;
  m->nf = (int)m->h_fhe.size();
  if ((int64_t)m->nf >= (1 << 30)) fail(TM_ERR_ARG, "too many faces");
  std::vector<int> bout(nv, -1);
  m->closed = true;
  for (int h = 0; h < nh; ++h)
    if (fc[h] < 0) {
      m->closed = false;
      int a = to[h ^ 1];
      if (bout[a] >= 0) fail(TM_ERR_TOPOLOGY, "non-manifold vertex (several boundary fans)");
      bout[a] = h;
    }
  for (int h = 0; h < nh; ++h)
    if (fc[h] < 0) nx[h] = bout[to[h]];
  for (int h = 0; h < nh; ++h) {
    int a = to[h ^ 1];
    if (m->h_vout[a] < 0) m->h_vout[a] = h;
  }
  for (int v = 0; v < nv; ++v)
    if (bout[v] >= 0) m->h_vout[v] = bout[v];
  std::vector<int> deg(nv, 0);
  for (int h = 0; h < nh; ++h) deg[to[h ^ 1]]++;
  for (int v = 0; v < nv; ++v) {
    int h0 = m->h_vout[v];
    if (h0 < 0) continue;
    int c = 0, h = h0;
    do {
      ++c;
      h = nx[h ^ 1];
    } while (h != h0 && c <= deg[v]);
    if (c != deg[v]) fail(TM_ERR_TOPOLOGY, "non-manifold vertex");
    if (deg[v] > TM_MAXVAL)
      fail(TM_ERR_TOPOLOGY, "vertex valence " + std::to_string(deg[v]) + " exceeds TM_MAXVAL");
  }
}

static void upload_topology(tm_mesh* m) {
  int nh = 2 * m->ne;
  m->d_pts.ensure(3 * (size_t)m->nv);
  m->d_to.ensure(nh);
  m->d_next.ensure(nh);
  m->d_face.ensure(nh);
  m->d_vout.ensure(m->nv);
  m->d_fhe.ensure(m->nf);
  m->d_slot.ensure((size_t)TM_MAXVAL * m->nv);
  m->d_nbr.ensure((size_t)TM_MAXVAL * m->nv);
  m->d_val.ensure(m->nv);
  m->d_fv.ensure(3 * (size_t)m->nf);
  m->d_edge.ensure(m->ne);
  m->d_scratch.ensure(4096);
  m->d_status.ensure(4);
  m->d_topo_ver.ensure(1);
  TM_CUDA(cudaMemsetAsync(m->d_topo_ver.get(), 0, sizeof(int), m->stream));
  cudaStream_t s = m->stream;
  if (nh) {
    TM_CUDA(cudaMemcpyAsync(m->d_to.get(), m->h_to.data(), sizeof(int) * nh, cudaMemcpyHostToDevice, s));
    TM_CUDA(cudaMemcpyAsync(m->d_next.get(), m->h_next.data(), sizeof(int) * nh, cudaMemcpyHostToDevice, s));
    TM_CUDA(cudaMemcpyAsync(m->d_face.get(), m->h_face.data(), sizeof(int) * nh, cudaMemcpyHostToDevice, s));
  }
  if (m->nv)
    TM_CUDA(cudaMemcpyAsync(m->d_vout.get(), m->h_vout.data(), sizeof(int) * m->nv, cudaMemcpyHostToDevice, s));
  if (m->nf)
    TM_CUDA(cudaMemcpyAsync(m->d_fhe.get(), m->h_fhe.data(), sizeof(int) * m->nf, cudaMemcpyHostToDevice, s));
  m->upload_points(s);
  m->rebuild_tables(s);
}

static void check_he(tm_mesh* m, int64_t h) {
  if (h < 0 || h >= 2 * (int64_t)m->ne) fail(TM_ERR_ARG, "halfedge handle out of range");
}

static void run_prims(tm_mesh* m, int64_t he, double* host40) {
  check_he(m, he);
  m->upload_points(m->stream);
  HE h{m->d_to.get(), m->d_next.get(), m->d_face.get(), m->d_pts.get(), 2 * m->ne};
  k_prims<<<1, 32, 0, m->stream>>>(h, (int)he, m->d_scratch.get());
  TM_LAUNCH();
  TM_CUDA(cudaMemcpyAsync(host40, m->d_scratch.get(), sizeof(double) * 40, cudaMemcpyDeviceToHost, m->stream));
  TM_CUDA(cudaStreamSynchronize(m->stream));
}

static double device_sum(tm_mesh* m, int what) {
  int n = what == 0 ? m->nf : m->ne;
  if (n == 0) return 0.0;
  int nb = std::min(1024, nblk(n, 256));
  m->d_scratch.ensure(4096 + nb + 1);
  m->upload_points(m->stream);
  double* part = m->d_scratch.get() + 2048;
  k_sum_terms<<<nb, 256, 0, m->stream>>>(n, what, m->topo(), m->d_pts.get(), part);
  TM_LAUNCH();
  k_sum_final<<<1, 256, 0, m->stream>>>(nb, part, part + nb);
  TM_LAUNCH();
  double r = 0;
  TM_CUDA(cudaMemcpyAsync(&r, part + nb, sizeof(double), cudaMemcpyDeviceToHost, m->stream));
  TM_CUDA(cudaStreamSynchronize(m->stream));
  return r;
}

// --------------------------------------------------------------------------
// C ABI
// --------------------------------------------------------------------------
extern "C" {

int tm_mesh_create(const double* points, int64_t n_points, const int32_t* faces, int64_t n_faces, tm_mesh** out) {
  TM_API_BEGIN
  if (!out) fail(TM_ERR_ARG, "out is NULL");
  *out = nullptr;
  if (n_points < 0 || n_faces < 0) fail(TM_ERR_ARG, "negative size");
  if (n_points > 0 && !points) fail(TM_ERR_ARG, "points is NULL");
  if (n_faces > 0 && !faces) fail(TM_ERR_ARG, "faces is NULL");
  if (n_points >= (1LL << 30)) fail(TM_ERR_ARG, "too many vertices");
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    fail(TM_ERR_CUDA, "no CUDA device available");
  }
  std::unique_ptr<tm_mesh> m(new tm_mesh());
  build_halfedges(m.get(), points, n_points, faces, n_faces);
  TM_CUDA(cudaStreamCreateWithFlags(&m->stream, cudaStreamNonBlocking));
  size_t bytes = sizeof(double) * 3 * std::max<int64_t>(n_points, 1);
  if (cudaMallocHost(&m->h_pts, bytes) != cudaSuccess) {
    cudaGetLastError();
    fail(TM_ERR_NOMEM, "page-locked allocation failed");
  }
  if (n_points) std::memcpy(m->h_pts, points, sizeof(double) * 3 * n_points);
  upload_topology(m.get());
  *out = m.release();
  TM_API_END
}

int tm_mesh_destroy(tm_mesh* m) {
  delete m;
  return TM_OK;
}

int tm_mesh_counts(tm_mesh* m, int64_t* nv, int64_t* ne, int64_t* nf) {
  if (!m) return TM_ERR_ARG;
  if (nv) *nv = m->nv;
  if (ne) *ne = m->ne;
  if (nf) *nf = m->nf;
  return TM_OK;
}

double* tm_mesh_points(tm_mesh* m) { return m ? m->h_pts : nullptr; }

int tm_mesh_fv_indices(tm_mesh* m, int32_t* out) {
  TM_API_BEGIN
  if (!m || (!out && m->nf)) fail(TM_ERR_ARG, "NULL argument");
  if (m->nf == 0) return TM_OK;
  TM_CUDA(cudaMemcpyAsync(out, m->d_fv.get(), sizeof(int) * 3 * m->nf, cudaMemcpyDeviceToHost, m->stream));
  TM_CUDA(cudaStreamSynchronize(m->stream));
  TM_API_END
}

int tm_mesh_halfedge(tm_mesh* m, int op, int64_t h, int64_t* out) {
  TM_API_BEGIN
  if (!m || !out) fail(TM_ERR_ARG, "NULL argument");
  m->sync_host_topology();
  switch (op) {
    case 0:
      if (h < 0 || h >= m->ne) fail(TM_ERR_ARG, "edge handle out of range");
      *out = 2 * h;
      break;
    case 1: check_he(m, h); *out = m->h_next[h]; break;
    case 2: check_he(m, h); *out = h ^ 1; break;
    case 3: check_he(m, h); *out = m->h_to[h]; break;
    case 4: check_he(m, h); *out = m->h_to[h ^ 1]; break;
    case 5: check_he(m, h); *out = m->h_face[h]; break;
    default: fail(TM_ERR_ARG, "unknown halfedge query");
  }
  TM_API_END
}

int tm_mesh_topology(tm_mesh* m, int32_t* to, int32_t* next, int32_t* face, int32_t* vout, int32_t* fhe) {
  TM_API_BEGIN
  if (!m) fail(TM_ERR_ARG, "NULL mesh");
  m->sync_host_topology();
  int nh = 2 * m->ne;
  if (to) std::copy(m->h_to.begin(), m->h_to.begin() + nh, to);
  if (next) std::copy(m->h_next.begin(), m->h_next.begin() + nh, next);
  if (face) std::copy(m->h_face.begin(), m->h_face.begin() + nh, face);
  if (vout) std::copy(m->h_vout.begin(), m->h_vout.end(), vout);
  if (fhe) std::copy(m->h_fhe.begin(), m->h_fhe.end(), fhe);
  TM_API_END
}

int tm_mesh_set_topology(tm_mesh* m, const int32_t* to, const int32_t* next, const int32_t* face,
                         const int32_t* vout, const int32_t* fhe) {
  TM_API_BEGIN
  if (!m || !to || !next || !face || !vout || !fhe) fail(TM_ERR_ARG, "NULL argument");
  const int nh = 2 * m->ne, nv = m->nv, nf = m->nf;
  // the arrays must describe a valid half-edge mesh of the same size
  for (int h = 0; h < nh; ++h) {
    if (to[h] < 0 || to[h] >= nv || next[h] < 0 || next[h] >= nh || face[h] < -1 || face[h] >= nf)
      fail(TM_ERR_TOPOLOGY, "half-edge index out of range");
    if (to[h] == to[h ^ 1]) fail(TM_ERR_TOPOLOGY, "degenerate edge");
  }
  for (int f = 0; f < nf; ++f) {
    int h = fhe[f];
    if (h < 0 || h >= nh || face[h] != f) fail(TM_ERR_TOPOLOGY, "face half-edge mismatch");
    int h1 = next[h], h2 = next[h1];
    if (face[h1] != f || face[h2] != f || next[h2] != h) fail(TM_ERR_TOPOLOGY, "face is not a triangle");
  }
  std::vector<int> deg(nv, 0);
  for (int h = 0; h < nh; ++h) deg[to[h ^ 1]]++;
  for (int v = 0; v < nv; ++v) {
    const int h0 = vout[v];
    if (h0 < -1 || h0 >= nh || (h0 >= 0 && to[h0 ^ 1] != v) || (h0 < 0 && deg[v] > 0))
      fail(TM_ERR_TOPOLOGY, "vertex half-edge mismatch");
    if (deg[v] > TM_MAXVAL) fail(TM_ERR_TOPOLOGY, "vertex valence exceeds TM_MAXVAL");
    if (h0 < 0) continue;
    int c = 0, h = h0;
    do {
      ++c;
      h = next[h ^ 1];
    } while (h != h0 && c <= deg[v]);
    if (c != deg[v]) fail(TM_ERR_TOPOLOGY, "non-manifold vertex");
  }
  m->h_to.assign(to, to + nh);
  m->h_next.assign(next, next + nh);
  m->h_face.assign(face, face + nh);
  m->h_vout.assign(vout, vout + nv);
  m->h_fhe.assign(fhe, fhe + nf);
  m->closed = true;
  for (int h = 0; h < nh; ++h) m->closed = m->closed && face[h] >= 0;
  upload_topology(m);
  m->host_topo_stale = false;
  // a new topology: exclusion flags kept with neighbour rows are not trusted
  ++m->topo_version;
  const int ver = (int)(m->topo_version & 0x7fffffff);
  TM_CUDA(cudaMemcpyAsync(m->d_topo_ver.get(), &ver, sizeof(int), cudaMemcpyHostToDevice, m->stream));
  TM_CUDA(cudaStreamSynchronize(m->stream));
  TM_API_END
}

int tm_mesh_check(tm_mesh* m, int* status) {
  TM_API_BEGIN
  if (!m || !status) fail(TM_ERR_ARG, "NULL argument");
  int zero = 0;
  TM_CUDA(cudaMemcpyAsync(m->d_status.get(), &zero, sizeof(int), cudaMemcpyHostToDevice, m->stream));
  if (m->nv) k_check<<<nblk(m->nv, 256), 256, 0, m->stream>>>(m->topo(), m->d_status.get());
  TM_LAUNCH();
  if (m->nf) k_check_faces<<<nblk(m->nf, 256), 256, 0, m->stream>>>(m->topo(), m->d_status.get());
  TM_LAUNCH();
  TM_CUDA(cudaMemcpyAsync(status, m->d_status.get(), sizeof(int), cudaMemcpyDeviceToHost, m->stream));
  TM_CUDA(cudaStreamSynchronize(m->stream));
  TM_API_END
}

int tm_edge_length(tm_mesh* m, int64_t he, double* value, double* grad) {
  TM_API_BEGIN
  if (!m) fail(TM_ERR_ARG, "NULL mesh");
  double r[40];
  run_prims(m, he, r);
  if (value) *value = r[0];
  if (grad) std::memcpy(grad, r + 1, sizeof(double) * 6);
  TM_API_END
}
int tm_face_area(tm_mesh* m, int64_t he, double* value, double* grad) {
  TM_API_BEGIN
  if (!m) fail(TM_ERR_ARG, "NULL mesh");
  double r[40];
  run_prims(m, he, r);
  if (value) *value = r[7];
  if (grad) std::memcpy(grad, r + 8, sizeof(double) * 9);
  TM_API_END
}
int tm_face_volume(tm_mesh* m, int64_t he, double* value, double* grad) {
  TM_API_BEGIN
  if (!m) fail(TM_ERR_ARG, "NULL mesh");
  double r[40];
  run_prims(m, he, r);
  if (value) *value = r[17];
  if (grad) std::memcpy(grad, r + 18, sizeof(double) * 9);
  TM_API_END
}
int tm_dihedral_angle(tm_mesh* m, int64_t he, double* value, double* grad) {
  TM_API_BEGIN
  if (!m) fail(TM_ERR_ARG, "NULL mesh");
  double r[40];
  run_prims(m, he, r);
  if (value) *value = r[27];
  if (grad) std::memcpy(grad, r + 28, sizeof(double) * 12);
  TM_API_END
}

int tm_area(tm_mesh* m, double* out) {
  TM_API_BEGIN
  if (!m || !out) fail(TM_ERR_ARG, "NULL argument");
  *out = device_sum(m, 0);
  TM_API_END
}
int tm_edges_length(tm_mesh* m, double* out) {
  TM_API_BEGIN
  if (!m || !out) fail(TM_ERR_ARG, "NULL argument");
  *out = device_sum(m, 1);
  TM_API_END
}
int tm_avg_tri_props(tm_mesh* m, double* a, double* l) {
  TM_API_BEGIN
  if (!m || !a || !l) fail(TM_ERR_ARG, "NULL argument");
  double A = device_sum(m, 0), L = device_sum(m, 1);
  *a = A / m->nf;
  *l = L / m->ne;
  TM_API_END
}

}  // extern "C"
