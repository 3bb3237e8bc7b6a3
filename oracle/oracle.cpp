// Oracle for the trimem hot path -- TEST INFRASTRUCTURE ONLY.
//
// A CPU restatement (C++17 + OpenMP) of the reference algorithms, used by
// tests/ as the checker and by bench.py as the timed CPU baseline.  The
// product never links it.  Each block cites the reference file:line it
// restates.  The data-structure choices of the reference are kept where they
// drive its cost (per-call std::vector results, a std::map cell list, virtual
// bond/repulsion dispatch, a per-vertex gradient buffer, four OpenMP regions
// per gradient) so that timing it is representative of the reference.
//
// OpenMesh is not available, so the half-edge operations the reference calls
// are restated from their documented behaviour:
//   add_face        new edges numbered in order of first appearance (faces in
//                   input order, face edges v0v1, v1v2, v2v0); halfedge 0 of an
//                   edge points along its first appearance; a face's halfedge
//                   is its v2->v0 halfedge, so fv_indices returns input order;
//                   a face whose directed edge is already used is skipped
//                   ("complex edge").
//   voh/vv circ.    h -> next(opposite(h)); only the summation order depends
//                   on it.
//   flip            rotates the edge inside its quad and keeps the edge index.
//   is_flip_ok      not boundary, opposite vertices differ and are not
//                   adjacent.
//   calc_sector_normal(h) = edge(next h) x edge(opp h)
//   calc_sector_angle(h)  = acos of the normalised dot of those two vectors
//   calc_dihedral_angle(h) = sign((n0 x n1).e) * acos(n0.n1/|n0||n1|), 0 on a
//                   boundary edge.
// Build: -O3 -fopenmp -ffp-contract=off (no FMA contraction, so pair
// distances are rounded exactly like the product's explicit-rounding code).

#include "oracle.h"

#include <omp.h>

#include <algorithm>
#include <array>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <map>
#include <memory>
#include <random>
#include <stdexcept>
#include <string>
#include <unordered_map>
#include <unordered_set>
#include <vector>

namespace orc {

static thread_local std::string g_err;

struct V3 {
  double x = 0, y = 0, z = 0;
  V3() = default;
  V3(double a, double b, double c) : x(a), y(b), z(c) {}
  V3 operator+(const V3& o) const { return {x + o.x, y + o.y, z + o.z}; }
  V3 operator-(const V3& o) const { return {x - o.x, y - o.y, z - o.z}; }
  V3 operator-() const { return {-x, -y, -z}; }
  V3 operator*(double s) const { return {x * s, y * s, z * s}; }
  V3 operator/(double s) const { return {x / s, y / s, z / s}; }
  V3& operator+=(const V3& o) { x += o.x; y += o.y; z += o.z; return *this; }
  V3& operator-=(const V3& o) { x -= o.x; y -= o.y; z -= o.z; return *this; }
  V3& operator*=(double s) { x *= s; y *= s; z *= s; return *this; }
  V3& operator/=(double s) { x /= s; y /= s; z /= s; return *this; }
  double sqrnorm() const { return x * x + y * y + z * z; }
  double norm() const { return std::sqrt(sqrnorm()); }
};
static inline V3 operator*(double s, const V3& v) { return v * s; }
static inline double dot(const V3& a, const V3& b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline V3 cross(const V3& a, const V3& b) {
  return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}

// ---------------------------------------------------------------------------
// Half-edge mesh (restates the OpenMesh TriMesh the reference is built on,
// src/mesh.h:15-31; construction as src/mesh_py.cpp:12-70).
// ---------------------------------------------------------------------------
struct Mesh {
  std::vector<V3> P;
  std::vector<int> to, nxt, fc;  // per halfedge; edge e owns 2e, 2e+1
  std::vector<int> vout;          // one outgoing halfedge per vertex (-1 isolated)
  std::vector<int> fhe;           // one halfedge per face

  int nv() const { return (int)P.size(); }
  int ne() const { return (int)to.size() / 2; }
  int nf() const { return (int)fhe.size(); }
  static int opp(int h) { return h ^ 1; }
  int from(int h) const { return to[h ^ 1]; }
  int next(int h) const { return nxt[h]; }
  int prev(int h) const {  // walk the loop (boundary loops can be long)
    int g = h;
    while (nxt[g] != h) g = nxt[g];
    return g;
  }
  bool bnd(int h) const { return fc[h] < 0; }
  bool edge_bnd(int e) const { return fc[2 * e] < 0 || fc[2 * e + 1] < 0; }

  template <class F>
  void voh(int v, F&& f) const {
    int h0 = vout[v];
    if (h0 < 0) return;
    int h = h0;
    int guard = 0;
    do {
      f(h);
      h = nxt[h ^ 1];
      if (++guard > 100000) throw std::runtime_error("circulator does not close");
    } while (h != h0);
  }
  template <class F>
  void vv(int v, F&& f) const {
    voh(v, [&](int h) { f(to[h]); });
  }

  V3 edge_vec(int h) const { return P[to[h]] - P[from(h)]; }
  V3 sector_normal(int h) const { return cross(edge_vec(next(h)), edge_vec(opp(h))); }
  double sector_angle(int h) const {
    V3 a = edge_vec(next(h)), b = edge_vec(opp(h));
    double den = a.norm() * b.norm();
    if (den == 0.0) return 0.0;
    double c = dot(a, b) / den;
    c = std::min(1.0, std::max(-1.0, c));
    return std::acos(c);
  }
  double dihedral(int h) const {
    if (fc[h] < 0 || fc[h ^ 1] < 0) return 0.0;
    V3 n0 = sector_normal(h), n1 = sector_normal(opp(h));
    V3 e = edge_vec(h);
    double den = n0.norm() * n1.norm();
    if (den == 0.0) return 0.0;
    double c = dot(n0, n1) / den;
    c = std::min(1.0, std::max(-1.0, c));
    double s = dot(cross(n0, n1), e);
    double a = std::acos(c);
    return s >= 0.0 ? a : -a;
  }

  bool adjacent(int a, int b) const {
    bool found = false;
    voh(a, [&](int h) { if (to[h] == b) found = true; });
    return found;
  }
  bool flip_ok(int e) const {
    if (edge_bnd(e)) return false;
    int c = to[nxt[2 * e]], d = to[nxt[2 * e + 1]];
    if (c == d) return false;
    return !adjacent(c, d);
  }
  // Edge rotation inside its quad; the edge keeps its index.
  void flip(int e) {
    int a0 = 2 * e, b0 = 2 * e + 1;
    int a1 = nxt[a0], a2 = nxt[a1], b1 = nxt[b0], b2 = nxt[b1];
    int va0 = to[a0], va1 = to[a1], vb0 = to[b0], vb1 = to[b1];
    int fa = fc[a0], fb = fc[b0];
    to[a0] = va1;
    to[b0] = vb1;
    nxt[a0] = a2; nxt[a2] = b1; nxt[b1] = a0;
    nxt[b0] = b2; nxt[b2] = a1; nxt[a1] = b0;
    fc[a1] = fb;
    fc[b1] = fa;
    fhe[fa] = a0;
    fhe[fb] = b0;
    if (vout[va0] == b0) vout[va0] = a1;
    if (vout[vb0] == a0) vout[vb0] = b1;
  }
};

static Mesh build_mesh(const double* pts, int nv, const int* faces, int nf) {
  Mesh m;
  m.P.resize(nv);
  for (int i = 0; i < nv; ++i) m.P[i] = V3(pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]);
  m.vout.assign(nv, -1);
  if (nv < 3) return m;
  std::unordered_map<uint64_t, int> emap;
  auto key = [](int a, int b) { return ((uint64_t)(uint32_t)std::min(a, b) << 32) | (uint32_t)std::max(a, b); };
  auto find_he = [&](int a, int b) -> int {
    auto it = emap.find(key(a, b));
    if (it == emap.end()) return -1;
    int h = 2 * it->second;
    return m.to[h] == b ? h : h + 1;
  };
  for (int f = 0; f < nf; ++f) {
    int v[3];
    int n = 0;
    for (int k = 0; k < 3; ++k) {
      int x = faces[3 * f + k];
      if (x >= 0 && x < nv) v[n++] = x;
    }
    if (n < 3) continue;
    if (v[0] == v[1] || v[1] == v[2] || v[0] == v[2]) continue;
    int hs[3];
    bool bad = false;
    for (int k = 0; k < 3; ++k) {
      hs[k] = find_he(v[k], v[(k + 1) % 3]);
      if (hs[k] >= 0 && m.fc[hs[k]] >= 0) bad = true;  // complex edge
    }
    if (bad) continue;
    for (int k = 0; k < 3; ++k) {
      if (hs[k] < 0) {
        int e = m.ne();
        emap[key(v[k], v[(k + 1) % 3])] = e;
        m.to.push_back(v[(k + 1) % 3]);
        m.to.push_back(v[k]);
        m.nxt.push_back(-1);
        m.nxt.push_back(-1);
        m.fc.push_back(-1);
        m.fc.push_back(-1);
        hs[k] = 2 * e;
      }
    }
    int fid = m.nf();
    for (int k = 0; k < 3; ++k) {
      m.nxt[hs[k]] = hs[(k + 1) % 3];
      m.fc[hs[k]] = fid;
    }
    m.fhe.push_back(hs[2]);
  }
  // boundary halfedges: link each to the boundary halfedge leaving its target
  int nh = (int)m.to.size();
  std::vector<int> bout(nv, -1);
  for (int h = 0; h < nh; ++h)
    if (m.fc[h] < 0) {
      int a = m.from(h);
      if (bout[a] >= 0) throw std::runtime_error("non-manifold vertex (several boundary fans)");
      bout[a] = h;
    }
  for (int h = 0; h < nh; ++h)
    if (m.fc[h] < 0) m.nxt[h] = bout[m.to[h]];
  for (int h = 0; h < nh; ++h) {
    int a = m.from(h);
    if (m.vout[a] < 0) m.vout[a] = h;
  }
  for (int v = 0; v < nv; ++v)
    if (bout[v] >= 0) m.vout[v] = bout[v];
  // every vertex's outgoing halfedges must form one fan
  std::vector<int> deg(nv, 0);
  for (int h = 0; h < nh; ++h) deg[m.from(h)]++;
  for (int v = 0; v < nv; ++v) {
    int c = 0;
    if (m.vout[v] >= 0) m.voh(v, [&](int) { ++c; });
    if (c != deg[v]) throw std::runtime_error("non-manifold vertex");
  }
  return m;
}

// ---------------------------------------------------------------------------
// Geometry primitives (src/mesh_util.h:15-185)
// ---------------------------------------------------------------------------
static inline double edge_length(const Mesh& m, int h) { return m.edge_vec(h).norm(); }
static inline std::vector<V3> edge_length_grad(const Mesh& m, int h, int bits) {
  V3 e = m.edge_vec(h);
  e /= e.norm();
  std::vector<V3> g;
  if (bits & 1) g.push_back(-e);
  if (bits & 2) g.push_back(e);
  return g;
}
static inline V3 face_normal(const Mesh& m, int h) {
  V3 n = m.sector_normal(h);
  return n / n.norm();
}
static inline double face_area(const Mesh& m, int h) { return m.sector_normal(h).norm() / 2; }
static inline std::vector<V3> face_area_grad(const Mesh& m, int h, int bits) {
  V3 n = face_normal(m, h);
  n /= n.norm();
  std::vector<V3> g;
  if (bits & 1) g.push_back(0.5 * cross(n, m.edge_vec(m.next(h))));
  if (bits & 2) g.push_back(0.5 * cross(n, m.edge_vec(m.prev(h))));
  if (bits & 4) g.push_back(0.5 * cross(n, m.edge_vec(h)));
  return g;
}
static inline double face_volume(const Mesh& m, int h) {
  const V3& p0 = m.P[m.from(h)];
  const V3& p1 = m.P[m.to[h]];
  const V3& p2 = m.P[m.to[m.next(h)]];
  return dot(cross(p1, p2), p0) / 6;
}
static inline std::vector<V3> face_volume_grad(const Mesh& m, int h, int bits) {
  const V3& p0 = m.P[m.from(h)];
  const V3& p1 = m.P[m.to[h]];
  const V3& p2 = m.P[m.to[m.next(h)]];
  std::vector<V3> g;
  if (bits & 1) g.push_back(cross(p1, p2) / 6);
  if (bits & 2) g.push_back(cross(p2, p0) / 6);
  if (bits & 4) g.push_back(cross(p0, p1) / 6);
  return g;
}
static inline double dihedral_angle(const Mesh& m, int h) { return m.dihedral(h); }
// Only the faces that exist are used; a boundary edge has a constant zero
// angle, so its gradient is zero (the reference reads undefined geometry
// there; the path is only used on closed meshes).
static inline std::vector<V3> dihedral_angle_grad(const Mesh& m, int h, int bits) {
  std::vector<V3> g;
  if (m.fc[h] < 0 || m.fc[h ^ 1] < 0) {
    for (int k = 0; k < 4; ++k)
      if (bits & (1 << k)) g.push_back(V3());
    return g;
  }
  V3 n0 = face_normal(m, h);
  V3 n1 = face_normal(m, Mesh::opp(h));
  double l = edge_length(m, h);
  double a01 = 0, a02 = 0, a03 = 0, a04 = 0;
  if (bits & (2 | 4)) a01 = m.sector_angle(m.prev(h));
  if (bits & (1 | 4)) a03 = m.sector_angle(h);
  if (bits & (2 | 8)) a02 = m.sector_angle(Mesh::opp(h));
  if (bits & (1 | 8)) a04 = m.sector_angle(m.prev(Mesh::opp(h)));
  if (bits & 1) g.push_back((1. / std::tan(a03) * n0 + 1. / std::tan(a04) * n1) / l);
  if (bits & 2) g.push_back((1. / std::tan(a01) * n0 + 1. / std::tan(a02) * n1) / l);
  if (bits & 4) g.push_back(-(1. / std::tan(a01) + 1. / std::tan(a03)) * n0 / l);
  if (bits & 8) g.push_back(-(1. / std::tan(a02) + 1. / std::tan(a04)) * n1 / l);
  return g;
}

// ---------------------------------------------------------------------------
// Parameters, bond potentials (src/mesh_tether.h:15-135)
// ---------------------------------------------------------------------------
struct Bond {
  virtual ~Bond() = default;
  virtual double value(const Mesh& m, int h) const = 0;
  virtual V3 grad_from(const Mesh& m, int h) const = 0;  // wrt from-vertex
  virtual int valence() const = 0;
};
struct EdgeBond : Bond {
  double lc0, lc1;
  int r;
  EdgeBond(double a, double b, int c) : lc0(a), lc1(b), r(c) {}
  double value(const Mesh& m, int h) const override {
    double l = edge_length(m, h);
    if (l > lc0) return std::pow(r, r + 1) * std::pow(l - lc0, r);
    if (l < lc1) return std::exp(l / (l - lc1)) / std::pow(l, r);
    return 0.0;
  }
  V3 grad_from(const Mesh& m, int h) const override {
    double l = edge_length(m, h);
    auto g = edge_length_grad(m, h, 1);
    double fac = 0.0;
    if (l > lc0) fac = std::pow(r, r + 2) * std::pow(l - lc0, r - 1);
    if (l < lc1) {
      double lr = std::pow(l, r), lmc = l - lc1;
      fac -= lc1 / (lmc * lmc) + r / l;
      fac /= lr;
      fac *= std::exp(l / lmc);
    }
    return g[0] * fac;
  }
  int valence() const override { return 2; }
};
struct AreaBond : Bond {
  double a0;
  explicit AreaBond(double a) : a0(a) {}
  double value(const Mesh& m, int h) const override {
    double d = face_area(m, h) / a0 - 1.0;
    return d * d;
  }
  V3 grad_from(const Mesh& m, int h) const override {
    double a = face_area(m, h);
    auto g = face_area_grad(m, h, 1);
    return g[0] * (2.0 * (a / a0 - 1.0) / a0);
  }
  int valence() const override { return 3; }
};
static std::unique_ptr<Bond> make_bond(const om_params& p) {
  if (p.bond_type == 0) return std::make_unique<EdgeBond>(p.bond_lc0, p.bond_lc1, p.bond_r);
  if (p.bond_type == 1) return std::make_unique<AreaBond>(p.bond_a0);
  throw std::runtime_error("Unknown bond potential");
}

// ---------------------------------------------------------------------------
// Neighbour lists (src/nlists/cell_list.h, verlet_list.h, nlist.cpp)
// ---------------------------------------------------------------------------
struct NList {
  virtual ~NList() = default;
  virtual void distance_matrix(const Mesh& m, double dmax, std::vector<double>& d, std::vector<int>& i,
                               std::vector<int>& j) const = 0;
  virtual void point_distances(const Mesh& m, int pid, double dmax, std::vector<V3>& d,
                               std::vector<int>& j) const = 0;
  // cell geometry, for tests of the binning
  double box[6] = {0, 0, 0, 0, 0, 0};
  double rl[3] = {0, 0, 0};
  int shp[3] = {0, 0, 0};
};

static inline double sq_dist(const double* a, const double* b) {
  double s = 0.0;
  for (int k = 0; k < 3; ++k) {
    double d = a[k] - b[k];
    s += d * d;
  }
  return s;
}

template <int EXCL>
static bool excluded(const Mesh& m, int pid, int jid) {
  if (pid == jid) return true;
  if constexpr (EXCL > 0) {
    bool in = false;
    int h0 = m.vout[pid];
    if (h0 < 0) return false;
    int h = h0;
    do {
      int w = m.to[h];
      if (w == jid) return true;
      if constexpr (EXCL > 1) {
        m.vv(w, [&](int u) { if (u == jid) in = true; });
        if (in) return true;
      }
      h = m.nxt[h ^ 1];
    } while (h != h0);
  }
  return false;
}

template <int EXCL>
struct CellList : NList {
  std::map<int, std::vector<int>> cells;
  std::array<int, 3> shape{}, strides{};
  std::array<double, 3> r_list{}, bmin{}, bmax{};
  std::vector<std::pair<int, int>> cell_pairs;

  CellList(const Mesh& m, double rlist, double box_eps = 1.0e-6) {
    // only element 0 of the initialisers is set, the rest are zero
    // (src/nlists/cell_list.h:46-47)
    bmin = {std::numeric_limits<double>::max(), 0.0, 0.0};
    bmax = {-1.0, 0.0, 0.0};
    for (int i = 0; i < m.nv(); ++i) {
      const double* p = &m.P[i].x;
      for (int k = 0; k < 3; ++k) {
        if (p[k] < bmin[k]) bmin[k] = p[k];
        if (p[k] > bmax[k]) bmax[k] = p[k];
      }
    }
    for (int k = 0; k < 3; ++k) {
      double dim = bmax[k] - bmin[k] + box_eps;
      int nk = int(dim / rlist);
      r_list[k] = nk > 0 ? dim / nk : dim;
      shape[k] = nk > 0 ? nk : 1;
    }
    strides = {1, shape[0], shape[0] * shape[1]};
    for (int i = 0; i < m.nv(); ++i) {
      const double* p = &m.P[i].x;
      int id = 0;
      for (int k = 0; k < 3; ++k) id += int((p[k] - bmin[k]) / r_list[k]) * strides[k];
      cells[id].push_back(i);
    }
    for (auto& it : cells) {
      int ic = it.first;
      int kc = ic / strides[2], rem = ic % strides[2], jc = rem / strides[1], icc = rem % strides[1];
      for (int a = -1; a < 2; ++a) {
        int ii = icc + a;
        if (ii < 0 || ii >= shape[0]) continue;
        for (int b = -1; b < 2; ++b) {
          int jj = jc + b;
          if (jj < 0 || jj >= shape[1]) continue;
          for (int c = -1; c < 2; ++c) {
            int kk = kc + c;
            if (kk < 0 || kk >= shape[2]) continue;
            int oc = ii * strides[0] + jj * strides[1] + kk * strides[2];
            if (cells.find(oc) == cells.end()) continue;
            if (ic <= oc) cell_pairs.push_back({ic, oc});
          }
        }
      }
    }
    for (int k = 0; k < 3; ++k) {
      box[k] = bmin[k];
      box[3 + k] = bmax[k];
      rl[k] = r_list[k];
      shp[k] = shape[k];
    }
  }

  void point_distances(const Mesh& m, int pid, double dmax, std::vector<V3>& dist,
                       std::vector<int>& nb) const override {
    dist.clear();
    nb.clear();
    const V3 p = m.P[pid];
    const double* pp = &p.x;
    int co[3];
    for (int k = 0; k < 3; ++k) co[k] = int((pp[k] - bmin[k]) / r_list[k]);
    for (int a = -1; a < 2; ++a) {
      int ii = co[0] + a;
      if (ii < 0 || ii >= shape[0]) continue;
      for (int b = -1; b < 2; ++b) {
        int jj = co[1] + b;
        if (jj < 0 || jj >= shape[1]) continue;
        for (int c = -1; c < 2; ++c) {
          int kk = co[2] + c;
          if (kk < 0 || kk >= shape[2]) continue;
          auto it = cells.find(ii * strides[0] + jj * strides[1] + kk * strides[2]);
          if (it == cells.end()) continue;
          for (int jid : it->second) {
            if (excluded<EXCL>(m, pid, jid)) continue;
            V3 d = p - m.P[jid];
            if (d.norm() < dmax) {
              dist.push_back(d);
              nb.push_back(jid);
            }
          }
        }
      }
    }
  }

  void distance_matrix(const Mesh& m, double rlist, std::vector<double>& dd, std::vector<int>& ii,
                       std::vector<int>& jj) const override {
    dd.clear();
    ii.clear();
    jj.clear();
    const double* data = &m.P[0].x;
    for (auto& cp : cell_pairs) {
      const auto& ic = cells.at(cp.first);
      const auto& oc = cells.at(cp.second);
      bool same = cp.first == cp.second;
      for (int a : ic) {
        for (int b : oc) {
          if (excluded<EXCL>(m, a, b)) continue;
          if (same && a > b) continue;
          double d = std::sqrt(sq_dist(data + 3 * a, data + 3 * b));
          if (d <= rlist) {
            dd.push_back(d);
            ii.push_back(std::min(a, b));
            jj.push_back(std::max(a, b));
          }
        }
      }
    }
  }
};

template <int EXCL>
struct VerletList : NList {
  std::vector<std::vector<int>> nbrs;
  VerletList(const Mesh& m, double rlist, double box_eps = 1.0e-6) {
    CellList<EXCL> cl(m, rlist, box_eps);
    std::vector<double> d;
    std::vector<int> i, j;
    cl.distance_matrix(m, rlist, d, i, j);
    nbrs.assign(m.nv(), {});
    for (size_t k = 0; k < i.size(); ++k) {
      nbrs[i[k]].push_back(j[k]);
      nbrs[j[k]].push_back(i[k]);
    }
    std::copy(cl.box, cl.box + 6, box);
    std::copy(cl.rl, cl.rl + 3, rl);
    std::copy(cl.shp, cl.shp + 3, shp);
  }
  void distance_matrix(const Mesh& m, double dmax, std::vector<double>& dd, std::vector<int>& ii,
                       std::vector<int>& jj) const override {
    dd.clear();
    ii.clear();
    jj.clear();
    const double* data = &m.P[0].x;
    for (int a = 0; a < m.nv(); ++a)
      for (int b : nbrs.at(a)) {
        double d = std::sqrt(sq_dist(data + 3 * a, data + 3 * b));
        if (d < dmax) {
          dd.push_back(d);
          ii.push_back(a);
          jj.push_back(b);
        }
      }
  }
  void point_distances(const Mesh& m, int pid, double dmax, std::vector<V3>& dist,
                       std::vector<int>& nb) const override {
    dist.clear();
    nb.clear();
    const V3 p = m.P[pid];
    for (int j : nbrs.at(pid)) {
      V3 d = p - m.P[j];
      if (d.norm() < dmax) {
        dist.push_back(d);
        nb.push_back(j);
      }
    }
  }
};

static std::unique_ptr<NList> make_nlist(const Mesh& m, int n_search, int excl, double rlist) {
  if (n_search == 0) {
    if (excl == 0) return std::make_unique<CellList<0>>(m, rlist);
    if (excl == 1) return std::make_unique<CellList<1>>(m, rlist);
    if (excl == 2) return std::make_unique<CellList<2>>(m, rlist);
    throw std::runtime_error("Unsupported exclusion level");
  }
  if (n_search == 1) {
    if (excl == 0) return std::make_unique<VerletList<0>>(m, rlist);
    if (excl == 1) return std::make_unique<VerletList<1>>(m, rlist);
    if (excl == 2) return std::make_unique<VerletList<2>>(m, rlist);
    throw std::runtime_error("Unsupported exclusion level");
  }
  throw std::runtime_error("Unknown neighbour search algorithm.");
}

// Surface repulsion (src/mesh_repulsion.h:28-79)
struct Repulsion {
  int r;
  double lc1;
  const NList& nl;
  Repulsion(const NList& n, double l, int rr) : r(rr), lc1(l), nl(n) {}
  double value(const Mesh& m, int pid) const {
    std::vector<V3> d;
    std::vector<int> j;
    nl.point_distances(m, pid, lc1, d, j);
    double pot = 0;
    for (auto& x : d) {
      double l = x.norm();
      pot += std::exp(l / (l - lc1)) / std::pow(l, r);
    }
    return pot;
  }
  void grad(const Mesh& m, int pid, std::vector<V3>& d, std::vector<int>& j) const {
    nl.point_distances(m, pid, lc1, d, j);
    for (auto& x : d) {
      double l = x.norm();
      double lr = std::pow(l, r + 1), lmc = l - lc1;
      double fac = -(lc1 / (lmc * lmc) + r / l);
      fac /= lr;
      fac *= std::exp(l / lmc);
      x *= fac;
    }
  }
};

// ---------------------------------------------------------------------------
// Vertex properties and their gradient (src/mesh_properties.cpp:12-148)
// ---------------------------------------------------------------------------
struct Props {
  double area = 0, volume = 0, curvature = 0, bending = 0, tethering = 0, repulsion = 0;
  Props& operator+=(const Props& o) {
    area += o.area; volume += o.volume; curvature += o.curvature;
    bending += o.bending; tethering += o.tethering; repulsion += o.repulsion;
    return *this;
  }
  Props& operator-=(const Props& o) {
    area -= o.area; volume -= o.volume; curvature -= o.curvature;
    bending -= o.bending; tethering -= o.tethering; repulsion -= o.repulsion;
    return *this;
  }
};
struct PropsGrad {
  V3 area, volume, curvature, bending, tethering, repulsion;
};

static Props vertex_properties(const Mesh& m, const Bond& bond, const Repulsion& rep, int v) {
  Props p;
  m.voh(v, [&](int h) {
    if (m.bnd(h)) return;
    double el = edge_length(m, h);
    double da = dihedral_angle(m, h);
    p.curvature += 0.5 * el * da;
    p.area += face_area(m, h);
    p.volume += face_volume(m, h);
    p.tethering += bond.value(m, h);
  });
  p.area /= 3;
  p.volume /= 3;
  p.curvature /= 2;
  p.tethering /= bond.valence();
  p.bending = 2 * p.curvature * p.curvature / p.area;
  p.repulsion = rep.value(m, v);
  return p;
}

// gather form: only the gradient entry of vertex v is written
static void vertex_properties_grad(const Mesh& m, const Bond& bond, const Repulsion& rep, int v,
                                   const std::vector<Props>& P, std::vector<PropsGrad>& G) {
  double rho[3];
  rho[0] = P[v].curvature / P[v].area;
  PropsGrad& g = G[v];
  m.voh(v, [&](int h) {
    if (m.bnd(h)) return;
    int nh = m.next(h);
    int j = m.to[h], k = m.to[nh];
    rho[1] = P[j].curvature / P[j].area;
    rho[2] = P[k].curvature / P[k].area;

    double el = edge_length(m, h), ea = dihedral_angle(m, h);
    V3 dl = edge_length_grad(m, h, 1)[0];
    V3 dth = dihedral_angle_grad(m, h, 1)[0];
    for (int i = 0; i < 2; ++i) {  // edge (v,j) belongs to the patches of v and j
      V3 val = 0.25 * (ea * dl + el * dth);
      g.curvature += val;
      g.bending += 4.0 * rho[i] * val;
    }
    V3 dA = face_area_grad(m, h, 1)[0];
    for (int i = 0; i < 3; ++i) {  // face (v,j,k) belongs to three patches
      V3 val = dA / 3;
      g.area += val;
      g.bending -= 2.0 * rho[i] * rho[i] * val;
    }
    V3 dV = face_volume_grad(m, h, 1)[0];
    for (int i = 0; i < 3; ++i) g.volume += dV / 3;

    double ln = edge_length(m, nh);
    V3 dthn = dihedral_angle_grad(m, nh, 4)[0];  // wrt the vertex opposite (j,k)
    for (int i = 1; i < 3; ++i) {
      V3 val = 0.25 * ln * dthn;
      g.curvature += val;
      g.bending += 4.0 * rho[i] * val;
    }
    g.tethering += bond.grad_from(m, h);
  });
  std::vector<V3> d;
  std::vector<int> j;
  rep.grad(m, v, d, j);
  for (auto& x : d) g.repulsion += 2 * x;
}

// ---------------------------------------------------------------------------
// Penalty assembly (src/kernel.h:18-137) and EnergyManager (src/energy.cpp)
// ---------------------------------------------------------------------------
struct Energy {
  om_params prm;
  std::unique_ptr<Bond> bond;
  std::unique_ptr<NList> nl;
  std::unique_ptr<Repulsion> rep;
  Props initial;

  Energy(const Mesh& m, const om_params& p) : prm(p) {
    bond = make_bond(prm);
    nl = make_nlist(m, prm.n_search, prm.exclusion_level, prm.rlist);
    rep = std::make_unique<Repulsion>(*nl, prm.rep_lc1, prm.rep_r);
    initial = properties(m);
  }
  Props ref_props() const {
    double lam = prm.cont_lambda;
    Props r;
    r.area = (1.0 - lam * (1.0 - prm.area_frac)) * initial.area;
    r.volume = (1.0 - lam * (1.0 - prm.volume_frac)) * initial.volume;
    r.curvature = (1.0 - lam * (1.0 - prm.curvature_frac)) * initial.curvature;
    return r;
  }
  void update_reference() {
    if (prm.cont_lambda < 1.0) prm.cont_lambda += prm.cont_delta;
  }
  void update_repulsion(const Mesh& m) {
    nl = make_nlist(m, prm.n_search, prm.exclusion_level, prm.rlist);
    rep = std::make_unique<Repulsion>(*nl, prm.rep_lc1, prm.rep_r);
  }
  void vertex_props(const Mesh& m, std::vector<Props>& vp) const {
    int n = m.nv();
    vp.assign(n, Props());
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; ++i) vp[i] = vertex_properties(m, *bond, *rep, i);
  }
  static Props reduce(const std::vector<Props>& vp) {
    Props s;
#pragma omp declare reduction(psum : Props : omp_out += omp_in) initializer(omp_priv = Props())
#pragma omp parallel for reduction(psum : s)
    for (int i = 0; i < (int)vp.size(); ++i) s += vp[i];
    return s;
  }
  Props properties(const Mesh& m) const {
    std::vector<Props> vp;
    vertex_props(m, vp);
    return reduce(vp);
  }
  void components(const Props& p, double* out7) const {
    Props r = ref_props();
    double da = p.area / r.area - 1.0, dv = p.volume / r.volume - 1.0, dc = p.curvature / r.curvature - 1.0;
    out7[0] = prm.kappa_a * da * da;
    out7[1] = prm.kappa_v * dv * dv;
    out7[2] = prm.kappa_c * dc * dc;
    out7[3] = prm.kappa_b * p.bending;
    out7[4] = prm.kappa_t * p.tethering;
    out7[5] = prm.kappa_r * p.repulsion;
    out7[6] = out7[0] + out7[1] + out7[2] + out7[4] + out7[5] + out7[3];
  }
  double energy(const Props& p) const {
    double c[7];
    components(p, c);
    double e = 0.0;
    e += c[0]; e += c[1]; e += c[2]; e += c[4]; e += c[5]; e += c[3];
    return e;
  }
  double energy(const Mesh& m) const { return energy(properties(m)); }
  void gradient(const Mesh& m, double* out) const {
    int n = m.nv();
    std::vector<Props> vp;
    vertex_props(m, vp);
    Props s = reduce(vp);
    Props r = ref_props();
    std::vector<PropsGrad> gp(n);
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; ++i) vertex_properties_grad(m, *bond, *rep, i, vp, gp);
    double fa = 2.0 * prm.kappa_a / r.area * (s.area / r.area - 1.0);
    double fv = 2.0 * prm.kappa_v / r.volume * (s.volume / r.volume - 1.0);
    double fcv = 2.0 * prm.kappa_c / r.curvature * (s.curvature / r.curvature - 1.0);
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; ++i) {
      const PropsGrad& g = gp[i];
      V3 t;
      t += fa * g.area;
      t += fv * g.volume;
      t += fcv * g.curvature;
      t += prm.kappa_t * g.tethering;
      t += prm.kappa_r * g.repulsion;
      t += prm.kappa_b * g.bending;
      out[3 * i] = t.x;
      out[3 * i + 1] = t.y;
      out[3 * i + 2] = t.z;
    }
  }
};

// ---------------------------------------------------------------------------
// Flips (src/flips.cpp:22-165, src/flip_utils.cpp:19-114)
// ---------------------------------------------------------------------------
static Props edge_vertex_properties(const Mesh& m, int e, const Energy& E) {
  Props p;
  for (int i = 0; i < 2; ++i) {
    int h = 2 * e + i;
    p += vertex_properties(m, *E.bond, *E.rep, m.to[h]);
    p += vertex_properties(m, *E.bond, *E.rep, m.to[m.next(h)]);
  }
  return p;
}

static void flip_patch(const Mesh& m, int e, std::vector<int>& out) {
  out.clear();
  for (int i = 0; i < 2; ++i) {
    int h = 2 * e + i;
    for (int v : {m.to[h], m.to[m.next(h)]})
      m.voh(v, [&](int g) {
        out.push_back(g >> 1);
        out.push_back(m.next(g) >> 1);
      });
  }
  std::sort(out.begin(), out.end());
  out.erase(std::unique(out.begin(), out.end()), out.end());
}

// The windowed sweep's patch of a proposal (the device's k_claim_win): the
// claim is the quad's four vertices and their ring neighbours, the test the
// quad's four vertices (va0, va1, vb0, vb1 as the device's quad_of).
static void flip_vertex_patch(const Mesh& m, int e, std::vector<int>& claim, int quad[4]) {
  quad[0] = m.to[2 * e];
  quad[1] = m.to[m.next(2 * e)];
  quad[2] = m.to[2 * e + 1];
  quad[3] = m.to[m.next(2 * e + 1)];
  claim.clear();
  for (int k = 0; k < 4; ++k) {
    claim.push_back(quad[k]);
    m.voh(quad[k], [&](int g) { claim.push_back(m.to[g]); });
  }
  std::sort(claim.begin(), claim.end());
  claim.erase(std::unique(claim.begin(), claim.end()), claim.end());
}

static int flip_serial(Mesh& m, const Energy& E, double ratio, uint64_t seed) {
  // the reference constructs but does not throw an error for ratio > 1
  int ne = m.ne();
  int nflips = (int)(ne * ratio);
  Props props = E.properties(m);
  double e0 = E.energy(props);
  std::mt19937 gen((uint32_t)seed);
  std::uniform_real_distribution<double> accept(0.0, 1.0);
  std::uniform_int_distribution<int> propose(0, ne - 1);
  int acc = 0;
  for (int i = 0; i < nflips; ++i) {
    int e = propose(gen);
    if (m.flip_ok(e) && !m.edge_bnd(e)) {
      Props op = edge_vertex_properties(m, e, E);
      props -= op;
      m.flip(e);
      Props np = edge_vertex_properties(m, e, E);
      props += np;
      double en = E.energy(props);
      double de = en - e0;
      double alpha = de < 0.0 ? 1.0 : std::exp(-de);
      double u = accept(gen);
      if (u <= alpha) {
        e0 = en;
        acc += 1;
      } else {
        m.flip(e);
        props -= np;
        props += op;
      }
    }
  }
  return acc;
}

static int flip_parallel(Mesh& m, const Energy& E, double ratio, uint64_t seed) {
  if (ratio > 1.0) throw std::range_error("flip_ratio must be <= 1.0");
  int ne = m.ne();
  int nflips = (int)(ne * ratio);
  Props props = E.properties(m);
  double e0 = E.energy(props);
  std::vector<omp_lock_t> locks(ne);
  for (auto& l : locks) omp_init_lock(&l);
  int acc = 0;
#pragma omp parallel reduction(+ : acc)
  {
    int tid = omp_get_thread_num(), nth = omp_get_num_threads();
    std::mt19937 prng((uint32_t)((tid + 1) * seed));
    std::uniform_real_distribution<double> accept(0.0, 1.0);
    std::uniform_int_distribution<int> propose(0, ne - 1);
    int iflips = nflips / nth;
    std::vector<int> patch, held;
    for (int it = 0; it < iflips; ++it) {
#pragma omp barrier
      int e = propose(prng);
      held.clear();
      bool ok = false;
      if (omp_test_lock(&locks[e])) {
        held.push_back(e);
        flip_patch(m, e, patch);
        ok = true;
        for (int x : patch) {
          if (x == e) continue;
          if (omp_test_lock(&locks[x])) {
            held.push_back(x);
          } else {
            ok = false;
            break;
          }
        }
        if (!ok) {
          for (int x : held) omp_unset_lock(&locks[x]);
          held.clear();
        }
      }
#pragma omp barrier
      for (int x : held) omp_unset_lock(&locks[x]);
      if (!ok) continue;
      if (!m.flip_ok(e)) continue;
      Props dp = edge_vertex_properties(m, e, E);
      m.flip(e);
      dp -= edge_vertex_properties(m, e, E);
      double u = accept(prng);
#pragma omp critical
      {
        props -= dp;
        double en = E.energy(props);
        double de = en - e0;
        double alpha = de < 0.0 ? 1.0 : std::exp(-de);
        if (u <= alpha) {
          e0 = en;
          acc += 1;
        } else {
          m.flip(e);
          props += dp;
        }
      }
    }
  }
  for (auto& l : locks) omp_destroy_lock(&l);
  return acc;
}

// Counter-based proposal stream shared with the device flip sweep:
// SplitMix64 (Steele, Lea & Flood 2014) over (seed, proposal, stream).
static inline uint64_t splitmix64(uint64_t z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
static inline uint64_t flip_key(uint64_t seed, uint64_t p, uint64_t stream) {
  return splitmix64(splitmix64(seed) ^ (2 * p + stream));
}
static inline int flip_edge_of(uint64_t seed, uint64_t p, int ne) {
  return (int)(((flip_key(seed, p, 0) >> 32) * (uint64_t)ne) >> 32);
}
static inline double flip_u_of(uint64_t seed, uint64_t p) {
  return (double)(flip_key(seed, p, 1) >> 11) * 0x1.0p-53;
}

// ---- ring form of vertex_properties used by the device flip sweep --------
// The device evaluates the four quad vertices over explicit rings (before and
// after a virtual flip); this restates that arithmetic operation by operation
// (the device file is compiled without FMA contraction), so ill-conditioned
// quads (nearly antiparallel faces, where the sign of the dihedral angle is
// decided by rounding) are decided identically.
struct PortRing {
  int n = 0;
  int r[40];
  bool f[40];
};
static void port_ring_before(const Mesh& m, int v, PortRing& R) {
  R.n = 0;
  m.voh(v, [&](int h) {
    R.r[R.n] = m.to[h];
    R.f[R.n] = m.fc[h] >= 0;
    R.n++;
  });
}
static void port_ring_remove(PortRing& R, int x) {
  int p = 0;
  while (p < R.n && R.r[p] != x) ++p;
  for (int k = p; k + 1 < R.n; ++k) {
    R.r[k] = R.r[k + 1];
    R.f[k] = R.f[k + 1];
  }
  if (p < R.n) R.n -= 1;
}
static void port_ring_insert_before(PortRing& R, int x, int y) {
  int p = 0;
  while (p < R.n && R.r[p] != x) ++p;
  for (int k = R.n; k > p; --k) {
    R.r[k] = R.r[k - 1];
    R.f[k] = R.f[k - 1];
  }
  R.r[p] = y;
  R.f[p] = true;
  R.n += 1;
}
static inline double port_ipow(double x, int n) {
  int a = n < 0 ? -n : n;
  double r = 1.0;
  for (int k = 0; k < a; ++k) r *= x;
  return n < 0 ? 1.0 / r : r;
}
// geometry and tether part; the repulsion term is added by the caller
static void port_ring_props(const Mesh& m, const PortRing& R, int v, const om_params& prm, double* out) {
  const V3 xv = m.P[v];
  double A = 0, Vv = 0, C = 0, T = 0;
  int n = R.n;
  double tdiv = prm.bond_type == 0 ? 2.0 : 3.0;
  for (int k = 0; k < n; ++k) {
    if (!R.f[k]) continue;
    int j = R.r[k], kk = R.r[k == 0 ? n - 1 : k - 1];
    int mn = k + 1 == n ? 0 : k + 1;
    V3 xj = m.P[j], xk = m.P[kk];
    V3 ev = xj - xv;
    double el = ev.norm();
    V3 N0 = cross(ev, xk - xv);
    double fa = N0.norm() / 2;
    double th = 0.0;
    if (R.f[mn]) {
      V3 xn = m.P[R.r[mn]];
      V3 N1 = cross(xn - xv, ev);
      double den = N0.norm() * N1.norm();
      if (den != 0.0) {
        double c = std::min(1.0, std::max(-1.0, dot(N0, N1) / den));
        double a = std::acos(c);
        th = dot(cross(N0, N1), ev) >= 0.0 ? a : -a;
      }
    }
    C += 0.5 * el * th;
    A += fa;
    Vv += dot(cross(xj, xk), xv) / 6;
    if (prm.bond_type == 0) {
      int r = prm.bond_r;
      if (el > prm.bond_lc0)
        T += port_ipow((double)r, r + 1) * port_ipow(el - prm.bond_lc0, r);
      else if (el < prm.bond_lc1)
        T += std::exp(el / (el - prm.bond_lc1)) / port_ipow(el, r);
    } else {
      double q = fa / prm.bond_a0 - 1.0;
      T += q * q;
    }
  }
  A /= 3;
  Vv /= 3;
  C /= 2;
  T /= tdiv;
  out[0] = A;
  out[1] = Vv;
  out[2] = C;
  out[3] = 2 * C * C / A;
  out[4] = T;
}
static double port_repulsion(const Mesh& m, const Energy& E, int v) {
  std::vector<V3> d;
  std::vector<int> j;
  double lc1 = E.prm.rep_lc1;
  int rr = E.prm.rep_r;
  E.nl->point_distances(m, v, lc1, d, j);
  double pot = 0.0;
  for (auto& x : d) {
    double l = x.norm();
    pot += std::exp(l / (l - lc1)) / port_ipow(l, rr);
  }
  return pot;
}

// CPU port of the device sweep (see oracle.h).
static int flip_windowed(Mesh& m, const Energy& E, double ratio, uint64_t seed, int mode, int batch) {
  if (ratio > 1.0 && mode == 1) throw std::range_error("flip_ratio must be <= 1.0");
  int ne = m.ne();
  long nflips = (long)(ne * ratio);
  Props props = E.properties(m);
  // the Metropolis energy change E(props - dp) - E(props) as the device's
  // flip_delta: the penalty energy (src/kernel.h:110-122) with the
  // reciprocals of the reference properties instead of divisions, written
  // without cancellation (k t (t - 2 d0) for the quadratic penalties,
  // d0 = props/ref - 1, t = dp/ref; -k dp for the linear terms), the same
  // operations in the same order
  const Props ref = E.ref_props();
  const double irA = 1.0 / ref.area, irV = 1.0 / ref.volume, irC = 1.0 / ref.curvature;
  const om_params& q = E.prm;
  auto flip_delta = [&](const Props& p, const Props& dp) {
    const double da = p.area * irA - 1.0, dv = p.volume * irV - 1.0, dc = p.curvature * irC - 1.0;
    const double ta = dp.area * irA, tv = dp.volume * irV, tc = dp.curvature * irC;
    double de = 0.0;
    de += q.kappa_a * ta * (ta - 2.0 * da);
    de += q.kappa_v * tv * (tv - 2.0 * dv);
    de += q.kappa_c * tc * (tc - 2.0 * dc);
    de -= q.kappa_t * dp.tethering;
    de -= q.kappa_r * dp.repulsion;
    de -= q.kappa_b * dp.bending;
    return de;
  };
  // per vertex: the lowest slot of the window whose patch claims it
  std::vector<int> owner(m.nv(), std::numeric_limits<int>::max());
  std::vector<long> pending;
  long next_new = 0;
  int acc = 0;
  std::vector<std::vector<int>> patches;
  std::vector<std::array<int, 4>> quads;
  while (!pending.empty() || next_new < nflips) {
    std::vector<long> win(pending.begin(), pending.end());
    pending.clear();
    while ((int)win.size() < batch && next_new < nflips) win.push_back(next_new++);
    int W = (int)win.size();
    patches.assign(W, {});
    quads.assign(W, {});
    for (int s = 0; s < W; ++s) {
      flip_vertex_patch(m, flip_edge_of(seed, win[s], ne), patches[s], quads[s].data());
      for (int x : patches[s]) owner[x] = std::min(owner[x], s);
    }
    std::vector<char> winner(W, 1);
    for (int s = 0; s < W; ++s)
      for (int x : quads[s])
        if (owner[x] != s) winner[s] = 0;
    for (int s = 0; s < W; ++s)
      for (int x : patches[s]) owner[x] = std::numeric_limits<int>::max();
    int limit = W;
    if (mode == 0) {
      for (int s = 0; s < W; ++s)
        if (!winner[s]) { limit = s; break; }
    }
    std::vector<long> keep;
    for (int s = 0; s < W; ++s)
      if (s >= limit || !winner[s]) keep.push_back(win[s]);
    // parallel part: differential properties on the window-start topology
    std::vector<Props> dps(limit);
    std::vector<char> ok(limit, 0);
    for (int s = 0; s < limit; ++s) {
      if (!winner[s]) continue;
      int e = flip_edge_of(seed, win[s], ne);
      if (!m.flip_ok(e)) continue;
      {  // the device refuses flips that would raise a valence above 32
        int c = m.to[m.nxt[2 * e]], d = m.to[m.nxt[2 * e + 1]];
        int vc = 0, vd = 0;
        m.voh(c, [&](int) { ++vc; });
        m.voh(d, [&](int) { ++vd; });
        if (vc >= 32 || vd >= 32) continue;
      }
      ok[s] = 1;
      int a0 = 2 * e, b0 = 2 * e + 1;
      int a1 = m.nxt[a0], a2 = m.nxt[a1], b1 = m.nxt[b0], b2 = m.nxt[b1];
      int va0 = m.to[a0], va1 = m.to[a1], vb0 = m.to[b0], vb1 = m.to[b1];
      int fa = m.fc[a0], fb = m.fc[b0];
      int quad[4] = {va0, va1, vb0, vb1};
      double ob[4][6], oa[4][6];
      PortRing R;
      for (int q = 0; q < 4; ++q) {  // before: the current rings
        port_ring_before(m, quad[q], R);
        port_ring_props(m, R, quad[q], E.prm, ob[q]);
        ob[q][5] = port_repulsion(m, E, quad[q]);
      }
      for (int q = 0; q < 4; ++q) {  // after: rings edited like the device
        int v = quad[q];
        port_ring_before(m, v, R);
        if (v == va0) port_ring_remove(R, vb0);
        else if (v == vb0) port_ring_remove(R, va0);
        else if (v == va1) port_ring_insert_before(R, vb0, vb1);
        else port_ring_insert_before(R, va0, va1);
        port_ring_props(m, R, v, E.prm, oa[q]);
      }
      // the repulsion after the flip sees the flipped exclusion rings
      int sv_to[2] = {m.to[a0], m.to[b0]};
      int sv_nx[6] = {m.nxt[a0], m.nxt[a1], m.nxt[a2], m.nxt[b0], m.nxt[b1], m.nxt[b2]};
      int sv_fc[2] = {m.fc[a1], m.fc[b1]};
      int sv_fh[2] = {m.fhe[fa], m.fhe[fb]};
      int sv_vo[2] = {m.vout[va0], m.vout[vb0]};
      m.flip(e);
      for (int q = 0; q < 4; ++q) oa[q][5] = port_repulsion(m, E, quad[q]);
      m.to[a0] = sv_to[0]; m.to[b0] = sv_to[1];
      m.nxt[a0] = sv_nx[0]; m.nxt[a1] = sv_nx[1]; m.nxt[a2] = sv_nx[2];
      m.nxt[b0] = sv_nx[3]; m.nxt[b1] = sv_nx[4]; m.nxt[b2] = sv_nx[5];
      m.fc[a1] = sv_fc[0]; m.fc[b1] = sv_fc[1];
      m.fhe[fa] = sv_fh[0]; m.fhe[fb] = sv_fh[1];
      m.vout[va0] = sv_vo[0]; m.vout[vb0] = sv_vo[1];
      // summation orders of edge_vertex_properties before (va0, va1, vb0,
      // vb1) and after the flip (va1, vb0, vb1, va0)
      double dpv[6];
      for (int k = 0; k < 6; ++k) {
        double bsum = ((ob[0][k] + ob[1][k]) + ob[2][k]) + ob[3][k];
        double asum = ((oa[1][k] + oa[2][k]) + oa[3][k]) + oa[0][k];
        dpv[k] = bsum - asum;
      }
      Props before;
      before.area = dpv[0]; before.volume = dpv[1]; before.curvature = dpv[2];
      before.bending = dpv[3]; before.tethering = dpv[4]; before.repulsion = dpv[5];
      dps[s] = before;
    }
    // sequential Metropolis in window order, then commit: each slot is tried
    // on the state left by the accepted slots before it and accepted when
    // E(props - dp) - E <= -log(u) (the device's k_metro decides the same)
    for (int s = 0; s < limit; ++s) {
      if (!ok[s]) continue;
      if (flip_delta(props, dps[s]) <= -std::log(flip_u_of(seed, win[s]))) {
        props -= dps[s];
        acc += 1;
        m.flip(flip_edge_of(seed, win[s], ne));
      }
    }
    pending.swap(keep);
  }
  return acc;
}

struct NListHandle {
  std::unique_ptr<NList> nl;
  std::vector<double> d;
  std::vector<int> i, j;
  std::vector<V3> d3;
};

}  // namespace orc

using namespace orc;

#define GUARD(expr, fail)          \
  try {                            \
    expr;                          \
  } catch (std::exception & ex) {  \
    g_err = ex.what();             \
    return fail;                   \
  }

extern "C" {

const char* om_last_error(void) { return g_err.c_str(); }
void om_set_threads(int n) { omp_set_num_threads(n); }
int om_get_threads(void) { return omp_get_max_threads(); }

void* om_mesh_create(const double* pts, int nv, const int* faces, int nf) {
  GUARD(return new Mesh(build_mesh(pts, nv, faces, nf)), nullptr);
}
void* om_mesh_clone(void* m) { return new Mesh(*(Mesh*)m); }
void om_mesh_destroy(void* m) { delete (Mesh*)m; }
int om_mesh_nv(void* m) { return ((Mesh*)m)->nv(); }
int om_mesh_ne(void* m) { return ((Mesh*)m)->ne(); }
int om_mesh_nf(void* m) { return ((Mesh*)m)->nf(); }
double* om_mesh_points(void* m) { return ((Mesh*)m)->P.empty() ? nullptr : &((Mesh*)m)->P[0].x; }
void om_mesh_fv(void* mp, int* out) {
  Mesh& m = *(Mesh*)mp;
  for (int f = 0; f < m.nf(); ++f) {
    int h = m.fhe[f];
    out[3 * f] = m.to[h];
    out[3 * f + 1] = m.to[m.nxt[h]];
    out[3 * f + 2] = m.to[m.nxt[m.nxt[h]]];
  }
}
void om_mesh_topology(void* mp, int* to, int* nx, int* fcc, int* vout, int* fhe) {
  Mesh& m = *(Mesh*)mp;
  std::copy(m.to.begin(), m.to.end(), to);
  std::copy(m.nxt.begin(), m.nxt.end(), nx);
  std::copy(m.fc.begin(), m.fc.end(), fcc);
  std::copy(m.vout.begin(), m.vout.end(), vout);
  std::copy(m.fhe.begin(), m.fhe.end(), fhe);
}
int om_mesh_next(void* m, int h) { return ((Mesh*)m)->nxt[h]; }
int om_mesh_to(void* m, int h) { return ((Mesh*)m)->to[h]; }
int om_mesh_check(void* mp) {
  Mesh& m = *(Mesh*)mp;
  int nh = (int)m.to.size();
  for (int h = 0; h < nh; ++h) {
    if (m.to[h] == m.from(h)) return -1;
    if (m.fc[h] >= 0) {
      if (m.nxt[m.nxt[m.nxt[h]]] != h) return -2;
      if (m.fc[m.nxt[h]] != m.fc[h]) return -3;
    }
  }
  std::unordered_set<uint64_t> seen;
  for (int e = 0; e < m.ne(); ++e) {
    int a = m.to[2 * e], b = m.to[2 * e + 1];
    uint64_t k = ((uint64_t)std::min(a, b) << 32) | (uint32_t)std::max(a, b);
    if (!seen.insert(k).second) return -4;  // double edge
  }
  std::vector<int> deg(m.nv(), 0);
  for (int h = 0; h < nh; ++h) deg[m.from(h)]++;
  for (int v = 0; v < m.nv(); ++v) {
    int c = 0;
    if (m.vout[v] >= 0) {
      if (m.from(m.vout[v]) != v) return -5;
      m.voh(v, [&](int) { ++c; });
    }
    if (c != deg[v]) return -6;  // not a single fan
    if (deg[v] > 0 && deg[v] < 3) return -7;
  }
  for (int f = 0; f < m.nf(); ++f)
    if (m.fc[m.fhe[f]] != f) return -8;
  return 0;
}

double om_edge_length(void* m, int he) { return edge_length(*(Mesh*)m, he); }
static void put(const std::vector<V3>& g, double* out) {
  for (size_t k = 0; k < g.size(); ++k) {
    out[3 * k] = g[k].x;
    out[3 * k + 1] = g[k].y;
    out[3 * k + 2] = g[k].z;
  }
}
void om_edge_length_grad(void* m, int he, double* out) { put(edge_length_grad(*(Mesh*)m, he, 3), out); }
double om_face_area(void* m, int he) { return face_area(*(Mesh*)m, he); }
void om_face_area_grad(void* m, int he, double* out) { put(face_area_grad(*(Mesh*)m, he, 7), out); }
double om_face_volume(void* m, int he) { return face_volume(*(Mesh*)m, he); }
void om_face_volume_grad(void* m, int he, double* out) { put(face_volume_grad(*(Mesh*)m, he, 7), out); }
double om_dihedral_angle(void* m, int he) { return dihedral_angle(*(Mesh*)m, he); }
void om_dihedral_angle_grad(void* m, int he, double* out) { put(dihedral_angle_grad(*(Mesh*)m, he, 15), out); }

void* om_energy_create(void* m, const om_params* p) { GUARD(return new Energy(*(Mesh*)m, *p), nullptr); }
void om_energy_destroy(void* e) { delete (Energy*)e; }
static void put_props(const Props& p, double* o) {
  o[0] = p.area; o[1] = p.volume; o[2] = p.curvature; o[3] = p.bending; o[4] = p.tethering; o[5] = p.repulsion;
}
void om_energy_properties(void* e, void* m, double* out) { put_props(((Energy*)e)->properties(*(Mesh*)m), out); }
void om_energy_vertex_properties(void* e, void* m, double* out) {
  std::vector<Props> vp;
  ((Energy*)e)->vertex_props(*(Mesh*)m, vp);
  for (size_t i = 0; i < vp.size(); ++i) put_props(vp[i], out + 6 * i);
}
double om_energy_energy(void* e, void* m) { return ((Energy*)e)->energy(*(Mesh*)m); }
double om_energy_energy_props(void* e, const double* p) {
  Props q;
  q.area = p[0]; q.volume = p[1]; q.curvature = p[2]; q.bending = p[3]; q.tethering = p[4]; q.repulsion = p[5];
  return ((Energy*)e)->energy(q);
}
void om_energy_components(void* e, void* m, double* out7) {
  Energy& E = *(Energy*)e;
  E.components(E.properties(*(Mesh*)m), out7);
}
void om_energy_gradient(void* e, void* m, double* out) { ((Energy*)e)->gradient(*(Mesh*)m, out); }
void om_energy_update_reference(void* e) { ((Energy*)e)->update_reference(); }
void om_energy_update_repulsion(void* e, void* m) { ((Energy*)e)->update_repulsion(*(Mesh*)m); }
void om_energy_initial_props(void* e, double* out) { put_props(((Energy*)e)->initial, out); }
void om_energy_set_initial_props(void* e, const double* p) {
  Props& q = ((Energy*)e)->initial;
  q.area = p[0]; q.volume = p[1]; q.curvature = p[2]; q.bending = p[3]; q.tethering = p[4]; q.repulsion = p[5];
}
void om_energy_ref_props(void* e, double* out) { put_props(((Energy*)e)->ref_props(), out); }
double om_energy_lambda(void* e) { return ((Energy*)e)->prm.cont_lambda; }

void* om_nlist_create(void* m, int n_search, int excl, double rlist) {
  GUARD(auto* h = new NListHandle(); h->nl = make_nlist(*(Mesh*)m, n_search, excl, rlist); return h, nullptr);
}
void om_nlist_destroy(void* nl) { delete (NListHandle*)nl; }
int64_t om_nlist_distance_matrix(void* nl, void* m, double dmax) {
  auto* h = (NListHandle*)nl;
  h->nl->distance_matrix(*(Mesh*)m, dmax, h->d, h->i, h->j);
  return (int64_t)h->d.size();
}
int64_t om_nlist_point_distances(void* nl, void* m, int pid, double dmax) {
  auto* h = (NListHandle*)nl;
  h->nl->point_distances(*(Mesh*)m, pid, dmax, h->d3, h->j);
  return (int64_t)h->j.size();
}
void om_nlist_fetch(void* nl, double* d, int* i, int* j) {
  auto* h = (NListHandle*)nl;
  std::copy(h->d.begin(), h->d.end(), d);
  std::copy(h->i.begin(), h->i.end(), i);
  std::copy(h->j.begin(), h->j.end(), j);
}
void om_nlist_fetch_points(void* nl, double* d3, int* j) {
  auto* h = (NListHandle*)nl;
  put(h->d3, d3);
  std::copy(h->j.begin(), h->j.end(), j);
}
void om_nlist_cell_info(void* nl, double* box6, double* rl3, int* shape3) {
  auto* h = (NListHandle*)nl;
  std::copy(h->nl->box, h->nl->box + 6, box6);
  std::copy(h->nl->rl, h->nl->rl + 3, rl3);
  std::copy(h->nl->shp, h->nl->shp + 3, shape3);
}

int om_flip_serial(void* m, void* e, double ratio, uint64_t seed) {
  GUARD(return flip_serial(*(Mesh*)m, *(Energy*)e, ratio, seed), -1);
}
int om_flip_parallel(void* m, void* e, double ratio, uint64_t seed) {
  GUARD(return flip_parallel(*(Mesh*)m, *(Energy*)e, ratio, seed), -1);
}
int om_flip_windowed(void* m, void* e, double ratio, uint64_t seed, int mode, int batch) {
  GUARD(return flip_windowed(*(Mesh*)m, *(Energy*)e, ratio, seed, mode, batch), -1);
}

double om_area(void* mp) {
  Mesh& m = *(Mesh*)mp;
  double a = 0.0;
#pragma omp parallel for reduction(+ : a)
  for (int f = 0; f < m.nf(); ++f) a += face_area(m, m.fhe[f]);
  return a;
}
double om_edges_length(void* mp) {
  Mesh& m = *(Mesh*)mp;
  double l = 0.0;
#pragma omp parallel for reduction(+ : l)
  for (int e = 0; e < m.ne(); ++e) l += edge_length(m, 2 * e);
  return l;
}
void om_fd_gradient(void* mp, void* ep, double eps, double* out) {
  Mesh& m = *(Mesh*)mp;
  Energy& E = *(Energy*)ep;
  double e0 = E.energy(m);
  for (int i = 0; i < m.nv(); ++i) {
    double* p = &m.P[i].x;
    for (int k = 0; k < 3; ++k) {
      p[k] += eps;
      out[3 * i + k] = (E.energy(m) - e0) / eps;
      p[k] -= eps;
    }
  }
}
double om_time_energy_gradient(void* ep, void* mp, int n) {
  Energy& E = *(Energy*)ep;
  Mesh& m = *(Mesh*)mp;
  std::vector<double> g(3 * (size_t)m.nv());
  volatile double sink = 0;
  auto t0 = std::chrono::steady_clock::now();
  for (int k = 0; k < n; ++k) {
    sink = sink + E.energy(m);
    E.gradient(m, g.data());
  }
  auto t1 = std::chrono::steady_clock::now();
  return std::chrono::duration<double>(t1 - t0).count();
}

}  // extern "C"
