// pybind11 module `core`: the reference's `trimem.core` API
// (src/bindings.cpp:52-1093) implemented over the C ABI of libtrimem_gpu.
// Names, keyword arguments, defaults and exception types follow the
// reference: std::runtime_error -> RuntimeError, std::range_error ->
// ValueError.
#include <pybind11/iostream.h>
#include <pybind11/numpy.h>
#include <pybind11/pybind11.h>
#include <pybind11/stl.h>

#include <chrono>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iostream>
#include <map>
#include <sstream>
#include <string>
#include <tuple>
#include <vector>

#include "trimem_gpu.h"


namespace py = pybind11;

namespace {

// Result arrays of gradients live in page-locked memory, recycled through a
// small pool: the device writes them without staging, and their pages are
// never first touched inside a timed copy.  A buffer returns to the pool
// when numpy releases the array.
struct PinnedPool {
  std::multimap<size_t, void*> free_list;
  void* take(size_t bytes) {
    auto it = free_list.find(bytes);
    if (it != free_list.end()) {
      void* p = it->second;
      free_list.erase(it);
      return p;
    }
    void* p = nullptr;
    if (tm_host_alloc((int64_t)bytes, &p) != TM_OK) return nullptr;
    return p;
  }
  void give(size_t bytes, void* p) {
    if (free_list.size() < 8)
      free_list.emplace(bytes, p);
    else
      tm_host_free(p);
  }
};
PinnedPool& pinned_pool() {
  static PinnedPool* pool = new PinnedPool();  // outlives module teardown
  return *pool;
}
struct PoolBlock {
  size_t bytes;
  void* p;
};

// (rows, cols) float64 array in pooled page-locked memory (plain numpy
// memory when page-locked memory is not available)
py::array_t<double> pinned_array(py::ssize_t rows, py::ssize_t cols) {
  size_t bytes = sizeof(double) * (size_t)rows * (size_t)cols;
  void* p = pinned_pool().take(bytes);
  if (!p) return py::array_t<double>({rows, cols});
  auto* blk = new PoolBlock{bytes, p};
  py::capsule owner(blk, [](void* q) {
    auto* b = static_cast<PoolBlock*>(q);
    pinned_pool().give(b->bytes, b->p);
    delete b;
  });
  return py::array_t<double>({rows, cols}, {(py::ssize_t)(cols * sizeof(double)), (py::ssize_t)sizeof(double)},
                             static_cast<double*>(p), owner);
}

}  // namespace

namespace {

void check(int rc) {
  if (rc == TM_OK) return;
  std::string msg = tm_last_error();
  if (rc == TM_ERR_RANGE) throw py::value_error(msg);
  throw std::runtime_error(msg);
}

// ---- parameters (src/params.h:11-71) --------------------------------------
enum class BondType : int { Edge = 0, Area = 1, None = 2 };

struct BondParams {
  double lc0 = 1;
  double lc1 = 0;
  double a0 = 1;
  int r = 2;
  BondType type = BondType::Edge;
};
struct ContinuationParams {
  double delta = 0;
  double lambda = 1;
};
struct SurfaceRepulsionParams {
  double lc1 = 0;
  int r = 2;
  std::string n_search = "cell-list";
  double rlist = 0.1;
  int exclusion_level = 2;
};
struct EnergyParams {
  double kappa_b = 0, kappa_a = 0, kappa_v = 0, kappa_c = 0, kappa_t = 0, kappa_r = 0;
  double area_frac = 1, volume_frac = 1, curvature_frac = 1;
  BondParams bond_params;
  ContinuationParams continuation_params;
  SurfaceRepulsionParams repulse_params;
};

tm_params to_c(const EnergyParams& p) {
  tm_params c{};
  c.kappa_b = p.kappa_b;
  c.kappa_a = p.kappa_a;
  c.kappa_v = p.kappa_v;
  c.kappa_c = p.kappa_c;
  c.kappa_t = p.kappa_t;
  c.kappa_r = p.kappa_r;
  c.area_frac = p.area_frac;
  c.volume_frac = p.volume_frac;
  c.curvature_frac = p.curvature_frac;
  c.bond_lc0 = p.bond_params.lc0;
  c.bond_lc1 = p.bond_params.lc1;
  c.bond_a0 = p.bond_params.a0;
  c.bond_r = p.bond_params.r;
  c.bond_type = (int)p.bond_params.type;
  c.rep_lc1 = p.repulse_params.lc1;
  c.rep_r = p.repulse_params.r;
  const std::string& ns = p.repulse_params.n_search;
  c.n_search = ns == "cell-list" ? 0 : (ns == "verlet-list" ? 1 : -1);
  c.rlist = p.repulse_params.rlist;
  c.exclusion_level = p.repulse_params.exclusion_level;
  c.cont_delta = p.continuation_params.delta;
  c.cont_lambda = p.continuation_params.lambda;
  return c;
}

struct VertexProperties {
  double area = 0, volume = 0, curvature = 0, bending = 0, tethering = 0, repulsion = 0;
};
VertexProperties vp_from(const double* a) {
  VertexProperties p;
  p.area = a[0];
  p.volume = a[1];
  p.curvature = a[2];
  p.bending = a[3];
  p.tethering = a[4];
  p.repulsion = a[5];
  return p;
}

struct HalfedgeHandle {
  int64_t h = -1;
};

struct Point {
  double x = 0, y = 0, z = 0;
};

// ---- mesh -----------------------------------------------------------------
struct TriMesh {
  tm_mesh* h = nullptr;
  TriMesh() { check(tm_mesh_create(nullptr, 0, nullptr, 0, &h)); }
  TriMesh(const double* p, int64_t np, const int32_t* f, int64_t nf) { check(tm_mesh_create(p, np, f, nf, &h)); }
  TriMesh(const TriMesh&) = delete;
  ~TriMesh() {
    if (h) tm_mesh_destroy(h);
  }
  int64_t nv() const {
    int64_t a, b, c;
    tm_mesh_counts(h, &a, &b, &c);
    return a;
  }
  int64_t ne() const {
    int64_t a, b, c;
    tm_mesh_counts(h, &a, &b, &c);
    return b;
  }
  int64_t nf() const {
    int64_t a, b, c;
    tm_mesh_counts(h, &a, &b, &c);
    return c;
  }
};

TriMesh* from_points_cells(py::array points, py::array cells) {
  // empty points -> empty mesh; wrong shapes -> RuntimeError
  // (src/mesh_py.cpp:12-70)
  auto P = py::array_t<double, py::array::c_style | py::array::forcecast>::ensure(points);
  if (!P) throw std::runtime_error("Array 'points' must have shape (n,3)");
  if (P.size() == 0) return new TriMesh();
  if (P.ndim() != 2 || P.shape(1) != 3) throw std::runtime_error("Array 'points' must have shape (n,3)");
  int64_t np = P.shape(0);
  auto C = py::array_t<int32_t, py::array::c_style | py::array::forcecast>::ensure(cells);
  if (np < 3 || !C || C.size() == 0) return new TriMesh(P.data(), np, nullptr, 0);
  if (C.ndim() != 2 || C.shape(1) != 3) throw std::runtime_error("Array 'cells' must have shape (n,3)");
  return new TriMesh(P.data(), np, C.data(), C.shape(0));
}

py::array_t<int32_t> fv_indices(TriMesh& m) {
  int64_t nf = m.nf();
  if (nf == 0) return py::array_t<int32_t>();
  py::array_t<int32_t> out({(py::ssize_t)nf, (py::ssize_t)3});
  check(tm_mesh_fv_indices(m.h, out.mutable_data()));
  return out;
}

py::array_t<double> points_view(py::object self) {
  TriMesh& m = self.cast<TriMesh&>();
  int64_t nv = m.nv();
  double* p = tm_mesh_points(m.h);
  std::vector<py::ssize_t> shape = {(py::ssize_t)nv, 3};
  std::vector<py::ssize_t> strides = {3 * (py::ssize_t)sizeof(double), (py::ssize_t)sizeof(double)};
  return py::array_t<double>(shape, strides, p, self);
}

// read_mesh: OFF, OBJ and STL (ASCII or binary).  STL vertices are merged by
// exact coordinates in order of first appearance.
TriMesh* read_mesh(const std::string& fname) {
  std::ifstream in(fname, std::ios::binary);
  if (!in) throw std::runtime_error("read error on file " + fname);
  std::string data((std::istreambuf_iterator<char>(in)), std::istreambuf_iterator<char>());
  std::vector<double> P;
  std::vector<int32_t> F;
  auto ext = fname.substr(fname.find_last_of('.') + 1);
  for (auto& ch : ext) ch = (char)tolower(ch);
  auto add_stl = [&](std::map<std::tuple<double, double, double>, int>& idx, const double* v) {
    int ids[3];
    for (int k = 0; k < 3; ++k) {
      auto key = std::make_tuple(v[3 * k], v[3 * k + 1], v[3 * k + 2]);
      auto it = idx.find(key);
      if (it == idx.end()) {
        int n = (int)(P.size() / 3);
        idx[key] = n;
        P.insert(P.end(), {v[3 * k], v[3 * k + 1], v[3 * k + 2]});
        ids[k] = n;
      } else {
        ids[k] = it->second;
      }
    }
    F.insert(F.end(), {ids[0], ids[1], ids[2]});
  };
  if (ext == "off") {
    std::istringstream s(data);
    std::string tag;
    s >> tag;
    if (tag != "OFF") throw std::runtime_error("read error on file " + fname);
    long nv, nf, ne;
    s >> nv >> nf >> ne;
    P.resize(3 * nv);
    for (long i = 0; i < 3 * nv; ++i) s >> P[i];
    for (long i = 0; i < nf; ++i) {
      int k;
      s >> k;
      std::vector<int> ids(k);
      for (int q = 0; q < k; ++q) s >> ids[q];
      for (int q = 1; q + 1 < k; ++q) F.insert(F.end(), {ids[0], ids[q], ids[q + 1]});
    }
    if (!s) throw std::runtime_error("read error on file " + fname);
  } else if (ext == "obj") {
    std::istringstream s(data);
    std::string line;
    while (std::getline(s, line)) {
      std::istringstream ls(line);
      std::string t;
      ls >> t;
      if (t == "v") {
        double x, y, z;
        ls >> x >> y >> z;
        P.insert(P.end(), {x, y, z});
      } else if (t == "f") {
        std::vector<int> ids;
        std::string tok;
        while (ls >> tok) ids.push_back(std::stoi(tok.substr(0, tok.find('/'))) - 1);
        for (size_t q = 1; q + 1 < ids.size(); ++q) F.insert(F.end(), {ids[0], ids[q], ids[q + 1]});
      }
    }
  } else if (ext == "stl") {
    std::map<std::tuple<double, double, double>, int> idx;
    bool binary = data.size() >= 84;
    if (binary) {
      uint32_t n;
      std::memcpy(&n, data.data() + 80, 4);
      binary = data.size() == 84 + 50 * (size_t)n;
    }
    if (binary) {
      uint32_t n;
      std::memcpy(&n, data.data() + 80, 4);
      for (uint32_t i = 0; i < n; ++i) {
        float f[12];
        std::memcpy(f, data.data() + 84 + 50 * (size_t)i, 48);
        double v[9];
        for (int k = 0; k < 9; ++k) v[k] = f[3 + k];
        add_stl(idx, v);
      }
    } else {
      std::istringstream s(data);
      std::string tok;
      double v[9];
      int c = 0;
      while (s >> tok) {
        if (tok == "vertex") {
          s >> v[3 * c] >> v[3 * c + 1] >> v[3 * c + 2];
          if (++c == 3) {
            add_stl(idx, v);
            c = 0;
          }
        }
      }
    }
  } else {
    throw std::runtime_error("read error on file " + fname);
  }
  return new TriMesh(P.data(), (int64_t)(P.size() / 3), F.data(), (int64_t)(F.size() / 3));
}

// ---- energy manager --------------------------------------------------------
struct EnergyManager {
  tm_energy* h = nullptr;
  EnergyParams params;
  EnergyManager(TriMesh& m, const EnergyParams& p) : params(p) {
    tm_params c = to_c(p);
    if (c.n_search < 0) throw std::runtime_error("Unknown neighbour search algorithm.");
    check(tm_energy_create(m.h, &c, &h));
  }
  EnergyManager(const EnergyManager&) = delete;
  ~EnergyManager() {
    if (h) tm_energy_destroy(h);
  }
  EnergyParams eparams() const {
    tm_params c;
    tm_energy_get_params(h, &c);
    EnergyParams p = params;
    p.continuation_params.lambda = c.cont_lambda;
    return p;
  }
  VertexProperties initial_props() const {
    double a[6];
    check(tm_energy_initial_props(h, a));
    return vp_from(a);
  }
  VertexProperties properties(TriMesh& m) {
    double a[6];
    check(tm_energy_properties(h, m.h, a));
    return vp_from(a);
  }
  double energy(TriMesh& m) {
    double e;
    check(tm_energy_energy(h, m.h, &e));
    return e;
  }
  double energy_props(const VertexProperties& p) {
    double a[6] = {p.area, p.volume, p.curvature, p.bending, p.tethering, p.repulsion};
    double e;
    check(tm_energy_energy_props(h, a, &e));
    return e;
  }
  py::array_t<double> gradient(TriMesh& m) {
    py::array_t<double> out = pinned_array((py::ssize_t)m.nv(), 3);
    check(tm_energy_gradient(h, m.h, out.mutable_data(), nullptr));
    return out;
  }
  void print_info(TriMesh& m) {
    double c[7], pr[6], ref[6];
    check(tm_energy_components(h, m.h, c));
    check(tm_energy_properties(h, m.h, pr));
    tm_params p;
    tm_energy_get_params(h, &p);
    double ini[6];
    tm_energy_initial_props(h, ini);
    double lam = p.cont_lambda;
    ref[0] = (1.0 - lam * (1.0 - p.area_frac)) * ini[0];
    ref[1] = (1.0 - lam * (1.0 - p.volume_frac)) * ini[1];
    ref[2] = (1.0 - lam * (1.0 - p.curvature_frac)) * ini[2];
    std::ostream& out = std::cout;
    out << "----- EnergyManager info\n";
    out << "reference properties:\n";
    out << "  area:      " << ref[0] << "\n";
    out << "  volume:    " << ref[1] << "\n";
    out << "  curvature: " << ref[2] << "\n";
    out << "current properties:\n";
    out << "  area:      " << pr[0] << "\n";
    out << "  volume:    " << pr[1] << "\n";
    out << "  curvature: " << pr[2] << "\n";
    out << "energies:\n";
    out << "  area:      " << c[0] << "\n";
    out << "  volume:    " << c[1] << "\n";
    out << "  area diff: " << c[2] << "\n";
    out << "  bending:   " << c[3] << "\n";
    out << "  tether:    " << c[4] << "\n";
    out << "  repulsion: " << c[5] << "\n";
    out << "  total:     " << c[6] << "\n";
    out << std::endl;
  }
};

struct NeighbourList {
  tm_nlist* h = nullptr;
  int kind = 0;
  NeighbourList(TriMesh& m, const EnergyParams& p) {
    tm_params c = to_c(p);
    if (c.n_search < 0) throw std::runtime_error("Unknown neighbour search algorithm.");
    kind = c.n_search;
    check(tm_nlist_create(m.h, &c, &h));
  }
  NeighbourList(const NeighbourList&) = delete;
  ~NeighbourList() {
    if (h) tm_nlist_destroy(h);
  }
  std::tuple<std::vector<double>, std::vector<int>, std::vector<int>> distance_matrix(TriMesh& m, double rd) {
    int64_t n = 0;
    check(tm_nlist_distance_matrix(h, m.h, rd, &n));
    std::vector<double> d(n);
    std::vector<int> i(n), j(n);
    check(tm_nlist_fetch(h, d.data(), i.data(), j.data()));
    return {d, i, j};
  }
  std::tuple<std::vector<Point>, std::vector<int>> point_distances(TriMesh& m, int pid, double rd) {
    int64_t n = 0;
    check(tm_nlist_point_distances(h, m.h, pid, rd, &n));
    std::vector<double> d(3 * n);
    std::vector<int> j(n);
    check(tm_nlist_fetch(h, d.data(), nullptr, j.data()));
    std::vector<Point> pts(n);
    for (int64_t k = 0; k < n; ++k) pts[k] = Point{d[3 * k], d[3 * k + 1], d[3 * k + 2]};
    return {pts, j};
  }
};

uint64_t default_seed(py::object seed) {
  if (seed.is_none()) return (uint64_t)std::chrono::high_resolution_clock::now().time_since_epoch().count();
  return seed.cast<uint64_t>();
}

}  // namespace

PYBIND11_MODULE(core, m) {
  m.doc() = "GB300 implementation of the trimem.core API (energy, gradient, neighbour lists, flips).";

  py::class_<HalfedgeHandle>(m, "HalfedgeHandle")
      .def(py::init())
      .def("idx", [](const HalfedgeHandle& h) { return h.h; })
      .def("is_valid", [](const HalfedgeHandle& h) { return h.h >= 0; })
      .def("__repr__", [](const HalfedgeHandle& h) { return "HalfedgeHandle(" + std::to_string(h.h) + ")"; });

  py::class_<TriMesh>(m, "TriMesh")
      .def(py::init([]() { return new TriMesh(); }))
      .def(py::init(&from_points_cells), py::arg("points"), py::arg("faces"))
      .def("fv_indices", &fv_indices)
      .def("points", &points_view)
      .def("n_vertices", [](TriMesh& t) { return t.nv(); })
      .def("n_edges", [](TriMesh& t) { return t.ne(); })
      .def("n_faces", [](TriMesh& t) { return t.nf(); })
      .def(
          "halfedge_handle",
          [](TriMesh& t, int64_t i) {
            int64_t o;
            check(tm_mesh_halfedge(t.h, 0, i, &o));
            return HalfedgeHandle{o};
          },
          py::arg("edge"))
      .def(
          "opposite_halfedge_handle",
          [](TriMesh& t, const HalfedgeHandle& he) {
            int64_t o;
            check(tm_mesh_halfedge(t.h, 2, he.h, &o));
            return HalfedgeHandle{o};
          },
          py::arg("edge"))
      .def(
          "next_halfedge_handle",
          [](TriMesh& t, const HalfedgeHandle& he) {
            int64_t o;
            check(tm_mesh_halfedge(t.h, 1, he.h, &o));
            return HalfedgeHandle{o};
          },
          py::arg("edge"))
      .def("check", [](TriMesh& t) {
        int s = 0;
        check(tm_mesh_check(t.h, &s));
        return s;
      })
      .def("topology", [](TriMesh& t) {
        int64_t nv = t.nv(), ne = t.ne(), nf = t.nf();
        py::array_t<int32_t> to(2 * ne), nx(2 * ne), fc(2 * ne), vo(nv), fh(nf);
        check(tm_mesh_topology(t.h, to.mutable_data(), nx.mutable_data(), fc.mutable_data(), vo.mutable_data(),
                               fh.mutable_data()));
        py::dict d;
        d["to"] = to;
        d["next"] = nx;
        d["face"] = fc;
        d["vout"] = vo;
        d["fhe"] = fh;
        return d;
      })
      .def("__deepcopy__", [](py::object self, py::dict) {
        TriMesh& t = self.cast<TriMesh&>();
        auto f = fv_indices(t);
        int64_t nv = t.nv();
        return new TriMesh(tm_mesh_points(t.h), nv, f.size() ? f.data() : nullptr, t.nf());
      });

  m.def("read_mesh", &read_mesh, py::arg("fname"));

  py::class_<VertexProperties>(m, "VertexProperties")
      .def(py::init())
      .def_readwrite("area", &VertexProperties::area)
      .def_readwrite("volume", &VertexProperties::volume)
      .def_readwrite("curvature", &VertexProperties::curvature)
      .def_readwrite("bending", &VertexProperties::bending)
      .def_readwrite("tethering", &VertexProperties::tethering)
      .def_readwrite("repulsion", &VertexProperties::repulsion);

  auto prim = [](int which) {
    return [which](TriMesh& t, const HalfedgeHandle& he) {
      double v;
      int rc = which == 0   ? tm_edge_length(t.h, he.h, &v, nullptr)
               : which == 1 ? tm_face_area(t.h, he.h, &v, nullptr)
               : which == 2 ? tm_face_volume(t.h, he.h, &v, nullptr)
                            : tm_dihedral_angle(t.h, he.h, &v, nullptr);
      check(rc);
      return v;
    };
  };
  auto primg = [](int which) {
    return [which](TriMesh& t, const HalfedgeHandle& he) {
      int rows = which == 0 ? 2 : (which == 3 ? 4 : 3);
      py::array_t<double> g({(py::ssize_t)rows, (py::ssize_t)3});
      double v;
      int rc = which == 0   ? tm_edge_length(t.h, he.h, &v, g.mutable_data())
               : which == 1 ? tm_face_area(t.h, he.h, &v, g.mutable_data())
               : which == 2 ? tm_face_volume(t.h, he.h, &v, g.mutable_data())
                            : tm_dihedral_angle(t.h, he.h, &v, g.mutable_data());
      check(rc);
      return g;
    };
  };
  m.def("edge_length", prim(0), py::arg("mesh"), py::arg("halfedge_handle"));
  m.def("edge_length_grad", primg(0), py::arg("mesh"), py::arg("halfedge_handle"));
  m.def("face_area", prim(1), py::arg("mesh"), py::arg("halfedge_handle"));
  m.def("face_area_grad", primg(1), py::arg("mesh"), py::arg("halfedge_handle"));
  m.def("face_volume", prim(2), py::arg("mesh"), py::arg("halfedge_handle"));
  m.def("face_volume_grad", primg(2), py::arg("mesh"), py::arg("halfedge_handle"));
  m.def("dihedral_angle", prim(3), py::arg("mesh"), py::arg("halfedge_handle"));
  m.def("dihedral_angle_grad", primg(3), py::arg("mesh"), py::arg("halfedge_handle"));

  py::enum_<BondType>(m, "BondType")
      .value("Edge", BondType::Edge)
      .value("Area", BondType::Area)
      .value("None", BondType::None);

  py::class_<BondParams>(m, "BondParams")
      .def(py::init())
      .def_readwrite("lc0", &BondParams::lc0)
      .def_readwrite("lc1", &BondParams::lc1)
      .def_readwrite("a0", &BondParams::a0)
      .def_readwrite("r", &BondParams::r)
      .def_readwrite("type", &BondParams::type);

  py::class_<SurfaceRepulsionParams>(m, "SurfaceRepulsionParams")
      .def(py::init())
      .def_readwrite("lc1", &SurfaceRepulsionParams::lc1)
      .def_readwrite("r", &SurfaceRepulsionParams::r)
      .def_readwrite("n_search", &SurfaceRepulsionParams::n_search)
      .def_readwrite("rlist", &SurfaceRepulsionParams::rlist)
      .def_readwrite("exclusion_level", &SurfaceRepulsionParams::exclusion_level);

  py::class_<ContinuationParams>(m, "ContinuationParams")
      .def(py::init())
      .def_readwrite("delta", &ContinuationParams::delta)
      .def_readwrite("lam", &ContinuationParams::lambda);

  py::class_<EnergyParams>(m, "EnergyParams")
      .def(py::init())
      .def_readwrite("kappa_b", &EnergyParams::kappa_b)
      .def_readwrite("kappa_a", &EnergyParams::kappa_a)
      .def_readwrite("kappa_v", &EnergyParams::kappa_v)
      .def_readwrite("kappa_c", &EnergyParams::kappa_c)
      .def_readwrite("kappa_t", &EnergyParams::kappa_t)
      .def_readwrite("kappa_r", &EnergyParams::kappa_r)
      .def_readwrite("area_frac", &EnergyParams::area_frac)
      .def_readwrite("volume_frac", &EnergyParams::volume_frac)
      .def_readwrite("curvature_frac", &EnergyParams::curvature_frac)
      .def_readwrite("bond_params", &EnergyParams::bond_params)
      .def_readwrite("repulse_params", &EnergyParams::repulse_params)
      .def_readwrite("continuation_params", &EnergyParams::continuation_params);

  py::class_<EnergyManager>(m, "EnergyManager")
      .def(py::init<TriMesh&, const EnergyParams&>(), py::arg("mesh"), py::arg("eparams"))
      .def("properties", &EnergyManager::properties, py::arg("mesh"))
      .def("energy", &EnergyManager::energy, py::arg("mesh"))
      .def("energy", &EnergyManager::energy_props, py::arg("vprops"))
      .def("gradient", &EnergyManager::gradient, py::arg("mesh"))
      .def("update_reference_properties",
           [](EnergyManager& e) { check(tm_energy_update_reference_properties(e.h)); })
      .def("update_repulsion", [](EnergyManager& e, TriMesh& t) { check(tm_energy_update_repulsion(e.h, t.h)); })
      .def("print_info", &EnergyManager::print_info,
           py::call_guard<py::scoped_ostream_redirect, py::scoped_estream_redirect>(), py::arg("mesh"))
      .def_property_readonly("eparams", &EnergyManager::eparams)
      .def_property_readonly("initial_props", &EnergyManager::initial_props)
      // GB300 additions
      .def(
          "vertex_properties",
          [](EnergyManager& e, TriMesh& t) {
            py::array_t<double> out({(py::ssize_t)t.nv(), (py::ssize_t)6});
            check(tm_energy_vertex_properties(e.h, t.h, out.mutable_data()));
            return out;
          },
          py::arg("mesh"))
      .def(
          "energy_gradient",
          [](EnergyManager& e, TriMesh& t) {
            py::array_t<double> out = pinned_array((py::ssize_t)t.nv(), 3);
            double en = 0;
            check(tm_energy_gradient(e.h, t.h, out.mutable_data(), &en));
            return py::make_tuple(en, out);
          },
          py::arg("mesh"))
      .def(
          "set_stencil_precision",
          [](EnergyManager& e, const std::string& p) {
            int mode = p == "fp64" ? 0 : (p == "fp32" ? 1 : (p == "df64" ? 2 : -1));
            if (mode < 0) throw py::value_error("precision must be 'fp64', 'fp32' or 'df64'");
            check(tm_energy_set_stencil_precision(e.h, mode));
          },
          py::arg("precision"))
      .def(
          "eval_device",
          [](EnergyManager& e, TriMesh& t, uintptr_t x, uintptr_t g, uintptr_t en, uintptr_t stream) {
            check(tm_energy_eval_device(e.h, t.h, (const double*)x, (double*)g, (double*)en, (void*)stream));
          },
          py::arg("mesh"), py::arg("x_ptr"), py::arg("grad_ptr"), py::arg("energy_ptr"), py::arg("stream") = 0)
      .def(
          "update_repulsion_device",
          [](EnergyManager& e, TriMesh& t, uintptr_t x, uintptr_t stream) {
            check(tm_energy_update_repulsion_device(e.h, t.h, (const double*)x, (void*)stream));
          },
          py::arg("mesh"), py::arg("x_ptr"), py::arg("stream") = 0)
      .def(
          "hmc_step_device",
          [](EnergyManager& e, TriMesh& t, uintptr_t x, double mass, double dt, int n_steps, double temp,
             uint64_t seed, uint64_t step, double u, uintptr_t stream) {
            double out[4];
            check(tm_hmc_step_device(e.h, t.h, (double*)x, mass, dt, n_steps, temp, seed, step, u, out, nullptr,
                                     (void*)stream));
            return py::make_tuple(out[0] != 0.0, out[1], out[2], out[3]);
          },
          py::arg("mesh"), py::arg("x_ptr"), py::arg("mass"), py::arg("dt"), py::arg("n_steps"),
          py::arg("temperature"), py::arg("seed"), py::arg("step"), py::arg("u"), py::arg("stream") = 0);

  m.def(
      "flip",
      [](TriMesh& t, EnergyManager& e, double ratio, py::object seed) {
        int32_t acc = 0;
        check(tm_flip(t.h, e.h, ratio, default_seed(seed), 0, 256, &acc));
        return acc;
      },
      py::arg("mesh"), py::arg("estore"), py::arg("flip_ratio"), py::arg("seed") = py::none());
  m.def(
      "pflip",
      [](TriMesh& t, EnergyManager& e, double ratio, py::object seed, int batch) {
        int32_t acc = 0;
        check(tm_flip(t.h, e.h, ratio, default_seed(seed), 1, batch, &acc));
        return acc;
      },
      py::arg("mesh"), py::arg("estore"), py::arg("flip_ratio"), py::arg("seed") = py::none(),
      py::arg("batch") = 4096);

  py::class_<Point>(m, "Point")
      .def("__getitem__",
           [](const Point& p, int k) {
             if (k < 0 || k > 2) throw py::index_error();
             return k == 0 ? p.x : (k == 1 ? p.y : p.z);
           })
      .def("__len__", [](const Point&) { return 3; })
      .def("__repr__", [](const Point& p) {
        char b[128];
        snprintf(b, sizeof(b), "Point(%.17g, %.17g, %.17g)", p.x, p.y, p.z);
        return std::string(b);
      });

  py::class_<NeighbourList>(m, "NeighbourList")
      .def("distance_matrix", &NeighbourList::distance_matrix, py::arg("mesh"), py::arg("rdist"))
      .def("point_distances", &NeighbourList::point_distances, py::arg("mesh"), py::arg("pid"), py::arg("rdist"));

  m.def(
      "make_nlist", [](TriMesh& t, const EnergyParams& p) { return new NeighbourList(t, p); }, py::arg("mesh"),
      py::arg("eparams"));

  m.def(
      "area",
      [](TriMesh& t) {
        double a;
        check(tm_area(t.h, &a));
        return a;
      },
      py::arg("mesh"));
  m.def(
      "edges_length",
      [](TriMesh& t) {
        double a;
        check(tm_edges_length(t.h, &a));
        return a;
      },
      py::arg("mesh"));
  m.def(
      "avg_tri_props",
      [](TriMesh& t) {
        double a, l;
        check(tm_avg_tri_props(t.h, &a, &l));
        return py::make_tuple(a, l);
      },
      py::arg("mesh"));

  m.def(
      "gradient",
      [](TriMesh& t, EnergyManager& e, py::array_t<double, py::array::c_style> grad, double eps) {
        if (grad.ndim() != 2 || grad.shape(0) != t.nv() || grad.shape(1) != 3)
          throw std::runtime_error("gradient must have shape (n_vertices, 3)");
        check(tm_fd_gradient(t.h, e.h, eps, grad.mutable_data()));
      },
      py::arg("mesh"), py::arg("estore"), py::arg("gradient"), py::arg("epsilon"));

  m.def("device_name", []() {
    char b[256];
    check(tm_device_name(b, sizeof(b)));
    return std::string(b);
  });
}
