// Internal declarations shared by the translation units of libtrimem_gpu.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "trimem_gpu.h"

namespace tmg {

// Errors travel as exceptions inside the library and become a status code
// plus tm_last_error() text at the C ABI.
struct Error : std::runtime_error {
  int code;
  Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};
void set_last_error(const std::string& m);
[[noreturn]] void fail(int code, const std::string& m);
void cuda_check(cudaError_t e, const char* what, const char* file, int line);
#define TM_CUDA(x) ::tmg::cuda_check((x), #x, __FILE__, __LINE__)
#define TM_LAUNCH() ::tmg::cuda_check(cudaGetLastError(), "kernel launch", __FILE__, __LINE__)

// Owning device buffer (no copy; grows on demand).
template <class T>
struct DevBuf {
  T* p = nullptr;
  size_t n = 0;
  DevBuf() = default;
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  ~DevBuf() { release(); }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
  }
  void ensure(size_t count) {
    if (count <= n && p) return;
    release();
    size_t c = count ? count : 1;
    if (cudaMalloc(&p, c * sizeof(T)) != cudaSuccess) {
      cudaGetLastError();
      p = nullptr;
      fail(TM_ERR_NOMEM, "device allocation of " + std::to_string(c * sizeof(T)) + " bytes failed");
    }
    n = c;
  }
  T* get() const { return p; }
};

// One ring slot of a vertex v (slot-major tables [TM_MAXVAL][nv]):
//   x: neighbour r_m (target of the m-th outgoing halfedge h_m)
//   y: face of h_m in bits 0..29, corner of v in that face's stored vertex
//      order in bits 30..31; -1 (all bits) on a boundary halfedge
//   z: edge of h_m
//   w: edge of next(h_m), the edge opposite v in the face
// Slots follow the rotation h -> next(opposite(h)), so the face of slot m is
// (v, r_m, r_{m-1}) in face orientation.
__host__ __device__ inline int slot_face(int y) { return y == -1 ? -1 : (y & 0x3fffffff); }
__host__ __device__ inline int slot_corner(int y) { return (int)(((unsigned)y) >> 30); }

// Read-only topology view handed to kernels.
struct Topo {
  int nv, ne, nf;
  const int* to;
  const int* next;
  const int* face;
  const int* vout;
  const int* fhe;
  const int4* slot;  // [TM_MAXVAL][nv]
  const int* nbr;    // [TM_MAXVAL][nv]
  const int* val;    // [nv]
  const int* fv;     // [3*nf]
  const int4* edge;  // [ne]: from, to, face of 2e, face of 2e+1
};

// Neighbour-list view used by the repulsion penalty.
struct CellEntry {
  long long key;  // cell id, -1 empty
  int start, count;
};
// Cell geometry, derived on the device from the bounding box.
struct NLGeom {
  double bmin[3], rl[3], inv_rl[3];
  float bminf[3], inv_rlf[3];  // float copies for the fast binning test
  int shape[3];
  int pad;
  long long stride[3];
};
constexpr int TM_NEAR_CAP = 48;  // near-row capacity per vertex
// grid of dihedral angles k/128, k < TM_SCT_N (covers [0, pi]), whose sine
// and cosine each energy handle keeps on the device
constexpr int TM_SCT_N = 404;

struct NLView {
  int kind;  // 0 cell list, 1 Verlet list
  int excl;  // exclusion level; for a batch the largest of its replicas' levels
  // batch of replicas: each replica's exclusion level (by vrep), else NULL
  const int* rexcl;
  // cell geometry; for a batch of replicas one entry per replica selected by
  // vrep (vertex -> replica), and hash keys carry the replica in bits 44+
  const NLGeom* geom;
  const int* vrep;
  const CellEntry* table;
  unsigned long long tmask;
  const int* cell_verts;
  const int* vrow;  // Verlet CSR
  const int* vcol;
  // cell list: members of the 27 build-time neighbour cells of each vertex
  // (reference scan order, self excluded), used while the query point is
  // still inside its build cell
  const int* crow;
  const int* ccol;
  const int* bcoord;   // build-time cell coordinates, 3 per vertex
  const float* pos32;  // positions rounded to float (prefilter), may be NULL
  // near rows: per vertex (fixed stride TM_NEAR_CAP) the vertices closer
  // than 2 lc1 when the rows were built, bit 31 set when the pair was
  // excluded on the topology of that time; ncnt = row lengths.  nflag[0]:
  // some vertex moved lc1/2 or more since (set per evaluation), nflag[1]:
  // rows unusable (never built, overflow), nflag[2]: device topology
  // version at the build; dtopo: the mesh's current device topology version
  const int* nent;
  const int* ncnt;
  const int* nflag;
  const int* dtopo;
};

#ifdef __CUDACC__
__device__ __forceinline__ int rep_of(const NLView& nl, int v) { return nl.vrep ? nl.vrep[v] : 0; }
__device__ __forceinline__ const NLGeom& geom_of(const NLView& nl, int v) { return nl.geom[rep_of(nl, v)]; }
__device__ __forceinline__ long long cell_key(long long cid, int rep) { return cid + ((long long)rep << 44); }
// exclusion level that applies to vertex v
__device__ __forceinline__ int excl_of(const NLView& nl, int v) { return nl.rexcl ? nl.rexcl[rep_of(nl, v)] : nl.excl; }
#endif

struct TopoW;

}  // namespace tmg

// --------------------------------------------------------------------------
// Handles (opaque in the C ABI)
// --------------------------------------------------------------------------
struct tm_surrogate;  // surrogate.cu

struct tm_mesh {
  int nv = 0, ne = 0, nf = 0;
  bool closed = true;
  double* h_pts = nullptr;  // page-locked host positions (points() view)
  std::vector<int> h_to, h_next, h_face, h_vout, h_fhe;
  bool host_topo_stale = false;
  tmg::DevBuf<double> d_pts;
  tmg::DevBuf<int> d_to, d_next, d_face, d_vout, d_fhe;
  tmg::DevBuf<int4> d_slot;
  tmg::DevBuf<int> d_nbr, d_val, d_fv;
  tmg::DevBuf<int4> d_edge;
  tmg::DevBuf<double> d_scratch;  // primitives / utilities
  tmg::DevBuf<int> d_status;
  tmg::DevBuf<int> d_topo_ver;  // device copy of topo_version (low 31 bits)
  cudaStream_t stream = nullptr;
  unsigned long long topo_version = 0;  // advanced by every flip sweep that flips
  tmg::Topo topo() const;
  tmg::TopoW topo_w();
  void rebuild_tables(cudaStream_t s);  // faces, edges, rings from halfedges
  void upload_points(cudaStream_t s);
  void sync_host_topology();
  ~tm_mesh();
};

struct tm_nlist {
  tmg::NLView view{};
  tm_params prm{};
  int nv = 0;
  tmg::DevBuf<tmg::CellEntry> table;
  tmg::DevBuf<int> cell_verts, vslot, vcoord, vrank, cnt, fill, vrow, vcol, crow, ccol, tmp;
  tmg::DevBuf<tmg::NLGeom> geom;
  tmg::DevBuf<long long> vcid;
  tmg::DevBuf<double> bbox;
  // near rows (see NLView) and what they were built for
  tmg::DevBuf<int> nent, ncnt, nflag;
  tmg::DevBuf<double> xb;  // positions when the near rows were built
  double near_lc1 = 0.0, near_move2 = 0.0;
  int near_nv = -1;
  // last query result
  std::vector<double> res_d;
  std::vector<int> res_i, res_j;
  tmg::DevBuf<double> d_res;
  tmg::DevBuf<int> d_resi, d_resj, d_count;
  void build(tm_mesh* m, const double* d_points, cudaStream_t s);
};

namespace tmg {
struct EP;
// device-side scalar state of an energy manager
struct Globals {
  double props[8];  // area, volume, curvature, bending, tethering, repulsion
  double comps[8];  // area, volume, area-diff, bending, tether, repulsion, total
  double gA, gV, gC;
  float gdf[6];  // gA, gV, gC as double-float (hi, lo) pairs
  unsigned int ticket;
  int status;
};
}  // namespace tmg

struct tm_energy {
  tm_params prm{};
  double initial[6] = {0, 0, 0, 0, 0, 0};
  int stencil = 2;  // 0 FP64, 1 FP32, 2 double-word (FP64-accurate, FP32 pipe; the default)
  tm_nlist nl;
  int nv = 0, ne = 0, nf = 0;
  tmg::DevBuf<double> face, edge, ebond, fav, rho, repg, reppot, vprops, partials, grad, work;
  tmg::DevBuf<int> slow;  // vertices that left their build cell (+ count)
  tmg::DevBuf<float> pos32, poslo;
  tmg::DevBuf<float4> posdw;  // double-word stencils: hi parts [nv], lo parts [nv]
  tmg::DevBuf<tmg::Globals> glob;
  tmg::DevBuf<double2> sct;  // {sin, cos}(k / 128), k < TM_SCT_N
  tmg::DevBuf<float4> sctf;  // the same as double-words (sin hi, sin lo, cos hi, cos lo)
  // flip-sweep workspace, kept between sweeps (grown on demand)
  tmg::DevBuf<int> fw_owner, fw_limit, fw_accl;
  tmg::DevBuf<long long> fw_win, fw_pend;
  tmg::DevBuf<unsigned char> fw_winner, fw_state;
  tmg::DevBuf<double> fw_dpn;
  tmg::DevBuf<float> fw_dpf;
  cudaStream_t stream = nullptr;
  // second stream: the repulsion pass runs there, concurrent with the
  // edge kernels, between a fork and a join event
  cudaStream_t aux = nullptr;
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
  // FP64 evaluation graphs (captured launch sequences), each with the key
  // of what its launches depend on; a few are kept (with and without the
  // gradient, several position buffers), the least recently used is replaced
  struct EvalGraph {
    std::vector<unsigned char> key;
    cudaGraphExec_t exec = nullptr;
    unsigned long long used = 0;
  };
  bool use_graphs = true;
  std::vector<EvalGraph> eval_graphs;
  unsigned long long eval_tick = 0;
  EvalGraph flip_graph;  // one group of flip-sweep windows
  int flip_coop = 0;     // claim + winner as one cooperative launch: 0 unknown, 1 yes, -1 no
  void ensure(int nv_, int ne_, int nf_);
  // copies n doubles from device memory to host memory dst and synchronises
  void to_host(double* dst, const double* src, size_t n);
  ~tm_energy();
};

namespace tmg {
// energy.cu
void energy_eval(tm_energy* e, tm_mesh* m, const double* d_points, bool want_grad, bool want_vprops,
                 double* d_grad, cudaStream_t s);
// same, recording ev[0..4] around the face, edge, vertex and gradient kernels
void energy_eval_marked(tm_energy* e, tm_mesh* m, const double* d_points, bool want_grad, bool want_vprops,
                        double* d_grad, cudaStream_t s, cudaEvent_t* ev);
// repulsion stage: per-vertex potential (and 2 x its gradient) into pot /
// repg; slow must hold nv + 1 ints
void repulsion_eval(tm_energy* e, tm_mesh* m, const double* P, const float* pos32, bool want_grad, double* pot,
                    double* repg, int* slow, int* nslow, cudaStream_t s, const EP* eps = nullptr);
// the repulsion pass of an evaluation into e->reppot / e->repg, started on
// e->aux after the work already queued on s (concurrent = false: on s);
// join_repulsion makes s wait for it
void fork_repulsion(tm_energy* e, tm_mesh* m, const double* P, bool want_grad, cudaStream_t s, bool concurrent);
void join_repulsion(tm_energy* e, cudaStream_t s, bool concurrent);
// learned surrogate gradient (surrogate.cu)
void surrogate_grad(tm_surrogate* sg, tm_energy* e, tm_mesh* m, const double* d_points, double* d_grad,
                    cudaStream_t s);
// local terms only (bending and repulsion weights zero), FP32 stencils
void energy_eval32_local(tm_energy* e, tm_mesh* m, const double* d_points, double* d_grad, cudaStream_t s);
// batch of replicas, FP32 stencils and FP64 sums per replica.  A size class
// is a run of consecutive replicas of similar size: its vertex, face and
// edge ranges in the union mesh and the block sizes tuned for it
// {split, face, edge, gradient}.
struct BatchClass {
  int v0, v1, f0, f1, e0, e1;
  int blk[4];
};
constexpr int TM_MAX_CLASSES = 8;
// side streams of the classes and the fork / join events between them
struct BatchStreams {
  cudaStream_t cs[TM_MAX_CLASSES];
  cudaEvent_t fork[2], join[TM_MAX_CLASSES];
};
void energy_eval_batch32(tm_energy* e, tm_mesh* m, const double* d_points, double* d_grad, const EP* eps,
                         const int* vrep, const int2* rblocks, Globals* gs, const BatchClass* cls, int ncls,
                         const BatchStreams* bs, cudaStream_t s);
void batch32_class_kernel(int which, const BatchClass& c, int blk, tm_energy* e, tm_mesh* m, const double* P,
                          double* d_grad, const EP* eps, const int* vrep, const Globals* gs, cudaStream_t s);
// double-float stencil variant (stencil mode 2)
void energy_eval_df(tm_energy* e, tm_mesh* m, const double* d_points, bool want_grad, double* d_grad,
                    cudaStream_t s, cudaEvent_t* ev);
// FP32-stencil variant (stencil mode 1); per-vertex properties are not
// produced by it
void energy_eval32(tm_energy* e, tm_mesh* m, const double* d_points, bool want_grad, bool want_vprops,
                   double* d_grad, cudaStream_t s, cudaEvent_t* ev);
void energy_from_props_device(tm_energy* e, const double* d_props6, double* d_out8, cudaStream_t s);
// nlist.cu
void nlist_make(tm_nlist* nl, tm_mesh* m, const tm_params& p, const double* d_points, cudaStream_t s);
int64_t nlist_distance_matrix(tm_nlist* nl, tm_mesh* m, const double* d_points, double rdist, cudaStream_t s);
// cell list over a batch of replicas (disjoint-union mesh with replica-aligned
// 256-vertex blocks): per-replica boxes and cut-offs, replica-tagged cells
// excl: the largest level of the replicas, d_rexcl: each replica's level;
// verlet: Verlet rows at each replica's cut-off on top of the cells
void nlist_make_batch(tm_nlist* nl, tm_mesh* m, int R, const int* d_vrep, const int2* d_rblocks,
                      const double* d_rlist, int excl, const int* d_rexcl, const double* d_points, cudaStream_t s,
                      const EP* d_eps, bool near, bool verlet);
int64_t nlist_point_distances(tm_nlist* nl, tm_mesh* m, const double* d_points, int pid, double rdist,
                              cudaStream_t s);
// smallest double T with sqrt(T) >= d (IEEE round-to-nearest sqrt), so that
// sqrt(s) < d  <=>  s < T for every double s >= 0
double sq_threshold(double d);
// scan.cu helpers
void exclusive_scan_int(const int* in, int* out, int n, int* total_host, DevBuf<int>& tmp, cudaStream_t s);
}  // namespace tmg
