/*
 * Oracle for the trimem energy / gradient / neighbour-list / edge-flip path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a CPU restatement (C++17 + OpenMP) of
 * the reference's algorithms.  It is used by the test-suite as the checker,
 * by smoke() as the checker, and by bench.py as the timed CPU baseline.  The
 * product (trimem_gb300) never links, imports or calls it.
 *
 * The reference itself cannot be compiled (its OpenMesh submodule is empty),
 * so the half-edge mesh semantics of OpenMesh that the reference relies on
 * (add_face, circulators, flip, is_flip_ok, calc_sector_*, calc_dihedral_*)
 * are restated from their documented behaviour in oracle.cpp.
 *
 * Plain C ABI so that Python reaches it through ctypes.
 */
#ifndef TRIMEM_ORACLE_H
#define TRIMEM_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Energy parameters: the fields of EnergyParams / BondParams /
 * SurfaceRepulsionParams / ContinuationParams (src/params.h:11-71). */
typedef struct om_params {
  double kappa_b, kappa_a, kappa_v, kappa_c, kappa_t, kappa_r;
  double area_frac, volume_frac, curvature_frac;
  double bond_lc0, bond_lc1, bond_a0;
  int32_t bond_r, bond_type; /* 0 Edge, 1 Area, 2 None */
  double rep_lc1;
  int32_t rep_r, n_search; /* 0 cell-list, 1 verlet-list */
  double rlist;
  int32_t exclusion_level, pad0;
  double cont_delta, cont_lambda;
} om_params;

const char* om_last_error(void);
void om_set_threads(int n);
int om_get_threads(void);

/* mesh (src/mesh_py.cpp:12-70 construction semantics) */
void* om_mesh_create(const double* pts, int nv, const int* faces, int nf);
void* om_mesh_clone(void* m);
void om_mesh_destroy(void* m);
int om_mesh_nv(void* m);
int om_mesh_ne(void* m);
int om_mesh_nf(void* m);
double* om_mesh_points(void* m);
void om_mesh_fv(void* m, int* out);
void om_mesh_topology(void* m, int* he_to, int* he_next, int* he_face, int* v_out, int* f_he);
int om_mesh_next(void* m, int h);
int om_mesh_to(void* m, int h);
int om_mesh_check(void* m); /* 0 = valid closed/open manifold; <0 otherwise */

/* geometry primitives (src/mesh_util.h:15-185); grads row-major (k,3) */
double om_edge_length(void* m, int he);
void om_edge_length_grad(void* m, int he, double* out6);
double om_face_area(void* m, int he);
void om_face_area_grad(void* m, int he, double* out9);
double om_face_volume(void* m, int he);
void om_face_volume_grad(void* m, int he, double* out9);
double om_dihedral_angle(void* m, int he);
void om_dihedral_angle_grad(void* m, int he, double* out12);

/* energy manager (src/energy.cpp) */
void* om_energy_create(void* m, const om_params* p);
void om_energy_destroy(void* e);
void om_energy_properties(void* e, void* m, double* out6);
void om_energy_vertex_properties(void* e, void* m, double* out6v);
double om_energy_energy(void* e, void* m);
double om_energy_energy_props(void* e, const double* props6);
void om_energy_components(void* e, void* m, double* out7);
void om_energy_gradient(void* e, void* m, double* out3v);
void om_energy_update_reference(void* e);
void om_energy_update_repulsion(void* e, void* m);
void om_energy_initial_props(void* e, double* out6);
/* reference properties of a chain started elsewhere (the reference's
 * checkpoint restart keeps the original initial properties) */
void om_energy_set_initial_props(void* e, const double* props6);
void om_energy_ref_props(void* e, double* out6);
double om_energy_lambda(void* e);

/* neighbour lists (src/nlists) */
void* om_nlist_create(void* m, int n_search, int exclusion, double rlist);
void om_nlist_destroy(void* nl);
int64_t om_nlist_distance_matrix(void* nl, void* m, double dmax);
int64_t om_nlist_point_distances(void* nl, void* m, int pid, double dmax);
void om_nlist_fetch(void* nl, double* d, int* i, int* j);
void om_nlist_fetch_points(void* nl, double* d3, int* j);
void om_nlist_cell_info(void* nl, double* box6, double* rl3, int* shape3);

/* flips (src/flips.cpp) */
int om_flip_serial(void* m, void* e, double ratio, uint64_t seed);
int om_flip_parallel(void* m, void* e, double ratio, uint64_t seed);
/* CPU port of the device flip sweep: windows of proposals whose quads lie
 * at least two edges from the quads of lower slots of the window (vertex
 * patches: the quad's vertices and their ring neighbours), sequential
 * Metropolis in proposal order; mode 0 = window is the longest conflict-free
 * prefix (serial order), 1 = batch with deferral. */
int om_flip_windowed(void* m, void* e, double ratio, uint64_t seed, int mode, int batch);

/* utilities (src/util.cpp) and the FD gradient (src/bindings.cpp:25-50) */
double om_area(void* m);
double om_edges_length(void* m);
void om_fd_gradient(void* m, void* e, double eps, double* out3v);

/* time `n` energy+gradient evaluations; returns seconds */
double om_time_energy_gradient(void* e, void* m, int n);

#ifdef __cplusplus
}
#endif
#endif
