/*
 * trimem_gb300 C ABI -- the drop-in boundary of the GB300 implementation of
 * trimem's energy / gradient / neighbour-list / edge-flip path.
 *
 * Every entry point takes plain pointers and sizes, returns an int status
 * (TM_OK == 0, negative on failure) and leaves a message for
 * tm_last_error().  Calls are synchronous with respect to the host unless the
 * name ends in _device; a handle is not re-entrant (one CUDA stream each).
 *
 * Reference interfaces are cited as path:line within bio-phys/trimem.
 */
#ifndef TRIMEM_GPU_H
#define TRIMEM_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
  TM_OK = 0,
  TM_ERR_ARG = -1,      /* invalid argument (RuntimeError / ValueError)   */
  TM_ERR_CUDA = -2,     /* CUDA runtime failure                            */
  TM_ERR_TOPOLOGY = -3, /* non-manifold input or valence above TM_MAXVAL   */
  TM_ERR_RANGE = -4,    /* std::range_error in the reference (flip ratio)   */
  TM_ERR_TIMEOUT = -5,  /* a bounded device wait gave up                    */
  TM_ERR_NOMEM = -6     /* device or pinned allocation failed               */
};

/* Largest vertex valence the device ring tables hold. */
#define TM_MAXVAL 32

/* EnergyParams with its nested BondParams, SurfaceRepulsionParams and
 * ContinuationParams flattened (src/params.h:11-71). */
typedef struct tm_params {
  double kappa_b, kappa_a, kappa_v, kappa_c, kappa_t, kappa_r;
  double area_frac, volume_frac, curvature_frac;
  double bond_lc0, bond_lc1, bond_a0;
  int32_t bond_r, bond_type; /* BondType: 0 Edge, 1 Area, 2 None */
  double rep_lc1;
  int32_t rep_r, n_search; /* n_search: 0 "cell-list", 1 "verlet-list" */
  double rlist;
  int32_t exclusion_level, pad0;
  double cont_delta, cont_lambda;
} tm_params;

typedef struct tm_mesh tm_mesh;
typedef struct tm_energy tm_energy;
typedef struct tm_nlist tm_nlist;

const char* tm_last_error(void);
/* Name of the CUDA device the library runs on; fails when none is present. */
int tm_device_name(char* buf, int len);
/* Page-locked host memory (results copied there from the device need no
 * staging); the Python module hands such buffers to numpy. */
int tm_host_alloc(int64_t bytes, void** out);
int tm_host_free(void* p);

/* ---- mesh ---------------------------------------------------------------
 * TriMesh(points, faces): src/bindings.cpp:87-109, src/mesh_py.cpp:12-70.
 * Face entries outside [0, n_points) are dropped; faces with fewer than three
 * valid vertices, repeated vertices or an already used directed edge are
 * skipped.  Edge e owns halfedges 2e and 2e+1. */
int tm_mesh_create(const double* points, int64_t n_points, const int32_t* faces, int64_t n_faces,
                   tm_mesh** out);
int tm_mesh_destroy(tm_mesh* m);
int tm_mesh_counts(tm_mesh* m, int64_t* n_vertices, int64_t* n_edges, int64_t* n_faces);
/* Host copy of the positions (TriMesh.points(), src/mesh_py.cpp:96-106).
 * It is page-locked and stays valid for the life of the mesh; callers write
 * it in place and every host-side compute call uploads it. */
double* tm_mesh_points(tm_mesh* m);
/* TriMesh.fv_indices (src/mesh_py.cpp:73-93); out is (n_faces, 3). */
int tm_mesh_fv_indices(tm_mesh* m, int32_t* out);
/* Half-edge queries (src/bindings.cpp:147-175).  op: 0 halfedge_handle(edge
 * = h) (first halfedge), 1 next, 2 opposite, 3 to-vertex, 4 from-vertex,
 * 5 face (-1 on boundary). */
int tm_mesh_halfedge(tm_mesh* m, int op, int64_t h, int64_t* out);
/* Whole topology: to/next/face per halfedge, outgoing halfedge per vertex,
 * halfedge per face (any pointer may be NULL). */
int tm_mesh_topology(tm_mesh* m, int32_t* to, int32_t* next, int32_t* face, int32_t* vout, int32_t* fhe);
/* replaces the connectivity by half-edge arrays of the same sizes (as
 * tm_mesh_topology returns them, e.g. of a flipped mesh saved in a
 * checkpoint), so that edge and face numbering are restored too; validated
 * (ranges, triangles, manifold fans, TM_MAXVAL) before anything changes */
int tm_mesh_set_topology(tm_mesh* m, const int32_t* to, const int32_t* next, const int32_t* face,
                         const int32_t* vout, const int32_t* fhe);
/* Device-side invariant check: closed 2-manifold fans, valence >= 3, no
 * double edges.  *status = 0 when valid, else a negative code. */
int tm_mesh_check(tm_mesh* m, int* status);

/* ---- geometry primitives (src/mesh_util.h:15-185, src/bindings.cpp:251-407)
 * value and gradient of one halfedge's quantity; grad (rows x 3, row-major)
 * may be NULL.  Rows: edge_length 2, face_area 3, face_volume 3,
 * dihedral_angle 4. */
int tm_edge_length(tm_mesh* m, int64_t he, double* value, double* grad);
int tm_face_area(tm_mesh* m, int64_t he, double* value, double* grad);
int tm_face_volume(tm_mesh* m, int64_t he, double* value, double* grad);
int tm_dihedral_angle(tm_mesh* m, int64_t he, double* value, double* grad);

/* ---- energy manager (src/energy.h:18-56, src/energy.cpp:13-151) --------
 * Properties are ordered (area, volume, curvature, bending, tethering,
 * repulsion) like VertexProperties (src/mesh_properties.h:14-48). */
int tm_energy_create(tm_mesh* m, const tm_params* p, tm_energy** out);
int tm_energy_destroy(tm_energy* e);
int tm_energy_get_params(tm_energy* e, tm_params* out);
int tm_energy_initial_props(tm_energy* e, double* out6);
/* restores the initial properties (the reference's EnergyManager computes
 * them once from the constructing mesh, src/energy.cpp:13-28): a resumed
 * run keeps the reference properties of the original one */
int tm_energy_set_initial_props(tm_energy* e, const double* in6);
int tm_energy_properties(tm_energy* e, tm_mesh* m, double* out6);
int tm_energy_vertex_properties(tm_energy* e, tm_mesh* m, double* out6v);
int tm_energy_energy(tm_energy* e, tm_mesh* m, double* energy);
int tm_energy_energy_props(tm_energy* e, const double* props6, double* energy);
/* area, volume, area-difference, bending, tether, repulsion, total energy
 * (the print_info breakdown, src/energy.cpp:126-151). */
int tm_energy_components(tm_energy* e, tm_mesh* m, double* out7);
/* Gradient of the energy wrt the positions, (n_vertices, 3); energy may be
 * NULL (src/energy.cpp:93-124). */
int tm_energy_gradient(tm_energy* e, tm_mesh* m, double* grad, double* energy);
int tm_energy_update_reference_properties(tm_energy* e);
int tm_energy_update_repulsion(tm_energy* e, tm_mesh* m);
/* Local stencil precision: 0 FP64, 1 FP32 (positions split into float
 * hi/lo parts, FP64 global sums), 2 double-word (the default: pairs of
 * floats on the FP32 pipe, ~48-bit significands, results within ~1e-13 of
 * FP64; FP64 global sums, penalty assembly and exact pair tests).
 * Per-vertex properties are always computed with the FP64 stencil. */
int tm_energy_set_stencil_precision(tm_energy* e, int mode);

/* Device-resident evaluation: positions, gradient and energy live in device
 * memory, nothing is copied to the host and the call does not synchronise.
 * Runs on `stream` (a cudaStream_t, NULL for the handle's own stream).
 * d_grad or d_energy may be NULL. */
int tm_energy_eval_device(tm_energy* e, tm_mesh* m, const double* d_points, double* d_grad,
                          double* d_energy, void* stream);
/* tm_energy_eval_device with CUDA events on the launching stream around each
 * kernel; ms5 = {face, edge, vertex (+reduction), gradient, total} in ms.
 * Synchronises.  A measurement aid, no counterpart in the reference. */
int tm_energy_eval_timed(tm_energy* e, tm_mesh* m, const double* d_points, double* d_grad, float* ms5,
                         void* stream);
/* Size of the device scratch array used by tm_energy_eval_device_noalloc. */
#define TM_NOALLOC_SCRATCH_BYTES (16 * 1024 * 1024)
/* tm_energy_eval_device (FP64 stencil) for callers that must not allocate
 * device memory during the evaluation: the scratch lives in one file-scope
 * device array of TM_NOALLOC_SCRATCH_BYTES (about 380 bytes per vertex, so
 * about 44,000 vertices; larger meshes are rejected with TM_ERR_ARG) instead
 * of the energy manager's buffers.  d_grad must not be NULL (TM_ERR_ARG), and
 * the stencil precision set by tm_energy_set_stencil_precision is ignored:
 * the stencil is always FP64.  The first call on a device looks up the
 * array's address and must precede any stream capture; the address is kept
 * for the life of the process and does not survive cudaDeviceReset.  Calls
 * that overlap on the GPU share the array and race.  No counterpart in the
 * reference. */
int tm_energy_eval_device_noalloc(tm_energy* e, tm_mesh* m, const double* d_points, double* d_grad,
                                  double* d_energy, void* stream);
/* Rebuilds the neighbour list from device-resident positions. */
int tm_energy_update_repulsion_device(tm_energy* e, tm_mesh* m, const double* d_points, void* stream);

/* ---- neighbour lists (src/nlists/nlist.h:15-40, nlist.cpp:10-53) --------
 * n_search, exclusion_level and rlist are read from p.  Unknown n_search or
 * exclusion level: TM_ERR_ARG (RuntimeError in the reference). */
int tm_nlist_create(tm_mesh* m, const tm_params* p, tm_nlist** out);
int tm_nlist_destroy(tm_nlist* nl);
/* distance_matrix(mesh, rdist): the cell list returns each pair once as
 * (i < j) with d <= rdist, the Verlet list both orders with d < rdist. */
int tm_nlist_distance_matrix(tm_nlist* nl, tm_mesh* m, double rdist, int64_t* count);
/* point_distances(mesh, pid, rdist): x_pid - x_j for the neighbours j with
 * |x_pid - x_j| < rdist. */
int tm_nlist_point_distances(tm_nlist* nl, tm_mesh* m, int64_t pid, double rdist, int64_t* count);
/* Copies the last result: distance_matrix -> (d, i, j); point_distances ->
 * (d as (count,3), j); i may be NULL for the latter. */
int tm_nlist_fetch(tm_nlist* nl, double* d, int32_t* i, int32_t* j);

/* ---- edge flips (src/flips.cpp:22-165, src/bindings.cpp:839-891) --------
 * Metropolis edge-flip sweep over floor(n_edges * ratio) proposals.
 * mode 0 (flip): proposals are evaluated in proposal order; mode 1 (pflip):
 * proposals are evaluated in conflict-free batches of `batch`, a proposal
 * whose quad lies within one edge of a lower proposal's quad waits for the
 * next batch (1 <= batch <= 4096; pflip's default is 4096).  ratio > 1 is
 * TM_ERR_RANGE in mode 1.  Deterministic for a given seed, and the same
 * flips as the CPU port of the sweep (om_flip_windowed of the oracle). */
int tm_flip(tm_mesh* m, tm_energy* e, double ratio, uint64_t seed, int mode, int batch, int32_t* accepted);
/* The same sweep on device-resident positions (n_vertices*3 doubles); the
 * topology of m is updated in place, *accepted is returned after the sweep. */
int tm_flip_device(tm_mesh* m, tm_energy* e, const double* d_points, double ratio, uint64_t seed, int mode,
                   int batch, int32_t* accepted, void* stream);

/* ---- utilities (src/util.cpp:9-41, src/bindings.cpp:25-50) -------------- */
int tm_area(tm_mesh* m, double* out);
int tm_edges_length(tm_mesh* m, double* out);
int tm_avg_tri_props(tm_mesh* m, double* mean_area, double* mean_length);
/* Forward-difference gradient with step eps (3 * n_vertices energies). */
int tm_fd_gradient(tm_mesh* m, tm_energy* e, double eps, double* grad);

/* ---- device-resident HMC (src/trimem/mc/hmc.py:14-26,133-158) -----------
 * One Metropolis step: momenta ~ N(0, m*T) drawn on the device from
 * (seed, step), n_steps velocity-Verlet steps of size dt with mass m, then
 * accept with probability min(1, exp(-dH/T)) using the uniform u.
 * d_x (n_vertices*3) is updated in place when accepted.  out[0] = accepted,
 * out[1] = H(start), out[2] = H(end), out[3] = energy of the returned state;
 * props6 (may be NULL) receives the six global properties of the returned
 * state (area, volume, curvature, bending, tethering, repulsion).
 * The neighbour list is the one of the energy manager (not rebuilt). */
int tm_hmc_step_device(tm_energy* e, tm_mesh* m, double* d_x, double mass, double dt, int n_steps,
                       double temperature, uint64_t seed, uint64_t step, double u, double* out4, double* props6,
                       void* stream);

/* ---- minimisation (src/trimem/mc/util.py:240-306) --------------------------
 * Energy minimisation of the device positions d_x (n_vertices*3, updated in
 * place) by L-BFGS with `history` correction pairs and an Armijo
 * backtracking line search; the cell list is rebuilt at every evaluation
 * like the reference's refresh = 1.  Stops when max |gradient| <= gtol, the
 * relative energy decrease of a step is <= ftol, no decrease is found, or
 * after maxiter iterations. */
int tm_minimize_device(tm_energy* e, tm_mesh* m, double* d_x, int maxiter, int history, double gtol, double ftol,
                       int32_t* iterations, double* energy, void* stream);

/* ---- learned surrogate force (no counterpart in the reference) ---------------
 * A message-passing network (3 rounds, width 64, bf16 dense layers on the
 * tensor cores) that stands in for the bending and repulsion forces; the
 * local penalty forces stay exact (FP32 stencils).  weights: the float32 blob
 * written by trimem_gb300.surrogate (26,442 values).  The surrogate drives
 * the leapfrog of tm_surrogate_hmc_step_device; acceptance uses the exact
 * FP64 Hamiltonian of the energy manager. */
typedef struct tm_surrogate tm_surrogate;
int tm_surrogate_create(tm_mesh* m, const float* weights, int64_t n_weights, tm_surrogate** out);
int tm_surrogate_destroy(tm_surrogate* s);
/* surrogate gradient (the force is its negative), device arrays n_vertices*3 */
int tm_surrogate_gradient_device(tm_surrogate* s, tm_energy* e, tm_mesh* m, const double* d_points, double* d_grad,
                                 void* stream);
/* network inputs for training, device arrays: d_u (nv x 8), d_normals (nv x 4),
 * slot-major [max_valence][nv] neighbours (-1 past the valence), edge
 * features (x 4) and unit edge directions (x 3), and the exact gradient of
 * the local terms (nv x 3 doubles) */
int tm_surrogate_inputs_device(tm_surrogate* s, tm_energy* e, tm_mesh* m, const double* d_points, int32_t max_valence,
                               float* d_u, float* d_normals, int32_t* d_nbr, float* d_edge_feat, float* d_dirs,
                               double* d_grad_local, void* stream);
/* HMC step of tm_hmc_step_device with surrogate forces in the leapfrog */
int tm_surrogate_hmc_step_device(tm_surrogate* s, tm_energy* e, tm_mesh* m, double* d_x, double mass, double dt,
                                 int n_steps, double temperature, uint64_t seed, uint64_t step, double u, double* out4,
                                 double* props6, void* stream);
/* One dense layer of the network on the tensor cores: out = h + SiLU([h | m] W^T + b)
 * with h, m, out bf16 (rows x 64, row-major, 16-byte aligned), W bf16 (64 x 128)
 * and b float (64). */
int tm_dense_silu_bf16(const void* d_h, const void* d_m, const void* d_w, const float* d_bias, void* d_out,
                       int64_t rows, void* stream);
/* tm_dense_silu_bf16 with the poll limit of its two device waits (tile loads,
 * MMA completion) given.  A wait that gives up makes the call return
 * TM_ERR_TIMEOUT with the context still usable: the kernel records it,
 * skips the dependent work, lets its own copies land and frees its tensor
 * memory.  wait_polls = 0 makes the first wait give up at once; a test aid
 * for the failure path, no counterpart in the reference. */
int tm_dense_silu_bf16_bounded(const void* d_h, const void* d_m, const void* d_w, const float* d_bias, void* d_out,
                               int64_t rows, int wait_polls, void* stream);

/* ---- training of the surrogate on the GPU (no counterpart in the
 * reference) ----------------------------------------------------------------
 * Hand-written forward and backward kernels of the network and Adam:
 * activations and dense weights bf16 (the dense layer on the tensor cores,
 * as in inference), FP32 accumulation and FP32 master parameters.  The
 * inputs are the device arrays tm_surrogate_inputs_device exports for one
 * state (u n x 8, normals n x 4, ring neighbours [D][n] int32 with -1
 * padding, edge features [D][n][4] 16-byte aligned, unit edge directions
 * [D][n][3]) and the target force n x 3 (float).  The loss is
 * mean((F - T)^2) / target_rms^2 over the 3 n force components.  Parameter
 * gradients are reduced in a fixed order: a step is bit-reproducible.
 * A training state serves meshes of n_vertices and up to max_valence ring
 * slots; weights use the blob layout of tm_surrogate_create. */
typedef struct tm_strain tm_strain;
int tm_surrogate_train_create(int64_t n_vertices, int32_t max_valence, const float* weights, int64_t n_weights,
                              tm_strain** out);
int tm_surrogate_train_destroy(tm_strain* t);
/* current weights (host blob of n_weights floats) */
int tm_surrogate_train_get_weights(tm_strain* t, float* weights, int64_t n_weights);
/* forward pass (force into d_force and loss into d_loss, each may be NULL)
 * and, when d_grad is not NULL, the loss gradient wrt the parameters in
 * blob order without the 8-float header; synchronises */
int tm_surrogate_train_grad(tm_strain* t, const float* d_u, const float* d_nrm, const int32_t* d_nbr,
                            const float* d_ef, const float* d_dirs, const float* d_target, int64_t n_vertices,
                            int32_t max_valence, float target_rms, float* d_force, float* d_loss, float* d_grad,
                            void* stream);
/* one Adam step (Kingma & Ba, with bias correction) on one state; the
 * loss before the step goes to d_loss (may be NULL); does not synchronise */
int tm_surrogate_train_step(tm_strain* t, const float* d_u, const float* d_nrm, const int32_t* d_nbr,
                            const float* d_ef, const float* d_dirs, const float* d_target, int64_t n_vertices,
                            int32_t max_valence, float target_rms, float lr, float beta1, float beta2, float eps,
                            float* d_loss, void* stream);
/* synchronises; TM_ERR_TIMEOUT if a tensor-core wait of a past step gave up */
int tm_surrogate_train_status(tm_strain* t);

/* ---- batches of replicas (no counterpart in the reference: the reference
 * runs one membrane per process) -------------------------------------------
 * n_rep independent meshes with their own parameters (exclusion levels
 * included) evaluated and sampled together: FP32 stencils, FP64 global
 * sums.  Replicas are grouped into size classes (runs of consecutive
 * replicas whose vertex counts share a power of two); the element kernels
 * run per class with block sizes the autotuner picks for that class at
 * creation, side by side on the classes' streams, and the vertex stage and
 * repulsion run once for all replicas.  The replicas share one kind of
 * neighbour list (params[r].n_search all 0, the cell list, or all 1, the
 * Verlet list; each at the replica's own cut-off), else TM_ERR_ARG.
 * Positions live on the device in a padded layout: replica r occupies
 * vertices [offsets[r], offsets[r] + n_points[r]) of [0, n_total) (see
 * tm_batch_layout); padding vertices are inert. */
typedef struct tm_batch tm_batch;
int tm_batch_create(int n_rep, const double* const* points, const int64_t* n_points, const int32_t* const* faces,
                    const int64_t* n_faces, const tm_params* params, tm_batch** out);
int tm_batch_destroy(tm_batch* b);
/* the size classes: their number, and per class (up to 8) six ints: first
 * and end vertex of its range, tuned block sizes of the split, face, edge
 * and gradient kernels */
int tm_batch_tuning(tm_batch* b, int32_t* n_classes, int32_t* info);
int tm_batch_layout(tm_batch* b, int64_t* n_total, int64_t* offsets);
/* direction 0: device -> host_x, 1: host_x -> device; host_x is n_total x 3 */
int tm_batch_positions(tm_batch* b, double* host_x, int direction);
/* energy of every replica (n_rep values) and optionally the gradient */
int tm_batch_energy(tm_batch* b, double* energies, double* grad);
int tm_batch_update_repulsion(tm_batch* b);
/* neighbour list rebuilt after every `every`-th HMC step of tm_batch_hmc
 * (0: never; default 1), like the evaluator callback of the reference's HMC
 * (src/trimem/mc/evaluators.py) */
int tm_batch_set_refresh(tm_batch* b, int every);
/* n_steps HMC steps of every replica (n_leapfrog velocity-Verlet steps of
 * size dt, mass, temperature; per-replica Metropolis); use_graph replays one
 * captured step as a CUDA graph.  accepted[r] = accepted steps. */
int tm_batch_hmc(tm_batch* b, int n_steps, int n_leapfrog, double dt, double mass, double temperature, uint64_t seed,
                 int use_graph, int32_t* accepted);

#ifdef __cplusplus
}
#endif
#endif
