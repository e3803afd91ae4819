/*
 * ipcg.h — C ABI of the GB300-native IPC contact hot path.
 *
 * Every entry point is extern "C", takes plain pointers and sizes, and
 * returns an int status (IPCG_OK = 0).  On failure ipcg_last_error() gives a
 * message for the calling thread.  Position arrays are row-major (n, 3)
 * float64, index arrays row-major int32, exactly as the reference's
 * Eigen::MatrixXd / Eigen::MatrixXi arguments are laid out.
 *
 * Pointer arguments may be host memory or device memory of the current CUDA
 * device (unified addressing decides which); host inputs are copied to the
 * device inside the call and host outputs are written before the call
 * returns.  Host buffers in page-locked memory (cudaHostAlloc, or
 * cudaHostRegister on an existing array) are copied at the link's rate;
 * pageable ones go through a staging copy.  Objects are not thread-safe: do not use one ipcg_mesh or
 * ipcg_collisions from two threads at once.
 */
#ifndef IPCG_H
#define IPCG_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define IPCG_OK 0
#define IPCG_ERR_INVALID 1      /* bad argument (maps to std::invalid_argument) */
#define IPCG_ERR_CUDA 2         /* CUDA runtime error (maps to std::runtime_error) */
#define IPCG_ERR_OOM 3          /* device allocation failed */
#define IPCG_ERR_TOPOLOGY 4     /* face edge missing from E ("Unable to find edge!") */
#define IPCG_ERR_NO_DEVICE 5    /* no CUDA device */

/* PSD projection methods (src/ipc/utils/eigen_ext.hpp:202-206) */
#define IPCG_PSD_NONE 0
#define IPCG_PSD_CLAMP 1
#define IPCG_PSD_ABS 2

/* Bits of the barrier calls' use_physical_barrier argument.  Bit 0 is the
 * reference's flag (BarrierPotential(dhat, stiffness, use_physical_barrier),
 * barrier_potential.hpp:24-27); 0 and 1 mean what they mean there.  Bit 1
 * (no counterpart in the reference) selects mixed precision: face-vertex
 * (point-triangle) contacts on non-degenerate triangles compute the
 * distance, its derivatives and the barrier derivatives in FP32 from FP64
 * relative vectors; every other contact type, the PSD projection and the
 * assembly stay FP64.  Energy, gradient and Hessian then agree with FP64 to
 * about 1e-6 relative. */
#define IPCG_BARRIER_PHYSICAL 1
#define IPCG_BARRIER_FP32_PT 2
/* Bit 2 (no counterpart in the reference) widens the mixed precision to
 * every contact but near-parallel (mollified) edge-edge ones and face-vertex
 * ones on degenerate triangles: the point-point, point-line, point-plane and
 * line-line distance gradients and Hessians and the barrier derivatives of
 * the energy + gradient + Hessian pass run in FP32, with the squared distance
 * and the cancellation-prone scalars (the point-plane / line-line numerator
 * a.(u x v), the point-line cross product) from FP64.  The PSD
 * eigen-projection, the mollifier, assembly and CCD stay FP64.  Results agree
 * with FP64 to about 1e-6 relative. */
#define IPCG_BARRIER_FP32_LOCAL 4
/* Bit 3 (no counterpart in the reference) computes the negative eigenpairs
 * of the PSD projection in df64 (pairs of FP32 values, about 48 significant
 * bits, with exact power-of-two rescaling) instead of FP64, on the FP32
 * pipes, which GB300 runs at 64 times its FP64 rate.  The correction
 * sum lam w w^T is subtracted from the FP64 local Hessian in FP64.  The
 * projected Hessians agree with the FP64 projection to about 1e-13 relative.
 * It applies to the calls that return a Hessian (the cached-pattern pass);
 * other calls ignore it. */
#define IPCG_BARRIER_DF64_PSD 8

/* Bits 4-7 of the same argument select the barrier function
 * (src/ipc/barrier/barrier.hpp; BarrierPotential(barrier, dhat, stiffness,
 * use_physical_barrier), barrier_potential.hpp:29-37): 0 (the default)
 * ClampedLogBarrier, then NormalizedBarrier<ClampedLogBarrier>,
 * ClampedLogSqBarrier, CubicBarrier and TwoStageBarrier.  The physical
 * scaling divides by the chosen barrier's units(). */
#define IPCG_BARRIER_CLAMPED_LOG 0
#define IPCG_BARRIER_NORMALIZED_CLAMPED_LOG 1
#define IPCG_BARRIER_CLAMPED_LOG_SQ 2
#define IPCG_BARRIER_CUBIC 3
#define IPCG_BARRIER_TWO_STAGE 4
#define IPCG_BARRIER_FUNCTION(kind) ((kind) << 4)

typedef struct ipcg_mesh ipcg_mesh;
typedef struct ipcg_collisions ipcg_collisions;
typedef struct ipcg_csr ipcg_csr;

/* Message of the last failed call on this thread ("" if none). */
const char* ipcg_last_error(void);

/* Library version string. */
const char* ipcg_version(void);

/* Per-kernel timing: with profiling on, every kernel launch (and every CUB
 * device call) is bracketed by CUDA events on its stream.  Enabling or
 * disabling clears the accumulated statistics. */
int ipcg_profile_enable(int on);
/* JSON {"kernel": {"launches": n, "ms": total}, ...} into buf (truncated to
 * buflen); *needed receives the full length including the terminator. */
int ipcg_profile_report(char* buf, int64_t buflen, int64_t* needed);
/* Number of kernel launches issued by the library since it was loaded. */
int ipcg_launch_count(int64_t* count);

/* ---------------------------------------------------------------------- */
/* CollisionMesh                                                           */
/* ---------------------------------------------------------------------- */

/* Replaces CollisionMesh::CollisionMesh(V, E, F)
 * (src/ipc/collision_mesh.hpp:21-26, src/ipc/collision_mesh.cpp:15-125):
 * uploads rest positions, edges and faces, builds faces_to_edges
 * (collision_mesh.cpp:510-543) and keeps them resident on the device. */
int ipcg_mesh_create(const double* rest_positions, int64_t num_vertices,
                     const int32_t* edges, int64_t num_edges,
                     const int32_t* faces, int64_t num_faces,
                     ipcg_mesh** out);
int ipcg_mesh_destroy(ipcg_mesh* mesh);

/* CollisionMesh::num_vertices/num_edges/num_faces (collision_mesh.hpp) */
int ipcg_mesh_sizes(const ipcg_mesh* mesh, int64_t sizes[3]);

/* CollisionMesh::num_codim_vertices() / num_codim_edges() (collision_mesh.cpp:
 * 145-183): counts[0] vertices that belong to no edge, counts[1] edges that
 * belong to no face.  The reference finds extra vertex-vertex candidates among
 * codimensional vertices and edge-vertex candidates between codimensional
 * edges and codimensional vertices (candidates.cpp:66-116, 152-210).  Those
 * passes are not provided: collision-set builds, candidate builds and step-size
 * calls on a mesh where they would find pairs -- two or more codimensional
 * vertices, or one together with a codimensional edge -- fail with
 * IPCG_ERR_INVALID instead of returning an incomplete result.  Codimensional
 * edges alone, or a single codimensional vertex without them, need no extra
 * pass (their contacts are edge-edge or face-vertex candidates) and are
 * supported. */
int ipcg_mesh_codim_counts(const ipcg_mesh* mesh, int64_t counts[2]);

/* CollisionMesh::faces_to_edges() (collision_mesh.hpp:327-329): num_faces*3 */
int ipcg_mesh_faces_to_edges(const ipcg_mesh* mesh, int32_t* out);

/* CollisionMesh::vertex_areas() / edge_areas() (collision_mesh.cpp:309-374):
 * per-vertex and per-edge areas of the rest mesh (a vertex or edge takes a
 * third of each incident face's area; without faces, half the incident edge
 * lengths or the edge's length; an isolated vertex 1).  Either output may be
 * NULL; sizes num_vertices and num_edges. */
int ipcg_mesh_areas(const ipcg_mesh* mesh, double* vertex_areas, double* edge_areas);

/* The cudaStream_t (as void*) on which all work for this mesh runs. */
int ipcg_mesh_stream(const ipcg_mesh* mesh, void** stream);

/* Batched scenes: n_scenes independent CollisionMesh objects packed into
 * one mesh (the reference runs one CollisionMesh per simulation; a batch
 * evaluates many simulations in one set of launches).  Scene k owns the
 * vertex range [vertex_offsets[k], vertex_offsets[k+1]); edges and faces use
 * packed (global) vertex indices and may not join two scenes.  Contacts are
 * only found within a scene.  Every per-scene result equals that of the
 * scene's own ipcg_mesh_create mesh.  ipcg_mesh_create is the n_scenes = 1
 * case.  The *_batch calls below take one dhat / dmin / stiffness /
 * min_distance per scene (host arrays of n_scenes) and return per-scene
 * energies and step sizes; the gradient and the Hessian are the packed
 * (block-diagonal) ones. */
int ipcg_mesh_create_batch(const double* rest_positions, int64_t num_vertices,
                           const int32_t* edges, int64_t num_edges,
                           const int32_t* faces, int64_t num_faces,
                           int64_t n_scenes, const int64_t* vertex_offsets,
                           ipcg_mesh** out);
int ipcg_mesh_scenes(const ipcg_mesh* mesh, int64_t* n_scenes);

/* Memory bound of the batched Hessian: the local 12x12 blocks of at most
 * `contacts` contacts (1152 bytes each) are held at once; a batch with more
 * contacts is assembled a run of whole scenes at a time.  0 restores the
 * default 4,194,304 (4.8 GB).  Process-wide; results do not depend on it. */
int ipcg_set_hessian_chunk_contacts(int64_t contacts);

/* ---------------------------------------------------------------------- */
/* NormalCollisions                                                        */
/* ---------------------------------------------------------------------- */

int ipcg_collisions_create(ipcg_collisions** out);
int ipcg_collisions_destroy(ipcg_collisions* collisions);

/* NormalCollisions::set_use_area_weighting / use_area_weighting
 * (normal_collisions.cpp:160-175); applies to the next build.  Weights
 * become FV vertex_area(v)/4 and EE (edge_area(ea) + edge_area(eb))/4
 * (normal_collisions_builder.cpp:146,181-183), carried by their VV / EV
 * reductions; duplicate VV / EV keys sum their weights in ascending order
 * (the reference's order is thread-dependent). */
int ipcg_collisions_set_use_area_weighting(ipcg_collisions* collisions, int use_area_weighting);
int ipcg_collisions_use_area_weighting(const ipcg_collisions* collisions, int* use_area_weighting);

/* NormalCollisions::set_collision_set_type / collision_set_type
 * (normal_collisions.cpp:177-192); applies to the next build.
 * IMPROVED_MAX_APPROX (normal_collisions.cpp:84-128,
 * normal_collisions_builder.cpp:340-543) adds negative edge-vertex and
 * edge-edge terms and positive vertex-vertex terms so that a contact near a
 * shared edge or vertex is counted once; merged weights that cancel to zero
 * are dropped.  Equal edge-edge records (unordered pair and type) merge into
 * the orientation with ea < eb when one exists.  OGC is not provided. */
/* NormalCollisions::set_enable_shape_derivatives / enable_shape_derivatives
 * (normal_collisions.hpp); must be on at build time for
 * ipcg_barrier_shape_derivative. */
int ipcg_collisions_set_enable_shape_derivatives(ipcg_collisions* collisions, int enable);
int ipcg_collisions_enable_shape_derivatives(const ipcg_collisions* collisions, int* enable);

#define IPCG_COLLISION_SET_IPC 0
#define IPCG_COLLISION_SET_IMPROVED_MAX_APPROX 1
int ipcg_collisions_set_collision_set_type(ipcg_collisions* collisions, int type);
int ipcg_collisions_collision_set_type(const ipcg_collisions* collisions, int* type);

/* Replaces NormalCollisions::build(mesh, V, dhat, dmin, broad_phase=nullptr)
 * (src/ipc/collisions/normal/normal_collisions.hpp:45-50,
 *  normal_collisions.cpp:20-158): device LBVH broad phase, FP64 distance
 * filter d^2 < (dhat+dmin)^2, reduction to VV/EV/EE/FV with summed weights.
 * The result stays on the device; entries are sorted by index key. */
int ipcg_collisions_build(ipcg_collisions* collisions, const ipcg_mesh* mesh,
                          const double* vertices, double dhat, double dmin);

/* NormalCollisions::build on every scene of a batch: dhat[n_scenes],
 * dmin[n_scenes].  The result is the concatenation of the scenes' sets
 * (each list stays sorted by packed index key). */
int ipcg_collisions_build_batch(ipcg_collisions* collisions, const ipcg_mesh* mesh,
                                const double* vertices, const double* dhat, const double* dmin);

/* Number of vv, ev, ee, fv collisions (NormalCollisions::{vv,ev,ee,fv}_collisions.size())
 * and of broad-phase candidates of the last build (ee, fv): counts[6]. */
int ipcg_collisions_counts(const ipcg_collisions* collisions, int64_t counts[6]);

/* Copy the collision set out (any pointer may be NULL to skip it).
 * vv: (nvv,2) sorted vertex pairs (min,max); ev: (nev,2) (edge, vertex);
 * ee: (nee,2) edge pairs (ea<eb) with mollifier threshold eps_x and the
 * stored distance type (EdgeEdgeDistanceType, distance_type.hpp);
 * fv: (nfv,2) (face, vertex). *_w are the merged weights. */
int ipcg_collisions_get(const ipcg_collisions* collisions,
                        int32_t* vv, double* vv_w,
                        int32_t* ev, double* ev_w,
                        int32_t* ee, double* ee_eps_x, int8_t* ee_dtype, double* ee_w,
                        int32_t* fv, double* fv_w);

/* Load an explicit collision set (same layout as ipcg_collisions_get),
 * e.g. one built elsewhere, for evaluating the potential on it. */
int ipcg_collisions_set(ipcg_collisions* collisions, double dmin,
                        int64_t nvv, const int32_t* vv, const double* vv_w,
                        int64_t nev, const int32_t* ev, const double* ev_w,
                        int64_t nee, const int32_t* ee, const double* ee_eps_x,
                        const int8_t* ee_dtype, const double* ee_w,
                        int64_t nfv, const int32_t* fv, const double* fv_w);

/* ---------------------------------------------------------------------- */
/* BarrierPotential (ClampedLogBarrier)                                    */
/* ---------------------------------------------------------------------- */

/* Replaces BarrierPotential::operator()(collisions, mesh, V)
 * (src/ipc/potentials/potential.hpp:34-40, potential.cpp:36-56,
 *  normal_potential.cpp:127-136, barrier_potential.cpp:62-73). */
int ipcg_barrier_energy(const ipcg_collisions* collisions, const ipcg_mesh* mesh,
                        const double* vertices, double dhat, double stiffness,
                        int use_physical_barrier, double* energy);

/* Replaces BarrierPotential::gradient(collisions, mesh, V)
 * (potential.hpp:42-48, potential.cpp:59-95, normal_potential.cpp:138-172):
 * gradient is a dense 3*num_vertices vector, vertex-major (3v+d). */
int ipcg_barrier_gradient(const ipcg_collisions* collisions, const ipcg_mesh* mesh,
                          const double* vertices, double dhat, double stiffness,
                          int use_physical_barrier, double* gradient);

/* Replaces BarrierPotential::hessian(collisions, mesh, V, project_hessian_to_psd)
 * (potential.hpp:50-60, potential.cpp:97-222, normal_potential.cpp:174-232,
 *  eigen_ext.tpp:64-108).  Produces a (3nV x 3nV) CSR matrix held by *out;
 * read it with ipcg_csr_* and release it with ipcg_csr_destroy.  The
 * matrix is symmetric, so these arrays are also its CSC (Eigen ColMajor)
 * form.  Every 3x3 vertex block touched by a contact is stored, so entries
 * the reference skips as exact zeros may appear as explicit zeros. */
int ipcg_barrier_hessian(const ipcg_collisions* collisions, const ipcg_mesh* mesh,
                         const double* vertices, double dhat, double stiffness,
                         int use_physical_barrier, int psd_method, ipcg_csr** out);

/* Energy, gradient and Hessian in one pass over the contacts (any output
 * may be NULL).  Same values as the three calls above. */
int ipcg_barrier_energy_gradient_hessian(const ipcg_collisions* collisions, const ipcg_mesh* mesh,
                                         const double* vertices, double dhat, double stiffness,
                                         int use_physical_barrier, int psd_method,
                                         double* energy, double* gradient, ipcg_csr** hessian);

/* Energy, gradient and Hessian on a batch (any output may be NULL):
 * dhat[n_scenes], stiffness[n_scenes], energies[n_scenes] (host). */
int ipcg_barrier_batch(const ipcg_collisions* collisions, const ipcg_mesh* mesh,
                       const double* vertices, const double* dhat, const double* stiffness,
                       int use_physical_barrier, int psd_method,
                       double* energies, double* gradient, ipcg_csr** hessian);

/* Every call above that asks for a Hessian evaluates energy, gradient and
 * Hessian in one pass over a sparsity pattern cached with the collision set
 * (the reference's SparseMatrixCache, matrix_cache.cpp:80-214, does the same
 * between Newton iterations): the pattern is built at the first such call
 * after each build or load of the set, and each later call replays one
 * captured CUDA graph (no host synchronisation inside it).  Each chunk of
 * contacts runs two persistent work-queue kernels: stage 0 computes every
 * contact's energy, gradient and local Hessian, stage 1 projects the local
 * Hessians to PSD and writes their blocks to block-sorted slots, which
 * streaming reductions sum into the CSR values.  Each stage's launch shape is
 * per device: ipcg_barrier_autotune times candidate shapes (threads per block
 * 32/64/128, resident blocks per SM, 32-contact tiles taken per work-queue
 * grab) on this set's largest chunk and keeps the fastest for each stage;
 * the report is JSON ({"local": {"candidates": [...], "chosen": {...}},
 * "psd": {...}}) in report (truncated to report_len; *needed gets the full
 * length with the terminator; both may be NULL).  No counterpart in the
 * reference. */
int ipcg_barrier_autotune(const ipcg_collisions* collisions, const ipcg_mesh* mesh, const double* vertices,
                          const double* dhat, const double* stiffness, int use_physical_barrier, int psd_method,
                          char* report, int64_t report_len, int64_t* needed);
/* A stage's launch shape on the current device (get / set): the local
 * Hessians, the FP64 projection, the df64 projection (IPCG_BARRIER_DF64_PSD).
 * ipcg_barrier_autotune sets the local stage and the projection stage its
 * options select. */
#define IPCG_STAGE_LOCAL 0
#define IPCG_STAGE_PSD 1
#define IPCG_STAGE_PSD_DF64 2
int ipcg_barrier_tuning(int stage, int* threads, int* blocks_per_sm, int* tiles_per_grab);
int ipcg_barrier_set_tuning(int stage, int threads, int blocks_per_sm, int tiles_per_grab);
/* The current device's FP64 fused multiply-add rate in TFLOP/s, measured by
 * a kernel of independent DFMA chains (the pipe's peak for non-tensor FP64
 * code such as this path's per-contact work).  No counterpart in the
 * reference. */
int ipcg_fp64_fma_rate(double* tflops);
/* Testing switch: with on != 0, the df64 projection (IPCG_BARRIER_DF64_PSD)
 * hands every local Hessian to its FP64 fix-up pass, the path taken by the
 * rare matrix on which the df64 eigensolver does not converge.  No
 * counterpart in the reference. */
int ipcg_testing_defer_df64_psd(int on);
/* Testing: statistics of the step-size passes (compute_collision_free_stepsize
 * and the other CCD calls on this mesh).  out (12 values, may be NULL) gets,
 * for the seed, budgeted and hard passes in turn, the queries run, the boxes
 * they examined, the most boxes of one query and the hits, accumulated since
 * the previous call; enable != 0 keeps collecting (for every mesh).  No
 * counterpart in the reference. */
int ipcg_testing_ccd_stats(const ipcg_mesh* mesh, int enable, int64_t* out);
/* Testing: the box budget of the step-size passes' one-thread pass, after
 * which a query moves to the warp-per-query pass (0 restores the default). */
int ipcg_testing_ccd_budget(int64_t boxes);

/* NormalPotential::shape_derivative(collisions, mesh, V)
 * (normal_potential.cpp:85-123, 310-416): the derivative of the gradient with
 * respect to the rest positions, ndof x ndof (rows: displacement dofs,
 * columns: rest dofs; not symmetric).  Per collision w times the unprojected
 * local Hessian, edge-edge collisions in the reference's mollified form with
 * eps_x from the rest positions; with area weighting also
 * (grad_u f / w)(grad_x w)^T, grad_x w from the rest mesh's area Jacobians
 * (collision_mesh.cpp:376-432) summed over each record's merged candidates.
 * Area-weighted IMPROVED_MAX_APPROX sets are not provided. */
int ipcg_barrier_shape_derivative(const ipcg_collisions* collisions, const ipcg_mesh* mesh,
                                  const double* vertices, double dhat, double stiffness,
                                  int use_physical_barrier, ipcg_csr** out);

/* Gauss-Newton forms of the barrier Hessian
 * (NormalPotential::gauss_newton_hessian_diagonal / _quadratic_form,
 * normal_potential.cpp:15-83 and 236-308): with t = sum_i c_i x_i the
 * collision's distance vector, the Hessian is approximated by
 * w (4 f''(|t|^2) (J t)(J t)^T + 2 f'(|t|^2) J J^T), mollifier ignored.
 * diagonal: 3 nV doubles (host or device); p: 3 nV doubles (host or device),
 * out: the scalar p^T H p. */
int ipcg_barrier_gauss_newton_hessian_diagonal(const ipcg_collisions* collisions, const ipcg_mesh* mesh,
                                               const double* vertices, double dhat, double stiffness,
                                               int use_physical_barrier, double* diagonal);
int ipcg_barrier_gauss_newton_hessian_quadratic_form(const ipcg_collisions* collisions, const ipcg_mesh* mesh,
                                                     const double* vertices, double dhat, double stiffness,
                                                     int use_physical_barrier, const double* p, double* out);

/* Allocation-free barrier energy.  No counterpart in the reference: it exists
 * for callers that cannot let the library allocate device memory during a
 * call, such as codes that give all device memory to their own pool under a
 * hard budget, or that cannot afford cudaMalloc/cudaFree synchronising the
 * device under their other streams.  It computes the same value as
 * ipcg_barrier_energy from a collision set held entirely in caller-owned
 * DEVICE arrays of the current device (layout of ipcg_collisions_get,
 * topology as for ipcg_mesh_create) and writes it to the device double
 * *energy.  It allocates nothing: the reduction's partial sums live in a
 * static device array of 16385 doubles (128 KiB) that every GPU loading this
 * library keeps until exit.  At most 2,097,152 contacts per call (larger sets
 * are rejected with IPCG_ERR_INVALID before anything is launched).  The
 * indices are checked on the device against num_vertices / num_edges /
 * num_faces (and edge-edge distance types against 0..8): a contact with an
 * index out of range is not evaluated and the energy comes back NaN.  The
 * work is enqueued on `stream` (a cudaStream_t, NULL for the default stream)
 * and the call returns without waiting; *energy is valid once the stream
 * reaches it.  The first call on a device (and the first after its context
 * is replaced, e.g. by cudaDeviceReset) looks up the array's device address
 * (cudaGetSymbolAddress), so make that first call before any stream capture.
 * All calls share the array: calls that overlap on the GPU (on different
 * streams or host threads) race and must be serialised by the caller. */
int ipcg_barrier_energy_noalloc(const double* vertices, int64_t num_vertices,
                                const int32_t* edges, int64_t num_edges,
                                const int32_t* faces, int64_t num_faces,
                                int64_t nvv, const int32_t* vv, const double* vv_w,
                                int64_t nev, const int32_t* ev, const double* ev_w,
                                int64_t nee, const int32_t* ee, const double* ee_eps_x,
                                const int8_t* ee_dtype, const double* ee_w,
                                int64_t nfv, const int32_t* fv, const double* fv_w,
                                double dhat, double stiffness, double dmin,
                                int use_physical_barrier, double* energy, void* stream);

int ipcg_csr_shape(const ipcg_csr* csr, int64_t* rows, int64_t* nnz);
/* row_ptr: rows+1 int64, col: nnz int32, val: nnz float64 (host or device) */
int ipcg_csr_get(const ipcg_csr* csr, int64_t* row_ptr, int32_t* col, double* val);
/* Same with 32-bit row pointers (converted on the device), for callers whose
 * sparse format keeps both index arrays 32-bit (scipy, Eigen with int
 * StorageIndex); fails when nnz >= 2^31. */
int ipcg_csr_get_int32(const ipcg_csr* hessian, int32_t* row_ptr, int32_t* col, double* val);
int ipcg_csr_destroy(ipcg_csr* csr);

/* ---------------------------------------------------------------------- */
/* compute_collision_free_stepsize                                         */
/* ---------------------------------------------------------------------- */

/* Replaces compute_collision_free_stepsize(mesh, V0, V1, min_distance,
 * broad_phase=nullptr, TightInclusionCCD(tolerance, max_iterations,
 * conservative_rescaling)) (src/ipc/ipc.hpp:41-47, ipc.cpp:42-106,
 * candidates.cpp:252-292, tight_inclusion_ccd.cpp:33-336).
 * Defaults of the reference: tolerance 1e-6, max_iterations 1e7,
 * conservative_rescaling 0.8.  n_candidates (may be NULL) receives the
 * broad-phase candidate count. */
int ipcg_collision_free_stepsize(const ipcg_mesh* mesh,
                                 const double* vertices_t0, const double* vertices_t1,
                                 double min_distance, double tolerance,
                                 int64_t max_iterations, double conservative_rescaling,
                                 double* step, int64_t* n_candidates);

/* compute_collision_free_stepsize on every scene of a batch:
 * min_distance[n_scenes] in, steps[n_scenes] out (host arrays). */
int ipcg_collision_free_stepsize_batch(const ipcg_mesh* mesh,
                                       const double* vertices_t0, const double* vertices_t1,
                                       const double* min_distance, double tolerance,
                                       int64_t max_iterations, double conservative_rescaling,
                                       double* steps, int64_t* n_candidates);

/* ---------------------------------------------------------------------- */
/* Newton-loop neighbours of the path                                      */
/* ---------------------------------------------------------------------- */

/* Replaces NormalCollisions::compute_minimum_distance(mesh, V)
 * (normal_collisions.cpp:209-233): the smallest SQUARED distance over the
 * collision set, each contact measured with its own distance; +inf when the
 * set is empty. */
int ipcg_collisions_minimum_distance(const ipcg_collisions* collisions, const ipcg_mesh* mesh,
                                     const double* vertices, double* out);

/* Replaces initial_barrier_stiffness(bbox_diagonal, barrier, dhat,
 * average_mass, grad_energy, grad_barrier, max_barrier_stiffness,
 * min_barrier_stiffness_scale, dmin) (barrier/adaptive_stiffness.cpp:12-48):
 * barrier_kind is an IPCG_BARRIER_* kind (0 ClampedLogBarrier); grad_energy
 * and grad_barrier are n doubles (host or device; both in the same memory).
 * *kappa receives the clamped stiffness, *max_barrier_stiffness 100 times the
 * minimum. */
int ipcg_initial_barrier_stiffness(double bbox_diagonal, int barrier_kind, double dhat, double average_mass,
                                   const double* grad_energy, const double* grad_barrier, int64_t n,
                                   double min_barrier_stiffness_scale, double dmin, double* kappa,
                                   double* max_barrier_stiffness);
/* Replaces update_barrier_stiffness(prev_min_distance, min_distance,
 * max_barrier_stiffness, barrier_stiffness, bbox_diagonal,
 * dhat_epsilon_scale, dmin) (barrier/adaptive_stiffness.cpp:51-68): the
 * stiffness doubles (up to the maximum) while the minimum (squared) distance
 * keeps shrinking below (dhat_epsilon_scale (bbox_diagonal + dmin))^2. */
int ipcg_update_barrier_stiffness(double prev_min_distance, double min_distance, double max_barrier_stiffness,
                                  double barrier_stiffness, double bbox_diagonal, double dhat_epsilon_scale,
                                  double dmin, double* out);

/* Replaces is_step_collision_free(mesh, V0, V1, min_distance, nullptr,
 * TightInclusionCCD(tolerance, max_iterations, conservative_rescaling))
 * (ipc.hpp, ipc.cpp:20-40, candidates.cpp:224-250): *out = 1 when no
 * swept-box candidate's CCD reports a hit over the step. */
int ipcg_is_step_collision_free(const ipcg_mesh* mesh,
                                const double* vertices_t0, const double* vertices_t1,
                                double min_distance, double tolerance,
                                int64_t max_iterations, double conservative_rescaling, int* out);

/* Replaces has_intersections(mesh, V) (ipc.cpp:110-167) for 3D meshes: *out
 * = 1 when some edge crosses a triangle it does not share a vertex with
 * (exact orientation predicates, then the crossing point's coordinates as
 * in geometry/intersection.cpp:120-147). */
int ipcg_has_intersections(const ipcg_mesh* mesh, const double* vertices, int* out);

/* Candidates (src/ipc/candidates/candidates.hpp): a kept broad-phase
 * candidate set on the device (EE pairs, then FV (face, vertex) pairs) and
 * the step-size rules that read it.  Single-scene 3D meshes. */
/* ---------------------------------------------------------------------- */
/* Friction: TangentialCollisions and FrictionPotential (isotropic)        */
/* ---------------------------------------------------------------------- */

typedef struct ipcg_tangential ipcg_tangential;
int ipcg_tangential_create(ipcg_tangential** out);
int ipcg_tangential_destroy(ipcg_tangential* tangential);

/* TangentialCollisions::build(mesh, V, collisions, BarrierPotential(dhat,
 * stiffness, use_physical_barrier), mu_s, mu_k) (tangential_collisions.cpp:
 * 60-170) with the default blend (mu0 + mu1) / 2: for each normal collision
 * but the near-parallel edge-edge ones (cross^2 < eps_x), the normal force
 * magnitude -kappa b'(d^2 - dmin^2) 2 d (times the physical scaling), the
 * closest point, the tangent basis and the blended coefficients.  mu_s,
 * mu_k: num_vertices doubles (host or device).  Single-scene meshes. */
int ipcg_tangential_build(ipcg_tangential* tangential, const ipcg_mesh* mesh, const double* vertices,
                          const ipcg_collisions* collisions, double dhat, double stiffness,
                          int use_physical_barrier, const double* mu_s, const double* mu_k);
/* The same on a batch mesh (ipcg_mesh_create_batch): dhat[n_scenes],
 * stiffness[n_scenes] (host); the normal set must come from
 * ipcg_collisions_build_batch on the same mesh. */
int ipcg_tangential_build_batch(ipcg_tangential* tangential, const ipcg_mesh* mesh, const double* vertices,
                                const ipcg_collisions* collisions, const double* dhat, const double* stiffness,
                                int use_physical_barrier, const double* mu_s, const double* mu_k);
/* counts[4]: VV, EV, EE, FV tangential collisions */
int ipcg_tangential_counts(const ipcg_tangential* tangential, int64_t counts[4]);
/* Any output may be NULL.  Stencils as in ipcg_collisions_get; per collision
 * (VV | EV | EE | FV order): weight, normal_force, closest_point (2),
 * tangent_basis (6: the two 3-vector columns), mu_s, mu_k. */
int ipcg_tangential_get(const ipcg_tangential* tangential, int32_t* vv, int32_t* ev, int32_t* ee, int32_t* fv,
                        double* weight, double* normal_force, double* closest_point, double* tangent_basis,
                        double* mu_s, double* mu_k);

/* Anisotropic friction (tangential_collision.hpp:104-139): per collision
 * (VV | EV | EE | FV order) the slip scaling mu_aniso, the directional static
 * and kinetic coefficients mu_s_aniso, mu_k_aniso (2 doubles each, along the
 * collision's tangent basis; host or device; NULL restores the defaults
 * (1, 1), (0, 0), (0, 0)).  A build restores every default and sets the
 * lagged effective coefficients to the scalar ones. */
int ipcg_tangential_set_anisotropy(ipcg_tangential* tangential, const double* mu_aniso, const double* mu_s_aniso,
                                   const double* mu_k_aniso);
/* TangentialCollisions::update_lagged_anisotropic_friction_coefficients
 * (tangential_collisions.cpp:387-420): the elliptical effective
 * coefficients along the scaled slip at rest + lagged displacements. */
int ipcg_tangential_update_lagged_mu(ipcg_tangential* tangential, const ipcg_mesh* mesh, const double* rest_positions,
                                     const double* lagged_displacements, const double* velocities);
/* TangentialCollisions::reset_lagged_anisotropic_friction_coefficients */
int ipcg_tangential_reset_lagged_mu(ipcg_tangential* tangential);
/* The lagged effective coefficients (n doubles each; either may be NULL). */
int ipcg_tangential_lagged_mu(const ipcg_tangential* tangential, double* mu_s_effective, double* mu_k_effective);

/* TangentialPotential::force(collisions, mesh, rest, lagged_displacements,
 * velocities, BarrierPotential(dhat, stiffness, physical), dmin, no_mu)
 * (tangential_potential.cpp:40-77, 333-410) with FrictionPotential(eps_v):
 * 3 nV doubles (host or device). */
int ipcg_friction_force(const ipcg_tangential* tangential, const ipcg_mesh* mesh, const double* rest_positions,
                        const double* lagged_displacements, const double* velocities, double dhat, double stiffness,
                        int use_physical_barrier, double dmin, double eps_v, int no_mu, double* force);

/* FrictionPotential(eps_v) energy, gradient and Hessian at velocities
 * (tangential_potential.cpp:156-331; potential.cpp:36-222): any output may
 * be NULL; the Hessian's inner 2x2 blocks are projected with psd_method. */
int ipcg_friction_potential(const ipcg_tangential* tangential, const ipcg_mesh* mesh, const double* velocities,
                            double eps_v, int psd_method, double* energy, double* gradient, ipcg_csr** hessian);
/* The same on a batch mesh: energies[n_scenes] (one eps_v for every scene);
 * the gradient and the Hessian are the packed (block-diagonal) ones. */
int ipcg_friction_potential_batch(const ipcg_tangential* tangential, const ipcg_mesh* mesh,
                                  const double* velocities, double eps_v, int psd_method, double* energies,
                                  double* gradient, ipcg_csr** hessian);

typedef struct ipcg_candidates ipcg_candidates;
int ipcg_candidates_create(ipcg_candidates** out);
int ipcg_candidates_destroy(ipcg_candidates* candidates);
/* Candidates::build(mesh, V, inflation_radius) (candidates.cpp:43-125) */
int ipcg_candidates_build(ipcg_candidates* candidates, const ipcg_mesh* mesh,
                          const double* vertices, double inflation_radius);
/* Candidates::build(mesh, V0, V1, inflation_radius) (candidates.cpp:128-222) */
int ipcg_candidates_build_swept(ipcg_candidates* candidates, const ipcg_mesh* mesh,
                                const double* vertices_t0, const double* vertices_t1,
                                double inflation_radius);
/* number of EE and FV pairs: counts[2]; the pairs (any order) as (n, 2) int32 */
int ipcg_candidates_counts(const ipcg_candidates* candidates, int64_t counts[2]);
int ipcg_candidates_get(const ipcg_candidates* candidates, int32_t* ee, int32_t* fv);
/* Candidates::compute_per_vertex_safe_distances (candidates.cpp:362-404): out[nV] */
int ipcg_candidates_per_vertex_safe_distances(const ipcg_candidates* candidates, const ipcg_mesh* mesh,
                                              const double* vertices, double inflation_radius,
                                              double min_distance, double* out);
/* Candidates::compute_collision_free_stepsize over the kept pairs (candidates.cpp:252-292) */
int ipcg_candidates_collision_free_stepsize(const ipcg_candidates* candidates, const ipcg_mesh* mesh,
                                            const double* vertices_t0, const double* vertices_t1,
                                            double min_distance, double tolerance,
                                            int64_t max_iterations, double conservative_rescaling,
                                            double* step);
/* Candidates::compute_noncandidate_conservative_stepsize (candidates.cpp:294-329) */
int ipcg_candidates_noncandidate_conservative_stepsize(const ipcg_candidates* candidates,
                                                       const ipcg_mesh* mesh,
                                                       const double* displacements, double dhat,
                                                       double* step);
/* Candidates::compute_cfl_stepsize (candidates.cpp:331-360) */
int ipcg_candidates_cfl_stepsize(const ipcg_candidates* candidates, const ipcg_mesh* mesh,
                                 const double* vertices_t0, const double* vertices_t1, double dhat,
                                 double min_distance, double tolerance, int64_t max_iterations,
                                 double conservative_rescaling, double* step);

/* ---------------------------------------------------------------------- */
/* Serving: requests from many simulations over resident scenes            */
/* ---------------------------------------------------------------------- */

/* No counterpart in the reference, which serves one simulation per call.
 * A server takes the two per-iteration requests of a Newton loop -- a barrier
 * request (NormalCollisions::build at the given positions, then the energy,
 * gradient and PSD-projected Hessian: normal_collisions.hpp:45-50,
 * potential.hpp:34-60) and a step-size request (compute_collision_free_stepsize,
 * ipc.hpp:41-47, with the reference's default TightInclusionCCD) -- from many
 * scenes at once.  Each scene's mesh, broad-phase work space and collision
 * set stay on the device.  `workers` host threads take requests in arrival
 * order, at most one per scene at a time, and run them on their scene's own
 * streams, so requests of different scenes overlap on the GPU as they
 * arrive.  A request starts only when the working memory of all scenes plus
 * its own expected need fits `hbm_budget_bytes`; to make room the server
 * releases idle scenes' work space (never their collision sets), least
 * recently used first.  Results are those of the same calls made directly. */
typedef struct ipcg_server ipcg_server;

typedef struct {
    int status;                 /* IPCG_OK or the request's error code */
    int kind;                   /* 0 barrier, 1 step size */
    double energy;              /* barrier requests */
    double step;                /* step-size requests */
    int64_t contacts;           /* collision-set size (barrier) or CCD candidates (step) */
    int64_t t_submit_ns, t_start_ns, t_end_ns; /* steady clock */
} ipcg_request_result;

int ipcg_server_create(int workers, int64_t hbm_budget_bytes, ipcg_server** out);
int ipcg_server_destroy(ipcg_server* server);
/* Registers a single-scene mesh with the collision set it keeps (both stay
 * owned by the caller and must outlive the server) and its barrier
 * parameters. */
int ipcg_server_add_scene(ipcg_server* server, ipcg_mesh* mesh, ipcg_collisions* collisions,
                          double dhat, double dmin, double stiffness, int64_t* scene);
/* The barrier option bits (use_physical_barrier of ipcg_barrier_*: physical
 * scaling, precision modes, barrier function) of a scene's barrier requests;
 * 0 (the default) is the reference's plain FP64 form. */
int ipcg_server_set_scene_options(ipcg_server* server, int64_t scene, int barrier_options);
/* Host positions are copied at submission. */
int ipcg_server_submit_barrier(ipcg_server* server, int64_t scene, const double* vertices,
                               int psd_method, int64_t* ticket);
int ipcg_server_submit_stepsize(ipcg_server* server, int64_t scene, const double* vertices_t0,
                                const double* vertices_t1, double min_distance, int64_t* ticket);
/* Blocks until the request is done.  gradient (3 nV doubles, host) and
 * hessian (the caller then owns it) may be NULL. */
int ipcg_server_wait(ipcg_server* server, int64_t ticket, ipcg_request_result* out,
                     double* gradient, ipcg_csr** hessian);
/* completed, queued, running, work-space releases, resident bytes */
int ipcg_server_stats(ipcg_server* server, int64_t stats[5]);

/* ---------------------------------------------------------------------- */
/* Single-stencil primitives (for known-answer tests and plugin use)       */
/* ---------------------------------------------------------------------- */

/* TightInclusionCCD::point_triangle_ccd / edge_edge_ccd
 * (tight_inclusion_ccd.cpp:229-336) on a batch of n stencils:
 * x0, x1: (n, 4, 3) positions at t=0 and t=1 (VF: p,t0,t1,t2; EE: a0,a1,b0,b1);
 * hit[n] (int8), toi[n]. */
int ipcg_ccd_stencils(int is_edge_edge, int64_t n, const double* x0, const double* x1,
                      double min_distance, double tmax, double tolerance,
                      int64_t max_iterations, double conservative_rescaling,
                      int8_t* hit, double* toi);

/* Distance types and squared distances of a batch of n stencils
 * (distance_type.cpp:10-211, point_triangle.cpp:11-48, edge_edge.cpp:13-56,
 * point_edge.cpp:10-38).  kind: 0 point-edge (x: n,3,3), 1 point-triangle
 * (n,4,3), 2 edge-edge (n,4,3).  dtype[n] (int8), dist[n]. */
int ipcg_distance_stencils(int kind, int64_t n, const double* x, int8_t* dtype, double* dist);

#ifdef __cplusplus
}
#endif

#endif /* IPCG_H */
