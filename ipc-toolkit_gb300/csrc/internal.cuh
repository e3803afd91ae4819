// internal.cuh — host-side objects of the C ABI (device-resident state).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <stdexcept>
#include <string>
#include <atomic>
#include <memory>
#include <vector>

#include "../../include/ipcg.h"

namespace ipcg {

struct Error : std::runtime_error {
    int code;
    Error(int c, const std::string& m) : std::runtime_error(m), code(c) { }
};

#define IPCG_CUDA(x)                                                                                              \
    do {                                                                                                          \
        cudaError_t e_ = (x);                                                                                     \
        if (e_ != cudaSuccess) {                                                                                  \
            throw ::ipcg::Error(e_ == cudaErrorMemoryAllocation ? IPCG_ERR_OOM : IPCG_ERR_CUDA,                  \
                std::string(#x) + ": " + cudaGetErrorString(e_));                                                 \
        }                                                                                                         \
    } while (0)

#define IPCG_CHECK_LAUNCH() IPCG_CUDA(cudaGetLastError())

// Grow-only device buffer.
template <typename T> struct DBuf {
    T* p = nullptr;
    size_t cap = 0;
    DBuf() = default;
    DBuf(const DBuf&) = delete;
    DBuf& operator=(const DBuf&) = delete;
    void reserve(size_t n)
    {
        if (n <= cap && p) return;
        release();
        size_t c = n < 16 ? 16 : n + n / 4;
        IPCG_CUDA(cudaMalloc((void**)&p, c * sizeof(T)));
        cap = c;
    }
    // Grow to at least n elements keeping the first `used` ones (stream-ordered copy).
    void grow_keep(size_t n, size_t used, cudaStream_t s)
    {
        if (n <= cap && p) return;
        const size_t c = n < 16 ? 16 : n + n / 4;
        T* q = nullptr;
        IPCG_CUDA(cudaMalloc((void**)&q, c * sizeof(T)));
        if (used && p) {
            cudaError_t e = cudaMemcpyAsync(q, p, used * sizeof(T), cudaMemcpyDeviceToDevice, s);
            if (e == cudaSuccess) e = cudaStreamSynchronize(s); // the old buffer is freed next
            if (e != cudaSuccess) {
                cudaFree(q);
                IPCG_CUDA(e);
            }
        }
        release();
        p = q;
        cap = c;
    }
    void release()
    {
        if (p) cudaFree(p);
        p = nullptr;
        cap = 0;
    }
    ~DBuf() { release(); }
};

// The library's stream-ordered memory pool on the current device (memory is
// kept in the pool when freed, so per-call outputs are reused without
// cudaMalloc / cudaFree and the device synchronisation cudaFree implies).
cudaMemPool_t device_pool();

// Device buffer from device_pool(), allocated and freed in stream order;
// used for per-call outputs handed to the caller.
template <typename T> struct PBuf {
    T* p = nullptr;
    size_t cap = 0;
    cudaStream_t s = nullptr;
    PBuf() = default;
    PBuf(const PBuf&) = delete;
    PBuf& operator=(const PBuf&) = delete;
    // Grow to at least n elements keeping the first `used` ones.
    void grow_keep(size_t n, size_t used, cudaStream_t stream)
    {
        if (n <= cap && p) return;
        const size_t c = n < 16 ? 16 : n + n / 4;
        T* q = nullptr;
        IPCG_CUDA(cudaMallocFromPoolAsync((void**)&q, c * sizeof(T), device_pool(), stream));
        if (used && p) IPCG_CUDA(cudaMemcpyAsync(q, p, used * sizeof(T), cudaMemcpyDeviceToDevice, stream));
        release();
        p = q;
        cap = c;
        s = stream;
    }
    void reserve(size_t n, cudaStream_t stream) { grow_keep(n, 0, stream); }
    void release()
    {
        if (p) cudaFreeAsync(p, s);
        p = nullptr;
        cap = 0;
    }
    ~PBuf() { release(); }
};

// Pinned host staging (for small count read-backs).
template <typename T> struct HBuf {
    T* p = nullptr;
    size_t cap = 0;
    void reserve(size_t n)
    {
        if (n <= cap && p) return;
        release();
        IPCG_CUDA(cudaMallocHost((void**)&p, n * sizeof(T)));
        cap = n;
    }
    void release()
    {
        if (p) cudaFreeHost(p);
        p = nullptr;
        cap = 0;
    }
    ~HBuf() { release(); }
};

// Linear BVH over FP32 outward-rounded boxes.  Nodes 0..n-2 are internal
// (root = 0), n-1..2n-2 leaves in Morton order.  lo.w / hi.w hold the two
// child indices (internal) or the primitive id / -1 (leaf) as int bits;
// last[i] is the largest sorted leaf index under node i.
// Scenes of a batch are kept apart by putting the scene id above the Morton
// code in the 64-bit sort key: each scene's leaves are contiguous, and
// leaf_scene[first[i]] .. leaf_scene[last[i]] is the scene range of node i.
struct LBVH {
    int n = 0;
    DBuf<float4> lo, hi;
    DBuf<int> first, last, parent, flags, leaf_scene;
    DBuf<unsigned long long> codes, codes_sorted;
    DBuf<int> ids, ids_sorted;
    DBuf<float4> plo, phi; // per-primitive leaf boxes before sorting
};

// Per-scene view passed to kernels.  For a single scene vscene is null and
// every array has one entry.
struct SceneView {
    int n;                 // number of scenes
    const int* vscene;     // per-vertex scene id, or null (one scene)
    __device__ __forceinline__ int of(int v) const { return vscene ? __ldg(vscene + v) : 0; }
};

// Flags of device-side guards (bit set => the call fails loudly).
enum : int { GUARD_STACK = 1, GUARD_CAPACITY = 2 };

} // namespace ipcg

namespace ipcg {
struct EghCache;   // egh.cu: cached Hessian pattern and captured graph of a collision set
struct EghPattern; // egh.cu: CSR row pointers and columns shared with the matrices built on them
}

struct ipcg_mesh {
    int device = 0;
    uint64_t serial = 0;             // unique per mesh created in this process (cache keys)
    int64_t nV = 0, nE = 0, nF = 0;
    int64_t n_scenes = 1;
    // CollisionMesh::num_codim_vertices / num_codim_edges (collision_mesh.cpp:
    // 145-183): vertices in no edge, edges in no face
    int64_t n_codim_vertices = 0, n_codim_edges = 0;
    std::vector<int64_t> h_voff;     // vertex offsets of the scenes (n_scenes + 1)
    ipcg::DBuf<int64_t> scene_offs;  // batches: vertex, edge, edge, face offsets (4 x (n_scenes + 1))
    ipcg::DBuf<int> vscene;          // per-vertex scene id (batches only)
    ipcg::DBuf<double> scene_r;      // per-scene inflation radius of the current build
    ipcg::DBuf<double> scene_off2;   // per-scene (dhat + dmin)^2 of the current build
    ipcg::DBuf<unsigned char> params_buf; // per-scene barrier parameters
    std::vector<unsigned char> params_host; // what params_buf holds
    ipcg::DBuf<double> scene_md;     // CCD: per-scene 0.5*min_distance, then min_distance
    cudaStream_t stream = nullptr;
    // streams for work that overlaps the main one (the Hessian's VV, EV and
    // FV local Hessians on `side`, its sparsity pattern on `side2`), with the
    // events that fork and join them
    cudaStream_t side = nullptr, side2 = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_side = nullptr, ev_pattern = nullptr;
    ipcg::DBuf<double> rest;
    ipcg::DBuf<int> E, F, F2E;
    std::vector<int32_t> h_F2E;
    ipcg::DBuf<double> rec_w;        // area weighting: VV / EV record weights
    ipcg::DBuf<int2> rec_src;        // area-weighted shape derivatives: VV / EV record sources
    ipcg::DBuf<unsigned long long> wkeys; // weighted merge scratch
    ipcg::DBuf<int> widx;
    // adjacencies of CollisionMesh::init_adjacencies (built on first use):
    // CSR offsets + sorted lists; boundary flags per vertex
    bool adj_ready = false;
    int max_vertex_edges = 0;
    ipcg::DBuf<int> vv_off, vv_adj, ve_off, ve_adj, ev_off, ev_adj;
    ipcg::DBuf<int> vf_off, vf_adj, ef_off, ef_adj; // vertex -> faces, edge -> faces
    ipcg::DBuf<uint8_t> boundary;
    // improved-max-approximation scratch
    ipcg::DBuf<unsigned long long> imp_keys;
    ipcg::DBuf<int2> imp_ids;
    ipcg::DBuf<double> imp_w, imp_eps, rec_ee_w;
    ipcg::DBuf<int8_t> imp_dt;
    ipcg::DBuf<int> imp_flag, imp_offs;
    ipcg::DBuf<double> vertex_area;  // rest-mesh areas (area weighting)
    ipcg::DBuf<double> edge_area;
    // work space shared by the calls on this mesh
    ipcg::DBuf<double> V0, V1;       // device copies of host position inputs
    ipcg::DBuf<double> grad_stage;   // device gradient for a host gradient output
    ipcg::DBuf<double> bounds;       // mesh AABB scratch
    ipcg::LBVH ebvh, fbvh;
    ipcg::DBuf<int2> cand;           // broad-phase candidates (EE then FV)
    ipcg::DBuf<int> counters;        // device counters
    ipcg::HBuf<int> h_counters;
    ipcg::DBuf<char> tmp;            // CUB temporary storage
    ipcg::DBuf<unsigned long long> keys_a, keys_b;
    ipcg::DBuf<double> ccd_lb; // per CCD candidate: lower bound on its time of impact
    ipcg::DBuf<long long> ccd_stats; // testing: CCD pass statistics (ipcg_testing_ccd_stats)
    bool ccd_stats_live = false;
    ipcg::DBuf<int> ivals_a, ivals_b;
    ipcg::DBuf<int8_t> i8tmp;
    ipcg::DBuf<double> partial;      // reduction partials
    ipcg::DBuf<unsigned long long> toi_bits;
    ipcg::DBuf<long long> guard;     // device-side index self-check record
    ipcg::DBuf<double> hs;           // per-contact local Hessian slabs (144 doubles each)
    ipcg::DBuf<uint8_t> proj;        // per-contact "project to PSD" flags
    long long h_guard[4] = { 0, 0, 0, 0 };
    int64_t cand_cap = 0;
    ~ipcg_mesh();
};

struct ipcg_collisions {
    int64_t nvv = 0, nev = 0, nee = 0, nfv = 0;
    uint64_t version = 0;            // bumped by every build or load (cache keys)
    std::shared_ptr<ipcg::EghCache> egh; // cached Hessian pattern + graph (egh.cu)
    int64_t n_cand_ee = 0, n_cand_fv = 0;
    double dmin = 0;
    std::vector<double> scene_dmin;  // per scene (batches)
    bool sorted = false;             // lists sorted by key (built here, not loaded)
    int use_area_weighting = 0;      // NormalCollisions::use_area_weighting()
    int set_type = 0;                // CollisionSetType: 0 IPC, 1 IMPROVED_MAX_APPROX
    int enable_shape_derivatives = 0; // NormalCollisions::enable_shape_derivatives()
    int built_with_shape = 0;        // the flag as it was at the last build
    int built_with_area = 0;         // area weighting at the last build
    // area-weighted shape derivatives: the weight sources of each merged VV /
    // EV record ((v, -1) for a face-vertex candidate's vertex, (ea, eb) for an
    // edge-edge candidate's edges), with per-record offsets
    ipcg::DBuf<int> vv_src_off, ev_src_off;
    ipcg::DBuf<int2> vv_src, ev_src;
    ipcg::DBuf<int2> vv, ev, ee, fv;
    ipcg::DBuf<double> vv_w, ev_w, ee_w, fv_w, ee_eps;
    ipcg::DBuf<int8_t> ee_dtype;
    int64_t size() const { return nvv + nev + nee + nfv; }
};

// TangentialCollisions: stencils (and weights) in an ipcg_collisions, plus
// per collision the normal force, closest point (2), tangent basis (6) and
// blended mu_s / mu_k.
struct ipcg_tangential {
    ipcg_collisions st;
    ipcg::DBuf<double> N, cp, P, mu_s, mu_k;
    // anisotropy: slip scaling (2 per collision), directional static and
    // kinetic coefficients (2 each), lagged effective coefficients
    ipcg::DBuf<double> mu_aniso, mu_s_aniso, mu_k_aniso, mu_s_eff, mu_k_eff;
    const ipcg_mesh* mesh = nullptr;
};

struct ipcg_csr {
    int64_t rows = 0, nnz = 0;
    ipcg::PBuf<int64_t> row_ptr;
    ipcg::PBuf<int> col;
    ipcg::PBuf<double> val;
    cudaStream_t stream = nullptr;
    // A matrix built on a cached pattern shares its row pointers and columns
    // (kept alive by `pattern`) instead of owning copies.
    std::shared_ptr<const ipcg::EghPattern> pattern;
    const int64_t* row_ptr_shared = nullptr;
    const int* col_shared = nullptr;
    const int64_t* rowp() const { return row_ptr_shared ? row_ptr_shared : row_ptr.p; }
    const int* colp() const { return col_shared ? col_shared : col.p; }
    // Freed on the default stream: the matrix may outlive its mesh's stream,
    // and every call that produced or read it has finished by then.
    ~ipcg_csr() { row_ptr.s = col.s = val.s = nullptr; }
};

namespace ipcg {

// Stage a position array on the device: returns a device pointer (the input
// itself if it already is device memory).
const double* stage_positions(ipcg_mesh* m, const double* V, DBuf<double>& buf);
bool is_device_ptr(const void* p);

inline SceneView scene_view(const ipcg_mesh* m) { return SceneView { (int)m->n_scenes, m->n_scenes > 1 ? m->vscene.p : nullptr }; }

// abi.cu: the calling thread's message for ipcg_last_error()
void set_last_error(const std::string& msg);

// Collision-set builds, candidate builds and step sizes find contacts through
// the edge-edge and face-vertex passes only.  The reference adds
// vertex-vertex candidates among codimensional vertices (vertices in no edge)
// and edge-vertex candidates between codimensional edges and those vertices
// (candidates.cpp:66-116, 152-210); those passes are not built here, so a mesh
// on which they would find anything -- two or more codimensional vertices, or
// one with a codimensional edge -- is refused instead of giving an incomplete
// set.  (A single loose vertex is still found by the face-vertex pass.)
void require_no_codim_vertices(const ipcg_mesh* m);

// barrier.cu: contacts per Hessian chunk of a batch (scratch memory bound)
extern std::atomic<int64_t> g_hess_chunk_contacts;

// broad_phase.cu
void build_lbvh(ipcg_mesh* m, LBVH& bvh, int kind /*2 edges, 3 faces*/, const double* V0, const double* V1,
    const double* scene_r);
// Detect EE + FV candidates into m->cand with the per-scene inflation radii
// scene_r (device, one per scene); returns (n_ee, n_fv).
void detect_candidates(ipcg_mesh* m, const double* V0, const double* V1, const double* scene_r, int64_t& n_ee,
    int64_t& n_fv);

// collisions.cu: per-vertex and per-edge areas of the rest mesh
// (collision_mesh.cpp:309-374), summed in face order on the host.
void mesh_areas_host(const double* rest, int64_t nV, const int32_t* E, int64_t nE, const int32_t* F, int64_t nF,
    const int32_t* F2E, double* vertex_area, double* edge_area);
// collisions.cu: the mesh adjacencies (built once, on first use)
void ensure_adjacency(ipcg_mesh* m);
// collisions.cu: per-scene dhat / dmin (host arrays of n_scenes)
void build_collision_set(ipcg_collisions* c, ipcg_mesh* m, const double* V, const double* dhat, const double* dmin);

// barrier.cu
struct BarrierArgs {
    double dhat, kappa, dmin;
    int physical;
    int psd;
    const double* scene_dhat = nullptr;  // per scene (batches), host
    const double* scene_kappa = nullptr; // per scene (batches), host
    int mixed = 0;                       // FP32 point-triangle contacts
    int kind = 0;                        // barrier function (IPCG_BARRIER_* kinds)
    int shape = 0;                       // Hessian slot holds the shape derivative
    int fp32_local = 0;                  // FP32 local Hessians but near-parallel EE
    int df64_psd = 0;                    // PSD eigenpairs in df64 (cached-pattern pass)
};
// The barrier option bits of the C ABI (physical scaling, precision modes,
// barrier function) into a; throws IPCG_ERR_INVALID on unknown bits.
void barrier_options(int bits, BarrierArgs& a);
struct FrictionView;
void barrier_evaluate(const ipcg_collisions* c, ipcg_mesh* m, const double* V, const BarrierArgs& a,
    double* energy_host, double* grad_dev_or_null, ipcg_csr* hess_or_null, const FrictionView* friction = nullptr);
// Friction (tangential_potential.cpp): per tangential collision, in the
// order of its stencil lists, the normal force N, closest point cp (2), tangent
// basis P (b0 xyz, b1 xyz) and blended mu_s / mu_k.
struct FrictionView {
    const double *N, *cp, *P, *mu_s, *mu_k; // mu: the lagged effective coefficients
    const double* aniso;                     // slip scaling per collision (2)
    double eps_v;
};
void barrier_evaluate_friction(const ipcg_collisions* stencils, ipcg_mesh* m, const double* U, const FrictionView& f,
    int psd, double* energy_host, double* grad_dev, ipcg_csr* hess);
// TangentialCollisions::build: from the normal set at positions V with the
// barrier potential a, per-vertex mu (device); fills t (isotropic defaults).
void tangential_build(const ipcg_collisions* normal, ipcg_mesh* m, const double* V, const BarrierArgs& a,
    const double* mu_s_dev, const double* mu_k_dev, ipcg_tangential* t);
// TangentialPotential::force into force_dev (3 nV, zeroed first; device inputs)
void friction_force(const ipcg_tangential* t, ipcg_mesh* m, const double* rest, const double* lagged,
    const double* vel, const BarrierArgs& a, double eps_v, int no_mu, double* force_dev);
// update_lagged_anisotropic_friction_coefficients (device inputs)
void tangential_update_lagged(ipcg_tangential* t, ipcg_mesh* m, const double* rest, const double* lagged,
    const double* vel);
// Gauss-Newton Hessian diagonal (device, 3 nV) and/or quadratic form p^T H p
// (p on the device, result on the host).
void barrier_gauss_newton(const ipcg_collisions* c, ipcg_mesh* m, const double* V, const BarrierArgs& a,
    double* diag_dev_or_null, const double* p_dev, double* qf_host_or_null);
// has_intersections (ipc.cpp:110-167): some edge crosses a triangle it does
// not share a vertex with (a batch answers for all its scenes together).
bool has_intersections(ipcg_mesh* m, const double* V);
// Smallest squared distance over the collision set (+inf when empty).
double collisions_min_distance(const ipcg_collisions* c, ipcg_mesh* m, const double* V);
// is_step_collision_free (ipc.cpp:20-40): no candidate has a hit in [0, 1].
bool step_collision_free(ipcg_mesh* m, const double* V0, const double* V1, double min_distance, double tolerance,
    int64_t max_iterations, double rescale);

// egh.cu: energy (host, one per scene), gradient (device, 3 nV) and Hessian of
// the barrier in one pass with the collision set's cached pattern, replayed as
// one CUDA graph.  Returns false (nothing done) when the request is not one
// this pipeline serves (shape derivatives, no Hessian, or a batch set loaded
// unsorted); the caller then uses barrier_evaluate.
bool barrier_egh(const ipcg_collisions* c, ipcg_mesh* m, const double* V, const BarrierArgs& a, double* energy_host,
    double* grad_dev, ipcg_csr* hess);
// Tuning of the fused kernel on the current device: threads per block, blocks
// per SM and warp tiles taken per work-queue grab.
struct EghTuning {
    int threads = 64, blocks_per_sm = 4, tiles_per_grab = 1;
};
// Launch shapes of the per-contact stages of the cached-pattern pass on the
// current device: 0 the local Hessians, 1 the FP64 projection and scatter,
// 2 the df64 one.
EghTuning egh_tuning(int stage);
// The device's FP64 fused multiply-add rate (TFLOP/s), measured by a kernel
// of independent DFMA chains: the roofline of FP64-bound, non-tensor code.
double fp64_fma_rate();
// Testing: the df64 projection defers every contact to its FP64 fix-up pass.
void egh_defer_df64(bool on);
// ccd.cu: testing switch for the step-size passes' statistics
extern std::atomic<int> g_ccd_stats;
// ccd_bound.cu: per step-size query (EE candidates, then FV), a lower bound
// on its time of impact (lb), and sort keys (scene | estimate) with the
// query indices
void ccd_bound_launch(cudaStream_t s, const int2* cee, int n_ee, const int2* cfv, int n_fv, const double* V0,
    const double* V1, const int* E, const int* F, const double* min_distance, SceneView sv, double tolerance,
    double rescale, double* lb, unsigned long long* keys, int* ids);
extern std::atomic<long long> g_ccd_thread_budget;
void egh_set_tuning(int stage, const EghTuning& t);
// Time both stages over candidate tunings on this set's largest chunk and
// keep the fastest for the device; returns a JSON report.
std::string egh_autotune(const ipcg_collisions* c, ipcg_mesh* m, const double* V, const BarrierArgs& a);
// barrier.cu: derivative `order` (0-2) of barrier function `kind`
// (IPCG_BARRIER_* kinds) at x with activation xhat, on the host.
double barrier_derivative_host(int kind, int order, double x, double xhat);
// barrier.cu: a . b and b . b of two device vectors of n doubles (deterministic).
void dot_pair_device(const double* a, const double* b, int64_t n, double* ab, double* bb);

// Caller-owned device arrays of a collision set (layout of ipcg_collisions_get).
struct ContactsNoAlloc {
    int64_t nvv, nev, nee, nfv;
    const int32_t *vv, *ev, *ee, *fv;
    const double *vv_w, *ev_w, *ee_w, *fv_w, *ee_eps;
    const int8_t* ee_dtype;
};
// barrier.cu: the energy with its reduction scratch in a static device array;
// every index is checked against nV / nE / nF on the device (a bad one makes
// the energy NaN instead of reading out of bounds)
void barrier_energy_noalloc(const double* V, const int* E, const int* F, int64_t nV, int64_t nE, int64_t nF,
    const ContactsNoAlloc& in, double dhat, double kappa, double dmin, int physical, double* energy, cudaStream_t s);
// whether p is device (or managed) memory that the current device can address
bool is_device_ptr_on_current(const void* p);

// ccd.cu
// Per scene: min_distance[n_scenes] (host) in, steps[n_scenes] (host) out.
void collision_free_stepsize(ipcg_mesh* m, const double* V0, const double* V1, const double* min_distance,
    double tolerance, int64_t max_iterations, double rescale, double* steps, int64_t* n_candidates);
void ccd_stencils(cudaStream_t s, int is_ee, int64_t n, const double* x0, const double* x1, double min_distance,
    double tmax, double tolerance, int64_t max_iterations, double rescale, int8_t* hit, double* toi);
void distance_stencils(cudaStream_t s, int kind, int64_t n, const double* x, int8_t* dtype, double* dist);

// sort.cu (CUB wrappers)
void sort_pairs_u32(ipcg_mesh* m, cudaStream_t st, const unsigned* k_in, unsigned* k_out, const int* v_in, int* v_out, int n,
    int end_bit);
void sort_keys_u64(ipcg_mesh* m, cudaStream_t st, const unsigned long long* k_in, unsigned long long* k_out, int n, int end_bit);
void sort_pairs_u64(ipcg_mesh* m, cudaStream_t st, const unsigned long long* k_in, unsigned long long* k_out, const int* v_in,
    int* v_out, int n, int end_bit);
// run-length encode sorted keys; writes the number of runs to d_num (device)
void rle_u64(ipcg_mesh* m, cudaStream_t st, const unsigned long long* k_in, unsigned long long* uniq, int* counts, int* d_num, int n);
void unique_u64(ipcg_mesh* m, cudaStream_t st, const unsigned long long* k_in, unsigned long long* uniq, int* d_num, int n);
void exclusive_sum_i32(ipcg_mesh* m, cudaStream_t st, const int* in, int* out, int n);
void exclusive_sum_i64(ipcg_mesh* m, cudaStream_t st, const int64_t* in, int64_t* out, int n);
// barrier.cu: NormalPotential::shape_derivative of an area-weighted set
void shape_derivative_area(const ipcg_collisions* c, ipcg_mesh* m, const double* V, const BarrierArgs& a,
    ipcg_csr* out);

inline int grid_for(int64_t n, int block) { return (int)((n + block - 1) / block); }
inline int bits_for(int64_t n)
{
    int b = 1;
    while ((1ll << b) < n) ++b;
    return b;
}

} // namespace ipcg
