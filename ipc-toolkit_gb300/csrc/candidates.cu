// candidates.cu — a kept broad-phase candidate set and the step-size rules
// that read it (src/ipc/candidates/candidates.cpp).
//
// The reference's Candidates object holds the broad-phase pairs of one
// build: static (boxes inflated by a radius around the positions,
// candidates.cpp:43-125) or swept (boxes around each vertex's motion,
// candidates.cpp:128-222).  The IPC Newton loop uses it for the per-vertex
// safe distances (candidates.cpp:362-404), the step that no non-candidate
// vertex can make unsafe (candidates.cpp:294-329) and the CFL-style step that
// combines that with CCD over the kept pairs (candidates.cpp:252-292,
// 331-360).  Here the pairs stay on the device: EE pairs (ea, eb) and FV
// pairs (face, vertex), the mesh is 3D and single-scene.  This file is
// compiled with -fmad=false: the distances match the oracle bit for bit.
#include <algorithm>
#include <vector>

#include "geom.cuh"
#include "internal.cuh"
#include "profile.cuh"

using namespace ipcg;

struct ipcg_candidates {
    int64_t nee = 0, nfv = 0;
    DBuf<int2> ee, fv;
    const ipcg_mesh* mesh = nullptr; // the mesh they were built on
};

namespace ipcg {
double candidates_collision_free_stepsize(ipcg_mesh* m, const int2* cee, int64_t n_ee, const int2* cfv,
    int64_t n_fv, const double* V0, const double* V1, double min_distance, double tolerance, int64_t max_iterations,
    double rescale);
}

namespace {

constexpr int BLOCK = 128;

// Order-preserving integer key of a finite double (signed comparison).
__device__ __forceinline__ long long okey(double x)
{
    const long long b = __double_as_longlong(x);
    return b ^ ((b >> 63) & 0x7fffffffffffffffLL);
}
__device__ __forceinline__ double ovalue(long long k) { return __longlong_as_double(k ^ ((k >> 63) & 0x7fffffffffffffffLL)); }

__global__ void k_fill_keys(long long* __restrict__ out, int n, double value)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = okey(value);
}
__global__ void k_keys_to_values(const long long* __restrict__ in, double* __restrict__ out, int n)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = ovalue(in[i]);
}

// Per-vertex safe distances (candidates.cpp:362-404): every candidate's
// distance (the closest-feature squared distance, square-rooted, minus the
// minimum separation) lowers the value of each of its vertices.
__global__ void k_safe_distances(const int2* __restrict__ ee, int nee, const int2* __restrict__ fv, int nfv,
    const int* __restrict__ E, const int* __restrict__ F, const double* __restrict__ V, double min_distance,
    long long* __restrict__ key)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nee + nfv) return;
    int ids[4];
    double d2;
    if (i < nee) {
        const int2 c = ee[i];
        ids[0] = E[2 * c.x];
        ids[1] = E[2 * c.x + 1];
        ids[2] = E[2 * c.y];
        ids[3] = E[2 * c.y + 1];
        const V3 a = load_v3(V, ids[0]), b = load_v3(V, ids[1]), c2 = load_v3(V, ids[2]), d = load_v3(V, ids[3]);
        d2 = edge_edge_distance(a, b, c2, d, edge_edge_distance_type(a, b, c2, d));
    } else {
        const int2 c = fv[i - nee];
        ids[0] = c.y;
        ids[1] = F[3 * c.x];
        ids[2] = F[3 * c.x + 1];
        ids[3] = F[3 * c.x + 2];
        const V3 p = load_v3(V, ids[0]), a = load_v3(V, ids[1]), b = load_v3(V, ids[2]), c2 = load_v3(V, ids[3]);
        d2 = point_triangle_distance(p, a, b, c2, point_triangle_distance_type(p, a, b, c2));
    }
    const long long k = okey(sqrt(d2) - min_distance);
    for (int j = 0; j < 4; ++j) atomicMin(key + ids[j], k);
}

// Vertices that appear in some candidate (candidates.cpp:306-321).
__global__ void k_mark_vertices(const int2* __restrict__ ee, int nee, const int2* __restrict__ fv, int nfv,
    const int* __restrict__ E, const int* __restrict__ F, int* __restrict__ mark)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nee + nfv) return;
    if (i < nee) {
        const int2 c = ee[i];
        mark[E[2 * c.x]] = 1;
        mark[E[2 * c.x + 1]] = 1;
        mark[E[2 * c.y]] = 1;
        mark[E[2 * c.y + 1]] = 1;
    } else {
        const int2 c = fv[i - nee];
        mark[c.y] = 1;
        mark[F[3 * c.x]] = 1;
        mark[F[3 * c.x + 1]] = 1;
        mark[F[3 * c.x + 2]] = 1;
    }
}

// Largest displacement norm over marked vertices (candidates.cpp:323-329).
// Norms are non-negative: their bit patterns order like their values.
__global__ void k_max_marked_norm(const double* __restrict__ U, const int* __restrict__ mark, int nV,
    unsigned long long* __restrict__ out)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nV || !mark[i]) return;
    const V3 u = load_v3(U, i);
    const double nrm = sqrt(dot(u, u));
    atomicMax(out, (unsigned long long)__double_as_longlong(nrm));
}

__global__ void k_displacements(const double* __restrict__ V0, const double* __restrict__ V1, double* __restrict__ U,
    int n)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) U[i] = V1[i] - V0[i];
}

template <typename F> int cand_call(F&& f)
{
    try {
        f();
        set_last_error("");
        return IPCG_OK;
    } catch (const Error& e) {
        set_last_error(e.what());
        return e.code;
    } catch (const std::bad_alloc&) {
        set_last_error("host allocation failed");
        return IPCG_ERR_OOM;
    } catch (const std::exception& e) {
        set_last_error(e.what());
        return IPCG_ERR_INVALID;
    }
}

void check(bool ok, const char* msg)
{
    if (!ok) throw Error(IPCG_ERR_INVALID, msg);
}

ipcg_mesh* checked_mesh(const ipcg_candidates* c, const ipcg_mesh* mesh)
{
    check(c && mesh, "NULL argument");
    check(mesh->n_scenes == 1, "candidate sets are built on single-scene meshes");
    check(c->mesh == nullptr || c->mesh == mesh, "the candidates were built on another mesh");
    require_no_codim_vertices(mesh);
    ipcg_mesh* m = const_cast<ipcg_mesh*>(mesh);
    IPCG_CUDA(cudaSetDevice(m->device));
    return m;
}

void build(ipcg_candidates* c, ipcg_mesh* m, const double* V0, const double* V1, double inflation_radius)
{
    cudaStream_t s = m->stream;
    m->scene_md.reserve(2);
    IPCG_CUDA(cudaMemcpyAsync(m->scene_md.p, &inflation_radius, sizeof(double), cudaMemcpyHostToDevice, s));
    int64_t nee = 0, nfv = 0;
    detect_candidates(m, V0, V1, m->scene_md.p, nee, nfv);
    c->ee.reserve(nee + 1);
    c->fv.reserve(nfv + 1);
    if (nee) IPCG_CUDA(cudaMemcpyAsync(c->ee.p, m->cand.p, sizeof(int2) * nee, cudaMemcpyDeviceToDevice, s));
    if (nfv)
        IPCG_CUDA(cudaMemcpyAsync(c->fv.p, m->cand.p + m->cand_cap, sizeof(int2) * nfv, cudaMemcpyDeviceToDevice, s));
    IPCG_CUDA(cudaStreamSynchronize(s));
    c->nee = nee;
    c->nfv = nfv;
    c->mesh = m;
}

double noncandidate_step(const ipcg_candidates* c, ipcg_mesh* m, const double* U, double dhat)
{
    if (c->nee + c->nfv == 0) return 1.0;
    cudaStream_t s = m->stream;
    const int nV = (int)m->nV, n = (int)(c->nee + c->nfv);
    m->ivals_b.reserve(nV + 1);
    m->toi_bits.reserve(1);
    IPCG_CUDA(cudaMemsetAsync(m->ivals_b.p, 0, sizeof(int) * nV, s));
    IPCG_CUDA(cudaMemsetAsync(m->toi_bits.p, 0, sizeof(unsigned long long), s));
    IPCG_LAUNCH("k_mark_vertices", s, k_mark_vertices<<<(n + BLOCK - 1) / BLOCK, BLOCK, 0, s>>>(c->ee.p,
        (int)c->nee, c->fv.p, (int)c->nfv, m->E.p, m->F.p, m->ivals_b.p));
    IPCG_LAUNCH("k_max_marked_norm", s, k_max_marked_norm<<<(nV + BLOCK - 1) / BLOCK, BLOCK, 0, s>>>(U,
        m->ivals_b.p, nV, m->toi_bits.p));
    unsigned long long bits = 0;
    IPCG_CUDA(cudaMemcpyAsync(&bits, m->toi_bits.p, sizeof(bits), cudaMemcpyDeviceToHost, s));
    IPCG_CUDA(cudaStreamSynchronize(s));
    double mx;
    memcpy(&mx, &bits, sizeof(mx));
    return 0.5 * dhat / mx;
}

} // namespace

extern "C" {

int ipcg_candidates_create(ipcg_candidates** out)
{
    return cand_call([&] {
        check(out != nullptr, "out is NULL");
        *out = new ipcg_candidates();
    });
}

int ipcg_candidates_destroy(ipcg_candidates* c)
{
    return cand_call([&] { delete c; });
}

int ipcg_candidates_build(ipcg_candidates* c, const ipcg_mesh* mesh, const double* V, double inflation_radius)
{
    return cand_call([&] {
        if (c) c->mesh = nullptr; // a rebuild may use another mesh
        ipcg_mesh* m = checked_mesh(c, mesh);
        check(V || m->nV == 0, "vertices is NULL");
        check(inflation_radius >= 0, "inflation_radius must be non-negative");
        const double* dV = stage_positions(m, V, m->V0);
        build(c, m, dV, dV, inflation_radius);
    });
}

int ipcg_candidates_build_swept(ipcg_candidates* c, const ipcg_mesh* mesh, const double* V0, const double* V1,
    double inflation_radius)
{
    return cand_call([&] {
        if (c) c->mesh = nullptr; // a rebuild may use another mesh
        ipcg_mesh* m = checked_mesh(c, mesh);
        check((V0 && V1) || m->nV == 0, "vertices is NULL");
        check(inflation_radius >= 0, "inflation_radius must be non-negative");
        const double* d0 = stage_positions(m, V0, m->V0);
        const double* d1 = stage_positions(m, V1, m->V1);
        build(c, m, d0, d1, inflation_radius);
    });
}

int ipcg_candidates_counts(const ipcg_candidates* c, int64_t counts[2])
{
    return cand_call([&] {
        check(c && counts, "NULL argument");
        counts[0] = c->nee;
        counts[1] = c->nfv;
    });
}

int ipcg_candidates_get(const ipcg_candidates* c, int32_t* ee, int32_t* fv)
{
    return cand_call([&] {
        check(c != nullptr, "NULL argument");
        if (ee && c->nee) IPCG_CUDA(cudaMemcpy(ee, c->ee.p, sizeof(int2) * c->nee, cudaMemcpyDefault));
        if (fv && c->nfv) IPCG_CUDA(cudaMemcpy(fv, c->fv.p, sizeof(int2) * c->nfv, cudaMemcpyDefault));
    });
}

int ipcg_candidates_per_vertex_safe_distances(const ipcg_candidates* c, const ipcg_mesh* mesh, const double* V,
    double inflation_radius, double min_distance, double* out)
{
    return cand_call([&] {
        ipcg_mesh* m = checked_mesh(c, mesh);
        check(out && (V || m->nV == 0), "NULL argument");
        check(inflation_radius >= min_distance, "inflation_radius must be at least min_distance");
        cudaStream_t s = m->stream;
        const int nV = (int)m->nV, n = (int)(c->nee + c->nfv);
        const double* dV = stage_positions(m, V, m->V0);
        DBuf<long long> keys;
        DBuf<double> vals;
        keys.reserve(nV + 1);
        vals.reserve(nV + 1);
        if (nV)
            IPCG_LAUNCH("k_fill_keys", s, k_fill_keys<<<(nV + BLOCK - 1) / BLOCK, BLOCK, 0, s>>>(keys.p, nV,
                inflation_radius - min_distance));
        if (n)
            IPCG_LAUNCH("k_safe_distances", s, k_safe_distances<<<(n + BLOCK - 1) / BLOCK, BLOCK, 0, s>>>(c->ee.p,
                (int)c->nee, c->fv.p, (int)c->nfv, m->E.p, m->F.p, dV, min_distance, keys.p));
        if (nV)
            IPCG_LAUNCH("k_keys_to_values", s, k_keys_to_values<<<(nV + BLOCK - 1) / BLOCK, BLOCK, 0, s>>>(keys.p,
                vals.p, nV));
        if (nV) IPCG_CUDA(cudaMemcpyAsync(out, vals.p, sizeof(double) * nV, cudaMemcpyDefault, s));
        IPCG_CUDA(cudaStreamSynchronize(s));
    });
}

int ipcg_candidates_collision_free_stepsize(const ipcg_candidates* c, const ipcg_mesh* mesh, const double* V0,
    const double* V1, double min_distance, double tolerance, int64_t max_iterations, double rescale, double* step)
{
    return cand_call([&] {
        ipcg_mesh* m = checked_mesh(c, mesh);
        check(step && ((V0 && V1) || m->nV == 0), "NULL argument");
        check(min_distance >= 0 && tolerance > 0 && rescale > 0 && rescale <= 1, "bad CCD parameters");
        const double* d0 = stage_positions(m, V0, m->V0);
        const double* d1 = stage_positions(m, V1, m->V1);
        *step = candidates_collision_free_stepsize(m, c->ee.p, c->nee, c->fv.p, c->nfv, d0, d1, min_distance,
            tolerance, max_iterations, rescale);
    });
}

int ipcg_candidates_noncandidate_conservative_stepsize(const ipcg_candidates* c, const ipcg_mesh* mesh,
    const double* displacements, double dhat, double* step)
{
    return cand_call([&] {
        ipcg_mesh* m = checked_mesh(c, mesh);
        check(step && (displacements || m->nV == 0), "NULL argument");
        const double* dU = stage_positions(m, displacements, m->V1);
        *step = noncandidate_step(c, m, dU, dhat);
    });
}

int ipcg_candidates_cfl_stepsize(const ipcg_candidates* c, const ipcg_mesh* mesh, const double* V0, const double* V1,
    double dhat, double min_distance, double tolerance, int64_t max_iterations, double rescale, double* step)
{
    return cand_call([&] {
        ipcg_mesh* m = checked_mesh(c, mesh);
        check(step && ((V0 && V1) || m->nV == 0), "NULL argument");
        check(min_distance >= 0 && tolerance > 0 && rescale > 0 && rescale <= 1, "bad CCD parameters");
        cudaStream_t s = m->stream;
        const double* d0 = stage_positions(m, V0, m->V0);
        const double* d1 = stage_positions(m, V1, m->V1);
        const double alpha_C = candidates_collision_free_stepsize(m, c->ee.p, c->nee, c->fv.p, c->nfv, d0, d1,
            min_distance, tolerance, max_iterations, rescale);
        DBuf<double> U;
        U.reserve(3 * m->nV + 1);
        if (m->nV)
            IPCG_LAUNCH("k_displacements", s, k_displacements<<<(int)((3 * m->nV + BLOCK - 1) / BLOCK), BLOCK, 0, s>>>(
                d0, d1, U.p, (int)(3 * m->nV)));
        const double alpha_F = noncandidate_step(c, m, U.p, dhat);
        if (alpha_F < 0.5 * alpha_C) {
            // candidates.cpp:349-356: too little margin; full CCD instead
            collision_free_stepsize(m, d0, d1, &min_distance, tolerance, max_iterations, rescale, step, nullptr);
            return;
        }
        *step = std::min(alpha_C, alpha_F);
    });
}

} // extern "C"
