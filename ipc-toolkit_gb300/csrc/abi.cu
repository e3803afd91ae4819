// abi.cu — the extern "C" boundary (include/ipcg.h).
//
// Each entry point validates its arguments, stages host inputs on the
// device, runs the device path and converts C++ exceptions into status
// codes with a per-thread error message.  No entry point falls back to host
// computation: without a CUDA device every compute call fails with
// IPCG_ERR_NO_DEVICE.
#include <atomic>
#include <cmath>
#include <cstring>
#include <map>
#include <mutex>
#include <unordered_map>

#include "internal.cuh"
#include "profile.cuh"

using namespace ipcg;

namespace {

thread_local std::string g_last_error;

template <typename F> int guarded(F&& f)
{
    try {
        f();
        g_last_error.clear();
        return IPCG_OK;
    } catch (const Error& e) {
        g_last_error = e.what();
        return e.code;
    } catch (const std::bad_alloc&) {
        g_last_error = "host allocation failed";
        return IPCG_ERR_OOM;
    } catch (const std::exception& e) {
        g_last_error = e.what();
        return IPCG_ERR_INVALID;
    }
}

void require(bool ok, const char* msg)
{
    if (!ok) throw Error(IPCG_ERR_INVALID, msg);
}

void require_device()
{
    int n = 0;
    const cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess || n == 0) {
        cudaGetLastError();
        throw Error(IPCG_ERR_NO_DEVICE, "no CUDA device available");
    }
}

void copy_out(void* dst, const void* src_dev, size_t bytes, cudaStream_t s)
{
    if (bytes == 0 || dst == nullptr) return;
    IPCG_CUDA(cudaMemcpyAsync(dst, src_dev, bytes, cudaMemcpyDefault, s));
}

} // namespace

namespace ipcg {

namespace prof {
namespace {
std::atomic<bool> g_enabled { false };
std::atomic<long long> g_launches { 0 };
std::mutex g_mu;
struct Pending {
    const char* name;
    cudaEvent_t a, b;
};
std::vector<Pending> g_pending;
std::vector<cudaEvent_t> g_free_events;
struct Stat {
    long long launches = 0;
    double ms = 0;
};
std::map<std::string, Stat> g_stats;

void drain()
{
    for (auto& p : g_pending) {
        float ms = 0;
        if (cudaEventSynchronize(p.b) == cudaSuccess && cudaEventElapsedTime(&ms, p.a, p.b) == cudaSuccess) {
            Stat& s = g_stats[p.name];
            s.launches++;
            s.ms += ms;
        }
        g_free_events.push_back(p.a);
        g_free_events.push_back(p.b);
    }
    g_pending.clear();
    cudaGetLastError();
}
} // namespace

bool enabled() { return g_enabled.load(std::memory_order_relaxed); }
void count() { g_launches.fetch_add(1, std::memory_order_relaxed); }
void count_graph(int kernels) { g_launches.fetch_add(kernels, std::memory_order_relaxed); }
void make_events(cudaEvent_t* a, cudaEvent_t* b)
{
    std::lock_guard<std::mutex> lk(g_mu);
    for (cudaEvent_t* e : { a, b }) {
        if (!g_free_events.empty()) {
            *e = g_free_events.back();
            g_free_events.pop_back();
        } else {
            cudaEventCreate(e);
        }
    }
}
void record(const char* name, cudaEvent_t a, cudaEvent_t b)
{
    std::lock_guard<std::mutex> lk(g_mu);
    g_pending.push_back({ name, a, b });
}
} // namespace prof

bool is_device_ptr(const void* p)
{
    cudaPointerAttributes a;
    const cudaError_t e = cudaPointerGetAttributes(&a, p);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

bool is_device_ptr_on_current(const void* p)
{
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    if (a.type == cudaMemoryTypeManaged) return true;
    if (a.type != cudaMemoryTypeDevice) return false;
    // memory of another device is rejected: a kernel on this device would
    // fault on it unless peer access happened to be enabled
    int dev = -1;
    return cudaGetDevice(&dev) == cudaSuccess && a.device == dev;
}

const double* stage_positions(ipcg_mesh* m, const double* V, DBuf<double>& buf)
{
    if (is_device_ptr(V)) return V;
    buf.reserve(3 * m->nV + 1);
    if (m->nV) IPCG_CUDA(cudaMemcpyAsync(buf.p, V, sizeof(double) * 3 * m->nV, cudaMemcpyHostToDevice, m->stream));
    return buf.p;
}

void set_last_error(const std::string& msg) { g_last_error = msg; }

void require_no_codim_vertices(const ipcg_mesh* m)
{
    // the vertex-vertex pass pairs codimensional vertices (needs two), the
    // edge-vertex pass pairs them with codimensional edges (needs one of each)
    if (m && (m->n_codim_vertices >= 2 || (m->n_codim_vertices >= 1 && m->n_codim_edges >= 1)))
        throw Error(IPCG_ERR_INVALID,
            "the mesh has " + std::to_string(m->n_codim_vertices) + " codimensional vertices (vertices in no edge) and "
                + std::to_string(m->n_codim_edges)
                + " codimensional edges: their vertex-vertex and edge-vertex candidate passes are not provided");
}

} // namespace ipcg

ipcg_mesh::~ipcg_mesh()
{
    if (ev_fork) cudaEventDestroy(ev_fork);
    if (ev_side) cudaEventDestroy(ev_side);
    if (ev_pattern) cudaEventDestroy(ev_pattern);
    if (side) cudaStreamDestroy(side);
    if (side2) cudaStreamDestroy(side2);
    if (stream) cudaStreamDestroy(stream);
}

namespace {
template <typename T> void upload(DBuf<T>& b, const T* src, size_t n, cudaStream_t s)
{
    b.reserve(n + 1);
    if (n) IPCG_CUDA(cudaMemcpyAsync(b.p, src, n * sizeof(T), cudaMemcpyDefault, s));
}
template <typename T> std::vector<T> to_host(const T* src, size_t n)
{
    std::vector<T> v(n);
    if (n) IPCG_CUDA(cudaMemcpy(v.data(), src, n * sizeof(T), cudaMemcpyDefault));
    return v;
}
} // namespace

namespace ipcg {
cudaMemPool_t device_pool()
{
    constexpr int MAXDEV = 64;
    static std::mutex mu;
    static cudaMemPool_t pools[MAXDEV] = {};
    int dev = 0;
    IPCG_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= MAXDEV) throw Error(IPCG_ERR_INVALID, "device index out of range");
    std::lock_guard<std::mutex> lk(mu);
    if (!pools[dev]) {
        cudaMemPoolProps props = {};
        props.allocType = cudaMemAllocationTypePinned;
        props.location.type = cudaMemLocationTypeDevice;
        props.location.id = dev;
        cudaMemPool_t pool;
        IPCG_CUDA(cudaMemPoolCreate(&pool, &props));
        uint64_t keep = UINT64_MAX; // keep freed memory for reuse
        IPCG_CUDA(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep));
        pools[dev] = pool;
    }
    return pools[dev];
}
} // namespace ipcg

extern "C" {

const char* ipcg_last_error(void) { return g_last_error.c_str(); }

const char* ipcg_version(void) { return "ipcg 0.1.0 (sm_103a)"; }

int ipcg_profile_enable(int on)
{
    return guarded([&] {
        std::lock_guard<std::mutex> lk(prof::g_mu);
        prof::drain();
        prof::g_stats.clear();
        prof::g_enabled.store(on != 0);
    });
}

int ipcg_launch_count(int64_t* count)
{
    return guarded([&] {
        require(count != nullptr, "NULL argument");
        *count = prof::g_launches.load();
    });
}

int ipcg_profile_report(char* buf, int64_t buflen, int64_t* needed)
{
    return guarded([&] {
        std::lock_guard<std::mutex> lk(prof::g_mu);
        prof::drain();
        std::string js = "{";
        bool first = true;
        for (auto& kv : prof::g_stats) {
            char line[256];
            snprintf(line, sizeof(line), "%s\"%s\": {\"launches\": %lld, \"ms\": %.6f}", first ? "" : ", ",
                kv.first.c_str(), kv.second.launches, kv.second.ms);
            js += line;
            first = false;
        }
        js += "}";
        if (needed) *needed = (int64_t)js.size() + 1;
        if (buf && buflen > 0) {
            const size_t n = std::min<size_t>((size_t)buflen - 1, js.size());
            memcpy(buf, js.data(), n);
            buf[n] = 0;
        }
    });
}

int ipcg_mesh_stream(const ipcg_mesh* m, void** stream)
{
    return guarded([&] {
        require(m && stream, "NULL argument");
        *stream = (void*)m->stream;
    });
}

} // extern "C"

namespace {
// One scene is the n_scenes == 1 case of a batch (vertex_offsets {0, nV}).
int mesh_create(const double* rest, int64_t nV, const int32_t* edges, int64_t nE, const int32_t* faces, int64_t nF,
    int64_t n_scenes, const int64_t* vertex_offsets, ipcg_mesh** out)
{
    return guarded([&] {
        require(out != nullptr, "out is NULL");
        require(n_scenes >= 1 && n_scenes < (1 << 30), "n_scenes must be in [1, 2^30)");
        require(nV >= 0 && nE >= 0 && nF >= 0, "negative size");
        require(nV < INT32_MAX && nE < INT32_MAX && nF < INT32_MAX, "mesh too large for int32 indices");
        require(nV == 0 || rest, "rest_positions is NULL");
        require(nE == 0 || edges, "edges is NULL");
        require(nF == 0 || faces, "faces is NULL");
        require(nF == 0 || nE > 0, "faces given without edges");
        require_device();
        // host copies of topology (for validation and faces_to_edges)
        std::vector<int32_t> hE = to_host(edges, 2 * nE), hF = to_host(faces, 3 * nF);
        for (int32_t v : hE) require(v >= 0 && v < nV, "edge vertex index out of range");
        for (int32_t v : hF) require(v >= 0 && v < nV, "face vertex index out of range");
        // scenes: consecutive vertex ranges; no edge or face spans two scenes
        std::vector<int64_t> voff(n_scenes + 1);
        std::vector<int32_t> vscene;
        if (vertex_offsets) {
            for (int64_t k = 0; k <= n_scenes; ++k) voff[k] = vertex_offsets[k];
            require(voff[0] == 0 && voff[n_scenes] == nV, "vertex_offsets must start at 0 and end at num_vertices");
            for (int64_t k = 0; k < n_scenes; ++k) require(voff[k] <= voff[k + 1], "vertex_offsets must not decrease");
        } else {
            require(n_scenes == 1, "vertex_offsets is NULL");
            voff[1] = nV;
        }
        // offsets: vertex, edge, edge, face (edges and faces are numbered scene by scene)
        std::vector<int64_t> soff(4 * (n_scenes + 1), 0);
        if (n_scenes > 1) {
            vscene.resize(nV);
            for (int64_t k = 0; k < n_scenes; ++k)
                for (int64_t v = voff[k]; v < voff[k + 1]; ++v) vscene[v] = (int32_t)k;
            std::vector<int64_t> ecount(n_scenes, 0), fcount(n_scenes, 0);
            int32_t prev = 0;
            for (int64_t e = 0; e < nE; ++e) {
                const int32_t k = vscene[hE[2 * e]];
                require(k == vscene[hE[2 * e + 1]], "an edge joins two scenes");
                require(k >= prev, "edges must be grouped by scene in scene order");
                prev = k;
                ++ecount[k];
            }
            prev = 0;
            for (int64_t f = 0; f < nF; ++f) {
                const int32_t k = vscene[hF[3 * f]];
                require(k == vscene[hF[3 * f + 1]] && k == vscene[hF[3 * f + 2]], "a face joins two scenes");
                require(k >= prev, "faces must be grouped by scene in scene order");
                prev = k;
                ++fcount[k];
            }
            const int64_t S = n_scenes + 1;
            for (int64_t k = 0; k <= n_scenes; ++k) soff[k] = voff[k];
            for (int64_t k = 0; k < n_scenes; ++k) {
                soff[S + k + 1] = soff[S + k] + ecount[k];
                soff[3 * S + k + 1] = soff[3 * S + k] + fcount[k];
            }
            for (int64_t k = 0; k <= n_scenes; ++k) soff[2 * S + k] = soff[S + k];
        }
        // faces_to_edges (collision_mesh.cpp:510-543)
        std::unordered_map<uint64_t, int32_t> emap;
        emap.reserve(2 * nE + 1);
        for (int64_t e = 0; e < nE; ++e) {
            const uint32_t a = std::min(hE[2 * e], hE[2 * e + 1]), b = std::max(hE[2 * e], hE[2 * e + 1]);
            emap.emplace(((uint64_t)a << 32) | b, (int32_t)e);
        }
        std::vector<int32_t> f2e(3 * nF);
        for (int64_t f = 0; f < nF; ++f)
            for (int j = 0; j < 3; ++j) {
                const uint32_t vi = hF[3 * f + j], vj = hF[3 * f + (j + 1) % 3];
                auto it = emap.find(((uint64_t)std::min(vi, vj) << 32) | std::max(vi, vj));
                if (it == emap.end()) throw Error(IPCG_ERR_TOPOLOGY, "Unable to find edge!");
                f2e[3 * f + j] = it->second;
            }
        // codimensional vertices (in no edge) and edges (in no face)
        int64_t n_codim_v = 0, n_codim_e = 0;
        {
            std::vector<uint8_t> used(nV, 0), in_face(nE, 0);
            for (int32_t v : hE) used[v] = 1;
            for (int32_t e : f2e) in_face[e] = 1;
            for (uint8_t u : used) n_codim_v += !u;
            for (uint8_t u : in_face) n_codim_e += !u;
        }
        static std::atomic<uint64_t> serials { 0 };
        auto* m = new ipcg_mesh();
        try {
            m->serial = ++serials;
            m->n_codim_vertices = n_codim_v;
            m->n_codim_edges = n_codim_e;
            IPCG_CUDA(cudaGetDevice(&m->device));
            IPCG_CUDA(cudaStreamCreateWithFlags(&m->stream, cudaStreamNonBlocking));
            IPCG_CUDA(cudaStreamCreateWithFlags(&m->side, cudaStreamNonBlocking));
            IPCG_CUDA(cudaStreamCreateWithFlags(&m->side2, cudaStreamNonBlocking));
            IPCG_CUDA(cudaEventCreateWithFlags(&m->ev_fork, cudaEventDisableTiming));
            IPCG_CUDA(cudaEventCreateWithFlags(&m->ev_side, cudaEventDisableTiming));
            IPCG_CUDA(cudaEventCreateWithFlags(&m->ev_pattern, cudaEventDisableTiming));
            m->nV = nV;
            m->nE = nE;
            m->nF = nF;
            upload(m->rest, rest, 3 * nV, m->stream);
            upload(m->E, (const int*)hE.data(), 2 * nE, m->stream);
            upload(m->F, (const int*)hF.data(), 3 * nF, m->stream);
            upload(m->F2E, (const int*)f2e.data(), 3 * nF, m->stream);
            {
                const std::vector<double> hR = to_host(rest, 3 * nV);
                std::vector<double> va(nV), ea(nE);
                mesh_areas_host(hR.data(), nV, hE.data(), nE, hF.data(), nF, f2e.data(), va.data(), ea.data());
                upload(m->vertex_area, va.data(), nV, m->stream);
                upload(m->edge_area, ea.data(), nE, m->stream);
                IPCG_CUDA(cudaStreamSynchronize(m->stream));
            }
            m->h_F2E = std::move(f2e);
            m->n_scenes = n_scenes;
            m->h_voff = std::move(voff);
            if (n_scenes > 1) {
                upload(m->vscene, (const int*)vscene.data(), nV, m->stream);
                upload(m->scene_offs, (const int64_t*)soff.data(), soff.size(), m->stream);
            }
            m->counters.reserve(16);
            m->h_counters.reserve(16);
            IPCG_CUDA(cudaStreamSynchronize(m->stream));
        } catch (...) {
            delete m;
            throw;
        }
        *out = m;
    });
}
} // namespace

namespace ipcg {
// The barrier calls' option bits: physical scaling, the precision modes and
// the barrier function.
void barrier_options(int bits, BarrierArgs& a)
{
    const int kind = (bits >> 4) & 15;
    require(bits >= 0
            && (bits & ~(IPCG_BARRIER_PHYSICAL | IPCG_BARRIER_FP32_PT | IPCG_BARRIER_FP32_LOCAL
                           | IPCG_BARRIER_DF64_PSD | IPCG_BARRIER_FUNCTION(15)))
                == 0
            && kind <= IPCG_BARRIER_TWO_STAGE,
        "unknown barrier option bits");
    a.physical = (bits & IPCG_BARRIER_PHYSICAL) ? 1 : 0;
    a.mixed = (bits & IPCG_BARRIER_FP32_PT) ? 1 : 0;
    a.fp32_local = (bits & IPCG_BARRIER_FP32_LOCAL) ? 1 : 0;
    a.df64_psd = (bits & IPCG_BARRIER_DF64_PSD) ? 1 : 0;
    a.kind = kind;
}
} // namespace ipcg

extern "C" {

int ipcg_mesh_create(const double* rest, int64_t nV, const int32_t* edges, int64_t nE, const int32_t* faces,
    int64_t nF, ipcg_mesh** out)
{
    return mesh_create(rest, nV, edges, nE, faces, nF, 1, nullptr, out);
}

int ipcg_mesh_create_batch(const double* rest, int64_t nV, const int32_t* edges, int64_t nE, const int32_t* faces,
    int64_t nF, int64_t n_scenes, const int64_t* vertex_offsets, ipcg_mesh** out)
{
    if (!vertex_offsets) {
        g_last_error = "vertex_offsets is NULL";
        return IPCG_ERR_INVALID;
    }
    return mesh_create(rest, nV, edges, nE, faces, nF, n_scenes, vertex_offsets, out);
}

int ipcg_set_hessian_chunk_contacts(int64_t contacts)
{
    return guarded([&] {
        require(contacts >= 0, "contacts must be non-negative");
        g_hess_chunk_contacts.store(contacts ? contacts : (int64_t(1) << 22));
    });
}

int ipcg_mesh_scenes(const ipcg_mesh* m, int64_t* n_scenes)
{
    return guarded([&] {
        require(m && n_scenes, "NULL argument");
        *n_scenes = m->n_scenes;
    });
}

int ipcg_mesh_destroy(ipcg_mesh* mesh)
{
    return guarded([&] { delete mesh; });
}

int ipcg_mesh_sizes(const ipcg_mesh* m, int64_t sizes[3])
{
    return guarded([&] {
        require(m && sizes, "NULL argument");
        sizes[0] = m->nV;
        sizes[1] = m->nE;
        sizes[2] = m->nF;
    });
}

int ipcg_mesh_codim_counts(const ipcg_mesh* m, int64_t counts[2])
{
    return guarded([&] {
        require(m && counts, "NULL argument");
        counts[0] = m->n_codim_vertices;
        counts[1] = m->n_codim_edges;
    });
}

int ipcg_mesh_faces_to_edges(const ipcg_mesh* m, int32_t* out)
{
    return guarded([&] {
        require(m && (out || m->nF == 0), "NULL argument");
        if (m->nF) IPCG_CUDA(cudaMemcpy(out, m->h_F2E.data(), sizeof(int32_t) * 3 * m->nF, cudaMemcpyDefault));
    });
}

int ipcg_collisions_create(ipcg_collisions** out)
{
    return guarded([&] {
        require(out != nullptr, "out is NULL");
        *out = new ipcg_collisions();
    });
}

int ipcg_collisions_destroy(ipcg_collisions* c)
{
    return guarded([&] { delete c; });
}

int ipcg_collisions_set_use_area_weighting(ipcg_collisions* c, int on)
{
    return guarded([&] {
        require(c != nullptr, "NULL argument");
        c->use_area_weighting = on ? 1 : 0;
    });
}

int ipcg_collisions_use_area_weighting(const ipcg_collisions* c, int* on)
{
    return guarded([&] {
        require(c && on, "NULL argument");
        *on = c->use_area_weighting;
    });
}

int ipcg_collisions_set_collision_set_type(ipcg_collisions* c, int type)
{
    return guarded([&] {
        require(c != nullptr, "NULL argument");
        require(type == IPCG_COLLISION_SET_IPC || type == IPCG_COLLISION_SET_IMPROVED_MAX_APPROX,
            "collision set type must be IPCG_COLLISION_SET_IPC or IPCG_COLLISION_SET_IMPROVED_MAX_APPROX");
        c->set_type = type;
    });
}

int ipcg_collisions_collision_set_type(const ipcg_collisions* c, int* type)
{
    return guarded([&] {
        require(c && type, "NULL argument");
        *type = c->set_type;
    });
}

int ipcg_collisions_set_enable_shape_derivatives(ipcg_collisions* c, int on)
{
    return guarded([&] {
        require(c != nullptr, "NULL argument");
        c->enable_shape_derivatives = on ? 1 : 0;
    });
}

int ipcg_collisions_enable_shape_derivatives(const ipcg_collisions* c, int* on)
{
    return guarded([&] {
        require(c && on, "NULL argument");
        *on = c->enable_shape_derivatives;
    });
}

int ipcg_mesh_areas(const ipcg_mesh* m, double* vertex_areas, double* edge_areas)
{
    return guarded([&] {
        require(m != nullptr, "NULL argument");
        if (vertex_areas && m->nV)
            IPCG_CUDA(cudaMemcpy(vertex_areas, m->vertex_area.p, sizeof(double) * m->nV, cudaMemcpyDefault));
        if (edge_areas && m->nE)
            IPCG_CUDA(cudaMemcpy(edge_areas, m->edge_area.p, sizeof(double) * m->nE, cudaMemcpyDefault));
    });
}

int ipcg_collisions_build(ipcg_collisions* c, const ipcg_mesh* mesh, const double* V, double dhat, double dmin)
{
    if (mesh && mesh->n_scenes != 1) {
        g_last_error = "mesh is a batch: use ipcg_collisions_build_batch";
        return IPCG_ERR_INVALID;
    }
    return ipcg_collisions_build_batch(c, mesh, V, &dhat, &dmin);
}

int ipcg_collisions_build_batch(ipcg_collisions* c, const ipcg_mesh* mesh, const double* V, const double* dhat,
    const double* dmin)
{
    return guarded([&] {
        require(c && mesh && dhat && dmin && (V || mesh->nV == 0), "NULL argument");
        for (int64_t k = 0; k < mesh->n_scenes; ++k) {
            require(dhat[k] > 0, "dhat must be positive");
            require(dmin[k] >= 0, "dmin must be non-negative");
        }
        require_no_codim_vertices(mesh);
        ipcg_mesh* m = const_cast<ipcg_mesh*>(mesh);
        IPCG_CUDA(cudaSetDevice(m->device));
        const double* dV = stage_positions(m, V, m->V0);
        build_collision_set(c, m, dV, dhat, dmin);
    });
}

int ipcg_collisions_counts(const ipcg_collisions* c, int64_t counts[6])
{
    return guarded([&] {
        require(c && counts, "NULL argument");
        counts[0] = c->nvv;
        counts[1] = c->nev;
        counts[2] = c->nee;
        counts[3] = c->nfv;
        counts[4] = c->n_cand_ee;
        counts[5] = c->n_cand_fv;
    });
}

int ipcg_collisions_get(const ipcg_collisions* c, int32_t* vv, double* vv_w, int32_t* ev, double* ev_w, int32_t* ee,
    double* ee_eps, int8_t* ee_dtype, double* ee_w, int32_t* fv, double* fv_w)
{
    return guarded([&] {
        require(c != nullptr, "NULL argument");
        cudaStream_t s = 0;
        copy_out(vv, c->vv.p, sizeof(int2) * c->nvv, s);
        copy_out(vv_w, c->vv_w.p, sizeof(double) * c->nvv, s);
        copy_out(ev, c->ev.p, sizeof(int2) * c->nev, s);
        copy_out(ev_w, c->ev_w.p, sizeof(double) * c->nev, s);
        copy_out(ee, c->ee.p, sizeof(int2) * c->nee, s);
        copy_out(ee_eps, c->ee_eps.p, sizeof(double) * c->nee, s);
        copy_out(ee_dtype, c->ee_dtype.p, sizeof(int8_t) * c->nee, s);
        copy_out(ee_w, c->ee_w.p, sizeof(double) * c->nee, s);
        copy_out(fv, c->fv.p, sizeof(int2) * c->nfv, s);
        copy_out(fv_w, c->fv_w.p, sizeof(double) * c->nfv, s);
        IPCG_CUDA(cudaStreamSynchronize(s));
    });
}

int ipcg_collisions_set(ipcg_collisions* c, double dmin, int64_t nvv, const int32_t* vv, const double* vv_w,
    int64_t nev, const int32_t* ev, const double* ev_w, int64_t nee, const int32_t* ee, const double* ee_eps,
    const int8_t* ee_dtype, const double* ee_w, int64_t nfv, const int32_t* fv, const double* fv_w)
{
    return guarded([&] {
        require(c != nullptr, "NULL argument");
        require(nvv >= 0 && nev >= 0 && nee >= 0 && nfv >= 0, "negative count");
        require_device();
        for (int64_t i = 0; i < nee; ++i) {
            if (ee_dtype && !is_device_ptr(ee_dtype)) require(ee_dtype[i] >= 0 && ee_dtype[i] <= 8, "bad EE dtype");
        }
        cudaStream_t s = 0;
        upload(c->vv, (const int2*)vv, nvv, s);
        upload(c->vv_w, vv_w, nvv, s);
        upload(c->ev, (const int2*)ev, nev, s);
        upload(c->ev_w, ev_w, nev, s);
        upload(c->ee, (const int2*)ee, nee, s);
        upload(c->ee_eps, ee_eps, nee, s);
        upload(c->ee_dtype, ee_dtype, nee, s);
        upload(c->ee_w, ee_w, nee, s);
        upload(c->fv, (const int2*)fv, nfv, s);
        upload(c->fv_w, fv_w, nfv, s);
        IPCG_CUDA(cudaStreamSynchronize(s));
        ++c->version;
        c->nvv = nvv;
        c->nev = nev;
        c->nee = nee;
        c->nfv = nfv;
        c->dmin = dmin;
        c->scene_dmin.clear();
        c->sorted = false;
        c->n_cand_ee = c->n_cand_fv = 0;
    });
}


// dhat / stiffness: one value (scene_params == 0) or one per scene (host arrays).
static int barrier_call(const ipcg_collisions* c, const ipcg_mesh* mesh, const double* V, const double* dhat,
    const double* stiffness, int scene_params, int physical, int psd, double* energy, double* gradient,
    ipcg_csr** hessian)
{
    return guarded([&] {
        require(c && mesh && dhat && stiffness && (V || mesh->nV == 0), "NULL argument");
        require(scene_params || mesh->n_scenes == 1, "mesh is a batch: use ipcg_barrier_batch");
        for (int64_t k = 0; k < (scene_params ? mesh->n_scenes : 1); ++k) require(dhat[k] > 0, "dhat must be positive");
        require(psd >= IPCG_PSD_NONE && psd <= IPCG_PSD_ABS, "Invalid type of PSD projection!");
        ipcg_mesh* m = const_cast<ipcg_mesh*>(mesh);
        IPCG_CUDA(cudaSetDevice(m->device));
        const double* dV = stage_positions(m, V, m->V0);
        BarrierArgs a { dhat[0], stiffness[0], c->dmin, 0, psd };
        barrier_options(physical, a);
        if (scene_params) {
            a.scene_dhat = dhat;
            a.scene_kappa = stiffness;
        }
        double* gdev = nullptr;
        if (gradient) {
            if (is_device_ptr(gradient)) gdev = gradient;
            else {
                // a host gradient is computed in the mesh's staging buffer
                m->grad_stage.reserve(3 * m->nV + 1);
                gdev = m->grad_stage.p;
            }
        }
        ipcg_csr* H = nullptr;
        if (hessian) H = new ipcg_csr();
        try {
            if (!(H && barrier_egh(c, m, dV, a, energy, gdev, H))) barrier_evaluate(c, m, dV, a, energy, gdev, H);
            if (gradient && gdev != gradient) {
                IPCG_CUDA(cudaMemcpyAsync(gradient, gdev, sizeof(double) * 3 * m->nV, cudaMemcpyDeviceToHost,
                    m->stream));
                IPCG_CUDA(cudaStreamSynchronize(m->stream));
            }
        } catch (...) {
            delete H;
            throw;
        }
        if (hessian) *hessian = H;
    });
}

int ipcg_barrier_energy(const ipcg_collisions* c, const ipcg_mesh* mesh, const double* V, double dhat,
    double stiffness, int physical, double* energy)
{
    if (!energy) {
        g_last_error = "energy is NULL";
        return IPCG_ERR_INVALID;
    }
    return barrier_call(c, mesh, V, &dhat, &stiffness, 0, physical, IPCG_PSD_NONE, energy, nullptr, nullptr);
}

int ipcg_barrier_gradient(const ipcg_collisions* c, const ipcg_mesh* mesh, const double* V, double dhat,
    double stiffness, int physical, double* gradient)
{
    if (!gradient) {
        g_last_error = "gradient is NULL";
        return IPCG_ERR_INVALID;
    }
    return barrier_call(c, mesh, V, &dhat, &stiffness, 0, physical, IPCG_PSD_NONE, nullptr, gradient, nullptr);
}

int ipcg_barrier_hessian(const ipcg_collisions* c, const ipcg_mesh* mesh, const double* V, double dhat,
    double stiffness, int physical, int psd, ipcg_csr** out)
{
    if (!out) {
        g_last_error = "out is NULL";
        return IPCG_ERR_INVALID;
    }
    return barrier_call(c, mesh, V, &dhat, &stiffness, 0, physical, psd, nullptr, nullptr, out);
}

int ipcg_barrier_energy_gradient_hessian(const ipcg_collisions* c, const ipcg_mesh* mesh, const double* V,
    double dhat, double stiffness, int physical, int psd, double* energy, double* gradient, ipcg_csr** hessian)
{
    return barrier_call(c, mesh, V, &dhat, &stiffness, 0, physical, psd, energy, gradient, hessian);
}

int ipcg_barrier_batch(const ipcg_collisions* c, const ipcg_mesh* mesh, const double* V, const double* dhat,
    const double* stiffness, int physical, int psd, double* energies, double* gradient, ipcg_csr** hessian)
{
    return barrier_call(c, mesh, V, dhat, stiffness, 1, physical, psd, energies, gradient, hessian);
}

int ipcg_barrier_autotune(const ipcg_collisions* c, const ipcg_mesh* mesh, const double* V, const double* dhat,
    const double* stiffness, int physical, int psd, char* report, int64_t report_len, int64_t* needed)
{
    return guarded([&] {
        require(c && mesh && dhat && stiffness && (V || mesh->nV == 0), "NULL argument");
        for (int64_t k = 0; k < mesh->n_scenes; ++k) require(dhat[k] > 0, "dhat must be positive");
        require(psd >= IPCG_PSD_NONE && psd <= IPCG_PSD_ABS, "Invalid type of PSD projection!");
        ipcg_mesh* m = const_cast<ipcg_mesh*>(mesh);
        IPCG_CUDA(cudaSetDevice(m->device));
        const double* dV = stage_positions(m, V, m->V0);
        BarrierArgs a { dhat[0], stiffness[0], c->dmin, 0, psd };
        barrier_options(physical, a);
        a.scene_dhat = dhat;
        a.scene_kappa = stiffness;
        const std::string rep = egh_autotune(c, m, dV, a);
        if (needed) *needed = (int64_t)rep.size() + 1;
        if (report && report_len > 0) {
            const size_t k = std::min<size_t>(rep.size(), (size_t)report_len - 1);
            memcpy(report, rep.data(), k);
            report[k] = 0;
        }
    });
}

int ipcg_barrier_tuning(int stage, int* threads, int* blocks_per_sm, int* tiles_per_grab)
{
    return guarded([&] {
        require(stage == IPCG_STAGE_LOCAL || stage == IPCG_STAGE_PSD || stage == IPCG_STAGE_PSD_DF64, "unknown stage");
        require_device();
        const EghTuning t = egh_tuning(stage);
        if (threads) *threads = t.threads;
        if (blocks_per_sm) *blocks_per_sm = t.blocks_per_sm;
        if (tiles_per_grab) *tiles_per_grab = t.tiles_per_grab;
    });
}

int ipcg_barrier_set_tuning(int stage, int threads, int blocks_per_sm, int tiles_per_grab)
{
    return guarded([&] {
        require(stage == IPCG_STAGE_LOCAL || stage == IPCG_STAGE_PSD || stage == IPCG_STAGE_PSD_DF64, "unknown stage");
        require_device();
        egh_set_tuning(stage, EghTuning { threads, blocks_per_sm, tiles_per_grab });
    });
}

int ipcg_testing_ccd_stats(const ipcg_mesh* mesh, int enable, int64_t* out)
{
    return guarded([&] {
        require(mesh, "NULL argument");
        ipcg_mesh* m = const_cast<ipcg_mesh*>(mesh);
        IPCG_CUDA(cudaSetDevice(m->device));
        if (out) {
            for (int k = 0; k < 12; ++k) out[k] = 0;
            if (m->ccd_stats_live) {
                IPCG_CUDA(cudaMemcpyAsync(out, m->ccd_stats.p, sizeof(int64_t) * 12, cudaMemcpyDeviceToHost,
                    m->stream));
                IPCG_CUDA(cudaStreamSynchronize(m->stream));
            }
        }
        m->ccd_stats_live = false;
        g_ccd_stats.store(enable ? 1 : 0);
    });
}

int ipcg_fp64_fma_rate(double* tflops)
{
    return guarded([&] {
        require(tflops, "NULL argument");
        require_device();
        *tflops = fp64_fma_rate();
    });
}

int ipcg_testing_ccd_budget(int64_t boxes)
{
    return guarded([&] {
        require(boxes >= 0, "the budget is a box count (0: the default)");
        g_ccd_thread_budget.store(boxes);
    });
}

int ipcg_testing_defer_df64_psd(int on)
{
    return guarded([&] { egh_defer_df64(on != 0); });
}

// Gauss-Newton forms (normal_potential.cpp:15-83): the FP64 path serves
// every option; the FP32 bit does not apply to them.
static int gauss_newton_call(const ipcg_collisions* c, const ipcg_mesh* mesh, const double* V, double dhat,
    double stiffness, int physical, double* diag, const double* p, double* qf)
{
    return guarded([&] {
        require(c && mesh && (V || mesh->nV == 0), "NULL argument");
        require(diag || (p && qf) || mesh->nV == 0, "NULL argument");
        require(dhat > 0, "dhat must be positive");
        ipcg_mesh* m = const_cast<ipcg_mesh*>(mesh);
        IPCG_CUDA(cudaSetDevice(m->device));
        const double* dV = stage_positions(m, V, m->V0);
        BarrierArgs a { dhat, stiffness, c->dmin, 0, IPCG_PSD_NONE };
        barrier_options(physical, a);
        const size_t bytes = sizeof(double) * 3 * m->nV;
        if (diag) {
            double* ddev = diag;
            if (!is_device_ptr(diag)) {
                m->grad_stage.reserve(3 * m->nV + 1);
                ddev = m->grad_stage.p;
            }
            barrier_gauss_newton(c, m, dV, a, ddev, nullptr, nullptr);
            if (ddev != diag) IPCG_CUDA(cudaMemcpyAsync(diag, ddev, bytes, cudaMemcpyDeviceToHost, m->stream));
            IPCG_CUDA(cudaStreamSynchronize(m->stream));
        } else {
            // a host p is staged in the mesh's second position buffer
            const double* pdev = stage_positions(m, p, m->V1);
            barrier_gauss_newton(c, m, dV, a, nullptr, pdev, qf);
        }
    });
}

int ipcg_barrier_gauss_newton_hessian_diagonal(const ipcg_collisions* c, const ipcg_mesh* mesh, const double* V,
    double dhat, double stiffness, int physical, double* diagonal)
{
    if (!diagonal) {
        g_last_error = "diagonal is NULL";
        return IPCG_ERR_INVALID;
    }
    return gauss_newton_call(c, mesh, V, dhat, stiffness, physical, diagonal, nullptr, nullptr);
}

int ipcg_barrier_gauss_newton_hessian_quadratic_form(const ipcg_collisions* c, const ipcg_mesh* mesh,
    const double* V, double dhat, double stiffness, int physical, const double* p, double* out)
{
    if (!p || !out) {
        g_last_error = "p or out is NULL";
        return IPCG_ERR_INVALID;
    }
    return gauss_newton_call(c, mesh, V, dhat, stiffness, physical, nullptr, p, out);
}

int ipcg_tangential_create(ipcg_tangential** out)
{
    return guarded([&] {
        require(out != nullptr, "out is NULL");
        *out = new ipcg_tangential();
    });
}

int ipcg_tangential_destroy(ipcg_tangential* t)
{
    return guarded([&] { delete t; });
}

// dhat / stiffness: one value, or one per scene (scene_params) for batches
static int tangential_build_call(ipcg_tangential* t, const ipcg_mesh* mesh, const double* V, const ipcg_collisions* c,
    const double* dhat, const double* stiffness, int scene_params, int physical, const double* mu_s,
    const double* mu_k)
{
    return guarded([&] {
        require(t && mesh && c && dhat && stiffness && mu_s && mu_k && (V || mesh->nV == 0), "NULL argument");
        require(scene_params || mesh->n_scenes == 1, "mesh is a batch: use ipcg_tangential_build_batch");
        for (int64_t k = 0; k < (scene_params ? mesh->n_scenes : 1); ++k) require(dhat[k] > 0, "dhat must be positive");
        ipcg_mesh* m = const_cast<ipcg_mesh*>(mesh);
        IPCG_CUDA(cudaSetDevice(m->device));
        const double* dV = stage_positions(m, V, m->V0);
        BarrierArgs a { dhat[0], stiffness[0], c->dmin, 0, IPCG_PSD_NONE };
        barrier_options(physical, a);
        if (scene_params) {
            a.scene_dhat = dhat;
            a.scene_kappa = stiffness;
        }
        DBuf<double> ms, mk;
        upload(ms, mu_s, m->nV, m->stream);
        upload(mk, mu_k, m->nV, m->stream);
        tangential_build(c, m, dV, a, ms.p, mk.p, t);
        t->mesh = mesh;
    });
}

int ipcg_tangential_build(ipcg_tangential* t, const ipcg_mesh* mesh, const double* V, const ipcg_collisions* c,
    double dhat, double stiffness, int physical, const double* mu_s, const double* mu_k)
{
    return tangential_build_call(t, mesh, V, c, &dhat, &stiffness, 0, physical, mu_s, mu_k);
}

int ipcg_tangential_build_batch(ipcg_tangential* t, const ipcg_mesh* mesh, const double* V, const ipcg_collisions* c,
    const double* dhat, const double* stiffness, int physical, const double* mu_s, const double* mu_k)
{
    return tangential_build_call(t, mesh, V, c, dhat, stiffness, 1, physical, mu_s, mu_k);
}

int ipcg_tangential_counts(const ipcg_tangential* t, int64_t counts[4])
{
    return guarded([&] {
        require(t && counts, "NULL argument");
        counts[0] = t->st.nvv;
        counts[1] = t->st.nev;
        counts[2] = t->st.nee;
        counts[3] = t->st.nfv;
    });
}

int ipcg_tangential_get(const ipcg_tangential* t, int32_t* vv, int32_t* ev, int32_t* ee, int32_t* fv,
    double* weight, double* normal_force, double* closest_point, double* tangent_basis, double* mu_s, double* mu_k)
{
    return guarded([&] {
        require(t != nullptr, "NULL argument");
        const ipcg_collisions& st = t->st;
        const int64_t n = st.size();
        cudaStream_t s = 0;
        copy_out(vv, st.vv.p, sizeof(int2) * st.nvv, s);
        copy_out(ev, st.ev.p, sizeof(int2) * st.nev, s);
        copy_out(ee, st.ee.p, sizeof(int2) * st.nee, s);
        copy_out(fv, st.fv.p, sizeof(int2) * st.nfv, s);
        if (weight) {
            copy_out(weight, st.vv_w.p, sizeof(double) * st.nvv, s);
            copy_out(weight + st.nvv, st.ev_w.p, sizeof(double) * st.nev, s);
            copy_out(weight + st.nvv + st.nev, st.ee_w.p, sizeof(double) * st.nee, s);
            copy_out(weight + st.nvv + st.nev + st.nee, st.fv_w.p, sizeof(double) * st.nfv, s);
        }
        copy_out(normal_force, t->N.p, sizeof(double) * n, s);
        copy_out(closest_point, t->cp.p, sizeof(double) * 2 * n, s);
        copy_out(tangent_basis, t->P.p, sizeof(double) * 6 * n, s);
        copy_out(mu_s, t->mu_s.p, sizeof(double) * n, s);
        copy_out(mu_k, t->mu_k.p, sizeof(double) * n, s);
        IPCG_CUDA(cudaStreamSynchronize(s));
    });
}

int ipcg_tangential_set_anisotropy(ipcg_tangential* t, const double* mu_aniso, const double* mu_s_aniso,
    const double* mu_k_aniso)
{
    return guarded([&] {
        require(t && t->mesh, "tangential collisions are not built");
        ipcg_mesh* m = const_cast<ipcg_mesh*>(t->mesh);
        IPCG_CUDA(cudaSetDevice(m->device));
        const int64_t n = t->st.size();
        cudaStream_t s = m->stream;
        auto set = [&](DBuf<double>& dst, const double* src, double fill) {
            if (!n) return;
            if (src) IPCG_CUDA(cudaMemcpyAsync(dst.p, src, sizeof(double) * 2 * n, cudaMemcpyDefault, s));
            else if (fill == 0) IPCG_CUDA(cudaMemsetAsync(dst.p, 0, sizeof(double) * 2 * n, s));
            else {
                std::vector<double> ones(2 * n, fill);
                IPCG_CUDA(cudaMemcpyAsync(dst.p, ones.data(), sizeof(double) * 2 * n, cudaMemcpyHostToDevice, s));
                IPCG_CUDA(cudaStreamSynchronize(s));
            }
        };
        set(t->mu_aniso, mu_aniso, 1.0);
        set(t->mu_s_aniso, mu_s_aniso, 0.0);
        set(t->mu_k_aniso, mu_k_aniso, 0.0);
        IPCG_CUDA(cudaStreamSynchronize(s));
    });
}

int ipcg_tangential_update_lagged_mu(ipcg_tangential* t, const ipcg_mesh* mesh, const double* rest,
    const double* lagged_displacements, const double* velocities)
{
    return guarded([&] {
        require(t && mesh && (mesh->nV == 0 || (rest && lagged_displacements && velocities)), "NULL argument");
        require(t->mesh == mesh, "tangential collisions were built on another mesh");
        ipcg_mesh* m = const_cast<ipcg_mesh*>(mesh);
        IPCG_CUDA(cudaSetDevice(m->device));
        DBuf<double> lag;
        const double* dR = stage_positions(m, rest, m->V0);
        const double* dL = stage_positions(m, lagged_displacements, m->V1);
        const double* dU = stage_positions(m, velocities, lag);
        tangential_update_lagged(t, m, dR, dL, dU);
    });
}

int ipcg_tangential_reset_lagged_mu(ipcg_tangential* t)
{
    return guarded([&] {
        require(t && t->mesh, "tangential collisions are not built");
        ipcg_mesh* m = const_cast<ipcg_mesh*>(t->mesh);
        const int64_t n = t->st.size();
        if (n) {
            IPCG_CUDA(cudaMemcpyAsync(t->mu_s_eff.p, t->mu_s.p, sizeof(double) * n, cudaMemcpyDeviceToDevice, m->stream));
            IPCG_CUDA(cudaMemcpyAsync(t->mu_k_eff.p, t->mu_k.p, sizeof(double) * n, cudaMemcpyDeviceToDevice, m->stream));
        }
        IPCG_CUDA(cudaStreamSynchronize(m->stream));
    });
}

int ipcg_tangential_lagged_mu(const ipcg_tangential* t, double* mu_s_eff, double* mu_k_eff)
{
    return guarded([&] {
        require(t != nullptr, "NULL argument");
        const int64_t n = t->st.size();
        cudaStream_t s = 0;
        copy_out(mu_s_eff, t->mu_s_eff.p, sizeof(double) * n, s);
        copy_out(mu_k_eff, t->mu_k_eff.p, sizeof(double) * n, s);
        IPCG_CUDA(cudaStreamSynchronize(s));
    });
}

int ipcg_friction_force(const ipcg_tangential* t, const ipcg_mesh* mesh, const double* rest,
    const double* lagged_displacements, const double* velocities, double dhat, double stiffness, int physical,
    double dmin, double eps_v, int no_mu, double* force)
{
    return guarded([&] {
        require(t && mesh && force && (mesh->nV == 0 || (rest && lagged_displacements && velocities)),
            "NULL argument");
        require(t->mesh == mesh, "tangential collisions were built on another mesh");
        require(mesh->n_scenes == 1, "the friction force takes one normal potential: single-scene meshes");
        require(dhat > 0 && eps_v > 0, "dhat and eps_v must be positive");
        ipcg_mesh* m = const_cast<ipcg_mesh*>(mesh);
        IPCG_CUDA(cudaSetDevice(m->device));
        DBuf<double> vbuf;
        const double* dR = stage_positions(m, rest, m->V0);
        const double* dL = stage_positions(m, lagged_displacements, m->V1);
        const double* dU = stage_positions(m, velocities, vbuf);
        BarrierArgs a { dhat, stiffness, dmin, 0, IPCG_PSD_NONE };
        barrier_options(physical, a);
        double* fdev = force;
        if (!is_device_ptr(force)) {
            m->grad_stage.reserve(3 * m->nV + 1);
            fdev = m->grad_stage.p;
        }
        friction_force(t, m, dR, dL, dU, a, eps_v, no_mu ? 1 : 0, fdev);
        if (fdev != force)
            IPCG_CUDA(cudaMemcpyAsync(force, fdev, sizeof(double) * 3 * m->nV, cudaMemcpyDeviceToHost, m->stream));
        IPCG_CUDA(cudaStreamSynchronize(m->stream));
    });
}

// batch: the energy output holds one value per scene
static int friction_call(const ipcg_tangential* t, const ipcg_mesh* mesh, const double* U, double eps_v, int psd,
    double* energy, double* gradient, ipcg_csr** hessian, int batch)
{
    return guarded([&] {
        require(t && mesh && (U || mesh->nV == 0), "NULL argument");
        require(batch || mesh->n_scenes == 1, "mesh is a batch: use ipcg_friction_potential_batch");
        require(t->mesh == mesh, "tangential collisions were built on another mesh");
        require(eps_v > 0, "eps_v must be positive");
        require(psd >= IPCG_PSD_NONE && psd <= IPCG_PSD_ABS, "Invalid type of PSD projection!");
        ipcg_mesh* m = const_cast<ipcg_mesh*>(mesh);
        IPCG_CUDA(cudaSetDevice(m->device));
        const double* dU = stage_positions(m, U, m->V0);
        const FrictionView f { t->N.p, t->cp.p, t->P.p, t->mu_s_eff.p, t->mu_k_eff.p, t->mu_aniso.p, eps_v };
        double* gdev = nullptr;
        if (gradient) {
            if (is_device_ptr(gradient)) gdev = gradient;
            else {
                // a host gradient is computed in the mesh's staging buffer
                m->grad_stage.reserve(3 * m->nV + 1);
                gdev = m->grad_stage.p;
            }
        }
        ipcg_csr* H = hessian ? new ipcg_csr() : nullptr;
        try {
            barrier_evaluate_friction(&t->st, m, dU, f, psd, energy, gdev, H);
            if (gradient && gdev != gradient) {
                IPCG_CUDA(cudaMemcpyAsync(gradient, gdev, sizeof(double) * 3 * m->nV, cudaMemcpyDeviceToHost,
                    m->stream));
                IPCG_CUDA(cudaStreamSynchronize(m->stream));
            }
        } catch (...) {
            delete H;
            throw;
        }
        if (hessian) *hessian = H;
    });
}

int ipcg_friction_potential(const ipcg_tangential* t, const ipcg_mesh* mesh, const double* U, double eps_v, int psd,
    double* energy, double* gradient, ipcg_csr** hessian)
{
    return friction_call(t, mesh, U, eps_v, psd, energy, gradient, hessian, 0);
}

int ipcg_friction_potential_batch(const ipcg_tangential* t, const ipcg_mesh* mesh, const double* U, double eps_v,
    int psd, double* energies, double* gradient, ipcg_csr** hessian)
{
    return friction_call(t, mesh, U, eps_v, psd, energies, gradient, hessian, 1);
}

int ipcg_barrier_shape_derivative(const ipcg_collisions* c, const ipcg_mesh* mesh, const double* V, double dhat,
    double stiffness, int physical, ipcg_csr** out)
{
    return guarded([&] {
        require(c && mesh && out && (V || mesh->nV == 0), "NULL argument");
        require(mesh->n_scenes == 1, "mesh is a batch: shape derivatives are per scene");
        require(c->built_with_shape, "Shape derivative is not computed for collisions!");
        require(!(c->built_with_area && c->set_type != IPCG_COLLISION_SET_IPC),
            "shape derivatives of area-weighted IMPROVED_MAX_APPROX sets are not provided");
        require(dhat > 0, "dhat must be positive");
        ipcg_mesh* m = const_cast<ipcg_mesh*>(mesh);
        IPCG_CUDA(cudaSetDevice(m->device));
        const double* dV = stage_positions(m, V, m->V0);
        BarrierArgs a { dhat, stiffness, c->dmin, 0, IPCG_PSD_NONE };
        barrier_options(physical, a);
        a.mixed = 0;
        a.shape = 1;
        ipcg_csr* H = new ipcg_csr();
        try {
            if (c->built_with_area) shape_derivative_area(c, m, dV, a, H);
            else barrier_evaluate(c, m, dV, a, nullptr, nullptr, H);
        } catch (...) {
            delete H;
            throw;
        }
        *out = H;
    });
}

int ipcg_csr_shape(const ipcg_csr* h, int64_t* rows, int64_t* nnz)
{
    return guarded([&] {
        require(h != nullptr, "NULL argument");
        if (rows) *rows = h->rows;
        if (nnz) *nnz = h->nnz;
    });
}

namespace {
__global__ void k_row_ptr_i32(const int64_t* __restrict__ in, int64_t n, int32_t* __restrict__ out)
{
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = (int32_t)in[i];
}
} // namespace

int ipcg_csr_get_int32(const ipcg_csr* h, int32_t* row_ptr, int32_t* col, double* val)
{
    return guarded([&] {
        require(h != nullptr, "NULL argument");
        require(h->nnz < INT32_MAX, "matrix too large for 32-bit row pointers: use ipcg_csr_get");
        cudaStream_t s = 0;
        if (row_ptr) {
            PBuf<int32_t> tmp; // stream-ordered pool memory, freed after the copy
            tmp.reserve(h->rows + 1, s);
            k_row_ptr_i32<<<(int)((h->rows + 1 + 255) / 256), 256, 0, s>>>(h->rowp(), h->rows + 1, tmp.p);
            IPCG_CUDA(cudaGetLastError());
            copy_out(row_ptr, tmp.p, sizeof(int32_t) * (h->rows + 1), s);
            IPCG_CUDA(cudaStreamSynchronize(s));
        }
        copy_out(col, h->colp(), sizeof(int32_t) * h->nnz, s);
        copy_out(val, h->val.p, sizeof(double) * h->nnz, s);
        IPCG_CUDA(cudaStreamSynchronize(s));
    });
}

int ipcg_csr_get(const ipcg_csr* h, int64_t* row_ptr, int32_t* col, double* val)
{
    return guarded([&] {
        require(h != nullptr, "NULL argument");
        cudaStream_t s = 0;
        copy_out(row_ptr, h->rowp(), sizeof(int64_t) * (h->rows + 1), s);
        copy_out(col, h->colp(), sizeof(int32_t) * h->nnz, s);
        copy_out(val, h->val.p, sizeof(double) * h->nnz, s);
        IPCG_CUDA(cudaStreamSynchronize(s));
    });
}

int ipcg_csr_destroy(ipcg_csr* h)
{
    return guarded([&] { delete h; });
}

int ipcg_collision_free_stepsize(const ipcg_mesh* mesh, const double* V0, const double* V1, double min_distance,
    double tolerance, int64_t max_iterations, double rescale, double* step, int64_t* n_candidates)
{
    if (mesh && mesh->n_scenes != 1) {
        g_last_error = "mesh is a batch: use ipcg_collision_free_stepsize_batch";
        return IPCG_ERR_INVALID;
    }
    return ipcg_collision_free_stepsize_batch(mesh, V0, V1, &min_distance, tolerance, max_iterations, rescale, step,
        n_candidates);
}

int ipcg_collision_free_stepsize_batch(const ipcg_mesh* mesh, const double* V0, const double* V1,
    const double* min_distance, double tolerance, int64_t max_iterations, double rescale, double* steps,
    int64_t* n_candidates)
{
    return guarded([&] {
        require(mesh && steps && min_distance && ((V0 && V1) || mesh->nV == 0), "NULL argument");
        for (int64_t k = 0; k < mesh->n_scenes; ++k)
            require(min_distance[k] >= 0, "min_distance must be non-negative");
        require(tolerance > 0, "tolerance must be positive");
        require(rescale > 0 && rescale <= 1, "conservative_rescaling must be in (0, 1]");
        require_no_codim_vertices(mesh);
        ipcg_mesh* m = const_cast<ipcg_mesh*>(mesh);
        IPCG_CUDA(cudaSetDevice(m->device));
        const double* d0 = stage_positions(m, V0, m->V0);
        const double* d1 = stage_positions(m, V1, m->V1);
        collision_free_stepsize(m, d0, d1, min_distance, tolerance, max_iterations, rescale, steps, n_candidates);
    });
}

int ipcg_collisions_minimum_distance(const ipcg_collisions* c, const ipcg_mesh* mesh, const double* V, double* out)
{
    return guarded([&] {
        require(c && mesh && out && (V || mesh->nV == 0), "NULL argument");
        ipcg_mesh* m = const_cast<ipcg_mesh*>(mesh);
        IPCG_CUDA(cudaSetDevice(m->device));
        const double* dV = stage_positions(m, V, m->V0);
        *out = collisions_min_distance(c, m, dV);
    });
}

int ipcg_initial_barrier_stiffness(double bbox_diagonal, int kind, double dhat, double average_mass,
    const double* grad_energy, const double* grad_barrier, int64_t n, double min_scale, double dmin, double* kappa,
    double* max_kappa)
{
    return guarded([&] {
        require(kappa && max_kappa && (n == 0 || (grad_energy && grad_barrier)), "NULL argument");
        require(n >= 0, "negative size");
        require(average_mass > 0 && min_scale > 0, "average_mass and min_barrier_stiffness_scale must be positive");
        require(bbox_diagonal > 0, "bbox_diagonal must be positive");
        require(dhat > 0 && dmin >= 0, "dhat must be positive and dmin non-negative");
        require(kind >= IPCG_BARRIER_CLAMPED_LOG && kind <= IPCG_BARRIER_TWO_STAGE, "unknown barrier kind");
        const double dhat2 = dhat * dhat, dmin2 = dmin * dmin;
        double d0 = 1e-8 * bbox_diagonal + dmin;
        d0 *= d0;
        if (d0 - dmin2 >= 2 * dmin * dhat + dhat2) d0 = dmin * dhat + 0.5 * dhat2;
        double kmin = 4 * d0 * barrier_derivative_host(kind, 2, d0 - dmin2, 2 * dmin * dhat + dhat2);
        kmin = min_scale * average_mass / kmin;
        require(std::isfinite(kmin), "minimum barrier stiffness is not finite");
        const double kmax = 100 * kmin;
        double ab = 0, bb = 0;
        if (n > 0) {
            const bool de = is_device_ptr(grad_energy), db = is_device_ptr(grad_barrier);
            require(de == db, "grad_energy and grad_barrier must both be host or both be device memory");
            if (de) {
                dot_pair_device(grad_energy, grad_barrier, n, &ab, &bb);
            } else {
                for (int64_t i = 0; i < n; ++i) {
                    ab += grad_barrier[i] * grad_energy[i];
                    bb += grad_barrier[i] * grad_barrier[i];
                }
            }
        }
        double k = 1.0;
        if (bb > 0) k = -ab / bb;
        *kappa = std::min(std::max(k, kmin), kmax);
        *max_kappa = kmax;
    });
}

int ipcg_update_barrier_stiffness(double prev_min_distance, double min_distance, double max_kappa, double kappa,
    double bbox_diagonal, double dhat_epsilon_scale, double dmin, double* out)
{
    return guarded([&] {
        require(out != nullptr, "NULL argument");
        double eps = dhat_epsilon_scale * (bbox_diagonal + dmin);
        eps *= eps;
        *out = (prev_min_distance < eps && min_distance < eps && min_distance < prev_min_distance)
            ? std::min(max_kappa, 2 * kappa)
            : kappa;
    });
}

int ipcg_is_step_collision_free(const ipcg_mesh* mesh, const double* V0, const double* V1, double min_distance,
    double tolerance, int64_t max_iterations, double rescale, int* out)
{
    return guarded([&] {
        require(mesh && out && ((V0 && V1) || mesh->nV == 0), "NULL argument");
        require(min_distance >= 0, "min_distance must be non-negative");
        require(tolerance > 0, "tolerance must be positive");
        require(rescale > 0 && rescale <= 1, "conservative_rescaling must be in (0, 1]");
        require_no_codim_vertices(mesh);
        ipcg_mesh* m = const_cast<ipcg_mesh*>(mesh);
        IPCG_CUDA(cudaSetDevice(m->device));
        const double* d0 = stage_positions(m, V0, m->V0);
        const double* d1 = stage_positions(m, V1, m->V1);
        *out = step_collision_free(m, d0, d1, min_distance, tolerance, max_iterations, rescale) ? 1 : 0;
    });
}

int ipcg_has_intersections(const ipcg_mesh* mesh, const double* V, int* out)
{
    return guarded([&] {
        require(mesh && out && (V || mesh->nV == 0), "NULL argument");
        ipcg_mesh* m = const_cast<ipcg_mesh*>(mesh);
        IPCG_CUDA(cudaSetDevice(m->device));
        const double* dV = stage_positions(m, V, m->V0);
        *out = has_intersections(m, dV) ? 1 : 0;
    });
}

int ipcg_ccd_stencils(int is_ee, int64_t n, const double* x0, const double* x1, double min_distance, double tmax,
    double tolerance, int64_t max_iterations, double rescale, int8_t* hit, double* toi)
{
    return guarded([&] {
        require(n >= 0 && n < INT32_MAX, "bad n");
        require(n == 0 || (x0 && x1 && hit && toi), "NULL argument");
        require(tmax >= 0 && tmax <= 1, "tmax must be in [0, 1]");
        require_device();
        if (n == 0) return;
        DBuf<double> a, b, t;
        DBuf<int8_t> h;
        upload(a, x0, 12 * n, 0);
        upload(b, x1, 12 * n, 0);
        t.reserve(n);
        h.reserve(n);
        ccd_stencils(0, is_ee, n, a.p, b.p, min_distance, tmax, tolerance, max_iterations, rescale, h.p, t.p);
        copy_out(hit, h.p, n, 0);
        copy_out(toi, t.p, sizeof(double) * n, 0);
        IPCG_CUDA(cudaStreamSynchronize(0));
    });
}

int ipcg_distance_stencils(int kind, int64_t n, const double* x, int8_t* dtype, double* dist)
{
    return guarded([&] {
        require(kind >= 0 && kind <= 2, "bad kind");
        require(n >= 0 && n < INT32_MAX, "bad n");
        require(n == 0 || (x && dtype && dist), "NULL argument");
        require_device();
        if (n == 0) return;
        const int per = kind == 0 ? 9 : 12;
        DBuf<double> a, d;
        DBuf<int8_t> t;
        upload(a, x, per * n, 0);
        d.reserve(n);
        t.reserve(n);
        distance_stencils(0, kind, n, a.p, t.p, d.p);
        copy_out(dtype, t.p, n, 0);
        copy_out(dist, d.p, sizeof(double) * n, 0);
        IPCG_CUDA(cudaStreamSynchronize(0));
    });
}

int ipcg_barrier_energy_noalloc(const double* vertices, int64_t num_vertices, const int32_t* edges,
    int64_t num_edges, const int32_t* faces, int64_t num_faces, int64_t nvv, const int32_t* vv, const double* vv_w,
    int64_t nev, const int32_t* ev, const double* ev_w, int64_t nee, const int32_t* ee, const double* ee_eps_x,
    const int8_t* ee_dtype, const double* ee_w, int64_t nfv, const int32_t* fv, const double* fv_w, double dhat,
    double stiffness, double dmin, int use_physical_barrier, double* energy, void* stream)
{
    return guarded([&] {
        require(num_vertices >= 0 && num_edges >= 0 && num_faces >= 0, "negative size");
        require(nvv >= 0 && nev >= 0 && nee >= 0 && nfv >= 0, "negative count");
        require(dhat > 0, "dhat must be positive");
        require(dmin >= 0, "dmin must be non-negative");
        require(energy != nullptr, "energy is NULL");
        // every array must already be device memory: this entry point copies
        // nothing (a host copy could need a staging allocation)
        const void* must_be_device[] = { energy, vertices, nvv ? vv : nullptr, nvv ? vv_w : nullptr,
            nev ? ev : nullptr, nev ? ev_w : nullptr, nev ? edges : nullptr, nee ? ee : nullptr,
            nee ? ee_eps_x : nullptr, nee ? ee_dtype : nullptr, nee ? ee_w : nullptr, nee ? edges : nullptr,
            nfv ? fv : nullptr, nfv ? fv_w : nullptr, nfv ? faces : nullptr };
        for (const void* p : must_be_device)
            if (p != nullptr)
                require(is_device_ptr_on_current(p),
                    "allocation-free energy: every array must be device memory of the current device");
        require(nvv + nev + nee + nfv == 0 || vertices, "vertices is NULL");
        require(nvv == 0 || (vv && vv_w), "vv arrays are NULL");
        require(nev == 0 || (ev && ev_w && edges), "ev arrays are NULL");
        require(nee == 0 || (ee && ee_eps_x && ee_dtype && ee_w && edges), "ee arrays are NULL");
        require(nfv == 0 || (fv && fv_w && faces), "fv arrays are NULL");
        const ContactsNoAlloc in { nvv, nev, nee, nfv, vv, ev, ee, fv, vv_w, ev_w, ee_w, fv_w, ee_eps_x, ee_dtype };
        barrier_energy_noalloc(vertices, edges, faces, num_vertices, num_edges, num_faces, in, dhat, stiffness, dmin,
            use_physical_barrier ? 1 : 0, energy, (cudaStream_t)stream);
    });
}

} // extern "C"
