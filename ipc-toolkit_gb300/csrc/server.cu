// server.cu — a continuous-batching request loop over resident scenes.
//
// The reference is used one simulation at a time: each Newton iteration
// calls NormalCollisions::build, BarrierPotential's energy / gradient /
// Hessian (normal_collisions.cpp:20-36, potential.cpp:36-222) and, in the
// line search, compute_collision_free_stepsize (ipc.cpp:42-106).  The server
// takes those calls as requests from many simulations at once:
//
//  * every scene's mesh, LBVH scratch and collision set stay on the device
//    between requests;
//  * worker threads take requests in arrival order, at most one per scene
//    at a time (a scene's requests are a Newton loop: they are ordered), and
//    run each on its scene's own streams, so requests of different scenes
//    overlap on the GPU as they arrive ("continuous batching": a request is
//    admitted as soon as a worker, its scene and memory are free, not when a
//    batch fills);
//  * admission is bounded by an HBM budget: a request starts only if the
//    resident working memory of all scenes plus its own expected need fits;
//    otherwise idle scenes' scratch (LBVH, candidates, Hessian work space --
//    not their collision sets) is released, least recently used first, and
//    if it still does not fit the request waits for running ones to finish.
//
// A request's result does not depend on what else runs: each scene's work is
// issued in order on its own streams and every reduction is deterministic
// except the gradient's atomic adds (rounding-level differences).
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "internal.cuh"

using namespace ipcg;

namespace {

int64_t now_ns()
{
    return std::chrono::duration_cast<std::chrono::nanoseconds>(
        std::chrono::steady_clock::now().time_since_epoch())
        .count();
}

template <typename T> int64_t bytes_of(const DBuf<T>& b) { return (int64_t)(b.cap * sizeof(T)); }

int64_t bvh_bytes(const LBVH& b)
{
    return bytes_of(b.lo) + bytes_of(b.hi) + bytes_of(b.first) + bytes_of(b.last) + bytes_of(b.parent)
        + bytes_of(b.flags) + bytes_of(b.leaf_scene) + bytes_of(b.codes) + bytes_of(b.codes_sorted) + bytes_of(b.ids)
        + bytes_of(b.ids_sorted) + bytes_of(b.plo) + bytes_of(b.phi);
}

void bvh_release(LBVH& b)
{
    b.lo.release();
    b.hi.release();
    b.first.release();
    b.last.release();
    b.parent.release();
    b.flags.release();
    b.leaf_scene.release();
    b.codes.release();
    b.codes_sorted.release();
    b.ids.release();
    b.ids_sorted.release();
    b.plo.release();
    b.phi.release();
    b.n = 0;
}

// Work space of a mesh that is rebuilt on demand (not its topology, its
// per-scene parameters or any collision set).
int64_t scratch_bytes(const ipcg_mesh* m)
{
    return bytes_of(m->V0) + bytes_of(m->V1) + bytes_of(m->bounds) + bvh_bytes(m->ebvh) + bvh_bytes(m->fbvh)
        + bytes_of(m->cand) + bytes_of(m->tmp) + bytes_of(m->keys_a) + bytes_of(m->keys_b) + bytes_of(m->ivals_a)
        + bytes_of(m->ivals_b) + bytes_of(m->i8tmp) + bytes_of(m->partial) + bytes_of(m->toi_bits) + bytes_of(m->hs)
        + bytes_of(m->proj);
}

void release_scratch(ipcg_mesh* m)
{
    m->V0.release();
    m->V1.release();
    m->bounds.release();
    bvh_release(m->ebvh);
    bvh_release(m->fbvh);
    m->cand.release();
    m->cand_cap = 0;
    m->tmp.release();
    m->keys_a.release();
    m->keys_b.release();
    m->ivals_a.release();
    m->ivals_b.release();
    m->i8tmp.release();
    m->partial.release();
    m->toi_bits.release();
    m->hs.release();
    m->proj.release();
}

int64_t collision_bytes(const ipcg_collisions* c)
{
    return bytes_of(c->vv) + bytes_of(c->ev) + bytes_of(c->ee) + bytes_of(c->fv) + bytes_of(c->vv_w)
        + bytes_of(c->ev_w) + bytes_of(c->ee_w) + bytes_of(c->fv_w) + bytes_of(c->ee_eps) + bytes_of(c->ee_dtype);
}

struct Scene {
    ipcg_mesh* mesh;
    ipcg_collisions* col;
    double dhat, dmin, kappa;
    int options = 0;       // barrier option bits of its barrier requests
    bool busy = false;
    int64_t need = 0;      // expected peak working memory of one request
    int64_t last_used = 0; // admission order of its last request (LRU)
    DBuf<double> grad;     // device gradient of barrier requests
};

struct Request {
    int64_t scene = 0;
    int kind = 0;
    int psd = IPCG_PSD_NONE;
    double min_distance = 0;
    std::vector<double> V, V1;
    // results
    bool done = false;
    int status = IPCG_OK;
    std::string error;
    double energy = 0, step = 1;
    int64_t contacts = 0;
    std::vector<double> grad;
    ipcg_csr* hess = nullptr;
    int64_t t_submit = 0, t_start = 0, t_end = 0;
};

} // namespace

struct ipcg_server {
    int device = 0;
    int64_t budget = 0;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::vector<Scene*> scenes;
    std::deque<int64_t> queue;
    std::unordered_map<int64_t, Request> reqs;
    std::vector<std::thread> workers;
    bool stop = false;
    int64_t next_ticket = 1, admitted = 0, completed = 0, running = 0, releases = 0;

    ~ipcg_server()
    {
        {
            std::lock_guard<std::mutex> lk(mu);
            stop = true;
        }
        cv_work.notify_all();
        for (auto& t : workers)
            if (t.joinable()) t.join();
        for (auto& kv : reqs) delete kv.second.hess;
        for (Scene* s : scenes) delete s;
    }

    // Memory held by scene s (resident work space, collision set, gradient).
    int64_t resident(const Scene* s) const
    {
        return scratch_bytes(s->mesh) + collision_bytes(s->col) + bytes_of(s->grad);
    }

    // Whether a request of scene `s` may start now; may release idle
    // scenes' scratch (LRU first) to make room.  Called with mu held.
    bool admit(Scene* s)
    {
        auto total = [&]() {
            int64_t t = 0;
            for (const Scene* x : scenes) t += x->busy ? std::max(x->need, resident(x)) : resident(x);
            return t - resident(s) + std::max(s->need, resident(s));
        };
        if (total() <= budget) return true;
        std::vector<Scene*> idle;
        for (Scene* x : scenes)
            if (!x->busy && x != s && scratch_bytes(x->mesh) > 0) idle.push_back(x);
        std::sort(idle.begin(), idle.end(), [](const Scene* a, const Scene* b) { return a->last_used < b->last_used; });
        for (Scene* x : idle) {
            release_scratch(x->mesh);
            x->grad.release();
            ++releases;
            if (total() <= budget) return true;
        }
        return running == 0; // alone it may exceed the budget: nothing else would free memory
    }

    void run(Request& r, Scene& sc)
    {
        ipcg_mesh* m = sc.mesh;
        if (r.kind == 0) {
            const double* dV = stage_positions(m, r.V.data(), m->V0);
            build_collision_set(sc.col, m, dV, &sc.dhat, &sc.dmin);
            BarrierArgs a { sc.dhat, sc.kappa, sc.col->dmin, 0, r.psd };
            barrier_options(sc.options, a);
            sc.grad.reserve(3 * m->nV + 1);
            r.hess = new ipcg_csr();
            // the same cached-pattern pass as a direct call, so results are identical
            if (!(r.hess && barrier_egh(sc.col, m, dV, a, &r.energy, sc.grad.p, r.hess)))
                barrier_evaluate(sc.col, m, dV, a, &r.energy, sc.grad.p, r.hess);
            r.grad.resize(3 * m->nV);
            if (m->nV)
                IPCG_CUDA(cudaMemcpyAsync(r.grad.data(), sc.grad.p, sizeof(double) * 3 * m->nV,
                    cudaMemcpyDeviceToHost, m->stream));
            IPCG_CUDA(cudaStreamSynchronize(m->stream));
            r.contacts = sc.col->size();
        } else {
            const double* d0 = stage_positions(m, r.V.data(), m->V0);
            const double* d1 = stage_positions(m, r.V1.data(), m->V1);
            collision_free_stepsize(m, d0, d1, &r.min_distance, 1e-6, 10000000, 0.8, &r.step, &r.contacts);
        }
    }

    void worker_loop()
    {
        cudaSetDevice(device);
        std::unique_lock<std::mutex> lk(mu);
        for (;;) {
            // first queued request whose scene is idle and which fits the budget
            auto pick = queue.end();
            for (auto it = queue.begin(); it != queue.end(); ++it) {
                Scene* s = scenes[reqs[*it].scene];
                if (s->busy) continue;
                if (admit(s)) pick = it;
                break; // arrival order: a request that does not fit blocks the later ones
            }
            if (pick == queue.end()) {
                if (stop) return;
                cv_work.wait(lk);
                continue;
            }
            const int64_t ticket = *pick;
            queue.erase(pick);
            Request& r = reqs[ticket];
            Scene& sc = *scenes[r.scene];
            sc.busy = true;
            sc.last_used = ++admitted;
            ++running;
            lk.unlock();
            r.t_start = now_ns();
            try {
                run(r, sc);
            } catch (const Error& e) {
                r.status = e.code;
                r.error = e.what();
            } catch (const std::bad_alloc&) {
                r.status = IPCG_ERR_OOM;
                r.error = "host allocation failed";
            } catch (const std::exception& e) {
                r.status = IPCG_ERR_INVALID;
                r.error = e.what();
            }
            r.t_end = now_ns();
            lk.lock();
            const int64_t out = r.hess ? (int64_t)(r.hess->col.cap * sizeof(int) + r.hess->val.cap * sizeof(double)
                                                   + r.hess->row_ptr.cap * sizeof(int64_t))
                                       : 0;
            sc.need = std::max(sc.need, resident(&sc) + out);
            sc.busy = false;
            --running;
            ++completed;
            r.done = true;
            cv_done.notify_all();
            cv_work.notify_all();
        }
    }
};

namespace {

template <typename F> int server_call(F&& f)
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

int64_t enqueue(ipcg_server* sv, Request&& r)
{
    r.t_submit = now_ns();
    int64_t ticket;
    {
        std::lock_guard<std::mutex> lk(sv->mu);
        ticket = sv->next_ticket++;
        sv->reqs.emplace(ticket, std::move(r));
        sv->queue.push_back(ticket);
    }
    sv->cv_work.notify_one();
    return ticket;
}

} // namespace

extern "C" {

int ipcg_server_create(int workers, int64_t hbm_budget_bytes, ipcg_server** out)
{
    return server_call([&] {
        check(out != nullptr, "out is NULL");
        check(workers >= 1 && workers <= 64, "workers must be in [1, 64]");
        check(hbm_budget_bytes > 0, "hbm_budget_bytes must be positive");
        auto* sv = new ipcg_server();
        sv->budget = hbm_budget_bytes;
        if (cudaGetDevice(&sv->device) != cudaSuccess) sv->device = 0;
        cudaGetLastError();
        for (int i = 0; i < workers; ++i) sv->workers.emplace_back([sv] { sv->worker_loop(); });
        *out = sv;
    });
}

int ipcg_server_destroy(ipcg_server* server)
{
    return server_call([&] { delete server; });
}

int ipcg_server_add_scene(ipcg_server* sv, ipcg_mesh* mesh, ipcg_collisions* col, double dhat, double dmin,
    double stiffness, int64_t* scene)
{
    return server_call([&] {
        check(sv && mesh && col && scene, "NULL argument");
        check(mesh->n_scenes == 1, "a server scene is a single-scene mesh");
        check(dhat > 0, "dhat must be positive");
        check(dmin >= 0, "dmin must be non-negative");
        auto* s = new Scene();
        s->mesh = mesh;
        s->col = col;
        s->dhat = dhat;
        s->dmin = dmin;
        s->kappa = stiffness;
        s->need = 3072 * (mesh->nV + 1); // first estimate; measured after each request
        std::lock_guard<std::mutex> lk(sv->mu);
        for (const Scene* x : sv->scenes)
            check(x->mesh != mesh && x->col != col, "mesh or collision set already registered");
        *scene = (int64_t)sv->scenes.size();
        sv->scenes.push_back(s);
    });
}

int ipcg_server_set_scene_options(ipcg_server* sv, int64_t scene, int barrier_options_bits)
{
    return server_call([&] {
        check(sv != nullptr, "NULL argument");
        BarrierArgs probe { 1.0, 1.0, 0.0, 0, IPCG_PSD_NONE };
        barrier_options(barrier_options_bits, probe); // validates the bits
        std::lock_guard<std::mutex> lk(sv->mu);
        check(scene >= 0 && scene < (int64_t)sv->scenes.size(), "unknown scene");
        sv->scenes[scene]->options = barrier_options_bits;
    });
}

int ipcg_server_submit_barrier(ipcg_server* sv, int64_t scene, const double* vertices, int psd_method, int64_t* ticket)
{
    return server_call([&] {
        check(sv && ticket, "NULL argument");
        check(psd_method >= IPCG_PSD_NONE && psd_method <= IPCG_PSD_ABS, "Invalid type of PSD projection!");
        Request r;
        {
            std::lock_guard<std::mutex> lk(sv->mu);
            check(scene >= 0 && scene < (int64_t)sv->scenes.size(), "unknown scene");
            const int64_t nV = sv->scenes[scene]->mesh->nV;
            check(vertices || nV == 0, "vertices is NULL");
            r.V.assign(vertices, vertices + 3 * nV);
        }
        r.scene = scene;
        r.kind = 0;
        r.psd = psd_method;
        *ticket = enqueue(sv, std::move(r));
    });
}

int ipcg_server_submit_stepsize(ipcg_server* sv, int64_t scene, const double* vertices_t0, const double* vertices_t1,
    double min_distance, int64_t* ticket)
{
    return server_call([&] {
        check(sv && ticket, "NULL argument");
        check(min_distance >= 0, "min_distance must be non-negative");
        Request r;
        {
            std::lock_guard<std::mutex> lk(sv->mu);
            check(scene >= 0 && scene < (int64_t)sv->scenes.size(), "unknown scene");
            const int64_t nV = sv->scenes[scene]->mesh->nV;
            check((vertices_t0 && vertices_t1) || nV == 0, "vertices is NULL");
            r.V.assign(vertices_t0, vertices_t0 + 3 * nV);
            r.V1.assign(vertices_t1, vertices_t1 + 3 * nV);
        }
        r.scene = scene;
        r.kind = 1;
        r.min_distance = min_distance;
        *ticket = enqueue(sv, std::move(r));
    });
}

int ipcg_server_wait(ipcg_server* sv, int64_t ticket, ipcg_request_result* out, double* gradient, ipcg_csr** hessian)
{
    return server_call([&] {
        check(sv && out, "NULL argument");
        std::unique_lock<std::mutex> lk(sv->mu);
        check(sv->reqs.count(ticket) == 1, "unknown ticket");
        // look the request up again each time: other submits may rehash the map
        sv->cv_done.wait(lk, [&] { return sv->reqs.at(ticket).done; });
        auto it = sv->reqs.find(ticket);
        Request r = std::move(it->second);
        sv->reqs.erase(it);
        lk.unlock();
        out->status = r.status;
        out->kind = r.kind;
        out->energy = r.energy;
        out->step = r.step;
        out->contacts = r.contacts;
        out->t_submit_ns = r.t_submit;
        out->t_start_ns = r.t_start;
        out->t_end_ns = r.t_end;
        if (gradient && !r.grad.empty()) memcpy(gradient, r.grad.data(), sizeof(double) * r.grad.size());
        if (r.status != IPCG_OK) {
            delete r.hess;
            if (hessian) *hessian = nullptr;
            throw Error(r.status, r.error);
        }
        if (hessian) *hessian = r.hess;
        else delete r.hess;
    });
}

int ipcg_server_stats(ipcg_server* sv, int64_t stats[5])
{
    return server_call([&] {
        check(sv && stats, "NULL argument");
        std::lock_guard<std::mutex> lk(sv->mu);
        stats[0] = sv->completed;
        stats[1] = (int64_t)sv->queue.size();
        stats[2] = sv->running;
        stats[3] = sv->releases;
        int64_t res = 0;
        for (const Scene* x : sv->scenes) res += sv->resident(x);
        stats[4] = res;
    });
}

} // extern "C"
