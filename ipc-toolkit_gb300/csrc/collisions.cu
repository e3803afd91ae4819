// collisions.cu — NormalCollisions::build on the device.
//
// Restates src/ipc/collisions/normal/normal_collisions.cpp:20-158 and
// normal_collisions_builder.cpp:26-336,547-689: every EE / FV broad-phase
// candidate is classified and measured in FP64 (bit-exact with the
// reference's unfused evaluation; this file is compiled with -fmad=false),
// kept if d^2 < (dhat+dmin)^2 (strict), and reduced by distance type to a
// VV / EV / EE / FV record.  VV and EV records are merged by key with summed
// weights (weights are 1 without area weighting, so the merged weight is the
// multiplicity); EE and FV records are unique by construction.  All four
// lists are sorted by key, which fixes the (thread-dependent) order of the
// reference.
#include <cooperative_groups.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "geom.cuh"
#include "internal.cuh"
#include "profile.cuh"

namespace cg = cooperative_groups;

namespace ipcg {

namespace {

constexpr int BLOCK = 256;

__device__ __forceinline__ unsigned long long key2(unsigned a, unsigned b)
{
    return ((unsigned long long)a << 32) | (unsigned long long)b;
}

__device__ __forceinline__ int append(int* __restrict__ count)
{
    cg::coalesced_group g = cg::coalesced_threads();
    int base = 0;
    if (g.thread_rank() == 0) base = atomicAdd(count, (int)g.size());
    return g.shfl(base, 0) + (int)g.thread_rank();
}

struct Out {
    unsigned long long* vv; // VV keys (min,max)
    unsigned long long* ev; // EV keys (e,v)
    double* vv_w;           // VV / EV record weights (area weighting; else null)
    double* ev_w;
    const double* varea;    // rest-mesh areas (area weighting; else null)
    const double* earea;
    unsigned long long* ee; // EE keys (ea,eb)
    int* ee_rec;            // EE record slot -> candidate id
    double* ee_eps;
    int8_t* ee_dt;
    unsigned long long* fv; // FV keys (f,v)
    int* count;             // [vv, ev, ee, fv]
};

__device__ __forceinline__ void put_vv(const Out& o, int a, int b, double w)
{
    const int s = append(o.count + 0);
    o.vv[s] = key2(min(a, b), max(a, b));
    if (o.vv_w) o.vv_w[s] = w;
}
__device__ __forceinline__ void put_ev(const Out& o, int e, int v, double w)
{
    const int s = append(o.count + 1);
    o.ev[s] = key2(e, v);
    if (o.ev_w) o.ev_w[s] = w;
}
// Area weights (normal_collisions_builder.cpp:146, 181-183): FV and its
// reductions vertex_area(v) / 4, EE and its reductions
// (edge_area(ea) + edge_area(eb)) / 4; 1 without area weighting.
__device__ __forceinline__ double fv_weight(const double* __restrict__ varea, int v)
{
    return varea ? 0.25 * __ldg(varea + v) : 1.0;
}
__device__ __forceinline__ double ee_weight(const double* __restrict__ earea, int ea, int eb)
{
    return earea ? 0.25 * (__ldg(earea + ea) + __ldg(earea + eb)) : 1.0;
}

// normal_collisions_builder.cpp:140-237, candidate oriented ea < eb
__global__ void k_filter_ee(const int2* __restrict__ cand, int n, const double* __restrict__ V,
    const double* __restrict__ rest, const int* __restrict__ E, const double* __restrict__ scene_off2, SceneView sv,
    Out o)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int2 c = cand[i];
    const int ea = c.x, eb = c.y;
    const int a0 = E[2 * ea], a1 = E[2 * ea + 1], b0 = E[2 * eb], b1 = E[2 * eb + 1];
    const double offset_sqr = __ldg(scene_off2 + sv.of(a0));
    const V3 xa0 = load_v3(V, a0), xa1 = load_v3(V, a1), xb0 = load_v3(V, b0), xb1 = load_v3(V, b1);
    const int actual = edge_edge_distance_type(xa0, xa1, xb0, xb1);
    const double d = edge_edge_distance(xa0, xa1, xb0, xb1, actual);
    if (!(d < offset_sqr)) return;
    const double eps_x = ee_mollifier_threshold(load_v3(rest, a0), load_v3(rest, a1), load_v3(rest, b0),
        load_v3(rest, b1));
    const double cr = ee_cross_sqnorm(xa0, xa1, xb0, xb1);
    const int dtype = cr < eps_x ? (int)EA_EB : actual;
    const double w = ee_weight(o.earea, ea, eb);
    switch (dtype) {
    case EA0_EB0: put_vv(o, a0, b0, w); break;
    case EA0_EB1: put_vv(o, a0, b1, w); break;
    case EA1_EB0: put_vv(o, a1, b0, w); break;
    case EA1_EB1: put_vv(o, a1, b1, w); break;
    case EA_EB0: put_ev(o, ea, b0, w); break;
    case EA_EB1: put_ev(o, ea, b1, w); break;
    case EA0_EB: put_ev(o, eb, a0, w); break;
    case EA1_EB: put_ev(o, eb, a1, w); break;
    default: {
        const int s = append(o.count + 2);
        o.ee[s] = key2(ea, eb);
        o.ee_rec[s] = s;
        o.ee_eps[s] = eps_x;
        o.ee_dt[s] = (int8_t)actual;
    }
    }
}

// normal_collisions_builder.cpp:239-336
__global__ void k_filter_fv(const int2* __restrict__ cand, int n, const double* __restrict__ V,
    const int* __restrict__ F, const int* __restrict__ F2E, const double* __restrict__ scene_off2, SceneView sv,
    Out o)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int2 c = cand[i];
    const int fi = c.x, vi = c.y;
    const double offset_sqr = __ldg(scene_off2 + sv.of(vi));
    const int f0 = F[3 * fi], f1 = F[3 * fi + 1], f2 = F[3 * fi + 2];
    const V3 p = load_v3(V, vi), t0 = load_v3(V, f0), t1 = load_v3(V, f1), t2 = load_v3(V, f2);
    const int dtype = point_triangle_distance_type(p, t0, t1, t2);
    const double d = point_triangle_distance(p, t0, t1, t2, dtype);
    if (!(d < offset_sqr)) return;
    const double w = fv_weight(o.varea, vi);
    switch (dtype) {
    case P_T0: put_vv(o, vi, f0, w); break;
    case P_T1: put_vv(o, vi, f1, w); break;
    case P_T2: put_vv(o, vi, f2, w); break;
    case P_E0T: put_ev(o, F2E[3 * fi + 0], vi, w); break;
    case P_E1T: put_ev(o, F2E[3 * fi + 1], vi, w); break;
    case P_E2T: put_ev(o, F2E[3 * fi + 2], vi, w); break;
    default: {
        const int s = append(o.count + 3);
        o.fv[s] = key2(fi, vi);
    }
    }
}

__global__ void k_unpack_rle(const unsigned long long* __restrict__ uniq, const int* __restrict__ counts,
    const int* __restrict__ d_num, int2* __restrict__ ids, double* __restrict__ w)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= *d_num) return;
    const unsigned long long k = uniq[i];
    ids[i] = make_int2((int)(k >> 32), (int)(k & 0xffffffffu));
    w[i] = (double)counts[i];
}

__global__ void k_unpack_keys(const unsigned long long* __restrict__ keys, int n, int2* __restrict__ ids,
    double* __restrict__ w, const double* __restrict__ varea)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const unsigned long long k = keys[i];
    const int2 fv = make_int2((int)(k >> 32), (int)(k & 0xffffffffu));
    ids[i] = fv;
    w[i] = fv_weight(varea, fv.y);
}

__global__ void k_gather_ee(const unsigned long long* __restrict__ keys, const int* __restrict__ perm, int n,
    const double* __restrict__ eps_in, const int8_t* __restrict__ dt_in, int2* __restrict__ ids,
    double* __restrict__ eps, int8_t* __restrict__ dt, double* __restrict__ w, const double* __restrict__ earea)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const unsigned long long k = keys[i];
    const int p = perm[i];
    const int2 ee = make_int2((int)(k >> 32), (int)(k & 0xffffffffu));
    ids[i] = ee;
    eps[i] = eps_in[p];
    dt[i] = dt_in[p];
    w[i] = ee_weight(earea, ee.x, ee.y);
}

// Weighted merge of duplicate VV / EV keys (normal_collisions_builder.cpp:
// 547-689).  Records are ordered by (key, weight) with two stable radix
// sorts, so each key's weights are summed in ascending order, whatever order
// the filter kernels appended them in.
__device__ __forceinline__ unsigned long long weight_key(double w)
{
    // order-preserving bits of a finite double
    const long long b = __double_as_longlong(w);
    return (unsigned long long)(b ^ ((b >> 63) | (long long)0x8000000000000000ULL));
}
__global__ void k_weight_keys(const double* __restrict__ w, int n, unsigned long long* __restrict__ wk,
    int* __restrict__ idx)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    wk[i] = weight_key(w[i]);
    idx[i] = i;
}
__global__ void k_gather_keys(const unsigned long long* __restrict__ keys, const int* __restrict__ idx, int n,
    unsigned long long* __restrict__ out)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    out[i] = keys[idx[i]];
}
__global__ void k_sum_runs(const unsigned long long* __restrict__ uniq, const int* __restrict__ counts,
    const int* __restrict__ offs, const int* __restrict__ d_num, const int* __restrict__ idx,
    const double* __restrict__ w, int2* __restrict__ ids, double* __restrict__ wout)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= *d_num) return;
    const unsigned long long k = uniq[i];
    ids[i] = make_int2((int)(k >> 32), (int)(k & 0xffffffffu));
    double s = 0.0;
    for (int j = offs[i], e = offs[i] + counts[i]; j < e; ++j) s += w[idx[j]];
    wout[i] = s;
}

} // namespace

void build_collision_set(ipcg_collisions* c, ipcg_mesh* m, const double* V, const double* dhat, const double* dmin)
{
    cudaStream_t s = m->stream;
    // per-scene inflation 0.5 (dhat + dmin) (normal_collisions.cpp:30) and
    // activation threshold (dmin + dhat)^2 (normal_collisions.cpp:52-54)
    const int ns = (int)m->n_scenes;
    std::vector<double> hr(ns), hoff(ns);
    for (int k = 0; k < ns; ++k) {
        hr[k] = 0.5 * (dhat[k] + dmin[k]);
        hoff[k] = (dmin[k] + dhat[k]) * (dmin[k] + dhat[k]);
    }
    m->scene_r.reserve(ns);
    m->scene_off2.reserve(ns);
    IPCG_CUDA(cudaMemcpyAsync(m->scene_r.p, hr.data(), sizeof(double) * ns, cudaMemcpyHostToDevice, s));
    IPCG_CUDA(cudaMemcpyAsync(m->scene_off2.p, hoff.data(), sizeof(double) * ns, cudaMemcpyHostToDevice, s));
    int64_t n_ee = 0, n_fv = 0;
    detect_candidates(m, V, nullptr, m->scene_r.p, n_ee, n_fv);
    c->n_cand_ee = n_ee;
    c->n_cand_fv = n_fv;
    c->dmin = dmin[0];
    c->scene_dmin.assign(dmin, dmin + ns);
    c->sorted = true;
    const int64_t nc = n_ee + n_fv;
    // raw records: at most one per candidate
    const int64_t cap = nc + 16;
    m->keys_a.reserve(4 * cap);
    m->keys_b.reserve(4 * cap);
    m->ivals_a.reserve(2 * cap);
    m->ivals_b.reserve(3 * cap);
    m->partial.reserve(cap);
    m->i8tmp.reserve(cap);
    unsigned long long* kv = m->keys_a.p;           // [vv | ev | ee | fv] regions of size cap
    Out o;
    o.vv = kv;
    o.ev = kv + cap;
    o.ee = kv + 2 * cap;
    o.fv = kv + 3 * cap;
    o.ee_rec = m->ivals_a.p;
    o.ee_eps = m->partial.p;
    o.ee_dt = m->i8tmp.p;
    const bool weighted = c->use_area_weighting != 0;
    o.vv_w = o.ev_w = nullptr;
    o.varea = weighted ? m->vertex_area.p : nullptr;
    o.earea = weighted ? m->edge_area.p : nullptr;
    if (weighted) {
        m->rec_w.reserve(2 * cap);
        o.vv_w = m->rec_w.p;
        o.ev_w = m->rec_w.p + cap;
    }
    m->counters.reserve(16);
    o.count = m->counters.p + 4;
    IPCG_CUDA(cudaMemsetAsync(o.count, 0, sizeof(int) * 8, s));
    const SceneView sv = scene_view(m);
    if (n_ee)
        IPCG_LAUNCH("k_filter_ee", s, k_filter_ee<<<grid_for(n_ee, BLOCK), BLOCK, 0, s>>>(m->cand.p, (int)n_ee, V,
            m->rest.p, m->E.p, m->scene_off2.p, sv, o));
    if (n_fv)
        IPCG_LAUNCH("k_filter_fv", s, k_filter_fv<<<grid_for(n_fv, BLOCK), BLOCK, 0, s>>>(m->cand.p + m->cand_cap,
            (int)n_fv, V, m->F.p, m->F2E.p, m->scene_off2.p, sv, o));
    IPCG_CHECK_LAUNCH();
    IPCG_CUDA(cudaMemcpyAsync(m->h_counters.p, o.count, sizeof(int) * 4, cudaMemcpyDeviceToHost, s));
    IPCG_CUDA(cudaStreamSynchronize(s));
    const int rvv = m->h_counters.p[0], rev = m->h_counters.p[1], ree = m->h_counters.p[2], rfv = m->h_counters.p[3];

    unsigned long long* ks = m->keys_b.p;
    int* d_num = m->counters.p + 12;
    const int idbits = 32 + bits_for(std::max(std::max(m->nV, m->nE), std::max(m->nF, (int64_t)2)));
    int* counts = m->ivals_b.p;
    c->vv.reserve(rvv + 1);
    c->vv_w.reserve(rvv + 1);
    c->ev.reserve(rev + 1);
    c->ev_w.reserve(rev + 1);
    if (!weighted) {
        // VV / EV: sort + run-length (weights = multiplicities); unique keys
        // are written back into the raw regions
        sort_keys_u64(m, m->stream, o.vv, ks, rvv, idbits);
        rle_u64(m, m->stream, ks, o.vv, counts, d_num + 0, rvv);
        if (rvv) IPCG_LAUNCH("k_unpack_rle", s, k_unpack_rle<<<grid_for(rvv, BLOCK), BLOCK, 0, s>>>(o.vv, counts, d_num + 0, c->vv.p, c->vv_w.p));
        sort_keys_u64(m, m->stream, o.ev, ks + cap, rev, idbits);
        rle_u64(m, m->stream, ks + cap, o.ev, counts + cap, d_num + 1, rev);
        if (rev) IPCG_LAUNCH("k_unpack_rle", s, k_unpack_rle<<<grid_for(rev, BLOCK), BLOCK, 0, s>>>(o.ev, counts + cap, d_num + 1, c->ev.p, c->ev_w.p));
    } else {
        m->wkeys.reserve(2 * cap);
        m->widx.reserve(3 * cap);
        auto merge = [&](unsigned long long* raw, const double* w, int n, unsigned long long* sorted, int* cnt,
                         int* num, int2* ids, double* wout) {
            if (n == 0) {
                IPCG_CUDA(cudaMemsetAsync(num, 0, sizeof(int), s));
                return;
            }
            unsigned long long *wk = m->wkeys.p, *wk2 = m->wkeys.p + cap;
            int *i0 = m->widx.p, *i1 = m->widx.p + cap, *i2 = m->widx.p + 2 * cap;
            IPCG_LAUNCH("k_weight_keys", s, k_weight_keys<<<grid_for(n, BLOCK), BLOCK, 0, s>>>(w, n, wk, i0));
            sort_pairs_u64(m, m->stream, wk, wk2, i0, i1, n, 64);
            IPCG_LAUNCH("k_gather_keys", s, k_gather_keys<<<grid_for(n, BLOCK), BLOCK, 0, s>>>(raw, i1, n, wk));
            sort_pairs_u64(m, m->stream, wk, sorted, i1, i2, n, idbits);
            IPCG_CUDA(cudaMemsetAsync(cnt, 0, sizeof(int) * n, s));
            rle_u64(m, m->stream, sorted, raw, cnt, num, n);
            exclusive_sum_i32(m, m->stream, cnt, i0, n);
            IPCG_LAUNCH("k_sum_runs", s, k_sum_runs<<<grid_for(n, BLOCK), BLOCK, 0, s>>>(raw, cnt, i0, num, i2, w,
                ids, wout));
        };
        merge(o.vv, o.vv_w, rvv, ks, counts, d_num + 0, c->vv.p, c->vv_w.p);
        merge(o.ev, o.ev_w, rev, ks + cap, counts + cap, d_num + 1, c->ev.p, c->ev_w.p);
    }
    // EE: sort keys with record ids, gather eps / dtype
    c->ee.reserve(ree + 1);
    c->ee_w.reserve(ree + 1);
    c->ee_eps.reserve(ree + 1);
    c->ee_dtype.reserve(ree + 1);
    if (ree) {
        sort_pairs_u64(m, m->stream, o.ee, ks + 2 * cap, o.ee_rec, m->ivals_b.p + 2 * cap, ree, idbits);
        IPCG_LAUNCH("k_gather_ee", s, k_gather_ee<<<grid_for(ree, BLOCK), BLOCK, 0, s>>>(ks + 2 * cap, m->ivals_b.p + 2 * cap, ree, o.ee_eps, o.ee_dt,
            c->ee.p, c->ee_eps.p, c->ee_dtype.p, c->ee_w.p, o.earea));
    }
    // FV
    c->fv.reserve(rfv + 1);
    c->fv_w.reserve(rfv + 1);
    if (rfv) {
        sort_keys_u64(m, m->stream, o.fv, ks + 3 * cap, rfv, idbits);
        IPCG_LAUNCH("k_unpack_keys", s, k_unpack_keys<<<grid_for(rfv, BLOCK), BLOCK, 0, s>>>(ks + 3 * cap, rfv, c->fv.p, c->fv_w.p,
            o.varea));
    }
    IPCG_CHECK_LAUNCH();
    IPCG_CUDA(cudaMemcpyAsync(m->h_counters.p, d_num, sizeof(int) * 2, cudaMemcpyDeviceToHost, s));
    IPCG_CUDA(cudaStreamSynchronize(s));
    c->nvv = m->h_counters.p[0];
    c->nev = m->h_counters.p[1];
    c->nee = ree;
    c->nfv = rfv;
}

void mesh_areas_host(const double* R, int64_t nV, const int32_t* E, int64_t nE, const int32_t* F, int64_t nF,
    const int32_t* F2E, double* va, double* ea)
{
    // vertex: 1/3 of each incident face area, else 1/2 of each incident edge
    // length, else 1; edge: 1/3 of each incident face area, else its length.
    // -1 marks "not touched yet", as in the reference.
    auto len = [&](int64_t e) {
        const int a = E[2 * e], b = E[2 * e + 1];
        const V3 d = V3 { R[3 * b] - R[3 * a], R[3 * b + 1] - R[3 * a + 1], R[3 * b + 2] - R[3 * a + 2] };
        return std::sqrt(sqnorm(d));
    };
    std::vector<double> by_edges(nV, -1.0), by_faces(nV, -1.0);
    for (int64_t e = 0; e < nE; ++e) {
        const double l = len(e);
        for (int j = 0; j < 2; ++j) {
            double& a = by_edges[E[2 * e + j]];
            a = std::max(a, 0.0) + 0.5 * l;
        }
    }
    for (int64_t e = 0; e < nE; ++e) ea[e] = -1.0;
    for (int64_t f = 0; f < nF; ++f) {
        auto P = [&](int k) {
            const int v = F[3 * f + k];
            return V3 { R[3 * v], R[3 * v + 1], R[3 * v + 2] };
        };
        const V3 t0 = P(0), t1 = P(1), t2 = P(2);
        const double third = 0.5 * std::sqrt(sqnorm(cross(t1 - t0, t2 - t0))) / 3.0;
        for (int j = 0; j < 3; ++j) {
            double& a = by_faces[F[3 * f + j]];
            a = std::max(a, 0.0) + third;
            double& b = ea[F2E[3 * f + j]];
            b = std::max(b, 0.0) + third;
        }
    }
    for (int64_t v = 0; v < nV; ++v) va[v] = by_faces[v] < 0 ? (by_edges[v] < 0 ? 1.0 : by_edges[v]) : by_faces[v];
    for (int64_t e = 0; e < nE; ++e)
        if (ea[e] < 0) ea[e] = len(e);
}

} // namespace ipcg
