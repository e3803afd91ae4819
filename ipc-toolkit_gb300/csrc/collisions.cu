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
    int2* vv_src;           // VV / EV record weight sources (area-weighted shape derivatives; else null)
    int2* ev_src;
    int2 src;               // the weight source of the candidate being filtered
    const double* varea;    // rest-mesh areas (area weighting; else null)
    const double* earea;
    unsigned long long* ee; // EE keys (ea,eb)
    int* ee_rec;            // EE record slot -> candidate id
    double* ee_eps;
    double* ee_w;           // EE record weights (improved max approximation; else null)
    int8_t* ee_dt;
    unsigned long long* fv; // FV keys (f,v)
    int* count;             // [vv, ev, ee, fv]
};

__device__ __forceinline__ void put_vv(const Out& o, int a, int b, double w)
{
    const int s = append(o.count + 0);
    o.vv[s] = key2(min(a, b), max(a, b));
    if (o.vv_w) o.vv_w[s] = w;
    if (o.vv_src) o.vv_src[s] = o.src;
}
__device__ __forceinline__ void put_ev(const Out& o, int e, int v, double w)
{
    const int s = append(o.count + 1);
    o.ev[s] = key2(e, v);
    if (o.ev_w) o.ev_w[s] = w;
    if (o.ev_src) o.ev_src[s] = o.src;
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
    o.src = make_int2(ea, eb);
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
        if (o.ee_w) o.ee_w[s] = w;
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
    o.src = make_int2(vi, -1);
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

// ---- CollisionSetType::IMPROVED_MAX_APPROX ----------------------------------
// normal_collisions.cpp:84-128, normal_collisions_builder.cpp:340-543 and the
// candidate conversions of candidates.cpp:583-692.  The conversions emit
// keys that are sorted and made unique; the three term kernels then append
// weighted VV / EV / EE records next to the ordinary ones.

__device__ __forceinline__ double pe_distance(V3 p, V3 e0, V3 e1)
{
    return point_edge_distance(p, e0, e1, point_edge_distance_type(p, e0, e1));
}

// edge-edge candidate -> edge-vertex keys (edge, vertex of the other edge)
__global__ void k_imp_ee_to_ev(const int2* __restrict__ cand, int n, const double* __restrict__ V,
    const int* __restrict__ E, const double* __restrict__ off2, SceneView sv, unsigned long long* __restrict__ keys,
    int* __restrict__ count)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int2 c = cand[i];
    const double off = __ldg(off2 + sv.of(E[2 * c.x]));
    for (int s = 0; s < 2; ++s) {
        const int ei = s ? c.y : c.x, ej = s ? c.x : c.y;
        const V3 x0 = load_v3(V, E[2 * ei]), x1 = load_v3(V, E[2 * ei + 1]);
        for (int j = 0; j < 2; ++j) {
            const int vj = E[2 * ej + j];
            if (pe_distance(load_v3(V, vj), x0, x1) < off) keys[append(count)] = key2(ei, vj);
        }
    }
}

// face-vertex candidate -> edge-vertex keys (face edge, vertex) and
// vertex-vertex keys (unordered: vertex, face vertex)
__global__ void k_imp_fv_to_ev_vv(const int2* __restrict__ cand, int n, const double* __restrict__ V,
    const int* __restrict__ E, const int* __restrict__ F, const int* __restrict__ F2E,
    const double* __restrict__ off2, SceneView sv, unsigned long long* __restrict__ kev, int* __restrict__ nev,
    unsigned long long* __restrict__ kvv, int* __restrict__ nvv)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int2 c = cand[i];
    const int f = c.x, v = c.y;
    const double off = __ldg(off2 + sv.of(v));
    const V3 p = load_v3(V, v);
    for (int j = 0; j < 3; ++j) {
        const int ei = F2E[3 * f + j];
        if (pe_distance(p, load_v3(V, E[2 * ei]), load_v3(V, E[2 * ei + 1])) < off) kev[append(nev)] = key2(ei, v);
        const int vj = F[3 * f + j];
        if (point_point_distance(p, load_v3(V, vj)) < off) kvv[append(nvv)] = key2(min(v, vj), max(v, vj));
    }
}

// An edge-vertex term reduced by its point-edge type
// (normal_collisions_builder.cpp:108-126).
__device__ __forceinline__ void put_typed(const Out& o, const int* __restrict__ E, int e, int v, int pe, double w)
{
    if (pe == P_E0) put_vv(o, v, E[2 * e], w);
    else if (pe == P_E1) put_vv(o, v, E[2 * e + 1], w);
    else put_ev(o, e, v, w);
}

__device__ __forceinline__ bool sorted_contains(const int* __restrict__ a, int lo, int hi, int x)
{
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        const int y = a[mid];
        if (y == x) return true;
        if (y < x) lo = mid + 1;
        else hi = mid;
    }
    return false;
}

// add_edge_edge_negative_edge_vertex_collision (builder.cpp:457-541):
// (ea, p) with p on edges eb of p's star; mollified pairs become EE terms of
// weight -w_ea, the rest are counted and leave one EV term of (count-1) w.
__global__ void k_imp_ee_negative(const unsigned long long* __restrict__ l1, int n, const double* __restrict__ V,
    const double* __restrict__ rest, const int* __restrict__ E, const int* __restrict__ ve_off,
    const int* __restrict__ ve_adj, Out o)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const unsigned long long k = l1[i];
    const int e = (int)(k >> 32), p = (int)(k & 0xffffffffu);
    const int a0 = E[2 * e], a1 = E[2 * e + 1];
    const double w = o.earea ? -0.25 * __ldg(o.earea + e) : -1.0;
    const V3 xp = load_v3(V, p), xa0 = load_v3(V, a0), xa1 = load_v3(V, a1);
    const int pe = point_edge_distance_type(xp, xa0, xa1);
    int nonmollified = 0;
    for (int j = ve_off[p], je = ve_off[p + 1]; j < je; ++j) {
        const int eb = ve_adj[j];
        const int b0 = E[2 * eb], b1 = E[2 * eb + 1];
        const int q = p == b0 ? b1 : b0;
        if (q == a0 || q == a1) continue;
        const double eps_x = ee_mollifier_threshold(load_v3(rest, a0), load_v3(rest, a1), load_v3(rest, b0),
            load_v3(rest, b1));
        const double cr = ee_cross_sqnorm(xa0, xa1, load_v3(V, b0), load_v3(V, b1));
        if (cr >= eps_x) {
            ++nonmollified;
            continue;
        }
        const bool first = p == b0;
        const int dt = pe == P_E0 ? (first ? EA0_EB0 : EA0_EB1)
                                  : (pe == P_E1 ? (first ? EA1_EB0 : EA1_EB1) : (first ? EA_EB0 : EA_EB1));
        const int s = append(o.count + 2);
        o.ee[s] = key2(e, eb);
        o.ee_rec[s] = s;
        o.ee_eps[s] = eps_x;
        o.ee_dt[s] = (int8_t)dt;
        o.ee_w[s] = w;
    }
    if (nonmollified == 1) return;
    put_typed(o, E, e, p, pe, (nonmollified - 1) * w);
}

// add_face_vertex_negative_edge_vertex_collision (builder.cpp:421-455)
__global__ void k_imp_fv_negative(const unsigned long long* __restrict__ l2, int n, const double* __restrict__ V,
    const int* __restrict__ E, const int* __restrict__ ev_off, const int* __restrict__ ev_adj, Out o)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const unsigned long long k = l2[i];
    const int e = (int)(k >> 32), v = (int)(k & 0xffffffffu);
    const int lo = ev_off[e], hi = ev_off[e + 1];
    const int amt = (hi - lo) - (sorted_contains(ev_adj, lo, hi, v) ? 1 : 0);
    if (amt <= 1) return;
    const double w = (1 - amt) * (o.varea ? 0.25 * __ldg(o.varea + v) : 1.0);
    const int pe = point_edge_distance_type(load_v3(V, v), load_v3(V, E[2 * e]), load_v3(V, E[2 * e + 1]));
    put_typed(o, E, e, v, pe, w);
}

// add_face_vertex_positive_vertex_vertex_collision (builder.cpp:382-419)
__global__ void k_imp_fv_positive(const unsigned long long* __restrict__ l3, int n, const int* __restrict__ vv_off,
    const int* __restrict__ vv_adj, const uint8_t* __restrict__ boundary, Out o)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const unsigned long long k = l3[i];
    const int a = (int)(k >> 32), b = (int)(k & 0xffffffffu);
    double w = 0;
    const int vi[2] = { a, b }, vj[2] = { b, a };
    for (int t = 0; t < 2; ++t) {
        if (boundary[vj[t]] || sorted_contains(vv_adj, vv_off[vj[t]], vv_off[vj[t] + 1], vi[t])) continue;
        w += o.varea ? 0.25 * __ldg(o.varea + vi[t]) : 1.0;
    }
    if (w != 0) put_vv(o, a, b, w);
}

// EE merge of the improved set: records are equal when their edges match as
// an unordered pair and their types match (normal/edge_edge.cpp:123-142).
// Composite key (min, max, type); weights summed in ascending order; the
// merged record keeps the orientation and eps_x of a record with ea < eb
// when there is one.
__global__ void k_ee_group_keys(const unsigned long long* __restrict__ pair, const int8_t* __restrict__ dt,
    const double* __restrict__ w, int n, int bits, unsigned long long* __restrict__ ck, unsigned long long* __restrict__ wk,
    int* __restrict__ idx)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const unsigned long long k = pair[i];
    const unsigned a = (unsigned)(k >> 32), b = (unsigned)(k & 0xffffffffu);
    const unsigned long long lo = min(a, b), hi = max(a, b);
    ck[i] = (((lo << bits) | hi) << 4) | (unsigned long long)(uint8_t)dt[i];
    wk[i] = weight_key(w[i]);
    idx[i] = i;
}
__global__ void k_ee_group_runs(const int* __restrict__ counts, const int* __restrict__ offs,
    const int* __restrict__ d_num, const int* __restrict__ idx, const unsigned long long* __restrict__ pair,
    const double* __restrict__ eps, const int8_t* __restrict__ dt, const double* __restrict__ w,
    int2* __restrict__ ids_out, double* __restrict__ eps_out, int8_t* __restrict__ dt_out, double* __restrict__ w_out,
    int* __restrict__ keep)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= *d_num) return;
    int rep = idx[offs[i]];
    bool rep_sorted = (pair[rep] >> 32) < (pair[rep] & 0xffffffffu);
    double sum = 0.0;
    for (int j = offs[i], e = offs[i] + counts[i]; j < e; ++j) {
        const int q = idx[j];
        sum += w[q];
        if (!rep_sorted && (pair[q] >> 32) < (pair[q] & 0xffffffffu)) {
            rep = q;
            rep_sorted = true;
        }
    }
    const unsigned long long k = pair[rep];
    ids_out[i] = make_int2((int)(k >> 32), (int)(k & 0xffffffffu));
    eps_out[i] = eps[rep];
    dt_out[i] = dt[rep];
    w_out[i] = sum;
    keep[i] = sum != 0 ? 1 : 0;
}

__global__ void k_gather_src(const int2* __restrict__ src, const int* __restrict__ idx, int n, int2* __restrict__ out)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = src[idx[i]];
}

// Zero-weight removal (builder.cpp:666-688): keep[i] -> compacted slot offs[i].
__global__ void k_flag_nonzero(const double* __restrict__ w, const int* __restrict__ d_num, int* __restrict__ keep)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= *d_num) return;
    keep[i] = w[i] != 0 ? 1 : 0;
}
__global__ void k_compact(const int* __restrict__ d_num, const int* __restrict__ keep, const int* __restrict__ offs,
    const int2* __restrict__ ids, const double* __restrict__ w, const double* __restrict__ eps,
    const int8_t* __restrict__ dt, int2* __restrict__ ids_out, double* __restrict__ w_out, double* __restrict__ eps_out,
    int8_t* __restrict__ dt_out, int* __restrict__ n_out)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int n = *d_num;
    if (i == 0) *n_out = n > 0 ? offs[n - 1] + keep[n - 1] : 0;
    if (i >= n || !keep[i]) return;
    const int o = offs[i];
    ids_out[o] = ids[i];
    w_out[o] = w[i];
    if (eps) eps_out[o] = eps[i];
    if (dt) dt_out[o] = dt[i];
}

} // namespace

// The improved set's EE group key packs (min edge, max edge, type) in 64 bits.
static void require_ee_bits(const ipcg_mesh* m)
{
    if (2 * bits_for(std::max(m->nE, (int64_t)2)) + 4 > 64)
        throw Error(IPCG_ERR_INVALID, "IMPROVED_MAX_APPROX supports at most 2^30 edges");
}

// CollisionMesh::init_adjacencies (collision_mesh.cpp:247-291) on the host,
// uploaded as CSR lists; built the first time a build needs them.
void ensure_adjacency(ipcg_mesh* m)
{
    if (m->adj_ready) return;
    const int64_t nV = m->nV, nE = m->nE, nF = m->nF;
    std::vector<int32_t> E(2 * nE), F(3 * nF);
    if (nE) IPCG_CUDA(cudaMemcpy(E.data(), m->E.p, sizeof(int32_t) * 2 * nE, cudaMemcpyDeviceToHost));
    if (nF) IPCG_CUDA(cudaMemcpy(F.data(), m->F.p, sizeof(int32_t) * 3 * nF, cudaMemcpyDeviceToHost));
    auto csr = [](std::vector<std::pair<int32_t, int32_t>>& pairs, int64_t rows, std::vector<int32_t>& off,
                   std::vector<int32_t>& adj) {
        std::sort(pairs.begin(), pairs.end());
        pairs.erase(std::unique(pairs.begin(), pairs.end()), pairs.end());
        off.assign(rows + 1, 0);
        adj.resize(pairs.size());
        for (size_t i = 0; i < pairs.size(); ++i) {
            ++off[pairs[i].first + 1];
            adj[i] = pairs[i].second;
        }
        for (int64_t r = 0; r < rows; ++r) off[r + 1] += off[r];
    };
    std::vector<std::pair<int32_t, int32_t>> vv, ve, ev;
    vv.reserve(2 * nE);
    ve.reserve(2 * nE);
    ev.reserve(3 * nF);
    for (int64_t e = 0; e < nE; ++e) {
        vv.emplace_back(E[2 * e], E[2 * e + 1]);
        vv.emplace_back(E[2 * e + 1], E[2 * e]);
        ve.emplace_back(E[2 * e], (int32_t)e);
        ve.emplace_back(E[2 * e + 1], (int32_t)e);
    }
    for (int64_t f = 0; f < nF; ++f)
        for (int j = 0; j < 3; ++j) ev.emplace_back(m->h_F2E[3 * f + j], F[3 * f + (j + 2) % 3]);
    std::vector<std::pair<int32_t, int32_t>> vf, ef;
    vf.reserve(3 * nF);
    ef.reserve(3 * nF);
    for (int64_t f = 0; f < nF; ++f)
        for (int j = 0; j < 3; ++j) {
            vf.emplace_back(F[3 * f + j], (int32_t)f);
            ef.emplace_back(m->h_F2E[3 * f + j], (int32_t)f);
        }
    std::vector<int32_t> vv_off, vv_adj, ve_off, ve_adj, ev_off, ev_adj, vf_off, vf_adj, ef_off, ef_adj;
    csr(vv, nV, vv_off, vv_adj);
    csr(ve, nV, ve_off, ve_adj);
    csr(ev, nE, ev_off, ev_adj);
    csr(vf, nV, vf_off, vf_adj);
    csr(ef, nE, ef_off, ef_adj);
    std::vector<uint8_t> boundary(nV, 1);
    for (int64_t e = 0; e < nE; ++e)
        if (ev_off[e + 1] - ev_off[e] >= 2) boundary[E[2 * e]] = boundary[E[2 * e + 1]] = 0;
    int maxdeg = 0;
    for (int64_t v = 0; v < nV; ++v) maxdeg = std::max(maxdeg, ve_off[v + 1] - ve_off[v]);
    auto up = [&](auto& buf, const auto& host) {
        buf.reserve(host.size() + 1);
        if (!host.empty())
            IPCG_CUDA(cudaMemcpy(buf.p, host.data(), sizeof(host[0]) * host.size(), cudaMemcpyHostToDevice));
    };
    up(m->vv_off, vv_off);
    up(m->vv_adj, vv_adj);
    up(m->ve_off, ve_off);
    up(m->ve_adj, ve_adj);
    up(m->ev_off, ev_off);
    up(m->ev_adj, ev_adj);
    up(m->vf_off, vf_off);
    up(m->vf_adj, vf_adj);
    up(m->ef_off, ef_off);
    up(m->ef_adj, ef_adj);
    up(m->boundary, boundary);
    m->max_vertex_edges = maxdeg;
    m->adj_ready = true;
}

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
    ++c->version;
    c->built_with_shape = c->enable_shape_derivatives;
    const int64_t nc = n_ee + n_fv;
    const bool improved = c->set_type == 1;
    // improved max approximation: candidate conversions (sorted, unique keys)
    int64_t nl1 = 0, nl2 = 0, nl3 = 0;
    unsigned long long *l1 = nullptr, *l2 = nullptr, *l3 = nullptr;
    if (improved) {
        require_ee_bits(m);
        ensure_adjacency(m);
        const int64_t r1 = 4 * n_ee, r23 = 3 * n_fv, tot = r1 + 2 * r23 + 16;
        m->imp_keys.reserve(2 * tot);
        unsigned long long* raw = m->imp_keys.p;
        unsigned long long* srt = m->imp_keys.p + tot;
        l1 = raw;
        l2 = raw + r1;
        l3 = raw + r1 + r23;
        m->counters.reserve(32);
        int* kc = m->counters.p + 20;
        IPCG_CUDA(cudaMemsetAsync(kc, 0, sizeof(int) * 8, s));
        const SceneView sv0 = scene_view(m);
        if (n_ee)
            IPCG_LAUNCH("k_imp_ee_to_ev", s, k_imp_ee_to_ev<<<grid_for(n_ee, BLOCK), BLOCK, 0, s>>>(m->cand.p,
                (int)n_ee, V, m->E.p, m->scene_off2.p, sv0, l1, kc + 0));
        if (n_fv)
            IPCG_LAUNCH("k_imp_fv_to_ev_vv", s, k_imp_fv_to_ev_vv<<<grid_for(n_fv, BLOCK), BLOCK, 0, s>>>(
                m->cand.p + m->cand_cap, (int)n_fv, V, m->E.p, m->F.p, m->F2E.p, m->scene_off2.p, sv0, l2, kc + 1,
                l3, kc + 2));
        m->h_counters.reserve(32);
        IPCG_CUDA(cudaMemcpyAsync(m->h_counters.p, kc, sizeof(int) * 3, cudaMemcpyDeviceToHost, s));
        IPCG_CUDA(cudaStreamSynchronize(s));
        const int k1 = m->h_counters.p[0], k2 = m->h_counters.p[1], k3 = m->h_counters.p[2];
        const int kbits = 32 + bits_for(std::max(std::max(m->nV, m->nE), (int64_t)2));
        sort_keys_u64(m, s, l1, srt, k1, kbits);
        unique_u64(m, s, srt, l1, kc + 3, k1);
        sort_keys_u64(m, s, l2, srt + r1, k2, kbits);
        unique_u64(m, s, srt + r1, l2, kc + 4, k2);
        sort_keys_u64(m, s, l3, srt + r1 + r23, k3, kbits);
        unique_u64(m, s, srt + r1 + r23, l3, kc + 5, k3);
        IPCG_CUDA(cudaMemcpyAsync(m->h_counters.p, kc + 3, sizeof(int) * 3, cudaMemcpyDeviceToHost, s));
        IPCG_CUDA(cudaStreamSynchronize(s));
        nl1 = k1 ? m->h_counters.p[0] : 0;
        nl2 = k2 ? m->h_counters.p[1] : 0;
        nl3 = k3 ? m->h_counters.p[2] : 0;
    }
    // raw records: at most one per candidate, plus the improved terms
    const int64_t cap = nc + (improved ? nl1 * (m->max_vertex_edges + 1) + nl2 + nl3 : 0) + 16;
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
    const bool area = c->use_area_weighting != 0;
    const bool weighted = area || improved; // VV / EV records carry weights
    o.vv_w = o.ev_w = o.ee_w = nullptr;
    o.varea = area ? m->vertex_area.p : nullptr;
    o.earea = area ? m->edge_area.p : nullptr;
    if (weighted) {
        m->rec_w.reserve(2 * cap);
        o.vv_w = m->rec_w.p;
        o.ev_w = m->rec_w.p + cap;
    }
    if (improved) {
        m->rec_ee_w.reserve(cap);
        o.ee_w = m->rec_ee_w.p;
    }
    o.vv_src = o.ev_src = nullptr;
    o.src = make_int2(-1, -1);
    c->built_with_area = area ? 1 : 0;
    if (area && c->enable_shape_derivatives && !improved) {
        m->rec_src.reserve(2 * cap);
        o.vv_src = m->rec_src.p;
        o.ev_src = m->rec_src.p + cap;
    }
    m->counters.reserve(32);
    m->h_counters.reserve(32);
    o.count = m->counters.p + 4;
    IPCG_CUDA(cudaMemsetAsync(o.count, 0, sizeof(int) * 8, s));
    const SceneView sv = scene_view(m);
    if (n_ee)
        IPCG_LAUNCH("k_filter_ee", s, k_filter_ee<<<grid_for(n_ee, BLOCK), BLOCK, 0, s>>>(m->cand.p, (int)n_ee, V,
            m->rest.p, m->E.p, m->scene_off2.p, sv, o));
    if (n_fv)
        IPCG_LAUNCH("k_filter_fv", s, k_filter_fv<<<grid_for(n_fv, BLOCK), BLOCK, 0, s>>>(m->cand.p + m->cand_cap,
            (int)n_fv, V, m->F.p, m->F2E.p, m->scene_off2.p, sv, o));
    if (improved) {
        if (nl1)
            IPCG_LAUNCH("k_imp_ee_negative", s, k_imp_ee_negative<<<grid_for(nl1, BLOCK), BLOCK, 0, s>>>(l1, (int)nl1,
                V, m->rest.p, m->E.p, m->ve_off.p, m->ve_adj.p, o));
        if (nl2)
            IPCG_LAUNCH("k_imp_fv_negative", s, k_imp_fv_negative<<<grid_for(nl2, BLOCK), BLOCK, 0, s>>>(l2, (int)nl2,
                V, m->E.p, m->ev_off.p, m->ev_adj.p, o));
        if (nl3)
            IPCG_LAUNCH("k_imp_fv_positive", s, k_imp_fv_positive<<<grid_for(nl3, BLOCK), BLOCK, 0, s>>>(l3,
                (int)nl3, m->vv_off.p, m->vv_adj.p, m->boundary.p, o));
    }
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
        const int2* src_raw = nullptr;
        DBuf<int2>* src_out = nullptr;
        DBuf<int>* src_off = nullptr;
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
            IPCG_CUDA(cudaMemsetAsync(cnt, 0, sizeof(int) * (n + 1), s));
            rle_u64(m, m->stream, sorted, raw, cnt, num, n);
            // n + 1 offsets: past the last run they all equal n
            exclusive_sum_i32(m, m->stream, cnt, i0, n + 1);
            IPCG_LAUNCH("k_sum_runs", s, k_sum_runs<<<grid_for(n, BLOCK), BLOCK, 0, s>>>(raw, cnt, i0, num, i2, w,
                ids, wout));
            if (src_raw) {
                // keep each merged record's weight sources (in merge order)
                src_out->reserve(n + 1);
                src_off->reserve(n + 2);
                IPCG_LAUNCH("k_gather_src", s, k_gather_src<<<grid_for(n, BLOCK), BLOCK, 0, s>>>(src_raw, i2, n,
                    src_out->p));
                IPCG_CUDA(cudaMemcpyAsync(src_off->p, i0, sizeof(int) * (n + 1), cudaMemcpyDeviceToDevice, s));
            }
        };
        if (!improved) {
            if (o.vv_src) {
                src_raw = o.vv_src;
                src_out = &c->vv_src;
                src_off = &c->vv_src_off;
            }
            merge(o.vv, o.vv_w, rvv, ks, counts, d_num + 0, c->vv.p, c->vv_w.p);
            if (o.ev_src) {
                src_raw = o.ev_src;
                src_out = &c->ev_src;
                src_off = &c->ev_src_off;
            }
            merge(o.ev, o.ev_w, rev, ks + cap, counts + cap, d_num + 1, c->ev.p, c->ev_w.p);
            src_raw = nullptr;
        } else {
            // sums that cancel to zero are dropped (builder.cpp:666-688)
            m->imp_ids.reserve(cap);
            m->imp_w.reserve(cap);
            m->imp_flag.reserve(cap);
            m->imp_offs.reserve(cap);
            auto merge_drop = [&](unsigned long long* raw, const double* w, int n, unsigned long long* sorted,
                                  int* cnt, int* num, int2* ids, double* wout, int* n_out) {
                merge(raw, w, n, sorted, cnt, num, m->imp_ids.p, m->imp_w.p);
                if (n == 0) {
                    IPCG_CUDA(cudaMemsetAsync(n_out, 0, sizeof(int), s));
                    return;
                }
                IPCG_CUDA(cudaMemsetAsync(m->imp_flag.p, 0, sizeof(int) * n, s));
                IPCG_LAUNCH("k_flag_nonzero", s, k_flag_nonzero<<<grid_for(n, BLOCK), BLOCK, 0, s>>>(m->imp_w.p, num,
                    m->imp_flag.p));
                exclusive_sum_i32(m, m->stream, m->imp_flag.p, m->imp_offs.p, n);
                IPCG_LAUNCH("k_compact", s, k_compact<<<grid_for(n, BLOCK), BLOCK, 0, s>>>(num, m->imp_flag.p,
                    m->imp_offs.p, m->imp_ids.p, m->imp_w.p, nullptr, nullptr, ids, wout, nullptr, nullptr, n_out));
            };
            // compacted counts go to their own slots: k_compact reads the run
            // count while it writes the kept count
            merge_drop(o.vv, o.vv_w, rvv, ks, counts, d_num + 0, c->vv.p, c->vv_w.p, d_num + 4);
            merge_drop(o.ev, o.ev_w, rev, ks + cap, counts + cap, d_num + 1, c->ev.p, c->ev_w.p, d_num + 5);
        }
    }
    // EE: sort keys with record ids, gather eps / dtype
    c->ee.reserve(ree + 1);
    c->ee_w.reserve(ree + 1);
    c->ee_eps.reserve(ree + 1);
    c->ee_dtype.reserve(ree + 1);
    int nee_out = ree;
    if (ree && improved) {
        // group equal (unordered pair, type) records, sum their weights in
        // ascending order, drop zero sums
        const int ebits = bits_for(std::max(m->nE, (int64_t)2));
        m->wkeys.reserve(2 * cap);
        unsigned long long* ck = m->wkeys.p;
        unsigned long long* wk = m->wkeys.p + cap;
        m->widx.reserve(3 * cap);
        int *i0 = m->widx.p, *i1 = m->widx.p + cap, *i2 = m->widx.p + 2 * cap;
        unsigned long long* sorted = ks + 2 * cap;
        IPCG_LAUNCH("k_ee_group_keys", s, k_ee_group_keys<<<grid_for(ree, BLOCK), BLOCK, 0, s>>>(o.ee, o.ee_dt,
            o.ee_w, ree, ebits, ck, wk, i0));
        sort_pairs_u64(m, m->stream, wk, sorted, i0, i1, ree, 64);
        IPCG_LAUNCH("k_gather_keys", s, k_gather_keys<<<grid_for(ree, BLOCK), BLOCK, 0, s>>>(ck, i1, ree, wk));
        sort_pairs_u64(m, m->stream, wk, sorted, i1, i2, ree, 2 * ebits + 4);
        int* ecnt = m->ivals_b.p + 2 * cap;
        IPCG_CUDA(cudaMemsetAsync(ecnt, 0, sizeof(int) * ree, s));
        rle_u64(m, m->stream, sorted, ck, ecnt, d_num + 2, ree);
        exclusive_sum_i32(m, m->stream, ecnt, i0, ree);
        m->imp_ids.reserve(cap);
        m->imp_w.reserve(cap);
        m->imp_eps.reserve(cap);
        m->imp_dt.reserve(cap);
        m->imp_flag.reserve(cap);
        m->imp_offs.reserve(cap);
        IPCG_CUDA(cudaMemsetAsync(m->imp_flag.p, 0, sizeof(int) * ree, s));
        IPCG_LAUNCH("k_ee_group_runs", s, k_ee_group_runs<<<grid_for(ree, BLOCK), BLOCK, 0, s>>>(ecnt, i0, d_num + 2,
            i2, o.ee, o.ee_eps, o.ee_dt, o.ee_w, m->imp_ids.p, m->imp_eps.p, m->imp_dt.p, m->imp_w.p, m->imp_flag.p));
        exclusive_sum_i32(m, m->stream, m->imp_flag.p, m->imp_offs.p, ree);
        IPCG_LAUNCH("k_compact", s, k_compact<<<grid_for(ree, BLOCK), BLOCK, 0, s>>>(d_num + 2, m->imp_flag.p,
            m->imp_offs.p, m->imp_ids.p, m->imp_w.p, m->imp_eps.p, m->imp_dt.p, c->ee.p, c->ee_w.p, c->ee_eps.p,
            c->ee_dtype.p, d_num + 3));
        nee_out = -1; // read back below
    } else if (ree) {
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
    IPCG_CUDA(cudaMemcpyAsync(m->h_counters.p, d_num, sizeof(int) * 6, cudaMemcpyDeviceToHost, s));
    IPCG_CUDA(cudaStreamSynchronize(s));
    c->nvv = improved ? m->h_counters.p[4] : m->h_counters.p[0];
    c->nev = improved ? m->h_counters.p[5] : m->h_counters.p[1];
    c->nee = nee_out >= 0 ? nee_out : m->h_counters.p[3];
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
