// broad_phase.cu — device LBVH broad phase.
//
// Restates the reference's default broad phase (src/ipc/broad_phase/lbvh.cpp)
// for the GPU: per-vertex boxes inflated outward with nextafter
// (aabb.cpp:35-126), edge/face boxes as unions, FP32 node boxes rounded
// outward (lbvh.cpp:29-41), Morton order, a Karras radix tree with atomic
// bottom-up refit, and one-thread-per-query stack traversal emitting
// candidates with warp-aggregated appends.  EE uses the triangular
// self-traversal (lbvh.cpp:409-418) and FV queries vertex boxes against the
// face tree (lbvh.cpp:756-769); both reject stencils that share a vertex
// (lbvh.cpp:810-834).
#include <cooperative_groups.h>

#include <cfloat>

#include "geom.cuh"
#include "internal.cuh"
#include "predicates.cuh"
#include "profile.cuh"

namespace cg = cooperative_groups;

namespace ipcg {

namespace {

constexpr int BLOCK = 256;
constexpr int STACK = 64;

__device__ __forceinline__ void vertex_box(const double* V0, const double* V1, int v, const double* scene_r,
    SceneView sv, double mn[3], double mx[3])
{
    const double r = __ldg(scene_r + sv.of(v));
    for (int d = 0; d < 3; ++d) {
        double a = V0[3 * v + d], b = a;
        if (V1) {
            const double c = V1[3 * v + d];
            a = fmin(a, c);
            b = fmax(b, c);
        }
        mn[d] = nextafter(a - r, __longlong_as_double(0xfff0000000000000ULL));
        mx[d] = nextafter(b + r, __longlong_as_double(0x7ff0000000000000ULL));
    }
}

__global__ void k_bounds_partial(const double* __restrict__ V0, const double* __restrict__ V1, int nV,
    double* __restrict__ partial)
{
    double mn[3] = { DBL_MAX, DBL_MAX, DBL_MAX }, mx[3] = { -DBL_MAX, -DBL_MAX, -DBL_MAX };
    for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < nV; v += gridDim.x * blockDim.x)
        for (int d = 0; d < 3; ++d) {
            double a = V0[3 * v + d];
            mn[d] = fmin(mn[d], a);
            mx[d] = fmax(mx[d], a);
            if (V1) {
                a = V1[3 * v + d];
                mn[d] = fmin(mn[d], a);
                mx[d] = fmax(mx[d], a);
            }
        }
    __shared__ double s[6][BLOCK];
    for (int d = 0; d < 3; ++d) {
        s[d][threadIdx.x] = mn[d];
        s[3 + d][threadIdx.x] = mx[d];
    }
    __syncthreads();
    for (int w = BLOCK / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w)
            for (int d = 0; d < 3; ++d) {
                s[d][threadIdx.x] = fmin(s[d][threadIdx.x], s[d][threadIdx.x + w]);
                s[3 + d][threadIdx.x] = fmax(s[3 + d][threadIdx.x], s[3 + d][threadIdx.x + w]);
            }
        __syncthreads();
    }
    if (threadIdx.x < 6) partial[6 * blockIdx.x + threadIdx.x] = s[threadIdx.x][0];
}

__global__ void k_bounds_final(double* __restrict__ partial, int nblocks)
{
    // single thread: few hundred partials
    if (threadIdx.x != 0) return;
    double b[6] = { DBL_MAX, DBL_MAX, DBL_MAX, -DBL_MAX, -DBL_MAX, -DBL_MAX };
    for (int i = 0; i < nblocks; ++i)
        for (int d = 0; d < 3; ++d) {
            b[d] = fmin(b[d], partial[6 * i + d]);
            b[3 + d] = fmax(b[3 + d], partial[6 * i + 3 + d]);
        }
    for (int d = 0; d < 6; ++d) partial[d] = b[d];
}

__device__ __forceinline__ unsigned spread10(unsigned x)
{
    x &= 0x3ff;
    x = (x | (x << 16)) & 0x030000FF;
    x = (x | (x << 8)) & 0x0300F00F;
    x = (x | (x << 4)) & 0x030C30C3;
    x = (x | (x << 2)) & 0x09249249;
    return x;
}

template <int K>
__global__ void k_prim_boxes(const int* __restrict__ ids, int n, const double* __restrict__ V0,
    const double* __restrict__ V1, const double* __restrict__ scene_r, SceneView sv,
    const double* __restrict__ bounds, float4* __restrict__ plo, float4* __restrict__ phi,
    unsigned long long* __restrict__ codes, int* __restrict__ order)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double mn[3] = { DBL_MAX, DBL_MAX, DBL_MAX }, mx[3] = { -DBL_MAX, -DBL_MAX, -DBL_MAX };
    for (int k = 0; k < K; ++k) {
        double a[3], b[3];
        vertex_box(V0, V1, ids[K * i + k], scene_r, sv, a, b);
        for (int d = 0; d < 3; ++d) {
            mn[d] = fmin(mn[d], a[d]);
            mx[d] = fmax(mx[d], b[d]);
        }
    }
    plo[i] = make_float4(__double2float_rd(mn[0]), __double2float_rd(mn[1]), __double2float_rd(mn[2]), 0.f);
    phi[i] = make_float4(__double2float_ru(mx[0]), __double2float_ru(mx[1]), __double2float_ru(mx[2]), 0.f);
    unsigned q[3];
    for (int d = 0; d < 3; ++d) {
        const double ext = bounds[3 + d] - bounds[d];
        double c = ext > 0 ? (0.5 * (mn[d] + mx[d]) - bounds[d]) / ext : 0.0;
        c = fmin(fmax(c * 1024.0, 0.0), 1023.0);
        q[d] = (unsigned)c;
    }
    const unsigned morton = (spread10(q[0]) << 2) | (spread10(q[1]) << 1) | spread10(q[2]);
    codes[i] = ((unsigned long long)sv.of(ids[K * i]) << 32) | morton;
    order[i] = i;
}

__device__ __forceinline__ int delta(const unsigned long long* __restrict__ c, int n, int i, int j)
{
    if (j < 0 || j >= n) return -1;
    const unsigned long long a = c[i], b = c[j];
    if (a == b) return 64 + __clz(i ^ j);
    return __clzll(a ^ b);
}

// Karras (2012) radix-tree construction, one thread per internal node.
__global__ void k_karras(const unsigned long long* __restrict__ c, int n, float4* __restrict__ lo,
    float4* __restrict__ hi, int* __restrict__ first, int* __restrict__ last, int* __restrict__ parent)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n - 1) return;
    const int dir = (delta(c, n, i, i + 1) - delta(c, n, i, i - 1)) >= 0 ? 1 : -1;
    const int dmin = delta(c, n, i, i - dir);
    int lmax = 2;
    while (delta(c, n, i, i + lmax * dir) > dmin) lmax *= 2;
    int l = 0;
    for (int t = lmax / 2; t >= 1; t /= 2)
        if (delta(c, n, i, i + (l + t) * dir) > dmin) l += t;
    const int j = i + l * dir;
    const int dnode = delta(c, n, i, j);
    int s = 0, t = l;
    do {
        t = (t + 1) / 2;
        if (delta(c, n, i, i + (s + t) * dir) > dnode) s += t;
    } while (t > 1);
    const int gamma = i + s * dir + min(dir, 0);
    const int lo_i = min(i, j), hi_i = max(i, j);
    const int left = (lo_i == gamma) ? (n - 1 + gamma) : gamma;
    const int right = (hi_i == gamma + 1) ? (n - 1 + gamma + 1) : gamma + 1;
    lo[i].w = __int_as_float(left);
    hi[i].w = __int_as_float(right);
    first[i] = lo_i;
    last[i] = hi_i;
    parent[left] = i;
    parent[right] = i;
    if (i == 0) parent[0] = -1;
}

__global__ void k_leaves(const int* __restrict__ ids_sorted, const unsigned long long* __restrict__ codes_sorted,
    int n, const float4* __restrict__ plo, const float4* __restrict__ phi, float4* __restrict__ lo,
    float4* __restrict__ hi, int* __restrict__ first, int* __restrict__ last, int* __restrict__ parent,
    int* __restrict__ leaf_scene)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int p = ids_sorted[i];
    leaf_scene[i] = (int)(codes_sorted[i] >> 32);
    first[n - 1 + i] = i;
    float4 a = plo[p], b = phi[p];
    a.w = __int_as_float(p);
    b.w = __int_as_float(-1);
    lo[n - 1 + i] = a;
    hi[n - 1 + i] = b;
    last[n - 1 + i] = i;
    if (n == 1) parent[0] = -1;
}

// Bottom-up refit: the second thread to reach a node merges its children.
__global__ void k_refit(int n, float4* lo, float4* hi, const int* __restrict__ parent, int* flags)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int node = parent[n - 1 + i];
    while (node >= 0) {
        __threadfence();
        if (atomicAdd(flags + node, 1) == 0) return;
        __threadfence();
        const float4 nlo = __ldcg(lo + node), nhi = __ldcg(hi + node);
        const int l = __float_as_int(nlo.w), r = __float_as_int(nhi.w);
        const float4 a0 = __ldcg(lo + l), a1 = __ldcg(hi + l), b0 = __ldcg(lo + r), b1 = __ldcg(hi + r);
        __stcg(lo + node, make_float4(fminf(a0.x, b0.x), fminf(a0.y, b0.y), fminf(a0.z, b0.z), nlo.w));
        __stcg(hi + node, make_float4(fmaxf(a1.x, b1.x), fmaxf(a1.y, b1.y), fmaxf(a1.z, b1.z), nhi.w));
        node = parent[node];
    }
}

__device__ __forceinline__ bool overlap(float4 alo, float4 ahi, float4 blo, float4 bhi)
{
    return alo.x <= bhi.x && blo.x <= ahi.x && alo.y <= bhi.y && blo.y <= ahi.y && alo.z <= bhi.z && blo.z <= ahi.z;
}

__device__ __forceinline__ void emit(int2* __restrict__ out, int* __restrict__ count, int cap, int2 val)
{
    cg::coalesced_group g = cg::coalesced_threads();
    int base = 0;
    if (g.thread_rank() == 0) base = atomicAdd(count, (int)g.size());
    base = g.shfl(base, 0) + (int)g.thread_rank();
    if (base < cap) out[base] = val;
}

// EE: triangular self traversal, one thread per sorted edge leaf.
// Scene range check of node v for a query in scene qs (batches only).
__device__ __forceinline__ bool other_scenes(const int* __restrict__ first, const int* __restrict__ last,
    const int* __restrict__ leaf_scene, bool batched, int v, int qs)
{
    return batched && (qs < __ldg(leaf_scene + __ldg(first + v)) || qs > __ldg(leaf_scene + __ldg(last + v)));
}

__global__ void k_traverse_ee(const float4* __restrict__ lo, const float4* __restrict__ hi,
    const int* __restrict__ first, const int* __restrict__ last, const int* __restrict__ leaf_scene, bool batched,
    int n, const int* __restrict__ E, int2* __restrict__ out, int* __restrict__ count, int cap,
    int* __restrict__ guard)
{
    const int qi = blockIdx.x * blockDim.x + threadIdx.x;
    if (qi >= n || n < 2) return;
    const float4 qlo = lo[n - 1 + qi], qhi = hi[n - 1 + qi];
    const int ea = __float_as_int(qlo.w);
    const int a0 = E[2 * ea], a1 = E[2 * ea + 1];
    const int qs = leaf_scene[qi];
    int stack[STACK];
    int sp = 0;
    stack[sp++] = 0;
    while (sp > 0) {
        const int v = stack[--sp];
        if (last[v] <= qi) continue;
        if (other_scenes(first, last, leaf_scene, batched, v, qs)) continue;
        const float4 vlo = lo[v], vhi = hi[v];
        if (!overlap(qlo, qhi, vlo, vhi)) continue;
        if (v >= n - 1) {
            const int eb = __float_as_int(vlo.w);
            const int b0 = E[2 * eb], b1 = E[2 * eb + 1];
            if (a0 != b0 && a0 != b1 && a1 != b0 && a1 != b1) emit(out, count, cap, make_int2(min(ea, eb), max(ea, eb)));
        } else {
            if (sp + 2 > STACK) {
                atomicOr(guard, GUARD_STACK);
                return;
            }
            stack[sp++] = __float_as_int(vhi.w);
            stack[sp++] = __float_as_int(vlo.w);
        }
    }
}

// FV: each vertex box queries the face tree.
__global__ void k_traverse_fv(const float4* __restrict__ lo, const float4* __restrict__ hi,
    const int* __restrict__ first, const int* __restrict__ last, const int* __restrict__ leaf_scene, int n,
    const double* __restrict__ V0, const double* __restrict__ V1, const double* __restrict__ scene_r, SceneView sv,
    int nV, const int* __restrict__ F, int2* __restrict__ out, int* __restrict__ count, int cap,
    int* __restrict__ guard)
{
    const int vi = blockIdx.x * blockDim.x + threadIdx.x;
    if (vi >= nV || n < 1) return;
    double mn[3], mx[3];
    vertex_box(V0, V1, vi, scene_r, sv, mn, mx);
    const int qs = sv.of(vi);
    const bool batched = sv.vscene != nullptr;
    const float4 qlo = make_float4(__double2float_rd(mn[0]), __double2float_rd(mn[1]), __double2float_rd(mn[2]), 0.f);
    const float4 qhi = make_float4(__double2float_ru(mx[0]), __double2float_ru(mx[1]), __double2float_ru(mx[2]), 0.f);
    int stack[STACK];
    int sp = 0;
    stack[sp++] = 0;
    while (sp > 0) {
        const int v = stack[--sp];
        if (other_scenes(first, last, leaf_scene, batched, v, qs)) continue;
        const float4 vlo = lo[v], vhi = hi[v];
        if (!overlap(qlo, qhi, vlo, vhi)) continue;
        if (v >= n - 1) {
            const int f = __float_as_int(vlo.w);
            if (F[3 * f] != vi && F[3 * f + 1] != vi && F[3 * f + 2] != vi) emit(out, count, cap, make_int2(f, vi));
        } else {
            if (sp + 2 > STACK) {
                atomicOr(guard, GUARD_STACK);
                return;
            }
            stack[sp++] = __float_as_int(vhi.w);
            stack[sp++] = __float_as_int(vlo.w);
        }
    }
}

// has_intersections (ipc.cpp:110-167): every edge (a leaf of the edge
// tree) queries the face tree; pairs sharing a vertex are skipped
// (broad_phase.cpp:164-179) and the others get the exact edge-triangle test.
// The first intersection sets *found, which every thread polls so the
// search stops early.
__global__ void k_edges_cross_faces(const float4* __restrict__ elo, const float4* __restrict__ ehi, int ne,
    const float4* __restrict__ flo, const float4* __restrict__ fhi, const int* __restrict__ ffirst,
    const int* __restrict__ flast, const int* __restrict__ leaf_scene, SceneView sv, int nf,
    const int* __restrict__ E, const int* __restrict__ F, const double* __restrict__ V, int* found, int* guard)
{
    const int qi = blockIdx.x * blockDim.x + threadIdx.x;
    if (qi >= ne || nf < 1) return;
    const float4 qlo = elo[ne - 1 + qi], qhi = ehi[ne - 1 + qi];
    const int e = __float_as_int(qlo.w);
    const int a0 = E[2 * e], a1 = E[2 * e + 1];
    const int qs = sv.of(a0);
    const bool batched = sv.vscene != nullptr;
    const V3 e0 = load_v3(V, a0), e1 = load_v3(V, a1);
    int stack[STACK];
    int sp = 0;
    stack[sp++] = 0;
    int visits = 0;
    while (sp > 0) {
        if ((++visits & 31) == 0 && *(volatile int*)found) return;
        const int v = stack[--sp];
        if (other_scenes(ffirst, flast, leaf_scene, batched, v, qs)) continue;
        const float4 vlo = flo[v], vhi = fhi[v];
        if (!overlap(qlo, qhi, vlo, vhi)) continue;
        if (v >= nf - 1) {
            const int f = __float_as_int(vlo.w);
            const int b0 = F[3 * f], b1 = F[3 * f + 1], b2 = F[3 * f + 2];
            if (a0 == b0 || a0 == b1 || a0 == b2 || a1 == b0 || a1 == b1 || a1 == b2) continue;
            if (exact::edge_intersects_triangle(e0, e1, load_v3(V, b0), load_v3(V, b1), load_v3(V, b2))) {
                atomicExch(found, 1);
                return;
            }
        } else {
            if (sp + 2 > STACK) {
                atomicOr(guard, GUARD_STACK);
                return;
            }
            stack[sp++] = __float_as_int(vhi.w);
            stack[sp++] = __float_as_int(vlo.w);
        }
    }
}

} // namespace

void build_lbvh(ipcg_mesh* m, LBVH& bvh, int kind, const double* V0, const double* V1, const double* scene_r)
{
    const int n = (int)(kind == 2 ? m->nE : m->nF);
    bvh.n = n;
    if (n == 0) return;
    const int nn = 2 * n - 1;
    bvh.lo.reserve(nn);
    bvh.hi.reserve(nn);
    bvh.first.reserve(nn);
    bvh.last.reserve(nn);
    bvh.parent.reserve(nn);
    bvh.flags.reserve(n);
    bvh.leaf_scene.reserve(n);
    bvh.codes.reserve(n);
    bvh.codes_sorted.reserve(n);
    bvh.ids.reserve(n);
    bvh.ids_sorted.reserve(n);
    bvh.plo.reserve(n);
    bvh.phi.reserve(n);
    cudaStream_t s = m->stream;
    const SceneView sv = scene_view(m);
    if (kind == 2)
        IPCG_LAUNCH("k_prim_boxes", s, k_prim_boxes<2><<<grid_for(n, BLOCK), BLOCK, 0, s>>>(m->E.p, n, V0, V1,
            scene_r, sv, m->bounds.p, bvh.plo.p, bvh.phi.p, bvh.codes.p, bvh.ids.p));
    else
        IPCG_LAUNCH("k_prim_boxes", s, k_prim_boxes<3><<<grid_for(n, BLOCK), BLOCK, 0, s>>>(m->F.p, n, V0, V1,
            scene_r, sv, m->bounds.p, bvh.plo.p, bvh.phi.p, bvh.codes.p, bvh.ids.p));
    sort_pairs_u64(m, m->stream, bvh.codes.p, bvh.codes_sorted.p, bvh.ids.p, bvh.ids_sorted.p, n,
        32 + bits_for(m->n_scenes + 1));
    if (n > 1)
        IPCG_LAUNCH("k_karras", s, k_karras<<<grid_for(n - 1, BLOCK), BLOCK, 0, s>>>(bvh.codes_sorted.p, n, bvh.lo.p,
            bvh.hi.p, bvh.first.p, bvh.last.p, bvh.parent.p));
    IPCG_LAUNCH("k_leaves", s, k_leaves<<<grid_for(n, BLOCK), BLOCK, 0, s>>>(bvh.ids_sorted.p, bvh.codes_sorted.p, n,
        bvh.plo.p, bvh.phi.p, bvh.lo.p, bvh.hi.p, bvh.first.p, bvh.last.p, bvh.parent.p, bvh.leaf_scene.p));
    if (n > 1) {
        IPCG_CUDA(cudaMemsetAsync(bvh.flags.p, 0, sizeof(int) * (n - 1), s));
        IPCG_LAUNCH("k_refit", s, k_refit<<<grid_for(n, BLOCK), BLOCK, 0, s>>>(n, bvh.lo.p, bvh.hi.p, bvh.parent.p,
            bvh.flags.p));
    }
}

bool has_intersections(ipcg_mesh* m, const double* V)
{
    cudaStream_t s = m->stream;
    const int nV = (int)m->nV;
    if (m->nE == 0 || m->nF == 0) return false;
    // boxes inflated by 1e-6 of the bounding-box diagonal (ipc.cpp:127-128)
    const int nb = 256;
    m->bounds.reserve(6 * nb);
    IPCG_LAUNCH("k_bounds_partial", s, k_bounds_partial<<<nb, BLOCK, 0, s>>>(V, V, nV, m->bounds.p));
    IPCG_LAUNCH("k_bounds_final", s, k_bounds_final<<<1, 32, 0, s>>>(m->bounds.p, nb));
    double b[6];
    IPCG_CUDA(cudaMemcpyAsync(b, m->bounds.p, sizeof(b), cudaMemcpyDeviceToHost, s));
    IPCG_CUDA(cudaStreamSynchronize(s));
    const double dx = b[3] - b[0], dy = b[4] - b[1], dz = b[5] - b[2];
    const int ns = (int)m->n_scenes;
    std::vector<double> r(ns, 1e-6 * sqrt(dx * dx + dy * dy + dz * dz));
    m->scene_r.reserve(ns);
    IPCG_CUDA(cudaMemcpyAsync(m->scene_r.p, r.data(), sizeof(double) * ns, cudaMemcpyHostToDevice, s));
    build_lbvh(m, m->ebvh, 2, V, V, m->scene_r.p);
    build_lbvh(m, m->fbvh, 3, V, V, m->scene_r.p);
    m->counters.reserve(8);
    m->h_counters.reserve(8);
    IPCG_CUDA(cudaMemsetAsync(m->counters.p, 0, sizeof(int) * 8, s));
    const SceneView sv = scene_view(m);
    IPCG_LAUNCH("k_edges_cross_faces", s, k_edges_cross_faces<<<grid_for(m->ebvh.n, 128), 128, 0, s>>>(m->ebvh.lo.p,
        m->ebvh.hi.p, m->ebvh.n, m->fbvh.lo.p, m->fbvh.hi.p, m->fbvh.first.p, m->fbvh.last.p, m->fbvh.leaf_scene.p,
        sv, m->fbvh.n, m->E.p, m->F.p, V, m->counters.p + 0, m->counters.p + 2));
    IPCG_CUDA(cudaMemcpyAsync(m->h_counters.p, m->counters.p, sizeof(int) * 3, cudaMemcpyDeviceToHost, s));
    IPCG_CUDA(cudaStreamSynchronize(s));
    if (m->h_counters.p[2] & GUARD_STACK) throw Error(IPCG_ERR_CUDA, "LBVH traversal stack overflow");
    return m->h_counters.p[0] != 0;
}

void detect_candidates(ipcg_mesh* m, const double* V0, const double* V1, const double* scene_r, int64_t& n_ee,
    int64_t& n_fv)
{
    cudaStream_t s = m->stream;
    const int nV = (int)m->nV;
    // mesh bounds for the Morton normalisation
    const int nb = 256;
    m->bounds.reserve(6 * nb);
    IPCG_LAUNCH("k_bounds_partial", s, k_bounds_partial<<<nb, BLOCK, 0, s>>>(V0, V1, nV, m->bounds.p));
    IPCG_LAUNCH("k_bounds_final", s, k_bounds_final<<<1, 32, 0, s>>>(m->bounds.p, nb));
    IPCG_CHECK_LAUNCH();
    build_lbvh(m, m->ebvh, 2, V0, V1, scene_r);
    build_lbvh(m, m->fbvh, 3, V0, V1, scene_r);
    const SceneView sv = scene_view(m);
    const bool batched = sv.vscene != nullptr;
    m->counters.reserve(8);
    m->h_counters.reserve(8);
    if (m->cand_cap == 0) m->cand_cap = 4 * (m->nE + m->nV) + 1024;
    for (int attempt = 0; attempt < 8; ++attempt) {
        const int64_t cap = m->cand_cap; // per region
        m->cand.reserve(2 * cap);
        IPCG_CUDA(cudaMemsetAsync(m->counters.p, 0, sizeof(int) * 8, s));
        const int icap = (int)std::min<int64_t>(cap, INT32_MAX);
        if (m->ebvh.n >= 2)
            IPCG_LAUNCH("k_traverse_ee", s, k_traverse_ee<<<grid_for(m->ebvh.n, 128), 128, 0, s>>>(m->ebvh.lo.p,
                m->ebvh.hi.p, m->ebvh.first.p, m->ebvh.last.p, m->ebvh.leaf_scene.p, batched, m->ebvh.n, m->E.p,
                m->cand.p, m->counters.p + 0, icap, m->counters.p + 2));
        if (m->fbvh.n >= 1 && nV > 0)
            IPCG_LAUNCH("k_traverse_fv", s, k_traverse_fv<<<grid_for(nV, 128), 128, 0, s>>>(m->fbvh.lo.p,
                m->fbvh.hi.p, m->fbvh.first.p, m->fbvh.last.p, m->fbvh.leaf_scene.p, m->fbvh.n, V0, V1, scene_r, sv,
                nV, m->F.p, m->cand.p + cap, m->counters.p + 1, icap, m->counters.p + 2));
        IPCG_CHECK_LAUNCH();
        IPCG_CUDA(cudaMemcpyAsync(m->h_counters.p, m->counters.p, sizeof(int) * 3, cudaMemcpyDeviceToHost, s));
        IPCG_CUDA(cudaStreamSynchronize(s));
        if (m->h_counters.p[2] & GUARD_STACK) throw Error(IPCG_ERR_CUDA, "LBVH traversal stack overflow");
        const int64_t ce = (unsigned)m->h_counters.p[0], cf = (unsigned)m->h_counters.p[1];
        if (ce <= cap && cf <= cap) {
            n_ee = ce;
            n_fv = cf;
            return;
        }
        m->cand_cap = std::max(ce, cf) + std::max(ce, cf) / 2 + 1024;
    }
    throw Error(IPCG_ERR_OOM, "candidate buffer could not be sized");
}

} // namespace ipcg
