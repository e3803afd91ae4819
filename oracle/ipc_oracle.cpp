// ipc_oracle.cpp — CPU restatement of IPC Toolkit's contact hot path.
//
// TEST INFRASTRUCTURE ONLY.  This file is the checker for the GPU library:
// only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load
// it.  Nothing in the product links or calls it.
//
// It restates, in plain C++17 (no Eigen/TBB), the reference algorithms of
// ipc-sim/ipc-toolkit v1.6.0 for:
//   * collision-mesh topology     src/ipc/collision_mesh.cpp:510-543
//   * AABB inflation + LBVH       src/ipc/broad_phase/aabb.cpp:35-126,
//                                 src/ipc/broad_phase/lbvh.cpp:29-330,368-455
//   * distance types / distances  src/ipc/distance/distance_type.cpp:10-211,
//                                 point_point.cpp:5-9, point_line.cpp:5-23,
//                                 point_plane.cpp:10-26, line_line.cpp:7-16,
//                                 point_triangle.cpp:11-48, edge_edge.cpp:13-56
//   * collision-set build         src/ipc/collisions/normal/normal_collisions.cpp:20-158,
//                                 normal_collisions_builder.cpp:26-336,547-689
//   * barrier potential E/G/H     src/ipc/barrier/barrier.cpp:11-43,
//                                 src/ipc/potentials/barrier_potential.cpp:62-99,
//                                 normal_potential.cpp:127-232, potential.cpp:36-222
//   * PSD projection              src/ipc/utils/eigen_ext.tpp:64-108 (own Jacobi solver)
//   * collision-free step size    src/ipc/ipc.cpp:42-106, candidates.cpp:252-292,
//                                 src/ipc/ccd/tight_inclusion_ccd.cpp:33-336
//     with an inclusion-based root finder restated from the published
//     Tight-Inclusion method (Wang et al., ACM TOG 2021; the library
//     Tight-Inclusion v1.0.6 is not vendored in the reference).
//
// Floating point: every expression is evaluated unfused and left to right,
// as an SSE2 build of the reference evaluates Eigen's 3-vector reductions
// ((x0*y0 + x1*y1) + x2*y2).  Build with -ffp-contract=off.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <limits>
#include <mutex>
#include <map>
#include <numeric>
#include <thread>
#include <unordered_map>
#include <queue>
#include <tuple>
#include <vector>

namespace orc {

// ---------------------------------------------------------------------------
// 3-vectors
// ---------------------------------------------------------------------------
struct V3 {
    double x, y, z;
};
static inline V3 sub(V3 a, V3 b) { return { a.x - b.x, a.y - b.y, a.z - b.z }; }
static inline V3 add(V3 a, V3 b) { return { a.x + b.x, a.y + b.y, a.z + b.z }; }
static inline V3 scale(V3 a, double s) { return { a.x * s, a.y * s, a.z * s }; }
static inline double dot(V3 a, V3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
static inline double sqnorm(V3 a) { return dot(a, a); }
static inline V3 cross(V3 a, V3 b)
{
    return { a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x };
}
static inline double comp(V3 a, int i) { return i == 0 ? a.x : (i == 1 ? a.y : a.z); }
static inline V3 row(const double* V, int64_t i) { return { V[3 * i], V[3 * i + 1], V[3 * i + 2] }; }

// ---------------------------------------------------------------------------
// Distance types (src/ipc/distance/distance_type.hpp enum order)
// ---------------------------------------------------------------------------
enum PE { P_E0 = 0, P_E1 = 1, P_E = 2 };
enum PT { P_T0 = 0, P_T1, P_T2, P_E0t, P_E1t, P_E2t, P_T };
enum EE { EA0_EB0 = 0, EA0_EB1, EA1_EB0, EA1_EB1, EA_EB0, EA_EB1, EA0_EB, EA1_EB, EA_EB };

// distance_type.cpp:10-34
static int point_edge_distance_type(V3 p, V3 e0, V3 e1)
{
    const V3 e = sub(e1, e0);
    const double e_length_sqr = sqnorm(e);
    if (e_length_sqr == 0) return P_E0;
    const double ratio = dot(e, sub(p, e0)) / e_length_sqr;
    if (ratio < 0) return P_E0;
    if (ratio > 1) return P_E1;
    return P_E;
}

// Solve (B Bᵀ) x = B r for the 2×3 basis B=[b0;b1] with the pivoted LDLᵀ
// factorisation used by distance_type.cpp:48,55,62 (diagonal pivoting on the
// larger diagonal, unit-lower L, D⁻¹ with a DBL_MIN cutoff).
static void ldlt2_solve(V3 b0, V3 b1, V3 r, double& x0, double& x1)
{
    double a00 = dot(b0, b0);
    double a10 = dot(b1, b0);
    double a11 = dot(b1, b1);
    double y0 = dot(b0, r), y1 = dot(b1, r);
    bool swapped = false;
    if (std::fabs(a11) > std::fabs(a00)) {
        std::swap(a00, a11);
        swapped = true;
        std::swap(y0, y1);
    }
    const double d0 = a00;
    double l10 = a10;
    if (d0 == 0.0) {
        // Whole diagonal zero: factorisation stops with L = I, D = 0.
        x0 = 0;
        x1 = 0;
        return;
    }
    l10 = a10 / d0;
    const double d1 = a11 - l10 * (d0 * l10);
    // forward: L y = P b
    y1 = y1 - l10 * y0;
    // diagonal (pseudo-inverse with DBL_MIN tolerance)
    const double tiny = std::numeric_limits<double>::min();
    y0 = (std::fabs(d0) > tiny) ? y0 / d0 : 0.0;
    y1 = (std::fabs(d1) > tiny) ? y1 / d1 : 0.0;
    // backward: Lᵀ x = y
    y0 = y0 - l10 * y1;
    if (swapped) std::swap(y0, y1);
    x0 = y0;
    x1 = y1;
}

// distance_type.cpp:36-79
static int point_triangle_distance_type(V3 p, V3 t0, V3 t1, V3 t2)
{
    const V3 normal = cross(sub(t1, t0), sub(t2, t0));
    double param0[3], param1[3];
    V3 b0, b1;

    b0 = sub(t1, t0);
    b1 = cross(b0, normal);
    ldlt2_solve(b0, b1, sub(p, t0), param0[0], param1[0]);
    if (param0[0] > 0.0 && param0[0] < 1.0 && param1[0] >= 0.0) return P_E0t;

    b0 = sub(t2, t1);
    b1 = cross(b0, normal);
    ldlt2_solve(b0, b1, sub(p, t1), param0[1], param1[1]);
    if (param0[1] > 0.0 && param0[1] < 1.0 && param1[1] >= 0.0) return P_E1t;

    b0 = sub(t0, t2);
    b1 = cross(b0, normal);
    ldlt2_solve(b0, b1, sub(p, t2), param0[2], param1[2]);
    if (param0[2] > 0.0 && param0[2] < 1.0 && param1[2] >= 0.0) return P_E2t;

    if (param0[0] <= 0.0 && param0[2] >= 1.0) return P_T0;
    if (param0[1] <= 0.0 && param0[0] >= 1.0) return P_T1;
    if (param0[2] <= 0.0 && param0[1] >= 1.0) return P_T2;
    return P_T;
}

// distance_type.cpp:176-211
static int edge_edge_parallel_distance_type(V3 ea0, V3 ea1, V3 eb0, V3 eb1)
{
    const V3 ea = sub(ea1, ea0);
    const double alpha = dot(sub(eb0, ea0), ea) / sqnorm(ea);
    const double beta = dot(sub(eb1, ea0), ea) / sqnorm(ea);
    int eac, ebc;
    if (alpha < 0) {
        eac = (0 <= beta && beta <= 1) ? 2 : 0;
        ebc = (beta <= alpha) ? 0 : (beta <= 1 ? 1 : 2);
    } else if (alpha > 1) {
        eac = (0 <= beta && beta <= 1) ? 2 : 1;
        ebc = (beta >= alpha) ? 0 : (0 <= beta ? 1 : 2);
    } else {
        eac = 2;
        ebc = 0;
    }
    return ebc < 2 ? ((eac << 1) | ebc) : (6 + eac);
}

// distance_type.cpp:82-174
static int edge_edge_distance_type(V3 ea0, V3 ea1, V3 eb0, V3 eb1)
{
    const double PARALLEL_THRESHOLD = 2.5e-16;
    const V3 u = sub(ea1, ea0), v = sub(eb1, eb0), w = sub(ea0, eb0);
    const double a = sqnorm(u), b = dot(u, v), c = sqnorm(v), d = dot(u, w), e = dot(v, w);
    const double D = a * c - b * b;
    if (a == 0.0 && c == 0.0) return EA0_EB0;
    if (a == 0.0) return EA0_EB;
    if (c == 0.0) return EA_EB0;
    const double parallel_tolerance = PARALLEL_THRESHOLD * a * c;
    if (sqnorm(cross(u, v)) < parallel_tolerance)
        return edge_edge_parallel_distance_type(ea0, ea1, eb0, eb1);

    int default_case = EA_EB;
    const double sN = (b * e - c * d);
    double tN, tD;
    if (sN <= 0.0) {
        tN = e;
        tD = c;
        default_case = EA0_EB;
    } else if (sN >= D) {
        tN = e + b;
        tD = c;
        default_case = EA1_EB;
    } else {
        tN = (a * e - b * d);
        tD = D;
        if (tN > 0.0 && tN < tD && sqnorm(cross(u, v)) < parallel_tolerance) {
            if (sN < D / 2) {
                tN = e;
                tD = c;
                default_case = EA0_EB;
            } else {
                tN = e + b;
                tD = c;
                default_case = EA1_EB;
            }
        }
    }
    if (tN <= 0.0) {
        if (-d <= 0.0) return EA0_EB0;
        if (-d >= a) return EA1_EB0;
        return EA_EB0;
    } else if (tN >= tD) {
        if ((-d + b) <= 0.0) return EA0_EB1;
        if ((-d + b) >= a) return EA1_EB1;
        return EA_EB1;
    }
    return default_case;
}

// ---------------------------------------------------------------------------
// Squared distances
// ---------------------------------------------------------------------------
static double point_point_distance(V3 p0, V3 p1) { return sqnorm(sub(p1, p0)); }   // point_point.cpp:5-9
static double point_line_distance(V3 p, V3 e0, V3 e1)                              // point_line.cpp:19-21
{
    return sqnorm(cross(sub(e0, p), sub(e1, p))) / sqnorm(sub(e1, e0));
}
static V3 triangle_normal(V3 a, V3 b, V3 c)                                       // normal.hpp:149-168
{
    const V3 n = cross(sub(b, a), sub(c, a));
    const double z = sqnorm(n);
    if (z > 0) {
        const double s = std::sqrt(z);
        return { n.x / s, n.y / s, n.z / s };
    }
    return n;
}
static double point_plane_distance(V3 p, V3 t0, V3 t1, V3 t2)                     // point_plane.cpp:10-26
{
    const V3 n = triangle_normal(t0, t1, t2);
    const double ptp = dot(sub(p, t0), n);
    return ptp * ptp / sqnorm(n);
}
static double line_line_distance(V3 ea0, V3 ea1, V3 eb0, V3 eb1)                  // line_line.cpp:7-16
{
    const V3 n = cross(sub(ea1, ea0), sub(eb1, eb0));
    const double ltl = dot(sub(eb0, ea0), n);
    return ltl * ltl / sqnorm(n);
}
static double point_triangle_distance(V3 p, V3 t0, V3 t1, V3 t2, int dtype)       // point_triangle.cpp:11-48
{
    switch (dtype) {
    case P_T0: return point_point_distance(p, t0);
    case P_T1: return point_point_distance(p, t1);
    case P_T2: return point_point_distance(p, t2);
    case P_E0t: return point_line_distance(p, t0, t1);
    case P_E1t: return point_line_distance(p, t1, t2);
    case P_E2t: return point_line_distance(p, t2, t0);
    default: return point_plane_distance(p, t0, t1, t2);
    }
}
static double edge_edge_distance(V3 ea0, V3 ea1, V3 eb0, V3 eb1, int dtype)         // edge_edge.cpp:13-56
{
    switch (dtype) {
    case EA0_EB0: return point_point_distance(ea0, eb0);
    case EA0_EB1: return point_point_distance(ea0, eb1);
    case EA1_EB0: return point_point_distance(ea1, eb0);
    case EA1_EB1: return point_point_distance(ea1, eb1);
    case EA_EB0: return point_line_distance(eb0, ea0, ea1);
    case EA_EB1: return point_line_distance(eb1, ea0, ea1);
    case EA0_EB: return point_line_distance(ea0, eb0, eb1);
    case EA1_EB: return point_line_distance(ea1, eb0, eb1);
    default: return line_line_distance(ea0, ea1, eb0, eb1);
    }
}
static double point_edge_distance(V3 p, V3 e0, V3 e1, int dtype)                  // point_edge.cpp:10-38
{
    switch (dtype) {
    case P_E0: return point_point_distance(p, e0);
    case P_E1: return point_point_distance(p, e1);
    default: return point_line_distance(p, e0, e1);
    }
}
// edge_edge_mollifier.cpp:7-14, 194-202
static double ee_cross_sqnorm(V3 ea0, V3 ea1, V3 eb0, V3 eb1) { return sqnorm(cross(sub(ea1, ea0), sub(eb1, eb0))); }
static double ee_mollifier_threshold(V3 ea0, V3 ea1, V3 eb0, V3 eb1)
{
    return 1e-3 * sqnorm(sub(ea0, ea1)) * sqnorm(sub(eb0, eb1));
}

// ---------------------------------------------------------------------------
// Boxes and LBVH (aabb.cpp:35-126; lbvh.cpp)
// ---------------------------------------------------------------------------
struct Box {
    double mn[3], mx[3];
};
static inline double down(double v) { return std::nextafter(v, -std::numeric_limits<double>::infinity()); }
static inline double up(double v) { return std::nextafter(v, std::numeric_limits<double>::infinity()); }

static void vertex_boxes_static(const double* V, int64_t nV, double r, std::vector<Box>& out)
{
    out.resize(nV);
    for (int64_t i = 0; i < nV; ++i)
        for (int d = 0; d < 3; ++d) {
            out[i].mn[d] = down(V[3 * i + d] - r);
            out[i].mx[d] = up(V[3 * i + d] + r);
        }
}
static void vertex_boxes_dynamic(const double* V0, const double* V1, int64_t nV, double r, std::vector<Box>& out)
{
    out.resize(nV);
    for (int64_t i = 0; i < nV; ++i)
        for (int d = 0; d < 3; ++d) {
            const double a = V0[3 * i + d], b = V1[3 * i + d];
            out[i].mn[d] = down(std::min(a, b) - r);
            out[i].mx[d] = up(std::max(a, b) + r);
        }
}
static void prim_boxes(const std::vector<Box>& vb, const int32_t* ids, int64_t n, int k, std::vector<Box>& out)
{
    out.resize(n);
    for (int64_t i = 0; i < n; ++i) {
        Box b = vb[ids[k * i]];
        for (int j = 1; j < k; ++j) {
            const Box& c = vb[ids[k * i + j]];
            for (int d = 0; d < 3; ++d) {
                b.mn[d] = std::min(b.mn[d], c.mn[d]);
                b.mx[d] = std::max(b.mx[d], c.mx[d]);
            }
        }
        out[i] = b;
    }
}

// FP32 node with outward rounding (lbvh.cpp:29-41)
struct FBox {
    float mn[3], mx[3];
};
static inline float f_down(double v)
{
    float f = (float)v;
    if ((double)f > v) f = std::nextafter(f, -std::numeric_limits<float>::infinity());
    return f;
}
static inline float f_up(double v)
{
    float f = (float)v;
    if ((double)f < v) f = std::nextafter(f, std::numeric_limits<float>::infinity());
    return f;
}
static inline FBox to_fbox(const Box& b)
{
    FBox f;
    for (int d = 0; d < 3; ++d) {
        f.mn[d] = f_down(b.mn[d]);
        f.mx[d] = f_up(b.mx[d]);
    }
    return f;
}
static inline bool overlap(const FBox& a, const FBox& b)
{
    return a.mn[0] <= b.mx[0] && b.mn[0] <= a.mx[0] && a.mn[1] <= b.mx[1] && b.mn[1] <= a.mx[1]
        && a.mn[2] <= b.mx[2] && b.mn[2] <= a.mx[2];
}

// 21-bit-per-axis Morton code (morton.hpp:53-62 semantics: clamp to [0,2^21-1])
static inline uint64_t spread21(uint64_t x)
{
    x &= 0x1fffff;
    x = (x | x << 32) & 0x1f00000000ffffULL;
    x = (x | x << 16) & 0x1f0000ff0000ffULL;
    x = (x | x << 8) & 0x100f00f00f00f00fULL;
    x = (x | x << 4) & 0x10c30c30c30c30c3ULL;
    x = (x | x << 2) & 0x1249249249249249ULL;
    return x;
}
static inline uint64_t morton63(double x, double y, double z)
{
    auto q = [](double t) -> uint64_t {
        double s = t * 2097152.0;
        if (!(s > 0)) s = 0;
        if (s > 2097151.0) s = 2097151.0;
        return (uint64_t)s;
    };
    return (spread21(q(x)) << 2) | (spread21(q(y)) << 1) | spread21(q(z));
}

// Karras (2012) radix-tree LBVH over sorted Morton codes.  Internal nodes
// 0..n-2, leaves n-1..2n-2 in sorted order.  Each node records the sorted
// leaf range it covers so that triangular self-traversal can skip subtrees
// entirely to the left of the query (lbvh.cpp:409-418).
struct LBVH {
    int n = 0;
    std::vector<FBox> box;       // 2n-1
    std::vector<int> left, right; // children (internal nodes only)
    std::vector<int> last;       // rightmost sorted leaf index of each subtree
    std::vector<int> prim;       // sorted position -> primitive id
};

static void build_lbvh(const std::vector<Box>& boxes, const double mesh_min[3], const double mesh_max[3], LBVH& bvh)
{
    const int n = (int)boxes.size();
    bvh.n = n;
    bvh.box.assign(n > 0 ? 2 * n - 1 : 0, FBox {});
    bvh.left.assign(n > 1 ? n - 1 : 0, -1);
    bvh.right.assign(n > 1 ? n - 1 : 0, -1);
    bvh.last.assign(n > 0 ? 2 * n - 1 : 0, 0);
    bvh.prim.resize(n);
    if (n == 0) return;
    std::vector<uint64_t> code(n);
    double ext[3];
    for (int d = 0; d < 3; ++d) ext[d] = mesh_max[d] - mesh_min[d];
    for (int i = 0; i < n; ++i) {
        double c[3];
        for (int d = 0; d < 3; ++d) {
            const double mid = 0.5 * (boxes[i].mn[d] + boxes[i].mx[d]);
            c[d] = ext[d] > 0 ? (mid - mesh_min[d]) / ext[d] : 0.0;
        }
        code[i] = morton63(c[0], c[1], c[2]);
    }
    std::iota(bvh.prim.begin(), bvh.prim.end(), 0);
    std::stable_sort(bvh.prim.begin(), bvh.prim.end(), [&](int a, int b) { return code[a] < code[b]; });
    std::vector<uint64_t> sc(n);
    for (int i = 0; i < n; ++i) sc[i] = code[bvh.prim[i]];
    for (int i = 0; i < n; ++i) {
        bvh.box[n - 1 + i] = to_fbox(boxes[bvh.prim[i]]);
        bvh.last[n - 1 + i] = i;
    }
    if (n == 1) return;
    // delta(i,j): common-prefix length of the (code, index) keys; -1 outside
    auto delta_safe = [&](int i, int j) -> int {
        if (j < 0 || j >= n) return -1;
        if (sc[i] == sc[j]) return 64 + __builtin_clz((unsigned)(i ^ j));
        return __builtin_clzll(sc[i] ^ sc[j]);
    };
    for (int i = 0; i < n - 1; ++i) {
        const int dir = (delta_safe(i, i + 1) - delta_safe(i, i - 1)) >= 0 ? 1 : -1;
        const int dmin = delta_safe(i, i - dir);
        int lmax = 2;
        while (delta_safe(i, i + lmax * dir) > dmin) lmax *= 2;
        int l = 0;
        for (int t = lmax / 2; t >= 1; t /= 2)
            if (delta_safe(i, i + (l + t) * dir) > dmin) l += t;
        const int j = i + l * dir;
        const int dnode = delta_safe(i, j);
        int s = 0;
        int t = l;
        do {
            t = (t + 1) / 2;
            if (delta_safe(i, i + (s + t) * dir) > dnode) s += t;
        } while (t > 1);
        const int gamma = i + s * dir + std::min(dir, 0);
        const int lo = std::min(i, j), hi = std::max(i, j);
        bvh.left[i] = (lo == gamma) ? (n - 1 + gamma) : gamma;
        bvh.right[i] = (hi == gamma + 1) ? (n - 1 + gamma + 1) : gamma + 1;
        bvh.last[i] = hi;
    }
    // bottom-up boxes: post-order via explicit stack from the root (node 0)
    std::vector<int> order;
    order.reserve(n - 1);
    std::vector<int> st { 0 };
    while (!st.empty()) {
        int v = st.back();
        st.pop_back();
        order.push_back(v);
        if (bvh.left[v] < n - 1) st.push_back(bvh.left[v]);
        if (bvh.right[v] < n - 1) st.push_back(bvh.right[v]);
    }
    for (auto it = order.rbegin(); it != order.rend(); ++it) {
        const int v = *it;
        const FBox& a = bvh.box[bvh.left[v]];
        const FBox& b = bvh.box[bvh.right[v]];
        FBox& c = bvh.box[v];
        for (int d = 0; d < 3; ++d) {
            c.mn[d] = std::min(a.mn[d], b.mn[d]);
            c.mx[d] = std::max(a.mx[d], b.mx[d]);
        }
    }
}

// Visit every leaf whose box overlaps q; triangular => only leaves with sorted
// index > qi.  cb(primitive_id).
template <typename F>
static void traverse(const LBVH& bvh, const FBox& q, int qi, bool triangular, F&& cb)
{
    const int n = bvh.n;
    if (n == 0) return;
    if (n == 1) {
        if (!triangular && overlap(bvh.box[0], q)) cb(bvh.prim[0]);
        return;
    }
    int stack[128];
    int sp = 0;
    stack[sp++] = 0;
    while (sp) {
        const int v = stack[--sp];
        if (triangular && bvh.last[v] <= qi) continue;
        if (!overlap(bvh.box[v], q)) continue;
        if (v >= n - 1) {
            const int li = v - (n - 1);
            if (!triangular || li > qi) cb(bvh.prim[li]);
        } else {
            if (sp + 2 > 128) std::abort();
            stack[sp++] = bvh.right[v];
            stack[sp++] = bvh.left[v];
        }
    }
}

static void mesh_aabb(const std::vector<Box>& vb, double mn[3], double mx[3])
{
    for (int d = 0; d < 3; ++d) {
        mn[d] = std::numeric_limits<double>::max();
        mx[d] = std::numeric_limits<double>::lowest();
    }
    for (const Box& b : vb)
        for (int d = 0; d < 3; ++d) {
            mn[d] = std::min(mn[d], b.mn[d]);
            mx[d] = std::max(mx[d], b.mx[d]);
        }
}

template <typename F>
static void parallel_for(int64_t n, int nthreads, F&& f)
{
    if (nthreads <= 1 || n < 1024) {
        f(0, n, 0);
        return;
    }
    std::vector<std::thread> th;
    std::atomic<int64_t> next { 0 };
    const int64_t chunk = std::max<int64_t>(256, n / (nthreads * 16));
    for (int t = 0; t < nthreads; ++t)
        th.emplace_back([&, t] {
            for (;;) {
                const int64_t b = next.fetch_add(chunk);
                if (b >= n) break;
                f(b, std::min(n, b + chunk), t);
            }
        });
    for (auto& x : th) x.join();
}

struct Candidates {
    std::vector<int32_t> ee; // pairs (ea, eb) with ea < eb
    std::vector<int32_t> fv; // pairs (f, v)
};

// BroadPhase::detect_collision_candidates in 3D (broad_phase.cpp:79-91):
// EE by triangular self-traversal, FV by vertex queries into the face BVH,
// with the shared-vertex filters of lbvh.cpp:810-834.
static void detect_candidates(const std::vector<Box>& vb, const int32_t* E, int64_t nE, const int32_t* F, int64_t nF,
    int nthreads, Candidates& out)
{
    std::vector<Box> eb, fb;
    prim_boxes(vb, E, nE, 2, eb);
    prim_boxes(vb, F, nF, 3, fb);
    double mn[3], mx[3];
    mesh_aabb(vb, mn, mx);
    LBVH ebvh, fbvh;
    build_lbvh(eb, mn, mx, ebvh);
    build_lbvh(fb, mn, mx, fbvh);
    const int nt = std::max(1, nthreads);
    std::vector<std::vector<int32_t>> ee_local(nt), fv_local(nt);
    parallel_for(nE, nt, [&](int64_t b, int64_t e, int t) {
        for (int64_t qi = b; qi < e; ++qi) {
            const int ea = ebvh.prim[qi];
            const FBox& q = ebvh.box[ebvh.n - 1 + qi];
            traverse(ebvh, q, (int)qi, true, [&](int ebi) {
                const int a0 = E[2 * ea], a1 = E[2 * ea + 1], b0 = E[2 * ebi], b1 = E[2 * ebi + 1];
                if (a0 == b0 || a0 == b1 || a1 == b0 || a1 == b1) return;
                ee_local[t].push_back(std::min(ea, ebi));
                ee_local[t].push_back(std::max(ea, ebi));
            });
        }
    });
    const int64_t nV = (int64_t)vb.size();
    parallel_for(nV, nt, [&](int64_t b, int64_t e, int t) {
        for (int64_t vi = b; vi < e; ++vi) {
            const FBox q = to_fbox(vb[vi]);
            traverse(fbvh, q, -1, false, [&](int fi) {
                if (F[3 * fi] == vi || F[3 * fi + 1] == vi || F[3 * fi + 2] == vi) return;
                fv_local[t].push_back(fi);
                fv_local[t].push_back((int32_t)vi);
            });
        }
    });
    out.ee.clear();
    out.fv.clear();
    for (int t = 0; t < nt; ++t) {
        out.ee.insert(out.ee.end(), ee_local[t].begin(), ee_local[t].end());
        out.fv.insert(out.fv.end(), fv_local[t].begin(), fv_local[t].end());
    }
}

// ---------------------------------------------------------------------------
// Collision set (normal_collisions_builder.cpp)
// ---------------------------------------------------------------------------
struct Collisions {
    std::vector<int32_t> vv;   // (v0 < v1)
    std::vector<double> vv_w;
    std::vector<int32_t> ev;   // (e, v)
    std::vector<double> ev_w;
    std::vector<int32_t> ee;   // (ea < eb)
    std::vector<double> ee_eps;
    std::vector<int8_t> ee_dtype;
    std::vector<double> ee_w;
    std::vector<int32_t> fv;   // (f, v)
    std::vector<double> fv_w;
    std::vector<int32_t> cand; // last candidate set: ee pairs then fv pairs
    int64_t n_cand_ee = 0, n_cand_fv = 0;
    // weight sources of each merged VV / EV record (area weighting): a face-
    // vertex candidate's vertex (v, -1) or an edge-edge candidate's edges
    // (ea, eb), in the record's merge order; offsets per record
    std::vector<int64_t> vv_src_off, ev_src_off;
    std::vector<int32_t> vv_src, ev_src;
};

struct Raw {
    std::vector<uint64_t> vv, ev;
    std::vector<double> vv_w, ev_w;
    std::vector<int32_t> vv_src, ev_src; // pairs: the weight source of each record
    std::vector<int32_t> ee;
    std::vector<double> ee_eps, ee_w;
    std::vector<int8_t> ee_dt;
    std::vector<int32_t> fv;
    std::vector<double> fv_w;
};

// Per-vertex and per-edge areas of the rest mesh (collision_mesh.cpp:309-374):
// a vertex takes 1/3 of each incident face's area, else 1/2 of each incident
// edge's length, else 1; an edge takes 1/3 of each incident face's area, else
// its length.  Sums run in face (edge) order, as the reference's loops do.
static void mesh_areas(const double* R, int64_t nV, const int32_t* E, int64_t nE, const int32_t* F, int64_t nF,
    const int32_t* F2E, double* va, double* ea)
{
    std::vector<double> vea(nV, -1.0), vfa(nV, -1.0);
    auto len = [&](int64_t e) { return std::sqrt(sqnorm(sub(row(R, E[2 * e + 1]), row(R, E[2 * e])))); };
    for (int64_t i = 0; i < nE; ++i) {
        const double l = len(i);
        for (int j = 0; j < 2; ++j) {
            double& a = vea[E[2 * i + j]];
            a = std::max(a, 0.0);
            a += 0.5 * l;
        }
    }
    for (int64_t i = 0; i < nE; ++i) ea[i] = -1.0;
    for (int64_t i = 0; i < nF; ++i) {
        const V3 t0 = row(R, F[3 * i]), t1 = row(R, F[3 * i + 1]), t2 = row(R, F[3 * i + 2]);
        const double fa = 0.5 * std::sqrt(sqnorm(cross(sub(t1, t0), sub(t2, t0))));
        for (int j = 0; j < 3; ++j) {
            double& a = vfa[F[3 * i + j]];
            a = std::max(a, 0.0);
            a += fa / 3.0;
            double& b = ea[F2E[3 * i + j]];
            b = std::max(b, 0.0);
            b += fa / 3.0;
        }
    }
    for (int64_t v = 0; v < nV; ++v) va[v] = vfa[v] < 0 ? (vea[v] < 0 ? 1.0 : vea[v]) : vfa[v];
    for (int64_t i = 0; i < nE; ++i)
        if (ea[i] < 0) ea[i] = len(i);
}

static inline uint64_t key2(uint32_t a, uint32_t b) { return ((uint64_t)a << 32) | b; }

// the weight source of the records being added (set by the candidate's adder)
static thread_local int32_t g_src[2] = { -1, -1 };
static void add_vv(Raw& r, int a, int b, double w)
{
    r.vv.push_back(key2(std::min(a, b), std::max(a, b)));
    r.vv_w.push_back(w);
    r.vv_src.push_back(g_src[0]);
    r.vv_src.push_back(g_src[1]);
}
static void add_ev(Raw& r, int e, int v, double w)
{
    r.ev.push_back(key2(e, v));
    r.ev_w.push_back(w);
    r.ev_src.push_back(g_src[0]);
    r.ev_src.push_back(g_src[1]);
}

// builder.cpp:239-336
// Area weighting (va, ea non-null): FV weight vertex_area(v) / 4
// (builder.cpp:146), EE weight (edge_area(ea) + edge_area(eb)) / 4
// (builder.cpp:181-183); their reductions carry the same weight.
static void add_face_vertex(Raw& r, const double* V, const int32_t* F, const int32_t* F2E, int fi, int vi,
    double offset_sqr, const double* va)
{
    const double w = va ? 0.25 * va[vi] : 1.0;
    g_src[0] = vi;
    g_src[1] = -1;
    const int f0 = F[3 * fi], f1 = F[3 * fi + 1], f2 = F[3 * fi + 2];
    const V3 p = row(V, vi), t0 = row(V, f0), t1 = row(V, f1), t2 = row(V, f2);
    const int dtype = point_triangle_distance_type(p, t0, t1, t2);
    const double d = point_triangle_distance(p, t0, t1, t2, dtype);
    if (!(d < offset_sqr)) return;
    switch (dtype) {
    case P_T0: add_vv(r, vi, f0, w); break;
    case P_T1: add_vv(r, vi, f1, w); break;
    case P_T2: add_vv(r, vi, f2, w); break;
    case P_E0t: add_ev(r, F2E[3 * fi + 0], vi, w); break;
    case P_E1t: add_ev(r, F2E[3 * fi + 1], vi, w); break;
    case P_E2t: add_ev(r, F2E[3 * fi + 2], vi, w); break;
    default:
        r.fv.push_back(fi);
        r.fv.push_back(vi);
        r.fv_w.push_back(w);
    }
}

// builder.cpp:140-237 (candidate oriented ea < eb)
static void add_edge_edge(Raw& r, const double* V, const double* Vrest, const int32_t* E, int ea, int eb,
    double offset_sqr, const double* earea)
{
    const double w = earea ? 0.25 * (earea[ea] + earea[eb]) : 1.0;
    g_src[0] = ea;
    g_src[1] = eb;
    const int a0 = E[2 * ea], a1 = E[2 * ea + 1], b0 = E[2 * eb], b1 = E[2 * eb + 1];
    const V3 xa0 = row(V, a0), xa1 = row(V, a1), xb0 = row(V, b0), xb1 = row(V, b1);
    const int actual = edge_edge_distance_type(xa0, xa1, xb0, xb1);
    const double d = edge_edge_distance(xa0, xa1, xb0, xb1, actual);
    if (!(d < offset_sqr)) return;
    const double eps_x = ee_mollifier_threshold(row(Vrest, a0), row(Vrest, a1), row(Vrest, b0), row(Vrest, b1));
    const double c = ee_cross_sqnorm(xa0, xa1, xb0, xb1);
    const int dtype = c < eps_x ? (int)EA_EB : actual;
    switch (dtype) {
    case EA0_EB0: add_vv(r, a0, b0, w); break;
    case EA0_EB1: add_vv(r, a0, b1, w); break;
    case EA1_EB0: add_vv(r, a1, b0, w); break;
    case EA1_EB1: add_vv(r, a1, b1, w); break;
    case EA_EB0: add_ev(r, ea, b0, w); break;
    case EA_EB1: add_ev(r, ea, b1, w); break;
    case EA0_EB: add_ev(r, eb, a0, w); break;
    case EA1_EB: add_ev(r, eb, a1, w); break;
    default:
        r.ee.push_back(ea);
        r.ee.push_back(eb);
        r.ee_eps.push_back(eps_x);
        r.ee_dt.push_back((int8_t)actual);
        r.ee_w.push_back(w);
    }
}

// Mesh adjacencies of CollisionMesh::init_adjacencies (collision_mesh.cpp:247-291):
// sorted unique vertex->vertex and vertex->edge lists, edge->opposite-vertex
// lists from the faces, and the boundary flag (a vertex is interior once an
// incident edge has two or more opposite vertices).
struct Adjacency {
    std::vector<std::vector<int32_t>> vv, ve, ev;
    std::vector<uint8_t> boundary;
};
static void build_adjacency(int64_t nV, const int32_t* E, int64_t nE, const int32_t* F, int64_t nF,
    const int32_t* F2E, Adjacency& A)
{
    A.vv.assign(nV, {});
    A.ve.assign(nV, {});
    A.ev.assign(nE, {});
    for (int64_t e = 0; e < nE; ++e) {
        A.vv[E[2 * e]].push_back(E[2 * e + 1]);
        A.vv[E[2 * e + 1]].push_back(E[2 * e]);
        A.ve[E[2 * e]].push_back((int32_t)e);
        A.ve[E[2 * e + 1]].push_back((int32_t)e);
    }
    for (int64_t f = 0; f < nF; ++f)
        for (int j = 0; j < 3; ++j) A.ev[F2E[3 * f + j]].push_back(F[3 * f + (j + 2) % 3]);
    auto uniq = [](std::vector<std::vector<int32_t>>& L) {
        for (auto& l : L) {
            std::sort(l.begin(), l.end());
            l.erase(std::unique(l.begin(), l.end()), l.end());
        }
    };
    uniq(A.vv);
    uniq(A.ve);
    uniq(A.ev);
    A.boundary.assign(nV, 1);
    for (int64_t e = 0; e < nE; ++e)
        if (A.ev[e].size() >= 2) A.boundary[E[2 * e]] = A.boundary[E[2 * e + 1]] = 0;
}

// An edge-vertex record reduced by its point-edge type
// (normal_collisions_builder.cpp:108-126): P_E0 / P_E1 -> VV with that
// endpoint, P_E -> EV.
static void add_ev_typed(Raw& r, const int32_t* E, int ei, int vi, int pe, double w)
{
    if (pe == P_E0) add_vv(r, vi, E[2 * ei], w);
    else if (pe == P_E1) add_vv(r, vi, E[2 * ei + 1], w);
    else add_ev(r, ei, vi, w);
}

// CollisionSetType::IMPROVED_MAX_APPROX (normal_collisions.cpp:84-128 with
// normal_collisions_builder.cpp:340-543 and the candidate conversions of
// candidates.cpp:583-692): edge-edge candidates give negative edge-vertex
// terms, face-vertex candidates negative edge-vertex and positive
// vertex-vertex terms, so that a contact near a shared edge or vertex is
// counted once instead of once per incident element.
static void improved_max_approx(Raw& r, const double* V, const double* Vrest, const int32_t* E, const int32_t* F,
    const int32_t* F2E, const std::vector<int32_t>& cee, const std::vector<int32_t>& cfv, double offset_sqr,
    const double* va, const double* ea, const Adjacency& A)
{
    g_src[0] = g_src[1] = -2; // improved terms: no area-weighted shape derivative
    auto active = [&](double d2) { return d2 < offset_sqr; };
    auto pe_dist = [&](int v, int e) {
        const V3 p = row(V, v), e0 = row(V, E[2 * e]), e1 = row(V, E[2 * e + 1]);
        return point_edge_distance(p, e0, e1, point_edge_distance_type(p, e0, e1));
    };
    auto sorted_unique = [](std::vector<uint64_t>& k) {
        std::sort(k.begin(), k.end());
        k.erase(std::unique(k.begin(), k.end()), k.end());
    };
    // edge-edge -> edge-vertex (candidates.cpp:665-692)
    std::vector<uint64_t> l1;
    for (size_t c = 0; 2 * c < cee.size(); ++c)
        for (int i = 0; i < 2; ++i) {
            const int ei = cee[2 * c + i], ej = cee[2 * c + 1 - i];
            for (int j = 0; j < 2; ++j) {
                const int vj = E[2 * ej + j];
                if (active(pe_dist(vj, ei))) l1.push_back(key2(ei, vj));
            }
        }
    sorted_unique(l1);
    // add_edge_edge_negative_edge_vertex_collision (builder.cpp:457-541)
    for (uint64_t k : l1) {
        const int e = (int)(k >> 32), p = (int)(k & 0xffffffffu);
        const int a0 = E[2 * e], a1 = E[2 * e + 1];
        const double w = ea ? -0.25 * ea[e] : -1.0;
        const int pe = point_edge_distance_type(row(V, p), row(V, a0), row(V, a1));
        int nonmollified = 0;
        for (int eb : A.ve[p]) {
            const int b0 = E[2 * eb], b1 = E[2 * eb + 1];
            const int q = p == b0 ? b1 : b0;
            if (q == a0 || q == a1) continue;
            const double eps_x = ee_mollifier_threshold(row(Vrest, a0), row(Vrest, a1), row(Vrest, b0), row(Vrest, b1));
            const double cr = ee_cross_sqnorm(row(V, a0), row(V, a1), row(V, b0), row(V, b1));
            if (cr >= eps_x) {
                ++nonmollified;
                continue;
            }
            const bool first = p == b0;
            const int dt = pe == P_E0 ? (first ? EA0_EB0 : EA0_EB1)
                                      : (pe == P_E1 ? (first ? EA1_EB0 : EA1_EB1) : (first ? EA_EB0 : EA_EB1));
            r.ee.push_back(e);
            r.ee.push_back(eb);
            r.ee_eps.push_back(eps_x);
            r.ee_dt.push_back((int8_t)dt);
            r.ee_w.push_back(w);
        }
        if (nonmollified == 1) continue;
        add_ev_typed(r, E, e, p, pe, (nonmollified - 1) * w);
    }
    // face-vertex -> edge-vertex (candidates.cpp:640-663)
    std::vector<uint64_t> l2, l3;
    for (size_t c = 0; 2 * c < cfv.size(); ++c) {
        const int f = cfv[2 * c], v = cfv[2 * c + 1];
        for (int j = 0; j < 3; ++j) {
            const int ei = F2E[3 * f + j];
            if (active(pe_dist(v, ei))) l2.push_back(key2(ei, v));
            // face-vertex -> vertex-vertex (candidates.cpp:583-611), unordered pairs
            const int vj = F[3 * f + j];
            if (active(point_point_distance(row(V, v), row(V, vj)))) l3.push_back(key2(std::min(v, vj), std::max(v, vj)));
        }
    }
    sorted_unique(l2);
    sorted_unique(l3);
    // add_face_vertex_negative_edge_vertex_collision (builder.cpp:421-455)
    for (uint64_t k : l2) {
        const int e = (int)(k >> 32), v = (int)(k & 0xffffffffu);
        const auto& inc = A.ev[e];
        const int amt = (int)inc.size() - (std::binary_search(inc.begin(), inc.end(), v) ? 1 : 0);
        if (amt <= 1) continue;
        const double w = (1 - amt) * (va ? 0.25 * va[v] : 1.0);
        add_ev_typed(r, E, e, v, point_edge_distance_type(row(V, v), row(V, E[2 * e]), row(V, E[2 * e + 1])), w);
    }
    // add_face_vertex_positive_vertex_vertex_collision (builder.cpp:382-419)
    for (uint64_t k : l3) {
        const int a = (int)(k >> 32), b = (int)(k & 0xffffffffu);
        double w = 0;
        auto add_w = [&](int vi, int vj) {
            const auto& inc = A.vv[vj];
            if (A.boundary[vj] || std::binary_search(inc.begin(), inc.end(), vi)) return;
            w += va ? 0.25 * va[vi] : 1.0;
        };
        add_w(a, b);
        add_w(b, a);
        if (w != 0) add_vv(r, a, b, w);
    }
}

static void finalize(Raw& all, Collisions& C)
{
    // builder.cpp:547-689: duplicate VV / EV keys merge with summed weights.
    // Lists are sorted by key and each key's weights are summed in ascending
    // order (without area weighting they are all 1, so the sum is a count);
    // the reference's order is thread-dependent, this one is not.
    auto merge = [](const std::vector<uint64_t>& keys, const std::vector<double>& win, const std::vector<int32_t>& src,
                     std::vector<int32_t>& ids, std::vector<double>& w, std::vector<int64_t>& soff,
                     std::vector<int32_t>& sout) {
        soff.assign(1, 0);
        sout.clear();
        std::vector<size_t> perm(keys.size());
        std::iota(perm.begin(), perm.end(), 0);
        std::sort(perm.begin(), perm.end(), [&](size_t a, size_t b) {
            return keys[a] != keys[b] ? keys[a] < keys[b] : win[a] < win[b];
        });
        ids.clear();
        w.clear();
        for (size_t i = 0; i < perm.size();) {
            size_t j = i;
            double sum = 0.0;
            while (j < perm.size() && keys[perm[j]] == keys[perm[i]]) sum += win[perm[j++]];
            if (sum != 0) {
                // weights that cancel to zero are dropped (builder.cpp:666-688)
                ids.push_back((int32_t)(keys[perm[i]] >> 32));
                ids.push_back((int32_t)(keys[perm[i]] & 0xffffffffu));
                w.push_back(sum);
                if (!src.empty()) {
                    for (size_t q = i; q < j; ++q) {
                        sout.push_back(src[2 * perm[q]]);
                        sout.push_back(src[2 * perm[q] + 1]);
                    }
                    soff.push_back((int64_t)sout.size() / 2);
                }
            }
            i = j;
        }
    };
    merge(all.vv, all.vv_w, all.vv_src, C.vv, C.vv_w, C.vv_src_off, C.vv_src);
    merge(all.ev, all.ev_w, all.ev_src, C.ev, C.ev_w, C.ev_src_off, C.ev_src);
    // EE: records are equal when their edges match as an unordered pair and
    // their distance types match (normal/edge_edge.cpp:123-142); equal
    // records sum their weights (ascending order) and zero sums are dropped.
    // The merged record keeps the orientation and eps_x of a record with
    // ea < eb when there is one (the candidate's own orientation); the
    // reference keeps whichever came first.  Sorted by (min, max, type).
    const size_t nee = all.ee_eps.size();
    auto ekey = [&](size_t i) {
        const uint32_t a = all.ee[2 * i], b = all.ee[2 * i + 1];
        return std::make_tuple(std::min(a, b), std::max(a, b), (int)all.ee_dt[i]);
    };
    std::vector<size_t> perm(nee);
    std::iota(perm.begin(), perm.end(), 0);
    std::sort(perm.begin(), perm.end(), [&](size_t a, size_t b) {
        return ekey(a) != ekey(b) ? ekey(a) < ekey(b) : all.ee_w[a] < all.ee_w[b];
    });
    C.ee.clear();
    C.ee_eps.clear();
    C.ee_dtype.clear();
    C.ee_w.clear();
    for (size_t i = 0; i < nee;) {
        size_t j = i, rep = perm[i];
        bool rep_sorted = all.ee[2 * rep] < all.ee[2 * rep + 1];
        double sum = 0.0;
        while (j < nee && ekey(perm[j]) == ekey(perm[i])) {
            const size_t q = perm[j++];
            sum += all.ee_w[q];
            if (!rep_sorted && all.ee[2 * q] < all.ee[2 * q + 1]) {
                rep = q;
                rep_sorted = true;
            }
        }
        if (sum != 0) {
            C.ee.push_back(all.ee[2 * rep]);
            C.ee.push_back(all.ee[2 * rep + 1]);
            C.ee_eps.push_back(all.ee_eps[rep]);
            C.ee_dtype.push_back(all.ee_dt[rep]);
            C.ee_w.push_back(sum);
        }
        i = j;
    }
    const size_t nfv = all.fv.size() / 2;
    std::vector<size_t> fp(nfv);
    std::iota(fp.begin(), fp.end(), 0);
    auto fkey = [&](size_t i) { return key2(all.fv[2 * i], all.fv[2 * i + 1]); };
    std::sort(fp.begin(), fp.end(), [&](size_t a, size_t b) { return fkey(a) < fkey(b); });
    C.fv.resize(2 * nfv);
    C.fv_w.resize(nfv);
    for (size_t i = 0; i < nfv; ++i) {
        C.fv[2 * i] = all.fv[2 * fp[i]];
        C.fv[2 * i + 1] = all.fv[2 * fp[i] + 1];
        C.fv_w[i] = all.fv_w[fp[i]];
    }
}

// ---------------------------------------------------------------------------
// Barrier functions (barrier.cpp:11-154, barrier.hpp:82-340) and the
// potential's scaling (barrier_potential.cpp:62-99).  kind: 0 ClampedLog,
// 1 NormalizedBarrier<ClampedLog>, 2 ClampedLogSq, 3 Cubic, 4 TwoStage.
// ---------------------------------------------------------------------------
static double barrier(double d, double dhat)
{
    if (d <= 0.0) return std::numeric_limits<double>::infinity();
    if (d >= dhat) return 0;
    const double dm = (d - dhat);
    return -dm * dm * std::log(d / dhat);
}
static double barrier_d1(double d, double dhat)
{
    if (d <= 0.0 || d >= dhat) return 0.0;
    return (dhat - d) * (2 * std::log(d / dhat) - dhat / d + 1);
}
static double barrier_d2(double d, double dhat)
{
    if (d <= 0.0 || d >= dhat) return 0.0;
    const double dd = dhat / d;
    return (dd + 2) * dd - 2 * std::log(d / dhat) - 3;
}
// ClampedLogSqBarrier (barrier.cpp:47-86)
static double logsq(int deriv, double d, double dhat)
{
    if (deriv == 0 && d <= 0.0) return std::numeric_limits<double>::infinity();
    if (d <= 0.0 || d >= dhat) return 0.0;
    const double l = std::log(d / dhat);
    if (deriv == 0) return (d - dhat) * (d - dhat) * l * l;
    if (deriv == 1) return 2 * (d - dhat) * l * (l + (d - dhat) / d);
    const double t0 = dhat - d, t2 = (t0 * t0) / (d * d);
    return 2 * ((l * l) - (l - 1) * t2 - 4 * l * t0 / d);
}
// CubicBarrier (barrier.cpp:90-117)
static double cubic(int deriv, double d, double dhat)
{
    if (!(d < dhat)) return 0.0;
    const double dm = d - dhat;
    if (deriv == 0) return -2.0 / 3.0 / dhat * dm * dm * dm;
    if (deriv == 1) return -2 / dhat * dm * dm;
    return 4 * (1 - d / dhat);
}
// TwoStageBarrier (barrier.cpp:121-152)
static double two_stage(int deriv, double d, double dhat)
{
    if (d >= dhat) return 0.0;
    if (d >= 0.5 * dhat) return deriv == 0 ? 0.5 * (dhat - d) * (dhat - d) : (deriv == 1 ? d - dhat : 1.0);
    if (deriv == 0) return -0.25 * dhat * dhat * (std::log(2 * d / dhat) - 0.5);
    if (deriv == 1) return -0.25 * dhat * dhat / d;
    return (0.25 * dhat * dhat) / (d * d);
}
static double clamped_log(int deriv, double d, double dhat)
{
    return deriv == 0 ? barrier(d, dhat) : (deriv == 1 ? barrier_d1(d, dhat) : barrier_d2(d, dhat));
}
static double barrier_any(int kind, int deriv, double d, double dhat)
{
    switch (kind) {
    case 1: {
        // NormalizedBarrier (barrier.hpp:145-175): b(d / dhat, 1) / dhat^deriv
        const double v = clamped_log(deriv, d / dhat, 1.0);
        return deriv == 0 ? v : (deriv == 1 ? v / dhat : v / (dhat * dhat));
    }
    case 2: return logsq(deriv, d, dhat);
    case 3: return cubic(deriv, d, dhat);
    case 4: return two_stage(deriv, d, dhat);
    default: return clamped_log(deriv, d, dhat);
    }
}
// bits: 1 = physical barrier, bits 4-7 = barrier kind (the C ABI's encoding)
struct BarrierParams {
    double dhat, kappa, dmin;
    int physical;
};
static inline int barrier_kind(const BarrierParams& P) { return (P.physical >> 4) & 15; }
// Barrier::units(x̂): x̂² (dimensionless 1 for the normalized barrier); the
// physical scaling is dhat / units(x̂) with x̂ = (2 dmin + dhat) dhat.
static inline double phys_scale(const BarrierParams& P)
{
    const double xh = (2 * P.dmin + P.dhat) * P.dhat;
    if (!(P.physical & 1)) return 1.0;
    return P.dhat / (barrier_kind(P) == 1 ? 1.0 : xh * xh);
}
static double fk(const BarrierParams& P, int deriv, double d2)
{
    return P.kappa
        * (barrier_any(barrier_kind(P), deriv, d2 - P.dmin * P.dmin, (2 * P.dmin + P.dhat) * P.dhat) * phys_scale(P));
}
static double f0(const BarrierParams& P, double d2) { return fk(P, 0, d2); }
static double f1(const BarrierParams& P, double d2) { return fk(P, 1, d2); }
static double f2(const BarrierParams& P, double d2) { return fk(P, 2, d2); }

// ---------------------------------------------------------------------------
// Closed-form squared-distance derivatives (own derivation).
//
// PT (point-plane) and EE (line-line) both have the form
//     d = N² / D,   N = a·(u×v),   D = |u×v|²
// in reduced variables r = (a, u, v) ∈ R⁹ that are vertex differences.
// PE (point-line) is d = |a×b|² / |b−a|² in r = (a, b) ∈ R⁶, PP is |r|².
// Derivatives in r are mapped to the 3n stencil coordinates through the ±1
// selection map S (r = S x):  ∇ₓd = Sᵀ∇ᵣd,  ∇²ₓd = Sᵀ∇²ᵣd S.
// ---------------------------------------------------------------------------
static inline void skew(V3 a, double M[3][3])
{
    M[0][0] = 0;
    M[0][1] = -a.z;
    M[0][2] = a.y;
    M[1][0] = a.z;
    M[1][1] = 0;
    M[1][2] = -a.x;
    M[2][0] = -a.y;
    M[2][1] = a.x;
    M[2][2] = 0;
}

// d = N²/D with N = a·(u×v), D = |u×v|² ; outputs value, g[9], H[9][9]
static double triple_quot(V3 a, V3 u, V3 v, double g[9], double H[9][9])
{
    const V3 w = cross(u, v);
    const double N = dot(a, w);
    const double D = sqnorm(w);
    // ∇N = (w, v×a, a×u)
    double gN[9], gD[9];
    const V3 gNu = cross(v, a), gNv = cross(a, u);
    // ∇D = (0, 2 v×w, 2 w×u)
    const V3 gDu = scale(cross(v, w), 2.0), gDv = scale(cross(w, u), 2.0);
    const V3 gNa = w;
    const V3 parts_N[3] = { gNa, gNu, gNv };
    const V3 parts_D[3] = { { 0, 0, 0 }, gDu, gDv };
    for (int b = 0; b < 3; ++b)
        for (int i = 0; i < 3; ++i) {
            gN[3 * b + i] = comp(parts_N[b], i);
            gD[3 * b + i] = comp(parts_D[b], i);
        }
    // ∇²N: blocks (a,u) = -[v]×, (a,v) = [u]×, (u,v) = -[a]× ; symmetric
    double HN[9][9] = {}, HD[9][9] = {};
    double Sv[3][3], Su[3][3], Sa[3][3], Sw[3][3];
    skew(v, Sv);
    skew(u, Su);
    skew(a, Sa);
    skew(w, Sw);
    // ∂²N/∂a_i∂u_j = ε_ijk v_k = -[v]×_ij ; ∂²N/∂a_i∂v_j = ε_ikj u_k = [u]×_ij ;
    // ∂²N/∂u_i∂v_j = ε_kij a_k = -[a]×_ij
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            HN[i][3 + j] = -Sv[i][j];
            HN[3 + j][i] = -Sv[i][j];
            HN[i][6 + j] = Su[i][j];
            HN[6 + j][i] = Su[i][j];
            HN[3 + i][6 + j] = -Sa[i][j];
            HN[6 + j][3 + i] = -Sa[i][j];
        }
    // ∇²D = 2(JᵀJ + Σ w_k ∇²w_k), J = [-[v]×, [u]×] over (u,v)
    // uu: 2 [v]×ᵀ[v]× ; vv: 2 [u]×ᵀ[u]× ; uv: 2(-[v]×ᵀ[u]× - [w]×)
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            double uu = 0, vv = 0, uv = 0;
            for (int k = 0; k < 3; ++k) {
                uu += Sv[k][i] * Sv[k][j];
                vv += Su[k][i] * Su[k][j];
                uv += -Sv[k][i] * Su[k][j];
            }
            HD[3 + i][3 + j] = 2 * uu;
            HD[6 + i][6 + j] = 2 * vv;
            HD[3 + i][6 + j] = 2 * (uv - Sw[i][j]);
            HD[6 + j][3 + i] = HD[3 + i][6 + j];
        }
    const double iD = 1.0 / D;
    const double d = N * N * iD;
    for (int i = 0; i < 9; ++i) g[i] = 2 * N * gN[i] * iD - N * N * gD[i] * iD * iD;
    for (int i = 0; i < 9; ++i)
        for (int j = 0; j < 9; ++j) {
            H[i][j] = 2 * gN[i] * gN[j] * iD + 2 * N * HN[i][j] * iD
                - 2 * N * (gN[i] * gD[j] + gD[i] * gN[j]) * iD * iD - N * N * HD[i][j] * iD * iD
                + 2 * N * N * gD[i] * gD[j] * iD * iD * iD;
        }
    return d;
}

// D = |u×v|² alone (edge-edge cross squared norm) in r=(u,v) ∈ R⁶
static double cross_sq(V3 u, V3 v, double g[6], double H[6][6])
{
    const V3 w = cross(u, v);
    const V3 gu = scale(cross(v, w), 2.0), gv = scale(cross(w, u), 2.0);
    for (int i = 0; i < 3; ++i) {
        g[i] = comp(gu, i);
        g[3 + i] = comp(gv, i);
    }
    double Sv[3][3], Su[3][3], Sw[3][3];
    skew(v, Sv);
    skew(u, Su);
    skew(w, Sw);
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            double uu = 0, vv = 0, uv = 0;
            for (int k = 0; k < 3; ++k) {
                uu += Sv[k][i] * Sv[k][j];
                vv += Su[k][i] * Su[k][j];
                uv += -Sv[k][i] * Su[k][j];
            }
            H[i][j] = 2 * uu;
            H[3 + i][3 + j] = 2 * vv;
            H[i][3 + j] = 2 * (uv - Sw[i][j]);
            H[3 + j][i] = H[i][3 + j];
        }
    return sqnorm(w);
}

// d = |a×b|²/|b−a|² in r=(a,b) ∈ R⁶
static double point_line_r(V3 a, V3 b, double g[6], double H[6][6])
{
    const V3 c = cross(a, b);
    const double P = sqnorm(c);
    const V3 e = sub(b, a);
    const double L = sqnorm(e);
    double Sa[3][3], Sb[3][3], Sc[3][3];
    skew(a, Sa);
    skew(b, Sb);
    skew(c, Sc);
    // J = [-[b]×, [a]×]; ∇P = 2Jᵀc ; ∇²P = 2(JᵀJ + Σ c_k∇²c_k), ∂²c_k/∂a_i∂b_j = ε_kij
    double gP[6], HP[6][6], gL[6], HL[6][6];
    const V3 gPa = scale(cross(b, c), 2.0); // 2(-[b]×)ᵀc = 2 [b]× c = 2 b×c
    const V3 gPb = scale(cross(c, a), 2.0); // 2 [a]×ᵀ c = -2 a×c = 2 c×a
    for (int i = 0; i < 3; ++i) {
        gP[i] = comp(gPa, i);
        gP[3 + i] = comp(gPb, i);
        gL[i] = -2 * comp(e, i);
        gL[3 + i] = 2 * comp(e, i);
    }
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            double aa = 0, bb = 0, ab = 0;
            for (int k = 0; k < 3; ++k) {
                aa += Sb[k][i] * Sb[k][j];
                bb += Sa[k][i] * Sa[k][j];
                ab += -Sb[k][i] * Sa[k][j];
            }
            HP[i][j] = 2 * aa;
            HP[3 + i][3 + j] = 2 * bb;
            HP[i][3 + j] = 2 * (ab - Sc[i][j]);
            HP[3 + j][i] = HP[i][3 + j];
            const double id = (i == j) ? 2.0 : 0.0;
            HL[i][j] = id;
            HL[3 + i][3 + j] = id;
            HL[i][3 + j] = -id;
            HL[3 + j][i] = -id;
        }
    const double iL = 1.0 / L;
    for (int i = 0; i < 6; ++i) g[i] = gP[i] * iL - P * gL[i] * iL * iL;
    for (int i = 0; i < 6; ++i)
        for (int j = 0; j < 6; ++j)
            H[i][j] = HP[i][j] * iL - (gP[i] * gL[j] + gL[i] * gP[j]) * iL * iL - P * HL[i][j] * iL * iL
                + 2 * P * gL[i] * gL[j] * iL * iL * iL;
    return P * iL;
}

// Stencil-local distance derivative: x = n vertices (3n coords).  A reduced
// variable k is x[pos[k]] - x[neg[k]] (vertex indices).  Returns d.
struct Reduced {
    int m;          // number of reduced 3-vectors (1,2,3)
    int pos[3], neg[3];
};

static void expand(const Reduced& R, int n, const double* gr, const double* Hr, int ldr, double* g, double* H)
{
    const int N = 3 * n;
    for (int i = 0; i < N; ++i) g[i] = 0;
    for (int i = 0; i < N * N; ++i) H[i] = 0;
    for (int k = 0; k < R.m; ++k)
        for (int c = 0; c < 3; ++c) {
            g[3 * R.pos[k] + c] += gr[3 * k + c];
            g[3 * R.neg[k] + c] -= gr[3 * k + c];
        }
    for (int k = 0; k < R.m; ++k)
        for (int l = 0; l < R.m; ++l)
            for (int c = 0; c < 3; ++c)
                for (int e = 0; e < 3; ++e) {
                    const double h = Hr[(3 * k + c) * ldr + 3 * l + e];
                    H[(3 * R.pos[k] + c) * N + 3 * R.pos[l] + e] += h;
                    H[(3 * R.pos[k] + c) * N + 3 * R.neg[l] + e] -= h;
                    H[(3 * R.neg[k] + c) * N + 3 * R.pos[l] + e] -= h;
                    H[(3 * R.neg[k] + c) * N + 3 * R.neg[l] + e] += h;
                }
}

// PP over local vertices (i, j)
static double dist_pp(const V3* x, int n, int i, int j, double* g, double* H)
{
    const V3 r = sub(x[i], x[j]);
    double gr[3] = { 2 * r.x, 2 * r.y, 2 * r.z };
    double Hr[9] = { 2, 0, 0, 0, 2, 0, 0, 0, 2 };
    Reduced R { 1, { i, 0, 0 }, { j, 0, 0 } };
    expand(R, n, gr, Hr, 3, g, H);
    return point_point_distance(x[i], x[j]);
}
// point p vs line (e0,e1) over local vertices
static double dist_pl(const V3* x, int n, int p, int e0, int e1, double* g, double* H)
{
    double gr[6], Hr[6][6];
    point_line_r(sub(x[e0], x[p]), sub(x[e1], x[p]), gr, Hr);
    Reduced R { 2, { e0, e1, 0 }, { p, p, 0 } };
    expand(R, n, gr, &Hr[0][0], 6, g, H);
    return point_line_distance(x[p], x[e0], x[e1]);
}
// point p vs plane (t0,t1,t2)
static double dist_pplane(const V3* x, int n, int p, int t0, int t1, int t2, double* g, double* H)
{
    double gr[9], Hr[9][9];
    triple_quot(sub(x[p], x[t0]), sub(x[t1], x[t0]), sub(x[t2], x[t0]), gr, Hr);
    Reduced R { 3, { p, t1, t2 }, { t0, t0, t0 } };
    expand(R, n, gr, &Hr[0][0], 9, g, H);
    return point_plane_distance(x[p], x[t0], x[t1], x[t2]);
}
// line (a0,a1) vs line (b0,b1)
static double dist_ll(const V3* x, int n, int a0, int a1, int b0, int b1, double* g, double* H)
{
    double gr[9], Hr[9][9];
    triple_quot(sub(x[b0], x[a0]), sub(x[a1], x[a0]), sub(x[b1], x[b0]), gr, Hr);
    Reduced R { 3, { b0, a1, b1 }, { a0, a0, b0 } };
    expand(R, n, gr, &Hr[0][0], 9, g, H);
    return line_line_distance(x[a0], x[a1], x[b0], x[b1]);
}
// EE distance with known dtype over local (ea0,ea1,eb0,eb1) = (0,1,2,3)
static double dist_ee(const V3* x, int dtype, double* g, double* H)
{
    switch (dtype) {
    case EA0_EB0: return dist_pp(x, 4, 0, 2, g, H);
    case EA0_EB1: return dist_pp(x, 4, 0, 3, g, H);
    case EA1_EB0: return dist_pp(x, 4, 1, 2, g, H);
    case EA1_EB1: return dist_pp(x, 4, 1, 3, g, H);
    case EA_EB0: return dist_pl(x, 4, 2, 0, 1, g, H);
    case EA_EB1: return dist_pl(x, 4, 3, 0, 1, g, H);
    case EA0_EB: return dist_pl(x, 4, 0, 2, 3, g, H);
    case EA1_EB: return dist_pl(x, 4, 1, 2, 3, g, H);
    default: return dist_ll(x, 4, 0, 1, 2, 3, g, H);
    }
}

// ---------------------------------------------------------------------------
// PSD projection (eigen_ext.tpp:64-108) via cyclic Jacobi
// ---------------------------------------------------------------------------
static void jacobi_eig(int n, const double* A_in, double* lam, double* Vec)
{
    double A[144];
    std::memcpy(A, A_in, sizeof(double) * n * n);
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j) Vec[i * n + j] = (i == j) ? 1.0 : 0.0;
    for (int sweep = 0; sweep < 100; ++sweep) {
        double off = 0, tot = 0;
        for (int i = 0; i < n; ++i)
            for (int j = 0; j < n; ++j) {
                tot += A[i * n + j] * A[i * n + j];
                if (i != j) off += A[i * n + j] * A[i * n + j];
            }
        if (off <= 1e-34 * tot || off == 0) break;
        for (int p = 0; p < n - 1; ++p)
            for (int q = p + 1; q < n; ++q) {
                const double apq = A[p * n + q];
                if (apq == 0) continue;
                const double app = A[p * n + p], aqq = A[q * n + q];
                const double theta = (aqq - app) / (2 * apq);
                const double t = (theta >= 0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1));
                const double c = 1 / std::sqrt(t * t + 1), s = t * c;
                for (int k = 0; k < n; ++k) {
                    const double akp = A[k * n + p], akq = A[k * n + q];
                    A[k * n + p] = c * akp - s * akq;
                    A[k * n + q] = s * akp + c * akq;
                }
                for (int k = 0; k < n; ++k) {
                    const double apk = A[p * n + k], aqk = A[q * n + k];
                    A[p * n + k] = c * apk - s * aqk;
                    A[q * n + k] = s * apk + c * aqk;
                }
                for (int k = 0; k < n; ++k) {
                    const double vkp = Vec[k * n + p], vkq = Vec[k * n + q];
                    Vec[k * n + p] = c * vkp - s * vkq;
                    Vec[k * n + q] = s * vkp + c * vkq;
                }
            }
    }
    for (int i = 0; i < n; ++i) lam[i] = A[i * n + i];
}

// Householder tridiagonalisation + implicit symmetric QR with Wilkinson
// shifts (Golub & Van Loan, Alg. 8.3.1/8.3.2) -- the method family of
// Eigen::SelfAdjointEigenSolver.  Eigenvectors are the columns of Q.
static bool ql_eig(int n, const double* A_in, double* d, double* Q)
{
    double A[144], e[12];
    std::memcpy(A, A_in, sizeof(double) * n * n);
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j) Q[i * n + j] = (i == j) ? 1.0 : 0.0;
    for (int k = 0; k + 2 < n; ++k) {
        double sig = 0;
        for (int i = k + 2; i < n; ++i) sig += A[i * n + k] * A[i * n + k];
        const double x0 = A[(k + 1) * n + k];
        if (sig == 0) {
            e[k] = x0;
            continue;
        }
        const double nx = std::sqrt(x0 * x0 + sig);
        const double alpha = (x0 >= 0) ? -nx : nx;
        double v[12], p[12];
        v[k + 1] = x0 - alpha;
        for (int i = k + 2; i < n; ++i) v[i] = A[i * n + k];
        const double tau = 2.0 / (v[k + 1] * v[k + 1] + sig);
        double K = 0;
        for (int i = k + 1; i < n; ++i) {
            double s = 0;
            for (int j = k + 1; j < n; ++j) s += A[i * n + j] * v[j];
            p[i] = tau * s;
            K += p[i] * v[i];
        }
        K *= 0.5 * tau;
        for (int i = k + 1; i < n; ++i) p[i] -= K * v[i];
        for (int i = k + 1; i < n; ++i)
            for (int j = k + 1; j < n; ++j) A[i * n + j] -= v[i] * p[j] + p[i] * v[j];
        e[k] = alpha;
        for (int r = 0; r < n; ++r) {
            double s = 0;
            for (int j = k + 1; j < n; ++j) s += Q[r * n + j] * v[j];
            s *= tau;
            for (int j = k + 1; j < n; ++j) Q[r * n + j] -= s * v[j];
        }
    }
    if (n >= 2) e[n - 2] = A[(n - 1) * n + n - 2];
    e[n - 1] = 0;
    for (int i = 0; i < n; ++i) d[i] = A[i * n + i];
    const double eps = 2.220446049250313e-16;
    int end = n - 1, iter = 0;
    while (end > 0) {
        for (int i = 0; i < end; ++i)
            if (std::fabs(e[i]) <= eps * (std::fabs(d[i]) + std::fabs(d[i + 1])) || std::fabs(e[i]) <= 1e-300) e[i] = 0;
        while (end > 0 && e[end - 1] == 0) --end;
        if (end <= 0) break;
        if (++iter > 40 * n) return false;
        int start = end - 1;
        while (start > 0 && e[start - 1] != 0) --start;
        const double td = 0.5 * (d[end - 1] - d[end]);
        const double b = e[end - 1];
        double mu = d[end];
        if (td == 0) mu -= std::fabs(b);
        else {
            const double h = std::hypot(td, b);
            mu -= b * b / (td + (td > 0 ? h : -h));
        }
        double x = d[start] - mu, z = e[start];
        for (int k = start; k < end; ++k) {
            const double r = std::hypot(x, z);
            double c = 1, s = 0;
            if (r != 0) {
                c = x / r;
                s = -z / r;
            }
            if (k > start) e[k - 1] = c * e[k - 1] - s * z;
            const double dk = d[k], dk1 = d[k + 1], ek = e[k];
            d[k] = c * c * dk - 2 * c * s * ek + s * s * dk1;
            d[k + 1] = s * s * dk + 2 * c * s * ek + c * c * dk1;
            e[k] = c * s * (dk - dk1) + (c * c - s * s) * ek;
            if (k < end - 1) {
                z = -s * e[k + 1];
                e[k + 1] = c * e[k + 1];
            }
            x = e[k];
            for (int q = 0; q < n; ++q) {
                const double qa = Q[q * n + k], qb = Q[q * n + k + 1];
                Q[q * n + k] = c * qa - s * qb;
                Q[q * n + k + 1] = s * qa + c * qb;
            }
        }
    }
    return true;
}

// 0: tridiagonal QR (default), 1: cyclic Jacobi (independent cross-check)
static int g_psd_solver = 0;

static void project_psd(int n, double* H, int method)
{
    if (method == 0) return;
    double lam[12], V[144];
    if (g_psd_solver == 1 || !ql_eig(n, H, lam, V)) jacobi_eig(n, H, lam, V);
    double mn = lam[0];
    for (int i = 1; i < n; ++i) mn = std::min(mn, lam[i]);
    if (mn >= 0.0) return;
    for (int i = 0; i < n; ++i)
        if (lam[i] < 0) lam[i] = (method == 1) ? 0.0 : -lam[i];
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j) {
            double s = 0;
            for (int k = 0; k < n; ++k) s += V[i * n + k] * lam[k] * V[j * n + k];
            H[i * n + j] = s;
        }
}

// ---------------------------------------------------------------------------
// Per-contact E/G/H (normal_potential.cpp:127-232)
// ---------------------------------------------------------------------------
enum CType { CT_VV = 0, CT_EV = 1, CT_EE = 2, CT_FV = 3 };

struct Contact {
    int type;
    int n;          // stencil vertices
    int vid[4];
    double w;
    double eps;     // EE only
    int dtype;      // EE only
};

static void contact_stencil(const Collisions& C, const int32_t* E, const int32_t* F, int64_t idx, Contact& c)
{
    const int64_t nvv = C.vv_w.size(), nev = C.ev_w.size(), nee = C.ee_w.size();
    if (idx < nvv) {
        c.type = CT_VV;
        c.n = 2;
        c.vid[0] = C.vv[2 * idx];
        c.vid[1] = C.vv[2 * idx + 1];
        c.w = C.vv_w[idx];
        return;
    }
    idx -= nvv;
    if (idx < nev) {
        const int e = C.ev[2 * idx], v = C.ev[2 * idx + 1];
        c.type = CT_EV;
        c.n = 3;
        c.vid[0] = v;
        c.vid[1] = E[2 * e];
        c.vid[2] = E[2 * e + 1];
        c.w = C.ev_w[idx];
        return;
    }
    idx -= nev;
    if (idx < nee) {
        const int ea = C.ee[2 * idx], eb = C.ee[2 * idx + 1];
        c.type = CT_EE;
        c.n = 4;
        c.vid[0] = E[2 * ea];
        c.vid[1] = E[2 * ea + 1];
        c.vid[2] = E[2 * eb];
        c.vid[3] = E[2 * eb + 1];
        c.w = C.ee_w[idx];
        c.eps = C.ee_eps[idx];
        c.dtype = C.ee_dtype[idx];
        return;
    }
    idx -= nee;
    const int f = C.fv[2 * idx], v = C.fv[2 * idx + 1];
    c.type = CT_FV;
    c.n = 4;
    c.vid[0] = v;
    c.vid[1] = F[3 * f];
    c.vid[2] = F[3 * f + 1];
    c.vid[3] = F[3 * f + 2];
    c.w = C.fv_w[idx];
}

// distance value + derivatives for a contact (stencil-local x)
static double contact_distance(const Contact& c, const V3* x, double* g, double* H)
{
    switch (c.type) {
    case CT_VV: return dist_pp(x, 2, 0, 1, g, H);
    case CT_EV: return dist_pl(x, 3, 0, 1, 2, g, H);
    case CT_EE: return dist_ee(x, c.dtype, g, H);
    default: return dist_pplane(x, 4, 0, 1, 2, 3, g, H);
    }
}

// mollifier m(x) and derivatives for EE (edge_edge_mollifier.cpp:42-136)
static double mollifier(const Contact& c, const V3* x, double* gm, double* Hm, bool& active)
{
    active = false;
    if (c.type != CT_EE) return 1.0;
    double gr[6], Hr[6][6];
    const double s = cross_sq(sub(x[1], x[0]), sub(x[3], x[2]), gr, Hr);
    if (!(s < c.eps)) return 1.0;
    active = true;
    const double xe = s / c.eps;
    const double m = (-xe + 2) * xe;
    const double inv = 1 / c.eps;
    const double m1 = 2 * inv * std::fma(-inv, s, 1);
    const double m2 = -2 / (c.eps * c.eps);
    double gs[12], Hs[144];
    Reduced R { 2, { 1, 3, 0 }, { 0, 2, 0 } };
    expand(R, 4, gr, &Hr[0][0], 6, gs, Hs);
    for (int i = 0; i < 12; ++i) gm[i] = m1 * gs[i];
    for (int i = 0; i < 12; ++i)
        for (int j = 0; j < 12; ++j) Hm[i * 12 + j] = m1 * Hs[i * 12 + j] + m2 * gs[i] * gs[j];
    return m;
}

// Distance-vector coefficients c (t = sum_i c_i x_i) with the collision's
// known distance type (compute_coefficients in candidates/vertex_vertex.cpp:40-46,
// edge_vertex.cpp:45-75, edge_edge.cpp:42-96, face_vertex.cpp:42-89): VV and
// EV (P_E) fixed, EE by its stored type, FV point-plane (P_T).
static void contact_coefficients(const Contact& c, const V3* x, double* co)
{
    auto pe_alpha = [](V3 p, V3 e0, V3 e1) {
        const V3 e = sub(e1, e0);
        return dot(sub(p, e0), e) / sqnorm(e);
    };
    if (c.type == CT_VV) {
        co[0] = 1.0;
        co[1] = -1.0;
    } else if (c.type == CT_EV) {
        const double a = pe_alpha(x[0], x[1], x[2]);
        co[0] = 1.0;
        co[1] = -1.0 + a;
        co[2] = -a;
    } else if (c.type == CT_FV) {
        double u, v;
        ldlt2_solve(sub(x[2], x[1]), sub(x[3], x[1]), sub(x[0], x[1]), u, v);
        co[0] = 1.0;
        co[1] = -1.0 + u + v;
        co[2] = -u;
        co[3] = -v;
    } else {
        const double Z[4] = { 0, 0, 0, 0 };
        for (int i = 0; i < 4; ++i) co[i] = Z[i];
        switch (c.dtype) {
        case EA0_EB0: co[0] = 1.0, co[2] = -1.0; break;
        case EA0_EB1: co[0] = 1.0, co[3] = -1.0; break;
        case EA1_EB0: co[1] = 1.0, co[2] = -1.0; break;
        case EA1_EB1: co[1] = 1.0, co[3] = -1.0; break;
        case EA_EB0: {
            const double a = pe_alpha(x[2], x[0], x[1]);
            co[0] = 1.0 - a, co[1] = a, co[2] = -1.0;
        } break;
        case EA_EB1: {
            const double a = pe_alpha(x[3], x[0], x[1]);
            co[0] = 1.0 - a, co[1] = a, co[3] = -1.0;
        } break;
        case EA0_EB: {
            const double a = pe_alpha(x[0], x[2], x[3]);
            co[0] = 1.0, co[2] = -1.0 + a, co[3] = -a;
        } break;
        case EA1_EB: {
            const double a = pe_alpha(x[1], x[2], x[3]);
            co[1] = 1.0, co[2] = -1.0 + a, co[3] = -a;
        } break;
        default: {
            // edge_edge_closest_point (tangent/closest_point.cpp:65-87):
            // [|ea|^2, -eb.ea; -eb.ea, |eb|^2] x = [-(ea0-eb0).ea, (ea0-eb0).eb]
            const V3 ea = sub(x[1], x[0]), eb = sub(x[3], x[2]);
            double a, b;
            ldlt2_solve(ea, scale(eb, -1.0), sub(x[2], x[0]), a, b);
            co[0] = 1.0 - a, co[1] = a, co[2] = -1.0 + b, co[3] = -b;
        }
        }
    }
}

// t = sum_i c_i x_i, accumulated in vertex order (collision_stencil.cpp:14-25)
static V3 distance_vector(const Contact& c, const V3* x, const double* co)
{
    V3 t { 0, 0, 0 };
    for (int i = 0; i < c.n; ++i) t = add(t, scale(x[i], co[i]));
    return t;
}

// Gauss-Newton Hessian diagonal of one collision (normal_potential.cpp:236-269):
// w (4 f''(|t|^2) c_i^2 t_d^2 + 2 f'(|t|^2) c_i^2).  The mollifier plays no part.
static void contact_gn_diagonal(const BarrierParams& P, const Contact& c, const V3* x, double* out)
{
    double co[4];
    contact_coefficients(c, x, co);
    const V3 t = distance_vector(c, x, co);
    const double d2 = sqnorm(t);
    const double s1 = c.w * 4.0 * f2(P, d2), s2 = c.w * 2.0 * f1(P, d2);
    const double t2[3] = { t.x * t.x, t.y * t.y, t.z * t.z };
    for (int i = 0; i < c.n; ++i) {
        const double ci2 = co[i] * co[i];
        for (int k = 0; k < 3; ++k) out[3 * i + k] = s1 * (ci2 * t2[k]) + s2 * ci2;
    }
}

// p^T H_GN p of one collision (normal_potential.cpp:271-308):
// w (4 f'' (J^T p . t)^2 + 2 f' |J^T p|^2) with J^T p = sum_i c_i p_i.
static double contact_gn_quadratic_form(const BarrierParams& P, const Contact& c, const V3* x, const V3* pl)
{
    double co[4];
    contact_coefficients(c, x, co);
    const V3 t = distance_vector(c, x, co);
    const double d2 = sqnorm(t);
    const V3 pj = distance_vector(c, pl, co);
    const double pjt = dot(pj, t);
    return c.w * (4.0 * f2(P, d2) * (pjt * pjt) + 2.0 * f1(P, d2) * sqnorm(pj));
}

static double contact_energy(const BarrierParams& P, const Contact& c, const V3* x)
{
    double g[12], H[144];
    const double d = contact_distance(c, x, g, H);
    double gm[12], Hm[144];
    bool act;
    const double m = mollifier(c, x, gm, Hm, act);
    return c.w * m * f0(P, d);
}

static void contact_gradient(const BarrierParams& P, const Contact& c, const V3* x, double* out)
{
    const int N = 3 * c.n;
    double gm[12], Hm[144];
    bool act;
    const double m = mollifier(c, x, gm, Hm, act);
    if (m <= 0) {
        for (int i = 0; i < N; ++i) out[i] = 0;
        return;
    }
    double g[12], H[144];
    const double d = contact_distance(c, x, g, H);
    const double fv = f0(P, d), fd = f1(P, d);
    if (c.type != CT_EE) {
        for (int i = 0; i < N; ++i) out[i] = (c.w * fd) * g[i];
        return;
    }
    for (int i = 0; i < N; ++i) out[i] = (c.w * fv) * (act ? gm[i] : 0.0) + (c.w * m * fd) * g[i];
}

static void contact_hessian(const BarrierParams& P, const Contact& c, const V3* x, int psd, double* out)
{
    const int N = 3 * c.n;
    double g[12], H[144];
    const double d = contact_distance(c, x, g, H);
    double gm[12] = {}, Hm[144] = {};
    bool act;
    const double m = mollifier(c, x, gm, Hm, act);
    if (c.type == CT_EE && m <= 0) {
        const double fv = f0(P, d);
        for (int i = 0; i < N * N; ++i) out[i] = (c.w * fv) * Hm[i];
        return;
    }
    const double fd = f1(P, d), fdd = f2(P, d);
    if (c.type != CT_EE) {
        for (int i = 0; i < N; ++i)
            for (int j = 0; j < N; ++j) out[i * N + j] = (c.w * fdd) * g[i] * g[j] + (c.w * fd) * H[i * N + j];
    } else {
        const double fv = f0(P, d);
        const double wm = c.w * m;
        for (int i = 0; i < N; ++i)
            for (int j = 0; j < N; ++j) {
                const double gfm_ij = (c.w * fd) * g[i] * gm[j];
                const double gfm_ji = (c.w * fd) * g[j] * gm[i];
                out[i * N + j] = (c.w * fv) * Hm[i * N + j] + gfm_ij + gfm_ji + (wm * fdd) * g[i] * g[j]
                    + (wm * fd) * H[i * N + j];
            }
    }
    project_psd(N, out, psd);
}

// ---------------------------------------------------------------------------
// Tight-Inclusion-style inclusion-based CCD (restated from the published
// method) + IPC strategy (tight_inclusion_ccd.cpp:33-75).
// ---------------------------------------------------------------------------
static thread_local long long g_ccd_iters = 0; // boxes examined (diagnostics)

struct CCDQuery {
    V3 s[4], e[4]; // start/end positions; VF: p,t0,t1,t2 ; EE: a0,a1,b0,b1
    bool vf;
};

// F(t,u,v) component c at one corner (Tight-Inclusion evaluation form)
static inline double ccd_F(const CCDQuery& q, int c, double t, double u, double v)
{
    double x[4];
    for (int k = 0; k < 4; ++k) {
        const double a = comp(q.s[k], c), b = comp(q.e[k], c);
        x[k] = (b - a) * t + a;
    }
    if (q.vf) {
        // p - (t0 + u (t1 - t0) + v (t2 - t0))
        const double pt = (x[2] - x[1]) * u + (x[3] - x[1]) * v + x[1];
        return x[0] - pt;
    }
    const double ea = (x[1] - x[0]) * u + x[0];
    const double eb = (x[3] - x[2]) * v + x[2];
    return ea - eb;
}

static void ccd_numerical_error(const CCDQuery& q, bool use_ms, double err[3])
{
    const double vf_f = use_ms ? 7.549516567451064e-15 : 6.661338147750939e-15;
    const double ee_f = use_ms ? 7.105427357601002e-15 : 6.217248937900877e-15;
    const double filt = q.vf ? vf_f : ee_f;
    for (int c = 0; c < 3; ++c) {
        double m = 0;
        for (int k = 0; k < 4; ++k) {
            m = std::max(m, std::fabs(comp(q.s[k], c)));
            m = std::max(m, std::fabs(comp(q.e[k], c)));
        }
        const double dl = std::min(m, 1.0);
        err[c] = filt * (dl * dl * dl);
    }
}

// Domain tolerances: δ divided by 3× the largest ∞-norm change of F along
// each parameter between opposite corners of the unit box.
static void ccd_domain_tol(const CCDQuery& q, double delta, double tol[3])
{
    for (int dim = 0; dim < 3; ++dim) {
        double L = 0;
        for (int a = 0; a < 2; ++a)
            for (int b = 0; b < 2; ++b) {
                // corners with parameter `dim` at 0 and 1, the others at (a, b)
                double c0[3], c1[3];
                int o = 0;
                for (int k = 0; k < 3; ++k) {
                    if (k == dim) {
                        c0[k] = 0;
                        c1[k] = 1;
                    } else {
                        c0[k] = c1[k] = (o++ == 0) ? a : b;
                    }
                }
                double m = 0;
                for (int c = 0; c < 3; ++c)
                    m = std::max(m, std::fabs(ccd_F(q, c, c1[0], c1[1], c1[2]) - ccd_F(q, c, c0[0], c0[1], c0[2])));
                L = std::max(L, m);
            }
        L *= 3;
        tol[dim] = (L == 0) ? delta : delta / L;
    }
}

struct CBox {
    double lo[3];
    int8_t lvl[3]; // width = 2^-lvl
};

// Total order of boxes: lower corner (t, u, v), then levels.  A child is
// always after its parent (it keeps the parent's corner with one level more,
// or moves the corner up), so the first accepted box in this order is the
// same however the tree is walked.
static inline bool cbox_before(const CBox& a, const CBox& b)
{
    for (int d = 0; d < 3; ++d)
        if (a.lo[d] != b.lo[d]) return a.lo[d] < b.lo[d];
    for (int d = 0; d < 3; ++d)
        if (a.lvl[d] != b.lvl[d]) return a.lvl[d] < b.lvl[d];
    return false;
}

static inline double cbox_w(const CBox& b, int d) { return std::ldexp(1.0, -b.lvl[d]); }

// Corner values of F over a box: f[c][i][j][k] at (t_i, u_j, v_k), and the
// separation radius eps_c + ms of each component.
struct CCorners {
    double f[3][2][2][2];
    double r[3];
};

// Inclusion test.  Returns zero_in; sets box_in, the codomain widths cw[c],
// whether component c lies inside [-eps-ms, eps+ms] (inside[c]), the
// largest change of component c between the two faces of the box across
// parameter d (var[c][d]) and the corner values.
static bool ccd_inclusion(const CCDQuery& q, const CBox& b, const double err[3], double ms, bool& box_in, double cw[3],
    double var[3][3], bool inside[3], CCorners& cc)
{
    const double ts[2] = { b.lo[0], b.lo[0] + cbox_w(b, 0) };
    const double us[2] = { b.lo[1], b.lo[1] + cbox_w(b, 1) };
    const double vs[2] = { b.lo[2], b.lo[2] + cbox_w(b, 2) };
    bool zin = true;
    box_in = true;
    for (int c = 0; c < 3; ++c) {
        double f[2][2][2];
        var[c][0] = var[c][1] = var[c][2] = 0;
        double mn = std::numeric_limits<double>::infinity(), mx = -mn;
        for (int i = 0; i < 2; ++i)
            for (int j = 0; j < 2; ++j)
                for (int k = 0; k < 2; ++k) {
                    f[i][j][k] = ccd_F(q, c, ts[i], us[j], vs[k]);
                    mn = std::min(mn, f[i][j][k]);
                    mx = std::max(mx, f[i][j][k]);
                }
        for (int j = 0; j < 2; ++j)
            for (int k = 0; k < 2; ++k) {
                var[c][0] = std::max(var[c][0], std::fabs(f[1][j][k] - f[0][j][k]));
                var[c][1] = std::max(var[c][1], std::fabs(f[j][1][k] - f[j][0][k]));
                var[c][2] = std::max(var[c][2], std::fabs(f[j][k][1] - f[j][k][0]));
            }
        const double r = err[c] + ms;
        if (mn > r || mx < -r) zin = false;
        inside[c] = (mn >= -r && mx <= r);
        if (!inside[c]) box_in = false;
        cw[c] = mx - mn;
        cc.r[c] = r;
        for (int i = 0; i < 2; ++i)
            for (int j = 0; j < 2; ++j)
                for (int k = 0; k < 2; ++k) cc.f[c][i][j][k] = f[i][j][k];
    }
    return zin;
}

// Whether halving the box across parameter d leaves a half whose corner box
// (the parent's corners, with the halving face's values taken as averages of
// the two opposite corners -- exact for the multilinear F up to rounding)
// misses the separation box in some component.  Only used to pick a split.
static bool ccd_split_excludes(const CCorners& cc, int d)
{
    for (int half = 0; half < 2; ++half)
        for (int c = 0; c < 3; ++c) {
            double mn = std::numeric_limits<double>::infinity(), mx = -mn;
            for (int i = 0; i < 2; ++i)
                for (int j = 0; j < 2; ++j)
                    for (int k = 0; k < 2; ++k) {
                        const int idx[3] = { i, j, k };
                        double v = cc.f[c][i][j][k];
                        if (idx[d] != half) {
                            int o[3] = { i, j, k };
                            o[d] = half;
                            v = (v + cc.f[c][o[0]][o[1]][o[2]]) * 0.5;
                        }
                        mn = std::min(mn, v);
                        mx = std::max(mx, v);
                    }
            if (mn > cc.r[c] || mx < -cc.r[c]) return true;
        }
    return false;
}

// Split parameter of a box that is neither discarded nor accepted:
// (1) a parameter whose halving discards a half at once (the one across
//     which the straddling components change most, if several);
// (2) else time, if the straddling components' change across time is at
//     least 1/16 of their largest change across any parameter: boxes are
//     visited in order of their earliest time, so a time split defers its
//     later half, while a u or v split leaves two boxes with the same
//     earliest time to resolve (this keeps near-parallel edge pairs, whose
//     root set is a whole segment, from being resolved point by point);
// (3) else the parameter across which the straddling components change
//     most.  Parameters at the depth limit are not split.
static int ccd_split_dim(const CBox& b, const double var[3][3], const bool inside[3], const CCorners& cc)
{
    double vmax[3] = { 0, 0, 0 };
    for (int c = 0; c < 3; ++c)
        if (!inside[c])
            for (int d = 0; d < 3; ++d) vmax[d] = std::max(vmax[d], var[c][d]);
    int sd = -1;
    double best = -1;
    for (int d = 0; d < 3; ++d)
        if (b.lvl[d] < 60 && ccd_split_excludes(cc, d) && vmax[d] > best) {
            best = vmax[d];
            sd = d;
        }
    if (sd >= 0) return sd;
    if (b.lvl[0] < 60 && vmax[0] * 16.0 >= std::max(vmax[0], std::max(vmax[1], vmax[2]))) return 0;
    for (int d = 0; d < 3; ++d)
        if (b.lvl[d] < 60 && vmax[d] > best) {
            best = vmax[d];
            sd = d;
        }
    return sd;
}

// Earliest-time branch and bound over (t,u,v) in [0,1]^3.  A box is
// accepted when every component of its function box is inside the
// separation box or narrower than the codomain tolerance delta (the union of
// Tight-Inclusion's "box inside the eps-box" and "codomain width below
// delta" tests), or when it is below the domain tolerances; otherwise it is
// halved across ccd_split_dim's parameter.  Returns whether a root box was found before tmax; toi = the
// smallest lower time bound of an accepted box.
//
// The boxes form a fixed binary tree (a box's children depend only on the
// box) whose boxes increase along every path in the order cbox_before, so
// the result is the first accepted box in that order (toi = its lower time
// bound, out_tol = its codomain width) whatever order the tree is walked in;
// boxes starting at or after tmax are skipped.  Here the boxes are visited
// best first, in that order, which examines the fewest boxes.  Only a query
// that exceeds the iteration cap depends on the order: it returns the
// earliest unresolved time, which in best-first order is the current box's.
static bool ccd_root_finder(const CCDQuery& q, const double err[3], double ms, const double tol[3], double delta,
    double tmax, long max_itr, double& toi, double& out_tol)
{
    auto later = [](const CBox& a, const CBox& b) { return cbox_before(b, a); };
    std::priority_queue<CBox, std::vector<CBox>, decltype(later)> pq(later);
    pq.push(CBox { { 0, 0, 0 }, { 0, 0, 0 } });
    double best = tmax;
    bool found = false;
    // "unlimited" iterations are capped so that no query can run away; the
    // cap falls back to the conservative earliest unresolved time
    const long cap = max_itr > 0 ? max_itr : (long)100000000;
    long itr = 0;
    out_tol = 0;
    while (!pq.empty()) {
        const CBox b = pq.top();
        pq.pop();
        if (b.lo[0] >= best) break; // every remaining box starts later
        ++itr;
        ++g_ccd_iters;
        bool box_in;
        double cw[3], var[3][3];
        bool inside[3];
        CCorners cc;
        if (!ccd_inclusion(q, b, err, ms, box_in, cw, var, inside, cc)) continue;
        const double w[3] = { cbox_w(b, 0), cbox_w(b, 1), cbox_w(b, 2) };
        // every component of the function box is either inside the
        // [-eps-ms, eps+ms] box or narrower than the codomain tolerance
        const bool small_co = (inside[0] || cw[0] <= delta) && (inside[1] || cw[1] <= delta)
            && (inside[2] || cw[2] <= delta);
        const bool small_dom = w[0] <= tol[0] && w[1] <= tol[1] && w[2] <= tol[2];
        const bool too_deep = b.lvl[0] >= 60 && b.lvl[1] >= 60 && b.lvl[2] >= 60;
        if (small_co || box_in || small_dom || too_deep) {
            best = b.lo[0];
            found = true;
            out_tol = std::max(cw[0], std::max(cw[1], cw[2]));
            break; // best first: every remaining box comes later
        }
        if (itr > cap) {
            // Out of iterations: the earliest unresolved time bounds the root.
            best = b.lo[0];
            found = true;
            out_tol = std::max(cw[0], std::max(cw[1], cw[2]));
            break;
        }
        const int sd = ccd_split_dim(b, var, inside, cc);
        CBox lo = b, hi = b;
        lo.lvl[sd] = hi.lvl[sd] = (int8_t)(b.lvl[sd] + 1);
        hi.lo[sd] = b.lo[sd] + cbox_w(lo, sd);
        // VF: drop halves entirely outside u + v <= 1
        const bool keep_hi = !(q.vf && sd != 0 && hi.lo[1] + hi.lo[2] > 1.0);
        const bool keep_lo = !(q.vf && sd != 0 && lo.lo[1] + lo.lo[2] > 1.0);
        if (keep_hi) pq.push(hi);
        if (keep_lo) pq.push(lo);
    }
    if (found) toi = best;
    return found;
}

// ticcd::{vertexFace,edgeEdge}CCD with automatic error and the no-zero-toi loop
static bool ti_ccd(const CCDQuery& q, double ms_in, double& toi, double tol_in, double tmax_in, long max_itr,
    double& out_tol, bool no_zero_toi)
{
    double err[3];
    ccd_numerical_error(q, ms_in > 0, err);
    double tmax = tmax_in, delta = tol_in, ms = ms_in;
    double tol[3];
    ccd_domain_tol(q, delta, tol);
    bool hit = false;
    for (int it = 0; it < 256; ++it) {
        double t = 0;
        hit = ccd_root_finder(q, err, ms, tol, delta, tmax, max_itr, t, out_tol);
        if (hit) toi = t;
        if (!(no_zero_toi && hit && toi == 0)) return hit;
        if (out_tol > delta) tmax *= 0.9;
        else if (10 * delta < ms) ms *= 0.5;
        else {
            delta *= 0.5;
            ccd_domain_tol(q, delta, tol);
        }
    }
    return hit;
}

struct CCDParams {
    double tolerance;
    long max_iterations;
    double rescale;
};

// tight_inclusion_ccd.cpp:33-75
static bool ccd_strategy(const CCDQuery& q, double min_distance, double d0, const CCDParams& P, double adjusted_tol,
    double tmax, double& toi)
{
    if (d0 <= min_distance) {
        toi = 0;
        return true;
    }
    double mind = (1.0 - P.rescale) * (d0 - min_distance);
    mind = std::min(mind, 1e-4);
    mind += min_distance;
    double out_tol;
    bool hit = ti_ccd(q, mind, toi, adjusted_tol, tmax, P.max_iterations, out_tol, false);
    if (hit && toi < 1e-6) {
        hit = ti_ccd(q, min_distance, toi, adjusted_tol, tmax, -1, out_tol, true);
        if (hit) toi *= P.rescale;
    }
    return hit;
}

static inline bool v3eq(V3 a, V3 b) { return a.x == b.x && a.y == b.y && a.z == b.z; }

// FaceVertexCandidate::ccd -> point_triangle_ccd (tight_inclusion_ccd.cpp:285-336)
static bool fv_ccd(const double* V0, const double* V1, const int32_t* F, int f, int v, double min_distance,
    const CCDParams& P, double tmax, double& toi)
{
    CCDQuery q;
    q.vf = true;
    const int ids[4] = { v, F[3 * f], F[3 * f + 1], F[3 * f + 2] };
    for (int k = 0; k < 4; ++k) {
        q.s[k] = row(V0, ids[k]);
        q.e[k] = row(V1, ids[k]);
    }
    const double d0 = std::sqrt(point_triangle_distance(q.s[0], q.s[1], q.s[2], q.s[3],
        point_triangle_distance_type(q.s[0], q.s[1], q.s[2], q.s[3])));
    if (v3eq(q.s[0], q.e[0]) && v3eq(q.s[1], q.e[1]) && v3eq(q.s[2], q.e[2]) && v3eq(q.s[3], q.e[3])) {
        if (d0 <= min_distance) {
            toi = 0;
            return true;
        }
        return false;
    }
    const double adj = std::min(0.5 * d0, P.tolerance);
    return ccd_strategy(q, min_distance, d0, P, adj, tmax, toi);
}

// EdgeEdgeCandidate::ccd -> edge_edge_ccd (tight_inclusion_ccd.cpp:229-283)
static bool ee_ccd(const double* V0, const double* V1, const int32_t* E, int ea, int eb, double min_distance,
    const CCDParams& P, double tmax, double& toi)
{
    CCDQuery q;
    q.vf = false;
    const int ids[4] = { E[2 * ea], E[2 * ea + 1], E[2 * eb], E[2 * eb + 1] };
    for (int k = 0; k < 4; ++k) {
        q.s[k] = row(V0, ids[k]);
        q.e[k] = row(V1, ids[k]);
    }
    const double d0 = std::sqrt(edge_edge_distance(q.s[0], q.s[1], q.s[2], q.s[3],
        edge_edge_distance_type(q.s[0], q.s[1], q.s[2], q.s[3])));
    if (v3eq(q.s[0], q.e[0]) && v3eq(q.s[1], q.e[1]) && v3eq(q.s[2], q.e[2]) && v3eq(q.s[3], q.e[3])) {
        if (d0 <= min_distance) {
            toi = 0;
            return true;
        }
        return false;
    }
    const double adj = std::min(0.5 * d0, P.tolerance);
    return ccd_strategy(q, min_distance, d0, P, adj, tmax, toi);
}

} // namespace orc

// ===========================================================================
// C ABI for the test harness (ctypes)
// ===========================================================================
using namespace orc;

extern "C" {

// --- primitives (for known-answer tests) ---
int orc_point_edge_distance_type(const double* p, const double* e0, const double* e1)
{
    return point_edge_distance_type(row(p, 0), row(e0, 0), row(e1, 0));
}
int orc_point_triangle_distance_type(const double* p, const double* t0, const double* t1, const double* t2)
{
    return point_triangle_distance_type(row(p, 0), row(t0, 0), row(t1, 0), row(t2, 0));
}
int orc_edge_edge_distance_type(const double* a0, const double* a1, const double* b0, const double* b1)
{
    return edge_edge_distance_type(row(a0, 0), row(a1, 0), row(b0, 0), row(b1, 0));
}
double orc_point_triangle_distance(const double* p, const double* t0, const double* t1, const double* t2, int dtype)
{
    const V3 P = row(p, 0), T0 = row(t0, 0), T1 = row(t1, 0), T2 = row(t2, 0);
    if (dtype < 0) dtype = point_triangle_distance_type(P, T0, T1, T2);
    return point_triangle_distance(P, T0, T1, T2, dtype);
}
double orc_edge_edge_distance(const double* a0, const double* a1, const double* b0, const double* b1, int dtype)
{
    const V3 A0 = row(a0, 0), A1 = row(a1, 0), B0 = row(b0, 0), B1 = row(b1, 0);
    if (dtype < 0) dtype = edge_edge_distance_type(A0, A1, B0, B1);
    return edge_edge_distance(A0, A1, B0, B1, dtype);
}
double orc_point_edge_distance(const double* p, const double* e0, const double* e1, int dtype)
{
    const V3 P = row(p, 0), E0 = row(e0, 0), E1 = row(e1, 0);
    if (dtype < 0) dtype = point_edge_distance_type(P, E0, E1);
    return point_edge_distance(P, E0, E1, dtype);
}
void orc_set_psd_solver(int which) { g_psd_solver = which; }

double orc_barrier(double d, double dhat, int deriv)
{
    return clamped_log(deriv, d, dhat);
}
double orc_barrier_kind(int kind, double d, double dhat, int deriv)
{
    return barrier_any(kind, deriv, d, dhat);
}

// Squared-distance gradient/Hessian of a stencil.  kind: 0 PP(2 verts),
// 1 PE-line(3: p,e0,e1), 2 PT-plane(4: p,t0,t1,t2), 3 EE(4) with dtype.
double orc_distance_derivatives(int kind, int dtype, const double* x, double* g, double* H)
{
    V3 v[4];
    const int n = kind == 0 ? 2 : (kind == 1 ? 3 : 4);
    for (int i = 0; i < n; ++i) v[i] = row(x, i);
    switch (kind) {
    case 0: return dist_pp(v, 2, 0, 1, g, H);
    case 1: return dist_pl(v, 3, 0, 1, 2, g, H);
    case 2: return dist_pplane(v, 4, 0, 1, 2, 3, g, H);
    default: return dist_ee(v, dtype, g, H);
    }
}

// faces_to_edges (collision_mesh.cpp:510-543); returns 0 or -1 if an edge is missing
int orc_faces_to_edges(const int32_t* F, int64_t nF, const int32_t* E, int64_t nE, int32_t* out)
{
    std::unordered_map<uint64_t, int32_t> m;
    m.reserve(nE * 2);
    for (int64_t e = 0; e < nE; ++e) {
        const uint32_t a = std::min(E[2 * e], E[2 * e + 1]), b = std::max(E[2 * e], E[2 * e + 1]);
        m.emplace(key2(a, b), (int32_t)e);
    }
    for (int64_t f = 0; f < nF; ++f)
        for (int j = 0; j < 3; ++j) {
            const uint32_t vi = F[3 * f + j], vj = F[3 * f + (j + 1) % 3];
            auto it = m.find(key2(std::min(vi, vj), std::max(vi, vj)));
            if (it == m.end()) return -1;
            out[3 * f + j] = it->second;
        }
    return 0;
}

// --- collision set ---
void orc_mesh_areas(const double* Vrest, int64_t nV, const int32_t* E, int64_t nE, const int32_t* F, int64_t nF,
    const int32_t* F2E, double* vertex_area, double* edge_area)
{
    mesh_areas(Vrest, nV, E, nE, F, nF, F2E, vertex_area, edge_area);
}

void* orc_collisions_build(const double* V, const double* Vrest, int64_t nV, const int32_t* E, int64_t nE,
    const int32_t* F, int64_t nF, const int32_t* F2E, double dhat, double dmin, int area_weighting, int set_type,
    int nthreads)
{
    Collisions* C = new Collisions();
    std::vector<double> va, ea;
    if (area_weighting) {
        va.resize(nV);
        ea.resize(nE);
        mesh_areas(Vrest, nV, E, nE, F, nF, F2E, va.data(), ea.data());
    }
    const double* pva = area_weighting ? va.data() : nullptr;
    const double* pea = area_weighting ? ea.data() : nullptr;
    std::vector<Box> vb;
    vertex_boxes_static(V, nV, 0.5 * (dhat + dmin), vb);
    Candidates cand;
    detect_candidates(vb, E, nE, F, nF, nthreads, cand);
    const double offset_sqr = (dmin + dhat) * (dmin + dhat);
    const int nt = std::max(1, nthreads);
    std::vector<Raw> raw(nt);
    const int64_t nee = cand.ee.size() / 2, nfv = cand.fv.size() / 2;
    parallel_for(nee, nt, [&](int64_t b, int64_t e, int t) {
        for (int64_t i = b; i < e; ++i) add_edge_edge(raw[t], V, Vrest, E, cand.ee[2 * i], cand.ee[2 * i + 1], offset_sqr, pea);
    });
    parallel_for(nfv, nt, [&](int64_t b, int64_t e, int t) {
        for (int64_t i = b; i < e; ++i) add_face_vertex(raw[t], V, F, F2E, cand.fv[2 * i], cand.fv[2 * i + 1], offset_sqr, pva);
    });
    Raw all;
    for (auto& r : raw) {
        all.vv.insert(all.vv.end(), r.vv.begin(), r.vv.end());
        all.vv_w.insert(all.vv_w.end(), r.vv_w.begin(), r.vv_w.end());
        all.vv_src.insert(all.vv_src.end(), r.vv_src.begin(), r.vv_src.end());
        all.ev_src.insert(all.ev_src.end(), r.ev_src.begin(), r.ev_src.end());
        all.ev.insert(all.ev.end(), r.ev.begin(), r.ev.end());
        all.ev_w.insert(all.ev_w.end(), r.ev_w.begin(), r.ev_w.end());
        all.ee_w.insert(all.ee_w.end(), r.ee_w.begin(), r.ee_w.end());
        all.fv_w.insert(all.fv_w.end(), r.fv_w.begin(), r.fv_w.end());
        all.ee.insert(all.ee.end(), r.ee.begin(), r.ee.end());
        all.ee_eps.insert(all.ee_eps.end(), r.ee_eps.begin(), r.ee_eps.end());
        all.ee_dt.insert(all.ee_dt.end(), r.ee_dt.begin(), r.ee_dt.end());
        all.fv.insert(all.fv.end(), r.fv.begin(), r.fv.end());
    }
    if (set_type == 1) {
        Adjacency A;
        build_adjacency(nV, E, nE, F, nF, F2E, A);
        improved_max_approx(all, V, Vrest, E, F, F2E, cand.ee, cand.fv, offset_sqr, pva, pea, A);
    }
    finalize(all, *C);
    C->n_cand_ee = nee;
    C->n_cand_fv = nfv;
    return C;
}

// Build from explicit arrays (to evaluate potentials on a given set)
void* orc_collisions_from_arrays(int64_t nvv, const int32_t* vv, const double* vvw, int64_t nev, const int32_t* ev,
    const double* evw, int64_t nee, const int32_t* ee, const double* eeeps, const int8_t* eedt, const double* eew,
    int64_t nfv, const int32_t* fv, const double* fvw)
{
    Collisions* C = new Collisions();
    C->vv.assign(vv, vv + 2 * nvv);
    C->vv_w.assign(vvw, vvw + nvv);
    C->ev.assign(ev, ev + 2 * nev);
    C->ev_w.assign(evw, evw + nev);
    C->ee.assign(ee, ee + 2 * nee);
    C->ee_eps.assign(eeeps, eeeps + nee);
    C->ee_dtype.assign(eedt, eedt + nee);
    C->ee_w.assign(eew, eew + nee);
    C->fv.assign(fv, fv + 2 * nfv);
    C->fv_w.assign(fvw, fvw + nfv);
    return C;
}

void orc_collisions_counts(void* h, int64_t* out)
{
    Collisions* C = (Collisions*)h;
    out[0] = C->vv_w.size();
    out[1] = C->ev_w.size();
    out[2] = C->ee_w.size();
    out[3] = C->fv_w.size();
    out[4] = C->n_cand_ee;
    out[5] = C->n_cand_fv;
}

void orc_collisions_get(void* h, int32_t* vv, double* vvw, int32_t* ev, double* evw, int32_t* ee, double* eeeps,
    int8_t* eedt, double* eew, int32_t* fv, double* fvw)
{
    Collisions* C = (Collisions*)h;
    std::copy(C->vv.begin(), C->vv.end(), vv);
    std::copy(C->vv_w.begin(), C->vv_w.end(), vvw);
    std::copy(C->ev.begin(), C->ev.end(), ev);
    std::copy(C->ev_w.begin(), C->ev_w.end(), evw);
    std::copy(C->ee.begin(), C->ee.end(), ee);
    std::copy(C->ee_eps.begin(), C->ee_eps.end(), eeeps);
    std::copy(C->ee_dtype.begin(), C->ee_dtype.end(), eedt);
    std::copy(C->ee_w.begin(), C->ee_w.end(), eew);
    std::copy(C->fv.begin(), C->fv.end(), fv);
    std::copy(C->fv_w.begin(), C->fv_w.end(), fvw);
}

void orc_collisions_free(void* h) { delete (Collisions*)h; }

// --- potentials ---
static inline void gather(const double* V, const Contact& c, V3* x)
{
    for (int i = 0; i < c.n; ++i) x[i] = row(V, c.vid[i]);
}

double orc_barrier_energy(void* h, const double* V, const int32_t* E, const int32_t* F, double dhat, double kappa,
    double dmin, int physical, int nthreads)
{
    Collisions* C = (Collisions*)h;
    const BarrierParams P { dhat, kappa, dmin, physical };
    const int64_t n = C->vv_w.size() + C->ev_w.size() + C->ee_w.size() + C->fv_w.size();
    const int nt = std::max(1, nthreads);
    std::vector<double> part(nt, 0.0);
    parallel_for(n, nt, [&](int64_t b, int64_t e, int t) {
        double s = 0;
        for (int64_t i = b; i < e; ++i) {
            Contact c;
            contact_stencil(*C, E, F, i, c);
            V3 x[4];
            gather(V, c, x);
            s += contact_energy(P, c, x);
        }
        part[t] += s;
    });
    double s = 0;
    for (double p : part) s += p;
    return s;
}

void orc_barrier_gradient(void* h, const double* V, int64_t nV, const int32_t* E, const int32_t* F, double dhat,
    double kappa, double dmin, int physical, int nthreads, double* grad)
{
    Collisions* C = (Collisions*)h;
    const BarrierParams P { dhat, kappa, dmin, physical };
    const int64_t n = C->vv_w.size() + C->ev_w.size() + C->ee_w.size() + C->fv_w.size();
    const int nt = std::max(1, nthreads);
    std::vector<std::vector<double>> loc(nt, std::vector<double>(3 * nV, 0.0));
    parallel_for(n, nt, [&](int64_t b, int64_t e, int t) {
        for (int64_t i = b; i < e; ++i) {
            Contact c;
            contact_stencil(*C, E, F, i, c);
            V3 x[4];
            gather(V, c, x);
            double g[12];
            contact_gradient(P, c, x, g);
            for (int k = 0; k < c.n; ++k)
                for (int d = 0; d < 3; ++d) loc[t][3 * c.vid[k] + d] += g[3 * k + d];
        }
    });
    for (int64_t i = 0; i < 3 * nV; ++i) {
        double s = 0;
        for (int t = 0; t < nt; ++t) s += loc[t][i];
        grad[i] = s;
    }
}

void orc_barrier_gn_diagonal(void* h, const double* V, int64_t nV, const int32_t* E, const int32_t* F, double dhat,
    double kappa, double dmin, int physical, int nthreads, double* diag)
{
    Collisions* C = (Collisions*)h;
    const BarrierParams P { dhat, kappa, dmin, physical };
    const int64_t n = C->vv_w.size() + C->ev_w.size() + C->ee_w.size() + C->fv_w.size();
    const int nt = std::max(1, nthreads);
    std::vector<std::vector<double>> loc(nt, std::vector<double>(3 * nV, 0.0));
    parallel_for(n, nt, [&](int64_t b, int64_t e, int t) {
        for (int64_t i = b; i < e; ++i) {
            Contact c;
            contact_stencil(*C, E, F, i, c);
            V3 x[4];
            gather(V, c, x);
            double g[12];
            contact_gn_diagonal(P, c, x, g);
            for (int k = 0; k < c.n; ++k)
                for (int d = 0; d < 3; ++d) loc[t][3 * c.vid[k] + d] += g[3 * k + d];
        }
    });
    for (int64_t i = 0; i < 3 * nV; ++i) {
        double s = 0;
        for (int t = 0; t < nt; ++t) s += loc[t][i];
        diag[i] = s;
    }
}

double orc_barrier_gn_quadratic_form(void* h, const double* V, const int32_t* E, const int32_t* F, double dhat,
    double kappa, double dmin, int physical, const double* p, int nthreads)
{
    Collisions* C = (Collisions*)h;
    const BarrierParams P { dhat, kappa, dmin, physical };
    const int64_t n = C->vv_w.size() + C->ev_w.size() + C->ee_w.size() + C->fv_w.size();
    const int nt = std::max(1, nthreads);
    std::vector<double> part(nt, 0.0);
    parallel_for(n, nt, [&](int64_t b, int64_t e, int t) {
        double s = 0;
        for (int64_t i = b; i < e; ++i) {
            Contact c;
            contact_stencil(*C, E, F, i, c);
            V3 x[4], pl[4];
            gather(V, c, x);
            gather(p, c, pl);
            s += contact_gn_quadratic_form(P, c, x, pl);
        }
        part[t] += s;
    });
    double s = 0;
    for (double v : part) s += v;
    return s;
}

// ---------------------------------------------------------------------------
// Friction: TangentialCollisions::build (tangential_collisions.cpp:60-170)
// and FrictionPotential (tangential_potential.cpp:156-331, friction_potential.cpp,
// friction/smooth_mu.cpp, friction/smooth_friction_mollifier.cpp), isotropic.
// ---------------------------------------------------------------------------
static V3 normalized(V3 a)
{
    const double n = sqnorm(a);
    if (!(n > 0)) return a;
    const double r = std::sqrt(n);
    return { a.x / r, a.y / r, a.z / r };
}
// tangent bases (tangent/tangent_basis.cpp): columns b0, b1
static void pp_basis(V3 p0, V3 p1, V3& b0, V3& b1)
{
    const V3 d = sub(p1, p0);
    const V3 cx = cross(V3 { 1, 0, 0 }, d), cy = cross(V3 { 0, 1, 0 }, d);
    const V3 c = sqnorm(cx) > sqnorm(cy) ? cx : cy;
    b0 = normalized(c);
    b1 = normalized(cross(d, c));
}
static void pe_basis(V3 p, V3 e0, V3 e1, V3& b0, V3& b1)
{
    const V3 e = sub(e1, e0);
    b0 = normalized(e);
    b1 = normalized(cross(e, sub(p, e0)));
}
static void ee_basis(V3 ea0, V3 ea1, V3 eb0, V3 eb1, V3& b0, V3& b1)
{
    const V3 ea = sub(ea1, ea0);
    const V3 n = cross(ea, sub(eb1, eb0));
    b0 = normalized(ea);
    b1 = normalized(cross(n, ea));
}
static void pt_basis(V3 p, V3 t0, V3 t1, V3 t2, V3& b0, V3& b1)
{
    (void)p;
    const V3 e0 = sub(t1, t0);
    const V3 n = cross(e0, sub(t2, t0));
    b0 = normalized(e0);
    b1 = normalized(cross(n, e0));
}
// smooth friction mollifier f0, f1/x, (f2 x - f1)/x^3 and the smooth mu
// blend of static and kinetic coefficients (isotropic)
static double mu_f0(double y, double ms, double mk, double ev)
{
    if (ms == mk || std::abs(y) >= ev) {
        const double f0 = std::abs(y) >= ev ? y : y * y * (1 - y / (3 * ev)) / ev + ev / 3;
        return mk * f0;
    }
    const double dm = mk - ms, z = std::abs(y) / ev;
    if (std::abs(y) < 0.5 * ev)
        return y * z * (z * (z * (1 - 0.4 * z) * dm - ms / 3.0) + ms) + (9.0 / 16.0) * ev * mk - (11.0 / 48.0) * ev * ms;
    return y * z * (z * (z * (0.4 * z - 2) * dm + (3 * mk - (10.0 / 3.0) * ms)) + (2 * ms - mk)) + 0.6 * ev * mk
        - (4.0 / 15.0) * ev * ms;
}
static double smooth_mu_value(double y, double ms, double mk, double ev)
{
    if (ms == mk || std::abs(y) >= ev) return mk;
    const double z = std::abs(y) / ev;
    if (std::abs(y) < 0.5 * ev) return 2 * (mk - ms) * z * z + ms;
    return -2 * (mk - ms) * (z * (z - 2) + 1) + mk;
}
static double mu_f1_over_x(double y, double ms, double mk, double ev)
{
    const double f1x = std::abs(y) >= ev ? 1 / y : (2 - y / ev) / ev;
    return smooth_mu_value(y, ms, mk, ev) * f1x;
}
static double mu_f2_x_minus_f1_over_x3(double y, double ms, double mk, double ev)
{
    if (ms == mk || std::abs(y) >= ev) {
        const double f = std::abs(y) >= ev ? -1 / (y * y * y) : -1 / (y * ev * ev);
        return mk * f;
    }
    const double dm = mk - ms, z = 1 / ev;
    if (std::abs(y) < 0.5 * ev) return z * z * (z * (8 - 6 * y * z) * dm - ms / y);
    return z * z * (z * (6 * y * z - 16) * dm + (9 * mk - 10 * ms) / y);
}

struct Tangential {
    Collisions base;                        // stencils and weights (vv | ev | ee | fv)
    std::vector<double> N, cp, P, mu_s, mu_k; // per collision: cp 2, P 6 (b0 xyz, b1 xyz)
    // anisotropy (tangential_collision.hpp:104-139): slip scaling (default 1),
    // directional coefficients (default 0 = isotropic), lagged effective mu
    std::vector<double> mu_aniso, mu_s_aniso, mu_k_aniso, mu_s_eff, mu_k_eff;
};

// smooth_mu.cpp:117-171: elliptical effective coefficients along the slip
// direction (default (1, 0) when the slip is below 1e-10).
static void aniso_mu_eff(const double* tau, const double* ms_a, const double* mk_a, double ms, double mk, double* out)
{
    const bool use_s = ms_a[0] * ms_a[0] + ms_a[1] * ms_a[1] > 0;
    const bool use_k = mk_a[0] * mk_a[0] + mk_a[1] * mk_a[1] > 0;
    if (!use_s && !use_k) {
        out[0] = ms;
        out[1] = mk;
        return;
    }
    const double nt = std::sqrt(tau[0] * tau[0] + tau[1] * tau[1]);
    double t0 = 1.0, t1 = 0.0;
    if (!(nt < 1e-10)) t0 = tau[0] / nt, t1 = tau[1] / nt;
    const double a = ms_a[0] * t0, b = ms_a[1] * t1, c = mk_a[0] * t0, d = mk_a[1] * t1;
    out[0] = use_s ? std::sqrt(a * a + b * b) : ms;
    out[1] = use_k ? std::sqrt(c * c + d * d) : mk;
}

// Relative-velocity coefficients g (relative velocity = sum_k g_k v_k) of a
// tangential collision (tangent/relative_velocity.cpp jacobians).
static void friction_gamma(const Contact& c, const double* cp, double* g)
{
    if (c.type == CT_VV) g[0] = 1, g[1] = -1;
    else if (c.type == CT_EV) g[0] = 1, g[1] = cp[0] - 1, g[2] = -cp[0];
    else if (c.type == CT_EE) g[0] = 1 - cp[0], g[1] = cp[0], g[2] = cp[1] - 1, g[3] = -cp[1];
    else g[0] = 1, g[1] = cp[0] + cp[1] - 1, g[2] = -cp[0], g[3] = -cp[1];
}
// relative velocity in the reference's functional forms
static V3 friction_rel_velocity(const Contact& c, const double* cp, const V3* v)
{
    if (c.type == CT_VV) return sub(v[0], v[1]);
    if (c.type == CT_EV) return sub(v[0], add(scale(sub(v[2], v[1]), cp[0]), v[1]));
    if (c.type == CT_EE)
        return sub(add(scale(sub(v[1], v[0]), cp[0]), v[0]), add(scale(sub(v[3], v[2]), cp[1]), v[2]));
    return sub(v[0], add(add(v[1], scale(sub(v[2], v[1]), cp[0])), scale(sub(v[3], v[1]), cp[1])));
}

// One tangential collision's energy, gradient (3n) and Hessian (3n x 3n).
static void friction_local(const Tangential& T, int64_t i, const Contact& c, const V3* v, double ev, int psd,
    double* e, double* g, double* H)
{
    const double* cp = &T.cp[2 * i];
    const double* P = &T.P[6 * i];
    const V3 rv = friction_rel_velocity(c, cp, v);
    const V3 b0 { P[0], P[1], P[2] }, b1 { P[3], P[4], P[5] };
    const double a0 = T.mu_aniso[2 * i], a1 = T.mu_aniso[2 * i + 1];
    const double u0 = a0 * dot(b0, rv), u1 = a1 * dot(b1, rv);
    const double nu = std::sqrt(u0 * u0 + u1 * u1);
    const double ms = T.mu_s_eff[i], mk = T.mu_k_eff[i];
    const double scl = c.w * T.N[i];
    if (e) *e = scl * mu_f0(nu, ms, mk, ev);
    double gm[4];
    friction_gamma(c, cp, gm);
    const int N = 3 * c.n;
    // T = Gamma^T P: row 3k+d = g_k (P(d,0), P(d,1))
    double Tm[12][2];
    for (int k = 0; k < c.n; ++k)
        for (int d = 0; d < 3; ++d) {
            Tm[3 * k + d][0] = (gm[k] * P[d]) * a0;
            Tm[3 * k + d][1] = (gm[k] * P[3 + d]) * a1;
        }
    const double f1x = mu_f1_over_x(nu, ms, mk, ev);
    if (g) {
        const double s0 = (f1x * u0) * scl, s1 = (f1x * u1) * scl;
        for (int r = 0; r < N; ++r) g[r] = Tm[r][0] * s0 + Tm[r][1] * s1;
    }
    if (!H) return;
    for (int r = 0; r < N * N; ++r) H[r] = 0;
    if (nu > ev) {
        if (psd != 0 && scl <= 0) return;
        const double cc = scl * f1x / (nu * nu);
        const double q0 = cc * -u1, q1 = cc * u0;
        double a[12], b[12];
        for (int r = 0; r < N; ++r) {
            a[r] = Tm[r][0] * q0 + Tm[r][1] * q1;
            b[r] = -u1 * Tm[r][0] + u0 * Tm[r][1];
        }
        for (int r = 0; r < N; ++r)
            for (int s = 0; s < N; ++s) H[r * N + s] = a[r] * b[s];
    } else if (nu == 0) {
        if (psd != 0 && scl <= 0) return;
        const double cc = scl * f1x;
        for (int r = 0; r < N; ++r)
            for (int s = 0; s < N; ++s) H[r * N + s] = (cc * Tm[r][0]) * Tm[s][0] + (cc * Tm[r][1]) * Tm[s][1];
    } else {
        const double f2 = mu_f2_x_minus_f1_over_x3(nu, ms, mk, ev);
        double in[4] = { f2 * u0 * u0, f2 * u0 * u1, f2 * u1 * u0, f2 * u1 * u1 };
        in[0] += f1x;
        in[3] += f1x;
        for (double& x : in) x *= scl;
        project_psd(2, in, psd);
        for (int r = 0; r < N; ++r) {
            const double t0 = Tm[r][0] * in[0] + Tm[r][1] * in[2], t1 = Tm[r][0] * in[1] + Tm[r][1] * in[3];
            for (int s = 0; s < N; ++s) H[r * N + s] = t0 * Tm[s][0] + t1 * Tm[s][1];
        }
    }
}

struct CSR {
    int64_t n = 0;
    std::vector<int64_t> rowptr;
    std::vector<int32_t> col;
    std::vector<double> val;
};

} // extern "C"
template <typename LocalFn>
static CSR* assemble_csr(int64_t n, int64_t nV, int nthreads, LocalFn&& local)
{
    struct Trip {
        int64_t key;
        double v;
    };
    const int nt = std::max(1, nthreads);
    std::vector<std::vector<Trip>> loc(nt);
    const int64_t ndof = 3 * nV;
    parallel_for(n, nt, [&](int64_t b, int64_t e, int t) {
        for (int64_t i = b; i < e; ++i) {
            int nv = 0;
            int vid[4];
            double Hl[144];
            local(i, nv, vid, Hl);
            const int N = 3 * nv;
            for (int a = 0; a < nv; ++a)
                for (int bb = 0; bb < nv; ++bb)
                    for (int k = 0; k < 3; ++k)
                        for (int l = 0; l < 3; ++l) {
                            const double val = Hl[(3 * a + k) * N + 3 * bb + l];
                            if (val != 0)
                                loc[t].push_back({ (3 * (int64_t)vid[a] + k) * ndof + 3 * (int64_t)vid[bb] + l, val });
                        }
        }
    });
    std::vector<Trip> all;
    for (auto& l : loc) all.insert(all.end(), l.begin(), l.end());
    std::stable_sort(all.begin(), all.end(), [](const Trip& a, const Trip& b) { return a.key < b.key; });
    CSR* M = new CSR();
    M->n = ndof;
    M->rowptr.assign(ndof + 1, 0);
    for (size_t i = 0; i < all.size();) {
        size_t j = i;
        double sum = 0;
        while (j < all.size() && all[j].key == all[i].key) sum += all[j++].v;
        M->col.push_back((int32_t)(all[i].key % ndof));
        M->val.push_back(sum);
        M->rowptr[all[i].key / ndof + 1]++;
        i = j;
    }
    for (int64_t r = 0; r < ndof; ++r) M->rowptr[r + 1] += M->rowptr[r];
    return M;
}
extern "C" {

// TangentialCollisions::build (tangential_collisions.cpp:60-170): normal
// force, closest point, tangent basis and blended mu per collision; EE
// collisions with cross^2 < eps_x are skipped.  dists use the classified
// (AUTO) type at V, as the tangential collision's compute_distance does.
void* orc_tangential_build(void* h, const double* V, const int32_t* E, const int32_t* F, double dhat, double kappa,
    double dmin, int physical, const double* mu_s, const double* mu_k)
{
    const Collisions& C = *(const Collisions*)h;
    const BarrierParams P { dhat, kappa, dmin, physical };
    Tangential* T = new Tangential();
    Collisions& B = T->base;
    const int64_t n = C.vv_w.size() + C.ev_w.size() + C.ee_w.size() + C.fv_w.size();
    const double xh = (2 * dmin + dhat) * dhat;
    for (int64_t i = 0; i < n; ++i) {
        Contact c;
        contact_stencil(C, E, F, i, c);
        V3 x[4];
        gather(V, c, x);
        if (c.type == CT_EE && ee_cross_sqnorm(x[0], x[1], x[2], x[3]) < c.eps) continue;
        double d2;
        if (c.type == CT_VV) d2 = point_point_distance(x[0], x[1]);
        else if (c.type == CT_EV) d2 = point_edge_distance(x[0], x[1], x[2], point_edge_distance_type(x[0], x[1], x[2]));
        else if (c.type == CT_EE)
            d2 = edge_edge_distance(x[0], x[1], x[2], x[3], edge_edge_distance_type(x[0], x[1], x[2], x[3]));
        else d2 = point_triangle_distance(x[0], x[1], x[2], x[3], point_triangle_distance_type(x[0], x[1], x[2], x[3]));
        // barrier_force_magnitude.cpp:5-15 with the physical scaling
        double Nf = -kappa * barrier_any(barrier_kind(P), 1, d2 - dmin * dmin, xh) * 2 * std::sqrt(d2);
        if (P.physical & 1) Nf *= dhat / (barrier_kind(P) == 1 ? 1.0 : xh * xh);
        double cp[2] = { 0, 0 };
        V3 b0, b1;
        double ms, mk;
        auto blend = [](double a, double b) { return (a + b) / 2; };
        const int* v = c.vid;
        if (c.type == CT_VV) {
            pp_basis(x[0], x[1], b0, b1);
            ms = blend(mu_s[v[0]], mu_s[v[1]]);
            mk = blend(mu_k[v[0]], mu_k[v[1]]);
        } else if (c.type == CT_EV) {
            const V3 e = sub(x[2], x[1]);
            cp[0] = dot(sub(x[0], x[1]), e) / sqnorm(e);
            pe_basis(x[0], x[1], x[2], b0, b1);
            ms = blend((mu_s[v[2]] - mu_s[v[1]]) * cp[0] + mu_s[v[1]], mu_s[v[0]]);
            mk = blend((mu_k[v[2]] - mu_k[v[1]]) * cp[0] + mu_k[v[1]], mu_k[v[0]]);
        } else if (c.type == CT_EE) {
            ldlt2_solve(sub(x[1], x[0]), scale(sub(x[3], x[2]), -1.0), sub(x[2], x[0]), cp[0], cp[1]);
            ee_basis(x[0], x[1], x[2], x[3], b0, b1);
            ms = blend((mu_s[v[1]] - mu_s[v[0]]) * cp[0] + mu_s[v[0]], (mu_s[v[3]] - mu_s[v[2]]) * cp[1] + mu_s[v[2]]);
            mk = blend((mu_k[v[1]] - mu_k[v[0]]) * cp[0] + mu_k[v[0]], (mu_k[v[3]] - mu_k[v[2]]) * cp[1] + mu_k[v[2]]);
        } else {
            ldlt2_solve(sub(x[2], x[1]), sub(x[3], x[1]), sub(x[0], x[1]), cp[0], cp[1]);
            pt_basis(x[0], x[1], x[2], x[3], b0, b1);
            ms = blend(mu_s[v[1]] + cp[0] * (mu_s[v[2]] - mu_s[v[1]]) + cp[1] * (mu_s[v[3]] - mu_s[v[1]]), mu_s[v[0]]);
            mk = blend(mu_k[v[1]] + cp[0] * (mu_k[v[2]] - mu_k[v[1]]) + cp[1] * (mu_k[v[3]] - mu_k[v[1]]), mu_k[v[0]]);
        }
        // stencil record, in the normal set's order
        const int64_t nvv = C.vv_w.size(), nev = C.ev_w.size(), nee = C.ee_w.size();
        if (c.type == CT_VV) {
            B.vv.push_back(C.vv[2 * i]);
            B.vv.push_back(C.vv[2 * i + 1]);
            B.vv_w.push_back(c.w);
        } else if (c.type == CT_EV) {
            const int64_t j = i - nvv;
            B.ev.push_back(C.ev[2 * j]);
            B.ev.push_back(C.ev[2 * j + 1]);
            B.ev_w.push_back(c.w);
        } else if (c.type == CT_EE) {
            const int64_t j = i - nvv - nev;
            B.ee.push_back(C.ee[2 * j]);
            B.ee.push_back(C.ee[2 * j + 1]);
            B.ee_w.push_back(c.w);
            B.ee_eps.push_back(C.ee_eps[j]);
            B.ee_dtype.push_back(C.ee_dtype[j]);
        } else {
            const int64_t j = i - nvv - nev - nee;
            B.fv.push_back(C.fv[2 * j]);
            B.fv.push_back(C.fv[2 * j + 1]);
            B.fv_w.push_back(c.w);
        }
        T->N.push_back(Nf);
        T->cp.push_back(cp[0]);
        T->cp.push_back(cp[1]);
        for (V3 b : { b0, b1 }) {
            T->P.push_back(b.x);
            T->P.push_back(b.y);
            T->P.push_back(b.z);
        }
        T->mu_s.push_back(ms);
        T->mu_k.push_back(mk);
    }
    const size_t nt = T->N.size();
    T->mu_aniso.assign(2 * nt, 1.0);
    T->mu_s_aniso.assign(2 * nt, 0.0);
    T->mu_k_aniso.assign(2 * nt, 0.0);
    T->mu_s_eff = T->mu_s; // reset_lagged_anisotropic_friction_coefficients
    T->mu_k_eff = T->mu_k;
    return T;
}

void orc_tangential_set_anisotropy(void* h, const double* mu_aniso, const double* mu_s_aniso, const double* mu_k_aniso)
{
    Tangential* T = (Tangential*)h;
    const size_t n = T->N.size();
    T->mu_aniso.assign(2 * n, 1.0);
    T->mu_s_aniso.assign(2 * n, 0.0);
    T->mu_k_aniso.assign(2 * n, 0.0);
    if (mu_aniso) std::copy(mu_aniso, mu_aniso + 2 * n, T->mu_aniso.begin());
    if (mu_s_aniso) std::copy(mu_s_aniso, mu_s_aniso + 2 * n, T->mu_s_aniso.begin());
    if (mu_k_aniso) std::copy(mu_k_aniso, mu_k_aniso + 2 * n, T->mu_k_aniso.begin());
}

// update_lagged_anisotropic_friction_coefficients (tangential_collisions.cpp:
// 19-58, 387-420): tangent basis and closest point at rest + lagged
// displacement, tau = T^T v with T = Gamma^T P, tau_aniso = mu_aniso . tau.
void orc_tangential_update_lagged_mu(void* h, const double* rest, const double* lagged, const double* vel,
    const int32_t* E, const int32_t* F)
{
    Tangential* T = (Tangential*)h;
    const int64_t n = T->N.size();
    for (int64_t i = 0; i < n; ++i) {
        Contact c;
        contact_stencil(T->base, E, F, i, c);
        V3 x[4], v[4];
        for (int k = 0; k < c.n; ++k) {
            x[k] = add(row(rest, c.vid[k]), row(lagged, c.vid[k]));
            v[k] = row(vel, c.vid[k]);
        }
        double cp[2] = { 0, 0 };
        V3 b0, b1;
        if (c.type == CT_VV) pp_basis(x[0], x[1], b0, b1);
        else if (c.type == CT_EV) {
            const V3 e = sub(x[2], x[1]);
            cp[0] = dot(sub(x[0], x[1]), e) / sqnorm(e);
            pe_basis(x[0], x[1], x[2], b0, b1);
        } else if (c.type == CT_EE) {
            ldlt2_solve(sub(x[1], x[0]), scale(sub(x[3], x[2]), -1.0), sub(x[2], x[0]), cp[0], cp[1]);
            ee_basis(x[0], x[1], x[2], x[3], b0, b1);
        } else {
            ldlt2_solve(sub(x[2], x[1]), sub(x[3], x[1]), sub(x[0], x[1]), cp[0], cp[1]);
            pt_basis(x[0], x[1], x[2], x[3], b0, b1);
        }
        const double* ms_a = &T->mu_s_aniso[2 * i];
        if (ms_a[0] * ms_a[0] + ms_a[1] * ms_a[1] == 0) {
            T->mu_s_eff[i] = T->mu_s[i];
            T->mu_k_eff[i] = T->mu_k[i];
            continue;
        }
        double g[4];
        friction_gamma(c, cp, g);
        double tau[2] = { 0, 0 };
        for (int k = 0; k < c.n; ++k) {
            tau[0] += g[k] * dot(b0, v[k]);
            tau[1] += g[k] * dot(b1, v[k]);
        }
        tau[0] *= T->mu_aniso[2 * i];
        tau[1] *= T->mu_aniso[2 * i + 1];
        double out[2];
        aniso_mu_eff(tau, ms_a, &T->mu_k_aniso[2 * i], T->mu_s[i], T->mu_k[i], out);
        T->mu_s_eff[i] = out[0];
        T->mu_k_eff[i] = out[1];
    }
}

// TangentialPotential::force (tangential_potential.cpp:40-77, 333-410):
// F = -w N(x+u) mu f1(|tau_a|)/|tau_a| T(x+u) tau_a, tau = T^T v,
// tau_a = mu_aniso . tau, with N, P and the closest point at the lagged
// positions x + u (distance type classified there) and the lagged effective
// mu (1 with no_mu).
void orc_friction_force(void* h, const double* rest, const double* lagged, const double* vel, int64_t nV,
    const int32_t* E, const int32_t* F, double dhat, double kappa, double dmin, int physical, double eps_v, int no_mu,
    double* force)
{
    const Tangential* T = (const Tangential*)h;
    const BarrierParams P { dhat, kappa, dmin, physical };
    const double xh = (2 * dmin + dhat) * dhat;
    const int64_t n = T->N.size();
    std::fill(force, force + 3 * nV, 0.0);
    for (int64_t i = 0; i < n; ++i) {
        Contact c;
        contact_stencil(T->base, E, F, i, c);
        V3 x[4], v[4];
        for (int k = 0; k < c.n; ++k) {
            x[k] = add(row(rest, c.vid[k]), row(lagged, c.vid[k]));
            v[k] = row(vel, c.vid[k]);
        }
        double d2;
        if (c.type == CT_VV) d2 = point_point_distance(x[0], x[1]);
        else if (c.type == CT_EV) d2 = point_edge_distance(x[0], x[1], x[2], point_edge_distance_type(x[0], x[1], x[2]));
        else if (c.type == CT_EE)
            d2 = edge_edge_distance(x[0], x[1], x[2], x[3], edge_edge_distance_type(x[0], x[1], x[2], x[3]));
        else d2 = point_triangle_distance(x[0], x[1], x[2], x[3], point_triangle_distance_type(x[0], x[1], x[2], x[3]));
        double Nf = -kappa * barrier_any(barrier_kind(P), 1, d2 - dmin * dmin, xh) * 2 * std::sqrt(d2);
        if (P.physical & 1) Nf *= dhat / (barrier_kind(P) == 1 ? 1.0 : xh * xh);
        double cp[2] = { 0, 0 };
        V3 b0, b1;
        if (c.type == CT_VV) pp_basis(x[0], x[1], b0, b1);
        else if (c.type == CT_EV) {
            const V3 e = sub(x[2], x[1]);
            cp[0] = dot(sub(x[0], x[1]), e) / sqnorm(e);
            pe_basis(x[0], x[1], x[2], b0, b1);
        } else if (c.type == CT_EE) {
            ldlt2_solve(sub(x[1], x[0]), scale(sub(x[3], x[2]), -1.0), sub(x[2], x[0]), cp[0], cp[1]);
            ee_basis(x[0], x[1], x[2], x[3], b0, b1);
        } else {
            ldlt2_solve(sub(x[2], x[1]), sub(x[3], x[1]), sub(x[0], x[1]), cp[0], cp[1]);
            pt_basis(x[0], x[1], x[2], x[3], b0, b1);
        }
        double g[4];
        friction_gamma(c, cp, g);
        double tau[2] = { 0, 0 };
        for (int k = 0; k < c.n; ++k) {
            tau[0] += g[k] * dot(b0, v[k]);
            tau[1] += g[k] * dot(b1, v[k]);
        }
        const double ta0 = T->mu_aniso[2 * i] * tau[0], ta1 = T->mu_aniso[2 * i + 1] * tau[1];
        const double ms = no_mu ? 1.0 : T->mu_s_eff[i], mk = no_mu ? 1.0 : T->mu_k_eff[i];
        const double f1x = mu_f1_over_x(std::sqrt(ta0 * ta0 + ta1 * ta1), ms, mk, eps_v);
        const double s = -c.w * Nf * f1x;
        for (int k = 0; k < c.n; ++k)
            for (int d = 0; d < 3; ++d) {
                const double Tr0 = g[k] * comp(b0, d), Tr1 = g[k] * comp(b1, d);
                force[3 * c.vid[k] + d] += s * (Tr0 * ta0 + Tr1 * ta1);
            }
    }
}

void orc_tangential_lagged_mu(void* h, double* mu_s_eff, double* mu_k_eff)
{
    const Tangential* T = (const Tangential*)h;
    std::copy(T->mu_s_eff.begin(), T->mu_s_eff.end(), mu_s_eff);
    std::copy(T->mu_k_eff.begin(), T->mu_k_eff.end(), mu_k_eff);
}

void orc_aniso_mu_eff(const double* tau_aniso, const double* mu_s_aniso, const double* mu_k_aniso, double mu_s,
    double mu_k, double* out)
{
    aniso_mu_eff(tau_aniso, mu_s_aniso, mu_k_aniso, mu_s, mu_k, out);
}

// The records are stored per type; reorder the per-collision arrays (built
// in normal-set order, which is also vv | ev | ee | fv) - nothing to do.
void orc_tangential_counts(void* h, int64_t* out)
{
    const Tangential* T = (const Tangential*)h;
    out[0] = T->base.vv_w.size();
    out[1] = T->base.ev_w.size();
    out[2] = T->base.ee_w.size();
    out[3] = T->base.fv_w.size();
}
void orc_tangential_get(void* h, int32_t* vv, int32_t* ev, int32_t* ee, int32_t* fv, double* w, double* N, double* cp,
    double* P, double* mu_s, double* mu_k)
{
    const Tangential* T = (const Tangential*)h;
    const Collisions& B = T->base;
    std::copy(B.vv.begin(), B.vv.end(), vv);
    std::copy(B.ev.begin(), B.ev.end(), ev);
    std::copy(B.ee.begin(), B.ee.end(), ee);
    std::copy(B.fv.begin(), B.fv.end(), fv);
    double* o = w;
    for (auto* a : { &B.vv_w, &B.ev_w, &B.ee_w, &B.fv_w }) o = std::copy(a->begin(), a->end(), o);
    std::copy(T->N.begin(), T->N.end(), N);
    std::copy(T->cp.begin(), T->cp.end(), cp);
    std::copy(T->P.begin(), T->P.end(), P);
    std::copy(T->mu_s.begin(), T->mu_s.end(), mu_s);
    std::copy(T->mu_k.begin(), T->mu_k.end(), mu_k);
}
void orc_tangential_free(void* h) { delete (Tangential*)h; }

static int64_t tangential_size(const Tangential& T)
{
    return T.base.vv_w.size() + T.base.ev_w.size() + T.base.ee_w.size() + T.base.fv_w.size();
}

double orc_friction_energy(void* h, const double* U, const int32_t* E, const int32_t* F, double eps_v, int nthreads)
{
    const Tangential& T = *(const Tangential*)h;
    const int64_t n = tangential_size(T);
    const int nt = std::max(1, nthreads);
    std::vector<double> part(nt, 0.0);
    parallel_for(n, nt, [&](int64_t b, int64_t e, int t) {
        double sum = 0;
        for (int64_t i = b; i < e; ++i) {
            Contact c;
            contact_stencil(T.base, E, F, i, c);
            V3 v[4];
            gather(U, c, v);
            double en;
            friction_local(T, i, c, v, eps_v, 0, &en, nullptr, nullptr);
            sum += en;
        }
        part[t] += sum;
    });
    double sum = 0;
    for (double x : part) sum += x;
    return sum;
}

void orc_friction_gradient(void* h, const double* U, int64_t nV, const int32_t* E, const int32_t* F, double eps_v,
    int nthreads, double* grad)
{
    const Tangential& T = *(const Tangential*)h;
    const int64_t n = tangential_size(T);
    const int nt = std::max(1, nthreads);
    std::vector<std::vector<double>> loc(nt, std::vector<double>(3 * nV, 0.0));
    parallel_for(n, nt, [&](int64_t b, int64_t e, int t) {
        for (int64_t i = b; i < e; ++i) {
            Contact c;
            contact_stencil(T.base, E, F, i, c);
            V3 v[4];
            gather(U, c, v);
            double g[12];
            friction_local(T, i, c, v, eps_v, 0, nullptr, g, nullptr);
            for (int k = 0; k < c.n; ++k)
                for (int d = 0; d < 3; ++d) loc[t][3 * c.vid[k] + d] += g[3 * k + d];
        }
    });
    for (int64_t i = 0; i < 3 * nV; ++i) {
        double sum = 0;
        for (int t = 0; t < nt; ++t) sum += loc[t][i];
        grad[i] = sum;
    }
}

void* orc_friction_hessian(void* h, const double* U, int64_t nV, const int32_t* E, const int32_t* F, double eps_v,
    int psd, int nthreads)
{
    const Tangential& T = *(const Tangential*)h;
    return assemble_csr(tangential_size(T), nV, nthreads, [&](int64_t i, int& nv, int* vid, double* Hl) {
        Contact c;
        contact_stencil(T.base, E, F, i, c);
        V3 v[4];
        gather(U, c, v);
        friction_local(T, i, c, v, eps_v, psd, nullptr, nullptr, Hl);
        nv = c.n;
        for (int k = 0; k < c.n; ++k) vid[k] = c.vid[k];
    });
}

// NormalPotential::shape_derivative (normal_potential.cpp:85-123, 310-416)
// for sets without area weighting (zero weight gradients): per collision
// w times the unprojected local Hessian, and for edge-edge collisions the
// reference's mollified form
//   f jac_m + gradx_m gradu_f^T + gradu_f gradu_m^T + gradu_m gradu_f^T + m hessu_f
// with eps_x and its gradient taken from the rest positions.
static void shape_local_ee(const BarrierParams& P, const Contact& c, const V3* x, const V3* xr, double* out)
{
    double g[12], H[144];
    const double d = contact_distance(c, x, g, H);
    const double f = c.w * f0(P, d), a1 = c.w * f1(P, d), a2 = c.w * f2(P, d);
    double gf[12];
    for (int i = 0; i < 12; ++i) gf[i] = a1 * g[i];
    const double eps = ee_mollifier_threshold(xr[0], xr[1], xr[2], xr[3]);
    double gr[6], Hr[6][6];
    const double sq = cross_sq(sub(x[1], x[0]), sub(x[3], x[2]), gr, Hr);
    double gm[12] = {}, gx[12] = {}, jm[144] = {};
    double m = 1.0;
    if (sq < eps) {
        const double xe = sq / eps;
        m = (-xe + 2) * xe;
        const double inv = 1 / eps;
        const double m1 = 2 * inv * std::fma(-inv, sq, 1);
        const double dme = 2 * sq * (-eps + sq) / (eps * eps * eps);
        const double dmse = 2 * (-eps + 2 * sq) / (eps * eps * eps);
        double gs[12], Hs[144];
        Reduced R { 2, { 1, 3, 0 }, { 0, 2, 0 } };
        expand(R, 4, gr, &Hr[0][0], 6, gs, Hs);
        // gradient of eps_x = 1e-3 |ea|^2 |eb|^2 with respect to the rest positions
        const V3 ea = sub(xr[0], xr[1]), eb = sub(xr[2], xr[3]);
        const double la = sqnorm(ea), lb = sqnorm(eb);
        double ge[12];
        for (int k = 0; k < 3; ++k) {
            ge[k] = 1e-3 * 2 * comp(ea, k) * lb;
            ge[3 + k] = -ge[k];
            ge[6 + k] = 1e-3 * la * 2 * comp(eb, k);
            ge[9 + k] = -ge[6 + k];
        }
        for (int i = 0; i < 12; ++i) {
            gm[i] = m1 * gs[i];
            gx[i] = dme * ge[i];
            for (int j = 0; j < 12; ++j) jm[i * 12 + j] = dmse * ge[i] * gs[j] + m1 * Hs[i * 12 + j];
        }
    }
    for (int i = 0; i < 12; ++i)
        for (int j = 0; j < 12; ++j) {
            const double hf = a2 * g[i] * g[j] + a1 * H[i * 12 + j];
            out[i * 12 + j] = f * jm[i * 12 + j] + gx[i] * gf[j] + gf[i] * gm[j] + gm[i] * gf[j] + m * hf;
        }
}

// Area Jacobians of the rest mesh (collision_mesh.cpp:376-432): per vertex
// the sum of its faces' area gradients / 3 (else half its edges' length
// gradients), per edge its faces' area gradients / 3 (else its length
// gradient); sparse over the 3 nV dofs.
typedef std::map<int64_t, double> SpVec;
static void add_to(SpVec& v, const int32_t* ids, int n, const double* g, double s)
{
    for (int a = 0; a < n; ++a)
        for (int d = 0; d < 3; ++d) v[3 * (int64_t)ids[a] + d] += s * g[3 * a + d];
}
static void area_jacobians(const double* R, int64_t nV, const int32_t* E, int64_t nE, const int32_t* F, int64_t nF,
    const int32_t* F2E, std::vector<SpVec>& vj, std::vector<SpVec>& ej)
{
    vj.assign(nV, {});
    ej.assign(nE, {});
    std::vector<char> vis_v(nV, 0), vis_e(nE, 0);
    for (int64_t f = 0; f < nF; ++f) {
        const V3 t0 = row(R, F[3 * f]), t1 = row(R, F[3 * f + 1]), t2 = row(R, F[3 * f + 2]);
        const V3 n = normalized(cross(sub(t1, t0), sub(t2, t0)));
        // d|A|/dt_i = n x (t_{i+2} - t_{i+1}) / 2
        const V3 g0 = scale(cross(n, sub(t2, t1)), 0.5), g1 = scale(cross(n, sub(t0, t2)), 0.5),
                 g2 = scale(cross(n, sub(t1, t0)), 0.5);
        const double g[9] = { g0.x, g0.y, g0.z, g1.x, g1.y, g1.z, g2.x, g2.y, g2.z };
        for (int j = 0; j < 3; ++j) {
            vis_v[F[3 * f + j]] = 1;
            add_to(vj[F[3 * f + j]], F + 3 * f, 3, g, 1.0 / 3.0);
            vis_e[F2E[3 * f + j]] = 1;
            add_to(ej[F2E[3 * f + j]], F + 3 * f, 3, g, 1.0 / 3.0);
        }
    }
    for (int64_t e = 0; e < nE; ++e) {
        const int32_t a = E[2 * e];
        if (vis_v[a] && vis_e[e]) continue;
        const V3 d = sub(row(R, E[2 * e]), row(R, E[2 * e + 1]));
        const double l = std::sqrt(sqnorm(d));
        const double g[6] = { d.x / l, d.y / l, d.z / l, -d.x / l, -d.y / l, -d.z / l };
        if (!vis_v[a])
            for (int j = 0; j < 2; ++j) add_to(vj[E[2 * e + j]], E + 2 * e, 2, g, 0.5);
        if (!vis_e[e]) add_to(ej[e], E + 2 * e, 2, g, 1.0);
    }
}

// General triplets -> CSR with duplicates summed.
static CSR* csr_from_triplets(int64_t ndof, std::vector<std::pair<int64_t, double>>& t)
{
    std::stable_sort(t.begin(), t.end(), [](const auto& a, const auto& b) { return a.first < b.first; });
    CSR* M = new CSR();
    M->n = ndof;
    M->rowptr.assign(ndof + 1, 0);
    for (size_t i = 0; i < t.size();) {
        size_t j = i;
        double sum = 0;
        while (j < t.size() && t[j].first == t[i].first) sum += t[j++].second;
        M->col.push_back((int32_t)(t[i].first % ndof));
        M->val.push_back(sum);
        M->rowptr[t[i].first / ndof + 1]++;
        i = j;
    }
    for (int64_t r = 0; r < ndof; ++r) M->rowptr[r + 1] += M->rowptr[r];
    return M;
}

void* orc_barrier_shape_derivative(void* h, const double* V, const double* Vrest, int64_t nV, const int32_t* E,
    int64_t nE, const int32_t* F, int64_t nF, const int32_t* F2E, double dhat, double kappa, double dmin, int physical,
    int area_weighting, int nthreads)
{
    (void)nthreads;
    const Collisions& C = *(const Collisions*)h;
    const BarrierParams P { dhat, kappa, dmin, physical };
    const int64_t nvv = C.vv_w.size(), nev = C.ev_w.size(), nee = C.ee_w.size();
    const int64_t n = nvv + nev + nee + C.fv_w.size();
    const int64_t ndof = 3 * nV;
    std::vector<SpVec> vj, ej;
    if (area_weighting) area_jacobians(Vrest, nV, E, nE, F, nF, F2E, vj, ej);
    std::vector<std::pair<int64_t, double>> trip;
    for (int64_t i = 0; i < n; ++i) {
        Contact c;
        contact_stencil(C, E, F, i, c);
        V3 x[4], xr[4];
        gather(V, c, x);
        gather(Vrest, c, xr);
        // second term: w times the unprojected local Hessian (mollified form for EE)
        double Hl[144];
        if (c.type == CT_EE) shape_local_ee(P, c, x, xr, Hl);
        else contact_hessian(P, c, x, 0, Hl);
        const int N = 3 * c.n;
        for (int a = 0; a < c.n; ++a)
            for (int b = 0; b < c.n; ++b)
                for (int k = 0; k < 3; ++k)
                    for (int l = 0; l < 3; ++l) {
                        const double val = Hl[(3 * a + k) * N + 3 * b + l];
                        if (val != 0)
                            trip.push_back({ (3 * (int64_t)c.vid[a] + k) * ndof + 3 * (int64_t)c.vid[b] + l, val });
                    }
        if (!area_weighting) continue;
        // first term: (grad_u f / w) (grad_x w)^T, grad_x w from the sources'
        // area Jacobians (normal_potential.cpp:330-355)
        SpVec wg;
        auto add_src = [&](int32_t s0, int32_t s1) {
            if (s1 < 0) {
                for (const auto& kv : vj[s0]) wg[kv.first] += 0.25 * kv.second;
            } else {
                SpVec sum = ej[s0];
                for (const auto& kv : ej[s1]) sum[kv.first] += kv.second;
                for (const auto& kv : sum) wg[kv.first] += 0.25 * kv.second;
            }
        };
        if (c.type == CT_VV)
            for (int64_t q = C.vv_src_off[i]; q < C.vv_src_off[i + 1]; ++q) add_src(C.vv_src[2 * q], C.vv_src[2 * q + 1]);
        else if (c.type == CT_EV) {
            const int64_t r = i - nvv;
            for (int64_t q = C.ev_src_off[r]; q < C.ev_src_off[r + 1]; ++q) add_src(C.ev_src[2 * q], C.ev_src[2 * q + 1]);
        } else if (c.type == CT_EE) {
            const int64_t r = i - nvv - nev;
            add_src(C.ee[2 * r], C.ee[2 * r + 1]);
        } else {
            add_src(c.vid[0], -1);
        }
        double g[12];
        contact_gradient(P, c, x, g);
        for (int r = 0; r < N; ++r) g[r] /= c.w;
        for (int a = 0; a < c.n; ++a)
            for (int d = 0; d < 3; ++d)
                for (const auto& kv : wg) trip.push_back({ (3 * (int64_t)c.vid[a] + d) * ndof + kv.first, g[3 * a + d] * kv.second });
    }
    return csr_from_triplets(ndof, trip);
}

// scalar smooth-friction functions for derivative checks
double orc_friction_mu(int which, double y, double mu_s, double mu_k, double eps_v)
{
    switch (which) {
    case 0: return mu_f0(y, mu_s, mu_k, eps_v);
    case 1: return mu_f1_over_x(y, mu_s, mu_k, eps_v);
    case 2: return mu_f2_x_minus_f1_over_x3(y, mu_s, mu_k, eps_v);
    default: return smooth_mu_value(y, mu_s, mu_k, eps_v);
    }
}

// Local Hessians → triplets (skip exact zeros, local_to_global.hpp:291) →
// duplicates summed → compressed rows.
void* orc_barrier_hessian(void* h, const double* V, int64_t nV, const int32_t* E, const int32_t* F, double dhat,
    double kappa, double dmin, int physical, int psd, int nthreads)
{
    Collisions* C = (Collisions*)h;
    const BarrierParams P { dhat, kappa, dmin, physical };
    const int64_t n = C->vv_w.size() + C->ev_w.size() + C->ee_w.size() + C->fv_w.size();
    const int nt = std::max(1, nthreads);
    struct Trip {
        int64_t key;
        double v;
    };
    std::vector<std::vector<Trip>> loc(nt);
    const int64_t ndof = 3 * nV;
    parallel_for(n, nt, [&](int64_t b, int64_t e, int t) {
        for (int64_t i = b; i < e; ++i) {
            Contact c;
            contact_stencil(*C, E, F, i, c);
            V3 x[4];
            gather(V, c, x);
            double Hl[144];
            contact_hessian(P, c, x, psd, Hl);
            const int N = 3 * c.n;
            for (int a = 0; a < c.n; ++a)
                for (int bb = 0; bb < c.n; ++bb)
                    for (int k = 0; k < 3; ++k)
                        for (int l = 0; l < 3; ++l) {
                            const double val = Hl[(3 * a + k) * N + 3 * bb + l];
                            if (val != 0) {
                                const int64_t r = 3 * (int64_t)c.vid[a] + k, cc = 3 * (int64_t)c.vid[bb] + l;
                                loc[t].push_back({ r * ndof + cc, val });
                            }
                        }
        }
    });
    std::vector<Trip> all;
    for (auto& l : loc) all.insert(all.end(), l.begin(), l.end());
    std::stable_sort(all.begin(), all.end(), [](const Trip& a, const Trip& b) { return a.key < b.key; });
    CSR* M = new CSR();
    M->n = ndof;
    M->rowptr.assign(ndof + 1, 0);
    for (size_t i = 0; i < all.size();) {
        size_t j = i;
        double s = 0;
        while (j < all.size() && all[j].key == all[i].key) s += all[j++].v;
        const int64_t r = all[i].key / ndof, c = all[i].key % ndof;
        M->col.push_back((int32_t)c);
        M->val.push_back(s);
        M->rowptr[r + 1]++;
        i = j;
    }
    for (int64_t r = 0; r < ndof; ++r) M->rowptr[r + 1] += M->rowptr[r];
    return M;
}

int64_t orc_csr_nnz(void* h) { return (int64_t)((CSR*)h)->val.size(); }
void orc_csr_get(void* h, int64_t* rowptr, int32_t* col, double* val)
{
    CSR* M = (CSR*)h;
    std::copy(M->rowptr.begin(), M->rowptr.end(), rowptr);
    std::copy(M->col.begin(), M->col.end(), col);
    std::copy(M->val.begin(), M->val.end(), val);
}
void orc_csr_free(void* h) { delete (CSR*)h; }

// Local (stencil) Hessian of one contact for kernel-level tests.
// type: 0 VV,1 EV,2 EE,3 FV; x: stencil positions (3n)
// Edge-edge cross product norm and mollifier (edge_edge_mollifier.cpp:7-14,
// 42-136, 194-202): x = (ea0, ea1, eb0, eb1) rows.  s = |ea x eb|^2 with its
// gradient (12) and Hessian (144); the threshold 1e-3 |ea|^2 |eb|^2; the
// mollifier m (1 when s >= eps) with its gradient and Hessian (zero when
// inactive).
double orc_ee_cross_sqnorm(const double* x, double* g, double* H)
{
    double gr[6], Hr[6][6];
    const double s = cross_sq(sub(row(x, 1), row(x, 0)), sub(row(x, 3), row(x, 2)), gr, Hr);
    Reduced R { 2, { 1, 3, 0 }, { 0, 2, 0 } };
    double Hs[144];
    expand(R, 4, gr, &Hr[0][0], 6, g, Hs);
    if (H)
        for (int i = 0; i < 144; ++i) H[i] = Hs[i];
    return s;
}
double orc_ee_mollifier_threshold(const double* x)
{
    return ee_mollifier_threshold(row(x, 0), row(x, 1), row(x, 2), row(x, 3));
}
double orc_ee_mollifier(const double* x, double eps, double* g, double* H)
{
    Contact c {};
    c.type = CT_EE;
    c.n = 4;
    c.eps = eps;
    V3 v[4];
    for (int i = 0; i < 4; ++i) v[i] = row(x, i);
    bool act = false;
    double gm[12], Hm[144];
    const double m = mollifier(c, v, gm, Hm, act);
    for (int i = 0; i < 12; ++i) g[i] = act ? gm[i] : 0.0;
    for (int i = 0; i < 144; ++i) H[i] = act ? Hm[i] : 0.0;
    return m;
}

void orc_contact_local(int type, int dtype, double eps, double w, const double* x, double dhat, double kappa,
    double dmin, int physical, int psd, double* energy, double* grad, double* hess)
{
    Contact c {};
    c.type = type;
    c.n = type == 0 ? 2 : (type == 1 ? 3 : 4);
    c.w = w;
    c.eps = eps;
    c.dtype = dtype;
    V3 v[4];
    for (int i = 0; i < c.n; ++i) v[i] = row(x, i);
    const BarrierParams P { dhat, kappa, dmin, physical };
    *energy = contact_energy(P, c, v);
    contact_gradient(P, c, v, grad);
    contact_hessian(P, c, v, psd, hess);
}

// --- CCD ---
int orc_point_triangle_ccd(const double* x0, const double* x1, double min_distance, double tmax, double tolerance,
    long max_iterations, double rescale, double* toi)
{
    // x0/x1: (p, t0, t1, t2) rows
    const int32_t F[3] = { 1, 2, 3 };
    const CCDParams P { tolerance, max_iterations, rescale };
    double t = std::numeric_limits<double>::infinity();
    const bool hit = fv_ccd(x0, x1, F, 0, 0, min_distance, P, tmax, t);
    *toi = t;
    return hit;
}
int orc_edge_edge_ccd(const double* x0, const double* x1, double min_distance, double tmax, double tolerance,
    long max_iterations, double rescale, double* toi)
{
    const int32_t E[4] = { 0, 1, 2, 3 };
    const CCDParams P { tolerance, max_iterations, rescale };
    double t = std::numeric_limits<double>::infinity();
    const bool hit = ee_ccd(x0, x1, E, 0, 1, min_distance, P, tmax, t);
    *toi = t;
    return hit;
}

// Batched single-stencil CCD (VF: p,t0,t1,t2; EE: a0,a1,b0,b1 rows) with the
// number of boxes each query examined.
void orc_ccd_stencils(int is_ee, int64_t n, const double* x0, const double* x1, double min_distance, double tmax,
    double tolerance, long max_iterations, double rescale, int8_t* hit, double* toi, int64_t* iters)
{
    const CCDParams P { tolerance, max_iterations, rescale };
    for (int64_t i = 0; i < n; ++i) {
        g_ccd_iters = 0;
        double t = std::numeric_limits<double>::infinity();
        bool h;
        if (is_ee) {
            const int32_t E[4] = { 0, 1, 2, 3 };
            h = ee_ccd(x0 + 12 * i, x1 + 12 * i, E, 0, 1, min_distance, P, tmax, t);
        } else {
            const int32_t F[3] = { 1, 2, 3 };
            h = fv_ccd(x0 + 12 * i, x1 + 12 * i, F, 0, 0, min_distance, P, tmax, t);
        }
        hit[i] = h;
        toi[i] = t;
        if (iters) iters[i] = g_ccd_iters;
    }
}

// Broad-phase candidates of the swept boxes (candidates.cpp:128-222):
// returns counts; fills ee / fv pairs when the output pointers are given.
void* orc_ccd_candidates(const double* V0, const double* V1, int64_t nV, const int32_t* E, int64_t nE,
    const int32_t* F, int64_t nF, double min_distance, int nthreads, int64_t* counts)
{
    std::vector<Box> vb;
    vertex_boxes_dynamic(V0, V1, nV, 0.5 * min_distance, vb);
    Candidates* cand = new Candidates();
    detect_candidates(vb, E, nE, F, nF, nthreads, *cand);
    std::vector<std::pair<int, int>> ee(cand->ee.size() / 2), fv(cand->fv.size() / 2);
    counts[0] = cand->ee.size() / 2;
    counts[1] = cand->fv.size() / 2;
    return cand;
}
void orc_ccd_candidates_get(void* h, int32_t* ee, int32_t* fv)
{
    Candidates* c = (Candidates*)h;
    std::copy(c->ee.begin(), c->ee.end(), ee);
    std::copy(c->fv.begin(), c->fv.end(), fv);
    delete c;
}

// compute_collision_free_stepsize (ipc.cpp:42-106, candidates.cpp:252-292)
double orc_collision_free_stepsize(const double* V0, const double* V1, int64_t nV, const int32_t* E, int64_t nE,
    const int32_t* F, int64_t nF, double min_distance, double tolerance, long max_iterations, double rescale,
    int nthreads, int64_t* n_candidates)
{
    std::vector<Box> vb;
    vertex_boxes_dynamic(V0, V1, nV, 0.5 * min_distance, vb);
    Candidates cand;
    detect_candidates(vb, E, nE, F, nF, nthreads, cand);
    const int64_t nee = cand.ee.size() / 2, nfv = cand.fv.size() / 2;
    if (n_candidates) *n_candidates = nee + nfv;
    if (nee + nfv == 0) return 1.0;
    const CCDParams P { tolerance, max_iterations, rescale };
    std::atomic<double> earliest(1.0);
    const int nt = std::max(1, nthreads);
    parallel_for(nee + nfv, nt, [&](int64_t b, int64_t e, int) {
        for (int64_t i = b; i < e; ++i) {
            const double tmax = earliest.load(std::memory_order_relaxed);
            double toi = std::numeric_limits<double>::infinity();
            bool hit;
            if (i < nee) hit = ee_ccd(V0, V1, E, cand.ee[2 * i], cand.ee[2 * i + 1], min_distance, P, tmax, toi);
            else {
                const int64_t k = i - nee;
                hit = fv_ccd(V0, V1, F, cand.fv[2 * k], cand.fv[2 * k + 1], min_distance, P, tmax, toi);
            }
            if (hit) {
                double prev = earliest.load(std::memory_order_relaxed);
                while (toi < prev && !earliest.compare_exchange_weak(prev, toi, std::memory_order_relaxed)) { }
            }
        }
    });
    return earliest.load();
}

} // extern "C"
