// geom.cuh — FP64 geometry shared by the device kernels.
//
// Evaluation order follows the reference's Eigen 3-vector code on an SSE2
// build: dot = (x0*y0 + x1*y1) + x2*y2, cross as in Eigen::cross, no fused
// multiply-add.  Translation units that need bit-exact values (collision
// filter, CCD) are compiled with -fmad=false.
#pragma once
#include <cstdint>
#include <math.h>

namespace ipcg {

struct V3 {
    double x, y, z;
};

__host__ __device__ __forceinline__ V3 v3(double x, double y, double z) { return V3 { x, y, z }; }
__host__ __device__ __forceinline__ V3 operator-(V3 a, V3 b) { return V3 { a.x - b.x, a.y - b.y, a.z - b.z }; }
__host__ __device__ __forceinline__ V3 operator+(V3 a, V3 b) { return V3 { a.x + b.x, a.y + b.y, a.z + b.z }; }
__host__ __device__ __forceinline__ V3 operator*(V3 a, double s) { return V3 { a.x * s, a.y * s, a.z * s }; }
__host__ __device__ __forceinline__ double dot(V3 a, V3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
__host__ __device__ __forceinline__ double sqnorm(V3 a) { return dot(a, a); }
__host__ __device__ __forceinline__ V3 cross(V3 a, V3 b)
{
    return V3 { a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x };
}
__host__ __device__ __forceinline__ double comp(V3 a, int i) { return i == 0 ? a.x : (i == 1 ? a.y : a.z); }
__device__ __forceinline__ V3 load_v3(const double* __restrict__ V, int i)
{
    return V3 { __ldg(V + 3 * i), __ldg(V + 3 * i + 1), __ldg(V + 3 * i + 2) };
}

// distance-type enums (src/ipc/distance/distance_type.hpp)
enum : int { P_E0 = 0, P_E1 = 1, P_E = 2 };
enum : int { P_T0 = 0, P_T1 = 1, P_T2 = 2, P_E0T = 3, P_E1T = 4, P_E2T = 5, P_T = 6 };
enum : int {
    EA0_EB0 = 0, EA0_EB1 = 1, EA1_EB0 = 2, EA1_EB1 = 3, EA_EB0 = 4, EA_EB1 = 5, EA0_EB = 6, EA1_EB = 7, EA_EB = 8
};

// distance_type.cpp:10-34
__host__ __device__ inline int point_edge_distance_type(V3 p, V3 e0, V3 e1)
{
    const V3 e = e1 - e0;
    const double len2 = sqnorm(e);
    if (len2 == 0) return P_E0;
    const double ratio = dot(e, p - e0) / len2;
    if (ratio < 0) return P_E0;
    if (ratio > 1) return P_E1;
    return P_E;
}

// (B Bᵀ) x = B r with Eigen's pivoted LDLᵀ on the 2×2 Gram matrix
// (distance_type.cpp:48,55,62).
__host__ __device__ inline void ldlt2_solve(V3 b0, V3 b1, V3 r, double& x0, double& x1)
{
    double a00 = dot(b0, b0);
    const double a10 = dot(b1, b0);
    double a11 = dot(b1, b1);
    double y0 = dot(b0, r), y1 = dot(b1, r);
    bool swapped = false;
    if (fabs(a11) > fabs(a00)) {
        const double t = a00;
        a00 = a11;
        a11 = t;
        const double u = y0;
        y0 = y1;
        y1 = u;
        swapped = true;
    }
    const double d0 = a00;
    if (d0 == 0.0) {
        x0 = 0;
        x1 = 0;
        return;
    }
    const double l10 = a10 / d0;
    const double d1 = a11 - l10 * (d0 * l10);
    y1 = y1 - l10 * y0;
    const double tiny = 2.2250738585072014e-308; // DBL_MIN
    y0 = (fabs(d0) > tiny) ? y0 / d0 : 0.0;
    y1 = (fabs(d1) > tiny) ? y1 / d1 : 0.0;
    y0 = y0 - l10 * y1;
    if (swapped) {
        x0 = y1;
        x1 = y0;
    } else {
        x0 = y0;
        x1 = y1;
    }
}

// distance_type.cpp:36-79
__host__ __device__ inline int point_triangle_distance_type(V3 p, V3 t0, V3 t1, V3 t2)
{
    const V3 normal = cross(t1 - t0, t2 - t0);
    double a0, b0, a1, b1, a2, b2;
    V3 e = t1 - t0;
    ldlt2_solve(e, cross(e, normal), p - t0, a0, b0);
    if (a0 > 0.0 && a0 < 1.0 && b0 >= 0.0) return P_E0T;
    e = t2 - t1;
    ldlt2_solve(e, cross(e, normal), p - t1, a1, b1);
    if (a1 > 0.0 && a1 < 1.0 && b1 >= 0.0) return P_E1T;
    e = t0 - t2;
    ldlt2_solve(e, cross(e, normal), p - t2, a2, b2);
    if (a2 > 0.0 && a2 < 1.0 && b2 >= 0.0) return P_E2T;
    if (a0 <= 0.0 && a2 >= 1.0) return P_T0;
    if (a1 <= 0.0 && a0 >= 1.0) return P_T1;
    if (a2 <= 0.0 && a1 >= 1.0) return P_T2;
    return P_T;
}

// distance_type.cpp:176-211
__host__ __device__ inline int edge_edge_parallel_distance_type(V3 ea0, V3 ea1, V3 eb0, V3 eb1)
{
    const V3 ea = ea1 - ea0;
    const double alpha = dot(eb0 - ea0, ea) / sqnorm(ea);
    const double beta = dot(eb1 - ea0, ea) / sqnorm(ea);
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
__host__ __device__ inline int edge_edge_distance_type(V3 ea0, V3 ea1, V3 eb0, V3 eb1)
{
    const double PARALLEL_THRESHOLD = 2.5e-16;
    const V3 u = ea1 - ea0, v = eb1 - eb0, w = ea0 - eb0;
    const double a = sqnorm(u), b = dot(u, v), c = sqnorm(v), d = dot(u, w), e = dot(v, w);
    const double D = a * c - b * b;
    if (a == 0.0 && c == 0.0) return EA0_EB0;
    if (a == 0.0) return EA0_EB;
    if (c == 0.0) return EA_EB0;
    const double par_tol = PARALLEL_THRESHOLD * a * c;
    const double uxv2 = sqnorm(cross(u, v));
    if (uxv2 < par_tol) return edge_edge_parallel_distance_type(ea0, ea1, eb0, eb1);
    int def = EA_EB;
    const double sN = (b * e - c * d);
    double tN, tD;
    if (sN <= 0.0) {
        tN = e;
        tD = c;
        def = EA0_EB;
    } else if (sN >= D) {
        tN = e + b;
        tD = c;
        def = EA1_EB;
    } else {
        tN = (a * e - b * d);
        tD = D;
        if (tN > 0.0 && tN < tD && uxv2 < par_tol) {
            if (sN < D / 2) {
                tN = e;
                tD = c;
                def = EA0_EB;
            } else {
                tN = e + b;
                tD = c;
                def = EA1_EB;
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
    return def;
}

// squared distances (point_point.cpp, point_line.cpp, point_plane.cpp + normal.hpp, line_line.cpp)
__host__ __device__ __forceinline__ double point_point_distance(V3 p0, V3 p1) { return sqnorm(p1 - p0); }
__host__ __device__ __forceinline__ double point_line_distance(V3 p, V3 e0, V3 e1)
{
    return sqnorm(cross(e0 - p, e1 - p)) / sqnorm(e1 - e0);
}
__host__ __device__ inline double point_plane_distance(V3 p, V3 t0, V3 t1, V3 t2)
{
    V3 n = cross(t1 - t0, t2 - t0);
    const double z = sqnorm(n);
    if (z > 0) {
        const double s = sqrt(z);
        n = V3 { n.x / s, n.y / s, n.z / s };
    }
    const double ptp = dot(p - t0, n);
    return ptp * ptp / sqnorm(n);
}
__host__ __device__ __forceinline__ double line_line_distance(V3 ea0, V3 ea1, V3 eb0, V3 eb1)
{
    const V3 n = cross(ea1 - ea0, eb1 - eb0);
    const double ltl = dot(eb0 - ea0, n);
    return ltl * ltl / sqnorm(n);
}
__host__ __device__ inline double point_triangle_distance(V3 p, V3 t0, V3 t1, V3 t2, int dtype)
{
    switch (dtype) {
    case P_T0: return point_point_distance(p, t0);
    case P_T1: return point_point_distance(p, t1);
    case P_T2: return point_point_distance(p, t2);
    case P_E0T: return point_line_distance(p, t0, t1);
    case P_E1T: return point_line_distance(p, t1, t2);
    case P_E2T: return point_line_distance(p, t2, t0);
    default: return point_plane_distance(p, t0, t1, t2);
    }
}
__host__ __device__ inline double edge_edge_distance(V3 ea0, V3 ea1, V3 eb0, V3 eb1, int dtype)
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
__host__ __device__ inline double point_edge_distance(V3 p, V3 e0, V3 e1, int dtype)
{
    switch (dtype) {
    case P_E0: return point_point_distance(p, e0);
    case P_E1: return point_point_distance(p, e1);
    default: return point_line_distance(p, e0, e1);
    }
}
// edge_edge_mollifier.cpp:7-14, 194-202
__host__ __device__ __forceinline__ double ee_cross_sqnorm(V3 ea0, V3 ea1, V3 eb0, V3 eb1)
{
    return sqnorm(cross(ea1 - ea0, eb1 - eb0));
}
__host__ __device__ __forceinline__ double ee_mollifier_threshold(V3 ea0, V3 ea1, V3 eb0, V3 eb1)
{
    return 1e-3 * sqnorm(ea0 - ea1) * sqnorm(eb0 - eb1);
}

} // namespace ipcg
