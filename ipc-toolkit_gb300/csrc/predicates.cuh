// predicates.cuh — exact orientation test and the edge-triangle intersection
// test of has_intersections (geometry/intersection.cpp:120-147).
//
// orient3d restates the adaptive-precision method of J. R. Shewchuk,
// "Adaptive Precision Floating-Point Arithmetic and Fast Robust Geometric
// Predicates" (Discrete & Computational Geometry 18, 1997), which the
// reference reaches through igl::predicates: the determinant is evaluated in
// FP64 with the static error bound (7 + 56 eps) eps * permanent
// (eps = 2^-53); when that does not decide the sign, it is recomputed exactly
// as a floating-point expansion (error-free sums, and exact products from a
// fused multiply-add).  Only the sign is used, so the orientation convention
// does not matter to the caller.  Compile with -fmad=false: the error-free
// transformations must not be contracted.
#pragma once

#include "geom.cuh"

namespace ipcg {
namespace exact {

__host__ __device__ __forceinline__ void two_sum(double a, double b, double& x, double& y)
{
    x = a + b;
    const double bv = x - a;
    const double av = x - bv;
    y = (a - av) + (b - bv);
}
__host__ __device__ __forceinline__ void fast_two_sum(double a, double b, double& x, double& y)
{
    x = a + b;
    y = b - (x - a);
}
__host__ __device__ __forceinline__ void two_diff(double a, double b, double& x, double& y)
{
    x = a - b;
    const double bv = a - x;
    const double av = x + bv;
    y = (a - av) + (bv - b);
}
__host__ __device__ __forceinline__ void two_prod(double a, double b, double& x, double& y)
{
    x = a * b;
    y = fma(a, b, -x);
}

// h = e + b for a nonoverlapping expansion e (increasing magnitude); zero
// components dropped.  Returns the length of h (h may not alias e).
__host__ __device__ inline int grow(const double* e, int elen, double b, double* h)
{
    double q = b;
    int k = 0;
    for (int i = 0; i < elen; ++i) {
        double s, hh;
        two_sum(q, e[i], s, hh);
        q = s;
        if (hh != 0) h[k++] = hh;
    }
    if (q != 0 || k == 0) h[k++] = q;
    return k;
}

// h = e + f (h may not alias e or f); tmp has room for elen + flen.
__host__ __device__ inline int sum(const double* e, int elen, const double* f, int flen, double* h, double* tmp)
{
    int hlen = elen;
    for (int i = 0; i < elen; ++i) h[i] = e[i];
    for (int j = 0; j < flen; ++j) {
        const int n = grow(h, hlen, f[j], tmp);
        for (int i = 0; i < n; ++i) h[i] = tmp[i];
        hlen = n;
    }
    return hlen;
}

// h = b * e (2 elen components at most; zeros dropped).
__host__ __device__ inline int scale(const double* e, int elen, double b, double* h)
{
    double q, hh;
    two_prod(e[0], b, q, hh);
    int k = 0;
    if (hh != 0) h[k++] = hh;
    for (int i = 1; i < elen; ++i) {
        double p1, p0, s;
        two_prod(e[i], b, p1, p0);
        two_sum(q, p0, s, hh);
        if (hh != 0) h[k++] = hh;
        fast_two_sum(p1, s, q, hh);
        if (hh != 0) h[k++] = hh;
    }
    if (q != 0 || k == 0) h[k++] = q;
    return k;
}

// h = e * f for short expansions (|e| * |f| * 2 <= 64 components).
__host__ __device__ inline int product(const double* e, int elen, const double* f, int flen, double* h)
{
    double part[32], acc[64], tmp[64];
    int alen = 1;
    acc[0] = 0;
    for (int j = 0; j < flen; ++j) {
        const int plen = scale(e, elen, f[j], part);
        alen = sum(acc, alen, part, plen, h, tmp);
        for (int i = 0; i < alen; ++i) acc[i] = h[i];
    }
    for (int i = 0; i < alen; ++i) h[i] = acc[i];
    return alen;
}

__host__ __device__ inline int sign_of(const double* e, int elen)
{
    for (int i = elen - 1; i >= 0; --i)
        if (e[i] != 0) return e[i] > 0 ? 1 : -1;
    return 0;
}

// Exact sign of the orientation determinant of (a - d, b - d, c - d).
__host__ __device__ inline int orient3d_exact(V3 a, V3 b, V3 c, V3 d)
{
    double ad[3][2], bd[3][2], cd[3][2];
    for (int k = 0; k < 3; ++k) {
        two_diff(comp(a, k), comp(d, k), ad[k][1], ad[k][0]);
        two_diff(comp(b, k), comp(d, k), bd[k][1], bd[k][0]);
        two_diff(comp(c, k), comp(d, k), cd[k][1], cd[k][0]);
    }
    // det = adx (bdy cdz - bdz cdy) + bdx (cdy adz - cdz ady) + cdx (ady bdz - adz bdy)
    const double(*rows[3])[2] = { ad, bd, cd };
    double total[200], acc[200], tmp[200];
    int tlen = 1;
    total[0] = 0;
    for (int r = 0; r < 3; ++r) {
        const double(*p)[2] = rows[r];
        const double(*q)[2] = rows[(r + 1) % 3];
        const double(*s)[2] = rows[(r + 2) % 3];
        double m1[16], m2[16], minor_[40], neg[16], term[80], t2[40];
        const int l1 = product(q[1], 2, s[2], 2, m1);
        const int l2 = product(q[2], 2, s[1], 2, m2);
        for (int i = 0; i < l2; ++i) neg[i] = -m2[i];
        const int lm = sum(m1, l1, neg, l2, minor_, t2);
        const int lt = product(minor_, lm, p[0], 2, term);
        tlen = sum(total, tlen, term, lt, acc, tmp);
        for (int i = 0; i < tlen; ++i) total[i] = acc[i];
    }
    return sign_of(total, tlen);
}

// Sign of the orientation of d against the plane through a, b, c:
// FP64 with Shewchuk's static error bound, exact when it cannot decide.
__host__ __device__ inline int orient3d(V3 a, V3 b, V3 c, V3 d)
{
    const double adx = a.x - d.x, bdx = b.x - d.x, cdx = c.x - d.x;
    const double ady = a.y - d.y, bdy = b.y - d.y, cdy = c.y - d.y;
    const double adz = a.z - d.z, bdz = b.z - d.z, cdz = c.z - d.z;
    const double bdxcdy = bdx * cdy, cdxbdy = cdx * bdy;
    const double cdxady = cdx * ady, adxcdy = adx * cdy;
    const double adxbdy = adx * bdy, bdxady = bdx * ady;
    const double det = adz * (bdxcdy - cdxbdy) + bdz * (cdxady - adxcdy) + cdz * (adxbdy - bdxady);
    const double permanent = (fabs(bdxcdy) + fabs(cdxbdy)) * fabs(adz) + (fabs(cdxady) + fabs(adxcdy)) * fabs(bdz)
        + (fabs(adxbdy) + fabs(bdxady)) * fabs(cdz);
    const double eps = 1.1102230246251565e-16; // 2^-53
    const double bound = (7.0 + 56.0 * eps) * eps * permanent;
    if (det > bound) return 1;
    if (-det > bound) return -1;
    return orient3d_exact(a, b, c, d);
}

// x = M^-1 r by Gaussian elimination with complete pivoting (the method of
// Eigen's FullPivLU, which the reference's float path uses): pivots at most
// 3 eps |largest pivot| count as zero, and the unknowns of a rank-deficient
// system beyond its rank are set to 0.
__host__ __device__ inline void full_pivot_solve(double M[3][3], double r[3], double x[3])
{
    int colp[3] = { 0, 1, 2 };
    int rank = 3;
    double maxpivot = 0;
    for (int k = 0; k < 3; ++k) {
        int pi = k, pj = k;
        double best = -1;
        for (int i = k; i < 3; ++i)
            for (int j = k; j < 3; ++j)
                if (fabs(M[i][j]) > best) {
                    best = fabs(M[i][j]);
                    pi = i;
                    pj = j;
                }
        if (k == 0) maxpivot = best;
        if (best <= 3 * 2.220446049250313e-16 * maxpivot || best == 0) {
            rank = k;
            break;
        }
        if (pi != k) {
            for (int j = 0; j < 3; ++j) {
                const double t = M[k][j];
                M[k][j] = M[pi][j];
                M[pi][j] = t;
            }
            const double t = r[k];
            r[k] = r[pi];
            r[pi] = t;
        }
        if (pj != k) {
            for (int i = 0; i < 3; ++i) {
                const double t = M[i][k];
                M[i][k] = M[i][pj];
                M[i][pj] = t;
            }
            const int t = colp[k];
            colp[k] = colp[pj];
            colp[pj] = t;
        }
        for (int i = k + 1; i < 3; ++i) {
            const double f = M[i][k] / M[k][k];
            M[i][k] = f;
            for (int j = k + 1; j < 3; ++j) M[i][j] -= f * M[k][j];
            r[i] -= f * r[k];
        }
    }
    double c[3] = { 0, 0, 0 };
    for (int k = rank - 1; k >= 0; --k) {
        double s = r[k];
        for (int j = k + 1; j < rank; ++j) s -= M[k][j] * c[j];
        c[k] = s / M[k][k];
    }
    for (int k = 0; k < 3; ++k) x[colp[k]] = c[k];
}

// is_edge_intersecting_triangle (geometry/intersection.cpp:120-147, the
// build without rational arithmetic): the edge misses if both endpoints lie
// strictly on the same side of the triangle's plane; otherwise the crossing
// point's barycentric coordinates (u, v) and edge parameter t decide.
__host__ __device__ inline bool edge_intersects_triangle(V3 e0, V3 e1, V3 t0, V3 t1, V3 t2)
{
    const int o1 = orient3d(t0, t1, t2, e0);
    const int o2 = orient3d(t0, t1, t2, e1);
    if (o1 != 0 && o2 != 0 && o1 == o2) return false;
    const V3 a = t1 - t0, b = t2 - t0, c = e0 - e1, rr = e0 - t0;
    double M[3][3] = { { a.x, b.x, c.x }, { a.y, b.y, c.y }, { a.z, b.z, c.z } };
    double r[3] = { rr.x, rr.y, rr.z };
    double uvt[3];
    full_pivot_solve(M, r, uvt);
    return uvt[0] >= 0.0 && uvt[1] >= 0.0 && uvt[0] + uvt[1] <= 1.0 && uvt[2] >= 0.0 && uvt[2] <= 1.0;
}

} // namespace exact
} // namespace ipcg
