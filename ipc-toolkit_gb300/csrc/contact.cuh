// contact.cuh — per-contact device math shared by the barrier kernels.
//
// Contact records and their stencils (ContactsView / Local), the barrier
// functions (barrier.cpp:11-154), the closed-form squared-distance
// derivatives, the edge-edge mollifier (edge_edge_mollifier.cpp:42-136), the
// FP32 forms of the mixed-precision modes, and the PSD projection of a local
// Hessian (eigen_ext.tpp:64-108).  barrier.cu (the per-type kernels behind
// friction and shape derivatives) and egh.cu (the cached-pattern energy /
// gradient / Hessian pipeline) both include it.
#pragma once
#include <cub/block/block_reduce.cuh>

#include <cmath>

#include "df64.cuh"
#include "geom.cuh"
#include "internal.cuh"

namespace ipcg {

namespace {
constexpr int BLOCK = 128;

struct ContactsView {
    int64_t nvv, nev, nee, nfv;
    const int2 *vv, *ev, *ee, *fv;
    const double *vv_w, *ev_w, *ee_w, *fv_w, *ee_eps;
    const int8_t* ee_dt;
};

enum : int { CT_VV = 0, CT_EV = 1, CT_EE = 2, CT_FV = 3 };

struct Local {
    int type, n, dtype;
    int vid[4];
    double w, eps;
};

__device__ __forceinline__ void load_contact(const ContactsView& cv, const int* __restrict__ E,
    const int* __restrict__ F, int64_t i, Local& c)
{
    if (i < cv.nvv) {
        const int2 p = cv.vv[i];
        c.type = CT_VV;
        c.n = 2;
        c.vid[0] = p.x;
        c.vid[1] = p.y;
        c.w = cv.vv_w[i];
        return;
    }
    i -= cv.nvv;
    if (i < cv.nev) {
        const int2 p = cv.ev[i];
        c.type = CT_EV;
        c.n = 3;
        c.vid[0] = p.y;
        c.vid[1] = E[2 * p.x];
        c.vid[2] = E[2 * p.x + 1];
        c.w = cv.ev_w[i];
        return;
    }
    i -= cv.nev;
    if (i < cv.nee) {
        const int2 p = cv.ee[i];
        c.type = CT_EE;
        c.n = 4;
        c.vid[0] = E[2 * p.x];
        c.vid[1] = E[2 * p.x + 1];
        c.vid[2] = E[2 * p.y];
        c.vid[3] = E[2 * p.y + 1];
        c.w = cv.ee_w[i];
        c.eps = cv.ee_eps[i];
        c.dtype = cv.ee_dt[i];
        return;
    }
    i -= cv.nee;
    const int2 p = cv.fv[i];
    c.type = CT_FV;
    c.n = 4;
    c.vid[0] = p.y;
    c.vid[1] = F[3 * p.x];
    c.vid[2] = F[3 * p.x + 1];
    c.vid[3] = F[3 * p.x + 2];
    c.w = cv.fv_w[i];
}

// ---- barrier functions (barrier.cpp:11-154, barrier.hpp:82-340) ----
// kind: 0 ClampedLogBarrier, 1 NormalizedBarrier<ClampedLogBarrier>,
// 2 ClampedLogSqBarrier, 3 CubicBarrier, 4 TwoStageBarrier; D = derivative
// order.  One template serves the FP64 path and the FP32 (mixed) path.
__host__ __device__ __forceinline__ double blog(double x) { return log(x); }
__host__ __device__ __forceinline__ float blog(float x) { return logf(x); }
__host__ __device__ __forceinline__ double binf(double) { return HUGE_VAL; }
__host__ __device__ __forceinline__ float binf(float) { return HUGE_VALF; }

template <int D, class T> __host__ __device__ __forceinline__ T clamped_log(T d, T dh)
{
    if (D == 0) {
        if (d <= T(0)) return binf(d);
        if (d >= dh) return T(0);
        const T dm = d - dh;
        return -dm * dm * blog(d / dh);
    }
    if (d <= T(0) || d >= dh) return T(0);
    if (D == 1) return (dh - d) * (T(2) * blog(d / dh) - dh / d + T(1));
    const T r = dh / d;
    return (r + T(2)) * r - T(2) * blog(d / dh) - T(3);
}
template <int D, class T> __host__ __device__ __forceinline__ T clamped_log_sq(T d, T dh)
{
    if (D == 0) {
        if (d <= T(0)) return binf(d);
        if (d >= dh) return T(0);
        const T dm = d - dh, l = blog(d / dh);
        return dm * dm * l * l;
    }
    if (d <= T(0) || d >= dh) return T(0);
    if (D == 1) {
        const T dm = d - dh, l = blog(d / dh);
        return T(2) * dm * l * (l + dm / d);
    }
    const T t0 = dh - d, t1 = blog(d / dh), t2 = (t0 * t0) / (d * d);
    return T(2) * ((t1 * t1) - (t1 - T(1)) * t2 - T(4) * t1 * t0 / d);
}
template <int D, class T> __host__ __device__ __forceinline__ T cubic(T d, T dh)
{
    if (!(d < dh)) return T(0);
    const T dm = d - dh;
    if (D == 0) return T(-2) / T(3) / dh * dm * dm * dm;
    if (D == 1) return T(-2) / dh * dm * dm;
    return T(4) * (T(1) - d / dh);
}
template <int D, class T> __host__ __device__ __forceinline__ T two_stage(T d, T dh)
{
    if (d >= dh) return T(0);
    if (d >= T(0.5) * dh) return D == 0 ? T(0.5) * (dh - d) * (dh - d) : (D == 1 ? d - dh : T(1));
    if (D == 0) return T(-0.25) * dh * dh * (blog(T(2) * d / dh) - T(0.5));
    if (D == 1) return T(-0.25) * dh * dh / d;
    return (T(0.25) * dh * dh) / (d * d);
}
// The other barriers are called out of line so that the default one adds
// no registers to the local-Hessian kernels.
template <int D, class T> __host__ __device__ __noinline__ T barrier_other(int kind, T d, T dh)
{
    switch (kind) {
    case 1: {
        // NormalizedBarrier: b(d / dh, 1) / dh^D
        const T v = clamped_log<D, T>(d / dh, T(1));
        return D == 0 ? v : (D == 1 ? v / dh : v / (dh * dh));
    }
    case 2: return clamped_log_sq<D, T>(d, dh);
    case 3: return cubic<D, T>(d, dh);
    case 4: return two_stage<D, T>(d, dh);
    default: return clamped_log<D, T>(d, dh);
    }
}
template <int D, class T> __host__ __device__ __forceinline__ T barrier_fn(int kind, T d, T dh)
{
    return kind == 0 ? clamped_log<D, T>(d, dh) : barrier_other<D, T>(kind, d, dh);
}

struct Params {
    double kappa, dmin2, xhat, scale; // scale = physical factor (or 1)
    int psd;
    int mixed; // point-triangle contacts in FP32 (IPCG_BARRIER_FP32_PT)
    int kind;  // barrier function (barrier_fn)
    int fp32_local; // every contact but near-parallel edge-edge ones in FP32 (IPCG_BARRIER_FP32_LOCAL)
};
// Barrier::units(x̂) (barrier.hpp): x̂² for every barrier but the normalized
// one, which is dimensionless (1).  The physical barrier scales by dhat / units.
__host__ __device__ inline double barrier_units(int kind, double xhat) { return kind == 1 ? 1.0 : xhat * xhat; }

// ---- FP32 point-triangle contacts (mixed precision) ----
// The point-plane squared distance d = N^2/D (N = a.(u x v), D = |u x v|^2,
// a = p - t0, u = t1 - t0, v = t2 - t0) and its derivatives, and the barrier
// derivatives, in FP32.  The relative vectors are formed in FP64 first, so
// FP32 only sees edge-sized numbers.  Used for triangles that are not
// degenerate (sin^2 of the corner angle above 1e-6); FV contacts whose
// triangles are, and every other contact type, stay FP64.
struct F3 {
    float x, y, z;
};
__device__ __forceinline__ F3 to_f3(V3 a) { return F3 { (float)a.x, (float)a.y, (float)a.z }; }
__device__ __forceinline__ F3 f3_cross(F3 a, F3 b)
{
    return F3 { a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x };
}
__device__ __forceinline__ float f3_dot(F3 a, F3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ float f3c(F3 a, int i) { return i == 0 ? a.x : (i == 1 ? a.y : a.z); }
__device__ __forceinline__ void f3_skew(F3 a, float M[3][3])
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

// FP64 test of the triangle's corner angle at t0 (u = t1 - t0, v = t2 - t0).
__device__ __forceinline__ bool fv_fp32_ok(const V3* x)
{
    const V3 u = x[2] - x[1], v = x[3] - x[1];
    return sqnorm(cross(u, v)) > 1e-6 * sqnorm(u) * sqnorm(v);
}

// d = N^2 / D, reduced gradient g (9, in r = (a, u, v)) and Hessian H (81
// or null) in FP32.  w = u x v, N = a . w and D = |w|^2 come from FP64: N is
// the cancellation-prone quantity (it is d |w|, small next to |a| |w| for a
// close contact), so rounding it from FP64 keeps d, g and H at FP32 relative
// accuracy however small the distance is against the edge lengths.
__device__ float triple_quot_f(F3 a, F3 u, F3 v, F3 w, float Nn, float D, float* g, float* H)
{
    const float iD = 1.0f / D;
    const F3 gNa = w, gNu = f3_cross(v, a), gNv = f3_cross(a, u);
    const F3 cvw = f3_cross(v, w), cwu = f3_cross(w, u);
    float gN[9], gD[9];
    for (int i = 0; i < 3; ++i) {
        gN[i] = f3c(gNa, i);
        gN[3 + i] = f3c(gNu, i);
        gN[6 + i] = f3c(gNv, i);
        gD[i] = 0;
        gD[3 + i] = 2.0f * f3c(cvw, i);
        gD[6 + i] = 2.0f * f3c(cwu, i);
    }
    const float c1 = 2 * Nn * iD, c2 = Nn * Nn * iD * iD;
    for (int i = 0; i < 9; ++i) g[i] = c1 * gN[i] - c2 * gD[i];
    if (H) {
        float Sv[3][3], Su[3][3], Sa[3][3], Sw[3][3];
        f3_skew(v, Sv);
        f3_skew(u, Su);
        f3_skew(a, Sa);
        f3_skew(w, Sw);
        float HN[81], HD[81];
        for (int i = 0; i < 81; ++i) {
            HN[i] = 0;
            HD[i] = 0;
        }
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) {
                HN[i * 9 + 3 + j] = HN[(3 + j) * 9 + i] = -Sv[i][j];
                HN[i * 9 + 6 + j] = HN[(6 + j) * 9 + i] = Su[i][j];
                HN[(3 + i) * 9 + 6 + j] = HN[(6 + j) * 9 + 3 + i] = -Sa[i][j];
                float uu = 0, vv = 0, uv = 0;
                for (int k = 0; k < 3; ++k) {
                    uu += Sv[k][i] * Sv[k][j];
                    vv += Su[k][i] * Su[k][j];
                    uv -= Sv[k][i] * Su[k][j];
                }
                HD[(3 + i) * 9 + 3 + j] = 2 * uu;
                HD[(6 + i) * 9 + 6 + j] = 2 * vv;
                HD[(3 + i) * 9 + 6 + j] = HD[(6 + j) * 9 + 3 + i] = 2 * (uv - Sw[i][j]);
            }
        const float iD2 = iD * iD;
        const float k1 = 2 * iD, k2 = 2 * Nn * iD, k3 = 2 * Nn * iD2, k4 = Nn * Nn * iD2, k5 = 2 * Nn * Nn * iD2 * iD;
        for (int i = 0; i < 9; ++i)
            for (int j = 0; j < 9; ++j)
                H[i * 9 + j] = k1 * gN[i] * gN[j] + k2 * HN[i * 9 + j] - k3 * (gN[i] * gD[j] + gD[i] * gN[j])
                    - k4 * HD[i * 9 + j] + k5 * gD[i] * gD[j];
    }
    return Nn * Nn * iD;
}

// FV contact in FP32: stencil gradient (12) and Hessian (144 or null) of d
// as floats; returns the squared distance d from FP64.
__device__ double fv_local_f(const V3* x, float* g, float* H)
{
    // a = p - t0, u = t1 - t0, v = t2 - t0 (FP64 differences, then FP32);
    // w = u x v, N = a . w and D = |w|^2 in FP64, d = N^2 / D in FP64
    const V3 a64 = x[0] - x[1], u64 = x[2] - x[1], v64 = x[3] - x[1];
    const V3 w64 = cross(u64, v64);
    const double N64 = dot(a64, w64), D64 = sqnorm(w64);
    const F3 a = to_f3(a64), u = to_f3(u64), v = to_f3(v64);
    float gr[9], Hr[81];
    triple_quot_f(a, u, v, to_f3(w64), (float)N64, (float)D64, gr, H ? Hr : nullptr);
    const double d = N64 * N64 / D64;
    // expand to the stencil (p, t0, t1, t2): reduced vectors (0-1, 2-1, 3-1)
    const int pos[3] = { 0, 2, 3 };
    for (int i = 0; i < 12; ++i) g[i] = 0;
    for (int k = 0; k < 3; ++k)
        for (int c = 0; c < 3; ++c) {
            g[3 * pos[k] + c] += gr[3 * k + c];
            g[3 + c] -= gr[3 * k + c];
        }
    if (H) {
        for (int i = 0; i < 144; ++i) H[i] = 0;
        for (int k = 0; k < 3; ++k)
            for (int l = 0; l < 3; ++l)
                for (int c = 0; c < 3; ++c)
                    for (int e = 0; e < 3; ++e) {
                        const float h = Hr[(3 * k + c) * 9 + 3 * l + e];
                        H[(3 * pos[k] + c) * 12 + 3 * pos[l] + e] += h;
                        H[(3 * pos[k] + c) * 12 + 3 + e] -= h;
                        H[(3 + c) * 12 + 3 * pos[l] + e] -= h;
                        H[(3 + c) * 12 + 3 + e] += h;
                    }
    }
    return d;
}

// ---- closed-form squared-distance derivatives ----
__device__ __forceinline__ void skew(V3 a, double M[3][3])
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

// Accumulate reduced derivatives into stencil coordinates: reduced vector k
// is x[pos[k]] - x[neg[k]].
template <int M>
__device__ __forceinline__ void expand_g(int N, const int* pos, const int* neg, const double* gr, double* g)
{
    for (int i = 0; i < N; ++i) g[i] = 0;
    for (int k = 0; k < M; ++k)
        for (int c = 0; c < 3; ++c) {
            g[3 * pos[k] + c] += gr[3 * k + c];
            g[3 * neg[k] + c] -= gr[3 * k + c];
        }
}
template <int M>
__device__ __forceinline__ void expand_h(int N, const int* pos, const int* neg, const double* Hr, double* H)
{
    for (int i = 0; i < N * N; ++i) H[i] = 0;
    for (int k = 0; k < M; ++k)
        for (int l = 0; l < M; ++l)
            for (int c = 0; c < 3; ++c)
                for (int e = 0; e < 3; ++e) {
                    const double h = Hr[(3 * k + c) * (3 * M) + 3 * l + e];
                    H[(3 * pos[k] + c) * N + 3 * pos[l] + e] += h;
                    H[(3 * pos[k] + c) * N + 3 * neg[l] + e] -= h;
                    H[(3 * neg[k] + c) * N + 3 * pos[l] + e] -= h;
                    H[(3 * neg[k] + c) * N + 3 * neg[l] + e] += h;
                }
}

// d = N²/D, N = a·(u×v), D = |u×v|²; r = (a,u,v)
__device__ void triple_quot(V3 a, V3 u, V3 v, double* g, double* H /*81 or null*/)
{
    const V3 w = cross(u, v);
    const double Nn = dot(a, w);
    const double D = sqnorm(w);
    const double iD = 1.0 / D;
    const V3 gNa = w, gNu = cross(v, a), gNv = cross(a, u);
    const V3 gDu = cross(v, w) * 2.0, gDv = cross(w, u) * 2.0;
    double gN[9], gD[9];
    for (int i = 0; i < 3; ++i) {
        gN[i] = comp(gNa, i);
        gN[3 + i] = comp(gNu, i);
        gN[6 + i] = comp(gNv, i);
        gD[i] = 0;
        gD[3 + i] = comp(gDu, i);
        gD[6 + i] = comp(gDv, i);
    }
    const double c1 = 2 * Nn * iD, c2 = Nn * Nn * iD * iD;
    for (int i = 0; i < 9; ++i) g[i] = c1 * gN[i] - c2 * gD[i];
    if (!H) return;
    double Sv[3][3], Su[3][3], Sa[3][3], Sw[3][3];
    skew(v, Sv);
    skew(u, Su);
    skew(a, Sa);
    skew(w, Sw);
    double HN[81], HD[81];
    for (int i = 0; i < 81; ++i) {
        HN[i] = 0;
        HD[i] = 0;
    }
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            HN[i * 9 + 3 + j] = HN[(3 + j) * 9 + i] = -Sv[i][j];
            HN[i * 9 + 6 + j] = HN[(6 + j) * 9 + i] = Su[i][j];
            HN[(3 + i) * 9 + 6 + j] = HN[(6 + j) * 9 + 3 + i] = -Sa[i][j];
            double uu = 0, vv = 0, uv = 0;
            for (int k = 0; k < 3; ++k) {
                uu += Sv[k][i] * Sv[k][j];
                vv += Su[k][i] * Su[k][j];
                uv -= Sv[k][i] * Su[k][j];
            }
            HD[(3 + i) * 9 + 3 + j] = 2 * uu;
            HD[(6 + i) * 9 + 6 + j] = 2 * vv;
            HD[(3 + i) * 9 + 6 + j] = HD[(6 + j) * 9 + 3 + i] = 2 * (uv - Sw[i][j]);
        }
    const double iD2 = iD * iD;
    const double k1 = 2 * iD, k2 = 2 * Nn * iD, k3 = 2 * Nn * iD2, k4 = Nn * Nn * iD2, k5 = 2 * Nn * Nn * iD2 * iD;
    for (int i = 0; i < 9; ++i)
        for (int j = 0; j < 9; ++j)
            H[i * 9 + j] = k1 * gN[i] * gN[j] + k2 * HN[i * 9 + j] - k3 * (gN[i] * gD[j] + gD[i] * gN[j])
                - k4 * HD[i * 9 + j] + k5 * gD[i] * gD[j];
}

// D = |u×v|² in r = (u,v)
__device__ void cross_sq(V3 u, V3 v, double* g, double* H /*36 or null*/)
{
    const V3 w = cross(u, v);
    const V3 gu = cross(v, w) * 2.0, gv = cross(w, u) * 2.0;
    for (int i = 0; i < 3; ++i) {
        g[i] = comp(gu, i);
        g[3 + i] = comp(gv, i);
    }
    if (!H) return;
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
                uv -= Sv[k][i] * Su[k][j];
            }
            H[i * 6 + j] = 2 * uu;
            H[(3 + i) * 6 + 3 + j] = 2 * vv;
            H[i * 6 + 3 + j] = H[(3 + j) * 6 + i] = 2 * (uv - Sw[i][j]);
        }
}

// d = |a×b|²/|b−a|² in r = (a,b)
__device__ void point_line_r(V3 a, V3 b, double* g, double* H /*36 or null*/)
{
    const V3 c = cross(a, b);
    const double P = sqnorm(c);
    const V3 e = b - a;
    const double L = sqnorm(e);
    const double iL = 1.0 / L;
    double gP[6], gL[6];
    const V3 gPa = cross(b, c) * 2.0, gPb = cross(c, a) * 2.0;
    for (int i = 0; i < 3; ++i) {
        gP[i] = comp(gPa, i);
        gP[3 + i] = comp(gPb, i);
        gL[i] = -2 * comp(e, i);
        gL[3 + i] = 2 * comp(e, i);
    }
    const double iL2 = iL * iL;
    for (int i = 0; i < 6; ++i) g[i] = gP[i] * iL - P * gL[i] * iL2;
    if (!H) return;
    double Sa[3][3], Sb[3][3], Sc[3][3];
    skew(a, Sa);
    skew(b, Sb);
    skew(c, Sc);
    // ∇²P = 2(JᵀJ + Σ c_k ∇²c_k) with J = [-[b]×, [a]×], ∂²c_k/∂a_i∂b_j = ε_kij
    double HP[36];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            double aa = 0, bb = 0, ab = 0;
            for (int k = 0; k < 3; ++k) {
                aa += Sb[k][i] * Sb[k][j];
                bb += Sa[k][i] * Sa[k][j];
                ab -= Sb[k][i] * Sa[k][j];
            }
            HP[i * 6 + j] = 2 * aa;
            HP[(3 + i) * 6 + 3 + j] = 2 * bb;
            HP[i * 6 + 3 + j] = HP[(3 + j) * 6 + i] = 2 * (ab - Sc[i][j]);
        }
    // ∇²L = 2 [[I, -I], [-I, I]]
    const double k5 = 2 * P * iL2 * iL;
    for (int r = 0; r < 6; ++r)
        for (int q = 0; q < 6; ++q) {
            const double hl = (r % 3 == q % 3) ? ((r < 3) == (q < 3) ? 2.0 : -2.0) : 0.0;
            H[r * 6 + q] = HP[r * 6 + q] * iL - (gP[r] * gL[q] + gL[r] * gP[q]) * iL2 - P * hl * iL2
                + k5 * gL[r] * gL[q];
        }
}

// stencil-local squared distance + derivatives (H may be null)
__device__ double pp_local(const V3* x, int N, int i, int j, double* g, double* H)
{
    const V3 r = x[i] - x[j];
    const double gr[3] = { 2 * r.x, 2 * r.y, 2 * r.z };
    const int pos[1] = { i }, neg[1] = { j };
    expand_g<1>(N, pos, neg, gr, g);
    if (H) {
        const double Hr[9] = { 2, 0, 0, 0, 2, 0, 0, 0, 2 };
        expand_h<1>(N, pos, neg, Hr, H);
    }
    return point_point_distance(x[i], x[j]);
}
__device__ double pl_local(const V3* x, int N, int p, int e0, int e1, double* g, double* H)
{
    double gr[6], Hr[36];
    point_line_r(x[e0] - x[p], x[e1] - x[p], gr, H ? Hr : nullptr);
    const int pos[2] = { e0, e1 }, neg[2] = { p, p };
    expand_g<2>(N, pos, neg, gr, g);
    if (H) expand_h<2>(N, pos, neg, Hr, H);
    return point_line_distance(x[p], x[e0], x[e1]);
}
__device__ double pplane_local(const V3* x, double* g, double* H)
{
    double gr[9], Hr[81];
    triple_quot(x[0] - x[1], x[2] - x[1], x[3] - x[1], gr, H ? Hr : nullptr);
    const int pos[3] = { 0, 2, 3 }, neg[3] = { 1, 1, 1 };
    expand_g<3>(12, pos, neg, gr, g);
    if (H) expand_h<3>(12, pos, neg, Hr, H);
    return point_plane_distance(x[0], x[1], x[2], x[3]);
}
__device__ double ll_local(const V3* x, double* g, double* H)
{
    double gr[9], Hr[81];
    triple_quot(x[2] - x[0], x[1] - x[0], x[3] - x[2], gr, H ? Hr : nullptr);
    const int pos[3] = { 2, 1, 3 }, neg[3] = { 0, 0, 2 };
    expand_g<3>(12, pos, neg, gr, g);
    if (H) expand_h<3>(12, pos, neg, Hr, H);
    return line_line_distance(x[0], x[1], x[2], x[3]);
}
__device__ double ee_local(const V3* x, int dtype, double* g, double* H)
{
    switch (dtype) {
    case EA0_EB0: return pp_local(x, 12, 0, 2, g, H);
    case EA0_EB1: return pp_local(x, 12, 0, 3, g, H);
    case EA1_EB0: return pp_local(x, 12, 1, 2, g, H);
    case EA1_EB1: return pp_local(x, 12, 1, 3, g, H);
    case EA_EB0: return pl_local(x, 12, 2, 0, 1, g, H);
    case EA_EB1: return pl_local(x, 12, 3, 0, 1, g, H);
    case EA0_EB: return pl_local(x, 12, 0, 2, 3, g, H);
    case EA1_EB: return pl_local(x, 12, 1, 2, 3, g, H);
    default: return ll_local(x, g, H);
    }
}
__device__ double contact_distance(const Local& c, const V3* x, double* g, double* H)
{
    switch (c.type) {
    case CT_VV: return pp_local(x, 6, 0, 1, g, H);
    case CT_EV: return pl_local(x, 9, 0, 1, 2, g, H);
    case CT_EE: return ee_local(x, c.dtype, g, H);
    default: return pplane_local(x, g, H);
    }
}

// EE mollifier m(x) (edge_edge_mollifier.cpp:42-136); gm/Hm filled iff active
__device__ double mollifier(const Local& c, const V3* x, double* gm, double* Hm, bool& active)
{
    active = false;
    if (c.type != CT_EE) return 1.0;
    const double s = ee_cross_sqnorm(x[0], x[1], x[2], x[3]);
    if (!(s < c.eps)) return 1.0;
    active = true;
    const double xe = s / c.eps;
    const double m = (-xe + 2) * xe;
    if (!gm) return m;
    const double inv = 1 / c.eps;
    const double m1 = 2 * inv * fma(-inv, s, 1.0);
    double gr[6], Hr[36];
    cross_sq(x[1] - x[0], x[3] - x[2], gr, Hm ? Hr : nullptr);
    const int pos[2] = { 1, 3 }, neg[2] = { 0, 2 };
    double gs[12];
    expand_g<2>(12, pos, neg, gr, gs);
    for (int i = 0; i < 12; ++i) gm[i] = m1 * gs[i];
    if (Hm) {
        const double m2 = -2 / (c.eps * c.eps);
        expand_h<2>(12, pos, neg, Hr, Hm);
        for (int i = 0; i < 12; ++i)
            for (int j = 0; j < 12; ++j) Hm[i * 12 + j] = m1 * Hm[i * 12 + j] + m2 * gs[i] * gs[j];
    }
    return m;
}

// ---- PSD projection (eigen_ext.tpp:64-108) -------------------------------
// The local Hessian annihilates rigid translations (per coordinate its rows
// sum to zero over the stencil's vertices), so it is projected in the
// 3(n-1)-dimensional translation-free subspace spanned by orthonormal vertex
// contrasts: M = C H C^T (at most 9 x 9), and H+ = H - f sum_{lam<0} lam w w^T
// with w = C^T q over the negative eigenpairs (lam, q) of M (f = 1 to clamp,
// 2 for the absolute value).  M = Q_h T Q_h^T (Householder), T = G D G^T
// (implicit QL with Wilkinson shifts, G = G_1 ... G_R plane rotations).
// Only the negative eigenvectors are formed: q_i = Q_h G_1 ... G_R e_i,
// replaying the recorded rotations on e_i, which costs a few hundred flops
// per vector instead of updating all of Q at every rotation.
// Arithmetic of the PSD solver: FP64 (the plain path), or df64 (pairs of
// FP32, about 48 bits) with exact power-of-two rescaling so that FP32's
// exponent range never clips a square.  in() reads an FP64 entry scaled by
// 2^-sc, out() returns a df64 value scaled back to FP64.
template <class T> struct PsdReal;
template <> struct PsdReal<double> {
    static constexpr bool rescale = false;
    __device__ static double eps() { return 2.220446049250313e-16; }
    __device__ static double eps_norm() { return 2.220446049250313e-16; } // 2^-52
    __device__ static double tiny() { return 1e-300; }
    __device__ static double in(double x, int) { return x; }
    __device__ static double out(double x, int) { return x; }
    template <class Acc> __device__ static int scale_of(const Acc&, int) { return 0; }
    // deflation test of a QL off-diagonal entry e between diagonal entries
    // d0 and d1, on the exponent bits (the integer pipe; GB300's FP64 pipe
    // is the projection's limit): e is negligible when its exponent is at
    // least 52 below the larger neighbour's (|e| < 2^-51 max(|d0|, |d1|), the
    // reference's eps (|d0| + |d1|) within a factor 2), not above the
    // floor's (2^-52 of the tridiagonal matrix's norm, within a factor 2),
    // or when it is zero or subnormal
    __device__ static int expo(double x) { return (__double2hiint(x) >> 20) & 0x7ff; }
    __device__ static bool negligible(double e, double d0, double d1, double, double floor_)
    {
        const int ee = expo(e);
        return ee == 0 || ee + 52 <= max(expo(d0), expo(d1)) || ee <= expo(floor_);
    }
    __device__ static bool is_zero(double x) { return (__double_as_longlong(x) << 1) == 0; }
    // Wilkinson shift of the trailing 2x2 block [[d0, b], [b, d1]]: its
    // eigenvalue closer to d1
    __device__ static double shift(double d0, double d1, double b)
    {
        const double td = 0.5 * (d0 - d1);
        double mu = d1;
        if (td == 0) mu -= fabs(b);
        else {
            const double h = hypot(td, b);
            mu -= b * b / (td + (td > 0 ? h : -h));
        }
        return mu;
    }
};
template <> struct PsdReal<dd> {
    static constexpr bool rescale = true;
    __device__ static dd eps() { return dd { 7.1e-15f, 0.f }; }
    __device__ static dd eps_norm() { return dd { 2.842170943040401e-14f, 0.f }; } // 2^-45
    __device__ static dd tiny() { return dd { 1e-36f, 0.f }; }
    __device__ static dd in(double x, int sc) { return dd_from_double(scalbn(x, -sc)); }
    __device__ static double out(dd x, int sc) { return scalbn(dd_to_double(x), sc); }
    // exponent of the largest |entry| (from the FP64 bit patterns, integer ops)
    template <class Acc> __device__ static int scale_of(const Acc& hs, int N)
    {
        unsigned long long mx = 0;
        for (int k = 0; k < N * N; ++k) {
            const unsigned long long b = (unsigned long long)__double_as_longlong(hs(k)) & 0x7fffffffffffffffULL;
            mx = b > mx ? b : mx;
        }
        return mx == 0 ? 0 : (int)(mx >> 52) - 1022;
    }
    // the deflation test and the shift only steer the iteration (neither
    // enters the result but through where it stops), so they run in FP32
    // on the leading parts
    __device__ static bool is_zero(dd x) { return x.hi == 0.f; }
    __device__ static bool negligible(dd e, dd d0, dd d1, dd eps, dd floor_)
    {
        const float ae = fabsf(e.hi);
        return ae <= eps.hi * (fabsf(d0.hi) + fabsf(d1.hi)) || ae <= tiny().hi || ae <= floor_.hi;
    }
    __device__ static dd shift(dd d0, dd d1, dd b)
    {
        // d1 minus an FP32 correction (exact in df64)
        const float td = 0.5f * (d0.hi - d1.hi), bf = b.hi;
        float corr;
        if (td == 0.f) corr = fabsf(bf);
        else {
            const float h = hypotf(td, bf);
            corr = bf * bf / (td + (td > 0.f ? h : -h));
        }
        return d1 - dd { corr, 0.f };
    }
};

constexpr int MAXR = 9;
constexpr int MAXROT = 128; // recorded rotations; beyond, Q is accumulated
// The projection keeps the smaller of the negative and the non-negative
// eigenpair sets: at most MAXR / 2 pairs.
constexpr int MAXPAIRS = MAXR / 2;

template <class T> __device__ bool sym_eig_impl(int n, T* A /*MAXR*MAXR, full symmetric*/, T* d, T* Q, T* rc, T* rs,
    int8_t* rk, int& nrot, T* htau, unsigned wm)
{
    // Householder tridiagonalisation; reflector k is I - htau[k] v v^T with
    // v[k+1..n) kept in A[k+1..n)[k], the column it annihilates (the updates
    // below touch only rows and columns past k)
    T e[MAXR];
    for (int k = 0; k + 2 < n; ++k) {
        T sig = 0;
        for (int i = k + 2; i < n; ++i) sig += A[i * MAXR + k] * A[i * MAXR + k];
        T x0 = A[(k + 1) * MAXR + k];
        htau[k] = 0;
        if (sig == 0) {
            e[k] = x0;
            continue;
        }
        // df64: the column is scaled by a power of two (exact) so that its
        // squares stay inside FP32's exponent range; the reflector
        // I - tau v v^T is unchanged and alpha is scaled back
        int cex = 0;
        if constexpr (PsdReal<T>::rescale) {
            T amax = fabs(x0);
            for (int i = k + 2; i < n; ++i) amax = dmax(amax, fabs(A[i * MAXR + k]));
            cex = pow2_exp(amax);
            x0 = scale2(x0, -cex);
            sig = T(0);
            for (int i = k + 2; i < n; ++i) {
                A[i * MAXR + k] = scale2(A[i * MAXR + k], -cex);
                sig += A[i * MAXR + k] * A[i * MAXR + k];
            }
        }
        const T nx = sqrt(x0 * x0 + sig);
        const T alpha = (x0 >= 0) ? -nx : nx;
        const T v0 = x0 - alpha;
        A[(k + 1) * MAXR + k] = v0;
        T p[MAXR];
        const T tau = 2.0 / (v0 * v0 + sig);
        T K = 0;
        for (int i = k + 1; i < n; ++i) {
            T s = 0;
            for (int j = k + 1; j < n; ++j) s += A[i * MAXR + j] * A[j * MAXR + k];
            p[i] = tau * s;
            K += p[i] * A[i * MAXR + k];
        }
        K *= 0.5 * tau;
        for (int i = k + 1; i < n; ++i) p[i] -= K * A[i * MAXR + k];
        // the update is symmetric: form the upper triangle, mirror it
        for (int i = k + 1; i < n; ++i)
            for (int j = i; j < n; ++j) {
                const T a = A[i * MAXR + j] - (A[i * MAXR + k] * p[j] + p[i] * A[j * MAXR + k]);
                A[i * MAXR + j] = a;
                A[j * MAXR + i] = a;
            }
        if constexpr (PsdReal<T>::rescale) e[k] = scale2(alpha, cex);
        else e[k] = alpha;
        htau[k] = tau;
    }
    if (n >= 2) e[n - 2] = A[(n - 1) * MAXR + n - 2];
    e[n - 1] = 0;
    for (int i = 0; i < n; ++i) d[i] = A[i * MAXR + i];
    nrot = 0;
    bool record = true; // false once MAXROT is exceeded: then Q holds G
    // an off-diagonal entry is zero when it is negligible next to its two
    // diagonal neighbours, or next to the whole tridiagonal matrix (the
    // latter as EISPACK's tql2 tests it: a QL sweep cannot drive an entry
    // below its own rounding of the matrix's largest entries, which decides
    // when the neighbours are small, and more so in df64)
    const T eps = PsdReal<T>::eps();
    T tnorm = T(0);
    for (int i = 0; i < n; ++i) tnorm = dmax(tnorm, fabs(d[i]) + fabs(e[i]));
    const T floor_ = PsdReal<T>::eps_norm() * tnorm;
    // The lanes of warp mask wm (0: this lane alone) iterate in step: the
    // loop runs while any of them still has an unreduced block and a lane
    // that has finished idles through the rest.  Left to themselves the
    // lanes leave the loop at different iterations and stay apart for the
    // rest of the projection, each group issuing it on its own.
    int end = n - 1, iter = 0;
    bool ok = true;
    for (;;) {
        if (wm ? !__any_sync(wm, end > 0) : end <= 0) break;
        // deflate at the bottom, then walk up to the top of the unreduced
        // block; an entry is set to zero where the walks stop at it (the
        // entries above the block are tested when their block's turn comes,
        // with the same neighbours: the sweeps below do not touch them)
        int start = 0;
        bool sweep = false;
        if (end > 0) {
            while (end > 0
                && (PsdReal<T>::is_zero(e[end - 1])
                    || PsdReal<T>::negligible(e[end - 1], d[end - 1], d[end], eps, floor_))) {
                e[end - 1] = 0;
                --end;
            }
            if (end > 0 && ++iter > 40 * n) {
                ok = false;
                end = 0;
            }
            if (end > 0) {
                start = end - 1;
                while (start > 0 && !PsdReal<T>::is_zero(e[start - 1])
                    && !PsdReal<T>::negligible(e[start - 1], d[start - 1], d[start], eps, floor_))
                    --start;
                if (start > 0) e[start - 1] = 0;
                if (record && nrot + (end - start) > MAXROT) {
                    // too many rotations to record: form G from those so far
                    // and accumulate the rest into it
                    for (int i = 0; i < n; ++i)
                        for (int j = 0; j < n; ++j) Q[i * MAXR + j] = (i == j) ? 1.0 : 0.0;
                    for (int r = 0; r < nrot; ++r) {
                        const int k = rk[r];
                        const T c = rc[r], s = rs[r];
                        for (int q = 0; q < n; ++q) {
                            const T qa = Q[q * MAXR + k], qb = Q[q * MAXR + k + 1];
                            Q[q * MAXR + k] = c * qa - s * qb;
                            Q[q * MAXR + k + 1] = s * qa + c * qb;
                        }
                    }
                    record = false;
                    nrot = -1;
                }
                sweep = true;
            }
        }
        // the lanes meet again before the sweeps (each of its own length)
        if (wm) __syncwarp(wm);
        if (!sweep) continue;
        // One implicitly shifted QL sweep down the block [start, end], in the
        // carried form of the EISPACK tql / Numerical Recipes tqli recurrence
        // (mirrored: the bulge is chased from the top, the shift is taken at
        // the bottom).  Per step, (c, s) from one reciprocal square root of
        // f^2 + g^2 (entries of a local Hessian, far from overflow) and the
        // carried correction p of the diagonal.
        const T mu = PsdReal<T>::shift(d[end - 1], d[end], e[end - 1]);
        T g = d[start] - mu, s = 1, c = 1, p = 0;
        bool whole = true;
        for (int k = start; k < end; ++k) {
            const T f = s * e[k], b = c * e[k];
            T r = 0;
            bool zero;
            if constexpr (PsdReal<T>::rescale) {
                // df64: (f, g) scaled by a power of two before squaring
                const T fg = dmax(fabs(f), fabs(g));
                zero = fg == T(0);
                if (!zero) {
                    const int rex = pow2_exp(fg);
                    const T fs = scale2(f, -rex), gs = scale2(g, -rex);
                    const T r2 = fs * fs + gs * gs, ir = rsqrt(r2);
                    r = scale2(r2 * ir, rex);
                    s = fs * ir;
                    c = gs * ir;
                }
            } else {
                const T r2 = f * f + g * g;
                zero = r2 == 0;
                if (!zero) {
                    const T ir = rsqrt(r2);
                    r = r2 * ir;
                    s = f * ir;
                    c = g * ir;
                }
            }
            if (k > start) e[k - 1] = r;
            if (zero) {
                // the block split exactly above k
                d[k] = d[k] - p;
                whole = false;
                break;
            }
            g = d[k] - p;
            const T q = (d[k + 1] - g) * s + 2 * c * b;
            p = s * q;
            d[k] = g + p;
            g = c * q - b;
            // the step's rotation of coordinates (k, k + 1): cos c, sin -s
            if (record) {
                rc[nrot] = c;
                rs[nrot] = -s;
                rk[nrot] = (int8_t)k;
                ++nrot;
            } else {
                for (int j = 0; j < n; ++j) {
                    const T qa = Q[j * MAXR + k], qb = Q[j * MAXR + k + 1];
                    Q[j * MAXR + k] = c * qa + s * qb;
                    Q[j * MAXR + k + 1] = c * qb - s * qa;
                }
            }
        }
        if (whole) {
            d[end] = d[end] - p;
            e[end - 1] = g;
        }
    }
    return ok;
}

// Eigenvectors idx[0..cnt) of M, rows of Y (stride MAXR): Q_h G e_i.  G e_i
// comes from the recorded rotations, applied last first to all cnt vectors in
// one pass (each rotation loaded once), or, if they were not recorded
// (nrot < 0), from column i of Q; then the Householder reflectors kept in A's
// lower columns, H_{n-3} first.  wm: the lanes of this warp that call it
// together (cnt may be 0), which meet again after the rotations and after
// every reflector, or 0.
template <class T> __device__ void eigvecs_impl(int n, const int* idx, int cnt, const T* Q, const T* rc, const T* rs,
    const int8_t* rk, int nrot, const T* A, const T* htau, T* Y, unsigned wm)
{
    for (int t = 0; t < cnt; ++t)
        for (int q = 0; q < n; ++q)
            Y[t * MAXR + q] = nrot >= 0 ? (q == idx[t] ? 1.0 : 0.0) : Q[q * MAXR + idx[t]];
    // FP64: the pair loops run MAXPAIRS times with a predicate (unrolled);
    // df64: as counted loops (its operations are long: unrolled copies
    // would not fit the instruction cache)
    for (int r = (cnt > 0 ? nrot : 0) - 1; r >= 0; --r) {
        const int k = rk[r];
        const T c = rc[r], s = rs[r];
        const auto rotate = [&](int t) {
            T* y = Y + t * MAXR;
            const T ya = y[k], yb = y[k + 1];
            y[k] = c * ya + s * yb;
            y[k + 1] = c * yb - s * ya;
        };
        if constexpr (PsdReal<T>::rescale) {
            for (int t = 0; t < cnt; ++t) rotate(t);
        } else {
#pragma unroll
            for (int t = 0; t < MAXPAIRS; ++t)
                if (t < cnt) rotate(t);
        }
    }
    if (wm) __syncwarp(wm);
    for (int k = n - 3; k >= 0; --k) {
        const auto reflect = [&](int t) {
            T* y = Y + t * MAXR;
            T s = 0;
            for (int q = k + 1; q < n; ++q) s += A[q * MAXR + k] * y[q];
            s *= htau[k];
            for (int q = k + 1; q < n; ++q) y[q] -= s * A[q * MAXR + k];
        };
        if (htau[k] != 0) {
            if constexpr (PsdReal<T>::rescale) {
                for (int t = 0; t < cnt; ++t) reflect(t);
            } else {
#pragma unroll
                for (int t = 0; t < MAXPAIRS; ++t)
                    if (t < cnt) reflect(t);
            }
        }
        if (wm) __syncwarp(wm);
    }
}

// The df64 solver is long (each df64 operation is tens of FP32
// instructions): one out-of-line copy serves every stencil size, which keeps
// the kernel inside the instruction cache; the FP64 solver is inlined.
__device__ __noinline__ bool sym_eig_dd(int n, dd* A, dd* d, dd* Q, dd* rc, dd* rs, int8_t* rk, int& nrot, dd* htau,
    unsigned wm)
{
    return sym_eig_impl<dd>(n, A, d, Q, rc, rs, rk, nrot, htau, wm);
}
__device__ __noinline__ void eigvecs_dd(int n, const int* idx, int cnt, const dd* Q, const dd* rc, const dd* rs,
    const int8_t* rk, int nrot, const dd* A, const dd* htau, dd* Y, unsigned wm)
{
    eigvecs_impl<dd>(n, idx, cnt, Q, rc, rs, rk, nrot, A, htau, Y, wm);
}
template <class T> __device__ __forceinline__ bool sym_eig(int n, T* A, T* d, T* Q, T* rc, T* rs, int8_t* rk,
    int& nrot, T* htau, unsigned wm)
{
    if constexpr (PsdReal<T>::rescale) return sym_eig_dd(n, A, d, Q, rc, rs, rk, nrot, htau, wm);
    else return sym_eig_impl<T>(n, A, d, Q, rc, rs, rk, nrot, htau, wm);
}
template <class T> __device__ __forceinline__ void eigvecs(int n, const int* idx, int cnt, const T* Q, const T* rc,
    const T* rs, const int8_t* rk, int nrot, const T* A, const T* htau, T* Y, unsigned wm)
{
    if constexpr (PsdReal<T>::rescale) eigvecs_dd(n, idx, cnt, Q, rc, rs, rk, nrot, A, htau, Y, wm);
    else eigvecs_impl<T>(n, idx, cnt, Q, rc, rs, rk, nrot, A, htau, Y, wm);
}

// Orthonormal contrasts (rows orthogonal to (1,..,1)) for NS = 2, 3, 4
// stencil vertices: C[k][a], k < NS - 1 (compile-time constants).
template <int NS> __device__ __forceinline__ constexpr double contrast(int k, int a)
{
    return NS == 4 ? 0.5 * ((k == 0 ? (a & 1) : k == 1 ? (a >> 1) : ((a ^ (a >> 1)) & 1)) ? -1.0 : 1.0)
        : NS == 3 ? (k == 0 ? (a == 0 ? 0.70710678118654752440 : a == 1 ? -0.70710678118654752440 : 0.0)
                            : (a == 2 ? -0.81649658092772603273 : 0.40824829046386301637))
                  : (a == 0 ? 0.70710678118654752440 : -0.70710678118654752440);
}

// w = C^T q (length 3 NS) for a length-3(NS-1) vector q.
template <int NS, class T> __device__ __forceinline__ void from_contrasts(const T* q, T* w)
{
#pragma unroll
    for (int a = 0; a < NS; ++a)
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            T s = 0;
#pragma unroll
            for (int k = 0; k < NS - 1; ++k) s += contrast<NS>(k, a) * q[3 * k + c];
            w[3 * a + c] = s;
        }
}

__device__ __forceinline__ double fval(const Params& P, double d2)
{
    return P.kappa * (barrier_fn<0, double>(P.kind, d2 - P.dmin2, P.xhat) * P.scale);
}
__device__ __forceinline__ double fd1(const Params& P, double d2)
{
    return P.kappa * (barrier_fn<1, double>(P.kind, d2 - P.dmin2, P.xhat) * P.scale);
}
__device__ __forceinline__ double fd2(const Params& P, double d2)
{
    return P.kappa * (barrier_fn<2, double>(P.kind, d2 - P.dmin2, P.xhat) * P.scale);
}
// FP32 barrier derivatives of an FP64 squared distance: d2 - dmin^2 is
// formed in FP64 (it cancels when d approaches dmin), then rounded.
__device__ __forceinline__ float fvalf(const Params& P, double d2)
{
    return (float)P.kappa * (barrier_fn<0, float>(P.kind, (float)(d2 - P.dmin2), (float)P.xhat) * (float)P.scale);
}
__device__ __forceinline__ float fd1f(const Params& P, double d2)
{
    return (float)P.kappa * (barrier_fn<1, float>(P.kind, (float)(d2 - P.dmin2), (float)P.xhat) * (float)P.scale);
}
__device__ __forceinline__ float fd2f(const Params& P, double d2)
{
    return (float)P.kappa * (barrier_fn<2, float>(P.kind, (float)(d2 - P.dmin2), (float)P.xhat) * (float)P.scale);
}
// Whether contact c is evaluated in FP32 (mixed precision, FV, triangle not
// degenerate).
__device__ __forceinline__ bool fp32_contact(const Params& P, const Local& c, const V3* x)
{
    return P.mixed && c.type == CT_FV && fv_fp32_ok(x);
}

__device__ __forceinline__ void gather(const double* __restrict__ V, const Local& c, V3* x)
{
    for (int i = 0; i < c.n; ++i) x[i] = load_v3(V, c.vid[i]);
}


// Self-check of the Hessian path: an index outside its buffer is recorded
// (first one wins) and the access is skipped.
struct Guard {
    long long* rec; // [code, index, limit, contact]
};
__device__ __forceinline__ bool in_range(const Guard& gd, int code, long long idx, long long limit, long long who)
{
    if (idx >= 0 && idx < limit) return true;
    if (atomicCAS((unsigned long long*)gd.rec, 0ull, (unsigned long long)code) == 0ull) {
        gd.rec[1] = idx;
        gd.rec[2] = limit;
        gd.rec[3] = who;
    }
    return false;
}

__device__ __forceinline__ int lower_bound_u64(const unsigned long long* __restrict__ a, int lo, int hi,
    unsigned long long key)
{
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (a[mid] < key) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

// Local-Hessian scratch, element-major: element k (row-major within the
// 3n x 3n matrix) of contact i is at p[k * stride + i].  A warp's 32
// consecutive contacts then read and write 256 contiguous bytes per element
// instead of 32 addresses 1,152 bytes apart.
struct Slab {
    double* p;
    int64_t stride;
    __device__ __forceinline__ double& at(int64_t i, int k) const { return p[(int64_t)k * stride + i]; }
};

// Element accessors for the PSD projection: one contact's local Hessian in
// the element-major slab, or in a per-thread array (row-major, N = 3n).
struct SlabAcc {
    const Slab& s;
    int64_t i;
    __device__ __forceinline__ double& operator()(int k) const { return s.at(i, k); }
};
struct LocalAcc {
    double* p;
    __device__ __forceinline__ double& operator()(int k) const { return p[k]; }
};

// Launch width of the local Hessian and PSD kernels: one warp per block.
// Their per-contact work is long and even, and a type's contacts can be few
// (5,465 FV contacts fill only 43 blocks of 128 threads on 152 SMs), so small
// blocks spread them over all SMs without a ragged last wave.
constexpr int LH_BLOCK = 32;

__device__ __forceinline__ int stencil_size(const ContactsView& cv, int64_t i)
{
    return i < cv.nvv ? 2 : (i < cv.nvv + cv.nev ? 3 : 4);
}

// PSD projection (eigen_ext.tpp:64-108) of every local Hessian, in place.
constexpr int PSD_BLOCK = LH_BLOCK;

// The NS - 1 contrasts sum_a C[k][a] v[a] of one value per stencil vertex.
// NS = 4: C is the Hadamard matrix's rows without the all-ones one, times
// 1/2; the butterflies here leave out that 1/2 (applied once by the caller).
// NS = 3, 2: scaled in place.
template <int NS, class T> __device__ __forceinline__ void contrast_apply(const T* v, T* o)
{
    const T R2 = T(0.70710678118654752440), R6 = T(0.40824829046386301637);
    if (NS == 4) {
        const T s01 = v[0] + v[1], d01 = v[0] - v[1], s23 = v[2] + v[3], d23 = v[2] - v[3];
        o[0] = d01 + d23;
        o[1] = s01 - s23;
        o[2] = d01 - d23;
    } else if (NS == 3) {
        o[0] = (v[0] - v[1]) * R2;
        o[1] = fma(T(-2.0), v[2], v[0] + v[1]) * R6;
    } else {
        o[0] = (v[0] - v[1]) * R2;
    }
}

// M = C H C^T (rows of M with stride MAXR) straight from contact i's slab:
// for each coordinate c, T = C H restricted to the rows of coordinate c (each
// slab element loaded once, coalesced across the warp's contacts), then row
// 3k+c of M from T's row k.
template <int NS, class T, class Acc> __device__ void to_contrasts(const Acc& hs, T* M, int sc)
{
    // the butterflies run in FP64 whatever the solver's arithmetic; the
    // entries are stored as T (scaled by 2^-sc for df64)
    constexpr int N = 3 * NS, K = NS - 1;
    const double S = NS == 4 ? 0.25 : 1.0; // the two butterfly stages' missing (1/2)^2
#pragma unroll 1
    for (int c = 0; c < 3; ++c) {
        double Tm[K][N];
#pragma unroll
        for (int j = 0; j < N; ++j) {
            double v[NS], o[K];
#pragma unroll
            for (int a = 0; a < NS; ++a) v[a] = hs((3 * a + c) * N + j);
            contrast_apply<NS, double>(v, o);
#pragma unroll
            for (int k = 0; k < K; ++k) Tm[k][j] = o[k];
        }
#pragma unroll
        for (int k = 0; k < K; ++k)
#pragma unroll
            for (int e = 0; e < 3; ++e) {
                double v[NS], o[K];
#pragma unroll
                for (int b = 0; b < NS; ++b) v[b] = Tm[k][3 * b + e];
                contrast_apply<NS, double>(v, o);
#pragma unroll
                for (int l = 0; l < K; ++l)
                    M[(3 * k + c) * MAXR + 3 * l + e] = PsdReal<T>::in(NS == 4 ? S * o[l] : o[l], sc);
            }
    }
}

// The eigenpairs of one local Hessian that its PSD projection
// (eigen_ext.tpp:64-108) needs.  M = C H C^T from the accessor; H is
// translation invariant, so H = C^T M C and with w = C^T q for each unit
// eigenvector q of M, H = sum lam w w^T over all eigenpairs.  The eigenpairs
// are computed in arithmetic T (FP64, or df64 on the matrix scaled by a power
// of two) and the smaller of two sets is kept: the negative eigenvalues, with
//   H+ = H - sum f lam w w^T,
// or the non-negative ones, with
//   H+ = (1 - f) H + sum f lam w w^T
// (f = 1 clamps, 2 takes the absolute value).  Out, in FP64: np pairs, the
// stencil vectors w (rows of 12 in wv), sl and sigma, such that
//   H+ = sigma H - sum_t sl[t] w_t w_t^T.
// An already PSD matrix gives np = 0 and sigma = 1: H as it is.  Returns
// false (np = 0, sigma = 1) if the eigensolver did not converge.  wm: the
// lanes of this warp that call it together (each of them makes the same
// __syncwarp calls), or 0 for a lane on its own.
template <class T, class Acc>
__device__ bool psd_pairs(int n, const Acc& hs, int method, double* wv /*MAXPAIRS*12*/, double* sl, int& np,
    double& sigma, unsigned wm = 0)
{
    const int N = 3 * n, m = 3 * (n - 1);
    T M[MAXR * MAXR], Q[MAXR * MAXR], lam[MAXR];
    // df64: the matrix is read scaled by 2^-sc so that its entries are O(1)
    const int sc = PsdReal<T>::scale_of(hs, N);
    if (n == 4) to_contrasts<4, T>(hs, M, sc);
    else if (n == 3) to_contrasts<3, T>(hs, M, sc);
    else to_contrasts<2, T>(hs, M, sc);
    for (int r = 0; r < m; ++r)
        for (int s = r + 1; s < m; ++s) {
            const T avg = T(0.5) * (M[r * MAXR + s] + M[s * MAXR + r]);
            M[r * MAXR + s] = M[s * MAXR + r] = avg;
        }
    T rc[MAXROT], rs[MAXROT], htau[MAXR];
    int8_t rk[MAXROT];
    int nrot;
    const bool ok = sym_eig(m, M, lam, Q, rc, rs, rk, nrot, htau, wm);
    if (wm) __syncwarp(wm);
    const double f = (method == IPCG_PSD_CLAMP) ? 1.0 : 2.0;
    int nneg = 0;
    if (ok)
        for (int k = 0; k < m; ++k) nneg += lam[k] < T(0) ? 1 : 0;
    const bool flip = 2 * nneg > m;
    int idx[MAXR];
    np = 0;
    if (ok && nneg > 0)
        for (int k = 0; k < m; ++k)
            if ((lam[k] < T(0)) != flip) idx[np++] = k;
    sigma = flip ? 1.0 - f : 1.0;
    const double fs = flip ? -f : f;
    // The eigenvectors (rows of 9) and then the w = C^T q (rows of 12) share
    // wv: row t of w is written after rows t.. of q are read (t descending),
    // and rows below t lie below 12 t.
    if constexpr (PsdReal<T>::rescale) {
        T Y[MAXPAIRS * MAXR];
        eigvecs(m, idx, np, Q, rc, rs, rk, nrot, M, htau, Y, wm);
        for (int i = 0; i < np * MAXR; ++i) wv[i] = dd_to_double(Y[i]);
    } else {
        eigvecs(m, idx, np, Q, rc, rs, rk, nrot, M, htau, wv, wm);
    }
    if (wm) __syncwarp(wm);
    for (int t = np - 1; t >= 0; --t) {
        double q[MAXR];
        for (int j = 0; j < m; ++j) q[j] = wv[t * MAXR + j];
        double* w = wv + 12 * t;
        if (n == 4) from_contrasts<4, double>(q, w);
        else if (n == 3) from_contrasts<3, double>(q, w);
        else from_contrasts<2, double>(q, w);
        sl[t] = fs * PsdReal<T>::out(lam[idx[t]], sc);
    }
    return ok;
}

// H+ entry by entry from psd_pairs' output: out(r, c, v) for every r <= c
// (H+ is symmetric; the caller mirrors).  With np = 0 and sigma = 1 the
// entries are H's own bits.  wm: the lanes of this warp that call it together
// with the same n (they meet after every row), or 0.
template <class Acc, class Out>
__device__ __forceinline__ void psd_apply(int n, const Acc& hs, const double* wv, const double* sl, int np,
    double sigma, const Out& out, unsigned wm = 0)
{
    const int N = 3 * n;
#pragma unroll 1
    for (int r = 0; r < N; ++r) {
        double swr[MAXPAIRS];
#pragma unroll
        for (int t = 0; t < MAXPAIRS; ++t) swr[t] = t < np ? sl[t] * wv[12 * t + r] : 0.0;
        for (int c = r; c < N; ++c) {
            double v = sigma * hs(r * N + c);
#pragma unroll
            for (int t = 0; t < MAXPAIRS; ++t)
                if (t < np) v = fma(-swr[t], wv[12 * t + c], v);
            out(r, c, v);
        }
        if (wm) __syncwarp(wm);
    }
}

// PSD projection of one local Hessian in place.  Returns false if the
// eigensolver did not converge.
template <class T, class Acc> __device__ bool project_psd(int n, const Acc& hs, int method)
{
    double wv[MAXPAIRS * 12], sl[MAXPAIRS], sigma;
    int np;
    if (!psd_pairs<T>(n, hs, method, wv, sl, np, sigma)) return false;
    if (np == 0 && sigma == 1.0) return true;
    const int N = 3 * n;
    psd_apply(n, hs, wv, sl, np, sigma, [&](int r, int c, double v) {
        hs(r * N + c) = v;
        if (c != r) hs(c * N + r) = v;
    });
    return true;
}

// ---- fused energy, gradient and local Hessian of one contact ----
// (normal_potential.cpp:127-232 in one pass; the PSD projection follows.)

// FP32 stencil expansions of reduced derivatives (reduced vector k is
// x[pos[k]] - x[neg[k]]).
template <int M> __device__ __forceinline__ void expand_g_f(int N, const int* pos, const int* neg, const float* gr,
    float* g)
{
    for (int i = 0; i < N; ++i) g[i] = 0;
    for (int k = 0; k < M; ++k)
        for (int c = 0; c < 3; ++c) {
            g[3 * pos[k] + c] += gr[3 * k + c];
            g[3 * neg[k] + c] -= gr[3 * k + c];
        }
}
template <int M> __device__ __forceinline__ void expand_h_f(int N, const int* pos, const int* neg, const float* Hr,
    float* H)
{
    for (int i = 0; i < N * N; ++i) H[i] = 0;
    for (int k = 0; k < M; ++k)
        for (int l = 0; l < M; ++l)
            for (int c = 0; c < 3; ++c)
                for (int e = 0; e < 3; ++e) {
                    const float h = Hr[(3 * k + c) * (3 * M) + 3 * l + e];
                    H[(3 * pos[k] + c) * N + 3 * pos[l] + e] += h;
                    H[(3 * pos[k] + c) * N + 3 * neg[l] + e] -= h;
                    H[(3 * neg[k] + c) * N + 3 * pos[l] + e] -= h;
                    H[(3 * neg[k] + c) * N + 3 * neg[l] + e] += h;
                }
}

// FP32 point-line form d = |c|^2 / L in r = (a, b) (a = e0 - p, b = e1 - p),
// with c = a x b and L = |b - a|^2 from FP64 (c is the small, cancellation-
// prone quantity: |c| = d |b - a|).
__device__ void point_line_f(F3 a, F3 b, F3 c, float P, float L, float* g /*6*/, float* H /*36*/)
{
    const F3 e { b.x - a.x, b.y - a.y, b.z - a.z };
    const float iL = 1.0f / L, iL2 = iL * iL;
    const F3 gPa = f3_cross(b, c), gPb = f3_cross(c, a);
    float gP[6], gL[6];
    for (int i = 0; i < 3; ++i) {
        gP[i] = 2.0f * f3c(gPa, i);
        gP[3 + i] = 2.0f * f3c(gPb, i);
        gL[i] = -2.0f * f3c(e, i);
        gL[3 + i] = 2.0f * f3c(e, i);
    }
    for (int i = 0; i < 6; ++i) g[i] = gP[i] * iL - P * gL[i] * iL2;
    float Sa[3][3], Sb[3][3], Sc[3][3];
    f3_skew(a, Sa);
    f3_skew(b, Sb);
    f3_skew(c, Sc);
    float HP[36];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            float aa = 0, bb = 0, ab = 0;
            for (int k = 0; k < 3; ++k) {
                aa += Sb[k][i] * Sb[k][j];
                bb += Sa[k][i] * Sa[k][j];
                ab -= Sb[k][i] * Sa[k][j];
            }
            HP[i * 6 + j] = 2 * aa;
            HP[(3 + i) * 6 + 3 + j] = 2 * bb;
            HP[i * 6 + 3 + j] = HP[(3 + j) * 6 + i] = 2 * (ab - Sc[i][j]);
        }
    const float k5 = 2 * P * iL2 * iL;
    for (int r = 0; r < 6; ++r)
        for (int q = 0; q < 6; ++q) {
            const float hl = (r % 3 == q % 3) ? ((r < 3) == (q < 3) ? 2.0f : -2.0f) : 0.0f;
            H[r * 6 + q] = HP[r * 6 + q] * iL - (gP[r] * gL[q] + gL[r] * gP[q]) * iL2 - P * hl * iL2
                + k5 * gL[r] * gL[q];
        }
}

// FP32 stencil gradient and Hessian of the squared distance of each form;
// each returns the squared distance itself in FP64 (the barrier's argument).
__device__ double pp_f(const V3* x, int N, int i, int j, float* g, float* K)
{
    const F3 r = to_f3(x[i] - x[j]);
    const float gr[3] = { 2 * r.x, 2 * r.y, 2 * r.z };
    const int pos[1] = { i }, neg[1] = { j };
    expand_g_f<1>(N, pos, neg, gr, g);
    const float Hr[9] = { 2, 0, 0, 0, 2, 0, 0, 0, 2 };
    expand_h_f<1>(N, pos, neg, Hr, K);
    return point_point_distance(x[i], x[j]);
}
__device__ double pl_f(const V3* x, int N, int p, int e0, int e1, float* g, float* K)
{
    const V3 a = x[e0] - x[p], b = x[e1] - x[p];
    const V3 c = cross(a, b);
    float gr[6], Hr[36];
    point_line_f(to_f3(a), to_f3(b), to_f3(c), (float)sqnorm(c), (float)sqnorm(b - a), gr, Hr);
    const int pos[2] = { e0, e1 }, neg[2] = { p, p };
    expand_g_f<2>(N, pos, neg, gr, g);
    expand_h_f<2>(N, pos, neg, Hr, K);
    return point_line_distance(x[p], x[e0], x[e1]);
}
// d = N^2 / D in r = (a, u, v) with a = x[pos[0]] - x[neg[0]], u = x[pos[1]] -
// x[neg[1]], v = x[pos[2]] - x[neg[2]]: point-plane (p, t0, t1, t2) and
// line-line forms.
__device__ void triple_f(const V3* x, const int* pos, const int* neg, float* g, float* K)
{
    const V3 a = x[pos[0]] - x[neg[0]], u = x[pos[1]] - x[neg[1]], v = x[pos[2]] - x[neg[2]];
    const V3 w = cross(u, v);
    float gr[9], Hr[81];
    triple_quot_f(to_f3(a), to_f3(u), to_f3(v), to_f3(w), (float)dot(a, w), (float)sqnorm(w), gr, Hr);
    expand_g_f<3>(12, pos, neg, gr, g);
    expand_h_f<3>(12, pos, neg, Hr, K);
}
__device__ double ee_f(const V3* x, int dtype, float* g, float* K)
{
    switch (dtype) {
    case EA0_EB0: return pp_f(x, 12, 0, 2, g, K);
    case EA0_EB1: return pp_f(x, 12, 0, 3, g, K);
    case EA1_EB0: return pp_f(x, 12, 1, 2, g, K);
    case EA1_EB1: return pp_f(x, 12, 1, 3, g, K);
    case EA_EB0: return pl_f(x, 12, 2, 0, 1, g, K);
    case EA_EB1: return pl_f(x, 12, 3, 0, 1, g, K);
    case EA0_EB: return pl_f(x, 12, 0, 2, 3, g, K);
    case EA1_EB: return pl_f(x, 12, 1, 2, 3, g, K);
    default: {
        const int pos[3] = { 2, 1, 3 }, neg[3] = { 0, 0, 2 };
        triple_f(x, pos, neg, g, K);
        return line_line_distance(x[0], x[1], x[2], x[3]);
    }
    }
}
__device__ double contact_distance_f(const Local& c, const V3* x, float* g, float* K)
{
    switch (c.type) {
    case CT_VV: return pp_f(x, 6, 0, 1, g, K);
    case CT_EV: return pl_f(x, 9, 0, 1, 2, g, K);
    case CT_EE: return ee_f(x, c.dtype, g, K);
    default: {
        const int pos[3] = { 0, 2, 3 }, neg[3] = { 1, 1, 1 };
        triple_f(x, pos, neg, g, K);
        return point_plane_distance(x[0], x[1], x[2], x[3]);
    }
    }
}

// EE mollifier in reduced form: m, the stencil gradient gs of s = |ea x eb|^2
// (gm = m1 gs), the reduced Hessian Hr (6 x 6, in (ea, eb)) of s, m1 and m2,
// so that the mollifier Hessian's stencil entry (3a+c, 3b+e) is
// m1 sg(a) sg(b) Hr[3 k(a) + c][3 k(b) + e] + m2 gs_r gs_q with k(a) = a / 2
// and sg(a) = +1 for a = 1, 3, -1 for a = 0, 2 (the values of mollifier()'s
// expanded matrix: each stencil entry is one reduced entry).
struct MollifierR {
    bool active;
    double m, m1, m2;
    double gs[12], Hr[36];
};
__device__ void mollifier_reduced(const Local& c, const V3* x, bool want_h, MollifierR& o)
{
    o.active = false;
    o.m = 1.0;
    if (c.type != CT_EE) return;
    const double s = ee_cross_sqnorm(x[0], x[1], x[2], x[3]);
    if (!(s < c.eps)) return;
    o.active = true;
    const double xe = s / c.eps;
    o.m = (-xe + 2) * xe;
    const double inv = 1 / c.eps;
    o.m1 = 2 * inv * fma(-inv, s, 1.0);
    o.m2 = -2 / (c.eps * c.eps);
    double gr[6];
    cross_sq(x[1] - x[0], x[3] - x[2], gr, want_h ? o.Hr : nullptr);
    const int pos[2] = { 1, 3 }, neg[2] = { 0, 2 };
    expand_g<2>(12, pos, neg, gr, o.gs);
}
__device__ __forceinline__ double mollifier_h(const MollifierR& o, int r, int q)
{
    const int a = r / 3, cc = r % 3, b = q / 3, e = q % 3;
    const double sg = ((a & 1) ? 1.0 : -1.0) * ((b & 1) ? 1.0 : -1.0);
    return o.m1 * (sg * o.Hr[(3 * (a >> 1) + cc) * 6 + 3 * (b >> 1) + e]) + o.m2 * o.gs[r] * o.gs[q];
}

// Whether contact c is evaluated in FP32: with IPCG_BARRIER_FP32_LOCAL every
// contact but near-parallel (mollified) edge-edge ones and face-vertex ones
// on degenerate triangles; with IPCG_BARRIER_FP32_PT only face-vertex ones on
// non-degenerate triangles.
__device__ __forceinline__ bool fp32_local_contact(const Params& P, const Local& c, const V3* x)
{
    if (c.type == CT_FV) return (P.mixed || P.fp32_local) && fv_fp32_ok(x);
    if (!P.fp32_local) return false;
    if (c.type == CT_EE) return !(ee_cross_sqnorm(x[0], x[1], x[2], x[3]) < c.eps);
    return true;
}

// Energy e, stencil gradient g (3n) and local Hessian H (3n x 3n row-major,
// both triangles written) of one contact.  Returns whether H is to be
// projected: the mollified edge-edge case with m <= 0 is returned as is, as
// the reference does (normal_potential.cpp:185-189).
// The FP32 path (fp32_local_contact true).
__device__ __forceinline__ bool contact_egh_f32(const Local& c, const V3* x, const Params& P, double& e, double* g,
    double* H)
{
    const int N = 3 * c.n;
    float gf[12], Kf[144];
    const double d = contact_distance_f(c, x, gf, Kf);
    e = c.w * (double)fvalf(P, d);
    const float wf = (float)c.w, a = wf * fd2f(P, d), b = wf * fd1f(P, d);
    for (int k = 0; k < N; ++k) g[k] = (double)(b * gf[k]);
    for (int r = 0; r < N; ++r)
        for (int q = r; q < N; ++q) {
            const double v = (double)(a * gf[r] * gf[q] + b * Kf[r * N + q]);
            H[r * N + q] = v;
            H[q * N + r] = v;
        }
    return true;
}

// The FP64 path.
__device__ __forceinline__ bool contact_egh_f64(const Local& c, const V3* x, const Params& P, double& e, double* g,
    double* H)
{
    const int N = 3 * c.n;
    double gd[12];
    const double d = contact_distance(c, x, gd, H); // H: the distance Hessian, overwritten below
    const double fv = fval(P, d), fd = fd1(P, d), fdd = fd2(P, d);
    if (c.type != CT_EE) {
        e = c.w * 1.0 * fv;
        for (int k = 0; k < N; ++k) g[k] = (c.w * fd) * gd[k];
        for (int r = 0; r < N; ++r)
            for (int q = r; q < N; ++q) {
                const double v = (c.w * fdd) * gd[r] * gd[q] + (c.w * fd) * H[r * N + q];
                H[r * N + q] = v;
                H[q * N + r] = v;
            }
        return true;
    }
    MollifierR mo;
    mollifier_reduced(c, x, true, mo);
    const double m = mo.m;
    e = c.w * m * fv;
    if (m <= 0) {
        for (int k = 0; k < 12; ++k) g[k] = 0;
    } else {
        for (int k = 0; k < 12; ++k)
            g[k] = (c.w * fv) * (mo.active ? mo.m1 * mo.gs[k] : 0.0) + (c.w * m * fd) * gd[k];
    }
    if (mo.active && m <= 0) {
        for (int r = 0; r < 12; ++r)
            for (int q = r; q < 12; ++q) {
                const double v = (c.w * fv) * mollifier_h(mo, r, q);
                H[r * 12 + q] = v;
                H[q * 12 + r] = v;
            }
        return false;
    }
    const double wm = c.w * m;
    for (int r = 0; r < 12; ++r)
        for (int q = r; q < 12; ++q) {
            double v = (wm * fdd) * gd[r] * gd[q] + (wm * fd) * H[r * 12 + q];
            if (mo.active) {
                const double gfm_rq = (c.w * fd) * gd[r] * (mo.m1 * mo.gs[q]);
                const double gfm_qr = (c.w * fd) * gd[q] * (mo.m1 * mo.gs[r]);
                v = v + ((c.w * fv) * mollifier_h(mo, r, q) + gfm_rq + gfm_qr);
            }
            H[r * 12 + q] = v;
            H[q * 12 + r] = v;
        }
    return true;
}

} // namespace

} // namespace ipcg
