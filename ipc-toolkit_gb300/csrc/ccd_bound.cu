// ccd_bound.cu -- per step-size query, a lower bound on the time of impact
// the inclusion search can return and an estimate of it (for ordering).
// This file is compiled with fused multiply-adds: its results only need to
// be conservative (they carry margins far above the rounding differences),
// not bit-identical to the search's own arithmetic.
#include "ccd_query.cuh"
#include "profile.cuh"

namespace ipcg {

namespace {

// A lower bound on the time of impact stencil_ccd can return for a query
// (+inf when it can only miss).  For one coordinate c, the co-planarity
// function F_c(t, u, v) is linear in t at each corner (u, v) of [0, 1]^2, so
// g(t) = min and h(t) = max of F_c(t, ., .) over [0, 1]^2 are the min and max
// of four lines.  A box [t0, t1] x U x V that the inclusion test keeps has,
// in every coordinate, a corner box meeting [-r, r] (r = err + ms), hence a
// time t in [t0, t1] with g(t) <= r and h(t) >= -r (g and h bound F_c over
// any (u, v), and are continuous).  So every kept box ends at or after
// T = max_c T_c, T_c the first such time, and an accepted box starts at or
// after T minus its own width in t -- which is below the time tolerance
// unless the box was accepted for its narrow codomain (then every coordinate
// lies within r + delta over the whole box, so T computed with r + delta is
// at most its start) or for lying inside (then T is at most its start).  T is
// computed with r + delta + 2 err (the corner values' rounding); the search
// for the first time runs in FP32 on the FP64 corner lines, with slacks that
// cover its rounding, and the result is lowered by 2^-20, the time tolerance
// and a relative 1e-6.  Only used to skip queries that cannot lower the
// earliest time found so far (and only when it is at least 1e-6, above which
// the strategy's small-ToI rerun cannot apply).
// First time in [0, 1] at which min_k (A_k + B_k t) <= R and max_k (...)
// >= -R (+inf if none): 0 or a time where a line enters one of the two sets.
__device__ __forceinline__ float first_time(const float A[4], const float B[4], float R, float slack)
{
    float Tc = __int_as_float(0x7f800000);
    for (int j = 0; j < 9; ++j) {
        float tj;
        if (j == 0) tj = 0.f;
        else {
            const int k = (j - 1) >> 1;
            if (j & 1) {
                if (!(B[k] < 0.f)) continue;
                tj = (R - A[k]) / B[k];
            } else {
                if (!(B[k] > 0.f)) continue;
                tj = (-R - A[k]) / B[k];
            }
            if (!(tj >= 0.f && tj <= 1.f) || !(tj < Tc)) continue;
        }
        float g = A[0] + B[0] * tj, h = g;
        for (int k = 1; k < 4; ++k) {
            const float f = A[k] + B[k] * tj;
            g = fminf(g, f);
            h = fmaxf(h, f);
        }
        if (g <= R + slack && h >= -R - slack) Tc = fminf(Tc, tj);
    }
    return Tc;
}

// min over t in [0, 1] of |a + t b| (3-vectors)
__device__ __forceinline__ double min_norm_on_segment(const double a[3], const double b[3])
{
    const double bb = b[0] * b[0] + b[1] * b[1] + b[2] * b[2];
    const double ab = a[0] * b[0] + a[1] * b[1] + a[2] * b[2];
    const double t = bb > 0 ? fmin(1.0, fmax(0.0, -ab / bb)) : 0.0;
    double n = 0;
    for (int c = 0; c < 3; ++c) {
        const double x = a[c] + t * b[c];
        n += x * x;
    }
    return sqrt(n);
}

struct F3b {
    float x, y, z;
};
__device__ __forceinline__ F3b f3(V3 a) { return F3b { (float)a.x, (float)a.y, (float)a.z }; }
__device__ __forceinline__ F3b operator-(F3b a, F3b b) { return F3b { a.x - b.x, a.y - b.y, a.z - b.z }; }
__device__ __forceinline__ float fdot(F3b a, F3b b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ float clamp01(float x) { return fminf(1.f, fmaxf(0.f, x)); }

// An upper bound on the distance between the primitives at t = 0: the FP64
// distance between two points on them, at closest-point parameters found in
// FP32 (the region tests of the standard point-triangle and segment-segment
// closest-point algorithms; the parameters are clamped onto the primitives,
// so the points lie on them whatever the FP32 rounding).  Only used to size
// the separation of the bound, where a larger distance is the conservative
// side.
__device__ double distance_upper_bound(const Query& q)
{
    double s, t;
    if (q.vf) {
        // point s0, triangle (s1, s2, s3): parameters along s2 - s1 and s3 - s1
        const F3b p = f3(q.s[0]), a = f3(q.s[1]), b = f3(q.s[2]), c = f3(q.s[3]);
        const F3b ab = b - a, ac = c - a, ap = p - a, bp = p - b, cp = p - c;
        const float d1 = fdot(ab, ap), d2 = fdot(ac, ap), d3 = fdot(ab, bp), d4 = fdot(ac, bp);
        const float d5 = fdot(ab, cp), d6 = fdot(ac, cp);
        const float vc = d1 * d4 - d3 * d2, vb = d5 * d2 - d1 * d6, va = d3 * d6 - d5 * d4;
        if (d1 <= 0.f && d2 <= 0.f) s = t = 0;
        else if (d3 >= 0.f && d4 <= d3) s = 1, t = 0;
        else if (d6 >= 0.f && d5 <= d6) s = 0, t = 1;
        else if (vc <= 0.f && d1 >= 0.f && d3 <= 0.f) s = clamp01(d1 / (d1 - d3)), t = 0;
        else if (vb <= 0.f && d2 >= 0.f && d6 <= 0.f) s = 0, t = clamp01(d2 / (d2 - d6));
        else if (va <= 0.f && d4 - d3 >= 0.f && d5 - d6 >= 0.f) {
            const float w = clamp01((d4 - d3) / ((d4 - d3) + (d5 - d6)));
            s = 1.f - w, t = w;
        } else {
            const float den = va + vb + vc;
            const float v = den != 0.f ? clamp01(vb / den) : 0.f, w = den != 0.f ? clamp01(vc / den) : 0.f;
            s = v, t = fminf(w, 1.f - v);
        }
        const V3 x = q.s[1] + (q.s[2] - q.s[1]) * s + (q.s[3] - q.s[1]) * t;
        return sqrt(sqnorm(q.s[0] - x));
    }
    // segments (s0, s1) and (s2, s3)
    const F3b p1 = f3(q.s[0]), p2 = f3(q.s[2]);
    const F3b d1 = f3(q.s[1]) - p1, d2 = f3(q.s[3]) - p2, r = p1 - p2;
    const float a = fdot(d1, d1), e = fdot(d2, d2), f = fdot(d2, r);
    float sf = 0.f, tf = 0.f;
    if (a > 0.f || e > 0.f) {
        if (!(a > 0.f)) tf = clamp01(f / e);
        else {
            const float c = fdot(d1, r);
            if (!(e > 0.f)) sf = clamp01(-c / a);
            else {
                const float b = fdot(d1, d2), den = a * e - b * b;
                sf = den > 0.f ? clamp01((b * f - c * e) / den) : 0.f;
                tf = (b * sf + f) / e;
                if (tf < 0.f) tf = 0.f, sf = clamp01(-c / a);
                else if (tf > 1.f) tf = 1.f, sf = clamp01((b - c) / a);
            }
        }
    }
    s = sf, t = clamp01(tf);
    const V3 x = q.s[0] + (q.s[1] - q.s[0]) * s, y = q.s[2] + (q.s[3] - q.s[2]) * t;
    return sqrt(sqnorm(x - y));
}

__device__ double toi_lower_bound(const Query& q, double min_distance, const CCDParams& P)
{
    const double INF = __longlong_as_double(0x7ff0000000000000LL);
    const float FINF = __int_as_float(0x7f800000);
    // an upper bound of the distance at t = 0 gives a larger separation, the
    // conservative side (0 if it is within the minimum distance)
    const double d0 = distance_upper_bound(q);
    if (d0 <= min_distance) return 0.0;
    if (v3eq(q.s[0], q.e[0]) && v3eq(q.s[1], q.e[1]) && v3eq(q.s[2], q.e[2]) && v3eq(q.s[3], q.e[3])) {
        // a query that does not move is a miss unless its exact distance is
        // within the minimum distance; the upper bound exceeds the exact
        // distance by at most the FP32 parameters' error along the edges
        const double ext = sqrt(sqnorm(q.s[1] - q.s[0])) + sqrt(sqnorm(q.s[2] - q.s[0])) + sqrt(sqnorm(q.s[3] - q.s[0]));
        return d0 > min_distance + 1e-5 * ext ? INF : 0.0;
    }
    const double ms = fmin((1.0 - P.rescale) * (d0 - min_distance), 1e-4) + min_distance;
    const double delta = fmin(0.5 * d0, P.tolerance);
    double err[3];
    numerical_error(q, ms > 0, err);
    // per coordinate, F = A00 + u Au + v Av + t (B00 + u Bu + v Bv) (FP64)
    double a00[3], au[3], av[3], b00[3], bu[3], bv[3];
    for (int c = 0; c < 3; ++c) {
        const double s0 = comp(q.s[0], c), s1 = comp(q.s[1], c), s2 = comp(q.s[2], c), s3 = comp(q.s[3], c);
        const double e0 = comp(q.d[0], c), e1 = comp(q.d[1], c), e2 = comp(q.d[2], c), e3 = comp(q.d[3], c);
        if (q.vf) {
            a00[c] = s0 - s1;
            au[c] = -(s2 - s1);
            av[c] = -(s3 - s1);
            b00[c] = e0 - e1;
            bu[c] = -(e2 - e1);
            bv[c] = -(e3 - e1);
        } else {
            a00[c] = s0 - s2;
            au[c] = s1 - s0;
            av[c] = -(s3 - s2);
            b00[c] = e0 - e2;
            bu[c] = e1 - e0;
            bv[c] = -(e3 - e2);
        }
    }
    double T = 0.0, bmax = 0.0, rmax = 0.0;
    float R[3], scale[3];
    for (int c = 0; c < 3; ++c) {
        // corner lines at (u, v) in {0, 1}^2, the search in FP32 with a
        // slack that covers its rounding (2^-20 of the lines' size) and a
        // final 2^-20 margin on the time
        float A[4], B[4];
        for (int k = 0; k < 4; ++k) {
            const double u = (k & 1) ? 1.0 : 0.0, v = (k & 2) ? 1.0 : 0.0;
            const double a = a00[c] + u * au[c] + v * av[c], b = b00[c] + u * bu[c] + v * bv[c];
            bmax = fmax(bmax, fabs(b));
            A[k] = (float)a;
            B[k] = (float)b;
        }
        R[c] = (float)(3.0 * err[c] + ms + delta);
        rmax = fmax(rmax, 3.0 * err[c] + ms + delta);
        scale[c] = (float)(fabs(a00[c]) + fabs(au[c]) + fabs(av[c]) + fabs(b00[c]) + fabs(bu[c]) + fabs(bv[c]));
        const float Tc = first_time(A, B, R[c], (scale[c] + R[c]) * 0x1p-20f);
        if (!(Tc <= 1.f)) return INF;
        T = fmax(T, (double)Tc);
    }
    // Cells of the (u, v) square (4 x 4): when both primitives' edges along u
    // and v stay longer than 2 sqrt(3) (2 r + delta) over the step, no box
    // wider than 1/4 in u or v can be accepted (one coordinate of F would
    // change by more than 2 r + delta across it, while acceptance needs every
    // coordinate inside the separation box or narrower than delta, and the
    // domain tolerance would be below 1/4), so the accepted box lies in one
    // cell and the bound is the least of the cells' bounds.
    constexpr int NCELL = 4;
    const double lu = min_norm_on_segment(au, bu), lv = min_norm_on_segment(av, bv);
    const double need = 1.7320508075688772 * (2.0 * rmax + delta) * (0.5 * NCELL) * (1.0 + 1e-6);
    if (lu > need && lv > need) {
        const float w = 1.f / NCELL;
        float Tq_min = FINF;
        for (int cell = 0; cell < NCELL * NCELL; ++cell) {
            const float uq = w * (float)(cell % NCELL), vq = w * (float)(cell / NCELL);
            float Tq = 0.f;
            for (int c = 0; c < 3 && Tq <= 1.f && Tq < Tq_min; ++c) {
                float A[4], B[4];
                for (int k = 0; k < 4; ++k) {
                    const float u = uq + ((k & 1) ? w : 0.f), v = vq + ((k & 2) ? w : 0.f);
                    A[k] = (float)a00[c] + u * (float)au[c] + v * (float)av[c];
                    B[k] = (float)b00[c] + u * (float)bu[c] + v * (float)bv[c];
                }
                const float Tc = first_time(A, B, R[c], (scale[c] + R[c]) * 0x1p-20f);
                Tq = fmaxf(Tq, Tc);
            }
            Tq_min = fminf(Tq_min, Tq);
        }
        if (!(Tq_min <= 1.f)) return INF;
        T = fmax(T, (double)Tq_min);
    }
    // the time tolerance of the inclusion search: delta / (3 max |F(1) - F(0)|)
    // over the corners, F(1) - F(0) being the corner lines' slopes
    const double tol0 = bmax == 0.0 ? delta : delta / (3.0 * bmax);
    return fmax(0.0, (T - 0x1p-20 - tol0 * (1.0 + 1e-6) - 0x1p-60) * (1.0 - 1e-6));
}

// An estimate of a query's time of impact, for ordering only: the time at
// which the signed volume of its four points (linear between its values at
// t = 0 and t = 1) changes sign, if the two primitives' closest points lie
// on them (with a 10 % margin) at that time; otherwise 1 + its lower bound
// (after every likely hit).
__device__ double toi_estimate(const Query& q, double lower)
{
    auto at = [&](int k, double t) { return q.s[k] + q.d[k] * t; };
    auto vol = [&](double t) {
        const V3 a = at(0, t), b = at(1, t), c = at(2, t), d = at(3, t);
        return q.vf ? dot(cross(c - b, d - b), a - b) : dot(cross(b - a, d - c), c - a);
    };
    const double v0 = vol(0.0), v1 = vol(1.0);
    if (!(lower < 1.0) || !((v0 > 0) != (v1 > 0) || v1 == 0)) return 1.0 + lower;
    const double t = fmax(lower, fmin(1.0, v0 / (v0 - v1)));
    const V3 a = at(0, t), b = at(1, t), c = at(2, t), d = at(3, t);
    double x, y, z = 0;
    if (q.vf) {
        // barycentric coordinates of a's projection onto triangle (b, c, d)
        const V3 e0 = c - b, e1 = d - b, w = a - b;
        const double d00 = dot(e0, e0), d01 = dot(e0, e1), d11 = dot(e1, e1), d20 = dot(w, e0), d21 = dot(w, e1);
        const double den = d00 * d11 - d01 * d01;
        if (!(den > 0)) return 1.0 + lower;
        x = (d11 * d20 - d01 * d21) / den;
        y = (d00 * d21 - d01 * d20) / den;
        z = 1.0 - x - y;
    } else {
        // closest-point parameters of the lines (a, b) and (c, d)
        const V3 u = b - a, v = d - c, w = a - c;
        const double aa = dot(u, u), bb = dot(u, v), cc = dot(v, v), dd = dot(u, w), ee = dot(v, w);
        const double den = aa * cc - bb * bb;
        if (!(den > 0)) return 1.0 + lower;
        x = (bb * ee - cc * dd) / den;
        y = (aa * ee - bb * dd) / den;
    }
    const bool on = x >= -0.1 && x <= 1.1 && y >= -0.1 && y <= 1.1 && z >= -0.1 && z <= 1.1;
    return on ? t : 1.0 + lower;
}

// keys: scene in the top 20 bits, then the leading 44 bits of the query's
// time-of-impact estimate (its sign is clear), so that a scene's likely
// earliest impacts sort first.
__global__ void k_ccd_bound(const int2* __restrict__ cand_ee, int n_ee, const int2* __restrict__ cand_fv, int n_fv,
    const double* __restrict__ V0, const double* __restrict__ V1, const int* __restrict__ E, const int* __restrict__ F,
    const double* __restrict__ min_distance, SceneView sv, CCDParams P, double* __restrict__ lb,
    unsigned long long* __restrict__ keys, int* __restrict__ ids)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_ee + n_fv) return;
    Query q;
    const int scene = sv.of(load_query(i, cand_ee, n_ee, cand_fv, V0, V1, E, F, q));
    const double b = toi_lower_bound(q, __ldg(min_distance + scene), P);
    lb[i] = b;
    const double est = toi_estimate(q, b);
    keys[i] = ((unsigned long long)scene << CCD_SCENE_SHIFT) | ((unsigned long long)__double_as_longlong(est) >> 20);
    ids[i] = i;
}

} // namespace

void ccd_bound_launch(cudaStream_t s, const int2* cee, int n_ee, const int2* cfv, int n_fv, const double* V0,
    const double* V1, const int* E, const int* F, const double* min_distance, SceneView sv, double tolerance,
    double rescale, double* lb, unsigned long long* keys, int* ids)
{
    const int nc = n_ee + n_fv;
    if (nc <= 0) return;
    const CCDParams P { tolerance, 0, rescale };
    IPCG_LAUNCH("k_ccd_bound", s, k_ccd_bound<<<grid_for(nc, 128), 128, 0, s>>>(cee, n_ee, cfv, n_fv, V0, V1, E, F,
        min_distance, sv, P, lb, keys, ids));
}

} // namespace ipcg
