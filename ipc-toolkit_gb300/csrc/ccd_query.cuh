// ccd_query.cuh -- a step-size query (one edge-edge or face-vertex candidate
// over the step) and what both step-size translation units share: its load,
// the numerical error filter of the inclusion search and the strategy's
// parameters (tight_inclusion_ccd.cpp:33-336).
#pragma once
#include "geom.cuh"
#include "internal.cuh"

namespace ipcg {
namespace {

struct Query {
    V3 s[4], e[4];
    V3 d[4]; // e - s: the same value the evaluation form (b - a) t + a computes per box
    bool vf;
    __device__ void set_deltas()
    {
        for (int k = 0; k < 4; ++k) d[k] = e[k] - s[k];
    }
};

struct CCDParams {
    double tolerance;
    long long max_iterations;
    double rescale;
};


__device__ __forceinline__ bool v3eq(V3 a, V3 b) { return a.x == b.x && a.y == b.y && a.z == b.z; }

__device__ void numerical_error(const Query& q, bool use_ms, double err[3])
{
    const double vf_f = use_ms ? 7.549516567451064e-15 : 6.661338147750939e-15;
    const double ee_f = use_ms ? 7.105427357601002e-15 : 6.217248937900877e-15;
    const double filt = q.vf ? vf_f : ee_f;
    for (int c = 0; c < 3; ++c) {
        double m = 0;
        for (int k = 0; k < 4; ++k) {
            m = fmax(m, fabs(comp(q.s[k], c)));
            m = fmax(m, fabs(comp(q.e[k], c)));
        }
        const double dl = fmin(m, 1.0);
        err[c] = filt * (dl * dl * dl);
    }
}


// Loads candidate i; returns its first vertex (which names its scene).
__device__ __forceinline__ int load_query(int i, const int2* __restrict__ cand_ee, int n_ee,
    const int2* __restrict__ cand_fv, const double* __restrict__ V0, const double* __restrict__ V1,
    const int* __restrict__ E, const int* __restrict__ F, Query& q)
{
    int ids[4];
    if (i < n_ee) {
        const int2 c = cand_ee[i];
        q.vf = false;
        ids[0] = E[2 * c.x];
        ids[1] = E[2 * c.x + 1];
        ids[2] = E[2 * c.y];
        ids[3] = E[2 * c.y + 1];
    } else {
        const int2 c = cand_fv[i - n_ee];
        q.vf = true;
        ids[0] = c.y;
        ids[1] = F[3 * c.x];
        ids[2] = F[3 * c.x + 1];
        ids[3] = F[3 * c.x + 2];
    }
    for (int k = 0; k < 4; ++k) {
        q.s[k] = load_v3(V0, ids[k]);
        q.e[k] = load_v3(V1, ids[k]);
    }
    q.set_deltas();
    return ids[0];
}


// sort keys of the step-size queries: scene in the top 20 bits, then the
// leading 44 bits of a non-negative double
constexpr int CCD_SCENE_SHIFT = 44;

} // namespace
} // namespace ipcg
