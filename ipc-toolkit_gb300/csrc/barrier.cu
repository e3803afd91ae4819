// barrier.cu — BarrierPotential energy, gradient and Hessian on the device.
//
// Restates src/ipc/potentials/potential.cpp:36-222 (sum over contacts,
// dense gradient, sparse Hessian), normal_potential.cpp:127-232 (per-contact
// w·m(x)·f(d(x)) with the mollifier product rule for edge-edge contacts),
// barrier_potential.cpp:62-99 and barrier.cpp:11-43 (clamped log barrier on
// d² - dmin² against (2 dmin + dhat) dhat), and eigen_ext.tpp:64-108 (PSD
// projection by clamping or flipping negative eigenvalues).
//
// Design: one thread per contact.  GB300 executes FP64 at a small fraction
// of its FP32 rate, so the per-contact 12×12 work is FP64-issue-bound and a
// full warp of independent contacts keeps that pipe busy without any
// intra-warp reductions.  Distance derivatives use closed forms in vertex-
// difference variables (d = N²/D for point-plane and line-line, |a×b|²/|b−a|²
// for point-line); the PSD projection works in the 3(n-1)-dimensional
// complement of rigid translations (the barrier is translation invariant),
// where a Householder tridiagonalisation plus implicit QR with Wilkinson
// shifts gives the eigenpairs, and only the negative ones are removed from
// the 3n×3n Hessian.  The Hessian is assembled into a CSR matrix whose
// pattern is the union of the contacts' 3×3 vertex blocks: the (block key,
// contribution) pairs are radix-sorted and run-length encoded, which gives
// the CSR pattern and, per block, its contributions in a fixed order;
// k_assemble then sums each stored value's contributions in that order and
// writes it once (no atomics, deterministic).  This file holds the per-type
// kernels used by friction and shape derivatives and the energy / gradient
// kernels; the barrier's own energy + gradient + Hessian pass with a cached
// pattern lives in egh.cu, and the per-contact math in contact.cuh.
#include <cub/block/block_reduce.cuh>

#include <cstdio>
#include <cstring>
#include <algorithm>
#include <atomic>
#include <mutex>
#include <vector>

#include "contact.cuh"
#include "profile.cuh"

namespace ipcg {

namespace {

// ---- kernels ----
__global__ void __launch_bounds__(BLOCK) k_energy(ContactsView cv, const int* __restrict__ E,
    const int* __restrict__ F, const double* __restrict__ V, Params P, double* __restrict__ partial)
{
    // one scene: deterministic per-block partial sums
    const int64_t n = cv.nvv + cv.nev + cv.nee + cv.nfv;
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    double e = 0;
    if (i < n) {
        Local c;
        load_contact(cv, E, F, i, c);
        V3 x[4];
        gather(V, c, x);
        if (fp32_contact(P, c, x)) {
            float gf[12];
            e = c.w * (double)fvalf(P, fv_local_f(x, gf, nullptr));
        } else {
            double g[12];
            const double d = contact_distance(c, x, g, nullptr);
            bool act;
            const double m = mollifier(c, x, nullptr, nullptr, act);
            e = c.w * m * fval(P, d);
        }
    }
    typedef cub::BlockReduce<double, BLOCK> BR;
    __shared__ typename BR::TempStorage tmp;
    const double s = BR(tmp).Sum(e);
    if (threadIdx.x == 0) partial[blockIdx.x] = s;
}

__global__ void k_sum_partials(const double* __restrict__ partial, int n, double* __restrict__ out)
{
    typedef cub::BlockReduce<double, 1024> BR;
    __shared__ typename BR::TempStorage tmp;
    double s = 0;
    // fixed per-thread strided order => deterministic
    for (int i = threadIdx.x; i < n; i += 1024) s += partial[i];
    const double t = BR(tmp).Sum(s);
    if (threadIdx.x == 0) *out = t;
}

// Batches: per-scene energies.  Contact lists are sorted by index key and
// the scenes occupy consecutive index ranges, so a block almost always holds
// one scene: it then adds one block sum, otherwise each contact adds its own.
__global__ void __launch_bounds__(BLOCK) k_energy_scenes(ContactsView cv, const int* __restrict__ E,
    const int* __restrict__ F, const double* __restrict__ V, const Params* __restrict__ sp, SceneView sv,
    double* __restrict__ energy)
{
    const int64_t n = cv.nvv + cv.nev + cv.nee + cv.nfv;
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    double e = 0;
    int scene = -1;
    if (i < n) {
        Local c;
        load_contact(cv, E, F, i, c);
        scene = sv.of(c.vid[0]);
        const Params P = sp[scene];
        V3 x[4];
        gather(V, c, x);
        if (fp32_contact(P, c, x)) {
            float gf[12];
            e = c.w * (double)fvalf(P, fv_local_f(x, gf, nullptr));
        } else {
            double g[12];
            const double d = contact_distance(c, x, g, nullptr);
            bool act;
            const double m = mollifier(c, x, nullptr, nullptr, act);
            e = c.w * m * fval(P, d);
        }
    }
    __shared__ int s_lo, s_hi;
    if (threadIdx.x == 0) {
        s_lo = 0x7fffffff;
        s_hi = -1;
    }
    __syncthreads();
    if (scene >= 0) {
        atomicMin(&s_lo, scene);
        atomicMax(&s_hi, scene);
    }
    __syncthreads();
    if (s_lo == s_hi) {
        typedef cub::BlockReduce<double, BLOCK> BR;
        __shared__ typename BR::TempStorage tmp;
        const double sum = BR(tmp).Sum(e);
        if (threadIdx.x == 0 && s_hi >= 0) atomicAdd(energy + s_hi, sum);
    } else if (scene >= 0 && e != 0) {
        atomicAdd(energy + scene, e);
    }
}

__global__ void __launch_bounds__(BLOCK) k_gradient(ContactsView cv, const int* __restrict__ E,
    const int* __restrict__ F, const double* __restrict__ V, const Params* __restrict__ sp, SceneView sv,
    double* __restrict__ grad)
{
    const int64_t n = cv.nvv + cv.nev + cv.nee + cv.nfv;
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    Local c;
    load_contact(cv, E, F, i, c);
    const Params P = sp[sv.of(c.vid[0])];
    V3 x[4];
    gather(V, c, x);
    if (fp32_contact(P, c, x)) {
        float gf[12];
        const float fd = fd1f(P, fv_local_f(x, gf, nullptr)) * (float)c.w;
        for (int a = 0; a < 4; ++a)
            for (int k = 0; k < 3; ++k) {
                const double v = (double)(fd * gf[3 * a + k]);
                if (v != 0) atomicAdd(grad + 3 * (int64_t)c.vid[a] + k, v);
            }
        return;
    }
    const int N = 3 * c.n;
    double gm[12];
    bool act;
    const double m = mollifier(c, x, gm, nullptr, act);
    if (m <= 0) return;
    double g[12];
    const double d = contact_distance(c, x, g, nullptr);
    const double fd = fd1(P, d);
    double out[12];
    if (c.type != CT_EE) {
        for (int k = 0; k < N; ++k) out[k] = (c.w * fd) * g[k];
    } else {
        const double fv = fval(P, d);
        for (int k = 0; k < N; ++k) out[k] = (c.w * fv) * (act ? gm[k] : 0.0) + (c.w * m * fd) * g[k];
    }
    for (int a = 0; a < c.n; ++a)
        for (int k = 0; k < 3; ++k) {
            const double v = out[3 * a + k];
            if (v != 0) atomicAdd(grad + 3 * (int64_t)c.vid[a] + k, v);
        }
}

// ---- Gauss-Newton forms (normal_potential.cpp:15-83, 236-308) ----
// Distance-vector coefficients c with t = sum_i c_i x_i, for the collision's
// known distance type (compute_coefficients in candidates/vertex_vertex.cpp:40-46,
// edge_vertex.cpp:45-75, edge_edge.cpp:42-96, face_vertex.cpp:42-89): VV and
// EV (P_E) fixed, EE by its stored type, FV point-plane (P_T).
__device__ __forceinline__ double pe_alpha(V3 p, V3 e0, V3 e1)
{
    const V3 e = e1 - e0;
    return dot(p - e0, e) / sqnorm(e);
}
__device__ void contact_coefficients(const Local& c, const V3* x, double* co)
{
    co[0] = co[1] = co[2] = co[3] = 0.0;
    if (c.type == CT_VV) {
        co[0] = 1.0;
        co[1] = -1.0;
    } else if (c.type == CT_EV) {
        const double a = pe_alpha(x[0], x[1], x[2]);
        co[0] = 1.0;
        co[1] = -1.0 + a;
        co[2] = -a;
    } else if (c.type == CT_FV) {
        // point_triangle_closest_point (tangent/closest_point.cpp:123-137)
        double u, v;
        ldlt2_solve(x[2] - x[1], x[3] - x[1], x[0] - x[1], u, v);
        co[0] = 1.0;
        co[1] = -1.0 + u + v;
        co[2] = -u;
        co[3] = -v;
    } else {
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
            // edge_edge_closest_point (tangent/closest_point.cpp:65-87): the
            // Gram system of (ea, -eb) against eb0 - ea0
            const V3 ea = x[1] - x[0], eb = x[3] - x[2];
            double a, b;
            ldlt2_solve(ea, eb * -1.0, x[2] - x[0], a, b);
            co[0] = 1.0 - a, co[1] = a, co[2] = -1.0 + b, co[3] = -b;
        }
        }
    }
}
// t = sum_i c_i x_i in vertex order (collision_stencil.cpp:14-25)
__device__ __forceinline__ V3 distance_vector(int n, const V3* x, const double* co)
{
    V3 t { 0, 0, 0 };
    for (int i = 0; i < n; ++i) t = t + x[i] * co[i];
    return t;
}

// Gauss-Newton Hessian diagonal: w (4 f'' c_i^2 t_d^2 + 2 f' c_i^2) at
// d^2 = |t|^2, scattered like the gradient.  The mollifier plays no part.
__global__ void __launch_bounds__(BLOCK) k_gn_diagonal(ContactsView cv, const int* __restrict__ E,
    const int* __restrict__ F, const double* __restrict__ V, const Params* __restrict__ sp, SceneView sv,
    double* __restrict__ diag)
{
    const int64_t n = cv.nvv + cv.nev + cv.nee + cv.nfv;
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    Local c;
    load_contact(cv, E, F, i, c);
    const Params P = sp[sv.of(c.vid[0])];
    V3 x[4];
    gather(V, c, x);
    double co[4];
    contact_coefficients(c, x, co);
    const V3 t = distance_vector(c.n, x, co);
    const double d2 = sqnorm(t);
    const double s1 = c.w * 4.0 * fd2(P, d2), s2 = c.w * 2.0 * fd1(P, d2);
    const double t2[3] = { t.x * t.x, t.y * t.y, t.z * t.z };
    for (int a = 0; a < c.n; ++a) {
        const double ci2 = co[a] * co[a];
        for (int k = 0; k < 3; ++k) {
            const double v = s1 * (ci2 * t2[k]) + s2 * ci2;
            if (v != 0) atomicAdd(diag + 3 * (int64_t)c.vid[a] + k, v);
        }
    }
}

// Gauss-Newton quadratic form p^T H p: w (4 f'' (J^T p . t)^2 + 2 f' |J^T p|^2)
// with J^T p = sum_i c_i p_i; per-block partial sums (deterministic).
__global__ void __launch_bounds__(BLOCK) k_gn_quadratic_form(ContactsView cv, const int* __restrict__ E,
    const int* __restrict__ F, const double* __restrict__ V, const double* __restrict__ pv,
    const Params* __restrict__ sp, SceneView sv, double* __restrict__ partial)
{
    const int64_t n = cv.nvv + cv.nev + cv.nee + cv.nfv;
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    double q = 0;
    if (i < n) {
        Local c;
        load_contact(cv, E, F, i, c);
        const Params P = sp[sv.of(c.vid[0])];
        V3 x[4], pl[4];
        gather(V, c, x);
        gather(pv, c, pl);
        double co[4];
        contact_coefficients(c, x, co);
        const V3 t = distance_vector(c.n, x, co);
        const double d2 = sqnorm(t);
        const V3 pj = distance_vector(c.n, pl, co);
        const double pjt = dot(pj, t);
        q = c.w * (4.0 * fd2(P, d2) * (pjt * pjt) + 2.0 * fd1(P, d2) * sqnorm(pj));
    }
    typedef cub::BlockReduce<double, BLOCK> BR;
    __shared__ typename BR::TempStorage tmp;
    const double s = BR(tmp).Sum(q);
    if (threadIdx.x == 0) partial[blockIdx.x] = s;
}


// Local Hessian of one contact (normal_potential.cpp:174-232 before the PSD
// projection) written to its 144-double slab of Hs (row-major, N = 3n).
// One instantiation per contact type (contacts of a type are contiguous:
// VV, EV, EE, FV), so each kernel holds only its own distance function.
// proj[i] = 0 marks the mollified edge-edge case with m(x) <= 0, which the
// reference returns without projection.
template <int TYPE>
__global__ void __launch_bounds__(LH_BLOCK) k_local_hessian(ContactsView cv, const int* __restrict__ E,
    const int* __restrict__ F, const double* __restrict__ V, const Params* __restrict__ sp, SceneView sv,
    Slab hs, uint8_t* __restrict__ proj, int64_t first, int64_t count)
{
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= count) return;
    const int64_t i = first + t;
    Local c;
    load_contact(cv, E, F, i, c);
    const Params P = sp[sv.of(c.vid[0])];
    V3 x[4];
    gather(V, c, x);
    constexpr int NS = TYPE == CT_VV ? 2 : (TYPE == CT_EV ? 3 : 4);
    constexpr int N = 3 * NS;
    if (TYPE == CT_FV && fp32_contact(P, c, x)) {
        float gf[12], Hf[144];
        const double d = fv_local_f(x, gf, Hf);
        const float w = (float)c.w, a = w * fd2f(P, d), b = w * fd1f(P, d);
        for (int r = 0; r < 12; ++r)
            for (int q = r; q < 12; ++q) {
                const double v = (double)(a * gf[r] * gf[q] + b * Hf[r * 12 + q]);
                hs.at(i, r * 12 + q) = v;
                hs.at(i, q * 12 + r) = v;
            }
        proj[i] = 1;
        return;
    }
    double g[12], H[144];
    double d;
    if (TYPE == CT_VV) d = pp_local(x, 6, 0, 1, g, H);
    else if (TYPE == CT_EV) d = pl_local(x, 9, 0, 1, 2, g, H);
    else if (TYPE == CT_EE) d = ee_local(x, c.dtype, g, H);
    else d = pplane_local(x, g, H);
    uint8_t pr = 1;
    if (TYPE == CT_EE) {
        // w m(x) f(d(x)): the distance terms first, then the mollifier terms
        // added in place (the distance Hessian buffer is reused for the
        // mollifier Hessian to halve the local memory of this kernel)
        bool act;
        const double m = mollifier(c, x, nullptr, nullptr, act);
        const double fv = fval(P, d);
        if (act && m <= 0) {
            double gm[12];
            mollifier(c, x, gm, H, act);
            for (int r = 0; r < 12; ++r)
                for (int q = r; q < 12; ++q) {
                    const double v = (c.w * fv) * H[r * 12 + q];
                    hs.at(i, r * 12 + q) = v;
                    hs.at(i, q * 12 + r) = v;
                }
            pr = 0;
        } else {
            const double fd = fd1(P, d), fdd = fd2(P, d);
            const double wm = c.w * m;
            // the matrices are symmetric: upper triangles formed, mirrored
            for (int r = 0; r < 12; ++r)
                for (int q = r; q < 12; ++q) {
                    const double v = (wm * fdd) * g[r] * g[q] + (wm * fd) * H[r * 12 + q];
                    hs.at(i, r * 12 + q) = v;
                    hs.at(i, q * 12 + r) = v;
                }
            if (act) {
                double gm[12];
                mollifier(c, x, gm, H, act);
                for (int r = 0; r < 12; ++r)
                    for (int q = r; q < 12; ++q) {
                        const double gfm_rq = (c.w * fd) * g[r] * gm[q];
                        const double gfm_qr = (c.w * fd) * g[q] * gm[r];
                        const double v = hs.at(i, r * 12 + q) + ((c.w * fv) * H[r * 12 + q] + gfm_rq + gfm_qr);
                        hs.at(i, r * 12 + q) = v;
                        hs.at(i, q * 12 + r) = v;
                    }
            }
        }
    } else {
        const double fd = fd1(P, d), fdd = fd2(P, d);
#pragma unroll
        for (int r = 0; r < N; ++r)
#pragma unroll
            for (int q = r; q < N; ++q) {
                const double v = (c.w * fdd) * g[r] * g[q] + (c.w * fd) * H[r * N + q];
                hs.at(i, r * N + q) = v;
                hs.at(i, q * N + r) = v;
            }
    }
    proj[i] = pr;
}


// Contacts [first, first + count) of the chunk.
__global__ void __launch_bounds__(PSD_BLOCK) k_psd(ContactsView cv, Slab hs,
    const uint8_t* __restrict__ proj, int method, int* __restrict__ fail, int64_t first, int64_t count)
{
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= count) return;
    const int64_t i = first + t;
    if (!proj[i]) return;
    if (!project_psd<double>(stencil_size(cv, i), SlabAcc { hs, i }, method)) atomicOr(fail, 1);
}

// Contribution id j (position in the block-key list) -> contact, local
// vertex pair (a, b) and stencil size.
__device__ __forceinline__ void decode_contribution(const ContactsView& cv, int64_t j, int64_t& i, int& a, int& b,
    int& ns)
{
    const int64_t e1 = 4 * cv.nvv, e2 = e1 + 9 * cv.nev;
    if (j < e1) {
        i = j / 4;
        ns = 2;
        const int r = (int)(j % 4);
        a = r / 2;
        b = r % 2;
    } else if (j < e2) {
        i = cv.nvv + (j - e1) / 9;
        ns = 3;
        const int r = (int)((j - e1) % 9);
        a = r / 3;
        b = r % 3;
    } else {
        i = cv.nvv + cv.nev + (j - e2) / 16;
        ns = 4;
        const int r = (int)((j - e2) % 16);
        a = r / 4;
        b = r % 4;
    }
}

// Sort-by-key reduction into CSR: one thread per stored value (block q,
// entry k,l) sums the contributions of block q in sorted (deterministic)
// order and writes the value once.
// ---- Shape derivative (normal_potential.cpp:310-416), edge-edge part ----
// Without area weighting the shape derivative of a collision is w times its
// unprojected local Hessian; edge-edge collisions use the reference's
// mollified form
//   f jac_m + gradx_m gradu_f^T + gradu_f gradu_m^T + gradu_m gradu_f^T + m hessu_f
// with eps_x and its gradient from the rest positions (rows and columns as
// the reference writes them).
__global__ void __launch_bounds__(LH_BLOCK) k_shape_local_ee(ContactsView cv, const int* __restrict__ E,
    const int* __restrict__ F, const double* __restrict__ V, const double* __restrict__ rest,
    const Params* __restrict__ sp, SceneView sv, Slab hs, int64_t first, int64_t count)
{
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= count) return;
    const int64_t i = first + t;
    Local c;
    load_contact(cv, E, F, i, c);
    const Params P = sp[sv.of(c.vid[0])];
    V3 x[4], xr[4];
    gather(V, c, x);
    gather(rest, c, xr);
    double g[12], H[144];
    const double d = ee_local(x, c.dtype, g, H);
    const double f = c.w * fval(P, d), a1 = c.w * fd1(P, d), a2 = c.w * fd2(P, d);
    const double eps = ee_mollifier_threshold(xr[0], xr[1], xr[2], xr[3]);
    const double sq = ee_cross_sqnorm(x[0], x[1], x[2], x[3]);
    double gs[12], ge[12], Hs[144];
    double m = 1.0, m1 = 0, dme = 0, dmse = 0;
    const bool act = sq < eps;
    if (act) {
        const double xe = sq / eps;
        m = (-xe + 2) * xe;
        const double inv = 1 / eps;
        m1 = 2 * inv * fma(-inv, sq, 1.0);
        dme = 2 * sq * (-eps + sq) / (eps * eps * eps);
        dmse = 2 * (-eps + 2 * sq) / (eps * eps * eps);
        double gr[6], Hr[36];
        cross_sq(x[1] - x[0], x[3] - x[2], gr, Hr);
        const int pos[2] = { 1, 3 }, neg[2] = { 0, 2 };
        expand_g<2>(12, pos, neg, gr, gs);
        expand_h<2>(12, pos, neg, Hr, Hs);
        // gradient of eps_x = 1e-3 |ea|^2 |eb|^2 with respect to the rest positions
        const V3 ea = xr[0] - xr[1], eb = xr[2] - xr[3];
        const double la = sqnorm(ea), lb = sqnorm(eb);
        for (int k = 0; k < 3; ++k) {
            ge[k] = 1e-3 * 2 * comp(ea, k) * lb;
            ge[3 + k] = -ge[k];
            ge[6 + k] = 1e-3 * la * 2 * comp(eb, k);
            ge[9 + k] = -ge[6 + k];
        }
    }
    for (int r = 0; r < 12; ++r)
        for (int q = 0; q < 12; ++q) {
            const double gfr = a1 * g[r], gfq = a1 * g[q];
            const double hf = a2 * g[r] * g[q] + a1 * H[r * 12 + q];
            double v = m * hf;
            if (act) {
                const double jm = dmse * ge[r] * gs[q] + m1 * Hs[r * 12 + q];
                v = f * jm + (dme * ge[r]) * gfq + gfr * (m1 * gs[q]) + (m1 * gs[r]) * gfq + m * hf;
            }
            hs.at(i, r * 12 + q) = v;
        }
}

// ---- Area-weighted shape derivative (normal_potential.cpp:310-416 with the
// weight gradients of normal_collisions_builder.cpp:146,181-191 and the area
// Jacobians of collision_mesh.cpp:376-432) ----
// Both terms are emitted as (row * ndof + col, value) triplets and summed
// by key: the second term from the local slabs, the first term
// (grad_u f / w)(grad_x w)^T with grad_x w summed over the record's weight
// sources, 0.25 times a vertex's or the two edges' area Jacobians.
struct ShapeSources {
    const int *vv_off, *ev_off;
    const int2 *vv_src, *ev_src;
    const int *vf_off, *vf_adj, *ef_off, *ef_adj, *ve_off, *ve_adj;
};
__device__ __forceinline__ int vertex_jac_entries(const ShapeSources& S, int v)
{
    const int nf = S.vf_off[v + 1] - S.vf_off[v];
    return nf > 0 ? 9 * nf : 6 * (S.ve_off[v + 1] - S.ve_off[v]);
}
__device__ __forceinline__ int edge_jac_entries(const ShapeSources& S, int e)
{
    const int nf = S.ef_off[e + 1] - S.ef_off[e];
    return nf > 0 ? 9 * nf : 6;
}
// d|A_f|/dx / 3 over the face's 9 rest dofs: n x (t_{i+2} - t_{i+1}) / 6
__device__ __forceinline__ void face_area_grad3(const double* __restrict__ R, const int* __restrict__ F, int f,
    double* g)
{
    const V3 t0 = load_v3(R, F[3 * f]), t1 = load_v3(R, F[3 * f + 1]), t2 = load_v3(R, F[3 * f + 2]);
    V3 n = cross(t1 - t0, t2 - t0);
    const double nn = sqnorm(n);
    if (nn > 0) {
        const double r = sqrt(nn);
        n = V3 { n.x / r, n.y / r, n.z / r };
    }
    const V3 a = cross(n, t2 - t1) * 0.5, b = cross(n, t0 - t2) * 0.5, c = cross(n, t1 - t0) * 0.5;
    const V3 gg[3] = { a, b, c };
    for (int k = 0; k < 3; ++k)
        for (int d = 0; d < 3; ++d) g[3 * k + d] = (1.0 / 3.0) * comp(gg[k], d);
}
// d|e|/dx over the edge's 6 rest dofs
__device__ __forceinline__ void edge_len_grad(const double* __restrict__ R, const int* __restrict__ E, int e, double* g)
{
    const V3 d = load_v3(R, E[2 * e]) - load_v3(R, E[2 * e + 1]);
    const double l = sqrt(sqnorm(d));
    g[0] = d.x / l, g[1] = d.y / l, g[2] = d.z / l;
    g[3] = -g[0], g[4] = -g[1], g[5] = -g[2];
}
// visit (dof, value) of 0.25 x an entity's area Jacobian
template <class Fn> __device__ void visit_vertex_jac(const ShapeSources& S, const double* R, const int* E,
    const int* F, int v, Fn&& fn)
{
    const int f0 = S.vf_off[v], f1 = S.vf_off[v + 1];
    if (f1 > f0) {
        for (int q = f0; q < f1; ++q) {
            const int f = S.vf_adj[q];
            double g[9];
            face_area_grad3(R, F, f, g);
            for (int k = 0; k < 3; ++k)
                for (int d = 0; d < 3; ++d) fn(3 * (int64_t)F[3 * f + k] + d, 0.25 * g[3 * k + d]);
        }
    } else {
        for (int q = S.ve_off[v]; q < S.ve_off[v + 1]; ++q) {
            const int e = S.ve_adj[q];
            double g[6];
            edge_len_grad(R, E, e, g);
            for (int k = 0; k < 2; ++k)
                for (int d = 0; d < 3; ++d) fn(3 * (int64_t)E[2 * e + k] + d, 0.25 * (0.5 * g[3 * k + d]));
        }
    }
}
template <class Fn> __device__ void visit_edge_jac(const ShapeSources& S, const double* R, const int* E,
    const int* F, int e, Fn&& fn)
{
    const int f0 = S.ef_off[e], f1 = S.ef_off[e + 1];
    if (f1 > f0) {
        for (int q = f0; q < f1; ++q) {
            const int f = S.ef_adj[q];
            double g[9];
            face_area_grad3(R, F, f, g);
            for (int k = 0; k < 3; ++k)
                for (int d = 0; d < 3; ++d) fn(3 * (int64_t)F[3 * f + k] + d, 0.25 * g[3 * k + d]);
        }
    } else {
        double g[6];
        edge_len_grad(R, E, e, g);
        for (int k = 0; k < 2; ++k)
            for (int d = 0; d < 3; ++d) fn(3 * (int64_t)E[2 * e + k] + d, 0.25 * g[3 * k + d]);
    }
}
// the weight sources of contact i: calls fn(s0, s1) for each
template <class Fn> __device__ void visit_sources(const ContactsView& cv, const ShapeSources& S, int64_t i, Fn&& fn)
{
    if (i < cv.nvv) {
        for (int q = S.vv_off[i]; q < S.vv_off[i + 1]; ++q) fn(S.vv_src[q].x, S.vv_src[q].y);
    } else if (i < cv.nvv + cv.nev) {
        const int64_t j = i - cv.nvv;
        for (int q = S.ev_off[j]; q < S.ev_off[j + 1]; ++q) fn(S.ev_src[q].x, S.ev_src[q].y);
    } else if (i < cv.nvv + cv.nev + cv.nee) {
        const int2 p = cv.ee[i - cv.nvv - cv.nev];
        fn(p.x, p.y);
    } else {
        const int2 p = cv.fv[i - cv.nvv - cv.nev - cv.nee];
        fn(p.y, -1);
    }
}

__global__ void k_shape_count(ContactsView cv, const int* __restrict__ E, const int* __restrict__ F,
    ShapeSources S, int64_t* __restrict__ counts)
{
    const int64_t n = cv.nvv + cv.nev + cv.nee + cv.nfv;
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    Local c;
    load_contact(cv, E, F, i, c);
    const int N = 3 * c.n;
    int64_t cnt = (int64_t)N * N;
    visit_sources(cv, S, i, [&](int s0, int s1) {
        cnt += (int64_t)N * (s1 < 0 ? vertex_jac_entries(S, s0) : edge_jac_entries(S, s0) + edge_jac_entries(S, s1));
    });
    counts[i] = cnt;
}

__global__ void k_shape_emit(ContactsView cv, const int* __restrict__ E, const int* __restrict__ F,
    const double* __restrict__ V, const double* __restrict__ R, const Params* __restrict__ sp, SceneView sv, Slab hs,
    ShapeSources S, const int64_t* __restrict__ offs, int64_t ndof, unsigned long long* __restrict__ keys,
    double* __restrict__ vals)
{
    const int64_t n = cv.nvv + cv.nev + cv.nee + cv.nfv;
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    Local c;
    load_contact(cv, E, F, i, c);
    const int N = 3 * c.n;
    int64_t o = offs[i];
    // second term: the local matrix of the slab
    for (int a = 0; a < c.n; ++a)
        for (int b = 0; b < c.n; ++b)
            for (int k = 0; k < 3; ++k)
                for (int l = 0; l < 3; ++l) {
                    keys[o] = (unsigned long long)((3 * (int64_t)c.vid[a] + k) * ndof + 3 * (int64_t)c.vid[b] + l);
                    vals[o] = hs.at(i, (3 * a + k) * N + 3 * b + l);
                    ++o;
                }
    // first term: q = (per-collision gradient) / w, times the weight gradient
    const Params P = sp[sv.of(c.vid[0])];
    V3 x[4];
    gather(V, c, x);
    double q[12];
    double gm[12];
    bool act;
    const double mm = mollifier(c, x, gm, nullptr, act);
    if (mm <= 0) {
        for (int r = 0; r < N; ++r) q[r] = 0;
    } else {
        double g[12];
        const double d = contact_distance(c, x, g, nullptr);
        const double fd = fd1(P, d);
        if (c.type != CT_EE) {
            for (int r = 0; r < N; ++r) q[r] = ((c.w * fd) * g[r]) / c.w;
        } else {
            const double fv = fval(P, d);
            for (int r = 0; r < N; ++r) q[r] = ((c.w * fv) * (act ? gm[r] : 0.0) + (c.w * mm * fd) * g[r]) / c.w;
        }
    }
    auto emit = [&](int64_t col, double wv) {
        for (int a = 0; a < c.n; ++a)
            for (int k = 0; k < 3; ++k) {
                keys[o] = (unsigned long long)((3 * (int64_t)c.vid[a] + k) * ndof + col);
                vals[o] = q[3 * a + k] * wv;
                ++o;
            }
    };
    visit_sources(cv, S, i, [&](int s0, int s1) {
        if (s1 < 0) visit_vertex_jac(S, R, E, F, s0, emit);
        else {
            visit_edge_jac(S, R, E, F, s0, emit);
            visit_edge_jac(S, R, E, F, s1, emit);
        }
    });
}

__global__ void k_iota(int* __restrict__ p, int n)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) p[i] = i;
}
__global__ void k_gather_vals(const double* __restrict__ v, const int* __restrict__ idx, int n, double* __restrict__ out)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = v[idx[i]];
}
// duplicates summed in key order; column of each unique key
__global__ void k_sum_key_runs(const unsigned long long* __restrict__ uniq, const int* __restrict__ counts,
    const int* __restrict__ offs, const int* __restrict__ d_num, const double* __restrict__ v, int64_t ndof,
    int* __restrict__ col, double* __restrict__ val)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= *d_num) return;
    double s = 0.0;
    for (int j = offs[i], e = offs[i] + counts[i]; j < e; ++j) s += v[j];
    col[i] = (int)((int64_t)uniq[i] % ndof);
    val[i] = s;
}
// row pointers of sorted unique keys: the first key of each row
__global__ void k_rows_from_keys(const unsigned long long* __restrict__ uniq, const int* __restrict__ d_num,
    int64_t ndof, int64_t* __restrict__ row_ptr)
{
    const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r > ndof) return;
    const unsigned long long key = (unsigned long long)(r * ndof);
    int lo = 0, hi = *d_num;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (uniq[mid] < key) lo = mid + 1;
        else hi = mid;
    }
    row_ptr[r] = lo;
}

// ---- Friction (tangential_potential.cpp:156-331, friction/smooth_mu.cpp,
// friction/smooth_friction_mollifier.cpp; isotropic) ----
__device__ __forceinline__ double fr_smooth_mu(double y, double ms, double mk, double ev)
{
    if (ms == mk || fabs(y) >= ev) return mk;
    const double z = fabs(y) / ev;
    if (fabs(y) < 0.5 * ev) return 2 * (mk - ms) * z * z + ms;
    return -2 * (mk - ms) * (z * (z - 2) + 1) + mk;
}
__device__ __forceinline__ double fr_mu_f0(double y, double ms, double mk, double ev)
{
    if (ms == mk || fabs(y) >= ev) {
        const double f0 = fabs(y) >= ev ? y : y * y * (1 - y / (3 * ev)) / ev + ev / 3;
        return mk * f0;
    }
    const double dm = mk - ms, z = fabs(y) / ev;
    if (fabs(y) < 0.5 * ev)
        return y * z * (z * (z * (1 - 0.4 * z) * dm - ms / 3.0) + ms) + (9.0 / 16.0) * ev * mk - (11.0 / 48.0) * ev * ms;
    return y * z * (z * (z * (0.4 * z - 2) * dm + (3 * mk - (10.0 / 3.0) * ms)) + (2 * ms - mk)) + 0.6 * ev * mk
        - (4.0 / 15.0) * ev * ms;
}
__device__ __forceinline__ double fr_mu_f1_over_x(double y, double ms, double mk, double ev)
{
    const double f1x = fabs(y) >= ev ? 1 / y : (2 - y / ev) / ev;
    return fr_smooth_mu(y, ms, mk, ev) * f1x;
}
__device__ __forceinline__ double fr_mu_f2_x_minus_f1_over_x3(double y, double ms, double mk, double ev)
{
    if (ms == mk || fabs(y) >= ev) return mk * (fabs(y) >= ev ? -1 / (y * y * y) : -1 / (y * ev * ev));
    const double dm = mk - ms, z = 1 / ev;
    if (fabs(y) < 0.5 * ev) return z * z * (z * (8 - 6 * y * z) * dm - ms / y);
    return z * z * (z * (6 * y * z - 16) * dm + (9 * mk - 10 * ms) / y);
}

// One tangential collision at velocities v: u = P^T (relative velocity),
// T = Gamma^T P (rows 3k+d = g_k (P(d,0), P(d,1))), mu and w N.
struct FrictionLocal {
    double T[12][2];
    double u0, u1, nu, ms, mk, scl;
};
__device__ __forceinline__ void friction_setup(const FrictionView& f, int64_t i, const Local& c, const V3* v,
    FrictionLocal& L)
{
    const double c0 = f.cp[2 * i], c1 = f.cp[2 * i + 1];
    const double* P = f.P + 6 * i;
    const V3 b0 { P[0], P[1], P[2] }, b1 { P[3], P[4], P[5] };
    V3 rv;
    double g[4] = { 0, 0, 0, 0 };
    if (c.type == CT_VV) {
        rv = v[0] - v[1];
        g[0] = 1, g[1] = -1;
    } else if (c.type == CT_EV) {
        rv = v[0] - ((v[2] - v[1]) * c0 + v[1]);
        g[0] = 1, g[1] = c0 - 1, g[2] = -c0;
    } else if (c.type == CT_EE) {
        rv = ((v[1] - v[0]) * c0 + v[0]) - ((v[3] - v[2]) * c1 + v[2]);
        g[0] = 1 - c0, g[1] = c0, g[2] = c1 - 1, g[3] = -c1;
    } else {
        rv = v[0] - ((v[1] + (v[2] - v[1]) * c0) + (v[3] - v[1]) * c1);
        g[0] = 1, g[1] = c0 + c1 - 1, g[2] = -c0, g[3] = -c1;
    }
    // anisotropic slip scaling (tangential_potential.cpp:166-175, 200-212)
    const double a0 = f.aniso[2 * i], a1 = f.aniso[2 * i + 1];
    L.u0 = a0 * dot(b0, rv);
    L.u1 = a1 * dot(b1, rv);
    L.nu = sqrt(L.u0 * L.u0 + L.u1 * L.u1);
    L.ms = f.mu_s[i];
    L.mk = f.mu_k[i];
    L.scl = c.w * f.N[i];
    for (int k = 0; k < c.n; ++k)
        for (int d = 0; d < 3; ++d) {
            L.T[3 * k + d][0] = (g[k] * P[d]) * a0;
            L.T[3 * k + d][1] = (g[k] * P[3 + d]) * a1;
        }
}

// Symmetric 2x2 PSD projection (eigen_ext.tpp:64-108 for n = 2): unchanged
// when the smaller eigenvalue is >= 0, else negative eigenvalues clamped to 0
// (CLAMP) or flipped (ABS).  Row-major A; the lower entry is the off-diagonal.
__device__ void project_psd2(double* A, int method)
{
    if (method == IPCG_PSD_NONE) return;
    const double a = A[0], b = A[2], c = A[3];
    double l1, l2, vx, vy;
    if (b == 0) {
        l1 = a <= c ? a : c;
        l2 = a <= c ? c : a;
        vx = a <= c ? 1.0 : 0.0;
        vy = a <= c ? 0.0 : 1.0;
    } else {
        const double m = 0.5 * (a + c), h = 0.5 * (a - c);
        const double r = sqrt(h * h + b * b);
        l1 = m - r;
        l2 = m + r;
        // eigenvector of l1 from the better-conditioned row
        const double px = l1 - c, py = b, qx = b, qy = l1 - a;
        if (px * px + py * py >= qx * qx + qy * qy) vx = px, vy = py;
        else vx = qx, vy = qy;
        const double nv = sqrt(vx * vx + vy * vy);
        vx /= nv;
        vy /= nv;
    }
    if (l1 >= 0.0) return;
    l1 = method == IPCG_PSD_CLAMP ? 0.0 : -l1;
    if (l2 < 0) l2 = method == IPCG_PSD_CLAMP ? 0.0 : -l2;
    const double wx = -vy, wy = vx;
    A[0] = l1 * vx * vx + l2 * wx * wx;
    A[1] = A[2] = l1 * vx * vy + l2 * wx * wy;
    A[3] = l1 * vy * vy + l2 * wy * wy;
}

__global__ void __launch_bounds__(BLOCK) k_friction_energy(ContactsView cv, const int* __restrict__ E,
    const int* __restrict__ F, const double* __restrict__ U, FrictionView f, double* __restrict__ partial)
{
    const int64_t n = cv.nvv + cv.nev + cv.nee + cv.nfv;
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    double e = 0;
    if (i < n) {
        Local c;
        load_contact(cv, E, F, i, c);
        V3 v[4];
        gather(U, c, v);
        FrictionLocal L;
        friction_setup(f, i, c, v, L);
        e = L.scl * fr_mu_f0(L.nu, L.ms, L.mk, f.eps_v);
    }
    typedef cub::BlockReduce<double, BLOCK> BR;
    __shared__ typename BR::TempStorage tmp;
    const double sum = BR(tmp).Sum(e);
    if (threadIdx.x == 0) partial[blockIdx.x] = sum;
}

// Batches: per-scene friction energies (a block almost always holds one
// scene, as in k_energy_scenes).
__global__ void __launch_bounds__(BLOCK) k_friction_energy_scenes(ContactsView cv, const int* __restrict__ E,
    const int* __restrict__ F, const double* __restrict__ U, FrictionView f, SceneView sv, double* __restrict__ energy)
{
    const int64_t n = cv.nvv + cv.nev + cv.nee + cv.nfv;
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    double e = 0;
    int scene = -1;
    if (i < n) {
        Local c;
        load_contact(cv, E, F, i, c);
        scene = sv.of(c.vid[0]);
        V3 v[4];
        gather(U, c, v);
        FrictionLocal L;
        friction_setup(f, i, c, v, L);
        e = L.scl * fr_mu_f0(L.nu, L.ms, L.mk, f.eps_v);
    }
    __shared__ int s_lo, s_hi;
    if (threadIdx.x == 0) {
        s_lo = 0x7fffffff;
        s_hi = -1;
    }
    __syncthreads();
    if (scene >= 0) {
        atomicMin(&s_lo, scene);
        atomicMax(&s_hi, scene);
    }
    __syncthreads();
    if (s_lo == s_hi) {
        typedef cub::BlockReduce<double, BLOCK> BR;
        __shared__ typename BR::TempStorage tmp;
        const double sum = BR(tmp).Sum(e);
        if (threadIdx.x == 0 && s_hi >= 0) atomicAdd(energy + s_hi, sum);
    } else if (scene >= 0 && e != 0) {
        atomicAdd(energy + scene, e);
    }
}

__global__ void __launch_bounds__(BLOCK) k_friction_gradient(ContactsView cv, const int* __restrict__ E,
    const int* __restrict__ F, const double* __restrict__ U, FrictionView f, double* __restrict__ grad)
{
    const int64_t n = cv.nvv + cv.nev + cv.nee + cv.nfv;
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    Local c;
    load_contact(cv, E, F, i, c);
    V3 v[4];
    gather(U, c, v);
    FrictionLocal L;
    friction_setup(f, i, c, v, L);
    const double f1x = fr_mu_f1_over_x(L.nu, L.ms, L.mk, f.eps_v);
    const double s0 = (f1x * L.u0) * L.scl, s1 = (f1x * L.u1) * L.scl;
    for (int a = 0; a < c.n; ++a)
        for (int k = 0; k < 3; ++k) {
            const int r = 3 * a + k;
            const double val = L.T[r][0] * s0 + L.T[r][1] * s1;
            if (val != 0) atomicAdd(grad + 3 * (int64_t)c.vid[a] + k, val);
        }
}

// Local friction Hessian (tangential_potential.cpp:233-331) into the slab:
// dynamic (|u| > eps_v) rank one along u's perpendicular, |u| = 0 the
// isotropic limit, otherwise the 2x2 inner matrix projected in place.
template <int TYPE>
__global__ void __launch_bounds__(LH_BLOCK) k_friction_local_hessian(ContactsView cv, const int* __restrict__ E,
    const int* __restrict__ F, const double* __restrict__ U, FrictionView f, Slab hs, int64_t first, int64_t count,
    int psd)
{
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= count) return;
    const int64_t i = first + t;
    constexpr int NS = TYPE == CT_VV ? 2 : (TYPE == CT_EV ? 3 : 4);
    constexpr int N = 3 * NS;
    Local c;
    load_contact(cv, E, F, i, c);
    V3 v[4];
    gather(U, c, v);
    FrictionLocal L;
    friction_setup(f, i, c, v, L);
    const double f1x = fr_mu_f1_over_x(L.nu, L.ms, L.mk, f.eps_v);
    if (L.nu > f.eps_v) {
        if (psd != IPCG_PSD_NONE && L.scl <= 0) {
            for (int k = 0; k < N * N; ++k) hs.at(i, k) = 0.0;
            return;
        }
        const double cc = L.scl * f1x / (L.nu * L.nu);
        const double q0 = cc * -L.u1, q1 = cc * L.u0;
        for (int r = 0; r < N; ++r) {
            const double ar = L.T[r][0] * q0 + L.T[r][1] * q1;
            for (int q = 0; q < N; ++q) hs.at(i, r * N + q) = ar * (-L.u1 * L.T[q][0] + L.u0 * L.T[q][1]);
        }
    } else if (L.nu == 0) {
        if (psd != IPCG_PSD_NONE && L.scl <= 0) {
            for (int k = 0; k < N * N; ++k) hs.at(i, k) = 0.0;
            return;
        }
        const double cc = L.scl * f1x;
        for (int r = 0; r < N; ++r)
            for (int q = 0; q < N; ++q)
                hs.at(i, r * N + q) = (cc * L.T[r][0]) * L.T[q][0] + (cc * L.T[r][1]) * L.T[q][1];
    } else {
        const double f2 = fr_mu_f2_x_minus_f1_over_x3(L.nu, L.ms, L.mk, f.eps_v);
        double in[4] = { f2 * L.u0 * L.u0, f2 * L.u0 * L.u1, f2 * L.u1 * L.u0, f2 * L.u1 * L.u1 };
        in[0] += f1x;
        in[3] += f1x;
        for (int k = 0; k < 4; ++k) in[k] *= L.scl;
        project_psd2(in, psd);
        for (int r = 0; r < N; ++r) {
            const double t0 = L.T[r][0] * in[0] + L.T[r][1] * in[2], t1 = L.T[r][0] * in[1] + L.T[r][1] * in[3];
            for (int q = 0; q < N; ++q) hs.at(i, r * N + q) = t0 * L.T[q][0] + t1 * L.T[q][1];
        }
    }
}

// ---- TangentialCollisions::build (tangential_collisions.cpp:60-170) ----
__device__ __forceinline__ V3 normalized(V3 a)
{
    const double n = sqnorm(a);
    if (!(n > 0)) return a;
    const double r = sqrt(n);
    return V3 { a.x / r, a.y / r, a.z / r };
}

// Closest point and tangent basis of a tangential collision of the given
// type at stencil positions x (tangent/closest_point.cpp,
// tangent/tangent_basis.cpp).
__device__ void tangential_frame(int type, const V3* x, double& cp0, double& cp1, V3& b0, V3& b1)
{
    cp0 = cp1 = 0;
    if (type == CT_VV) {
        const V3 d = x[1] - x[0];
        const V3 cx = cross(V3 { 1, 0, 0 }, d), cy = cross(V3 { 0, 1, 0 }, d);
        const V3 cc = sqnorm(cx) > sqnorm(cy) ? cx : cy;
        b0 = normalized(cc);
        b1 = normalized(cross(d, cc));
    } else if (type == CT_EV) {
        const V3 e = x[2] - x[1];
        cp0 = dot(x[0] - x[1], e) / sqnorm(e);
        b0 = normalized(e);
        b1 = normalized(cross(e, x[0] - x[1]));
    } else if (type == CT_EE) {
        const V3 ea = x[1] - x[0], eb = x[3] - x[2];
        ldlt2_solve(ea, eb * -1.0, x[2] - x[0], cp0, cp1);
        b0 = normalized(ea);
        b1 = normalized(cross(cross(ea, eb), ea));
    } else {
        const V3 e0 = x[2] - x[1];
        ldlt2_solve(e0, x[3] - x[1], x[0] - x[1], cp0, cp1);
        b0 = normalized(e0);
        b1 = normalized(cross(cross(e0, x[3] - x[1]), e0));
    }
}

// update_lagged_anisotropic_friction_coefficients (tangential_collisions.cpp:
// 19-58, 387-420): at rest + lagged displacement, tau = T^T v with T =
// Gamma^T P, scaled by mu_aniso; the elliptical effective coefficients along
// tau (smooth_mu.cpp:117-171), or the scalar ones without directional
// static coefficients.
__global__ void k_tangential_update_lagged(ContactsView cv, const int* __restrict__ E, const int* __restrict__ F,
    const double* __restrict__ rest, const double* __restrict__ lagged, const double* __restrict__ vel,
    const double* __restrict__ aniso, const double* __restrict__ ms_a, const double* __restrict__ mk_a,
    const double* __restrict__ mu_s, const double* __restrict__ mu_k, double* __restrict__ ms_eff,
    double* __restrict__ mk_eff)
{
    const int64_t n = cv.nvv + cv.nev + cv.nee + cv.nfv;
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double s0 = ms_a[2 * i], s1 = ms_a[2 * i + 1];
    if (s0 * s0 + s1 * s1 == 0) {
        ms_eff[i] = mu_s[i];
        mk_eff[i] = mu_k[i];
        return;
    }
    Local c;
    load_contact(cv, E, F, i, c);
    V3 x[4], v[4];
    for (int k = 0; k < c.n; ++k) {
        x[k] = load_v3(rest, c.vid[k]) + load_v3(lagged, c.vid[k]);
        v[k] = load_v3(vel, c.vid[k]);
    }
    double cp0, cp1;
    V3 b0, b1;
    tangential_frame(c.type, x, cp0, cp1, b0, b1);
    double g[4] = { 0, 0, 0, 0 };
    if (c.type == CT_VV) g[0] = 1, g[1] = -1;
    else if (c.type == CT_EV) g[0] = 1, g[1] = cp0 - 1, g[2] = -cp0;
    else if (c.type == CT_EE) g[0] = 1 - cp0, g[1] = cp0, g[2] = cp1 - 1, g[3] = -cp1;
    else g[0] = 1, g[1] = cp0 + cp1 - 1, g[2] = -cp0, g[3] = -cp1;
    double t0 = 0, t1 = 0;
    for (int k = 0; k < c.n; ++k) {
        t0 += g[k] * dot(b0, v[k]);
        t1 += g[k] * dot(b1, v[k]);
    }
    t0 *= aniso[2 * i];
    t1 *= aniso[2 * i + 1];
    const double k0 = mk_a[2 * i], k1 = mk_a[2 * i + 1];
    const bool use_k = k0 * k0 + k1 * k1 > 0;
    const double nt = sqrt(t0 * t0 + t1 * t1);
    double d0 = 1.0, d1 = 0.0;
    if (!(nt < 1e-10)) d0 = t0 / nt, d1 = t1 / nt;
    const double a = s0 * d0, b = s1 * d1, cc = k0 * d0, dd = k1 * d1;
    ms_eff[i] = sqrt(a * a + b * b);
    mk_eff[i] = use_k ? sqrt(cc * cc + dd * dd) : mu_k[i];
}

// TangentialPotential::force (tangential_potential.cpp:40-77, 333-410):
// F = -w N(x+u) mu f1(|tau_a|)/|tau_a| T(x+u) tau_a with tau = T^T v and
// tau_a = mu_aniso . tau; N, the basis and the closest point at the lagged
// positions (distance type classified there); scattered like a gradient.
__global__ void k_friction_force(ContactsView cv, const int* __restrict__ E, const int* __restrict__ F,
    const double* __restrict__ rest, const double* __restrict__ lagged, const double* __restrict__ vel, Params P,
    const double* __restrict__ aniso, const double* __restrict__ ms_eff, const double* __restrict__ mk_eff,
    double eps_v, int no_mu, double* __restrict__ force)
{
    const int64_t n = cv.nvv + cv.nev + cv.nee + cv.nfv;
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    Local c;
    load_contact(cv, E, F, i, c);
    V3 x[4], v[4];
    for (int k = 0; k < c.n; ++k) {
        x[k] = load_v3(rest, c.vid[k]) + load_v3(lagged, c.vid[k]);
        v[k] = load_v3(vel, c.vid[k]);
    }
    double d2;
    if (c.type == CT_VV) d2 = point_point_distance(x[0], x[1]);
    else if (c.type == CT_EV) d2 = point_edge_distance(x[0], x[1], x[2], point_edge_distance_type(x[0], x[1], x[2]));
    else if (c.type == CT_EE)
        d2 = edge_edge_distance(x[0], x[1], x[2], x[3], edge_edge_distance_type(x[0], x[1], x[2], x[3]));
    else d2 = point_triangle_distance(x[0], x[1], x[2], x[3], point_triangle_distance_type(x[0], x[1], x[2], x[3]));
    const double Nf = -P.kappa * barrier_fn<1, double>(P.kind, d2 - P.dmin2, P.xhat) * 2 * sqrt(d2) * P.scale;
    double cp0, cp1;
    V3 b0, b1;
    tangential_frame(c.type, x, cp0, cp1, b0, b1);
    double g[4] = { 0, 0, 0, 0 };
    if (c.type == CT_VV) g[0] = 1, g[1] = -1;
    else if (c.type == CT_EV) g[0] = 1, g[1] = cp0 - 1, g[2] = -cp0;
    else if (c.type == CT_EE) g[0] = 1 - cp0, g[1] = cp0, g[2] = cp1 - 1, g[3] = -cp1;
    else g[0] = 1, g[1] = cp0 + cp1 - 1, g[2] = -cp0, g[3] = -cp1;
    double t0 = 0, t1 = 0;
    for (int k = 0; k < c.n; ++k) {
        t0 += g[k] * dot(b0, v[k]);
        t1 += g[k] * dot(b1, v[k]);
    }
    const double ta0 = aniso[2 * i] * t0, ta1 = aniso[2 * i + 1] * t1;
    const double ms = no_mu ? 1.0 : ms_eff[i], mk = no_mu ? 1.0 : mk_eff[i];
    const double f1x = fr_mu_f1_over_x(sqrt(ta0 * ta0 + ta1 * ta1), ms, mk, eps_v);
    const double s = -c.w * Nf * f1x;
    for (int k = 0; k < c.n; ++k)
        for (int d = 0; d < 3; ++d) {
            const double val = s * ((g[k] * comp(b0, d)) * ta0 + (g[k] * comp(b1, d)) * ta1);
            if (val != 0) atomicAdd(force + 3 * (int64_t)c.vid[k] + d, val);
        }
}

__global__ void k_fill(double* __restrict__ p, int64_t n, double v)
{
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) p[i] = v;
}

// EE collisions with cross^2 < eps_x are left out of the tangential set.
__global__ void k_tangential_keep_ee(ContactsView cv, const int* __restrict__ E, const double* __restrict__ V,
    int* __restrict__ keep)
{
    const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= cv.nee) return;
    const int2 p = cv.ee[j];
    const V3 a0 = load_v3(V, E[2 * p.x]), a1 = load_v3(V, E[2 * p.x + 1]);
    const V3 b0 = load_v3(V, E[2 * p.y]), b1 = load_v3(V, E[2 * p.y + 1]);
    keep[j] = ee_cross_sqnorm(a0, a1, b0, b1) < cv.ee_eps[j] ? 0 : 1;
}

struct TangentialOut {
    int2 *vv, *ev, *ee, *fv;
    double *vv_w, *ev_w, *ee_w, *fv_w, *ee_eps;
    int8_t* ee_dtype;
    double *N, *cp, *P, *mu_s, *mu_k;
};

__global__ void k_tangential_build(ContactsView cv, const int* __restrict__ E, const int* __restrict__ F,
    const double* __restrict__ V, const Params* __restrict__ sp, SceneView sv, const double* __restrict__ mu_s,
    const double* __restrict__ mu_k, const int* __restrict__ keep, const int* __restrict__ offs, int64_t nee_kept,
    TangentialOut o)
{
    const int64_t n = cv.nvv + cv.nev + cv.nee + cv.nfv;
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    Local c;
    load_contact(cv, E, F, i, c);
    int64_t slot, j;
    if (c.type == CT_VV) slot = j = i;
    else if (c.type == CT_EV) {
        j = i - cv.nvv;
        slot = i;
    } else if (c.type == CT_EE) {
        j = i - cv.nvv - cv.nev;
        if (!keep[j]) return;
        slot = cv.nvv + cv.nev + offs[j];
    } else {
        j = i - cv.nvv - cv.nev - cv.nee;
        slot = cv.nvv + cv.nev + nee_kept + j;
    }
    const Params P = sp[sv.of(c.vid[0])];
    V3 x[4];
    gather(V, c, x);
    double d2;
    if (c.type == CT_VV) d2 = point_point_distance(x[0], x[1]);
    else if (c.type == CT_EV) d2 = point_edge_distance(x[0], x[1], x[2], point_edge_distance_type(x[0], x[1], x[2]));
    else if (c.type == CT_EE)
        d2 = edge_edge_distance(x[0], x[1], x[2], x[3], edge_edge_distance_type(x[0], x[1], x[2], x[3]));
    else d2 = point_triangle_distance(x[0], x[1], x[2], x[3], point_triangle_distance_type(x[0], x[1], x[2], x[3]));
    // barrier_force_magnitude.cpp:5-15, then the physical scaling
    const double Nf = -P.kappa * barrier_fn<1, double>(P.kind, d2 - P.dmin2, P.xhat) * 2 * sqrt(d2) * P.scale;
    double cp0, cp1, ms, mk;
    V3 b0, b1;
    const int* v = c.vid;
    auto blend = [](double a, double b) { return (a + b) / 2; };
    tangential_frame(c.type, x, cp0, cp1, b0, b1);
    if (c.type == CT_VV) {
        ms = blend(mu_s[v[0]], mu_s[v[1]]);
        mk = blend(mu_k[v[0]], mu_k[v[1]]);
    } else if (c.type == CT_EV) {
        ms = blend((mu_s[v[2]] - mu_s[v[1]]) * cp0 + mu_s[v[1]], mu_s[v[0]]);
        mk = blend((mu_k[v[2]] - mu_k[v[1]]) * cp0 + mu_k[v[1]], mu_k[v[0]]);
    } else if (c.type == CT_EE) {
        ms = blend((mu_s[v[1]] - mu_s[v[0]]) * cp0 + mu_s[v[0]], (mu_s[v[3]] - mu_s[v[2]]) * cp1 + mu_s[v[2]]);
        mk = blend((mu_k[v[1]] - mu_k[v[0]]) * cp0 + mu_k[v[0]], (mu_k[v[3]] - mu_k[v[2]]) * cp1 + mu_k[v[2]]);
    } else {
        ms = blend(mu_s[v[1]] + cp0 * (mu_s[v[2]] - mu_s[v[1]]) + cp1 * (mu_s[v[3]] - mu_s[v[1]]), mu_s[v[0]]);
        mk = blend(mu_k[v[1]] + cp0 * (mu_k[v[2]] - mu_k[v[1]]) + cp1 * (mu_k[v[3]] - mu_k[v[1]]), mu_k[v[0]]);
    }
    if (c.type == CT_VV) {
        o.vv[slot] = cv.vv[j];
        o.vv_w[slot] = c.w;
    } else if (c.type == CT_EV) {
        o.ev[slot - cv.nvv] = cv.ev[j];
        o.ev_w[slot - cv.nvv] = c.w;
    } else if (c.type == CT_EE) {
        const int64_t k = slot - cv.nvv - cv.nev;
        o.ee[k] = cv.ee[j];
        o.ee_w[k] = c.w;
        o.ee_eps[k] = cv.ee_eps[j];
        o.ee_dtype[k] = cv.ee_dt[j];
    } else {
        const int64_t k = slot - cv.nvv - cv.nev - nee_kept;
        o.fv[k] = cv.fv[j];
        o.fv_w[k] = c.w;
    }
    o.N[slot] = Nf;
    o.cp[2 * slot] = cp0;
    o.cp[2 * slot + 1] = cp1;
    double* Po = o.P + 6 * slot;
    Po[0] = b0.x, Po[1] = b0.y, Po[2] = b0.z;
    Po[3] = b1.x, Po[4] = b1.y, Po[5] = b1.z;
    o.mu_s[slot] = ms;
    o.mu_k[slot] = mk;
}

__global__ void k_assemble(ContactsView cv, const unsigned long long* __restrict__ ukeys,
    const int* __restrict__ run_start, const int* __restrict__ run_len, const int* __restrict__ contrib,
    Slab hs, const int* __restrict__ bptr, int r0, int64_t B0, int nb, double* __restrict__ val)
{
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= 9 * (int64_t)nb) return;
    const int q = (int)(t / 9), kl = (int)(t % 9), k = kl / 3, l = kl % 3;
    double sum = 0;
    const int s0 = run_start[q], s1 = s0 + run_len[q];
    for (int s = s0; s < s1; ++s) {
        int64_t i;
        int a, b, ns;
        decode_contribution(cv, contrib[s], i, a, b, ns);
        const int N = 3 * ns;
        sum += hs.at(i, (3 * a + k) * N + 3 * b + l);
    }
    const unsigned long long key = ukeys[q];
    const int j = (int)(key >> 32) - r0;
    const int b0 = bptr[j];
    const int64_t nbr = bptr[j + 1] - b0;
    val[9 * (B0 + b0) + 3 * (int64_t)(q - b0) + 3 * k * nbr + l] = sum;
}

__global__ void k_block_keys(ContactsView cv, const int* __restrict__ E, const int* __restrict__ F,
    unsigned long long* __restrict__ keys, int* __restrict__ ids, long long nk, Guard gd)
{
    const int64_t n = cv.nvv + cv.nev + cv.nee + cv.nfv;
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    Local c;
    load_contact(cv, E, F, i, c);
    int64_t off;
    if (i < cv.nvv) off = 4 * i;
    else if (i < cv.nvv + cv.nev) off = 4 * cv.nvv + 9 * (i - cv.nvv);
    else off = 4 * cv.nvv + 9 * cv.nev + 16 * (i - cv.nvv - cv.nev);
    for (int a = 0; a < c.n; ++a)
        for (int b = 0; b < c.n; ++b)
            if (in_range(gd, 6, off + a * c.n + b, nk, i)) {
                keys[off + a * c.n + b] = ((unsigned long long)c.vid[a] << 32) | (unsigned)c.vid[b];
                ids[off + a * c.n + b] = (int)(off + a * c.n + b);
            }
}

// Block row pointers of rows r0 .. r0 + nr (local to this chunk's blocks).
__global__ void k_block_rowptr(const unsigned long long* __restrict__ ukeys, const int* __restrict__ d_nb, int r0,
    int nr, int* __restrict__ bptr, long long ucap, Guard gd)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j > nr) return;
    const int nb = *d_nb;
    if (!in_range(gd, 7, nb, ucap + 1, j)) return;
    bptr[j] = lower_bound_u64(ukeys, 0, nb, (unsigned long long)(r0 + j) << 32);
}

// CSR row pointers of the 3 nr scalar rows starting at 3 r0; B0 blocks of
// earlier chunks come first in the value arrays.
__global__ void k_csr_rows(const int* __restrict__ bptr, int r0, int nr, int64_t B0, int64_t* __restrict__ row_ptr)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j > nr) return;
    const int64_t b0 = B0 + bptr[j];
    const int64_t r = r0 + (int64_t)j;
    if (j == nr) {
        row_ptr[3 * r] = 9 * b0;
        return;
    }
    const int64_t nbr = bptr[j + 1] - bptr[j];
    for (int k = 0; k < 3; ++k) row_ptr[3 * r + k] = 9 * b0 + 3 * k * nbr;
}

__global__ void k_csr_cols(const unsigned long long* __restrict__ ukeys, int nb, const int* __restrict__ bptr,
    int r0, int nr, int64_t B0, int* __restrict__ col, Guard gd)
{
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= nb) return;
    const unsigned long long key = ukeys[q];
    const int j = (int)(key >> 32) - r0, cc = (int)(key & 0xffffffffu);
    if (!in_range(gd, 8, j, nr, q)) return;
    const int b0 = bptr[j];
    const int64_t nbr = bptr[j + 1] - b0;
    const int64_t base = 9 * (int64_t)b0 + 3 * (int64_t)(q - b0);
    for (int k = 0; k < 3; ++k)
        for (int l = 0; l < 3; ++l)
            if (in_range(gd, 9, base + 3 * k * nbr + l, 9LL * nb, q)) col[9 * B0 + base + 3 * k * nbr + l] = 3 * cc + l;
}

// Contact range of every scene boundary in each type list: lists are sorted
// by their first index (vertex, edge, edge, face) and edges and faces are
// numbered scene by scene, so scene k's contacts of a type are contiguous.
__global__ void k_scene_ranges(ContactsView cv, const int64_t* __restrict__ offs, int S, int64_t* __restrict__ out)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= 4 * S) return;
    const int type = t / S;
    const int2* list = type == 0 ? cv.vv : (type == 1 ? cv.ev : (type == 2 ? cv.ee : cv.fv));
    const int64_t n = type == 0 ? cv.nvv : (type == 1 ? cv.nev : (type == 2 ? cv.nee : cv.nfv));
    const int64_t key = offs[t];
    int64_t lo = 0, hi = n;
    while (lo < hi) {
        const int64_t mid = (lo + hi) >> 1;
        if (list[mid].x < key) lo = mid + 1;
        else hi = mid;
    }
    out[t] = lo;
}

// A run of consecutive scenes whose Hessian is assembled together: contacts
// [lo[t], hi[t]) of each type t touch only rows of vertices [r0, r1).
struct Chunk {
    int64_t lo[4], hi[4];
    int64_t r0, r1;
    int64_t size() const { return (hi[0] - lo[0]) + (hi[1] - lo[1]) + (hi[2] - lo[2]) + (hi[3] - lo[3]); }
};

} // namespace

// Contacts per Hessian chunk of a batch: bounds the 1152-byte-per-contact
// local-Hessian scratch (4.8 GB at the default 2^22) however large the batch.
std::atomic<int64_t> g_hess_chunk_contacts { int64_t(1) << 22 };

namespace {

ContactsView sub_view(const ContactsView& cv, const Chunk& c)
{
    ContactsView v = cv;
    v.nvv = c.hi[0] - c.lo[0];
    v.nev = c.hi[1] - c.lo[1];
    v.nee = c.hi[2] - c.lo[2];
    v.nfv = c.hi[3] - c.lo[3];
    v.vv = cv.vv + c.lo[0];
    v.vv_w = cv.vv_w + c.lo[0];
    v.ev = cv.ev + c.lo[1];
    v.ev_w = cv.ev_w + c.lo[1];
    v.ee = cv.ee + c.lo[2];
    v.ee_w = cv.ee_w + c.lo[2];
    v.ee_eps = cv.ee_eps + c.lo[2];
    v.ee_dt = cv.ee_dt + c.lo[2];
    v.fv = cv.fv + c.lo[3];
    v.fv_w = cv.fv_w + c.lo[3];
    return v;
}

// One chunk per run of scenes holding at most g_hess_chunk_contacts contacts (a
// single chunk for one scene, a small batch, or a set loaded from outside).
std::vector<Chunk> plan_chunks(const ipcg_collisions* cs, ipcg_mesh* m, const ContactsView& cv)
{
    const int64_t n = cs->size();
    Chunk all { { 0, 0, 0, 0 }, { cs->nvv, cs->nev, cs->nee, cs->nfv }, 0, m->nV };
    const int64_t ns = m->n_scenes;
    const int64_t budget = g_hess_chunk_contacts.load();
    if (ns <= 1 || !cs->sorted || n <= budget) return { all };
    const int S = (int)(ns + 1);
    cudaStream_t s = m->stream;
    DBuf<int64_t> d_out;
    d_out.reserve(4 * S);
    IPCG_LAUNCH("k_scene_ranges", s, k_scene_ranges<<<grid_for(4 * S, 256), 256, 0, s>>>(cv, m->scene_offs.p, S,
        d_out.p));
    std::vector<int64_t> h(4 * S);
    IPCG_CUDA(cudaMemcpyAsync(h.data(), d_out.p, sizeof(int64_t) * 4 * S, cudaMemcpyDeviceToHost, s));
    IPCG_CUDA(cudaStreamSynchronize(s));
    std::vector<Chunk> out;
    int64_t k0 = 0;
    while (k0 < ns) {
        int64_t k1 = k0 + 1;
        auto count = [&](int64_t a, int64_t b) {
            int64_t c = 0;
            for (int t = 0; t < 4; ++t) c += h[t * S + b] - h[t * S + a];
            return c;
        };
        while (k1 < ns && count(k0, k1 + 1) <= budget) ++k1;
        Chunk c;
        for (int t = 0; t < 4; ++t) {
            c.lo[t] = h[t * S + k0];
            c.hi[t] = h[t * S + k1];
        }
        c.r0 = m->h_voff[k0];
        c.r1 = m->h_voff[k1];
        out.push_back(c);
        k0 = k1;
    }
    return out;
}

// Smallest squared distance over the collision set
// (normal_collisions.cpp:209-233: "actually distance squared"), each contact
// measured with its own distance (the one its energy uses).  Squared
// distances are non-negative, so their bit patterns order like the values.
__global__ void __launch_bounds__(BLOCK) k_min_distance(ContactsView cv, const int* __restrict__ E,
    const int* __restrict__ F, const double* __restrict__ V, unsigned long long* __restrict__ out)
{
    const int64_t n = cv.nvv + cv.nev + cv.nee + cv.nfv;
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    double d = __longlong_as_double(0x7ff0000000000000ULL);
    if (i < n) {
        Local c;
        load_contact(cv, E, F, i, c);
        V3 x[4];
        gather(V, c, x);
        double g[12];
        d = fmax(contact_distance(c, x, g, nullptr), 0.0);
    }
    typedef cub::BlockReduce<double, BLOCK> BR;
    __shared__ typename BR::TempStorage tmp;
    const double mn = BR(tmp).Reduce(d, [](double a, double b) { return fmin(a, b); });
    if (threadIdx.x == 0) atomicMin(out, (unsigned long long)__double_as_longlong(mn));
}

} // namespace

// Per-scene barrier parameters (barrier_potential.cpp:62-99) on the device,
// uploaded only when they change (a Newton loop repeats them); P0 = scene 0's.
static const Params* upload_params(const ipcg_collisions* cs, ipcg_mesh* m, const BarrierArgs& a, Params& P0)
{
    const int ns = (int)m->n_scenes;
    std::vector<Params> hp(ns);
    for (int k = 0; k < ns; ++k) {
        const double dh = a.scene_dhat ? a.scene_dhat[k] : a.dhat;
        const double kap = a.scene_kappa ? a.scene_kappa[k] : a.kappa;
        const double dm = (k < (int)cs->scene_dmin.size()) ? cs->scene_dmin[k] : cs->dmin;
        const double xh = (2 * dm + dh) * dh;
        hp[k] = Params { kap, dm * dm, xh, a.physical ? dh / barrier_units(a.kind, xh) : 1.0, a.psd, a.mixed, a.kind };
    }
    const size_t pbytes = sizeof(Params) * ns;
    const unsigned char* hb = reinterpret_cast<const unsigned char*>(hp.data());
    if (m->params_host.size() != pbytes || memcmp(m->params_host.data(), hb, pbytes) != 0) {
        m->params_buf.reserve(pbytes);
        IPCG_CUDA(cudaMemcpyAsync(m->params_buf.p, hb, pbytes, cudaMemcpyHostToDevice, m->stream));
        m->params_host.assign(hb, hb + pbytes);
    }
    P0 = hp[0];
    return reinterpret_cast<const Params*>(m->params_buf.p);
}

// With fr set, the same pipeline evaluates the friction potential of the
// tangential set whose stencils are cs at velocities V (single scene).
void barrier_evaluate(const ipcg_collisions* cs, ipcg_mesh* m, const double* V, const BarrierArgs& a,
    double* energy_host, double* grad_dev, ipcg_csr* hess, const FrictionView* fr)
{
    cudaStream_t s = m->stream;
    ContactsView cv { cs->nvv, cs->nev, cs->nee, cs->nfv, cs->vv.p, cs->ev.p, cs->ee.p, cs->fv.p, cs->vv_w.p,
        cs->ev_w.p, cs->ee_w.p, cs->fv_w.p, cs->ee_eps.p, cs->ee_dtype.p };
    const int64_t n = cs->size();
    const int ns = (int)m->n_scenes;
    Params P {};
    const Params* sp = fr ? nullptr : upload_params(cs, m, a, P);
    const SceneView sv = scene_view(m);
    const int nblk = grid_for(n, BLOCK);
    const int64_t nV = m->nV;
    if (energy_host && ns > 1) {
        // per-scene energies (batches)
        m->partial.reserve(ns + 2);
        IPCG_CUDA(cudaMemsetAsync(m->partial.p, 0, sizeof(double) * ns, s));
        if (n > 0 && fr)
            IPCG_LAUNCH("k_friction_energy_scenes", s, k_friction_energy_scenes<<<nblk, BLOCK, 0, s>>>(cv, m->E.p,
                m->F.p, V, *fr, sv, m->partial.p));
        else if (n > 0)
            IPCG_LAUNCH("k_energy_scenes", s, k_energy_scenes<<<nblk, BLOCK, 0, s>>>(cv, m->E.p, m->F.p, V, sp, sv,
                m->partial.p));
        IPCG_CUDA(cudaMemcpyAsync(energy_host, m->partial.p, sizeof(double) * ns, cudaMemcpyDefault, s));
    } else if (energy_host) {
        m->partial.reserve(nblk + 2);
        if (n > 0) {
            if (fr)
                IPCG_LAUNCH("k_friction_energy", s, k_friction_energy<<<nblk, BLOCK, 0, s>>>(cv, m->E.p, m->F.p, V,
                    *fr, m->partial.p));
            else
                IPCG_LAUNCH("k_energy", s, k_energy<<<nblk, BLOCK, 0, s>>>(cv, m->E.p, m->F.p, V, P, m->partial.p));
            IPCG_LAUNCH("k_sum_partials", s, k_sum_partials<<<1, 1024, 0, s>>>(m->partial.p, nblk, m->partial.p + nblk));
            IPCG_CHECK_LAUNCH();
            IPCG_CUDA(cudaMemcpyAsync(energy_host, m->partial.p + nblk, sizeof(double), cudaMemcpyDeviceToHost, s));
        } else {
            *energy_host = 0;
        }
    }
    if (grad_dev) {
        IPCG_CUDA(cudaMemsetAsync(grad_dev, 0, sizeof(double) * 3 * nV, s));
        if (n > 0) {
            if (fr)
                IPCG_LAUNCH("k_friction_gradient", s, k_friction_gradient<<<nblk, BLOCK, 0, s>>>(cv, m->E.p, m->F.p,
                    V, *fr, grad_dev));
            else
                IPCG_LAUNCH("k_gradient", s, k_gradient<<<nblk, BLOCK, 0, s>>>(cv, m->E.p, m->F.p, V, sp, sv,
                    grad_dev));
            IPCG_CHECK_LAUNCH();
        }
    }
    if (hess) {
        hess->rows = 3 * nV;
        hess->stream = s;
        const std::vector<Chunk> chunks = plan_chunks(cs, m, cv);
        int64_t max_n = 0, max_nk = 0, max_nr = 0;
        for (const Chunk& c : chunks) {
            const int64_t nk = 4 * (c.hi[0] - c.lo[0]) + 9 * (c.hi[1] - c.lo[1])
                + 16 * ((c.hi[2] - c.lo[2]) + (c.hi[3] - c.lo[3]));
            max_n = std::max(max_n, c.size());
            max_nk = std::max(max_nk, nk);
            max_nr = std::max(max_nr, c.r1 - c.r0);
        }
        if (max_nk >= INT32_MAX) throw Error(IPCG_ERR_INVALID, "too many Hessian contributions in one scene");
        m->keys_a.reserve(max_nk + 1);
        m->keys_b.reserve(max_nk + 1);
        m->ivals_a.reserve(max_nk + max_nr + 3);
        m->ivals_b.reserve(3 * max_nk + 3);
        m->hs.reserve(144 * (max_n + 1));
        const Slab slab { m->hs.p, max_n + 1 };
        m->proj.reserve(max_n + 1);
        m->counters.reserve(16);
        int* d_nb = m->counters.p + 14;
        int* d_fail = m->counters.p + 15;
        IPCG_CUDA(cudaMemsetAsync(d_fail, 0, sizeof(int), s));
        m->guard.reserve(4);
        IPCG_CUDA(cudaMemsetAsync(m->guard.p, 0, sizeof(long long) * 4, s));
        const Guard gd { m->guard.p };
        hess->row_ptr.reserve(3 * nV + 1, s);
        int64_t B0 = 0, done = 0;
        for (const Chunk& ch : chunks) {
            const ContactsView cc = sub_view(cv, ch);
            const int64_t nc = ch.size();
            const int64_t nk = 4 * cc.nvv + 9 * cc.nev + 16 * (cc.nee + cc.nfv);
            const int r0 = (int)ch.r0, nr = (int)(ch.r1 - ch.r0);
            const int nblk_c = grid_for(nc, BLOCK);
            int* ids_in = m->ivals_b.p;                  // contribution ids (unsorted)
            int* contrib = m->ivals_b.p + (nk + 1);      // contribution ids sorted by block key
            int* run_len = m->ivals_b.p + 2 * (nk + 1);  // contributions per block
            int* bptr = m->ivals_a.p;                    // block row pointers of this chunk's rows
            int* run_start = m->ivals_a.p + (nr + 2);    // first contribution of each block
            int nb = 0;
            // Three streams, forked after everything queued so far on the main
            // one.  The side stream computes the VV, EV and FV local Hessians
            // while the main one computes the EE ones (each launch fills only
            // a few warps per SM, so side by side they keep the FP64 pipes
            // busier than in turn); the main stream then projects them all.
            // The pattern stream builds the sparsity pattern (block keys, sort,
            // run-length encoding, row and column arrays), which does not
            // depend on the values, beside both.
            cudaStream_t t = m->side, u = m->side2;
            IPCG_CUDA(cudaEventRecord(m->ev_fork, s));
            IPCG_CUDA(cudaStreamWaitEvent(t, m->ev_fork, 0));
            IPCG_CUDA(cudaStreamWaitEvent(u, m->ev_fork, 0));
            if (nc > 0) {
                const int64_t first[4] = { 0, cc.nvv, cc.nvv + cc.nev, cc.nvv + cc.nev + cc.nee };
                const int64_t count[4] = { cc.nvv, cc.nev, cc.nee, cc.nfv };
                if (fr) {
                    // friction: local Hessians are projected in place (2x2 inner matrix)
                    const FrictionView f = *fr;
                    if (count[0])
                        IPCG_LAUNCH("k_friction_local_hessian_vv", t, k_friction_local_hessian<CT_VV><<<grid_for(count[0],
                            LH_BLOCK), LH_BLOCK, 0, t>>>(cc, m->E.p, m->F.p, V, f, slab, first[0], count[0], a.psd));
                    if (count[1])
                        IPCG_LAUNCH("k_friction_local_hessian_ev", t, k_friction_local_hessian<CT_EV><<<grid_for(count[1],
                            LH_BLOCK), LH_BLOCK, 0, t>>>(cc, m->E.p, m->F.p, V, f, slab, first[1], count[1], a.psd));
                    if (count[3])
                        IPCG_LAUNCH("k_friction_local_hessian_fv", t, k_friction_local_hessian<CT_FV><<<grid_for(count[3],
                            LH_BLOCK), LH_BLOCK, 0, t>>>(cc, m->E.p, m->F.p, V, f, slab, first[3], count[3], a.psd));
                    IPCG_CUDA(cudaEventRecord(m->ev_side, t));
                    if (count[2])
                        IPCG_LAUNCH("k_friction_local_hessian_ee", s, k_friction_local_hessian<CT_EE><<<grid_for(count[2],
                            LH_BLOCK), LH_BLOCK, 0, s>>>(cc, m->E.p, m->F.p, V, f, slab, first[2], count[2], a.psd));
                } else {
                    if (count[0])
                        IPCG_LAUNCH("k_local_hessian_vv", t, k_local_hessian<CT_VV><<<grid_for(count[0], LH_BLOCK),
                            LH_BLOCK, 0, t>>>(cc, m->E.p, m->F.p, V, sp, sv, slab, m->proj.p, first[0], count[0]));
                    if (count[1])
                        IPCG_LAUNCH("k_local_hessian_ev", t, k_local_hessian<CT_EV><<<grid_for(count[1], LH_BLOCK),
                            LH_BLOCK, 0, t>>>(cc, m->E.p, m->F.p, V, sp, sv, slab, m->proj.p, first[1], count[1]));
                    if (count[3])
                        IPCG_LAUNCH("k_local_hessian_fv", t, k_local_hessian<CT_FV><<<grid_for(count[3], LH_BLOCK),
                            LH_BLOCK, 0, t>>>(cc, m->E.p, m->F.p, V, sp, sv, slab, m->proj.p, first[3], count[3]));
                    IPCG_CUDA(cudaEventRecord(m->ev_side, t));
                    if (count[2] && a.shape)
                        IPCG_LAUNCH("k_shape_local_ee", s, k_shape_local_ee<<<grid_for(count[2], LH_BLOCK), LH_BLOCK,
                            0, s>>>(cc, m->E.p, m->F.p, V, m->rest.p, sp, sv, slab, first[2], count[2]));
                    else if (count[2])
                        IPCG_LAUNCH("k_local_hessian_ee", s, k_local_hessian<CT_EE><<<grid_for(count[2], LH_BLOCK),
                            LH_BLOCK, 0, s>>>(cc, m->E.p, m->F.p, V, sp, sv, slab, m->proj.p, first[2], count[2]));
                    IPCG_CUDA(cudaStreamWaitEvent(s, m->ev_side, 0));
                    if (a.psd != IPCG_PSD_NONE)
                        IPCG_LAUNCH("k_psd", s, k_psd<<<grid_for(nc, PSD_BLOCK), PSD_BLOCK, 0, s>>>(cc, slab,
                            m->proj.p, a.psd, d_fail, 0, nc));
                }
                IPCG_CUDA(cudaStreamWaitEvent(s, m->ev_side, 0));
                // sparsity pattern: sort (block key, contribution) and run-length encode
                IPCG_LAUNCH("k_block_keys", u, k_block_keys<<<nblk_c, BLOCK, 0, u>>>(cc, m->E.p, m->F.p,
                    m->keys_a.p, ids_in, nk, gd));
                sort_pairs_u64(m, u, m->keys_a.p, m->keys_b.p, ids_in, contrib, (int)nk, 32 + bits_for(nV + 1));
                rle_u64(m, u, m->keys_b.p, m->keys_a.p, run_len, d_nb, (int)nk);
                IPCG_CUDA(cudaMemcpyAsync(m->h_counters.p, d_nb, sizeof(int), cudaMemcpyDeviceToHost, u));
                IPCG_CUDA(cudaStreamSynchronize(u)); // the other streams keep running
                nb = m->h_counters.p[0];
                exclusive_sum_i32(m, u, run_len, run_start, nb);
            } else {
                IPCG_CUDA(cudaMemsetAsync(d_nb, 0, sizeof(int), u));
            }
            // output arrays grow as chunks finish (the last chunk's estimate is exact)
            done += nc;
            const int64_t need = 9 * (B0 + nb);
            const int64_t guess = done < n ? (int64_t)((double)need * (double)n / (double)std::max<int64_t>(done, 1))
                                           : need;
            hess->col.grow_keep(std::max(need, guess) + 1, 9 * B0, u);
            hess->val.grow_keep(std::max(need, guess) + 1, 9 * B0, u);
            IPCG_LAUNCH("k_block_rowptr", u, k_block_rowptr<<<grid_for(nr + 1, 256), 256, 0, u>>>(m->keys_a.p, d_nb,
                r0, nr, bptr, nk, gd));
            IPCG_LAUNCH("k_csr_rows", u, k_csr_rows<<<grid_for(nr + 1, 256), 256, 0, u>>>(bptr, r0, nr, B0,
                hess->row_ptr.p));
            if (nb > 0)
                IPCG_LAUNCH("k_csr_cols", u, k_csr_cols<<<grid_for(nb, 256), 256, 0, u>>>(m->keys_a.p, nb, bptr, r0,
                    nr, B0, hess->col.p, gd));
            // join: values need the projected local Hessians and the pattern
            IPCG_CUDA(cudaEventRecord(m->ev_pattern, u));
            IPCG_CUDA(cudaStreamWaitEvent(s, m->ev_pattern, 0));
            if (nb > 0)
                IPCG_LAUNCH("k_assemble", s, k_assemble<<<grid_for(9 * (int64_t)nb, 256), 256, 0, s>>>(cc,
                    m->keys_a.p, run_start, run_len, contrib, slab, bptr, r0, B0, nb, hess->val.p));
            B0 += nb;
        }
        hess->nnz = 9 * B0;
        IPCG_CUDA(cudaMemcpyAsync(m->h_counters.p + 1, d_fail, sizeof(int), cudaMemcpyDeviceToHost, s));
        IPCG_CUDA(cudaMemcpyAsync(m->h_guard, m->guard.p, sizeof(long long) * 4, cudaMemcpyDeviceToHost, s));
    }
    IPCG_CUDA(cudaStreamSynchronize(s));
    if (hess && m->h_guard[0]) {
        char msg[256];
        snprintf(msg, sizeof(msg), "Hessian assembly index check %lld failed: index %lld, limit %lld, item %lld",
            m->h_guard[0], m->h_guard[1], m->h_guard[2], m->h_guard[3]);
        throw Error(IPCG_ERR_CUDA, msg);
    }
    if (hess && (m->h_counters.p[1] & 1))
        throw Error(IPCG_ERR_CUDA, "unable to project matrix onto positive semi-definite cone");
}

double barrier_derivative_host(int kind, int order, double x, double xhat)
{
    return order == 0 ? barrier_fn<0, double>(kind, x, xhat)
                      : (order == 1 ? barrier_fn<1, double>(kind, x, xhat) : barrier_fn<2, double>(kind, x, xhat));
}

namespace {
// a . b and b . b over n entries: per-block partial sums, then one thread
// adds them in a fixed order (deterministic)
__global__ void __launch_bounds__(BLOCK) k_dots(const double* __restrict__ a, const double* __restrict__ b, int64_t n,
    double* __restrict__ partial)
{
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    double ab = 0, bb = 0;
    for (int64_t j = i; j < n; j += (int64_t)gridDim.x * blockDim.x) {
        ab += a[j] * b[j];
        bb += b[j] * b[j];
    }
    typedef cub::BlockReduce<double, BLOCK> BR;
    __shared__ typename BR::TempStorage tmp;
    const double s1 = BR(tmp).Sum(ab);
    __syncthreads();
    const double s2 = BR(tmp).Sum(bb);
    if (threadIdx.x == 0) {
        partial[2 * blockIdx.x] = s1;
        partial[2 * blockIdx.x + 1] = s2;
    }
}
__global__ void k_dots_final(const double* __restrict__ partial, int nb, double* __restrict__ out)
{
    if (threadIdx.x != 0) return;
    double s1 = 0, s2 = 0;
    for (int i = 0; i < nb; ++i) {
        s1 += partial[2 * i];
        s2 += partial[2 * i + 1];
    }
    out[0] = s1;
    out[1] = s2;
}
} // namespace

void dot_pair_device(const double* a, const double* b, int64_t n, double* ab, double* bb)
{
    const int nb = (int)std::min<int64_t>(1024, std::max<int64_t>(1, grid_for(n, BLOCK)));
    DBuf<double> part;
    part.reserve(2 * nb + 2);
    cudaStream_t s = 0;
    IPCG_LAUNCH("k_dots", s, k_dots<<<nb, BLOCK, 0, s>>>(a, b, n, part.p));
    IPCG_LAUNCH("k_dots_final", s, k_dots_final<<<1, 32, 0, s>>>(part.p, nb, part.p + 2 * nb));
    double h[2];
    IPCG_CUDA(cudaMemcpyAsync(h, part.p + 2 * nb, sizeof(h), cudaMemcpyDeviceToHost, s));
    IPCG_CUDA(cudaStreamSynchronize(s));
    *ab = h[0];
    *bb = h[1];
}

double collisions_min_distance(const ipcg_collisions* cs, ipcg_mesh* m, const double* V)
{
    const int64_t n = cs->size();
    if (n == 0) return __builtin_inf();
    cudaStream_t s = m->stream;
    ContactsView cv { cs->nvv, cs->nev, cs->nee, cs->nfv, cs->vv.p, cs->ev.p, cs->ee.p, cs->fv.p, cs->vv_w.p,
        cs->ev_w.p, cs->ee_w.p, cs->fv_w.p, cs->ee_eps.p, cs->ee_dtype.p };
    m->toi_bits.reserve(1);
    const unsigned long long inf = 0x7ff0000000000000ULL;
    IPCG_CUDA(cudaMemcpyAsync(m->toi_bits.p, &inf, sizeof(inf), cudaMemcpyHostToDevice, s));
    IPCG_LAUNCH("k_min_distance", s, k_min_distance<<<grid_for(n, BLOCK), BLOCK, 0, s>>>(cv, m->E.p, m->F.p, V,
        m->toi_bits.p));
    unsigned long long bits = 0;
    IPCG_CUDA(cudaMemcpyAsync(&bits, m->toi_bits.p, sizeof(bits), cudaMemcpyDeviceToHost, s));
    IPCG_CUDA(cudaStreamSynchronize(s));
    double d;
    memcpy(&d, &bits, sizeof(d));
    return d;
}

void barrier_gauss_newton(const ipcg_collisions* cs, ipcg_mesh* m, const double* V, const BarrierArgs& a,
    double* diag_dev, const double* p_dev, double* qf_host)
{
    cudaStream_t s = m->stream;
    ContactsView cv { cs->nvv, cs->nev, cs->nee, cs->nfv, cs->vv.p, cs->ev.p, cs->ee.p, cs->fv.p, cs->vv_w.p,
        cs->ev_w.p, cs->ee_w.p, cs->fv_w.p, cs->ee_eps.p, cs->ee_dtype.p };
    const int64_t n = cs->size();
    Params P;
    const Params* sp = upload_params(cs, m, a, P);
    const SceneView sv = scene_view(m);
    const int nblk = grid_for(n, BLOCK);
    if (diag_dev) {
        IPCG_CUDA(cudaMemsetAsync(diag_dev, 0, sizeof(double) * 3 * m->nV, s));
        if (n > 0)
            IPCG_LAUNCH("k_gn_diagonal", s, k_gn_diagonal<<<nblk, BLOCK, 0, s>>>(cv, m->E.p, m->F.p, V, sp, sv,
                diag_dev));
    }
    if (qf_host) {
        if (n == 0) {
            *qf_host = 0;
            return;
        }
        m->partial.reserve(nblk + 2);
        IPCG_LAUNCH("k_gn_quadratic_form", s, k_gn_quadratic_form<<<nblk, BLOCK, 0, s>>>(cv, m->E.p, m->F.p, V,
            p_dev, sp, sv, m->partial.p));
        IPCG_LAUNCH("k_sum_partials", s, k_sum_partials<<<1, 1024, 0, s>>>(m->partial.p, nblk, m->partial.p + nblk));
        IPCG_CUDA(cudaMemcpyAsync(qf_host, m->partial.p + nblk, sizeof(double), cudaMemcpyDeviceToHost, s));
        IPCG_CUDA(cudaStreamSynchronize(s));
    }
}

void shape_derivative_area(const ipcg_collisions* cs, ipcg_mesh* m, const double* V, const BarrierArgs& a,
    ipcg_csr* out)
{
    cudaStream_t s = m->stream;
    ensure_adjacency(m);
    ContactsView cv { cs->nvv, cs->nev, cs->nee, cs->nfv, cs->vv.p, cs->ev.p, cs->ee.p, cs->fv.p, cs->vv_w.p,
        cs->ev_w.p, cs->ee_w.p, cs->fv_w.p, cs->ee_eps.p, cs->ee_dtype.p };
    const int64_t n = cs->size();
    const int64_t ndof = 3 * m->nV;
    Params P0;
    const Params* sp = upload_params(cs, m, a, P0);
    const SceneView sv = scene_view(m);
    out->rows = ndof;
    out->stream = s;
    out->row_ptr.reserve(ndof + 1, s);
    if (n == 0) {
        IPCG_CUDA(cudaMemsetAsync(out->row_ptr.p, 0, sizeof(int64_t) * (ndof + 1), s));
        out->nnz = 0;
        IPCG_CUDA(cudaStreamSynchronize(s));
        return;
    }
    // second-term local matrices
    m->hs.reserve(144 * (n + 1));
    const Slab slab { m->hs.p, n + 1 };
    m->proj.reserve(n + 1);
    const int64_t first[4] = { 0, cs->nvv, cs->nvv + cs->nev, cs->nvv + cs->nev + cs->nee };
    const int64_t count[4] = { cs->nvv, cs->nev, cs->nee, cs->nfv };
    if (count[0])
        IPCG_LAUNCH("k_local_hessian_vv", s, k_local_hessian<CT_VV><<<grid_for(count[0], LH_BLOCK), LH_BLOCK, 0, s>>>(
            cv, m->E.p, m->F.p, V, sp, sv, slab, m->proj.p, first[0], count[0]));
    if (count[1])
        IPCG_LAUNCH("k_local_hessian_ev", s, k_local_hessian<CT_EV><<<grid_for(count[1], LH_BLOCK), LH_BLOCK, 0, s>>>(
            cv, m->E.p, m->F.p, V, sp, sv, slab, m->proj.p, first[1], count[1]));
    if (count[2])
        IPCG_LAUNCH("k_shape_local_ee", s, k_shape_local_ee<<<grid_for(count[2], LH_BLOCK), LH_BLOCK, 0, s>>>(cv,
            m->E.p, m->F.p, V, m->rest.p, sp, sv, slab, first[2], count[2]));
    if (count[3])
        IPCG_LAUNCH("k_local_hessian_fv", s, k_local_hessian<CT_FV><<<grid_for(count[3], LH_BLOCK), LH_BLOCK, 0, s>>>(
            cv, m->E.p, m->F.p, V, sp, sv, slab, m->proj.p, first[3], count[3]));
    const ShapeSources S { cs->vv_src_off.p, cs->ev_src_off.p, cs->vv_src.p, cs->ev_src.p, m->vf_off.p, m->vf_adj.p,
        m->ef_off.p, m->ef_adj.p, m->ve_off.p, m->ve_adj.p };
    // triplet counts and offsets
    PBuf<int64_t> cnt, offs;
    cnt.reserve(n + 1, s);
    offs.reserve(n + 1, s);
    IPCG_CUDA(cudaMemsetAsync(cnt.p + n, 0, sizeof(int64_t), s));
    IPCG_LAUNCH("k_shape_count", s, k_shape_count<<<grid_for(n, BLOCK), BLOCK, 0, s>>>(cv, m->E.p, m->F.p, S,
        cnt.p));
    exclusive_sum_i64(m, s, cnt.p, offs.p, (int)(n + 1));
    int64_t T = 0;
    IPCG_CUDA(cudaMemcpyAsync(&T, offs.p + n, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
    IPCG_CUDA(cudaStreamSynchronize(s));
    if (T >= INT32_MAX) throw Error(IPCG_ERR_INVALID, "shape derivative too large (2^31 triplets)");
    const int Ti = (int)T;
    PBuf<unsigned long long> keys, skeys, uniq;
    PBuf<double> vals, svals;
    PBuf<int> idx, sidx, rcnt, roff;
    keys.reserve(T + 1, s);
    skeys.reserve(T + 1, s);
    uniq.reserve(T + 1, s);
    vals.reserve(T + 1, s);
    svals.reserve(T + 1, s);
    idx.reserve(T + 1, s);
    sidx.reserve(T + 1, s);
    rcnt.reserve(T + 2, s);
    roff.reserve(T + 2, s);
    IPCG_LAUNCH("k_shape_emit", s, k_shape_emit<<<grid_for(n, BLOCK), BLOCK, 0, s>>>(cv, m->E.p, m->F.p, V,
        m->rest.p, sp, sv, slab, S, offs.p, ndof, keys.p, vals.p));
    IPCG_LAUNCH("k_iota", s, k_iota<<<grid_for(T, BLOCK), BLOCK, 0, s>>>(idx.p, Ti));
    const int kbits = std::min(64, bits_for(ndof) * 2 + 1);
    sort_pairs_u64(m, s, keys.p, skeys.p, idx.p, sidx.p, Ti, kbits);
    IPCG_LAUNCH("k_gather_vals", s, k_gather_vals<<<grid_for(T, BLOCK), BLOCK, 0, s>>>(vals.p, sidx.p, Ti, svals.p));
    m->counters.reserve(32);
    int* d_num = m->counters.p + 28;
    IPCG_CUDA(cudaMemsetAsync(rcnt.p, 0, sizeof(int) * (T + 1), s));
    rle_u64(m, s, skeys.p, uniq.p, rcnt.p, d_num, Ti);
    exclusive_sum_i32(m, s, rcnt.p, roff.p, Ti + 1);
    int nnz = 0;
    IPCG_CUDA(cudaMemcpyAsync(&nnz, d_num, sizeof(int), cudaMemcpyDeviceToHost, s));
    IPCG_CUDA(cudaStreamSynchronize(s));
    out->col.reserve(nnz + 1, s);
    out->val.reserve(nnz + 1, s);
    out->nnz = nnz;
    if (nnz)
        IPCG_LAUNCH("k_sum_key_runs", s, k_sum_key_runs<<<grid_for(nnz, BLOCK), BLOCK, 0, s>>>(uniq.p, rcnt.p, roff.p,
            d_num, svals.p, ndof, out->col.p, out->val.p));
    IPCG_LAUNCH("k_rows_from_keys", s, k_rows_from_keys<<<grid_for(ndof + 1, BLOCK), BLOCK, 0, s>>>(uniq.p, d_num,
        ndof, out->row_ptr.p));
    IPCG_CUDA(cudaStreamSynchronize(s));
}

void barrier_evaluate_friction(const ipcg_collisions* stencils, ipcg_mesh* m, const double* U, const FrictionView& f,
    int psd, double* energy_host, double* grad_dev, ipcg_csr* hess)
{
    BarrierArgs a { 1.0, 1.0, 0.0, 0, psd };
    barrier_evaluate(stencils, m, U, a, energy_host, grad_dev, hess, &f);
}

void tangential_build(const ipcg_collisions* cs, ipcg_mesh* m, const double* V, const BarrierArgs& a,
    const double* mu_s, const double* mu_k, ipcg_tangential* t)
{
    ipcg_collisions* st = &t->st;
    DBuf<double>&N = t->N, &cp = t->cp, &P = t->P, &ms = t->mu_s, &mk = t->mu_k;
    cudaStream_t s = m->stream;
    ContactsView cv { cs->nvv, cs->nev, cs->nee, cs->nfv, cs->vv.p, cs->ev.p, cs->ee.p, cs->fv.p, cs->vv_w.p,
        cs->ev_w.p, cs->ee_w.p, cs->fv_w.p, cs->ee_eps.p, cs->ee_dtype.p };
    Params P0;
    const Params* sp = upload_params(cs, m, a, P0);
    // EE collisions kept: flags, then their compacted slots
    m->widx.reserve(2 * (cs->nee + 1));
    int* keep = m->widx.p;
    int* offs = m->widx.p + cs->nee + 1;
    int64_t nee_kept = 0;
    if (cs->nee) {
        IPCG_LAUNCH("k_tangential_keep_ee", s, k_tangential_keep_ee<<<grid_for(cs->nee, BLOCK), BLOCK, 0, s>>>(cv,
            m->E.p, V, keep));
        exclusive_sum_i32(m, s, keep, offs, (int)cs->nee);
        int tail[2];
        IPCG_CUDA(cudaMemcpyAsync(&tail[0], keep + cs->nee - 1, sizeof(int), cudaMemcpyDeviceToHost, s));
        IPCG_CUDA(cudaMemcpyAsync(&tail[1], offs + cs->nee - 1, sizeof(int), cudaMemcpyDeviceToHost, s));
        IPCG_CUDA(cudaStreamSynchronize(s));
        nee_kept = tail[0] + tail[1];
    }
    st->nvv = cs->nvv;
    st->nev = cs->nev;
    st->nee = nee_kept;
    st->nfv = cs->nfv;
    st->dmin = cs->dmin;
    st->scene_dmin = cs->scene_dmin;
    st->sorted = cs->sorted;
    st->vv.reserve(st->nvv + 1);
    st->ev.reserve(st->nev + 1);
    st->ee.reserve(st->nee + 1);
    st->fv.reserve(st->nfv + 1);
    st->vv_w.reserve(st->nvv + 1);
    st->ev_w.reserve(st->nev + 1);
    st->ee_w.reserve(st->nee + 1);
    st->fv_w.reserve(st->nfv + 1);
    st->ee_eps.reserve(st->nee + 1);
    st->ee_dtype.reserve(st->nee + 1);
    const int64_t nt = st->size();
    N.reserve(nt + 1);
    cp.reserve(2 * nt + 2);
    P.reserve(6 * nt + 6);
    ms.reserve(nt + 1);
    mk.reserve(nt + 1);
    const TangentialOut o { st->vv.p, st->ev.p, st->ee.p, st->fv.p, st->vv_w.p, st->ev_w.p, st->ee_w.p, st->fv_w.p,
        st->ee_eps.p, st->ee_dtype.p, N.p, cp.p, P.p, ms.p, mk.p };
    const int64_t n = cs->size();
    if (n)
        IPCG_LAUNCH("k_tangential_build", s, k_tangential_build<<<grid_for(n, BLOCK), BLOCK, 0, s>>>(cv, m->E.p,
            m->F.p, V, sp, scene_view(m), mu_s, mu_k, keep, offs, nee_kept, o));
    // isotropic defaults and reset_lagged_anisotropic_friction_coefficients
    t->mu_aniso.reserve(2 * nt + 2);
    t->mu_s_aniso.reserve(2 * nt + 2);
    t->mu_k_aniso.reserve(2 * nt + 2);
    t->mu_s_eff.reserve(nt + 1);
    t->mu_k_eff.reserve(nt + 1);
    if (nt) {
        IPCG_LAUNCH("k_fill", s, k_fill<<<grid_for(2 * nt, BLOCK), BLOCK, 0, s>>>(t->mu_aniso.p, 2 * nt, 1.0));
        IPCG_CUDA(cudaMemsetAsync(t->mu_s_aniso.p, 0, sizeof(double) * 2 * nt, s));
        IPCG_CUDA(cudaMemsetAsync(t->mu_k_aniso.p, 0, sizeof(double) * 2 * nt, s));
        IPCG_CUDA(cudaMemcpyAsync(t->mu_s_eff.p, ms.p, sizeof(double) * nt, cudaMemcpyDeviceToDevice, s));
        IPCG_CUDA(cudaMemcpyAsync(t->mu_k_eff.p, mk.p, sizeof(double) * nt, cudaMemcpyDeviceToDevice, s));
    }
    IPCG_CUDA(cudaStreamSynchronize(s));
}

void friction_force(const ipcg_tangential* t, ipcg_mesh* m, const double* rest, const double* lagged,
    const double* vel, const BarrierArgs& a, double eps_v, int no_mu, double* force_dev)
{
    cudaStream_t s = m->stream;
    const ipcg_collisions* st = &t->st;
    ContactsView cv { st->nvv, st->nev, st->nee, st->nfv, st->vv.p, st->ev.p, st->ee.p, st->fv.p, st->vv_w.p,
        st->ev_w.p, st->ee_w.p, st->fv_w.p, st->ee_eps.p, st->ee_dtype.p };
    const double xh = (2 * a.dmin + a.dhat) * a.dhat;
    const Params P { a.kappa, a.dmin * a.dmin, xh, a.physical ? a.dhat / barrier_units(a.kind, xh) : 1.0,
        IPCG_PSD_NONE, 0, a.kind };
    IPCG_CUDA(cudaMemsetAsync(force_dev, 0, sizeof(double) * 3 * m->nV, s));
    const int64_t n = st->size();
    if (n)
        IPCG_LAUNCH("k_friction_force", s, k_friction_force<<<grid_for(n, BLOCK), BLOCK, 0, s>>>(cv, m->E.p, m->F.p,
            rest, lagged, vel, P, t->mu_aniso.p, t->mu_s_eff.p, t->mu_k_eff.p, eps_v, no_mu, force_dev));
}

void tangential_update_lagged(ipcg_tangential* t, ipcg_mesh* m, const double* rest, const double* lagged,
    const double* vel)
{
    cudaStream_t s = m->stream;
    const ipcg_collisions* st = &t->st;
    ContactsView cv { st->nvv, st->nev, st->nee, st->nfv, st->vv.p, st->ev.p, st->ee.p, st->fv.p, st->vv_w.p,
        st->ev_w.p, st->ee_w.p, st->fv_w.p, st->ee_eps.p, st->ee_dtype.p };
    const int64_t n = st->size();
    if (n)
        IPCG_LAUNCH("k_tangential_update_lagged", s, k_tangential_update_lagged<<<grid_for(n, BLOCK), BLOCK, 0, s>>>(
            cv, m->E.p, m->F.p, rest, lagged, vel, t->mu_aniso.p, t->mu_s_aniso.p, t->mu_k_aniso.p, t->mu_s.p,
            t->mu_k.p, t->mu_s_eff.p, t->mu_k_eff.p));
    IPCG_CUDA(cudaStreamSynchronize(s));
}

} // namespace ipcg

// ---------------------------------------------------------------------------
// Allocation-free barrier energy.
//
// Some callers cannot let a library allocate device memory during a call:
// codes that hand all device memory to their own pool or arena under a hard
// budget, and codes that must not pay for cudaMalloc/cudaFree, which can
// synchronise the whole device and stall their other streams.  For them,
// ipcg_barrier_energy_noalloc evaluates the barrier energy of a collision set
// given entirely as caller-owned device arrays.  The only scratch it needs,
// the per-block partial sums of the reduction, lives in the file-scope
// device array below; every GPU that loads this library keeps that array
// (NOALLOC_MAX_BLOCKS + 1 doubles, 128 KiB) until the process exits.
// ---------------------------------------------------------------------------
namespace ipcg {
namespace {
constexpr int NOALLOC_MAX_BLOCKS = 16384; // at most 16384 * BLOCK = 2,097,152 contacts per call
constexpr int NOALLOC_MAX_DEVICES = 64;
std::mutex g_noalloc_mu;
double* g_noalloc_ptr[NOALLOC_MAX_DEVICES] = {};
void* g_noalloc_ctx[NOALLOC_MAX_DEVICES] = {}; // the context each cached address belongs to

// The caller's topology arrays hold indices this library did not check, so
// this path validates every index before it reads through it: a contact with
// an edge, face or vertex index outside [0, num_*) (or an edge-edge distance
// type outside 0..8) reads nothing further and contributes NaN, which makes
// its block's partial sum, and so the returned energy, NaN.
__device__ __forceinline__ bool load_contact_checked(const ContactsView& cv, const int* __restrict__ E,
    const int* __restrict__ F, int64_t nV, int64_t nE, int64_t nF, int64_t i, Local& c)
{
    auto vok = [nV](int v) { return v >= 0 && (int64_t)v < nV; };
    if (i < cv.nvv) {
        const int2 p = cv.vv[i];
        if (!vok(p.x) || !vok(p.y)) return false;
    } else if (i < cv.nvv + cv.nev) {
        const int2 p = cv.ev[i - cv.nvv];
        if (!vok(p.y) || p.x < 0 || (int64_t)p.x >= nE) return false;
        if (!vok(E[2 * p.x]) || !vok(E[2 * p.x + 1])) return false;
    } else if (i < cv.nvv + cv.nev + cv.nee) {
        const int64_t k = i - cv.nvv - cv.nev;
        const int2 p = cv.ee[k];
        if (p.x < 0 || (int64_t)p.x >= nE || p.y < 0 || (int64_t)p.y >= nE) return false;
        if (!vok(E[2 * p.x]) || !vok(E[2 * p.x + 1]) || !vok(E[2 * p.y]) || !vok(E[2 * p.y + 1])) return false;
        const int dt = cv.ee_dt[k];
        if (dt < 0 || dt > 8) return false;
    } else {
        const int2 p = cv.fv[i - cv.nvv - cv.nev - cv.nee];
        if (!vok(p.y) || p.x < 0 || (int64_t)p.x >= nF) return false;
        if (!vok(F[3 * p.x]) || !vok(F[3 * p.x + 1]) || !vok(F[3 * p.x + 2])) return false;
    }
    load_contact(cv, E, F, i, c);
    return true;
}

__global__ void __launch_bounds__(BLOCK) k_energy_checked(ContactsView cv, const int* __restrict__ E,
    const int* __restrict__ F, int64_t nV, int64_t nE, int64_t nF, const double* __restrict__ V, Params P,
    double* __restrict__ partial)
{
    const int64_t n = cv.nvv + cv.nev + cv.nee + cv.nfv;
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    double e = 0;
    if (i < n) {
        Local c;
        if (!load_contact_checked(cv, E, F, nV, nE, nF, i, c)) {
            e = __longlong_as_double(0x7ff8000000000000ULL); // NaN
        } else {
            V3 x[4];
            gather(V, c, x);
            double g[12];
            const double d = contact_distance(c, x, g, nullptr);
            bool act;
            const double m = mollifier(c, x, nullptr, nullptr, act);
            e = c.w * m * fval(P, d);
        }
    }
    typedef cub::BlockReduce<double, BLOCK> BR;
    __shared__ typename BR::TempStorage tmp;
    const double s = BR(tmp).Sum(e);
    if (threadIdx.x == 0) partial[blockIdx.x] = s;
}
} // namespace
} // namespace ipcg

static __device__ __align__(256) double g_noalloc_partials[ipcg::NOALLOC_MAX_BLOCKS + 1];

namespace ipcg {
namespace {
// The current CUDA context (driver handle), read through the runtime's driver
// entry point so that this library does not link the driver library itself.
void* current_context()
{
    typedef int (*CtxGetCurrent)(void**);
    static CtxGetCurrent fn = [] {
        void* f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) != cudaSuccess
            || q != cudaDriverEntryPointSuccess)
            f = nullptr;
        return reinterpret_cast<CtxGetCurrent>(f);
    }();
    void* ctx = nullptr;
    if (fn) fn(&ctx);
    return ctx;
}

// Device address of the partial-sum array on `device` (which must be
// current).  In host code the array's name is only a host-side stand-in, not
// a device address, so the address is looked up with cudaGetSymbolAddress
// once per device and context: the first call on a device (and the first one
// after its context was replaced, e.g. by cudaDeviceReset) does the look-up.
double* noalloc_scratch(int device)
{
    if (device < 0 || device >= NOALLOC_MAX_DEVICES) throw Error(IPCG_ERR_INVALID, "device index out of range");
    void* ctx = current_context();
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if (!g_noalloc_ptr[device] || g_noalloc_ctx[device] != ctx) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_partials);
        if (e != cudaSuccess || p == nullptr)
            throw Error(IPCG_ERR_CUDA, std::string("cudaGetSymbolAddress of the energy scratch failed: ")
                    + cudaGetErrorString(e));
        g_noalloc_ptr[device] = static_cast<double*>(p);
        g_noalloc_ctx[device] = ctx;
    }
    return g_noalloc_ptr[device];
}
} // namespace

void barrier_energy_noalloc(const double* V, const int* E, const int* F, int64_t nV, int64_t nE, int64_t nF,
    const ContactsNoAlloc& in, double dhat, double kappa, double dmin, int physical, double* energy, cudaStream_t s)
{
    const int64_t n = in.nvv + in.nev + in.nee + in.nfv;
    // the limit is checked on the 64-bit count, before any block count is formed
    if (n > (int64_t)NOALLOC_MAX_BLOCKS * BLOCK) {
        char msg[160];
        snprintf(msg, sizeof(msg), "too many contacts for the allocation-free energy: %lld > %lld",
            (long long)n, (long long)NOALLOC_MAX_BLOCKS * BLOCK);
        throw Error(IPCG_ERR_INVALID, msg);
    }
    const int nblk = grid_for(n, BLOCK);
    int dev = 0;
    IPCG_CUDA(cudaGetDevice(&dev));
    double* partial = noalloc_scratch(dev);
    if (n == 0) {
        IPCG_CUDA(cudaMemsetAsync(energy, 0, sizeof(double), s));
        return;
    }
    ContactsView cv { in.nvv, in.nev, in.nee, in.nfv, (const int2*)in.vv, (const int2*)in.ev, (const int2*)in.ee,
        (const int2*)in.fv, in.vv_w, in.ev_w, in.ee_w, in.fv_w, in.ee_eps, in.ee_dtype };
    const double xhat = (2 * dmin + dhat) * dhat;
    Params P { kappa, dmin * dmin, xhat, physical ? dhat / barrier_units(0, xhat) : 1.0, IPCG_PSD_NONE, 0, 0 };
    // every block overwrites its partial and the final kernel overwrites the
    // result, so nothing in the shared array needs clearing between calls
    IPCG_LAUNCH("k_energy_checked", s, k_energy_checked<<<nblk, BLOCK, 0, s>>>(cv, E, F, nV, nE, nF, V, P,
        partial));
    IPCG_LAUNCH("k_sum_partials", s, k_sum_partials<<<1, 1024, 0, s>>>(partial, nblk, energy));
}

} // namespace ipcg
