"""ctypes front-end of the CPU oracle (test infrastructure only).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import
this module: it is the checker for the GPU library, never part of it.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libipc_oracle.so")
_lib = None

PSD = {"none": 0, "clamp": 1, "abs": 2}


def build(force: bool = False) -> str:
    """Compile the oracle shared library with its Makefile."""
    src = os.path.join(_HERE, "ipc_oracle.cpp")
    if force or not os.path.exists(_LIB_PATH) or os.path.getmtime(_LIB_PATH) < os.path.getmtime(src):
        subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(_LIB_PATH)
        d, i64, i32, vp = C.c_double, C.c_int64, C.c_int, C.c_void_p
        P = C.c_void_p
        L.orc_point_edge_distance_type.restype = i32
        L.orc_point_triangle_distance_type.restype = i32
        L.orc_edge_edge_distance_type.restype = i32
        L.orc_point_triangle_distance.restype = d
        L.orc_point_triangle_distance.argtypes = [P, P, P, P, i32]
        L.orc_edge_edge_distance.restype = d
        L.orc_edge_edge_distance.argtypes = [P, P, P, P, i32]
        L.orc_point_edge_distance.restype = d
        L.orc_point_edge_distance.argtypes = [P, P, P, i32]
        L.orc_set_psd_solver.argtypes = [i32]
        L.orc_barrier.restype = d
        L.orc_barrier.argtypes = [d, d, i32]
        L.orc_barrier_kind.restype = d
        L.orc_barrier_kind.argtypes = [i32, d, d, i32]
        L.orc_barrier_gn_diagonal.argtypes = [vp, P, i64, P, P, d, d, d, i32, i32, P]
        L.orc_barrier_gn_quadratic_form.restype = d
        L.orc_barrier_gn_quadratic_form.argtypes = [vp, P, P, P, d, d, d, i32, P, i32]
        L.orc_distance_derivatives.restype = d
        L.orc_distance_derivatives.argtypes = [i32, i32, P, P, P]
        L.orc_faces_to_edges.restype = i32
        L.orc_faces_to_edges.argtypes = [P, i64, P, i64, P]
        L.orc_collisions_build.restype = vp
        L.orc_collisions_build.argtypes = [P, P, i64, P, i64, P, i64, P, d, d, i32, i32, i32]
        L.orc_mesh_areas.argtypes = [P, i64, P, i64, P, i64, P, P, P]
        L.orc_collisions_from_arrays.restype = vp
        L.orc_collisions_from_arrays.argtypes = [i64, P, P, i64, P, P, i64, P, P, P, P, i64, P, P]
        L.orc_collisions_counts.argtypes = [vp, P]
        L.orc_collisions_get.argtypes = [vp] + [P] * 10
        L.orc_collisions_free.argtypes = [vp]
        L.orc_barrier_energy.restype = d
        L.orc_barrier_energy.argtypes = [vp, P, P, P, d, d, d, i32, i32]
        L.orc_barrier_gradient.argtypes = [vp, P, i64, P, P, d, d, d, i32, i32, P]
        L.orc_barrier_hessian.restype = vp
        L.orc_barrier_hessian.argtypes = [vp, P, i64, P, P, d, d, d, i32, i32, i32]
        L.orc_csr_nnz.restype = i64
        L.orc_csr_nnz.argtypes = [vp]
        L.orc_csr_get.argtypes = [vp, P, P, P]
        L.orc_csr_free.argtypes = [vp]
        L.orc_contact_local.argtypes = [i32, i32, d, d, P, d, d, d, i32, i32, P, P, P]
        L.orc_ee_cross_sqnorm.restype = d
        L.orc_ee_cross_sqnorm.argtypes = [P, P, P]
        L.orc_ee_mollifier_threshold.restype = d
        L.orc_ee_mollifier_threshold.argtypes = [P]
        L.orc_ee_mollifier.restype = d
        L.orc_ee_mollifier.argtypes = [P, d, P, P]
        L.orc_point_triangle_ccd.restype = i32
        L.orc_point_triangle_ccd.argtypes = [P, P, d, d, d, C.c_long, d, P]
        L.orc_edge_edge_ccd.restype = i32
        L.orc_edge_edge_ccd.argtypes = [P, P, d, d, d, C.c_long, d, P]
        L.orc_ccd_stencils.argtypes = [i32, i64, P, P, d, d, d, C.c_long, d, P, P, P]
        L.orc_ccd_candidates.restype = vp
        L.orc_ccd_candidates.argtypes = [P, P, i64, P, i64, P, i64, d, i32, P]
        L.orc_ccd_candidates_get.argtypes = [vp, P, P]
        L.orc_collision_free_stepsize.restype = d
        L.orc_collision_free_stepsize.argtypes = [P, P, i64, P, i64, P, i64, d, d, C.c_long, d, i32, P]
        L.orc_tangential_build.restype = vp
        L.orc_tangential_build.argtypes = [vp, P, P, P, d, d, d, i32, P, P]
        L.orc_tangential_counts.argtypes = [vp, P]
        L.orc_tangential_get.argtypes = [vp] + [P] * 10
        L.orc_tangential_free.argtypes = [vp]
        L.orc_friction_energy.restype = d
        L.orc_friction_energy.argtypes = [vp, P, P, P, d, i32]
        L.orc_friction_gradient.argtypes = [vp, P, i64, P, P, d, i32, P]
        L.orc_friction_hessian.restype = vp
        L.orc_friction_hessian.argtypes = [vp, P, i64, P, P, d, i32, i32]
        L.orc_barrier_shape_derivative.restype = vp
        L.orc_barrier_shape_derivative.argtypes = [vp, P, P, i64, P, i64, P, i64, P, d, d, d, i32, i32, i32]
        L.orc_tangential_set_anisotropy.argtypes = [vp, P, P, P]
        L.orc_tangential_update_lagged_mu.argtypes = [vp, P, P, P, P, P]
        L.orc_tangential_lagged_mu.argtypes = [vp, P, P]
        L.orc_aniso_mu_eff.argtypes = [P, P, P, d, d, P]
        L.orc_friction_force.argtypes = [vp, P, P, P, i64, P, P, d, d, d, i32, d, i32, P]
        L.orc_friction_mu.restype = d
        L.orc_friction_mu.argtypes = [i32, d, d, d, d]
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


# --- primitives -------------------------------------------------------------
def point_triangle_distance_type(p, t0, t1, t2):
    return lib().orc_point_triangle_distance_type(*(_p(_f64(x)) for x in (p, t0, t1, t2)))


def edge_edge_distance_type(a0, a1, b0, b1):
    return lib().orc_edge_edge_distance_type(*(_p(_f64(x)) for x in (a0, a1, b0, b1)))


def point_edge_distance_type(p, e0, e1):
    return lib().orc_point_edge_distance_type(*(_p(_f64(x)) for x in (p, e0, e1)))


def point_triangle_distance(p, t0, t1, t2, dtype=-1):
    a = [_f64(x) for x in (p, t0, t1, t2)]
    return lib().orc_point_triangle_distance(*(_p(x) for x in a), dtype)


def edge_edge_distance(a0, a1, b0, b1, dtype=-1):
    a = [_f64(x) for x in (a0, a1, b0, b1)]
    return lib().orc_edge_edge_distance(*(_p(x) for x in a), dtype)


def point_edge_distance(p, e0, e1, dtype=-1):
    a = [_f64(x) for x in (p, e0, e1)]
    return lib().orc_point_edge_distance(*(_p(x) for x in a), dtype)


def set_psd_solver(name: str):
    """'ql' (tridiagonal QR, default) or 'jacobi' (independent cross-check)."""
    lib().orc_set_psd_solver({"ql": 0, "jacobi": 1}[name])


def barrier(d, dhat, deriv=0, kind=0):
    """Barrier function kind (0 clamped log, 1 normalized clamped log, 2 clamped
    log squared, 3 cubic, 4 two-stage) or its derivative."""
    if kind == 0:
        return lib().orc_barrier(float(d), float(dhat), int(deriv))
    return lib().orc_barrier_kind(int(kind), float(d), float(dhat), int(deriv))


def distance_derivatives(kind, x, dtype=8):
    """kind 0 PP, 1 point-line, 2 point-plane, 3 edge-edge(dtype)."""
    x = _f64(x).ravel()
    n = x.size
    g = np.zeros(n)
    H = np.zeros((n, n))
    d = lib().orc_distance_derivatives(kind, dtype, _p(x), _p(g), _p(H))
    return d, g, H


def contact_local(ctype, x, dhat, kappa, dmin=0.0, physical=False, psd="none", w=1.0, eps=0.0, dtype=8):
    x = _f64(x).ravel()
    n = x.size
    e = np.zeros(1)
    g = np.zeros(n)
    H = np.zeros((n, n))
    lib().orc_contact_local(ctype, dtype, eps, w, _p(x), dhat, kappa, dmin, int(physical), PSD[psd], _p(e), _p(g), _p(H))
    return e[0], g, H


def ee_cross_sqnorm(x):
    """|ea x eb|^2 of x = (ea0, ea1, eb0, eb1) with its gradient and Hessian."""
    x = _f64(x).reshape(4, 3)
    g, H = np.zeros(12), np.zeros((12, 12))
    s = lib().orc_ee_cross_sqnorm(_p(x), _p(g), _p(H))
    return s, g, H


def ee_mollifier_threshold(x_rest):
    return lib().orc_ee_mollifier_threshold(_p(_f64(x_rest).reshape(4, 3)))


def ee_mollifier(x, eps_x):
    """Edge-edge mollifier m(x) with its gradient and Hessian."""
    x = _f64(x).reshape(4, 3)
    g, H = np.zeros(12), np.zeros((12, 12))
    m = lib().orc_ee_mollifier(_p(x), float(eps_x), _p(g), _p(H))
    return m, g, H


def faces_to_edges(F, E):
    F, E = _i32(F), _i32(E)
    out = np.zeros_like(F)
    if lib().orc_faces_to_edges(_p(F), F.shape[0], _p(E), E.shape[0], _p(out)) != 0:
        raise RuntimeError("Unable to find edge!")
    return out


# --- collision set ------------------------------------------------------------
class Collisions:
    """Sorted collision set: vv (min,max), ev (e,v), ee (ea<eb)+eps+dtype, fv (f,v)."""

    def __init__(self, handle):
        self.h = handle
        L = lib()
        cnt = np.zeros(6, np.int64)
        L.orc_collisions_counts(self.h, _p(cnt))
        nvv, nev, nee, nfv, self.n_cand_ee, self.n_cand_fv = (int(c) for c in cnt)
        self.vv = np.zeros((nvv, 2), np.int32)
        self.vv_w = np.zeros(nvv)
        self.ev = np.zeros((nev, 2), np.int32)
        self.ev_w = np.zeros(nev)
        self.ee = np.zeros((nee, 2), np.int32)
        self.ee_eps = np.zeros(nee)
        self.ee_dtype = np.zeros(nee, np.int8)
        self.ee_w = np.zeros(nee)
        self.fv = np.zeros((nfv, 2), np.int32)
        self.fv_w = np.zeros(nfv)
        L.orc_collisions_get(self.h, *(_p(a) for a in (self.vv, self.vv_w, self.ev, self.ev_w, self.ee,
                                                        self.ee_eps, self.ee_dtype, self.ee_w, self.fv, self.fv_w)))

    def __len__(self):
        return len(self.vv_w) + len(self.ev_w) + len(self.ee_w) + len(self.fv_w)

    def __del__(self):
        try:
            lib().orc_collisions_free(self.h)
        except Exception:
            pass

    @staticmethod
    def from_arrays(vv, vv_w, ev, ev_w, ee, ee_eps, ee_dtype, ee_w, fv, fv_w):
        arrs = [_i32(vv), _f64(vv_w), _i32(ev), _f64(ev_w), _i32(ee), _f64(ee_eps),
                np.ascontiguousarray(ee_dtype, np.int8), _f64(ee_w), _i32(fv), _f64(fv_w)]
        h = lib().orc_collisions_from_arrays(
            len(arrs[1]), _p(arrs[0]), _p(arrs[1]), len(arrs[3]), _p(arrs[2]), _p(arrs[3]),
            len(arrs[5]), _p(arrs[4]), _p(arrs[5]), _p(arrs[6]), _p(arrs[7]),
            len(arrs[9]), _p(arrs[8]), _p(arrs[9]))
        c = Collisions(h)
        c._keep = arrs
        return c


def mesh_areas(rest, E, F):
    """(vertex_area, edge_area) of the rest mesh (collision_mesh.cpp:309-374)."""
    rest, E, F = _f64(rest), _i32(E), _i32(F)
    F2E = faces_to_edges(F, E)
    va, ea = np.zeros(rest.shape[0]), np.zeros(E.shape[0])
    lib().orc_mesh_areas(_p(rest), rest.shape[0], _p(E), E.shape[0], _p(F), F.shape[0], _p(F2E), _p(va), _p(ea))
    return va, ea


def build_collisions(V, E, F, dhat, dmin=0.0, rest=None, nthreads=None, area_weighting=False,
                     improved_max_approx=False):
    V, E, F = _f64(V), _i32(E), _i32(F)
    rest = V if rest is None else _f64(rest)
    F2E = faces_to_edges(F, E)
    nt = nthreads or os.cpu_count() or 1
    h = lib().orc_collisions_build(_p(V), _p(rest), V.shape[0], _p(E), E.shape[0], _p(F), F.shape[0], _p(F2E),
                                   float(dhat), float(dmin), int(bool(area_weighting)),
                                   int(bool(improved_max_approx)), int(nt))
    return Collisions(h)


def barrier_energy(col, V, E, F, dhat, kappa, dmin=0.0, physical=False, nthreads=None):
    V, E, F = _f64(V), _i32(E), _i32(F)
    return lib().orc_barrier_energy(col.h, _p(V), _p(E), _p(F), dhat, kappa, dmin, int(physical),
                                    int(nthreads or os.cpu_count() or 1))


def barrier_gradient(col, V, E, F, dhat, kappa, dmin=0.0, physical=False, nthreads=None):
    V, E, F = _f64(V), _i32(E), _i32(F)
    g = np.zeros(V.size)
    lib().orc_barrier_gradient(col.h, _p(V), V.shape[0], _p(E), _p(F), dhat, kappa, dmin, int(physical),
                               int(nthreads or os.cpu_count() or 1), _p(g))
    return g


def barrier_gauss_newton_diagonal(col, V, E, F, dhat, kappa, dmin=0.0, physical=False, nthreads=None):
    V, E, F = _f64(V), _i32(E), _i32(F)
    g = np.zeros(V.size)
    lib().orc_barrier_gn_diagonal(col.h, _p(V), V.shape[0], _p(E), _p(F), dhat, kappa, dmin, int(physical),
                                  int(nthreads or os.cpu_count() or 1), _p(g))
    return g


def barrier_gauss_newton_quadratic_form(col, V, E, F, p, dhat, kappa, dmin=0.0, physical=False, nthreads=None):
    V, E, F, p = _f64(V), _i32(E), _i32(F), _f64(p)
    return lib().orc_barrier_gn_quadratic_form(col.h, _p(V), _p(E), _p(F), dhat, kappa, dmin, int(physical), _p(p),
                                               int(nthreads or os.cpu_count() or 1))


def barrier_hessian(col, V, E, F, dhat, kappa, dmin=0.0, physical=False, psd="none", nthreads=None):
    """Returns (indptr int64, indices int32, data float64) of the ndof x ndof CSR."""
    V, E, F = _f64(V), _i32(E), _i32(F)
    L = lib()
    h = L.orc_barrier_hessian(col.h, _p(V), V.shape[0], _p(E), _p(F), dhat, kappa, dmin, int(physical),
                              PSD[psd], int(nthreads or os.cpu_count() or 1))
    nnz = L.orc_csr_nnz(h)
    rp = np.zeros(V.size + 1, np.int64)
    ci = np.zeros(nnz, np.int32)
    va = np.zeros(nnz)
    L.orc_csr_get(h, _p(rp), _p(ci), _p(va))
    L.orc_csr_free(h)
    return rp, ci, va


# --- CCD -----------------------------------------------------------------------
def point_triangle_ccd(x0, x1, min_distance=0.0, tmax=1.0, tolerance=1e-6, max_iterations=10_000_000,
                       rescale=0.8):
    x0, x1 = _f64(x0).reshape(4, 3), _f64(x1).reshape(4, 3)
    toi = np.zeros(1)
    hit = lib().orc_point_triangle_ccd(_p(x0), _p(x1), min_distance, tmax, tolerance, max_iterations, rescale, _p(toi))
    return bool(hit), float(toi[0])


def edge_edge_ccd(x0, x1, min_distance=0.0, tmax=1.0, tolerance=1e-6, max_iterations=10_000_000, rescale=0.8):
    x0, x1 = _f64(x0).reshape(4, 3), _f64(x1).reshape(4, 3)
    toi = np.zeros(1)
    hit = lib().orc_edge_edge_ccd(_p(x0), _p(x1), min_distance, tmax, tolerance, max_iterations, rescale, _p(toi))
    return bool(hit), float(toi[0])


def collision_free_stepsize(V0, V1, E, F, min_distance=0.0, tolerance=1e-6, max_iterations=10_000_000,
                            rescale=0.8, nthreads=None):
    V0, V1, E, F = _f64(V0), _f64(V1), _i32(E), _i32(F)
    nc = np.zeros(1, np.int64)
    t = lib().orc_collision_free_stepsize(_p(V0), _p(V1), V0.shape[0], _p(E), E.shape[0], _p(F), F.shape[0],
                                          min_distance, tolerance, max_iterations, rescale,
                                          int(nthreads or os.cpu_count() or 1), _p(nc))
    return float(t), int(nc[0])


def ccd_stencils(is_ee, x0, x1, min_distance=0.0, tmax=1.0, tolerance=1e-6, max_iterations=10_000_000,
                 rescale=0.8):
    """Batched single-stencil CCD; returns (hit bool[n], toi[n], boxes examined[n])."""
    x0 = _f64(x0).reshape(-1, 4, 3)
    x1 = _f64(x1).reshape(-1, 4, 3)
    n = x0.shape[0]
    hit = np.zeros(n, np.int8)
    toi = np.zeros(n)
    it = np.zeros(n, np.int64)
    lib().orc_ccd_stencils(int(is_ee), n, _p(x0), _p(x1), min_distance, tmax, tolerance, max_iterations, rescale,
                           _p(hit), _p(toi), _p(it))
    return hit.astype(bool), toi, it


def ccd_candidates(V0, V1, E, F, min_distance=0.0, nthreads=None):
    """Swept-box broad-phase candidates: (ee pairs (k,2), fv pairs (k,2))."""
    V0, V1, E, F = _f64(V0), _f64(V1), _i32(E), _i32(F)
    cnt = np.zeros(2, np.int64)
    h = lib().orc_ccd_candidates(_p(V0), _p(V1), V0.shape[0], _p(E), E.shape[0], _p(F), F.shape[0], min_distance,
                                 int(nthreads or os.cpu_count() or 1), _p(cnt))
    ee = np.zeros((int(cnt[0]), 2), np.int32)
    fv = np.zeros((int(cnt[1]), 2), np.int32)
    lib().orc_ccd_candidates_get(h, _p(ee), _p(fv))
    return ee, fv


def ccd_stencil_positions(V0, V1, E, F, ee, fv):
    """Stencil positions (x0, x1) of EE candidates then FV candidates."""
    ids_ee = np.concatenate([E[ee[:, 0]], E[ee[:, 1]]], axis=1)
    ids_fv = np.concatenate([fv[:, 1:2], F[fv[:, 0]]], axis=1)
    return (V0[ids_ee], V1[ids_ee]), (V0[ids_fv], V1[ids_fv])


def orient3d_exact(a, b, c, d):
    """Exact sign of det(a-d, b-d, c-d) with rational arithmetic (small cases)."""
    from fractions import Fraction as Fr
    A = [[Fr(float(p[k])) - Fr(float(d[k])) for k in range(3)] for p in (a, b, c)]
    det = (A[0][0] * (A[1][1] * A[2][2] - A[1][2] * A[2][1]) - A[0][1] * (A[1][0] * A[2][2] - A[1][2] * A[2][0])
           + A[0][2] * (A[1][0] * A[2][1] - A[1][1] * A[2][0]))
    return (det > 0) - (det < 0)


def has_intersections_bruteforce(V, E, F):
    """has_intersections (ipc.cpp:110-167) over every edge-face pair that shares
    no vertex: exact orientations of the edge's endpoints against the face's
    plane (geometry/intersection.cpp:120-147), then the crossing point's
    barycentric coordinates and edge parameter from a dense solve.  Pure
    Python: for small meshes only."""
    V = np.asarray(V, np.float64)
    for e in np.asarray(E):
        for f in np.asarray(F):
            if set(e.tolist()) & set(f.tolist()):
                continue
            e0, e1 = V[e[0]], V[e[1]]
            t0, t1, t2 = V[f[0]], V[f[1]], V[f[2]]
            o1 = orient3d_exact(t0, t1, t2, e0)
            o2 = orient3d_exact(t0, t1, t2, e1)
            if o1 != 0 and o2 != 0 and o1 == o2:
                continue
            M = np.stack([t1 - t0, t2 - t0, e0 - e1], axis=1)
            try:
                uvt = np.linalg.solve(M, e0 - t0)
            except np.linalg.LinAlgError:
                uvt = np.linalg.lstsq(M, e0 - t0, rcond=None)[0]
            if uvt[0] >= 0 and uvt[1] >= 0 and uvt[0] + uvt[1] <= 1 and 0 <= uvt[2] <= 1:
                return True
    return False



# --- friction -----------------------------------------------------------------

class Tangential:
    """TangentialCollisions built by the oracle: stencils (vv, ev, ee, fv),
    and per collision (vv | ev | ee | fv order) w, N, cp (2), P (3x2 as b0, b1),
    mu_s, mu_k."""

    def __init__(self, handle):
        self.h = handle
        L = lib()
        cnt = np.zeros(4, np.int64)
        L.orc_tangential_counts(self.h, _p(cnt))
        nvv, nev, nee, nfv = (int(c) for c in cnt)
        n = nvv + nev + nee + nfv
        self.vv = np.zeros((nvv, 2), np.int32)
        self.ev = np.zeros((nev, 2), np.int32)
        self.ee = np.zeros((nee, 2), np.int32)
        self.fv = np.zeros((nfv, 2), np.int32)
        self.w, self.N = np.zeros(n), np.zeros(n)
        self.cp, self.P = np.zeros((n, 2)), np.zeros((n, 6))
        self.mu_s, self.mu_k = np.zeros(n), np.zeros(n)
        L.orc_tangential_get(self.h, _p(self.vv), _p(self.ev), _p(self.ee), _p(self.fv), _p(self.w), _p(self.N),
                             _p(self.cp), _p(self.P), _p(self.mu_s), _p(self.mu_k))

    def __len__(self):
        return len(self.w)

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.orc_tangential_free(self.h)
            self.h = None


def tangential_build(col, V, E, F, dhat, kappa, mu_s, mu_k=None, dmin=0.0, physical=0):
    V, E, F = _f64(V), _i32(E), _i32(F)
    nV = V.shape[0]
    ms = _f64(np.broadcast_to(np.asarray(mu_s, np.float64), (nV,)))
    mk = _f64(np.broadcast_to(np.asarray(mu_s if mu_k is None else mu_k, np.float64), (nV,)))
    t = Tangential(lib().orc_tangential_build(col.h, _p(V), _p(E), _p(F), float(dhat), float(kappa), float(dmin),
                                              int(physical), _p(ms), _p(mk)))
    t._keep = (ms, mk)
    return t


def friction_energy(t, U, E, F, eps_v, nthreads=None):
    U, E, F = _f64(U), _i32(E), _i32(F)
    return lib().orc_friction_energy(t.h, _p(U), _p(E), _p(F), float(eps_v), int(nthreads or os.cpu_count() or 1))


def friction_gradient(t, U, E, F, eps_v, nthreads=None):
    U, E, F = _f64(U), _i32(E), _i32(F)
    g = np.zeros(U.size)
    lib().orc_friction_gradient(t.h, _p(U), U.shape[0], _p(E), _p(F), float(eps_v),
                                int(nthreads or os.cpu_count() or 1), _p(g))
    return g


def friction_hessian(t, U, E, F, eps_v, psd="none", nthreads=None):
    """(rowptr, col, val) of the friction Hessian."""
    U, E, F = _f64(U), _i32(E), _i32(F)
    h = lib().orc_friction_hessian(t.h, _p(U), U.shape[0], _p(E), _p(F), float(eps_v), PSD[psd],
                                   int(nthreads or os.cpu_count() or 1))
    L = lib()
    nnz = L.orc_csr_nnz(h)
    rp = np.zeros(U.size + 1, np.int64)
    ci = np.zeros(nnz, np.int32)
    va = np.zeros(nnz)
    L.orc_csr_get(h, _p(rp), _p(ci), _p(va))
    L.orc_csr_free(h)
    return rp, ci, va


def friction_mu(which, y, mu_s, mu_k, eps_v):
    """0: mu f0, 1: mu f1 / y, 2: (mu f1)' y - mu f1) / y^3, 3: mu(y)."""
    return lib().orc_friction_mu(int(which), float(y), float(mu_s), float(mu_k), float(eps_v))


def barrier_shape_derivative(col, V, E, F, dhat, kappa, rest=None, dmin=0.0, physical=0, area_weighting=False,
                             nthreads=None):
    """(rowptr, col, val) of NormalPotential::shape_derivative (rows:
    displacement dofs, columns: rest dofs); area_weighting adds the weight
    gradient term of a set built with area weighting."""
    V, E, F = _f64(V), _i32(E), _i32(F)
    rest = V if rest is None else _f64(rest)
    F2E = faces_to_edges(F, E)
    L = lib()
    h = L.orc_barrier_shape_derivative(col.h, _p(V), _p(rest), V.shape[0], _p(E), E.shape[0], _p(F), F.shape[0],
                                       _p(F2E), float(dhat), float(kappa), float(dmin), int(physical),
                                       int(bool(area_weighting)), int(nthreads or os.cpu_count() or 1))
    nnz = L.orc_csr_nnz(h)
    rp = np.zeros(V.size + 1, np.int64)
    ci = np.zeros(nnz, np.int32)
    va = np.zeros(nnz)
    L.orc_csr_get(h, _p(rp), _p(ci), _p(va))
    L.orc_csr_free(h)
    return rp, ci, va


def tangential_set_anisotropy(t, mu_aniso=None, mu_s_aniso=None, mu_k_aniso=None):
    arrs = [None if a is None else _f64(np.asarray(a).reshape(-1, 2)) for a in (mu_aniso, mu_s_aniso, mu_k_aniso)]
    t._aniso = arrs
    lib().orc_tangential_set_anisotropy(t.h, *[None if a is None else _p(a) for a in arrs])


def tangential_update_lagged_mu(t, rest, lagged, velocities, E, F):
    rest, lagged, velocities, E, F = _f64(rest), _f64(lagged), _f64(velocities), _i32(E), _i32(F)
    lib().orc_tangential_update_lagged_mu(t.h, _p(rest), _p(lagged), _p(velocities), _p(E), _p(F))


def tangential_lagged_mu(t):
    ms, mk = np.zeros(len(t)), np.zeros(len(t))
    lib().orc_tangential_lagged_mu(t.h, _p(ms), _p(mk))
    return ms, mk


def aniso_mu_eff(tau_aniso, mu_s_aniso, mu_k_aniso, mu_s, mu_k):
    a, b, c = (_f64(np.asarray(x, np.float64).reshape(2)) for x in (tau_aniso, mu_s_aniso, mu_k_aniso))
    out = np.zeros(2)
    lib().orc_aniso_mu_eff(_p(a), _p(b), _p(c), float(mu_s), float(mu_k), _p(out))
    return out[0], out[1]


def friction_force(t, rest, lagged, velocities, E, F, dhat, kappa, eps_v, dmin=0.0, physical=0, no_mu=False):
    rest, lagged, velocities, E, F = _f64(rest), _f64(lagged), _f64(velocities), _i32(E), _i32(F)
    out = np.zeros(velocities.size)
    lib().orc_friction_force(t.h, _p(rest), _p(lagged), _p(velocities), rest.shape[0], _p(E), _p(F), float(dhat),
                             float(kappa), float(dmin), int(physical), float(eps_v), int(bool(no_mu)), _p(out))
    return out
