"""ipctk_gb300 — the reference's ``ipctk`` contact API, computed on a GB300.

Mirrors the names, argument meanings and defaults of the reference's Python
bindings for the contact hot path (python/src/collision_mesh.cpp,
python/src/collisions/normal/normal_collisions.cpp,
python/src/potentials/barrier_potential.cpp, python/src/ipc.cpp,
python/src/ccd/tight_inclusion_ccd.cpp):

    mesh = CollisionMesh(V, E, F)
    collisions = NormalCollisions()
    collisions.build(mesh, V, dhat, dmin=0.0)
    B = BarrierPotential(dhat, stiffness)
    E = B(collisions, mesh, V)
    g = B.gradient(collisions, mesh, V)
    H = B.hessian(collisions, mesh, V, PSDProjectionMethod.CLAMP)
    alpha = compute_collision_free_stepsize(mesh, V0, V1)

Every computation runs in the CUDA library ``libipcg.so`` through its C ABI
(include/ipcg.h).  Inputs may be numpy arrays (host) or CUDA torch tensors
(device, passed without copies).  There is no CPU fallback: if the library
or a GPU is missing, calls raise.
"""
from __future__ import annotations

import ctypes as C
import enum
import os

import math

import numpy as np

from . import scenes  # noqa: F401  (seeded benchmark scenes)

_PKG_DIR = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB_PATH = os.path.join(_PKG_DIR, "_build", "libipcg.so")
_lib = None

OK = 0
_ERRORS = {1: ValueError, 2: RuntimeError, 3: MemoryError, 4: RuntimeError, 5: RuntimeError}


def _load():
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(
            f"CUDA library not built: {LIB_PATH} is missing (run the package build first)")
    L = C.CDLL(LIB_PATH)
    P, i64, i32, d = C.c_void_p, C.c_int64, C.c_int, C.c_double
    PP = C.POINTER(C.c_void_p)
    sig = {
        "ipcg_last_error": (C.c_char_p, []),
        "ipcg_version": (C.c_char_p, []),
        "ipcg_mesh_create": (i32, [P, i64, P, i64, P, i64, PP]),
        "ipcg_mesh_destroy": (i32, [P]),
        "ipcg_mesh_sizes": (i32, [P, P]),
        "ipcg_mesh_codim_counts": (i32, [P, P]),
        "ipcg_mesh_faces_to_edges": (i32, [P, P]),
        "ipcg_collisions_create": (i32, [PP]),
        "ipcg_collisions_destroy": (i32, [P]),
        "ipcg_collisions_build": (i32, [P, P, P, d, d]),
        "ipcg_collisions_counts": (i32, [P, P]),
        "ipcg_collisions_get": (i32, [P] + [P] * 10),
        "ipcg_collisions_set": (i32, [P, d, i64, P, P, i64, P, P, i64, P, P, P, P, i64, P, P]),
        "ipcg_barrier_energy": (i32, [P, P, P, d, d, i32, P]),
        "ipcg_barrier_gradient": (i32, [P, P, P, d, d, i32, P]),
        "ipcg_barrier_hessian": (i32, [P, P, P, d, d, i32, i32, PP]),
        "ipcg_barrier_energy_gradient_hessian": (i32, [P, P, P, d, d, i32, i32, P, P, PP]),
        "ipcg_csr_shape": (i32, [P, P, P]),
        "ipcg_csr_get": (i32, [P, P, P, P]),
        "ipcg_csr_destroy": (i32, [P]),
        "ipcg_collision_free_stepsize": (i32, [P, P, P, d, d, i64, d, P, P]),
        "ipcg_ccd_stencils": (i32, [i32, i64, P, P, d, d, d, i64, d, P, P]),
        "ipcg_distance_stencils": (i32, [i32, i64, P, P, P]),
        "ipcg_profile_enable": (i32, [i32]),
        "ipcg_profile_report": (i32, [C.c_char_p, i64, P]),
        "ipcg_launch_count": (i32, [P]),
        "ipcg_mesh_stream": (i32, [P, PP]),
        "ipcg_mesh_create_batch": (i32, [P, i64, P, i64, P, i64, i64, P, PP]),
        "ipcg_mesh_scenes": (i32, [P, P]),
        "ipcg_collisions_build_batch": (i32, [P, P, P, P, P]),
        "ipcg_barrier_batch": (i32, [P, P, P, P, P, i32, i32, P, P, PP]),
        "ipcg_collision_free_stepsize_batch": (i32, [P, P, P, P, d, i64, d, P, P]),
        "ipcg_set_hessian_chunk_contacts": (i32, [i64]),
        "ipcg_collisions_minimum_distance": (i32, [P, P, P, P]),
        "ipcg_is_step_collision_free": (i32, [P, P, P, d, d, i64, d, P]),
        "ipcg_has_intersections": (i32, [P, P, P]),
        "ipcg_barrier_gauss_newton_hessian_diagonal": (i32, [P, P, P, d, d, i32, P]),
        "ipcg_barrier_gauss_newton_hessian_quadratic_form": (i32, [P, P, P, d, d, i32, P, P]),
        "ipcg_mesh_areas": (i32, [P, P, P]),
        "ipcg_collisions_set_use_area_weighting": (i32, [P, i32]),
        "ipcg_collisions_use_area_weighting": (i32, [P, P]),
        "ipcg_collisions_set_collision_set_type": (i32, [P, i32]),
        "ipcg_collisions_set_enable_shape_derivatives": (i32, [P, i32]),
        "ipcg_collisions_enable_shape_derivatives": (i32, [P, P]),
        "ipcg_barrier_shape_derivative": (i32, [P, P, P, d, d, i32, PP]),
        "ipcg_collisions_collision_set_type": (i32, [P, P]),
        "ipcg_tangential_create": (i32, [PP]),
        "ipcg_tangential_destroy": (i32, [P]),
        "ipcg_tangential_build": (i32, [P, P, P, P, d, d, i32, P, P]),
        "ipcg_tangential_counts": (i32, [P, P]),
        "ipcg_tangential_get": (i32, [P] + [P] * 10),
        "ipcg_friction_potential": (i32, [P, P, P, d, i32, P, P, PP]),
        "ipcg_tangential_set_anisotropy": (i32, [P, P, P, P]),
        "ipcg_friction_force": (i32, [P, P, P, P, P, d, d, i32, d, d, i32, P]),
        "ipcg_tangential_build_batch": (i32, [P, P, P, P, P, P, i32, P, P]),
        "ipcg_friction_potential_batch": (i32, [P, P, P, d, i32, P, P, PP]),
        "ipcg_tangential_update_lagged_mu": (i32, [P, P, P, P, P]),
        "ipcg_tangential_reset_lagged_mu": (i32, [P]),
        "ipcg_tangential_lagged_mu": (i32, [P, P, P]),
        "ipcg_csr_get_int32": (i32, [P, P, P, P]),
        "ipcg_candidates_create": (i32, [PP]),
        "ipcg_candidates_destroy": (i32, [P]),
        "ipcg_candidates_build": (i32, [P, P, P, d]),
        "ipcg_candidates_build_swept": (i32, [P, P, P, P, d]),
        "ipcg_candidates_counts": (i32, [P, P]),
        "ipcg_candidates_get": (i32, [P, P, P]),
        "ipcg_candidates_per_vertex_safe_distances": (i32, [P, P, P, d, d, P]),
        "ipcg_candidates_collision_free_stepsize": (i32, [P, P, P, P, d, d, i64, d, P]),
        "ipcg_candidates_noncandidate_conservative_stepsize": (i32, [P, P, P, d, P]),
        "ipcg_candidates_cfl_stepsize": (i32, [P, P, P, P, d, d, d, i64, d, P]),
        "ipcg_server_create": (i32, [i32, i64, PP]),
        "ipcg_server_destroy": (i32, [P]),
        "ipcg_server_add_scene": (i32, [P, P, P, d, d, d, P]),
        "ipcg_server_submit_barrier": (i32, [P, i64, P, i32, P]),
        "ipcg_server_set_scene_options": (i32, [P, i64, i32]),
        "ipcg_server_submit_stepsize": (i32, [P, i64, P, P, d, P]),
        "ipcg_server_wait": (i32, [P, i64, P, P, PP]),
        "ipcg_server_stats": (i32, [P, P]),
        "ipcg_barrier_autotune": (i32, [P, P, P, P, P, i32, i32, C.c_char_p, i64, P]),
        "ipcg_barrier_tuning": (i32, [i32, P, P, P]),
        "ipcg_barrier_set_tuning": (i32, [i32, i32, i32, i32]),
        "ipcg_testing_defer_df64_psd": (i32, [i32]),
        "ipcg_testing_ccd_stats": (i32, [P, i32, P]),
        "ipcg_testing_ccd_budget": (i32, [i64]),
        "ipcg_fp64_fma_rate": (i32, [P]),
        "ipcg_initial_barrier_stiffness": (i32, [d, i32, d, d, P, P, i64, d, d, P, P]),
        "ipcg_update_barrier_stiffness": (i32, [d, d, d, d, d, d, d, P]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


def lib():
    """The loaded C-ABI library (ctypes.CDLL)."""
    return _load()


def _check(status):
    if status != OK:
        msg = _load().ipcg_last_error().decode()
        raise _ERRORS.get(status, RuntimeError)(msg)


def _is_torch_cuda(x):
    return type(x).__module__.startswith("torch") and getattr(x, "is_cuda", False)


def _ptr(x):
    if x is None:
        return None
    if _is_torch_cuda(x):
        return C.c_void_p(x.data_ptr())
    return x.ctypes.data_as(C.c_void_p)


def _as_f64(x, ncols=3):
    if _is_torch_cuda(x):
        import torch
        x = x.to(torch.float64).contiguous()
        return x
    a = np.ascontiguousarray(x, dtype=np.float64)
    if a.ndim != 2 or (ncols and a.shape[1] != ncols):
        raise ValueError(f"expected an (n, {ncols}) array")
    return a


def _as_f64_vec(x):
    """A flat float64 vector (numpy array or contiguous CUDA tensor)."""
    if _is_torch_cuda(x):
        import torch
        return x.to(torch.float64).contiguous().reshape(-1)
    return np.ascontiguousarray(x, dtype=np.float64).reshape(-1)


def _as_i32(x, ncols):
    a = np.ascontiguousarray(np.asarray(x), dtype=np.int32)
    if a.size == 0:
        return np.zeros((0, ncols), np.int32)
    if a.ndim != 2 or a.shape[1] != ncols:
        raise ValueError(f"expected an (n, {ncols}) index array")
    return a


def profile_enable(on: bool = True):
    """Time every library kernel with CUDA events on its stream (clears stats)."""
    _check(_load().ipcg_profile_enable(int(on)))


def profile_report() -> dict:
    """{kernel: {"launches": n, "ms": total}} accumulated since profile_enable."""
    import json
    L = _load()
    need = C.c_int64()
    _check(L.ipcg_profile_report(None, 0, C.byref(need)))
    buf = C.create_string_buffer(need.value)
    _check(L.ipcg_profile_report(buf, need.value, C.byref(need)))
    return json.loads(buf.value.decode())


def set_hessian_chunk_contacts(contacts: int = 0):
    """Memory bound of batched Hessians: at most ``contacts`` local 12x12
    blocks are held at once (0 = default 4,194,304).  Results do not change."""
    _check(_load().ipcg_set_hessian_chunk_contacts(int(contacts)))


def _precision_bits(mode) -> int:
    """Option bits of a mixed-precision mode: False / "fp64", True / "pt",
    "local" (IPCG_BARRIER_FP32_PT = 2, IPCG_BARRIER_FP32_LOCAL = 4), and
    "psd_df64" / "local_df64": FP64 or "local" with the PSD projection's
    eigenpairs in df64 (IPCG_BARRIER_DF64_PSD = 8)."""
    if mode in (False, None, "fp64"):
        return 0
    if mode in (True, "pt"):
        return 2
    if mode == "local":
        return 2 | 4
    if mode == "psd_df64":
        return 8
    if mode == "local_df64":
        return 2 | 4 | 8
    raise ValueError(f"unknown mixed-precision mode {mode!r}")


def autotune_barrier(collisions, mesh, vertices, dhat, stiffness, options: int = 0, project_hessian_to_psd=1) -> dict:
    """ipcg_barrier_autotune: dhat / stiffness one per scene; returns the
    JSON report as a dict (candidates and the chosen launch shape)."""
    import json
    V = _as_f64(vertices)
    dh = np.ascontiguousarray(np.atleast_1d(np.asarray(dhat, np.float64)))
    kap = np.ascontiguousarray(np.atleast_1d(np.asarray(stiffness, np.float64)))
    need = C.c_int64()
    buf = C.create_string_buffer(1 << 16)
    _check(_load().ipcg_barrier_autotune(collisions._h, mesh._h, _ptr(V), _ptr(dh), _ptr(kap), int(options),
                                         int(project_hessian_to_psd), buf, len(buf), C.byref(need)))
    return json.loads(buf.value.decode())


STAGE_LOCAL, STAGE_PSD, STAGE_PSD_DF64 = 0, 1, 2


def barrier_tuning(stage: int = STAGE_PSD) -> dict:
    """A stage's launch shape on the current device (ipcg_barrier_tuning):
    STAGE_LOCAL the local Hessians, STAGE_PSD the FP64 projection and
    scatter, STAGE_PSD_DF64 the df64 one."""
    t, b, g = C.c_int(), C.c_int(), C.c_int()
    _check(_load().ipcg_barrier_tuning(int(stage), C.byref(t), C.byref(b), C.byref(g)))
    return {"threads": t.value, "blocks_per_sm": b.value, "tiles_per_grab": g.value}


def set_barrier_tuning(stage: int, threads: int, blocks_per_sm: int, tiles_per_grab: int = 1):
    _check(_load().ipcg_barrier_set_tuning(int(stage), int(threads), int(blocks_per_sm), int(tiles_per_grab)))


def testing_defer_df64_psd(on: bool):
    """Testing switch (ipcg_testing_defer_df64_psd): the df64 projection
    hands every local Hessian to its FP64 fix-up pass."""
    _check(_load().ipcg_testing_defer_df64_psd(int(bool(on))))


def testing_ccd_stats(mesh, enable: bool = True) -> dict:
    """Testing (ipcg_testing_ccd_stats): per step-size pass (seeds, budgeted,
    hard) the queries run, boxes examined, the largest query's boxes and the
    hits since the previous call; enable keeps collecting."""
    out = np.zeros(12, np.int64)
    _check(_load().ipcg_testing_ccd_stats(mesh._h, int(bool(enable)), _ptr(out)))
    keys = ("queries", "boxes", "max_boxes", "hits")
    return {p: dict(zip(keys, (int(x) for x in out[4 * k:4 * k + 4]))) for k, p in enumerate(("seeds", "budgeted", "hard"))}


def fp64_fma_rate() -> float:
    """ipcg_fp64_fma_rate: the device's FP64 fused multiply-add rate, TFLOP/s."""
    r = C.c_double()
    _check(_load().ipcg_fp64_fma_rate(C.byref(r)))
    return float(r.value)


def testing_ccd_budget(boxes: int = 0):
    """Testing (ipcg_testing_ccd_budget): the one-thread step-size pass's box
    budget, after which a query moves to the warp-per-query pass; 0 restores
    the default."""
    _check(_load().ipcg_testing_ccd_budget(int(boxes)))


def launch_count() -> int:
    """Kernel launches issued by the library since it was loaded."""
    n = C.c_int64()
    _check(_load().ipcg_launch_count(C.byref(n)))
    return int(n.value)


class DeviceCSR:
    """A CSR matrix held on the device by the library (ipcg_csr)."""

    def __init__(self, handle, ndof):
        self._h = handle
        self.ndof = ndof
        rows, nnz = C.c_int64(), C.c_int64()
        _check(_load().ipcg_csr_shape(handle, C.byref(rows), C.byref(nnz)))
        self.nnz = int(nnz.value)

    def to_scipy(self):
        h, self._h = self._h, None
        return _csr_to_scipy(h, self.ndof)

    def values_into(self, out):
        """Copy the nnz values into ``out`` (a float64 torch CUDA tensor or
        numpy array of nnz entries) without the index arrays."""
        if self._h is None:
            raise ValueError("matrix already released")
        _check(_load().ipcg_csr_get(self._h, None, None, _ptr(out)))
        return out

    def free(self):
        if self._h:
            _load().ipcg_csr_destroy(self._h)
            self._h = None

    def __del__(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.ipcg_csr_destroy(self._h)


class PSDProjectionMethod(enum.IntEnum):
    """src/ipc/utils/eigen_ext.hpp:202-206"""
    NONE = 0
    CLAMP = 1
    ABS = 2


class EdgeEdgeDistanceType(enum.IntEnum):
    EA0_EB0 = 0
    EA0_EB1 = 1
    EA1_EB0 = 2
    EA1_EB1 = 3
    EA_EB0 = 4
    EA_EB1 = 5
    EA0_EB = 6
    EA1_EB = 7
    EA_EB = 8
    AUTO = 9


class PointTriangleDistanceType(enum.IntEnum):
    P_T0 = 0
    P_T1 = 1
    P_T2 = 2
    P_E0 = 3
    P_E1 = 4
    P_E2 = 5
    P_T = 6
    AUTO = 7


class PointEdgeDistanceType(enum.IntEnum):
    P_E0 = 0
    P_E1 = 1
    P_E = 2
    AUTO = 3


class CollisionMesh:
    """CollisionMesh(rest_positions, edges, faces) (src/ipc/collision_mesh.hpp:21-26).

    Topology and rest positions are uploaded once and stay on the device."""

    def __init__(self, rest_positions, edges=None, faces=None):
        L = _load()
        V = np.ascontiguousarray(np.asarray(rest_positions, dtype=np.float64))
        if V.ndim != 2 or V.shape[1] != 3:
            raise ValueError("only 3D meshes are supported: rest_positions must be (n, 3)")
        E = _as_i32(edges if edges is not None else np.zeros((0, 2)), 2)
        F = _as_i32(faces if faces is not None else np.zeros((0, 3)), 3)
        h = C.c_void_p()
        _check(L.ipcg_mesh_create(_ptr(V), V.shape[0], _ptr(E), E.shape[0], _ptr(F), F.shape[0], C.byref(h)))
        self._h = h
        self._rest = V
        self._E = E
        self._F = F

    def __del__(self):
        h = getattr(self, "_h", None)
        if h and _lib is not None:
            _lib.ipcg_mesh_destroy(h)
            self._h = None

    @property
    def num_vertices(self):
        return self._rest.shape[0]

    @property
    def num_edges(self):
        return self._E.shape[0]

    @property
    def num_faces(self):
        return self._F.shape[0]

    @property
    def dim(self):
        return 3

    @property
    def ndof(self):
        return 3 * self.num_vertices

    @property
    def rest_positions(self):
        return self._rest

    @property
    def edges(self):
        return self._E

    @property
    def faces(self):
        return self._F

    @property
    def stream(self) -> int:
        """Address of the cudaStream_t all work on this mesh runs on."""
        p = C.c_void_p()
        _check(_load().ipcg_mesh_stream(self._h, C.byref(p)))
        return int(p.value or 0)

    def _codim_counts(self):
        c = np.zeros(2, np.int64)
        _check(_load().ipcg_mesh_codim_counts(self._h, _ptr(c)))
        return c

    @property
    def num_codim_vertices(self):
        """CollisionMesh::num_codim_vertices(): vertices that belong to no edge.
        Collision builds, candidate builds and step sizes refuse meshes that
        have any (their extra candidate passes are not provided)."""
        return int(self._codim_counts()[0])

    @property
    def num_codim_edges(self):
        """CollisionMesh::num_codim_edges(): edges that belong to no face."""
        return int(self._codim_counts()[1])

    @property
    def faces_to_edges(self):
        out = np.zeros_like(self._F)
        _check(_load().ipcg_mesh_faces_to_edges(self._h, _ptr(out)))
        return out

    @property
    def vertex_areas(self):
        """CollisionMesh::vertex_areas() (collision_mesh.cpp:309-374)."""
        out = np.zeros(self.num_vertices)
        _check(_load().ipcg_mesh_areas(self._h, _ptr(out), None))
        return out

    @property
    def edge_areas(self):
        """CollisionMesh::edge_areas() (collision_mesh.cpp:309-374)."""
        out = np.zeros(self.num_edges)
        _check(_load().ipcg_mesh_areas(self._h, None, _ptr(out)))
        return out


class SceneBatch(CollisionMesh):
    """Many independent scenes (one CollisionMesh each in the reference)
    packed into one device mesh: ``SceneBatch([(V0, E0, F0), (V1, E1, F1), ...])``.

    Edges and faces of each scene use its own vertex indices; they are
    shifted into the packed numbering here.  Contacts never join two scenes.
    NormalCollisions.build, BatchBarrierPotential and
    compute_collision_free_stepsize_batch take one parameter per scene."""

    def __init__(self, scenes):
        L = _load()
        Vs, Es, Fs, voff = [], [], [], [0]
        for sc in scenes:
            V, E, F = (tuple(sc) + (None, None))[:3]
            V = np.ascontiguousarray(np.asarray(V, dtype=np.float64))
            if V.ndim != 2 or V.shape[1] != 3:
                raise ValueError("only 3D meshes are supported: rest_positions must be (n, 3)")
            Vs.append(V)
            Es.append(_as_i32(E if E is not None else np.zeros((0, 2)), 2) + voff[-1])
            Fs.append(_as_i32(F if F is not None else np.zeros((0, 3)), 3) + voff[-1])
            voff.append(voff[-1] + V.shape[0])
        if not Vs:
            raise ValueError("a batch needs at least one scene")
        V = np.ascontiguousarray(np.concatenate(Vs))
        E = np.ascontiguousarray(np.concatenate(Es), dtype=np.int32)
        F = np.ascontiguousarray(np.concatenate(Fs), dtype=np.int32)
        self.vertex_offsets = np.asarray(voff, np.int64)
        h = C.c_void_p()
        _check(L.ipcg_mesh_create_batch(_ptr(V), V.shape[0], _ptr(E), E.shape[0], _ptr(F), F.shape[0],
                                        len(Vs), _ptr(self.vertex_offsets), C.byref(h)))
        self._h = h
        self._rest = V
        self._E = E
        self._F = F

    @property
    def num_scenes(self):
        return len(self.vertex_offsets) - 1

    def per_scene(self, x):
        """Broadcast a scalar (or check an array) to one float per scene."""
        return np.ascontiguousarray(np.broadcast_to(np.asarray(x, np.float64), (self.num_scenes,)))

    def pack(self, vertices_per_scene):
        """Concatenate per-scene (n_k, 3) position arrays."""
        return np.ascontiguousarray(np.concatenate([np.asarray(v, np.float64) for v in vertices_per_scene]))

    def unpack(self, packed):
        """Split a packed (nV, 3) array (or 3nV vector) into per-scene arrays."""
        a = np.asarray(packed)
        per = 3 if a.ndim == 1 else 1
        o = self.vertex_offsets * per
        return [a[o[k]:o[k + 1]] for k in range(self.num_scenes)]


class NormalCollisions:
    """NormalCollisions (src/ipc/collisions/normal/normal_collisions.hpp).

    The set lives on the device; the ``*_collisions`` properties copy it out
    as index arrays (sorted by key)."""

    def __init__(self):
        h = C.c_void_p()
        _check(_load().ipcg_collisions_create(C.byref(h)))
        self._h = h
        self._cache = None

    @property
    def use_area_weighting(self) -> bool:
        """NormalCollisions::use_area_weighting (applies to the next build)."""
        v = C.c_int()
        _check(_load().ipcg_collisions_use_area_weighting(self._h, C.byref(v)))
        return bool(v.value)

    @use_area_weighting.setter
    def use_area_weighting(self, on: bool):
        _check(_load().ipcg_collisions_set_use_area_weighting(self._h, int(bool(on))))

    @property
    def enable_shape_derivatives(self) -> bool:
        """NormalCollisions::enable_shape_derivatives (applies to the next build)."""
        v = C.c_int()
        _check(_load().ipcg_collisions_enable_shape_derivatives(self._h, C.byref(v)))
        return bool(v.value)

    @enable_shape_derivatives.setter
    def enable_shape_derivatives(self, on: bool):
        _check(_load().ipcg_collisions_set_enable_shape_derivatives(self._h, int(bool(on))))

    class CollisionSetType(enum.IntEnum):
        """NormalCollisions::CollisionSetType (normal_collisions.hpp); OGC is
        not provided."""
        IPC = 0
        IMPROVED_MAX_APPROX = 1
        OGC = 2

    @property
    def collision_set_type(self):
        v = C.c_int()
        _check(_load().ipcg_collisions_collision_set_type(self._h, C.byref(v)))
        return NormalCollisions.CollisionSetType(v.value)

    @collision_set_type.setter
    def collision_set_type(self, t):
        _check(_load().ipcg_collisions_set_collision_set_type(self._h, int(t)))

    def __del__(self):
        h = getattr(self, "_h", None)
        if h and _lib is not None:
            _lib.ipcg_collisions_destroy(h)
            self._h = None

    def build(self, mesh: CollisionMesh, vertices, dhat: float, dmin: float = 0.0, broad_phase=None):
        """normal_collisions.cpp:20-36.  ``broad_phase`` is accepted for API
        compatibility; the device LBVH is always used."""
        V = _as_f64(vertices)
        if isinstance(mesh, SceneBatch):
            dh, dm = mesh.per_scene(dhat), mesh.per_scene(dmin)
            _check(_load().ipcg_collisions_build_batch(self._h, mesh._h, _ptr(V), _ptr(dh), _ptr(dm)))
        else:
            _check(_load().ipcg_collisions_build(self._h, mesh._h, _ptr(V), float(dhat), float(dmin)))
        self._cache = None

    def counts(self):
        c = np.zeros(6, np.int64)
        _check(_load().ipcg_collisions_counts(self._h, _ptr(c)))
        return c

    def __len__(self):
        return int(self.counts()[:4].sum())

    def size(self):
        return len(self)

    def empty(self):
        return len(self) == 0

    @property
    def num_candidates(self):
        c = self.counts()
        return int(c[4] + c[5])

    def to_arrays(self):
        """dict with vv, vv_w, ev, ev_w, ee, ee_eps_x, ee_dtype, ee_w, fv, fv_w."""
        if self._cache is None:
            nvv, nev, nee, nfv = (int(x) for x in self.counts()[:4])
            a = dict(vv=np.zeros((nvv, 2), np.int32), vv_w=np.zeros(nvv), ev=np.zeros((nev, 2), np.int32),
                     ev_w=np.zeros(nev), ee=np.zeros((nee, 2), np.int32), ee_eps_x=np.zeros(nee),
                     ee_dtype=np.zeros(nee, np.int8), ee_w=np.zeros(nee), fv=np.zeros((nfv, 2), np.int32),
                     fv_w=np.zeros(nfv))
            _check(_load().ipcg_collisions_get(self._h, *(_ptr(a[k]) for k in (
                "vv", "vv_w", "ev", "ev_w", "ee", "ee_eps_x", "ee_dtype", "ee_w", "fv", "fv_w"))))
            self._cache = a
        return self._cache

    def set_arrays(self, vv, vv_w, ev, ev_w, ee, ee_eps_x, ee_dtype, ee_w, fv, fv_w, dmin=0.0):
        arrs = [_as_i32(vv, 2), np.ascontiguousarray(vv_w, np.float64), _as_i32(ev, 2),
                np.ascontiguousarray(ev_w, np.float64), _as_i32(ee, 2), np.ascontiguousarray(ee_eps_x, np.float64),
                np.ascontiguousarray(ee_dtype, np.int8), np.ascontiguousarray(ee_w, np.float64),
                _as_i32(fv, 2), np.ascontiguousarray(fv_w, np.float64)]
        _check(_load().ipcg_collisions_set(
            self._h, float(dmin), len(arrs[1]), _ptr(arrs[0]), _ptr(arrs[1]), len(arrs[3]), _ptr(arrs[2]),
            _ptr(arrs[3]), len(arrs[5]), _ptr(arrs[4]), _ptr(arrs[5]), _ptr(arrs[6]), _ptr(arrs[7]),
            len(arrs[9]), _ptr(arrs[8]), _ptr(arrs[9])))
        self._cache = None

    def compute_minimum_distance(self, mesh: CollisionMesh, vertices) -> float:
        """normal_collisions.cpp:209-233: smallest squared distance (+inf if empty)."""
        V = _as_f64(vertices)
        out = np.zeros(1)
        _check(_load().ipcg_collisions_minimum_distance(self._h, mesh._h, _ptr(V), _ptr(out)))
        return float(out[0])

    @property
    def vv_collisions(self):
        return self.to_arrays()["vv"]

    @property
    def ev_collisions(self):
        return self.to_arrays()["ev"]

    @property
    def ee_collisions(self):
        return self.to_arrays()["ee"]

    @property
    def fv_collisions(self):
        return self.to_arrays()["fv"]


def _csr_to_scipy(h, ndof):
    import scipy.sparse as sp
    L = _load()
    rows, nnz = C.c_int64(), C.c_int64()
    _check(L.ipcg_csr_shape(h, C.byref(rows), C.byref(nnz)))
    # both index arrays 32-bit when they fit, so scipy keeps them as given
    # (mixed widths make it copy and convert); outputs are fully written
    small = nnz.value < 2 ** 31 - 1
    rp = np.empty(rows.value + 1, np.int32 if small else np.int64)
    ci = np.empty(nnz.value, np.int32)
    va = np.empty(nnz.value)
    try:
        if small:
            _check(L.ipcg_csr_get_int32(h, _ptr(rp), _ptr(ci), _ptr(va)))
        else:
            _check(L.ipcg_csr_get(h, _ptr(rp), _ptr(ci), _ptr(va)))
    finally:
        _check(L.ipcg_csr_destroy(h))
    # symmetric: CSR arrays are also the CSC arrays (Eigen ColMajor)
    return sp.csc_matrix((va, ci, rp), shape=(ndof, ndof), copy=False)


class Barrier:
    """A barrier function b(d, dhat) (src/ipc/barrier/barrier.hpp).  The
    potential evaluates it on the device; these host methods are the scalar
    functions themselves, for callers that tune stiffness or plot them."""

    kind = 0

    def __call__(self, d: float, dhat: float) -> float:
        return self._eval(0, float(d), float(dhat))

    def first_derivative(self, d: float, dhat: float) -> float:
        return self._eval(1, float(d), float(dhat))

    def second_derivative(self, d: float, dhat: float) -> float:
        return self._eval(2, float(d), float(dhat))

    def units(self, dhat: float) -> float:
        return float(dhat) * float(dhat)

    def __repr__(self):
        return type(self).__name__ + "()"


def _clamped_log(k, d, dh):
    if k == 0:
        if d <= 0:
            return math.inf
        return 0.0 if d >= dh else -(d - dh) * (d - dh) * math.log(d / dh)
    if d <= 0 or d >= dh:
        return 0.0
    if k == 1:
        return (dh - d) * (2 * math.log(d / dh) - dh / d + 1)
    r = dh / d
    return (r + 2) * r - 2 * math.log(d / dh) - 3


class ClampedLogBarrier(Barrier):
    """-(d - dhat)^2 ln(d / dhat) (barrier.cpp:11-43), the default."""
    kind = 0

    def _eval(self, k, d, dh):
        return _clamped_log(k, d, dh)


class NormalizedClampedLogBarrier(Barrier):
    """ClampedLogBarrier of d / dhat against 1 (barrier.hpp:145-175)."""
    kind = 1

    def _eval(self, k, d, dh):
        return _clamped_log(k, d / dh, 1.0) / dh ** k

    def units(self, dhat):
        return 1.0


class ClampedLogSqBarrier(Barrier):
    """(d - dhat)^2 ln^2(d / dhat) (barrier.cpp:47-86)."""
    kind = 2

    def _eval(self, k, d, dh):
        if k == 0 and d <= 0:
            return math.inf
        if d <= 0 or d >= dh:
            return 0.0
        lg = math.log(d / dh)
        if k == 0:
            return (d - dh) * (d - dh) * lg * lg
        if k == 1:
            return 2 * (d - dh) * lg * (lg + (d - dh) / d)
        t0 = dh - d
        t2 = (t0 * t0) / (d * d)
        return 2 * ((lg * lg) - (lg - 1) * t2 - 4 * lg * t0 / d)


class CubicBarrier(Barrier):
    """-2/(3 dhat) (d - dhat)^3 (barrier.cpp:90-117)."""
    kind = 3

    def _eval(self, k, d, dh):
        if not d < dh:
            return 0.0
        dm = d - dh
        return (-2.0 / 3.0 / dh * dm * dm * dm, -2 / dh * dm * dm, 4 * (1 - d / dh))[k]


class TwoStageBarrier(Barrier):
    """Two-stage activation (barrier.cpp:121-152)."""
    kind = 4

    def _eval(self, k, d, dh):
        if d >= dh:
            return 0.0
        if d >= 0.5 * dh:
            return (0.5 * (dh - d) * (dh - d), d - dh, 1.0)[k]
        if k == 0:
            return -0.25 * dh * dh * (math.log(2 * d / dh) - 0.5)
        return -0.25 * dh * dh / d if k == 1 else (0.25 * dh * dh) / (d * d)


class BarrierPotential:
    """BarrierPotential(dhat, stiffness, use_physical_barrier=False) or
    BarrierPotential(barrier, dhat, stiffness, use_physical_barrier=False)
    (src/ipc/potentials/barrier_potential.hpp:24-37); ClampedLogBarrier by
    default."""

    def __init__(self, *args, use_physical_barrier: bool = False, mixed_precision=False, **kw):
        """``mixed_precision`` (no counterpart in the reference): False for
        FP64 throughout; True or "pt" for face-vertex contacts in FP32
        (IPCG_BARRIER_FP32_PT); "local" for every contact but near-parallel
        edge-edge ones in FP32 (IPCG_BARRIER_FP32_LOCAL); "psd_df64" and
        "local_df64" add the PSD projection's eigenpairs in df64
        (IPCG_BARRIER_DF64_PSD, about 1e-13 from FP64) to FP64 or "local".
        The mollifier, the projected Hessian's subtraction and assembly stay
        FP64 in every mode."""
        args = list(args)
        barrier = kw.pop("barrier", None)
        if args and isinstance(args[0], Barrier):
            barrier = args.pop(0)
        names = ["dhat", "stiffness", "use_physical_barrier"]
        vals = dict(zip(names, args))
        vals.update(kw)
        if "use_physical_barrier" not in vals:
            vals["use_physical_barrier"] = use_physical_barrier
        dhat, stiffness = vals["dhat"], vals["stiffness"]
        if not dhat > 0:
            raise ValueError("dhat must be positive")
        self.barrier = barrier if barrier is not None else ClampedLogBarrier()
        self.dhat = float(dhat)
        self.stiffness = float(stiffness)
        self.use_physical_barrier = bool(vals["use_physical_barrier"])
        self.mixed_precision = mixed_precision

    @property
    def _options(self):
        return (int(self.use_physical_barrier) | _precision_bits(self.mixed_precision)
                | (int(self.barrier.kind) << 4))

    def shape_derivative(self, collisions: NormalCollisions, mesh: CollisionMesh, vertices):
        """NormalPotential::shape_derivative (normal_potential.cpp:85-123):
        scipy CSR, rows displacement dofs, columns rest dofs."""
        import scipy.sparse as sp
        V = _as_f64(vertices)
        h = C.c_void_p()
        _check(_load().ipcg_barrier_shape_derivative(collisions._h, mesh._h, _ptr(V), self.dhat, self.stiffness,
                                                     self._options & ~14, C.byref(h)))
        A = _csr_to_scipy(h, 3 * mesh.num_vertices)  # CSC view of the CSR arrays = transpose
        return sp.csr_matrix((A.data, A.indices, A.indptr), shape=A.shape)

    def gauss_newton_hessian_diagonal(self, collisions: NormalCollisions, mesh: CollisionMesh, vertices):
        """NormalPotential::gauss_newton_hessian_diagonal (normal_potential.cpp:15-48)."""
        V = _as_f64(vertices)
        if _is_torch_cuda(V):
            import torch
            g = torch.empty(V.numel(), dtype=torch.float64, device=V.device)
        else:
            g = np.empty(V.size)
        _check(_load().ipcg_barrier_gauss_newton_hessian_diagonal(collisions._h, mesh._h, _ptr(V), self.dhat,
                                                                  self.stiffness, self._options, _ptr(g)))
        return g

    def gauss_newton_hessian_quadratic_form(self, collisions: NormalCollisions, mesh: CollisionMesh, vertices,
                                            p) -> float:
        """NormalPotential::gauss_newton_hessian_quadratic_form (normal_potential.cpp:50-83)."""
        V = _as_f64(vertices)
        P = _as_f64(p if _is_torch_cuda(p) else np.reshape(p, (-1, 3)))
        out = np.zeros(1)
        _check(_load().ipcg_barrier_gauss_newton_hessian_quadratic_form(
            collisions._h, mesh._h, _ptr(V), self.dhat, self.stiffness, self._options, _ptr(P), _ptr(out)))
        return float(out[0])

    def __call__(self, collisions: NormalCollisions, mesh: CollisionMesh, vertices) -> float:
        V = _as_f64(vertices)
        e = np.zeros(1)
        _check(_load().ipcg_barrier_energy(collisions._h, mesh._h, _ptr(V), self.dhat, self.stiffness,
                                           self._options, _ptr(e)))
        return float(e[0])

    def gradient(self, collisions: NormalCollisions, mesh: CollisionMesh, vertices):
        V = _as_f64(vertices)
        if _is_torch_cuda(V):
            import torch
            g = torch.empty(V.numel(), dtype=torch.float64, device=V.device)
        else:
            g = np.empty(V.size)
        _check(_load().ipcg_barrier_gradient(collisions._h, mesh._h, _ptr(V), self.dhat, self.stiffness,
                                             self._options, _ptr(g)))
        return g

    def hessian(self, collisions: NormalCollisions, mesh: CollisionMesh, vertices,
                project_hessian_to_psd=PSDProjectionMethod.NONE):
        V = _as_f64(vertices)
        h = C.c_void_p()
        _check(_load().ipcg_barrier_hessian(collisions._h, mesh._h, _ptr(V), self.dhat, self.stiffness,
                                            self._options, int(project_hessian_to_psd),
                                            C.byref(h)))
        return _csr_to_scipy(h, 3 * mesh.num_vertices)

    def hessian_device(self, collisions, mesh, vertices, project_hessian_to_psd=PSDProjectionMethod.NONE):
        """Like hessian() but the CSR stays on the device (DeviceCSR)."""
        V = _as_f64(vertices)
        h = C.c_void_p()
        _check(_load().ipcg_barrier_hessian(collisions._h, mesh._h, _ptr(V), self.dhat, self.stiffness,
                                            self._options, int(project_hessian_to_psd),
                                            C.byref(h)))
        return DeviceCSR(h, 3 * mesh.num_vertices)

    def energy_gradient_hessian_device(self, collisions, mesh, vertices,
                                       project_hessian_to_psd=PSDProjectionMethod.NONE):
        """Energy (float), gradient (device tensor when vertices is one) and
        a DeviceCSR Hessian from one call; results stay on the device."""
        V = _as_f64(vertices)
        e = np.zeros(1)
        if _is_torch_cuda(V):
            import torch
            g = torch.empty(V.numel(), dtype=torch.float64, device=V.device)
        else:
            g = np.empty(3 * mesh.num_vertices)
        h = C.c_void_p()
        _check(_load().ipcg_barrier_energy_gradient_hessian(
            collisions._h, mesh._h, _ptr(V), self.dhat, self.stiffness, self._options,
            int(project_hessian_to_psd), _ptr(e), _ptr(g), C.byref(h)))
        return float(e[0]), g, DeviceCSR(h, 3 * mesh.num_vertices)

    def energy_gradient_hessian(self, collisions, mesh, vertices, project_hessian_to_psd=PSDProjectionMethod.NONE):
        """Energy, gradient and Hessian from one call."""
        V = _as_f64(vertices)
        e = np.zeros(1)
        g = np.empty(3 * mesh.num_vertices)
        h = C.c_void_p()
        _check(_load().ipcg_barrier_energy_gradient_hessian(
            collisions._h, mesh._h, _ptr(V), self.dhat, self.stiffness, self._options,
            int(project_hessian_to_psd), _ptr(e), _ptr(g), C.byref(h)))
        return float(e[0]), g, _csr_to_scipy(h, 3 * mesh.num_vertices)


class BatchBarrierPotential:
    """BarrierPotential with one dhat and one stiffness per scene of a
    SceneBatch.  Energies come back per scene; the gradient and Hessian are
    the packed ones (block diagonal over scenes).  ``mixed_precision`` as for
    BarrierPotential."""

    def __init__(self, dhat, stiffness, use_physical_barrier: bool = False, mixed_precision=False):
        self.dhat = np.asarray(dhat, np.float64)
        self.stiffness = np.asarray(stiffness, np.float64)
        if not np.all(self.dhat > 0):
            raise ValueError("dhat must be positive")
        self.use_physical_barrier = bool(use_physical_barrier)
        self.mixed_precision = mixed_precision

    @property
    def _options(self):
        return int(self.use_physical_barrier) | _precision_bits(self.mixed_precision)

    def autotune(self, collisions, batch, vertices, project_hessian_to_psd=None) -> dict:
        """Time the launch shapes of the energy / gradient / local Hessian stage
        and of the projection stage on this set and keep the fastest of each
        for the device (ipcg_barrier_autotune)."""
        psd = PSDProjectionMethod.CLAMP if project_hessian_to_psd is None else project_hessian_to_psd
        return autotune_barrier(collisions, batch, vertices, batch.per_scene(self.dhat),
                                batch.per_scene(self.stiffness), self._options, psd)

    def evaluate(self, collisions: NormalCollisions, batch: SceneBatch, vertices, energy=True, gradient=False,
                 hessian=False, project_hessian_to_psd=PSDProjectionMethod.NONE, device=False, out_gradient=None):
        """(energies, gradient or None, Hessian or None) from one call.  With
        ``device`` the Hessian is a DeviceCSR, else a scipy matrix.
        ``out_gradient`` (with ``gradient``): the array the gradient is written
        to and returned as -- 3 x vertices float64 values, contiguous: a host
        array (page-locked memory, e.g. a pinned torch tensor's ``.numpy()``,
        makes the copy out fastest) or a CUDA tensor; by default a new array
        of the same kind as ``vertices``."""
        V = _as_f64(vertices)
        dh, kap = batch.per_scene(self.dhat), batch.per_scene(self.stiffness)
        e = np.zeros(batch.num_scenes) if energy else None
        g = None
        if gradient:
            n = 3 * batch.num_vertices
            if out_gradient is not None:
                g = out_gradient
                if _is_torch_cuda(g):
                    import torch
                    ok = g.dtype == torch.float64 and g.is_contiguous() and g.numel() == n
                else:
                    ok = (isinstance(g, np.ndarray) and g.dtype == np.float64 and g.flags.c_contiguous
                          and g.flags.writeable and g.size == n)
                if not ok:
                    raise ValueError(f"out_gradient must be a contiguous, writable float64 array of {n} values")
            elif _is_torch_cuda(V):
                import torch
                g = torch.empty(V.numel(), dtype=torch.float64, device=V.device)
            else:
                g = np.zeros(n)
        h = C.c_void_p()
        _check(_load().ipcg_barrier_batch(collisions._h, batch._h, _ptr(V), _ptr(dh), _ptr(kap),
                                          self._options, int(project_hessian_to_psd), _ptr(e),
                                          _ptr(g), C.byref(h) if hessian else None))
        H = None
        if hessian:
            H = DeviceCSR(h, 3 * batch.num_vertices) if device else _csr_to_scipy(h, 3 * batch.num_vertices)
        return e, g, H

    def __call__(self, collisions, batch, vertices):
        return self.evaluate(collisions, batch, vertices)[0]

    def gradient(self, collisions, batch, vertices):
        return self.evaluate(collisions, batch, vertices, energy=False, gradient=True)[1]

    def hessian(self, collisions, batch, vertices, project_hessian_to_psd=PSDProjectionMethod.NONE):
        return self.evaluate(collisions, batch, vertices, energy=False, hessian=True,
                             project_hessian_to_psd=project_hessian_to_psd)[2]


class TightInclusionCCD:
    """TightInclusionCCD(tolerance, max_iterations, conservative_rescaling)
    (src/ipc/ccd/tight_inclusion_ccd.hpp:11-28)."""
    DEFAULT_TOLERANCE = 1e-6
    DEFAULT_MAX_ITERATIONS = 10_000_000
    DEFAULT_CONSERVATIVE_RESCALING = 0.8
    SMALL_TOI = 1e-6

    def __init__(self, tolerance=DEFAULT_TOLERANCE, max_iterations=DEFAULT_MAX_ITERATIONS,
                 conservative_rescaling=DEFAULT_CONSERVATIVE_RESCALING):
        self.tolerance = float(tolerance)
        self.max_iterations = int(max_iterations)
        self.conservative_rescaling = float(conservative_rescaling)

    def _batch(self, is_ee, x0, x1, min_distance, tmax):
        x0 = np.ascontiguousarray(x0, np.float64).reshape(-1, 4, 3)
        x1 = np.ascontiguousarray(x1, np.float64).reshape(-1, 4, 3)
        n = x0.shape[0]
        hit = np.zeros(n, np.int8)
        toi = np.zeros(n)
        _check(_load().ipcg_ccd_stencils(int(is_ee), n, _ptr(x0), _ptr(x1), float(min_distance), float(tmax),
                                         self.tolerance, self.max_iterations, self.conservative_rescaling,
                                         _ptr(hit), _ptr(toi)))
        return hit.astype(bool), toi

    def point_triangle_ccd(self, p_t0, t0_t0, t1_t0, t2_t0, p_t1, t0_t1, t1_t1, t2_t1, min_distance=0.0, tmax=1.0):
        hit, toi = self._batch(False, np.stack([p_t0, t0_t0, t1_t0, t2_t0]), np.stack([p_t1, t0_t1, t1_t1, t2_t1]),
                               min_distance, tmax)
        return bool(hit[0]), float(toi[0])

    def edge_edge_ccd(self, ea0_t0, ea1_t0, eb0_t0, eb1_t0, ea0_t1, ea1_t1, eb0_t1, eb1_t1, min_distance=0.0,
                      tmax=1.0):
        hit, toi = self._batch(True, np.stack([ea0_t0, ea1_t0, eb0_t0, eb1_t0]),
                               np.stack([ea0_t1, ea1_t1, eb0_t1, eb1_t1]), min_distance, tmax)
        return bool(hit[0]), float(toi[0])

    def point_edge_ccd(self, p_t0, e0_t0, e1_t0, p_t1, e0_t1, e1_t1, min_distance=0.0, tmax=1.0):
        """Degenerate edge-edge, as tight_inclusion_ccd.cpp:171-180."""
        return self.edge_edge_ccd(p_t0, p_t0, e0_t0, e1_t0, p_t1, p_t1, e0_t1, e1_t1, min_distance, tmax)

    def point_point_ccd(self, p0_t0, p1_t0, p0_t1, p1_t1, min_distance=0.0, tmax=1.0):
        """Degenerate edge-edge, as tight_inclusion_ccd.cpp:98-107."""
        return self.edge_edge_ccd(p0_t0, p0_t0, p1_t0, p1_t0, p0_t1, p0_t1, p1_t1, p1_t1, min_distance, tmax)


DEFAULT_NARROW_PHASE_CCD = TightInclusionCCD()


def compute_collision_free_stepsize(mesh: CollisionMesh, vertices_t0, vertices_t1, min_distance: float = 0.0,
                                    broad_phase=None, narrow_phase_ccd: TightInclusionCCD = DEFAULT_NARROW_PHASE_CCD):
    """src/ipc/ipc.hpp:41-47.  ``broad_phase`` is accepted for API
    compatibility; the device LBVH is always used."""
    V0, V1 = _as_f64(vertices_t0), _as_f64(vertices_t1)
    step = np.zeros(1)
    _check(_load().ipcg_collision_free_stepsize(
        mesh._h, _ptr(V0), _ptr(V1), float(min_distance), narrow_phase_ccd.tolerance,
        narrow_phase_ccd.max_iterations, narrow_phase_ccd.conservative_rescaling, _ptr(step), None))
    return float(step[0])


class RequestResult(C.Structure):
    """ipcg_request_result (include/ipcg.h)."""
    _fields_ = [("status", C.c_int), ("kind", C.c_int), ("energy", C.c_double), ("step", C.c_double),
                ("contacts", C.c_int64), ("t_submit_ns", C.c_int64), ("t_start_ns", C.c_int64),
                ("t_end_ns", C.c_int64)]


class Server:
    """Request loop over resident scenes (ipcg_server_*): barrier requests
    (collision set rebuilt at the given positions, then energy, gradient and
    Hessian) and step-size requests from many simulations, run concurrently
    on their scenes' streams under an HBM admission budget."""

    def __init__(self, workers: int = 4, hbm_budget_bytes: float = 120e9):
        h = C.c_void_p()
        _check(_load().ipcg_server_create(int(workers), int(hbm_budget_bytes), C.byref(h)))
        self._h = h
        self._scenes = []
        self._tickets = {}

    def close(self):
        h = getattr(self, "_h", None)
        if h and _lib is not None:
            _lib.ipcg_server_destroy(h)
            self._h = None

    def __del__(self):
        self.close()

    def add_scene(self, mesh: CollisionMesh, collisions: NormalCollisions, dhat: float, dmin: float = 0.0,
                  stiffness: float = 1.0) -> int:
        sid = C.c_int64()
        _check(_load().ipcg_server_add_scene(self._h, mesh._h, collisions._h, float(dhat), float(dmin),
                                             float(stiffness), C.byref(sid)))
        self._scenes.append((mesh, collisions))  # keep them alive
        return sid.value

    def set_scene_options(self, scene: int, use_physical_barrier: bool = False, mixed_precision=False):
        """ipcg_server_set_scene_options: the physical scaling and mixed
        precision mode (as for BarrierPotential) of a scene's barrier
        requests."""
        bits = int(bool(use_physical_barrier)) | _precision_bits(mixed_precision)
        _check(_load().ipcg_server_set_scene_options(self._h, int(scene), bits))

    def submit_barrier(self, scene: int, vertices, project_hessian_to_psd=PSDProjectionMethod.CLAMP) -> int:
        V = np.ascontiguousarray(vertices, np.float64)
        t = C.c_int64()
        _check(_load().ipcg_server_submit_barrier(self._h, int(scene), _ptr(V), int(project_hessian_to_psd),
                                                  C.byref(t)))
        self._tickets[t.value] = int(scene)
        return t.value

    def submit_stepsize(self, scene: int, vertices_t0, vertices_t1, min_distance: float = 0.0) -> int:
        V0 = np.ascontiguousarray(vertices_t0, np.float64)
        V1 = np.ascontiguousarray(vertices_t1, np.float64)
        t = C.c_int64()
        _check(_load().ipcg_server_submit_stepsize(self._h, int(scene), _ptr(V0), _ptr(V1), float(min_distance),
                                                   C.byref(t)))
        self._tickets[t.value] = int(scene)
        return t.value

    def wait(self, ticket: int, gradient: bool = False, hessian: str | None = None):
        """Blocks for a request; returns a dict with energy / step, contacts,
        times (ns) and, on request, the gradient (numpy) and the Hessian
        ("device": DeviceCSR, "scipy": scipy matrix)."""
        scene = self._tickets.pop(int(ticket), None)
        if scene is None:
            raise ValueError("unknown ticket")
        ndof = 3 * self._scenes[scene][0].num_vertices
        res = RequestResult()
        gbuf = np.zeros(ndof) if gradient else None
        h = C.c_void_p()
        _check(_load().ipcg_server_wait(self._h, int(ticket), C.byref(res), _ptr(gbuf),
                                        C.byref(h) if hessian else None))
        out = {"kind": res.kind, "energy": res.energy, "step": res.step, "contacts": res.contacts,
               "t_submit_ns": res.t_submit_ns, "t_start_ns": res.t_start_ns, "t_end_ns": res.t_end_ns}
        if gradient:
            out["gradient"] = gbuf
        if hessian == "device":
            out["hessian"] = DeviceCSR(h, ndof)
        elif hessian:
            out["hessian"] = _csr_to_scipy(h, ndof)
        return out

    def stats(self) -> dict:
        st = np.zeros(5, np.int64)
        _check(_load().ipcg_server_stats(self._h, _ptr(st)))
        return {"completed": int(st[0]), "queued": int(st[1]), "running": int(st[2]), "releases": int(st[3]),
                "resident_bytes": int(st[4])}


class TangentialCollisions:
    """TangentialCollisions (src/ipc/collisions/tangential/tangential_collisions.hpp),
    isotropic, built from a NormalCollisions set on the device."""

    def __init__(self):
        h = C.c_void_p()
        _check(_load().ipcg_tangential_create(C.byref(h)))
        self._h = h
        self._mesh = None

    def __del__(self):
        h = getattr(self, "_h", None)
        if h and _lib is not None:
            _lib.ipcg_tangential_destroy(h)
            self._h = None

    def build(self, mesh: CollisionMesh, vertices, collisions: NormalCollisions, normal_potential, mu_s, mu_k=None):
        """tangential_collisions.cpp:60-170; mu_s / mu_k scalars or per-vertex
        arrays (mu_k defaults to mu_s)."""
        V = _as_f64(vertices)
        nV = mesh.num_vertices
        ms = np.ascontiguousarray(np.broadcast_to(np.asarray(mu_s, np.float64), (nV,)))
        mk = np.ascontiguousarray(np.broadcast_to(np.asarray(mu_s if mu_k is None else mu_k, np.float64), (nV,)))
        if isinstance(mesh, SceneBatch):
            # a BatchBarrierPotential (or any potential): one dhat / stiffness per scene
            dh = mesh.per_scene(normal_potential.dhat)
            kap = mesh.per_scene(normal_potential.stiffness)
            opts = int(getattr(normal_potential, "use_physical_barrier", False))
            _check(_load().ipcg_tangential_build_batch(self._h, mesh._h, _ptr(V), collisions._h, _ptr(dh),
                                                       _ptr(kap), opts, _ptr(ms), _ptr(mk)))
        else:
            _check(_load().ipcg_tangential_build(self._h, mesh._h, _ptr(V), collisions._h, normal_potential.dhat,
                                                 normal_potential.stiffness, normal_potential._options, _ptr(ms),
                                                 _ptr(mk)))
        self._mesh = mesh

    def counts(self):
        c = np.zeros(4, np.int64)
        _check(_load().ipcg_tangential_counts(self._h, _ptr(c)))
        return c

    def set_anisotropy(self, mu_aniso=None, mu_s_aniso=None, mu_k_aniso=None):
        """Per-collision (n, 2) arrays: the slip scaling and the directional
        static / kinetic coefficients (None restores the isotropic default)."""
        n = len(self)
        arrs = [None if a is None else np.ascontiguousarray(np.broadcast_to(np.asarray(a, np.float64), (n, 2)))
                for a in (mu_aniso, mu_s_aniso, mu_k_aniso)]
        _check(_load().ipcg_tangential_set_anisotropy(self._h, *[None if a is None else _ptr(a) for a in arrs]))

    def update_lagged_anisotropic_friction_coefficients(self, mesh, rest_positions, lagged_displacements,
                                                        velocities):
        """tangential_collisions.cpp:387-420."""
        R, L, U = _as_f64(rest_positions), _as_f64(lagged_displacements), _as_f64(velocities)
        _check(_load().ipcg_tangential_update_lagged_mu(self._h, mesh._h, _ptr(R), _ptr(L), _ptr(U)))

    def reset_lagged_anisotropic_friction_coefficients(self):
        _check(_load().ipcg_tangential_reset_lagged_mu(self._h))

    def lagged_mu(self):
        """(mu_s_effective, mu_k_effective) per collision."""
        n = len(self)
        ms, mk = np.zeros(n), np.zeros(n)
        _check(_load().ipcg_tangential_lagged_mu(self._h, _ptr(ms), _ptr(mk)))
        return ms, mk

    def __len__(self):
        return int(self.counts().sum())

    def to_arrays(self):
        """dict: vv, ev, ee, fv stencils; per collision weight, normal_force,
        closest_point (n, 2), tangent_basis (n, 3, 2), mu_s, mu_k."""
        nvv, nev, nee, nfv = (int(x) for x in self.counts())
        n = nvv + nev + nee + nfv
        out = {k: np.zeros((m, 2), np.int32) for k, m in (("vv", nvv), ("ev", nev), ("ee", nee), ("fv", nfv))}
        w, N, mus, muk = np.zeros(n), np.zeros(n), np.zeros(n), np.zeros(n)
        cp, P = np.zeros((n, 2)), np.zeros((n, 6))
        _check(_load().ipcg_tangential_get(self._h, _ptr(out["vv"]), _ptr(out["ev"]), _ptr(out["ee"]),
                                           _ptr(out["fv"]), _ptr(w), _ptr(N), _ptr(cp), _ptr(P), _ptr(mus),
                                           _ptr(muk)))
        out.update(weight=w, normal_force=N, closest_point=cp, tangent_basis=P.reshape(n, 2, 3).transpose(0, 2, 1),
                   mu_s=mus, mu_k=muk)
        return out


class FrictionPotential:
    """FrictionPotential(eps_v) (src/ipc/potentials/friction_potential.hpp):
    energy, gradient and Hessian of the lagged smooth friction at velocities."""

    def __init__(self, eps_v: float):
        if not eps_v > 0:
            raise ValueError("eps_v must be positive")
        self.eps_v = float(eps_v)

    def _call(self, collisions, mesh, velocities, psd, e=None, g=None, h=None):
        U = _as_f64(velocities)
        fn = _load().ipcg_friction_potential_batch if isinstance(mesh, SceneBatch) else _load().ipcg_friction_potential
        _check(fn(collisions._h, mesh._h, _ptr(U), self.eps_v, int(psd), _ptr(e) if e is not None else None,
                  _ptr(g) if g is not None else None, C.byref(h) if h is not None else None))

    def __call__(self, collisions: TangentialCollisions, mesh: CollisionMesh, velocities):
        """The friction energy (on a SceneBatch: one energy per scene)."""
        batch = isinstance(mesh, SceneBatch)
        e = np.zeros(mesh.num_scenes if batch else 1)
        self._call(collisions, mesh, velocities, 0, e=e)
        return e if batch else float(e[0])

    def gradient(self, collisions, mesh, velocities):
        U = _as_f64(velocities)
        if _is_torch_cuda(U):
            import torch
            g = torch.empty(U.numel(), dtype=torch.float64, device=U.device)
        else:
            g = np.empty(3 * mesh.num_vertices)
        self._call(collisions, mesh, U, 0, g=g)
        return g

    def hessian(self, collisions, mesh, velocities, project_hessian_to_psd=PSDProjectionMethod.NONE):
        h = C.c_void_p()
        self._call(collisions, mesh, velocities, int(project_hessian_to_psd), h=h)
        return _csr_to_scipy(h, 3 * mesh.num_vertices)

    def force(self, collisions, mesh, rest_positions, lagged_displacements, velocities, normal_potential,
              dmin: float = 0.0, no_mu: bool = False):
        """TangentialPotential::force (tangential_potential.cpp:40-77)."""
        R, L, U = _as_f64(rest_positions), _as_f64(lagged_displacements), _as_f64(velocities)
        out = np.empty(3 * mesh.num_vertices)
        _check(_load().ipcg_friction_force(collisions._h, mesh._h, _ptr(R), _ptr(L), _ptr(U), normal_potential.dhat,
                                           normal_potential.stiffness, normal_potential._options & ~2, float(dmin),
                                           self.eps_v, int(bool(no_mu)), _ptr(out)))
        return out

    def energy_gradient_hessian(self, collisions, mesh, velocities, project_hessian_to_psd=PSDProjectionMethod.NONE):
        """Energy, gradient and Hessian from one call (velocities staged once)."""
        U = _as_f64(velocities)
        batch = isinstance(mesh, SceneBatch)
        e = np.zeros(mesh.num_scenes if batch else 1)
        if _is_torch_cuda(U):
            import torch
            g = torch.empty(U.numel(), dtype=torch.float64, device=U.device)
        else:
            g = np.empty(3 * mesh.num_vertices)
        h = C.c_void_p()
        self._call(collisions, mesh, U, int(project_hessian_to_psd), e=e, g=g, h=h)
        return (e if batch else float(e[0])), g, _csr_to_scipy(h, 3 * mesh.num_vertices)


class Candidates:
    """Candidates (src/ipc/candidates/candidates.hpp): a broad-phase candidate
    set kept on the device (edge-edge and face-vertex pairs, 3D meshes) and
    the step-size rules that read it."""

    def __init__(self):
        h = C.c_void_p()
        _check(_load().ipcg_candidates_create(C.byref(h)))
        self._h = h

    def __del__(self):
        h = getattr(self, "_h", None)
        if h and _lib is not None:
            _lib.ipcg_candidates_destroy(h)
            self._h = None

    def build(self, mesh: CollisionMesh, vertices_t0, vertices_t1=None, inflation_radius: float = 0.0,
              broad_phase=None):
        """candidates.cpp:43-125 (static) or, with vertices_t1, 128-222 (swept)."""
        V0 = _as_f64(vertices_t0)
        if vertices_t1 is None:
            _check(_load().ipcg_candidates_build(self._h, mesh._h, _ptr(V0), float(inflation_radius)))
        else:
            V1 = _as_f64(vertices_t1)
            _check(_load().ipcg_candidates_build_swept(self._h, mesh._h, _ptr(V0), _ptr(V1),
                                                       float(inflation_radius)))

    def counts(self):
        c = np.zeros(2, np.int64)
        _check(_load().ipcg_candidates_counts(self._h, _ptr(c)))
        return c

    def __len__(self):
        return int(self.counts().sum())

    def to_arrays(self):
        n = self.counts()
        ee = np.zeros((int(n[0]), 2), np.int32)
        fv = np.zeros((int(n[1]), 2), np.int32)
        _check(_load().ipcg_candidates_get(self._h, _ptr(ee), _ptr(fv)))
        return ee, fv

    def compute_per_vertex_safe_distances(self, mesh: CollisionMesh, vertices, inflation_radius: float,
                                          min_distance: float = 0.0):
        V = _as_f64(vertices)
        out = np.zeros(mesh.num_vertices)
        _check(_load().ipcg_candidates_per_vertex_safe_distances(self._h, mesh._h, _ptr(V), float(inflation_radius),
                                                                 float(min_distance), _ptr(out)))
        return out

    def compute_collision_free_stepsize(self, mesh: CollisionMesh, vertices_t0, vertices_t1,
                                        min_distance: float = 0.0,
                                        narrow_phase_ccd: TightInclusionCCD = DEFAULT_NARROW_PHASE_CCD) -> float:
        V0, V1 = _as_f64(vertices_t0), _as_f64(vertices_t1)
        out = np.zeros(1)
        _check(_load().ipcg_candidates_collision_free_stepsize(
            self._h, mesh._h, _ptr(V0), _ptr(V1), float(min_distance), narrow_phase_ccd.tolerance,
            narrow_phase_ccd.max_iterations, narrow_phase_ccd.conservative_rescaling, _ptr(out)))
        return float(out[0])

    def compute_noncandidate_conservative_stepsize(self, mesh: CollisionMesh, displacements, dhat: float) -> float:
        U = _as_f64(displacements)
        out = np.zeros(1)
        _check(_load().ipcg_candidates_noncandidate_conservative_stepsize(self._h, mesh._h, _ptr(U), float(dhat),
                                                                          _ptr(out)))
        return float(out[0])

    def compute_cfl_stepsize(self, mesh: CollisionMesh, vertices_t0, vertices_t1, dhat: float,
                             min_distance: float = 0.0, broad_phase=None,
                             narrow_phase_ccd: TightInclusionCCD = DEFAULT_NARROW_PHASE_CCD) -> float:
        V0, V1 = _as_f64(vertices_t0), _as_f64(vertices_t1)
        out = np.zeros(1)
        _check(_load().ipcg_candidates_cfl_stepsize(
            self._h, mesh._h, _ptr(V0), _ptr(V1), float(dhat), float(min_distance), narrow_phase_ccd.tolerance,
            narrow_phase_ccd.max_iterations, narrow_phase_ccd.conservative_rescaling, _ptr(out)))
        return float(out[0])


def initial_barrier_stiffness(bbox_diagonal: float, dhat: float, average_mass: float, grad_energy, grad_barrier,
                              min_barrier_stiffness_scale: float = 1e11, dmin: float = 0.0, barrier=None):
    """barrier/adaptive_stiffness.cpp:12-48 (ipcg_initial_barrier_stiffness):
    returns (kappa, max_barrier_stiffness).  The gradients may be numpy
    arrays or CUDA tensors (the two dot products run where they live);
    ``barrier`` defaults to ClampedLogBarrier."""
    ge, gb = _as_f64_vec(grad_energy), _as_f64_vec(grad_barrier)
    n = int(ge.shape[0])
    if int(gb.shape[0]) != n:
        raise ValueError("grad_energy and grad_barrier must have the same size")
    kind = 0 if barrier is None else int(barrier.kind)
    k, kmax = C.c_double(), C.c_double()
    _check(_load().ipcg_initial_barrier_stiffness(float(bbox_diagonal), kind, float(dhat), float(average_mass),
                                                  _ptr(ge), _ptr(gb), n, float(min_barrier_stiffness_scale),
                                                  float(dmin), C.byref(k), C.byref(kmax)))
    return k.value, kmax.value


def update_barrier_stiffness(prev_min_distance: float, min_distance: float, max_barrier_stiffness: float,
                             barrier_stiffness: float, bbox_diagonal: float, dhat_epsilon_scale: float = 1e-9,
                             dmin: float = 0.0) -> float:
    """barrier/adaptive_stiffness.cpp:51-68 (ipcg_update_barrier_stiffness):
    double the stiffness (up to the maximum) while the minimum distance keeps
    shrinking below (dhat_epsilon_scale (bbox_diagonal + dmin))^2."""
    out = C.c_double()
    _check(_load().ipcg_update_barrier_stiffness(float(prev_min_distance), float(min_distance),
                                                 float(max_barrier_stiffness), float(barrier_stiffness),
                                                 float(bbox_diagonal), float(dhat_epsilon_scale), float(dmin),
                                                 C.byref(out)))
    return out.value


def is_step_collision_free(mesh: CollisionMesh, vertices_t0, vertices_t1, min_distance: float = 0.0,
                           broad_phase=None, narrow_phase_ccd: TightInclusionCCD = DEFAULT_NARROW_PHASE_CCD) -> bool:
    """ipc.hpp is_step_collision_free (ipc.cpp:20-40)."""
    V0, V1 = _as_f64(vertices_t0), _as_f64(vertices_t1)
    out = np.zeros(1, np.int32)
    _check(_load().ipcg_is_step_collision_free(
        mesh._h, _ptr(V0), _ptr(V1), float(min_distance), narrow_phase_ccd.tolerance,
        narrow_phase_ccd.max_iterations, narrow_phase_ccd.conservative_rescaling, _ptr(out)))
    return bool(out[0])


def has_intersections(mesh: CollisionMesh, vertices, broad_phase=None) -> bool:
    """ipc.hpp has_intersections (ipc.cpp:110-167), 3D meshes."""
    V = _as_f64(vertices)
    out = np.zeros(1, np.int32)
    _check(_load().ipcg_has_intersections(mesh._h, _ptr(V), _ptr(out)))
    return bool(out[0])


def compute_collision_free_stepsize_batch(batch: SceneBatch, vertices_t0, vertices_t1, min_distance=0.0,
                                          narrow_phase_ccd: TightInclusionCCD = DEFAULT_NARROW_PHASE_CCD):
    """compute_collision_free_stepsize on every scene of a SceneBatch: one
    step per scene (equal to the scene's own call)."""
    V0, V1 = _as_f64(vertices_t0), _as_f64(vertices_t1)
    md = batch.per_scene(min_distance)
    steps = np.zeros(batch.num_scenes)
    _check(_load().ipcg_collision_free_stepsize_batch(
        batch._h, _ptr(V0), _ptr(V1), _ptr(md), narrow_phase_ccd.tolerance, narrow_phase_ccd.max_iterations,
        narrow_phase_ccd.conservative_rescaling, _ptr(steps), None))
    return steps


def distance_stencils(kind: int, x):
    """Batched distance types + squared distances (kind 0 point-edge, 1
    point-triangle, 2 edge-edge) computed on the device."""
    per = 3 if kind == 0 else 4
    x = np.ascontiguousarray(x, np.float64).reshape(-1, per, 3)
    n = x.shape[0]
    dt = np.zeros(n, np.int8)
    d = np.zeros(n)
    _check(_load().ipcg_distance_stencils(int(kind), n, _ptr(x), _ptr(dt), _ptr(d)))
    return dt, d


def edges(F):
    """Unique undirected edges of a triangle mesh (like igl::edges)."""
    return scenes.edges_from_faces(np.asarray(F))


# -- the reference's free distance functions (src/ipc/distance/*.hpp), with
#    the classified (AUTO) type, on the device; arguments may be single points
#    or stacked (n, 3) arrays, results scalars or (n,) arrays --

def _stencil(kind, pts, _unused=None):
    X = np.stack([np.asarray(q, np.float64).reshape(-1, 3) for q in pts], axis=1)
    dt, d = distance_stencils(kind, X)
    single = all(np.asarray(q).ndim == 1 for q in pts)
    return (dt[0], d[0]) if single else (dt, d)


def _auto_only(dtype):
    if dtype is not None and int(dtype) != -1:
        raise ValueError("only the classified (AUTO) distance type is provided by these free functions")


def point_point_distance(p0, p1):
    """point_point.hpp: squared distance (a degenerate edge on the device)."""
    return _stencil(0, (p0, p1, p1), None)[1]


def point_edge_distance(p, e0, e1, dtype=None):
    """point_edge.hpp: squared distance with the classified type."""
    _auto_only(dtype)
    return _stencil(0, (p, e0, e1), None)[1]


def point_triangle_distance(p, t0, t1, t2, dtype=None):
    """point_triangle.hpp: squared distance with the classified type."""
    _auto_only(dtype)
    return _stencil(1, (p, t0, t1, t2), None)[1]


def edge_edge_distance(ea0, ea1, eb0, eb1, dtype=None):
    """edge_edge.hpp: squared distance with the classified type."""
    _auto_only(dtype)
    return _stencil(2, (ea0, ea1, eb0, eb1), None)[1]


def point_edge_distance_type(p, e0, e1):
    t = _stencil(0, (p, e0, e1), None)[0]
    return PointEdgeDistanceType(int(t)) if np.ndim(t) == 0 else t


def point_triangle_distance_type(p, t0, t1, t2):
    t = _stencil(1, (p, t0, t1, t2), None)[0]
    return PointTriangleDistanceType(int(t)) if np.ndim(t) == 0 else t


def edge_edge_distance_type(ea0, ea1, eb0, eb1):
    t = _stencil(2, (ea0, ea1, eb0, eb1), None)[0]
    return EdgeEdgeDistanceType(int(t)) if np.ndim(t) == 0 else t


# -- barrier.hpp's free functions (the clamped log barrier) --

def barrier(d: float, dhat: float) -> float:
    return ClampedLogBarrier()(d, dhat)


def barrier_first_derivative(d: float, dhat: float) -> float:
    return ClampedLogBarrier().first_derivative(d, dhat)


def barrier_second_derivative(d: float, dhat: float) -> float:
    return ClampedLogBarrier().second_derivative(d, dhat)


__all__ = [
    "CollisionMesh", "SceneBatch", "NormalCollisions", "TangentialCollisions", "Candidates", "BarrierPotential",
    "BatchBarrierPotential", "FrictionPotential", "Barrier", "ClampedLogBarrier", "NormalizedClampedLogBarrier",
    "ClampedLogSqBarrier", "CubicBarrier", "TwoStageBarrier", "PSDProjectionMethod", "TightInclusionCCD",
    "DEFAULT_NARROW_PHASE_CCD", "compute_collision_free_stepsize", "compute_collision_free_stepsize_batch",
    "is_step_collision_free", "has_intersections", "initial_barrier_stiffness", "update_barrier_stiffness",
    "EdgeEdgeDistanceType", "PointTriangleDistanceType", "PointEdgeDistanceType", "point_point_distance",
    "point_edge_distance", "point_triangle_distance", "edge_edge_distance", "point_edge_distance_type",
    "point_triangle_distance_type", "edge_edge_distance_type", "barrier", "barrier_first_derivative",
    "barrier_second_derivative", "distance_stencils", "edges", "Server", "RequestResult", "DeviceCSR", "lib",
    "LIB_PATH", "profile_enable", "profile_report", "launch_count", "set_hessian_chunk_contacts",
]
