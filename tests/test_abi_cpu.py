"""Host-side checks of the C ABI that need no GPU: the library loads, exports
every entry point declared in include/ipcg.h, and refuses to compute (with
IPCG_ERR_NO_DEVICE, never a CPU fallback) when no CUDA device is present."""
import ctypes as C
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    txt = open(os.path.join(ROOT, "include", "ipcg.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(ipcg_\w+)\s*\(", txt)))


def test_header_declares_the_hot_path():
    syms = declared_symbols()
    for s in ("ipcg_mesh_create", "ipcg_collisions_build", "ipcg_barrier_energy", "ipcg_barrier_gradient",
              "ipcg_barrier_hessian", "ipcg_collision_free_stepsize"):
        assert s in syms


def test_library_exports_every_declared_symbol(ipctk):
    lib = C.CDLL(ipctk.LIB_PATH)
    missing = [s for s in declared_symbols() if not hasattr(lib, s)]
    assert not missing, missing


def test_version_and_error_strings(ipctk):
    L = ipctk.lib()
    assert L.ipcg_version().decode().startswith("ipcg")
    assert L.ipcg_last_error() is not None


def _has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.mark.skipif(_has_gpu(), reason="checks the no-device path")
def test_no_device_fails_loudly(ipctk):
    V = np.zeros((3, 3))
    E = np.array([[0, 1], [1, 2], [2, 0]])
    F = np.array([[0, 1, 2]])
    with pytest.raises(RuntimeError, match="no CUDA device"):
        ipctk.CollisionMesh(V, E, F)
    x = np.zeros((1, 4, 3))
    with pytest.raises(RuntimeError, match="no CUDA device"):
        ipctk.distance_stencils(1, x)


def test_argument_validation_precedes_device(ipctk):
    # invalid sizes are rejected as invalid arguments, before any device work
    L = ipctk.lib()
    h = C.c_void_p()
    st = L.ipcg_mesh_create(None, -1, None, 0, None, 0, C.byref(h))
    assert st == 1
    assert "negative" in L.ipcg_last_error().decode()


def test_server_argument_validation_without_gpu(ipctk):
    """The request server's arguments are checked before any device work."""
    L = C.CDLL(ipctk.LIB_PATH)
    L.ipcg_last_error.restype = C.c_char_p
    h = C.c_void_p()
    L.ipcg_server_create.restype = C.c_int
    L.ipcg_server_create.argtypes = [C.c_int, C.c_int64, C.POINTER(C.c_void_p)]
    assert L.ipcg_server_create(0, 1 << 30, C.byref(h)) == 1
    assert L.ipcg_server_create(2, 0, C.byref(h)) == 1
    assert L.ipcg_server_create(2, 1 << 30, None) == 1
    assert L.ipcg_server_create(2, 1 << 30, C.byref(h)) == 0
    L.ipcg_server_submit_barrier.restype = C.c_int
    L.ipcg_server_submit_barrier.argtypes = [C.c_void_p, C.c_int64, C.c_void_p, C.c_int, C.POINTER(C.c_int64)]
    t = C.c_int64()
    assert L.ipcg_server_submit_barrier(h, 0, None, 1, C.byref(t)) == 1  # no scene registered
    assert b"unknown scene" in L.ipcg_last_error()
    L.ipcg_server_destroy.argtypes = [C.c_void_p]
    assert L.ipcg_server_destroy(h) == 0


def test_adaptive_stiffness_formulas(ipctk):
    """initial/update_barrier_stiffness (barrier/adaptive_stiffness.cpp:12-68)
    on hand-checked values."""
    import math
    dhat, diag, mass = 1e-3, 2.0, 0.5
    d0 = (1e-8 * diag) ** 2
    r = dhat * dhat / d0
    b2 = (r + 2) * r - 2 * math.log(d0 / (dhat * dhat)) - 3
    kmin = 1e11 * mass / (4 * d0 * b2)
    gE = np.array([1.0, -2.0, 0.5])
    gB = np.array([-0.5, 1.0, 0.0])
    kappa, kmax = ipctk.initial_barrier_stiffness(diag, dhat, mass, gE, gB)
    assert math.isclose(kmax, 100 * kmin, rel_tol=1e-14)
    k_raw = -(gB @ gE) / (gB @ gB)
    assert kappa == min(max(k_raw, kmin), kmax)
    eps = (1e-9 * diag) ** 2
    assert ipctk.update_barrier_stiffness(0.5 * eps, 0.25 * eps, 10.0, 3.0, diag) == 6.0
    assert ipctk.update_barrier_stiffness(0.5 * eps, 0.25 * eps, 5.0, 3.0, diag) == 5.0
    assert ipctk.update_barrier_stiffness(0.25 * eps, 0.5 * eps, 10.0, 3.0, diag) == 3.0


def test_collision_set_type_validation_without_gpu(ipctk):
    """OGC is not provided and is rejected; the setters touch no device."""
    L = C.CDLL(ipctk.LIB_PATH)
    L.ipcg_last_error.restype = C.c_char_p
    h = C.c_void_p()
    assert L.ipcg_collisions_create(C.byref(h)) == 0
    L.ipcg_collisions_set_collision_set_type.argtypes = [C.c_void_p, C.c_int]
    L.ipcg_collisions_collision_set_type.argtypes = [C.c_void_p, C.POINTER(C.c_int)]
    assert L.ipcg_collisions_set_collision_set_type(h, 2) == 1
    assert b"collision set type" in L.ipcg_last_error()
    assert L.ipcg_collisions_set_collision_set_type(h, 1) == 0
    t = C.c_int()
    assert L.ipcg_collisions_collision_set_type(h, C.byref(t)) == 0 and t.value == 1
    L.ipcg_collisions_destroy.argtypes = [C.c_void_p]
    assert L.ipcg_collisions_destroy(h) == 0


def test_public_names(ipctk):
    """Every name the package exports exists (the reference's ipctk names the
    path uses: classes, free functions, enums)."""
    missing = [n for n in ipctk.__all__ if not hasattr(ipctk, n)]
    assert not missing, missing
    for n in ("CollisionMesh", "NormalCollisions", "BarrierPotential", "FrictionPotential", "TangentialCollisions",
              "Candidates", "compute_collision_free_stepsize", "is_step_collision_free", "has_intersections",
              "point_triangle_distance", "edge_edge_distance", "barrier"):
        assert n in ipctk.__all__
