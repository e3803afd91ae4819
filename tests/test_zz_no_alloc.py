"""The allocation-free barrier energy (ipcg_barrier_energy_noalloc).

Some callers of this library cannot let it allocate device memory during a
call: simulation codes that hand all device memory to their own pool under a
hard budget, or that cannot afford cudaMalloc/cudaFree synchronising the
device under their other streams.  For them the library offers an energy
evaluation whose only scratch (the reduction's partial sums) lives in a
static device array, with every input and the output in caller-owned device
memory.  These tests call that entry point through the C ABI: twice in a row
on two different collision sets (the second one smaller, so stale partial
sums left by the first call in the shared array must not leak into the
second), with and without a minimum distance and the physical scaling, each
result checked against the regular ipcg_barrier_energy within the 1e-10
relative tolerance used by the other parity tests; an empty set; a count
beyond the limit (rejected on the host); and a contact whose face index is
out of range (checked on the device: the energy comes back NaN).

The file name sorts last so that a run stopping at the first failure has
already run every other test; the test also passes alone in a fresh process.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

REL = 1e-10


def _bind(lib):
    fn = lib.ipcg_barrier_energy_noalloc
    P, i64, d = C.c_void_p, C.c_int64, C.c_double
    fn.restype = C.c_int
    fn.argtypes = [P, i64, P, i64, P, i64,
                   i64, P, P, i64, P, P, i64, P, P, P, P, i64, P, P,
                   d, d, d, C.c_int, P, P]
    return fn


def _dev(x, dtype):
    import torch
    return torch.as_tensor(np.ascontiguousarray(x), dtype=dtype, device=torch.device("cuda", 0))


def _call(ipctk, V, E, F, a, dhat, kappa, dmin, physical, counts=None):
    """One call through the C ABI; returns (status, energy).  `counts`
    overrides the contact counts passed (the arrays stay as given)."""
    import torch
    out = torch.full((1,), float("nan"), dtype=torch.float64, device=torch.device("cuda", 0))
    p = lambda x: C.c_void_p(x.data_ptr()) if x.numel() else None
    n = counts or (len(a["vv_w"]), len(a["ev_w"]), len(a["ee_w"]), len(a["fv_w"]))
    fn = _bind(ipctk.lib())
    status = fn(p(V), V.shape[0], p(E), E.shape[0], p(F), F.shape[0],
                n[0], p(a["vv"]), p(a["vv_w"]),
                n[1], p(a["ev"]), p(a["ev_w"]),
                n[2], p(a["ee"]), p(a["ee_eps_x"]), p(a["ee_dtype"]), p(a["ee_w"]),
                n[3], p(a["fv"]), p(a["fv_w"]),
                dhat, kappa, dmin, int(physical), p(out), None)
    torch.cuda.synchronize()
    return status, float(out.item())


def _device_arrays(sc, arrays):
    import torch
    V = _dev(sc["V"], torch.float64)
    E = _dev(sc["E"], torch.int32)
    F = _dev(sc["F"], torch.int32)
    a = {k: _dev(v, torch.int8 if k == "ee_dtype" else (torch.int32 if v.dtype == np.int32 else torch.float64))
         for k, v in arrays.items()}
    return V, E, F, a


@pytest.mark.parametrize("dmin,physical", [(0.0, False), (1e-4, False), (0.0, True), (2e-4, True)])
def test_noalloc_energy_matches_regular_entry_point(ipctk, dmin, physical):
    from ipctk_gb300 import scenes
    # two calls in a row: a larger set first, then a smaller one
    for sc in (scenes.two_sheet(side=48, seed=21), scenes.sphere_pack(n_side=2, seed=22)):
        mesh = ipctk.CollisionMesh(sc["V"], sc["E"], sc["F"])
        col = ipctk.NormalCollisions()
        col.build(mesh, sc["V"], sc["dhat"], dmin)
        assert len(col) > 0
        expected = ipctk.BarrierPotential(sc["dhat"], sc["kappa"], physical)(col, mesh, sc["V"])
        V, E, F, a = _device_arrays(sc, col.to_arrays())
        status, got = _call(ipctk, V, E, F, a, sc["dhat"], sc["kappa"], dmin, physical)
        assert status == 0, ipctk.lib().ipcg_last_error()
        assert abs(got - expected) <= REL * abs(expected), (got, expected)


def test_noalloc_energy_empty_set_is_zero(ipctk):
    from ipctk_gb300 import scenes
    sc = scenes.two_sheet(side=8, seed=23)
    mesh = ipctk.CollisionMesh(sc["V"], sc["E"], sc["F"])
    col = ipctk.NormalCollisions()
    col.build(mesh, sc["V"], sc["dhat"])
    arrays = {k: v[:0] for k, v in col.to_arrays().items()}
    V, E, F, a = _device_arrays(sc, arrays)
    status, got = _call(ipctk, V, E, F, a, sc["dhat"], sc["kappa"], 0.0, False)
    assert status == 0 and got == 0.0


def test_noalloc_energy_rejects_oversized_set(ipctk):
    # the count limit is checked on the host before anything is launched, so
    # small arrays with a count beyond the limit are never read
    from ipctk_gb300 import scenes
    sc = scenes.two_sheet(side=8, seed=24)
    mesh = ipctk.CollisionMesh(sc["V"], sc["E"], sc["F"])
    col = ipctk.NormalCollisions()
    col.build(mesh, sc["V"], sc["dhat"])
    V, E, F, a = _device_arrays(sc, col.to_arrays())
    status, _ = _call(ipctk, V, E, F, a, sc["dhat"], sc["kappa"], 0.0, False,
                      counts=(2_097_153, 0, 0, 0))
    assert status == 1
    assert "too many contacts" in ipctk.lib().ipcg_last_error().decode()


def test_noalloc_energy_out_of_range_index_gives_nan(ipctk):
    # one face-vertex contact names a face past the end of F: the device-side
    # check skips its reads and the energy comes back NaN
    from ipctk_gb300 import scenes
    sc = scenes.two_sheet(side=12, seed=25)
    mesh = ipctk.CollisionMesh(sc["V"], sc["E"], sc["F"])
    col = ipctk.NormalCollisions()
    col.build(mesh, sc["V"], sc["dhat"])
    arrays = dict(col.to_arrays())  # a copy: to_arrays() returns the set's cached dict
    assert len(arrays["fv_w"]) > 0
    arrays["fv"] = arrays["fv"].copy()
    arrays["fv"][0, 0] = sc["F"].shape[0] + 1000
    V, E, F, a = _device_arrays(sc, arrays)
    status, got = _call(ipctk, V, E, F, a, sc["dhat"], sc["kappa"], 0.0, False)
    assert status == 0
    assert np.isnan(got)
    # a valid call afterwards is unaffected
    V, E, F, a = _device_arrays(sc, col.to_arrays())
    expected = ipctk.BarrierPotential(sc["dhat"], sc["kappa"])(col, mesh, sc["V"])
    status, got = _call(ipctk, V, E, F, a, sc["dhat"], sc["kappa"], 0.0, False)
    assert status == 0 and abs(got - expected) <= REL * abs(expected)


def test_noalloc_energy_rejects_host_memory(ipctk):
    fn = _bind(ipctk.lib())
    V = np.zeros((3, 3))
    out = np.zeros(1)
    vv = np.array([[0, 1]], np.int32)
    w = np.ones(1)
    status = fn(V.ctypes.data_as(C.c_void_p), 3, None, 0, None, 0, 1, vv.ctypes.data_as(C.c_void_p),
                w.ctypes.data_as(C.c_void_p), 0, None, None, 0, None, None, None, None, 0, None, None,
                1e-3, 1.0, 0.0, 0, out.ctypes.data_as(C.c_void_p), None)
    assert status == 1
    assert "device memory" in ipctk.lib().ipcg_last_error().decode()
