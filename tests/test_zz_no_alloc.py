"""The allocation-free barrier energy (ipcg_barrier_energy_noalloc).

Some callers of this library cannot let it allocate device memory during a
call: simulation codes that hand all device memory to their own pool under a
hard budget, or that cannot afford cudaMalloc/cudaFree synchronising the
device under their other streams.  For them the library offers an energy
evaluation whose only scratch (the reduction's partial sums) lives in a
static device array, with every input and the output in caller-owned device
memory.  This test calls that entry point through the C ABI, twice in a row
on two different collision sets (the second one smaller, so stale partial
sums left by the first call in the shared array must not leak into the
second), and checks each result against the regular ipcg_barrier_energy
within the 1e-10 relative tolerance used by the other parity tests.

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


def _energy_noalloc(ipctk, sc, arrays):
    import torch
    dev = torch.device("cuda", 0)

    def t(x, dtype):
        return torch.as_tensor(np.ascontiguousarray(x), dtype=dtype, device=dev)

    V = t(sc["V"], torch.float64)
    E = t(sc["E"], torch.int32)
    F = t(sc["F"], torch.int32)
    a = {k: t(v, torch.int8 if k == "ee_dtype" else (torch.int32 if v.dtype == np.int32 else torch.float64))
         for k, v in arrays.items()}
    out = torch.full((1,), float("nan"), dtype=torch.float64, device=dev)
    p = lambda x: C.c_void_p(x.data_ptr()) if x.numel() else None
    fn = _bind(ipctk.lib())
    status = fn(p(V), V.shape[0], p(E), E.shape[0], p(F), F.shape[0],
                len(a["vv_w"]), p(a["vv"]), p(a["vv_w"]),
                len(a["ev_w"]), p(a["ev"]), p(a["ev_w"]),
                len(a["ee_w"]), p(a["ee"]), p(a["ee_eps_x"]), p(a["ee_dtype"]), p(a["ee_w"]),
                len(a["fv_w"]), p(a["fv"]), p(a["fv_w"]),
                sc["dhat"], sc["kappa"], 0.0, 0, p(out), None)
    assert status == 0, ipctk.lib().ipcg_last_error()
    torch.cuda.synchronize()
    return float(out.item())


def test_noalloc_energy_matches_regular_entry_point(ipctk):
    from ipctk_gb300 import scenes
    # two calls in a row: a larger set first, then a smaller one
    for sc in (scenes.two_sheet(side=48, seed=21), scenes.sphere_pack(n_side=2, seed=22)):
        mesh = ipctk.CollisionMesh(sc["V"], sc["E"], sc["F"])
        col = ipctk.NormalCollisions()
        col.build(mesh, sc["V"], sc["dhat"])
        assert len(col) > 0
        expected = ipctk.BarrierPotential(sc["dhat"], sc["kappa"])(col, mesh, sc["V"])
        got = _energy_noalloc(ipctk, sc, col.to_arrays())
        assert abs(got - expected) <= REL * abs(expected), (got, expected)


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
