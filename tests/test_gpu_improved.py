"""CollisionSetType.IMPROVED_MAX_APPROX on the device against the oracle:
collision sets bit-exact (indices, weights, eps_x, types; zero sums dropped),
potentials within 1e-10 relative, with and without area weighting."""
import numpy as np
import pytest
import scipy.sparse as sp

from test_gpu_parity import REL, _scene

pytestmark = pytest.mark.gpu

NAMES = ["two_sheet_16", "two_sheet_64", "spheres_27", "cloth_4x48"]


def _improved(ipctk, mesh, V, dhat, area):
    col = ipctk.NormalCollisions()
    col.use_area_weighting = area
    col.collision_set_type = ipctk.NormalCollisions.CollisionSetType.IMPROVED_MAX_APPROX
    col.build(mesh, V, dhat)
    return col


def _assert_same_set(a, ref):
    for k, r in (("vv", ref.vv), ("vv_w", ref.vv_w), ("ev", ref.ev), ("ev_w", ref.ev_w), ("ee", ref.ee),
                 ("ee_w", ref.ee_w), ("ee_eps_x", ref.ee_eps), ("ee_dtype", ref.ee_dtype), ("fv", ref.fv),
                 ("fv_w", ref.fv_w)):
        np.testing.assert_array_equal(a[k], np.asarray(r).reshape(np.asarray(a[k]).shape), err_msg=k)


@pytest.mark.parametrize("name", NAMES)
@pytest.mark.parametrize("area", [False, True])
def test_improved_set_and_potential(ipctk, oracle_mod, name, area):
    sc = _scene(name)
    V, E, F = sc["V"], sc["E"], sc["F"]
    mesh = ipctk.CollisionMesh(V, E, F)
    col = _improved(ipctk, mesh, V, sc["dhat"], area)
    ref = oracle_mod.build_collisions(V, E, F, sc["dhat"], area_weighting=area, improved_max_approx=True)
    a = col.to_arrays()
    _assert_same_set(a, ref)
    assert len(col) == len(ref) > 0
    B = ipctk.BarrierPotential(sc["dhat"], sc["kappa"], True)
    e, g, H = B.energy_gradient_hessian(col, mesh, V, ipctk.PSDProjectionMethod.CLAMP)
    e_ref = oracle_mod.barrier_energy(ref, V, E, F, sc["dhat"], sc["kappa"], physical=True)
    assert abs(e - e_ref) <= REL * abs(e_ref)
    g_ref = oracle_mod.barrier_gradient(ref, V, E, F, sc["dhat"], sc["kappa"], physical=True)
    assert np.linalg.norm(g - g_ref) <= REL * np.linalg.norm(g_ref)
    rp, ci, va = oracle_mod.barrier_hessian(ref, V, E, F, sc["dhat"], sc["kappa"], physical=True, psd="clamp")
    H_ref = sp.csr_matrix((va, ci, rp), shape=H.shape)
    assert sp.linalg.norm(H - H_ref) <= REL * sp.linalg.norm(H_ref)


def test_improved_fan_and_edge_cases(ipctk, oracle_mod):
    """The hand-checked cases: one contact over a fan centre and one over a
    shared edge each weigh one contact's energy."""
    from test_oracle import _fan_with_point
    cases = [_fan_with_point([0.0, 0.0, 1e-3]),
             (np.array([[0.0, 0, 0], [1, 0, 0], [0.5, 1, 0], [0.5, -1, 0], [0.5, 0, 1e-3]]),
              np.array([[0, 1], [1, 2], [2, 0], [0, 3], [3, 1]]), np.array([[0, 1, 2], [1, 0, 3]]))]
    for V, E, F in cases:
        mesh = ipctk.CollisionMesh(V, E, F)
        col = _improved(ipctk, mesh, V, 1e-2, False)
        ref = oracle_mod.build_collisions(V, E, F, 1e-2, improved_max_approx=True)
        _assert_same_set(col.to_arrays(), ref)
        e = ipctk.BarrierPotential(1e-2, 1.0)(col, mesh, V)
        assert e == pytest.approx(oracle_mod.barrier(1e-6, 1e-4), rel=1e-12)


def test_improved_then_ipc_again(ipctk):
    sc = _scene("two_sheet_16")
    mesh = ipctk.CollisionMesh(sc["V"], sc["E"], sc["F"])
    col = ipctk.NormalCollisions()
    col.build(mesh, sc["V"], sc["dhat"])
    plain = col.to_arrays()
    col.collision_set_type = ipctk.NormalCollisions.CollisionSetType.IMPROVED_MAX_APPROX
    col.build(mesh, sc["V"], sc["dhat"])
    col.collision_set_type = ipctk.NormalCollisions.CollisionSetType.IPC
    col.build(mesh, sc["V"], sc["dhat"])
    again = col.to_arrays()
    for k in plain:
        np.testing.assert_array_equal(plain[k], again[k])


def test_improved_batch_equals_scenes(ipctk):
    from ipctk_gb300 import scenes
    parts = [scenes.two_sheet(side=s, seed=s) for s in (8, 12, 16)]
    batch = ipctk.SceneBatch([(p["V"], p["E"], p["F"]) for p in parts])
    V = np.concatenate([p["V"] for p in parts])
    col = _improved(ipctk, batch, V, [p["dhat"] for p in parts], True)
    got = col.to_arrays()
    want = {k: [] for k in ("vv_w", "ev_w", "ee_w", "fv_w", "ee_dtype")}
    for p in parts:
        m = ipctk.CollisionMesh(p["V"], p["E"], p["F"])
        a = _improved(ipctk, m, p["V"], p["dhat"], True).to_arrays()
        for k in want:
            want[k].append(a[k])
    for k in want:
        np.testing.assert_array_equal(got[k], np.concatenate(want[k]), err_msg=k)
