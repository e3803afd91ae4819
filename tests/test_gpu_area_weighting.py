"""Area weighting (NormalCollisions::set_use_area_weighting) on the device
against the oracle: rest-mesh areas bit-exact, collision sets bit-exact
(indices and weights; duplicate VV / EV keys sum their weights in ascending
order on both sides), potentials within 1e-10 relative."""
import numpy as np
import pytest
import scipy.sparse as sp

from test_gpu_parity import REL, _scene

pytestmark = pytest.mark.gpu

NAMES = ["two_sheet_16", "two_sheet_64", "spheres_27", "cloth_4x48"]


@pytest.mark.parametrize("name", NAMES)
def test_mesh_areas(ipctk, oracle_mod, name):
    sc = _scene(name)
    mesh = ipctk.CollisionMesh(sc["V"], sc["E"], sc["F"])
    va, ea = oracle_mod.mesh_areas(sc["V"], sc["E"], sc["F"])
    np.testing.assert_array_equal(mesh.vertex_areas, va)
    np.testing.assert_array_equal(mesh.edge_areas, ea)


@pytest.mark.parametrize("name", NAMES)
def test_area_weighted_set_and_potential(ipctk, oracle_mod, name):
    sc = _scene(name)
    V, E, F = sc["V"], sc["E"], sc["F"]
    mesh = ipctk.CollisionMesh(V, E, F)
    col = ipctk.NormalCollisions()
    col.use_area_weighting = True
    assert col.use_area_weighting
    col.build(mesh, V, sc["dhat"])
    ref = oracle_mod.build_collisions(V, E, F, sc["dhat"], area_weighting=True)
    a = col.to_arrays()
    for k, r in (("vv", ref.vv), ("vv_w", ref.vv_w), ("ev", ref.ev), ("ev_w", ref.ev_w), ("ee", ref.ee),
                 ("ee_w", ref.ee_w), ("ee_dtype", ref.ee_dtype), ("fv", ref.fv), ("fv_w", ref.fv_w)):
        np.testing.assert_array_equal(a[k], r, err_msg=k)
    assert np.any(a["vv_w"] != np.round(a["vv_w"])) or len(a["vv_w"]) == 0
    B = ipctk.BarrierPotential(sc["dhat"], sc["kappa"])
    e, g, H = B.energy_gradient_hessian(col, mesh, V, ipctk.PSDProjectionMethod.CLAMP)
    e_ref = oracle_mod.barrier_energy(ref, V, E, F, sc["dhat"], sc["kappa"])
    assert abs(e - e_ref) <= REL * abs(e_ref)
    g_ref = oracle_mod.barrier_gradient(ref, V, E, F, sc["dhat"], sc["kappa"])
    assert np.linalg.norm(g - g_ref) <= REL * np.linalg.norm(g_ref)
    rp, ci, va = oracle_mod.barrier_hessian(ref, V, E, F, sc["dhat"], sc["kappa"], psd="clamp")
    H_ref = sp.csr_matrix((va, ci, rp), shape=H.shape)
    assert sp.linalg.norm(H - H_ref) <= REL * sp.linalg.norm(H_ref)


def test_area_weighting_toggles_back(ipctk):
    sc = _scene("two_sheet_16")
    mesh = ipctk.CollisionMesh(sc["V"], sc["E"], sc["F"])
    col = ipctk.NormalCollisions()
    col.build(mesh, sc["V"], sc["dhat"])
    plain = col.to_arrays()
    col.use_area_weighting = True
    col.build(mesh, sc["V"], sc["dhat"])
    col.use_area_weighting = False
    col.build(mesh, sc["V"], sc["dhat"])
    again = col.to_arrays()
    for k in plain:
        np.testing.assert_array_equal(plain[k], again[k])


def test_area_weighting_batch_equals_scenes(ipctk):
    from ipctk_gb300 import scenes
    parts = [scenes.two_sheet(side=s, seed=s) for s in (8, 12, 16)]
    batch = ipctk.SceneBatch([(p["V"], p["E"], p["F"]) for p in parts])
    V = np.concatenate([p["V"] for p in parts])
    col = ipctk.NormalCollisions()
    col.use_area_weighting = True
    col.build(batch, V, [p["dhat"] for p in parts])
    got = col.to_arrays()
    voff = np.cumsum([0] + [len(p["V"]) for p in parts])
    eoff = np.cumsum([0] + [len(p["E"]) for p in parts])
    foff = np.cumsum([0] + [len(p["F"]) for p in parts])
    want = {k: [] for k in ("vv_w", "ev_w", "ee_w", "fv_w")}
    for i, p in enumerate(parts):
        m = ipctk.CollisionMesh(p["V"], p["E"], p["F"])
        c = ipctk.NormalCollisions()
        c.use_area_weighting = True
        c.build(m, p["V"], p["dhat"])
        a = c.to_arrays()
        for k in want:
            want[k].append(a[k])
    for k in want:
        np.testing.assert_array_equal(got[k], np.concatenate(want[k]), err_msg=k)
