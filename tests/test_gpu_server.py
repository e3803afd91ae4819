"""The request server (ipcg_server_*): results served concurrently, in any
mix, equal those of the same calls made directly.

Barrier requests rebuild the scene's collision set at the given positions
and return energy, gradient and CLAMP-projected Hessian; step-size requests
return compute_collision_free_stepsize.  Tolerances: energy, Hessian and
step bit-identical (their reductions are deterministic); gradient within
1e-12 relative (it sums contacts with atomic adds, in any order).
"""
import numpy as np
import pytest
import scipy.sparse as sp

pytestmark = pytest.mark.gpu


def _scenes():
    from ipctk_gb300 import scenes
    return [scenes.two_sheet(side=16, seed=41), scenes.sphere_pack(n_side=2, subdiv=2, seed=42),
            scenes.two_sheet(side=24, gap=2e-3, jitter=2e-4, dhat=3e-3, kappa=1e2, ccd_dz=4e-3, ccd_noise=4e-4,
                             seed=43),
            scenes.layered_cloth(layers=3, side=16, seed=44)]


def _direct(ipctk, sc, V, V1, mode=False):
    mesh = ipctk.CollisionMesh(sc["V"], sc["E"], sc["F"])
    col = ipctk.NormalCollisions()
    col.build(mesh, V, sc["dhat"])
    B = ipctk.BarrierPotential(sc["dhat"], sc["kappa"], mixed_precision=mode)
    e, g, H = B.energy_gradient_hessian(col, mesh, V, ipctk.PSDProjectionMethod.CLAMP)
    step = ipctk.compute_collision_free_stepsize(mesh, V, V1)
    return e, g, H, step


# the mixed mode too: a scene's barrier options (ipcg_server_set_scene_options)
@pytest.mark.parametrize("budget,mode", [(120e9, False), (2e6, False), (120e9, "local")])
def test_served_results_equal_direct_calls(ipctk, budget, mode):
    scs = _scenes()
    rng = np.random.default_rng(5)
    # two Newton-like iterations per scene: perturbed positions, then a step
    plans = []
    for sc in scs:
        its = []
        for _ in range(2):
            V = sc["V"] + rng.uniform(-0.1, 0.1, sc["V"].shape) * sc["dhat"]
            its.append((V, V + (sc["V1"] - sc["V"])))
        plans.append(its)
    server = ipctk.Server(workers=3, hbm_budget_bytes=budget)
    ids = []
    for sc in scs:
        mesh = ipctk.CollisionMesh(sc["V"], sc["E"], sc["F"])
        col = ipctk.NormalCollisions()
        ids.append(server.add_scene(mesh, col, sc["dhat"], 0.0, sc["kappa"]))
        if mode:
            server.set_scene_options(ids[-1], mixed_precision=mode)
    tickets = []
    for it in range(2):  # interleave the scenes' requests
        for k, sc in enumerate(scs):
            V, V1 = plans[k][it]
            tickets.append((k, it, "barrier", server.submit_barrier(ids[k], V)))
            tickets.append((k, it, "step", server.submit_stepsize(ids[k], V, V1)))
    results = {}
    for k, it, kind, t in tickets:
        results[(k, it, kind)] = server.wait(t, gradient=(kind == "barrier"), hessian="scipy" if kind == "barrier"
                                             else None)
    st = server.stats()
    assert st["completed"] == len(tickets) and st["queued"] == 0 and st["running"] == 0
    if budget < 1e7:
        assert st["releases"] > 0  # the small budget made the server release idle work space
    for k, sc in enumerate(scs):
        for it in range(2):
            V, V1 = plans[k][it]
            e, g, H, step = _direct(ipctk, sc, V, V1, mode)
            rb, rs = results[(k, it, "barrier")], results[(k, it, "step")]
            assert rb["energy"] == e, (k, it)
            assert np.linalg.norm(rb["gradient"] - g) <= 1e-12 * max(np.linalg.norm(g), 1e-300)
            Hs = rb["hessian"]
            assert Hs.shape == H.shape
            np.testing.assert_array_equal(Hs.indptr, H.indptr)
            np.testing.assert_array_equal(Hs.indices, H.indices)
            np.testing.assert_array_equal(Hs.data, H.data)
            assert rs["step"] == step, (k, it)
            assert rb["t_submit_ns"] <= rb["t_start_ns"] <= rb["t_end_ns"]
    server.close()


def test_server_rejects_bad_requests(ipctk):
    server = ipctk.Server(workers=1, hbm_budget_bytes=1e9)
    with pytest.raises(ValueError):
        server.submit_barrier(0, np.zeros((3, 3)))
    with pytest.raises(ValueError):
        server.set_scene_options(0, mixed_precision="local")
    server.close()
