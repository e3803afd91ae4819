"""Empty inputs through every entry point added beside the hot path: a scene
with no contact at all (two sheets farther apart than dhat) gives empty
collision sets of every kind, zero energies and forces, zero / empty
derivatives, and full steps, without error."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _far(ipctk):
    from ipctk_gb300 import scenes
    sc = scenes.two_sheet(side=8, seed=1)
    V = sc["V"].copy()
    V[V[:, 2] > 1e-5, 2] += 1.0  # the upper sheet far above the lower one
    return sc, V, ipctk.CollisionMesh(V, sc["E"], sc["F"])


def test_empty_collision_sets_and_potentials(ipctk):
    sc, V, mesh = _far(ipctk)
    dhat, kappa = sc["dhat"], sc["kappa"]
    B = ipctk.BarrierPotential(dhat, kappa)
    for area, improved, shape in ((False, False, True), (True, False, False), (True, True, False),
                                  (False, True, False)):
        col = ipctk.NormalCollisions()
        col.use_area_weighting = area
        col.enable_shape_derivatives = shape
        if improved:
            col.collision_set_type = ipctk.NormalCollisions.CollisionSetType.IMPROVED_MAX_APPROX
        col.build(mesh, V, dhat)
        assert len(col) == 0
        e, g, H = B.energy_gradient_hessian(col, mesh, V, ipctk.PSDProjectionMethod.CLAMP)
        assert e == 0 and not np.any(g) and H.nnz == 0
        assert not np.any(B.gauss_newton_hessian_diagonal(col, mesh, V))
        assert B.gauss_newton_hessian_quadratic_form(col, mesh, V, np.ones(V.size)) == 0
        if shape:
            assert B.shape_derivative(col, mesh, V).nnz == 0
        assert col.compute_minimum_distance(mesh, V) == float("inf")
        tc = ipctk.TangentialCollisions()
        tc.build(mesh, V, col, B, 0.5)
        assert len(tc) == 0
        tc.set_anisotropy(None, None, None)
        U = np.zeros_like(V)
        tc.update_lagged_anisotropic_friction_coefficients(mesh, V, U, U)
        D = ipctk.FrictionPotential(1e-3)
        e, g, H = D.energy_gradient_hessian(tc, mesh, U)
        assert e == 0 and not np.any(g) and H.nnz == 0
        assert not np.any(D.force(tc, mesh, V, U, U, B))


def test_empty_candidates_and_steps(ipctk):
    sc, V, mesh = _far(ipctk)
    V1 = V + np.array([0.1, 0.0, 0.0])  # a rigid slide: swept boxes overlap, nothing collides
    cand = ipctk.Candidates()
    cand.build(mesh, V, V1, inflation_radius=0.0)
    assert cand.compute_collision_free_stepsize(mesh, V, V1) == 1.0
    # no motion, no inflation: the non-candidate step is defined
    far = ipctk.Candidates()
    far.build(mesh, V, inflation_radius=0.0)
    assert far.compute_noncandidate_conservative_stepsize(mesh, np.zeros_like(V), sc["dhat"]) >= 0
    assert cand.compute_cfl_stepsize(mesh, V, V1, sc["dhat"]) == 1.0
    assert ipctk.compute_collision_free_stepsize(mesh, V, V1) == 1.0
    assert ipctk.is_step_collision_free(mesh, V, V1)
    assert not ipctk.has_intersections(mesh, V)
