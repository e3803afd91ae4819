"""NormalPotential::shape_derivative on the device against the oracle
(within 1e-10 relative), with and without area weighting, and its argument
rules: the set must have been built with shape derivatives enabled, and
area-weighted IMPROVED_MAX_APPROX sets are not provided."""
import numpy as np
import pytest
import scipy.sparse as sp

from test_gpu_parity import REL, _scene

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", ["two_sheet_16", "two_sheet_64", "spheres_27", "cloth_4x48"])
@pytest.mark.parametrize("physical", [False, True])
@pytest.mark.parametrize("area", [False, True])
def test_shape_derivative(ipctk, oracle_mod, name, physical, area):
    sc = _scene(name)
    V, E, F = sc["V"], sc["E"], sc["F"]
    mesh = ipctk.CollisionMesh(V, E, F)
    col = ipctk.NormalCollisions()
    col.enable_shape_derivatives = True
    col.use_area_weighting = area
    col.build(mesh, V, sc["dhat"])
    ref = oracle_mod.build_collisions(V, E, F, sc["dhat"], area_weighting=area)
    B = ipctk.BarrierPotential(sc["dhat"], sc["kappa"], physical)
    S = B.shape_derivative(col, mesh, V)
    rp, ci, va = oracle_mod.barrier_shape_derivative(ref, V, E, F, sc["dhat"], sc["kappa"], physical=int(physical),
                                                     area_weighting=area)
    S_ref = sp.csr_matrix((va, ci, rp), shape=S.shape)
    assert sp.linalg.norm(S_ref) > 0
    assert sp.linalg.norm(S - S_ref) <= REL * sp.linalg.norm(S_ref)


def test_shape_derivative_rules(ipctk):
    sc = _scene("two_sheet_16")
    mesh = ipctk.CollisionMesh(sc["V"], sc["E"], sc["F"])
    B = ipctk.BarrierPotential(sc["dhat"], sc["kappa"])
    col = ipctk.NormalCollisions()
    col.build(mesh, sc["V"], sc["dhat"])
    with pytest.raises(ValueError, match="Shape derivative is not computed"):
        B.shape_derivative(col, mesh, sc["V"])
    col.enable_shape_derivatives = True
    col.use_area_weighting = True
    col.collision_set_type = ipctk.NormalCollisions.CollisionSetType.IMPROVED_MAX_APPROX
    col.build(mesh, sc["V"], sc["dhat"])
    with pytest.raises(ValueError, match="area-weighted IMPROVED_MAX_APPROX"):
        B.shape_derivative(col, mesh, sc["V"])
