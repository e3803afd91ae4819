"""Candidates (candidates.cpp): the kept broad-phase set and the step-size
rules that read it, against the oracle (same pairs; distances bit-exact;
CCD steps identical)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _sorted(a):
    a = np.asarray(a)
    return a[np.lexsort((a[:, 1], a[:, 0]))] if len(a) else a


@pytest.mark.parametrize("name", ["two_sheet_16", "spheres_27", "cloth_4x48"])
def test_candidates_and_safe_distances(ipctk, oracle_mod, name):
    from test_gpu_parity import _scene
    sc = _scene(name)
    V, V1, E, F = sc["V"], sc["V1"], sc["E"], sc["F"]
    mesh = ipctk.CollisionMesh(V, E, F)
    r = 2 * sc["dhat"]
    cand = ipctk.Candidates()
    cand.build(mesh, V, inflation_radius=r)
    ee, fv = cand.to_arrays()
    ree, rfv = oracle_mod.ccd_candidates(V, V, E, F, 2 * r)  # the oracle inflates by half its argument
    np.testing.assert_array_equal(_sorted(ee), _sorted(ree))
    np.testing.assert_array_equal(_sorted(fv), _sorted(rfv))
    md = 0.1 * sc["dhat"]
    safe = cand.compute_per_vertex_safe_distances(mesh, V, r, md)
    ref = np.full(V.shape[0], r - md)
    for ea, eb in ee:
        ids = [E[ea, 0], E[ea, 1], E[eb, 0], E[eb, 1]]
        d = np.sqrt(oracle_mod.edge_edge_distance(*(V[i] for i in ids))) - md
        for i in ids:
            ref[i] = min(ref[i], d)
    for f, v in fv:
        ids = [v, F[f, 0], F[f, 1], F[f, 2]]
        d = np.sqrt(oracle_mod.point_triangle_distance(*(V[i] for i in ids))) - md
        for i in ids:
            ref[i] = min(ref[i], d)
    np.testing.assert_array_equal(safe, ref)


@pytest.mark.parametrize("name", ["two_sheet_16", "spheres_27", "cloth_4x48"])
def test_candidate_step_sizes(ipctk, name):
    from test_gpu_parity import _scene
    sc = _scene(name)
    V0, V1, E, F = sc["V"], sc["V1"], sc["E"], sc["F"]
    mesh = ipctk.CollisionMesh(V0, E, F)
    cand = ipctk.Candidates()
    cand.build(mesh, V0, V1, inflation_radius=0.0)  # swept, as compute_collision_free_stepsize builds them
    a_c = cand.compute_collision_free_stepsize(mesh, V0, V1)
    assert a_c == ipctk.compute_collision_free_stepsize(mesh, V0, V1)
    U = V1 - V0
    ee, fv = cand.to_arrays()
    ids = set()
    for ea, eb in ee:
        ids.update([E[ea, 0], E[ea, 1], E[eb, 0], E[eb, 1]])
    for f, v in fv:
        ids.update([v, F[f, 0], F[f, 1], F[f, 2]])
    mx = max(np.linalg.norm(U[i]) for i in ids)
    a_f = cand.compute_noncandidate_conservative_stepsize(mesh, U, sc["dhat"])
    assert a_f == 0.5 * sc["dhat"] / mx
    cfl = cand.compute_cfl_stepsize(mesh, V0, V1, sc["dhat"])
    full = ipctk.compute_collision_free_stepsize(mesh, V0, V1)
    assert cfl == (full if a_f < 0.5 * a_c else min(a_c, a_f))
