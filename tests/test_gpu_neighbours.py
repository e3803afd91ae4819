"""The Newton-loop neighbours of the path: NormalCollisions::compute_minimum_distance,
is_step_collision_free and has_intersections, against the oracle."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", ["two_sheet_16", "spheres_27", "cloth_4x48"])
def test_minimum_distance_matches_oracle_contacts(ipctk, oracle_mod, name):
    from test_gpu_parity import _scene
    sc = _scene(name)
    V, E, F = sc["V"], sc["E"], sc["F"]
    mesh = ipctk.CollisionMesh(V, E, F)
    col = ipctk.NormalCollisions()
    col.build(mesh, V, sc["dhat"])
    got = col.compute_minimum_distance(mesh, V)
    a = col.to_arrays()
    ds = []
    for v0, v1 in a["vv"]:
        ds.append(float(np.sum((V[v0] - V[v1]) ** 2)))
    for e, v in a["ev"]:
        ds.append(oracle_mod.point_edge_distance(V[v], V[E[e, 0]], V[E[e, 1]], 2))   # point-line
    for (ea, eb), dt in zip(a["ee"], a["ee_dtype"]):
        ds.append(oracle_mod.edge_edge_distance(V[E[ea, 0]], V[E[ea, 1]], V[E[eb, 0]], V[E[eb, 1]], int(dt)))
    for f, v in a["fv"]:
        ds.append(oracle_mod.point_triangle_distance(V[v], V[F[f, 0]], V[F[f, 1]], V[F[f, 2]], 6))  # point-plane
    ref = min(ds)
    assert abs(got - ref) <= 1e-12 * ref, (got, ref)
    empty = ipctk.NormalCollisions()
    assert empty.compute_minimum_distance(mesh, V) == float("inf")


@pytest.mark.parametrize("name", ["two_sheet_16", "spheres_27", "cloth_4x48"])
def test_is_step_collision_free_matches_oracle(ipctk, oracle_mod, name):
    from test_gpu_parity import _scene
    sc = _scene(name)
    V0, V1, E, F = sc["V"], sc["V1"], sc["E"], sc["F"]
    mesh = ipctk.CollisionMesh(V0, E, F)
    for end in (V1, V0 + 0.25 * (V1 - V0), V0):
        ee, fv = oracle_mod.ccd_candidates(V0, end, E, F)
        (xe0, xe1), (xf0, xf1) = oracle_mod.ccd_stencil_positions(V0, end, E, F, ee, fv)
        hit = False
        for is_ee, x0, x1 in ((1, xe0, xe1), (0, xf0, xf1)):
            if len(x0):
                h, _, _ = oracle_mod.ccd_stencils(is_ee, x0, x1)
                hit |= bool(h.any())
        assert ipctk.is_step_collision_free(mesh, V0, end) == (not hit)
    assert ipctk.is_step_collision_free(mesh, V0, V0)


def _pierce(offset):
    """A triangle in z = 0 and a vertical edge through (x, y) = (0.25, 0.25) + offset."""
    V = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0],
                  [0.25 + offset[0], 0.25 + offset[1], -0.5], [0.25 + offset[0], 0.25 + offset[1], 0.5]], float)
    return V, np.array([[0, 1], [1, 2], [2, 0], [3, 4]], np.int32), np.array([[0, 1, 2]], np.int32)


def test_has_intersections_known_cases(ipctk, oracle_mod):
    for offset, expected in (((0, 0), True), ((1.0, 1.0), False), ((0.25, 0.25), True), ((0.26, 0.25), False)):
        V, E, F = _pierce(offset)
        mesh = ipctk.CollisionMesh(V, E, F)
        assert ipctk.has_intersections(mesh, V) == expected, offset
        assert oracle_mod.has_intersections_bruteforce(V, E, F) == expected
    # the edge's tip exactly on the face (orientation 0: the exact predicate decides)
    V, E, F = _pierce((0, 0))
    V[4, 2] = 0.0
    assert ipctk.has_intersections(ipctk.CollisionMesh(V, E, F), V)
    V[4, 2] = 1e-300  # just above the plane, still on the edge's side of touching
    assert ipctk.has_intersections(ipctk.CollisionMesh(V, E, F), V) == oracle_mod.has_intersections_bruteforce(V, E,
                                                                                                                F)


def test_has_intersections_sheets(ipctk, oracle_mod):
    from ipctk_gb300 import scenes
    sc = scenes.two_sheet(side=6, seed=51)
    mesh = ipctk.CollisionMesh(sc["V"], sc["E"], sc["F"])
    assert not ipctk.has_intersections(mesh, sc["V"])
    assert not oracle_mod.has_intersections_bruteforce(sc["V"], sc["E"], sc["F"])
    # halfway through the step the upper sheet crosses the lower one
    Vm = 0.5 * (sc["V"] + sc["V1"])
    assert ipctk.has_intersections(mesh, Vm)
    assert oracle_mod.has_intersections_bruteforce(Vm, sc["E"], sc["F"])
    # at the end of the step it lies wholly below it
    assert ipctk.has_intersections(mesh, sc["V1"]) == oracle_mod.has_intersections_bruteforce(sc["V1"], sc["E"],
                                                                                             sc["F"])


def test_free_distance_functions(ipctk, oracle_mod):
    """The reference's free distance functions (AUTO type) on the device
    against the oracle, single and stacked."""
    rng = np.random.Generator(np.random.PCG64(12))
    for _ in range(20):
        x = rng.uniform(-1, 1, (4, 3))
        assert ipctk.point_triangle_distance(*x) == oracle_mod.point_triangle_distance(*x)
        assert ipctk.edge_edge_distance(*x) == oracle_mod.edge_edge_distance(*x)
        assert ipctk.point_edge_distance(*x[:3]) == oracle_mod.point_edge_distance(*x[:3])
        assert int(ipctk.point_triangle_distance_type(*x)) == oracle_mod.point_triangle_distance_type(*x)
        assert int(ipctk.edge_edge_distance_type(*x)) == oracle_mod.edge_edge_distance_type(*x)
        assert ipctk.point_point_distance(x[0], x[1]) == float(np.sum((x[1] - x[0]) ** 2))
    X = rng.uniform(-1, 1, (50, 4, 3))
    d = ipctk.point_triangle_distance(X[:, 0], X[:, 1], X[:, 2], X[:, 3])
    assert d.shape == (50,)
    assert np.all(d == [oracle_mod.point_triangle_distance(*x) for x in X])
    with pytest.raises(ValueError):
        ipctk.point_triangle_distance(*X[0], dtype=ipctk.PointTriangleDistanceType.P_T0)


def test_initial_barrier_stiffness_device_vectors(ipctk):
    """The dot products of initial_barrier_stiffness run on the device when
    the gradients live there, and agree with the host path."""
    import torch
    rng = np.random.default_rng(51)
    gE = rng.normal(size=300_000)
    gB = rng.normal(size=300_000)
    host = ipctk.initial_barrier_stiffness(2.0, 1e-3, 0.5, gE, gB, min_barrier_stiffness_scale=1e3)
    dev = ipctk.initial_barrier_stiffness(2.0, 1e-3, 0.5, torch.from_numpy(gE).cuda(), torch.from_numpy(gB).cuda(),
                                          min_barrier_stiffness_scale=1e3)
    assert dev[1] == host[1]
    assert abs(dev[0] - host[0]) <= 1e-12 * abs(host[0])
