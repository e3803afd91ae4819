"""Codimensional meshes (collision_mesh.cpp:145-183).

The reference finds vertex-vertex candidates among codimensional vertices
(vertices in no edge) and edge-vertex candidates between codimensional edges
and those vertices (candidates.cpp:66-116, 152-210).  Those passes are not
provided here, so every call that would need them -- the collision-set build,
candidate builds and the step-size calls -- must refuse a mesh on which they
would find pairs (two codimensional vertices, or one with a codimensional
edge) instead of returning an incomplete result.  A mesh whose only
codimensional elements are free edges, or a single loose vertex, needs no
extra pass and stays supported."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _cloud_and_free_edge():
    # a triangle, a free edge above it and three loose points (a point cloud)
    V = np.array([[0.0, 0, 0], [1, 0, 0], [0, 1, 0],
                  [0.2, 0.2, 5e-4], [0.6, 0.2, 5e-4],
                  [0.3, 0.3, 4e-4], [0.3, 0.3, 8e-4], [0.31, 0.3, 6e-4]])
    E = np.array([[0, 1], [1, 2], [0, 2], [3, 4]], np.int32)
    F = np.array([[0, 1, 2]], np.int32)
    return V, E, F


def test_codim_counts(ipctk):
    V, E, F = _cloud_and_free_edge()
    mesh = ipctk.CollisionMesh(V, E, F)
    assert mesh.num_codim_vertices == 3
    assert mesh.num_codim_edges == 1


def test_codim_vertices_are_refused(ipctk):
    V, E, F = _cloud_and_free_edge()
    mesh = ipctk.CollisionMesh(V, E, F)
    V1 = V.copy()
    V1[3:, 2] -= 1e-3
    with pytest.raises(ValueError, match="codimensional vertices"):
        ipctk.NormalCollisions().build(mesh, V, 1e-3)
    with pytest.raises(ValueError, match="codimensional vertices"):
        ipctk.compute_collision_free_stepsize(mesh, V, V1)
    with pytest.raises(ValueError, match="codimensional vertices"):
        ipctk.is_step_collision_free(mesh, V, V1)
    with pytest.raises(ValueError, match="codimensional vertices"):
        ipctk.Candidates().build(mesh, V, inflation_radius=1e-3)


def test_free_edge_only_is_supported(ipctk, oracle_mod):
    # the free edge lies just above the triangle: its contacts are edge-edge
    # candidates of the regular passes, and the set matches the oracle's
    V, E, F = _cloud_and_free_edge()
    V, E = V[:5], E
    mesh = ipctk.CollisionMesh(V, E, F)
    assert mesh.num_codim_vertices == 0 and mesh.num_codim_edges == 1
    col = ipctk.NormalCollisions()
    col.build(mesh, V, 1e-3)
    ref = oracle_mod.build_collisions(V, E, F, 1e-3)
    a = col.to_arrays()
    assert len(col) == len(ref) > 0
    for k in ("vv", "ev", "ee", "fv"):
        np.testing.assert_array_equal(a[k], np.asarray(getattr(ref, k)).reshape(np.asarray(a[k]).shape), err_msg=k)


def test_single_loose_vertex_is_supported(ipctk, oracle_mod):
    # one point above the triangle and no free edge: nothing for the
    # codimensional passes to pair, its contact is a face-vertex candidate
    V, E, F = _cloud_and_free_edge()
    V = np.concatenate([V[:3], V[5:6]])
    E = E[:3]
    mesh = ipctk.CollisionMesh(V, E, F)
    assert mesh.num_codim_vertices == 1 and mesh.num_codim_edges == 0
    col = ipctk.NormalCollisions()
    col.build(mesh, V, 1e-3)
    ref = oracle_mod.build_collisions(V, E, F, 1e-3)
    a = col.to_arrays()
    assert len(col) == len(ref) > 0
    for k in ("vv", "ev", "ee", "fv"):
        np.testing.assert_array_equal(a[k], np.asarray(getattr(ref, k)).reshape(np.asarray(a[k]).shape), err_msg=k)
    V1 = V.copy()
    V1[3, 2] -= 1e-3
    t = ipctk.compute_collision_free_stepsize(mesh, V, V1)
    assert 0.0 < t < 1.0
