"""Codimensional meshes (collision_mesh.cpp:145-183).

The reference finds vertex-vertex candidates among codimensional vertices
(vertices in no edge) and edge-vertex candidates between codimensional edges
and those vertices (candidates.cpp:66-116, 152-210).  Those passes are not
provided here, so every call that would need them -- the collision-set build,
candidate builds and the step-size calls -- must refuse a mesh with
codimensional vertices instead of returning an incomplete result.  A mesh
whose only codimensional elements are free edges needs no extra pass and stays
supported."""
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
