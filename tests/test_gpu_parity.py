"""GPU parity: the CUDA path (through the C ABI) against the CPU oracle.

Tolerances (the bar of the contact hot path):
  * collision sets: bit-exact as sorted index tuples, weights and EE types;
  * barrier energy, gradient, Hessian: within 1e-10 relative
    (|a-b| <= 1e-10 |b| for the energy, ||a-b||_2 <= 1e-10 ||b||_2 for the
    gradient, ||A-B||_F <= 1e-10 ||B||_F for the Hessian);
  * collision-free step size: identical to the oracle (same algorithm, same
    FP64 operation order on both sides).
"""
import numpy as np
import pytest
import scipy.sparse as sp

pytestmark = pytest.mark.gpu

REL = 1e-10


def _scene(name):
    from ipctk_gb300 import scenes
    if name == "two_sheet_16":
        return scenes.two_sheet(side=16, seed=3)
    if name == "two_sheet_64":
        return scenes.two_sheet(side=64, seed=0)
    if name == "spheres_27":
        return scenes.sphere_pack(n_side=3, seed=5)
    if name == "spheres_64_sub2":
        return scenes.sphere_pack(n_side=4, subdiv=2, seed=9)
    if name == "cloth_4x48":
        return scenes.layered_cloth(layers=4, side=48, seed=11)
    raise KeyError(name)


SCENES = ["two_sheet_16", "two_sheet_64", "spheres_27", "spheres_64_sub2", "cloth_4x48"]


@pytest.fixture(scope="module")
def built(ipctk, oracle_mod):
    cache = {}

    def get(name):
        if name not in cache:
            sc = _scene(name)
            mesh = ipctk.CollisionMesh(sc["V"], sc["E"], sc["F"])
            col = ipctk.NormalCollisions()
            col.build(mesh, sc["V"], sc["dhat"])
            ref = oracle_mod.build_collisions(sc["V"], sc["E"], sc["F"], sc["dhat"])
            cache[name] = (sc, mesh, col, ref)
        return cache[name]

    return get


@pytest.mark.parametrize("name", SCENES)
def test_collision_set_bit_exact(built, name):
    sc, mesh, col, ref = built(name)
    a = col.to_arrays()
    assert len(col) == len(ref) and len(ref) > 0
    np.testing.assert_array_equal(a["vv"], ref.vv)
    np.testing.assert_array_equal(a["vv_w"], ref.vv_w)
    np.testing.assert_array_equal(a["ev"], ref.ev)
    np.testing.assert_array_equal(a["ev_w"], ref.ev_w)
    np.testing.assert_array_equal(a["ee"], ref.ee)
    np.testing.assert_array_equal(a["ee_dtype"], ref.ee_dtype)
    np.testing.assert_array_equal(a["ee_eps_x"], ref.ee_eps)
    np.testing.assert_array_equal(a["fv"], ref.fv)


@pytest.mark.parametrize("name", SCENES)
def test_faces_to_edges(built, oracle_mod, name):
    sc, mesh, _, _ = built(name)
    np.testing.assert_array_equal(mesh.faces_to_edges, oracle_mod.faces_to_edges(sc["F"], sc["E"]))


@pytest.mark.parametrize("name", SCENES)
@pytest.mark.parametrize("physical", [False, True])
def test_energy_gradient(built, ipctk, oracle_mod, name, physical):
    sc, mesh, col, ref = built(name)
    V, E, F = sc["V"], sc["E"], sc["F"]
    B = ipctk.BarrierPotential(sc["dhat"], sc["kappa"], physical)
    e = B(col, mesh, V)
    e_ref = oracle_mod.barrier_energy(ref, V, E, F, sc["dhat"], sc["kappa"], physical=physical)
    assert abs(e - e_ref) <= REL * abs(e_ref)
    g = B.gradient(col, mesh, V)
    g_ref = oracle_mod.barrier_gradient(ref, V, E, F, sc["dhat"], sc["kappa"], physical=physical)
    assert np.linalg.norm(g - g_ref) <= REL * np.linalg.norm(g_ref)


@pytest.mark.parametrize("name", SCENES)
@pytest.mark.parametrize("psd", ["none", "clamp", "abs"])
def test_hessian(built, ipctk, oracle_mod, name, psd):
    sc, mesh, col, ref = built(name)
    V, E, F = sc["V"], sc["E"], sc["F"]
    B = ipctk.BarrierPotential(sc["dhat"], sc["kappa"])
    method = {"none": ipctk.PSDProjectionMethod.NONE, "clamp": ipctk.PSDProjectionMethod.CLAMP,
              "abs": ipctk.PSDProjectionMethod.ABS}[psd]
    H = B.hessian(col, mesh, V, method)
    rp, ci, va = oracle_mod.barrier_hessian(ref, V, E, F, sc["dhat"], sc["kappa"], psd=psd)
    H_ref = sp.csr_matrix((va, ci, rp), shape=H.shape)
    assert sp.linalg.norm(H - H_ref) <= REL * sp.linalg.norm(H_ref)
    # pattern: every stored oracle entry is stored by the GPU matrix; the GPU
    # stores whole 3x3 vertex blocks, so it may hold entries the oracle skips
    # as exact zeros -- those must be zero up to the same tolerance
    Hc = H.tocsr()
    Hc.sort_indices()
    pat = sp.csr_matrix((np.ones_like(H_ref.data), H_ref.indices, H_ref.indptr), shape=H.shape)
    gpat = sp.csr_matrix((np.ones_like(Hc.data), Hc.indices, Hc.indptr), shape=H.shape)
    assert (pat - pat.multiply(gpat)).nnz == 0
    extra = Hc.multiply(gpat - pat.multiply(gpat))
    if extra.nnz:
        assert abs(extra).max() <= REL * sp.linalg.norm(H_ref)
    # symmetric
    assert sp.linalg.norm(H - H.T) <= 1e-14 * sp.linalg.norm(H)


def test_fused_matches_separate(built, ipctk):
    sc, mesh, col, _ = built("spheres_27")
    B = ipctk.BarrierPotential(sc["dhat"], sc["kappa"])
    e, g, H = B.energy_gradient_hessian(col, mesh, sc["V"], ipctk.PSDProjectionMethod.CLAMP)
    assert e == B(col, mesh, sc["V"])
    g2 = B.gradient(col, mesh, sc["V"])
    assert np.linalg.norm(g - g2) <= 1e-14 * np.linalg.norm(g2)
    H2 = B.hessian(col, mesh, sc["V"], ipctk.PSDProjectionMethod.CLAMP)
    assert sp.linalg.norm(H - H2) <= 1e-14 * sp.linalg.norm(H2)


@pytest.mark.parametrize("name", ["two_sheet_16", "two_sheet_64", "spheres_27", "spheres_64_sub2", "cloth_4x48"])
def test_collision_free_stepsize(built, ipctk, oracle_mod, name):
    sc, mesh, _, _ = built(name)
    V0, V1 = sc["V"], sc["V1"]
    step = ipctk.compute_collision_free_stepsize(mesh, V0, V1)
    ref, _ = oracle_mod.collision_free_stepsize(V0, V1, sc["E"], sc["F"])
    assert 0 <= step <= 1
    assert step == ref


def test_stepsize_no_motion_and_separated(built, ipctk):
    sc, mesh, _, _ = built("two_sheet_16")
    V = sc["V"]
    assert ipctk.compute_collision_free_stepsize(mesh, V, V) == 1.0
    # lift the upper sheet far away: full step
    V1 = V.copy()
    n = V.shape[0] // 2
    V1[n:, 2] += 0.5
    assert ipctk.compute_collision_free_stepsize(mesh, V, V1) == 1.0


def _pt_grid():
    """Point-triangle cases of tests/src/tests/distance/test_point_triangle.cpp:31-112."""
    t0, t1, t2 = np.array([-1.0, 0, 1]), np.array([1.0, 0, 1]), np.array([0.0, 0, -1])
    pts = []
    for py in (-10, -1, -1e-12, 0, 1e-12, 1, 10):
        for pz in (0, -1 + 1e-12, -1, 1, 1 - 1e-12):
            pts.append(([0, py, pz], [0, 0, pz]))
        for px in (-1, -1 - 1e-12, -11):
            pts.append(([px, py, 1], t0))
        for px in (1, 1 + 1e-12, 11):
            pts.append(([px, py, 1], t1))
        for pz in (-1, -1 - 1e-12, -11):
            pts.append(([0, py, pz], t2))
        for (a, b) in ((t0, t1), (t1, t2), (t2, t0)):
            e = np.array([b[0] - a[0], b[2] - a[2]])
            perp = np.array([-e[1], e[0]]) / np.linalg.norm(e)
            for alpha in (0.0, 1e-4, 0.5, 1 - 1e-4, 1.0):
                cp = (b - a) * alpha + a
                for scale in (0, 1e-12, 1e-4, 1, 2, 11, 1000):
                    p = np.array([cp[0] + scale * perp[0], py, cp[2] + scale * perp[1]])
                    pts.append((p, cp))
    x = np.array([[p, t0, t1, t2] for p, _ in pts], dtype=np.float64)
    cps = np.array([c for _, c in pts], dtype=np.float64)
    return x, cps


def test_point_triangle_distance_known_answers(ipctk, oracle_mod):
    x, cps = _pt_grid()
    dt, d = ipctk.distance_stencils(1, x)
    for i in range(len(x)):
        assert oracle_mod.point_triangle_distance_type(*x[i]) == dt[i]
        assert oracle_mod.point_triangle_distance(*x[i]) == d[i]
    # Catch::Approx(|p - closest|^2).margin(1e-12) of the reference test
    exp = ((x[:, 0] - cps) ** 2).sum(1)
    assert np.all(np.isclose(d, exp, rtol=100 * np.finfo(np.float32).eps, atol=1e-12))


def test_edge_edge_distance_types_match_oracle(ipctk, oracle_mod):
    rng = np.random.Generator(np.random.PCG64(4))
    x = rng.uniform(-1, 1, (4000, 4, 3))
    # near-parallel and coincident families (the two-sheet stencils)
    x[:1000, 3] = x[:1000, 2] + (x[:1000, 1] - x[:1000, 0]) * rng.uniform(0.2, 2, (1000, 1))
    x[1000:1500, 2:] = x[1000:1500, :2] + np.array([0, 0, 5e-4])
    dt, d = ipctk.distance_stencils(2, x)
    for i in range(len(x)):
        assert oracle_mod.edge_edge_distance_type(*x[i]) == dt[i]
        assert oracle_mod.edge_edge_distance(*x[i]) == d[i]
    xp = x[:, :3].copy()
    dt, d = ipctk.distance_stencils(0, xp)
    for i in range(len(xp)):
        assert oracle_mod.point_edge_distance_type(*xp[i]) == dt[i]
        assert oracle_mod.point_edge_distance(*xp[i]) == d[i]


def _pt_ccd_cases():
    """tests/src/tests/ccd/test_point_triangle_ccd.cpp:25-97."""
    eps = np.finfo(np.float32).eps
    cases = []
    for v0z in (0.0, -1.0):
        for u0y in [-v for v in (-1.0, 0.0, 0.5 - eps, 0.5, 0.5 + eps, 1.0, 2.0)]:
            for u0z in (-eps, 0.0, eps):
                for u1y in (-1.0, 0.0, 0.5 - eps, 0.5, 0.5 + eps, 1.0, 2.0):
                    x0 = np.array([[0, 1, v0z], [-1, 0, 1], [1, 0, 1], [0, 0, -1]], float)
                    x1 = x0 + np.array([[0, u0y, u0z], [0, u1y, 0], [0, u1y, 0], [0, u1y, 0]])
                    exp = (-u0y + u1y >= 1) and (v0z + u0z >= x0[3, 2])
                    cases.append((x0, x1, exp, True))
    for qy in (-eps, 0.0, eps):
        x0 = np.array([[0, qy, 0], [0, 0, 0], [0, 1, 0], [1, 0, 0]], float)
        x1 = np.array([[0, qy, 0], [0, 0, 1], [0, 1, 1], [1, 0, 1]], float)
        cases.append((x0, x1, qy >= 0, True))
    x0 = np.array([[0.1, 0.1, 0.1], [0, 0, 1], [1, 0, 1], [0, 1, 1]], float)
    x1 = np.array([[0.1, 0.1, 0.1], [0, 0, 0], [0, 1, 0], [1, 0, 0]], float)
    cases.append((x0, x1, True, True))
    x0 = np.array([[0.0133653, 0.100651, -0.0215935], [0.0100485, 0.0950896, -0.0171013],
                   [0.0130388, 0.100666, -0.0218112], [0.015413, 0.100554, -0.0202265]])
    x1 = np.array([[0.0133652999767858, 0.099670000268615, -0.0215934999996444],
                   [0.0100484999799995, 0.0941086002577558, -0.0171012999972189],
                   [0.0130387999724314, 0.0996850002629403, -0.0218111999936902],
                   [0.0154129999740718, 0.0995730002646605, -0.020226499996014]])
    cases.append((x0, x1, False, False))
    return cases


def test_point_triangle_ccd_cases(ipctk, oracle_mod):
    cases = _pt_ccd_cases()
    x0 = np.stack([c[0] for c in cases])
    x1 = np.stack([c[1] for c in cases])
    ccd = ipctk.TightInclusionCCD()
    hit, toi = ccd._batch(False, x0, x1, 0.0, 1.0)
    for i, (a, b, exp, conservative) in enumerate(cases):
        h_ref, t_ref = oracle_mod.point_triangle_ccd(a, b)
        assert bool(hit[i]) == h_ref
        if h_ref:
            assert toi[i] == t_ref
        if conservative:
            assert hit[i] or not exp
        else:
            assert bool(hit[i]) == exp


@pytest.mark.parametrize("name", ["two_sheet_16", "spheres_27", "cloth_4x48"])
def test_ccd_every_candidate_matches_oracle(built, ipctk, oracle_mod, name):
    """Every swept-box candidate of a scene, queried alone (no pruning by
    other candidates): the GPU's walk (bounded best-first heap, depth first
    past it) must return the oracle's (unbounded best-first) hit and time of
    impact exactly."""
    sc, _, _, _ = built(name)
    V0, V1, E, F = sc["V"], sc["V1"], sc["E"], sc["F"]
    ee, fv = oracle_mod.ccd_candidates(V0, V1, E, F)
    (xe0, xe1), (xf0, xf1) = oracle_mod.ccd_stencil_positions(V0, V1, E, F, ee, fv)
    rng = np.random.default_rng(7)
    ccd = ipctk.TightInclusionCCD()
    for is_ee, x0, x1 in ((True, xe0, xe1), (False, xf0, xf1)):
        if len(x0) > 4000:
            idx = rng.choice(len(x0), 4000, replace=False)
            x0, x1 = x0[idx], x1[idx]
        hit, toi = ccd._batch(is_ee, x0, x1, 0.0, 1.0)
        h_ref, t_ref, _ = oracle_mod.ccd_stencils(int(is_ee), x0, x1)
        np.testing.assert_array_equal(hit, h_ref)
        np.testing.assert_array_equal(toi[h_ref], t_ref[h_ref])
