"""Friction on the device against the oracle: TangentialCollisions::build
(stencils and weights exact; normal forces, closest points, tangent bases and
blended mu within 1e-12 relative) and FrictionPotential energy, gradient and
Hessian within 1e-10 relative, in the static, transition and kinetic regimes."""
import numpy as np
import pytest
import scipy.sparse as sp

from test_gpu_parity import REL, _scene

pytestmark = pytest.mark.gpu

NAMES = ["two_sheet_16", "two_sheet_64", "spheres_27", "cloth_4x48"]
EPS_V = 1e-3


def _setup(ipctk, oracle_mod, name, improved=False, physical=False):
    sc = _scene(name)
    V, E, F = sc["V"], sc["E"], sc["F"]
    mesh = ipctk.CollisionMesh(V, E, F)
    col = ipctk.NormalCollisions()
    if improved:
        col.use_area_weighting = True
        col.collision_set_type = ipctk.NormalCollisions.CollisionSetType.IMPROVED_MAX_APPROX
    col.build(mesh, V, sc["dhat"])
    ref = oracle_mod.build_collisions(V, E, F, sc["dhat"], area_weighting=improved, improved_max_approx=improved)
    rng = np.random.Generator(np.random.PCG64(17))
    mu_s = rng.uniform(0.3, 0.6, len(V))
    mu_k = mu_s * rng.uniform(0.6, 1.0, len(V))
    B = ipctk.BarrierPotential(sc["dhat"], sc["kappa"], physical)
    tc = ipctk.TangentialCollisions()
    tc.build(mesh, V, col, B, mu_s, mu_k)
    tref = oracle_mod.tangential_build(ref, V, E, F, sc["dhat"], sc["kappa"], mu_s, mu_k, physical=int(physical))
    return sc, mesh, tc, tref, rng


def _close(a, b, rel=1e-12):
    a, b = np.asarray(a, float).ravel(), np.asarray(b, float).ravel()
    assert a.shape == b.shape
    assert np.linalg.norm(a - b) <= rel * max(np.linalg.norm(b), 1e-300)


@pytest.mark.parametrize("name", NAMES)
def test_tangential_build(ipctk, oracle_mod, name):
    sc, mesh, tc, tref, _ = _setup(ipctk, oracle_mod, name)
    a = tc.to_arrays()
    assert len(tc) == len(tref) > 0
    for k in ("vv", "ev", "ee", "fv"):
        np.testing.assert_array_equal(a[k], getattr(tref, k), err_msg=k)
    np.testing.assert_array_equal(a["weight"], tref.w)
    _close(a["normal_force"], tref.N)
    _close(a["closest_point"], tref.cp)
    _close(a["tangent_basis"].transpose(0, 2, 1).reshape(-1, 6), tref.P)
    _close(a["mu_s"], tref.mu_s)
    _close(a["mu_k"], tref.mu_k)


@pytest.mark.parametrize("name", NAMES)
@pytest.mark.parametrize("regime", ["static", "mixed", "kinetic"])
def test_friction_potential(ipctk, oracle_mod, name, regime):
    sc, mesh, tc, tref, rng = _setup(ipctk, oracle_mod, name)
    E, F = sc["E"], sc["F"]
    U = rng.uniform(-1, 1, sc["V"].shape) * {"static": 0.2, "mixed": 1.0, "kinetic": 20.0}[regime] * EPS_V
    D = ipctk.FrictionPotential(EPS_V)
    e = D(tc, mesh, U)
    e_ref = oracle_mod.friction_energy(tref, U, E, F, EPS_V)
    assert abs(e - e_ref) <= REL * abs(e_ref)
    g = D.gradient(tc, mesh, U)
    g_ref = oracle_mod.friction_gradient(tref, U, E, F, EPS_V)
    assert np.linalg.norm(g - g_ref) <= REL * np.linalg.norm(g_ref)
    for psd, method in (("none", ipctk.PSDProjectionMethod.NONE), ("clamp", ipctk.PSDProjectionMethod.CLAMP),
                        ("abs", ipctk.PSDProjectionMethod.ABS)):
        H = D.hessian(tc, mesh, U, method)
        rp, ci, va = oracle_mod.friction_hessian(tref, U, E, F, EPS_V, psd=psd)
        H_ref = sp.csr_matrix((va, ci, rp), shape=H.shape)
        assert sp.linalg.norm(H - H_ref) <= REL * sp.linalg.norm(H_ref), psd
        assert sp.linalg.norm(H - H.T) <= 1e-13 * sp.linalg.norm(H)


@pytest.mark.parametrize("name", ["two_sheet_16", "cloth_4x48"])
def test_friction_on_improved_physical_set(ipctk, oracle_mod, name):
    """Negative weights of the improved set reach the w N <= 0 branches."""
    sc, mesh, tc, tref, rng = _setup(ipctk, oracle_mod, name, improved=True, physical=True)
    a = tc.to_arrays()
    assert np.any(a["weight"] < 0)
    _close(a["normal_force"], tref.N)
    E, F = sc["E"], sc["F"]
    U = rng.uniform(-1, 1, sc["V"].shape) * EPS_V
    D = ipctk.FrictionPotential(EPS_V)
    e = D(tc, mesh, U)
    assert abs(e - oracle_mod.friction_energy(tref, U, E, F, EPS_V)) <= REL * abs(e)
    H = D.hessian(tc, mesh, U, ipctk.PSDProjectionMethod.CLAMP)
    rp, ci, va = oracle_mod.friction_hessian(tref, U, E, F, EPS_V, psd="clamp")
    H_ref = sp.csr_matrix((va, ci, rp), shape=H.shape)
    assert sp.linalg.norm(H - H_ref) <= REL * sp.linalg.norm(H_ref)


def test_friction_device_inputs(ipctk, oracle_mod):
    torch = pytest.importorskip("torch")
    sc, mesh, tc, tref, rng = _setup(ipctk, oracle_mod, "spheres_27")
    U = rng.uniform(-1, 1, sc["V"].shape) * EPS_V
    D = ipctk.FrictionPotential(EPS_V)
    g_host = D.gradient(tc, mesh, U)
    g_dev = D.gradient(tc, mesh, torch.from_numpy(U).cuda())
    assert np.linalg.norm(g_dev.cpu().numpy() - g_host) <= 1e-14 * np.linalg.norm(g_host)


def test_friction_fused_matches_separate(ipctk, oracle_mod):
    sc, mesh, tc, tref, rng = _setup(ipctk, oracle_mod, "two_sheet_16")
    U = rng.uniform(-1, 1, sc["V"].shape) * EPS_V
    D = ipctk.FrictionPotential(EPS_V)
    e, g, H = D.energy_gradient_hessian(tc, mesh, U, ipctk.PSDProjectionMethod.CLAMP)
    assert e == D(tc, mesh, U)
    g2 = D.gradient(tc, mesh, U)  # atomics: summation order may differ
    assert np.linalg.norm(g - g2) <= 1e-14 * np.linalg.norm(g2)
    H2 = D.hessian(tc, mesh, U, ipctk.PSDProjectionMethod.CLAMP)
    assert sp.linalg.norm(H - H2) == 0


@pytest.mark.parametrize("name", ["two_sheet_16", "spheres_27", "cloth_4x48"])
def test_anisotropic_friction(ipctk, oracle_mod, name):
    """Slip scaling and lagged directional coefficients
    (tangential_collisions.cpp:387-420, smooth_mu.cpp:117-171): lagged mu within
    1e-12, energy, gradient and Hessian within 1e-10 of the oracle."""
    sc, mesh, tc, tref, rng = _setup(ipctk, oracle_mod, name)
    V, E, F = sc["V"], sc["E"], sc["F"]
    n = len(tc)
    aniso = rng.uniform(0.5, 2.0, (n, 2))
    ms_a = rng.uniform(0.2, 0.8, (n, 2))
    ms_a[::5] = 0  # some collisions stay isotropic
    mk_a = rng.uniform(0.1, 0.5, (n, 2))
    mk_a[::7] = 0
    tc.set_anisotropy(aniso, ms_a, mk_a)
    oracle_mod.tangential_set_anisotropy(tref, aniso, ms_a, mk_a)
    lag = rng.uniform(-1, 1, V.shape) * 0.05 * sc["dhat"]
    U = rng.uniform(-1, 1, V.shape) * EPS_V
    tc.update_lagged_anisotropic_friction_coefficients(mesh, V, lag, U)
    oracle_mod.tangential_update_lagged_mu(tref, V, lag, U, E, F)
    ms, mk = tc.lagged_mu()
    rms, rmk = oracle_mod.tangential_lagged_mu(tref)
    _close(ms, rms)
    _close(mk, rmk)
    D = ipctk.FrictionPotential(EPS_V)
    e, g, H = D.energy_gradient_hessian(tc, mesh, U, ipctk.PSDProjectionMethod.CLAMP)
    e_ref = oracle_mod.friction_energy(tref, U, E, F, EPS_V)
    assert abs(e - e_ref) <= REL * abs(e_ref)
    g_ref = oracle_mod.friction_gradient(tref, U, E, F, EPS_V)
    assert np.linalg.norm(g - g_ref) <= REL * np.linalg.norm(g_ref)
    rp, ci, va = oracle_mod.friction_hessian(tref, U, E, F, EPS_V, psd="clamp")
    H_ref = sp.csr_matrix((va, ci, rp), shape=H.shape)
    assert sp.linalg.norm(H - H_ref) <= REL * sp.linalg.norm(H_ref)
    # reset: back to the scalar coefficients
    tc.reset_lagged_anisotropic_friction_coefficients()
    a = tc.to_arrays()
    ms, mk = tc.lagged_mu()
    np.testing.assert_array_equal(ms, a["mu_s"])
    np.testing.assert_array_equal(mk, a["mu_k"])


@pytest.mark.parametrize("name", ["two_sheet_16", "spheres_27"])
@pytest.mark.parametrize("no_mu", [False, True])
def test_friction_force(ipctk, oracle_mod, name, no_mu):
    """TangentialPotential::force at lagged positions, with anisotropy, against
    the oracle within 1e-10 relative."""
    sc, mesh, tc, tref, rng = _setup(ipctk, oracle_mod, name, physical=True)
    V, E, F = sc["V"], sc["E"], sc["F"]
    n = len(tc)
    aniso = rng.uniform(0.5, 2.0, (n, 2))
    tc.set_anisotropy(aniso)
    oracle_mod.tangential_set_anisotropy(tref, aniso)
    lag = rng.uniform(-1, 1, V.shape) * 0.05 * sc["dhat"]
    U = rng.uniform(-1, 1, V.shape) * EPS_V
    B = ipctk.BarrierPotential(sc["dhat"], sc["kappa"], True)
    D = ipctk.FrictionPotential(EPS_V)
    f = D.force(tc, mesh, V, lag, U, B, no_mu=no_mu)
    f_ref = oracle_mod.friction_force(tref, V, lag, U, E, F, sc["dhat"], sc["kappa"], EPS_V, physical=1, no_mu=no_mu)
    assert np.linalg.norm(f_ref) > 0
    assert np.linalg.norm(f - f_ref) <= REL * np.linalg.norm(f_ref)


def test_friction_batch_equals_scenes(ipctk):
    """Friction on a SceneBatch: per-scene energies, the packed gradient and
    the block-diagonal Hessian equal each scene's own evaluation."""
    from ipctk_gb300 import scenes
    parts = [scenes.two_sheet(side=s, seed=s) for s in (8, 12, 16)]
    batch = ipctk.SceneBatch([(p["V"], p["E"], p["F"]) for p in parts])
    V = np.concatenate([p["V"] for p in parts])
    dh = [p["dhat"] for p in parts]
    kap = [p["kappa"] for p in parts]
    col = ipctk.NormalCollisions()
    col.build(batch, V, dh)
    tc = ipctk.TangentialCollisions()
    tc.build(batch, V, col, ipctk.BatchBarrierPotential(dh, kap), 0.5, 0.4)
    rng = np.random.Generator(np.random.PCG64(2))
    U = rng.uniform(-1, 1, V.shape) * EPS_V
    D = ipctk.FrictionPotential(EPS_V)
    e, g, H = D.energy_gradient_hessian(tc, batch, U, ipctk.PSDProjectionMethod.CLAMP)
    off = 0
    blocks = []
    for k, p in enumerate(parts):
        n = len(p["V"])
        m = ipctk.CollisionMesh(p["V"], p["E"], p["F"])
        c = ipctk.NormalCollisions()
        c.build(m, p["V"], p["dhat"])
        t = ipctk.TangentialCollisions()
        t.build(m, p["V"], c, ipctk.BarrierPotential(p["dhat"], p["kappa"]), 0.5, 0.4)
        ek, gk, Hk = D.energy_gradient_hessian(t, m, U[off:off + n], ipctk.PSDProjectionMethod.CLAMP)
        assert e[k] == pytest.approx(ek, rel=1e-12)
        np.testing.assert_allclose(g[3 * off:3 * (off + n)], gk, rtol=0, atol=1e-14 * np.abs(gk).max())
        blocks.append(Hk)
        off += n
    Hb = sp.block_diag(blocks)
    assert sp.linalg.norm(H - Hb) <= 1e-14 * sp.linalg.norm(Hb)
