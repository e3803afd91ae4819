"""Collision-set and potential variants against the oracle: the other barrier
functions (barrier.cpp:47-154) through BarrierPotential, and the
Gauss-Newton Hessian diagonal and quadratic form (normal_potential.cpp:15-83,
236-308).  Tolerance: 1e-10 relative, as for the default barrier."""
import numpy as np
import pytest
import scipy.sparse as sp

from test_gpu_parity import REL, _scene

pytestmark = pytest.mark.gpu

KINDS = ["ClampedLogBarrier", "NormalizedClampedLogBarrier", "ClampedLogSqBarrier", "CubicBarrier",
         "TwoStageBarrier"]


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


@pytest.mark.parametrize("name", ["two_sheet_16", "spheres_27", "cloth_4x48"])
@pytest.mark.parametrize("kind", KINDS)
@pytest.mark.parametrize("physical", [False, True])
def test_barrier_functions(built, ipctk, oracle_mod, name, kind, physical):
    sc, mesh, col, ref = built(name)
    V, E, F = sc["V"], sc["E"], sc["F"]
    barrier = getattr(ipctk, kind)()
    B = ipctk.BarrierPotential(barrier, sc["dhat"], sc["kappa"], physical)
    bits = int(physical) | (barrier.kind << 4)
    e, g, H = B.energy_gradient_hessian(col, mesh, V, ipctk.PSDProjectionMethod.CLAMP)
    e_ref = oracle_mod.barrier_energy(ref, V, E, F, sc["dhat"], sc["kappa"], physical=bits)
    assert abs(e - e_ref) <= REL * abs(e_ref)
    g_ref = oracle_mod.barrier_gradient(ref, V, E, F, sc["dhat"], sc["kappa"], physical=bits)
    assert np.linalg.norm(g - g_ref) <= REL * np.linalg.norm(g_ref)
    rp, ci, va = oracle_mod.barrier_hessian(ref, V, E, F, sc["dhat"], sc["kappa"], physical=bits, psd="clamp")
    H_ref = sp.csr_matrix((va, ci, rp), shape=H.shape)
    assert sp.linalg.norm(H - H_ref) <= REL * sp.linalg.norm(H_ref)


def test_barrier_host_functions_match_oracle(ipctk, oracle_mod):
    for kind in KINDS:
        b = getattr(ipctk, kind)()
        for dh in (1e-6, 1e-3, 1.0):
            for r in (1e-3, 0.3, 0.5, 0.7, 0.999, 1.5):
                d = r * dh
                for k, f in enumerate((b, b.first_derivative, b.second_derivative)):
                    assert f(d, dh) == oracle_mod.barrier(d, dh, k, b.kind)


@pytest.mark.parametrize("name", ["two_sheet_16", "two_sheet_64", "spheres_27", "cloth_4x48"])
@pytest.mark.parametrize("kind", ["ClampedLogBarrier", "CubicBarrier"])
def test_gauss_newton_forms(built, ipctk, oracle_mod, name, kind):
    sc, mesh, col, ref = built(name)
    V, E, F = sc["V"], sc["E"], sc["F"]
    barrier = getattr(ipctk, kind)()
    B = ipctk.BarrierPotential(barrier, sc["dhat"], sc["kappa"])
    bits = barrier.kind << 4
    d = B.gauss_newton_hessian_diagonal(col, mesh, V)
    d_ref = oracle_mod.barrier_gauss_newton_diagonal(ref, V, E, F, sc["dhat"], sc["kappa"], physical=bits)
    assert np.linalg.norm(d_ref) > 0
    assert np.linalg.norm(d - d_ref) <= REL * np.linalg.norm(d_ref)
    rng = np.random.Generator(np.random.PCG64(7))
    p = rng.standard_normal(V.size)
    q = B.gauss_newton_hessian_quadratic_form(col, mesh, V, p)
    q_ref = oracle_mod.barrier_gauss_newton_quadratic_form(ref, V, E, F, p, sc["dhat"], sc["kappa"], physical=bits)
    assert abs(q - q_ref) <= REL * abs(q_ref)
    # the quadratic form along a coordinate axis is that diagonal entry
    i = int(np.argmax(np.abs(d_ref)))
    ei = np.zeros(V.size)
    ei[i] = 1.0
    assert B.gauss_newton_hessian_quadratic_form(col, mesh, V, ei) == pytest.approx(d[i], rel=1e-12)


def test_gauss_newton_device_inputs(built, ipctk):
    torch = pytest.importorskip("torch")
    sc, mesh, col, _ = built("spheres_27")
    B = ipctk.BarrierPotential(sc["dhat"], sc["kappa"])
    Vd = torch.from_numpy(sc["V"]).cuda()
    d_host = B.gauss_newton_hessian_diagonal(col, mesh, sc["V"])
    d_dev = B.gauss_newton_hessian_diagonal(col, mesh, Vd)
    assert np.linalg.norm(d_dev.cpu().numpy() - d_host) <= 1e-14 * np.linalg.norm(d_host)
    p = np.linspace(-1, 1, sc["V"].size)
    q_host = B.gauss_newton_hessian_quadratic_form(col, mesh, sc["V"], p)
    q_dev = B.gauss_newton_hessian_quadratic_form(col, mesh, Vd, torch.from_numpy(p).cuda())
    assert q_dev == q_host
