"""Parity at the benchmark's own sizes.

The benchmark times two workloads; both are held to the oracle here:
  * the full 512-icosphere sphere pack (328,704 vertices, 31,066 contacts):
    collision set bit-exact, energy / gradient / CLAMP Hessian within 1e-10
    relative, step size identical;
  * sixteen scenes of the 256-scene batch, one from each sixteenth of its
    dhat range (the smallest scene of each bin, so the oracle stays quick),
    evaluated together as a SceneBatch: per scene the collision set
    bit-exact, energy / gradient / Hessian within 1e-10 in FP64 and with the
    projection's eigenpairs in df64 (IPCG_BARRIER_DF64_PSD), within 1e-6 in
    the mixed modes the benchmark runs (IPCG_BARRIER_FP32_LOCAL, with and
    without df64 eigenpairs), and the batched step sizes identical to the
    oracle's.
Norms as in the other parity tests: |a-b| <= tol |b| for energies,
||a-b||_2 <= tol ||b||_2 for gradients, ||A-B||_F <= tol ||B||_F for
Hessians (the reference skips exact-zero local entries; whole blocks are
stored here, so the comparison is by value).
"""
import numpy as np
import pytest
import scipy.sparse as sp

pytestmark = pytest.mark.gpu

REL = 1e-10
MIXED_REL = 1e-6


def _assert_set(a, ref, vshift=0, eshift=0, fshift=0):
    np.testing.assert_array_equal(a["vv"] - vshift, np.asarray(ref.vv).reshape(-1, 2))
    np.testing.assert_array_equal(a["vv_w"], ref.vv_w)
    ev = a["ev"].copy()
    ev[:, 0] -= eshift
    ev[:, 1] -= vshift
    np.testing.assert_array_equal(ev, np.asarray(ref.ev).reshape(-1, 2))
    np.testing.assert_array_equal(a["ev_w"], ref.ev_w)
    np.testing.assert_array_equal(a["ee"] - eshift, np.asarray(ref.ee).reshape(-1, 2))
    np.testing.assert_array_equal(a["ee_dtype"], ref.ee_dtype)
    np.testing.assert_array_equal(a["ee_eps_x"], ref.ee_eps)
    fv = a["fv"].copy()
    fv[:, 0] -= fshift
    fv[:, 1] -= vshift
    np.testing.assert_array_equal(fv, np.asarray(ref.fv).reshape(-1, 2))


def test_sphere_pack_full_size(ipctk, oracle_mod):
    from ipctk_gb300 import scenes
    sc = scenes.sphere_pack()
    V, E, F, V1 = sc["V"], sc["E"], sc["F"], sc["V1"]
    mesh = ipctk.CollisionMesh(V, E, F)
    col = ipctk.NormalCollisions()
    col.build(mesh, V, sc["dhat"])
    ref = oracle_mod.build_collisions(V, E, F, sc["dhat"])
    assert len(col) == len(ref) == 31066
    _assert_set(col.to_arrays(), ref)
    B = ipctk.BarrierPotential(sc["dhat"], sc["kappa"])
    e, g, H = B.energy_gradient_hessian(col, mesh, V, ipctk.PSDProjectionMethod.CLAMP)
    e_ref = oracle_mod.barrier_energy(ref, V, E, F, sc["dhat"], sc["kappa"])
    g_ref = oracle_mod.barrier_gradient(ref, V, E, F, sc["dhat"], sc["kappa"])
    rp, ci, va = oracle_mod.barrier_hessian(ref, V, E, F, sc["dhat"], sc["kappa"], psd="clamp")
    H_ref = sp.csr_matrix((va, ci, rp), shape=H.shape)
    assert abs(e - e_ref) <= REL * abs(e_ref)
    assert np.linalg.norm(g - g_ref) <= REL * np.linalg.norm(g_ref)
    assert sp.linalg.norm(H - H_ref) <= REL * sp.linalg.norm(H_ref)
    step = ipctk.compute_collision_free_stepsize(mesh, V, V1)
    step_ref, _ = oracle_mod.collision_free_stepsize(V, V1, E, F)
    assert step == step_ref
    # the df64 projection meets the FP64 tolerance on the same set
    B64 = ipctk.BarrierPotential(sc["dhat"], sc["kappa"], mixed_precision="psd_df64")
    e2, g2, H2 = B64.energy_gradient_hessian(col, mesh, V, ipctk.PSDProjectionMethod.CLAMP)
    assert e2 == e and np.array_equal(g2, g)
    assert sp.linalg.norm(H2 - H_ref) <= REL * sp.linalg.norm(H_ref)
    assert sp.linalg.norm(H2 - H) <= 1e-12 * sp.linalg.norm(H)


def _batch_sample():
    from ipctk_gb300 import scenes
    scs = scenes.batch()
    order = sorted(range(len(scs)), key=lambda k: scs[k]["dhat"])
    pick = [min(b, key=lambda k: scs[k]["V"].shape[0]) for b in np.array_split(order, 16)]
    return [scs[k] for k in pick]


@pytest.fixture(scope="module")
def batch16(ipctk, oracle_mod):
    scs = _batch_sample()
    batch = ipctk.SceneBatch([(s["V"], s["E"], s["F"]) for s in scs])
    V = batch.pack([s["V"] for s in scs])
    dh = np.array([s["dhat"] for s in scs])
    kap = np.array([s["kappa"] for s in scs])
    col = ipctk.NormalCollisions()
    col.build(batch, V, dh)
    refs = [oracle_mod.build_collisions(s["V"], s["E"], s["F"], s["dhat"]) for s in scs]
    return scs, batch, V, dh, kap, col, refs


def test_batch_sample_spans_dhat(batch16):
    scs = batch16[0]
    dh = sorted(s["dhat"] for s in scs)
    assert len(scs) == 16 and dh[0] < 2e-4 and dh[-1] > 5e-3


def test_batch_sample_collision_sets(batch16):
    scs, batch, V, dh, kap, col, refs = batch16
    a = col.to_arrays()
    voff = batch.vertex_offsets
    eoff = np.cumsum([0] + [s["E"].shape[0] for s in scs])
    foff = np.cumsum([0] + [s["F"].shape[0] for s in scs])
    assert len(col) == sum(len(r) for r in refs) > 0
    for k, (s, ref) in enumerate(zip(scs, refs)):
        sl = {}
        for key, lo, hi in (("vv", voff[k], voff[k + 1]), ("ev", eoff[k], eoff[k + 1]),
                            ("ee", eoff[k], eoff[k + 1]), ("fv", foff[k], foff[k + 1])):
            m = (a[key][:, 0] >= lo) & (a[key][:, 0] < hi)
            sl[key] = a[key][m]
            extra = {"vv": ("vv_w",), "ev": ("ev_w",), "ee": ("ee_dtype", "ee_eps_x"), "fv": ()}[key]
            for x in extra:
                sl[x] = a[x][m]
        _assert_set(sl, ref, vshift=voff[k], eshift=eoff[k], fshift=foff[k])


# "psd_df64": FP64 local Hessians, projection eigenpairs in df64 -- held to
# the FP64 tolerance; "local_df64": the benchmark's mixed mode with them
@pytest.mark.parametrize("mode,tol", [(False, REL), ("local", MIXED_REL), ("psd_df64", REL),
                                      ("local_df64", MIXED_REL)])
def test_batch_sample_potential(ipctk, oracle_mod, batch16, mode, tol):
    scs, batch, V, dh, kap, col, refs = batch16
    BB = ipctk.BatchBarrierPotential(dh, kap, mixed_precision=mode)
    e, g, H = BB.evaluate(col, batch, V, energy=True, gradient=True, hessian=True,
                          project_hessian_to_psd=ipctk.PSDProjectionMethod.CLAMP)
    H = sp.csr_matrix(H)
    voff = batch.vertex_offsets
    for k, (s, ref) in enumerate(zip(scs, refs)):
        Vk, Ek, Fk = s["V"], s["E"], s["F"]
        e_ref = oracle_mod.barrier_energy(ref, Vk, Ek, Fk, s["dhat"], s["kappa"])
        assert abs(e[k] - e_ref) <= tol * abs(e_ref), (k, e[k], e_ref)
        g_ref = oracle_mod.barrier_gradient(ref, Vk, Ek, Fk, s["dhat"], s["kappa"])
        gk = g[3 * voff[k]:3 * voff[k + 1]]
        assert np.linalg.norm(gk - g_ref) <= tol * np.linalg.norm(g_ref), k
        rp, ci, va = oracle_mod.barrier_hessian(ref, Vk, Ek, Fk, s["dhat"], s["kappa"], psd="clamp")
        n = 3 * Vk.shape[0]
        H_ref = sp.csr_matrix((va, ci, rp), shape=(n, n))
        Hk = H[3 * voff[k]:3 * voff[k + 1], 3 * voff[k]:3 * voff[k + 1]]
        assert sp.linalg.norm(Hk - H_ref) <= tol * sp.linalg.norm(H_ref), k
    # the packed Hessian is block diagonal over the scenes
    coo = H.tocoo()
    scene_of = np.searchsorted(3 * voff, np.arange(H.shape[0]), side="right") - 1
    assert np.all(scene_of[coo.row] == scene_of[coo.col])


def test_batch_sample_step_sizes(ipctk, oracle_mod, batch16):
    scs, batch, V, dh, kap, col, refs = batch16
    V1 = batch.pack([s["V1"] for s in scs])
    steps = ipctk.compute_collision_free_stepsize_batch(batch, V, V1)
    for k, s in enumerate(scs):
        step_ref, _ = oracle_mod.collision_free_stepsize(s["V"], s["V1"], s["E"], s["F"])
        assert steps[k] == step_ref, (k, steps[k], step_ref)
