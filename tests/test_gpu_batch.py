"""Batched scenes: a SceneBatch must give every scene exactly what the scene
gives alone.

Each scene of the batch is also built as its own CollisionMesh; the batch's
results, split per scene and shifted back to the scene's own indices, must
match:
  * collision sets: bit-exact (the batch's lists are the concatenation of the
    scenes' lists, each sorted by key);
  * energies per scene: within 1e-10 relative;
  * gradient and Hessian: the packed ones are the per-scene ones stacked
    block-diagonally, within 1e-10 relative (norms as in the other parity
    tests);
  * collision-free step per scene: identical.
One scene of the batch is also checked against the oracle directly.
"""
import numpy as np
import pytest
import scipy.sparse as sp

pytestmark = pytest.mark.gpu

REL = 1e-10


def _scenes():
    from ipctk_gb300 import scenes
    out = [
        scenes.two_sheet(side=16, seed=31),
        scenes.sphere_pack(n_side=2, subdiv=2, seed=32),
        scenes.two_sheet(side=24, gap=3e-3, jitter=4e-4, dhat=5e-3, kappa=1e2, ccd_dz=6e-3, ccd_noise=6e-4,
                         seed=33),
        scenes.layered_cloth(layers=3, side=20, seed=34),
        # a scene far from contact: empty collision set, full step
        scenes.two_sheet(side=8, gap=0.2, jitter=0.0, dhat=1e-3, ccd_dz=0.0, ccd_noise=0.0, seed=35),
        scenes.two_sheet(side=32, gap=4e-5, jitter=1e-5, dhat=1e-4, kappa=1e5, ccd_dz=8e-5, ccd_noise=8e-6,
                         seed=36),
    ]
    # overlapping coordinates on purpose: every scene sits in the unit box,
    # so only the scene split keeps them from colliding with each other
    return out


@pytest.fixture(scope="module")
def batch_setup(ipctk):
    scs = _scenes()
    batch = ipctk.SceneBatch([(s["V"], s["E"], s["F"]) for s in scs])
    V = batch.pack([s["V"] for s in scs])
    V1 = batch.pack([s["V1"] for s in scs])
    dhat = np.array([s["dhat"] for s in scs])
    kappa = np.array([s["kappa"] for s in scs])
    dmin = np.array([0.0, 0.0, 1e-4, 0.0, 0.0, 0.0])
    col = ipctk.NormalCollisions()
    col.build(batch, V, dhat, dmin)
    singles = []
    for s, dm in zip(scs, dmin):
        m = ipctk.CollisionMesh(s["V"], s["E"], s["F"])
        c = ipctk.NormalCollisions()
        c.build(m, s["V"], s["dhat"], dm)
        singles.append((m, c))
    return scs, batch, V, V1, dhat, kappa, dmin, col, singles


def _offsets(scs):
    ov = np.cumsum([0] + [s["V"].shape[0] for s in scs])
    oe = np.cumsum([0] + [s["E"].shape[0] for s in scs])
    of = np.cumsum([0] + [s["F"].shape[0] for s in scs])
    return ov, oe, of


def test_batch_collision_sets_equal_single_scenes(batch_setup):
    scs, batch, V, V1, dhat, kappa, dmin, col, singles = batch_setup
    assert batch.num_scenes == len(scs)
    ov, oe, of = _offsets(scs)
    want = {k: [] for k in ("vv", "vv_w", "ev", "ev_w", "ee", "ee_eps_x", "ee_dtype", "ee_w", "fv", "fv_w")}
    for k, (m, c) in enumerate(singles):
        a = c.to_arrays()
        shift = {"vv": np.array([ov[k], ov[k]]), "ev": np.array([oe[k], ov[k]]), "ee": np.array([oe[k], oe[k]]),
                 "fv": np.array([of[k], ov[k]])}
        for key in want:
            x = a[key]
            want[key].append(x + shift[key].astype(x.dtype) if key in shift else x)
    got = col.to_arrays()
    total = 0
    for key, parts in want.items():
        w = np.concatenate(parts)
        np.testing.assert_array_equal(got[key], w, err_msg=key)
        total += len(w) if key in ("vv", "ev", "ee", "fv") else 0
    assert len(col) == total and total > 0
    # the far-apart scene has no contacts
    assert len(singles[4][1]) == 0


def test_batch_one_scene_against_oracle(batch_setup, oracle_mod):
    scs, batch, V, V1, dhat, kappa, dmin, col, singles = batch_setup
    s = scs[2]
    ref = oracle_mod.build_collisions(s["V"], s["E"], s["F"], s["dhat"], dmin[2])
    a = singles[2][1].to_arrays()
    np.testing.assert_array_equal(a["vv"], ref.vv)
    np.testing.assert_array_equal(a["ev"], ref.ev)
    np.testing.assert_array_equal(a["ee"], ref.ee)
    np.testing.assert_array_equal(a["fv"], ref.fv)
    e_ref = oracle_mod.barrier_energy(ref, s["V"], s["E"], s["F"], s["dhat"], s["kappa"], dmin=dmin[2])
    import ipctk_gb300 as ipctk
    e = ipctk.BatchBarrierPotential(dhat, kappa)(col, batch, V)
    assert abs(e[2] - e_ref) <= REL * abs(e_ref)


@pytest.mark.parametrize("physical", [False, True])
def test_batch_energies_gradient(batch_setup, ipctk, physical):
    scs, batch, V, V1, dhat, kappa, dmin, col, singles = batch_setup
    B = ipctk.BatchBarrierPotential(dhat, kappa, physical)
    e, g, _ = B.evaluate(col, batch, V, energy=True, gradient=True)
    g_parts = batch.unpack(g)
    for k, (s, (m, c)) in enumerate(zip(scs, singles)):
        b = ipctk.BarrierPotential(s["dhat"], s["kappa"], physical)
        e1 = b(c, m, s["V"])
        assert abs(e[k] - e1) <= REL * abs(e1), (k, e[k], e1)
        g1 = b.gradient(c, m, s["V"])
        assert np.linalg.norm(g_parts[k] - g1) <= REL * np.linalg.norm(g1), k


def test_batch_gradient_into_caller_array(batch_setup, ipctk):
    # out_gradient: a pinned host array and a CUDA tensor receive the same
    # gradient as the default new array, and are what the call returns (the
    # fused energy / gradient / Hessian pass sums in a fixed order, so the
    # gradients are bit-identical)
    import torch
    scs, batch, V, V1, dhat, kappa, dmin, col, singles = batch_setup
    B = ipctk.BatchBarrierPotential(dhat, kappa)
    kw = dict(energy=True, gradient=True, hessian=True, project_hessian_to_psd=ipctk.PSDProjectionMethod.CLAMP,
              device=True)

    def run(x, **extra):
        e, g, H = B.evaluate(col, batch, x, **kw, **extra)
        H.free()
        return g

    g = run(V)
    pinned = torch.full((g.size,), np.nan, dtype=torch.float64).pin_memory()
    out = pinned.numpy()
    assert run(V, out_gradient=out) is out
    np.testing.assert_array_equal(out, g)
    gd = torch.full((g.size,), np.nan, dtype=torch.float64, device="cuda")
    assert run(torch.from_numpy(V).cuda(), out_gradient=gd) is gd
    np.testing.assert_array_equal(gd.cpu().numpy(), g)
    with pytest.raises(ValueError):
        B.evaluate(col, batch, V, energy=False, gradient=True, out_gradient=np.zeros(g.size - 3))
    with pytest.raises(ValueError):
        B.evaluate(col, batch, V, energy=False, gradient=True, out_gradient=np.zeros(g.size, np.float32))


@pytest.mark.parametrize("psd", ["none", "clamp"])
def test_batch_hessian_block_diagonal(batch_setup, ipctk, psd):
    scs, batch, V, V1, dhat, kappa, dmin, col, singles = batch_setup
    method = ipctk.PSDProjectionMethod.CLAMP if psd == "clamp" else ipctk.PSDProjectionMethod.NONE
    H = ipctk.BatchBarrierPotential(dhat, kappa).hessian(col, batch, V, method)
    blocks = [ipctk.BarrierPotential(s["dhat"], s["kappa"]).hessian(c, m, s["V"], method)
              for s, (m, c) in zip(scs, singles)]
    H_ref = sp.block_diag(blocks, format="csc")
    assert H.shape == H_ref.shape
    assert sp.linalg.norm(H - H_ref) <= REL * sp.linalg.norm(H_ref)
    # per block as well, so a small scene is not hidden by a large one
    ov = batch.vertex_offsets * 3
    for k, blk in enumerate(blocks):
        sub = H[ov[k]:ov[k + 1], ov[k]:ov[k + 1]]
        nrm = sp.linalg.norm(blk)
        assert sp.linalg.norm(sub - blk) <= REL * max(nrm, 1e-300), k


def test_batch_hessian_chunked_assembly_is_identical(batch_setup, ipctk):
    """Assembling the batch a few scenes at a time (a small chunk budget, so
    that several chunks run and some scene alone exceeds the budget) gives
    the same CSR arrays, bit for bit, as one pass over the whole batch."""
    scs, batch, V, V1, dhat, kappa, dmin, col, singles = batch_setup
    B = ipctk.BatchBarrierPotential(dhat, kappa)
    H_one = B.hessian(col, batch, V, ipctk.PSDProjectionMethod.CLAMP)
    try:
        ipctk.set_hessian_chunk_contacts(1500)
        H_chunked = B.hessian(col, batch, V, ipctk.PSDProjectionMethod.CLAMP)
    finally:
        ipctk.set_hessian_chunk_contacts(0)
    assert max(len(c) for _, c in singles) > 1500
    np.testing.assert_array_equal(H_chunked.indptr, H_one.indptr)
    np.testing.assert_array_equal(H_chunked.indices, H_one.indices)
    np.testing.assert_array_equal(H_chunked.data, H_one.data)


def test_batch_stepsizes_equal_single_scenes(batch_setup, ipctk):
    scs, batch, V, V1, dhat, kappa, dmin, col, singles = batch_setup
    md = np.array([0.0, 0.0, 1e-4, 0.0, 0.0, 0.0])
    steps = ipctk.compute_collision_free_stepsize_batch(batch, V, V1, md)
    for k, (s, (m, c)) in enumerate(zip(scs, singles)):
        one = ipctk.compute_collision_free_stepsize(m, s["V"], s["V1"], md[k])
        assert steps[k] == one, (k, steps[k], one)
    assert steps[4] == 1.0
    assert np.all(steps[[0, 2, 5]] < 1.0)


def test_batch_rejects_edge_across_scenes(ipctk):
    V = np.zeros((4, 3))
    V[:, 0] = np.arange(4)
    E = np.array([[0, 1], [1, 2], [2, 3]], np.int32)  # edge (1, 2) joins the two scenes
    lib = ipctk.lib()
    import ctypes as C
    h = C.c_void_p()
    off = np.array([0, 2, 4], np.int64)
    st = lib.ipcg_mesh_create_batch(V.ctypes.data_as(C.c_void_p), 4, E.ctypes.data_as(C.c_void_p), 3, None, 0, 2,
                                    off.ctypes.data_as(C.c_void_p), C.byref(h))
    assert st == 1
    assert b"joins two scenes" in lib.ipcg_last_error()
    # scalar entry points refuse a batch mesh
    b = ipctk.SceneBatch([(V[:2], E[:1]), (V[2:], E[:1])])
    c = ipctk.NormalCollisions()
    st = lib.ipcg_collisions_build(c._h, b._h, V.ctypes.data_as(C.c_void_p), 1e-3, 0.0)
    assert st == 1 and b"batch" in lib.ipcg_last_error()
