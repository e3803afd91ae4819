"""Launch shapes of the cached-pattern energy / gradient / Hessian pass.

Each contact's energy, gradient and local Hessian are computed by one lane
and summed by fixed-order reductions, so the values cannot depend on how the
work queue hands tiles to warps: every launch shape (threads per block,
resident blocks per SM, tiles per grab) must give bit-identical results.  The
autotuner must report both stages and leave the shapes it chose in force.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def small_batch(ipctk):
    from ipctk_gb300 import scenes
    scs = scenes.batch(n_scenes=12, side_lo=16, side_hi=48, seed=11)
    batch = ipctk.SceneBatch([(s["V"], s["E"], s["F"]) for s in scs])
    V = batch.pack([s["V"] for s in scs])
    dh = np.array([s["dhat"] for s in scs])
    kap = np.array([s["kappa"] for s in scs])
    col = ipctk.NormalCollisions()
    col.build(batch, V, dh)
    assert len(col) > 0
    return batch, V, dh, kap, col


def _evaluate(ipctk, small_batch, mode):
    batch, V, dh, kap, col = small_batch
    BB = ipctk.BatchBarrierPotential(dh, kap, mixed_precision=mode)
    e, g, H = BB.evaluate(col, batch, V, energy=True, gradient=True, hessian=True,
                          project_hessian_to_psd=ipctk.PSDProjectionMethod.CLAMP)
    return e, g, H


@pytest.mark.parametrize("mode", [False, "local_df64"])
def test_results_do_not_depend_on_launch_shape(ipctk, small_batch, mode):
    stages = (ipctk.STAGE_LOCAL, ipctk.STAGE_PSD, ipctk.STAGE_PSD_DF64)
    saved = [ipctk.barrier_tuning(s) for s in stages]
    try:
        ref = None
        for threads, bps, grab in ((32, 1, 1), (64, 4, 4), (128, 2, 1), (32, 16, 2)):
            for stage in stages:
                ipctk.set_barrier_tuning(stage, threads, bps, grab)
            assert ipctk.barrier_tuning(ipctk.STAGE_PSD) == {"threads": threads, "blocks_per_sm": bps,
                                                              "tiles_per_grab": grab}
            e, g, H = _evaluate(ipctk, small_batch, mode)
            if ref is None:
                ref = (e, g, H)
                continue
            np.testing.assert_array_equal(e, ref[0])
            np.testing.assert_array_equal(g, ref[1])
            np.testing.assert_array_equal(H.indptr, ref[2].indptr)
            np.testing.assert_array_equal(H.indices, ref[2].indices)
            np.testing.assert_array_equal(H.data, ref[2].data)
    finally:
        for stage, t in zip(stages, saved):
            ipctk.set_barrier_tuning(stage, t["threads"], t["blocks_per_sm"], t["tiles_per_grab"])


def test_tuning_rejects_bad_shapes(ipctk):
    with pytest.raises(ValueError):
        ipctk.set_barrier_tuning(ipctk.STAGE_LOCAL, 48, 1, 1)
    with pytest.raises(ValueError):
        ipctk.set_barrier_tuning(ipctk.STAGE_PSD, 64, 0, 1)
    with pytest.raises(ValueError):
        ipctk.set_barrier_tuning(3, 64, 1, 1)


def test_autotune_reports_both_stages(ipctk, small_batch):
    batch, V, dh, kap, col = small_batch
    saved = [ipctk.barrier_tuning(s) for s in (ipctk.STAGE_LOCAL, ipctk.STAGE_PSD_DF64)]
    try:
        BB = ipctk.BatchBarrierPotential(dh, kap, mixed_precision="local_df64")
        rep = BB.autotune(col, batch, V)
        assert rep["workload_contacts"] == len(col)
        assert rep["psd"]["stage"] == ipctk.STAGE_PSD_DF64
        for stage, name in ((ipctk.STAGE_LOCAL, "local"), (ipctk.STAGE_PSD_DF64, "psd")):
            cands = rep[name]["candidates"]
            assert len(cands) >= 3 and all(c["ms"] > 0 for c in cands)
            chosen = rep[name]["chosen"]
            assert chosen["ms"] == min(c["ms"] for c in cands)
            assert ipctk.barrier_tuning(stage) == {k: chosen[k] for k in ("threads", "blocks_per_sm",
                                                                          "tiles_per_grab")}
    finally:
        for stage, t in zip((ipctk.STAGE_LOCAL, ipctk.STAGE_PSD_DF64), saved):
            ipctk.set_barrier_tuning(stage, t["threads"], t["blocks_per_sm"], t["tiles_per_grab"])


def test_df64_fixup_pass_matches_fp64(ipctk, small_batch):
    # the FP64 fix-up pass behind the df64 projection (taken by matrices on
    # which the df64 eigensolver does not converge), forced for every
    # contact, gives the FP64 projection
    import scipy.sparse as sp
    e64, g64, H64 = _evaluate(ipctk, small_batch, False)
    ipctk.testing_defer_df64_psd(True)
    try:
        e, g, H = _evaluate(ipctk, small_batch, "psd_df64")
    finally:
        ipctk.testing_defer_df64_psd(False)
    np.testing.assert_array_equal(e, e64)
    np.testing.assert_array_equal(g, g64)
    assert sp.linalg.norm(sp.csr_matrix(H) - sp.csr_matrix(H64)) <= 1e-14 * sp.linalg.norm(sp.csr_matrix(H64))
    # and without the switch df64 stays within its own accuracy
    e2, g2, H2 = _evaluate(ipctk, small_batch, "psd_df64")
    assert sp.linalg.norm(sp.csr_matrix(H2) - sp.csr_matrix(H64)) <= 1e-12 * sp.linalg.norm(sp.csr_matrix(H64))
