"""The step-size passes (ccd.cu): every query gets a lower bound on its time
of impact and is skipped when that bound is not before its scene's earliest
impact so far; each scene's likeliest impacts run first as seeds with a warp
per query; the rest run one thread per query with a box budget, and what
exceeds it runs again with a warp per query.  None of this may change a step
size: the steps must equal the oracle's (ipc.cpp:42-106 with
tight_inclusion_ccd.cpp:33-336) with the default budget and with a budget of
one box, which sends every query that is not skipped through the warp search.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _scenes():
    from ipctk_gb300 import scenes
    out = [("two_sheet", scenes.two_sheet()), ("sphere_pack", scenes.sphere_pack())]
    b = scenes.batch()
    out += [(f"batch{k}", b[k]) for k in (0, 8, 40)]
    return out


@pytest.fixture(scope="module")
def refs(oracle_mod):
    return {name: oracle_mod.collision_free_stepsize(sc["V"], sc["V1"], sc["E"], sc["F"])[0]
            for name, sc in _scenes()}


@pytest.mark.parametrize("budget", [0, 1, 16])
def test_steps_equal_oracle_for_any_budget(ipctk, refs, budget):
    ipctk.testing_ccd_budget(budget)
    try:
        for name, sc in _scenes():
            mesh = ipctk.CollisionMesh(sc["V"], sc["E"], sc["F"])
            assert ipctk.compute_collision_free_stepsize(mesh, sc["V"], sc["V1"]) == refs[name], (name, budget)
    finally:
        ipctk.testing_ccd_budget(0)


def test_pass_statistics(ipctk):
    # the colliding two-sheet scene: seeds find impacts, most queries are
    # skipped, and the warp pass takes only what exceeds the budget
    from ipctk_gb300 import scenes
    sc = scenes.two_sheet()
    mesh = ipctk.CollisionMesh(sc["V"], sc["E"], sc["F"])
    ipctk.testing_ccd_stats(mesh, True)
    try:
        step = ipctk.compute_collision_free_stepsize(mesh, sc["V"], sc["V1"])
        st = ipctk.testing_ccd_stats(mesh, False)
    finally:
        ipctk.testing_ccd_stats(mesh, False)
    assert 0 < step < 1
    assert st["seeds"]["queries"] > 0 and st["seeds"]["hits"] > 0
    n_cand = ipctk.Candidates()
    n_cand.build(mesh, sc["V"], sc["V1"])
    assert st["budgeted"]["queries"] < 0.5 * len(n_cand)
