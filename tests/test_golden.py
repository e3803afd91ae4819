"""The committed golden fixtures (tests/golden/*.npz) against the CPU oracle:
the oracle still reproduces them, and they cover every contact type."""
import importlib.util
import os

import numpy as np
import pytest
import scipy.sparse as sp

import golden_util


def make_golden():
    path = os.path.join(golden_util.GOLDEN, "make_golden.py")
    spec = importlib.util.spec_from_file_location("make_golden", path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


@pytest.mark.parametrize("name", golden_util.NAMES)
def test_oracle_reproduces_fixture(oracle_mod, name):
    fix = golden_util.load(name)
    out = make_golden().oracle_outputs(oracle_mod, fix["V"], fix["V1"], fix["E"], fix["F"], float(fix["dhat"]),
                                       float(fix["kappa"]))
    n = fix["V"].size
    res = dict(out)
    res["hessian"] = sp.csr_matrix((out["hess_data"], out["hess_indices"], out["hess_indptr"]), shape=(n, n))
    golden_util.check(res, fix, rel=1e-12)


def test_fixtures_cover_every_contact_type():
    fixes = [golden_util.load(n) for n in golden_util.NAMES]
    for fix in fixes:
        assert 0 < float(fix["step"]) <= 1
        assert golden_util.fixture_hessian(fix).nnz > 0
    for k in ("vv", "ev", "ee", "fv"):
        assert sum(len(f[k]) for f in fixes) > 0, k
    # every edge-edge record carries its mollifier threshold eps_x > 0
    assert all((f["ee_eps"] > 0).all() for f in fixes)


def test_check_rejects_a_changed_fixture(oracle_mod):
    # the comparison is not vacuous: one flipped EE type or a 1e-9 energy change fails it
    fix = golden_util.load("two_sheet_8")
    out = make_golden().oracle_outputs(oracle_mod, fix["V"], fix["V1"], fix["E"], fix["F"], float(fix["dhat"]),
                                       float(fix["kappa"]))
    n = fix["V"].size
    res = dict(out)
    res["hessian"] = sp.csr_matrix((out["hess_data"], out["hess_indices"], out["hess_indptr"]), shape=(n, n))
    bad = dict(res)
    bad["ee_dtype"] = res["ee_dtype"].copy()
    bad["ee_dtype"][0] = (bad["ee_dtype"][0] + 1) % 9
    with pytest.raises(AssertionError):
        golden_util.check(bad, fix, rel=1e-12)
    bad = dict(res)
    bad["energy"] = float(res["energy"]) * (1 + 1e-9)
    with pytest.raises(AssertionError):
        golden_util.check(bad, fix, rel=1e-10)
