"""The golden fixtures of tests/golden/ (made by tests/golden/make_golden.py):
loading, and the one comparison that both the oracle (CPU) and the CUDA path
(GPU) are held to.

Bar: collision sets bit-exact (sorted index tuples, weights, EE types and
mollifier thresholds); energy within rel |e|, gradient within rel ||g||_2,
the CLAMP-projected Hessian within rel ||H||_F; the collision-free step size
identical."""
import os

import numpy as np
import scipy.sparse as sp

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
NAMES = ("two_sheet_8", "spheres_8_sub2")
SET_KEYS = ("vv", "vv_w", "ev", "ev_w", "ee", "ee_dtype", "ee_eps", "fv")


def load(name):
    with np.load(os.path.join(GOLDEN, name + ".npz"), allow_pickle=False) as z:
        return {k: z[k] for k in z.files}


def fixture_hessian(fix):
    n = fix["V"].size
    return sp.csr_matrix((fix["hess_data"], fix["hess_indices"], fix["hess_indptr"]), shape=(n, n))


def check(res, fix, rel):
    """res: the keys of SET_KEYS plus energy, gradient, hessian (a scipy
    sparse matrix) and step, computed on the fixture's inputs."""
    for k in SET_KEYS:
        np.testing.assert_array_equal(np.asarray(res[k]).reshape(fix[k].shape), fix[k], err_msg=k)
    e, e_ref = float(res["energy"]), float(fix["energy"])
    assert abs(e - e_ref) <= rel * abs(e_ref), (e, e_ref)
    g, g_ref = np.asarray(res["gradient"]).ravel(), fix["gradient"].ravel()
    assert np.linalg.norm(g - g_ref) <= rel * np.linalg.norm(g_ref)
    H_ref = fixture_hessian(fix)
    assert sp.linalg.norm(res["hessian"] - H_ref) <= rel * sp.linalg.norm(H_ref)
    assert float(res["step"]) == float(fix["step"])
