"""The CUDA path (through the C ABI) against the committed golden fixtures of
tests/golden/ (inputs and oracle outputs stored together), with the bar of
the GPU parity tests: collision sets bit-exact, energy / gradient / CLAMP
Hessian within 1e-10 relative, step size identical."""
import pytest

import golden_util

pytestmark = pytest.mark.gpu

REL = 1e-10


@pytest.mark.parametrize("name", golden_util.NAMES)
def test_cuda_path_matches_fixture(ipctk, name):
    fix = golden_util.load(name)
    V, V1, E, F = fix["V"], fix["V1"], fix["E"], fix["F"]
    dhat, kappa = float(fix["dhat"]), float(fix["kappa"])
    mesh = ipctk.CollisionMesh(V, E, F)
    col = ipctk.NormalCollisions()
    col.build(mesh, V, dhat)
    a = col.to_arrays()
    B = ipctk.BarrierPotential(dhat, kappa)
    res = {"vv": a["vv"], "vv_w": a["vv_w"], "ev": a["ev"], "ev_w": a["ev_w"], "ee": a["ee"],
           "ee_dtype": a["ee_dtype"], "ee_eps": a["ee_eps_x"], "fv": a["fv"],
           "energy": B(col, mesh, V), "gradient": B.gradient(col, mesh, V),
           "hessian": B.hessian(col, mesh, V, ipctk.PSDProjectionMethod.CLAMP),
           "step": ipctk.compute_collision_free_stepsize(mesh, V, V1)}
    golden_util.check(res, fix, REL)
