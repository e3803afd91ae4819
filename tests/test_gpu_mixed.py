"""Mixed precision (IPCG_BARRIER_FP32_PT): face-vertex contacts in FP32,
everything else FP64.  The collision set is untouched (its FP64 filter is
the same), and energy, gradient and Hessian stay within 1e-6 relative of the
FP64 oracle (|a-b| <= 1e-6 |b|; 2-norm for the gradient, Frobenius for the
Hessian).  The measured errors are printed (pytest -s)."""
import numpy as np
import pytest
import scipy.sparse as sp

pytestmark = pytest.mark.gpu

TOL = 1e-6


@pytest.mark.parametrize("name", ["spheres_27", "cloth_4x48", "two_sheet_64"])
def test_mixed_precision_within_1e6_of_oracle(ipctk, oracle_mod, name):
    from test_gpu_parity import _scene
    sc = _scene(name)
    V, E, F = sc["V"], sc["E"], sc["F"]
    mesh = ipctk.CollisionMesh(V, E, F)
    col = ipctk.NormalCollisions()
    col.build(mesh, V, sc["dhat"])
    ref = oracle_mod.build_collisions(V, E, F, sc["dhat"])
    assert len(col) == len(ref) and int(col.counts()[3]) > 0
    B = ipctk.BarrierPotential(sc["dhat"], sc["kappa"], mixed_precision=True)
    e, g, H = B.energy_gradient_hessian(col, mesh, V, ipctk.PSDProjectionMethod.CLAMP)
    e_ref = oracle_mod.barrier_energy(ref, V, E, F, sc["dhat"], sc["kappa"])
    g_ref = oracle_mod.barrier_gradient(ref, V, E, F, sc["dhat"], sc["kappa"])
    rp, ci, va = oracle_mod.barrier_hessian(ref, V, E, F, sc["dhat"], sc["kappa"], psd="clamp")
    H_ref = sp.csr_matrix((va, ci, rp), shape=H.shape)
    err = (abs(e - e_ref) / abs(e_ref), np.linalg.norm(g - g_ref) / np.linalg.norm(g_ref),
           sp.linalg.norm(H - H_ref) / sp.linalg.norm(H_ref))
    print(f"\n{name}: mixed-precision relative error energy {err[0]:.2e} gradient {err[1]:.2e} hessian {err[2]:.2e}")
    assert max(err) <= TOL, err
    # and it is really a different evaluation (not silently the FP64 path)
    e64 = ipctk.BarrierPotential(sc["dhat"], sc["kappa"])(col, mesh, V)
    assert e != e64
