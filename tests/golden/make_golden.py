"""Generate the golden fixtures of tests/golden/ from the CPU oracle.

Each fixture is self-contained: the scene's inputs (rest positions V, end
positions V1, edges E, faces F, dhat, stiffness) and the oracle's outputs on
them (the collision set, the barrier energy, gradient and CLAMP-projected
Hessian, the collision-free step size).  The scenes come from the seeded
generators of ipctk_gb300.scenes; storing the inputs keeps the fixtures
independent of the platform the generators run on.

    python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
for p in (os.path.join(ROOT, "ipc-toolkit_gb300"), os.path.join(ROOT, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)

# name -> (generator, keyword arguments): small enough that a fixture stays
# a few hundred KiB, large enough to hold every contact type
SCENES = {
    "two_sheet_8": ("two_sheet", {"side": 8, "seed": 3}),
    "spheres_8_sub2": ("sphere_pack", {"n_side": 2, "subdiv": 2, "seed": 3}),
}


def oracle_outputs(oracle, V, V1, E, F, dhat, kappa):
    col = oracle.build_collisions(V, E, F, dhat)
    rp, ci, va = oracle.barrier_hessian(col, V, E, F, dhat, kappa, psd="clamp")
    step, _ = oracle.collision_free_stepsize(V, V1, E, F)
    return {
        "vv": col.vv, "vv_w": col.vv_w, "ev": col.ev, "ev_w": col.ev_w, "ee": col.ee,
        "ee_dtype": col.ee_dtype, "ee_eps": col.ee_eps, "fv": col.fv,
        "energy": np.float64(oracle.barrier_energy(col, V, E, F, dhat, kappa)),
        "gradient": oracle.barrier_gradient(col, V, E, F, dhat, kappa),
        "hess_indptr": rp, "hess_indices": ci, "hess_data": va,
        "step": np.float64(step),
    }


def main():
    import oracle
    from ipctk_gb300 import scenes
    oracle.build()
    for name, (gen, kw) in SCENES.items():
        sc = getattr(scenes, gen)(**kw)
        V, V1 = np.ascontiguousarray(sc["V"], np.float64), np.ascontiguousarray(sc["V1"], np.float64)
        E, F = np.ascontiguousarray(sc["E"], np.int32), np.ascontiguousarray(sc["F"], np.int32)
        out = oracle_outputs(oracle, V, V1, E, F, sc["dhat"], sc["kappa"])
        path = os.path.join(HERE, name + ".npz")
        np.savez_compressed(path, V=V, V1=V1, E=E, F=F, dhat=np.float64(sc["dhat"]),
                            kappa=np.float64(sc["kappa"]), **out)
        counts = [len(out[k]) for k in ("vv", "ev", "ee", "fv")]
        print(f"{name}: {V.shape[0]} vertices, contacts vv/ev/ee/fv {counts}, "
              f"Hessian nnz {len(out['hess_data'])}, step {float(out['step'])}, "
              f"{os.path.getsize(path) / 1024:.0f} KiB")


if __name__ == "__main__":
    main()
