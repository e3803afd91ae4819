"""CCD tightness against analytic impact times.

Tight-Inclusion (the reference's narrow phase, tight_inclusion_ccd.cpp:33-75,
229-336) is not vendored, so its numeric times of impact cannot be
reproduced here.  What its method guarantees can be checked instead, on
linear motions whose first-contact time is known in closed form:

  * the strategy searches for contact at the effective separation
    ms = min((1 - 0.8) d0, 1e-4) (min_distance 0; d0 the initial distance)
    with the tolerance delta = min(0.5 d0, 1e-6);
  * for a point falling onto the inside of a face, or two crossing edges
    closing along the axis normal to both, the separation is exactly the
    gap along that axis, the same in the infinity norm Tight-Inclusion
    uses, so contact at separation ms happens at t_ms = (d0 - ms) / v;
  * the returned time of impact is conservative (toi <= t_ms) and tight to
    the tolerance: toi >= t_ms - 2 delta / v - 1e-6 t_ms (a box is accepted
    once its image is within the separation or narrower than delta).

The cases cover static and moving primitives, lateral motion, and every
axis and direction (axis permutations and reflections keep the infinity
norm).  The oracle is checked on the CPU; the CUDA path through the C ABI on
the GPU, where it must also equal the oracle bit for bit.  Each test records
the worst relative gap (t_ms - toi) / t_ms (the oracle's is 6.2e-4, inside
0.95 delta / v).
"""
import itertools

import numpy as np
import pytest

RESCALE = 0.8
TOL = 1e-6


def _frames():
    # the 48 axis permutations with sign flips (isometries of the infinity norm)
    out = []
    for perm in itertools.permutations(range(3)):
        for signs in itertools.product((1.0, -1.0), repeat=3):
            M = np.zeros((3, 3))
            for i, (p, sgn) in enumerate(zip(perm, signs)):
                M[i, p] = sgn
            out.append(M)
    return out


def _cases(seed=41, n=96):
    """(is_ee, x0 (4,3), x1 (4,3), t_ms, v, d0) with contact along the local z."""
    rng = np.random.Generator(np.random.PCG64(seed))
    frames = _frames()
    out = []
    for k in range(n):
        is_ee = k % 2 == 1
        d0 = float(np.exp(rng.uniform(np.log(1e-3), np.log(5e-2))))
        ms = min((1 - RESCALE) * d0, 1e-4)
        t_ms = float(rng.uniform(0.05, 0.95))
        v = (d0 - ms) / t_ms
        # share of the closing speed carried by the lower primitive
        share = float(rng.choice([0.0, 0.3, 1.0]))
        lat = rng.uniform(-0.05, 0.05, 2)
        if not is_ee:
            a = np.array([[rng.uniform(0.15, 0.3), rng.uniform(0.15, 0.3), d0],
                          [0, 0, 0], [1, 0, 0], [0, 1, 0]], float)
            dz = np.array([-(1 - share) * v, 0, 0, 0])
            dz[1:] = share * v
        else:
            a = np.array([[-1, 0.2, d0], [1, 0.2, d0], [0.3, -1, 0], [0.3, 1, 0]], float)
            dz = np.array([-(1 - share) * v, -(1 - share) * v, share * v, share * v])
        b = a.copy()
        b[:, 2] += dz
        b[:, :2] += lat  # a common lateral drift does not change the gap
        M = frames[k % len(frames)]
        off = rng.uniform(-1, 1, 3)
        out.append((is_ee, a @ M.T + off, b @ M.T + off, t_ms, v, d0))
    return out


def _check(tois, cases):
    worst = 0.0
    for toi, (is_ee, x0, x1, t_ms, v, d0) in zip(tois, cases):
        delta = min(0.5 * d0, TOL)
        assert toi <= t_ms, (toi, t_ms)
        assert toi >= t_ms - 2 * delta / v - 1e-6 * t_ms, (toi, t_ms, delta / v)
        worst = max(worst, (t_ms - toi) / t_ms)
    return worst


def test_ccd_tightness_oracle(oracle_mod, record_property):
    cases = _cases()
    tois = []
    for is_ee, x0, x1, t_ms, v, d0 in cases:
        fn = oracle_mod.edge_edge_ccd if is_ee else oracle_mod.point_triangle_ccd
        hit, toi = fn(x0, x1, tolerance=TOL, rescale=RESCALE)
        assert hit
        tois.append(toi)
    worst = _check(tois, cases)
    record_property("worst_relative_gap", worst)
    assert worst < 1e-2


@pytest.mark.gpu
def test_ccd_tightness_gpu(ipctk, oracle_mod, record_property):
    cases = _cases()
    worst = 0.0
    for is_ee in (False, True):
        sel = [c for c in cases if c[0] == is_ee]
        x0 = np.stack([c[1] for c in sel])
        x1 = np.stack([c[2] for c in sel])
        hit, toi = ipctk.TightInclusionCCD(TOL, 10_000_000, RESCALE)._batch(is_ee, x0, x1, 0.0, 1.0)
        assert np.all(hit)
        rhit, rtoi, _ = oracle_mod.ccd_stencils(is_ee, x0, x1, tolerance=TOL, rescale=RESCALE)
        np.testing.assert_array_equal(toi, rtoi)
        worst = max(worst, _check(toi, sel))
    record_property("worst_relative_gap", worst)
    assert worst < 1e-2
