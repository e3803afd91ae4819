"""The lower bound on a query's time of impact that lets the step-size pass
skip queries (ccd_bound.cu, toi_lower_bound), restated in numpy and checked against
the oracle's Tight-Inclusion times of impact (oracle ccd_stencils, which
follows tight_inclusion_ccd.cpp:33-336) on the candidates of the two-sheet
scene and of batch scenes: the bound must never exceed a query's time of
impact, so a query whose bound is at or after the earliest time found so far
cannot change the step.  Also checks that the bound prunes: most queries of
a colliding scene (over 95 % here) have bounds after the scene's earliest
impact.  The restatement sizes the separation from the exact distance at
t = 0; the kernel uses an upper bound of it (the distance between two points
on the primitives), which only lowers the bound.
"""
import numpy as np
import pytest

INF = np.inf


def _num_err(s, e, vf):
    filt = 7.549516567451064e-15 if vf else 7.105427357601002e-15  # with a minimum separation
    m = np.maximum(np.abs(s).max(axis=1), np.abs(e).max(axis=1))
    return filt * np.minimum(m, 1.0) ** 3


def _first_time(A, B, R, scale):
    """First t in [0, 1] with min_k(A_k + B_k t) <= R and max_k(...) >= -R,
    searched in FP32 with a slack of 2^-20 (scale + R)."""
    A = A.astype(np.float32)
    B = B.astype(np.float32)
    R = R.astype(np.float32)
    n = A.shape[1]
    slack = (scale.astype(np.float32) + R) * np.float32(2.0 ** -20)
    starts = [np.zeros(n, np.float32)]
    with np.errstate(divide="ignore", invalid="ignore"):
        for k in range(4):
            starts.append(np.where(B[k] < 0, (R - A[k]) / B[k], np.nan).astype(np.float32))
            starts.append(np.where(B[k] > 0, (-R - A[k]) / B[k], np.nan).astype(np.float32))
    T = np.full(n, INF)
    for t in starts:
        ok = (t >= 0) & (t <= 1)
        tc = np.clip(np.nan_to_num(t, nan=0.0), 0.0, 1.0).astype(np.float32)
        f = A + B * tc
        T = np.where(ok & (f.min(axis=0) <= R + slack) & (f.max(axis=0) >= -R - slack), np.minimum(T, tc), T)
    return T


def _lines(x0, d, vf, c):
    """F_c = A00 + u Au + v Av + t (B00 + u Bu + v Bv)."""
    s_, e_ = x0[:, :, c], d[:, :, c]
    if vf:
        return (s_[:, 0] - s_[:, 1], -(s_[:, 2] - s_[:, 1]), -(s_[:, 3] - s_[:, 1]),
                e_[:, 0] - e_[:, 1], -(e_[:, 2] - e_[:, 1]), -(e_[:, 3] - e_[:, 1]))
    return (s_[:, 0] - s_[:, 2], s_[:, 1] - s_[:, 0], -(s_[:, 3] - s_[:, 2]),
            e_[:, 0] - e_[:, 2], e_[:, 1] - e_[:, 0], -(e_[:, 3] - e_[:, 2]))


def _min_norm(a, b):
    bb = (b * b).sum(0)
    with np.errstate(invalid="ignore", divide="ignore"):
        t = np.where(bb > 0, np.clip(-(a * b).sum(0) / np.where(bb > 0, bb, 1.0), 0, 1), 0.0)
    return np.sqrt(((a + t * b) ** 2).sum(0))


def _first_time_grid(A00, Au, Av, B00, Bu, Bv, R, uq, vq, w):
    """_first_time over the corners of the cell [uq, uq + w] x [vq, vq + w],
    the corner lines formed in FP32 from the FP64 coefficients."""
    f32 = np.float32
    A = np.array([f32(A00) + f32(uq + w * (k & 1)) * Au.astype(f32) + f32(vq + w * ((k >> 1) & 1)) * Av.astype(f32)
                  for k in range(4)], dtype=f32)
    B = np.array([f32(B00) + f32(uq + w * (k & 1)) * Bu.astype(f32) + f32(vq + w * ((k >> 1) & 1)) * Bv.astype(f32)
                  for k in range(4)], dtype=f32)
    return A, B


def toi_lower_bound(x0, x1, d0, vf, min_distance=0.0, tolerance=1e-6, rescale=0.8):
    ms = np.minimum((1 - rescale) * (d0 - min_distance), 1e-4) + min_distance
    delta = np.minimum(0.5 * d0, tolerance)
    err = _num_err(x0, x1, vf)
    d = x1 - x0
    n = x0.shape[0]
    coef = [_lines(x0, d, vf, c) for c in range(3)]
    T = np.zeros(n)
    bmax = np.zeros(n)
    Rs, scales = [], []
    for c in range(3):
        A00, Au, Av, B00, Bu, Bv = coef[c]
        A = np.array([A00 + (k & 1) * Au + ((k >> 1) & 1) * Av for k in range(4)])
        B = np.array([B00 + (k & 1) * Bu + ((k >> 1) & 1) * Bv for k in range(4)])
        bmax = np.maximum(bmax, np.abs(B).max(axis=0))
        R = 3 * err[:, c] + ms + delta
        Rs.append(R)
        scales.append(np.abs(A00) + np.abs(Au) + np.abs(Av) + np.abs(B00) + np.abs(Bu) + np.abs(Bv))
        T = np.maximum(T, _first_time(A, B, R, scales[c]))
    # 4 x 4 cells of the (u, v) square, for primitives whose edges stay long
    # next to the separation
    ncell = 4
    rmax = np.max(Rs, axis=0)
    au = np.array([coef[c][1] for c in range(3)]); bu = np.array([coef[c][4] for c in range(3)])
    av = np.array([coef[c][2] for c in range(3)]); bv = np.array([coef[c][5] for c in range(3)])
    need = np.sqrt(3.0) * (2 * rmax + delta) * (0.5 * ncell) * (1 + 1e-6)
    longp = (_min_norm(au, bu) > need) & (_min_norm(av, bv) > need)
    w = 1.0 / ncell
    Tq = np.full(n, INF)
    for iu in range(ncell):
        for iv in range(ncell):
            t = np.zeros(n)
            for c in range(3):
                A, B = _first_time_grid(*coef[c], Rs[c], iu * w, iv * w, w)
                t = np.maximum(t, _first_time(A, B, Rs[c], scales[c]))
            Tq = np.minimum(Tq, t)
    T = np.where(longp, np.maximum(T, Tq), T)
    with np.errstate(invalid="ignore", divide="ignore"):
        tol0 = np.where(bmax == 0, delta, delta / (3 * np.where(bmax == 0, 1.0, bmax)))
        out = np.maximum(0.0, (T - 2.0 ** -20 - tol0 * (1 + 1e-6) - 2.0 ** -60) * (1 - 1e-6))
    out = np.where(np.isinf(T), INF, out)
    # queries that do not move miss unless within the minimum distance
    out = np.where(np.all(x0 == x1, axis=(1, 2)), INF, out)
    return np.where(d0 <= min_distance, 0.0, out)


def _d0(oracle_mod, x0, vf):
    f = oracle_mod.point_triangle_distance if vf else oracle_mod.edge_edge_distance
    return np.sqrt(np.array([f(a[0], a[1], a[2], a[3]) for a in x0]))


@pytest.mark.parametrize("scene", ["two_sheet", "batch0", "batch8"])
def test_bound_never_exceeds_time_of_impact(oracle_mod, scene):
    from ipctk_gb300 import scenes
    if scene == "two_sheet":
        sc = scenes.two_sheet()
    else:
        sc = scenes.batch()[int(scene[5:])]
    V0, V1, E, F = sc["V"], sc["V1"], sc["E"], sc["F"]
    ee, fv = oracle_mod.ccd_candidates(V0, V1, E, F)
    (xe0, xe1), (xf0, xf1) = oracle_mod.ccd_stencil_positions(V0, V1, E, F, ee, fv)
    rng = np.random.default_rng(0)
    earliest, pruned, total = INF, 0, 0
    bounds = []
    for vf, x0, x1 in ((False, xe0, xe1), (True, xf0, xf1)):
        # a seeded sample keeps the oracle's root finding to seconds
        pick = rng.choice(x0.shape[0], size=min(x0.shape[0], 6000), replace=False)
        x0, x1 = x0[pick], x1[pick]
        hit, toi, _ = oracle_mod.ccd_stencils(0 if vf else 1, x0, x1)
        lb = toi_lower_bound(x0, x1, _d0(oracle_mod, x0, vf), vf)
        assert np.all(lb[hit] <= toi[hit]), (vf, np.max(lb[hit] - toi[hit]))
        earliest = min(earliest, toi[hit].min() if hit.any() else INF)
        bounds.append(lb)
    lb = np.concatenate(bounds)
    # the scenes collide: most queries are skipped once the earliest impact is known
    assert earliest < 1.0
    assert np.mean(lb >= earliest) > 0.95
