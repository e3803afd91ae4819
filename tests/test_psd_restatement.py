"""The PSD projection of a local Hessian as the device solver computes it
(contact.cuh: to_contrasts, sym_eig_impl, eigvecs_impl, psd_pairs, psd_apply),
restated in numpy and checked against numpy.linalg.eigh on local Hessians of
the oracle (contact_local, which follows normal_potential.cpp:127-232) and on
constructed cases.

The steps restated: M = C H C^T in contrast coordinates (the local Hessian is
translation invariant, so H = C^T M C); Householder tridiagonalisation; QL
sweeps in the carried-shift form of the tql / tqli recurrence, mirrored so
that the bulge is chased from the top of the unreduced block with the
Wilkinson shift taken at its bottom, with the deflation walks of the kernel;
eigenvectors of the kept pairs by replaying the recorded rotations and the
reflectors; and the smaller of the two eigenpair sets:
  H+ = H - sum f lam w w^T            over the negative eigenvalues, or
  H+ = (1 - f) H + sum f lam w w^T    over the non-negative ones
(f = 1 clamps, 2 takes absolute values), whichever set is smaller.
"""
import numpy as np
import pytest

EPS = 2.0 ** -52
R2, R6 = np.sqrt(0.5), 1.0 / np.sqrt(6.0)


def contrasts(ns):
    """Orthonormal rows orthogonal to (1, .., 1) for ns stencil vertices,
    times the 3x3 identity (row 3k + c)."""
    if ns == 4:
        C = 0.5 * np.array([[1, -1, 1, -1], [1, 1, -1, -1], [1, -1, -1, 1]], float)
    elif ns == 3:
        C = np.array([[R2, -R2, 0.0], [R6, R6, -2 * R6]])
    else:
        C = np.array([[R2, -R2]])
    return np.kron(C, np.eye(3))


def tridiagonalise(M):
    m = M.shape[0]
    A = M.copy()
    e = np.zeros(m)
    refl = []
    for k in range(m - 2):
        x = A[k + 1:, k].copy()
        sig = x[1:] @ x[1:]
        if sig == 0:
            e[k] = x[0]
            continue
        alpha = -np.sqrt(x[0] ** 2 + sig) if x[0] >= 0 else np.sqrt(x[0] ** 2 + sig)
        v = x.copy()
        v[0] -= alpha
        tau = 2 / (v @ v)
        S = A[k + 1:, k + 1:]
        p = tau * (S @ v)
        p -= 0.5 * tau * (p @ v) * v
        A[k + 1:, k + 1:] = S - np.outer(v, p) - np.outer(p, v)
        e[k] = alpha
        refl.append((k, v, tau))
    if m >= 2:
        e[m - 2] = A[m - 1, m - 2]
    return np.diag(A).copy(), e, refl


def ql(d, e):
    """Eigenvalues (in d) and the recorded rotations (k, c, s) of coordinates
    (k, k + 1)."""
    m = len(d)
    d, e = d.copy(), e.copy()
    floor = EPS * max(np.abs(d) + np.abs(e))

    def negligible(i):
        return abs(e[i]) <= EPS * (abs(d[i]) + abs(d[i + 1])) or abs(e[i]) <= floor

    rots = []
    end, it = m - 1, 0
    while end > 0:
        while end > 0 and (e[end - 1] == 0 or negligible(end - 1)):
            e[end - 1] = 0
            end -= 1
        if end <= 0:
            break
        it += 1
        assert it <= 40 * m
        start = end - 1
        while start > 0 and e[start - 1] != 0 and not negligible(start - 1):
            start -= 1
        if start > 0:
            e[start - 1] = 0
        td, b = 0.5 * (d[end - 1] - d[end]), e[end - 1]
        mu = d[end] - (abs(b) if td == 0 else b * b / (td + np.copysign(np.hypot(td, b), td)))
        g, s, c, p = d[start] - mu, 1.0, 1.0, 0.0
        whole = True
        for k in range(start, end):
            f, bb = s * e[k], c * e[k]
            r2 = f * f + g * g
            r = 0.0
            if r2 != 0:
                ir = 1 / np.sqrt(r2)
                r, s, c = r2 * ir, f * ir, g * ir
            if k > start:
                e[k - 1] = r
            if r2 == 0:
                d[k] -= p
                whole = False
                break
            g = d[k] - p
            q = (d[k + 1] - g) * s + 2 * c * bb
            p = s * q
            d[k] = g + p
            g = c * q - bb
            rots.append((k, c, -s))
        if whole:
            d[end] -= p
            e[end - 1] = g
    return d, rots


def eigenvectors(m, idx, rots, refl):
    Y = np.zeros((len(idx), m))
    for t, i in enumerate(idx):
        Y[t, i] = 1
    for k, c, s in reversed(rots):
        ya, yb = Y[:, k].copy(), Y[:, k + 1].copy()
        Y[:, k] = c * ya + s * yb
        Y[:, k + 1] = c * yb - s * ya
    for k, v, tau in reversed(refl):
        for t in range(len(idx)):
            Y[t, k + 1:] -= tau * (v @ Y[t, k + 1:]) * v
    return Y


def project(H, ns, f):
    """(H+, number of pairs used)."""
    C = contrasts(ns)
    M = C @ H @ C.T
    M = 0.5 * (M + M.T)
    m = M.shape[0]
    d, e, refl = tridiagonalise(M)
    lam, rots = ql(d, e)
    neg = lam < 0
    flip = 2 * neg.sum() > m
    idx = [k for k in range(m) if neg[k] != flip] if neg.any() else []
    sigma = 1 - f if flip else 1.0
    W = eigenvectors(m, idx, rots, refl) @ C  # rows w = C^T q
    sl = (-f if flip else f) * lam[idx]
    return sigma * H - (W.T * sl) @ W, len(idx)


def reference(H, f):
    w, V = np.linalg.eigh(0.5 * (H + H.T))
    w = np.maximum(w, 0) if f == 1 else np.abs(w)
    return (V * w) @ V.T


def _oracle_hessians(oracle_mod, n_each=60, seed=0):
    rng = np.random.default_rng(seed)
    out = []
    for ctype, ns in ((0, 2), (1, 3), (2, 4), (3, 4)):
        for _ in range(n_each):
            x = rng.normal(size=(ns, 3))
            if ctype == 2:
                # nearly parallel edges inside dhat: the mollified case
                x[2:] = x[:2] + 0.05 * rng.normal(size=(2, 3)) + [0, 0, 0.02]
            else:
                x[1:] = x[0] + 0.3 * rng.normal(size=(ns - 1, 3))
            x[0] += [0.0, 0.0, 0.01]
            eps = 1e-3 if ctype == 2 else 0.0
            _, _, H = oracle_mod.contact_local(ctype, x, 0.5, 1.0, eps=eps)
            if np.all(np.isfinite(H)) and np.abs(H).max() > 0:
                out.append((H, ns))
    return out


@pytest.mark.parametrize("f", [1, 2])
def test_restatement_equals_eigh_projection(oracle_mod, f):
    cases = _oracle_hessians(oracle_mod)
    assert len(cases) > 150
    worst = 0.0
    pairs = []
    for H, ns in cases:
        got, np_ = project(H, ns, f)
        ref = reference(H, f)
        worst = max(worst, np.linalg.norm(got - ref) / np.linalg.norm(ref))
        pairs.append((np_, 3 * (ns - 1)))
    assert worst <= 1e-12, worst
    # the kept set is never more than half of the contrast space
    assert all(k <= m // 2 for k, m in pairs)
    # both sets are exercised: more negative than non-negative eigenvalues
    # (the non-negative set kept) and fewer (the negative set kept)
    kinds = set()
    for H, ns in cases:
        C = contrasts(ns)
        nneg = int((np.linalg.eigvalsh(C @ H @ C.T) < 0).sum())
        kinds.add("non-negative" if 2 * nneg > 3 * (ns - 1) else ("negative" if nneg else "none"))
    assert {"non-negative", "negative"} <= kinds


def test_translation_invariant_by_construction():
    # H = C^T M C for any symmetric M: the identity the smaller set rests on
    rng = np.random.default_rng(1)
    for ns in (2, 3, 4):
        C = contrasts(ns)
        np.testing.assert_allclose(C @ C.T, np.eye(3 * (ns - 1)), atol=1e-15)
        np.testing.assert_allclose(C @ np.kron(np.ones(ns), np.eye(3)).T, 0, atol=1e-15)
        A = rng.normal(size=(3 * (ns - 1),) * 2)
        H = C.T @ (A + A.T) @ C
        np.testing.assert_allclose(C.T @ (C @ H @ C.T) @ C, H, atol=1e-13)


def test_constructed_cases():
    rng = np.random.default_rng(2)
    for ns in (2, 3, 4):
        C = contrasts(ns)
        m = 3 * (ns - 1)
        Q, _ = np.linalg.qr(rng.normal(size=(m, m)))
        # already PSD: returned bit for bit (no pairs, sigma 1)
        H = C.T @ (Q * rng.uniform(0.1, 2, m)) @ Q.T @ C
        got, k = project(H, ns, 1)
        assert k == 0 and np.array_equal(got, H)
        # negative definite in the contrast space: clamped to zero
        H = C.T @ (Q * -rng.uniform(0.1, 2, m)) @ Q.T @ C
        got, k = project(H, ns, 1)
        assert k == 0 and np.abs(got).max() <= 1e-14 * np.abs(H).max()
        got, _ = project(H, ns, 2)
        np.testing.assert_allclose(got, -H, atol=1e-13 * np.abs(H).max())
        # a repeated negative eigenvalue (the point-point case's shape)
        w = np.full(m, -1.0)
        w[0] = 3.0
        H = C.T @ (Q * w) @ Q.T @ C
        got, k = project(H, ns, 1)
        assert k <= m // 2
        np.testing.assert_allclose(got, reference(H, 1), atol=1e-13)
