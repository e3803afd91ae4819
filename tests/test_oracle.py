"""The CPU oracle pinned against the reference's own known-answer tests.

Each test restates an analytic test of the reference (cited by file:line of
tests/src/tests/ in ipc-toolkit) or checks a derivative by central finite
differences, the way the reference's FD tests do.  The reference itself
cannot be built in this container (its CMake dependencies are absent), so
these restated known-answer tests are what pins the oracle to the reference.
The fixtures in tests/golden/ (inputs stored with the oracle's outputs) then
hold the oracle (test_golden.py) and the CUDA path (test_gpu_golden.py) to
those results.
"""
import numpy as np
import pytest

EPS32 = float(np.finfo(np.float32).eps)


def approx(a, b, margin=0.0, eps=100 * EPS32):
    """Catch::Approx semantics: |a-b| <= margin or relative eps."""
    return abs(a - b) <= margin or abs(a - b) <= eps * (max(abs(a), abs(b)))


# --- distances ---------------------------------------------------------------

def test_point_triangle_distance_grid(oracle_mod):
    """distance/test_point_triangle.cpp:31-112"""
    from test_gpu_parity import _pt_grid
    x, cps = _pt_grid()
    for i in range(len(x)):
        d = oracle_mod.point_triangle_distance(*x[i])
        assert approx(d, float(((x[i, 0] - cps[i]) ** 2).sum()), margin=1e-12)


def test_edge_edge_distance_grid(oracle_mod):
    """distance/test_edge_edge.cpp:31-66"""
    n = 0
    for e0y in (-10, -1, -1e-4, 0, 1e-4, 1, 10):
        for shiftx in (-2, 0, 2):
            for shiftz in (-2, 0, 2):
                for ox in (-1, -0.5, 0, 0.5, 1):
                    for oz in (-1, -0.5, 0, 0.5, 1):
                        e0x, e0z = shiftx + ox, shiftz + oz
                        e00 = np.array([-1 + e0x, e0y, e0z])
                        e01 = np.array([1 + e0x, e0y, e0z])
                        e10 = np.array([0.0, 0, -1])
                        e11 = np.array([0.0, 0, 1])
                        c0 = e00 if shiftx > 1 else (e01 if shiftx < -1 else np.array([0, e0y, e0z]))
                        c1 = e11 if shiftz > 1 else (e10 if shiftz < -1 else np.array([0, 0, e0z]))
                        d = oracle_mod.edge_edge_distance(e00, e01, e10, e11)
                        assert approx(d, float(((c0 - c1) ** 2).sum()), margin=1e-12)
                        n += 1
    assert n == 7 * 9 * 25


def test_edge_edge_distance_not_line_line(oracle_mod):
    """distance/test_edge_edge.cpp:68-128 (closest points at an endpoint)"""
    rng = np.random.Generator(np.random.PCG64(11))
    sign = lambda x: -1 if x < 0 else 1
    for alpha0 in np.arange(-1.0, 2.0, 0.1):
        for s0 in np.arange(-10.0, 10.0, 1.0):
            if s0 == 0:
                continue
            for swap_ea in (False, True):
                for swap_eb in (False, True):
                    for swap_edges in (False, True):
                        for _ in range(3):
                            alpha, s = alpha0, s0
                            ea0, ea1 = rng.uniform(-1, 1, 3), rng.uniform(-1, 1, 3)
                            n = np.cross(ea1 - ea0, [1, 0, 0])
                            n /= np.linalg.norm(n)
                            eb0 = ((ea1 - ea0) * alpha + ea0) + s * n
                            if alpha < 0:
                                alpha = 0
                                n = eb0 - ea0
                                s = np.linalg.norm(n)
                                n /= s
                            elif alpha > 1:
                                alpha = 1
                                n = eb0 - ea1
                                s = np.linalg.norm(n)
                                n /= s
                            eb1 = ((ea1 - ea0) * alpha + ea0) + (s + sign(s) * 1) * n
                            a0, a1, b0, b1 = ea0, ea1, eb0, eb1
                            if swap_ea:
                                a0, a1 = a1, a0
                            if swap_eb:
                                b0, b1 = b1, b0
                            if swap_edges:
                                a0, b0 = b0, a0
                                a1, b1 = b1, a1
                            d = oracle_mod.edge_edge_distance(a0, a1, b0, b1)
                            assert approx(d, s * s, margin=1e-15)


def test_edge_edge_distance_line_line(oracle_mod):
    """distance/test_edge_edge.cpp:130-180 (interior closest points)"""
    rng = np.random.Generator(np.random.PCG64(12))
    for _ in range(500):
        alpha, beta = rng.uniform(0.01, 0.99, 2)
        s = rng.uniform(-5, 5)
        ea1, eb1 = rng.uniform(-1, 1, 3), rng.uniform(-1, 1, 3)
        u = rng.normal(size=3)
        v = rng.normal(size=3)
        n = np.cross(u, v)
        n /= np.linalg.norm(n)
        pa = rng.uniform(-1, 1, 3)
        pb = pa + s * n
        ea0 = pa - alpha * u
        ea1 = ea0 + u
        eb0 = pb - beta * v
        eb1 = eb0 + v
        d = oracle_mod.edge_edge_distance(ea0, ea1, eb0, eb1)
        assert oracle_mod.edge_edge_distance_type(ea0, ea1, eb0, eb1) == 8
        assert abs(d - s * s) <= 1e-12 * max(1, s * s)


def test_point_edge_distance(oracle_mod):
    """distance/test_point_edge.cpp: closest to e0 / e1 / interior"""
    e0, e1 = np.array([-1.0, 0, 0]), np.array([1.0, 0, 0])
    for px in np.linspace(-3, 3, 25):
        for py in (-2, -1e-8, 0, 1e-8, 2):
            p = np.array([px, py, 0.5])
            cx = min(max(px, -1), 1)
            exp = (px - cx) ** 2 + py ** 2 + 0.25
            assert approx(oracle_mod.point_edge_distance(p, e0, e1), exp, margin=1e-12)
            t = oracle_mod.point_edge_distance_type(p, e0, e1)
            assert t == (0 if px < -1 else (1 if px > 1 else 2))


def test_edge_edge_parallel_types(oracle_mod):
    """distance/test_distance_type.cpp: parallel edges classify by overlap"""
    a0, a1 = np.array([0.0, 0, 0]), np.array([1.0, 0, 0])
    # b entirely beyond a1 -> EA1_EB0
    assert oracle_mod.edge_edge_distance_type(a0, a1, np.array([2.0, 1, 0]), np.array([3.0, 1, 0])) == 2
    # b before a0 -> EA0_EB1
    assert oracle_mod.edge_edge_distance_type(a0, a1, np.array([-3.0, 1, 0]), np.array([-2.0, 1, 0])) == 1
    # overlapping -> an edge-point type, never line-line
    t = oracle_mod.edge_edge_distance_type(a0, a1, np.array([0.5, 1, 0]), np.array([1.5, 1, 0]))
    assert t in (4, 5, 6, 7)
    d = oracle_mod.edge_edge_distance(a0, a1, np.array([0.5, 1, 0]), np.array([1.5, 1, 0]))
    assert approx(d, 1.0, margin=1e-15)


def test_degenerate_edges(oracle_mod):
    """distance_type.cpp:19-24 and :97-103: zero-length edges"""
    p = np.array([0.0, 1, 0])
    z = np.zeros(3)
    assert oracle_mod.point_edge_distance_type(p, z, z) == 0
    assert oracle_mod.edge_edge_distance_type(z, z, p, p) == 0
    assert oracle_mod.edge_edge_distance_type(z, z, p, 2 * p) == 6
    assert oracle_mod.edge_edge_distance_type(p, 2 * p, z, z) == 4


# --- barrier -----------------------------------------------------------------

@pytest.mark.parametrize("use_sq", [False, True])
def test_barrier_derivatives_fd(oracle_mod, use_sq):
    """barrier/test_barrier.cpp:398-461 (ClampedLogBarrier)"""
    for k in range(-2 if use_sq else -5, 0):
        dhat = 10.0 ** k
        for d in np.linspace(0.5 * dhat, 0.9 * dhat, 10, endpoint=False):
            if use_sq:
                d, dh = d * d, dhat * dhat
            else:
                dh = dhat
            h = 1e-10 * max(1.0, d) if not use_sq else d * 1e-6
            fd1 = (oracle_mod.barrier(d + h, dh) - oracle_mod.barrier(d - h, dh)) / (2 * h)
            fd2 = (oracle_mod.barrier(d + h, dh, 1) - oracle_mod.barrier(d - h, dh, 1)) / (2 * h)
            assert abs(oracle_mod.barrier(d, dh, 1) - fd1) <= 1e-4 * max(abs(fd1), 1e-30) + 1e-9 * dh
            assert abs(oracle_mod.barrier(d, dh, 2) - fd2) <= 1e-4 * max(abs(fd2), 1e-30) + 1e-9


@pytest.mark.parametrize("kind", [1, 2, 3, 4])
@pytest.mark.parametrize("use_sq", [False, True])
def test_barrier_kinds_derivatives_fd(oracle_mod, kind, use_sq):
    """barrier/test_barrier.cpp:398-461 for the Normalized, ClampedLogSq, Cubic
    and TwoStage barriers: first and second derivatives against central
    differences over the same dhat and d grid."""
    for k in range(-2 if use_sq else -5, 0):
        dhat = 10.0 ** k
        for d in np.linspace(0.5 * dhat, 0.9 * dhat, 10, endpoint=False):
            if use_sq:
                d, dh = d * d, dhat * dhat
            else:
                dh = dhat
            h = d * 1e-6
            b = lambda x, n=0: oracle_mod.barrier(x, dh, n, kind)
            fd1 = (b(d + h) - b(d - h)) / (2 * h)
            fd2 = (b(d + h, 1) - b(d - h, 1)) / (2 * h)
            assert abs(b(d, 1) - fd1) <= 1e-5 * max(abs(fd1), abs(b(d, 1)))
            assert abs(b(d, 2) - fd2) <= 1e-5 * max(abs(fd2), abs(b(d, 2)))


def test_barrier_kind_values(oracle_mod):
    """Closed forms at hand-checked points (barrier.cpp:47-154)."""
    dh = 2.0
    # normalized = clamped log of d / dhat against 1, derivatives / dhat^k
    for k in range(3):
        assert oracle_mod.barrier(0.6, dh, k, 1) == oracle_mod.barrier(0.3, 1.0, k) / dh ** k
    # cubic: -2/(3 dhat) (d - dhat)^3, 4 (1 - d / dhat) and 0 at/after dhat
    assert oracle_mod.barrier(1.0, dh, 0, 3) == pytest.approx(-2.0 / 3.0 / 2.0 * (-1.0) ** 3, rel=1e-15)
    assert oracle_mod.barrier(1.0, dh, 2, 3) == 2.0
    assert oracle_mod.barrier(2.0, dh, 0, 3) == 0.0
    # two-stage: quadratic on [dhat/2, dhat), log below, continuous at dhat/2
    assert oracle_mod.barrier(1.5, dh, 0, 4) == 0.5 * 0.5 * 0.5
    assert oracle_mod.barrier(1.5, dh, 2, 4) == 1.0
    lo = oracle_mod.barrier(1.0 - 1e-12, dh, 0, 4)
    assert lo == pytest.approx(oracle_mod.barrier(1.0, dh, 0, 4), rel=1e-9)
    # clamped log squared: (d - dhat)^2 ln^2(d / dhat); infinite at d <= 0
    assert oracle_mod.barrier(0.5, dh, 0, 2) == pytest.approx(1.5 ** 2 * np.log(0.25) ** 2, rel=1e-15)
    assert oracle_mod.barrier(0.0, dh, 0, 2) == float("inf")


def _vv_collisions(oracle_mod, rng, n):
    """A VV-only collision set of n random close pairs (weights 1)."""
    V = rng.uniform(0, 1, (2 * n, 3))
    V[1::2] = V[0::2] + rng.uniform(-1e-2, 1e-2, (n, 3))
    vv = np.arange(2 * n, dtype=np.int32).reshape(n, 2)
    z2, z1 = np.zeros((0, 2), np.int32), np.zeros(0)
    col = oracle_mod.Collisions.from_arrays(vv, np.ones(n), z2, z1, z2, z1, np.zeros(0, np.int8), z1, z2, z1)
    return V, col


def test_gauss_newton_equals_hessian_on_vertex_pairs(oracle_mod):
    """For vertex-vertex contacts d^2 = |t|^2 is quadratic in the positions,
    so the Gauss-Newton Hessian is the Hessian: its diagonal and quadratic
    form match the assembled Hessian's."""
    import scipy.sparse as sps
    rng = np.random.Generator(np.random.PCG64(41))
    V, col = _vv_collisions(oracle_mod, rng, 50)
    E, F = np.zeros((0, 2), np.int32), np.zeros((0, 3), np.int32)
    dhat, kappa = 2e-2, 3.0
    for kind in range(5):
        bits = kind << 4
        rp, ci, va = oracle_mod.barrier_hessian(col, V, E, F, dhat, kappa, physical=bits)
        H = sps.csr_matrix((va, ci, rp), shape=(V.size, V.size))
        d = oracle_mod.barrier_gauss_newton_diagonal(col, V, E, F, dhat, kappa, physical=bits)
        assert np.linalg.norm(d - H.diagonal()) <= 1e-12 * np.linalg.norm(d)
        p = rng.standard_normal(V.size)
        q = oracle_mod.barrier_gauss_newton_quadratic_form(col, V, E, F, p, dhat, kappa, physical=bits)
        assert q == pytest.approx(p @ (H @ p), rel=1e-10)


def test_gauss_newton_quadratic_form_axes(oracle_mod):
    """p = e_i gives diagonal entry i, for every contact type."""
    from ipctk_gb300 import scenes
    sc = scenes.two_sheet(side=12, seed=2)
    V, E, F = sc["V"], sc["E"], sc["F"]
    col = oracle_mod.build_collisions(V, E, F, sc["dhat"])
    d = oracle_mod.barrier_gauss_newton_diagonal(col, V, E, F, sc["dhat"], sc["kappa"])
    for i in np.argsort(-np.abs(d))[:12]:
        e = np.zeros(V.size)
        e[i] = 1.0
        q = oracle_mod.barrier_gauss_newton_quadratic_form(col, V, E, F, e, sc["dhat"], sc["kappa"])
        assert q == pytest.approx(d[i], rel=1e-12)


def test_barrier_values(oracle_mod):
    """barrier.cpp:11-43: b(d)=-(d-dh)^2 ln(d/dh) on (0,dh), 0 beyond, inf at 0"""
    assert oracle_mod.barrier(0.0, 1.0) == float("inf")
    assert oracle_mod.barrier(1.0, 1.0) == 0.0
    assert oracle_mod.barrier(2.0, 1.0) == 0.0
    assert oracle_mod.barrier(2.0, 1.0, 1) == 0.0
    d, dh = 0.3, 1.0
    assert oracle_mod.barrier(d, dh) == pytest.approx(-(d - dh) ** 2 * np.log(d / dh), rel=1e-15)


# --- distance derivatives (finite differences) --------------------------------

def _fd(f, x, h=1e-7):
    g = np.zeros_like(x)
    for i in range(x.size):
        e = np.zeros_like(x)
        e[i] = h
        g[i] = (f(x + e) - f(x - e)) / (2 * h)
    return g


@pytest.mark.parametrize("kind,dtype", [(0, 8), (1, 8), (2, 8), (3, 8), (3, 0), (3, 4), (3, 6)])
def test_distance_derivatives_fd(oracle_mod, kind, dtype):
    rng = np.random.Generator(np.random.PCG64(100 + kind * 10 + dtype))
    n = {0: 2, 1: 3, 2: 4, 3: 4}[kind]
    for _ in range(20):
        x = rng.uniform(-1, 1, 3 * n)
        d, g, H = oracle_mod.distance_derivatives(kind, x, dtype)
        fg = _fd(lambda y: oracle_mod.distance_derivatives(kind, y, dtype)[0], x)
        assert np.linalg.norm(g - fg) <= 1e-6 * max(1.0, np.linalg.norm(fg))
        fH = np.stack([_fd(lambda y: oracle_mod.distance_derivatives(kind, y, dtype)[1][i], x)
                       for i in range(3 * n)])
        assert np.linalg.norm(H - fH) <= 1e-5 * max(1.0, np.linalg.norm(fH))
        assert np.allclose(H, H.T, atol=1e-12 * max(1, np.abs(H).max()))


@pytest.mark.parametrize("ctype", [0, 1, 2, 3])
def test_contact_local_derivatives_fd(oracle_mod, ctype):
    """potential/test_barrier_potential.cpp:119-246 style FD checks of the
    per-contact energy / gradient / Hessian, including mollified EE."""
    rng = np.random.Generator(np.random.PCG64(200 + ctype))
    n = {0: 2, 1: 3, 2: 4, 3: 4}[ctype]
    dhat, kappa = 1e-1, 1.0
    checked = 0
    for _ in range(200):
        x = rng.uniform(-0.1, 0.1, (n, 3))
        if ctype == 2:
            # nearly parallel edges close together -> mollified
            x[1] = x[0] + np.array([0.2, 0.0, 0.0])
            x[2] = x[0] + np.array([0.05, 0.03, 0.01]) + rng.uniform(-0.005, 0.005, 3)
            x[3] = x[2] + np.array([0.2, 0.001, 0.0]) + rng.uniform(-0.002, 0.002, 3)
            eps = 1e-3 * 0.04 * 0.04
            dtype = oracle_mod.edge_edge_distance_type(*x)
        else:
            eps, dtype = 0.0, 8
        x = x.ravel()
        e, g, H = oracle_mod.contact_local(ctype, x, dhat, kappa, eps=eps, dtype=dtype)
        if e == 0 or not np.isfinite(e):
            continue
        fe = lambda y: oracle_mod.contact_local(ctype, y, dhat, kappa, eps=eps, dtype=dtype)[0]
        fg = _fd(fe, x, 1e-8)
        assert np.linalg.norm(g - fg) <= 1e-4 * np.linalg.norm(fg) + 1e-12
        fH = np.stack([_fd(lambda y: oracle_mod.contact_local(ctype, y, dhat, kappa, eps=eps, dtype=dtype)[1][i],
                           x, 1e-8) for i in range(x.size)])
        assert np.linalg.norm(H - fH) <= 1e-3 * np.linalg.norm(fH) + 1e-9
        checked += 1
        if checked >= 5:
            break
    assert checked > 0


@pytest.mark.parametrize("psd", ["clamp", "abs"])
def test_psd_projection(oracle_mod, psd):
    """eigen_ext.tpp:64-108: projected Hessian is PSD; clamp keeps the
    non-negative spectrum, abs flips the negative part."""
    rng = np.random.Generator(np.random.PCG64(7))
    for ctype in (0, 1, 3):
        n = {0: 2, 1: 3, 3: 4}[ctype]
        for _ in range(5):
            x = rng.uniform(-0.02, 0.02, 3 * n)
            _, _, H0 = oracle_mod.contact_local(ctype, x, 0.1, 1.0, psd="none")
            _, _, H = oracle_mod.contact_local(ctype, x, 0.1, 1.0, psd=psd)
            lam0 = np.linalg.eigvalsh(H0)
            lam = np.linalg.eigvalsh(H)
            scale = np.abs(lam0).max()
            assert lam.min() >= -1e-12 * scale
            exp = np.sort(np.maximum(lam0, 0) if psd == "clamp" else np.abs(lam0))
            assert np.allclose(np.sort(lam), exp, atol=1e-11 * scale)


# --- CCD ---------------------------------------------------------------------

def test_point_triangle_ccd_cases(oracle_mod):
    """ccd/test_point_triangle_ccd.cpp:25-123"""
    from test_gpu_parity import _pt_ccd_cases
    for a, b, exp, conservative in _pt_ccd_cases():
        hit, toi = oracle_mod.point_triangle_ccd(a, b)
        if conservative:
            assert hit or not exp
        else:
            assert hit == exp
        if hit:
            assert 0 <= toi <= 1


def _ee_ccd_general():
    """ccd/test_edge_edge_ccd.cpp:29-56"""
    out = []
    for uy in (-1.0, 0.0, 1 - EPS32, 1.0, 1 + EPS32, 2.0):
        for e1x in (-1 - EPS32, -1, -1 + EPS32, -0.5, 0, 0.5, 1 - EPS32, 1, 1 + EPS32):
            x0 = np.array([[-1, -1, 0], [1, -1, 0], [e1x, 1, -1], [e1x, 1, 1]], float)
            for moving in (True, False):
                if moving:
                    u0, u1 = np.array([0, uy, 0]), np.array([0, -uy, 0])
                    exp = uy >= 1.0 and -1 <= e1x <= 1
                else:
                    u0, u1 = np.array([0, 2 * uy, 0]), np.zeros(3)
                    exp = uy >= 2.0 and -1 <= e1x <= 1
                x1 = x0 + np.stack([u0, u0, u1, u1])
                out.append((x0, x1, exp))
    return out


def test_edge_edge_ccd_cases(oracle_mod):
    for a, b, exp in _ee_ccd_general():
        hit, toi = oracle_mod.edge_edge_ccd(a, b)
        assert hit or not exp


def test_edge_edge_ccd_adversarial(oracle_mod):
    """ccd/test_edge_edge_ccd.cpp 'Adversarial ACCD Case'"""
    for d0 in (1e-2, 1e-4, 1e-6, 1e-8):
        x0 = np.array([[-1.0, -d0 / 2, 0], [1.0, -d0 / 2, 0], [0, d0 / 2, -1.0], [0, d0 / 2, 1.0]])
        s = 1e-3
        x1 = x0 + np.array([[-s, d0, -s], [s, d0, s], [s, -d0, s], [-s, -d0, -s]])
        hit, toi = oracle_mod.edge_edge_ccd(x0, x1)
        assert hit


def test_ccd_conservative_on_linear_impacts(oracle_mod):
    """A point falling onto a static triangle at a known time: the returned
    ToI never exceeds the analytic impact time and is within the TI
    tolerance of it (rescaled by 0.8 only for tiny ToIs)."""
    rng = np.random.Generator(np.random.PCG64(21))
    for _ in range(40):
        t_hit = rng.uniform(0.05, 0.95)
        z0 = rng.uniform(0.01, 0.1)
        p0 = np.array([rng.uniform(0.1, 0.3), rng.uniform(0.1, 0.3), z0])
        tri = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], float)
        p1 = p0 - np.array([0, 0, z0 / t_hit])
        hit, toi = oracle_mod.point_triangle_ccd(np.vstack([p0, tri]), np.vstack([p1, tri]))
        assert hit
        assert toi <= t_hit
        # effective minimum separation min(0.2*d0, 1e-4) plus tolerance
        speed = z0 / t_hit
        slack = (min(0.2 * z0, 1e-4) + 2e-6) / speed
        assert toi >= t_hit - slack - 1e-9


# --- collision set -------------------------------------------------------------

def _brute_force(V, E, F, dhat, oracle_mod):
    """All EE and FV pairs without a broad phase (brute_force.cpp semantics),
    then the same filter: the collision set must not depend on the broad phase."""
    from itertools import combinations
    off = dhat * dhat
    vv, ev, ee, fv = {}, {}, [], []
    F2E = oracle_mod.faces_to_edges(F, E)
    for ea, eb in combinations(range(len(E)), 2):
        if set(E[ea]) & set(E[eb]):
            continue
        x = V[[E[ea][0], E[ea][1], E[eb][0], E[eb][1]]]
        t = oracle_mod.edge_edge_distance_type(*x)
        if not oracle_mod.edge_edge_distance(*x, dtype=t) < off:
            continue
        ids = [E[ea][0], E[ea][1], E[eb][0], E[eb][1]]
        ra = V[ids]
        eps = 1e-3 * np.sum((ra[0] - ra[1]) ** 2) * np.sum((ra[2] - ra[3]) ** 2)
        c = np.sum(np.cross(x[1] - x[0], x[3] - x[2]) ** 2)
        tt = 8 if c < eps else t
        if tt < 4:
            a, b = [(0, 2), (0, 3), (1, 2), (1, 3)][tt]
            k = (min(ids[a], ids[b]), max(ids[a], ids[b]))
            vv[k] = vv.get(k, 0) + 1
        elif tt < 8:
            e, v = [(ea, ids[2]), (ea, ids[3]), (eb, ids[0]), (eb, ids[1])][tt - 4]
            ev[(e, v)] = ev.get((e, v), 0) + 1
        else:
            ee.append((ea, eb, t))
    for f in range(len(F)):
        for v in range(len(V)):
            if v in F[f]:
                continue
            x = V[[v, F[f][0], F[f][1], F[f][2]]]
            t = oracle_mod.point_triangle_distance_type(*x)
            if not oracle_mod.point_triangle_distance(*x, dtype=t) < off:
                continue
            if t < 3:
                k = (min(v, F[f][t]), max(v, F[f][t]))
                vv[k] = vv.get(k, 0) + 1
            elif t < 6:
                k = (F2E[f][t - 3], v)
                ev[k] = ev.get(k, 0) + 1
            else:
                fv.append((f, v))
    return vv, ev, sorted(ee), sorted(fv)


@pytest.mark.parametrize("seed", [0, 1])
def test_collision_set_independent_of_broad_phase(oracle_mod, seed):
    from ipctk_gb300 import scenes
    sc = scenes.two_sheet(side=6, seed=seed, gap=3e-3, jitter=1e-3, dhat=4e-3)
    V, E, F = sc["V"], sc["E"], sc["F"]
    vv, ev, ee, fv = _brute_force(V, E, F, sc["dhat"], oracle_mod)
    col = oracle_mod.build_collisions(V, E, F, sc["dhat"])
    assert dict(zip(map(tuple, col.vv.tolist()), col.vv_w.tolist())) == vv
    assert dict(zip(map(tuple, col.ev.tolist()), col.ev_w.tolist())) == ev
    assert [(a, b, int(t)) for (a, b), t in zip(col.ee.tolist(), col.ee_dtype)] == ee
    assert list(map(tuple, col.fv.tolist())) == fv
    assert len(col) > 0


def test_collision_set_thread_independent(oracle_mod):
    from ipctk_gb300 import scenes
    sc = scenes.two_sheet(side=32, seed=2)
    a = oracle_mod.build_collisions(sc["V"], sc["E"], sc["F"], sc["dhat"], nthreads=1)
    b = oracle_mod.build_collisions(sc["V"], sc["E"], sc["F"], sc["dhat"], nthreads=8)
    for k in ("vv", "vv_w", "ev", "ev_w", "ee", "ee_dtype", "ee_eps", "fv"):
        assert np.array_equal(getattr(a, k), getattr(b, k))


def test_faces_to_edges_missing_edge(oracle_mod):
    F = np.array([[0, 1, 2]])
    E = np.array([[0, 1], [1, 2]])
    with pytest.raises(RuntimeError, match="Unable to find edge"):
        oracle_mod.faces_to_edges(F, E)


def test_psd_solvers_agree(oracle_mod):
    """The tridiagonal-QR projection used by default and an independent
    cyclic-Jacobi projection give the same projected Hessian."""
    rng = np.random.Generator(np.random.PCG64(31))
    try:
        for ctype in (0, 1, 3):
            n = {0: 2, 1: 3, 3: 4}[ctype]
            for _ in range(10):
                x = rng.uniform(-0.02, 0.02, 3 * n)
                oracle_mod.set_psd_solver("ql")
                _, _, A = oracle_mod.contact_local(ctype, x, 0.1, 1.0, psd="clamp")
                oracle_mod.set_psd_solver("jacobi")
                _, _, B = oracle_mod.contact_local(ctype, x, 0.1, 1.0, psd="clamp")
                assert np.linalg.norm(A - B) <= 1e-12 * np.linalg.norm(B)
    finally:
        oracle_mod.set_psd_solver("ql")


# --- area weighting ---------------------------------------------------------------

def test_mesh_areas_hand_checked(oracle_mod):
    """collision_mesh.cpp:309-374 on small meshes: one triangle, a codim
    polyline with an isolated vertex."""
    V = np.array([[0.0, 0, 0], [1, 0, 0], [0, 1, 0]])
    E = np.array([[0, 1], [1, 2], [2, 0]])
    F = np.array([[0, 1, 2]])
    va, ea = oracle_mod.mesh_areas(V, E, F)
    np.testing.assert_array_equal(va, np.full(3, 0.5 / 3.0))
    np.testing.assert_array_equal(ea, np.full(3, 0.5 / 3.0))
    # edges only: vertex = half its incident edge lengths; edge = its length;
    # an isolated vertex = 1
    V = np.array([[0.0, 0, 0], [2, 0, 0], [2, 3, 0], [9, 9, 9]])
    E = np.array([[0, 1], [1, 2]])
    va, ea = oracle_mod.mesh_areas(V, E, np.zeros((0, 3), np.int32))
    np.testing.assert_array_equal(va, [1.0, 2.5, 1.5, 1.0])
    np.testing.assert_array_equal(ea, [2.0, 3.0])


def test_mesh_areas_partition_the_surface(oracle_mod):
    """Vertex areas and edge areas each sum to the total surface area."""
    from ipctk_gb300 import scenes
    sc = scenes.sphere_pack(n_side=2, subdiv=2, seed=1)
    V, E, F = sc["V"], sc["E"], sc["F"]
    va, ea = oracle_mod.mesh_areas(V, E, F)
    a = 0.5 * np.linalg.norm(np.cross(V[F[:, 1]] - V[F[:, 0]], V[F[:, 2]] - V[F[:, 0]]), axis=1).sum()
    assert va.sum() == pytest.approx(a, rel=1e-12)
    assert ea.sum() == pytest.approx(a, rel=1e-12)


def test_area_weighted_collision_set(oracle_mod):
    """Same contacts as without weighting; FV weight vertex_area/4, EE weight
    (edge_area(ea)+edge_area(eb))/4 (normal_collisions_builder.cpp:146,181-183);
    merged VV/EV weights sum their contributions."""
    from ipctk_gb300 import scenes
    sc = scenes.two_sheet(side=12, seed=4)
    V, E, F = sc["V"], sc["E"], sc["F"]
    plain = oracle_mod.build_collisions(V, E, F, sc["dhat"])
    aw = oracle_mod.build_collisions(V, E, F, sc["dhat"], area_weighting=True)
    for k in ("vv", "ev", "ee", "fv"):
        np.testing.assert_array_equal(getattr(plain, k), getattr(aw, k))
    va, ea = oracle_mod.mesh_areas(V, E, F)
    np.testing.assert_array_equal(aw.fv_w, 0.25 * va[aw.fv[:, 1]])
    np.testing.assert_array_equal(aw.ee_w, 0.25 * (ea[aw.ee[:, 0]] + ea[aw.ee[:, 1]]))
    # every VV/EV contribution is a positive area over 4, at most
    # multiplicity * (largest contribution)
    assert np.all(aw.vv_w > 0) and np.all(aw.ev_w > 0)
    big = 0.25 * max(va.max(), 2 * ea.max())
    assert np.all(aw.vv_w <= plain.vv_w * big * (1 + 1e-15))
    assert np.all(aw.ev_w <= plain.ev_w * big * (1 + 1e-15))


# --- improved max approximation --------------------------------------------------

def _fan_with_point(p):
    """Six triangles around a centre vertex 0 on z = 0, plus a free vertex 7 at p."""
    ang = np.arange(6) * np.pi / 3
    V = np.vstack([[0.0, 0, 0], np.c_[np.cos(ang), np.sin(ang), np.zeros(6)], [p]])
    F = np.array([[0, 1 + k, 1 + (k + 1) % 6] for k in range(6)])
    E = np.array(sorted({tuple(sorted(e)) for f in F for e in ((f[0], f[1]), (f[1], f[2]), (f[2], f[0]))}))
    return V, E, F


def test_improved_max_approx_counts_a_vertex_contact_once(oracle_mod):
    """A vertex over the centre of a 6-triangle fan: the IPC set counts the
    vertex-vertex contact once per incident face (weight 6); the improved max
    approximation (normal_collisions_builder.cpp:340-455) brings it to 1."""
    h, dhat, kappa = 1e-3, 1e-2, 1.0
    V, E, F = _fan_with_point([0.0, 0.0, h])
    one = kappa * oracle_mod.barrier(h * h, dhat * dhat)
    ipc = oracle_mod.build_collisions(V, E, F, dhat)
    assert ipc.vv.tolist() == [[0, 7]] and ipc.vv_w.tolist() == [6.0]
    assert oracle_mod.barrier_energy(ipc, V, E, F, dhat, kappa) == pytest.approx(6 * one, rel=1e-14)
    imp = oracle_mod.build_collisions(V, E, F, dhat, improved_max_approx=True)
    # +1 on the vertex pair (face-vertex -> vertex-vertex), -1 on each of the
    # six spokes (face-vertex -> edge-vertex; the projection ratio is exactly 0,
    # so the point-edge type is P_E and the records stay edge-vertex)
    assert imp.vv.tolist() == [[0, 7]] and imp.vv_w.tolist() == [7.0]
    assert imp.ev.tolist() == [[e, 7] for e in range(6)] and imp.ev_w.tolist() == [-1.0] * 6
    assert oracle_mod.barrier_energy(imp, V, E, F, dhat, kappa) == pytest.approx(one, rel=1e-12)


def test_improved_max_approx_counts_an_edge_contact_once(oracle_mod):
    """A vertex over the middle of an edge shared by two triangles: IPC gives
    the edge-vertex contact weight 2, the improved set weight 1."""
    V = np.array([[0.0, 0, 0], [1, 0, 0], [0.5, 1, 0], [0.5, -1, 0], [0.5, 0, 1e-3]])
    F = np.array([[0, 1, 2], [1, 0, 3]])
    E = np.array([[0, 1], [1, 2], [2, 0], [0, 3], [3, 1]])
    ipc = oracle_mod.build_collisions(V, E, F, 1e-2)
    assert ipc.ev.tolist() == [[0, 4]] and ipc.ev_w.tolist() == [2.0]
    imp = oracle_mod.build_collisions(V, E, F, 1e-2, improved_max_approx=True)
    assert imp.ev.tolist() == [[0, 4]] and imp.ev_w.tolist() == [1.0]
    assert len(imp.vv) == len(imp.ee) == len(imp.fv) == 0
    one = oracle_mod.barrier(1e-6, 1e-4)
    assert oracle_mod.barrier_energy(imp, V, E, F, 1e-2, 1.0) == pytest.approx(one, rel=1e-12)
    # area weighting scales the weight to a quarter of the vertex's area
    aw = oracle_mod.build_collisions(V, E, F, 1e-2, improved_max_approx=True, area_weighting=True)
    va, _ = oracle_mod.mesh_areas(V, E, F)
    assert aw.ev.tolist() == [[0, 4]]
    assert aw.ev_w[0] == pytest.approx(0.25 * va[4], rel=1e-15)


def test_improved_max_approx_face_interior_unchanged(oracle_mod):
    V = np.array([[0.0, 0, 0], [1, 0, 0], [0, 1, 0], [0.25, 0.25, 1e-3]])
    F = np.array([[0, 1, 2]])
    E = np.array([[0, 1], [1, 2], [2, 0]])
    imp = oracle_mod.build_collisions(V, E, F, 1e-2, improved_max_approx=True)
    assert imp.fv.tolist() == [[0, 3]] and imp.fv_w.tolist() == [1.0]
    assert len(imp.vv) == len(imp.ev) == len(imp.ee) == 0


def test_improved_max_approx_on_sheets(oracle_mod):
    """On two close sheets every contact of the improved set has a nonzero
    weight, none of the IPC set's face-vertex contacts is lost, and the
    total weight does not grow (the improved set removes double counting)."""
    from ipctk_gb300 import scenes
    sc = scenes.two_sheet(side=12, seed=4)
    V, E, F = sc["V"], sc["E"], sc["F"]
    ipc = oracle_mod.build_collisions(V, E, F, sc["dhat"])
    imp = oracle_mod.build_collisions(V, E, F, sc["dhat"], improved_max_approx=True)
    for w in (imp.vv_w, imp.ev_w, imp.ee_w, imp.fv_w):
        assert np.all(w != 0)
    np.testing.assert_array_equal(imp.fv, ipc.fv)
    total = lambda c: sum(float(np.sum(w)) for w in (c.vv_w, c.ev_w, c.ee_w, c.fv_w))
    assert total(imp) <= total(ipc)


# --- friction ---------------------------------------------------------------------

@pytest.mark.parametrize("ms,mk", [(0.5, 0.5), (0.8, 0.4), (0.3, 0.6)])
def test_smooth_mu_derivatives(oracle_mod, ms, mk):
    """friction/smooth_mu.cpp: d/dy (mu f0) = (mu f1/y) y and
    d/dy (mu f1) = ((mu f1)' y - mu f1)/y^3 * y^3 + mu f1 / y, over the static,
    transition and kinetic ranges (friction/test_smooth_mu.cpp style)."""
    ev = 1e-3
    for y in np.linspace(0.05 * ev, 2 * ev, 23):
        if abs(y - ev) < 0.02 * ev or abs(y - 0.5 * ev) < 0.02 * ev:
            continue
        h = 1e-7 * ev
        f0 = lambda t: oracle_mod.friction_mu(0, t, ms, mk, ev)
        f1 = lambda t: oracle_mod.friction_mu(1, t, ms, mk, ev) * t
        d0 = (f0(y + h) - f0(y - h)) / (2 * h)
        assert d0 == pytest.approx(f1(y), rel=1e-6)
        d1 = (f1(y + h) - f1(y - h)) / (2 * h)
        f2 = oracle_mod.friction_mu(2, y, ms, mk, ev) * y ** 3 + f1(y)
        assert d1 == pytest.approx(f2 / y, rel=1e-5, abs=1e-9 / ev)
    # mu(y): mu_s at rest, mu_k beyond eps_v
    assert oracle_mod.friction_mu(3, 0.0, ms, mk, ev) == ms
    assert oracle_mod.friction_mu(3, 2 * ev, ms, mk, ev) == mk


def _friction_case(oracle_mod, seed=3):
    from ipctk_gb300 import scenes
    sc = scenes.two_sheet(side=10, seed=seed)
    V, E, F = sc["V"], sc["E"], sc["F"]
    col = oracle_mod.build_collisions(V, E, F, sc["dhat"])
    rng = np.random.Generator(np.random.PCG64(seed))
    mu_s = rng.uniform(0.3, 0.6, len(V))
    mu_k = mu_s * rng.uniform(0.6, 1.0, len(V))
    t = oracle_mod.tangential_build(col, V, E, F, sc["dhat"], sc["kappa"], mu_s, mu_k)
    return sc, V, E, F, col, t, rng


def test_tangential_build_properties(oracle_mod):
    """Orthonormal tangent bases orthogonal to the contact normal direction,
    positive normal forces, mu between the per-vertex extremes; one record per
    normal collision but the near-parallel edge-edge ones."""
    sc, V, E, F, col, t, _ = _friction_case(oracle_mod)
    assert len(t) > 0 and len(t.vv) == len(col.vv) and len(t.fv) == len(col.fv) and len(t.ev) == len(col.ev)
    assert len(t.ee) <= len(col.ee)
    B = t.P.reshape(-1, 2, 3)
    np.testing.assert_allclose(np.einsum("nij,nkj->nik", B, B), np.broadcast_to(np.eye(2), (len(t), 2, 2)),
                               atol=1e-12)
    assert np.all(t.N > 0)
    assert np.all((t.mu_s >= 0.3 - 1e-12) & (t.mu_s <= 0.6 + 1e-12))
    # face-vertex: the basis spans the triangle plane
    nvv, nev, nee = len(t.vv), len(t.ev), len(t.ee)
    for j, (f, v) in enumerate(t.fv[:50]):
        a, b, c = V[F[f]]
        n = np.cross(b - a, c - a)
        i = nvv + nev + nee + j
        assert abs(B[i] @ n).max() <= 1e-12 * np.linalg.norm(n)


@pytest.mark.parametrize("regime", ["static", "mixed", "kinetic"])
def test_friction_potential_derivatives_fd(oracle_mod, regime):
    """FrictionPotential gradient and Hessian against central differences of
    the energy and gradient (tangential_potential.cpp:156-331)."""
    sc, V, E, F, col, t, rng = _friction_case(oracle_mod)
    ev = 1e-3
    scale = {"static": 0.2 * ev, "mixed": 1.0 * ev, "kinetic": 20 * ev}[regime]
    U = rng.uniform(-1, 1, V.shape) * scale
    e = oracle_mod.friction_energy(t, U, E, F, ev)
    g = oracle_mod.friction_gradient(t, U, E, F, ev)
    assert e > 0 and np.linalg.norm(g) > 0
    idx = np.argsort(-np.abs(g))[:8]
    h = 1e-6 * scale
    for k in idx:
        d = np.zeros(U.size)
        d[k] = h
        fd = (oracle_mod.friction_energy(t, U + d.reshape(U.shape), E, F, ev)
              - oracle_mod.friction_energy(t, U - d.reshape(U.shape), E, F, ev)) / (2 * h)
        assert fd == pytest.approx(g[k], rel=1e-5, abs=1e-9 * np.abs(g).max())
    import scipy.sparse as sps
    rp, ci, va = oracle_mod.friction_hessian(t, U, E, F, ev)
    H = sps.csr_matrix((va, ci, rp), shape=(U.size, U.size))
    for k in idx[:4]:
        d = np.zeros(U.size)
        d[k] = h
        fd = (oracle_mod.friction_gradient(t, U + d.reshape(U.shape), E, F, ev)
              - oracle_mod.friction_gradient(t, U - d.reshape(U.shape), E, F, ev)) / (2 * h)
        col_k = H[:, k].toarray().ravel()
        assert np.linalg.norm(fd - col_k) <= 1e-4 * np.linalg.norm(col_k) + 1e-9 * abs(va).max()
    # the projected Hessian is positive semi-definite
    rp, ci, va = oracle_mod.friction_hessian(t, U, E, F, ev, psd="clamp")
    Hp = sps.csr_matrix((va, ci, rp), shape=(U.size, U.size)).toarray()
    used = np.unique(np.concatenate([t.vv.ravel(), t.ev[:, 1], t.fv[:, 1]]))
    assert np.linalg.eigvalsh(Hp).min() >= -1e-9 * abs(Hp).max()


def test_friction_energy_identities(oracle_mod):
    """Zero velocity: energy = sum w N mu_s eps_v / 3 (f0(0) = eps_v / 3,
    mu(0) = mu_s) for mu_s = mu_k; rigid translation in the normal direction
    gives no tangential slip."""
    sc, V, E, F, col, t, _ = _friction_case(oracle_mod)
    ev = 1e-3
    same = oracle_mod.tangential_build(col, V, E, F, sc["dhat"], sc["kappa"], 0.4)
    e0 = oracle_mod.friction_energy(same, np.zeros_like(V), E, F, ev)
    assert e0 == pytest.approx(float(np.sum(same.w * same.N)) * 0.4 * ev / 3, rel=1e-12)
    g0 = oracle_mod.friction_gradient(same, np.zeros_like(V), E, F, ev)
    assert np.abs(g0).max() == 0


# --- shape derivative -------------------------------------------------------------

def test_shape_derivative_structure(oracle_mod):
    """normal_potential.cpp:310-416 without area weighting: w times the
    unprojected local Hessian for every collision whose mollifier is inactive;
    only edge-edge stencils with cross^2 < eps_x differ from the Hessian."""
    import scipy.sparse as sps
    from ipctk_gb300 import scenes
    sc = scenes.two_sheet(side=12, seed=4)
    V, E, F = sc["V"], sc["E"], sc["F"]
    col = oracle_mod.build_collisions(V, E, F, sc["dhat"])
    n = V.size
    mat = lambda t: sps.csr_matrix((t[2], t[1], t[0]), shape=(n, n))
    S = mat(oracle_mod.barrier_shape_derivative(col, V, E, F, sc["dhat"], sc["kappa"]))
    H = mat(oracle_mod.barrier_hessian(col, V, E, F, sc["dhat"], sc["kappa"]))
    # without edge-edge records the two are the same matrix
    z2, z1 = np.zeros((0, 2), np.int32), np.zeros(0)
    noee = oracle_mod.Collisions.from_arrays(col.vv, col.vv_w, col.ev, col.ev_w, z2, z1, np.zeros(0, np.int8), z1,
                                             col.fv, col.fv_w)
    S0 = mat(oracle_mod.barrier_shape_derivative(noee, V, E, F, sc["dhat"], sc["kappa"]))
    H0 = mat(oracle_mod.barrier_hessian(noee, V, E, F, sc["dhat"], sc["kappa"]))
    assert sps.linalg.norm(S0 - H0) == 0
    # with them, differences stay inside the stencils of active (mollified) pairs
    active = set()
    for (ea, eb), eps in zip(col.ee, col.ee_eps):
        x = V[[E[ea, 0], E[ea, 1], E[eb, 0], E[eb, 1]]]
        if np.sum(np.cross(x[1] - x[0], x[3] - x[2]) ** 2) < eps:
            active.update(int(v) for v in (E[ea, 0], E[ea, 1], E[eb, 0], E[eb, 1]))
    assert active, "the two-sheet scene has mollified edge pairs"
    D = (S - H).tocoo()
    big = np.abs(D.data) > 1e-12 * abs(H).max()
    assert big.any()
    assert all(r // 3 in active and c // 3 in active for r, c in zip(D.row[big], D.col[big]))


def test_anisotropic_mu_eff(oracle_mod):
    """friction/test_anisotropic_friction.cpp:23-180: the elliptical effective
    coefficients along a direction, the principal axes, the (1, 0) default for
    a vanishing slip, and the isotropic fallback."""
    for ms0, ms1, mk0, mk1 in ((0.1, 0.7, 0.3, 0.5), (0.9, 0.3, 0.5, 0.1)):
        for ang in np.arange(0.0, 2 * np.pi, np.pi / 4):
            t = np.array([np.cos(ang), np.sin(ang)]) * 3.0
            s, k = oracle_mod.aniso_mu_eff(t, [ms0, ms1], [mk0, mk1], 0.5, 0.4)
            d = t / np.linalg.norm(t)
            assert s == pytest.approx(np.hypot(ms0 * d[0], ms1 * d[1]), rel=1e-14)
            assert k == pytest.approx(np.hypot(mk0 * d[0], mk1 * d[1]), rel=1e-14)
        assert oracle_mod.aniso_mu_eff([0, 2.0], [ms0, ms1], [mk0, mk1], 0.5, 0.4) == pytest.approx((ms1, mk1))
        assert oracle_mod.aniso_mu_eff([1e-12, 1e-12], [ms0, ms1], [mk0, mk1], 0.5, 0.4) == pytest.approx((ms0, mk0))
    assert oracle_mod.aniso_mu_eff([0.6, 0.8], [0, 0], [0, 0], 0.5, 0.4) == (0.5, 0.4)
    # only the static coefficients directional: kinetic stays isotropic
    assert oracle_mod.aniso_mu_eff([1.0, 0.0], [0.3, 0.6], [0, 0], 0.5, 0.4) == pytest.approx((0.3, 0.4))


def test_anisotropic_friction_fd(oracle_mod):
    """Anisotropic slip scaling and lagged directional coefficients: the
    gradient and Hessian stay the derivatives of the energy at fixed lagged mu."""
    import scipy.sparse as sps
    sc, V, E, F, col, t, rng = _friction_case(oracle_mod, seed=8)
    n = len(t)
    ev = 1e-3
    same = oracle_mod.friction_energy(t, np.zeros_like(V), E, F, ev)
    oracle_mod.tangential_set_anisotropy(t, np.ones((n, 2)), None, None)
    assert oracle_mod.friction_energy(t, np.zeros_like(V), E, F, ev) == same
    oracle_mod.tangential_set_anisotropy(t, rng.uniform(0.5, 2.0, (n, 2)), rng.uniform(0.2, 0.8, (n, 2)),
                                         rng.uniform(0.1, 0.5, (n, 2)))
    U = rng.uniform(-1, 1, V.shape) * ev
    oracle_mod.tangential_update_lagged_mu(t, V, np.zeros_like(V), U, E, F)
    ms, mk = oracle_mod.tangential_lagged_mu(t)
    assert np.any(ms != t.mu_s)
    e = oracle_mod.friction_energy(t, U, E, F, ev)
    g = oracle_mod.friction_gradient(t, U, E, F, ev)
    h = 1e-6 * ev
    for k in np.argsort(-np.abs(g))[:6]:
        d = np.zeros(U.size)
        d[k] = h
        fd = (oracle_mod.friction_energy(t, U + d.reshape(U.shape), E, F, ev)
              - oracle_mod.friction_energy(t, U - d.reshape(U.shape), E, F, ev)) / (2 * h)
        assert fd == pytest.approx(g[k], rel=1e-5, abs=1e-9 * np.abs(g).max())
        rp, ci, va = oracle_mod.friction_hessian(t, U, E, F, ev)
    H = sps.csr_matrix((va, ci, rp), shape=(U.size, U.size))
    for k in np.argsort(-np.abs(g))[:3]:
        d = np.zeros(U.size)
        d[k] = h
        fd = (oracle_mod.friction_gradient(t, U + d.reshape(U.shape), E, F, ev)
              - oracle_mod.friction_gradient(t, U - d.reshape(U.shape), E, F, ev)) / (2 * h)
        col_k = H[:, k].toarray().ravel()
        assert np.linalg.norm(fd - col_k) <= 1e-4 * np.linalg.norm(col_k) + 1e-9 * abs(va).max()


def test_friction_force_is_minus_gradient_at_build_state(oracle_mod):
    """With zero lagged displacement, isotropic coefficients and mu from the
    build, the force at velocity v is minus the potential's gradient at v
    (tangential_potential.cpp:333-410 against :184-231)."""
    sc, V, E, F, col, t, rng = _friction_case(oracle_mod, seed=9)
    ev = 1e-3
    U = rng.uniform(-1, 1, V.shape) * ev
    f = oracle_mod.friction_force(t, V, np.zeros_like(V), U, E, F, sc["dhat"], sc["kappa"], ev)
    g = oracle_mod.friction_gradient(t, U, E, F, ev)
    assert np.linalg.norm(f + g) <= 1e-12 * np.linalg.norm(g)
    # no_mu: the force of unit coefficients
    f1 = oracle_mod.friction_force(t, V, np.zeros_like(V), U, E, F, sc["dhat"], sc["kappa"], ev, no_mu=True)
    assert np.linalg.norm(f1) > np.linalg.norm(f)


def test_area_weighted_shape_derivative_weight_term_fd(oracle_mod):
    """The area-weighted shape derivative's extra term (grad_u f / w)(grad_x w)^T
    (normal_potential.cpp:330-355) against central differences of the
    gradient with respect to the rest positions (positions fixed), on a scene
    with no active mollifier, where that derivative is the whole term."""
    import scipy.sparse as sps
    from ipctk_gb300 import scenes
    sc = scenes.sphere_pack(n_side=2, subdiv=2, seed=3)
    V, E, F, dh, kp = sc["V"], sc["E"], sc["F"], sc["dhat"], sc["kappa"]
    col = oracle_mod.build_collisions(V, E, F, dh, area_weighting=True)
    assert len(col) > 0
    for (ea, eb), eps in zip(col.ee, col.ee_eps):
        x = V[[E[ea, 0], E[ea, 1], E[eb, 0], E[eb, 1]]]
        assert np.sum(np.cross(x[1] - x[0], x[3] - x[2]) ** 2) >= eps
    n = V.size
    mat = lambda t: sps.csr_matrix((t[2], t[1], t[0]), shape=(n, n))
    S = mat(oracle_mod.barrier_shape_derivative(col, V, E, F, dh, kp, area_weighting=True))
    S2 = mat(oracle_mod.barrier_shape_derivative(col, V, E, F, dh, kp, area_weighting=False))
    W = (S - S2).tocsc()
    assert abs(W).max() > 0
    g = lambda R: oracle_mod.barrier_gradient(oracle_mod.build_collisions(V, E, F, dh, rest=R, area_weighting=True),
                                              V, E, F, dh, kp)
    cols = np.unique(W.indices)[:: max(1, len(np.unique(W.indices)) // 8)]
    h = 1e-7
    for j in cols:
        d = np.zeros(n)
        d[j] = h
        fd = (g(V + d.reshape(V.shape)) - g(V - d.reshape(V.shape))) / (2 * h)
        wj = W[:, j].toarray().ravel()
        assert np.linalg.norm(fd - wj) <= 1e-5 * np.linalg.norm(wj) + 1e-9 * abs(W).max()


# --- edge-edge mollifier (distance/test_edge_edge_mollifier.cpp:14-292) --------

def _mollifier_edges(which):
    # get_edges(): "Perp" and "Almost parallel" (test_edge_edge_mollifier.cpp:14-38)
    if which == "perp":
        return np.array([[-1, 0, 0], [1, 0, 0], [0, -1, 0], [0, 1, 0]], float)
    return np.array([[-1, 0, 0], [1, 0, 0], [-1, 1e-9, 0], [1, -1e-9, 0]], float)


@pytest.mark.parametrize("which", ["perp", "almost_parallel"])
def test_ee_cross_squarednorm_kat_and_fd(oracle_mod, which):
    """Edge-Edge Cross Squarednorm (test_edge_edge_mollifier.cpp:40-80):
    16 for the perpendicular pair, 0 (margin 1e-9) for the almost parallel
    one; gradient and Hessian against finite differences."""
    x = _mollifier_edges(which)
    s, g, H = oracle_mod.ee_cross_sqnorm(x)
    if which == "perp":
        assert s == pytest.approx(16)
    else:
        assert abs(s) <= 1e-9
    f = lambda y: oracle_mod.ee_cross_sqnorm(y)[0]
    fg = _fd(f, x.ravel(), 1e-6)
    assert np.linalg.norm(g - fg) <= 1e-6 * max(1.0, np.linalg.norm(fg))
    fH = np.stack([_fd(lambda y: oracle_mod.ee_cross_sqnorm(y)[1][i], x.ravel(), 1e-6) for i in range(12)])
    assert np.linalg.norm(H - fH) <= 1e-5 * max(1.0, np.linalg.norm(fH))


@pytest.mark.parametrize("rel_x", [0.0, 0.5, 1.0, 2.0])
@pytest.mark.parametrize("eps_x", [1e-3, 1e-1, 1.0, 2.0])
def test_ee_mollifier_scalar(oracle_mod, rel_x, eps_x):
    """Edge-Edge Mollifier Scalar (test_edge_edge_mollifier.cpp:82-157):
    m in [0, 1], m = 1 beyond eps_x, and dm/dx against finite differences.
    The scalar is read through edges whose cross norm squared is x: ea along
    x with length 2, eb = (2 cos t, 2 sin t, 0) with 16 sin^2 t = x."""
    x = rel_x * eps_x

    def edges(xv):
        st = np.sqrt(min(xv / 16.0, 1.0))
        ct = np.sqrt(1.0 - st * st)
        return np.array([[-1, 0, 0], [1, 0, 0], [0, 0, 0.5], [2 * ct, 2 * st, 0.5]], float)

    m = oracle_mod.ee_mollifier(edges(x), eps_x)[0]
    assert 0 <= m <= 1
    if x > eps_x:
        assert m == 1
    # the closed form (edge_edge_mollifier.cpp:42-60) on the cross norm the edges really have
    s = oracle_mod.ee_cross_sqnorm(edges(x))[0]
    expect = 1.0 if s >= eps_x else (-s / eps_x + 2) * (s / eps_x)
    assert m == pytest.approx(expect, rel=1e-12, abs=1e-15)
    if abs(x - eps_x) > 1e-6 and 1e-4 < x < eps_x:
        h = 1e-8 * eps_x
        fd = (oracle_mod.ee_mollifier(edges(x + h), eps_x)[0] - oracle_mod.ee_mollifier(edges(x - h), eps_x)[0]) / (2 * h)
        assert fd == pytest.approx(2 / eps_x * (1 - x / eps_x), rel=1e-4)


@pytest.mark.parametrize("which", ["perp", "almost_parallel"])
def test_ee_mollifier_kat_and_fd(oracle_mod, which):
    """Edge-Edge Mollifier (test_edge_edge_mollifier.cpp:159-266) with rest
    edges along x and y (eps_x = 1e-3): m in [0, 1] (1 for the perpendicular
    pair, 0 for the parallel one), gradient and Hessian against finite
    differences."""
    rest = np.array([[0, 0, 0], [1, 0, 0], [0, 0, 0], [0, 1, 0]], float)
    eps = oracle_mod.ee_mollifier_threshold(rest)
    assert eps == pytest.approx(1e-3)
    x = _mollifier_edges(which)
    m, g, H = oracle_mod.ee_mollifier(x, eps)
    assert 0 <= m <= 1
    assert m == (1.0 if which == "perp" else pytest.approx(0.0, abs=1e-12))
    f = lambda y: oracle_mod.ee_mollifier(y, eps)[0]
    fg = _fd(f, x.ravel(), 1e-7)
    assert np.linalg.norm(g - fg) <= 1e-5 * max(1.0, np.linalg.norm(fg))
    fH = np.stack([_fd(lambda y: oracle_mod.ee_mollifier(y, eps)[1][i], x.ravel(), 1e-7) for i in range(12)])
    assert np.linalg.norm(H - fH) <= 1e-4 * max(1.0, np.linalg.norm(fH))


def test_ee_mollifier_threshold_kat(oracle_mod):
    """Edge-Edge Mollifier Threshold (test_edge_edge_mollifier.cpp:268-292):
    the perpendicular pair's eps_x is 1e-3 * 4 * 4 = 0.016."""
    assert oracle_mod.ee_mollifier_threshold(_mollifier_edges("perp")) == pytest.approx(0.016)
