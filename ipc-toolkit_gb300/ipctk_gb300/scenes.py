"""Seeded synthetic contact scenes for the benchmark workloads.

The reference publishes no dataset for this path, so every workload is a
seeded synthetic scene built here with numpy's PCG64 generator.  Each scene
is returned as a dict with:

    V      (nV, 3) float64 rest / current positions
    E      (nE, 2) int32 edges (unique, sorted (min, max) pairs)
    F      (nF, 3) int32 triangles
    V1     (nV, 3) float64 end-of-step positions for the collision-free
           step-size query
    dhat, kappa    barrier activation distance and stiffness

Workloads:
    two_sheet(...)    two 64x64 triangulated sheets 0.5e-3 apart (+-1e-4 jitter)
    sphere_pack(...)  512 icospheres (642 verts each) on a jittered 8x8x8 lattice
    layered_cloth(..) 8 stacked 256x256 sheets with sinusoidal in-plane waves
    batch(...)        256 uneven two-sheet scenes
"""
from __future__ import annotations

import numpy as np


def edges_from_faces(F: np.ndarray) -> np.ndarray:
    """Unique undirected edges of a triangle mesh as sorted (min, max) pairs."""
    e = np.concatenate([F[:, [0, 1]], F[:, [1, 2]], F[:, [2, 0]]], axis=0).astype(np.int64)
    e = np.sort(e, axis=1)
    n = int(e.max()) + 1 if e.size else 1
    key = np.unique(e[:, 0] * n + e[:, 1])  # row order of np.unique(e, axis=0)
    return np.ascontiguousarray(np.stack([key // n, key % n], axis=1).astype(np.int32))


def grid_sheet(n: int, z: float = 0.0, size: float = 1.0):
    """n x n vertex grid on [0,size]^2 at height z, two triangles per cell split
    on the same diagonal."""
    xs = np.linspace(0.0, size, n)
    X, Y = np.meshgrid(xs, xs, indexing="xy")
    V = np.stack([X.ravel(), Y.ravel(), np.full(n * n, z)], axis=1)
    i, j = np.meshgrid(np.arange(n - 1), np.arange(n - 1), indexing="xy")
    v00 = (j * n + i).ravel()
    v10 = v00 + 1
    v01 = v00 + n
    v11 = v01 + 1
    F = np.concatenate(
        [np.stack([v00, v10, v11], axis=1), np.stack([v00, v11, v01], axis=1)],
        axis=0,
    )
    return V.astype(np.float64), F.astype(np.int32)


def two_sheet(side: int = 64, gap: float = 5e-4, jitter: float = 1e-4,
              dhat: float = 1e-3, kappa: float = 1e3, ccd_dz: float = 1e-3,
              ccd_noise: float = 2e-4, seed: int = 0):
    """Two sheets: the lower at z=0, the upper at z=gap +- jitter per vertex with
    identical xy (every upper vertex sits exactly above a lower one).  V1 moves
    the upper sheet by -ccd_dz in z plus +-ccd_noise per coordinate."""
    rng = np.random.Generator(np.random.PCG64(seed))
    V0, F0 = grid_sheet(side, 0.0)
    V1s, F1 = grid_sheet(side, 0.0)
    nv = V0.shape[0]
    V1s[:, 2] = gap + rng.uniform(-jitter, jitter, nv)
    V = np.concatenate([V0, V1s], axis=0)
    F = np.concatenate([F0, F1 + nv], axis=0).astype(np.int32)
    Vend = V.copy()
    Vend[nv:, 2] -= ccd_dz
    Vend[nv:, :] += rng.uniform(-ccd_noise, ccd_noise, (nv, 3))
    return dict(V=V, F=F, E=edges_from_faces(F), V1=Vend, dhat=dhat,
                kappa=kappa, name=f"two_sheet_{side}", seed=seed)


def icosphere(subdiv: int = 3):
    """Unit icosphere by midpoint subdivision (subdiv 3: 642 verts, 1280 tris)."""
    t = (1.0 + 5 ** 0.5) / 2.0
    verts = [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t),
             (0, -1, -t), (0, 1, -t), (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]
    verts = [np.array(v, dtype=np.float64) / np.linalg.norm(v) for v in verts]
    faces = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9),
             (5, 11, 4), (11, 10, 2), (10, 7, 6), (7, 1, 8), (3, 9, 4), (3, 4, 2),
             (3, 2, 6), (3, 6, 8), (3, 8, 9), (4, 9, 5), (2, 4, 11), (6, 2, 10),
             (8, 6, 7), (9, 8, 1)]
    for _ in range(subdiv):
        cache = {}

        def mid(a, b):
            key = (min(a, b), max(a, b))
            if key not in cache:
                m = verts[a] + verts[b]
                verts.append(m / np.linalg.norm(m))
                cache[key] = len(verts) - 1
            return cache[key]

        nf = []
        for a, b, c in faces:
            ab, bc, ca = mid(a, b), mid(b, c), mid(c, a)
            nf += [(a, ab, ca), (b, bc, ab), (c, ca, bc), (ab, bc, ca)]
        faces = nf
    return np.array(verts), np.array(faces, dtype=np.int32)


def _random_rotation(rng):
    q = rng.normal(size=4)
    q /= np.linalg.norm(q)
    w, x, y, z = q
    return np.array([
        [1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
        [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
        [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]])


def sphere_pack(n_side: int = 8, radius: float = 0.02, subdiv: int = 3,
                gap_lo: float = 0.1e-3, gap_hi: float = 1.5e-3,
                dhat: float = 1e-3, kappa: float = 1e4, vmax: float = 2e-3,
                seed: int = 1):
    """n_side^3 icospheres with seeded random rotations on a lattice whose
    neighbouring centres are 2*radius + g apart, g ~ U(gap_lo, gap_hi) per
    axis gap.  V1 moves every sphere rigidly by |v| ~ U(0, vmax) toward its
    nearest neighbour."""
    rng = np.random.Generator(np.random.PCG64(seed))
    sv, sf = icosphere(subdiv)
    spacing = 2 * radius
    axes = []
    for _ in range(3):
        g = rng.uniform(gap_lo, gap_hi, n_side - 1)
        axes.append(np.concatenate([[0.0], np.cumsum(spacing + g)]))
    centers = np.stack(np.meshgrid(*axes, indexing="ij"), axis=-1).reshape(-1, 3)
    ns = centers.shape[0]
    Vs, Fs = [], []
    for k in range(ns):
        R = _random_rotation(rng)
        Vs.append(centers[k] + radius * sv @ R.T)
        Fs.append(sf + k * sv.shape[0])
    V = np.concatenate(Vs, 0)
    F = np.concatenate(Fs, 0).astype(np.int32)
    # rigid motion toward the nearest neighbouring centre
    d2 = ((centers[:, None, :] - centers[None, :, :]) ** 2).sum(-1)
    np.fill_diagonal(d2, np.inf)
    nn = np.argmin(d2, axis=1)
    dirs = centers[nn] - centers
    dirs /= np.linalg.norm(dirs, axis=1, keepdims=True)
    speed = rng.uniform(0.0, vmax, ns)
    disp = np.repeat(dirs * speed[:, None], sv.shape[0], axis=0)
    return dict(V=V, F=F, E=edges_from_faces(F), V1=V + disp, dhat=dhat,
                kappa=kappa, name="sphere_pack", seed=seed)


def layered_cloth(layers: int = 8, side: int = 256, gap_lo: float = 0.3e-3,
                  gap_hi: float = 1.2e-3, amp: float = 1e-2,
                  wl_lo: float = 0.05, wl_hi: float = 0.2, dhat: float = 1e-3,
                  kappa: float = 1e4, seed: int = 2):
    """Stacked sheets with per-layer gaps U(gap_lo, gap_hi) and in-plane
    sinusoidal displacement (amplitude amp, random phase and wavelength)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    Vs, Fs = [], []
    z = 0.0
    base_V, base_F = grid_sheet(side, 0.0)
    for layer in range(layers):
        if layer:
            z += rng.uniform(gap_lo, gap_hi)
        V = base_V.copy()
        V[:, 2] = z
        wl = rng.uniform(wl_lo, wl_hi, 2)
        ph = rng.uniform(0, 2 * np.pi, 2)
        V[:, 0] += amp * np.sin(2 * np.pi * V[:, 1] / wl[0] + ph[0])
        V[:, 1] += amp * np.sin(2 * np.pi * V[:, 0] / wl[1] + ph[1])
        Vs.append(V)
        Fs.append(base_F + layer * base_V.shape[0])
    V = np.concatenate(Vs, 0)
    F = np.concatenate(Fs, 0).astype(np.int32)
    V1 = V.copy()
    V1[:, 2] -= rng.uniform(0, 1e-3, V.shape[0])
    return dict(V=V, F=F, E=edges_from_faces(F), V1=V1, dhat=dhat,
                kappa=kappa, name="layered_cloth", seed=seed)


def batch(n_scenes: int = 256, side_lo: int = 16, side_hi: int = 256,
          seed: int = 3):
    """Uneven two-sheet scenes: side log-uniform in [side_lo, side_hi], dhat
    log-uniform in [1e-4, 1e-2], gap U(0.2, 0.9) dhat, CCD displacement
    -2 gap in z plus +-0.2 gap noise."""
    rng = np.random.Generator(np.random.PCG64(seed))
    out = []
    for k in range(n_scenes):
        side = int(round(np.exp(rng.uniform(np.log(side_lo), np.log(side_hi)))))
        dhat = float(np.exp(rng.uniform(np.log(1e-4), np.log(1e-2))))
        gap = float(rng.uniform(0.2, 0.9) * dhat)
        out.append(two_sheet(side=side, gap=gap, jitter=0.1 * gap, dhat=dhat,
                             kappa=1e4, ccd_dz=2 * gap, ccd_noise=0.2 * gap,
                             seed=int(rng.integers(1 << 31))))
    return out
