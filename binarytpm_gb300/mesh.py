"""Seeded synthetic shape models in the reference's text mesh format.

The reference reads a shape as ``NV`` lines ``x y z`` (km) followed by ``NF``
lines ``i j k`` (0-based vertex indices), see ``3905/Shape_Convert/main.cpp:19-34``
and the readers ``3905/Thermal/NominalPole/main.cpp:400-410`` and
``3905/Shape_Selfheating/main.cpp:168-178``.  Facet normals are taken as
``(v1 - v0) x (v2 - v0)`` (``main.cpp:976-978``), so every facet here is wound
counter-clockwise seen from outside.

Shapes:
  * ``icosphere(subdiv)``: a regular icosahedron split ``subdiv`` times
    (20 * 4**subdiv facets, 10 * 4**subdiv + 2 vertices).
  * ``perturbed_body``: an icosphere of radius ``r`` whose vertex radii are
    scaled by ``1 + U(-noise, +noise)`` (seeded), followed by one Laplacian
    smoothing pass of the radius field,
    ``r_i <- 0.5 r_i + 0.5 mean_{j in N(i)} r_j``.
  * ``grf_body``: radii ``r (1 + sigma g(x))`` with ``g`` a seeded Gaussian
    random field on the sphere of unit variance and Gaussian correlation
    length ``corr`` (radians), synthesised from random Fourier modes.
  * ``binary_system``: primary and secondary merged into one rigid mesh (the
    synchronous-binary form of ``3905/Thermal``), secondary offset by ``a`` km
    along +x.
"""
from __future__ import annotations

import numpy as np


def _icosahedron():
    t = (1.0 + 5.0 ** 0.5) / 2.0
    v = np.array([
        [-1, t, 0], [1, t, 0], [-1, -t, 0], [1, -t, 0],
        [0, -1, t], [0, 1, t], [0, -1, -t], [0, 1, -t],
        [t, 0, -1], [t, 0, 1], [-t, 0, -1], [-t, 0, 1],
    ], dtype=np.float64)
    f = np.array([
        [0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11],
        [1, 5, 9], [5, 11, 4], [11, 10, 2], [10, 7, 6], [7, 1, 8],
        [3, 9, 4], [3, 4, 2], [3, 2, 6], [3, 6, 8], [3, 8, 9],
        [4, 9, 5], [2, 4, 11], [6, 2, 10], [8, 6, 7], [9, 8, 1],
    ], dtype=np.int64)
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    return v, f


def icosphere(subdiv: int):
    """Unit icosphere; returns (vertices[nv,3] float64, facets[nf,3] int64)."""
    v, f = _icosahedron()
    verts = [tuple(x) for x in v]
    for _ in range(subdiv):
        cache: dict[tuple[int, int], int] = {}
        nf = []

        def mid(a: int, b: int) -> int:
            key = (a, b) if a < b else (b, a)
            idx = cache.get(key)
            if idx is None:
                p = np.add(verts[a], verts[b]) * 0.5
                p /= np.linalg.norm(p)
                verts.append(tuple(p))
                idx = len(verts) - 1
                cache[key] = idx
            return idx

        for a, b, c in f:
            ab, bc, ca = mid(a, b), mid(b, c), mid(c, a)
            nf += [(a, ab, ca), (b, bc, ab), (c, ca, bc), (ab, bc, ca)]
        f = np.array(nf, dtype=np.int64)
    v = np.array(verts, dtype=np.float64)
    # orient every facet outward: (v1-v0)x(v2-v0) . centroid > 0
    n = np.cross(v[f[:, 1]] - v[f[:, 0]], v[f[:, 2]] - v[f[:, 0]])
    c = v[f].mean(axis=1)
    flip = (n * c).sum(axis=1) < 0
    f[flip] = f[flip][:, [0, 2, 1]]
    return v, f


def _neighbours(nv: int, f: np.ndarray):
    edges = np.concatenate([f[:, [0, 1]], f[:, [1, 2]], f[:, [2, 0]]])
    edges = np.concatenate([edges, edges[:, ::-1]])
    edges = np.unique(edges, axis=0)
    return edges  # directed pairs (i, j)


def _laplacian_radius(r: np.ndarray, f: np.ndarray) -> np.ndarray:
    e = _neighbours(len(r), f)
    s = np.zeros_like(r)
    cnt = np.zeros_like(r)
    np.add.at(s, e[:, 0], r[e[:, 1]])
    np.add.at(cnt, e[:, 0], 1.0)
    return 0.5 * r + 0.5 * s / cnt


def perturbed_body(subdiv: int, radius_km: float, noise: float, seed: int):
    """Icosphere with seeded uniform radial noise and one Laplacian pass."""
    u, f = icosphere(subdiv)
    rng = np.random.default_rng(seed)
    r = radius_km * (1.0 + rng.uniform(-noise, noise, size=len(u)))
    r = _laplacian_radius(r, f)
    return u * r[:, None], f


def grf_body(subdiv: int, radius_km: float, sigma: float, corr_rad: float,
             seed: int, nmodes: int = 512):
    """Icosphere with a seeded Gaussian-random-field radial perturbation.

    g(x) = sqrt(2/M) sum_k cos(w_k . x + phi_k) with w_k ~ N(0, 1/corr^2 I),
    phi_k ~ U(0, 2 pi): a stationary unit-variance field in 3-D restricted to
    the unit sphere, with covariance exp(-|x-y|^2 / (2 corr^2)) (chord
    distance ~ angle for small separations).
    """
    u, f = icosphere(subdiv)
    rng = np.random.default_rng(seed)
    w = rng.normal(0.0, 1.0 / corr_rad, size=(nmodes, 3))
    phi = rng.uniform(0.0, 2.0 * np.pi, size=nmodes)
    g = np.sqrt(2.0 / nmodes) * np.cos(u @ w.T + phi).sum(axis=1)
    r = radius_km * np.clip(1.0 + sigma * g, 0.3, None)
    return u * r[:, None], f


def binary_system(primary, secondary, separation_km: float):
    """Merge two bodies into one rigid mesh; secondary shifted by +x."""
    vp, fp = primary
    vs, fs = secondary
    vs = vs + np.array([separation_km, 0.0, 0.0])
    v = np.concatenate([vp, vs])
    f = np.concatenate([fp, fs + len(vp)])
    return v, f


def write_shape(path, v: np.ndarray, f: np.ndarray) -> None:
    """Write the reference's text mesh format (17 significant digits so the
    reference's ``double`` reader recovers the exact values)."""
    with open(path, "w") as fh:
        for x in v:
            fh.write("%.17g\t%.17g\t%.17g\n" % (x[0], x[1], x[2]))
        for t in f:
            fh.write("%d\t%d\t%d\n" % (t[0], t[1], t[2]))


def read_shape(path, nv: int, nf: int):
    """Read the reference's text mesh format (values as float64)."""
    tok = open(path).read().split()
    v = np.array(tok[: 3 * nv], dtype=np.float64).reshape(nv, 3)
    f = np.array(tok[3 * nv: 3 * nv + 3 * nf], dtype=np.int64).reshape(nf, 3)
    return v, f
