"""FP64 restatement of the Observe stage's disk-integrated flux (numpy).

TEST INFRASTRUCTURE ONLY: the checker of ``atpm_disk_flux``.  It follows
``observe`` (3905/Observe/NominalPole/wise_main.cpp:662-730, smooth surface)
over the stage's geometry (wise_main.cpp:555-645): vertices rotated by the
step's rotation angle, transformed by the pole matrix and offset to the
heliocentric centre; per facet the midpoint, unit normal, the frame
(edge 0 direction, normal x edge, normal), the view vector toward the
observer in that frame, its angle; the facet area as the geometry loop leaves
it (its last step); Planck radiance with the stage's constants
(wise_main.cpp:10-12).  The rotation table and the pole matrix use Python's
``math`` (the host libm), the rest is float64 numpy.
"""
from __future__ import annotations

import math

import numpy as np

AU = 149.6e9            # m (wise_main.cpp:8; the shape keeps its own units)
CVEL = 299792458.0      # wise_main.cpp:10
HCON = 6.626068963e-34  # wise_main.cpp:11
KCON = 1.380650424e-23  # wise_main.cpp:12


def pole_matrix(pole):
    """Pole transformation (3905/Thermal/NominalPole/main.cpp:907-919)."""
    r0, r1 = pole
    g = math.acos(math.cos(r0) * math.sin(abs(r1)))
    sg = math.sin(g)
    return np.array([
        [math.sin(r0) / sg, -1.0 * math.cos(r0) * math.cos(r0) * math.sin(r1) * math.cos(r1) / sg,
         math.cos(r0) * math.cos(r1)],
        [0.0, ((math.sin(r0) * math.sin(r0)) + (math.cos(r0) * math.cos(r0) * math.cos(r1) * math.cos(r1))) / sg,
         math.cos(r0) * math.sin(r1)],
        [-1.0 * math.cos(r0) * math.cos(r1) / sg, -1.0 * math.sin(r0) * math.cos(r0) * math.sin(r1) / sg,
         math.sin(r0)],
    ])


def centre(polar):
    return np.array([AU * polar[0] * math.cos(polar[1]) * math.cos(polar[2]),
                     AU * polar[0] * math.cos(polar[1]) * math.sin(polar[2]),
                     AU * polar[0] * math.sin(polar[1])])


def _vertices(v, tm, car, step, ntau):
    ang = 2.0 * math.pi * step / ntau
    c, sn = math.cos(ang), math.sin(ang)
    rq0 = v[:, 0] * c - v[:, 1] * sn
    rq1 = v[:, 0] * sn + v[:, 1] * c
    rq2 = v[:, 2]
    return np.stack([car[k] + ((tm[k, 0] * rq0 + tm[k, 1] * rq1) + tm[k, 2] * rq2) for k in range(3)], axis=1)


def _cross(a, b):
    return np.stack([a[:, 1] * b[:, 2] - a[:, 2] * b[:, 1],
                     a[:, 2] * b[:, 0] - a[:, 0] * b[:, 2],
                     a[:, 0] * b[:, 1] - a[:, 1] * b[:, 0]], axis=1)


def _norm(a):
    return np.sqrt((a[:, 0] * a[:, 0] + a[:, 1] * a[:, 1]) + a[:, 2] * a[:, 2])


def disk_flux(vertices, facets, ntau, pole, polar, observer, eps, temps, visibility, wavelengths_um):
    """polar: the body's heliocentric position, observer: its geocentric one
    (wise_main.cpp:530-538); temps: [ntau][nf]; visibility: [nf][ntau] or
    None.  Returns [ntau][nwl]."""
    v = np.asarray(vertices, np.float64)
    fc = np.asarray(facets)
    tm = pole_matrix(pole)
    car = centre(polar)
    obs = car - centre(observer)
    wl = np.asarray(wavelengths_um, np.float64) * 1.0e-6
    b1 = (2.0 * HCON * CVEL * CVEL) / wl ** 5.0
    lk = wl * KCON
    hc = HCON * CVEL

    def edges(step):
        h = _vertices(v, tm, car, step, ntau)
        h0, h1, h2 = h[fc[:, 0]], h[fc[:, 1]], h[fc[:, 2]]
        return ((h0 + h1) + h2) / 3.0, h1 - h0, h2 - h0

    _, e0, e1 = edges(ntau - 1)
    area = _norm(_cross(e0, e1)) / 2.0
    out = np.zeros((ntau, len(wl)))
    for s in range(ntau):
        hm, e0, e1 = edges(s)
        n = _cross(e0, e1)
        n = n / _norm(n)[:, None]
        xh = e0 / _norm(e0)[:, None]
        y = _cross(n, xh)
        ov = hm - obs
        o = _norm(ov)
        vv = -np.stack([(xh * ov).sum(1), (y * ov).sum(1), (n * ov).sum(1)], axis=1)
        va = np.arccos(vv[:, 2] / o)
        vis = ~(va > math.pi / 2.0)
        if visibility is not None:
            vis &= np.asarray(visibility)[:, s] != 0
        d = _norm(vv)
        mult = np.nan_to_num((eps * area) * np.cos(va) / (d * d))
        T = np.asarray(temps, np.float64)[s]
        with np.errstate(over="ignore", divide="ignore", invalid="ignore"):
            inten = b1[None, :] * (1.0 / (np.exp(hc / (lk[None, :] * T[:, None])) - 1.0))
        inten = np.nan_to_num(inten, nan=0.0)
        out[s] = np.where(vis[:, None], inten * mult[:, None], 0.0).sum(axis=0)
    return out


def crater_geometry(crater_vertices, crater_facets):
    """The crater's sub-facet unit normals and areas, and its projected area
    sum(area * n_z), in double from the float vertex positions the stage
    reads from the roughness visibility file (wise_main.cpp:407-420 read,
    464-490 surfacegeometry)."""
    p = np.asarray(crater_vertices, np.float32).astype(np.float64)
    fc = np.asarray(crater_facets)
    a, b, c = p[fc[:, 0]], p[fc[:, 1]], p[fc[:, 2]]
    n = _cross(b - a, c - a)
    nn = _norm(n)
    area = nn / 2.0
    n = n / nn[:, None]
    total = 0.0
    for j in range(len(fc)):  # the stage's summation order
        total = total + (area[j] * n[j, 2])
    return n, area, total


def rough_disk_flux(vertices, facets, ntau, pole, polar, observer, eps, sub_temps, sub_vis, crater_vertices,
                    crater_facets, visibility, wavelengths_um):
    """The rough-surface sum of observe (wise_main.cpp:695-727): for every
    facet visible at a step, the crater sub-facets with a visible fraction
    > 0 add B(T_sub) eps a_sub vis_sub cos(e_sub) / d^2 (e_sub from the view
    vector in the facet frame and the sub-facet normal, wise_main.cpp:515),
    and the facet's sum enters the disk total scaled by its area over the
    crater's projected area.  sub_temps, sub_vis: [nf][nsf][ntau] (the
    stage's file order).  Returns [ntau][nwl]."""
    v = np.asarray(vertices, np.float64)
    fc = np.asarray(facets)
    tm = pole_matrix(pole)
    car = centre(polar)
    obs = car - centre(observer)
    wl = np.asarray(wavelengths_um, np.float64) * 1.0e-6
    b1 = (2.0 * HCON * CVEL * CVEL) / wl ** 5.0
    lk = wl * KCON
    hc = HCON * CVEL
    sn, sa, stot = crater_geometry(crater_vertices, crater_facets)
    ST = np.asarray(sub_temps, np.float32).astype(np.float64)
    SV = np.asarray(sub_vis, np.float32).astype(np.float64)

    def edges(step):
        h = _vertices(v, tm, car, step, ntau)
        h0, h1, h2 = h[fc[:, 0]], h[fc[:, 1]], h[fc[:, 2]]
        return ((h0 + h1) + h2) / 3.0, h1 - h0, h2 - h0

    _, e0, e1 = edges(ntau - 1)
    area = _norm(_cross(e0, e1)) / 2.0
    out = np.zeros((ntau, len(wl)))
    for s in range(ntau):
        hm, e0, e1 = edges(s)
        n = _cross(e0, e1)
        n = n / _norm(n)[:, None]
        xh = e0 / _norm(e0)[:, None]
        y = _cross(n, xh)
        ov = hm - obs
        o = _norm(ov)
        vv = -np.stack([(xh * ov).sum(1), (y * ov).sum(1), (n * ov).sum(1)], axis=1)
        va = np.arccos(vv[:, 2] / o)
        vis = ~(va > math.pi / 2.0)
        if visibility is not None:
            vis &= np.asarray(visibility)[:, s] != 0
        d = _norm(vv)
        dots = ((vv[:, None, 0] * sn[None, :, 0] + vv[:, None, 1] * sn[None, :, 1]) + vv[:, None, 2] * sn[None, :, 2])
        ca = np.cos(np.arccos(dots / d[:, None]))
        T = ST[:, :, s]
        vsub = SV[:, :, s]
        with np.errstate(over="ignore", divide="ignore", invalid="ignore"):
            mult = (eps * sa[None, :]) * vsub * ca / (d * d)[:, None]
            mult = np.nan_to_num(mult, nan=0.0)
            for li in range(len(wl)):
                inten = b1[li] * (1.0 / (np.exp(hc / (lk[li] * T)) - 1.0))
                inten = np.nan_to_num(inten, nan=0.0)
                term = np.where(vsub > 0.0, inten * mult, 0.0)
                sfc = np.zeros(len(fc))
                for j in range(term.shape[1]):  # the stage's sub-facet order
                    sfc = sfc + term[:, j]
                out[s, li] = np.where(vis, sfc * area / stot, 0.0).sum()
    return out
