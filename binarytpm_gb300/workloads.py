"""Seeded synthetic workloads with the shapes and sizes of the benchmark
configurations, their view-factor lists computed on the GPU
(atpm_viewfactors_compute), and the FP64 disk-integrated flux used as the
relative-flux error metric.

binary: primary icosphere subdivision 5 (20,480 facets, r = 0.39 km, +-5 %)
        + secondary subdivision 3 (1,280 facets, r = 0.08 km, +-8 %) merged
        rigidly 1.19 km apart (synchronous binary, P = 11.9 h), pole 85 deg from
        the Sun line (mutual orbit plane tilted 5 deg: eclipses occur);
        NX = 56, NTAU = 720, 1 AU, A = 0.02, eps = 0.9, TACC = 0.005 K.
single: one body, subdivision 3 (1,280 facets), P = 2.26 h, pole normal to
        the orbit, NX = 56, NTAU = 720 (the reference's explicit scheme needs
        NTAU >= 616 at NX = 56; 360 steps would be unstable).
"""
from __future__ import annotations

import math

import numpy as np

from . import problem as P

# thermal inertias of the batched sweep (SI), log-spaced over the reference's range
BATCH_TI = [25.0, 50.0, 100.0, 200.0, 400.0, 800.0, 1400.0, 2000.0]


def _lists(ctx, v, f):
    from . import lib

    ptr, idx, vf, vec, photo = lib.viewfactors(ctx, v, f, refine=True)
    return ptr, idx, vf


def binary_problem(ctx, p_subdiv=5, s_subdiv=3, ntau=720, nx=56, seed=2) -> P.Problem:
    v, f = P.binary_mesh(p_subdiv, s_subdiv, seed)
    ptr, idx, vf = _lists(ctx, v, f)
    return P.Problem(vertices=v, facets=f.astype(np.int32), dep_ptr=ptr, dep_idx=idx, dep_vf=vf,
                     ntau=ntau, nx=nx, polar=(1.0, 0.0, 0.0), pole=P.BINARY_POLE,
                     rotation_period_s=11.9 * 3600.0, albedo=0.02, emissivity=0.9,
                     thermal_inertia=200.0, tacc=0.005, name=f"binary_s{p_subdiv}s{s_subdiv}")


def single_problem(ctx, subdiv=3, ntau=720, nx=56, seed=1) -> P.Problem:
    v, f = P.single_body_mesh(subdiv, 0.39, 0.05, seed)
    ptr, idx, vf = _lists(ctx, v, f)
    return P.Problem(vertices=v, facets=f.astype(np.int32), dep_ptr=ptr, dep_idx=idx, dep_vf=vf,
                     ntau=ntau, nx=nx, polar=(1.0, 0.0, 0.0), pole=(math.pi / 2, 0.0),
                     rotation_period_s=2.26 * 3600.0, albedo=0.02, emissivity=0.9,
                     thermal_inertia=200.0, tacc=0.005, name=f"single_s{subdiv}")


def facet_areas(problem) -> np.ndarray:
    v, f = problem.vertices, problem.facets
    n = np.cross(v[f[:, 1]] - v[f[:, 0]], v[f[:, 2]] - v[f[:, 0]])
    return 0.5 * np.linalg.norm(n, axis=1) * 1e6  # m^2


def planck(wavelength_um: float, T: np.ndarray) -> np.ndarray:
    """Spectral radiance B_lambda (W m^-2 sr^-1 m^-1), FP64."""
    h, c, k = 6.62607015e-34, 299792458.0, 1.380649e-23
    lam = wavelength_um * 1e-6
    x = h * c / (lam * k * np.maximum(T, 1e-3))
    return 2.0 * h * c * c / lam ** 5 / np.expm1(np.minimum(x, 700.0))


def disk_flux(problem, stemp1: np.ndarray, cosillum: np.ndarray, shadow: np.ndarray,
              wavelength_um: float = 12.0) -> np.ndarray:
    """FP64 disk-integrated thermal emission seen from the Sun direction
    (zero phase): per step sum over illuminated facets of
    eps * A_f * cos(e) * B_lambda(T), the smooth-surface form of the
    reference's flux synthesis (3905/Observe/NominalPole/wise_main.cpp:662-796)."""
    A = facet_areas(problem)[:, None]
    vis = (shadow > 0) & (cosillum > 0)
    w = np.where(vis, A * cosillum.astype(np.float64), 0.0) * problem.emissivity
    return (w * planck(wavelength_um, stemp1.astype(np.float64))).sum(axis=0)
