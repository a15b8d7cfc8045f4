"""A thermophysical solve description: shape, view-factor lists and the
physical/numerical parameters the reference fixes as compile-time constants
(``3905/Thermal/NominalPole/main.cpp:17-64``), held at run time instead.

Synthetic workloads
-------------------
``cfg_single``  one body: icosphere subdivision 3 (1,280 facets), r = 0.39 km,
                +-5 % seeded radial noise + one Laplacian pass; P = 2.26 h; pole
                normal to the orbit; 1 AU; A = 0.02, eps = 0.9, Gamma = 200;
                NX = 56 to 8 skin depths; shadowing + self-heating on;
                TACC = 0.005 K.
``cfg_binary``  primary subdivision 5 (20,480 facets, 0.39 km, +-5 %) + secondary
                subdivision 3 (1,280 facets, 0.08 km, +-8 %), rigidly merged with
                a 1.19 km separation (synchronous binary, P = 11.9 h); pole 85 deg
                from the Sun line so the mutual orbit plane is tilted 5 deg and
                eclipses occur; NX = 56, NTAU = 720; no roughness.

Explicit-scheme stability: the reference's FTCS update is stable only for
r = (2 pi / NTAU) / (8 / NX)^2 <= 1/2.  At NX = 56 that needs NTAU >= 616 and at
NX = 48 NTAU >= 453; every workload here therefore uses NTAU = 720 (r = 0.428 at
NX = 56, 0.314 at NX = 48), for the reference runs and the GPU runs alike.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field, replace

import numpy as np

from . import mesh


@dataclass
class Problem:
    vertices: np.ndarray            # [nv,3] float64 km
    facets: np.ndarray              # [nf,3] int32
    dep_ptr: np.ndarray             # [nf+1] int32
    dep_idx: np.ndarray             # [nnz] int32
    dep_vf: np.ndarray              # [nnz] float32
    ntau: int = 720
    nx: int = 56
    polar: tuple = (1.0, 0.0, 0.0)  # AU, ecliptic latitude, longitude (rad)
    pole: tuple = (math.pi / 2, 0.0)  # pole ecliptic latitude, longitude (rad)
    rotation_period_s: float = 2.26 * 3600.0
    albedo: float = 0.02
    emissivity: float = 0.9
    thermal_inertia: object = 200.0  # scalar or sweep list
    tacc: float = 0.005
    scattering_accuracy: float = 1e-4
    shadowing: int = 1               # 0 off, 1 dependent list, 2 all pairs
    multiple_scattering: int = 1
    name: str = "shape"
    meta: dict = field(default_factory=dict)

    @property
    def nf(self) -> int:
        return len(self.facets)

    @property
    def nv(self) -> int:
        return len(self.vertices)

    @property
    def nnz(self) -> int:
        return int(self.dep_ptr[-1])

    def with_(self, **kw) -> "Problem":
        return replace(self, **kw)

    def stability_r(self) -> float:
        return (2.0 * math.pi / self.ntau) / (8.0 / self.nx) ** 2


def empty_lists(nf: int):
    return (np.zeros(nf + 1, np.int32), np.zeros(0, np.int32), np.zeros(0, np.float32))


def single_body_mesh(subdiv=3, radius_km=0.39, noise=0.05, seed=1):
    return mesh.perturbed_body(subdiv, radius_km, noise, seed)


def binary_mesh(p_subdiv=5, s_subdiv=3, seed=2):
    prim = mesh.perturbed_body(p_subdiv, 0.39, 0.05, seed)
    sec = mesh.perturbed_body(s_subdiv, 0.08, 0.08, seed + 1000)
    return mesh.binary_system(prim, sec, 1.19)


# pole 85 deg from the +x axis: latitude 85 deg, longitude 0 (the Sun lies along -x
# from an asteroid at ecliptic longitude 0), so the mutual orbit plane is tilted 5 deg
BINARY_POLE = (math.radians(85.0), 0.0)
