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


def _lists(ctx, v, f, with_vectors=False):
    from . import lib

    ptr, idx, vf, vec, photo = lib.viewfactors(ctx, v, f, refine=True)
    return (ptr, idx, vf, vec) if with_vectors else (ptr, idx, vf)


def binary_problem(ctx, p_subdiv=5, s_subdiv=3, ntau=720, nx=56, seed=2) -> P.Problem:
    """The synchronous binary; meta["dep_vec"] keeps the list entries'
    direction vectors (the crater forcing needs them)."""
    v, f = P.binary_mesh(p_subdiv, s_subdiv, seed)
    ptr, idx, vf, vec = _lists(ctx, v, f, with_vectors=True)
    return P.Problem(vertices=v, facets=f.astype(np.int32), dep_ptr=ptr, dep_idx=idx, dep_vf=vf,
                     ntau=ntau, nx=nx, polar=(1.0, 0.0, 0.0), pole=P.BINARY_POLE,
                     rotation_period_s=11.9 * 3600.0, albedo=0.02, emissivity=0.9,
                     thermal_inertia=200.0, tacc=0.005, name=f"binary_s{p_subdiv}s{s_subdiv}",
                     meta={"dep_vec": np.asarray(vec, np.float32).reshape(-1, 3)})


def stress_problem(ctx, p_subdiv=6, s_subdiv=4, ntau=720, nx=56, seed=3) -> P.Problem:
    """Precision stress: a concave primary (icosphere subdivision 6 = 81,920
    facets, r = 0.39 km, seeded Gaussian-random-field radii, sigma 15 %,
    correlation 0.3 rad) + a 5,120-facet secondary (subdivision 4, r = 0.08
    km, +-8 %), merged 1.19 km apart like the binary; view factors from
    mutual visibility on the GPU."""
    from . import mesh

    prim = mesh.grf_body(p_subdiv, 0.39, 0.15, 0.3, seed)
    sec = mesh.perturbed_body(s_subdiv, 0.08, 0.08, seed + 1000)
    v, f = mesh.binary_system(prim, sec, 1.19)
    ptr, idx, vf = _lists(ctx, v, f)
    return P.Problem(vertices=v, facets=f.astype(np.int32), dep_ptr=ptr, dep_idx=idx, dep_vf=vf,
                     ntau=ntau, nx=nx, polar=(1.0, 0.0, 0.0), pole=P.BINARY_POLE,
                     rotation_period_s=11.9 * 3600.0, albedo=0.02, emissivity=0.9,
                     thermal_inertia=200.0, tacc=0.005, name=f"stress_s{p_subdiv}s{s_subdiv}")


def fast_vs_fp64(ctx, prob, tis, revs, shadow, illum):
    """FAST (batched) vs plain FP64 after the same ``revs`` revolutions with
    every facet advancing every revolution (freeze off), so both runs follow
    the same schedule: max |T_fast - T_fp64| over facets, steps and thermal
    inertias, and the relative error of the disk-integrated 12 um flux seen
    from the Sun, reduced in FP64 on the GPU (atpm_disk_flux)."""
    from . import lib

    fast = [lib.Solve(ctx, prob, precision=lib.FAST, revcap=revs, freeze=False) for _ in tis]
    for s, ti in zip(fast, tis):
        s.set_forcing(shadow, illum)
        s.set_thermal_inertia(ti)
        s.initialise_temperatures()
    lib.batch_run(fast)
    ref = lib.Solve(ctx, prob, precision=lib.FP64, revcap=revs, freeze=False)
    ref.set_forcing(shadow, illum)
    errs, ferrs = {}, {}
    for s, ti in zip(fast, tis):
        ref.set_thermal_inertia(ti)
        ref.initialise_temperatures()
        ref.run()
        t64 = ref.surface_temperature64()
        t32 = s.surface_temperature64()
        errs[str(ti)] = float(np.max(np.abs(t32 - t64)))
        F64 = ref.disk_flux(prob.polar, (12.0,), shadow)[:, 0]
        F32 = s.disk_flux(prob.polar, (12.0,), shadow)[:, 0]
        ferrs[str(ti)] = float(np.max(np.abs(F32 - F64) / np.abs(F64)))
        s.close()
    ref.close()
    return {"max_temperature_error_K": max(errs.values()), "max_rel_flux_error_12um": max(ferrs.values()),
            "per_ti_max_K": errs, "per_ti_rel_flux": ferrs,
            "schedule": f"{revs} revolutions, every facet advancing (freeze off), same forcing"}


def fp64_errors(ctx, prob, solves, tis, revs, shadow, illum, freeze=True, run=False):
    """Errors of already-prepared solves (any precision, one per thermal
    inertia in ``tis``) against plain FP64 run on the same schedule: FP64
    solves from the same forcing and initial temperatures for ``revs``
    revolutions with the same freeze setting.  With ``run`` the given
    solves are first given the forcing and run as one batch; otherwise
    their current state is compared (they must have run that schedule).
    Returns the max |T - T_fp64| and the relative error of the
    disk-integrated 12 um flux seen from the Sun (FP64 on the GPU)."""
    from . import lib

    if run:
        for s, ti in zip(solves, tis):
            s.set_forcing(shadow, illum)
            s.set_thermal_inertia(ti)
            s.initialise_temperatures()
        lib.batch_run(solves)
    ref = lib.Solve(ctx, prob, precision=lib.FP64, revcap=revs, freeze=freeze)
    ref.set_forcing(shadow, illum)
    errs, ferrs, nrev = {}, {}, {}
    for s, ti in zip(solves, tis):
        ref.set_thermal_inertia(ti)
        ref.initialise_temperatures()
        nrev[str(ti)] = int(len(ref.run()))
        t64 = ref.surface_temperature64()
        errs[str(ti)] = float(np.max(np.abs(s.surface_temperature64() - t64)))
        F64 = ref.disk_flux(prob.polar, (12.0,), shadow)[:, 0]
        F = s.disk_flux(prob.polar, (12.0,), shadow)[:, 0]
        ferrs[str(ti)] = float(np.max(np.abs(F - F64) / np.abs(F64)))
    ref.close()
    return {"max_temperature_error_K": max(errs.values()), "max_rel_flux_error_12um": max(ferrs.values()),
            "per_ti_max_K": errs, "per_ti_rel_flux": ferrs, "fp64_revolutions": nrev,
            "schedule": f"revolution cap {revs}, freeze {'on' if freeze else 'off'}, same forcing and "
                        "initial temperatures"}


def single_problem(ctx, subdiv=3, ntau=720, nx=56, seed=1) -> P.Problem:
    v, f = P.single_body_mesh(subdiv, 0.39, 0.05, seed)
    ptr, idx, vf = _lists(ctx, v, f)
    return P.Problem(vertices=v, facets=f.astype(np.int32), dep_ptr=ptr, dep_idx=idx, dep_vf=vf,
                     ntau=ntau, nx=nx, polar=(1.0, 0.0, 0.0), pole=(math.pi / 2, 0.0),
                     rotation_period_s=2.26 * 3600.0, albedo=0.02, emissivity=0.9,
                     thermal_inertia=200.0, tacc=0.005, name=f"single_s{subdiv}")


# fewest list entries a (128-row, 64-column) cell needs to become a
# tensor-core tile (the library's default, ATPM_TC_MIN_ENTRIES)
TC_MIN_ENTRIES = 32


def tc_tile_structure(nf, dep_ptr, dep_idx, dep_vf, min_entries=TC_MIN_ENTRIES):
    """The FAST tensor-core tiling of a view-factor list, restated in numpy:
    the 128 x 64 tiles kept (keys row block * nkb + column block, sorted:
    cells holding at least ``min_entries`` list entries), the tile of every
    list entry (-1 for the entries of sparser cells, the sparse remainder
    summed in FP32 outside the tensor cores), the entries' 16-wide K slices,
    and which tiles carry the residual V - bf16(V): a view factor >= 1e-4,
    or, for some facet row, at least 1 % of that row's mean |view factor|
    per 64-facet column block it touches (the rule of build_tc/k_tc_rowneed;
    that mean counts every column block the row touches, tile or not)."""
    nkb = (nf + 63) // 64
    rows = np.repeat(np.arange(nf), np.diff(dep_ptr))
    av = np.abs(np.asarray(dep_vf, np.float32))
    key = (rows // 128).astype(np.int64) * nkb + np.asarray(dep_idx) // 64
    cells, cinv, ccount = np.unique(key, return_inverse=True, return_counts=True)
    keep = ccount >= min_entries
    tiles = cells[keep]
    tile_of_cell = np.full(len(cells), -1, np.int64)
    tile_of_cell[keep] = np.arange(keep.sum())
    inv = tile_of_cell[cinv] if len(cinv) else np.zeros(0, np.int64)
    vmax = np.zeros(len(cells), np.float32)
    np.maximum.at(vmax, cinv, av)
    has_lo = vmax >= np.float32(1e-4)
    rk = rows.astype(np.int64) * nkb + np.asarray(dep_idx) // 64
    u, rinv = np.unique(rk, return_inverse=True)
    m = np.bincount(rinv, weights=av.astype(np.float64))
    r = u // nkb
    M = np.bincount(r, weights=m, minlength=nf)
    n = np.bincount(r, minlength=nf)
    need = 100.0 * n[r] * m >= M[r]
    need_keys = np.unique((r[need] // 128) * nkb + u[need] % nkb)
    has_lo |= np.isin(cells, need_keys)
    slices = np.asarray(dep_idx) % 64 // 16
    return tiles, inv, slices, has_lo[keep]


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


def roughness_mix(smooth, rough, fraction):
    """The fitting's model flux for a surface covered by craters over the
    given fraction of its area: fraction * rough + (1 - fraction) * smooth
    (175706/Run-04/fitting.cpp:460-461), per step and wavelength."""
    return fraction * np.asarray(rough) + (1.0 - fraction) * np.asarray(smooth)
