"""ctypes binding of libatpm (include/atpm.h) and a thin Python mirror of the
reference driver's single_model flow (3905/Thermal/NominalPole/main.cpp:2417-2590).

The CUDA library is the only compute path: if ``libatpm.so`` is missing or
fails to load, :func:`load` raises; there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

PKG = Path(__file__).resolve().parent
LIB_PATH = PKG / "libatpm.so"

REFERENCE, FP64, FAST = 0, 1, 2
PRECISIONS = {"reference": REFERENCE, "fp64": FP64, "fast": FAST}


class AtpmError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"atpm status {status}: {msg}")
        self.status = status


class Shape(C.Structure):
    _fields_ = [("nv", C.c_int32), ("nf", C.c_int32),
                ("vertices", C.c_void_p), ("facets", C.c_void_p),
                ("dep_ptr", C.c_void_p), ("dep_idx", C.c_void_p), ("dep_vf", C.c_void_p)]


class Params(C.Structure):
    _fields_ = [("ntau", C.c_int32), ("nx", C.c_int32),
                ("polar", C.c_double * 3), ("pole", C.c_double * 2),
                ("rotation_period_s", C.c_float), ("albedo", C.c_float), ("emissivity", C.c_float),
                ("tacc", C.c_float), ("scattering_accuracy", C.c_float),
                ("shadowing", C.c_int32), ("multiple_scattering", C.c_int32),
                ("revcap", C.c_int32), ("precision", C.c_int32), ("freeze", C.c_int32)]


_lib = None

_SIGS = {
    "atpm_status_string": (C.c_char_p, [C.c_int]),
    "atpm_last_error": (C.c_char_p, []),
    "atpm_version": (C.c_int32, []),
    "atpm_context_create": (C.c_int, [C.c_int32, C.POINTER(C.c_void_p)]),
    "atpm_context_destroy": (C.c_int, [C.c_void_p]),
    "atpm_solve_create": (C.c_int, [C.c_void_p, C.POINTER(Shape), C.POINTER(Params), C.POINTER(C.c_void_p)]),
    "atpm_solve_destroy": (C.c_int, [C.c_void_p]),
    "atpm_solve_clone": (C.c_int, [C.c_void_p, C.POINTER(C.c_void_p)]),
    "atpm_solve_footprint": (C.c_int, [C.POINTER(Shape), C.POINTER(Params), C.POINTER(C.c_uint64)]),
    "atpm_geometry_shadow": (C.c_int, [C.c_void_p]),
    "atpm_scattering": (C.c_int, [C.c_void_p]),
    "atpm_set_forcing": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "atpm_set_thermal_inertia": (C.c_int, [C.c_void_p, C.c_float]),
    "atpm_initialise_temperatures": (C.c_int, [C.c_void_p]),
    "atpm_revolution": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p]),
    "atpm_run": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "atpm_single_model": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p]),
    "atpm_batch_run": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p]),
    "atpm_get_shadow": (C.c_int, [C.c_void_p, C.c_void_p]),
    "atpm_get_illumination": (C.c_int, [C.c_void_p, C.c_void_p]),
    "atpm_get_surface_temperature": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "atpm_get_surface_temperature64": (C.c_int, [C.c_void_p, C.c_void_p]),
    "atpm_get_surface_temperatures": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p]),
    "atpm_get_depth_temperature": (C.c_int, [C.c_void_p, C.c_void_p]),
    "atpm_get_converged": (C.c_int, [C.c_void_p, C.c_void_p]),
    "atpm_energy_balance": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "atpm_orbital_position": (C.c_int, [C.c_double, C.c_double, C.c_double, C.c_double, C.c_double, C.c_double,
                                        C.c_void_p]),
    "atpm_set_position": (C.c_int, [C.c_void_p, C.c_void_p]),
    "atpm_set_binary_rotation": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.c_int32, C.c_int32]),
    "atpm_set_ir_absorptivity": (C.c_int, [C.c_void_p, C.c_float]),
    "atpm_disk_flux": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_double, C.c_int32, C.c_void_p,
                                 C.c_void_p]),
    "atpm_last_run_stats": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "atpm_last_run_config": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "atpm_get_cosillum": (C.c_int, [C.c_void_p, C.c_void_p]),
    "atpm_selftest_bounded_wait": (C.c_int, [C.c_int32, C.c_int64, C.c_void_p]),
    "atpm_last_shadow_stats": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "atpm_selfheating_flux": (C.c_int, [C.c_void_p, C.c_void_p]),
    "atpm_profile_revolution": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p]),
    "atpm_scattering_noalloc": (C.c_int, [C.c_int32, C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                          C.c_void_p, C.c_float, C.c_float, C.c_float, C.c_int32, C.c_void_p,
                                          C.c_void_p, C.c_void_p]),
    "atpm_server_create": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.c_uint64, C.c_int32, C.c_int32,
                                     C.POINTER(C.c_void_p)]),
    "atpm_server_add_shape": (C.c_int, [C.c_void_p, C.POINTER(Shape), C.POINTER(Params), C.POINTER(C.c_int32)]),
    "atpm_server_submit": (C.c_int, [C.c_void_p, C.c_int32, C.c_float, C.POINTER(C.c_int64)]),
    "atpm_server_cancel": (C.c_int, [C.c_void_p, C.c_int64]),
    "atpm_server_wait": (C.c_int, [C.c_void_p, C.c_int64, C.c_double, C.c_void_p, C.c_void_p, C.c_void_p]),
    "atpm_server_stats": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "atpm_server_destroy": (C.c_int, [C.c_void_p]),
    "atpm_viewfactors_compute": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.c_void_p, C.c_void_p, C.c_int32,
                                           C.POINTER(C.c_void_p), C.POINTER(C.c_int64)]),
    "atpm_viewfactors_get": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "atpm_viewfactors_free": (C.c_int, [C.c_void_p]),
    "atpm_crater_create": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_int32,
                                     C.POINTER(C.c_void_p)]),
    "atpm_crater_destroy": (C.c_int, [C.c_void_p]),
    "atpm_crater_set_model": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                        C.c_float]),
    "atpm_crater_set_properties": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "atpm_crater_get_properties": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "atpm_crater_set_array": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p]),
    "atpm_crater_get_array": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p]),
    "atpm_crater_partial_shadow": (C.c_int, [C.c_void_p]),
    "atpm_crater_scattering": (C.c_int, [C.c_void_p, C.c_float, C.c_float, C.c_int32]),
    "atpm_crater_zero_temperatures": (C.c_int, [C.c_void_p]),
    "atpm_crater_initialise_temperatures": (C.c_int, [C.c_void_p, C.c_float, C.c_float]),
    "atpm_crater_inertia_difference": (C.c_int, [C.c_void_p, C.c_float, C.c_float, C.c_float]),
    "atpm_crater_inst_equilibrium": (C.c_int, [C.c_void_p, C.c_float, C.c_float]),
    "atpm_crater_converged": (C.c_int, [C.c_void_p, C.c_float]),
    "atpm_crater_get_temperatures": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "atpm_crater_set_array_strided": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p, C.c_uint64]),
    "atpm_crater_get_array_strided": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p, C.c_uint64]),
    "atpm_disk_flux_rough": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p,
                                       C.c_void_p, C.c_void_p, C.c_double, C.c_int32, C.c_void_p, C.c_void_p]),
    "atpm_crater_set_surface": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p, C.c_float]),
    "atpm_crater_forcing": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int32, C.c_void_p]),
    "atpm_crater_prepare_part": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int32, C.c_int32, C.c_int32, C.c_void_p]),
    "atpm_crater_global_heating": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int32]),
    "atpm_solve_solar": (C.c_int, [C.c_void_p, C.POINTER(C.c_float)]),
    "atpm_set_albedo": (C.c_int, [C.c_void_p, C.c_float]),
}


def load(path: Path | None = None):
    """Load libatpm.so (raises if it is absent: no fallback exists)."""
    global _lib
    if _lib is not None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise FileNotFoundError(f"{p} not built; run __graft_entry__.build() or python -m binarytpm_gb300.build")
    lib = C.CDLL(str(p))
    for name, (res, args) in _SIGS.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def exported_symbols():
    return list(_SIGS)


def host_buffer(shape, dtype) -> np.ndarray:
    """Uninitialised host array in page-locked memory (torch's cached pinned
    allocator) when torch sees a CUDA device, so copies to and from it run
    as direct DMA; plain numpy otherwise.  For inputs a caller uploads every
    job and for read-back buffers it reuses (``Solve.surface_temperature(out=)``):
    the allocator hands a block back only once its array is freed, so a
    caller that keeps its previous results page-locks fresh memory per call."""
    try:
        import torch

        if torch.cuda.is_available():
            tdt = {np.dtype(np.float32): torch.float32, np.dtype(np.float64): torch.float64,
                   np.dtype(np.int32): torch.int32}[np.dtype(dtype)]
            return torch.empty(shape, dtype=tdt, pin_memory=True).numpy()
    except (ImportError, KeyError, RuntimeError):
        pass
    return np.empty(shape, dtype)


def pinned_copy(a: np.ndarray) -> np.ndarray:
    """``a`` copied into a page-locked host array of the same shape and dtype."""
    out = host_buffer(a.shape, a.dtype)
    out[...] = a
    return out


_host_out = host_buffer


def _out_arg(a, shape, dtype, name) -> np.ndarray:
    if not isinstance(a, np.ndarray) or a.shape != shape or a.dtype != np.dtype(dtype) or not a.flags.c_contiguous \
            or not a.flags.writeable:
        raise ValueError(f"{name}: expected a writable C-contiguous {np.dtype(dtype).name} array of shape {shape}")
    return a


def _ck(rc: int):
    if rc != 0:
        lib = load()
        raise AtpmError(rc, lib.atpm_last_error().decode(errors="replace"))


def _p(a):
    return None if a is None else C.c_void_p(a.ctypes.data)


class Context:
    def __init__(self, device: int = 0):
        lib = load()
        h = C.c_void_p()
        _ck(lib.atpm_context_create(device, C.byref(h)))
        self.h = h

    def close(self):
        if self.h:
            load().atpm_context_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def make_params(problem, precision: int, revcap: int = 301, freeze: bool = True) -> Params:
    p = Params()
    p.ntau, p.nx = problem.ntau, problem.nx
    for i in range(3):
        p.polar[i] = problem.polar[i]
    p.pole[0], p.pole[1] = problem.pole
    p.rotation_period_s = problem.rotation_period_s
    p.albedo = problem.albedo
    p.emissivity = problem.emissivity
    p.tacc = problem.tacc
    p.scattering_accuracy = problem.scattering_accuracy
    p.shadowing = problem.shadowing
    p.multiple_scattering = problem.multiple_scattering
    p.revcap = revcap
    p.precision = precision
    p.freeze = 1 if freeze else 0
    return p


class Solve:
    """One resident solve (shape + state on the device)."""

    def __init__(self, ctx: Context, problem, precision: int = REFERENCE, revcap: int = 301, freeze: bool = True):
        lib = load()
        self.ctx, self.problem, self.precision, self.revcap = ctx, problem, precision, revcap
        self._keep = [np.ascontiguousarray(problem.vertices, np.float64),
                      np.ascontiguousarray(problem.facets, np.int32),
                      np.ascontiguousarray(problem.dep_ptr, np.int32),
                      np.ascontiguousarray(problem.dep_idx, np.int32),
                      np.ascontiguousarray(problem.dep_vf, np.float32)]
        v, f, dp, di, dv = self._keep
        sh = Shape(len(v), len(f), v.ctypes.data, f.ctypes.data, dp.ctypes.data,
                   di.ctypes.data if len(di) else None, dv.ctypes.data if len(dv) else None)
        self.shape = sh
        self.params = make_params(problem, precision, revcap, freeze)
        h = C.c_void_p()
        _ck(lib.atpm_solve_create(ctx.h, C.byref(sh), C.byref(self.params), C.byref(h)))
        self.h = h
        self.nf, self.ntau, self.nx = len(f), problem.ntau, problem.nx

    def clone(self) -> "Solve":
        """A new solve with this one's shape, parameters and device state
        (forcing, temperatures, tiles), copied on the device
        (atpm_solve_clone): a thermal-inertia sweep prepares the shape once."""
        h = C.c_void_p()
        _ck(load().atpm_solve_clone(self.h, C.byref(h)))
        c = Solve.__new__(Solve)
        c.__dict__.update({k: v for k, v in self.__dict__.items() if k != "h"})
        c.h = h
        return c

    def close(self):
        if getattr(self, "h", None):
            load().atpm_solve_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # stages -----------------------------------------------------------
    def geometry_shadow(self):
        _ck(load().atpm_geometry_shadow(self.h))

    def scattering(self):
        _ck(load().atpm_scattering(self.h))

    def set_forcing(self, shadow, illumination):
        s = np.ascontiguousarray(shadow, np.int32)
        e = np.ascontiguousarray(illumination, np.float32)
        _ck(load().atpm_set_forcing(self.h, _p(s), _p(e)))

    def set_thermal_inertia(self, ti: float):
        _ck(load().atpm_set_thermal_inertia(self.h, float(ti)))
        self._ti = float(ti)

    def initialise_temperatures(self):
        _ck(load().atpm_initialise_temperatures(self.h))

    def revolution(self, rev: int):
        n, c = C.c_int32(), C.c_int32()
        _ck(load().atpm_revolution(self.h, rev, C.byref(n), C.byref(c)))
        return n.value, c.value

    def run(self):
        nrev = np.zeros(1, np.int32)
        counts = np.zeros(self.revcap, np.int32)
        _ck(load().atpm_run(self.h, _p(nrev), _p(counts)))
        return counts[: nrev[0]].copy()

    def single_model(self, ti_list):
        ti = np.ascontiguousarray(np.atleast_1d(ti_list), np.float32)
        nrev = np.zeros(len(ti), np.int32)
        counts = np.zeros((len(ti), self.revcap), np.int32)
        _ck(load().atpm_single_model(self.h, _p(ti), len(ti), _p(nrev), _p(counts), None))
        return [counts[k, : nrev[k]].copy() for k in range(len(ti))]

    # getters ------------------------------------------------------------
    def shadow(self):
        out = _host_out((self.nf, self.ntau), np.int32)
        _ck(load().atpm_get_shadow(self.h, _p(out)))
        return out

    def illumination(self):
        out = _host_out((self.nf, self.ntau), np.float32)
        _ck(load().atpm_get_illumination(self.h, _p(out)))
        return out

    def cosillum(self):
        out = _host_out((self.nf, self.ntau), np.float32)
        _ck(load().atpm_get_cosillum(self.h, _p(out)))
        return out

    def selfheating_flux(self):
        """Q [ntau][nf] for the current temperatures."""
        out = _host_out((self.ntau, self.nf), np.float32)
        _ck(load().atpm_selfheating_flux(self.h, _p(out)))
        return out

    def surface_temperature(self, out=None):
        """(stemp1, stemp0) as [nf][ntau] FP32.  ``out``: an (stemp1, stemp0)
        pair of arrays to fill instead of new ones (see ``host_buffer``)."""
        shp = (self.nf, self.ntau)
        if out is None:
            s1, s0 = _host_out(shp, np.float32), _host_out(shp, np.float32)
        else:
            s1 = _out_arg(out[0], shp, np.float32, "out[0]")
            s0 = _out_arg(out[1], shp, np.float32, "out[1]")
        _ck(load().atpm_get_surface_temperature(self.h, _p(s1), _p(s0)))
        return s1, s0

    def result_temperature(self, out=None):
        """stemp1 alone as [nf][ntau] FP32: the surface temperature of every
        facet and step that the Thermal stage writes as its result
        (writeglobaltemperature, 3905/Thermal/NominalPole/main.cpp:2302-2306).
        ``out``: an array to fill instead of a new one."""
        shp = (self.nf, self.ntau)
        s1 = _host_out(shp, np.float32) if out is None else _out_arg(out, shp, np.float32, "out")
        _ck(load().atpm_get_surface_temperature(self.h, _p(s1), None))
        return s1

    def surface_temperature64(self):
        s1 = _host_out((self.nf, self.ntau), np.float64)
        _ck(load().atpm_get_surface_temperature64(self.h, _p(s1)))
        return s1

    def converged(self) -> np.ndarray:
        """Per-facet convergence flags after the last revolution (bool [nf])."""
        out = np.zeros(self.nf, np.uint8)
        _ck(load().atpm_get_converged(self.h, _p(out)))
        return out.astype(bool)

    def depth_temperature(self):
        t = np.zeros((self.nf, self.nx + 1), np.float32)
        _ck(load().atpm_get_depth_temperature(self.h, _p(t)))
        return t

    def set_binary_rotation(self, primary_vertices: int, primary_facets: int, primary_revs: int,
                            secondary_revs: int):
        """Non-synchronous binary: the first vertices/facets (the primary)
        turn primary_revs times per model period, the rest secondary_revs."""
        _ck(load().atpm_set_binary_rotation(self.h, int(primary_vertices), int(primary_facets), int(primary_revs),
                                            int(secondary_revs)))

    def set_ir_absorptivity(self, ir_abs: float):
        _ck(load().atpm_set_ir_absorptivity(self.h, float(ir_abs)))

    def set_position(self, car_km):
        """Place the body at a heliocentric centre (km) instead of its polar."""
        c = np.ascontiguousarray(car_km, np.float64)
        _ck(load().atpm_set_position(self.h, _p(c)))

    def disk_flux(self, observer, wavelengths_um=(12.0,), visibility=None, emissivity=0.9):
        """FP64 disk-integrated flux [ntau][nwl]; `observer` is the body's
        geocentric (AU, lat, lon) -- the solve's own polar means seen from the
        Sun; `visibility` [nf][ntau] flags or None for each facet's own
        horizon test."""
        ob = np.ascontiguousarray(observer, np.float64)
        wl = np.ascontiguousarray(wavelengths_um, np.float64)
        vis = None if visibility is None else np.ascontiguousarray(visibility, np.int32)
        out = np.zeros((self.ntau, len(wl)), np.float64)
        _ck(load().atpm_disk_flux(self.h, _p(ob), _p(vis), float(emissivity), len(wl), _p(wl), _p(out)))
        return out

    def disk_flux_rough(self, temperatures: "Crater", sub_visibility: "Crater", crater_vertices, crater_facets,
                        observer, wavelengths_um=(12.0,), visibility=None, emissivity=0.9):
        """[ntau][nwl] FP64 rough-surface flux (atpm_disk_flux_rough): the
        sub-facet temperatures of ``temperatures``, the visible fractions in
        ``sub_visibility``'s sub-facet shadow array."""
        cv = np.ascontiguousarray(crater_vertices, np.float32)
        cf = np.ascontiguousarray(crater_facets, np.int32)
        ob = np.ascontiguousarray(observer, np.float64)
        wl = np.ascontiguousarray(wavelengths_um, np.float64)
        vis = None if visibility is None else np.ascontiguousarray(visibility, np.int32)
        out = np.zeros((self.ntau, len(wl)), np.float64)
        _ck(load().atpm_disk_flux_rough(self.h, temperatures.h, sub_visibility.h, len(cv), _p(cv), _p(cf), _p(ob),
                                        _p(vis), float(emissivity), len(wl), _p(wl), _p(out)))
        return out

    def energy_balance(self):
        a, e, m = C.c_double(), C.c_double(), C.c_double()
        _ck(load().atpm_energy_balance(self.h, C.byref(a), C.byref(e), C.byref(m)))
        return a.value, e.value, m.value

    def last_run_config(self):
        """(conduction variant, tensor-core pipeline depth, tuned-this-run) of
        the last batch this solve led."""
        v, d, t = C.c_int32(), C.c_int32(), C.c_int32()
        _ck(load().atpm_last_run_config(self.h, C.byref(v), C.byref(d), C.byref(t)))
        return v.value, d.value, bool(t.value)

    def set_albedo(self, albedo: float):
        """Change the Bond albedo (scatter again before the next revolution)."""
        _ck(load().atpm_set_albedo(self.h, float(albedo)))

    def solar(self) -> float:
        """The solar flux at the body, W/m^2."""
        v = C.c_float()
        _ck(load().atpm_solve_solar(self.h, C.byref(v)))
        return float(v.value)

    def last_shadow_stats(self):
        """(device ms, rays, exact ray-triangle tests or -1) of the last
        geometry_shadow's shadow drivers."""
        ms, r, t = C.c_double(), C.c_int64(), C.c_int64()
        _ck(load().atpm_last_shadow_stats(self.h, C.byref(ms), C.byref(r), C.byref(t)))
        return ms.value, r.value, t.value

    def last_run_stats(self):
        ms, la, fs = C.c_double(), C.c_int64(), C.c_int64()
        _ck(load().atpm_last_run_stats(self.h, C.byref(ms), C.byref(la), C.byref(fs)))
        return ms.value, la.value, fs.value


def batch_run(solves):
    """Advance several solves together until each converges (atpm_batch_run)."""
    n = len(solves)
    arr = (C.c_void_p * n)(*[s.h.value for s in solves])
    cap = max(s.revcap for s in solves)
    nrev = np.zeros(n, np.int32)
    counts = np.zeros((n, cap), np.int32)
    _ck(load().atpm_batch_run(arr, n, _p(nrev), _p(counts)))
    return [counts[i, : nrev[i]].copy() for i in range(n)]


def result_temperatures(solves, outs=None):
    """The Thermal stage's result of several solves at once
    (atpm_get_surface_temperatures): each solve's [nf][ntau] FP32 surface
    temperatures, their copies to the host overlapping.  ``outs``: arrays to
    fill (page-locked ones from host_buffer copy fastest)."""
    n = len(solves)
    if outs is None:
        outs = [_host_out((s.nf, s.ntau), np.float32) for s in solves]
    else:
        outs = [_out_arg(o, (s.nf, s.ntau), np.float32, "out") for s, o in zip(solves, outs)]
    if len(outs) != n:
        raise ValueError("one output per solve")
    arr = (C.c_void_p * n)(*[s.h.value for s in solves])
    ptrs = (C.c_void_p * n)(*[o.ctypes.data for o in outs])
    _ck(load().atpm_get_surface_temperatures(arr, n, ptrs))
    return outs


def footprint(problem, precision: int, revcap: int = 301) -> int:
    v = np.ascontiguousarray(problem.vertices, np.float64)
    f = np.ascontiguousarray(problem.facets, np.int32)
    dp = np.ascontiguousarray(problem.dep_ptr, np.int32)
    di = np.ascontiguousarray(problem.dep_idx, np.int32)
    dv = np.ascontiguousarray(problem.dep_vf, np.float32)
    sh = Shape(len(v), len(f), v.ctypes.data, f.ctypes.data, dp.ctypes.data,
               di.ctypes.data if len(di) else None, dv.ctypes.data if len(dv) else None)
    p = make_params(problem, precision, revcap)
    out = C.c_uint64()
    _ck(load().atpm_solve_footprint(C.byref(sh), C.byref(p), C.byref(out)))
    return out.value


def viewfactors(ctx: Context, vertices, facets, refine: bool = True):
    """Shape_Selfheating on the GPU: returns (dep_ptr, dep_idx, dep_vf, dep_vec, photovectors)."""
    lib = load()
    v = np.ascontiguousarray(vertices, np.float32)
    f = np.ascontiguousarray(facets, np.int32)
    h = C.c_void_p()
    nnz = C.c_int64()
    _ck(lib.atpm_viewfactors_compute(ctx.h, len(v), len(f), _p(v), _p(f), 1 if refine else 0,
                                     C.byref(h), C.byref(nnz)))
    try:
        n = nnz.value
        ptr = np.zeros(len(f) + 1, np.int32)
        idx = np.zeros(n, np.int32)
        vf = np.zeros(n, np.float32)
        vec = np.zeros((n, 3), np.float32)
        photo = np.zeros((len(f), 3), np.float32)
        _ck(lib.atpm_viewfactors_get(h, _p(ptr), _p(idx), _p(vf), _p(vec), _p(photo)))
    finally:
        lib.atpm_viewfactors_free(h)
    return ptr, idx, vf, vec, photo


KERNEL_NAMES = ["selfheat_w", "selfheat_q", "conduction", "converge", "advance"]


def profile_revolution(solves):
    """Per-kernel device ms of one revolution of the batch (CUDA events).

    The convergence flags are reset first (same thermal inertia), so every
    facet is active, as in the early revolutions of a solve."""
    for s in solves:
        _ck(load().atpm_set_thermal_inertia(s.h, float(s._ti)))
    n = len(solves)
    arr = (C.c_void_p * n)(*[s.h.value for s in solves])
    ms = np.zeros(5, np.float64)
    fs, act = C.c_int64(), C.c_int64()
    _ck(load().atpm_profile_revolution(arr, n, _p(ms), C.byref(fs), C.byref(act)))
    out = {k: {"ms": float(v)} for k, v in zip(KERNEL_NAMES, ms)}
    out["conduction"].update(facet_steps=fs.value, active_facets=act.value)
    return out


class Server:
    """Continuous-batching solve server (atpm_server_*)."""

    def __init__(self, ctx: Context, precision: int = FAST, nx: int = 56, budget_bytes: int = 64 << 30,
                 max_active: int = 64, revs_per_tick: int = 2):
        h = C.c_void_p()
        _ck(load().atpm_server_create(ctx.h, precision, nx, budget_bytes, max_active, revs_per_tick, C.byref(h)))
        self.h, self.precision, self._shapes = h, precision, {}

    def add_shape(self, problem, revcap: int = 301, freeze: bool = True) -> int:
        v = np.ascontiguousarray(problem.vertices, np.float64)
        f = np.ascontiguousarray(problem.facets, np.int32)
        dp = np.ascontiguousarray(problem.dep_ptr, np.int32)
        di = np.ascontiguousarray(problem.dep_idx, np.int32)
        dv = np.ascontiguousarray(problem.dep_vf, np.float32)
        sh = Shape(len(v), len(f), v.ctypes.data, f.ctypes.data, dp.ctypes.data,
                   di.ctypes.data if len(di) else None, dv.ctypes.data if len(dv) else None)
        p = make_params(problem, self.precision, revcap, freeze)
        sid = C.c_int32()
        _ck(load().atpm_server_add_shape(self.h, C.byref(sh), C.byref(p), C.byref(sid)))
        self._shapes[sid.value] = (len(f), problem.ntau)
        return sid.value

    def submit(self, shape_id: int, ti: float) -> int:
        rid = C.c_int64()
        _ck(load().atpm_server_submit(self.h, shape_id, float(ti), C.byref(rid)))
        return rid.value

    def cancel(self, rid: int):
        _ck(load().atpm_server_cancel(self.h, rid))

    def wait(self, rid: int, shape_id: int, timeout_s: float = 600.0):
        nf, ntau = self._shapes[shape_id]
        out = np.empty((nf, ntau), np.float32)
        nrev, lat = C.c_int32(), C.c_double()
        _ck(load().atpm_server_wait(self.h, rid, timeout_s, _p(out), C.byref(nrev), C.byref(lat)))
        return out, nrev.value, lat.value

    def stats(self):
        p50, p99, fs = C.c_double(), C.c_double(), C.c_double()
        n, res = C.c_int64(), C.c_uint64()
        _ck(load().atpm_server_stats(self.h, C.byref(p50), C.byref(p99), C.byref(fs), C.byref(n), C.byref(res)))
        return {"p50_s": p50.value, "p99_s": p99.value, "facet_steps_per_s": fs.value, "completed": n.value,
                "resident_bytes": res.value}

    def close(self):
        if self.h:
            rc = load().atpm_server_destroy(self.h)
            self.h = None
            _ck(rc)

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Crater:
    """Per-facet crater (surface roughness) state on the GPU: the calls of the
    reference's roughness GPU module (3905/Thermal/NominalPole/GPU_code.cu:600-1026)
    with runtime sizes.  Sub-facet arrays are [facet][step][sub-facet]."""

    # set_array / get_array slots
    SHADOW, SFC_SHADOW, SUN_VECTOR, SFC_SUN_ANGLE, ILLUMINATION, GLOBAL_ILLUMINATION, GLOBAL_HEATING = range(7)

    def __init__(self, ctx: Context, nf: int, ntau: int, nx: int, nsf: int = 100, precision: int = REFERENCE):
        h = C.c_void_p()
        _ck(load().atpm_crater_create(ctx.h, nf, ntau, nx, nsf, precision, C.byref(h)))
        self.h, self.nf, self.ntau, self.nx, self.nsf = h, nf, ntau, nx, nsf

    def set_model(self, vertices, facets, trivectors, viewfactors, rotation_period_s: float):
        v = np.ascontiguousarray(vertices, np.float32)
        f = np.ascontiguousarray(facets, np.int32)
        t = np.ascontiguousarray(trivectors, np.float32)
        vf = np.ascontiguousarray(viewfactors, np.float32)
        _ck(load().atpm_crater_set_model(self.h, len(v), _p(v), _p(f), _p(t), _p(vf), float(rotation_period_s)))

    def set_surface(self, vertices, facets, viewfactors, rotation_period_s: float):
        """The crater model from its mesh (sub-point grid vectors and sub-facet
        normals derived on the host as the reference's surfacegeometry does);
        viewfactors: dense V[i][j] (``crater_viewfactors``)."""
        v = np.ascontiguousarray(vertices, np.float32)
        f = np.ascontiguousarray(facets, np.int32)
        vf = np.ascontiguousarray(viewfactors, np.float32)
        _ck(load().atpm_crater_set_surface(self.h, len(v), _p(v), _p(f), _p(vf), float(rotation_period_s)))

    def forcing(self, solve: "Solve", f0: int = 0, dep_vec=None):
        """Arrays 0-3 and 5 for facets f0 .. f0+nf-1 of ``solve``, computed on
        the device; dep_vec: the solve's list entries' direction vectors [nnz][3]."""
        d = None if dep_vec is None else np.ascontiguousarray(np.asarray(dep_vec, np.float32).reshape(-1, 3))
        _ck(load().atpm_crater_forcing(solve.h, self.h, int(f0), _p(d)))

    def global_heating(self, solve: "Solve", f0: int = 0):
        """Array 6 from the solve's current surface temperatures."""
        _ck(load().atpm_crater_global_heating(solve.h, self.h, int(f0)))

    def prepare_part(self, solve: "Solve", f0: int, c0: int, n: int, dep_vec=None):
        """Facets f0 .. f0+n-1 of ``solve`` into facets c0 .. c0+n-1 of this
        crater: their forcing and their global heating from the solve's current
        surface temperatures (parts of several solves then share the crater's
        launches)."""
        d = None if dep_vec is None else np.ascontiguousarray(np.asarray(dep_vec, np.float32).reshape(-1, 3))
        _ck(load().atpm_crater_prepare_part(solve.h, self.h, int(f0), int(c0), int(n), _p(d)))

    def set_properties(self, converged=None, albedo=None, thermal_inertia=None):
        c = None if converged is None else np.ascontiguousarray(converged, np.uint8)
        a = None if albedo is None else np.ascontiguousarray(albedo, np.float32)
        t = None if thermal_inertia is None else np.ascontiguousarray(thermal_inertia, np.float32)
        _ck(load().atpm_crater_set_properties(self.h, _p(c), _p(a), _p(t)))

    def converged(self) -> np.ndarray:
        out = np.zeros(self.nf, np.uint8)
        _ck(load().atpm_crater_get_properties(self.h, _p(out), None, None))
        return out

    def _shape(self, which: int):
        if which == self.SHADOW:
            return (self.nf, self.ntau), np.int32
        if which == self.SUN_VECTOR:
            return (self.nf, self.ntau, 3), np.float32
        return (self.nf, self.ntau, self.nsf), np.float32

    def set_array(self, which: int, data):
        shape, dt = self._shape(which)
        a = np.ascontiguousarray(np.asarray(data, dt).reshape(shape))
        _ck(load().atpm_crater_set_array(self.h, which, _p(a)))

    def get_array(self, which: int) -> np.ndarray:
        shape, dt = self._shape(which)
        out = np.zeros(shape, dt)
        _ck(load().atpm_crater_get_array(self.h, which, _p(out)))
        return out

    # strided-transfer slots of the temperature arrays ([nf][ntau][nsf], depth [nf][nx+1][nsf])
    STEMP0, STEMP1, DEPTH = 7, 8, 9

    def get_temperatures(self):
        """(stemp0, stemp1, depth): [nf][ntau][nsf] twice and [nf][nx+1][nsf]."""
        s0 = np.zeros((self.nf, self.ntau, self.nsf), np.float32)
        s1 = np.zeros((self.nf, self.ntau, self.nsf), np.float32)
        d = np.zeros((self.nf, self.nx + 1, self.nsf), np.float32)
        _ck(load().atpm_crater_get_temperatures(self.h, _p(s0), _p(s1), _p(d)))
        return s0, s1, d

    def set_temperatures(self, stemp1, stemp0=None):
        """Sub-facet surface temperatures [nf][ntau][nsf] (and the previous
        revolution's) into the crater's state."""
        for which, a in ((self.STEMP1, stemp1), (self.STEMP0, stemp0)):
            if a is None:
                continue
            a = np.ascontiguousarray(np.asarray(a, np.float32).reshape(self.nf, self.ntau, self.nsf))
            _ck(load().atpm_crater_set_array_strided(self.h, which, _p(a), self.ntau * self.nsf * 4))

    def partial_shadow(self):
        _ck(load().atpm_crater_partial_shadow(self.h))

    def scattering(self, solar: float, accuracy: float = 1e-4, multiple: bool = True):
        _ck(load().atpm_crater_scattering(self.h, solar, accuracy, 1 if multiple else 0))

    def zero_temperatures(self):
        _ck(load().atpm_crater_zero_temperatures(self.h))

    def initialise_temperatures(self, eps: float = 0.9, sigma: float = 5.67e-8):
        _ck(load().atpm_crater_initialise_temperatures(self.h, eps, sigma))

    def inertia_difference(self, eps: float = 0.9, sigma: float = 5.67e-8, tacc: float = 0.005):
        _ck(load().atpm_crater_inertia_difference(self.h, eps, sigma, tacc))

    def inst_equilibrium(self, eps: float = 0.9, sigma: float = 5.67e-8):
        _ck(load().atpm_crater_inst_equilibrium(self.h, eps, sigma))

    def update_converged(self, tacc: float = 0.005):
        _ck(load().atpm_crater_converged(self.h, tacc))

    def temperatures(self):
        s0 = np.zeros((self.nf, self.ntau, self.nsf), np.float32)
        s1 = np.zeros_like(s0)
        t = np.zeros((self.nf, self.nx + 1, self.nsf), np.float32)
        _ck(load().atpm_crater_get_temperatures(self.h, _p(s0), _p(s1), _p(t)))
        return s0, s1, t

    def close(self):
        if self.h:
            load().atpm_crater_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def orbital_position(a_au, e, inc_deg, node_deg, peri_deg, ta_deg):
    """Heliocentric body centre (km) at true anomaly ta_deg (degrees)."""
    out = np.zeros(3, np.float64)
    _ck(load().atpm_orbital_position(a_au, e, inc_deg, node_deg, peri_deg, ta_deg, _p(out)))
    return out


def _sweep(ctx, placements, thermal_inertia, precision, revcap):
    """Solves at (problem, position) placements, swept over thermal inertias
    with the reference's warm start, all advanced together per inertia."""
    solves = []
    for prob, car in placements:
        s = Solve(ctx, prob, precision=precision, revcap=revcap)
        s.set_position(car)
        s.geometry_shadow()
        s.scattering()
        solves.append(s)
    out = {}
    initialised = False
    for ti in thermal_inertia:
        for s in solves:
            s.set_thermal_inertia(ti)
        if ti != 0.0 and not initialised:
            for s in solves:
                s.initialise_temperatures()
            initialised = True
        counts = batch_run(solves)
        out[ti] = (np.stack([s.surface_temperature()[0] for s in solves]), counts)
    for s in solves:
        s.close()
    return out


def orbital_sweep(ctx, problem, elements, norb, thermal_inertia, precision=REFERENCE, revcap=301):
    """The reference's orbital_model (main.cpp:2612-2810) as one batch per
    thermal inertia: a solve per orbital point (true anomaly 360 i / norb),
    each with its own geometry, shadows and scattered sunlight, the thermal
    inertias swept in order with the reference's warm start, every orbital
    point advanced together in atpm_batch_run.  elements = (a_au, e, inc_deg,
    node_deg, peri_deg).  Returns {ti: (temperatures [norb][nf][ntau],
    convergence counts per point)}."""
    places = [(problem, orbital_position(*elements, 360.0 * i / norb)) for i in range(norb)]
    return _sweep(ctx, places, thermal_inertia, precision, revcap)


def obliquity_sweep(ctx, problem, elements, norb, nobl, thermal_inertia, js=range(1, 18), precision=REFERENCE,
                    revcap=301):
    """The reference's obliquity_model (main.cpp:2816-3003): pole latitude
    90 - j (90 / nobl) degrees (longitude 0) for each j, at every orbital
    point, at the one thermal inertia; every (j, point) solve in one batch.
    Returns (temperatures [len(js) * norb][nf][ntau] in (j, point) order,
    convergence counts in that order)."""
    import dataclasses
    import math

    places = []
    for j in js:
        obliquity = 90.0 - (j * (90.0 / nobl))
        pj = dataclasses.replace(problem, pole=(obliquity * (math.pi / 180.0), 0.0))
        for i in range(norb):
            places.append((pj, orbital_position(*elements, 360.0 * i / norb)))
    return _sweep(ctx, places, [thermal_inertia], precision, revcap)[thermal_inertia]
