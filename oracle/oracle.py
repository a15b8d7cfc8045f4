"""ctypes front end of the CPU oracle (oracle/atpm_oracle.cpp).

TEST INFRASTRUCTURE ONLY: tests, ``__graft_entry__.smoke`` and ``bench.py``'s
CPU-baseline leg use it as the checker.  It restates the reference Thermal /
Visibility smooth-shape path (citations in atpm_oracle.cpp).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "_build" / "liboracle.so"
SRC = HERE / "atpm_oracle.cpp"


class OracleParams(C.Structure):
    _fields_ = [
        ("nv", C.c_int), ("nf", C.c_int), ("ntau", C.c_int), ("nx", C.c_int),
        ("vertices", C.c_void_p), ("facets", C.c_void_p),
        ("dep_ptr", C.c_void_p), ("dep_idx", C.c_void_p), ("dep_vf", C.c_void_p),
        ("polar0", C.c_double), ("polar1", C.c_double), ("polar2", C.c_double),
        ("rot0", C.c_double), ("rot1", C.c_double),
        ("tacc", C.c_float), ("scattering_accuracy", C.c_float), ("eps", C.c_float),
        ("rotation_period", C.c_float), ("albedo", C.c_float),
        ("shadowing", C.c_int), ("multiple_scattering", C.c_int), ("precision", C.c_int),
        ("revcap", C.c_int), ("nti", C.c_int), ("ti", C.c_void_p), ("nthreads", C.c_int),
    ]


class OracleOutputs(C.Structure):
    _fields_ = [
        ("shadow", C.c_void_p), ("illumination", C.c_void_p), ("cosillum", C.c_void_p),
        ("illumination64", C.c_void_p),
        ("stemp1", C.c_void_p), ("stemp0", C.c_void_p), ("temp", C.c_void_p),
        ("stemp1_64", C.c_void_p),
        ("numconverged", C.c_void_p), ("nrev", C.c_void_p),
    ]


def build() -> Path:
    LIB.parent.mkdir(exist_ok=True)
    if not LIB.exists() or LIB.stat().st_mtime < SRC.stat().st_mtime:
        subprocess.run(["g++", "-O3", "-fopenmp", "-ffp-contract=off", "-std=c++14",
                        "-shared", "-fPIC", str(SRC), "-o", str(LIB)], check=True)
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        _lib = C.CDLL(str(build()))
        _lib.oracle_single_model.argtypes = [C.POINTER(OracleParams), C.POINTER(OracleOutputs)]
        _lib.oracle_shadows.argtypes = [C.POINTER(OracleParams), C.c_void_p, C.c_void_p]
        _lib.oracle_powf_range.argtypes = [C.c_void_p, C.c_float, C.c_void_p, C.c_int64]
    return _lib


def _ptr(a):
    return None if a is None else a.ctypes.data


def make_params(problem, keep, precision=0, nthreads=None, revcap=301):
    """``problem`` is a ``binarytpm_gb300.problem.Problem``; arrays are kept alive in ``keep``."""
    v = np.ascontiguousarray(problem.vertices, np.float64)
    f = np.ascontiguousarray(problem.facets, np.int32)
    dp = np.ascontiguousarray(problem.dep_ptr, np.int32)
    di = np.ascontiguousarray(problem.dep_idx, np.int32)
    dv = np.ascontiguousarray(problem.dep_vf, np.float32)
    ti = np.ascontiguousarray(np.atleast_1d(problem.thermal_inertia), np.float32)
    keep += [v, f, dp, di, dv, ti]
    p = OracleParams()
    p.nv, p.nf, p.ntau, p.nx = len(v), len(f), problem.ntau, problem.nx
    p.vertices, p.facets = _ptr(v), _ptr(f)
    p.dep_ptr, p.dep_idx, p.dep_vf = _ptr(dp), _ptr(di), _ptr(dv)
    p.polar0, p.polar1, p.polar2 = problem.polar
    p.rot0, p.rot1 = problem.pole
    p.tacc = problem.tacc
    p.scattering_accuracy = problem.scattering_accuracy
    p.eps = problem.emissivity
    p.rotation_period = problem.rotation_period_s
    p.albedo = problem.albedo
    p.shadowing = problem.shadowing
    p.multiple_scattering = problem.multiple_scattering
    p.precision = precision
    p.revcap = revcap
    p.nti = len(ti)
    p.ti = _ptr(ti)
    p.nthreads = nthreads or os.cpu_count() or 1
    return p


def single_model(problem, precision=0, nthreads=None, revcap=301):
    """Run the reference single_model flow; returns a dict of numpy arrays."""
    keep = []
    p = make_params(problem, keep, precision, nthreads, revcap)
    nf, ntau, nx, nti = p.nf, p.ntau, p.nx, p.nti
    out = dict(
        shadow=np.zeros((nf, ntau), np.int32),
        illumination=np.zeros((nf, ntau), np.float32),
        cosillum=np.zeros((nf, ntau), np.float32),
        stemp1=np.zeros((nf, ntau), np.float32),
        stemp0=np.zeros((nf, ntau), np.float32),
        temp=np.zeros((nf, nx + 1), np.float32),
        numconverged=np.full((nti, revcap), -1, np.int32),
        nrev=np.zeros(nti, np.int32),
    )
    if precision == 1:
        out["illumination64"] = np.zeros((nf, ntau), np.float64)
        out["stemp1_64"] = np.zeros((nf, ntau), np.float64)
    o = OracleOutputs()
    for k in ("shadow", "illumination", "cosillum", "stemp1", "stemp0", "temp",
              "numconverged", "nrev", "illumination64", "stemp1_64"):
        setattr(o, k, _ptr(out.get(k)))
    lib().oracle_single_model(C.byref(p), C.byref(o))
    out["counts"] = [out["numconverged"][k, : out["nrev"][k]].copy() for k in range(nti)]
    return out


def shadows(problem, nthreads=None):
    keep = []
    p = make_params(problem, keep, 0, nthreads)
    sh = np.zeros((p.nf, p.ntau), np.int32)
    cs = np.zeros((p.nf, p.ntau), np.float32)
    lib().oracle_shadows(C.byref(p), _ptr(sh), _ptr(cs))
    return sh, cs


def glibc_powf(x: np.ndarray, e: float) -> np.ndarray:
    x = np.ascontiguousarray(x, np.float32)
    out = np.empty_like(x)
    lib().oracle_powf_range(_ptr(x), e, _ptr(out), len(x))
    return out
