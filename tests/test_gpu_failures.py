"""Failure handling on the paths callers hit: bad inputs are refused with a
status (never a fault), a non-finite state stops the solve with
ATPM_E_NONFINITE, an iteration cap stops it with ATPM_E_ITERATION, a bounded
device wait gives up and reports instead of spinning, and after each of these
the context (and a server) keeps working.

Every failure is made on the host (a NaN written into an input, an
out-of-range index, a low Newton cap, a wait on a barrier that nothing
arrives at); no test faults, traps or hangs the GPU.
"""
import os
import time

import numpy as np
import pytest

from conftest import golden

pytestmark = pytest.mark.gpu

INVALID, NONFINITE, ITERATION = 1, 6, 7


def _ok_run(ctx, prob, lib):
    """A normal solve on the same context still runs to its end."""
    s = lib.Solve(ctx, prob, precision=lib.FAST, revcap=8)
    s.geometry_shadow()
    s.scattering()
    s.set_thermal_inertia(200.0)
    s.initialise_temperatures()
    counts = s.run()
    assert len(counts) == 8
    assert np.isfinite(s.surface_temperature()[0]).all()
    s.close()


def test_nan_thermal_inertia_is_refused(gpu_ctx):
    from binarytpm_gb300 import lib

    prob, _ = golden("binary_s3s1")
    s = lib.Solve(gpu_ctx, prob, precision=lib.FAST, revcap=8)
    s.geometry_shadow()
    s.scattering()
    for bad in (float("nan"), float("inf"), -1.0):
        with pytest.raises(lib.AtpmError) as ei:
            s.set_thermal_inertia(bad)
        assert ei.value.status == INVALID
    s.close()
    _ok_run(gpu_ctx, prob, lib)


def test_corrupt_mesh_is_refused(gpu_ctx):
    from binarytpm_gb300 import lib

    prob, _ = golden("binary_s3s1")
    f = prob.facets.copy()
    f[17, 1] = prob.nv + 5  # vertex index out of range
    with pytest.raises(lib.AtpmError) as ei:
        lib.Solve(gpu_ctx, prob.with_(facets=f), precision=lib.FAST)
    assert ei.value.status == INVALID
    idx = prob.dep_idx.copy()
    idx[3] = -2  # view-factor list entry out of range
    with pytest.raises(lib.AtpmError) as ei:
        lib.Solve(gpu_ctx, prob.with_(dep_idx=idx), precision=lib.FAST)
    assert ei.value.status == INVALID
    v = prob.vertices.copy()
    v[4, 2] = np.nan
    with pytest.raises(lib.AtpmError) as ei:
        lib.Solve(gpu_ctx, prob.with_(vertices=v), precision=lib.FAST)
    assert ei.value.status == NONFINITE
    _ok_run(gpu_ctx, prob, lib)


@pytest.mark.parametrize("precision", ["REFERENCE", "FAST"])
def test_nan_in_the_forcing_stops_the_solve(gpu_ctx, precision):
    """A NaN absorbed flux on one facet at one step makes that facet's
    temperature non-finite; the revolution loop stops and reports it."""
    from binarytpm_gb300 import lib

    prob, _ = golden("binary_s3s1")
    s = lib.Solve(gpu_ctx, prob, precision=getattr(lib, precision), revcap=12)
    s.geometry_shadow()
    s.scattering()
    shadow, illum = s.shadow(), s.illumination()
    illum = illum.copy()
    illum[100, 7] = np.nan
    s.set_forcing(shadow, illum)
    s.set_thermal_inertia(200.0)
    s.initialise_temperatures()
    with pytest.raises(lib.AtpmError) as ei:
        s.run()
    assert ei.value.status == NONFINITE
    s.close()
    _ok_run(gpu_ctx, prob, lib)


@pytest.mark.parametrize("precision", ["REFERENCE", "FP64", "FAST"])
def test_newton_cap_stops_the_solve(gpu_ctx, precision, monkeypatch):
    """With the Newton cap at 1 iteration the surface boundary condition
    cannot meet TACC/10 and the first revolution reports the cap; a solve
    made afterwards with the default cap runs normally."""
    from binarytpm_gb300 import lib

    prob, _ = golden("binary_s3s1")
    monkeypatch.setenv("ATPM_NEWTON_CAP", "1")
    s = lib.Solve(gpu_ctx, prob, precision=getattr(lib, precision), revcap=4)
    s.geometry_shadow()
    s.scattering()
    s.set_thermal_inertia(200.0)
    s.initialise_temperatures()
    t0 = time.perf_counter()
    with pytest.raises(lib.AtpmError) as ei:
        s.run()
    assert ei.value.status == ITERATION
    assert b"Newton" in lib.load().atpm_last_error()
    assert time.perf_counter() - t0 < 30.0
    s.close()
    monkeypatch.delenv("ATPM_NEWTON_CAP")
    _ok_run(gpu_ctx, prob, lib)


def test_bounded_wait_gives_up_and_reports(gpu_ctx):
    """A wait on an mbarrier nothing arrives at, with the tensor-core
    pipeline's bounded wait at a short limit (2e6 cycles, ~1 ms), returns
    ATPM_E_ITERATION with ST_TC_TIMEOUT; the context stays usable."""
    import ctypes as C

    from binarytpm_gb300 import lib

    L = lib.load()
    bits = C.c_int32(0)
    t0 = time.perf_counter()
    rc = L.atpm_selftest_bounded_wait(0, 2_000_000, C.byref(bits))
    assert rc == ITERATION, L.atpm_last_error()
    assert bits.value == 16
    assert time.perf_counter() - t0 < 10.0
    prob, _ = golden("binary_s3s1")
    _ok_run(gpu_ctx, prob, lib)


def test_server_refuses_bad_requests_and_keeps_serving(gpu_ctx):
    from binarytpm_gb300 import lib

    prob, _ = golden("binary_s3s1")
    srv = lib.Server(gpu_ctx, precision=lib.FAST, nx=8, max_active=4, revs_per_tick=3)
    sid = srv.add_shape(prob)
    f = prob.facets.copy()
    f[0, 0] = -1
    with pytest.raises(lib.AtpmError) as ei:
        srv.add_shape(prob.with_(facets=f))
    assert ei.value.status == INVALID
    for bad in (float("nan"), float("-inf")):
        with pytest.raises(lib.AtpmError) as ei:
            srv.submit(sid, bad)
        assert ei.value.status == INVALID
    with pytest.raises(lib.AtpmError) as ei:
        srv.submit(sid + 7, 200.0)
    assert ei.value.status == INVALID
    out, nrev, lat = srv.wait(srv.submit(sid, 200.0), sid)
    assert nrev > 0 and np.isfinite(out).all() and lat > 0
    srv.close()
