"""Parity at the benchmark's depth and step counts: NX = 56, NTAU = 720.

The golden case single_s3_nx56 is the reference Thermal program's own run of
the single-body configuration (icosphere subdivision 3, 1,280 facets,
P = 2.26 h, A = 0.02, TACC = 0.005 K): TI 0 (instantaneous equilibrium,
3905/Thermal/NominalPole/main.cpp:1563-1612) then TI 200 from fresh initial
temperatures to convergence (main.cpp:1473-1557, 2521-2539).  Its forcing,
surface temperatures of both revolution halves and depth profiles are stored
as SHA-256 digests of the raw floats, with every per-revolution convergence
count.  REFERENCE precision through the C ABI must reproduce every digest
and count; FP64 must match the FP64 oracle at the same NX and NTAU.
"""
import hashlib

import numpy as np
import pytest

from conftest import golden
from oracle import oracle

pytestmark = pytest.mark.gpu

NAME = "single_s3_nx56"


def _sha(a) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def _check_temps(s, ref, ti):
    s1, s0 = s.surface_temperature()
    if _sha(s1) != str(ref["sha256_stemp1_%g" % ti]):
        sample = s1.reshape(-1)[::97]
        want = ref["stemp1_sample_%g" % ti]
        bad = np.flatnonzero(sample.view(np.uint32) != want.view(np.uint32))
        pytest.fail(f"TI {ti}: surface temperatures differ (sampled: {bad.size} of {sample.size}, "
                    f"max {np.abs(sample - want).max()} K)")
    assert _sha(s0) == str(ref["sha256_stemp0_%g" % ti])
    assert _sha(s.depth_temperature()) == str(ref["sha256_temp_%g" % ti])


def test_reference_precision_bit_exact_nx56(gpu_ctx):
    from binarytpm_gb300 import lib

    prob, ref = golden(NAME)
    assert (prob.nf, prob.nx, prob.ntau) == (1280, 56, 720)
    # TI 0 alone: instantaneous equilibrium on the smooth shape
    s = lib.Solve(gpu_ctx, prob, precision=lib.REFERENCE)
    c0 = s.single_model([0.0])
    assert _sha(s.shadow().astype(np.int32)) == str(ref["sha256_shadow"])
    assert _sha(s.illumination()) == str(ref["sha256_illumination"])
    assert _sha(s.cosillum()) == str(ref["sha256_cosillum"])
    assert np.array_equal(c0[0], ref["counts_list"][0])
    _check_temps(s, ref, 0.0)
    s.close()
    # the reference's TI loop: 0 then 200 (fresh initial temperatures)
    s = lib.Solve(gpu_ctx, prob, precision=lib.REFERENCE)
    counts = s.single_model([0.0, 200.0])
    for got, want in zip(counts, ref["counts_list"]):
        assert np.array_equal(got, want)
    _check_temps(s, ref, 200.0)
    assert int(s.converged().sum()) == int(counts[-1][-1])
    s.close()


def test_fp64_matches_fp64_oracle_nx56(gpu_ctx):
    """Plain FP64 against the FP64 oracle for the first 12 revolutions at
    TI 200 (the convergence test runs from revolution 6 on, so the counts of
    revolutions 6-11 are compared too)."""
    from binarytpm_gb300 import lib

    prob, ref = golden(NAME)
    prob = prob.with_(thermal_inertia=[200.0])
    o = oracle.single_model(prob, precision=1, revcap=12)
    s = lib.Solve(gpu_ctx, prob, precision=lib.FP64, revcap=12)
    counts = s.single_model([200.0])
    t = s.surface_temperature64()
    assert np.max(np.abs(t - o["stemp1_64"])) < 1e-9
    for got, want in zip(counts, o["counts"]):
        assert np.array_equal(got, want)


def test_fast_within_tolerance_nx56(gpu_ctx):
    """FAST against plain FP64 on the same schedule (freeze off, 40
    revolutions at TI 200 and 2000) at NX = 56: within 0.01 K."""
    from binarytpm_gb300 import lib

    prob, _ = golden(NAME)
    s = lib.Solve(gpu_ctx, prob, precision=lib.FAST)
    s.geometry_shadow()
    s.scattering()
    shadow, illum = s.shadow(), s.illumination()
    s.close()
    for ti in (200.0, 2000.0):
        out = {}
        for prec in (lib.FAST, lib.FP64):
            x = lib.Solve(gpu_ctx, prob, precision=prec, revcap=40, freeze=False)
            x.set_forcing(shadow, illum)
            x.set_thermal_inertia(ti)
            x.initialise_temperatures()
            x.run()
            out[prec] = x.surface_temperature64()
            x.close()
        err = np.max(np.abs(out[lib.FAST] - out[lib.FP64]))
        assert err <= 0.01, (ti, err)
