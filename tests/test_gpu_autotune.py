"""The autotuner's knobs (conduction variant: register/occupancy variants 1-3
and the paired-facet sweep 4; tensor-core pipeline depth) change launch
configurations only: a FAST batch gives bit-identical temperatures and
convergence counts with the tuner on, off, and with each variant forced
(the run goes to convergence, so the active-list and warp-per-facet forms
and pairs with one frozen facet are exercised too); the first batch of a
kind times the candidates on its first five revolutions (whole revolutions of
both batch groups) and later batches of that kind reuse the choice."""
import os

import numpy as np
import pytest

from conftest import golden

pytestmark = pytest.mark.gpu


def _batch(ctx, prob, ref, env):
    from binarytpm_gb300 import lib

    old = {k: os.environ.get(k) for k in env}
    os.environ.update(env)
    try:
        solves = [lib.Solve(ctx, prob, precision=lib.FAST) for _ in range(3)]
        for s, ti in zip(solves, (50.0, 200.0, 800.0)):
            s.set_forcing(ref["shadow"], ref["illumination"])
            s.set_thermal_inertia(ti)
            s.initialise_temperatures()
        counts = lib.batch_run(solves)
        temps = [s.surface_temperature()[0] for s in solves]
        cfg = solves[0].last_run_config()
        for s in solves:
            s.close()
    finally:
        for k, v in old.items():
            if v is None:
                os.environ.pop(k, None)
            else:
                os.environ[k] = v
    return np.stack(temps), counts, cfg


def test_autotune_choices_do_not_change_results(gpu_ctx):
    from binarytpm_gb300 import lib

    prob, ref = golden("binary_s3s1")
    ctx = lib.Context(0)   # a fresh context: nothing tuned yet
    t0, c0, cfg0 = _batch(ctx, prob, ref, {"ATPM_AUTOTUNE": "1"})
    assert cfg0[2] and cfg0[0] in (1, 2, 3, 4)
    t1, c1, cfg1 = _batch(ctx, prob, ref, {"ATPM_AUTOTUNE": "1"})
    assert not cfg1[2] and cfg1[:2] == cfg0[:2]
    assert np.array_equal(t0.view(np.uint32), t1.view(np.uint32))
    assert all(np.array_equal(a, b) for a, b in zip(c1, c0))
    for v in ("1", "2", "3", "4"):
        t, cnt, cfg = _batch(ctx, prob, ref, {"ATPM_AUTOTUNE": "0", "ATPM_COND_VARIANT": v})
        assert cfg[0] == int(v) and not cfg[2]
        assert np.array_equal(t.view(np.uint32), t0.view(np.uint32))
        assert all(np.array_equal(a, b) for a, b in zip(cnt, c0))
    ctx.close()
