"""FAST late revolutions: once at most half a solve's facets are active, its
sweep runs over the list of active facets (thread per facet, whole warps of
active facets), and once the batch has at most 12 active facets per SM, one
warp per active facet (k_conduction_warp).  All forms share their arithmetic,
so temperatures, depth profiles and the per-revolution convergence counts are
identical with the list forms on (the default) and off (ATPM_WARP_TAIL=0: one
thread per facet over every facet block).  Each case is checked to have
reached the warp form: some revolution from the 7th on started with at most
12 active facets per SM over the batch's running solves.
"""
import dataclasses
import os

import numpy as np
import pytest

from conftest import golden

pytestmark = pytest.mark.gpu

TIS = [50.0, 200.0, 800.0]


def _run(ctx, prob, warp_tail: bool):
    from binarytpm_gb300 import lib

    old = os.environ.get("ATPM_WARP_TAIL")
    os.environ["ATPM_WARP_TAIL"] = "1" if warp_tail else "0"
    solves = []
    try:
        s0 = lib.Solve(ctx, prob, precision=lib.FAST)
        solves.append(s0)
        s0.geometry_shadow()
        s0.scattering()
        sh, il = s0.shadow(), s0.illumination()
        for _ in TIS[1:]:
            s = lib.Solve(ctx, prob, precision=lib.FAST)
            s.set_forcing(sh, il)
            solves.append(s)
        for s, ti in zip(solves, TIS):
            s.set_thermal_inertia(ti)
            s.initialise_temperatures()
        counts = lib.batch_run(solves)
        return [(s.surface_temperature(), s.depth_temperature(), s.converged(), c) for s, c in zip(solves, counts)]
    finally:
        for s in solves:
            s.close()
        if old is None:
            os.environ.pop("ATPM_WARP_TAIL", None)
        else:
            os.environ["ATPM_WARP_TAIL"] = old


@pytest.mark.parametrize("ntau,nx", [(48, 8), (720, 56)])
def test_warp_per_facet_tail_matches_thread_per_facet(gpu_ctx, ntau, nx):
    prob, _ = golden("binary_s3s1")
    prob = dataclasses.replace(prob, ntau=ntau, nx=nx)
    on = _run(gpu_ctx, prob, True)
    off = _run(gpu_ctx, prob, False)
    import torch

    lim = 12 * torch.cuda.get_device_properties(0).multi_processor_count
    for (t_on, d_on, c_on, n_on), (t_off, d_off, c_off, n_off) in zip(on, off):
        assert np.array_equal(n_on, n_off), "convergence counts differ"
        for a, b in zip(t_on, t_off):
            bad = np.flatnonzero(a.view(np.uint32) != b.view(np.uint32))
            assert bad.size == 0, f"{bad.size} surface temperatures differ, max {np.abs(a - b).max()} K"
        assert np.array_equal(d_on.view(np.uint32), d_off.view(np.uint32))
        assert np.array_equal(c_on, c_off)
    runs = [n for *_, n in on]
    last = max(len(n) for n in runs)
    active = [sum(prob.nf - int(n[r - 1]) for n in runs if len(n) > r) for r in range(7, last)]
    assert any(a <= lim for a in active), "no revolution ran in the warp-per-facet form"
