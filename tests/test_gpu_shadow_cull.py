"""The culled shadow drivers (projected-box test in front of the exact FP64
test; a per-step grid for all pairs) give the same flags as the plain
drivers, which the golden tests pin to the reference: dependent-list
shadowing toward the Sun (Thermal) and all-pairs occultation toward an
observer (Visibility), on a 6,400-facet binary with eclipses."""
import dataclasses
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _flags(ctx, prob, cull: bool):
    from binarytpm_gb300 import lib

    os.environ["ATPM_SHADOW_CULL"] = "1" if cull else "0"
    try:
        s = lib.Solve(ctx, prob, precision=lib.REFERENCE)
        s.geometry_shadow()
        out = s.shadow()
        s.close()
    finally:
        os.environ.pop("ATPM_SHADOW_CULL", None)
    return out


@pytest.mark.parametrize("shadowing,polar", [(1, (1.0, 0.0, 0.0)), (2, (1.2, 0.1, 0.3)), (2, (0.02, -0.3, 1.0))])
def test_culled_shadows_equal_plain(gpu_ctx, shadowing, polar):
    from binarytpm_gb300 import workloads

    prob = workloads.binary_problem(gpu_ctx, p_subdiv=4, ntau=96)
    prob = dataclasses.replace(prob, shadowing=shadowing, polar=polar)
    a = _flags(gpu_ctx, prob, True)
    b = _flags(gpu_ctx, prob, False)
    assert np.array_equal(a, b)
    # the case exercises occlusion beyond each facet's own horizon
    horizon_only = dataclasses.replace(prob, shadowing=0)
    c = _flags(gpu_ctx, horizon_only, True)
    assert (c - a).sum() > 0


def test_shadow_stats_count_the_exact_tests(gpu_ctx):
    """atpm_last_shadow_stats: the rays are every facet x step; the culled
    drivers run far fewer exact tests than the pairs an all-pairs sweep would
    test, at least one per ray they turn dark; the plain drivers report -1."""
    from binarytpm_gb300 import lib, workloads

    prob = workloads.binary_problem(gpu_ctx, p_subdiv=4, ntau=96)
    prob = dataclasses.replace(prob, shadowing=2, polar=(1.2, 0.1, 0.3))
    s = lib.Solve(gpu_ctx, prob, precision=lib.REFERENCE)
    s.geometry_shadow()
    ms, rays, tests = s.last_shadow_stats()
    dark_by_others = int(((s.shadow() == 0) & (_flags(gpu_ctx, dataclasses.replace(prob, shadowing=0), True) == 1)).sum())
    assert rays == prob.nf * prob.ntau and ms > 0
    assert dark_by_others <= tests < rays * prob.nf // 100
    s.close()
    os.environ["ATPM_SHADOW_CULL"] = "0"
    try:
        s = lib.Solve(gpu_ctx, prob, precision=lib.REFERENCE)
        s.geometry_shadow()
        assert s.last_shadow_stats()[2] == -1
        s.close()
    finally:
        os.environ.pop("ATPM_SHADOW_CULL", None)
