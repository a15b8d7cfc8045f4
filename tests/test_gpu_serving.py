"""Continuous-batching server: admission by HBM budget, resident state,
results independent of the batch a request ran in."""
import time

import numpy as np
import pytest

from conftest import golden

pytestmark = pytest.mark.gpu

JOBS = [(0, 50.0), (1, 200.0), (0, 400.0), (1, 25.0), (1, 800.0), (0, 100.0), (1, 0.0)]


def _shapes():
    pa, _ = golden("single_s2")
    pb, _ = golden("binary_s3s1")
    return pa, pb


def test_results_identical_alone_and_in_mix(gpu_ctx):
    from binarytpm_gb300 import lib

    pa, pb = _shapes()
    alone = []
    for k, ti in JOBS:
        srv = lib.Server(gpu_ctx, precision=lib.FAST, nx=8)
        sids = [srv.add_shape(pa), srv.add_shape(pb)]
        out, nrev, _ = srv.wait(srv.submit(sids[k], ti), sids[k])
        alone.append((out, nrev))
        srv.close()
    # the mix: a budget that holds two solves at a time, requests arriving
    # while others are on the GPU
    fp = max(lib.footprint(pa, lib.FAST), lib.footprint(pb, lib.FAST))
    srv = lib.Server(gpu_ctx, precision=lib.FAST, nx=8, budget_bytes=int(2.5 * fp), max_active=4,
                     revs_per_tick=3)
    sids = [srv.add_shape(pa), srv.add_shape(pb)]
    rids = []
    for i, (k, ti) in enumerate(JOBS):
        rids.append(srv.submit(sids[k], ti))
        if i % 2:
            time.sleep(0.002)
    for (k, ti), rid, (want, want_rev) in zip(JOBS, rids, alone):
        got, nrev, lat = srv.wait(rid, sids[k])
        assert nrev == want_rev
        assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), (k, ti)
        assert lat > 0
    st = srv.stats()
    assert st["completed"] == len(JOBS)
    assert st["p99_s"] >= st["p50_s"] > 0
    assert st["resident_bytes"] == 0
    srv.close()


def test_request_larger_than_budget_is_rejected(gpu_ctx):
    from binarytpm_gb300 import lib

    pa, pb = _shapes()
    srv = lib.Server(gpu_ctx, precision=lib.FAST, nx=8, budget_bytes=lib.footprint(pa, lib.FAST) + 1)
    sa, sb = srv.add_shape(pa), srv.add_shape(pb)
    with pytest.raises(lib.AtpmError) as e:
        srv.submit(sb, 200.0)
    assert e.value.status == 8
    out, nrev, _ = srv.wait(srv.submit(sa, 200.0), sa)
    assert nrev > 6 and np.isfinite(out).all()
    srv.close()


def test_cancel_before_admission(gpu_ctx):
    from binarytpm_gb300 import lib

    pa, pb = _shapes()
    fp = lib.footprint(pb, lib.FAST)
    srv = lib.Server(gpu_ctx, precision=lib.FAST, nx=8, budget_bytes=int(1.5 * fp), max_active=1)
    sb = srv.add_shape(pb)
    r1 = srv.submit(sb, 2000.0)
    r2 = srv.submit(sb, 100.0)
    srv.cancel(r2)
    with pytest.raises(lib.AtpmError) as e:
        srv.wait(r2, sb)
    assert e.value.status == 9
    out, nrev, _ = srv.wait(r1, sb)
    assert np.isfinite(out).all()
    srv.close()
