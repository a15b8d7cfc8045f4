"""FP64 disk-integrated flux on the device (atpm_disk_flux) against the numpy
restatement of the Observe stage's observe (oracle/flux.py), on the golden
shapes' own temperatures: from the Sun with the illumination flags as the
visibility, and from an off-phase observer with each facet's horizon test.
Facet sums run in a different order on the two sides, so the bar is 1e-12
relative to the step's flux."""
import numpy as np
import pytest

from conftest import golden

pytestmark = pytest.mark.gpu

WL = (4.6028, 11.0984, 22.6405)   # the Observe stage's three wavelengths (wise_main.cpp:40)


@pytest.mark.parametrize("name,precision", [("single_s2", 0), ("binary_s3s1", 0), ("binary_s3s1", 1),
                                            ("binary_s3s1", 2)])
def test_disk_flux_matches_restatement(gpu_ctx, name, precision):
    from binarytpm_gb300 import lib
    from oracle import flux

    prob, _ = golden(name)
    s = lib.Solve(gpu_ctx, prob, precision=precision)
    s.single_model(prob.thermal_inertia)
    T = s.surface_temperature64() if precision == 1 else s.surface_temperature()[0].astype(np.float64)
    for observer, vis in [(prob.polar, s.shadow()), ((0.9, 0.1, 0.3), None)]:
        got = s.disk_flux(observer, WL, vis)
        want = flux.disk_flux(prob.vertices, prob.facets, prob.ntau, prob.pole, prob.polar, observer,
                              prob.emissivity, T.T, vis, WL)
        assert got.shape == want.shape
        scale = np.maximum(np.abs(want).max(axis=0, keepdims=True), 1e-300)
        assert np.all(np.abs(got - want) <= 1e-12 * scale), np.max(np.abs(got - want) / scale)
        assert np.all(want.sum(axis=0) > 0)
    s.close()


def test_disk_flux_deterministic(gpu_ctx):
    from binarytpm_gb300 import lib

    prob, _ = golden("binary_s3s1")
    s = lib.Solve(gpu_ctx, prob, precision=2)
    s.single_model(prob.thermal_inertia)
    a = s.disk_flux((0.9, 0.1, 0.3), WL)
    b = s.disk_flux((0.9, 0.1, 0.3), WL)
    assert np.array_equal(a, b)
    s.close()


def test_rough_disk_flux_matches_restatement(gpu_ctx):
    """The rough-surface sum (atpm_disk_flux_rough) against its restatement
    (oracle.flux.rough_disk_flux, pinned to the reference's Observe stage
    by tests/test_oracle_flux.py): seeded sub-facet temperatures and visible
    fractions in two crater handles, the shipped crater model."""
    import sys
    from pathlib import Path

    from binarytpm_gb300 import lib
    from oracle import flux

    sys.path.insert(0, str(Path(__file__).resolve().parent))
    from test_oracle_flux import _crater_model

    prob, _ = golden("single_s2")
    nf, ntau = prob.nf, prob.ntau
    cv, cf = _crater_model()
    rng = np.random.default_rng(11)
    sub_t = rng.uniform(80.0, 400.0, (nf, ntau, 100)).astype(np.float32)
    sub_v = np.where(rng.random((nf, ntau, 100)) < 0.3, 0.0, rng.integers(1, 101, (nf, ntau, 100)) / 100.0)
    sub_v = sub_v.astype(np.float32)
    s = lib.Solve(gpu_ctx, prob, precision=lib.REFERENCE)
    s.geometry_shadow()
    ct = lib.Crater(gpu_ctx, nf, ntau, 8, 100, lib.REFERENCE)
    ct.set_temperatures(sub_t)
    cvis = lib.Crater(gpu_ctx, nf, ntau, 0, 100, lib.REFERENCE)
    cvis.set_array(lib.Crater.SFC_SHADOW, sub_v)
    obs = (0.9, 0.1, 0.3)
    flags = (rng.random((nf, ntau)) < 0.9).astype(np.int32)
    for vis in (None, flags):
        got = s.disk_flux_rough(ct, cvis, cv, cf, obs, WL, vis)
        want = flux.rough_disk_flux(prob.vertices, prob.facets, ntau, prob.pole, prob.polar, obs, prob.emissivity,
                                    sub_t.transpose(0, 2, 1), sub_v.transpose(0, 2, 1), cv, cf, vis, WL)
        scale = np.abs(want).max(axis=0, keepdims=True)
        assert np.all(scale > 0)
        assert np.all(np.abs(got - want) <= 1e-11 * scale), np.max(np.abs(got - want) / scale)
    ct.close()
    cvis.close()
    s.close()
