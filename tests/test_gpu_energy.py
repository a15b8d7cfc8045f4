"""FP64 energy balance of a revolution on the device (atpm_energy_balance)
against FP64 sums on the host of the same quantities: absorbed flux
(1 - A) E + Q and emitted flux eps sigma T^4 over every facet and step, and
the mean surface temperature.

The self-heating flux a revolution uses is computed from the previous
revolution's temperatures (3905/Thermal/NominalPole/main.cpp:1519-1529), so
the test reads it (atpm_selfheating_flux) right before the revolution whose
balance it checks.
"""
import numpy as np
import pytest

from conftest import golden

pytestmark = pytest.mark.gpu

SIGMA = np.float32(5.67e-8)


@pytest.mark.parametrize("precision,rtol", [("REFERENCE", 1e-9), ("FP64", 1e-7), ("FAST", 2e-6)])
def test_energy_balance_matches_host_sums(gpu_ctx, precision, rtol):
    from binarytpm_gb300 import lib

    prob, _ = golden("binary_s3s1")
    s = lib.Solve(gpu_ctx, prob, precision=getattr(lib, precision), revcap=20, freeze=False)
    s.geometry_shadow()
    s.scattering()
    s.set_thermal_inertia(200.0)
    s.initialise_temperatures()
    for rev in range(3):
        s.revolution(rev)
    q = s.selfheating_flux().astype(np.float64)
    s.revolution(3)
    ab, em, tm = s.energy_balance()
    E = s.illumination().astype(np.float64)
    T = s.surface_temperature64()
    oma = 1.0 - np.float64(np.float32(prob.albedo))
    es = np.float64(np.float32(prob.emissivity)) * np.float64(SIGMA)
    want_ab = oma * E.sum() + q.sum()
    want_em = es * ((T * T) * (T * T)).sum()
    assert abs(ab - want_ab) <= rtol * abs(want_ab), (ab, want_ab)
    assert abs(em - want_em) <= 1e-9 * abs(want_em), (em, want_em)
    assert abs(tm - T.mean()) <= 1e-9 * T.mean()
    s.close()


def test_energy_balance_closes_at_convergence(gpu_ctx):
    """Over a converged revolution the heat stored in the subsurface returns
    to where it started, so absorbed and emitted energy agree closely."""
    from binarytpm_gb300 import lib

    prob, _ = golden("binary_s3s1")
    s = lib.Solve(gpu_ctx, prob, precision=lib.FP64, revcap=200, freeze=False)
    s.geometry_shadow()
    s.scattering()
    s.set_thermal_inertia(200.0)
    s.initialise_temperatures()
    imb = []
    for rev in range(200):
        s.revolution(rev)
        if rev in (0, 199):
            ab, em, _ = s.energy_balance()
            imb.append(abs(ab - em) / ab)
    assert imb[1] < 1e-3 and imb[1] < imb[0], imb
    s.close()
