"""Rough solves sharing one crater's launches (atpm_crater_prepare_part):
parts of three solves of one shape, with different thermal inertias and
albedos, go into one crater and advance in the same launches.  Each part's
crater forcing, temperatures and convergence flags must be bit-identical to
those of a crater holding that part alone, prepared through
atpm_crater_forcing and atpm_crater_global_heating."""
import sys
from pathlib import Path

import numpy as np
import pytest

from conftest import golden

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT / "tests" / "golden"))

pytestmark = pytest.mark.gpu
SIGMA = 5.67e-8
# (thermal inertia, albedo, first facet of the part) of the three solves
SOLVES = [(200.0, None, 0), (50.0, 0.1, 20), (400.0, 0.05, 100)]
PART = 40


def _solves(ctx, prob, prec):
    from binarytpm_gb300 import lib

    out = []
    for ti, alb, _ in SOLVES:
        s = lib.Solve(ctx, prob, precision=prec, revcap=20)
        s.geometry_shadow()
        if alb is not None:
            s.set_albedo(alb)
        s.scattering()
        s.set_thermal_inertia(ti)
        s.initialise_temperatures()
        s.run()
        out.append((s, ti, prob.albedo if alb is None else alb))
    return out


def _advance(c, prob, solar, revs=12):
    c.partial_shadow()
    c.scattering(solar, prob.scattering_accuracy, multiple=True)
    c.initialise_temperatures(prob.emissivity, SIGMA)
    for rev in range(revs):
        c.inertia_difference(prob.emissivity, SIGMA, prob.tacc)
        if rev > 5:
            c.update_converged(prob.tacc)


@pytest.mark.parametrize("precision", ["REFERENCE", "FAST"])
def test_parts_of_three_solves_in_one_crater_match_each_alone(gpu_ctx, precision):
    import make_golden
    from binarytpm_gb300 import formats, lib

    prob, ref = golden("rough_s1s1")
    assert prob.nf >= SOLVES[-1][2] + PART
    texts = make_golden.crater_texts_from(ref)
    cv, cf, V = formats.crater_model(texts["new_crater2.txt"], texts["new_crater2_selfheating_list.txt"])
    prec = getattr(lib, precision)
    solves = _solves(gpu_ctx, prob, prec)
    solar = solves[0][0].solar()

    # one crater, the three parts side by side
    mixed = lib.Crater(gpu_ctx, PART * len(SOLVES), prob.ntau, prob.nx, precision=prec)
    mixed.set_surface(cv, cf, V, prob.rotation_period_s)
    mixed.set_properties(np.zeros(PART * len(SOLVES), np.uint8),
                         np.repeat([a for _, _, a in solves], PART).astype(np.float32),
                         np.repeat([t for _, t, _ in solves], PART).astype(np.float32))
    for k, ((s, _, _), (_, _, f0)) in enumerate(zip(solves, SOLVES)):
        mixed.prepare_part(s, f0, k * PART, PART, ref["dep_vec"])
    _advance(mixed, prob, solar)
    m0, m1, mt = mixed.temperatures()
    mconv = mixed.converged()
    mforce = [mixed.get_array(w) for w in (mixed.SFC_SHADOW, mixed.SFC_SUN_ANGLE, mixed.ILLUMINATION)]

    for k, ((s, ti, alb), (_, _, f0)) in enumerate(zip(solves, SOLVES)):
        alone = lib.Crater(gpu_ctx, PART, prob.ntau, prob.nx, precision=prec)
        alone.set_surface(cv, cf, V, prob.rotation_period_s)
        alone.set_properties(np.zeros(PART, np.uint8), np.full(PART, alb, np.float32), np.full(PART, ti, np.float32))
        alone.forcing(s, f0, ref["dep_vec"])
        alone.global_heating(s, f0)
        _advance(alone, prob, solar)
        a0, a1, at = alone.temperatures()
        sl = slice(k * PART, (k + 1) * PART)
        for w, m in zip((alone.SFC_SHADOW, alone.SFC_SUN_ANGLE, alone.ILLUMINATION), mforce):
            assert np.array_equal(alone.get_array(w).view(np.uint32), m[sl].view(np.uint32))
        for a, m in ((a0, m0), (a1, m1), (at, mt)):
            assert np.array_equal(a.view(np.uint32), m[sl].view(np.uint32)), f"part {k} temperatures differ"
        assert np.array_equal(alone.converged(), mconv[sl])
        alone.close()
    mixed.close()
    for s, _, _ in solves:
        s.close()


def test_prepare_part_checks_ranges(gpu_ctx):
    import make_golden
    from binarytpm_gb300 import formats, lib

    prob, ref = golden("rough_s1s1")
    texts = make_golden.crater_texts_from(ref)
    cv, cf, V = formats.crater_model(texts["new_crater2.txt"], texts["new_crater2_selfheating_list.txt"])
    s = lib.Solve(gpu_ctx, prob, precision=lib.REFERENCE)
    s.geometry_shadow()
    s.scattering()
    c = lib.Crater(gpu_ctx, 2 * PART, prob.ntau, prob.nx, precision=lib.REFERENCE)
    c.set_surface(cv, cf, V, prob.rotation_period_s)
    with pytest.raises(lib.AtpmError):
        c.prepare_part(s, 0, PART + 1, PART, ref["dep_vec"])       # past the crater's last facet
    with pytest.raises(lib.AtpmError):
        c.prepare_part(s, prob.nf - PART + 1, 0, PART, ref["dep_vec"])  # past the solve's last facet
    c.prepare_part(s, 0, PART, PART, ref["dep_vec"])
    c.close()
    s.close()
