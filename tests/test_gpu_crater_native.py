"""The crater (roughness) model run natively: its forcing computed on the
device from the solve (atpm_crater_forcing / atpm_crater_global_heating)
instead of by the reference Thermal driver on the host, then the crater
module's kernels, in the driver's order (3905/Thermal/NominalPole/
main.cpp:2417-2590: shadows and scattering once, then per thermal inertia
the global heating, the crater's starting temperatures, the shape's
revolutions, the global heating again and the crater's revolutions).

Against the golden case rough_s1s1, made by the reference driver itself with
its crater model on (through the CPU restatement of its GPU module): the
crater forcing it dumps (sub-facet shadows, Sun angles, scattered
illumination), its roughness temperature files at TI 0 and 200 and every
per-revolution roughness count must come out byte for byte.
"""
import hashlib
import sys
from pathlib import Path

import numpy as np
import pytest

from conftest import golden

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT / "tests" / "golden"))

pytestmark = pytest.mark.gpu
CASE = "rough_s1s1"
SIGMA = 5.67e-8


def _digest(ref, name):
    return str(ref["sha256"][list(map(str, ref["files"])).index(name)])


def _crater_loop(c, ti, eps, tacc, cap=301):
    """The driver's roughness revolution loop (main.cpp:2541-2566): counts of
    converged facets per revolution, tested from revolution 6 on."""
    counts = []
    rev, done = 0, False
    while not done and rev < cap:
        if ti == 0.0:
            c.inst_equilibrium(eps, SIGMA)
        else:
            c.inertia_difference(eps, SIGMA, tacc)
        n = 0
        if rev > 5:
            c.update_converged(tacc)
            n = int(c.converged().sum())
            done = n == c.nf
        counts.append(n)
        rev += 1
    return counts


def _temperature_file(cv, cf, stemp1):
    """binary_writesurfacetemperature (main.cpp:2314-2341): crater vertices,
    facets, then every facet's sub-facets' stemp1 over the steps."""
    return (np.asarray(cv, np.float32).tobytes() + np.asarray(cf, np.int32).tobytes()
            + np.ascontiguousarray(stemp1.transpose(0, 2, 1), np.float32).tobytes())


def test_native_crater_pipeline_matches_the_reference_driver(gpu_ctx):
    import make_golden
    from binarytpm_gb300 import formats, lib

    prob, ref = golden(CASE)
    texts = make_golden.crater_texts_from(ref)
    cv, cf, V = formats.crater_model(texts["new_crater2.txt"], texts["new_crater2_selfheating_list.txt"])
    nf, ntau, nsf = prob.nf, prob.ntau, 100
    eps, tacc = prob.emissivity, prob.tacc
    s = lib.Solve(gpu_ctx, prob, precision=lib.REFERENCE)
    s.geometry_shadow()
    s.scattering()
    c = lib.Crater(gpu_ctx, nf, ntau, prob.nx, precision=lib.REFERENCE)
    c.set_surface(cv, cf, V, prob.rotation_period_s)
    alb = np.full(nf, prob.albedo, np.float32)
    zero = np.zeros(nf, np.uint8)
    c.set_properties(zero, alb, np.zeros(nf, np.float32))
    c.forcing(s, 0, ref["dep_vec"])
    c.partial_shadow()
    c.scattering(s.solar(), prob.scattering_accuracy, multiple=True)
    blocks = [c.get_array(w).transpose(0, 2, 1) for w in (c.SFC_SHADOW, c.SFC_SUN_ANGLE, c.ILLUMINATION)]
    blob = b"".join(np.ascontiguousarray(b, np.float32).tobytes() for b in blocks)
    assert hashlib.sha256(blob).hexdigest() == _digest(ref, "oracle_rough_forcing.bin")

    counts, initialised = [], False
    for ti in prob.thermal_inertia:
        s.set_thermal_inertia(ti)
        c.set_properties(zero, alb, np.full(nf, ti, np.float32))
        if ti == 0.0:
            c.global_heating(s, 0)
            c.zero_temperatures()
        elif not initialised:
            s.initialise_temperatures()
            c.global_heating(s, 0)
            c.initialise_temperatures(eps, SIGMA)
            initialised = True
        s.run()
        c.global_heating(s, 0)
        counts += _crater_loop(c, ti, eps, tacc)
        stemp1 = c.get_temperatures()[1].reshape(nf, ntau, nsf)
        name = "shape_roughness_temperature(%g).dat" % ti
        got = hashlib.sha256(_temperature_file(cv, cf, stemp1)).hexdigest()
        assert got == _digest(ref, name), f"{name} differs"
    assert np.array_equal(np.array(counts, np.int32), ref["rough_counts"])


def test_global_heating_needs_the_forcing_of_the_same_part(gpu_ctx):
    """The global heating reuses the view factors of the last forcing call:
    another facet range, or no forcing at all, is refused."""
    import make_golden
    from binarytpm_gb300 import formats, lib

    prob, ref = golden(CASE)
    texts = make_golden.crater_texts_from(ref)
    cv, cf, V = formats.crater_model(texts["new_crater2.txt"], texts["new_crater2_selfheating_list.txt"])
    s = lib.Solve(gpu_ctx, prob, precision=lib.REFERENCE)
    s.geometry_shadow()
    s.scattering()
    c = lib.Crater(gpu_ctx, 40, prob.ntau, prob.nx, precision=lib.REFERENCE)
    c.set_surface(cv, cf, V, prob.rotation_period_s)
    with pytest.raises(lib.AtpmError):
        c.global_heating(s, 0)
    c.forcing(s, 40, ref["dep_vec"])
    with pytest.raises(lib.AtpmError):
        c.global_heating(s, 0)
    c.global_heating(s, 40)
    with pytest.raises(lib.AtpmError):
        c.forcing(s, prob.nf - 39, ref["dep_vec"])   # beyond the last facet
