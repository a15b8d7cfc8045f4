"""The disk-integrated flux restatement (oracle/flux.py) against the
reference's own Observe stage (3905/Observe/NominalPole/wise_main.cpp,
compiled from a scratch copy by oracle/refbuild.py, its raw per-step smooth
flux dumped before the colour-correction fit).  Both read the same stage
files: the shape and visibility flags (Visibility format), the surface
temperatures of the golden reference run (Thermal format, 6 significant
digits), so the bar is FP64 summation order: 1e-12 of the step's flux."""
import numpy as np
import pytest

from conftest import golden

WL = (4.6028, 11.0984, 22.6405)


@pytest.mark.parametrize("observer", [(0.9, 0.1, 0.3), "sun"])
def test_flux_restatement_matches_reference_observe(tmp_path, observer):
    from binarytpm_gb300 import formats
    from oracle import flux, refbuild

    prob, ref = golden("single_s2")
    nv, nf, ntau = prob.nv, prob.nf, prob.ntau
    obs = prob.polar if observer == "sun" else observer
    ti = 200
    v, f = prob.vertices, prob.facets
    formats.write_shadow(tmp_path / "shape_visibility.txt", v, f, np.ones((nf, ntau), np.int32))
    formats.write_temperature(tmp_path / ("shape_temperature(%d).txt" % ti), v, f, ref["stemp1"])
    blank = np.zeros(61 * 3 + 100 * 3 + nf * 100 * ntau, np.float32).tobytes()
    (tmp_path / "shape_roughness_visibility.dat").write_bytes(blank)
    (tmp_path / ("shape_roughness_temperature(%d).dat" % ti)).write_bytes(blank)
    (tmp_path / "wise_colour_corrections.txt").write_text("1\t1\t1\n" * 467)
    exe = refbuild.build_observe(dict(nv=nv, nf=nf, ntau=ntau, polar=prob.polar, observer=obs, rot=prob.pole, ti=ti))
    refbuild.run(exe, tmp_path)
    got = np.fromfile(tmp_path / "oracle_flux.bin", dtype=np.float64).reshape(ntau, 3)
    # the stage's inputs as it parsed them: 6-digit text vertices and temperatures
    raw = (tmp_path / "shape_visibility.txt").read_text().split()
    vv = np.array(raw[:3 * nv], dtype=np.float64).reshape(nv, 3)
    T = formats.read_values_after_header(tmp_path / ("shape_temperature(%d).txt" % ti), nv, nf, np.float64)
    want = flux.disk_flux(vv, f, ntau, prob.pole, prob.polar, obs, 0.9, T.reshape(nf, ntau).T, None, WL)
    scale = np.abs(want).max(axis=0, keepdims=True)
    assert np.all(scale > 0)
    assert np.all(np.abs(got - want) <= 1e-12 * scale), np.max(np.abs(got - want) / scale)


def _crater_model():
    """The crater (roughness) model the reference ships, carried in the crater
    golden fixture: vertices [61][3], facets [100][3]."""
    import sys
    from pathlib import Path

    sys.path.insert(0, str(Path(__file__).resolve().parent / "golden"))
    import make_golden

    _, ref = golden("rough_s1s1")
    tok = make_golden.crater_texts_from(ref)["new_crater2.txt"].split()
    cv = np.array(tok[:183], dtype=np.float64).reshape(61, 3)
    cf = np.array(tok[183:483], dtype=np.int32).reshape(100, 3)
    return cv, cf


def _rough_file(path, cv, cf, per_facet):
    """The stage's binary crater file: float crater vertices, int facets, then
    [nf][nsf][ntau] floats (binary_writesfcroughshadow layout)."""
    with open(path, "wb") as fh:
        fh.write(np.asarray(cv, np.float32).tobytes())
        fh.write(np.asarray(cf, np.int32).tobytes())
        fh.write(np.ascontiguousarray(per_facet, np.float32).tobytes())


def test_rough_flux_restatement_matches_reference_observe(tmp_path):
    """The rough-surface sum of the Observe stage (observe,
    3905/Observe/NominalPole/wise_main.cpp:695-727): seeded sub-facet
    temperatures and visible fractions (some zero) in the stage's files."""
    from binarytpm_gb300 import formats
    from oracle import flux, refbuild

    prob, ref = golden("single_s2")
    nv, nf, ntau = prob.nv, prob.nf, prob.ntau
    obs = (0.9, 0.1, 0.3)
    ti = 200
    v, f = prob.vertices, prob.facets
    cv, cf = _crater_model()
    rng = np.random.default_rng(7)
    sub_t = rng.uniform(80.0, 400.0, (nf, 100, ntau)).astype(np.float32)
    sub_v = np.where(rng.random((nf, 100, ntau)) < 0.3, 0.0, rng.integers(1, 101, (nf, 100, ntau)) / 100.0)
    sub_v = sub_v.astype(np.float32)
    flags = (rng.random((nf, ntau)) < 0.9).astype(np.int32)
    formats.write_shadow(tmp_path / "shape_visibility.txt", v, f, flags)
    formats.write_temperature(tmp_path / ("shape_temperature(%d).txt" % ti), v, f, ref["stemp1"])
    _rough_file(tmp_path / "shape_roughness_visibility.dat", cv, cf, sub_v)
    _rough_file(tmp_path / ("shape_roughness_temperature(%d).dat" % ti), cv, cf, sub_t)
    (tmp_path / "wise_colour_corrections.txt").write_text("1\t1\t1\n" * 467)
    exe = refbuild.build_observe(dict(nv=nv, nf=nf, ntau=ntau, polar=prob.polar, observer=obs, rot=prob.pole, ti=ti))
    refbuild.run(exe, tmp_path)
    got = np.fromfile(tmp_path / "oracle_rough_flux.bin", dtype=np.float64).reshape(ntau, 3)
    raw = (tmp_path / "shape_visibility.txt").read_text().split()
    vv = np.array(raw[:3 * nv], dtype=np.float64).reshape(nv, 3)
    want = flux.rough_disk_flux(vv, f, ntau, prob.pole, prob.polar, obs, 0.9, sub_t, sub_v, cv, cf, flags, WL)
    scale = np.abs(want).max(axis=0, keepdims=True)
    assert np.all(scale > 0)
    assert np.all(np.abs(got - want) <= 1e-12 * scale), np.max(np.abs(got - want) / scale)
