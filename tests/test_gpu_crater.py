"""Crater (surface roughness) module through the reference's own Thermal driver.

With roughness on, the driver calls its GPU module through 27 extern "C"
functions (3905/Thermal/NominalPole/GPU_code.cu:600-1026).  Linked against
binarytpm_gb300/driver/atpm_ref_gpu_shim.cpp over libatpm (REFERENCE
precision) it must write the same bytes as when linked against the CPU
restatement of that module (oracle/ref_gpu_cpu.cpp), whose outputs are the
golden digests: crater shadows, Sun angles and scattered illumination of every
sub-facet, roughness temperature maps at TI 0 (instantaneous equilibrium) and
TI 200, per-revolution roughness convergence counts, and the shape's own files.

The reference's own GPU module, compiled from its source for sm_103a, runs on
the same driver as the pin of the CPU restatement: nvcc contracts
multiply-adds and uses CUDA's powf there, so it agrees to float rounding and
the convergence schedule it produces, not bit for bit.
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


def _inputs(wd: Path):
    import make_golden

    prob, ref = golden(CASE)
    make_golden.write_thermal_inputs(wd, prob.vertices, prob.facets, prob.dep_ptr, prob.dep_idx, prob.dep_vf,
                                     ref["dep_vec"], ref["photovectors"])
    make_golden.write_crater_files(wd, make_golden.crater_texts_from(ref))
    return prob, ref


def _rough_temps(wd: Path, ti: float, nf: int, ntau: int) -> np.ndarray:
    raw = np.fromfile(wd / ("shape_roughness_temperature(%g).dat" % ti), dtype=np.float32)
    return raw[61 * 3 + 100 * 3:].reshape(nf, 100, ntau)


def test_reference_driver_crater_through_shim_bit_exact(gpu_ctx, tmp_path):
    import make_golden
    from binarytpm_gb300 import build
    from oracle import refbuild

    lib = build.build()
    exe = refbuild.build_thermal_shim(make_golden.thermal_cfg(CASE), lib.parent, ROOT / "include",
                                      ROOT / "binarytpm_gb300" / "driver" / "atpm_ref_gpu_shim.cpp")
    prob, ref = _inputs(tmp_path)
    refbuild.run(exe, tmp_path)
    for name, want in zip(ref["files"], ref["sha256"]):
        got = hashlib.sha256((tmp_path / str(name)).read_bytes()).hexdigest()
        assert got == str(want), f"{name} differs from the oracle run"
    rr = np.loadtxt(tmp_path / "oracle_rough_revs.txt", ndmin=2)
    assert np.array_equal(rr[:, 2].astype(np.int32), ref["rough_counts"])
    sr = np.loadtxt(tmp_path / "oracle_revs.txt", ndmin=2)
    assert np.array_equal(sr[:, 2].astype(np.int32), ref["shape_counts"])
    T = _rough_temps(tmp_path, prob.thermal_inertia[-1], prob.nf, prob.ntau)
    assert np.array_equal(T[0].ravel().view(np.uint32), ref["rough_stemp1_head"].view(np.uint32))


def test_reference_gpu_module_pins_the_crater_restatement(gpu_ctx, tmp_path):
    """The reference's GPU module itself against its CPU restatement on the
    same driver.  nvcc contracts multiply-adds in the module: a sub-point at the
    crater rim can change sides (one sub-facet shadow fraction moves by 0.01 =
    one of the 10x10 sub-points), and where a sub-facet's absorbed flux is
    near zero its 4th root magnifies rounding (0 K against 2 K is 1e-6 W/m^2).
    So the comparison is made in emitted flux eps*sigma*T^4: all but a handful
    of the 768,000 cells per TI agree within 0.1 W/m^2, and the convergence
    schedule is the same to within a facet per revolution."""
    import make_golden
    from oracle import refbuild

    cfg = make_golden.thermal_cfg(CASE)
    exe = refbuild.build_thermal_refgpu(cfg)
    wd_ref, wd_orc = tmp_path / "refgpu", tmp_path / "oracle"
    wd_ref.mkdir()
    wd_orc.mkdir()
    prob, _ = _inputs(wd_ref)
    _inputs(wd_orc)
    refbuild.run(exe, wd_ref)
    refbuild.run(refbuild.build_thermal(cfg), wd_orc)
    nf, ntau = prob.nf, prob.ntau
    F_ref = np.fromfile(wd_ref / "oracle_rough_forcing.bin", dtype=np.float32).reshape(3, nf, 100, ntau)
    F_orc = np.fromfile(wd_orc / "oracle_rough_forcing.bin", dtype=np.float32).reshape(3, nf, 100, ntau)
    ds = np.abs(F_ref[0] - F_orc[0])
    assert np.sum(ds > 0) <= 10 and ds.max() <= 0.0100001              # sub-facet shadow fractions
    assert np.max(np.abs(F_ref[1] - F_orc[1])) < 1e-5                  # Sun angle cosines
    rel = np.abs(F_ref[2] - F_orc[2]) / np.maximum(1.0, np.abs(F_orc[2]))
    assert np.quantile(rel, 0.999) < 1e-4                              # scattered illumination
    es = 0.9 * 5.67e-8
    for ti in prob.thermal_inertia:
        a = _rough_temps(wd_ref, ti, nf, ntau).astype(np.float64)
        b = _rough_temps(wd_orc, ti, nf, ntau).astype(np.float64)
        dF = np.abs(es * a ** 4 - es * b ** 4)
        assert np.sum(dF > 0.1) <= 10, f"TI {ti}: {np.sum(dF > 0.1)} cells"
        assert np.quantile(dF, 0.999) < 0.01
    a = np.loadtxt(wd_ref / "oracle_rough_revs.txt", ndmin=2)
    b = np.loadtxt(wd_orc / "oracle_rough_revs.txt", ndmin=2)
    assert a.shape == b.shape
    assert np.max(np.abs(a[:, 2] - b[:, 2])) <= 2


def test_fast_crater_within_tolerance_of_reference(gpu_ctx, tmp_path):
    """ATPM_FAST crater kernels (contracted FP32) on the same driver: the forcing
    within float rounding of the REFERENCE run, temperatures within 0.01 K
    wherever the emitted flux is above 1 W/m^2 (the 4th root of a near-zero
    flux magnifies rounding, as for the reference's own GPU module)."""
    import make_golden
    from binarytpm_gb300 import build
    from oracle import refbuild

    lib = build.build()
    cfg = make_golden.thermal_cfg(CASE)
    shim = ROOT / "binarytpm_gb300" / "driver" / "atpm_ref_gpu_shim.cpp"
    exe = refbuild.build_thermal_shim(cfg, lib.parent, ROOT / "include", shim, precision="FAST")
    prob, ref = _inputs(tmp_path)
    refbuild.run(exe, tmp_path)
    nf, ntau = prob.nf, prob.ntau
    wd_orc = tmp_path / "oracle"
    wd_orc.mkdir()
    _inputs(wd_orc)
    refbuild.run(refbuild.build_thermal(cfg), wd_orc)
    F = np.fromfile(tmp_path / "oracle_rough_forcing.bin", dtype=np.float32).reshape(3, nf, 100, ntau)
    G = np.fromfile(wd_orc / "oracle_rough_forcing.bin", dtype=np.float32).reshape(3, nf, 100, ntau)
    assert np.sum(F[0] != G[0]) <= 10
    rel = np.abs(F[2] - G[2]) / np.maximum(1.0, np.abs(G[2]))
    assert np.quantile(rel, 0.999) < 1e-4
    es = 0.9 * 5.67e-8
    for ti in prob.thermal_inertia:
        a = _rough_temps(tmp_path, ti, nf, ntau).astype(np.float64)
        b = _rough_temps(wd_orc, ti, nf, ntau).astype(np.float64)
        lit = es * b ** 4 > 1.0
        assert np.quantile(np.abs(a - b)[lit], 0.9999) < 0.01, ti


VIS_CASE = "vis_rough_s1s1"


def _vis_inputs(wd: Path):
    import make_golden
    from binarytpm_gb300 import mesh

    prob, ref = golden(VIS_CASE)
    mesh.write_shape(wd / "shape.txt", prob.vertices, prob.facets)
    make_golden.write_crater_files(wd, make_golden.crater_texts_from(ref))
    return prob, ref


def test_reference_visibility_driver_crater_through_shim_bit_exact(gpu_ctx, tmp_path):
    """The Visibility driver's crater partial visibility through
    binarytpm_gb300/driver/atpm_ref_vis_gpu_shim.cpp: the same bytes as the
    CPU restatement of its GPU module, and the same shape flags."""
    import make_golden
    from binarytpm_gb300 import build, formats
    from oracle import refbuild

    lib = build.build()
    exe = refbuild.build_visibility_shim(make_golden.visibility_cfg(VIS_CASE), lib.parent, ROOT / "include",
                                         ROOT / "binarytpm_gb300" / "driver" / "atpm_ref_vis_gpu_shim.cpp")
    prob, ref = _vis_inputs(tmp_path)
    refbuild.run(exe, tmp_path)
    raw = (tmp_path / "shape_roughness_visibility.dat").read_bytes()
    assert hashlib.sha256(raw).hexdigest() == str(ref["sha256"][0])
    flags = formats.read_values_after_header(tmp_path / "shape_visibility.txt", prob.nv, prob.nf, np.int32)
    assert np.array_equal(flags.reshape(prob.nf, prob.ntau), ref["visibility"])


def test_reference_visibility_gpu_module_pins_the_restatement(gpu_ctx, tmp_path):
    """The Visibility driver's own GPU module (nvcc, sm_103a) against its CPU
    restatement: sub-facet visibilities equal except where a rim sub-point
    changes sides under multiply-add contraction (one sub-point = 0.01)."""
    import make_golden
    from oracle import refbuild

    cfg = make_golden.visibility_cfg(VIS_CASE)
    wd_ref, wd_orc = tmp_path / "refgpu", tmp_path / "oracle"
    wd_ref.mkdir()
    wd_orc.mkdir()
    prob, _ = _vis_inputs(wd_ref)
    _vis_inputs(wd_orc)
    refbuild.run(refbuild.build_visibility_refgpu(cfg), wd_ref)
    refbuild.run(refbuild.build_visibility(cfg), wd_orc)
    a = np.fromfile(wd_ref / "shape_roughness_visibility.dat", dtype=np.float32)[61 * 3 + 100 * 3:]
    b = np.fromfile(wd_orc / "shape_roughness_visibility.dat", dtype=np.float32)[61 * 3 + 100 * 3:]
    d = np.abs(a - b)
    assert d.max() <= 0.0100001
    assert np.sum(d > 0) <= 1e-4 * d.size
