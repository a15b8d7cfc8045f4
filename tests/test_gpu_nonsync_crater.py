"""Crater (surface roughness) model of the non-synchronous binary program
(175706/Run-04/thermal.cpp) through its GPU module's 27 extern "C" functions
(175706/Run-04/thermal_GPU.cu:698-1279): flat [facet][step][sub-facet]
arrays, per-facet revolution counts (primary 3, secondary 1 per model period)
and IR absorptivity 0.9, the 160 facets in 5 parts of 32 whose per-part maps
the program stitches into one file.

Linked against binarytpm_gb300/driver/atpm_ref_nonsync_gpu_shim.cpp over
libatpm (REFERENCE precision) the program must write the same bytes as when
linked against the CPU restatement of the module (oracle/ref_gpu_cpu.cpp with
REF_NONSYNC_MODULE), whose outputs are the golden digests.  The reference's
own module, compiled from its source for sm_103a, pins that restatement to
float rounding (nvcc contracts multiply-adds and uses CUDA's powf).
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
SHIM = ROOT / "binarytpm_gb300" / "driver" / "atpm_ref_nonsync_gpu_shim.cpp"
ES = 0.9 * 5.67e-8


def _rough_temps(wd: Path, ti: float, nf: int, ntau: int) -> np.ndarray:
    raw = np.fromfile(wd / ("shape_roughness_temperature(%g).dat" % ti), dtype=np.float32)
    return raw[61 * 3 + 100 * 3:].reshape(nf, 100, ntau)


def _run(name, exe, wd: Path):
    import make_golden
    from oracle import refbuild

    _, ref = golden(name)
    wd.mkdir(exist_ok=True)
    make_golden.write_nonsync_inputs(wd, name, ref)
    refbuild.run(exe, wd)
    return ref


@pytest.mark.parametrize("name", ["nonsync_rough_s1s1", "nonsync_rough0_s1s1"])
def test_nonsync_crater_through_shim_bit_exact(gpu_ctx, tmp_path, name):
    import make_golden
    from binarytpm_gb300 import build
    from oracle import refbuild

    lib = build.build()
    exe = refbuild.build_nonsync_shim(make_golden.nonsync_cfg(name), lib.parent, ROOT / "include", SHIM)
    ref = _run(name, exe, tmp_path)
    for fname, want in zip(ref["files"], ref["sha256"]):
        got = hashlib.sha256((tmp_path / str(fname)).read_bytes()).hexdigest()
        assert got == str(want), f"{fname} differs from the oracle run"
    T = _rough_temps(tmp_path, make_golden.CASES[name]["ti"][0], 160, 72)
    want = ref["rough_stemp1_first_last"]
    assert np.array_equal(np.stack([T[0], T[-1]]).view(np.uint32), want.view(np.uint32))


def test_reference_nonsync_gpu_module_pins_the_crater_restatement(gpu_ctx, tmp_path):
    """The program's own GPU module against the CPU restatement on the same
    program (TI 200).  The global illumination the module hands back is the
    host's own array (bit-identical); sub-facet shadow fractions may move by
    one of the 10x10 sub-points at the crater rim; temperatures agree in
    emitted flux eps*sigma*T^4 to 0.1 W/m^2 in all but a handful of cells;
    each part converges within a revolution or two of the restatement."""
    import make_golden
    from oracle import refbuild

    name = "nonsync_rough_s1s1"
    cfg = make_golden.nonsync_cfg(name)
    wd_ref, wd_orc = tmp_path / "refgpu", tmp_path / "oracle"
    _run(name, refbuild.build_nonsync_refgpu(cfg), wd_ref)
    _run(name, refbuild.build_nonsync(cfg), wd_orc)
    nf, ntau = 160, 72
    F_ref = np.fromfile(wd_ref / "oracle_rough_forcing.bin", dtype=np.float32).reshape(3, nf, 100, ntau)
    F_orc = np.fromfile(wd_orc / "oracle_rough_forcing.bin", dtype=np.float32).reshape(3, nf, 100, ntau)
    ds = np.abs(F_ref[0] - F_orc[0])
    assert np.sum(ds > 0) <= 10 and ds.max() <= 0.0100001
    assert np.array_equal(F_ref[1], F_orc[1])
    assert np.array_equal(F_ref[2], F_orc[2])
    a = _rough_temps(wd_ref, 200.0, nf, ntau).astype(np.float64)
    b = _rough_temps(wd_orc, 200.0, nf, ntau).astype(np.float64)
    dF = np.abs(ES * a ** 4 - ES * b ** 4)
    assert np.sum(dF > 0.1) <= 10, np.sum(dF > 0.1)
    assert np.quantile(dF, 0.999) < 0.01
    ra = np.loadtxt(wd_ref / "oracle_rough_revs.txt", ndmin=2)
    rb = np.loadtxt(wd_orc / "oracle_rough_revs.txt", ndmin=2)
    for k in range(1, 6):
        na, nb = ra[ra[:, 0] == k], rb[rb[:, 0] == k]
        assert abs(len(na) - len(nb)) <= 2, (k, len(na), len(nb))
        assert na[-1, 2] == nb[-1, 2] == 32


def test_fast_nonsync_crater_within_tolerance(gpu_ctx, tmp_path):
    """ATPM_FAST crater kernels (contracted FP32) through the same shim: the
    forcing within float rounding of the restatement, temperatures within
    0.01 K wherever the emitted flux is above 1 W/m^2."""
    import make_golden
    from binarytpm_gb300 import build
    from oracle import refbuild

    name = "nonsync_rough_s1s1"
    cfg = make_golden.nonsync_cfg(name)
    lib = build.build()
    exe = refbuild.build_nonsync_shim(cfg, lib.parent, ROOT / "include", SHIM, precision="FAST")
    wd, wd_orc = tmp_path / "fast", tmp_path / "oracle"
    _run(name, exe, wd)
    _run(name, refbuild.build_nonsync(cfg), wd_orc)
    nf, ntau = 160, 72
    F = np.fromfile(wd / "oracle_rough_forcing.bin", dtype=np.float32).reshape(3, nf, 100, ntau)
    G = np.fromfile(wd_orc / "oracle_rough_forcing.bin", dtype=np.float32).reshape(3, nf, 100, ntau)
    assert np.sum(F[0] != G[0]) <= 10
    a = _rough_temps(wd, 200.0, nf, ntau).astype(np.float64)
    b = _rough_temps(wd_orc, 200.0, nf, ntau).astype(np.float64)
    lit = ES * b ** 4 > 1.0
    assert np.quantile(np.abs(a - b)[lit], 0.9999) < 0.01
