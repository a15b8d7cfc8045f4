"""The reference Thermal driver itself, with single_model routed through the
C ABI (binarytpm_gb300/driver/thermal_dropin.inc), reproduces the
reference CPU run's files bit for bit: shadows, scattered illumination,
final temperatures and per-revolution convergence counts."""
import sys
from pathlib import Path

import numpy as np
import pytest

from conftest import golden

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT / "tests" / "golden"))

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", ["single_s2", "binary_s3s1"])
def test_reference_driver_through_c_abi(gpu_ctx, name, tmp_path):
    import make_golden
    from binarytpm_gb300 import build
    from oracle import refbuild

    prob, ref = golden(name)
    lib = build.build()
    exe = refbuild.build_thermal_dropin(make_golden.thermal_cfg(name), lib.parent, ROOT / "include",
                                        ROOT / "binarytpm_gb300" / "driver")
    make_golden.write_thermal_inputs(tmp_path, prob.vertices, prob.facets, prob.dep_ptr, prob.dep_idx, prob.dep_vf)
    refbuild.run(exe, tmp_path)
    nf, ntau = prob.nf, prob.ntau
    F = np.fromfile(tmp_path / "oracle_forcing.bin", dtype=np.int32).reshape(3, nf, ntau)
    assert np.array_equal(F[0], ref["shadow"])
    assert np.array_equal(F[1], ref["illumination"].view(np.int32))
    T = np.fromfile(tmp_path / ("oracle_temps_%g.bin" % prob.thermal_inertia[-1]), dtype=np.float32)
    n = nf * ntau
    assert np.array_equal(T[:n].view(np.uint32), ref["stemp1"].ravel().view(np.uint32))
    assert np.array_equal(T[2 * n:].view(np.uint32), ref["temp"].ravel().view(np.uint32))
    revs = np.loadtxt(tmp_path / "oracle_revs.txt", ndmin=2)
    assert np.array_equal(revs[:, 2].astype(np.int32), ref["counts"])
