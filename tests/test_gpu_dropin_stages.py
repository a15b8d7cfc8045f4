"""The reference Visibility and Shape_Selfheating programs themselves, with
their hot functions routed through the C ABI (binarytpm_gb300/driver/
visibility_dropin.inc, selfheating_dropin.inc), against the same programs
run unmodified on the CPU: the files their own writers produce.

* Visibility: the all-pairs occultation flags toward the observer
  (astshadow, 3905/Visibility/NominalPole/main.cpp:674-704), written by
  writeglobalshadow (main.cpp:830-850): _visibility.txt byte for byte.
* Shape_Selfheating: selfheating + hidden + betterviewfactors
  (3905/Shape_Selfheating/main.cpp:628-744, 187-368, 374-622), written by
  main() (main.cpp:837-888): the same index lists and counts; view factors,
  direction vectors, photon vectors and total view factors at the files'
  6 significant digits, within the bars of the view-factor parity test (the
  device's acosf/cosf are not glibc's).
"""
import sys
from pathlib import Path

import numpy as np
import pytest

from conftest import golden

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT / "tests" / "golden"))

pytestmark = pytest.mark.gpu


def _run_both(tmp_path, ref_exe, drop_exe, write_inputs):
    out = {}
    for tag, exe in (("ref", ref_exe), ("gpu", drop_exe)):
        d = tmp_path / tag
        d.mkdir()
        write_inputs(d)
        from oracle import refbuild

        refbuild.run(exe, d)
        out[tag] = d
    return out["ref"], out["gpu"]


def test_visibility_driver_through_c_abi(gpu_ctx, tmp_path):
    import make_golden
    from binarytpm_gb300 import build, mesh
    from oracle import refbuild

    prob, ref = golden("vis_s3s1")
    lib = build.build()
    cfg = make_golden.visibility_cfg("vis_s3s1")
    ref_exe = refbuild.build_visibility(cfg)
    drop_exe = refbuild.build_visibility_dropin(cfg, lib.parent, ROOT / "include", ROOT / "binarytpm_gb300" / "driver")
    a, b = _run_both(tmp_path, ref_exe, drop_exe, lambda d: mesh.write_shape(d / "shape.txt", prob.vertices,
                                                                             prob.facets))
    want = (a / "shape_visibility.txt").read_bytes()
    got = (b / "shape_visibility.txt").read_bytes()
    assert got == want
    # and the flags are the golden run's
    from binarytpm_gb300 import formats

    flags = formats.read_values_after_header(b / "shape_visibility.txt", prob.nv, prob.nf, np.int32)
    assert np.array_equal(flags.reshape(prob.nf, prob.ntau), ref["visibility"])


def _tokens(path):
    return [line.split() for line in Path(path).read_text().splitlines()]


def _close_tokens(ra, rb, rel=1e-4, absolute=0.0):
    """Two text files of numbers: same shape, integers equal, floats within
    ``rel`` of each other (or ``absolute``, for vector components near
    zero); returns the relative difference of every token (0 where equal)."""
    assert len(ra) == len(rb)
    out = []
    for la, lb in zip(ra, rb):
        assert len(la) == len(lb)
        for x, y in zip(la, lb):
            if x == y:
                out.append(0.0)
                continue
            fx, fy = float(x), float(y)
            assert abs(fx - fy) <= max(rel * max(abs(fx), abs(fy)), absolute) + 1e-30, (x, y)
            out.append(abs(fx - fy) / max(abs(fx), abs(fy), 1e-30))
    return np.array(out)


def test_selfheating_program_through_c_abi(gpu_ctx, tmp_path):
    import make_golden
    from binarytpm_gb300 import build, mesh
    from oracle import refbuild

    v, f = make_golden.case_mesh(("binary", 3, 1))
    lib = build.build()
    ref_exe = refbuild.build_selfheating(len(v), len(f), "shape", threads=8)
    drop_exe = refbuild.build_selfheating_dropin(len(v), len(f), "shape", lib.parent, ROOT / "include",
                                                 ROOT / "binarytpm_gb300" / "driver")
    a, b = _run_both(tmp_path, ref_exe, drop_exe, lambda d: mesh.write_shape(d / "shape.txt", v, f))
    # vertices, facets and dependency counts: identical bytes
    assert (b / "shape_selfheating_map.txt").read_bytes() == (a / "shape_selfheating_map.txt").read_bytes()
    la, lb = _tokens(a / "shape_selfheating_list.txt"), _tokens(b / "shape_selfheating_list.txt")
    nvals = 0
    for k, (ta, tb) in enumerate(zip(la, lb)):
        n = int(ta[0])
        assert tb[:n + 1] == ta[:n + 1]  # count and indices
        la[k], lb[k] = ta[n + 1:], tb[n + 1:]  # the view factors
        nvals += n
    # The bars of the view-factor parity test (device values against the
    # reference's printed list): every value within 1e-4 relative, 99.9% of
    # them within 5e-6.  Here both sides are printed at 6 significant digits,
    # so two values a float rounding apart can print one unit of the 6th digit
    # apart (up to 1e-5 relative): the 99.9% bar is that one unit.
    rel = _close_tokens(la, lb)
    assert nvals > 10000 and rel.size == nvals
    assert np.quantile(rel, 0.999) <= 1.0001e-5, np.quantile(rel, 0.999)
    for name, absolute in (("shape_selfheating_vector_list.txt", 1e-4), ("shape_photovectors.txt", 1e-5),
                           ("shape_total_viewfactor_map.txt", 0.0)):
        ta, tb = _tokens(a / name), _tokens(b / name)
        r = _close_tokens(ta, tb, rel=1e-4, absolute=absolute)
        assert np.mean(r > 0) <= 0.05, (name, np.mean(r > 0))
