"""The CPU oracle (oracle/atpm_oracle.cpp) against the reference's own outputs.

The golden fixtures were produced by the reference Thermal / Visibility /
Shape_Selfheating programs themselves (tests/golden/make_golden.py); the
oracle restatement must reproduce every float bit-for-bit in its reference
precision mode, and stay within 0.01 K in FP64 mode.
"""
import numpy as np
import pytest

from conftest import golden
from oracle import oracle


@pytest.mark.parametrize("name", ["single_s2", "binary_s3s1"])
def test_oracle_reproduces_reference_thermal(name):
    prob, ref = golden(name)
    o = oracle.single_model(prob, precision=0)
    assert np.array_equal(o["shadow"], ref["shadow"])
    assert np.array_equal(o["cosillum"].view(np.uint32), ref["cosillum"].view(np.uint32))
    assert np.array_equal(o["illumination"].view(np.uint32), ref["illumination"].view(np.uint32))
    assert np.array_equal(o["stemp1"].view(np.uint32), ref["stemp1"].view(np.uint32))
    assert np.array_equal(o["stemp0"].view(np.uint32), ref["stemp0"].view(np.uint32))
    assert np.array_equal(o["temp"].view(np.uint32), ref["temp"].view(np.uint32))
    for got, want in zip(o["counts"], ref["counts_list"]):
        assert np.array_equal(got, want)


def test_oracle_reproduces_reference_visibility():
    prob, ref = golden("vis_s3s1")
    sh, _ = oracle.shadows(prob)
    assert np.array_equal(sh, ref["visibility"])


@pytest.mark.parametrize("name", ["single_s2", "binary_s3s1"])
def test_fp64_oracle_within_tolerance(name):
    prob, ref = golden(name)
    o = oracle.single_model(prob, precision=1)
    # the reference is FP32: the FP64 state may differ by float rounding only
    assert np.max(np.abs(o["stemp1_64"] - ref["stemp1"])) < 0.01
    assert np.max(np.abs(o["illumination64"] - ref["illumination"]) / np.maximum(1.0, np.abs(ref["illumination"]))) < 1e-5


def test_golden_cases_exercise_the_path():
    prob, ref = golden("binary_s3s1")
    # eclipses/mutual shadowing present beyond self-shadowing, mutual heating present
    assert prob.nnz > 10000
    assert ref["shadow"].sum() < (ref["cosillum"] > 0).sum()
    assert len(ref["counts_list"]) == 2 and ref["counts_list"][1][-1] == prob.nf


def test_crater_oracle_reproduces_golden_digests(tmp_path):
    """The reference Thermal driver with its crater (roughness) model on, linked
    with the CPU restatement of its GPU module (oracle/ref_gpu_cpu.cpp), writes
    the bytes the golden digests record on this host too."""
    import hashlib
    import sys
    from pathlib import Path

    sys.path.insert(0, str(Path(__file__).resolve().parent / "golden"))
    import make_golden
    from oracle import refbuild

    prob, ref = golden("rough_s1s1")
    make_golden.write_thermal_inputs(tmp_path, prob.vertices, prob.facets, prob.dep_ptr, prob.dep_idx, prob.dep_vf,
                                     ref["dep_vec"], ref["photovectors"])
    make_golden.write_crater_files(tmp_path, make_golden.crater_texts_from(ref))
    refbuild.run(refbuild.build_thermal(make_golden.thermal_cfg("rough_s1s1")), tmp_path)
    for name, want in zip(ref["files"], ref["sha256"]):
        assert hashlib.sha256((tmp_path / str(name)).read_bytes()).hexdigest() == str(want), name
    # both TI branches ran: equilibrium (TI 0) and conduction (TI 200), each to full convergence
    assert set(ref["rough_ti"].tolist()) == {0.0, 200.0}
    assert ref["rough_counts"][-1] == prob.nf


@pytest.mark.parametrize("name", ["nonsync_rough_s1s1", "nonsync_rough0_s1s1"])
def test_nonsync_crater_oracle_reproduces_golden_digests(tmp_path, name):
    """The non-synchronous program with its crater model on (5 parts, per-facet
    revolution counts 3 and 1, IR absorptivity 0.9), linked with the CPU
    restatement of its GPU module, writes the bytes the golden digests record;
    every part's crater facets converge."""
    import hashlib
    import sys
    from pathlib import Path

    sys.path.insert(0, str(Path(__file__).resolve().parent / "golden"))
    import make_golden
    from oracle import refbuild

    _, ref = golden(name)
    make_golden.write_nonsync_inputs(tmp_path, name, ref)
    refbuild.run(refbuild.build_nonsync(make_golden.nonsync_cfg(name)), tmp_path)
    for fname, want in zip(ref["files"], ref["sha256"]):
        assert hashlib.sha256((tmp_path / str(fname)).read_bytes()).hexdigest() == str(want), fname
    parts, counts = ref["rough_parts"], ref["rough_counts"]
    assert sorted(set(parts.tolist())) == [1, 2, 3, 4, 5]
    assert all(counts[parts == k][-1] == 32 for k in range(1, 6))


def test_crater_visibility_oracle_reproduces_golden_digest(tmp_path):
    """The reference Visibility driver with crater visibility on, linked with
    the CPU restatement of its GPU module, writes the golden bytes."""
    import hashlib
    import sys
    from pathlib import Path

    sys.path.insert(0, str(Path(__file__).resolve().parent / "golden"))
    import make_golden
    from binarytpm_gb300 import mesh
    from oracle import refbuild

    prob, ref = golden("vis_rough_s1s1")
    mesh.write_shape(tmp_path / "shape.txt", prob.vertices, prob.facets)
    make_golden.write_crater_files(tmp_path, make_golden.crater_texts_from(ref))
    refbuild.run(refbuild.build_visibility(make_golden.visibility_cfg("vis_rough_s1s1")), tmp_path)
    raw = (tmp_path / "shape_roughness_visibility.dat").read_bytes()
    assert hashlib.sha256(raw).hexdigest() == str(ref["sha256"][0])


def test_oracle_reproduces_reference_at_nx56():
    """At the benchmark's NX = 56 and NTAU = 720 (single body, 1,280 facets,
    TI 0 then 200 to convergence): the oracle's float mode reproduces the
    reference run's digests and every per-revolution count."""
    import hashlib

    prob, ref = golden("single_s3_nx56")
    sha = lambda a: hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()
    o = oracle.single_model(prob, precision=0)
    assert sha(o["shadow"]) == str(ref["sha256_shadow"])
    assert sha(o["illumination"]) == str(ref["sha256_illumination"])
    assert sha(o["cosillum"]) == str(ref["sha256_cosillum"])
    assert sha(o["stemp1"]) == str(ref["sha256_stemp1_200"])
    assert sha(o["stemp0"]) == str(ref["sha256_stemp0_200"])
    assert sha(o["temp"]) == str(ref["sha256_temp_200"])
    for got, want in zip(o["counts"], ref["counts_list"]):
        assert np.array_equal(got, want)
