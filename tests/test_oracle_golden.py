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
