"""Non-synchronous binary (the reference's 175706 Thermal program,
175706/Run-04/thermal.cpp): the primary turns three times per model period
and the secondary once, each body's conduction with its own time step,
all-pairs shadowing toward the Sun for the changing mutual eclipses, with and
without self-heating lists (IR absorptivity 0.9).  REFERENCE precision
reproduces that program's temperatures and per-revolution convergence counts
bit for bit."""
import dataclasses
import json

import numpy as np
import pytest

from conftest import GOLDEN, golden

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", ["nonsync_s2s1", "nonsync_sh_s2s1"])
def test_nonsync_binary_bit_exact(gpu_ctx, name):
    from binarytpm_gb300 import lib

    prob, ref = golden(name)
    case = json.loads(str(np.load(GOLDEN / f"{name}.npz")["case"]))
    prob = dataclasses.replace(prob, shadowing=2)
    if not case["selfheating"]:
        prob = dataclasses.replace(prob, dep_ptr=np.zeros(prob.nf + 1, np.int32), dep_idx=np.zeros(0, np.int32),
                                   dep_vf=np.zeros(0, np.float32))
    s = lib.Solve(gpu_ctx, prob, precision=lib.REFERENCE)
    s.set_binary_rotation(int(ref["prinumvtx"]), int(ref["prinumface"]), case["prirevs"], case["secrevs"])
    s.set_ir_absorptivity(case["ir_abs"])
    counts = s.single_model(prob.thermal_inertia)
    T = s.surface_temperature()[0]
    s.close()
    assert np.array_equal(T.view(np.uint32), ref["stemp1"].view(np.uint32)), np.max(np.abs(T - ref["stemp1"]))
    assert np.array_equal(counts[0], ref["counts"])
