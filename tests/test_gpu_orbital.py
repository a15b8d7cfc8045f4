"""Orbital sweep (the reference's orbital_model, 3905/Thermal/NominalPole/
main.cpp:2612-2810) through lib.orbital_sweep: every orbital point a solve
placed with atpm_orbital_position / atpm_set_position, all points advanced
together in one batch.  REFERENCE precision reproduces the reference
program's orbital run bit for bit: temperatures at each point and the
per-revolution convergence counts."""
import json

import numpy as np
import pytest

from conftest import GOLDEN, golden

pytestmark = pytest.mark.gpu


def test_orbital_sweep_bit_exact(gpu_ctx):
    from binarytpm_gb300 import lib

    prob, ref = golden("orbit_s2")
    orb = json.loads(str(np.load(GOLDEN / "orbit_s2.npz")["case"]))["orbital"]
    out = lib.orbital_sweep(gpu_ctx, prob, (orb["a"], orb["e"], orb["inc"], orb["node"], orb["peri"]), orb["norb"],
                            prob.thermal_inertia, precision=lib.REFERENCE)
    T, counts = out[prob.thermal_inertia[-1]]
    assert np.array_equal(T.view(np.uint32), ref["orbit_stemp1"].view(np.uint32))
    for i in range(orb["norb"]):
        assert np.array_equal(counts[i], ref["orbit_counts"][ref["orbit_index"] == i])


def test_obliquity_sweep_bit_exact(gpu_ctx):
    """The reference's obliquity_model (17 pole latitudes x 2 orbital points
    at one thermal inertia): all 34 solves in one batch, temperatures
    byte-identical to the reference run (SHA-256 over all of them in the
    reference's loop order) and every per-revolution convergence count."""
    import hashlib

    from binarytpm_gb300 import lib

    prob, ref = golden("obliquity_s2")
    obl = json.loads(str(np.load(GOLDEN / "obliquity_s2.npz")["case"]))["obliquity"]
    T, counts = lib.obliquity_sweep(gpu_ctx, prob, (obl["a"], obl["e"], obl["inc"], obl["node"], obl["peri"]),
                                    obl["norb"], obl["nobl"], prob.thermal_inertia[0], precision=lib.REFERENCE)
    assert np.array_equal(T[0].view(np.uint32), ref["obl_stemp1_first_last"][0].view(np.uint32))
    assert np.array_equal(T[-1].view(np.uint32), ref["obl_stemp1_first_last"][1].view(np.uint32))
    assert hashlib.sha256(np.ascontiguousarray(T).tobytes()).hexdigest() == str(ref["obl_temps_sha256"])
    k = 0
    for j in range(1, 18):
        for i in range(obl["norb"]):
            sel = (ref["obl_j"] == j) & (ref["obl_i"] == i)
            assert np.array_equal(counts[k], ref["obl_counts"][sel]), (j, i)
            k += 1
