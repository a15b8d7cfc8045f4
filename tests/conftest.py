import json
import math
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))
GOLDEN = Path(__file__).resolve().parent / "golden"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and libatpm.so")


def golden(name: str):
    """Load a golden case: (Problem, dict of reference outputs)."""
    from binarytpm_gb300.problem import Problem

    z = np.load(GOLDEN / f"{name}.npz")
    c = json.loads(str(z["case"]))
    nf = len(z["facets"])
    ntau = c["ntau"]
    prob = Problem(
        vertices=z["vertices"], facets=z["facets"], dep_ptr=z["dep_ptr"], dep_idx=z["dep_idx"],
        dep_vf=z["dep_vf"], ntau=ntau, nx=c.get("nx", 8),
        polar=tuple(c.get("polar", c.get("observer", (1.0, 0.0, 0.0)))), pole=tuple(c["pole"]),
        rotation_period_s=c.get("period_h", 2.26) * 3600.0, albedo=c.get("albedo", 0.02),
        tacc=c.get("tacc", 0.005), thermal_inertia=c.get("ti", [200.0]),
        shadowing=2 if c["kind"] == "visibility" else 1, name=name)
    ref = {k: z[k] for k in z.files if k not in ("case",)}
    for key in ("shadow", "visibility"):
        if key in ref:
            ref[key] = np.unpackbits(ref[key])[: nf * ntau].reshape(nf, ntau).astype(np.int32)
    if "counts" in ref and "counts_split" in ref:
        split = np.cumsum(ref["counts_split"])[:-1]
        ref["counts_list"] = np.split(ref["counts"], split)
    return prob, ref


@pytest.fixture(scope="session")
def gpu_ctx():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from binarytpm_gb300 import lib

    lib.load()
    ctx = lib.Context(0)
    yield ctx
    ctx.close()
