"""The seeded synthetic shapes behind every benchmark and parity workload
(binarytpm_gb300/mesh.py, problem.py): facet and vertex counts, closed and
consistently outward-wound surfaces (the reference takes a facet's normal as
(v1 - v0) x (v2 - v0)), determinism by seed, the merged binary's index
offsets, the text mesh format, and the explicit scheme's stability ratio of
the configurations."""
import math

import numpy as np
import pytest

from binarytpm_gb300 import mesh
from binarytpm_gb300 import problem as P


def _closed_and_consistent(f):
    """Every directed edge once and its reverse once: a closed surface with
    one winding throughout."""
    d = np.concatenate([f[:, [0, 1]], f[:, [1, 2]], f[:, [2, 0]]])
    key = d[:, 0].astype(np.int64) * (f.max() + 1) + d[:, 1]
    rev = d[:, 1].astype(np.int64) * (f.max() + 1) + d[:, 0]
    return np.unique(key).size == key.size and np.array_equal(np.sort(key), np.sort(rev))


def _signed_volume(v, f):
    return float(np.einsum("ij,ij->i", v[f[:, 0]], np.cross(v[f[:, 1]], v[f[:, 2]])).sum() / 6.0)


@pytest.mark.parametrize("subdiv", [0, 1, 2, 3])
def test_icosphere_counts_and_orientation(subdiv):
    v, f = mesh.icosphere(subdiv)
    assert f.shape == (20 * 4 ** subdiv, 3) and v.shape == (10 * 4 ** subdiv + 2, 3)
    edges = 3 * len(f) // 2
    assert len(v) - edges + len(f) == 2  # Euler characteristic of a sphere
    assert _closed_and_consistent(f)
    n = np.cross(v[f[:, 1]] - v[f[:, 0]], v[f[:, 2]] - v[f[:, 0]])
    assert np.all((n * v[f].mean(axis=1)).sum(axis=1) > 0)  # every normal points outward
    assert np.allclose(np.linalg.norm(v, axis=1), 1.0)


def test_perturbed_and_grf_bodies_are_seeded_and_closed():
    a = mesh.perturbed_body(3, 0.39, 0.05, 1)
    b = mesh.perturbed_body(3, 0.39, 0.05, 1)
    c = mesh.perturbed_body(3, 0.39, 0.05, 2)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
    assert not np.array_equal(a[0], c[0])
    r = np.linalg.norm(a[0], axis=1)
    assert r.min() >= 0.39 * 0.95 and r.max() <= 0.39 * 1.05  # smoothing keeps the noise band
    g = mesh.grf_body(3, 0.39, 0.15, 0.3, 3)
    assert np.array_equal(g[0], mesh.grf_body(3, 0.39, 0.15, 0.3, 3)[0])
    rg = np.linalg.norm(g[0], axis=1)
    assert rg.min() >= 0.39 * 0.3 and 0.05 < rg.std() / rg.mean() < 0.3  # a ~15 % field
    for v, f in (a, g):
        assert _closed_and_consistent(f)
        assert _signed_volume(v, f) > 0  # outward as a whole


def test_benchmark_binary_mesh():
    v, f = P.binary_mesh(5, 3, 2)
    assert f.shape == (20480 + 1280, 3) and v.shape == (10242 + 642, 3)
    assert f[:20480].max() < 10242 and f[20480:].min() == 10242  # secondary indices offset
    sec_c = v[10242:].mean(axis=0)
    assert abs(sec_c[0] - 1.19) < 0.01 and np.linalg.norm(sec_c[1:]) < 0.01
    assert _closed_and_consistent(f[:20480]) and _closed_and_consistent(f[20480:] - 10242)
    assert _signed_volume(v[:10242], f[:20480]) > 0 and _signed_volume(v, f[20480:]) > 0


def test_text_mesh_round_trip(tmp_path):
    v, f = mesh.perturbed_body(2, 0.39, 0.05, 4)
    mesh.write_shape(tmp_path / "shape.txt", v, f)
    v2, f2 = mesh.read_shape(tmp_path / "shape.txt", len(v), len(f))
    assert np.array_equal(v2, v) and np.array_equal(f2, f)  # 17 digits: exact doubles


def test_stability_ratio_of_the_configurations():
    def r(ntau, nx):
        return P.Problem(vertices=np.zeros((3, 3)), facets=np.zeros((1, 3), np.int32),
                         dep_ptr=np.zeros(2, np.int32), dep_idx=np.zeros(0, np.int32),
                         dep_vf=np.zeros(0, np.float32), ntau=ntau, nx=nx).stability_r()
    assert math.isclose(r(720, 56), 0.4276, rel_tol=1e-3)  # every workload here: stable
    assert math.isclose(r(720, 48), 0.3142, rel_tol=1e-3)
    assert r(360, 56) > 0.5 and r(360, 48) > 0.5            # 360 steps would diverge
