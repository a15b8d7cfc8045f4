"""The reference's stage files (binarytpm_gb300/formats.py) written and read
back: view-factor lists in CSR with facets that have no dependencies, values
at the reference's default ostream precision (6 significant digits, parsed as
``operator>>`` into float does), and the temperature / shadow files whose
values follow a vertex and facet header."""
import numpy as np
import pytest

from binarytpm_gb300 import formats


def _g6_f32(x):
    return np.array(["%.6g" % v for v in np.asarray(x, np.float64)], dtype=np.float64).astype(np.float32)


def test_selfheating_list_round_trip_with_empty_rows(tmp_path):
    rng = np.random.default_rng(7)
    nf = 9
    lens = np.array([3, 0, 5, 1, 0, 0, 4, 2, 0])
    ptr = np.concatenate([[0], np.cumsum(lens)]).astype(np.int32)
    idx = rng.integers(0, nf, ptr[-1]).astype(np.int32)
    vf = (rng.random(ptr[-1]) * 10.0 ** rng.integers(-7, 0, ptr[-1])).astype(np.float32)
    path = tmp_path / "shape_selfheating_list.txt"
    formats.write_selfheating_list(path, ptr, idx, vf)
    lines = path.read_text().splitlines()
    assert len(lines) == nf and all(ln.split()[0] == str(n) for ln, n in zip(lines, lens))
    p2, i2, v2 = formats.read_selfheating_list(path, nf)
    assert p2.dtype == np.int32 and i2.dtype == np.int32 and v2.dtype == np.float32
    assert np.array_equal(p2, ptr) and np.array_equal(i2, idx)
    assert np.array_equal(v2, _g6_f32(vf))  # what the reference's reader would hold
    # writing what was read reproduces the file byte for byte
    formats.write_selfheating_list(tmp_path / "again.txt", p2, i2, v2)
    assert (tmp_path / "again.txt").read_text() == path.read_text()


def test_temperature_and_shadow_files_skip_their_header(tmp_path):
    rng = np.random.default_rng(3)
    nv, nf, ntau = 6, 8, 5
    v = rng.normal(size=(nv, 3))
    f = rng.integers(0, nv, (nf, 3)).astype(np.int32)
    T = (150.0 + 250.0 * rng.random((nf, ntau))).astype(np.float32)
    sh = rng.integers(0, 2, (nf, ntau)).astype(np.int32)
    formats.write_temperature(tmp_path / "t.txt", v, f, T)
    formats.write_shadow(tmp_path / "s.txt", v, f, sh)
    t_back = formats.read_values_after_header(tmp_path / "t.txt", nv, nf, np.float64)
    s_back = formats.read_values_after_header(tmp_path / "s.txt", nv, nf, np.int32)
    assert t_back.shape == (nf * ntau,) and s_back.shape == (nf * ntau,)
    assert np.array_equal(t_back.astype(np.float32), _g6_f32(T.ravel()))  # facet-major, 6 digits
    assert np.array_equal(s_back, sh.ravel())
    head = (tmp_path / "t.txt").read_text().splitlines()
    assert head[nv].split() == [str(x) for x in f[0]]  # facets follow the vertices


def test_float_stream_reader(tmp_path):
    p = tmp_path / "pv.txt"
    pv = np.array([[0.1, -2.5e-7, 3.0], [1.0, 2.0, 1.0 / 3.0]])
    formats.write_photovectors(p, pv)
    assert np.array_equal(formats.read_float_stream(p, 6), _g6_f32(pv.ravel()))
    with pytest.raises(ValueError):
        formats.read_float_stream(p, 7)


def test_selfheating_vectors_follow_the_list_rows(tmp_path):
    ptr = np.array([0, 2, 2, 3], np.int32)
    vec = np.arange(9, dtype=np.float32).reshape(3, 3) / 7.0
    p = tmp_path / "vec.txt"
    formats.write_selfheating_vectors(p, ptr, vec)
    rows = p.read_text().split("\n")
    assert [len(r.split()) for r in rows[:3]] == [6, 0, 3]
    assert np.array_equal(formats.read_float_stream(p, 9), _g6_f32(vec.ravel()))


def test_crater_model_parses_the_reference_crater_files():
    """formats.crater_model reads the reference's crater mesh and its
    self-heating list as the driver does: 61 float vertices, 100 facets, and
    the dense V[d][i] with every sub-facet's 99 entries and a zero diagonal
    (each sub-facet of the hemispherical bowl sees about half of the rest)."""
    import sys
    from pathlib import Path

    sys.path.insert(0, str(Path(__file__).resolve().parent / "golden"))
    import make_golden
    from conftest import golden

    from binarytpm_gb300 import formats

    _, ref = golden("rough_s1s1")
    texts = make_golden.crater_texts_from(ref)
    v, f, V = formats.crater_model(texts["new_crater2.txt"], texts["new_crater2_selfheating_list.txt"])
    assert v.shape == (61, 3) and v.dtype == np.float32
    assert f.shape == (100, 3) and f.min() >= 0 and f.max() < 61
    assert np.all(np.diag(V) == 0.0)
    assert np.all((V > 0).sum(axis=0) == 99)
    assert np.allclose(V.sum(axis=0), 0.5, atol=0.05)
