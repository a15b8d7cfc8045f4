"""Readers and writers for the reference's stage files.

* ``<shape>_selfheating_list.txt`` -- one line per facet: ``n idx_1 .. idx_n
  vf_1 .. vf_n`` (``3905/Shape_Selfheating/main.cpp:859-870``, read by
  ``3905/Thermal/NominalPole/main.cpp:418-434``).  Returned as CSR arrays.
* ``<shape>_selfheating_vector_list.txt`` -- per facet with dependencies,
  three floats per dependent facet (``3905/Shape_Selfheating/main.cpp:872-882``,
  read by ``3905/Thermal/NominalPole/main.cpp:436-449``); the crater model's
  global view factors are built from them.
* ``<shape>_photovectors.txt`` -- three floats per facet
  (``3905/Shape_Selfheating/main.cpp:884-887``).
* ``<shape>_temperature(TI).txt`` -- vertices, facets, then ``NF*NTAU``
  surface temperatures, facet-major (``main.cpp:2290-2308``).
* ``<shape>_shadow.txt`` / ``_visibility.txt`` -- same header, then
  ``NF*NTAU`` 0/1 integers (``main.cpp:2242-2262``,
  ``3905/Visibility/NominalPole/main.cpp:830-850``).

Text written by the reference uses default ``ostream`` precision (6
significant digits); the writers here do the same so files compare textually.
"""
from __future__ import annotations

import numpy as np


def read_selfheating_list(path, nf: int):
    """Parse a view-factor list into CSR (ptr[int32 nf+1], idx[int32], vf[float32]).

    Values are parsed as float32 the way ``operator>>`` into ``float`` does
    (correctly rounded decimal -> float)."""
    ptr = np.zeros(nf + 1, dtype=np.int64)
    idx_parts, vf_parts = [], []
    with open(path) as fh:
        for f in range(nf):
            tok = fh.readline().split()
            n = int(tok[0]) if tok else 0
            ptr[f + 1] = ptr[f] + n
            if n:
                idx_parts.append(np.array(tok[1:1 + n], dtype=np.int32))
                vf_parts.append(np.array(tok[1 + n:1 + 2 * n], dtype=np.float64).astype(np.float32))
    idx = np.concatenate(idx_parts) if idx_parts else np.zeros(0, np.int32)
    vf = np.concatenate(vf_parts) if vf_parts else np.zeros(0, np.float32)
    return ptr.astype(np.int32), idx.astype(np.int32), vf


def _g6(x) -> str:
    return "%.6g" % x


def write_selfheating_list(path, ptr, idx, vf) -> None:
    """Write CSR view factors in the reference's list format."""
    with open(path, "w") as fh:
        for f in range(len(ptr) - 1):
            a, b = int(ptr[f]), int(ptr[f + 1])
            fh.write("%d\t" % (b - a))
            if b > a:
                fh.write("".join("%d\t" % i for i in idx[a:b]))
                fh.write("".join(_g6(v) + "\t" for v in vf[a:b]))
            fh.write("\n")


def read_float_stream(path, n: int) -> np.ndarray:
    """The first n whitespace-separated floats of a file (float32, as the
    reference's ``operator>>`` into ``float``)."""
    with open(path) as fh:
        tok = fh.read().split()
    if len(tok) < n:
        raise ValueError(f"{path}: {len(tok)} values, {n} expected")
    return np.array(tok[:n], dtype=np.float64).astype(np.float32)


def write_selfheating_vectors(path, ptr, vec) -> None:
    """One line per facet: the three vector components of each dependency."""
    vec = np.asarray(vec).reshape(-1, 3)
    with open(path, "w") as fh:
        for f in range(len(ptr) - 1):
            a, b = int(ptr[f]), int(ptr[f + 1])
            fh.write("".join("%s\t%s\t%s\t" % (_g6(x[0]), _g6(x[1]), _g6(x[2])) for x in vec[a:b]))
            fh.write("\n")


def write_photovectors(path, pv) -> None:
    with open(path, "w") as fh:
        for x in np.asarray(pv).reshape(-1, 3):
            fh.write("%s\t%s\t%s\n" % (_g6(x[0]), _g6(x[1]), _g6(x[2])))


def _header(fh, v, f):
    for x in v:
        fh.write("%s\t%s\t%s\n" % (_g6(x[0]), _g6(x[1]), _g6(x[2])))
    for t in f:
        fh.write("%d\t%d\t%d\n" % (t[0], t[1], t[2]))


def write_temperature(path, v, f, stemp1) -> None:
    """``<shape>_temperature(TI).txt`` (facet-major [nf][ntau])."""
    with open(path, "w") as fh:
        _header(fh, v, f)
        fh.write("\n".join(_g6(x) for x in np.asarray(stemp1, np.float32).ravel()))
        fh.write("\n")


def write_shadow(path, v, f, shadow) -> None:
    """``<shape>_shadow.txt`` / ``<shape>_visibility.txt``."""
    with open(path, "w") as fh:
        _header(fh, v, f)
        fh.write("\n".join("%d" % x for x in np.asarray(shadow).ravel()))
        fh.write("\n")


def read_values_after_header(path, nv: int, nf: int, dtype=np.float64):
    tok = open(path).read().split()
    return np.array(tok[3 * nv + 3 * nf:], dtype=dtype)


def crater_model(mesh_text: str, list_text: str, nsv: int = 61, nsf: int = 100):
    """The crater (roughness) model from the text of its two files, as the
    reference reads them (Surface::readmodel / readselfheating,
    3905/Thermal/NominalPole/main.cpp:641-668): float vertices [nsv][3],
    facets [nsf][3] and the dense view-factor matrix the driver hands its GPU
    module, V[d][i] = view factor of sub-facet i's entry for sub-facet d and
    V[i][i] = 0 (load_GPU_constants, main.cpp:1951-2001)."""
    tok = mesh_text.split()
    v = np.array(tok[:3 * nsv], dtype=np.float64).astype(np.float32).reshape(nsv, 3)
    f = np.array(tok[3 * nsv:3 * nsv + 3 * nsf], dtype=np.int32).reshape(nsf, 3)
    V = np.zeros((nsf, nsf), np.float32)
    lines = list_text.splitlines()
    for i in range(nsf):
        t = lines[i].split()
        n = int(t[0])
        dep = np.array(t[1:1 + n], dtype=np.int64)
        vf = np.array(t[1 + n:1 + 2 * n], dtype=np.float64).astype(np.float32)
        V[dep, i] = vf
        V[i, i] = 0.0
    return v, f, V

