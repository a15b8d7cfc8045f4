"""The C-ABI library: builds, loads, exports every symbol include/atpm.h declares."""
import re
import subprocess
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]


def _declared():
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        names |= set(re.findall(r"ATPM_API\s+[^;(]*?\b(atpm_\w+)\s*\(", h.read_text()))
    return names


def test_header_declares_entry_points():
    names = _declared()
    assert {"atpm_solve_create", "atpm_run", "atpm_batch_run", "atpm_viewfactors_compute"} <= names


def test_library_exports_every_declared_symbol():
    from binarytpm_gb300 import build

    lib = build.build()
    out = subprocess.run(["nm", "-D", "--defined-only", str(lib)], capture_output=True, text=True, check=True).stdout
    exported = set(re.findall(r"\b(atpm_\w+)\b", out))
    missing = _declared() - exported
    assert not missing, missing


def test_library_loads_and_binds():
    from binarytpm_gb300 import build, lib

    build.build()
    L = lib.load()
    assert L.atpm_version() >= 100
    assert L.atpm_status_string(0) == b"ok"
    # every Python binding names a declared symbol
    assert set(lib.exported_symbols()) <= _declared()


def test_no_gpu_is_an_error_not_a_fallback():
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("GPU present")
    from binarytpm_gb300 import lib

    with pytest.raises(lib.AtpmError):
        lib.Context(0)


@pytest.mark.parametrize("header,shim,count,defines", [
    ("atpm_ref_gpu.h", "atpm_ref_gpu_shim.cpp", 27, ["-DREF_ASTNUMFACE=4", "-DREF_NTAU=8", "-DREF_NX=8"]),
    ("atpm_ref_vis_gpu.h", "atpm_ref_vis_gpu_shim.cpp", 6, ["-DREF_ASTNUMFACE=4", "-DREF_NTAU=8"]),
    ("atpm_ref_nonsync_gpu.h", "atpm_ref_nonsync_gpu_shim.cpp", 27,
     ["-DREF_ASTNUMFACE=4", "-DREF_NTAU=8", "-DREF_NX=8"]),
])
def test_reference_gpu_module_shim_defines_every_symbol(tmp_path, header, shim, count, defines):
    """Each shim in binarytpm_gb300/driver defines, with C linkage, every
    function its header declares (the Thermal driver's 27-entry roughness
    module, the Visibility driver's 6-entry crater-visibility module, the
    non-synchronous program's 27-entry flat-array module)."""
    hdr = (ROOT / "include" / header).read_text()
    body = hdr[hdr.index('extern "C" {'):]
    declared = set(re.findall(r"\bvoid\s+(\w+)\s*\(", body))
    assert len(declared) == count
    obj = tmp_path / "shim.o"
    subprocess.run(["g++", "-std=c++14", "-c", *defines, "-I", str(ROOT / "include"),
                    str(ROOT / "binarytpm_gb300" / "driver" / shim), "-o", str(obj)], check=True)
    out = subprocess.run(["nm", "--defined-only", str(obj)], capture_output=True, text=True, check=True).stdout
    defined = set(re.findall(r"\s[Tt]\s+(\w+)$", out, re.M))
    assert declared <= defined, declared - defined


def test_read_back_buffers_are_checked():
    """Caller-owned read-back buffers (Solve.surface_temperature(out=)) are
    checked for shape, dtype, layout and writability before any C call."""
    from binarytpm_gb300 import lib

    a = lib.host_buffer((3, 5), np.float32)
    assert a.shape == (3, 5) and a.dtype == np.float32
    assert lib._out_arg(a, (3, 5), np.float32, "out") is a
    for bad in (np.empty((5, 3), np.float32), np.empty((3, 5), np.float64), np.empty((5, 3), np.float32).T):
        with pytest.raises(ValueError):
            lib._out_arg(bad, (3, 5), np.float32, "out")
    ro = np.empty((3, 5), np.float32)
    ro.flags.writeable = False
    with pytest.raises(ValueError):
        lib._out_arg(ro, (3, 5), np.float32, "out")
    src = np.arange(6, dtype=np.int32).reshape(2, 3)
    c = lib.pinned_copy(src)
    assert c.dtype == src.dtype and np.array_equal(c, src)


def test_noalloc_entry_point_rejects_bad_arguments_before_any_device_work():
    """atpm_scattering_noalloc checks its arguments on the host before it
    touches the GPU: a NULL list pointer, multiple scattering without a
    status word, and more facets than its launch grid covers are errors
    (no kernel is launched, so this runs without a GPU)."""
    from binarytpm_gb300 import build, lib

    build.build()
    L = lib.load()
    p = 4096  # never dereferenced: every call below is rejected first
    args = dict(solar=1367.0, albedo=0.1, acc=1e-4)
    call = lambda nf, ntau, idx, vf, multiple, status: L.atpm_scattering_noalloc(
        nf, ntau, p, idx, vf, p, p, args["solar"], args["albedo"], args["acc"], multiple, p, status, None)
    assert call(16, 8, None, p, 0, p) == 1          # ATPM_E_INVALID: dep_idx NULL
    assert call(16, 8, p, None, 0, p) == 1          # ATPM_E_INVALID: dep_vf NULL
    assert call(16, 8, p, p, 1, None) == 1          # ATPM_E_INVALID: no status word for the Gauss-Seidel cap
    assert b"status" in L.atpm_last_error()
    assert call(600_000, 1, p, p, 0, p) == 4        # ATPM_E_UNSUPPORTED: nf beyond the launch grid
    assert call(2048, 1024, p, p, 0, p) == 4        # ATPM_E_UNSUPPORTED: nf * ntau beyond the scratch


def test_surface_temperatures_of_many_checks_arguments_first():
    """atpm_get_surface_temperatures rejects null arrays before any device
    call, and an empty request is a no-op (no GPU needed for either)."""
    import ctypes as C

    from binarytpm_gb300 import build, lib

    build.build()
    L = lib.load()
    assert L.atpm_get_surface_temperatures(None, 1, None) != 0
    one = (C.c_void_p * 1)(None)
    assert L.atpm_get_surface_temperatures(one, 1, one) != 0  # null solve
    assert L.atpm_get_surface_temperatures(one, -1, one) != 0
    assert L.atpm_get_surface_temperatures(one, 0, one) == 0
