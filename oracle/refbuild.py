"""Build recipe for the reference's own CPU code (test infrastructure only).

The reference configures every program by editing compile-time constants at
the top of its source (``3905/Thermal/NominalPole/main.cpp:17-76``,
``3905/Shape_Selfheating/main.cpp:10-17``).  This recipe

  1. reads the unmodified sources from the reference checkout (``REF_ROOT``),
  2. rewrites the constant definitions for one configuration, inserts a few
     instrumentation hooks (per-revolution timer and convergence count, binary
     dumps of the forcing and temperatures at full float precision), and
  3. writes the scratch copy to ``oracle/_ref/<tag>/`` (git-ignored) and
     compiles it there with ``g++ -O3 -fopenmp -ffp-contract=off``.

``-ffp-contract=off`` pins the x86-64 reference semantics (no fused
multiply-add) on every host, so an aarch64 build gives the same floats.

The Thermal driver links against the 27 ``extern "C"`` symbols of its GPU
module (``3905/Thermal/NominalPole/GPU_code.cu:600-1026``); for GPU-free runs
they come from ``oracle/ref_gpu_cpu.cpp``, a CPU restatement of that module.

Where the reference checkout is absent (the GPU host), a scratch copy that was
generated earlier is compiled as it is; without one the build fails loudly.
Nothing here is part of the product: only tests, ``__graft_entry__.smoke`` and
``bench.py``'s CPU baseline call it.
"""
from __future__ import annotations

import hashlib
import json
import os
import re
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
# the reference checkout: ATPM_REFERENCE_ROOT, else a directory named
# "reference" beside this repository's root
REF_ROOT = Path(os.environ.get("ATPM_REFERENCE_ROOT", str(HERE.parent.parent / "reference")))
OUT_ROOT = HERE / "_ref"

THERMAL_SRC = "3905/Thermal/NominalPole/main.cpp"
SELFHEAT_SRC = "3905/Shape_Selfheating/main.cpp"
VISIB_SRC = "3905/Visibility/NominalPole/main.cpp"
OBSERVE_SRC = "3905/Observe/NominalPole/wise_main.cpp"
NONSYNC_SRC = "175706/Run-04/thermal.cpp"
CRATER_FILES = ["new_crater2.txt", "new_crater2_selfheating_list.txt",
                "new_crater2_photovectors.txt"]
CRATER_DIR = "3905/Thermal/NominalPole"

CXXFLAGS = ["-O3", "-fopenmp", "-ffp-contract=off", "-std=c++14", "-w"]


def _sub_const(src: str, name: str, value: str) -> str:
    pat = re.compile(r"^([ \t]*(?:const[ \t]+)?(?:int|float|double|string)[ \t]+"
                     + re.escape(name) + r"[ \t]*=[ \t]*)[^;]*;", re.M)
    out, n = pat.subn(lambda m: m.group(1) + value + ";", src, count=1)
    if n != 1:
        raise RuntimeError(f"constant {name} not found in reference source")
    return out


def _insert_after(src: str, start: int, anchor: str, text: str) -> str:
    i = src.find(anchor, start)
    if i < 0:
        raise RuntimeError(f"anchor not found: {anchor!r}")
    j = i + len(anchor)
    return src[:j] + text + src[j:]


def _replace_from(src: str, start: int, anchor: str, text: str) -> str:
    i = src.find(anchor, start)
    if i < 0:
        raise RuntimeError(f"anchor not found: {anchor!r}")
    return src[:i] + text + src[i + len(anchor):]


def _f(x: float) -> str:
    s = "%.9g" % x
    if not any(ch in s for ch in ".en"):
        s += ".0"
    return s + "f"


def _d(x: float) -> str:
    return "%.17g" % x


# Instrumentation compiled into the scratch copy of the Thermal driver.  It
# only reads the driver's objects through their public accessors.
_THERMAL_HOOKS = r'''
#include <chrono>
#include <cstdio>
static std::chrono::steady_clock::time_point __oracle_t0;
static double __oracle_loop_s = 0.0;
static void __oracle_dump_forcing(Asteroid& A) {
	FILE* fp = fopen("oracle_forcing.bin", "wb");
	for (AstFacet* C = A.beginf(); C != A.endf(); ++C) {
		for (int s = 0; s != NTAU; ++s) { int v = C->rtnshadow(s); fwrite(&v, 4, 1, fp); }
	}
	for (AstFacet* C = A.beginf(); C != A.endf(); ++C) {
		for (int s = 0; s != NTAU; ++s) { float v = C->rtntotalillumination(s); fwrite(&v, 4, 1, fp); }
	}
	for (AstFacet* C = A.beginf(); C != A.endf(); ++C) {
		for (int s = 0; s != NTAU; ++s) { float v = (float)cos(C->rtnillumangle(s)); fwrite(&v, 4, 1, fp); }
	}
	fclose(fp);
}
static void __oracle_rev_begin() { __oracle_t0 = std::chrono::steady_clock::now(); }
static void __oracle_rev_end(Asteroid& A, int rev, float ti) {
	auto t1 = std::chrono::steady_clock::now();
	double s = std::chrono::duration<double>(t1 - __oracle_t0).count();
	__oracle_loop_s += s;
	FILE* fp = fopen("oracle_revs.txt", "a");
	fprintf(fp, "%.9g %d %d %.9g\n", ti, rev, A.rtnnumconverged(), s);
	fclose(fp);
	__oracle_t0 = std::chrono::steady_clock::now();
}
static void __oracle_dump_temps(Asteroid& A, float ti) {
	char name[64];
	snprintf(name, sizeof(name), "oracle_temps_%.9g.bin", ti);
	FILE* fp = fopen(name, "wb");
	for (AstFacet* C = A.beginf(); C != A.endf(); ++C) {
		for (int s = 0; s != NTAU; ++s) { float v = C->rtnstemp(1, s); fwrite(&v, 4, 1, fp); }
	}
	for (AstFacet* C = A.beginf(); C != A.endf(); ++C) {
		for (int s = 0; s != NTAU; ++s) { float v = C->rtnstemp(0, s); fwrite(&v, 4, 1, fp); }
	}
	for (AstFacet* C = A.beginf(); C != A.endf(); ++C) {
		for (int i = 0; i != NX + 1; ++i) { float v = C->rtntemp(i); fwrite(&v, 4, 1, fp); }
	}
	fclose(fp);
}
'''


# Extra instrumentation when the crater (roughness) model is on: per-revolution
# roughness convergence counts and a dump of the crater forcing.
_ROUGH_HOOKS = r'''
static void __oracle_dump_rough_forcing(Asteroid& A) {
	FILE* fp = fopen("oracle_rough_forcing.bin", "wb");
	for (AstFacet* C = A.beginf(); C != A.endf(); ++C)
		for (int j = 0; j != SFCNUMFACE; ++j)
			for (int s = 0; s != NTAU; ++s) { float v = (C->beginsf() + j)->rtnshadow(s); fwrite(&v, 4, 1, fp); }
	for (AstFacet* C = A.beginf(); C != A.endf(); ++C)
		for (int j = 0; j != SFCNUMFACE; ++j)
			for (int s = 0; s != NTAU; ++s) { float v = (C->beginsf() + j)->rtnillumangle(s); fwrite(&v, 4, 1, fp); }
	for (AstFacet* C = A.beginf(); C != A.endf(); ++C)
		for (int j = 0; j != SFCNUMFACE; ++j)
			for (int s = 0; s != NTAU; ++s) { float v = (C->beginsf() + j)->rtntotalillumination(s); fwrite(&v, 4, 1, fp); }
	fclose(fp);
}
static void __oracle_rough_rev(Asteroid& A, int rev, float ti) {
	FILE* fp = fopen("oracle_rough_revs.txt", "a");
	fprintf(fp, "%.9g %d %d\n", ti, rev, A.rtnsfcnumconverged());
	fclose(fp);
}
'''


# Orbital sweep instrumentation (orbital_model): per orbital point i, the
# forcing, the per-revolution counts and the final temperatures.
_ORBIT_HOOKS = r'''
static void __oracle_orbit_rev(Asteroid& A, int i, int rev, float ti) {
	FILE* fp = fopen("oracle_orbit_revs.txt", "a");
	fprintf(fp, "%d %.9g %d %d\n", i, ti, rev, A.rtnnumconverged());
	fclose(fp);
}
static void __oracle_obl_rev(Asteroid& A, int j, int i, int rev, float ti) {
	FILE* fp = fopen("oracle_obl_revs.txt", "a");
	fprintf(fp, "%d %d %.9g %d %d\n", j, i, ti, rev, A.rtnnumconverged());
	fclose(fp);
}
static void __oracle_obl_temps(Asteroid& A, int j, int i, float ti) {
	FILE* fp = fopen("oracle_obl_temps.bin", "ab");
	for (AstFacet* C = A.beginf(); C != A.endf(); ++C) {
		for (int s = 0; s != NTAU; ++s) { float v = C->rtnstemp(1, s); fwrite(&v, 4, 1, fp); }
	}
	fclose(fp);
}
static void __oracle_orbit_temps(Asteroid& A, int i, float ti) {
	char name[96];
	snprintf(name, sizeof(name), "oracle_orbit_temps_%d_%.9g.bin", i, ti);
	FILE* fp = fopen(name, "wb");
	for (AstFacet* C = A.beginf(); C != A.endf(); ++C) {
		for (int s = 0; s != NTAU; ++s) { float v = C->rtnstemp(1, s); fwrite(&v, 4, 1, fp); }
	}
	fclose(fp);
}
'''


def thermal_defaults() -> dict:
    return dict(
        nv=642, nf=1280, shape="shape", ntau=720, nx=56,
        polar=(1.0, 0.0, 0.0), rot=(3.14159265358979 / 2, 0.0),
        shadowing=1, roughness=0, multiple_scattering=1,
        tacc=0.005, scattering_accuracy=1e-4, eps=0.9,
        rotation_period_s=2.26 * 3600.0, albedo=0.02,
        ti_min=200.0, ti_max=200.0, ti_step=10.0,
        threads=1, revcap=301,
    )


def _tag(prefix: str, cfg: dict) -> str:
    h = hashlib.sha1(json.dumps(cfg, sort_keys=True).encode()).hexdigest()[:12]
    return f"{prefix}_{h}"


def patch_thermal(cfg: dict) -> str:
    src = (REF_ROOT / THERMAL_SRC).read_text(errors="replace")
    c = cfg
    src = _sub_const(src, "ASTNUMVTX", str(c["nv"]))
    src = _sub_const(src, "ASTNUMFACE", str(c["nf"]))
    src = _sub_const(src, "shape_filename", '"%s"' % c["shape"])
    src = _sub_const(src, "polar0", _d(c["polar"][0]))
    src = _sub_const(src, "polar1", _d(c["polar"][1]))
    src = _sub_const(src, "polar2", _d(c["polar"][2]))
    src = _sub_const(src, "rot0", _d(c["rot"][0]))
    src = _sub_const(src, "rot1", _d(c["rot"][1]))
    src = _sub_const(src, "NTAU", str(c["ntau"]))
    src = _sub_const(src, "NX", str(c["nx"]))
    src = _sub_const(src, "shape_shadowing", str(c["shadowing"]))
    src = _sub_const(src, "roughness_thermal_model", str(c["roughness"]))
    src = _sub_const(src, "multiple_scattering", str(c["multiple_scattering"]))
    src = _sub_const(src, "TACC", _f(c["tacc"]))
    src = _sub_const(src, "scattering_accuracy", _f(c["scattering_accuracy"]))
    src = _sub_const(src, "EPS", _f(c["eps"]))
    src = _sub_const(src, "rotation_period", _f(c["rotation_period_s"]))
    src = _sub_const(src, "bond_albedo", _f(c["albedo"]))
    src = _sub_const(src, "minimum_thermal_inertia", _f(c["ti_min"]))
    src = _sub_const(src, "maximum_thermal_inertia", _f(c["ti_max"]))
    src = _sub_const(src, "thermal_inertia_step", _f(c["ti_step"]))
    # thread count and revolution cap are compile-time macros so one scratch
    # copy serves every host
    src = _sub_const(src, "num_threads", "ORACLE_THREADS")
    for w in ("write_shape_shadow", "write_shape_illumination",
              "write_shape_temperature", "write_roughness_temperature"):
        src = _sub_const(src, w, str(c.get(w, 0)))
    # hooks
    i = src.find("void single_model(Asteroid& A, Surface& S) {")
    if i < 0:
        raise RuntimeError("single_model not found")
    src = src[:i] + _THERMAL_HOOKS + "\n" + src[i:]
    i = src.find("void single_model(Asteroid& A, Surface& S) {")
    src = _insert_after(src, i, "if (multiple_scattering == 1) { multiplescattering(A); }",
                        "\n\t__oracle_dump_forcing(A);")
    src = _replace_from(src, i, "while (A.rtnconverged() == 0 && rev < 301) {",
                        "__oracle_rev_begin();\n\t\twhile (A.rtnconverged() == 0 && rev < ORACLE_REVCAP) {")
    j = src.find("__oracle_rev_begin();", i)
    src = _replace_from(src, j, "rev = rev + 1;",
                        "__oracle_rev_end(A, rev, t_inertia);\n\t\t\trev = rev + 1;")
    j = src.find("__oracle_rev_end(A, rev, t_inertia);", i)
    src = _insert_after(src, j, "if (roughness_thermal_model == 1) { retrieve_GPU_roughness_temperatures(A); }",
                        "\n\t\t__oracle_dump_temps(A, t_inertia);")
    obl = c.get("obliquity")
    if obl:
        src = _sub_const(src, "single_run", "0")
        src = _sub_const(src, "obliquity_run", "1")
        src = _sub_const(src, "NORB", str(obl["norb"]))
        src = _sub_const(src, "NOBL", str(obl["nobl"]))
        for key, name in (("a", "semimajor_axis"), ("e", "eccentricity"), ("inc", "inclination"),
                          ("node", "ascending_node"), ("peri", "argument_periapsis")):
            src = _sub_const(src, name, _d(obl[key]))
        k = src.find("void orbital_model(Asteroid& A, Surface& S) {")
        src = src[:k] + _ORBIT_HOOKS + "\n" + src[k:]
        k = src.find("void obliquity_model(Asteroid& A, Surface& S) {")
        if k < 0:
            raise RuntimeError("obliquity_model not found")
        src = _replace_from(src, k, "while (A.rtnconverged() == 0 && rev < 301) {",
                            "while (A.rtnconverged() == 0 && rev < ORACLE_REVCAP) {")
        j = src.find("while (A.rtnconverged() == 0 && rev < ORACLE_REVCAP) {", k)
        # the obliquity model runs the facets' default inertia, the minimum TI
        src = _replace_from(src, j, "rev = rev + 1;",
                            "__oracle_obl_rev(A, j, i, rev, minimum_thermal_inertia);\n\t\t\t\trev = rev + 1;")
        j = src.find("__oracle_obl_rev(A, j, i, rev, minimum_thermal_inertia);", k)
        src = _insert_after(src, j, "if (roughness_thermal_model == 1) { retrieve_GPU_roughness_temperatures(A); }",
                            "\n\t\t\t__oracle_obl_temps(A, j, i, minimum_thermal_inertia);")
    orb = c.get("orbital")
    if orb:
        src = _sub_const(src, "single_run", "0")
        src = _sub_const(src, "orbital_run", "1")
        src = _sub_const(src, "NORB", str(orb["norb"]))
        src = _sub_const(src, "semimajor_axis", _d(orb["a"]))
        src = _sub_const(src, "eccentricity", _d(orb["e"]))
        src = _sub_const(src, "inclination", _d(orb["inc"]))
        src = _sub_const(src, "ascending_node", _d(orb["node"]))
        src = _sub_const(src, "argument_periapsis", _d(orb["peri"]))
        k = src.find("void orbital_model(Asteroid& A, Surface& S) {")
        if k < 0:
            raise RuntimeError("orbital_model not found")
        src = src[:k] + _ORBIT_HOOKS + "\n" + src[k:]
        k = src.find("void orbital_model(Asteroid& A, Surface& S) {")
        src = _replace_from(src, k, "while (A.rtnconverged() == 0 && rev < 301) {",
                            "while (A.rtnconverged() == 0 && rev < ORACLE_REVCAP) {")
        j = src.find("while (A.rtnconverged() == 0 && rev < ORACLE_REVCAP) {", k)
        src = _replace_from(src, j, "rev = rev + 1;", "__oracle_orbit_rev(A, i, rev, t_inertia);\n\t\t\t\trev = rev + 1;")
        j = src.find("__oracle_orbit_rev(A, i, rev, t_inertia);", k)
        src = _insert_after(src, j, "if (roughness_thermal_model == 1) { retrieve_GPU_roughness_temperatures(A); }",
                            "\n\t\t\t__oracle_orbit_temps(A, i, t_inertia);")
    if c["roughness"]:
        src = src[:i] + _ROUGH_HOOKS + "\n" + src[i:]
        i = src.find("void single_model(Asteroid& A, Surface& S) {")
        src = _insert_after(src, i, "retrieve_GPU_roughness_illumination(A);",
                            "\n\t\t__oracle_dump_rough_forcing(A);")
        src = _replace_from(src, i, "while (A.rtnsfcconverged() == 0 && rev < 301) {",
                            "while (A.rtnsfcconverged() == 0 && rev < ORACLE_REVCAP) {")
        j = src.find("while (A.rtnsfcconverged() == 0 && rev < ORACLE_REVCAP) {", i)
        src = _replace_from(src, j, "rev = rev + 1;", "__oracle_rough_rev(A, rev, t_inertia);\n\t\t\t\trev = rev + 1;")
    return src


def _gpu_module_defines(cfg: dict) -> list[str]:
    return [f"-DREF_ASTNUMFACE={cfg['nf']}", f"-DREF_NTAU={cfg['ntau']}",
            f"-DREF_NX={cfg['nx']}"]


def thermal_source(cfg: dict) -> Path:
    """Write (once) the scratch copy of the Thermal driver for ``cfg``."""
    full = dict(thermal_defaults())
    full.update(cfg)
    threads, revcap = full.pop("threads"), full.pop("revcap")
    d = OUT_ROOT / _tag("thermal", full)
    src_path = d / "main.cpp"
    if not src_path.exists():
        if not (REF_ROOT / THERMAL_SRC).exists():
            raise RuntimeError("reference sources unavailable and no scratch copy in " + str(d))
        d.mkdir(parents=True, exist_ok=True)
        src_path.write_text(patch_thermal(full))
        (d / "config.json").write_text(json.dumps(full, indent=1))
    return src_path


def build_thermal(cfg: dict) -> Path:
    """Return the path of a compiled reference Thermal driver for ``cfg``."""
    full = dict(thermal_defaults())
    full.update(cfg)
    src_path = thermal_source(full)
    exe = src_path.parent / ("thermal_t%d_r%d" % (full["threads"], full["revcap"]))
    if exe.exists():
        return exe
    cmd = ["g++", *CXXFLAGS, *_gpu_module_defines(full), "-DORACLE_THREADS=%d" % full["threads"],
           "-DORACLE_REVCAP=%d" % full["revcap"], str(src_path), str(HERE / "ref_gpu_cpu.cpp"), "-o", str(exe)]
    subprocess.run(cmd, check=True)
    return exe


_DROPIN_HOOKS = r'''
#define ATPM_DROPIN_REVCAP ORACLE_REVCAP
#define ATPM_DROPIN_AFTER_FORCING(A) __oracle_dump_forcing(A)
#define ATPM_DROPIN_AFTER_TI(A, ti, nrev, counts) do { \
    FILE* fp_ = fopen("oracle_revs.txt", "a"); \
    for (int r_ = 0; r_ < (nrev); ++r_) fprintf(fp_, "%.9g %d %d %.9g\n", (ti), r_, (counts)[r_], 0.0); \
    fclose(fp_); __oracle_dump_temps(A, ti); } while (0)
#include "thermal_dropin.inc"
'''


def build_thermal_dropin(cfg: dict, lib_dir: Path, include_dir: Path, glue_dir: Path) -> Path:
    """The reference Thermal driver with single_model replaced by the drop-in
    glue (binarytpm_gb300/driver/thermal_dropin.inc) over libatpm."""
    full = dict(thermal_defaults())
    full.update(cfg)
    src_path = thermal_source(full)
    d = src_path.parent
    exe = d / ("thermal_dropin_t%d_r%d" % (full["threads"], full["revcap"]))
    drop = d / "main_dropin.cpp"
    src = src_path.read_text()
    i = src.find("int main() {")
    if i < 0:
        raise RuntimeError("main() not found in the scratch copy")
    src = src[:i] + _DROPIN_HOOKS + "\n" + src[i:]
    src = _replace_from(src, 0, "if (single_run == 1) { single_model(A, S); }",
                        "if (single_run == 1) { single_model_atpm(A, S); }")
    drop.write_text(src)
    cmd = ["g++", *CXXFLAGS, *_gpu_module_defines(full), "-DORACLE_THREADS=%d" % full["threads"],
           "-DORACLE_REVCAP=%d" % full["revcap"], "-I", str(include_dir), "-I", str(glue_dir), str(drop),
           str(HERE / "ref_gpu_cpu.cpp"), "-L", str(lib_dir), "-latpm", "-Wl,-rpath," + str(lib_dir),
           "-o", str(exe)]
    subprocess.run(cmd, check=True)
    return exe


GPU_MODULE_SRC = "3905/Thermal/NominalPole/GPU_code.cu"


def gpu_module_source(cfg: dict) -> Path:
    """Scratch copy of the reference's own GPU module (GPU_code.cu) with the
    driver's sizes, beside the driver's scratch copy."""
    full = dict(thermal_defaults())
    full.update(cfg)
    d = thermal_source(full).parent
    out = d / "GPU_code.cu"
    if not out.exists():
        if not (REF_ROOT / GPU_MODULE_SRC).exists():
            raise RuntimeError("reference sources unavailable and no scratch GPU module in " + str(d))
        src = (REF_ROOT / GPU_MODULE_SRC).read_text(errors="replace")
        src = _sub_const(src, "ASTNUMFACE", str(full["nf"]))
        src = _sub_const(src, "NTAU", str(full["ntau"]))
        src = _sub_const(src, "NX", str(full["nx"]))
        out.write_text(src)
    return out


def build_thermal_shim(cfg: dict, lib_dir: Path, include_dir: Path, shim: Path, precision: str = "REFERENCE") -> Path:
    """The reference Thermal driver, unmodified flow, with its GPU module
    replaced by binarytpm_gb300/driver/atpm_ref_gpu_shim.cpp over libatpm
    (crater precision ATPM_REFERENCE or ATPM_FAST)."""
    full = dict(thermal_defaults())
    full.update(cfg)
    src_path = thermal_source(full)
    tag = "" if precision == "REFERENCE" else "_" + precision.lower()
    exe = src_path.parent / ("thermal_shim%s_t%d_r%d" % (tag, full["threads"], full["revcap"]))
    cmd = ["g++", *CXXFLAGS, *_gpu_module_defines(full), "-DORACLE_THREADS=%d" % full["threads"],
           "-DATPM_REF_GPU_PRECISION=ATPM_" + precision,
           "-DORACLE_REVCAP=%d" % full["revcap"], "-I", str(include_dir), str(src_path), str(shim),
           "-L", str(lib_dir), "-latpm", "-Wl,-rpath," + str(lib_dir), "-o", str(exe)]
    subprocess.run(cmd, check=True)
    return exe


def build_thermal_refgpu(cfg: dict, cuda_home: str = "/usr/local/cuda") -> Path:
    """The reference Thermal driver linked with the reference's own GPU module
    (scratch copy of GPU_code.cu, nvcc for sm_103a with nvcc's defaults, as the
    reference's Makefile builds it).  Runs only on a GPU host."""
    full = dict(thermal_defaults())
    full.update(cfg)
    src_path = thermal_source(full)
    cu = gpu_module_source(full)
    d = src_path.parent
    obj = d / "gpu_code_sm103a.o"
    exe = d / ("thermal_refgpu_t%d_r%d" % (full["threads"], full["revcap"]))
    subprocess.run([cuda_home + "/bin/nvcc", "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-w",
                    "-c", str(cu), "-o", str(obj)], check=True)
    subprocess.run(["g++", *CXXFLAGS, "-DORACLE_THREADS=%d" % full["threads"],
                    "-DORACLE_REVCAP=%d" % full["revcap"], str(src_path), str(obj),
                    "-L", cuda_home + "/lib64", "-lcudart", "-Wl,-rpath," + cuda_home + "/lib64",
                    "-o", str(exe)], check=True)
    return exe


_NONSYNC_HOOKS = r'''
#include <cstdio>
static void __oracle_rev(Asteroid& A, int rev) {
	FILE* fp = fopen("oracle_revs.txt", "a");
	fprintf(fp, "%d %d\n", rev, A.rtnnumconverged());
	fclose(fp);
}
'''

# With the crater model on: per part, the crater forcing the module returns
# (sub-facet shadow fractions, Sun angles, and what the program stores as the
# sub-facet total illumination) appended in facet order, and the per-revolution
# crater convergence counts.
_NONSYNC_ROUGH_HOOKS = r'''
static void __oracle_dump_rough_forcing(Asteroid& A) {
	FILE* fp = fopen("oracle_rough_forcing.bin", "ab");
	for (int i = STARTROUGHFACE; i != ENDROUGHFACE + 1; ++i)
		for (int j = 0; j != SFCNUMFACE; ++j)
			for (int s = 0; s != NTAU; ++s) { float v = ((A.beginf() + i)->beginsf() + j)->rtnshadow(s); fwrite(&v, 4, 1, fp); }
	for (int i = STARTROUGHFACE; i != ENDROUGHFACE + 1; ++i)
		for (int j = 0; j != SFCNUMFACE; ++j)
			for (int s = 0; s != NTAU; ++s) { float v = ((A.beginf() + i)->beginsf() + j)->rtnillumangle(s); fwrite(&v, 4, 1, fp); }
	for (int i = STARTROUGHFACE; i != ENDROUGHFACE + 1; ++i)
		for (int j = 0; j != SFCNUMFACE; ++j)
			for (int s = 0; s != NTAU; ++s) { float v = ((A.beginf() + i)->beginsf() + j)->rtntotalillumination(s); fwrite(&v, 4, 1, fp); }
	fclose(fp);
}
static void __oracle_rough_rev(Asteroid& A, int rev) {
	FILE* fp = fopen("oracle_rough_revs.txt", "a");
	fprintf(fp, "%s %d %d\n", part.c_str(), rev, A.rtnsfcnumconverged());
	fclose(fp);
}
'''


def patch_nonsync(cfg: dict) -> str:
    """The reference's non-synchronous binary Thermal program
    (175706/Run-04/thermal.cpp) for one configuration: a fixed thermal
    inertia (0: instantaneous equilibrium), per-revolution convergence counts
    logged; it writes its full-precision temperatures itself
    (binary_writeglobaltemperature, thermal.cpp:3291-3316).  Roughness off:
    one part.  With ``roughness`` the crater model runs over ``parts`` parts
    (thermal.cpp:4380-4401; parts after the first read the shape's shadows,
    illumination and temperatures back from the files the first wrote) and
    the per-part crater temperature maps are stitched into one file
    (stitch_temperatures, thermal.cpp:104-244)."""
    src = (REF_ROOT / NONSYNC_SRC).read_text(errors="replace")
    c = cfg
    rough = int(c.get("roughness", 0))
    parts = int(c.get("parts", 1)) if rough else 1
    if c["nf"] % parts:
        raise ValueError("the facet count must split evenly into parts")
    instant = 1 if c["thermal_inertia"] == 0.0 else 0
    for name, val in (("ASTNUMVTX", c["nv"]), ("ASTNUMFACE", c["nf"]), ("NUMROUGHFACE", c["nf"] // parts),
                      ("NUMPARTS", parts),
                      ("PRINUMVTX", c["prinumvtx"]), ("PRINUMFACE", c["prinumface"]),
                      ("NUMPRIREV", c["prirevs"]), ("NUMSECREV", c["secrevs"]), ("NTAU", c["ntau"]), ("NX", c["nx"]),
                      ("fixed_thermal_inertia", 1), ("instant_equib_model", instant),
                      ("roughness_thermal_model", rough),
                      ("load_shape_selfheating", c["selfheating"]), ("multiple_scattering", 1),
                      ("write_roughness_temperature", rough)):
        src = _sub_const(src, name, str(val))
    src = _sub_const(src, "shape_filename", '"%s"' % c.get("shape", "shape"))
    src = _sub_const(src, "polar0", _d(c["polar"][0]))
    src = _sub_const(src, "polar1", _d(c["polar"][1]))
    src = _sub_const(src, "polar2", _d(c["polar"][2]))
    src = _sub_const(src, "rot0", _d(c["rot"][0]))
    src = _sub_const(src, "rot1", _d(c["rot"][1]))
    for name in ("EPS", "rotation_period", "bond_albedo", "thermal_inertia", "TACC", "scattering_accuracy", "IR_ABS"):
        src = _sub_const(src, name, _f(c[name]))
    src = _sub_const(src, "num_threads", "ORACLE_THREADS")
    i = src.find("void single_model(Asteroid &A, Surface &S) {")
    if i < 0:
        raise RuntimeError("single_model not found")
    src = src[:i] + _NONSYNC_HOOKS + "\n" + src[i:]
    i = src.find("void single_model(Asteroid &A, Surface &S) {")
    src = _replace_from(src, i, "while (A.rtnconverged()==0 && rev<301) {",
                        "while (A.rtnconverged()==0 && rev<ORACLE_REVCAP) {")
    j = src.find("while (A.rtnconverged()==0 && rev<ORACLE_REVCAP) {", i)
    src = _replace_from(src, j, "rev=rev+1;", "__oracle_rev(A, rev);\n\t\t\t\trev=rev+1;")
    if not rough:
        # the per-part roughness maps are not written: nothing to stitch
        return _replace_from(src, i, "\tstitch_temperatures();", "")
    src = src[:i] + _NONSYNC_ROUGH_HOOKS + "\n" + src[i:]
    i = src.find("void single_model(Asteroid &A, Surface &S) {")
    src = _insert_after(src, i, "retrieve_GPU_roughness_illumination(A);", "\n\t\t__oracle_dump_rough_forcing(A);")
    src = _replace_from(src, i, "while (A.rtnsfcconverged()==0 && rev<301) {",
                        "while (A.rtnsfcconverged()==0 && rev<ORACLE_REVCAP) {")
    j = src.find("while (A.rtnsfcconverged()==0 && rev<ORACLE_REVCAP) {", i)
    return _replace_from(src, j, "rev=rev+1;", "__oracle_rough_rev(A, rev);\n\t\t\t\trev=rev+1;")


def _nonsync_module_defines(cfg: dict) -> list[str]:
    parts = int(cfg.get("parts", 1))
    return [f"-DREF_ASTNUMFACE={cfg['nf'] // parts}", f"-DREF_NTAU={cfg['ntau']}", f"-DREF_NX={cfg['nx']}"]


def nonsync_source(cfg: dict) -> Path:
    """Write (once) the scratch copy of the non-synchronous program for ``cfg``."""
    d = OUT_ROOT / _tag("nonsync", cfg)
    src_path = d / "thermal.cpp"
    if not src_path.exists():
        if not (REF_ROOT / NONSYNC_SRC).exists():
            raise RuntimeError("reference sources unavailable and no scratch copy in " + str(d))
        d.mkdir(parents=True, exist_ok=True)
        src_path.write_text(patch_nonsync(cfg))
    return src_path


def build_nonsync(cfg: dict, threads: int = 1, revcap: int = 301) -> Path:
    """Reference non-synchronous Thermal program, scratch copy.  Roughness
    off: linked with stand-ins for its (unused) GPU module.  Roughness on:
    linked with the CPU restatement of that module (oracle/ref_gpu_cpu.cpp
    with REF_NONSYNC_MODULE)."""
    src_path = nonsync_source(cfg)
    exe = src_path.parent / ("nonsync_t%d_r%d" % (threads, revcap))
    if exe.exists():
        return exe
    if cfg.get("roughness"):
        module = ["-DREF_NONSYNC_MODULE", *_nonsync_module_defines(cfg), str(HERE / "ref_gpu_cpu.cpp")]
    else:
        module = [str(HERE / "ref_nonsync_gpu_stub.cpp")]
    subprocess.run(["g++", *CXXFLAGS, "-DORACLE_THREADS=%d" % threads, "-DORACLE_REVCAP=%d" % revcap, str(src_path),
                    *module, "-o", str(exe)], check=True)
    return exe


def build_nonsync_shim(cfg: dict, lib_dir: Path, include_dir: Path, shim: Path, precision: str = "REFERENCE",
                       threads: int = 1, revcap: int = 301) -> Path:
    """The non-synchronous program with its GPU module replaced by
    binarytpm_gb300/driver/atpm_ref_nonsync_gpu_shim.cpp over libatpm."""
    src_path = nonsync_source(cfg)
    tag = "" if precision == "REFERENCE" else "_" + precision.lower()
    exe = src_path.parent / ("nonsync_shim%s_t%d_r%d" % (tag, threads, revcap))
    subprocess.run(["g++", *CXXFLAGS, *_nonsync_module_defines(cfg), "-DORACLE_THREADS=%d" % threads,
                    "-DORACLE_REVCAP=%d" % revcap, "-DATPM_REF_GPU_PRECISION=ATPM_" + precision,
                    "-I", str(include_dir), str(src_path), str(shim), "-L", str(lib_dir), "-latpm",
                    "-Wl,-rpath," + str(lib_dir), "-o", str(exe)], check=True)
    return exe


NONSYNC_GPU_MODULE_SRC = "175706/Run-04/thermal_GPU.cu"


def nonsync_gpu_module_source(cfg: dict) -> Path:
    """Scratch copy of the non-synchronous program's own GPU module
    (thermal_GPU.cu) with the program's sizes.  Two allocations get a few
    floats of slack, nothing else changes: finite_difference reads depth row
    NX+1 of the last facet (thermal_GPU.cu:468, one row past sfc_temp_D) and
    sfcpartialshadow reads a 4th Sun-vector component (thermal_GPU.cu:195, one
    float past sfc_illumvector_D at the last facet's last step); neither value
    is used."""
    src_path = nonsync_source(cfg)
    out = src_path.parent / "thermal_GPU.cu"
    if not out.exists():
        if not (REF_ROOT / NONSYNC_GPU_MODULE_SRC).exists():
            raise RuntimeError("reference sources unavailable and no scratch GPU module in " + str(out.parent))
        src = (REF_ROOT / NONSYNC_GPU_MODULE_SRC).read_text(errors="replace")
        src = _sub_const(src, "ASTNUMFACE", str(cfg["nf"] // int(cfg.get("parts", 1))))
        src = _sub_const(src, "NTAU", str(cfg["ntau"]))
        src = _sub_const(src, "NX", str(cfg["nx"]))
        for alloc, pad in (("cudaMalloc((void **)&sfc_temp_D, size);", "SFCNUMFACE"),
                           ("cudaMalloc((void **)&sfc_illumvector_D, size);", "4")):
            if src.count(alloc) != 1:
                raise RuntimeError("allocation not found: " + alloc)
            src = src.replace(alloc, alloc.replace("size);", "size + %s * sizeof(float));" % pad))
        out.write_text(src)
    return out


def build_nonsync_refgpu(cfg: dict, threads: int = 1, revcap: int = 301, cuda_home: str = "/usr/local/cuda") -> Path:
    """The non-synchronous program linked with its own GPU module (scratch
    copy of thermal_GPU.cu, nvcc for sm_103a with nvcc's defaults).  Runs only
    on a GPU host."""
    src_path = nonsync_source(cfg)
    cu = nonsync_gpu_module_source(cfg)
    d = src_path.parent
    obj = d / "thermal_gpu_sm103a.o"
    exe = d / ("nonsync_refgpu_t%d_r%d" % (threads, revcap))
    subprocess.run([cuda_home + "/bin/nvcc", "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-w",
                    "-c", str(cu), "-o", str(obj)], check=True)
    subprocess.run(["g++", *CXXFLAGS, "-DORACLE_THREADS=%d" % threads, "-DORACLE_REVCAP=%d" % revcap,
                    str(src_path), str(obj), "-L", cuda_home + "/lib64", "-lcudart",
                    "-Wl,-rpath," + cuda_home + "/lib64", "-o", str(exe)], check=True)
    return exe


def patch_selfheating(nv: int, nf: int, shape: str) -> str:
    src = (REF_ROOT / SELFHEAT_SRC).read_text(errors="replace")
    src = _sub_const(src, "ASTNUMVTX", str(nv))
    src = _sub_const(src, "ASTNUMFACE", str(nf))
    src = _sub_const(src, "filename", '"%s"' % shape)
    # a compile-time macro, so one scratch copy serves every host
    src = _sub_const(src, "num_threads", "ORACLE_THREADS")
    return src


def selfheating_source(nv: int, nf: int, shape: str) -> Path:
    """Write (once) the scratch copy of Shape_Selfheating for this mesh size."""
    d = OUT_ROOT / _tag("selfheating", dict(nv=nv, nf=nf, shape=shape))
    src_path = d / "main.cpp"
    if not src_path.exists():
        if not (REF_ROOT / SELFHEAT_SRC).exists():
            raise RuntimeError("reference sources unavailable and no scratch copy in " + str(d))
        d.mkdir(parents=True, exist_ok=True)
        src_path.write_text(patch_selfheating(nv, nf, shape))
    return src_path


def build_selfheating(nv: int, nf: int, shape: str, threads: int = 8) -> Path:
    src_path = selfheating_source(nv, nf, shape)
    exe = src_path.parent / ("selfheating_t%d" % threads)
    if exe.exists():
        return exe
    subprocess.run(["g++", *CXXFLAGS, "-DORACLE_THREADS=%d" % threads, str(src_path), "-o", str(exe)], check=True)
    return exe


def build_selfheating_dropin(nv: int, nf: int, shape: str, lib_dir: Path, include_dir: Path, glue_dir: Path,
                             threads: int = 8) -> Path:
    """Shape_Selfheating with selfheating(A) (hidden + betterviewfactors
    included) replaced by the drop-in glue
    (binarytpm_gb300/driver/selfheating_dropin.inc) over libatpm; the
    program's own main() and writers run unchanged."""
    src_path = selfheating_source(nv, nf, shape)
    d = src_path.parent
    src = src_path.read_text()
    i = src.find("void initialise(Asteroid &A) {")
    if i < 0:
        raise RuntimeError("initialise() not found in the scratch copy")
    src = src[:i] + '#include "selfheating_dropin.inc"\n' + src[i:]
    src = _replace_from(src, src.find("void initialise(Asteroid &A) {"), "\tselfheating(A);", "\tselfheating_atpm(A);")
    drop = d / "main_dropin.cpp"
    drop.write_text(src)
    exe = d / ("selfheating_dropin_t%d" % threads)
    subprocess.run(["g++", *CXXFLAGS, "-DORACLE_THREADS=%d" % threads, "-I", str(include_dir), "-I", str(glue_dir),
                    str(drop), "-L", str(lib_dir), "-latpm", "-Wl,-rpath," + str(lib_dir), "-o", str(exe)], check=True)
    return exe


SELFHEATING_OUTPUTS = ("_selfheating_list.txt", "_selfheating_vector_list.txt", "_photovectors.txt")


def _write_shape(path: Path, vertices, facets) -> None:
    """The reference's text mesh: vertex rows (17 significant digits) then
    facet rows of 0-based vertex indices, the layout its readers take
    (3905/Shape_Selfheating/main.cpp:118-121, used as offsets from beginv())."""
    with open(path, "w") as fh:
        for x in vertices:
            fh.write("%.17g\t%.17g\t%.17g\n" % (x[0], x[1], x[2]))
        for t in facets:
            fh.write("%d\t%d\t%d\n" % (t[0], t[1], t[2]))


def selfheating_inputs(vertices, facets, threads: int, cache_root: Path, shape: str = "shape") -> Path:
    """The Thermal stage's inputs for a mesh made the reference's way: the
    mesh in the reference's text format and the view-factor lists, vector
    list and photon vectors written by the reference's own Shape_Selfheating
    program (scratch copy, compiled here).  Cached under
    ``cache_root/refinputs_<mesh digest>/``; returns that directory."""
    import numpy as np

    v = np.ascontiguousarray(vertices, np.float64)
    f = np.ascontiguousarray(facets, np.int32)
    digest = hashlib.sha1(v.tobytes() + f.tobytes()).hexdigest()[:16]
    d = Path(cache_root) / f"refinputs_{digest}"
    if all((d / (shape + s)).exists() for s in SELFHEATING_OUTPUTS) and (d / "done").exists():
        return d
    d.mkdir(parents=True, exist_ok=True)
    _write_shape(d / (shape + ".txt"), v, f)
    exe = build_selfheating(len(v), len(f), shape, threads=threads)
    run(exe, d)
    (d / "done").write_text("reference Shape_Selfheating outputs complete\n")
    return d


def patch_visibility(cfg: dict) -> str:
    src = (REF_ROOT / VISIB_SRC).read_text(errors="replace")
    c = cfg
    src = _sub_const(src, "ASTNUMVTX", str(c["nv"]))
    src = _sub_const(src, "ASTNUMFACE", str(c["nf"]))
    src = _sub_const(src, "shape_filename", '"%s"' % c["shape"])
    src = _sub_const(src, "rot0", _d(c["rot"][0]))
    src = _sub_const(src, "rot1", _d(c["rot"][1]))
    src = _sub_const(src, "ob0", _d(c["observer"][0]))
    src = _sub_const(src, "ob1", _d(c["observer"][1]))
    src = _sub_const(src, "ob2", _d(c["observer"][2]))
    src = _sub_const(src, "NTAU", str(c["ntau"]))
    src = _sub_const(src, "num_threads", str(c["threads"]))
    rough = str(int(c.get("roughness", 0)))
    src = _sub_const(src, "roughness_visibility_test", rough)
    src = _sub_const(src, "write_roughness_visibility", rough)
    src = _sub_const(src, "shape_visibility_test", "1")
    src = _sub_const(src, "write_shape_visibility", "1")
    return src


def visibility_source(cfg: dict) -> Path:
    """Write (once) the scratch copy of the Visibility driver for ``cfg``."""
    full = dict(nv=642, nf=1280, shape="shape", ntau=720, rot=(3.14159265358979 / 2, 0.0),
                observer=(1.0, 0.0, 0.0), threads=1)
    full.update(cfg)
    d = OUT_ROOT / _tag("visibility", full)
    src_path = d / "main.cpp"
    if not src_path.exists():
        if not (REF_ROOT / VISIB_SRC).exists():
            raise RuntimeError("reference sources unavailable and no scratch copy in " + str(d))
        d.mkdir(parents=True, exist_ok=True)
        src_path.write_text(patch_visibility(full))
    return src_path


def _vis_defines(cfg: dict) -> list[str]:
    return ["-DREF_VISIBILITY_MODULE", f"-DREF_ASTNUMFACE={cfg['nf']}", f"-DREF_NTAU={cfg['ntau']}"]


def build_visibility(cfg: dict) -> Path:
    """Reference Visibility driver (all-pairs occultation toward an observer;
    with ``roughness`` the crater partial visibility too, through the CPU
    restatement of its GPU module)."""
    src_path = visibility_source(cfg)
    exe = src_path.parent / "visibility"
    if exe.exists():
        return exe
    subprocess.run(["g++", *CXXFLAGS, *_vis_defines(cfg), str(src_path), str(HERE / "ref_gpu_cpu.cpp"),
                    "-o", str(exe)], check=True)
    return exe


def build_visibility_shim(cfg: dict, lib_dir: Path, include_dir: Path, shim: Path) -> Path:
    """The Visibility driver with its GPU module replaced by
    binarytpm_gb300/driver/atpm_ref_vis_gpu_shim.cpp over libatpm."""
    src_path = visibility_source(cfg)
    exe = src_path.parent / "visibility_shim"
    subprocess.run(["g++", *CXXFLAGS, *_vis_defines(cfg), "-I", str(include_dir), str(src_path), str(shim),
                    "-L", str(lib_dir), "-latpm", "-Wl,-rpath," + str(lib_dir), "-o", str(exe)], check=True)
    return exe


def build_visibility_dropin(cfg: dict, lib_dir: Path, include_dir: Path, glue_dir: Path) -> Path:
    """The Visibility driver with its all-pairs shape visibility loop
    (main.cpp:929-936) replaced by the drop-in glue
    (binarytpm_gb300/driver/visibility_dropin.inc) over libatpm; the crater
    visibility, when on, goes through the Visibility GPU module shim."""
    import re

    src_path = visibility_source(cfg)
    d = src_path.parent
    drop = d / "main_dropin.cpp"
    src = src_path.read_text()
    i = src.find("int main() {")
    if i < 0:
        raise RuntimeError("main() not found in the scratch copy")
    src = src[:i] + '#include "visibility_dropin.inc"\n' + src[i:]
    pat = re.compile(r"if \(shape_visibility_test==1\) \{\s*omp_set_num_threads\(num_threads\);\s*"
                     r"#pragma omp parallel for schedule\(dynamic\)\s*for \(step=0;step<NTAU;step\+\+\) \{"
                     r"\s*astshadow\(A,step\);[^\n]*\n[^\n]*\n\s*\}\n\s*\}")
    src, n = pat.subn("if (shape_visibility_test==1) { shape_visibility_atpm(A, O); }", src, count=1)
    if n != 1:
        raise RuntimeError("shape visibility loop not found in the scratch copy")
    drop.write_text(src)
    exe = d / "visibility_dropin"
    extra = [str(HERE.parent / "binarytpm_gb300" / "driver" / "atpm_ref_vis_gpu_shim.cpp")] \
        if cfg.get("roughness") else [str(HERE / "ref_gpu_cpu.cpp")]
    subprocess.run(["g++", *CXXFLAGS, *_vis_defines(cfg), "-I", str(include_dir), "-I", str(glue_dir), str(drop),
                    *extra, "-L", str(lib_dir), "-latpm", "-Wl,-rpath," + str(lib_dir), "-o", str(exe)],
                   check=True)
    return exe


VIS_GPU_MODULE_SRC = "3905/Visibility/NominalPole/GPU_code.cu"


def visibility_gpu_module_source(cfg: dict) -> Path:
    """Scratch copy of the Visibility driver's own GPU module with its sizes."""
    d = visibility_source(cfg).parent
    out = d / "GPU_code.cu"
    if not out.exists():
        if not (REF_ROOT / VIS_GPU_MODULE_SRC).exists():
            raise RuntimeError("reference sources unavailable and no scratch GPU module in " + str(d))
        src = (REF_ROOT / VIS_GPU_MODULE_SRC).read_text(errors="replace")
        src = _sub_const(src, "ASTNUMFACE", str(cfg["nf"]))
        src = _sub_const(src, "NTAU", str(cfg["ntau"]))
        out.write_text(src)
    return out


def build_visibility_refgpu(cfg: dict, cuda_home: str = "/usr/local/cuda") -> Path:
    """The Visibility driver linked with its own GPU module (nvcc, sm_103a)."""
    src_path = visibility_source(cfg)
    cu = visibility_gpu_module_source(cfg)
    d = src_path.parent
    obj = d / "vis_gpu_code_sm103a.o"
    exe = d / "visibility_refgpu"
    subprocess.run([cuda_home + "/bin/nvcc", "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-w",
                    "-c", str(cu), "-o", str(obj)], check=True)
    subprocess.run(["g++", *CXXFLAGS, str(src_path), str(obj), "-L", cuda_home + "/lib64", "-lcudart",
                    "-Wl,-rpath," + cuda_home + "/lib64", "-o", str(exe)], check=True)
    return exe


_OBSERVE_HOOK = r'''
#include <cstdio>
static void __oracle_dump_flux(const double* smooth, const double* rough) {
	FILE* fp = fopen("oracle_flux.bin", "ab");
	fwrite(smooth, sizeof(double), num_wavelengths, fp);
	fclose(fp);
	fp = fopen("oracle_rough_flux.bin", "ab");
	fwrite(rough, sizeof(double), num_wavelengths, fp);
	fclose(fp);
}
'''


def patch_observe(cfg: dict) -> str:
    """The Observe stage with its constants set and the raw smooth flux of
    every step dumped (binary, before the colour-correction fit)."""
    src = (REF_ROOT / OBSERVE_SRC).read_text(errors="replace")
    c = cfg
    src = _sub_const(src, "ASTNUMVTX", str(c["nv"]))
    src = _sub_const(src, "ASTNUMFACE", str(c["nf"]))
    src = _sub_const(src, "NTAU", str(c["ntau"]))
    src = _sub_const(src, "shape_filename", '"%s"' % c.get("shape", "shape"))
    for k, name in enumerate(("hel_polar0", "hel_polar1", "hel_polar2")):
        src = _sub_const(src, name, _d(c["polar"][k]))
    for k, name in enumerate(("obs_polar0", "obs_polar1", "obs_polar2")):
        src = _sub_const(src, name, _d(c["observer"][k]))
    src = _sub_const(src, "rot0", _d(c["rot"][0]))
    src = _sub_const(src, "rot1", _d(c["rot"][1]))
    src = _sub_const(src, "minimum_thermal_inertia", str(int(c["ti"])))
    src = _sub_const(src, "maximum_thermal_inertia", str(int(c["ti"])))
    i = src.find("void observe(Surface &S, Asteroid &A, string smooth_outname, string rough_outname) {")
    if i < 0:
        raise RuntimeError("observe() not found")
    src = src[:i] + _OBSERVE_HOOK + "\n" + src[i:]
    src = _insert_after(src, i, "\t\tchisqr_smooth=100.0, chisqr_rough=100.0;", "")
    j = src.find("\t\tchisqr_smooth=100.0, chisqr_rough=100.0;", i)
    src = src[:j] + "\t\t__oracle_dump_flux(astsmoothfluxtotal, astroughfluxtotal);\n" + src[j:]
    return src


def build_observe(cfg: dict) -> Path:
    """Reference Observe stage (disk-integrated flux), scratch copy."""
    full = dict(shape="shape", hooks=2)  # hooks: the instrumentation's version (smooth + rough flux dumps)
    full.update(cfg)
    d = OUT_ROOT / _tag("observe", full)
    exe = d / "observe"
    src_path = d / "wise_main.cpp"
    if exe.exists():
        return exe
    d.mkdir(parents=True, exist_ok=True)
    if not src_path.exists():
        if not (REF_ROOT / OBSERVE_SRC).exists():
            raise RuntimeError("reference sources unavailable and no scratch copy in " + str(d))
        src_path.write_text(patch_observe(full))
    subprocess.run(["g++", *CXXFLAGS, str(src_path), "-o", str(exe)], check=True)
    return exe


def crater_files() -> dict[str, str]:
    """Text of the reference's crater (roughness) model files."""
    return {n: (REF_ROOT / CRATER_DIR / n).read_text() for n in CRATER_FILES}


def run(exe: Path, workdir: Path, env_threads: int | None = None, quiet: bool = True):
    env = dict(os.environ)
    if env_threads:
        env["OMP_NUM_THREADS"] = str(env_threads)
    out = subprocess.DEVNULL if quiet else None
    subprocess.run([str(exe)], cwd=str(workdir), check=True, stdout=out, env=env)
