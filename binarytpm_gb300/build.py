"""Build libatpm.so in-tree for sm_103a (GB300).

Each translation unit is compiled in parallel (nvcc for .cu, g++ for host
.cpp), then linked with nvcc.  Host code is compiled with -ffp-contract=off
because the REFERENCE precision mode reproduces the reference's float
arithmetic on the host side too (scalars, libm exception tables).
"""
from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
OUT = PKG / "_build"
LIB = PKG / "libatpm.so"

CUDA_HOME = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda"))
NVCC = str(CUDA_HOME / "bin" / "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CU_SOURCES = ["atpm_thermal.cu", "atpm_scatter.cu", "atpm_geom.cu", "atpm_viewfactor.cu", "atpm_spmm_tc.cu", "atpm_crater.cu", "atpm_crater_forcing.cu", "atpm_flux.cu"]
CPP_SOURCES = ["atpm_capi.cpp", "atpm_powtab.cpp", "atpm_vfapi.cpp", "atpm_server.cpp", "atpm_crater_api.cpp"]


def _sources():
    return [CSRC / s for s in CU_SOURCES + CPP_SOURCES]


def _stale() -> bool:
    if not LIB.exists():
        return True
    t = LIB.stat().st_mtime
    deps = _sources() + list(CSRC.glob("*.h")) + [PKG.parent / "include" / "atpm.h", Path(__file__)]
    return any(p.stat().st_mtime > t for p in deps if p.exists())


def _compile(src: Path) -> Path:
    obj = OUT / (src.name + ".o")
    inc = ["-I", str(CSRC), "-I", str(PKG.parent / "include"), "-I", str(CUDA_HOME / "include")]
    if src.suffix == ".cu":
        cmd = [NVCC, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off",
               "-Xptxas", "-warn-spills", *inc, "-c", str(src), "-o", str(obj)]
    else:
        cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-fvisibility=hidden", "-pthread",
               *inc, "-c", str(src), "-o", str(obj)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return obj


def build(force: bool = False) -> Path:
    if not force and not _stale():
        return LIB
    OUT.mkdir(exist_ok=True)
    with ThreadPoolExecutor(max_workers=len(_sources())) as ex:
        objs = list(ex.map(_compile, _sources()))
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [NVCC, *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-lpthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    shutil.move(str(tmp), str(LIB))
    return LIB


if __name__ == "__main__":
    print(build(force=True))
