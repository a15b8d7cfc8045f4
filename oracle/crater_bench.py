"""Crater module timing: the reference's own GPU module against libatpm's,
through the same 27-function interface (oracle/crater_bench.cpp).

MEASUREMENT INFRASTRUCTURE, not product: it compiles the reference's
GPU_code.cu (a scratch copy with the harness's sizes, written by ``prepare``
where the reference checkout exists) and runs it on the GPU host, next to the
harness linked with binarytpm_gb300/driver/atpm_ref_gpu_shim.cpp over
libatpm (REFERENCE and FAST crater precision).

    python -m oracle.crater_bench [--nf 6400 --ntau 650 --nx 56 --revs 10]

prints one JSON object per module.  The default sizes are the module's own
shipped constants (GPU_code.cu:6-10).
"""
from __future__ import annotations

import argparse
import json
import subprocess
import sys
import tempfile
from pathlib import Path

import numpy as np

from oracle import refbuild

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent
DEFAULT = dict(nf=6400, ntau=650, nx=56)


def _dir(cfg: dict) -> Path:
    return refbuild.OUT_ROOT / refbuild._tag("craterbench", cfg)


def prepare(cfg: dict | None = None) -> Path:
    """Scratch copy of the reference GPU module with the harness sizes."""
    cfg = dict(DEFAULT, **(cfg or {}))
    d = _dir(cfg)
    out = d / "GPU_code.cu"
    if not out.exists():
        src_path = refbuild.REF_ROOT / refbuild.GPU_MODULE_SRC
        if not src_path.exists():
            raise RuntimeError("reference sources unavailable and no scratch GPU module in " + str(d))
        d.mkdir(parents=True, exist_ok=True)
        src = src_path.read_text(errors="replace")
        src = refbuild._sub_const(src, "ASTNUMFACE", str(cfg["nf"]))
        src = refbuild._sub_const(src, "NTAU", str(cfg["ntau"]))
        src = refbuild._sub_const(src, "NX", str(cfg["nx"]))
        out.write_text(src)
    return out


def _defines(cfg):
    return [f"-DREF_ASTNUMFACE={cfg['nf']}", f"-DREF_NTAU={cfg['ntau']}", f"-DREF_NX={cfg['nx']}"]


def build(cfg: dict, module: str, cuda_home: str = "/usr/local/cuda") -> Path:
    d = _dir(cfg)
    d.mkdir(parents=True, exist_ok=True)
    exe = d / f"crater_bench_{module}"
    common = ["g++", "-O3", "-std=c++14", "-w", *_defines(cfg), "-I", str(ROOT / "include"),
              str(HERE / "crater_bench.cpp")]
    if module == "reference_gpu":
        obj = d / "gpu_code_sm103a.o"
        subprocess.run([cuda_home + "/bin/nvcc", "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-w",
                        "-c", str(prepare(cfg)), "-o", str(obj)], check=True)
        cmd = common + [str(obj), "-L", cuda_home + "/lib64", "-lcudart", "-Wl,-rpath," + cuda_home + "/lib64"]
    else:
        from binarytpm_gb300 import build as pkg_build

        lib = pkg_build.build()
        prec = "ATPM_FAST" if module == "atpm_fast" else "ATPM_REFERENCE"
        cmd = common + ["-DATPM_REF_GPU_PRECISION=" + prec,
                        str(ROOT / "binarytpm_gb300" / "driver" / "atpm_ref_gpu_shim.cpp"),
                        "-L", str(lib.parent), "-latpm", "-Wl,-rpath," + str(lib.parent)]
    subprocess.run(cmd + ["-o", str(exe)], check=True)
    return exe


def crater_texts() -> dict:
    """The crater model files: from the reference checkout, else from the
    crater golden fixture (which carries them verbatim)."""
    try:
        return refbuild.crater_files()
    except OSError:
        z = np.load(ROOT / "tests" / "golden" / "rough_s1s1.npz")
        return {str(k): str(v) for k, v in zip(z["crater_names"], z["crater_texts"])}


def run(cfg: dict, modules=("reference_gpu", "atpm_reference", "atpm_fast"), revs: int = 10) -> list[dict]:
    out = []
    with tempfile.TemporaryDirectory() as td:
        wd = Path(td)
        for n, t in crater_texts().items():
            (wd / n).write_text(t, newline="")
        for m in modules:
            exe = build(cfg, m)
            r = subprocess.run([str(exe), str(revs)], cwd=str(wd), check=True, capture_output=True, text=True)
            rec = json.loads(r.stdout.strip().splitlines()[-1])
            rec["module"] = m
            out.append(rec)
    return out


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--nf", type=int, default=DEFAULT["nf"])
    ap.add_argument("--ntau", type=int, default=DEFAULT["ntau"])
    ap.add_argument("--nx", type=int, default=DEFAULT["nx"])
    ap.add_argument("--revs", type=int, default=10)
    ap.add_argument("--modules", default="reference_gpu,atpm_reference,atpm_fast")
    a = ap.parse_args(argv)
    cfg = dict(nf=a.nf, ntau=a.ntau, nx=a.nx)
    for rec in run(cfg, a.modules.split(","), a.revs):
        print(json.dumps(rec))
        sys.stdout.flush()


if __name__ == "__main__":
    main()
