#!/usr/bin/env python
"""Benchmark: facet-steps/s of the batched FP32 thermal solve vs the plain
FP64 GPU path on the binary-asteroid workload, with the reference's own
OpenMP CPU code timed on this host beside it.

Workload (one "step", the same in both arms): the synchronous binary
(20,480 + 1,280 = 21,760 facets, NX = 56, NTAU = 720, shadowing +
self-heating on, TACC = 0.005 K) for 8 thermal inertias (25 ... 2,000 SI),
each run from the reference's initial temperatures for revolutions 0-5 of
the reference's protocol.  The protocol tests convergence only after
revolution 5, so every facet advances in every one of these revolutions.
facet-steps = facets x NTAU x revolutions.  The same binary solved to
convergence under the freeze protocol is reported beside it
("converged_batch").

  python bench.py [--steps K] [--warmup W] [--gpus N] [--impl reference]

--impl reference times the reference's own Thermal program (compiled from a
scratch copy, OpenMP on every host core) on the same mesh, with view-factor
lists written by the reference's own Shape_Selfheating program; it loads no
part of this repository's library.  Each of its steps is one revolution of
one thermal inertia.

Under torchrun (N > 1) every rank runs an independent replica (the solves do
not shard); value = facet-steps of all ranks / max time over ranks.
"""
from __future__ import annotations

import argparse
import dataclasses
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "facet-steps/s, batched FP32 vs plain FP64 GPU at <=0.01 K; p50/p99 solve latency"
UNIT = "facet-steps/s"
PEAKS = ROOT / "MEASURED_PEAKS.json"
CACHE = ROOT / "_cache"

# the timed workload, identical in both arms
HEADLINE_REVS = 6
BATCH_TI = [25.0, 50.0, 100.0, 200.0, 400.0, 800.0, 1400.0, 2000.0]
WORKLOAD = ("binary asteroid 20480+1280 facets, NX=56, NTAU=720, TACC=0.005 K, shadowing + self-heating on; "
            "8 thermal inertias 25-2000 SI, each run for revolutions 0-5 of the reference protocol from its "
            "initial temperatures (convergence is tested only after revolution 5: every facet advances)")


def headline_config() -> dict:
    return {"workload": WORKLOAD, "facets": 21760, "nx": 56, "ntau": 720, "thermal_inertia": BATCH_TI,
            "revolutions_per_solve": HEADLINE_REVS, "parallelism": "replicas"}


def _peaks():
    if PEAKS.exists():
        d = json.loads(PEAKS.read_text())
        return d["hbm_gbs"], d["bf16_tflops"], "measured"
    return 6800.0, 1900.0, "fallback"


class Clocks:
    """nvidia-smi sampling of SM clocks and throttle reasons."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.path = None

    def start(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "20"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        self.proc.wait()
        rows = [r.split(",") for r in open(self.path).read().strip().splitlines() if r.strip()]
        os.unlink(self.path)
        sm = [float(r[1]) for r in rows if len(r) >= 9 and r[1].strip().replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if len(r) >= 9 and r[2].strip().replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows if len(r) >= 9 for i in range(4) if r[5 + i].strip() == "Active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist_mod

        dist_mod.init_process_group("nccl" if _cuda() else "gloo")
        dist = dist_mod
    return world, rank, local, dist


def _cuda():
    import torch

    return torch.cuda.is_available()


def _max_over_ranks(x: float, dist, device) -> float:
    if dist is None:
        return x
    import torch

    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def _sum_over_ranks(x: float, dist, device) -> float:
    if dist is None:
        return x
    import torch

    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def _barrier(dist):
    if dist is not None:
        dist.barrier()


# ----------------------------------------------------------------------------------------
def reference_revolutions(inputs: Path, dims: dict, ti: float, revs: int, threads: int):
    """Run the reference's own Thermal program (scratch copy compiled by
    oracle/refbuild.py, OpenMP on ``threads`` host cores) on the stage files
    in ``inputs`` (mesh, view-factor lists, vector list, photon vectors) for
    ``revs`` revolutions at one thermal inertia.  Returns one row per
    revolution: (revolution, active facet-steps, seconds of its revolution
    loop, facets converged after it)."""
    import shutil

    from oracle import refbuild

    exe = refbuild.build_thermal(_ref_cfg(dims, ti, threads, revs))
    with tempfile.TemporaryDirectory() as td:
        wd = Path(td)
        for name in ("shape.txt",) + tuple("shape" + x for x in refbuild.SELFHEATING_OUTPUTS):
            os.symlink(Path(inputs).resolve() / name, wd / name)
        refbuild.run(exe, wd, env_threads=threads)
        tab = np.loadtxt(wd / "oracle_revs.txt", ndmin=2)
    rows, prev = [], 0
    for r in range(len(tab)):
        # facets frozen after revolution r-1 are skipped in revolution r (the
        # convergence test runs only after revolution 5)
        active = dims["nf"] - (prev if r > 6 else 0)
        rows.append((int(tab[r, 1]), active * dims["ntau"], float(tab[r, 3]), int(tab[r, 2])))
        prev = int(tab[r, 2])
    return rows


def _ref_cfg(dims, ti, threads, revs):
    return dict(nv=dims["nv"], nf=dims["nf"], ntau=dims["ntau"], nx=dims["nx"], polar=list(dims["polar"]),
                rot=list(dims["pole"]), rotation_period_s=dims["rotation_period_s"], albedo=dims["albedo"],
                tacc=dims["tacc"], ti_min=ti, ti_max=ti, threads=threads, revcap=revs)


def binary_dims():
    """The headline binary's mesh and the constants the reference program
    takes for it (the same seeded synthetic mesh as the GPU arm)."""
    from binarytpm_gb300 import problem as P

    v, f = P.binary_mesh(5, 3, 2)
    return v, f, dict(nv=len(v), nf=len(f), ntau=720, nx=56, polar=(1.0, 0.0, 0.0), pole=P.BINARY_POLE,
                      rotation_period_s=11.9 * 3600.0, albedo=0.02, tacc=0.005)


def reference_inputs(threads: int):
    """Stage files of the headline binary made by the reference's own
    Shape_Selfheating program (cached under _cache/)."""
    from oracle import refbuild

    v, f, dims = binary_dims()
    return refbuild.selfheating_inputs(v, f, threads, CACHE), dims


def prepare():
    """Write the reference scratch copies this bench compiles (needs the
    reference checkout; the GPU host then compiles the copies it receives):
    the Thermal driver for each revolution count it runs and the
    Shape_Selfheating program for the binary."""
    from oracle import refbuild

    v, f, dims = binary_dims()
    out = [refbuild.thermal_source(_ref_cfg(dims, ti, 1, HEADLINE_REVS)) for ti in BATCH_TI]
    out.append(refbuild.thermal_source(_ref_cfg(dims, 200.0, 1, 2)))
    sh = refbuild.selfheating_source(len(v), len(f), "shape")
    return "\n".join(str(p) for p in out + [sh])


def activity(caps=(10, 25, 50, 75, 100, 150, 200, 250, 300)):
    """Active facets per solve late in the batch: the bench's 8-inertia binary
    is run to each revolution cap in turn (freeze on, fresh solves each time)
    and the facets not yet converged are counted per solve.  One JSON line:
    per cap, the counts in thermal-inertia order."""
    from binarytpm_gb300 import lib, workloads

    ctx = lib.Context(0)
    prob = workloads.binary_problem(ctx)
    tis = workloads.BATCH_TI
    s0 = lib.Solve(ctx, prob, precision=lib.FAST)
    s0.geometry_shadow()
    s0.scattering()
    shadow, illum = s0.shadow(), s0.illumination()
    s0.close()
    out = {}
    for cap in caps:
        solves = [lib.Solve(ctx, prob, precision=lib.FAST, revcap=cap) for _ in tis]
        for s, ti in zip(solves, tis):
            s.set_forcing(shadow, illum)
            s.set_thermal_inertia(ti)
            s.initialise_temperatures()
        lib.batch_run(solves)
        out[str(cap)] = [int(prob.nf - s.converged().sum()) for s in solves]
        for s in solves:
            s.close()
    ctx.close()
    print(json.dumps({"active_facets_per_solve": out, "thermal_inertia": tis, "nf": prob.nf}), flush=True)


def profile_case(nsolves: int = 2, p_subdiv: int = 4):
    """A small, fast case of the same kernels for ncu --set full captures:
    the binary with a subdivision-4 primary (5,120 + 1,280 facets, NX = 56,
    NTAU = 720), ``nsolves`` FAST solves (thermal inertias from the batched
    sweep), three instrumented revolutions.  With ``p_subdiv`` 5 it is the
    headline binary (20,480 + 1,280 facets), for one-pass metric captures
    (DRAM bytes and durations) at full size."""
    from binarytpm_gb300 import lib, workloads

    ctx = lib.Context(0)
    prob = workloads.binary_problem(ctx, p_subdiv=p_subdiv)
    s0 = lib.Solve(ctx, prob, precision=lib.FAST)
    s0.geometry_shadow()
    s0.scattering()
    sh, il = s0.shadow(), s0.illumination()
    solves = [s0]
    for _ in range(nsolves - 1):
        s1 = lib.Solve(ctx, prob, precision=lib.FAST)
        s1.set_forcing(sh, il)
        solves.append(s1)
    tis = [200.0, 800.0] if nsolves == 2 else workloads.BATCH_TI
    for i, s in enumerate(solves):
        s.set_thermal_inertia(tis[i % len(tis)])
        s.initialise_temperatures()
    for _ in range(3):
        k = lib.profile_revolution(solves)
    tiles, lo, rem = _tile_stats(prob)
    print(json.dumps({"profile_case": k, "nf": prob.nf, "nnz": prob.nnz, "tiles": tiles, "lo_tiles": lo,
                      "remainder_entries": rem}))


def precision_stress(p_subdiv: int):
    """The precision-stress configuration: concave 81,920-facet primary +
    5,120-facet secondary (workloads.stress_problem), view factors on the
    GPU, FAST vs plain FP64 on the same schedule at two thermal inertias."""
    from binarytpm_gb300 import lib, workloads

    ctx = lib.Context(0)
    t0 = time.perf_counter()
    prob = workloads.stress_problem(ctx, p_subdiv=p_subdiv)
    vf_s = time.perf_counter() - t0
    s0 = lib.Solve(ctx, prob, precision=lib.FAST)
    s0.geometry_shadow()
    s0.scattering()
    shadow, illum = s0.shadow(), s0.illumination()
    s0.close()
    tiles, lo, rem = _tile_stats(prob)
    t1 = time.perf_counter()
    err = workloads.fast_vs_fp64(ctx, prob, [50.0, 800.0], ACC_REVS, shadow, illum)
    print(json.dumps({"precision_stress": err, "workload": prob.name, "nf": prob.nf, "nnz": int(prob.nnz),
                      "mean_list_length": prob.nnz / prob.nf, "tiles": tiles, "lo_tiles": lo, "remainder_entries": rem,
                      "viewfactor_s": vf_s, "comparison_s": time.perf_counter() - t1}), flush=True)


# exact ray-triangle test (astshadowtest, 3905/Thermal/NominalPole/main.cpp:1187-1247):
# FP64 operations executed per test (a plane intersection, three edge cross
# products and their projections on the normal)
SHADOW_TEST_FLOP = 74
FP64_NOMINAL_TFLOPS = 1.25  # GB300 dense FP64, nominal


def visibility(ctx):
    """The Visibility stage's all-pairs occultation toward an observer
    (astshadow, 3905/Visibility/NominalPole/main.cpp:674-704) at 720 steps,
    REFERENCE precision (FP64 tests, the reference's flags): the 21,760-facet
    binary and the 87,040-facet precision-stress system.  rays = facet x step
    queries; exact tests = ray-triangle tests run after the box cull."""
    from binarytpm_gb300 import lib, mesh, problem as P

    out = {}
    prim = mesh.grf_body(6, 0.39, 0.15, 0.3, 3)
    sec = mesh.perturbed_body(4, 0.08, 0.08, 1003)
    sv, sf = mesh.binary_system(prim, sec, 1.19)
    bv, bf = P.binary_mesh(5, 3, 2)
    for name, (v, f) in (("binary_21760", (bv, bf)), ("stress_87040", (sv, sf))):
        ptr, idx, vf = P.empty_lists(len(f))
        prob = P.Problem(vertices=v, facets=f.astype(np.int32), dep_ptr=ptr, dep_idx=idx, dep_vf=vf, ntau=720,
                         nx=56, polar=(1.2, 0.1, 0.3), pole=P.BINARY_POLE, shadowing=2)
        s = lib.Solve(ctx, prob, precision=lib.REFERENCE)
        best = None
        for _ in range(3):
            s.geometry_shadow()
            st = s.last_shadow_stats()
            if best is None or st[0] < best[0]:
                best = st
        s.close()
        ms, rays, tests = best
        sec_ = ms / 1e3
        out[name] = {"facets": len(f), "steps": 720, "shadow_ms": ms, "rays_per_s": rays / sec_,
                     "exact_tests_per_s": tests / sec_, "exact_tests_per_ray": tests / rays,
                     "fp64_tflops": tests * SHADOW_TEST_FLOP / sec_ / 1e12,
                     "fp64_frac_of_nominal": tests * SHADOW_TEST_FLOP / sec_ / 1e12 / FP64_NOMINAL_TFLOPS,
                     "all_pairs": len(f) * (len(f) - 1) // 2 * 720}
    out["note"] = ("exact tests are FP64 in the reference's operand order (bit-identical flags); "
                   f"{SHADOW_TEST_FLOP} FP64 operations per test against the nominal FP64 rate; best of 3")
    return out


def run_reference_arm(args, world, rank):
    """The reference's own CPU implementation of the timed workload on this
    host's cores.  Nothing of this repository's library is loaded: the
    view-factor lists come from the reference's Shape_Selfheating program
    and the revolutions from its Thermal program.  Each step is one
    revolution of one thermal inertia; the thermal inertias are taken in the
    headline order, 6 revolutions each (revolutions 0-5, every facet
    active), until W + K revolutions are done; the first W are warm-up."""
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    t0 = time.perf_counter()
    inputs, dims = reference_inputs(threads)
    inputs_s = time.perf_counter() - t0
    need = args.warmup + args.steps
    plan, k = [], 0
    while sum(n for _, n in plan) < need:
        plan.append((BATCH_TI[k % len(BATCH_TI)], min(HEADLINE_REVS, need - sum(n for _, n in plan))))
        k += 1
    # the thermal inertia is a compile-time constant of the reference program:
    # one build per run, compiled in parallel before any timing
    from concurrent.futures import ThreadPoolExecutor

    from oracle import refbuild

    with ThreadPoolExecutor(max_workers=min(len(plan), threads)) as ex:
        list(ex.map(lambda p: refbuild.build_thermal(_ref_cfg(dims, p[0], threads, p[1])), plan))
    build_s = time.perf_counter() - t0 - inputs_s
    samples = []
    for ti, n in plan:
        samples += [(ti,) + r for r in reference_revolutions(inputs, dims, ti, n, threads)]
    timed = samples[args.warmup:need]
    fs = sum(r[2] for r in timed)
    secs = sum(r[3] for r in timed)
    value = fs / secs
    sample = (f"{len(timed)} timed revolutions (after {args.warmup} warm-up) of the reference Thermal program's "
              f"revolution loop, thermal inertias {sorted({r[0] for r in timed})}, revolutions 0-5 of each "
              f"(every facet active), {threads} OpenMP threads")
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * secs / len(timed),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": headline_config(),
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "reference", "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "reference_inputs": {"viewfactor_lists": "the reference's Shape_Selfheating program on the same mesh",
                                 "seconds": inputs_s, "nnz": _count_list_entries(inputs)},
            "reference_build_s": build_s,
            "per_revolution_s": [r[3] for r in timed]}
    print(json.dumps(line), flush=True)


def _count_list_entries(inputs: Path) -> int:
    n = 0
    with open(Path(inputs) / "shape_selfheating_list.txt") as fh:
        for line in fh:
            t = line.split(None, 1)
            n += int(t[0]) if t else 0
    return n


# ----------------------------------------------------------------------------------------
def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU reference timing")
    ap.add_argument("--no-fp64", action="store_true", help="skip the plain FP64 comparison")
    ap.add_argument("--no-visibility", action="store_true", help="skip the all-pairs visibility measurement")
    ap.add_argument("--prepare", action="store_true", help="write the reference scratch copy and exit")
    ap.add_argument("--serve-requests", type=int, default=2000, help="requests in the serving run (0: skip)")
    ap.add_argument("--serve-rate", type=float, default=50.0, help="Poisson arrival rate of the serving run (1/s)")
    ap.add_argument("--sweep-solves", type=int, default=256,
                    help="solves in the batched-sweep run (mixed sizes, albedos, inertias; 0: skip)")
    ap.add_argument("--profile-solves", type=int, default=2, help="solves in the --profile-case batch")
    ap.add_argument("--profile-subdiv", type=int, default=4, choices=[4, 5],
                    help="primary subdivision of the --profile-case binary (5: the headline binary)")
    ap.add_argument("--precision-stress", type=int, default=0, metavar="SUBDIV",
                    help="run the precision-stress configuration with this primary subdivision (6: 81,920 facets)")
    ap.add_argument("--activity", action="store_true",
                    help="active facets per solve of the 8-inertia binary at revolution caps 10 ... 300")
    ap.add_argument("--profile-case", action="store_true",
                    help="small case for ncu captures: binary 5120+1280 facets, 2 solves, 3 instrumented revolutions")
    args = ap.parse_args()
    if args.prepare:
        print(prepare())
        return
    if args.precision_stress:
        precision_stress(args.precision_stress)
        return
    if args.profile_case:
        profile_case(args.profile_solves, args.profile_subdiv)
        return
    if args.activity:
        activity()
        return
    world, rank, local, dist = dist_setup()
    if args.impl == "reference":
        run_reference_arm(args, world, rank)
        return

    import torch

    from binarytpm_gb300 import lib, workloads

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    ctx = lib.Context(local)
    t_setup = time.perf_counter()
    prob = workloads.binary_problem(ctx)
    tis = BATCH_TI
    s0 = lib.Solve(ctx, prob, precision=lib.FAST, revcap=HEADLINE_REVS)
    s0.geometry_shadow()
    s0.scattering()
    # the other inertias: device clones of the prepared solve (shared tiles)
    solves = [s0] + [s0.clone() for _ in tis[1:]]
    setup_s = time.perf_counter() - t_setup

    def step(batch):
        for s, ti in zip(batch, tis):
            s.set_thermal_inertia(ti)
            s.initialise_temperatures()
        counts = lib.batch_run(batch)
        ms, launches, fs = batch[0].last_run_stats()
        return ms, launches + 2 * len(batch), fs, counts

    for _ in range(args.warmup):
        step(solves)
    torch.cuda.synchronize()
    _barrier(dist)
    clk = Clocks(local)
    clk.start()
    t0 = time.perf_counter()
    dev_ms, launches, fsteps, nrevs = 0.0, 0, 0, []
    for _ in range(args.steps):
        ms, la, fs, counts = step(solves)
        dev_ms += ms
        launches += la
        fsteps += fs
        nrevs.append([len(c) for c in counts])
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    clocks = clk.stop()
    _barrier(dist)
    dev_ms_max = _max_over_ranks(dev_ms, dist, dev)
    fsteps_all = _sum_over_ranks(float(fsteps), dist, dev)
    value = fsteps_all / (dev_ms_max / 1e3)
    wall_value = fsteps_all / _max_over_ranks(wall, dist, dev)
    # the state the timed schedule ends in: FP64 energy balance and the error
    # against plain FP64 on exactly this schedule
    energy = energy_balance(solves, tis)
    shadow, illum = s0.shadow(), s0.illumination()
    timed_err = None if args.no_fp64 else workloads.fp64_errors(ctx, prob, solves, tis, HEADLINE_REVS, shadow,
                                                                illum, freeze=True)

    cond_v, tc_depth, _ = s0.last_run_config()
    launch_config = {"conduction_variant": cond_v, "tc_pipeline_depth": tc_depth,
                     "chosen_by": "autotuner: the first batch of this kind (a warm-up step) ran its first 5 revolutions "
                                  "with one candidate each, both batch groups together, and timed each "
                                  "revolution whole; results do not depend on the choice"}

    # per-kernel durations of one instrumented (all-active) revolution
    kern = lib.profile_revolution(solves)
    for s in solves:
        s.close()

    # the same binary solved to convergence under the freeze protocol
    conv = converged_batch(ctx, prob, tis, shadow, illum, step, args)

    # plain FP64 GPU path: one solve at a time on the timed workload
    fp64 = None
    conv_err = None
    rev40 = None
    if not args.no_fp64:
        fp64 = fp64_plain(ctx, prob, shadow, illum)
        conv_err = converged_errors(ctx, prob, shadow, illum)
        rev40 = workloads.fast_vs_fp64(ctx, prob, [25.0, 200.0, 2000.0], ACC_REVS, shadow, illum)

    # end to end through the C ABI from host buffers
    e2e = e2e_run(ctx, prob, tis, max(1, min(args.steps, 3)))  # median of up to 3 jobs

    serve = serving(ctx, args.serve_requests, args.serve_rate) if args.serve_requests > 0 else None
    vis = None if args.no_visibility else visibility(ctx)
    sweep = batched_sweep(ctx, args.sweep_solves) if args.sweep_solves > 0 else None

    cpu = None
    if rank == 0 and not args.no_cpu:
        cpu = cpu_baseline(prob)

    hbm, bf16, kind = _peaks()
    roof = _roofline(kern, len(tis), prob, hbm, bf16, kind, cond_v)
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": dev_ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": headline_config(),
        "precision": "FAST (batched FP32 state, BF16 view factors on the tensor cores, FP32 accumulation)",
        "l2": "state per step 8 x 250 MB > L2 (inputs larger than L2)",
        "fp64_plain": fp64,
        "speedup_vs_fp64_plain": (value / fp64["value"]) if fp64 else None,
        "errors_vs_fp64": {"timed_schedule": timed_err, "converged_freeze_on": conv_err,
                           "freeze_off_40_revolutions": rev40},
        "converged_batch": conv,
        "cpu_baseline": cpu,
        "e2e": e2e,
        "gpu_launches": int(launches),
        "clocks": clocks,
        "roofline": roof,
        "latency_ms": ({"p50": serve["p50_ms"], "p99": serve["p99_ms"],
                        "what": f"serving: submit to result, Poisson arrivals {serve['arrival_rate_per_s']}/s, "
                                f"{serve['requests']} requests"} if serve else None),
        "serving": serve,
        "batched_sweep": sweep,
        "visibility": vis,
        "energy_balance_fp64": energy,
        "kernels_ms": kern,
        "launch_config": launch_config,
        "wall_clock_value": wall_value, "setup_s": setup_s, "nnz_viewfactors": int(prob.nnz),
        "revolutions_per_solve": nrevs[-1],
    }
    ctx.close()
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


def energy_balance(solves, tis):
    """FP64 per-revolution energy balance of each solve's last revolution
    (atpm_energy_balance): absorbed (1-A)E + Q and emitted eps sigma T^4,
    summed over facets and steps, and their relative difference."""
    out = {}
    for s, ti in zip(solves, tis):
        ab, em, tm = s.energy_balance()
        out[str(ti)] = {"absorbed": ab, "emitted": em, "mean_temperature_K": tm,
                        "rel_imbalance": (ab - em) / ab if ab else None}
    return out


def converged_batch(ctx, prob, tis, shadow, illum, step, args, steps: int = 2):
    """The 8-inertia batch solved to convergence (freeze protocol, revolution
    cap 301): facet-steps/s over the revolutions actually executed, counting
    a frozen facet only while it is active."""
    import torch

    from binarytpm_gb300 import lib

    c0 = lib.Solve(ctx, prob, precision=lib.FAST)
    c0.set_forcing(shadow, illum)
    batch = [c0] + [c0.clone() for _ in tis[1:]]
    step(batch)  # warm-up: the autotuner times this kind's candidates here
    torch.cuda.synchronize()
    ms_all, fs_all, nrev = 0.0, 0, None
    for _ in range(steps):
        ms, _, fs, counts = step(batch)
        ms_all += ms
        fs_all += fs
        nrev = [len(c) for c in counts]
    energy = energy_balance(batch, tis)
    for s in batch:
        s.close()
    return {"value": fs_all / (ms_all / 1e3), "unit": UNIT, "ms_per_step": ms_all / steps, "steps": steps,
            "revolutions_per_solve": nrev, "energy_balance_fp64": energy,
            "workload": "the same binary and 8 thermal inertias solved to convergence (TACC = 0.005 K, "
                        "freeze protocol, revolution cap 301)"}


def fp64_plain(ctx, prob, shadow, illum):
    """Plain FP64 GPU path, one solve at a time, on the timed workload."""
    from binarytpm_gb300 import lib

    p = lib.Solve(ctx, prob, precision=lib.FP64, revcap=HEADLINE_REVS)
    p.set_forcing(shadow, illum)
    f64_ms, f64_fs = 0.0, 0
    for ti in FP64_TI:
        p.set_thermal_inertia(ti)
        p.initialise_temperatures()
        p.run()
        ms, _, fs = p.last_run_stats()
        f64_ms += ms
        f64_fs += fs
    p.close()
    return {"value": f64_fs / (f64_ms / 1e3), "unit": UNIT, "device_ms": f64_ms, "facet_steps": f64_fs,
            "thermal_inertia": FP64_TI, "mode": "plain FP64, one solve at a time, revolutions 0-5"}


def converged_errors(ctx, prob, shadow, illum):
    """Final-state error after convergence under the freeze protocol, FAST
    and REFERENCE precision each against plain FP64 run the same way.  The
    three precisions freeze some facets in different revolutions, so these
    errors include the protocol's own schedule sensitivity (the bit-exact
    REFERENCE replica shows it too)."""
    from binarytpm_gb300 import lib, workloads

    out = {}
    for name, prec in (("fast", lib.FAST), ("reference", lib.REFERENCE)):
        batch = [lib.Solve(ctx, prob, precision=prec) for _ in CONV_ERR_TI]
        out[name] = workloads.fp64_errors(ctx, prob, batch, CONV_ERR_TI, 301, shadow, illum, freeze=True,
                                          run=True)
        for s in batch:
            s.close()
    return out


def cpu_baseline(prob):
    """The reference's own Thermal program on this host's cores, a bounded
    sample of the timed workload: 2 revolutions at TI 200 (every facet
    active).  Its view-factor lists are the reference Shape_Selfheating
    program's when the reference arm has cached them on this host, else
    this library's (identical index lists, values written at the
    reference's 6 significant digits)."""
    from binarytpm_gb300 import formats, mesh

    threads = os.cpu_count() or 1
    v, f, dims = binary_dims()
    try:
        digest_dir = CACHE / f"refinputs_{_mesh_digest(v, f)}"
        src = "reference Shape_Selfheating (cached)"
        if not (digest_dir / "done").exists():
            digest_dir = Path(tempfile.mkdtemp(prefix="atpm_cpu_inputs_"))
            mesh.write_shape(digest_dir / "shape.txt", prob.vertices, prob.facets)
            formats.write_selfheating_list(digest_dir / "shape_selfheating_list.txt", prob.dep_ptr, prob.dep_idx,
                                           prob.dep_vf)
            (digest_dir / "shape_selfheating_vector_list.txt").write_text("")
            (digest_dir / "shape_photovectors.txt").write_text("0 0 0\n" * prob.nf)
            src = "this library's view factors in the reference's list format"
        rows = reference_revolutions(digest_dir, dims, 200.0, 2, threads)
        fs = sum(r[1] for r in rows)
        secs = sum(r[2] for r in rows)
        return {"value": fs / secs, "unit": UNIT, "cores": threads, "kind": "reference",
                "sample": f"reference Thermal revolution loop, {len(rows)} revolutions of the binary at TI=200 "
                          f"(every facet active, {secs:.1f} s); view-factor lists: {src}"}
    except Exception as ex:  # the checker must not hide the GPU result
        return {"value": None, "unit": UNIT, "cores": threads, "kind": "reference", "sample": f"failed: {ex}"}


def _tc_min_entries() -> int:
    from binarytpm_gb300 import workloads

    e = os.environ.get("ATPM_TC_MIN_ENTRIES")
    return int(e) if e and e.isdigit() and 1 <= int(e) <= 8192 else workloads.TC_MIN_ENTRIES


def _mesh_digest(v, f) -> str:
    import hashlib

    v = np.ascontiguousarray(v, np.float64)
    f = np.ascontiguousarray(f, np.int32)
    return hashlib.sha1(v.tobytes() + f.tobytes()).hexdigest()[:16]


def serving(ctx, n_requests: int, rate: float, seed: int = 5):
    """The serving configuration: a Poisson stream (mean rate ``rate``) of
    binary thermal solves through the continuous-batching server.  Each
    request: a primary icosphere of subdivision 3, 4, 5 or 6 (1,280 ...
    81,920 facets; equally likely, i.e. log-uniform in facets, r = 0.39 km,
    +-5 %), a secondary of subdivision 3 or 4 (1,280 / 5,120 facets, r = 0.08
    km, +-8 %), thermal inertia log-uniform in [10, 2000] SI; NX = 56,
    NTAU = 720, FAST, solved to convergence.  The 8 shapes are registered
    once (view factors, shadows and scattering on the device); requests are
    admitted by HBM budget and batch slots, results collected by a waiter
    thread as they finish."""
    import queue
    import threading

    from binarytpm_gb300 import lib, workloads

    rng = np.random.default_rng(seed)
    srv = lib.Server(ctx, precision=lib.FAST, nx=56, budget_bytes=160 << 30, max_active=128, revs_per_tick=8)
    shapes = {}
    t_reg = time.perf_counter()
    for p in (3, 4, 5, 6):
        for q in (3, 4):
            prob = workloads.binary_problem(ctx, p_subdiv=p, s_subdiv=q)
            shapes[(p, q)] = (srv.add_shape(prob), prob.nf)
    register_s = time.perf_counter() - t_reg
    subs = rng.integers(3, 7, size=n_requests)
    secs = rng.integers(3, 5, size=n_requests)
    tis = np.exp(rng.uniform(np.log(10.0), np.log(2000.0), size=n_requests))
    gaps = rng.exponential(1.0 / rate, size=n_requests)
    pending = queue.Queue()
    lats, errors = [], []

    def waiter():
        while True:
            item = pending.get()
            if item is None:
                return
            rid, sid = item
            try:
                lats.append(srv.wait(rid, sid, timeout_s=3600.0)[2])
            except lib.AtpmError as ex:
                errors.append(str(ex))

    th = threading.Thread(target=waiter)
    th.start()
    t0 = time.perf_counter()
    for p, q, ti, gap in zip(subs, secs, tis, gaps):
        target = time.perf_counter() + gap
        while time.perf_counter() < target:
            time.sleep(min(0.001, max(0.0, target - time.perf_counter())))
        sid = shapes[(int(p), int(q))][0]
        pending.put((srv.submit(sid, float(ti)), sid))
    submit_s = time.perf_counter() - t0
    pending.put(None)
    th.join()
    wall = time.perf_counter() - t0
    st = srv.stats()
    srv.close()
    mix = {f"primary_subdiv{p}": int((subs == p).sum()) for p in (3, 4, 5, 6)}
    mix.update({f"secondary_subdiv{q}": int((secs == q).sum()) for q in (3, 4)})
    return {"requests": n_requests, "completed": len(lats), "errors": errors[:5], "arrival_rate_per_s": rate,
            "p50_ms": 1e3 * float(np.percentile(lats, 50)), "p99_ms": 1e3 * float(np.percentile(lats, 99)),
            "facet_steps_per_s": st["facet_steps_per_s"], "wall_s": wall, "arrivals_s": submit_s,
            "shape_registration_s": register_s, "mix": mix,
            "what": "continuous batching, HBM-budget admission (160 GB, 128 slots, 8 revolutions per tick), "
                    "state resident on the device, solves pooled per shape"}


CRATER_FIXTURE = ROOT / "tests" / "golden" / "rough_s1s1.npz"  # carries the reference's crater model files


def batched_sweep(ctx, n_solves: int, seed: int = 7, rough_revs: int = 2, part: int = 1280, group: int = 4):
    """The batched-sweep configuration: ``n_solves`` binary solves advanced in
    one batch (every kernel launch spans all of them).  Each solve: a primary
    icosphere of subdivision 3, 4 or 5 (1,280 / 5,120 / 20,480 facets,
    equally likely) with a subdivision-3 secondary, thermal inertia
    log-uniform in [10, 2000] SI, Bond albedo uniform in [0.01, 0.2] (its own
    scattering), NX = 48, NTAU = 720, FAST, revolutions 0-5 of the reference
    protocol.  Each solve is a device clone of its shape's prototype (shared
    view-factor tiles), with its own albedo and scattering.

    Roughness (hemispherical craters of 100 sub-facets, the reference's crater
    model; each solve draws a covering fraction in [0, 1] that weights the
    rough flux against the smooth one): one solve of each primary size runs
    the crater model natively -- its forcing from the solve on the device,
    partial shadows, scattering, global heating from the batch's final
    temperatures, starting temperatures, then ``rough_revs`` crater
    revolutions -- in parts of ``part`` facets, ``group`` parts (of any of
    the solves) sharing one crater's launches, timed as sub-facet-steps/s."""
    from binarytpm_gb300 import formats, lib, workloads

    rng = np.random.default_rng(seed)
    t0 = time.perf_counter()
    protos = {}
    for p in (3, 4, 5):
        prob = workloads.binary_problem(ctx, p_subdiv=p, s_subdiv=3, nx=48)
        s = lib.Solve(ctx, prob, precision=lib.FAST, revcap=HEADLINE_REVS)
        s.geometry_shadow()
        protos[p] = (prob, s)
    subs = rng.integers(3, 6, size=n_solves)
    tis = np.exp(rng.uniform(np.log(10.0), np.log(2000.0), size=n_solves))
    albs = rng.uniform(0.01, 0.2, size=n_solves)
    fracs = rng.uniform(0.0, 1.0, size=n_solves)
    solves = []
    for p, ti, a in zip(subs, tis, albs):
        c = protos[int(p)][1].clone()
        c.set_albedo(float(a))
        c.scattering()
        c.set_thermal_inertia(float(ti))
        c.initialise_temperatures()
        solves.append(c)
    setup_s = time.perf_counter() - t0
    counts = lib.batch_run(solves)
    ms, launches, fs = solves[0].last_run_stats()
    out = {"solves": n_solves, "nx": 48, "ntau": 720, "revolutions_per_solve": HEADLINE_REVS,
           "mix": {f"primary_subdiv{p}": int((subs == p).sum()) for p in (3, 4, 5)},
           "facets": int(sum(protos[int(p)][0].nf for p in subs)),
           "facet_steps": int(fs), "device_ms": ms, "facet_steps_per_s": fs / (ms / 1e3),
           "gpu_launches": int(launches), "setup_s": setup_s,
           "all_active": all(len(c) == HEADLINE_REVS for c in counts)}
    # roughness: one solve of each primary size, its parts of ``part`` facets
    # packed ``group`` at a time into one crater (parts of different solves
    # share the crater's launches, each facet with its own inertia and albedo)
    fx = np.load(CRATER_FIXTURE)
    texts = {str(k): str(v) for k, v in zip(fx["crater_names"], fx["crater_texts"])}
    cv, cf, V = formats.crater_model(texts["new_crater2.txt"], texts["new_crater2_selfheating_list.txt"])
    sampled, parts = [], []
    for p in (3, 4, 5):
        i = int(np.flatnonzero(subs == p)[0])
        prob = protos[p][0]
        parts += [(i, prob, f0) for f0 in range(0, prob.nf, part)]
        sampled.append({"primary_subdiv": p, "facets": prob.nf, "thermal_inertia": float(tis[i]),
                        "albedo": float(albs[i]), "roughness_fraction": float(fracs[i])})
    crater = lib.Crater(ctx, part * group, 720, 48, precision=lib.FAST)
    crater.set_surface(cv, cf, V, 11.9 * 3600.0)
    forcing_s, rev_s, sub_steps, craters = 0.0, 0.0, 0, 0
    for g0 in range(0, len(parts), group):
        grp = parts[g0:g0 + group]
        n = part * len(grp)
        tf = time.perf_counter()
        crater.set_properties(np.zeros(part * group, np.uint8),
                              np.repeat([albs[i] for i, _, _ in grp] + [0.0] * (group - len(grp)), part).astype(np.float32),
                              np.repeat([tis[i] for i, _, _ in grp] + [1.0] * (group - len(grp)), part).astype(np.float32))
        for k, (i, prob, f0) in enumerate(grp):
            crater.prepare_part(solves[i], f0, k * part, part, prob.meta["dep_vec"])
        crater.partial_shadow()
        crater.scattering(solves[grp[0][0]].solar(), grp[0][1].scattering_accuracy, multiple=True)
        crater.initialise_temperatures(grp[0][1].emissivity, 5.67e-8)
        tr = time.perf_counter()
        for _ in range(rough_revs):
            crater.inertia_difference(grp[0][1].emissivity, 5.67e-8, grp[0][1].tacc)
        crater.update_converged(grp[0][1].tacc)
        rev_s += time.perf_counter() - tr
        forcing_s += tr - tf
        sub_steps += n * 100 * 720 * rough_revs
        craters += 1
    crater.close()
    out["rough"] = {"sampled": sampled, "part_facets": part, "parts_per_crater": group, "crater_runs": craters,
                    "revolutions": rough_revs, "sub_facet_steps": sub_steps, "sub_facet_steps_per_s": sub_steps / rev_s,
                    "forcing_s": forcing_s,
                    "what": "crater model run natively for every part of the sampled solves, parts of different "
                            "solves packed into one crater (atpm_crater_prepare_part) and advanced in the same "
                            "launches: forcing and global heating on the device from each solve, partial shadows, "
                            "scattering, starting temperatures (forcing_s), then crater revolutions (host clock "
                            "around synchronous calls; the last crater run's unused facets, if any, still advance)"}
    for s in solves:
        s.close()
    for _, s in protos.values():
        s.close()
    return out


FP64_TI = [200.0, 2000.0]
CONV_ERR_TI = [200.0, 2000.0]
# executed instructions per facet-step of the FAST sweep by conduction
# variant (ncu: profiles/conduction_and_spmm_binary_s4s3_fast.md for the
# scalar k_conduction<FAST,56>, profiles/conduction_pairs_binary_s4s3_8solves.md
# for the paired k_conduction_pairs<56>)
COND_INSTR_PER_FACET_STEP = {1: 327, 2: 327, 3: 327, 4: 188}
COND_KERNEL = {1: "k_conduction<FAST,56,1>", 2: "k_conduction<FAST,56,2>", 3: "k_conduction<FAST,56,3>",
               4: "k_conduction_pairs<56>"}
ACC_REVS = 40


def _tile_stats(prob, slices=False):
    """Tile structure of the FAST tensor-core product: 128x64 tiles kept,
    how many of them carry the residual, and the list entries left to the
    sparse FP32 remainder (workloads.tc_tile_structure); with ``slices`` also
    the 128x16 K slices holding an entry (all tiles; residual tiles): the
    products the kernel issues."""
    from binarytpm_gb300 import workloads

    tiles, inv, sl, has_lo = workloads.tc_tile_structure(prob.nf, prob.dep_ptr, prob.dep_idx, prob.dep_vf)
    rem = int((inv < 0).sum())
    if not slices:
        return len(tiles), int(has_lo.sum()), rem
    t = inv >= 0
    sk = np.unique(inv[t].astype(np.int64) * 4 + sl[t])
    return len(tiles), int(has_lo.sum()), rem, len(sk), int(has_lo[sk // 4].sum())


def _roofline(kern, n, prob, hbm, bf16, kind, cond_variant=4):
    """Dominant kernel of the revolution loop: the self-heating product
    (k_spmm_tc over the tensor-core tiles, k_spmm_rem over the FP32 sparse
    remainder beside it on a second stream, then k_rem_add; timed together
    on the launch stream).  Its algorithmic intensity, 2 nnz NTAU FLOP over nnz (2 B
    BF16 + 4 B index) + 8 F NTAU bytes per solve, is ~65 FLOP/B, below the
    GB300 ridge (~290), so the bound is HBM: achieved = algorithmic bytes per
    launch (view factors once, shared by the batch's clones; W read and Q
    written per solve) / CUDA-event duration; traffic = the three kernels'
    ncu DRAM bytes per batch revolution, measured on the headline binary.  The tensor-pipe figures are
    beside it: algorithmic FLOP/s, and executed = every issued 128x16 K
    slice x step chunk x (2 or 3 BF16 products for the hi/lo compensation).
    The conduction sweep is reported beside it."""
    out = {}
    k = kern.get("selfheat_q")
    if k and k["ms"]:
        sec = k["ms"] / 1e3
        flops = 2.0 * prob.nnz * prob.ntau * n
        alg_bytes = prob.nnz * 6.0 + n * 8.0 * prob.nf * prob.ntau
        tiles, lo, rem, sl, sl_lo = _tile_stats(prob, slices=True)
        ntau_pad = -(-prob.ntau // 144) * 144 if prob.ntau > 160 else -(-prob.ntau // 16) * 16
        exe = (2 * sl + sl_lo) * 128.0 * 16 * ntau_pad * 2 * n
        traffic = None
        tf = ROOT / "profiles" / "spmm_tc_traffic.json"
        if tf.exists():
            t = json.loads(tf.read_text())
            if "dram_bytes_per_solve_revolution" in t:
                traffic = t["dram_bytes_per_solve_revolution"] * n
        gbs = alg_bytes / sec / 1e9
        out = {"kernel": "k_spmm_tc", "bound": "hbm", "achieved": gbs, "peak": hbm, "unit": "GB/s",
               "frac": gbs / hbm, "peak_kind": kind, "traffic": traffic, "algorithmic_bytes": alg_bytes,
               "tensor": {"achieved_tflops": flops / sec / 1e12, "peak_tflops": bf16,
                          "frac": flops / sec / 1e12 / bf16, "algorithmic_flop": flops,
                          "executed_tflops": exe / sec / 1e12, "executed_frac": exe / sec / 1e12 / bf16},
               "tiles": tiles, "residual_tiles": lo, "remainder_entries": rem, "nnz": int(prob.nnz),
               "note": "algorithmic bytes = nnz x 6 B + solves x 8 B x F x NTAU; executed tensor FLOP count the "
                       f"zero padding of the issued 128x16 K slices ({sl} of the {4 * tiles} in {tiles} tiles; "
                       f"{sl_lo} in the {lo} tiles with residual) and the hi/lo products; {rem} of {prob.nnz} "
                       f"entries (cells with < {_tc_min_entries()} entries) are summed in FP32 by k_spmm_rem beside "
                       "the product and added to Q by k_rem_add"}
    c = kern.get("conduction")
    if c and c["ms"]:
        nx = prob.nx
        # per facet-step: E, Q and stemp read, E and stemp written (20 B), W
        # as BF16 hi/lo tile entries (4 B) and as FP32 (4 B); the depth column
        # read and written once per facet
        bytes_ = c["facet_steps"] * 28 + c["active_facets"] * 2 * (nx + 1) * 4
        gbs = bytes_ / (c["ms"] / 1e3) / 1e9
        traffic = None
        tf = ROOT / "profiles" / "conduction_fast_nx56_traffic.json"
        if tf.exists():
            per = json.loads(tf.read_text()).get("by_variant", {}).get(str(cond_variant))
            if per:
                traffic = per["dram_bytes_per_facet_step"] * c["facet_steps"]
        # FP32 issue: one warp instruction per SM sub-partition per clock
        issue_peak = 152 * 4 * 32 * 2.07e9
        ipfs = COND_INSTR_PER_FACET_STEP[cond_variant]
        instr = ipfs * c["facet_steps"]
        out["conduction"] = {"kernel": COND_KERNEL[cond_variant], "bound": "fp32_issue",
                             "achieved": instr / (c["ms"] / 1e3) / 1e12, "peak": issue_peak / 1e12,
                             "unit": "T thread-instructions/s",
                             "frac": instr / (c["ms"] / 1e3) / issue_peak,
                             "instructions_per_facet_step": ipfs,
                             # scalar: 55 nodes x 3 FP32 ops + Newton; paired: half of that per facet
                             "minimum_instructions_per_facet_step": 115 if cond_variant == 4 else 230,
                             "hbm": {"achieved": gbs, "peak": hbm, "unit": "GB/s", "frac": gbs / hbm,
                                     "algorithmic_bytes": bytes_, "traffic": traffic},
                             "note": "issue peak = 152 SMs x 4 sub-partitions x 32 lanes x 2.07 GHz (nominal); "
                                     "instructions per facet-step from the ncu capture of this kernel"}
    return out


def e2e_run(ctx, prob, tis, steps):
    """Whole job from host buffers through the C ABI: upload shape + lists,
    geometry/shadowing/scattering once, forcing to the other solves, batched
    revolution loop, temperatures back to the host."""
    from binarytpm_gb300 import lib

    import torch

    # the job's inputs in page-locked host memory, and read-back buffers the
    # caller owns, allocated once (the copies themselves are timed every job)
    prob = dataclasses.replace(prob, **{k: lib.pinned_copy(getattr(prob, k))
                                        for k in ("vertices", "facets", "dep_ptr", "dep_idx", "dep_vf")})
    outs = [lib.host_buffer((prob.nf, prob.ntau), np.float32) for _ in tis]
    vals, h2d, d2h = [], 0, 0
    phases = {}

    def mark(name, t):
        # phase boundaries of the one extra, untimed job (synchronised there)
        if split:
            torch.cuda.synchronize()
            now = time.perf_counter()
            phases[name] = round((now - t) * 1e3, 3)
            return now
        return t

    for j in range(steps + 1):
        split = j == steps
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        t = t0
        s0 = lib.Solve(ctx, prob, precision=lib.FAST, revcap=HEADLINE_REVS)
        t = mark("solve_create_h2d", t)
        s0.geometry_shadow()
        t = mark("geometry_shadow", t)
        s0.scattering()
        t = mark("scattering", t)
        # one prepared shape, cloned on the device for the other inertias
        solves = [s0] + [s0.clone() for _ in tis[1:]]
        for s, ti in zip(solves, tis):
            s.set_thermal_inertia(ti)
            s.initialise_temperatures()
        t = mark("clones_initial_temperatures", t)
        lib.batch_run(solves)
        t = mark("batched_revolutions", t)
        fs = solves[0].last_run_stats()[2]
        # the stage's result: every facet's surface temperature at every step,
        # the solves' copies overlapping
        temps = lib.result_temperatures(solves, outs)
        torch.cuda.synchronize()
        t = mark("temperatures_d2h", t)
        dt = time.perf_counter() - t0
        if not split:
            vals.append(fs / dt)
        shape_bytes = prob.vertices.nbytes + prob.facets.nbytes + prob.dep_ptr.nbytes + prob.dep_idx.nbytes + prob.dep_vf.nbytes
        h2d = shape_bytes
        d2h = sum(t.nbytes for t in temps)
        for s in solves:
            s.close()
    return {"value": statistics.median(vals), "unit": UNIT, "h2d_bytes_per_step": int(h2d),
            "d2h_bytes_per_step": int(d2h), "phases_ms": phases,
            "what": "C-ABI job from host arrays: solve create (H2D), geometry+shadowing+scattering, "
                    "device clones for the other inertias, the timed workload's batched revolutions, "
                    "surface temperatures (the Thermal stage's result) D2H; "
                    "inputs and read-back buffers page-locked, allocated once before the timed jobs; "
                    "phases_ms: host time of each phase in one more job, synchronised between phases"}


if __name__ == "__main__":
    main()
