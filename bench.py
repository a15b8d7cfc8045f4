#!/usr/bin/env python
"""Benchmark: facet-steps/s of the batched FP32 thermal solve vs the plain
FP64 GPU path on the binary-asteroid workload, with the reference's own
OpenMP CPU code timed on this host beside it.

Workload (one "step"): the synchronous binary (20,480 + 1,280 = 21,760
facets, NX = 56, NTAU = 720, shadowing + self-heating on, TACC = 0.005 K)
solved to convergence for a batch of 8 thermal inertias at once, starting
from the reference's initial temperatures.  facet-steps = active facets x
NTAU summed over the revolutions actually executed.

  python bench.py [--steps K] [--warmup W] [--gpus N] [--impl reference]

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
                 "-lms", "100"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
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
def reference_cpu(problem, ti: float, revs: int, threads: int):
    """Time the reference's own Thermal program (compiled from a scratch copy by
    oracle/refbuild.py) on this host: per-revolution wall time of its
    revolution loop.  Returns (facet-steps/s, seconds, revolutions, threads)."""
    from binarytpm_gb300 import formats, mesh
    from oracle import refbuild

    cfg = _ref_cfg(problem, ti, threads, revs)
    exe = refbuild.build_thermal(cfg)
    with tempfile.TemporaryDirectory() as td:
        wd = Path(td)
        mesh.write_shape(wd / "shape.txt", problem.vertices, problem.facets)
        formats.write_selfheating_list(wd / "shape_selfheating_list.txt", problem.dep_ptr, problem.dep_idx,
                                       problem.dep_vf)
        (wd / "shape_selfheating_vector_list.txt").write_text("")
        (wd / "shape_photovectors.txt").write_text("0 0 0\n" * problem.nf)
        refbuild.run(exe, wd, env_threads=threads)
        revs_tab = np.loadtxt(wd / "oracle_revs.txt", ndmin=2)
    secs = float(revs_tab[:, 3].sum())
    fs = 0
    for r in range(len(revs_tab)):
        active = problem.nf if r - 1 <= 5 else problem.nf - int(revs_tab[r - 1, 2])
        fs += active * problem.ntau
    return fs / secs, secs, len(revs_tab), threads


def _ref_cfg(problem, ti, threads, revs):
    return dict(nv=problem.nv, nf=problem.nf, ntau=problem.ntau, nx=problem.nx, polar=list(problem.polar),
                rot=list(problem.pole), rotation_period_s=problem.rotation_period_s, albedo=problem.albedo,
                tacc=problem.tacc, ti_min=ti, ti_max=ti, threads=threads, revcap=revs)


def prepare():
    """Write the reference scratch copy for this workload (needs the reference
    checkout; the GPU host then compiles the copy it receives)."""
    from binarytpm_gb300 import problem as P
    from oracle import refbuild

    v, f = P.binary_mesh(5, 3, 2)
    prob = P.Problem(vertices=v, facets=f, dep_ptr=None, dep_idx=None, dep_vf=None, ntau=720, nx=56,
                     polar=(1.0, 0.0, 0.0), pole=P.BINARY_POLE, rotation_period_s=11.9 * 3600.0,
                     albedo=0.02, tacc=0.005)
    return refbuild.thermal_source(_ref_cfg(prob, 200.0, 1, 3))


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


def profile_case(nsolves: int = 2):
    """A small, fast case of the same kernels for ncu --set full captures:
    the binary with a subdivision-4 primary (5,120 + 1,280 facets, NX = 56,
    NTAU = 720), ``nsolves`` FAST solves (thermal inertias from the batched
    sweep), three instrumented revolutions."""
    from binarytpm_gb300 import lib, workloads

    ctx = lib.Context(0)
    prob = workloads.binary_problem(ctx, p_subdiv=4)
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
    tiles, lo = _tile_stats(prob)
    print(json.dumps({"profile_case": k, "nf": prob.nf, "nnz": prob.nnz, "tiles": tiles, "lo_tiles": lo}))


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
    tiles, lo = _tile_stats(prob)
    t1 = time.perf_counter()
    err = workloads.fast_vs_fp64(ctx, prob, [50.0, 800.0], ACC_REVS, shadow, illum)
    print(json.dumps({"precision_stress": err, "workload": prob.name, "nf": prob.nf, "nnz": int(prob.nnz),
                      "mean_list_length": prob.nnz / prob.nf, "tiles": tiles, "lo_tiles": lo,
                      "viewfactor_s": vf_s, "comparison_s": time.perf_counter() - t1}), flush=True)


def run_reference_arm(args, world, rank):
    if rank != 0:
        return
    from binarytpm_gb300 import lib, workloads

    ctx = lib.Context(0)
    prob = workloads.binary_problem(ctx)
    ctx.close()
    threads = os.cpu_count() or 1
    vals = []
    for _ in range(args.steps):
        v, secs, nrev, _ = reference_cpu(prob, 200.0, 3, threads)
        vals.append(v)
    value = statistics.median(vals)
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": "binary 20480+1280 facets, NX=56, NTAU=720, TI=200, reference OpenMP CPU",
                       "sample": "3 revolutions per step (all facets active)"},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "reference",
                             "sample": "reference Thermal revolution loop, 3 revolutions of the binary at TI=200"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ----------------------------------------------------------------------------------------
def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU reference timing")
    ap.add_argument("--no-fp64", action="store_true", help="skip the plain FP64 comparison")
    ap.add_argument("--prepare", action="store_true", help="write the reference scratch copy and exit")
    ap.add_argument("--serve-requests", type=int, default=48, help="requests in the serving run (0: skip)")
    ap.add_argument("--serve-rate", type=float, default=50.0, help="Poisson arrival rate of the serving run (1/s)")
    ap.add_argument("--profile-solves", type=int, default=2, help="solves in the --profile-case batch")
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
        profile_case(args.profile_solves)
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
    tis = workloads.BATCH_TI
    s0 = lib.Solve(ctx, prob, precision=lib.FAST)
    s0.geometry_shadow()
    s0.scattering()
    # the other inertias: device clones of the prepared solve (shared tiles)
    solves = [s0] + [s0.clone() for _ in tis[1:]]
    setup_s = time.perf_counter() - t_setup

    def step():
        for s, ti in zip(solves, tis):
            s.set_thermal_inertia(ti)
            s.initialise_temperatures()
        counts = lib.batch_run(solves)
        ms, launches, fs = s0.last_run_stats()
        return ms, launches + 2 * len(solves), fs, counts

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    _barrier(dist)
    clk = Clocks(local)
    clk.start()
    t0 = time.perf_counter()
    dev_ms, launches, fsteps, nrevs = 0.0, 0, 0, []
    for _ in range(args.steps):
        ms, la, fs, counts = step()
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

    cond_v, tc_depth, _ = s0.last_run_config()
    launch_config = {"conduction_variant": cond_v, "tc_pipeline_depth": tc_depth,
                     "chosen_by": "autotuner: the first batch of this kind (a warm-up step) timed the candidates "
                                  "on its first 3 revolutions; results do not depend on the choice"}

    # per-kernel durations of one instrumented revolution of the same batch
    kern = lib.profile_revolution(solves)

    # plain FP64 GPU path: one solve at a time under the same protocol
    fp64 = None
    err = None
    if not args.no_fp64:
        shadow, illum = s0.shadow(), s0.illumination()
        p = lib.Solve(ctx, prob, precision=lib.FP64)
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
        fp64 = {"value": f64_fs / (f64_ms / 1e3), "unit": UNIT, "device_ms": f64_ms, "facet_steps": f64_fs,
                "thermal_inertia": FP64_TI, "mode": "plain FP64, one solve at a time, reference protocol"}
        err = accuracy(ctx, prob, tis, shadow, illum)

    # end to end through the C ABI from host buffers
    e2e = e2e_run(ctx, prob, tis, max(1, min(args.steps, 3)))  # median of up to 3 jobs

    serve = serving(ctx, args.serve_requests, args.serve_rate) if args.serve_requests > 0 else None

    cpu = None
    if rank == 0 and not args.no_cpu:
        try:
            v, secs, nrev, th = reference_cpu(prob, 200.0, 3, os.cpu_count() or 1)
            cpu = {"value": v, "unit": UNIT, "cores": th, "kind": "reference",
                   "sample": f"reference Thermal revolution loop, {nrev} revolutions of the binary at TI=200 "
                             f"({secs:.1f} s)"}
        except Exception as ex:  # the checker must not hide the GPU result
            cpu = {"value": None, "unit": UNIT, "cores": os.cpu_count(), "kind": "reference",
                   "sample": f"failed: {ex}"}

    hbm, bf16, kind = _peaks()
    roof = _roofline(kern, solves, prob, hbm, bf16, kind)
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": dev_ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": "binary asteroid 20480+1280 facets, NX=56, NTAU=720, batch of 8 thermal inertias "
                               "solved to convergence (TACC=0.005 K)",
                   "thermal_inertia": tis, "precision": "FAST (batched FP32)", "parallelism": "replicas",
                   "l2": "state per step 8 x 250 MB > L2 (inputs larger than L2)",
                   "revolutions_per_solve": nrevs[-1], "nnz_viewfactors": int(prob.nnz)},
        "wall_clock_value": wall_value, "setup_s": setup_s,
        "fp64_plain": fp64,
        "speedup_vs_fp64_plain": (value / fp64["value"]) if fp64 else None,
        "errors_vs_fp64": err,
        "latency_ms": ({"p50": serve["p50_ms"], "p99": serve["p99_ms"],
                        "what": f"serving: submit to result, Poisson arrivals {serve['arrival_rate_per_s']}/s, "
                                f"{serve['requests']} requests"} if serve else None),
        "serving": serve,
        "roofline": roof,
        "kernels_ms": kern,
        "launch_config": launch_config,
        "cpu_baseline": cpu,
        "e2e": e2e,
        "gpu_launches": int(launches),
        "clocks": clocks,
    }
    for s in solves:
        s.close()
    ctx.close()
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


def serving(ctx, n_requests: int, rate: float, seed: int = 5):
    """Poisson stream of thermal solves through the continuous-batching
    server: binaries with a subdivision-3/4/5 primary (2,560 / 6,400 / 21,760
    facets, secondary subdivision 3), thermal inertia log-uniform in
    [10, 2000] SI, NX = 56, NTAU = 720, FAST precision.  Shapes are
    registered once (view factors, shadows and scattering on the device);
    requests arrive at exponential intervals of mean 1/rate."""
    from binarytpm_gb300 import lib, workloads

    rng = np.random.default_rng(seed)
    srv = lib.Server(ctx, precision=lib.FAST, nx=56, budget_bytes=48 << 30, max_active=48, revs_per_tick=4)
    shapes = {}
    for sub in (3, 4, 5):
        prob = workloads.binary_problem(ctx, p_subdiv=sub)
        shapes[sub] = (srv.add_shape(prob), prob.nf)
    subs = rng.choice([3, 4, 5], size=n_requests, p=[0.4, 0.35, 0.25])
    tis = np.exp(rng.uniform(np.log(10.0), np.log(2000.0), size=n_requests))
    gaps = rng.exponential(1.0 / rate, size=n_requests)
    t0 = time.perf_counter()
    rids = []
    for sub, ti, gap in zip(subs, tis, gaps):
        target = time.perf_counter() + gap
        while time.perf_counter() < target:
            time.sleep(min(0.001, max(0.0, target - time.perf_counter())))
        rids.append((srv.submit(shapes[sub][0], float(ti)), shapes[sub][0]))
    lats = []
    for rid, sid in rids:
        _, _, lat = srv.wait(rid, sid)
        lats.append(lat)
    wall = time.perf_counter() - t0
    st = srv.stats()
    srv.close()
    return {"requests": n_requests, "arrival_rate_per_s": rate, "p50_ms": 1e3 * float(np.percentile(lats, 50)),
            "p99_ms": 1e3 * float(np.percentile(lats, 99)), "facet_steps_per_s": st["facet_steps_per_s"],
            "wall_s": wall, "mix": {"subdiv3": int((subs == 3).sum()), "subdiv4": int((subs == 4).sum()),
                                    "subdiv5": int((subs == 5).sum())},
            "what": "continuous batching, HBM-budget admission, state resident on the device"}


FP64_TI = [200.0, 2000.0]
ACC_REVS = 40


def accuracy(ctx, prob, tis, shadow, illum):
    """FAST vs plain FP64 on the same schedule (workloads.fast_vs_fp64)."""
    from binarytpm_gb300 import workloads

    return workloads.fast_vs_fp64(ctx, prob, tis, ACC_REVS, shadow, illum)


def _tile_stats(prob, slices=False):
    """Tile structure of the FAST tensor-core product: 128x64 tiles touched,
    how many of them carry the residual (workloads.tc_tile_structure), and
    with ``slices`` the 128x16 K slices holding an entry (all tiles; residual
    tiles): the products the kernel issues."""
    from binarytpm_gb300 import workloads

    tiles, inv, sl, has_lo = workloads.tc_tile_structure(prob.nf, prob.dep_ptr, prob.dep_idx, prob.dep_vf)
    if not slices:
        return len(tiles), int(has_lo.sum())
    sk = np.unique(inv.astype(np.int64) * 4 + sl)
    return len(tiles), int(has_lo.sum()), len(sk), int(has_lo[sk // 4].sum())


def _roofline(kern, solves, prob, hbm, bf16, kind):
    """Dominant kernel of the revolution loop: the tensor-core self-heating
    product (k_spmm_tc).  Algorithmic FLOP per solve-revolution =
    2 * nnz * NTAU (the list sum); executed = every issued 128x16 K slice x
    step chunk x (2 or 3 BF16 products for the hi/lo compensation).  The conduction sweep
    is reported beside it: 20 B algorithmic HBM per facet-step."""
    out = {}
    k = kern.get("selfheat_q")
    n = len(solves)
    if k and k["ms"]:
        flops = 2.0 * prob.nnz * prob.ntau * n
        tiles, lo, sl, sl_lo = _tile_stats(prob, slices=True)
        ntau_pad = -(-prob.ntau // 144) * 144 if prob.ntau > 160 else -(-prob.ntau // 16) * 16
        exe = (2 * sl + sl_lo) * 128.0 * 16 * ntau_pad * 2 * n
        traffic = None
        tf = ROOT / "profiles" / "spmm_tc_traffic.json"
        if tf.exists():
            t = json.loads(tf.read_text())
            traffic = t["dram_bytes_per_tile_chunk"] * tiles * (ntau_pad // 144 if prob.ntau > 160 else 1) * n
        ach = flops / (k["ms"] / 1e3) / 1e12
        out = {"kernel": "k_spmm_tc", "bound": "tensor", "achieved": ach, "peak": bf16, "unit": "TFLOP/s",
               "frac": ach / bf16, "peak_kind": kind, "traffic": traffic, "algorithmic_flop": flops,
               "executed_tflops": exe / (k["ms"] / 1e3) / 1e12, "executed_frac": exe / (k["ms"] / 1e3) / 1e12 / bf16,
               "note": "algorithmic = 2 nnz NTAU; executed counts the zero padding of the issued 128x16 K "
                       f"slices ({sl} of the {4 * tiles} in {tiles} tiles; {sl_lo} in the {lo} tiles with "
                       "residual) and the hi/lo products"}
    c = kern.get("conduction")
    if c and c["ms"]:
        nx = solves[0].nx
        bytes_ = c["facet_steps"] * 20 + c["active_facets"] * 2 * (nx + 1) * 4
        gbs = bytes_ / (c["ms"] / 1e3) / 1e9
        traffic = None
        tf = ROOT / "profiles" / "conduction_fast_nx56_traffic.json"
        if tf.exists():
            traffic = json.loads(tf.read_text())["dram_bytes_per_facet_step"] * c["facet_steps"]
        flops = c["facet_steps"] * (5 * (nx - 1) + 20 * 2)
        out["conduction"] = {"kernel": "k_conduction<FAST,56,3>", "bound": "hbm", "achieved": gbs, "peak": hbm,
                             "unit": "GB/s", "frac": gbs / hbm, "traffic": traffic, "algorithmic_bytes": bytes_,
                             "fp32_tflops": flops / (c["ms"] / 1e3) / 1e12,
                             "note": "FP32-issue bound (about 230 instructions per facet-step at minimum)"}
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
    outs = [(lib.host_buffer((prob.nf, prob.ntau), np.float32), lib.host_buffer((prob.nf, prob.ntau), np.float32))
            for _ in tis]
    vals, h2d, d2h = [], 0, 0
    for _ in range(steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        s0 = lib.Solve(ctx, prob, precision=lib.FAST)
        s0.geometry_shadow()
        s0.scattering()
        # one prepared shape, cloned on the device for the other inertias
        solves = [s0] + [s0.clone() for _ in tis[1:]]
        for s, ti in zip(solves, tis):
            s.set_thermal_inertia(ti)
            s.initialise_temperatures()
        lib.batch_run(solves)
        fs = solves[0].last_run_stats()[2]
        temps = [s.surface_temperature(out=o) for s, o in zip(solves, outs)]
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        vals.append(fs / dt)
        shape_bytes = prob.vertices.nbytes + prob.facets.nbytes + prob.dep_ptr.nbytes + prob.dep_idx.nbytes + prob.dep_vf.nbytes
        h2d = shape_bytes
        d2h = sum(t[0].nbytes + t[1].nbytes for t in temps)
        for s in solves:
            s.close()
    return {"value": statistics.median(vals), "unit": UNIT, "h2d_bytes_per_step": int(h2d),
            "d2h_bytes_per_step": int(d2h),
            "what": "C-ABI job from host arrays: solve create (H2D), geometry+shadowing+scattering, "
                    "device clones for the other inertias, batched revolution loop, temperatures D2H; "
                    "inputs and read-back buffers page-locked, allocated once before the timed jobs"}


if __name__ == "__main__":
    main()
