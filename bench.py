#!/usr/bin/env python
"""Benchmark: ms per solve to 1e-10 relative residual on one GB300.

Headline workload (the reference's configuration 2): 4096^2 vertex-centred
2D 9-point masked Laplacian, F-cycle, Jacobi 3/3 (omega 0.8), smoothed-noise
coastline with 30 % land, N(0,1) right-hand side with the wet mean removed
(tests/workloads.py), run with 5 levels: the configuration names 10, and
with 6 or more the reference algorithm's F-cycle diverges on this coastline
(tests/golden/config2_levels.json; the bench also records the FP64 residual
history of a few 10-level cycles). One step = one solve from x = 0 to
||r||_2/||b||_2 <= 1e-10. `value` is the mixed-precision form (FP32 cycles
inside FP64 defect correction); the plain FP64 drop-in is timed beside it.

The default run also times the other configurations, each in a short
sub-run reported under "workloads": config 1 (256^2 cell-centred 5-point,
the plain FP64 method and the mixed form, with the single-thread CPU oracle
beside them), config 3 (512 x 512 x 256 cell-centred 7-point), config 4
(2048 batched solves of uneven sizes in one graph launch) and config 5
(16 forward + adjoint variable-coefficient solves with a finite-difference
check). --headline-only skips them.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

The reference arm (--impl reference) times the CPU restatement of the
reference (oracle/, OpenMP over all host cores; the Julia reference cannot
run on this machine) on the same workload and prints the same JSON line.
With N > 1 (torchrun), every rank solves its own replica (replicas only:
the path has no data exchange between independent solves), and `value` is
the time per solve amortised over the N replicas.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
for _p in (os.path.join(ROOT, "cfmultigrid.jl_gb300"), os.path.join(ROOT, "tests")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = "ms/solve to 1e-10 rel residual (mixed FP32-in-FP64), 4096^2 vertex 9-point F-cycle"
UNIT = "ms/solve"
TOL = 1e-10
MAXITE = 60


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=None,
                    help="timed steps (default 30 for our config-2 arm, about 0.4 s, so that the clock sampler "
                         "sees the region; 5 otherwise)")
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", type=int, default=4096, help="grid size (4096 = the configuration)")
    ap.add_argument("--nlevels", type=int, default=0, help="levels (0: the deepest hierarchy that converges, 5)")
    ap.add_argument("--cpu-seconds", type=float, default=12.0, help="budget of the single-thread CPU sample")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--workload", default="config2", choices=["config1", "config2", "config3", "config4", "config5"],
                    help="config1: the plain-method 256^2 case; config3: the 3D 7-point case; config4: batched "
                         "solves of uneven sizes (one graph launch per batch); config5: forward + adjoint solves")
    ap.add_argument("--ninst", type=int, default=2048, help="config4 batch size")
    ap.add_argument("--no-tune", action="store_true", help="config4: F(2,2) without the autotuner")
    ap.add_argument("--fd-dirs", type=int, default=64, help="config5: finite-difference directions")
    ap.add_argument("--host-loop", action="store_true",
                    help="the host repeats the solve iteration instead of one graph launch per solve (for the "
                         "ncu launch list, which does not descend into conditional graph nodes)")
    ap.add_argument("--quick", action="store_true",
                    help="mixed form only: one warm-up and one timed solve (a short run for ncu)")
    ap.add_argument("--headline-only", action="store_true",
                    help="time configuration 2 only (no sub-runs of configurations 1, 3, 4 and 5)")
    # --quick only: the earlier default forms, for ncu captures of their kernels
    ap.add_argument("--tb", type=int, default=None, choices=[0, 1, 3, 5],
                    help="--quick: FP32 smoothing form (temporal_blocking option; 5 is the default)")
    ap.add_argument("--no-int", action="store_true", help="--quick: level-1 residual in FP64 arithmetic")
    ap.add_argument("--no-fuse", action="store_true",
                    help="--quick: no fused descent or fused solution update (plain smoothing passes)")
    ap.add_argument("--fp64", action="store_true",
                    help="--quick: the FP64 drop-in instead of the mixed form (for ncu captures of its kernels)")
    args = ap.parse_args()
    if (args.tb is not None or args.no_int or args.no_fuse or args.fp64) and not (
            args.quick and args.workload == "config2"):
        ap.error("--tb, --no-int, --no-fuse and --fp64 go with --quick (config 2) only")
    if args.steps is None:
        args.steps = 30 if (args.impl == "ours" and args.workload == "config2") else 5
    return args


# ------------------------------------------------------------ distributed
def dist_init():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch
        import torch.distributed as dist

        backend = "nccl" if torch.cuda.is_available() else "gloo"
        dist.init_process_group(backend)
    return rank, world, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist

        dist.barrier()


def max_over_ranks(v: float, world: int) -> float:
    """Max of a float over all ranks (identity when world == 1)."""
    if world == 1:
        return v
    import torch
    import torch.distributed as dist

    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([v], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# ------------------------------------------------------------------ clocks
class Clocks:
    """nvidia-smi sampling of SM clock and throttle reasons during a region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        # the timed region starts once the sampler runs: its start-up (NVML
        # initialisation) stalled the GPU work of a region it overlapped
        # (5 config-2 solves: 23.9 against 13.5 ms per solve)
        t0 = time.time()
        while self.proc is not None and self.proc.poll() is None and time.time() - t0 < 3.0:
            if os.path.getsize(self.path) > 0:
                break
            time.sleep(0.02)
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        rows = []
        if self.path and os.path.exists(self.path):
            for line in open(self.path):
                f = [x.strip() for x in line.split(",")]
                if len(f) >= 9:
                    rows.append(f)
            os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


# ------------------------------------------------------------- our arm
def make_gmg(cfmg, param, vmsk, noise, precision, stream_ptr, tol=TOL, maxite=MAXITE):
    import workloads as W

    p = cfmg.Param(**param, tol=tol, maxite=maxite, residual_norm="l2", precision=precision, verbose=False)
    mg = cfmg.get_gmg(p)
    mg.set_stream(stream_ptr)
    mg.oper[1].msk = vmsk
    cfmg.setup_operators(mg)
    for lev in range(1, mg.nlevels + 1):
        for f in ("b", "x", "y", "r"):
            cfmg.set_to_zero(mg, lev, f)
    b = W.rhs(noise, mg.download(1, "msk"))
    mg.data[1].b = b
    return mg, b


def launch_count(cfmg, mg):
    import ctypes

    n = ctypes.c_longlong()
    mg._check(mg._L.cfmg_launch_count(mg.handle, ctypes.byref(n)))
    return n.value


def profile(cfmg, mg, cls, lev, precision, fn):
    import ctypes

    L = mg._L
    mg._check(L.cfmg_profile(mg.handle, cfmg._lib.KERNEL_CLASSES[cls], lev, cfmg._lib.PRECISIONS[precision]))
    fn()
    n = ctypes.c_longlong()
    ms = ctypes.c_double()
    mg._check(L.cfmg_profile_read(mg.handle, ctypes.byref(n), ctypes.byref(ms)))
    mg._check(L.cfmg_profile(mg.handle, -1, 0, 0))
    return n.value, ms.value


def config2_config(n: int, levels: int, world: int) -> dict:
    """The `config` of the headline line: the same dict in both arms."""
    fine = (n + 6) ** 2
    return {"workload": f"config2: {n}^2 vertex-centred 2D 9-point masked Laplacian, F-cycle, {levels} levels "
                        f"(10 diverge with the reference algorithm), Jacobi 3/3, omega 0.8, 30% land",
            "levels": levels, "fine_cells": fine, "tol_l2": TOL,
            "l2_flush": "inputs larger than L2 (level-1 FP64 field = %.0f MB)" % (fine * 8 / 1e6),
            "parallelism": f"replicas x{world}"}


def metric_for(world: int) -> str:
    return METRIC if world == 1 else METRIC + f", amortised over {world} replicas"


def hbm_peak():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        return float(json.load(open(path))["hbm_gbs"]), "measured (MEASURED_PEAKS.json hbm_gbs)"
    return 6800.0, "fallback 6.8 TB/s"


def ncu_traffic(key: str):
    """DRAM bytes of one launch (dram__bytes_read.sum + dram__bytes_write.sum)
    from the ncu captures summarised in profiles/roofline_traffic.json."""
    tpath = os.path.join(ROOT, "profiles", "roofline_traffic.json")
    if not os.path.exists(tpath):
        return None, None
    e = json.load(open(tpath)).get(key)
    return (e["bytes"], e["capture"]) if e else (None, None)


def run_ours(args, rank, world, local):
    import numpy as np
    import torch

    import cfmg
    import workloads as W

    torch.cuda.set_device(local)
    stream = torch.cuda.Stream()
    sp = stream.cuda_stream
    param, vmsk, noise = W.config2(args.n, nlevels=args.nlevels or W.CONFIG2_LEVELS)
    mgm, b = make_gmg(cfmg, param, vmsk, noise, "fp64" if args.fp64 else "mixed", sp)
    if args.host_loop:
        mgm.set_option("host_loop", 1)
    if args.tb is not None:
        mgm.set_option("temporal_blocking", args.tb)
    if args.no_int:
        mgm.set_option("int_residual", 0)
    if args.no_fuse:
        mgm.set_option("fused_descent", 0)
        mgm.set_option("fused_update", 0)
    if args.quick:
        cfmg.set_to_zero(mgm, 1, "x")
        cfmg.solve(mgm)
        cfmg.set_to_zero(mgm, 1, "x")
        torch.cuda.synchronize()
        t = time.perf_counter()
        res, nit = cfmg.solve(mgm)
        return {"quick": True, "ms": (time.perf_counter() - t) * 1e3, "cycles": nit, "res": res}
    mgd, _ = make_gmg(cfmg, param, vmsk, noise, "fp64", sp)

    def solve(mg):
        cfmg.set_to_zero(mg, 1, "x")
        return cfmg.solve(mg)

    # warm-up (graph capture happens in the first solve)
    for _ in range(max(args.warmup, 3)):
        res_m, nit_m = solve(mgm)
    barrier(world)
    torch.cuda.synchronize()
    n0 = launch_count(cfmg, mgm)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with Clocks(local) as clk:
        e0.record(stream)
        for _ in range(args.steps):
            res_m, nit_m = solve(mgm)
        e1.record(stream)
        e1.synchronize()
    torch.cuda.synchronize()
    barrier(world)
    ms_mixed = e0.elapsed_time(e1) / args.steps
    launches = launch_count(cfmg, mgm) - n0
    clocks = clk.summary()
    x_mixed = mgm.download(1, "x")

    # the same mixed form with the coarsest level forced to FP64
    mgm.set_option("coarsest_fp64", 1)
    solve(mgm)
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(args.steps):
        res_c64, nit_c64 = solve(mgm)
    e1.record(stream)
    e1.synchronize()
    ms_mixed_c64 = e0.elapsed_time(e1) / args.steps
    mgm.set_option("coarsest_fp64", -1)

    # plain FP64 drop-in, same workload
    res_d, nit_d = solve(mgd)
    k64 = max(1, min(args.steps, 3))
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(k64):
        res_d, nit_d = solve(mgd)
    e1.record(stream)
    e1.synchronize()
    ms_fp64 = e0.elapsed_time(e1) / k64
    x_fp64 = mgd.download(1, "x")
    wet = mgm.download(1, "msk").astype(bool)
    err = float(np.linalg.norm((x_mixed - x_fp64)[wet]) / np.linalg.norm(x_fp64[wet]))

    # end to end through the C ABI with host buffers: b in from pinned host
    # memory, solve, x out to pinned host memory, every step
    hb = torch.from_numpy(np.ascontiguousarray(b.ravel(order="F"))).pin_memory()
    hx = torch.empty_like(hb).pin_memory()
    nbytes = hb.numel() * 8
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    e0.record(stream)
    for _ in range(args.steps):
        mgm.upload_ptr(1, "b", hb.data_ptr())
        cfmg.set_to_zero(mgm, 1, "x")
        cfmg.solve(mgm)
        mgm.download_ptr(1, "x", hx.data_ptr())
    e1.record(stream)
    e1.synchronize()
    wall_e2e = (time.perf_counter() - t0) * 1e3 / args.steps
    ms_e2e = e0.elapsed_time(e1) / args.steps

    # Per-launch device times of the level-1 blocked passes, with CUDA events
    # on the library's stream during one default solve (cfmg_profile). The
    # dominant kernel of the default solve is the fused descent pass of
    # level 1: 3 Jacobi pairs, then the residual of its core, restricted to
    # level 2's b, and level 2's x zeroed. Its algorithmic bytes: FP32 x, b,
    # omega*idiag and diag read and x written (20 B) and the mask (1 B) per
    # fine cell of the update box, Rcoef read, b and x written (12 B) per
    # coarse cell. The post-smoothing pass with the FP64 solution update
    # reads FP32 x, b, omega*idiag and the FP64 x and writes the FP64 x
    # (28 B per cell); the plain pass (measured with the update taken out)
    # reads FP32 x, b, omega*idiag and writes x (16 B per cell).
    peak, peak_src = hbm_peak()
    g1, g2 = mgm.levels[1], mgm.levels[2]
    box_cells = (g1.nx + 2) * (g1.ny + 2) * g1.nz  # the update box U = [nh, nx+nh+1]^2
    coarse_cells = g2.nx * g2.ny * g2.nz
    nld, tld = profile(cfmg, mgm, "descent", 1, "mixed", lambda: solve(mgm))
    nlu, tlu = profile(cfmg, mgm, "sweep", 1, "mixed", lambda: solve(mgm))
    mgm.set_option("fused_update", 0)
    nlp, tlp = profile(cfmg, mgm, "sweep", 1, "mixed", lambda: solve(mgm))
    mgm.set_option("fused_update", 1)

    def rate(nbytes_, n, t):
        ms = t / max(n, 1)
        gbs = nbytes_ / (ms * 1e-3) / 1e9 if ms > 0 else 0.0
        return ms, gbs

    bytes_descent = 21.0 * box_cells + 12.0 * coarse_cells
    ms_descent, ach_descent = rate(bytes_descent, nld, tld)
    bytes_update = 28.0 * box_cells
    ms_update, ach_update = rate(bytes_update, nlu, tlu)
    bytes_plain = 16.0 * box_cells
    ms_plain, ach_plain = rate(bytes_plain, nlp, tlp)
    key = f"config2 {args.n} level 1"
    tr_d, cap_d = ncu_traffic(f"k_smooth_tb5<9,3,EPI> {key}") if args.n == 4096 else (None, None)
    tr_u, _ = ncu_traffic(f"k_smooth_tb5<9,3,UPD> {key}") if args.n == 4096 else (None, None)
    tr_p, _ = ncu_traffic(f"k_smooth_tb5<9,3> {key}") if args.n == 4096 else (None, None)
    # FP64 sweep of the drop-in: FP64-issue bound, reported beside it
    nl64, tl64 = profile(cfmg, mgd, "sweep", 1, "fp64", lambda: solve(mgd))
    ms_launch64, ach64 = rate(32.0 * box_cells, nl64, tl64)

    # The configuration's own 10 levels in the FP64 drop-in: the residual
    # history of its first cycles (the reference algorithm diverges there)
    mgd.close()
    p10 = dict(param, nlevels=10)
    mg10, _ = make_gmg(cfmg, p10, vmsk, noise, "fp64", sp, tol=0.0, maxite=4)
    _, _, h10 = cfmg.solve(mg10, history=True)
    mg10.close()
    levels10 = {"levels": 10, "cycles": len(h10) - 1, "hist_l2": [float(v) for v in h10],
                "factors": [float(h10[k] / h10[k - 1]) for k in range(1, len(h10))],
                "note": "FP64 drop-in, F-cycle 3/3 from x = 0 with the configuration's 10 levels"}

    ms_mixed = max_over_ranks(ms_mixed, world)
    ms_e2e = max_over_ranks(ms_e2e, world)
    out = {
        "metric": metric_for(world), "value": ms_mixed / world, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": max(args.warmup, 3), "ms_per_step": ms_mixed, "higher_is_better": False,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32-in-f64",
        "data": "synthetic (seeded coastline mask, N(0,1) rhs)",
        "config": config2_config(args.n, mgm.nlevels, world),
        "cycles_mixed": nit_m, "res_mixed": res_m, "cycles_fp64": nit_d, "res_fp64": res_d,
        "ms_per_solve_fp64": ms_fp64, "mixed_speedup_vs_fp64": ms_fp64 / ms_mixed,
        "mixed_coarsest_fp64": {"ms_per_solve": ms_mixed_c64, "cycles": nit_c64, "res": res_c64,
                                "note": "coarsest-level smoothing in FP64 (the default runs it in FP32 "
                                        "when the coarsest level exceeds 1250 cells)"},
        "mixed_rel_err_vs_fp64": err,
        "e2e": {"value": ms_e2e / world, "unit": UNIT, "h2d_bytes_per_step": nbytes, "d2h_bytes_per_step": nbytes,
                "wall_ms_per_step": wall_e2e},
        "gpu_launches": launches,
        "roofline": {"kernel": "k_smooth_tb5<9,3,EPI>: level-1 fused descent pass (6 Jacobi sweeps, residual, "
                               "its restriction to level 2, level-2 x zeroed)",
                     "bound": "hbm", "achieved": ach_descent, "peak": peak, "unit": "GB/s",
                     "frac": ach_descent / peak, "peak_source": peak_src, "traffic": tr_d,
                     "traffic_source": cap_d, "launches_timed": nld, "ms_per_launch": ms_descent,
                     "bytes_per_launch": bytes_descent},
        "level1_passes": {
            "update": {"kernel": "k_smooth_tb5<9,3,UPD>: level-1 post-smoothing pass with the FP64 solution "
                                 "update and max |x|", "launches_timed": nlu, "ms_per_launch": ms_update,
                       "bytes_per_launch": bytes_update, "achieved_gbs": ach_update, "frac": ach_update / peak,
                       "traffic": tr_u},
            "plain": {"kernel": "k_smooth_tb5<9,3>: the same post-smoothing pass without the update (not run "
                                "at level 1 by the default solve)", "launches_timed": nlp,
                      "ms_per_launch": ms_plain, "bytes_per_launch": bytes_plain, "achieved_gbs": ach_plain,
                      "frac": ach_plain / peak, "traffic": tr_p,
                      "effective_sweep_gbs": ach_plain * 2 * min(param["npre"], 3)},
        },
        "roofline_fp64_sweep": {"kernel": "FP64 9-point Jacobi sweep, level 1 (drop-in)", "ms_per_launch": ms_launch64,
                                "effective_gbs": ach64, "bound": "fp64 issue (DADD/DMUL at 506 Gop/s measured)"},
        "levels10_fp64": levels10,
        "clocks": clocks,
    }
    mgm.close()
    if rank == 0 and world == 1 and not args.no_cpu:
        out["cpu_baseline"] = cpu_baseline(param, vmsk, noise, nit_d, args.cpu_seconds)
    if world == 1 and not args.headline_only:
        out["workloads"] = {}
        for name, fn in (("config1", bench_config1), ("config3", bench_config3), ("config4", bench_config4),
                         ("config5", bench_config5)):
            t0 = time.perf_counter()
            try:
                out["workloads"][name] = fn(args, local, sub=True)
            except Exception as e:  # a sub-run that fails is reported, the headline stands
                out["workloads"][name] = {"error": f"{type(e).__name__}: {e}"}
            out["workloads"][name]["wall_s"] = time.perf_counter() - t0
            torch.cuda.empty_cache()
    return out


# -------------------------------------------------------------- CPU side
def _oracle_setup(param, vmsk, noise):
    import oracle as O
    import workloads as W

    p = dict(param, tol=TOL, maxite=MAXITE)
    og = O.OracleGmg(p)
    og.field(1, "msk")[...] = vmsk
    og.setup_operators()
    for lev in range(1, og.nlevels + 1):
        for f in ("x", "y", "r", "b"):
            og.field(lev, f)[...] = 0.0
    og.field(1, "b")[...] = W.rhs(noise, og.field(1, "msk"))
    return og


def cpu_baseline(param, vmsk, noise, cycles_needed, budget_s):
    """The single-thread oracle (the reference's PlainCPU arithmetic) on a
    bounded sample: full-size F-cycles + residual norms until the budget is
    spent, scaled to one solve of `cycles_needed` cycles."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    os.environ["CFMG_ORACLE_THREADS"] = "1"
    og = _oracle_setup(param, vmsk, noise)
    t0 = time.perf_counter()
    normb = og.norm(1, "b")
    og.normresidual(normb)
    t_head = time.perf_counter() - t0
    times = []
    while len(times) < cycles_needed and sum(times) < budget_s:
        t = time.perf_counter()
        og.cycle("f")
        og.normresidual(normb)
        times.append(time.perf_counter() - t)
    per = sum(times) / len(times)
    ms = (t_head + per * cycles_needed) * 1e3
    return {"value": ms, "unit": UNIT, "cores": 1, "kind": "port",
            "sample": f"{len(times)} of {cycles_needed} full-size F-cycles (+ residual norm) timed, "
                      f"scaled to one solve; single thread, FP64, oracle restatement of the reference"}


def run_reference(args, rank, world):
    """Reference arm: the CPU restatement (OpenMP, all host cores), full
    solves of the same workload to the same tolerance."""
    if rank != 0:
        return None
    cores = os.cpu_count() or 1
    os.environ["CFMG_ORACLE_THREADS"] = str(cores)
    os.environ.setdefault("OMP_NUM_THREADS", str(cores))
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import workloads as W

    param, vmsk, noise = W.config2(args.n, nlevels=args.nlevels or W.CONFIG2_LEVELS)
    og = _oracle_setup(param, vmsk, noise)

    def one():
        og.field(1, "x")[...] = 0.0
        t = time.perf_counter()
        r = solve_l2(og)
        return time.perf_counter() - t, r

    for _ in range(args.warmup):
        one()
    ts = []
    for _ in range(args.steps):
        dt, (res, nite) = one()
        ts.append(dt)
    ms = sum(ts) / len(ts) * 1e3
    return {"metric": metric_for(world), "value": ms, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": False, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded coastline mask, N(0,1) rhs)",
            "impl": "reference", "config": config2_config(args.n, og.nlevels, world),
            "cycles": nite, "res": res,
            "cpu_baseline": {"value": ms, "unit": UNIT, "cores": cores, "kind": "port",
                             "sample": "full FP64 solves with the oracle restatement of the reference "
                                       f"(OpenMP, {cores} threads); Julia is not installed on this box"},
            "e2e": {"value": ms, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def solve_l2(og):
    """solve! with the ||r||/||b|| <= TOL rule (the reference's loop,
    src/gmg_solver.jl:9-42, on the square root of its ratio)."""
    normb = og.norm(1, "b")
    res = og.normresidual(normb) ** 0.5
    nite = 0
    while res > TOL and nite < MAXITE:
        nite += 1
        og.cycle("f")
        res = og.normresidual(normb) ** 0.5
    return res, nite


def _timed(stream, fn, steps):
    """Device time per call of fn() (CUDA events on `stream`), and its last result."""
    import torch

    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(steps):
        r = fn()
    e1.record(stream)
    e1.synchronize()
    return e0.elapsed_time(e1) / steps, r


def bench_config1(args, local, sub=False):
    """Configuration 1, the plain method: 256^2 cell-centred 5-point masked
    Poisson, disk of radius 0.45 N, seed-0 N(0,1) right-hand side, V-cycle
    2/2, 6 levels, omega 0.8, to 1e-10. The FP64 drop-in (the reference's
    arithmetic, bit for bit) is the config's own method; the mixed form is
    timed beside it, and the single-thread CPU oracle solve of the same
    problem is the CPU baseline."""
    import numpy as np
    import torch

    import cfmg
    import workloads as W

    torch.cuda.set_device(local)
    stream = torch.cuda.Stream()
    sp = stream.cuda_stream
    param, msk, noise = W.config1()
    steps = 20 if sub else args.steps
    out = {}
    for prec in ("fp64", "mixed"):
        mg, b = make_gmg(cfmg, param, msk, noise, prec, sp)

        def solve(mg=mg):
            cfmg.set_to_zero(mg, 1, "x")
            return cfmg.solve(mg)

        for _ in range(max(args.warmup, 3)):
            solve()
        ms, (res, nit) = _timed(stream, solve, steps)
        out[prec] = {"ms_per_solve": ms, "cycles": nit, "res": res, "x": mg.download(1, "x")}
        mg.close()
    wet = msk.astype(bool)
    xd, xm = out["fp64"].pop("x"), out["mixed"].pop("x")
    err = float(np.linalg.norm((xm - xd)[wet]) / np.linalg.norm(xd[wet]))
    cpu = None
    if not args.no_cpu:  # the single-thread oracle's full FP64 solve of the same problem
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        os.environ["CFMG_ORACLE_THREADS"] = "1"
        og = _oracle_setup(param, msk, noise)
        t = time.perf_counter()
        normb = og.norm(1, "b")
        res = og.normresidual(normb) ** 0.5
        nite = 0
        while res > TOL and nite < MAXITE:
            nite += 1
            og.cycle("v")
            res = og.normresidual(normb) ** 0.5
        cpu = {"value": (time.perf_counter() - t) * 1e3, "unit": UNIT, "cores": 1, "kind": "port",
               "sample": f"one full FP64 solve ({nite} V-cycles), single thread, oracle restatement of the "
                         "reference"}
    return {"metric": "ms/solve to 1e-10 rel residual, 256^2 cell-centred 5-point V-cycle (FP64 drop-in)",
            "value": out["fp64"]["ms_per_solve"], "unit": UNIT, "higher_is_better": False, "dtype": "f64",
            "steps": steps, "data": "synthetic (disk mask r = 0.45 N, N(0,1) rhs from seed 0)",
            "config": {"workload": "config1: 256^2 cell-centred 2D 5-point masked Poisson, V-cycle 2/2, 6 levels, "
                                   "omega 0.8", "levels": param["nlevels"], "tol_l2": TOL,
                       "l2_flush": "none (level-1 FP64 field = 0.55 MB, L2-resident)"},
            "fp64": out["fp64"], "mixed": out["mixed"], "mixed_rel_err_vs_fp64": err, "cpu_baseline": cpu}


def bench_config3(args, local, sub=False):
    """Configuration 3: 512 x 512 x 256 cell-centred 7-point masked Poisson
    (coastline extruded in z, cut by a bottom topography), V-cycle,
    8 levels, Jacobi 2/2, solved to ||r||/||b|| <= 1e-9 in the mixed form and
    in the FP64 drop-in (whose pointwise arithmetic is the reference's, bit
    for bit); the mixed solution's error against the FP64 one is reported."""
    import numpy as np
    import torch

    import cfmg
    import workloads as W

    torch.cuda.set_device(local)
    stream = torch.cuda.Stream()
    sp = stream.cuda_stream
    tol = 1e-9
    n = args.n if (args.n != 4096 and not sub) else 512
    param, msk, noise = W.config3(n, n, n // 2, nlevels=(args.nlevels if not sub else 0) or 8)
    mgm, b = make_gmg(cfmg, param, msk, noise, "mixed", sp, tol=tol, maxite=400)
    if args.host_loop and not sub:
        mgm.set_option("host_loop", 1)

    def solve(mg):
        cfmg.set_to_zero(mg, 1, "x")
        return cfmg.solve(mg)

    if args.quick and not sub:
        solve(mgm)
        torch.cuda.synchronize()
        t = time.perf_counter()
        res, nit = solve(mgm)
        return {"quick": True, "ms": (time.perf_counter() - t) * 1e3, "cycles": nit, "res": res}
    level_cells = [g.tx * g.ty * g.tz for g in mgm.levels]
    steps = 3 if sub else args.steps
    for _ in range(max(args.warmup, 3)):
        solve(mgm)
    n0 = launch_count(cfmg, mgm)
    with Clocks(local) as clk:
        ms_mixed, (res_m, nit_m) = _timed(stream, lambda: solve(mgm), steps)
    launches = (launch_count(cfmg, mgm) - n0) // steps
    x_mixed = mgm.download(1, "x")

    mgd, _ = make_gmg(cfmg, param, msk, noise, "fp64", sp, tol=tol, maxite=400)
    solve(mgd)
    ms_fp64, (res_d, nit_d) = _timed(stream, lambda: solve(mgd), 1)
    x_fp64 = mgd.download(1, "x")
    mgd.close()
    wet = mgm.download(1, "msk").astype(bool)
    err = float(np.linalg.norm((x_mixed - x_fp64)[wet]) / np.linalg.norm(x_fp64[wet]))

    hb = torch.from_numpy(np.ascontiguousarray(b.ravel(order="F"))).pin_memory()
    hx = torch.empty_like(hb).pin_memory()
    nbytes = hb.numel() * 8

    def e2e():
        mgm.upload_ptr(1, "b", hb.data_ptr())
        cfmg.set_to_zero(mgm, 1, "x")
        cfmg.solve(mgm)
        mgm.download_ptr(1, "x", hx.data_ptr())

    ms_e2e, _ = _timed(stream, e2e, steps)

    # roofline: the level-1 FP32 7-point Jacobi sweep of the mixed form. A
    # sweep moves 13 B a cell (x, b and y as FP32, omega*idiag as a one-byte
    # code); the first sweep of each cycle takes x as +0 without reading it
    # (9 B a cell)
    got = {}

    def solve_n():
        got["r"] = solve(mgm)

    nl, tl = profile(cfmg, mgm, "sweep", 1, "mixed", solve_n)
    ncyc = got["r"][1]
    g1 = mgm.levels[1]
    sweep_cells = g1.tx * g1.ty * (g1.tz - 2)  # linear range 1+tx*ty : len-tx*ty
    # the sweep skips quads (4 consecutive cells of a plane) that are dry in
    # every plane of their run of 4 planes: count the cells it does sweep
    n2 = g1.tx * g1.ty
    wet = mgm.download(1, "msk").ravel(order="F").reshape(g1.tz, n2)[1:g1.tz - 1] != 0
    wq = wet.reshape(g1.tz - 2, n2 // 4, 4).any(axis=2)
    swept = 0
    for r0 in range(0, g1.tz - 2, 4):
        swept += int(wq[r0:r0 + 4].any(axis=0).sum()) * 4 * min(4, g1.tz - 2 - r0)
    ms_launch = tl / max(nl, 1)
    peak, peak_src = hbm_peak()
    nzero = min(ncyc, nl)
    bytes_per_launch = swept * (13.0 * (nl - nzero) + 9.0 * nzero) / max(nl, 1)
    achieved = bytes_per_launch / (ms_launch * 1e-3) / 1e9 if ms_launch > 0 else 0.0
    # the fixed-point level-1 residual pass (TMA-staged): x, b (FP64) and
    # Q*diag (one byte) read, the FP32 right-hand side written: 21 B a cell,
    # counted over the (32 x 16 tile, plane) pairs that hold a wet cell (the
    # pass skips runs of planes that are all dry, so this is a lower bound of
    # the cells it covers)
    nr, trr = profile(cfmg, mgm, "residual", 1, "fp64", lambda: solve(mgm))
    nh = g1.nh
    box = mgm.download(1, "msk")[nh:nh + n, nh:nh + n, nh:nh + n // 2] != 0
    ti, tj = -(-n // 32), -(-n // 16)
    pad = np.zeros((ti * 32, tj * 16, n // 2), dtype=bool)
    pad[:n, :n] = box
    wet_tp = pad.reshape(ti, 32, tj, 16, n // 2).any(axis=(1, 3))  # (tile i, tile j, plane)
    interior = int(wet_tp.sum()) * 32 * 16
    ms_r = trr / max(nr, 1)
    bytes_r = 21.0 * interior
    ach_r = bytes_r / (ms_r * 1e-3) / 1e9 if ms_r > 0 else 0.0
    mgm.close()
    return {"metric": f"ms/solve to 1e-9 rel residual (mixed FP32-in-FP64), {n}x{n}x{n // 2} cell-centred "
                      "7-point V-cycle",
            "value": ms_mixed, "unit": UNIT, "n_gpus": 1, "steps": steps, "warmup": max(args.warmup, 3),
            "ms_per_step": ms_mixed, "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32-in-f64", "data": "synthetic (seeded coastline x bottom-topography mask, N(0,1) rhs)",
            "config": {"workload": f"config3: {n}x{n}x{n // 2} cell-centred 3D 7-point masked Poisson, V-cycle, "
                                   f"{len(level_cells)} levels, Jacobi 2/2, omega 0.8",
                       "levels": len(level_cells), "fine_cells": level_cells[0], "tol_l2": tol,
                       "l2_flush": "inputs larger than L2 (level-1 FP64 field = %.0f MB)" % (level_cells[0] * 8 / 1e6),
                       "parallelism": "replicas x1"},
            "cycles_mixed": nit_m, "res_mixed": res_m, "cycles_fp64": nit_d, "res_fp64": res_d,
            "ms_per_solve_fp64": ms_fp64, "mixed_speedup_vs_fp64": ms_fp64 / ms_mixed,
            "mixed_rel_err_vs_fp64": err,
            "e2e": {"value": ms_e2e, "unit": UNIT, "h2d_bytes_per_step": nbytes, "d2h_bytes_per_step": nbytes},
            "gpu_launches": launches,
            "roofline": {"kernel": "k_sweep7_3d_q4: FP32 7-point Jacobi sweep, level 1 (13 B a swept cell, 9 for "
                                   "each cycle's first sweep; dry quads skipped)", "bound": "hbm",
                         "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                         "peak_source": peak_src, "traffic": None, "launches_timed": nl, "ms_per_launch": ms_launch,
                         "bytes_per_launch": bytes_per_launch, "cells_swept": swept, "cells_in_range": sweep_cells},
            "roofline_residual": {"kernel": "k_resid_int3d: TMA-staged fixed-point level-1 residual (with its "
                                            "one-block final reduction); 21 B a cell over the wet (32x16 tile, "
                                            "plane) pairs", "bound": "hbm", "achieved": ach_r,
                                  "peak": peak, "unit": "GB/s", "frac": ach_r / peak, "launches_timed": nr,
                                  "ms_per_launch": ms_r, "bytes_per_launch": bytes_r},
            "clocks": clk.summary()}


def bench_config4(args, local, sub=False):
    """Configuration 4: 2048 independent 2D cell-centred 5-point masked
    solves (sizes log-uniform 64^2..1024^2, disk or noise masks) to 1e-10 in
    one graph launch of the batched solver; the schedule and the tile form of
    the blocked passes are picked by the autotuner on a stratified sample.
    Reports the batch time and the p50/p99 of the per-instance completion
    time (device clock)."""
    import numpy as np
    import torch

    import cfmg
    from cfmg import autotune
    import fixtures as F
    import workloads as W

    torch.cuda.set_device(local)
    t0 = time.perf_counter()
    probs = W.config4(args.ninst if not sub else 2048)
    t_gen = time.perf_counter() - t0
    sizes = [q[0] for q in probs]
    # the slowest noise-coastline instances contract by ~0.8 per V-cycle
    # (CPU oracle): 1e-10 takes up to ~110 cycles
    base = cfmg.Param(nx=64, ny=64, nz=1, case="twod", location="centers", operator="laplacian", cycle="v",
                      npre=2, npost=2, omega=0.8, ndeepest=20, tol=TOL, maxite=200, residual_norm="l2",
                      precision="mixed", verbose=False)

    def make(p, idx):
        batch = cfmg.Batch(p, [probs[i][0] for i in idx], [probs[i][0] for i in idx], [probs[i][1] for i in idx])
        for k, i in enumerate(idx):
            g = batch.instance(k)
            g.oper[1].msk = probs[i][2]
            cfmg.setup_operators(g)
            for lev in range(1, g.nlevels + 1):
                for f in ("b", "x", "y", "r"):
                    cfmg.set_to_zero(g, lev, f)
            m = g.download(1, "msk").astype(np.float64)
            bb = np.asfortranarray(probs[i][3] * m)
            F.subtract_mean(bb, m)
            g.data[1].b = bb
        return batch

    t0 = time.perf_counter()
    if args.no_tune and not sub:
        p, report = dataclasses_replace(base, cycle="f"), {"skipped": True}
    else:
        p, report = autotune.tune(base, sizes, make)
    t_tune = time.perf_counter() - t0
    t0 = time.perf_counter()
    batch = make(p, list(range(len(probs))))
    autotune.apply_form(batch, report.get("form", autotune.DEFAULT_FORM))
    if args.host_loop and not sub:
        batch.set_option("host_loop", 1)
    t_setup = time.perf_counter() - t0
    steps = 2 if sub else args.steps
    for _ in range(max(args.warmup, 3)):
        batch.solve()
    torch.cuda.synchronize()
    times, dones = [], []
    with Clocks(local) as clk:
        for _ in range(steps):
            t = time.perf_counter()
            res, nite, tdone = batch.solve()
            times.append((time.perf_counter() - t) * 1e3)
            dones.append(tdone)
    batch.close()
    ms = float(np.mean(times))
    td = np.concatenate(dones)
    cells = int(sum((n + 6) ** 2 for n in sizes))
    return {"metric": f"ms per batch of {len(probs)} masked solves to 1e-10 (mixed, one graph launch)",
            "value": ms, "unit": "ms/batch", "n_gpus": 1, "steps": steps, "warmup": max(args.warmup, 3),
            "ms_per_step": ms, "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32-in-f64", "data": "synthetic (seeded sizes, disk/noise masks, N(0,1) rhs)",
            "config": {"workload": "config4: batched 2D cell-centred 5-point, sizes log-uniform 64^2..1024^2",
                       "instances": len(probs), "fine_cells": cells, "schedule": dataclasses_asdict(p),
                       "tile_form": report.get("form", autotune.DEFAULT_FORM),
                       "autotune": report, "tune_s": t_tune, "setup_s": t_setup, "inputs_s": t_gen,
                       "timing": "host wall clock around each one-launch batch solve (it returns after the "
                                 "device finished)"},
            "per_instance_ms": {"p50": float(np.percentile(td, 50)), "p99": float(np.percentile(td, 99)),
                                "amortized": ms / len(probs)},
            "cycles": {"max": int(nite.max()), "median": float(np.median(nite))},
            "all_converged": bool(np.all(res <= TOL)), "clocks": clk.summary()}


def bench_config5(args, local, sub=False):
    """Configuration 5: forward + adjoint solves of variable-coefficient
    problems (mixed precision, FP64 residuals, to 1e-12), the gradients
    dL/db and dL/dkappa of L = 1/2 |P x - x*|^2, and a central finite-
    difference check along random directions at full size."""
    import numpy as np
    import torch

    import cfmg
    import fixtures as F
    import workloads as W

    torch.cuda.set_device(local)
    n = args.n if (args.n != 4096 and not sub) else 2048
    param, probs = W.config5(ninst=args.ninst if (args.ninst != 2048 and not sub) else 16, n=n)
    fd_dirs = 8 if sub else args.fd_dirs
    mg = cfmg.get_gmg(cfmg.Param(**param, tol=1e-12, maxite=80, residual_norm="l2", precision="mixed",
                                 verbose=False))
    # the finite-difference check needs the loss far below its own differences:
    # solves to 1e-14 there (x error ~ cond * tol) and a step of 1e-4
    mgfd = cfmg.get_gmg(cfmg.Param(**param, tol=1e-14, maxite=120, residual_norm="l2", precision="mixed",
                                   verbose=False))

    def loss(msk, kap, b, xs, mg=mg):
        mg.oper[1].msk = msk
        mg.oper[1].kappa = kap
        cfmg.setup_operators(mg)
        for lev in range(1, mg.nlevels + 1):
            for f in ("x", "y", "r", "b"):
                cfmg.set_to_zero(mg, lev, f)
        m = mg.download(1, "msk").astype(np.float64)
        bb = b * m
        F.subtract_mean(bb, m)
        return cfmg.loss_and_grad(mg, bb, xs * m), m

    times, fd_err = [], []
    rng = np.random.default_rng(64)
    loss(*probs[0])  # warm-up: graph capture
    for k, (msk, kap, b, xs) in enumerate(probs):
        torch.cuda.synchronize()
        t = time.perf_counter()
        (L0, gb, gk), m = loss(msk, kap, b, xs)
        times.append((time.perf_counter() - t) * 1e3)
        if k == 0:  # central finite differences along random directions, first instance
            (_, gb, gk), m = loss(msk, kap, b, xs, mgfd)
            for _ in range(fd_dirs):
                db = rng.standard_normal(b.shape) * m
                db -= m * (db.sum() / m.sum())
                dk = rng.standard_normal(b.shape) * m * 0.1
                eps = 1e-4
                lp = loss(msk, kap + eps * dk, b + eps * db, xs, mgfd)[0][0]
                lm = loss(msk, kap - eps * dk, b - eps * db, xs, mgfd)[0][0]
                fd = (lp - lm) / (2 * eps)
                an = float(np.sum(gb * db) + np.sum(gk * dk))
                fd_err.append(abs(fd - an) / abs(an))
    nlev = mg.nlevels
    mg.close()
    mgfd.close()
    ms = float(np.median(times))
    return {"metric": f"ms per forward+adjoint solve ({n}^2 variable-coefficient, mixed, tol 1e-12)",
            "value": ms, "unit": "ms/instance", "n_gpus": 1, "steps": len(probs), "warmup": 1,
            "ms_per_step": ms, "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32-in-f64", "data": "synthetic (kappa = exp(0.5 smoothed N(0,1)), disk mask, seed 4)",
            "config": {"workload": f"config5: {len(probs)} x {n}^2 div(kappa grad x) = b, forward + adjoint + "
                                   f"dL/dkappa", "levels": nlev,
                       "timing": "host wall clock per instance: coefficient setup, forward solve, adjoint solve "
                                 "and the host copies of x, dL/db and dL/dkappa"},
            "fd_check": {"directions": len(fd_err), "max_rel_err": max(fd_err) if fd_err else None,
                         "median_rel_err": float(np.median(fd_err)) if fd_err else None, "bound": 1e-6,
                         "solve_tol": 1e-14, "step": 1e-4}}


def dataclasses_replace(p, **kw):
    import dataclasses

    return dataclasses.replace(p, **kw)


def dataclasses_asdict(p):
    import dataclasses

    return {k: v for k, v in dataclasses.asdict(p).items() if k in ("cycle", "npre", "npost", "omega", "ndeepest")}


def main():
    args = parse()
    rank, world, local = dist_init()
    if args.impl == "reference":
        out = run_reference(args, rank, world)
    elif args.workload == "config1":
        out = bench_config1(args, local)
    elif args.workload == "config3":
        out = bench_config3(args, local)
    elif args.workload == "config4":
        out = bench_config4(args, local)
    elif args.workload == "config5":
        out = bench_config5(args, local)
    else:
        out = run_ours(args, rank, world, local)
    if rank == 0 and out is not None:
        print(json.dumps(out), flush=True)
    if world > 1:
        import torch.distributed as dist

        dist.destroy_process_group()


if __name__ == "__main__":
    main()
