"""Benchmark of the NSphere step loop on one GB300 (or N independent replicas).

Workload (default): N = 1e7 equal-mass Hernquist halo (a = 1, truncated at r = 100,
isotropic distribution function, seed 2), G = M = 1, adaptive leapfrog with at most
8 refinement levels (max_subdiv = 128), adaptive Levi-Civita below r = 1e-3,
tolerance 1e-7, Richardson output, dt = 5e-4.  One step = radial sort + rank
enclosed mass / force + adaptive integration of every particle.  Metric:
particle-steps/s.  The state (28 B/particle plus sort buffers) is far larger than
the 129 MB L2, so no flush is needed between steps.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

``--impl reference`` times the reference's own CPU step (its functions built from
its sources into oracle/_ref; the oracle port when those are absent) on the same
workload with every host thread, on a bounded sample per step.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "particle-steps/s at N=1e7: learned vs plain GPU at equal |ΔE/E|; HBM GB/s"
UNIT = "particle-steps/s"
HBM_BYTES_SORT = 72.0       # algorithmic bytes per particle of the sort + rank/force pass
HBM_BYTES_INTEGRATE = 48.0  # read r, v_r, ell, a0; write r, v_r


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--n", type=int, default=10_000_000)
    ap.add_argument("--workload", choices=["adaptive", "kdk"], default="adaptive")
    ap.add_argument("--sched", choices=["plain", "learned"], default="plain")
    ap.add_argument("--e2e-steps", type=int, default=5)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-seconds", type=float, default=20.0)
    return ap.parse_args()


def workload(args):
    from nsphere_gb300 import ics
    if args.workload == "kdk":
        name = "plummer_kdk_fixed_step"
        cfg = dict(workload=name, n=args.n, profile="plummer", seed=1, dt=1e-3, method="kdk (reference method 2)")
        state = ics.plummer(args.n, seed=1)
        params = dict(dt=1e-3, method=2)
    else:
        name = "hernquist_adaptive_lc"
        cfg = dict(workload=name, n=args.n, profile="hernquist a=1 r<=100 isotropic", seed=2, dt=5e-4,
                   max_levels=8, max_subdiv=128, lc="levi-civita below r=1e-3", tol=1e-7, out_type=2)
        state = ics.hernquist(args.n, seed=2)
        params = dict(dt=5e-4, max_subdiv=128, lc_rule=1, lc_radius=1e-3, method=5, max_tau_steps=1_000_000)
    cfg["l2"] = "inputs larger than L2 (state %.0f MB vs 129 MB L2); no flush" % (args.n * 28 / 1e6)
    cfg["sched"] = args.sched
    return cfg, state, params


class Clocks:
    """Samples nvidia-smi during the timed region."""

    def __init__(self, index=0):
        self.index = index
        self.rows = []
        self.proc = None

    def __enter__(self):
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except FileNotFoundError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm = [float(r[0]) for r in self.rows if len(r) >= 7 and r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in self.rows if len(r) >= 7 and r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in self.rows if len(r) >= 7 for k in range(4)
                          if r[3 + k].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(sm)}


def cpu_baseline(state, params, args, seconds, use_reference=True):
    """Times the reference CPU step (oracle/_ref, every host thread) on a bounded sample."""
    from oracle import build_oracle
    from oracle.oracle import Oracle, Reference
    r, vr, ell, ids = state
    kind = "reference"
    try:
        if not use_reference or not build_oracle.build_reference():
            raise FileNotFoundError
        R = Reference(fast=True)
        cores = R.num_threads()

        def step(cur):
            if params.get("method") == 2:
                tab, _ = R.step_kdk(cur[0], cur[1], cur[2], cur[3], params["dt"], parallel_sort=True)
            else:
                tab, _ = R.step_method5(cur[0], cur[1], cur[2], cur[3], params["dt"],
                                        max_subdiv=params["max_subdiv"], lc_rule=params["lc_rule"],
                                        lc_radius=params["lc_radius"], parallel_sort=True)
            return tab[0], tab[1], tab[2], tab[3]
    except (FileNotFoundError, RuntimeError, OSError):
        kind = "port"
        build_oracle.build_oracle()
        O = Oracle()
        cores = O.num_threads()
        if params.get("method") == 2:
            op = O.params(dt=params["dt"])

            def step(cur):
                return O.step_kdk(op, *cur)
        else:
            op = O.params(dt=params["dt"], max_subdiv=params["max_subdiv"], lc_rule=params["lc_rule"],
                          lc_radius=params["lc_radius"])

            def step(cur):
                return O.step_adaptive(op, *cur)[:4]
    # bounded sample: whole state while a step fits the budget, else a prefix subsample
    n = len(r)
    m = n
    cur = (r[:m], vr[:m], ell[:m], ids[:m].astype(np.float64))
    t0 = time.perf_counter()
    cur = step(cur)
    t1 = time.perf_counter()
    steps, elapsed = 1, t1 - t0
    while elapsed < seconds and steps < 1000:
        t0 = time.perf_counter()
        cur = step(cur)
        elapsed += time.perf_counter() - t0
        steps += 1
    return {"value": m * steps / elapsed, "unit": UNIT, "cores": cores, "kind": kind,
            "sample": "%d steps of the full N=%d state (%.1f s of CPU work, quadsort_parallel, "
                      "gcc -O2 -ffast-math -fopenmp)" % (steps, m, elapsed)}


def run_reference_arm(args, rank, world):
    if rank != 0:
        return
    cfg, state, params = workload(args)
    # each step is a bounded sample of the workload: one full step of the N-particle state
    res = cpu_baseline(state, params, args, seconds=1e-9)
    from oracle.oracle import Reference
    steps = args.steps + args.warmup
    t_total = 0.0
    vals = []
    # one measurement per step (warmup steps untimed)
    r, vr, ell, ids = state
    cur = (r, vr, ell, ids.astype(np.float64))
    kind = res["kind"]
    if kind == "reference":
        R = Reference(fast=True)

        def step(c):
            if params.get("method") == 2:
                tab, _ = R.step_kdk(c[0], c[1], c[2], c[3], params["dt"], parallel_sort=True)
            else:
                tab, _ = R.step_method5(c[0], c[1], c[2], c[3], params["dt"], max_subdiv=params["max_subdiv"],
                                        lc_rule=params["lc_rule"], lc_radius=params["lc_radius"],
                                        parallel_sort=True)
            return tab[0], tab[1], tab[2], tab[3]
    else:
        from oracle.oracle import Oracle
        O = Oracle()
        op = O.params(dt=params["dt"], max_subdiv=params.get("max_subdiv", 128),
                      lc_rule=params.get("lc_rule", 0), lc_radius=params.get("lc_radius", 1e-3))

        def step(c):
            return O.step_kdk(op, *c) if params.get("method") == 2 else O.step_adaptive(op, *c)[:4]
    # bound the run: at most ~3 minutes of CPU time in total
    budget = 180.0
    done = 0
    for j in range(steps):
        t0 = time.perf_counter()
        cur = step(cur)
        dt_ = time.perf_counter() - t0
        if j >= args.warmup:
            t_total += dt_
            done += 1
        if t_total > budget and done >= 1:
            break
        vals.append(dt_)
    n = len(r)
    value = n * done / t_total
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": done, "warmup": args.warmup, "ms_per_step": 1e3 * t_total / done, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded ICs)",
        "config": cfg,
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": res["cores"], "kind": kind,
                         "sample": "%d timed steps of the full N=%d state after %d warm-up steps" % (done, n, args.warmup)},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        run_reference_arm(args, rank, world)
        return

    import torch
    import torch.distributed as dist
    import nsphere_gb300 as ns

    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    cfg, state, params = workload(args)
    if world > 1:
        # independent replica per rank (the path does not shard across GPUs)
        from nsphere_gb300 import ics
        state = ics.hernquist(args.n, seed=2 + rank) if args.workload == "adaptive" else ics.plummer(args.n, seed=1 + rank)
    r, vr, ell, ids = state
    n = len(r)
    # a dedicated (non-default) stream shared by the library and the timing events
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    p = ns.default_params(**params)
    if args.sched == "learned":
        p.sched = ns.SCHED_LEARNED
    ctx = ns.Context(p, stream=stream.cuda_stream)
    ctx.upload(r, vr, ell, ids)
    E0 = sum(ctx.energy())
    ctx.step(args.warmup)
    torch.cuda.synchronize()
    l0, _ = ctx.counters()

    def barrier():
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()

    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with Clocks(local) as clk:
        barrier()
        e0.record(stream)
        ctx.step(args.steps)
        e1.record(stream)
        barrier()
    ms = e0.elapsed_time(e1)
    l1, _ = ctx.counters()
    E1 = sum(ctx.energy())
    ms_t = torch.tensor([ms], dtype=torch.float64, device="cuda")
    if world > 1:
        dist.all_reduce(ms_t, op=dist.ReduceOp.MAX)
    ms_max = float(ms_t.item())
    value = n * world * args.steps / (ms_max / 1e3)
    hist = ctx.level_hist(10)
    status = ctx.status()

    # per-kernel breakdown from the library's own CUDA events (short profiled pass)
    ctx.profile(True)
    ctx.step(3)
    prof = ctx.profile_read()
    ctx.profile(False)

    # end to end through the public C ABI with host buffers: upload (pinned), step, download
    pin = [torch.empty(n, dtype=torch.float64).pin_memory() for _ in range(8)]
    h_r, h_v, h_l, h_i, o_r, o_v, o_l, o_i = [t.numpy() for t in pin]
    h_r[:], h_v[:], h_l[:], h_i[:] = r, vr, ell, ids
    lib = ns.lib()
    import ctypes as C

    def P(a):
        return C.c_void_p(a.ctypes.data)

    barrier()
    t0 = time.perf_counter()
    ee0, ee1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ee0.record(stream)
    for _ in range(args.e2e_steps):
        ctx._check(lib.nsg_upload(ctx.handle, P(h_r), P(h_v), P(h_l), P(h_i), None, n))
        ctx._check(lib.nsg_step(ctx.handle, 1))
        ctx._check(lib.nsg_download(ctx.handle, P(o_r), P(o_v), P(o_l), P(o_i), None))
    ee1.record(stream)
    barrier()
    e2e_ms = ee0.elapsed_time(ee1)
    et = torch.tensor([e2e_ms], dtype=torch.float64, device="cuda")
    if world > 1:
        dist.all_reduce(et, op=dist.ReduceOp.MAX)
    e2e_value = n * world * args.e2e_steps / (float(et.item()) / 1e3)

    if rank == 0:
        tot = sum(k["total_ms"] for k in prof) or 1.0
        dom = max(prof, key=lambda k: k["total_ms"]) if prof else None
        peaks = {}
        try:
            peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
        except Exception:
            pass
        hbm_peak = peaks.get("hbm_gbs", 6800.0)
        peak_src = "measured" if "hbm_gbs" in peaks else "fallback"
        sort_ms = sum(k["total_ms"] for k in prof if k["name"] in ("sort_seed", "sort_radix", "rank_force")) / 3
        sort_gbs = HBM_BYTES_SORT * n / (sort_ms / 1e3) / 1e9 if sort_ms else None
        roof = None
        if dom is not None:
            per_launch = dom["total_ms"] / dom["launches"]
            ach = (dom["bytes"] / dom["launches"]) / (per_launch / 1e3) / 1e9
            roof = {"bound": "hbm", "kernel": dom["name"], "achieved": ach, "peak": hbm_peak, "unit": "GB/s",
                    "frac": ach / hbm_peak, "traffic": None, "peak_source": peak_src,
                    "share": dom["total_ms"] / tot}
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded ICs)",
            "config": cfg, "clocks": clk.summary(),
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": 32 * n,
                    "d2h_bytes_per_step": 32 * n},
            "gpu_launches": int(l1 - l0),
            "roofline": roof,
            "sort_scan_force": {"ms": sort_ms, "GBps": sort_gbs, "frac": (sort_gbs / hbm_peak) if sort_gbs else None,
                                "bytes_per_particle": HBM_BYTES_SORT},
            "kernels": [{"name": k["name"], "ms_per_step": k["total_ms"] / 3, "share": k["total_ms"] / tot}
                        for k in prof],
            "energy_drift": abs(E1 - E0) / abs(E0),
            "level_hist": [int(x) for x in hist],
            "status": status,
        }
        if not args.no_cpu_baseline and world == 1:
            line["cpu_baseline"] = cpu_baseline(state, params, args, args.cpu_seconds)
        print(json.dumps(line), flush=True)
    ctx.close()
    if world > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
