"""Benchmark of the NSphere step loop on one GB300 (or N independent replicas).

Workload (default): N = 1e7 equal-mass Hernquist halo (a = 1, truncated at r = 100,
isotropic distribution function, seed 2), G = M = 1, adaptive leapfrog with at most
8 refinement levels (max_subdiv = 128), adaptive Levi-Civita below r = 1e-3,
tolerance 1e-7, Richardson output, dt = 4e-5: the step at which |dE/E| stays below
1e-6 over 1000 steps (the drift grows linearly in steps and as dt^2: 9.9e-5 at
dt = 5e-4, 3.9e-6 at 1e-4, 6.3e-7 at 4e-5 over 1000 steps of this halo).  One
step = radial sort + rank enclosed mass / force + adaptive integration of every
particle.  Metric: particle-steps/s.  The state (28 B/particle plus sort buffers)
is far larger than the 129 MB L2, so no flush is needed between steps.

Besides the timed region, both level schedules run 1000 steps from the same start
state (|dE/E| over those 1000 steps and their rate): the learned one after its
network is trained on levels logged from 200 plain steps of the N = 1e7 Hernquist
halo.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

``--impl reference`` times the reference's own CPU step (its functions built from
its sources into oracle/_ref; the oracle port when those are absent) on the same
workload with every host thread, one full N-particle step per timed step.
"""
from __future__ import annotations

import argparse
import ctypes as C
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
# sort + scan + force pass, algorithmic bytes per particle: read r key 8, gather r v ell id 28,
# write them 28, write the rank force 8
SORT_PASS_BYTES = 72.0
# DRAM bytes per particle of one k_fused_level0 launch (read + write), from an ncu capture
# of that kernel on the Hernquist state at N = 5e6 (172.8 MB read + 114.5 MB written per
# launch; traffic grows in proportion to N)
FUSED_LEVEL0_TRAFFIC = (172.847872e6 + 114.468352e6) / 5e6
# DRAM bytes per particle of the fixed-step sort + scan + force pass (k_bucket_scatter_idx
# and k_fused_rank_force with the kick), from an ncu capture of both on the Plummer state
# at N = 5e6 (40.1 + 0.1 MB and 160.7 + 147.3 MB read + written per launch)
SORT_PASS_TRAFFIC = (40.116224e6 + 0.082688e6 + 160.690432e6 + 147.293696e6) / 5e6
# DRAM bytes of one k_levi_civita_pair launch, from an ncu capture of the Hernquist step
# at N = 2e6 (62.7 KB read, nothing written back to DRAM during the launch); it does not
# grow with N -- the launch touches only the Levi-Civita particles
LC_TRAFFIC_PER_LAUNCH = 62.7e3
# IEEE double operations per particle that the level-0 pass issues
# (rank numerator 3, start force 5, coarse pass 9, fine pass 16, test 6, Richardson 6, l^2 1)
LEVEL0_FLOPS = 46.0


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--n", type=int, default=10_000_000)
    ap.add_argument("--workload", choices=["adaptive", "kdk", "ensemble", "om", "stress"], default="adaptive")
    ap.add_argument("--sched", choices=["plain", "learned"], default="plain")
    ap.add_argument("--e2e-steps", type=int, default=30)
    ap.add_argument("--ab-steps", type=int, default=1000,
                    help="steps of each schedule in the learned/plain comparison and drift run (0: skip)")
    ap.add_argument("--train-steps", type=int, default=200, help="plain steps whose levels train the scheduler")
    ap.add_argument("--dt", type=float, default=None, help="time step (default: the workload's)")
    ap.add_argument("--nonfinite-stop", type=int, default=1, help="stress workload: 0 follows the reference on non-finite passes")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--post-runs", type=int, default=3,
                    help="timed runs of the snapshot post-processing of the final state (0: skip)")
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--no-graph", action="store_true",
                    help="launch every step eagerly (for profilers that cannot see into graphs with "
                         "conditional nodes); results are identical")
    return ap.parse_args()


# time step of the adaptive workloads: |dE/E| <= 1e-6 over 1000 steps of the N = 1e7
# Hernquist halo (6.3e-7 measured; 9.8e-7 at 5e-5, 3.9e-6 at 1e-4, 9.9e-5 at 5e-4)
DT_EQUAL_DRIFT = 4e-5


def workload(args, seed_offset=0):
    from nsphere_gb300.replicas import replica_seed
    from nsphere_gb300 import ics
    dt_eq = DT_EQUAL_DRIFT
    if args.workload == "kdk":
        cfg = dict(workload="plummer_kdk_fixed_step", n=args.n, profile="plummer", seed=replica_seed(1, seed_offset),
                   dt=1e-3, method="fixed-step leapfrog (reference method 2)")
        state = ics.plummer(args.n, seed=replica_seed(1, seed_offset))
        params = dict(dt=1e-3, method=2)
    elif args.workload == "ensemble":
        r, vr, ell, ids, sizes = ics.plummer_ensemble(256, 10_000, 1_000_000, seed=replica_seed(3, seed_offset))
        cfg = dict(workload="plummer_ensemble_adaptive_lc", n=int(len(r)), halos=256,
                   halo_n="log-uniform in [1e4, 1e6]", profile="plummer", seed=replica_seed(3, seed_offset), dt=1e-3,
                   max_levels=8, max_subdiv=128, lc="adaptive levi-civita below r=1e-3", tol=1e-7, out_type=2)
        state = (r, vr, ell, ids, sizes)
        params = dict(dt=1e-3, max_subdiv=128, lc_rule=1, lc_radius=1e-3, method=5, max_tau_steps=1_000_000)
        args.n = int(len(r))
    elif args.workload == "om":
        cfg = dict(workload="hernquist_om_adaptive_lc", n=args.n, profile="hernquist a=1 r<=100 osipkov-merritt r_a=1",
                   seed=replica_seed(4, seed_offset), dt=dt_eq, max_levels=8, max_subdiv=128,
                   lc="adaptive levi-civita below r=1e-3", tol=1e-7, out_type=2)
        # generated on the GPU (nsg_generate_om, closed-form Osipkov-Merritt f(Q))
        import nsphere_gb300 as ns
        with ns.Context(ns.default_params()) as g:
            g.generate_om(args.n, replica_seed(4, seed_offset), 100.0, 1.0)
            state = g.download()
        cfg["generator"] = "nsg_generate_om"
        params = dict(dt=dt_eq, max_subdiv=128, lc_rule=1, lc_radius=1e-3, method=5, max_tau_steps=1_000_000)
    elif args.workload == "stress":
        # Hernquist, 20 % of the particles on near-radial orbits (ell uniform in [0, 1e-4]),
        # a central point mass ramped from 0 to 0.01 over 500 steps
        # generated on the GPU (nsg_generate): the host generator is slow at 1e8
        import nsphere_gb300 as ns
        with ns.Context(ns.default_params()) as g:
            g.generate(ns.IC_HERNQUIST, args.n, replica_seed(5, seed_offset), 100.0)
            r, vr, ell, ids = g.download()
        rng = np.random.default_rng(replica_seed(5, seed_offset))
        pick = rng.random(args.n) < 0.2
        ell = ell.copy()
        ell[pick] = rng.uniform(0.0, 1e-4, int(pick.sum()))
        cfg = dict(workload="hernquist_radial_point_mass", n=args.n, profile="hernquist a=1 r<=100 isotropic",
                   radial_fraction=0.2, radial_ell="U[0, 1e-4]", point_mass="0 -> 0.01 over 500 steps",
                   nonfinite_stop=args.nonfinite_stop,
                   seed=replica_seed(5, seed_offset), dt=5e-4, max_levels=8, max_subdiv=128,
                   lc="adaptive levi-civita below r=1e-3", tol=1e-7, out_type=2)
        state = (r, vr, ell, ids)
        params = dict(dt=5e-4, max_subdiv=128, lc_rule=1, lc_radius=1e-3, method=5, max_tau_steps=1_000_000,
                      point_mass_rate=0.01 / (500 * 5e-4), nonfinite_stop=args.nonfinite_stop)
    else:
        cfg = dict(workload="hernquist_adaptive_lc", n=args.n, profile="hernquist a=1 r<=100 isotropic",
                   seed=replica_seed(2, seed_offset), dt=dt_eq, max_levels=8, max_subdiv=128,
                   lc="adaptive levi-civita below r=1e-3", tol=1e-7, out_type=2)
        state = ics.hernquist(args.n, seed=replica_seed(2, seed_offset))
        params = dict(dt=dt_eq, max_subdiv=128, lc_rule=1, lc_radius=1e-3, method=5, max_tau_steps=1_000_000)
    if args.no_graph:
        params["graph"] = 0
    if args.dt is not None:
        # an explicit time step replaces the workload's (the point-mass ramp keeps its 500 steps)
        if "point_mass_rate" in params:
            params["point_mass_rate"] = 0.01 / (500 * args.dt)
        params["dt"] = cfg["dt"] = args.dt
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
        ok = [r for r in self.rows if len(r) >= 7 and r[0].replace(".", "").isdigit()]
        sm = [float(r[0]) for r in ok]
        mx = [float(r[1]) for r in ok if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in ok for k in range(4) if r[3 + k].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(sm)}


def cpu_stepper(params, parallel_sort=True):
    """The reference's own step functions (oracle/_ref, all host threads), else the port.
    parallel_sort: the reference's default quadsort_parallel (True) or its exact
    sequential quadsort (False)."""
    from oracle import build_oracle
    from oracle.oracle import Oracle, Reference
    try:
        if not build_oracle.build_reference():
            raise FileNotFoundError
        R = Reference(fast=True)
        cores, kind = R.num_threads(), "reference"

        def step(cur):
            if params.get("method") == 2:
                tab, _ = R.step_kdk(cur[0], cur[1], cur[2], cur[3], params["dt"], parallel_sort=parallel_sort)
            else:
                tab, _ = R.step_method5(cur[0], cur[1], cur[2], cur[3], params["dt"],
                                        max_subdiv=params["max_subdiv"], lc_rule=params["lc_rule"],
                                        lc_radius=params["lc_radius"], parallel_sort=parallel_sort)
            return tab[0], tab[1], tab[2], tab[3]
    except (FileNotFoundError, RuntimeError, OSError):
        build_oracle.build_oracle()
        O = Oracle()
        cores, kind = O.num_threads(), "port"
        if params.get("method") == 2:
            op = O.params(dt=params["dt"])

            def step(cur):
                return O.step_kdk(op, *cur)
        else:
            op = O.params(dt=params["dt"], max_subdiv=params["max_subdiv"], lc_rule=params["lc_rule"],
                          lc_radius=params["lc_radius"])

            def step(cur):
                return O.step_adaptive(op, *cur)[:4]
    return step, cores, kind


def cpu_baseline(state, params, seconds):
    """Reference CPU step on the full N-particle state, repeated for about `seconds`
    with its default parallel sort, then for about a third of that with its exact
    sequential quadsort."""
    from oracle import build_oracle
    r, vr, ell, ids = state
    n = len(r)
    out = {}
    for par, budget in ((True, seconds), (False, seconds / 3)):
        step, cores, kind = cpu_stepper(params, parallel_sort=par)
        cur = (r, vr, ell, ids.astype(np.float64))
        steps, elapsed = 0, 0.0
        while (elapsed < budget or steps == 0) and steps < 1000:
            t0 = time.perf_counter()
            cur = step(cur)
            elapsed += time.perf_counter() - t0
            steps += 1
        out[par] = (n * steps / elapsed, steps, elapsed, cores, kind)
    value, steps, elapsed, cores, kind = out[True]
    flags = build_oracle.fast_flags_used() if kind == "reference" else "gcc -O2 -fopenmp (oracle port)"
    return {"value": value, "unit": UNIT, "cores": cores, "kind": kind,
            "value_exact_quadsort": out[False][0],
            "sample": "%d full steps of the N=%d state (%.1f s of CPU work) with the default quadsort_parallel; "
                      "%d steps (%.1f s) with the exact sequential quadsort (value_exact_quadsort); built with: %s"
                      % (steps, n, elapsed, out[False][1], out[False][2], flags)}


def run_reference_arm(args, rank, world):
    if rank != 0:
        return
    cfg, state, params = workload(args)
    step, cores, kind = cpu_stepper(params)
    r, vr, ell, ids = state
    n = len(r)
    cur = (r, vr, ell, ids.astype(np.float64))
    budget, t_total, done = 180.0, 0.0, 0
    for j in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        cur = step(cur)
        dt_ = time.perf_counter() - t0
        if j >= args.warmup:
            t_total += dt_
            done += 1
            if t_total > budget:
                break
    value = n * done / t_total
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": done, "warmup": args.warmup, "ms_per_step": 1e3 * t_total / done,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded ICs)", "config": cfg,
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": kind,
                         "sample": "%d timed full steps of the N=%d state after %d warm-up steps"
                                   % (done, n, args.warmup)},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    from nsphere_gb300.replicas import job_rate, max_over_ranks, rank_env
    rank, local, world = rank_env()
    if args.impl == "reference":
        run_reference_arm(args, rank, world)
        return

    import torch
    import torch.distributed as dist
    import nsphere_gb300 as ns

    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    # independent replica per rank (the path does not shard across GPUs)
    cfg, state, params = workload(args, seed_offset=rank)
    r, vr, ell, ids = state[:4]
    sizes = state[4] if len(state) > 4 else None
    n = len(r)
    fp64 = ns.probe_fp64()
    fp64["latency_cycles"] = ns.probe_latency()

    # a dedicated (non-default) stream shared by the library and the timing events
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    p = ns.default_params(**params)
    if args.sched == "learned":
        p.sched = ns.SCHED_LEARNED
    ctx = ns.Context(p, stream=stream.cuda_stream)
    if sizes is None:
        ctx.upload(r, vr, ell, ids)
    else:
        ctx.upload_ensemble(r, vr, ell, ids, sizes)
        ctx.step(1)
        cfg["tuned_shapes"] = ctx.autotune(steps=1)["chosen"]
    E0 = sum(ctx.energy())
    ctx.step(args.warmup)
    torch.cuda.synchronize()
    l0, steps0 = ctx.counters()
    # the state the timed steps start from, so that the per-kernel profile below
    # replays exactly those steps (download/upload and eager steps leave every bit
    # as the graph replay does)
    snap0 = ctx.download()
    pm0 = p.point_mass
    for _ in range(steps0):
        pm0 += p.point_mass_rate * p.dt

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
    ms_max = max_over_ranks(ms, world, device="cuda")
    value = job_rate(n * args.steps, world, ms_max)
    hist = ctx.level_hist(10)
    status = ctx.status()

    # per-kernel breakdown from the library's own CUDA events over the same steps as
    # the timed region, replayed from its starting state
    nprof = args.steps
    q = ns.default_params(**params)
    q.sched = p.sched
    q.point_mass = pm0
    ctx.set_params(q)
    if sizes is None:
        ctx.upload(*snap0)
    else:
        ctx.upload_ensemble(*snap0, sizes)
    ctx.profile(True)
    ctx.step(nprof)
    prof = ctx.profile_read()
    ctx.profile(False)
    del snap0
    n_lc = int(np.count_nonzero(ctx.levels() >= 99))   # levels 99 and 100+ mark Levi-Civita particles

    # the sort + scan + force pass on its own: fixed-step leapfrog steps of the same
    # state (kick + drift, then bucket sort and the gather that writes the rank force)
    kp = ns.default_params(dt=params["dt"], method=ns.METHOD_KDK, graph=params.get("graph", 1))
    ctx.set_params(kp)
    ctx.step(2)
    ctx.clear_status()
    ctx.profile(True)
    ctx.step(nprof)
    kprof = ctx.profile_read()
    ctx.profile(False)
    kdk_fallback = bool(ctx.status() & ns.ST_SORT_FALLBACK)
    ctx.set_params(p)

    # learned against plain schedule, and the energy drift of each over 1000 steps.
    # Training set: the accepted levels of `train_steps` plain steps of the N = 1e7
    # Hernquist halo (the default workload), collected and trained on the GPU.  Then
    # each schedule runs `ab_steps` steps from the workload's start state; both give
    # bit-identical states (the plain error test judges every particle), so their
    # |dE/E| are equal by construction and measured here over the whole run.
    learned = None
    if args.workload in ("adaptive", "om", "stress") and args.ab_steps > 0 and sizes is None:
        if args.workload == "stress":
            # N = 1e8 at ~40 ms per step: a shorter comparison
            args.ab_steps = min(args.ab_steps, 100)
            args.train_steps = min(args.train_steps, 20)
        ctx.set_params(ns.default_params(**params))
        if args.workload == "adaptive":
            ctx.upload(r, vr, ell, ids)
        else:
            ctx.generate(ns.IC_HERNQUIST, n, 2, 100.0)
        ctx.mlp_init(4)
        # level 0 holds all but ~1e-5 of the particles at this dt: keep 1e-4 of them
        ctx.mlp_collect(args.train_steps, keep_level0=1e-4, capacity=1 << 21)
        _, ytrain = ctx.mlp_dataset()
        loss = ctx.mlp_train(epochs=4, batch=2048, lr=3e-3, seed=4)
        warm = 3

        def run_schedule(sched):
            q = ns.default_params(**params)
            q.sched = sched
            ctx.set_params(q)
            ctx.upload(r, vr, ell, ids)
            e_start = sum(ctx.energy())
            ctx.step(warm)
            barrier()
            t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            t0.record(stream)
            ctx.step(args.ab_steps - warm)
            t1.record(stream)
            barrier()
            ms_ = t0.elapsed_time(t1)
            e_end = sum(ctx.energy())
            final = ctx.download()
            lv = ctx.level_hist(10)
            # the kernels beside the Levi-Civita chains, per step, over 20 further steps
            ctx.profile(True)
            ctx.step(20)
            pr = ctx.profile_read()
            ctx.profile(False)
            bulk_ms = sum(k["total_ms"] for k in pr if k["name"] not in ("levi_civita", "lc_late")) / 20
            return {"value": n * (args.ab_steps - warm) / (ms_ / 1e3), "ms_per_step": ms_ / (args.ab_steps - warm),
                    "dE_over_E": abs(e_end - e_start) / abs(e_start), "steps": args.ab_steps,
                    "timed_steps": args.ab_steps - warm, "bulk_ms_per_step": bulk_ms,
                    "level_hist_last_step": [int(x) for x in lv],
                    "kernels": {k["name"]: k["total_ms"] / 20 for k in pr}}, final

        res_p, s_p = run_schedule(ns.SCHED_PLAIN)
        res_l, s_l = run_schedule(ns.SCHED_LEARNED)
        # bit for bit, NaN where both have NaN (the stress workload's non-finite passes)
        same = all(np.array_equal(a_, b_, equal_nan=True) and
                   np.array_equal(np.signbit(a_), np.signbit(b_)) for a_, b_ in zip(s_l, s_p))
        del s_l, s_p
        learned = {"train_steps": args.train_steps, "train_halo": "hernquist a=1 r<=100 isotropic, N=%d" % n,
                   "train_samples": int(len(ytrain)),
                   "train_class_counts": [int(x) for x in np.bincount(ytrain.astype(np.int64), minlength=8)],
                   "train_loss": loss, "plain": res_p, "learned": res_l,
                   "learned_value": res_l["value"], "plain_value": res_p["value"],
                   "speedup": res_l["value"] / res_p["value"],
                   "bulk_speedup": res_p["bulk_ms_per_step"] / res_l["bulk_ms_per_step"],
                   "identical_states": bool(same),
                   "dE_over_E_learned": res_l["dE_over_E"], "dE_over_E_plain": res_p["dE_over_E"],
                   "energy_drift_steps": args.ab_steps}
        del ytrain
        ctx.set_params(p)
        ctx.upload(r, vr, ell, ids)

    # End to end through the public C ABI with host buffers, as a driver whose state
    # lives on the host (the reference's loop) runs it: every step uploads the host
    # state (pinned), steps once and reads the result back into the host state the
    # next step uploads.  The host state starts as the state after two steps of the
    # context's current state (in the order of a sort, as a driver's state is after
    # its first step).
    pin = [torch.empty(n, dtype=torch.float64).pin_memory() for _ in range(8)]
    bufs = [[t.numpy() for t in pin[:4]], [t.numpy() for t in pin[4:]]]
    ctx.step(2)
    for dst, src in zip(bufs[0], ctx.download()):
        dst[:] = src
    lib = ns.lib()

    def P(a):
        return C.c_void_p(a.ctypes.data)

    barrier()
    ee0, ee1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ee0.record(stream)
    hn = None if sizes is None else np.ascontiguousarray(sizes, dtype=np.int64)
    for k in range(args.e2e_steps):
        h_r, h_v, h_l, h_i = bufs[k & 1]
        o_r, o_v, o_l, o_i = bufs[(k + 1) & 1]
        if hn is None:
            ctx._check(lib.nsg_upload(ctx.handle, P(h_r), P(h_v), P(h_l), P(h_i), None, n))
        else:
            ctx._check(lib.nsg_upload_ensemble(ctx.handle, P(h_r), P(h_v), P(h_l), P(h_i), None, P(hn), len(hn)))
        # one step and the read-back of its result (the copy overlaps the step's chains)
        ctx._check(lib.nsg_step_download(ctx.handle, 1, P(o_r), P(o_v), P(o_l), P(o_i), None))
    ee1.record(stream)
    barrier()
    e2e_value = job_rate(n * args.e2e_steps, world, max_over_ranks(ee0.elapsed_time(ee1), world, device="cuda"))

    # per-snapshot post-processing (Rank-file records with Psi_A and the smoothed
    # density) of the final state, through the C ABI from host records to host records
    post = None
    if args.post_runs > 0 and sizes is None and world == 1:
        from nsphere_gb300 import ics
        recs = ics.snapshot_records(*ctx.download())
        with ns.Context(ns.default_params(), stream=stream.cuda_stream) as pc:
            pc.post_snapshot(recs)
            times = []
            for _ in range(args.post_runs):
                torch.cuda.synchronize()
                t0 = time.perf_counter()
                pc.post_snapshot(recs)
                times.append(time.perf_counter() - t0)
            pc.profile(True)
            pc.post_snapshot(recs)
            stages = pc.profile_read()
            pc.profile(False)
        post = {"n": n, "ms": 1e3 * statistics.median(times), "runs": args.post_runs,
                "h2d_bytes": 16 * n, "d2h_bytes": 60 * n,
                "stages": [{"name": k["name"], "ms": k["total_ms"], "GBps": (k["bytes"] / k["total_ms"] / 1e6)
                            if k["total_ms"] > 0 else None} for k in stages],
                "note": "nsg_post_snapshot, host records in, host Rank records out (blocking call); "
                        "stages from the library's CUDA events in one further run"}
        if not args.no_cpu_baseline:
            from oracle import build_oracle
            from oracle.oracle import Oracle
            build_oracle.build_oracle()
            t0 = time.perf_counter()
            Oracle().post_snapshot(recs["r"], recs["v"], recs["l"])
            post["cpu_baseline"] = {"ms": 1e3 * (time.perf_counter() - t0), "cores": 1, "kind": "port",
                                    "sample": "the same snapshot, sequential restatement (oracle)"}

    if rank == 0:
        peaks = {}
        try:
            peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
        except Exception:
            pass
        hbm_peak = peaks.get("hbm_gbs", 6800.0)
        peak_src = "measured (MEASURED_PEAKS.json)" if "hbm_gbs" in peaks else "fallback"
        by = {k["name"]: k for k in prof}
        kby = {k["name"]: k for k in kprof}
        main_ms = sum(k["total_ms"] for k in prof if k["name"] != "levi_civita") / nprof
        tot = sum(k["total_ms"] for k in prof) or 1.0
        lat = fp64["latency_cycles"]
        bulk = None
        l0name = "fused_level0" if "fused_level0" in by else "gather_level0"
        if l0name in by:
            g = by[l0name]
            per = g["total_ms"] / g["launches"]
            ach = (g["bytes"] / g["launches"]) / (per / 1e3) / 1e9
            flops = LEVEL0_FLOPS * n / (per / 1e3) / 1e12
            bulk = {"bound": "hbm", "kernel": "k_" + l0name, "achieved": ach, "peak": hbm_peak,
                    "unit": "GB/s", "frac": ach / hbm_peak,
                    "traffic": (FUSED_LEVEL0_TRAFFIC * n) if (FUSED_LEVEL0_TRAFFIC and l0name == "fused_level0")
                    else None,
                    "peak_source": peak_src, "ms": per,
                    "note": "the sort of the step (in shared memory) and adaptive level 0 in one kernel; "
                            "65 algorithmic bytes per particle; bound by the FP64 pipe (46 IEEE operations "
                            "per particle at level 0); FP64 view below",
                    "fp64": {"achieved_tflops": flops, "peak_tflops": fp64["dfma_tflops"],
                             "frac": flops / fp64["dfma_tflops"],
                             "peak_source": "measured live by nsg_probe_fp64 (FMA = 2 flops)"}}
        # the dominant kernel: the Levi-Civita chains.  Algorithmic bytes per launch:
        # each Levi-Civita particle reads r, v_r, ell and its list entry (32 B) and
        # writes r, v_r and its level (17 B).
        roof = None
        lcs = by.get("levi_civita")
        roof_lc = None
        if lcs:
            per = lcs["total_ms"] / lcs["launches"]
            alg = 49.0 * n_lc
            ach = alg / (per / 1e3) / 1e9
            roof = {"bound": "hbm", "kernel": "k_levi_civita_pair", "achieved": ach, "peak": hbm_peak,
                    "unit": "GB/s", "frac": ach / hbm_peak, "traffic": LC_TRAFFIC_PER_LAUNCH,
                    "peak_source": peak_src, "lc_particles": n_lc,
                    "note": "neither HBM nor tensor bound: each Levi-Civita particle is one serial "
                            "chain of dependent FP64 operations; its bound is the dependent latency, "
                            "latency_frac = floor / measured cycles per substep",
                    "latency_frac": (9 * lat["fp64_fma"] + lat["div_latency_form"]) / lat["levi_civita_substep"]}
            roof_lc = dict(roof)
        # The pass of a fixed-step leapfrog step: index scatter + bucket scan, then the
        # fused sort + rank force + kick.  The radix fallback's kernels (launched eagerly
        # here, returning at once; skipped by the conditional graph node of a replayed
        # step) count only when the fallback ran.
        if "fused_kick" in kby:
            sort_names = ["bucket_scatter", "fused_kick"]
            if kdk_fallback:
                sort_names += ["sort_seed", "sort_radix", "gather_kick_fallback"]
        else:
            sort_names = ["bucket_scatter", "bucket_sort", "sort_seed", "sort_radix", "gather_kick"]
        sort_ms = sum(kby[k]["total_ms"] for k in sort_names if k in kby) / nprof
        sort_gbs = SORT_PASS_BYTES * n / (sort_ms / 1e3) / 1e9 if sort_ms else None
        # the roofline object names the kernel with the largest share of the timed steps
        top = max(prof, key=lambda k: k["total_ms"]) if prof else None
        if top is not None and top["name"] == l0name and bulk is not None:
            roof = dict(bulk)
        if roof is None and sort_gbs:
            # no Levi-Civita chains (fixed-step leapfrog): the sort + scan + force pass dominates
            roof = {"bound": "hbm", "kernel": "sort + scan + force pass (k_bucket_scatter_idx, k_fused_rank_force "
                                              "with the bucket starts by look-back)",
                    "achieved": sort_gbs, "peak": hbm_peak, "unit": "GB/s", "frac": sort_gbs / hbm_peak,
                    "traffic": SORT_PASS_TRAFFIC * n, "peak_source": peak_src,
                    "note": "72 algorithmic bytes per particle"}
        lc = by.get("levi_civita")
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded ICs)",
            "config": cfg, "clocks": clk.summary(),
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": 32 * n,
                    "d2h_bytes_per_step": 32 * n},
            "gpu_launches": int(l1 - l0),
            "roofline": roof,
            "bulk_roofline": bulk,
            "critical_path": {
                "kernel": "k_levi_civita_pair",
                "bound": "dependent latency of one serial chain (neither HBM nor tensor)",
                # one substep: 10 dependent FP64 operations and one latency-form
                # division; the probe's division entry includes one of the 10
                "substep_cycles": lat["levi_civita_substep"],
                "substep_floor_cycles": 9 * lat["fp64_fma"] + lat["div_latency_form"],
                "latency_frac": (9 * lat["fp64_fma"] + lat["div_latency_form"]) / lat["levi_civita_substep"],
                "levi_civita_ms": (lc["total_ms"] / lc["launches"]) if lc else 0.0,
                "main_stream_ms": main_ms,
                "note": "main_stream_ms: every other kernel of the step (sort, leapfrog levels), which runs "
                        "beside the Levi-Civita chains; the step ends when the longest chain ends",
                "fp64_dependent_latency_cycles": {"fma": fp64["fma_latency_cycles"],
                                                  "division": fp64["div_latency_cycles"]}},
            "sort_scan_force": {"ms": sort_ms, "GBps": sort_gbs,
                                "frac": (sort_gbs / hbm_peak) if sort_gbs else None,
                                "bytes_per_particle": SORT_PASS_BYTES,
                                "kernels": {k: kby[k]["total_ms"] / nprof for k in sort_names if k in kby},
                                "radix_fallback_ran": kdk_fallback,
                                "workload": "fixed-step leapfrog steps of the timed state"},
            "lc_roofline": roof_lc,
            "kernels": [{"name": k["name"], "ms_per_step": k["total_ms"] / nprof, "share": k["total_ms"] / tot}
                        for k in prof],
            "fp64_probe": fp64,
            # |dE/E| over 1000 steps of each schedule (the learned/plain runs), else over the
            # warm-up and timed steps
            "energy_drift": learned["dE_over_E_plain"] if learned else abs(E1 - E0) / abs(E0),
            "energy_drift_steps": learned["energy_drift_steps"] if learned else args.warmup + args.steps,
            "energy_drift_learned": learned["dE_over_E_learned"] if learned else None,
            "energy_drift_timed_region": abs(E1 - E0) / abs(E0),
            "level_hist": [int(x) for x in hist],
            "status": status,
            "learned_vs_plain": learned,
            "post_snapshot": post,
        }
        if not args.no_cpu_baseline and world == 1 and sizes is None:
            line["cpu_baseline"] = cpu_baseline(state, params, args.cpu_seconds)
        print(json.dumps(line), flush=True)
    ctx.close()
    if world > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
