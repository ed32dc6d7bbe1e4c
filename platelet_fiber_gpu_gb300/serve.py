"""Batched and served operation of many independent jobs on one GPU.

`run_batched` -- a fixed set of jobs (the many-job workload of
  workloads.batch_job: 64 lattices of 32^3 .. 128x64x64 nodes, 1-8
  platelets, 1k-5k fibrin nodes), all admitted at once and advanced
  together for a fixed number of steps; reports aggregate MLUPS.
`run_served`  -- jobs arriving as a Poisson process with a requested step
  count each, admitted against a device-memory budget as they arrive
  (continuous batching: jobs join between batch steps of `chunk` steps and
  leave by themselves when they reach their step count); reports
  aggregate MLUPS over the makespan and the p50 / p99 job latency
  (arrival to completion).

    python -m platelet_fiber_gpu_gb300.serve --mode served --precision 2
"""
from __future__ import annotations

import argparse
import json
import time

import numpy as np

from . import workloads as W
from .gpu import Batch


def run_batched(precision: int, n_jobs: int = 64, steps: int = 1000, seed: int = 3, budget: float = 150e9,
                chunk: int = 100, scenes=None) -> dict:
    """`scenes`: the job set (default: n_jobs jobs of workloads.batch_job)."""
    if scenes is None:
        scenes = [W.batch_job(seed, i) for i in range(n_jobs)]
    n_jobs = len(scenes)
    b = Batch(int(budget))
    slots = []
    for sc in scenes:
        s = b.admit(sc, precision)
        if s is None:
            raise RuntimeError("the job set does not fit the budget")
        slots.append(s)
    b.step(1)  # captures the step graph
    # the autotuner measures its candidate shapes on real steps; they run
    # before the timed region (every job advances by them)
    tune_steps = b.tune(max_steps=400, chunk=20)
    shape, state = b.shape()
    nodes = sum(sc.n_nodes for sc in scenes)
    t0 = time.perf_counter()
    left = steps
    while left > 0:
        k = min(chunk, left)
        b.step(k)
        left -= k
    dt = time.perf_counter() - t0
    b.close()
    return {"mode": "batched", "precision": precision, "jobs": n_jobs, "steps": steps, "nodes": nodes,
            "seconds": round(dt, 4), "mlups": round(nodes * steps / dt / 1e6, 1), "tune_steps": tune_steps,
            "shape": {"lbm_rows": shape[0], "list_per_sm": shape[1], "marker_threads": shape[2],
                      "state": state}}


def run_served(precision: int, rate: float = 20.0, duration: float = 10.0, seed: int = 4, budget: float = 150e9,
               chunk: int = 50, steps_range=(500, 5000), pool: int = 32, batch_factory=Batch,
               scenes=None, on_finish=None) -> dict:
    """Poisson arrivals at `rate` per second for `duration` seconds; each job
    is one of `pool` pre-built scenes of the many-job workload with its own
    requested step count drawn from `steps_range`.  `batch_factory` and
    `scenes` replace the GPU batch and the scene pool (host-logic tests);
    `on_finish(scene_index, requested_steps, job)` sees each finished job
    before it leaves the batch (its results are read there)."""
    rng = np.random.default_rng(seed)
    if scenes is None:
        scenes = [W.batch_job(seed, i) for i in range(pool)]
    pool = len(scenes)
    arrivals = []
    t = 0.0
    while True:
        t += float(rng.exponential(1.0 / rate))
        if t > duration:
            break
        arrivals.append((t, int(rng.integers(pool)), int(rng.integers(steps_range[0], steps_range[1] + 1))))
    b = batch_factory(int(budget))
    live = {}  # slot -> [arrival, steps left, nodes, requested]
    waiting = []
    latencies = []
    work = 0
    i = 0
    host = {"admit": 0.0, "step": 0.0, "retire": 0.0}
    calls = 0
    live_sum = 0
    t0 = time.perf_counter()
    while i < len(arrivals) or waiting or live:
        now = time.perf_counter() - t0
        while i < len(arrivals) and arrivals[i][0] <= now:
            waiting.append(arrivals[i])
            i += 1
        still = []
        ta = time.perf_counter()
        for a in waiting:
            sc = scenes[a[1]]
            s = b.admit(sc, precision)
            if s is None:
                still.append(a)
                continue
            # the job leaves the fused step by itself after its requested steps
            b.set_stop(s, a[2])
            live[s] = [a[0], a[2], sc.n_nodes, a[2], a[1]]
        waiting = still
        host["admit"] += time.perf_counter() - ta
        if not live:
            if i < len(arrivals):
                time.sleep(max(0.0, arrivals[i][0] - (time.perf_counter() - t0)))
            continue
        ts = time.perf_counter()
        b.step(chunk)
        calls += 1
        live_sum += len(live)
        tr = time.perf_counter()
        host["step"] += tr - ts
        for s in list(live):
            live[s][1] -= chunk
            if b.status(s) != 0:
                arr, _, n, req, idx = live.pop(s)
                work += n * req
                latencies.append(time.perf_counter() - t0 - arr)
                if on_finish is not None:
                    on_finish(idx, req, b.job(s))
                b.retire(s)
        host["retire"] += time.perf_counter() - tr
    span = time.perf_counter() - t0
    b.close()
    lat = np.array(latencies) if latencies else np.zeros(1)
    return {"mode": "served", "precision": precision, "jobs": len(arrivals), "rate_per_s": rate,
            "duration_s": duration, "makespan_s": round(span, 3), "mlups": round(work / span / 1e6, 1),
            "latency_p50_s": round(float(np.percentile(lat, 50)), 4),
            "latency_p99_s": round(float(np.percentile(lat, 99)), 4), "scene_pool": pool,
            "node_steps": int(work), "host_s": {k: round(v, 3) for k, v in host.items()}, "step_calls": calls,
            "mean_live_jobs": round(live_sum / max(1, calls), 1)}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--mode", choices=["batched", "served"], default="served")
    ap.add_argument("--precision", type=int, default=1)
    ap.add_argument("--jobs", type=int, default=64)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--rate", type=float, default=20.0)
    ap.add_argument("--duration", type=float, default=10.0)
    ap.add_argument("--budget-gb", type=float, default=150.0)
    args = ap.parse_args()
    from .build import build
    build()
    if args.mode == "batched":
        r = run_batched(args.precision, args.jobs, args.steps, budget=args.budget_gb * 1e9)
    else:
        r = run_served(args.precision, args.rate, args.duration, budget=args.budget_gb * 1e9)
    print(json.dumps(r), flush=True)


if __name__ == "__main__":
    main()
