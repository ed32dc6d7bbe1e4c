"""Benchmark of the coupled platelet / fibrin / lattice-Boltzmann step.

Workload (one step = one coupled step of the whole scene): D3Q19 BGK FP32
channel 256x128x128, shear 1000 1/s through the reference's unit chain,
50 platelets x 600 SEM elements (Poisson-disk placed), 20k-node / 40k-link
fibrin mesh on the bottom wall, 200 receptors per platelet with constant
per-step bond probabilities 1e-2 / 1e-3, Morse pairs.  Seeded synthetic
inputs; the working set (2 x 318 MB of populations) is larger than L2.

Prints one JSON line (rank 0):
  value   MLUPS with the state resident in HBM (CUDA events around K graph
          replays of the step),
  e2e     the same K-step job through the C ABI from host buffers: scene
          upload (pfgpu_job_create), K steps, download of the lattice and
          element state (pfgpu_job_get_*), all inside the timed region,
  roofline  the fused collide-stream kernel: 152 B/node algorithmic bytes
          over its CUDA-event-measured duration (serialised pass),
  cpu_baseline  the CPU oracle (FP64, all host threads) on a bounded sample.
`--impl reference` times the CPU restatement of the reference's kernels
(the oracle) instead and prints the same line with impl "reference".
Multi-GPU: one independent replica per rank (no collective); value is the
sum of the ranks' node updates over the slowest rank's time.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

BYTES_PER_NODE = {0: 304, 1: 152, 2: 76}  # algorithmic bytes per node-step (19 loads + 19 stores)
PREC_NAME = {0: "f64", 1: "f32", 2: "f16-shifted"}


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []
        self.n0 = 0

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
            # the sampler is live before the timed region starts; samples
            # taken before it are left out of the summary
            t_end = time.time() + 3.0
            while not self.lines and time.time() < t_end and self.proc.poll() is None:
                time.sleep(0.01)
            self.n0 = len(self.lines)
        except (FileNotFoundError, OSError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            # a timed region shorter than the sampling interval still gets
            # the sample that closes it
            t_end = time.time() + 0.5
            while len(self.lines) <= self.n0 and time.time() < t_end and self.proc.poll() is None:
                time.sleep(0.01)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=2)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.t.join(timeout=2)

    def summary(self):
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines[getattr(self, "n0", 0):]:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 8:
                continue
            try:
                sm.append(float(f[0]))
                smax = float(f[1])
            except ValueError:
                continue
            for nm, v in zip(names, f[4:8]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": smax, "reasons": sorted(reasons), "samples": len(sm)}


def measured_peak():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        try:
            d = json.loads(p.read_text())
            return float(d["hbm_gbs"]), "measured"
        except (ValueError, KeyError):
            pass
    return 6800.0, "fallback"


def lattice_traffic(prec: int, kernel: str, nodes: int):
    """DRAM bytes (read + write) of one step's lattice passes from the
    committed full-size ncu capture (profiles/lattice_traffic.json), when it
    was taken of the same kernels, precision and lattice; else None."""
    p = ROOT / "profiles" / "lattice_traffic.json"
    if not p.exists():
        return None
    try:
        e = json.loads(p.read_text()).get(PREC_NAME[prec])
    except ValueError:
        return None
    if not e or e.get("kernel") != kernel or e.get("nodes") != nodes:
        return None
    return e["dram_bytes_per_step"]


def reduce_max(dist, x: float, device: str) -> float:
    """Maximum of x over the ranks of an initialised process group (the
    slowest replica's time); x itself without one."""
    if dist is None:
        return x
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_value(world: int, nodes_per_replica: int, t_step_max: float) -> float:
    """Whole-job MLUPS of `world` independent replicas: all node updates
    over the slowest replica's step time."""
    return world * nodes_per_replica / t_step_max / 1e6


def build_scene(args):
    from platelet_fiber_gpu_gb300 import workloads as W
    if getattr(args, "workload", "single_large") == "plain_small":
        return W.plain_small()
    return W.single_large(seed=args.seed, nx=args.nx, ny=args.ny, nz=args.nz, n_platelets=args.platelets,
                          n_fib=args.fibrin, n_links=2 * args.fibrin)


def cpu_oracle_rate(scene, budget_s: float, max_steps: int, threads: int):
    """Oracle steps on the host until the budget is spent; returns
    (MLUPS, steps, seconds, threads)."""
    from oracle import binding as ob
    ob.set_threads(threads)
    o = ob.Oracle(scene)
    o.step(1)  # warm-up
    t0 = time.perf_counter()
    n = 0
    while n < max_steps:
        o.step(1)
        n += 1
        if time.perf_counter() - t0 > budget_s:
            break
    dt = time.perf_counter() - t0
    o.close()
    return scene.n_nodes * n / dt / 1e6, n, dt


def run_reference(args, rank):
    if rank != 0:
        return 0
    scene = build_scene(args)
    threads = os.cpu_count() or 1
    total_budget = float(os.environ.get("PF_REF_BUDGET_S", "120"))
    mlups, n, dt = cpu_oracle_rate(scene, total_budget, args.steps, threads)
    line = {
        "impl": "reference", "metric": "MLUPS (coupled LBM+IBM+SEM+fibrin step)", "value": round(mlups, 3),
        "unit": "MLUPS", "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": dt / n * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64", "data": "synthetic",
        "config": dict(bench_config(args, scene, args.precision, args.gpus), timed_steps=n),
        "cpu_baseline": {"value": round(mlups, 3), "unit": "MLUPS", "cores": threads, "kind": "port",
                         "sample": f"{n} coupled steps of the full scene after 1 warm-up step (budget "
                                   f"{total_budget:.0f} s); CPU restatement of the reference kernels, FP64, "
                                   f"stencil-local IBM, OpenMP {threads} threads"},
        "e2e": {"value": round(mlups, 3), "unit": "MLUPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def bench_config(args, scene, prec, world):
    """The config object of both arms' lines (same keys, same workload)."""
    return {"workload": workload_name(args), "lattice": [scene.nx, scene.ny, scene.nz], "nodes": scene.n_nodes,
            "elements": scene.n_platelets * scene.n_elem, "fibrin_nodes": scene.n_fib,
            "receptors": scene.n_platelets * scene.n_rec, "parallelism": f"replicas x{world}",
            "l2": "working set > L2 (2 x 19 x N x 4 B populations)", "precision": PREC_NAME[prec]}


def workload_name(args):
    if getattr(args, "workload", "single_large") == "plain_small":
        return ("plain_small: D3Q19 64x32x32 body-force channel, bounce-back walls on y and z, periodic x, "
                "1 platelet x 600 SEM elements, 200-node/400-link Hookean fibrin mesh")
    return (f"single_large: D3Q19 {args.nx}x{args.ny}x{args.nz} shear 1000/s Zou/He walls, {args.platelets} platelets"
            f" x 600 SEM elements (400 membrane + 200 cytoplasm, Morse U0=1 rho=2 r_eq=0.3 cut 1.0 um), "
            f"{args.fibrin}-node/{2 * args.fibrin}-link Hookean fibrin on the bottom wall, 200 receptors/platelet, "
            f"bond p_on/p_off 1e-2/1e-3 per step")


def batched_served(args, gpu, plain_f32_mlups, fp16_scale):
    """The metric's other parts, measured after the headline: the same
    channel with FP16-shifted populations; the 64-job ensemble (32^3 ..
    128x64x64 nodes, log-uniform; 1-8 platelets; 1k-5k fibrin nodes) as one
    autotuned fused batch in FP32 and FP16; and the served loop (Poisson
    arrivals, 20 jobs/s, requested steps U{500..5000}, 150 GB budget) over a
    short arrival window, with p50 / p99 time to completion."""
    import torch
    from platelet_fiber_gpu_gb300 import serve
    from platelet_fiber_gpu_gb300 import workloads as W
    out = {}
    scene = build_scene(args)
    job = gpu.Job(scene, 2, fp16_scale)
    job.step(args.warmup, graph=True)
    st = torch.cuda.current_stream()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    a.record(st)
    rc = job.step(args.steps, graph=True)
    b.record(st)
    torch.cuda.synchronize()
    if rc != gpu.PFGPU_OK or job.steps != args.warmup + args.steps:
        raise RuntimeError("FP16 channel run incomplete")
    ms = a.elapsed_time(b) / args.steps
    job.close()
    out["single_f16"] = {"mlups": round(scene.n_nodes / (ms / 1e3) / 1e6, 1), "ms_per_step": round(ms, 4),
                         "steps": args.steps}
    scenes = [W.batch_job(3, i) for i in range(64)]
    bt = {}
    for prec in (1, 2):
        r = serve.run_batched(prec, steps=args.batch_steps, scenes=scenes, chunk=50)
        bt[PREC_NAME[prec]] = {"mlups": r["mlups"], "seconds": r["seconds"], "shape": r["shape"]}
    bt["jobs"], bt["nodes"], bt["steps"] = 64, sum(sc.n_nodes for sc in scenes), args.batch_steps
    bt["f16_over_f32"] = round(bt["f16-shifted"]["mlups"] / bt["f32"]["mlups"], 3)
    out["batched"] = bt
    sv = {}
    for prec in (1, 2):
        r = serve.run_served(prec, rate=20.0, duration=args.served_seconds, scenes=scenes[:32])
        sv[PREC_NAME[prec]] = {k: r[k] for k in ("mlups", "latency_p50_s", "latency_p99_s", "jobs", "makespan_s",
                                                  "mean_live_jobs")}
    sv["rate_per_s"], sv["arrival_window_s"] = 20.0, args.served_seconds
    out["served"] = sv
    out["f16_batched_over_plain_f32"] = round(bt["f16-shifted"]["mlups"] / plain_f32_mlups, 3)
    out["f16_served_over_plain_f32"] = round(sv["f16-shifted"]["mlups"] / plain_f32_mlups, 3)
    out["target"] = "batched+served FP16-shifted >= 1.6x the plain FP32 channel's aggregate MLUPS"
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precision", type=int, default=1, help="0 fp64, 1 fp32, 2 fp16-shifted")
    ap.add_argument("--seed", type=int, default=2)
    ap.add_argument("--nx", type=int, default=256)
    ap.add_argument("--ny", type=int, default=128)
    ap.add_argument("--nz", type=int, default=128)
    ap.add_argument("--platelets", type=int, default=50)
    ap.add_argument("--fibrin", type=int, default=20000)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-budget", type=float, default=20.0)
    ap.add_argument("--profile-steps", type=int, default=200)
    ap.add_argument("--no-batch", action="store_true",
                    help="skip the FP16 single-channel, batched-ensemble and served runs")
    ap.add_argument("--batch-steps", type=int, default=100)
    ap.add_argument("--served-seconds", type=float, default=8.0)
    ap.add_argument("--workload", default="single_large", choices=["single_large", "plain_small"],
                    help="single_large (the 256x128x128 channel) or plain_small (the 64x32x32 body-force channel)")
    args = ap.parse_args()
    rank, world, local = dist_env()

    if args.impl == "reference":
        return run_reference(args, rank)

    import torch
    torch.cuda.set_device(local)
    pg = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
        pg = dist
    from platelet_fiber_gpu_gb300 import gpu
    from platelet_fiber_gpu_gb300.build import build
    if rank == 0:
        build()
    if pg:
        pg.barrier()

    scene = build_scene(args)
    prec = args.precision
    fp16_scale = 0.0
    N = scene.n_nodes
    PE = scene.n_platelets * scene.n_elem

    def barrier_sync():
        torch.cuda.synchronize()
        if pg:
            pg.barrier()
        torch.cuda.synchronize()

    def max_over_ranks(x: float) -> float:
        return reduce_max(pg, x, "cuda")

    # ---- device-resident throughput: K graph replays of the step
    job = gpu.Job(scene, prec, fp16_scale)
    job.step(args.warmup, graph=True)
    launches = job.launches_per_step
    lbm_kernel = job.lbm_kernel
    barrier_sync()
    start = torch.cuda.Event(enable_timing=True)
    stop = torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clocks:
        stream = torch.cuda.current_stream()
        start.record(stream)
        t0 = time.perf_counter()
        rc_timed = job.step(args.steps, graph=True)  # synchronises the job's stream before returning
        stop.record(stream)
        barrier_sync()
        wall = time.perf_counter() - t0
    # every timed step ran: no stop, detachment or device error bit (step()
    # raises on error bits and returns PFGPU_DONE once the job stopped)
    if rc_timed != gpu.PFGPU_OK or job.steps != args.warmup + args.steps:
        raise RuntimeError(f"timed region incomplete: status {rc_timed}, {job.steps} steps of "
                           f"{args.warmup + args.steps}")
    # the job runs on its own stream and step() returns after it finished, so
    # the host wall time and the event pair bracket the same work
    dev_ms = start.elapsed_time(stop)
    t_step = max_over_ranks(max(dev_ms / 1e3, wall) / args.steps)
    value = replica_value(world, N, t_step)
    clk = clocks.summary()

    # ---- live per-phase CUDA-event timing (serialised pass, same job)
    phases = job.profile(args.profile_steps)
    lbm_ms = phases["lbm"] / args.profile_steps
    job.close()

    # ---- end to end through the C ABI from host buffers
    # the caller's host buffers, in pinned memory as a driver holding its
    # arrays for the whole run keeps them: the initial populations (the
    # equilibrium of the channel flow, made before timing) and the arrays the
    # lattice and element state are read back into
    scene.f_init = None
    j0 = gpu.Job(scene, prec, fp16_scale)
    f_host = gpu.pinned((19, N))
    f_host[:] = j0.lattice(fIN=True)["fIN"]
    j0.close()
    scene.f_init = f_host
    lat_out = {"fIN": gpu.pinned((19, N)), "rho": gpu.pinned(N), "u": gpu.pinned((3, N)), "F": gpu.pinned((3, N))}
    el_out = {"X": gpu.pinned(PE), "Y": gpu.pinned(PE), "RY": gpu.pinned(PE), "Z": gpu.pinned(PE),
              "V": gpu.pinned((3, PE)), "F": gpu.pinned((3, PE))}
    for a in (*lat_out.values(), *el_out.values()):
        a.fill(0.0)
    # every host array the scene hands to pfgpu_job_create, and what
    # pfgpu_job_get_lattice (fIN, rho, u, F) and _get_elements (X, Y, RY, Z,
    # V, F) return
    from platelet_fiber_gpu_gb300.scene import _ARRAY_FIELDS
    h2d_bytes = sum(np.asarray(getattr(scene, f)).nbytes for f in _ARRAY_FIELDS if getattr(scene, f) is not None)
    d2h_bytes = sum(a.nbytes for a in (*lat_out.values(), *el_out.values()))
    barrier_sync()
    t0 = time.perf_counter()
    j2 = gpu.Job(scene, prec, fp16_scale)
    t1 = time.perf_counter()
    j2.step(0, graph=True)  # captures and instantiates the step graph
    t2 = time.perf_counter()
    rc_e2e = j2.step(args.steps, graph=True)
    t3 = time.perf_counter()
    j2.lattice(out=lat_out)
    j2.elements(out=el_out)
    torch.cuda.synchronize()
    t4 = time.perf_counter()
    e2e_s = t4 - t0
    if rc_e2e != gpu.PFGPU_OK or j2.steps != args.steps:
        raise RuntimeError(f"end-to-end run incomplete: status {rc_e2e}, {j2.steps} of {args.steps} steps")
    j2.close()
    e2e_breakdown = {"create_upload": round((t1 - t0) * 1e3, 3), "graph_capture": round((t2 - t1) * 1e3, 3),
                     "steps": round((t3 - t2) * 1e3, 3), "download": round((t4 - t3) * 1e3, 3)}
    e2e_s = max_over_ranks(e2e_s)
    e2e_value = replica_value(world, N * args.steps, e2e_s)

    peak, peak_kind = measured_peak()
    bpn = BYTES_PER_NODE[prec]
    achieved = N * bpn / (lbm_ms / 1e3) / 1e9
    traffic_per_launch = lattice_traffic(prec, lbm_kernel, N)

    line = {
        "metric": "MLUPS (coupled LBM+IBM+SEM+fibrin step)",
        "value": round(value, 1),
        "unit": "MLUPS",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": round(t_step * 1e3, 4),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": PREC_NAME[prec],
        "data": "synthetic",
        "config": bench_config(args, scene, prec, world),
        "sem_elem_steps_per_s": round(world * PE / t_step, 1),
        "e2e": {"value": round(e2e_value, 1), "unit": "MLUPS",
                "h2d_bytes_per_step": int(h2d_bytes / args.steps), "d2h_bytes_per_step": int(d2h_bytes / args.steps),
                "seconds": round(e2e_s, 4), "breakdown_ms": e2e_breakdown,
                "what": "pfgpu_job_create from pinned host arrays (read in place by the device) + step graph "
                        "capture + K graph steps + pfgpu_job_get_lattice/elements into pinned host arrays"},
        "roofline": {"bound": "hbm", "kernel": lbm_kernel, "achieved": round(achieved, 1), "peak": peak,
                     "unit": "GB/s", "frac": round(achieved / peak, 4), "peak_kind": peak_kind,
                     "bytes_per_node": bpn, "launch_ms": round(lbm_ms, 5),
                     "traffic": traffic_per_launch},
        "phases_ms_per_step": {k: round(v / args.profile_steps, 5) for k, v in phases.items()},
        "clocks": clk,
        "gpu_launches": launches * args.steps,
    }
    if rank == 0 and not args.no_batch and args.workload == "single_large":
        line["batched_served"] = batched_served(args, gpu, value, fp16_scale)
    if rank == 0 and not args.no_cpu_baseline:
        small = build_scene(args)
        mlups, n, dt = cpu_oracle_rate(small, args.cpu_budget, 1000, os.cpu_count() or 1)
        line["cpu_baseline"] = {"value": round(mlups, 3), "unit": "MLUPS", "cores": os.cpu_count() or 1,
                                "kind": "port",
                                "sample": f"{n} coupled steps of the same scene after 1 warm-up step "
                                          f"({dt:.1f} s), FP64 CPU restatement of the reference kernels, "
                                          f"stencil-local IBM"}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if pg:
        pg.barrier()
        pg.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
