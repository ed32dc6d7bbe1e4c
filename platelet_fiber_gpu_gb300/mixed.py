"""Mixed-precision large run: the 512x256x256 channel (500 platelets x 600
elements, 100k-node / 200k-link fibrin) with FP16-shifted populations and
FP32 collision, its MLUPS, and its velocity and element-trajectory error
against an FP64 run of the same seed on the GPU (FP32 beside it for
comparison).  Every run takes the same number of steps from the same
initial state; the first `warmup` steps are not timed.

    python -m platelet_fiber_gpu_gb300.mixed --steps 1000
"""
from __future__ import annotations

import argparse
import json
import time

import numpy as np

from . import workloads as W
from .gpu import Job, lib


def _rel_l2(a, b) -> float:
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def run(steps: int = 1000, seed: int = 5, warmup: int = 3, precisions=(2, 1, 0)) -> dict:
    sc = W.mixed_large(seed)
    N = sc.n_nodes
    runs = {}
    for prec in precisions:
        j = Job(sc, prec)
        j.step(warmup)
        lib().pfgpu_job_sync(j.h)
        t0 = time.perf_counter()
        j.step(steps - warmup)
        dt = time.perf_counter() - t0
        L = j.lattice(fIN=False)
        E = j.elements()
        runs[prec] = dict(mlups=N * (steps - warmup) / dt / 1e6, s_per_step=dt / (steps - warmup),
                          u=L["u"], pos=np.stack([E["X"], E["RY"], E["Z"]]))
        j.close()
    out = {"workload": "mixed_large: D3Q19 512x256x256 shear 1000/s, 500 platelets x 600 elements, "
                       "100k-node/200k-link fibrin", "nodes": N, "elements": sc.n_platelets * sc.n_elem,
           "steps": steps, "seed": seed}
    names = {0: "fp64", 1: "fp32", 2: "fp16_shifted"}
    ref = runs.get(0)
    for prec, r in runs.items():
        o = {"mlups": round(r["mlups"], 1), "ms_per_step": round(r["s_per_step"] * 1e3, 4)}
        if ref is not None and prec != 0:
            o["velocity_rel_l2_vs_fp64"] = _rel_l2(r["u"], ref["u"])
            o["position_rel_l2_vs_fp64"] = _rel_l2(r["pos"], ref["pos"])
            o["position_max_abs_um_vs_fp64"] = float(np.abs(r["pos"] - ref["pos"]).max())
        out[names[prec]] = o
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--seed", type=int, default=5)
    args = ap.parse_args()
    print(json.dumps(run(args.steps, args.seed)), flush=True)


if __name__ == "__main__":
    main()
